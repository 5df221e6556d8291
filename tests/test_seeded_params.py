"""The package's seeded parameter stream (used by bench.py and the examples) is the oracle's
splitmix64 stream, so the workloads' inputs are the ones the oracle checks."""
import numpy as np
import pytest


@pytest.mark.parametrize("seed,count", [(0, 5), (26, 104), (6023, 216), (2**64 - 1, 7), (123456789, 1000), (3, 0)])
def test_seeded_params_match_the_oracle_stream(seed, count):
    import quantum_geometric_tensor_gb300 as Q
    from oracle import oracle as O
    a = Q.seeded_params(seed, count)
    assert a.shape == (count,) and a.dtype == np.float64
    assert np.array_equal(a, O.splitmix64_params(seed, count))
    assert np.all((a >= 0) & (a < 2 * np.pi))
