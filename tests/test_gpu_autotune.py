"""Measured plan configuration (qgt_plan_autotune) and its cache, and the
explicit tile / pass-kernel options.

The tuner times the candidate plans of a circuit (13- or 14-qubit register
tiles, interpreted or compiled pass kernels, 32 or 16 amplitudes per thread on
14-qubit tiles) and keeps the fastest in a text
cache; a circuit in the cache is not timed again.  Whatever it picks computes
the same QGT: tuned plans and tuned ragged batches are checked against the
FP64 plan and the untuned batch (metric 1e-6, Q 2e-6, Berry maps 1e-6)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def test_autotune_picks_and_caches(Q, tmp_path):
    n, L = 15, 3
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    cache = tmp_path / "tune.txt"
    tile, kern, amps, ms = Q.autotune(n, gates, P, cache=cache, steps=3)
    assert tile in (13, 14) and kern in (Q.PASS_INTERPRET, Q.PASS_COMPILED) and amps in (0, 16) and ms > 0
    lines = [x for x in cache.read_text().splitlines() if x and not x.startswith("#")]
    assert len(lines) == 1
    assert Q.autotune(n, gates, P, cache=cache, steps=3) == (tile, kern, amps, pytest.approx(ms, rel=1e-6, abs=1e-6))
    assert len([x for x in cache.read_text().splitlines() if x]) == 1   # read back, not timed again
    theta = O.splitmix64_params(81, P)
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(theta)
    with Q.Plan(n, gates, P, precision=Q.MIXED, tile_bits=tile, pass_kernels=kern, thread_amps=amps) as p:
        info = p.info()
        out = p.run(theta)
    assert info.tile_bits == tile and (info.jit_passes > 0) == (kern == Q.PASS_COMPILED)
    assert info.thread_amps == (16 if amps == 16 else 32)
    assert rel(out["Q"].real, ref["Q"].real) < 1e-6 and rel(out["Q"], ref["Q"]) < 2e-6


@pytest.mark.parametrize("tile,kern,amps", [(13, 1, 0), (13, 2, 0), (14, 1, 0), (14, 2, 0), (13, 2, 16), (14, 2, 16)])
def test_every_configuration_agrees(Q, tile, kern, amps):
    n, L = 16, 2
    gates = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L
    theta = O.splitmix64_params(82, P)
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(theta)
    with Q.Plan(n, gates, P, precision=Q.MIXED, tile_bits=tile, pass_kernels=kern, thread_amps=amps) as p:
        info = p.info()
        assert info.tile_bits == tile and info.thread_amps == (amps or 32)
        out = p.run(theta)
    assert rel(out["Q"].real, ref["Q"].real) < 1e-6 and rel(out["grad"], ref["grad"]) < 2e-6


@pytest.mark.parametrize("n,L,ent,tile", [(20, 8, "cz", 14), (18, 4, "cnot", 14), (20, 8, "cz", 13)])
def test_sixteen_amplitude_tiles_match_fp64(Q, n, L, ent, tile):
    """16 amplitudes per thread (1024-thread 14-qubit or 512-thread 13-qubit tiles, compiled
    kernels, checkpointed and meet-in-the-middle passes) against the FP64 plan at 18-20 qubits."""
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    theta = O.splitmix64_params(83, P)
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(theta)
    with Q.Plan(n, gates, P, precision=Q.MIXED, tile_bits=tile, thread_amps=16) as p:
        assert p.info().thread_amps == 16 and p.info().jit_passes > 0
        out = p.run(theta)
    assert rel(out["Q"].real, ref["Q"].real) < 1e-6 and rel(out["Q"], ref["Q"]) < 2e-6
    assert rel(out["grad"], ref["grad"]) < 2e-6 and abs(out["energy"] - ref["energy"]) < 1e-6


def test_bad_configuration_rejected(Q):
    gates = Q.ansatz_gates(14, 1, "cz")
    for kw in ({"tile_bits": 12}, {"tile_bits": 15}, {"pass_kernels": 3}, {"thread_amps": 8},
               {"thread_amps": 16, "pass_kernels": 1}):
        with pytest.raises(Q.QGTError):
            Q.Plan(14, gates, 28, precision=Q.MIXED, **kw)


def test_tuned_ragged_batch(Q, tmp_path):
    rng = np.random.default_rng(9)
    spec, thetas = [], []
    for c in range(10):
        n, L = int(rng.integers(12, 17)), int(rng.integers(2, 4))
        spec.append((n, Q.ansatz_gates(n, L, "cnot"), 2 * n * L))
        thetas.append(O.splitmix64_params(700 + c, 2 * n * L))
    pairs = [(0, s[0]) for s in spec]
    with Q.Batch(spec, pairs, precision=Q.MIXED, grid=8) as b:
        Qs, maps = b.run(thetas)
    cache = tmp_path / "batch_tune.txt"
    with Q.Batch(spec, pairs, precision=Q.MIXED, grid=8, tune_cache=cache) as b:
        Qt, mapt = b.run(thetas)
    assert cache.exists() and len(cache.read_text().splitlines()) >= 1
    for a, r in zip(Qt, Qs):
        assert rel(a.real, r.real) < 1e-6
    assert np.abs(mapt - maps).max() < 1e-6
