"""Failure paths on the GPU, exercised without a GPU fault.

* The integer-digit Gram's mbarrier waits are bounded by the global timer.  The
  fault-injection hook makes the converter warps wait on a barrier that nothing
  arrives on; each CTA gives up after the short limit, drains its own TMA loads
  and MMAs, frees its tensor memory and reports QGT_ERROR_TIMEOUT (-13).  The
  same plan's next step (hook off) succeeds and matches its earlier result
  bit for bit: the error word is cleared on the stream before every run.
* A natural-gradient solve that stays singular after the lambda x 10 retries
  (lambda = 0 and a parameter that no gate uses, so Re Q has a zero row) returns
  QGT_ERROR_NOT_POSITIVE_DEFINITE (-34) from the single-point plans (whose
  graph solve is retried outside the graph) and from batched plans."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TIMEOUT, NOT_PD = -13, -34


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def test_gram_wait_timeout_reports_and_recovers(Q):
    n, L = 14, 2
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    theta = O.splitmix64_params(77, P)
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(theta)
    with Q.Plan(n, gates, P, precision=Q.MIXED) as pm:
        good = pm.run(theta)
        assert pm.status()[0] == 0
        pm.test_gram_stall(True, 2_000_000)   # every wait of the Gram gives up after 2 ms
        with pytest.raises(Q.QGTError) as ei:
            pm.run(theta)
        assert ei.value.code == TIMEOUT
        assert pm.status()[0] == TIMEOUT
        pm.test_gram_stall(False, 0)
        out = pm.run(theta)
        assert pm.status()[0] == 0
    assert np.array_equal(out["Q"], good["Q"]) and np.array_equal(out["natgrad"], good["natgrad"])
    assert rel(out["Q"].real, ref["Q"].real) < 1e-6
    assert rel(out["grad"], ref["grad"]) < 2e-6


def test_gram_stall_hook_rejects_bad_settings(Q):
    n, L = 10, 1
    gates = Q.ansatz_gates(n, L, "cnot")
    with Q.Plan(n, gates, 2 * n * L, precision=Q.MIXED) as pm:
        with pytest.raises(Q.QGTError):
            pm.test_gram_stall(True, 0)           # a stall needs a limit
        with pytest.raises(Q.QGTError):
            pm.test_gram_stall(True, 5_000_000_000)
    with Q.Plan(n, gates, 2 * n * L, precision=Q.FP64) as p64:
        with pytest.raises(Q.QGTError):
            p64.test_gram_stall(True, 1_000_000)  # FP64 plans have no digit Gram


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
@pytest.mark.parametrize("batch", [1, 2])
def test_singular_solve_after_retries_is_an_error(Q, prec, batch):
    n, L = 6, 2
    gates = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L + 1                      # the last parameter drives no gate: zero row and column in Re Q
    th = np.stack([O.splitmix64_params(3 + b, P) for b in range(batch)])
    with Q.Plan(n, gates, P, precision=getattr(Q, prec), lam=0.0, batch=batch) as p:
        with pytest.raises(Q.QGTError) as ei:
            p.run(th if batch > 1 else th[0])
        assert ei.value.code == NOT_PD
        assert p.status()[0] == NOT_PD
    # the same circuit with a positive lambda solves
    with Q.Plan(n, gates, P, precision=getattr(Q, prec), lam=1e-3, batch=batch) as p:
        out = p.run(th if batch > 1 else th[0])
        assert p.status()[0] == 0
        assert np.all(np.isfinite(out["natgrad"]))
