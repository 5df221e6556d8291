"""Learned metric preconditioner, GPU PCG and the natural-gradient VQE loop
through the C ABI, against the numpy checker (oracle/mlp.py) and the FP64
oracle.

- forward / backward kernels: loss within 1e-5 relative, weight gradient
  within 2e-4 relative (FP32 accumulation against FP64, same BF16 weights);
- PCG: the same iterates as the checker (iterations equal, x within 1e-9);
- training lowers the loss, and on held-out points the trained network cuts
  PCG iterations against unpreconditioned CG at the same residual;
- the VQE loop on the device follows the oracle's FP64 trajectory (1e-9),
  and the learned-PCG loop gives the Cholesky loop's energies within 1e-6."""
import ctypes as C

import numpy as np
import pytest

from oracle import mlp
from oracle import oracle as O

pytestmark = pytest.mark.gpu


class PCfg(C.Structure):
    _fields_ = [("num_params", C.c_int32), ("width", C.c_int32), ("rank", C.c_int32), ("lam", C.c_double),
                ("u_scale", C.c_double), ("seed", C.c_uint64), ("device", C.c_int32)]


class TOpt(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_double), ("weight_decay", C.c_double),
                ("seed", C.c_uint64)]


class VOpt(C.Structure):
    _fields_ = [("steps", C.c_int32), ("eta", C.c_double), ("pcg_tol", C.c_double), ("pcg_max_iter", C.c_int32),
                ("solver", C.c_int32)]


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    vp = C.c_void_p
    L.qgt_precond_default_config.argtypes = [C.POINTER(PCfg)]
    L.qgt_precond_default_train_options.argtypes = [C.POINTER(TOpt)]
    L.qgt_precond_create.argtypes = [C.POINTER(PCfg), C.POINTER(vp)]
    L.qgt_precond_destroy.argtypes = [vp]
    L.qgt_precond_num_weights.argtypes = [vp]
    L.qgt_precond_num_weights.restype = C.c_int64
    L.qgt_precond_get_weights.argtypes = [vp, vp]
    L.qgt_precond_set_weights.argtypes = [vp, vp]
    L.qgt_precond_loss_grad.argtypes = [vp, vp, vp, C.c_int32, vp, vp]
    L.qgt_precond_predict.argtypes = [vp, vp, C.c_int32, vp, vp]
    L.qgt_precond_train.argtypes = [vp, vp, vp, C.c_int32, C.POINTER(TOpt), vp]
    L.qgt_precond_train_circuit.argtypes = [vp, vp, vp, C.c_int32, C.c_int, C.POINTER(TOpt), vp]
    L.qgt_metric_dataset.argtypes = [vp, vp, C.c_int32, C.c_int, C.c_int32, vp]
    L.qgt_pcg_solve_f64.argtypes = [vp, vp, C.c_double, C.c_int32, vp, vp, C.c_int32, C.c_double, C.c_int32, vp, vp, vp]
    L.qgt_vqe_default_options.argtypes = [C.POINTER(VOpt)]
    L.qgt_vqe_run.argtypes = [vp, vp, vp, C.POINTER(VOpt), vp, vp, vp, vp]
    return Q


def p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def make_pc(Q, P, W, r, seed=3):
    L = Q.lib()
    cfg = PCfg()
    L.qgt_precond_default_config(C.byref(cfg))
    cfg.num_params, cfg.width, cfg.rank, cfg.seed = P, W, r, seed
    h = C.c_void_p()
    assert L.qgt_precond_create(C.byref(cfg), C.byref(h)) == 0, L.qgt_last_error()
    return h, cfg


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_forward_backward_match_checker(Q, orc):
    L = Q.lib()
    n, layers = 5, 2
    P, W, r = 2 * n * layers, 48, 4
    h, cfg = make_pc(Q, P, W, r)
    nw = L.qgt_precond_num_weights(h)
    rng = np.random.default_rng(5)
    w = (rng.standard_normal(nw) * 0.2).astype(np.float32)
    assert L.qgt_precond_set_weights(h, p(w)) == 0
    S = 6
    gates = O.gates_array(Q.ansatz_gates(n, layers, "cnot"))
    th = rng.uniform(0, 2 * np.pi, (S, P))
    metric = np.stack([orc.qgt_from_states(*orc.derivatives(n, gates, t)).real for t in th])
    loss = np.zeros(1)
    g = np.zeros(nw, dtype=np.float32)
    assert L.qgt_precond_loss_grad(h, p(th), p(metric), S, p(loss), p(g)) == 0, L.qgt_last_error()
    lref, gref = mlp.loss_grad(w, th, metric.astype(np.float32).astype(np.float64), P, W, r, cfg.lam, cfg.u_scale)
    assert abs(loss[0] - lref) / lref < 1e-5
    assert rel(g.astype(np.float64), gref) < 2e-4
    d = np.zeros((S, P))
    U = np.zeros((S, P, r))
    assert L.qgt_precond_predict(h, p(th), S, p(d), p(U)) == 0
    f = mlp.forward(w, th, P, W, r, cfg.lam, cfg.u_scale)
    assert rel(d, f["d"]) < 1e-5 and rel(U, f["U"]) < 1e-5
    L.qgt_precond_destroy(h)


@pytest.mark.parametrize("r", [0, 6])
def test_pcg_matches_checker(Q, r):
    L = Q.lib()
    rng = np.random.default_rng(11 + r)
    P = 64
    B = rng.standard_normal((P, 10))
    A = B @ B.T / 10 + np.diag(rng.uniform(0, 0.1, P))
    b = rng.standard_normal(P)
    d = rng.uniform(0.5, 2.0, P)
    U = rng.standard_normal((P, r)) * 0.3 if r else None
    x = np.zeros(P)
    it = np.zeros(1, dtype=np.int32)
    res = np.zeros(1)
    assert L.qgt_pcg_solve_f64(p(A), p(b), 1e-3, P, p(d), p(U), r, 1e-10, 500, p(x), p(it), p(res)) == 0
    xr, itr, _ = mlp.pcg(A, b, 1e-3, d=d, U=U, tol=1e-10, max_iter=500)
    assert abs(int(it[0]) - itr) <= 1 and res[0] <= 1e-10
    assert rel(x, np.linalg.solve(A + 1e-3 * np.eye(P), b)) < 1e-9


def test_training_cuts_pcg_iterations(Q):
    """Train on exact metrics of a 10-qubit, 2-layer circuit (P = 40); on
    held-out points the learned M = diag(d) + U U^T needs fewer PCG iterations
    than unpreconditioned CG for the same relative residual."""
    L = Q.lib()
    n, layers = 10, 2
    P, W, r = 2 * n * layers, 128, 8
    gates = Q.ansatz_gates(n, layers, "cnot")
    desc = Q.circuit_desc(n, gates, P)
    rng = np.random.default_rng(2)
    S, H = 1536, 16
    th = rng.uniform(0, 2 * np.pi, (S + H, P))
    metric = np.zeros((S + H, P, P))
    assert L.qgt_metric_dataset(C.byref(desc), p(th), S + H, Q.FP64, 0, p(metric)) == 0, L.qgt_last_error()
    h, cfg = make_pc(Q, P, W, r)
    opt = TOpt()
    L.qgt_precond_default_train_options(C.byref(opt))
    opt.epochs, opt.batch, opt.lr = 60, 128, 2e-3
    hist = np.zeros(opt.epochs)
    assert L.qgt_precond_train(h, p(th[:S]), p(metric[:S]), S, C.byref(opt), p(hist)) == 0, L.qgt_last_error()
    assert hist[-1] < 0.5 * hist[0]
    d = np.zeros((H, P))
    U = np.zeros((H, P, r))
    assert L.qgt_precond_predict(h, p(th[S:]), H, p(d), p(U)) == 0
    its_cg, its_pc = [], []
    for k in range(H):
        A = metric[S + k]
        b = rng.standard_normal(P)
        x = np.zeros(P)
        it = np.zeros(1, dtype=np.int32)
        res = np.zeros(1)
        assert L.qgt_pcg_solve_f64(p(A), p(b), 1e-3, P, None, None, 0, 1e-8, 2000, p(x), p(it), p(res)) == 0
        its_cg.append(int(it[0]))
        Uk = np.ascontiguousarray(U[k])
        assert L.qgt_pcg_solve_f64(p(A), p(b), 1e-3, P, p(d[k]), p(Uk), r, 1e-8, 2000, p(x), p(it), p(res)) == 0
        its_pc.append(int(it[0]))
        assert res[0] <= 1e-8
    print(f"loss {hist[0]:.3e} -> {hist[-1]:.3e}; CG {np.mean(its_cg):.1f} its, learned PCG {np.mean(its_pc):.1f} its")
    assert np.mean(its_pc) < np.mean(its_cg)
    L.qgt_precond_destroy(h)


def test_limits_of_the_diag_rank_r_form(Q):
    """What diag + rank-r preconditioners of the metric gain on held-out points of a 10-qubit,
    3-layer circuit (P = 60, r = 8), with exact GPU metrics: the deflation form built from the
    point's own smallest eigenvectors cuts CG iterations by at least 1.5x, but the same form
    built from the nearest of 3000 training points gains nothing (its eigenspace overlaps the
    held-out one no more than a random point's does), while a point 0.1 rad away still gives
    nearly the same subspace: the map from theta to the useful subspace changes on a scale far
    below the spacing of any training set in 60 dimensions."""
    from quantum_geometric_tensor_gb300 import precond_limits as PL
    n, layers, r = 10, 3, 8
    P = 2 * n * layers
    gates = Q.ansatz_gates(n, layers, "cnot")
    rng = np.random.default_rng(4)
    tr = rng.uniform(0, 2 * np.pi, (3000, P))
    ho = rng.uniform(0, 2 * np.pi, (12, P))
    res = PL.analyse(lambda t: Q.metric_dataset(n, gates, t, precision=Q.FP64), tr, ho, r=r, rhos=(0.1, 1.0))
    red, ov = res["reduction_vs_cg"], res["overlap"]
    print(res["iterations"], ov, res["distance"])
    assert red["deflation"] >= 1.5
    assert red["deflation_nn"] <= 1.1
    assert ov["nn"] <= ov["random"] + 0.1
    assert ov["at_0.1"] >= 0.9 and red["deflation_at_0.1"] >= 0.9 * red["deflation"]
    assert res["distance"]["nearest_train"] >= 0.7 * res["distance"]["random_point"]


def oracle_vqe(orc, n, gates, th0, steps, eta, lam):
    th = th0.copy()
    E = []
    g = O.gates_array(gates)
    for _ in range(steps):
        psi, D = orc.derivatives(n, g, th)
        Hpsi = orc.tfim_apply(n, psi)
        E.append(float(np.real(np.vdot(psi, Hpsi))))
        Qm = orc.qgt_from_states(psi, D)
        grad = orc.energy_grad(D, Hpsi)
        x, _ = orc.cholesky_solve(Qm.real, grad, lam)
        th = th - eta * x
    return np.array(E)


def test_vqe_loop_matches_oracle_and_solvers_agree(Q, orc):
    L = Q.lib()
    n, layers = 6, 2
    P = 2 * n * layers
    gates = Q.ansatz_gates(n, layers, "cnot")
    desc = Q.circuit_desc(n, gates, P)
    th0 = O.splitmix64_params(9, P)
    steps = 25
    popt = Q.PlanOptions()
    L.qgt_plan_default_options(C.byref(popt))
    popt.precision = Q.FP64
    vo = VOpt()
    L.qgt_vqe_default_options(C.byref(vo))
    vo.steps, vo.eta = steps, 0.05
    E_chol = np.zeros(steps)
    assert L.qgt_vqe_run(C.byref(desc), C.byref(popt), None, C.byref(vo), p(th0), p(E_chol), None, None) == 0, \
        L.qgt_last_error()
    E_ref = oracle_vqe(orc, n, gates, th0, steps, 0.05, 1e-3)
    assert np.abs(E_chol - E_ref).max() < 1e-9
    assert E_chol[-1] < E_chol[0]
    # CG and learned-PCG loops (untrained network: still an SPD preconditioner) at a tight tolerance
    h, _ = make_pc(Q, P, 32, 4)
    for solver, pc in ((1, None), (2, h)):
        vo.solver, vo.pcg_tol = solver, 1e-12
        E = np.zeros(steps)
        its = np.zeros(steps, dtype=np.int32)
        assert L.qgt_vqe_run(C.byref(desc), C.byref(popt), pc, C.byref(vo), p(th0), p(E), p(its), None) == 0, \
            L.qgt_last_error()
        assert np.abs(E - E_chol).max() < 1e-6
        assert its.min() >= 1
    L.qgt_precond_destroy(h)
