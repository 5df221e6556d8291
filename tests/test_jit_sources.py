"""The straight-line pass kernels a plan generates compile for sm_103a (no GPU
needed: the schedule is built on the host and every generated source goes
through the runtime compiler).  The GPU tests in test_gpu_jit_passes.py check
what they compute."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    L.qgt_plan_jit_check.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_double)]
    return Q


def check(Q, n, gates, P, tmp_path, compile=1, **opts):
    d = Q.circuit_desc(n, gates, P)
    o = Q.PlanOptions()
    Q.lib().qgt_plan_default_options(C.byref(o))
    o.precision = Q.MIXED
    for k_, v_ in opts.items():
        setattr(o, k_, v_)
    sec = C.c_double()
    rc = Q.lib().qgt_plan_jit_check(C.cast(C.pointer(d), C.c_void_p), C.cast(C.pointer(o), C.c_void_p),
                                    str(tmp_path).encode(), compile, C.byref(sec))
    assert rc > 0, Q.lib().qgt_last_error()
    return rc, sec.value


def test_hea_pass_kernels_compile(Q, tmp_path):
    n, L = 14, 2
    k, s = check(Q, n, Q.ansatz_gates(n, L, "cz"), 2 * n * L, tmp_path)
    srcs = sorted(p.name for p in tmp_path.iterdir())
    assert len(srcs) == k and all(x.startswith("qgt_pass") for x in srcs)
    print(f"{k} kernels compiled in {s:.1f} s")


def test_all_gate_kinds_compile(Q, tmp_path):
    rng = np.random.default_rng(5)
    n = 13
    kinds = [Q.H, Q.X, Q.Y, Q.Z, Q.S, Q.T, Q.RX, Q.RY, Q.RZ, Q.CNOT, Q.CZ, Q.SWAP]
    gates, p = [], 0
    for _ in range(60):
        t = int(rng.choice(kinds))
        q0 = int(rng.integers(n))
        q1 = int((q0 + 1 + rng.integers(n - 1)) % n)
        if t in (Q.RX, Q.RY, Q.RZ):
            gates.append((t, q0, -1, p, 0.0))
            p += 1
        elif t in (Q.CNOT, Q.CZ, Q.SWAP):
            gates.append((t, q0, q1, -1, 0.0))
        else:
            gates.append((t, q0, -1, -1, 0.0))
    check(Q, n, gates, p, tmp_path)


def test_twenty_qubit_sources(Q, tmp_path):
    """The headline plan's kernels are generated (not compiled here: that takes minutes on this host)."""
    n, L = 20, 8
    k, _ = check(Q, n, Q.ansatz_gates(n, L, "cz"), 2 * n * L, tmp_path, compile=0)
    assert k >= 6


@pytest.mark.parametrize("tile,bounds", [(14, "__launch_bounds__(1024, 1)"), (13, "__launch_bounds__(512, 2)")])
def test_sixteen_amplitude_tile_sources(Q, tmp_path, tile, bounds):
    """16 amplitudes per thread (thread_amps = 16): 1024-thread 14-qubit tiles and 512-thread
    13-qubit tiles (two per SM) generate and compile."""
    n, L = 16, 2
    k, s = check(Q, n, Q.ansatz_gates(n, L, "cz"), 2 * n * L, tmp_path, tile_bits=tile, thread_amps=16)
    srcs = [p.read_text() for p in tmp_path.iterdir()]
    assert k == len(srcs) and all(bounds in x for x in srcs)


def test_prologue_order_and_tables(Q, tmp_path):
    """Generated kernels issue the tile loads of every entry point before the coefficient staging
    (so the loads overlap the staging's reads and its barrier), stage behind one barrier, look up
    the slot and generator tables in constant memory, and end without a CTA-wide barrier (the row
    maximum is one atomicMax per warp)."""
    n, L = 16, 3
    check(Q, n, Q.ansatz_gates(n, L, "cz"), 2 * n * L, tmp_path, compile=0)
    srcs = {p.name: p.read_text() for p in tmp_path.iterdir()}
    assert srcs
    for name, src in srcs.items():
        body = src[src.index("__global__"):]
        assert "static __device__ const int qslot_" not in src, name
        assert "static __constant__ int qslot_" in src, name
        stg = body.index("STG_:")
        loads = [i for i in range(len(body)) if body.startswith("const T* src = Vp", i)]
        assert loads and max(loads) < stg, name
        dispatch = body.index("switch (start)", stg)
        assert body[stg:dispatch].count("__syncthreads()") == 1, name
        tail = body[body.rindex("if (flags & "):]
        assert "__syncthreads" not in tail and "atomicMax" in tail, name
        if "zgen_apply" in body:
            assert "static __constant__ int zg_" in src, name
