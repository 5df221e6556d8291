"""Headline benchmark: QGTs/sec at 20 qubits, P = 320.

Workload (one "step"): one parameter point of the 20-qubit hardware-efficient
ansatz -- 8 layers of RY(q), RZ(q) on every qubit and a CZ ring (P = 320,
480 gates), complex64 evolution, split-FP16 integer-digit tcgen05 Gram, FP64
projector + renormalisation, TFIM ring (J = h = 1) energy gradient and the
FP64 Cholesky natural-gradient step (Re Q + 1e-3 I) x = grad E.  Parameters
are seeded uniform in [0, 2pi) (splitmix64); data are synthetic (the
reference publishes no dataset for this path).  The working set (2.6 GB of
derivative vectors) is far larger than L2, so no flush is needed between
steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The gb300 arm prints one JSON line with value (device-resident theta and
outputs), e2e (host buffers through qgt_plan_execute_host), roofline of the
dominant kernel, the FP64 GPU path timed on the same point with the mixed
path's error against it, clocks sampled during the timed region, and the
oracle's CPU baseline (one complete QGT step on the host cores, measured).
The reference arm times the CPU implementation of the path (the FP64 oracle
port of the reference algorithms; the reference's own tree is not present on
the GPU host) on the host cores: its K steps are the K slices of one complete
QGT step, so their total time is one measured QGT.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS, LAYERS, ENT, LAMBDA, SEED = 20, 8, "cz", 1e-3, 2026
WORKLOAD = "hea20_L8_czring_P320_tfim_natgrad"
METRIC = "QGTs/sec @20q,P=320 (mixed vs FP64 GPU, rel err<=1e-6); gate HBM GB/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.rows, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, local):
    if ws <= 1:
        return None
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return dist


def max_over_ranks(x: float, dist, device=None) -> float:
    """Max of a per-rank scalar over the ranks (timing of replicas; the only
    collective of the benchmark, none on the data path)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_max: float, ws: int) -> float:
    """Whole-job QGT/s of ws independent replicas, each one QGT per step."""
    return ws * 1000.0 / ms_max


def workload_config(ws: int = 1) -> dict:
    """The workload of both arms (identical dicts: implementation details live outside it)."""
    return {"workload": WORKLOAD, "qubits": N_QUBITS, "layers": LAYERS, "params": 2 * N_QUBITS * LAYERS,
            "entangler": "cz_ring", "hamiltonian": "tfim_ring J=h=1", "lambda": LAMBDA,
            "parallelism": f"replicas{ws}" if ws > 1 else "single",
            "l2": "working set > L2 (3.6 GB device, 5.4 GB host): no flush needed"}


def cpu_qgt_job(slices: int):
    """The FP64 CPU oracle's full QGT step of the headline workload, cut into `slices` calls that
    together compute one complete QGT (psi, all 320 derivative states, the full Gram, projector,
    TFIM energy and gradient, Cholesky step), each piece of work once."""
    from oracle import oracle as O
    O.build()
    orc = O.Oracle()
    g = O.ansatz(N_QUBITS, LAYERS, ENT)
    th = O.splitmix64_params(SEED, O.num_params(g))
    return orc.qgt_job(N_QUBITS, g, th, slices, 1.0, 1.0, LAMBDA)


def cpu_baseline(slices: int = 20):
    """One complete QGT step of the workload on the host cores (OpenMP, all threads), timed end to
    end: no extrapolation."""
    job = cpu_qgt_job(slices)
    t0 = time.perf_counter()
    while job.step() > 0:
        pass
    total = time.perf_counter() - t0
    job.close()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": 1.0 / total, "unit": "QGTs/sec", "cores": cores, "kind": "port",
            "sample": (f"one full QGT step of the workload on the host (FP64 oracle port, OpenMP {cores} threads): "
                       f"psi + all 320 derivative states through the 480 gates, full 320x320 Gram, projector, "
                       f"TFIM energy/gradient, Cholesky step; {total:.1f} s measured"),
            "seconds_per_qgt": total}


def run_reference(args, ws, rank):
    """The CPU implementation of the path (FP64 oracle port of the reference algorithms) on the host
    cores.  A step is 1/K of one full QGT step of the workload (K = --steps): a slice of the 320
    derivative states with their Gram rows, the last step also the projector, gradient and solve, so
    the K timed steps compute exactly one complete QGT and value = 1 / (their total time)."""
    if rank != 0:
        return 0
    K, W = max(1, args.steps), max(0, args.warmup)
    if W:
        warm = cpu_qgt_job(K)
        for _ in range(min(W, warm.slices)):
            warm.step()
        warm.close()
    job = cpu_qgt_job(K)
    ts = []
    t_all = time.perf_counter()
    for _ in range(job.slices):
        t0 = time.perf_counter()
        job.step()
        ts.append(time.perf_counter() - t0)
    total = time.perf_counter() - t_all
    job.close()
    steps = len(ts)
    v = 1.0 / total
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    sample = (f"{steps} steps = one full QGT step of the workload (each 1/{steps} of it: a slice of the 320 "
              f"derivative states through the remaining gates and their Gram rows; the last step also the "
              f"projector, TFIM gradient and Cholesky solve); FP64 oracle port, OpenMP {cores} threads; "
              f"{total:.1f} s measured")
    line = {"metric": METRIC, "value": v, "unit": "QGTs/sec", "n_gpus": ws, "steps": steps,
            "warmup": W, "ms_per_step": 1000.0 * total / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(ws),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "QGTs/sec", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "QGTs/sec", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "step_seconds": [round(t, 3) for t in ts]}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args, ws, rank, local):
    import torch
    import quantum_geometric_tensor_gb300 as Q

    dist = init_dist(ws, local)
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    nq, nl = args.qubits, args.layers
    workload = WORKLOAD if (nq, nl) == (N_QUBITS, LAYERS) else f"hea{nq}_L{nl}_czring_P{2 * nq * nl}_tfim_natgrad"
    gates = Q.ansatz_gates(nq, nl, ENT)
    P = 2 * nq * nl
    theta = Q.seeded_params(SEED + rank, P)
    t0 = time.perf_counter()
    plan = Q.Plan(nq, gates, P, precision=Q.MIXED, lam=LAMBDA, device=dev)
    t_create = time.perf_counter() - t0
    info = plan.info()
    th_d = torch.tensor(theta, dtype=torch.float64, device=f"cuda:{dev}")
    Q_d = torch.zeros((P, P, 2), dtype=torch.float64, device=f"cuda:{dev}")
    g_d = torch.zeros(P, dtype=torch.float64, device=f"cuda:{dev}")
    e_d = torch.zeros(1, dtype=torch.float64, device=f"cuda:{dev}")
    x_d = torch.zeros(P, dtype=torch.float64, device=f"cuda:{dev}")
    stream = torch.cuda.ExternalStream(plan.stream(), device=f"cuda:{dev}")
    L = Q.lib()
    torch.cuda.synchronize()

    def step():
        rc = L.qgt_plan_execute_device(plan.h, th_d.data_ptr(), Q_d.data_ptr(), g_d.data_ptr(), e_d.data_ptr(),
                                       x_d.data_ptr())
        if rc:
            raise Q.QGTError(rc, "qgt_plan_execute_device")

    for _ in range(args.warmup):
        step()
    plan.status()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    st, lam_used = plan.status()
    if st != 0:
        raise RuntimeError(f"device status {st} after the timed steps")
    ms = max_over_ranks(ms, dist, f"cuda:{dev}")
    value = replica_value(ms, ws)

    # e2e: host theta in, host Q / grad / energy / natgrad out, through the public C ABI
    e2e_steps = max(2, min(args.steps, 10))
    bufs = plan.output_buffers()   # host outputs reused across steps, as a training loop would
    plan.run(theta, out=bufs)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        out = plan.run(theta, out=bufs)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / e2e_steps
    e2e_ms = max_over_ranks(e2e_ms, dist, f"cuda:{dev}")
    h2d = P * 8
    d2h = P * P * 16 + 2 * P * 8 + 8

    if rank != 0:
        plan.close()
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return 0

    # phase breakdown + roofline of the dominant kernel (device events on the plan's stream)
    prof = Q.StepProfile()
    L.qgt_plan_profile_step(plan.h, C_byref(prof))
    phases = {"passes": prof.passes_ms, "gram": prof.gram_ms, "hamiltonian": prof.hamiltonian_ms,
              "post": prof.post_ms, "solve": prof.solve_ms, "prepare": prof.prepare_ms}
    hbm, tfl, peak_src = peaks()
    gate_gbs = info.gate_bytes / (prof.passes_ms * 1e-3) / 1e9
    gram_tf = info.gram_flops / (prof.gram_ms * 1e-3) / 1e12
    dom = max(("passes", "gram"), key=lambda k: phases[k])
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        try:
            tj = json.load(open(tp))
            # measured for this workload and this build of the pass kernels only
            kinds = "compiled" if info.jit_passes > 0 else "interpreted"
            same = (tj.get("passes_kernels") == kinds and tj.get("tile_bits") == info.tile_bits and
                    tj.get("thread_amps", 32) == info.thread_amps)
            if tj.get("workload") == workload and (dom != "passes" or same):
                traffic = tj.get(dom)
        except Exception:
            traffic = None
    if dom == "passes":
        kname = ("qgt_passK_run / qgt_passK_ckpt (compiled pass kernels)" if info.jit_passes > 0
                 else "pass2_kernel (interpreted pass programs)")
        roof = {"bound": "hbm", "kernel": kname + ": all register-tile passes of a step", "achieved": gate_gbs,
                "peak": hbm, "unit": "GB/s", "frac": gate_gbs / hbm, "traffic": traffic,
                "peak_source": peak_src, "algorithmic_bytes": info.gate_bytes, "ms": prof.passes_ms}
    else:
        roof = {"bound": "tensor", "kernel": "dg_gram_kernel (+ split-K reduce)", "achieved": gram_tf, "peak": tfl,
                "unit": "TFLOP/s", "frac": gram_tf / tfl, "traffic": traffic, "peak_source": peak_src,
                "algorithmic_flops": info.gram_flops, "ms": prof.gram_ms}

    # FP64 GPU path on the same point; mixed error against it
    fp64 = None
    try:
        if args.no_fp64:
            raise RuntimeError("skipped (--no-fp64)")
        out_m = plan.run(theta)
        with Q.Plan(nq, gates, P, precision=Q.FP64, lam=LAMBDA, device=dev) as p64:
            p64.run(theta)
            t0 = time.perf_counter()
            r64 = p64.run(theta)
            t64 = (time.perf_counter() - t0) * 1000.0
            pr64 = Q.StepProfile()
            L.qgt_plan_profile_step(p64.h, C_byref(pr64))

        def rel(a, b):
            return float(np.linalg.norm(a - b) / np.linalg.norm(b))

        fp64 = {"ms_per_step": pr64.total_ms, "e2e_ms": t64, "value": 1000.0 / pr64.total_ms,
                "speedup_mixed_vs_fp64": pr64.total_ms / ms,
                "rel_err": {"metric": rel(out_m["Q"].real, r64["Q"].real), "berry": rel(out_m["Q"].imag, r64["Q"].imag),
                            "qgt": rel(out_m["Q"], r64["Q"]), "grad": rel(out_m["grad"], r64["grad"]),
                            "natgrad_step": rel(out_m["natgrad"], r64["natgrad"]),
                            "energy_abs": abs(out_m["energy"] - r64["energy"])},
                "phases_ms": {"passes": pr64.passes_ms, "gram": pr64.gram_ms, "solve": pr64.solve_ms}}
    except Exception as ex:
        fp64 = {"error": str(ex)[:200]}

    cb = None
    if ws == 1 and not args.no_cpu and (nq, nl) == (N_QUBITS, LAYERS):
        try:
            cb = cpu_baseline()
            cb.pop("seconds_per_qgt", None)
        except Exception as ex:
            cb = {"error": str(ex)[:200]}

    line = {"metric": METRIC, "value": value, "unit": "QGTs/sec", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64/fp16-digits/f64", "data": "synthetic",
            "config": workload_config(ws) if workload == WORKLOAD else
            {"workload": workload, "qubits": nq, "layers": nl, "params": P, "entangler": "cz_ring",
             "hamiltonian": "tfim_ring J=h=1", "lambda": LAMBDA,
             "parallelism": f"replicas{ws}" if ws > 1 else "single",
             "l2": f"working set {info.device_bytes / 1e9:.1f} GB > L2 (no flush needed)"},
            "precision": "mixed (complex64 evolution, FP16-digit tcgen05 Gram, FP64 projector and solve)",
            "e2e": {"value": ws * 1000.0 / e2e_ms, "unit": "QGTs/sec", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "gpu_launches": info.num_launches * args.steps,
            "roofline": roof,
            "phases_ms": phases,
            "gate_hbm_gbs": gate_gbs,
            "gram_tflops_algorithmic": gram_tf,
            "plan": {"passes": info.num_passes, "vector_passes": info.vector_passes, "tile_bits": info.tile_bits,
                     "thread_amps": info.thread_amps,
                     "device_gb": info.device_bytes / 1e9, "compiled_passes": info.jit_passes,
                     "create_s": t_create},
            "fp64_gpu": fp64,
            "clocks": clk.summary(),
            "cpu_baseline": cb}
    print(json.dumps(line), flush=True)
    plan.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def _line(metric, value, unit, steps, warmup, ms, cfg, extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": steps, "warmup": warmup,
         "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic",
         "config": cfg}
    d.update(extra)
    print(json.dumps(d), flush=True)


def run_ragged(args):
    """1024 circuits (qubits U{12..18}, layers U{2..6}, RY/RZ + CNOT ladder), full QGT of each plus a
    32 x 32 Berry map over (first RY, first RZ of qubit 0), one graph launch per batch."""
    import torch
    import quantum_geometric_tensor_gb300 as Q
    rng = np.random.default_rng(SEED)
    ns, Ls = rng.integers(12, 19, 1024), rng.integers(2, 7, 1024)
    spec = [(int(n), Q.ansatz_gates(int(n), int(L), "cnot"), 2 * int(n) * int(L)) for n, L in zip(ns, Ls)]
    thetas = [Q.seeded_params(5000 + c, s_[2]) for c, s_ in enumerate(spec)]
    tune = args.tune_cache or None
    tuned_before = 0
    if tune and os.path.exists(tune):
        tuned_before = sum(1 for x in open(tune) if x.strip() and not x.startswith("#"))
    t0 = time.perf_counter()
    b = Q.Batch(spec, [(0, s_[0]) for s_ in spec], precision=Q.MIXED, grid=32, tune_cache=tune)
    t_create = time.perf_counter() - t0
    tuning = None
    if tune:
        lines = [x.split() for x in open(tune) if x.strip() and not x.startswith("#")]
        tuning = {"cache": tune, "entries_before": tuned_before, "entries": len(lines),
                  "choices": sorted({f"tile{x[1]}/{'compiled' if x[2] == '2' else 'interpreted' if x[2] == '1' else 'default'}"
                                     for x in lines if len(x) >= 3})}
    info = b.info()
    for _ in range(args.warmup):
        Qs, maps = b.run(thetas)
        b.run_device()
    # value: the batch graph on device-resident thetas (CUDA events on the batch's stream);
    # e2e: the public call with host thetas in and host Q matrices and maps out
    stream = torch.cuda.ExternalStream(b.stream(), device="cuda:0")
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            b.run_device()
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
        bufs = b.output_buffers()   # host outputs reused across batches, as a training loop would
        Qs, maps = b.run(thetas, out=bufs)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            Qs, maps = b.run(thetas, out=bufs)
        e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    errs = []
    for c in (0, 511, 1023):
        n, g, P = spec[c]
        with Q.Plan(n, g, P, precision=Q.FP64, hamiltonian=Q.HAM_NONE) as p64:
            r = p64.run(thetas[c], want=("Q",))
        errs.append(float(np.linalg.norm(Qs[c].real - r["Q"].real) / np.linalg.norm(r["Q"].real)))
    b.close()
    _line("QGTs/sec (ragged batch of 1024 circuits, 12-18 qubits, each with a 32x32 Berry map)", 1024000.0 / ms,
          "QGTs/sec", args.steps, args.warmup, ms,
          {"workload": "ragged1024_q12-18_L2-6_cnot_berry32", "circuits": 1024, "groups": info.num_groups,
           "berry_plans": info.num_berry_plans, "precision": "mixed",
           "plan_configuration": "measured per group (tune cache)" if tune else "defaults"},
          {"dtype": "c64/fp16-digits/f64", "e2e": {"value": 1024000.0 / e2e_ms, "unit": "QGTs/sec", "ms_per_step": e2e_ms,
                                                    "h2d_bytes_per_step": int(sum(len(t) for t in thetas) * 8),
                                                    "d2h_bytes_per_step": int(sum(s_[2] ** 2 * 16 for s_ in spec)
                                                                              + 1024 * 32 * 32 * 8)},
           "graph_kernels": info.graph_kernels, "device_gb": info.device_bytes / 1e9, "create_s": t_create,
           "metric_rel_err_vs_fp64": errs, "tuning": tuning, "clocks": clk.summary()})


def run_hea26(args):
    """26 qubits, 2 layers RY/RZ + CNOT ladder (P = 104), mixed step against the FP64 GPU step."""
    import quantum_geometric_tensor_gb300 as Q
    n, L = 26, 2
    g = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L
    th = Q.seeded_params(26, P)
    with Q.Plan(n, g, P, precision=Q.MIXED) as pm:
        info = pm.info()
        for _ in range(args.warmup):
            om = pm.run(th)
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                om = pm.run(th)
            ms = (time.perf_counter() - t0) * 1000.0 / args.steps
        prof = Q.StepProfile()
        Q.lib().qgt_plan_profile_step(pm.h, C_byref(prof))
    with Q.Plan(n, g, P, precision=Q.FP64) as p64:
        p64.run(th)
        t0 = time.perf_counter()
        o64 = p64.run(th)
        ms64 = (time.perf_counter() - t0) * 1000.0

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))
    hbm, tfl, src = peaks()
    gate_gbs = info.gate_bytes / (prof.passes_ms * 1e-3) / 1e9
    _line("QGTs/sec @26q,P=104 (mixed vs FP64 GPU)", 1000.0 / ms, "QGTs/sec", args.steps, args.warmup, ms,
          {"workload": "hea26_L2_cnot_P104_tfim_natgrad", "qubits": n, "layers": L, "params": P, "precision": "mixed"},
          {"dtype": "c64/fp16-digits/f64",
           "e2e": {"value": 1000.0 / ms, "unit": "QGTs/sec", "h2d_bytes_per_step": P * 8,
                   "d2h_bytes_per_step": P * P * 16 + 2 * P * 8 + 8},
           "phases_ms": {"passes": prof.passes_ms, "gram": prof.gram_ms, "solve": prof.solve_ms},
           "roofline": {"bound": "hbm", "achieved": gate_gbs, "peak": hbm, "unit": "GB/s", "frac": gate_gbs / hbm,
                        "traffic": None, "peak_source": src},
           "gram_tflops_algorithmic": info.gram_flops / (prof.gram_ms * 1e-3) / 1e12,
           "device_gb": info.device_bytes / 1e9,
           "fp64_gpu": {"ms_per_step": ms64, "speedup_mixed_vs_fp64": ms64 / ms,
                        "rel_err": {"metric": rel(om["Q"].real, o64["Q"].real), "berry": rel(om["Q"].imag, o64["Q"].imag),
                                    "grad": rel(om["grad"], o64["grad"]), "natgrad_step": rel(om["natgrad"], o64["natgrad"])}},
           "clocks": clk.summary()})


def run_learned(args):
    """Learned preconditioner: 16 qubits, 6 layers RY/RZ + CNOT ladder (P = 192); train the MLP
    (width 512, rank 16) on 20000 exact metrics generated on the GPU, then PCG iterations on held-out
    points and a 500-step natural-gradient VQE (TFIM ring) against the Cholesky step."""
    import quantum_geometric_tensor_gb300 as Q
    n, L = 16, 6
    g = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L
    rng = np.random.default_rng(SEED)
    S = 20000
    th = rng.uniform(0, 2 * np.pi, (S, P))
    pc = Q.Precond(P, width=512, rank=16)
    t0 = time.perf_counter()
    hist = pc.train_circuit(n, g, th, precision=Q.MIXED, epochs=30, batch=256)
    t_train = time.perf_counter() - t0
    H = 32
    th_h = rng.uniform(0, 2 * np.pi, (H, P))
    met = Q.metric_dataset(n, g, th_h, precision=Q.FP64)
    d, U = pc.predict(th_h)
    its = {"cg": [], "jacobi": [], "learned": []}
    for k in range(H):
        b = rng.standard_normal(P)
        its["cg"].append(Q.pcg_solve(met[k], b, 1e-3, tol=1e-8, max_iter=5000)[1])
        its["jacobi"].append(Q.pcg_solve(met[k], b, 1e-3, d=np.diag(met[k]) + 1e-3, tol=1e-8, max_iter=5000)[1])
        its["learned"].append(Q.pcg_solve(met[k], b, 1e-3, d=d[k], U=U[k], tol=1e-8, max_iter=5000)[1])
    th0 = Q.seeded_params(500, P)
    vqe = {}
    for name, solver, p_ in (("cholesky", Q.VQE_CHOLESKY, None), ("cg", Q.VQE_CG, None),
                             ("learned", Q.VQE_PCG_LEARNED, pc)):
        t0 = time.perf_counter()
        E, it, _ = Q.vqe_run(n, g, th0, steps=500, eta=0.05, solver=solver, precond=p_, pcg_tol=1e-8,
                             pcg_max_iter=5000)
        vqe[name] = {"E_first": float(E[0]), "E_last": float(E[-1]), "s": time.perf_counter() - t0,
                     "pcg_iters_mean": float(it.mean()), "E": E}
    dE = float(np.abs(vqe["learned"]["E"] - vqe["cholesky"]["E"]).max())
    dE_cg = float(np.abs(vqe["cg"]["E"] - vqe["cholesky"]["E"]).max())
    dE_final = {k: float(abs(vqe[k]["E"][-1] - vqe["cholesky"]["E"][-1])) for k in ("cg", "learned")}
    for v in vqe.values():
        v.pop("E")
    ratio = float(np.mean(its["cg"]) / np.mean(its["learned"]))
    # what any diag + rank-16 preconditioner of this form can gain at these points, and whether the
    # training set pins down the part that gains (exact metrics of the held-out points, their
    # nearest training points, random points and perturbed points)
    from quantum_geometric_tensor_gb300 import precond_limits as PL
    t0 = time.perf_counter()
    limits = PL.analyse(lambda t_: Q.metric_dataset(n, g, t_, precision=Q.MIXED), th, th_h, lam=1e-3, r=16,
                        learned=(d, U))
    limits["seconds"] = time.perf_counter() - t0
    pc.close()
    _line("PCG iteration reduction, learned vs unpreconditioned (16q, P=192, held-out points)", ratio, "x",
          1, 0, 0.0,
          {"workload": "hea16_L6_cnot_P192_learned_precond", "samples": S, "width": 512, "rank": 16},
          {"dtype": "bf16-weights/f32-acc; f64 PCG",
           "heldout_pcg_iters_mean": {k: float(np.mean(v)) for k, v in its.items()},
           "train_s": t_train, "loss_first": float(hist[0]), "loss_last": float(hist[-1]),
           "vqe_500": vqe, "vqe_max_abs_dE_learned_vs_cholesky": dE, "vqe_max_abs_dE_cg_vs_cholesky": dE_cg,
           "vqe_final_abs_dE_vs_cholesky": dE_final, "limits": limits})


def C_byref(x):
    import ctypes
    return ctypes.byref(x)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU comparison")
    ap.add_argument("--qubits", type=int, default=N_QUBITS, help="smaller register for profiling captures")
    ap.add_argument("--layers", type=int, default=LAYERS)
    ap.add_argument("--workload", default="hea20", choices=["hea20", "ragged1024", "hea26", "learned16"],
                    help="hea20: the headline step; the others reproduce the batch, 26-qubit and "
                         "learned-preconditioner measurements")
    ap.add_argument("--tune-cache", default="",
                    help="ragged1024: measure each structural group's plan configuration and keep the "
                         "choices in this text file (qgt_batch_options_t.tune_cache)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if args.workload == "ragged1024":
        return run_ragged(args)
    if args.workload == "hea26":
        return run_hea26(args)
    if args.workload == "learned16":
        return run_learned(args)
    return run_gb300(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
