"""Benchmark of the GB300 finite-volume hot path.

Workload (the configuration the headline metric is quoted on): implicit heat
transfer  ddt(T) - laplacian(k, T) = 0  on a 128^3 hex box (2,097,152 cells,
6,242,304 internal faces) with interior vertices jittered by +-10% of the
spacing (seed 12345), per-cell lognormal conductivity k (mu 0, sigma 0.5,
same seed stream; face conductivity by linear interpolation), T0 = 300, a
fixed 400 wall at x = 0, zero-gradient elsewhere, implicit Euler dt = 0.01.
One step = CSR assembly of the system + FP64 Jacobi-PCG to a 1e-8 relative
residual + boundary update, i.e. the reference's heatTransfer time step.

metric: face-updates/s = (internal faces + active boundary faces) * steps / s.
Inputs are synthetic (seeded), resident in HBM for `value`; `e2e` adds the
host->device copy of T and the device->host copy of the result every step.
Multi-GPU: independent replicas (the path has no data-parallel exchange).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HEAT = dict(n=128, jitter=0.1, seed=12345, dt=0.01, sigma=0.5, T0=300.0, Twall=400.0, rel_tol=1e-8)


def heat_inputs(n, oracle_mesh=False):
    """The 128^3 (or n^3) jittered box and its lognormal conductivity.  With
    oracle_mesh the arrays come from the oracle's own box builder (the same
    bits), so a CPU-only leg never loads the GPU library."""
    if oracle_mesh:
        from oracle import build_oracle
        from oracle.pyoracle import BoxMesh

        build_oracle.build()
        hm = BoxMesh(n, n, n, jitter=HEAT["jitter"], seed=HEAT["seed"])
    else:
        from foamadapter_gb300 import mesh

        hm = mesh.box(n, n, n, jitter=HEAT["jitter"], seed=HEAT["seed"])
    rng = np.random.default_rng(HEAT["seed"])
    k = np.exp(HEAT["sigma"] * rng.standard_normal(hm.n))
    return hm, k


def active_bfaces(hm):
    s = hm.patch_slice("xmin")
    return s.stop - s.start


def alg_bytes(hm):
    n, nnz, nif = hm.n, hm.nnz, hm.nif
    nbfa = active_bfaces(hm)
    return {
        "pcg_spmv": 12 * nnz + 4 * (n + 1) + 16 * n,
        "pcg_update": 56 * n,
        "pcg_dir": 32 * n,
        "pcg_iteration": 12 * nnz + 4 * (n + 1) + 104 * n,
        "assembly": 8 * nnz + 24 * nif + 28 * n + 28 * nbfa,
    }


def aggregate_replicas(local_ms: float, local_e2e_ms: float, local_units: float, device=None):
    """Replicas-only scaling: every rank runs its own copy of the workload; the
    job time is the maximum over ranks, the units are summed.  Returns
    (ms, e2e_ms, units) on every rank (plain values when not distributed)."""
    import torch

    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return local_ms, local_e2e_ms, local_units
    t = torch.tensor([local_ms, local_e2e_ms], dtype=torch.float64, device=device)
    u = torch.tensor([local_units], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(u, op=torch.distributed.ReduceOp.SUM)
    return float(t[0]), float(t[1]), float(u[0])


def fp64_issue_peak():
    """FP64 lanes per second: 2 per clock per SM (ncu's peak_sustained of the DFMA
    counter on GB300) x SMs x the maximum SM clock of MEASURED_PEAKS.json."""
    import torch

    mhz = 2070.0
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        mhz = float(json.loads(p.read_text()).get("sm_max_mhz", mhz))
    return 2.0 * torch.cuda.get_device_properties(0).multi_processor_count * mhz * 1e6


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# ----------------------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world):
    import torch

    from foamadapter_gb300 import abi, neon
    from foamadapter_gb300.mesh import DeviceMesh

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    n = args.n
    hm, k = heat_inputs(n)
    dm = DeviceMesh(hm)
    nbfa = active_bfaces(hm)
    face_updates = hm.nif + nbfa
    bcs = [("fixedValue", HEAT["Twall"])] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T = neon.VolumeField(dm, np.full(hm.n, HEAT["T0"]), bcs)
    kf = neon.VolumeField(dm, k, [("zeroGradient", 0.0)] * hm.npatch)
    gamma = neon.SurfaceInterpolation(dm, "linear").interpolate(kf)
    T_old = T.internal.clone()
    ls = neon.LinearSystem(dm)
    terms = [neon.ddt(T_old), neon.laplacian(gamma, -1.0)]
    tarr = (abi.Term * 2)(*[t.struct() for t in terms])
    bc = T.bc_struct()
    L = abi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cfg = abi.SolverCfg(HEAT["rel_tol"], 0.0, 1000, abi.PREC_FP64, 0.0, 0, 0)
    stats_dev = torch.zeros((max(args.steps, args.warmup) + 8) * 8, dtype=torch.int32, device="cuda")
    SZ = C.sizeof(abi.SolverStats)

    def step(i, cfg=cfg):
        T_old.copy_(T.internal)
        abi.check(L.fvgb_assemble(ls.handle, tarr, 2, HEAT["dt"], C.byref(bc), abi.ptr(T.boundary), stream))
        abi.check(L.fvgb_solve_async(ls.handle, abi.ptr(T.internal), C.byref(cfg),
                                     stats_dev.data_ptr() + i * SZ, stream))
        abi.check(L.fvgb_bc_correct(dm.handle, 1, C.byref(bc), abi.ptr(T.internal), abi.ptr(T.boundary),
                                    stream))

    def read_stats(count):
        raw = stats_dev[: count * SZ // 4].cpu().numpy().tobytes()
        return [abi.SolverStats.from_buffer_copy(raw[i * SZ:(i + 1) * SZ]) for i in range(count)]

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    warm_stats = read_stats(args.warmup)
    # ---- device-resident timed region
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        ev0.record()
        for i in range(args.steps):
            step(i)
        ev1.record()
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    stats = read_stats(args.steps)
    assert all(s.status == abi.OK for s in stats), [s.status for s in stats]
    iters = [s.num_iter for s in stats]
    if args.profile:
        # the same kernels outside the graph, where ncu can capture them one by one
        kt = (C.c_double * 4)()
        abi.check(L.fvgb_solve_kernel_times(ls.handle, abi.ptr(T.internal), 3, kt, stream))
        return hm, dict(ms=ms, iters=iters)
    # ---- end to end through the ABI with host buffers (pinned), copies inside the region
    h_in = torch.empty(hm.n, dtype=torch.float64, pin_memory=True)
    h_out = torch.empty(hm.n, dtype=torch.float64, pin_memory=True)
    h_in.copy_(T.internal.cpu())
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(args.steps):
        T.internal.copy_(h_in, non_blocking=True)
        step(i)
        h_out.copy_(T.internal, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_iters = [s.num_iter for s in read_stats(args.steps)]
    # every e2e step started from h_in: h_out and the last step's iteration count are
    # what the CPU oracle must reproduce from the same state
    step_in, step_out = h_in.numpy().copy(), h_out.numpy().copy()
    # ---- per-kernel times for the roofline (outside the graph, same system)
    kt = (C.c_double * 4)()
    abi.check(L.fvgb_solve_kernel_times(ls.handle, abi.ptr(T.internal), 30, kt, stream))
    # ---- FP64 vs mixed-precision solve of one step's system
    mixed = compare_precisions(torch, abi, L, ls, T, T_old, tarr, bc, dm, hm, stream)
    # ---- the autotuner's choices for this system (timed at its first solve)
    chosen, tms = (C.c_int32 * 4)(), (C.c_float * 16)()
    abi.check(L.fvgb_solve_tuning(ls.handle, None, chosen, tms))
    kinds = ["fp64_spmv", "fp64_update", "fp32_spmv", "fp32_update"]
    tuning = {k: {"min_blocks_per_sm": int(chosen[i]),
                  "ms_by_min_blocks": {str(b): round(float(tms[4 * i + j]), 5) for j, b in enumerate((2, 4, 6, 8))}}
              for i, k in enumerate(kinds)}
    result = dict(ms=ms, iters=iters, e2e_ms=e2e_ms, e2e_iters=e2e_iters, kt=list(kt), clocks=clk.summary(),
                  mixed=mixed, face_updates=face_updates, warm_iters=[s.num_iter for s in warm_stats],
                  mesh_bytes=dm.device_bytes(), tuning=tuning, step_in=step_in, step_out=step_out)
    return hm, result


def compare_precisions(torch, abi, L, ls, T, T_old, tarr, bc, dm, hm, stream):
    """Solve one step's system both ways from the same start; time, iterations, error."""
    T_old.copy_(T.internal)
    abi.check(L.fvgb_assemble(ls.handle, tarr, 2, HEAT["dt"], C.byref(bc), abi.ptr(T.boundary), stream))
    out = {}
    sols = {}
    for name, prec, inner in (("fp64", abi.PREC_FP64, 0.0), ("mixed", abi.PREC_MIXED_IR, 0.1)):
        cfg = abi.SolverCfg(HEAT["rel_tol"], 0.0, 4000, prec, inner, 1000, 50)
        best = None
        for rep in range(3):
            x = T_old.clone()
            st = abi.SolverStats()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            abi.check(L.fvgb_solve(ls.handle, abi.ptr(x), C.byref(cfg), C.byref(st), stream))
            e1.record()
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1)
            best = t if best is None else min(best, t)
        sols[name] = x
        # true FP64 residual of the returned solution
        r = torch.empty_like(x)
        abi.check(L.fvgb_apply_operator(ls.handle, abi.ptr(x), abi.ptr(r), stream))
        out[name] = {"ms": best, "iters": st.num_iter, "outer": st.num_outer,
                     "rel_residual": float(torch.linalg.vector_norm(r).item() / st.init_res_norm)}
    # FP64 CG with the multigrid preconditioner (Ginkgo Multigrid + PGM as the
    # reference's cylinder2D configuration selects it): first solve with the
    # setup, then best of 3 with the hierarchy cached, then after a
    # re-assembly (coarse values recomputed on the device)
    cfg = abi.SolverCfg(HEAT["rel_tol"], 0.0, 4000, abi.PREC_FP64, 0.0, 0, 0, 0, 0, abi.SOLVER_CG,
                        abi.PRECOND_MULTIGRID)
    times = []
    for rep in range(5):
        if rep == 4:
            abi.check(L.fvgb_assemble(ls.handle, tarr, 2, HEAT["dt"], C.byref(bc), abi.ptr(T.boundary), stream))
        x = T_old.clone()
        st = abi.SolverStats()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        abi.check(L.fvgb_solve(ls.handle, abi.ptr(x), C.byref(cfg), C.byref(st), stream))
        torch.cuda.synchronize()
        times.append(1e3 * (time.perf_counter() - t0))
    r = torch.empty_like(x)
    abi.check(L.fvgb_apply_operator(ls.handle, abi.ptr(x), abi.ptr(r), stream))
    nl = C.c_int32()
    rows = (C.c_int32 * 32)()
    abi.check(L.fvgb_amg_info(ls.handle, C.byref(nl), rows, None, 32))
    # the same with the V-cycle in FP32 inside the FP64 CG (mixed precision)
    cfg32 = abi.SolverCfg(HEAT["rel_tol"], 0.0, 4000, abi.PREC_MIXED_IR, 0.1, 1000, 50, 0, 0, abi.SOLVER_CG,
                          abi.PRECOND_MULTIGRID)
    t32 = []
    for rep in range(4):
        x32 = T_old.clone()
        st32 = abi.SolverStats()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        abi.check(L.fvgb_solve(ls.handle, abi.ptr(x32), C.byref(cfg32), C.byref(st32), stream))
        torch.cuda.synchronize()
        t32.append(1e3 * (time.perf_counter() - t0))
    r32 = torch.empty_like(x32)
    abi.check(L.fvgb_apply_operator(ls.handle, abi.ptr(x32), abi.ptr(r32), stream))
    out["multigrid_fp32_vcycle"] = {"ms": min(t32[1:]), "iters": st32.num_iter,
                                    "rel_residual": float(torch.linalg.vector_norm(r32).item() / st32.init_res_norm),
                                    "max_abs_err_vs_fp64": float((x32 - sols["fp64"]).abs().max().item()),
                                    "speedup_vs_fp64_jacobi": out["fp64"]["ms"] / min(t32[1:])}
    out["fp64_multigrid"] = {"ms": min(times[1:4]), "first_solve_ms_with_setup": times[0],
                             "solve_after_reassembly_ms": times[4], "iters": st.num_iter,
                             "levels": [int(rows[i]) for i in range(nl.value)],
                             "rel_residual": float(torch.linalg.vector_norm(r).item() / st.init_res_norm),
                             "max_abs_err_vs_fp64": float((x - sols["fp64"]).abs().max().item()),
                             "speedup_vs_fp64_jacobi": out["fp64"]["ms"] / min(times[1:4])}
    d = (sols["mixed"] - sols["fp64"]).abs()
    out["speedup"] = out["fp64"]["ms"] / out["mixed"]["ms"]
    out["max_abs_err_vs_fp64"] = float(d.max().item())
    out["l2_rel_err_vs_fp64"] = float((torch.linalg.vector_norm(sols["mixed"] - sols["fp64"]) /
                                       torch.linalg.vector_norm(sols["fp64"])).item())
    return out


# ----------------------------------------------------------------------------- CPU (oracle)
def cpu_steps(hm, k, nsteps, threads, T_start=None, first_only=False):
    """The same heat-transfer steps on the host cores with the CPU oracle, from
    T0 or from T_start.  Returns the step times, iteration counts, threads and
    the field after the first step."""
    from oracle import build_oracle
    from oracle.pyoracle import Oracle, get_threads, set_threads

    build_oracle.build()
    if threads:
        set_threads(threads)
    o = Oracle(hm)
    o.csr()
    nbf = hm.nbf
    kb = np.ascontiguousarray(k[hm.bcells])
    gamma = o.interp_linear(1, k, kb)
    types = np.asarray([1] + [2] * (hm.npatch - 1), np.int32)
    ref = np.zeros(nbf)
    ref[hm.patch_slice("xmin")] = HEAT["Twall"]
    T = np.full(hm.n, HEAT["T0"]) if T_start is None else np.array(T_start, dtype=np.float64)
    Tb = np.zeros(nbf)
    o.bc_correct(1, types, ref, T, Tb)
    times, iters, first = [], [], None
    for _ in range(nsteps):
        t0 = time.perf_counter()
        told = T.copy()
        terms = [(0, 0, 1.0, told, None), (1, 0, -1.0, None, gamma)]
        v, r, _, _ = o.assemble(1, terms, HEAT["dt"], types, ref, Tb)
        st = o.solve(v, r, T, rel_tol=HEAT["rel_tol"], max_iter=1000)
        o.bc_correct(1, types, ref, T, Tb)
        times.append(time.perf_counter() - t0)
        iters.append(st.num_iter)
        if first is None:
            first = T.copy()
    return times, iters, get_threads(), first


def run_reference(args, rank, world):
    """--impl reference: the oracle port of the reference's CPU path, all host threads."""
    if rank != 0:
        return
    hm, k = heat_inputs(args.n, oracle_mesh=True)
    nbfa = active_bfaces(hm)
    # the GPU arm's own step sequence: W untimed steps from T0, then K timed ones
    w = max(0, args.warmup)
    ksteps = max(1, min(args.steps, args.ref_max_steps))
    times, iters, threads, _ = cpu_steps(hm, k, w + ksteps, os.cpu_count())
    t = sum(times[w:])
    val = (hm.nif + nbfa) * ksteps / t
    line = {
        "impl": "reference", "metric": "face-updates/s", "value": val, "unit": "face-updates/s",
        "n_gpus": world, "steps": ksteps, "warmup": w, "ms_per_step": 1e3 * t / ksteps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(args),
        "cpu_baseline": {"value": val, "unit": "face-updates/s", "cores": threads, "kind": "port",
                         "sample": f"steps {w + 1}-{w + ksteps} of the {args.n}^3 case from T0 (assembly + FP64 "
                                   f"Jacobi-PCG to 1e-8, iterations {iters[w:]}), OpenMP x{threads}"},
        "e2e": {"value": val, "unit": "face-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ----------------------------------------------------------------------------- other workloads
def run_advection(args):
    """Explicit upwind advection, 64x64x1, 100 forward-Euler steps, vs the oracle bit for bit."""
    import torch

    from foamadapter_gb300 import apps
    from oracle.pyoracle import Oracle

    case = apps.Advection(n=64)
    hm = case.hm
    T0 = case.T.host().copy()
    Tb0 = case.T.boundary.cpu().numpy()[:hm.nbf].copy()
    nsteps = 100

    def reset():
        case.T.internal.copy_(torch.as_tensor(T0).cuda())
        case.T.boundary[:hm.nbf].copy_(torch.as_tensor(Tb0).cuda())
        torch.cuda.synchronize()

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # one call per step (the reference's loop calling the operator each step)
    for _ in range(5):                      # warm-up on a copy of the state
        case.step()
    reset()
    e0.record()
    for _ in range(nsteps):
        case.step()
    e1.record()
    torch.cuda.synchronize()
    ms_per_call = e0.elapsed_time(e1)
    per_call_T = case.T.host().copy()
    # the whole loop in one call (fvgb_advect_euler_steps: one single-block kernel)
    case.run(5)
    reset()
    e0.record()
    case.run(nsteps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    assert np.array_equal(case.T.host(), per_call_T)
    o = Oracle(hm)
    types = np.full(hm.npatch, 2, np.int32)
    T, Tb = T0.copy(), Tb0.copy()
    t0 = time.perf_counter()
    for _ in range(nsteps):
        T, Tb = o.advect_euler(case.flux.host(), T, Tb, case.dt, types, np.zeros(hm.nbf))
    cpu_s = time.perf_counter() - t0
    fu = (hm.nif + hm.nbf) * nsteps
    return {"workload": "advection 64x64x1 upwind forward Euler, 100 steps", "metric": "face-updates/s",
            "value": fu / (ms / 1e3), "us_per_step": 1e3 * ms / nsteps,
            "one_call_per_step": {"value": fu / (ms_per_call / 1e3), "us_per_step": 1e3 * ms_per_call / nsteps},
            "bit_exact_vs_oracle": bool(np.array_equal(case.T.host(), T)),
            "cpu_baseline": {"value": fu / cpu_s, "cores": 1, "kind": "port", "sample": "100 steps, serial"}}


def run_explicit(args, hm=None, dm=None):
    """Every explicit operator once per launch on the 128^3 jittered box, each launch
    timed alone with CUDA events after an L2 flush, against the HBM roofline and
    GB300's FP64 issue rate.  Algorithmic bytes: int32 labels, every listed array
    once at its width.  Each operator's floor is the larger of its bytes at the
    measured HBM bandwidth and its FP64 operations at the FP64 issue rate."""
    import torch

    from foamadapter_gb300 import abi, neon
    from foamadapter_gb300.mesh import DeviceMesh

    if hm is None:
        hm, k = heat_inputs(args.explicit_n)
    if dm is None:
        dm = DeviceMesh(hm)
    n, nif, nbf = hm.n, hm.nif, hm.nbf
    nbfa = active_bfaces(hm)
    rng = np.random.default_rng(7)
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T = neon.VolumeField(dm, 300.0 + rng.standard_normal(n), bcs)
    F = neon.dev(rng.standard_normal(nif + nbf))
    gamma = neon.dev(np.exp(rng.standard_normal(nif + nbf)))
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    out3 = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    fout = torch.zeros(nif + nbf, dtype=torch.float64, device="cuda")
    T2 = torch.empty_like(T.internal)
    Tb2 = torch.empty_like(T.boundary)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    L, h, s = abi.lib(), dm.handle, torch.cuda.current_stream().cuda_stream
    P = abi.ptr
    bc = T.bc_struct()
    # the face-pass tile (faces per thread) by the autotuner, cached per mesh shape
    tile, tile_ms = C.c_int32(), (C.c_float * 3)()
    abi.check(L.fvgb_explicit_tune(h, s, C.byref(tile), tile_ms))
    face_tile = {"chosen": tile.value, "ms_grad_plus_div_upwind_face_passes": dict(zip(("2", "4", "8"),
                                                                                      [round(x, 5) for x in tile_ms]))}
    # FP64 operations of the reference's face loop (each face's value and flux formed
    # once, added to the owner and subtracted from the neighbour, then the 1/V scale)
    fp64 = {"interp_linear": 3 * nif, "interp_upwind": 0, "div_upwind": 3 * nif + 2 * nbf + 2 * n,
            "div_linear": 6 * nif + 2 * nbf + 2 * n, "grad": 12 * nif + 6 * nbf + 6 * n,
            "laplacian": 5 * nif + 4 * nbf + 2 * n, "sngrad": 2 * (nif + nbf),
            "laplacian_corrected": 28 * nif + 10 * nbf + 8 * n,  # gradient 12, fused face pass 14, gather 2
            "advect_euler": 3 * nif + 2 * nbf + 4 * n}
    sm_mhz = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("sm_max_mhz", 2070.0) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else 2070.0
    fp64_peak = 2 * torch.cuda.get_device_properties(0).multi_processor_count * sm_mhz * 1e6
    ops = {
        "interp_linear": (lambda: L.fvgb_interp_linear(h, 1, P(T.internal), P(T.boundary), P(fout), s),
                          24 * nif + 8 * n + 16 * nbf),
        "interp_upwind": (lambda: L.fvgb_interp_upwind(h, 1, P(F), P(T.internal), P(T.boundary), P(fout), s),
                          24 * nif + 8 * n + 24 * nbf),
        "div_upwind": (lambda: L.fvgb_div_explicit(h, 1, 1, P(F), P(T.internal), P(T.boundary), 1.0, P(out), s),
                       16 * nif + 20 * nbf + 32 * n),
        "div_linear": (lambda: L.fvgb_div_explicit(h, 0, 1, P(F), P(T.internal), P(T.boundary), 1.0, P(out), s),
                       24 * nif + 20 * nbf + 32 * n),
        "grad": (lambda: L.fvgb_grad(h, P(T.internal), P(T.boundary), 1.0, P(out3), s),
                 40 * nif + 36 * nbf + 40 * n),
        "laplacian": (lambda: L.fvgb_laplacian_explicit(h, 1, P(gamma), P(T.internal), P(T.boundary), 1.0, P(out), s),
                      24 * nif + 28 * nbfa + 24 * n),
        "sngrad": (lambda: L.fvgb_sngrad(h, P(T.internal), P(T.boundary), P(fout), s),
                   24 * nif + 8 * n + 28 * nbf),
        # Gauss linear corrected: the laplacian's arrays, the gradient's (Sf, w, Sf_b, T_b),
        # the correction vectors and |Sf|, and the cell gradient written and read once
        "laplacian_corrected": (lambda: L.fvgb_laplacian_explicit_corrected(h, 1, P(gamma), P(T.internal),
                                                                           P(T.boundary), 1.0, P(out), s),
                                88 * nif + 28 * nbfa + 32 * nbf + 72 * n),
        "advect_euler": (lambda: L.fvgb_advect_euler_step(h, P(F), P(T.internal), P(T.boundary), 1e-3, C.byref(bc),
                                                          P(T2), P(Tb2), s),
                         16 * nif + 12 * nbfa + 24 * n),
    }
    peak, peak_kind = load_peaks()
    res = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    only = [o for o in args.explicit_ops.split(",") if o] if args.explicit_ops else list(ops)
    for name, (fn, nbytes) in ops.items():
        if name not in only:
            continue
        for _ in range(3):
            abi.check(fn())
        times = []
        for _ in range(args.explicit_reps):
            # the reference's benchmark fills its output with 0 before every
            # call (bench_explicitOperators.cpp, "No allocation"); here too,
            # before the flush and outside the timed region
            out.zero_()
            out3.zero_()
            flush.fill_(1.0)
            e0.record()
            abi.check(fn())
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        us = 1e3 * float(np.median(times))
        gbs = nbytes / (us * 1e-6) / 1e9
        floor_us = 1e6 * max(nbytes / (peak * 1e9), fp64[name] / fp64_peak)
        res[name] = {"us": us, "alg_bytes": nbytes, "GBps": gbs, "frac_of_peak": gbs / peak,
                     "fp64_ops": fp64[name], "fp64_frac_of_peak": fp64[name] / (us * 1e-6) / fp64_peak,
                     "floor_us": floor_us, "bound": "hbm" if nbytes / (peak * 1e9) >= fp64[name] / fp64_peak
                     else "fp64", "frac_of_floor": floor_us / us}
    return {"workload": f"explicit operators, {round(hm.n ** (1 / 3))}^3 jittered box, one launch each, L2 flushed",
            "n": n, "n_ifaces": nif, "n_bfaces": nbf, "peak_GBps": peak, "peak_source": peak_kind,
            "fp64_peak_ops_per_s": fp64_peak,
            "fp64_peak_source": "2 FP64 lanes per clock per SM (ncu peak_sustained) x SMs x max SM clock",
            "timing": "median of CUDA-event times of single launches on zeroed outputs (as the reference's "
                      "benchmark fills its field with 0 before each call), 512 MB written between launches",
            "face_tile": face_tile, "ops": res}


def run_convection(args):
    """One implicit step of ddt(T) + div(F, T) - laplacian(1e-3, T) = 0 (upwind, a
    nonsymmetric system) on the 128^3 jittered box, U = (1, 0.4, -0.2), Courant 2,
    solved to 1e-8 by BiCGStab in FP64 and in mixed precision from the same start."""
    import torch

    from foamadapter_gb300 import abi, neon
    from foamadapter_gb300.mesh import DeviceMesh

    hm, _ = heat_inputs(args.explicit_n)
    dm = DeviceMesh(hm)
    L, s, P = abi.lib(), torch.cuda.current_stream().cuda_stream, abi.ptr
    U = np.array([1.0, 0.4, -0.2])
    Uc, Ub = neon.dev(np.tile(U, hm.n)), neon.dev(np.tile(U, hm.nbf))
    F = neon.SurfaceField(dm)
    abi.check(L.fvgb_flux_vec(dm.handle, P(Uc), P(Ub), P(F.values), s))
    rng = np.random.default_rng(11)
    T = neon.VolumeField(dm, rng.random(hm.n), [("fixedValue", 1.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1))
    T_old = T.internal.clone()
    dt = 2.0 / args.explicit_n / float(np.linalg.norm(U))
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T_old), neon.div(F, "upwind"),
                 neon.laplacian(neon.SurfaceField(dm, np.full(hm.nif + hm.nbf, 1e-3)), -1.0)], dt, T)
    out, sols = {}, {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    runs = [("fp64", abi.PREC_FP64, 0.1, abi.PRECOND_JACOBI)] + \
        [(f"mixed_inner_{t:g}", abi.PREC_MIXED_IR, t, abi.PRECOND_JACOBI) for t in (0.1, 0.03, 1e-2, 1e-3)] + \
        [("fp64_ilu", abi.PREC_FP64, 0.1, abi.PRECOND_ILU)]
    for name, prec, inner, pc in runs:
        cfg = abi.SolverCfg(1e-8, 0.0, 5000, prec, inner, 1000, 50, 0, 0, abi.SOLVER_BICGSTAB, pc)
        times = []
        for rep in range(4):                               # the first builds the graph
            x = T_old.clone()
            st = abi.SolverStats()
            torch.cuda.synchronize()
            e0.record()
            abi.check(L.fvgb_solve(ls.handle, P(x), C.byref(cfg), C.byref(st), s))
            e1.record()
            torch.cuda.synchronize()
            if rep:
                times.append(e0.elapsed_time(e1))
        sols[name] = x
        r = torch.empty_like(x)
        abi.check(L.fvgb_apply_operator(ls.handle, P(x), P(r), s))
        out[name] = {"ms": float(np.median(times)), "iters": st.num_iter, "outer": st.num_outer,
                     "status": st.status,
                     "rel_residual": float(torch.linalg.vector_norm(r).item() / st.init_res_norm)}
    best = min((k for k in out if k.startswith("mixed_inner_")), key=lambda k: out[k]["ms"])
    out["mixed"] = dict(out[best], inner_rel_tol=float(best.split("_")[-1]))
    sols["mixed"] = sols[best]
    d = sols["mixed"] - sols["fp64"]
    out["speedup"] = out["fp64"]["ms"] / out["mixed"]["ms"]
    out["max_abs_err_vs_fp64"] = float(d.abs().max().item())
    out["l2_rel_err_vs_fp64"] = float((torch.linalg.vector_norm(d) / torch.linalg.vector_norm(sols["fp64"])).item())
    return {"workload": f"implicit upwind convection-diffusion, {args.explicit_n}^3 jittered box, Courant 2, "
                        "BiCGStab + Jacobi to 1e-8", "n": hm.n, "dt": dt, **out}


def run_cavity(args, multigrid=True):
    """Lid-driven cavity PISO on 512x512x1: FP64 vs mixed-precision pressure solve
    (and the multigrid CG with FP64 and FP32 V-cycles)."""
    import torch

    from foamadapter_gb300 import abi, apps

    nsteps = args.cavity_steps
    out = {}
    fields = {}
    legs = [("fp64", abi.PREC_FP64, abi.PRECOND_JACOBI), ("mixed", abi.PREC_MIXED_IR, abi.PRECOND_JACOBI)]
    if multigrid:
        legs += [("fp64_multigrid", abi.PREC_FP64, abi.PRECOND_MULTIGRID),
                 ("multigrid_fp32_vcycle", abi.PREC_MIXED_IR, abi.PRECOND_MULTIGRID)]
    for name, prec, pc in legs:
        case = apps.CavityPiso(n=512, precision=prec, preconditioner=pc)
        case.step()                                     # warm-up (builds the solver graphs)
        torch.cuda.synchronize()
        case = apps.CavityPiso(n=512, precision=prec, preconditioner=pc)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(nsteps):
            case.step()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        its = [s[0] for s in case.stats]
        out[name] = {"ms_per_step": ms / nsteps, "pressure_iters_mean": float(np.mean(its)),
                     "all_solves_ok": all(s[4] == abi.OK for s in case.stats),
                     "max_final_rel_residual": max(s[3] / s[2] if s[2] > 0 else 0.0 for s in case.stats)}
        fields[name] = (case.p.host(), case.U.host())
    (p64, U64), (pm, Um) = fields["fp64"], fields["mixed"]

    def err(p, U):
        return {"p_max": float(np.abs(p - p64).max()),
                "p_l2_rel": float(np.linalg.norm(p - p64) / max(np.linalg.norm(p64), 1e-300)),
                "U_max": float(np.abs(U - U64).max()),
                "U_l2_rel": float(np.linalg.norm(U - U64) / max(np.linalg.norm(U64), 1e-300))}

    out["speedup_step"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    out["err_vs_fp64"] = err(pm, Um)
    if not multigrid:
        return {"workload": f"lid-driven cavity PISO 512x512x1, +-5% jitter, dt 5e-4, 2 correctors, {nsteps} steps",
                "pressure_solve_to": "1e-8 relative FP64 residual", **out}
    pg, Ug = fields["fp64_multigrid"]
    out["speedup_step_multigrid"] = out["fp64"]["ms_per_step"] / out["fp64_multigrid"]["ms_per_step"]
    out["err_vs_fp64_multigrid"] = err(pg, Ug)
    out["speedup_step_multigrid_fp32_vcycle"] = out["fp64"]["ms_per_step"] / out["multigrid_fp32_vcycle"]["ms_per_step"]
    out["err_vs_fp64_multigrid_fp32_vcycle"] = err(*fields["multigrid_fp32_vcycle"])
    return {"workload": f"lid-driven cavity PISO 512x512x1, +-5% jitter, dt 5e-4, 2 correctors, {nsteps} steps",
            "pressure_solve_to": "1e-8 relative FP64 residual", **out}


def run_multigrid(args):
    """The multigrid preconditioner on the 128^3 heat system: the hierarchy,
    one V-cycle (fvgb_amg_apply, a plain graph whose kernels ncu can capture
    one by one) and the whole CG solve against the Jacobi-PCG."""
    import torch

    from foamadapter_gb300 import abi, neon
    from foamadapter_gb300.mesh import DeviceMesh

    hm, k = heat_inputs(args.n)
    dm = DeviceMesh(hm)
    bcs = [("fixedValue", HEAT["Twall"])] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T = neon.VolumeField(dm, np.full(hm.n, HEAT["T0"]), bcs)
    kf = neon.VolumeField(dm, k, [("zeroGradient", 0.0)] * hm.npatch)
    gamma = neon.SurfaceInterpolation(dm, "linear").interpolate(kf)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gamma, -1.0)], HEAT["dt"], T)
    L = abi.lib()
    x0 = T.internal.clone()
    out = {}
    # --profile: the V-cycles only (no conditional graphs, so ncu can capture every kernel)
    legs = (("jacobi", abi.PRECOND_JACOBI, abi.PREC_FP64, abi.SOLVER_CG),
            ("multigrid", abi.PRECOND_MULTIGRID, abi.PREC_FP64, abi.SOLVER_CG),
            ("multigrid_fp32_vcycle", abi.PRECOND_MULTIGRID, abi.PREC_MIXED_IR, abi.SOLVER_CG),
            ("multigrid_solver", abi.PRECOND_JACOBI, abi.PREC_FP64, abi.SOLVER_MULTIGRID),
            ("multigrid_solver_fp32_vcycle", abi.PRECOND_JACOBI, abi.PREC_MIXED_IR, abi.SOLVER_MULTIGRID),
            ("ilu_cg", abi.PRECOND_ILU, abi.PREC_FP64, abi.SOLVER_CG))
    for name, pc, prec, method in () if args.profile else legs:
        times = []
        for rep in range(4):
            x = x0.clone()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = ls.solve(x, rel_tol=HEAT["rel_tol"], max_iter=4000, preconditioner=pc, precision=prec,
                          method=method)
            torch.cuda.synchronize()
            times.append(1e3 * (time.perf_counter() - t0))
        out[name] = {"ms": min(times[1:]), "first_ms": times[0], "iters": st.num_iter, "status": st.status}
    r = torch.randn(hm.n, dtype=torch.float64, device="cuda")
    z = torch.zeros_like(r)
    reps = args.explicit_reps
    for _ in range(2):
        abi.check(L.fvgb_amg_apply(ls.handle, abi.ptr(r), abi.ptr(z), None))
    t0 = time.perf_counter()
    for _ in range(reps):
        abi.check(L.fvgb_amg_apply(ls.handle, abi.ptr(r), abi.ptr(z), None))
    vms = 1e3 * (time.perf_counter() - t0) / max(1, reps)
    nl = C.c_int32()
    rows, nnz = (C.c_int32 * 32)(), (C.c_int64 * 32)()
    abi.check(L.fvgb_amg_info(ls.handle, C.byref(nl), rows, nnz, 32))
    return {"workload": f"multigrid-preconditioned CG on the {args.n}^3 heat system, to 1e-8",
            "levels": [[int(rows[i]), int(nnz[i])] for i in range(nl.value)],
            "vcycle_ms_incl_graph_build": vms, **out,
            "speedup_solve": out["jacobi"]["ms"] / out["multigrid"]["ms"] if out else None,
            "speedup_solve_fp32_vcycle": out["jacobi"]["ms"] / out["multigrid_fp32_vcycle"]["ms"] if out else None}


def batch_cases(ncases, seed=4):
    """512 hex boxes, nx,ny,nz = round(exp(U(ln 16, ln 64))), +-10% jitter, lognormal k (sigma 0.5),
    wall temperature U[350, 450]."""
    from foamadapter_gb300 import mesh

    rng = np.random.default_rng(seed)
    dims = np.rint(np.exp(rng.uniform(np.log(16), np.log(64), size=(ncases, 3)))).astype(int)
    cases = []
    for k, d in enumerate(dims):
        hm = mesh.box(int(d[0]), int(d[1]), int(d[2]), jitter=0.1, seed=seed * 100000 + k)
        cases.append((hm, np.exp(0.5 * rng.standard_normal(hm.n)), float(rng.uniform(350.0, 450.0))))
    return cases


def run_batch(args):
    """One launch per operator for all cases (packed), mixed-precision inner solve,
    against one-at-a-time plain FP64 launches of the same cases."""
    import torch

    from foamadapter_gb300 import abi, mesh, neon
    from foamadapter_gb300.mesh import DeviceMesh

    t0 = time.perf_counter()
    cases = batch_cases(args.cases)
    big, ranges, slices = mesh.concat([c[0] for c in cases])
    setup_s = time.perf_counter() - t0
    dm = DeviceMesh(big)
    ref = np.zeros(big.nbf)
    kap = np.ones(big.n)
    for k, (hm, kk, tw) in enumerate(cases):
        ref[slices[k][0]] = tw
        kap[ranges[2 * k]:ranges[2 * k + 1]] = kk
    xmin = slice(slices[0][0].start, slices[-1][0].stop)
    T = neon.VolumeField(dm, np.full(big.n, 300.0), [("fixedValue", ref[xmin])] + [("zeroGradient", 0.0)] * 5)
    kf = neon.VolumeField(dm, kap, [("zeroGradient", 0.0)] * 6)
    gamma = neon.SurfaceInterpolation(dm, "linear").interpolate(kf)
    T_old = T.internal.clone()
    ls = neon.LinearSystem(dm)
    batch = neon.Batch(ls, ranges)
    L, s = abi.lib(), torch.cuda.current_stream().cuda_stream
    terms = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(T_old), neon.laplacian(gamma, -1.0))])
    bc = T.bc_struct()
    stats_dev = torch.zeros(len(cases) * 8, dtype=torch.int32, device="cuda")

    def packed_step(cfg):
        T_old.copy_(T.internal)
        abi.check(L.fvgb_assemble(ls.handle, terms, 2, 0.01, C.byref(bc), abi.ptr(T.boundary), s))
        abi.check(L.fvgb_batch_solve_async(batch.handle, abi.ptr(T.internal), C.byref(cfg), stats_dev.data_ptr(), s))
        abi.check(L.fvgb_bc_correct(dm.handle, 1, C.byref(bc), abi.ptr(T.internal), abi.ptr(T.boundary), s))

    def timed(fn, nsteps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(nsteps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    out = {"cases": len(cases), "cells_total": int(sum(c[0].n for c in cases)),
           "cells_min_max": [int(min(c[0].n for c in cases)), int(max(c[0].n for c in cases))],
           "host_mesh_build_s": setup_s}
    cfg_mixed = abi.SolverCfg(1e-8, 0.0, 4000, abi.PREC_MIXED_IR, args.inner_tol, 2000, 50)
    cfg_fp64 = abi.SolverCfg(1e-8, 0.0, 4000, abi.PREC_FP64, 0.0, 0, 0)
    for name, cfg in (("packed_mixed", cfg_mixed), ("packed_fp64", cfg_fp64)):
        T.internal.fill_(300.0)
        packed_step(cfg)                                      # warm-up (graph build)
        T.internal.fill_(300.0)
        sec = timed(lambda: packed_step(cfg), args.batch_steps)
        st = stats_dev.cpu().numpy().tobytes()
        stl = [abi.SolverStats.from_buffer_copy(st[i * 32:(i + 1) * 32]) for i in range(len(cases))]
        out[name] = {"case_steps_per_s": len(cases) * args.batch_steps / sec, "s": sec,
                     "all_ok": all(x.status == 0 for x in stl),
                     "iters_last_step_mean": float(np.mean([x.num_iter for x in stl]))}
    # the same packed mixed step as ONE CUDA graph per time step (fvgb_step_*)
    step = C.c_void_p()
    abi.check(L.fvgb_step_create(ls.handle, batch.handle, terms, 2, 0.01, C.byref(bc), abi.ptr(T.internal),
                                 abi.ptr(T.boundary), abi.ptr(T_old), C.byref(cfg_mixed), stats_dev.data_ptr(),
                                 C.byref(step)))
    T.internal.fill_(300.0)
    abi.check(L.fvgb_step_launch(step, s))                    # warm-up
    T.internal.fill_(300.0)
    sec = timed(lambda: abi.check(L.fvgb_step_launch(step, s)), args.batch_steps)
    st = stats_dev.cpu().numpy().tobytes()
    stl = [abi.SolverStats.from_buffer_copy(st[i * 32:(i + 1) * 32]) for i in range(len(cases))]
    out["packed_mixed_step_graph"] = {"case_steps_per_s": len(cases) * args.batch_steps / sec, "s": sec,
                                      "all_ok": all(x.status == 0 for x in stl),
                                      "iters_last_step_mean": float(np.mean([x.num_iter for x in stl]))}
    abi.check(L.fvgb_step_destroy(step))
    # one case at a time, plain FP64 (a sample of cases, every case its own mesh/system/launches)
    sample = cases[:: max(1, len(cases) // args.alone_cases)][: args.alone_cases]
    solo = []
    for hm, kk, tw in sample:
        d1 = DeviceMesh(hm)
        T1 = neon.VolumeField(d1, np.full(hm.n, 300.0), [("fixedValue", tw)] + [("zeroGradient", 0.0)] * 5)
        g1 = neon.SurfaceInterpolation(d1, "linear").interpolate(
            neon.VolumeField(d1, kk, [("zeroGradient", 0.0)] * 6))
        o1 = T1.internal.clone()
        l1 = neon.LinearSystem(d1)
        t1 = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(o1), neon.laplacian(g1, -1.0))])
        b1 = T1.bc_struct()
        solo.append((d1, T1, g1, o1, l1, t1, b1))

    def solo_step(cfg):
        for d1, T1, g1, o1, l1, t1, b1 in solo:
            o1.copy_(T1.internal)
            abi.check(L.fvgb_assemble(l1.handle, t1, 2, 0.01, C.byref(b1), abi.ptr(T1.boundary), s))
            abi.check(L.fvgb_solve_async(l1.handle, abi.ptr(T1.internal), C.byref(cfg), None, s))
            abi.check(L.fvgb_bc_correct(d1.handle, 1, C.byref(b1), abi.ptr(T1.internal), abi.ptr(T1.boundary), s))

    for name, cfg in (("one_at_a_time_fp64", cfg_fp64), ("one_at_a_time_mixed", cfg_mixed)):
        solo_step(cfg)
        for _, T1, *_ in solo:
            T1.internal.fill_(300.0)
        steps = max(1, args.batch_steps // 5)
        sec = timed(lambda: solo_step(cfg), steps)
        out[name] = {"case_steps_per_s": len(solo) * steps / sec, "cases_sampled": len(solo)}
    out["speedup_packed_mixed_vs_one_at_a_time_fp64"] = (out["packed_mixed"]["case_steps_per_s"] /
                                                         out["one_at_a_time_fp64"]["case_steps_per_s"])
    return {"workload": f"{len(cases)} implicit heat-transfer cases, dims logU[16,64], {args.batch_steps} steps",
            **out}


def serve_requests(count, seed=5, rate=200.0):
    """Poisson arrivals (200/s), edges logU[16,160] per axis, |U| in [0.1,2] with a random
    direction, D logU[1e-4,1e-2], 10..200 steps."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    reqs = []
    for k in range(count):
        e = np.rint(np.exp(rng.uniform(np.log(16), np.log(160), size=3))).astype(int)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        U = d * rng.uniform(0.1, 2.0)
        D = float(np.exp(rng.uniform(np.log(1e-4), np.log(1e-2))))
        reqs.append((float(t[k]), int(e[0]), int(e[1]), int(e[2]), int(rng.integers(10, 201)), U, D))
    return reqs


def run_serve(args):
    """Continuous-batching server (mixed precision, the stated configuration, and FP64
    beside it) against one-at-a-time FP64 runs of the same requests: plain launches
    (host-driven CG loop, the reference's launch pattern) and this library's
    single-request path (graph / persistent kernel)."""
    from foamadapter_gb300 import abi

    L = abi.lib()
    reqs = serve_requests(args.requests, rate=args.serve_rate)

    def serve(sample, precision, paced, streams, budget, kernel_mode=0, flags=0, max_active=100000):
        cfg = abi.ServerCfg(int(budget), streams, max_active)
        sv = C.c_void_p()
        abi.check(L.fvgb_server_create(C.byref(cfg), C.byref(sv)))
        buf = (abi.ServeResult * 1024)()
        results, t0 = {}, time.perf_counter()
        keep, ids = [], []
        for (ta, nx, ny, nz, steps, U, D) in sample:
            if paced:
                while time.perf_counter() - t0 < ta:
                    time.sleep(0.0005)
            km = kernel_mode
            if km == -1:  # this library's best single-request path: persistent kernel for small systems
                km = 2 if nx * ny * nz <= (1 << 20) else 1
            req = abi.ServeRequest(nx=nx, ny=ny, nz=nz, steps=steps, U=(C.c_double * 3)(*U), D=D, dt=0.0,
                                   precision=precision, kernel_mode=km, flags=flags, T_out=None)
            rid = C.c_int64()
            abi.check(L.fvgb_server_submit(sv, C.byref(req), C.byref(rid)))
            keep.append(req)
            ids.append(rid.value)
            if not paced:  # sequential: wait for this one before the next
                while rid.value not in results:
                    cnt = C.c_int32()
                    L.fvgb_server_poll(sv, buf, 1024, C.byref(cnt))
                    for i in range(cnt.value):
                        results[buf[i].id] = abi.ServeResult.from_buffer_copy(buf[i])
                    time.sleep(0.0002)
        while len(results) < len(sample):
            cnt = C.c_int32()
            L.fvgb_server_poll(sv, buf, 1024, C.byref(cnt))
            for i in range(cnt.value):
                results[buf[i].id] = abi.ServeResult.from_buffer_copy(buf[i])
            time.sleep(0.001)
        wall = time.perf_counter() - t0
        info = (C.c_int64 * 6)()
        L.fvgb_server_info(sv, info)
        abi.check(L.fvgb_server_destroy(sv))
        r = [results[i] for i in ids]
        lat = np.array([x.finish_s - x.submit_s for x in r])
        failed = [{"request": k, "status": x.status, "steps_done": x.steps_done, "cells": sample[k][1:4],
                   "steps": sample[k][4], "D": sample[k][6], "U": float(np.linalg.norm(sample[k][5]))}
                  for k, x in enumerate(r) if x.status != 0]
        cell_steps = int(sum(x[1] * x[2] * x[3] * x[4] for x in sample))
        return {"requests": len(r), "wall_s": wall, "solves_per_s": len(r) / wall,
                "cell_steps_per_s": cell_steps / wall,
                "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                "all_ok": not failed, "failed": failed[:8], "n_failed": len(failed),
                "peak_device_GB": info[4] / 1e9, "ticks": int(info[5]),
                "total_cg_iters": int(sum(x.total_iters for x in r)),
                "cell_steps": int(sum(x[1] * x[2] * x[3] * x[4] for x in sample))}

    # at most serve_max_active requests resident at once (the rest wait in arrival order): fewer
    # concurrent working sets share the 129 MB L2 better, and early requests finish sooner.
    # The stated configuration serves mixed-precision PCG (the server refines with an inner
    # reduction of 1e-4, the fastest for warm-started solves of ~7 iterations); FP64 beside it
    served_mixed = serve(reqs, abi.PREC_MIXED_IR, True, args.serve_streams, 150e9,
                         max_active=args.serve_max_active)
    served = None if args.serve_mixed_only else serve(reqs, abi.PREC_FP64, True, args.serve_streams, 150e9,
                                                      max_active=args.serve_max_active)
    seq_n = min(args.seq_requests, len(reqs))
    # one at a time as the reference runs a solve: full assembly every step, FP64 CG
    # with a host-driven loop (plain launches)
    plain = serve(reqs[:seq_n], abi.PREC_FP64, False, 1, 150e9, kernel_mode=3, flags=abi.SERVE_REASSEMBLE)
    # one at a time with this library's best single-request path (matrix kept across steps,
    # persistent kernel for small systems, graph otherwise)
    best = serve(reqs[:seq_n], abi.PREC_FP64, False, 1, 150e9, kernel_mode=-1)
    out = {"workload": f"serving: {len(reqs)} Poisson arrivals at {args.serve_rate:g}/s, edges logU[16,160], "
                       "10-200 IMEX steps",
           "served_config": {"streams": args.serve_streams, "max_active": args.serve_max_active,
                             "budget_GB": 150},
           "served_mixed": served_mixed, "served_fp64": served, "sequential_plain_launches_fp64": plain,
           "sequential_best_fp64": best}
    # solves/s ratios, and the same per unit of work (cell-steps/s), which is not biased by how
    # heavy the sequential sample is
    out["mixed_solves_per_s_ratio_vs_plain"] = served_mixed["solves_per_s"] / plain["solves_per_s"]
    out["mixed_work_ratio_vs_plain"] = served_mixed["cell_steps_per_s"] / plain["cell_steps_per_s"]
    out["mixed_solves_per_s_ratio_vs_best_sequential"] = served_mixed["solves_per_s"] / best["solves_per_s"]
    if served:
        out["solves_per_s_ratio_vs_plain"] = served["solves_per_s"] / plain["solves_per_s"]
        out["work_ratio_vs_plain"] = served["cell_steps_per_s"] / plain["cell_steps_per_s"]
        out["solves_per_s_ratio_vs_best_sequential"] = served["solves_per_s"] / best["solves_per_s"]
    if seq_n != len(reqs):
        out["note"] = (f"the sequential runs time the first {seq_n} requests (same distribution); the ratios "
                       "compare solves/s")
    return out


def run_targets(args, hm):
    """The other targets' evidence, measured in the default run: every explicit
    operator on the same 128^3 box (HBM and FP64 fractions, floor), the 512^2
    cavity's 200 PISO steps with the pressure solved in FP64 and in mixed
    precision, a 64-case slice of the batched workload, and a 400-arrival slice
    of the served stream (mixed precision; one at a time on its first 100 requests)."""
    import copy

    out = {}
    a = copy.copy(args)
    a.explicit_ops = "interp_linear,interp_upwind,div_upwind,div_linear,grad,laplacian,sngrad,advect_euler"
    a.explicit_reps = 10
    a.cavity_steps = 200  # the configuration's 200 steps: early steps need more mixed inner iterations
    a.cases, a.batch_steps, a.alone_cases = 64, 10, 16
    s = copy.copy(args)
    s.requests, s.seq_requests, s.serve_mixed_only, s.serve_rate = 400, 100, True, 200.0
    for key, fn in (("advection_64x64_100_steps", lambda: run_advection(a)),
                    ("explicit_operators", lambda: run_explicit(a, hm=hm)),
                    ("cavity_512_pressure_solve", lambda: run_cavity(a, multigrid=False)),
                    ("batch_64_case_slice", lambda: run_batch(a)),
                    ("serving_400_arrivals_slice", lambda: run_serve(s))):
        try:
            out[key] = fn()
        except Exception as e:  # the headline line is printed whatever a side measurement does
            out[key] = {"error": repr(e)}
    return out


def workload_config(args):
    return {"workload": f"implicit heat transfer {args.n}^3 jittered hex box, FP64 Jacobi-PCG to 1e-8",
            "cells": args.n ** 3, "dt": HEAT["dt"], "parallelism": "replicas",
            "l2": "working set > 129 MB L2 (matrix 175 MB + vectors), no flush needed"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=HEAT["n"])
    ap.add_argument("--cpu-steps", type=int, default=12)
    ap.add_argument("--ref-max-steps", type=int, default=1000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the other targets' measurements")
    ap.add_argument("--workload", default="heat", choices=["heat", "advection", "cavity", "batch", "serve", "explicit",
                                                           "convection", "multigrid"])
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--seq-requests", type=int, default=400)
    ap.add_argument("--serve-streams", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=200.0, help="mean Poisson arrival rate, requests/s")
    ap.add_argument("--serve-mixed-only", action="store_true", help="skip the FP64 served run")
    ap.add_argument("--serve-max-active", type=int, default=16,
                    help="requests resident at once in the served runs (the rest wait)")
    ap.add_argument("--explicit-n", type=int, default=128)
    ap.add_argument("--explicit-reps", type=int, default=20)
    ap.add_argument("--explicit-ops", default="", help="comma-separated subset of the explicit operators")
    ap.add_argument("--cases", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--alone-cases", type=int, default=64)
    ap.add_argument("--inner-tol", type=float, default=0.1)
    ap.add_argument("--cavity-steps", type=int, default=200)
    ap.add_argument("--profile", action="store_true",
                    help="one warm-up and one timed FP64 step only (the command the ncu captures run)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    if world > 1:
        torch.distributed.init_process_group("nccl")
    from foamadapter_gb300 import _build

    if rank == 0:
        _build.build()
    if world > 1:
        torch.distributed.barrier()
    if args.workload != "heat":
        fn = {"advection": run_advection, "cavity": run_cavity, "batch": run_batch, "serve": run_serve,
              "explicit": run_explicit, "convection": run_convection, "multigrid": run_multigrid}[args.workload]
        if rank == 0:
            print(json.dumps(fn(args)))
        return
    if args.profile:
        args.steps, args.warmup = 1, 1
    hm, r = run_gpu(args, rank, world)
    if args.profile:
        print(json.dumps({"profile_run": True, "ms": r["ms"], "iters": r["iters"]}))
        return
    fu = r["face_updates"]
    ms, e2e_ms, units = aggregate_replicas(r["ms"], r["e2e_ms"], float(fu * args.steps), device="cuda")
    if rank != 0:
        return
    value = units / (ms / 1e3)
    e2e_value = units / (e2e_ms / 1e3)
    peak, peak_kind = load_peaks()
    ab = alg_bytes(hm)
    t_spmv = r["kt"][0] * 1e-3
    achieved = ab["pcg_spmv"] / t_spmv / 1e9
    traffic = read_traffic("k_pcg_spmv")
    launches = sum(5 + 3 * it for it in r["iters"])
    line = {
        "metric": "face-updates/s", "value": value, "unit": "face-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(args),
        "roofline": {"bound": "hbm", "kernel": "k_pcg_spmv (SpMV + p.Ap)", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic, "alg_bytes_per_launch": ab["pcg_spmv"],
                     "kernel_ms": {"spmv": r["kt"][0], "update": r["kt"][1], "dir": r["kt"][2]},
                     # GB300 issues FP64 at 2 lanes per clock per SM: the SpMV's DFMAs (one per
                     # stored slot, one per row for p.Ap) bound it together with HBM
                     "fp64_ops_per_launch": hm.nnz + hm.n,
                     "fp64_frac_of_issue_peak": (hm.nnz + hm.n) / (r["kt"][0] * 1e-3) / fp64_issue_peak(),
                     "iteration_GBps": ab["pcg_iteration"] / (sum(r["kt"][:3]) * 1e-3) / 1e9},
        "e2e": {"value": e2e_value, "unit": "face-updates/s", "h2d_bytes_per_step": 8 * hm.n,
                "d2h_bytes_per_step": 8 * hm.n},
        "gpu_launches": launches,
        "clocks": r["clocks"],
        "pcg_iterations_per_step": r["iters"],
        "mixed_precision": r["mixed"],
        "autotune": r["tuning"],
    }
    if not args.no_extras and world == 1:
        line["targets"] = run_targets(args, hm)
    if not args.no_cpu and world == 1:
        # the oracle continues from the state the end-to-end steps started from
        # (after W + K steps): its first step must give the GPU's step bit for bit,
        # and the steps it times are as hard as the GPU's timed ones
        hm2, k = heat_inputs(args.n, oracle_mesh=True)
        times, iters, threads, first = cpu_steps(hm2, k, args.cpu_steps, os.cpu_count(), T_start=r["step_in"])
        t = sum(times)
        exact = bool(np.array_equal(first, r["step_out"])) and iters[0] == r["e2e_iters"][-1]
        line["parity"] = {"check": f"one {args.n}^3 step from the GPU's state after {args.warmup + args.steps} "
                                   "steps, GPU (end-to-end call) vs CPU oracle",
                          "result": "bit-exact" if exact else "MISMATCH",
                          "iters_gpu": r["e2e_iters"][-1], "iters_oracle": iters[0],
                          "max_abs_diff": float(np.abs(first - r["step_out"]).max())}
        line["cpu_baseline"] = {"value": fu * len(times) / t, "unit": "face-updates/s", "cores": threads,
                                "kind": "port",
                                "sample": f"{len(times)} implicit steps of the same {args.n}^3 case from the GPU's "
                                          f"state after {args.warmup + args.steps} steps (assembly + FP64 "
                                          f"Jacobi-PCG to 1e-8, {iters} iterations) on the CPU oracle, "
                                          f"OpenMP x{threads}"}
    print(json.dumps(line))


def read_traffic(kernel, summary="pcg_fp64_kernels_128cube.md"):
    """DRAM bytes per launch of `kernel` (dram__bytes_read.sum + dram__bytes_write.sum)
    from the table of the committed ncu summary, whose header names the columns
    'DRAM read (bytes)' and 'DRAM write (bytes)'; None when absent."""
    p = ROOT / "profiles" / summary
    if not p.exists():
        return None
    cols = None
    for line in p.read_text().splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if cols is None and "DRAM read (bytes)" in cells and "DRAM write (bytes)" in cells:
            cols = (cells.index("DRAM read (bytes)"), cells.index("DRAM write (bytes)"))
        elif cols is not None and cells and cells[0].split(" ")[0] == kernel:
            try:
                return int(cells[cols[0]].replace(",", "")) + int(cells[cols[1]].replace(",", ""))
            except (ValueError, IndexError):
                return None
    return None


if __name__ == "__main__":
    main()
