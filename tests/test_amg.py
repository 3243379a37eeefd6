"""Multigrid-preconditioned CG (csrc/amg.cu) against its numpy restatement
(oracle/amg.py): the aggregation exactly, the V-cycle to rounding, and the
solve by its properties (the FP64 residual reached, the Jacobi-PCG solution
within the tolerance, determinism).  Ginkgo's own multigrid is not in the
reference checkout, so parity with it is unpinned."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from foamadapter_gb300 import abi, mesh
from oracle import amg as oamg
from oracle.pyoracle import Oracle


def heat_system(nx, ny, nz, seed=3, dt=0.01, lengths=(1.0, 1.0, 1.0), kspread=0.5):
    hm = mesh.box(nx, ny, nz, *lengths, jitter=0.1, seed=seed)
    o = Oracle(hm)
    k = np.exp(kspread * np.random.default_rng(seed).standard_normal(hm.n))
    kf = o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
    types = np.asarray([abi.BC_FIXED_VALUE] + [abi.BC_FIXED_GRADIENT] * (hm.npatch - 1), np.int32)
    ref = np.zeros(hm.nbf)
    ref[hm.patch_slice("xmin")] = 400.0
    T = np.full(hm.n, 300.0)
    Tb = np.zeros(hm.nbf)
    o.bc_correct(1, types, ref, T, Tb)
    v, rhs, _, _ = o.assemble(1, [(abi.TERM_DDT, 0, 1.0, T.copy(), None), (abi.TERM_LAPLACIAN, 0, -1.0, None, kf)],
                              dt, types, ref, Tb)
    ro, col = o.csr_arrays()[:2]
    return hm, o, kf, types, ref, T, Tb, v, rhs, ro, col


@pytest.mark.parametrize("dims", [(9, 7, 5), (16, 12, 1), (13, 11, 6)])
def test_pgm_aggregation_matches_restatement(dims):
    _, _, _, _, _, _, _, v, _, ro, col = heat_system(*dims)
    n = len(ro) - 1
    agg = np.zeros(n, np.int32)
    nc = C.c_int32()
    abi.check(abi.lib().fvgb_pgm_aggregate(n, ro.ctypes.data, col.ctypes.data, v.ctypes.data, agg.ctypes.data,
                                           C.byref(nc)))
    want, want_nc = oamg.pgm_aggregate(n, ro, col, v)
    assert nc.value == want_nc
    np.testing.assert_array_equal(agg, want)
    # aggregates: numbered by first row, at least one row each, mostly pairs
    sizes = np.bincount(agg, minlength=nc.value)
    assert sizes.min() >= 1 and nc.value < 0.6 * n
    first = np.full(nc.value, n)
    np.minimum.at(first, agg, np.arange(n))
    assert np.all(np.diff(first) > 0)


def test_pgm_aggregation_threaded_matches_restatement():
    """73,728 rows: the host aggregation runs on several threads (chunks of
    at least 2^15 rows) and must give the sequential restatement's aggregates."""
    _, _, _, _, _, _, _, v, _, ro, col = heat_system(48, 48, 32)
    n = len(ro) - 1
    agg = np.zeros(n, np.int32)
    nc = C.c_int32()
    abi.check(abi.lib().fvgb_pgm_aggregate(n, ro.ctypes.data, col.ctypes.data, v.ctypes.data, agg.ctypes.data,
                                           C.byref(nc)))
    want, want_nc = oamg.pgm_aggregate(n, ro, col, v)
    assert nc.value == want_nc
    np.testing.assert_array_equal(agg, want)


def test_pgm_edge_cases():
    L = abi.lib()
    nc = C.c_int32()
    # a diagonal matrix: no neighbours, every row alone
    n = 5
    ro = np.arange(n + 1, dtype=np.int32)
    col = np.arange(n, dtype=np.int32)
    v = np.ones(n)
    agg = np.zeros(n, np.int32)
    abi.check(L.fvgb_pgm_aggregate(n, ro.ctypes.data, col.ctypes.data, v.ctypes.data, agg.ctypes.data, C.byref(nc)))
    assert nc.value == n and list(agg) == list(range(n))
    # a path 0-1-2: the strongest pair forms, the third row joins it
    ro = np.array([0, 2, 5, 7], np.int32)
    col = np.array([0, 1, 0, 1, 2, 1, 2], np.int32)
    v = np.array([2.0, -1.0, -1.0, 2.0, -0.5, -0.5, 2.0])
    agg = np.zeros(3, np.int32)
    abi.check(L.fvgb_pgm_aggregate(3, ro.ctypes.data, col.ctypes.data, v.ctypes.data, agg.ctypes.data, C.byref(nc)))
    assert nc.value == 1 and list(agg) == [0, 0, 0]
    assert oamg.pgm_aggregate(3, ro, col, v)[1] == 1
    # empty
    abi.check(L.fvgb_pgm_aggregate(0, ro.ctypes.data, col.ctypes.data, v.ctypes.data, agg.ctypes.data, C.byref(nc)))
    assert nc.value == 0


def test_multigrid_selected_by_dictionary():
    from foamadapter_gb300.dictionary import Dictionary, solver_config
    d = Dictionary.parse('solver Ginkgo; type "solver::Cg"; preconditioner { type "solver::Multigrid"; }'
                         'criteria { iteration 200; relative_residual_norm 1e-9; }')
    cfg = solver_config(d)
    assert cfg["preconditioner"] == abi.PRECOND_MULTIGRID and cfg["max_iter"] == 200
    bad = Dictionary.parse('solver Ginkgo; type "solver::Bicgstab"; preconditioner { type "solver::Multigrid"; }')
    with pytest.raises(abi.FvgbError) as e:
        solver_config(bad)
    assert e.value.status == abi.ERR_UNSUPPORTED


def test_multigrid_solver_restatement_converges():
    """The oracle's multigrid solver reaches the direct solution; its cap and
    its ||b|| baseline behave as stated."""
    from scipy.sparse.linalg import spsolve

    _, _, _, _, _, T, _, v, rhs, ro, col = heat_system(13, 11, 6)
    levels = oamg.hierarchy(ro, col, v)
    x, it, res0, res, status = oamg.mg_solve(levels, rhs, T, 1e-10, 0.0, 300)
    assert status == 0 and 3 < it < 300 and res <= 1e-10 * res0
    xs = spsolve(levels[0][0].tocsc(), rhs)
    assert np.linalg.norm(x - xs) <= 1e-8 * np.linalg.norm(xs)
    assert oamg.mg_solve(levels, rhs, T, 1e-14, 0.0, 2)[1:] [::3] == (2, 3)
    xb, itb, _, resb, _ = oamg.mg_solve(levels, rhs, T, 1e-10, 0.0, 300, rhs_baseline=True)
    assert resb <= 1e-10 * np.linalg.norm(rhs) and itb != it


# ------------------------------------------------------------------ GPU
def gpu_system(cuda, dims, **kw):
    import torch

    from foamadapter_gb300 import neon
    from foamadapter_gb300.mesh import DeviceMesh

    hm, o, kf, types, ref, T, Tb, v, rhs, ro, col = heat_system(*dims, **kw)
    dm = DeviceMesh(hm)
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    Tf = neon.VolumeField(dm, np.full(hm.n, 300.0), bcs)
    gamma = neon.SurfaceField(dm, kf)
    ls = neon.LinearSystem(dm)
    old = Tf.internal.clone()
    ls.assemble([neon.ddt(old), neon.laplacian(gamma, -1.0)], kw.get("dt", 0.01), Tf)
    x0 = Tf.internal.clone()
    return dict(hm=hm, ls=ls, x0=x0, v=v, rhs=rhs, ro=ro, col=col, torch=torch, T=Tf, old=old, gamma=gamma,
                dm=dm)


@pytest.mark.gpu
def test_vcycle_matches_restatement(cuda):
    s = gpu_system(cuda, (18, 14, 10))
    torch = s["torch"]
    levels = oamg.hierarchy(s["ro"], s["col"], s["v"])
    rng = np.random.default_rng(5)
    for _ in range(2):
        r = rng.standard_normal(s["hm"].n)
        rd = torch.tensor(r, dtype=torch.float64, device="cuda")
        zd = torch.zeros_like(rd)
        abi.check(abi.lib().fvgb_amg_apply(s["ls"].handle, abi.ptr(rd), abi.ptr(zd), None))
        z = zd.cpu().numpy()
        want = oamg.vcycle(levels, r)
        assert np.linalg.norm(z - want) <= 1e-10 * np.linalg.norm(want)
    nl = C.c_int32()
    rows = np.zeros(32, np.int32)
    nnz = np.zeros(32, np.int64)
    abi.check(abi.lib().fvgb_amg_info(s["ls"].handle, C.byref(nl), rows.ctypes.data, nnz.ctypes.data, 32))
    assert nl.value == len(levels)
    assert list(rows[:nl.value]) == [lv[0].shape[0] for lv in levels]
    assert list(nnz[:nl.value]) == [lv[0].nnz for lv in levels]


@pytest.mark.gpu
def test_threaded_hierarchy_matches_restatement(cuda):
    """A system large enough for the host setup's threads (aggregation and
    Galerkin products in chunks): level sizes, nonzeros and the V-cycle as the
    sequential restatement."""
    s = gpu_system(cuda, (48, 48, 32))
    torch = s["torch"]
    levels = oamg.hierarchy(s["ro"], s["col"], s["v"])
    r = np.random.default_rng(8).standard_normal(s["hm"].n)
    rd = torch.tensor(r, dtype=torch.float64, device="cuda")
    zd = torch.zeros_like(rd)
    abi.check(abi.lib().fvgb_amg_apply(s["ls"].handle, abi.ptr(rd), abi.ptr(zd), None))
    want = oamg.vcycle(levels, r)
    assert np.linalg.norm(zd.cpu().numpy() - want) <= 1e-10 * np.linalg.norm(want)
    nl = C.c_int32()
    rows = np.zeros(32, np.int32)
    nnz = np.zeros(32, np.int64)
    abi.check(abi.lib().fvgb_amg_info(s["ls"].handle, C.byref(nl), rows.ctypes.data, nnz.ctypes.data, 32))
    assert list(rows[:nl.value]) == [lv[0].shape[0] for lv in levels]
    assert list(nnz[:nl.value]) == [lv[0].nnz for lv in levels]


@pytest.mark.gpu
def test_vcycle_is_symmetric_positive(cuda):
    s = gpu_system(cuda, (20, 16, 12))
    torch = s["torch"]
    rng = np.random.default_rng(9)
    r1, r2 = (torch.tensor(rng.standard_normal(s["hm"].n), dtype=torch.float64, device="cuda") for _ in range(2))
    z1, z2 = torch.zeros_like(r1), torch.zeros_like(r2)
    for r, z in ((r1, z1), (r2, z2)):
        abi.check(abi.lib().fvgb_amg_apply(s["ls"].handle, abi.ptr(r), abi.ptr(z), None))
    a, b = float(r2 @ z1), float(r1 @ z2)
    assert abs(a - b) <= 1e-11 * max(abs(a), abs(b))
    assert float(r1 @ z1) > 0 and float(r2 @ z2) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(24, 20, 16), (64, 48, 1)])
def test_multigrid_cg_converges_to_the_jacobi_solution(cuda, dims):
    s = gpu_system(cuda, dims)
    torch, ls = s["torch"], s["ls"]
    xj = s["x0"].clone()
    sj = ls.solve(xj, rel_tol=1e-11, max_iter=5000)
    xm = s["x0"].clone()
    sm = ls.solve(xm, rel_tol=1e-11, max_iter=500, preconditioner=abi.PRECOND_MULTIGRID)
    assert sj.status == abi.OK and sm.status == abi.OK
    assert sm.num_iter < sj.num_iter / 3, (sm.num_iter, sj.num_iter)
    assert sm.final_res_norm <= 1e-11 * sm.init_res_norm
    # the true residual on the host, from the oracle's matrix
    import scipy.sparse as sp
    A = sp.csr_matrix((s["v"], s["col"], s["ro"]))
    x = xm.cpu().numpy()
    x0 = s["x0"].cpu().numpy()
    assert np.linalg.norm(s["rhs"] - A @ x) <= 1e-9 * np.linalg.norm(s["rhs"] - A @ x0)
    xjh = xj.cpu().numpy()
    assert np.max(np.abs(x - xjh)) <= 1e-8 * np.max(np.abs(xjh))
    # deterministic: the same bits again
    xm2 = s["x0"].clone()
    sm2 = ls.solve(xm2, rel_tol=1e-11, max_iter=500, preconditioner=abi.PRECOND_MULTIGRID)
    assert sm2.num_iter == sm.num_iter and torch.equal(xm2, xm)


@pytest.mark.gpu
def test_multigrid_follows_matrix_changes(cuda):
    """A new matrix (another dt) recomputes the coarse values: the solve
    matches the Jacobi-PCG of the new system."""
    from foamadapter_gb300 import neon

    s = gpu_system(cuda, (20, 18, 10))
    ls, torch = s["ls"], s["torch"]
    x = s["x0"].clone()
    assert ls.solve(x, rel_tol=1e-10, preconditioner=abi.PRECOND_MULTIGRID).status == abi.OK
    ls.assemble([neon.ddt(s["old"]), neon.laplacian(s["gamma"], -1.0)], 0.5, s["T"])
    xm, xj = s["x0"].clone(), s["x0"].clone()
    sm = ls.solve(xm, rel_tol=1e-11, preconditioner=abi.PRECOND_MULTIGRID)
    sj = ls.solve(xj, rel_tol=1e-11, max_iter=5000)
    assert sm.status == abi.OK and sj.status == abi.OK
    assert float((xm - xj).abs().max()) <= 1e-8 * float(xj.abs().max())


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(24, 20, 16), (64, 48, 1)])
def test_fp32_vcycle_in_fp64_cg(cuda, dims):
    """Mixed precision: the FP64 CG with the V-cycle in FP32 reaches the same
    FP64 residual and the Jacobi-PCG solution; deterministic; the FP64
    V-cycle solve is unchanged after it."""
    s = gpu_system(cuda, dims)
    torch, ls = s["torch"], s["ls"]
    x64 = s["x0"].clone()
    s64 = ls.solve(x64, rel_tol=1e-11, max_iter=500, preconditioner=abi.PRECOND_MULTIGRID)
    xm = s["x0"].clone()
    sm = ls.solve(xm, rel_tol=1e-11, max_iter=500, precision=abi.PREC_MIXED_IR,
                  preconditioner=abi.PRECOND_MULTIGRID)
    assert sm.status == abi.OK and sm.final_res_norm <= 1e-11 * sm.init_res_norm
    assert sm.num_iter <= s64.num_iter + 3, (sm.num_iter, s64.num_iter)
    import scipy.sparse as sp
    A = sp.csr_matrix((s["v"], s["col"], s["ro"]))
    x = xm.cpu().numpy()
    x0 = s["x0"].cpu().numpy()
    assert np.linalg.norm(s["rhs"] - A @ x) <= 1e-9 * np.linalg.norm(s["rhs"] - A @ x0)
    assert float((xm - x64).abs().max()) <= 1e-8 * float(x64.abs().max())
    xm2 = s["x0"].clone()
    sm2 = ls.solve(xm2, rel_tol=1e-11, max_iter=500, precision=abi.PREC_MIXED_IR,
                   preconditioner=abi.PRECOND_MULTIGRID)
    assert sm2.num_iter == sm.num_iter and torch.equal(xm2, xm)
    x64b = s["x0"].clone()
    s64b = ls.solve(x64b, rel_tol=1e-11, max_iter=500, preconditioner=abi.PRECOND_MULTIGRID)
    assert s64b.num_iter == s64.num_iter and torch.equal(x64b, x64)


@pytest.mark.gpu
@pytest.mark.parametrize("dims,lengths,dt", [((40, 40, 8), (1.0, 1.0, 0.01), 1e3),
                                             ((48, 48, 6), (1.0, 1.0, 0.001), 1e6)])
def test_fp32_vcycle_on_stretched_cells(cuda, dims, lengths, dt):
    """The CG keeps the fixed-preconditioner beta (r.z / r_old.z_old) with the
    FP32 V-cycle. On cells of aspect ratio 100 and 1000, conductivities over
    e^(+-4.5) and near-steady time steps, solved to 1e-12, it needs no more
    iterations than with the FP64 V-cycle (a numpy emulation of both gives the
    same counts, 90 and 176)."""
    s = gpu_system(cuda, dims, dt=dt, lengths=lengths, kspread=1.5)
    ls = s["ls"]
    x64 = s["x0"].clone()
    s64 = ls.solve(x64, rel_tol=1e-12, max_iter=1000, preconditioner=abi.PRECOND_MULTIGRID)
    xm = s["x0"].clone()
    sm = ls.solve(xm, rel_tol=1e-12, max_iter=1000, precision=abi.PREC_MIXED_IR,
                  preconditioner=abi.PRECOND_MULTIGRID)
    assert s64.status == sm.status == abi.OK
    assert s64.num_iter > 40
    assert sm.final_res_norm <= 1e-12 * sm.init_res_norm
    assert sm.num_iter <= s64.num_iter + 3, (sm.num_iter, s64.num_iter)


@pytest.mark.gpu
def test_multigrid_rejects_what_it_does_not_cover(cuda):
    s = gpu_system(cuda, (12, 10, 8))
    x = s["x0"].clone()
    with pytest.raises(abi.FvgbError) as e:
        s["ls"].solve(x, method=abi.SOLVER_BICGSTAB, preconditioner=abi.PRECOND_MULTIGRID)
    assert e.value.status == abi.ERR_UNSUPPORTED


@pytest.mark.gpu
def test_multigrid_rejected_by_batches(cuda):
    from foamadapter_gb300 import neon

    s = gpu_system(cuda, (12, 10, 8))
    n = s["hm"].n
    b = neon.Batch(s["ls"], [0, n])
    cfg = abi.SolverCfg(1e-8, 0.0, 100, abi.PREC_FP64, 0.1, 1000, 50, 0, 0, abi.SOLVER_CG, abi.PRECOND_MULTIGRID)
    x = s["x0"].clone()
    assert abi.lib().fvgb_batch_solve(b.handle, abi.ptr(x), C.byref(cfg), None, None) == abi.ERR_UNSUPPORTED


@pytest.mark.gpu
def test_first_mixed_multigrid_solve_refuses_capture(cuda):
    """The first FP32 V-cycle sets up its copies and graph (allocations, a
    synchronous upload): issued on a capturing stream after an uncaptured FP64
    multigrid solve, it is refused with ERR_UNSUPPORTED before any GPU work, and
    the same solve outside the capture then works."""
    s = gpu_system(cuda, (12, 10, 8))
    torch, ls = s["torch"], s["ls"]
    x = s["x0"].clone()
    assert ls.solve(x, rel_tol=1e-9, preconditioner=abi.PRECOND_MULTIGRID).status == abi.OK
    cfg = abi.SolverCfg(1e-9, 0.0, 500, abi.PREC_MIXED_IR, 0.1, 1000, 50, 0, 0, abi.SOLVER_CG,
                        abi.PRECOND_MULTIGRID)
    stats = torch.zeros(8, dtype=torch.int32, device="cuda")
    xm = s["x0"].clone()
    g = torch.cuda.CUDAGraph()
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")            # the refused capture leaves an empty graph
        with torch.cuda.graph(g):
            status = abi.lib().fvgb_solve_async(ls.handle, abi.ptr(xm), C.byref(cfg), stats.data_ptr(),
                                                torch.cuda.current_stream().cuda_stream)
    assert status == abi.ERR_UNSUPPORTED
    assert b"captured" in abi.lib().fvgb_last_error()
    st = ls.solve(xm, rel_tol=1e-9, precision=abi.PREC_MIXED_IR, preconditioner=abi.PRECOND_MULTIGRID)
    assert st.status == abi.OK


# ------------------------------------------------------ the multigrid solver
@pytest.mark.gpu
@pytest.mark.parametrize("rhs_baseline", [False, True])
def test_multigrid_solver_matches_restatement(cuda, rhs_baseline):
    """OpenFOAM's GAMG as FoamAdapter maps it (Ginkgo solver::Multigrid):
    x += V(b - A x) until the criteria.  The cycles and the result follow the
    numpy restatement (the V-cycle agrees to rounding, so the count may
    differ by one only at a tolerance boundary)."""
    s = gpu_system(cuda, (18, 14, 10))
    ls, x0 = s["ls"], s["x0"]
    levels = oamg.hierarchy(s["ro"], s["col"], s["v"])
    flags = abi.SOLVE_RHS_BASELINE if rhs_baseline else 0
    x = x0.clone()
    st = ls.solve(x, rel_tol=1e-9, max_iter=300, method=abi.SOLVER_MULTIGRID, flags=flags)
    xw, it, res0, res, status = oamg.mg_solve(levels, s["rhs"], x0.cpu().numpy(), 1e-9, 0.0, 300,
                                              rhs_baseline=rhs_baseline)
    assert st.status == status == abi.OK
    assert abs(st.num_iter - it) <= 1 and it > 3
    assert st.init_res_norm == pytest.approx(res0, rel=1e-12)
    base = np.linalg.norm(s["rhs"]) if rhs_baseline else st.init_res_norm
    assert st.final_res_norm <= 1e-9 * base
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xw) <= 1e-9 * np.linalg.norm(xw)
    # the same system with multigrid-preconditioned CG reaches the same solution
    xc = x0.clone()
    assert ls.solve(xc, rel_tol=1e-11, preconditioner=abi.PRECOND_MULTIGRID).status == abi.OK
    assert np.linalg.norm(xg - xc.cpu().numpy()) <= 1e-7 * np.linalg.norm(xg)
    # deterministic
    x2 = x0.clone()
    st2 = ls.solve(x2, rel_tol=1e-9, max_iter=300, method=abi.SOLVER_MULTIGRID, flags=flags)
    assert st2.num_iter == st.num_iter and np.array_equal(x2.cpu().numpy(), xg)


@pytest.mark.gpu
def test_multigrid_solver_fp32_vcycle(cuda):
    """With mixed precision the V-cycle runs in FP32; the iteration, its
    residuals and its stopping test stay FP64 and reach the FP64 tolerance."""
    s = gpu_system(cuda, (24, 20, 16))
    ls, x0 = s["ls"], s["x0"]
    x64, x32 = x0.clone(), x0.clone()
    st64 = ls.solve(x64, rel_tol=1e-10, max_iter=400, method=abi.SOLVER_MULTIGRID)
    st32 = ls.solve(x32, rel_tol=1e-10, max_iter=400, method=abi.SOLVER_MULTIGRID, precision=abi.PREC_MIXED_IR)
    assert st64.status == st32.status == abi.OK
    assert st32.final_res_norm <= 1e-10 * st32.init_res_norm
    assert abs(st32.num_iter - st64.num_iter) <= 2
    a, b = x64.cpu().numpy(), x32.cpu().numpy()
    assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(a)


@pytest.mark.gpu
def test_multigrid_solver_cap_and_refusals(cuda):
    from foamadapter_gb300 import neon

    s = gpu_system(cuda, (12, 10, 8))
    ls, x0 = s["ls"], s["x0"]
    st = ls.solve(x0.clone(), rel_tol=1e-14, max_iter=3, method=abi.SOLVER_MULTIGRID)
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_iter == 3
    st = ls.solve(x0.clone(), rel_tol=1e-8, max_iter=0, method=abi.SOLVER_MULTIGRID)
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_iter == 0
    n = s["hm"].n
    b = neon.Batch(ls, [0, n])
    x = x0.clone()
    with pytest.raises(abi.FvgbError) as e:
        b.solve(x, method=abi.SOLVER_MULTIGRID)
    assert e.value.status == abi.ERR_UNSUPPORTED
    with pytest.raises(abi.FvgbError) as e:
        ls.solve(x, method=abi.SOLVER_MULTIGRID, precision=7)
    assert e.value.status == abi.ERR_INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["cg", "multigrid"])
def test_fp32_vcycle_is_scale_invariant(cuda, solver):
    """The FP32 V-cycle runs on the residual times a power of two near 1/|r|.
    A x = b and (2^-100 A) x = 2^-100 b then take the same iterations and give
    bit-identical x: every FP64 and FP32 operation commutes with the scale while
    the matrices stay in FP32's normal range.  Unscaled, the second system's
    late residuals (below 1e-40) would underflow FP32."""
    from foamadapter_gb300 import neon

    s = gpu_system(cuda, (24, 20, 16))
    torch = s["torch"]
    scale = 2.0 ** -100
    ls2 = neon.LinearSystem(s["dm"])
    ls2.assemble([neon.ddt(s["old"], scale), neon.laplacian(s["gamma"], -scale)], 0.01, s["T"])
    kw = dict(rel_tol=1e-10, max_iter=500, precision=abi.PREC_MIXED_IR)
    kw.update(dict(preconditioner=abi.PRECOND_MULTIGRID) if solver == "cg" else dict(method=abi.SOLVER_MULTIGRID))
    x1, x2 = s["x0"].clone(), s["x0"].clone()
    st1 = s["ls"].solve(x1, **kw)
    st2 = ls2.solve(x2, **kw)
    assert st1.status == st2.status == abi.OK
    assert st1.num_iter == st2.num_iter > 3
    assert st2.init_res_norm == st1.init_res_norm * scale
    assert torch.equal(x1, x2)
