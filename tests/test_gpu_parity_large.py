"""GPU solves against the CPU oracle at the sizes the workloads run.

Systems of at least 2^15 rows use the 8-rows-per-thread reduction tree (256
threads x 8 rows per 2048-row block) in the CG and BiCGStab dot products, both
on the GPU and in the oracle; smaller systems use 4 rows per thread.  Every
test here runs systems above that threshold and compares the GPU with the
oracle bit for bit: iterates, iteration counts (inner and outer), initial and
final residual norms.

* FP64 CG in the three launch modes (graph with a device-side loop, one
  persistent cooperative kernel, host-driven plain launches), the mixed
  precision CG (graph and persistent), FP64 and mixed BiCGStab;
* a batch holding one case above 2^15 rows beside small ones, every case
  against the oracle's solve of that case alone;
* one implicit heat-transfer step on a 64^3 jittered box (the shape of the
  128^3 workload at 1/8 the size);
* two PISO steps of the 512 x 512 lid-driven cavity (the pressure system of
  262,144 rows), FP64 and mixed precision, against the oracle's PISO loop
  (oracle/apps.py).
"""
import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, apps, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh
from oracle.apps import CavityPisoCPU, HeatTransferCPU
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu

BIG = 1 << 15


def heat_system(nx, ny, nz, seed=12345, dt=0.01):
    """ddt - laplacian(k) with lognormal k, a fixed 400 wall at xmin, T0 = 300."""
    hm = mesh.box(nx, ny, nz, jitter=0.1, seed=seed)
    dm = DeviceMesh(hm)
    o = Oracle(hm)
    k = np.exp(0.5 * np.random.default_rng(seed).standard_normal(hm.n))
    kf = o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T = neon.VolumeField(dm, np.full(hm.n, 300.0), bcs)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(neon.SurfaceField(dm, kf), -1.0)], dt, T)
    v, r, _, _ = [t.cpu().numpy() for t in ls.export()]
    # the oracle's own assembly of the same system is bit-identical
    types = np.asarray([abi.BC_FIXED_VALUE] + [abi.BC_FIXED_GRADIENT] * (hm.npatch - 1), np.int32)
    ref = np.zeros(hm.nbf)
    ref[hm.patch_slice("xmin")] = 400.0
    Th, Tb = np.full(hm.n, 300.0), np.zeros(hm.nbf)
    o.bc_correct(1, types, ref, Th, Tb)
    ov, orr, _, _ = o.assemble(1, [(abi.TERM_DDT, 0, 1.0, Th.copy(), None), (abi.TERM_LAPLACIAN, 0, -1.0, None, kf)],
                               dt, types, ref, Tb)
    np.testing.assert_array_equal(v, ov)
    np.testing.assert_array_equal(r, orr)
    return hm, T, o, ls, v, r


def same(st, so, x, xo):
    assert st.status == so.status == abi.OK, (st.status, so.status)
    assert (st.num_iter, st.num_outer) == (so.num_iter, so.num_outer)
    assert st.init_res_norm == so.init_res_norm and st.final_res_norm == so.final_res_norm
    np.testing.assert_array_equal(x.cpu().numpy(), xo)


@pytest.fixture(scope="module")
def heat40k(cuda):
    hm, T, o, ls, v, r = heat_system(40, 32, 28)       # 35,840 rows
    assert hm.n >= BIG
    return hm, T, o, ls, v, r


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_fp64_cg_eight_row_tree_vs_oracle(heat40k, mode):
    hm, T, o, ls, v, r = heat40k
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-8, max_iter=2000, kernel_mode=mode)
    xo = np.full(hm.n, 300.0)
    so = o.solve(v, r, xo, rel_tol=1e-8, max_iter=2000)
    same(st, so, x, xo)
    assert st.num_iter > 20


@pytest.mark.parametrize("mode", [1, 2])
def test_mixed_cg_eight_row_tree_vs_oracle(heat40k, mode):
    hm, T, o, ls, v, r = heat40k
    kw = dict(rel_tol=1e-8, max_iter=4000, inner_rel_tol=0.1, inner_max_iter=1000, max_outer=50)
    x = T.internal.clone()
    st = ls.solve(x, precision=abi.PREC_MIXED_IR, kernel_mode=mode, **kw)
    xo = np.full(hm.n, 300.0)
    so = o.solve(v, r, xo, precision=1, **kw)
    same(st, so, x, xo)
    assert st.num_outer > 1


def convection_system(nx, ny, nz, seed=5):
    hm = mesh.box(nx, ny, nz, jitter=0.1, seed=seed)
    dm = DeviceMesh(hm)
    o = Oracle(hm)
    rng = np.random.default_rng(seed)
    U = np.array([1.0, 0.4, -0.2])
    F = o.flux_vec(np.tile(U, hm.n), np.tile(U, hm.nbf))
    T = neon.VolumeField(dm, rng.random(hm.n), [("fixedValue", 1.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1))
    ls = neon.LinearSystem(dm)
    dt = 2.0 / nx / float(np.linalg.norm(U))            # Courant 2, as the convection workload
    ls.assemble([neon.ddt(T.internal.clone()), neon.div(neon.SurfaceField(dm, F), "upwind"),
                 neon.laplacian(neon.SurfaceField(dm, np.full(hm.nif + hm.nbf, 1e-3)), -1.0)], dt, T)
    v, r, _, _ = [t.cpu().numpy() for t in ls.export()]
    return hm, T, o, ls, v, r


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_bicgstab_eight_row_tree_vs_oracle(cuda, precision):
    hm, T, o, ls, v, r = convection_system(34, 32, 31)  # 33,728 rows
    assert hm.n >= BIG
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-8, max_iter=3000, precision=precision, method=abi.SOLVER_BICGSTAB)
    xo = T.host().copy()
    so = o.solve(v, r, xo, rel_tol=1e-8, max_iter=3000, precision=1 if precision == abi.PREC_MIXED_IR else 0,
                 method=1)
    same(st, so, x, xo)
    assert st.num_iter > 5


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_batch_with_a_large_case_vs_oracle(cuda, precision):
    """One case of 35,840 rows (8-row tree) packed with three small ones (4-row
    tree): each case's iterate and counts equal the oracle's solve of that
    case alone."""
    dims = [(9, 8, 7), (40, 32, 28), (13, 5, 11), (16, 16, 16)]
    rng = np.random.default_rng(21)
    cases = []
    for q, d in enumerate(dims):
        hm = mesh.box(*d, jitter=0.1, seed=300 + q)
        cases.append((hm, np.exp(0.5 * rng.standard_normal(hm.n)), float(rng.uniform(350.0, 450.0))))
    big, ranges, slices = mesh.concat([c[0] for c in cases])
    dm = DeviceMesh(big)
    kap, ref = np.ones(big.n), np.zeros(big.nbf)
    for q, (hm, kk, tw) in enumerate(cases):
        kap[ranges[2 * q]:ranges[2 * q + 1]] = kk
        ref[slices[q][0]] = tw
    T = neon.VolumeField(dm, np.full(big.n, 300.0), [("fixedValue", ref[slices[0][0].start:slices[-1][0].stop])]
                         + [("zeroGradient", 0.0)] * 5)
    gamma = neon.SurfaceInterpolation(dm, "linear").interpolate(
        neon.VolumeField(dm, kap, [("zeroGradient", 0.0)] * 6))
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gamma, -1.0)], 0.01, T)
    kw = dict(rel_tol=1e-8, max_iter=4000, inner_rel_tol=0.1, inner_max_iter=1000, max_outer=50)
    x = T.internal.clone()
    stats = neon.Batch(ls, ranges).solve(x, precision=precision, **kw)
    xb = x.cpu().numpy()
    for q, (hm, kk, tw) in enumerate(cases):
        o = Oracle(hm)
        kf = o.interp_linear(1, kk, np.ascontiguousarray(kk[hm.bcells]))
        types = np.asarray([abi.BC_FIXED_VALUE] + [abi.BC_FIXED_GRADIENT] * 5, np.int32)
        rf = np.zeros(hm.nbf)
        rf[hm.patch_slice("xmin")] = tw
        Th, Tb = np.full(hm.n, 300.0), np.zeros(hm.nbf)
        o.bc_correct(1, types, rf, Th, Tb)
        v, r, _, _ = o.assemble(1, [(abi.TERM_DDT, 0, 1.0, Th.copy(), None),
                                    (abi.TERM_LAPLACIAN, 0, -1.0, None, kf)], 0.01, types, rf, Tb)
        so = o.solve(v, r, Th, precision=1 if precision == abi.PREC_MIXED_IR else 0, **kw)
        st = stats[q]
        assert st.status == so.status == abi.OK
        assert (st.num_iter, st.num_outer) == (so.num_iter, so.num_outer), q
        assert st.init_res_norm == so.init_res_norm and st.final_res_norm == so.final_res_norm
        np.testing.assert_array_equal(xb[ranges[2 * q]:ranges[2 * q + 1]], Th)
    assert max(c[0].n for c in cases) >= BIG


def test_heat_steps_64cube_vs_oracle(cuda):
    """Two implicit heat-transfer steps (assembly + FP64 Jacobi-PCG to 1e-8 +
    boundary update) on a 64^3 jittered box through the application driver,
    against the oracle's twin of the same driver."""
    hm = mesh.box(64, 64, 64, jitter=0.1, seed=12345)
    k = np.exp(0.5 * np.random.default_rng(12345).standard_normal(hm.n))
    gpu = apps.HeatTransfer(hm, k)
    cpu = HeatTransferCPU(hm, k)
    for _ in range(2):
        gpu.step()
        cpu.step()
    assert [s[:4] for s in gpu.stats] == [s[:4] for s in cpu.stats]
    np.testing.assert_array_equal(gpu.T.host(), cpu.T)
    assert min(s[0] for s in cpu.stats) > 50


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_cavity_512_piso_steps_vs_oracle(cuda, precision):
    """The 512 x 512 lid-driven cavity with +-5% jitter, dt 5e-4, two
    correctors: two PISO steps (four pressure solves of 262,144 rows) equal
    the oracle's PISO loop bit for bit, pressure and velocity."""
    nsteps = 2 if precision == abi.PREC_FP64 else 1
    gpu = apps.CavityPiso(n=512, precision=precision)
    cpu = CavityPisoCPU(gpu.hm, precision=1 if precision == abi.PREC_MIXED_IR else 0)
    for _ in range(nsteps):
        gpu.step()
        cpu.step()
    assert [tuple(s) for s in gpu.stats] == [tuple(s) for s in cpu.stats]
    np.testing.assert_array_equal(gpu.p.host(), cpu.p)
    np.testing.assert_array_equal(gpu.U.host(), cpu.U)
    torch.cuda.synchronize()


@pytest.mark.parametrize("precision,mode", [(abi.PREC_FP64, 1), (abi.PREC_FP64, 2), (abi.PREC_FP64, 3),
                                            (abi.PREC_MIXED_IR, 1), (abi.PREC_MIXED_IR, 2)])
def test_rhs_norm_baseline_vs_oracle(heat40k, precision, mode):
    """Ginkgo's ResidualNorm with its default baseline (||r|| <= rel_tol ||b||,
    the reference's gko/config.bj.json): ||b|| by the solver's reduction tree,
    the same stop as the oracle's, bit for bit."""
    hm, T, o, ls, v, r = heat40k
    kw = dict(rel_tol=1e-5, max_iter=2000, inner_rel_tol=0.1, inner_max_iter=1000, max_outer=50)
    x = T.internal.clone()
    st = ls.solve(x, precision=precision, kernel_mode=mode, flags=abi.SOLVE_RHS_BASELINE, **kw)
    xo = np.full(hm.n, 300.0)
    so = o.solve(v, r, xo, precision=1 if precision == abi.PREC_MIXED_IR else 0, flags=2, **kw)
    same(st, so, x, xo)
    assert st.final_res_norm <= 1e-5 * float(np.linalg.norm(r))
    # the baseline matters: relative to the initial residual the same rel_tol stops elsewhere
    st0 = ls.solve(T.internal.clone(), precision=precision, kernel_mode=mode, **kw)
    assert st0.num_iter != st.num_iter


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_rhs_norm_baseline_bicgstab_vs_oracle(cuda, precision):
    hm, T, o, ls, v, r = convection_system(34, 32, 31)
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-6, max_iter=3000, precision=precision, method=abi.SOLVER_BICGSTAB,
                  flags=abi.SOLVE_RHS_BASELINE)
    xo = T.host().copy()
    so = o.solve(v, r, xo, rel_tol=1e-6, max_iter=3000, precision=1 if precision == abi.PREC_MIXED_IR else 0,
                 method=1, flags=2)
    same(st, so, x, xo)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_rhs_norm_baseline_with_multigrid(heat40k, precision):
    """The multigrid-preconditioned CG stops at ||r|| <= rel_tol ||b|| with
    the flag: the baseline changes where it stops, and it stops in time."""
    hm, T, o, ls, v, r = heat40k
    bn = float(np.linalg.norm(r))
    st = ls.solve(T.internal.clone(), rel_tol=1e-5, precision=precision, preconditioner=abi.PRECOND_MULTIGRID,
                  flags=abi.SOLVE_RHS_BASELINE)
    assert st.status == abi.OK and st.final_res_norm <= 1e-5 * bn
    st0 = ls.solve(T.internal.clone(), rel_tol=1e-5, precision=precision, preconditioner=abi.PRECOND_MULTIGRID)
    assert st0.final_res_norm <= 1e-5 * st0.init_res_norm
    assert st0.num_iter != st.num_iter


@pytest.mark.parametrize("flags", [0, abi.SOLVE_RHS_BASELINE])
def test_bicg_eight_row_tree_vs_oracle(cuda, flags):
    hm, T, o, ls, v, r = convection_system(34, 32, 31)
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-8, max_iter=3000, method=abi.SOLVER_BICG, flags=flags)
    xo = T.host().copy()
    so = o.solve(v, r, xo, rel_tol=1e-8, max_iter=3000, method=2, flags=2 if flags else 0)
    same(st, so, x, xo)
    assert st.num_iter > 5
