"""GPU implicit assembly, LinearSystem utilities and Krylov solves against the
CPU oracle.

Assembly, SetReference, applyOperator and diag are bit-exact.  The FP64
Jacobi-CG follows the same reduction tree as the oracle, so its iterates,
iteration count and residual norms are bit-exact too.  The mixed-precision
solve must reach the same 1e-8 relative FP64 residual (checked by an FP64
residual computed on the CPU) and its error against the FP64 solution is
bounded by the conditioning of the system.
"""
import numpy as np
import pytest
import torch

from conftest import load_polymesh
from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def heat_case(nx=12, ny=10, nz=8, jitter=0.1, seed=12345, dt=0.01):
    hm = mesh.box(nx, ny, nz, jitter=jitter, seed=seed)
    rng = np.random.default_rng(seed)
    k = np.exp(0.5 * rng.standard_normal(hm.n))
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    return hm, k, bcs, dt


def csr_of(o, values_csr):
    return values_csr


def assemble_both(hm, dm, terms_fn, bcs, ncomp=1, dt=0.01, seed=0):
    rng = np.random.default_rng(seed)
    o = Oracle(hm)
    T = neon.VolumeField(dm, 300.0 + rng.standard_normal(hm.n * ncomp), bcs, ncomp)
    gpu_terms, host_terms = terms_fn(dm, T, rng)
    ls = neon.LinearSystem(dm, ncomp)
    ls.assemble(gpu_terms, dt, T)
    v, r, bm, br = [t.cpu().numpy() for t in ls.export()]
    ov, orr, obm, obr = o.assemble(ncomp, host_terms, dt, T.types, T.ref.cpu().numpy(),
                                   T.boundary.cpu().numpy())
    return ls, T, o, (v, r, bm, br), (ov, orr, obm, obr)


def test_sparsity_matches_oracle(cuda):
    hm, _ = load_polymesh("setup_stencil3D")
    dm = DeviceMesh(hm)
    gpu = dm.sparsity()
    host = Oracle(hm).csr_arrays()
    for a, b in zip(gpu, host):
        np.testing.assert_array_equal(a, b)
    assert gpu[0][-1] == 135


@pytest.mark.parametrize("ncomp", [1, 3])
def test_assembly_all_terms_bit_exact(cuda, ncomp):
    hm = mesh.box(7, 6, 5, jitter=0.12, seed=9)
    dm = DeviceMesh(hm)
    nf = hm.nif + hm.nbf
    bcs = [("fixedValue", 400.0), ("zeroGradient", 0.0), ("fixedGradient", 2.0),
           ("fixedValue", 1.5), ("calculated", 0.0), ("zeroGradient", 0.0)]

    def terms(dm, T, rng):
        old = rng.standard_normal(hm.n * ncomp)
        gamma = np.exp(rng.standard_normal(nf))
        F = rng.standard_normal(nf)
        s = rng.random(hm.n)
        E = rng.standard_normal(hm.n * ncomp)
        g = [neon.ddt(neon.dev(old)), neon.laplacian(neon.SurfaceField(dm, gamma), -0.8),
             neon.div(neon.SurfaceField(dm, F), "upwind", 1.3), neon.div(neon.SurfaceField(dm, F), "linear", 0.6),
             neon.source(0.4, neon.dev(s)), neon.explicit(neon.dev(E), -1.0),
             neon.div_explicit(neon.SurfaceField(dm, F), neon.dev(old), "upwind", 0.9)]
        h = [(abi.TERM_DDT, 0, 1.0, old, None), (abi.TERM_LAPLACIAN, 0, -0.8, None, gamma),
             (abi.TERM_DIV, abi.SCHEME_UPWIND, 1.3, None, F), (abi.TERM_DIV, abi.SCHEME_LINEAR, 0.6, None, F),
             (abi.TERM_SOURCE, 0, 0.4, s, None), (abi.TERM_EXPLICIT, 0, -1.0, E, None),
             (abi.TERM_DIV_EXPLICIT, abi.SCHEME_UPWIND, 0.9, old, F)]
        return g, h

    ls, T, o, gpu, ref = assemble_both(hm, dm, terms, bcs, ncomp)
    for a, b in zip(gpu, ref):
        np.testing.assert_array_equal(a, b)
    # diag and applyOperator (A x - b)
    v = gpu[0]
    ro, col, do, oo, no = o.csr_arrays()
    np.testing.assert_array_equal(ls.diag().cpu().numpy(), v[ro[:-1] + do])
    x = np.random.default_rng(1).standard_normal(hm.n * ncomp)
    np.testing.assert_array_equal(ls.apply(neon.dev(x)).cpu().numpy(), o.apply_operator(v, gpu[1], ncomp, x))


def test_ddt_and_source_semantics(cuda):
    """Implicit ddt: diag V/dt, rhs V/dt*T_old, A T - b = V (T - T_old)/dt
    (test/test_implicitOperators.cpp:170-234); implicit source diag = c*V (:236-286)."""
    hm = mesh.box(5, 4, 3, jitter=0.1, seed=2)
    dm = DeviceMesh(hm)
    T = neon.VolumeField(dm, np.arange(hm.n, dtype=float))
    old = T.host() - 1.0
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(neon.dev(old))], 1.0, T)
    np.testing.assert_allclose(ls.apply(T.internal).cpu().numpy(), hm.V, rtol=1e-14, atol=0)
    ls.assemble([neon.source(2.0)], 1.0, T)
    np.testing.assert_array_equal(ls.diag().cpu().numpy(), 2.0 * hm.V)


def test_laplacian_matches_explicit_operator(cuda):
    """A T - b of the implicit laplacian equals the explicit laplacian times V
    (the check of test/test_implicitOperators.cpp:344-396, 1e-14)."""
    hm = mesh.box(8, 6, 5, jitter=0.1, seed=4)
    dm = DeviceMesh(hm)
    rng = np.random.default_rng(0)
    T = neon.VolumeField(dm, rng.standard_normal(hm.n), [("fixedValue", 1.0)] + [("zeroGradient", 0)] * 5)
    gamma = neon.SurfaceField(dm, np.full(hm.nif + hm.nbf, 0.1))
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.laplacian(gamma)], 1.0, T)
    imp = ls.apply(T.internal).cpu().numpy()
    exp = neon.GaussGreenLaplacian(dm).laplacian(torch.zeros(hm.n, dtype=torch.float64, device="cuda"),
                                                 gamma, T).cpu().numpy() * hm.V
    np.testing.assert_allclose(imp, exp, rtol=0, atol=1e-14 * max(1.0, np.abs(exp).max()))


def test_set_reference(cuda):
    hm = mesh.box(6, 6, 1, two_d=True)
    dm = DeviceMesh(hm)
    p = neon.VolumeField(dm, np.zeros(hm.n), [("zeroGradient", 0)] * 4)
    gamma = neon.SurfaceField(dm, np.ones(hm.nif + hm.nbf))
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.laplacian(gamma)], 1.0, p)
    v0 = ls.export()
    ls.setReference(3, 0.25)
    v1 = ls.export()
    o = Oracle(hm)
    ov, orr = v0[0].cpu().numpy().copy(), v0[1].cpu().numpy().copy()
    o.set_reference(ov, orr, 3, 0.25)
    np.testing.assert_array_equal(v1[0].cpu().numpy(), ov)
    np.testing.assert_array_equal(v1[1].cpu().numpy(), orr)


def solve_case(nx=14, ny=12, nz=10, scale=1.0):
    hm, k, bcs, dt = heat_case(nx, ny, nz)
    bcs = [(kind, val * scale) for kind, val in bcs]
    dm = DeviceMesh(hm)
    T = neon.VolumeField(dm, np.full(hm.n, 300.0 * scale), bcs)
    o = Oracle(hm)
    kf = o.interp_linear(1, k, k[hm.bcells].copy())
    gamma = neon.SurfaceField(dm, kf)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gamma, -1.0)], dt, T)
    v, r, bm, br = [t.cpu().numpy() for t in ls.export()]
    return hm, dm, T, o, ls, v, r


def test_pcg_fp64_bit_exact(cuda):
    hm, dm, T, o, ls, v, r = solve_case()
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-8, max_iter=1000)
    xo = np.full(hm.n, 300.0)
    so = o.solve(v, r, xo, rel_tol=1e-8, max_iter=1000)
    assert st.status == abi.OK and so.status == 0
    assert st.num_iter == so.num_iter > 5
    assert st.init_res_norm == so.init_res_norm and st.final_res_norm == so.final_res_norm
    np.testing.assert_array_equal(x.cpu().numpy(), xo)
    true = np.linalg.norm(o.apply_operator(v, r, 1, xo))
    assert true <= 1.01e-8 * so.init_res_norm


def test_pcg_iteration_cap_and_abs_tol(cuda):
    hm, dm, T, o, ls, v, r = solve_case(8, 8, 8)
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-12, max_iter=3)
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_iter == 3
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=0.0, abs_tol=1e300, max_iter=50)
    assert st.status == abi.OK and st.num_iter == 0


@pytest.mark.parametrize("inner", [1e-2, 1e-4])
def test_mixed_ir_reaches_fp64_residual(cuda, inner):
    hm, dm, T, o, ls, v, r = solve_case()
    x64 = T.internal.clone()
    ls.solve(x64, rel_tol=1e-8)
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-8, precision=abi.PREC_MIXED_IR, inner_rel_tol=inner, inner_max_iter=500,
                  max_outer=40)
    assert st.status == abi.OK, st.status
    xh = x.cpu().numpy()
    true = np.linalg.norm(o.apply_operator(v, r, 1, xh))
    assert true <= 1.01e-8 * st.init_res_norm
    # the same algorithm on the CPU (FP32 inner CG emulated with fmaf) gives the same bits
    xo = np.full(hm.n, 300.0)
    so = o.solve(v, r, xo, rel_tol=1e-8, precision=1, inner_rel_tol=inner, inner_max_iter=500, max_outer=40)
    assert (st.num_iter, st.num_outer) == (so.num_iter, so.num_outer)
    np.testing.assert_array_equal(xh, xo)
    # error against the FP64 solve
    err = np.abs(xh - x64.cpu().numpy()).max()
    assert err < 1e-6 * 400.0


def test_persistent_graph_and_host_loop_agree(cuda):
    """The one-kernel cooperative solve, the graph of kernels and the host-driven
    loop (plain launches) give the same bits."""
    hm, dm, T, o, ls, v, r = solve_case(40, 32, 24)
    out = []
    for mode in (1, 2, 3):
        x = T.internal.clone()
        st = ls.solve(x, rel_tol=1e-9, max_iter=2000, kernel_mode=mode)
        out.append((x.cpu().numpy(), st.num_iter, st.final_res_norm))
    for other in out[1:]:
        np.testing.assert_array_equal(out[0][0], other[0])
        assert out[0][1:] == other[1:]


@pytest.mark.parametrize("shape", [(40, 32, 24), (7, 5, 3)])
def test_mixed_persistent_and_graph_agree(cuda, shape):
    """The cooperative mixed-precision solve (two grid barriers per inner
    iteration, the direction folded into the SpMV) gives the bits of the graph
    of kernels and of the oracle."""
    hm, dm, T, o, ls, v, r = solve_case(*shape)
    kw = dict(rel_tol=1e-9, inner_rel_tol=0.1, inner_max_iter=1000, max_outer=50)
    out = []
    for mode in (1, 2):
        x = T.internal.clone()
        st = ls.solve(x, precision=abi.PREC_MIXED_IR, kernel_mode=mode, max_iter=4000, **kw)
        assert st.status == abi.OK
        out.append((x.cpu().numpy(), st.num_iter, st.num_outer, st.final_res_norm))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert out[0][1:] == out[1][1:]
    xo = np.full(hm.n, 300.0)
    so = o.solve(v, r, xo, precision=1, max_iter=4000, **kw)
    assert (so.num_iter, so.num_outer) == out[0][1:3]
    np.testing.assert_array_equal(out[0][0], xo)


def test_host_loop_is_fp64_only(cuda):
    hm, dm, T, o, ls, v, r = solve_case(6, 6, 6)
    with pytest.raises(RuntimeError):
        ls.solve(T.internal.clone(), precision=abi.PREC_MIXED_IR, kernel_mode=3)


def test_mixed_tiny_residual_is_scale_invariant(cuda):
    """Initial field and wall value scaled by 2^-100 (so b and x0 are, exactly):
    the power-of-two scaling of the FP32 residual keeps the inner solve identical,
    so x is the unscaled solution times 2^-100 (the FP32 dot products would
    otherwise underflow), and the oracle agrees bit for bit."""
    sc = 2.0 ** -100
    hm, dm, T1, o, ls1, v1, r1 = solve_case()
    _, _, T2, _, ls2, v2, r2 = solve_case(scale=sc)
    np.testing.assert_array_equal(v2, v1)
    np.testing.assert_array_equal(r2, r1 * sc)
    x1, x2 = T1.internal.clone(), T2.internal.clone()
    kw = dict(rel_tol=1e-8, inner_rel_tol=0.1, inner_max_iter=1000, max_outer=50)
    s1 = ls1.solve(x1, precision=abi.PREC_MIXED_IR, **kw)
    s2 = ls2.solve(x2, precision=abi.PREC_MIXED_IR, **kw)
    assert s1.status == abi.OK and s2.status == abi.OK
    assert (s1.num_iter, s1.num_outer) == (s2.num_iter, s2.num_outer)
    assert s2.final_res_norm == s1.final_res_norm * sc
    np.testing.assert_array_equal(x2.cpu().numpy(), x1.cpu().numpy() * sc)
    xo = np.full(hm.n, 300.0 * sc)
    so = o.solve(v2, r2, xo, precision=1, **kw)
    assert so.status == 0 and so.num_iter == s2.num_iter
    np.testing.assert_array_equal(x2.cpu().numpy(), xo)


def test_kernel_variants_give_the_same_bits(cuda):
    """The autotuner's launch-bound variants of the SpMV and update kernels
    (fvgb_solve_tuning) execute the same arithmetic: forcing each variant gives
    identical FP64 and mixed-precision solves."""
    import ctypes as C

    hm, dm, T, o, ls, v, r = solve_case(40, 32, 24)
    L = abi.lib()
    chosen = (C.c_int32 * 4)()
    ms = (C.c_float * 16)()
    out = {}
    for var in range(4):
        force = (C.c_int32 * 4)(var, var, var, var)
        abi.check(L.fvgb_solve_tuning(ls.handle, force, chosen, ms))
        assert list(chosen) == [(2, 4, 6, 8)[var]] * 4
        for prec in (abi.PREC_FP64, abi.PREC_MIXED_IR):
            x = T.internal.clone()
            st = ls.solve(x, rel_tol=1e-9, max_iter=3000, precision=prec, kernel_mode=1)
            assert st.status == abi.OK
            out.setdefault(prec, []).append((x.cpu().numpy(), st.num_iter, st.final_res_norm))
    for prec, runs in out.items():
        for run in runs[1:]:
            np.testing.assert_array_equal(runs[0][0], run[0])
            assert runs[0][1:] == run[1:]
    # back to the tuned choice
    force = (C.c_int32 * 4)(-1, -1, -1, -1)
    abi.check(L.fvgb_solve_tuning(ls.handle, force, chosen, ms))
    assert all(c in (2, 4, 6, 8) for c in chosen)


def test_rhs_only_assembly_and_reused_fp32_matrix(cuda):
    """fvgb_assemble_rhs with unchanged implicit terms writes exactly what a full
    assembly writes, and a mixed solve after it (FP32 matrix copy kept) gives the
    bits of a solve on a freshly assembled system."""
    import ctypes as C

    hm, k, bcs, dt = heat_case(14, 12, 10)
    o = Oracle(hm)
    kf = o.interp_linear(1, k, k[hm.bcells].copy())

    def setup():
        dm = DeviceMesh(hm)
        T = neon.VolumeField(dm, np.full(hm.n, 300.0), bcs)
        return dm, T, neon.SurfaceField(dm, kf), neon.LinearSystem(dm)

    L, s = abi.lib(), torch.cuda.current_stream().cuda_stream
    kw = dict(rel_tol=1e-9, precision=abi.PREC_MIXED_IR, inner_rel_tol=0.1, inner_max_iter=1000, max_outer=50)
    # system A: step 1 full assembly + solve, step 2 rhs-only assembly + solve (reused FP32 matrix)
    dm, T, gamma, ls = setup()
    old = T.internal.clone()
    terms = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(old), neon.laplacian(gamma, -1.0))])
    bc = T.bc_struct()
    abi.check(L.fvgb_assemble(ls.handle, terms, 2, dt, C.byref(bc), abi.ptr(T.boundary), s))
    ls.solve(T.internal, **kw)
    T.correctBoundaryConditions()
    old.copy_(T.internal)
    abi.check(L.fvgb_assemble_rhs(ls.handle, terms, 2, dt, C.byref(bc), abi.ptr(T.boundary), s))
    got = [t.cpu().numpy() for t in ls.export()]
    x_a = T.internal.clone()
    st_a = ls.solve(x_a, **kw)
    # system B: the same second step with a full assembly on a fresh system
    dm2, T2, gamma2, ls2 = setup()
    T2.internal.copy_(old)
    T2.correctBoundaryConditions()
    old2 = old.clone()
    terms2 = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(old2), neon.laplacian(gamma2, -1.0))])
    bc2 = T2.bc_struct()
    abi.check(L.fvgb_assemble(ls2.handle, terms2, 2, dt, C.byref(bc2), abi.ptr(T2.boundary), s))
    want = [t.cpu().numpy() for t in ls2.export()]
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    x_b = T2.internal.clone()
    st_b = ls2.solve(x_b, **kw)
    assert (st_a.num_iter, st_a.num_outer) == (st_b.num_iter, st_b.num_outer)
    np.testing.assert_array_equal(x_a.cpu().numpy(), x_b.cpu().numpy())


def convection_case(nx=13, ny=11, nz=9, seed=5):
    hm = mesh.box(nx, ny, nz, jitter=0.1, seed=seed)
    dm = DeviceMesh(hm)
    o = Oracle(hm)
    rng = np.random.default_rng(seed)
    U = np.array([1.0, 0.4, -0.2])
    F = o.flux_vec(np.tile(U, hm.n), np.tile(U, hm.nbf))
    bcs = [("fixedValue", 1.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T = neon.VolumeField(dm, rng.random(hm.n), bcs)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.div(neon.SurfaceField(dm, F), "upwind"),
                 neon.laplacian(neon.SurfaceField(dm, np.full(hm.nif + hm.nbf, 1e-2)), -1.0)], 0.05, T)
    v, r, _, _ = [t.cpu().numpy() for t in ls.export()]
    return hm, dm, T, o, ls, v, r


def test_bicgstab_bit_exact_on_nonsymmetric_system(cuda):
    """Implicit upwind convection makes the system nonsymmetric: BiCGStab (Ginkgo's
    Bicgstab, fvSolution.cpp:25-26) against the oracle's restatement, bit for bit."""
    hm, dm, T, o, ls, v, r = convection_case()
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-10, max_iter=500, method=abi.SOLVER_BICGSTAB)
    xo = T.host().copy()
    so = o.solve(v, r, xo, rel_tol=1e-10, max_iter=500, method=1)
    assert st.status == so.status == abi.OK and st.num_iter == so.num_iter > 3
    assert (st.init_res_norm, st.final_res_norm) == (so.init_res_norm, so.final_res_norm)
    np.testing.assert_array_equal(x.cpu().numpy(), xo)
    true = np.linalg.norm(o.apply_operator(v, r, 1, xo))
    assert true <= 1e-9 * so.init_res_norm
    # iteration cap
    st = ls.solve(T.internal.clone(), rel_tol=1e-14, max_iter=2, method=abi.SOLVER_BICGSTAB)
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_iter == 2


@pytest.mark.parametrize("rel_tol", [1e-8, 1e-12])
def test_mixed_bicgstab_bit_exact(cuda, rel_tol):
    """FP32 inner BiCGStab with FP64 refinement against the oracle's restatement,
    bit for bit (iterate, inner and outer counts, norms), reaching the FP64
    residual; a second solve of the unchanged system reuses the FP32 copy."""
    hm, dm, T, o, ls, v, r = convection_case(nx=21, ny=19, nz=17)
    for _ in range(2):
        x = T.internal.clone()
        st = ls.solve(x, rel_tol=rel_tol, max_iter=3000, precision=abi.PREC_MIXED_IR, method=abi.SOLVER_BICGSTAB)
        xo = T.host().copy()
        so = o.solve(v, r, xo, rel_tol=rel_tol, max_iter=3000, precision=1, method=1)
        assert st.status == so.status == abi.OK
        assert (st.num_iter, st.num_outer) == (so.num_iter, so.num_outer) and st.num_outer > 1
        assert (st.init_res_norm, st.final_res_norm) == (so.init_res_norm, so.final_res_norm)
        np.testing.assert_array_equal(x.cpu().numpy(), xo)
        assert np.linalg.norm(o.apply_operator(v, r, 1, xo)) <= rel_tol * so.init_res_norm
    # caps: refinement steps and total inner iterations
    st = ls.solve(T.internal.clone(), rel_tol=1e-14, max_iter=3000, max_outer=2, precision=abi.PREC_MIXED_IR,
                  method=abi.SOLVER_BICGSTAB, allow=(abi.ERR_NOT_CONVERGED,))
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_outer == 2


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_bicgstab_batch_equals_alone(cuda, precision):
    parts = [mesh.box(7, 6, 5, jitter=0.1, seed=s) for s in (1, 2, 3)]
    big, ranges, _ = mesh.concat(parts)
    ranges = np.asarray(ranges, np.int32)
    dm = DeviceMesh(big)
    o = Oracle(big)
    U = np.array([0.3, -1.0, 0.5])
    F = o.flux_vec(np.tile(U, big.n), np.tile(U, big.nbf))
    T = neon.VolumeField(dm, np.full(big.n, 0.5), [("fixedValue", 1.0)] * big.npatch)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.div(neon.SurfaceField(dm, F), "upwind"),
                 neon.laplacian(neon.SurfaceField(dm, np.full(big.nif + big.nbf, 1e-2)), -1.0)], 0.1, T)
    x = T.internal.clone()
    stats = neon.Batch(ls, ranges).solve(x, rel_tol=1e-10, max_iter=500, precision=precision,
                                         method=abi.SOLVER_BICGSTAB)
    for k in range(len(ranges) // 2):
        lo, hi = int(ranges[2 * k]), int(ranges[2 * k + 1])
        y = T.internal.clone()
        s1 = neon.Batch(ls, np.asarray([lo, hi], np.int32)).solve(y, rel_tol=1e-10, max_iter=500,
                                                                  precision=precision,
                                                                  method=abi.SOLVER_BICGSTAB)
        assert stats[k].status == s1[0].status == abi.OK and stats[k].num_iter == s1[0].num_iter
        np.testing.assert_array_equal(x[lo:hi].cpu().numpy(), y[lo:hi].cpu().numpy())


def test_bicg_bit_exact_on_nonsymmetric_system(cuda):
    """BiCG (Ginkgo's solver::Bicg, the mapping of OpenFOAM's PBiCG,
    fvSolution.cpp:24) on implicit upwind convection against the oracle's
    restatement, bit for bit; the shadow residual runs on A^T."""
    hm, dm, T, o, ls, v, r = convection_case()
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-10, max_iter=500, method=abi.SOLVER_BICG)
    xo = T.host().copy()
    so = o.solve(v, r, xo, rel_tol=1e-10, max_iter=500, method=2)
    assert st.status == so.status == abi.OK and st.num_iter == so.num_iter > 3
    assert (st.init_res_norm, st.final_res_norm) == (so.init_res_norm, so.final_res_norm)
    np.testing.assert_array_equal(x.cpu().numpy(), xo)
    assert np.linalg.norm(o.apply_operator(v, r, 1, xo)) <= 1e-10 * so.init_res_norm
    st = ls.solve(T.internal.clone(), rel_tol=1e-14, max_iter=2, method=abi.SOLVER_BICG)
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_iter == 2
    with pytest.raises(abi.FvgbError) as e:
        ls.solve(T.internal.clone(), precision=abi.PREC_MIXED_IR, method=abi.SOLVER_BICG)
    assert e.value.status == abi.ERR_UNSUPPORTED


def test_bicg_batch_equals_alone_and_symmetric_case(cuda):
    """Batched BiCG gives every case its bits alone; on a symmetric system BiCG
    reaches the CG solution."""
    parts = [mesh.box(7, 6, 5, jitter=0.1, seed=s) for s in (1, 2, 3)]
    big, ranges, _ = mesh.concat(parts)
    ranges = np.asarray(ranges, np.int32)
    dm = DeviceMesh(big)
    o = Oracle(big)
    U = np.array([0.3, -1.0, 0.5])
    F = o.flux_vec(np.tile(U, big.n), np.tile(U, big.nbf))
    T = neon.VolumeField(dm, np.full(big.n, 0.5), [("fixedValue", 1.0)] * big.npatch)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.div(neon.SurfaceField(dm, F), "upwind"),
                 neon.laplacian(neon.SurfaceField(dm, np.full(big.nif + big.nbf, 1e-2)), -1.0)], 0.1, T)
    x = T.internal.clone()
    stats = neon.Batch(ls, ranges).solve(x, rel_tol=1e-10, max_iter=500, method=abi.SOLVER_BICG)
    for k in range(len(ranges) // 2):
        lo, hi = int(ranges[2 * k]), int(ranges[2 * k + 1])
        y = T.internal.clone()
        s1 = neon.Batch(ls, np.asarray([lo, hi], np.int32)).solve(y, rel_tol=1e-10, max_iter=500,
                                                                  method=abi.SOLVER_BICG)
        assert stats[k].status == s1[0].status == abi.OK and stats[k].num_iter == s1[0].num_iter
        np.testing.assert_array_equal(x[lo:hi].cpu().numpy(), y[lo:hi].cpu().numpy())
    hm, dm2, T2, o2, ls2, v2, r2 = solve_case(12, 10, 8)
    xb, xc = T2.internal.clone(), T2.internal.clone()
    assert ls2.solve(xb, rel_tol=1e-12, method=abi.SOLVER_BICG).status == abi.OK
    assert ls2.solve(xc, rel_tol=1e-12).status == abi.OK
    np.testing.assert_allclose(xb.cpu().numpy(), xc.cpu().numpy(), rtol=1e-9, atol=0)
