"""Non-orthogonal correction (`Gauss linear corrected`) on the GPU through the
C ABI, bit for bit against the oracle: the explicit corrected laplacian and
snGrad, the face-flux correction, the corrected implicit laplacian (assembly,
solve, step graph), and the refusal on a mesh without cell centres."""
import ctypes as C

import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def rand_bcs(hm, rng, ncomp):
    kinds = ["fixedValue", "zeroGradient", "fixedGradient", "calculated"]
    return [(kinds[p % 4], rng.standard_normal(int(hm.patch_offsets[p + 1] - hm.patch_offsets[p]) * ncomp))
            for p in range(hm.npatch)]


@pytest.mark.parametrize("dims,jitter", [((13, 11, 9), 0.25), ((40, 37, 1), 0.2), ((1, 1, 1), 0.0)])
@pytest.mark.parametrize("ncomp", [1, 3])
def test_explicit_corrected_laplacian_and_flux(cuda, dims, jitter, ncomp):
    hm = mesh.box(*dims, jitter=jitter, seed=5, two_d=dims[2] == 1)
    dm, o = DeviceMesh(hm), Oracle(hm)
    rng = np.random.default_rng(6)
    T = neon.VolumeField(dm, rng.standard_normal(hm.n * ncomp), rand_bcs(hm, rng, ncomp), ncomp=ncomp)
    Th, Tb = T.host(), T.boundary.cpu().numpy()[:hm.nbf * ncomp].copy()
    gamma = np.exp(rng.standard_normal(hm.nif + hm.nbf))
    for coeff in (1.0, -0.3):
        base = rng.standard_normal(hm.n * ncomp)
        out = neon.dev(base)
        neon.GaussGreenLaplacian(dm, "Gauss linear corrected").laplacian(out, neon.SurfaceField(dm, gamma), T, coeff)
        ref = o.laplacian_corrected(ncomp, gamma, Th, Tb, coeff, base.copy())
        np.testing.assert_array_equal(out.cpu().numpy(), ref)
    fbase = rng.standard_normal((hm.nif + hm.nbf) * ncomp)
    fc = neon.nonorth_flux(neon.SurfaceField(dm, gamma), T, -0.7, neon.SurfaceField(dm, fbase.copy(), ncomp=ncomp))
    np.testing.assert_array_equal(fc.host(), o.nonorth_flux(ncomp, gamma, Th, Tb, -0.7, fbase.copy()))
    if ncomp == 1:
        sg = neon.FaceNormalGradient(dm, "corrected").faceNormalGrad(T).host()
        np.testing.assert_array_equal(sg, o.sngrad_corrected(Th, Tb))


def corrected_system(hm, seed=0):
    dm, o = DeviceMesh(hm), Oracle(hm)
    rng = np.random.default_rng(seed)
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T = neon.VolumeField(dm, 300.0 + rng.standard_normal(hm.n), bcs)
    gamma = np.exp(rng.standard_normal(hm.nif + hm.nbf))
    return dm, o, T, gamma


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_corrected_implicit_laplacian_assembly_and_solve(cuda, precision):
    hm = mesh.box(17, 15, 13, jitter=0.2, seed=8)
    dm, o, T, gamma = corrected_system(hm)
    T_old = T.internal.clone()
    ls = neon.LinearSystem(dm)
    terms = [neon.ddt(T_old), neon.laplacian(neon.SurfaceField(dm, gamma), -1.0, "corrected", field=T.internal)]
    ls.assemble(terms, 0.01, T)
    v, r, bm, br = [t.cpu().numpy() for t in ls.export()]
    Th, Tb = T.host(), T.boundary.cpu().numpy()[:hm.nbf].copy()
    ov, orhs, obm, obr = o.assemble(1, [(abi.TERM_DDT, 0, 1.0, Th.copy(), None),
                                        (abi.TERM_LAPLACIAN, abi.SCHEME_CORRECTED, -1.0, Th.copy(), gamma)],
                                    0.01, T.types, T.ref.cpu().numpy(), Tb)
    np.testing.assert_array_equal(v, ov)
    np.testing.assert_array_equal(r, orhs)
    # the correction is there: the rhs differs from the uncorrected assembly
    ls2 = neon.LinearSystem(dm)
    ls2.assemble([neon.ddt(T_old), neon.laplacian(neon.SurfaceField(dm, gamma), -1.0)], 0.01, T)
    assert not np.array_equal(ls2.export()[1].cpu().numpy(), r)
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-10, max_iter=2000, precision=precision)
    xo = Th.copy()
    so = o.solve(ov, orhs, xo, rel_tol=1e-10, max_iter=2000, precision=1 if precision == abi.PREC_MIXED_IR else 0)
    assert st.status == so.status == abi.OK and st.num_iter == so.num_iter
    np.testing.assert_array_equal(x.cpu().numpy(), xo)


def test_corrected_step_graph_equals_separate_calls(cuda):
    """A captured time step whose laplacian is corrected (the correction of the
    current T recomputed inside the graph every launch)."""
    L, s = abi.lib(), torch.cuda.current_stream().cuda_stream
    out = []
    for use_graph in (False, True):
        hm = mesh.box(14, 12, 10, jitter=0.2, seed=9)
        dm, _, T, gamma = corrected_system(hm, seed=1)
        T_old = T.internal.clone()
        ls = neon.LinearSystem(dm)
        g = neon.SurfaceField(dm, gamma)
        terms = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(T_old),
                                                      neon.laplacian(g, -1.0, "corrected", field=T.internal))])
        bc = T.bc_struct()
        cfg = abi.SolverCfg(1e-9, 0.0, 2000, abi.PREC_FP64, 0.1, 1000, 50, 1)
        stats = torch.zeros(8, dtype=torch.int32, device="cuda")
        if use_graph:
            step = C.c_void_p()
            abi.check(L.fvgb_step_create(ls.handle, None, terms, 2, 0.01, C.byref(bc), abi.ptr(T.internal),
                                         abi.ptr(T.boundary), abi.ptr(T_old), C.byref(cfg), abi.ptr(stats),
                                         C.byref(step)))
            for _ in range(3):
                abi.check(L.fvgb_step_launch(step, s))
            torch.cuda.synchronize()
            abi.check(L.fvgb_step_destroy(step))
        else:
            for _ in range(3):
                T_old.copy_(T.internal)
                abi.check(L.fvgb_assemble(ls.handle, terms, 2, 0.01, C.byref(bc), abi.ptr(T.boundary), s))
                abi.check(L.fvgb_solve_async(ls.handle, abi.ptr(T.internal), C.byref(cfg), abi.ptr(stats), s))
                T.correctBoundaryConditions()
            torch.cuda.synchronize()
        out.append((T.internal.cpu().numpy(), stats.cpu().numpy()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_corrected_needs_cell_centres(cuda):
    hm = mesh.box(5, 4, 3, jitter=0.1, seed=2)
    d = hm.desc()
    d.cell_centres = None
    h = C.c_void_p()
    abi.check(abi.lib().fvgb_mesh_create(C.byref(d), C.byref(h)))
    try:
        phi = torch.zeros(hm.n, dtype=torch.float64, device="cuda")
        phib = torch.zeros(hm.nbf, dtype=torch.float64, device="cuda")
        gam = torch.ones(hm.nif + hm.nbf, dtype=torch.float64, device="cuda")
        r = abi.lib().fvgb_laplacian_explicit_corrected(h, 1, abi.ptr(gam), abi.ptr(phi), abi.ptr(phib), 1.0,
                                                        abi.ptr(phi), None)
        assert r == abi.ERR_INVALID_ARG
        # the uncorrected operator is unaffected
        abi.check(abi.lib().fvgb_laplacian_explicit(h, 1, abi.ptr(gam), abi.ptr(phi), abi.ptr(phib), 1.0,
                                                    abi.ptr(phi), None))
    finally:
        abi.lib().fvgb_mesh_destroy(h)
