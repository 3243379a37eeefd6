"""GPU explicit operators against the CPU oracle: bit-exact.

The oracle runs the reference's Serial face loops; the GPU gathers per cell in
ascending face order with no multiply-add contraction, so every value must be
identical (the reference's own tolerance for these operators is 1e-15,
test/test_operators.cpp:61,113).
"""
import numpy as np
import pytest
import torch

from conftest import load_polymesh, unpack_reference_files
from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def meshes():
    yield "setup_operator", load_polymesh("setup_operator")[0]
    yield "setup_stencil3D", load_polymesh("setup_stencil3D")[0]
    yield "box_jitter", mesh.box(9, 7, 5, 1.0, 0.7, 0.5, jitter=0.15, seed=11)
    yield "box2d_jitter", mesh.box(17, 13, 1, two_d=True, jitter=0.1, seed=5)


def rand_bcs(hm, rng, ncomp):
    kinds = ["fixedValue", "zeroGradient", "fixedGradient", "calculated"]
    out = []
    for p in range(hm.npatch):
        k = kinds[p % 4]
        nfp = int(hm.patch_offsets[p + 1] - hm.patch_offsets[p])
        out.append((k, rng.standard_normal(nfp * ncomp)))
    return out


def host_bc(vf: neon.VolumeField):
    return vf.types, vf.ref.cpu().numpy(), vf.boundary.cpu().numpy()


@pytest.mark.parametrize("name,hm", list(meshes()))
@pytest.mark.parametrize("ncomp", [1, 3])
@pytest.mark.parametrize("tile", [2, 4, 8])
def test_interpolation_div_laplacian(cuda, name, hm, ncomp, tile):
    """Every face-pass tile (faces per thread) gives the oracle's bits."""
    rng = np.random.default_rng(hash(name) % 2**32 + ncomp)
    dm = DeviceMesh(hm)
    abi.check(abi.lib().fvgb_mesh_face_tile(dm.handle, tile))
    o = Oracle(hm)
    nf = hm.nif + hm.nbf
    T = neon.VolumeField(dm, rng.standard_normal(hm.n * ncomp), rand_bcs(hm, rng, ncomp), ncomp)
    types, ref, Tb = host_bc(T)
    Th = T.host()
    # boundary correction
    Tb_o = np.zeros(hm.nbf * ncomp)
    o.bc_correct(ncomp, types, ref, Th, Tb_o)
    np.testing.assert_array_equal(Tb[:hm.nbf * ncomp], Tb_o)
    flux = neon.SurfaceField(dm, rng.standard_normal(nf))
    fh = flux.host()
    lin = neon.SurfaceInterpolation(dm, "linear").interpolate(T).host()
    np.testing.assert_array_equal(lin, o.interp_linear(ncomp, Th, Tb_o))
    upw = neon.SurfaceInterpolation(dm, "upwind").interpolate(T, flux=flux).host()
    np.testing.assert_array_equal(upw, o.interp_upwind(ncomp, fh, Th, Tb_o))
    for scheme in ("linear", "upwind"):
        for coeff in (1.0, -0.37):
            base = rng.standard_normal(hm.n * ncomp)
            out = neon.dev(base)
            neon.GaussGreenDiv(dm, scheme).div(out, flux, T, coeff)
            ref_out = o.div(neon._scheme(scheme), ncomp, fh, Th, Tb_o, coeff, base.copy())
            np.testing.assert_array_equal(out.cpu().numpy(), ref_out)
    gamma = neon.SurfaceField(dm, np.exp(rng.standard_normal(nf)))
    for coeff in (1.0, 2.5):
        base = rng.standard_normal(hm.n * ncomp)
        out = neon.dev(base)
        neon.GaussGreenLaplacian(dm).laplacian(out, gamma, T, coeff)
        ref_out = o.laplacian(ncomp, gamma.host(), Th, Tb_o, coeff, base.copy())
        np.testing.assert_array_equal(out.cpu().numpy(), ref_out)


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.mark.parametrize("name,hm", list(meshes()))
def test_zero_outputs_and_signed_zeros(cuda, name, hm):
    """The gathers take the first term of a cell's sum from +0 on the integer
    pipes (+-x, a zero result +0). Outputs of +0, of -0, and of zeros mixed
    with values inside a warp, and fluxes with +-0 faces, all give the
    oracle's bits with the sign of every zero (compared as integers)."""
    rng = np.random.default_rng(17)
    dm = DeviceMesh(hm)
    o = Oracle(hm)
    nf = hm.nif + hm.nbf
    T = neon.VolumeField(dm, rng.standard_normal(hm.n), rand_bcs(hm, rng, 1))
    types, ref, Tb = host_bc(T)
    Th, Tb = T.host(), Tb[:hm.nbf].copy()
    fl = rng.standard_normal(nf)
    fl[::3] = 0.0
    fl[1::5] = -0.0
    flux = neon.SurfaceField(dm, fl)
    mixed = rng.standard_normal(3 * hm.n)
    mixed[::2] = 0.0
    mixed[1::7] = -0.0
    bases = {"+0": np.zeros(3 * hm.n), "-0": np.full(3 * hm.n, -0.0), "mixed": mixed}
    gamma = neon.SurfaceField(dm, np.exp(rng.standard_normal(nf)))
    for bname, b3 in bases.items():
        b1 = b3[:hm.n].copy()
        for scheme in ("linear", "upwind"):
            out = neon.dev(b1)
            neon.GaussGreenDiv(dm, scheme).div(out, flux, T, 1.0)
            want = o.div(neon._scheme(scheme), 1, fl, Th, Tb, 1.0, b1.copy())
            assert np.array_equal(bits(out.cpu().numpy()), bits(want)), (bname, scheme)
        out = neon.dev(b1)
        neon.GaussGreenLaplacian(dm).laplacian(out, gamma, T, 1.0)
        want = o.laplacian(1, gamma.host(), Th, Tb, 1.0, b1.copy())
        assert np.array_equal(bits(out.cpu().numpy()), bits(want)), bname
        out = neon.GaussGreenGrad(dm).grad(T, 1.0, neon.dev(b3))
        assert np.array_equal(bits(out.cpu().numpy()), bits(o.grad(Th, Tb, 1.0, b3.copy()))), bname


@pytest.mark.parametrize("name,hm", list(meshes()))
@pytest.mark.parametrize("tile", [2, 4, 8])
def test_grad_sngrad(cuda, name, hm, tile):
    rng = np.random.default_rng(3)
    dm = DeviceMesh(hm)
    abi.check(abi.lib().fvgb_mesh_face_tile(dm.handle, tile))
    o = Oracle(hm)
    T = neon.VolumeField(dm, rng.standard_normal(hm.n), rand_bcs(hm, rng, 1))
    Th, Tb = T.host(), T.boundary.cpu().numpy()[:hm.nbf].copy()
    for coeff in (1.0, 0.3):
        base = rng.standard_normal(3 * hm.n)
        out = neon.GaussGreenGrad(dm).grad(T, coeff, neon.dev(base))
        np.testing.assert_array_equal(out.cpu().numpy(), o.grad(Th, Tb, coeff, base.copy()))
    sg = neon.FaceNormalGradient(dm).faceNormalGrad(T).host()
    np.testing.assert_array_equal(sg, o.sngrad(Th, Tb))


def test_golden_div_grad_on_gpu(cuda):
    """The reference golden case end to end on the GPU."""
    hm, d = load_polymesh("setup_operator")
    dm = DeviceMesh(hm)
    T = neon.VolumeField(dm, d["field_T"], [("zeroGradient", 0.0)])
    flux = np.zeros(hm.nif + hm.nbf)
    flux[:hm.nif] = d["field_phi"]
    out = torch.zeros(hm.n, dtype=torch.float64, device="cuda")
    neon.GaussGreenDiv(dm, ("Gauss", "linear")).div(out, neon.SurfaceField(dm, flux), T, 1.0)
    g = d["field_divT_Serial"]
    assert np.max(np.abs(out.cpu().numpy() - g)) / np.abs(g).max() < 2e-15
    grad = neon.GaussGreenGrad(dm).grad(T).cpu().numpy().reshape(-1, 3)
    np.testing.assert_allclose(grad, d["field_gradT_Serial"], rtol=0, atol=1e-15 * np.abs(grad).max())


def test_golden_case_from_openfoam_files(cuda, tmp_path):
    """The same case read from the reference's own OpenFOAM files (polyMesh,
    0/T with its zeroGradient walls, 0/phi), the result written as field files
    (ascii and binary) and read back bit for bit."""
    root = unpack_reference_files(tmp_path)
    pm = mesh.PolyMesh(root / "setup_operator" / "constant" / "polyMesh")
    case = root / "setup_operator" / "0"
    dm = DeviceMesh(pm.host)
    T = neon.read_vol_field(dm, pm, case / "T", name="T")
    _, _, phib = pm.read_bc(case / "phi")
    flux = np.concatenate([pm.read_field(case / "phi", surface=True), phib])
    div = neon.VolumeField(dm, np.zeros(pm.host.n), name="divT")
    neon.GaussGreenDiv(dm, ("Gauss", "linear")).div(div.internal, neon.SurfaceField(dm, flux), T, 1.0)
    _, d = load_polymesh("setup_operator")
    g = d["field_divT_Serial"]
    assert np.max(np.abs(div.host() - g)) / np.abs(g).max() < 2e-15
    grad = neon.GaussGreenGrad(dm).grad(T).cpu().numpy()
    np.testing.assert_allclose(grad.reshape(-1, 3), d["field_gradT_Serial"], rtol=0,
                               atol=1e-15 * np.abs(grad).max())
    div.correctBoundaryConditions()
    for binary in (False, True):
        neon.write(div, pm, tmp_path / "divT", binary=binary)
        np.testing.assert_array_equal(pm.read_field(tmp_path / "divT"), div.host())
        back = neon.read_vol_field(dm, pm, tmp_path / "divT")
        np.testing.assert_array_equal(back.boundary.cpu().numpy(), div.boundary.cpu().numpy())


def advection_case(n=64):
    """64x64x1 unit square, U = (1, 0.5, 0), Gaussian blob at (0.25, 0.25), sigma 0.05."""
    hm = mesh.box(n, n, 1, 1.0, 1.0, 1.0 / n, two_d=True)
    U = np.array([1.0, 0.5, 0.0])
    o = Oracle(hm)
    flux = o.flux_vec(np.tile(U, hm.n), np.tile(U, hm.nbf))
    x, y = hm.C[:, 0], hm.C[:, 1]
    T0 = np.exp(-((x - 0.25) ** 2 + (y - 0.25) ** 2) / (2 * 0.05 ** 2))
    return hm, o, flux, T0


def test_advection_config_bit_exact(cuda):
    """Explicit upwind advection, forward Euler dt 1e-3, 100 steps: GPU == oracle bit for bit."""
    hm, o, flux, T0 = advection_case(64)
    dm = DeviceMesh(hm)
    types = np.full(hm.npatch, abi.BC_FIXED_GRADIENT, np.int32)     # zeroGradient walls
    ref = np.zeros(hm.nbf)
    Tb0 = T0[hm.bcells].copy()
    # oracle
    T, Tb = T0.copy(), Tb0.copy()
    for _ in range(100):
        T, Tb = o.advect_euler(flux, T, Tb, 1e-3, types, ref)
    # GPU: flux through the ABI, then 100 fused steps ping-ponging two buffers
    fg = neon.dev(np.zeros(hm.nif + hm.nbf))
    Ug, Ubg = neon.dev(np.tile([1.0, 0.5, 0.0], hm.n)), neon.dev(np.tile([1.0, 0.5, 0.0], hm.nbf))
    abi.check(abi.lib().fvgb_flux_vec(dm.handle, abi.ptr(Ug), abi.ptr(Ubg), abi.ptr(fg), neon._stream()))
    np.testing.assert_array_equal(fg.cpu().numpy(), flux)
    a, ab = neon.dev(T0), neon.dev(Tb0)
    b, bb = torch.empty_like(a), torch.empty_like(ab)
    refd = neon.dev(ref)
    bc = abi.BC(abi.ptr(types), abi.ptr(refd))
    import ctypes as C
    for _ in range(100):
        abi.check(abi.lib().fvgb_advect_euler_step(dm.handle, abi.ptr(fg), abi.ptr(a), abi.ptr(ab), 1e-3,
                                                   C.byref(bc), abi.ptr(b), abi.ptr(bb), neon._stream()))
        a, b, ab, bb = b, a, bb, ab
    np.testing.assert_array_equal(a.cpu().numpy(), T)
    np.testing.assert_array_equal(ab.cpu().numpy(), Tb)
    assert abs(T.sum() - T0.sum()) / T0.sum() < 1e-2   # nearly conservative (outflow of a small tail)


@pytest.mark.parametrize("n,nsteps", [(64, 100), (64, 7), (300, 5), (8, 0)])
def test_advection_many_steps_in_one_call(cuda, n, nsteps):
    """fvgb_advect_euler_steps (the one-pass step kernel for meshes up to 65536
    cells, the two-pass step above) gives the bits of nsteps single steps and of
    the oracle."""
    from foamadapter_gb300 import apps

    a, b = apps.Advection(n=n), apps.Advection(n=n)
    hm = a.hm
    T0, Tb0 = a.T.host().copy(), a.T.boundary.cpu().numpy()[:hm.nbf].copy()
    a.run(nsteps)
    for _ in range(nsteps):
        b.step()
    np.testing.assert_array_equal(a.T.host(), b.T.host())
    np.testing.assert_array_equal(a.T.boundary.cpu().numpy()[:hm.nbf], b.T.boundary.cpu().numpy()[:hm.nbf])
    o = Oracle(hm)
    T, Tb = T0, Tb0
    for _ in range(nsteps):
        T, Tb = o.advect_euler(a.flux.host(), T, Tb, a.dt, np.full(hm.npatch, 2, np.int32), np.zeros(hm.nbf))
    np.testing.assert_array_equal(a.T.host(), T)
