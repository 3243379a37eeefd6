"""PISO helpers and the neoIcoFoam loop on the GPU against the CPU oracle.

The reference checks rAU at 1e-15, HbyA and the matrix flux at 1e-14 against
OpenFOAM (test/test_pressureVelocityCoupling.cpp:130-277); here the GPU must
equal the Serial-order restatement bit for bit, including a few full PISO
steps of a jittered lid-driven cavity with two correctors and the pressure
reference (mixed-precision pressure solves are compared on the FP64 residual).
"""
import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, apps, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh
from oracle.apps import CavityPisoCPU
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def test_piso_helpers_bit_exact(cuda):
    hm = mesh.box(9, 8, 6, jitter=0.1, seed=21)
    dm = DeviceMesh(hm)
    o = Oracle(hm)
    rng = np.random.default_rng(0)
    nf = hm.nif + hm.nbf
    ubcs = [("fixedValue", rng.standard_normal(3)), ("noSlip", 0.0), ("zeroGradient", 0.0),
            ("fixedValue", [1.0, 0.0, 0.0]), ("noSlip", 0.0), ("zeroGradient", 0.0)]
    U = neon.VolumeField(dm, rng.standard_normal(3 * hm.n), ubcs, ncomp=3)
    phi = neon.SurfaceField(dm, rng.standard_normal(nf))
    nu = neon.SurfaceField(dm, np.exp(rng.standard_normal(nf)))
    old = rng.standard_normal(3 * hm.n)
    ls = neon.LinearSystem(dm, 3)
    ls.assemble([neon.ddt(neon.dev(old)), neon.div(phi, "linear"), neon.laplacian(nu, -1.0)], 1e-3, U)
    v, r, bm, br = [t.cpu().numpy() for t in ls.export()]
    ov, orr, obm, obr = o.assemble(3, [(0, 0, 1.0, old, None), (2, 0, 1.0, None, phi.host()),
                                       (1, 0, -1.0, None, nu.host())], 1e-3, U.types, U.ref.cpu().numpy(),
                                   U.boundary.cpu().numpy())
    np.testing.assert_array_equal(v, ov)
    np.testing.assert_array_equal(r, orr)
    Uh, Ubh = U.host(), U.boundary.cpu().numpy()
    rAU = torch.empty(hm.n, dtype=torch.float64, device="cuda")
    H = torch.empty(3 * hm.n, dtype=torch.float64, device="cuda")
    L, s = abi.lib(), torch.cuda.current_stream().cuda_stream
    abi.check(L.fvgb_piso_rau_hbya(ls.handle, abi.ptr(U.internal), abi.ptr(rAU), abi.ptr(H), s))
    orau, oH = o.rau_hbya(ov, orr, Uh)
    np.testing.assert_array_equal(rAU.cpu().numpy(), orau)
    np.testing.assert_array_equal(H.cpu().numpy(), oH)
    # constrainHbyA on the non-assignable (fixed value) patches
    assignable = np.asarray([0, 0, 1, 0, 0, 1], np.int32)
    Hb = neon.dev(rng.standard_normal(3 * hm.nbf))
    oHb = Hb.cpu().numpy().copy()
    abi.check(L.fvgb_piso_constrain_hbya(dm.handle, abi.ptr(assignable), abi.ptr(U.boundary), abi.ptr(Hb), s))
    o.constrain_hbya(assignable, Ubh, oHb)
    np.testing.assert_array_equal(Hb.cpu().numpy(), oHb)
    # flux(HbyA)
    F = torch.empty(nf, dtype=torch.float64, device="cuda")
    abi.check(L.fvgb_flux_vec(dm.handle, abi.ptr(H), abi.ptr(Hb), abi.ptr(F), s))
    oF = o.flux_vec(oH, oHb)
    np.testing.assert_array_equal(F.cpu().numpy(), oF)
    # pressure system, face and cell velocity updates
    p = neon.VolumeField(dm, rng.standard_normal(hm.n), [("zeroGradient", 0.0), ("fixedValue", 0.5)] +
                         [("zeroGradient", 0.0)] * 4)
    rAUf = neon.SurfaceField(dm, o.interp_linear(1, orau, np.ascontiguousarray(orau[hm.bcells])))
    pe = neon.LinearSystem(dm, 1)
    pe.assemble([neon.laplacian(rAUf), neon.div_flux(neon.SurfaceField(dm, oF), -1.0)], 1e-3, p)
    pv, pr, pbm, pbr = [t.cpu().numpy() for t in pe.export()]
    opv, opr, opbm, opbr = o.assemble(1, [(1, 0, 1.0, None, rAUf.host()), (5, 0, -1.0, None, oF)], 1e-3,
                                      p.types, p.ref.cpu().numpy(), p.boundary.cpu().numpy())
    for a, b in ((pv, opv), (pr, opr), (pbm, opbm), (pbr, opbr)):
        np.testing.assert_array_equal(a, b)
    phi_new = torch.empty(nf, dtype=torch.float64, device="cuda")
    abi.check(L.fvgb_piso_face_update(pe.handle, abi.ptr(F), abi.ptr(p.internal), abi.ptr(phi_new), s))
    np.testing.assert_array_equal(phi_new.cpu().numpy(), o.face_update(opv, opbm, opbr, oF, p.host()))
    Unew = torch.empty(3 * hm.n, dtype=torch.float64, device="cuda")
    abi.check(L.fvgb_piso_velocity_update(dm.handle, abi.ptr(H), abi.ptr(rAU), abi.ptr(p.internal),
                                          abi.ptr(p.boundary), abi.ptr(Unew), s))
    np.testing.assert_array_equal(Unew.cpu().numpy(),
                                  o.velocity_update(oH, orau, p.host(), p.boundary.cpu().numpy()[:hm.nbf].copy()))


def test_cavity_piso_steps_bit_exact(cuda):
    gpu = apps.CavityPiso(n=24, jitter=0.05, seed=7, dt=5e-3, n_corr=2)
    cpu = CavityPisoCPU(gpu.hm, dt=5e-3, n_corr=2)
    for _ in range(4):
        gpu.step()
        cpu.step()
    assert [s[0] for s in gpu.stats] == [s[0] for s in cpu.stats]
    np.testing.assert_array_equal(gpu.p.host(), cpu.p)
    np.testing.assert_array_equal(gpu.U.host(), cpu.U)
    np.testing.assert_array_equal(gpu.phi.host(), cpu.phi)
    # the lid drives a clockwise vortex: u < 0 near the bottom, > 0 near the lid
    Uc = cpu.U.reshape(-1, 3)
    y = gpu.hm.C[:, 1]
    assert Uc[y > 0.9, 0].mean() > 0 and Uc[y < 0.3, 0].mean() < 0


def test_cavity_mixed_pressure_matches_fp64(cuda):
    a = apps.CavityPiso(n=32, jitter=0.05, seed=3, dt=5e-3, n_corr=2)
    b = apps.CavityPiso(n=32, jitter=0.05, seed=3, dt=5e-3, n_corr=2, precision=abi.PREC_MIXED_IR)
    for _ in range(3):
        a.step()
        b.step()
    assert all(s[4] == abi.OK for s in b.stats)
    assert all(s[3] <= 1.0001e-8 * s[2] for s in b.stats)      # FP64 residual reached each solve
    dU = np.abs(a.U.host() - b.U.host()).max()
    dp = np.abs(a.p.host() - b.p.host()).max()
    assert dU < 1e-6 and dp < 1e-6 * max(1.0, np.abs(a.p.host()).max())


def test_ddt_corr_and_constrain_pressure_bit_exact(cuda):
    hm = mesh.box(9, 8, 6, jitter=0.15, seed=22)
    dm, o = DeviceMesh(hm), Oracle(hm)
    rng = np.random.default_rng(1)
    nf = hm.nif + hm.nbf
    ubcs = [("fixedValue", rng.standard_normal(3)), ("noSlip", 0.0), ("zeroGradient", 0.0),
            ("fixedValue", [1.0, 0.0, 0.0]), ("calculated", rng.standard_normal(3)), ("zeroGradient", 0.0)]
    U = neon.VolumeField(dm, rng.standard_normal(3 * hm.n), ubcs, ncomp=3)
    phi_old = rng.standard_normal(nf)
    phi_old[::7] = 0.0                                   # |phi_old| = 0: the 1e-15 guard
    rAUf = np.exp(rng.standard_normal(nf))
    base = rng.standard_normal(nf)
    out = neon.dev(base)
    L, s = abi.lib(), torch.cuda.current_stream().cuda_stream
    d_phi_old, d_rAUf = neon.dev(phi_old), neon.dev(rAUf)   # held until the kernels have run
    abi.check(L.fvgb_piso_ddt_corr(dm.handle, abi.ptr(U.types), abi.ptr(U.internal), abi.ptr(U.boundary),
                                   abi.ptr(d_phi_old), abi.ptr(d_rAUf), 2e-3, abi.ptr(out), s))
    ref = o.ddt_corr(U.types, U.host(), U.boundary.cpu().numpy()[:3 * hm.nbf].copy(), phi_old, rAUf, 2e-3,
                     base.copy())
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    fixed = np.concatenate([np.arange(int(hm.patch_offsets[p]), int(hm.patch_offsets[p + 1]))
                            for p in (0, 1, 3)]) + hm.nif
    np.testing.assert_array_equal(ref[fixed], base[fixed])  # no correction where U is a fixed value
    # constrainPressure on two fixedFluxPressure patches
    flags = np.asarray([0, 1, 0, 0, 1, 0], np.int32)
    phiHbyA = rng.standard_normal(nf)
    pref = rng.standard_normal(hm.nbf)
    dref, d_phiHbyA = neon.dev(pref), neon.dev(phiHbyA)
    abi.check(L.fvgb_piso_constrain_pressure(dm.handle, abi.ptr(flags), abi.ptr(d_phiHbyA),
                                             abi.ptr(U.boundary), abi.ptr(d_rAUf), abi.ptr(dref), s))
    oref = o.constrain_pressure(flags, phiHbyA, U.boundary.cpu().numpy()[:3 * hm.nbf].copy(), rAUf, pref.copy())
    np.testing.assert_array_equal(dref.cpu().numpy(), oref)


@pytest.mark.parametrize("opts", [dict(ddt_corr=True), dict(corrected=True, n_non_orth=1),
                                  dict(ddt_corr=True, corrected=True, n_non_orth=1)])
def test_cavity_icofoam_options_bit_exact(cuda, opts):
    """icoFoam's ddtCorr and non-orthogonal pressure correctors, which the
    reference's loop leaves out, on a strongly jittered cavity: GPU = oracle."""
    gpu = apps.CavityPiso(n=20, jitter=0.25, seed=5, dt=5e-3, n_corr=2, **opts)
    cpu = CavityPisoCPU(gpu.hm, dt=5e-3, n_corr=2, **opts)
    for _ in range(3):
        gpu.step()
        cpu.step()
    assert [s[0] for s in gpu.stats] == [s[0] for s in cpu.stats]
    np.testing.assert_array_equal(gpu.p.host(), cpu.p)
    np.testing.assert_array_equal(gpu.U.host(), cpu.U)
    np.testing.assert_array_equal(gpu.phi.host(), cpu.phi)
