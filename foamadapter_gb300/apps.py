"""The reference's example solvers as drivers of the GB300 path.

* ``Advection``: explicit scalar advection, Gauss upwind, forward Euler
  (test/test_advection.cpp:116-170 with a uniform velocity).
* ``HeatTransfer``: ddt(T) - laplacian(kappa, T) = 0, implicit Euler
  (examples/heatTransfer/heatTransfer.cpp:60-83).
* ``CavityPiso``: neoIcoFoam's PISO loop without momentum predictor
  (examples/neoIcoFoam/neoIcoFoam.cpp:80-170).

Every operation is a call into libfvgb; torch only allocates device memory.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import abi, mesh, neon
from .mesh import DeviceMesh


def _s():
    return torch.cuda.current_stream().cuda_stream


class Advection:
    """Explicit upwind advection of a Gaussian blob with a uniform velocity."""

    def __init__(self, n=64, U=(1.0, 0.5, 0.0), centre=(0.25, 0.25), sigma=0.05, dt=1e-3):
        self.hm = mesh.box(n, n, 1, 1.0, 1.0, 1.0 / n, two_d=True)
        self.dm = DeviceMesh(self.hm)
        hm = self.hm
        self.dt = dt
        x, y = hm.C[:, 0], hm.C[:, 1]
        T0 = np.exp(-((x - centre[0]) ** 2 + (y - centre[1]) ** 2) / (2 * sigma ** 2))
        self.T = neon.VolumeField(self.dm, T0, [("zeroGradient", 0.0)] * hm.npatch)
        Ud = neon.dev(np.tile(U, hm.n))
        Ub = neon.dev(np.tile(U, hm.nbf))
        self.flux = neon.SurfaceField(self.dm)
        abi.check(abi.lib().fvgb_flux_vec(self.dm.handle, abi.ptr(Ud), abi.ptr(Ub), abi.ptr(self.flux.values), _s()))
        self.T2 = torch.empty_like(self.T.internal)
        self.Tb2 = torch.empty_like(self.T.boundary)

    def step(self):
        bc = self.T.bc_struct()
        abi.check(abi.lib().fvgb_advect_euler_step(self.dm.handle, abi.ptr(self.flux.values),
                                                   abi.ptr(self.T.internal), abi.ptr(self.T.boundary), self.dt,
                                                   C.byref(bc), abi.ptr(self.T2), abi.ptr(self.Tb2), _s()))
        self.T.internal, self.T2 = self.T2, self.T.internal
        self.T.boundary, self.Tb2 = self.Tb2, self.T.boundary

    def run(self, nsteps):
        """nsteps steps in one call (fvgb_advect_euler_steps): the same bits as
        nsteps calls of step()."""
        bc = self.T.bc_struct()
        abi.check(abi.lib().fvgb_advect_euler_steps(self.dm.handle, abi.ptr(self.flux.values),
                                                    abi.ptr(self.T.internal), abi.ptr(self.T.boundary), self.dt,
                                                    C.byref(bc), nsteps, abi.ptr(self.T2), abi.ptr(self.Tb2), _s()))


class HeatTransfer:
    """ddt(T) - laplacian(kappa, T) = 0 with implicit Euler, the time loop of
    examples/heatTransfer/heatTransfer.cpp:60-83: every step assembles the
    system from the old field, solves it with Jacobi-PCG and corrects the
    boundary values.  Face conductivity is the linear interpolation of the cell
    values; xmin is a fixed-value wall, every other patch zero-gradient."""

    def __init__(self, hm, kappa, T0=300.0, Twall=400.0, dt=0.01, rel_tol=1e-8, max_iter=1000,
                 precision=abi.PREC_FP64):
        self.hm, self.dm = hm, DeviceMesh(hm)
        self.dt = dt
        self.cfg = abi.SolverCfg(rel_tol, 0.0, max_iter, precision, 0.1, 1000, 50)
        bcs = [("fixedValue", Twall)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
        self.T = neon.VolumeField(self.dm, np.full(hm.n, T0), bcs, name="T")
        kf = neon.VolumeField(self.dm, kappa, [("zeroGradient", 0.0)] * hm.npatch)
        self.gamma = neon.SurfaceInterpolation(self.dm, "linear").interpolate(kf)
        self.T_old = self.T.internal.clone()
        self.ls = neon.LinearSystem(self.dm)
        self.terms = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(self.T_old), neon.laplacian(self.gamma, -1.0))])
        self.stats = []

    def step(self):
        L, s = abi.lib(), _s()
        bc = self.T.bc_struct()
        self.T_old.copy_(self.T.internal)
        abi.check(L.fvgb_assemble(self.ls.handle, self.terms, 2, self.dt, C.byref(bc), abi.ptr(self.T.boundary), s))
        st = abi.SolverStats()
        abi.check(L.fvgb_solve(self.ls.handle, abi.ptr(self.T.internal), C.byref(self.cfg), C.byref(st), s),
                  allow=(abi.ERR_NOT_CONVERGED,))
        self.stats.append((st.num_iter, st.init_res_norm, st.final_res_norm, st.status))
        abi.check(L.fvgb_bc_correct(self.dm.handle, 1, C.byref(bc), abi.ptr(self.T.internal),
                                    abi.ptr(self.T.boundary), s))


class CavityPiso:
    """Lid-driven cavity, neoIcoFoam PISO (no momentum predictor), pressure
    reference cell 0 = 0.

    The defaults are the reference's loop.  ``ddt_corr`` adds
    fvc::interpolate(rAU)*fvc::ddtCorr(U, phi) to phiHbyA, ``corrected`` makes
    laplacian(rAUf, p) `Gauss linear corrected` (its face-flux correction, taken
    with the pressure the matrix was assembled with, enters the new face flux
    as in pEqn.flux()), and ``n_non_orth`` runs that many extra non-orthogonal
    pressure correctors: icoFoam's loop, which neoIcoFoam.cpp:127-137 leaves as
    TODOs."""

    def __init__(self, n=512, jitter=0.05, seed=12345, nu=0.01, dt=5e-4, n_corr=2, lid=(1.0, 0.0, 0.0),
                 precision=abi.PREC_FP64, p_rel_tol=1e-8, p_max_iter=20000, inner_rel_tol=0.1,
                 ddt_corr=False, corrected=False, n_non_orth=0, preconditioner=abi.PRECOND_JACOBI):
        self.hm = hm = mesh.box(n, n, 1, 1.0, 1.0, 1.0 / n, jitter=jitter, seed=seed, two_d=True)
        self.dm = dm = DeviceMesh(hm)
        self.dt, self.n_corr = dt, n_corr
        self.ddt_corr, self.corrected, self.n_non_orth = ddt_corr, corrected, n_non_orth
        self.cfg = abi.SolverCfg(p_rel_tol, 0.0, p_max_iter, precision, inner_rel_tol, 2000, 50, 0, 0,
                                 abi.SOLVER_CG, preconditioner)
        ubcs = [("noSlip", 0.0), ("noSlip", 0.0), ("noSlip", 0.0), ("fixedValue", list(lid))]
        self.U = neon.VolumeField(dm, np.zeros(3 * hm.n), ubcs, ncomp=3, name="U")
        self.p = neon.VolumeField(dm, np.zeros(hm.n), [("zeroGradient", 0.0)] * 4, name="p")
        nf = hm.nif + hm.nbf
        self.nu = neon.SurfaceField(dm, np.full(nf, nu))
        self.phi = neon.SurfaceField(dm)
        self.U_old = self.U.internal.clone()
        self.UEqn = neon.LinearSystem(dm, 3)
        self.pEqn = neon.LinearSystem(dm, 1)
        self.rAU = neon.VolumeField(dm, np.zeros(hm.n), [("zeroGradient", 0.0)] * 4)
        self.HbyA = neon.VolumeField(dm, np.zeros(3 * hm.n), [("zeroGradient", 0.0)] * 4, ncomp=3)
        self.rAUf = neon.SurfaceField(dm)
        self.phiHbyA = neon.SurfaceField(dm)
        self.assignable = np.zeros(hm.npatch, np.int32)   # every U patch is a fixed value
        self.stats = []
        self.phi_old = torch.zeros_like(self.phi.values)
        self.U_old_b = torch.zeros_like(self.U.boundary)
        self.p_pre = torch.zeros_like(self.p.internal)
        self.pb_pre = torch.zeros_like(self.p.boundary)
        L, dmh = abi.lib(), dm.handle
        abi.check(L.fvgb_flux_vec(dmh, abi.ptr(self.U.internal), abi.ptr(self.U.boundary), abi.ptr(self.phi.values),
                                  _s()))

    def step(self):
        L, dmh, s = abi.lib(), self.dm.handle, _s()
        self.U_old.copy_(self.U.internal)
        if self.ddt_corr:
            self.U_old_b.copy_(self.U.boundary)
            self.phi_old.copy_(self.phi.values)
        self.UEqn.assemble([neon.ddt(self.U_old), neon.div(self.phi, "linear"), neon.laplacian(self.nu, -1.0)],
                           self.dt, self.U)
        for _ in range(self.n_corr):
            abi.check(L.fvgb_piso_rau_hbya(self.UEqn.handle, abi.ptr(self.U.internal), abi.ptr(self.rAU.internal),
                                           abi.ptr(self.HbyA.internal), s))
            self.HbyA.correctBoundaryConditions()
            self.rAU.correctBoundaryConditions()
            abi.check(L.fvgb_piso_constrain_hbya(dmh, abi.ptr(self.assignable), abi.ptr(self.U.boundary),
                                                 abi.ptr(self.HbyA.boundary), s))
            abi.check(L.fvgb_interp_linear(dmh, 1, abi.ptr(self.rAU.internal), abi.ptr(self.rAU.boundary),
                                           abi.ptr(self.rAUf.values), s))
            abi.check(L.fvgb_flux_vec(dmh, abi.ptr(self.HbyA.internal), abi.ptr(self.HbyA.boundary),
                                      abi.ptr(self.phiHbyA.values), s))
            if self.ddt_corr:
                abi.check(L.fvgb_piso_ddt_corr(dmh, abi.ptr(self.U.types), abi.ptr(self.U_old),
                                               abi.ptr(self.U_old_b), abi.ptr(self.phi_old),
                                               abi.ptr(self.rAUf.values), self.dt, abi.ptr(self.phiHbyA.values), s))
            for k in range(self.n_non_orth + 1):
                final = k == self.n_non_orth
                lap = neon.laplacian(self.rAUf, 1.0, "corrected" if self.corrected else "uncorrected",
                                     field=self.p.internal)
                self.pEqn.assemble([lap, neon.div_flux(self.phiHbyA, -1.0)], self.dt, self.p)
                self.pEqn.setReference(0, 0.0)
                if final and self.corrected:
                    self.p_pre.copy_(self.p.internal)
                    self.pb_pre.copy_(self.p.boundary)
                st = abi.SolverStats()
                r = L.fvgb_solve(self.pEqn.handle, abi.ptr(self.p.internal), C.byref(self.cfg), C.byref(st), s)
                abi.check(r, allow=(abi.ERR_NOT_CONVERGED,))
                self.stats.append((st.num_iter, st.num_outer, st.init_res_norm, st.final_res_norm, st.status))
                self.p.correctBoundaryConditions()
                if final:
                    abi.check(L.fvgb_piso_face_update(self.pEqn.handle, abi.ptr(self.phiHbyA.values),
                                                      abi.ptr(self.p.internal), abi.ptr(self.phi.values), s))
                    if self.corrected:
                        abi.check(L.fvgb_nonorth_flux(dmh, 1, abi.ptr(self.rAUf.values), abi.ptr(self.p_pre),
                                                      abi.ptr(self.pb_pre), -1.0, abi.ptr(self.phi.values), s))
            abi.check(L.fvgb_piso_velocity_update(dmh, abi.ptr(self.HbyA.internal), abi.ptr(self.rAU.internal),
                                                  abi.ptr(self.p.internal), abi.ptr(self.p.boundary),
                                                  abi.ptr(self.U.internal), s))
            self.U.correctBoundaryConditions()
