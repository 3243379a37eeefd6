"""CPU twins of the example solvers, on the oracle (TEST INFRASTRUCTURE ONLY).

Same steps, same order as foamadapter_gb300/apps.py, every operation a call
into the CPU restatement; used by the parity tests and the CPU baseline.
"""
from __future__ import annotations

import numpy as np

from .pyoracle import Oracle

DDT, LAP, DIV, SRC, EXP, DIV_FLUX = range(6)
LINEAR, UPWIND = 0, 1
CALC, FIXED_VALUE, FIXED_GRADIENT = 0, 1, 2


class CavityPisoCPU:
    def __init__(self, hm, nu=0.01, dt=5e-4, n_corr=2, lid=(1.0, 0.0, 0.0), precision=0, p_rel_tol=1e-8,
                 p_max_iter=20000, inner_rel_tol=0.1, ddt_corr=False, corrected=False, n_non_orth=0):
        self.hm, self.o = hm, Oracle(hm)
        self.dt, self.n_corr = dt, n_corr
        self.ddt_corr, self.corrected, self.n_non_orth = ddt_corr, corrected, n_non_orth
        self.solve_kw = dict(rel_tol=p_rel_tol, max_iter=p_max_iter, precision=precision,
                             inner_rel_tol=inner_rel_tol, inner_max_iter=2000, max_outer=50)
        n, nbf = hm.n, hm.nbf
        self.U = np.zeros(3 * n)
        self.Ub = np.zeros(3 * nbf)
        self.Utypes = np.full(hm.npatch, FIXED_VALUE, np.int32)
        self.Uref = np.zeros(3 * nbf)
        lid_sl = hm.patch_slice("ymax")
        self.Uref.reshape(-1, 3)[lid_sl] = lid
        self.o.bc_correct(3, self.Utypes, self.Uref, self.U, self.Ub)
        self.p = np.zeros(n)
        self.pb = np.zeros(nbf)
        self.zg = np.full(hm.npatch, FIXED_GRADIENT, np.int32)
        self.z1, self.z3 = np.zeros(nbf), np.zeros(3 * nbf)
        self.o.bc_correct(1, self.zg, self.z1, self.p, self.pb)
        self.nu = np.full(hm.nif + nbf, nu)
        self.phi = self.o.flux_vec(self.U, self.Ub)
        self.assignable = np.zeros(hm.npatch, np.int32)
        self.stats = []

    def step(self):
        o, hm = self.o, self.hm
        U_old, Ub_old, phi_old = self.U.copy(), self.Ub.copy(), self.phi.copy()
        v, r, _, _ = o.assemble(3, [(DDT, 0, 1.0, U_old, None), (DIV, LINEAR, 1.0, None, self.phi),
                                    (LAP, 0, -1.0, None, self.nu)], self.dt, self.Utypes, self.Uref, self.Ub)
        for _ in range(self.n_corr):
            rAU, H = o.rau_hbya(v, r, self.U)
            Hb, rAUb = np.zeros(3 * hm.nbf), np.zeros(hm.nbf)
            o.bc_correct(3, self.zg, self.z3, H, Hb)
            o.bc_correct(1, self.zg, self.z1, rAU, rAUb)
            o.constrain_hbya(self.assignable, self.Ub, Hb)
            rAUf = o.interp_linear(1, rAU, rAUb)
            phiHbyA = o.flux_vec(H, Hb)
            if self.ddt_corr:
                o.ddt_corr(self.Utypes, U_old, Ub_old, phi_old, rAUf, self.dt, phiHbyA)
            for k in range(self.n_non_orth + 1):
                lap = (LAP, 2, 1.0, self.p.copy(), rAUf) if self.corrected else (LAP, 0, 1.0, None, rAUf)
                pv, pr, pbm, pbr = o.assemble(1, [lap, (DIV_FLUX, 0, -1.0, None, phiHbyA)],
                                              self.dt, self.zg, self.z1, self.pb)
                o.set_reference(pv, pr, 0, 0.0)
                p_pre, pb_pre = self.p.copy(), self.pb.copy()
                st = o.solve(pv, pr, self.p, **self.solve_kw)
                self.stats.append((st.num_iter, st.num_outer, st.init_res_norm, st.final_res_norm, st.status))
                o.bc_correct(1, self.zg, self.z1, self.p, self.pb)
                if k == self.n_non_orth:
                    self.phi = o.face_update(pv, pbm, pbr, phiHbyA, self.p)
                    if self.corrected:
                        o.nonorth_flux(1, rAUf, p_pre, pb_pre, -1.0, self.phi)
            self.U = o.velocity_update(H, rAU, self.p, self.pb)
            o.bc_correct(3, self.Utypes, self.Uref, self.U, self.Ub)


class HeatTransferCPU:
    """ddt(T) - laplacian(k, T) = 0 with a fixed-value xmin wall."""

    def __init__(self, hm, k, T0=300.0, Twall=400.0, dt=0.01, rel_tol=1e-8, max_iter=1000):
        self.hm, self.o = hm, Oracle(hm)
        self.dt, self.rel_tol, self.max_iter = dt, rel_tol, max_iter
        self.gamma = self.o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
        self.types = np.asarray([FIXED_VALUE] + [FIXED_GRADIENT] * (hm.npatch - 1), np.int32)
        self.ref = np.zeros(hm.nbf)
        self.ref[hm.patch_slice("xmin")] = Twall
        self.T = np.full(hm.n, T0)
        self.Tb = np.zeros(hm.nbf)
        self.o.bc_correct(1, self.types, self.ref, self.T, self.Tb)
        self.stats = []

    def step(self):
        v, r, _, _ = self.o.assemble(1, [(DDT, 0, 1.0, self.T.copy(), None), (LAP, 0, -1.0, None, self.gamma)],
                                     self.dt, self.types, self.ref, self.Tb)
        st = self.o.solve(v, r, self.T, rel_tol=self.rel_tol, max_iter=self.max_iter)
        self.stats.append((st.num_iter, st.init_res_norm, st.final_res_norm, st.status))
        self.o.bc_correct(1, self.types, self.ref, self.T, self.Tb)


class ServedRequestCPU:
    """One request of the serving loop on the oracle: the unit box with nx*ny*nz
    cells (unjittered), uniform velocity U, diffusivity D, and `steps` IMEX
    steps of ddt(T) + div(phi, T) - laplacian(D, T) = 0 -- explicit upwind
    convection of the old field, implicit ddt + diffusion, zero-gradient walls,
    Jacobi-PCG (FP64 or mixed) to 1e-8 with the server's solver settings."""

    def __init__(self, nx, ny, nz, U, D, dt, T0, precision=0):
        from .pyoracle import BoxMesh

        self.hm = hm = BoxMesh(nx, ny, nz)
        self.o = o = Oracle(hm)
        self.dt, self.precision = dt, precision
        U = np.asarray(U, np.float64)
        self.F = o.flux_vec(np.tile(U, hm.n), np.tile(U, hm.nbf))
        self.gamma = np.full(hm.nif + hm.nbf, D)
        self.types = np.full(hm.npatch, FIXED_GRADIENT, np.int32)
        self.ref = np.zeros(hm.nbf)
        self.T = np.array(T0, dtype=np.float64)
        self.Tb = np.zeros(hm.nbf)
        o.bc_correct(1, self.types, self.ref, self.T, self.Tb)
        self.iters = 0

    def step(self):
        o = self.o
        old = self.T.copy()
        v, r, _, _ = o.assemble(1, [(DDT, 0, 1.0, old, None), (6, UPWIND, 1.0, old, self.F),
                                    (LAP, 0, -1.0, None, self.gamma)], self.dt, self.types, self.ref, self.Tb)
        st = o.solve(v, r, self.T, rel_tol=1e-8, max_iter=2000, precision=self.precision, inner_rel_tol=1e-4,
                     inner_max_iter=1000, max_outer=50)
        if st.status != 0:
            raise RuntimeError(f"oracle solve status {st.status}")
        self.iters += st.num_iter
        o.bc_correct(1, self.types, self.ref, self.T, self.Tb)
