"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py as the checker; never by the product package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_build" / "libfvoracle.so"

vp, i32, dbl = C.c_void_p, C.c_int32, C.c_double


class OrMesh(C.Structure):
    _fields_ = [("n", i32), ("nif", i32), ("nbf", i32), ("npatch", i32),
                ("V", vp), ("Sf", vp), ("magSf", vp), ("w", vp), ("delta", vp), ("own", vp), ("nei", vp),
                ("bcells", vp), ("bSf", vp), ("bmagSf", vp), ("bw", vp), ("bdelta", vp), ("patch_offs", vp)]


class OrBoxArrays(C.Structure):
    _fields_ = [(name, vp) for name in ("V", "C", "own", "nei", "Sf", "Cf", "magSf", "w", "delta", "bcells", "bSf",
                                        "bCf", "bmagSf", "bw", "bdelta", "patch_offs", "points")]


class OrCsr(C.Structure):
    _fields_ = [("n", i32), ("nnz", i32), ("row_offs", vp), ("col", vp), ("diag_off", vp),
                ("own_off", vp), ("nei_off", vp)]


class OrTerm(C.Structure):
    _fields_ = [("kind", i32), ("scheme", i32), ("coeff", dbl), ("cell", vp), ("face", vp)]


class OrCfg(C.Structure):
    _fields_ = [("rel_tol", dbl), ("abs_tol", dbl), ("max_iter", i32), ("precision", i32),
                ("inner_rel_tol", dbl), ("inner_max_iter", i32), ("max_outer", i32), ("method", i32),
                ("flags", i32), ("preconditioner", i32), ("pad", i32)]


class OrStats(C.Structure):
    _fields_ = [("init_res_norm", dbl), ("final_res_norm", dbl), ("num_iter", i32),
                ("num_outer", i32), ("status", i32), ("reserved", i32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} is missing: run oracle/build_oracle.py")
        _lib = C.CDLL(str(LIB))
        _lib.or_dot_tree.restype = dbl
        _lib.or_sparsity.restype = i32
        _lib.or_solve.restype = i32
        _lib.or_get_threads.restype = i32
        _lib.or_box_sizes.restype = i32
        _lib.or_box_build.restype = i32
        _lib.or_box_build.argtypes = [i32, i32, i32, dbl, dbl, dbl, dbl, C.c_uint64, i32, C.c_void_p]
    return _lib


def p(a):
    if a is None:
        return None
    assert isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"], type(a)
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """Oracle bound to one host mesh (keeps the arrays alive)."""

    def __init__(self, hm):
        self.hm = hm
        self.keep = [np.ascontiguousarray(x) for x in (hm.V, hm.Sf, hm.magSf, hm.w, hm.delta, hm.own, hm.nei,
                                                         hm.bcells, hm.bSf, hm.bmagSf, hm.bw, hm.bdelta,
                                                         hm.patch_offsets)]
        k = self.keep
        self.m = OrMesh(hm.n, hm.nif, hm.nbf, hm.npatch, *[x.ctypes.data for x in k])
        self.L = lib()
        self._csr = None
        self._k = None

    # ---------------------------------------------------------------- explicit
    def bc_correct(self, ncomp, types, ref, internal, boundary):
        t = np.asarray(types, np.int32)
        self.L.or_bc_correct(C.byref(self.m), ncomp, p(t), p(ref), p(internal), p(boundary))

    def interp_linear(self, ncomp, src, src_b):
        dst = np.zeros((self.hm.nif + self.hm.nbf) * ncomp)
        self.L.or_interp_linear(C.byref(self.m), ncomp, p(src), p(src_b), p(dst))
        return dst

    def interp_upwind(self, ncomp, flux, src, src_b):
        dst = np.zeros((self.hm.nif + self.hm.nbf) * ncomp)
        self.L.or_interp_upwind(C.byref(self.m), ncomp, p(flux), p(src), p(src_b), p(dst))
        return dst

    def div(self, scheme, ncomp, flux, phi, phi_b, coeff, out):
        self.L.or_div(C.byref(self.m), scheme, ncomp, p(flux), p(phi), p(phi_b), dbl(coeff), p(out))
        return out

    def grad(self, phi, phi_b, coeff, out):
        self.L.or_grad(C.byref(self.m), p(phi), p(phi_b), dbl(coeff), p(out))
        return out

    def laplacian(self, ncomp, gamma, phi, phi_b, coeff, out):
        self.L.or_laplacian(C.byref(self.m), ncomp, p(gamma), p(phi), p(phi_b), dbl(coeff), p(out))
        return out

    def sngrad(self, phi, phi_b):
        out = np.zeros(self.hm.nif + self.hm.nbf)
        self.L.or_sngrad(C.byref(self.m), p(phi), p(phi_b), p(out))
        return out

    def nonorth_vectors(self):
        """[nif*3] non-orthogonal correction vectors from the cell centres."""
        if self._k is None:
            hm = self.hm
            cc = np.ascontiguousarray(hm.C, np.float64).reshape(-1)
            self._k = np.zeros(max(1, 3 * hm.nif))
            self.L.or_nonorth_vectors(C.byref(self.m), p(cc), p(self._k))
        return self._k

    def laplacian_corrected(self, ncomp, gamma, phi, phi_b, coeff, out):
        self.L.or_laplacian_corrected(C.byref(self.m), ncomp, p(self.nonorth_vectors()), p(gamma), p(phi),
                                      p(phi_b), dbl(coeff), p(out))
        return out

    def sngrad_corrected(self, phi, phi_b):
        out = np.zeros(self.hm.nif + self.hm.nbf)
        self.L.or_sngrad_corrected(C.byref(self.m), p(self.nonorth_vectors()), p(phi), p(phi_b), p(out))
        return out

    def nonorth_flux(self, ncomp, gamma, phi, phi_b, coeff, out):
        self.L.or_nonorth_flux(C.byref(self.m), ncomp, p(self.nonorth_vectors()), p(gamma), p(phi), p(phi_b),
                               dbl(coeff), p(out))
        return out

    def advect_euler(self, flux, T, Tb, dt, types, ref):
        Tn, Tnb = np.zeros_like(T), np.zeros_like(Tb)
        t = np.asarray(types, np.int32)
        self.L.or_advect_euler(C.byref(self.m), p(flux), p(T), p(Tb), dbl(dt), p(t), p(ref), p(Tn), p(Tnb))
        return Tn, Tnb

    # ---------------------------------------------------------------- implicit
    def csr(self):
        if self._csr is None:
            hm = self.hm
            nnz = hm.n + 2 * hm.nif
            ro, col = np.zeros(hm.n + 1, np.int32), np.zeros(nnz, np.int32)
            do, oo, no = np.zeros(hm.n, np.int32), np.zeros(hm.nif, np.int32), np.zeros(hm.nif, np.int32)
            r = self.L.or_sparsity(C.byref(self.m), p(ro), p(col), p(do), p(oo), p(no))
            if r < 0:
                raise ValueError("two faces between one pair of cells")
            self._csr_arrays = (ro, col, do, oo, no)
            self._csr = OrCsr(hm.n, nnz, *[x.ctypes.data for x in (ro, col, do, oo, no)])
        return self._csr

    def csr_arrays(self):
        self.csr()
        return self._csr_arrays

    def assemble(self, ncomp, terms, dt, types, ref, psi_b):
        """terms: list of (kind, scheme, coeff, cell_array|None, face_array|None)"""
        A = self.csr()
        hm = self.hm
        arr = (OrTerm * max(1, len(terms)))()
        for i, (kind, scheme, coeff, cell, face) in enumerate(terms):
            arr[i] = OrTerm(kind, scheme, coeff, None if cell is None else cell.ctypes.data,
                            None if face is None else face.ctypes.data)
        values = np.zeros(A.nnz)
        rhs = np.zeros(hm.n * ncomp)
        bmat = np.zeros(max(1, hm.nbf))
        brhs = np.zeros(max(1, hm.nbf * ncomp))
        t = np.asarray(types, np.int32)
        self.L.or_assemble(C.byref(self.m), C.byref(A), ncomp, arr, len(terms), dbl(dt), p(t), p(ref),
                           p(psi_b), p(values), p(rhs), p(bmat), p(brhs))
        # corrected laplacians: their explicit non-orthogonal part, after all terms, in term order
        for kind, scheme, coeff, cell, face in terms:
            if kind == 1 and scheme == 2 and hm.nif > 0:
                self.L.or_nonorth_rhs(C.byref(self.m), ncomp, p(self.nonorth_vectors()), p(face), p(cell),
                                      p(psi_b), dbl(-coeff), p(rhs))
        return values, rhs, bmat[:hm.nbf], brhs[:hm.nbf * ncomp]

    def set_reference(self, values, rhs, cell, value):
        self.L.or_set_reference(C.byref(self.csr()), p(values), p(rhs), cell, dbl(value))

    def apply_operator(self, values, rhs, ncomp, x):
        out = np.zeros(self.hm.n * ncomp)
        self.L.or_apply_operator(C.byref(self.csr()), p(values), p(rhs), ncomp, p(x), p(out))
        return out

    def solve(self, values, rhs, x, rel_tol=1e-8, abs_tol=0.0, max_iter=1000, precision=0,
              inner_rel_tol=None, inner_max_iter=1000, max_outer=50, method=0, flags=0, preconditioner=0):
        """flags & 2: rel_tol relative to ||b|| (Ginkgo ResidualNorm, baseline rhs_norm);
        preconditioner 2: ILU(0) (CG or BiCGStab, FP64)."""
        if inner_rel_tol is None:  # the host API's defaults: 0.1 for CG, 0.01 for BiCGStab
            inner_rel_tol = 0.01 if method == 1 else 0.1
        cfg = OrCfg(rel_tol, abs_tol, max_iter, precision, inner_rel_tol, inner_max_iter, max_outer, method, flags,
                    preconditioner, 0)
        st = OrStats()
        self.L.or_solve(C.byref(self.csr()), p(values), p(rhs), p(x), C.byref(cfg), C.byref(st))
        return st

    def ilu_factor(self, values):
        lu = np.zeros(len(values))
        self.L.or_ilu_factor(C.byref(self.csr()), p(values), p(lu))
        return lu

    def ilu_apply(self, lu, r):
        y, z = np.zeros(self.hm.n), np.zeros(self.hm.n)
        self.L.or_ilu_apply(C.byref(self.csr()), p(lu), p(np.ascontiguousarray(r, float)), p(y), p(z))
        return z

    # -------------------------------------------------------------------- PISO
    def rau_hbya(self, values, rhs, U):
        rAU, H = np.zeros(self.hm.n), np.zeros(3 * self.hm.n)
        self.L.or_rau_hbya(C.byref(self.m), C.byref(self.csr()), p(values), p(rhs), p(U), p(rAU), p(H))
        return rAU, H

    def constrain_hbya(self, assignable, U_b, H_b):
        a = np.asarray(assignable, np.int32)
        self.L.or_constrain_hbya(C.byref(self.m), p(a), p(U_b), p(H_b))

    def flux_vec(self, U, U_b):
        out = np.zeros(self.hm.nif + self.hm.nbf)
        self.L.or_flux_vec(C.byref(self.m), p(U), p(U_b), p(out))
        return out

    def face_update(self, values, bmat, brhs, phiHbyA, pp):
        out = np.zeros(self.hm.nif + self.hm.nbf)
        self.L.or_face_update(C.byref(self.m), C.byref(self.csr()), p(values), p(bmat), p(brhs),
                              p(phiHbyA), p(pp), p(out))
        return out

    def velocity_update(self, H, rAU, pp, p_b):
        U = np.zeros(3 * self.hm.n)
        self.L.or_velocity_update(C.byref(self.m), p(H), p(rAU), p(pp), p(p_b), p(U))
        return U

    def ddt_corr(self, U_types, U, U_b, phi_old, rAUf, dt, out):
        t = np.asarray(U_types, np.int32)
        self.L.or_ddt_corr(C.byref(self.m), p(t), p(U), p(U_b), p(phi_old), p(rAUf), dbl(dt), p(out))
        return out

    def constrain_pressure(self, fixed_flux, phiHbyA, U_b, rAUf, p_ref):
        fl = np.asarray(fixed_flux, np.int32)
        self.L.or_constrain_pressure(C.byref(self.m), p(fl), p(phiHbyA), p(U_b), p(rAUf), p(p_ref))
        return p_ref


class BoxMesh:
    """The arrays of a hex box as the oracle builds it (boxmesh.c), with the
    attribute names of the library's host mesh: n, nif, nbf, npatch, V, C, own,
    nei, Sf, Cf, magSf, w, delta, bcells, bSf, bCf, bmagSf, bw, bdelta,
    patch_offsets, patch_names, points."""

    def __init__(self, nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, jitter=0.0, seed=0, two_d=False):
        L = lib()
        sz = (C.c_int64 * 6)()
        if L.or_box_sizes(nx, ny, nz, 1 if two_d else 0, sz) != 0:
            raise ValueError("bad box size")
        npts, n, nif, nbf, npatch, _ = (int(v) for v in sz)
        self.n, self.nif, self.nbf, self.npatch = n, nif, nbf, npatch
        self.V, self.C = np.zeros(n), np.zeros((n, 3))
        self.own, self.nei = np.zeros(nif, np.int32), np.zeros(nif, np.int32)
        self.Sf, self.Cf = np.zeros((nif, 3)), np.zeros((nif, 3))
        self.magSf, self.w, self.delta = np.zeros(nif), np.zeros(nif), np.zeros(nif)
        self.bcells = np.zeros(nbf, np.int32)
        self.bSf, self.bCf = np.zeros((nbf, 3)), np.zeros((nbf, 3))
        self.bmagSf, self.bw, self.bdelta = np.zeros(nbf), np.zeros(nbf), np.zeros(nbf)
        self.patch_offsets = np.zeros(npatch + 1, np.int32)
        self.points = np.zeros((npts, 3))
        self.patch_names = ["xmin", "xmax", "ymin", "ymax"] + ([] if two_d else ["zmin", "zmax"])
        arr = OrBoxArrays(*[a.ctypes.data for a in (self.V, self.C, self.own, self.nei, self.Sf, self.Cf, self.magSf,
                                                     self.w, self.delta, self.bcells, self.bSf, self.bCf, self.bmagSf,
                                                     self.bw, self.bdelta, self.patch_offsets, self.points)])
        r = L.or_box_build(nx, ny, nz, lx, ly, lz, jitter, seed, 1 if two_d else 0, C.byref(arr))
        if r != 0:
            raise ValueError(f"or_box_build failed ({r})")

    @property
    def nnz(self) -> int:
        return self.n + 2 * self.nif

    def patch_slice(self, name: str) -> slice:
        p = self.patch_names.index(name)
        return slice(int(self.patch_offsets[p]), int(self.patch_offsets[p + 1]))


def dot_tree(a: np.ndarray, b: np.ndarray) -> float:
    return lib().or_dot_tree(len(a), p(a), p(b))


def set_threads(n: int):
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return int(lib().or_get_threads())
