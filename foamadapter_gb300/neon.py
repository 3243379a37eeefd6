"""NeoN-shaped Python mirror of the drop-in, on top of the C ABI.

Class and method names follow the NeoN operators FoamAdapter calls
(GaussGreenDiv(exec, mesh, scheme).div(out, phi, T, coeff),
GaussGreenGrad(exec, mesh).grad(T, coeff, out), SurfaceInterpolation,
GaussGreenLaplacian, FaceNormalGradient, la::createSparsity,
LinearSystem, PDESolver::{assemble, setReference, solve}, applyOperator, diag)
so that the tests read like the reference's own tests
(test/test_operators.cpp, test/test_implicitOperators.cpp).  Device storage
is torch CUDA tensors: torch is only the allocator here; every operation is a
call into libfvgb.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import abi
from .mesh import DeviceMesh, HostMesh, PolyMesh

_SCHEMES = {"linear": abi.SCHEME_LINEAR, "upwind": abi.SCHEME_UPWIND}
_BC = {"calculated": abi.BC_CALCULATED, "fixedValue": abi.BC_FIXED_VALUE,
       "fixedGradient": abi.BC_FIXED_GRADIENT, "zeroGradient": abi.BC_FIXED_GRADIENT,
       "noSlip": abi.BC_FIXED_VALUE}


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _scheme(s) -> int:
    if isinstance(s, (list, tuple)):
        s = [t for t in s if t not in ("Gauss", "uncorrected")][0]
    return _SCHEMES[s] if isinstance(s, str) else int(s)


def dev(a, dtype=torch.float64) -> torch.Tensor:
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).cuda()


class VolumeField:
    """Cell values [n*ncomp] plus flat boundary values [nbf*ncomp] and a BC per patch.

    bcs: list of (type, value) per non-empty patch; value is a scalar/Vec3 or a
    per-face array (fixed value or fixed gradient); zeroGradient = fixedGradient 0
    and noSlip = fixedValue 0, as FoamAdapter's readers map them (readers.hpp:43-95).
    """

    def __init__(self, mesh: DeviceMesh, internal, bcs=None, ncomp: int = 1, name: str = ""):
        self.mesh, self.ncomp, self.name = mesh, ncomp, name
        hm = mesh.host
        self.internal = dev(np.asarray(internal, np.float64).reshape(-1))
        assert self.internal.numel() == hm.n * ncomp
        bcs = bcs or [("calculated", 0.0)] * hm.npatch
        assert len(bcs) == hm.npatch
        self.types = np.asarray([_BC[t] for t, _ in bcs], np.int32)
        ref = np.zeros((hm.nbf, ncomp))
        for p, (t, v) in enumerate(bcs):
            sl = slice(int(hm.patch_offsets[p]), int(hm.patch_offsets[p + 1]))
            if t in ("zeroGradient", "noSlip"):
                v = 0.0
            v = np.asarray(v, np.float64).reshape(-1)
            nfp = sl.stop - sl.start
            if v.size == 1 or (v.size == ncomp and nfp != 1):
                ref[sl] = np.broadcast_to(v if v.size == ncomp else np.repeat(v, ncomp), (nfp, ncomp))
            else:
                ref[sl] = v.reshape(nfp, ncomp)
        self.ref = dev(ref.reshape(-1))
        self.boundary = torch.zeros(max(1, hm.nbf * ncomp), dtype=torch.float64, device="cuda")
        self.correctBoundaryConditions()

    def bc_struct(self) -> abi.BC:
        return abi.BC(abi.ptr(self.types), abi.ptr(self.ref))

    def correctBoundaryConditions(self):
        bc = self.bc_struct()
        abi.check(abi.lib().fvgb_bc_correct(self.mesh.handle, self.ncomp, C.byref(bc),
                                            abi.ptr(self.internal), abi.ptr(self.boundary), _stream()))

    def host(self):
        return self.internal.cpu().numpy()


_BC_NAME = {abi.BC_CALCULATED: "calculated", abi.BC_FIXED_VALUE: "fixedValue",
            abi.BC_FIXED_GRADIENT: "fixedGradient"}


def read_vol_field(mesh: DeviceMesh, poly: PolyMesh, path, ncomp: int = 1, name: str = "") -> VolumeField:
    """A VolumeField from an OpenFOAM field file: its internalField and the
    boundary conditions of its boundaryField, as FoamAdapter's constructFrom
    builds one (readers.hpp:110-126, the mapping of readers.hpp:43-95)."""
    internal = poly.read_field(path, ncomp)
    types, ref, _ = poly.read_bc(path, ncomp)
    hm = mesh.host
    bcs = [(_BC_NAME[int(t)], ref[int(hm.patch_offsets[p]) * ncomp:int(hm.patch_offsets[p + 1]) * ncomp])
           for p, t in enumerate(types)]
    return VolumeField(mesh, internal, bcs, ncomp=ncomp, name=name)


def write(field: VolumeField, poly: PolyMesh, path, binary: bool = False):
    """Write a VolumeField as an OpenFOAM field file with calculated patches
    holding its boundary values (writers.cpp:67-135)."""
    nb = field.mesh.nbf * field.ncomp
    poly.write_field(path, field.name or str(path).rsplit("/", 1)[-1], field.host(),
                     field.boundary.cpu().numpy()[:nb], ncomp=field.ncomp, binary=binary)


class SurfaceField:
    """Face values: internal faces then boundary faces [(nif+nbf)*ncomp]."""

    def __init__(self, mesh: DeviceMesh, values=None, ncomp: int = 1):
        self.mesh, self.ncomp = mesh, ncomp
        nf = mesh.nif + mesh.nbf
        if values is None:
            self.values = torch.zeros(max(1, nf * ncomp), dtype=torch.float64, device="cuda")
        else:
            self.values = dev(np.asarray(values, np.float64).reshape(-1))

    def host(self):
        return self.values.cpu().numpy()


class SurfaceInterpolation:
    def __init__(self, mesh: DeviceMesh, scheme="linear"):
        self.mesh, self.scheme = mesh, _scheme(scheme)

    def interpolate(self, src: VolumeField, dst: SurfaceField | None = None, flux: SurfaceField | None = None):
        dst = dst or SurfaceField(self.mesh, ncomp=src.ncomp)
        L = abi.lib()
        if self.scheme == abi.SCHEME_LINEAR:
            abi.check(L.fvgb_interp_linear(self.mesh.handle, src.ncomp, abi.ptr(src.internal),
                                           abi.ptr(src.boundary), abi.ptr(dst.values), _stream()))
        else:
            assert flux is not None, "upwind interpolation needs the face flux"
            abi.check(L.fvgb_interp_upwind(self.mesh.handle, src.ncomp, abi.ptr(flux.values),
                                           abi.ptr(src.internal), abi.ptr(src.boundary),
                                           abi.ptr(dst.values), _stream()))
        return dst


class GaussGreenDiv:
    def __init__(self, mesh: DeviceMesh, scheme="linear"):
        self.mesh, self.scheme = mesh, _scheme(scheme)

    def div(self, out: torch.Tensor, faceFlux: SurfaceField, phi: VolumeField, coeff: float = 1.0):
        abi.check(abi.lib().fvgb_div_explicit(self.mesh.handle, self.scheme, phi.ncomp,
                                              abi.ptr(faceFlux.values), abi.ptr(phi.internal),
                                              abi.ptr(phi.boundary), float(coeff), abi.ptr(out),
                                              _stream()))
        return out


class GaussGreenGrad:
    def __init__(self, mesh: DeviceMesh):
        self.mesh = mesh

    def grad(self, phi: VolumeField, coeff: float = 1.0, out: torch.Tensor | None = None):
        if out is None:
            out = torch.zeros(3 * self.mesh.n, dtype=torch.float64, device="cuda")
        abi.check(abi.lib().fvgb_grad(self.mesh.handle, abi.ptr(phi.internal), abi.ptr(phi.boundary),
                                      float(coeff), abi.ptr(out), _stream()))
        return out


def _corrected(scheme) -> bool:
    """True for a `corrected` snGrad scheme ("Gauss linear corrected", "corrected")."""
    toks = scheme if isinstance(scheme, (list, tuple)) else str(scheme).split()
    if "corrected" in toks:
        return True
    if "uncorrected" in toks or not toks or toks in (["Gauss", "linear"], ["linear"]):
        return False
    raise ValueError(f"unsupported snGrad scheme {scheme!r}")


class GaussGreenLaplacian:
    """scheme: "Gauss linear uncorrected" or "Gauss linear corrected" (tokens or a string)."""

    def __init__(self, mesh: DeviceMesh, scheme=("Gauss", "linear", "uncorrected")):
        self.mesh = mesh
        self.corrected = _corrected(scheme)

    def laplacian(self, out: torch.Tensor, gamma: SurfaceField, phi: VolumeField, coeff: float = 1.0):
        fn = abi.lib().fvgb_laplacian_explicit_corrected if self.corrected else abi.lib().fvgb_laplacian_explicit
        abi.check(fn(self.mesh.handle, phi.ncomp, abi.ptr(gamma.values), abi.ptr(phi.internal),
                     abi.ptr(phi.boundary), float(coeff), abi.ptr(out), _stream()))
        return out


class FaceNormalGradient:
    """scheme: "uncorrected" or "corrected"."""

    def __init__(self, mesh: DeviceMesh, scheme="uncorrected"):
        self.mesh = mesh
        self.corrected = _corrected(scheme)

    def faceNormalGrad(self, phi: VolumeField, out: SurfaceField | None = None):
        out = out or SurfaceField(self.mesh)
        fn = abi.lib().fvgb_sngrad_corrected if self.corrected else abi.lib().fvgb_sngrad
        abi.check(fn(self.mesh.handle, abi.ptr(phi.internal), abi.ptr(phi.boundary), abi.ptr(out.values),
                     _stream()))
        return out


def nonorth_flux(gamma: SurfaceField, phi: VolumeField, coeff: float = 1.0, out: SurfaceField | None = None):
    """faceFluxCorrection of laplacian(gamma, phi) with the corrected scheme,
    out_f += coeff*(gamma_f|Sf|)(k_f . grad(phi)_f) on the internal faces."""
    mesh = phi.mesh
    out = out or SurfaceField(mesh, ncomp=phi.ncomp)
    abi.check(abi.lib().fvgb_nonorth_flux(mesh.handle, phi.ncomp, abi.ptr(gamma.values), abi.ptr(phi.internal),
                                          abi.ptr(phi.boundary), float(coeff), abi.ptr(out.values), _stream()))
    return out


def createSparsity(mesh: DeviceMesh):
    """la::createSparsity: (rowOffs, colIdxs, diagOffset, ownerOffset, neighbourOffset) on the host."""
    return mesh.sparsity()


@dataclass
class Term:
    """One operator of a dsl::Expression (see fvgb_term in include/fvgb.h)."""
    kind: int
    coeff: float = 1.0
    scheme: int = abi.SCHEME_LINEAR
    cell: torch.Tensor | None = None
    face: torch.Tensor | None = None

    def struct(self) -> abi.Term:
        return abi.Term(self.kind, self.scheme, self.coeff, abi.ptr(self.cell), abi.ptr(self.face))


def ddt(old: torch.Tensor, coeff: float = 1.0) -> Term:
    return Term(abi.TERM_DDT, coeff, cell=old)


def laplacian(gamma: SurfaceField, coeff: float = 1.0, scheme="uncorrected",
              field: torch.Tensor | None = None) -> Term:
    """Implicit laplacian(gamma, psi).  With a corrected scheme, `field` is the
    current psi whose explicit non-orthogonal correction goes to the rhs."""
    if _corrected(scheme):
        if field is None:
            raise ValueError("a corrected laplacian needs the current field")
        return Term(abi.TERM_LAPLACIAN, coeff, scheme=abi.SCHEME_CORRECTED, cell=field, face=gamma.values)
    return Term(abi.TERM_LAPLACIAN, coeff, face=gamma.values)


def div(flux: SurfaceField, scheme="linear", coeff: float = 1.0) -> Term:
    return Term(abi.TERM_DIV, coeff, scheme=_scheme(scheme), face=flux.values)


def source(coeff: float = 1.0, s: torch.Tensor | None = None) -> Term:
    return Term(abi.TERM_SOURCE, coeff, cell=s)


def explicit(values: torch.Tensor, coeff: float = 1.0) -> Term:
    return Term(abi.TERM_EXPLICIT, coeff, cell=values)


def div_explicit(flux: SurfaceField, field: torch.Tensor, scheme="upwind", coeff: float = 1.0) -> Term:
    """dsl::exp::div(phi, psi) of `field` (psi's boundary values are taken from
    the assembled field), volume integrated into the rhs."""
    return Term(abi.TERM_DIV_EXPLICIT, coeff, scheme=_scheme(scheme), cell=field, face=flux.values)


def div_flux(flux: SurfaceField, coeff: float = 1.0) -> Term:
    """dsl::exp::div(phi) of a face flux, volume integrated, into the rhs."""
    return Term(abi.TERM_DIV_FLUX, coeff, face=flux.values)


class LinearSystem:
    """la::LinearSystem on the mesh pattern (device resident)."""

    def __init__(self, mesh: DeviceMesh, ncomp: int = 1):
        self.mesh, self.ncomp = mesh, ncomp
        h = C.c_void_p()
        abi.check(abi.lib().fvgb_ls_create(mesh.handle, ncomp, C.byref(h)))
        self.handle = h

    def assemble(self, terms, dt: float, psi: VolumeField):
        arr = (abi.Term * max(1, len(terms)))(*[t.struct() for t in terms])
        bc = psi.bc_struct()
        abi.check(abi.lib().fvgb_assemble(self.handle, arr, len(terms), float(dt), C.byref(bc),
                                          abi.ptr(psi.boundary), _stream()))

    def setReference(self, cell: int, value: float):
        abi.check(abi.lib().fvgb_set_reference(self.handle, int(cell), float(value), _stream()))

    def apply(self, x: torch.Tensor) -> torch.Tensor:
        out = torch.empty(self.mesh.n * self.ncomp, dtype=torch.float64, device="cuda")
        abi.check(abi.lib().fvgb_apply_operator(self.handle, abi.ptr(x), abi.ptr(out), _stream()))
        return out

    def diag(self) -> torch.Tensor:
        out = torch.empty(self.mesh.n, dtype=torch.float64, device="cuda")
        abi.check(abi.lib().fvgb_ls_diag(self.handle, abi.ptr(out), _stream()))
        return out

    def export(self):
        hm = self.mesh.host
        v = torch.empty(hm.nnz, dtype=torch.float64, device="cuda")
        r = torch.empty(hm.n * self.ncomp, dtype=torch.float64, device="cuda")
        bm = torch.empty(max(1, hm.nbf), dtype=torch.float64, device="cuda")
        br = torch.empty(max(1, hm.nbf * self.ncomp), dtype=torch.float64, device="cuda")
        abi.check(abi.lib().fvgb_ls_export(self.handle, abi.ptr(v), abi.ptr(r), abi.ptr(bm), abi.ptr(br),
                                           _stream()))
        return v, r, bm[:hm.nbf], br[:hm.nbf * self.ncomp]

    def solve(self, x: torch.Tensor, rel_tol=1e-8, abs_tol=0.0, max_iter=1000, precision=abi.PREC_FP64,
              inner_rel_tol=None, inner_max_iter=1000, max_outer=50, allow=(abi.ERR_NOT_CONVERGED,), kernel_mode=0,
              method=abi.SOLVER_CG, flags=0, preconditioner=abi.PRECOND_JACOBI):
        """inner_rel_tol (mixed precision) defaults to 0.1 for CG and 0.01 for the
        restarted inner BiCGStab, the fastest settings measured on 128^3 systems.
        preconditioner=abi.PRECOND_MULTIGRID: CG with the aggregation
        multigrid V-cycle (single systems); with precision=abi.PREC_MIXED_IR
        the V-cycle runs in FP32 inside the FP64 CG."""
        if inner_rel_tol is None:
            inner_rel_tol = 0.01 if method == abi.SOLVER_BICGSTAB else 0.1
        cfg = abi.SolverCfg(rel_tol, abs_tol, max_iter, precision, inner_rel_tol, inner_max_iter, max_outer,
                            kernel_mode, flags, method, preconditioner)
        st = abi.SolverStats()
        abi.check(abi.lib().fvgb_solve(self.handle, abi.ptr(x), C.byref(cfg), C.byref(st), _stream()),
                  allow=allow)
        return st

    def close(self):
        if self.handle:
            abi.lib().fvgb_ls_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Independent cases packed into one LinearSystem, solved together
    (fvgb_batch_*): one launch per kernel for all cases, per-case criteria."""

    def __init__(self, ls: LinearSystem, row_ranges):
        self.ls = ls
        self.ranges = np.ascontiguousarray(row_ranges, dtype=np.int32)
        self.ncases = len(self.ranges) // 2
        h = C.c_void_p()
        abi.check(abi.lib().fvgb_batch_create(ls.handle, self.ncases, abi.ptr(self.ranges), C.byref(h)))
        self.handle = h

    def solve(self, x: torch.Tensor, rel_tol=1e-8, abs_tol=0.0, max_iter=1000, precision=abi.PREC_FP64,
              inner_rel_tol=1e-3, inner_max_iter=1000, max_outer=50, allow=(abi.ERR_NOT_CONVERGED,),
              method=abi.SOLVER_CG):
        cfg = abi.SolverCfg(rel_tol, abs_tol, max_iter, precision, inner_rel_tol, inner_max_iter, max_outer, 0, 0,
                            method)
        stats = (abi.SolverStats * self.ncases)()
        abi.check(abi.lib().fvgb_batch_solve(self.handle, abi.ptr(x), C.byref(cfg), stats, _stream()), allow=allow)
        return list(stats)

    def close(self):
        if self.handle:
            abi.lib().fvgb_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PDESolver:
    """FoamAdapter::PDESolver (expression.hpp:23-179): owns the system of one PDE."""

    def __init__(self, terms, psi: VolumeField, dt: float):
        self.terms, self.psi, self.dt = terms, psi, dt
        self.ls = LinearSystem(psi.mesh, psi.ncomp)
        self.ref = None

    def assemble(self):
        self.ls.assemble(self.terms, self.dt, self.psi)
        return self.ls

    def setReference(self, cell: int, value: float):
        self.ref = (cell, value)

    def solve(self, fvSolution=None, **cfg):
        """Assemble, set the reference, solve, correct the boundary values.
        With ``fvSolution`` (a ``dictionary.Dictionary`` of the case's
        system/fvSolution), the entry solvers/<psi.name> configures the solve,
        as PDESolver::solve reads it (expression.hpp:141-153); an entry in
        OpenFOAM form (solver PCG; ...) is mapped by mapFvSolution first.
        Keyword arguments override the entry."""
        if fvSolution is not None:
            from . import dictionary

            entry = fvSolution.subDict("solvers").subDict(self.psi.name)
            if not (entry.contains("solver") and entry.get("solver") == "Ginkgo"):
                entry = dictionary.map_fv_solution(entry)
            cfg = {**dictionary.solver_config(entry), **cfg}
        self.assemble()
        if self.ref is not None:
            self.ls.setReference(*self.ref)
        st = self.ls.solve(self.psi.internal, **cfg)
        self.psi.correctBoundaryConditions()
        return st
