"""Host-side mesh arrays and their upload through the C ABI.

``HostMesh`` is the array set of NeoN::UnstructuredMesh + BoundaryMesh that
FoamAdapter's MeshAdapter builds from a Foam::fvMesh
(src/datastructures/meshAdapter.cpp:59-136): int32 labels, FP64 geometry,
Vec3 as 3 interleaved doubles, boundary arrays flat over the non-empty patches.
It is produced by the library's hex-box builder or from a polyMesh (points,
faces, owner, neighbour, patches) through the library's OpenFOAM geometry.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi


@dataclass
class HostMesh:
    n: int
    nif: int
    nbf: int
    npatch: int
    V: np.ndarray
    C: np.ndarray
    own: np.ndarray
    nei: np.ndarray
    Sf: np.ndarray
    Cf: np.ndarray
    magSf: np.ndarray
    w: np.ndarray
    delta: np.ndarray
    bcells: np.ndarray
    bSf: np.ndarray
    bCf: np.ndarray
    bmagSf: np.ndarray
    bw: np.ndarray
    bdelta: np.ndarray
    patch_offsets: np.ndarray
    patch_names: list = field(default_factory=list)
    points: np.ndarray | None = None

    @property
    def nnz(self) -> int:
        return self.n + 2 * self.nif

    def patch_slice(self, name: str) -> slice:
        p = self.patch_names.index(name)
        return slice(int(self.patch_offsets[p]), int(self.patch_offsets[p + 1]))

    def desc(self) -> abi.MeshDesc:
        d = abi.MeshDesc()
        d.n_cells, d.n_ifaces, d.n_bfaces, d.n_patches = self.n, self.nif, self.nbf, self.npatch
        for name, arr in (("cell_volumes", self.V), ("cell_centres", self.C), ("owner", self.own),
                          ("neighbour", self.nei), ("face_areas", self.Sf), ("mag_face_areas", self.magSf),
                          ("weights", self.w), ("delta_coeffs", self.delta), ("bface_cells", self.bcells),
                          ("bface_areas", self.bSf), ("bmag_face_areas", self.bmagSf),
                          ("bweights", self.bw), ("bdelta_coeffs", self.bdelta),
                          ("patch_offsets", self.patch_offsets)):
            setattr(d, name, abi.ptr(arr))
        return d


def _alloc_arrays(n, nif, nbf, npatch, npoints=0):
    a = dict(
        points=np.zeros(3 * npoints) if npoints else None,
        cell_volumes=np.zeros(n), cell_centres=np.zeros(3 * n), owner=np.zeros(nif, np.int32),
        neighbour=np.zeros(nif, np.int32), face_areas=np.zeros(3 * nif), face_centres=np.zeros(3 * nif),
        mag_face_areas=np.zeros(nif), weights=np.zeros(nif), delta_coeffs=np.zeros(nif),
        bface_cells=np.zeros(nbf, np.int32), bface_areas=np.zeros(3 * nbf), bface_centres=np.zeros(3 * nbf),
        bmag_face_areas=np.zeros(nbf), bweights=np.zeros(nbf), bdelta_coeffs=np.zeros(nbf),
        patch_offsets=np.zeros(npatch + 1, np.int32))
    ma = abi.MeshArrays()
    for k, v in a.items():
        setattr(ma, k, abi.ptr(v) if v is not None else None)
    return a, ma


def _to_host(a, n, nif, nbf, npatch, names) -> HostMesh:
    return HostMesh(
        n=n, nif=nif, nbf=nbf, npatch=npatch, V=a["cell_volumes"], C=a["cell_centres"].reshape(-1, 3),
        own=a["owner"], nei=a["neighbour"], Sf=a["face_areas"].reshape(-1, 3),
        Cf=a["face_centres"].reshape(-1, 3), magSf=a["mag_face_areas"], w=a["weights"],
        delta=a["delta_coeffs"], bcells=a["bface_cells"], bSf=a["bface_areas"].reshape(-1, 3),
        bCf=a["bface_centres"].reshape(-1, 3), bmagSf=a["bmag_face_areas"], bw=a["bweights"],
        bdelta=a["bdelta_coeffs"], patch_offsets=a["patch_offsets"], patch_names=list(names),
        points=None if a["points"] is None else a["points"].reshape(-1, 3))


def box(nx: int, ny: int, nz: int, lx: float = 1.0, ly: float = 1.0, lz: float = 1.0,
        jitter: float = 0.0, seed: int = 0, two_d: bool = False) -> HostMesh:
    """OpenFOAM-ordered hex box; patches xmin xmax ymin ymax [zmin zmax]."""
    spec = abi.BoxSpec(nx, ny, nz, lx, ly, lz, jitter, seed, 1 if two_d else 0)
    sizes = (C.c_int64 * 7)()
    abi.check(abi.lib().fvgb_box_sizes(C.byref(spec), sizes))
    npoints, _, n, nif, nbf, npatch, _ = list(sizes)
    a, ma = _alloc_arrays(n, nif, nbf, npatch, npoints)
    abi.check(abi.lib().fvgb_box_build(C.byref(spec), C.byref(ma)))
    names = ["xmin", "xmax", "ymin", "ymax"] + ([] if two_d else ["zmin", "zmax"])
    return _to_host(a, n, nif, nbf, npatch, names)


def from_polymesh(points: np.ndarray, faces: list, owner: np.ndarray, neighbour: np.ndarray,
                  patches: list) -> tuple[HostMesh, np.ndarray]:
    """Geometry of an OpenFOAM polyMesh.

    ``patches`` is a list of (name, type, nFaces, startFace).  Empty patches are
    left out of the flat boundary, as fvPatch sizes them 0.  Returns the mesh
    and the polyMesh face index of every internal and flat boundary face.
    """
    n_cells = int(max(owner.max(), neighbour.max() if len(neighbour) else -1)) + 1
    nif = len(neighbour)
    order = list(range(nif))
    names, offs, empties = [], [0], []
    for name, typ, nfaces, start in patches:
        rng = list(range(start, start + nfaces))
        if typ == "empty":
            empties += rng
        else:
            names.append(name)
            order += rng
            offs.append(offs[-1] + nfaces)
    nbf = len(order) - nif
    perm = order + empties
    face_offs = np.zeros(len(perm) + 1, np.int32)
    pts = []
    for i, f in enumerate(perm):
        pts += list(faces[f])
        face_offs[i + 1] = len(pts)
    face_pts = np.asarray(pts, np.int32)
    owner_all = np.asarray(owner, np.int32)[perm].copy()
    nei = np.ascontiguousarray(neighbour, dtype=np.int32)
    points = np.ascontiguousarray(points, dtype=np.float64)
    a, ma = _alloc_arrays(n_cells, nif, nbf, len(names))
    abi.check(abi.lib().fvgb_geometry_compute(
        len(points), abi.ptr(points), n_cells, len(perm), abi.ptr(face_offs), abi.ptr(face_pts),
        abi.ptr(owner_all), nif, abi.ptr(nei), nbf, C.byref(ma)))
    a["patch_offsets"][:] = np.asarray(offs, np.int32)
    return _to_host(a, n_cells, nif, nbf, len(names), names), np.asarray(order, np.int64)


def _copy(ptr, count: int, ctype=C.c_double) -> np.ndarray:
    if count == 0:
        return np.zeros(0, np.float64 if ctype is C.c_double else np.int32)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).copy()


class PolyMesh:
    """An OpenFOAM case mesh read from its constant/polyMesh directory
    (fvgb_polymesh_read, ascii or binary), with the field files that belong to it.

    ``host`` is the HostMesh MeshAdapter would build from the Foam::fvMesh
    (meshAdapter.cpp:59-136); ``patch_types`` are the polyMesh patch types of
    the non-empty patches.  Field files: ``read_field`` (internalField),
    ``read_bc`` (boundaryField mapped as readers.hpp:43-95) and ``write_field``
    (writers.cpp:9-135: calculated patches, empty patches kept).
    """

    def __init__(self, directory):
        L = abi.lib()
        self.handle = C.c_void_p()
        d = abi.MeshDesc()
        abi.check(L.fvgb_polymesh_read(str(directory).encode(), C.byref(self.handle), C.byref(d)))
        n, nif, nbf, npatch = d.n_cells, d.n_ifaces, d.n_bfaces, d.n_patches
        names, types = [], []
        for p in range(npatch):
            nm, ty = C.c_char_p(), C.c_char_p()
            abi.check(L.fvgb_polymesh_patch(self.handle, p, C.byref(nm), C.byref(ty)))
            names.append(nm.value.decode())
            types.append(ty.value.decode())
        npts, pts, cf, bcf = C.c_int32(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        abi.check(L.fvgb_polymesh_geometry(self.handle, C.byref(npts), C.byref(pts), C.byref(cf), C.byref(bcf)))
        i32 = C.c_int32
        self.host = HostMesh(
            n=n, nif=nif, nbf=nbf, npatch=npatch, V=_copy(d.cell_volumes, n),
            C=_copy(d.cell_centres, 3 * n).reshape(-1, 3), own=_copy(d.owner, nif, i32),
            nei=_copy(d.neighbour, nif, i32), Sf=_copy(d.face_areas, 3 * nif).reshape(-1, 3),
            Cf=_copy(cf, 3 * nif).reshape(-1, 3), magSf=_copy(d.mag_face_areas, nif), w=_copy(d.weights, nif),
            delta=_copy(d.delta_coeffs, nif), bcells=_copy(d.bface_cells, nbf, i32),
            bSf=_copy(d.bface_areas, 3 * nbf).reshape(-1, 3), bCf=_copy(bcf, 3 * nbf).reshape(-1, 3),
            bmagSf=_copy(d.bmag_face_areas, nbf), bw=_copy(d.bweights, nbf), bdelta=_copy(d.bdelta_coeffs, nbf),
            patch_offsets=_copy(d.patch_offsets, npatch + 1, i32), patch_names=names,
            points=_copy(pts, 3 * npts.value).reshape(-1, 3))
        self.patch_types = types

    def read_field(self, path, ncomp: int = 1, surface: bool = False) -> np.ndarray:
        """internalField values, [n] or [n, 3] (n = cells, or internal faces for a surface field)."""
        n = self.host.nif if surface else self.host.n
        out = np.zeros(n * ncomp)
        abi.check(abi.lib().fvgb_field_read(str(path).encode(), n, ncomp, abi.ptr(out)))
        return out if ncomp == 1 else out.reshape(n, ncomp)

    def read_bc(self, path, ncomp: int = 1):
        """(patch types [npatch] as fvgb_bc_type, ref [nbf*ncomp], boundary values [nbf*ncomp])."""
        h = self.host
        types = np.zeros(max(1, h.npatch), np.int32)
        ref, bval = np.zeros(max(1, h.nbf * ncomp)), np.zeros(max(1, h.nbf * ncomp))
        abi.check(abi.lib().fvgb_field_read_bc(str(path).encode(), self.handle, ncomp, abi.ptr(types),
                                               abi.ptr(ref), abi.ptr(bval)))
        return types[:h.npatch], ref[:h.nbf * ncomp], bval[:h.nbf * ncomp]

    def write_field(self, path, obj: str, internal, boundary, ncomp: int = 1, surface: bool = False,
                    binary: bool = False):
        internal = np.ascontiguousarray(internal, np.float64).reshape(-1)
        boundary = np.ascontiguousarray(boundary, np.float64).reshape(-1)
        flags = (abi.IO_BINARY if binary else 0) | (abi.IO_SURFACE if surface else 0)
        abi.check(abi.lib().fvgb_field_write(str(path).encode(), obj.encode(), self.handle, ncomp,
                                             abi.ptr(internal), abi.ptr(boundary), flags))

    def close(self):
        if self.handle:
            abi.lib().fvgb_polymesh_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def concat(meshes: list, align: int = 32) -> tuple[HostMesh, np.ndarray, list]:
    """Pack independent meshes into one block-diagonal mesh.

    Case k's cells start at a multiple of ``align`` (so 32-row slices never mix
    cases); the cells between cases are isolated placeholders (volume 1, no
    faces).  Internal faces are concatenated case by case; boundary faces are
    grouped by patch, then by case, so every cell keeps the ascending order of
    its own faces and each case computes exactly what it computes alone.
    All meshes must share the patch list.  Returns the mesh, the row ranges
    [2*ncases] (case k = rows [ranges[2k], ranges[2k+1])) and, per case, the
    slice of its faces inside each merged patch.
    """
    names = meshes[0].patch_names
    assert all(m.patch_names == names for m in meshes), "cases must share the patch list"
    starts, pos = [], 0
    for m in meshes:
        pos = -(-pos // align) * align
        starts.append(pos)
        pos += m.n
    N = -(-pos // align) * align
    V = np.ones(N)
    Cc = np.zeros((N, 3))
    for m, s0 in zip(meshes, starts):
        V[s0:s0 + m.n] = m.V
        Cc[s0:s0 + m.n] = m.C
    cat = lambda key: np.concatenate([getattr(m, key) for m in meshes])
    own = np.concatenate([m.own + s0 for m, s0 in zip(meshes, starts)]).astype(np.int32)
    nei = np.concatenate([m.nei + s0 for m, s0 in zip(meshes, starts)]).astype(np.int32)
    bcells, poffs = [], [0]
    # per-case slices inside the merged flat boundary
    case_slices = [[None] * len(names) for _ in meshes]
    cursor = 0
    parts = {key: [] for key in ("bSf", "bCf", "bmagSf", "bw", "bdelta")}
    for p in range(len(names)):
        for k, (m, s0) in enumerate(zip(meshes, starts)):
            lo, hi = int(m.patch_offsets[p]), int(m.patch_offsets[p + 1])
            case_slices[k][p] = slice(cursor, cursor + hi - lo)
            cursor += hi - lo
            bcells.append(m.bcells[lo:hi] + s0)
            for key in parts:
                parts[key].append(getattr(m, key)[lo:hi])
        poffs.append(cursor)
    hm = HostMesh(
        n=N, nif=len(own), nbf=cursor, npatch=len(names), V=V, C=Cc, own=own, nei=nei,
        Sf=np.ascontiguousarray(cat("Sf")), Cf=np.ascontiguousarray(cat("Cf")), magSf=cat("magSf"), w=cat("w"),
        delta=cat("delta"), bcells=np.concatenate(bcells).astype(np.int32),
        bSf=np.ascontiguousarray(np.concatenate(parts["bSf"])), bCf=np.ascontiguousarray(np.concatenate(parts["bCf"])),
        bmagSf=np.concatenate(parts["bmagSf"]), bw=np.concatenate(parts["bw"]), bdelta=np.concatenate(parts["bdelta"]),
        patch_offsets=np.asarray(poffs, np.int32), patch_names=list(names))
    ranges = np.asarray([v for m, s0 in zip(meshes, starts) for v in (s0, s0 + m.n)], np.int32)
    return hm, ranges, case_slices


class DeviceMesh:
    """A mesh uploaded and indexed on the GPU (fvgb_mesh handle)."""

    def __init__(self, host: HostMesh):
        self.host = host
        h = C.c_void_p()
        d = host.desc()
        abi.check(abi.lib().fvgb_mesh_create(C.byref(d), C.byref(h)))
        self.handle = h

    @property
    def n(self):
        return self.host.n

    @property
    def nif(self):
        return self.host.nif

    @property
    def nbf(self):
        return self.host.nbf

    def device_bytes(self) -> int:
        return int(abi.lib().fvgb_mesh_device_bytes(self.handle))

    def sparsity(self):
        n, nif = self.host.n, self.host.nif
        nnz = n + 2 * nif
        ro, col = np.zeros(n + 1, np.int32), np.zeros(nnz, np.int32)
        do, oo, no = np.zeros(n, np.int32), np.zeros(nif, np.int32), np.zeros(nif, np.int32)
        abi.check(abi.lib().fvgb_mesh_sparsity(self.handle, abi.ptr(ro), abi.ptr(col), abi.ptr(do),
                                               abi.ptr(oo), abi.ptr(no)))
        return ro, col, do, oo, no

    def close(self):
        if self.handle:
            abi.lib().fvgb_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
