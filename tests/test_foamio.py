"""OpenFOAM ASCII polyMesh and volScalarField files (fvgb_polymesh_read,
fvgb_field_read/write), on the host.  The polyMesh files are written here from
the committed fixtures of the reference's test meshes; reading them must give
the geometry of the Python polyMesh path bit for bit."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_polymesh
from foamadapter_gb300 import abi

HEADER = "FoamFile\n{{\n    version 2.0;\n    format {fmt};\n    class {cls};\n    object {obj};\n}}\n"


def write_polymesh(d, fx, fmt="ascii"):
    d.mkdir(parents=True, exist_ok=True)
    pts = fx["points"]
    with open(d / "points", "w") as f:
        f.write(HEADER.format(fmt=fmt, cls="vectorField", obj="points"))
        f.write(f"// a comment\n{len(pts)}\n(\n")
        f.writelines(f"({x!r} {y!r} {z!r})\n" for x, y, z in pts.tolist())
        f.write(")\n")
    offs, fp = fx["face_offs"], fx["face_points"]
    with open(d / "faces", "w") as f:
        f.write(HEADER.format(fmt=fmt, cls="faceList", obj="faces"))
        f.write(f"{len(offs) - 1}\n(\n")
        for i in range(len(offs) - 1):
            q = fp[offs[i]:offs[i + 1]]
            f.write(f"{len(q)}(" + " ".join(map(str, q)) + ")\n")
        f.write(")\n")
    for name in ("owner", "neighbour"):
        lab = fx[name]
        with open(d / name, "w") as f:
            f.write(HEADER.format(fmt=fmt, cls="labelList", obj=name) + "/* labels */\n")
            f.write(f"{len(lab)}\n(\n" + "\n".join(map(str, lab)) + "\n)\n")
    with open(d / "boundary", "w") as f:
        f.write(HEADER.format(fmt=fmt, cls="polyBoundaryMesh", obj="boundary"))
        f.write(f"{len(fx['patch_names'])}\n(\n")
        for nm, ty, nf, st in zip(fx["patch_names"], fx["patch_types"], fx["patch_nfaces"], fx["patch_start"]):
            f.write(f"    {nm}\n    {{\n        type {ty};\n        inGroups 1({ty});\n"
                    f"        nFaces {nf};\n        startFace {st};\n    }}\n")
        f.write(")\n")


def arr(ptr, count, dtype):
    ct = C.c_double if dtype == np.float64 else C.c_int32
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(count,)).copy()


@pytest.mark.parametrize("case", ["setup_operator", "setup_stencil3D", "setup_unstructuredMesh"])
def test_polymesh_read_matches_python_path(tmp_path, case):
    hm, fx = load_polymesh(case)
    write_polymesh(tmp_path / case, fx)
    L = abi.lib()
    pm, desc = C.c_void_p(), abi.MeshDesc()
    abi.check(L.fvgb_polymesh_read(str(tmp_path / case).encode(), C.byref(pm), C.byref(desc)))
    try:
        assert (desc.n_cells, desc.n_ifaces, desc.n_bfaces, desc.n_patches) == (hm.n, hm.nif, hm.nbf, hm.npatch)
        n, nif, nbf = hm.n, hm.nif, hm.nbf
        f64 = np.float64
        checks = [("cell_volumes", n, f64, hm.V), ("cell_centres", 3 * n, f64, hm.C.ravel()),
                  ("owner", nif, np.int32, hm.own), ("neighbour", nif, np.int32, hm.nei),
                  ("face_areas", 3 * nif, f64, hm.Sf.ravel()), ("mag_face_areas", nif, f64, hm.magSf),
                  ("weights", nif, f64, hm.w), ("delta_coeffs", nif, f64, hm.delta),
                  ("bface_cells", nbf, np.int32, hm.bcells), ("bface_areas", 3 * nbf, f64, hm.bSf.ravel()),
                  ("bmag_face_areas", nbf, f64, hm.bmagSf), ("bweights", nbf, f64, hm.bw),
                  ("bdelta_coeffs", nbf, f64, hm.bdelta), ("patch_offsets", hm.npatch + 1, np.int32,
                                                           hm.patch_offsets)]
        for name, count, dt, want in checks:
            np.testing.assert_array_equal(arr(getattr(desc, name), count, dt), np.asarray(want, dt), err_msg=name)
        for p, want in enumerate(hm.patch_names):
            nm, ty = C.c_char_p(), C.c_char_p()
            abi.check(L.fvgb_polymesh_patch(pm, p, C.byref(nm), C.byref(ty)))
            assert nm.value.decode() == want
    finally:
        L.fvgb_polymesh_free(pm)


def test_field_write_read_round_trip(tmp_path):
    hm, fx = load_polymesh("setup_operator")
    write_polymesh(tmp_path / "mesh", fx)
    L = abi.lib()
    pm, desc = C.c_void_p(), abi.MeshDesc()
    abi.check(L.fvgb_polymesh_read(str(tmp_path / "mesh").encode(), C.byref(pm), C.byref(desc)))
    try:
        rng = np.random.default_rng(0)
        T = rng.standard_normal(hm.n) * 1e3
        Tb = rng.standard_normal(hm.nbf)
        path = str(tmp_path / "T").encode()
        abi.check(L.fvgb_field_write(path, b"T", pm, abi.ptr(T), abi.ptr(Tb)))
        back = np.zeros(hm.n)
        abi.check(L.fvgb_field_read(path, hm.n, abi.ptr(back)))
        np.testing.assert_array_equal(back, T)
        text = (tmp_path / "T").read_text()
        assert "frontAndBack" in text and "type            empty;" in text
        # the reference's own field file: internalField uniform
        (tmp_path / "U").write_text(HEADER.format(fmt="ascii", cls="volScalarField", obj="U")
                                    + "dimensions [0 0 0 0 0 0 0];\ninternalField   uniform 300;\n"
                                    + "boundaryField\n{\n}\n")
        abi.check(L.fvgb_field_read(str(tmp_path / "U").encode(), hm.n, abi.ptr(back)))
        assert (back == 300.0).all()
        # a size that does not match
        assert L.fvgb_field_read(path, hm.n + 1, abi.ptr(np.zeros(hm.n + 1))) == abi.ERR_INVALID_ARG
    finally:
        L.fvgb_polymesh_free(pm)


def test_binary_and_missing_files_are_reported(tmp_path):
    hm, fx = load_polymesh("setup_operator")
    write_polymesh(tmp_path / "bin", fx, fmt="binary")
    L = abi.lib()
    pm, desc = C.c_void_p(), abi.MeshDesc()
    assert L.fvgb_polymesh_read(str(tmp_path / "bin").encode(), C.byref(pm), C.byref(desc)) == abi.ERR_UNSUPPORTED
    assert L.fvgb_polymesh_read(str(tmp_path / "nothing").encode(), C.byref(pm),
                                C.byref(desc)) == abi.ERR_INVALID_ARG
