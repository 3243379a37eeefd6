"""OpenFOAM polyMesh and field files on the host (fvgb_polymesh_read,
fvgb_field_read / fvgb_field_read_bc / fvgb_field_write and the PolyMesh /
read_vol_field / write mirror).

The reference's own files (its test meshes, the field files of its test
cases, including the ones its writer produced) are read from the committed
fixture foam_files.npz; their geometry must equal the Python polyMesh path bit
for bit, their fields the parsed fixture values.  Binary meshes are written
here from the same arrays and must read back identical to the ascii ones."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_polymesh, unpack_reference_files
from foamadapter_gb300 import abi
from foamadapter_gb300.mesh import PolyMesh

CASES = ["setup_operator", "setup_stencil3D", "setup_unstructuredMesh"]
MESH_ARRAYS = ["V", "C", "own", "nei", "Sf", "Cf", "magSf", "w", "delta", "bcells", "bSf", "bCf", "bmagSf", "bw",
               "bdelta", "patch_offsets"]


def header(fmt, cls, obj, arch="LSB;label=32;scalar=64"):
    return (f'FoamFile\n{{\n    version 2.0;\n    format {fmt};\n    arch "{arch}";\n    class {cls};\n'
            f'    note "nPoints:0 nCells:0";\n    object {obj};\n}}\n').encode()


@pytest.fixture(scope="module")
def ref_cases(tmp_path_factory):
    return unpack_reference_files(tmp_path_factory.mktemp("ref"))


def assert_same_mesh(a, b):
    assert (a.n, a.nif, a.nbf, a.npatch) == (b.n, b.nif, b.nbf, b.npatch)
    for k in MESH_ARRAYS:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)
    assert a.patch_names == b.patch_names


def write_boundary(d, fx, fmt):
    body = [header(fmt, "polyBoundaryMesh", "boundary"), f"{len(fx['patch_names'])}\n(\n".encode()]
    for nm, ty, nf, st in zip(fx["patch_names"], fx["patch_types"], fx["patch_nfaces"], fx["patch_start"]):
        body.append(f"    {nm}\n    {{\n        type {ty};\n        inGroups 1({ty});\n"
                    f"        nFaces {nf};\n        startFace {st};\n    }}\n".encode())
    body.append(b")\n")
    (d / "boundary").write_bytes(b"".join(body))


def write_polymesh_binary(d, fx, label_bits=32, scalar_bits=64):
    """OpenFOAM's binary layout: raw little-endian list bodies, faces as a faceCompactList."""
    d.mkdir(parents=True, exist_ok=True)
    arch = f"LSB;label={label_bits};scalar={scalar_bits}"
    lab, sca = f"<i{label_bits // 8}", f"<f{scalar_bits // 8}"

    def blist(a, dt):
        a = np.asarray(a)
        return f"{a.shape[0]}\n(".encode() + a.astype(dt).tobytes() + b")\n"

    (d / "points").write_bytes(header("binary", "vectorField", "points", arch) + blist(fx["points"], sca))
    (d / "faces").write_bytes(header("binary", "faceCompactList", "faces", arch) + blist(fx["face_offs"], lab)
                              + blist(fx["face_points"], lab))
    for name in ("owner", "neighbour"):
        (d / name).write_bytes(header("binary", "labelList", name, arch) + blist(fx[name], lab))
    write_boundary(d, fx, "binary")


def write_polymesh_ascii(d, fx):
    """The ascii layout in the shapes OpenFOAM also emits (one-line short
    lists, comments between tokens)."""
    d.mkdir(parents=True, exist_ok=True)
    pts = fx["points"].tolist()
    (d / "points").write_bytes(header("ascii", "vectorField", "points") + f"// pts\n{len(pts)}\n(\n".encode()
                               + "".join(f"({x!r} {y!r} {z!r})\n" for x, y, z in pts).encode() + b")\n")
    offs, fp = fx["face_offs"], fx["face_points"]
    faces = "".join(f"{offs[i + 1] - offs[i]}(" + " ".join(map(str, fp[offs[i]:offs[i + 1]])) + ")\n"
                    for i in range(len(offs) - 1))
    (d / "faces").write_bytes(header("ascii", "faceList", "faces") + f"{len(offs) - 1}\n(\n{faces})\n".encode())
    for name in ("owner", "neighbour"):
        lab = fx[name]
        (d / name).write_bytes(header("ascii", "labelList", name)
                               + f"/* labels */ {len(lab)}\n(\n".encode() + "\n".join(map(str, lab)).encode()
                               + b"\n)\n")
    write_boundary(d, fx, "ascii")


@pytest.mark.parametrize("case", CASES)
def test_reference_polymesh_files_match_python_path(ref_cases, case):
    hm, fx = load_polymesh(case)
    pm = PolyMesh(ref_cases / case / "constant" / "polyMesh")
    assert_same_mesh(pm.host, hm)
    np.testing.assert_array_equal(pm.host.points, fx["points"])
    assert pm.patch_types == [t for t in fx["patch_types"].tolist() if t != "empty"]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("bits", [(32, 64), (64, 64)])
def test_binary_and_ascii_polymesh_read_the_same(tmp_path, case, bits):
    hm, fx = load_polymesh(case)
    write_polymesh_binary(tmp_path / "bin", fx, *bits)
    write_polymesh_ascii(tmp_path / "asc", fx)
    assert_same_mesh(PolyMesh(tmp_path / "bin").host, hm)
    assert_same_mesh(PolyMesh(tmp_path / "asc").host, hm)


def test_reference_field_files(ref_cases):
    """Fields of the reference's test case, among them files its writer produced."""
    _, fx = load_polymesh("setup_operator")
    pm = PolyMesh(ref_cases / "setup_operator" / "constant" / "polyMesh")
    z = ref_cases / "setup_operator" / "0"
    np.testing.assert_array_equal(pm.read_field(z / "T"), fx["field_T"])
    np.testing.assert_array_equal(pm.read_field(z / "divT_Serial"), fx["field_divT_Serial"])
    np.testing.assert_array_equal(pm.read_field(z / "gradT_Serial", ncomp=3), fx["field_gradT_Serial"])
    np.testing.assert_array_equal(pm.read_field(z / "phi", surface=True), fx["field_phi"])
    assert (pm.read_field(z / "U", ncomp=3) == 1.0).all()
    # boundary conditions: T zeroGradient; gradT_Serial calculated with value (0 0 0); U has no entry
    # for the empty patch, which needs none
    types, ref, bval = pm.read_bc(z / "T")
    assert types.tolist() == [abi.BC_FIXED_GRADIENT] and not ref.any()
    types, ref, bval = pm.read_bc(z / "gradT_Serial", ncomp=3)
    assert types.tolist() == [abi.BC_CALCULATED] and not bval.any()
    types, _, _ = pm.read_bc(z / "U", ncomp=3)
    assert types.tolist() == [abi.BC_FIXED_GRADIENT]
    # the wrong component count is an error, not a misread
    with pytest.raises(abi.FvgbError):
        pm.read_field(z / "gradT_Serial", ncomp=1)


def test_reference_fixed_value_patches(ref_cases):
    pm = PolyMesh(ref_cases / "setup_stencil3D" / "constant" / "polyMesh")
    h = pm.host
    types, ref, bval = pm.read_bc(ref_cases / "setup_stencil3D" / "0" / "T")
    want = {"fixedWalls": (abi.BC_FIXED_GRADIENT, 0.0), "inlet": (abi.BC_FIXED_VALUE, 0.01),
            "outlet": (abi.BC_FIXED_VALUE, 0.1)}
    for p, name in enumerate(h.patch_names):
        assert types[p] == want[name][0]
        assert (ref[h.patch_slice(name)] == want[name][1]).all()
    assert (pm.read_field(ref_cases / "setup_stencil3D" / "0" / "T") == 0.0).all()


@pytest.mark.parametrize("binary", [False, True])
@pytest.mark.parametrize("ncomp", [1, 3])
@pytest.mark.parametrize("surface", [False, True])
def test_field_write_read_round_trip(ref_cases, tmp_path, binary, ncomp, surface):
    pm = PolyMesh(ref_cases / "setup_stencil3D" / "constant" / "polyMesh")
    h = pm.host
    rng = np.random.default_rng(ncomp + 2 * binary)
    n = h.nif if surface else h.n
    internal = rng.standard_normal(n * ncomp) * 1e3
    boundary = rng.standard_normal(h.nbf * ncomp) / 7.0
    path = tmp_path / "F"
    pm.write_field(path, "F", internal, boundary, ncomp=ncomp, surface=surface, binary=binary)
    back = pm.read_field(path, ncomp=ncomp, surface=surface)
    np.testing.assert_array_equal(back.reshape(-1), internal)
    types, ref, bval = pm.read_bc(path, ncomp=ncomp)
    assert (types == abi.BC_CALCULATED).all()
    np.testing.assert_array_equal(bval, boundary)
    text = path.read_bytes()
    assert (b"format      binary" in text) == binary
    assert (b"surface" in text) == surface and ((b"Vector" in text) == (ncomp == 3))


def bc_file(path, internal, entries):
    body = "".join(f"    {name}\n    {{\n{body}    }}\n" for name, body in entries)
    path.write_bytes(header("ascii", "volScalarField", path.name)
                     + f"dimensions [0 0 0 1 0 0 0];\n#include \"nothing\"\ninternalField {internal};\n"
                       f"boundaryField\n{{\n    #includeEtc \"caseDicts/setConstraintTypes\"\n{body}}}\n".encode())


def test_boundary_condition_mapping_and_matching(ref_cases, tmp_path):
    pm = PolyMesh(ref_cases / "setup_stencil3D" / "constant" / "polyMesh")
    h = pm.host
    assert h.patch_names == ["fixedWalls", "inlet", "outlet"]
    f = tmp_path / "T"
    # an exact name beats a group name (inGroups of the patch), which beats a quoted regular expression
    bc_file(f, "uniform 5", [("wall", "        type noSlip;\n"),
                             ('"(in|out)let"', "        type fixedGradient;\n        gradient uniform 1;\n"
                                               "        value uniform 3;\n"),
                             ("outlet", "        type fixedValue;\n        value $internalField;\n")])
    types, ref, bval = pm.read_bc(f)
    assert types.tolist() == [abi.BC_FIXED_VALUE, abi.BC_FIXED_GRADIENT, abi.BC_FIXED_VALUE]
    assert (ref[h.patch_slice("fixedWalls")] == 0).all()
    assert (ref[h.patch_slice("inlet")] == 3.0).all()  # the `value` entry, as the reference reads it
    assert (ref[h.patch_slice("outlet")] == 5.0).all()
    assert (pm.read_field(f) == 5.0).all()
    # a nonuniform fixed value, per face; a uniform list N{v} of the wrong size
    sl = h.patch_slice("inlet")
    nfp = sl.stop - sl.start
    vals = " ".join(str(v) for v in range(nfp))
    bc_file(f, "nonuniform List<scalar> 2{7}",
            [('".*"', "        type zeroGradient;\n"),
             ("inlet", f"        type fixedValue;\n        value nonuniform List<scalar> {nfp}({vals});\n")])
    with pytest.raises(abi.FvgbError):
        pm.read_field(f)
    types, ref, _ = pm.read_bc(f)
    assert types.tolist() == [abi.BC_FIXED_GRADIENT, abi.BC_FIXED_VALUE, abi.BC_FIXED_GRADIENT]
    np.testing.assert_array_equal(ref[sl], np.arange(nfp, dtype=float))
    bc_file(f, f"nonuniform List<scalar> {h.n}{{7}}", [('".*"', "        type zeroGradient;\n")])
    assert (pm.read_field(f) == 7.0).all()
    # an unknown boundary condition and a missing patch entry
    bc_file(f, "uniform 0", [('".*"', "        type cyclic;\n")])
    with pytest.raises(abi.FvgbError) as e:
        pm.read_bc(f)
    assert e.value.status == abi.ERR_UNSUPPORTED
    bc_file(f, "uniform 0", [("inlet", "        type zeroGradient;\n")])
    with pytest.raises(abi.FvgbError) as e:
        pm.read_bc(f)
    assert e.value.status == abi.ERR_INVALID_ARG


def test_unsupported_and_missing_files(tmp_path):
    _, fx = load_polymesh("setup_operator")
    L = abi.lib()
    pm, desc = C.c_void_p(), abi.MeshDesc()

    def read(d):
        return L.fvgb_polymesh_read(str(d).encode(), C.byref(pm), C.byref(desc))

    write_polymesh_binary(tmp_path / "msb", fx)
    p = tmp_path / "msb" / "points"
    p.write_bytes(p.read_bytes().replace(b"LSB;", b"MSB;"))
    assert read(tmp_path / "msb") == abi.ERR_UNSUPPORTED
    write_polymesh_binary(tmp_path / "fl", fx)
    f = tmp_path / "fl" / "faces"
    f.write_bytes(f.read_bytes().replace(b"faceCompactList", b"faceList"))
    assert read(tmp_path / "fl") == abi.ERR_UNSUPPORTED
    assert read(tmp_path / "nothing") == abi.ERR_INVALID_ARG
    # a truncated binary list
    write_polymesh_binary(tmp_path / "cut", fx)
    o = tmp_path / "cut" / "owner"
    o.write_bytes(o.read_bytes()[:-9])
    assert read(tmp_path / "cut") == abi.ERR_INVALID_ARG
