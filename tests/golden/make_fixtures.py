"""Extract golden fixtures from the reference's committed test cases.

Reads the ascii OpenFOAM cases under the reference checkout's ``test/`` tree
(polyMesh points/faces/owner/neighbour/boundary and the field files of
``test/setup_operator/0``) and writes them as small ``.npz`` files next to this
script, so that the tests run where the reference checkout is absent.
``foam_files.npz`` keeps the unparsed bytes of the small polyMesh and field
files (key: the path with "/" written as "__"), the input of the tests of the
library's own OpenFOAM file reader; ``foam_dicts.npz`` keeps the cases'
``system/`` dictionaries (fvSolution, fvSchemes, controlDict, blockMeshDict,
simulationParameters, testDictionary) the same way, for the dictionary
reader's tests.
Run:  python tests/golden/make_fixtures.py [/path/to/reference]
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CASES = ["setup_operator", "setup_stencil3D", "setup_unstructuredMesh", "setup_advection"]


def _strip(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    return text


def _body(text: str) -> str:
    """Text after the FoamFile header dictionary."""
    text = _strip(text)
    i = text.index("FoamFile")
    depth, j = 0, text.index("{", i)
    for k in range(j, len(text)):
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                return text[k + 1:]
    raise ValueError("unterminated header")


def read_list(path: Path):
    """A top-level list file (points, faces, owner, neighbour)."""
    body = _body(path.read_text())
    m = re.search(r"(\d+)\s*\(", body)
    n = int(m.group(1))
    inner = body[m.end():]
    if "faces" in path.name:
        faces = [list(map(int, f.split())) for f in re.findall(r"\d+\s*\(([^()]*)\)", inner)][:n]
        assert len(faces) == n
        return faces
    if "points" in path.name:
        pts = [list(map(float, t.split())) for t in re.findall(r"\(([^()]*)\)", inner)][:n]
        return np.asarray(pts, np.float64)
    vals = inner[: inner.index(")")].split()
    return np.asarray(list(map(int, vals[:n])), np.int64)


def read_boundary(path: Path):
    body = _body(path.read_text())
    out = []
    for name, block in re.findall(r"(\w+)\s*\{([^{}]*)\}", body):
        typ = re.search(r"\btype\s+(\w+)\s*;", block).group(1)
        nf = int(re.search(r"nFaces\s+(\d+)", block).group(1))
        sf = int(re.search(r"startFace\s+(\d+)", block).group(1))
        out.append((name, typ, nf, sf))
    return out


def read_internal_field(path: Path):
    body = _body(path.read_text())
    m = re.search(r"internalField\s+nonuniform\s+List<(\w+)>\s*(\d+)\s*\(", body)
    kind, n = m.group(1), int(m.group(2))
    inner = body[m.end():]
    if kind == "vector":
        vals = [list(map(float, t.split())) for t in re.findall(r"\(([^()]*)\)", inner)][:n]
        return np.asarray(vals, np.float64)
    vals = inner[: inner.index(")")].split()[:n]
    return np.asarray(list(map(float, vals)), np.float64)


def main(ref: Path):
    for case in CASES:
        pm = ref / "test" / case / "constant" / "polyMesh"
        arrays = dict(
            points=read_list(pm / "points"),
            owner=read_list(pm / "owner"),
            neighbour=read_list(pm / "neighbour"),
        )
        faces = read_list(pm / "faces")
        arrays["face_offs"] = np.cumsum([0] + [len(f) for f in faces]).astype(np.int64)
        arrays["face_points"] = np.asarray([p for f in faces for p in f], np.int64)
        patches = read_boundary(pm / "boundary")
        arrays["patch_names"] = np.asarray([p[0] for p in patches])
        arrays["patch_types"] = np.asarray([p[1] for p in patches])
        arrays["patch_nfaces"] = np.asarray([p[2] for p in patches], np.int64)
        arrays["patch_start"] = np.asarray([p[3] for p in patches], np.int64)
        if case == "setup_operator":
            z = ref / "test" / case / "0"
            for name in ("T", "phi", "divT_Serial", "divT_OpenMP", "ofDivT", "gradT_Serial", "gradT_OpenMP",
                         "ofGradT"):
                arrays["field_" + name] = read_internal_field(z / name)
        np.savez_compressed(HERE / f"{case}.npz", **arrays)
        print(case, {k: v.shape for k, v in arrays.items()})
    files = {}
    for case in CASES[:3]:
        for name in ("points", "faces", "owner", "neighbour", "boundary"):
            files[f"{case}/constant/polyMesh/{name}"] = None
    for rel in ("setup_operator/0/T", "setup_operator/0/U", "setup_operator/0/phi", "setup_operator/0/divT_Serial",
                "setup_operator/0/gradT_Serial", "setup_stencil3D/0/T", "setup_unstructuredMesh/0/T"):
        files[rel] = None
    raw = {k.replace("/", "__"): np.frombuffer((ref / "test" / k).read_bytes(), np.uint8) for k in files}
    np.savez_compressed(HERE / "foam_files.npz", **raw)
    print("foam_files", {k: v.size for k, v in raw.items()})
    # the cases' system dictionaries, unparsed (input of the dictionary reader's tests)
    dicts = sorted(p.relative_to(ref).as_posix() for top in ("test", "tutorials")
                   for p in [*(ref / top).glob("*/system/*"), *(ref / top).glob("*/system/gko/*.json")]
                   if p.is_file())
    raw = {k.replace("/", "__").replace("-", "_"): np.frombuffer((ref / k).read_bytes(), np.uint8) for k in dicts}
    names = {k.replace("/", "__").replace("-", "_"): k for k in dicts}
    np.savez_compressed(HERE / "foam_dicts.npz", _names=np.asarray([f"{a}={b}" for a, b in names.items()]), **raw)
    print("foam_dicts", len(raw))


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
