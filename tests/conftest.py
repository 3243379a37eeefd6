"""Shared test setup: builds libfvgb and the CPU oracle once per session.

GPU tests are marked ``gpu``; everything else runs on a CPU-only machine.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def pytest_sessionstart(session):
    from foamadapter_gb300 import _build
    from oracle import build_oracle

    _build.build()
    build_oracle.build()


def load_polymesh(case: str):
    """HostMesh of a committed reference test case plus the raw fixture arrays."""
    from foamadapter_gb300 import mesh

    d = np.load(GOLDEN / f"{case}.npz")
    offs = d["face_offs"]
    faces = [d["face_points"][offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
    patches = [(str(a), str(b), int(c), int(e)) for a, b, c, e in
               zip(d["patch_names"], d["patch_types"], d["patch_nfaces"], d["patch_start"])]
    hm, order = mesh.from_polymesh(d["points"], faces, d["owner"], d["neighbour"], patches)
    return hm, d


def unpack_reference_files(root):
    """The reference's committed OpenFOAM case files (foam_files.npz), as they
    were, under root/<case>/..."""
    d = np.load(GOLDEN / "foam_files.npz")
    for key in d.files:
        p = root / key.replace("__", "/")
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_bytes(d[key].tobytes())
    return root


def unpack_reference_dicts(root):
    """The reference cases' system dictionaries (foam_dicts.npz), as they were,
    under root/<test|tutorials>/<case>/system/..."""
    d = np.load(GOLDEN / "foam_dicts.npz")
    for item in d["_names"]:
        key, rel = str(item).split("=", 1)
        p = root / rel
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_bytes(d[key].tobytes())
    return root


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
