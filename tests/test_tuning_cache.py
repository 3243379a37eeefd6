"""The autotuner's cache file (tunecache.cpp): load, merge, save and clear on
the host, and -- on a GPU -- a cached choice used for a new system of the same
shape without timing it."""
import ctypes as C
import json

import numpy as np
import pytest

from foamadapter_gb300 import abi


def entry(key, variants):
    return {"key": key, "variants": variants, "ms": [[0.1, 0.2, 0.3, 0.4]] * 4}


def test_cache_file_round_trip(tmp_path):
    L = abi.lib()
    abi.check(L.fvgb_tuning_cache_clear())
    assert L.fvgb_tuning_cache_size() == 0
    f = tmp_path / "cache.json"
    f.write_text(json.dumps({"version": 1, "entries": [entry("a", [0, 1, 2, 3]), entry("b", [3, -1, 2, -1])]}))
    abi.check(L.fvgb_tuning_cache_load(str(f).encode()))
    assert L.fvgb_tuning_cache_size() == 2
    g = tmp_path / "out.json"
    abi.check(L.fvgb_tuning_cache_save(str(g).encode()))
    d = json.loads(g.read_text())
    assert d["version"] == 1
    assert {e["key"]: e["variants"] for e in d["entries"]} == {"a": [0, 1, 2, 3], "b": [3, -1, 2, -1]}
    # merging keeps the other keys and replaces a key's entry
    f.write_text(json.dumps({"version": 1, "entries": [entry("a", [3, 3, 3, 3])]}))
    abi.check(L.fvgb_tuning_cache_load(str(f).encode()))
    abi.check(L.fvgb_tuning_cache_save(str(g).encode()))
    d = json.loads(g.read_text())
    assert {e["key"]: e["variants"] for e in d["entries"]} == {"a": [3, 3, 3, 3], "b": [3, -1, 2, -1]}
    # malformed files change nothing
    for text in ("{", '{"version": 2, "entries": []}', '{"version": 1, "entries": [{"key": "c"}]}',
                 json.dumps({"version": 1, "entries": [entry("c", [0, 9, 0, 0])]})):
        f.write_text(text)
        with pytest.raises(abi.FvgbError):
            abi.check(L.fvgb_tuning_cache_load(str(f).encode()))
    assert L.fvgb_tuning_cache_size() == 2
    abi.check(L.fvgb_tuning_cache_clear())
    assert L.fvgb_tuning_cache_size() == 0


def test_cache_keys_with_quotes_round_trip(tmp_path):
    """Keys are written as JSON strings (quotes and backslashes escaped), so a
    saved file is valid JSON and loads back to the same keys; a key with a
    control character is refused."""
    L = abi.lib()
    abi.check(L.fvgb_tuning_cache_clear())
    f, g = tmp_path / "in.json", tmp_path / "out.json"
    key = 'sm103 "GB300" \\ path / café \U0001f680'  # json.dumps writes \u escapes and a surrogate pair
    f.write_text(json.dumps({"version": 1, "entries": [entry(key, [1, 2, -1, 0])]}))
    abi.check(L.fvgb_tuning_cache_load(str(f).encode()))
    abi.check(L.fvgb_tuning_cache_save(str(g).encode()))
    d = json.loads(g.read_text())
    assert [e["key"] for e in d["entries"]] == [key]
    abi.check(L.fvgb_tuning_cache_clear())
    abi.check(L.fvgb_tuning_cache_load(str(g).encode()))
    abi.check(L.fvgb_tuning_cache_save(str(f).encode()))
    assert json.loads(f.read_text()) == d
    f.write_text(json.dumps({"version": 1, "entries": [entry("a\u0001b", [0, 0, 0, 0])]}))
    with pytest.raises(abi.FvgbError):
        abi.check(L.fvgb_tuning_cache_load(str(f).encode()))
    abi.check(L.fvgb_tuning_cache_clear())


@pytest.mark.gpu
def test_cached_choice_is_used_without_timing(cuda, tmp_path):
    """A system of 2^18 rows is timed at its first solve and its choice cached;
    after the cache is replaced by a file naming other variants, a new system of
    the same shape uses them untimed, with the same bits."""
    from foamadapter_gb300 import mesh, neon
    from foamadapter_gb300.mesh import DeviceMesh

    L = abi.lib()
    abi.check(L.fvgb_tuning_cache_clear())
    hm = mesh.box(64, 64, 64, jitter=0.1, seed=3)
    dm = DeviceMesh(hm)

    def system():
        T = neon.VolumeField(dm, np.full(hm.n, 300.0), [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * 5)
        ls = neon.LinearSystem(dm)
        ls.assemble([neon.ddt(T.internal.clone()),
                     neon.laplacian(neon.SurfaceField(dm, np.ones(hm.nif + hm.nbf)), -1.0)], 0.01, T)
        return T, ls

    chosen, ms = (C.c_int32 * 4)(), (C.c_float * 16)()
    T, ls = system()
    x1 = T.internal.clone()
    assert ls.solve(x1, rel_tol=1e-8).status == abi.OK
    abi.check(L.fvgb_solve_tuning(ls.handle, None, chosen, ms))
    assert all(ms[v] > 0 for v in range(8))  # FP64 kinds timed
    assert L.fvgb_tuning_cache_size() == 1
    f = tmp_path / "cache.json"
    abi.check(L.fvgb_tuning_cache_save(str(f).encode()))
    d = json.loads(f.read_text())
    key = d["entries"][0]["key"]
    assert key.startswith("sm") and "/rows2^18/" in key
    d["entries"][0]["variants"] = [0, 1, 0, 1]
    f.write_text(json.dumps(d))
    abi.check(L.fvgb_tuning_cache_clear())
    abi.check(L.fvgb_tuning_cache_load(str(f).encode()))
    T2, ls2 = system()
    x2 = T2.internal.clone()
    assert ls2.solve(x2, rel_tol=1e-8).status == abi.OK
    abi.check(L.fvgb_solve_tuning(ls2.handle, None, chosen, ms))
    assert list(chosen) == [2, 4, 2, 4]
    assert all(t == 0.0 for t in ms)  # nothing timed
    assert np.array_equal(x1.cpu().numpy(), x2.cpu().numpy())
    abi.check(L.fvgb_tuning_cache_clear())


@pytest.mark.gpu
def test_face_tile_tuned_and_cached(cuda):
    """fvgb_explicit_tune times the face-pass tiles 2, 4, 8 on a mesh, sets the
    fastest and records it; a second mesh of the same shape takes it untimed."""
    import ctypes as C

    from foamadapter_gb300 import mesh
    from foamadapter_gb300.mesh import DeviceMesh

    L = abi.lib()
    abi.check(L.fvgb_tuning_cache_clear())
    # the DeviceMesh objects are kept in names: a handle taken from a temporary
    # would outlive its mesh (CPython frees the temporary at once)
    dm = DeviceMesh(mesh.box(48, 40, 32, jitter=0.1, seed=2))
    tile, ms = C.c_int32(), (C.c_float * 3)()
    abi.check(L.fvgb_explicit_tune(dm.handle, None, C.byref(tile), ms))
    assert tile.value in (2, 4, 8) and all(t > 0 for t in ms)
    assert ms[(2, 4, 8).index(tile.value)] == min(ms)
    dm2 = DeviceMesh(mesh.box(48, 40, 32, jitter=0.1, seed=3))
    tile2, ms2 = C.c_int32(), (C.c_float * 3)()
    abi.check(L.fvgb_explicit_tune(dm2.handle, None, C.byref(tile2), ms2))
    assert tile2.value == tile.value and list(ms2) == [0.0, 0.0, 0.0]
    with pytest.raises(abi.FvgbError):
        abi.check(L.fvgb_mesh_face_tile(dm.handle, 3))
    abi.check(L.fvgb_tuning_cache_clear())
