"""Edge cases of the GPU path against the oracle: degenerate and ragged meshes,
trivial and invalid right-hand sides, indefinite systems, empty batch cases,
and a system above the persistent-kernel threshold (the multi-block path of the
cooperative solve)."""
import ctypes as C

import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu

MODES = [(abi.PREC_FP64, 1), (abi.PREC_FP64, 2), (abi.PREC_FP64, 3), (abi.PREC_MIXED_IR, 1), (abi.PREC_MIXED_IR, 2)]


def system(hm, dt=0.1, wall=2.0, seed=0):
    """ddt + laplacian with fixed-value walls, assembled on the GPU and by the oracle."""
    dm = DeviceMesh(hm)
    rng = np.random.default_rng(seed)
    T0 = 1.0 + rng.random(hm.n)
    bcs = [("fixedValue", wall)] * hm.npatch
    T = neon.VolumeField(dm, T0, bcs)
    gamma = np.exp(rng.standard_normal(hm.nif + hm.nbf))
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(neon.SurfaceField(dm, gamma), -1.0)], dt, T)
    v, r, _, _ = [t.cpu().numpy() for t in ls.export()]
    return dm, T, ls, v, r


@pytest.mark.parametrize("dims", [(1, 1, 1), (37, 1, 1), (5, 3, 1), (33, 2, 2)])
def test_degenerate_meshes_explicit_and_solve(cuda, dims):
    hm = mesh.box(*dims, jitter=0.0)
    o = Oracle(hm)
    dm, T, ls, v, r = system(hm)
    # explicit operators (a single cell has no internal face)
    rng = np.random.default_rng(1)
    F = rng.standard_normal(hm.nif + hm.nbf)
    out = torch.zeros(hm.n, dtype=torch.float64, device="cuda")
    neon.GaussGreenDiv(dm, "upwind").div(out, neon.SurfaceField(dm, F), T, 0.7)
    Tb = T.boundary.cpu().numpy()[:hm.nbf].copy()
    ref = o.div(abi.SCHEME_UPWIND, 1, F, T.host(), Tb, 0.7, np.zeros(hm.n))
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    # every solve mode against the oracle
    for prec, mode in MODES:
        x = T.internal.clone()
        st = ls.solve(x, rel_tol=1e-10, max_iter=500, precision=prec, kernel_mode=mode)
        xo = T.host().copy()
        so = o.solve(v, r, xo, rel_tol=1e-10, max_iter=500, precision=1 if prec == abi.PREC_MIXED_IR else 0)
        assert st.status == so.status == abi.OK
        assert st.num_iter == so.num_iter
        np.testing.assert_array_equal(x.cpu().numpy(), xo)


def test_zero_rhs_converges_at_once(cuda):
    hm = mesh.box(9, 8, 7, jitter=0.1, seed=3)
    dm = DeviceMesh(hm)
    T = neon.VolumeField(dm, np.zeros(hm.n), [("fixedValue", 0.0)] * hm.npatch)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(neon.SurfaceField(dm, np.ones(hm.nif + hm.nbf)), -1.0)],
                0.1, T)
    for prec, mode in MODES:
        x = torch.zeros(hm.n, dtype=torch.float64, device="cuda")
        st = ls.solve(x, rel_tol=1e-8, precision=prec, kernel_mode=mode)
        assert st.status == abi.OK and st.num_iter == 0 and st.init_res_norm == 0.0
        assert not x.any()


def test_nan_input_is_a_breakdown(cuda):
    """A NaN in the initial field is reported, never taken for convergence."""
    hm = mesh.box(9, 8, 7, jitter=0.1, seed=3)
    dm, T, ls, v, r = system(hm)
    for prec, mode in MODES:
        x = T.internal.clone()
        x[5] = float("nan")
        st = ls.solve(x, rel_tol=1e-8, precision=prec, kernel_mode=mode, allow=(abi.ERR_BREAKDOWN,))
        assert st.status == abi.ERR_BREAKDOWN, (prec, mode, st.status)
    xo = T.host().copy()
    xo[5] = np.nan
    assert Oracle(hm).solve(v, r, xo, rel_tol=1e-8).status == abi.ERR_BREAKDOWN


def test_mixed_rejects_mixed_sign_diagonal(cuda):
    hm = mesh.box(6, 5, 4, jitter=0.1, seed=3)
    dm = DeviceMesh(hm)
    rng = np.random.default_rng(0)
    T = neon.VolumeField(dm, rng.random(hm.n), [("zeroGradient", 0.0)] * hm.npatch)
    s = np.where(np.arange(hm.n) % 2 == 0, 1.0, -1.0)  # implicit source of alternating sign
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.source(1.0, neon.dev(s))], 1.0, T)
    with pytest.raises(RuntimeError):
        ls.solve(T.internal.clone(), precision=abi.PREC_MIXED_IR)


def test_batch_with_empty_and_single_cell_cases(cuda):
    parts = [mesh.box(1, 1, 1), mesh.box(7, 5, 3, jitter=0.1, seed=2), mesh.box(37, 1, 1)]
    big, ranges, slices = mesh.concat(parts)
    ranges = np.asarray(ranges, np.int32)
    # an empty case between the others: [r, r)
    ranges = np.concatenate([ranges[:2], [ranges[1], ranges[1]], ranges[2:]]).astype(np.int32)
    dm, T, ls, v, r = system(big)
    batch = neon.Batch(ls, ranges)
    for prec in (abi.PREC_FP64, abi.PREC_MIXED_IR):
        x = T.internal.clone()
        stats = batch.solve(x, rel_tol=1e-10, max_iter=500, precision=prec)
        assert [s.status for s in stats] == [abi.OK] * 4
        assert stats[1].num_iter == 0
        for k in (0, 2, 3):
            lo, hi = int(ranges[2 * k]), int(ranges[2 * k + 1])
            y = T.internal.clone()
            sub = neon.Batch(ls, np.asarray([lo, hi], np.int32))
            sub.solve(y, rel_tol=1e-10, max_iter=500, precision=prec)
            np.testing.assert_array_equal(x[lo:hi].cpu().numpy(), y[lo:hi].cpu().numpy())


def test_persistent_multiblock_path_above_threshold(cuda):
    """1,050,291 rows (> 2^20): the automatic mode uses the graph; forcing the
    cooperative kernel runs ~7 virtual blocks per resident block; same bits."""
    abi.lib().fvgb_tuning_cache_clear()  # a cached choice for this shape would skip the timing checked below
    hm = mesh.box(103, 103, 99, jitter=0.05, seed=7)
    dm, T, ls, v, r = system(hm, dt=0.01)
    out = []
    for prec in (abi.PREC_FP64, abi.PREC_MIXED_IR):
        res = []
        for mode in (1, 2):
            x = T.internal.clone()
            st = ls.solve(x, rel_tol=1e-8, max_iter=2000, precision=prec, kernel_mode=mode)
            assert st.status == abi.OK
            res.append((x.cpu().numpy(), st.num_iter, st.final_res_norm))
        np.testing.assert_array_equal(res[0][0], res[1][0])
        assert res[0][1:] == res[1][1:]
        out.append(res[0])
    # the autotuner measured every variant on this system
    chosen, ms = (C.c_int32 * 4)(), (C.c_float * 16)()
    abi.check(abi.lib().fvgb_solve_tuning(ls.handle, None, chosen, ms))
    assert all(t > 0.0 for t in ms)
