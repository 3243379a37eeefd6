"""Batched solves: independent cases packed into one system and solved with
one launch per kernel must give every case exactly the bits it gets alone
(same reduction tree per case), in FP64 and in mixed precision, and the
packed explicit/assembly operators must match the per-case ones."""
import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh

pytestmark = pytest.mark.gpu


def make_cases(seed=5):
    rng = np.random.default_rng(seed)
    dims = [(13, 11, 9), (20, 7, 12), (9, 9, 9), (31, 17, 5), (16, 16, 16)]
    cases = []
    for k, d in enumerate(dims):
        hm = mesh.box(*d, jitter=0.1, seed=100 + k)
        kap = np.exp(0.5 * rng.standard_normal(hm.n))
        tw = rng.uniform(350, 450)
        cases.append((hm, kap, tw))
    return cases


def assemble_case(dm, kap, tw, ncomp_bcs=None):
    hm = dm.host
    T = neon.VolumeField(dm, np.full(hm.n, 300.0), [("fixedValue", tw)] + [("zeroGradient", 0.0)] * 5)
    kf = neon.VolumeField(dm, kap, [("zeroGradient", 0.0)] * 6)
    gamma = neon.SurfaceInterpolation(dm, "linear").interpolate(kf)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gamma, -1.0)], 0.01, T)
    return T, ls


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_batch_equals_alone(cuda, precision):
    cases = make_cases()
    alone = []
    for hm, kap, tw in cases:
        dm = DeviceMesh(hm)
        T, ls = assemble_case(dm, kap, tw)
        x = T.internal.clone()
        st = ls.solve(x, rel_tol=1e-8, precision=precision, inner_rel_tol=1e-3, inner_max_iter=1000,
                      max_outer=50)
        alone.append((x.cpu().numpy(), st, ls.export()[0].cpu().numpy()))
    big, ranges, slices = mesh.concat([c[0] for c in cases])
    dm = DeviceMesh(big)
    kap = np.ones(big.n)
    ref = np.zeros(big.nbf)
    for k, (hm, kk, tw) in enumerate(cases):
        kap[ranges[2 * k]:ranges[2 * k + 1]] = kk
        ref[slices[k][0]] = tw
    T = neon.VolumeField(dm, np.full(big.n, 300.0), [("fixedValue", ref[slices[0][0].start:slices[-1][0].stop])]
                         + [("zeroGradient", 0.0)] * 5)
    kf = neon.VolumeField(dm, kap, [("zeroGradient", 0.0)] * 6)
    gamma = neon.SurfaceInterpolation(dm, "linear").interpolate(kf)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gamma, -1.0)], 0.01, T)
    batch = neon.Batch(ls, ranges)
    x = T.internal.clone()
    stats = batch.solve(x, rel_tol=1e-8, precision=precision, inner_rel_tol=1e-3, inner_max_iter=1000, max_outer=50)
    xb = x.cpu().numpy()
    for k, (xa, st, _) in enumerate(alone):
        sl = slice(ranges[2 * k], ranges[2 * k + 1])
        np.testing.assert_array_equal(xb[sl], xa)
        assert (stats[k].num_iter, stats[k].num_outer, stats[k].status) == (st.num_iter, st.num_outer, st.status)
        assert stats[k].init_res_norm == st.init_res_norm and stats[k].final_res_norm == st.final_res_norm
    # placeholder rows between cases are untouched
    gaps = np.ones(big.n, bool)
    for k in range(len(cases)):
        gaps[ranges[2 * k]:ranges[2 * k + 1]] = False
    assert np.all(xb[gaps] == 300.0)


def test_batch_cases_stop_independently(cuda):
    """A capped case reports NOT_CONVERGED while the others converge."""
    cases = make_cases(9)[:3]
    big, ranges, slices = mesh.concat([c[0] for c in cases])
    dm = DeviceMesh(big)
    ref = np.zeros(big.nbf)
    for k, (_, _, tw) in enumerate(cases):
        ref[slices[k][0]] = tw
    T = neon.VolumeField(dm, np.full(big.n, 300.0), [("fixedValue", ref[slices[0][0].start:slices[-1][0].stop])]
                         + [("zeroGradient", 0.0)] * 5)
    gamma = neon.SurfaceField(dm, np.ones(big.nif + big.nbf))
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gamma, -1.0)], 0.01, T)
    batch = neon.Batch(ls, ranges)
    x = T.internal.clone()
    stats = batch.solve(x, rel_tol=1e-10, max_iter=12)
    assert all(s.num_iter <= 12 for s in stats)
    assert any(s.status == abi.ERR_NOT_CONVERGED for s in stats)


def test_batch_kernel_variants_give_the_same_bits(cuda):
    """fvgb_batch_tuning forces the launch-bound variants of a batch's solver:
    every variant gives every case the same bits."""
    import ctypes as C

    cases = make_cases()[:3]
    big, ranges, slices = mesh.concat([c[0] for c in cases])
    dm = DeviceMesh(big)
    T = neon.VolumeField(dm, np.full(big.n, 300.0), [("fixedValue", 350.0)] + [("zeroGradient", 0.0)] * 5)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()),
                 neon.laplacian(neon.SurfaceField(dm, np.ones(big.nif + big.nbf)), -1.0)], 0.01, T)
    L = abi.lib()
    chosen, ms = (C.c_int32 * 4)(), (C.c_float * 16)()
    out = []
    for var in range(4):
        b = neon.Batch(ls, ranges)
        abi.check(L.fvgb_batch_tuning(b.handle, (C.c_int32 * 4)(var, var, var, var), chosen, ms))
        assert list(chosen) == [(2, 4, 6, 8)[var]] * 4
        for prec in (abi.PREC_FP64, abi.PREC_MIXED_IR):
            x = T.internal.clone()
            stats = b.solve(x, rel_tol=1e-9, precision=prec, inner_rel_tol=1e-3)
            assert all(s.status == abi.OK for s in stats)
            out.append((prec, x.cpu().numpy(), [s.num_iter for s in stats]))
    for prec in (abi.PREC_FP64, abi.PREC_MIXED_IR):
        runs = [o for o in out if o[0] == prec]
        for run in runs[1:]:
            np.testing.assert_array_equal(runs[0][1], run[1])
            assert runs[0][2] == run[2]
    bad = neon.Batch(ls, ranges)  # kept alive for the call: its handle must not outlive the object
    with pytest.raises(abi.FvgbError):
        abi.check(L.fvgb_batch_tuning(bad.handle, (C.c_int32 * 4)(7, -1, -1, -1), chosen, ms))
