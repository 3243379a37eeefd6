"""Device-built box meshes and the serving loop.

* fvgb_mesh_create_boxes builds packed boxes on the device; its analytic
  geometry must reproduce the host-built mesh's operators to round-off.
* The server runs every request exactly as it would run alone: a request's
  final field is bit-identical whether it ran by itself or among others
  (the continuous-batching equivalence the serving design promises), and it
  agrees with the same IMEX steps driven through the Python API on a
  host-built mesh to round-off.
"""
import ctypes as C
import time

import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh

pytestmark = pytest.mark.gpu


def device_boxes(dims):
    specs = (abi.BoxSpec * len(dims))(*[abi.BoxSpec(nx, ny, nz, 1.0, 1.0, 1.0, 0.0, 0, 0) for nx, ny, nz in dims])
    ranges = np.zeros(2 * len(dims), np.int32)
    h = C.c_void_p()
    abi.check(abi.lib().fvgb_mesh_create_boxes(specs, len(dims), C.byref(h), abi.ptr(ranges),
                                               torch.cuda.current_stream().cuda_stream))
    return h, ranges


class _Wrap:  # minimal DeviceMesh-like holder for a device-built mesh
    def __init__(self, handle, host):
        self.handle, self.host = handle, host

    @property
    def n(self):
        return self.host.n

    @property
    def nif(self):
        return self.host.nif

    @property
    def nbf(self):
        return self.host.nbf


def test_device_boxes_match_host_boxes(cuda):
    dims = [(7, 5, 4), (3, 9, 6), (10, 2, 3)]
    hh, ranges_h, slices = mesh.concat([mesh.box(*d) for d in dims])
    hdev, ranges_d = device_boxes(dims)
    np.testing.assert_array_equal(ranges_h, ranges_d)
    sizes = (C.c_int64 * 5)()
    abi.check(abi.lib().fvgb_mesh_sizes(hdev, sizes))
    assert list(sizes)[:4] == [hh.n, hh.nif, hh.nbf, hh.npatch]
    dh = DeviceMesh(hh)
    dd = _Wrap(hdev, hh)
    rng = np.random.default_rng(0)
    T0 = rng.standard_normal(hh.n)
    outs = []
    for dm in (dh, dd):
        T = neon.VolumeField(dm, T0, [("fixedValue", 1.0), ("zeroGradient", 0.0)] * 3)
        F = neon.SurfaceField(dm)
        U = neon.dev(np.tile([0.3, -0.2, 0.1], hh.n))
        Ub = neon.dev(np.tile([0.3, -0.2, 0.1], hh.nbf))
        abi.check(abi.lib().fvgb_flux_vec(dm.handle, abi.ptr(U), abi.ptr(Ub), abi.ptr(F.values),
                                          torch.cuda.current_stream().cuda_stream))
        div = neon.GaussGreenDiv(dm, "upwind").div(torch.zeros(hh.n, dtype=torch.float64, device="cuda"), F, T)
        grad = neon.GaussGreenGrad(dm).grad(T)
        gam = neon.SurfaceField(dm, np.full(hh.nif + hh.nbf, 0.7))
        ls = neon.LinearSystem(dm)
        ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gam, -1.0),
                     neon.div_explicit(F, T.internal.clone())], 0.01, T)
        x = T.internal.clone()
        ls.solve(x, rel_tol=1e-10)
        outs.append([a.cpu().numpy() for a in (F.values, div, grad, ls.apply(T.internal), x)])
    for a, b in zip(*outs):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(a).max()))
    abi.lib().fvgb_mesh_destroy(hdev)


def make_server(budget=8 << 30, streams=4, max_active=64):
    cfg = abi.ServerCfg(budget, streams, max_active)
    h = C.c_void_p()
    abi.check(abi.lib().fvgb_server_create(C.byref(cfg), C.byref(h)))
    return h


def submit(server, nx, ny, nz, steps, U, D, precision=abi.PREC_FP64, flags=0):
    out = np.zeros(nx * ny * nz)
    req = abi.ServeRequest(nx=nx, ny=ny, nz=nz, steps=steps, U=(C.c_double * 3)(*U), D=D, dt=0.0,
                           precision=precision, kernel_mode=0, flags=flags, T_out=out.ctypes.data)
    rid = C.c_int64()
    st = abi.lib().fvgb_server_submit(server, C.byref(req), C.byref(rid))
    return st, rid.value, out


def drain(server, expected, timeout=120.0):
    res = {}
    buf = (abi.ServeResult * 256)()
    t0 = time.time()
    while len(res) < expected and time.time() - t0 < timeout:
        cnt = C.c_int32()
        abi.check(abi.lib().fvgb_server_poll(server, buf, 256, C.byref(cnt)))
        for i in range(cnt.value):
            res[buf[i].id] = abi.ServeResult.from_buffer_copy(buf[i])
        time.sleep(0.01)
    return res


REQS = [(12, 10, 9, 7, (1.0, 0.5, 0.2), 1e-3), (20, 8, 8, 12, (-0.3, 0.9, 0.0), 1e-2),
        (9, 9, 16, 5, (0.1, 0.1, 1.5), 1e-4), (16, 16, 16, 9, (0.7, -0.7, 0.1), 3e-3)]


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_served_results_same_alone_and_in_the_mix(cuda, precision):
    alone = []
    for r in REQS:
        sv = make_server()
        st, rid, out = submit(sv, *r, precision=precision)
        assert st == abi.OK
        res = drain(sv, 1)
        abi.lib().fvgb_server_destroy(sv)
        assert res[rid].status == abi.OK and res[rid].steps_done == r[3]
        alone.append(out)
    sv = make_server(streams=3)
    ids = []
    for r in REQS * 2:                         # every request twice, all in flight together
        st, rid, out = submit(sv, *r, precision=precision)
        assert st == abi.OK
        ids.append((rid, out))
    res = drain(sv, len(ids))
    abi.lib().fvgb_server_destroy(sv)
    for k, (rid, out) in enumerate(ids):
        assert res[rid].status == abi.OK
        np.testing.assert_array_equal(out, alone[k % len(REQS)])
        assert res[rid].finish_s >= res[rid].start_s >= res[rid].submit_s


def test_served_matches_python_driver(cuda):
    nx, ny, nz, steps, U, D = REQS[0]
    sv = make_server()
    st, rid, out = submit(sv, nx, ny, nz, steps, U, D)
    drain(sv, 1)
    abi.lib().fvgb_server_destroy(sv)
    hm = mesh.box(nx, ny, nz)
    dm = DeviceMesh(hm)
    x, y, z = (hm.C[:, 0] - 0.5), (hm.C[:, 1] - 0.5), (hm.C[:, 2] - 0.5)
    T = neon.VolumeField(dm, np.exp(-(x * x + y * y + z * z) / (2 * 0.1 * 0.1)), [("zeroGradient", 0.0)] * 6)
    F = neon.SurfaceField(dm)
    Uc, Ub = neon.dev(np.tile(U, hm.n)), neon.dev(np.tile(U, hm.nbf))  # held until the kernel has run
    abi.check(abi.lib().fvgb_flux_vec(dm.handle, abi.ptr(Uc), abi.ptr(Ub), abi.ptr(F.values),
                                      torch.cuda.current_stream().cuda_stream))
    gam = neon.SurfaceField(dm, np.full(hm.nif + hm.nbf, D))
    dt = 0.5 * (1.0 / max(nx, ny, nz)) / np.linalg.norm(U)
    ls = neon.LinearSystem(dm)
    old = T.internal.clone()
    for _ in range(steps):
        old.copy_(T.internal)
        ls.assemble([neon.ddt(old), neon.div_explicit(F, old), neon.laplacian(gam, -1.0)], dt, T)
        ls.solve(T.internal, rel_tol=1e-8, max_iter=2000)
        T.correctBoundaryConditions()
    np.testing.assert_allclose(out, T.host(), rtol=1e-7, atol=1e-9)


def test_server_budget_and_cancel(cuda):
    sv = make_server(budget=64 << 20)
    st, _, _ = submit(sv, 160, 160, 160, 3, (1, 0, 0), 1e-3)
    assert st == abi.ERR_BUDGET
    st1, r1, _ = submit(sv, 30, 30, 30, 400, (1, 0, 0), 1e-3)
    st2, r2, _ = submit(sv, 30, 30, 30, 400, (1, 0, 0), 1e-3)
    assert st1 == st2 == abi.OK
    abi.check(abi.lib().fvgb_server_cancel(sv, r2))
    abi.check(abi.lib().fvgb_server_cancel(sv, r1))
    res = drain(sv, 2)
    abi.lib().fvgb_server_destroy(sv)
    assert res[r1].status == abi.ERR_CANCELLED and res[r2].status == abi.ERR_CANCELLED
    assert res[r1].steps_done < 400


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_rhs_only_steps_equal_full_reassembly(cuda, precision):
    """Served requests assemble the matrix once and only the rhs afterwards (the
    mixed solve then keeps its FP32 matrix copy); the results are those of a
    full reassembly every step, bit for bit."""
    outs = []
    for flags in (0, abi.SERVE_REASSEMBLE):
        sv = make_server()
        subs = [submit(sv, *r, precision=precision, flags=flags) for r in REQS]
        res = drain(sv, len(REQS))
        abi.check(abi.lib().fvgb_server_destroy(sv))
        assert all(res[rid].status == abi.OK for _, rid, _ in subs)
        outs.append([o.copy() for _, _, o in subs])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)
