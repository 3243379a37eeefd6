"""Device-built box meshes and the serving loop.

* fvgb_mesh_create_boxes builds packed boxes on the device with the host
  builder's OpenFOAM geometry and operation order: every operator and solve
  on it gives the bits of the host-built mesh.
* The server runs every request exactly as it would run alone: a request's
  final field is bit-identical whether it ran by itself or among others
  (the continuous-batching equivalence the serving design promises), and
  bit-identical to the CPU oracle running the same IMEX steps.
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
        np.testing.assert_array_equal(a, b)
    abi.lib().fvgb_mesh_destroy(hdev)


def make_server(budget=8 << 30, streams=4, max_active=64):
    cfg = abi.ServerCfg(budget, streams, max_active)
    h = C.c_void_p()
    abi.check(abi.lib().fvgb_server_create(C.byref(cfg), C.byref(h)))
    return h


_KEEP = []  # initial fields stay alive until their requests are reported


def submit(server, nx, ny, nz, steps, U, D, precision=abi.PREC_FP64, flags=0, dt=0.0, T0=None):
    out = np.zeros(nx * ny * nz)
    req = abi.ServeRequest(nx=nx, ny=ny, nz=nz, steps=steps, U=(C.c_double * 3)(*U), D=D, dt=dt,
                           precision=precision, kernel_mode=0, flags=flags, T_out=out.ctypes.data,
                           T_init=None if T0 is None else T0.ctypes.data)
    if T0 is not None:
        _KEEP.append(T0)
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


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
def test_served_requests_match_the_oracle(cuda, precision):
    """Every request of a mix (served together, and one of them also alone)
    gives the oracle's field bit for bit after the same IMEX steps from the same
    initial field, with the same total number of CG iterations."""
    from oracle.apps import ServedRequestCPU

    rng = np.random.default_rng(17)
    reqs = []
    for nx, ny, nz, steps, U, D in REQS:
        dt = 0.5 * (1.0 / max(nx, ny, nz)) / float(np.sqrt(np.dot(U, U)))
        reqs.append((nx, ny, nz, steps, U, D, dt, 1.0 + rng.random(nx * ny * nz)))
    sv = make_server(streams=3)
    subs = [submit(sv, nx, ny, nz, st, U, D, precision=precision, dt=dt, T0=T0)
            for nx, ny, nz, st, U, D, dt, T0 in reqs]
    res = drain(sv, len(subs))
    abi.lib().fvgb_server_destroy(sv)
    sv = make_server()
    nx, ny, nz, st, U, D, dt, T0 = reqs[1]
    _, rid1, alone = submit(sv, nx, ny, nz, st, U, D, precision=precision, dt=dt, T0=T0)
    res1 = drain(sv, 1)
    abi.lib().fvgb_server_destroy(sv)
    for (nx, ny, nz, steps, U, D, dt, T0), (status, rid, out) in zip(reqs, subs):
        cpu = ServedRequestCPU(nx, ny, nz, U, D, dt, T0, precision=1 if precision == abi.PREC_MIXED_IR else 0)
        for _ in range(steps):
            cpu.step()
        assert status == abi.OK and res[rid].status == abi.OK and res[rid].steps_done == steps
        assert res[rid].total_iters == cpu.iters
        np.testing.assert_array_equal(out, cpu.T)
        if (nx, ny, nz) == reqs[1][:3]:
            assert res1[rid1].total_iters == cpu.iters
            np.testing.assert_array_equal(alone, cpu.T)


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
