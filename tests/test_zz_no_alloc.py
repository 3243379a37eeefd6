"""The allocation-free FP64 CG entry point (fvgb_pcg_csr_noalloc).

It serves callers that cannot call cudaMalloc, for example a solver embedded
in a host application that owns the device memory under a fixed budget.  The
test hands it a system in NeoN's CSR layout, exported from a LinearSystem
into device buffers the test allocated, and checks its solution against the
regular entry point, fvgb_solve, on two calls in a row: the array it keeps its
work vectors in persists between calls, so the second call must clear what
must start at zero.  Both entry points run the same arithmetic and reduction
order, so the tolerance is the one the FP64 CG tests use: bit for bit.
This file runs last so that a failure here leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh

pytestmark = pytest.mark.gpu

MAX_ROWS = 262144


def heat_system(nx, ny, nz, seed=12345):
    hm = mesh.box(nx, ny, nz, jitter=0.1, seed=seed)
    dm = DeviceMesh(hm)
    rng = np.random.default_rng(seed)
    k = neon.VolumeField(dm, np.exp(0.5 * rng.standard_normal(hm.n)), [("zeroGradient", 0.0)] * hm.npatch)
    gamma = neon.SurfaceInterpolation(dm, "linear").interpolate(k)
    T = neon.VolumeField(dm, np.full(hm.n, 300.0), [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * 5)
    ls = neon.LinearSystem(dm)
    ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(gamma, -1.0)], 0.01, T)
    return hm, dm, T, ls


def csr_on_device(dm, ls):
    ro, col, do, _, _ = dm.sparsity()
    values, rhs, _, _ = ls.export()
    dev = [torch.as_tensor(a, dtype=torch.int32).cuda() for a in (ro, col, do)]
    return dev, values, rhs


def call_noalloc(n, pattern, values, rhs, x, cfg):
    st = abi.SolverStats()
    ro, col, do = pattern
    status = abi.lib().fvgb_pcg_csr_noalloc(n, abi.ptr(ro), abi.ptr(col), abi.ptr(do), abi.ptr(values),
                                            abi.ptr(rhs), abi.ptr(x), C.byref(cfg), C.byref(st),
                                            torch.cuda.current_stream().cuda_stream)
    return status, st


def test_noalloc_matches_fvgb_solve_twice(cuda):
    hm, dm, T, ls = heat_system(40, 36, 30)
    assert hm.n <= MAX_ROWS
    pattern, values, rhs = csr_on_device(dm, ls)
    cfg = abi.SolverCfg(1e-8, 0.0, 1000, abi.PREC_FP64, 0.0, 0, 0)
    x_ref = T.internal.clone()
    st_ref = abi.SolverStats()
    abi.check(abi.lib().fvgb_solve(ls.handle, abi.ptr(x_ref), C.byref(cfg), C.byref(st_ref),
                                   torch.cuda.current_stream().cuda_stream))
    assert st_ref.num_iter > 10
    for call in range(2):
        x = T.internal.clone()
        status, st = call_noalloc(hm.n, pattern, values, rhs, x, cfg)
        assert status == abi.OK, (call, abi.status_string(status))
        assert (st.num_iter, st.status) == (st_ref.num_iter, st_ref.status), call
        assert st.init_res_norm == st_ref.init_res_norm and st.final_res_norm == st_ref.final_res_norm
        torch.testing.assert_close(x, x_ref, rtol=0, atol=0)


def test_noalloc_second_system_after_first(cuda):
    """A smaller system after a larger one: the shared array's old contents must not leak in."""
    cfg = abi.SolverCfg(1e-8, 0.0, 1000, abi.PREC_FP64, 0.0, 0, 0)
    for dims in ((30, 30, 30), (12, 10, 9)):
        hm, dm, T, ls = heat_system(*dims, seed=dims[0])
        pattern, values, rhs = csr_on_device(dm, ls)
        x_ref = T.internal.clone()
        ls.solve(x_ref, rel_tol=1e-8)
        x = T.internal.clone()
        status, st = call_noalloc(hm.n, pattern, values, rhs, x, cfg)
        assert status == abi.OK
        torch.testing.assert_close(x, x_ref, rtol=0, atol=0)


def test_noalloc_rejects_oversize_and_mixed(cuda):
    cfg = abi.SolverCfg(1e-8, 0.0, 10, abi.PREC_FP64, 0.0, 0, 0)
    dummy_i = torch.zeros(4, dtype=torch.int32, device="cuda")
    dummy_d = torch.zeros(4, dtype=torch.float64, device="cuda")
    status, _ = call_noalloc(MAX_ROWS + 1, (dummy_i, dummy_i, dummy_i), dummy_d, dummy_d, dummy_d, cfg)
    assert status == abi.ERR_INVALID_ARG
    assert b"262144" in abi.lib().fvgb_last_error()
    cfg.precision = abi.PREC_MIXED_IR
    status, _ = call_noalloc(4, (dummy_i, dummy_i, dummy_i), dummy_d, dummy_d, dummy_d, cfg)
    assert status == abi.ERR_INVALID_ARG
    # CG only: another method is refused, not run as CG
    cfg.precision = abi.PREC_FP64
    for method in (abi.SOLVER_BICGSTAB, abi.SOLVER_BICG, abi.SOLVER_MULTIGRID):
        cfg.method = method
        status, _ = call_noalloc(4, (dummy_i, dummy_i, dummy_i), dummy_d, dummy_d, dummy_d, cfg)
        assert status == abi.ERR_UNSUPPORTED


def test_noalloc_without_iteration_cap(cuda):
    """max_iter = INT32_MAX, a common way to say "no cap": the host-side
    bookkeeping of launched iterations must not overflow."""
    hm, dm, T, ls = heat_system(14, 12, 10)
    pattern, values, rhs = csr_on_device(dm, ls)
    x_ref = T.internal.clone()
    ls.solve(x_ref, rel_tol=1e-8)
    cfg = abi.SolverCfg(1e-8, 0.0, 2 ** 31 - 1, abi.PREC_FP64, 0.0, 0, 0)
    x = T.internal.clone()
    status, st = call_noalloc(hm.n, pattern, values, rhs, x, cfg)
    assert status == abi.OK and st.num_iter > 10
    torch.testing.assert_close(x, x_ref, rtol=0, atol=0)


def test_noalloc_refuses_a_capturing_stream(cuda):
    """The entry point is synchronous: on a stream being captured into a CUDA
    graph it returns ERR_UNSUPPORTED before any GPU work, and works afterwards."""
    import warnings

    hm, dm, T, ls = heat_system(10, 9, 8)
    pattern, values, rhs = csr_on_device(dm, ls)
    cfg = abi.SolverCfg(1e-8, 0.0, 1000, abi.PREC_FP64, 0.0, 0, 0)
    x = T.internal.clone()
    g = torch.cuda.CUDAGraph()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")            # the refused capture leaves an empty graph
        with torch.cuda.graph(g):
            status, _ = call_noalloc(hm.n, pattern, values, rhs, x, cfg)
    assert status == abi.ERR_UNSUPPORTED
    assert torch.equal(x, T.internal)
    status, st = call_noalloc(hm.n, pattern, values, rhs, x, cfg)
    assert status == abi.OK and st.num_iter > 5
