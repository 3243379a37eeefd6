"""A whole implicit time step as one CUDA graph (fvgb_step_*): copy of the old
field, assembly, the batched solve with its device-side loops, boundary
update.  Launching it gives the bits of the same calls made one by one."""
import ctypes as C

import numpy as np
import pytest
import torch

from foamadapter_gb300 import abi, mesh, neon
from foamadapter_gb300.mesh import DeviceMesh

pytestmark = pytest.mark.gpu


def packed_case(seed=3):
    rng = np.random.default_rng(seed)
    parts = [mesh.box(*rng.integers(5, 14, size=3), jitter=0.1, seed=seed + k) for k in range(5)]
    big, ranges, _ = mesh.concat(parts)
    dm = DeviceMesh(big)
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (big.npatch - 1)
    T = neon.VolumeField(dm, np.full(big.n, 300.0), bcs)
    gamma = neon.SurfaceField(dm, np.exp(rng.standard_normal(big.nif + big.nbf)))
    return big, np.asarray(ranges, np.int32), dm, T, gamma


@pytest.mark.parametrize("method", [abi.SOLVER_CG, abi.SOLVER_BICGSTAB])
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED_IR])
@pytest.mark.parametrize("batched", [True, False])
def test_step_graph_equals_separate_calls(cuda, precision, batched, method):
    L, s = abi.lib(), torch.cuda.current_stream().cuda_stream
    out = []
    for use_graph in (False, True):
        big, ranges, dm, T, gamma = packed_case()
        T_old = T.internal.clone()
        ls = neon.LinearSystem(dm)
        terms = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(T_old), neon.laplacian(gamma, -1.0))])
        bc = T.bc_struct()
        batch = neon.Batch(ls, ranges) if batched else None
        ncases = len(ranges) // 2 if batched else 1
        cfg = abi.SolverCfg(1e-9, 0.0, 2000, precision, 0.1, 1000, 50, 1, 0, method)
        stats = torch.zeros(ncases * 8, dtype=torch.int32, device="cuda")  # fvgb_solver_stats is 32 bytes
        if use_graph:
            step = C.c_void_p()
            abi.check(L.fvgb_step_create(ls.handle, batch.handle if batched else None, terms, 2, 0.01, C.byref(bc),
                                         abi.ptr(T.internal), abi.ptr(T.boundary), abi.ptr(T_old), C.byref(cfg),
                                         abi.ptr(stats), C.byref(step)))
            for _ in range(3):
                abi.check(L.fvgb_step_launch(step, s))
            torch.cuda.synchronize()
            abi.check(L.fvgb_step_destroy(step))
        else:
            for _ in range(3):
                T_old.copy_(T.internal)
                abi.check(L.fvgb_assemble(ls.handle, terms, 2, 0.01, C.byref(bc), abi.ptr(T.boundary), s))
                if batched:
                    abi.check(L.fvgb_batch_solve_async(batch.handle, abi.ptr(T.internal), C.byref(cfg),
                                                       abi.ptr(stats), s))
                else:
                    abi.check(L.fvgb_solve_async(ls.handle, abi.ptr(T.internal), C.byref(cfg), abi.ptr(stats), s))
                T.correctBoundaryConditions()
            torch.cuda.synchronize()
        st = stats.view(ncases, 8).cpu().numpy()
        out.append((T.internal.cpu().numpy(), T.boundary.cpu().numpy(), st))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])
    assert (out[1][2][:, 6] == abi.OK).all()  # status word of every case
    assert (out[1][2][:, 4] > 0).all()         # iterations of the last step


def test_step_graph_rejects_host_loop(cuda):
    big, ranges, dm, T, gamma = packed_case()
    ls = neon.LinearSystem(dm)
    T_old = T.internal.clone()
    terms = (abi.Term * 2)(*[t.struct() for t in (neon.ddt(T_old), neon.laplacian(gamma, -1.0))])
    bc = T.bc_struct()
    cfg = abi.SolverCfg(1e-9, 0.0, 2000, abi.PREC_FP64, 0.1, 1000, 50, 3)
    step = C.c_void_p()
    r = abi.lib().fvgb_step_create(ls.handle, None, terms, 2, 0.01, C.byref(bc), abi.ptr(T.internal),
                                   abi.ptr(T.boundary), abi.ptr(T_old), C.byref(cfg), None, C.byref(step))
    assert r == abi.ERR_INVALID_ARG
