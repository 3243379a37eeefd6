"""The oracle's Jacobi-CG and mixed-precision refinement on the CPU (no GPU).

The mixed solve scales the FP32 residual of every refinement step by a power
of two, so a system whose right-hand side and initial guess are scaled by 2^-100
is solved with exactly the same FP32 inner iterates: the solution is the
unscaled one times 2^-100, bit for bit, with the same iteration counts.
Without the scaling the FP32 dot products of that residual (about 1e-60)
underflow and the refinement stalls.
"""
import numpy as np
import pytest

from foamadapter_gb300 import mesh
from oracle.pyoracle import Oracle

DDT, LAP = 0, 1
FIXED_VALUE, FIXED_GRADIENT = 1, 2


def heat_system(nx=10, ny=9, nz=7, seed=3):
    hm = mesh.box(nx, ny, nz, jitter=0.1, seed=seed)
    o = Oracle(hm)
    rng = np.random.default_rng(seed)
    k = np.exp(0.5 * rng.standard_normal(hm.n))
    gamma = o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
    types = np.asarray([FIXED_VALUE] + [FIXED_GRADIENT] * (hm.npatch - 1), np.int32)
    ref = np.zeros(hm.nbf)
    ref[hm.patch_slice("xmin")] = 400.0
    T = np.full(hm.n, 300.0)
    Tb = np.zeros(hm.nbf)
    o.bc_correct(1, types, ref, T, Tb)
    v, r, _, _ = o.assemble(1, [(DDT, 0, 1.0, T.copy(), None), (LAP, 0, -1.0, None, gamma)], 0.01, types, ref, Tb)
    return o, v, r, T


@pytest.mark.parametrize("precision", [0, 1])
def test_solve_reaches_tolerance(precision):
    o, v, r, T = heat_system()
    x = T.copy()
    st = o.solve(v, r, x, rel_tol=1e-8, precision=precision)
    assert st.status == 0 and st.num_iter > 5
    true = np.linalg.norm(o.apply_operator(v, r, 1, x))
    assert true <= 1.01e-8 * st.init_res_norm


def test_mixed_is_exactly_scale_invariant():
    o, v, r, T = heat_system()
    x1 = T.copy()
    s1 = o.solve(v, r, x1, rel_tol=1e-8, precision=1)
    sc = 2.0 ** -100
    x2 = T * sc
    s2 = o.solve(v, r * sc, x2, rel_tol=1e-8, precision=1)
    assert s1.status == 0 and s2.status == 0
    assert (s1.num_iter, s1.num_outer) == (s2.num_iter, s2.num_outer)
    assert s2.init_res_norm == s1.init_res_norm * sc and s2.final_res_norm == s1.final_res_norm * sc
    np.testing.assert_array_equal(x2, x1 * sc)


def convection_system(nx=10, ny=9, nz=7, seed=4):
    """ddt + implicit upwind convection - laplacian: a nonsymmetric system."""
    hm = mesh.box(nx, ny, nz, jitter=0.1, seed=seed)
    o = Oracle(hm)
    rng = np.random.default_rng(seed)
    U = np.array([1.0, 0.4, -0.2])
    F = o.flux_vec(np.tile(U, hm.n), np.tile(U, hm.nbf))
    gamma = np.full(hm.nif + hm.nbf, 1e-2)
    types = np.asarray([FIXED_VALUE] + [FIXED_GRADIENT] * (hm.npatch - 1), np.int32)
    ref = np.zeros(hm.nbf)
    ref[hm.patch_slice("xmin")] = 1.0
    T = rng.random(hm.n)
    Tb = np.zeros(hm.nbf)
    o.bc_correct(1, types, ref, T, Tb)
    DIV = 2
    v, r, _, _ = o.assemble(1, [(DDT, 0, 1.0, T.copy(), None), (DIV, 1, 1.0, None, F), (LAP, 0, -1.0, None, gamma)],
                            0.05, types, ref, Tb)
    return o, v, r, T


def test_bicgstab_solves_nonsymmetric_system():
    o, v, r, T = convection_system()
    x = T.copy()
    st = o.solve(v, r, x, rel_tol=1e-10, max_iter=500, method=1)
    assert st.status == 0 and 0 < st.num_iter < 500
    true = np.linalg.norm(o.apply_operator(v, r, 1, x))
    assert true <= 1e-9 * st.init_res_norm



@pytest.mark.parametrize("rel_tol", [1e-8, 1e-12])
def test_mixed_bicgstab_reaches_the_fp64_residual(rel_tol):
    """FP32 inner BiCGStab in FP64 refinement: the FP64 residual of the result
    reaches rel_tol, and the solution agrees with the FP64 BiCGStab's."""
    o, v, r, T = convection_system()
    x64 = T.copy()
    s64 = o.solve(v, r, x64, rel_tol=rel_tol, max_iter=2000, method=1)
    xm = T.copy()
    sm = o.solve(v, r, xm, rel_tol=rel_tol, max_iter=2000, method=1, precision=1)
    assert sm.status == 0 and sm.num_outer >= 1 and sm.init_res_norm == s64.init_res_norm
    true = np.linalg.norm(o.apply_operator(v, r, 1, xm))
    assert true <= rel_tol * sm.init_res_norm
    assert sm.final_res_norm <= rel_tol * sm.init_res_norm
    assert np.abs(xm - x64).max() <= 10 * rel_tol * np.abs(x64).max()


def test_mixed_bicgstab_scale_invariance():
    """A power-of-two scale of the system scales every iterate exactly."""
    o, v, r, T = convection_system(seed=6)
    x1, x2 = T.copy(), T.copy() * 2.0 ** -40
    s1 = o.solve(v, r, x1, rel_tol=1e-9, max_iter=2000, method=1, precision=1)
    s2 = o.solve(v, r * 2.0 ** -40, x2, rel_tol=1e-9, max_iter=2000, method=1, precision=1)
    assert s1.status == s2.status == 0 and s1.num_iter == s2.num_iter
    np.testing.assert_array_equal(x2, x1 * 2.0 ** -40)
