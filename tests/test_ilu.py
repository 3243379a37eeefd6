"""The ILU(0) preconditioner (csrc/ilu.cu): OpenFOAM's DILU as FoamAdapter
maps it, Ginkgo preconditioner::Ilu with a factorization::ParIlu
(src/compatibility/fvSolution.cpp:56-63).

The library forms the exact ILU(0) factors (the fixed point of ParIlu's
sweeps) level by level and applies them by triangular sweeps over the rows in
level order (one launch each, bounded waits for the rows a row depends on);
CG and BiCGStab around them use the solver's reduction tree.  The oracle
(oracle/fvoracle.c or_ilu_factor, or_ilu_apply, solve_cg_ilu, solve_bicgstab)
restates the sequential factorization and solves, so the GPU must match it
bit for bit: iterates, iteration counts and residual norms.  The factors
themselves are checked on the CPU by the ILU(0) property (L U = A on A's
pattern) and, on hex meshes, by OpenFOAM's DILU recurrence.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest
import scipy.sparse as sp

from foamadapter_gb300 import abi, mesh
from oracle.pyoracle import Oracle

BIG = 1 << 15


def diag_mesh(nx, ny, seed=7):
    """A 2-D box with an extra face between every cell and its (+x, +y)
    diagonal neighbour: cells c, c+1, c+nx+1 are pairwise adjacent, so ILU(0)
    updates off-diagonal entries too (on a plain hex box only the diagonal
    changes).  The extra faces get small positive areas and the centre-to-centre
    delta; faces stay in owner-then-neighbour order."""
    hm = mesh.box(nx, ny, 1, 1.0, 1.0, 1.0 / nx, jitter=0.05, seed=seed, two_d=True)
    own, nei = [hm.own], [hm.nei]
    Sf, Cf, magSf, w, delta = [hm.Sf], [hm.Cf], [hm.magSf], [hm.w], [hm.delta]
    a = 0.3 * float(hm.magSf.min())
    eo, en = [], []
    for j in range(ny - 1):
        for i in range(nx - 1):
            eo.append(j * nx + i)
            en.append((j + 1) * nx + i + 1)
    eo, en = np.asarray(eo, np.int32), np.asarray(en, np.int32)
    d = hm.C[en] - hm.C[eo]
    dist = np.linalg.norm(d, axis=1)
    unit = d / dist[:, None]
    own.append(eo)
    nei.append(en)
    Sf.append(a * unit)
    Cf.append(0.5 * (hm.C[en] + hm.C[eo]))
    magSf.append(np.full(len(eo), a))
    w.append(np.full(len(eo), 0.5))
    delta.append(1.0 / dist)
    own, nei = np.concatenate(own), np.concatenate(nei)
    order = np.lexsort((nei, own))
    cat3 = lambda xs: np.ascontiguousarray(np.concatenate([x.reshape(-1, 3) for x in xs])[order])  # noqa: E731
    cat = lambda xs: np.concatenate(xs)[order]  # noqa: E731
    return dataclasses.replace(hm, nif=len(own), own=own[order].astype(np.int32), nei=nei[order].astype(np.int32),
                               Sf=cat3(Sf), Cf=cat3(Cf), magSf=cat(magSf), w=cat(w), delta=cat(delta))


def heat_arrays(hm, seed=3, dt=0.01):
    """The oracle's assembly of ddt - laplacian(k) (lognormal k, fixed wall on
    the first patch, T0 = 300)."""
    o = Oracle(hm)
    k = np.exp(0.5 * np.random.default_rng(seed).standard_normal(hm.n))
    kf = o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
    types = np.asarray([abi.BC_FIXED_VALUE] + [abi.BC_FIXED_GRADIENT] * (hm.npatch - 1), np.int32)
    ref = np.zeros(hm.nbf)
    ref[hm.patch_offsets[0]:hm.patch_offsets[1]] = 400.0
    T, Tb = np.full(hm.n, 300.0), np.zeros(hm.nbf)
    o.bc_correct(1, types, ref, T, Tb)
    v, rhs, _, _ = o.assemble(1, [(abi.TERM_DDT, 0, 1.0, T.copy(), None), (abi.TERM_LAPLACIAN, 0, -1.0, None, kf)],
                              dt, types, ref, Tb)
    return o, kf, v, rhs


def csr_matrix(o, v):
    ro, col = o.csr_arrays()[:2]
    return sp.csr_matrix((v, col, ro))


def factors(o, lu):
    ro, col, do = o.csr_arrays()[:3]
    n = len(ro) - 1
    F = sp.csr_matrix((lu, col, ro), shape=(n, n))
    L = sp.tril(F, -1) + sp.identity(n)
    U = sp.triu(F)
    return L.tocsr(), U.tocsr()


# ------------------------------------------------------------------ CPU
@pytest.mark.parametrize("make", [lambda: mesh.box(9, 7, 5, jitter=0.1, seed=2), lambda: diag_mesh(12, 9)])
def test_ilu0_property(make):
    """(L U)_ij = a_ij on A's pattern (the defining property of ILU(0)), and
    z = M^-1 r solves L U z = r."""
    hm = make()
    o, _, v, _ = heat_arrays(hm)
    A = csr_matrix(o, v)
    lu = o.ilu_factor(v)
    L, U = factors(o, lu)
    LU = (L @ U).tocsr()
    pat = A.copy()
    pat.data[:] = 1.0
    diff = LU.multiply(pat) - A
    assert abs(diff).max() <= 1e-12 * abs(A).max()
    r = np.random.default_rng(1).standard_normal(hm.n)
    z = o.ilu_apply(lu, r)
    assert np.linalg.norm(LU @ z - r) <= 1e-12 * np.linalg.norm(r)


def test_ilu0_on_hex_is_dilu():
    """On a hex box no three cells are pairwise adjacent: the factors keep A's
    off-diagonal entries and only the diagonal changes, by OpenFOAM's DILU
    recurrence d_i = a_ii - sum_{k<i} a_ik a_ki / d_k."""
    hm = mesh.box(8, 6, 5, jitter=0.1, seed=4)
    o, _, v, _ = heat_arrays(hm)
    A = csr_matrix(o, v)
    lu = o.ilu_factor(v)
    L, U = factors(o, lu)
    Au = sp.triu(A, 1).tocsr()
    np.testing.assert_array_equal(sp.triu(U, 1).tocsr().data, Au.data)
    d = np.zeros(hm.n)
    Ad = A.toarray()
    for i in range(hm.n):
        s = Ad[i, i]
        for k in np.nonzero(Ad[i, :i])[0]:
            s -= Ad[i, k] * Ad[k, i] / d[k]
        d[i] = s
    np.testing.assert_allclose(U.diagonal(), d, rtol=1e-13)
    # and on the mesh with diagonal faces the off-diagonal entries change (fill of the pattern)
    hm2 = diag_mesh(10, 8)
    o2, _, v2, _ = heat_arrays(hm2)
    _, U2 = factors(o2, o2.ilu_factor(v2))
    assert np.any(sp.triu(U2, 1).tocsr().data != sp.triu(csr_matrix(o2, v2), 1).tocsr().data)


def test_oracle_ilu_solves_converge():
    hm = mesh.box(14, 12, 10, jitter=0.1, seed=9)
    o, _, v, rhs = heat_arrays(hm)
    xj, xi = np.full(hm.n, 300.0), np.full(hm.n, 300.0)
    sj = o.solve(v, rhs, xj, rel_tol=1e-10, max_iter=2000)
    si = o.solve(v, rhs, xi, rel_tol=1e-10, max_iter=2000, preconditioner=2)
    assert sj.status == si.status == 0 and si.num_iter < sj.num_iter
    assert np.linalg.norm(xi - xj) <= 1e-8 * np.linalg.norm(xj)
    sb = o.solve(v, rhs, np.full(hm.n, 300.0), rel_tol=1e-10, max_iter=2000, method=1, preconditioner=2)
    assert sb.status == 0
    bad = o.solve(v, rhs, np.full(hm.n, 300.0), precision=1, preconditioner=2)
    assert bad.status == 6


# ------------------------------------------------------------------ GPU
def gpu_system(hm, kind="heat", seed=3):
    import torch  # noqa: F401

    from foamadapter_gb300 import neon
    from foamadapter_gb300.mesh import DeviceMesh

    dm = DeviceMesh(hm)
    o = Oracle(hm)
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T = neon.VolumeField(dm, np.full(hm.n, 300.0), bcs)
    ls = neon.LinearSystem(dm)
    if kind == "heat":
        k = np.exp(0.5 * np.random.default_rng(seed).standard_normal(hm.n))
        kf = o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
        ls.assemble([neon.ddt(T.internal.clone()), neon.laplacian(neon.SurfaceField(dm, kf), -1.0)], 0.01, T)
    else:  # implicit upwind convection-diffusion, Courant 2
        U = np.array([1.0, 0.4, -0.2])
        F = o.flux_vec(np.tile(U, hm.n), np.tile(U, hm.nbf))
        dt = 2.0 / round(hm.n ** (1 / 3)) / float(np.linalg.norm(U))
        ls.assemble([neon.ddt(T.internal.clone()), neon.div(neon.SurfaceField(dm, F), "upwind"),
                     neon.laplacian(neon.SurfaceField(dm, np.full(hm.nif + hm.nbf, 1e-3)), -1.0)], dt, T)
    v, r, _, _ = [t.cpu().numpy() for t in ls.export()]
    return T, o, ls, v, r


def same(st, so, x, xo):
    assert st.status == so.status == abi.OK, (st.status, so.status)
    assert (st.num_iter, st.num_outer) == (so.num_iter, so.num_outer)
    assert st.init_res_norm == so.init_res_norm and st.final_res_norm == so.final_res_norm
    np.testing.assert_array_equal(x.cpu().numpy(), xo)


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(12, 10, 8), (34, 32, 31)])
@pytest.mark.parametrize("flags", [0, abi.SOLVE_RHS_BASELINE])
def test_ilu_cg_vs_oracle(cuda, dims, flags):
    """Both reduction trees (4 rows per thread below 2^15 rows, 8 above)."""
    hm = mesh.box(*dims, jitter=0.1, seed=12345)
    T, o, ls, v, r = gpu_system(hm)
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-9, max_iter=2000, preconditioner=abi.PRECOND_ILU, flags=flags)
    xo = T.host().copy()
    so = o.solve(v, r, xo, rel_tol=1e-9, max_iter=2000, preconditioner=2, flags=2 if flags else 0)
    same(st, so, x, xo)
    sj = ls.solve(T.internal.clone(), rel_tol=1e-9, max_iter=2000, flags=flags)
    assert st.num_iter < sj.num_iter


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(13, 11, 9), (34, 32, 31)])
def test_ilu_bicgstab_vs_oracle(cuda, dims):
    hm = mesh.box(*dims, jitter=0.1, seed=5)
    T, o, ls, v, r = gpu_system(hm, "convection")
    x = T.internal.clone()
    st = ls.solve(x, rel_tol=1e-10, max_iter=3000, method=abi.SOLVER_BICGSTAB, preconditioner=abi.PRECOND_ILU)
    xo = T.host().copy()
    so = o.solve(v, r, xo, rel_tol=1e-10, max_iter=3000, method=1, preconditioner=2)
    same(st, so, x, xo)
    sj = ls.solve(T.internal.clone(), rel_tol=1e-10, max_iter=3000, method=abi.SOLVER_BICGSTAB)
    assert st.num_iter < sj.num_iter


@pytest.mark.gpu
def test_ilu_repeated_solves_are_identical(cuda):
    """The triangular sweeps leave their work vectors pending for the next
    application, and each solve starts from a filled one: CG, BiCGStab, CG
    again and BiCGStab again on one system give the same bits each time."""
    hm = mesh.box(34, 32, 31, jitter=0.1, seed=8)
    T, o, ls, v, r = gpu_system(hm)
    runs = []
    for method in (abi.SOLVER_CG, abi.SOLVER_BICGSTAB, abi.SOLVER_CG, abi.SOLVER_BICGSTAB, abi.SOLVER_CG):
        x = T.internal.clone()
        st = ls.solve(x, rel_tol=1e-10, max_iter=2000, method=method, preconditioner=abi.PRECOND_ILU)
        assert st.status == abi.OK
        runs.append((method, st.num_iter, st.final_res_norm, x.cpu().numpy()))
    for a, b in ((0, 2), (2, 4), (1, 3)):
        assert runs[a][:3] == runs[b][:3]
        np.testing.assert_array_equal(runs[a][3], runs[b][3])


@pytest.mark.gpu
def test_ilu_with_fill_updates_vs_oracle(cuda):
    """A mesh whose matrix graph has triangles: the factorization's update
    list changes off-diagonal entries; CG and BiCGStab stay bit-exact."""
    hm = diag_mesh(40, 31)
    T, o, ls, v, r = gpu_system(hm)
    for method, om in ((abi.SOLVER_CG, 0), (abi.SOLVER_BICGSTAB, 1)):
        x = T.internal.clone()
        st = ls.solve(x, rel_tol=1e-10, max_iter=2000, method=method, preconditioner=abi.PRECOND_ILU)
        xo = T.host().copy()
        so = o.solve(v, r, xo, rel_tol=1e-10, max_iter=2000, method=om, preconditioner=2)
        same(st, so, x, xo)


@pytest.mark.gpu
def test_ilu_follows_matrix_changes_and_caps(cuda):
    """The factorization is part of every solve: a reassembled matrix is
    factored again.  The iteration cap and max_iter 0 behave as in Jacobi-PCG."""
    from foamadapter_gb300 import neon

    hm = mesh.box(12, 10, 8, jitter=0.1, seed=6)
    T, o, ls, v, r = gpu_system(hm)
    x = T.internal.clone()
    ls.solve(x, rel_tol=1e-9, preconditioner=abi.PRECOND_ILU)
    # a new matrix (twice the time step) on the same system
    ls.assemble([neon.ddt(T.internal.clone()),
                 neon.laplacian(neon.SurfaceField(ls.mesh, np.full(hm.nif + hm.nbf, 2.0)), -1.0)], 0.02, T)
    v2, r2, _, _ = [t.cpu().numpy() for t in ls.export()]
    x2 = T.internal.clone()
    st = ls.solve(x2, rel_tol=1e-9, preconditioner=abi.PRECOND_ILU)
    xo = T.host().copy()
    so = o.solve(v2, r2, xo, rel_tol=1e-9, preconditioner=2)
    same(st, so, x2, xo)
    st = ls.solve(T.internal.clone(), rel_tol=1e-14, max_iter=2, preconditioner=abi.PRECOND_ILU)
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_iter == 2
    st = ls.solve(T.internal.clone(), rel_tol=1e-9, max_iter=0, preconditioner=abi.PRECOND_ILU)
    assert st.status == abi.ERR_NOT_CONVERGED and st.num_iter == 0


@pytest.mark.gpu
def test_ilu_refuses_what_it_does_not_cover(cuda):
    from foamadapter_gb300 import neon

    hm = mesh.box(10, 8, 6, jitter=0.1, seed=6)
    T, o, ls, v, r = gpu_system(hm)
    x = T.internal.clone()
    for kw in (dict(precision=abi.PREC_MIXED_IR), dict(method=abi.SOLVER_BICG)):
        with pytest.raises(abi.FvgbError) as e:
            ls.solve(x, preconditioner=abi.PRECOND_ILU, **kw)
        assert e.value.status == abi.ERR_UNSUPPORTED
    b = neon.Batch(ls, [0, hm.n])
    import ctypes as C
    cfg = abi.SolverCfg(1e-8, 0.0, 100, abi.PREC_FP64, 0.1, 1000, 50, 0, 0, abi.SOLVER_CG, abi.PRECOND_ILU)
    assert abi.lib().fvgb_batch_solve(b.handle, abi.ptr(x), C.byref(cfg), None, None) == abi.ERR_UNSUPPORTED


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["setup_operator", "setup_stencil3D", "setup_unstructuredMesh"])
def test_ilu_on_reference_meshes_vs_oracle(cuda, case):
    """The reference's own test meshes (polyMesh fixtures): ILU(0) CG on a
    heat system and ILU(0) BiCGStab on an upwind convection-diffusion system,
    bit-exact against the oracle."""
    from conftest import load_polymesh

    hm, _ = load_polymesh(case)
    for kind, method, om in (("heat", abi.SOLVER_CG, 0), ("convection", abi.SOLVER_BICGSTAB, 1)):
        T, o, ls, v, r = gpu_system(hm, kind)
        x = T.internal.clone()
        st = ls.solve(x, rel_tol=1e-12, max_iter=500, method=method, preconditioner=abi.PRECOND_ILU)
        xo = T.host().copy()
        so = o.solve(v, r, xo, rel_tol=1e-12, max_iter=500, method=om, preconditioner=2)
        same(st, so, x, xo)
