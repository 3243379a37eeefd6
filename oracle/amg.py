"""Aggregation multigrid restated in numpy: test infrastructure only.

Only ``tests/`` import this module, as the checker of the library's
multigrid preconditioner (``foamadapter_gb300/csrc/amg.cu``).  The reference
reaches multigrid through Ginkgo (solver::Multigrid with multigrid::Pgm,
``tutorials/cylinder2D/system/gko/config.mg.json``), which is not in the
reference checkout: parity with Ginkgo is unpinned.  This file restates the
same published method independently of the CUDA/C++ code, so that the
library's aggregation is checked exactly and its V-cycle to rounding:

* parallel graph match: strength |a_ij|; up to 15 rounds in which every
  unaggregated row picks its strongest unaggregated neighbour (ties: the lower
  index) and mutual picks form pairs, until at most 5% of the rows are left or
  no pair forms; a row left over joins its strongest aggregated neighbour's
  aggregate or stays alone; aggregates numbered by their lowest row;
* two matchings per level (the pairs matched again on their Galerkin
  matrix, double pairwise aggregation);
* Galerkin coarse matrices P^T A P with the piecewise-constant P, levels until
  at most 256 rows remain, a level keeps more than 90% of the rows, or 25
  levels;
* V-cycle: x = w D^-1 b, r = b - A x, restriction by aggregate sums, the
  coarser level (the coarsest solved exactly), y = x + P x_c,
  out = y + w D^-1 (b - A y), w = 0.9;
* the multigrid solver on its own (Ginkgo's solver::Multigrid, which
  FoamAdapter maps OpenFOAM's GAMG to, src/compatibility/fvSolution.cpp:27):
  x += V(b - A x) until ||b - A x|| <= max(rel_tol * baseline, abs_tol).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

OMEGA = 0.9
COARSE_ROWS = 256
MAX_LEVELS = 25


def pgm_aggregate(n, rp, ci, v, rounds=15, left_ratio=0.05):
    tmp = np.full(n, -1, np.int64)
    nxt = 0
    left = n
    for _ in range(rounds):
        pick = np.full(n, -1, np.int64)
        for i in range(n):
            if tmp[i] >= 0:
                continue
            best = 0.0
            for k in range(rp[i], rp[i + 1]):
                j = ci[k]
                if j == i or tmp[j] >= 0:
                    continue
                w = abs(v[k])
                if w > best:  # columns ascend: the first of equal strengths is the lower index
                    best, pick[i] = w, j
        formed = 0
        for i in range(n):
            j = pick[i]
            if tmp[i] < 0 and j > i and pick[j] == i:
                tmp[i] = tmp[j] = nxt
                nxt += 1
                formed += 1
                left -= 2
        if formed == 0 or left <= left_ratio * n:
            break
    late = np.full(n, -1, np.int64)
    for i in range(n):
        if tmp[i] >= 0:
            continue
        best, to = 0.0, -1
        for k in range(rp[i], rp[i + 1]):
            j = ci[k]
            if j == i or tmp[j] < 0:
                continue
            w = abs(v[k])
            if w > best:
                best, to = w, j
        late[i] = tmp[to] if to >= 0 else -1
    for i in range(n):
        if tmp[i] < 0:
            if late[i] >= 0:
                tmp[i] = late[i]
            else:
                tmp[i] = nxt
                nxt += 1
    renum = np.full(nxt, -1, np.int64)
    agg = np.empty(n, np.int32)
    nc = 0
    for i in range(n):
        if renum[tmp[i]] < 0:
            renum[tmp[i]] = nc
            nc += 1
        agg[i] = renum[tmp[i]]
    return agg, nc


def hierarchy(rp, ci, v):
    """[(A_l, agg_l)] with A_l scipy CSR and agg_l the aggregation to level l+1 (None for the last)."""
    A = sp.csr_matrix((np.asarray(v, float), np.asarray(ci), np.asarray(rp)))
    levels = []
    while len(levels) + 1 < MAX_LEVELS and A.shape[0] > COARSE_ROWS:
        A.sort_indices()
        agg, nc = pgm_aggregate(A.shape[0], A.indptr, A.indices, A.data)
        if nc > 0.9 * A.shape[0]:
            break
        if nc > COARSE_ROWS:  # double pairwise: match the pairs again on their Galerkin matrix
            P1 = sp.csr_matrix((np.ones(A.shape[0]), (np.arange(A.shape[0]), agg)), shape=(A.shape[0], nc))
            A1 = (P1.T @ A @ P1).tocsr()
            A1.sort_indices()
            agg2, nc2 = pgm_aggregate(nc, A1.indptr, A1.indices, A1.data)
            if nc2 <= 0.9 * nc:
                agg = agg2[agg]
                _, first = np.unique(agg, return_index=True)
                order = np.argsort(first)          # aggregates numbered by their lowest row
                renum = np.empty(nc2, np.int64)
                renum[order] = np.arange(nc2)
                agg = renum[agg].astype(np.int32)
                nc = nc2
        P = sp.csr_matrix((np.ones(A.shape[0]), (np.arange(A.shape[0]), agg)), shape=(A.shape[0], nc))
        levels.append((A, agg, P))
        A = (P.T @ A @ P).tocsr()
    levels.append((A, None, None))
    return levels


def vcycle(levels, b, l=0):
    A, agg, P = levels[l]
    if agg is None:
        return np.linalg.solve(A.toarray(), b)
    dinv = 1.0 / A.diagonal()
    x = OMEGA * dinv * b
    r = b - A @ x
    xc = vcycle(levels, P.T @ r, l + 1)
    y = x + xc[agg]
    return y + OMEGA * dinv * (b - A @ y)


def mg_solve(levels, b, x, rel_tol, abs_tol, max_iter, rhs_baseline=False):
    """The multigrid solver: (x, cycles, initial and final residual norms,
    status 0 / 3 not converged / 4 breakdown as fvgb_status), with the
    library's stopping rules (checked after every cycle; the baseline is
    ||r_0||, or ||b|| when rhs_baseline)."""
    A = levels[0][0]
    x = np.array(x, dtype=float)
    r = b - A @ x
    res0 = float(np.linalg.norm(r))
    base = float(np.linalg.norm(b)) if rhs_baseline else res0
    tol = max(rel_tol * base, abs_tol)
    if not np.isfinite(res0):
        return x, 0, res0, res0, 4
    if not res0 > tol or res0 == 0.0:
        return x, 0, res0, res0, 0
    if max_iter <= 0:
        return x, 0, res0, res0, 3
    it, res = 0, res0
    while True:
        x = x + vcycle(levels, r)
        r = b - A @ x
        res = float(np.linalg.norm(r))
        it += 1
        if not np.isfinite(res):
            return x, it, res0, res, 4
        if not res > tol:
            return x, it, res0, res, 0
        if it >= max_iter:
            return x, it, res0, res, 3
