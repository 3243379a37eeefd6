// ILU(0)-preconditioned CG and BiCGStab (FP64) for a single scalar system.
//
// OpenFOAM's DILU preconditioner maps, through FoamAdapter, to Ginkgo's
// preconditioner::Ilu with a factorization::ParIlu and reverse_apply false
// (src/compatibility/fvSolution.cpp:56-63; the reference's
// test/setup_advection case names it beside PBiCGStab).  ParIlu's fixed-point
// sweeps approach the ILU(0) factors of A's sparsity pattern, and Ginkgo runs
// them asynchronously (not reproducible on a GPU); this file forms those
// factors exactly, which makes the preconditioner deterministic:
//
//  * symbolic (host, once per system, from the mesh's CSR pattern): for every
//    entry (i,k) left of the diagonal the pairs of entries (i,j), (k,j) with
//    j > k in both rows (the IKJ update list), and the rows grouped by level
//    of the lower and of the upper triangle (a row's level is one more than
//    the highest level of the rows it depends on);
//  * factorization (device, inside every solve's graph, so it follows the
//    matrix): level by level, one thread per row, entries k ascending:
//    l_ik = a_ik / u_kk, then a_ij = fma(-l_ik, u_kj, a_ij) over the update
//    list.  On hex meshes (no three cells pairwise adjacent) only the diagonal
//    changes: OpenFOAM's DILU;
//  * application z = U^-1 L^-1 r: forward y_i = r_i - sum_k l_ik y_k, then
//    backward z_i = (y_i - sum_j u_ij z_j) / u_ii, each a single sweep over
//    the rows in level order, fma chains in column order.
//
// Each factorization level is one kernel node of the solve's CUDA graph.  Each
// triangular solve of an application is one launch: rows in level order,
// each waiting (bounded) for the rows it depends on (the sweeps below).
// Every row is computed by the same operations in the same order as the
// sequential restatement (oracle/fvoracle.c or_ilu_*): the bits are those of
// the exact sequential factorization and solves.  A 128^3 box has 382 levels
// per triangle, which bound the sweeps' speed: one dependent row after another.
//
// CG and BiCGStab (right preconditioning) around it follow the Jacobi solvers'
// stopping rules; every dot product uses the solver's reduction tree (256
// threads of R rows, R = 8 from 2^15 rows, else 4; block tree; last-block
// final tree), so the oracle's restatements give the same bits.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace {

constexpr int kT = 256;

struct IluState {
    double* x;
    double rel_tol, abs_tol;
    int32_t max_iter, want_bbase;
    double bbase;
    double res0, res, tol;
    double rz, alpha, beta;           // CG
    double rho, rho_prev, omega;      // BiCGStab
    int32_t iter, status, done, half;
    unsigned counter;
    unsigned ticket;      // the next chunk of a triangular sweep (0 between launches)
    int32_t sweep_abort;  // a sweep's wait ran out: the solve ends with FVGB_ERR_CUDA
    fvgb_solver_stats* stats_out;
    fvgb_solver_stats stats;
};

struct Csr {
    int n;
    const int* ro;
    const int* col;
    const int* dof;  // diagonal offset of every row
};

__device__ __forceinline__ volatile const int32_t& done_flag(const IluState* st) { return st->done; }

// ------------------------------------------------------------ reduction tree
// Row j of this thread: the solver's tree layout.
__device__ __forceinline__ int tree_row(int R, int j) {
    return blockIdx.x * (kT * R) + (threadIdx.x >> 5) * (32 * R) + j * 32 + (threadIdx.x & 31);
}

// Block sum of one value per thread; valid in warp 0.
__device__ __forceinline__ double block_tree(double v, double* sm) {
    sm[threadIdx.x] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x < 32) {
        s = sm[threadIdx.x];
#pragma unroll
        for (int k = 1; k < kT / 32; ++k) s = s + sm[threadIdx.x + 32 * k];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, off);
    }
    __syncthreads();
    return s;
}

__device__ __forceinline__ double final_tree(const double* part, int nb, double* sm) {
    double a = 0.0;
    for (int i = threadIdx.x; i < nb; i += kT) a = a + __ldcg(&part[i]);
    return block_tree(a, sm);
}

// true in the block that arrives last (the counter wraps back to 0)
__device__ __forceinline__ bool arrive_last(unsigned* counter) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicInc(counter, gridDim.x - 1) == gridDim.x - 1;
    }
    __syncthreads();
    return last;
}

// Up to two tree dots of this launch: the block partials, then in the last
// block the totals (valid in thread 0).  Returns false outside the last block.
__device__ __forceinline__ bool tree_dots(IluState* st, double* pa, double* pb, double a, double b, int ndots,
                                          double* ta, double* tb) {
    __shared__ double sma[kT], smb[kT];
    const double ba = block_tree(a, sma);
    const double bb = ndots > 1 ? block_tree(b, smb) : 0.0;
    if (threadIdx.x == 0) {
        pa[blockIdx.x] = ba;
        if (ndots > 1) pb[blockIdx.x] = bb;
    }
    if (!arrive_last(&st->counter)) return false;
    *ta = final_tree(pa, gridDim.x, sma);
    if (ndots > 1) *tb = final_tree(pb, gridDim.x, smb);
    return true;
}

__device__ __forceinline__ double csr_row(const Csr& A, const double* __restrict__ a, const double* x, int i) {
    double s = 0.0;
    for (int e = __ldg(&A.ro[i]); e < __ldg(&A.ro[i + 1]); ++e) s = fma(__ldg(&a[e]), x[__ldg(&A.col[e])], s);
    return s;
}

// ------------------------------------------------------------ setup kernels
__global__ void k_il_params(IluState* st, double* x, double rel_tol, double abs_tol, int max_iter,
                            fvgb_solver_stats* out, int want_bbase) {
    st->x = x;
    st->rel_tol = rel_tol;
    st->abs_tol = abs_tol;
    st->max_iter = max_iter;
    st->want_bbase = want_bbase;
    st->bbase = -1.0;
    st->stats_out = out;
    st->counter = 0;
    st->ticket = 0;
    st->sweep_abort = 0;
    st->done = 0;
    st->half = 0;
    st->iter = 0;
    st->status = FVGB_OK;
}

// ||b|| when the solve asks for Ginkgo's default ResidualNorm baseline
__global__ void __launch_bounds__(kT)
    k_il_bnorm(IluState* st, int n, int R, const double* __restrict__ b, double* pa) {
    if (!st->want_bbase) return;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i < n) acc = fma(__ldg(&b[i]), __ldg(&b[i]), acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) st->bbase = sqrt(t);
}

// A's values in CSR order, into the matrix copy and the factor
__global__ void __launch_bounds__(kT)
    k_il_gather(int nnz, const int* __restrict__ csr_pos, const double* __restrict__ slots, double* __restrict__ a,
                double* __restrict__ lu) {
    const int k = blockIdx.x * kT + threadIdx.x;
    if (k < nnz) a[k] = lu[k] = __ldg(&slots[__ldg(&csr_pos[k])]);
}

// One level of the factorization: row i's entries left of the diagonal in
// column order, each dividing by the pivot of its row and updating row i.
__global__ void __launch_bounds__(kT)
    k_il_factor(Csr A, const int* __restrict__ rows, int cnt, const int* __restrict__ op_ptr,
                const int* __restrict__ op_f, const int* __restrict__ op_g, double* lu) {
    const int t = blockIdx.x * kT + threadIdx.x;
    if (t >= cnt) return;
    const int i = __ldg(&rows[t]);
    const int b = __ldg(&A.ro[i]), d = b + __ldg(&A.dof[i]);
    for (int e = b; e < d; ++e) {
        const int k = __ldg(&A.col[e]);
        const double l = lu[e] / __ldcg(&lu[__ldg(&A.ro[k]) + __ldg(&A.dof[k])]);
        lu[e] = l;
        for (int o = __ldg(&op_ptr[e]); o < __ldg(&op_ptr[e + 1]); ++o) {
            const int f = __ldg(&op_f[o]);
            lu[f] = fma(-l, __ldcg(&lu[__ldg(&op_g[o])]), lu[f]);
        }
    }
}

// ------------------------------------------------------ triangular sweeps
// One launch per triangle.  The rows are taken in level order, a chunk of kT
// rows at a time, by a block ticket: a row depends only on rows of lower
// levels, which sit earlier in that order, in chunks that blocks already
// running took before (or in its own block), so every wait ends.  A row's
// output holds kPending until the row is computed; the one 64-bit store of
// the value is the signal (relaxed loads and stores at GPU scope, no flag and
// no fence).  kPending is a signalling NaN: FP64 arithmetic writes quiet NaNs
// at most, and every value a sweep writes is an arithmetic result.  The
// forward sweep sets the backward sweep's output to kPending row by row, the
// backward sweep the forward sweep's output after reading it; the solve graph
// fills the latter once at its start.
constexpr unsigned long long kPending = 0x7ff00000deadbeefull;
constexpr int kSweepBlocksPerSM = 1;  // 128^3 ILU-CG: 144 ms at 1, 157 at 2

__device__ __forceinline__ bool pending(double v) { return (unsigned long long)__double_as_longlong(v) == kPending; }

__device__ __forceinline__ double ld_relaxed(const double* p) {
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(double* p, double v) {
    asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The wait for a pending row value: false when the sweep is aborted, because
// this wait ran out (about a second, or 2^26 polls) or another one did.
__device__ __noinline__ bool await_pending(const double* p, double& v, IluState* st) {
    const unsigned long long t0 = now_ns();
    for (unsigned k = 1; k < (1u << 26); ++k) {
        if (k > 2) __nanosleep(k < 16 ? 32 : 256);  // rows far from the wavefront poll less
        v = ld_relaxed(p);
        if (!pending(v)) return true;
        if ((k & 31) == 0) {
            if (*(volatile const int32_t*)&st->sweep_abort) return false;
            if (now_ns() - t0 > 1000000000ull) break;
        }
    }
    atomicExch(&st->sweep_abort, 1);
    return false;
}

// Row value of this sweep at p (see await_pending)
__device__ __forceinline__ bool await_row(const double* p, double& v, IluState* st) {
    v = ld_relaxed(p);
    return !pending(v) || await_pending(p, v, st);
}

__global__ void __launch_bounds__(kT) k_il_pending(int n, double* y) {
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) y[i] = __longlong_as_double((long long)kPending);
}

// out = (s - sum over entries e in [e0, e1) of lu_e v_{col_e}) [/ piv], the
// sum in entry order over values of this sweep.  The first kDeps values are
// polled together, and a row stores its value from inside the polling loop as
// soon as its own values are there: a lane that had left its wait would
// otherwise hold its store at the warp's reconvergence point until the slowest
// lane of the warp (a row one level up, or one whose values come from a
// farther SM) arrived, and every level would wait for the slowest warp lane.
// Entries past the first kDeps (none on hex meshes) are waited for one by
// one.  Gives up, raising the abort flag, after about a second (or 2^26
// polls), or when another wait of the sweep did.
constexpr int kDeps = 4;
template <bool DIV>
__device__ __forceinline__ void sweep_store(IluState* st, const Csr& A, const double* __restrict__ lu, int e0,
                                            int e1, const double* v, double s, double piv, double* out) {
    int cj[kDeps];
    double l[kDeps], x[kDeps];
#pragma unroll
    for (int k = 0; k < kDeps; ++k) {
        x[k] = 0.0;  // not pending
        if (e0 + k < e1) {
            cj[k] = __ldg(&A.col[e0 + k]);
            l[k] = __ldg(&lu[e0 + k]);
        }
    }
#pragma unroll
    for (int k = 0; k < kDeps; ++k)
        if (e0 + k < e1) x[k] = ld_relaxed(&v[cj[k]]);
    unsigned long long t0 = 0;
    for (unsigned it = 0; it < (1u << 26); ++it) {
        bool ready = true;
#pragma unroll
        for (int k = 0; k < kDeps; ++k) ready = ready && !pending(x[k]);
        if (ready) {
#pragma unroll
            for (int k = 0; k < kDeps; ++k)
                if (e0 + k < e1) s = fma(-l[k], x[k], s);
            for (int e = e0 + kDeps; e < e1; ++e) {
                double xe;
                if (!await_row(&v[__ldg(&A.col[e])], xe, st)) return;
                s = fma(-__ldg(&lu[e]), xe, s);
            }
            st_relaxed(out, DIV ? s / piv : s);
            return;
        }
        if (it == 0) t0 = now_ns();
        if (it > 2) __nanosleep(it < 16 ? 32 : 256);
#pragma unroll
        for (int k = 0; k < kDeps; ++k)
            if (pending(x[k])) x[k] = ld_relaxed(&v[cj[k]]);
        if ((it & 31) == 31) {
            if (*(volatile const int32_t*)&st->sweep_abort) return;
            if (now_ns() - t0 > 1000000000ull) break;
        }
    }
    atomicExch(&st->sweep_abort, 1);
}

// Chunk of this block (the same in all its threads), or >= nchunks when none is left.
__device__ __forceinline__ unsigned next_chunk(IluState* st) {
    __shared__ unsigned chunk;
    __syncthreads();
    if (threadIdx.x == 0) chunk = atomicAdd(&st->ticket, 1u);
    __syncthreads();
    return chunk;
}

// The last block resets the ticket and ends an aborted solve.
__device__ __forceinline__ void end_sweep(IluState* st) {
    if (arrive_last(&st->counter) && threadIdx.x == 0) {
        st->ticket = 0;
        if (st->sweep_abort) {
            st->status = FVGB_ERR_CUDA;
            st->done = 1;
        }
    }
}

// y_i = r_i - sum_k l_ik y_k, rows in the lower triangle's level order; the
// backward sweep's output z set to kPending on the way
__global__ void __launch_bounds__(kT)
    k_il_fwd(IluState* st, Csr A, const int* __restrict__ rows, unsigned nchunks, const double* __restrict__ lu,
             const double* __restrict__ r, double* y, double* z) {
    if (done_flag(st)) return;
    for (unsigned c = next_chunk(st); c < nchunks; c = next_chunk(st)) {
        const int t = (int)c * kT + threadIdx.x;
        if (t >= A.n) continue;
        const int i = __ldg(&rows[t]);
        z[i] = __longlong_as_double((long long)kPending);
        const int b = __ldg(&A.ro[i]), d = b + __ldg(&A.dof[i]);
        double s = __ldg(&r[i]);
        sweep_store<false>(st, A, lu, b, d, y, s, 1.0, &y[i]);
    }
    end_sweep(st);
}

// z_i = (y_i - sum_j u_ij z_j) / u_ii, rows in the upper triangle's level
// order; y_i set back to kPending once read
__global__ void __launch_bounds__(kT)
    k_il_bwd(IluState* st, Csr A, const int* __restrict__ rows, unsigned nchunks, const double* __restrict__ lu,
             double* y, double* z) {
    if (done_flag(st)) return;
    for (unsigned c = next_chunk(st); c < nchunks; c = next_chunk(st)) {
        const int t = (int)c * kT + threadIdx.x;
        if (t >= A.n) continue;
        const int i = __ldg(&rows[t]);
        const int d = __ldg(&A.ro[i]) + __ldg(&A.dof[i]), end = __ldg(&A.ro[i + 1]);
        double s = __ldcg(&y[i]);
        y[i] = __longlong_as_double((long long)kPending);
        sweep_store<true>(st, A, lu, d + 1, end, z, s, __ldg(&lu[d]), &z[i]);
    }
    end_sweep(st);
}

// The tolerance and the first stopping test from the initial residual norm
__device__ void start(IluState* st, double res) {
    st->res0 = st->res = res;
    double tol = st->rel_tol * (st->bbase >= 0.0 ? st->bbase : res);
    if (st->abs_tol > tol) tol = st->abs_tol;
    st->tol = tol;
    int done = !(res > tol) || res == 0.0;
    if (!isfinite(res)) {
        done = 1;
        st->status = FVGB_ERR_BREAKDOWN;
    } else if (!done && st->max_iter <= 0) {
        done = 1;
        st->status = FVGB_ERR_NOT_CONVERGED;
    }
    st->done = done;
}

// the stopping tests after an iteration's residual norm
__device__ void after_step(IluState* st, double res) {
    st->res = res;
    st->iter += 1;
    if (!isfinite(res)) {
        st->status = FVGB_ERR_BREAKDOWN;
        st->done = 1;
    } else if (!(res > st->tol)) {
        st->done = 1;
    } else if (st->iter >= st->max_iter) {
        st->status = FVGB_ERR_NOT_CONVERGED;
        st->done = 1;
    }
}

// ------------------------------------------------------------ CG
// r = b - A x, |r|
__global__ void __launch_bounds__(kT)
    k_ic_init(IluState* st, Csr A, int R, const double* __restrict__ a, const double* __restrict__ b,
              double* __restrict__ r, double* pa) {
    const double* x = st->x;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= A.n) continue;
        const double ri = __ldg(&b[i]) - csr_row(A, a, x, i);
        r[i] = ri;
        acc = fma(ri, ri, acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) start(st, sqrt(t));
}

// p = z, rz = (r, z)
__global__ void __launch_bounds__(kT)
    k_ic_first(IluState* st, int n, int R, const double* __restrict__ r, const double* __restrict__ z,
               double* __restrict__ p, double* pa) {
    if (done_flag(st)) return;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= n) continue;
        const double zi = z[i];
        p[i] = zi;
        acc = fma(r[i], zi, acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) st->rz = t;
}

// q = A p, alpha = rz / (p, q)
__global__ void __launch_bounds__(kT)
    k_ic_spmv(IluState* st, Csr A, int R, const double* __restrict__ a, const double* __restrict__ p,
              double* __restrict__ q, double* pa) {
    if (done_flag(st)) return;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= A.n) continue;
        const double qi = csr_row(A, a, p, i);
        q[i] = qi;
        acc = fma(__ldg(&p[i]), qi, acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) {
        const double alpha = st->rz / t;
        st->alpha = alpha;
        if (t == 0.0 || !isfinite(alpha)) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        }
    }
}

// x += alpha p, r -= alpha q, |r|, stopping tests
__global__ void __launch_bounds__(kT)
    k_ic_update(IluState* st, int n, int R, const double* __restrict__ p, const double* __restrict__ q,
                double* __restrict__ r, double* pa) {
    if (done_flag(st)) return;
    const double alpha = st->alpha;
    double* x = st->x;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= n) continue;
        x[i] = fma(alpha, __ldg(&p[i]), x[i]);
        const double ri = fma(-alpha, __ldg(&q[i]), r[i]);
        r[i] = ri;
        acc = fma(ri, ri, acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) after_step(st, sqrt(t));
}

// beta = (r, z) / rz
__global__ void __launch_bounds__(kT)
    k_ic_rz(IluState* st, int n, int R, const double* __restrict__ r, const double* __restrict__ z, double* pa) {
    if (done_flag(st)) return;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i < n) acc = fma(__ldg(&r[i]), __ldg(&z[i]), acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) {
        st->beta = t / st->rz;
        st->rz = t;
    }
}

// p = z + beta p
__global__ void __launch_bounds__(kT)
    k_ic_dir(const IluState* st, int n, const double* __restrict__ z, double* __restrict__ p) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) p[i] = fma(st->beta, p[i], __ldg(&z[i]));
}

// ------------------------------------------------------------ BiCGStab
// r = b - A x, rr = r, p = v = 0, rho = (rr, r), |r|; rho_prev = alpha = omega = 1
__global__ void __launch_bounds__(kT)
    k_ib_init(IluState* st, Csr A, int R, const double* __restrict__ a, const double* __restrict__ b,
              double* __restrict__ r, double* __restrict__ rr, double* __restrict__ p, double* __restrict__ v,
              double* pa, double* pb) {
    const double* x = st->x;
    double arho = 0.0, arr = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= A.n) continue;
        const double ri = __ldg(&b[i]) - csr_row(A, a, x, i);
        r[i] = ri;
        rr[i] = ri;
        p[i] = 0.0;
        v[i] = 0.0;
        arho = fma(ri, ri, arho);
        arr = fma(ri, ri, arr);
    }
    double rho, rsq;
    if (tree_dots(st, pa, pb, arho, arr, 2, &rho, &rsq) && threadIdx.x == 0) {
        st->rho = rho;
        st->rho_prev = st->alpha = st->omega = 1.0;
        start(st, sqrt(rsq));
    }
}

// p = r + beta (p - omega v), beta = (rho / rho_prev)(alpha / omega)
__global__ void __launch_bounds__(kT)
    k_ib_p(const IluState* st, int n, const double* __restrict__ r, const double* __restrict__ v,
           double* __restrict__ p) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i >= n) return;
    const double beta = (st->rho / st->rho_prev) * (st->alpha / st->omega);
    p[i] = fma(beta, fma(-st->omega, __ldg(&v[i]), p[i]), __ldg(&r[i]));
}

// v = A y, alpha = rho / (rr, v)
__global__ void __launch_bounds__(kT)
    k_ib_v(IluState* st, Csr A, int R, const double* __restrict__ a, const double* __restrict__ y,
           const double* __restrict__ rr, double* __restrict__ v, double* pa) {
    if (done_flag(st)) return;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= A.n) continue;
        const double vi = csr_row(A, a, y, i);
        v[i] = vi;
        acc = fma(__ldg(&rr[i]), vi, acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) {
        const double alpha = st->rho / t;
        st->alpha = alpha;
        if (t == 0.0 || !isfinite(alpha)) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        }
    }
}

// s = r - alpha v, |s|: converged at the half step (x += alpha y follows in k_ib_half)
__global__ void __launch_bounds__(kT)
    k_ib_s(IluState* st, int n, int R, const double* __restrict__ r, const double* __restrict__ v,
           double* __restrict__ s, double* pa) {
    if (done_flag(st)) return;
    const double alpha = st->alpha;
    double acc = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= n) continue;
        const double si = fma(-alpha, __ldg(&v[i]), __ldg(&r[i]));
        s[i] = si;
        acc = fma(si, si, acc);
    }
    double t, u;
    if (tree_dots(st, pa, nullptr, acc, 0.0, 1, &t, &u) && threadIdx.x == 0) {
        const double sres = sqrt(t);
        if (!isfinite(sres)) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->res = sres;
            st->done = 1;
        } else if (!(sres > st->tol)) {
            st->res = sres;
            st->iter += 1;
            st->half = 1;
            st->done = 1;
        }
    }
}

// the half-step convergence's x += alpha y (runs whatever the done flag)
__global__ void __launch_bounds__(kT) k_ib_half(IluState* st, int n, const double* __restrict__ y) {
    if (!st->half) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    double* x = st->x;
    if (i < n) x[i] = fma(st->alpha, __ldg(&y[i]), x[i]);
}

// t = A z, omega = (t, s) / (t, t)
__global__ void __launch_bounds__(kT)
    k_ib_t(IluState* st, Csr A, int R, const double* __restrict__ a, const double* __restrict__ z,
           const double* __restrict__ s, double* __restrict__ t, double* pa, double* pb) {
    if (done_flag(st)) return;
    double ats = 0.0, att = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= A.n) continue;
        const double ti = csr_row(A, a, z, i);
        t[i] = ti;
        ats = fma(ti, __ldg(&s[i]), ats);
        att = fma(ti, ti, att);
    }
    double ts, tt;
    if (tree_dots(st, pa, pb, ats, att, 2, &ts, &tt) && threadIdx.x == 0) {
        const double omega = ts / tt;
        st->omega = omega;
        if (tt == 0.0 || !isfinite(omega) || omega == 0.0) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        }
    }
}

// x += alpha y + omega z, r = s - omega t, rho = (rr, r), |r|, stopping tests
__global__ void __launch_bounds__(kT)
    k_ib_x(IluState* st, int n, int R, const double* __restrict__ y, const double* __restrict__ z,
           const double* __restrict__ s, const double* __restrict__ t, const double* __restrict__ rr,
           double* __restrict__ r, double* pa, double* pb) {
    if (done_flag(st)) return;
    const double alpha = st->alpha, omega = st->omega;
    double* x = st->x;
    double arho = 0.0, arr = 0.0;
    for (int j = 0; j < R; ++j) {
        const int i = tree_row(R, j);
        if (i >= n) continue;
        x[i] = fma(omega, __ldg(&z[i]), fma(alpha, __ldg(&y[i]), x[i]));
        const double ri = fma(-omega, __ldg(&t[i]), __ldg(&s[i]));
        r[i] = ri;
        arho = fma(__ldg(&rr[i]), ri, arho);
        arr = fma(ri, ri, arr);
    }
    double rho, rsq;
    if (tree_dots(st, pa, pb, arho, arr, 2, &rho, &rsq) && threadIdx.x == 0) {
        st->rho_prev = st->rho;
        st->rho = rho;
        after_step(st, sqrt(rsq));
        if (!st->done && rho == 0.0) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        }
    }
}

__global__ void k_il_cond(const IluState* st, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, st->done ? 0u : 1u);
}

__global__ void k_il_stats(IluState* st) {
    fvgb_solver_stats s{};
    s.init_res_norm = st->res0;
    s.final_res_norm = st->res;
    s.num_iter = st->iter;
    s.num_outer = 0;
    s.status = st->status;
    st->stats = s;
    if (st->stats_out) *st->stats_out = s;
}

}  // namespace

// ------------------------------------------------------------ host side
struct IluCache {
    const fvgb_ls* ls = nullptr;
    int n = 0, nnz = 0, R = 4, nb = 1;
    unsigned sweep_grid = 1;  // resident blocks of a triangular sweep
    int *ro = nullptr, *col = nullptr, *dof = nullptr;
    int *op_ptr = nullptr, *op_f = nullptr, *op_g = nullptr;
    int *fwd_rows = nullptr, *bwd_rows = nullptr;
    std::vector<int> fwd_ptr, bwd_ptr;  // level offsets into fwd_rows / bwd_rows (host)
    double *a = nullptr, *lu = nullptr;
    double *r = nullptr, *rr = nullptr, *p = nullptr, *q = nullptr, *v = nullptr, *y = nullptr, *z = nullptr,
           *s = nullptr, *t = nullptr, *w = nullptr, *pa = nullptr, *pb = nullptr;
    IluState* st = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // CG, BiCGStab
    std::vector<void*> allocs;
};

namespace {

template <class T>
cudaError_t il_alloc(IluCache* c, T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) c->allocs.push_back(*p);
    return e;
}

template <class T>
cudaError_t il_upload(IluCache* c, T** p, const std::vector<T>& h) {
    cudaError_t e = il_alloc(c, p, h.size());
    if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
    return e;
}

// rows grouped by level (stable in row order), level offsets in ptr
void by_level(const std::vector<int>& lev, std::vector<int>& ptr, std::vector<int>& rows) {
    const int nl = lev.empty() ? 0 : 1 + *std::max_element(lev.begin(), lev.end());
    ptr.assign((size_t)nl + 1, 0);
    for (int l : lev) ++ptr[(size_t)l + 1];
    for (int l = 0; l < nl; ++l) ptr[(size_t)l + 1] += ptr[(size_t)l];
    rows.assign(lev.size(), 0);
    std::vector<int> at(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < (int)lev.size(); ++i) rows[(size_t)at[(size_t)lev[(size_t)i]]++] = i;
}

fvgb_status symbolic(IluCache* c) {
    const fvgb_mesh* m = c->ls->mesh;
    const int n = m->v.n, nnz = m->nnz;
    if ((int)m->h_row_offs.size() != n + 1 || (int)m->h_col.size() != nnz || (int)m->h_diag_off.size() != n)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "ILU: the mesh keeps no host sparsity pattern (device-built boxes)");
    const std::vector<int32_t>& ro = m->h_row_offs;
    const std::vector<int32_t>& col = m->h_col;
    const std::vector<int32_t>& dof = m->h_diag_off;
    std::vector<int> op_ptr((size_t)nnz + 1, 0), op_f, op_g, lev_f((size_t)n, 0), lev_b((size_t)n, 0);
    for (int i = 0; i < n; ++i) {
        const int d = ro[i] + dof[i], end = ro[i + 1];
        for (int e = ro[i]; e < end; ++e) {
            if (e < d) {
                const int k = col[e];
                lev_f[i] = std::max(lev_f[i], lev_f[k] + 1);
                int f = e + 1, g = ro[k] + dof[k] + 1;
                while (f < end && g < ro[k + 1]) {  // j > k in rows i and k, ascending
                    if (col[f] < col[g]) ++f;
                    else if (col[f] > col[g]) ++g;
                    else {
                        op_f.push_back(f++);
                        op_g.push_back(g++);
                    }
                }
            }
            op_ptr[(size_t)e + 1] = (int)op_f.size();
        }
    }
    for (int i = n - 1; i >= 0; --i)
        for (int e = ro[i] + dof[i] + 1; e < ro[i + 1]; ++e) lev_b[i] = std::max(lev_b[i], lev_b[col[e]] + 1);
    std::vector<int> fwd_rows, bwd_rows;
    by_level(lev_f, c->fwd_ptr, fwd_rows);
    by_level(lev_b, c->bwd_ptr, bwd_rows);
    c->n = n;
    c->nnz = nnz;
    c->R = n >= (1 << 15) ? 8 : 4;
    c->nb = std::max(1, (n + kT * c->R - 1) / (kT * c->R));
    {
        // the sweep's blocks stay resident (a persistent grid taking chunks);
        // one per SM keeps the rows at the wavefront busy, and more rows in
        // flight only add polls of rows far behind it
        int dev = 0, sms = 1, per = 1;
        FVGB_CUDA_TRY(cudaGetDevice(&dev));
        FVGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FVGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_il_fwd, kT, 0));
        const long chunks = (n + kT - 1) / kT;
        c->sweep_grid = (unsigned)std::max(1L, std::min(chunks, (long)sms * std::min(per, kSweepBlocksPerSM)));
    }
    cudaError_t e = il_upload(c, &c->ro, ro);
    if (e == cudaSuccess) e = il_upload(c, &c->col, col);
    if (e == cudaSuccess) e = il_upload(c, &c->dof, dof);
    if (e == cudaSuccess) e = il_upload(c, &c->op_ptr, op_ptr);
    if (e == cudaSuccess) e = il_upload(c, &c->op_f, op_f);
    if (e == cudaSuccess) e = il_upload(c, &c->op_g, op_g);
    if (e == cudaSuccess) e = il_upload(c, &c->fwd_rows, fwd_rows);
    if (e == cudaSuccess) e = il_upload(c, &c->bwd_rows, bwd_rows);
    if (e == cudaSuccess) e = il_alloc(c, &c->a, (size_t)nnz);
    if (e == cudaSuccess) e = il_alloc(c, &c->lu, (size_t)nnz);
    double** vecs[] = {&c->r, &c->rr, &c->p, &c->q, &c->v, &c->y, &c->z, &c->s, &c->t, &c->w};
    for (double** v : vecs)
        if (e == cudaSuccess) e = il_alloc(c, v, (size_t)n);
    if (e == cudaSuccess) e = il_alloc(c, &c->pa, (size_t)c->nb);
    if (e == cudaSuccess) e = il_alloc(c, &c->pb, (size_t)c->nb);
    if (e == cudaSuccess) e = il_alloc(c, &c->st, 1);
    if (e == cudaSuccess) e = cudaMemset(c->st, 0, sizeof(IluState));
    if (e != cudaSuccess) return cuda_fail(e, "ILU setup");
    FVGB_CUDA_TRY(settle_creation());
    return FVGB_OK;
}

// Graph construction: kernel nodes in a chain.  The arguments are passed by
// value; cudaGraphAddKernelNode copies the values the pointers point to.
struct Chain {
    cudaGraph_t g;
    cudaGraphNode_t prev = nullptr;
    bool has_prev = false;
    cudaError_t e = cudaSuccess;

    template <class... A>
    void add(void* fn, unsigned grid, A... args) {
        if (e != cudaSuccess) return;
        void* params[] = {(void*)&args...};
        cudaKernelNodeParams kp{};
        kp.func = fn;
        kp.gridDim = dim3(grid);
        kp.blockDim = dim3(fn == (void*)k_il_cond || fn == (void*)k_il_stats ? 1 : kT);
        kp.kernelParams = params;
        cudaGraphNode_t node;
        e = cudaGraphAddKernelNode(&node, g, has_prev ? &prev : nullptr, has_prev ? 1 : 0, &kp);
        if (e == cudaSuccess) {
            prev = node;
            has_prev = true;
        }
    }
};

unsigned grid_of(int count) { return count > 0 ? (unsigned)((count + kT - 1) / kT) : 1u; }

// z = U^-1 L^-1 src through c->w: a forward and a backward sweep
void add_apply(IluCache* c, Chain& ch, const double* src, double* dst) {
    const Csr A{c->n, c->ro, c->col, c->dof};
    const unsigned nchunks = (unsigned)((c->n + kT - 1) / kT);
    const double* lu = c->lu;
    ch.add((void*)k_il_fwd, c->sweep_grid, c->st, A, (const int*)c->fwd_rows, nchunks, lu, src, c->w, dst);
    ch.add((void*)k_il_bwd, c->sweep_grid, c->st, A, (const int*)c->bwd_rows, nchunks, lu, c->w, dst);
}

fvgb_status build_graph(IluCache* c, bool bicgstab) {
    cudaGraphExec_t& out = c->graph[bicgstab ? 1 : 0];
    const fvgb_ls* ls = c->ls;
    const Csr A{c->n, c->ro, c->col, c->dof};
    const int n = c->n, R = c->R;
    const unsigned nb = (unsigned)c->nb, ng = grid_of(n);
    IluState* st = c->st;
    const double* a = c->a;
    const double* b = ls->rhs;
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    Chain ch;
    ch.g = g;
    cudaGraphConditionalHandle h{};
    ch.e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    ch.add((void*)k_il_bnorm, nb, st, n, R, b, c->pa);
    ch.add((void*)k_il_pending, ng, n, c->w);  // the forward sweeps' output, pending
    ch.add((void*)k_il_gather, grid_of(c->nnz), c->nnz, (const int*)ls->mesh->csr_pos, (const double*)ls->values,
           c->a, c->lu);
    for (size_t l = 0; l + 1 < c->fwd_ptr.size(); ++l) {
        const int cnt = c->fwd_ptr[l + 1] - c->fwd_ptr[l];
        ch.add((void*)k_il_factor, grid_of(cnt), A, (const int*)(c->fwd_rows + c->fwd_ptr[l]), cnt,
               (const int*)c->op_ptr, (const int*)c->op_f, (const int*)c->op_g, c->lu);
    }
    if (!bicgstab) {
        ch.add((void*)k_ic_init, nb, st, A, R, a, b, c->r, c->pa);
        add_apply(c, ch, c->r, c->z);
        ch.add((void*)k_ic_first, nb, st, n, R, (const double*)c->r, (const double*)c->z, c->p, c->pa);
    } else {
        ch.add((void*)k_ib_init, nb, st, A, R, a, b, c->r, c->rr, c->p, c->v, c->pa, c->pb);
    }
    ch.add((void*)k_il_cond, 1, (const IluState*)st, h);
    cudaGraph_t body = nullptr;
    if (ch.e == cudaSuccess) {
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        ch.e = cudaGraphAddNode(&node, g, &ch.prev, nullptr, 1, &np);
        if (ch.e == cudaSuccess) {
            body = np.conditional.phGraph_out[0];
            ch.prev = node;
        }
    }
    Chain bc;
    bc.g = body;
    if (ch.e == cudaSuccess) {
        if (!bicgstab) {
            bc.add((void*)k_ic_spmv, nb, st, A, R, a, (const double*)c->p, c->q, c->pa);
            bc.add((void*)k_ic_update, nb, st, n, R, (const double*)c->p, (const double*)c->q, c->r, c->pa);
            add_apply(c, bc, c->r, c->z);
            bc.add((void*)k_ic_rz, nb, st, n, R, (const double*)c->r, (const double*)c->z, c->pa);
            bc.add((void*)k_ic_dir, ng, (const IluState*)st, n, (const double*)c->z, c->p);
        } else {
            bc.add((void*)k_ib_p, ng, (const IluState*)st, n, (const double*)c->r, (const double*)c->v, c->p);
            add_apply(c, bc, c->p, c->y);
            bc.add((void*)k_ib_v, nb, st, A, R, a, (const double*)c->y, (const double*)c->rr, c->v, c->pa);
            bc.add((void*)k_ib_s, nb, st, n, R, (const double*)c->r, (const double*)c->v, c->s, c->pa);
            bc.add((void*)k_ib_half, ng, st, n, (const double*)c->y);
            add_apply(c, bc, c->s, c->z);
            bc.add((void*)k_ib_t, nb, st, A, R, a, (const double*)c->z, (const double*)c->s, c->t, c->pa, c->pb);
            bc.add((void*)k_ib_x, nb, st, n, R, (const double*)c->y, (const double*)c->z, (const double*)c->s,
                   (const double*)c->t, (const double*)c->rr, c->r, c->pa, c->pb);
        }
        bc.add((void*)k_il_cond, 1, (const IluState*)st, h);
        ch.e = bc.e;
    }
    ch.add((void*)k_il_stats, 1, st);
    cudaError_t e = ch.e;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        out = nullptr;
        return cuda_fail(e, "ILU solve graph");
    }
    return FVGB_OK;
}

}  // namespace

void fvgb_ilu_free(IluCache* c) {
    if (!c) return;
    for (cudaGraphExec_t g : c->graph)
        if (g) cudaGraphExecDestroy(g);
    for (void* p : c->allocs) cudaFree(p);
    delete c;
}

fvgb_status fvgb_ilu_solve_async(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats_dev,
                                 cudaStream_t s) {
    if (ls->ncomp != 1) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_solve: scalar systems only");
    if (cfg->method != FVGB_SOLVER_CG && cfg->method != FVGB_SOLVER_BICGSTAB)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "ILU: the preconditioner of CG and BiCGStab only");
    if (cfg->precision != FVGB_PREC_FP64)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "ILU: FP64 only (no mixed-precision ILU solve)");
    FVGB_CHECK_ARG(cfg->rel_tol >= 0 && cfg->abs_tol >= 0, "fvgb_solve: negative tolerance");
    FVGB_CHECK_ARG(cfg->max_iter >= 0 && cfg->max_iter <= 100000000, "fvgb_solve: bad max_iter");
    FVGB_CHECK_ARG((cfg->flags & ~(FVGB_SOLVE_NO_TUNE | FVGB_SOLVE_RHS_BASELINE)) == 0, "fvgb_solve: unknown flags");
    const bool bicgstab = cfg->method == FVGB_SOLVER_BICGSTAB;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FVGB_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (!ls->ilu || !ls->ilu->graph[bicgstab ? 1 : 0]) {
        // setup allocates, uploads synchronously and builds a graph
        if (cs != cudaStreamCaptureStatusNone)
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "ILU: the first solve (setup) cannot be stream-captured");
        if (!ls->ilu) {
            IluCache* c = new IluCache();
            c->ls = ls;
            fvgb_status st = symbolic(c);
            if (st != FVGB_OK) {
                fvgb_ilu_free(c);
                return st;
            }
            ls->ilu = c;
        }
        fvgb_status st = build_graph(ls->ilu, bicgstab);
        if (st != FVGB_OK) return st;
    }
    IluCache* c = ls->ilu;
    k_il_params<<<1, 1, 0, s>>>(c->st, x, cfg->rel_tol, cfg->abs_tol, cfg->max_iter, stats_dev,
                                (cfg->flags & FVGB_SOLVE_RHS_BASELINE) ? 1 : 0);
    FVGB_LAUNCH_CHECK("ILU params");
    FVGB_CUDA_TRY(cudaGraphLaunch(c->graph[bicgstab ? 1 : 0], s));
    return FVGB_OK;
}

fvgb_status fvgb_ilu_sync_stats(fvgb_ls* ls, fvgb_solver_stats* out, cudaStream_t s) {
    fvgb_solver_stats h{};
    FVGB_CUDA_TRY(cudaMemcpyAsync(&h, &ls->ilu->st->stats, sizeof h, cudaMemcpyDeviceToHost, s));
    FVGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (out) *out = h;
    return (fvgb_status)h.status;
}
