// Krylov solves of assembled systems, entirely on the device, for one case or
// a batch of independent cases packed into one system.
//
// FP64: Jacobi-preconditioned CG, the algorithm of Ginkgo solver::Cg with
// preconditioner::Jacobi (max_block_size 1) that FoamAdapter maps OpenFOAM's
// PCG/DIC to (src/compatibility/fvSolution.cpp:19-104), with its stopping
// criteria (fvSolution.cpp:106-142).  MIXED_IR: CG on the Jacobi-scaled system
// in FP32 with reliable updates: whenever the FP32 residual has dropped by
// inner_rel_tol (or should be below the tolerance), x is updated in FP64, the
// true residual b - A x is recomputed in FP64 and tested for convergence, and
// it replaces the FP32 residual while the search direction is kept (not
// restarted), so the iteration count stays close to the FP64 solver's.
//
// Batches.  A system may hold several independent cases (a block-diagonal
// matrix); case c owns rows [begin_c, end_c).  Every kernel is ONE launch
// over all cases: a block map assigns each 256-thread block to one case and
// 256*R consecutive rows of it, every case keeps its own CG scalars, and
// converged cases idle.  A single solve is a batch of one case.
//
// Each solve is one CUDA graph: an init kernel, a device-side WHILE
// conditional node whose body holds one iteration (three kernels), and a
// finish kernel; the mixed solve nests the inner CG loop inside the refinement
// loop.  The last block to finish an iteration's kernel sets the loop
// condition (any case still active), so there is no host round trip per
// iteration.  Every loop is bounded by an iteration cap.
//
// Reductions are deterministic.  Block b of case c owns rows
// row0_b + (t/32)*32R + j*32 + t%32 (thread t, j < R = rows_per_thread(case rows)); a
// thread sums its rows sequentially, warp 0 sums the 256 partials (lane l:
// l, l+32, ..., l+224) and a xor butterfly finishes; the last block of the case
// to arrive sums the case's block partials in index order with the same tree.
// The CPU oracle reproduces this tree, so the FP64 iterates match it bit for
// bit, and a case solved in a batch gives exactly the bits it gives alone.
#include <cmath>
#include <vector>

#include "internal.cuh"
#include "tunecache.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>

namespace {

constexpr int kT = 256;
constexpr int kRowsPerThread = 8;  // the most rows per thread of any case

// Rows per thread of a case's reduction tree: 8 (2048-row blocks, half the
// block reductions) for cases of at least kBigCaseRows rows; 4 for smaller
// cases, whose single solves run the persistent kernel and need the blocks
// to fill the GPU.  A function of the case's own size, so a case solved in a
// batch keeps the tree it has alone.  Measured on 512 cases of 4 k-262 k rows:
// a threshold of 2^15 rows keeps 97% of the packed throughput of 8 rows
// everywhere (7,797 against 8,006 case-steps/s) and speeds single small
// solves up 8%; 2^18 speeds them up 27% but costs 13% packed.
constexpr int kBigCaseRows = 1 << 15;
__host__ __device__ inline int rows_per_thread(int64_t case_rows) { return case_rows >= kBigCaseRows ? 8 : 4; }

struct SolverParams {
    double* x;
    fvgb_solver_stats* stats_out;  // device pointer [ncases] or null
    double rel_tol, abs_tol, inner_rel_tol;
    int32_t max_iter, inner_max_iter, max_outer;
    int32_t convert;  // mixed: form the FP32 matrix (0: the copy of an unchanged matrix is still valid)
};

struct CaseState {
    double rz, alpha, beta, res0, res, tol;
    double rho, rho_prev, itol;
    double sres, sig, isig;     // mixed: |s r| of the latest residual; power-of-two scale of rhat and 1/scale
    double omega;               // BiCGStab
    float falpha, fbeta, frel;  // frel: direction factor after a reliable update (-1: restart)
    float fomega;               // mixed BiCGStab
    int32_t iter, status, total, outer, inner_it;
    int32_t active;        // FP64: iterating; mixed: refinement loop running
    int32_t inner_active;  // mixed: inner CG running
    unsigned int counter;  // arrivals of this case's blocks
    unsigned int signflags;
    int32_t half;          // BiCGStab: converged at the half step, x update pending
    double bbase;          // ||b|| when the relative tolerance refers to it (-1: to the initial residual)
};

struct BatchState {
    SolverParams prm;
    int32_t ncases, n_active, n_inner, pad;
    unsigned int gcounter;
};

// Block map and per-case data, passed to every kernel by value.
struct Layout {
    const int32_t* blk_case;   // [nb]
    const int32_t* blk_row0;   // [nb]
    const int32_t* case_end;   // [ncases]
    const int32_t* case_blk0;  // [ncases+1]
    CaseState* cases;
    BatchState* bs;
    fvgb_solver_stats* stats;  // [ncases] internal copy for the synchronous API
    const int32_t* case_rpt;   // [ncases] rows per thread of every case's tree
};

struct Blk {
    int c, row0, end, nbc, blk0, R;
};

__device__ __forceinline__ Blk blk_info(const Layout& L) {
    Blk k;
    k.c = __ldg(&L.blk_case[blockIdx.x]);
    k.row0 = __ldg(&L.blk_row0[blockIdx.x]);
    k.end = __ldg(&L.case_end[k.c]);
    k.blk0 = __ldg(&L.case_blk0[k.c]);
    k.nbc = __ldg(&L.case_blk0[k.c + 1]) - k.blk0;
    k.R = __ldg(&L.case_rpt[k.c]);
    return k;
}

// Row j of this thread in its block; past the case's end (skipped by every
// caller's `i >= k.end` test) when j is beyond the case's rows per thread.
__device__ __forceinline__ int blk_row(const Blk& k, int j) {
    return j < k.R ? k.row0 + (threadIdx.x >> 5) * (32 * k.R) + j * 32 + (threadIdx.x & 31) : INT_MAX;
}

// Block sum of one value per thread; result valid in warp 0 (every lane).
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

// FP32 block sum (inner solve of the mixed scheme: keeps the FP64 pipe free).
__device__ __forceinline__ float block_tree_f(float v, float* sm) {
    sm[threadIdx.x] = v;
    __syncthreads();
    float s = 0.0f;
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

// Thread 0 has written this block's partials; true in the block that arrives
// last among `count` blocks sharing `counter` (which wraps back to 0).  The
// leading barrier keeps a second call in the same kernel from overwriting the
// flag before every thread has read the first result.
__device__ __forceinline__ bool arrive_last(unsigned int* counter, unsigned int count) {
    __shared__ bool am_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicInc(counter, count - 1);
        am_last = (t == count - 1);
    }
    __syncthreads();
    return am_last;
}

__device__ __forceinline__ int ld_volatile(const int32_t* p) { return *(const volatile int32_t*)p; }

// Columns of a row's first 8 slots (the row itself past its width), the
// offset or column array chosen once per row so the index loads are issued
// together.
__device__ __forceinline__ void slot_cols(const MeshView& m, int base, int w, int i, int* col) {
    if (m.m_off) {
#pragma unroll
        for (int k = 0; k < 8; ++k) col[k] = k < w ? i + (int)__ldg(&m.m_off[base + k * 32]) : i;
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) col[k] = k < w ? __ldg(&m.m_col[base + k * 32]) : i;
    }
}

// s = sum of v[k] x[k], k < W, as an fma chain from +0 in k order
template <int W>
__device__ __forceinline__ double fma_chain(const double* v, const double* x) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < W; ++k) s = fma(v[k], x[k], s);
    return s;
}

// Row sum of a sliced-ELL row, fma chain in slot (= column) order.  The slot
// loads of the first 8 slots are issued before the dependent gathers.
// The row of a W-slot slice: every slot real or padding (value 0, column =
// row), exactly W fmas from +0.
template <int W>
__device__ __forceinline__ double spmv_row_w(const MeshView& m, const double* __restrict__ val,
                                             const double* __restrict__ x, int base, int i) {
    int col[W];
    if (m.m_off) {
#pragma unroll
        for (int k = 0; k < W; ++k) col[k] = i + (int)__ldg(&m.m_off[base + k * 32]);
    } else {
#pragma unroll
        for (int k = 0; k < W; ++k) col[k] = __ldg(&m.m_col[base + k * 32]);
    }
    double v[W], xv[W];
#pragma unroll
    for (int k = 0; k < W; ++k) {
        v[k] = __ldg(&val[base + k * 32]);
        xv[k] = __ldg(&x[col[k]]);
    }
    return fma_chain<W>(v, xv);
}

__device__ __forceinline__ double spmv_row(const MeshView& m, const double* __restrict__ val,
                                           const double* __restrict__ x, int i) {
    const int slice = i >> 5, lane = i & 31;
    const int b0 = __ldg(&m.m_ptr[slice]);
    const int base = b0 + lane;
    const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
    // A chain predicated on k < w over 8 slots is compiled as 8 unconditional
    // fmas (fma(0, 0, s) == s for the chain's s, which is never -0): one wasted
    // DFMA per row of a 7-slot stencil (3-D hex meshes).  Slices of width 7
    // take an exact 7-fma path (w is the same for the whole slice, so the
    // branch is uniform); the bits are the same either way.
    if (w == 7) return spmv_row_w<7>(m, val, x, base, i);
    int col[8];
    slot_cols(m, base, w, i, col);
    double v[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = 0.0;
        xv[k] = 0.0;
        if (k < w) {
            v[k] = __ldg(&val[base + k * 32]);
            xv[k] = __ldg(&x[col[k]]);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) s = fma(v[k], xv[k], s);
    for (int k = 8; k < w; ++k) s = fma(__ldg(&val[base + k * 32]), __ldg(&x[slot_col(m, base + k * 32, i)]), s);
    return s;
}

// FP32 row of the difference-form SpMV: e_i x_i + sum_k a_k (x_{col_k} - x_i),
// fmaf chain in slot order (the diagonal and padding slots hold 0 and add 0).
__device__ __forceinline__ float spmv_row_diff(const MeshView& m, const float* __restrict__ a,
                                               const float* __restrict__ x, int i, float xi, float ei) {
    const int slice = i >> 5, lane = i & 31;
    const int b0 = __ldg(&m.m_ptr[slice]);
    const int base = b0 + lane;
    const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
    int col[8];
    slot_cols(m, base, w, i, col);
    float v[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = 0.0f;
        xv[k] = 0.0f;
        if (k < w) {
            v[k] = __ldg(&a[base + k * 32]);
            xv[k] = __ldg(&x[col[k]]);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) s = fmaf(v[k], xv[k] - xi, s);
    for (int k = 8; k < w; ++k) s = fmaf(__ldg(&a[base + k * 32]), __ldg(&x[slot_col(m, base + k * 32, i)]) - xi, s);
    return fmaf(ei, xi, s);
}

// The baseline of the relative tolerance: ||b|| (Ginkgo's ResidualNorm with its
// default baseline, rhs_norm) when k_case_bnorm has set it, else the initial
// residual norm.
__device__ __forceinline__ double tol_base(const CaseState* cs, double res0) {
    const double b = *(const volatile double*)&cs->bbase;
    return b >= 0.0 ? b : res0;
}

__device__ __forceinline__ void case_done(BatchState* bs, CaseState* cs) {
    cs->active = 0;
    atomicSub(&bs->n_active, 1);
}

// ------------------------------------------------------------------ FP64 PCG
__global__ void __launch_bounds__(kT)
    k_pcg_init(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
               double* __restrict__ dinv, double* __restrict__ r, double* __restrict__ p,
               double* __restrict__ pa, double* __restrict__ pb, cudaGraphConditionalHandle h, int setc) {
    __shared__ double sma[kT], smb[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    const double* __restrict__ x = L.bs->prm.x;
    double arz = 0.0, arr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double di = 1.0 / __ldg(&val[__ldg(&m.diag_pos[i])]);
        dinv[i] = di;
        const double ri = __ldg(&b[i]) - spmv_row(m, val, x, i);
        const double zi = di * ri;
        r[i] = ri;
        p[i] = zi;
        arz = fma(ri, zi, arz);
        arr = fma(ri, ri, arr);
    }
    const double ba = block_tree(arz, sma), bb = block_tree(arr, smb);
    if (threadIdx.x == 0) {
        pa[blockIdx.x] = ba;
        pb[blockIdx.x] = bb;
    }
    if (arrive_last(&cs->counter, k.nbc)) {
        const double rz = final_tree(pa + k.blk0, k.nbc, sma), rr = final_tree(pb + k.blk0, k.nbc, smb);
        if (threadIdx.x == 0) {
            const SolverParams& prm = L.bs->prm;
            const double res0 = sqrt(rr);
            double tol = prm.rel_tol * tol_base(cs, res0);
            if (prm.abs_tol > tol) tol = prm.abs_tol;
            cs->rz = rz;
            cs->res0 = res0;
            cs->res = res0;
            cs->tol = tol;
            bool done = !(res0 > tol) || res0 == 0.0;
            if (!isfinite(res0)) {  // NaN or inf in b or x: not "converged"
                done = true;
                cs->status = FVGB_ERR_BREAKDOWN;
            } else if (!done && prm.max_iter <= 0) {
                done = true;
                cs->status = FVGB_ERR_NOT_CONVERGED;
            }
            if (done) case_done(L.bs, cs);
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0 && setc)
        cudaGraphSetConditional(h, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
}

template <int MINB>
__global__ void __launch_bounds__(kT, MINB)
    k_pcg_spmv(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ p,
               double* __restrict__ q, double* __restrict__ pa) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    __shared__ double sma[kT];
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double qi = spmv_row(m, val, p, i);
        q[i] = qi;
        acc = fma(__ldg(&p[i]), qi, acc);
    }
    const double ba = block_tree(acc, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double pq = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        const double alpha = cs->rz / pq;
        cs->alpha = alpha;
        if (pq == 0.0 || !isfinite(alpha)) {
            cs->status = FVGB_ERR_BREAKDOWN;
            case_done(L.bs, cs);
        }
    }
}

template <int MINB>
__global__ void __launch_bounds__(kT, MINB)
    k_pcg_update(Layout L, const double* __restrict__ dinv, const double* __restrict__ p,
                 const double* __restrict__ q, double* __restrict__ r, double* __restrict__ z,
                 double* __restrict__ pa, double* __restrict__ pb, cudaGraphConditionalHandle h, int setc) {
    __shared__ double sma[kT], smb[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (ld_volatile(&cs->active)) {
        double* __restrict__ x = L.bs->prm.x;
        const double alpha = cs->alpha;
        double arz = 0.0, arr = 0.0;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            x[i] = fma(alpha, __ldg(&p[i]), x[i]);
            const double ri = fma(-alpha, __ldg(&q[i]), r[i]);
            r[i] = ri;
            const double zi = __ldg(&dinv[i]) * ri;
            z[i] = zi;
            arz = fma(ri, zi, arz);
            arr = fma(ri, ri, arr);
        }
        const double ba = block_tree(arz, sma), bb = block_tree(arr, smb);
        if (threadIdx.x == 0) {
            pa[blockIdx.x] = ba;
            pb[blockIdx.x] = bb;
        }
        if (arrive_last(&cs->counter, k.nbc)) {
            const double rzn = final_tree(pa + k.blk0, k.nbc, sma), rr = final_tree(pb + k.blk0, k.nbc, smb);
            if (threadIdx.x == 0) {
                const double res = sqrt(rr);
                cs->res = res;
                cs->iter += 1;
                cs->beta = rzn / cs->rz;
                cs->rz = rzn;
                bool done = false;
                if (!isfinite(res)) {
                    cs->status = FVGB_ERR_BREAKDOWN;
                    done = true;
                } else if (!(res > cs->tol)) {
                    done = true;
                } else if (cs->iter >= L.bs->prm.max_iter) {
                    cs->status = FVGB_ERR_NOT_CONVERGED;
                    done = true;
                }
                if (done) case_done(L.bs, cs);
            }
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0 && setc)
        cudaGraphSetConditional(h, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
}

__global__ void __launch_bounds__(kT)
    k_pcg_dir(Layout L, const double* __restrict__ z, double* __restrict__ p) {
    const Blk k = blk_info(L);
    const CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    const double beta = cs->beta;
    double pv[kRowsPerThread], zv[kRowsPerThread];
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {  // every load first
        const int i = blk_row(k, j);
        pv[j] = zv[j] = 0.0;
        if (i >= k.end) continue;
        pv[j] = p[i];
        zv[j] = __ldg(&z[i]);  // z = dinv*r, stored by the update
    }
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        p[i] = fma(beta, pv[j], zv[j]);
    }
}

__global__ void k_finish(Layout L) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= L.bs->ncases) return;
    const CaseState* cs = &L.cases[c];
    fvgb_solver_stats s;
    s.init_res_norm = cs->res0;
    s.final_res_norm = cs->res;
    s.num_iter = cs->iter + cs->total;  // FP64 counts iter, mixed counts total (the other is 0)
    s.num_outer = cs->outer;
    s.status = cs->status;
    s.reserved = 0;
    L.stats[c] = s;
    if (L.bs->prm.stats_out) L.bs->prm.stats_out[c] = s;
}

__global__ void k_set_params(Layout L, int ncases, SolverParams prm) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c == 0) {
        L.bs->prm = prm;
        L.bs->ncases = ncases;
        L.bs->n_active = ncases;
        L.bs->n_inner = 0;
        L.bs->gcounter = 0u;
    }
    if (c < ncases) {
        CaseState* cs = &L.cases[c];
        cs->iter = 0;
        cs->total = 0;
        cs->outer = 0;
        cs->inner_it = 0;
        cs->status = FVGB_OK;
        cs->active = 1;
        cs->inner_active = 0;
        cs->res0 = 0.0;
        cs->res = 0.0;
        cs->signflags = 0u;
        cs->counter = 0u;
        cs->bbase = -1.0;
    }
}

// ||b|| of every case, with the reduction tree of the solver's dot products
// (FVGB_SOLVE_RHS_BASELINE); runs after k_set_params, before the solve.
__global__ void __launch_bounds__(kT) k_case_bnorm(Layout L, const double* __restrict__ b, double* __restrict__ pa) {
    __shared__ double sma[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double bi = __ldg(&b[i]);
        acc = fma(bi, bi, acc);
    }
    const double ba = block_tree(acc, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (arrive_last(&cs->counter, k.nbc)) {
        const double bb = final_tree(pa + k.blk0, k.nbc, sma);
        if (threadIdx.x == 0) cs->bbase = sqrt(bb);
    }
}

// ------------------------------------------------------------- BiCGStab (FP64)
// Jacobi-preconditioned BiCGStab with right preconditioning, Ginkgo's
// solver::Bicgstab as FoamAdapter selects it (fvSolution.cpp:25-26, 106-142),
// for nonsymmetric systems (implicit convection).  One iteration, five kernels:
//   k_bi_dir:    p = r + beta (p - omega v), y = D^-1 p
//   k_bi_spmv1:  v = A y, alpha = rho / (rr, v)
//   k_bi_s:      s = r - alpha v, z = D^-1 s, |s| (converged: half step)
//   k_bi_spmv2:  half step: x += alpha y, done; else t = A z, omega = (t,s)/(t,t)
//   k_bi_update: x += alpha y + omega z, r = s - omega t, rho = (rr, r), |r|
// rr is the shadow residual (the initial r).  Scalars are formed by the last
// block of each case, every dot product by the same tree as the CG kernels.
__global__ void __launch_bounds__(kT)
    k_bi_init(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
              double* __restrict__ dinv, double* __restrict__ r, double* __restrict__ rr, double* __restrict__ p,
              double* __restrict__ v, double* __restrict__ pa, cudaGraphConditionalHandle h) {
    __shared__ double sma[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    const double* __restrict__ x = L.bs->prm.x;
    double arr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        dinv[i] = 1.0 / __ldg(&val[__ldg(&m.diag_pos[i])]);
        const double ri = __ldg(&b[i]) - spmv_row(m, val, x, i);
        r[i] = ri;
        rr[i] = ri;
        p[i] = 0.0;
        v[i] = 0.0;
        arr = fma(ri, ri, arr);
    }
    const double ba = block_tree(arr, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (arrive_last(&cs->counter, k.nbc)) {
        const double rr2 = final_tree(pa + k.blk0, k.nbc, sma);
        if (threadIdx.x == 0) {
            const SolverParams& prm = L.bs->prm;
            const double res0 = sqrt(rr2);
            double tol = prm.rel_tol * tol_base(cs, res0);
            if (prm.abs_tol > tol) tol = prm.abs_tol;
            cs->res0 = cs->res = res0;
            cs->tol = tol;
            cs->rho = rr2;  // (rr, r) with rr = r
            cs->rho_prev = 1.0;
            cs->alpha = 1.0;
            cs->omega = 1.0;
            cs->beta = rr2;  // (rho / 1) (1 / 1)
            cs->half = 0;
            bool done = !(res0 > tol) || res0 == 0.0;
            if (!isfinite(res0)) {
                done = true;
                cs->status = FVGB_ERR_BREAKDOWN;
            } else if (!done && prm.max_iter <= 0) {
                done = true;
                cs->status = FVGB_ERR_NOT_CONVERGED;
            }
            if (done) case_done(L.bs, cs);
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0)
        cudaGraphSetConditional(h, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
}

__global__ void __launch_bounds__(kT)
    k_bi_dir(Layout L, const double* __restrict__ dinv, const double* __restrict__ r, const double* __restrict__ v,
             double* __restrict__ p, double* __restrict__ y) {
    const Blk k = blk_info(L);
    const CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    const double beta = cs->beta, omega = cs->omega;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double pi = fma(beta, fma(-omega, __ldg(&v[i]), p[i]), __ldg(&r[i]));
        p[i] = pi;
        y[i] = __ldg(&dinv[i]) * pi;
    }
}

__global__ void __launch_bounds__(kT)
    k_bi_spmv1(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ y,
               const double* __restrict__ rr, double* __restrict__ v, double* __restrict__ pa) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    __shared__ double sma[kT];
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double vi = spmv_row(m, val, y, i);
        v[i] = vi;
        acc = fma(__ldg(&rr[i]), vi, acc);
    }
    const double ba = block_tree(acc, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double rv = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        const double alpha = cs->rho / rv;
        cs->alpha = alpha;
        if (rv == 0.0 || !isfinite(alpha)) {
            cs->status = FVGB_ERR_BREAKDOWN;
            case_done(L.bs, cs);
        }
    }
}

__global__ void __launch_bounds__(kT)
    k_bi_s(Layout L, const double* __restrict__ dinv, const double* __restrict__ r, const double* __restrict__ v,
           double* __restrict__ sv, double* __restrict__ z, double* __restrict__ pa) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    __shared__ double sma[kT];
    const double alpha = cs->alpha;
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double si = fma(-alpha, __ldg(&v[i]), __ldg(&r[i]));
        sv[i] = si;
        z[i] = __ldg(&dinv[i]) * si;
        acc = fma(si, si, acc);
    }
    const double ba = block_tree(acc, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double ss = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        const double sres = sqrt(ss);
        if (!isfinite(sres)) {
            cs->res = sres;
            cs->status = FVGB_ERR_BREAKDOWN;
            case_done(L.bs, cs);
        } else if (!(sres > cs->tol)) {
            cs->res = sres;
            cs->half = 1;
        }
    }
}

__global__ void __launch_bounds__(kT)
    k_bi_spmv2(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ z,
               const double* __restrict__ sv, const double* __restrict__ y, double* __restrict__ t,
               double* __restrict__ pa, double* __restrict__ pb) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    __shared__ double sma[kT], smb[kT];
    if (ld_volatile(&cs->half)) {  // converged at the half step: x += alpha y, done
        double* __restrict__ x = L.bs->prm.x;
        const double alpha = cs->alpha;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            x[i] = fma(alpha, __ldg(&y[i]), x[i]);
        }
        if (arrive_last(&cs->counter, k.nbc) && threadIdx.x == 0) {
            cs->iter += 1;
            case_done(L.bs, cs);
        }
        return;
    }
    double ats = 0.0, att = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double ti = spmv_row(m, val, z, i);
        t[i] = ti;
        ats = fma(ti, __ldg(&sv[i]), ats);
        att = fma(ti, ti, att);
    }
    const double ba = block_tree(ats, sma), bb = block_tree(att, smb);
    if (threadIdx.x == 0) {
        pa[blockIdx.x] = ba;
        pb[blockIdx.x] = bb;
    }
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double ts = final_tree(pa + k.blk0, k.nbc, sma), tt = final_tree(pb + k.blk0, k.nbc, smb);
    if (threadIdx.x == 0) {
        const double omega = ts / tt;
        cs->omega = omega;
        if (tt == 0.0 || !isfinite(omega) || omega == 0.0) {
            cs->status = FVGB_ERR_BREAKDOWN;
            case_done(L.bs, cs);
        }
    }
}

__global__ void __launch_bounds__(kT)
    k_bi_update(Layout L, const double* __restrict__ y, const double* __restrict__ z, const double* __restrict__ sv,
                const double* __restrict__ t, const double* __restrict__ rr, double* __restrict__ r,
                double* __restrict__ pa, double* __restrict__ pb, cudaGraphConditionalHandle h) {
    __shared__ double sma[kT], smb[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (ld_volatile(&cs->active)) {
        double* __restrict__ x = L.bs->prm.x;
        const double alpha = cs->alpha, omega = cs->omega;
        double arho = 0.0, arr = 0.0;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            x[i] = fma(omega, __ldg(&z[i]), fma(alpha, __ldg(&y[i]), x[i]));
            const double ri = fma(-omega, __ldg(&t[i]), __ldg(&sv[i]));
            r[i] = ri;
            arho = fma(__ldg(&rr[i]), ri, arho);
            arr = fma(ri, ri, arr);
        }
        const double ba = block_tree(arho, sma), bb = block_tree(arr, smb);
        if (threadIdx.x == 0) {
            pa[blockIdx.x] = ba;
            pb[blockIdx.x] = bb;
        }
        if (arrive_last(&cs->counter, k.nbc)) {
            const double rho = final_tree(pa + k.blk0, k.nbc, sma), rr2 = final_tree(pb + k.blk0, k.nbc, smb);
            if (threadIdx.x == 0) {
                const double res = sqrt(rr2);
                cs->res = res;
                cs->iter += 1;
                cs->rho_prev = cs->rho;
                cs->rho = rho;
                cs->beta = (rho / cs->rho_prev) * (alpha / omega);
                bool done = false;
                if (!isfinite(res)) {
                    cs->status = FVGB_ERR_BREAKDOWN;
                    done = true;
                } else if (!(res > cs->tol)) {
                    done = true;
                } else if (cs->iter >= L.bs->prm.max_iter) {
                    cs->status = FVGB_ERR_NOT_CONVERGED;
                    done = true;
                } else if (rho == 0.0) {
                    cs->status = FVGB_ERR_BREAKDOWN;
                    done = true;
                }
                if (done) case_done(L.bs, cs);
            }
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0)
        cudaGraphSetConditional(h, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
}

// ------------------------------------------------------------------ BiCG (FP64)
// Jacobi-preconditioned BiCG, the method of Ginkgo's solver::Bicg that
// FoamAdapter maps OpenFOAM's PBiCG to (fvSolution.cpp:24), for nonsymmetric
// systems.  The shadow system is the transpose: r~ starts as r, and its
// direction is multiplied by A^T.  Jacobi is its own transpose.
//   init:    r = b - A x, r~ = r, z = D^-1 r, z~ = D^-1 r~, p = p~ = 0,
//            rho = (r~, z), beta = rho / 1
//   dir:     p = z + beta p, p~ = z~ + beta p~
//   spmv:    q = A p, q~ = A^T p~, alpha = rho / (p~, q)
//   update:  x += alpha p, r -= alpha q, r~ -= alpha q~, z = D^-1 r,
//            z~ = D^-1 r~, rho' = (r~, z), |r|, beta = rho' / rho
// A^T p~ is a gather over the matrix slots: the value of (A^T)_ij is the slot
// of a_ji, which the face code of slot (i, j) names (own_pos / nei_pos).  The
// fma chain of a row runs in slot (= column) order as in A p.

// (A^T x)_i in slot order
__device__ __forceinline__ double spmv_row_t(const MeshView& m, const double* __restrict__ val,
                                             const double* __restrict__ x, int i) {
    const int slice = i >> 5, lane = i & 31;
    const int b0 = __ldg(&m.m_ptr[slice]);
    const int base = b0 + lane;
    const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
    double s = 0.0;
    for (int k = 0; k < w; ++k) {
        const int pos = base + k * 32;
        const int code = __ldg(&m.m_code[pos]);
        if (code == FVGB_PAD) continue;
        const int tpos = code >= 0 ? __ldg(&m.nei_pos[code]) : (code == -1 ? pos : __ldg(&m.own_pos[-code - 2]));
        s = fma(__ldg(&val[tpos]), __ldg(&x[slot_col(m, pos, i)]), s);
    }
    return s;
}

__global__ void __launch_bounds__(kT)
    k_bg_init(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
              double* __restrict__ dinv, double* __restrict__ r, double* __restrict__ r2, double* __restrict__ z,
              double* __restrict__ z2, double* __restrict__ p, double* __restrict__ p2, double* __restrict__ pa,
              double* __restrict__ pb, cudaGraphConditionalHandle h) {
    __shared__ double sma[kT], smb[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    const double* __restrict__ x = L.bs->prm.x;
    double arho = 0.0, arr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double di = 1.0 / __ldg(&val[__ldg(&m.diag_pos[i])]);
        dinv[i] = di;
        const double ri = __ldg(&b[i]) - spmv_row(m, val, x, i);
        const double zi = di * ri;
        r[i] = ri;
        r2[i] = ri;
        z[i] = zi;
        z2[i] = zi;
        p[i] = 0.0;
        p2[i] = 0.0;
        arho = fma(ri, zi, arho);
        arr = fma(ri, ri, arr);
    }
    const double ba = block_tree(arho, sma), bb = block_tree(arr, smb);
    if (threadIdx.x == 0) {
        pa[blockIdx.x] = ba;
        pb[blockIdx.x] = bb;
    }
    if (arrive_last(&cs->counter, k.nbc)) {
        const double rho = final_tree(pa + k.blk0, k.nbc, sma), rr = final_tree(pb + k.blk0, k.nbc, smb);
        if (threadIdx.x == 0) {
            const SolverParams& prm = L.bs->prm;
            const double res0 = sqrt(rr);
            double tol = prm.rel_tol * tol_base(cs, res0);
            if (prm.abs_tol > tol) tol = prm.abs_tol;
            cs->res0 = cs->res = res0;
            cs->tol = tol;
            cs->rho = rho;
            cs->beta = rho / 1.0;
            bool done = !(res0 > tol) || res0 == 0.0;
            if (!isfinite(res0)) {
                done = true;
                cs->status = FVGB_ERR_BREAKDOWN;
            } else if (!done && prm.max_iter <= 0) {
                done = true;
                cs->status = FVGB_ERR_NOT_CONVERGED;
            } else if (!done && !(rho != 0.0 && isfinite(rho))) {
                done = true;
                cs->status = FVGB_ERR_BREAKDOWN;
            }
            if (done) case_done(L.bs, cs);
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0)
        cudaGraphSetConditional(h, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
}

__global__ void __launch_bounds__(kT)
    k_bg_dir(Layout L, const double* __restrict__ z, const double* __restrict__ z2, double* __restrict__ p,
             double* __restrict__ p2) {
    const Blk k = blk_info(L);
    const CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    const double beta = cs->beta;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        p[i] = fma(beta, p[i], __ldg(&z[i]));
        p2[i] = fma(beta, p2[i], __ldg(&z2[i]));
    }
}

__global__ void __launch_bounds__(kT)
    k_bg_spmv(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ p,
              const double* __restrict__ p2, double* __restrict__ q, double* __restrict__ q2,
              double* __restrict__ pa) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    __shared__ double sma[kT];
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double qi = spmv_row(m, val, p, i);
        q[i] = qi;
        q2[i] = spmv_row_t(m, val, p2, i);
        acc = fma(__ldg(&p2[i]), qi, acc);
    }
    const double ba = block_tree(acc, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double pq = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        const double alpha = cs->rho / pq;
        cs->alpha = alpha;
        if (pq == 0.0 || !isfinite(alpha)) {
            cs->status = FVGB_ERR_BREAKDOWN;
            case_done(L.bs, cs);
        }
    }
}

__global__ void __launch_bounds__(kT)
    k_bg_update(Layout L, const double* __restrict__ dinv, const double* __restrict__ p,
                const double* __restrict__ q, const double* __restrict__ q2, double* __restrict__ r,
                double* __restrict__ r2, double* __restrict__ z, double* __restrict__ z2, double* __restrict__ pa,
                double* __restrict__ pb, cudaGraphConditionalHandle h) {
    __shared__ double sma[kT], smb[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (ld_volatile(&cs->active)) {
        double* __restrict__ x = L.bs->prm.x;
        const double alpha = cs->alpha;
        double arho = 0.0, arr = 0.0;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            x[i] = fma(alpha, __ldg(&p[i]), x[i]);
            const double ri = fma(-alpha, __ldg(&q[i]), r[i]);
            const double r2i = fma(-alpha, __ldg(&q2[i]), r2[i]);
            const double di = __ldg(&dinv[i]);
            const double zi = di * ri;
            r[i] = ri;
            r2[i] = r2i;
            z[i] = zi;
            z2[i] = di * r2i;
            arho = fma(r2i, zi, arho);
            arr = fma(ri, ri, arr);
        }
        const double ba = block_tree(arho, sma), bb = block_tree(arr, smb);
        if (threadIdx.x == 0) {
            pa[blockIdx.x] = ba;
            pb[blockIdx.x] = bb;
        }
        if (arrive_last(&cs->counter, k.nbc)) {
            const double rho = final_tree(pa + k.blk0, k.nbc, sma), rr = final_tree(pb + k.blk0, k.nbc, smb);
            if (threadIdx.x == 0) {
                const double res = sqrt(rr);
                cs->res = res;
                cs->iter += 1;
                cs->beta = rho / cs->rho;
                cs->rho = rho;
                bool done = false;
                if (!isfinite(res)) {
                    cs->status = FVGB_ERR_BREAKDOWN;
                    done = true;
                } else if (!(res > cs->tol)) {
                    done = true;
                } else if (cs->iter >= L.bs->prm.max_iter) {
                    cs->status = FVGB_ERR_NOT_CONVERGED;
                    done = true;
                } else if (!(rho != 0.0 && isfinite(rho))) {
                    cs->status = FVGB_ERR_BREAKDOWN;
                    done = true;
                }
                if (done) case_done(L.bs, cs);
            }
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0)
        cudaGraphSetConditional(h, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
}

// --------------------------------------------------- mixed precision (FP32 inner)
// The inner CG runs in FP32 on the row-sign-normalised system  D_s A y = D_s r
// (D_s = the sign of each row's diagonal: the solution is unchanged, and for a
// case whose diagonals share one sign every dot product is positive), Jacobi
// preconditioned with |1/a_ii|.  The FP32 SpMV uses the difference form
//     (A p)_i = e_i p_i + sum_{j != i} a_ij (p_j - p_i),   e_i = sum_j a_ij,
// which keeps the near-null space of a Laplacian (smooth fields) exact in FP32:
// in a pressure equation every e_i but the reference cell's is zero up to
// round-off, so rounding a_ij to FP32 no longer perturbs the smallest
// eigenvalues (the plain form needs about 20% more inner iterations there).
// Dots: per-thread fmaf and block trees in FP32, block partials summed in FP64.

// Power-of-two scale bringing |D^-1/2 r| to [1, 2): the FP32 residual is
// (float)(sig * r).  Scaling by a power of two is exact, so the inner iterates
// are the unscaled ones times sig, except that the FP32 products of a tiny
// residual (a field that has almost stopped changing) no longer underflow.
__device__ __host__ __forceinline__ void residual_scale(double sres, double* sig, double* isig) {
    int e = 0;
    if (sres > 0.0 && isfinite(sres)) {
        e = ilogb(sres);
        e = e > 900 ? 900 : (e < -900 ? -900 : e);
    }
    *sig = ldexp(1.0, -e);
    *isig = ldexp(1.0, e);
}

// Per row: dinv = (float)(1/a_ii) (signed), a32 = (float)(sign * a_ij) at the
// off-diagonal slots (0 at the diagonal and the padding), ev = (float)(sign * e_i)
// with e_i summed in FP64 in slot order; signflags bit0: a positive diagonal,
// bit1: negative, bit2: zero/NaN; sres = sqrt(sum r_i^2 |1/a_ii|) of r = b - A x0,
// the magnitude the first residual is scaled by.
__global__ void __launch_bounds__(kT)
    k_ir_prepare(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
                 float* __restrict__ a32, float* __restrict__ ev, float* __restrict__ dinv, double* __restrict__ r0,
                 double* __restrict__ pa) {
    __shared__ double sma[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    const double* __restrict__ x = L.bs->prm.x;
    const bool convert = L.bs->prm.convert != 0;
    unsigned int f = 0;
    double asr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const double d = __ldg(&val[__ldg(&m.diag_pos[i])]);
        f |= d > 0.0 ? 1u : (d < 0.0 ? 2u : 4u);
        float di;
        if (convert) {
            di = (float)(1.0 / d);
            dinv[i] = di;
            const double sg = d < 0.0 ? -1.0 : 1.0;
            const int slice = i >> 5, lane = i & 31;
            const int b0 = __ldg(&m.m_ptr[slice]);
            const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
            double e = 0.0;
            for (int kk = 0; kk < w; ++kk) {
                const int pos = b0 + kk * 32 + lane;
                const int code = __ldg(&m.m_code[pos]);
                if (code == FVGB_PAD) {
                    a32[pos] = 0.0f;
                    continue;
                }
                const double a = __ldg(&val[pos]);
                e = e + a;
                a32[pos] = code == -1 ? 0.0f : (float)(sg * a);
            }
            ev[i] = (float)(sg * e);
        } else {
            di = dinv[i];
        }
        const double ri = __ldg(&b[i]) - spmv_row(m, val, x, i);
        r0[i] = ri;  // the first refinement step takes it from here
        asr = fma(ri * (double)fabsf(di), ri, asr);
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(&cs->signflags, f);
    const double ba = block_tree(asr, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double sr2 = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        cs->sres = sqrt(sr2);
        cs->sig = 1.0;
        cs->isig = 1.0;
    }
}

// refinement step: r = b - A x (FP64), |r|; rh = sign * (float)(sig r); y = 0;
// rho = rh . (|dinv| rh).  FIRST: p = |dinv| rh.  Later steps keep p;
// k_ir_reliable_dir folds the new residual into it.
template <bool FIRST>
__global__ void __launch_bounds__(kT)
    k_ir_residual(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
                  const double* __restrict__ r0, const float* __restrict__ dinv, float* __restrict__ rh,
                  float* __restrict__ y,
                  float* __restrict__ p, double* __restrict__ pa, double* __restrict__ pb, double* __restrict__ pc,
                  cudaGraphConditionalHandle h_outer, cudaGraphConditionalHandle h_inner) {
    __shared__ double sma[kT], smb[kT], smc[kT];
    __shared__ float smf[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (FIRST || ld_volatile(&cs->active)) {
        const double* __restrict__ x = L.bs->prm.x;
        double sig, isig;
        residual_scale(cs->sres, &sig, &isig);  // from the previous residual (k_ir_prepare's for the first)
        double arr = 0.0, asr = 0.0;
        float arho = 0.0f;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            const double ri = FIRST ? r0[i] : __ldg(&b[i]) - spmv_row(m, val, x, i);
            arr = fma(ri, ri, arr);
            const float di = __ldg(&dinv[i]);
            asr = fma(ri * (double)fabsf(di), ri, asr);
            float rhi = (float)(ri * sig);
            if (di < 0.0f) rhi = -rhi;
            rh[i] = rhi;
            y[i] = 0.0f;
            const float zi = fabsf(di) * rhi;
            if (FIRST) p[i] = zi;
            arho = fmaf(rhi, zi, arho);
        }
        const double ba = block_tree(arr, sma);
        const double bc = block_tree(asr, smc);
        const float bb = block_tree_f(arho, smf);
        if (threadIdx.x == 0) {
            pa[blockIdx.x] = ba;
            pb[blockIdx.x] = (double)bb;
            pc[blockIdx.x] = bc;
        }
        if (arrive_last(&cs->counter, k.nbc)) {
            const double rr = final_tree(pa + k.blk0, k.nbc, sma), rho = final_tree(pb + k.blk0, k.nbc, smb);
            const double sr2 = final_tree(pc + k.blk0, k.nbc, smc);
            if (threadIdx.x == 0) {
                const SolverParams& prm = L.bs->prm;
                const double res = sqrt(rr);
                if (!FIRST) cs->outer += 1;
                cs->res = res;
                bool done = false;
                if (FIRST) {
                    cs->res0 = res;
                    double tol = prm.rel_tol * tol_base(cs, res);
                    if (prm.abs_tol > tol) tol = prm.abs_tol;
                    cs->tol = tol;
                    const unsigned int sf = cs->signflags;
                    if ((sf & 4u) || sf == 3u) {
                        cs->status = FVGB_ERR_UNSUPPORTED;
                        done = true;
                    }
                }
                if (!done) {
                    if (!isfinite(res)) {
                        cs->status = FVGB_ERR_BREAKDOWN;
                        done = true;
                    } else if (!(res > cs->tol) || res == 0.0) {
                        done = true;
                    } else if (cs->outer >= prm.max_outer || cs->total >= prm.max_iter) {
                        cs->status = FVGB_ERR_NOT_CONVERGED;
                        done = true;
                    }
                }
                // direction after this update: keep p (beta = rho/rho_prev, with p brought
                // from the previous scale to this one), or restart from the new
                // preconditioned residual when no inner iteration ran since the last update
                // or the FP32 recursion has drifted (true rho above 4x the recursive one:
                // the old direction would then swamp the new residual)
                const double g = sig * cs->isig;  // new scale / old scale, a power of two
                const double rho_rec = cs->rho * g * g;
                const bool restart = FIRST || cs->inner_it == 0 || rho > 4.0 * rho_rec;
                cs->frel = restart ? -1.0f : (float)((rho / cs->rho_prev) * (cs->sig * isig));
                cs->sig = sig;
                cs->isig = isig;
                cs->sres = sqrt(sr2);
                cs->rho = rho;
                // leave the inner loop when the FP32 residual dropped by inner_rel_tol or
                // should be below the FP64 tolerance (estimated through this update's ratio)
                const double dr = prm.inner_rel_tol * prm.inner_rel_tol;
                const double dt = (cs->tol / res) * (cs->tol / res);
                cs->itol = rho * (dr > dt ? dr : dt);
                cs->inner_it = 0;
                const bool inner = !done && rho > cs->itol && prm.inner_max_iter > 0 && cs->total < prm.max_iter;
                cs->inner_active = inner ? 1 : 0;
                if (inner) atomicAdd(&L.bs->n_inner, 1);
                if (done) case_done(L.bs, cs);
            }
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0) {
        cudaGraphSetConditional(h_inner, ld_volatile(&L.bs->n_inner) > 0 ? 1u : 0u);
        cudaGraphSetConditional(h_outer, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
    }
}

// p = z + frel * p after a reliable update (p = z when frel < 0), z = |dinv| rh
__global__ void __launch_bounds__(kT)
    k_ir_reliable_dir(Layout L, const float* __restrict__ dinv, const float* __restrict__ rh, float* __restrict__ p) {
    const Blk k = blk_info(L);
    const CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->inner_active)) return;
    const float fb = cs->frel;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const float zi = fabsf(__ldg(&dinv[i])) * __ldg(&rh[i]);
        p[i] = fb < 0.0f ? zi : fmaf(fb, p[i], zi);
    }
}

__device__ __forceinline__ void inner_stop(const Layout& L, CaseState* cs) {
    cs->inner_active = 0;
    atomicSub(&L.bs->n_inner, 1);
}

// q = (D_s A) p in the difference form; p.q -> alpha
template <int MINB>
__global__ void __launch_bounds__(kT, MINB)
    k_ir_spmv(Layout L, MeshView m, const float* __restrict__ a32, const float* __restrict__ ev,
              const float* __restrict__ p, float* __restrict__ q, double* __restrict__ pa) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->inner_active)) return;
    __shared__ double sma[kT];
    __shared__ float smf[kT];
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const float pi = __ldg(&p[i]);
        const float qi = spmv_row_diff(m, a32, p, i, pi, __ldg(&ev[i]));
        q[i] = qi;
        acc = fmaf(pi, qi, acc);
    }
    const float ba = block_tree_f(acc, smf);
    if (threadIdx.x == 0) pa[blockIdx.x] = (double)ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double pq = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        const double alpha = cs->rho / pq;
        if (pq == 0.0 || !isfinite(alpha)) {
            inner_stop(L, cs);
            if (cs->inner_it == 0) {
                cs->status = FVGB_ERR_BREAKDOWN;
                case_done(L.bs, cs);
            }
        } else {
            cs->falpha = (float)alpha;
        }
    }
}

// y += alpha p, rh -= alpha q, rho = rh . (|dinv| rh)
template <int MINB>
__global__ void __launch_bounds__(kT, MINB)
    k_ir_update(Layout L, const float* __restrict__ dinv, const float* __restrict__ p, const float* __restrict__ q,
                float* __restrict__ y, float* __restrict__ rh, double* __restrict__ pa,
                cudaGraphConditionalHandle h_inner, int setc) {
    __shared__ double sma[kT];
    __shared__ float smf[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (ld_volatile(&cs->inner_active)) {
        const float fa = cs->falpha;
        float acc = 0.0f;
        constexpr int G = 4;  // rows whose loads are issued together (more spill at 32-40 registers)
        static_assert(kRowsPerThread % G == 0, "rows per thread in whole load groups");
#pragma unroll
        for (int j0 = 0; j0 < kRowsPerThread; j0 += G) {
            float pv[G], qv[G], yv[G], rv[G], dv[G];
#pragma unroll
            for (int u = 0; u < G; ++u) {  // every load of the group first
                const int i = blk_row(k, j0 + u);
                pv[u] = qv[u] = yv[u] = rv[u] = dv[u] = 0.0f;
                if (i >= k.end) continue;
                pv[u] = __ldg(&p[i]);
                qv[u] = __ldg(&q[i]);
                dv[u] = __ldg(&dinv[i]);
                yv[u] = y[i];
                rv[u] = rh[i];
            }
#pragma unroll
            for (int u = 0; u < G; ++u) {
                const int i = blk_row(k, j0 + u);
                if (i >= k.end) continue;
                y[i] = fmaf(fa, pv[u], yv[u]);
                const float ri = fmaf(-fa, qv[u], rv[u]);
                rh[i] = ri;
                acc = fmaf(ri, fabsf(dv[u]) * ri, acc);
            }
        }
        const float ba = block_tree_f(acc, smf);
        if (threadIdx.x == 0) pa[blockIdx.x] = (double)ba;
        if (arrive_last(&cs->counter, k.nbc)) {
            const double rhon = final_tree(pa + k.blk0, k.nbc, sma);
            if (threadIdx.x == 0) {
                const SolverParams& prm = L.bs->prm;
                cs->fbeta = (float)(rhon / cs->rho);
                cs->rho_prev = cs->rho;
                cs->rho = rhon;
                cs->inner_it += 1;
                cs->total += 1;
                const bool more = rhon > cs->itol && cs->inner_it < prm.inner_max_iter && cs->total < prm.max_iter;
                if (!more) inner_stop(L, cs);
            }
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0 && setc)
        cudaGraphSetConditional(h_inner, ld_volatile(&L.bs->n_inner) > 0 ? 1u : 0u);
}

// p = z + beta p, z = |dinv| rh
__global__ void __launch_bounds__(kT)
    k_ir_dir(Layout L, const float* __restrict__ dinv, const float* __restrict__ rh, float* __restrict__ p) {
    const Blk k = blk_info(L);
    const CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->inner_active)) return;
    const float fb = cs->fbeta;
    float pv[kRowsPerThread], dv[kRowsPerThread], rv[kRowsPerThread];
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {  // every load first
        const int i = blk_row(k, j);
        pv[j] = dv[j] = rv[j] = 0.0f;
        if (i >= k.end) continue;
        pv[j] = p[i];
        dv[j] = __ldg(&dinv[i]);
        rv[j] = __ldg(&rh[i]);
    }
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        p[i] = fmaf(fb, pv[j], fabsf(dv[j]) * rv[j]);
    }
}

// x += y / sig (y carries the power-of-two scale of its residual)
__global__ void __launch_bounds__(kT) k_ir_xupdate(Layout L, const float* __restrict__ y) {
    const Blk k = blk_info(L);
    const CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->active)) return;
    double* __restrict__ x = L.bs->prm.x;
    const double isig = cs->isig;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        x[i] = fma((double)__ldg(&y[i]), isig, x[i]);
    }
}

// ------------------------------------------------ mixed-precision BiCGStab
// FP64 iterative refinement around a restarted FP32 BiCGStab (Jacobi, right
// preconditioning) on the row-sign-normalised FP32 system of the mixed CG
// (k_ir_prepare: a32, ev, dinv; difference-form SpMV; power-of-two residual
// scale).  Each refinement step: r = b - A x in FP64, rh = sign*(float)(sig r),
// then BiCGStab on (D_s A) e = rh from e = 0 with shadow residual rh, until
// |r_inner|^2 <= itol = |rh|^2 max(inner_rel_tol^2, (tol/|r|)^2), the FP32
// recursion breaks down, or the iteration caps are hit; x += e / sig.
// Inner vectors (FP32): rh = r, rr (shadow), p, v, yv = |dinv| p, s, z =
// |dinv| s, t, e.  Dots: per-thread fmaf, FP32 block trees, FP64 sums of the
// block partials (as the mixed CG).

// refinement step: r = b - A x (FP64) or the preparation's r0 (FIRST), |r|;
// rh = rr = sign*(float)(sig r); p = v = e = 0; rho = rh.rh
template <bool FIRST>
__global__ void __launch_bounds__(kT)
    k_mb_residual(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
                  const double* __restrict__ r0, const float* __restrict__ dinv, float* __restrict__ rh,
                  float* __restrict__ rr, float* __restrict__ p, float* __restrict__ v, float* __restrict__ e,
                  double* __restrict__ pa, double* __restrict__ pb, double* __restrict__ pc,
                  cudaGraphConditionalHandle h_outer, cudaGraphConditionalHandle h_inner) {
    __shared__ double sma[kT], smb[kT], smc[kT];
    __shared__ float smf[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (FIRST || ld_volatile(&cs->active)) {
        const double* __restrict__ x = L.bs->prm.x;
        double sig, isig;
        residual_scale(cs->sres, &sig, &isig);
        double arr = 0.0, asr = 0.0;
        float arho = 0.0f;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            const double ri = FIRST ? r0[i] : __ldg(&b[i]) - spmv_row(m, val, x, i);
            arr = fma(ri, ri, arr);
            const float di = __ldg(&dinv[i]);
            asr = fma(ri * (double)fabsf(di), ri, asr);
            float rhi = (float)(ri * sig);
            if (di < 0.0f) rhi = -rhi;
            rh[i] = rhi;
            rr[i] = rhi;
            p[i] = 0.0f;
            v[i] = 0.0f;
            e[i] = 0.0f;
            arho = fmaf(rhi, rhi, arho);
        }
        const double ba = block_tree(arr, sma);
        const double bc = block_tree(asr, smc);
        const float bb = block_tree_f(arho, smf);
        if (threadIdx.x == 0) {
            pa[blockIdx.x] = ba;
            pb[blockIdx.x] = (double)bb;
            pc[blockIdx.x] = bc;
        }
        if (arrive_last(&cs->counter, k.nbc)) {
            const double rr2 = final_tree(pa + k.blk0, k.nbc, sma), rho = final_tree(pb + k.blk0, k.nbc, smb);
            const double sr2 = final_tree(pc + k.blk0, k.nbc, smc);
            if (threadIdx.x == 0) {
                const SolverParams& prm = L.bs->prm;
                const double res = sqrt(rr2);
                if (!FIRST) cs->outer += 1;
                cs->res = res;
                bool done = false;
                if (FIRST) {
                    cs->res0 = res;
                    double tol = prm.rel_tol * tol_base(cs, res);
                    if (prm.abs_tol > tol) tol = prm.abs_tol;
                    cs->tol = tol;
                    const unsigned int sf = cs->signflags;
                    if ((sf & 4u) || sf == 3u) {
                        cs->status = FVGB_ERR_UNSUPPORTED;
                        done = true;
                    }
                }
                if (!done) {
                    if (!isfinite(res)) {
                        cs->status = FVGB_ERR_BREAKDOWN;
                        done = true;
                    } else if (!(res > cs->tol) || res == 0.0) {
                        done = true;
                    } else if (cs->outer >= prm.max_outer || cs->total >= prm.max_iter) {
                        cs->status = FVGB_ERR_NOT_CONVERGED;
                        done = true;
                    }
                }
                cs->sig = sig;
                cs->isig = isig;
                cs->sres = sqrt(sr2);
                cs->rho = rho;
                cs->rho_prev = 1.0;
                cs->alpha = 1.0;
                cs->omega = 1.0;
                cs->falpha = 1.0f;
                cs->fomega = 1.0f;
                cs->fbeta = 0.0f;  // p = r on the first inner iteration
                cs->half = 0;
                const double dr = prm.inner_rel_tol * prm.inner_rel_tol;
                const double dt = (cs->tol / res) * (cs->tol / res);
                cs->itol = rho * (dr > dt ? dr : dt);
                cs->inner_it = 0;
                const bool inner = !done && rho > cs->itol && prm.inner_max_iter > 0 && cs->total < prm.max_iter;
                cs->inner_active = inner ? 1 : 0;
                if (inner) atomicAdd(&L.bs->n_inner, 1);
                if (done) case_done(L.bs, cs);
            }
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0) {
        cudaGraphSetConditional(h_inner, ld_volatile(&L.bs->n_inner) > 0 ? 1u : 0u);
        cudaGraphSetConditional(h_outer, ld_volatile(&L.bs->n_active) > 0 ? 1u : 0u);
    }
}

// an FP32 breakdown ends the inner solve; before its first iteration it ends the case
__device__ __forceinline__ void mb_breakdown(const Layout& L, CaseState* cs) {
    inner_stop(L, cs);
    if (cs->inner_it == 0) {
        cs->status = FVGB_ERR_BREAKDOWN;
        case_done(L.bs, cs);
    }
}

// p = r + beta (p - omega v), yv = |dinv| p
__global__ void __launch_bounds__(kT)
    k_mb_dir(Layout L, const float* __restrict__ dinv, const float* __restrict__ rh, const float* __restrict__ v,
             float* __restrict__ p, float* __restrict__ yv) {
    const Blk k = blk_info(L);
    const CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->inner_active)) return;
    const float fb = cs->fbeta, fo = cs->fomega;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const float pi = fmaf(fb, fmaf(-fo, __ldg(&v[i]), p[i]), __ldg(&rh[i]));
        p[i] = pi;
        yv[i] = fabsf(__ldg(&dinv[i])) * pi;
    }
}

// v = (D_s A) yv, alpha = rho / (rr . v)
__global__ void __launch_bounds__(kT)
    k_mb_spmv1(Layout L, MeshView m, const float* __restrict__ a32, const float* __restrict__ ev,
               const float* __restrict__ yv, const float* __restrict__ rr, float* __restrict__ v,
               double* __restrict__ pa) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->inner_active)) return;
    __shared__ double sma[kT];
    __shared__ float smf[kT];
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const float vi = spmv_row_diff(m, a32, yv, i, __ldg(&yv[i]), __ldg(&ev[i]));
        v[i] = vi;
        acc = fmaf(__ldg(&rr[i]), vi, acc);
    }
    const float ba = block_tree_f(acc, smf);
    if (threadIdx.x == 0) pa[blockIdx.x] = (double)ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double rv = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        const double alpha = cs->rho / rv;
        if (rv == 0.0 || !isfinite(alpha)) {
            mb_breakdown(L, cs);
        } else {
            cs->alpha = alpha;
            cs->falpha = (float)alpha;
        }
    }
}

// s = r - alpha v, z = |dinv| s, |s|^2 (at or below itol: the half step ends the inner solve)
__global__ void __launch_bounds__(kT)
    k_mb_s(Layout L, const float* __restrict__ dinv, const float* __restrict__ rh, const float* __restrict__ v,
           float* __restrict__ sv, float* __restrict__ z, double* __restrict__ pa) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->inner_active)) return;
    __shared__ double sma[kT];
    __shared__ float smf[kT];
    const float fa = cs->falpha;
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const float si = fmaf(-fa, __ldg(&v[i]), __ldg(&rh[i]));
        sv[i] = si;
        z[i] = fabsf(__ldg(&dinv[i])) * si;
        acc = fmaf(si, si, acc);
    }
    const float ba = block_tree_f(acc, smf);
    if (threadIdx.x == 0) pa[blockIdx.x] = (double)ba;
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double ss = final_tree(pa + k.blk0, k.nbc, sma);
    if (threadIdx.x == 0) {
        if (!isfinite(ss)) mb_breakdown(L, cs);
        else if (!(ss > cs->itol)) cs->half = 1;
    }
}

// half step: e += alpha yv, inner solve done; else t = (D_s A) z, omega = (t.s)/(t.t)
__global__ void __launch_bounds__(kT)
    k_mb_spmv2(Layout L, MeshView m, const float* __restrict__ a32, const float* __restrict__ ev,
               const float* __restrict__ z, const float* __restrict__ sv, const float* __restrict__ yv,
               float* __restrict__ t, float* __restrict__ e, double* __restrict__ pa, double* __restrict__ pb) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (!ld_volatile(&cs->inner_active)) return;
    __shared__ double sma[kT], smb[kT];
    __shared__ float smf[kT], smg[kT];
    if (ld_volatile(&cs->half)) {
        const float fa = cs->falpha;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            e[i] = fmaf(fa, __ldg(&yv[i]), e[i]);
        }
        if (arrive_last(&cs->counter, k.nbc) && threadIdx.x == 0) {
            cs->inner_it += 1;
            cs->total += 1;
            cs->half = 0;
            inner_stop(L, cs);
        }
        return;
    }
    float ats = 0.0f, att = 0.0f;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const float ti = spmv_row_diff(m, a32, z, i, __ldg(&z[i]), __ldg(&ev[i]));
        t[i] = ti;
        ats = fmaf(ti, __ldg(&sv[i]), ats);
        att = fmaf(ti, ti, att);
    }
    const float ba = block_tree_f(ats, smf), bb = block_tree_f(att, smg);
    if (threadIdx.x == 0) {
        pa[blockIdx.x] = (double)ba;
        pb[blockIdx.x] = (double)bb;
    }
    if (!arrive_last(&cs->counter, k.nbc)) return;
    const double ts = final_tree(pa + k.blk0, k.nbc, sma), tt = final_tree(pb + k.blk0, k.nbc, smb);
    if (threadIdx.x == 0) {
        const double omega = ts / tt;
        if (tt == 0.0 || !isfinite(omega) || omega == 0.0) {
            mb_breakdown(L, cs);
        } else {
            cs->omega = omega;
            cs->fomega = (float)omega;
        }
    }
}

// e += alpha yv + omega z, r = s - omega t, rho = rr . r, |r|^2
__global__ void __launch_bounds__(kT)
    k_mb_update(Layout L, const float* __restrict__ yv, const float* __restrict__ z, const float* __restrict__ sv,
                const float* __restrict__ t, const float* __restrict__ rr, float* __restrict__ rh,
                float* __restrict__ e, double* __restrict__ pa, double* __restrict__ pb,
                cudaGraphConditionalHandle h_inner) {
    __shared__ double sma[kT], smb[kT];
    __shared__ float smf[kT], smg[kT];
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (ld_volatile(&cs->inner_active)) {
        const float fa = cs->falpha, fo = cs->fomega;
        float arho = 0.0f, arr = 0.0f;
#pragma unroll
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int i = blk_row(k, j);
            if (i >= k.end) continue;
            e[i] = fmaf(fo, __ldg(&z[i]), fmaf(fa, __ldg(&yv[i]), e[i]));
            const float ri = fmaf(-fo, __ldg(&t[i]), __ldg(&sv[i]));
            rh[i] = ri;
            arho = fmaf(__ldg(&rr[i]), ri, arho);
            arr = fmaf(ri, ri, arr);
        }
        const float ba = block_tree_f(arho, smf), bb = block_tree_f(arr, smg);
        if (threadIdx.x == 0) {
            pa[blockIdx.x] = (double)ba;
            pb[blockIdx.x] = (double)bb;
        }
        if (arrive_last(&cs->counter, k.nbc)) {
            const double rho = final_tree(pa + k.blk0, k.nbc, sma), r2 = final_tree(pb + k.blk0, k.nbc, smb);
            if (threadIdx.x == 0) {
                const SolverParams& prm = L.bs->prm;
                cs->inner_it += 1;
                cs->total += 1;
                const double beta = (rho / cs->rho) * (cs->alpha / cs->omega);
                cs->rho_prev = cs->rho;
                cs->rho = rho;
                cs->fbeta = (float)beta;
                const bool more = r2 > cs->itol && isfinite(r2) && rho != 0.0 && isfinite(beta) &&
                                  cs->inner_it < prm.inner_max_iter && cs->total < prm.max_iter;
                if (!more) inner_stop(L, cs);
            }
        }
    }
    if (arrive_last(&L.bs->gcounter, gridDim.x) && threadIdx.x == 0)
        cudaGraphSetConditional(h_inner, ld_volatile(&L.bs->n_inner) > 0 ? 1u : 0u);
}

// State for timing the FP32 kernels outside a solve: every case's inner solve
// active with rho = 1, a direction of pseudo-random O(1) values.
__global__ void k_tune_mixed_state(Layout L, float* __restrict__ p, float* __restrict__ rh, float* __restrict__ y) {
    const Blk k = blk_info(L);
    CaseState* cs = &L.cases[k.c];
    if (threadIdx.x == 0 && blockIdx.x == __ldg(&L.case_blk0[k.c])) {
        cs->inner_active = 1;
        cs->rho = 1.0;
        cs->itol = 0.0;
    }
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = blk_row(k, j);
        if (i >= k.end) continue;
        const unsigned int hsh = (unsigned int)i * 2654435761u;
        p[i] = 0.5f + (float)(hsh >> 8) * (1.0f / 16777216.0f);
        rh[i] = 1.0f;
        y[i] = 0.0f;
    }
}

// ------------------------------------------------------------ kernel variants
// The SpMV and update kernels of both solves exist in launch-bound variants
// (minimum resident blocks per SM 2, 4, 6, 8: a register budget of 128, 64,
// 42, 32 per thread).  They execute the same instructions in the same order on
// the same data, so every variant gives the same bits; which one is fastest
// depends on the mesh (row width, size against L2).  The autotuner below times
// them on the system being solved and the graphs are built with the winner.
constexpr int kNumVariants = 4;
constexpr int kVariantMinBlocks[kNumVariants] = {2, 4, 6, 8};
enum { kTuneSpmv64 = 0, kTuneUpdate64 = 1, kTuneSpmvMixed = 2, kTuneUpdateMixed = 3, kTuneKinds = 4 };

const void* variant_fn(int kind, int v) {
    switch (kind * kNumVariants + v) {
        case 0: return (const void*)k_pcg_spmv<2>;
        case 1: return (const void*)k_pcg_spmv<4>;
        case 2: return (const void*)k_pcg_spmv<6>;
        case 3: return (const void*)k_pcg_spmv<8>;
        case 4: return (const void*)k_pcg_update<2>;
        case 5: return (const void*)k_pcg_update<4>;
        case 6: return (const void*)k_pcg_update<6>;
        case 7: return (const void*)k_pcg_update<8>;
        case 8: return (const void*)k_ir_spmv<2>;
        case 9: return (const void*)k_ir_spmv<4>;
        case 10: return (const void*)k_ir_spmv<6>;
        case 11: return (const void*)k_ir_spmv<8>;
        case 12: return (const void*)k_ir_update<2>;
        case 13: return (const void*)k_ir_update<4>;
        case 14: return (const void*)k_ir_update<6>;
        default: return (const void*)k_ir_update<8>;
    }
}

// Launch of a kernel variant; the arguments are passed with the kernel's exact parameter types.
template <class... A>
cudaError_t launch_variant(const void* fn, unsigned grid, cudaStream_t s, A... args) {
    void* a[] = {(void*)&args...};
    return cudaLaunchKernel(fn, dim3(grid), dim3(kT), a, 0, s);
}

// ------------------------------------------------------ persistent solves (one case)
// For systems small enough that launch latency dominates an iteration, ONE
// cooperative launch runs the whole solve.  A persistent block has 1024 threads
// and walks the 256*R-row virtual blocks vb = blockIdx.x, blockIdx.x + gridDim.x,
// ...; thread t computes rows vb*256R + t (and vb*256R + 1024 + t when R = 8).
// Dot products are staged in shared memory and summed by 256 "tree threads"
// with exactly the row assignment and order of the graph kernels (R rows per
// thread, then the block tree), so the
// per-virtual-block partials, and after a grid barrier the final trees that
// EVERY block computes over all partials, are the bits of the graph path; all
// blocks then take identical decisions.  Data written during the kernel is
// read through L2 (__ldcg).  Grid barriers spin a bounded number of times; on
// time-out a block raises the abort flag, every block leaves at its next
// barrier and the solve reports FVGB_ERR_CUDA.
constexpr int kPT = 1024;
static_assert((kT * 4) % kPT == 0, "a virtual block is a whole number of rows per thread");

struct GridBar {
    unsigned long long count;  // arrivals since the launch (never reset inside it)
    int abort, pad;
};

// Barrier number `epoch` (1, 2, ...) of a grid of `nblocks` blocks.
__device__ __forceinline__ bool grid_sync(GridBar* g, unsigned long long target) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        unsigned long long v;
        asm volatile("atom.add.release.gpu.u64 %0, [%1], 1;" : "=l"(v) : "l"(&g->count) : "memory");
        v += 1;
        unsigned long long spins = 0;
        while (v < target) {
            int ab;
            asm volatile("ld.relaxed.gpu.s32 %0, [%1];" : "=r"(ab) : "l"(&g->abort) : "memory");
            if (ab) {
                good = 0;
                break;
            }
            if (++spins > (1ull << 26)) {  // a few seconds
                atomicExch(&g->abort, 1);
                good = 0;
                break;
            }
            if (spins > 32) __nanosleep(32);
            asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(&g->count) : "memory");
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// row (within a virtual block) of tree thread tp's j-th row: the graph kernels' blk_row
template <int R>
__device__ __forceinline__ int tree_row(int tp, int j) { return (tp >> 5) * (32 * R) + j * 32 + (tp & 31); }

// block_tree over the partials of threads 0..kT-1 of a kPT-thread block; valid in warp 0
__device__ __forceinline__ double tree256(double v, double* sm) {
    if (threadIdx.x < kT) sm[threadIdx.x] = v;
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

__device__ __forceinline__ float tree256f(float v, float* sm) {
    if (threadIdx.x < kT) sm[threadIdx.x] = v;
    __syncthreads();
    float s = 0.0f;
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

// final_tree over nvb partials, broadcast to every thread of the block
__device__ __forceinline__ double final_all(const double* part, int nvb, double* sm, double* cell) {
    double a = 0.0;
    if (threadIdx.x < kT)
        for (int i = threadIdx.x; i < nvb; i += kT) a = a + __ldcg(&part[i]);
    const double s = tree256(a, sm);
    if (threadIdx.x == 0) *cell = s;
    __syncthreads();
    const double r = *cell;
    __syncthreads();
    return r;
}

__device__ __forceinline__ double spmv_row_cg(const MeshView& m, const double* __restrict__ val, const double* x,
                                              int i) {
    const int slice = i >> 5, lane = i & 31;
    const int b0 = __ldg(&m.m_ptr[slice]);
    const int base = b0 + lane;
    const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
    int col[8];
    slot_cols(m, base, w, i, col);
    double v[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = 0.0;
        xv[k] = 0.0;
        if (k < w) {
            v[k] = __ldg(&val[base + k * 32]);
            xv[k] = __ldcg(&x[col[k]]);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) s = fma(v[k], xv[k], s);
    for (int k = 8; k < w; ++k) s = fma(__ldg(&val[base + k * 32]), __ldcg(&x[slot_col(m, base + k * 32, i)]), s);
    return s;
}

// Thread 0 of every block keeps the solver scalars; the other threads read
// what a phase needs from shared memory after a barrier (FP64 division and
// square root are long FP64 sequences: evaluated by every thread they would
// cost more FP64 issue than the iteration's arithmetic).
struct PcgShared {
    double alpha, beta;
    int done;
};

template <int R>
__global__ void __launch_bounds__(kPT, 1)
    k_pcg_persistent(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
                     double* dinv, double* r, double* p, double* q, double* z, double* pa, double* pb, GridBar* gb,
                     int nvb) {
    __shared__ double sA[(kT * R)], sB[(kT * R)], sm[kT], sm2[kT], cell;
    __shared__ PcgShared sh;
    const int n = m.n, T = threadIdx.x;
    const SolverParams prm = L.bs->prm;
    double* x = prm.x;
    const unsigned long long G = gridDim.x;
    unsigned long long epoch = 0;
    // init: r = b - A x, z = p = dinv r, r.z, r.r
    for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
        for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
            const int t = T + h * kPT;
            const int i = vb * (kT * R) + t;
            double ri = 0.0, zi = 0.0;
            if (i < n) {
                const double di = 1.0 / __ldg(&val[__ldg(&m.diag_pos[i])]);
                dinv[i] = di;
                ri = __ldg(&b[i]) - spmv_row_cg(m, val, x, i);
                zi = di * ri;
                r[i] = ri;
                p[i] = zi;
            }
            sA[t] = ri;
            sB[t] = zi;
        }
        __syncthreads();
        double arz = 0.0, arr = 0.0;
        if (T < kT)
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const int rr = tree_row<R>(T, j);
                if (vb * (kT * R) + rr >= n) continue;
                arz = fma(sA[rr], sB[rr], arz);
                arr = fma(sA[rr], sA[rr], arr);
            }
        const double ba = tree256(arz, sm), bb = tree256(arr, sm2);
        if (T == 0) {
            pa[vb] = ba;
            pb[vb] = bb;
        }
    }
    bool aborted = !grid_sync(gb, ++epoch * G);
    // solver scalars: meaningful in thread 0 only
    double rz = 0.0, res0 = 0.0, res = 0.0, tol = 0.0;
    int iter = 0, status = FVGB_OK;
    if (!aborted) {
        rz = final_all(pa, nvb, sm, &cell);
        const double rr = final_all(pb, nvb, sm, &cell);
        if (T == 0) {
            res0 = res = sqrt(rr);
            tol = prm.rel_tol * tol_base(&L.cases[0], res0);
            if (prm.abs_tol > tol) tol = prm.abs_tol;
            bool done = !(res0 > tol) || res0 == 0.0;
            if (!isfinite(res0)) {
                done = true;
                status = FVGB_ERR_BREAKDOWN;
            } else if (!done && prm.max_iter <= 0) {
                done = true;
                status = FVGB_ERR_NOT_CONVERGED;
            }
            sh.done = done;
        }
        __syncthreads();
    }
    bool done = aborted || sh.done;
    while (!done) {
        // q = A p, p.q
        for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
            for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
                const int t = T + h * kPT;
                const int i = vb * (kT * R) + t;
                double pi = 0.0, qi = 0.0;
                if (i < n) {
                    qi = spmv_row_cg(m, val, p, i);
                    q[i] = qi;
                    pi = __ldcg(&p[i]);
                }
                sA[t] = pi;
                sB[t] = qi;
            }
            __syncthreads();
            double acc = 0.0;
            if (T < kT)
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    const int rw = tree_row<R>(T, j);
                    if (vb * (kT * R) + rw < n) acc = fma(sA[rw], sB[rw], acc);
                }
            const double ba = tree256(acc, sm);
            if (T == 0) pa[vb] = ba;
        }
        if (!grid_sync(gb, ++epoch * G)) {
            aborted = true;
            break;
        }
        const double pq = final_all(pa, nvb, sm, &cell);
        if (T == 0) {
            const double alpha = rz / pq;
            sh.alpha = alpha;
            sh.done = 0;
            if (pq == 0.0 || !isfinite(alpha)) {
                status = FVGB_ERR_BREAKDOWN;
                sh.done = 1;
            }
        }
        __syncthreads();
        if (sh.done) break;
        const double alpha = sh.alpha;
        // x += alpha p, r -= alpha q, z = dinv r, r.z, r.r
        for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
            for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
                const int t = T + h * kPT;
                const int i = vb * (kT * R) + t;
                double ri = 0.0, zi = 0.0;
                if (i < n) {
                    x[i] = fma(alpha, __ldcg(&p[i]), __ldcg(&x[i]));
                    ri = fma(-alpha, __ldcg(&q[i]), __ldcg(&r[i]));
                    r[i] = ri;
                    zi = __ldcg(&dinv[i]) * ri;
                    z[i] = zi;
                }
                sA[t] = ri;
                sB[t] = zi;
            }
            __syncthreads();
            double arz = 0.0, arr = 0.0;
            if (T < kT)
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    const int rw = tree_row<R>(T, j);
                    if (vb * (kT * R) + rw >= n) continue;
                    arz = fma(sA[rw], sB[rw], arz);
                    arr = fma(sA[rw], sA[rw], arr);
                }
            const double ba = tree256(arz, sm), bb = tree256(arr, sm2);
            if (T == 0) {
                pa[vb] = ba;
                pb[vb] = bb;
            }
        }
        if (!grid_sync(gb, ++epoch * G)) {
            aborted = true;
            break;
        }
        const double rzn = final_all(pa, nvb, sm, &cell);
        const double rr = final_all(pb, nvb, sm, &cell);
        if (T == 0) {
            res = sqrt(rr);
            ++iter;
            sh.beta = rzn / rz;
            rz = rzn;
            int d = 0;
            if (!isfinite(res)) {
                status = FVGB_ERR_BREAKDOWN;
                d = 1;
            } else if (!(res > tol)) {
                d = 1;
            } else if (iter >= prm.max_iter) {
                status = FVGB_ERR_NOT_CONVERGED;
                d = 1;
            }
            sh.done = d;
        }
        __syncthreads();
        if (sh.done) break;
        const double beta = sh.beta;
        // p = z + beta p
        for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
            for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
                const int t = T + h * kPT;
                const int i = vb * (kT * R) + t;
                if (i < n) p[i] = fma(beta, __ldcg(&p[i]), __ldcg(&z[i]));
            }
        }
        if (!grid_sync(gb, ++epoch * G)) {
            aborted = true;
            break;
        }
    }
    if (blockIdx.x == 0 && T == 0) {
        CaseState* cs = &L.cases[0];
        cs->res0 = res0;
        cs->res = res;
        cs->iter = iter;
        cs->status = aborted ? FVGB_ERR_CUDA : status;
    }
}

// Mixed-precision solve in one cooperative launch: the algorithm, arithmetic
// and decisions of the graph kernels (k_ir_prepare ... k_ir_reliable_dir).  An
// inner iteration takes two grid barriers: the direction update p = z + beta p
// is folded into the SpMV, which forms the new direction of every row it reads
// from the previous direction and z (double-buffered p: the new one goes to the
// other buffer while other blocks still read the old).
struct DirMode {
    int kind;  // 0: p as stored, 1: p = z, 2: p = coef*p + z
    float coef;
};

__device__ __forceinline__ float dir_of(const DirMode& d, float pold, float zv) {
    return d.kind == 0 ? pold : (d.kind == 1 ? zv : fmaf(d.coef, pold, zv));
}

__device__ __forceinline__ float spmv_row_diff_dir(const MeshView& m, const float* __restrict__ a, const float* pold,
                                                   const float* zz, const DirMode& d, int i, float xi, float ei) {
    const int slice = i >> 5, lane = i & 31;
    const int b0 = __ldg(&m.m_ptr[slice]);
    const int base = b0 + lane;
    const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
    int col[8];
    slot_cols(m, base, w, i, col);
    float v[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = 0.0f;
        xv[k] = 0.0f;
        if (k < w) {
            v[k] = __ldg(&a[base + k * 32]);
            xv[k] = dir_of(d, __ldcg(&pold[col[k]]), d.kind == 0 ? 0.0f : __ldcg(&zz[col[k]]));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) s = fmaf(v[k], xv[k] - xi, s);
    for (int k = 8; k < w; ++k) {
        const int cidx = slot_col(m, base + k * 32, i);
        const float xc = dir_of(d, __ldcg(&pold[cidx]), d.kind == 0 ? 0.0f : __ldcg(&zz[cidx]));
        s = fmaf(__ldg(&a[base + k * 32]), xc - xi, s);
    }
    return fmaf(ei, xi, s);
}

// Scalars of the refinement live in thread 0 of every block (the graph path
// keeps them in CaseState); what the phases need is broadcast here.
struct IrShared {
    double nsig, isig;  // scale of the residual being formed; 1/scale of the current y
    float fa;           // alpha of the current inner iteration
    DirMode dm;         // how the next SpMV forms the direction
    int done, inner, brk;
};

template <int R>
__global__ void __launch_bounds__(kPT, 1)
    k_ir_persistent(Layout L, MeshView m, const double* __restrict__ val, const double* __restrict__ b,
                    float* a32, float* ev, float* dinv, double* r0, float* rh, float* y, float* pbuf0, float* pbuf1,
                    float* z, float* q, double* pa, double* pb, double* pc, GridBar* gb, int nvb) {
    __shared__ double sD[(kT * R)], sm[kT], sm3[kT], cell;
    __shared__ float sF1[(kT * R)], sF2[(kT * R)], smf[kT];
    __shared__ unsigned int sflags;
    __shared__ IrShared sh;
    const int n = m.n, T = threadIdx.x;
    const SolverParams prm = L.bs->prm;
    double* x = prm.x;
    const unsigned long long G = gridDim.x;
    unsigned long long epoch = 0;
    CaseState* cs = &L.cases[0];
    bool aborted = false;
    // prepare: dinv, a32, ev, sign flags, |D^-1/2 (b - A x0)|
    if (T == 0) sflags = 0u;
    __syncthreads();
    for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
        for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
            const int t = T + h * kPT;
            const int i = vb * (kT * R) + t;
            double ri = 0.0;
            float di = 0.0f;
            if (i < n) {
                const double d = __ldg(&val[__ldg(&m.diag_pos[i])]);
                atomicOr(&sflags, d > 0.0 ? 1u : (d < 0.0 ? 2u : 4u));
                if (prm.convert) {
                    di = (float)(1.0 / d);
                    dinv[i] = di;
                    const double sg = d < 0.0 ? -1.0 : 1.0;
                    const int slice = i >> 5, lane = i & 31;
                    const int b0 = __ldg(&m.m_ptr[slice]);
                    const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
                    double e = 0.0;
                    for (int kk = 0; kk < w; ++kk) {
                        const int pos = b0 + kk * 32 + lane;
                        const int code = __ldg(&m.m_code[pos]);
                        if (code == FVGB_PAD) {
                            a32[pos] = 0.0f;
                            continue;
                        }
                        const double av = __ldg(&val[pos]);
                        e = e + av;
                        a32[pos] = code == -1 ? 0.0f : (float)(sg * av);
                    }
                    ev[i] = (float)(sg * e);
                } else {
                    di = __ldcg(&dinv[i]);
                }
                ri = __ldg(&b[i]) - spmv_row_cg(m, val, x, i);
                r0[i] = ri;
            }
            sD[t] = ri;
            sF1[t] = di;
        }
        __syncthreads();
        double asr = 0.0;
        if (T < kT)
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const int rw = tree_row<R>(T, j);
                if (vb * (kT * R) + rw < n) asr = fma(sD[rw] * (double)fabsf(sF1[rw]), sD[rw], asr);
            }
        const double ba = tree256(asr, sm);
        if (T == 0) pa[vb] = ba;
    }
    __syncthreads();
    if (T == 0 && sflags) atomicOr(&cs->signflags, sflags);
    aborted = !grid_sync(gb, ++epoch * G);
    // refinement state, meaningful in thread 0 only
    double sres = 0.0, sig = 1.0, isig = 1.0, res0 = 0.0, res = 0.0, tol = 0.0, rho = 0.0, rho_prev = 0.0,
           itol = 0.0;
    int total = 0, outer = 0, inner_it = 0, status = FVGB_OK;
    unsigned int flags = 0u;
    if (!aborted) {
        const double s2 = final_all(pa, nvb, sm, &cell);
        if (T == 0) {
            sres = sqrt(s2);
            flags = *(volatile unsigned int*)&cs->signflags;
        }
    }
    float* pcur = pbuf0;
    float* pnext = pbuf1;
    bool first = true;
    bool done = aborted;
    while (!done) {
        if (!first) {
            // x += y / sig
            const double is = sh.isig;
            for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
                for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
                    const int t = T + h * kPT;
                    const int i = vb * (kT * R) + t;
                    if (i < n) x[i] = fma((double)__ldcg(&y[i]), is, __ldcg(&x[i]));
                }
            }
            if (!grid_sync(gb, ++epoch * G)) {
                aborted = true;
                break;
            }
        }
        if (T == 0) {
            double nsig, nisig;
            residual_scale(sres, &nsig, &nisig);
            sh.nsig = nsig;
        }
        __syncthreads();
        const double nsig_all = sh.nsig;
        // residual: r = b - A x (FP64), rh = sign*(float)(sig r), y = 0, z = |dinv| rh
        for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
            for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
                const int t = T + h * kPT;
                const int i = vb * (kT * R) + t;
                double ri = 0.0;
                float di = 0.0f, rhi = 0.0f;
                if (i < n) {
                    ri = first ? __ldcg(&r0[i]) : __ldg(&b[i]) - spmv_row_cg(m, val, x, i);
                    di = __ldcg(&dinv[i]);
                    rhi = (float)(ri * nsig_all);
                    if (di < 0.0f) rhi = -rhi;
                    rh[i] = rhi;
                    y[i] = 0.0f;
                    const float zi = fabsf(di) * rhi;
                    z[i] = zi;
                    if (first) pcur[i] = zi;
                }
                sD[t] = ri;
                sF1[t] = rhi;
                sF2[t] = di;
            }
            __syncthreads();
            double arr = 0.0, asr = 0.0;
            float arho = 0.0f;
            if (T < kT)
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    const int rw = tree_row<R>(T, j);
                    if (vb * (kT * R) + rw >= n) continue;
                    const double rv = sD[rw];
                    arr = fma(rv, rv, arr);
                    asr = fma(rv * (double)fabsf(sF2[rw]), rv, asr);
                    arho = fmaf(sF1[rw], fabsf(sF2[rw]) * sF1[rw], arho);
                }
            const double ba = tree256(arr, sm), bc = tree256(asr, sm3);
            const float bb = tree256f(arho, smf);
            if (T == 0) {
                pa[vb] = ba;
                pb[vb] = (double)bb;
                pc[vb] = bc;
            }
        }
        if (!grid_sync(gb, ++epoch * G)) {
            aborted = true;
            break;
        }
        const double rr = final_all(pa, nvb, sm, &cell);
        const double nrho = final_all(pb, nvb, sm, &cell);
        const double sr2 = final_all(pc, nvb, sm, &cell);
        if (T == 0) {
            double nsig, nisig;
            residual_scale(sres, &nsig, &nisig);
            bool d = false;
            res = sqrt(rr);
            if (!first) outer += 1;
            if (first) {
                res0 = res;
                tol = prm.rel_tol * tol_base(&L.cases[0], res);
                if (prm.abs_tol > tol) tol = prm.abs_tol;
                if ((flags & 4u) || flags == 3u) {
                    status = FVGB_ERR_UNSUPPORTED;
                    d = true;
                }
            }
            if (!d) {
                if (!isfinite(res)) {
                    status = FVGB_ERR_BREAKDOWN;
                    d = true;
                } else if (!(res > tol) || res == 0.0) {
                    d = true;
                } else if (outer >= prm.max_outer || total >= prm.max_iter) {
                    status = FVGB_ERR_NOT_CONVERGED;
                    d = true;
                }
            }
            const double g = nsig * isig;
            const double rho_rec = rho * g * g;
            const bool restart = first || inner_it == 0 || nrho > 4.0 * rho_rec;
            const float frel = restart ? -1.0f : (float)((nrho / rho_prev) * (sig * nisig));
            sig = nsig;
            isig = nisig;
            sres = sqrt(sr2);
            rho = nrho;
            const double dr = prm.inner_rel_tol * prm.inner_rel_tol;
            const double dt = (tol / res) * (tol / res);
            itol = rho * (dr > dt ? dr : dt);
            inner_it = 0;
            sh.inner = !d && rho > itol && prm.inner_max_iter > 0 && total < prm.max_iter;
            sh.done = d;
            sh.isig = isig;
            sh.dm = first ? DirMode{0, 0.0f} : (frel < 0.0f ? DirMode{1, 0.0f} : DirMode{2, frel});
        }
        __syncthreads();
        first = false;
        done = sh.done;
        if (done) break;
        while (sh.inner) {
            const DirMode dm = sh.dm;
            // direction (into pnext unless p is taken as stored), q = A p, p.q
            for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
                for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
                    const int t = T + h * kPT;
                    const int i = vb * (kT * R) + t;
                    float pi = 0.0f, qi = 0.0f;
                    if (i < n) {
                        pi = dir_of(dm, __ldcg(&pcur[i]), dm.kind == 0 ? 0.0f : __ldcg(&z[i]));
                        if (dm.kind != 0) pnext[i] = pi;
                        qi = spmv_row_diff_dir(m, a32, pcur, z, dm, i, pi, __ldg(&ev[i]));
                        q[i] = qi;
                    }
                    sF1[t] = pi;
                    sF2[t] = qi;
                }
                __syncthreads();
                float acc = 0.0f;
                if (T < kT)
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int rw = tree_row<R>(T, j);
                        if (vb * (kT * R) + rw < n) acc = fmaf(sF1[rw], sF2[rw], acc);
                    }
                const float ba = tree256f(acc, smf);
                if (T == 0) pa[vb] = (double)ba;
            }
            if (dm.kind != 0) {
                float* t = pcur;
                pcur = pnext;
                pnext = t;
            }
            if (!grid_sync(gb, ++epoch * G)) {
                aborted = true;
                break;
            }
            const double pq = final_all(pa, nvb, sm, &cell);
            if (T == 0) {
                const double alpha = rho / pq;
                sh.brk = 0;
                if (pq == 0.0 || !isfinite(alpha)) {
                    sh.brk = 1;
                    sh.inner = 0;
                    if (inner_it == 0) {
                        status = FVGB_ERR_BREAKDOWN;
                        sh.done = 1;
                    }
                } else {
                    sh.fa = (float)alpha;
                }
            }
            __syncthreads();
            if (sh.brk) break;
            const float fa = sh.fa;
            // y += alpha p, rh -= alpha q, z = |dinv| rh, rh.z
            for (int vb = blockIdx.x; vb < nvb; vb += (int)G) {
                for (int h = 0; h < (kT * R / kPT); ++h) {  // the thread's rows T + h*kPT of the virtual block
                    const int t = T + h * kPT;
                    const int i = vb * (kT * R) + t;
                    float ri = 0.0f, zi = 0.0f;
                    if (i < n) {
                        y[i] = fmaf(fa, __ldcg(&pcur[i]), __ldcg(&y[i]));
                        ri = fmaf(-fa, __ldcg(&q[i]), __ldcg(&rh[i]));
                        rh[i] = ri;
                        zi = fabsf(__ldcg(&dinv[i])) * ri;
                        z[i] = zi;
                    }
                    sF1[t] = ri;
                    sF2[t] = zi;
                }
                __syncthreads();
                float acc = 0.0f;
                if (T < kT)
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int rw = tree_row<R>(T, j);
                        if (vb * (kT * R) + rw < n) acc = fmaf(sF1[rw], sF2[rw], acc);
                    }
                const float ba = tree256f(acc, smf);
                if (T == 0) pa[vb] = (double)ba;
            }
            if (!grid_sync(gb, ++epoch * G)) {
                aborted = true;
                break;
            }
            const double rhon = final_all(pa, nvb, sm, &cell);
            if (T == 0) {
                const float fbeta = (float)(rhon / rho);
                rho_prev = rho;
                rho = rhon;
                inner_it += 1;
                total += 1;
                sh.inner = rhon > itol && inner_it < prm.inner_max_iter && total < prm.max_iter;
                sh.dm = DirMode{2, fbeta};
            }
            __syncthreads();
        }
        if (aborted) break;
        done = sh.done;
    }
    if (blockIdx.x == 0 && T == 0) {
        cs->res0 = res0;
        cs->res = res;
        cs->iter = 0;
        cs->total = total;
        cs->outer = outer;
        cs->status = aborted ? FVGB_ERR_CUDA : status;
    }
}

// ---------------------------------------------------------------- graph glue
cudaError_t add_kernel_deps(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, size_t ndeps,
                            void* func, unsigned grid, unsigned block, void** args) {
    cudaKernelNodeParams kp{};
    kp.func = func;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(block);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    return cudaGraphAddKernelNode(node, g, deps, ndeps, &kp);
}

cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t* dep, void* func, unsigned grid,
                       unsigned block, void** args) {
    cudaKernelNodeParams kp{};
    kp.func = func;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(block);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    return cudaGraphAddKernelNode(node, g, dep, dep ? 1 : 0, &kp);
}

cudaError_t add_while(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t* dep, cudaGraphConditionalHandle h,
                      cudaGraph_t* body) {
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaError_t e = cudaGraphAddNode(node, g, dep, nullptr, dep ? 1 : 0, &np);
    if (e == cudaSuccess) *body = np.conditional.phGraph_out[0];
    return e;
}

}  // namespace

// A solve context: the block map of a set of cases on one linear system, the
// work vectors and the instantiated graphs.
struct SolverCache {
    const fvgb_ls* ls = nullptr;
    int n = 0, nb = 0, ncases = 0;
    bool whole = false;  // one case covering rows [0, n): the persistent kernels' assumption
    Layout L{};
    std::vector<void*> allocs;
    bool pooled = false;  // device memory from the serving pool (devmem_*)
    double *dinv = nullptr, *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr, *pa = nullptr, *pb = nullptr;
    double* pc = nullptr;
    float *ah = nullptr, *dinvf = nullptr, *ev = nullptr, *rh = nullptr, *y = nullptr, *pf = nullptr,
          *qf = nullptr;
    cudaGraphExec_t g64 = nullptr, gmix = nullptr, gbi = nullptr, gmb = nullptr;
    float *mb_rr = nullptr, *mb_yv = nullptr, *mb_t = nullptr;  // mixed BiCGStab (with rh, y, pf, qf, pf2, zf)
    double *bi_rr = nullptr, *bi_v = nullptr, *bi_y = nullptr, *bi_s = nullptr, *bi_t = nullptr;  // BiCGStab
    double *bg_r2 = nullptr, *bg_z2 = nullptr, *bg_p2 = nullptr, *bg_q2 = nullptr;                 // BiCG
    cudaGraphExec_t gbg = nullptr;
    fvgb_solver_stats* h_stats = nullptr;  // pinned [ncases]
    GridBar* bar = nullptr;
    float *pf2 = nullptr, *zf = nullptr;   // second direction buffer and z of the persistent mixed solve
    double* r0 = nullptr;                   // mixed: first FP64 residual, from the preparation kernel
    uint64_t converted_version = 0;        // fvgb_ls::version the FP32 matrix copy was formed from
    int pgrid_fp64 = 0, pgrid_mixed = 0;   // co-resident blocks of the persistent kernels (0: not asked yet)
    // chosen launch-bound variant per kernel kind; untuned solves (small systems,
    // FVGB_SOLVE_NO_TUNE) use the 128^3 heat system's choices: at least 8 resident
    // blocks per SM for the FP64 kernels and the FP32 update, 6 for the FP32 SpMV
    int variant[kTuneKinds] = {3, 3, 2, 3};
    int forced[kTuneKinds] = {-1, -1, -1, -1};
    int cached[kTuneKinds] = {-1, -1, -1, -1};  // from the tuning cache (tunecache.cpp), -1: none
    bool tuned64 = false, tunedmx = false;
    float tune_ms[kTuneKinds][kNumVariants] = {};
    int32_t* h_active = nullptr;           // pinned copy of n_active for the host-driven loop
};

struct fvgb_batch {
    SolverCache* c = nullptr;
};

void fvgb_solver_cache_free(SolverCache* c) {
    if (!c) return;
    if (c->g64) cudaGraphExecDestroy(c->g64);
    if (c->gmix) cudaGraphExecDestroy(c->gmix);
    if (c->gbi) cudaGraphExecDestroy(c->gbi);
    if (c->gmb) cudaGraphExecDestroy(c->gmb);
    if (c->gbg) cudaGraphExecDestroy(c->gbg);
    for (void* p : c->allocs) devmem_free(p, c->pooled);
    if (c->h_stats) {
        if (c->pooled) std::free(c->h_stats);  // cudaFreeHost would synchronise the device
        else cudaFreeHost(c->h_stats);
    }
    if (c->h_active) cudaFreeHost(c->h_active);
    delete c;
}

namespace {

template <class T>
cudaError_t calloc_dev(SolverCache* c, T** p, size_t count) {
    cudaError_t e = devmem_alloc((void**)p, sizeof(T) * (count ? count : 1), c->pooled);
    if (e == cudaSuccess) {
        c->allocs.push_back(*p);
        e = cudaMemset(*p, 0, sizeof(T) * (count ? count : 1));
    }
    return e;
}

// ranges: [2*ncases] begin/end rows of every case, validated by the caller
fvgb_status cache_create(const fvgb_ls* ls, int ncases, const int32_t* ranges, SolverCache** out) {
    SolverCache* c = new SolverCache();
    c->pooled = devmem_pooled_now();
    c->ls = ls;
    c->n = ls->mesh->v.n;
    c->ncases = ncases;
    c->whole = ncases == 1 && ranges[0] == 0 && ranges[1] == c->n;
    std::vector<int32_t> blk_case, blk_row0, case_end(ncases), case_blk0(ncases + 1), case_rpt(ncases);
    for (int k = 0; k < ncases; ++k) {
        case_blk0[k] = (int32_t)blk_case.size();
        case_end[k] = ranges[2 * k + 1];
        const int32_t nr = ranges[2 * k + 1] - ranges[2 * k];
        case_rpt[k] = rows_per_thread(nr);
        const int32_t rb = kT * case_rpt[k];
        const int32_t nbk = nr > 0 ? (nr + rb - 1) / rb : 1;  // an empty case gets one idle block
        for (int32_t b = 0; b < nbk; ++b) {
            blk_case.push_back(k);
            blk_row0.push_back(ranges[2 * k] + b * rb);
        }
    }
    case_blk0[ncases] = (int32_t)blk_case.size();
    c->nb = (int)blk_case.size();
    int32_t *d_bc = nullptr, *d_br = nullptr, *d_ce = nullptr, *d_cb = nullptr, *d_rpt = nullptr;
    cudaError_t e = calloc_dev(c, &d_bc, blk_case.size());
    if (e == cudaSuccess) e = calloc_dev(c, &d_rpt, case_rpt.size());
    if (e == cudaSuccess) e = cudaMemcpy(d_rpt, case_rpt.data(), 4 * case_rpt.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = calloc_dev(c, &d_br, blk_row0.size());
    if (e == cudaSuccess) e = calloc_dev(c, &d_ce, case_end.size());
    if (e == cudaSuccess) e = calloc_dev(c, &d_cb, case_blk0.size());
    if (e == cudaSuccess) e = cudaMemcpy(d_bc, blk_case.data(), 4 * blk_case.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_br, blk_row0.data(), 4 * blk_row0.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_ce, case_end.data(), 4 * case_end.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_cb, case_blk0.data(), 4 * case_blk0.size(), cudaMemcpyHostToDevice);
    CaseState* cs = nullptr;
    BatchState* bs = nullptr;
    fvgb_solver_stats* st = nullptr;
    if (e == cudaSuccess) e = calloc_dev(c, &cs, (size_t)ncases);
    if (e == cudaSuccess) e = calloc_dev(c, &bs, 1);
    if (e == cudaSuccess) e = calloc_dev(c, &st, (size_t)ncases);
    if (e == cudaSuccess) e = calloc_dev(c, &c->pa, (size_t)c->nb);
    if (e == cudaSuccess) e = calloc_dev(c, &c->pb, (size_t)c->nb);
    if (e == cudaSuccess) e = calloc_dev(c, &c->pc, (size_t)c->nb);
    if (e == cudaSuccess) {
        if (c->pooled) {  // pageable: released without the device synchronisation of cudaFreeHost
            c->h_stats = (fvgb_solver_stats*)std::malloc(sizeof(fvgb_solver_stats) * (size_t)ncases);
            if (!c->h_stats) e = cudaErrorMemoryAllocation;
        } else {
            e = cudaMallocHost(&c->h_stats, sizeof(fvgb_solver_stats) * (size_t)ncases);
        }
    }
    if (e == cudaSuccess) e = settle_creation();
    if (e != cudaSuccess) {
        fvgb_solver_cache_free(c);
        return cuda_fail(e, "solver workspace");
    }
    c->L = Layout{d_bc, d_br, d_ce, d_cb, cs, bs, st, d_rpt};
    *out = c;
    return FVGB_OK;
}

// ---------------------------------------------------------------- autotuner
// Median of 3 timed launches (after one untimed) of `fn` on a private stream.
float time_launch(const void* fn, unsigned grid, void** args, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1) {
    float best[3] = {0, 0, 0};
    cudaLaunchKernel(fn, dim3(grid), dim3(kT), args, 0, s);
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0, s);
        cudaLaunchKernel(fn, dim3(grid), dim3(kT), args, 0, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&best[r], e0, e1);
    }
    std::sort(best, best + 3);
    return best[1];
}

// Systems smaller than this keep the default variants (their solves run as a
// persistent kernel or are launch bound).
constexpr int kTuneMinRows = 1 << 18;

static_assert(kTuneKinds == kTuneCacheKinds && kNumVariants == kTuneCacheVariants, "tuning cache layout");
constexpr int kDefaultVariant[kTuneKinds] = {3, 3, 2, 3};

// the fastest measured variant of a kind, -1 when none was measured
int best_measured(const SolverCache* c, int kind) {
    int b = -1;
    for (int v = 0; v < kNumVariants; ++v)
        if (c->tune_ms[kind][v] > 0.0f && (b < 0 || c->tune_ms[kind][v] < c->tune_ms[kind][b])) b = v;
    return b;
}

// the variant in use: forced, else measured on this system, else cached for
// its shape, else the default
void pick(SolverCache* c, int kind) {
    const int b = best_measured(c, kind);
    c->variant[kind] = c->forced[kind] >= 0 ? c->forced[kind]
                       : b >= 0             ? b
                       : c->cached[kind] >= 0 ? c->cached[kind]
                                              : kDefaultVariant[kind];
}

// The shape a cached choice applies to: rows (nearest power of two), stored
// slots per row, 16- or 32-bit column offsets, and the GPU (compute capability
// and SM count).
std::string tune_key(const SolverCache* c) {
    int dev = 0, sms = 0, cmaj = 0, cmin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&cmaj, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&cmin, cudaDevAttrComputeCapabilityMinor, dev);
    const MeshView& m = c->ls->mesh->v;
    const int lg = c->n > 0 ? (int)std::lround(std::log2((double)c->n)) : 0;
    const long spr = c->n > 0 ? std::lround((double)c->ls->mesh->nnz / c->n) : 0;
    return "sm" + std::to_string(cmaj * 10 + cmin) + "x" + std::to_string(sms) + "/rows2^" + std::to_string(lg) +
           "/slots" + std::to_string(spr) + "/off" + (m.m_off ? "16" : "32");
}

// Looks the kinds [k0, k0 + 2) up in the tuning cache; true when both are known.
bool cache_lookup(SolverCache* c, const std::string& key, int k0) {
    int v0 = -1, v1 = -1;
    if (!tune_cache_get(key, k0, &v0) || !tune_cache_get(key, k0 + 1, &v1)) return false;
    c->cached[k0] = v0;
    c->cached[k0 + 1] = v1;
    return true;
}

// Times the FP64 SpMV and update variants on this system: CG iterations from a
// zero vector (a scratch x, never the caller's), the solver state reset by the
// next solve's parameter kernel.
fvgb_status tune_fp64(SolverCache* c, bool measure) {
    c->tuned64 = true;
    const std::string key = c->n >= kTuneMinRows ? tune_key(c) : std::string();
    const bool hit = !key.empty() && cache_lookup(c, key, kTuneSpmv64);
    if (measure && c->n >= kTuneMinRows && !hit) {
        FVGB_CUDA_TRY(cudaDeviceSynchronize());  // the system's assembly may still run on the caller's stream
        double* tmp = nullptr;
        cudaStream_t s = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaError_t e = cudaMalloc(&tmp, sizeof(double) * (size_t)c->n);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        if (e == cudaSuccess) e = cudaMemsetAsync(tmp, 0, sizeof(double) * (size_t)c->n, s);
        if (e == cudaSuccess) {
            SolverParams prm{};
            prm.x = tmp;
            prm.max_iter = 1 << 30;
            MeshView m = c->ls->mesh->v;
            Layout L = c->L;
            const double* val = c->ls->values;
            const double* b = c->ls->rhs;
            const cudaGraphConditionalHandle h{};
            int setc = 0;
            const unsigned nb = (unsigned)c->nb;
            k_set_params<<<grid_for(c->ncases, 128), 128, 0, s>>>(c->L, c->ncases, prm);
            k_pcg_init<<<nb, kT, 0, s>>>(c->L, m, val, b, c->dinv, c->r, c->p, c->pa, c->pb, h, 0);
            void* a_spmv[] = {&L, &m, &val, &c->p, &c->q, &c->pa};
            void* a_upd[] = {&L, &c->dinv, &c->p, &c->q, &c->r, &c->z, &c->pa, &c->pb, (void*)&h, &setc};
            for (int v = 0; v < kNumVariants; ++v)
                c->tune_ms[kTuneSpmv64][v] = time_launch(variant_fn(kTuneSpmv64, v), nb, a_spmv, s, e0, e1);
            for (int v = 0; v < kNumVariants; ++v)
                c->tune_ms[kTuneUpdate64][v] = time_launch(variant_fn(kTuneUpdate64, v), nb, a_upd, s, e0, e1);
            e = cudaStreamSynchronize(s);
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (s) cudaStreamDestroy(s);
        if (tmp) cudaFree(tmp);
        if (e != cudaSuccess) return cuda_fail(e, "FP64 CG autotuning");
        for (int k = kTuneSpmv64; k <= kTuneUpdate64; ++k) tune_cache_put(key, k, best_measured(c, k), c->tune_ms[k]);
    }
    pick(c, kTuneSpmv64);
    pick(c, kTuneUpdate64);
    return FVGB_OK;
}

// The FP64 solve as graph nodes in `g` after `deps`: init, a device-side while
// loop over (SpMV, update, direction), the statistics; *last = the final node.
cudaError_t add_fp64_nodes(SolverCache* c, cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps,
                           cudaGraphNode_t* last) {
    const fvgb_ls* ls = c->ls;
    MeshView m = ls->mesh->v;
    Layout L = c->L;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t n0, n1, b0, b1, b2;
    cudaGraph_t body;
    const double* val = ls->values;
    const double* b = ls->rhs;
    const unsigned nb = (unsigned)c->nb;
    int setc = 1;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    void* a_init[] = {&L, &m, &val, &b, &c->dinv, &c->r, &c->p, &c->pa, &c->pb, &h, &setc};
    void* a_spmv[] = {&L, &m, &val, &c->p, &c->q, &c->pa};
    void* a_upd[] = {&L, &c->dinv, &c->p, &c->q, &c->r, &c->z, &c->pa, &c->pb, &h, &setc};
    void* a_dir[] = {&L, &c->z, &c->p};
    void* a_fin[] = {&L};
    if (e == cudaSuccess) e = add_kernel_deps(g, &n0, deps, ndeps, (void*)k_pcg_init, nb, kT, a_init);
    if (e == cudaSuccess) e = add_while(g, &n1, &n0, h, &body);
    if (e == cudaSuccess)
        e = add_kernel(body, &b0, nullptr, (void*)variant_fn(kTuneSpmv64, c->variant[kTuneSpmv64]), nb, kT, a_spmv);
    if (e == cudaSuccess)
        e = add_kernel(body, &b1, &b0, (void*)variant_fn(kTuneUpdate64, c->variant[kTuneUpdate64]), nb, kT, a_upd);
    if (e == cudaSuccess) e = add_kernel(body, &b2, &b1, (void*)k_pcg_dir, nb, kT, a_dir);
    if (e == cudaSuccess) e = add_kernel(g, last, &n1, (void*)k_finish, grid_for(c->ncases, 128), 128, a_fin);
    return e;
}

fvgb_status graph_fp64(SolverCache* c) {
    if (c->g64) {
        cudaGraphExecDestroy(c->g64);
        c->g64 = nullptr;
    }
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphNode_t last;
    cudaError_t e = add_fp64_nodes(c, g, nullptr, 0, &last);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->g64, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "FP64 CG graph");
    return FVGB_OK;
}

fvgb_status build_fp64(SolverCache* c, bool measure = true) {
    const size_t n = (size_t)c->n;
    if (!c->dinv) {
        cudaError_t e = calloc_dev(c, &c->dinv, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->r, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->p, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->q, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->z, n);
        if (e == cudaSuccess) e = settle_creation();
        if (e != cudaSuccess) return cuda_fail(e, "FP64 CG workspace");
    }
    if (!c->tuned64) {
        fvgb_status st = tune_fp64(c, measure);
        if (st != FVGB_OK) return st;
    }
    return graph_fp64(c);
}

// Times the FP32 SpMV and update variants of the mixed solve on this system
// (after the preparation kernel, from a zero scratch vector).
fvgb_status tune_mixed(SolverCache* c, bool measure) {
    c->tunedmx = true;
    const std::string key = c->n >= kTuneMinRows ? tune_key(c) : std::string();
    const bool hit = !key.empty() && cache_lookup(c, key, kTuneSpmvMixed);
    if (measure && c->n >= kTuneMinRows && !hit) {
        FVGB_CUDA_TRY(cudaDeviceSynchronize());
        double* tmp = nullptr;
        cudaStream_t s = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaError_t e = cudaMalloc(&tmp, sizeof(double) * (size_t)c->n);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        if (e == cudaSuccess) e = cudaMemsetAsync(tmp, 0, sizeof(double) * (size_t)c->n, s);
        if (e == cudaSuccess) {
            SolverParams prm{};
            prm.x = tmp;
            prm.max_iter = 1 << 30;
            prm.inner_max_iter = 1 << 30;
            prm.max_outer = 1 << 30;
            prm.inner_rel_tol = 0.5;
            prm.convert = 1;
            MeshView m = c->ls->mesh->v;
            Layout L = c->L;
            const double* val = c->ls->values;
            const double* b = c->ls->rhs;
            const cudaGraphConditionalHandle h{};
            int setc = 0;
            const unsigned nb = (unsigned)c->nb;
            k_set_params<<<grid_for(c->ncases, 128), 128, 0, s>>>(c->L, c->ncases, prm);
            k_ir_prepare<<<nb, kT, 0, s>>>(c->L, m, val, b, c->ah, c->ev, c->dinvf, c->r0, c->pa);
            k_tune_mixed_state<<<nb, kT, 0, s>>>(c->L, c->pf, c->rh, c->y);
            void* a_spmv[] = {&L, &m, &c->ah, &c->ev, &c->pf, &c->qf, &c->pa};
            void* a_upd[] = {&L, &c->dinvf, &c->pf, &c->qf, &c->y, &c->rh, &c->pa, (void*)&h, &setc};
            for (int v = 0; v < kNumVariants; ++v)
                c->tune_ms[kTuneSpmvMixed][v] = time_launch(variant_fn(kTuneSpmvMixed, v), nb, a_spmv, s, e0, e1);
            for (int v = 0; v < kNumVariants; ++v)
                c->tune_ms[kTuneUpdateMixed][v] = time_launch(variant_fn(kTuneUpdateMixed, v), nb, a_upd, s, e0, e1);
            e = cudaStreamSynchronize(s);
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (s) cudaStreamDestroy(s);
        if (tmp) cudaFree(tmp);
        if (e != cudaSuccess) return cuda_fail(e, "mixed CG autotuning");
        for (int k = kTuneSpmvMixed; k <= kTuneUpdateMixed; ++k)
            tune_cache_put(key, k, best_measured(c, k), c->tune_ms[k]);
    }
    pick(c, kTuneSpmvMixed);
    pick(c, kTuneUpdateMixed);
    return FVGB_OK;
}

// The mixed-precision solve as graph nodes in `g` after `deps` (see add_fp64_nodes).
cudaError_t add_mixed_nodes(SolverCache* c, cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps,
                            cudaGraphNode_t* last) {
    const fvgb_ls* ls = c->ls;
    MeshView m = ls->mesh->v;
    Layout L = c->L;
    cudaGraphConditionalHandle ho, hi;
    const double* val = ls->values;
    const double* b = ls->rhs;
    const unsigned nb = (unsigned)c->nb;
    int setc = 1;
    cudaError_t e = cudaGraphConditionalHandleCreate(&ho, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hi, g, 0, cudaGraphCondAssignDefault);
    cudaGraphNode_t n_prep, n_res0, n_outer, o_inner, o_x, o_res, o_dir, i_spmv, i_upd, i_dir;
    cudaGraph_t obody = nullptr, ibody = nullptr;
    void* a_prep[] = {&L, &m, &val, &b, &c->ah, &c->ev, &c->dinvf, &c->r0, &c->pa};
    void* a_res[] = {&L, &m, &val, &b, &c->r0, &c->dinvf, &c->rh, &c->y, &c->pf, &c->pa, &c->pb, &c->pc, &ho, &hi};
    void* a_spmv[] = {&L, &m, &c->ah, &c->ev, &c->pf, &c->qf, &c->pa};
    void* a_upd[] = {&L, &c->dinvf, &c->pf, &c->qf, &c->y, &c->rh, &c->pa, &hi, &setc};
    void* a_dir[] = {&L, &c->dinvf, &c->rh, &c->pf};
    void* a_x[] = {&L, &c->y};
    void* a_rdir[] = {&L, &c->dinvf, &c->rh, &c->pf};
    void* a_fin[] = {&L};
    if (e == cudaSuccess) e = add_kernel_deps(g, &n_prep, deps, ndeps, (void*)k_ir_prepare, nb, kT, a_prep);
    if (e == cudaSuccess) e = add_kernel(g, &n_res0, &n_prep, (void*)k_ir_residual<true>, nb, kT, a_res);
    if (e == cudaSuccess) e = add_while(g, &n_outer, &n_res0, ho, &obody);
    if (e == cudaSuccess) e = add_while(obody, &o_inner, nullptr, hi, &ibody);
    if (e == cudaSuccess)
        e = add_kernel(ibody, &i_spmv, nullptr, (void*)variant_fn(kTuneSpmvMixed, c->variant[kTuneSpmvMixed]), nb,
                       kT, a_spmv);
    if (e == cudaSuccess)
        e = add_kernel(ibody, &i_upd, &i_spmv, (void*)variant_fn(kTuneUpdateMixed, c->variant[kTuneUpdateMixed]),
                       nb, kT, a_upd);
    if (e == cudaSuccess) e = add_kernel(ibody, &i_dir, &i_upd, (void*)k_ir_dir, nb, kT, a_dir);
    if (e == cudaSuccess) e = add_kernel(obody, &o_x, &o_inner, (void*)k_ir_xupdate, nb, kT, a_x);
    if (e == cudaSuccess) e = add_kernel(obody, &o_res, &o_x, (void*)k_ir_residual<false>, nb, kT, a_res);
    if (e == cudaSuccess) e = add_kernel(obody, &o_dir, &o_res, (void*)k_ir_reliable_dir, nb, kT, a_rdir);
    if (e == cudaSuccess) e = add_kernel(g, last, &n_outer, (void*)k_finish, grid_for(c->ncases, 128), 128, a_fin);
    return e;
}

fvgb_status graph_mixed(SolverCache* c) {
    if (c->gmix) {
        cudaGraphExecDestroy(c->gmix);
        c->gmix = nullptr;
    }
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphNode_t last;
    cudaError_t e = add_mixed_nodes(c, g, nullptr, 0, &last);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gmix, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "mixed CG graph");
    return FVGB_OK;
}

fvgb_status alloc_mixed(SolverCache* c) {
    const size_t n = (size_t)c->n;
    if (!c->ah) {
        cudaError_t e = calloc_dev(c, &c->ah, (size_t)c->ls->mesh->m_len);
        if (e == cudaSuccess) e = calloc_dev(c, &c->dinvf, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->ev, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->rh, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->y, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->pf, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->qf, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->pf2, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->zf, n);
        if (e == cudaSuccess) e = calloc_dev(c, &c->r0, n);
        if (e == cudaSuccess) e = settle_creation();
        if (e != cudaSuccess) return cuda_fail(e, "mixed CG workspace");
    }
    return FVGB_OK;
}

fvgb_status build_mixed(SolverCache* c, bool measure = true) {
    fvgb_status ast = alloc_mixed(c);
    if (ast != FVGB_OK) return ast;
    if (!c->tunedmx) {
        fvgb_status st = tune_mixed(c, measure);
        if (st != FVGB_OK) return st;
    }
    return graph_mixed(c);
}

// The BiCGStab solve as graph nodes in `g` after `deps` (see add_fp64_nodes).
cudaError_t add_bicgstab_nodes(SolverCache* c, cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps,
                               cudaGraphNode_t* last) {
    const fvgb_ls* ls = c->ls;
    MeshView m = ls->mesh->v;
    Layout L = c->L;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t n0, n1, b0, b1, b2, b3, b4;
    cudaGraph_t body;
    const double* val = ls->values;
    const double* b = ls->rhs;
    const unsigned nb = (unsigned)c->nb;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    // r, p, z: the CG vectors; rr, v, y, s, t: BiCGStab's own
    void* a_init[] = {&L, &m, &val, &b, &c->dinv, &c->r, &c->bi_rr, &c->p, &c->bi_v, &c->pa, &h};
    void* a_dir[] = {&L, &c->dinv, &c->r, &c->bi_v, &c->p, &c->bi_y};
    void* a_sp1[] = {&L, &m, &val, &c->bi_y, &c->bi_rr, &c->bi_v, &c->pa};
    void* a_s[] = {&L, &c->dinv, &c->r, &c->bi_v, &c->bi_s, &c->z, &c->pa};
    void* a_sp2[] = {&L, &m, &val, &c->z, &c->bi_s, &c->bi_y, &c->bi_t, &c->pa, &c->pb};
    void* a_upd[] = {&L, &c->bi_y, &c->z, &c->bi_s, &c->bi_t, &c->bi_rr, &c->r, &c->pa, &c->pb, &h};
    void* a_fin[] = {&L};
    if (e == cudaSuccess) e = add_kernel_deps(g, &n0, deps, ndeps, (void*)k_bi_init, nb, kT, a_init);
    if (e == cudaSuccess) e = add_while(g, &n1, &n0, h, &body);
    if (e == cudaSuccess) e = add_kernel(body, &b0, nullptr, (void*)k_bi_dir, nb, kT, a_dir);
    if (e == cudaSuccess) e = add_kernel(body, &b1, &b0, (void*)k_bi_spmv1, nb, kT, a_sp1);
    if (e == cudaSuccess) e = add_kernel(body, &b2, &b1, (void*)k_bi_s, nb, kT, a_s);
    if (e == cudaSuccess) e = add_kernel(body, &b3, &b2, (void*)k_bi_spmv2, nb, kT, a_sp2);
    if (e == cudaSuccess) e = add_kernel(body, &b4, &b3, (void*)k_bi_update, nb, kT, a_upd);
    if (e == cudaSuccess) e = add_kernel(g, last, &n1, (void*)k_finish, grid_for(c->ncases, 128), 128, a_fin);
    return e;
}

fvgb_status build_bicgstab(SolverCache* c) {
    const size_t n = (size_t)c->n;
    cudaError_t e = cudaSuccess;
    if (!c->dinv) e = calloc_dev(c, &c->dinv, n);
    if (e == cudaSuccess && !c->r) e = calloc_dev(c, &c->r, n);
    if (e == cudaSuccess && !c->p) e = calloc_dev(c, &c->p, n);
    if (e == cudaSuccess && !c->z) e = calloc_dev(c, &c->z, n);
    if (e == cudaSuccess && !c->bi_rr) e = calloc_dev(c, &c->bi_rr, n);
    if (e == cudaSuccess && !c->bi_v) e = calloc_dev(c, &c->bi_v, n);
    if (e == cudaSuccess && !c->bi_y) e = calloc_dev(c, &c->bi_y, n);
    if (e == cudaSuccess && !c->bi_s) e = calloc_dev(c, &c->bi_s, n);
    if (e == cudaSuccess && !c->bi_t) e = calloc_dev(c, &c->bi_t, n);
    if (e == cudaSuccess) e = settle_creation();
    if (e != cudaSuccess) return cuda_fail(e, "BiCGStab workspace");
    if (c->gbi) {
        cudaGraphExecDestroy(c->gbi);
        c->gbi = nullptr;
    }
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphNode_t last;
    e = add_bicgstab_nodes(c, g, nullptr, 0, &last);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gbi, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "BiCGStab graph");
    return FVGB_OK;
}

// The BiCG solve as graph nodes in `g` after `deps` (see add_fp64_nodes).
cudaError_t add_bicg_nodes(SolverCache* c, cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps,
                           cudaGraphNode_t* last) {
    const fvgb_ls* ls = c->ls;
    MeshView m = ls->mesh->v;
    Layout L = c->L;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t n0, n1, b0, b1, b2;
    cudaGraph_t body;
    const double* val = ls->values;
    const double* b = ls->rhs;
    const unsigned nb = (unsigned)c->nb;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    void* a_init[] = {&L, &m, &val, &b, &c->dinv, &c->r, &c->bg_r2, &c->z, &c->bg_z2, &c->p, &c->bg_p2,
                      &c->pa, &c->pb, &h};
    void* a_dir[] = {&L, &c->z, &c->bg_z2, &c->p, &c->bg_p2};
    void* a_spmv[] = {&L, &m, &val, &c->p, &c->bg_p2, &c->q, &c->bg_q2, &c->pa};
    void* a_upd[] = {&L, &c->dinv, &c->p, &c->q, &c->bg_q2, &c->r, &c->bg_r2, &c->z, &c->bg_z2, &c->pa, &c->pb, &h};
    void* a_fin[] = {&L};
    if (e == cudaSuccess) e = add_kernel_deps(g, &n0, deps, ndeps, (void*)k_bg_init, nb, kT, a_init);
    if (e == cudaSuccess) e = add_while(g, &n1, &n0, h, &body);
    if (e == cudaSuccess) e = add_kernel(body, &b0, nullptr, (void*)k_bg_dir, nb, kT, a_dir);
    if (e == cudaSuccess) e = add_kernel(body, &b1, &b0, (void*)k_bg_spmv, nb, kT, a_spmv);
    if (e == cudaSuccess) e = add_kernel(body, &b2, &b1, (void*)k_bg_update, nb, kT, a_upd);
    if (e == cudaSuccess) e = add_kernel(g, last, &n1, (void*)k_finish, grid_for(c->ncases, 128), 128, a_fin);
    return e;
}

fvgb_status build_bicg(SolverCache* c) {
    const size_t n = (size_t)c->n;
    cudaError_t e = cudaSuccess;
    if (!c->dinv) e = calloc_dev(c, &c->dinv, n);
    if (e == cudaSuccess && !c->r) e = calloc_dev(c, &c->r, n);
    if (e == cudaSuccess && !c->p) e = calloc_dev(c, &c->p, n);
    if (e == cudaSuccess && !c->q) e = calloc_dev(c, &c->q, n);
    if (e == cudaSuccess && !c->z) e = calloc_dev(c, &c->z, n);
    if (e == cudaSuccess && !c->bg_r2) e = calloc_dev(c, &c->bg_r2, n);
    if (e == cudaSuccess && !c->bg_z2) e = calloc_dev(c, &c->bg_z2, n);
    if (e == cudaSuccess && !c->bg_p2) e = calloc_dev(c, &c->bg_p2, n);
    if (e == cudaSuccess && !c->bg_q2) e = calloc_dev(c, &c->bg_q2, n);
    if (e == cudaSuccess) e = settle_creation();
    if (e != cudaSuccess) return cuda_fail(e, "BiCG workspace");
    if (c->gbg) {
        cudaGraphExecDestroy(c->gbg);
        c->gbg = nullptr;
    }
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphNode_t last;
    e = add_bicg_nodes(c, g, nullptr, 0, &last);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gbg, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "BiCG graph");
    return FVGB_OK;
}

// The mixed-precision BiCGStab as graph nodes in `g` after `deps`: the
// preparation of the FP32 system, the first refinement step, then
// while (refining) { while (inner) { dir, spmv1, s, spmv2, update }; x += e/sig;
// refinement step }.  Vectors: rh = r, y = e, pf = p, qf = v, pf2 = s, zf = z.
cudaError_t add_mixed_bicgstab_nodes(SolverCache* c, cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps,
                                     cudaGraphNode_t* last) {
    const fvgb_ls* ls = c->ls;
    MeshView m = ls->mesh->v;
    Layout L = c->L;
    cudaGraphConditionalHandle ho, hi;
    const double* val = ls->values;
    const double* b = ls->rhs;
    const unsigned nb = (unsigned)c->nb;
    cudaError_t e = cudaGraphConditionalHandleCreate(&ho, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hi, g, 0, cudaGraphCondAssignDefault);
    cudaGraphNode_t n_prep, n_res0, n_outer, o_inner, o_x, o_res, i0, i1, i2, i3, i4;
    cudaGraph_t obody = nullptr, ibody = nullptr;
    void* a_prep[] = {&L, &m, &val, &b, &c->ah, &c->ev, &c->dinvf, &c->r0, &c->pa};
    void* a_res[] = {&L,     &m,     &val,  &b,     &c->r0, &c->dinvf, &c->rh, &c->mb_rr,
                     &c->pf, &c->qf, &c->y, &c->pa, &c->pb, &c->pc,    &ho,    &hi};
    void* a_dir[] = {&L, &c->dinvf, &c->rh, &c->qf, &c->pf, &c->mb_yv};
    void* a_sp1[] = {&L, &m, &c->ah, &c->ev, &c->mb_yv, &c->mb_rr, &c->qf, &c->pa};
    void* a_s[] = {&L, &c->dinvf, &c->rh, &c->qf, &c->pf2, &c->zf, &c->pa};
    void* a_sp2[] = {&L, &m, &c->ah, &c->ev, &c->zf, &c->pf2, &c->mb_yv, &c->mb_t, &c->y, &c->pa, &c->pb};
    void* a_upd[] = {&L, &c->mb_yv, &c->zf, &c->pf2, &c->mb_t, &c->mb_rr, &c->rh, &c->y, &c->pa, &c->pb, &hi};
    void* a_x[] = {&L, &c->y};
    void* a_fin[] = {&L};
    if (e == cudaSuccess) e = add_kernel_deps(g, &n_prep, deps, ndeps, (void*)k_ir_prepare, nb, kT, a_prep);
    if (e == cudaSuccess) e = add_kernel(g, &n_res0, &n_prep, (void*)k_mb_residual<true>, nb, kT, a_res);
    if (e == cudaSuccess) e = add_while(g, &n_outer, &n_res0, ho, &obody);
    if (e == cudaSuccess) e = add_while(obody, &o_inner, nullptr, hi, &ibody);
    if (e == cudaSuccess) e = add_kernel(ibody, &i0, nullptr, (void*)k_mb_dir, nb, kT, a_dir);
    if (e == cudaSuccess) e = add_kernel(ibody, &i1, &i0, (void*)k_mb_spmv1, nb, kT, a_sp1);
    if (e == cudaSuccess) e = add_kernel(ibody, &i2, &i1, (void*)k_mb_s, nb, kT, a_s);
    if (e == cudaSuccess) e = add_kernel(ibody, &i3, &i2, (void*)k_mb_spmv2, nb, kT, a_sp2);
    if (e == cudaSuccess) e = add_kernel(ibody, &i4, &i3, (void*)k_mb_update, nb, kT, a_upd);
    if (e == cudaSuccess) e = add_kernel(obody, &o_x, &o_inner, (void*)k_ir_xupdate, nb, kT, a_x);
    if (e == cudaSuccess) e = add_kernel(obody, &o_res, &o_x, (void*)k_mb_residual<false>, nb, kT, a_res);
    if (e == cudaSuccess) e = add_kernel(g, last, &n_outer, (void*)k_finish, grid_for(c->ncases, 128), 128, a_fin);
    return e;
}

fvgb_status build_mixed_bicgstab(SolverCache* c) {
    fvgb_status st = alloc_mixed(c);
    if (st != FVGB_OK) return st;
    const size_t n = (size_t)c->n;
    cudaError_t e = cudaSuccess;
    if (!c->mb_rr) e = calloc_dev(c, &c->mb_rr, n);
    if (e == cudaSuccess && !c->mb_yv) e = calloc_dev(c, &c->mb_yv, n);
    if (e == cudaSuccess && !c->mb_t) e = calloc_dev(c, &c->mb_t, n);
    if (e == cudaSuccess) e = settle_creation();
    if (e != cudaSuccess) return cuda_fail(e, "mixed BiCGStab workspace");
    if (c->gmb) {
        cudaGraphExecDestroy(c->gmb);
        c->gmb = nullptr;
    }
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphNode_t last;
    e = add_mixed_bicgstab_nodes(c, g, nullptr, 0, &last);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gmb, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "mixed BiCGStab graph");
    return FVGB_OK;
}

fvgb_status check_cfg(const fvgb_solver_cfg* cfg) {
    FVGB_CHECK_ARG(cfg->precision == FVGB_PREC_FP64 || cfg->precision == FVGB_PREC_MIXED_IR,
                   "fvgb_solve: unknown precision");
    FVGB_CHECK_ARG(cfg->rel_tol >= 0 && cfg->abs_tol >= 0, "fvgb_solve: negative tolerance");
    FVGB_CHECK_ARG(cfg->max_iter >= 0 && cfg->max_iter <= 100000000, "fvgb_solve: bad max_iter");
    FVGB_CHECK_ARG(cfg->kernel_mode >= 0 && cfg->kernel_mode <= 3, "fvgb_solve: bad kernel_mode");
    FVGB_CHECK_ARG((cfg->flags & ~(FVGB_SOLVE_NO_TUNE | FVGB_SOLVE_RHS_BASELINE)) == 0, "fvgb_solve: unknown flags");
    if (cfg->method == FVGB_SOLVER_MULTIGRID)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED,
                         "fvgb_solve: the multigrid solver solves single systems through fvgb_solve only");
    FVGB_CHECK_ARG(cfg->method == FVGB_SOLVER_CG || cfg->method == FVGB_SOLVER_BICGSTAB ||
                       cfg->method == FVGB_SOLVER_BICG,
                   "fvgb_solve: unknown method");
    if (cfg->method != FVGB_SOLVER_CG)
        FVGB_CHECK_ARG(cfg->kernel_mode != 3, "fvgb_solve: the host-driven loop is CG only");
    if (cfg->method == FVGB_SOLVER_BICG && cfg->precision != FVGB_PREC_FP64)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_solve: BiCG is FP64 only");
    FVGB_CHECK_ARG(cfg->kernel_mode != 3 || cfg->precision == FVGB_PREC_FP64,
                   "fvgb_solve: the host-driven loop (kernel_mode 3) is FP64 only");
    if (cfg->precision == FVGB_PREC_MIXED_IR)
        FVGB_CHECK_ARG(cfg->inner_rel_tol > 0 && cfg->inner_rel_tol < 1 && cfg->inner_max_iter > 0 &&
                           cfg->max_outer > 0,
                       "fvgb_solve: mixed precision needs inner_rel_tol in (0,1), inner_max_iter > 0, max_outer > 0");
    return FVGB_OK;
}

// Single-case solves of small systems run as one persistent cooperative kernel
// (launch latency dominates their iterations); everything else runs the graph.
// cfg->kernel_mode: 0 automatic, 1 graph, 2 persistent when possible,
// 3 host-driven loop (see host_loop).
int persistent_grid(SolverCache* c, bool mixed) {
    int& g = mixed ? c->pgrid_mixed : c->pgrid_fp64;
    if (g == 0) {
        int dev = 0, sms = 0, per_sm = 0, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ir_persistent<8>, kPT, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_persistent<8>, kPT, 0);
        g = (!coop || per_sm <= 0) ? -1 : sms * per_sm;
    }
    return g;
}

bool use_persistent(SolverCache* c, const fvgb_solver_cfg* cfg) {
    if (!c->whole || cfg->kernel_mode == 1 || cfg->kernel_mode == 3) return false;
    if (cfg->kernel_mode != 2 && c->n > (1 << 20)) return false;
    if (persistent_grid(c, cfg->precision == FVGB_PREC_MIXED_IR) <= 0) return false;
    if (!c->bar) {
        if (devmem_alloc((void**)&c->bar, sizeof(GridBar), c->pooled) != cudaSuccess) {
            c->bar = nullptr;
            return false;
        }
        c->allocs.push_back(c->bar);
    }
    return true;
}

// FP64 CG driven from the host: three launches per iteration and a read of the
// number of unconverged cases after each, the way a solver that evaluates its
// stopping criterion on the host runs (Ginkgo's CG checks its criteria between
// iterations).  Same kernels in the same order as the graph, so the same bits;
// it blocks the calling thread until the solve ends.  Kept as the plain-launch
// baseline the graph and the persistent kernel are measured against.
fvgb_status host_loop(SolverCache* c, cudaStream_t s) {
    if (!c->h_active) FVGB_CUDA_TRY(cudaMallocHost(&c->h_active, sizeof(int32_t)));
    const MeshView m = c->ls->mesh->v;
    const double* val = c->ls->values;
    const double* b = c->ls->rhs;
    const unsigned nb = (unsigned)c->nb;
    const cudaGraphConditionalHandle h{};  // not used: setc = 0 outside a graph
    k_pcg_init<<<nb, kT, 0, s>>>(c->L, m, val, b, c->dinv, c->r, c->p, c->pa, c->pb, h, 0);
    FVGB_LAUNCH_CHECK("fvgb_solve: init");
    for (;;) {
        FVGB_CUDA_TRY(cudaMemcpyAsync(c->h_active, &c->L.bs->n_active, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        FVGB_CUDA_TRY(cudaStreamSynchronize(s));
        if (*c->h_active <= 0) break;  // the update kernel retires every case by max_iter at the latest
        launch_variant(variant_fn(kTuneSpmv64, c->variant[kTuneSpmv64]), nb, s, c->L, m, val, (const double*)c->p,
                       c->q, c->pa);
        launch_variant(variant_fn(kTuneUpdate64, c->variant[kTuneUpdate64]), nb, s, c->L, (const double*)c->dinv,
                       (const double*)c->p, (const double*)c->q, c->r, c->z, c->pa, c->pb, h, 0);
        k_pcg_dir<<<nb, kT, 0, s>>>(c->L, c->z, c->p);
        FVGB_LAUNCH_CHECK("fvgb_solve: iteration");
    }
    k_finish<<<grid_for(c->ncases, 128), 128, 0, s>>>(c->L);
    FVGB_LAUNCH_CHECK("fvgb_solve: finish");
    return FVGB_OK;
}

fvgb_status launch(SolverCache* c, double* x, const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats_dev,
                   cudaStream_t s) {
    fvgb_status stt = check_cfg(cfg);
    if (stt != FVGB_OK) return stt;
    const bool measure = !(cfg->flags & FVGB_SOLVE_NO_TUNE);
    const bool mixed_ir = cfg->precision == FVGB_PREC_MIXED_IR;
    if (cfg->method == FVGB_SOLVER_BICGSTAB && !mixed_ir && !c->gbi) {
        stt = build_bicgstab(c);
        if (stt != FVGB_OK) return stt;
    }
    if (cfg->method == FVGB_SOLVER_BICGSTAB && mixed_ir && !c->gmb) {
        stt = build_mixed_bicgstab(c);
        if (stt != FVGB_OK) return stt;
    }
    if (cfg->method == FVGB_SOLVER_BICG && !c->gbg) {
        stt = build_bicg(c);
        if (stt != FVGB_OK) return stt;
    }
    if (cfg->method == FVGB_SOLVER_CG && cfg->precision == FVGB_PREC_FP64 && !c->g64) {
        stt = build_fp64(c, measure);
        if (stt != FVGB_OK) return stt;
    }
    if (cfg->method == FVGB_SOLVER_CG && cfg->precision == FVGB_PREC_MIXED_IR && !c->gmix) {
        stt = build_mixed(c, measure);
        if (stt != FVGB_OK) return stt;
    }
    SolverParams prm{};
    prm.x = x;
    prm.stats_out = stats_dev;
    prm.rel_tol = cfg->rel_tol;
    prm.abs_tol = cfg->abs_tol;
    prm.inner_rel_tol = cfg->inner_rel_tol;
    prm.max_iter = cfg->max_iter;
    prm.inner_max_iter = cfg->inner_max_iter;
    prm.max_outer = cfg->max_outer;
    prm.convert = c->converted_version != c->ls->version ? 1 : 0;
    if (cfg->precision == FVGB_PREC_MIXED_IR) c->converted_version = c->ls->version;
    k_set_params<<<grid_for(c->ncases, 128), 128, 0, s>>>(c->L, c->ncases, prm);
    if (cfg->flags & FVGB_SOLVE_RHS_BASELINE) k_case_bnorm<<<c->nb, kT, 0, s>>>(c->L, c->ls->rhs, c->pa);
    FVGB_LAUNCH_CHECK("fvgb_solve: parameters");
    if (cfg->method == FVGB_SOLVER_BICGSTAB) {
        FVGB_CUDA_TRY(cudaGraphLaunch(mixed_ir ? c->gmb : c->gbi, s));
        return FVGB_OK;
    }
    if (cfg->method == FVGB_SOLVER_BICG) {
        FVGB_CUDA_TRY(cudaGraphLaunch(c->gbg, s));
        return FVGB_OK;
    }
    if (cfg->kernel_mode == 3) return host_loop(c, s);
    if (use_persistent(c, cfg)) {
        MeshView m = c->ls->mesh->v;
        Layout L = c->L;
        const double* val = c->ls->values;
        const double* b = c->ls->rhs;
        int nvb = c->nb;
        const bool mixed = cfg->precision == FVGB_PREC_MIXED_IR;
        const int pg = persistent_grid(c, mixed);
        const int grid = nvb < pg ? nvb : pg;
        FVGB_CUDA_TRY(cudaMemsetAsync(c->bar, 0, sizeof(GridBar), s));
        if (mixed) {
            // k_ir_persistent(L, m, val, b, a32, ev, dinv, r0, rh, y, pbuf0, pbuf1, z, q, pa, pb, pc, gb, nvb)
            void* args[] = {&L,     &m,    &val,   &b,     &c->ah, &c->ev, &c->dinvf, &c->r0, &c->rh, &c->y,
                            &c->pf, &c->pf2, &c->zf, &c->qf, &c->pa, &c->pb, &c->pc,   &c->bar, &nvb};
            const void* fn = rows_per_thread(c->n) == 8 ? (const void*)k_ir_persistent<8> : (const void*)k_ir_persistent<4>;
            FVGB_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kPT), args, 0, s));
        } else {
            void* args[] = {&L, &m, &val, &b, &c->dinv, &c->r, &c->p, &c->q, &c->z, &c->pa, &c->pb, &c->bar, &nvb};
            const void* fn = rows_per_thread(c->n) == 8 ? (const void*)k_pcg_persistent<8> : (const void*)k_pcg_persistent<4>;
            FVGB_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kPT), args, 0, s));
        }
        k_finish<<<grid_for(c->ncases, 128), 128, 0, s>>>(c->L);
        FVGB_LAUNCH_CHECK("fvgb_solve: finish");
        return FVGB_OK;
    }
    FVGB_CUDA_TRY(cudaGraphLaunch(cfg->precision == FVGB_PREC_FP64 ? c->g64 : c->gmix, s));
    return FVGB_OK;
}

fvgb_status single_cache(fvgb_ls* ls, SolverCache** out) {
    if (!ls->solver) {
        int32_t range[2] = {0, ls->mesh->v.n};
        fvgb_status st = cache_create(ls, 1, range, &ls->solver);
        if (st != FVGB_OK) return st;
    }
    *out = ls->solver;
    return FVGB_OK;
}

fvgb_status status_of(const fvgb_solver_stats* st, int ncases) {
    int worst = FVGB_OK;
    for (int k = 0; k < ncases; ++k) {
        const int r = st[k].status;
        if (r == FVGB_ERR_UNSUPPORTED) worst = FVGB_ERR_UNSUPPORTED;
        else if (r == FVGB_ERR_BREAKDOWN && worst != FVGB_ERR_UNSUPPORTED) worst = FVGB_ERR_BREAKDOWN;
        else if (r == FVGB_ERR_NOT_CONVERGED && worst == FVGB_OK) worst = FVGB_ERR_NOT_CONVERGED;
    }
    if (worst == FVGB_ERR_UNSUPPORTED)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_solve: mixed precision needs diagonals of one sign");
    if (worst == FVGB_ERR_BREAKDOWN) return fvgb_fail(FVGB_ERR_BREAKDOWN, "fvgb_solve: breakdown");
    if (worst == FVGB_ERR_NOT_CONVERGED) return fvgb_fail(FVGB_ERR_NOT_CONVERGED, "fvgb_solve: iteration cap reached");
    return FVGB_OK;
}

fvgb_status sync_stats(SolverCache* c, fvgb_solver_stats* stats, cudaStream_t s) {
    FVGB_CUDA_TRY(cudaMemcpyAsync(c->h_stats, c->L.stats, sizeof(fvgb_solver_stats) * (size_t)c->ncases,
                                  cudaMemcpyDeviceToHost, s));
    FVGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (stats)
        for (int k = 0; k < c->ncases; ++k) stats[k] = c->h_stats[k];
    return status_of(c->h_stats, c->ncases);
}

}  // namespace

namespace {
// multigrid as CG's preconditioner or as the solver: amg.cu
bool uses_multigrid(const fvgb_solver_cfg* cfg) {
    return cfg->preconditioner == FVGB_PRECOND_MULTIGRID || cfg->method == FVGB_SOLVER_MULTIGRID;
}
// (the multigrid solver does not use `preconditioner`, so it takes precedence over ILU)
}  // namespace

extern "C" fvgb_status fvgb_solve_async(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg,
                                        fvgb_solver_stats* stats_dev, fvgb_stream stream) {
    FVGB_CHECK_ARG(ls && x && cfg, "fvgb_solve: null argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_solve: scalar systems only");
    FVGB_CHECK_ARG(cfg->preconditioner == FVGB_PRECOND_JACOBI || cfg->preconditioner == FVGB_PRECOND_MULTIGRID ||
                       cfg->preconditioner == FVGB_PRECOND_ILU,
                   "fvgb_solve: unknown preconditioner");
    if (uses_multigrid(cfg)) return fvgb_amg_solve_async(ls, x, cfg, stats_dev, (cudaStream_t)stream);
    if (cfg->preconditioner == FVGB_PRECOND_ILU) return fvgb_ilu_solve_async(ls, x, cfg, stats_dev, (cudaStream_t)stream);
    SolverCache* c = nullptr;
    fvgb_status st = single_cache(ls, &c);
    if (st != FVGB_OK) return st;
    return launch(c, x, cfg, stats_dev, (cudaStream_t)stream);
}

extern "C" fvgb_status fvgb_solve(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats,
                                  fvgb_stream stream) {
    fvgb_status st = fvgb_solve_async(ls, x, cfg, nullptr, stream);
    if (st != FVGB_OK) return st;
    if (uses_multigrid(cfg)) return fvgb_amg_sync_stats(ls, stats, (cudaStream_t)stream);
    if (cfg->preconditioner == FVGB_PRECOND_ILU) return fvgb_ilu_sync_stats(ls, stats, (cudaStream_t)stream);
    return sync_stats(ls->solver, stats, (cudaStream_t)stream);
}

extern "C" fvgb_status fvgb_batch_create(fvgb_ls* ls, int32_t ncases, const int32_t* row_ranges,
                                         fvgb_batch** out) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(ls && row_ranges && out, "fvgb_batch_create: null argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_batch_create: scalar systems only");
    FVGB_CHECK_ARG(ncases > 0, "fvgb_batch_create: no cases");
    for (int k = 0; k < ncases; ++k) {
        FVGB_CHECK_ARG(row_ranges[2 * k] >= 0 && row_ranges[2 * k] <= row_ranges[2 * k + 1] &&
                           row_ranges[2 * k + 1] <= ls->mesh->v.n,
                       "fvgb_batch_create: case rows outside the system");
        FVGB_CHECK_ARG(k == 0 || row_ranges[2 * k] >= row_ranges[2 * k - 1],
                       "fvgb_batch_create: cases must be in row order without overlap");
    }
    SolverCache* c = nullptr;
    fvgb_status st = cache_create(ls, ncases, row_ranges, &c);
    if (st != FVGB_OK) return st;
    fvgb_batch* b = new fvgb_batch();
    b->c = c;
    *out = b;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_batch_destroy(fvgb_batch* b) {
    if (!b) return FVGB_OK;
    cudaDeviceSynchronize();
    fvgb_solver_cache_free(b->c);
    delete b;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_batch_solve_async(fvgb_batch* b, double* x, const fvgb_solver_cfg* cfg,
                                              fvgb_solver_stats* stats_dev, fvgb_stream stream) {
    FVGB_CHECK_ARG(b && x && cfg, "fvgb_batch_solve: null argument");
    if (cfg->preconditioner != FVGB_PRECOND_JACOBI)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_batch_solve: the multigrid preconditioner solves single systems only");
    return launch(b->c, x, cfg, stats_dev, (cudaStream_t)stream);
}

extern "C" fvgb_status fvgb_batch_solve(fvgb_batch* b, double* x, const fvgb_solver_cfg* cfg,
                                        fvgb_solver_stats* stats, fvgb_stream stream) {
    fvgb_status st = fvgb_batch_solve_async(b, x, cfg, nullptr, stream);
    if (st != FVGB_OK) return st;
    return sync_stats(b->c, stats, (cudaStream_t)stream);
}

// ------------------------------------------------------------- step graphs
struct fvgb_step {
    cudaGraphExec_t exec = nullptr;
};

// One implicit time step as ONE CUDA graph: psi -> psi_old copy, assembly, the
// solve (all cases of `batch`, or the whole system), boundary update.  The
// plain launches are stream-captured; the solve's nodes (with their device-side
// while loops) are added to the capture graph directly.
extern "C" fvgb_status fvgb_step_create(fvgb_ls* ls, fvgb_batch* batch, const fvgb_term* terms, int32_t nterms,
                                        double dt, const fvgb_bc* bc, double* psi, double* psi_b, double* psi_old,
                                        const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats_dev, fvgb_step** out) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(ls && terms && nterms > 0 && bc && psi && cfg && out, "fvgb_step_create: null argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_step_create: scalar systems only");
    if (cfg->preconditioner != FVGB_PRECOND_JACOBI)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_step_create: step graphs use the Jacobi preconditioner");
    FVGB_CHECK_ARG(!batch || batch->c->ls == ls, "fvgb_step_create: the batch belongs to another system");
    fvgb_status fst = check_cfg(cfg);
    if (fst != FVGB_OK) return fst;
    FVGB_CHECK_ARG(cfg->kernel_mode != 3, "fvgb_step_create: the host-driven loop cannot be part of a graph");
    SolverCache* c = batch ? batch->c : nullptr;
    if (!c) {
        fst = single_cache(ls, &c);
        if (fst != FVGB_OK) return fst;
    }
    const bool mixed = cfg->precision == FVGB_PREC_MIXED_IR;
    const bool measure = !(cfg->flags & FVGB_SOLVE_NO_TUNE);
    const bool bicg = cfg->method == FVGB_SOLVER_BICGSTAB;
    const bool bg = cfg->method == FVGB_SOLVER_BICG;
    fst = bg ? build_bicg(c)
             : bicg ? (mixed ? build_mixed_bicgstab(c) : build_bicgstab(c))
                    : (mixed ? build_mixed(c, measure) : build_fp64(c, measure));
    if (fst != FVGB_OK) return fst;
    SolverParams prm{};
    prm.x = psi;
    prm.stats_out = stats_dev;
    prm.rel_tol = cfg->rel_tol;
    prm.abs_tol = cfg->abs_tol;
    prm.inner_rel_tol = cfg->inner_rel_tol;
    prm.max_iter = cfg->max_iter;
    prm.inner_max_iter = cfg->inner_max_iter;
    prm.max_outer = cfg->max_outer;
    prm.convert = 1;  // the graph assembles the matrix every launch
    cudaStream_t cs = nullptr;
    FVGB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    const bool capturing = e == cudaSuccess;
    if (e == cudaSuccess && psi_old)
        e = cudaMemcpyAsync(psi_old, psi, sizeof(double) * (size_t)c->n, cudaMemcpyDeviceToDevice, cs);
    if (e == cudaSuccess) fst = fvgb_assemble(ls, terms, nterms, dt, bc, psi_b, (fvgb_stream)cs);
    if (e == cudaSuccess && fst == FVGB_OK) {
        k_set_params<<<grid_for(c->ncases, 128), 128, 0, cs>>>(c->L, c->ncases, prm);
        if (cfg->flags & FVGB_SOLVE_RHS_BASELINE) k_case_bnorm<<<c->nb, kT, 0, cs>>>(c->L, ls->rhs, c->pa);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && fst == FVGB_OK) {
        cudaStreamCaptureStatus cst;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &nd);
        cudaGraphNode_t last;
        if (e == cudaSuccess)
            e = bg     ? add_bicg_nodes(c, cg, deps, nd, &last)
                : bicg ? (mixed ? add_mixed_bicgstab_nodes(c, cg, deps, nd, &last)
                                : add_bicgstab_nodes(c, cg, deps, nd, &last))
                       : (mixed ? add_mixed_nodes(c, cg, deps, nd, &last) : add_fp64_nodes(c, cg, deps, nd, &last));
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(cs, &last, nullptr, 1, cudaStreamSetCaptureDependencies);
    }
    if (e == cudaSuccess && fst == FVGB_OK) fst = fvgb_bc_correct(ls->mesh, 1, bc, psi, psi_b, (fvgb_stream)cs);
    if (capturing) {
        const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess && fst == FVGB_OK) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (fst != FVGB_OK) return fst;
    if (e != cudaSuccess) return cuda_fail(e, "fvgb_step_create");
    *out = new fvgb_step{exec};
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_step_launch(fvgb_step* step, fvgb_stream stream) {
    FVGB_CHECK_ARG(step && step->exec, "fvgb_step_launch: null step");
    FVGB_CUDA_TRY(cudaGraphLaunch(step->exec, (cudaStream_t)stream));
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_step_destroy(fvgb_step* step) {
    if (!step) return FVGB_OK;
    if (step->exec) cudaGraphExecDestroy(step->exec);
    delete step;
    return FVGB_OK;
}

namespace {

// Launch-bound variants of the CG kernels: the autotuner's measurements and
// choices for a solver cache, optionally forcing a variant per kernel kind.
fvgb_status tuning(SolverCache* c, const int32_t* force, int32_t* chosen, float* ms, const char* who) {
    if (force)
        for (int k = 0; k < kTuneKinds; ++k)
            if (!(force[k] >= -1 && force[k] < kNumVariants))
                return fvgb_fail(FVGB_ERR_INVALID_ARG, (std::string(who) + ": bad variant").c_str());
    FVGB_CUDA_TRY(cudaDeviceSynchronize());  // no solve of this system in flight while its graphs are rebuilt
    if (force)
        for (int k = 0; k < kTuneKinds; ++k) c->forced[k] = force[k];
    fvgb_status st = build_fp64(c);  // allocates and tunes once, then (re)builds the graph
    if (st == FVGB_OK) st = build_mixed(c);
    if (st != FVGB_OK) return st;
    if (force) {
        for (int k = 0; k < kTuneKinds; ++k) pick(c, k);
        st = graph_fp64(c);
        if (st == FVGB_OK) st = graph_mixed(c);
        if (st != FVGB_OK) return st;
    }
    for (int k = 0; k < kTuneKinds; ++k) {
        chosen[k] = kVariantMinBlocks[c->variant[k]];
        for (int v = 0; v < kNumVariants; ++v) ms[k * kNumVariants + v] = c->tune_ms[k][v];
    }
    return FVGB_OK;
}

}  // namespace

extern "C" fvgb_status fvgb_solve_tuning(fvgb_ls* ls, const int32_t* force, int32_t* chosen, float* ms) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(ls && chosen && ms, "fvgb_solve_tuning: null argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_solve_tuning: scalar systems only");
    SolverCache* c = nullptr;
    fvgb_status st = single_cache(ls, &c);
    if (st != FVGB_OK) return st;
    return tuning(c, force, chosen, ms, "fvgb_solve_tuning");
}

extern "C" fvgb_status fvgb_batch_tuning(fvgb_batch* b, const int32_t* force, int32_t* chosen, float* ms) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(b && b->c && chosen && ms, "fvgb_batch_tuning: null argument");
    return tuning(b->c, force, chosen, ms, "fvgb_batch_tuning");
}

// Per-kernel timing of the FP64 CG iteration (outside any graph): runs init and
// `iters` iterations on a private copy of x with CUDA events around each kernel
// and returns the mean milliseconds of [spmv, update, direction, init].  A
// measurement aid for roofline reports; the solve itself always runs as a graph.
extern "C" fvgb_status fvgb_solve_kernel_times(fvgb_ls* ls, const double* x0, int32_t iters, double* ms_out,
                                               fvgb_stream stream) {
    FVGB_CHECK_ARG(ls && x0 && ms_out && iters > 0, "fvgb_solve_kernel_times: bad argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_solve_kernel_times: scalar systems only");
    cudaStream_t s = (cudaStream_t)stream;
    SolverCache* c = nullptr;
    fvgb_status stt = single_cache(ls, &c);
    if (stt != FVGB_OK) return stt;
    if (!c->g64) {
        stt = build_fp64(c);
        if (stt != FVGB_OK) return stt;
    }
    double* x = nullptr;
    FVGB_CUDA_TRY(cudaMalloc(&x, sizeof(double) * (size_t)c->n));
    cudaMemcpyAsync(x, x0, sizeof(double) * (size_t)c->n, cudaMemcpyDeviceToDevice, s);
    SolverParams prm{};
    prm.x = x;
    prm.max_iter = 1 << 30;
    k_set_params<<<1, 128, 0, s>>>(c->L, 1, prm);
    cudaGraphConditionalHandle h{};  // not used: setc = 0 outside a graph
    cudaError_t e = cudaSuccess;
    cudaEvent_t ev[6];
    for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreate(&ev[i]);
    if (e != cudaSuccess) {
        cudaFree(x);
        return cuda_fail(e, "fvgb_solve_kernel_times: setup");
    }
    const MeshView m = ls->mesh->v;
    const unsigned nb = (unsigned)c->nb;
    double acc[4] = {0, 0, 0, 0};
    float t;
    cudaEventRecord(ev[0], s);
    k_pcg_init<<<nb, kT, 0, s>>>(c->L, m, ls->values, ls->rhs, c->dinv, c->r, c->p, c->pa, c->pb, h, 0);
    cudaEventRecord(ev[1], s);
    for (int it = 0; it < iters; ++it) {
        cudaEventRecord(ev[2], s);
        launch_variant(variant_fn(kTuneSpmv64, c->variant[kTuneSpmv64]), nb, s, c->L, m, (const double*)ls->values,
                       (const double*)c->p, c->q, c->pa);
        cudaEventRecord(ev[3], s);
        launch_variant(variant_fn(kTuneUpdate64, c->variant[kTuneUpdate64]), nb, s, c->L, (const double*)c->dinv,
                       (const double*)c->p, (const double*)c->q, c->r, c->z, c->pa, c->pb, h, 0);
        cudaEventRecord(ev[4], s);
        k_pcg_dir<<<nb, kT, 0, s>>>(c->L, c->z, c->p);
        cudaEventRecord(ev[5], s);
        e = cudaEventSynchronize(ev[5]);
        if (e != cudaSuccess) break;
        cudaEventElapsedTime(&t, ev[2], ev[3]);
        acc[0] += t;
        cudaEventElapsedTime(&t, ev[3], ev[4]);
        acc[1] += t;
        cudaEventElapsedTime(&t, ev[4], ev[5]);
        acc[2] += t;
    }
    if (e == cudaSuccess) {
        cudaEventElapsedTime(&t, ev[0], ev[1]);
        acc[3] = t * iters;
    }
    for (int i = 0; i < 4; ++i) ms_out[i] = acc[i] / iters;
    for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
    cudaFree(x);
    if (e != cudaSuccess) return cuda_fail(e, "fvgb_solve_kernel_times");
    return FVGB_OK;
}
