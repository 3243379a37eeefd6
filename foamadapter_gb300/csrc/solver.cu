// Krylov solves of the assembled system, entirely on the device.
//
// FP64: Jacobi-preconditioned CG, the algorithm of Ginkgo solver::Cg with
// preconditioner::Jacobi (max_block_size 1) that FoamAdapter maps OpenFOAM's
// PCG/DIC to (src/compatibility/fvSolution.cpp:19-104), with its stopping
// criteria (fvSolution.cpp:106-142).  MIXED_IR: CG on the Jacobi-scaled system
// in FP32 inside FP64 iterative refinement; the true residual b - A x, the
// update of x and the convergence test stay in FP64.
//
// Each solve is one CUDA graph: an init kernel, a device-side WHILE
// conditional node whose body holds one iteration (three kernels), and a
// finish kernel; the mixed solve nests the inner CG loop inside the refinement
// loop.  The kernel that finishes an iteration's reductions sets the loop
// condition, so there is no host round trip per iteration.  Every loop is
// bounded by an iteration cap.
//
// Reductions are deterministic: each 256-thread block owns 256*R rows
// (thread t: rows blk*256R + (t/32)*32R + j*32 + t%32, j < R; R = kRowsPerThread),
// sums its rows sequentially, then warp 0 sums the 256 partials (lane l: l, l+32, ..., l+224)
// and a xor butterfly finishes; the last block to arrive sums the block
// partials in index order with the same tree.  The CPU oracle reproduces this
// tree, so the FP64 iterates match it bit for bit.
#include <cmath>

#include "internal.cuh"

namespace {

constexpr int kT = 256;
constexpr int kRowsPerThread = 4;
constexpr int kRowsPerBlock = kT * kRowsPerThread;

struct SolverParams {
    double* x;
    fvgb_solver_stats* stats_out;  // device pointer or null
    double rel_tol, abs_tol, inner_rel_tol;
    int32_t max_iter, inner_max_iter, max_outer, pad;
};

struct SolverState {
    SolverParams prm;
    double rz, alpha, beta, res0, res, tol;
    double rho, rho0, itol;
    float falpha, fbeta;
    int32_t iter, status, total, outer, inner_it, inner_brk;
    unsigned int counter;
    unsigned int signflags;
    fvgb_solver_stats stats;
};

__device__ __forceinline__ int red_row(int j) {
    return blockIdx.x * kRowsPerBlock + (threadIdx.x >> 5) * (32 * kRowsPerThread) + j * 32 + (threadIdx.x & 31);
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

// FP32 block sum (inner solve of the mixed scheme: keeps the FP64 pipe free);
// same tree shape as block_tree.
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

// Thread 0 has written this block's partials; true in the block that arrives last.
__device__ __forceinline__ bool arrive_last(unsigned int* counter) {
    __shared__ bool am_last;
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicInc(counter, gridDim.x - 1);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return am_last;
}

// Row sum of a sliced-ELL row, fma chain in slot (= column) order.  The slot
// loads of the first 8 slots are issued before the dependent gathers.
__device__ __forceinline__ double spmv_row(const MeshView& m, const double* __restrict__ val,
                                           const double* __restrict__ x, int i) {
    const int slice = i >> 5, lane = i & 31;
    const int base = __ldg(&m.m_ptr[slice]) + lane;
    const int w = (__ldg(&m.m_ptr[slice + 1]) - __ldg(&m.m_ptr[slice])) >> 5;
    double v[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = 0.0;
        xv[k] = 0.0;
        if (k < w) {
            v[k] = __ldg(&val[base + k * 32]);
            xv[k] = __ldg(&x[__ldg(&m.m_col[base + k * 32])]);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) s = fma(v[k], xv[k], s);
    for (int k = 8; k < w; ++k) s = fma(__ldg(&val[base + k * 32]), __ldg(&x[__ldg(&m.m_col[base + k * 32])]), s);
    return s;
}

__device__ __forceinline__ float spmv_row_f(const MeshView& m, const float* __restrict__ val,
                                            const float* __restrict__ x, int i, float diag) {
    const int slice = i >> 5, lane = i & 31;
    const int base = __ldg(&m.m_ptr[slice]) + lane;
    const int w = (__ldg(&m.m_ptr[slice + 1]) - __ldg(&m.m_ptr[slice])) >> 5;
    float v[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = 0.0f;
        xv[k] = 0.0f;
        if (k < w) {
            v[k] = __ldg(&val[base + k * 32]);
            xv[k] = __ldg(&x[__ldg(&m.m_col[base + k * 32])]);
        }
    }
    float s = diag;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) s = fmaf(v[k], xv[k], s);
    for (int k = 8; k < w; ++k) s = fmaf(__ldg(&val[base + k * 32]), __ldg(&x[__ldg(&m.m_col[base + k * 32])]), s);
    return s;
}

__device__ __forceinline__ bool stop_status(SolverState* st, double res) {
    if (!isfinite(res)) {
        st->status = FVGB_ERR_BREAKDOWN;
        return true;
    }
    if (!(res > st->tol)) return true;
    return false;
}

// ------------------------------------------------------------------ FP64 PCG
__global__ void __launch_bounds__(kT)
    k_pcg_init(SolverState* st, MeshView m, const double* __restrict__ val,
               const double* __restrict__ b, double* __restrict__ dinv, double* __restrict__ r,
               double* __restrict__ p, double* __restrict__ pa, double* __restrict__ pb,
               cudaGraphConditionalHandle h, int setc) {
    __shared__ double sma[kT], smb[kT];
    const int n = m.n;
    const double* __restrict__ x = st->prm.x;
    double arz = 0.0, arr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
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
    if (!arrive_last(&st->counter)) return;
    const double rz = final_tree(pa, gridDim.x, sma), rr = final_tree(pb, gridDim.x, smb);
    if (threadIdx.x == 0) {
        const double res0 = sqrt(rr);
        double tol = st->prm.rel_tol * res0;
        if (st->prm.abs_tol > tol) tol = st->prm.abs_tol;
        st->rz = rz;
        st->res0 = res0;
        st->res = res0;
        st->tol = tol;
        st->iter = 0;
        st->status = FVGB_OK;
        bool done = !(res0 > tol) || res0 == 0.0;
        if (!done && st->prm.max_iter <= 0) {
            done = true;
            st->status = FVGB_ERR_NOT_CONVERGED;
        }
        if (setc) cudaGraphSetConditional(h, done ? 0u : 1u);
    }
}

__global__ void __launch_bounds__(kT)
    k_pcg_spmv(SolverState* st, MeshView m, const double* __restrict__ val,
               const double* __restrict__ p, double* __restrict__ q, double* __restrict__ pa,
               cudaGraphConditionalHandle h, int setc) {
    __shared__ double sma[kT];
    const int n = m.n;
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
        const double qi = spmv_row(m, val, p, i);
        q[i] = qi;
        acc = fma(__ldg(&p[i]), qi, acc);
    }
    const double ba = block_tree(acc, sma);
    if (threadIdx.x == 0) pa[blockIdx.x] = ba;
    if (!arrive_last(&st->counter)) return;
    const double pq = final_tree(pa, gridDim.x, sma);
    if (threadIdx.x == 0) {
        const double alpha = st->rz / pq;
        st->alpha = alpha;
        if (pq == 0.0 || !isfinite(alpha)) {
            st->status = FVGB_ERR_BREAKDOWN;
            if (setc) cudaGraphSetConditional(h, 0u);
        }
    }
}

__global__ void __launch_bounds__(kT)
    k_pcg_update(SolverState* st, MeshView m, const double* __restrict__ dinv,
                 const double* __restrict__ p, const double* __restrict__ q,
                 double* __restrict__ r, double* __restrict__ z, double* __restrict__ pa,
                 double* __restrict__ pb, cudaGraphConditionalHandle h, int setc) {
    if (st->status == FVGB_ERR_BREAKDOWN) return;
    __shared__ double sma[kT], smb[kT];
    const int n = m.n;
    double* __restrict__ x = st->prm.x;
    const double alpha = st->alpha;
    double arz = 0.0, arr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
        const double pi = __ldg(&p[i]);
        x[i] = fma(alpha, pi, x[i]);
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
    if (!arrive_last(&st->counter)) return;
    const double rzn = final_tree(pa, gridDim.x, sma), rr = final_tree(pb, gridDim.x, smb);
    if (threadIdx.x == 0) {
        const double res = sqrt(rr);
        st->res = res;
        st->iter += 1;
        st->beta = rzn / st->rz;
        st->rz = rzn;
        bool done = stop_status(st, res);
        if (!done && st->iter >= st->prm.max_iter) {
            st->status = FVGB_ERR_NOT_CONVERGED;
            done = true;
        }
        if (setc) cudaGraphSetConditional(h, done ? 0u : 1u);
    }
}

__global__ void __launch_bounds__(kT)
    k_pcg_dir(const SolverState* st, int n, const double* __restrict__ z, double* __restrict__ p) {
    if (st->status == FVGB_ERR_BREAKDOWN) return;
    const double beta = st->beta;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
        p[i] = fma(beta, p[i], __ldg(&z[i]));  // z = dinv*r, stored by the update
    }
}

__global__ void k_finish(SolverState* st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    fvgb_solver_stats s;
    s.init_res_norm = st->res0;
    s.final_res_norm = st->res;
    s.num_iter = st->iter + st->total;  // FP64 counts iter, mixed counts total (the other is 0)
    s.num_outer = st->outer;
    s.status = st->status;
    s.reserved = 0;
    st->stats = s;
    if (st->prm.stats_out) *st->prm.stats_out = s;
}

__global__ void k_set_params(SolverState* st, SolverParams prm) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->prm = prm;
        st->iter = 0;
        st->total = 0;
        st->outer = 0;
        st->status = FVGB_OK;
        st->res0 = 0.0;
        st->res = 0.0;
        st->signflags = 0u;
        st->counter = 0u;
    }
}

// --------------------------------------------------- mixed precision (FP32 inner)
// s_i = 1/sqrt|a_ii|; signflags bit0: a positive diagonal, bit1: negative, bit2: zero/NaN
__global__ void __launch_bounds__(kT)
    k_ir_scale(SolverState* st, MeshView m, const double* __restrict__ val, double* __restrict__ s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int f = 0;
    if (i < m.n) {
        const double d = __ldg(&val[__ldg(&m.diag_pos[i])]);
        f = d > 0.0 ? 1u : (d < 0.0 ? 2u : 4u);
        s[i] = 1.0 / sqrt(fabs(d));
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(&st->signflags, f);
}

// ahat at every slot: (float)((a * s_row) * s_col); diagonal and padding slots 0
__global__ void __launch_bounds__(kT)
    k_ir_scaled_values(MeshView m, const double* __restrict__ val, const double* __restrict__ s,
                       float* __restrict__ ah) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n) return;
    const int slice = i >> 5, lane = i & 31;
    const int base = __ldg(&m.m_ptr[slice]);
    const int w = (__ldg(&m.m_ptr[slice + 1]) - base) >> 5;
    const double si = s[i];
    for (int k = 0; k < w; ++k) {
        const int pos = base + k * 32 + lane;
        const int code = __ldg(&m.m_code[pos]);
        float v = 0.0f;
        if (code != FVGB_PAD && code != -1) v = (float)((__ldg(&val[pos]) * si) * s[__ldg(&m.m_col[pos])]);
        ah[pos] = v;
    }
}

// outer step: r = b - A x (FP64), rr; rhat = (float)(s r); y = 0; p = rhat; rho = rhat.rhat
template <bool FIRST>
__global__ void __launch_bounds__(kT)
    k_ir_residual(SolverState* st, MeshView m, const double* __restrict__ val,
                  const double* __restrict__ b, const double* __restrict__ s,
                  float* __restrict__ rh, float* __restrict__ y, float* __restrict__ p,
                  double* __restrict__ pa, double* __restrict__ pb,
                  cudaGraphConditionalHandle h_outer, cudaGraphConditionalHandle h_inner) {
    if (st->status == FVGB_ERR_BREAKDOWN) return;
    __shared__ double sma[kT], smb[kT];
    const int n = m.n;
    const double* __restrict__ x = st->prm.x;
    double arr = 0.0;
    float arho = 0.0f;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
        const double ri = __ldg(&b[i]) - spmv_row(m, val, x, i);
        arr = fma(ri, ri, arr);
        const float rhi = (float)(__ldg(&s[i]) * ri);
        rh[i] = rhi;
        y[i] = 0.0f;
        p[i] = rhi;
        arho = fmaf(rhi, rhi, arho);
    }
    __shared__ float smf[kT];
    const double ba = block_tree(arr, sma);
    const float bb = block_tree_f(arho, smf);
    if (threadIdx.x == 0) {
        pa[blockIdx.x] = ba;
        pb[blockIdx.x] = (double)bb;
    }
    if (!arrive_last(&st->counter)) return;
    const double rr = final_tree(pa, gridDim.x, sma), rho = final_tree(pb, gridDim.x, smb);
    if (threadIdx.x == 0) {
        const double res = sqrt(rr);
        if (!FIRST) st->outer += 1;
        st->res = res;
        bool done = false;
        if (FIRST) {
            st->res0 = res;
            double tol = st->prm.rel_tol * res;
            if (st->prm.abs_tol > tol) tol = st->prm.abs_tol;
            st->tol = tol;
            const unsigned int sf = st->signflags;
            if ((sf & 4u) || sf == 3u) {
                st->status = FVGB_ERR_UNSUPPORTED;
                done = true;
            }
        }
        if (!done) {
            done = stop_status(st, res) || res == 0.0;
            if (!done && (st->outer >= st->prm.max_outer || st->total >= st->prm.max_iter)) {
                st->status = FVGB_ERR_NOT_CONVERGED;
                done = true;
            }
        }
        st->rho = rho;
        st->rho0 = rho;
        st->itol = st->prm.inner_rel_tol * st->prm.inner_rel_tol * rho;
        st->inner_it = 0;
        st->inner_brk = 0;
        const bool inner = !done && rho > st->itol && st->prm.inner_max_iter > 0 &&
                           st->total < st->prm.max_iter;
        cudaGraphSetConditional(h_inner, inner ? 1u : 0u);
        cudaGraphSetConditional(h_outer, done ? 0u : 1u);
    }
}

// q = (S A S) p with unit diagonal sign; pq -> alpha
__global__ void __launch_bounds__(kT)
    k_ir_spmv(SolverState* st, MeshView m, const float* __restrict__ ah,
              const float* __restrict__ p, float* __restrict__ q, double* __restrict__ pa,
              cudaGraphConditionalHandle h_outer, cudaGraphConditionalHandle h_inner) {
    __shared__ double sma[kT];
    const int n = m.n;
    const float dsign = st->signflags == 2u ? -1.0f : 1.0f;  // sign of every diagonal
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
        const float pi = __ldg(&p[i]);
        const float qi = spmv_row_f(m, ah, p, i, dsign * pi);
        q[i] = qi;
        acc = fmaf(pi, qi, acc);
    }
    __shared__ float smf[kT];
    const float ba = block_tree_f(acc, smf);
    if (threadIdx.x == 0) pa[blockIdx.x] = (double)ba;
    if (!arrive_last(&st->counter)) return;
    const double pq = final_tree(pa, gridDim.x, sma);
    if (threadIdx.x == 0) {
        const double alpha = st->rho / pq;
        if (pq == 0.0 || !isfinite(alpha)) {
            st->inner_brk = 1;
            cudaGraphSetConditional(h_inner, 0u);
            if (st->inner_it == 0) {
                st->status = FVGB_ERR_BREAKDOWN;
                cudaGraphSetConditional(h_outer, 0u);
            }
        } else {
            st->falpha = (float)alpha;
        }
    }
}

__global__ void __launch_bounds__(kT)
    k_ir_update(SolverState* st, int n, const float* __restrict__ p, const float* __restrict__ q,
                float* __restrict__ y, float* __restrict__ rh, double* __restrict__ pa,
                cudaGraphConditionalHandle h_inner) {
    if (st->inner_brk) return;
    __shared__ double sma[kT];
    const float fa = st->falpha;
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
        const float pi = __ldg(&p[i]);
        y[i] = fmaf(fa, pi, y[i]);
        const float ri = fmaf(-fa, __ldg(&q[i]), rh[i]);
        rh[i] = ri;
        acc = fmaf(ri, ri, acc);
    }
    __shared__ float smf[kT];
    const float ba = block_tree_f(acc, smf);
    if (threadIdx.x == 0) pa[blockIdx.x] = (double)ba;
    if (!arrive_last(&st->counter)) return;
    const double rhon = final_tree(pa, gridDim.x, sma);
    if (threadIdx.x == 0) {
        st->fbeta = (float)(rhon / st->rho);
        st->rho = rhon;
        st->inner_it += 1;
        st->total += 1;
        const bool more = rhon > st->itol && st->inner_it < st->prm.inner_max_iter &&
                          st->total < st->prm.max_iter;
        cudaGraphSetConditional(h_inner, more ? 1u : 0u);
    }
}

__global__ void __launch_bounds__(kT)
    k_ir_dir(const SolverState* st, int n, const float* __restrict__ rh, float* __restrict__ p) {
    if (st->inner_brk) return;
    const float fb = st->fbeta;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j);
        if (i >= n) continue;
        p[i] = fmaf(fb, p[i], __ldg(&rh[i]));
    }
}

__global__ void __launch_bounds__(kT)
    k_ir_xupdate(const SolverState* st, int n, const double* __restrict__ s,
                 const float* __restrict__ y) {
    if (st->status == FVGB_ERR_BREAKDOWN) return;
    double* __restrict__ x = st->prm.x;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = fma(__ldg(&s[i]), (double)__ldg(&y[i]), x[i]);
}

// ---------------------------------------------------------------- graph glue
cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t* dep, void* func,
                       unsigned grid, void** args) {
    cudaKernelNodeParams kp{};
    kp.func = func;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(kT);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    return cudaGraphAddKernelNode(node, g, dep, dep ? 1 : 0, &kp);
}

cudaError_t add_while(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t* dep,
                      cudaGraphConditionalHandle h, cudaGraph_t* body) {
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

struct SolverCache {
    const fvgb_ls* ls = nullptr;
    int n = 0, nb = 0;
    SolverState* st = nullptr;
    double *dinv = nullptr, *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr, *pa = nullptr,
           *pb = nullptr;
    double* s = nullptr;
    float *ah = nullptr, *rh = nullptr, *y = nullptr, *pf = nullptr, *qf = nullptr;
    cudaGraphExec_t g64 = nullptr, gmix = nullptr;
    fvgb_solver_stats* h_stats = nullptr;  // pinned
};

void fvgb_solver_cache_free(SolverCache* c) {
    if (!c) return;
    if (c->g64) cudaGraphExecDestroy(c->g64);
    if (c->gmix) cudaGraphExecDestroy(c->gmix);
    void* ptrs[] = {c->st, c->dinv, c->r, c->p, c->q, c->z, c->pa, c->pb, c->s, c->ah, c->rh, c->y, c->pf, c->qf};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->h_stats) cudaFreeHost(c->h_stats);
    delete c;
}

namespace {

fvgb_status cache_get(fvgb_ls* ls, SolverCache** out) {
    if (ls->solver) {
        *out = ls->solver;
        return FVGB_OK;
    }
    SolverCache* c = new SolverCache();
    c->ls = ls;
    c->n = ls->mesh->v.n;
    c->nb = (c->n + kRowsPerBlock - 1) / kRowsPerBlock;
    const size_t n = (size_t)c->n, nb = (size_t)c->nb;
    cudaError_t e = cudaMalloc(&c->st, sizeof(SolverState));
    if (e == cudaSuccess) e = cudaMemset(c->st, 0, sizeof(SolverState));
    if (e == cudaSuccess) e = cudaMalloc(&c->pa, sizeof(double) * nb);
    if (e == cudaSuccess) e = cudaMalloc(&c->pb, sizeof(double) * nb);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_stats, sizeof(fvgb_solver_stats));
    if (e != cudaSuccess) {
        fvgb_solver_cache_free(c);
        return cuda_fail(e, "solver workspace");
    }
    (void)n;
    ls->solver = c;
    *out = c;
    return FVGB_OK;
}

fvgb_status build_fp64(SolverCache* c) {
    const size_t n = (size_t)c->n;
    cudaError_t e = cudaMalloc(&c->dinv, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->r, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->p, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->q, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->z, sizeof(double) * n);
    if (e != cudaSuccess) return cuda_fail(e, "FP64 CG workspace");
    const fvgb_ls* ls = c->ls;
    MeshView m = ls->mesh->v;
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaGraphNode_t n0, n1, n2, b0, b1, b2;
    cudaGraph_t body;
    SolverState* st = c->st;
    const double* val = ls->values;
    const double* b = ls->rhs;
    int nn = c->n;
    unsigned nb = (unsigned)c->nb;
    e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    int setc = 1;
    void* a_init[] = {&st, &m, &val, &b, &c->dinv, &c->r, &c->p, &c->pa, &c->pb, &h, &setc};
    if (e == cudaSuccess) e = add_kernel(g, &n0, nullptr, (void*)k_pcg_init, nb, a_init);
    if (e == cudaSuccess) e = add_while(g, &n1, &n0, h, &body);
    void* a_spmv[] = {&st, &m, &val, &c->p, &c->q, &c->pa, &h, &setc};
    void* a_upd[] = {&st, &m, &c->dinv, &c->p, &c->q, &c->r, &c->z, &c->pa, &c->pb, &h, &setc};
    void* a_dir[] = {&st, &nn, &c->z, &c->p};
    if (e == cudaSuccess) e = add_kernel(body, &b0, nullptr, (void*)k_pcg_spmv, nb, a_spmv);
    if (e == cudaSuccess) e = add_kernel(body, &b1, &b0, (void*)k_pcg_update, nb, a_upd);
    if (e == cudaSuccess) e = add_kernel(body, &b2, &b1, (void*)k_pcg_dir, nb, a_dir);
    void* a_fin[] = {&st};
    if (e == cudaSuccess) {
        cudaKernelNodeParams kp{};
        kp.func = (void*)k_finish;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(32);
        kp.kernelParams = a_fin;
        e = cudaGraphAddKernelNode(&n2, g, &n1, 1, &kp);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->g64, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "FP64 CG graph");
    return FVGB_OK;
}

fvgb_status build_mixed(SolverCache* c) {
    const size_t n = (size_t)c->n;
    const fvgb_ls* ls = c->ls;
    const fvgb_mesh* mesh = ls->mesh;
    cudaError_t e = cudaMalloc(&c->s, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->ah, sizeof(float) * (size_t)mesh->m_len);
    if (e == cudaSuccess) e = cudaMalloc(&c->rh, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->y, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->pf, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&c->qf, sizeof(float) * n);
    if (e != cudaSuccess) return cuda_fail(e, "mixed CG workspace");
    MeshView m = mesh->v;
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle ho, hi;
    SolverState* st = c->st;
    const double* val = ls->values;
    const double* b = ls->rhs;
    int nn = c->n;
    unsigned nb = (unsigned)c->nb, ncb = grid_for(c->n, kT);
    e = cudaGraphConditionalHandleCreate(&ho, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hi, g, 0, cudaGraphCondAssignDefault);
    cudaGraphNode_t n_scale, n_vals, n_res0, n_outer, n_fin, o_inner, o_x, o_res, i_spmv, i_upd, i_dir;
    cudaGraph_t obody = nullptr, ibody = nullptr;
    void* a_scale[] = {&st, &m, &val, &c->s};
    void* a_vals[] = {&m, &val, &c->s, &c->ah};
    void* a_res[] = {&st, &m, &val, &b, &c->s, &c->rh, &c->y, &c->pf, &c->pa, &c->pb, &ho, &hi};
    if (e == cudaSuccess) e = add_kernel(g, &n_scale, nullptr, (void*)k_ir_scale, ncb, a_scale);
    if (e == cudaSuccess) e = add_kernel(g, &n_vals, &n_scale, (void*)k_ir_scaled_values, ncb, a_vals);
    if (e == cudaSuccess) e = add_kernel(g, &n_res0, &n_vals, (void*)k_ir_residual<true>, nb, a_res);
    if (e == cudaSuccess) e = add_while(g, &n_outer, &n_res0, ho, &obody);
    if (e == cudaSuccess) e = add_while(obody, &o_inner, nullptr, hi, &ibody);
    void* a_spmv[] = {&st, &m, &c->ah, &c->pf, &c->qf, &c->pa, &ho, &hi};
    void* a_upd[] = {&st, &nn, &c->pf, &c->qf, &c->y, &c->rh, &c->pa, &hi};
    void* a_dir[] = {&st, &nn, &c->rh, &c->pf};
    void* a_x[] = {&st, &nn, &c->s, &c->y};
    if (e == cudaSuccess) e = add_kernel(ibody, &i_spmv, nullptr, (void*)k_ir_spmv, nb, a_spmv);
    if (e == cudaSuccess) e = add_kernel(ibody, &i_upd, &i_spmv, (void*)k_ir_update, nb, a_upd);
    if (e == cudaSuccess) e = add_kernel(ibody, &i_dir, &i_upd, (void*)k_ir_dir, nb, a_dir);
    if (e == cudaSuccess) e = add_kernel(obody, &o_x, &o_inner, (void*)k_ir_xupdate, ncb, a_x);
    if (e == cudaSuccess) e = add_kernel(obody, &o_res, &o_x, (void*)k_ir_residual<false>, nb, a_res);
    void* a_fin[] = {&st};
    if (e == cudaSuccess) {
        cudaKernelNodeParams kp{};
        kp.func = (void*)k_finish;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(32);
        kp.kernelParams = a_fin;
        e = cudaGraphAddKernelNode(&n_fin, g, &n_outer, 1, &kp);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gmix, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "mixed CG graph");
    return FVGB_OK;
}

fvgb_status launch_solve(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg,
                         fvgb_solver_stats* stats_dev, cudaStream_t s, SolverCache** out) {
    FVGB_CHECK_ARG(ls && x && cfg, "fvgb_solve: null argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_solve: scalar systems only");
    FVGB_CHECK_ARG(cfg->precision == FVGB_PREC_FP64 || cfg->precision == FVGB_PREC_MIXED_IR,
                   "fvgb_solve: unknown precision");
    FVGB_CHECK_ARG(cfg->rel_tol >= 0 && cfg->abs_tol >= 0, "fvgb_solve: negative tolerance");
    FVGB_CHECK_ARG(cfg->max_iter >= 0 && cfg->max_iter <= 100000000, "fvgb_solve: bad max_iter");
    if (cfg->precision == FVGB_PREC_MIXED_IR)
        FVGB_CHECK_ARG(cfg->inner_rel_tol > 0 && cfg->inner_rel_tol < 1 && cfg->inner_max_iter > 0 &&
                           cfg->max_outer > 0,
                       "fvgb_solve: mixed precision needs inner_rel_tol in (0,1), inner_max_iter > 0, max_outer > 0");
    SolverCache* c = nullptr;
    fvgb_status stt = cache_get(ls, &c);
    if (stt != FVGB_OK) return stt;
    if (cfg->precision == FVGB_PREC_FP64 && !c->g64) {
        stt = build_fp64(c);
        if (stt != FVGB_OK) return stt;
    }
    if (cfg->precision == FVGB_PREC_MIXED_IR && !c->gmix) {
        stt = build_mixed(c);
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
    k_set_params<<<1, 32, 0, s>>>(c->st, prm);
    FVGB_LAUNCH_CHECK("fvgb_solve: parameters");
    FVGB_CUDA_TRY(cudaGraphLaunch(cfg->precision == FVGB_PREC_FP64 ? c->g64 : c->gmix, s));
    *out = c;
    return FVGB_OK;
}

}  // namespace

extern "C" fvgb_status fvgb_solve_async(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg,
                                        fvgb_solver_stats* stats_dev, fvgb_stream stream) {
    SolverCache* c = nullptr;
    return launch_solve(ls, x, cfg, stats_dev, (cudaStream_t)stream, &c);
}

extern "C" fvgb_status fvgb_solve(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg,
                                  fvgb_solver_stats* stats, fvgb_stream stream) {
    SolverCache* c = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    fvgb_status st = launch_solve(ls, x, cfg, nullptr, s, &c);
    if (st != FVGB_OK) return st;
    FVGB_CUDA_TRY(cudaMemcpyAsync(c->h_stats, &c->st->stats, sizeof(fvgb_solver_stats),
                                  cudaMemcpyDeviceToHost, s));
    FVGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (stats) *stats = *c->h_stats;
    const int32_t r = c->h_stats->status;
    if (r == FVGB_ERR_UNSUPPORTED)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_solve: mixed precision needs diagonals of one sign");
    if (r == FVGB_ERR_NOT_CONVERGED) return fvgb_fail(FVGB_ERR_NOT_CONVERGED, "fvgb_solve: iteration cap reached");
    if (r == FVGB_ERR_BREAKDOWN) return fvgb_fail(FVGB_ERR_BREAKDOWN, "fvgb_solve: breakdown");
    return FVGB_OK;
}

// Per-kernel timing of the FP64 CG iteration (outside any graph): runs init and
// `iters` iterations on a private copy of x with CUDA events around each kernel
// and returns the mean milliseconds of [spmv, update, direction, init].  A
// measurement aid for roofline reports; the solve itself always runs as a graph.
extern "C" fvgb_status fvgb_solve_kernel_times(fvgb_ls* ls, const double* x0, int32_t iters,
                                               double* ms_out, fvgb_stream stream) {
    FVGB_CHECK_ARG(ls && x0 && ms_out && iters > 0, "fvgb_solve_kernel_times: bad argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_solve_kernel_times: scalar systems only");
    cudaStream_t s = (cudaStream_t)stream;
    SolverCache* c = nullptr;
    fvgb_status stt = cache_get(ls, &c);
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
    prm.rel_tol = 0.0;
    prm.abs_tol = 0.0;
    prm.max_iter = 1 << 30;
    k_set_params<<<1, 32, 0, s>>>(c->st, prm);
    cudaGraphConditionalHandle h{};  // not used: setc = 0 outside a graph
    cudaError_t e = cudaSuccess;
    cudaEvent_t ev[8];
    for (int i = 0; i < 8 && e == cudaSuccess; ++i) e = cudaEventCreate(&ev[i]);
    if (e != cudaSuccess) {
        cudaFree(x);
        return cuda_fail(e, "fvgb_solve_kernel_times: setup");
    }
    const MeshView m = ls->mesh->v;
    const unsigned nb = (unsigned)c->nb;
    double acc[4] = {0, 0, 0, 0};
    float t;
    // the loop condition can only be set from inside a graph: setc = 0 here
    cudaEventRecord(ev[0], s);
    k_pcg_init<<<nb, kT, 0, s>>>(c->st, m, ls->values, ls->rhs, c->dinv, c->r, c->p, c->pa, c->pb, h, 0);
    cudaEventRecord(ev[1], s);
    for (int it = 0; it < iters; ++it) {
        cudaEventRecord(ev[2], s);
        k_pcg_spmv<<<nb, kT, 0, s>>>(c->st, m, ls->values, c->p, c->q, c->pa, h, 0);
        cudaEventRecord(ev[3], s);
        k_pcg_update<<<nb, kT, 0, s>>>(c->st, m, c->dinv, c->p, c->q, c->r, c->z, c->pa, c->pb, h, 0);
        cudaEventRecord(ev[4], s);
        k_pcg_dir<<<nb, kT, 0, s>>>(c->st, c->n, c->z, c->p);
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
    for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
    cudaFree(x);
    if (e != cudaSuccess) return cuda_fail(e, "fvgb_solve_kernel_times");
    return FVGB_OK;
}
