// fvgb_pcg_csr_noalloc: the FP64 Jacobi-CG for callers that cannot allocate
// device memory.
//
// Some callers of this library cannot call cudaMalloc: a solver embedded as a
// plugin in a larger simulation whose host application has already claimed
// the device memory through its own allocator and fixed budget, or code that
// must not let an allocation implicitly synchronize the device (cudaMalloc and
// cudaFree may).  This entry point takes the system in NeoN's CSR layout in
// device memory the caller already owns, and keeps its own work vectors in a
// file-scope device array of fixed size instead of allocating them.
//
// Limits and sharing rules:
//  * at most kMaxRows rows (262,144: the 512x512 pressure system); larger
//    systems are rejected with FVGB_ERR_INVALID_ARG before any GPU work;
//  * the array (about 8.2 MiB) is part of the library image: every GPU that
//    loads the library holds it until the process exits;
//  * every call on a device uses the same array, so calls that overlap on the
//    GPU (different streams or threads without ordering) race and corrupt each
//    other; the array keeps the last call's contents, so each call clears the
//    counters it needs before use;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and caches it;
//  * every call is synchronous: it reads the solver state back between chunks
//    of iterations, so it cannot run on a stream that is being captured into a
//    CUDA graph and refuses one with FVGB_ERR_UNSUPPORTED before any work.
// The arithmetic and the reduction tree are those of the graph-based FP64 solve
// in solver.cu (same fma order per row, same 256-thread blocks and rows per thread), so the
// iterates are the same bits.
#include <climits>
#include <cmath>
#include <mutex>

#include "internal.cuh"

namespace {

constexpr int kT = 256;
constexpr int kRowsPerThread = 8;  // the most rows per thread (systems of 2^18 rows)
constexpr int kMaxRows = 262144;
constexpr int kMaxBlocks = kMaxRows / (kT * 4);
// rows per thread of the reduction tree, as the graph-based solve chooses it for a system of n rows
__host__ __device__ inline int na_rows_per_thread(int n) { return n >= (1 << 15) ? 8 : 4; }
constexpr int kMaxDevices = 64;

struct NaState {
    double rz, alpha, beta, res0, res, tol;
    double rel_tol, abs_tol;
    int32_t iter, max_iter, status, done;
    unsigned int counter, pending;
};

// [dinv | r | p | q] * kMaxRows, [pa | pb] * kMaxBlocks, then the state
constexpr size_t kStateDoubles = (sizeof(NaState) + sizeof(double) - 1) / sizeof(double);
constexpr size_t kScratchDoubles = 4 * (size_t)kMaxRows + 2 * (size_t)kMaxBlocks + kStateDoubles;

static __device__ __align__(256) double g_pcg_scratch[kScratchDoubles];

struct Scratch {
    double *dinv, *r, *p, *q, *pa, *pb;
    NaState* st;
};

__host__ __device__ inline Scratch carve(double* base) {
    Scratch s;
    s.dinv = base;
    s.r = base + kMaxRows;
    s.p = base + 2 * (size_t)kMaxRows;
    s.q = base + 3 * (size_t)kMaxRows;
    s.pa = base + 4 * (size_t)kMaxRows;
    s.pb = s.pa + kMaxBlocks;
    s.st = reinterpret_cast<NaState*>(s.pb + kMaxBlocks);
    return s;
}

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

__device__ __forceinline__ int red_row(int j, int n) {
    const int R = na_rows_per_thread(n);
    return j < R ? blockIdx.x * (kT * R) + (threadIdx.x >> 5) * (32 * R) + j * 32 + (threadIdx.x & 31) : INT_MAX;
}

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

__device__ __forceinline__ double csr_row(const int32_t* __restrict__ ro, const int32_t* __restrict__ col,
                                          const double* __restrict__ val, const double* __restrict__ x,
                                          int i) {
    double s = 0.0;
    for (int j = __ldg(&ro[i]); j < __ldg(&ro[i + 1]); ++j) s = fma(__ldg(&val[j]), x[__ldg(&col[j])], s);
    return s;
}

__global__ void k_na_reset(double* base, double rel_tol, double abs_tol, int max_iter) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        NaState* st = carve(base).st;
        st->counter = 0u;
        st->iter = 0;
        st->status = FVGB_OK;
        st->done = 0;
        st->rel_tol = rel_tol;
        st->abs_tol = abs_tol;
        st->max_iter = max_iter;
        st->res0 = 0.0;
        st->res = 0.0;
        st->pending = 0u;
    }
}

__global__ void __launch_bounds__(kT)
    k_na_init(double* base, int n, const int32_t* __restrict__ ro, const int32_t* __restrict__ col,
              const int32_t* __restrict__ doff, const double* __restrict__ val,
              const double* __restrict__ b, const double* __restrict__ x) {
    __shared__ double sma[kT], smb[kT];
    const Scratch S = carve(base);
    double arz = 0.0, arr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j, n);
        if (i >= n) continue;
        const double di = 1.0 / __ldg(&val[__ldg(&ro[i]) + __ldg(&doff[i])]);
        S.dinv[i] = di;
        const double ri = __ldg(&b[i]) - csr_row(ro, col, val, x, i);
        const double zi = di * ri;
        S.r[i] = ri;
        S.p[i] = zi;
        arz = fma(ri, zi, arz);
        arr = fma(ri, ri, arr);
    }
    const double ba = block_tree(arz, sma), bb = block_tree(arr, smb);
    if (threadIdx.x == 0) {
        S.pa[blockIdx.x] = ba;
        S.pb[blockIdx.x] = bb;
    }
    if (!arrive_last(&S.st->counter)) return;
    const double rz = final_tree(S.pa, gridDim.x, sma), rr = final_tree(S.pb, gridDim.x, smb);
    if (threadIdx.x == 0) {
        NaState* st = S.st;
        const double res0 = sqrt(rr);
        double tol = st->rel_tol * res0;
        if (st->abs_tol > tol) tol = st->abs_tol;
        st->rz = rz;
        st->res0 = res0;
        st->res = res0;
        st->tol = tol;
        bool done = !(res0 > tol) || res0 == 0.0;
        if (!isfinite(res0)) {  // NaN or inf in b or x: not "converged"
            done = true;
            st->status = FVGB_ERR_BREAKDOWN;
        } else if (!done && st->max_iter <= 0) {
            done = true;
            st->status = FVGB_ERR_NOT_CONVERGED;
        }
        st->done = done ? 1 : 0;
    }
}

__global__ void __launch_bounds__(kT)
    k_na_spmv(double* base, int n, const int32_t* __restrict__ ro, const int32_t* __restrict__ col,
              const double* __restrict__ val) {
    const Scratch S = carve(base);
    if (*(volatile int32_t*)&S.st->done) return;
    __shared__ double sma[kT];
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j, n);
        if (i >= n) continue;
        const double qi = csr_row(ro, col, val, S.p, i);
        S.q[i] = qi;
        acc = fma(S.p[i], qi, acc);
    }
    const double ba = block_tree(acc, sma);
    if (threadIdx.x == 0) S.pa[blockIdx.x] = ba;
    if (!arrive_last(&S.st->counter)) return;
    const double pq = final_tree(S.pa, gridDim.x, sma);
    if (threadIdx.x == 0) {
        NaState* st = S.st;
        const double alpha = st->rz / pq;
        st->alpha = alpha;
        if (pq == 0.0 || !isfinite(alpha)) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        }
    }
}

__global__ void __launch_bounds__(kT) k_na_update(double* base, int n, double* __restrict__ x) {
    const Scratch S = carve(base);
    if (*(volatile int32_t*)&S.st->done) return;
    __shared__ double sma[kT], smb[kT];
    const double alpha = S.st->alpha;
    double arz = 0.0, arr = 0.0;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j, n);
        if (i >= n) continue;
        x[i] = fma(alpha, S.p[i], x[i]);
        const double ri = fma(-alpha, S.q[i], S.r[i]);
        S.r[i] = ri;
        const double zi = S.dinv[i] * ri;
        arz = fma(ri, zi, arz);
        arr = fma(ri, ri, arr);
    }
    const double ba = block_tree(arz, sma), bb = block_tree(arr, smb);
    if (threadIdx.x == 0) {
        S.pa[blockIdx.x] = ba;
        S.pb[blockIdx.x] = bb;
    }
    if (!arrive_last(&S.st->counter)) return;
    const double rzn = final_tree(S.pa, gridDim.x, sma), rr = final_tree(S.pb, gridDim.x, smb);
    if (threadIdx.x == 0) {
        NaState* st = S.st;
        const double res = sqrt(rr);
        st->res = res;
        st->iter += 1;
        st->beta = rzn / st->rz;
        st->rz = rzn;
        bool done = false;
        if (!isfinite(res)) {
            st->status = FVGB_ERR_BREAKDOWN;
            done = true;
        } else if (!(res > st->tol)) {
            done = true;
        } else if (st->iter >= st->max_iter) {
            st->status = FVGB_ERR_NOT_CONVERGED;
            done = true;
        }
        // the direction update of this iteration still runs (as in the graph
        // version); the flag stops the next iteration
        st->pending = done ? 1u : 0u;
    }
}

__global__ void __launch_bounds__(kT) k_na_dir(double* base, int n) {
    const Scratch S = carve(base);
    if (*(volatile int32_t*)&S.st->done) return;
    const double beta = S.st->beta;
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int i = red_row(j, n);
        if (i >= n) continue;
        S.p[i] = fma(beta, S.p[i], S.dinv[i] * S.r[i]);
    }
}

// makes the stop decided in the update kernel visible to the next iteration
__global__ void k_na_latch(double* base) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        NaState* st = carve(base).st;
        if (st->pending) st->done = 1;
    }
}

fvgb_status scratch_for_current_device(double** out) {
    int dev = 0;
    FVGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_pcg_csr_noalloc: device ordinal >= 64");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_pcg_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "fvgb_pcg_csr_noalloc: cudaGetSymbolAddress");
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return FVGB_OK;
}

}  // namespace

extern "C" fvgb_status fvgb_pcg_csr_noalloc(int32_t n, const int32_t* row_offs, const int32_t* col_idxs,
                                            const int32_t* diag_offset, const double* values,
                                            const double* rhs, double* x, const fvgb_solver_cfg* cfg,
                                            fvgb_solver_stats* stats, fvgb_stream stream) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(row_offs && col_idxs && diag_offset && values && rhs && x && cfg,
                   "fvgb_pcg_csr_noalloc: null argument");
    if (cfg->preconditioner != FVGB_PRECOND_JACOBI)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_pcg_csr_noalloc: Jacobi preconditioner only");
    if (cfg->method != FVGB_SOLVER_CG)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_pcg_csr_noalloc: CG only");
    FVGB_CHECK_ARG(n > 0, "fvgb_pcg_csr_noalloc: n must be positive");
    if (n > kMaxRows)
        return fvgb_fail(FVGB_ERR_INVALID_ARG,
                         "fvgb_pcg_csr_noalloc: n exceeds the fixed work area of 262144 rows");
    FVGB_CHECK_ARG(cfg->precision == FVGB_PREC_FP64, "fvgb_pcg_csr_noalloc: FP64 precision only");
    if (cfg->flags & FVGB_SOLVE_RHS_BASELINE)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_pcg_csr_noalloc: the ||b|| tolerance baseline is not implemented");
    FVGB_CHECK_ARG(cfg->rel_tol >= 0 && cfg->abs_tol >= 0 && cfg->max_iter >= 0,
                   "fvgb_pcg_csr_noalloc: bad tolerances or iteration cap");
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FVGB_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED,
                         "fvgb_pcg_csr_noalloc: synchronous, cannot be called on a capturing stream");
    double* base = nullptr;
    fvgb_status stt = scratch_for_current_device(&base);
    if (stt != FVGB_OK) return stt;
    const int rb = kT * na_rows_per_thread(n);
    const unsigned nb = (unsigned)((n + rb - 1) / rb);
    k_na_reset<<<1, 32, 0, s>>>(base, cfg->rel_tol, cfg->abs_tol, cfg->max_iter);
    k_na_init<<<nb, kT, 0, s>>>(base, n, row_offs, col_idxs, diag_offset, values, rhs, x);
    FVGB_LAUNCH_CHECK("fvgb_pcg_csr_noalloc: init");
    NaState host{};
    const double* st_dev = base + 4 * (size_t)kMaxRows + 2 * (size_t)kMaxBlocks;
    const int chunk = 16;
    for (int64_t launched = 0;; launched += chunk) {
        FVGB_CUDA_TRY(cudaMemcpyAsync(&host, st_dev, sizeof(NaState), cudaMemcpyDeviceToHost, s));
        FVGB_CUDA_TRY(cudaStreamSynchronize(s));
        if (host.done) break;
        if (launched > (int64_t)cfg->max_iter + chunk)  // defensive: the device loop stops at max_iter
            return fvgb_fail(FVGB_ERR_CUDA, "fvgb_pcg_csr_noalloc: iteration bookkeeping lost");
        for (int k = 0; k < chunk; ++k) {
            k_na_spmv<<<nb, kT, 0, s>>>(base, n, row_offs, col_idxs, values);
            k_na_update<<<nb, kT, 0, s>>>(base, n, x);
            k_na_dir<<<nb, kT, 0, s>>>(base, n);
            k_na_latch<<<1, 32, 0, s>>>(base);
        }
        FVGB_LAUNCH_CHECK("fvgb_pcg_csr_noalloc: iteration");
    }
    fvgb_solver_stats out{};
    out.init_res_norm = host.res0;
    out.final_res_norm = host.res;
    out.num_iter = host.iter;
    out.num_outer = 0;
    out.status = host.status;
    if (stats) *stats = out;
    if (host.status == FVGB_ERR_NOT_CONVERGED)
        return fvgb_fail(FVGB_ERR_NOT_CONVERGED, "fvgb_pcg_csr_noalloc: iteration cap reached");
    if (host.status == FVGB_ERR_BREAKDOWN) return fvgb_fail(FVGB_ERR_BREAKDOWN, "fvgb_pcg_csr_noalloc: breakdown");
    return FVGB_OK;
}
