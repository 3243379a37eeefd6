// Multigrid-preconditioned CG (FP64) for a single scalar system, and the
// multigrid solver on its own.
//
// The reference selects the first through a Ginkgo configuration: solver::Cg
// whose preconditioner is solver::Multigrid with multigrid::Pgm levels
// (tutorials/cylinder2D/system/gko/config.mg.json).  GAMG in an fvSolution
// maps to Ginkgo's solver::Multigrid as the solver
// (src/compatibility/fvSolution.cpp:27): cfg->method = FVGB_SOLVER_MULTIGRID
// iterates x += V(b - A x) with the same hierarchy and V-cycle.  Ginkgo is not
// part of the reference checkout; this is this library's own aggregation AMG
// built on the published parallel-graph-match (PGM) idea:
//
// Setup, symbolic (host, once per system, from the first matrix solved):
//  * PGM aggregation (pgm_aggregate): strength |a_ij| between rows; in up to
//    15 rounds every unaggregated row picks its strongest unaggregated
//    neighbour (ties: the lower index) and mutual picks become pairs; the
//    rounds stop when at most 5% of the rows are left or no pair forms.  A row
//    left over joins the aggregate of its strongest aggregated neighbour, or
//    stays alone.  Aggregates are numbered by their lowest row.  Each level
//    applies it twice (double pairwise aggregation, as in Notay's AGMG): the
//    pairs are matched again on their Galerkin matrix, so a level keeps about
//    a quarter of the rows and the hierarchy has half as many levels.
//  * Galerkin coarse matrix A_c = P^T A P for the piecewise-constant P: its
//    pattern and, for each coarse entry, the fine entries it sums (fine rows
//    ascending, entries in row order).  Levels are added until at most
//    kCoarseRows rows remain, the aggregation stops shrinking the system
//    (more than 90% of the rows left), or kMaxLevels is reached.
// Setup, numeric (device, whenever the matrix values changed): the coarse
// values by those fixed sums, the Jacobi diagonals, and the inverse of the
// coarsest matrix by Gauss-Jordan elimination in one block (no pivoting: the
// matrix is symmetric positive definite).
// V-cycle z = M r: per level one damped-Jacobi sweep from zero (weight 0.9),
// the residual, restriction by aggregate sums, the coarser level, then the
// coarse correction and one more damped-Jacobi sweep; the coarsest level is
// solved exactly with the dense inverse.  Pre- and post-smoothing are the same
// symmetric sweep, so M is symmetric positive definite and CG applies.
// Kernels: the first sweep of level 0 is formed by the CG kernels that produce
// r (k_init, k_update), a coarse level's by the restriction that produces its
// right-hand side; the residual is one gather per slot (k_resid); level 0
// adds the coarse correction (k_prolong) before its second sweep (k_post),
// coarser levels form it inside the sweep (k_post_fused); the coarsest level
// runs in one block (k_tail, which can take more levels: kTailRows).  Coarse
// levels are sliced ELL like the system matrix.
//
// A solve is one CUDA graph (init, a device-side while loop over the CG
// iteration with the V-cycle inside, or over the multigrid iteration, bounded
// by max_iter).  Its stopping test and statistics are those of the Jacobi-PCG
// (Ginkgo criteria: ||r|| below max(rel_tol ||r_0||, abs_tol), or
// max(rel_tol ||b||, abs_tol) with FVGB_SOLVE_RHS_BASELINE).  Every reduction
// has a fixed order, so a solve is deterministic; its iterates are not those
// of the Jacobi-PCG.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <thread>
#include <type_traits>
#include <vector>

#include "internal.cuh"

namespace {

constexpr int kT = 256;
constexpr int kCoarseRows = 256;
constexpr int kMaxLevels = 25;
constexpr double kOmega = 0.9;
constexpr int kPgmRounds = 15;
constexpr double kPgmLeftRatio = 0.05;
constexpr int kTailRows = 0;  // levels this small run in the single-block tail (0: the coarsest only)

struct HostCsr {
    int n = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
};

// ------------------------------------------------------------ host threads
// f(begin, end, chunk) over [0, n) in contiguous chunks on up to 16 threads
// (one when n is small).  Every use below writes only its own rows, or
// per-chunk results that are joined in chunk order: the results are those of
// the sequential loop.
template <class F>
int parallel_chunks(int n, int min_per_chunk, F f) {
    const int hw = (int)std::thread::hardware_concurrency();
    const int nt = std::max(1, std::min({16, hw > 0 ? hw : 1, n / std::max(1, min_per_chunk)}));
    if (nt == 1) {
        f(0, n, 0);
        return 1;
    }
    std::vector<std::thread> th;
    th.reserve((size_t)nt);
    for (int t = 0; t < nt; ++t)
        th.emplace_back(f, (int)((int64_t)n * t / nt), (int)((int64_t)n * (t + 1) / nt), t);
    for (std::thread& x : th) x.join();
    return nt;
}

// Ids next, next+1, ... for the rows with flag set, in row order (a prefix
// sum over chunks); returns how many.
int number_flagged(int n, const std::vector<char>& flag, std::vector<int>& id, int next) {
    std::vector<int> cnt(16, 0), base(17, 0);
    const int nt = parallel_chunks(n, 1 << 15, [&](int b, int e, int t) {
        int c = 0;
        for (int i = b; i < e; ++i) c += flag[i] ? 1 : 0;
        cnt[t] = c;
    });
    for (int t = 0; t < nt; ++t) base[t + 1] = base[t] + cnt[t];
    parallel_chunks(n, 1 << 15, [&](int b, int e, int t) {
        int k = next + base[t];
        for (int i = b; i < e; ++i)
            if (flag[i]) id[i] = k++;
    });
    return base[nt];
}

// ------------------------------------------------------------ PGM (host)
int pgm_aggregate(int n, const int* rp, const int* ci, const double* v, std::vector<int>& agg) {
    agg.assign(n, -1);
    std::vector<int> pick(n, -1);
    std::vector<int> tmp(n, -1);  // provisional aggregate id of each row
    std::vector<int> id(n, -1);
    std::vector<char> flag(n, 0);
    int next = 0, left = n;
    for (int round = 0; round < kPgmRounds; ++round) {
        parallel_chunks(n, 1 << 15, [&](int b, int e, int) {
            for (int i = b; i < e; ++i) {
                pick[i] = -1;
                if (tmp[i] >= 0) continue;
                double best = 0.0;
                for (int k = rp[i]; k < rp[i + 1]; ++k) {
                    const int j = ci[k];
                    if (j == i || tmp[j] >= 0) continue;
                    const double w = std::fabs(v[k]);
                    if (w > best || (w == best && w > 0.0 && (pick[i] < 0 || j < pick[i]))) {
                        best = w;
                        pick[i] = j;
                    }
                }
            }
        });
        // mutual picks pair up (pairs are disjoint); the lower row numbers the
        // pair, pairs numbered in the order of their lower rows
        parallel_chunks(n, 1 << 15, [&](int b, int e, int) {
            for (int i = b; i < e; ++i) {
                const int j = pick[i];
                flag[i] = (tmp[i] < 0 && j > i && pick[j] == i) ? 1 : 0;
            }
        });
        const int formed = number_flagged(n, flag, id, next);
        parallel_chunks(n, 1 << 15, [&](int b, int e, int) {
            for (int i = b; i < e; ++i)
                if (flag[i]) tmp[i] = tmp[pick[i]] = id[i];
        });
        next += formed;
        left -= 2 * formed;
        if (formed == 0 || left <= kPgmLeftRatio * n) break;
    }
    // rows left over: the strongest aggregated neighbour's aggregate, else alone
    std::vector<int> late(n, -1);
    parallel_chunks(n, 1 << 15, [&](int b, int e, int) {
        for (int i = b; i < e; ++i) {
            if (tmp[i] >= 0) continue;
            double best = 0.0;
            int to = -1;
            for (int k = rp[i]; k < rp[i + 1]; ++k) {
                const int j = ci[k];
                if (j == i || tmp[j] < 0) continue;
                const double w = std::fabs(v[k]);
                if (w > best || (w == best && w > 0.0 && (to < 0 || j < to))) {
                    best = w;
                    to = j;
                }
            }
            late[i] = to >= 0 ? tmp[to] : -1;
            flag[i] = late[i] < 0 ? 1 : 0;
        }
    });
    parallel_chunks(n, 1 << 15, [&](int b, int e, int) {
        for (int i = b; i < e; ++i)
            if (tmp[i] >= 0) flag[i] = 0;
    });
    next += number_flagged(n, flag, id, next);  // rows alone
    parallel_chunks(n, 1 << 15, [&](int b, int e, int) {
        for (int i = b; i < e; ++i)
            if (tmp[i] < 0) tmp[i] = late[i] >= 0 ? late[i] : id[i];
    });
    // number the aggregates by their lowest row
    std::vector<int> renum(next, -1);
    int nc = 0;
    for (int i = 0; i < n; ++i) {
        if (renum[tmp[i]] < 0) renum[tmp[i]] = nc++;
        agg[i] = renum[tmp[i]];
    }
    return nc;
}

// A_c = P^T A P: pattern (columns ascending), values, and for every coarse
// entry the fine entries it sums (gptr/gsrc), in the order they are summed.
void galerkin(const HostCsr& A, const std::vector<int>& agg, int nc, HostCsr& Ac, std::vector<int>& mptr,
              std::vector<int>& mem, std::vector<int>& gptr, std::vector<int>& gsrc) {
    mptr.assign(nc + 1, 0);
    for (int i = 0; i < A.n; ++i) ++mptr[agg[i] + 1];
    for (int c = 0; c < nc; ++c) mptr[c + 1] += mptr[c];
    mem.assign(A.n, 0);
    {
        std::vector<int> fill(mptr.begin(), mptr.end() - 1);
        for (int i = 0; i < A.n; ++i) mem[fill[agg[i]]++] = i;  // ascending within an aggregate
    }
    // coarse rows in chunks, each chunk's rows built apart, then joined in order
    struct Part {
        std::vector<int> rlen, ci, glen, gsrc;
        std::vector<double> v;
    };
    std::vector<Part> parts(16);
    const int nt = parallel_chunks(nc, 4096, [&](int cb, int ce, int t) {
        Part& P = parts[t];
        std::vector<std::pair<int, int>> items;  // (coarse column, fine entry) in summation order
        for (int c = cb; c < ce; ++c) {
            items.clear();
            for (int m = mptr[c]; m < mptr[c + 1]; ++m) {
                const int i = mem[m];
                for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) items.emplace_back(agg[A.ci[k]], k);
            }
            std::stable_sort(items.begin(), items.end(), [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
                return a.first < b.first;
            });
            int len = 0;
            size_t s = 0;
            while (s < items.size()) {
                const int col = items[s].first;
                double sum = 0.0;
                size_t e = s;
                while (e < items.size() && items[e].first == col) {
                    sum += A.v[items[e].second];
                    P.gsrc.push_back(items[e].second);
                    ++e;
                }
                P.ci.push_back(col);
                P.v.push_back(sum);
                P.glen.push_back((int)(e - s));
                ++len;
                s = e;
            }
            P.rlen.push_back(len);
        }
    });
    Ac.n = nc;
    Ac.rp.assign(nc + 1, 0);
    Ac.ci.clear();
    Ac.v.clear();
    gptr.assign(1, 0);
    gsrc.clear();
    gsrc.reserve(A.ci.size());
    int c = 0;
    for (int t = 0; t < nt; ++t) {
        const Part& P = parts[t];
        for (int len : P.rlen) {
            Ac.rp[c + 1] = Ac.rp[c] + len;
            ++c;
        }
        Ac.ci.insert(Ac.ci.end(), P.ci.begin(), P.ci.end());
        Ac.v.insert(Ac.v.end(), P.v.begin(), P.v.end());
        for (int g : P.glen) gptr.push_back(gptr.back() + g);
        gsrc.insert(gsrc.end(), P.gsrc.begin(), P.gsrc.end());
    }
}

// ------------------------------------------------------------ device state
struct AmgState {
    double* x;
    double rel_tol, abs_tol;
    int32_t max_iter;
    double rz, alpha, beta, res0, res, tol;
    int32_t iter, status, done;
    unsigned counter;
    int32_t want_bbase;            // FVGB_SOLVE_RHS_BASELINE: rel_tol is relative to ||b||
    double bbase;                  // ||b|| when asked for (k_bnorm), else -1
    double vinv;                   // FP32 V-cycle: 1/sigma of the residual it was given (sigma_scale)
    fvgb_solver_stats* stats_out;  // device, or null
    fvgb_solver_stats stats;
};

// Levels >= 1 are stored sliced ELL like the system matrix (32-row slices,
// column-major inside a slice, padding slots: column = row, value 0).
struct Level {
    int n = 0, nnz = 0;
    int *sptr = nullptr, *scol = nullptr, *dpos = nullptr;  // levels >= 1 (level 0: the mesh's sliced ELL)
    double *val = nullptr, *dinv = nullptr;
    int* agg = nullptr;                    // [n], when a coarser level follows
    int *mptr = nullptr, *mem = nullptr;   // members of the next level's rows
    int *gptr = nullptr, *gsrc = nullptr;  // sums forming the next level's values
    int* gdst = nullptr;                   // the next level's slot of each sum
    int nnz_next = 0;
    int64_t slots = 0;                     // value slots (level 0: the system's m_len)
    double *b = nullptr, *x = nullptr, *xo = nullptr, *r = nullptr;
    // FP32 copies for the FP32 V-cycle (allocated at the first mixed-precision solve)
    float *valf = nullptr, *dinvf = nullptr, *bf = nullptr, *xf = nullptr, *xof = nullptr, *rf = nullptr;
    // typed views used by the V-cycle builder
    template <class T> T* vals() const;
    template <class T> T* dinvs() const;
    template <class T> T* bs() const;
    template <class T> T* xs() const;
    template <class T> T* xos() const;
    template <class T> T* rs() const;
};
template <> double* Level::vals<double>() const { return val; }
template <> float* Level::vals<float>() const { return valf; }
template <> double* Level::dinvs<double>() const { return dinv; }
template <> float* Level::dinvs<float>() const { return dinvf; }
template <> double* Level::bs<double>() const { return b; }
template <> float* Level::bs<float>() const { return bf; }
template <> double* Level::xs<double>() const { return x; }
template <> float* Level::xs<float>() const { return xf; }
template <> double* Level::xos<double>() const { return xo; }
template <> float* Level::xos<float>() const { return xof; }
template <> double* Level::rs<double>() const { return r; }
template <> float* Level::rs<float>() const { return rf; }

template <class T>
struct TailLevelT;

}  // namespace

struct AmgCache {
    const fvgb_ls* ls = nullptr;
    uint64_t version = 0;
    std::vector<Level> lv;
    int nc = 0;            // rows of the coarsest level
    double* ainv = nullptr;  // [nc*nc] inverse of the coarsest matrix
    double *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr, *part = nullptr;
    AmgState* st = nullptr;
    int tail_from = 1;             // first level run by the single-block tail
    TailLevelT<double>* tail = nullptr;    // device descriptors of levels tail_from..L-1
    cudaGraphExec_t graph = nullptr;
    // the FP32 V-cycle of mixed-precision solves
    bool f32 = false;              // FP32 copies allocated
    uint64_t f32_version = 0;      // matrix version the FP32 copies were made from
    float* ainvf = nullptr;
    TailLevelT<float>* tailf = nullptr;
    cudaGraphExec_t graph32 = nullptr;
    cudaGraphExec_t graph_mg[2] = {nullptr, nullptr};  // the standalone multigrid solver, FP64 / FP32 V-cycle
    std::vector<void*> allocs;
    int nblk = 0;
};

namespace {

template <class T>
cudaError_t dev_alloc(AmgCache* c, T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) c->allocs.push_back(*p);
    return e;
}

template <class T>
cudaError_t upload(AmgCache* c, T** p, const std::vector<T>& h) {
    cudaError_t e = dev_alloc(c, p, h.size());
    if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
    return e;
}

// ------------------------------------------------------------ row access
// Row i of a sliced-ELL matrix with values of type V: f(column, value) for
// every slot, the column and value loads of the first slots issued before the
// caller's gathers.
template <class V>
struct EllRowsT {  // level 0: the system's sliced-ELL matrix (or its FP32 copy)
    MeshView m;
    const V* val;
    template <class F>
    __device__ __forceinline__ void each(int i, F f) const {
        const int slice = i >> 5;
        const int b0 = __ldg(&m.m_ptr[slice]);
        const int base = b0 + (i & 31);
        const int w = (__ldg(&m.m_ptr[slice + 1]) - b0) >> 5;
        int col[8];
        V a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            col[k] = i;
            a[k] = V(0);
            if (k < w) {
                col[k] = slot_col(m, base + k * 32, i);
                a[k] = __ldg(&val[base + k * 32]);
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < w) f(col[k], a[k]);
        for (int k = 8; k < w; ++k) f(slot_col(m, base + k * 32, i), __ldg(&val[base + k * 32]));
    }
};

template <class V>
struct SellRowsT {  // levels >= 1
    const int* ptr;
    const int* col;
    const V* val;
    template <class F>
    __device__ __forceinline__ void each(int i, F f) const {
        const int slice = i >> 5;
        const int b0 = __ldg(&ptr[slice]);
        const int base = b0 + (i & 31);
        const int w = (__ldg(&ptr[slice + 1]) - b0) >> 5;
        constexpr int P = 16;  // coarse rows hold up to ~20 entries
        int c[P];
        V a[P];
#pragma unroll
        for (int k = 0; k < P; ++k) {
            c[k] = i;
            a[k] = V(0);
            if (k < w) {
                c[k] = __ldg(&col[base + k * 32]);
                a[k] = __ldg(&val[base + k * 32]);
            }
        }
#pragma unroll
        for (int k = 0; k < P; ++k)
            if (k < w) f(c[k], a[k]);
        for (int k = P; k < w; ++k) f(__ldg(&col[base + k * 32]), __ldg(&val[base + k * 32]));
    }
};

using EllRows = EllRowsT<double>;
using SellRows = SellRowsT<double>;

__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double block_sum(double v, double* sm) {
    sm[threadIdx.x] = v;
    __syncthreads();
    for (int s = kT / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    const double r = sm[0];
    __syncthreads();
    return r;
}

// Block partial into part[blockIdx.x]; true in the last block to arrive, which
// then sums part[0..gridDim.x) in index order (the same tree every time).
__device__ __forceinline__ bool arrive(AmgState* st, double* part, double partial, double* sm, double* total) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = partial;
        __threadfence();
        last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += kT) s += __ldcg(&part[k]);
    *total = block_sum(s, sm);
    if (threadIdx.x == 0) st->counter = 0;
    return true;
}

__device__ __forceinline__ volatile const int32_t& done_flag(const AmgState* st) { return st->done; }

// ------------------------------------------------------------ numeric setup
__global__ void __launch_bounds__(kT) k_dinv_ell(MeshView m, const double* __restrict__ val, double* __restrict__ dinv) {
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < m.n) dinv[i] = 1.0 / __ldg(&val[__ldg(&m.diag_pos[i])]);
}

__global__ void __launch_bounds__(kT)
    k_galerkin(int nnz_c, const int* __restrict__ gptr, const int* __restrict__ gsrc, const int* __restrict__ gdst,
               const double* __restrict__ vf, double* __restrict__ vc) {
    const int k = blockIdx.x * kT + threadIdx.x;
    if (k >= nnz_c) return;
    double s = 0.0;
    for (int t = __ldg(&gptr[k]); t < __ldg(&gptr[k + 1]); ++t) s += __ldg(&vf[__ldg(&gsrc[t])]);
    vc[__ldg(&gdst[k])] = s;
}

__global__ void __launch_bounds__(kT)
    k_dinv_csr(int n, const int* __restrict__ dpos, const double* __restrict__ val, double* __restrict__ dinv) {
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) dinv[i] = 1.0 / __ldg(&val[__ldg(&dpos[i])]);
}

// dense copy of the coarsest level (padding slots add 0 to the diagonal)
__global__ void __launch_bounds__(kT) k_dense(int n, SellRows rows, double* __restrict__ a) {
    const int i = blockIdx.x;
    for (int j = threadIdx.x; j < n; j += kT) a[(size_t)i * n + j] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0) rows.each(i, [&](int j, double v) { a[(size_t)i * n + j] += v; });
}

// In-place Gauss-Jordan inverse of an n x n SPD matrix, one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_gauss_jordan(int n, double* __restrict__ a) {
    extern __shared__ double f[];  // [n]: column k of the step
    for (int k = 0; k < n; ++k) {
        const double piv = a[(size_t)k * n + k];
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) f[i] = a[(size_t)i * n + k];
        __syncthreads();
        const double ip = 1.0 / piv;
        for (int j = threadIdx.x; j < n; j += blockDim.x) a[(size_t)k * n + j] = (j == k ? 1.0 : a[(size_t)k * n + j]) * ip;
        __syncthreads();
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            const int i = t / n, j = t - i * n;
            if (i == k) continue;
            const double akj = a[(size_t)k * n + j];
            a[(size_t)i * n + j] = (j == k ? 0.0 : a[(size_t)i * n + j]) - f[i] * akj;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ V-cycle
// The V-cycle kernels run in the type T of the V-cycle: double, or float for
// the FP32 V-cycle of a mixed-precision solve (the CG around it stays FP64).

// Level 0's pre-smoothing sweep from zero: x = w D^-1 b
__global__ void __launch_bounds__(kT)
    k_smooth0(const AmgState* st, int n, const double* __restrict__ dinv, const double* __restrict__ b,
              double* __restrict__ x) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) x[i] = kOmega * __ldg(&dinv[i]) * __ldg(&b[i]);
}

// r = b - A x
template <class R, class T>
__global__ void __launch_bounds__(kT)
    k_resid(const AmgState* st, R rows, int n, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ r) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i >= n) return;
    T s = T(0);
    rows.each(i, [&](int j, T a) { s = fmaT(a, __ldg(&x[j]), s); });
    r[i] = __ldg(&b[i]) - s;
}

// b_c[I] = sum of r over the rows of aggregate I, and the coarse level's
// pre-smoothing sweep from zero x_c = w D_c^-1 b_c
template <class T>
__global__ void __launch_bounds__(kT)
    k_restrict(const AmgState* st, int nc, const int* __restrict__ mptr, const int* __restrict__ mem,
               const T* __restrict__ r, const T* __restrict__ dinv_c, T* __restrict__ bc, T* __restrict__ xc) {
    if (done_flag(st)) return;
    const int c = blockIdx.x * kT + threadIdx.x;
    if (c >= nc) return;
    T s = T(0);
    for (int k = __ldg(&mptr[c]); k < __ldg(&mptr[c + 1]); ++k) s += __ldg(&r[__ldg(&mem[k])]);
    bc[c] = s;
    xc[c] = T(kOmega) * __ldg(&dinv_c[c]) * s;
}

// The small levels t..L-1 of a V-cycle in one block of 1024 threads: their
// kernels would each be a few blocks that wait on latency, so one block runs
// the same steps with barriers between them.  Level t's b and x (its
// pre-smoothing sweep) come from the restriction above it; its xo is the
// correction handed back up.
template <class T>
struct TailLevelT {
    int n;
    SellRowsT<T> A;
    const T* dinv;
    const int* agg;   // to level l+1
    const int* mptr;  // members of level l+1's rows
    const int* mem;
    T *b, *x, *xo, *r;
};

template <class T>
__global__ void __launch_bounds__(1024)
    k_tail(const AmgState* st, const TailLevelT<T>* __restrict__ lv, int nl, const T* __restrict__ ainv) {
    if (done_flag(st)) return;
    const int Tt = threadIdx.x, NT = blockDim.x;
    for (int l = 0; l + 1 < nl; ++l) {  // down
        const TailLevelT<T>& F = lv[l];
        const TailLevelT<T>& C = lv[l + 1];
        for (int i = Tt; i < F.n; i += NT) {
            T s = T(0);
            F.A.each(i, [&](int j, T a) { s = fmaT(a, F.x[j], s); });
            F.r[i] = F.b[i] - s;
        }
        __syncthreads();
        for (int c = Tt; c < C.n; c += NT) {
            T s = T(0);
            for (int k = F.mptr[c]; k < F.mptr[c + 1]; ++k) s += F.r[F.mem[k]];
            C.b[c] = s;
            C.x[c] = T(kOmega) * C.dinv[c] * s;
        }
        __syncthreads();
    }
    {  // coarsest: xo = A^-1 b, a warp per row
        const TailLevelT<T>& B = lv[nl - 1];
        const int lane = Tt & 31;
        for (int row = Tt >> 5; row < B.n; row += NT >> 5) {
            T s = T(0);
            for (int j = lane; j < B.n; j += 32) s = fmaT(__ldg(&ainv[(size_t)row * B.n + j]), B.b[j], s);
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) B.xo[row] = s;
        }
        __syncthreads();
    }
    for (int l = nl - 2; l >= 0; --l) {  // up
        const TailLevelT<T>& F = lv[l];
        const TailLevelT<T>& C = lv[l + 1];
        for (int i = Tt; i < F.n; i += NT) F.r[i] = F.x[i] + C.xo[F.agg[i]];
        __syncthreads();
        for (int i = Tt; i < F.n; i += NT) {
            T s = T(0);
            F.A.each(i, [&](int j, T a) { s = fmaT(a, F.r[j], s); });
            F.xo[i] = fmaT(T(kOmega) * F.dinv[i], F.b[i] - s, F.r[i]);
        }
        __syncthreads();
    }
}

// y = x + P xc
template <class T>
__global__ void __launch_bounds__(kT)
    k_prolong(const AmgState* st, int n, const T* __restrict__ x, const T* __restrict__ xc,
              const int* __restrict__ agg, T* __restrict__ y) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) y[i] = __ldg(&x[i]) + __ldg(&xc[__ldg(&agg[i])]);
}

// y = x + P xc; out = y + w D^-1 (b - A y), y formed on the fly (coarse
// levels, where a launch costs more than the extra dependent load)
template <class T>
__global__ void __launch_bounds__(kT)
    k_post_fused(const AmgState* st, SellRowsT<T> rows, int n, const T* __restrict__ dinv, const T* __restrict__ b,
                 const T* __restrict__ x, const T* __restrict__ xc, const int* __restrict__ agg, T* __restrict__ out) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i >= n) return;
    const T yi = __ldg(&x[i]) + __ldg(&xc[__ldg(&agg[i])]);
    T s = T(0);
    rows.each(i, [&](int j, T a) { s = fmaT(a, __ldg(&x[j]) + __ldg(&xc[__ldg(&agg[j])]), s); });
    out[i] = fmaT(T(kOmega) * __ldg(&dinv[i]), __ldg(&b[i]) - s, yi);
}

// out = y + w D^-1 (b - A y), stored as TO (level 0 hands z back as double;
// from the FP32 V-cycle, times 1/sigma of the residual it was given)
template <class R, class T, class TO>
__global__ void __launch_bounds__(kT)
    k_post(const AmgState* st, R rows, int n, const T* __restrict__ dinv, const T* __restrict__ b,
           const T* __restrict__ y, TO* __restrict__ out) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i >= n) return;
    T s = T(0);
    rows.each(i, [&](int j, T a) { s = fmaT(a, __ldg(&y[j]), s); });
    const T v = fmaT(T(kOmega) * __ldg(&dinv[i]), __ldg(&b[i]) - s, __ldg(&y[i]));
    if constexpr (std::is_same<T, float>::value && std::is_same<TO, double>::value)
        out[i] = (double)v * st->vinv;
    else
        out[i] = (TO)v;
}

__global__ void __launch_bounds__(kT) k_to_float(int64_t count, const double* __restrict__ src, float* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
    if (i < count) dst[i] = (float)src[i];
}

// ------------------------------------------------------------ CG
__global__ void k_params(AmgState* st, double* x, double rel_tol, double abs_tol, int max_iter,
                         fvgb_solver_stats* out, int want_bbase) {
    st->want_bbase = want_bbase;
    st->bbase = -1.0;
    st->vinv = 1.0;
    st->x = x;
    st->rel_tol = rel_tol;
    st->abs_tol = abs_tol;
    st->max_iter = max_iter;
    st->stats_out = out;
    st->counter = 0;
    st->done = 0;
}

// The FP32 V-cycle runs on sigma r, sigma = 2^-ilogb(|r_prev|) (the previous
// residual norm, known when the new residual is formed): the residual's entries
// sit near 1 whatever the system's scale, so neither underflow nor overflow
// FP32.  The V-cycle is linear and every FP32 operation commutes exactly with a
// power-of-two scale in the normal range, so z = (double)z_sigma / sigma has
// the bits of the unscaled V-cycle wherever that one stays in range.
__device__ __forceinline__ double sigma_scale(double res) {
    return (res > 0.0 && isfinite(res)) ? ldexp(1.0, -ilogb(res)) : 1.0;
}

// The V-cycle's first sweep from the new residual r_i: x0 = w D^-1 r in FP64,
// or, for the FP32 V-cycle (b0f set), b0 = (float)(sigma r) and x0 = w D^-1 b0
// in FP32; neither when both are null (the FP32 first sweep of a solve runs
// after its initial residual norm, k_first_f32).
__device__ __forceinline__ void first_sweep(int i, double ri, const double* __restrict__ dinv0, double* __restrict__ x0,
                                            const float* __restrict__ d0f, float* __restrict__ b0f,
                                            float* __restrict__ x0f, double sigma) {
    if (b0f) {
        const float bf = (float)(ri * sigma);
        b0f[i] = bf;
        x0f[i] = float(kOmega) * __ldg(&d0f[i]) * bf;
    } else if (x0) {
        x0[i] = kOmega * __ldg(&dinv0[i]) * ri;
    }
}

// The FP32 V-cycle's first sweep from the initial residual, once its norm is known
__global__ void __launch_bounds__(kT)
    k_first_f32(AmgState* st, int n, const double* __restrict__ r, const float* __restrict__ d0f,
                float* __restrict__ b0f, float* __restrict__ x0f) {
    if (done_flag(st)) return;
    const double sigma = sigma_scale(st->res0);
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) first_sweep(i, __ldg(&r[i]), nullptr, nullptr, d0f, b0f, x0f, sigma);
    if (i == 0) st->vinv = 1.0 / sigma;
}

// ||b||, the baseline of the relative tolerance when the solve asks for it
// (Ginkgo's ResidualNorm with its default baseline, rhs_norm)
__global__ void __launch_bounds__(kT) k_bnorm(AmgState* st, int n, const double* __restrict__ b, double* part) {
    __shared__ double sm[kT];
    if (!st->want_bbase) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    const double bi = i < n ? __ldg(&b[i]) : 0.0;
    double tot;
    if (arrive(st, part, block_sum(bi * bi, sm), sm, &tot) && threadIdx.x == 0) st->bbase = sqrt(tot);
}

// r = b - A x, ||r||; the V-cycle's first sweep
__global__ void __launch_bounds__(kT)
    k_init(AmgState* st, EllRows A, int n, const double* __restrict__ b, double* __restrict__ r, double* part,
           const double* __restrict__ dinv0, double* __restrict__ x0, const float* __restrict__ d0f,
           float* __restrict__ b0f, float* __restrict__ x0f) {
    __shared__ double sm[kT];
    const int i = blockIdx.x * kT + threadIdx.x;
    const double* x = st->x;
    double ri = 0.0;
    if (i < n) {
        double s = 0.0;
        A.each(i, [&](int j, double a) { s = fma(a, x[j], s); });
        ri = __ldg(&b[i]) - s;
        r[i] = ri;
        first_sweep(i, ri, dinv0, x0, d0f, b0f, x0f, 1.0);
    }
    double tot;
    if (arrive(st, part, block_sum(ri * ri, sm), sm, &tot) && threadIdx.x == 0) {
        const double res = sqrt(tot);
        st->res0 = st->res = res;
        st->iter = 0;
        st->status = FVGB_OK;
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
}

// p = z, rz = r.z (first direction)
__global__ void __launch_bounds__(kT)
    k_first_dir(AmgState* st, int n, const double* __restrict__ r, const double* __restrict__ z, double* __restrict__ p,
                double* part) {
    __shared__ double sm[kT];
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        const double zi = z[i];
        p[i] = zi;
        v = r[i] * zi;
    }
    double tot;
    if (arrive(st, part, block_sum(v, sm), sm, &tot) && threadIdx.x == 0) st->rz = tot;
}

// q = A p, alpha = rz / p.q
__global__ void __launch_bounds__(kT)
    k_spmv(AmgState* st, EllRows A, int n, const double* __restrict__ p, double* __restrict__ q, double* part) {
    __shared__ double sm[kT];
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        double s = 0.0;
        A.each(i, [&](int j, double a) { s = fma(a, __ldg(&p[j]), s); });
        q[i] = s;
        v = __ldg(&p[i]) * s;
    }
    double tot;
    if (arrive(st, part, block_sum(v, sm), sm, &tot) && threadIdx.x == 0) {
        const double alpha = st->rz / tot;
        st->alpha = alpha;
        if (tot == 0.0 || !isfinite(alpha)) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        }
    }
}

// x += alpha p, r -= alpha q, ||r||, convergence; x0 = w D^-1 r (the V-cycle's first sweep)
__global__ void __launch_bounds__(kT)
    k_update(AmgState* st, int n, const double* __restrict__ p, const double* __restrict__ q, double* __restrict__ r,
             double* part, const double* __restrict__ dinv0, double* __restrict__ x0, const float* __restrict__ d0f,
             float* __restrict__ b0f, float* __restrict__ x0f) {
    __shared__ double sm[kT];
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    const double alpha = st->alpha;
    const double sigma = sigma_scale(st->res);  // the previous residual norm (rewritten by the last block below)
    double* x = st->x;
    double v = 0.0;
    if (i < n) {
        x[i] = fma(alpha, __ldg(&p[i]), x[i]);
        const double ri = fma(-alpha, __ldg(&q[i]), r[i]);
        r[i] = ri;
        first_sweep(i, ri, dinv0, x0, d0f, b0f, x0f, sigma);
        v = ri * ri;
    }
    double tot;
    if (arrive(st, part, block_sum(v, sm), sm, &tot) && threadIdx.x == 0) {
        const double res = sqrt(tot);
        st->res = res;
        st->vinv = 1.0 / sigma;
        st->iter += 1;
        if (!isfinite(res)) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        } else if (res <= st->tol) {
            st->done = 1;
        } else if (st->iter >= st->max_iter) {
            st->status = FVGB_ERR_NOT_CONVERGED;
            st->done = 1;
        }
    }
}

// beta = r.z / rz_old
__global__ void __launch_bounds__(kT)
    k_rz(AmgState* st, int n, const double* __restrict__ r, const double* __restrict__ z, double* part) {
    __shared__ double sm[kT];
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    const double v = i < n ? __ldg(&r[i]) * __ldg(&z[i]) : 0.0;
    double tot;
    if (arrive(st, part, block_sum(v, sm), sm, &tot) && threadIdx.x == 0) {
        st->beta = tot / st->rz;
        st->rz = tot;
        if (!isfinite(st->beta)) {
            st->status = FVGB_ERR_BREAKDOWN;
            st->done = 1;
        }
    }
}

// p = z + beta p
__global__ void __launch_bounds__(kT)
    k_dir(const AmgState* st, int n, const double* __restrict__ z, double* __restrict__ p) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) p[i] = fma(st->beta, p[i], __ldg(&z[i]));
}

// ------------------------------------------------------------ standalone multigrid
// Ginkgo's solver::Multigrid (OpenFOAM's GAMG as FoamAdapter maps it): one
// V-cycle per iteration on the current residual, x += V(b - A x), the
// residual formed again from x, until the criteria hold.  The iteration starts
// with k_init (r = b - A x, its norm, the tolerance, the V-cycle's first sweep).

// x += z
__global__ void __launch_bounds__(kT) k_mg_add(const AmgState* st, int n, const double* __restrict__ z) {
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    double* x = st->x;
    if (i < n) x[i] = x[i] + __ldg(&z[i]);
}

// r = b - A x, ||r||, convergence; the V-cycle's first sweep of the next iteration
__global__ void __launch_bounds__(kT)
    k_mg_resid(AmgState* st, EllRows A, int n, const double* __restrict__ b, double* __restrict__ r, double* part,
               const double* __restrict__ dinv0, double* __restrict__ x0, const float* __restrict__ d0f,
               float* __restrict__ b0f, float* __restrict__ x0f) {
    __shared__ double sm[kT];
    if (done_flag(st)) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    const double sigma = sigma_scale(st->res);  // the previous residual norm (rewritten by the last block below)
    const double* x = st->x;
    double ri = 0.0;
    if (i < n) {
        double s = 0.0;
        A.each(i, [&](int j, double a) { s = fma(a, x[j], s); });
        ri = __ldg(&b[i]) - s;
        r[i] = ri;
        first_sweep(i, ri, dinv0, x0, d0f, b0f, x0f, sigma);
    }
    double tot;
    if (arrive(st, part, block_sum(ri * ri, sm), sm, &tot) && threadIdx.x == 0) {
        const double res = sqrt(tot);
        st->res = res;
        st->vinv = 1.0 / sigma;
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
}

__global__ void k_cond(AmgState* st, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, st->done ? 0u : 1u);
}

__global__ void k_stats(AmgState* st) {
    fvgb_solver_stats s{};
    s.init_res_norm = st->res0;
    s.final_res_norm = st->res;
    s.num_iter = st->iter;
    s.num_outer = 0;
    s.status = st->status;
    st->stats = s;
    if (st->stats_out) *st->stats_out = s;
}

// ------------------------------------------------------------ host side
fvgb_status symbolic(AmgCache* c, cudaStream_t s) {
    const fvgb_ls* ls = c->ls;
    const fvgb_mesh* mesh = ls->mesh;
    const int n = mesh->v.n, nnz = mesh->nnz;
    if ((int)mesh->h_row_offs.size() != n + 1 || (int)mesh->h_col.size() != nnz)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "multigrid: the mesh keeps no host sparsity pattern (device-built boxes)");
    // level 0 in CSR on the host: pattern from the mesh, values from the device
    std::vector<int> csr_pos(nnz);
    std::vector<double> slots(mesh->m_len);
    FVGB_CUDA_TRY(cudaStreamSynchronize(s));
    FVGB_CUDA_TRY(cudaMemcpy(csr_pos.data(), mesh->csr_pos, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    FVGB_CUDA_TRY(cudaMemcpy(slots.data(), ls->values, sizeof(double) * mesh->m_len, cudaMemcpyDeviceToHost));
    HostCsr A;
    A.n = n;
    A.rp = mesh->h_row_offs;
    A.ci = mesh->h_col;
    A.v.resize(nnz);
    for (int k = 0; k < nnz; ++k) A.v[k] = slots[csr_pos[k]];
    c->lv.clear();
    c->lv.emplace_back();
    c->lv[0].n = n;
    c->lv[0].nnz = nnz;
    c->lv[0].slots = mesh->m_len;
    std::vector<int> slot_of = csr_pos;  // the current level's slot of each of its CSR entries
    while ((int)c->lv.size() < kMaxLevels && A.n > kCoarseRows) {
        // two rounds of pairwise matching per level (double pairwise): the pairs
        // of the first round are matched again on their Galerkin matrix, so a
        // level has about a quarter of the rows and half as many levels are
        // needed
        std::vector<int> agg;
        int nc = pgm_aggregate(A.n, A.rp.data(), A.ci.data(), A.v.data(), agg);
        if (nc > 0.9 * A.n) break;
        if (nc > kCoarseRows) {
            HostCsr A1;
            std::vector<int> m1, e1, g1, s1, agg2;
            galerkin(A, agg, nc, A1, m1, e1, g1, s1);
            const int nc2 = pgm_aggregate(A1.n, A1.rp.data(), A1.ci.data(), A1.v.data(), agg2);
            if (nc2 <= 0.9 * nc) {
                for (int& a : agg) a = agg2[a];
                nc = nc2;
                // aggregates numbered by their lowest row again
                std::vector<int> renum(nc, -1);
                int k = 0;
                for (int& a : agg) {
                    if (renum[a] < 0) renum[a] = k++;
                    a = renum[a];
                }
            }
        }
        HostCsr Ac;
        std::vector<int> mptr, mem, gptr, gsrc;
        galerkin(A, agg, nc, Ac, mptr, mem, gptr, gsrc);
        Level& L = c->lv.back();
        for (int& k : gsrc) k = slot_of[k];  // the sums read the fine level's sliced-ELL slots
        cudaError_t e = upload(c, &L.agg, agg);
        if (e == cudaSuccess) e = upload(c, &L.mptr, mptr);
        if (e == cudaSuccess) e = upload(c, &L.mem, mem);
        if (e == cudaSuccess) e = upload(c, &L.gptr, gptr);
        if (e == cudaSuccess) e = upload(c, &L.gsrc, gsrc);
        if (e != cudaSuccess) return cuda_fail(e, "multigrid setup");
        L.nnz_next = (int)Ac.ci.size();
        Level C;
        C.n = Ac.n;
        C.nnz = (int)Ac.ci.size();
        // sliced ELL of the coarse matrix; gdst: the slot of each CSR entry
        const int ns = (Ac.n + 31) / 32;
        std::vector<int> sptr(ns + 1, 0);
        for (int sl = 0; sl < ns; ++sl) {
            int w = 0;
            for (int i = sl * 32; i < std::min(Ac.n, sl * 32 + 32); ++i) w = std::max(w, Ac.rp[i + 1] - Ac.rp[i]);
            sptr[sl + 1] = sptr[sl] + 32 * w;
        }
        std::vector<int> scol(sptr[ns]), gdst(C.nnz), dpos(Ac.n, -1);
        for (int i = 0; i < Ac.n; ++i) {
            const int base = sptr[i / 32] + (i & 31), w = (sptr[i / 32 + 1] - sptr[i / 32]) / 32;
            for (int k = 0; k < w; ++k) scol[base + 32 * k] = i;  // padding
            for (int k = Ac.rp[i]; k < Ac.rp[i + 1]; ++k) {
                const int pos = base + 32 * (k - Ac.rp[i]);
                scol[pos] = Ac.ci[k];
                gdst[k] = pos;
                if (Ac.ci[k] == i) dpos[i] = pos;
            }
        }
        for (int i = 0; i < Ac.n; ++i)
            if (dpos[i] < 0) return fvgb_fail(FVGB_ERR_INVALID_ARG, "multigrid: a coarse row without a diagonal entry");
        C.slots = std::max(1, sptr[ns]);
        e = upload(c, &L.gdst, gdst);
        if (e == cudaSuccess) e = upload(c, &C.sptr, sptr);
        if (e == cudaSuccess) e = upload(c, &C.scol, scol);
        if (e == cudaSuccess) e = upload(c, &C.dpos, dpos);
        if (e == cudaSuccess) e = dev_alloc(c, &C.val, (size_t)std::max(1, sptr[ns]));
        if (e == cudaSuccess) e = cudaMemset(C.val, 0, sizeof(double) * (size_t)std::max(1, sptr[ns]));
        if (e != cudaSuccess) return cuda_fail(e, "multigrid setup");
        c->lv.push_back(C);
        slot_of = std::move(gdst);
        A = std::move(Ac);
    }
    if (c->lv.size() < 2) return fvgb_fail(FVGB_ERR_UNSUPPORTED, "multigrid: the system does not coarsen (too small?)");
    c->nc = c->lv.back().n;
    if (c->nc > 1024) return fvgb_fail(FVGB_ERR_UNSUPPORTED, "multigrid: the coarsest level keeps above 1024 rows");
    for (size_t l = 0; l < c->lv.size(); ++l) {
        Level& L = c->lv[l];
        cudaError_t e = dev_alloc(c, &L.dinv, (size_t)L.n);
        if (e == cudaSuccess) e = dev_alloc(c, &L.x, (size_t)L.n);
        if (e == cudaSuccess) e = dev_alloc(c, &L.xo, (size_t)L.n);
        if (e == cudaSuccess) e = dev_alloc(c, &L.r, (size_t)L.n);
        if (e == cudaSuccess && l > 0) e = dev_alloc(c, &L.b, (size_t)L.n);
        if (e != cudaSuccess) return cuda_fail(e, "multigrid vectors");
    }
    {
        const int L = (int)c->lv.size();
        int t = 1;
        while (t < L - 1 && c->lv[t].n > kTailRows) ++t;
        c->tail_from = t;
        std::vector<TailLevelT<double>> tl;
        for (int l = t; l < L; ++l) {
            const Level& V = c->lv[l];
            tl.push_back(TailLevelT<double>{V.n, SellRows{V.sptr, V.scol, V.val}, V.dinv, V.agg, V.mptr, V.mem, V.b,
                                            V.x, V.xo, V.r});
        }
        cudaError_t e = upload(c, &c->tail, tl);
        if (e != cudaSuccess) return cuda_fail(e, "multigrid setup");
    }
    c->nblk = (int)grid_for(n, kT);
    cudaError_t e = dev_alloc(c, &c->ainv, (size_t)c->nc * c->nc);
    if (e == cudaSuccess) e = dev_alloc(c, &c->r, (size_t)n);
    if (e == cudaSuccess) e = dev_alloc(c, &c->p, (size_t)n);
    if (e == cudaSuccess) e = dev_alloc(c, &c->q, (size_t)n);
    if (e == cudaSuccess) e = dev_alloc(c, &c->z, (size_t)n);
    if (e == cudaSuccess) e = dev_alloc(c, &c->part, (size_t)c->nblk);
    if (e == cudaSuccess) e = dev_alloc(c, &c->st, 1);
    if (e == cudaSuccess) e = cudaMemset(c->st, 0, sizeof(AmgState));
    if (e != cudaSuccess) return cuda_fail(e, "multigrid vectors");
    FVGB_CUDA_TRY(settle_creation());
    return FVGB_OK;
}

fvgb_status numeric(AmgCache* c, cudaStream_t s) {
    const fvgb_ls* ls = c->ls;
    const MeshView m = ls->mesh->v;
    k_dinv_ell<<<grid_for(m.n, kT), kT, 0, s>>>(m, ls->values, c->lv[0].dinv);
    for (size_t l = 0; l + 1 < c->lv.size(); ++l) {
        const Level& F = c->lv[l];
        Level& C = c->lv[l + 1];
        const double* vf = l == 0 ? ls->values : F.val;
        k_galerkin<<<grid_for(C.nnz, kT), kT, 0, s>>>(C.nnz, F.gptr, F.gsrc, F.gdst, vf, C.val);
        k_dinv_csr<<<grid_for(C.n, kT), kT, 0, s>>>(C.n, C.dpos, C.val, C.dinv);
    }
    const Level& B = c->lv.back();
    k_dense<<<B.n, kT, 0, s>>>(B.n, SellRows{B.sptr, B.scol, B.val}, c->ainv);
    k_gauss_jordan<<<1, 1024, sizeof(double) * B.n, s>>>(B.n, c->ainv);
    FVGB_LAUNCH_CHECK("multigrid numeric setup");
    c->version = ls->version;
    return FVGB_OK;
}

// FP32 copies of the level matrices, diagonals and coarsest inverse
fvgb_status to_f32(AmgCache* c, cudaStream_t s) {
    const fvgb_ls* ls = c->ls;
    if (!c->f32) {
        for (size_t l = 0; l < c->lv.size(); ++l) {
            Level& V = c->lv[l];
            cudaError_t e = dev_alloc(c, &V.valf, (size_t)V.slots);
            if (e == cudaSuccess) e = dev_alloc(c, &V.dinvf, (size_t)V.n);
            if (e == cudaSuccess) e = dev_alloc(c, &V.bf, (size_t)V.n);
            if (e == cudaSuccess) e = dev_alloc(c, &V.xf, (size_t)V.n);
            if (e == cudaSuccess) e = dev_alloc(c, &V.xof, (size_t)V.n);
            if (e == cudaSuccess) e = dev_alloc(c, &V.rf, (size_t)V.n);
            if (e != cudaSuccess) return cuda_fail(e, "multigrid FP32 copies");
        }
        cudaError_t e = dev_alloc(c, &c->ainvf, (size_t)c->nc * c->nc);
        std::vector<TailLevelT<float>> tl;
        for (int l = c->tail_from; l < (int)c->lv.size(); ++l) {
            const Level& V = c->lv[l];
            tl.push_back(TailLevelT<float>{V.n, SellRowsT<float>{V.sptr, V.scol, V.valf}, V.dinvf, V.agg, V.mptr, V.mem,
                                           V.bf, V.xf, V.xof, V.rf});
        }
        if (e == cudaSuccess) e = upload(c, &c->tailf, tl);
        if (e != cudaSuccess) return cuda_fail(e, "multigrid FP32 copies");
        c->f32 = true;
    }
    for (size_t l = 0; l < c->lv.size(); ++l) {
        const Level& V = c->lv[l];
        const double* src = l == 0 ? ls->values : V.val;
        k_to_float<<<grid_for(V.slots, kT), kT, 0, s>>>(V.slots, src, V.valf);
        k_to_float<<<grid_for(V.n, kT), kT, 0, s>>>(V.n, V.dinv, V.dinvf);
    }
    k_to_float<<<grid_for((int64_t)c->nc * c->nc, kT), kT, 0, s>>>((int64_t)c->nc * c->nc, c->ainv, c->ainvf);
    FVGB_LAUNCH_CHECK("multigrid FP32 copies");
    c->f32_version = ls->version;
    return FVGB_OK;
}

cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t* dep, void* func, unsigned grid,
                       unsigned block, void** args, unsigned smem = 0) {
    cudaKernelNodeParams kp{};
    kp.func = func;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(block);
    kp.sharedMemBytes = smem;
    kp.kernelParams = args;
    kp.extra = nullptr;
    const bool has_dep = dep && *dep;  // a null predecessor node means: no dependency
    return cudaGraphAddKernelNode(node, g, has_dep ? dep : nullptr, has_dep ? 1 : 0, &kp);
}

// The V-cycle z = M r as a chain of kernel nodes after *prev: levels
// 0..t-1 one kernel per step, levels t..L-1 in the single-block tail.  T is
// the V-cycle's type; with T = float, level 0's b and x are FP32 copies the
// CG kernels write and z comes back as double.
template <class T>
struct VcycleArgs {
    std::vector<std::vector<void*>> args;
    std::vector<EllRowsT<T>> ell;
    std::vector<SellRowsT<T>> sell;
    std::vector<int> ns;
    std::vector<const T*> bs;
    std::vector<T*> outs;
    std::vector<T*> xcs;
    std::vector<T*> dv, xv, rv, bv;
    int nl_tail = 0;
    const TailLevelT<T>* tail = nullptr;
    const T* ainv = nullptr;
};

template <class T> const T* ainv_of(const AmgCache* c);
template <> const double* ainv_of<double>(const AmgCache* c) { return c->ainv; }
template <> const float* ainv_of<float>(const AmgCache* c) { return c->ainvf; }
template <class T> const TailLevelT<T>* tail_of(const AmgCache* c);
template <> const TailLevelT<double>* tail_of<double>(const AmgCache* c) { return c->tail; }
template <> const TailLevelT<float>* tail_of<float>(const AmgCache* c) { return c->tailf; }

// r_in: level 0's b (double* for T = double; the FP32 copy otherwise).
// z_out: the result (always double).  first_sweep_done: level 0's x was
// formed by the kernel that produced r_in.
template <class T>
cudaError_t add_vcycle(AmgCache* c, cudaGraph_t g, cudaGraphNode_t* prev, const T* r_in, double* z_out,
                       VcycleArgs<T>& va, bool first_sweep_done = false) {
    const size_t L = c->lv.size();
    const size_t t = (size_t)c->tail_from;
    if (!first_sweep_done && !std::is_same<T, double>::value) return cudaErrorInvalidValue;  // FP64 only
    va.ell.assign(1, EllRowsT<T>{c->ls->mesh->v, c->lv[0].vals<T>() ? c->lv[0].vals<T>() : nullptr});
    if (std::is_same<T, double>::value) va.ell[0].val = (const T*)c->ls->values;
    va.sell.resize(L);
    for (size_t l = 1; l < L; ++l) va.sell[l] = SellRowsT<T>{c->lv[l].sptr, c->lv[l].scol, c->lv[l].vals<T>()};
    va.ns.resize(L);
    va.bs.resize(L);
    va.outs.resize(L);
    va.xcs.resize(L);
    va.dv.resize(L);
    va.xv.resize(L);
    va.rv.resize(L);
    va.bv.resize(L);
    va.args.clear();
    va.args.reserve(6 * L + 4);
    for (size_t l = 0; l < L; ++l) {
        const Level& V = c->lv[l];
        va.ns[l] = V.n;
        va.bs[l] = l == 0 ? r_in : V.bs<T>();
        va.outs[l] = V.xos<T>();
        va.dv[l] = V.dinvs<T>();
        va.xv[l] = V.xs<T>();
        va.rv[l] = V.rs<T>();
        va.bv[l] = V.bs<T>();
    }
    va.nl_tail = (int)(L - t);
    va.tail = tail_of<T>(c);
    va.ainv = ainv_of<T>(c);
    double* z = z_out;
    cudaError_t e = cudaSuccess;
    cudaGraphNode_t node;
    auto add = [&](void* fn, unsigned grid, unsigned block) {
        if (e != cudaSuccess) return;
        e = add_kernel(g, &node, prev, fn, grid, block, va.args.back().data());
        if (e == cudaSuccess) *prev = node;
    };
    for (size_t l = 0; l < t && e == cudaSuccess; ++l) {  // down
        Level& F = c->lv[l];
        if (l == 0) {
            if (!first_sweep_done) {  // the solve's CG kernels form x0 = w D^-1 r themselves
                va.args.push_back({&c->st, &va.ns[0], &F.dinv, &va.bs[0], &F.x});
                add((void*)k_smooth0, grid_for(F.n, kT), kT);
            }
            va.args.push_back({&c->st, &va.ell[0], &va.ns[0], &va.bs[0], &va.xv[0], &va.rv[0]});
            add((void*)k_resid<EllRowsT<T>, T>, grid_for(F.n, kT), kT);
        } else {
            va.args.push_back({&c->st, &va.sell[l], &va.ns[l], &va.bs[l], &va.xv[l], &va.rv[l]});
            add((void*)k_resid<SellRowsT<T>, T>, grid_for(F.n, kT), kT);
        }
        Level& C = c->lv[l + 1];
        va.args.push_back({&c->st, &va.ns[l + 1], &F.mptr, &F.mem, &va.rv[l], &va.dv[l + 1], &va.bv[l + 1], &va.xv[l + 1]});
        add((void*)k_restrict<T>, grid_for(C.n, kT), kT);
    }
    va.args.push_back({&c->st, &va.tail, &va.nl_tail, &va.ainv});
    add((void*)k_tail<T>, 1, 1024);
    for (size_t l = t; l-- > 0 && e == cudaSuccess;) {  // up
        Level& F = c->lv[l];
        va.xcs[l] = va.outs[l + 1];
        if (l == 0) {
            va.args.push_back({&c->st, &va.ns[l], &va.xv[l], &va.xcs[l], &F.agg, &va.rv[l]});  // y = x + P xc
            add((void*)k_prolong<T>, grid_for(F.n, kT), kT);
            va.args.push_back({&c->st, &va.ell[0], &va.ns[l], &va.dv[l], &va.bs[l], &va.rv[l], &z});
            add((void*)k_post<EllRowsT<T>, T, double>, grid_for(F.n, kT), kT);
        } else {
            va.args.push_back({&c->st, &va.sell[l], &va.ns[l], &va.dv[l], &va.bs[l], &va.xv[l], &va.xcs[l], &F.agg,
                               &va.outs[l]});
            add((void*)k_post_fused<T>, grid_for(F.n, kT), kT);
        }
    }
    return e;
}

fvgb_status build_graph(AmgCache* c, bool f32) {
    cudaGraphExec_t& out = f32 ? c->graph32 : c->graph;
    if (out) {
        cudaGraphExecDestroy(out);
        out = nullptr;
    }
    const fvgb_ls* ls = c->ls;
    EllRows A{ls->mesh->v, ls->values};
    int n = ls->mesh->v.n;
    const unsigned nb = (unsigned)c->nblk;
    const double* b = ls->rhs;
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    cudaGraphNode_t prev = nullptr, node;
    VcycleArgs<double> v0, v1;
    VcycleArgs<float> f0, f1;
    // FP64 V-cycle: the CG kernels write x0 (double); FP32: b0 and x0 as float
    double* x0 = f32 ? nullptr : c->lv[0].x;
    const float* d0f = f32 ? c->lv[0].dinvf : nullptr;
    float* b0f = f32 ? c->lv[0].bf : nullptr;
    float* x0f = f32 ? c->lv[0].xf : nullptr;
    // FP32: k_init forms no sweep (its norm is not known yet), k_first_f32 follows it
    float* nof = nullptr;
    void* a_init[] = {&c->st, &A, &n, &b, &c->r, &c->part, &c->lv[0].dinv, &x0, &d0f, f32 ? &nof : &b0f, &x0f};
    void* a_f32[] = {&c->st, &n, &c->r, &d0f, &b0f, &x0f};
    void* a_first[] = {&c->st, &n, &c->r, &c->z, &c->p, &c->part};
    void* a_cond[] = {&c->st, &h};
    void* a_spmv[] = {&c->st, &A, &n, &c->p, &c->q, &c->part};
    void* a_upd[] = {&c->st, &n, &c->p, &c->q, &c->r, &c->part, &c->lv[0].dinv, &x0, &d0f, &b0f, &x0f};
    void* a_rz[] = {&c->st, &n, &c->r, &c->z, &c->part};
    void* a_dir[] = {&c->st, &n, &c->z, &c->p};
    void* a_stats[] = {&c->st};
    void* a_bnorm[] = {&c->st, &n, &b, &c->part};
    if (e == cudaSuccess) e = add_kernel(g, &node, nullptr, (void*)k_bnorm, nb, kT, a_bnorm);
    prev = node;
    if (e == cudaSuccess) e = add_kernel(g, &node, &prev, (void*)k_init, nb, kT, a_init);
    prev = node;
    if (e == cudaSuccess && f32) {
        e = add_kernel(g, &node, &prev, (void*)k_first_f32, nb, kT, a_f32);
        prev = node;
    }
    if (e == cudaSuccess)
        e = f32 ? add_vcycle<float>(c, g, &prev, b0f, c->z, f0, true) : add_vcycle<double>(c, g, &prev, c->r, c->z, v0, true);
    if (e == cudaSuccess) e = add_kernel(g, &node, &prev, (void*)k_first_dir, nb, kT, a_first);
    prev = node;
    if (e == cudaSuccess) e = add_kernel(g, &node, &prev, (void*)k_cond, 1, 1, a_cond);
    prev = node;
    cudaGraph_t body = nullptr;
    if (e == cudaSuccess) {
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&node, g, &prev, nullptr, 1, &np);
        if (e == cudaSuccess) body = np.conditional.phGraph_out[0];
        prev = node;
    }
    cudaGraphNode_t bprev = nullptr, bnode;
    if (e == cudaSuccess) e = add_kernel(body, &bnode, nullptr, (void*)k_spmv, nb, kT, a_spmv);
    bprev = bnode;
    if (e == cudaSuccess) e = add_kernel(body, &bnode, &bprev, (void*)k_update, nb, kT, a_upd);
    bprev = bnode;
    if (e == cudaSuccess)
        e = f32 ? add_vcycle<float>(c, body, &bprev, b0f, c->z, f1, true)
                : add_vcycle<double>(c, body, &bprev, c->r, c->z, v1, true);
    if (e == cudaSuccess) e = add_kernel(body, &bnode, &bprev, (void*)k_rz, nb, kT, a_rz);
    bprev = bnode;
    if (e == cudaSuccess) e = add_kernel(body, &bnode, &bprev, (void*)k_dir, nb, kT, a_dir);
    bprev = bnode;
    if (e == cudaSuccess) e = add_kernel(body, &bnode, &bprev, (void*)k_cond, 1, 1, a_cond);
    if (e == cudaSuccess) e = add_kernel(g, &node, &prev, (void*)k_stats, 1, 1, a_stats);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "multigrid CG graph");
    return FVGB_OK;
}

// The standalone multigrid solve as one graph: k_init, then a device-side
// while loop over {V-cycle, x += z, r = b - A x}, bounded by max_iter.
fvgb_status build_graph_mg(AmgCache* c, bool f32) {
    cudaGraphExec_t& out = c->graph_mg[f32 ? 1 : 0];
    if (out) {
        cudaGraphExecDestroy(out);
        out = nullptr;
    }
    const fvgb_ls* ls = c->ls;
    EllRows A{ls->mesh->v, ls->values};
    int n = ls->mesh->v.n;
    const unsigned nb = (unsigned)c->nblk;
    const double* b = ls->rhs;
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    cudaGraphNode_t prev = nullptr, node;
    VcycleArgs<double> v1;
    VcycleArgs<float> f1;
    double* x0 = f32 ? nullptr : c->lv[0].x;
    const float* d0f = f32 ? c->lv[0].dinvf : nullptr;
    float* b0f = f32 ? c->lv[0].bf : nullptr;
    float* x0f = f32 ? c->lv[0].xf : nullptr;
    float* nof = nullptr;
    void* a_init[] = {&c->st, &A, &n, &b, &c->r, &c->part, &c->lv[0].dinv, &x0, &d0f, f32 ? &nof : &b0f, &x0f};
    void* a_f32[] = {&c->st, &n, &c->r, &d0f, &b0f, &x0f};
    void* a_cond[] = {&c->st, &h};
    void* a_add[] = {&c->st, &n, &c->z};
    void* a_res[] = {&c->st, &A, &n, &b, &c->r, &c->part, &c->lv[0].dinv, &x0, &d0f, &b0f, &x0f};
    void* a_stats[] = {&c->st};
    void* a_bnorm[] = {&c->st, &n, &b, &c->part};
    if (e == cudaSuccess) e = add_kernel(g, &node, nullptr, (void*)k_bnorm, nb, kT, a_bnorm);
    prev = node;
    if (e == cudaSuccess) e = add_kernel(g, &node, &prev, (void*)k_init, nb, kT, a_init);
    prev = node;
    if (e == cudaSuccess && f32) {
        e = add_kernel(g, &node, &prev, (void*)k_first_f32, nb, kT, a_f32);
        prev = node;
    }
    if (e == cudaSuccess) e = add_kernel(g, &node, &prev, (void*)k_cond, 1, 1, a_cond);
    prev = node;
    cudaGraph_t body = nullptr;
    if (e == cudaSuccess) {
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&node, g, &prev, nullptr, 1, &np);
        if (e == cudaSuccess) body = np.conditional.phGraph_out[0];
        prev = node;
    }
    cudaGraphNode_t bprev = nullptr, bnode;
    if (e == cudaSuccess)
        e = f32 ? add_vcycle<float>(c, body, &bprev, b0f, c->z, f1, true)
                : add_vcycle<double>(c, body, &bprev, c->r, c->z, v1, true);
    if (e == cudaSuccess) e = add_kernel(body, &bnode, &bprev, (void*)k_mg_add, nb, kT, a_add);
    bprev = bnode;
    if (e == cudaSuccess) e = add_kernel(body, &bnode, &bprev, (void*)k_mg_resid, nb, kT, a_res);
    bprev = bnode;
    if (e == cudaSuccess) e = add_kernel(body, &bnode, &bprev, (void*)k_cond, 1, 1, a_cond);
    if (e == cudaSuccess) e = add_kernel(g, &node, &prev, (void*)k_stats, 1, 1, a_stats);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "multigrid solver graph");
    return FVGB_OK;
}

fvgb_status prepare(fvgb_ls* ls, cudaStream_t s, bool f32 = false) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FVGB_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (!ls->amg) {
        if (cs != cudaStreamCaptureStatusNone)
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "multigrid: the first solve (setup) cannot be stream-captured");
        AmgCache* c = new AmgCache();
        c->ls = ls;
        fvgb_status st = symbolic(c, s);
        if (st == FVGB_OK) st = build_graph(c, false);
        if (st != FVGB_OK) {
            fvgb_amg_free(c);
            return st;
        }
        ls->amg = c;
    }
    AmgCache* c = ls->amg;
    if (c->version != ls->version) {
        fvgb_status st = numeric(c, s);
        if (st != FVGB_OK) return st;
    }
    if (f32) {
        // the first FP32 V-cycle allocates its copies, uploads their descriptors and
        // builds its graph: none of that may happen inside a caller's capture
        if (!c->f32 && cs != cudaStreamCaptureStatusNone)
            return fvgb_fail(FVGB_ERR_UNSUPPORTED,
                             "multigrid: the first mixed-precision solve (FP32 setup) cannot be stream-captured");
        if (!c->f32 || c->f32_version != ls->version) {
            const bool first = !c->f32;
            fvgb_status st = to_f32(c, s);
            if (st != FVGB_OK) return st;
            if (first) {
                FVGB_CUDA_TRY(cudaStreamSynchronize(s));
                st = build_graph(c, true);
                if (st != FVGB_OK) return st;
            }
        }
    }
    return FVGB_OK;
}

}  // namespace

void fvgb_amg_free(AmgCache* c) {
    if (!c) return;
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->graph32) cudaGraphExecDestroy(c->graph32);
    for (cudaGraphExec_t g : c->graph_mg)
        if (g) cudaGraphExecDestroy(g);
    for (void* p : c->allocs) cudaFree(p);
    delete c;
}

fvgb_status fvgb_amg_solve_async(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats_dev,
                                 cudaStream_t s) {
    if (ls->ncomp != 1) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_solve: scalar systems only");
    const bool standalone = cfg->method == FVGB_SOLVER_MULTIGRID;
    if (cfg->method != FVGB_SOLVER_CG && !standalone)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "multigrid: as the preconditioner of CG only");
    FVGB_CHECK_ARG(cfg->precision == FVGB_PREC_FP64 || cfg->precision == FVGB_PREC_MIXED_IR,
                   "fvgb_solve: unknown precision");
    FVGB_CHECK_ARG(cfg->rel_tol >= 0 && cfg->abs_tol >= 0, "fvgb_solve: negative tolerance");
    FVGB_CHECK_ARG(cfg->max_iter >= 0 && cfg->max_iter <= 100000000, "fvgb_solve: bad max_iter");
    FVGB_CHECK_ARG((cfg->flags & ~(FVGB_SOLVE_NO_TUNE | FVGB_SOLVE_RHS_BASELINE)) == 0, "fvgb_solve: unknown flags");
    // mixed precision: the CG (or the multigrid iteration), its residuals and
    // its stopping test stay FP64; the V-cycle runs in FP32
    const bool f32 = cfg->precision == FVGB_PREC_MIXED_IR;
    fvgb_status st = prepare(ls, s, f32);
    if (st != FVGB_OK) return st;
    AmgCache* c = ls->amg;
    if (standalone && !c->graph_mg[f32 ? 1 : 0]) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        FVGB_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "multigrid: the first solve of the multigrid solver cannot be stream-captured");
        st = build_graph_mg(c, f32);
        if (st != FVGB_OK) return st;
    }
    k_params<<<1, 1, 0, s>>>(c->st, x, cfg->rel_tol, cfg->abs_tol, cfg->max_iter, stats_dev,
                             (cfg->flags & FVGB_SOLVE_RHS_BASELINE) ? 1 : 0);
    FVGB_LAUNCH_CHECK("multigrid params");
    FVGB_CUDA_TRY(cudaGraphLaunch(standalone ? c->graph_mg[f32 ? 1 : 0] : (f32 ? c->graph32 : c->graph), s));
    return FVGB_OK;
}

fvgb_status fvgb_amg_sync_stats(fvgb_ls* ls, fvgb_solver_stats* out, cudaStream_t s) {
    AmgCache* c = ls->amg;
    fvgb_solver_stats h{};
    FVGB_CUDA_TRY(cudaMemcpyAsync(&h, &c->st->stats, sizeof h, cudaMemcpyDeviceToHost, s));
    FVGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (out) *out = h;
    return (fvgb_status)(h.status == FVGB_ERR_NOT_CONVERGED ? FVGB_ERR_NOT_CONVERGED
                                                             : (h.status == FVGB_OK ? FVGB_OK : h.status));
}

extern "C" fvgb_status fvgb_amg_apply(fvgb_ls* ls, const double* r, double* z, fvgb_stream stream) {
    FVGB_CHECK_ARG(ls && r && z, "fvgb_amg_apply: null argument");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_amg_apply: scalar systems only");
    cudaStream_t s = (cudaStream_t)stream;
    fvgb_status st = prepare(ls, s);
    if (st != FVGB_OK) return st;
    AmgCache* c = ls->amg;
    // a one-off graph of the V-cycle alone, with the done flag cleared
    k_params<<<1, 1, 0, s>>>(c->st, nullptr, 0.0, 0.0, 0, nullptr, 0);
    cudaGraph_t g = nullptr;
    FVGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphNode_t prev = nullptr;
    VcycleArgs<double> va;
    cudaError_t e = add_vcycle<double>(c, g, &prev, r, z, va);
    cudaGraphExec_t ge = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(ge, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (ge) cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "fvgb_amg_apply");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_amg_info(fvgb_ls* ls, int32_t* nlevels, int32_t* rows, int64_t* nnz, int32_t cap) {
    FVGB_CHECK_ARG(ls && nlevels, "fvgb_amg_info: null argument");
    if (!ls->amg) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_amg_info: no multigrid hierarchy yet (solve first)");
    const AmgCache* c = ls->amg;
    *nlevels = (int32_t)c->lv.size();
    for (int32_t l = 0; l < *nlevels && l < cap; ++l) {
        if (rows) rows[l] = c->lv[l].n;
        if (nnz) nnz[l] = c->lv[l].nnz;
    }
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_pgm_aggregate(int32_t n, const int32_t* row_offs, const int32_t* cols,
                                          const double* values, int32_t* agg, int32_t* n_coarse) {
    FVGB_CHECK_ARG(n >= 0 && row_offs && cols && values && agg && n_coarse, "fvgb_pgm_aggregate: null argument");
    std::vector<int> a;
    *n_coarse = pgm_aggregate(n, row_offs, cols, values, a);
    std::memcpy(agg, a.data(), sizeof(int32_t) * (size_t)n);
    return FVGB_OK;
}
