// Internal definitions of libfvgb: the device-resident mesh and linear-system
// handles and the index layouts the kernels read.
//
// Layouts (all device arrays):
//  * Gather lists: for every cell the faces it touches, in ascending face
//    index (internal faces, then its boundary faces), stored sliced-ELL with
//    32-cell slices, column-major inside a slice: entry k of cell c sits at
//    g_ptr[c/32] + 32*k + c%32.  g_code: 0 <= code < nif: c owns internal face
//    `code`; code < 0: c is the neighbour of face -code-1; code >= nif: boundary
//    face code-nif; FVGB_PAD: padding (only at the end of a row).  g_other: the
//    cell across an internal face.
//  * Matrix: the CSR pattern of NeoN (row = [lower, diagonal, upper] in column
//    order) stored sliced-ELL the same way: m_ptr, m_col, values.  m_code per
//    slot: code >= 0: a_PN with P the owner of face code; code <= -2: a_NP with
//    P the neighbour of face -code-2; -1: diagonal; FVGB_PAD: padding (value 0,
//    column = row).  diag_pos / own_pos / nei_pos give the slot of a_PP, a_PN
//    (row owner) and a_NP (row neighbour).
#pragma once
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <string>
#include <vector>

#include "fvgb.h"
#include "fvgb_host_common.h"

#define FVGB_PAD INT32_MIN
#define FVGB_MAX_PATCHES 256
#define FVGB_MAX_TERMS 8

constexpr int kSlice = 32;

struct MeshView {
    int32_t n, nif, nbf, npatch;
    const double* V;
    const double* invV;
    const int32_t* own;
    const int32_t* nei;
    const double* Sf;
    const double* magSf;
    const double* w;
    const double* delta;
    const double* geo;       // |Sf| * delta
    const double* corr;      // [nif*3] non-orthogonal correction vectors (null: mesh without cell centres)
    const int32_t* bcells;
    const double* bSf;
    const double* bmagSf;
    const double* bdelta;
    const double* bgeo;      // |Sf_b| * delta_b
    const int32_t* bpatch;   // patch index of every boundary face
    const int32_t* g_ptr;
    const int32_t* g_code;
    const int32_t* g_other;
    const int32_t* m_ptr;
    const int32_t* m_col;
    const int16_t* m_off;    // [m_len] column - row of every slot when all fit in 16 bits (banded
                             // meshes), else null: the SpMVs then read 2 instead of 4 bytes per slot
    const int32_t* m_code;
    const int32_t* diag_pos;
    const int32_t* own_pos;
    const int32_t* nei_pos;
    // 1.0, -1.0, -0.0 and +0.0 as run-time values: the exact FP64 additions and
    // products of the bit-exact kernels are issued as fused multiply-adds with
    // one of them (fadd/fsub/fmul below), which the compiler cannot fold back
    double k_one = 1.0, k_mone = -1.0, k_nzero = -0.0, k_zero = 0.0;
};

// Exact FP64 arithmetic issued as DFMA.  GB300 retires DFMA at ~1.9 lanes per
// clock per SM but DADD and DMUL at ~1.6 (measured: 596 vs 502 G operations/s
// on independent chains), and the bit-exact face loops are bound by that rate.
// fma(a, 1, b) rounds the exact sum a + b once, fma(b, -1, a) the exact
// difference a - b once, fma(a, b, -0) the exact product a * b once: the bits of
// a + b, a - b and a * b, signed zeros included (x + -0 = x, -0 + -0 = -0),
// and infinities and overflow alike.
__device__ __forceinline__ double fadd(const MeshView& m, double a, double b) { return __fma_rn(a, m.k_one, b); }
__device__ __forceinline__ double fsub(const MeshView& m, double a, double b) { return __fma_rn(b, m.k_mone, a); }
__device__ __forceinline__ double fmul(const MeshView& m, double a, double b) { return __fma_rn(a, b, m.k_nzero); }
// s + x (plus) or s - x: the owner/neighbour accumulation of a face term
__device__ __forceinline__ double facc(const MeshView& m, double s, bool plus, double x) {
    return __fma_rn(x, plus ? m.k_one : m.k_mone, s);
}
// The first accumulation of a sum from +0, +0 + x (plus) or +0 - x, on the
// integer pipes: the IEEE result is x or -x exactly, except that a zero result
// is +0 (a sum of opposite zeros rounds to +0 to nearest).  One FP64
// instruction fewer per sum.
__device__ __forceinline__ double facc0(bool plus, double x) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    if (!plus) u ^= 0x8000000000000000ull;
    return __longlong_as_double((u << 1) == 0 ? 0ll : (long long)u);
}

// ---- device memory of served requests
// Objects (meshes, linear systems, solver workspaces) created while the calling
// thread has a memory pool set take all their device memory from that pool
// (cudaMallocFromPoolAsync ordered on the context's allocation stream, waited
// for at once) and release it with cudaFreeAsync on the context's release
// stream, so releasing them never synchronises the device as cudaFree does.
// The serving loop sets the context on its thread; everything else uses
// cudaMalloc and cudaFree.  An object keeps the mode it was created in.
struct DevMemCtx {
    cudaMemPool_t pool = nullptr;
    cudaStream_t alloc = nullptr;    // private stream of the allocations
    cudaStream_t release = nullptr;  // stream whose work last used what is released
};
inline DevMemCtx& devmem_ctx() {
    static thread_local DevMemCtx c;
    return c;
}
inline bool devmem_pooled_now() { return devmem_ctx().pool != nullptr; }
inline cudaError_t devmem_alloc(void** p, size_t bytes, bool pooled) {
    if (!pooled) return cudaMalloc(p, bytes);
    const DevMemCtx& c = devmem_ctx();
    if (!c.pool) return cudaErrorInvalidValue;  // a pooled object grows only on the thread that owns the pool
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, c.pool, c.alloc);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.alloc);
    return e;
}
inline void devmem_free(void* p, bool pooled) {
    if (!p) return;
    if (pooled) cudaFreeAsync(p, devmem_ctx().release);
    else cudaFree(p);
}

struct fvgb_mesh {
    MeshView v{};
    int32_t nnz = 0;
    int32_t nslices = 0;
    int64_t m_len = 0, g_len = 0;
    int32_t* csr_pos = nullptr;  // [nnz] slot of CSR entry j
    std::vector<int32_t> h_patch_offs;
    std::vector<int32_t> h_row_offs, h_col, h_diag_off, h_own_off, h_nei_off;
    std::vector<void*> allocs;
    int64_t bytes = 0;
    bool pooled = false;  // device memory from the serving pool (devmem_*)
    int32_t face_tile = 4;  // faces per thread of the explicit face passes (2, 4, 8; same bits)
};

struct SolverCache;  // solver.cu
struct AmgCache;     // amg.cu
struct IluCache;     // ilu.cu

struct fvgb_ls {
    const fvgb_mesh* mesh = nullptr;
    int32_t ncomp = 1;
    double* values = nullptr;  // [m_len]
    double* rhs = nullptr;     // [n*ncomp]
    double* bmat = nullptr;    // [nbf]
    double* brhs = nullptr;    // [nbf*ncomp]
    SolverCache* solver = nullptr;
    AmgCache* amg = nullptr;   // multigrid hierarchy (amg.cu), built at the first multigrid solve
    IluCache* ilu = nullptr;   // ILU(0) pattern data and graphs (ilu.cu), built at the first ILU solve
    uint64_t version = 1;      // bumped whenever `values` change (assembly, SetReference)
    bool pooled = false;       // device memory from the serving pool (devmem_*)
};

// amg.cu: multigrid-preconditioned CG (cfg->preconditioner == FVGB_PRECOND_MULTIGRID)
void fvgb_amg_free(AmgCache* c);
fvgb_status fvgb_amg_solve_async(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats_dev,
                                 cudaStream_t s);
fvgb_status fvgb_amg_sync_stats(fvgb_ls* ls, fvgb_solver_stats* out, cudaStream_t s);

// ilu.cu: ILU(0)-preconditioned CG / BiCGStab (cfg->preconditioner == FVGB_PRECOND_ILU)
void fvgb_ilu_free(IluCache* c);
fvgb_status fvgb_ilu_solve_async(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats_dev,
                                 cudaStream_t s);
fvgb_status fvgb_ilu_sync_stats(fvgb_ls* ls, fvgb_solver_stats* out, cudaStream_t s);

// Per-call patch table passed to kernels by value.
struct PatchTable {
    int32_t n;
    int8_t type[FVGB_MAX_PATCHES];
};

inline fvgb_status cuda_fail(cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fvgb_fail(e == cudaErrorMemoryAllocation ? FVGB_ERR_OOM : FVGB_ERR_CUDA, m.c_str());
}

#define FVGB_CUDA_TRY(call)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

#define FVGB_LAUNCH_CHECK(where)                              \
    do {                                                      \
        cudaError_t e_ = cudaGetLastError();                  \
        if (e_ != cudaSuccess) return cuda_fail(e_, where);   \
    } while (0)

// Creation paths upload with cudaMemcpy and clear with cudaMemset: both run on
// the legacy default stream, which is not ordered with a caller's non-blocking
// streams, and both may return before the data is in place (pageable uploads
// return once staged; memsets are asynchronous).  They end with this wait on
// the legacy stream only, so kernels the caller then launches on any stream
// see the data.
inline cudaError_t settle_creation() { return cudaStreamSynchronize(0); }

// at least one block: every kernel bounds-checks its index, and a zero-block
// launch is a configuration error (empty boundary or face sets are legal)
// out_c += coeff * sum over the cell's faces (ascending, +- as owner/neighbour)
// of (gamma_f*|Sf|)*(k_f . gT_f): the explicit part of a corrected laplacian of
// psi, volume integrated (explicit_ops.cu).
fvgb_status nonorth_rhs(const fvgb_mesh* m, int nc, const double* gamma, const double* psi, const double* psi_b,
                        double coeff, double* out, cudaStream_t s);

// Column of matrix slot `pos` of row i (sliced ELL): from the 16-bit offset when
// the mesh has them, else from the 32-bit column array.  Same column either way.
__device__ __forceinline__ int slot_col(const MeshView& m, int pos, int i) {
    return m.m_off ? i + (int)__ldg(&m.m_off[pos]) : __ldg(&m.m_col[pos]);
}

inline unsigned grid_for(int64_t n, int threads) { return n > 0 ? (unsigned)((n + threads - 1) / threads) : 1u; }

// Builds a PatchTable from a host array of per-patch types; false if invalid.
inline bool make_patch_table(const fvgb_mesh* m, const int32_t* types, PatchTable* t) {
    t->n = m->v.npatch;
    if (t->n > FVGB_MAX_PATCHES) return false;
    for (int i = 0; i < t->n; ++i) {
        int32_t ty = types ? types[i] : FVGB_BC_CALCULATED;
        if (ty < FVGB_BC_CALCULATED || ty > FVGB_BC_FIXED_GRADIENT) return false;
        t->type[i] = (int8_t)ty;
    }
    return true;
}

inline bool patch_table_needs_ref(const PatchTable& t) {
    for (int i = 0; i < t.n; ++i)
        if (t.type[i] != FVGB_BC_CALCULATED) return true;
    return false;
}

// Device-side allocation helper that records the allocation on the mesh.
template <class T>
inline cudaError_t mesh_alloc(fvgb_mesh* m, T** p, int64_t count) {
    size_t bytes = sizeof(T) * (size_t)(count > 0 ? count : 1);
    cudaError_t e = devmem_alloc((void**)p, bytes, m->pooled);
    if (e == cudaSuccess) {
        m->allocs.push_back(*p);
        m->bytes += (int64_t)bytes;
    }
    return e;
}

#define FVGB_CHECK_ARG(cond, msg) \
    do {                          \
        if (!(cond)) return fvgb_fail(FVGB_ERR_INVALID_ARG, msg); \
    } while (0)
