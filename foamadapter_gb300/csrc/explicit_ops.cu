// Explicit finite-volume operators: surface interpolation (linear, upwind),
// Gauss-Green div / grad / laplacian, uncorrected snGrad and the fused
// upwind-advection forward-Euler step.
//
// The reference's Serial executor scatters face contributions into owner (+)
// and neighbour (-) cells in ascending face order.  Here one thread owns one
// cell and walks that cell's faces in the same ascending order through the
// gather list, so every cell sees the same sequence of IEEE operations and the
// result is bit-identical to the Serial face loop, with no atomics.  This file
// is compiled with -fmad=false so no multiply-add is contracted.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <string>

#include "internal.cuh"
#include "tunecache.h"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int gwidth(const MeshView& m, int slice) {
    return (__ldg(&m.g_ptr[slice + 1]) - __ldg(&m.g_ptr[slice])) >> 5;
}

// F >= 0.0 with IEEE semantics (true for +0 and -0 and +inf, false for NaN),
// decided on the bit pattern so it costs no FP64 instruction: GB300's FP64
// issue rate bounds every FP64 face loop here.
__device__ __forceinline__ bool nonneg(double F) {
    const long long u = __double_as_longlong(F);
    return u >= 0 ? u <= 0x7ff0000000000000LL : u == (long long)0x8000000000000000ULL;
}

// The owner/neighbour accumulation s + x or s - x is ONE fused multiply-add,
// fma(x, +-1, s) (facc): exactly the rounded sum or difference, with no branch
// and no separate negation.  Every other exact sum and product is a DFMA too
// (fadd, fsub, fmul): GB300 retires DFMA faster than DADD and DMUL.

// ---------------------------------------------------------------- interpolation
// Face kernels: a thread handles FPT faces spaced a block apart (coalesced
// across the block) and issues the loads of all of them before the dependent
// cell gathers, so each thread keeps several faces' bytes in flight.  FPT (the
// face-pass tile: 2, 4 or 8) is the mesh's `face_tile`, 4 unless
// fvgb_explicit_tune measured another; every face is computed alone, so every
// tile gives the same bits.
#define FVGB_FACE_TILE(tile, ...)          \
    switch (tile) {                         \
        case 2: {                           \
            constexpr int FPT = 2;          \
            __VA_ARGS__;                    \
        } break;                            \
        case 8: {                           \
            constexpr int FPT = 8;          \
            __VA_ARGS__;                    \
        } break;                            \
        default: {                          \
            constexpr int FPT = 4;          \
            __VA_ARGS__;                    \
        } break;                            \
    }

template <int FPT>
__device__ __forceinline__ int face_of(int k) { return (blockIdx.x * FPT + k) * blockDim.x + threadIdx.x; }

template <int NC, int FPT>
__global__ void __launch_bounds__(kThreads)
    k_interp_linear(MeshView m, const double* __restrict__ src, const double* __restrict__ src_b,
                    double* __restrict__ dst) {
    int P[FPT], N[FPT];
    double w[FPT];
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        P[k] = N[k] = 0;
        w[k] = 0.0;
        if (f < m.nif) {
            P[k] = __ldg(&m.own[f]);
            N[k] = __ldg(&m.nei[f]);
            w[k] = __ldg(&m.w[f]);
        }
    }
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const double sN = __ldg(&src[N[k] * NC + c]);
                dst[f * NC + c] = fadd(m, fmul(m, w[k], fsub(m, __ldg(&src[P[k] * NC + c]), sN)), sN);
            }
        } else if (f < m.nif + m.nbf) {
            const int b = f - m.nif;
#pragma unroll
            for (int c = 0; c < NC; ++c) dst[f * NC + c] = __ldg(&src_b[b * NC + c]);
        }
    }
}

template <int NC, int FPT>
__global__ void __launch_bounds__(kThreads)
    k_interp_upwind(MeshView m, const double* __restrict__ flux, const double* __restrict__ src,
                    const double* __restrict__ src_b, double* __restrict__ dst) {
    int cidx[FPT];
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        cidx[k] = 0;
        if (f < m.nif) {
            const double F = __ldg(&flux[f]);
            const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
            cidx[k] = nonneg(F) ? P : N;
        }
    }
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
#pragma unroll
            for (int c = 0; c < NC; ++c) dst[f * NC + c] = __ldg(&src[cidx[k] * NC + c]);
        } else if (f < m.nif + m.nbf) {
            const int b = f - m.nif;
#pragma unroll
            for (int c = 0; c < NC; ++c) dst[f * NC + c] = __ldg(&src_b[b * NC + c]);
        }
    }
}

// ------------------------------------------------------------ gather entries
// A cell's first kG gather entries are fetched together: the entry codes and
// the cells (or boundary faces) across, then every face and cell value they
// point to, so a thread has all its loads in flight at once instead of one
// dependent pair per face.  The arithmetic then runs in ascending face order
// exactly as the one-entry-at-a-time loop did; entries beyond kG (cells with
// more than kG faces) take the per-entry path.
constexpr int kG = 8;

struct Entries {
    int base, width;
    int code[kG], other[kG];  // code FVGB_PAD beyond the cell's row
};

__device__ __forceinline__ void load_entries(const MeshView& m, int c, Entries& e) {
    const int slice = c >> 5;
    e.base = __ldg(&m.g_ptr[slice]) + (c & 31);
    e.width = gwidth(m, slice);
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        e.code[j] = FVGB_PAD;
        e.other[j] = 0;
        if (j < e.width) {
            e.code[j] = __ldg(&m.g_code[e.base + j * 32]);
            e.other[j] = __ldg(&m.g_other[e.base + j * 32]);
        }
    }
}

// face index of an entry (a boundary entry's code is its index in face fields)
__device__ __forceinline__ int entry_face(int code) { return code >= 0 ? code : -code - 1; }

// ------------------------------------------------------------------------ div
// face value seen from cell c across internal face f: owner-side formulas of
// the reference with (P, N) = (owner, neighbour).
template <int NC, int SCHEME>
__device__ __forceinline__ void div_entry(const MeshView& m, int code, double F, const double* To, double wf,
                                          const double* Tc, double* s) {
    if (code >= m.nif) {  // boundary face: value from the boundary field
#pragma unroll
        for (int k = 0; k < NC; ++k) s[k] = fadd(m, s[k], fmul(m, F, To[k]));
        return;
    }
    const bool isOwner = code >= 0;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        const double Town = isOwner ? Tc[k] : To[k];
        const double Tnei = isOwner ? To[k] : Tc[k];
        double tf;
        if (SCHEME == FVGB_SCHEME_UPWIND) tf = nonneg(F) ? Town : Tnei;
        else tf = fadd(m, fmul(m, wf, fsub(m, Town, Tnei)), Tnei);
        s[k] = facc(m, s[k], isOwner, fmul(m, F, tf));
    }
}

template <int NC, int SCHEME>
__device__ __forceinline__ void div_cell(const MeshView& m, int c, const double* __restrict__ flux,
                                         const double* __restrict__ phi,
                                         const double* __restrict__ phi_b, double* s) {
    Entries e;
    load_entries(m, c, e);
    double Tc[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        Tc[k] = __ldg(&phi[c * NC + k]);
        s[k] = 0.0;
    }
    double F[kG], W[kG], T[kG][NC];
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        const int cd = e.code[j];
        F[j] = 0.0;
        W[j] = 0.0;
#pragma unroll
        for (int k = 0; k < NC; ++k) T[j][k] = 0.0;
        if (cd == FVGB_PAD) continue;
        const bool bnd = cd >= m.nif;
        const int f = entry_face(cd);
        F[j] = __ldg(&flux[f]);
        const double* src = bnd ? phi_b : phi;
#pragma unroll
        for (int k = 0; k < NC; ++k) T[j][k] = __ldg(&src[e.other[j] * NC + k]);
        if (SCHEME == FVGB_SCHEME_LINEAR && !bnd) W[j] = __ldg(&m.w[f]);
    }
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        if (e.code[j] == FVGB_PAD) break;
        div_entry<NC, SCHEME>(m, e.code[j], F[j], T[j], W[j], Tc, s);
    }
    for (int j = kG; j < e.width; ++j) {
        const int cd = __ldg(&m.g_code[e.base + j * 32]);
        if (cd == FVGB_PAD) break;
        const int o = __ldg(&m.g_other[e.base + j * 32]);
        const int f = entry_face(cd);
        const double* src = cd >= m.nif ? phi_b : phi;
        double To[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) To[k] = __ldg(&src[o * NC + k]);
        const double wf = (SCHEME == FVGB_SCHEME_LINEAR && cd < m.nif) ? __ldg(&m.w[f]) : 0.0;
        div_entry<NC, SCHEME>(m, cd, __ldg(&flux[f]), To, wf, Tc, s);
    }
}

template <int NC, int SCHEME>
__global__ void __launch_bounds__(kThreads)
    k_div(MeshView m, const double* __restrict__ flux, const double* __restrict__ phi,
          const double* __restrict__ phi_b, double coeff, int unit, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    double s[NC];
    div_cell<NC, SCHEME>(m, c, flux, phi, phi_b, s);
    const double sc = unit ? __ldg(&m.invV[c]) : coeff / __ldg(&m.V[c]);
#pragma unroll
    for (int k = 0; k < NC; ++k) out[c * NC + k] = fadd(m, out[c * NC + k], fmul(m, s[k], sc));
}

// Fused forward-Euler upwind advection step + boundary correction.
__global__ void __launch_bounds__(kThreads)
    k_advect_euler(MeshView m, PatchTable pt, const double* __restrict__ flux,
                   const double* __restrict__ Told, const double* __restrict__ Told_b, double dt,
                   const double* __restrict__ ref, const double* __restrict__ gq, double* __restrict__ Tnew,
                   double* __restrict__ Tnew_b) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    double s[1];
    div_cell<1, FVGB_SCHEME_UPWIND>(m, c, flux, Told, Told_b, s);
    const double dv = facc0(true, fmul(m, s[0], __ldg(&m.invV[c])));  // +0 + s/V
    const double tn = fsub(m, __ldg(&Told[c]), fmul(m, dt, dv));
    Tnew[c] = tn;
    // boundary faces of this cell (they follow its internal faces in the list)
    const int slice = c >> 5, lane = c & 31;
    const int base = __ldg(&m.g_ptr[slice]);
    const int width = gwidth(m, slice);
    for (int j = width - 1; j >= 0; --j) {
        const int code = __ldg(&m.g_code[base + j * 32 + lane]);
        if (code == FVGB_PAD) continue;
        if (code < m.nif) break;
        const int b = code - m.nif;
        const int t = pt.type[__ldg(&m.bpatch[b])];
        double v = __ldg(&Told_b[b]);
        if (t == FVGB_BC_FIXED_VALUE) v = __ldg(&ref[b]);
        else if (t == FVGB_BC_FIXED_GRADIENT) v = tn + (gq ? __ldg(&gq[b]) : __ldg(&ref[b]) / __ldg(&m.bdelta[b]));
        Tnew_b[b] = v;
    }
}

// meshes up to this size advance with the one-pass step kernel (k_advect_euler,
// one launch per step and no face buffer); larger ones with the two-pass step
constexpr int kStepsMaxCells = 1 << 16;

// ----------------------------------------------------------------------- grad
__device__ __forceinline__ void grad_entry(const MeshView& m, int code, double To, double wf, const double* S,
                                           double Tc, double& g0, double& g1, double& g2) {
    if (code >= m.nif) {
        g0 = fadd(m, g0, fmul(m, S[0], To));
        g1 = fadd(m, g1, fmul(m, S[1], To));
        g2 = fadd(m, g2, fmul(m, S[2], To));
        return;
    }
    const bool isOwner = code >= 0;
    const double Town = isOwner ? Tc : To;
    const double Tnei = isOwner ? To : Tc;
    const double tf = fadd(m, fmul(m, wf, fsub(m, Town, Tnei)), Tnei);
    g0 = facc(m, g0, isOwner, fmul(m, S[0], tf));
    g1 = facc(m, g1, isOwner, fmul(m, S[1], tf));
    g2 = facc(m, g2, isOwner, fmul(m, S[2], tf));
}

__global__ void __launch_bounds__(kThreads)
    k_grad(MeshView m, const double* __restrict__ phi, const double* __restrict__ phi_b,
           double coeff, int unit, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    Entries e;
    load_entries(m, c, e);
    const double Tc = __ldg(&phi[c]);
    double T[kG], W[kG], S[kG][3];
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        const int cd = e.code[j];
        T[j] = W[j] = S[j][0] = S[j][1] = S[j][2] = 0.0;
        if (cd == FVGB_PAD) continue;
        const bool bnd = cd >= m.nif;
        const int f = entry_face(cd);
        const double* src = bnd ? phi_b : phi;
        T[j] = __ldg(&src[e.other[j]]);
        const double* sf = bnd ? m.bSf + 3 * (cd - m.nif) : m.Sf + 3 * f;
        S[j][0] = __ldg(&sf[0]);
        S[j][1] = __ldg(&sf[1]);
        S[j][2] = __ldg(&sf[2]);
        if (!bnd) W[j] = __ldg(&m.w[f]);
    }
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        if (e.code[j] == FVGB_PAD) break;
        grad_entry(m, e.code[j], T[j], W[j], S[j], Tc, g0, g1, g2);
    }
    for (int j = kG; j < e.width; ++j) {
        const int cd = __ldg(&m.g_code[e.base + j * 32]);
        if (cd == FVGB_PAD) break;
        const int o = __ldg(&m.g_other[e.base + j * 32]);
        const bool bnd = cd >= m.nif;
        const int f = entry_face(cd);
        const double* sf = bnd ? m.bSf + 3 * (cd - m.nif) : m.Sf + 3 * f;
        const double Sv[3] = {__ldg(&sf[0]), __ldg(&sf[1]), __ldg(&sf[2])};
        grad_entry(m, cd, __ldg(&(bnd ? phi_b : phi)[o]), bnd ? 0.0 : __ldg(&m.w[f]), Sv, Tc, g0, g1, g2);
    }
    const double sc = unit ? __ldg(&m.invV[c]) : coeff / __ldg(&m.V[c]);
    out[3 * c] = fadd(m, out[3 * c], fmul(m, g0, sc));
    out[3 * c + 1] = fadd(m, out[3 * c + 1], fmul(m, g1, sc));
    out[3 * c + 2] = fadd(m, out[3 * c + 2], fmul(m, g2, sc));
}

// ------------------------------------------------------------------ laplacian
// face flux g*(T_nei - T_own); the owner adds it, the neighbour subtracts it;
// a boundary face adds g_b*(T_b - T_c)
template <int NC>
__device__ __forceinline__ void lap_entry(const MeshView& m, int code, double g, const double* To, const double* Tc,
                                          double* s) {
    if (code >= m.nif) {
#pragma unroll
        for (int k = 0; k < NC; ++k) s[k] = fadd(m, s[k], fmul(m, g, fsub(m, To[k], Tc[k])));
        return;
    }
    const bool isOwner = code >= 0;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        // owner: s + g*(To - Tc); neighbour: s - g*(Tc - To), the reference's face flux
        const double a = isOwner ? To[k] : Tc[k], b = isOwner ? Tc[k] : To[k];
        s[k] = facc(m, s[k], isOwner, fmul(m, g, fsub(m, a, b)));
    }
}

template <int NC>
__global__ void __launch_bounds__(kThreads)
    k_lap(MeshView m, const double* __restrict__ gamma, const double* __restrict__ phi,
          const double* __restrict__ phi_b, double coeff, int unit, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    Entries e;
    load_entries(m, c, e);
    double Tc[NC], s[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        Tc[k] = __ldg(&phi[c * NC + k]);
        s[k] = 0.0;
    }
    double Gm[kG], Ge[kG], T[kG][NC];
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        const int cd = e.code[j];
        Gm[j] = Ge[j] = 0.0;
#pragma unroll
        for (int k = 0; k < NC; ++k) T[j][k] = 0.0;
        if (cd == FVGB_PAD) continue;
        const bool bnd = cd >= m.nif;
        const int f = entry_face(cd);
        Gm[j] = __ldg(&gamma[f]);
        Ge[j] = bnd ? __ldg(&m.bgeo[cd - m.nif]) : __ldg(&m.geo[f]);
        const double* src = bnd ? phi_b : phi;
#pragma unroll
        for (int k = 0; k < NC; ++k) T[j][k] = __ldg(&src[e.other[j] * NC + k]);
    }
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        if (e.code[j] == FVGB_PAD) break;
        lap_entry<NC>(m, e.code[j], fmul(m, Gm[j], Ge[j]), T[j], Tc, s);
    }
    for (int j = kG; j < e.width; ++j) {
        const int cd = __ldg(&m.g_code[e.base + j * 32]);
        if (cd == FVGB_PAD) break;
        const int o = __ldg(&m.g_other[e.base + j * 32]);
        const bool bnd = cd >= m.nif;
        const int f = entry_face(cd);
        const double g = fmul(m, __ldg(&gamma[f]), bnd ? __ldg(&m.bgeo[cd - m.nif]) : __ldg(&m.geo[f]));
        double To[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) To[k] = __ldg(&(bnd ? phi_b : phi)[o * NC + k]);
        lap_entry<NC>(m, cd, g, To, Tc, s);
    }
    const double sc = unit ? __ldg(&m.invV[c]) : coeff / __ldg(&m.V[c]);
#pragma unroll
    for (int k = 0; k < NC; ++k) out[c * NC + k] = fadd(m, out[c * NC + k], fmul(m, s[k], sc));
}

// --------------------------------------------------------------------- snGrad
template <int FPT>
__global__ void __launch_bounds__(kThreads)
    k_sngrad(MeshView m, const double* __restrict__ phi, const double* __restrict__ phi_b, double* __restrict__ out) {
    int P[FPT], N[FPT];
    double d[FPT];
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        P[k] = N[k] = 0;
        d[k] = 0.0;
        if (f < m.nif) {
            P[k] = __ldg(&m.own[f]);
            N[k] = __ldg(&m.nei[f]);
            d[k] = __ldg(&m.delta[f]);
        } else if (f < m.nif + m.nbf) {
            const int b = f - m.nif;
            P[k] = __ldg(&m.bcells[b]);
            d[k] = __ldg(&m.bdelta[b]);
        }
    }
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) out[f] = fmul(m, d[k], fsub(m, __ldg(&phi[N[k]]), __ldg(&phi[P[k]])));
        else if (f < m.nif + m.nbf) out[f] = fmul(m, d[k], fsub(m, __ldg(&phi_b[f - m.nif]), __ldg(&phi[P[k]])));
    }
}

// ------------------------------------------------------ face-flux two passes
// Linear div, grad and laplacian: a face pass evaluates each face's flux ONCE
// (face value, then the product), as the reference's face loop does, into a
// face buffer; a cell pass then adds it (owner and boundary faces) or
// subtracts it (neighbour faces) in ascending face order.  The operations are
// those of the one-pass gather above, which evaluated every face from both of
// its cells: same bits, about half the FP64 work per face.  fx holds NC values
// per face, boundary faces after the internal ones (index nif + b = entry code).
template <int NC, int FPT>
__global__ void __launch_bounds__(kThreads)
    k_fx_div_linear(MeshView m, const double* __restrict__ flux, const double* __restrict__ phi,
                    const double* __restrict__ phi_b, double* __restrict__ fx) {
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
            const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
            const double F = __ldg(&flux[f]), wf = __ldg(&m.w[f]);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const double Tn = __ldg(&phi[N * NC + c]);
                fx[f * NC + c] = fmul(m, F, fadd(m, fmul(m, wf, fsub(m, __ldg(&phi[P * NC + c]), Tn)), Tn));
            }
        } else if (f < m.nif + m.nbf) {
            const double F = __ldg(&flux[f]);
#pragma unroll
            for (int c = 0; c < NC; ++c) fx[f * NC + c] = fmul(m, F, __ldg(&phi_b[(f - m.nif) * NC + c]));
        }
    }
}

template <int NC, int FPT>
__global__ void __launch_bounds__(kThreads)
    k_fx_div_upwind(MeshView m, const double* __restrict__ flux, const double* __restrict__ phi,
                    const double* __restrict__ phi_b, double* __restrict__ fx) {
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
            const double F = __ldg(&flux[f]);
            const int cu = nonneg(F) ? __ldg(&m.own[f]) : __ldg(&m.nei[f]);
#pragma unroll
            for (int c = 0; c < NC; ++c) fx[f * NC + c] = fmul(m, F, __ldg(&phi[cu * NC + c]));
        } else if (f < m.nif + m.nbf) {
            const double F = __ldg(&flux[f]);
#pragma unroll
            for (int c = 0; c < NC; ++c) fx[f * NC + c] = fmul(m, F, __ldg(&phi_b[(f - m.nif) * NC + c]));
        }
    }
}

template <int FPT>
__global__ void __launch_bounds__(kThreads)
    k_fx_grad(MeshView m, const double* __restrict__ phi, const double* __restrict__ phi_b, double* __restrict__ fx) {
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
            const double Tn = __ldg(&phi[__ldg(&m.nei[f])]);
            const double tf = fadd(m, fmul(m, __ldg(&m.w[f]), fsub(m, __ldg(&phi[__ldg(&m.own[f])]), Tn)), Tn);
            fx[3 * f] = fmul(m, __ldg(&m.Sf[3 * f]), tf);
            fx[3 * f + 1] = fmul(m, __ldg(&m.Sf[3 * f + 1]), tf);
            fx[3 * f + 2] = fmul(m, __ldg(&m.Sf[3 * f + 2]), tf);
        } else if (f < m.nif + m.nbf) {
            const int b = f - m.nif;
            const double tb = __ldg(&phi_b[b]);
            fx[3 * f] = fmul(m, __ldg(&m.bSf[3 * b]), tb);
            fx[3 * f + 1] = fmul(m, __ldg(&m.bSf[3 * b + 1]), tb);
            fx[3 * f + 2] = fmul(m, __ldg(&m.bSf[3 * b + 2]), tb);
        }
    }
}

template <int NC, int FPT>
__global__ void __launch_bounds__(kThreads)
    k_fx_lap(MeshView m, const double* __restrict__ gamma, const double* __restrict__ phi,
             const double* __restrict__ phi_b, double* __restrict__ fx) {
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
            const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
            const double g = fmul(m, __ldg(&gamma[f]), __ldg(&m.geo[f]));
#pragma unroll
            for (int c = 0; c < NC; ++c) fx[f * NC + c] = fmul(m, g, fsub(m, __ldg(&phi[N * NC + c]), __ldg(&phi[P * NC + c])));
        } else if (f < m.nif + m.nbf) {
            const int b = f - m.nif;
            const int P = __ldg(&m.bcells[b]);
            const double g = fmul(m, __ldg(&gamma[f]), __ldg(&m.bgeo[b]));
#pragma unroll
            for (int c = 0; c < NC; ++c) fx[f * NC + c] = fmul(m, g, fsub(m, __ldg(&phi_b[b * NC + c]), __ldg(&phi[P * NC + c])));
        }
    }
}

// ------------------------------------------- non-orthogonal correction
// OpenFOAM's correctedSnGrad: snGrad_f = delta_f (T_N - T_P) + k_f . (grad T)_f,
// k_f the mesh's correction vector, (grad T)_f the linear interpolation
// w (g_P - g_N) + g_N of the Gauss linear cell gradient; boundary faces of the
// (non-coupled) patches carry no correction.  The gradient of each of the NC
// components comes from k_fx_gradc + k_gather_fx<3*NC>: for NC = 1 the
// operations of fvgb_grad exactly.
template <int NC, int FPT>
__global__ void __launch_bounds__(kThreads)
    k_fx_gradc(MeshView m, const double* __restrict__ phi, const double* __restrict__ phi_b, double* __restrict__ fx) {
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
            const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
            const double wf = __ldg(&m.w[f]);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const double Tn = __ldg(&phi[N * NC + c]);
                const double tf = fadd(m, fmul(m, wf, fsub(m, __ldg(&phi[P * NC + c]), Tn)), Tn);
#pragma unroll
                for (int d = 0; d < 3; ++d) fx[(f * NC + c) * 3 + d] = fmul(m, __ldg(&m.Sf[3 * f + d]), tf);
            }
        } else if (f < m.nif + m.nbf) {
            const int b = f - m.nif;
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const double tb = __ldg(&phi_b[b * NC + c]);
#pragma unroll
                for (int d = 0; d < 3; ++d) fx[(f * NC + c) * 3 + d] = fmul(m, __ldg(&m.bSf[3 * b + d]), tb);
            }
        }
    }
}

enum CorrMode { kCorrLaplacian = 0, kCorrOnly = 1, kCorrSnGrad = 2 };

// kCorrLaplacian: fma(gamma_f|Sf|delta_f, T_N - T_P, gamma_f|Sf| (k . grad_f)),
//                 boundary faces gamma_b|Sf_b|delta_b (T_b - T_P) (as k_fx_lap);
// kCorrOnly:      gamma_f|Sf| (k . grad_f), boundary faces 0 (faceFluxCorrection);
// kCorrSnGrad:    fma(delta_f, T_N - T_P, k . grad_f), boundary delta_b (T_b - T_P).
// grad: [n][NC][3]; grad_f = fma(w, g_P - g_N, g_N) per direction and
// k . grad_f = fma(k_z, g_z, fma(k_y, g_y, k_x g_x)): fused multiply-adds, 14
// FP64 operations per face and component where separate roundings took 20 (the
// pass is bound by GB300's FP64 issue rate).  With k = 0 the flux is exactly the
// uncorrected one: fma(a, b, 0) rounds a*b once, as the plain product does.
template <int NC, int MODE, int FPT>
__global__ void __launch_bounds__(kThreads)
    k_fx_corr(MeshView m, const double* __restrict__ gamma, const double* __restrict__ phi,
              const double* __restrict__ phi_b, const double* __restrict__ grad, double* __restrict__ fx) {
#pragma unroll
    for (int k = 0; k < FPT; ++k) {
        const int f = face_of<FPT>(k);
        if (f < m.nif) {
            const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
            const double wf = __ldg(&m.w[f]);
            const double k0 = __ldg(&m.corr[3 * f]), k1 = __ldg(&m.corr[3 * f + 1]), k2 = __ldg(&m.corr[3 * f + 2]);
            const double gm = MODE == kCorrSnGrad ? 1.0 : fmul(m, __ldg(&gamma[f]), __ldg(&m.magSf[f]));
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                double gf[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const double gn = __ldg(&grad[(N * NC + c) * 3 + d]);
                    gf[d] = fma(wf, fsub(m, __ldg(&grad[(P * NC + c) * 3 + d]), gn), gn);
                }
                const double kg = fma(k2, gf[2], fma(k1, gf[1], fmul(m, k0, gf[0])));
                const double dT = fsub(m, __ldg(&phi[N * NC + c]), __ldg(&phi[P * NC + c]));
                if (MODE == kCorrLaplacian)
                    fx[f * NC + c] = fma(fmul(m, __ldg(&gamma[f]), __ldg(&m.geo[f])), dT, fmul(m, gm, kg));
                else if (MODE == kCorrOnly)
                    fx[f * NC + c] = fmul(m, gm, kg);
                else
                    fx[f * NC + c] = fma(__ldg(&m.delta[f]), dT, kg);
            }
        } else if (f < m.nif + m.nbf) {
            const int b = f - m.nif;
            const int P = __ldg(&m.bcells[b]);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const double dT = fsub(m, __ldg(&phi_b[b * NC + c]), __ldg(&phi[P * NC + c]));
                if (MODE == kCorrLaplacian) fx[f * NC + c] = fmul(m, fmul(m, __ldg(&gamma[f]), __ldg(&m.bgeo[b])), dT);
                else if (MODE == kCorrOnly) fx[f * NC + c] = 0.0;
                else fx[f * NC + c] = fmul(m, __ldg(&m.bdelta[b]), dT);
            }
        }
    }
}

// out_f += coeff * fx_f on the internal faces
__global__ void __launch_bounds__(kThreads)
    k_axpy_faces(int64_t count, double coeff, const double* __restrict__ fx, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = out[i] + coeff * __ldg(&fx[i]);
}

// out_c += (sum over the cell's faces, ascending, of +-fx_f) * scale, with
// scale = coeff/V_c (mode 0), 1/V_c (mode 1: coeff 1) or coeff (mode 2: volume integrated)
template <int NC>
__global__ void __launch_bounds__(kThreads)
    k_gather_fx(MeshView m, const double* __restrict__ fx, double coeff, int unit, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    Entries e;
    load_entries(m, c, e);
    double v[kG][NC];
#pragma unroll
    for (int j = 0; j < kG; ++j) {
#pragma unroll
        for (int k = 0; k < NC; ++k) v[j][k] = 0.0;
        if (e.code[j] == FVGB_PAD) continue;
        const int f = entry_face(e.code[j]);
#pragma unroll
        for (int k = 0; k < NC; ++k) v[j][k] = __ldg(&fx[f * NC + k]);
    }
    // owner and boundary faces add, neighbour faces subtract; the sum starts
    // from +0, so its first term is taken exactly on the integer pipes (a
    // padded first entry holds 0 and gives +0)
    double s[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) s[k] = facc0(e.code[0] >= 0, v[0][k]);
#pragma unroll
    for (int j = 1; j < kG; ++j) {
        if (e.code[j] == FVGB_PAD) break;
        const bool plus = e.code[j] >= 0;
#pragma unroll
        for (int k = 0; k < NC; ++k) s[k] = facc(m, s[k], plus, v[j][k]);
    }
    for (int j = kG; j < e.width; ++j) {
        const int cd = __ldg(&m.g_code[e.base + j * 32]);
        if (cd == FVGB_PAD) break;
        const int f = entry_face(cd);
#pragma unroll
        for (int k = 0; k < NC; ++k) s[k] = facc(m, s[k], cd >= 0, __ldg(&fx[f * NC + k]));
    }
    const double sc = unit == 1 ? __ldg(&m.invV[c]) : unit == 2 ? coeff : coeff / __ldg(&m.V[c]);
#pragma unroll
    for (int k = 0; k < NC; ++k) out[c * NC + k] = fadd(m, out[c * NC + k], fmul(m, s[k], sc));
}

// q_b = ref_b / delta_b of every fixed-gradient boundary face, whose boundary
// value is then T_P + q_b.  Formed here by whole warps over the boundary faces:
// in the gather only the one boundary lane of a cell warp needs it (a warp of
// cells along x meets one x wall), and the FP64 division's instruction sequence
// then ran at 1/32 lane use in half the warps, which kept the FP64 pipe busy.
__global__ void __launch_bounds__(kThreads)
    k_bc_gradq(MeshView m, PatchTable pt, const double* __restrict__ ref, double* __restrict__ q) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.nbf) return;
    q[b] = pt.type[__ldg(&m.bpatch[b])] == FVGB_BC_FIXED_GRADIENT ? __ldg(&ref[b]) / __ldg(&m.bdelta[b]) : 0.0;
}

// The fused upwind advection step on a face-flux buffer: the divergence as in
// k_gather_fx (coefficient 1), then the forward-Euler update and the boundary
// correction of k_advect_euler (the fixed-gradient quotients from k_bc_gradq).
__global__ void __launch_bounds__(kThreads, 6)
    k_advect_gather(MeshView m, PatchTable pt, const double* __restrict__ fx, const double* __restrict__ Told,
                    const double* __restrict__ Told_b, double dt, const double* __restrict__ ref,
                    const double* __restrict__ gq, double* __restrict__ Tnew, double* __restrict__ Tnew_b) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    Entries e;
    load_entries(m, c, e);
    double v[kG];
#pragma unroll
    for (int j = 0; j < kG; ++j) v[j] = e.code[j] == FVGB_PAD ? 0.0 : __ldg(&fx[entry_face(e.code[j])]);
    double s = facc0(e.code[0] >= 0, v[0]);  // the sum from +0: its first term exactly, on the integer pipes
#pragma unroll
    for (int j = 1; j < kG; ++j) {
        if (e.code[j] == FVGB_PAD) break;
        s = facc(m, s, e.code[j] >= 0, v[j]);
    }
    for (int j = kG; j < e.width; ++j) {
        const int cd = __ldg(&m.g_code[e.base + j * 32]);
        if (cd == FVGB_PAD) break;
        s = facc(m, s, cd >= 0, __ldg(&fx[entry_face(cd)]));
    }
    const double dv = facc0(true, fmul(m, s, __ldg(&m.invV[c])));  // +0 + s/V
    const double tn = fsub(m, __ldg(&Told[c]), fmul(m, dt, dv));
    Tnew[c] = tn;
    // boundary faces of this cell (its last entries): the entries held in
    // registers are tested in an unrolled loop, any beyond them reloaded
#pragma unroll
    for (int j = 0; j < kG; ++j) {
        const int code = e.code[j];
        if (code == FVGB_PAD || code < m.nif) continue;
        const int b = code - m.nif;
        const int t = pt.type[__ldg(&m.bpatch[b])];
        double bv = __ldg(&Told_b[b]);
        if (t == FVGB_BC_FIXED_VALUE) bv = __ldg(&ref[b]);
        else if (t == FVGB_BC_FIXED_GRADIENT) bv = tn + __ldg(&gq[b]);
        Tnew_b[b] = bv;
    }
    for (int j = kG; j < e.width; ++j) {
        const int code = __ldg(&m.g_code[e.base + j * 32]);
        if (code == FVGB_PAD || code < m.nif) continue;
        const int b = code - m.nif;
        const int t = pt.type[__ldg(&m.bpatch[b])];
        double bv = __ldg(&Told_b[b]);
        if (t == FVGB_BC_FIXED_VALUE) bv = __ldg(&ref[b]);
        else if (t == FVGB_BC_FIXED_GRADIENT) bv = tn + __ldg(&gq[b]);
        Tnew_b[b] = bv;
    }
}

// Face buffer from the stream-ordered pool (no device synchronisation); the
// pool keeps its memory between calls.  nullptr when it cannot be had: the
// caller then runs the one-pass gather, which needs none.
double* face_buffer(size_t count, cudaStream_t s) {
    static std::atomic<bool> pool_ready{false};  // the setting is idempotent: a racing second setter is harmless
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (!pool_ready.load(std::memory_order_acquire) && cudaStreamIsCapturing(s, &cap) == cudaSuccess &&
        cap == cudaStreamCaptureStatusNone) {
        // not while a graph is being captured (there the allocation becomes a graph memory node)
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool_ready.store(true, std::memory_order_release);
    }
    double* p = nullptr;
    if (cudaMallocAsync((void**)&p, sizeof(double) * (count ? count : 1), s) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

// The Gauss linear gradient of every component of psi into grad [n*nc*3]
// (zeroed first), on a face buffer.
fvgb_status gauss_grad_components(const fvgb_mesh* m, int nc, const double* psi, const double* psi_b, double* grad,
                                  cudaStream_t s) {
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    double* fx = face_buffer((size_t)(nf * nc * 3), s);
    if (!fx) return fvgb_fail(FVGB_ERR_OOM, "non-orthogonal correction: no face buffer");
    cudaMemsetAsync(grad, 0, sizeof(double) * (size_t)m->v.n * nc * 3, s);
    const unsigned g = grid_for(m->v.n, kThreads);
    if (nc == 1) {
        FVGB_FACE_TILE(m->face_tile, k_fx_gradc<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(m->v, psi, psi_b, fx))
        k_gather_fx<3><<<g, kThreads, 0, s>>>(m->v, fx, 1.0, 1, grad);
    } else {
        FVGB_FACE_TILE(m->face_tile, k_fx_gradc<3, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(m->v, psi, psi_b, fx))
        k_gather_fx<9><<<g, kThreads, 0, s>>>(m->v, fx, 1.0, 1, grad);
    }
    cudaFreeAsync(fx, s);
    return FVGB_OK;
}

// One corrected face pass (MODE) of psi into a face buffer fx [nf*nc]; the
// caller frees fx.  nullptr with the error set when buffers cannot be had.
template <int MODE>
double* corrected_faces(const fvgb_mesh* m, int nc, const double* gamma, const double* psi, const double* psi_b,
                        cudaStream_t s) {
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    double* grad = face_buffer((size_t)m->v.n * nc * 3, s);
    if (!grad) {
        fvgb_fail(FVGB_ERR_OOM, "non-orthogonal correction: no gradient buffer");
        return nullptr;
    }
    if (gauss_grad_components(m, nc, psi, psi_b, grad, s) != FVGB_OK) {
        cudaFreeAsync(grad, s);
        return nullptr;
    }
    double* fx = face_buffer((size_t)(nf * nc), s);
    if (fx) {
        if (nc == 1)
            FVGB_FACE_TILE(m->face_tile, k_fx_corr<1, MODE, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                             m->v, gamma, psi, psi_b, grad, fx))
        else
            FVGB_FACE_TILE(m->face_tile, k_fx_corr<3, MODE, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                             m->v, gamma, psi, psi_b, grad, fx))
    } else {
        fvgb_fail(FVGB_ERR_OOM, "non-orthogonal correction: no face buffer");
    }
    cudaFreeAsync(grad, s);
    return fx;
}

}  // namespace

fvgb_status nonorth_rhs(const fvgb_mesh* m, int nc, const double* gamma, const double* psi, const double* psi_b,
                        double coeff, double* out, cudaStream_t s) {
    double* fx = corrected_faces<kCorrOnly>(m, nc, gamma, psi, psi_b, s);
    if (!fx) return FVGB_ERR_OOM;
    const unsigned g = grid_for(m->v.n, kThreads);
    if (nc == 1) k_gather_fx<1><<<g, kThreads, 0, s>>>(m->v, fx, coeff, 2, out);
    else k_gather_fx<3><<<g, kThreads, 0, s>>>(m->v, fx, coeff, 2, out);
    cudaFreeAsync(fx, s);
    FVGB_LAUNCH_CHECK("non-orthogonal correction");
    return FVGB_OK;
}

// ==================================================================== C ABI
#define CHECK_MESH_NC(m, nc, name)                                                         \
    FVGB_CHECK_ARG(m, name ": null mesh");                                                 \
    FVGB_CHECK_ARG((nc) == 1 || (nc) == 3, name ": ncomp must be 1 or 3")

extern "C" fvgb_status fvgb_interp_linear(const fvgb_mesh* m, int32_t nc, const double* src,
                                          const double* src_b, double* dst, fvgb_stream stream) {
    CHECK_MESH_NC(m, nc, "fvgb_interp_linear");
    FVGB_CHECK_ARG(src && dst && (src_b || m->v.nbf == 0), "fvgb_interp_linear: null field");
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    if (nf == 0) return FVGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (nc == 1)
        FVGB_FACE_TILE(m->face_tile, k_interp_linear<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                         m->v, src, src_b, dst))
    else
        FVGB_FACE_TILE(m->face_tile, k_interp_linear<3, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                         m->v, src, src_b, dst))
    FVGB_LAUNCH_CHECK("fvgb_interp_linear");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_interp_upwind(const fvgb_mesh* m, int32_t nc, const double* flux,
                                          const double* src, const double* src_b, double* dst,
                                          fvgb_stream stream) {
    CHECK_MESH_NC(m, nc, "fvgb_interp_upwind");
    FVGB_CHECK_ARG(flux && src && dst && (src_b || m->v.nbf == 0), "fvgb_interp_upwind: null field");
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    if (nf == 0) return FVGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (nc == 1)
        FVGB_FACE_TILE(m->face_tile, k_interp_upwind<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                         m->v, flux, src, src_b, dst))
    else
        FVGB_FACE_TILE(m->face_tile, k_interp_upwind<3, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                         m->v, flux, src, src_b, dst))
    FVGB_LAUNCH_CHECK("fvgb_interp_upwind");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_div_explicit(const fvgb_mesh* m, int32_t scheme, int32_t nc,
                                         const double* flux, const double* phi,
                                         const double* phi_b, double coeff, double* out,
                                         fvgb_stream stream) {
    CHECK_MESH_NC(m, nc, "fvgb_div_explicit");
    FVGB_CHECK_ARG(scheme == FVGB_SCHEME_LINEAR || scheme == FVGB_SCHEME_UPWIND,
                   "fvgb_div_explicit: unknown scheme");
    FVGB_CHECK_ARG(flux && phi && out && (phi_b || m->v.nbf == 0), "fvgb_div_explicit: null field");
    const int unit = coeff == 1.0;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned g = grid_for(m->v.n, kThreads);
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    double* fx = face_buffer((size_t)(nf * nc), s);
    if (fx) {
        const bool up = scheme == FVGB_SCHEME_UPWIND;
        if (nc == 1) {
            if (up)
                FVGB_FACE_TILE(m->face_tile, k_fx_div_upwind<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                                 m->v, flux, phi, phi_b, fx))
            else
                FVGB_FACE_TILE(m->face_tile, k_fx_div_linear<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                                 m->v, flux, phi, phi_b, fx))
            k_gather_fx<1><<<g, kThreads, 0, s>>>(m->v, fx, coeff, unit, out);
        } else {
            if (up)
                FVGB_FACE_TILE(m->face_tile, k_fx_div_upwind<3, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                                 m->v, flux, phi, phi_b, fx))
            else
                FVGB_FACE_TILE(m->face_tile, k_fx_div_linear<3, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                                 m->v, flux, phi, phi_b, fx))
            k_gather_fx<3><<<g, kThreads, 0, s>>>(m->v, fx, coeff, unit, out);
        }
        FVGB_LAUNCH_CHECK("fvgb_div_explicit");
        cudaFreeAsync(fx, s);
        return FVGB_OK;
    }
    if (nc == 1 && scheme == FVGB_SCHEME_UPWIND)
        k_div<1, FVGB_SCHEME_UPWIND><<<g, kThreads, 0, s>>>(m->v, flux, phi, phi_b, coeff, unit, out);
    else if (nc == 1)
        k_div<1, FVGB_SCHEME_LINEAR><<<g, kThreads, 0, s>>>(m->v, flux, phi, phi_b, coeff, unit, out);
    else if (scheme == FVGB_SCHEME_UPWIND)
        k_div<3, FVGB_SCHEME_UPWIND><<<g, kThreads, 0, s>>>(m->v, flux, phi, phi_b, coeff, unit, out);
    else
        k_div<3, FVGB_SCHEME_LINEAR><<<g, kThreads, 0, s>>>(m->v, flux, phi, phi_b, coeff, unit, out);
    FVGB_LAUNCH_CHECK("fvgb_div_explicit");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_grad(const fvgb_mesh* m, const double* phi, const double* phi_b,
                                 double coeff, double* out, fvgb_stream stream) {
    FVGB_CHECK_ARG(m, "fvgb_grad: null mesh");
    FVGB_CHECK_ARG(phi && out && (phi_b || m->v.nbf == 0), "fvgb_grad: null field");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    double* fx = face_buffer((size_t)(3 * nf), s);
    if (fx) {
        FVGB_FACE_TILE(m->face_tile, k_fx_grad<FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(m->v, phi, phi_b, fx))
        k_gather_fx<3><<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, fx, coeff, coeff == 1.0, out);
        FVGB_LAUNCH_CHECK("fvgb_grad");
        cudaFreeAsync(fx, s);
        return FVGB_OK;
    }
    k_grad<<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, phi, phi_b, coeff, coeff == 1.0, out);
    FVGB_LAUNCH_CHECK("fvgb_grad");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_laplacian_explicit(const fvgb_mesh* m, int32_t nc, const double* gamma,
                                               const double* phi, const double* phi_b,
                                               double coeff, double* out, fvgb_stream stream) {
    CHECK_MESH_NC(m, nc, "fvgb_laplacian_explicit");
    FVGB_CHECK_ARG(gamma && phi && out && (phi_b || m->v.nbf == 0),
                   "fvgb_laplacian_explicit: null field");
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned g = grid_for(m->v.n, kThreads);
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    double* fx = face_buffer((size_t)(nf * nc), s);
    if (fx) {

        if (nc == 1) {
            FVGB_FACE_TILE(m->face_tile, k_fx_lap<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                             m->v, gamma, phi, phi_b, fx))
            k_gather_fx<1><<<g, kThreads, 0, s>>>(m->v, fx, coeff, coeff == 1.0, out);
        } else {
            FVGB_FACE_TILE(m->face_tile, k_fx_lap<3, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                             m->v, gamma, phi, phi_b, fx))
            k_gather_fx<3><<<g, kThreads, 0, s>>>(m->v, fx, coeff, coeff == 1.0, out);
        }
        FVGB_LAUNCH_CHECK("fvgb_laplacian_explicit");
        cudaFreeAsync(fx, s);
        return FVGB_OK;
    }
    if (nc == 1) k_lap<1><<<g, kThreads, 0, s>>>(m->v, gamma, phi, phi_b, coeff, coeff == 1.0, out);
    else k_lap<3><<<g, kThreads, 0, s>>>(m->v, gamma, phi, phi_b, coeff, coeff == 1.0, out);
    FVGB_LAUNCH_CHECK("fvgb_laplacian_explicit");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_sngrad(const fvgb_mesh* m, const double* phi, const double* phi_b,
                                   double* out, fvgb_stream stream) {
    FVGB_CHECK_ARG(m, "fvgb_sngrad: null mesh");
    FVGB_CHECK_ARG(phi && out && (phi_b || m->v.nbf == 0), "fvgb_sngrad: null field");
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    if (nf == 0) return FVGB_OK;
    FVGB_FACE_TILE(m->face_tile, k_sngrad<FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, (cudaStream_t)stream>>>(
                                     m->v, phi, phi_b, out))
    FVGB_LAUNCH_CHECK("fvgb_sngrad");
    return FVGB_OK;
}

#define CHECK_CORRECTED(m, name) \
    FVGB_CHECK_ARG((m)->v.corr || (m)->v.nif == 0, name ": the mesh was created without cell centres")

extern "C" fvgb_status fvgb_laplacian_explicit_corrected(const fvgb_mesh* m, int32_t nc, const double* gamma,
                                                         const double* phi, const double* phi_b, double coeff,
                                                         double* out, fvgb_stream stream) {
    fvgb_clear_error();
    CHECK_MESH_NC(m, nc, "fvgb_laplacian_explicit_corrected");
    CHECK_CORRECTED(m, "fvgb_laplacian_explicit_corrected");
    FVGB_CHECK_ARG(gamma && phi && out && (phi_b || m->v.nbf == 0), "fvgb_laplacian_explicit_corrected: null field");
    cudaStream_t s = (cudaStream_t)stream;
    double* fx = corrected_faces<kCorrLaplacian>(m, nc, gamma, phi, phi_b, s);
    if (!fx) return FVGB_ERR_OOM;
    const unsigned g = grid_for(m->v.n, kThreads);
    if (nc == 1) k_gather_fx<1><<<g, kThreads, 0, s>>>(m->v, fx, coeff, coeff == 1.0, out);
    else k_gather_fx<3><<<g, kThreads, 0, s>>>(m->v, fx, coeff, coeff == 1.0, out);
    cudaFreeAsync(fx, s);
    FVGB_LAUNCH_CHECK("fvgb_laplacian_explicit_corrected");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_sngrad_corrected(const fvgb_mesh* m, const double* phi, const double* phi_b, double* out,
                                             fvgb_stream stream) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(m, "fvgb_sngrad_corrected: null mesh");
    CHECK_CORRECTED(m, "fvgb_sngrad_corrected");
    FVGB_CHECK_ARG(phi && out && (phi_b || m->v.nbf == 0), "fvgb_sngrad_corrected: null field");
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    if (nf == 0) return FVGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    double* fx = corrected_faces<kCorrSnGrad>(m, 1, nullptr, phi, phi_b, s);
    if (!fx) return FVGB_ERR_OOM;
    cudaMemcpyAsync(out, fx, sizeof(double) * (size_t)nf, cudaMemcpyDeviceToDevice, s);
    cudaFreeAsync(fx, s);
    FVGB_LAUNCH_CHECK("fvgb_sngrad_corrected");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_nonorth_flux(const fvgb_mesh* m, int32_t nc, const double* gamma, const double* phi,
                                         const double* phi_b, double coeff, double* out, fvgb_stream stream) {
    fvgb_clear_error();
    CHECK_MESH_NC(m, nc, "fvgb_nonorth_flux");
    CHECK_CORRECTED(m, "fvgb_nonorth_flux");
    FVGB_CHECK_ARG(gamma && phi && out && (phi_b || m->v.nbf == 0), "fvgb_nonorth_flux: null field");
    if (m->v.nif == 0) return FVGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    double* fx = corrected_faces<kCorrOnly>(m, nc, gamma, phi, phi_b, s);
    if (!fx) return FVGB_ERR_OOM;
    const int64_t cnt = (int64_t)m->v.nif * nc;
    k_axpy_faces<<<grid_for(cnt, kThreads), kThreads, 0, s>>>(cnt, coeff, fx, out);
    cudaFreeAsync(fx, s);
    FVGB_LAUNCH_CHECK("fvgb_nonorth_flux");
    return FVGB_OK;
}

// One forward-Euler upwind step: the face pass and the fused gather on a
// face buffer (with the boundary quotients gq, formed here when null), or the
// one-pass step kernel when no face buffer can be had.
static fvgb_status advect_two_pass(const fvgb_mesh* m, const PatchTable& pt, const double* flux, const double* T_old,
                            const double* T_old_b, double dt, const double* ref, const double* gq, double* T_new,
                            double* T_new_b, cudaStream_t s) {
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    double* fx = face_buffer((size_t)(nf + (gq ? 0 : m->v.nbf)), s);  // face fluxes, then the quotients
    if (fx) {
        if (!gq) {
            double* q = fx + nf;
            k_bc_gradq<<<grid_for(m->v.nbf, kThreads), kThreads, 0, s>>>(m->v, pt, ref, q);
            gq = q;
        }
        FVGB_FACE_TILE(m->face_tile, k_fx_div_upwind<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                         m->v, flux, T_old, T_old_b, fx))
        k_advect_gather<<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, pt, fx, T_old, T_old_b, dt, ref, gq,
                                                                          T_new, T_new_b);
        FVGB_LAUNCH_CHECK("fvgb_advect_euler_step");
        cudaFreeAsync(fx, s);
        return FVGB_OK;
    }
    k_advect_euler<<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, pt, flux, T_old, T_old_b, dt, ref, gq,
                                                                   T_new, T_new_b);
    FVGB_LAUNCH_CHECK("fvgb_advect_euler_step");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_advect_euler_steps(const fvgb_mesh* m, const double* flux, double* T, double* T_b,
                                               double dt, const fvgb_bc* bc, int32_t nsteps, double* work,
                                               double* work_b, fvgb_stream stream) {
    FVGB_CHECK_ARG(m && bc && nsteps >= 0, "fvgb_advect_euler_steps: bad argument");
    FVGB_CHECK_ARG(flux && T && work && ((T_b && work_b) || m->v.nbf == 0), "fvgb_advect_euler_steps: null field");
    FVGB_CHECK_ARG(T != work && (m->v.nbf == 0 || T_b != work_b), "fvgb_advect_euler_steps: work must not alias T");
    PatchTable pt;
    FVGB_CHECK_ARG(make_patch_table(m, bc->patch_type, &pt), "fvgb_advect_euler_steps: bad patch types");
    FVGB_CHECK_ARG(bc->ref || !patch_table_needs_ref(pt), "fvgb_advect_euler_steps: ref is null");
    if (nsteps == 0) return FVGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    // the fixed-gradient boundary quotients ref/delta do not change between
    // steps: formed once for the whole call
    double* gq = nullptr;
    if (m->v.nbf > 0 && cudaMallocAsync(&gq, sizeof(double) * (size_t)m->v.nbf, s) == cudaSuccess)
        k_bc_gradq<<<grid_for(m->v.nbf, kThreads), kThreads, 0, s>>>(m->v, pt, bc->ref, gq);
    else
        cudaGetLastError();  // without the buffer each step forms its quotients itself
    fvgb_status st = FVGB_OK;
    if (m->v.n <= kStepsMaxCells) {
        for (int k = 0; k < nsteps; ++k) {
            const bool even = (k & 1) == 0;
            k_advect_euler<<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(
                m->v, pt, flux, even ? T : work, even ? T_b : work_b, dt, bc->ref, gq, even ? work : T,
                even ? work_b : T_b);
        }
    } else {
        for (int k = 0; k < nsteps && st == FVGB_OK; ++k) {
            const bool even = (k & 1) == 0;
            st = advect_two_pass(m, pt, flux, even ? T : work, even ? T_b : work_b, dt, bc->ref, gq,
                                 even ? work : T, even ? work_b : T_b, s);
        }
    }
    if (gq) cudaFreeAsync(gq, s);
    if (st != FVGB_OK) return st;
    FVGB_LAUNCH_CHECK("fvgb_advect_euler_steps");
    if (nsteps & 1) {  // the last step wrote the work buffers
        FVGB_CUDA_TRY(cudaMemcpyAsync(T, work, sizeof(double) * (size_t)m->v.n, cudaMemcpyDeviceToDevice, s));
        if (m->v.nbf > 0)
            FVGB_CUDA_TRY(cudaMemcpyAsync(T_b, work_b, sizeof(double) * (size_t)m->v.nbf, cudaMemcpyDeviceToDevice, s));
    }
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_advect_euler_step(const fvgb_mesh* m, const double* flux,
                                              const double* T_old, const double* T_old_b,
                                              double dt, const fvgb_bc* bc, double* T_new,
                                              double* T_new_b, fvgb_stream stream) {
    FVGB_CHECK_ARG(m && bc, "fvgb_advect_euler_step: null argument");
    FVGB_CHECK_ARG(flux && T_old && T_new && ((T_old_b && T_new_b) || m->v.nbf == 0),
                   "fvgb_advect_euler_step: null field");
    FVGB_CHECK_ARG(T_new != T_old, "fvgb_advect_euler_step: T_new must not alias T_old");
    PatchTable pt;
    FVGB_CHECK_ARG(make_patch_table(m, bc->patch_type, &pt), "fvgb_advect_euler_step: bad patch types");
    FVGB_CHECK_ARG(bc->ref || !patch_table_needs_ref(pt), "fvgb_advect_euler_step: ref is null");
    cudaStream_t s = (cudaStream_t)stream;
    if (m->v.n <= kStepsMaxCells) {  // small meshes: one launch of the one-pass step kernel
        k_advect_euler<<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, pt, flux, T_old, T_old_b, dt, bc->ref,
                                                                       nullptr, T_new, T_new_b);
        FVGB_LAUNCH_CHECK("fvgb_advect_euler_step");
        return FVGB_OK;
    }
    return advect_two_pass(m, pt, flux, T_old, T_old_b, dt, bc->ref, nullptr, T_new, T_new_b, s);
}

// ------------------------------------------------------- face-pass tile
extern "C" fvgb_status fvgb_mesh_face_tile(fvgb_mesh* m, int32_t tile) {
    FVGB_CHECK_ARG(m, "fvgb_mesh_face_tile: null mesh");
    FVGB_CHECK_ARG(tile == 0 || tile == 2 || tile == 4 || tile == 8, "fvgb_mesh_face_tile: the tile is 2, 4 or 8");
    m->face_tile = tile == 0 ? 4 : tile;
    return FVGB_OK;
}

namespace {
// The tuning cache's key of a mesh shape for the face passes
std::string face_tune_key(const fvgb_mesh* m) {
    int dev = 0, sms = 0, cmaj = 0, cmin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&cmaj, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&cmin, cudaDevAttrComputeCapabilityMinor, dev);
    const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
    const int lg = nf > 0 ? (int)std::lround(std::log2((double)nf)) : 0;
    return "faces/sm" + std::to_string(cmaj * 10 + cmin) + "x" + std::to_string(sms) + "/faces2^" + std::to_string(lg);
}
constexpr int kTiles[3] = {2, 4, 8};
}  // namespace

// Times the face passes of grad and upwind div (the FP64-issue-bound and the
// memory-latency-bound kind) with each tile on scratch fields of this mesh and
// keeps the fastest; a tile cached for this mesh shape is taken untimed.
// Synchronises `stream`.
extern "C" fvgb_status fvgb_explicit_tune(fvgb_mesh* m, fvgb_stream stream, int32_t* tile_out, float* ms_out) {
    FVGB_CHECK_ARG(m, "fvgb_explicit_tune: null mesh");
    cudaStream_t s = (cudaStream_t)stream;
    const std::string key = face_tune_key(m);
    int cached = -1;
    float ms[4] = {0, 0, 0, 0};
    if (tune_cache_get(key, 0, &cached) && cached >= 0 && cached < 3) {
        m->face_tile = kTiles[cached];
    } else {
        const int64_t nf = (int64_t)m->v.nif + m->v.nbf;
        double *phi = nullptr, *phi_b = nullptr, *flux = nullptr, *fx = nullptr;
        cudaError_t e = cudaMallocAsync(&phi, sizeof(double) * (size_t)std::max<int64_t>(1, m->v.n), s);
        if (e == cudaSuccess) e = cudaMallocAsync(&phi_b, sizeof(double) * (size_t)std::max<int32_t>(1, m->v.nbf), s);
        if (e == cudaSuccess) e = cudaMallocAsync(&flux, sizeof(double) * (size_t)std::max<int64_t>(1, nf), s);
        if (e == cudaSuccess) e = cudaMallocAsync(&fx, sizeof(double) * 3 * (size_t)std::max<int64_t>(1, nf), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(phi, 0, sizeof(double) * (size_t)std::max<int64_t>(1, m->v.n), s);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(phi_b, 0, sizeof(double) * (size_t)std::max<int32_t>(1, m->v.nbf), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(flux, 0, sizeof(double) * (size_t)std::max<int64_t>(1, nf), s);
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (e == cudaSuccess) e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        int best = 1;
        for (int t = 0; t < 3 && e == cudaSuccess; ++t) {
            float times[3];
            for (int r = 0; r < 4 && e == cudaSuccess; ++r) {  // the first run warms up
                cudaEventRecord(e0, s);
                FVGB_FACE_TILE(kTiles[t],
                               k_fx_grad<FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(m->v, phi, phi_b, fx);
                               k_fx_div_upwind<1, FPT><<<grid_for(nf, kThreads * FPT), kThreads, 0, s>>>(
                                   m->v, flux, phi, phi_b, fx))
                cudaEventRecord(e1, s);
                e = cudaEventSynchronize(e1);
                if (e == cudaSuccess && r > 0) e = cudaEventElapsedTime(&times[r - 1], e0, e1);
            }
            std::sort(times, times + 3);
            ms[t] = times[1];
        }
        for (int t = 0; t < 3; ++t)
            if (ms[t] < ms[best]) best = t;
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFreeAsync(phi, s);
        cudaFreeAsync(phi_b, s);
        cudaFreeAsync(flux, s);
        cudaFreeAsync(fx, s);
        if (e != cudaSuccess) return cuda_fail(e, "fvgb_explicit_tune");
        m->face_tile = kTiles[best];
        tune_cache_put(key, 0, best, ms);
    }
    if (tile_out) *tile_out = m->face_tile;
    if (ms_out)
        for (int t = 0; t < 3; ++t) ms_out[t] = ms[t];
    return FVGB_OK;
}
