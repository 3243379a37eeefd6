// Pressure-velocity coupling helpers of FoamAdapter's PISO loop
// (src/algorithms/pressureVelocityCoupling.cpp).  The off-diagonal sweep of
// computeRAUandHByA, which the reference does with two atomic subtractions per
// face, is a per-cell gather here: each cell walks its faces in ascending face
// order, which reproduces the Serial executor's result exactly.
// Compiled with -fmad=false.
#include "internal.cuh"

namespace {

constexpr int kThreads = 256;

struct FlagTable {
    int32_t n;
    int8_t flag[FVGB_MAX_PATCHES];
};

// rAU = V / a_PP; HbyA = (b - sum a_Pj U_j) * (rAU / V)
__global__ void __launch_bounds__(kThreads)
    k_rau_hbya(MeshView m, const double* __restrict__ val, const double* __restrict__ rhs,
               const double* __restrict__ U, double* __restrict__ rAU, double* __restrict__ H) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    const double Vc = __ldg(&m.V[c]);
    const double ra = Vc / __ldg(&val[__ldg(&m.diag_pos[c])]);
    rAU[c] = ra;
    const int slice = c >> 5, lane = c & 31;
    const int base = __ldg(&m.g_ptr[slice]);
    const int width = (__ldg(&m.g_ptr[slice + 1]) - base) >> 5;
    double h0 = 0.0, h1 = 0.0, h2 = 0.0;
    for (int j = 0; j < width; ++j) {
        const int pos = base + j * 32 + lane;
        const int code = __ldg(&m.g_code[pos]);
        if (code == FVGB_PAD || code >= m.nif) break;  // boundary faces add nothing
        const int o = __ldg(&m.g_other[pos]);
        // owner side uses a_PN (upper), neighbour side a_NP (lower) of this row
        const double a = code >= 0 ? __ldg(&val[__ldg(&m.own_pos[code])])
                                   : __ldg(&val[__ldg(&m.nei_pos[-code - 1])]);
        h0 = h0 - a * __ldg(&U[3 * o]);
        h1 = h1 - a * __ldg(&U[3 * o + 1]);
        h2 = h2 - a * __ldg(&U[3 * o + 2]);
    }
    const double sc = ra / Vc;
    h0 = h0 + __ldg(&rhs[3 * c]);
    h1 = h1 + __ldg(&rhs[3 * c + 1]);
    h2 = h2 + __ldg(&rhs[3 * c + 2]);
    H[3 * c] = h0 * sc;
    H[3 * c + 1] = h1 * sc;
    H[3 * c + 2] = h2 * sc;
}

__global__ void k_constrain(MeshView m, FlagTable ft, const double* __restrict__ U_b,
                            double* __restrict__ H_b) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.nbf) return;
    if (ft.flag[__ldg(&m.bpatch[b])]) return;
    H_b[3 * b] = U_b[3 * b];
    H_b[3 * b + 1] = U_b[3 * b + 1];
    H_b[3 * b + 2] = U_b[3 * b + 2];
}

__global__ void k_flux_vec(MeshView m, const double* __restrict__ U, const double* __restrict__ U_b,
                           double* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < m.nif) {
        const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
        const double w = __ldg(&m.w[f]);
        double t[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double uN = __ldg(&U[3 * N + k]);
            t[k] = w * (__ldg(&U[3 * P + k]) - uN) + uN;
        }
        out[f] = __ldg(&m.Sf[3 * f]) * t[0] + __ldg(&m.Sf[3 * f + 1]) * t[1] +
                 __ldg(&m.Sf[3 * f + 2]) * t[2];
    } else if (f < m.nif + m.nbf) {
        const int b = f - m.nif;
        out[f] = __ldg(&m.bSf[3 * b]) * __ldg(&U_b[3 * b]) +
                 __ldg(&m.bSf[3 * b + 1]) * __ldg(&U_b[3 * b + 1]) +
                 __ldg(&m.bSf[3 * b + 2]) * __ldg(&U_b[3 * b + 2]);
    }
}

__global__ void k_face_update(MeshView m, const double* __restrict__ val,
                              const double* __restrict__ bmat, const double* __restrict__ brhs,
                              const double* __restrict__ phiHbyA, const double* __restrict__ p,
                              double* __restrict__ phi) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < m.nif) {
        const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
        const double upper = __ldg(&val[__ldg(&m.nei_pos[f])]);
        const double lower = __ldg(&val[__ldg(&m.own_pos[f])]);
        phi[f] = __ldg(&phiHbyA[f]) - (upper * __ldg(&p[N]) - lower * __ldg(&p[P]));
    } else if (f < m.nif + m.nbf) {
        const int b = f - m.nif;
        const double bflux = __ldg(&brhs[b]) - __ldg(&bmat[b]) * __ldg(&p[__ldg(&m.bcells[b])]);
        phi[f] = __ldg(&phiHbyA[f]) - bflux;
    }
}

// U = HbyA - rAU * grad(p), grad gathered per cell exactly as fvgb_grad (coeff 1)
__global__ void __launch_bounds__(kThreads)
    k_velocity_update(MeshView m, const double* __restrict__ H, const double* __restrict__ rAU,
                      const double* __restrict__ p, const double* __restrict__ p_b,
                      double* __restrict__ U) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    const int slice = c >> 5, lane = c & 31;
    const int base = __ldg(&m.g_ptr[slice]);
    const int width = (__ldg(&m.g_ptr[slice + 1]) - base) >> 5;
    const double Tc = __ldg(&p[c]);
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int j = 0; j < width; ++j) {
        const int pos = base + j * 32 + lane;
        const int code = __ldg(&m.g_code[pos]);
        if (code == FVGB_PAD) break;
        if (code >= m.nif) {
            const int b = code - m.nif;
            const double tb = __ldg(&p_b[b]);
            g0 = g0 + __ldg(&m.bSf[3 * b]) * tb;
            g1 = g1 + __ldg(&m.bSf[3 * b + 1]) * tb;
            g2 = g2 + __ldg(&m.bSf[3 * b + 2]) * tb;
            continue;
        }
        const bool isOwner = code >= 0;
        const int f = isOwner ? code : -code - 1;
        const double To = __ldg(&p[__ldg(&m.g_other[pos])]);
        const double Town = isOwner ? Tc : To;
        const double Tnei = isOwner ? To : Tc;
        const double tf = __ldg(&m.w[f]) * (Town - Tnei) + Tnei;
        const double v0 = __ldg(&m.Sf[3 * f]) * tf;
        const double v1 = __ldg(&m.Sf[3 * f + 1]) * tf;
        const double v2 = __ldg(&m.Sf[3 * f + 2]) * tf;
        if (isOwner) {
            g0 = g0 + v0;
            g1 = g1 + v1;
            g2 = g2 + v2;
        } else {
            g0 = g0 - v0;
            g1 = g1 - v1;
            g2 = g2 - v2;
        }
    }
    const double iv = __ldg(&m.invV[c]);
    const double ra = __ldg(&rAU[c]);
    const double gr0 = 0.0 + g0 * iv, gr1 = 0.0 + g1 * iv, gr2 = 0.0 + g2 * iv;
    U[3 * c] = __ldg(&H[3 * c]) - ra * gr0;
    U[3 * c + 1] = __ldg(&H[3 * c + 1]) - ra * gr1;
    U[3 * c + 2] = __ldg(&H[3 * c + 2]) - ra * gr2;
}

// fvc::interpolate(rAU)*fvc::ddtCorr(U, phi) with Euler ddt (OpenFOAM's
// EulerDdtScheme::fvcDdtPhiCorr and ddtCorrCoeff for ddtPhiCoeff < 0):
//   d = phi_old - Sf . U_old_f,  c = 1 - min(|d| / (|phi_old| + 1e-15), 1),
//   out += rAUf * ((c / dt) * d);  c = 0 on patches where U is a fixed value.
// Sf . U_old_f as k_flux_vec forms it.
__global__ void k_ddt_corr(MeshView m, PatchTable pt, const double* __restrict__ U, const double* __restrict__ U_b,
                           const double* __restrict__ phi_old, const double* __restrict__ rAUf, double rdt,
                           double* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double fU;
    if (f < m.nif) {
        const int P = __ldg(&m.own[f]), N = __ldg(&m.nei[f]);
        const double w = __ldg(&m.w[f]);
        double t[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double uN = __ldg(&U[3 * N + k]);
            t[k] = w * (__ldg(&U[3 * P + k]) - uN) + uN;
        }
        fU = __ldg(&m.Sf[3 * f]) * t[0] + __ldg(&m.Sf[3 * f + 1]) * t[1] + __ldg(&m.Sf[3 * f + 2]) * t[2];
    } else if (f < m.nif + m.nbf) {
        const int b = f - m.nif;
        if (pt.type[__ldg(&m.bpatch[b])] == FVGB_BC_FIXED_VALUE) return;
        fU = __ldg(&m.bSf[3 * b]) * __ldg(&U_b[3 * b]) + __ldg(&m.bSf[3 * b + 1]) * __ldg(&U_b[3 * b + 1]) +
             __ldg(&m.bSf[3 * b + 2]) * __ldg(&U_b[3 * b + 2]);
    } else {
        return;
    }
    const double po = __ldg(&phi_old[f]);
    const double d = po - fU;
    const double c = 1.0 - fmin(fabs(d) / (fabs(po) + 1e-15), 1.0);
    out[f] = out[f] + __ldg(&rAUf[f]) * ((c * rdt) * d);
}

// Foam::constrainPressure: on fixedFluxPressure patches the pressure's fixed
// gradient becomes (phiHbyA_b - Sf_b . U_b) / (|Sf_b| * rAUf_b).
__global__ void k_constrain_pressure(MeshView m, FlagTable ft, const double* __restrict__ phiHbyA,
                                     const double* __restrict__ U_b, const double* __restrict__ rAUf,
                                     double* __restrict__ p_ref) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.nbf) return;
    if (!ft.flag[__ldg(&m.bpatch[b])]) return;
    const double fU = __ldg(&m.bSf[3 * b]) * __ldg(&U_b[3 * b]) + __ldg(&m.bSf[3 * b + 1]) * __ldg(&U_b[3 * b + 1]) +
                      __ldg(&m.bSf[3 * b + 2]) * __ldg(&U_b[3 * b + 2]);
    const int f = m.nif + b;
    p_ref[b] = (__ldg(&phiHbyA[f]) - fU) / (__ldg(&m.bmagSf[b]) * __ldg(&rAUf[f]));
}

}  // namespace

extern "C" fvgb_status fvgb_piso_ddt_corr(const fvgb_mesh* mesh, const int32_t* U_patch_type, const double* U_old,
                                          const double* U_old_b, const double* phi_old, const double* rAUf, double dt,
                                          double* phiHbyA, fvgb_stream stream) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(mesh && U_patch_type && U_old && phi_old && rAUf && phiHbyA && (U_old_b || mesh->v.nbf == 0),
                   "fvgb_piso_ddt_corr: null argument");
    FVGB_CHECK_ARG(dt > 0, "fvgb_piso_ddt_corr: dt must be positive");
    PatchTable pt;
    FVGB_CHECK_ARG(make_patch_table(mesh, U_patch_type, &pt), "fvgb_piso_ddt_corr: bad patch types");
    const int64_t nf = (int64_t)mesh->v.nif + mesh->v.nbf;
    if (nf == 0) return FVGB_OK;
    k_ddt_corr<<<grid_for(nf, kThreads), kThreads, 0, (cudaStream_t)stream>>>(mesh->v, pt, U_old, U_old_b, phi_old,
                                                                              rAUf, 1.0 / dt, phiHbyA);
    FVGB_LAUNCH_CHECK("fvgb_piso_ddt_corr");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_piso_constrain_pressure(const fvgb_mesh* mesh, const int32_t* patch_fixed_flux,
                                                    const double* phiHbyA, const double* U_b, const double* rAUf,
                                                    double* p_ref, fvgb_stream stream) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(mesh && patch_fixed_flux, "fvgb_piso_constrain_pressure: null argument");
    if (mesh->v.nbf == 0) return FVGB_OK;
    FVGB_CHECK_ARG(phiHbyA && U_b && rAUf && p_ref, "fvgb_piso_constrain_pressure: null field");
    FlagTable ft;
    ft.n = mesh->v.npatch;
    for (int i = 0; i < ft.n; ++i) ft.flag[i] = patch_fixed_flux[i] ? 1 : 0;
    k_constrain_pressure<<<grid_for(mesh->v.nbf, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        mesh->v, ft, phiHbyA, U_b, rAUf, p_ref);
    FVGB_LAUNCH_CHECK("fvgb_piso_constrain_pressure");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_piso_rau_hbya(const fvgb_ls* ueqn, const double* U, double* rAU,
                                          double* HbyA, fvgb_stream stream) {
    FVGB_CHECK_ARG(ueqn && U && rAU && HbyA, "fvgb_piso_rau_hbya: null argument");
    FVGB_CHECK_ARG(ueqn->ncomp == 3, "fvgb_piso_rau_hbya: needs the vector (ncomp 3) momentum system");
    const MeshView& m = ueqn->mesh->v;
    k_rau_hbya<<<grid_for(m.n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(m, ueqn->values, ueqn->rhs,
                                                                              U, rAU, HbyA);
    FVGB_LAUNCH_CHECK("fvgb_piso_rau_hbya");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_piso_constrain_hbya(const fvgb_mesh* mesh, const int32_t* patch_assignable,
                                                const double* U_b, double* HbyA_b, fvgb_stream stream) {
    FVGB_CHECK_ARG(mesh && patch_assignable, "fvgb_piso_constrain_hbya: null argument");
    if (mesh->v.nbf == 0) return FVGB_OK;
    FVGB_CHECK_ARG(U_b && HbyA_b, "fvgb_piso_constrain_hbya: null field");
    FlagTable ft;
    ft.n = mesh->v.npatch;
    for (int i = 0; i < ft.n; ++i) ft.flag[i] = patch_assignable[i] ? 1 : 0;
    k_constrain<<<grid_for(mesh->v.nbf, kThreads), kThreads, 0, (cudaStream_t)stream>>>(mesh->v, ft, U_b, HbyA_b);
    FVGB_LAUNCH_CHECK("fvgb_piso_constrain_hbya");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_flux_vec(const fvgb_mesh* mesh, const double* U, const double* U_b,
                                     double* out, fvgb_stream stream) {
    FVGB_CHECK_ARG(mesh && U && out && (U_b || mesh->v.nbf == 0), "fvgb_flux_vec: null argument");
    const int64_t nf = (int64_t)mesh->v.nif + mesh->v.nbf;
    if (nf == 0) return FVGB_OK;
    k_flux_vec<<<grid_for(nf, kThreads), kThreads, 0, (cudaStream_t)stream>>>(mesh->v, U, U_b, out);
    FVGB_LAUNCH_CHECK("fvgb_flux_vec");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_piso_face_update(const fvgb_ls* peqn, const double* phiHbyA,
                                             const double* p, double* phi, fvgb_stream stream) {
    FVGB_CHECK_ARG(peqn && phiHbyA && p && phi, "fvgb_piso_face_update: null argument");
    FVGB_CHECK_ARG(peqn->ncomp == 1, "fvgb_piso_face_update: needs the scalar pressure system");
    const MeshView& m = peqn->mesh->v;
    const int64_t nf = (int64_t)m.nif + m.nbf;
    if (nf == 0) return FVGB_OK;
    k_face_update<<<grid_for(nf, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        m, peqn->values, peqn->bmat, peqn->brhs, phiHbyA, p, phi);
    FVGB_LAUNCH_CHECK("fvgb_piso_face_update");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_piso_velocity_update(const fvgb_mesh* mesh, const double* HbyA,
                                                 const double* rAU, const double* p,
                                                 const double* p_b, double* U, fvgb_stream stream) {
    FVGB_CHECK_ARG(mesh && HbyA && rAU && p && U && (p_b || mesh->v.nbf == 0),
                   "fvgb_piso_velocity_update: null argument");
    k_velocity_update<<<grid_for(mesh->v.n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        mesh->v, HbyA, rAU, p, p_b, U);
    FVGB_LAUNCH_CHECK("fvgb_piso_velocity_update");
    return FVGB_OK;
}
