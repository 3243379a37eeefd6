/*
 * fvoracle.c -- CPU restatement of the FoamAdapter / NeoN finite-volume hot
 * path.  TEST INFRASTRUCTURE ONLY (the checker for the GPU path and the timed
 * CPU baseline); see fvoracle.h for scope and pinning.
 *
 * Floating point: compiled with -ffp-contract=off.  Where the algorithm uses a
 * fused multiply-add (the CG kernels), it calls fma()/fmaf() explicitly, and the
 * dot products follow the fixed two-stage reduction tree that the GPU kernels
 * use (blocks of 256 threads x R rows, warp sums, block sum, sum of block
 * partials), so the CG iterates are reproducible bit for bit.
 */
#include "fvoracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { BC_CALCULATED = 0, BC_FIXED_VALUE = 1, BC_FIXED_GRADIENT = 2 };
enum { SCHEME_LINEAR = 0, SCHEME_UPWIND = 1 };
enum { TERM_DDT = 0, TERM_LAPLACIAN = 1, TERM_DIV = 2, TERM_SOURCE = 3, TERM_EXPLICIT = 4, TERM_DIV_FLUX = 5,
       TERM_DIV_EXPLICIT = 6 };
enum { ST_OK = 0, ST_NOT_CONVERGED = 3, ST_BREAKDOWN = 4, ST_UNSUPPORTED = 6 };

#define RED_THREADS 256
/* rows per thread of the reduction tree: 8 for systems of at least 2^18 rows,
 * 4 below (the GPU solver's choice per case); set by or_solve for its system */
static int g_red_rpt = 8;
#define RED_ROWS_PER_THREAD g_red_rpt
#define RED_ROWS_PER_BLOCK (RED_THREADS * RED_ROWS_PER_THREAD)
static int red_rows_per_thread(int32_t n) { return n >= (1 << 15) ? 8 : 4; }

void or_set_threads(int32_t nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

int32_t or_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* patch type of every boundary face */
static int32_t face_bc(const or_mesh* m, const int32_t* patch_type, int32_t b) {
    for (int32_t p = 0; p < m->npatch; ++p)
        if (b >= m->patch_offs[p] && b < m->patch_offs[p + 1]) return patch_type[p];
    return BC_CALCULATED;
}

/* VolumeField::correctBoundaryConditions for fixedValue / fixedGradient / calculated
 * (readers.hpp:43-95: zeroGradient = fixedGradient 0, noSlip = fixedValue 0).
 * fixedGradient: b = P + g / deltaCoeff (OpenFOAM fixedGradientFvPatchField). */
void or_bc_correct(const or_mesh* m, int32_t nc, const int32_t* patch_type, const double* ref,
                   const double* internal, double* boundary) {
    for (int32_t b = 0; b < m->nbf; ++b) {
        int32_t t = face_bc(m, patch_type, b);
        int32_t P = m->bcells[b];
        for (int32_t k = 0; k < nc; ++k) {
            if (t == BC_FIXED_VALUE) boundary[b * nc + k] = ref[b * nc + k];
            else if (t == BC_FIXED_GRADIENT)
                boundary[b * nc + k] = internal[P * nc + k] + ref[b * nc + k] / m->bdelta[b];
        }
    }
}

/* linear: w*(P - N) + N (pressureVelocityCoupling.cpp:249-251 form); boundary = value */
void or_interp_linear(const or_mesh* m, int32_t nc, const double* src, const double* src_b,
                      double* dst) {
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        for (int32_t k = 0; k < nc; ++k)
            dst[f * nc + k] = m->w[f] * (src[P * nc + k] - src[N * nc + k]) + src[N * nc + k];
    }
    for (int32_t b = 0; b < m->nbf; ++b)
        for (int32_t k = 0; k < nc; ++k) dst[(m->nif + b) * nc + k] = src_b[b * nc + k];
}

void or_interp_upwind(const or_mesh* m, int32_t nc, const double* flux, const double* src,
                      const double* src_b, double* dst) {
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t c = flux[f] >= 0.0 ? m->own[f] : m->nei[f];
        for (int32_t k = 0; k < nc; ++k) dst[f * nc + k] = src[c * nc + k];
    }
    for (int32_t b = 0; b < m->nbf; ++b)
        for (int32_t k = 0; k < nc; ++k) dst[(m->nif + b) * nc + k] = src_b[b * nc + k];
}

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* GaussGreenDiv, Serial executor: res[own] += F*phi_f, res[nei] -= F*phi_f over
 * internal faces in order, res[faceCell] += F_b*phi_b over boundary faces, then
 * out += res * (coeff / V). */
void or_div(const or_mesh* m, int32_t scheme, int32_t nc, const double* flux, const double* phi,
            const double* phi_b, double coeff, double* out) {
    const int32_t nf = m->nif + m->nbf;
    double* phif = zalloc((size_t)nf * nc);
    if (scheme == SCHEME_UPWIND) or_interp_upwind(m, nc, flux, phi, phi_b, phif);
    else or_interp_linear(m, nc, phi, phi_b, phif);
    double* res = zalloc((size_t)m->n * nc);
    for (int32_t f = 0; f < m->nif; ++f)
        for (int32_t k = 0; k < nc; ++k) {
            double fl = flux[f] * phif[f * nc + k];
            res[m->own[f] * nc + k] += fl;
            res[m->nei[f] * nc + k] -= fl;
        }
    for (int32_t b = 0; b < m->nbf; ++b)
        for (int32_t k = 0; k < nc; ++k)
            res[m->bcells[b] * nc + k] += flux[m->nif + b] * phif[(m->nif + b) * nc + k];
    for (int32_t c = 0; c < m->n; ++c) {
        double s = coeff / m->V[c];
        for (int32_t k = 0; k < nc; ++k) out[c * nc + k] += res[c * nc + k] * s;
    }
    free(res);
    free(phif);
}

/* GaussGreenGrad: res[own] += Sf*T_f, res[nei] -= Sf*T_f, boundary += Sf_b*T_b */
void or_grad(const or_mesh* m, const double* phi, const double* phi_b, double coeff, double* out) {
    double* res = zalloc((size_t)m->n * 3);
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        double tf = m->w[f] * (phi[P] - phi[N]) + phi[N];
        for (int32_t k = 0; k < 3; ++k) {
            double v = m->Sf[3 * f + k] * tf;
            res[3 * P + k] += v;
            res[3 * N + k] -= v;
        }
    }
    for (int32_t b = 0; b < m->nbf; ++b)
        for (int32_t k = 0; k < 3; ++k) res[3 * m->bcells[b] + k] += m->bSf[3 * b + k] * phi_b[b];
    for (int32_t c = 0; c < m->n; ++c) {
        double s = coeff / m->V[c];
        for (int32_t k = 0; k < 3; ++k) out[3 * c + k] += res[3 * c + k] * s;
    }
    free(res);
}

/* GaussGreenLaplacian uncorrected: flux = gamma*(|Sf|*delta)*(T_N - T_P) */
void or_laplacian(const or_mesh* m, int32_t nc, const double* gamma, const double* phi,
                  const double* phi_b, double coeff, double* out) {
    double* res = zalloc((size_t)m->n * nc);
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        double g = gamma[f] * (m->magSf[f] * m->delta[f]);
        for (int32_t k = 0; k < nc; ++k) {
            double fl = g * (phi[N * nc + k] - phi[P * nc + k]);
            res[P * nc + k] += fl;
            res[N * nc + k] -= fl;
        }
    }
    for (int32_t b = 0; b < m->nbf; ++b) {
        int32_t P = m->bcells[b];
        double g = gamma[m->nif + b] * (m->bmagSf[b] * m->bdelta[b]);
        for (int32_t k = 0; k < nc; ++k) res[P * nc + k] += g * (phi_b[b * nc + k] - phi[P * nc + k]);
    }
    for (int32_t c = 0; c < m->n; ++c) {
        double s = coeff / m->V[c];
        for (int32_t k = 0; k < nc; ++k) out[c * nc + k] += res[c * nc + k] * s;
    }
    free(res);
}

void or_sngrad(const or_mesh* m, const double* phi, const double* phi_b, double* out) {
    for (int32_t f = 0; f < m->nif; ++f) out[f] = m->delta[f] * (phi[m->nei[f]] - phi[m->own[f]]);
    for (int32_t b = 0; b < m->nbf; ++b)
        out[m->nif + b] = m->bdelta[b] * (phi_b[b] - phi[m->bcells[b]]);
}

/* ---- non-orthogonal correction (OpenFOAM's correctedSnGrad, the method of
 * the `Gauss linear corrected` laplacian, test/setup_stencil3D/system/fvSchemes:43;
 * NeoN's own implementation is not in the reference checkout, so parity is on
 * the published method):
 *   k_f      = Sf/|Sf| - (C_N - C_P)*delta_f      (nonOrthCorrectionVectors)
 *   snGrad_f = delta_f*(T_N - T_P) + k_f . gT_f,  gT_f = w*(g_P - g_N) + g_N
 *   (evaluated with fused multiply-adds, as corr_kg and the callers spell out),
 * g the Gauss linear cell gradient (or_grad, per component); boundary faces of
 * non-coupled patches carry no correction. */
void or_nonorth_vectors(const or_mesh* m, const double* C, double* k) {
    for (int32_t f = 0; f < m->nif; ++f) {
        const int32_t P = m->own[f], N = m->nei[f];
        for (int i = 0; i < 3; ++i) {
            double nf = m->Sf[3 * f + i] / m->magSf[f];
            double df = C[3 * N + i] - C[3 * P + i];
            k[3 * f + i] = nf - df * m->delta[f];
        }
    }
}

/* grad[(c*nc + j)*3 + d]: or_grad of component j */
static double* grad_components(const or_mesh* m, int32_t nc, const double* phi, const double* phi_b) {
    double* grad = zalloc((size_t)m->n * nc * 3);
    double* pj = zalloc((size_t)m->n);
    double* pbj = zalloc((size_t)m->nbf);
    double* gj = zalloc((size_t)m->n * 3);
    for (int32_t j = 0; j < nc; ++j) {
        for (int32_t c = 0; c < m->n; ++c) pj[c] = phi[c * nc + j];
        for (int32_t b = 0; b < m->nbf; ++b) pbj[b] = phi_b[b * nc + j];
        memset(gj, 0, sizeof(double) * (size_t)m->n * 3);
        or_grad(m, pj, pbj, 1.0, gj);
        for (int32_t c = 0; c < m->n; ++c)
            for (int d = 0; d < 3; ++d) grad[(c * nc + j) * 3 + d] = gj[3 * c + d];
    }
    free(gj);
    free(pbj);
    free(pj);
    return grad;
}

/* k_f . gT_f of component j on internal face f with fused multiply-adds:
 * gT = fma(w, g_P - g_N, g_N) per direction, k.gT = fma(k_z, g_z, fma(k_y, g_y, k_x g_x)) */
static double corr_kg(const or_mesh* m, const double* k, const double* grad, int32_t nc, int32_t f, int32_t j) {
    const int32_t P = m->own[f], N = m->nei[f];
    double gf[3];
    for (int d = 0; d < 3; ++d) {
        double gn = grad[(N * nc + j) * 3 + d];
        gf[d] = fma(m->w[f], grad[(P * nc + j) * 3 + d] - gn, gn);
    }
    return fma(k[3 * f + 2], gf[2], fma(k[3 * f + 1], gf[1], k[3 * f] * gf[0]));
}

/* GaussGreenLaplacian corrected: flux_f = fma(gamma*(|Sf|*delta), T_N - T_P,
 * (gamma*|Sf|)*(k . gT_f)); boundary faces uncorrected; out += res*(coeff/V). */
void or_laplacian_corrected(const or_mesh* m, int32_t nc, const double* k, const double* gamma,
                            const double* phi, const double* phi_b, double coeff, double* out) {
    double* grad = grad_components(m, nc, phi, phi_b);
    double* res = zalloc((size_t)m->n * nc);
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        double g = gamma[f] * (m->magSf[f] * m->delta[f]);
        double gm = gamma[f] * m->magSf[f];
        for (int32_t j = 0; j < nc; ++j) {
            double fl = fma(g, phi[N * nc + j] - phi[P * nc + j], gm * corr_kg(m, k, grad, nc, f, j));
            res[P * nc + j] += fl;
            res[N * nc + j] -= fl;
        }
    }
    for (int32_t b = 0; b < m->nbf; ++b) {
        int32_t P = m->bcells[b];
        double g = gamma[m->nif + b] * (m->bmagSf[b] * m->bdelta[b]);
        for (int32_t j = 0; j < nc; ++j) res[P * nc + j] += g * (phi_b[b * nc + j] - phi[P * nc + j]);
    }
    for (int32_t c = 0; c < m->n; ++c) {
        double s = coeff / m->V[c];
        for (int32_t j = 0; j < nc; ++j) out[c * nc + j] += res[c * nc + j] * s;
    }
    free(res);
    free(grad);
}

void or_sngrad_corrected(const or_mesh* m, const double* k, const double* phi, const double* phi_b, double* out) {
    double* grad = grad_components(m, 1, phi, phi_b);
    for (int32_t f = 0; f < m->nif; ++f)
        out[f] = fma(m->delta[f], phi[m->nei[f]] - phi[m->own[f]], corr_kg(m, k, grad, 1, f, 0));
    for (int32_t b = 0; b < m->nbf; ++b)
        out[m->nif + b] = m->bdelta[b] * (phi_b[b] - phi[m->bcells[b]]);
    free(grad);
}

/* faceFluxCorrection: out_f += coeff*((gamma*|Sf|)*(k . gT_f)) on internal faces */
void or_nonorth_flux(const or_mesh* m, int32_t nc, const double* k, const double* gamma, const double* phi,
                     const double* phi_b, double coeff, double* out) {
    double* grad = grad_components(m, nc, phi, phi_b);
    for (int32_t f = 0; f < m->nif; ++f) {
        double gm = gamma[f] * m->magSf[f];
        for (int32_t j = 0; j < nc; ++j) out[f * nc + j] += coeff * (gm * corr_kg(m, k, grad, nc, f, j));
    }
    free(grad);
}

/* The explicit part of a corrected implicit laplacian, volume integrated:
 * rhs_P += coeff * sum_f(+-(gamma*|Sf|)*(k . gT_f)), faces in order (a
 * boundary face adds 0). */
void or_nonorth_rhs(const or_mesh* m, int32_t nc, const double* k, const double* gamma, const double* psi,
                    const double* psi_b, double coeff, double* rhs) {
    double* grad = grad_components(m, nc, psi, psi_b);
    double* res = zalloc((size_t)m->n * nc);
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        double gm = gamma[f] * m->magSf[f];
        for (int32_t j = 0; j < nc; ++j) {
            double fl = gm * corr_kg(m, k, grad, nc, f, j);
            res[P * nc + j] += fl;
            res[N * nc + j] -= fl;
        }
    }
    for (int32_t b = 0; b < m->nbf; ++b)
        for (int32_t j = 0; j < nc; ++j) res[m->bcells[b] * nc + j] += 0.0;
    for (int32_t c = 0; c < m->n; ++c)
        for (int32_t j = 0; j < nc; ++j) rhs[c * nc + j] += res[c * nc + j] * coeff;
    free(res);
    free(grad);
}

/* ddt(T) + div(phi,T) = 0, upwind, forward Euler: T_new = T_old - dt*div(T_old) */
void or_advect_euler(const or_mesh* m, const double* flux, const double* T_old,
                     const double* T_old_b, double dt, const int32_t* patch_type,
                     const double* ref, double* T_new, double* T_new_b) {
    double* dv = zalloc((size_t)m->n);
    or_div(m, SCHEME_UPWIND, 1, flux, T_old, T_old_b, 1.0, dv);
    for (int32_t c = 0; c < m->n; ++c) T_new[c] = T_old[c] - dt * dv[c];
    for (int32_t b = 0; b < m->nbf; ++b) T_new_b[b] = T_old_b[b];
    or_bc_correct(m, 1, patch_type, ref, T_new, T_new_b);
    free(dv);
}

/* la::createSparsity: row P = [lower neighbours ascending, P, upper neighbours
 * ascending]; owner_offset[f] = slot of a_PN in row P, neighbour_offset[f] =
 * slot of a_NP in row N (relative to the row start). Returns nnz or -1. */
int32_t or_sparsity(const or_mesh* m, int32_t* row_offs, int32_t* col, int32_t* diag_off,
                    int32_t* own_off, int32_t* nei_off) {
    const int32_t n = m->n;
    int32_t* cnt = (int32_t*)calloc((size_t)n + 1, sizeof(int32_t));
    for (int32_t f = 0; f < m->nif; ++f) {
        cnt[m->own[f]]++;
        cnt[m->nei[f]]++;
    }
    row_offs[0] = 0;
    for (int32_t c = 0; c < n; ++c) row_offs[c + 1] = row_offs[c] + cnt[c] + 1;
    /* gather neighbour columns per row, then sort (rows are short) */
    int32_t* fill = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    int32_t* slotface = (int32_t*)malloc(sizeof(int32_t) * (size_t)row_offs[n]);
    for (int32_t c = 0; c < n; ++c) {
        col[row_offs[c]] = c;
        slotface[row_offs[c]] = -1;
        fill[c] = 1;
    }
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        col[row_offs[P] + fill[P]] = N;
        slotface[row_offs[P] + fill[P]++] = 2 * f;
        col[row_offs[N] + fill[N]] = P;
        slotface[row_offs[N] + fill[N]++] = 2 * f + 1;
    }
    for (int32_t c = 0; c < n; ++c) {
        int32_t b = row_offs[c], e = row_offs[c + 1];
        for (int32_t i = b + 1; i < e; ++i) { /* insertion sort by column */
            int32_t cc = col[i], sf = slotface[i], j = i - 1;
            while (j >= b && col[j] > cc) {
                col[j + 1] = col[j];
                slotface[j + 1] = slotface[j];
                --j;
            }
            col[j + 1] = cc;
            slotface[j + 1] = sf;
        }
        for (int32_t i = b; i < e; ++i) {
            if (i > b && col[i] == col[i - 1]) { /* two faces between one cell pair */
                free(cnt); free(fill); free(slotface);
                return -1;
            }
            int32_t sf = slotface[i];
            if (sf < 0) diag_off[c] = i - b;
            else if ((sf & 1) == 0) own_off[sf >> 1] = i - b;
            else nei_off[sf >> 1] = i - b;
        }
    }
    int32_t nnz = row_offs[n];
    free(cnt);
    free(fill);
    free(slotface);
    return nnz;
}

/* Implicit assembly.  Terms are applied in order; inside a term the face loop is
 * in ascending face order, scattering like the reference's Serial executor.
 *   DDT:       a_PP += c*V*(1/dt);  b_P += (c*V*(1/dt))*psi_old
 *   SOURCE:    a_PP += (c*s)*V   (s = 1 if absent)
 *   EXPLICIT:  b_P  -= c*E
 *   DIV_FLUX:  E_P = sum of +-F_f (owner +, neighbour -, boundary +, face order); b_P -= c*E_P
 *   DIV_EXPLICIT: E_P = sum of +-F_f*psi_f (psi_f of the term's field, linear or upwind,
 *              boundary psi_b), the Serial face loop of GaussGreenDiv without 1/V; b_P -= c*E_P
 *   LAPLACIAN: g = c*(gamma*(|Sf|*delta)); a_PN += g, a_PP -= g, a_NP += g, a_NN -= g;
 *              boundary value faces: m = c*(gamma_b*(|Sf_b|*delta_b)), r = m*v_b;
 *              fixedGradient faces:  m = 0, r = (c*(gamma_b*|Sf_b|))*g_b
 *   DIV:       cF = c*F; upwind: owner (F>=0 ? a_PP : a_PN) += cF,
 *              neighbour (F>=0 ? a_NP : a_NN) -= cF; linear: owner a_PP += cF*w,
 *              a_PN += cF*(1-w), neighbour a_NP -= cF*w, a_NN -= cF*(1-w);
 *              boundary value faces: m = 0, r = cF*v_b; fixedGradient: m = -cF,
 *              r = cF*(g/delta_b)
 *   boundary faces: a_PP -= m; b_P -= r; bmat += m; brhs += r. */
void or_assemble(const or_mesh* m, const or_csr* A, int32_t nc, const or_term* terms,
                 int32_t nterms, double dt, const int32_t* patch_type, const double* ref,
                 const double* psi_b, double* values, double* rhs, double* bmat, double* brhs) {
    const int32_t n = m->n;
    memset(values, 0, sizeof(double) * (size_t)A->nnz);
    memset(rhs, 0, sizeof(double) * (size_t)n * nc);
    memset(bmat, 0, sizeof(double) * (size_t)m->nbf);
    memset(brhs, 0, sizeof(double) * (size_t)m->nbf * nc);
    const double dtInv = 1.0 / dt;
#define DIAG(c) values[A->row_offs[c] + A->diag_off[c]]
    for (int32_t t = 0; t < nterms; ++t) {
        const or_term* T = &terms[t];
        const double c = T->coeff;
        if (T->kind == TERM_DDT) {
            for (int32_t i = 0; i < n; ++i) {
                double cc = c * m->V[i] * dtInv;
                DIAG(i) += cc;
                for (int32_t k = 0; k < nc; ++k) rhs[i * nc + k] += cc * T->cell[i * nc + k];
            }
        } else if (T->kind == TERM_SOURCE) {
            for (int32_t i = 0; i < n; ++i) DIAG(i) += (T->cell ? c * T->cell[i] : c) * m->V[i];
        } else if (T->kind == TERM_EXPLICIT) {
            for (int32_t i = 0; i < n * nc; ++i) rhs[i] -= c * T->cell[i];
        } else if (T->kind == TERM_DIV_EXPLICIT) {
            const int32_t nf = m->nif + m->nbf;
            double* phif = zalloc((size_t)nf * nc);
            if (T->scheme == SCHEME_UPWIND) or_interp_upwind(m, nc, T->face, T->cell, psi_b, phif);
            else or_interp_linear(m, nc, T->cell, psi_b, phif);
            double* e = zalloc((size_t)n * nc);
            for (int32_t f = 0; f < m->nif; ++f)
                for (int32_t k = 0; k < nc; ++k) {
                    double fl = T->face[f] * phif[f * nc + k];
                    e[m->own[f] * nc + k] += fl;
                    e[m->nei[f] * nc + k] -= fl;
                }
            for (int32_t b = 0; b < m->nbf; ++b)
                for (int32_t k = 0; k < nc; ++k)
                    e[m->bcells[b] * nc + k] += T->face[m->nif + b] * phif[(m->nif + b) * nc + k];
            for (int32_t i = 0; i < n * nc; ++i) rhs[i] -= c * e[i];
            free(e);
            free(phif);
        } else if (T->kind == TERM_DIV_FLUX) {
            double* e = zalloc((size_t)n);
            for (int32_t f = 0; f < m->nif; ++f) {
                e[m->own[f]] += T->face[f];
                e[m->nei[f]] -= T->face[f];
            }
            for (int32_t b = 0; b < m->nbf; ++b) e[m->bcells[b]] += T->face[m->nif + b];
            for (int32_t i = 0; i < n; ++i)
                for (int32_t k = 0; k < nc; ++k) rhs[i * nc + k] -= c * e[i];
            free(e);
        } else if (T->kind == TERM_LAPLACIAN) {
            for (int32_t f = 0; f < m->nif; ++f) {
                int32_t P = m->own[f], N = m->nei[f];
                double g = c * (T->face[f] * (m->magSf[f] * m->delta[f]));
                values[A->row_offs[P] + A->own_off[f]] += g;
                DIAG(P) -= g;
                values[A->row_offs[N] + A->nei_off[f]] += g;
                DIAG(N) -= g;
            }
            for (int32_t b = 0; b < m->nbf; ++b) {
                int32_t P = m->bcells[b], bt = face_bc(m, patch_type, b);
                double gb = T->face[m->nif + b];
                double mm;
                if (bt == BC_FIXED_GRADIENT) {
                    mm = 0.0;
                    double q = c * (gb * m->bmagSf[b]);
                    for (int32_t k = 0; k < nc; ++k) {
                        double r = q * ref[b * nc + k];
                        rhs[P * nc + k] -= r;
                        brhs[b * nc + k] += r;
                    }
                } else {
                    mm = c * (gb * (m->bmagSf[b] * m->bdelta[b]));
                    for (int32_t k = 0; k < nc; ++k) {
                        double r = mm * psi_b[b * nc + k];
                        rhs[P * nc + k] -= r;
                        brhs[b * nc + k] += r;
                    }
                }
                DIAG(P) -= mm;
                bmat[b] += mm;
            }
        } else if (T->kind == TERM_DIV) {
            for (int32_t f = 0; f < m->nif; ++f) {
                int32_t P = m->own[f], N = m->nei[f];
                double F = T->face[f], cF = c * F;
                if (T->scheme == SCHEME_UPWIND) {
                    if (F >= 0.0) {
                        DIAG(P) += cF;
                        values[A->row_offs[N] + A->nei_off[f]] -= cF;
                    } else {
                        values[A->row_offs[P] + A->own_off[f]] += cF;
                        DIAG(N) -= cF;
                    }
                } else {
                    double w = m->w[f], wm = 1.0 - w;
                    DIAG(P) += cF * w;
                    values[A->row_offs[P] + A->own_off[f]] += cF * wm;
                    values[A->row_offs[N] + A->nei_off[f]] -= cF * w;
                    DIAG(N) -= cF * wm;
                }
            }
            for (int32_t b = 0; b < m->nbf; ++b) {
                int32_t P = m->bcells[b], bt = face_bc(m, patch_type, b);
                double cF = c * T->face[m->nif + b];
                double mm;
                if (bt == BC_FIXED_GRADIENT) {
                    mm = -cF;
                    for (int32_t k = 0; k < nc; ++k) {
                        double r = cF * (ref[b * nc + k] / m->bdelta[b]);
                        rhs[P * nc + k] -= r;
                        brhs[b * nc + k] += r;
                    }
                } else {
                    mm = 0.0;
                    for (int32_t k = 0; k < nc; ++k) {
                        double r = cF * psi_b[b * nc + k];
                        rhs[P * nc + k] -= r;
                        brhs[b * nc + k] += r;
                    }
                }
                DIAG(P) -= mm;
                bmat[b] += mm;
            }
        }
    }
#undef DIAG
}

/* PDESolver::SetReference (expression.hpp:102-111) */
void or_set_reference(const or_csr* A, double* values, double* rhs, int32_t r, double v) {
    int32_t d = A->row_offs[r] + A->diag_off[r];
    double dv = values[d];
    rhs[r] += dv * v;
    values[d] += dv;
}

/* out = A x - b, row sums as fma chains in column order */
void or_apply_operator(const or_csr* A, const double* values, const double* rhs, int32_t nc,
                       const double* x, double* out) {
    for (int32_t i = 0; i < A->n; ++i)
        for (int32_t k = 0; k < nc; ++k) {
            double s = 0.0;
            for (int32_t j = A->row_offs[i]; j < A->row_offs[i + 1]; ++j)
                s = fma(values[j], x[A->col[j] * nc + k], s);
            out[i * nc + k] = s - rhs[i * nc + k];
        }
}

/* ---------------------------------------------------------------- reductions */
/* The GPU reduction tree: thread t of a 256-thread block owns rows
 * base + (t/32)*32R + j*32 + t%32, j < R (R = RED_ROWS_PER_THREAD); its partial is a sequential sum;
 * then lane l of warp 0 sums partials l, l+32, ..., l+224 in order and a
 * butterfly (xor 16, 8, 4, 2, 1) finishes.  Stage two: thread t sums block
 * partials t, t+256, ... and the same block tree follows. */
static double block_tree(const double* tp) {
    double v[32], nv[32];
    for (int l = 0; l < 32; ++l) {
        double s = tp[l];
        for (int k = 1; k < RED_THREADS / 32; ++k) s = s + tp[l + 32 * k];
        v[l] = s;
    }
    for (int off = 16; off >= 1; off >>= 1) {
        for (int l = 0; l < 32; ++l) nv[l] = v[l] + v[l ^ off];
        memcpy(v, nv, sizeof v);
    }
    return v[0];
}

/* the same tree in float (block level of the FP32 inner solve) */
static float block_tree_f(const float* tp) {
    float v[32], nv[32];
    for (int l = 0; l < 32; ++l) {
        float s = tp[l];
        for (int k = 1; k < RED_THREADS / 32; ++k) s = s + tp[l + 32 * k];
        v[l] = s;
    }
    for (int off = 16; off >= 1; off >>= 1) {
        for (int l = 0; l < 32; ++l) nv[l] = v[l] + v[l ^ off];
        memcpy(v, nv, sizeof v);
    }
    return v[0];
}

static double final_tree(int32_t nb, const double* partials) {
    double tp[RED_THREADS];
    for (int t = 0; t < RED_THREADS; ++t) {
        double a = 0.0;
        for (int32_t i = t; i < nb; i += RED_THREADS) a = a + partials[i];
        tp[t] = a;
    }
    return block_tree(tp);
}

static inline int32_t red_row(int32_t blk, int t, int j) {
    return blk * RED_ROWS_PER_BLOCK + (t >> 5) * (32 * RED_ROWS_PER_THREAD) + j * 32 + (t & 31);
}

static int32_t nblocks_of(int32_t n) { return (n + RED_ROWS_PER_BLOCK - 1) / RED_ROWS_PER_BLOCK; }

double or_dot_tree(int32_t n, const double* a, const double* b) {
    int32_t nb = nblocks_of(n);
    double* part = zalloc((size_t)nb);
#pragma omp parallel for schedule(static)
    for (int32_t blk = 0; blk < nb; ++blk) {
        double tp[RED_THREADS];
        for (int t = 0; t < RED_THREADS; ++t) {
            double acc = 0.0;
            for (int j = 0; j < RED_ROWS_PER_THREAD; ++j) {
                int32_t i = red_row(blk, t, j);
                if (i < n) acc = fma(a[i], b[i], acc);
            }
            tp[t] = acc;
        }
        part[blk] = block_tree(tp);
    }
    double r = final_tree(nb, part);
    free(part);
    return r;
}

/* The baseline of the relative tolerance: ||b|| by the GPU's reduction tree when
 * the configuration asks for Ginkgo's default ResidualNorm baseline (rhs_norm),
 * else the initial residual norm. */
static double tol_base(const or_csr* A, const double* b, const or_solver_cfg* cfg, double res0) {
    return (cfg->flags & 2) ? sqrt(or_dot_tree(A->n, b, b)) : res0;
}

/* ------------------------------------------------------------ FP64 Jacobi CG */
static void spmv_row_fma(const or_csr* A, const double* val, const double* x, int32_t i, double* s) {
    double acc = 0.0;
    for (int32_t j = A->row_offs[i]; j < A->row_offs[i + 1]; ++j) acc = fma(val[j], x[A->col[j]], acc);
    *s = acc;
}

static int32_t solve_fp64(const or_csr* A, const double* val, const double* b, double* x,
                          const or_solver_cfg* cfg, or_solver_stats* st) {
    const int32_t n = A->n, nb = nblocks_of(n);
    double *dinv = zalloc(n), *r = zalloc(n), *p = zalloc(n), *q = zalloc(n);
    double *pa = zalloc(nb), *pb = zalloc(nb);
    for (int32_t i = 0; i < n; ++i) dinv[i] = 1.0 / val[A->row_offs[i] + A->diag_off[i]];
    /* init: r = b - A x; z = dinv*r; p = z; rz, rr */
#pragma omp parallel for schedule(static)
    for (int32_t blk = 0; blk < nb; ++blk) {
        double ta[RED_THREADS], tb[RED_THREADS];
        for (int t = 0; t < RED_THREADS; ++t) {
            double arz = 0.0, arr = 0.0;
            for (int j = 0; j < RED_ROWS_PER_THREAD; ++j) {
                int32_t i = red_row(blk, t, j);
                if (i >= n) continue;
                double s;
                spmv_row_fma(A, val, x, i, &s);
                double ri = b[i] - s, zi = dinv[i] * ri;
                r[i] = ri;
                p[i] = zi;
                arz = fma(ri, zi, arz);
                arr = fma(ri, ri, arr);
            }
            ta[t] = arz;
            tb[t] = arr;
        }
        pa[blk] = block_tree(ta);
        pb[blk] = block_tree(tb);
    }
    double rz = final_tree(nb, pa), rr = final_tree(nb, pb);
    double res0 = sqrt(rr), res = res0;
    double tol = cfg->rel_tol * tol_base(A, b, cfg, res0);
    if (cfg->abs_tol > tol) tol = cfg->abs_tol;
    int32_t it = 0, status = ST_OK;
    int done = !(res > tol) || res == 0.0;
    if (!isfinite(res)) { done = 1; status = ST_BREAKDOWN; }
    else if (!done && cfg->max_iter <= 0) { done = 1; status = ST_NOT_CONVERGED; }
    while (!done) {
        /* q = A p ; pq */
#pragma omp parallel for schedule(static)
        for (int32_t blk = 0; blk < nb; ++blk) {
            double ta[RED_THREADS];
            for (int t = 0; t < RED_THREADS; ++t) {
                double acc = 0.0;
                for (int j = 0; j < RED_ROWS_PER_THREAD; ++j) {
                    int32_t i = red_row(blk, t, j);
                    if (i >= n) continue;
                    double s;
                    spmv_row_fma(A, val, p, i, &s);
                    q[i] = s;
                    acc = fma(p[i], s, acc);
                }
                ta[t] = acc;
            }
            pa[blk] = block_tree(ta);
        }
        double pq = final_tree(nb, pa);
        double alpha = rz / pq;
        if (pq == 0.0 || !isfinite(alpha)) { status = ST_BREAKDOWN; break; }
        /* x += alpha p ; r -= alpha q ; z = dinv r ; rz, rr */
#pragma omp parallel for schedule(static)
        for (int32_t blk = 0; blk < nb; ++blk) {
            double ta[RED_THREADS], tb[RED_THREADS];
            for (int t = 0; t < RED_THREADS; ++t) {
                double arz = 0.0, arr = 0.0;
                for (int j = 0; j < RED_ROWS_PER_THREAD; ++j) {
                    int32_t i = red_row(blk, t, j);
                    if (i >= n) continue;
                    x[i] = fma(alpha, p[i], x[i]);
                    double ri = fma(-alpha, q[i], r[i]);
                    r[i] = ri;
                    double zi = dinv[i] * ri;
                    arz = fma(ri, zi, arz);
                    arr = fma(ri, ri, arr);
                }
                ta[t] = arz;
                tb[t] = arr;
            }
            pa[blk] = block_tree(ta);
            pb[blk] = block_tree(tb);
        }
        double rzn = final_tree(nb, pa);
        rr = final_tree(nb, pb);
        res = sqrt(rr);
        ++it;
        double beta = rzn / rz;
        rz = rzn;
        if (!isfinite(res)) { status = ST_BREAKDOWN; break; }
        if (!(res > tol)) break;
        if (it >= cfg->max_iter) { status = ST_NOT_CONVERGED; break; }
        /* p = z + beta p */
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i) p[i] = fma(beta, p[i], dinv[i] * r[i]);
    }
    st->init_res_norm = res0;
    st->final_res_norm = res;
    st->num_iter = it;
    st->num_outer = 0;
    st->status = status;
    free(dinv); free(r); free(p); free(q); free(pa); free(pb);
    return status;
}

/* ---------------------------------- mixed precision CG with reliable updates
 * (solver.cu, mixed-precision section)
 * FP32 CG on the row-sign-normalised system D_s A y = D_s r (D_s = sign of each
 * row's diagonal; all diagonals must share one sign), Jacobi-preconditioned with
 * |1/a_ii| held as the FP32 dinv = (float)(1/a_ii).  The FP32 SpMV is the
 * difference form: a32_ij = (float)(sign*a_ij) off the diagonal, ev_i =
 * (float)(sign*e_i) with e_i the FP64 row sum in column order, and
 * q_i = fmaf(ev_i, p_i, sum fmaf(a32_ij, p_j - p_i, .)) over the row in column
 * order (the diagonal entry holds 0).
 * Dots: per-thread fmaf and block tree in float, block partials summed in double.
 * Residuals are scaled by sig = 2^-ilogb(|D^-1/2 r_prev|), exactly.
 * Reliable update (FP64): when rho has dropped below rho_ref*max(d^2, (tol/res)^2)
 * (d = inner_rel_tol) or after inner_max_iter steps, x += y/sig, r = b - A x is
 * recomputed, tested, and replaces the FP32 residual; the direction continues
 * with beta = rho_true/rho_prev, restarted from z when no step ran or when
 * rho_true > 4 rho_recursive (drift of the FP32 recursion). */
static double dot_tree_f(int32_t n, const float* a, const float* b, double* part) {
    int32_t nb = nblocks_of(n);
#pragma omp parallel for schedule(static)
    for (int32_t blk = 0; blk < nb; ++blk) {
        float tp[RED_THREADS];
        for (int t = 0; t < RED_THREADS; ++t) {
            float acc = 0.0f;
            for (int j = 0; j < RED_ROWS_PER_THREAD; ++j) {
                int32_t i = red_row(blk, t, j);
                if (i < n) acc = fmaf(a[i], b[i], acc);
            }
            tp[t] = acc;
        }
        part[blk] = (double)block_tree_f(tp);
    }
    return final_tree(nb, part);
}

/* Power-of-two scale bringing |D^-1/2 r| to [1, 2) (solver.cu residual_scale): exact,
 * it only keeps the FP32 products of a tiny residual out of the subnormal range. */
static void residual_scale(double sres, double* sig, double* isig) {
    int e = 0;
    if (sres > 0.0 && isfinite(sres)) {
        e = ilogb(sres);
        e = e > 900 ? 900 : (e < -900 ? -900 : e);
    }
    *sig = ldexp(1.0, -e);
    *isig = ldexp(1.0, e);
}

/* r = b - A x; rh = sign*(float)(r*sig), z = |dinv|*rh; returns |r|,
 * *sres = sqrt(sum r^2 |dinv|) (both by the GPU's tree) */
static double residual_step(const or_csr* A, const double* val, const double* b, const double* x,
                            const float* dinv, double sig, float* rh, float* z, double* part, double* part2,
                            int32_t n, int32_t nb, double* sres) {
#pragma omp parallel for schedule(static)
    for (int32_t blk = 0; blk < nb; ++blk) {
        double tp[RED_THREADS], tq[RED_THREADS];
        for (int t = 0; t < RED_THREADS; ++t) {
            double arr = 0.0, asr = 0.0;
            for (int j = 0; j < RED_ROWS_PER_THREAD; ++j) {
                int32_t i = red_row(blk, t, j);
                if (i >= n) continue;
                double sm;
                spmv_row_fma(A, val, x, i, &sm);
                double ri = b[i] - sm;
                arr = fma(ri, ri, arr);
                asr = fma(ri * (double)fabsf(dinv[i]), ri, asr);
                float rhi = (float)(ri * sig);
                if (dinv[i] < 0.0f) rhi = -rhi;
                rh[i] = rhi;
                z[i] = fabsf(dinv[i]) * rhi;
            }
            tp[t] = arr;
            tq[t] = asr;
        }
        part[blk] = block_tree(tp);
        part2[blk] = block_tree(tq);
    }
    *sres = sqrt(final_tree(nb, part2));
    return sqrt(final_tree(nb, part));
}

/* The row-sign-normalised FP32 system (solver.cu k_ir_prepare): dinv = (float)(1/a_ii),
 * a32 = (float)(sign*a_ij) off the diagonal (0 on it), ev = (float)(sign*e_i), e_i the
 * FP64 row sum in column order.  Returns the sign flags: bit0 a positive diagonal,
 * bit1 negative, bit2 zero/NaN. */
static unsigned prepare_f32(const or_csr* A, const double* val, float* dinv, float* ev, float* a32) {
    unsigned flags = 0;
    for (int32_t i = 0; i < A->n; ++i) {
        double d = val[A->row_offs[i] + A->diag_off[i]];
        flags |= d > 0.0 ? 1u : (d < 0.0 ? 2u : 4u);
        dinv[i] = (float)(1.0 / d);
        double sg = d < 0.0 ? -1.0 : 1.0, e = 0.0;
        for (int32_t j = A->row_offs[i]; j < A->row_offs[i + 1]; ++j) {
            e = e + val[j];
            a32[j] = A->col[j] == i ? 0.0f : (float)(sg * val[j]);
        }
        ev[i] = (float)(sg * e);
    }
    return flags;
}

/* q = (D_s A) x in the difference form, fmaf chain in column order */
static void spmv_diff_f(const or_csr* A, const float* a32, const float* ev, const float* x, float* q) {
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < A->n; ++i) {
        const float xi = x[i];
        float acc = 0.0f;
        for (int32_t j = A->row_offs[i]; j < A->row_offs[i + 1]; ++j) acc = fmaf(a32[j], x[A->col[j]] - xi, acc);
        q[i] = fmaf(ev[i], xi, acc);
    }
}

static int32_t solve_mixed(const or_csr* A, const double* val, const double* b, double* x,
                           const or_solver_cfg* cfg, or_solver_stats* st) {
    const int32_t n = A->n, nb = nblocks_of(n), nnz = A->nnz;
    float* dinv = (float*)calloc(n ? n : 1, sizeof(float));
    float* ev = (float*)calloc(n ? n : 1, sizeof(float));
    float* a32 = (float*)calloc((size_t)(nnz ? nnz : 1), sizeof(float));
    unsigned flags = prepare_f32(A, val, dinv, ev, a32);
    if ((flags & 4u) || flags == 3u) {
        free(dinv); free(ev); free(a32);
        st->status = ST_UNSUPPORTED;
        return ST_UNSUPPORTED;
    }
    const double dr = cfg->inner_rel_tol * cfg->inner_rel_tol;
    double *part = zalloc(nb), *part2 = zalloc(nb);
    float *rh = (float*)calloc(n, sizeof(float)), *y = (float*)calloc(n, sizeof(float));
    float *p = (float*)calloc(n, sizeof(float)), *q = (float*)calloc(n, sizeof(float));
    float *z = (float*)calloc(n, sizeof(float));
    int32_t total = 0, outer = 0, status = ST_OK, inner_it = 0;
    double rho, rho_prev = 0.0, itol, res, res0, tol, sres, sig, isig;
    /* |D^-1/2 r0| sets the scale of the first residual (k_ir_prepare), then the first residual */
    residual_step(A, val, b, x, dinv, 1.0, rh, z, part, part2, n, nb, &sres);
    residual_scale(sres, &sig, &isig);
    res = residual_step(A, val, b, x, dinv, sig, rh, z, part, part2, n, nb, &sres);
    for (int32_t i = 0; i < n; ++i) { y[i] = 0.0f; p[i] = z[i]; }
    rho = dot_tree_f(n, rh, z, part);
    res0 = res;
    tol = cfg->rel_tol * tol_base(A, b, cfg, res0);
    if (cfg->abs_tol > tol) tol = cfg->abs_tol;
    int done = 0;
    if (!isfinite(res)) { status = ST_BREAKDOWN; done = 1; }
    else if (!(res > tol) || res == 0.0) done = 1;
    else if (cfg->max_outer <= 0 || cfg->max_iter <= 0) { status = ST_NOT_CONVERGED; done = 1; }
    { double dt = (tol / res) * (tol / res); itol = rho * (dr > dt ? dr : dt); }
    int inner = !done && rho > itol && cfg->inner_max_iter > 0 && total < cfg->max_iter;
    while (!done) {
        while (inner) {
#pragma omp parallel for schedule(static)
            for (int32_t i = 0; i < n; ++i) {
                const float pi = p[i];
                float acc = 0.0f;
                for (int32_t j = A->row_offs[i]; j < A->row_offs[i + 1]; ++j)
                    acc = fmaf(a32[j], p[A->col[j]] - pi, acc);
                q[i] = fmaf(ev[i], pi, acc);
            }
            double pq = dot_tree_f(n, p, q, part);
            double alpha = rho / pq;
            if (pq == 0.0 || !isfinite(alpha)) {
                inner = 0;
                if (inner_it == 0) { status = ST_BREAKDOWN; done = 1; }
                break;
            }
            float fa = (float)alpha;
            for (int32_t i = 0; i < n; ++i) {
                y[i] = fmaf(fa, p[i], y[i]);
                rh[i] = fmaf(-fa, q[i], rh[i]);
                z[i] = fabsf(dinv[i]) * rh[i];
            }
            double rhon = dot_tree_f(n, rh, z, part);
            float fb = (float)(rhon / rho);
            rho_prev = rho;
            rho = rhon;
            ++inner_it;
            ++total;
            int more = rhon > itol && inner_it < cfg->inner_max_iter && total < cfg->max_iter;
            if (!more) { inner = 0; break; }
            for (int32_t i = 0; i < n; ++i) p[i] = fmaf(fb, p[i], z[i]);
        }
        if (done) break;
        /* reliable update; the new residual takes the scale of the previous |D^-1/2 r| */
        for (int32_t i = 0; i < n; ++i) x[i] = fma((double)y[i], isig, x[i]);
        const double sig_old = sig, isig_old = isig;
        residual_scale(sres, &sig, &isig);
        res = residual_step(A, val, b, x, dinv, sig, rh, z, part, part2, n, nb, &sres);
        for (int32_t i = 0; i < n; ++i) y[i] = 0.0f;
        double rho_true = dot_tree_f(n, rh, z, part);
        ++outer;
        if (!isfinite(res)) { status = ST_BREAKDOWN; done = 1; }
        else if (!(res > tol) || res == 0.0) done = 1;
        else if (outer >= cfg->max_outer || total >= cfg->max_iter) { status = ST_NOT_CONVERGED; done = 1; }
        /* restart when no step ran or the FP32 recursion drifted (true rho > 4x recursive) */
        const double g = sig * isig_old, rho_rec = rho * g * g;
        const int restart = inner_it == 0 || rho_true > 4.0 * rho_rec;
        float frel = restart ? -1.0f : (float)((rho_true / rho_prev) * (sig_old * isig));
        rho = rho_true;
        { double dt = (tol / res) * (tol / res); itol = rho * (dr > dt ? dr : dt); }
        inner_it = 0;
        inner = !done && rho > itol && cfg->inner_max_iter > 0 && total < cfg->max_iter;
        if (inner)
            for (int32_t i = 0; i < n; ++i) p[i] = frel < 0.0f ? z[i] : fmaf(frel, p[i], z[i]);
    }
    st->init_res_norm = res0;
    st->final_res_norm = res;
    st->num_iter = total;
    st->num_outer = outer;
    st->status = status;
    free(dinv); free(ev); free(a32); free(part); free(part2); free(rh); free(y); free(p); free(q); free(z);
    return status;
}

/* ------------------------------------------------------------- BiCGStab
 * Jacobi-preconditioned BiCGStab (Ginkgo's solver::Bicgstab as FoamAdapter
 * selects it, fvSolution.cpp:25-26, 106-142), right preconditioning, FP64,
 * in the operation order of the GPU kernels (solver.cu BiCGStab section); every
 * dot product by the GPU's reduction tree.  With an ILU(0) factor (lu), y and
 * z below are M^-1 p and M^-1 s (ilu.cu) instead of D^-1 p and D^-1 s.
 *   r = b - A x, rr = r, p = v = 0, rho = (rr, r), rho_prev = alpha = omega = 1
 *   loop: beta = (rho/rho_prev)(alpha/omega); p = r + beta (p - omega v); y = D^-1 p
 *         v = A y; alpha = rho / (rr, v); s = r - alpha v
 *         |s| converged: x += alpha y, stop
 *         z = D^-1 s; t = A z; omega = (t, s) / (t, t)
 *         x += alpha y + omega z; r = s - omega t; rho_prev = rho; rho = (rr, r); |r| */
static double dot64(int32_t n, const double* a, const double* b, double* part) {
    int32_t nb = nblocks_of(n);
#pragma omp parallel for schedule(static)
    for (int32_t blk = 0; blk < nb; ++blk) {
        double tp[RED_THREADS];
        for (int t = 0; t < RED_THREADS; ++t) {
            double acc = 0.0;
            for (int j = 0; j < RED_ROWS_PER_THREAD; ++j) {
                int32_t i = red_row(blk, t, j);
                if (i < n) acc = fma(a[i], b[i], acc);
            }
            tp[t] = acc;
        }
        part[blk] = block_tree(tp);
    }
    return final_tree(nb, part);
}

static void spmv_all(const or_csr* A, const double* val, const double* x, double* out) {
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < A->n; ++i) {
        double s;
        spmv_row_fma(A, val, x, i, &s);
        out[i] = s;
    }
}

static int32_t solve_bicgstab(const or_csr* A, const double* val, const double* b, double* x,
                              const or_solver_cfg* cfg, or_solver_stats* st, const double* lu) {
    const int32_t n = A->n, nb = nblocks_of(n);
    double *dinv = zalloc(n), *r = zalloc(n), *rr = zalloc(n), *p = zalloc(n), *v = zalloc(n);
    double *y = zalloc(n), *s = zalloc(n), *z = zalloc(n), *t = zalloc(n), *part = zalloc(nb);
    double* fw = lu ? zalloc(n) : NULL;  /* ILU: the forward solve's result */
    for (int32_t i = 0; i < n; ++i) dinv[i] = 1.0 / val[A->row_offs[i] + A->diag_off[i]];
    spmv_all(A, val, x, t);
    for (int32_t i = 0; i < n; ++i) {
        r[i] = b[i] - t[i];
        rr[i] = r[i];
    }
    double rho = dot64(n, rr, r, part);
    double res0 = sqrt(dot64(n, r, r, part)), res = res0;
    double tol = cfg->rel_tol * tol_base(A, b, cfg, res0);
    if (cfg->abs_tol > tol) tol = cfg->abs_tol;
    double rho_prev = 1.0, alpha = 1.0, omega = 1.0;
    int32_t it = 0, status = ST_OK;
    int done = !(res > tol) || res == 0.0;
    if (!isfinite(res)) { done = 1; status = ST_BREAKDOWN; }
    else if (!done && cfg->max_iter <= 0) { done = 1; status = ST_NOT_CONVERGED; }
    while (!done) {
        const double beta = (rho / rho_prev) * (alpha / omega);
        for (int32_t i = 0; i < n; ++i) {
            p[i] = fma(beta, fma(-omega, v[i], p[i]), r[i]);
            if (!lu) y[i] = dinv[i] * p[i];
        }
        if (lu) or_ilu_apply(A, lu, p, fw, y);
        spmv_all(A, val, y, v);
        const double rv = dot64(n, rr, v, part);
        alpha = rho / rv;
        if (rv == 0.0 || !isfinite(alpha)) { status = ST_BREAKDOWN; break; }
        for (int32_t i = 0; i < n; ++i) {
            s[i] = fma(-alpha, v[i], r[i]);
            if (!lu) z[i] = dinv[i] * s[i];
        }
        const double sres = sqrt(dot64(n, s, s, part));
        if (!isfinite(sres)) { status = ST_BREAKDOWN; res = sres; break; }
        if (!(sres > tol)) {  /* converged at the half step */
            for (int32_t i = 0; i < n; ++i) x[i] = fma(alpha, y[i], x[i]);
            ++it;
            res = sres;
            break;
        }
        if (lu) or_ilu_apply(A, lu, s, fw, z);
        spmv_all(A, val, z, t);
        const double ts = dot64(n, t, s, part), tt = dot64(n, t, t, part);
        omega = ts / tt;
        if (tt == 0.0 || !isfinite(omega) || omega == 0.0) { status = ST_BREAKDOWN; break; }
        for (int32_t i = 0; i < n; ++i) {
            x[i] = fma(omega, z[i], fma(alpha, y[i], x[i]));
            r[i] = fma(-omega, t[i], s[i]);
        }
        rho_prev = rho;
        rho = dot64(n, rr, r, part);
        res = sqrt(dot64(n, r, r, part));
        ++it;
        if (!isfinite(res)) { status = ST_BREAKDOWN; break; }
        if (!(res > tol)) break;
        if (it >= cfg->max_iter) { status = ST_NOT_CONVERGED; break; }
        if (rho == 0.0) { status = ST_BREAKDOWN; break; }
    }
    st->init_res_norm = res0;
    st->final_res_norm = res;
    st->num_iter = it;
    st->num_outer = 0;
    st->status = status;
    free(dinv); free(r); free(rr); free(p); free(v); free(y); free(s); free(z); free(t); free(part); free(fw);
    return status;
}

/* ---------------------------------------------------- mixed-precision BiCGStab
 * FP64 iterative refinement around a restarted FP32 BiCGStab on the
 * row-sign-normalised system (solver.cu mixed BiCGStab section, same operation
 * order): each refinement step r = b - A x, rh = sign*(float)(sig r), then from
 * e = 0, rr = rh, p = v = 0, rho = rh.rh, fbeta = 0, alpha = omega = 1:
 *   p = r + beta (p - omega v); yv = |dinv| p; v = A32 yv; alpha = rho/(rr.v)
 *   s = r - alpha v; z = |dinv| s; |s|^2 <= itol: e += alpha yv, stop
 *   t = A32 z; omega = (t.s)/(t.t); e += alpha yv + omega z; r = s - omega t
 *   beta = (rr.r / rho)(alpha/omega); stop when |r|^2 <= itol
 * itol = rho0 max(inner_rel_tol^2, (tol/|r|)^2); x += e / sig. */
static int32_t solve_mixed_bicgstab(const or_csr* A, const double* val, const double* b, double* x,
                                    const or_solver_cfg* cfg, or_solver_stats* st) {
    const int32_t n = A->n, nb = nblocks_of(n), nnz = A->nnz;
    const size_t nn = n ? (size_t)n : 1;
    float* dinv = (float*)calloc(nn, sizeof(float));
    float* ev = (float*)calloc(nn, sizeof(float));
    float* a32 = (float*)calloc((size_t)(nnz ? nnz : 1), sizeof(float));
    unsigned flags = prepare_f32(A, val, dinv, ev, a32);
    double *part = zalloc(nb), *part2 = zalloc(nb);
    float *r = (float*)calloc(nn, sizeof(float)), *rr = (float*)calloc(nn, sizeof(float));
    float *p = (float*)calloc(nn, sizeof(float)), *v = (float*)calloc(nn, sizeof(float));
    float *yv = (float*)calloc(nn, sizeof(float)), *sv = (float*)calloc(nn, sizeof(float));
    float *z = (float*)calloc(nn, sizeof(float)), *t = (float*)calloc(nn, sizeof(float));
    float *e = (float*)calloc(nn, sizeof(float)), *scratch = (float*)calloc(nn, sizeof(float));
    const double dr = cfg->inner_rel_tol * cfg->inner_rel_tol;
    int32_t total = 0, outer = 0, status = ST_OK;
    double res, res0, tol, sres, sig, isig;
    residual_step(A, val, b, x, dinv, 1.0, r, scratch, part, part2, n, nb, &sres);
    residual_scale(sres, &sig, &isig);
    res = residual_step(A, val, b, x, dinv, sig, r, scratch, part, part2, n, nb, &sres);
    res0 = res;
    tol = cfg->rel_tol * tol_base(A, b, cfg, res0);
    if (cfg->abs_tol > tol) tol = cfg->abs_tol;
    int done = 0;
    if ((flags & 4u) || flags == 3u) { status = ST_UNSUPPORTED; done = 1; }
    else if (!isfinite(res)) { status = ST_BREAKDOWN; done = 1; }
    else if (!(res > tol) || res == 0.0) done = 1;
    else if (cfg->max_outer <= 0 || cfg->max_iter <= 0) { status = ST_NOT_CONVERGED; done = 1; }
    for (;;) {
        /* the inner solve of this refinement step */
        for (int32_t i = 0; i < n; ++i) { rr[i] = r[i]; p[i] = 0.0f; v[i] = 0.0f; e[i] = 0.0f; }
        double rho = dot_tree_f(n, r, r, part), alpha = 1.0, omega = 1.0;
        float fa = 1.0f, fo = 1.0f, fb = 0.0f;
        double itol;
        { double dt = (tol / res) * (tol / res); itol = rho * (dr > dt ? dr : dt); }
        int32_t inner_it = 0;
        int inner = !done && rho > itol && cfg->inner_max_iter > 0 && total < cfg->max_iter;
        while (inner) {
            for (int32_t i = 0; i < n; ++i) {
                p[i] = fmaf(fb, fmaf(-fo, v[i], p[i]), r[i]);
                yv[i] = fabsf(dinv[i]) * p[i];
            }
            spmv_diff_f(A, a32, ev, yv, v);
            double rv = dot_tree_f(n, rr, v, part);
            double al = rho / rv;
            if (rv == 0.0 || !isfinite(al)) {
                if (inner_it == 0) { status = ST_BREAKDOWN; done = 1; }
                break;
            }
            alpha = al;
            fa = (float)alpha;
            for (int32_t i = 0; i < n; ++i) {
                sv[i] = fmaf(-fa, v[i], r[i]);
                z[i] = fabsf(dinv[i]) * sv[i];
            }
            double ss = dot_tree_f(n, sv, sv, part);
            if (!isfinite(ss)) {
                if (inner_it == 0) { status = ST_BREAKDOWN; done = 1; }
                break;
            }
            if (!(ss > itol)) { /* half step */
                for (int32_t i = 0; i < n; ++i) e[i] = fmaf(fa, yv[i], e[i]);
                ++inner_it;
                ++total;
                break;
            }
            spmv_diff_f(A, a32, ev, z, t);
            double ts = dot_tree_f(n, t, sv, part), tt = dot_tree_f(n, t, t, part2);
            double om = ts / tt;
            if (tt == 0.0 || !isfinite(om) || om == 0.0) {
                if (inner_it == 0) { status = ST_BREAKDOWN; done = 1; }
                break;
            }
            omega = om;
            fo = (float)omega;
            for (int32_t i = 0; i < n; ++i) {
                e[i] = fmaf(fo, z[i], fmaf(fa, yv[i], e[i]));
                r[i] = fmaf(-fo, t[i], sv[i]);
            }
            double rhon = dot_tree_f(n, rr, r, part), r2 = dot_tree_f(n, r, r, part2);
            ++inner_it;
            ++total;
            double beta = (rhon / rho) * (alpha / omega);
            rho = rhon;
            fb = (float)beta;
            int more = r2 > itol && isfinite(r2) && rho != 0.0 && isfinite(beta) && inner_it < cfg->inner_max_iter &&
                       total < cfg->max_iter;
            if (!more) break;
        }
        if (done) break;
        for (int32_t i = 0; i < n; ++i) x[i] = fma((double)e[i], isig, x[i]);
        residual_scale(sres, &sig, &isig);
        res = residual_step(A, val, b, x, dinv, sig, r, scratch, part, part2, n, nb, &sres);
        ++outer;
        if (!isfinite(res)) { status = ST_BREAKDOWN; done = 1; }
        else if (!(res > tol) || res == 0.0) done = 1;
        else if (outer >= cfg->max_outer || total >= cfg->max_iter) { status = ST_NOT_CONVERGED; done = 1; }
        if (done) break;
    }
    st->init_res_norm = res0;
    st->final_res_norm = res;
    st->num_iter = total;
    st->num_outer = outer;
    st->status = status;
    free(dinv); free(ev); free(a32); free(part); free(part2); free(r); free(rr); free(p); free(v); free(yv);
    free(sv); free(z); free(t); free(e); free(scratch);
    return status;
}

/* ------------------------------------------------------------------ BiCG (FP64)
 * Jacobi-preconditioned BiCG, Ginkgo's solver::Bicg (FoamAdapter maps PBiCG to
 * it, fvSolution.cpp:24), in the operation order of the GPU kernels
 * (solver.cu, BiCG section):
 *   r = b - A x; r2 = r; z = D^-1 r; z2 = D^-1 r2; p = p2 = 0; rho = (r2, z); beta = rho / 1
 *   loop: p = z + beta p; p2 = z2 + beta p2; q = A p; q2 = A^T p2;
 *         alpha = rho / (p2, q); x += alpha p; r -= alpha q; r2 -= alpha q2;
 *         z = D^-1 r; z2 = D^-1 r2; rho' = (r2, z); |r|; beta = rho' / rho
 * (A^T x)_i runs over row i's columns j in order with the value a_ji. */
static int32_t solve_bicg(const or_csr* A, const double* val, const double* b, double* x,
                          const or_solver_cfg* cfg, or_solver_stats* st) {
    const int32_t n = A->n, nb = nblocks_of(n);
    double *dinv = zalloc(n), *r = zalloc(n), *r2 = zalloc(n), *z = zalloc(n), *z2 = zalloc(n);
    double *p = zalloc(n), *p2 = zalloc(n), *q = zalloc(n), *q2 = zalloc(n), *part = zalloc(nb);
    int32_t* tpos = (int32_t*)calloc((size_t)(A->nnz ? A->nnz : 1), sizeof(int32_t));
    /* position of a_ji for every entry (i, j): binary search of column i in row j */
    for (int32_t i = 0; i < n; ++i)
        for (int32_t e = A->row_offs[i]; e < A->row_offs[i + 1]; ++e) {
            const int32_t j = A->col[e];
            int32_t lo = A->row_offs[j], hi = A->row_offs[j + 1] - 1, at = -1;
            while (lo <= hi) {
                const int32_t mid = (lo + hi) / 2;
                if (A->col[mid] == i) { at = mid; break; }
                if (A->col[mid] < i) lo = mid + 1; else hi = mid - 1;
            }
            tpos[e] = at;
        }
    for (int32_t i = 0; i < n; ++i) dinv[i] = 1.0 / val[A->row_offs[i] + A->diag_off[i]];
    spmv_all(A, val, x, q);
    for (int32_t i = 0; i < n; ++i) {
        r[i] = b[i] - q[i];
        r2[i] = r[i];
        z[i] = dinv[i] * r[i];
        z2[i] = z[i];
    }
    double rho = dot64(n, r2, z, part);
    double res0 = sqrt(dot64(n, r, r, part)), res = res0;
    double tol = cfg->rel_tol * tol_base(A, b, cfg, res0);
    if (cfg->abs_tol > tol) tol = cfg->abs_tol;
    double beta = rho / 1.0;
    int32_t it = 0, status = ST_OK;
    int done = !(res > tol) || res == 0.0;
    if (!isfinite(res)) { done = 1; status = ST_BREAKDOWN; }
    else if (!done && cfg->max_iter <= 0) { done = 1; status = ST_NOT_CONVERGED; }
    else if (!done && !(rho != 0.0 && isfinite(rho))) { done = 1; status = ST_BREAKDOWN; }
    while (!done) {
        for (int32_t i = 0; i < n; ++i) {
            p[i] = fma(beta, p[i], z[i]);
            p2[i] = fma(beta, p2[i], z2[i]);
        }
        spmv_all(A, val, p, q);
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i) {
            double s = 0.0;
            for (int32_t e = A->row_offs[i]; e < A->row_offs[i + 1]; ++e) s = fma(val[tpos[e]], p2[A->col[e]], s);
            q2[i] = s;
        }
        const double pq = dot64(n, p2, q, part);
        const double alpha = rho / pq;
        if (pq == 0.0 || !isfinite(alpha)) { status = ST_BREAKDOWN; break; }
        for (int32_t i = 0; i < n; ++i) {
            x[i] = fma(alpha, p[i], x[i]);
            r[i] = fma(-alpha, q[i], r[i]);
            r2[i] = fma(-alpha, q2[i], r2[i]);
            z[i] = dinv[i] * r[i];
            z2[i] = dinv[i] * r2[i];
        }
        const double rho_new = dot64(n, r2, z, part);
        res = sqrt(dot64(n, r, r, part));
        ++it;
        beta = rho_new / rho;
        rho = rho_new;
        if (!isfinite(res)) { status = ST_BREAKDOWN; break; }
        if (!(res > tol)) break;
        if (it >= cfg->max_iter) { status = ST_NOT_CONVERGED; break; }
        if (!(rho != 0.0 && isfinite(rho))) { status = ST_BREAKDOWN; break; }
    }
    st->init_res_norm = res0;
    st->final_res_norm = res;
    st->num_iter = it;
    st->num_outer = 0;
    st->status = status;
    free(dinv); free(r); free(r2); free(z); free(z2); free(p); free(p2); free(q); free(q2); free(part); free(tpos);
    return status;
}

/* ---------------------------------------------------------------- ILU(0)
 * DILU in an fvSolution maps to Ginkgo's preconditioner::Ilu with a
 * factorization::ParIlu (src/compatibility/fvSolution.cpp:56-63).  ParIlu's
 * fixed-point sweeps approach the ILU(0) factors of A's pattern; the library
 * (ilu.cu) forms those factors exactly, row after row in the IKJ order
 * restated here: for every entry (i,k) left of the diagonal, k ascending,
 * l_ik = a_ik / u_kk, then a_ij -= l_ik u_kj for every j > k present in both
 * rows i and k, j ascending (as fma(-l_ik, u_kj, a_ij)).  On a hex mesh (no
 * three cells pairwise adjacent) only the diagonal changes: OpenFOAM's DILU.
 * z = U^-1 L^-1 r: y_i = r_i - sum_k l_ik y_k (k ascending, fma chain), then
 * z_i = (y_i - sum_j u_ij z_j) / u_ii (j ascending). */
void or_ilu_factor(const or_csr* A, const double* val, double* lu) {
    const int32_t* ro = A->row_offs;
    memcpy(lu, val, sizeof(double) * (size_t)A->nnz);
    for (int32_t i = 0; i < A->n; ++i) {
        const int32_t d = ro[i] + A->diag_off[i], end = ro[i + 1];
        for (int32_t e = ro[i]; e < d; ++e) {
            const int32_t k = A->col[e];
            const int32_t dk = ro[k] + A->diag_off[k];
            const double l = lu[e] / lu[dk];
            lu[e] = l;
            int32_t f = e + 1, g = dk + 1;
            while (f < end && g < ro[k + 1]) {
                if (A->col[f] < A->col[g]) ++f;
                else if (A->col[f] > A->col[g]) ++g;
                else {
                    lu[f] = fma(-l, lu[g], lu[f]);
                    ++f;
                    ++g;
                }
            }
        }
    }
}

void or_ilu_apply(const or_csr* A, const double* lu, const double* r, double* y, double* z) {
    const int32_t* ro = A->row_offs;
    for (int32_t i = 0; i < A->n; ++i) {
        double s = r[i];
        for (int32_t e = ro[i]; e < ro[i] + A->diag_off[i]; ++e) s = fma(-lu[e], y[A->col[e]], s);
        y[i] = s;
    }
    for (int32_t i = A->n - 1; i >= 0; --i) {
        const int32_t d = ro[i] + A->diag_off[i];
        double s = y[i];
        for (int32_t e = d + 1; e < ro[i + 1]; ++e) s = fma(-lu[e], z[A->col[e]], s);
        z[i] = s / lu[d];
    }
}

/* CG with the ILU(0) preconditioner (ilu.cu), FP64, every dot by the GPU's tree:
 *   r = b - A x, |r|; z = M^-1 r; p = z; rz = (r, z)
 *   loop: q = A p; alpha = rz / (p, q); x += alpha p; r -= alpha q; |r|, stop tests;
 *         z = M^-1 r; rz' = (r, z); beta = rz' / rz; p = z + beta p */
static int32_t solve_cg_ilu(const or_csr* A, const double* val, const double* b, double* x,
                            const or_solver_cfg* cfg, or_solver_stats* st, const double* lu) {
    const int32_t n = A->n, nb = nblocks_of(n);
    double *r = zalloc(n), *p = zalloc(n), *q = zalloc(n), *z = zalloc(n), *fw = zalloc(n), *part = zalloc(nb);
    spmv_all(A, val, x, q);
    for (int32_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
    double res0 = sqrt(dot64(n, r, r, part)), res = res0;
    double tol = cfg->rel_tol * tol_base(A, b, cfg, res0);
    if (cfg->abs_tol > tol) tol = cfg->abs_tol;
    int32_t it = 0, status = ST_OK;
    int done = !(res > tol) || res == 0.0;
    if (!isfinite(res)) { done = 1; status = ST_BREAKDOWN; }
    else if (!done && cfg->max_iter <= 0) { done = 1; status = ST_NOT_CONVERGED; }
    double rz = 0.0;
    if (!done) {
        or_ilu_apply(A, lu, r, fw, z);
        memcpy(p, z, sizeof(double) * (size_t)n);
        rz = dot64(n, r, z, part);
    }
    while (!done) {
        spmv_all(A, val, p, q);
        const double pq = dot64(n, p, q, part);
        const double alpha = rz / pq;
        if (pq == 0.0 || !isfinite(alpha)) { status = ST_BREAKDOWN; break; }
        for (int32_t i = 0; i < n; ++i) {
            x[i] = fma(alpha, p[i], x[i]);
            r[i] = fma(-alpha, q[i], r[i]);
        }
        res = sqrt(dot64(n, r, r, part));
        ++it;
        if (!isfinite(res)) { status = ST_BREAKDOWN; break; }
        if (!(res > tol)) break;
        if (it >= cfg->max_iter) { status = ST_NOT_CONVERGED; break; }
        or_ilu_apply(A, lu, r, fw, z);
        const double rzn = dot64(n, r, z, part);
        const double beta = rzn / rz;
        rz = rzn;
        for (int32_t i = 0; i < n; ++i) p[i] = fma(beta, p[i], z[i]);
    }
    st->init_res_norm = res0;
    st->final_res_norm = res;
    st->num_iter = it;
    st->num_outer = 0;
    st->status = status;
    free(r); free(p); free(q); free(z); free(fw); free(part);
    return status;
}

int32_t or_solve(const or_csr* A, const double* values, const double* rhs, double* x,
                 const or_solver_cfg* cfg, or_solver_stats* stats) {
    g_red_rpt = red_rows_per_thread(A->n);
    if (cfg->preconditioner == 2) {
        if (cfg->precision != 0 || (cfg->method != 0 && cfg->method != 1)) {
            stats->status = ST_UNSUPPORTED;
            return ST_UNSUPPORTED;
        }
        double* lu = zalloc((size_t)A->nnz);
        or_ilu_factor(A, values, lu);
        const int32_t st = cfg->method == 1 ? solve_bicgstab(A, values, rhs, x, cfg, stats, lu)
                                            : solve_cg_ilu(A, values, rhs, x, cfg, stats, lu);
        free(lu);
        return st;
    }
    if (cfg->method == 2) {
        if (cfg->precision != 0) {
            stats->status = ST_UNSUPPORTED;
            return ST_UNSUPPORTED;
        }
        return solve_bicg(A, values, rhs, x, cfg, stats);
    }
    if (cfg->method == 1) {
        if (cfg->precision == 1) return solve_mixed_bicgstab(A, values, rhs, x, cfg, stats);
        return solve_bicgstab(A, values, rhs, x, cfg, stats, NULL);
    }
    if (cfg->precision == 1) return solve_mixed(A, values, rhs, x, cfg, stats);
    return solve_fp64(A, values, rhs, x, cfg, stats);
}

/* ------------------------------------------------------------------ PISO */
/* computeRAUandHByA (pressureVelocityCoupling.cpp:65-128), Serial order */
void or_rau_hbya(const or_mesh* m, const or_csr* A, const double* val, const double* rhs,
                 const double* U, double* rAU, double* H) {
    for (int32_t c = 0; c < m->n; ++c) rAU[c] = m->V[c] / val[A->row_offs[c] + A->diag_off[c]];
    memset(H, 0, sizeof(double) * 3 * (size_t)m->n);
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        double lower = val[A->row_offs[N] + A->nei_off[f]];
        double upper = val[A->row_offs[P] + A->own_off[f]];
        for (int32_t k = 0; k < 3; ++k) {
            H[3 * N + k] -= lower * U[3 * P + k];
            H[3 * P + k] -= upper * U[3 * N + k];
        }
    }
    for (int32_t c = 0; c < m->n; ++c) {
        double sc = rAU[c] / m->V[c];
        for (int32_t k = 0; k < 3; ++k) {
            H[3 * c + k] += rhs[3 * c + k];
            H[3 * c + k] *= sc;
        }
    }
}

void or_constrain_hbya(const or_mesh* m, const int32_t* assignable, const double* U_b,
                       double* H_b) {
    for (int32_t p = 0; p < m->npatch; ++p)
        if (!assignable[p])
            for (int32_t b = m->patch_offs[p]; b < m->patch_offs[p + 1]; ++b)
                for (int32_t k = 0; k < 3; ++k) H_b[3 * b + k] = U_b[3 * b + k];
}

/* flux (pressureVelocityCoupling.cpp:215-267) */
void or_flux_vec(const or_mesh* m, const double* U, const double* U_b, double* out) {
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        double t[3];
        for (int32_t k = 0; k < 3; ++k) t[k] = m->w[f] * (U[3 * P + k] - U[3 * N + k]) + U[3 * N + k];
        out[f] = m->Sf[3 * f] * t[0] + m->Sf[3 * f + 1] * t[1] + m->Sf[3 * f + 2] * t[2];
    }
    for (int32_t b = 0; b < m->nbf; ++b)
        out[m->nif + b] = m->bSf[3 * b] * U_b[3 * b] + m->bSf[3 * b + 1] * U_b[3 * b + 1] +
                          m->bSf[3 * b + 2] * U_b[3 * b + 2];
}

/* fvc::interpolate(rAU)*fvc::ddtCorr(U, phi), Euler (OpenFOAM's
 * EulerDdtScheme::fvcDdtPhiCorr with ddtCorrCoeff for ddtPhiCoeff < 0; the
 * reference's PISO leaves it as a TODO, neoIcoFoam.cpp:127-130):
 * d = phi_old - Sf.U_old_f, c = 1 - min(|d|/(|phi_old| + 1e-15), 1),
 * out += rAUf*((c/dt)*d); c = 0 on fixed-value U patches. */
void or_ddt_corr(const or_mesh* m, const int32_t* U_patch_type, const double* U, const double* U_b,
                 const double* phi_old, const double* rAUf, double dt, double* out) {
    const double rdt = 1.0 / dt;
    const int32_t nf = m->nif + m->nbf;
    double* fU = zalloc((size_t)nf);
    or_flux_vec(m, U, U_b, fU);
    for (int32_t f = 0; f < nf; ++f) {
        if (f >= m->nif && face_bc(m, U_patch_type, f - m->nif) == BC_FIXED_VALUE) continue;
        double d = phi_old[f] - fU[f];
        double c = 1.0 - fmin(fabs(d) / (fabs(phi_old[f]) + 1e-15), 1.0);
        out[f] += rAUf[f] * ((c * rdt) * d);
    }
    free(fU);
}

/* constrainPressure (neoIcoFoam.cpp:135-137 TODO): on fixedFluxPressure patches
 * p_ref_b = (phiHbyA_b - Sf_b.U_b) / (|Sf_b|*rAUf_b) */
void or_constrain_pressure(const or_mesh* m, const int32_t* patch_fixed_flux, const double* phiHbyA,
                           const double* U_b, const double* rAUf, double* p_ref) {
    for (int32_t b = 0; b < m->nbf; ++b) {
        if (!face_bc(m, patch_fixed_flux, b)) continue;
        double fU = m->bSf[3 * b] * U_b[3 * b] + m->bSf[3 * b + 1] * U_b[3 * b + 1] + m->bSf[3 * b + 2] * U_b[3 * b + 2];
        p_ref[b] = (phiHbyA[m->nif + b] - fU) / (m->bmagSf[b] * rAUf[m->nif + b]);
    }
}

/* updateFaceVelocity (pressureVelocityCoupling.cpp:131-197) */
void or_face_update(const or_mesh* m, const or_csr* A, const double* val, const double* bmat,
                    const double* brhs, const double* phiHbyA, const double* p, double* phi) {
    for (int32_t f = 0; f < m->nif; ++f) {
        int32_t P = m->own[f], N = m->nei[f];
        double upper = val[A->row_offs[N] + A->nei_off[f]];
        double lower = val[A->row_offs[P] + A->own_off[f]];
        phi[f] = phiHbyA[f] - (upper * p[N] - lower * p[P]);
    }
    for (int32_t b = 0; b < m->nbf; ++b) {
        double bflux = brhs[b] - bmat[b] * p[m->bcells[b]];
        phi[m->nif + b] = phiHbyA[m->nif + b] - bflux;
    }
}

/* updateVelocity (pressureVelocityCoupling.cpp:199-213) */
void or_velocity_update(const or_mesh* m, const double* H, const double* rAU, const double* p,
                        const double* p_b, double* U) {
    double* g = zalloc((size_t)3 * m->n);
    or_grad(m, p, p_b, 1.0, g);
    for (int32_t c = 0; c < m->n; ++c)
        for (int32_t k = 0; k < 3; ++k) U[3 * c + k] = H[3 * c + k] - rAU[c] * g[3 * c + k];
    free(g);
}
