// Implicit assembly of a dsl::Expression into the linear system, plus the
// small LinearSystem utilities FoamAdapter's PDESolver uses (SetReference,
// diag, applyOperator).  Reference: include/FoamAdapter/datastructures/
// expression.hpp:69-230; term semantics in fvgb.h.
//
// One thread owns one matrix row.  Pass 1 accumulates the diagonal, the rhs and
// the boundary coefficients of the row term by term, walking the row's faces in
// ascending face order (the order in which the reference's face loops scatter
// into a cell).  Pass 2 fills each off-diagonal slot: it corresponds to exactly
// one face, so its value is the term-ordered sum of that face's coefficients.
// Compiled with -fmad=false.
#include "internal.cuh"

namespace {

constexpr int kThreads = 256;

struct TermDev {
    int32_t kind, scheme;
    double coeff;
    const double* cell;
    const double* face;
};

struct TermPack {
    int32_t n;
    TermDev t[FVGB_MAX_TERMS];
};

template <int NC>
__global__ void __launch_bounds__(kThreads)
    k_assemble(MeshView m, TermPack tp, PatchTable pt, double dtInv,
               const double* __restrict__ ref, const double* __restrict__ psi_b,
               double* __restrict__ values, double* __restrict__ rhs, double* __restrict__ bmat,
               double* __restrict__ brhs, int rhs_only) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    const int slice = c >> 5, lane = c & 31;
    const int gbase = __ldg(&m.g_ptr[slice]);
    const int gw = (__ldg(&m.g_ptr[slice + 1]) - gbase) >> 5;
    const double Vc = __ldg(&m.V[c]);

    // ---- pass 1: diagonal, rhs, boundary coefficients
    double diag = 0.0, r[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) r[k] = 0.0;
    for (int j = gw - 1; j >= 0; --j) {  // zero this row's boundary coefficients
        const int code = __ldg(&m.g_code[gbase + j * 32 + lane]);
        if (code == FVGB_PAD) continue;
        if (code < m.nif) break;
        const int b = code - m.nif;
        bmat[b] = 0.0;
#pragma unroll
        for (int k = 0; k < NC; ++k) brhs[b * NC + k] = 0.0;
    }
    for (int t = 0; t < tp.n; ++t) {
        const TermDev T = tp.t[t];
        const double cf = T.coeff;
        if (T.kind == FVGB_TERM_DDT) {
            const double cc = cf * Vc * dtInv;
            diag = diag + cc;
#pragma unroll
            for (int k = 0; k < NC; ++k) r[k] = r[k] + cc * __ldg(&T.cell[c * NC + k]);
        } else if (T.kind == FVGB_TERM_SOURCE) {
            diag = diag + (T.cell ? cf * __ldg(&T.cell[c]) : cf) * Vc;
        } else if (T.kind == FVGB_TERM_EXPLICIT) {
#pragma unroll
            for (int k = 0; k < NC; ++k) r[k] = r[k] - cf * __ldg(&T.cell[c * NC + k]);
        } else if (T.kind == FVGB_TERM_DIV_EXPLICIT) {
            // sum of +-F*psi_f, psi_f interpolated from the term's field, faces ascending
            double e[NC];
#pragma unroll
            for (int k = 0; k < NC; ++k) e[k] = 0.0;
            for (int j = 0; j < gw; ++j) {
                const int pos = gbase + j * 32 + lane;
                const int code = __ldg(&m.g_code[pos]);
                if (code == FVGB_PAD) break;
                const double F = __ldg(&T.face[code >= 0 ? code : -code - 1]);
                if (code >= m.nif) {
                    const int b = code - m.nif;
#pragma unroll
                    for (int k = 0; k < NC; ++k) e[k] = e[k] + F * __ldg(&psi_b[b * NC + k]);
                    continue;
                }
                const bool isOwner = code >= 0;
                const int o = __ldg(&m.g_other[pos]);
                const double wf = T.scheme == FVGB_SCHEME_LINEAR ? __ldg(&m.w[isOwner ? code : -code - 1]) : 0.0;
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    const double Tc = __ldg(&T.cell[c * NC + k]), To = __ldg(&T.cell[o * NC + k]);
                    const double Town = isOwner ? Tc : To, Tnei = isOwner ? To : Tc;
                    const double tf = T.scheme == FVGB_SCHEME_UPWIND ? (F >= 0.0 ? Town : Tnei)
                                                                      : wf * (Town - Tnei) + Tnei;
                    const double fl = F * tf;
                    e[k] = isOwner ? e[k] + fl : e[k] - fl;
                }
            }
#pragma unroll
            for (int k = 0; k < NC; ++k) r[k] = r[k] - cf * e[k];
        } else if (T.kind == FVGB_TERM_DIV_FLUX) {
            double dv = 0.0;  // sum of +-F over the row's faces, ascending face order
            for (int j = 0; j < gw; ++j) {
                const int code = __ldg(&m.g_code[gbase + j * 32 + lane]);
                if (code == FVGB_PAD) break;
                if (code >= m.nif || code >= 0) dv = dv + __ldg(&T.face[code]);
                else dv = dv - __ldg(&T.face[-code - 1]);
            }
#pragma unroll
            for (int k = 0; k < NC; ++k) r[k] = r[k] - cf * dv;
        } else if (T.kind == FVGB_TERM_LAPLACIAN || T.kind == FVGB_TERM_DIV) {
            const bool lap = T.kind == FVGB_TERM_LAPLACIAN;
            for (int j = 0; j < gw; ++j) {
                const int code = __ldg(&m.g_code[gbase + j * 32 + lane]);
                if (code == FVGB_PAD) break;
                if (code >= m.nif) {
                    const int b = code - m.nif;
                    const int bt = pt.type[__ldg(&m.bpatch[b])];
                    const double fb = __ldg(&T.face[code]);
                    double mm;
                    if (lap) {
                        if (bt == FVGB_BC_FIXED_GRADIENT) {
                            mm = 0.0;
                            const double q = cf * (fb * __ldg(&m.bmagSf[b]));
#pragma unroll
                            for (int k = 0; k < NC; ++k) {
                                const double rr = q * __ldg(&ref[b * NC + k]);
                                r[k] = r[k] - rr;
                                brhs[b * NC + k] = brhs[b * NC + k] + rr;
                            }
                        } else {
                            mm = cf * (fb * __ldg(&m.bgeo[b]));
#pragma unroll
                            for (int k = 0; k < NC; ++k) {
                                const double rr = mm * __ldg(&psi_b[b * NC + k]);
                                r[k] = r[k] - rr;
                                brhs[b * NC + k] = brhs[b * NC + k] + rr;
                            }
                        }
                    } else {
                        const double cF = cf * fb;
                        if (bt == FVGB_BC_FIXED_GRADIENT) {
                            mm = -cF;
#pragma unroll
                            for (int k = 0; k < NC; ++k) {
                                const double rr = cF * (__ldg(&ref[b * NC + k]) / __ldg(&m.bdelta[b]));
                                r[k] = r[k] - rr;
                                brhs[b * NC + k] = brhs[b * NC + k] + rr;
                            }
                        } else {
                            mm = 0.0;
#pragma unroll
                            for (int k = 0; k < NC; ++k) {
                                const double rr = cF * __ldg(&psi_b[b * NC + k]);
                                r[k] = r[k] - rr;
                                brhs[b * NC + k] = brhs[b * NC + k] + rr;
                            }
                        }
                    }
                    diag = diag - mm;
                    bmat[b] = bmat[b] + mm;
                    continue;
                }
                if (rhs_only) continue;  // internal faces only feed the matrix
                const bool isOwner = code >= 0;
                const int f = isOwner ? code : -code - 1;
                if (lap) {
                    diag = diag - cf * (__ldg(&T.face[f]) * __ldg(&m.geo[f]));
                } else {
                    const double F = __ldg(&T.face[f]);
                    const double cF = cf * F;
                    if (T.scheme == FVGB_SCHEME_UPWIND) {
                        if (isOwner) {
                            if (F >= 0.0) diag = diag + cF;
                        } else {
                            if (!(F >= 0.0)) diag = diag - cF;
                        }
                    } else {
                        const double w = __ldg(&m.w[f]);
                        if (isOwner) diag = diag + cF * w;
                        else diag = diag - cF * (1.0 - w);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NC; ++k) rhs[c * NC + k] = r[k];
    if (rhs_only) return;

    // ---- pass 2: the row's slots
    const int mbase = __ldg(&m.m_ptr[slice]);
    const int mw = (__ldg(&m.m_ptr[slice + 1]) - mbase) >> 5;
    for (int j = 0; j < mw; ++j) {
        const int pos = mbase + j * 32 + lane;
        const int code = __ldg(&m.m_code[pos]);
        if (code == FVGB_PAD) break;
        if (code == -1) {
            values[pos] = diag;
            continue;
        }
        const bool isOwner = code >= 0;
        const int f = isOwner ? code : -code - 2;
        double v = 0.0;
        for (int t = 0; t < tp.n; ++t) {
            const TermDev T = tp.t[t];
            if (T.kind == FVGB_TERM_LAPLACIAN) {
                v = v + T.coeff * (__ldg(&T.face[f]) * __ldg(&m.geo[f]));
            } else if (T.kind == FVGB_TERM_DIV) {
                const double F = __ldg(&T.face[f]);
                const double cF = T.coeff * F;
                if (T.scheme == FVGB_SCHEME_UPWIND) {
                    if (isOwner) {
                        if (!(F >= 0.0)) v = v + cF;
                    } else {
                        if (F >= 0.0) v = v - cF;
                    }
                } else {
                    const double w = __ldg(&m.w[f]);
                    if (isOwner) v = v + cF * (1.0 - w);
                    else v = v - cF * w;
                }
            }
        }
        values[pos] = v;
    }
}

__global__ void k_set_reference(MeshView m, int r, double v, double* values, double* rhs) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int d = m.diag_pos[r];
        const double dv = values[d];
        rhs[r] = rhs[r] + dv * v;
        values[d] = values[d] + dv;
    }
}

template <int NC>
__global__ void __launch_bounds__(kThreads)
    k_apply(MeshView m, const double* __restrict__ values, const double* __restrict__ rhs,
            const double* __restrict__ x, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n) return;
    const int slice = c >> 5, lane = c & 31;
    const int base = __ldg(&m.m_ptr[slice]);
    const int w = (__ldg(&m.m_ptr[slice + 1]) - base) >> 5;
    double s[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) s[k] = 0.0;
    for (int j = 0; j < w; ++j) {
        const int pos = base + j * 32 + lane;
        const double a = __ldg(&values[pos]);
        const int col = __ldg(&m.m_col[pos]);
#pragma unroll
        for (int k = 0; k < NC; ++k) s[k] = fma(a, __ldg(&x[col * NC + k]), s[k]);
    }
#pragma unroll
    for (int k = 0; k < NC; ++k) out[c * NC + k] = s[k] - __ldg(&rhs[c * NC + k]);
}

__global__ void k_diag(MeshView m, const double* __restrict__ values, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < m.n) out[c] = values[m.diag_pos[c]];
}

__global__ void k_gather_csr(int nnz, const int32_t* __restrict__ csr_pos,
                             const double* __restrict__ values, double* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nnz) out[j] = values[csr_pos[j]];
}

}  // namespace

extern "C" fvgb_status fvgb_ls_create(const fvgb_mesh* mesh, int32_t ncomp, fvgb_ls** out) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(mesh && out, "fvgb_ls_create: null argument");
    FVGB_CHECK_ARG(ncomp == 1 || ncomp == 3, "fvgb_ls_create: ncomp must be 1 or 3");
    *out = nullptr;
    fvgb_ls* ls = new fvgb_ls();
    ls->mesh = mesh;
    ls->ncomp = ncomp;
    const int64_t n = mesh->v.n, nbf = mesh->v.nbf;
    ls->pooled = devmem_pooled_now();
    cudaError_t e = devmem_alloc((void**)&ls->values, sizeof(double) * (size_t)mesh->m_len, ls->pooled);
    if (e == cudaSuccess) e = devmem_alloc((void**)&ls->rhs, sizeof(double) * (size_t)(n * ncomp), ls->pooled);
    if (e == cudaSuccess) e = devmem_alloc((void**)&ls->bmat, sizeof(double) * (size_t)(nbf > 0 ? nbf : 1), ls->pooled);
    if (e == cudaSuccess)
        e = devmem_alloc((void**)&ls->brhs, sizeof(double) * (size_t)(nbf > 0 ? nbf * ncomp : 1), ls->pooled);
    if (e == cudaSuccess) e = cudaMemset(ls->values, 0, sizeof(double) * (size_t)mesh->m_len);
    if (e == cudaSuccess) e = cudaMemset(ls->rhs, 0, sizeof(double) * (size_t)(n * ncomp));
    if (e == cudaSuccess) e = cudaMemset(ls->bmat, 0, sizeof(double) * (size_t)(nbf > 0 ? nbf : 1));
    if (e == cudaSuccess) e = cudaMemset(ls->brhs, 0, sizeof(double) * (size_t)(nbf > 0 ? nbf * ncomp : 1));
    if (e == cudaSuccess) e = settle_creation();
    if (e != cudaSuccess) {
        fvgb_ls_destroy(ls);
        return cuda_fail(e, "fvgb_ls_create");
    }
    *out = ls;
    return FVGB_OK;
}

void fvgb_solver_cache_free(SolverCache* c);  // solver.cu

extern "C" fvgb_status fvgb_ls_destroy(fvgb_ls* ls) {
    if (!ls) return FVGB_OK;
    // work in flight may still read the system: wait for it, unless its memory
    // is pooled (then freed in order on the release stream of the thread's context)
    if (!ls->pooled) cudaDeviceSynchronize();
    if (ls->solver) fvgb_solver_cache_free(ls->solver);
    if (ls->amg) fvgb_amg_free(ls->amg);
    if (ls->ilu) fvgb_ilu_free(ls->ilu);
    devmem_free(ls->values, ls->pooled);
    devmem_free(ls->rhs, ls->pooled);
    devmem_free(ls->bmat, ls->pooled);
    devmem_free(ls->brhs, ls->pooled);
    delete ls;
    return FVGB_OK;
}

namespace {
fvgb_status assemble(fvgb_ls* ls, const fvgb_term* terms, int32_t nterms, double dt, const fvgb_bc* psi_bc,
                     const double* psi_b, fvgb_stream stream, int rhs_only) {
    FVGB_CHECK_ARG(ls && (terms || nterms == 0), "fvgb_assemble: null argument");
    FVGB_CHECK_ARG(nterms >= 0 && nterms <= FVGB_MAX_TERMS, "fvgb_assemble: 0..8 terms");
    const fvgb_mesh* m = ls->mesh;
    TermPack tp{};
    tp.n = nterms;
    bool needs_b = false, needs_dt = false;
    for (int i = 0; i < nterms; ++i) {
        const fvgb_term& t = terms[i];
        FVGB_CHECK_ARG(t.kind >= FVGB_TERM_DDT && t.kind <= FVGB_TERM_DIV_EXPLICIT, "fvgb_assemble: unknown term kind");
        if (t.kind == FVGB_TERM_DIV_EXPLICIT) {
            FVGB_CHECK_ARG(t.cell && t.face, "fvgb_assemble: explicit convection needs the field and the flux");
            FVGB_CHECK_ARG(t.scheme == FVGB_SCHEME_LINEAR || t.scheme == FVGB_SCHEME_UPWIND,
                           "fvgb_assemble: unknown div scheme");
            needs_b = true;
        }
        if (t.kind == FVGB_TERM_DDT) {
            FVGB_CHECK_ARG(t.cell, "fvgb_assemble: ddt needs the old-time field");
            needs_dt = true;
        }
        if (t.kind == FVGB_TERM_EXPLICIT) FVGB_CHECK_ARG(t.cell, "fvgb_assemble: explicit term needs its values");
        if (t.kind == FVGB_TERM_DIV_FLUX) FVGB_CHECK_ARG(t.face, "fvgb_assemble: flux divergence needs the flux");
        if (t.kind == FVGB_TERM_LAPLACIAN || t.kind == FVGB_TERM_DIV) {
            FVGB_CHECK_ARG(t.face, "fvgb_assemble: laplacian/div need a surface field");
            needs_b = true;
        }
        if (t.kind == FVGB_TERM_LAPLACIAN) {
            FVGB_CHECK_ARG(t.scheme == 0 || t.scheme == FVGB_SCHEME_CORRECTED, "fvgb_assemble: unknown laplacian scheme");
            if (t.scheme == FVGB_SCHEME_CORRECTED) {
                FVGB_CHECK_ARG(t.cell, "fvgb_assemble: a corrected laplacian needs the current field");
                FVGB_CHECK_ARG(m->v.corr || m->v.nif == 0,
                               "fvgb_assemble: corrected laplacian on a mesh created without cell centres");
            }
        }
        if (t.kind == FVGB_TERM_DIV)
            FVGB_CHECK_ARG(t.scheme == FVGB_SCHEME_LINEAR || t.scheme == FVGB_SCHEME_UPWIND,
                           "fvgb_assemble: unknown div scheme");
        tp.t[i].kind = t.kind;
        tp.t[i].scheme = t.scheme;
        tp.t[i].coeff = t.coeff;
        tp.t[i].cell = t.cell;
        tp.t[i].face = t.face;
    }
    if (needs_dt) FVGB_CHECK_ARG(dt > 0, "fvgb_assemble: dt must be positive");
    PatchTable pt;
    FVGB_CHECK_ARG(make_patch_table(m, psi_bc ? psi_bc->patch_type : nullptr, &pt),
                   "fvgb_assemble: bad patch types");
    const double* ref = psi_bc ? psi_bc->ref : nullptr;
    if (needs_b && m->v.nbf > 0) {
        FVGB_CHECK_ARG(psi_b, "fvgb_assemble: boundary values of psi are null");
        for (int p = 0; p < pt.n; ++p)
            FVGB_CHECK_ARG(pt.type[p] != FVGB_BC_FIXED_GRADIENT || ref,
                           "fvgb_assemble: fixedGradient patch without ref");
    }
    const double dtInv = needs_dt ? 1.0 / dt : 0.0;
    cudaStream_t s = (cudaStream_t)stream;
    if (ls->ncomp == 1)
        k_assemble<1><<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, tp, pt, dtInv, ref, psi_b,
                                                                     ls->values, ls->rhs, ls->bmat, ls->brhs,
                                                                     rhs_only);
    else
        k_assemble<3><<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, tp, pt, dtInv, ref, psi_b,
                                                                     ls->values, ls->rhs, ls->bmat, ls->brhs,
                                                                     rhs_only);
    FVGB_LAUNCH_CHECK("fvgb_assemble");
    // explicit non-orthogonal corrections of corrected laplacians, after all terms, in term order
    for (int i = 0; i < nterms; ++i) {
        const fvgb_term& t = terms[i];
        if (t.kind != FVGB_TERM_LAPLACIAN || t.scheme != FVGB_SCHEME_CORRECTED || m->v.nif == 0) continue;
        const fvgb_status st = nonorth_rhs(m, ls->ncomp, t.face, t.cell, psi_b, -t.coeff, ls->rhs, s);
        if (st != FVGB_OK) return st;
    }
    if (!rhs_only) ++ls->version;
    return FVGB_OK;
}
}  // namespace

extern "C" fvgb_status fvgb_assemble(fvgb_ls* ls, const fvgb_term* terms, int32_t nterms,
                                     double dt, const fvgb_bc* psi_bc, const double* psi_b,
                                     fvgb_stream stream) {
    return assemble(ls, terms, nterms, dt, psi_bc, psi_b, stream, 0);
}

// The same terms with the matrix kept: only rhs and the boundary coefficients
// are recomputed (their values are what fvgb_assemble would write; the matrix
// values it would write are those already there when the implicit terms, dt,
// mesh and boundary types are unchanged).
extern "C" fvgb_status fvgb_assemble_rhs(fvgb_ls* ls, const fvgb_term* terms, int32_t nterms,
                                         double dt, const fvgb_bc* psi_bc, const double* psi_b,
                                         fvgb_stream stream) {
    return assemble(ls, terms, nterms, dt, psi_bc, psi_b, stream, 1);
}

extern "C" fvgb_status fvgb_set_reference(fvgb_ls* ls, int32_t ref_cell, double ref_value,
                                          fvgb_stream stream) {
    FVGB_CHECK_ARG(ls, "fvgb_set_reference: null system");
    FVGB_CHECK_ARG(ls->ncomp == 1, "fvgb_set_reference: scalar systems only");
    FVGB_CHECK_ARG(ref_cell >= 0 && ref_cell < ls->mesh->v.n, "fvgb_set_reference: cell out of range");
    k_set_reference<<<1, 32, 0, (cudaStream_t)stream>>>(ls->mesh->v, ref_cell, ref_value, ls->values, ls->rhs);
    FVGB_LAUNCH_CHECK("fvgb_set_reference");
    ++ls->version;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_apply_operator(const fvgb_ls* ls, const double* x, double* out,
                                           fvgb_stream stream) {
    FVGB_CHECK_ARG(ls && x && out, "fvgb_apply_operator: null argument");
    const fvgb_mesh* m = ls->mesh;
    cudaStream_t s = (cudaStream_t)stream;
    if (ls->ncomp == 1)
        k_apply<1><<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, ls->values, ls->rhs, x, out);
    else
        k_apply<3><<<grid_for(m->v.n, kThreads), kThreads, 0, s>>>(m->v, ls->values, ls->rhs, x, out);
    FVGB_LAUNCH_CHECK("fvgb_apply_operator");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_ls_diag(const fvgb_ls* ls, double* out, fvgb_stream stream) {
    FVGB_CHECK_ARG(ls && out, "fvgb_ls_diag: null argument");
    k_diag<<<grid_for(ls->mesh->v.n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(ls->mesh->v, ls->values, out);
    FVGB_LAUNCH_CHECK("fvgb_ls_diag");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_ls_export(const fvgb_ls* ls, double* values, double* rhs,
                                      double* bmat, double* brhs, fvgb_stream stream) {
    FVGB_CHECK_ARG(ls, "fvgb_ls_export: null system");
    const fvgb_mesh* m = ls->mesh;
    cudaStream_t s = (cudaStream_t)stream;
    if (values && !m->csr_pos)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_ls_export: this mesh keeps no CSR map (built on the device)");
    if (values) {
        k_gather_csr<<<grid_for(m->nnz, kThreads), kThreads, 0, s>>>(m->nnz, m->csr_pos, ls->values, values);
        FVGB_LAUNCH_CHECK("fvgb_ls_export");
    }
    const size_t n = (size_t)m->v.n, nbf = (size_t)m->v.nbf, nc = (size_t)ls->ncomp;
    if (rhs) FVGB_CUDA_TRY(cudaMemcpyAsync(rhs, ls->rhs, sizeof(double) * n * nc, cudaMemcpyDeviceToDevice, s));
    if (bmat && nbf) FVGB_CUDA_TRY(cudaMemcpyAsync(bmat, ls->bmat, sizeof(double) * nbf, cudaMemcpyDeviceToDevice, s));
    if (brhs && nbf)
        FVGB_CUDA_TRY(cudaMemcpyAsync(brhs, ls->brhs, sizeof(double) * nbf * nc, cudaMemcpyDeviceToDevice, s));
    return FVGB_OK;
}
