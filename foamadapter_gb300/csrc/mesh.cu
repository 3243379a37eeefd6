// Mesh upload and indexing: validates the NeoN-shaped array set, builds the
// per-cell gather lists and the matrix pattern (NeoN la::SparsityPattern
// semantics, reference test/test_sparsityPattern.cpp:36-62) in the sliced-ELL
// layouts described in internal.cuh, and uploads everything once.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.cuh"

namespace {

// Sliced-ELL packing of per-row lists: rows of `offs` (CSR offsets) laid out
// in 32-row slices, column-major inside a slice, padded with `pad`.
struct SellPack {
    std::vector<int32_t> ptr;  // [nslices+1]
    int64_t len = 0;
};

SellPack sell_shape(const std::vector<int32_t>& offs, int32_t n) {
    SellPack s;
    int32_t ns = (n + kSlice - 1) / kSlice;
    s.ptr.resize(ns + 1);
    int64_t acc = 0;
    for (int32_t sl = 0; sl < ns; ++sl) {
        s.ptr[sl] = (int32_t)acc;
        int32_t wmax = 0;
        for (int32_t r = sl * kSlice; r < std::min(n, (sl + 1) * kSlice); ++r)
            wmax = std::max(wmax, offs[r + 1] - offs[r]);
        acc += (int64_t)wmax * kSlice;
    }
    s.ptr[ns] = (int32_t)acc;
    s.len = acc;
    return s;
}

inline int64_t sell_pos(const SellPack& s, int32_t row, int32_t k) {
    return (int64_t)s.ptr[row / kSlice] + (int64_t)k * kSlice + (row % kSlice);
}

__global__ void k_bc_correct(MeshView m, PatchTable pt, int ncomp, const double* __restrict__ ref,
                             const double* __restrict__ internal, double* __restrict__ boundary) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.nbf) return;
    int t = pt.type[m.bpatch[b]];
    int P = m.bcells[b];
    for (int k = 0; k < ncomp; ++k) {
        if (t == FVGB_BC_FIXED_VALUE) boundary[b * ncomp + k] = ref[b * ncomp + k];
        else if (t == FVGB_BC_FIXED_GRADIENT)
            boundary[b * ncomp + k] = internal[P * ncomp + k] + ref[b * ncomp + k] / m.bdelta[b];
    }
}

void free_mesh(fvgb_mesh* m) {
    if (!m) return;
    for (void* p : m->allocs) devmem_free(p, m->pooled);
    delete m;
}

template <class T>
cudaError_t upload(fvgb_mesh* m, T** dst, const T* src, int64_t count) {
    cudaError_t e = mesh_alloc(m, dst, count);
    if (e != cudaSuccess) return e;
    if (count > 0) e = cudaMemcpy(*dst, src, sizeof(T) * (size_t)count, cudaMemcpyHostToDevice);
    return e;
}

template <class T>
void up(fvgb_mesh* m, cudaError_t& e, const T*& dst, const T* src, int64_t count) {
    if (e != cudaSuccess) return;
    T* p = nullptr;
    e = upload<T>(m, &p, src, count);
    dst = p;
}

}  // namespace

extern "C" fvgb_status fvgb_mesh_create(const fvgb_mesh_desc* d, fvgb_mesh** out) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(d && out, "fvgb_mesh_create: null argument");
    *out = nullptr;
    const int32_t n = d->n_cells, nif = d->n_ifaces, nbf = d->n_bfaces, np = d->n_patches;
    FVGB_CHECK_ARG(n > 0 && nif >= 0 && nbf >= 0 && np >= 0, "fvgb_mesh_create: negative size");
    FVGB_CHECK_ARG(np <= FVGB_MAX_PATCHES, "fvgb_mesh_create: more than 256 non-empty patches");
    FVGB_CHECK_ARG((int64_t)n + 2 * (int64_t)nif < INT32_MAX / 2, "fvgb_mesh_create: mesh too large for int32 labels");
    FVGB_CHECK_ARG(d->cell_volumes, "fvgb_mesh_create: cell_volumes is null");
    FVGB_CHECK_ARG(nif == 0 || (d->owner && d->neighbour && d->face_areas && d->mag_face_areas &&
                                d->weights && d->delta_coeffs),
                   "fvgb_mesh_create: internal-face array is null");
    FVGB_CHECK_ARG(nbf == 0 || (d->bface_cells && d->bface_areas && d->bmag_face_areas &&
                                d->bweights && d->bdelta_coeffs),
                   "fvgb_mesh_create: boundary-face array is null");
    FVGB_CHECK_ARG(d->patch_offsets || np == 0, "fvgb_mesh_create: patch_offsets is null");
    for (int32_t c = 0; c < n; ++c)
        FVGB_CHECK_ARG(d->cell_volumes[c] > 0 && std::isfinite(d->cell_volumes[c]),
                       "fvgb_mesh_create: non-positive cell volume");
    for (int32_t f = 0; f < nif; ++f) {
        int32_t o = d->owner[f], nb = d->neighbour[f];
        FVGB_CHECK_ARG(o >= 0 && o < n && nb >= 0 && nb < n && o != nb,
                       "fvgb_mesh_create: owner/neighbour label out of range");
    }
    for (int32_t b = 0; b < nbf; ++b)
        FVGB_CHECK_ARG(d->bface_cells[b] >= 0 && d->bface_cells[b] < n,
                       "fvgb_mesh_create: boundary face cell out of range");
    if (np > 0) {
        FVGB_CHECK_ARG(d->patch_offsets[0] == 0 && d->patch_offsets[np] == nbf,
                       "fvgb_mesh_create: patch offsets must span [0, n_bfaces]");
        for (int32_t p = 0; p < np; ++p)
            FVGB_CHECK_ARG(d->patch_offsets[p + 1] >= d->patch_offsets[p],
                           "fvgb_mesh_create: patch offsets not monotone");
    } else {
        FVGB_CHECK_ARG(nbf == 0, "fvgb_mesh_create: boundary faces without patches");
    }

    fvgb_mesh* m = new fvgb_mesh();
    m->pooled = devmem_pooled_now();
    m->h_patch_offs.assign(d->patch_offsets, d->patch_offsets + np + 1);
    if (np == 0) m->h_patch_offs.assign(1, 0);

    // ---- CSR pattern, rows in column order
    std::vector<int32_t> cnt(n + 1, 0);
    for (int32_t f = 0; f < nif; ++f) {
        cnt[d->owner[f]]++;
        cnt[d->neighbour[f]]++;
    }
    auto& ro = m->h_row_offs;
    ro.assign(n + 1, 0);
    for (int32_t c = 0; c < n; ++c) ro[c + 1] = ro[c] + cnt[c] + 1;
    const int32_t nnz = ro[n];
    m->nnz = nnz;
    std::vector<int32_t> col(nnz), code(nnz), fill(n);
    for (int32_t c = 0; c < n; ++c) {
        col[ro[c]] = c;
        code[ro[c]] = -1;
        fill[c] = 1;
    }
    for (int32_t f = 0; f < nif; ++f) {
        int32_t P = d->owner[f], N = d->neighbour[f];
        col[ro[P] + fill[P]] = N;
        code[ro[P] + fill[P]++] = f;
        col[ro[N] + fill[N]] = P;
        code[ro[N] + fill[N]++] = -f - 2;
    }
    m->h_diag_off.assign(n, 0);
    m->h_own_off.assign(nif, 0);
    m->h_nei_off.assign(nif, 0);
    for (int32_t c = 0; c < n; ++c) {
        int32_t b = ro[c], e = ro[c + 1];
        for (int32_t i = b + 1; i < e; ++i) {
            int32_t cc = col[i], cd = code[i], j = i - 1;
            while (j >= b && col[j] > cc) {
                col[j + 1] = col[j];
                code[j + 1] = code[j];
                --j;
            }
            col[j + 1] = cc;
            code[j + 1] = cd;
        }
        for (int32_t i = b; i < e; ++i) {
            if (i > b && col[i] == col[i - 1]) {
                free_mesh(m);
                return fvgb_fail(FVGB_ERR_INVALID_ARG,
                                 "fvgb_mesh_create: two faces between the same pair of cells");
            }
            if (code[i] == -1) m->h_diag_off[c] = i - b;
            else if (code[i] >= 0) m->h_own_off[code[i]] = i - b;
            else m->h_nei_off[-code[i] - 2] = i - b;
        }
    }
    m->h_col = col;

    // ---- sliced-ELL matrix pattern
    SellPack ms = sell_shape(ro, n);
    m->nslices = (int32_t)ms.ptr.size() - 1;
    m->m_len = ms.len;
    std::vector<int32_t> s_col(ms.len), s_code(ms.len, FVGB_PAD), csr_pos(nnz), diag_pos(n),
        own_pos(nif), nei_pos(nif);
    for (int64_t i = 0; i < ms.len; ++i) s_col[i] = 0;
    for (int32_t sl = 0; sl < m->nslices; ++sl) {
        int32_t w = (ms.ptr[sl + 1] - ms.ptr[sl]) / kSlice;
        for (int32_t l = 0; l < kSlice; ++l) {
            int32_t r = sl * kSlice + l;
            for (int32_t k = 0; k < w; ++k) {
                int64_t pos = (int64_t)ms.ptr[sl] + (int64_t)k * kSlice + l;
                if (r < n && k < ro[r + 1] - ro[r]) {
                    s_col[pos] = col[ro[r] + k];
                    s_code[pos] = code[ro[r] + k];
                    csr_pos[ro[r] + k] = (int32_t)pos;
                } else {
                    s_col[pos] = r < n ? r : 0;
                    s_code[pos] = FVGB_PAD;
                }
            }
        }
    }
    // 16-bit column offsets when every slot's column is within +-32767 of its row
    std::vector<int16_t> s_off(ms.len, 0);
    bool off_fits = true;
    for (int32_t sl = 0; sl < m->nslices && off_fits; ++sl) {
        int32_t w = (ms.ptr[sl + 1] - ms.ptr[sl]) / kSlice;
        for (int32_t l = 0; l < kSlice && off_fits; ++l) {
            const int32_t r = sl * kSlice + l;
            if (r >= n) continue;
            for (int32_t k = 0; k < w; ++k) {
                const int64_t pos = (int64_t)ms.ptr[sl] + (int64_t)k * kSlice + l;
                const int64_t off = (int64_t)s_col[pos] - r;
                if (off < -32767 || off > 32767) {
                    off_fits = false;
                    break;
                }
                s_off[pos] = (int16_t)off;
            }
        }
    }
    for (int32_t c = 0; c < n; ++c) diag_pos[c] = (int32_t)sell_pos(ms, c, m->h_diag_off[c]);
    for (int32_t f = 0; f < nif; ++f) {
        own_pos[f] = (int32_t)sell_pos(ms, d->owner[f], m->h_own_off[f]);
        nei_pos[f] = (int32_t)sell_pos(ms, d->neighbour[f], m->h_nei_off[f]);
    }

    // ---- gather lists: faces of each cell in ascending face order
    std::vector<int32_t> go(n + 1, 0);
    for (int32_t c = 0; c < n; ++c) go[c + 1] = cnt[c];
    for (int32_t b = 0; b < nbf; ++b) go[d->bface_cells[b] + 1]++;
    for (int32_t c = 0; c < n; ++c) go[c + 1] += go[c];
    std::vector<int32_t> gcode(go[n]), gother(go[n]);
    std::fill(fill.begin(), fill.end(), 0);
    for (int32_t f = 0; f < nif; ++f) {
        int32_t P = d->owner[f], N = d->neighbour[f];
        gcode[go[P] + fill[P]] = f;
        gother[go[P] + fill[P]++] = N;
        gcode[go[N] + fill[N]] = -f - 1;
        gother[go[N] + fill[N]++] = P;
    }
    for (int32_t b = 0; b < nbf; ++b) {
        int32_t P = d->bface_cells[b];
        gcode[go[P] + fill[P]] = nif + b;
        gother[go[P] + fill[P]++] = b;
    }
    SellPack gs = sell_shape(go, n);
    m->g_len = gs.len;
    std::vector<int32_t> sg_code(gs.len, FVGB_PAD), sg_other(gs.len, 0);
    for (int32_t c = 0; c < n; ++c)
        for (int32_t k = 0; k < go[c + 1] - go[c]; ++k) {
            int64_t pos = sell_pos(gs, c, k);
            sg_code[pos] = gcode[go[c] + k];
            sg_other[pos] = gother[go[c] + k];
        }

    // ---- derived geometry
    std::vector<double> invV(n), geo(nif), bgeo(nbf);
    for (int32_t c = 0; c < n; ++c) invV[c] = 1.0 / d->cell_volumes[c];
    for (int32_t f = 0; f < nif; ++f) geo[f] = d->mag_face_areas[f] * d->delta_coeffs[f];
    for (int32_t b = 0; b < nbf; ++b) bgeo[b] = d->bmag_face_areas[b] * d->bdelta_coeffs[b];
    // non-orthogonal correction vectors k_f = Sf/|Sf| - d_f*delta_f, d_f = C_N - C_P
    // (OpenFOAM's nonOrthCorrectionVectors), when the cell centres are given
    std::vector<double> corr;
    if (d->cell_centres) {
        corr.resize(3 * (size_t)nif);
        const double* C = d->cell_centres;
        for (int32_t f = 0; f < nif; ++f) {
            const int64_t P = d->owner[f], N = d->neighbour[f];
            for (int i = 0; i < 3; ++i) {
                const double nf = d->face_areas[3 * (int64_t)f + i] / d->mag_face_areas[f];
                const double df = C[3 * N + i] - C[3 * P + i];
                corr[3 * (size_t)f + i] = nf - df * d->delta_coeffs[f];
            }
        }
    }
    std::vector<int32_t> bpatch(nbf);
    for (int32_t p = 0; p < np; ++p)
        for (int32_t b = d->patch_offsets[p]; b < d->patch_offsets[p + 1]; ++b) bpatch[b] = p;

    // ---- upload
    MeshView& v = m->v;
    v.n = n;
    v.nif = nif;
    v.nbf = nbf;
    v.npatch = np;
    cudaError_t e = cudaSuccess;
#define UP(dst, src, cnt_) up(m, e, dst, src, cnt_)
    UP(v.V, d->cell_volumes, n);
    UP(v.invV, invV.data(), n);
    UP(v.own, d->owner, nif);
    UP(v.nei, d->neighbour, nif);
    UP(v.Sf, d->face_areas, 3 * (int64_t)nif);
    UP(v.magSf, d->mag_face_areas, nif);
    UP(v.w, d->weights, nif);
    UP(v.delta, d->delta_coeffs, nif);
    UP(v.geo, geo.data(), nif);
    if (d->cell_centres) UP(v.corr, corr.data(), 3 * (int64_t)nif);
    UP(v.bcells, d->bface_cells, nbf);
    UP(v.bSf, d->bface_areas, 3 * (int64_t)nbf);
    UP(v.bmagSf, d->bmag_face_areas, nbf);
    UP(v.bdelta, d->bdelta_coeffs, nbf);
    UP(v.bgeo, bgeo.data(), nbf);
    UP(v.bpatch, bpatch.data(), nbf);
    UP(v.g_ptr, gs.ptr.data(), (int64_t)gs.ptr.size());
    UP(v.g_code, sg_code.data(), gs.len);
    UP(v.g_other, sg_other.data(), gs.len);
    UP(v.m_ptr, ms.ptr.data(), (int64_t)ms.ptr.size());
    UP(v.m_col, s_col.data(), ms.len);
    if (off_fits) UP(v.m_off, s_off.data(), ms.len);
    UP(v.m_code, s_code.data(), ms.len);
    UP(v.diag_pos, diag_pos.data(), n);
    UP(v.own_pos, own_pos.data(), nif);
    UP(v.nei_pos, nei_pos.data(), nif);
    if (e == cudaSuccess) e = upload<int32_t>(m, &m->csr_pos, csr_pos.data(), nnz);
#undef UP
    if (e == cudaSuccess) e = settle_creation();
    if (e != cudaSuccess) {
        free_mesh(m);
        return cuda_fail(e, "fvgb_mesh_create: upload");
    }
    *out = m;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_mesh_destroy(fvgb_mesh* mesh) {
    if (mesh) {
        // work in flight may still read the mesh: wait for it, unless its memory
        // is pooled (then freed in order on the release stream of the thread's context)
        if (!mesh->pooled) cudaDeviceSynchronize();
        free_mesh(mesh);
    }
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_mesh_sizes(const fvgb_mesh* m, int64_t out[5]) {
    FVGB_CHECK_ARG(m && out, "fvgb_mesh_sizes: null argument");
    out[0] = m->v.n;
    out[1] = m->v.nif;
    out[2] = m->v.nbf;
    out[3] = m->v.npatch;
    out[4] = m->nnz;
    return FVGB_OK;
}

extern "C" int64_t fvgb_mesh_device_bytes(const fvgb_mesh* m) { return m ? m->bytes : 0; }

extern "C" fvgb_status fvgb_mesh_sparsity(const fvgb_mesh* m, int32_t* row_offs, int32_t* col_idxs,
                                          int32_t* diag_offset, int32_t* owner_offset,
                                          int32_t* neighbour_offset) {
    FVGB_CHECK_ARG(m, "fvgb_mesh_sparsity: null mesh");
    if (m->h_row_offs.empty())
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_mesh_sparsity: this mesh keeps no CSR copy (built on the device)");
    auto cp = [](int32_t* dst, const std::vector<int32_t>& src) {
        if (dst && !src.empty()) std::memcpy(dst, src.data(), sizeof(int32_t) * src.size());
    };
    cp(row_offs, m->h_row_offs);
    cp(col_idxs, m->h_col);
    cp(diag_offset, m->h_diag_off);
    cp(owner_offset, m->h_own_off);
    cp(neighbour_offset, m->h_nei_off);
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_bc_correct(const fvgb_mesh* m, int32_t ncomp, const fvgb_bc* bc,
                                       const double* internal, double* boundary,
                                       fvgb_stream stream) {
    FVGB_CHECK_ARG(m && bc && internal && boundary, "fvgb_bc_correct: null argument");
    FVGB_CHECK_ARG(ncomp == 1 || ncomp == 3, "fvgb_bc_correct: ncomp must be 1 or 3");
    PatchTable pt;
    FVGB_CHECK_ARG(make_patch_table(m, bc->patch_type, &pt), "fvgb_bc_correct: bad patch types");
    FVGB_CHECK_ARG(bc->ref || !patch_table_needs_ref(pt), "fvgb_bc_correct: ref is null");
    if (m->v.nbf == 0) return FVGB_OK;
    k_bc_correct<<<grid_for(m->v.nbf, 256), 256, 0, (cudaStream_t)stream>>>(m->v, pt, ncomp, bc->ref,
                                                                          internal, boundary);
    FVGB_LAUNCH_CHECK("fvgb_bc_correct");
    return FVGB_OK;
}
