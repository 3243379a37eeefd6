// Device-side builder of packed uniform hex boxes.
//
// Serving admits many box-shaped cases per second; building their mesh
// arrays on the host (OpenFOAM geometry + sparsity + gather lists) costs about
// a microsecond per cell plus the upload.  For an unjittered box every array
// is a closed-form function of the cell index, so one kernel writes the whole
// device mesh (geometry, gather lists, matrix pattern, slot maps) in place.
//
// Numbering follows the host box builder (and blockMesh): cells i fastest,
// internal faces by owner then +x, +y, +z, boundary faces patch by patch
// (xmin, xmax, ymin, ymax, zmin, zmax), each patch grouped by box.  Boxes start
// at multiples of 32 cells; cells in the gaps are isolated placeholders
// (volume 1, no faces).  Geometry is OpenFOAM's triangle decomposition with
// the host builder's order of operations (meshgen.cpp; compiled here without
// contraction, and double division and square root are correctly rounded on
// the GPU as on the host): face centres and areas from the face's four points
// in face order, cell centres and volumes from pyramids on an estimated centre
// with the faces in face-list order (owned, then neighboured), weights and
// non-orthogonal delta coefficients from the cell centres.  The arrays are
// therefore bit-identical to those of the host builder (mesh.box + concat).
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace {

struct BoxDev {
    int32_t nx, ny, nz, n;
    int32_t cell0, face0;
    int32_t bface0[6];
    double hx, hy, hz;
    double lx, ly, lz;
};

// ---- OpenFOAM geometry of a box face, in the host builder's operation order
struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ D3 operator/(D3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ double dot3(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross3(D3 a, D3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double mag3(D3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// vertex (i, j, k) of an unjittered box (the far faces land exactly on l)
__device__ __forceinline__ D3 box_pt(const BoxDev& b, int i, int j, int k) {
    return {i == b.nx ? b.lx : (double)i * b.hx, j == b.ny ? b.ly : (double)j * b.hy,
            k == b.nz ? b.lz : (double)k * b.hz};
}

// the face of direction d (0 x, 1 y, 2 z) at vertex index (i, j, k), normal +d,
// or -d when flip (the min patches): its points in the host builder's order
__device__ __forceinline__ void face_pts(const BoxDev& b, int d, int i, int j, int k, bool flip, D3 p[4]) {
    D3 a, q, c, e;
    if (d == 0) {
        a = box_pt(b, i, j, k); q = box_pt(b, i, j + 1, k); c = box_pt(b, i, j + 1, k + 1); e = box_pt(b, i, j, k + 1);
    } else if (d == 1) {
        a = box_pt(b, i, j, k); q = box_pt(b, i, j, k + 1); c = box_pt(b, i + 1, j, k + 1); e = box_pt(b, i + 1, j, k);
    } else {
        a = box_pt(b, i, j, k); q = box_pt(b, i + 1, j, k); c = box_pt(b, i + 1, j + 1, k); e = box_pt(b, i, j + 1, k);
    }
    p[0] = a;
    p[1] = flip ? e : q;
    p[2] = c;
    p[3] = flip ? q : e;
}

// face centre and area vector: triangles about the mean of the points
__device__ __forceinline__ void face_geom(const D3 p[4], D3& fC, D3& fA) {
    D3 cen = p[0];
    cen = cen + p[1];
    cen = cen + p[2];
    cen = cen + p[3];
    cen = cen / 4.0;
    D3 sN{0.0, 0.0, 0.0}, sAc{0.0, 0.0, 0.0};
    double sA = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const D3 a = p[q], nb = p[(q + 1) & 3];
        const D3 c = a + nb + cen;
        const D3 nr = cross3(nb - a, cen - a);
        const double m = mag3(nr);
        sN = sN + nr;
        sA += m;
        sAc = sAc + m * c;
    }
    if (sA < 1.0e-150) {
        fC = cen;
        fA = D3{0.0, 0.0, 0.0};
    } else {
        fC = ((1.0 / 3.0) * sAc) / sA;
        fA = 0.5 * sN;
    }
}

// the faces of cell (i, j, k) in the order they contribute to it on the host
// (face-list order: owned internal +x +y +z, owned boundary by patch, then the
// internal faces it neighbours, -z -y -x): direction, vertex index, flip, owner
struct CellFace {
    int d, i, j, k;
    bool flip, owner;
};
__device__ __forceinline__ int cell_faces(const BoxDev& b, int i, int j, int k, CellFace f[6]) {
    int n = 0;
    if (i < b.nx - 1) f[n++] = {0, i + 1, j, k, false, true};
    if (j < b.ny - 1) f[n++] = {1, i, j + 1, k, false, true};
    if (k < b.nz - 1) f[n++] = {2, i, j, k + 1, false, true};
    if (i == 0) f[n++] = {0, 0, j, k, true, true};
    if (i == b.nx - 1) f[n++] = {0, b.nx, j, k, false, true};
    if (j == 0) f[n++] = {1, i, 0, k, true, true};
    if (j == b.ny - 1) f[n++] = {1, i, b.ny, k, false, true};
    if (k == 0) f[n++] = {2, i, j, 0, true, true};
    if (k == b.nz - 1) f[n++] = {2, i, j, b.nz, false, true};
    if (k > 0) f[n++] = {2, i, j, k, false, false};
    if (j > 0) f[n++] = {1, i, j, k, false, false};
    if (i > 0) f[n++] = {0, i, j, k, false, false};
    return n;
}

// centre and volume of cell (i, j, k): pyramids on the mean of its face centres
__device__ __forceinline__ void cell_geom(const BoxDev& b, int i, int j, int k, D3& cc, double& vol) {
    CellFace f[6];
    const int nf = cell_faces(b, i, j, k, f);
    D3 fC[6], fA[6];
    D3 est{0.0, 0.0, 0.0};
    for (int q = 0; q < nf; ++q) {
        D3 p[4];
        face_pts(b, f[q].d, f[q].i, f[q].j, f[q].k, f[q].flip, p);
        face_geom(p, fC[q], fA[q]);
        est = est + fC[q];
    }
    est = est / (double)nf;
    D3 c{0.0, 0.0, 0.0};
    double v = 0.0;
    for (int q = 0; q < nf; ++q) {
        const double pv = f[q].owner ? dot3(fA[q], fC[q] - est) : dot3(fA[q], est - fC[q]);
        const D3 pc = (3.0 / 4.0) * fC[q] + (1.0 / 4.0) * est;
        c = c + pv * pc;
        v += pv;
    }
    cc = fabs(v) > 1.0e-300 ? c / v : est;
    vol = v * (1.0 / 3.0);
}

__global__ void k_box_centres(const BoxDev* __restrict__ boxes, const int32_t* __restrict__ slice_box, int N,
                              double* __restrict__ V, double* __restrict__ invV, double* __restrict__ Cc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int bi = slice_box[c >> 5];
    int loc = -1;
    BoxDev b;
    if (bi >= 0) {
        b = boxes[bi];
        loc = c - b.cell0;
        if (loc >= b.n) loc = -1;
    }
    if (loc < 0) {  // placeholder cell
        V[c] = 1.0;
        invV[c] = 1.0;
        Cc[3 * c] = Cc[3 * c + 1] = Cc[3 * c + 2] = 0.0;
        return;
    }
    const int i = loc % b.nx, j = (loc / b.nx) % b.ny, k = loc / (b.nx * b.ny);
    D3 cc;
    double vol;
    cell_geom(b, i, j, k, cc, vol);
    V[c] = vol;
    invV[c] = 1.0 / vol;
    Cc[3 * c] = cc.x;
    Cc[3 * c + 1] = cc.y;
    Cc[3 * c + 2] = cc.z;
}

// internal faces owned by cells before local cell (i,j,k) of the box
__device__ __forceinline__ int32_t faces_before(const BoxDev& b, int i, int j, int k) {
    const int nx = b.nx, ny = b.ny, nz = b.nz;
    const int32_t rows = j + ny * k;
    const int32_t X = rows * (nx - 1) + min(i, nx - 1);
    const int32_t Y = k * nx * (ny - 1) + nx * min(j, ny - 1) + (j < ny - 1 ? i : 0);
    const int32_t Z = nx * ny * min(k, nz - 1) + (k < nz - 1 ? j * nx + i : 0);
    return X + Y + Z;
}

__device__ __forceinline__ int32_t face_of(const BoxDev& b, int i, int j, int k, int dir) {
    // global index of the +dir face owned by local cell (i,j,k) (that face must exist)
    int32_t f = b.face0 + faces_before(b, i, j, k);
    if (dir >= 1 && i < b.nx - 1) ++f;
    if (dir >= 2 && j < b.ny - 1) ++f;
    return f;
}

struct MeshOut {
    double *V, *invV, *Sf, *magSf, *w, *delta, *geo;
    int32_t *own, *nei;
    int32_t* bcells;
    double *bSf, *bmagSf, *bdelta, *bgeo;
    int32_t* bpatch;
    int32_t *g_code, *g_other, *m_col, *m_code, *diag_pos, *own_pos, *nei_pos;
    int16_t* m_off;  // column - row per slot, or null (a box with nx*ny > 32767)
};

constexpr int kGW = 6;  // gather-list width (every box cell has 6 faces)
constexpr int kMW = 7;  // matrix row width

__global__ void k_box_cells(const BoxDev* __restrict__ boxes, const int32_t* __restrict__ slice_box, int N,
                            int nif, const double* __restrict__ Cc, MeshOut o) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int slice = c >> 5, lane = c & 31;
    const int gbase = slice * 32 * kGW + lane, mbase = slice * 32 * kMW + lane;
    const int bi = slice_box[slice];
    int loc = -1;
    BoxDev b;
    if (bi >= 0) {
        b = boxes[bi];
        loc = c - b.cell0;
        if (loc >= b.n) loc = -1;
    }
    if (loc < 0) {  // placeholder: unit volume (k_box_centres), no faces, diagonal-only row
        for (int k = 0; k < kGW; ++k) {
            o.g_code[gbase + k * 32] = FVGB_PAD;
            o.g_other[gbase + k * 32] = 0;
        }
        for (int k = 0; k < kMW; ++k) {
            o.m_col[mbase + k * 32] = c;
            if (o.m_off) o.m_off[mbase + k * 32] = 0;
            o.m_code[mbase + k * 32] = k == 0 ? -1 : FVGB_PAD;
        }
        o.diag_pos[c] = mbase;
        return;
    }
    const int nx = b.nx, ny = b.ny, nz = b.nz;
    const int i = loc % nx, j = (loc / nx) % ny, k = loc / (nx * ny);
    const int sy = nx, sz = nx * ny;
    const D3 Co{Cc[3 * c], Cc[3 * c + 1], Cc[3 * c + 2]};
    // upper faces owned by this cell: weights and delta coefficients as
    // surfaceInterpolation::makeWeights / makeNonOrthDeltaCoeffs
    int32_t f = b.face0 + faces_before(b, i, j, k);
    const int32_t fx = i < nx - 1 ? f++ : -1;
    const int32_t fy = j < ny - 1 ? f++ : -1;
    const int32_t fz = k < nz - 1 ? f++ : -1;
    const int32_t up_f[3] = {fx, fy, fz};
    const int32_t up_n[3] = {c + 1, c + sy, c + sz};
    for (int d = 0; d < 3; ++d) {
        const int32_t ff = up_f[d];
        if (ff < 0) continue;
        D3 p[4], Cf, Sf;
        face_pts(b, d, i + (d == 0), j + (d == 1), k + (d == 2), false, p);
        face_geom(p, Cf, Sf);
        const int32_t cn = up_n[d];
        const D3 Cn{Cc[3 * cn], Cc[3 * cn + 1], Cc[3 * cn + 2]};
        const double mS = mag3(Sf);
        const double dOwn = fabs(dot3(Sf, Cf - Co));
        const double dNei = fabs(dot3(Sf, Cn - Cf));
        const D3 dl = Cn - Co;
        const double nd = dot3(Sf / mS, dl), md = 0.05 * mag3(dl);
        const double dc = 1.0 / (nd > md ? nd : md);
        o.own[ff] = c;
        o.nei[ff] = cn;
        o.Sf[3 * ff] = Sf.x;
        o.Sf[3 * ff + 1] = Sf.y;
        o.Sf[3 * ff + 2] = Sf.z;
        o.magSf[ff] = mS;
        o.w[ff] = dNei / (dOwn + dNei);
        o.delta[ff] = dc;
        o.geo[ff] = mS * dc;
    }
    // lower faces (this cell is the neighbour), ascending face index: -z, -y, -x
    int32_t lo_f[3], lo_o[3];
    int nlo = 0;
    if (k > 0) {
        lo_f[nlo] = face_of(b, i, j, k - 1, 2);
        lo_o[nlo++] = c - sz;
    }
    if (j > 0) {
        lo_f[nlo] = face_of(b, i, j - 1, k, 1);
        lo_o[nlo++] = c - sy;
    }
    if (i > 0) {
        lo_f[nlo] = face_of(b, i - 1, j, k, 0);
        lo_o[nlo++] = c - 1;
    }
    // boundary faces of this cell, patch order
    int32_t bf[6];
    int nb = 0;
    // the face at vertex index (fi, fj, fk) of direction d; the min patches flip it
    auto bface = [&](int patch, int32_t idx, int d, int fi, int fj, int fk) {
        const int32_t bb = b.bface0[patch] + idx;
        D3 p[4], Cf, Sf;
        face_pts(b, d, fi, fj, fk, (patch & 1) == 0, p);
        face_geom(p, Cf, Sf);
        const double mS = mag3(Sf);
        const D3 nf = Sf / mS;
        const D3 dl = dot3(nf, Cf - Co) * nf;
        const double nd = dot3(nf, dl), md = 0.05 * mag3(dl);
        const double dc = 1.0 / (nd > md ? nd : md);
        o.bcells[bb] = c;
        o.bSf[3 * bb] = Sf.x;
        o.bSf[3 * bb + 1] = Sf.y;
        o.bSf[3 * bb + 2] = Sf.z;
        o.bmagSf[bb] = mS;
        o.bdelta[bb] = dc;
        o.bgeo[bb] = mS * dc;
        o.bpatch[bb] = patch;
        bf[nb++] = bb;
    };
    if (i == 0) bface(0, j + ny * k, 0, 0, j, k);
    if (i == nx - 1) bface(1, j + ny * k, 0, nx, j, k);
    if (j == 0) bface(2, i + nx * k, 1, i, 0, k);
    if (j == ny - 1) bface(3, i + nx * k, 1, i, ny, k);
    if (k == 0) bface(4, i + nx * j, 2, i, j, 0);
    if (k == nz - 1) bface(5, i + nx * j, 2, i, j, nz);
    // gather list
    int g = 0;
    for (int q = 0; q < nlo; ++q, ++g) {
        o.g_code[gbase + g * 32] = -lo_f[q] - 1;
        o.g_other[gbase + g * 32] = lo_o[q];
    }
    for (int d = 0; d < 3; ++d) {
        if (up_f[d] < 0) continue;
        o.g_code[gbase + g * 32] = up_f[d];
        o.g_other[gbase + g * 32] = up_n[d];
        ++g;
    }
    for (int q = 0; q < nb; ++q, ++g) {
        o.g_code[gbase + g * 32] = nif + bf[q];
        o.g_other[gbase + g * 32] = bf[q];
    }
    for (; g < kGW; ++g) {
        o.g_code[gbase + g * 32] = FVGB_PAD;
        o.g_other[gbase + g * 32] = 0;
    }
    // matrix row in column order: lower neighbours (ascending), diagonal, upper
    int s = 0;
    for (int q = 0; q < nlo; ++q, ++s) {  // lo_o is ascending: c-sz < c-sy < c-1
        const int pos = mbase + s * 32;
        o.m_col[pos] = lo_o[q];
        if (o.m_off) o.m_off[pos] = (int16_t)(lo_o[q] - c);
        o.m_code[pos] = -lo_f[q] - 2;
        o.nei_pos[lo_f[q]] = pos;
    }
    o.m_col[mbase + s * 32] = c;
    if (o.m_off) o.m_off[mbase + s * 32] = 0;
    o.m_code[mbase + s * 32] = -1;
    o.diag_pos[c] = mbase + s * 32;
    ++s;
    for (int d = 0; d < 3; ++d) {
        if (up_f[d] < 0) continue;
        const int pos = mbase + s * 32;
        o.m_col[pos] = up_n[d];
        if (o.m_off) o.m_off[pos] = (int16_t)(up_n[d] - c);
        o.m_code[pos] = up_f[d];
        o.own_pos[up_f[d]] = pos;
        ++s;
    }
    for (; s < kMW; ++s) {
        o.m_col[mbase + s * 32] = c;
        if (o.m_off) o.m_off[mbase + s * 32] = 0;
        o.m_code[mbase + s * 32] = FVGB_PAD;
    }
}

__global__ void k_fill_ptr(int32_t* p, int count, int width) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s <= count) p[s] = s * 32 * width;
}

void free_mesh_partial(fvgb_mesh* m) {
    for (void* p : m->allocs) devmem_free(p, m->pooled);
    delete m;
}

}  // namespace

extern "C" fvgb_status fvgb_mesh_create_boxes(const fvgb_box_spec* specs, int32_t nboxes, fvgb_mesh** out,
                                              int32_t* row_ranges, fvgb_stream stream) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(specs && out && row_ranges && nboxes > 0, "fvgb_mesh_create_boxes: bad argument");
    *out = nullptr;
    std::vector<BoxDev> boxes(nboxes);
    int64_t N = 0, NIF = 0;
    int64_t nb_patch[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < nboxes; ++q) {
        const fvgb_box_spec& s = specs[q];
        FVGB_CHECK_ARG(s.nx >= 1 && s.ny >= 1 && s.nz >= 1 && s.lx > 0 && s.ly > 0 && s.lz > 0,
                       "fvgb_mesh_create_boxes: bad box size");
        FVGB_CHECK_ARG(s.jitter == 0.0 && !s.two_d, "fvgb_mesh_create_boxes: unjittered 3-D boxes only");
        BoxDev& b = boxes[q];
        b.nx = s.nx;
        b.ny = s.ny;
        b.nz = s.nz;
        const int64_t n = (int64_t)s.nx * s.ny * s.nz;
        FVGB_CHECK_ARG(n < INT32_MAX / 8, "fvgb_mesh_create_boxes: box too large");
        b.n = (int32_t)n;
        N = (N + 31) / 32 * 32;
        b.cell0 = (int32_t)N;
        row_ranges[2 * q] = (int32_t)N;
        row_ranges[2 * q + 1] = (int32_t)(N + n);
        N += n;
        b.face0 = (int32_t)NIF;
        NIF += (int64_t)(s.nx - 1) * s.ny * s.nz + (int64_t)s.nx * (s.ny - 1) * s.nz + (int64_t)s.nx * s.ny * (s.nz - 1);
        b.hx = s.lx / s.nx;
        b.hy = s.ly / s.ny;
        b.hz = s.lz / s.nz;
        b.lx = s.lx;
        b.ly = s.ly;
        b.lz = s.lz;
        const int64_t pf[6] = {(int64_t)s.ny * s.nz, (int64_t)s.ny * s.nz, (int64_t)s.nx * s.nz,
                               (int64_t)s.nx * s.nz, (int64_t)s.nx * s.ny, (int64_t)s.nx * s.ny};
        for (int p = 0; p < 6; ++p) nb_patch[p] += pf[p];
    }
    N = (N + 31) / 32 * 32;
    FVGB_CHECK_ARG(N + 2 * NIF < INT32_MAX / 2 && N * kMW < INT32_MAX, "fvgb_mesh_create_boxes: too large");
    // boundary face offsets: patch-major, box-minor
    int64_t NBF = 0;
    std::vector<int32_t> poffs(7, 0);
    for (int p = 0; p < 6; ++p) {
        poffs[p] = (int32_t)NBF;
        for (int q = 0; q < nboxes; ++q) {
            const fvgb_box_spec& s = specs[q];
            const int64_t pf = p < 2 ? (int64_t)s.ny * s.nz : (p < 4 ? (int64_t)s.nx * s.nz : (int64_t)s.nx * s.ny);
            boxes[q].bface0[p] = (int32_t)NBF;
            NBF += pf;
        }
    }
    poffs[6] = (int32_t)NBF;
    const int32_t nslices = (int32_t)(N / 32);
    std::vector<int32_t> slice_box(nslices, -1);
    for (int q = 0; q < nboxes; ++q)
        for (int32_t sl = boxes[q].cell0 / 32; sl < (boxes[q].cell0 + boxes[q].n + 31) / 32; ++sl) slice_box[sl] = q;

    fvgb_mesh* m = new fvgb_mesh();
    m->pooled = devmem_pooled_now();
    m->h_patch_offs = poffs;
    m->nnz = (int32_t)(N + 2 * NIF);
    m->nslices = nslices;
    m->m_len = (int64_t)N * kMW;
    m->g_len = (int64_t)N * kGW;
    MeshView& v = m->v;
    v.n = (int32_t)N;
    v.nif = (int32_t)NIF;
    v.nbf = (int32_t)NBF;
    v.npatch = 6;
    MeshOut o{};
    cudaError_t e = cudaSuccess;
    auto A = [&](auto** p, int64_t count) {
        if (e == cudaSuccess) e = mesh_alloc(m, p, count);
    };
    A(&o.V, N);
    A(&o.invV, N);
    A(&o.own, NIF);
    A(&o.nei, NIF);
    A(&o.Sf, 3 * NIF);
    A(&o.magSf, NIF);
    A(&o.w, NIF);
    A(&o.delta, NIF);
    A(&o.geo, NIF);
    A(&o.bcells, NBF);
    A(&o.bSf, 3 * NBF);
    A(&o.bmagSf, NBF);
    A(&o.bdelta, NBF);
    A(&o.bgeo, NBF);
    A(&o.bpatch, NBF);
    int32_t *g_ptr = nullptr, *m_ptr = nullptr, *d_slice_box = nullptr;
    BoxDev* d_boxes = nullptr;
    A(&g_ptr, nslices + 1);
    A(&m_ptr, nslices + 1);
    A(&o.g_code, N * kGW);
    A(&o.g_other, N * kGW);
    A(&o.m_col, N * kMW);
    // 16-bit column offsets fit when every box's largest neighbour offset does:
    // nx*ny (z neighbours) for a box more than one cell thick, else nx, else 1
    bool off_fits = true;
    for (int q = 0; q < nboxes; ++q) {
        const fvgb_box_spec& b = specs[q];
        const int64_t span = b.nz > 1 ? (int64_t)b.nx * b.ny : (b.ny > 1 ? (int64_t)b.nx : 1);
        off_fits = off_fits && span <= 32767;
    }
    o.m_off = nullptr;
    if (off_fits) A(&o.m_off, N * kMW);
    A(&o.m_code, N * kMW);
    A(&o.diag_pos, N);
    A(&o.own_pos, NIF);
    A(&o.nei_pos, NIF);
    A(&d_slice_box, nslices);
    A(&d_boxes, nboxes);
    double* d_centres = nullptr;  // cell centres, the weights' input
    A(&d_centres, 3 * N);
    cudaStream_t st = (cudaStream_t)stream;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_slice_box, slice_box.data(), 4 * (size_t)nslices, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_boxes, boxes.data(), sizeof(BoxDev) * (size_t)nboxes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        free_mesh_partial(m);
        return cuda_fail(e, "fvgb_mesh_create_boxes: allocation");
    }
    k_fill_ptr<<<grid_for(nslices + 1, 256), 256, 0, st>>>(g_ptr, nslices, kGW);
    k_fill_ptr<<<grid_for(nslices + 1, 256), 256, 0, st>>>(m_ptr, nslices, kMW);
    k_box_centres<<<grid_for(N, 128), 128, 0, st>>>(d_boxes, d_slice_box, (int)N, o.V, o.invV, d_centres);
    k_box_cells<<<grid_for(N, 128), 128, 0, st>>>(d_boxes, d_slice_box, (int)N, (int)NIF, d_centres, o);
    // no synchronisation: asynchronous copies from pageable host memory are staged
    // before the call returns, so the host vectors may go out of scope
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        free_mesh_partial(m);
        return cuda_fail(e, "fvgb_mesh_create_boxes: build");
    }
    v.V = o.V;
    v.invV = o.invV;
    v.own = o.own;
    v.nei = o.nei;
    v.Sf = o.Sf;
    v.magSf = o.magSf;
    v.w = o.w;
    v.delta = o.delta;
    v.geo = o.geo;
    v.bcells = o.bcells;
    v.bSf = o.bSf;
    v.bmagSf = o.bmagSf;
    v.bdelta = o.bdelta;
    v.bgeo = o.bgeo;
    v.bpatch = o.bpatch;
    v.g_ptr = g_ptr;
    v.g_code = o.g_code;
    v.g_other = o.g_other;
    v.m_ptr = m_ptr;
    v.m_col = o.m_col;
    v.m_off = o.m_off;
    v.m_code = o.m_code;
    v.diag_pos = o.diag_pos;
    v.own_pos = o.own_pos;
    v.nei_pos = o.nei_pos;
    m->csr_pos = nullptr;  // no host CSR copy: fvgb_mesh_sparsity / values export are not available
    *out = m;
    return FVGB_OK;
}
