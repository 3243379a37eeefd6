// Host-side mesh builder: an OpenFOAM-ordered hex box and OpenFOAM-style
// geometry for a general polyMesh.  In the reference these arrays come from
// Foam::fvMesh through MeshAdapter (src/datastructures/meshAdapter.cpp:59-136);
// here they are computed from the mathematics of OpenFOAM's
// primitiveMeshFaceCentresAndAreas / primitiveMeshCellCentresAndVols /
// surfaceInterpolation::makeWeights / makeNonOrthDeltaCoeffs.
//
// Compiled with -ffp-contract=off so that x86-64 and aarch64 hosts produce the
// same bits.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "fvgb.h"
#include "fvgb_host_common.h"

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double mag(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 ld(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
inline void st(double* p, int64_t i, V3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

const double kRootVSmall = 1.0e-150;
const double kVSmall = 1.0e-300;

// splitmix-style generator on top of a 64-bit LCG state: a fixed,
// library-independent stream so both host architectures draw the same jitter.
struct Rng64 {
    uint64_t s;
    explicit Rng64(uint64_t seed) : s(seed ^ 0x9E3779B97F4A7C15ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // uniform in [-1, 1)
    double sym() { return 2.0 * (double)(next() >> 11) * (1.0 / 9007199254740992.0) - 1.0; }
};

struct BoxTopo {
    int64_t np = 0, nc = 0, nif = 0, nbf = 0, nft = 0, npatch = 0;
    std::vector<int32_t> face_offs, face_pts, owner_all, neighbour;
    std::vector<int32_t> patch_offsets;  // non-empty patches only
};

bool box_check(const fvgb_box_spec* s) {
    if (!s || s->nx < 1 || s->ny < 1 || s->nz < 1) return false;
    if (s->two_d && s->nz != 1) return false;
    if (!(s->lx > 0 && s->ly > 0 && s->lz > 0)) return false;
    if (!(s->jitter >= 0 && s->jitter < 0.5)) return false;
    int64_t nc = (int64_t)s->nx * s->ny * s->nz;
    if (nc * 4 > INT32_MAX) return false;
    return true;
}

void box_counts(const fvgb_box_spec* s, int64_t* np, int64_t* nc, int64_t* nif, int64_t* nbf,
                int64_t* nft, int64_t* npatch) {
    int64_t nx = s->nx, ny = s->ny, nz = s->nz;
    *np = (nx + 1) * (ny + 1) * (nz + 1);
    *nc = nx * ny * nz;
    *nif = (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1);
    int64_t xb = 2 * ny * nz, yb = 2 * nx * nz, zb = 2 * nx * ny;
    if (s->two_d) {
        *nbf = xb + yb;
        *npatch = 4;
    } else {
        *nbf = xb + yb + zb;
        *npatch = 6;
    }
    *nft = *nif + xb + yb + zb;
}

// Builds face list in OpenFOAM order: internal faces upper-triangular (owner
// ascending, neighbour ascending per owner), then the patches xmin, xmax,
// ymin, ymax, zmin, zmax (zmin/zmax are the empty frontAndBack in 2-D and then
// come last and are excluded from the flat boundary).
void box_topology(const fvgb_box_spec* s, BoxTopo& t) {
    const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
    box_counts(s, &t.np, &t.nc, &t.nif, &t.nbf, &t.nft, &t.npatch);
    auto P = [&](int64_t i, int64_t j, int64_t k) {
        return (int32_t)(i + (nx + 1) * (j + (ny + 1) * k));
    };
    auto C = [&](int64_t i, int64_t j, int64_t k) { return (int32_t)(i + nx * (j + ny * k)); };
    t.face_offs.assign(1, 0);
    t.face_offs.reserve(t.nft + 1);
    t.face_pts.reserve(4 * t.nft);
    t.owner_all.reserve(t.nft);
    t.neighbour.reserve(t.nif);
    auto push = [&](int32_t a, int32_t b, int32_t c, int32_t d, int32_t own) {
        t.face_pts.push_back(a);
        t.face_pts.push_back(b);
        t.face_pts.push_back(c);
        t.face_pts.push_back(d);
        t.face_offs.push_back((int32_t)t.face_pts.size());
        t.owner_all.push_back(own);
    };
    // +x face at x index i (normal +x), +y face at y index j, +z face at z index k
    auto xface = [&](int64_t i, int64_t j, int64_t k, int32_t own, bool flip) {
        int32_t a = P(i, j, k), b = P(i, j + 1, k), c = P(i, j + 1, k + 1), d = P(i, j, k + 1);
        if (flip) push(a, d, c, b, own); else push(a, b, c, d, own);
    };
    auto yface = [&](int64_t i, int64_t j, int64_t k, int32_t own, bool flip) {
        int32_t a = P(i, j, k), b = P(i, j, k + 1), c = P(i + 1, j, k + 1), d = P(i + 1, j, k);
        if (flip) push(a, d, c, b, own); else push(a, b, c, d, own);
    };
    auto zface = [&](int64_t i, int64_t j, int64_t k, int32_t own, bool flip) {
        int32_t a = P(i, j, k), b = P(i + 1, j, k), c = P(i + 1, j + 1, k), d = P(i, j + 1, k);
        if (flip) push(a, d, c, b, own); else push(a, b, c, d, own);
    };
    for (int64_t k = 0; k < nz; ++k)
        for (int64_t j = 0; j < ny; ++j)
            for (int64_t i = 0; i < nx; ++i) {
                int32_t c = C(i, j, k);
                if (i + 1 < nx) { xface(i + 1, j, k, c, false); t.neighbour.push_back(C(i + 1, j, k)); }
                if (j + 1 < ny) { yface(i, j + 1, k, c, false); t.neighbour.push_back(C(i, j + 1, k)); }
                if (k + 1 < nz) { zface(i, j, k + 1, c, false); t.neighbour.push_back(C(i, j, k + 1)); }
            }
    t.patch_offsets.assign(1, 0);
    auto close_patch = [&]() {
        t.patch_offsets.push_back((int32_t)(t.owner_all.size() - t.nif));
    };
    for (int64_t k = 0; k < nz; ++k)
        for (int64_t j = 0; j < ny; ++j) xface(0, j, k, C(0, j, k), true);
    close_patch();
    for (int64_t k = 0; k < nz; ++k)
        for (int64_t j = 0; j < ny; ++j) xface(nx, j, k, C(nx - 1, j, k), false);
    close_patch();
    for (int64_t k = 0; k < nz; ++k)
        for (int64_t i = 0; i < nx; ++i) yface(i, 0, k, C(i, 0, k), true);
    close_patch();
    for (int64_t k = 0; k < nz; ++k)
        for (int64_t i = 0; i < nx; ++i) yface(i, ny, k, C(i, ny - 1, k), false);
    close_patch();
    for (int64_t j = 0; j < ny; ++j)
        for (int64_t i = 0; i < nx; ++i) zface(i, j, 0, C(i, j, 0), true);
    if (!s->two_d) close_patch();
    for (int64_t j = 0; j < ny; ++j)
        for (int64_t i = 0; i < nx; ++i) zface(i, j, nz, C(i, j, nz - 1), false);
    if (!s->two_d) close_patch();
}

void box_points(const fvgb_box_spec* s, std::vector<double>& pts) {
    const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
    const double hx = s->lx / nx, hy = s->ly / ny, hz = s->lz / nz;
    pts.resize(3 * (nx + 1) * (ny + 1) * (nz + 1));
    Rng64 rng(s->seed);
    // one draw per interior vertex per axis, vertices in point order; in 2-D the
    // in-plane draw of (i,j) is shared by both z layers and z is not jittered.
    std::vector<double> jx, jy;
    if (s->two_d) {
        jx.assign((nx + 1) * (ny + 1), 0.0);
        jy.assign((nx + 1) * (ny + 1), 0.0);
        for (int64_t j = 1; j < ny; ++j)
            for (int64_t i = 1; i < nx; ++i) {
                jx[i + (nx + 1) * j] = s->jitter * hx * rng.sym();
                jy[i + (nx + 1) * j] = s->jitter * hy * rng.sym();
            }
    }
    for (int64_t k = 0; k <= nz; ++k)
        for (int64_t j = 0; j <= ny; ++j)
            for (int64_t i = 0; i <= nx; ++i) {
                int64_t p = i + (nx + 1) * (j + (ny + 1) * k);
                double x = (i == nx) ? s->lx : i * hx;
                double y = (j == ny) ? s->ly : j * hy;
                double z = (k == nz) ? s->lz : k * hz;
                if (s->two_d) {
                    x += jx[i + (nx + 1) * j];
                    y += jy[i + (nx + 1) * j];
                } else if (i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz && s->jitter > 0) {
                    x += s->jitter * hx * rng.sym();
                    y += s->jitter * hy * rng.sym();
                    z += s->jitter * hz * rng.sym();
                }
                pts[3 * p] = x;
                pts[3 * p + 1] = y;
                pts[3 * p + 2] = z;
            }
}

}  // namespace

extern "C" fvgb_status fvgb_box_sizes(const fvgb_box_spec* spec, int64_t out[7]) {
    if (!box_check(spec) || !out) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_box_sizes: bad box spec");
    int64_t np, nc, nif, nbf, nft, npatch;
    box_counts(spec, &np, &nc, &nif, &nbf, &nft, &npatch);
    out[0] = np;
    out[1] = nft;
    out[2] = nc;
    out[3] = nif;
    out[4] = nbf;
    out[5] = npatch;
    out[6] = 4 * nft;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_geometry_compute(int32_t n_points, const double* points,
                                             int32_t n_cells, int32_t n_faces_total,
                                             const int32_t* face_offs, const int32_t* face_points,
                                             const int32_t* owner_all, int32_t n_ifaces,
                                             const int32_t* neighbour, int32_t n_bfaces,
                                             fvgb_mesh_arrays* out) {
    if (!points || !face_offs || !face_points || !owner_all || !out || n_cells <= 0 ||
        n_ifaces < 0 || n_bfaces < 0 || (int64_t)n_ifaces + n_bfaces > n_faces_total ||
        (n_ifaces > 0 && !neighbour))
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: bad arguments");
    if (!out->cell_volumes || !out->face_areas || !out->mag_face_areas || !out->weights ||
        !out->delta_coeffs || (n_bfaces > 0 && (!out->bface_cells || !out->bface_areas ||
        !out->bmag_face_areas || !out->bweights || !out->bdelta_coeffs)))
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: missing output array");
    const int64_t nft = n_faces_total;
    for (int64_t f = 0; f < nft; ++f) {
        if (face_offs[f + 1] - face_offs[f] < 3)
            return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: face with < 3 points");
        if (owner_all[f] < 0 || owner_all[f] >= n_cells)
            return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: owner out of range");
        for (int32_t q = face_offs[f]; q < face_offs[f + 1]; ++q)
            if (face_points[q] < 0 || face_points[q] >= n_points)
                return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: point out of range");
    }
    for (int64_t f = 0; f < n_ifaces; ++f)
        if (neighbour[f] < 0 || neighbour[f] >= n_cells)
            return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: neighbour out of range");

    // face centres and area vectors (triangle decomposition about the point average)
    std::vector<double> fC(3 * nft), fA(3 * nft);
    for (int64_t f = 0; f < nft; ++f) {
        const int32_t b = face_offs[f], e = face_offs[f + 1], np = e - b;
        if (np == 3) {
            V3 p0 = ld(points, face_points[b]), p1 = ld(points, face_points[b + 1]),
               p2 = ld(points, face_points[b + 2]);
            st(fC.data(), f, (1.0 / 3.0) * (p0 + p1 + p2));
            st(fA.data(), f, 0.5 * cross(p1 - p0, p2 - p0));
            continue;
        }
        V3 fCentre = ld(points, face_points[b]);
        for (int32_t q = b + 1; q < e; ++q) fCentre = fCentre + ld(points, face_points[q]);
        fCentre = fCentre / (double)np;
        V3 sumN{0, 0, 0}, sumAc{0, 0, 0};
        double sumA = 0.0;
        for (int32_t q = 0; q < np; ++q) {
            V3 thisP = ld(points, face_points[b + q]);
            V3 nextP = ld(points, face_points[b + (q + 1 == np ? 0 : q + 1)]);
            V3 c = thisP + nextP + fCentre;
            V3 n = cross(nextP - thisP, fCentre - thisP);
            double a = mag(n);
            sumN = sumN + n;
            sumA += a;
            sumAc = sumAc + a * c;
        }
        if (sumA < kRootVSmall) {
            st(fC.data(), f, fCentre);
            st(fA.data(), f, V3{0, 0, 0});
        } else {
            st(fC.data(), f, ((1.0 / 3.0) * sumAc) / sumA);
            st(fA.data(), f, 0.5 * sumN);
        }
    }
    // cell centre estimate: average of the face centres of the cell
    std::vector<double> cEst(3 * (int64_t)n_cells, 0.0);
    std::vector<int32_t> nCF(n_cells, 0);
    for (int64_t f = 0; f < nft; ++f) {
        int32_t o = owner_all[f];
        st(cEst.data(), o, ld(cEst.data(), o) + ld(fC.data(), f));
        nCF[o] += 1;
    }
    for (int64_t f = 0; f < n_ifaces; ++f) {
        int32_t nb = neighbour[f];
        st(cEst.data(), nb, ld(cEst.data(), nb) + ld(fC.data(), f));
        nCF[nb] += 1;
    }
    for (int64_t c = 0; c < n_cells; ++c) {
        if (nCF[c] == 0) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: cell without faces");
        st(cEst.data(), c, ld(cEst.data(), c) / (double)nCF[c]);
    }
    std::vector<double> cC(3 * (int64_t)n_cells, 0.0), cV(n_cells, 0.0);
    for (int64_t f = 0; f < nft; ++f) {
        int32_t o = owner_all[f];
        V3 Cf = ld(fC.data(), f), Sf = ld(fA.data(), f), ce = ld(cEst.data(), o);
        double pyr3Vol = dot(Sf, Cf - ce);
        V3 pc = (3.0 / 4.0) * Cf + (1.0 / 4.0) * ce;
        st(cC.data(), o, ld(cC.data(), o) + pyr3Vol * pc);
        cV[o] += pyr3Vol;
    }
    for (int64_t f = 0; f < n_ifaces; ++f) {
        int32_t nb = neighbour[f];
        V3 Cf = ld(fC.data(), f), Sf = ld(fA.data(), f), ce = ld(cEst.data(), nb);
        double pyr3Vol = dot(Sf, ce - Cf);
        V3 pc = (3.0 / 4.0) * Cf + (1.0 / 4.0) * ce;
        st(cC.data(), nb, ld(cC.data(), nb) + pyr3Vol * pc);
        cV[nb] += pyr3Vol;
    }
    for (int64_t c = 0; c < n_cells; ++c) {
        if (std::fabs(cV[c]) > kVSmall) st(cC.data(), c, ld(cC.data(), c) / cV[c]);
        else st(cC.data(), c, ld(cEst.data(), c));
        cV[c] *= (1.0 / 3.0);
        if (!(cV[c] > 0)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_geometry_compute: non-positive cell volume");
    }
    std::memcpy(out->cell_volumes, cV.data(), sizeof(double) * n_cells);
    if (out->cell_centres) std::memcpy(out->cell_centres, cC.data(), sizeof(double) * 3 * n_cells);
    // internal faces
    for (int64_t f = 0; f < n_ifaces; ++f) {
        int32_t o = owner_all[f], nb = neighbour[f];
        V3 Sf = ld(fA.data(), f), Cf = ld(fC.data(), f);
        V3 Co = ld(cC.data(), o), Cn = ld(cC.data(), nb);
        double magSf = mag(Sf);
        double SfdOwn = std::fabs(dot(Sf, Cf - Co));
        double SfdNei = std::fabs(dot(Sf, Cn - Cf));
        V3 delta = Cn - Co;
        V3 unitArea = Sf / magSf;
        double nd = dot(unitArea, delta), md = 0.05 * mag(delta);
        if (out->owner) out->owner[f] = o;
        if (out->neighbour) out->neighbour[f] = nb;
        st(out->face_areas, f, Sf);
        if (out->face_centres) st(out->face_centres, f, Cf);
        out->mag_face_areas[f] = magSf;
        out->weights[f] = SfdNei / (SfdOwn + SfdNei);
        out->delta_coeffs[f] = 1.0 / (nd > md ? nd : md);
    }
    // boundary faces of the non-empty patches
    for (int64_t b = 0; b < n_bfaces; ++b) {
        int64_t f = n_ifaces + b;
        int32_t o = owner_all[f];
        V3 Sf = ld(fA.data(), f), Cf = ld(fC.data(), f), Co = ld(cC.data(), o);
        double magSf = mag(Sf);
        V3 nf = Sf / magSf;
        V3 delta = dot(nf, Cf - Co) * nf;
        double nd = dot(nf, delta), md = 0.05 * mag(delta);
        out->bface_cells[b] = o;
        st(out->bface_areas, b, Sf);
        if (out->bface_centres) st(out->bface_centres, b, Cf);
        out->bmag_face_areas[b] = magSf;
        out->bweights[b] = 1.0;
        out->bdelta_coeffs[b] = 1.0 / (nd > md ? nd : md);
    }
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_box_build(const fvgb_box_spec* spec, fvgb_mesh_arrays* out) {
    if (!box_check(spec) || !out) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_box_build: bad box spec");
    BoxTopo t;
    box_topology(spec, t);
    std::vector<double> pts;
    box_points(spec, pts);
    if (out->points) std::memcpy(out->points, pts.data(), sizeof(double) * pts.size());
    if (out->patch_offsets)
        std::memcpy(out->patch_offsets, t.patch_offsets.data(), sizeof(int32_t) * t.patch_offsets.size());
    return fvgb_geometry_compute((int32_t)t.np, pts.data(), (int32_t)t.nc, (int32_t)t.nft,
                                 t.face_offs.data(), t.face_pts.data(), t.owner_all.data(),
                                 (int32_t)t.nif, t.neighbour.data(), (int32_t)t.nbf, out);
}
