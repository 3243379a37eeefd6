/*
 * boxmesh.c -- the synthetic hex-box meshes of the workloads, built on the CPU
 * for the oracle.  TEST INFRASTRUCTURE ONLY: the CPU legs of the benchmark
 * (the timed reference arm) and the parity tests build their meshes here, so
 * that they never load the GPU library.
 *
 * Topology: OpenFOAM ordering as blockMesh writes a box -- cells i fastest,
 * then j, then k; internal faces upper-triangular (by owner, then its +x, +y,
 * +z neighbours); boundary faces patch by patch: xmin, xmax, ymin, ymax, zmin,
 * zmax (in 2-D zmin/zmax are the empty frontAndBack patches: they exist in the
 * face list and the cell geometry but not in the flat boundary, as an fvPatch
 * of an empty patch has size 0; meshAdapter.cpp:104-133).
 *
 * Vertex jitter: one draw per interior vertex per axis, in point order, from
 * a splitmix64 stream (state seed ^ 0x9E3779B97F4A7C15, increment the golden
 * ratio constant), uniform in [-1, 1) from the top 53 bits, scaled by
 * jitter x spacing.  In 2-D one in-plane draw per (i, j) is shared by both z
 * layers.  This is the workloads' seeded input definition.
 *
 * Geometry: OpenFOAM's published method --
 *   primitiveMeshFaceCentresAndAreas: a face is split into triangles about the
 *     average of its points; its area vector is half the sum of the triangle
 *     normals, its centre the area-weighted mean of the triangle centroids;
 *   primitiveMeshCellCentresAndVols: pyramids from an estimated centre (the
 *     mean of the cell's face centres) to every face; volume = sum / 3, centre
 *     = volume-weighted pyramid centroids (3/4 face centre + 1/4 apex);
 *   surfaceInterpolation::makeWeights: w = |Sf.(C_N - Cf)| / (|Sf.(Cf - C_P)| +
 *     |Sf.(C_N - Cf)|); boundary w = 1;
 *   makeNonOrthDeltaCoeffs: 1 / max(n.d, 0.05 |d|), with d = C_N - C_P inside
 *     and the face-normal part of Cf - C_P on the boundary.
 * Faces contribute to a cell in face-list order: owned faces first (internal,
 * then boundary), then the faces it neighbours.  Compiled with
 * -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fvoracle.h"

typedef struct {
    double x, y, z;
} v3;

static v3 vadd(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 vscale(double s, v3 a) { v3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static v3 vdiv(v3 a, double s) { v3 r = {a.x / s, a.y / s, a.z / s}; return r; }
static double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 vcross(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static double vmag(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static v3 vld(const double* p, int64_t i) { v3 r = {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; return r; }
static void vst(double* p, int64_t i, v3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

static uint64_t sm_next(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double sm_sym(uint64_t* s) { return 2.0 * (double)(sm_next(s) >> 11) * (1.0 / 9007199254740992.0) - 1.0; }

int32_t or_box_sizes(int32_t nx, int32_t ny, int32_t nz, int32_t two_d, int64_t out[6]) {
    if (nx < 1 || ny < 1 || nz < 1 || (two_d && nz != 1)) return -1;
    int64_t X = nx, Y = ny, Z = nz;
    out[0] = (X + 1) * (Y + 1) * (Z + 1);                                   /* points */
    out[1] = X * Y * Z;                                                     /* cells */
    out[2] = (X - 1) * Y * Z + X * (Y - 1) * Z + X * Y * (Z - 1);           /* internal faces */
    out[3] = two_d ? 2 * Y * Z + 2 * X * Z : 2 * Y * Z + 2 * X * Z + 2 * X * Y; /* flat boundary faces */
    out[4] = two_d ? 4 : 6;                                                 /* non-empty patches */
    out[5] = out[2] + 2 * Y * Z + 2 * X * Z + 2 * X * Y;                    /* all faces */
    return 0;
}

int32_t or_box_build(int32_t nx, int32_t ny, int32_t nz, double lx, double ly, double lz, double jitter,
                     uint64_t seed, int32_t two_d, or_box_arrays* out) {
    int64_t sz[6];
    if (or_box_sizes(nx, ny, nz, two_d, sz) != 0 || !(lx > 0 && ly > 0 && lz > 0) || !(jitter >= 0 && jitter < 0.5))
        return -1;
    const int64_t NP = sz[0], NC = sz[1], NIF = sz[2], NBF = sz[3], NFT = sz[5];
    const int64_t X = nx, Y = ny, Z = nz;
    const double hx = lx / nx, hy = ly / ny, hz = lz / nz;
    /* ---- points */
    double* pts = out->points ? out->points : (double*)malloc(sizeof(double) * 3 * NP);
    uint64_t rs = seed ^ 0x9E3779B97F4A7C15ull;
    double *jx = NULL, *jy = NULL;
    if (two_d) {
        jx = (double*)calloc((size_t)((X + 1) * (Y + 1)), sizeof(double));
        jy = (double*)calloc((size_t)((X + 1) * (Y + 1)), sizeof(double));
        for (int64_t j = 1; j < Y; ++j)
            for (int64_t i = 1; i < X; ++i) {
                jx[i + (X + 1) * j] = jitter * hx * sm_sym(&rs);
                jy[i + (X + 1) * j] = jitter * hy * sm_sym(&rs);
            }
    }
    for (int64_t k = 0; k <= Z; ++k)
        for (int64_t j = 0; j <= Y; ++j)
            for (int64_t i = 0; i <= X; ++i) {
                const int64_t p = i + (X + 1) * (j + (Y + 1) * k);
                double x = (i == X) ? lx : i * hx;
                double y = (j == Y) ? ly : j * hy;
                double z = (k == Z) ? lz : k * hz;
                if (two_d) {
                    x += jx[i + (X + 1) * j];
                    y += jy[i + (X + 1) * j];
                } else if (i > 0 && i < X && j > 0 && j < Y && k > 0 && k < Z && jitter > 0) {
                    x += jitter * hx * sm_sym(&rs);
                    y += jitter * hy * sm_sym(&rs);
                    z += jitter * hz * sm_sym(&rs);
                }
                pts[3 * p] = x;
                pts[3 * p + 1] = y;
                pts[3 * p + 2] = z;
            }
    free(jx);
    free(jy);
    /* ---- faces: four points each, owner, neighbour */
    int32_t* fp = (int32_t*)malloc(sizeof(int32_t) * 4 * NFT);
    int32_t* fo = (int32_t*)malloc(sizeof(int32_t) * NFT);
    int32_t* fn = (int32_t*)malloc(sizeof(int32_t) * (NIF > 0 ? NIF : 1));
    int64_t nf = 0, ni = 0;
#define PT(i, j, k) ((int32_t)((i) + (X + 1) * ((j) + (Y + 1) * (k))))
#define CELL(i, j, k) ((int32_t)((i) + X * ((j) + Y * (k))))
#define PUSH(a, b, c, d, own, flip)                                                  \
    do {                                                                             \
        fp[4 * nf] = (a);                                                            \
        fp[4 * nf + 1] = (flip) ? (d) : (b);                                         \
        fp[4 * nf + 2] = (c);                                                        \
        fp[4 * nf + 3] = (flip) ? (b) : (d);                                         \
        fo[nf++] = (own);                                                            \
    } while (0)
    /* +x face at x index i spans (j..j+1, k..k+1); +y and +z alike; "flip" turns
     * the normal to -x (-y, -z) for the min patches */
#define XF(i, j, k, own, flip) PUSH(PT(i, j, k), PT(i, j + 1, k), PT(i, j + 1, k + 1), PT(i, j, k + 1), own, flip)
#define YF(i, j, k, own, flip) PUSH(PT(i, j, k), PT(i, j, k + 1), PT(i + 1, j, k + 1), PT(i + 1, j, k), own, flip)
#define ZF(i, j, k, own, flip) PUSH(PT(i, j, k), PT(i + 1, j, k), PT(i + 1, j + 1, k), PT(i, j + 1, k), own, flip)
    for (int64_t k = 0; k < Z; ++k)
        for (int64_t j = 0; j < Y; ++j)
            for (int64_t i = 0; i < X; ++i) {
                const int32_t c = CELL(i, j, k);
                if (i + 1 < X) { XF(i + 1, j, k, c, 0); fn[ni++] = CELL(i + 1, j, k); }
                if (j + 1 < Y) { YF(i, j + 1, k, c, 0); fn[ni++] = CELL(i, j + 1, k); }
                if (k + 1 < Z) { ZF(i, j, k + 1, c, 0); fn[ni++] = CELL(i, j, k + 1); }
            }
    int32_t* po = out->patch_offs;
    int np = 0;
    po[np++] = 0;
    for (int64_t k = 0; k < Z; ++k)
        for (int64_t j = 0; j < Y; ++j) XF(0, j, k, CELL(0, j, k), 1);
    po[np++] = (int32_t)(nf - NIF);
    for (int64_t k = 0; k < Z; ++k)
        for (int64_t j = 0; j < Y; ++j) XF(X, j, k, CELL(X - 1, j, k), 0);
    po[np++] = (int32_t)(nf - NIF);
    for (int64_t k = 0; k < Z; ++k)
        for (int64_t i = 0; i < X; ++i) YF(i, 0, k, CELL(i, 0, k), 1);
    po[np++] = (int32_t)(nf - NIF);
    for (int64_t k = 0; k < Z; ++k)
        for (int64_t i = 0; i < X; ++i) YF(i, Y, k, CELL(i, Y - 1, k), 0);
    po[np++] = (int32_t)(nf - NIF);
    for (int64_t j = 0; j < Y; ++j)
        for (int64_t i = 0; i < X; ++i) ZF(i, j, 0, CELL(i, j, 0), 1);
    if (!two_d) po[np++] = (int32_t)(nf - NIF);
    for (int64_t j = 0; j < Y; ++j)
        for (int64_t i = 0; i < X; ++i) ZF(i, j, Z, CELL(i, j, Z - 1), 0);
    if (!two_d) po[np++] = (int32_t)(nf - NIF);
#undef XF
#undef YF
#undef ZF
#undef PUSH
#undef CELL
#undef PT
    /* ---- face centres and area vectors */
    double* fC = (double*)malloc(sizeof(double) * 3 * NFT);
    double* fA = (double*)malloc(sizeof(double) * 3 * NFT);
    for (int64_t f = 0; f < NFT; ++f) {
        v3 cen = vld(pts, fp[4 * f]);
        for (int q = 1; q < 4; ++q) cen = vadd(cen, vld(pts, fp[4 * f + q]));
        cen = vdiv(cen, 4.0);
        v3 sN = {0, 0, 0}, sAc = {0, 0, 0};
        double sA = 0.0;
        for (int q = 0; q < 4; ++q) {
            v3 a = vld(pts, fp[4 * f + q]), b = vld(pts, fp[4 * f + (q + 1) % 4]);
            v3 c = vadd(vadd(a, b), cen);
            v3 nrm = vcross(vsub(b, a), vsub(cen, a));
            double m = vmag(nrm);
            sN = vadd(sN, nrm);
            sA += m;
            sAc = vadd(sAc, vscale(m, c));
        }
        if (sA < 1.0e-150) {
            vst(fC, f, cen);
            v3 zero = {0, 0, 0};
            vst(fA, f, zero);
        } else {
            vst(fC, f, vdiv(vscale(1.0 / 3.0, sAc), sA));
            vst(fA, f, vscale(0.5, sN));
        }
    }
    /* ---- cell centres and volumes */
    double* est = (double*)calloc((size_t)(3 * NC), sizeof(double));
    int32_t* cnt = (int32_t*)calloc((size_t)NC, sizeof(int32_t));
    for (int64_t f = 0; f < NFT; ++f) {
        vst(est, fo[f], vadd(vld(est, fo[f]), vld(fC, f)));
        cnt[fo[f]] += 1;
    }
    for (int64_t f = 0; f < NIF; ++f) {
        vst(est, fn[f], vadd(vld(est, fn[f]), vld(fC, f)));
        cnt[fn[f]] += 1;
    }
    for (int64_t c = 0; c < NC; ++c) vst(est, c, vdiv(vld(est, c), (double)cnt[c]));
    double* cc = (double*)calloc((size_t)(3 * NC), sizeof(double));
    double* vol = out->V;
    memset(vol, 0, sizeof(double) * NC);
    for (int64_t f = 0; f < NFT; ++f) {
        const int32_t o = fo[f];
        v3 Cf = vld(fC, f), Sf = vld(fA, f), e = vld(est, o);
        double pv = vdot(Sf, vsub(Cf, e));
        v3 pc = vadd(vscale(3.0 / 4.0, Cf), vscale(1.0 / 4.0, e));
        vst(cc, o, vadd(vld(cc, o), vscale(pv, pc)));
        vol[o] += pv;
    }
    for (int64_t f = 0; f < NIF; ++f) {
        const int32_t o = fn[f];
        v3 Cf = vld(fC, f), Sf = vld(fA, f), e = vld(est, o);
        double pv = vdot(Sf, vsub(e, Cf));
        v3 pc = vadd(vscale(3.0 / 4.0, Cf), vscale(1.0 / 4.0, e));
        vst(cc, o, vadd(vld(cc, o), vscale(pv, pc)));
        vol[o] += pv;
    }
    int32_t bad = 0;
    for (int64_t c = 0; c < NC; ++c) {
        if (fabs(vol[c]) > 1.0e-300) vst(cc, c, vdiv(vld(cc, c), vol[c]));
        else vst(cc, c, vld(est, c));
        vol[c] *= (1.0 / 3.0);
        if (!(vol[c] > 0)) bad = 1;
    }
    if (out->C) memcpy(out->C, cc, sizeof(double) * 3 * NC);
    /* ---- internal faces: weights and non-orthogonal delta coefficients */
    for (int64_t f = 0; f < NIF; ++f) {
        const int32_t o = fo[f], nb = fn[f];
        v3 Sf = vld(fA, f), Cf = vld(fC, f), Co = vld(cc, o), Cn = vld(cc, nb);
        double mS = vmag(Sf);
        double dOwn = fabs(vdot(Sf, vsub(Cf, Co)));
        double dNei = fabs(vdot(Sf, vsub(Cn, Cf)));
        v3 d = vsub(Cn, Co);
        double nd = vdot(vdiv(Sf, mS), d), md = 0.05 * vmag(d);
        out->own[f] = o;
        out->nei[f] = nb;
        vst(out->Sf, f, Sf);
        if (out->Cf) vst(out->Cf, f, Cf);
        out->magSf[f] = mS;
        out->w[f] = dNei / (dOwn + dNei);
        out->delta[f] = 1.0 / (nd > md ? nd : md);
    }
    /* ---- boundary faces of the non-empty patches */
    for (int64_t b = 0; b < NBF; ++b) {
        const int64_t f = NIF + b;
        const int32_t o = fo[f];
        v3 Sf = vld(fA, f), Cf = vld(fC, f), Co = vld(cc, o);
        double mS = vmag(Sf);
        v3 n = vdiv(Sf, mS);
        v3 d = vscale(vdot(n, vsub(Cf, Co)), n);
        double nd = vdot(n, d), md = 0.05 * vmag(d);
        out->bcells[b] = o;
        vst(out->bSf, b, Sf);
        if (out->bCf) vst(out->bCf, b, Cf);
        out->bmagSf[b] = mS;
        out->bw[b] = 1.0;
        out->bdelta[b] = 1.0 / (nd > md ? nd : md);
    }
    if (!out->points) free(pts);
    free(fp);
    free(fo);
    free(fn);
    free(fC);
    free(fA);
    free(est);
    free(cnt);
    free(cc);
    return bad ? -2 : 0;
}
