/*
 * fvoracle.h -- CPU restatement of the FoamAdapter / NeoN finite-volume hot
 * path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of bench.py call it as the checker; the product library
 * never links or calls it.
 *
 * The reference arithmetic lives in the NeoN module (exasim-project/NeoN,
 * unpinned: FoamAdapter's cmake/CxxThirdParty.cmake:11-28 fetches `main`) and
 * in FoamAdapter's own kernels (src/algorithms/pressureVelocityCoupling.cpp,
 * include/FoamAdapter/datastructures/expression.hpp).  The loops here follow
 * the reference's Serial executor: face loops in ascending face order that
 * scatter into owner (+) and neighbour (-) cells, internal faces before
 * boundary faces.  Pinned against test/setup_operator/0/{divT_Serial,
 * gradT_Serial} (see tests/test_oracle_golden.py).  Everything else (upwind,
 * laplacian, assembly, CG iteration behaviour, PISO helpers) is a restatement
 * of the formulas the reference's call sites and tests imply; the reference
 * cannot be built here, so that part is "parity unpinned" against NeoN itself.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp (no FMA contraction; explicit fma()
 * where the algorithm says fma).
 */
#ifndef FVORACLE_H
#define FVORACLE_H
#include <stdint.h>

typedef struct or_mesh {
    int32_t n, nif, nbf, npatch;
    const double *V, *Sf, *magSf, *w, *delta;
    const int32_t *own, *nei;
    const int32_t* bcells;
    const double *bSf, *bmagSf, *bw, *bdelta;
    const int32_t* patch_offs;
} or_mesh;

typedef struct or_csr {
    int32_t n, nnz;
    const int32_t *row_offs, *col, *diag_off, *own_off, *nei_off;
} or_csr;

typedef struct or_term {
    int32_t kind, scheme;
    double coeff;
    const double* cell;
    const double* face;
} or_term;

typedef struct or_solver_cfg {
    double rel_tol, abs_tol;
    int32_t max_iter, precision;
    double inner_rel_tol;
    int32_t inner_max_iter, max_outer;
    int32_t method;      /* 0 CG, 1 BiCGStab (FP64 or mixed), 2 BiCG (FP64) */
    int32_t flags;       /* 2: rel_tol relative to ||b|| (Ginkgo ResidualNorm, baseline rhs_norm) */
    int32_t preconditioner;  /* 0 Jacobi, 2 ILU(0) (CG or BiCGStab, FP64) */
    int32_t pad;
} or_solver_cfg;

typedef struct or_solver_stats {
    double init_res_norm, final_res_norm;
    int32_t num_iter, num_outer, status, reserved;
} or_solver_stats;

/* Caller-allocated HOST arrays of a hex box (boxmesh.c); C, Cf, bCf and points may be NULL. */
typedef struct or_box_arrays {
    double *V, *C;                                   /* [n], [3n]            */
    int32_t *own, *nei;                              /* [nif]                */
    double *Sf, *Cf, *magSf, *w, *delta;             /* [3nif] [3nif] [nif]  */
    int32_t* bcells;                                 /* [nbf]                */
    double *bSf, *bCf, *bmagSf, *bw, *bdelta;        /* [3nbf] [3nbf] [nbf]  */
    int32_t* patch_offs;                             /* [npatch + 1]         */
    double* points;                                  /* [3 n_points]         */
} or_box_arrays;
/* sizes: [n_points, n_cells, n_ifaces, n_bfaces (flat, non-empty), n_patches, n_faces_total] */
int32_t or_box_sizes(int32_t nx, int32_t ny, int32_t nz, int32_t two_d, int64_t out[6]);
int32_t or_box_build(int32_t nx, int32_t ny, int32_t nz, double lx, double ly, double lz, double jitter,
                     uint64_t seed, int32_t two_d, or_box_arrays* out);

void or_set_threads(int32_t nthreads);
int32_t or_get_threads(void);

void or_bc_correct(const or_mesh* m, int32_t ncomp, const int32_t* patch_type, const double* ref,
                   const double* internal, double* boundary);
void or_interp_linear(const or_mesh* m, int32_t ncomp, const double* src, const double* src_b,
                      double* dst);
void or_interp_upwind(const or_mesh* m, int32_t ncomp, const double* flux, const double* src,
                      const double* src_b, double* dst);
void or_div(const or_mesh* m, int32_t scheme, int32_t ncomp, const double* flux,
            const double* phi, const double* phi_b, double coeff, double* out);
void or_grad(const or_mesh* m, const double* phi, const double* phi_b, double coeff, double* out);
void or_laplacian(const or_mesh* m, int32_t ncomp, const double* gamma, const double* phi,
                  const double* phi_b, double coeff, double* out);
void or_sngrad(const or_mesh* m, const double* phi, const double* phi_b, double* out);
/* non-orthogonal correction (corrected scheme); k = or_nonorth_vectors [nif*3] */
void or_nonorth_vectors(const or_mesh* m, const double* C, double* k);
void or_laplacian_corrected(const or_mesh* m, int32_t ncomp, const double* k, const double* gamma,
                            const double* phi, const double* phi_b, double coeff, double* out);
void or_sngrad_corrected(const or_mesh* m, const double* k, const double* phi, const double* phi_b, double* out);
void or_nonorth_flux(const or_mesh* m, int32_t ncomp, const double* k, const double* gamma, const double* phi,
                     const double* phi_b, double coeff, double* out);
void or_nonorth_rhs(const or_mesh* m, int32_t ncomp, const double* k, const double* gamma, const double* psi,
                    const double* psi_b, double coeff, double* rhs);
void or_advect_euler(const or_mesh* m, const double* flux, const double* T_old,
                     const double* T_old_b, double dt, const int32_t* patch_type,
                     const double* ref, double* T_new, double* T_new_b);

int32_t or_sparsity(const or_mesh* m, int32_t* row_offs, int32_t* col, int32_t* diag_off,
                    int32_t* own_off, int32_t* nei_off);
void or_assemble(const or_mesh* m, const or_csr* A, int32_t ncomp, const or_term* terms,
                 int32_t nterms, double dt, const int32_t* patch_type, const double* ref,
                 const double* psi_b, double* values, double* rhs, double* bmat, double* brhs);
void or_set_reference(const or_csr* A, double* values, double* rhs, int32_t ref_cell,
                      double ref_value);
void or_apply_operator(const or_csr* A, const double* values, const double* rhs, int32_t ncomp,
                       const double* x, double* out);

double or_dot_tree(int32_t n, const double* a, const double* b);
/* ILU(0) factors of A's pattern in CSR order (unit lower L below the diagonal,
 * U on and above it), and z = U^-1 L^-1 r (y: the forward result). */
void or_ilu_factor(const or_csr* A, const double* values, double* lu);
void or_ilu_apply(const or_csr* A, const double* lu, const double* r, double* y, double* z);

int32_t or_solve(const or_csr* A, const double* values, const double* rhs, double* x,
                 const or_solver_cfg* cfg, or_solver_stats* stats);

void or_rau_hbya(const or_mesh* m, const or_csr* A, const double* values, const double* rhs,
                 const double* U, double* rAU, double* HbyA);
void or_constrain_hbya(const or_mesh* m, const int32_t* patch_assignable, const double* U_b,
                       double* HbyA_b);
void or_flux_vec(const or_mesh* m, const double* U, const double* U_b, double* out);
void or_ddt_corr(const or_mesh* m, const int32_t* U_patch_type, const double* U, const double* U_b,
                 const double* phi_old, const double* rAUf, double dt, double* out);
void or_constrain_pressure(const or_mesh* m, const int32_t* patch_fixed_flux, const double* phiHbyA,
                           const double* U_b, const double* rAUf, double* p_ref);
void or_face_update(const or_mesh* m, const or_csr* A, const double* values, const double* bmat,
                    const double* brhs, const double* phiHbyA, const double* p, double* phi);
void or_velocity_update(const or_mesh* m, const double* HbyA, const double* rAU, const double* p,
                        const double* p_b, double* U);

#endif
