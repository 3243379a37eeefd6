/*
 * fvgb.h -- C ABI of the GB300 (sm_103a) finite-volume hot path.
 *
 * This is the drop-in boundary for the NeoN / FoamAdapter operator and DSL
 * calls that FoamAdapter makes on its finite-volume hot path.  Every entry
 * point takes plain pointers and sizes; field and matrix data live in device
 * memory owned by the caller unless the entry point says otherwise, and every
 * asynchronous call takes the CUDA stream it is ordered on (a cudaStream_t
 * passed as fvgb_stream; NULL is the legacy default stream).
 *
 * Conventions shared by every entry point
 *   - Labels are int32, values are IEEE binary64 (double) unless a name says
 *     otherwise.  Vector (Vec3) fields are stored as 3 doubles per cell,
 *     interleaved (x,y,z), the in-memory layout of NeoN::Vec3.
 *   - A volume field is two device arrays: `internal` [n_cells*ncomp] and
 *     `boundary` [n_bfaces*ncomp] (the flat boundary values of every
 *     non-empty patch, in patch order).  Empty patches hold zero faces.
 *   - A surface field is one device array of n_ifaces + n_bfaces entries:
 *     internal faces first, then the boundary faces patch by patch.
 *   - Explicit operators ACCUMULATE into the caller's output: out += result.
 *     With `coeff` the operator scaling (NeoN dsl::Coeff, a scalar here),
 *     the per-cell scaling is exactly  sum * (coeff / V[c]).
 *   - All calls return an fvgb_status; fvgb_last_error() gives the message of
 *     the most recent failure on the calling thread.
 *   - Handles are not thread safe; distinct handles on distinct streams are.
 */
#ifndef FVGB_H
#define FVGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum fvgb_status {
    FVGB_OK = 0,
    FVGB_ERR_INVALID_ARG = 1,   /* bad size, null pointer, malformed mesh     */
    FVGB_ERR_OOM = 2,           /* device allocation failed                    */
    FVGB_ERR_NOT_CONVERGED = 3, /* iteration cap reached before the criteria   */
    FVGB_ERR_BREAKDOWN = 4,     /* p.Ap == 0 or a non-finite scalar in a solve */
    FVGB_ERR_CUDA = 5,          /* any other CUDA runtime error                */
    FVGB_ERR_UNSUPPORTED = 6,   /* valid request this build does not implement */
    FVGB_ERR_BUDGET = 7,        /* serving: request exceeds the HBM budget     */
    FVGB_ERR_CANCELLED = 8      /* serving: request cancelled before it ran    */
} fvgb_status;

typedef void* fvgb_stream; /* cudaStream_t */

/* Human readable name of a status code (static storage). */
const char* fvgb_status_string(int status);
/* Message of the last failing call on this thread ("" if none). */
const char* fvgb_last_error(void);
/* ABI version, (major << 16) | minor. */
int32_t fvgb_abi_version(void);

/* -------------------------------------------------------------------- mesh */
/*
 * Host-side description of an unstructured finite-volume mesh, the array set
 * of NeoN::UnstructuredMesh + NeoN::BoundaryMesh as FoamAdapter builds it from
 * a Foam::fvMesh (reference: src/datastructures/meshAdapter.cpp:59-136).
 * All pointers are HOST pointers; fvgb_mesh_create copies what it needs.
 *   weights / nonorth_delta_coeffs: internal faces; boundary faces use
 *   bweights / bdelta_coeffs.  The laplacian and snGrad use
 *   nonorth_delta_coeffs (1 / max(n.d, 0.05|d|), OpenFOAM's uncorrected
 *   scheme coefficient).
 */
typedef struct fvgb_mesh_desc {
    int32_t n_cells;
    int32_t n_ifaces;          /* internal faces                          */
    int32_t n_bfaces;          /* faces of all non-empty patches          */
    int32_t n_patches;         /* non-empty patches                       */
    const double* cell_volumes;     /* [n_cells]                          */
    const double* cell_centres;     /* [n_cells*3]   (optional, may be NULL) */
    const int32_t* owner;           /* [n_ifaces]                         */
    const int32_t* neighbour;       /* [n_ifaces]                         */
    const double* face_areas;       /* Sf  [n_ifaces*3]                   */
    const double* mag_face_areas;   /* |Sf| [n_ifaces]                    */
    const double* weights;          /* [n_ifaces]                         */
    const double* delta_coeffs;     /* [n_ifaces]                         */
    const int32_t* bface_cells;     /* [n_bfaces]                         */
    const double* bface_areas;      /* [n_bfaces*3]                       */
    const double* bmag_face_areas;  /* [n_bfaces]                         */
    const double* bweights;         /* [n_bfaces]                         */
    const double* bdelta_coeffs;    /* [n_bfaces]                         */
    const int32_t* patch_offsets;   /* [n_patches+1], patch p = [off[p], off[p+1]) */
} fvgb_mesh_desc;

typedef struct fvgb_mesh fvgb_mesh;

/* Validate, upload and index a mesh: builds the cell->face gather lists
 * (ascending face order per cell), the CSR/sliced-ELL matrix pattern with
 * owner/neighbour/diagonal slot maps (NeoN la::SparsityPattern,
 * test/test_sparsityPattern.cpp:36-62) on the device. Synchronous. */
fvgb_status fvgb_mesh_create(const fvgb_mesh_desc* desc, fvgb_mesh** out);
fvgb_status fvgb_mesh_destroy(fvgb_mesh* mesh);
/* Sizes: n_cells, n_ifaces, n_bfaces, n_patches, nnz (= n_cells + 2*n_ifaces). */
fvgb_status fvgb_mesh_sizes(const fvgb_mesh* mesh, int64_t out[5]);
/* Device bytes held by the mesh handle (geometry + index structures). */
int64_t fvgb_mesh_device_bytes(const fvgb_mesh* mesh);

/* Build ONE device mesh holding `nboxes` unjittered 3-D hex boxes packed
 * block-diagonally, entirely on the device (no host geometry, no upload of
 * mesh arrays).  Box q's cells are rows [row_ranges[2q], row_ranges[2q+1])
 * (HOST output array [2*nboxes]); boxes start at multiples of 32 cells and the
 * cells between them are isolated placeholders.  Patches: xmin, xmax, ymin,
 * ymax, zmin, zmax, each grouped by box.  Geometry is analytic (weights 0.5,
 * delta 1/h, boundary delta 2/h).  Such a mesh keeps no host CSR copy:
 * fvgb_mesh_sparsity and the values part of fvgb_ls_export return
 * FVGB_ERR_UNSUPPORTED.  No counterpart in the reference (its meshes come
 * from OpenFOAM); used by the serving loop, which admits many boxes per second. */
struct fvgb_box_spec;
fvgb_status fvgb_mesh_create_boxes(const struct fvgb_box_spec* specs, int32_t nboxes, fvgb_mesh** out,
                                   int32_t* row_ranges, fvgb_stream stream);

/* CSR sparsity pattern in NeoN's layout, copied to HOST arrays:
 * row_offs[n+1], col_idxs[nnz], diag_offset[n], owner_offset[n_ifaces],
 * neighbour_offset[n_ifaces] (offsets relative to the row start).
 * Reference: la::SparsityPattern (expression.hpp:35, test_sparsityPattern.cpp:36-62). */
fvgb_status fvgb_mesh_sparsity(const fvgb_mesh* mesh, int32_t* row_offs, int32_t* col_idxs,
                               int32_t* diag_offset, int32_t* owner_offset,
                               int32_t* neighbour_offset);

/* ------------------------------------------------------- boundary conditions */
typedef enum fvgb_bc_type {
    FVGB_BC_CALCULATED = 0,     /* boundary values are whatever was written      */
    FVGB_BC_FIXED_VALUE = 1,    /* value = ref (noSlip is fixedValue 0)          */
    FVGB_BC_FIXED_GRADIENT = 2  /* value = internal + ref/deltaCoeff; zeroGradient = ref 0 */
} fvgb_bc_type;

/* Boundary condition of a volume field: a type per patch (host array) and a
 * per-boundary-face reference (device array [n_bfaces*ncomp]: the fixed value
 * or the fixed gradient).  Reference semantics: readers.hpp:43-95. */
typedef struct fvgb_bc {
    const int32_t* patch_type; /* HOST [n_patches]                        */
    const double* ref;         /* DEVICE [n_bfaces*ncomp] (may be NULL when every patch is CALCULATED) */
} fvgb_bc;

/* VolumeField::correctBoundaryConditions: recompute boundary values. */
fvgb_status fvgb_bc_correct(const fvgb_mesh* mesh, int32_t ncomp, const fvgb_bc* bc,
                            const double* internal, double* boundary, fvgb_stream stream);

/* ------------------------------------------------------- explicit operators */
typedef enum fvgb_scheme {
    FVGB_SCHEME_LINEAR = 0,
    FVGB_SCHEME_UPWIND = 1,
    FVGB_SCHEME_CORRECTED = 2  /* laplacian: Gauss linear corrected (non-orthogonal correction) */
} fvgb_scheme;

/* SurfaceInterpolation linear (NeoN; reference call sites neoIcoFoam.cpp:118-124,
 * test_operators.cpp:52-58):  dst_f = w_f*(src_P - src_N) + src_N on internal
 * faces, dst_b = boundary value.  dst [(n_ifaces+n_bfaces)*ncomp] is overwritten. */
fvgb_status fvgb_interp_linear(const fvgb_mesh* mesh, int32_t ncomp, const double* src,
                               const double* src_b, double* dst, fvgb_stream stream);
/* SurfaceInterpolation upwind: dst_f = flux_f >= 0 ? src_P : src_N; dst_b = boundary value. */
fvgb_status fvgb_interp_upwind(const fvgb_mesh* mesh, int32_t ncomp, const double* flux,
                               const double* src, const double* src_b, double* dst,
                               fvgb_stream stream);
/* GaussGreenDiv::div(out, faceFlux, phi, coeff) (bench_explicitOperators.cpp:114-115):
 * out_P += (sum over faces of P in ascending face order of +-flux_f*phi_f) * (coeff/V_P),
 * + for owner and boundary faces, - for neighbour faces. */
fvgb_status fvgb_div_explicit(const fvgb_mesh* mesh, int32_t scheme, int32_t ncomp,
                              const double* flux, const double* phi, const double* phi_b,
                              double coeff, double* out, fvgb_stream stream);
/* GaussGreenGrad::grad(T, coeff, out) (test_operators.cpp:72): linear face values,
 * out_P[3] += (sum +-Sf*T_f) * (coeff/V_P). */
fvgb_status fvgb_grad(const fvgb_mesh* mesh, const double* phi, const double* phi_b,
                      double coeff, double* out, fvgb_stream stream);
/* GaussGreenLaplacian::laplacian(out, gamma, T, coeff), uncorrected
 * (bench_explicitOperators.cpp:212-213): flux_f = gamma_f*(|Sf|*delta_f)*(T_N - T_P),
 * boundary flux_b = gamma_b*(|Sf|*delta_b)*(T_b - T_P); out_P += (sum +-flux)*(coeff/V_P). */
fvgb_status fvgb_laplacian_explicit(const fvgb_mesh* mesh, int32_t ncomp, const double* gamma,
                                    const double* phi, const double* phi_b, double coeff,
                                    double* out, fvgb_stream stream);
/* The same with the `Gauss linear corrected` scheme (OpenFOAM's correctedSnGrad,
 * test/setup_stencil3D/system/fvSchemes:43): flux_f = fma(gamma_f*(|Sf|*delta_f),
 * T_N - T_P, (gamma_f*|Sf|)*(k_f . gT_f)), where k_f = Sf/|Sf| - (C_N - C_P)*delta_f
 * is the face's non-orthogonal correction vector, gT_f = fma(w_f, g_P - g_N, g_N)
 * per direction, k . gT = fma(k_z, gT_z, fma(k_y, gT_y, k_x*gT_x)) and g the Gauss
 * linear gradient of T (as fvgb_grad, per component); boundary faces as
 * uncorrected (with k = 0 the flux is exactly the uncorrected one).  Needs a mesh created with cell centres (FVGB_ERR_INVALID_ARG
 * otherwise).  Takes stream-ordered scratch memory for the gradient. */
fvgb_status fvgb_laplacian_explicit_corrected(const fvgb_mesh* mesh, int32_t ncomp, const double* gamma,
                                              const double* phi, const double* phi_b, double coeff,
                                              double* out, fvgb_stream stream);
/* faceFluxCorrection of a corrected laplacian: out_f += coeff*(gamma_f*|Sf|)*(k_f . gT_f)
 * on the internal faces [n_ifaces*ncomp] (boundary faces carry none).  The flux a
 * pressure equation's solution adds to the face velocity (pEqn.flux()). */
fvgb_status fvgb_nonorth_flux(const fvgb_mesh* mesh, int32_t ncomp, const double* gamma, const double* phi,
                              const double* phi_b, double coeff, double* out, fvgb_stream stream);
/* FaceNormalGradient uncorrected (bench_explicitOperators.cpp:455-479):
 * out_f = delta_f*(T_N - T_P), out_b = delta_b*(T_b - T_P); overwritten. */
fvgb_status fvgb_sngrad(const fvgb_mesh* mesh, const double* phi, const double* phi_b,
                        double* out, fvgb_stream stream);
/* FaceNormalGradient corrected: out_f = fma(delta_f, T_N - T_P, k_f . gT_f) (as above),
 * boundary faces delta_b*(T_b - T_P); overwritten. */
fvgb_status fvgb_sngrad_corrected(const fvgb_mesh* mesh, const double* phi, const double* phi_b,
                                  double* out, fvgb_stream stream);
/* Fused explicit step of  ddt(T) + div(phi, T) = 0, Gauss upwind, forward Euler
 * (test_advection.cpp:116-170): T_new_P = T_old_P - dt*(div_P) with div_P the
 * fvgb_div_explicit value for coeff 1; then the boundary values of T_new are
 * corrected with `bc` (bit-identical to the three unfused calls). */
fvgb_status fvgb_advect_euler_step(const fvgb_mesh* mesh, const double* flux,
                                   const double* T_old, const double* T_old_b, double dt,
                                   const fvgb_bc* bc, double* T_new, double* T_new_b,
                                   fvgb_stream stream);
/* nsteps of fvgb_advect_euler_step in place on (T, T_b), the time loop of
 * test_advection.cpp:116-170 in one call; work/work_b (same sizes) are the other
 * half of the ping-pong.  Meshes of at most 65536 cells take one launch of a
 * one-pass step kernel per step (no face buffer), larger ones the two-pass step
 * of fvgb_advect_euler_step; both give the bits of nsteps single calls. */
fvgb_status fvgb_advect_euler_steps(const fvgb_mesh* mesh, const double* flux, double* T, double* T_b,
                                    double dt, const fvgb_bc* bc, int32_t nsteps, double* work,
                                    double* work_b, fvgb_stream stream);

/* The face-pass tile of the explicit operators: how many faces one thread of a
 * face pass handles (2, 4 or 8; 0 restores the default 4).  Every face is
 * computed alone, so every tile gives the same bits. */
fvgb_status fvgb_mesh_face_tile(fvgb_mesh* mesh, int32_t tile);
/* The autotuner of that tile: times the grad and upwind-div face passes of this
 * mesh with each tile on scratch fields, sets the fastest and records it in the
 * tuning cache under the mesh's shape (face count, GPU), from which a later mesh
 * of that shape takes it untimed.  *tile = the tile set; ms[3] (optional) = the
 * times of tiles 2, 4, 8 (0 when taken from the cache).  Synchronises `stream`. */
fvgb_status fvgb_explicit_tune(fvgb_mesh* mesh, fvgb_stream stream, int32_t* tile, float* ms);

/* ----------------------------------------------- linear system and assembly */
typedef struct fvgb_ls fvgb_ls;

typedef enum fvgb_term_kind {
    FVGB_TERM_DDT = 0,             /* implicit Euler ddt  (DdtOperator)                */
    FVGB_TERM_LAPLACIAN = 1,       /* implicit laplacian(gamma, psi); scheme CORRECTED adds
                                      the non-orthogonal correction of `cell` (the current
                                      psi, boundary values psi_b) to the rhs:
                                      b -= coeff*sum_f(+-(gamma_f*|Sf|)*(k_f . gT_f)), after
                                      all terms, in term order                          */
    FVGB_TERM_DIV = 2,             /* implicit div(flux, psi), linear or upwind        */
    FVGB_TERM_SOURCE = 3,          /* implicit source: diag += coeff*s_P*V_P           */
    FVGB_TERM_EXPLICIT = 4,        /* rhs -= coeff*E_P (E already volume integrated)   */
    FVGB_TERM_DIV_FLUX = 5,        /* rhs -= coeff*sum_f(+-F_f): explicit div of a face
                                      flux, volume integrated (dsl::exp::div(phi))     */
    FVGB_TERM_DIV_EXPLICIT = 6     /* rhs -= coeff*sum_f(+-F_f*psi_f) with psi_f from the
                                      term's cell field (`cell`, boundary values psi_b),
                                      linear or upwind: dsl::exp::div(phi, psi), volume
                                      integrated (IMEX convection)                     */
} fvgb_term_kind;

/* One operator of a dsl::Expression. The expression is
 *   sum_t coeff_t * op_t(psi) = 0,
 * each implicit op_t(psi) = A_t psi - b_t, so A = sum coeff_t A_t and
 * b = sum coeff_t b_t (EXPLICIT: b -= coeff*E).  Terms are applied in array order. */
typedef struct fvgb_term {
    int32_t kind;
    int32_t scheme;        /* DIV: FVGB_SCHEME_LINEAR or FVGB_SCHEME_UPWIND;
                              LAPLACIAN: 0 (uncorrected) or FVGB_SCHEME_CORRECTED        */
    double coeff;          /* operator scaling                                        */
    const double* cell;    /* DDT: old-time psi [n*ncomp]; SOURCE: s [n] or NULL (=1);
                              EXPLICIT: E [n*ncomp]; DIV_EXPLICIT: the convected field  */
    const double* face;    /* LAPLACIAN: gamma [nIF+nBF]; DIV, DIV_FLUX, DIV_EXPLICIT:
                              face flux [nIF+nBF]                                       */
} fvgb_term;

/* LinearSystem on the mesh pattern: values[nnz], rhs[n*ncomp],
 * boundaryCoefficients {matrixValues[nBF], rhsValues[nBF*ncomp]}
 * (reference: expression.hpp:36-39, pressureVelocityCoupling.cpp:180-185).
 * Vector systems (ncomp 3) share one scalar coefficient per entry. */
fvgb_status fvgb_ls_create(const fvgb_mesh* mesh, int32_t ncomp, fvgb_ls** out);
fvgb_status fvgb_ls_destroy(fvgb_ls* ls);
/* Assemble all terms from zero (PDESolver::assemble, expression.hpp:69-73).
 * psi_bc / psi_b: boundary condition and current boundary values of psi. */
fvgb_status fvgb_assemble(fvgb_ls* ls, const fvgb_term* terms, int32_t nterms, double dt,
                          const fvgb_bc* psi_bc, const double* psi_b, fvgb_stream stream);
/* The same assembly with the matrix kept (no counterpart in the reference,
 * which reassembles every step): only rhs and the boundary coefficients are
 * recomputed.  Valid when the implicit terms, dt, mesh and boundary types are
 * those of the last fvgb_assemble (e.g. a time step whose implicit part does
 * not change); the result is then identical to a full assembly.  A solve that
 * follows reuses its FP32 copy of the unchanged matrix. */
fvgb_status fvgb_assemble_rhs(fvgb_ls* ls, const fvgb_term* terms, int32_t nterms, double dt,
                              const fvgb_bc* psi_bc, const double* psi_b, fvgb_stream stream);
/* PDESolver::SetReference (expression.hpp:102-111): rhs[r] += a_rr*value; a_rr += a_rr. */
fvgb_status fvgb_set_reference(fvgb_ls* ls, int32_t ref_cell, double ref_value,
                               fvgb_stream stream);
/* applyOperator / la::computeResidual (expression.hpp:204-220): out = A x - b. */
fvgb_status fvgb_apply_operator(const fvgb_ls* ls, const double* x, double* out,
                                fvgb_stream stream);
/* diag (expression.hpp:181-201): out[n] = a_PP. */
fvgb_status fvgb_ls_diag(const fvgb_ls* ls, double* out, fvgb_stream stream);
/* Copy the system out in NeoN's CSR order: values[nnz], rhs[n*ncomp],
 * bmatrix[nBF], brhs[nBF*ncomp] (DEVICE destination pointers, any may be NULL). */
fvgb_status fvgb_ls_export(const fvgb_ls* ls, double* values, double* rhs, double* bmatrix,
                           double* brhs, fvgb_stream stream);

/* ------------------------------------------------------------------- solve */
typedef enum fvgb_precision {
    FVGB_PREC_FP64 = 0,      /* Jacobi-PCG in FP64 (Ginkgo solver::Cg + Jacobi, block 1)        */
    FVGB_PREC_MIXED_IR = 1   /* FP32 inner CG on the Jacobi-scaled system inside FP64
                                iterative refinement: FP64 b-Ax, update and convergence test  */
} fvgb_precision;

/* Stopping criteria of fvSolution.cpp:106-142: relative (to the initial residual
 * norm) and absolute residual norm, iteration cap (default 1000). 0 disables a
 * tolerance.  The residual is the unpreconditioned r = b - A x, 2-norm. */
typedef struct fvgb_solver_cfg {
    double rel_tol;
    double abs_tol;
    int32_t max_iter;          /* FP64: CG iterations; MIXED_IR: total inner iterations */
    int32_t precision;
    double inner_rel_tol;      /* MIXED_IR: residual reduction asked of each inner solve */
    int32_t inner_max_iter;    /* MIXED_IR: inner iteration cap per refinement step    */
    int32_t max_outer;         /* MIXED_IR: refinement step cap                        */
    int32_t kernel_mode;       /* 0 automatic, 1 graph of kernels, 2 one persistent
                                  cooperative kernel (FP64 single case), 3 host-driven
                                  loop (FP64; blocks the caller); same results          */
    int32_t flags;             /* FVGB_SOLVE_NO_TUNE: default kernel variants, no timing
                                  at the first solve (the timing synchronises the device);
                                  FVGB_SOLVE_RHS_BASELINE: rel_tol is relative to ||b||,
                                  Ginkgo's ResidualNorm with its default baseline
                                  rhs_norm (the reference's gko/config.bj.json), not to
                                  the initial residual (Jacobi CG and BiCGStab) */
    int32_t method;            /* FVGB_SOLVER_CG (Ginkgo Cg), FVGB_SOLVER_BICGSTAB
                                  (Ginkgo Bicgstab, fvSolution.cpp:25-26: nonsymmetric
                                  systems; graph path; MIXED_IR: FP32 inner BiCGStab,
                                  restarted every refinement step), FVGB_SOLVER_BICG
                                  (Ginkgo Bicg, OpenFOAM's PBiCG, fvSolution.cpp:24:
                                  shadow residual driven by A^T; FP64, graph path) or
                                  FVGB_SOLVER_MULTIGRID (Ginkgo Multigrid as the solver,
                                  OpenFOAM's GAMG, fvSolution.cpp:27: x += V(b - A x)
                                  with the multigrid preconditioner's V-cycle until the
                                  criteria hold; num_iter counts V-cycles; single
                                  systems, fvgb_solve / fvgb_solve_async only;
                                  `preconditioner` is not used; with FVGB_PREC_MIXED_IR
                                  the V-cycle runs in FP32, the residuals in FP64)    */
    int32_t preconditioner;    /* FVGB_PRECOND_JACOBI (Ginkgo Jacobi, block size 1) or
                                  FVGB_PRECOND_MULTIGRID (Ginkgo Multigrid with PGM
                                  aggregation as tutorials/cylinder2D/system/gko/
                                  config.mg.json selects it; CG, single systems,
                                  fvgb_solve / fvgb_solve_async only; with
                                  FVGB_PREC_MIXED_IR the V-cycle runs in FP32 inside
                                  the FP64 CG) or FVGB_PRECOND_ILU (Ginkgo Ilu with a
                                  ParIlu factorization, OpenFOAM's DILU,
                                  fvSolution.cpp:56-63: the exact ILU(0) factors,
                                  formed level by level in every solve, and
                                  triangular solves of one launch each, rows in
                                  level order; CG or BiCGStab, FP64,
                                  single systems, fvgb_solve / fvgb_solve_async)       */
} fvgb_solver_cfg;
enum { FVGB_SOLVE_NO_TUNE = 1, FVGB_SOLVE_RHS_BASELINE = 2 };
enum { FVGB_SOLVER_CG = 0, FVGB_SOLVER_BICGSTAB = 1, FVGB_SOLVER_BICG = 2, FVGB_SOLVER_MULTIGRID = 3 };
enum { FVGB_PRECOND_JACOBI = 0, FVGB_PRECOND_MULTIGRID = 1, FVGB_PRECOND_ILU = 2 };

/* SolverStats {initResNorm, finalResNorm, numIter} (expression.hpp:155-158). */
typedef struct fvgb_solver_stats {
    double init_res_norm;
    double final_res_norm;
    int32_t num_iter;          /* FP64: CG iterations; MIXED_IR: total inner iterations */
    int32_t num_outer;         /* MIXED_IR refinement steps (0 for FP64)               */
    int32_t status;            /* FVGB_OK, FVGB_ERR_NOT_CONVERGED or FVGB_ERR_BREAKDOWN */
    int32_t reserved;
} fvgb_solver_stats;

/* dsl::solve / PDESolver::solve: solve A x = b in place (x holds the initial
 * guess).  Enqueues one CUDA graph (device-side while loop, no host round
 * trips per iteration) and waits for it; *stats is filled on return.
 * Returns FVGB_OK, FVGB_ERR_NOT_CONVERGED or FVGB_ERR_BREAKDOWN. */
fvgb_status fvgb_solve(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg,
                       fvgb_solver_stats* stats, fvgb_stream stream);
/* Asynchronous form: stats are written to DEVICE memory stats_dev when the
 * stream reaches the end of the solve; nothing is waited for. */
fvgb_status fvgb_solve_async(fvgb_ls* ls, double* x, const fvgb_solver_cfg* cfg,
                             fvgb_solver_stats* stats_dev, fvgb_stream stream);

/* Batched solve of independent cases packed into one linear system (a
 * block-diagonal matrix, e.g. the concatenated meshes of many cases): case c
 * owns rows [row_ranges[2c], row_ranges[2c+1]) (HOST array; cases in row order,
 * not overlapping); rows outside every case are left untouched.  One launch per kernel serves
 * every case, each case keeps its own CG scalars and stops on its own
 * criteria, and a case's iterates are bit-identical to solving it alone.
 * No counterpart in the reference, which solves one case per call. */
typedef struct fvgb_batch fvgb_batch;
fvgb_status fvgb_batch_create(fvgb_ls* ls, int32_t ncases, const int32_t* row_ranges, fvgb_batch** out);
fvgb_status fvgb_batch_destroy(fvgb_batch* batch);
/* stats: HOST array [ncases]; returns the worst case status. */
fvgb_status fvgb_batch_solve(fvgb_batch* batch, double* x, const fvgb_solver_cfg* cfg,
                             fvgb_solver_stats* stats, fvgb_stream stream);
/* stats_dev: DEVICE array [ncases] (may be NULL); nothing is waited for. */
fvgb_status fvgb_batch_solve_async(fvgb_batch* batch, double* x, const fvgb_solver_cfg* cfg,
                                   fvgb_solver_stats* stats_dev, fvgb_stream stream);

/* One implicit time step as one CUDA graph (no counterpart in the reference;
 * the steps of dsl::solve, expression.hpp:143-153, captured once): copy psi to
 * psi_old (skipped when psi_old is NULL; a DDT term's cell field is psi_old),
 * assemble `terms` with `bc`, solve every case of `batch` (or the whole system
 * when batch is NULL) into psi with `cfg` (graph path; kernel_mode 3 is not
 * allowed), update psi_b from psi.  The graph keeps the pointers it was created
 * with; per-case statistics of every launch go to stats_dev (device, may be
 * NULL).  fvgb_step_launch enqueues it on a stream. */
typedef struct fvgb_step fvgb_step;
fvgb_status fvgb_step_create(fvgb_ls* ls, fvgb_batch* batch, const fvgb_term* terms, int32_t nterms, double dt,
                             const fvgb_bc* bc, double* psi, double* psi_b, double* psi_old,
                             const fvgb_solver_cfg* cfg, fvgb_solver_stats* stats_dev, fvgb_step** out);
fvgb_status fvgb_step_launch(fvgb_step* step, fvgb_stream stream);
fvgb_status fvgb_step_destroy(fvgb_step* step);

/* Autotuner of the CG kernels (no counterpart in the reference): at the first
 * solve of a system with at least 2^18 rows the SpMV and update kernels of the
 * FP64 and mixed solves are timed in four launch-bound variants (at least 2, 4,
 * 6, 8 resident blocks per SM) and the solve graphs use the fastest; all
 * variants give the same bits.  chosen[4]: the minimum-blocks value in use for
 * [FP64 SpMV, FP64 update, FP32 SpMV, FP32 update]; ms[16]: the measured median
 * milliseconds per kind and variant (0 where not measured).  force[4] (or NULL):
 * a variant index 0..3 per kind, -1 to keep the tuned choice. */
fvgb_status fvgb_solve_tuning(fvgb_ls* ls, const int32_t* force, int32_t* chosen, float* ms);
/* The same for the solver of a batch (its variants are timed when the packed
 * system has at least 2^18 rows). */
fvgb_status fvgb_batch_tuning(fvgb_batch* batch, const int32_t* force, int32_t* chosen, float* ms);
/* The autotuner's cache (no counterpart in the reference): every measured choice
 * is kept for the process, keyed by the system's shape (rows to the nearest power
 * of two, stored slots per row, 16- or 32-bit column offsets, the GPU's compute
 * capability and SM count); a later system of that shape -- also one solved with
 * FVGB_SOLVE_NO_TUNE, as served requests are -- uses the cached choice and is not
 * timed (ms reports 0 for it).  The cache can be written to and merged from a JSON
 * file; the environment variable FVGB_TUNING_CACHE names a file that is read at
 * the first lookup and rewritten after every new measurement. */
fvgb_status fvgb_tuning_cache_load(const char* path);
fvgb_status fvgb_tuning_cache_save(const char* path);
fvgb_status fvgb_tuning_cache_clear(void);
int32_t fvgb_tuning_cache_size(void);
/* Measurement aid (no reference counterpart): runs the FP64 CG init and
 * `iters` iterations outside the graph on a private copy of x0, with CUDA
 * events around each kernel; ms_out[4] = mean milliseconds of
 * [spmv + p.Ap, x/r update + r.z, direction update, init].  Synchronous. */
fvgb_status fvgb_solve_kernel_times(fvgb_ls* ls, const double* x0, int32_t iters, double* ms_out,
                                    fvgb_stream stream);

/* Multigrid (cfg->preconditioner = FVGB_PRECOND_MULTIGRID): the hierarchy is
 * built at the first such solve of a system (PGM aggregation and Galerkin
 * pattern on the host from that matrix; it synchronises the stream and cannot
 * be stream-captured), and its values are recomputed on the device whenever
 * the matrix changed.  fvgb_amg_apply: z = M r, one V-cycle of the current
 * matrix (synchronous; a measurement and test aid).  fvgb_amg_info: number of
 * levels and rows / nonzeros per level (cap entries of each). */
fvgb_status fvgb_amg_apply(fvgb_ls* ls, const double* r, double* z, fvgb_stream stream);
fvgb_status fvgb_amg_info(fvgb_ls* ls, int32_t* nlevels, int32_t* rows, int64_t* nnz, int32_t cap);
/* The aggregation step of the multigrid setup on a HOST CSR matrix: agg[n]
 * receives the aggregate of every row, *n_coarse their number.  Strength
 * |a_ij|; up to 15 rounds of mutual strongest-neighbour pairing (ties: lower
 * index) until at most 5% of the rows are left; left-over rows join their
 * strongest aggregated neighbour or stay alone; aggregates are numbered by
 * their lowest row. */
fvgb_status fvgb_pgm_aggregate(int32_t n, const int32_t* row_offs, const int32_t* cols, const double* values,
                               int32_t* agg, int32_t* n_coarse);

/* FP64 Jacobi-CG that allocates nothing.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc (a solver embedded in a host
 * application that owns the device memory under a fixed budget, or code that
 * must not let an allocation synchronize the device).  The system is given in
 * NeoN's CSR layout in caller-owned device memory (row_offs[n+1],
 * col_idxs[nnz], diag_offset[n] relative to the row start, values[nnz],
 * rhs[n]); x[n] is the initial guess and the solution.  Work vectors live in a
 * fixed device array inside the library (about 8.2 MiB, held by every GPU that
 * loads the library until the process exits), so n is limited to 262,144 rows
 * (larger n: FVGB_ERR_INVALID_ARG).  All calls on a device share that array:
 * calls that overlap on the GPU race.  The first call on a device looks up the
 * array's address.  Synchronous (it reads the solver state back between chunks
 * of iterations): it must not be called on a stream that is being captured and
 * refuses one with FVGB_ERR_UNSUPPORTED.  Same criteria and the same iterates
 * as fvgb_solve (FP64). */
fvgb_status fvgb_pcg_csr_noalloc(int32_t n, const int32_t* row_offs, const int32_t* col_idxs,
                                 const int32_t* diag_offset, const double* values,
                                 const double* rhs, double* x, const fvgb_solver_cfg* cfg,
                                 fvgb_solver_stats* stats, fvgb_stream stream);

/* ------------------------------------------------- pressure-velocity (PISO) */
/* computeRAUandHByA (pressureVelocityCoupling.cpp:65-128) on an assembled vector
 * system: rAU_P = V_P / a_PP; HbyA_P = (b_P - sum_{faces asc} a_Pj U_j) * (rAU_P / V_P).
 * A deterministic cell gather in ascending face order replaces the atomics. */
fvgb_status fvgb_piso_rau_hbya(const fvgb_ls* ueqn, const double* U, double* rAU,
                               double* HbyA, fvgb_stream stream);
/* constrainHbyA (pressureVelocityCoupling.cpp:14-36): HbyA_b = U_b on every patch
 * whose U condition is not assignable (patch_assignable[p] == 0, HOST array). */
fvgb_status fvgb_piso_constrain_hbya(const fvgb_mesh* mesh, const int32_t* patch_assignable,
                                     const double* U_b, double* HbyA_b, fvgb_stream stream);
/* flux(volVectorField) (pressureVelocityCoupling.cpp:215-267):
 * F_f = Sf . (w (U_P - U_N) + U_N); F_b = Sf_b . U_b.  out [nIF+nBF] overwritten. */
fvgb_status fvgb_flux_vec(const fvgb_mesh* mesh, const double* U, const double* U_b,
                          double* out, fvgb_stream stream);
/* updateFaceVelocity (pressureVelocityCoupling.cpp:131-197):
 * phi_f = phiHbyA_f - (a_NP p_N - a_PN p_P); phi_b = phiHbyA_b - (brhs_b - bmat_b p_P). */
fvgb_status fvgb_piso_face_update(const fvgb_ls* peqn, const double* phiHbyA, const double* p,
                                  double* phi, fvgb_stream stream);
/* updateVelocity (pressureVelocityCoupling.cpp:199-213): U = HbyA - rAU * grad(p). */
fvgb_status fvgb_piso_velocity_update(const fvgb_mesh* mesh, const double* HbyA,
                                      const double* rAU, const double* p, const double* p_b,
                                      double* U, fvgb_stream stream);
/* The two steps the reference's PISO leaves as TODOs (neoIcoFoam.cpp:127-137),
 * with OpenFOAM's semantics.  ddtCorr: phiHbyA += fvc::interpolate(rAU) *
 * fvc::ddtCorr(U, phi) for Euler ddt,
 *   phiHbyA_f += rAUf_f*((c_f/dt)*d_f),  d_f = phi_old_f - Sf_f . U_old_f,
 *   c_f = 1 - min(|d_f| / (|phi_old_f| + 1e-15), 1),
 * U_old_f linearly interpolated (boundary faces: U_old_b), c = 0 on the faces of
 * patches whose U_patch_type is FVGB_BC_FIXED_VALUE; rAUf [n_ifaces+n_bfaces]. */
fvgb_status fvgb_piso_ddt_corr(const fvgb_mesh* mesh, const int32_t* U_patch_type, const double* U_old,
                               const double* U_old_b, const double* phi_old, const double* rAUf, double dt,
                               double* phiHbyA, fvgb_stream stream);
/* constrainPressure: on the patches flagged in patch_fixed_flux (host
 * [n_patches]; fixedFluxPressure, a FIXED_GRADIENT patch of p) the gradient
 * becomes p_ref_b = (phiHbyA_b - Sf_b . U_b) / (|Sf_b| * rAUf_b); other
 * patches' entries of p_ref are left as they are. */
fvgb_status fvgb_piso_constrain_pressure(const fvgb_mesh* mesh, const int32_t* patch_fixed_flux,
                                         const double* phiHbyA, const double* U_b, const double* rAUf,
                                         double* p_ref, fvgb_stream stream);

/* ----------------------------------------------------------------- serving */
/* A serving loop for scalar advection-diffusion solves (no counterpart in the
 * reference): requests arrive at any time, are admitted in arrival order as
 * the HBM budget allows, keep their mesh, fields, matrix and solver state on
 * the device while they run, and every tick advances all active requests by
 * one implicit step, overlapping their work on a pool of CUDA streams.
 * A request's result does not depend on what else runs (each request executes
 * exactly its own computation).  The loop runs on its own host thread. */
typedef struct fvgb_server fvgb_server;
typedef struct fvgb_server_cfg {
    int64_t budget_bytes;      /* device bytes requests may hold at once              */
    int32_t n_streams;         /* CUDA streams the active requests are spread over    */
    int32_t max_active;        /* cap on concurrently active requests                 */
} fvgb_server_cfg;
/* One request: the unit box [0,1]^3 with nx*ny*nz cells, a uniform velocity U,
 * diffusivity D, `steps` implicit steps of  ddt(T) + div(phi,T) - laplacian(D,T) = 0
 * (explicit upwind convection, implicit diffusion, zero-gradient walls, initial
 * Gaussian blob at the centre, or T_init); dt <= 0 picks 0.5*h/|U|.  T_out:
 * optional HOST buffer [nx*ny*nz] that receives the final field.  T_init:
 * optional HOST array [nx*ny*nz], the initial field instead of the blob; like
 * T_out it must stay valid until the request's result is reported. */
enum { FVGB_SERVE_REASSEMBLE = 1 };
typedef struct fvgb_serve_request {
    int32_t nx, ny, nz, steps;
    double U[3];
    double D;
    double dt;
    int32_t precision;         /* FVGB_PREC_FP64 or FVGB_PREC_MIXED_IR                */
    int32_t kernel_mode;       /* fvgb_solver_cfg.kernel_mode of every solve; 0 picks
                                  the graph path (requests overlap on the device)     */
    int32_t flags;             /* FVGB_SERVE_REASSEMBLE: the reference's step pattern
                                  (dsl::solve): a copy of the old-time field and the
                                  whole system assembled every step; otherwise the
                                  matrix is assembled once, each later step assembles
                                  only the rhs and reads the old field in place (same
                                  results)                                            */
    int32_t reserved;
    double* T_out;
    const double* T_init;
} fvgb_serve_request;
typedef struct fvgb_serve_result {
    int64_t id;
    int32_t status;            /* FVGB_OK, a solver status, FVGB_ERR_CANCELLED        */
    int32_t steps_done;
    int32_t total_iters;
    int32_t reserved;
    double submit_s, start_s, finish_s;   /* seconds since the server started        */
    int64_t device_bytes;      /* the budget the request held                         */
} fvgb_serve_result;
fvgb_status fvgb_server_create(const fvgb_server_cfg* cfg, fvgb_server** out);
/* Thread safe; FVGB_ERR_BUDGET if the request alone exceeds the budget. */
fvgb_status fvgb_server_submit(fvgb_server* server, const fvgb_serve_request* req, int64_t* id);
/* Cancel a waiting or running request (takes effect between steps). */
fvgb_status fvgb_server_cancel(fvgb_server* server, int64_t id);
/* Move up to `max` finished results out; *count = how many. */
fvgb_status fvgb_server_poll(fvgb_server* server, fvgb_serve_result* out, int32_t max, int32_t* count);
/* [waiting, active, finished-unpolled, bytes in use, peak bytes, ticks] */
fvgb_status fvgb_server_info(fvgb_server* server, int64_t out[6]);
/* Finishes every submitted request, then stops the loop. */
fvgb_status fvgb_server_destroy(fvgb_server* server);

/* ------------------------------------------------------------ mesh builder */
/* Host helpers (no GPU): an OpenFOAM-ordered hex box and OpenFOAM geometry.
 * They stand in for Foam::fvMesh, which provides these arrays in the reference. */
typedef struct fvgb_box_spec {
    int32_t nx, ny, nz;
    double lx, ly, lz;         /* box edge lengths, origin at 0                   */
    double jitter;             /* interior vertex jitter, fraction of the spacing */
    uint64_t seed;
    int32_t two_d;             /* 1: nz must be 1, front/back are empty patches   */
} fvgb_box_spec;

/* Array sizes of a box: [n_points, n_faces_total, n_cells, n_ifaces, n_bfaces,
 * n_patches, face_point_entries]. */
fvgb_status fvgb_box_sizes(const fvgb_box_spec* spec, int64_t out[7]);
/* Topology + geometry of a box into caller-allocated HOST arrays sized by
 * fvgb_box_sizes.  Patches (non-empty only): xmin, xmax, ymin, ymax[, zmin, zmax].
 * cell_centres [n*3], face_centres [nIF*3], bface_centres [nBF*3], points [np*3]
 * may be NULL.  Geometry as fvgb_geometry_compute. */
typedef struct fvgb_mesh_arrays {
    double* points;            /* [n_points*3]                 */
    double* cell_volumes;      /* [n_cells]                    */
    double* cell_centres;      /* [n_cells*3]                  */
    int32_t* owner;            /* [n_ifaces]                   */
    int32_t* neighbour;        /* [n_ifaces]                   */
    double* face_areas;        /* [n_ifaces*3]                 */
    double* face_centres;      /* [n_ifaces*3]                 */
    double* mag_face_areas;    /* [n_ifaces]                   */
    double* weights;           /* [n_ifaces]                   */
    double* delta_coeffs;      /* [n_ifaces]                   */
    int32_t* bface_cells;      /* [n_bfaces]                   */
    double* bface_areas;       /* [n_bfaces*3]                 */
    double* bface_centres;     /* [n_bfaces*3]                 */
    double* bmag_face_areas;   /* [n_bfaces]                   */
    double* bweights;          /* [n_bfaces]                   */
    double* bdelta_coeffs;     /* [n_bfaces]                   */
    int32_t* patch_offsets;    /* [n_patches+1]                */
} fvgb_mesh_arrays;
fvgb_status fvgb_box_build(const fvgb_box_spec* spec, fvgb_mesh_arrays* out);

/* OpenFOAM geometry of a general polyMesh (HOST): face centres/areas by triangle
 * decomposition about the point average, cell volumes/centres by pyramid
 * decomposition about the face-centre average, linear weights
 * |Sf.(C_N-Cf)| / (|Sf.(Cf-C_P)| + |Sf.(C_N-Cf)|) and non-orthogonal delta
 * coefficients 1/max(nf.d, 0.05|d|).  Faces: face_offs[n_faces_total+1] into
 * face_points; faces [0,n_ifaces) internal, then the boundary faces of the
 * `out` patches in order (faces of empty patches must be given after all of
 * them and are skipped: n_faces_total may exceed n_ifaces+n_bfaces).
 * `owner_all` has n_faces_total entries. */
fvgb_status fvgb_geometry_compute(int32_t n_points, const double* points, int32_t n_cells,
                                  int32_t n_faces_total, const int32_t* face_offs,
                                  const int32_t* face_points, const int32_t* owner_all,
                                  int32_t n_ifaces, const int32_t* neighbour,
                                  int32_t n_bfaces, fvgb_mesh_arrays* out);

/* ------------------------------------------------------- OpenFOAM files (HOST)
 * The steps before and after the hot path: FoamAdapter's MeshAdapter builds the
 * mesh from Foam::fvMesh (meshAdapter.cpp:59-136), readVolBoundaryConditions
 * maps a field's boundaryField to boundary conditions (readers.hpp:31-108) and
 * writers.cpp:9-135 write NeoN fields as OpenFOAM fields.  Ascii and binary
 * formats (binary: little-endian, 32/64-bit labels and scalars as the header's
 * arch declares).  Not thread-safe per handle; no device memory is touched. */
typedef struct fvgb_polymesh fvgb_polymesh;
enum { FVGB_IO_BINARY = 1, FVGB_IO_SURFACE = 2 };
/* Read `dir` (a constant/polyMesh directory: points, faces, owner, neighbour,
 * boundary) and compute its geometry (as fvgb_geometry_compute); *desc points
 * into arrays owned by *out until fvgb_polymesh_free.  Faces are ordered
 * internal first, then the non-empty patches in file order; empty patches are
 * left out of the flat boundary (fvPatch sizes them 0). */
fvgb_status fvgb_polymesh_read(const char* dir, fvgb_polymesh** out, fvgb_mesh_desc* desc);
/* Name and type of non-empty patch p, as written in `boundary` (valid until free). */
fvgb_status fvgb_polymesh_patch(const fvgb_polymesh* pm, int32_t p, const char** name, const char** type);
/* The points [n_points*3] and the internal [n_ifaces*3] and boundary
 * [n_bfaces*3] face centres (valid until free). */
fvgb_status fvgb_polymesh_geometry(const fvgb_polymesh* pm, int32_t* n_points, const double** points,
                                   const double** face_centres, const double** bface_centres);
fvgb_status fvgb_polymesh_free(fvgb_polymesh* pm);
/* internalField of a field file into values[n*ncomp] (ncomp 1: List<scalar>,
 * 3: List<vector>; uniform or nonuniform).  n is n_cells for a volume field,
 * n_ifaces for a surface field. */
fvgb_status fvgb_field_read(const char* path, int32_t n, int32_t ncomp, double* values);
/* boundaryField of a field file as boundary conditions of the non-empty
 * patches of pm, by patch name, then patch group, then quoted regular
 * expression: patch_type[n_patches] (fvgb_bc_type) and ref[n_bfaces*ncomp]
 * (host; what fvgb_bc.ref holds on the device).  Mapping (readers.hpp:43-95):
 * fixedValue -> FIXED_VALUE with its value; zeroGradient -> FIXED_GRADIENT 0;
 * fixedGradient -> FIXED_GRADIENT with the patch's `value` entry as the
 * reference takes it; noSlip -> FIXED_VALUE 0; calculated and
 * extrapolatedCalculated -> CALCULATED; any other type FVGB_ERR_UNSUPPORTED.
 * boundary[n_bfaces*ncomp] (may be NULL) receives each patch's `value` entry
 * where it has one, else 0. */
fvgb_status fvgb_field_read_bc(const char* path, const fvgb_polymesh* pm, int32_t ncomp, int32_t* patch_type,
                               double* ref, double* boundary);
/* Write a field file: internalField [n*ncomp] (n = n_cells, or n_ifaces with
 * FVGB_IO_SURFACE), boundaryField with a calculated value per non-empty patch
 * from boundary [n_bfaces*ncomp] (flat, patch order) and type empty for empty
 * patches.  Ascii uses 17 significant digits (every double round-trips);
 * FVGB_IO_BINARY writes the lists as raw little-endian doubles. */
fvgb_status fvgb_field_write(const char* path, const char* object, const fvgb_polymesh* pm, int32_t ncomp,
                             const double* internal, const double* boundary, int32_t flags);

/* ---------------------------------------------- OpenFOAM dictionaries (host)
 * system/fvSolution, system/fvSchemes and other OpenFOAM dictionaries, read
 * without OpenFOAM.  Replaces Foam::dictionary + FoamAdapter::convert
 * (src/auxiliary/foamDictionary.cpp:68-91, convert.cpp:17-45), which turn a
 * case's dictionaries into NeoN::Dictionary (setup.cpp:107-109).  A primitive
 * entry is kept as its token list; sub-dictionaries nest.  Supported syntax:
 * comments, quoted strings, lists "( ... )", words with balanced parentheses
 * (div(phi,T)), #include / #includeIfPresent / #sinclude, #inputMode,
 * #remove, $name inside a value and $name; as an entry, quoted (regular
 * expression) keywords.  Directives that run code give FVGB_ERR_UNSUPPORTED.
 * A handle returned by read/parse/create/copy/map is a top-level dictionary
 * and is released with fvgb_dict_free; fvgb_dict_sub returns a borrowed
 * sub-dictionary that lives as long as its entry. */
typedef struct fvgb_dict fvgb_dict;
enum {
    FVGB_TOK_WORD = 1,    /* word (yes/no/true/false included)          */
    FVGB_TOK_STRING = 2,  /* quoted string, quotes removed              */
    FVGB_TOK_LABEL = 3,   /* integer (label, and scalar = its value)    */
    FVGB_TOK_SCALAR = 4,  /* floating-point number                      */
    FVGB_TOK_PUNCT = 5    /* ( ) [ ] of a list                          */
};
fvgb_status fvgb_dict_read(const char* path, fvgb_dict** out);
fvgb_status fvgb_dict_parse(const char* text, const char* include_dir, fvgb_dict** out);
fvgb_status fvgb_dict_create(fvgb_dict** out);
fvgb_status fvgb_dict_copy(const fvgb_dict* d, fvgb_dict** out);
fvgb_status fvgb_dict_free(fvgb_dict* d);
int32_t fvgb_dict_size(const fvgb_dict* d);
const char* fvgb_dict_key(const fvgb_dict* d, int32_t i);       /* null when out of range */
int32_t fvgb_dict_is_pattern(const fvgb_dict* d, int32_t i);
/* Index of the entry a lookup finds (plain keyword, else the last-defined
 * matching pattern), -1 if none. */
int32_t fvgb_dict_find(const fvgb_dict* d, const char* keyword);
fvgb_dict* fvgb_dict_sub(const fvgb_dict* d, int32_t i);        /* null for a primitive entry */
int32_t fvgb_dict_ntokens(const fvgb_dict* d, int32_t i);       /* -1 for a sub-dictionary */
fvgb_status fvgb_dict_token(const fvgb_dict* d, int32_t i, int32_t j, int32_t* kind, const char** text,
                            int64_t* label, double* scalar);
/* Insert or replace a primitive entry; value is its text ("PCG", "1e-6",
 * "(1 2 3)", "\"solver::Cg\"", "$name" expands in d's scope). */
fvgb_status fvgb_dict_set(fvgb_dict* d, const char* keyword, const char* value);
/* Insert or replace a sub-dictionary: a copy of src, or empty if src is null. */
fvgb_status fvgb_dict_set_dict(fvgb_dict* d, const char* keyword, const fvgb_dict* src, fvgb_dict** sub);
fvgb_status fvgb_dict_remove(fvgb_dict* d, const char* keyword);  /* no-op when absent */
/* Dictionary text (OpenFOAM syntax) into buf[cap] (NUL-terminated,
 * truncated); *len = the full length. */
fvgb_status fvgb_dict_write(const fvgb_dict* d, char* buf, int64_t cap, int64_t* len);

/* FoamAdapter's fvSolution mapping, in place (fvSolution.cpp:19-142):
 * update_solver: PCG -> Ginkgo solver::Cg, PBiCG -> solver::Bicg, PBiCGStab
 *   and smoothSolver -> solver::Bicgstab, GAMG -> solver::Multigrid;
 * update_preconditioner: none given -> DIC; DIC -> preconditioner::Jacobi
 *   {max_block_size 1}; DILU -> preconditioner::Ilu {reverse_apply false;
 *   factorization {type factorization::ParIlu}}; smoother removed; a
 *   preconditioner dictionary whose type is a dictionary -> UNSUPPORTED;
 * update_criteria: criteria {iteration 1000} plus relTol ->
 *   relative_residual_norm, maxIter -> iteration, tolerance ->
 *   absolute_residual_norm (the fvSolution keywords are removed).
 * fvgb_fvsolution_map = mapFvSolution (fvSolution.cpp:145-159): a mapped copy,
 * or a plain copy when the entry names a configFile. */
fvgb_status fvgb_fvsolution_update_solver(fvgb_dict* solver_dict);
fvgb_status fvgb_fvsolution_update_preconditioner(fvgb_dict* solver_dict);
fvgb_status fvgb_fvsolution_update_criteria(fvgb_dict* solver_dict);
fvgb_status fvgb_fvsolution_map(const fvgb_dict* solver_dict, fvgb_dict** mapped);
/* A mapped (Ginkgo-form) solver entry as a solver configuration: type
 * solver::Cg or solver::Bicgstab, preconditioner::Jacobi with max_block_size
 * 1 (or, with solver::Cg, a preconditioner dictionary of type
 * solver::Multigrid), criteria iteration / relative_residual_norm /
 * absolute_residual_norm.
 * This library's own keywords: precision FP64|mixed, innerRelTol,
 * innerMaxIter, maxOuter.  Other solvers and preconditioners (Bicg,
 * Multigrid as a solver, Ilu, none, block Jacobi): FVGB_ERR_UNSUPPORTED; an
 * entry naming a configFile too (read that file with
 * fvgb_solver_cfg_from_json). */
fvgb_status fvgb_solver_cfg_from_dict(const fvgb_dict* mapped, fvgb_solver_cfg* cfg);
/* A Ginkgo JSON configuration (the configFile of a solver entry, e.g.
 * tutorials/cylinder2D/system/gko/config.mg.json) as a solver configuration:
 * type solver::Cg / solver::Bicgstab; preconditioner preconditioner::Jacobi
 * (max_block_size 1) or, with Cg, solver::Multigrid with multigrid::Pgm
 * levels; criteria Iteration (max_iters) and ResidualNorm (reduction_factor,
 * baseline absolute or initial_resnorm; Ginkgo's default baseline rhs_norm:
 * FVGB_ERR_UNSUPPORTED). */
fvgb_status fvgb_solver_cfg_from_json(const char* path, fvgb_solver_cfg* cfg);
/* The scheme fvSchemes gives `name` in `section` (its own entry, else
 * default): divSchemes / gradSchemes "Gauss linear" -> FVGB_SCHEME_LINEAR,
 * "Gauss upwind" -> FVGB_SCHEME_UPWIND; laplacianSchemes "Gauss linear
 * uncorrected" -> 0, "Gauss linear corrected" -> FVGB_SCHEME_CORRECTED;
 * snGradSchemes uncorrected -> 0, corrected -> FVGB_SCHEME_CORRECTED;
 * interpolationSchemes linear / upwind; ddtSchemes Euler -> 0.  No entry or
 * "none": FVGB_ERR_INVALID_ARG; other schemes: FVGB_ERR_UNSUPPORTED. */
fvgb_status fvgb_scheme_from_dict(const fvgb_dict* fv_schemes, const char* section, const char* name,
                                  int32_t* scheme);

#ifdef __cplusplus
}
#endif
#endif /* FVGB_H */
