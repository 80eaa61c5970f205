/*
 * formoniq_gpu.h -- C ABI of the GB300-native Galerkin assembly and Krylov solve
 * path of formoniq (Finite Element Exterior Calculus on Regge meshes).
 *
 * The entry points replace the reference's Rust API on that path; each one cites
 * the reference item it stands in for (paths relative to the formoniq workspace).
 * Conventions of the reference kept here:
 *   - a form's grade argument is the grade of the inner product (WhitneyPairing,
 *     crates/formoniq/src/operators.rs:118-192): mass(k) is N_k x N_k,
 *     dif_test(k) is N_{k-1} x N_k, dif_trial(k) is N_k x N_{k-1},
 *     dif_both(k) is N_{k-1} x N_{k-1};
 *   - simplices of every grade are numbered by colex order of their sorted vertex
 *     tuples (crates/simplicial/src/topology/skeleton.rs:50-83), cells included;
 *   - an assembled entry exists iff some cell contributes an element value that
 *     is not exactly 0.0 (crates/formoniq/src/galerkin.rs:170-177);
 *   - operators are total in the grade: out-of-range grades give correctly
 *     shaped empty matrices (crates/formoniq/src/whitney_complex.rs:113-122).
 *
 * Error behaviour: the reference panics on contract violations and returns
 * Option/Result elsewhere; here every call returns an fq_status, no exception or
 * abort crosses the ABI, and fq_ctx_last_error() holds a message. All device work
 * is ordered on the context's CUDA stream. A context is not thread-safe; use one
 * per host thread.
 */
#ifndef FORMONIQ_GPU_H
#define FORMONIQ_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fq_status {
  FQ_OK = 0,
  FQ_INVALID_ARG = 1,      /* reference: assert!/panic on a contract violation */
  FQ_DEGENERATE_CELL = 2,  /* a cell metric is singular (Metric::dual .expect) */
  FQ_NOT_CONVERGED = 3,    /* Report{converged: false} (iterative/src/lib.rs:212-219) */
  FQ_BREAKDOWN = 4,        /* non-positive preconditioner inner product / NaN */
  FQ_OOM_BUDGET = 5,       /* the context's HBM budget would be exceeded */
  FQ_TIMEOUT = 6,          /* a bounded device wait ran out */
  FQ_CUDA_ERROR = 7,       /* a CUDA runtime call failed */
  FQ_NO_DEVICE = 8,        /* no CUDA device / the library was built without one */
  FQ_UNSUPPORTED = 9       /* dimension or grade outside 0..4 */
} fq_status;

typedef enum fq_form {
  FQ_MASS = 0,      /* WhitneyPairing::mass       operators.rs:169-171 */
  FQ_DIF_TRIAL = 1, /* WhitneyPairing::dif_trial  operators.rs:175-177 */
  FQ_DIF_TEST = 2,  /* WhitneyPairing::dif_test   operators.rs:182-184 */
  FQ_DIF_BOTH = 3   /* WhitneyPairing::dif_both   operators.rs:189-191 */
} fq_form;

typedef enum fq_bc {
  FQ_ABSOLUTE = 0, /* WhitneyComplex: natural BC           whitney_complex.rs:322-465 */
  FQ_RELATIVE = 1  /* RelativeWhitneyComplex: essential BC whitney_complex.rs:523-714 */
} fq_bc;

typedef enum fq_precision {
  FQ_FP64 = 0,      /* FP64 values; Gram inverse and determinant in IEEE double, element
                       entries and scatter sums in float-float (48-bit significand) on
                       the FP32 pipe, well inside the 1e-12 relative element tolerance */
  FQ_FP32 = 1,      /* FP64 Gram inverse/determinant, FP32 element matrices and values */
  FQ_FP64_IEEE = 2  /* FP64 values computed in IEEE double throughout */
} fq_precision;

/* Block preconditioner of the mixed Hodge-Laplace solve. The reference
 * (problems/elliptic.rs:29-47) inverts each diagonal block hdif_gram(j) exactly
 * by a sparse Cholesky factorization; here a block is approximated. */
typedef enum fq_precond {
  FQ_PC_AUTO = 0,   /* FQ_PC_HX where it applies, else FQ_PC_JACOBI */
  FQ_PC_JACOBI = 1, /* diagonal of each block (Jacobi::new, iterative/src/precond.rs:62-64) */
  FQ_PC_HX = 2,     /* Hiptmair-Xu auxiliary-space blocks over a nodal multigrid V-cycle
                       (formoniq/src/hx.rs, multigrid.rs): Kuhn cube meshes with positive
                       squared lengths; FQ_UNSUPPORTED elsewhere */
  FQ_PC_DIRECT = 3, /* Dirac and mixed solves: the sparse direct factorization
                       (fq_sparse_lu_*) of the system preconditioning FP64 GMRES; Kuhn
                       cube meshes. FQ_PC_AUTO takes it for a mixed solve on a mesh with a
                       cell whose metric is not positive definite (Lorentzian: the
                       reference's block preconditioner does not exist there and FaerLu
                       carries the solve, elliptic.rs:153-160), and to finish a MINRES
                       that did not converge (elliptic.rs:147-152) */
  FQ_PC_COMPARISON = 4 /* Dirac solves: MINRES preconditioned by the inverse diagonal of the
                       relative masses of the Euclidean comparison lattice; Kuhn cube meshes */
} fq_precond;

typedef struct fq_ctx fq_ctx;
typedef struct fq_mesh fq_mesh;
typedef struct fq_matrix fq_matrix;
typedef struct fq_mixed fq_mixed;

/* StopCriterion (iterative/src/lib.rs:193-208) plus solver knobs. */
typedef struct fq_solve_opts {
  double rtol;             /* relative residual target; reference default 1e-10 */
  int64_t max_iters;       /* reference default 10_000 */
  int precision;           /* fq_precision of the inner Krylov solve */
  double refine_rtol;      /* FQ_FP32: outer FP64 refinement target (relative residual) */
  int64_t max_refinements; /* FQ_FP32: cap on outer refinement steps */
  int preconditioner;      /* fq_precond of the mixed solves; default FQ_PC_AUTO */
} fq_solve_opts;

/* Report (iterative/src/lib.rs:212-219) plus refinement telemetry. */
typedef struct fq_report {
  int64_t iters;        /* total inner Krylov iterations */
  double residual;      /* final relative residual of the last Krylov solve */
  int32_t converged;    /* 1 when rtol was met */
  int32_t refinements;  /* outer FP64 refinement steps taken (0 in FQ_FP64) */
  double true_residual; /* ||b - A x|| / ||b|| recomputed in FP64 at the end */
} fq_report;

/* ---- context ------------------------------------------------------------ */
/* No counterpart in the reference (a CPU crate on rayon's global pool): a
 * context holds the device, its CUDA stream, an optional HBM budget (0 = none)
 * and the last error message. fq_default_solve_opts fills the reference's
 * StopCriterion defaults (iterative/src/lib.rs:193-208) and FQ_PC_AUTO. */
fq_status fq_ctx_create(int device, void* cuda_stream, uint64_t hbm_budget_bytes, fq_ctx** out);
/* Destroy every mesh, matrix and mixed problem made on a context first. */
void fq_ctx_destroy(fq_ctx* ctx);
const char* fq_status_name(fq_status s);
const char* fq_ctx_last_error(const fq_ctx* ctx);
fq_status fq_ctx_synchronize(fq_ctx* ctx);
uint64_t fq_ctx_bytes_in_use(const fq_ctx* ctx);
/* Number of this library's kernels launched on the context so far. */
uint64_t fq_ctx_kernel_launches(const fq_ctx* ctx);
void fq_default_solve_opts(fq_solve_opts* opts);
/* Instrumentation, no counterpart in the reference (which times with
 * Instant::now() in ignored benches): while enabled, CUDA events recorded on the
 * context's stream bracket the element-kernel pass (slot 0) and the scatter
 * (slot 1) of every assembly; fq_ctx_profile returns the accumulated
 * milliseconds and launch counts per slot and optionally resets them. */
fq_status fq_ctx_set_profiling(fq_ctx* ctx, int enable);
fq_status fq_ctx_profile(fq_ctx* ctx, double* ms, int64_t* launches, int nslots, int reset);
/* Instrumentation, no counterpart in the reference: the sustained FMA rate of
 * this device's FP64 (fp64 != 0) or FP32 pipe, in TFLOP/s (2 flops per FMA),
 * from a register-resident FMA-chain kernel timed with CUDA events. */
fq_status fq_measure_fma_peak(fq_ctx* ctx, int fp64, double* tflops);
/* Launch shape of the symmetric scatter of this context's assemblies, no
 * counterpart in the reference: slots_per_thread -1 = by precision (the
 * default: one thread per upper slot for FQ_FP64, one slot per thread on a
 * persistent grid for FQ_FP32 and FQ_FP64_IEEE), 0 = one thread per upper slot,
 * 1/2/4/8 = that many upper slots per thread on a persistent grid of
 * blocks_per_sm 256-thread blocks per SM (0 = as many as are resident at once).
 * Every shape sums each slot's contributions in the same order: the values are
 * bit-identical. */
fq_status fq_ctx_set_scatter_shape(fq_ctx* ctx, int slots_per_thread, int blocks_per_sm);

/* ---- topology: Complex -------------------------------------------------- */
/* Complex::from_cells (crates/simplicial/src/topology/complex.rs:278-336):
 * cells is host int32 [ncells][dim+1], each row strictly increasing; the cells
 * are renumbered in colex order, every skeleton derived. dim in 0..4. */
fq_status fq_mesh_from_cells(fq_ctx* ctx, int dim, int64_t ncells, const int32_t* cells, fq_mesh** out);
/* CartesianGrid::new_unit(dim, n).triangulate() topology
 * (crates/regge/src/mesher/cartesian.rs:210-213, simplicial/src/mesher/grid.rs:77-98). */
fq_status fq_mesh_kuhn_cube(fq_ctx* ctx, int dim, int nboxes_per_axis, fq_mesh** out);
void fq_mesh_destroy(fq_mesh* mesh);
int fq_mesh_dim(const fq_mesh* mesh);
/* Complex::nsimplices (simplicial/src/topology/complex.rs:58-60); 0 off 0..dim. */
int64_t fq_mesh_nsimplices(const fq_mesh* mesh, int grade);
/* HilbertComplex::ndofs (whitney_complex.rs:376-383 / :588-595). */
int64_t fq_mesh_ndofs(const fq_mesh* mesh, int grade, fq_bc bc);
/* Complex::skeleton(k) (complex.rs:48-50): host int32 [N_k][k+1], colex order. */
fq_status fq_mesh_simplices(const fq_mesh* mesh, int grade, int32_t* out);
/* Kept (interior) kidx of the relative complex, increasing (whitney_complex.rs:548-566). */
fq_status fq_mesh_interior(const fq_mesh* mesh, int grade, int64_t* out);
/* A coherent orientation of the cells, +-1 (simplicial topology/orientation.rs). */
fq_status fq_mesh_orientation(const fq_mesh* mesh, int8_t* out);

/* ---- geometry: MeshLengthsSq ------------------------------------------- */
/* MeshLengthsSq::new (crates/regge/src/lengths/mesh.rs:34-36): one signed
 * squared length per edge in colex edge order. `on_device` != 0 means the pointer
 * is device memory on the context's device. */
fq_status fq_mesh_set_lengths_sq(fq_mesh* mesh, const double* lengths_sq, int on_device);
fq_status fq_mesh_get_lengths_sq(const fq_mesh* mesh, double* out_host);
/* MeshCoords::to_edge_lengths_sq (crates/regge/src/coord/mesh.rs:208-216):
 * s_e = (x_j - x_i)^T diag(ambient_signs) (x_j - x_i); coords host [nverts][adim]. */
fq_status fq_mesh_lengths_from_coords(fq_mesh* mesh, const double* coords, int adim, const double* ambient_signs);
/* Input generator for the Kuhn configs: CartesianGrid vertex placement
 * (cartesian.rs:158-169) on [0,side_a] per axis, seeded uniform +-jitter*h
 * jitter of every coordinate of every vertex, then the squared lengths
 * under diag(ambient_signs). Requires a mesh made by fq_mesh_kuhn_cube. */
fq_status fq_mesh_kuhn_lengths(fq_mesh* mesh, const double* side, const double* ambient_signs, double jitter,
                               uint64_t seed);

/* ---- kernel (a): per-cell Regge metric ---------------------------------- */
/* SimplexLengthsSq::metric (regge/src/lengths/simplex.rs:308-326),
 * Metric::dual (metric/src/lib.rs:250-257), cell_volume (regge/src/lib.rs:26-28),
 * for every cell. Device outputs: ginv [n*n][ncells] (entry-major), det [ncells],
 * vol [ncells]; any may be NULL. */
fq_status fq_cell_metrics(fq_ctx* ctx, fq_mesh* mesh, double* ginv, double* det, double* vol);

/* ---- kernel (b): element matrices --------------------------------------- */
/* BilinearForm::element for a WhitneyPairing (operators.rs:201-211), every cell.
 * Device output, entry-major [rows*cols][ncells] (row-major local entries),
 * double for FQ_FP64, float for FQ_FP32. rows/cols receive the local shape. */
fq_status fq_element_matrices(fq_ctx* ctx, fq_mesh* mesh, fq_form form, int grade, fq_precision prec,
                              void* out, int* rows, int* cols);

/* ---- assembly ----------------------------------------------------------- */
/* BilinearForm::assemble (galerkin.rs:52-57 -> assemble_matrix :138-188) through
 * HilbertComplex::{mass,dif_trial,dif_test,dif_both} (whitney_complex.rs:130-170),
 * on the full or the relative complex (E^T A E, whitney_complex.rs:620-624).
 * The pattern and the sorted scatter permutation are built on the first call per
 * (form, grade, bc) and cached on the mesh. */
fq_status fq_assemble(fq_ctx* ctx, fq_mesh* mesh, fq_form form, int grade, fq_bc bc, fq_precision prec,
                      fq_matrix** out);
/* BilinearForm::assemble again (galerkin.rs:52-57) into an existing matrix
 * (same mesh, form, grade, bc, precision) after new lengths: the hot loop of a
 * geometry sweep. */
fq_status fq_reassemble(fq_ctx* ctx, fq_mesh* mesh, fq_matrix* mat);
/* Several fq_reassemble calls in one (a geometry sweep that refreshes a set of
 * operators, e.g. the HilbertComplex masses and stiffnesses, whitney_complex.rs:
 * 130-183, each a BilinearForm::assemble, galerkin.rs:52-57): the element passes
 * and scatters of all matrices (any meshes of this context) are queued back to
 * back on the context's stream and the status is read once at the end. Same
 * results and errors as calling fq_reassemble on each in order. The matrices
 * are taken in groups of four (the last may be shorter); a group of two or
 * more that are all mass / dif_both matrices of one mesh of dimension 1-3 in
 * one precision shares a single element pass (each cell's metric and Gramian
 * computed once), into element buffers the matrices then keep; the values are
 * the per-matrix assembly's (bit for bit in FQ_FP64). */
fq_status fq_reassemble_many(fq_ctx* ctx, fq_matrix* const* mats, int count);
/* HilbertComplex::hdif_gram (whitney_complex.rs:180-183): M_k + dif_both(k+1). */
fq_status fq_hdif_gram(fq_ctx* ctx, fq_mesh* mesh, int grade, fq_bc bc, fq_matrix** out);
/* HilbertComplex::dif (whitney_complex.rs:417-423, relative :640-643): the
 * coboundary N_{k+1} x N_k, entries +-1. */
fq_status fq_coboundary(fq_ctx* ctx, fq_mesh* mesh, int grade, fq_bc bc, fq_matrix** out);
/* BilinearForm::assemble (galerkin.rs:52-57) from host lengths into host
 * values, the end-to-end call: uploads lengths_sq (N_1 doubles), assembles,
 * downloads the CSR values (nnz doubles or floats) into values_out. The
 * pattern comes from fq_matrix_copy_to_host of a prior fq_assemble. */
fq_status fq_assemble_host(fq_ctx* ctx, fq_mesh* mesh, fq_matrix* mat, const double* lengths_sq_host,
                           void* values_out_host);
/* fq_assemble_host for several matrices of one mesh (the operators a geometry
 * sweep refreshes, each a BilinearForm::assemble, galerkin.rs:52-57): the
 * lengths are uploaded once and each matrix's values are downloaded into
 * values_out_host[i] (its current nnz entries) while the next matrix's kernels
 * run. Pinned host buffers let the copies overlap. */
fq_status fq_assemble_host_many(fq_ctx* ctx, fq_mesh* mesh, const double* lengths_sq_host, fq_matrix* const* mats,
                                void* const* values_out_host, int count);

/* Re-assembly that allocates no device memory. It has no counterpart in the
 * reference. For callers that cannot let this library call cudaMalloc (a host
 * that owns all device memory through its own arena, or a latency-critical loop
 * where an allocation would synchronise the device): the per-cell element
 * buffer lives in a static device array of 32 MiB that every GPU loading the
 * library holds until exit, and the values (nnz of `pattern`, its precision)
 * are written to the caller's device buffer `values_out` in the CSR order of
 * `pattern`, a matrix fq_assemble made on this mesh. Rejects, with
 * FQ_INVALID_ARG and a message, a mesh whose element buffer (entries x cells x
 * value width) exceeds the array; returns FQ_UNSUPPORTED when the exact-zero
 * rule would change the pattern. Every call looks up the array's device address
 * with the context's device current, and synchronises ctx->stream before it
 * returns (it reads the status words back). All calls share the array: calls
 * whose work overlaps on the GPU race. */
fq_status fq_reassemble_noalloc(fq_ctx* ctx, fq_mesh* mesh, const fq_matrix* pattern, void* values_out);

/* The assembled matrix stands in for the reference's GalerkinMatrix, a CSR
 * matrix built from the COO triplets of assemble_matrix (galerkin.rs:138-188):
 * its shape, nnz, arrays (device or host copies) and release. */
fq_status fq_matrix_info(const fq_matrix* m, int64_t* nrows, int64_t* ncols, int64_t* nnz, int* precision);
/* The bytes one re-assembly's scatter reads and writes for this matrix: every
 * element value once, the plan's records and the indices it still reads, every
 * assembled value once (the roofline accounting of the scatter). 0 without a plan. */
fq_status fq_matrix_scatter_bytes(const fq_matrix* m, int64_t* bytes);
fq_status fq_matrix_device_arrays(const fq_matrix* m, const int32_t** row_ptr, const int32_t** col_idx,
                                  const void** values);
/* Host copies: row_ptr [nrows+1], col_idx [nnz], values [nnz] (double or float). */
fq_status fq_matrix_copy_to_host(fq_ctx* ctx, const fq_matrix* m, int32_t* row_ptr, int32_t* col_idx,
                                 void* values);
void fq_matrix_destroy(fq_matrix* m);

/* ---- kernel (d): operator, Krylov, preconditioner ------------------------ */
/* LinearOperator::apply for CsrMatrix (iterative/src/operator.rs:5-13):
 * y = A x, device vectors of the matrix's precision. */
fq_status fq_spmv(fq_ctx* ctx, const fq_matrix* a, const void* x, void* y);
/* krylov::minres (iterative/src/krylov.rs:113-211), device-resident, FP64, with
 * the SPD diagonal preconditioner y = inv_diag .* r (NULL = identity). b, x,
 * inv_diag are device pointers; x is overwritten (start from zero). */
fq_status fq_minres(fq_ctx* ctx, const fq_matrix* a, const double* inv_diag, const double* b, double* x,
                    const fq_solve_opts* opts, fq_report* report);
/* krylov::cg (iterative/src/krylov.rs:48-95), same conventions. */
fq_status fq_cg(fq_ctx* ctx, const fq_matrix* a, const double* inv_diag, const double* b, double* x,
                const fq_solve_opts* opts, fq_report* report);
/* GradeKHodgeHx::with_multigrid(..).solve (formoniq/src/hx.rs:140-240): CG on
 * hdif_gram(grade) (M_k + D_k^T M_{k+1} D_k) preconditioned by the grade-`grade`
 * Hiptmair-Xu auxiliary-space preconditioner whose auxiliary blocks are nodal
 * multigrid V-cycles (2 Jacobi sweeps, weight 2/3). Kuhn cube meshes with
 * positive squared lengths, else FQ_UNSUPPORTED. rhs_host and x_host hold the
 * grade's degrees of freedom (interior ones for FQ_RELATIVE). */
fq_status fq_hx_cg(fq_ctx* ctx, fq_mesh* mesh, int grade, fq_bc bc, const double* rhs_host, double* x_host,
                   const fq_solve_opts* opts, fq_report* report);
/* ApproxInverse::apply of that preconditioner (AuxiliarySpace::apply,
 * iterative/src/aux_space.rs): y = B r once, host arrays. */
fq_status fq_hx_apply(fq_ctx* ctx, fq_mesh* mesh, int grade, fq_bc bc, const double* r_host, double* y_host);

/* ---- the mixed Hodge-Laplace source problem ------------------------------ */
/* The resident form of elliptic::solve_source (problems/elliptic.rs:132-182):
 * assembles the symmetrised KKT system of assemble_mixed_kkt (:54-114) with the
 * harmonic border, and the diagonal of mixed_block_preconditioner (:29-47), once;
 * later solves reuse it. */
fq_status fq_mixed_create(fq_ctx* ctx, fq_mesh* mesh, int grade, fq_bc bc, int precision, fq_mixed** out);
/* Re-assemble the KKT system after new lengths on the same mesh. */
fq_status fq_mixed_reassemble(fq_mixed* prob);
/* Solve with a host source GalerkinVector (ambient N_k doubles); outputs host
 * sigma (ambient N_{k-1}), u (ambient N_k), p (harmonic_dim); any may be NULL.
 * Routes, as solve_source (elliptic.rs:140-160): block-preconditioned MINRES
 * on Riemannian meshes; the sparse direct solver on Lorentzian Kuhn meshes (a
 * cell metric not positive definite; float-float factors) or with FQ_PC_DIRECT
 * (FP32 factors first); the factors stay with the problem for later solves
 * until fq_mixed_reassemble; a MINRES (or FP32
 * refinement) that does not converge is finished by the sparse direct solver
 * on Kuhn meshes (its GMRES takes up to max(max_iters, 300) iterations; report
 * iters count both, refinements is then the direct solve's: 1 = float-float or
 * IEEE FP64 factors),
 * by a dense LU on other meshes of at most 8192 unknowns. */
fq_status fq_mixed_solve(fq_mixed* prob, const double* source_host, double* sigma_host, double* u_host,
                         double* p_host, const fq_solve_opts* opts, fq_report* report);
/* Same on device pointers (source ambient N_k; outputs in the same layouts). */
fq_status fq_mixed_solve_device(fq_mixed* prob, const double* source, double* sigma, double* u, double* p,
                                const fq_solve_opts* opts, fq_report* report);
/* Sizes: n_sigma, n_u, n_harmonic (relative-DOF counts), system nnz. */
fq_status fq_mixed_info(const fq_mixed* prob, int64_t* n_sigma, int64_t* n_u, int64_t* n_harmonic,
                        int64_t* nnz);
/* The assembled KKT matrix (owned by the problem; do not destroy). */
const fq_matrix* fq_mixed_system(const fq_mixed* prob);
void fq_mixed_destroy(fq_mixed* prob);
/* One-shot elliptic::solve_source (problems/elliptic.rs:132-182) with host buffers. */
fq_status fq_solve_source(fq_ctx* ctx, fq_mesh* mesh, int grade, fq_bc bc, const double* source_host,
                          double* sigma_host, double* u_host, double* p_host, const fq_solve_opts* opts,
                          fq_report* report);

/* ---- matrix-free operators --------------------------------------------- */
/* ElementOperator (formoniq/src/matfree.rs:54-141): a Whitney pairing applied
 * without assembling it, y = sum_K P_K^T A_K P_K x. Nothing is stored per
 * nonzero: every apply rebuilds each cell's element matrix from the mesh's
 * current squared lengths (float-float, as FQ_FP64 assembly) and gathers the
 * per-cell products at each degree of freedom in cell order, race-free. The
 * operator reads the mesh's lengths at every apply (fq_mesh_set_lengths_sq
 * takes effect at once). Rectangular for dif_test / dif_trial. */
typedef struct fq_elemop fq_elemop;
/* ElementOperator::new (matfree.rs:68-84): the test-face incidence, once. */
fq_status fq_elemop_create(fq_ctx* ctx, fq_mesh* mesh, fq_form form, int grade, fq_bc bc, fq_elemop** out);
fq_status fq_elemop_info(const fq_elemop* op, int64_t* nrows, int64_t* ncols);
/* ElementOperator::apply (matfree.rs:98-131): device x [ncols] -> y [nrows], FP64. */
fq_status fq_elemop_apply(fq_elemop* op, const double* x, double* y);
/* matfree::diagonal (:148-172): the assembled diagonal, gathered (square forms). */
fq_status fq_elemop_diagonal(fq_elemop* op, double* diag);
/* krylov::cg (iterative/src/krylov.rs:48-95) driven by the apply; inv_diag (device,
 * may be NULL) is the Jacobi preconditioner (matfree::jacobi, :174-180). */
fq_status fq_elemop_cg(fq_elemop* op, const double* b, double* x, const double* inv_diag, const fq_solve_opts* opts,
                       fq_report* report);
void fq_elemop_destroy(fq_elemop* op);

/* ---- Maxwell evolution: explicit leapfrog ---------------------------------- */
/* solve_dirac_leapfrog (problems/dirac.rs:404-434) with time::Leapfrog
 * (time.rs:271-420): M du/dt = A u, A = dif - delta (HodgeDirac::assemble,
 * dirac.rs:196-198), grades 2-coloured by parity, one step = half-kick of the odd
 * grades, drift of the even ones, half-kick. The coupling blocks are the
 * assembled dif_trial(k) / dif_test(k); each mass block is inverted by
 * Jacobi-preconditioned CG to mass_rtol (<= 0: 1e-13) where the reference
 * Cholesky-factors it. y is a device vector in the complex's DOFs (bc), flat by
 * grade at the offsets fq_leapfrog_info returns (n+2 entries); stable under
 * the CFL condition dt <= h_min / c, as the reference. */
typedef struct fq_leapfrog fq_leapfrog;
fq_status fq_leapfrog_create(fq_ctx* ctx, fq_mesh* mesh, fq_bc bc, double dt, double mass_rtol, fq_leapfrog** out);
fq_status fq_leapfrog_info(const fq_leapfrog* lf, int64_t* ndofs, int64_t* offsets, int64_t* inner_iters);
/* Leapfrog::step, nsteps times, in place. */
fq_status fq_leapfrog_step(fq_leapfrog* lf, double* y, int64_t nsteps);
/* HodgeDirac::energy (1/2 u^T M u) and Leapfrog::conserved_energy (time.rs:401-420). */
fq_status fq_leapfrog_energy(fq_leapfrog* lf, const double* y, double* energy, double* conserved);
void fq_leapfrog_destroy(fq_leapfrog* lf);

/* ---- the de Rham map (the right-hand-side side of a solve) --------------- */
/* derham_map (derham/src/project.rs:53-96): (R w)_s = integral of the k-form w
 * over each k-simplex s, by the Grundmann-Moeller rule exact to `degree`
 * (simplicial/src/atlas/quadrature.rs:38-82), paired with the simplex's tangent
 * blade (metric-free). A field is caller code, so it is evaluated by the caller
 * between two calls: fq_derham_nodes writes the nodes x[s][q][adim] of every
 * k-simplex (device coords [N_0][adim], adim <= 4), the caller writes
 * w(x)[s][q][C(adim,k)] (components on dx^I, I the k-subsets of the axes in
 * colex order), fq_derham_reduce writes the cochain [N_k]. All device arrays. */
int fq_derham_npoints(int grade, int degree);
fq_status fq_derham_nodes(fq_ctx* ctx, fq_mesh* mesh, const double* coords, int adim, int grade, int degree,
                          double* nodes);
fq_status fq_derham_reduce(fq_ctx* ctx, fq_mesh* mesh, const double* coords, int adim, int grade, int degree,
                           const double* values, double* cochain);

/* ---- the source load (the Galerkin vector of a source form) --------------- */
/* SourceForm::element (formoniq/src/operators.rs:598-635) summed by
 * assemble_vector (formoniq/src/galerkin.rs:279-312):
 *   l_s = sum_K vol_K sum_q w_q <f(x_q), W_s(x_q)>_{Lambda^k g_K^{-1}}
 * over the cells K containing the k-simplex s, in cell order, with the
 * Grundmann-Moeller rule of `degree` on the cell (the reference's default
 * CellQuadrature is degree 1). Like the de Rham map, the field is evaluated by
 * the caller between two calls. fq_source_nodes writes, with coords null, the
 * barycentric nodes [nq][n+1] shared by every cell; with device coords
 * [N_0][adim] (n <= adim <= 4), the ambient nodes [ncells][nq][adim]. The caller
 * writes values [ncells][nq][ncomp]: with coords null, the section's components
 * in each cell's reference frame (ncomp = C(n,k), on dxi^J with xi_j =
 * lambda_{j+1}, J colex; derham/src/section.rs:50-66); with coords, a flat
 * ambient form's components on dx^A (ncomp = C(adim,k)), pulled back through
 * each cell's affine map (Pullback::identity, section.rs:95-140).
 * fq_source_assemble writes out [ndofs(k, bc)] (FQ_RELATIVE: the interior
 * entries, RelativeWhitneyComplex::restrict). All arrays are device memory. */
int fq_source_npoints(int dim, int degree);
fq_status fq_source_nodes(fq_ctx* ctx, fq_mesh* mesh, const double* coords, int adim, int degree, double* nodes);
fq_status fq_source_assemble(fq_ctx* ctx, fq_mesh* mesh, int grade, fq_bc bc, int degree, const double* coords,
                             int adim, const double* values, double* out);

/* Direct fallback: the reference finishes a MINRES that did not converge with a
 * sparse LU (problems/elliptic.rs:147-159) and solves the Dirac source problem by
 * LU. Here the mixed solve and the Dirac solve finish an unconverged MINRES by
 * the sparse direct solver (fq_sparse_lu_*, GMRES on its factors) on Kuhn cube
 * meshes, at any size and in the server's lanes too (its allocations are
 * stream-ordered). On other meshes, a system of at most 8,192 unknowns is
 * finished by a dense LU with partial pivoting on the device (cuSOLVER, loaded
 * at run time): report.converged is then 1 with report.iters the MINRES
 * iterations spent, and report.true_residual that of the direct solution.
 * Larger systems on such meshes keep the MINRES result (FQ_NOT_CONVERGED), and
 * so do the server's lanes there (the dense factorization's synchronous
 * allocations would break the graph captures of the other lanes). */

/* ---- the covariant Hodge-Dirac source problem ---------------------------- */
/* dirac::solve_dirac_source (problems/dirac.rs:473-531): S = A + m M of
 * HodgeDirac::assemble_selfadjoint (:205-260) on the relative complex,
 * rhs = E^T (load - S lift). Solver (opts->preconditioner):
 *   FQ_PC_AUTO / FQ_PC_DIRECT on fq_mesh_kuhn_cube meshes: the reference's
 *     LU, here the sparse direct factorization (fq_sparse_lu_*, float-float
 *     factors) preconditioning FP64 GMRES to opts->rtol on the true residual
 *     (report.refinements = 1). At m = 0 the top-grade harmonic (top_harmonic,
 *     :552-570) is tested against the kernel (||S h|| <= 1e-8 ||h||) and, if
 *     it spans it, the system is bordered with it (solve_bordered, :578-598):
 *     the solution orthogonal to the kernel. When |m| is below a shift tau =
 *     1e-3 / (mesh diameter), the factored matrix carries mass term tau (the
 *     massless system's fronts have structurally zero pivots); GMRES runs on
 *     the system itself.
 *   FQ_PC_COMPARISON / FQ_PC_HX (Kuhn meshes): MINRES preconditioned from the
 *     Euclidean comparison lattice (the signed lengths' axis scales made
 *     positive): the inverse diagonal of its relative masses M_j, j = 0..n, or
 *     its relative hdif_gram(j) blocks, each an HX multigrid.
 *   FQ_PC_JACOBI, and FQ_PC_AUTO on other meshes: MINRES with |diag(S)|.
 * The MINRES routes need m != 0. load/lift/x are host, flattened by grade
 * (ambient offsets of HodgeDirac, :181-200). */
fq_status fq_solve_dirac_source(fq_ctx* ctx, fq_mesh* mesh, double mass_term, const double* load_host,
                                const double* lift_host, double* x_host, const fq_solve_opts* opts,
                                fq_report* report);
/* The assembled relative Dirac system S (for parity tests); caller destroys. */
fq_status fq_dirac_system(fq_ctx* ctx, fq_mesh* mesh, double mass_term, fq_matrix** out);

/* ---- sparse direct solver ----------------------------------------------- */
/* Stands in for FaerLu (formoniq/src/linalg/faer.rs:51-74) where the reference
 * factors: solve_dirac_source (problems/dirac.rs:525-531) and the LU fallback of
 * solve_source (problems/elliptic.rs:147-160). Multifrontal LU on a geometric
 * nested-dissection ordering of the Kuhn vertex lattice: the fronts of each
 * level of the elimination tree are assembled and partially factored together
 * on the device (the system scaled symmetrically, D A D with d_i the inverse
 * square root of row i's largest magnitude; the pivot rows of each tile chosen
 * over all the front's fully summed rows by tournament pivoting; pivots below
 * 1e-6 (FQ_FP32 factors), 1e-12 (float-float) or 1e-13 (IEEE FP64) of the
 * scaled matrix perturbed). The factors precondition a restarted GMRES in
 * FP64 on the FP64 matrix, which stops on the true relative residual
 * ||b - A x|| / ||b||. */
typedef struct fq_sparse_lu fq_sparse_lu;
/* Symbolic analysis of `a` (square, FP64 values, made by fq_assemble,
 * fq_dirac_system or fq_mixed_system on `mesh`, a fq_mesh_kuhn_cube mesh):
 * FQ_UNSUPPORTED on other meshes. */
fq_status fq_sparse_lu_create(fq_ctx* ctx, fq_mesh* mesh, const fq_matrix* a, fq_sparse_lu** out);
/* Numeric factorization of a's current values (after every re-assembly), in
 * precision FQ_FP32 (tiles of 128 columns on the FP32 pipe), FQ_FP64 (float-
 * float: each value a pair of floats, 48-bit significand, computed on the
 * FP32 pipe; tiles of 64 columns) or FQ_FP64_IEEE (IEEE double on the FP64
 * pipe, which runs at a small fraction of the FP32 pipe's rate on GB300). */
fq_status fq_sparse_lu_factor(fq_sparse_lu* lu, const fq_matrix* a, int precision);
/* x = A^-1 b (device vectors of a->nrows doubles) by GMRES to opts->rtol on the
 * true FP64 residual, or until the normwise backward error
 * ||b - A x|| / (||A||_F ||x|| + ||b||) reaches 1e-14 (the rounding level an LU
 * solve delivers; a nearly singular system may not allow rtol), at most
 * opts->max_iters iterations in all. On FP32
 * factors GMRES runs for at most 60 iterations (stopping earlier when three
 * iterations do not halve the residual); if it has not converged by then, `a`
 * is re-factored in FQ_FP64 (float-float; the factorization keeps that type
 * afterwards, until the next fq_sparse_lu_factor) and GMRES starts again from
 * zero: then report.refinements = 1. report.iters counts both. On FQ_FP64 or
 * FQ_FP64_IEEE factors report.refinements is 1. opts->max_refinements = 0
 * keeps the current factors whatever their type: GMRES runs on them for up to
 * opts->max_iters iterations and no re-factorization happens. */
fq_status fq_sparse_lu_solve(fq_sparse_lu* lu, const fq_matrix* a, const double* b_dev, double* x_dev,
                             const fq_solve_opts* opts, fq_report* report);
/* Fronts, levels, factorization flops, bytes of the current factors, pivots
 * perturbed in the last factorization. */
fq_status fq_sparse_lu_info(const fq_sparse_lu* lu, int64_t* fronts, int64_t* levels, double* flops,
                            int64_t* factor_bytes, int64_t* perturbed_pivots);
void fq_sparse_lu_destroy(fq_sparse_lu* lu);
/* The symbolic analysis alone, on the host (no device, no context), for
 * tests of the ordering: the pattern as host CSR, five vertex ids per unknown
 * (-1 padded). stats[0..5] = fronts, levels, factorization flops, factor bytes
 * (FP32), largest front, unknowns eliminated. Also checks every index the
 * kernels will form against its buffer. */
fq_status fq_sparse_lu_analyse_host(int dim, int nbox, int64_t n, const int32_t* rp, const int32_t* ci,
                                    const int32_t* dof_vertices, double* stats);

/* ---- batched assembly --------------------------------------------------- */
/* No counterpart in the reference (one mesh per assemble_matrix call,
 * galerkin.rs:138-188). A batch assembles one form per mesh on many meshes of
 * the context at once: per mesh the same element program, scatter plan and
 * summation order as fq_assemble (FP64 values, float-float compute, absolute
 * complex, topological pattern), the whole batch as one CUDA graph with one
 * grid-stride element launch per (dimension, degree) class present and one
 * scatter launch over all meshes' CSR slots. */
typedef struct fq_batch fq_batch;
typedef enum fq_batch_form {
  FQ_BATCH_MASS = 0, /* WhitneyPairing::mass(k)                    operators.rs:169-171 */
  FQ_BATCH_HDIF = 1  /* HilbertComplex::hdif_gram(k) = M_k + dif_both(k+1), whitney_complex.rs:180-183 */
} fq_batch_form;
/* meshes[i] (with lengths) and grades[i]: the form at grade k on mesh i. */
fq_status fq_batch_create(fq_ctx* ctx, int nmeshes, fq_mesh* const* meshes, const int* grades, int form,
                          fq_batch** out);
/* Tuner: times each candidate launch shape `reps` times on this batch (element
 * CTAs per SM per class; scatter symmetric, warp-staged or 1/2/4 threads per
 * slot, and CTAs per SM) and keeps the fastest. */
fq_status fq_batch_tune(fq_batch* batch, int reps);
/* Fixed launch shape: element grid (CTAs, 0 = one thread per cell), scatter
 * threads per slot (-1 = one per upper slot of the symmetric plans, 0 =
 * warp-staged, 1, 2 or 4) and grid. */
fq_status fq_batch_set_launch(fq_batch* batch, int element_grid, int scatter_tps, int scatter_grid);
/* One assembly of the whole batch (one graph launch). check != 0 waits and
 * checks the status words (degenerate cells; a slot that summed exact zeros
 * only, which the reference would drop: FQ_UNSUPPORTED). */
/* The element pass as one fused launch over every (dimension, grade) class
 * (fused = 1; a grid-stride grid of `grid` CTAs, 0 = one thread per cell) or
 * one launch per class (fused = 0, the default). The fused kernel covers
 * hdif_gram batches of dimensions 2-4 (FQ_UNSUPPORTED otherwise); it runs every
 * class at the register allocation of the heaviest program. Values are the
 * same bit for bit either way. */
fq_status fq_batch_set_element_launch(fq_batch* batch, int fused, int grid);
/* Registers per thread of the fused element kernel (-1 if unknown). */
int fq_batch_fused_registers(void);
fq_status fq_batch_assemble(fq_batch* batch, int check);
/* The same assembly as two launches per mesh (the per-mesh baseline). */
fq_status fq_batch_assemble_per_mesh(fq_batch* batch, int check);
fq_status fq_batch_info(const fq_batch* batch, int64_t* total_cells, int64_t* total_slots, int* nclasses,
                        int* launches_per_assembly);
fq_status fq_batch_launch_config(const fq_batch* batch, int* scatter_tps, int* scatter_grid, int* element_grids,
                                 int max_classes);
/* Device CSR of mesh i (row_ptr/col_idx of its plan, values in the batch). */
fq_status fq_batch_matrix(const fq_batch* batch, int i, int64_t* nrows, int64_t* nnz, const int32_t** row_ptr,
                          const int32_t** col_idx, const double** values);
/* Host copy of mesh i's CSR (row_ptr nrows+1, col_idx and values nnz). */
fq_status fq_batch_copy_to_host(const fq_batch* batch, int i, int32_t* row_ptr, int32_t* col_idx, double* values);
void fq_batch_destroy(fq_batch* batch);

/* ---- serving: continuously batched solve requests ----------------------- */
/* No counterpart in the reference (one problem per call there). A server runs
 * `lanes` lanes, each a host thread with its own context and CUDA stream, so the
 * device work of concurrent requests overlaps. Requests are taken in arrival
 * order; the next one starts as soon as a lane is free and its estimated HBM
 * footprint fits the budget beside the running requests and the resident
 * meshes (it always starts when nothing runs). With cache != 0, meshes, scatter
 * plans, operators and preconditioner hierarchies stay resident per lane and a
 * request goes to a free lane that holds its mesh; lanes drop resident meshes
 * when the budget needs the room. Results do not depend on the lane or on the
 * other requests in flight (deterministic kernels). */
typedef struct fq_server fq_server;

typedef enum fq_request_kind {
  FQ_REQ_HODGE = 0, /* elliptic::solve_source on a Kuhn cube (problems/elliptic.rs:132-182) */
  FQ_REQ_DIRAC = 1  /* dirac::solve_dirac_source, lift 0 (problems/dirac.rs:473-531) */
} fq_request_kind;

typedef struct fq_request {
  int kind;               /* fq_request_kind */
  int dim;                /* Kuhn cube dimension 1..4 */
  int nbox;               /* boxes per axis */
  int grade;              /* FQ_REQ_HODGE: form degree k */
  int bc;                 /* FQ_REQ_HODGE: fq_bc */
  int minkowski;          /* 1: Minkowski lengths (axis 0 timelike, time scale 0.7) */
  double jitter;          /* Riemannian: vertex jitter in units of h; Minkowski: relative length jitter */
  uint64_t seed;          /* lengths and source when not given */
  double mass_term;       /* FQ_REQ_DIRAC: m (nonzero) */
  double arrival_ms;      /* >= 0: arrival time after server creation (latency counts from it); < 0: now */
  const double* lengths;  /* optional host lengths (NULL: generated from seed); read while the request runs */
  const double* source;   /* optional host source / load (NULL: seeded N(0,1)); read while it runs */
  double* solution;       /* optional host output: (sigma, u) for HODGE, x for DIRAC */
  fq_solve_opts opts;
} fq_request;

typedef struct fq_result {
  int32_t status;       /* fq_status of the request */
  int32_t lane;         /* lane that ran it */
  fq_report report;
  double queue_ms;      /* arrival -> start */
  double run_ms;        /* start -> done */
  double latency_ms;    /* arrival -> done */
  double start_ms;      /* start, ms after server creation */
  double end_ms;        /* done, ms after server creation */
  double checksum;      /* sum of squares of the solution */
  uint64_t ndofs;       /* length of the solution */
  int32_t cache_hit;    /* 1 when the mesh was resident on the lane */
  int32_t pad;
} fq_result;

typedef struct fq_server_stats {
  uint64_t submitted, completed, cache_hits, evictions;
  uint64_t peak_committed_bytes; /* running estimates + resident bytes, at most */
  uint64_t resident_bytes;       /* bytes the idle lanes hold now */
  double busy_ms;                /* summed run time of completed requests */
} fq_server_stats;

fq_status fq_server_create(int device, int lanes, uint64_t hbm_budget_bytes, int cache, fq_server** out);
fq_status fq_server_submit(fq_server* server, const fq_request* request, uint64_t* ticket);
/* Blocks until the request is done; each ticket is waited on once. */
fq_status fq_server_wait(fq_server* server, uint64_t ticket, fq_result* result);
fq_status fq_server_get_stats(fq_server* server, fq_server_stats* stats);
/* Finishes the submitted requests, then stops the lanes. */
void fq_server_destroy(fq_server* server);

#ifdef __cplusplus
}
#endif
#endif /* FORMONIQ_GPU_H */
