/*
 * ug4gb.h -- C ABI of libug4gb, the GB300 (sm_103a) assemble-and-solve engine
 * for UG4/ugcore's FV1 + geometric-multigrid + Krylov hot path.
 *
 * Conventions
 *   - Every function returns an int status: UG4GB_OK (0) or a negative error
 *     code; ug4gb_last_error(ctx) returns the message of the last failure.
 *     No C++ exception crosses this boundary.
 *   - Array arguments may be host or device pointers (the library detects
 *     which); the caller owns them.  The library owns all device memory of a
 *     handle and frees it in the matching *_destroy.  A host output array is
 *     complete when the call returns, and a host input array may be reused
 *     then.  Device arrays are read and written in stream order on the
 *     context's stream (ug4gb_stream): a device input must stay unchanged,
 *     and a device output be read, only after that stream has passed the
 *     call (an event, or ug4gb_synchronize).  Work on the library's own
 *     objects (matrices, vectors, multigrids) is ordered on that stream.
 *   - One CUDA stream per context; calls on one context are not thread-safe
 *     (ugcore's hot path is single-threaded per process).
 *   - Indices are 0-based 32-bit ints; DoF numbering is lexicographic per
 *     level (i + nx*(j + ny*k)).
 * Each entry point names the ugcore interface it stands in for
 * (paths relative to ugcore's ugbase/).
 */
#ifndef UG4GB_H
#define UG4GB_H

#include <stdint.h>

#if defined(__GNUC__)
#define UG4GB_API __attribute__((visibility("default")))
#else
#define UG4GB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define UG4GB_OK 0
#define UG4GB_ERR_INVALID (-1)      /* bad argument / handle */
#define UG4GB_ERR_CUDA (-2)         /* a CUDA runtime call failed */
#define UG4GB_ERR_NOMEM (-3)        /* device allocation failed */
#define UG4GB_ERR_SINGULAR (-4)     /* base-level LU found a pivot < 1e-10 */
#define UG4GB_ERR_NOT_CONVERGED (-5)/* Krylov solver stopped without convergence */
#define UG4GB_ERR_BREAKDOWN (-6)    /* CG lambda == 0 / BiCGStab rho, alpha, tt, omega == 0 */
#define UG4GB_ERR_STATE (-7)        /* call order (e.g. apply before init) */

/* element types of a grid hierarchy */
#define UG4GB_QUAD 0                /* 2D quadrilaterals (ROID_QUADRILATERAL) */
#define UG4GB_HEX 1                 /* 3D hexahedra (ROID_HEXAHEDRON) */
#define UG4GB_TET 2                 /* 3D tetrahedra, 6 per hex, Kuhn split */
#define UG4GB_TRI 3                 /* 2D triangles (ROID_TRIANGLE; unstructured grids) */

/* smoothers, precisions, solvers */
#define UG4GB_SMOOTHER_JACOBI 0     /* damped Jacobi (lib_algebra/operator/preconditioner/jacobi.h:90) */
#define UG4GB_SMOOTHER_MCGS 1       /* multicolour Gauss-Seidel (GaussSeidel, gauss_seidel.h:271, in
                                       colour order); damp = the SOR factor (set_sor_relax) */
#define UG4GB_SMOOTHER_MCSGS 2      /* symmetric multicolour Gauss-Seidel, (D/w + U)^-1 D (D/w + L)^-1
                                       (SymmetricGaussSeidel, gauss_seidel.h:350, in colour order);
                                       damp = w, 0 < w < 2 */
#define UG4GB_SMOOTHER_ILU 3        /* ILU(0) in multicolour order (ILU, ilu.h:109-290, of the colour-
                                       permuted operator); damp scales the correction */
#define UG4GB_SMOOTHER_MCBGS 4      /* backward multicolour Gauss-Seidel: colours in decreasing order
                                       (BackwardGaussSeidel, gauss_seidel.h:316, in colour order) */
#define UG4GB_PREC_FP64 0           /* whole preconditioner in FP64 */
#define UG4GB_PREC_MIXED 1          /* FP32 smoother/transfers/SpMV, FP64 outer Krylov and base LU */
#define UG4GB_SOLVER_CG 0           /* lib_algebra/operator/linear_solver/cg.h:59 */
#define UG4GB_SOLVER_BICGSTAB 1     /* lib_algebra/operator/linear_solver/bicgstab.h:59 */
#define UG4GB_UPWIND_NONE 0
#define UG4GB_UPWIND_FULL 1         /* ConvectionShapesFullUpwind (lib_disc/spatial_disc/disc_util/conv_shape.h:277) */

typedef struct ug4gb_ctx ug4gb_ctx;
typedef struct ug4gb_grid ug4gb_grid;
typedef struct ug4gb_vector ug4gb_vector;
typedef struct ug4gb_matrix ug4gb_matrix;
typedef struct ug4gb_disc ug4gb_disc;
typedef struct ug4gb_gmg ug4gb_gmg;
typedef struct ug4gb_solver ug4gb_solver;

/* ------------------------------------------------------------- context -- */
/* Replaces the process-level setup of ugcore (ug::UGInit, ug.cpp) for one GPU. */
UG4GB_API int ug4gb_create(int device, ug4gb_ctx **out);
UG4GB_API void ug4gb_destroy(ug4gb_ctx *ctx);
UG4GB_API const char *ug4gb_last_error(const ug4gb_ctx *ctx);
UG4GB_API int ug4gb_synchronize(ug4gb_ctx *ctx);
/* the context's cudaStream_t, for callers that order their own work on it */
UG4GB_API void *ug4gb_stream(ug4gb_ctx *ctx);
/* number of kernels this context has launched so far (instrumentation) */
UG4GB_API int64_t ug4gb_kernel_launches(const ug4gb_ctx *ctx);
/* solve layout of operators set up after this call: UG4GB_FORMAT_AUTO (the
   constant-offset "diagonal" layout whenever an operator has <= 27 distinct
   column offsets, else SELL-32) or UG4GB_FORMAT_SELL (always SELL-32).  The
   exported CRS never changes; only the copy the kernels stream does. */
#define UG4GB_FORMAT_AUTO 0
#define UG4GB_FORMAT_SELL 1
UG4GB_API int ug4gb_set_operator_format(ug4gb_ctx *ctx, int format);
/* performance switches that leave every result bit-identical.
   UG4GB_TUNE_PDL (0 or 1): programmatic dependent launch of the solve-path
   kernels, each kernel scheduled while its predecessor still runs (default 1).
   UG4GB_TUNE_SWEEP_FUSION (bit mask, 0..3): two consecutive damped-Jacobi
   steps of a structured 3D FP32 level in one pass over its operator.  Bit 1:
   on; bit 2: levels of every size (else only levels of at least 2^18
   vertices).  Default 0: inside the solve's CUDA graph the one-step kernels
   overlap through programmatic dependent launch and are as fast.  Smoothed
   corrections and defects are bit-identical; inside a Krylov solve only the
   summation order of the fused (z, r) product changes.  Applies to
   multigrids set up after the call (the fused levels keep a line-padded
   copy of their operator). */
#define UG4GB_TUNE_PDL 1
#define UG4GB_TUNE_SWEEP_FUSION 2
/* UG4GB_TUNE_SWEEP_PLANES (2..128): z planes a block of the fused sweeps
   marches through (default 8). */
#define UG4GB_TUNE_SWEEP_PLANES 3
/* UG4GB_TUNE_ROW_ASSEMBLY (0, 1 or 2): stationary assembly of structured
   levels row by row from the per-class element geometry (1), in addition
   with a constant coefficient and no convection from the one interior
   stencil, computed once and written to every interior row (2, default;
   the same values as 1), or with the element kernel used for unstructured
   levels (0).  All give the same values to rounding (the cells of a
   structured level are congruent up to the rounding of their corner
   coordinates); each is bit-reproducible. */
#define UG4GB_TUNE_ROW_ASSEMBLY 4
/* UG4GB_TUNE_SWEEP_WAIT_TEST (bytes, multiple of 16, 0..4096; default 0):
   failure test of the fused sweeps only.  Block 0 of the next fused sweep
   launched after the call (one launch) announces this many bytes more than
   its first operator copy delivers, so its bounded wait runs out (half a
   second): the block issues no further copies and leaves, the solve returns
   UG4GB_ERR_CUDA ("a kernel's bounded wait ... ran out") and the context
   stays usable.  Never set outside such a test. */
#define UG4GB_TUNE_SWEEP_WAIT_TEST 5
/* UG4GB_TUNE_COARSE_LEVELS (-1..7; default -1): the coarse end of a V-cycle
   (Jacobi smoothers on both sides, dense LU base solver, structured levels
   with grid transfers) run by one block in one launch: the base level and
   up to this many levels above it (never the top level), their operators,
   Jacobi factors and vectors in shared memory.  -1: the levels where this
   was measured faster on GB300 (a Jacobi sweep of at most about 4000 FP64
   row-operations, rows x (stencil width + 3), an FP32 one counting a
   quarter; a base level of at most 32 rows); 0: every level by separate
   launches.  Corrections are bit-identical either way.  Applies to
   multigrids set up after the call. */
#define UG4GB_TUNE_COARSE_LEVELS 6
UG4GB_API int ug4gb_set_tuning(ug4gb_ctx *ctx, int knob, int value);
/* per-launch CUDA-event timing of every kernel until profile_end, which
   writes "tag|kernel<TAB>launches<TAB>total_ms" lines into buf.  While it is
   on, solvers launch kernels directly instead of replaying CUDA graphs.
   (Stands in for ugcore's PROFILE_BEGIN/END probes, common/profiler/profiler.h.) */
UG4GB_API int ug4gb_profile_begin(ug4gb_ctx *ctx);
UG4GB_API int ug4gb_profile_end(ug4gb_ctx *ctx, char *buf, int capacity);
/* Guarded (debug) builds only (compiled with UG4GB_GUARDED): every device
   buffer lies between two 4 KB guard zones, and zones and buffer start out
   as 0xFF bytes (NaN in every floating-point type, -1 in the integers), so
   a kernel that writes outside a buffer changes a zone and one that uses
   memory nobody wrote produces NaN.  Synchronises the device, checks the
   zones of every live buffer (freed buffers are checked when freed) and
   writes one line per damaged zone into buf; returns the number of damaged
   zones seen so far (0: none), or UG4GB_ERR_STATE in a normal build.  Stands
   in for the bounds checks of ugcore's debug builds (UG_ASSERT in
   lib_algebra) on the device.  No context needed. */
UG4GB_API int ug4gb_debug_guard_check(char *buf, int capacity);

/* ------------------------------------------------------ grid hierarchy -- */
/* Replaces MultiGrid + GlobalMultiGridRefiner::perform_refinement
   (lib_grid/refinement/global_multi_grid_refiner.cpp:135) and the level
   DoFDistribution (lib_disc/dof_manager/dof_distribution.cpp:1339) for
   structured boxes: the unit square/cube split into mx*my(*mz) coarse cells,
   refined num_refinements times. */
UG4GB_API int ug4gb_grid_create_structured(ug4gb_ctx *ctx, int elem_type, int mx, int my, int mz,
                                 int num_refinements, ug4gb_grid **out);
UG4GB_API int ug4gb_grid_num_levels(const ug4gb_grid *g);
UG4GB_API int ug4gb_grid_level_info(const ug4gb_grid *g, int level, int *num_vertices, int *num_elements,
                          int *corners_per_element, int *dim);
/* copies level geometry out (any pointer may be NULL) */
UG4GB_API int ug4gb_grid_level_export(const ug4gb_grid *g, int level, double *coords, int *elems,
                            unsigned char *boundary);
UG4GB_API void ug4gb_grid_destroy(ug4gb_grid *g);
/* Unstructured hierarchies: a coarse grid refined nref times regularly
   (GlobalMultiGridRefiner, lib_grid/refinement/global_multi_grid_refiner.h;
   triangles and quadrilaterals -> 4, tetrahedra and hexahedra -> 8, the inner
   octahedron of a tetrahedron cut along its shortest diagonal), built on the
   host at set-up and uploaded.  Dirichlet vertices follow subset membership
   through the refinement as in ugcore (objects created on an edge / face /
   element belong to its subset).
   ug4gb_grid_create_ugx reads a UGX file (lib_grid/file_io/file_io_ugx.cpp;
   vertices, edges, triangles, quadrilaterals, tetrahedrons, hexahedrons and
   the first subset_handler; one element type per grid): dirichlet_subsets is
   a comma-separated list of subset names whose vertices, edges, faces and
   volumes carry the zero Dirichlet condition (DirichletBoundary::add(0, "c",
   "Name, ...")); NULL or "" = the topological boundary.
   ug4gb_grid_create_unstructured takes the coarse grid as arrays: elements
   with the reference corner order of elem_type, Dirichlet vertices (NULL:
   none), Dirichlet edges (pairs) and faces (4 corners in cyclic order, -1 as
   the 4th of a triangle); no Dirichlet arguments at all = the topological
   boundary. */
UG4GB_API int ug4gb_grid_create_ugx(ug4gb_ctx *ctx, const char *filename, int nref, const char *dirichlet_subsets,
                                    ug4gb_grid **out);
UG4GB_API int ug4gb_grid_create_unstructured(ug4gb_ctx *ctx, int elem_type, int num_vertices, const double *coords,
                                             int num_elements, const int *elems,
                                             const unsigned char *dirichlet_vertices, int num_dirichlet_edges,
                                             const int *dirichlet_edges, int num_dirichlet_faces,
                                             const int *dirichlet_faces, int nref, ug4gb_grid **out);
/* 1 for a structured (box) hierarchy, 0 for an unstructured one */
UG4GB_API int ug4gb_grid_is_structured(const ug4gb_grid *g);
/* parents of the vertices of `level` >= 1 in level - 1: npar (nv) and par
   (nv x 8, increasing, -1 padded) */
UG4GB_API int ug4gb_grid_level_parents(const ug4gb_grid *g, int level, int *npar, int *par);
/* host only, no context or GPU: level `level` of the hierarchy that
   ug4gb_grid_create_ugx builds (sizes first with NULL arrays) */
UG4GB_API int ug4gb_io_ugx_level(const char *filename, int nref, const char *dirichlet_subsets, int level,
                                 int *elem_type, int *num_vertices, int *num_elements, double *coords, int *elems,
                                 unsigned char *dirichlet, int *npar, int *par, char *err, int err_capacity);

/* ------------------------------------------------------------- vectors -- */
/* Replaces ug::Vector<double> (lib_algebra/cpu_algebra/vector.h:54). */
UG4GB_API int ug4gb_vector_create(ug4gb_ctx *ctx, int n, ug4gb_vector **out);
/* non-owning view of caller device memory (e.g. a torch tensor) */
UG4GB_API int ug4gb_vector_wrap(ug4gb_ctx *ctx, double *device_ptr, int n, ug4gb_vector **out);
UG4GB_API int ug4gb_vector_size(const ug4gb_vector *v);
UG4GB_API double *ug4gb_vector_data(ug4gb_vector *v);
UG4GB_API int ug4gb_vector_set(ug4gb_vector *v, double value);                  /* vector.h set */
UG4GB_API int ug4gb_vector_copy_from(ug4gb_vector *v, const double *src);       /* host or device */
UG4GB_API int ug4gb_vector_copy_to(const ug4gb_vector *v, double *dst);         /* host or device */
UG4GB_API int ug4gb_vector_norm(const ug4gb_vector *v, double *out);            /* vector_impl.h:323 */
UG4GB_API int ug4gb_vector_dot(const ug4gb_vector *a, const ug4gb_vector *b, double *out); /* vector_impl.h:72 */
/* dest = alpha*a + beta*b (VecScaleAdd, lib_algebra/cpu_algebra/operations_vec.h:55) */
UG4GB_API int ug4gb_vector_scale_add(ug4gb_vector *dest, double alpha, const ug4gb_vector *a, double beta,
                           const ug4gb_vector *b);
UG4GB_API void ug4gb_vector_destroy(ug4gb_vector *v);
/* Vector::maxnorm (vector_impl.h) and entry access from the host (indices and
   values in host arrays; out-of-range indices are an error) */
UG4GB_API int ug4gb_vector_maxnorm(const ug4gb_vector *v, double *out);
UG4GB_API int ug4gb_vector_get_values(const ug4gb_vector *v, int n, const int *idx, double *vals);
UG4GB_API int ug4gb_vector_set_values(ug4gb_vector *v, int n, const int *idx, const double *vals);
/* (a, b) of two FP64 device arrays of the current device, for callers that
   may not allocate device memory (no context needed).  Has no counterpart in
   the reference.  The library allocates nothing for it, ever; but the first
   call in a CUDA context can make the CUDA runtime load the library's device
   code (with the 64 KiB static scratch) onto the device, so a caller with a
   strict no-allocation phase makes one warm-up call (n = 1) before that phase
   and before any stream capture.  The scratch exists once per CUDA context
   (its address is looked up once per context).  The result goes to *result,
   a device pointer, in stream order on `stream`; nothing is synchronised.
   n <= UG4GB_DOT_NOALLOC_MAX_N (else UG4GB_ERR_INVALID), and calls that
   overlap in time on one device race on the shared scratch: order them on
   one stream.  On failure a message goes to err (may be NULL). */
#define UG4GB_DOT_NOALLOC_MAX_N 67108864
UG4GB_API int ug4gb_vector_dot_noalloc(const double *a, const double *b, int64_t n, double *result, void *stream,
                                       char *err, int err_capacity);

/* ------------------------------------------------------------ matrices -- */
/* Replaces ug::SparseMatrix<double> (lib_algebra/cpu_algebra/sparsematrix.h:98)
   in its defragmented CRS form (columns sorted per row). */
UG4GB_API int ug4gb_matrix_create(ug4gb_ctx *ctx, ug4gb_matrix **out);
UG4GB_API int ug4gb_matrix_set_csr(ug4gb_matrix *A, int num_rows, int num_cols, int64_t nnz, const int *rowptr,
                         const int *col, const double *val);
UG4GB_API int ug4gb_matrix_info(const ug4gb_matrix *A, int *num_rows, int *num_cols, int64_t *nnz);
UG4GB_API int ug4gb_matrix_export_csr(const ug4gb_matrix *A, int *rowptr, int *col, double *val);
/* dest = alpha1*v1 + beta1*A*w1 (SparseMatrix::axpy, sparsematrix_impl.h:294) */
UG4GB_API int ug4gb_matrix_axpy(const ug4gb_matrix *A, ug4gb_vector *dest, double alpha1, const ug4gb_vector *v1,
                      double beta1, const ug4gb_vector *w1);
/* dest = alpha1*v1 + beta1*A^T*w1 (SparseMatrix::axpy_transposed, sparsematrix_impl.h:344) */
UG4GB_API int ug4gb_matrix_axpy_transposed(const ug4gb_matrix *A, ug4gb_vector *dest, double alpha1,
                                 const ug4gb_vector *v1, double beta1, const ug4gb_vector *w1);
/* T = B^T; keep_zeros=1 as set_as_transpose_of, 0 as set_as_transpose_of2
   (sparsematrix_impl.h:149,186) */
UG4GB_API int ug4gb_matrix_set_as_transpose_of(ug4gb_matrix *T, const ug4gb_matrix *B, int keep_zeros);
UG4GB_API void ug4gb_matrix_destroy(ug4gb_matrix *A);
/* the rest of the SparseMatrix interface ugcore's templates use (set-up and
   glue, not the solve path): resize_and_clear (sparsematrix_impl.h:91; empty
   rows), clear_retain_structure (:142; values 0), set_as_copy_of (:472;
   this = scale * B), scale (:487), apply_ignore_zero_rows (:270-288; dest =
   beta A w on rows with stored entries, others kept), row access (get_row:
   returns the row length, copies up to capacity entries to host arrays) and
   the scatter-add of element contributions into the existing pattern
   (add_entries; host arrays; an entry outside the pattern is an error) */
UG4GB_API int ug4gb_matrix_resize_and_clear(ug4gb_matrix *A, int num_rows, int num_cols);
UG4GB_API int ug4gb_matrix_clear_retain_structure(ug4gb_matrix *A);
UG4GB_API int ug4gb_matrix_set_as_copy_of(ug4gb_matrix *A, const ug4gb_matrix *B, double scale);
UG4GB_API int ug4gb_matrix_scale(ug4gb_matrix *A, double alpha);
UG4GB_API int ug4gb_matrix_apply_ignore_zero_rows(const ug4gb_matrix *A, ug4gb_vector *dest, double beta,
                                                  const ug4gb_vector *w);
UG4GB_API int ug4gb_matrix_get_row(const ug4gb_matrix *A, int row, int *cols, double *vals, int capacity);
UG4GB_API int ug4gb_matrix_add_entries(ug4gb_matrix *A, int n, const int *rows, const int *cols,
                                       const double *vals);

/* ----------------------------------------------------- DoF permutation -- */
/* No ugcore counterpart (ugcore has one numbering).  The engine numbers the
   vertices of a level its own way (lexicographic on structured levels, the
   refinement order on unstructured ones); ugcore numbers DoFs in lib_grid's
   element-list order (DoFDistribution::reinit, lib_disc/dof_manager/
   dof_distribution.cpp:1339-1440).  A ug4gb_perm moves vectors and operators
   between the two numberings: perm[i] = engine index of external DoF i (a
   bijection of 0..n-1; host or device array). */
typedef struct ug4gb_perm ug4gb_perm;
UG4GB_API int ug4gb_perm_create(ug4gb_ctx *ctx, int n, const int *engine_of_external, ug4gb_perm **out);
/* the permutation that matches external DoF positions (n x dim doubles, host
   or device; the vertex positions of ugcore's DoFs) to the vertices of
   `level` of g, each within distance tol of exactly one unused vertex */
UG4GB_API int ug4gb_perm_from_positions(ug4gb_ctx *ctx, const ug4gb_grid *g, int level, int n,
                                        const double *positions, double tol, ug4gb_perm **out);
/* to_external = 1: dst[i] = src[perm[i]] (engine -> external); 0: the inverse */
UG4GB_API int ug4gb_perm_vector(const ug4gb_perm *p, int to_external, const ug4gb_vector *src, ug4gb_vector *dst);
/* to_external = 1: B(i, j) = A(perm[i], perm[j]) (columns sorted per row);
   0: the inverse.  The pattern of B and the value map are built once per
   pattern of A (an assembled level operator); later calls after a
   re-assembly of the same pattern only gather the values. */
UG4GB_API int ug4gb_perm_matrix(ug4gb_perm *p, int to_external, const ug4gb_matrix *A, ug4gb_matrix *B);
UG4GB_API void ug4gb_perm_destroy(ug4gb_perm *p);

/* ------------------------------------------------------ discretisation -- */
/* Replaces DomainDiscretization (lib_disc/spatial_disc/domain_disc.h) with one
   FV1 convection-diffusion IElemDisc (elem_disc_interface.h:797; the
   ConvectionDiffusionFV1 plugin) and a zero DirichletBoundary on the whole
   boundary (lagrange_dirichlet_boundary_impl.h:754-870). */
UG4GB_API int ug4gb_disc_create(ug4gb_ctx *ctx, const ug4gb_grid *g, ug4gb_disc **out);
UG4GB_API int ug4gb_disc_set_diffusion_constant(ug4gb_disc *d, double K);
/* K = exp(factor * g(centroid)), g(x) = amp * sum_m cos(k_m . x + phase_m)
   (LognormalRandomField::eval_K form, lognormal_random_field_impl.h);
   k: nmodes*dim wavevectors, evaluated on every level */
UG4GB_API int ug4gb_disc_set_diffusion_fourier(ug4gb_disc *d, int nmodes, const double *k, const double *phase,
                                     double amp, double factor);
/* K = exp(m) per top-level element; coarse levels use the children's mean m */
UG4GB_API int ug4gb_disc_set_log_diffusion_elements(ug4gb_disc *d, const double *m_top);
/* v(x) = scale * sum_m -sin(k_m . x + phase_m) c_m (3D), evaluated at SCVF ips */
UG4GB_API int ug4gb_disc_set_velocity_fourier_curl(ug4gb_disc *d, int nmodes, const double *k, const double *c,
                                         const double *phase, double scale);
UG4GB_API int ug4gb_disc_set_upwind(ug4gb_disc *d, int upwind);
/* f per top-level vertex (host or device array) */
UG4GB_API int ug4gb_disc_set_source_vertices(ug4gb_disc *d, const double *f_top);
/* f_i = 2*u(seed,i) - 1, u = splitmix64 counter hash (seeded synthetic source) */
UG4GB_API int ug4gb_disc_set_source_uniform(ug4gb_disc *d, uint64_t seed);
/* DomainDiscretizationBase::assemble_linear (domain_disc_impl.h:837) */
UG4GB_API int ug4gb_disc_assemble_linear(ug4gb_disc *d, int level, ug4gb_matrix *A, ug4gb_vector *b);
/* DomainDiscretizationBase::assemble_jacobian (domain_disc_impl.h:471) */
UG4GB_API int ug4gb_disc_assemble_jacobian(ug4gb_disc *d, int level, ug4gb_matrix *A);
/* DomainDiscretizationBase::assemble_defect (domain_disc_impl.h:648):
   d = A(u) u - f assembled element by element (add_def_A_elem + add_rhs_elem,
   elem_disc_assemble_util.h:578-690), d = 0 at Dirichlet vertices
   (DirichletBoundary::adjust_defect).  The source enters on the top level. */
UG4GB_API int ug4gb_disc_assemble_defect(ug4gb_disc *d, int level, const ug4gb_vector *u, ug4gb_vector *dvec);
/* DomainDiscretizationBase::adjust_solution: u = 0 at the Dirichlet vertices */
UG4GB_API int ug4gb_disc_adjust_solution(ug4gb_disc *d, int level, ug4gb_vector *u);
/* AT = A^T with the Dirichlet rows of `level` reset to identity: the operator
   of the adjoint (transposed) solve.  No ugcore counterpart (ugcore has
   SparseMatrix::set_as_transpose_of, sparsematrix_impl.h:149, and
   SetDirichletRow, sparsematrix_util.h:850, but no adjoint). */
/* ---- time discretisation (ThetaTimeStep, lib_disc/time_disc/theta_time_step.h:165) ----
   theta scheme over the FV1 discretisation with one previous time point:
   (M + theta dt A) u_new = M u_old - (1 - theta) dt A u_old + dt f, where M is
   the lumped FV1 mass (|SCV_i| on the diagonal) and f the discretisation's
   source; assembled element by element as the instationary AssembleLinear /
   AssembleJacobian (lib_disc/spatial_disc/elem_disc/elem_disc_assemble_util.h:
   1032-1225, 439-560) with update_scaling's s_m = (1, -1), s_a = (theta dt,
   (1 - theta) dt) (theta_time_step.h:230-246); Dirichlet rows as in the
   stationary case. */
typedef struct ug4gb_timedisc ug4gb_timedisc;
UG4GB_API int ug4gb_timedisc_create(ug4gb_ctx *ctx, ug4gb_disc *d, ug4gb_timedisc **out);
UG4GB_API int ug4gb_timedisc_set_theta(ug4gb_timedisc *td, double theta);   /* set_theta; default 1 */
/* prepare_step(prevSol, dt): copies the previous (top-level) solution */
UG4GB_API int ug4gb_timedisc_prepare_step(ug4gb_timedisc *td, const ug4gb_vector *u_old, double t_old, double dt);
UG4GB_API int ug4gb_timedisc_future_time(const ug4gb_timedisc *td, double *t);
/* assemble_linear(A, b) of the step (top level) */
UG4GB_API int ug4gb_timedisc_assemble_linear(ug4gb_timedisc *td, int level, ug4gb_matrix *A, ug4gb_vector *b);
/* assemble_jacobian(J) = M + theta dt A of any level */
UG4GB_API int ug4gb_timedisc_assemble_jacobian(ug4gb_timedisc *td, int level, ug4gb_matrix *A);
/* ThetaTimeStep::assemble_defect (theta_time_step_impl.h:200-240, instationary
   AssembleDefect, elem_disc_assemble_util.h:713-860): the defect of u at the
   future time with the stored previous solution, top level only */
UG4GB_API int ug4gb_timedisc_assemble_defect(ug4gb_timedisc *td, int level, const ug4gb_vector *u,
                                             ug4gb_vector *dvec);
UG4GB_API void ug4gb_timedisc_destroy(ug4gb_timedisc *td);

/* AT may be A itself: the values are transposed in place (the level
   operators' patterns are symmetric; UG4GB_ERR_INVALID otherwise), which
   keeps the adjoint solve within the forward solve's memory */
UG4GB_API int ug4gb_disc_adjoint_operator(ug4gb_disc *d, int level, const ug4gb_matrix *A, ug4gb_matrix *AT);
/* element coefficient K of a level (host or device out array, num_elements) */
UG4GB_API int ug4gb_disc_export_coefficients(ug4gb_disc *d, int level, double *K);
UG4GB_API void ug4gb_disc_destroy(ug4gb_disc *d);

/* ----------------------------------------------------------------- GMG -- */
/* Replaces AssembledMultiGridCycle (lib_disc/operator/linear_operator/
   multi_grid_solver/mg_solver.h:82) with StdTransfer (std_transfer.h:57),
   Jacobi smoothing and an LU base solver (lu.h:50).  Defaults follow the
   constructor (mg_solver_impl.hpp:78): V-cycle, 2/2 smoothing steps, base
   level 0; Jacobi damping 0.6 as in the configured scripts. */
UG4GB_API int ug4gb_gmg_create(ug4gb_ctx *ctx, ug4gb_disc *disc, ug4gb_gmg **out);
UG4GB_API int ug4gb_gmg_set_smoother(ug4gb_gmg *m, int kind, double damp);            /* set_smoother */
/* set_presmoother / set_postsmoother (mg_solver.h:179-183): different pre-
   and post-smoothers.  damp is the Jacobi damping, the Gauss-Seidel SOR
   relaxation (set_sor_relax, gauss_seidel.h:96) or the ILU correction
   factor.  Any two of the Gauss-Seidel kinds and ILU combine, each with its
   own factor; the Jacobi smoother works on the column-scaled level operator
   and combines only with itself at the same damping (ug4gb_gmg_init returns
   UG4GB_ERR_INVALID otherwise). */
/* set_base_solver (mg_solver.h:136): UG4GB_BASE_LU (default), the dense
   partially pivoted LU of the base level (at most 4096 unknowns), or
   UG4GB_BASE_SMOOTHER: `steps` steps of the pre-smoother on the base level
   from a zero correction, c += B d, d -= A (B d) -- ugcore's LinearSolver
   with the pre-smoother as its preconditioner and StdConvCheck(steps, 0, 0)
   with unsuccessful ends suppressed (convergence_check.h:191) -- for base
   levels too large for the dense LU.  steps 1..1000. */
#define UG4GB_BASE_LU 0
#define UG4GB_BASE_SMOOTHER 1
UG4GB_API int ug4gb_gmg_set_base_solver(ug4gb_gmg *m, int kind, int steps);
UG4GB_API int ug4gb_gmg_set_presmoother(ug4gb_gmg *m, int kind, double damp);
UG4GB_API int ug4gb_gmg_set_postsmoother(ug4gb_gmg *m, int kind, double damp);
UG4GB_API int ug4gb_gmg_set_cycle_type(ug4gb_gmg *m, int cycle);  /* 1 = V, 2 = W, up to 4; -1 = F (mg_solver.h:339-341) */
UG4GB_API int ug4gb_gmg_set_num_presmooth(ug4gb_gmg *m, int n);
UG4GB_API int ug4gb_gmg_set_num_postsmooth(ug4gb_gmg *m, int n);
UG4GB_API int ug4gb_gmg_set_base_level(ug4gb_gmg *m, int level);
UG4GB_API int ug4gb_gmg_set_precision(ug4gb_gmg *m, int precision);
/* StdTransfer::set_prolongation_damping / set_restriction_damping
   (lib_disc/operator/linear_operator/std_transfer.h:92,95; Lua
   transfer:set_prolongation_damping(d), gmg:set_transfer(transfer)): the
   applied prolongation is d_p P c and the applied restriction d_r R d
   (std_transfer_impl.h:740,792); the assembled P and R (export_transfer) are
   not damped, as in ugcore.  Default 1; applies at the next init. */
UG4GB_API int ug4gb_gmg_set_prolongation_damping(ug4gb_gmg *m, double damp);
UG4GB_API int ug4gb_gmg_set_restriction_damping(ug4gb_gmg *m, double damp);
/* transposed = 1 builds the cycle on A^T of every level (Dirichlet rows reset
   to identity): the preconditioner of the adjoint solve.  The level operators
   are transposed in place, so one multigrid may alternate between the
   forward and the transposed cycle (set_transposed, then init) on the same
   buffers: re-assembly instead of a second stored hierarchy */
UG4GB_API int ug4gb_gmg_set_transposed(ug4gb_gmg *m, int transposed);
/* AssembledMultiGridCycle::set_rap (mg_solver.h:149; Lua gmg:set_rap(true),
   multigrid_bridge.cpp:214): rap = 1 makes every coarse level operator the
   Galerkin product R A P of the level above (init_rap_operator,
   mg_solver_impl.hpp:830-1012, with AddMultiplyOf, sparsematrix_util.h:167)
   instead of re-assembling it; default 0 */
UG4GB_API int ug4gb_gmg_set_rap(ug4gb_gmg *m, int rap);
/* AssembledMultiGridCycle::set_discretization (mg_solver.h:126) with a time
   discretisation: coarse levels are re-assembled as its jacobian M + theta dt A
   of the prepared step (init() must follow prepare_step); NULL: the plain
   stationary discretisation */
UG4GB_API int ug4gb_gmg_set_time_disc(ug4gb_gmg *m, ug4gb_timedisc *td);
/* AssembledMultiGridCycle::init (mg_solver_impl.hpp:380): copies the top
   operator, re-assembles coarser levels (or forms R A P), builds P/R,
   smoothers and the LU.  A base level of at most 160 unknowns is factorised
   on the device and the call does not wait for it: a singular base matrix
   (LU pivot below 1e-10) is then reported as UG4GB_ERR_SINGULAR by the next
   ug4gb_gmg_apply or solve with this multigrid; a larger base is factorised
   on the host and reported by this call. */
UG4GB_API int ug4gb_gmg_init(ug4gb_gmg *m, const ug4gb_matrix *A_top);
/* c = B d (AssembledMultiGridCycle::apply, mg_solver_impl.hpp:176) */
UG4GB_API int ug4gb_gmg_apply(ug4gb_gmg *m, ug4gb_vector *c, const ug4gb_vector *d);
/* transfer operators of fine level `level`: which = 0 P, 1 R */
UG4GB_API int ug4gb_gmg_transfer_info(const ug4gb_gmg *m, int level, int which, int *num_rows, int *num_cols,
                            int64_t *nnz);
/* the multigrid's FP64 operator of a level (base..top): re-assembled, or
   R A P with set_rap (what AssembledMultiGridCycle writes as "LevelMatrix"
   through write_debug, mg_solver_impl.hpp:898-902,966-970) */
UG4GB_API int ug4gb_gmg_level_info(const ug4gb_gmg *m, int level, int *num_rows, int64_t *nnz);
UG4GB_API int ug4gb_gmg_export_level(const ug4gb_gmg *m, int level, int *rowptr, int *col, double *val);
UG4GB_API int ug4gb_gmg_export_transfer(const ug4gb_gmg *m, int level, int which, int *rowptr, int *col, double *val);
UG4GB_API void ug4gb_gmg_destroy(ug4gb_gmg *m);

/* ------------------------------------------------------------- Krylov -- */
/* Replaces CG / BiCGStab with StdConvCheck (convergence_check_impl.h:85-172) */
UG4GB_API int ug4gb_solver_create(ug4gb_ctx *ctx, int kind, ug4gb_solver **out);
UG4GB_API int ug4gb_solver_set_preconditioner(ug4gb_solver *s, ug4gb_gmg *m);
UG4GB_API int ug4gb_solver_set_convergence_check(ug4gb_solver *s, int max_steps, double min_defect,
                                       double rel_reduction);
/* BiCGStab::set_restart (lib_algebra/operator/linear_solver/bicgstab.h:387):
   restart (r0 = r, p = v = 0) whenever the convergence check's step count,
   which counts half steps, is a multiple of num_restarts; 0 = off (default).
   BiCGStab::set_min_orthogonality (bicgstab.h:390): restart in the next
   iteration when |(r, r0)| <= min_ortho |r| |r0| (default 0).  Both are
   UG4GB_ERR_INVALID for a CG solver. */
UG4GB_API int ug4gb_solver_set_restart(ug4gb_solver *s, int num_restarts);
UG4GB_API int ug4gb_solver_set_min_orthogonality(ug4gb_solver *s, double min_ortho);
/* ILinearOperatorInverse::init (preconditioned_linear_operator_inverse.h:123) */
UG4GB_API int ug4gb_solver_init(ug4gb_solver *s, const ug4gb_matrix *A);
/* apply_return_defect (cg.h:103, bicgstab.h:112): x is the start iterate and
   the result, b is overwritten by the final defect */
UG4GB_API int ug4gb_solver_apply_return_defect(ug4gb_solver *s, ug4gb_vector *x, ug4gb_vector *b);
/* apply (preconditioned_linear_operator_inverse.h:150): b is kept */
UG4GB_API int ug4gb_solver_apply(ug4gb_solver *s, ug4gb_vector *x, const ug4gb_vector *b);
/* host-buffer solve: copies b in, solves from x = 0, copies x out */
UG4GB_API int ug4gb_solver_solve_host(ug4gb_solver *s, const double *b_host, double *x_host);
UG4GB_API int ug4gb_solver_get_stats(const ug4gb_solver *s, int *steps, double *initial_defect,
                           double *final_defect, int *converged);
/* defect history: hist[0] = initial defect, hist[i] = defect after step i */
UG4GB_API int ug4gb_solver_get_history(const ug4gb_solver *s, double *hist, int capacity);
UG4GB_API void ug4gb_solver_destroy(ug4gb_solver *s);

/* ------------------------------------------------------------- Newton -- */
/* NewtonSolver (lib_disc/operator/non_linear_operator/newton_solver/newton.h:62,
   newton_impl.h:171-340) without line search: the operator is the stationary
   FV1 discretisation (init(nw, d, NULL)) or a prepared ThetaTimeStep
   (init(nw, NULL, td)); every step assembles the jacobian, initialises the
   linear solver and its multigrid with it, solves J c = d from c = 0, sets
   u -= c and the Dirichlet values, and assembles the new defect.  Convergence
   by StdConvCheck rules on |d|; UG4GB_ERR_NOT_CONVERGED when the step limit is
   reached first, the linear solver's code when a linear solve fails. */
typedef struct ug4gb_newton ug4gb_newton;
UG4GB_API int ug4gb_newton_create(ug4gb_ctx *ctx, ug4gb_newton **out);
UG4GB_API int ug4gb_newton_set_linear_solver(ug4gb_newton *nw, ug4gb_solver *s);
UG4GB_API int ug4gb_newton_set_convergence_check(ug4gb_newton *nw, int max_steps, double min_defect,
                                                 double reduction);
UG4GB_API int ug4gb_newton_init(ug4gb_newton *nw, ug4gb_disc *d, ug4gb_timedisc *td);
UG4GB_API int ug4gb_newton_prepare(ug4gb_newton *nw, ug4gb_vector *u);     /* Dirichlet values into u */
UG4GB_API int ug4gb_newton_apply(ug4gb_newton *nw, ug4gb_vector *u);
/* Newton steps, |d| at start and end, and the linear solver's steps per Newton step */
UG4GB_API int ug4gb_newton_get_stats(const ug4gb_newton *nw, int *steps, double *initial_defect,
                                     double *final_defect, int *lin_steps, int capacity);
/* |d| after each Newton step (entry 0: start); returns the number available */
UG4GB_API int ug4gb_newton_get_history(const ug4gb_newton *nw, double *defects, int capacity);
/* StandardLineSearch (lib_disc/operator/non_linear_operator/line_search.h:
   115-400; the constructor's defaults 10, 1.0, 0.5, 0.25, false, false,
   1e10) for every Newton step: set_maximum_steps, set_lambda_start,
   set_reduce_factor, set_suff_descent_factor, set_accept_best, set_check_all,
   set_maximum_defect.  A failed search ends apply with
   UG4GB_ERR_NOT_CONVERGED, as NewtonSolver::apply returns false. */
UG4GB_API int ug4gb_newton_set_line_search(ug4gb_newton *nw, int max_steps, double lambda_start,
                                          double lambda_reduce, double suff_descent_factor, int accept_best,
                                          int check_all, double max_defect);
/* NewtonSolver::set_reassemble_J_freq (newton.h:156, newton_impl.h:246): the
   jacobian is assembled in Newton steps 0, freq, 2 freq, ... (0: every step);
   the linear solver and its multigrid are initialised every step, as there */
UG4GB_API int ug4gb_newton_set_reassemble_J_freq(ug4gb_newton *nw, int freq);
/* jacobian assemblies of the last apply */
UG4GB_API int ug4gb_newton_num_jacobian_assemblies(const ug4gb_newton *nw);
UG4GB_API int ug4gb_newton_clear_line_search(ug4gb_newton *nw);
/* per Newton step of the last apply: line-search tries evaluated and the
   lambda of the accepted solution; returns the number of steps recorded */
UG4GB_API int ug4gb_newton_get_line_search_history(const ug4gb_newton *nw, int *tries, double *lambdas,
                                                  int capacity);
UG4GB_API void ug4gb_newton_destroy(ug4gb_newton *nw);

/* ------------------------------------------------------------ adjoint -- */
/* No ugcore counterpart.  Gradients of J(u) with A(m) u = b(f), K = exp(m):
   dJ/dm_e = -K_e * sum_{i not Dirichlet} lambda_i (A1_e u_e)_i   (per element)
   dJ/df_i = lambda_i * |SCV(i)|                                  (per vertex)
   where A^T lambda = dJ/du, A1_e the unit-coefficient element matrix.
   u, lambda: top-level vectors; grad: host or device array. */
UG4GB_API int ug4gb_disc_grad_logk(ug4gb_disc *d, const ug4gb_vector *u, const ug4gb_vector *lambda, double *grad);
UG4GB_API int ug4gb_disc_grad_source(ug4gb_disc *d, const ug4gb_vector *lambda, double *grad);

/* ------------------------------------------------------- matrix files -- */
/* MatrixMarket and ConnectionViewer files, byte-identical to ugcore's writers.
   MatrixMarket write: SaveMatrixToMTX (lib_disc/function_spaces/
   grid_function_util.h:761-778) / MatrixIOMtx::write_from (lib_algebra/common/
   matrixio/matrix_io_mtx.h:243-275): the filename must end in ".mtx"; exact
   symmetry / skew-symmetry detection, lower triangle only for those, zero
   values skipped, entries column by column, values "%.13e"; comment NULL =
   "%Generated with ug4.", "" = no comment line, a comment not starting with
   '%' gets one prepended.  Read: MatrixIOMtx::read_into (matrix_io_mtx.h:
   202-236): coordinate real/integer files; symmetric and skew-symmetric
   entries are mirrored; a later assignment to a position replaces an earlier
   one; stored zeros are kept.
   ConnectionViewer: WriteMatrixToConnectionViewer / SaveMatrixForConnection
   Viewer (grid_function_util.h:714-749, connection_viewer_output.h:114-140;
   ".mat"), SaveVectorForConnectionViewer (connection_viewer_output.h:395-420;
   ".vec"), LoadVector / ReadVector (grid_function_util.h:917-923,
   connection_viewer_input.h:104-150).  Positions are the vertices of the
   given grid level.
   The ug4gb_io_* functions take host arrays (CRS with strictly increasing
   columns per row) and need no context or GPU; a message goes to err (may be
   NULL).  ug4gb_io_read_mtx_info gives the sizes to allocate for
   ug4gb_io_read_mtx (rowptr: num_rows + 1, col / val: nnz). */
UG4GB_API int ug4gb_io_write_mtx(int num_rows, int num_cols, const int *rowptr, const int *col, const double *val,
                                 const char *filename, const char *comment, char *err, int err_capacity);
UG4GB_API int ug4gb_io_read_mtx_info(const char *filename, int *num_rows, int *num_cols, int64_t *nnz, char *err,
                                     int err_capacity);
UG4GB_API int ug4gb_io_read_mtx(const char *filename, int *rowptr, int *col, double *val, char *err,
                                int err_capacity);
UG4GB_API int ug4gb_io_write_cv_matrix(int num_rows, const int *rowptr, const int *col, const double *val, int dim,
                                       const double *positions, const char *filename, char *err, int err_capacity);
UG4GB_API int ug4gb_io_write_cv_vector(int n, const double *values, int dim, const double *positions,
                                       const char *filename, char *err, int err_capacity);
UG4GB_API int ug4gb_io_read_cv_vector(const char *filename, int n, double *values, char *err, int err_capacity);
/* the same for device matrices and vectors (copied through the host) */
UG4GB_API int ug4gb_matrix_write_mtx(const ug4gb_matrix *A, const char *filename, const char *comment);
UG4GB_API int ug4gb_matrix_read_mtx(ug4gb_matrix *A, const char *filename);
UG4GB_API int ug4gb_matrix_write_cv(const ug4gb_matrix *A, const ug4gb_grid *g, int level, const char *filename);
UG4GB_API int ug4gb_vector_write_cv(const ug4gb_vector *v, const ug4gb_grid *g, int level, const char *filename);
UG4GB_API int ug4gb_vector_read_cv(ug4gb_vector *v, const char *filename);

#ifdef __cplusplus
}
#endif
#endif
