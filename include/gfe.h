/* gfe.h -- C ABI of the GB300 finite-element assembly engine (libgfe.so).
 *
 * The engine replaces OpenCMISS-Iron's element-loop hot path: the Gauss-point stiffness /
 * residual / Jacobian evaluation and its scatter into compressed-row storage.  Each entry point
 * below is a batched, whole-mesh equivalent of an Iron routine that loops over elements one at a
 * time; the citation beside each names the Iron routine (file:line, relative to the Iron source
 * tree) it stands in for.
 *
 * Conventions
 *  - Every function returns an int status: GFE_OK (0) or a negative GFE_ERR_* code.  The message
 *    of the last failure on the calling host thread is copied out by gfe_last_error().  This
 *    mirrors Iron's (err, error) pair and cmfe_ExtractErrorMessage (src/opencmiss_iron.F90:13159).
 *  - Array arguments are DEVICE pointers unless their name ends in _host.
 *  - Node, element and DOF numbers are 0-based in element/connectivity arrays; the CSR structure
 *    row_ptr / col_idx is 1-based, exactly as Iron stores it (src/types.F90:909-929).
 *  - Nodal field parameters are in Iron's separated-component order: all DOFs of component 1,
 *    then component 2, ... (src/field_routines.F90:10050-10060).
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default stream.  All work is
 *    stream-ordered; functions that must report a count to the host synchronise that stream.
 *  - Element connectivity uses Iron's local node order (xi1 fastest,
 *    src/basis_routines.F90:3243-3370).
 */
#ifndef GFE_H
#define GFE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFE_OK 0
#define GFE_ERR_ARG (-1)       /* invalid argument (sizes, null pointers, unsupported option) */
#define GFE_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define GFE_ERR_STRUCTURE (-3) /* an element entry has no slot in the CSR structure */
#define GFE_ERR_NUMERIC (-4)   /* non-finite value, non-positive Jacobian, or breakdown */
#define GFE_ERR_NOCONV (-5)    /* iterative solve did not reach its tolerance */
#define GFE_ERR_TIMEOUT (-6)   /* a bounded device-side wait ran out */
#define GFE_ERR_NOMEM (-7)     /* device allocation failed or an admission budget was exceeded */

/* precision selectors */
#define GFE_FP64 0  /* plain: element arithmetic and storage in FP64 */
#define GFE_MIXED 1 /* FP32 element arithmetic, FP64 accumulation */
#define GFE_MIXED_DF 2 /* float-float element arithmetic on the FP32 pipes (~48-bit), FP64 accumulation */
#define GFE_TC_TF32X3 3 /* MR Jacobian, hexahedral gfe_laplace_assemble_tp: tensor-core (tcgen05) TF32
                           contraction, 3-pass split (~FP32 accuracy) */
#define GFE_TC_TF32 4   /* MR Jacobian: tensor-core (tcgen05) TF32 contraction, one pass (~1e-3 relative) */

/* ---- library -------------------------------------------------------------------------- */

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int gfe_version(void);

/* Copy the last error message of this host thread into buf (NUL-terminated, truncated to len).
 * Returns the message length.  Replaces cmfe_ExtractErrorMessage (src/opencmiss_iron.F90:13159). */
int gfe_last_error(char* buf, int len);

/* Clear the CUDA runtime's error state of the calling host thread and return the cleared code
 * (0: none).  Each entry point reports the launch errors of its own launches by that state, so a
 * caller that mixes this library with other CUDA code calls it before an entry point; an error
 * left there by other code is then not reported as the entry point's.  The library's own failures
 * leave nothing behind.  No counterpart in the reference. */
int gfe_clear_stale_error(void);

/* The library's working memory (Krylov vectors, element matrices, Gauss-point blocks) comes from
 * the current device's default stream-ordered memory pool, whose release threshold the library
 * raises to 4 GiB so that freed scratch stays mapped for the next call.  This call synchronises
 * the device and returns all unused pool memory to the device (for a caller that needs it, e.g.
 * after an out-of-memory failure).  No counterpart in the reference. */
int gfe_release_scratch(void);

/* Read and clear the device error word (bit set of GFE_DEVERR_* raised by kernels). */
int gfe_device_errors(uint32_t* bits_host, void* stream);

/* Route this host thread's kernels to the caller's device error word (a zeroed uint32 in device
 * memory), or back to the library's per-device word with NULL.  A host that runs independent work
 * from several threads (a serving loop) gives each thread its own word, so that one request's
 * errors are neither reported for nor cleared by another.  Kernels captured into a CUDA graph keep
 * the word that was current at capture. */
int gfe_set_thread_error_word(uint32_t* dev_word);

#define GFE_DEVERR_SLOT 1u     /* CSR slot not found during a scatter */
#define GFE_DEVERR_JACOBIAN 2u /* non-positive Jacobian / det(F) at a Gauss point */
#define GFE_DEVERR_NONFINITE 4u
#define GFE_DEVERR_TIMEOUT 8u

/* ---- stage timing ------------------------------------------------------------------------ */

/* When enabled, entry points record CUDA events on their stream around the kernels of each
 * stage below; gfe_profile_read() waits for the recorded events and returns the summed device
 * time (ms) and the number of kernel launches of a stage since the last reset.  Off by default.
 * Plays the role of Iron's per-assembly timing output (src/equations_set_routines.F90:1239-1353). */
#define GFE_STAGE_LAPLACE_ELEMENTS 0 /* element + scatter kernels of gfe_laplace_assemble */
#define GFE_STAGE_SPMV 1             /* SpMV kernels of the CG solver */
#define GFE_STAGE_MR_RESIDUAL 2
#define GFE_STAGE_MR_JACOBIAN 3
#define GFE_STAGE_COUNT 8
int gfe_profile_enable(int on);
int gfe_profile_read(int stage, double* ms_host, int64_t* launches_host, int reset);

/* Diagnostic: runs a dependent fused-multiply-add chain on every SM and reports the device's
 * sustained arithmetic rate in GFLOP/s (2 flops per FMA) for precision GFE_FP64 or GFE_MIXED
 * (FP32).  Used as the FP64 / FP32 pipe roof of the element kernels. */
int gfe_probe_fma_rate(int32_t precision, double* gflops_host, void* stream);

/* ---- context and mesh handles ------------------------------------------------------------ */

/* A context owns what Iron keeps per rank around its element loops: the CUDA stream the work is
 * ordered on (borrowed; NULL = legacy default stream), a device error word of its own (kernels
 * launched through the context report there, read with gfe_ctx_device_errors), and a cache of
 * mesh structures keyed by a hash of the connectivity.  Use one context per host thread.  The
 * context is created on, and must be used with, the current device.  Iron's counterparts are the
 * equations set's matrices and their structure (EquationsMatrices_CreateFinish ->
 * EquationsMatrix_StructureCalculate, src/equations_matrices_routines.F90:4316-4602), built once and
 * reused by every assembly, and the per-rank error state of src/base_routines.F90. */
typedef struct gfe_ctx gfe_ctx;
typedef struct gfe_mesh gfe_mesh;
int gfe_ctx_create(void* stream, gfe_ctx** ctx);
/* Frees the context and its error word; structures still used by live mesh handles are freed with
 * the last of them.  Synchronises the context's stream. */
int gfe_ctx_destroy(gfe_ctx* ctx);
/* Read and clear the context's device error word (GFE_DEVERR_* bits).  Synchronises the stream. */
int gfe_ctx_device_errors(gfe_ctx* ctx, uint32_t* bits_host);
/* Number of distinct mesh structures in the context's cache. */
int gfe_ctx_cached_meshes(gfe_ctx* ctx, int32_t* count_host);

/* Mesh handle of a general mesh: elem_nodes_host [n_elem][nodes_per_elem] 0-based node numbers in
 * host memory.  The CSR structure (as gfe_csr_structure: Iron's, 1-based) and a greedy element
 * colouring are built on the first handle of a connectivity and shared by later handles of the
 * same connectivity (looked up by hash, confirmed by comparison).  Synchronises the stream. */
int gfe_mesh_create(gfe_ctx* ctx, int32_t n_elem, int32_t nodes_per_elem, const int32_t* elem_nodes_host,
                    int32_t n_nodes, gfe_mesh** mesh);
/* Mesh handle of Iron's regular generated mesh of nx x ny x nz trilinear hexahedra
 * (GENERATED_MESH_REGULAR_TYPE, src/generated_mesh_routines.F90:1568-1640): the connectivity is
 * generated, the structure verified as the clipped 27-point stencil, and the assembly may take the
 * row-owning regular-mesh kernel. */
int gfe_mesh_create_regular(gfe_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, gfe_mesh** mesh);
int gfe_mesh_destroy(gfe_mesh* mesh);
/* The mesh's CSR structure (device pointers owned by the context's cache, valid while the handle
 * lives): row_ptr [n_rows + 1], col_idx [nnz], both 1-based as Iron stores them; any output may be
 * NULL.  The analogue of cmfe_DistributedMatrix_StorageLocationsGet (src/opencmiss_iron.F90:45823). */
int gfe_mesh_csr(const gfe_mesh* mesh, const int32_t** row_ptr, const int32_t** col_idx, int64_t* nnz,
                 int32_t* n_rows);
/* Laplace assembly on a trilinear mesh handle (gfe_laplace_assemble, or on a regular mesh with an
 * FP32-pipe precision gfe_laplace_assemble_regular), on the context's stream and error word:
 * coords [3][n_nodes], kappa_e [n_elem] or NULL, values [nnz] (FP64) out, values32 / rhs optional.
 * Replaces EquationsSet_AssembleStaticLinearFEM (src/equations_set_routines.F90:1203-1364) for the
 * Laplace equations set. */
int gfe_assemble_laplace(gfe_ctx* ctx, const gfe_mesh* mesh, const double* coords, const double* kappa_e,
                         double* values, float* values32, double* rhs, int32_t precision);
/* Jacobi-CG on the mesh's matrix (gfe_cg_solve on the context's stream and error word). */
int gfe_solve_laplace(gfe_ctx* ctx, const gfe_mesh* mesh, const double* values, const float* values32,
                      const double* f, const uint8_t* fixed, double* x, double rtol, int32_t max_iters,
                      int32_t precision, int32_t* iters_host, double* rel_host);

/* ---- CSR structure (K3) ------------------------------------------------------------------ */

/* Compressed-row sparsity of an FEM matrix whose rows and columns are the DOFs of one field
 * variable.  Replaces EquationsMatrix_StructureCalculate / JacobianMatrix_StructureCalculate
 * (src/equations_matrices_routines.F90:4316-4602, :4609-4948): for every row DOF, the union of all
 * DOFs of all elements that contain it, sorted ascending, unique, 1-based.
 *  elem_dofs  [n_elem][dofs_per_elem] 0-based DOF numbers of each element (all components)
 *  row_ptr    [n_dofs+1] out, 1-based
 *  col_idx    [col_capacity] out, 1-based; may be NULL to query nnz only
 *  nnz_host   out: number of structural non-zeros
 * Synchronises `stream`.  Allocates and frees its scratch on `stream`. */
int gfe_csr_structure(int32_t n_elem, int32_t dofs_per_elem, const int32_t* elem_dofs, int32_t n_dofs,
                      int32_t* row_ptr, int32_t* col_idx, int64_t col_capacity, int64_t* nnz_host, void* stream);

/* ---- solver system: Dirichlet elimination -------------------------------------------------- */

/* The reduced system Iron hands to its linear solver for one linear equations set with Dirichlet
 * conditions on one rank: rows and columns of fixed DOFs removed, their coupling moved to the
 * right-hand side.  Replaces, for that case, the solver mapping (src/solver_mapping_routines.F90:
 * 398-520), SOLVER_MATRIX_STRUCTURE_CALCULATE (src/solver_matrices_routines.F90:1612-2431),
 * SOLVER_MATRIX_EQUATIONS_MATRIX_ADD (:806-1023) and the linear branch of
 * SOLVER_MATRICES_STATIC_ASSEMBLE (src/solver_routines.F90:14025-15050); structure, values and
 * right-hand side are bit-identical to Iron's.  Equations CSR 1-based (n rows), fixed[n] != 0
 * marks a Dirichlet DOF.
 *
 * gfe_solver_structure: solver_of_dof[n] out (0-based solver number, -1 for a fixed DOF; free
 * DOFs numbered in ascending order), s_row_ptr[n_free + 1] out (capacity n + 1), s_col_idx out
 * (1-based; may be NULL to query nnz only), n_free_host / nnz_host out.  Synchronises `stream`. */
int gfe_solver_structure(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const uint8_t* fixed,
                         int32_t* solver_of_dof, int32_t* s_row_ptr, int32_t* s_col_idx, int64_t col_capacity,
                         int32_t* n_free_host, int64_t* nnz_host, void* stream);
/* Solver matrix values from the equations matrix values: every free-free entry, 0 + K(i, j), into
 * s_values, and/or rounded to FP32 into s_values32 (for mixed-precision solves); either may be NULL. */
int gfe_solver_matrix(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                      const int32_t* solver_of_dof, const int32_t* s_row_ptr, double* s_values, float* s_values32,
                      void* stream);
/* Solver right-hand side: for free row i, in ascending order of the contributing equations row r,
 * f(i) at r = i and -1 * K(i, r) * u(r) for each fixed column r with |u(r)| and |K(i, r)| at least
 * ZERO_TOLERANCE = 5 EPSILON(1.0_DP).  f (equations RHS) may be NULL (zero).  u holds the
 * Dirichlet values at fixed DOFs.  col_listed (may be NULL = all): the fixed columns whose
 * coupling Iron moves to the right-hand side -- its Dirichlet column lists hold only DOFs on
 * boundary nodes (src/equations_matrices_routines.F90:4531-4561). */
int gfe_solver_rhs(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values, const double* f,
                   const double* u, const uint8_t* fixed, const uint8_t* col_listed, const int32_t* solver_of_dof,
                   double* s_rhs, void* stream);
/* Copy a solver solution back into the dependent vector: u[i] = x[solver_of_dof[i]] for free i
 * (the update of the dependent field from the solver variables, coupling coefficient 1). */
int gfe_solver_update_dependent(int32_t n, const int32_t* solver_of_dof, const double* x, double* u, void* stream);

/* The same structure for the Jacobian of Iron's regular generated mesh of nx x ny x nz triquadratic
 * displacement / trilinear pressure elements (DOFs: the three displacement components on the
 * (2n+1)^3 node grid, then the pressure on the (n+1)^3 vertex grid, nodes xi1 fastest), in closed
 * form: every row is the clipped boxes of displacement and pressure nodes of the elements around
 * its node, in ascending order.  Bit-identical to gfe_csr_structure of that mesh's element DOFs
 * (JacobianMatrix_StructureCalculate, src/equations_matrices_routines.F90:4609-4948), without the
 * per-row sort.  Arguments as for gfe_csr_structure.  Synchronises `stream`. */
int gfe_mr_regular_structure(int32_t nx, int32_t ny, int32_t nz, int32_t* row_ptr, int32_t* col_idx,
                             int64_t col_capacity, int64_t* nnz_host, void* stream);

/* ---- Laplace / diffusion assembly (K1 + K2) -------------------------------------------- */

/* Assemble the global stiffness matrix of the Laplace equation on trilinear-Lagrange hexahedra
 * with 2x2x2 Gauss quadrature into a fixed CSR structure, and zero the RHS.
 * Replaces the element loop of EquationsSet_AssembleStaticLinearFEM
 * (src/equations_set_routines.F90:1203-1364) around LaplaceEquation_FiniteElementCalculate
 * (src/Laplace_equations_routines.F90:433-747, standard and generalised-isotropic subtypes) and
 * EquationsMatrices_ElementAdd -> MATRIX_VALUES_ADD_DP2 (src/equations_matrices_routines.F90:1140-1265,
 * src/matrix_vector.F90:3202-3240).
 *  elem_nodes   [n_elem][8] 0-based node numbers (Iron local node order)
 *  coords       [3][n_nodes] geometric field, separated components
 *  kappa        [n_elem] element conductivity (generalised subtype, isotropic) or NULL (standard)
 *  color_elems  [n_elem] element numbers grouped by colour: no two elements of one colour share a node
 *  color_ptr_host [n_colors+1] host offsets into color_elems
 *  row_ptr/col_idx  CSR structure from gfe_csr_structure (1-based), nnz entries
 *  values       [nnz] out: assembled matrix (FP64)
 *  values32     [nnz] optional out (may be NULL): FP32 copy of the matrix for mixed-precision solves
 *  rhs          [n_nodes] optional out (may be NULL): zeroed RHS vector
 *  precision    GFE_FP64 or GFE_MIXED
 * The scatter is deterministic: colours are processed in order and each CSR entry receives at
 * most one addition per colour.  Asynchronous: device-side failures (missing CSR slot, degenerate
 * element) are reported through gfe_device_errors(). */
int gfe_laplace_assemble(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes, const double* coords,
                         const double* kappa, const int32_t* color_elems, const int32_t* color_ptr_host,
                         int32_t n_colors, const int32_t* row_ptr, const int32_t* col_idx, int64_t nnz,
                         double* values, float* values32, double* rhs, int32_t precision, void* stream);

/* Generalised Laplace: the conductivity is a full symmetric tensor in a material frame.
 * Replaces LaplaceEquation_FiniteElementCalculate's EQUATIONS_SET_GENERALISED_LAPLACE_SUBTYPE
 * branch (src/Laplace_equations_routines.F90:585-707) with Coordinates_MaterialSystemCalculate
 * (src/coordinate_routines.F90:3841-3947, 4020-4127) inside the same element loop and scatter as
 * gfe_laplace_assemble.  FP64.
 *  conductivity [6][n_elem] element-constant materials field, Iron's component order
 *               K11 K22 K33 K12 K23 K13 in material coordinates
 *  fibre        [n_angles][n_nodes] nodal fibre field (fibre, imbrication, sheet angles in radians,
 *               interpolated trilinearly), or NULL: no fibre field (the material frame is then the
 *               normalised columns of dX/dxi, as Iron's)
 *  n_angles     1..3 with a fibre field, 0 without
 * Other arguments as gfe_laplace_assemble; values are not symmetric in general (Iron rotates the
 * tensor into xi space by a similarity transform).  Asynchronous, device errors as
 * gfe_laplace_assemble (a non-finite conductivity raises GFE_DEVERR_NONFINITE). */
int gfe_laplace_assemble_generalised(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes, const double* coords,
                                     const double* conductivity, const double* fibre, int32_t n_angles,
                                     const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                                     const int32_t* row_ptr, const int32_t* col_idx, int64_t nnz, double* values,
                                     double* rhs, void* stream);

/* Same assembly for Iron's regular generated mesh of nx x ny x nz trilinear elements
 * (GENERATED_MESH_REGULAR_TYPE, src/generated_mesh_routines.F90:1568-1640: nodes and elements
 * numbered xi1 fastest), whose topology is implicit: no connectivity, colouring or column indices
 * are read.  row_ptr must be the structure of that mesh (gfe_csr_structure of its connectivity,
 * verified once with gfe_laplace_regular_check).  Every CSR entry is written exactly once (no
 * zeroing pass); values32 (optional) receives the FP32 copy in the same pass; rhs is zeroed. */
int gfe_laplace_assemble_regular(int32_t nx, int32_t ny, int32_t nz, const double* coords, const double* kappa,
                                 const int32_t* row_ptr, double* values, float* values32, double* rhs,
                                 int32_t precision, void* stream);

/* The same assembly with a caller-owned device workspace (16-byte aligned) of
 * gfe_laplace_regular_workspace_bytes(nx, ny, nz, precision) bytes, so that nothing is allocated:
 * the form to capture into a CUDA graph.  The workspace holds the converted coordinates and, for
 * GFE_MIXED_DF, every element's Gauss-point metrics and element matrix (float-float, 672 bytes an
 * element): the float-float element work runs as a metric kernel and a contraction kernel, each
 * element once, and the rows are then gathered from the element matrices.  workspace may be NULL
 * (then it is allocated and freed on `stream`, as gfe_laplace_assemble_regular does). */
int64_t gfe_laplace_regular_workspace_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t precision);
int gfe_laplace_assemble_regular_ws(int32_t nx, int32_t ny, int32_t nz, const double* coords, const double* kappa,
                                    const int32_t* row_ptr, double* values, float* values32, double* rhs,
                                    int32_t precision, void* workspace, void* stream);

/* The rows of node layers [layer_begin, layer_end) only (layer = node index along xi3; layer_begin a
 * multiple of 8): those rows form one contiguous range of the CSR values, so an assembly split into
 * layer slabs can copy each slab's values to the host while the next slab computes.
 * convert_coords: convert the coordinates into the workspace first (needed in the first call of an
 * assembly; later calls of the same assembly pass 0 and reuse it; requires a workspace).  An empty
 * range (layer_begin == layer_end) with convert_coords only converts, so that slab calls on
 * several streams can all start once the conversion is done. */
int gfe_laplace_assemble_regular_layers(int32_t nx, int32_t ny, int32_t nz, const double* coords, const double* kappa,
                                        const int32_t* row_ptr, double* values, float* values32, double* rhs,
                                        int32_t precision, void* workspace, int32_t layer_begin, int32_t layer_end,
                                        int32_t convert_coords, void* stream);

/* End-to-end assembly with host buffers: the regular-mesh assembly above with the geometry and
 * conductivity uploaded from host memory and the FP64 CSR values returned to host memory, as
 * Iron's caller sees the element loop (host arrays in, the assembled matrix in host memory out).
 * The work is pipelined over slabs of node layers (the first of 8 layers, then slab_layers each;
 * 0 = 16): per slab, the coordinate and conductivity layers it reads are copied in and converted
 * on an input stream, the slab is assembled on one of two alternating compute streams, and its
 * rows -- one contiguous range of the CSR values -- are copied to values_host on an output
 * stream while later slabs compute.  coords [3][N] / kappa [n_elem] are the device copies the
 * uploads fill (coords_host / kappa_host NULL: the device copy is already current; kappa NULL:
 * unit conductivity); values [nnz] is the device CSR value array.  Host buffers should be pinned
 * for the copies to overlap.  The FP32-pipe precisions need a 16-byte aligned workspace of
 * gfe_laplace_regular_workspace_bytes bytes; nothing is allocated.  Asynchronous: the pipeline's
 * own streams start after the work already on `stream`, and `stream` waits for all of them, so
 * values_host is complete once `stream` has reached this point.  Slab boundaries come from the
 * closed-form entry count of the clipped 27-point stencil, so row_ptr must be the structure of the
 * regular mesh (gfe_laplace_regular_check). */
int gfe_laplace_assemble_regular_host(int32_t nx, int32_t ny, int32_t nz, const double* coords_host,
                                      const double* kappa_host, double* coords, double* kappa,
                                      const int32_t* row_ptr, double* values, double* values_host, double* rhs,
                                      int32_t precision, void* workspace, int32_t slab_layers, void* stream);

/* The Laplace assembly of gfe_laplace_assemble on hexahedra of any tensor-product basis of Lagrange
 * order 1..3 or cubic Hermite per direction, with 1..4 Gauss points per direction, and on linear,
 * quadratic or cubic tetrahedra (Iron's element routine is basis-generic: LaplaceEquation_FiniteElementCalculate,
 * src/Laplace_equations_routines.F90:433-747, with the quadrature of BASIS_QUADRATURE_CREATE,
 * src/basis_routines.F90:3720-4090, and Gauss_Simplex, :6898-7600).
 *  order[3]   host array of Iron's interpolation specification per xi (INTERPOLATION_XI):
 *             1, 2, 3 = linear / quadratic / cubic Lagrange, 4 = cubic Hermite; 7 / 8 / 9 in all
 *             three = linear / quadratic / cubic simplex (tetrahedra of 4 / 10 / 20 nodes in
 *             Iron's node order)
 *  n_gauss[3] host array of Gauss points per xi; for tetrahedra n_gauss[0] is the Gauss_Simplex
 *             order 1..5 (1, 4, 5, 11 or 14 points)
 *  elem_nodes [n_elem][nns] 0-based element parameter DOFs in Iron's order (local nodes xi1 fastest,
 *             then each node's derivatives: value, d/ds1, d/ds2, d2/ds1ds2, d/ds3, ... over the
 *             Hermite directions); n_nodes = number of DOFs; coords [3][n_nodes] geometric
 *             parameters per DOF (positions and, for Hermite, derivatives)
 *  scale      optional [n_elem][nns] element parameter scale factors: the geometric parameters are
 *             interpolated scaled and the element matrix is scaled as K(m,n) SF(m) SF(n)
 *             (src/Laplace_equations_routines.F90:555-579); NULL = unscaled
 *  colouring and CSR as for gfe_laplace_assemble
 *  slots      optional [n_elem][nns][nns] CSR positions of the element entries from
 *             gfe_laplace_tp_slot_map (the same positions Iron's search finds, computed once per
 *             mesh); NULL = Iron's search per entry pair during the assembly
 *  values32 (optional) FP32 copy of the assembled values
 * precision GFE_FP64, GFE_MIXED (FP32 element arithmetic), GFE_MIXED_DF (float-float) or, for
 * hexahedral bases, GFE_TC_TF32X3: the contraction K(m,n) = sum_g dphi_m^T M_g dphi_n as an
 * M = 128 tcgen05 product (FP32 metrics, TF32 head / tail operands, FP32 accumulation in tensor
 * memory; about FP32 accuracy).  The matrix and rhs are zeroed first; each pair of element nodes
 * is added through Iron's CSR search.
 * Asynchronous; device-side failures are reported through gfe_device_errors(). */
int gfe_laplace_assemble_tp(const int32_t* order, const int32_t* n_gauss, int32_t n_elem, int32_t n_nodes,
                            const int32_t* elem_nodes, const double* coords, const double* scale, const double* kappa,
                            const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                            const int32_t* row_ptr, const int32_t* col_idx, int64_t nnz, const int32_t* slots,
                            double* values, float* values32, double* rhs, int32_t precision, void* stream);

/* Element slot map of a basis-generic mesh: slots[e][m][n] = the 0-based CSR position of the entry
 * (row elem_nodes[e][m], column elem_nodes[e][n]) found by Iron's row search (bisection to a
 * width of 10, then a linear scan: MATRIX_VALUES_ADD_DP2, src/matrix_vector.F90:3202-3240), or
 * -1 where the structure lacks it (the assembly then raises GFE_DEVERR_SLOT).  nns <= 64;
 * positions must fit int32 (nnz <= 2^31 - 1).  The map depends on the structure only: compute it
 * once per mesh and pass it to every gfe_laplace_assemble_tp call; for 27- to 64-node elements the
 * per-entry search otherwise dominates the assembly.  Asynchronous on `stream`. */
int gfe_laplace_tp_slot_map(int32_t n_elem, int32_t nns, const int32_t* elem_nodes, const int32_t* row_ptr,
                            const int32_t* col_idx, int64_t nnz, int32_t* slots, void* stream);

/* Number of CSR rows/entries that differ from the clipped 27-point stencil of the regular mesh
 * (0 = the structure is the one gfe_laplace_assemble_regular writes).  Synchronises `stream`. */
int gfe_laplace_regular_check(int32_t nx, int32_t ny, int32_t nz, const int32_t* row_ptr, const int32_t* col_idx,
                              int64_t* mismatches_host, void* stream);

/* Element matrices only (no scatter): K_out[n_elem][8][8] row-major, for parity checks of the
 * element routine itself (LaplaceEquation_FiniteElementCalculate). */
int gfe_laplace_element_matrices(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes, const double* coords,
                                 const double* kappa, double* K_out, int32_t precision, void* stream);

/* ---- finite elasticity: Mooney-Rivlin, mixed u-p (K4, K5) -------------------------------- */

/* Mesh of the mixed formulation: eq2 [n_elem][27] triquadratic element nodes (0-based, numbers of
 * the n_q2 quadratic-grid nodes), elin [n_elem][8] trilinear pressure nodes (0-based numbers of the
 * n_lin pressure-component nodes), xg [3][n_q2] geometric field.  The dependent vector `dep` of one
 * problem holds, in Iron's separated order, the deformed positions z1, z2, z3 over the quadratic
 * nodes followed by the pressure over the linear nodes (ndof = 3 n_q2 + n_lin).  Material
 * parameters cpar = (c10, c01) per problem.  3x3x3 Gauss quadrature. */

/* Global residual of `batch` independent problems on one mesh (dep and R are [batch][ndof], cpar
 * is [batch][2]).  Replaces the element loop of EquationsSet_ResidualEvaluateStaticFEM
 * (src/equations_set_routines.F90:5164-5286) around the MOONEY_RIVLIN_SUBTYPE branch of
 * FiniteElasticity_FiniteElementResidualEvaluate (src/finite_elasticity_routines.F90:1669-1756).
 * Colouring as in gfe_laplace_assemble.  R is zeroed first. */
int gfe_mr_residual(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t n_q2, int32_t n_lin,
                    const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                    int32_t batch, const double* dep, const double* cpar, double* R, void* stream);

/* Per-element CSR positions (0-based) of all 89x89 element entries, by element number:
 * slots[e][r][c] (-1 where absent).  color_elems lists the elements to map (normally all, in any
 * order).  Built once per mesh and structure. */
int gfe_mr_slot_map(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t n_q2, const int32_t* color_elems,
                    const int32_t* row_ptr, const int32_t* col_idx, int32_t* slots, void* stream);

/* Iron's analytic Jacobian of one problem assembled into CSR values (needs `slots` and `row_ptr`;
 * every value is written) and/or written as dense element matrices K_out[n_elem][89][89] (may be
 * NULL).  Replaces the element loop of EquationsSet_JacobianEvaluateStaticFEM
 * (src/equations_set_routines.F90:4677-4798) around FiniteElasticity_FiniteElementJacobianEvaluate
 * (src/finite_elasticity_routines.F90:879-1296) and EquationsMatrices_JacobianElementAdd
 * (src/equations_matrices_routines.F90:2866-2909).  The element matrices of the whole mesh are
 * formed first (no colouring needed: color_elems is read as the list of all elements); each CSR
 * row is then summed once from the rows of the elements around its node, in ascending element
 * order, and written once.  Allocates and frees the element matrices (n_elem x 89 x 89 in the
 * contraction type) and small scratch on `stream`. */
int gfe_mr_jacobian(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t n_q2, int32_t n_lin,
                    const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                    const double* dep, const double* cpar, const int32_t* slots, const int32_t* row_ptr,
                    double* values, int64_t nnz, double* K_out, int32_t precision, void* stream);
/* precision: GFE_FP64 (FP64 contraction), GFE_MIXED (FP32 CUDA-core contraction of the
 * basis-gradient x material blocks), GFE_TC_TF32X3 / GFE_TC_TF32 (the same contraction on the
 * tensor cores, tcgen05 kind::tf32 with FP32 accumulation in tensor memory, three-pass split or one
 * pass).  GFE_FP64 runs the Gauss-point kinematics in FP64; the other modes run them in FP32 from
 * FP32 basis tables with the volume Jacobians det(Z), det(X) evaluated in FP64 on exactly widened
 * gradients.  The assembled values are FP64 in every mode. */

/* Consistent tangent: the exact derivative of the residual of gfe_mr_residual with respect to
 * the dependent vector (what Iron's finite-difference Jacobian, EquationsSet_FiniteElementJacobianEvaluateFD
 * src/equations_set_routines.F90:2839-2962, approximates column by column).  Same outputs as
 * gfe_mr_jacobian.  Used by the Newton solver and checked against finite differences. */
int gfe_mr_tangent(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t n_q2, int32_t n_lin,
                   const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                   const double* dep, const double* cpar, const int32_t* slots, const int32_t* row_ptr,
                   double* values, int64_t nnz, double* K_out, int32_t precision, void* stream);

/* Iron's finite-difference Jacobian, its default for finite elasticity, in FP64: per element the
 * residual R0 and, for each of the 89 element parameters j, the residual with parameter j raised by
 * delta = (1 + ||dep||_2) step, column j = (R_j - R0) / delta, where ||dep||_2 is the L2 norm of the
 * whole dependent vector.  Replaces EquationsSet_FiniteElementJacobianEvaluateFD
 * (src/equations_set_routines.F90:2839-2962) inside EquationsSet_JacobianEvaluateStaticFEM;
 * `step` is Iron's jacobianFiniteDifferenceStepSize (default 1e-6, set by
 * cmfe_Equations_JacobianFiniteDifferenceStepSizeSet, src/opencmiss_iron.F90:25271-25348).  Outputs
 * as gfe_mr_jacobian, assembled colour by colour through the slot map (values zeroed first).
 * Allocates and frees a small norm scratch on `stream`. */
int gfe_mr_jacobian_fd(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t n_q2, int32_t n_lin,
                       const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                       const double* dep, const double* cpar, double step, const int32_t* slots, double* values,
                       int64_t nnz, double* K_out, void* stream);

/* Adjoint of the residual (K6): for `batch` problems, du[b] = v[b]^T dR/d(dep) ([batch][ndof]) and
 * dc[b] = v[b]^T dR/d(c10, c01) ([batch][2]).  No counterpart routine in Iron (its gradients come
 * from finite differences); checked against central differences and Iron-style one-sided FD.
 * Allocates and frees per-element partial sums on `stream`; the dc sum is in fixed element order. */
int gfe_mr_residual_vjp(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t n_q2, int32_t n_lin,
                        const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                        int32_t batch, const double* dep, const double* cpar, const double* v, double* du, double* dc,
                        void* stream);

/* ---- linear solve (K7) ------------------------------------------------------------------ */

/* y = A x on the rows with fixed[i] == 0; y[i] = 0 on fixed rows.  fixed may be NULL. */
int gfe_csr_spmv(int32_t n_rows, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                 const double* x, double* y, const uint8_t* fixed, void* stream);

/* Solve K x = f with Dirichlet conditions x[i] = x_in[i] where fixed[i] != 0, by
 * Jacobi-preconditioned conjugate gradients on the Dirichlet-eliminated system (the solver
 * matrix of SOLVER_MATRICES_STATIC_ASSEMBLE, src/solver_routines.F90:14025-15050, solved by
 * PETSc KSP in Iron, src/solver_routines.F90:11775-11991).
 *  f          [n] right-hand side (may be NULL = zero)
 *  x          [n] in: Dirichlet values on fixed DOFs; out: solution
 *  values32   optional FP32 copy of values: when given and precision == GFE_MIXED, runs FP32 CG
 *             with reliable updates (the true residual formed in FP64 with values replaces the
 *             FP32 one after each 1e3-fold reduction; the FP32 search direction is kept)
 *  rtol       relative residual target ||f - K x|| / ||f - K x0||
 *  iters_host out: total (inner) iterations;  rel_host out: final relative FP64 residual
 * Synchronises `stream`.  Allocates and frees its scratch on `stream`. */
int gfe_cg_solve(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                 const float* values32, const double* f, const uint8_t* fixed, double* x, double rtol,
                 int32_t max_iters, int32_t precision, int32_t* iters_host, double* rel_host, void* stream);

/* FP64 solve of gfe_cg_solve that allocates no device memory.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc (a host framework that owns all device memory
 * through its own pool, a serving process with a fixed memory partition).  The working vectors
 * live in one static device array of the library sized for GFE_NOALLOC_MAX_ROWS rows (about
 * 24 MiB), held by every GPU that loads the library until the process exits; larger systems are
 * rejected with GFE_ERR_ARG.  The first call on a device looks up the array's device address
 * (set-up, once per device).  All calls share the one array and it keeps the last call's contents
 * (each call clears what must start at zero): calls that overlap on the GPU, from any stream or
 * thread, race and must not be issued.  Synchronises `stream` (it reads scalars back between
 * iterations), so it cannot be captured into a CUDA graph: gfe_cg_begin / gfe_cg_steps are the
 * capturable form.  Arguments and solution as gfe_cg_solve with precision GFE_FP64, with one
 * difference in error reporting: a zero or non-finite diagonal entry on a free row, which
 * gfe_cg_solve raises as GFE_DEVERR_NONFINITE on the device error word, is returned here as
 * GFE_ERR_NUMERIC (this entry point uses no library error word). */
#define GFE_NOALLOC_MAX_ROWS 524288
int gfe_cg_solve_noalloc(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                         const double* f, const uint8_t* fixed, double* x, double rtol, int32_t max_iters,
                         int32_t* iters_host, double* rel_host, void* stream);

/* Graph-capturable FP64 Jacobi-CG (the solve of gfe_cg_solve split into enqueue-only steps, for a
 * serving loop that captures its launches into CUDA graphs).  The caller allocates a 256-byte
 * aligned device workspace of gfe_cg_workspace_bytes(n) bytes per concurrent solve.
 *  gfe_cg_begin   Jacobi inverse, x0 (Dirichlet values, zeros elsewhere), r0 = f - K x0 and the
 *                 first direction; converged when ||r_k||^2 <= rtol^2 ||r_0||^2 (recurrence residual)
 *  gfe_cg_steps   `steps` CG iterations; iterations after convergence or breakdown do nothing
 *  gfe_cg_status  copies the state to state_host (pinned memory when captured); the copy is
 *                 complete when `stream` reaches this point
 * None of them allocates or synchronises. */
typedef struct gfe_cg_state {
  double rr;          /* ||r_k||^2 */
  double rr0;         /* ||r_0||^2 */
  int32_t done;       /* 0 running, 2 converged, 1 breakdown */
  int32_t iterations;
  int32_t breakdown;
  int32_t reserved;
} gfe_cg_state;
int64_t gfe_cg_workspace_bytes(int32_t n);
int gfe_cg_begin(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values, const double* f,
                 const uint8_t* fixed, double* x, double rtol, void* workspace, void* stream);
int gfe_cg_steps(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                 const uint8_t* fixed, double* x, int32_t steps, void* workspace, void* stream);
int gfe_cg_status(int32_t n, void* workspace, gfe_cg_state* state_host, void* stream);

/* Solve K x = f for symmetric (possibly indefinite) K with Dirichlet conditions, by preconditioned
 * MINRES: the linear solve of the Newton step for the mixed u-p Jacobian, whose p-p block is zero.
 * Replaces the PETSc KSP solve Iron runs inside its Newton solver (GMRES + Jacobi by default,
 * src/solver_routines.F90:11320-11369; SNES linear solve call in src/solver_routines.F90:18942-18991).
 *  minv       [n] inverse of a symmetric positive definite diagonal preconditioner (> 0 on free
 *             rows), or NULL for 1/|K_ii| with 1 where K_ii = 0
 *  rtol       relative residual target in the preconditioner's norm, ||f - K x||_{M^-1} /
 *             ||f - K x0||_{M^-1} with ||r||_{M^-1}^2 = sum_i minv_i r_i^2 (the norm MINRES
 *             minimises, PETSc's default for KSPMINRES), x0 = Dirichlet values with zeros
 *             elsewhere; rel_host returns that ratio for the final FP64 residual.  Other arguments
 *             as gfe_cg_solve (GFE_MIXED: FP64-residual refinement around FP32 MINRES on values32).
 * Synchronises `stream`.  Allocates and frees its scratch on `stream`. */
int gfe_minres_solve(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                     const float* values32, const double* minv, const double* f, const uint8_t* fixed, double* x,
                     double rtol, int32_t max_iters, int32_t precision, int32_t* iters_host, double* rel_host,
                     void* stream);

/* gfe_minres_solve for a matrix whose first n_comp * n_node rows (n_comp = 2 or 3) are the
 * components of a vector field on n_node nodes in Iron's separated component DOF order (component
 * c of node i is row c * n_node + i), e.g. the displacement rows of the mixed u-p Mooney-Rivlin
 * system with n_node = the number of triquadratic nodes.  Where the n_comp rows of every node hold
 * one column list (components sharing one basis, as in Iron's element-coupling structure), the
 * sparse products load each column index and gathered vector entry once for the node's rows; the
 * solver checks that on the device and otherwise uses the per-row product.  Grouping applies to
 * the FP32 Krylov iterations of GFE_MIXED (FP32 matrix traffic 8 -> 5.3 bytes an entry); GFE_FP64
 * keeps the per-row product, whose cost is the FP64 pipe's.  *nodal_used (may be NULL) returns 1
 * when the grouped product ran.  Same results as gfe_minres_solve up to the rounding of the order
 * in which the inner products add their rows. */
int gfe_minres_solve_nodal(int32_t n, int32_t n_node, int32_t n_comp, const int32_t* row_ptr, const int32_t* col_idx,
                           const double* values, const float* values32, const double* minv, const double* f,
                           const uint8_t* fixed, double* x, double rtol, int32_t max_iters, int32_t precision,
                           int32_t* iters_host, double* rel_host, int32_t* nodal_used, void* stream);

/* Solve K x = f for general (non-symmetric) K with Dirichlet conditions by restarted GMRES(restart),
 * right-preconditioned by the diagonal minv (as gfe_minres_solve; NULL = Jacobi with 1 for a zero
 * diagonal), classical Gram-Schmidt.  Iron's default linear solver: PETSc GMRES, restart 30
 * (src/solver_routines.F90:11320-11369); needed for Iron's analytic Mooney-Rivlin Jacobian, whose
 * u-p and p-u blocks are not transposes of each other.  Each restart forms the residual in FP64;
 * GFE_MIXED runs the Krylov cycles in FP32 on values32.  restart: 1..64.  Other arguments as
 * gfe_minres_solve.  Synchronises `stream` once per cycle. */
int gfe_gmres_solve(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                    const float* values32, const double* minv, const double* f, const uint8_t* fixed, double* x,
                    double rtol, int32_t max_iters, int32_t restart, int32_t precision, int32_t* iters_host,
                    double* rel_host, void* stream);

/* Diagonal SPD preconditioner for gfe_minres_solve on a u-p saddle-point matrix whose first n_u
 * rows are the displacement block: minv[i] = 1/|K_ii| on u rows and, on p rows, the inverse of
 * sum_{free j < n_u} K_ij^2 / |K_jj| (the diagonal of B diag(K_uu)^-1 B^T); 1 where either is zero,
 * 0 on fixed rows.  Iron's default Jacobi preconditioner has no usable p-p diagonal (it is zero). */
int gfe_saddle_preconditioner(int32_t n, int32_t n_u, const int32_t* row_ptr, const int32_t* col_idx,
                              const double* values, const uint8_t* fixed, double* minv, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GFE_H */
