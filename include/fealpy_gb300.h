/*
 * fealpy_gb300.h -- C ABI of the GB300 (sm_103a) kernels behind the FEALPy
 * Lagrange assemble + Dirichlet + Jacobi-PCG path.
 *
 * Every entry point:
 *   - takes device pointers (unless the name ends in _host), plain sizes and a
 *     cudaStream_t passed as `void* stream`, and is stream-ordered;
 *   - returns an int status (FGB_OK == 0); conditions found on the device are
 *     written into the caller's `int32_t* status` device word (max of codes);
 *   - never allocates device memory: scratch comes from a caller workspace
 *     sized by the matching *_workspace_bytes() query, and the library never
 *     frees caller memory;
 *   - never traps or aborts; it keeps no global mutable state.
 * Two documented exceptions: fgb_pcg_f64_noalloc uses a static device array
 * of the library instead of a workspace, and an fgb_batch handle (host
 * object created by fgb_batch_create) owns the CUDA graph it captures.
 *
 * Index conventions follow FEALPy: cell-to-dof maps are int32 (NC, ldof)
 * row-major, CSR row pointers are int64 (FEALPy's `crow` dtype after
 * bincount+cumsum, fealpy/sparse/coo_tensor.py:144-146), CSR column indices
 * are int32.  Every CSR produced here is canonical: rows ascending, columns
 * strictly ascending, duplicates summed.
 */
#ifndef FEALPY_GB300_H
#define FEALPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum fgb_status_code {
  FGB_OK = 0,
  FGB_ERR_ARG = 1,        /* bad argument (sizes, null pointers, dtype)      */
  FGB_ERR_WORKSPACE = 2,  /* workspace missing or smaller than queried       */
  FGB_ERR_INDEX = 3,      /* an index read on the device was out of range    */
  FGB_ERR_PATTERN = 4,    /* a contribution's column is missing from the CSR */
  FGB_ERR_NONFINITE = 5,  /* NaN/Inf met (degenerate cell, NaN coefficient)  */
  FGB_ERR_BREAKDOWN = 6,  /* CG breakdown: p.Ap <= 0 (matrix not SPD)        */
  FGB_ERR_CUDA = 7,       /* a CUDA launch or copy failed                    */
  FGB_ERR_CAPACITY = 8    /* a size exceeds a documented fixed limit         */
};

enum fgb_dtype { FGB_F32 = 0, FGB_F64 = 1 };

/* Stop reasons reported by the PCG solvers (fgb_pcg_info.reason). */
enum fgb_pcg_reason {
  FGB_PCG_RUNNING = 0,
  FGB_PCG_ATOL = 1,     /* sqrt(r.z) < atol                                  */
  FGB_PCG_RTOL = 2,     /* sqrt(r.z) < rtol*||b|| (or true residual, mixed)  */
  FGB_PCG_MAXIT = 3,    /* iteration limit reached                           */
  FGB_PCG_ZERO_RHS = 4, /* ||b|| < 1e-15: x = 0 returned                     */
  FGB_PCG_BREAKDOWN = 5,
  FGB_PCG_NONFINITE = 6,
  FGB_PCG_STAGNATED = 7 /* the true residual stopped improving: FP32       */
                        /* iterations (fgb_pcg_sell_mixed, batched): the    */
                        /* caller continues in FP64 from x; batched FP64:   */
                        /* the attainable accuracy is above rtol            */
};

typedef struct fgb_pcg_info {
  int64_t niter;      /* CG iterations performed                            */
  double residual;    /* sqrt(r.z) at exit (FEALPy's `info['residual']`)    */
  double b_norm;      /* ||b||_2                                            */
  double true_relres; /* ||b - A x||_2/||b||_2 in FP64 (mixed solver), else -1 */
  int32_t reason;     /* enum fgb_pcg_reason                                */
  int32_t n_updates;  /* mixed solver: FP64 residual replacements performed */
  int64_t launches;   /* kernels launched by the call                       */
  double kernel_ms;   /* profile != 0: summed CUDA-event time of the SpMV   */
                      /* kernel of the iterations that did work             */
  int64_t kernel_launches; /* number of SpMV launches summed in kernel_ms   */
  double other_ms;    /* profile != 0: CUDA-event time of the vector-update */
                      /* kernel of those iterations                         */
  double extra_ms;    /* profile != 0: time of the remaining kernels of     */
                      /* those iterations (p update, reliable-update check) */
  int32_t graph;      /* 1 if the iterations ran as a device-side graph loop, */
                      /* 2 as one persistent cooperative kernel (mixed)      */
  int32_t reserved;
} fgb_pcg_info;

/* Cell-factor channel kinds for fgb_cell_factors (k, l, a in 0..TD-1):
 *   FGB_CH_MEASURE            signed cell measure |T| (simplex_measure)
 *   FGB_CH_METRIC + k*3 + l   |T| * grad(lambda_{k+1}) . grad(lambda_{l+1})
 *   FGB_CH_GRAD   + k*3 + a   d lambda_{k+1} / d x_a                      */
enum fgb_channel { FGB_CH_MEASURE = 0, FGB_CH_METRIC = 1, FGB_CH_GRAD = 16 };
#define FGB_MAX_CHANNELS 16

const char* fgb_status_string(int32_t status);
int32_t fgb_abi_version(void);

/* Exclusive scan of n int32 counts into n+1 int64 offsets (out[0] = 0).
 * Building block of COOTensor.tocsr's bincount+cumsum
 * (fealpy/sparse/coo_tensor.py:144-146). */
size_t fgb_scan_workspace_bytes(int64_t n);
int32_t fgb_exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, void* workspace,
                               size_t workspace_bytes, void* stream);

/* ---- mesh topology and dof numbering ------------------------------------ */

/* Unique sub-entities (edges, or faces) of a simplex mesh as MeshDS.construct
 * builds them (fealpy/mesh/mesh_data_structure.py:428-464, flocc in
 * fealpy/mesh/utils.py:81-110): the distinct sorted vertex tuples of the
 * cells' local entities local_host (nfc x k, host memory), numbered in
 * lexicographic order, each stored in the orientation of its first
 * occurrence (cell order, then local index); entity2cell (optional, ne x 4)
 * = [first cell, last cell, first local index, last local index];
 * cell2entity (n_cell x nfc).  count groups the occurrences by smallest
 * vertex, ranks the distinct tuples and writes their number to
 * *n_entity_host (it synchronises the stream); fill then writes the arrays,
 * with the same workspace (fgb_topology_workspace_bytes(n_node,
 * n_cell * nfc)), which carries the grouping from count to fill. */
size_t fgb_topology_workspace_bytes(int64_t n_node, int64_t n_occ);
int32_t fgb_topology_count(int64_t n_cell, int32_t nv, const int32_t* cell, int64_t n_node, int32_t k,
                           int32_t nfc, const int32_t* local_host, int64_t* n_entity_host,
                           int32_t* status, void* workspace, size_t workspace_bytes, void* stream);
int32_t fgb_topology_fill(int64_t n_cell, int32_t nv, const int32_t* cell, int64_t n_node, int32_t k,
                          int32_t nfc, const int32_t* local_host, int32_t* entity, int32_t* entity2cell,
                          int32_t* cell2entity, int32_t* status, void* workspace,
                          size_t workspace_bytes, void* stream);

/* cell_to_ipoint (fealpy/mesh/triangle_mesh.py:218-270,
 * fealpy/mesh/tetrahedron_mesh.py:388-441): per local point k (host tables,
 * ldof entries): kind 0 vertex a; kind 1 edge point between local vertices
 * a < b on local edge le, with multi-index entries ma, mb (numbered from the
 * global edge's first vertex); kind 2 the rank-th interior point of a
 * triangle; kind 3 the interior point of local face le of a P3
 * tetrahedron.  Writes cell2ipoint (n_cell x ldof, int32). */
int32_t fgb_cell_to_ipoint(int64_t n_cell, int32_t td, int32_t p, int32_t ldof, const int32_t* cell,
                           const int32_t* cell2edge, const int32_t* edge, const int32_t* cell2face,
                           int64_t n_node, int64_t n_edge, const int32_t* kind_host,
                           const int32_t* a_host, const int32_t* b_host, const int32_t* le_host,
                           const int32_t* ma_host, const int32_t* mb_host, const int32_t* rank_host,
                           int32_t* cell2ipoint, void* stream);

/* ---- symbolic assembly ------------------------------------------------- */

/* dof -> (cell, local index) adjacency, sorted by cell then local index:
 * adj_ptr (n_dof+1, int64), adj (n_cell*ldof, int32, packed cell*ldof+li).
 * This is the grouping that FEALPy's stable lexsort in COOTensor.coalesce
 * (fealpy/sparse/coo_tensor.py:184-200) imposes on the COO triplets built by
 * BilinearForm._scalar_assembly (fealpy/fem/bilinear_form.py:46-75).
 * Also writes the maximum adjacency length to max_degree (device int32). */
size_t fgb_adjacency_workspace_bytes(int64_t n_dof);
int32_t fgb_adjacency_build(int64_t n_cell, int32_t ldof, const int32_t* cell2dof, int64_t n_dof,
                            int64_t* adj_ptr, int32_t* adj, int32_t* max_degree, int32_t* status,
                            void* workspace, size_t workspace_bytes, void* stream);

/* Canonical CSR pattern of sum_c P_c^T K_c P_c: row i holds the sorted union
 * of the dofs of the cells around dof i.  Replaces the index half of
 * COOTensor.coalesce + tocsr (fealpy/sparse/coo_tensor.py:137-157,184-213).
 * count: writes indptr (n_dof+1) via an internal scan; fill: writes indices. */
size_t fgb_pattern_workspace_bytes(int64_t n_dof);
int32_t fgb_pattern_count(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj,
                          const int32_t* cell2dof, int32_t ldof, int64_t* indptr, int32_t* status,
                          void* workspace, size_t workspace_bytes, void* stream);
int32_t fgb_pattern_fill(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj,
                         const int32_t* cell2dof, int32_t ldof, const int64_t* indptr,
                         int32_t* indices, int32_t* status, void* workspace,
                         size_t workspace_bytes, void* stream);

/* The same pattern in one pass over the rows: build hashes and sorts every
 * row once, staging it at stage[adj_ptr[i] * ldof] (stage: n_adj * ldof
 * int32, n_adj = adj_ptr[n_dof]), and writes indptr; compact then copies the
 * staged rows into indices (after the caller has read nnz = indptr[n_dof]).
 * Both take the same workspace, which carries the list of rows too long for
 * the hash pass from build to compact.  positions (optional, n_adj * ldof
 * bytes): for adjacency entry k of row i (cell c, local index li) and local
 * dof j, positions[k * ldof + j] = the index within row i of column
 * cell2dof[c][j], recorded for rows of at most 128 entries; given to
 * fgb_assemble_scalar_acc, the numeric pass adds each contribution at its slot
 * without searching the row (a pattern reused across assemblies pays this
 * once). */
int32_t fgb_pattern_build(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj,
                          const int32_t* cell2dof, int32_t ldof, int64_t n_adj, int64_t* indptr,
                          int32_t* stage, size_t stage_bytes, uint8_t* positions, int32_t* status,
                          void* workspace, size_t workspace_bytes, void* stream);
int32_t fgb_pattern_compact(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj,
                            const int32_t* cell2dof, int32_t ldof, const int64_t* indptr,
                            const int32_t* stage, int32_t* indices, int32_t* status,
                            void* workspace, size_t workspace_bytes, void* stream);

/* Block expansion of a scalar pattern for vector spaces: bs components per
 * node; interleaved (3*node+comp, TensorFunctionSpace(space,(-1,GD)),
 * fealpy/functionspace/tensor_space.py:29-31) when dof_priority == 0, else
 * component-major (comp*n_node+node).  out_indptr has bs*n_node+1 entries. */
int32_t fgb_pattern_expand_blocks(int64_t n_node, int32_t bs, int32_t dof_priority,
                                  const int64_t* indptr, const int32_t* indices,
                                  int64_t* out_indptr, int32_t* out_indices, void* stream);

/* ---- numeric assembly -------------------------------------------------- */

/* Per-cell geometric factors (affine simplex, TD = 2 or 3, GD = TD): the
 * signed measure and Jacobian-inverse metric that FEALPy's simplex_measure,
 * triangle/tetrahedron_grad_lambda compute (fealpy/backend/numpy_backend.py:
 * 414-421, 587-598, 620-629), evaluated in FP64 and written as n_channel
 * columns of factors (n_cell, n_channel) in out_dtype.  Channel j is
 *   value(kind_j) * scale_j * (coef_index_j >= 0 ? coef[coef_index_j*n_cell + c] : 1).
 * chan_*_host are host arrays of n_channel <= FGB_MAX_CHANNELS entries. */
int32_t fgb_cell_factors(int32_t td, int64_t n_cell, const double* node, const int32_t* cell,
                         int32_t n_channel, const int32_t* chan_kind_host,
                         const int32_t* chan_coef_host, const double* chan_scale_host,
                         const double* coef, int32_t out_dtype, void* factors, int32_t* status,
                         void* stream);

/* Scalar Lagrange assembly straight into CSR values (no local-matrix
 * materialisation, no atomics): K_c[i][j] = sum_t factors[c][t]*tables[t][i][j],
 * which equals FEALPy's bilinear_integral einsum over quadrature points for
 * ScalarDiffusionIntegrator / ScalarMassIntegrator / their GroupIntegrator
 * (fealpy/functional.py:68-106, fealpy/fem/scalar_diffusion_integrator.py:54-63,
 * fealpy/fem/scalar_mass_integrator.py:47-54, fealpy/fem/integrator.py:361-378)
 * when coefficients are constant per cell.  Contributions to each CSR entry
 * are summed in (cell, local index) order.  values_f32 (optional) receives a
 * float copy.  dtype selects double or float tables/factors/values.
 * ldof <= 32; tables (n_table, ldof, ldof). */
size_t fgb_assemble_workspace_bytes(int64_t n_rows);
int32_t fgb_assemble_scalar(int32_t dtype, int64_t n_dof, const int64_t* adj_ptr,
                            const int32_t* adj, const int32_t* cell2dof, int32_t ldof,
                            int32_t n_table, const void* tables, const void* factors,
                            const int64_t* indptr, const int32_t* indices, void* values,
                            float* values_f32, int32_t* status, void* workspace,
                            size_t workspace_bytes, void* stream);
/* The same with accumulate != 0: values += this pass (values_f32, when given,
 * receives the FP32 rounding of the sum).  For local matrices with more than
 * FGB_MAX_CHANNELS factor channels (coefficients given per quadrature point,
 * fealpy/utils/utils.py:21-53): the channels are split into passes.
 * positions (optional): the within-row slots fgb_pattern_build recorded for
 * this pattern; rows up to 128 entries then take no column search. */
int32_t fgb_assemble_scalar_acc(int32_t dtype, int64_t n_dof, const int64_t* adj_ptr,
                                const int32_t* adj, const int32_t* cell2dof, int32_t ldof,
                                int32_t n_table, const void* tables, const void* factors,
                                const int64_t* indptr, const int32_t* indices,
                                const uint8_t* positions, void* values, float* values_f32,
                                int32_t accumulate, int32_t* status, void* workspace,
                                size_t workspace_bytes, void* stream);

/* P1 linear elasticity, interleaved vector dofs (LinearElasticityIntegrator
 * default variant, fealpy/fem/linear_elasticity_integrator.py:60-181, the
 * dof_priority=False branch).  adj/adj_ptr is the node->(cell, vertex)
 * adjacency, node_indptr/node_indices the scalar node pattern, indptr/indices
 * the expanded vector pattern (fgb_pattern_expand_blocks, dof_priority 0).
 * factors (n_cell, gd*gd + 3): grad(lambda_{1..gd}) components, then
 * |T|*D00, |T|*D_lambda, |T|*D_mu with D00 = 2*D55+D01 (3-D) or D[0,0]
 * (2-D), D_lambda = D01, D_mu = D55 (3-D) or D22 (2-D). */
int32_t fgb_assemble_elasticity_p1(int32_t dtype, int32_t gd, int64_t n_node,
                                   const int64_t* adj_ptr, const int32_t* adj,
                                   const int32_t* cell, const void* factors,
                                   const int64_t* node_indptr, const int32_t* node_indices,
                                   const int64_t* indptr, void* values, float* values_f32,
                                   int32_t* status, void* workspace, size_t workspace_bytes,
                                   void* stream);

/* Cell vectors to a global vector: out[i] = sum over the adjacency of dof i
 * (cell order) of local[cell*ldof + li].  Replaces the index_add scatter of
 * LinearForm._scalar_assembly (fealpy/fem/linear_form.py:36-86). */
int32_t fgb_gather_sum(int32_t dtype, int64_t n, const int64_t* adj_ptr, const int32_t* adj,
                       const void* local, void* out, void* stream);

/* Cell-local matrices for callers that want them (Integrator.assembly(space),
 * fealpy/fem/scalar_diffusion_integrator.py, scalar_mass_integrator.py):
 * out (n_cell, ldof, ldof) = sum_t factors[c][t] * tables[t] (device tables,
 * the factor dtype); accumulate != 0 adds to out (passes of split channels).
 * P1 elasticity (fealpy/fem/linear_elasticity_integrator.py:61-181): out
 * (n_cell, (gd+1) gd, (gd+1) gd) from the factor channels of
 * fgb_assemble_elasticity_p1; priority 0: local index vertex * gd + component
 * (interleaved), 1: component * (gd + 1) + vertex. */
int32_t fgb_local_matrices(int32_t dtype, int64_t n_cell, int32_t ldof, int32_t n_table,
                           const void* tables, const void* factors, void* out, int32_t accumulate,
                           void* stream);
int32_t fgb_local_elasticity_p1(int32_t dtype, int32_t gd, int64_t n_cell, const void* factors,
                                int32_t priority, void* out, void* stream);

/* Matrix-free y_cell = K_c x_c for every cell, K_c = sum_t factors[c][t] *
 * tables[t] (the factorisation of fgb_assemble_scalar), the cell-local half
 * of BilinearForm.__matmul__ without a global matrix
 * (fealpy/fem/bilinear_form.py:126-158: gather u at the cell dofs, einsum with
 * the cell-local matrices); fgb_gather_sum over the dof adjacency then adds
 * the cells' results per dof (the index_add, deterministic).  ycell:
 * (n_cell, ldof) in the factor dtype.  tables_host (n_table*ldof*ldof FP64,
 * host memory) is used for ldof in {3, 4, 6, 10} (the tables go into the
 * kernel's parameter space); otherwise `tables` (device, the factor dtype). */
int32_t fgb_cell_apply(int32_t dtype, int64_t n_cell, int32_t ldof, const int32_t* cell2dof,
                       int32_t n_table, const double* tables_host, const void* tables,
                       const void* factors, const void* x, void* ycell, void* stream);

/* Scalar source right-hand sides (ScalarSourceIntegrator, fealpy/fem/
 * scalar_source_integrator.py:51-58; LinearForm's scatter, fealpy/fem/
 * linear_form.py:36-86): b_c[i] = cm[c] sum_q w_q phi_i(q) f(c, q), the
 * source as one number (mode 0, f_scalar), one value per cell (mode 1, f
 * (NC)) or per quadrature point (mode 2, f (NC, NQ)); wphi (NQ x ldof) =
 * w_q phi_i(q), sv (ldof) its column sums (device).  local: the cell vectors
 * (NC x ldof); gather: the global vector over the dof adjacency in adjacency
 * order (accumulate != 0 adds to out). */
int32_t fgb_source_local(int64_t n_cell, int32_t ldof, int32_t nq, const double* cm, int32_t mode,
                         double f_scalar, const double* f, const double* wphi, const double* sv,
                         double* out, void* stream);
int32_t fgb_source_gather(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, int32_t ldof,
                          int32_t nq, const double* cm, int32_t mode, double f_scalar, const double* f,
                          const double* wphi, const double* sv, double* out, int32_t accumulate,
                          void* stream);

/* Split of a block-diagonal CSR of many systems assembled together (system s
 * owns rows and columns [row_off[s], row_off[s+1]), n_rows = row_off[n_sys]):
 * columns rebased in place to each system's numbering (a column outside its
 * system's range sets FGB_ERR_PATTERN in *status), and per system a row
 * pointer starting at 0 in indptr_out (n_rows + n_sys entries, system s at
 * offset row_off[s] + s).  Each system's entries stay a contiguous range of
 * the union's indices and values. */
int32_t fgb_csr_split_blocks(int32_t n_sys, const int64_t* row_off, const int64_t* indptr,
                             int32_t* indices, int64_t* indptr_out, int64_t n_rows, int32_t* status,
                             void* stream);

/* ---- Dirichlet boundary conditions ------------------------------------- */

/* DirichletBC.apply (fealpy/fem/dirichlet_bc.py:101-229): given is_bd (uint8,
 * n), the boundary values u_bd (n, zero off the boundary; NULL when they are
 * all zero, which skips the product A u_bd) and f:
 *   count: f_out = f - A u_bd off the boundary, f_out[bd] = u_bd[bd];
 *          row_nnz (n, int32) = kept entries per row (1 on boundary rows);
 *   fill:  new_indices/new_values of the eliminated matrix (boundary rows and
 *          columns removed, unit diagonal on boundary rows), in canonical order
 *          given new_indptr = exclusive scan of row_nnz. */
int32_t fgb_dirichlet_count(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                            const void* values, const uint8_t* is_bd, const void* f,
                            const void* u_bd, void* f_out, int32_t* row_nnz, void* stream);
int32_t fgb_dirichlet_fill(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                           const void* values, const uint8_t* is_bd, const int64_t* new_indptr,
                           int32_t* new_indices, void* new_values, void* stream);

/* ---- sparse kernels and solvers ----------------------------------------- */

/* y = A x for a CSR matrix (CSRTensor.matmul -> bm.csr_spmm,
 * fealpy/sparse/csr_tensor.py:411-452, fealpy/backend/numpy_backend.py:181-199).
 * lanes_per_row in {0 (auto), 1, 2, 4, 8, 16, 32}. */
int32_t fgb_csr_spmv(int32_t dtype, int64_t n_row, const int64_t* indptr, const int32_t* indices,
                     const void* values, const void* x, void* y, int32_t lanes_per_row,
                     void* stream);

/* Y = A X for k right-hand columns at once (the (n, batch) product of
 * bm.csr_spmm, fealpy/backend/numpy_backend.py:181-199): X (n_col, k) and
 * Y (n_row, k) row-major FP64, 1 <= k <= 64; the matrix is read once for all
 * columns.  Every entry of Y is the same sum in the same order as
 * fgb_csr_spmv with one lane per row. */
int32_t fgb_csr_spmm_f64(int64_t n_row, int32_t k, const int64_t* indptr, const int32_t* indices,
                         const double* values, const double* X, double* Y, void* stream);

/* out2[0] = ||b - A x||^2, out2[1] = ||b||^2 (FP64 CSR, device scalars,
 * deterministic): the true residual of FEALPy's stopping test
 * (fealpy/solver/cg.py:99-113) as the restart loops of the FP32-refined
 * solver's FP64 continuation and of the multigrid solve form it.  workspace:
 * fgb_residual_norm_workspace_bytes() bytes of device memory. */
size_t fgb_residual_norm_workspace_bytes(void);
int32_t fgb_residual_norm(int64_t n, const int64_t* indptr, const int32_t* indices,
                          const double* values, const double* b, const double* x, double* out2,
                          void* workspace, size_t workspace_bytes, void* stream);

/* diag(A) and 1/diag(A) (CSRTensor.diags + JacobiPreconditioner.apply,
 * fealpy/sparse/csr_tensor.py:467-475, fealpy/solver/iterative_solver_manger.py:
 * 273-280).  A missing diagonal yields 0 and 1/0 = inf, as in FEALPy. */
int32_t fgb_csr_diagonal(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                         const void* values, void* diag, void* diag_inv, void* stream);

/* Jacobi-preconditioned CG in FP64 with FEALPy's iteration and stopping rule
 * (fealpy/solver/cg.py:76-123): stop when sqrt(r.z) < atol or
 * < rtol*||b||_2 or after maxit iterations.  diag_inv == NULL means no
 * preconditioner.  x holds x0 on entry and the solution on exit.  Blocking:
 * the host polls a device flag every check_every iterations.  norm == 0
 * monitors FEALPy's sqrt(r.z); norm == 1 monitors the 2-norm of the iterated
 * residual instead.  lanes_per_row as in fgb_csr_spmv (0 = auto, >= 2).
 * profile != 0 brackets every SpMV launch with CUDA events (kernel_ms). */
size_t fgb_pcg_workspace_bytes(int64_t n);
int32_t fgb_pcg_f64(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                    const double* diag_inv, const double* b, double* x, double atol, double rtol,
                    int64_t maxit, int32_t check_every, int32_t lanes_per_row, int32_t norm,
                    int32_t profile, void* workspace, size_t workspace_bytes,
                    fgb_pcg_info* info_host, void* stream);

/* fgb_pcg_f64 without a workspace, for callers that cannot allocate device
 * memory at the point of the solve: a host code whose device memory is
 * handed out by its own pool or capped in advance, a plain C/Fortran caller
 * with no allocator of its own, or a loop that must not call cudaMalloc
 * (which may synchronise the whole device).  No counterpart in FEALPy.
 *
 * Same arguments, iteration, stopping rules and info as fgb_pcg_f64 (no
 * profile option).  The scratch is one static device array of this library
 * sized for FGB_PCG_NOALLOC_MAX_ROWS rows (about 2.6 MB); larger n returns
 * FGB_ERR_CAPACITY before any device work.  The caller zeroes nothing: each
 * call writes the solver state (with its block-arrival counters, which must
 * start at zero) before the first kernel, and every vector is written before
 * it is read.  Every call looks up the array's device address in the
 * context current on the calling thread (the address belongs to that
 * context, so a cudaDeviceReset or a new context between calls is safe); the
 * first call in a context may load this library's device code into it: make
 * that first call, with the device current, before any stream capture.
 * The scratch is shared by
 * all calls on a device, so calls that overlap in time (two host threads, or
 * two streams) race on it: serialise them. */
#define FGB_PCG_NOALLOC_MAX_ROWS 65536
int32_t fgb_pcg_f64_noalloc(int64_t n, const int64_t* indptr, const int32_t* indices,
                            const double* values, const double* diag_inv, const double* b,
                            double* x, double atol, double rtol, int64_t maxit,
                            int32_t check_every, int32_t lanes_per_row, int32_t norm,
                            fgb_pcg_info* info_host, void* stream);

/* Several right-hand sides of one matrix, the (n, batch) path of
 * fealpy/solver/cg.py:60-123: B and X row-major (n, k), 1 <= k <= 64; every
 * column runs its own recurrence (alpha, beta per column), all take the same
 * iterations, and the solve stops when sqrt(sum_c r_c . z_c) < atol or
 * < rtol * ||B||_F (diag_inv NULL: no preconditioner).  A zero B gives
 * X = 0.  The iterations run as one CUDA-graph launch. */
size_t fgb_pcg_multi_workspace_bytes(int64_t n, int32_t k);
int32_t fgb_pcg_multi_f64(int64_t n, int32_t k, const int64_t* indptr, const int32_t* indices,
                          const double* values, const double* diag_inv, const double* B, double* X,
                          double atol, double rtol, int64_t maxit, fgb_pcg_info* info_host,
                          void* workspace, size_t workspace_bytes, void* stream);

/* Mixed precision: Jacobi-PCG iterations in FP32 on values32 (FP32 SpMV,
 * dots and updates) with FP64 reliable updates: whenever the FP32 residual
 * has dropped by `delta` since the last update (or looks converged), the
 * FP32 correction is added to the FP64 iterate and the residual is recomputed
 * as b - A x with values64 in FP64.  Stops when that true residual satisfies
 * ||b - A x||_2 <= rtol*||b||_2.  No FEALPy counterpart: this is the
 * FP32-refined variant of fealpy/solver/cg.py. */
size_t fgb_pcg_mixed_workspace_bytes(int64_t n);
int32_t fgb_pcg_mixed(int64_t n, const int64_t* indptr, const int32_t* indices,
                      const double* values64, const float* values32, const double* diag_inv64,
                      const double* b, double* x, double rtol, double delta, int64_t maxit,
                      int32_t check_every, int32_t lanes_per_row, int32_t profile,
                      void* workspace, size_t workspace_bytes, fgb_pcg_info* info_host,
                      void* stream);

/* ---- SELL-32 solver copy ------------------------------------------------- */

/* Sliced-ELLPACK copy of a CSR matrix used by the SELL solvers: slices of 32
 * rows (rows sorted by length inside windows of 256), entries column-major
 * inside a slice, zero padding.  perm maps slot -> row (-1 = padding). */
typedef struct fgb_sell {
  int64_t n;                /* rows                                           */
  int64_t n_slices;         /* fgb_sell_slots(n) / 32                         */
  const int64_t* slice_ptr; /* n_slices + 1 entry offsets                     */
  const int32_t* perm;      /* fgb_sell_slots(n) slot -> row                  */
  const int32_t* col;       /* slice_ptr[n_slices] column indices             */
  const double* val64;      /* FP64 values (optional)                         */
  const float* val32;       /* FP32 values (optional)                         */
  int32_t threads;          /* launch shape of the slice kernels (SpMV, PCG   */
  int32_t blocks;           /* residual/SpMV steps); 0 = defaults.  threads a */
                            /* multiple of 32 in [32, 1024], blocks <= 1216   */
  const uint16_t* col16;    /* delta-coded columns (col unused) or NULL:      */
  const int32_t* col0;      /* column of entry k = col0[slot] + sum of the    */
                            /* steps col16 up to k (fgb_sell_fill_d16)        */
  int32_t node_triples;     /* 1: every slot is a node triple: col = 3c, and  */
                            /* three values (columns 3c..3c+2) per slot       */
                            /* (fgb_sell_fill_b3); 0: one entry per slot      */
  int32_t col_long;         /* 1: col16 holds 15-bit steps and long steps     */
                            /* (fgb_sell_fill_d15); 0: 16-bit steps           */
} fgb_sell;

/* No FEALPy counterpart: a solver-side layout of CSRTensor (the matrix the
 * reference hands to fealpy/solver/cg.py).  plan: perm + slice_ptr (one
 * host read of slice_ptr[n_slices] then sizes col/val); fill: col/val. */
int64_t fgb_sell_slots(int64_t n);
size_t fgb_sell_workspace_bytes(int64_t n);
int32_t fgb_sell_plan(int64_t n, const int64_t* indptr, int32_t* perm, int64_t* slice_ptr,
                      void* workspace, size_t workspace_bytes, void* stream);
int32_t fgb_sell_fill(int64_t n, const int64_t* indptr, const int32_t* indices,
                      const double* values64, const float* values32, const int32_t* perm,
                      const int64_t* slice_ptr, int32_t* col, double* val64, float* val32,
                      void* stream);
int32_t fgb_sell_spmv(int32_t dtype, const fgb_sell* A, const void* x, void* y, void* stream);

/* Delta-coded SELL copy: 2-byte column steps instead of 4-byte columns, for
 * a matrix renumbered so that the steps are small.  No FEALPy counterpart
 * (solver-side layout, as above); the solve is the same Jacobi-PCG on
 * P A P^T with b, x and the inverse diagonal permuted alike.
 *   renumber: order[k] = old index of new row k, inv = its inverse.  With
 *     the space's dof blocks (n_blocks > 0 sizes in dof order: vertex, edge,
 *     face and cell dofs, per component for component-major vector spaces):
 *     a stable merge of the blocks by relative position, which puts every
 *     edge/face/cell dof next to the vertex dofs of its region (FEALPy
 *     numbers entities by their vertices; block sizes of
 *     fealpy/functionspace/lagrange_fe_space.py number_of_global_dofs).
 *     Without blocks (n_blocks = 0): rows sorted by (smallest column, row);
 *     identity when a group of equal keys exceeds 64 rows.
 *   csr_permute: rows order[k] of the CSR with columns inv[col], ascending.
 *   d16_indptr: row pointer of the row lengths including the zero-valued
 *     bridge entries that split steps above 65535 (for fgb_sell_plan).
 *   fill_d16: col0/col16 and values of the plan's slots.
 *   permute: dst[k] = src[order[k]] (scatter = 0) or dst[order[k]] = src[k]. */
size_t fgb_sell_d16_workspace_bytes(int64_t n);
int32_t fgb_sell_renumber(int64_t n, const int64_t* indptr, const int32_t* indices, int32_t n_blocks,
                          const int64_t* block_sizes_host, int32_t* order, int32_t* inv,
                          void* workspace, size_t workspace_bytes, void* stream);
int32_t fgb_csr_permute(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                        const float* values32, const int32_t* order, const int32_t* inv,
                        int64_t* new_indptr, int32_t* new_indices, double* new_values64,
                        float* new_values32, void* workspace, size_t workspace_bytes, void* stream);
int32_t fgb_sell_d16_indptr(int64_t n, const int64_t* indptr, const int32_t* indices,
                            int64_t* bridged_indptr, void* workspace, size_t workspace_bytes,
                            void* stream);
int32_t fgb_sell_fill_d16(int64_t n, const int64_t* indptr, const int32_t* indices,
                          const double* values64, const float* values32, const int32_t* perm,
                          const int64_t* slice_ptr, int32_t* col0, uint16_t* col16, double* val64,
                          float* val32, void* stream);

/* The 15-bit column copy of a matrix in its own numbering (no renumbering;
 * columns must ascend strictly in every row).  Per slot the first column
 * (col0), per entry a 16-bit code: below 0x8000 a step from the previous
 * column; 0x8000 | h a zero-valued long-step entry that gathers the previous
 * column again and moves the running column on by h * 32768 (so any gap fits
 * with one or two such entries).  6 bytes per FP32 entry instead of 8, and
 * the solvers' vectors stay in the matrix's numbering.  The descriptor sets
 * col16, col0 and col_long = 1 (col = NULL).  d15_indptr: entries per row
 * with the long steps, scanned (a row whose columns do not ascend sets
 * FGB_ERR_ARG in *status); fgb_sell_plan on it gives perm and slice_ptr, and
 * fill_d15 writes col0, col16 and the values.  No FEALPy counterpart (storage
 * of the solver's copy). */
int32_t fgb_sell_d15_indptr(int64_t n, const int64_t* indptr, const int32_t* indices,
                            int64_t* entry_indptr, int32_t* status, void* workspace,
                            size_t workspace_bytes, void* stream);
int32_t fgb_sell_fill_d15(int64_t n, const int64_t* indptr, const int32_t* indices,
                          const double* values64, const float* values32, const int32_t* perm,
                          const int64_t* slice_ptr, int32_t* col0, uint16_t* col16,
                          double* val64, float* val32, void* stream);
int32_t fgb_permute(int32_t dtype, int64_t n, const int32_t* order, const void* src, void* dst,
                    int32_t scatter, void* stream);

/* Node-triple SELL copy for vector spaces with three interleaved components
 * (dof = 3 node + comp, FEALPy's TensorFunctionSpace(space, (-1, 3)),
 * fealpy/functionspace/tensor_space.py): one 4-byte column per run of three
 * consecutive columns 3c..3c+2 and its three values (zero where the matrix has
 * no entry), 16 bytes per three FP32 entries instead of 24.  n must be a
 * multiple of 3 and columns ascending in every row.
 *   b3_indptr: row pointer of the triple counts (for fgb_sell_plan).
 *   fill_b3: col (3c per slot) and three values per slot of the plan's slots
 *     (val64/val32 hold 3 * slice_ptr[n_slices] values). */
int32_t fgb_sell_b3_indptr(int64_t n, const int64_t* indptr, const int32_t* indices,
                           int64_t* triple_indptr, void* workspace, size_t workspace_bytes,
                           void* stream);
int32_t fgb_sell_fill_b3(int64_t n, const int64_t* indptr, const int32_t* indices,
                         const double* values64, const float* values32, const int32_t* perm,
                         const int64_t* slice_ptr, int32_t* col, double* val64, float* val32,
                         void* stream);

/* Jacobi-PCG on a SELL copy: same iteration, stopping rules and info as
 * fgb_pcg_f64 / fgb_pcg_mixed.  use_graph != 0 runs the iterations as a CUDA
 * graph with a device-side while loop (no host polling; profile ignored).
 * fgb_pcg_sell_mixed needs val32; its FP64 residual recomputation uses val64
 * when present, else the FP32 values themselves (an FP32-assembled operator,
 * accumulated in FP64), and then solves that operator to rtol.  Its
 * use_graph = 2 runs all iterations in one persistent cooperative kernel
 * (grid barriers between phases; falls back to the graph loop where
 * cooperative launch is unavailable): no launch overhead per iteration, but
 * its gathers bypass L1 (other blocks rewrite p within the launch), so it
 * suits small systems. */
size_t fgb_pcg_sell_workspace_bytes(int64_t n);
int32_t fgb_pcg_sell_f64(const fgb_sell* A, const double* diag_inv, const double* b, double* x,
                         double atol, double rtol, int64_t maxit, int32_t check_every,
                         int32_t norm, int32_t use_graph, int32_t profile, void* workspace,
                         size_t workspace_bytes, fgb_pcg_info* info_host, void* stream);
/* Process-wide switch for the FP32 products on 15-bit-step copies
 * (fgb_pcg_sell_mixed's SpMV, fgb_sell_spmv, the multigrid smoother): 1
 * (default) runs the pipelined kernel, which loads a warp's next trip of
 * packs before it gathers the current one; 0 runs the one-trip kernels.
 * Every row is the same sum in the same order either way. */
void fgb_sell_set_pipeline(int32_t enable);
int32_t fgb_pcg_sell_mixed(const fgb_sell* A, const double* diag_inv64, const double* b,
                           double* x, double rtol, double delta, int64_t maxit,
                           int32_t check_every, int32_t use_graph, int32_t profile,
                           void* workspace, size_t workspace_bytes, fgb_pcg_info* info_host,
                           void* stream);
/* fgb_pcg_sell_mixed with the persistent kernel's grid-barrier wait limit:
 * a block waits at most `barrier_polls` polls (about 64 ns apart) for the
 * others before it gives up, raises the shared error flag and returns, and
 * then every block returns and the call reports FGB_ERR_CUDA.  barrier_polls
 * <= 0 selects the default limit (2e7 polls, over a second), which a
 * cooperative launch with every block resident never reaches.  Only
 * use_graph = 2 waits on other blocks. */
int32_t fgb_pcg_sell_mixed_ex(const fgb_sell* A, const double* diag_inv64, const double* b,
                              double* x, double rtol, double delta, int64_t maxit,
                              int32_t check_every, int32_t use_graph, int32_t profile,
                              int64_t barrier_polls, void* workspace, size_t workspace_bytes,
                              fgb_pcg_info* info_host, void* stream);

/* ---- aggregation AMG preconditioner -------------------------------------- */

/* The `M` slot of fealpy/solver/cg.py filled with a multigrid V-cycle, the
 * role of FEALPy's GAMGSolver (fealpy/solver/gamg_solver.py:14-256, a
 * Ruge-Stuben hierarchy with Gauss-Seidel smoothing).  Here, with data-
 * parallel counterparts: aggregation by a maximal independent set of the
 * graph of entries |a_ij| > theta sqrt(|a_ii a_jj|) (a root and its
 * neighbours; rows without such entries, e.g. Dirichlet rows, join no
 * aggregate), Galerkin coarse matrices
 * P^T A P for the aggregate indicator P, Chebyshev smoothing with D^-1 and
 * the Gershgorin bound lmax of D^-1 A, coarse corrections scaled by omega,
 * a Chebyshev solve on the coarsest level.  PCG in FP64; the V-cycle in FP32
 * when the levels carry FP32 copies (values32, dinv32), else FP64.  No
 * FEALPy counterpart for
 * the individual kernels.
 *
 * One level (caller-owned arrays; agg, member_ptr, members and n_coarse for
 * every level but the coarsest). */
#define FGB_AMG_MAX_LEVELS 16
typedef struct fgb_amg_level {
  int64_t n, nnz;
  const int64_t* indptr;    /* CSR of the level's matrix                      */
  const int32_t* indices;
  const double* values;
  const double* dinv;       /* 1 / a_ii                                       */
  double lmax;              /* Gershgorin bound of D^-1 A                     */
  const int32_t* agg;       /* aggregate of every row, -1: none               */
  int64_t n_coarse;         /* aggregates = rows of the next level            */
  const int64_t* member_ptr; /* n_coarse + 1: rows of each aggregate,         */
  const int32_t* members;    /* ascending                                     */
  const float* values32;     /* optional FP32 copies of values and dinv, set  */
  const float* dinv32;       /* on every level or on none: with them the      */
                             /* V-cycle runs in FP32 (vectors and arithmetic) */
  const struct fgb_sell* sell; /* optional SELL copy of the level: its         */
                             /* smoothing and residual sweeps run on the copy */
                             /* when it holds values of the V-cycle's type;   */
                             /* on level 0 PCG's operator product runs on its */
                             /* FP64 values when present                      */
} fgb_amg_level;

/* Aggregates of a level: agg (n), their number, dinv (n) and lmax. */
size_t fgb_amg_setup_workspace_bytes(int64_t n);
int32_t fgb_amg_aggregate(int64_t n, const int64_t* indptr, const int32_t* indices,
                          const double* values, double theta, int32_t* agg, int64_t* n_agg_host,
                          double* dinv, double* lmax_host, int32_t* status, void* workspace,
                          size_t workspace_bytes, void* stream);
/* The next level: member lists and the coarse row pointer (count, which
 * returns its nnz on the host), then its columns and values (fill, same
 * workspace).  Columns ascending; every coarse value is the sum of its fine
 * entries taken member row by member row, in CSR order. */
size_t fgb_amg_coarse_workspace_bytes(int64_t n, int64_t n_coarse);
int32_t fgb_amg_coarse_count(int64_t n, const int64_t* indptr, const int32_t* indices,
                             const double* values, const int32_t* agg, int64_t n_coarse,
                             int64_t* member_ptr, int32_t* members, int64_t* coarse_indptr,
                             int64_t* nnz_host, int32_t* status, void* workspace,
                             size_t workspace_bytes, void* stream);
int32_t fgb_amg_coarse_fill(int64_t n, const int64_t* indptr, const int32_t* indices,
                            const double* values, const int32_t* agg, int64_t n_coarse,
                            const int64_t* member_ptr, const int32_t* members,
                            const int64_t* coarse_indptr, int32_t* coarse_indices,
                            double* coarse_values, int32_t* status, void* workspace,
                            size_t workspace_bytes, void* stream);
/* x = V-cycle(r) (x = 0 start; deg: smoothing degree, cdeg: degree of the
 * coarsest solve) and PCG with it (FEALPy's recurrence and stopping rule;
 * norm 0: sqrt(r.z), 1: ||r||; info->true_relres = -1). */
size_t fgb_amg_workspace_bytes(const fgb_amg_level* levels, int32_t n_levels);
int32_t fgb_amg_vcycle(const fgb_amg_level* levels, int32_t n_levels, int32_t deg, int32_t cdeg,
                       double omega, const double* r, double* x, void* workspace,
                       size_t workspace_bytes, void* stream);
int32_t fgb_pcg_amg(const fgb_amg_level* levels, int32_t n_levels, int32_t deg, int32_t cdeg,
                    double omega, const double* b, double* x, double atol, double rtol, int64_t maxit,
                    int32_t norm, fgb_pcg_info* info_host, void* workspace, size_t workspace_bytes,
                    void* stream);

/* ---- batched FP32-refined Jacobi-PCG over many systems ------------------ */

/* No FEALPy counterpart: FEALPy solves one system per fealpy/solver/cg.py
 * call.  Here many independent systems (meshes of uneven size and degree,
 * each with its own SELL copy and Krylov vectors) advance together: every
 * kernel of an iteration walks a list of tiles (a tile = one system's range
 * of slices or rows), every dot product is reduced per system in a fixed
 * order (so a system's iterates do not depend on the other systems in the
 * batch), and the loop runs as one CUDA graph with a device-side while node.
 * Systems are admitted into free slots and retired between runs (continuous
 * batching).  Same iteration, reliable updates and stopping rule as
 * fgb_pcg_sell_mixed, per system. */
typedef struct fgb_batch_system {
  int64_t n;                /* rows                                        */
  int64_t n_slices;         /* SELL slices (fgb_sell_slots(n) / 32)        */
  const int64_t* slice_ptr; /* SELL copy of the matrix (fgb_sell fields)   */
  const int32_t* perm;
  const int32_t* col;
  const float* val32;       /* FP32 values (required unless fp64)          */
  const double* val64;      /* FP64 values (required if fp64, else optional */
                            /* for the residual recomputation)             */
  const double* dinv64;     /* 1 / diag(A)                                 */
  const double* b;          /* right-hand side (FP64)                      */
  double* x;                /* x0 on admission, the solution on retirement */
  void* r;                  /* Krylov vectors, n entries each, owned by    */
  void* z;                  /* the caller: float, or double when fp64      */
  void* p;
  void* Ap;
  void* y;
  void* dinv32;             /* float inverse diagonal (unused when fp64)   */
  int32_t fp64;             /* 1: this system iterates in FP64             */
  int32_t reserved;
} fgb_batch_system;

/* Per-system state (device array; read back by fgb_batch_run). */
typedef struct fgb_batch_state {
  double rz, rz_prev, rr, alpha, beta, b_norm, tol, resid, r_upd, true_rel, delta;
  int64_t niter, maxit;
  int32_t active;      /* 1 while the system takes part in the loop       */
  int32_t done;        /* FGB_PCG_* reason once finished, 0 while running */
  int32_t need_update; /* 1: reliable update due, 2: admission pending,   */
                       /* 3: true-residual check on a plateau            */
  int32_t n_updates;
  int32_t reserved;
  int32_t stall;       /* true-residual checks without a 2x improvement   */
  double r_best;       /* best true residual norm so far                  */
  int64_t last_upd;    /* iteration of the last reliable update           */
  int64_t max_gap;     /* longest interval between reliable updates       */
} fgb_batch_state;

/* A tile: rows or slices [begin, end) of system `sys`.  Tiles of a system
 * are consecutive in their list; tile_ptr[s]..tile_ptr[s+1] are its tiles. */
typedef struct fgb_batch_tile {
  int32_t sys, begin, end, reserved;
} fgb_batch_tile;

typedef struct fgb_batch fgb_batch; /* opaque: device tables + the graph    */

size_t fgb_batch_bytes(int32_t max_sys, int32_t max_slice_tiles, int32_t max_row_tiles);
/* device_buffer (fgb_batch_bytes bytes, caller-owned) holds the tables, the
 * states and the per-tile partials.  slice_threads: threads per block of the
 * slice kernels (a multiple of 32 in [64, 1024]). */
int32_t fgb_batch_create(int32_t max_sys, int32_t max_slice_tiles, int32_t max_row_tiles,
                         int32_t slice_threads, void* device_buffer, size_t bytes,
                         fgb_batch** out);
int32_t fgb_batch_destroy(fgb_batch* batch);
/* Replace the system table and both tile lists (host arrays, copied). */
int32_t fgb_batch_set(fgb_batch* batch, int32_t n_sys, const fgb_batch_system* systems,
                      int32_t n_slice_tiles, const fgb_batch_tile* slice_tiles,
                      const int32_t* slice_tile_ptr, int32_t n_row_tiles,
                      const fgb_batch_tile* row_tiles, const int32_t* row_tile_ptr,
                      void* stream);
/* Admit systems (slot ids): reset their state, then ||b||, the initial FP64
 * residual, z and p on the device. */
int32_t fgb_batch_admit(fgb_batch* batch, int32_t n, const int32_t* slots, const double* rtol,
                        const int64_t* maxit, double delta, void* stream);
/* Iterate all admitted, unfinished systems for at most trip_limit
 * iterations (use_graph: one graph launch; else one launch per kernel) and
 * copy the first n_sys states to states_host.  *running: systems still
 * unfinished. */
int32_t fgb_batch_run(fgb_batch* batch, int64_t trip_limit, int32_t use_graph,
                      fgb_batch_state* states_host, int32_t* running, int32_t* used_graph,
                      void* stream);
/* Retire systems: add the pending FP32 correction into x, zero x of a zero
 * right-hand side, and mark the slots inactive. */
int32_t fgb_batch_retire(fgb_batch* batch, int32_t n, const int32_t* slots, void* stream);
/* y_s = A_s x_s in FP32 for every system of the table (x, y: per-system
 * device pointers, host arrays of n_sys entries); used by the autotuner. */
int32_t fgb_batch_spmv(fgb_batch* batch, const float* const* x, float* const* y, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FEALPY_GB300_H */
