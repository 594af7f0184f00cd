/*
 * fem2d_gb300 — C ABI of the GB300 implementation of fem_2d's Galerkin generalized-eigenproblem
 * path (H(curl) Maxwell, refinement-by-superposition meshes).
 *
 * Conventions: every function returns an int status (FEM2D_OK = 0) unless it returns a handle
 * count or pointer; fem2d_last_error() gives the message of the last failure on the calling thread.
 * Handles are not thread-safe. Output buffers are owned by the caller. No C++ exception crosses
 * this boundary. Matrix entries are FP64; row pointers int64; column indices int32.
 *
 * Each entry point cites the reference item (jeremiah-corrado/fem_2d, path:line) it stands in for.
 */
#ifndef FEM2D_GB300_H
#define FEM2D_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mirror GalerkinSamplingError galerkin.rs:190-195, NalgebraGEPError
 *      nalgebra_solve.rs:52-56, SlepcGEPError slepc_solve.rs:70-81, HRefError/PRefError) ---- */
enum {
  FEM2D_OK = 0,
  FEM2D_E_INVALID_ARG = 1,
  FEM2D_E_MESH = 2,            /* malformed mesh file / inconsistent mesh (Mesh::from_file panics) */
  FEM2D_E_HREF = 3,            /* HRefError (h_refinement.rs:290-302) */
  FEM2D_E_PREF = 4,            /* PRefError (p_refinement.rs:274-283) */
  FEM2D_E_WRONG_CC = 5,        /* GalerkinSamplingError::WrongContinuityCondition */
  FEM2D_E_EMPTY_DOFS = 6,      /* GalerkinSamplingError::EmptyDOFSet */
  FEM2D_E_INVALID_GLQ = 7,     /* GalerkinSamplingError::InvalidGLQSettings */
  FEM2D_E_B_NOT_SPD = 8,       /* NalgebraGEPError::FailedToInvertB */
  FEM2D_E_SPURIOUS = 9,        /* NalgebraGEPError::SpuriouslyConverged */
  FEM2D_E_TOO_LARGE = 10,      /* NalgebraGEPError::ProblemTooLarge */
  FEM2D_E_NOT_CONVERGED = 11,  /* SlepcGEPError::FailedToConverge */
  FEM2D_E_CUDA = 12,           /* CUDA runtime failure */
  FEM2D_E_TIMEOUT = 13,        /* a device-side bounded wait gave up */
  FEM2D_E_NO_DEVICE = 14,
  FEM2D_E_IO = 15
};

/* ContinuityCondition (domain.rs:17-23) */
enum { FEM2D_CC_HCURL = 0, FEM2D_CC_HDIV = 1, FEM2D_CC_DISCONTINUOUS = 2 };
/* HRef (h_refinement.rs:56-61): T, U, V; ext = -1 (None) or child index 0/1 for U->V / V->U */
enum { FEM2D_HREF_T = 0, FEM2D_HREF_U = 1, FEM2D_HREF_V = 2 };
/* Basis spaces: HierPoly (hierarchical_basis_fns.rs:1-199) and KOLeg, the Legendre space that
 * restates HierMaxOrtho (hierarchical_basis_fns.rs:201-647) */
enum { FEM2D_BASIS_HIERPOLY = 0, FEM2D_BASIS_KOLEG = 1 };
/* GEP matrices */
enum { FEM2D_MAT_A = 0, FEM2D_MAT_B = 1 };
/* preconditioners of the sparse shift-invert solve */
enum { FEM2D_PRECOND_BLOCK_JACOBI = 0, FEM2D_PRECOND_LEARNED = 1 };

typedef struct fem2d_mesh fem2d_mesh;
typedef struct fem2d_domain fem2d_domain;
typedef struct fem2d_ctx fem2d_ctx;
typedef struct fem2d_gep fem2d_gep;

const char* fem2d_last_error(void);
const char* fem2d_version(void);

/* ---------------- Mesh (src/fem_domain/domain/mesh.rs) ---------------- */
/* Mesh::from_file (mesh.rs:142-327): JSON text in the reference's format */
int fem2d_mesh_from_json(const char* json_text, fem2d_mesh** out);
/* Mesh::from_file with a path */
int fem2d_mesh_from_file(const char* path, fem2d_mesh** out);
/* Mesh::unit (mesh.rs:58-91) */
int fem2d_mesh_unit(fem2d_mesh** out);
/* Mesh::clone */
int fem2d_mesh_clone(const fem2d_mesh* m, fem2d_mesh** out);
void fem2d_mesh_free(fem2d_mesh* m);
/* set_global_expansion_orders / set_expansion_on_elems (mesh.rs:1446-1468); ids == NULL: all Elems */
int fem2d_mesh_set_expansion_orders(fem2d_mesh* m, const int64_t* ids, int64_t n, int i, int j);
/* global_p_refinement (mesh.rs:1236-1253, ids == NULL, clamped) / p_refine_elems (mesh.rs:1266-1276) */
int fem2d_mesh_p_refine(fem2d_mesh* m, const int64_t* ids, int64_t n, int di, int dj);
/* global_h_refinement (mesh.rs:681-696, ids == NULL) / h_refine_elems (mesh.rs:716-726) */
int fem2d_mesh_h_refine(fem2d_mesh* m, const int64_t* ids, int64_t n, int kind, int ext);
/* execute_h_refinements (mesh.rs:844-914): per-Elem refinement kinds (kinds[k] applies to ids[k]) */
int fem2d_mesh_execute_h_refinements(fem2d_mesh* m, const int64_t* ids, const int32_t* kinds, int64_t n);
int64_t fem2d_mesh_num_elems(const fem2d_mesh* m);
int64_t fem2d_mesh_num_edges(const fem2d_mesh* m);
int64_t fem2d_mesh_num_nodes(const fem2d_mesh* m);
/* per Elem, 14 int64: [is_leaf, ni, nj, parent(-1), nodes[4], edges[4], h_u, h_v] */
int fem2d_mesh_elem_info(const fem2d_mesh* m, int64_t* out);
/* per Elem: 4 doubles (x_min, y_min, x_max, y_max) of its real-space extent */
int fem2d_mesh_elem_bounds(const fem2d_mesh* m, double* out);

/* ---------------- Domain (src/fem_domain/domain.rs) ---------------- */
/* Domain::from_mesh (domain.rs:69-159): the mesh is copied (the reference consumes it) */
int fem2d_domain_from_mesh(const fem2d_mesh* m, int cc, fem2d_domain** out);
void fem2d_domain_free(fem2d_domain* d);
int64_t fem2d_domain_num_dofs(const fem2d_domain* d);
int64_t fem2d_domain_num_specs(const fem2d_domain* d);
/* Domain::basis_specs flattened in (elem, elem_idx) order: per spec 6 int64
 * [elem_id, elem_idx, i, j, dir(0=U,1=V), dof_id] */
int fem2d_domain_basis_specs(const fem2d_domain* d, int64_t* out);

/* Sparsity pattern of A and B (both share it) as the upper-triangle keys, sorted by (row, col): the
 * SparseMatrix BTreeMap keys (sparse_matrix.rs:12-15, 68-98) galerkin_sample_gep_hcurl would produce.
 * Host-only (no device work). Call with rows == cols == NULL to get *nnz_upper first. */
int fem2d_domain_pattern(const fem2d_domain* d, int64_t* nnz_upper, int32_t* rows, int32_t* cols);

/* Factorization plan of the shifted pencil (host-only): the nested dissection of the base Elems into
 * dense fronts used by the sparse eigensolver. No reference counterpart (the reference hands the
 * matrices to an external SLEPc process, slepc_solve.rs:26-36). Two-call pattern: with all array
 * pointers NULL it fills sizes[8] = {nfronts, dofs_len, asm_len, ea_len, nlevels, max_f, max_p,
 * factor_entries}; then fronts[4*nfronts] = {parent, level, f, p} and the CSR-style lists. */
int fem2d_domain_factor_plan(const fem2d_domain* d, int64_t* sizes, int32_t* fronts, int64_t* dof_ptr,
                             int32_t* dofs, int64_t* asm_ptr, int64_t* asm_pos, int64_t* asm_csr, int64_t* ea_ptr,
                             int32_t* ea_map);

/* ---------------- device context ---------------- */
int fem2d_ctx_create(int device, fem2d_ctx** out);
void fem2d_ctx_destroy(fem2d_ctx* c);
int fem2d_ctx_synchronize(fem2d_ctx* c);
/* writes a 256 MiB device buffer so the next launch starts from a cold L2 */
int fem2d_ctx_flush_l2(fem2d_ctx* c);
/* number of kernels this library launched on the context since creation */
int64_t fem2d_ctx_kernel_launches(const fem2d_ctx* c);
/* device timer on the context's stream (CUDA events): start, then stop returns elapsed ms */
int fem2d_ctx_timer_start(fem2d_ctx* c);
int fem2d_ctx_timer_stop(fem2d_ctx* c, double* ms);
/* per-region device timing (synchronising, for measurement runs): regions "assembly_values", "spmm",
 * "mf_factor", "mf_solve" (one forward + backward solve), "dense_block" (the eigensolver's FP64 grams and
 * block products); query returns total ms, calls and algorithmic bytes */
int fem2d_ctx_set_profiling(fem2d_ctx* c, int on);
int fem2d_ctx_profile_reset(fem2d_ctx* c);
int fem2d_ctx_profile_query(const fem2d_ctx* c, const char* region, double* ms, int64_t* count, double* bytes);
/* algorithmic FP64 flops of a profiled region ("spmm": 2 nnz nb per call; "mf_solve": 2 per factor
 * entry read, per right-hand side, both directions) */
int fem2d_ctx_profile_flops(const fem2d_ctx* c, const char* region, double* flops);
/* measured FP64 FMA throughput of this device (TFLOP/s): independent fused multiply-add chains on every
 * SM for about 20 ms; the denominator of the FP64-bound kernels' roofline (no reference counterpart) */
int fem2d_ctx_fp64_peak(fem2d_ctx* c, double* tflops);
/* measured issue cost of one tcgen05.mma (kind::f16, M = 128, K = 16) with the given N (a multiple of 16
 * in 16..256), in ns per instruction and SM: the cost model behind the shapes of the tensor-core FP64
 * emulation (no reference counterpart). FEM2D_E_TIMEOUT if the kernel's bounded wait expired. */
int fem2d_ctx_mma_ns(fem2d_ctx* c, int n, double* ns);

/* ---------------- Galerkin sampling (src/fem_problem/galerkin.rs:33-187) ---------------- */
/* galerkin_sample_gep_hcurl::<BSpace, CurlCurl, L2Inner>(&domain, Some([nq_u, nq_v])).
 * nq_u = nq_v = 0 means None (default_ngq, basis.rs:172-177). The sparsity pattern of A and B is
 * built on the host (bit-exact with the reference's BTreeMap keys); the values are computed on the
 * GPU and stay resident in device memory. */
int fem2d_galerkin_sample_gep_hcurl(fem2d_ctx* c, const fem2d_domain* d, int basis, int nq_u, int nq_v,
                                    fem2d_gep** out);
/* Numeric phase only: recompute the values of an existing GEP on the device (same domain and
 * settings). Used to time the device kernels with inputs resident in device memory. */
int fem2d_gep_recompute(fem2d_ctx* c, fem2d_gep* g);
/* Allocation-free recomputation of the A and B values (no counterpart in the reference).
 * For hosts that own all device memory themselves (a pool or arena that must account for every
 * byte, so the library may not allocate behind its back) or that cannot afford cudaMalloc/cudaFree
 * on their critical path. The caller passes device arrays d_a and d_b of nnz_full doubles (full CSR
 * order, as fem2d_gep_export_csr); the inputs are the GEP's resident pattern and contribution lists.
 * The 1-D contraction tables live in one file-scope device array of 4 MiB (524288 doubles); a GEP
 * needing more (2 x intervals x 5 x (max order + 1)^2) is rejected with FEM2D_E_TOO_LARGE. Each GPU
 * that loads the library holds that array until the process exits. The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress); make that first call before any stream
 * capture. Later calls outside a capture look it up again, so a context rebuilt after
 * cudaDeviceReset is handled. All calls share the one array: calls that overlap on the GPU (other
 * streams, other host threads) race on it. Nothing in it needs clearing between calls. d_a and d_b
 * must be device (or managed) memory of the context's device, else FEM2D_E_INVALID_ARG. The caller's
 * current device is restored on return. Returns after the work is queued on the context's stream;
 * synchronise before reading d_a and d_b. No cudaMalloc, cudaFree or other allocating call is made. */
int fem2d_gep_values_noalloc(fem2d_ctx* c, const fem2d_gep* g, double* d_a, double* d_b);
/* The FP64 contraction-table size (doubles) a GEP of this Domain needs: 2 x intervals x 5 x
 * (max order + 1)^2, the quantity fem2d_gep_values_noalloc checks against its capacity. Runs the host
 * symbolic phase only (no GPU needed); errors as fem2d_galerkin_sample_gep_hcurl's argument checks.
 * No counterpart in the reference. */
int fem2d_domain_table_doubles(const fem2d_domain* d, int basis, int nq_u, int nq_v, int64_t* doubles);
/* galerkin_sample_gep_hcurl over many Domains at once (galerkin.rs:33-187 per Domain; the reference
 * has no batched form: a caller loops over Domains). Each Domain gets its own host symbolic phase and
 * its own GEP (out[i], freed with fem2d_gep_free); the device numeric phase of ALL of them is two
 * launches: the 1-D contraction tables of every Domain in one, then one persistent launch over the
 * concatenated CSR entries of every GEP (uneven expansion orders share the launch). autotune != 0
 * picks the value kernel's launch shape by timing a fixed candidate list on the first batch of a
 * size class and caches it per process (fem2d_autotune_export/import). Errors as
 * fem2d_galerkin_sample_gep_hcurl, checked for every Domain before any work. report (optional,
 * 6 doubles): device ms of the table launch, device ms of the value launch, threads per CTA, CTAs
 * per SM, total CSR entries, total visit codes. */
int fem2d_galerkin_sample_gep_hcurl_batch(fem2d_ctx* c, const fem2d_domain* const* domains, int64_t count, int basis,
                                          int nq_u, int nq_v, int autotune, fem2d_gep** out, double* report);
/* Numeric phase only, for GEPs already built (by either entry point) on this device: the same two
 * batched launches over all of them. report as above. */
int fem2d_gep_batch_recompute(fem2d_ctx* c, fem2d_gep* const* geps, int64_t count, int autotune, double* report);
/* The autotuner's cache as text, one "key threads ctas_per_sm" line per entry (key = device name,
 * table stride and size class). export: length (without the NUL) is returned in *length; buf may be
 * NULL to query it. import: adds/overwrites entries; shapes outside the candidate list are
 * FEM2D_E_INVALID_ARG. */
int fem2d_autotune_export(char* buf, int64_t capacity, int64_t* length);
int fem2d_autotune_import(const char* text, int64_t* entries);
int fem2d_autotune_clear(void);
void fem2d_gep_free(fem2d_gep* g);
/* dims: ndofs, upper-triangle entry count (SparseMatrix::entries), full symmetric nnz
 * (SparseMatrix::num_entries, sparse_matrix.rs:32-35) */
int fem2d_gep_dims(const fem2d_gep* g, int64_t* ndofs, int64_t* nnz_upper, int64_t* nnz_full);
/* upper triangle as COO sorted by (row, col), like SparseMatrix::iter_upper_tri (sparse_matrix.rs:122-126) */
int fem2d_gep_export_upper(const fem2d_gep* g, int32_t* rows, int32_t* cols, double* a, double* b);
/* replace A and B by caller values, given per upper-triangle entry in fem2d_gep_export_upper's order
 * (mirrored into the full symmetric pattern on the device); the reference's GEP exposes its matrices as
 * public fields (`pub a: SparseMatrix, pub b: SparseMatrix`, linalg.rs:29-34) that callers may edit
 * before a solve. The pattern is kept. Rejects a non-finite entry with FEM2D_E_INVALID_ARG. A later
 * fem2d_gep_recompute overwrites the values with the assembled ones. */
int fem2d_gep_set_upper_values(fem2d_gep* g, const double* a, const double* b);
/* integrate_by_parts (CurlCurl integrals.rs:94-237, L2Inner integrals.rs:356-418) evaluated on the device
 * over the GEP's Galerkin visit set (galerkin.rs:73-184; the reference has no by-parts driver): per upper
 * entry, in fem2d_gep_export_upper's order, 6 doubles [CurlCurl face term, edge terms 0..3, L2Inner],
 * each summed over the entry's visits. Samplers with second derivatives and GLQ points plus the
 * endpoints (glq.rs:179-222), the GEP's own GLQ sizes. face + edges equals A up to rounding. */
int fem2d_gep_by_parts(fem2d_ctx* c, const fem2d_gep* g, double* vals6);
/* full symmetric CSR (row_ptr: ndofs+1, col/val: nnz_full) of A or B */
int fem2d_gep_export_csr(const fem2d_gep* g, int which, int64_t* row_ptr, int32_t* col, double* val);
/* timings (ms): [tables, values, tables + values] of the last galerkin/recompute call (device), then
   [host symbolic phase, upload] of the galerkin call that built the GEP */
int fem2d_gep_timings(const fem2d_gep* g, double* out5);
/* visit count P_visits = sum_E [n(E)(n(E)+1)/2 + n(E) sum_D n(D)] (the reference's integrate calls) */
int64_t fem2d_gep_num_visits(const fem2d_gep* g);
/* bytes copied host -> device when the GEP was built (pattern, contribution lists, tables) */
int64_t fem2d_gep_h2d_bytes(const fem2d_gep* g);

/* ---------------- Eigensolvers (src/fem_problem/linalg/{nalgebra_solve,slepc_solve}.rs) ---------------- */
/* nalgebra_solve_gep (nalgebra_solve.rs:14-50) on the device: B = L L^T, the product B^-1 A, the
 * symmetric eigen-decomposition of its lower triangle, the pair nearest target. ndofs <= 1000. */
int fem2d_dense_solve_gep(fem2d_ctx* c, const fem2d_gep* g, double target, double* value, double* vector);

/* Solve (c_a A + c_b B) X = R for nrhs right-hand sides (host, row-major n x nrhs) with the device
 * multifrontal LU (partial pivoting within fully-summed rows). No reference counterpart: the
 * reference only forms the GEP; this is the linear solve its shift-invert eigensolve relies on.
 * Returns FEM2D_E_B_NOT_SPD if spd != 0 and a non-positive pivot appears. */
int fem2d_gep_shifted_solve(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, int spd, int nrhs,
                            const double* rhs, double* x);

/* Y = c_a A X + c_b B X with the GEP's device-resident A and B: the operator products an external
 * eigensolver applies to the GEP (MatMult in the PETSc hand-off of slepc_solve.rs:14-68). d_x and
 * d_y are device pointers to row-major n x nb blocks (leading dimensions ldx, ldy), 1 <= nb <= 32,
 * d_x and d_y must not overlap. Queued on the context's stream; returns without synchronising. */
int fem2d_gep_spmm_device(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, const double* d_x, int64_t ldx,
                          int nb, double* d_y, int64_t ldy);
/* C = X^T Y for device blocks X (n x a, row-major, leading dimension ldx) and Y (n x b, ldy) into the
 * device array d_c (a x b, row-major): the block Gram product of gpu_solve_gep's B-orthogonalisation
 * and Rayleigh-Ritz steps (no counterpart in the reference, whose eigensolve runs in an external
 * process), exposed for checking and timing. method 0: FP64 emulated on the tensor cores (tcgen05 MMA
 * on exact 7-bit digit slices with exact FP32 accumulation; a <= 512, b <= 256; normwise accuracy at
 * FP64 rounding level), method 1: FP64 on the CUDA cores. Synchronises; FEM2D_E_TIMEOUT if a bounded
 * wait inside the tensor kernel expired. */
/* Y = coef M X with M = A (which 0) or B (which 1) of the GEP, on the tensor cores: FP64 emulated by
 * exact 7-bit digit slices of M's values (one exponent per row and 64-column chunk of each row run)
 * and of X (one exponent per column and chunk), FP32-exact digit sums in TMEM, exact int64 recombination;
 * every row of Y is written, and the result does not depend on scheduling (bitwise reproducible).
 * The operator product gpu_solve_gep uses for its T applications and basis products (no counterpart in the
 * reference), exposed for checking and timing; the values are sliced on every call here. Device row-major
 * n x nb blocks, 1 <= nb <= 32. Synchronises. */
int fem2d_gep_spmm_tensor_device(fem2d_ctx* c, const fem2d_gep* g, int which, double coef, const double* d_x,
                                 int64_t ldx, int nb, double* d_y, int64_t ldy);
int fem2d_block_gram_device(fem2d_ctx* c, int method, int64_t n, const double* d_x, int64_t ldx, int a,
                            const double* d_y, int64_t ldy, int b, double* d_c);
/* Z = beta Z + alpha X C for device blocks X (n x a, ldx), C (a x b, row-major) and Z (n x b, ldz): the
 * block updates of gpu_solve_gep's B-orthogonalisation and its Ritz-vector products (no counterpart in
 * the reference), exposed for checking and timing. method 0: FP64 emulated on the tensor cores (a <= 256,
 * b <= 32), 1: FP64 CUDA cores. Synchronises; FEM2D_E_TIMEOUT as fem2d_block_gram_device. */
int fem2d_block_gemm_device(fem2d_ctx* c, int method, int64_t n, const double* d_x, int64_t ldx, int a,
                            const double* d_c, int b, double alpha, double beta, double* d_z, int64_t ldz);
typedef struct fem2d_patchnet fem2d_patchnet;
typedef struct fem2d_solve_opts {
  int precond;          /* how T = (A - s B)^-1 A (A + c B)^-1 B solves its two shifted systems (the KSP
                           solves of the external SLEPc process, slepc_solve.rs:26-36):
                           0 = exact multifrontal LU (default);
                           1 = preconditioned CG on A + c B and preconditioned MINRES on A - s B, with
                               the plain additive-Schwarz (per-Elem block-Jacobi) preconditioner;
                           2 = the same with the learned two-level preconditioner of `net` */
  int max_outer;        /* outer (restart) cycles, 0 = default 40 */
  int max_inner;        /* iterations per inner CG / MINRES solve (precond 1, 2), 0 = default 5000 */
  double tol;           /* relative residual ||Ax - lambda Bx|| / (|lambda| ||Bx||), 0 = default 1e-10 */
  double inner_tol;     /* relative residual of each inner solve (precond 1, 2), 0 = default 1e-10 */
  int block;            /* block size, 0 = default (n_pairs + guard: guard = 4 from 100,000 DoFs, else
                           max(4, n_pairs / 2)) */
  int verbose;
  int krylov_steps;     /* block Krylov steps per restart cycle (at most 8), 0 = default (5 from 100,000
                           DoFs, else 4) */
  double damping;       /* null-space damping c / |sigma| of T = (A - sigma B)^-1 A (A + c B)^-1 B,
                           0 = default (1 from 10,000 DoFs, 0.05 below) */
  int scaling;          /* 0 = automatic (row-run blocks from 10,000 DoFs; below, Jacobi, switching to
                           row-run blocks when the Jacobi-scaled factorizations are inaccurate),
                           1 = Jacobi only, 2 = row-run blocks (Cholesky factors of B's diagonal blocks
                           over runs of rows with one column list) */
  int dense;            /* the eigensolver's FP64 contractions: 0 = default: from 50,000 DoFs the Gram
                           products and block updates of the B-orthogonalisation and Rayleigh-Ritz steps
                           emulated on the tensor cores (tcgen05, exact integer slicing), and from
                           1,000,000 nonzeros the operator products as well; below, FP64 CUDA cores;
                           1 = everything on the FP64 CUDA cores; 2 = everything on the tensor cores at
                           every size; 3 = tensor-core Gram products and block updates at every size,
                           operator products on the FP64 CUDA cores */
  const fem2d_patchnet* net;   /* trained patch network (precond 2), else NULL */
  int refine;           /* FP64 iterative-refinement steps per exact shifted solve: 0 = calibrated on a random
                           block (default: none when the solves are backward stable, normwise backward
                           error below 1e-13; else up to 3 while they reduce the residual), k > 0 = k
                           steps (at most 3), -1 = none */
} fem2d_solve_opts;

typedef struct fem2d_solve_stats {
  int outer_iters;
  int inner_iters_total;
  int converged;
  double t_setup_ms, t_solve_ms;
  double max_rel_residual;
  int64_t spmv_count;
  int refine_spd, refine_indefinite;   /* iterative-refinement steps per solve with A + cB and A - sigma B */
  int dense_plan;      /* 1: the factorization used one dense front (small, ill-conditioned GEP) */
  int floor_reached;   /* 1: some pair was accepted by its backward error (below 1e-14) or at the residual
                          floor (eight cycles without progress, below 1e-6) rather than by tol */
  int block_scaled;    /* 1: the pencil was scaled by Cholesky factors of B's row-run diagonal blocks */
  int delayed_pivots;  /* DoFs whose elimination moved to a parent front (no stable pivot in their own) */
  double max_backward_error;  /* max over the pairs of ||Ax - lambda Bx|| / ((||A|| + |lambda| ||B||) ||x||) */
  int64_t inner_cg_iters;      /* precond 1, 2: CG iterations summed over the inner block solves */
  int64_t inner_minres_iters;  /* precond 1, 2: MINRES iterations summed over the inner block solves */
  double inner_max_relres;     /* precond 1, 2: largest final relative residual of an inner solve */
} fem2d_solve_stats;

/* gpu_solve_gep: the n_pairs eigenpairs of (A, B) nearest target, by a shift-invert block
 * eigensolver on the device. Stands beside slepc_solve_gep (slepc_solve.rs:14-68).
 * values: n_pairs, sorted by |lambda - target|; vectors: n_pairs x ndofs row-major, B-normalised;
 * residuals: n_pairs relative residuals computed in FP64. Any output pointer may be NULL. */
int fem2d_gpu_solve_gep(fem2d_ctx* c, const fem2d_gep* g, double target, int n_pairs, const fem2d_solve_opts* opts,
                        double* values, double* vectors, double* residuals, fem2d_solve_stats* stats);

/* ---------------- Files of the external-solver hand-off (linalg.rs, sparse_matrix.rs, slepc_solve.rs) -------- */
/* GEP::print_to_petsc_binary_files (linalg.rs:44-52): writes {dir}/tmp/{prefix}_a.dat and _b.dat in the
 * AIJMatrixBinary layout of sparse_matrix.rs:184-265 (bytes "\0{P", then u32 rows, cols, nnz, the
 * per-row counts, the column indices, all big-endian, then the f64 values; both triangles, rows and
 * columns ascending). The directory {dir}/tmp must exist. */
int fem2d_gep_print_to_petsc_binary_files(const fem2d_gep* g, const char* dir, const char* prefix);
/* the same layout from a host CSR (columns ascending within each row) */
int fem2d_aij_write(const char* path, int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val);
/* reads that layout (or the standard PETSc one with the four-byte class id 1211216) into a CSR; call
 * with NULL arrays first to learn n and nnz */
int fem2d_aij_read(const char* path, int64_t* n, int64_t* nnz, int64_t* row_ptr, int32_t* col, double* val);
/* retrieve_eigenvector (slepc_solve.rs:114-135): PETSc Vec binary (i32 class id 1211214, i32 m, m f64,
 * big-endian); read: call with out == NULL to learn n */
int fem2d_petsc_vec_write(const char* path, const double* v, int64_t n);
int fem2d_petsc_vec_read(const char* path, double* out, int64_t capacity, int64_t* n);
/* retrieve_eigenvalue (slepc_solve.rs:137-147): one big-endian f64 */
int fem2d_petsc_scalar_write(const char* path, double x);
int fem2d_petsc_scalar_read(const char* path, double* x);

/* ---------------- Field evaluation (src/fem_domain/domain/fields.rs) ---------------- */
typedef struct fem2d_fields fem2d_fields;
/* UniformFieldSpace::new (fields.rs:29-39) plus the evaluation plan of xy_fields for one basis space
 * (the reference's BSpace type parameter): a d0 x d1 grid of uniform_range(-1, 1, d) points
 * (fields.rs:386-389) on every leaf Elem. Requires 2 <= d0, d1 <= 1024 and an H(curl) Domain. The
 * reference indexes its per-leaf arrays as [d1][d0] but fills them [m < d0][n < d1], which only runs
 * when d0 == d1; here the layout is [m][n] for every d0, d1, equal to the reference's when d0 == d1. */
int fem2d_fields_create(fem2d_ctx* c, const fem2d_domain* d, int basis, int d0, int d1, fem2d_fields** out);
void fem2d_fields_free(fem2d_fields* f);
/* leaf Elems in ascending id (the reference's BTreeMap order, fields.rs:330-346) */
int64_t fem2d_fields_num_leaves(const fem2d_fields* f);
int fem2d_fields_leaves(const fem2d_fields* f, int64_t* ids);
/* per leaf, 4 doubles: the real-space points of nodes[0] and nodes[3] (elem_diag_points, used for the
 * VTK point grid of print_quantities_to_vkt, fields.rs:181-193) as (x0, y0, x3, y3) */
int fem2d_fields_leaf_bounds(const fem2d_fields* f, double* out);
/* xy_fields (fields.rs:63-122): x and y field values, each num_leaves x d0 x d1 doubles, [leaf][m][n]
 * with m along u (x) and n along v (y). n_solution != num_dofs fails with FEM2D_E_INVALID_ARG
 * (MismatchedSolutionSize). Host pointers; synchronous. */
int fem2d_fields_xy(fem2d_fields* f, const double* solution, int64_t n_solution, double* x_out, double* y_out);
/* the same on device pointers (an eigenvector left on the device); asynchronous on the context's stream */
int fem2d_fields_xy_device(fem2d_fields* f, const double* d_solution, int64_t n_solution, double* d_x, double* d_y);

/* ---------------- inner PCG solver and learned preconditioner (no reference counterpart) ----------
 * The reference hands the shifted systems of its sparse eigensolve to SLEPc/PETSc KSP in an external
 * process (slepc_solve.rs:14-68). This is the device inner solver for SPD shifts K = c_a A + c_b B
 * (c_a, c_b > 0): conjugate gradients preconditioned by
 *   net == NULL: additive Schwarz over Elem patches (exact inverse of each Elem's block of K, every
 *                basis function of the Elem, shared edge functions included) -- the plain method;
 *   net != NULL: the same plus a two-level coarse correction whose basis the per-Elem-patch network
 *                produces (k vectors per Elem from the features of its basis functions; coarse
 *                operator Z^T K Z inverted densely, at most 16384 coarse vectors).
 * The network (an MLP 16 -> hidden -> hidden -> k, tanh, FP32) is trained on the GPU by its own
 * forward/backward/Adam kernels on error vectors of the plain solver. */
typedef struct fem2d_pcg fem2d_pcg;
int fem2d_patchnet_create(int k, int hidden, uint64_t seed, fem2d_patchnet** out);
void fem2d_patchnet_free(fem2d_patchnet* p);
int64_t fem2d_patchnet_num_params(const fem2d_patchnet* p);
/* parameters as floats: W1 (16 x hidden), b1, W2 (hidden x hidden), b2, W3 (hidden x k), b3; row-major */
int fem2d_patchnet_get_params(const fem2d_patchnet* p, float* out);
int fem2d_patchnet_set_params(fem2d_patchnet* p, const float* in);
/* the network's inputs on a Domain (host only): sizes[2] = {patches, rows}; per patch the row range
 * (patch_ptr, patches + 1), per row its DoF, 16 features and its partition-of-unity weight */
int fem2d_patchnet_features(const fem2d_domain* d, double shift, int64_t* sizes, int64_t* patch_ptr, int32_t* dof,
                            float* feat, float* weight);
/* mean projection loss over Elems and the S error samples (S vectors of ndofs doubles, one after
 * another, S <= 256) and its gradient with respect to the parameters (grad may be NULL) */
int fem2d_patchnet_loss_grad(fem2d_ctx* c, const fem2d_patchnet* p, const fem2d_gep* g, double shift,
                             const double* samples, int S, double* loss, float* grad);
/* Adam (beta 0.9/0.999) over `count` GEPs, each with S samples; loss_history[epochs] (may be NULL) */
int fem2d_patchnet_train(fem2d_ctx* c, fem2d_patchnet* p, const fem2d_gep* const* geps, int count, double shift,
                         const double* const* samples, int S, int epochs, double lr, double* loss_history);
int fem2d_pcg_create(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, const fem2d_patchnet* net,
                     fem2d_pcg** out);
/* x = K^-1 rhs (ndofs x nrhs row-major, host); every column to ||r|| <= tol ||b||. stats (may be NULL,
 * 5 doubles): iterations, worst relative residual, solve ms, set-up ms, coarse dimension.
 * FEM2D_E_NOT_CONVERGED if max_iter is reached first (x holds the last iterate). */
int fem2d_pcg_solve(fem2d_pcg* p, int nrhs, const double* rhs, double* x, double tol, int max_iter, double* stats);
/* the solver's training data: runs PCG on rhs and records, every `every` iterations from iteration
 * `first` on, the error xstar - x_i of each unconverged column (xstar: exact solutions, ndofs x nrhs
 * row-major), at most max_samples vectors of ndofs doubles into samples; *nsamples = the number */
int fem2d_pcg_harvest(fem2d_pcg* p, int nrhs, const double* rhs, const double* xstar, double tol, int max_iter,
                      int first, int every, int max_samples, double* samples, int* nsamples);
/* the two-level solver with a caller-given coarse basis instead of the network's: k vectors per Elem,
 * basis[rows x k] with rows in fem2d_patchnet_features order (a deflation basis of the caller's own) */
int fem2d_pcg_create_with_basis(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, int k, const float* basis,
                                fem2d_pcg** out);
void fem2d_pcg_free(fem2d_pcg* p);

#ifdef __cplusplus
}
#endif
#endif
