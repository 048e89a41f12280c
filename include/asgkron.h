/*
 * asgkron -- GB300 (sm_103a) operator application y = A*f for the sparse-grid DG prototype
 * of project-asgard/DG-SparseGrid (MATLAB).  Plain C ABI: caller-owned buffers, integer
 * status codes, no CUDA or framework types in the signatures (streams are void*).
 *
 * Each entry point names the reference function whose behaviour it replaces
 * (file:line within the reference project).
 *
 * Conventions
 *   - Element blocks are deg^d contiguous values, dimension 1 slowest and dimension d
 *     fastest (krond.m:17, combine_dimensions_D.m:40-51); element e occupies
 *     [e*deg^d, (e+1)*deg^d) of f and y (apply_A.m:116).
 *   - 1-D operators are dense column-major (n x n) matrices with leading dimension ld,
 *     rows in the hierarchical 1-D order of OperatorTwoScale_wavelet2.m:127-144; the rows
 *     of element e in dimension k are (idx1d[e][k]-base)*deg + (0..deg-1) (apply_A.m:119-122).
 *   - Index arrays carry an explicit base (0 for C callers, 1 for MATLAB/MEX callers).
 *   - Device-pointer entry points run asynchronously on the given stream (NULL = the
 *     legacy default stream); host-pointer entry points are synchronous.
 */
#ifndef ASGKRON_H
#define ASGKRON_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int asg_status;
enum {
  ASG_OK = 0,
  ASG_ERR_INVALID = 1,      /* bad argument, size or index (the reference's error(sprintf(...))) */
  ASG_ERR_UNSUPPORTED = 2,  /* valid but outside what the kernels handle (e.g. d > 6) */
  ASG_ERR_CUDA = 3,         /* a CUDA runtime call failed; asg_last_error has the text */
  ASG_ERR_NOMEM = 4,        /* host or device allocation failed */
  ASG_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
  ASG_ERR_CAPACITY = 6      /* caller buffer too small; the needed size is reported */
};

/* Structure handling of the 1-D operators (the work model the kernels execute). */
enum {
  ASG_STRUCT_NONE = 0,   /* reference work model: every listed pair x every term, full
                            d-mode Kronecker chain (apply_A.m:124-201) */
  ASG_STRUCT_DETECT = 1  /* skip (pair, term) products with a zero factor block and apply
                            identity factors as copies; |entry| <= drop_tol * max|op| counts
                            as zero (drop_tol = 0: exact zeros/identities only) */
};

enum { ASG_GRID_SG = 0, ASG_GRID_FG = 1 };

typedef struct asg_plan asg_plan;

typedef struct {
  int num_dims;                /* d, 1..6 (kron_multd.m:30-42) */
  int deg;                     /* p, 1..8, deg^d <= 4096 */
  int num_terms;               /* T, 1..16: the terms with pde.terms{t}.imex == imex_flag */
  int num_elems;               /* N = numel(A_data.element_global_row_index) */
  int index_base;              /* 0 or 1 for idx1d and cols */
  const int* idx1d;            /* [num_elems*num_dims]: A_data.element_local_index_D{k}(e) at [e*d+k] */
  const long long* row_ptr;    /* [num_elems+1] CSR of the pair list, or NULL = all pairs
                                  (opts.use_connectivity=false, apply_A.m:104-108) */
  const int* cols;             /* [row_ptr[N]] connected column elements (pde.connectivity{e}) */
  const double* const* ops;    /* [num_terms*num_dims]: pde.terms{t}.terms_1D{k}.mat at [t*d+k] */
  const int* op_ld;            /* [num_terms*num_dims] leading dimension (rows) of each operator */
  int structure;               /* ASG_STRUCT_* */
  double drop_tol;             /* see ASG_STRUCT_DETECT */
} asg_plan_desc;

typedef struct {
  long long num_pairs;         /* listed (row, col) pairs */
  long long num_entries;       /* (row, col, term) products the kernels execute */
  long long dof;               /* output values: num_elems * deg^d (a row slice: its rows') */
  double flops_reference;      /* num_pairs * T * d * 2 * deg^(d+1): the reference's work */
  double flops_executed;       /* flops of the executed work model */
  long long op_bytes_f64;      /* packed operator bytes on the device (FP64 copy) */
  int kernel_kind;             /* 0 warp chain, 1 CTA chain, 2-6 single-mode fiber kernels,
                                  7 streaming single-mode kernel, 8 kind 3 with two tiles
                                  per thread */
  int active_modes_max;        /* max over terms of non-identity factors */
} asg_plan_stats;

/* Library version string and last error text (per thread). */
const char* asg_version(void);
asg_status asg_last_error(char* buf, size_t len);

/* ---------------------------------------------------------------------------------------
 * apply_A (apply_A.m:1-252): plan once per operator set, apply many times.
 * ------------------------------------------------------------------------------------- */
/* Validates every index (the isok checks of kron_multd.m:7-12,24-28 and the asserts of
 * apply_A.m), analyses structure, builds the work list and uploads FP64 + FP32 operator
 * blocks.  Replaces the per-call setup inside apply_A.m:102-168. */
asg_status asg_plan_create(const asg_plan_desc* desc, asg_plan** plan);
asg_status asg_plan_destroy(asg_plan* plan);
asg_status asg_plan_stats_get(const asg_plan* plan, asg_plan_stats* stats);
/* Bit k of masks[t] is set when the plan applies operator (t, k); clear bits are factors the
 * structure analysis found to be the identity (always all set under ASG_STRUCT_NONE). */
asg_status asg_plan_active(const asg_plan* plan, unsigned* masks);
/* Re-upload operator values with the same sparsity class (time-dependent terms rebuilt by
 * get_coeff_mats.m with TD=1); the structure analysis is not redone. */
asg_status asg_plan_update_ops(asg_plan* plan, const double* const* ops, const int* op_ld);

/* Extended creation.  asg_plan_create(desc) is asg_plan_create_ex(desc, NULL). */
typedef struct {
  /* Output rows [row_begin, row_end) of the table (0 and num_elems: the whole table).  A
   * narrower range makes a row-slice plan (no reference counterpart: the prototype applies on
   * one node; a slice is one process's share when y = A f is split by output element): its
   * output y holds (row_end - row_begin) blocks in row order, and its input f holds those
   * rows' blocks followed by the halo blocks -- every other element the rows' work entries
   * read after structure detection, in table order (asg_plan_halo lists them).  A row-slice
   * plan runs the forward apply (device and host pointers) and the tuner; the adjoint,
   * gradients, steppers, batches, assembly and asg_plan_update_elements return
   * ASG_ERR_UNSUPPORTED for it. */
  int row_begin, row_end;
  /* NULL, or [num_dims]: pack at least op_blocks[k] deg x deg blocks per side of every operator
   * on dimension k, however high the table's 1-D indices reach, so that a later
   * asg_plan_update_elements can take tables with 1-D indices up to op_blocks[k] (base as the
   * table's).  The operators must hold op_blocks[k]*deg rows and columns. */
  const int* op_blocks;
} asg_plan_ext;
asg_status asg_plan_create_ex(const asg_plan_desc* desc, const asg_plan_ext* ext, asg_plan** plan);
/* Work entries (column, term products) of each output row, counts[num rows]: the cost to
 * balance when rows are split across processes (no reference counterpart). */
asg_status asg_plan_row_entries(const asg_plan* plan, long long* counts);
/* The halo of a row-slice plan: the table ids (in the creation's index base) of the input
 * elements after the rows, in the order f holds them; capacity 0 queries the count.  A
 * whole-table plan has none. */
asg_status asg_plan_halo(const asg_plan* plan, int* elems, long long capacity, long long* count);
/* A new element table and pair list (num_elems, idx1d, row_ptr, cols as in asg_plan_desc, same
 * index base) on the plan's operators, for the rebuild adapt.m:414-437 triggers after
 * coarsening or refinement when the operators keep their values (operators built at the
 * maximum level: single partial terms).  The operators' structure classes, packed blocks and
 * device copies are kept; the work list, the launch data and everything derived from the
 * table (transpose, gradient targets, the fused solve's partition, the tuner's choice) are
 * rebuilt or dropped.  ASG_ERR_CAPACITY when a 1-D index lies beyond the packed operator
 * extent (create the plan with asg_plan_ext.op_blocks to reserve it); after an argument error
 * the plan is unchanged.  Operators that change with the table (rechained LDG terms,
 * get_coeff_mats_rechain.m) need asg_plan_update_ops afterwards, or a new plan. */
asg_status asg_plan_update_elements(asg_plan* plan, int num_elems, const int* idx1d, const long long* row_ptr,
                                    const int* cols);

/* Force a kernel family for this plan: 0 warp chain (deg^d <= 256), 1 CTA chain,
 * 2 single-mode fiber kernel with direct loads, 3 single-mode fiber kernel with TMA bulk
 * copies (4 stages, 2 CTAs per SM), 4 the same with 3 stages, the FP32 compensation tile in
 * shared memory and 3 CTAs per SM, 5 the kind-3 pipeline in persistent CTAs that each walk
 * a balanced list of rows, 6 the small-block single-mode kernel (deg^d <= 256; grouped lanes
 * per row, no shared-memory staging), 7 the streaming kernel: FP32 in one persistent CTA per
 * SM walking a balanced stream of rows, each row's own block resident; FP64 runs kind 3,
 * 8 kind 3 in FP32 with two output tiles per consumer thread (4 consumer warps; results
 * bitwise those of kind 3); FP64 runs kind 3
 * (2-8 need one non-identity factor per term; 3-5, 7 and 8 need deg 4, d 6).
 * The default is chosen by asg_plan_create; this exists for testing one family against
 * another and for launch-shape tuning. */
asg_status asg_plan_set_kernel(asg_plan* plan, int kind);
/* Autotuner (no reference counterpart): times every kernel family asg_plan_set_kernel accepts
 * for this plan -- they differ in tile mapping, stages, CTAs per SM and rows per CTA -- on the
 * plan's own shape in one precision (0 FP64, 1 FP32), 2 warm-up and 10 timed launches each
 * on scratch vectors it allocates, and keeps the fastest for that precision (the plan's
 * applies in that precision use it from then on; asg_plan_set_kernel clears the choice).
 * Outputs (each may be NULL): the chosen kind, its time and the time of the kind used before,
 * in ms per launch.  Synchronous. */
asg_status asg_plan_tune(asg_plan* plan, int precision, void* stream, int* best_kind, float* best_ms,
                         float* default_ms);
/* The kernel family applies in this precision (0 FP64, 1 FP32) run. */
asg_status asg_plan_kernel_for(const asg_plan* plan, int precision, int* kind);
/* Synchronises and reads the plan's device status word: ASG_OK, or ASG_ERR_TIMEOUT when a
 * kernel's bounded shared-memory pipeline wait gave up (the y it wrote is then undefined).
 * The word is cleared after reading.  No reference counterpart: device-side waits are new. */
asg_status asg_plan_device_status(asg_plan* plan, int* status);

/* ftmp = A*f on device pointers (apply_A.m:185-201). FP64, or FP32 with Kahan-compensated
 * accumulation across the column reduction. */
asg_status asg_apply_f64(asg_plan* plan, const double* d_f, double* d_y, void* stream);
asg_status asg_apply_f32(asg_plan* plan, const float* d_f, float* d_y, void* stream);
/* Residual: r = A*f - ystar (device pointers, ystar laid out like y; the three buffers
 * distinct).  Bitwise the apply followed by an elementwise subtraction in the same
 * precision; one launch for the single-mode deg-3/4 kernels (subtracted as y is stored),
 * two for the others.  The first step of the gradient of L = 1/2 ||A f - ystar||^2 (r is then
 * the cotangent of asg_apply_T_* and asg_grad_ops_*).  No reference counterpart. */
asg_status asg_apply_residual_f64(asg_plan* plan, const double* d_f, const double* d_ystar, double* d_r,
                                  void* stream);
asg_status asg_apply_residual_f32(asg_plan* plan, const float* d_f, const float* d_ystar, float* d_r,
                                  void* stream);
/* Adjoint: fbar = A^T * ybar (device pointers).  No reference counterpart (the prototype has
 * no adjoint); built from the transposed operator blocks and the transposed work list. */
asg_status asg_apply_T_f64(asg_plan* plan, const double* d_ybar, double* d_fbar, void* stream);
asg_status asg_apply_T_f32(asg_plan* plan, const float* d_ybar, float* d_fbar, void* stream);
/* Gradient of a scalar L with cotangent r = dL/dy (y = A f) with respect to every applied
 * 1-D operator (t, k), including its zero blocks (the derivative there is generally nonzero):
 * every block some listed pair reaches is written (not added)
 * into G[t*d+k] (device, column-major, leading dimension ldg[t*d+k]); all other entries of G
 * are left as they are, so zero G first for the full gradient.  G[t*d+k] may be NULL to skip;
 * identity factors detected by ASG_STRUCT_DETECT are not differentiated.  G and ldg are host
 * arrays.  Deterministic (fixed-order sums, no atomics).  No reference counterpart. */
asg_status asg_grad_ops_f64(asg_plan* plan, const double* d_f, const double* d_r, double* const* G,
                            const int* ldg, void* stream);
asg_status asg_grad_ops_f32(asg_plan* plan, const float* d_f, const float* d_r, float* const* G,
                            const int* ldg, void* stream);
/* Same on host pointers: copies f in, applies, copies y out, synchronises (the call a
 * MATLAB MEX gateway makes). */
asg_status asg_apply_host_f64(asg_plan* plan, const double* h_f, double* h_y);
asg_status asg_apply_host_f32(asg_plan* plan, const float* h_f, float* h_y);
/* The adjoint and the operator gradients on host pointers (synchronous; the calls the adjoint
 * MEX gateway makes).  h_G[t*d+k] are host column-major matrices with leading dimension
 * ldg[t*d+k]; as in asg_grad_ops_f64, reached blocks are overwritten and the rest of each
 * matrix is left as it was.  No reference counterpart (the prototype has no adjoint). */
asg_status asg_apply_T_host_f64(asg_plan* plan, const double* h_ybar, double* h_fbar);
asg_status asg_grad_ops_host_f64(asg_plan* plan, const double* h_f, const double* h_r, double* const* h_G,
                                 const int* ldg);

/* The operator as block-sparse rows (apply_A.m:170-180,246-248, opts.build_A: A(I,J) +=
 * krond(...) over the terms).  Block (i, j) is deg^d x deg^d, the sum over the plan's terms of
 * kron_k A_{t,k}[I_k(i), J_k(j)] (identity factors exact, products with a structurally zero
 * factor block left out under ASG_STRUCT_DETECT): the matrix the kernels apply.  Writes the
 * block count to *num_blocks and, when not NULL, the structure to host row_ptr[N+1] and
 * cols[num_blocks] (0-based, columns ascending in each row); d_blocks == NULL stops there.
 * Otherwise d_blocks (device, capacity blocks) receives each block row-major, FP64.
 * deg^d <= 256.  Synchronous. */
asg_status asg_assemble_bsr_f64(asg_plan* plan, long long* row_ptr, int* cols, double* d_blocks, long long capacity,
                                long long* num_blocks, void* stream);

/* Measurement kernels (no reference counterpart): what the roofline of the apply is taken
 * against.  asg_probe_gather_f32 streams every work entry's column block of the plan from
 * global memory into shared memory with the apply's bulk copies (one CTA per row, `stages`
 * = 2, 4 or 8 blocks in flight, no arithmetic; one value per block summed into d_out[row],
 * N floats): time it to get the L2-to-SM rate of the plan's own gather pattern.
 * asg_probe_fma runs `blocks` x 256 threads of 8 independent FMA chains for `iters` rounds,
 * precision 1 the FP32 paired FMA (fma.rn.f32x2), 0 FP64 (d_out: one value of that type),
 * and reports the flops it executes: time it for the FP32 / FP64 issue peaks.  Both
 * asynchronous on `stream`. */
asg_status asg_probe_gather_f32(asg_plan* plan, const float* d_f, float* d_out, int stages, void* stream);
asg_status asg_probe_fma(int precision, int blocks, int iters, void* d_out, double* flops, void* stream);

/* ---------------------------------------------------------------------------------------
 * Element tables and index maps (hash_table_sparse_nD.m, global_matrix.m, connect_nD.m)
 * ------------------------------------------------------------------------------------- */
/* Element table in hash_table_sparse_nD.m order (hash_table_sparse_nD.m:35-116): level
 * tuples with sum <= max(lev_vec) walked from the largest sum down (perm_leq_d.m:26-45),
 * cells with dimension 1 fastest (lev_cell_to_1D_index_set.m:10-30).  grid ASG_GRID_FG
 * uses perm_max.m.  Outputs [count*d] levels and cells, and the 0-based md keys
 * (md_lev_pos_to_idx.m:10-26 minus one).  Pass capacity 0 to query count. */
asg_status asg_hash_table_sparse_nd(int num_dims, const int* lev_vec, int max_lev, int grid,
                                    int* levels, int* cells, unsigned long long* keys,
                                    long long capacity, long long* count);
/* Old-hash order of hash_table_nD.m:29-136 (perm_leq.m / perm_max.m), used with connectivity. */
asg_status asg_hash_table_nd(int num_dims, int lev, int grid, int* levels, int* cells,
                             long long capacity, long long* count);
/* 1-based 1-D index 2^(lev-1)+cell+1 (1 at level 0) per element and dimension
 * (lev_cell_to_1D_index.m:6-9, global_matrix.m:31-70). */
asg_status asg_element_idx1d(int num_dims, long long num_elems, const int* levels, const int* cells,
                             int* idx1d);
/* Per-element sorted connected element lists (connect_nD.m:34-105, connect_1D.m:8-50) as
 * CSR with 0-based columns. grid ASG_GRID_SG uses index_leq_max.m, ASG_GRID_FG index_max.m.
 * Pass capacity 0 to query the number of pairs. */
asg_status asg_connect_nd(int num_dims, long long num_elems, const int* levels, const int* cells,
                          int levsum, int levmax, int grid, long long* row_ptr, int* cols,
                          long long capacity, long long* num_pairs);

/* ---------------------------------------------------------------------------------------
 * Producer of the path's inputs on the host: wavelet-space 1-D DG operators
 * ------------------------------------------------------------------------------------- */
/* n-point Gauss-Legendre rule on [a, b], nodes ascending (Quadrature/lgwt.m). */
asg_status asg_gauss_legendre_f64(int n, double a, double b, double* x, double* w);
/* Two-scale filters H0, G0 (deg x deg, row-major) of the Alpert multiwavelets
 * (two_scale/MultiwaveletGen.m; entries below 1e-5 zeroed). */
asg_status asg_multiwavelet_filters_f64(int deg, double* H0, double* G0);
/* Forward multiwavelet transform F (n x n, n = deg 2^lev <= 16384, row-major): rows are the
 * level-0 scaling functions, then the wavelets level by level, cells left to right
 * (OperatorTwoScale_wavelet2.m:127-144). */
asg_status asg_fmwt_matrix_f64(int deg, int lev, double* F);
/* One partial term of a 1-D operator (PARTIAL_SD_TERM.m with MASS.m / DIV.m / GRAD.m). */
typedef struct asg_partial_term {
  int kind;              /* 0 mass, 1 div, 2 grad */
  double LF;             /* flux parameter as given to DIV / GRAD (GRAD negates it) */
  char bcl, bcr;         /* 'P', 'D' or 'N' as given (GRAD swaps D and N) */
  const double* g_quad;  /* [2^lev][nq] coefficient g at each cell's Gauss nodes, cells
                          * left to right, nq = max(deg + 1, 10) nodes of
                          * asg_gauss_legendre_f64(nq, -1, 1) mapped to the cell; NULL = 1 */
  const double* g_face;  /* [2^lev + 1] g at the cell faces lo + c h; NULL = 1 */
} asg_partial_term;
/* pde.terms{t}.terms_1D{d}.mat: the chain (M \ L_1)(M \ L_2)... of partial terms with the
 * unit LHS mass, in wavelet space (n x n row-major; coeff_matrix.m:105-342,
 * pterm_coeff_matrix.m:6-20, sd_term_coeff_matrix.m:9-22).  Chained in realspace and rotated
 * once by F: equal to rotating each factor to the transform's orthogonality round-off. */
asg_status asg_coeff_matrix_f64(int deg, int lev, double lo, double hi, int nterms, const asg_partial_term* terms,
                                double* out);

/* ---------------------------------------------------------------------------------------
 * Many independent problems in one persistent launch (no reference counterpart: the
 * prototype applies one operator at a time)
 * ------------------------------------------------------------------------------------- */
typedef struct asg_batch asg_batch;
/* A batch over existing plans (deg <= 4, deg^d <= 256); the plans must outlive it.  The packed
 * work list holds (problem, row block) items, most expensive first. */
asg_status asg_batch_create(asg_plan* const* plans, int count, asg_batch** batch);
asg_status asg_batch_destroy(asg_batch* batch);
/* Device input/output vectors of every problem (host arrays of device pointers). */
asg_status asg_batch_set_io_f64(asg_batch* batch, const double* const* d_f, double* const* d_y);
asg_status asg_batch_set_io_f32(asg_batch* batch, const float* const* d_f, float* const* d_y);
/* Uploads the problem table for a precision (0 FP64, 1 FP32); call after set_io and before
 * apply / graph capture. */
asg_status asg_batch_prepare(asg_batch* batch, int precision);
/* y_k = A_k f_k for every problem: one counter reset and one persistent launch (capturable). */
asg_status asg_batch_apply(asg_batch* batch, int precision, void* stream);
/* Times (warps per CTA, rows per work item) candidates and keeps the fastest. */
asg_status asg_batch_tune(asg_batch* batch, int precision, void* stream, float* best_ms);
/* Sets the launch shape instead of tuning: warps per CTA (4 or 8) and rows per work item (1,
 * 2 or 4; a warp computes up to that many rows of a problem side by side when the problem's
 * blocks are small).  Results do not depend on the shape. */
asg_status asg_batch_configure(asg_batch* batch, int warps_per_cta, int rows_per_item);
asg_status asg_batch_info(const asg_batch* batch, int* warps_per_cta, int* rows_per_item, double* flops);

/* ---------------------------------------------------------------------------------------
 * Time steppers on the operator application (time_advance.m)
 * ------------------------------------------------------------------------------------- */
/* One RK3 step f <- f + dt (k1/6 + 2 k2/3 + k3/6), k_s = A y_s + src_s (RungeKutta3,
 * time_advance.m:151-204, without LHS mass or boundary vectors).  d_src: host array of the
 * three device source vectors at t, t+dt/2, t+dt (NULL array or entries = zero sources).
 * d_work: 16-byte aligned device workspace of 4 * round_up(dof, 16 / sizeof(value)) values
 * (four vectors, each on a 16-byte boundary).  Asynchronous, allocation-free, capturable into
 * a CUDA graph.  For plans applied by the small-block kernel the step is one cooperative
 * launch (three applies separated by grid barriers), otherwise three applies and three
 * stage updates; the results are the same. */
asg_status asg_rk3_step_f64(asg_plan* plan, double* d_f, double dt, const double* const* d_src, double* d_work,
                            size_t work_bytes, void* stream);
asg_status asg_rk3_step_f32(asg_plan* plan, float* d_f, double dt, const float* const* d_src, float* d_work,
                            size_t work_bytes, void* stream);
/* The same step with the stage sources formed inside it: source_k = sum_q d_coef[k*ns + q] *
 * d_vecs[q] for the stage times k = 0, 1, 2 (t, t+dt/2, t+dt) -- the separable sources of
 * source_vector.m, spatial parts times time factors -- summed in FP64 as asg_lincomb_f64 does
 * and rounded once to the step's type.  d_coef (3*ns values) and d_vecs (ns device pointers to
 * FP64 vectors) live on the device, so a captured step reads new time factors on replay.
 * Equal to asg_lincomb_f64 per stage followed by asg_rk3_step_*; for plans applied by the
 * small-block kernel the whole step is one cooperative launch. */
asg_status asg_rk3_step_sources_f64(asg_plan* plan, double* d_f, double dt, int ns, const double* d_coef,
                                    const double* const* d_vecs, double* d_work, size_t work_bytes, void* stream);
asg_status asg_rk3_step_sources_f32(asg_plan* plan, float* d_f, double dt, int ns, const double* d_coef,
                                    const double* const* d_vecs, float* d_work, size_t work_bytes, void* stream);
/* d_out = sum_s d_coef[s] * d_vecs[s] (the separable sources of source_vector.m: spatial parts
 * times time factors); d_coef and d_vecs (an array of device pointers) live on the device. */
asg_status asg_lincomb_f64(long long n, int ns, const double* d_coef, const double* const* d_vecs, double* d_out,
                           void* stream);

/* Precision of the GMRES cycles inside iterative refinement (asg_gmres_opts.mixed).  The outer
 * residual b - (I - dt A) x, its norm and x are FP64 in every mode. */
enum {
  ASG_GMRES_FP64 = 0,        /* everything FP64 */
  ASG_GMRES_FP32_INNER = 1,  /* the whole inner cycle in FP32: operator, basis, dot products,
                                norms, Givens rotations and R y = g */
  ASG_GMRES_FP32_MATVEC = 2  /* only the operator application in FP32; the basis, the Arnoldi
                                dot products and norms, the Givens rotations and the solution
                                update in FP64 */
};
typedef struct {
  int restart;             /* GMRES(m) Krylov dimension per cycle, 1..64 */
  int max_outer;           /* refinement steps (each one GMRES cycle on the FP64 residual) */
  double tol;              /* stop when ||b - (I - dt A) x|| <= tol * ||b|| */
  double inner_reduction;  /* each cycle stops once its residual drops by this factor */
  int mixed;               /* ASG_GMRES_* */
} asg_gmres_opts;
typedef struct {
  int outer_iters;
  int inner_iters;
  int converged;
  double rel_residual;     /* final FP64 ||b - (I - dt A) x|| / ||b|| */
} asg_gmres_info;
/* Backward Euler solve (I - dt A) x = b (backward_euler, time_advance.m:267-349, which
 * assembles A and uses a direct solve): matrix-free GMRES(m) inside iterative refinement.
 * The outer residual b - (I - dt A) x, its norm and x are FP64; each GMRES cycle runs in the
 * precision opts->mixed selects (ASG_GMRES_*).  Plans on the small-block kernel with
 * deg 2..4 run the whole solve as one cooperative launch (one synchronisation); other plans
 * run it kernel by kernel.  d_x holds the initial guess on entry; d_b and d_x 16-byte
 * aligned.  ASG_ERR_TIMEOUT: a bounded grid-barrier wait of the one-launch solve gave up. */
asg_status asg_be_workspace(const asg_plan* plan, const asg_gmres_opts* opts, size_t* bytes);
asg_status asg_be_solve(asg_plan* plan, double dt, const double* d_b, double* d_x, const asg_gmres_opts* opts,
                        asg_gmres_info* info, void* d_work, size_t work_bytes, void* stream);
/* Test hook (no reference counterpart): in the next one-launch backward-Euler solve of this
 * process, CTA 0 withholds its arrival at grid barrier number `barrier` (0-based, counted
 * from the launch), so every CTA's bounded wait (~2^31 cycles) runs out and the solve returns
 * ASG_ERR_TIMEOUT with the context intact.  -1 clears it. */
asg_status asg_debug_withhold_arrival(int barrier);

/* ---------------------------------------------------------------------------------------
 * Kronecker products and batched small GEMMs (Kronmult/)
 * All matrices are column-major; pointer arguments are device pointers unless stated.
 * ------------------------------------------------------------------------------------- */
/* C_i = alpha*op(A_i)*op(B_i) + beta*C_i for a batch of independent small GEMMs with their own
 * sizes (Kronmult/gemm_vbatched.m:1-44, the MAGMA magmablas_dgemm_vbatched convention: every
 * array -- sizes, leading dimensions and the pointer arrays -- lives in device memory; one
 * transA/transB/alpha/beta for the whole batch).  k is read from k[] (the reference reads
 * nlist at gemm_vbatched.m:25; that is a bug, not reproduced here). */
asg_status asg_gemm_vbatched_f64(char trans_a, char trans_b, const int* m, const int* n, const int* k, double alpha,
                                 const double* const* A, const int* lda, const double* const* B, const int* ldb,
                                 double beta, double* const* C, const int* ldc, int batch, void* stream);
asg_status asg_gemm_vbatched_f32(char trans_a, char trans_b, const int* m, const int* n, const int* k, float alpha,
                                 const float* const* A, const int* lda, const float* const* B, const int* ldb,
                                 float beta, float* const* C, const int* ldc, int batch, void* stream);

/* One recorded GEMM of the kronmultN_batch lists (the fields of batch_list{level} entries,
 * Kronmult/kronmult2_batch.m:86-110).  Operands: 0..nkron-1 the factors A1..An, nkron = X,
 * nkron+1 = Y, nkron+2 = the workspace (the recursion's temporaries); offsets are element
 * offsets into them. */
typedef struct {
  int level;                   /* 1-based batch list the reference appends to */
  int m, n, k;
  char trans_a, trans_b;
  double alpha, beta;          /* always 1 and 0 in the reference */
  int a_operand, b_operand, c_operand;
  long long a_offset, b_offset, c_offset;
  int lda, ldb, ldc;
} asg_gemm_desc;

typedef struct asg_kron_plan asg_kron_plan;
/* Plans Y = kron(A1,...,An) * X for X with nvec columns the way kronmultN_batch.m does
 * (Kronmult/kronmult{1..6}_batch.m, method chosen per level by flops_kron{n}.m): the GEMMs
 * go into per-level lists executed level by level, each level one batched launch.  Planning
 * is host-only; the descriptor table moves to the device on the first execution. */
asg_status asg_kron_plan_create(int nkron, const int* nrow, const int* ncol, long long nvec, asg_kron_plan** plan);
asg_status asg_kron_plan_destroy(asg_kron_plan* plan);
/* Workspace (the recursion's Ytmp buffers) the executor needs, per precision. */
asg_status asg_kron_plan_workspace(const asg_kron_plan* plan, size_t* bytes_f64, size_t* bytes_f32);
/* The recorded batch lists (host memory), level by level; capacity 0 queries the count. */
asg_status asg_kron_plan_lists(const asg_kron_plan* plan, asg_gemm_desc* out, int capacity, int* count);
/* Y = kron(A1..An) * X (kron_multd.m / kronmultN.m results, kronmultN_batch.m execution).
 * A: host array of nkron device pointers; X, Y, work: device; work_bytes >= the workspace. */
asg_status asg_kron_batch_f64(const asg_kron_plan* plan, const double* const* A, const double* X, double* Y,
                              void* work, size_t work_bytes, void* stream);
asg_status asg_kron_batch_f32(const asg_kron_plan* plan, const float* const* A, const float* X, float* Y,
                              void* work, size_t work_bytes, void* stream);
/* Size of the fixed device array asg_kron_batch_static_f64 keeps its temporaries in. */
#define ASG_KRON_STATIC_SCRATCH_BYTES (8ull << 20)
/* asg_kron_batch_f64 without any allocation (no counterpart in the reference, whose
 * kronmultN_batch.m grows its temporaries at run time).  For callers that cannot call
 * cudaMalloc when they execute -- allocation forbidden or unsafe at that point, or no
 * allocator to hand: the recursion's temporaries live in one fixed device array of
 * ASG_KRON_STATIC_SCRATCH_BYTES (8 MiB) inside the library and the plan's GEMM descriptors
 * ride in the launch parameters.  Plans whose workspace (asg_kron_plan_workspace) exceeds
 * the array are rejected with ASG_ERR_CAPACITY.  The first call on each device, made with
 * that device current, looks the array up; make it before any stream capture.  All calls on
 * a device share the array, which keeps the last call's values (nothing in it needs to
 * start at zero: every temporary is written before it is read); calls that overlap on the
 * GPU race on it, so order them (one stream, or events).  A: host array of nkron device
 * pointers; X, Y: device. */
asg_status asg_kron_batch_static_f64(const asg_kron_plan* plan, const double* const* A, const double* X, double* Y,
                                     void* stream);
/* out = kron(A1, kron(A2, ...)) (krond.m:7-17), column-major prod(nrow) x prod(ncol).
 * A: host array of nkron device pointers (each nrow_i x ncol_i, ld = nrow_i). */
asg_status asg_krond_f64(int nkron, const int* nrow, const int* ncol, const double* const* A, double* out,
                         void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ASGKRON_H */
