/*
 * bilu.h -- C ABI of the GB300-native batched preconditioned BiCGSTAB library.
 *
 * Batches of small sparse systems A_s x_s = b_s (s = 0..nsys-1) that share one
 * CSR sparsity pattern ("pages" in the original code: values are stored
 * system-major, values[s*nnz + k], vectors [s*n + i]) are factorised and solved
 * on one GPU.  Every pointer named d_* is a device pointer; every pointer
 * named h_* is a host pointer.  All device work is ordered on the stream that
 * is passed in (a cudaStream_t given as void*, NULL = legacy default stream);
 * no entry point synchronises the device unless its comment says so.
 *
 * Every entry point returns a bilu_status (BILU_OK = 0) instead of asserting;
 * bilu_last_error() gives a one-line description of the last failure on the
 * calling thread.
 *
 * Reference interfaces replaced (paths inside Batched-ILU0-merged/ILU0_ISAI_bicgstab/):
 *   PrecondBiCGSTAB.h:15-30   the five Batched_*_BiCGSTAB_Gpu solver entry points
 *   ILU_0.h:9                 ILU_0_Factorization_Gpu(A, L, U, approach)
 *   parILU_0.h:7              ParILU_0_Factorization_Gpu(A, L, U, sweeps)
 *   isai.h:9                  GenerateISAI_gpu(aiA, A, mat_type, power)
 *   factorization.h:10-29     missing-diagonal insertion, diagonal pointers, L/U split
 *   Bicgstab_common.hpp:294   KernelFillTrueResNorms (true residual norms)
 *   SolverResults.h:7-134     per-system iteration count / convergence flag / norms
 */
#ifndef BILU_H
#define BILU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
typedef int bilu_status;
#define BILU_OK              0
#define BILU_ERR_INVALID     1  /* bad argument (null pointer, negative size, bad option) */
#define BILU_ERR_PATTERN     2  /* CSR pattern unsorted / column out of range / missing diagonal where not allowed */
#define BILU_ERR_CAPACITY    3  /* a size is beyond what the kernels support (e.g. ISAI row > 32 entries) */
#define BILU_ERR_CUDA        4  /* a CUDA runtime call failed */
#define BILU_ERR_NO_DEVICE   5  /* no CUDA device / kernels not loadable */
#define BILU_ERR_ALLOC       6  /* device or host allocation failed */

/* Per-system outcome written to bilu_results.status (conv_flags keeps the
 * reference's 1 / -1 convention). */
#define BILU_SYS_CONVERGED        1  /* recursive residual below the threshold                 */
#define BILU_SYS_MAX_ITER        -1  /* iteration limit reached                                */
#define BILU_SYS_BREAKDOWN_RHO   -2  /* rho = (r, r_hat) became exactly 0 (reference "Method failed") */
#define BILU_SYS_NONFINITE       -3  /* a NaN / Inf appeared in the recurrences (zero pivot etc.) */
#define BILU_SYS_ZERO_RHS         2  /* b = 0, x = 0 returned without iterating                  */
#define BILU_SYS_INITIAL_OK       3  /* initial residual already below the threshold             */

/* ---------------------------------------------------------------- options */
/* Preconditioner families (reference solver it replaces in brackets). */
#define BILU_PRECOND_ILU0         0  /* ILU(0) factorised inside the solver kernel
                                        [Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_merged_Gpu]        */
#define BILU_PRECOND_ILU0_SPLIT   1  /* ILU(0) by a separate factorisation launch, then the solve
                                        [Batched_ILU_Preconditioned_BiCGSTAB_Gpu, is_parilu = 0;
                                         ..._segregated_Gpu when approach = 1]                              */
#define BILU_PRECOND_PARILU0      2  /* ParILU(0) sweeps, then the solve with triangular solves
                                        [Batched_ILU_Preconditioned_BiCGSTAB_Gpu, is_parilu = 1]           */
#define BILU_PRECOND_ILU0_ISAI    3  /* ILU(0) then ISAI of L and U, applied as two SpMVs
                                        [Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu, is_parilu = 0]      */
#define BILU_PRECOND_PARILU0_ISAI 4  /* ParILU(0) then ISAI of L and U
                                        [Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu, is_parilu = 1]      */
#define BILU_PRECOND_NONE         5  /* unpreconditioned BiCGSTAB (identity preconditioner)               */
#define BILU_PRECOND_GENERAL_ISAI 6  /* ISAI of A itself (pattern of |A|^isai_power, Gauss-Jordan row solves
                                        with partial pivoting), applied as one SpMV
                                        [Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu, power 1]       */

#define BILU_TOL_ABS   0  /* stop when ||r||_2 < tol            (reference: ATOL = 1e-11, PrecondBiCGSTAB.h:12) */
#define BILU_TOL_REL   1  /* stop when ||r||_2 < tol * ||b||_2                                                   */

#define BILU_FP64      0
#define BILU_FP32      1  /* factors / ISAI stored and applied in FP32; recurrences, inner products,
                             SpMV with A and the true residual stay FP64 */

#define BILU_REDUCE_REF   0  /* reference operation order: bit-identical to the reference kernels        */
#define BILU_REDUCE_FAST  1  /* throughput order: sequential row sums, reciprocal-multiply divisions     */

typedef struct bilu_options {
  int    precond;            /* BILU_PRECOND_*                                             */
  int    ilu_approach;       /* 1..4: arithmetic of the reference's ILU approach
                                (1 and 4: in-place right-looking updates, 2: dependency sum in
                                descending k, 3: dependency sum in ascending k).  All four are
                                executed by one deterministic level-scheduled kernel.          */
  int    parilu_sweeps;      /* ParILU(0) fixed-point sweeps (Jacobi schedule)              */
  int    isai_power;         /* ISAI pattern = pattern of |T|^power, T = L or U (reference: 2) */
  int    tol_mode;           /* BILU_TOL_ABS | BILU_TOL_REL                                 */
  double tol;                /* threshold (reference: 1e-11 absolute)                      */
  int    max_iter;           /* full BiCGSTAB iterations (reference MAX_ITER = 500)         */
  int    factor_precision;   /* BILU_FP64 | BILU_FP32                                       */
  int    reduction;          /* BILU_REDUCE_REF | BILU_REDUCE_FAST                          */
  int    compute_true_residual; /* nonzero: fill bilu_results.true_res_norms              */
  int    threads_per_system; /* 0 = automatic; otherwise CTA size used per system           */
  double parilu_res_tol;     /* > 0: ParILU sweeps stop once the ILU residual
                                ||(A - LU)|_S||_F / ||A||_F <= parilu_res_tol (at most
                                parilu_sweeps sweeps); 0: exactly parilu_sweeps sweeps     */
  int    isai_lower_diag;    /* bilu_isai only.  0: aiL is the ISAI of the unit lower factor
                                of ILU factors stored in place (diagonal implicit).  1: the
                                values at the diagonal positions belong to the lower
                                triangular matrix itself and aiL divides by them, as
                                GenerateISAI_gpu(lower_tri) (isai_gpu.cu:325-355) does for a
                                stand-alone lower triangular matrix.  Solves reject 1.     */
  int    smem_staging;       /* register-resident solver only: -1 automatic; else a bit mask
                                of the operands copied to shared memory once per system
                                (bit 0: A, bit 1: aiL / aiA, bit 2: aiU), the rest read
                                through L1.  Operands that do not fit are left out.
                                Bit 3: A and aiU left in global memory are read from
                                SELL-32 copies made before the solver launch (same
                                arithmetic; the copies live in the plan's workspace).
                                Bit 4: the kernel variant bounded for occupancy (same
                                arithmetic, fewer registers, more threads per SM): 8 rows
                                per thread on 4 CTAs of 128 threads per SM, 4 rows on 4
                                CTAs of 256 (3 with ILU factors), 2 rows on 2 CTAs of
                                512; ignored for ILU factors at 8 rows per thread.        */
} bilu_options;

/* Fills *opts with the reference defaults: merged ILU(0), approach 1, 5 sweeps,
 * ISAI power 2, absolute tolerance 1e-11, 500 iterations, FP64, reference order. */
void bilu_default_options(bilu_options* opts);

/* ---------------------------------------------------------------- results */
/* Device arrays of length nsys (any pointer may be NULL to skip that output).
 * Mirrors SolverResults (SolverResults.h:7-134). */
typedef struct bilu_results {
  float*  iter_counts;     /* iterations in steps of 0.5 (half iterations), as the reference */
  int*    conv_flags;      /* 1 converged, -1 not converged (reference convention)          */
  double* iter_res_norms;  /* recursive residual norm at exit                                 */
  double* true_res_norms;  /* ||b - A x||_2 computed after the solve                          */
  int*    status;          /* BILU_SYS_* detailed outcome                                     */
  int*    parilu_sweeps;   /* ParILU preconditioners: sweeps performed                        */
  double* ilu_residual;    /* ParILU preconditioners: ILU residual of the factors used       */
} bilu_results;

/* ---------------------------------------------------------------- plans */
/* A plan holds everything derived from one sparsity pattern (diagonal
 * positions, L/U split, level schedules, factorisation dependency lists,
 * ISAI patterns and extraction maps, shared-memory layout), uploaded once to
 * the current device.  Creating a plan synchronises with the device (uploads).
 * h_row_ptrs/h_col_idxs: host CSR pattern with n+1 / nnz entries, columns
 * sorted ascending within each row.  Missing diagonals are inserted (value 0),
 * as Add_Missing_Diagonal_Elements (factorization.cu:425) does, except for
 * BILU_PRECOND_ILU0 which, like the merged reference solver
 * (PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:555-560), rejects them. */
typedef struct bilu_plan bilu_plan;

bilu_status bilu_plan_create(bilu_plan** plan, int n, int nnz,
                             const int* h_row_ptrs, const int* h_col_idxs,
                             const bilu_options* opts);
bilu_status bilu_plan_destroy(bilu_plan* plan);

typedef struct bilu_plan_info {
  int n;                 /* rows                                                   */
  int nnz;               /* nonzeros after diagonal insertion (factor pattern)     */
  int nnz_in;            /* nonzeros of the input pattern                          */
  int missing_diag;      /* diagonals inserted                                     */
  int nnz_L, nnz_U;      /* reference L (strict lower + unit diagonal) / U nnz    */
  int nnz_isai_L, nnz_isai_U; /* ISAI patterns (0 when the preconditioner has none) */
  int levels_lower, levels_upper;   /* triangular-solve level counts             */
  int max_row_len;       /* longest row of the factor pattern                      */
  int threads;           /* CTA size used per system by the solver kernel          */
  int smem_bytes;        /* dynamic shared memory per system of the solver kernel  */
  int operands_in_smem;  /* bit 0: A, bit 1: factors / aiL, bit 2: aiU in shared memory;
                            bit 3: A, and aiU, left in global memory are read from SELL-32
                            copies made by one extra launch each per solve; bit 4: the
                            occupancy variant of the register-resident kernel */
  int solver_kernel;     /* 0: one CTA per system, vectors in shared memory (every mode);
                            1: register-resident (BILU_REDUCE_FAST with n <= 1024, or
                            the reference order with n <= 1024, ILU factors or none and
                            rows of at most 16 entries): `threads` threads per system,
                            each owning rows t + k * threads                         */
} bilu_plan_info;
bilu_status bilu_plan_get_info(const bilu_plan* plan, bilu_plan_info* info);

/* Host copy of a pattern held by the plan.  which: 0 = factor pattern (A with
 * diagonals), 1 = ISAI(L), 2 = ISAI(U), 3 = L (reference L_pages), 4 = U
 * (reference U_pages).  Pass NULL arrays to query the sizes only. */
bilu_status bilu_plan_get_pattern(const bilu_plan* plan, int which, int* n, int* nnz,
                                  int* h_row_ptrs, int* h_col_idxs);

/* Scatter input values (input pattern, nsys*nnz_in) into the factor pattern
 * (nsys*nnz, inserted diagonals = 0).  Equivalent of
 * update_col_idxs_and_values_diagonal_add (factorization.cu:169). */
bilu_status bilu_expand_values(const bilu_plan* plan, int nsys, const double* d_values_in,
                               double* d_values_out, void* stream);

/* ---------------------------------------------------------------- solver */
/* Solve A_s x_s = b_s for all systems with the plan's preconditioner.
 * d_values: nsys*nnz_in values of the INPUT pattern; d_b, d_x: nsys*n.
 * x0 = 0 (as the reference).  d_x is overwritten.  Replaces the five
 * Batched_*_Preconditioned_BiCGSTAB_Gpu entry points (PrecondBiCGSTAB.h:15-30). */
bilu_status bilu_solve(bilu_plan* plan, int nsys, const double* d_values,
                       const double* d_b, double* d_x, const bilu_results* results,
                       void* stream);

/* Same, with the ParILU sweeps started from d_lu_init (nsys*nnz in the factor
 * pattern, L strictly-lower part and U upper part stored in place) instead of
 * the A-value initialisation.  Only for BILU_PRECOND_PARILU0[_ISAI]. */
bilu_status bilu_solve_warm(bilu_plan* plan, int nsys, const double* d_values,
                            const double* d_lu_init, const double* d_b, double* d_x,
                            const bilu_results* results, void* stream);

/* Stage timing, the reference's PST / IST / OET (PrecondBiCGSTAB.h:15-30,
 * PrecondBiCGSTAB_ilu_gpu.cu:449-495), measured with CUDA events on the solve's
 * stream instead of host clocks around device synchronisations:
 * setup_ms = preconditioner generation launches, solve_ms = the BiCGSTAB
 * kernel, total_ms = both.  Enable once per plan; bilu_plan_last_timing waits
 * for the last solve's events. */
typedef struct bilu_timing {
  float setup_ms;
  float solve_ms;
  float total_ms;
} bilu_timing;
bilu_status bilu_plan_enable_timing(bilu_plan* plan, int enable);
bilu_status bilu_plan_last_timing(bilu_plan* plan, bilu_timing* timing);

/* Times the register-resident solver's configurations on this batch -- threads
 * per system 1x, 2x and 4x the fewest that give 8 rows per thread, shared-memory
 * staging of none / aiL / aiL + aiU / A, SELL-32 copies of the operands left in
 * global memory or not -- and keeps the fastest for the plan's
 * later solves.  Plans that do not use that solver (bilu_plan_info.solver_kernel
 * 0) are left unchanged.  Runs full solves of the batch (d_x is overwritten) and
 * synchronises.  No reference counterpart. */
bilu_status bilu_plan_autotune(bilu_plan* plan, int nsys, const double* d_values, const double* d_b,
                               double* d_x, void* stream);

/* bilu_solve without any device allocation.  No counterpart in the reference
 * (its solvers cudaMalloc and cudaFree their temporaries on every call).
 * For callers that cannot let a solve allocate: a simulation calling the
 * batched solver inside its time-step loop keeps a fixed device-memory
 * footprint set at start-up, and cudaMalloc / cudaFree would also
 * synchronise the device mid-step.  Same scratch layout, kernels and
 * bit-identical results as bilu_solve (the SELL-32 operand copies of the
 * plan's configuration included); the intermediates (factors, ISAI values,
 * operand copies) live in one fixed 32 MiB device array per GPU, reserved when
 * the library is loaded and held until exit.  Calls needing more scratch than
 * that are rejected with BILU_ERR_CAPACITY (split the batch).  All calls on a
 * device share the array: calls whose kernels overlap on the GPU race.  The
 * first call on a device does the set-up (looks up the array's device address,
 * loading the library's device module there if needed); make it before any
 * stream capture.  The plan must exist already (bilu_plan_create allocates
 * once). */
bilu_status bilu_solve_noalloc(bilu_plan* plan, int nsys, const double* d_values, const double* d_b,
                               double* d_x, const bilu_results* results, void* stream);

/* ---------------------------------------------------------------- factorisations */
/* ILU(0) of every system, in place layout: d_lu (nsys*nnz, factor pattern)
 * holds L (strictly lower, unit diagonal implicit) and U (upper).
 * Replaces ILU_0_Factorization_Gpu (ILU_0.h:9) for approaches 1..4 and
 * ComputeILU0Approach1 (ILU_0.h:10). */
bilu_status bilu_ilu0(const bilu_plan* plan, int nsys, const double* d_values,
                      double* d_lu, int approach, void* stream);

/* ParILU(0): `sweeps` Jacobi fixed-point sweeps starting from d_lu_init (or
 * from L = strict-lower(A) + I, U = upper(A) when NULL).  Replaces
 * ParILU_0_Factorization_Gpu (parILU_0.h:7). */
bilu_status bilu_parilu0(const bilu_plan* plan, int nsys, const double* d_values,
                         const double* d_lu_init, double* d_lu, int sweeps, void* stream);

/* Split in-place factors into the reference's separate L / U CSR value arrays
 * (L: strict lower + explicit 1.0 diagonal last in each row; U: diagonal first).
 * Replaces Update_row_pointers_L_and_U_and_Allocate_Memory + Fill_L_and_U_col_idxs_and_vals
 * (factorization.cu:487-575).  d_L: nsys*nnz_L, d_U: nsys*nnz_U. */
bilu_status bilu_split_lu(const bilu_plan* plan, int nsys, const double* d_lu,
                          double* d_L, double* d_U, void* stream);

/* ISAI of L and U from in-place factors d_lu: d_ail (nsys*nnz_isai_L),
 * d_aiu (nsys*nnz_isai_U) on the plan's ISAI patterns (pattern of |T|^power).
 * For a BILU_PRECOND_GENERAL_ISAI plan: d_lu holds A's values (factor pattern),
 * d_ail receives the ISAI of A (GenerateISAI_gpu(aiA, A, general, p)) and
 * d_aiu is not used.
 * With a BILU_REDUCE_FAST plan the aiU entries are multiplied by the correctly
 * rounded reciprocal of the diagonal instead of divided by it, as the plan's
 * solver does; BILU_REDUCE_REF keeps the reference's divisions.
 * Replaces GenerateISAI_gpu(aiL, L, lower_tri, p) and (aiU, U, upper_tri, p)
 * (isai.h:9, isai_gpu.cu:720). */
bilu_status bilu_isai(const bilu_plan* plan, int nsys, const double* d_lu,
                      double* d_ail, double* d_aiu, void* stream);

/* ||b - A x||_2 per system (reference operation order).  Replaces
 * KernelFillTrueResNorms (Bicgstab_common.hpp:294-342), without its
 * n <= 54 / nnz <= 2560 static limits. */
bilu_status bilu_true_residual(const bilu_plan* plan, int nsys, const double* d_values,
                               const double* d_b, const double* d_x, double* d_norms,
                               void* stream);

/* ---------------------------------------------------------------- uneven batches */
/* Systems of different sizes and sparsity patterns in one solve (no reference
 * counterpart: the reference requires one pattern per batch,
 * ReadWriteData.cpp:398-433).  Supported preconditioners: BILU_PRECOND_ILU0
 * (merged, the reference's PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu
 * arithmetic per system) and BILU_PRECOND_NONE.
 * Host layout: systems back to back; row pointers n_s + 1 per system (local,
 * starting at 0), columns nnz_s per system; device values / b / x are the
 * concatenation of the systems' arrays in the same order (value offset of
 * system s = sum of the earlier sys_nnz, vector offset = sum of the earlier sys_n).
 * The plan sorts the systems into size buckets, in the reference order
 * n <= 128, 256, 512, 1024, larger (5 buckets), each run as one persistent
 * kernel over a work queue (largest systems first); in BILU_REDUCE_FAST order
 * n <= 64, 96, 128, 192, 256, 384, 512, 768, 1024, larger (10 buckets), those
 * with n <= 1024 run the register-resident solver, one CTA per system (largest
 * first) or a persistent grid over the bucket's work queue, whichever the
 * autotuner measures faster.
 * A solve replays one CUDA graph holding every bucket launch on concurrent
 * branches.  The graph is captured on the first solve and again whenever the
 * device pointers change. */
typedef struct bilu_uneven_plan bilu_uneven_plan;
bilu_status bilu_uneven_plan_create(bilu_uneven_plan** plan, int nsys, const int* h_sys_n, const int* h_sys_nnz,
                                    const int* h_row_ptrs, const int* h_col_idxs, const bilu_options* opts);
bilu_status bilu_uneven_plan_destroy(bilu_uneven_plan* plan);
/* Tunes every bucket's CTA size and grid on the given batch: persistent
 * shared-memory buckets time 64..1024 threads (grid from the occupancy of
 * each) on the bucket alone; register-resident buckets, largest systems
 * first, try 1x, 2x and 4x the fewest threads, each with one CTA per system
 * and with a persistent grid over the bucket's work queue, judged by the time
 * of the whole graph-launched batch (the buckets run concurrently there).
 * Synchronises the stream; overwrites d_x. */
bilu_status bilu_uneven_autotune(bilu_uneven_plan* plan, const double* d_values, const double* d_b, double* d_x,
                                 void* stream);
bilu_status bilu_uneven_solve(bilu_uneven_plan* plan, const double* d_values, const double* d_b, double* d_x,
                              const bilu_results* results, void* stream);
/* Pins bucket `bucket`'s CTA size (threads, 0 = keep) and grid (0 = one CTA
 * per system for register-resident buckets, the occupancy-sized persistent
 * grid otherwise; a smaller grid makes the bucket's CTAs persistent over its
 * work queue), instead of (or after) the autotuner's choice.  The results do
 * not depend on the grid; for register-resident buckets the CTA size is part
 * of the FAST order.  BILU_ERR_INVALID when the CTA size does not fit.  No
 * reference counterpart. */
bilu_status bilu_uneven_set_config(bilu_uneven_plan* plan, int bucket, int threads, int grid);
/* Bucket `bucket` (0 .. count - 1; BILU_ERR_INVALID past the last one): n
 * range (n_lo, n_hi], systems, chosen CTA size, grid (below `systems`:
 * persistent CTAs over the bucket's work queue), shared memory per CTA,
 * autotuned time (ms, -1 if not tuned; the bucket alone for persistent
 * shared-memory buckets, the whole batch after this bucket's choice for
 * register-resident ones). */
bilu_status bilu_uneven_get_info(const bilu_uneven_plan* plan, int bucket, int* n_lo, int* n_hi, int* systems,
                                 int* threads, int* grid, int* smem_bytes, float* tuned_ms);

/* Forward error against an FP64 dense LU with partial pivoting (no reference
 * counterpart): for each sampled system s = h_sys_ids[q], the dense solution
 * x_dense of A_s x = b_s and h_fwd_err[q] = ||x_s - x_dense||_2 / ||x_dense||_2
 * (d_x may be NULL: then the errors are ||x_dense||).  d_x_dense (nsample*n,
 * optional) receives the dense solutions.  Allocates n*n doubles per sampled
 * system and synchronises the stream. */
bilu_status bilu_forward_error(const bilu_plan* plan, int nsample, const int* h_sys_ids, const double* d_values,
                               const double* d_b, const double* d_x, double* h_fwd_err, double* d_x_dense,
                               void* stream);

/* ---------------------------------------------------------------- learned ParILU warm start */
/* A per-nonzero MLP (9 features -> 64 -> 64 -> 1, GELU, BF16 weights, FP32
 * accumulation) predicting the converged ParILU(0) factors from the matrix
 * values; no counterpart in the reference.  Features of entry (i,j), scaled
 * by |a_ii|: a_ij, a_ii, a_jj, ||A(i,:)||, ||A(:,j)||, level(i), sign(j-i),
 * and the first-order Schur corrections c_i, c_j (c_r = sum_{k<r} a_rk a_kr / a_kk).
 * The network outputs a relative correction y of the first-order factor
 * estimate; warm start lu0_ij = a_ij * base_ij * (1 + y).  Entries on or
 * above the diagonal without dependency pairs converge to a_ij exactly and are
 * copied instead.  Inference runs the 64x64 layer on the tensor cores.
 * Values are in the plan's factor pattern (the plan must have every diagonal). */
typedef struct bilu_mlp bilu_mlp;
bilu_status bilu_mlp_create(bilu_mlp** mlp, uint64_t seed);
bilu_status bilu_mlp_destroy(bilu_mlp* mlp);
int bilu_mlp_param_count(void);
/* FP32 master parameters: W1[64][9], b1[64], W2[64][64], b2[64], W3[64], b3. */
bilu_status bilu_mlp_get_params(const bilu_mlp* mlp, float* h_params);
bilu_status bilu_mlp_set_params(bilu_mlp* mlp, const float* h_params);
/* `steps` Adam steps (learning rate decaying from lr to lr/20 on a cosine;
 * beta 0.9 / 0.999) on random minibatches of `batch` nonzeros drawn from the
 * nsys systems (d_lu_target: their converged ParILU factors), among the
 * entries the network predicts; mean squared error of the factor correction.  Synchronises;
 * h_losses (steps entries, optional) receives the per-step loss. */
bilu_status bilu_mlp_train(bilu_mlp* mlp, const bilu_plan* plan, int nsys, const double* d_values,
                           const double* d_lu_target, int steps, int batch, float lr, uint64_t seed,
                           float* h_losses, void* stream);
/* Loss and gradient (not applied) over the given global entries
 * (s * nnz + e); synchronises.  For checking the backward pass. */
bilu_status bilu_mlp_loss_grad(bilu_mlp* mlp, const bilu_plan* plan, int nsys, const double* d_values,
                               const double* d_lu_target, int nsample, const int* h_idx, float* h_loss,
                               float* h_grad, void* stream);
/* Features (nsample * 9), network outputs and first-order estimates of the
 * given entries; synchronises.  For checking the forward pass. */
bilu_status bilu_mlp_eval(bilu_mlp* mlp, const bilu_plan* plan, int nsys, const double* d_values, int nsample,
                          const int* h_idx, float* h_features, float* h_out, double* h_base, void* stream);
/* Warm start of every system: the network's factors, or A itself where their
 * ILU residual ||(A - L0 U0)|_S||_F / ||A||_F exceeds `threshold`.  Optional
 * device outputs: the residual and 1 / 0 for warm start used / fallback.
 * d_lu0 feeds bilu_solve_warm or bilu_parilu0. */
bilu_status bilu_mlp_warm_start(bilu_mlp* mlp, const bilu_plan* plan, int nsys, const double* d_values,
                                double* d_lu0, double threshold, double* d_ilu_res, int* d_used, void* stream);
/* Flat binary file: "BILUMLP1", three ints (features, hidden, params), FP32 parameters. */
bilu_status bilu_mlp_save(const bilu_mlp* mlp, const char* path);
bilu_status bilu_mlp_load(bilu_mlp* mlp, const char* path);

/* ---------------------------------------------------------------- misc */
const char* bilu_last_error(void);
const char* bilu_version(void);
/* Number of CUDA devices visible (0 when none; never fails). */
int bilu_device_count(void);
/* FP64 FMA throughput of the current device in GFLOP/s (two FLOPs per FMA),
 * measured with CUDA events on independent DFMA chains that fill every SM
 * (the best of three launch shapes): the peak against which the FP64 roofline
 * of the solver kernels is quoted.  h_sm_mhz (optional) receives the SM clock
 * during the best launch, from the SM cycle counter and the global timer.
 * Allocates 32 bytes and synchronises the stream.  No reference counterpart. */
bilu_status bilu_probe_fp64_rate(double* h_gflops, double* h_sm_mhz, void* stream);

/* Checks the FP64 operations the kernels do with integer arithmetic against
 * the hardware: the FP64 <-> FP32 conversions of the FP32 preconditioner paths
 * (round to nearest even; the hardware conversion for float subnormal results,
 * infinities and NaNs) and the correctly rounded FP64 reciprocal of the FAST
 * ParILU and ISAI (against __drcp_rn; the hardware's for zero, subnormal,
 * infinite and NaN inputs and subnormal results), on n_per_thread bit patterns
 * per thread of 4 CTAs of 256 threads per SM: random doubles, doubles across
 * every float exponent boundary with rounding ties, random floats, and
 * doubles with short, long and zero mantissas.  h_mismatch[0] / [1] / [2]:
 * roundings / widenings / reciprocals that differ (0, 0, 0 expected).
 * Synchronises the stream.  No reference counterpart. */
bilu_status bilu_check_integer_fp(int n_per_thread, uint64_t seed, unsigned long long* h_mismatch, void* stream);

/* ---------------------------------------------------------------- synthetic inputs */
/* Seeded generators of the benchmark workloads (host memory; no GPU needed).
 * kind: 1 = 2D 5-point (gx*gy), diag 4+U(0,1), off -(1+0.2U(-1,1)), E/W skew +-0.3U(0,1);
 *       2 = 3D 7-point (gx*gy*gz), diag 6+U(0,1), off -(1+0.25U(-1,1)), per-system
 *           Peclet P~U(0,0.5) as a +-P/2 skew on the x neighbours;
 *       4 = 2D 5-point convection-diffusion, Peclet~U(0,2), first-order upwind in x;
 *       5 = 3D 7-point, diag 6+U(0,1), off -(1+0.3U(-1,1)).
 * b ~ U(-1,1).  Pattern arrays: (gx*gy*gz)+1 / nnz; values nsys*nnz; b nsys*n.
 * Pass NULL pattern/value arrays to query n / nnz only. */
bilu_status bilu_gen_stencil(int kind, int gx, int gy, int gz, int nsys, uint64_t seed,
                             int* n, int* nnz, int* h_row_ptrs, int* h_col_idxs,
                             double* h_values, double* h_b);

/* Systems first .. first+nsys-1 of the same seeded stream (system s of
 * bilu_gen_stencil is system s here): each rank of a multi-GPU run generates
 * its own slab of one global batch.  No reference counterpart. */
bilu_status bilu_gen_stencil_range(int kind, int gx, int gy, int gz, long long first, int nsys, uint64_t seed,
                                   int* n, int* nnz, int* h_row_ptrs, int* h_col_idxs,
                                   double* h_values, double* h_b);

/* Uneven batch (per-system sizes and patterns): n_s = floor(exp(U(ln nmin, ln nmax))),
 * per row k ~ U{kmin..kmax} distinct off-diagonal columns plus the diagonal
 * (sorted), off-diagonals ~ N(0,1), a_ii = 1.2 * sum_j |a_ij| * sign, sign ~ U{+-1};
 * b ~ U(-1,1).  Systems are stored back to back: row pointers n_s+1 per system
 * (local, starting at 0), columns / values sys_nnz[s] per system, b n_s per
 * system.  With h_row_ptrs == NULL only sys_n / sys_nnz are filled. */
bilu_status bilu_gen_uneven(int nsys, uint64_t seed, int nmin, int nmax, int kmin, int kmax,
                            int* sys_n, int* sys_nnz, int* h_row_ptrs, int* h_col_idxs,
                            double* h_values, double* h_b);

#ifdef __cplusplus
}
#endif
#endif /* BILU_H */
