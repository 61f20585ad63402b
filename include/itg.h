/*
 * itg.h — C ABI of libitg.so, a GB300 (sm_103a) dense FP64 tensor backend for
 * two-site DMRG.
 *
 * The reference (ITensorsGPU.jl) has no C boundary: it plugs into ITensors.jl by
 * adding Julia methods for `CuDense` / `CuDiag` storage (src/ITensorsGPU.jl:32-43).
 * Each entry point below is the device-side body of one of those methods; the
 * Julia `ccall` glue and the Python ctypes mirror call these functions with plain
 * device pointers.  Comments name the reference method each one replaces.
 *
 * Conventions
 *  - Every function returns an int status (ITG_OK = 0).  No C++ exception crosses
 *    this boundary.  itg_last_error(h) gives a message for the last failure.
 *  - Tensors are dense, column-major (first index fastest), exactly like the flat
 *    `Dense` storage of NDTensors (src/tensor/cudense.jl:19).  Dimensions are
 *    int64, mode labels are int32.
 *  - All device work is enqueued on the handle's stream and is asynchronous,
 *    except where an output is documented as a host scalar.  The blocked
 *    Householder QR inside the factorisations forks a second, internal stream
 *    from the handle's stream (through an event) and joins it again before the
 *    call returns, so later work on the handle's stream sees its results.
 *  - A handle is not thread-safe; use one per host thread.
 *  - The library never frees caller memory.  Memory the library needs beyond the
 *    caller's inputs and outputs (index tables, Jacobi scratch, reductions) comes
 *    from a per-handle workspace that grows on demand and is freed by
 *    itg_destroy.
 */
#ifndef ITG_H
#define ITG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define ITG_API __attribute__((visibility("default")))
#else
#define ITG_API
#endif

typedef struct itg_handle itg_handle;

enum {
  ITG_OK = 0,
  ITG_ERR_INVALID = 1,      /* bad argument (null pointer, bad enum)            */
  ITG_ERR_SHAPE = 2,        /* DimensionMismatch in the reference               */
  ITG_ERR_ALLOC = 3,        /* device allocation failed                         */
  ITG_ERR_CUDA = 4,         /* a CUDA runtime call failed                       */
  ITG_ERR_TIMEOUT = 5,      /* a bounded device-side wait ran out               */
  ITG_ERR_NOTCONVERGED = 6, /* an iterative solver hit its sweep limit          */
  ITG_ERR_UNSUPPORTED = 7   /* valid request the library does not implement     */
};

/* Element types.  ITG_C64 is complex FP64 stored interleaved (re, im): the
 * layout of Julia's ComplexF64, C99 double _Complex and torch.complex128.
 * itg_contract, itg_permute, itg_axpby_permuted and itg_diag_contract (a real
 * diagonal times a complex dense tensor) take either; their real alpha and
 * beta scale both parts.  Complex ranks are limited to 14 in contractions and
 * 15 elsewhere (the re/im parts run as extra modes of the real engine). */
enum { ITG_F64 = 0, ITG_C64 = 1 };

/* Arithmetic used by itg_contract.
 *  ITG_PREC_FP64  : native FP64 FMA; relative Frobenius error ~ K * 2^-53.
 *  ITG_PREC_SPLIT : FP64 operands split into bf16 integer slices, products on
 *                   the tcgen05 tensor cores with exact FP32 partial sums and an
 *                   exact integer recombination; error bound stated per call by
 *                   itg_split_error_bound. */
enum { ITG_PREC_FP64 = 0, ITG_PREC_SPLIT = 1 };

/* ---------------------------------------------------------------- handle */
/* No reference counterpart: CUDA.jl owns the context and default stream. */
ITG_API int itg_create(int device, itg_handle** out);
ITG_API int itg_destroy(itg_handle* h);
/* stream is a cudaStream_t (NULL = legacy default stream). */
ITG_API int itg_set_stream(itg_handle* h, void* stream);
ITG_API int itg_get_stream(itg_handle* h, void** stream);
ITG_API int itg_synchronize(itg_handle* h);
/* Device memory the handle holds now: its growable scratch arena, the
 * split-precision workspace, the autotuning buffer (bytes) and the number of
 * cached contraction plans (each with its device offset tables).  Any pointer
 * may be NULL.  No reference counterpart (CUDA.jl's pool is what the
 * reference's memory accounting goes through). */
ITG_API int itg_workspace_info(itg_handle* h, size_t* scratch_bytes, size_t* split_bytes, size_t* tune_bytes,
                               int64_t* plans);
/* enable = 1: itg_davidson_heff2 captures the H_eff chain once per call into a
 * CUDA graph (on a private capture stream) and replays it for every further
 * matvec.  Off by default. */
ITG_API int itg_set_graphs(itg_handle* h, int enable);
ITG_API const char* itg_last_error(itg_handle* h);
ITG_API const char* itg_status_string(int status);
/* Library version as major*10000 + minor*100 + patch. */
ITG_API int itg_version(void);

/* Kernel timing (tracing; the reference's analogue is its TimerOutputs
 * @timeit blocks, src/tensor/culinearalgebra.jl:41,82,91, which time launches
 * without a device sync).  itg_profile(h, 1) clears and starts recording CUDA
 * events on the handle's stream around the contraction kernels; 0 stops.
 * itg_profile_read synchronises the stream and returns the summed device time
 * and launch count of one kernel class:
 *   ITG_KERNEL_GEMM_F64   the FP64 gather-GEMM (k_gemm_gather_f64)
 *   ITG_KERNEL_GEMM_SPLIT the tcgen05 split-precision GEMM (k_split_gemm)
 *   ITG_KERNEL_SPLIT_PREP the split operand preparation (exponents + digits)
 *   ITG_KERNEL_HEFF_MID   the middle (merged-MPO) step of the H_eff matvec
 * and three phases of the SVD / bond factorisation (stream time from the
 * phase's first launch to its last, including the host reads it waits on):
 *   ITG_KERNEL_SVD_QR     Householder QR preconditioning and the application
 *                         of its Q to the kept columns
 *   ITG_KERNEL_SVD_JACOBI the Jacobi sweeps (FP32 in the mixed method)
 *   ITG_KERNEL_SVD_REFINE the mixed method's FP64 refinement, Newton-Schulz
 *                         steps and the polish of the isometric factor */
enum { ITG_KERNEL_GEMM_F64 = 0, ITG_KERNEL_GEMM_SPLIT = 1, ITG_KERNEL_SPLIT_PREP = 2, ITG_KERNEL_HEFF_MID = 3,
       ITG_KERNEL_SVD_QR = 4, ITG_KERNEL_SVD_JACOBI = 5, ITG_KERNEL_SVD_REFINE = 6 };
ITG_API int itg_profile(itg_handle* h, int enable);
ITG_API int itg_profile_read(itg_handle* h, int kernel, double* total_ms, int64_t* launches);
/* Measured FP64 FMA throughput of the handle's GPU in TFLOP/s (independent
 * DFMA chains on every SM, best of three timed launches after a warm-up; the
 * roofline denominator of the plain FP64 contraction).  Synchronises. */
ITG_API int itg_fp64_peak(itg_handle* h, double* tflops);

/* Autotuning of kernel variants per contraction shape.  Replaces the
 * reference's per-(mode, dim) algorithm cache (src/cudense.jl:284-326, cache
 * declared at src/ITensorsGPU.jl:55), which sweeps cuTENSOR algorithms on the
 * first use of a shape.  Here the first FP64 contraction of a shape whose
 * 128x128 tiling leaves the GPU under-filled times the tile variants
 * (128x128, 128x64, 64x64) on the call's own operands into a throw-away
 * output, and split contractions time the tcgen05 tile variants;
 * grouped launches choose their tile per shape class.  All variants compute
 * bit-identical results (the same k order per output element), so tuning only
 * changes speed.  The choices live in one per-process cache guarded by a
 * mutex; with the environment variable ITG_TUNE_FILE set they are also read
 * from and appended to that file.  Launches inside a CUDA-graph capture never
 * tune (they use the cached choice or the heuristic).
 * enable: 1 (default unless ITG_AUTOTUNE=0 in the environment) or 0
 * (heuristic choice only). */
enum { ITG_TILE_128x128 = 0, ITG_TILE_128x64 = 1, ITG_TILE_64x64 = 2 };
/* Split-precision tile variants (split_bn below): 128 and 256 columns per
 * CTA.  Either | ITG_SPLIT_STREAMK: one persistent CTA per resident slot, the
 * launch's work divided evenly between them, a tile shared by consecutive
 * ones at level boundaries and summed with exact integer atomics (same bits
 * as without). */
enum { ITG_SPLIT_BN_128 = 128, ITG_SPLIT_BN_256 = 256, ITG_SPLIT_STREAMK = 0x1000 };
ITG_API int itg_set_autotune(itg_handle* h, int enable);
/* entries: size of the process-wide cache; tunings: tuning runs by this handle. */
ITG_API int itg_autotune_info(itg_handle* h, int64_t* entries, int64_t* tunings);
/* Empty the process-wide cache and every cached choice of this handle's plans. */
ITG_API int itg_autotune_clear(itg_handle* h);
/* The variant a contraction of this shape would use now (without tuning):
 * *tile = ITG_TILE_* for FP64, *split_bn = ITG_SPLIT_BN_* (possibly
 * | ITG_SPLIT_STREAMK) for split. */
ITG_API int itg_autotune_query(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA,
                               int rankB, const int64_t* dimsB, const int32_t* modesB, int rankC,
                               const int64_t* dimsC, const int32_t* modesC, int* tile, int* split_bn);
/* Pin the variants of one shape (tile: ITG_TILE_*, split_bn: ITG_SPLIT_BN_*,
 * optionally | ITG_SPLIT_STREAMK; a negative / zero value leaves that choice
 * alone); stored in the process-wide cache like a tuned choice. */
ITG_API int itg_autotune_force(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA,
                               int rankB, const int64_t* dimsB, const int32_t* modesB, int rankC,
                               const int64_t* dimsC, const int32_t* modesC, int tile, int split_bn);

/* ---------------------------------------------------------------- memory */
/* Replace CuVector allocation and the H2D/D2H copies of
 * src/tensor/cudense.jl:4-13 (Dense{T,CuArray}(::Dense{T,Array}), cpu(x)). */
ITG_API int itg_malloc(itg_handle* h, void** ptr, size_t bytes);
ITG_API int itg_free(itg_handle* h, void* ptr);
ITG_API int itg_memcpy_h2d(itg_handle* h, void* dst, const void* src, size_t bytes);
ITG_API int itg_memcpy_d2h(itg_handle* h, void* dst, const void* src, size_t bytes);
ITG_API int itg_memcpy_d2d(itg_handle* h, void* dst, const void* src, size_t bytes);
ITG_API int itg_memset_zero(itg_handle* h, void* ptr, size_t bytes);

/* ---------------------------------------------------------- contraction */
/* C = alpha * A * B + beta * C over the modes A and B share.
 * Replaces contract!! (src/tensor/cudense.jl:83-110), _contract!
 * (src/tensor/cudense.jl:238-331) and _gemm_contract! (src/tensor/cudense.jl:170-236).
 * Modes that appear in A and B but not C are summed; every mode of C appears in
 * exactly one of A, B.  Ranks 0..16.  rank 0 tensors are scalars (one element).
 * A mode shared by A, B and C (a batch mode) is ITG_ERR_UNSUPPORTED, as the
 * reference's label construction (cudense.jl:255-283) never produces one.
 * C must not alias A or B. */
ITG_API int itg_contract(itg_handle* h, int dtype, double alpha,
                 const void* A, int rankA, const int64_t* dimsA, const int32_t* modesA,
                 const void* B, int rankB, const int64_t* dimsB, const int32_t* modesB,
                 double beta,
                 void* C, int rankC, const int64_t* dimsC, const int32_t* modesC,
                 int precision);

/* Complex and mixed contraction: dtypeA, dtypeB each ITG_F64 or ITG_C64 (C is
 * ITG_C64 when either is); alpha and beta are complex, two doubles (re, im)
 * each: C = alpha * A * B + beta * C.  A complex x complex product runs as one
 * real contraction of twice the rows and depth (the smaller operand expanded
 * into its 2 x 2 real representation); complex x real passes the re/im mode
 * through.  Replaces contract!! on CuDense{ComplexF64} and mixed real/complex
 * operands (src/tensor/cudense.jl:83-110; test/test_cucontract.jl:9,
 * test/test_cudiag.jl:54). */
ITG_API int itg_contract_z(itg_handle* h, int dtypeA, int dtypeB, const double* alpha,
                   const void* A, int rankA, const int64_t* dimsA, const int32_t* modesA,
                   const void* B, int rankB, const int64_t* dimsB, const int32_t* modesB,
                   const double* beta,
                   void* C, int rankC, const int64_t* dimsC, const int32_t* modesC,
                   int precision);

/* Truncated SVD of the complex m x n matrix A (ITG_C64, leading dimension
 * lda): A ~ U diag(S) V^H with U m x r, V n x r complex, S real descending,
 * r = min(m, n) columns written and *k kept (same truncation keywords as
 * itg_svd_trunc).  One-sided complex Jacobi.  Replaces svd on
 * CuDenseTensor{ComplexF64} (src/tensor/culinearalgebra.jl:33-72). */
ITG_API int itg_svd_trunc_z(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                    int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff, int doRelCutoff,
                    int legacy_gpu, double* U, double* S, double* V, int64_t* k, double* truncerr,
                    double* docut);

/* Eigendecomposition of the Hermitian complex n x n matrix A: A = U diag(D)
 * U^H with D real descending, U n x n complex, then truncation of D as a
 * spectrum (as itg_eigh_trunc).  Replaces eigen(::Hermitian) on ComplexF64
 * (src/tensor/culinearalgebra.jl:74-108). */
ITG_API int itg_eigh_trunc_z(itg_handle* h, int64_t n, const double* A, int64_t lda,
                     int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff, int doRelCutoff,
                     int legacy_gpu, double* D, double* U, int64_t* k, double* truncerr, double* docut);

/* Thin QR of the complex m x n matrix A: A = Q R, Q m x r with orthonormal
 * columns, R r x n, r = min(m, n) (complex Gram-Schmidt, re-orthogonalised
 * once).  Replaces qr on CuDenseTensor{ComplexF64}
 * (src/tensor/culinearalgebra.jl:110-121). */
ITG_API int itg_qr_z(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda, double* Q, double* R);

/* y = conj(x) for n complex elements (y may alias x): dag of a complex tensor. */
ITG_API int itg_conj(itg_handle* h, int64_t n, const double* x, double* y);

/* z = x + 0i for n elements (complex(::CuDense{Float64}), test/test_cudense.jl:60-70). */
ITG_API int itg_real_to_complex(itg_handle* h, int64_t n, const double* x, double* z);

/* x = alpha * x for n complex elements, alpha = (re, im). */
ITG_API int itg_zscal(itg_handle* h, int64_t n, const double* alpha, double* x);

/* Bound on |C_split - C_exact|_F / (|A|_F |B|_F) for ITG_PREC_SPLIT with the
 * library's slice count at contraction depth K (host-only arithmetic). */
ITG_API double itg_split_error_bound(int64_t K);
/* Limit of every bounded device-side wait (the split GEMM's mbarrier waits,
 * the cooperative Jacobi's grid barrier), in nanoseconds of %globaltimer;
 * 4 s by default, accepted range [1 us, 60 s].  A wait that runs out makes the
 * kernel record ITG_ERR_TIMEOUT, stop, wait (bounded) for its own copies in
 * flight, release what it holds and return; the calling entry point, or the
 * next synchronising one, reports ITG_ERR_TIMEOUT and the handle stays usable.
 * The reference's only failure handling on this path is the skip-and-warn
 * around its cuTENSOR calls (src/tensor/cudense.jl:321-323). */
ITG_API int itg_set_wait_limit_ns(itg_handle* h, uint64_t ns);
/* Runs one bounded wait that is designed to run out, through the same device
 * code as the library's kernels, and returns its status (ITG_ERR_TIMEOUT when
 * the wait ran out as designed):
 *   which = 0: the cooperative Jacobi's grid barrier, on 2 blocks, counting
 *              one participant that never arrives;
 *   which = 1: the split GEMM's mbarrier wait, on a barrier nobody arrives on.
 * Takes the handle's wait limit; synchronises.  Failure-path check for
 * callers and tests; nothing faults, traps or hangs. */
ITG_API int itg_wait_selftest(itg_handle* h, int which);
/* Work partition of the split GEMM's stream-K schedule (host-only arithmetic,
 * the code the kernel runs): the tile segments of cluster g when
 * cluster_tiles cluster tiles are shared by `clusters` persistent clusters.
 * Per segment 5 ints in seg: cluster tile, first level, end level (exclusive),
 * number of clusters contributing to that tile, the first of them.  *nseg =
 * the segment count; ITG_ERR_SHAPE when it exceeds cap. */
ITG_API int itg_split_partition(int64_t cluster_tiles, int clusters, int g, int32_t* seg, int cap, int* nseg);

/* ----------------------------------------------------------- permutation */
/* B = alpha * A, with B's modes a permutation of A's.
 * Replaces permute! (src/tensor/cudense.jl:447-500) and permutedims!!
 * (src/tensor/cudense.jl:38-60,112-127).  Ranks 0..16. B must not alias A. */
ITG_API int itg_permute(itg_handle* h, int dtype, double alpha,
                const void* A, int rank, const int64_t* dimsA, const int32_t* modesA,
                void* B, const int32_t* modesB);

/* C = alpha * permute(A -> modesB) + beta * B, with C laid out like B.
 * C may alias B (in place update).  Replaces Base.:+ / Base.:- on CuDense
 * (src/tensor/cudense.jl:333-445), which go through cuTENSOR elementwiseBinary!
 * into a fresh buffer and a copy back. */
ITG_API int itg_axpby_permuted(itg_handle* h, int dtype, double alpha,
                       const void* A, int rank, const int64_t* dimsA, const int32_t* modesA,
                       double beta, const void* B, const int32_t* modesB, void* C);

/* ------------------------------------------------------------- diagonal */
/* Contraction of a diagonal tensor D (all its modes share one diagonal index
 * of length dims[0]; `uniform` = 1 means D has one stored value d[0]) with a
 * dense tensor T.  C = alpha * D * T + beta * C.
 * Replaces contract! for (Uniform|Nonuniform)Diag x CuDense
 * (src/tensor/cudiag.jl:105-118,147-161), which densifies the diagonal, and
 * respects the index permutation that cudiag.jl:105-112 ignores. */
ITG_API int itg_diag_contract(itg_handle* h, int dtype, double alpha,
                      const double* d, int uniform, int rankD, const int64_t* dimsD, const int32_t* modesD,
                      const void* T, int rankT, const int64_t* dimsT, const int32_t* modesT,
                      double beta,
                      void* C, int rankC, const int64_t* dimsC, const int32_t* modesC);

/* Diag x Diag: c[i] = alpha * a[i or 0] * b[i or 0] (elementwise product of the
 * stored diagonals).  Replaces src/tensor/cudiag.jl:120-145. */
ITG_API int itg_diag_diag(itg_handle* h, int64_t n, double alpha,
                  const double* a, int a_uniform, const double* b, int b_uniform, double* c);

/* Scatter a diagonal into a dense tensor with all modes of length dims[0]
 * (dense(::NonuniformCuDiagTensor), src/tensor/cudiag.jl:8-13). */
ITG_API int itg_diag_to_dense(itg_handle* h, const double* d, int uniform, int rank,
                      const int64_t* dims, double* T);

/* ------------------------------------------------------- vector kernels */
/* FP64 level-1 operations on flat storage (norm, scalar *, /, axpy used by the
 * eigensolver: src/tensor/cudense.jl:22-27,502).  Reductions are
 * deterministic (fixed grid and tree order).  dot/nrm2 write a host double and
 * synchronise the stream; the _dev variants write a device double and do not. */
ITG_API int itg_scal(itg_handle* h, int64_t n, double alpha, double* x);
ITG_API int itg_axpy(itg_handle* h, int64_t n, double alpha, const double* x, double* y);
ITG_API int itg_axpby(itg_handle* h, int64_t n, double alpha, const double* x, double beta, double* y);
ITG_API int itg_fill(itg_handle* h, int64_t n, double value, double* x);
ITG_API int itg_dot(itg_handle* h, int64_t n, const double* x, const double* y, double* result);
ITG_API int itg_nrm2(itg_handle* h, int64_t n, const double* x, double* result);
ITG_API int itg_dot_dev(itg_handle* h, int64_t n, const double* x, const double* y, double* result_dev);
/* out[j] = sum_i X[i + j*ldx] * y[i] for j < k (X^T y, k small); device output. */
ITG_API int itg_gemv_t(itg_handle* h, int64_t n, int64_t k, const double* X, int64_t ldx,
               const double* y, double* out_dev);
/* y = beta*y + sum_j X[:, j] * c[j] (c is a device vector of length k). */
ITG_API int itg_gemv_n(itg_handle* h, int64_t n, int64_t k, const double* X, int64_t ldx,
               const double* c_dev, double beta, double* y);

/* Standard normal FP64 numbers from a counter-based Philox-4x32-10 generator
 * (Salmon et al., SC'11) followed by Box-Muller.  Element i depends only on
 * (seed, i), so the CPU restatement produces the same numbers.  Replaces the
 * CURAND randn! of src/cuitensor.jl:35-49 and src/mps/cumps.jl:44-53. */
ITG_API int itg_random_normal(itg_handle* h, int64_t n, uint64_t seed, uint64_t offset, double* x);

/* ------------------------------------------------------------ truncation */
/* Truncate a descending spectrum P (device, length n) and report how many
 * values to keep.  legacy_gpu = 1 restates src/tensor/cutruncate.jl:1-93
 * exactly (its per-element threshold rule); legacy_gpu = 0 is ITensors' CPU
 * rule (cumulative discarded weight <= cutoff * sum(P), then maxdim / mindim).
 * Host outputs; synchronises the stream.  maxdim <= 0 means no limit. */
ITG_API int itg_truncate(itg_handle* h, const double* P, int64_t n,
                 int64_t maxdim, int64_t mindim, double cutoff,
                 int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                 int64_t* n_keep, double* truncerr, double* docut);

/* ---------------------------------------------------------- factorisation */
/* Truncated SVD of the m x n column-major matrix A (lda >= m): A ~ U diag(S) V^T
 * with S descending.  One-sided blocked Jacobi in FP64.  U must hold m*min(m,n)
 * doubles (ldu = m), V n*min(m,n) (ldv = n), S min(m,n).  On return the first k
 * columns hold the kept factors.  A is not modified.  Host outputs k, truncerr,
 * docut; synchronises.  Replaces LinearAlgebra.svd(::CuDenseTensor)
 * (src/tensor/culinearalgebra.jl:33-72) + truncate! (src/tensor/cutruncate.jl). */
ITG_API int itg_svd_trunc(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                  int64_t maxdim, int64_t mindim, double cutoff,
                  int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                  double* U, double* S, double* V,
                  int64_t* k, double* truncerr, double* docut);

/* itg_svd_trunc with an explicit method and GEMM precision.
 *  ITG_SVD_JACOBI: one-sided FP64 Jacobi (every rotation in FP64).
 *  ITG_SVD_MIXED : FP32 one-sided Jacobi, then FP64-accurate refinement of the
 *                  singular vectors as eigenvectors of the Gram matrix
 *                  (matrix products through the contraction engine at
 *                  `precision`) and Newton-Schulz orthonormalisation.
 *                  P = sigma^2 to ~1e-13 P_max absolute; singular values and
 *                  vectors at FP64 accuracy above ~1e-4 sigma_max.  With QR
 *                  preconditioning (min(m,n) > 192) U is orthonormal for every
 *                  kept column and V only where sigma is resolved; use
 *                  itg_factorize_trunc when one factor must be orthonormal.
 *  ITG_SVD_AUTO  : Jacobi for min(m, n) <= 192, mixed above.
 * itg_svd_trunc always uses ITG_SVD_JACOBI (LAPACK-level accuracy). */
enum { ITG_SVD_AUTO = 0, ITG_SVD_JACOBI = 1, ITG_SVD_MIXED = 2 };
ITG_API int itg_svd_trunc_ex(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                             int64_t maxdim, int64_t mindim, double cutoff,
                             int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                             double* U, double* S, double* V,
                             int64_t* k, double* truncerr, double* docut,
                             int method, int precision);
/* Truncated factorisation A ~ L C with one exactly orthonormal factor, the
 * two-site bond split of the DMRG sweep: ITensors' factorize(phi, inds;
 * ortho, maxdim, mindim, cutoff) as called by replacebond! inside dmrg
 * (ITensors 0.2, external; used at examples/dmrg.jl:25, test/dmrg.jl:27,75),
 * built on the SVD that src/tensor/culinearalgebra.jl:33-72 provides.
 *  ortho = ITG_ORTHO_LEFT : L (m x k) has orthonormal columns, C = L^T A (k x n) = S V^T.
 *  ortho = ITG_ORTHO_RIGHT: L (n x k) has orthonormal columns, C = A L   (m x k) = U S.
 * The orthonormal factor is the one built from rotations (or refined
 * eigenvectors), never from a division by S, so it stays orthonormal for
 * kept singular values of any size; C is a matrix product at `precision`.
 * S (min(m,n)) holds the singular values, k/truncerr/docut as itg_svd_trunc.
 * L and C each hold max(m,n)*min(m,n) doubles (C's slot is also scratch). */
enum { ITG_ORTHO_LEFT = 0, ITG_ORTHO_RIGHT = 1 };
ITG_API int itg_factorize_trunc(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                                int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff,
                                int doRelCutoff, int legacy_gpu, int ortho, int method, int precision,
                                double* L, double* S, double* C, int64_t* k, double* truncerr,
                                double* docut);
/* Diagnostics of the last itg_svd_trunc / itg_svd_trunc_ex / itg_factorize_trunc /
 * itg_eigh_trunc call on this handle: Jacobi sweeps (FP32 sweeps for the mixed
 * method), whether the mixed method finished it (0: FP64 Jacobi), and the
 * handle's count of mixed SVDs whose refinement check failed and that were
 * redone with FP64 Jacobi.  Any pointer may be NULL. */
ITG_API int itg_svd_info(itg_handle* h, int* sweeps, int* mixed_used, int64_t* mixed_fallbacks);
/* SVD options of this handle.  qr_precondition = 1 (default): for
 * min(m, n) > 192 the working matrix is first factored A = Q R by Householder
 * reflections and the Jacobi iteration runs on R^T (far fewer sweeps on
 * graded spectra; A = (Q V_B) S U_B^T from R^T = U_B S V_B^T).  jacobi_mode:
 * 0 (default): block-cyclic Jacobi, block pairs staged in shared memory,
 * one launch per block step; 1: one CTA per column pair, one launch per
 * round-robin step; 2: element pairs with all sweeps in one cooperative
 * launch and a grid barrier between steps (measured slower than 1 on GB300);
 * 3: as 0 with 4-column blocks (half the shared memory per CTA, so several
 * CTAs share an SM). */
ITG_API int itg_set_svd_options(itg_handle* h, int qr_precondition, int jacobi_mode);

/* Eigendecomposition of the symmetric n x n matrix A: A = U diag(D) U^T with D
 * descending, then truncation of D as a spectrum.  U holds n*n doubles.
 * Replaces eigen(::Hermitian{CuDenseTensor}) (src/tensor/culinearalgebra.jl:74-108). */
ITG_API int itg_eigh_trunc(itg_handle* h, int64_t n, const double* A, int64_t lda,
                   int64_t maxdim, int64_t mindim, double cutoff,
                   int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                   double* D, double* U, int64_t* k, double* truncerr, double* docut);

/* Thin QR of the m x n matrix A: A = Q R, Q m x r, R r x n, r = min(m,n).
 * Replaces qr(::CuDenseTensor) (src/tensor/culinearalgebra.jl:110-121). */
ITG_API int itg_qr(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
           double* Q, double* R);

/* Plain matrix product C = A * B of column-major matrices
 * (Base.:* for order-2 tensors, src/tensor/culinearalgebra.jl:9-17). */
ITG_API int itg_matmul(itg_handle* h, int64_t m, int64_t n, int64_t k,
               const double* A, const double* B, double* C, int precision);

/* ------------------------------------------------- two-site DMRG kernels */
/* Effective Hamiltonian of two-site DMRG applied to psi:
 *   out[a', s1', s2', b'] = sum L[a, w, a'] W1[w, s1', s1, x] W2[x, s2', s2, y]
 *                               R[b, y, b'] psi[a, s1, s2, b]
 * L is (chiL, wL, chiL), W1 (wL, d, d, wM), W2 (wM, d, d, wR), R (chiR, wR, chiR),
 * psi and out (chiL, d, d, chiR), all column-major.  This is the ProjMPO product
 * ITensors' dmrg evaluates inside its eigensolver through four ITensor `*` calls
 * (each one contract!!, src/tensor/cudense.jl:83-110).  The call is a fixed chain
 * of four gather-GEMM contractions through workspace; with precision
 * ITG_PREC_SPLIT the two chi^3 steps run on the tensor cores. */
ITG_API int itg_heff2_apply(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d,
                    int64_t wL, int64_t wM, int64_t wR,
                    const double* L, const double* W1, const double* W2, const double* R,
                    const double* psi, double* out, int precision);

/* diag[a, s1, s2, b] = H_eff[(a,s1,s2,b),(a,s1,s2,b)] for the operator of
 * itg_heff2_apply (the Davidson diagonal preconditioner), O(chi^2) work. */
ITG_API int itg_heff2_diag(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d,
                           int64_t wL, int64_t wM, int64_t wR,
                           const double* L, const double* W1, const double* W2, const double* R,
                           double* diag);

/* itg_heff2_apply without any device allocation by the library.
 * No counterpart in the reference.  For callers that cannot let a library call
 * cudaMalloc: applications that own all device memory through their own
 * fixed-budget pool (the Julia side keeps ITensors' tensors in the CUDA.jl
 * pool), or that cannot accept the device synchronisation cudaMalloc may cause.
 * Intermediates live in one file-scope __device__ array of 4 Mi doubles
 * (32 MiB) that every GPU loading libitg.so holds until exit; problems needing
 * more return ITG_ERR_UNSUPPORTED (itg_heff2_apply has no such limit; with
 * d = 2, w = 5 the limit is about chiL * chiR <= 100000).  FP64 arithmetic
 * only.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  The
 * plans' offset tables are written into the array by a kernel, so a call makes
 * no host-to-device copy.  Sizes are checked factor by factor against the
 * array before any product is formed.  All calls share the array, so calls
 * that overlap on the GPU race. */
ITG_API int itg_heff2_apply_noalloc(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d,
                                    int64_t wL, int64_t wM, int64_t wR,
                                    const double* L, const double* W1, const double* W2,
                                    const double* R, const double* psi, double* out);

/* Lowest eigenpair of the two-site effective Hamiltonian by Davidson with the
 * diagonal preconditioner.  psi (device) is the start vector and is overwritten
 * with the normalised eigenvector; energy (host) receives the eigenvalue.
 * krylovdim = largest subspace before restart, maxiter = restarts, tol =
 * residual-norm tolerance.  nmatvec (host, may be NULL) receives the number of
 * H_eff applications.  This stands in for the eigensolver that ITensors' dmrg
 * calls (KrylovKit eigsolve / ITensors davidson, exercised by
 * test/test_cuiterativesolvers.jl:13-28). */
ITG_API int itg_davidson_heff2(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d,
                       int64_t wL, int64_t wM, int64_t wR,
                       const double* L, const double* W1, const double* W2, const double* R,
                       double* psi, int krylovdim, int maxiter, double tol, int precision,
                       double* energy, int* nmatvec);

/* ----------------------------------------- learned Davidson preconditioner */
/* A per-element MLP (F inputs -> 128 -> 128 -> 1, ReLU, BF16 weights, FP32
 * accumulation; FP32 master weights with Adam) with hand-written forward,
 * backward and optimizer kernels.  No counterpart in the reference: it stands
 * in for the diagonal preconditioner of the eigensolver.  X is element-major
 * (n x F floats). */
ITG_API int itg_mlp_create(itg_handle* h, int in_dim, uint64_t seed, void** mlp);
ITG_API int itg_mlp_destroy(itg_handle* h, void* mlp);
ITG_API int itg_mlp_num_params(void* mlp, int64_t* n);
ITG_API int itg_mlp_get_params(itg_handle* h, void* mlp, float* host);
ITG_API int itg_mlp_set_params(itg_handle* h, void* mlp, const float* host);
/* g[e] = network(X[e, :]) */
ITG_API int itg_mlp_forward(itg_handle* h, void* mlp, int64_t n, const float* X, float* g);
/* loss = mean_e (g[e] mult[e] - target[e])^2; writes the gradient w.r.t. the
 * master parameters to grad (device, num_params floats, may be NULL), the loss
 * to *loss (host, may be NULL), then takes one Adam step when lr > 0. */
ITG_API int itg_mlp_train_step(itg_handle* h, void* mlp, int64_t n, const float* X, const float* mult,
                               const float* target, float lr, float* grad, float* loss);
/* Features of the learned preconditioner for the residual r of the two-site
 * problem (F = 5): normalised residual, (diag - theta)/scale, clipped inverse,
 * left / right Schmidt values of each element's link indices (lamL: chiL
 * values, lamR: chiR values, either may be NULL).  mult = the diagonally
 * preconditioned normalised residual (normalised residual x clipped inverse). */
ITG_API int itg_heff2_features(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d,
                               const double* r, const double* diag, double theta,
                               const double* lamL, const double* lamR, float* X, float* mult);
/* itg_davidson_heff2 with the learned preconditioner: corrections are
 * t = (1 + network(features)) * mult (mult as in itg_heff2_features: an
 * untrained network with a zero output layer is the diagonal preconditioner);
 * convergence is still judged by the exact
 * residual norm, and when a learned correction fails to reduce the residual by
 * 10% the diagonal preconditioner takes over for the rest of the solve
 * (*fallbacks counts those hand-overs, may be NULL). */
ITG_API int itg_davidson_heff2_learned(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d,
                                       int64_t wL, int64_t wM, int64_t wR,
                                       const double* L, const double* W1, const double* W2, const double* R,
                                       double* psi, int krylovdim, int maxiter, double tol, int precision,
                                       void* mlp, const double* lamL, const double* lamR,
                                       double* energy, int* nmatvec, int* fallbacks);

/* ------------------------------------------- many independent instances */
/* Grouped FP64 contraction: `count` contractions with the same ranks and mode
 * labels but their own dims and pointers (dims arrays concatenated per problem),
 * C_i = alpha A_i B_i + beta C_i, all tiles of all problems in one launch. */
ITG_API int itg_contract_grouped(itg_handle* h, int count, double alpha,
                                 const void* const* A, int rankA, const int64_t* dimsA, const int32_t* modesA,
                                 const void* const* B, int rankB, const int64_t* dimsB, const int32_t* modesB,
                                 double beta,
                                 void* const* C, int rankC, const int64_t* dimsC, const int32_t* modesC);

/* Truncated SVDs of `count` matrices (each min(m, n) <= 512), one CTA per
 * matrix running FP64 one-sided Jacobi, on-device truncation per instance.
 * U_i, S_i, V_i sized as for itg_svd_trunc; k and truncerr are host arrays. */
ITG_API int itg_svd_trunc_batched(itg_handle* h, int count, const int64_t* m, const int64_t* n,
                                  const double* const* A, const int64_t* maxdim, int64_t mindim,
                                  double cutoff, int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                                  double* const* U, double* const* S, double* const* V,
                                  int64_t* k, double* truncerr);

/* itg_davidson_heff2 for `count` instances sharing d and the MPO bond
 * dimensions (the same bond of equally long chains), each with its own chiL,
 * chiR and tensors.  The H_eff chain runs as grouped launches over all
 * instances; energy and nmatvec are host arrays of length count. */
ITG_API int itg_davidson_heff2_batched(itg_handle* h, int count, const int64_t* chiL, const int64_t* chiR,
                                       int64_t d, int64_t wL, int64_t wM, int64_t wR,
                                       const double* const* L, const double* const* W1,
                                       const double* const* W2, const double* const* R,
                                       double* const* psi, int krylovdim, int maxiter, double tol,
                                       double* energy, int* nmatvec);

#ifdef __cplusplus
}
#endif

#endif /* ITG_H */
