// Internal declarations shared by the libitg.so translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstdarg>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/itg.h"

#define ITG_MAX_RANK 16
#define ITG_PINNED_DOUBLES 4096  // host staging for small results (Davidson subspace <= 32x32)
#define ITG_GEMV_MAX_PART 65536  // partial sums of itg_gemv_t
#define QR_NB 32                 // panel width of the blocked Householder QR
#define QR_NB_MAX 64

// A lowered contraction C[m,n] = sum_k A[m,k] B[k,n] with every operand
// addressed through offset tables (see itg_contract.cu).
struct ContractPlan {
  int64_t M = 0, N = 0, K = 0;
  int64_t* tables = nullptr;  // offAm[M] offCm[M] offBn[N] offCn[N] offAk[K] offBk[K]
  bool a_kmaj = false, b_kmaj = false;
  // Autotuning: the plan's canonical shape key (empty for plans that must not
  // be tuned) and the chosen variants (-1 / 0: not chosen yet).
  std::string key;
  mutable int tile = -1;      // FP64 tile variant (ITG_TILE_*)
  mutable int split_bn = 0;   // split GEMM tile width (128 or 256)
  const int64_t* offAm() const { return tables; }
  const int64_t* offCm() const { return tables + M; }
  const int64_t* offBn() const { return tables + 2 * M; }
  const int64_t* offCn() const { return tables + 2 * M + N; }
  const int64_t* offAk() const { return tables + 2 * M + 2 * N; }
  const int64_t* offBk() const { return tables + 2 * M + 2 * N + K; }
  ~ContractPlan() {
    if (tables) cudaFree(tables);
  }
};

// The six offset tables of a ContractPlan as mixed-radix sums: section g
// (0: M, 1: N, 2: K) has count[g] entries; entry l, written as digits of
// dim[g][0..nmodes[g]) (first mode fastest), gives sum digit * s1 to the
// section's first table and sum digit * s2 to its second.  Lets a kernel
// build the tables on the device (itg_noalloc.cu).
struct PlanTableDesc {
  int nmodes[3];
  int64_t count[3];
  int64_t dim[3][ITG_MAX_RANK];
  int64_t s1[3][ITG_MAX_RANK];
  int64_t s2[3][ITG_MAX_RANK];
};

// Operand slices of a split-precision contraction kept for reuse: the bf16
// digit slices and row exponents of one operand (src) under one plan and
// padding.  Used only while an entry point knows that operand is constant
// (the environments L and R during one Davidson solve).
struct SliceCache {
  const double* src = nullptr;
  const void* plan = nullptr;
  int64_t rows_pad = 0, kpad = 0;
  bool valid = false;
  void* buf = nullptr;
  size_t bytes = 0;
};

struct itg_handle {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  // Reusable device scratch.  Operations on one handle are ordered on its
  // stream, so a buffer can be handed to the next call once the previous
  // kernels using it were enqueued before the new ones.
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // Workspace of the split-precision path (slices, exponents, accumulators);
  // separate from `scratch` because split contractions run inside callers
  // (the H_eff chain, Davidson) that hold regions of `scratch`.
  void* split_ws = nullptr;
  size_t split_ws_bytes = 0;
  // Small pinned host buffer for scalar results (dot, truncation outputs).
  double* pinned = nullptr;
  // Partial sums of itg_gemv_t (its own buffer: callers hold scratch regions).
  double* gemv_part = nullptr;
  // Persistent device buffers of the contraction plans, keyed by shape.
  std::unordered_map<std::string, std::shared_ptr<ContractPlan>> plans;
  // Device status word for bounded waits (ITG_ERR_TIMEOUT reporting).
  int* dev_status = nullptr;
  // Limit of every bounded device-side wait, in %globaltimer nanoseconds
  // (itg_set_wait_limit_ns).
  uint64_t wait_ns = 4000000000ull;
  // Descriptor array of grouped launches (separate from scratch: grouped calls
  // run inside callers that hold scratch regions).
  void* group_desc = nullptr;
  size_t group_desc_bytes = 0;
  // CUDA-graph replay of the H_eff chain inside Davidson (itg_set_graphs).
  bool use_graphs = false;
  cudaStream_t cap_stream = nullptr;
  // Kernel timing (itg_profile): event pairs recorded around kernel launches.
  bool prof_on = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_events;
  std::vector<cudaEvent_t> prof_pool;
  // Autotuning (itg_set_autotune): on by default unless ITG_AUTOTUNE=0.
  bool autotune = true;
  void* tune_buf = nullptr;   // throw-away outputs of tuning launches
  size_t tune_buf_bytes = 0;
  int64_t tune_runs = 0;
  void* cplx_buf = nullptr;   // realified operands / temporaries of complex contractions
  size_t cplx_buf_bytes = 0;
  int64_t* tab_buf = nullptr; // offset tables of the blocked QR's submatrix products
  int64_t tab_buf_elems = 0;
  // Look-ahead of the blocked QR: the trailing updates run on qr_stream while
  // the next panel is factored on `stream` (own offset tables, two events).
  cudaStream_t qr_stream = nullptr;
  cudaEvent_t qr_ev_ready = nullptr;  // panel's reflectors and T are final (on `stream`)
  cudaEvent_t qr_ev_done = nullptr;   // trailing update finished (on qr_stream)
  int64_t* tab_buf2 = nullptr;
  int64_t tab_buf2_elems = 0;
  // Split operand slice reuse: [0] the A operand, [1] the B operand of the
  // next split contraction when slice_keep[i] is set (see SliceCache).
  SliceCache slice_cache[2];
  bool slice_keep[2] = {false, false};
  bool heff_keep_env_slices = false;  // set by Davidson for the duration of one solve
  int last_sweeps = 0;        // Jacobi sweeps of the last SVD / eigh call
  bool last_mixed = false;    // the last SVD finished on the mixed method
  int64_t svd_fallbacks = 0;  // mixed SVDs redone with FP64 Jacobi
  bool svd_qr_precond = true; // itg_set_svd_options
  int jacobi_mode = 0;        // 0 blocked, 1 element pairs per step, 2 one cooperative launch, 3 blocked narrow
};

// Record a timing event pair around a launch when profiling is on.
struct ProfScope {
  itg_handle* h;
  int kind;
  cudaEvent_t e1 = nullptr;
  ProfScope(itg_handle* hh, int k);
  ~ProfScope();
};

namespace itg {
// Persistent one-sided Jacobi (itg_jacobi.cu): all sweeps in one cooperative
// launch; aux holds jacobi_aux_ints(max_sweeps) device ints.
int jacobi_aux_ints(int max_sweeps);
template <class T>
int jacobi_persistent(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, int max_sweeps, int* aux,
                      int* sweeps, T amin_conv = T(0));
// Blocked Householder QR (itg_qr_blocked.cu): panels of QR_NB columns, WY
// trailing updates through the contraction engine at `precision`; nref
// reflectors (nref <= min(m, n)) applied to all n columns.
int qr_blocked(itg_handle* h, double* W, int64_t m, int64_t n, int64_t nref, double* Vh, double* tau, double* rd,
               double* Tbuf, double* ws, int precision);
int q_apply_blocked(itg_handle* h, double* Y, int64_t m, int64_t n, int64_t ncols, const double* Vh,
                    const double* Tbuf, double* ws);
size_t qr_blocked_ws_doubles(int64_t n);
size_t qr_blocked_t_doubles(int64_t n);
// Blocked one-sided Jacobi (itg_jacobi.cu): block pairs staged in shared
// memory, one launch per block step; ITG_ERR_UNSUPPORTED when m is too large.
template <class T>
int jacobi_blocked(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, int max_sweeps, int* flag,
                   int* sweeps, T amin_conv = T(0));
}  // namespace itg

// Error helpers ---------------------------------------------------------------
int itg_fail(itg_handle* h, int code, const char* fmt, ...);

#define ITG_CUDA(h, call)                                                        \
  do {                                                                           \
    cudaError_t _e = (call);                                                     \
    if (_e != cudaSuccess)                                                       \
      return itg_fail((h), ITG_ERR_CUDA, "%s failed: %s (%s:%d)", #call,          \
                      cudaGetErrorString(_e), __FILE__, __LINE__);               \
  } while (0)

#define ITG_CHECK_LAUNCH(h) ITG_CUDA((h), cudaGetLastError())

#define ITG_TRY(expr)            \
  do {                           \
    int _s = (expr);             \
    if (_s != ITG_OK) return _s; \
  } while (0)

// Device scratch management ---------------------------------------------------
// Stack-like arena: callers take `Scratch` regions for the duration of one API
// call.  Growth reallocates only when nothing from the arena is live.
struct ScratchArena {
  itg_handle* h;
  size_t used = 0;
  explicit ScratchArena(itg_handle* hh) : h(hh) {}
};

// Ensure the handle's scratch holds at least `bytes`; synchronises the stream
// before freeing an older, smaller buffer.
int itg_scratch_reserve(itg_handle* h, size_t bytes);

static inline size_t itg_align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Grid sizing helpers ---------------------------------------------------------
static inline int itg_blocks_for(int64_t n, int threads, int cap) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// Internal entry points shared between translation units ----------------------
namespace itg {

// Deterministic dot product into a device double (two-stage reduction).
int dot_dev(itg_handle* h, int64_t n, const double* x, const double* y, double* out,
            double* partials);
int nrm2_dev(itg_handle* h, int64_t n, const double* x, double* out, double* partials);

// Truncation on device: writes {n_keep (as double), truncerr, docut} to out[0..2].
int truncate_dev(itg_handle* h, const double* P, int64_t n, int64_t maxdim, int64_t mindim,
                 double cutoff, int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                 double* out3);

// Column-major transpose (out is n x m) of the m x n matrix in (lda).
int transpose(itg_handle* h, int64_t m, int64_t n, const double* in, int64_t lda, double* out);

// General contraction with explicit plan cache and no scratch use beyond the plan.
int contract_f64(itg_handle* h, double alpha, const double* A, int rankA, const int64_t* dimsA,
                 const int32_t* modesA, const double* B, int rankB, const int64_t* dimsB,
                 const int32_t* modesB, double beta, double* C, int rankC, const int64_t* dimsC,
                 const int32_t* modesC, int precision);

}  // namespace itg
