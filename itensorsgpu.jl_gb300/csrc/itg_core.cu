// Handle, memory, level-1 vector kernels and the Philox normal generator.
#include "itg_internal.cuh"

#include <cstdlib>

#include <cmath>

#define ITG_VERSION 10000  // 1.0.0

int itg_fail(itg_handle* h, int code, const char* fmt, ...) {
  if (h) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->last_error = buf;
  }
  return code;
}

extern "C" int itg_version(void) { return ITG_VERSION; }

extern "C" const char* itg_status_string(int s) {
  switch (s) {
    case ITG_OK: return "ITG_OK";
    case ITG_ERR_INVALID: return "ITG_ERR_INVALID";
    case ITG_ERR_SHAPE: return "ITG_ERR_SHAPE";
    case ITG_ERR_ALLOC: return "ITG_ERR_ALLOC";
    case ITG_ERR_CUDA: return "ITG_ERR_CUDA";
    case ITG_ERR_TIMEOUT: return "ITG_ERR_TIMEOUT";
    case ITG_ERR_NOTCONVERGED: return "ITG_ERR_NOTCONVERGED";
    case ITG_ERR_UNSUPPORTED: return "ITG_ERR_UNSUPPORTED";
    default: return "ITG_ERR_UNKNOWN";
  }
}

extern "C" int itg_create(int device, itg_handle** out) {
  if (!out) return ITG_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return ITG_ERR_CUDA;
  if (device < 0 || device >= ndev) return ITG_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return ITG_ERR_CUDA;
  itg_handle* h = new itg_handle();
  h->device = device;
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaMallocHost((void**)&h->pinned, ITG_PINNED_DOUBLES * sizeof(double)) != cudaSuccess) {
    delete h;
    return ITG_ERR_ALLOC;
  }
  if (cudaMalloc((void**)&h->gemv_part, sizeof(double) * ITG_GEMV_MAX_PART) != cudaSuccess) {
    cudaFreeHost(h->pinned);
    delete h;
    return ITG_ERR_ALLOC;
  }
  if (cudaMalloc((void**)&h->dev_status, 64) != cudaSuccess) {
    cudaFreeHost(h->pinned);
    delete h;
    return ITG_ERR_ALLOC;
  }
  cudaMemset(h->dev_status, 0, 64);
  if (const char* at = std::getenv("ITG_AUTOTUNE")) h->autotune = std::atoi(at) != 0;
  *out = h;
  return ITG_OK;
}

// ---------------------------------------------------------------- timing
static cudaEvent_t prof_event(itg_handle* h) {
  if (!h->prof_pool.empty()) {
    cudaEvent_t e = h->prof_pool.back();
    h->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

static void prof_clear(itg_handle* h) {
  for (auto& x : h->prof_events) {
    h->prof_pool.push_back(x.second.first);
    h->prof_pool.push_back(x.second.second);
  }
  h->prof_events.clear();
}

ProfScope::ProfScope(itg_handle* hh, int k) : h(hh), kind(k) {
  if (!h->prof_on) return;
  e1 = prof_event(h);
  cudaEventRecord(e1, h->stream);
}

ProfScope::~ProfScope() {
  if (!e1) return;
  cudaEvent_t e2 = prof_event(h);
  cudaEventRecord(e2, h->stream);
  h->prof_events.push_back({kind, {e1, e2}});
}

extern "C" int itg_profile(itg_handle* h, int enable) {
  if (!h) return ITG_ERR_INVALID;
  if (enable) {
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    prof_clear(h);
  }
  h->prof_on = enable != 0;
  return ITG_OK;
}

extern "C" int itg_profile_read(itg_handle* h, int kernel, double* total_ms, int64_t* launches) {
  if (!h || !total_ms) return ITG_ERR_INVALID;
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  double t = 0.0;
  int64_t n = 0;
  for (auto& x : h->prof_events) {
    if (x.first != kernel) continue;
    float ms = 0.f;
    ITG_CUDA(h, cudaEventElapsedTime(&ms, x.second.first, x.second.second));
    t += ms;
    n++;
  }
  *total_ms = t;
  if (launches) *launches = n;
  return ITG_OK;
}

void itg_release_plans(itg_handle* h);  // itg_contract.cu

extern "C" int itg_destroy(itg_handle* h) {
  if (!h) return ITG_ERR_INVALID;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  itg_release_plans(h);
  for (auto& c : h->slice_cache)
    if (c.buf) cudaFree(c.buf);
  prof_clear(h);
  for (auto e : h->prof_pool) cudaEventDestroy(e);
  if (h->scratch) cudaFree(h->scratch);
  if (h->split_ws) cudaFree(h->split_ws);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  if (h->group_desc) cudaFree(h->group_desc);
  if (h->tune_buf) cudaFree(h->tune_buf);
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->dev_status) cudaFree(h->dev_status);
  if (h->gemv_part) cudaFree(h->gemv_part);
  if (h->tab_buf) cudaFree(h->tab_buf);
  if (h->tab_buf2) cudaFree(h->tab_buf2);
  if (h->qr_ev_ready) cudaEventDestroy(h->qr_ev_ready);
  if (h->qr_ev_done) cudaEventDestroy(h->qr_ev_done);
  if (h->qr_stream) cudaStreamDestroy(h->qr_stream);
  if (h->cplx_buf) cudaFree(h->cplx_buf);
  delete h;
  return ITG_OK;
}

extern "C" int itg_set_stream(itg_handle* h, void* stream) {
  if (!h) return ITG_ERR_INVALID;
  h->stream = (cudaStream_t)stream;
  return ITG_OK;
}

extern "C" int itg_get_stream(itg_handle* h, void** stream) {
  if (!h || !stream) return ITG_ERR_INVALID;
  *stream = (void*)h->stream;
  return ITG_OK;
}

extern "C" int itg_set_graphs(itg_handle* h, int enable) {
  if (!h) return ITG_ERR_INVALID;
  h->use_graphs = enable != 0;
  return ITG_OK;
}

extern "C" int itg_synchronize(itg_handle* h) {
  if (!h) return ITG_ERR_INVALID;
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  return ITG_OK;
}

extern "C" const char* itg_last_error(itg_handle* h) {
  if (!h) return "null handle";
  return h->last_error.c_str();
}

extern "C" int itg_workspace_info(itg_handle* h, size_t* scratch_bytes, size_t* split_bytes,
                                  size_t* tune_bytes, int64_t* plans) {
  if (!h) return ITG_ERR_INVALID;
  if (scratch_bytes) *scratch_bytes = h->scratch_bytes;
  if (split_bytes) *split_bytes = h->split_ws_bytes;
  if (tune_bytes) *tune_bytes = h->tune_buf_bytes;
  if (plans) *plans = (int64_t)h->plans.size();
  return ITG_OK;
}

// FP64 FMA throughput of this GPU: 8 independent DFMA chains per thread,
// 8 CTAs of 256 threads per SM, a fixed trip count; the result sums the
// chains so nothing is dead code.  The roofline denominator of the plain FP64
// contraction (k_gemm_gather_f64 runs on the same DFMA pipe).
__global__ void k_dfma_rate(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" int itg_fp64_peak(itg_handle* h, double* tflops) {
  if (!h || !tflops) return ITG_ERR_INVALID;
  const int threads = 256, blocks = h->num_sms * 8, iters = 4096;
  ITG_TRY(itg_scratch_reserve(h, sizeof(double) * (size_t)threads * blocks));
  double* out = (double*)h->scratch;
  cudaEvent_t e0, e1;
  ITG_CUDA(h, cudaEventCreate(&e0));
  ITG_CUDA(h, cudaEventCreate(&e1));
  float best = 0.f;
  int st = ITG_OK;
  for (int rep = 0; rep < 4 && st == ITG_OK; ++rep) {  // the first run warms up
    cudaEventRecord(e0, h->stream);
    k_dfma_rate<<<blocks, threads, 0, h->stream>>>(out, iters, 1.0000001, 1e-7);
    cudaEventRecord(e1, h->stream);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
      st = itg_fail(h, ITG_ERR_CUDA, "FP64 rate kernel failed");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ITG_TRY(st);
  const double flop = 2.0 * 8 * iters * (double)threads * blocks;
  *tflops = best > 0.f ? flop / (best * 1e-3) / 1e12 : 0.0;
  return ITG_OK;
}

int itg_scratch_reserve(itg_handle* h, size_t bytes) {
  if (bytes <= h->scratch_bytes) return ITG_OK;
  size_t want = itg_align256(bytes + bytes / 4);
  if (h->scratch) {
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->scratch);
    h->scratch = nullptr;
    h->scratch_bytes = 0;
  }
  cudaError_t e = cudaMalloc(&h->scratch, want);
  if (e != cudaSuccess) {
    h->scratch = nullptr;
    return itg_fail(h, ITG_ERR_ALLOC, "scratch allocation of %zu bytes failed: %s", want,
                    cudaGetErrorString(e));
  }
  h->scratch_bytes = want;
  return ITG_OK;
}

// ---------------------------------------------------------------- memory
extern "C" int itg_malloc(itg_handle* h, void** ptr, size_t bytes) {
  if (!h || !ptr) return ITG_ERR_INVALID;
  *ptr = nullptr;
  if (bytes == 0) return ITG_OK;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess)
    return itg_fail(h, ITG_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
  return ITG_OK;
}

extern "C" int itg_free(itg_handle* h, void* ptr) {
  if (!h) return ITG_ERR_INVALID;
  if (ptr) ITG_CUDA(h, cudaFree(ptr));
  return ITG_OK;
}

extern "C" int itg_memcpy_h2d(itg_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (!dst && bytes) || (!src && bytes)) return ITG_ERR_INVALID;
  if (bytes == 0) return ITG_OK;
  ITG_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
  return ITG_OK;
}

extern "C" int itg_memcpy_d2h(itg_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (!dst && bytes) || (!src && bytes)) return ITG_ERR_INVALID;
  if (bytes == 0) return ITG_OK;
  ITG_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  return ITG_OK;
}

extern "C" int itg_memcpy_d2d(itg_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (!dst && bytes) || (!src && bytes)) return ITG_ERR_INVALID;
  if (bytes == 0) return ITG_OK;
  ITG_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, h->stream));
  return ITG_OK;
}

extern "C" int itg_memset_zero(itg_handle* h, void* ptr, size_t bytes) {
  if (!h || (!ptr && bytes)) return ITG_ERR_INVALID;
  if (bytes == 0) return ITG_OK;
  ITG_CUDA(h, cudaMemsetAsync(ptr, 0, bytes, h->stream));
  return ITG_OK;
}

// ------------------------------------------------------- level-1 kernels
// Grid-stride loops; HBM-bound.  Two doubles per thread per iteration where
// alignment allows would help little next to launch latency at DMRG sizes.
__global__ void k_scal(int64_t n, double a, double* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= a;
}

__global__ void k_axpby(int64_t n, double a, const double* __restrict__ x, double b,
                        double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (b == 0.0) ? a * x[i] : fma(a, x[i], b * y[i]);
}

__global__ void k_fill(int64_t n, double v, double* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

// Fixed-shape deterministic reduction: REDUCE_BLOCKS blocks write partial sums,
// one block folds them in a fixed tree order.
#define REDUCE_BLOCKS 512
#define REDUCE_THREADS 256

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  return v;
}

__global__ void k_dot_partial(int64_t n, const double* __restrict__ x,
                              const double* __restrict__ y, double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s = fma(x[i], y[i], s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_reduce_final(int np, const double* __restrict__ part, double* out, int sqrt_it) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = sqrt_it ? sqrt(s) : s;
}

namespace itg {

int dot_dev(itg_handle* h, int64_t n, const double* x, const double* y, double* out,
            double* partials) {
  int nb = itg_blocks_for(n, REDUCE_THREADS, REDUCE_BLOCKS);
  k_dot_partial<<<nb, REDUCE_THREADS, 0, h->stream>>>(n, x, y, partials);
  k_reduce_final<<<1, REDUCE_THREADS, 0, h->stream>>>(nb, partials, out, 0);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

int nrm2_dev(itg_handle* h, int64_t n, const double* x, double* out, double* partials) {
  int nb = itg_blocks_for(n, REDUCE_THREADS, REDUCE_BLOCKS);
  k_dot_partial<<<nb, REDUCE_THREADS, 0, h->stream>>>(n, x, x, partials);
  k_reduce_final<<<1, REDUCE_THREADS, 0, h->stream>>>(nb, partials, out, 1);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

}  // namespace itg

static int grid1(itg_handle* h, int64_t n) { return itg_blocks_for(n, 256, h->num_sms * 8); }

extern "C" int itg_scal(itg_handle* h, int64_t n, double a, double* x) {
  if (!h || (n > 0 && !x) || n < 0) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_scal<<<grid1(h, n), 256, 0, h->stream>>>(n, a, x);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_axpby(itg_handle* h, int64_t n, double a, const double* x, double b, double* y) {
  if (!h || (n > 0 && (!x || !y)) || n < 0) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_axpby<<<grid1(h, n), 256, 0, h->stream>>>(n, a, x, b, y);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_axpy(itg_handle* h, int64_t n, double a, const double* x, double* y) {
  return itg_axpby(h, n, a, x, 1.0, y);
}

extern "C" int itg_fill(itg_handle* h, int64_t n, double v, double* x) {
  if (!h || (n > 0 && !x) || n < 0) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_fill<<<grid1(h, n), 256, 0, h->stream>>>(n, v, x);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_dot_dev(itg_handle* h, int64_t n, const double* x, const double* y,
                           double* out) {
  if (!h || !out || n < 0 || (n > 0 && (!x || !y))) return ITG_ERR_INVALID;
  ITG_TRY(itg_scratch_reserve(h, REDUCE_BLOCKS * sizeof(double)));
  return itg::dot_dev(h, n, x, y, out, (double*)h->scratch);
}

extern "C" int itg_dot(itg_handle* h, int64_t n, const double* x, const double* y, double* result) {
  if (!h || !result) return ITG_ERR_INVALID;
  ITG_TRY(itg_scratch_reserve(h, (REDUCE_BLOCKS + 1) * sizeof(double)));
  double* part = (double*)h->scratch;
  ITG_TRY(itg::dot_dev(h, n, x, y, part + REDUCE_BLOCKS, part));
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, part + REDUCE_BLOCKS, sizeof(double),
                              cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  *result = h->pinned[0];
  return ITG_OK;
}

extern "C" int itg_nrm2(itg_handle* h, int64_t n, const double* x, double* result) {
  if (!h || !result || n < 0 || (n > 0 && !x)) return ITG_ERR_INVALID;
  ITG_TRY(itg_scratch_reserve(h, (REDUCE_BLOCKS + 1) * sizeof(double)));
  double* part = (double*)h->scratch;
  ITG_TRY(itg::nrm2_dev(h, n, x, part + REDUCE_BLOCKS, part));
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, part + REDUCE_BLOCKS, sizeof(double),
                              cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  *result = h->pinned[0];
  return ITG_OK;
}

// out[j] = X[:, j] . y for j < k.  Two-stage, fixed-order reduction: block (b, j) sums its chunk of column j
// into part[j * nb + b]; k_gemv_t_final adds the nb partials of each column.
__global__ void k_gemv_t_part(int64_t n, const double* __restrict__ X, int64_t ldx,
                              const double* __restrict__ y, double* __restrict__ part) {
  __shared__ double sh[32];
  const int nb = gridDim.x, b = blockIdx.x, j = blockIdx.y;
  const double* col = X + (int64_t)j * ldx;
  const int64_t chunk = (n + nb - 1) / nb;
  const int64_t lo = (int64_t)b * chunk, hi = lo + chunk < n ? lo + chunk : n;
  double s = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s = fma(col[i], y[i], s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[(int64_t)j * nb + b] = s;
}

__global__ void k_gemv_t_final(int nb, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[(int64_t)blockIdx.x * nb + i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// y = beta*y + X c  (k small; c on device).
__global__ void k_gemv_n(int64_t n, int k, const double* __restrict__ X, int64_t ldx,
                         const double* __restrict__ c, double beta, double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = (beta == 0.0) ? 0.0 : beta * y[i];
    for (int j = 0; j < k; ++j) s = fma(X[i + j * ldx], c[j], s);
    y[i] = s;
  }
}

extern "C" int itg_gemv_t(itg_handle* h, int64_t n, int64_t k, const double* X, int64_t ldx,
                          const double* y, double* out) {
  if (!h || n < 0 || k < 0 || ldx < n) return ITG_ERR_INVALID;
  if (k == 0) return ITG_OK;
  if (k > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "gemv_t: k=%lld too large", (long long)k);
  // enough blocks per column to fill the GPU (4 per SM over all columns),
  // each covering at least 2048 elements; partials in the handle's buffer
  int64_t nb = (4 * (int64_t)h->num_sms + k - 1) / k;
  const int64_t by_size = (n + 2047) / 2048;
  if (nb > by_size) nb = by_size;
  if (nb > ITG_GEMV_MAX_PART / k) nb = ITG_GEMV_MAX_PART / k;
  if (nb < 1) nb = 1;
  k_gemv_t_part<<<dim3((unsigned)nb, (unsigned)k), 256, 0, h->stream>>>(n, X, ldx, y, h->gemv_part);
  k_gemv_t_final<<<(unsigned)k, 256, 0, h->stream>>>((int)nb, h->gemv_part, out);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_gemv_n(itg_handle* h, int64_t n, int64_t k, const double* X, int64_t ldx,
                          const double* c, double beta, double* y) {
  if (!h || n < 0 || k < 0 || ldx < n) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_gemv_n<<<grid1(h, n), 256, 0, h->stream>>>(n, (int)k, X, ldx, c, beta, y);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

// ------------------------------------------------- Philox-4x32-10 normals
// Counter-based generator of Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3" (SC'11): ten rounds of the 4x32 Philox
// bijection keyed by the 64-bit seed.  Counter = (pair index, offset).  Each
// pair index yields two uniforms in (0,1) with 53 bits, mapped to two normals
// by Box-Muller (cos, sin).
__host__ __device__ inline void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                             uint32_t k0, uint32_t k1) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
  uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  uint32_t n0 = hi1 ^ c1 ^ k0;
  uint32_t n1 = lo1;
  uint32_t n2 = hi0 ^ c3 ^ k1;
  uint32_t n3 = lo0;
  c0 = n0; c1 = n1; c2 = n2; c3 = n3;
}

__global__ void k_random_normal(int64_t n, uint64_t seed, uint64_t offset, double* __restrict__ x) {
  const int64_t npairs = (n + 1) / 2;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npairs;
       p += (int64_t)gridDim.x * blockDim.x) {
    uint32_t c0 = (uint32_t)p, c1 = (uint32_t)((uint64_t)p >> 32);
    uint32_t c2 = (uint32_t)offset, c3 = (uint32_t)(offset >> 32);
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
      philox_round(c0, c1, c2, c3, k0, k1);
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t a = (((uint64_t)c0 << 32) | c1) >> 11;
    uint64_t b = (((uint64_t)c2 << 32) | c3) >> 11;
    double u = ((double)a + 0.5) * 0x1.0p-53;
    double v = ((double)b + 0.5) * 0x1.0p-53;
    double r = sqrt(-2.0 * log(u));
    double s, c;
    sincospi(2.0 * v, &s, &c);
    x[2 * p] = r * c;
    if (2 * p + 1 < n) x[2 * p + 1] = r * s;
  }
}

extern "C" int itg_random_normal(itg_handle* h, int64_t n, uint64_t seed, uint64_t offset,
                                 double* x) {
  if (!h || n < 0 || (n > 0 && !x)) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_random_normal<<<grid1(h, (n + 1) / 2), 256, 0, h->stream>>>(n, seed, offset, x);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}
