// Persistent one-sided Jacobi: every sweep of a large problem in one
// cooperative launch.
//
// The per-step formulation (one launch per round-robin step, 2n launches per
// sweep) is bound by launch latency and by re-fetching the pair's columns
// cold each step.  Here one launch runs all sweeps: the steps are separated
// by a grid-wide barrier, and the kernel leaves when a sweep rotated nothing.
// CTAs own column pairs (CTA b takes pairs b, b + gridDim.x, ... of the
// step; a pair's columns are cached in registers between the dot products and
// the rotation).  Same pairing (Brent-Luk round robin), rotation formula and
// skip rule as the one-CTA and per-step kernels of itg_factor.cu:
//   zeta = (b - a) / (2g), t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)),
//   c = 1/sqrt(1 + t^2), s = c t;  skip when |g| <= tol sqrt(a) sqrt(b).
//
// Columns move between SMs from step to step, so every load of W and V goes
// through L2 (ld.global.cg) and stores bypass L1 (st.global.cg); the barrier
// fences before arriving and after leaving.  The barrier wait is bounded by
// %globaltimer (4 s): a block that times out raises a status word that makes
// every other waiting block leave too, and the host reports ITG_ERR_TIMEOUT.
#include "itg_internal.cuh"

#include <cmath>

namespace {

constexpr int JP_THREADS = 256;
constexpr int JP_WARPS = JP_THREADS / 32;
constexpr unsigned long long JP_WAIT_NS = 4000000000ull;

__device__ __forceinline__ unsigned long long jp_timer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int jp_player(int pos, int step, int np) {
  if (pos == 0) return 0;
  return ((pos - 1 + step) % (np - 1)) + 1;
}

template <class T>
__device__ __forceinline__ T jp_warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Grid-wide barrier over `nblocks` co-resident blocks (count / generation
// words in global memory).  Returns false for every thread of the block when
// the wait timed out or another block reported a timeout.
__device__ bool jp_grid_sync(unsigned* count, unsigned* gen, int* status, unsigned nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = 1;
    const unsigned g = *(volatile unsigned*)gen;
    __threadfence();
    const unsigned arrived = atomicAdd(count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      const unsigned long long t0 = jp_timer();
      while (*(volatile unsigned*)gen == g) {
        if (*(volatile int*)status) {
          good = 0;
          break;
        }
        if (jp_timer() - t0 > JP_WAIT_NS) {
          atomicExch(status, 1);
          good = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Block-wide sums of three values (every thread gets the same totals: the
// per-warp partials are added in a fixed order).
template <class T>
__device__ __forceinline__ void jp_block_sum3(T& a, T& b, T& g, T (*sh)[JP_WARPS]) {
  a = jp_warp_sum(a);
  b = jp_warp_sum(b);
  g = jp_warp_sum(g);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sh[0][warp] = a;
    sh[1][warp] = b;
    sh[2][warp] = g;
  }
  __syncthreads();
  a = 0;
  b = 0;
  g = 0;
#pragma unroll
  for (int w = 0; w < JP_WARPS; ++w) {
    a += sh[0][w];
    b += sh[1][w];
    g += sh[2][w];
  }
  __syncthreads();  // sh is reused by the next pair
}

// aux (ints, zeroed by the host): [0] barrier count, [1] generation,
// [2] timeout status, [3] sweeps run (max_sweeps + 1: limit hit, -1: timed
// out), [8 + s] "sweep s rotated".
// One CTA per column pair (CTA b takes pairs b, b + gridDim.x, ... of the
// step).  RC = column elements cached per thread (m <= JP_THREADS * RC), so a
// pair's columns are read once per step; RC = 0 streams them (any m).
template <class T, int RC>
__global__ void __launch_bounds__(JP_THREADS)
k_jacobi_persist(T* __restrict__ W, int64_t m, int n, T* __restrict__ V, T tol, T amin, int max_sweeps,
                 int* aux) {
  __shared__ T sh[3][JP_WARPS];
  unsigned* count = (unsigned*)aux;
  unsigned* gen = (unsigned*)aux + 1;
  int* status = aux + 2;
  int* rot = aux + 8;
  const int np = n + (n & 1), npairs = np / 2;
  const int t = threadIdx.x;
  int done = max_sweeps + 1;  // not converged within max_sweeps
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    for (int step = 0; step < np - 1; ++step) {
      for (int pi = blockIdx.x; pi < npairs; pi += gridDim.x) {
        int p = jp_player(pi, step, np), q = jp_player(np - 1 - pi, step, np);
        if (p >= n || q >= n) continue;  // block-uniform
        if (p > q) {
          const int tmp = p;
          p = q;
          q = tmp;
        }
        T* wp = W + (int64_t)p * m;
        T* wq = W + (int64_t)q * m;
        T a = 0, b = 0, g = 0;
        T xr[RC > 0 ? RC : 1], yr[RC > 0 ? RC : 1];
        if (RC > 0) {
#pragma unroll
          for (int r = 0; r < RC; ++r) {
            const int64_t i = t + (int64_t)r * JP_THREADS;
            xr[r] = i < m ? __ldcg(wp + i) : T(0);
            yr[r] = i < m ? __ldcg(wq + i) : T(0);
          }
#pragma unroll
          for (int r = 0; r < RC; ++r) {
            a = fma(xr[r], xr[r], a);
            b = fma(yr[r], yr[r], b);
            g = fma(xr[r], yr[r], g);
          }
        } else {
          for (int64_t i = t; i < m; i += JP_THREADS) {
            const T x = __ldcg(wp + i), y = __ldcg(wq + i);
            a = fma(x, x, a);
            b = fma(y, y, b);
            g = fma(x, y, g);
          }
        }
        jp_block_sum3(a, b, g, sh);
        if (a <= amin || b <= amin || fabs(g) <= tol * sqrt(a) * sqrt(b)) continue;  // block-uniform
        const T zeta = (b - a) / (T(2) * g);
        const T tt = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T c = T(1) / sqrt(T(1) + tt * tt), s = c * tt;
        if (RC > 0) {
#pragma unroll
          for (int r = 0; r < RC; ++r) {
            const int64_t i = t + (int64_t)r * JP_THREADS;
            if (i < m) {
              __stcg(wp + i, c * xr[r] - s * yr[r]);
              __stcg(wq + i, s * xr[r] + c * yr[r]);
            }
          }
        } else {
          for (int64_t i = t; i < m; i += JP_THREADS) {
            const T x = __ldcg(wp + i), y = __ldcg(wq + i);
            __stcg(wp + i, c * x - s * y);
            __stcg(wq + i, s * x + c * y);
          }
        }
        T* vp = V + (int64_t)p * n;
        T* vq = V + (int64_t)q * n;
        for (int i = t; i < n; i += JP_THREADS) {
          const T x = __ldcg(vp + i), y = __ldcg(vq + i);
          __stcg(vp + i, c * x - s * y);
          __stcg(vq + i, s * x + c * y);
        }
        if (t == 0) __stcg(rot + sweep, 1);
      }
      if (!jp_grid_sync(count, gen, status, gridDim.x)) {
        done = -1;
        break;
      }
    }
    if (done < 0) break;
    if (__ldcg(rot + sweep) == 0) {
      done = sweep + 1;
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) aux[3] = done;
}

}  // namespace

namespace itg {

int jacobi_aux_ints(int max_sweeps) { return 8 + max_sweeps; }

// Runs up to max_sweeps sweeps on W (m x n) accumulating into V (n x n, set
// by the caller).  *sweeps = sweeps run; ITG_ERR_NOTCONVERGED when the limit
// was hit (results usable), ITG_ERR_UNSUPPORTED when the device cannot run a
// cooperative launch (the caller then uses per-step launches).
template <class T, int RC>
int launch_persist(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, int max_sweeps, int* aux) {
  int per_sm = 0;
  ITG_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi_persist<T, RC>, JP_THREADS, 0));
  if (per_sm < 1) return ITG_ERR_UNSUPPORTED;
  if (per_sm > 4) per_sm = 4;  // fewer arrivals per barrier
  const int np = n + (n & 1);
  int64_t grid = (int64_t)h->num_sms * per_sm;
  if ((int64_t)np / 2 < grid) grid = np / 2;
  if (grid < 1) grid = 1;
  void* args[] = {(void*)&W,   (void*)&m,          (void*)&n,  (void*)&V,
                  (void*)&tol, (void*)&amin, (void*)&max_sweeps, (void*)&aux};
  ITG_CUDA(h, cudaLaunchCooperativeKernel((const void*)k_jacobi_persist<T, RC>, dim3((unsigned)grid),
                                          dim3(JP_THREADS), args, 0, h->stream));
  return ITG_OK;
}

template <class T>
int jacobi_persistent(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, int max_sweeps, int* aux,
                      int* sweeps) {
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device);
  if (!coop) return ITG_ERR_UNSUPPORTED;
  ITG_CUDA(h, cudaMemsetAsync(aux, 0, sizeof(int) * jacobi_aux_ints(max_sweeps), h->stream));
  int st;
  if (m <= 4 * JP_THREADS) st = launch_persist<T, 4>(h, W, m, n, V, tol, amin, max_sweeps, aux);
  else if (m <= 8 * JP_THREADS) st = launch_persist<T, 8>(h, W, m, n, V, tol, amin, max_sweeps, aux);
  else if (m <= 16 * JP_THREADS) st = launch_persist<T, 16>(h, W, m, n, V, tol, amin, max_sweeps, aux);
  else st = launch_persist<T, 0>(h, W, m, n, V, tol, amin, max_sweeps, aux);
  if (st != ITG_OK) return st;
  int* hp = (int*)h->pinned;
  ITG_CUDA(h, cudaMemcpyAsync(hp, aux, sizeof(int) * 4, cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (hp[2] != 0 || hp[3] < 0)
    return itg_fail(h, ITG_ERR_TIMEOUT, "Jacobi grid barrier timed out (n=%d)", n);
  *sweeps = hp[3] > max_sweeps ? max_sweeps : hp[3];
  return hp[3] > max_sweeps ? ITG_ERR_NOTCONVERGED : ITG_OK;
}

template int jacobi_persistent<float>(itg_handle*, float*, int64_t, int, float*, float, float, int, int*, int*);
template int jacobi_persistent<double>(itg_handle*, double*, int64_t, int, double*, double, double, int, int*,
                                        int*);

}  // namespace itg
