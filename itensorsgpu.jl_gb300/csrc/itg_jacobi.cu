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
//   c = 1/sqrt(1 + t^2), s = c t;  skip when |g| <= tol sqrt(a) sqrt(b); a
//   sweep has converged when no rotated pair had |g| > conv_tol(tol) sqrt(a b).
//
// Columns move between SMs from step to step, so every load of W and V goes
// through L2 (ld.global.cg) and stores bypass L1 (st.global.cg); the barrier
// fences before arriving and after leaving.  The barrier wait is bounded by
// %globaltimer (the handle's wait limit, 4 s by default): a block that times
// out raises a status word that makes every other waiting block leave too,
// and the host reports ITG_ERR_TIMEOUT.
#include "itg_internal.cuh"

#include <cmath>
#include <cstdint>
#include <type_traits>

namespace {

constexpr int JP_THREADS = 256;
constexpr int JP_WARPS = JP_THREADS / 32;

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
__device__ bool jp_grid_sync(unsigned* count, unsigned* gen, int* status, unsigned nblocks,
                             unsigned long long wait_ns) {
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
        if (jp_timer() - t0 > wait_ns) {
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
k_jacobi_persist(T* __restrict__ W, int64_t m, int n, T* __restrict__ V, T tol, T tol_conv, T amin, T amin_conv,
                 int max_sweeps,
                 int* aux, unsigned long long wait_ns) {
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
        if (t == 0 && a > amin_conv && b > amin_conv && fabs(g) > tol_conv * sqrt(a) * sqrt(b))
          __stcg(rot + sweep, 1);
      }
      if (!jp_grid_sync(count, gen, status, gridDim.x, wait_ns)) {
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

// ------------------------------------------------------ blocked step
// Block-cyclic one-sided Jacobi: the columns form blocks of WB; step `step`
// of a sweep pairs the blocks round robin (nbp slots), one CTA per block
// pair.  The CTA stages the pair's 2 WB columns in shared memory, rotates
// every cross pair (i in block I, j in block J; WB rounds of WB disjoint
// pairs), accumulates the rotations into a 2WB x 2WB matrix Q, writes the
// columns back and applies Q to the pair's columns of V.  The first step of
// a sweep also rotates the pairs inside each block (a full round robin over
// the 2 WB columns), so every column pair is visited once per sweep.  Same
// rotation formula and skip rule as the element-wise kernels; a step moves
// 2 WB columns per CTA through shared memory instead of two per CTA.
constexpr int JB_THREADS = 512;

// Convergence threshold of a sweep (see the element-wise FP64 kernels): in
// FP64, pairs rotated with |g| <= 4 tol sqrt(a b) sit at the rounding floor of
// the dot product and do not keep the sweep loop running.  The FP32 start of
// the mixed method keeps its plain rule (its tol is far above FP32 rounding).
template <class T>
__host__ __device__ inline T conv_tol(T tol) {
  return sizeof(T) == 8 ? T(4) * tol : tol;
}

// Short FP64 columns (m <= JB_SMALL_M) run one warp per pair (THREADS =
// 32 WB): the pair's sums then come from warp shuffles alone, which saves a
// shared-memory reduction and one of the two barriers of every round
// (measured at n = 378: 104 -> 82 ms per FP64 split; the FP32 Jacobi of the
// mixed method was slower that way, 20.4 -> 22.7 ms, and keeps 512 threads).
constexpr int64_t JB_SMALL_M = 1024;

template <class T, int WB, int THREADS>
__global__ void __launch_bounds__(THREADS)
k_jacobi_block_step(T* __restrict__ W, int64_t m, int n, T* __restrict__ V, T tol, T tol_conv, T amin,
                    T amin_conv, int step, int first, int* __restrict__ rotated) {
  constexpr int C2 = 2 * WB;              // local columns
  constexpr int TP = THREADS / WB;        // threads per pair
  constexpr int WPG = TP / 32;            // warps per pair group
  extern __shared__ __align__(16) unsigned char jb_smem[];
  T* cols = (T*)jb_smem;                  // [C2][m]
  T* Q = cols + (int64_t)C2 * m;          // [C2][C2], column-major
  T* red = Q + C2 * C2;                   // [WB][WPG][3]
  __shared__ int any, major;
  const int nb = (n + WB - 1) / WB, nbp = nb + (nb & 1);
  const int bi = jp_player(blockIdx.x, step, nbp), bj = jp_player(nbp - 1 - blockIdx.x, step, nbp);
  const int t = threadIdx.x;
  auto gcol = [&](int c) -> int {  // global column of local c, or -1
    const int blk = c < WB ? bi : bj;
    const int gc = blk * WB + (c < WB ? c : c - WB);
    return (blk < nb && gc < n) ? gc : -1;
  };
  if (t == 0) any = major = 0;
  int gcs[C2];
#pragma unroll
  for (int c = 0; c < C2; ++c) gcs[c] = gcol(c);
  // Stage the pair's columns: a thread issues its loads of all 2 WB columns
  // (two rows at a time) before storing any of them, so the L2 latency is paid
  // once per 4 WB loads instead of once per element.
  for (int64_t i0 = t; i0 < m; i0 += 2 * THREADS) {
    const int64_t i1 = i0 + THREADS;
    T v0[C2], v1[C2];
#pragma unroll
    for (int c = 0; c < C2; ++c) {
      v0[c] = gcs[c] >= 0 ? W[(int64_t)gcs[c] * m + i0] : T(0);
      v1[c] = (gcs[c] >= 0 && i1 < m) ? W[(int64_t)gcs[c] * m + i1] : T(0);
    }
#pragma unroll
    for (int c = 0; c < C2; ++c) {
      cols[(int64_t)c * m + i0] = v0[c];
      if (i1 < m) cols[(int64_t)c * m + i1] = v1[c];
    }
  }
  for (int i = t; i < C2 * C2; i += THREADS) Q[i] = (i % (C2 + 1) == 0) ? T(1) : T(0);
  __syncthreads();
  const int g = t / TP, lt = t % TP, wg = lt / 32, lane = t & 31;
  const int rounds = first ? C2 - 1 : WB;
  for (int r = 0; r < rounds; ++r) {
    int p, q;
    if (first) {
      p = jp_player(g, r, C2);
      q = jp_player(C2 - 1 - g, r, C2);
    } else {
      p = g;
      q = WB + (g + r) % WB;
    }
    if (p > q) {
      const int tmp = p;
      p = q;
      q = tmp;
    }
    T* xp = cols + (int64_t)p * m;
    T* xq = cols + (int64_t)q * m;
    // the pair's column slices: four independent loads per iteration, two
    // accumulator sets (m fits in shared memory, so 32-bit indices)
    const int mi = (int)m;
    T a = 0, b = 0, gg = 0, a1 = 0, b1 = 0, g1 = 0;
    int i = lt;
    for (; i + 3 * TP < mi; i += 4 * TP) {
      const T x0 = xp[i], y0 = xq[i], x1 = xp[i + TP], y1 = xq[i + TP];
      const T x2 = xp[i + 2 * TP], y2 = xq[i + 2 * TP], x3 = xp[i + 3 * TP], y3 = xq[i + 3 * TP];
      a = fma(x0, x0, a);
      b = fma(y0, y0, b);
      gg = fma(x0, y0, gg);
      a1 = fma(x1, x1, a1);
      b1 = fma(y1, y1, b1);
      g1 = fma(x1, y1, g1);
      a = fma(x2, x2, a);
      b = fma(y2, y2, b);
      gg = fma(x2, y2, gg);
      a1 = fma(x3, x3, a1);
      b1 = fma(y3, y3, b1);
      g1 = fma(x3, y3, g1);
    }
    for (; i < mi; i += TP) {
      const T x = xp[i], y = xq[i];
      a = fma(x, x, a);
      b = fma(y, y, b);
      gg = fma(x, y, gg);
    }
    a += a1;
    b += b1;
    gg += g1;
    a = jp_warp_sum(a);
    b = jp_warp_sum(b);
    gg = jp_warp_sum(gg);
    if constexpr (WPG > 1) {
      if (lane == 0) {
        red[(g * WPG + wg) * 3 + 0] = a;
        red[(g * WPG + wg) * 3 + 1] = b;
        red[(g * WPG + wg) * 3 + 2] = gg;
      }
      __syncthreads();
      a = 0;
      b = 0;
      gg = 0;
#pragma unroll
      for (int w = 0; w < WPG; ++w) {
        a += red[(g * WPG + w) * 3 + 0];
        b += red[(g * WPG + w) * 3 + 1];
        gg += red[(g * WPG + w) * 3 + 2];
      }
    }
    const bool rot = !(a <= amin || b <= amin || fabs(gg) <= tol * sqrt(a) * sqrt(b));
    if (rot) {
      const T zeta = (b - a) / (T(2) * gg);
      const T tt = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
      const T c = T(1) / sqrt(T(1) + tt * tt), sn = c * tt;
      int j = lt;
      for (; j + 3 * TP < mi; j += 4 * TP) {
        T x[4], y[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          x[u] = xp[j + u * TP];
          y[u] = xq[j + u * TP];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          xp[j + u * TP] = c * x[u] - sn * y[u];
          xq[j + u * TP] = sn * x[u] + c * y[u];
        }
      }
      for (; j < mi; j += TP) {
        const T x = xp[j], y = xq[j];
        xp[j] = c * x - sn * y;
        xq[j] = sn * x + c * y;
      }
      if (lt < C2) {
        const T x = Q[lt + p * C2], y = Q[lt + q * C2];
        Q[lt + p * C2] = c * x - sn * y;
        Q[lt + q * C2] = sn * x + c * y;
      }
      if (lt == 0) {
        any = 1;
        if (a > amin_conv && b > amin_conv && fabs(gg) > tol_conv * sqrt(a) * sqrt(b)) major = 1;
      }
    }
    __syncthreads();  // columns, Q and red are reused by the next round
  }
  if (!any) return;  // block-uniform (read after the last barrier)
  for (int c = 0; c < C2; ++c) {
    const int gc = gcol(c);
    if (gc < 0) continue;
    const T* src = cols + (int64_t)c * m;
    T* dst = W + (int64_t)gc * m;
    for (int64_t i = t; i < m; i += THREADS) dst[i] = src[i];
  }
  // V[:, cols] <- V[:, cols] Q, one row per thread; the next row's loads are
  // issued before the current row is combined and stored
  int row = t;
  T v[C2];
#pragma unroll
  for (int c = 0; c < C2; ++c) v[c] = (gcs[c] >= 0 && row < n) ? V[row + (int64_t)gcs[c] * n] : T(0);
  for (; row < n; row += THREADS) {
    const int nrow = row + THREADS;
    T vn[C2];
#pragma unroll
    for (int c = 0; c < C2; ++c) vn[c] = (gcs[c] >= 0 && nrow < n) ? V[nrow + (int64_t)gcs[c] * n] : T(0);
#pragma unroll
    for (int c = 0; c < C2; ++c) {
      if (gcs[c] < 0) continue;
      T s = 0;
#pragma unroll
      for (int d = 0; d < C2; ++d) s = fma(v[d], Q[d + c * C2], s);
      V[row + (int64_t)gcs[c] * n] = s;
    }
#pragma unroll
    for (int c = 0; c < C2; ++c) v[c] = vn[c];
  }
  if (t == 0 && major) *rotated = 1;
}

// FP32 block step with 16-byte accesses (m and n multiples of 4, n <= m):
// the rotations of k_jacobi_block_step<float> in the same order, with the
// pair's columns staged, summed and rotated four rows at a time.  V's columns
// are staged in shared memory (the column buffer is free after the write-back)
// and each thread applies Q to four rows x four columns with its four Q
// columns held in registers; the per-output sums run over d in the same order
// as the element-wise kernel's.
template <int WB, int THREADS>
__global__ void __launch_bounds__(THREADS)
k_jacobi_block_step_f4(float* __restrict__ W, int64_t m, int n, float* __restrict__ V, float tol, float tol_conv,
                       float amin, float amin_conv, int step, int first, int* __restrict__ rotated) {
  constexpr int C2 = 2 * WB;          // local columns
  constexpr int TP = THREADS / WB;    // threads per pair
  constexpr int WPG = TP / 32;        // warps per pair group
  constexpr int NG = C2 / 4;          // output column groups of the V update
  extern __shared__ __align__(16) unsigned char jb_smem[];
  float* cols = (float*)jb_smem;       // [C2][m]
  float* Q = cols + (int64_t)C2 * m;   // [C2][C2], column-major
  float* red = Q + C2 * C2;            // [WB][WPG][3]
  __shared__ int any, major;
  const int nb = (n + WB - 1) / WB, nbp = nb + (nb & 1);
  const int bi = jp_player(blockIdx.x, step, nbp), bj = jp_player(nbp - 1 - blockIdx.x, step, nbp);
  const int t = threadIdx.x;
  const int m4 = (int)(m >> 2), n4 = n >> 2;
  float4* cols4 = reinterpret_cast<float4*>(cols);
  float4* W4 = reinterpret_cast<float4*>(W);
  float4* V4 = reinterpret_cast<float4*>(V);
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  int gcs[C2];
#pragma unroll
  for (int c = 0; c < C2; ++c) {
    const int blk = c < WB ? bi : bj;
    const int gc = blk * WB + (c < WB ? c : c - WB);
    gcs[c] = (blk < nb && gc < n) ? gc : -1;
  }
  if (t == 0) any = major = 0;
  for (int i = t; i < m4; i += THREADS) {
    float4 v[C2];
#pragma unroll
    for (int c = 0; c < C2; ++c) v[c] = gcs[c] >= 0 ? W4[(int64_t)gcs[c] * m4 + i] : zero4;
#pragma unroll
    for (int c = 0; c < C2; ++c) cols4[(int64_t)c * m4 + i] = v[c];
  }
  for (int i = t; i < C2 * C2; i += THREADS) Q[i] = (i % (C2 + 1) == 0) ? 1.f : 0.f;
  __syncthreads();
  const int g = t / TP, lt = t % TP, wg = lt / 32, lane = t & 31;
  const int rounds = first ? C2 - 1 : WB;
  for (int r = 0; r < rounds; ++r) {
    int p, q;
    if (first) {
      p = jp_player(g, r, C2);
      q = jp_player(C2 - 1 - g, r, C2);
    } else {
      p = g;
      q = WB + (g + r) % WB;
    }
    if (p > q) {
      const int tmp = p;
      p = q;
      q = tmp;
    }
    float4* xp = cols4 + (int64_t)p * m4;
    float4* xq = cols4 + (int64_t)q * m4;
    float a = 0.f, b = 0.f, gg = 0.f, a1 = 0.f, b1 = 0.f, g1 = 0.f;
    int i = lt;
    for (; i + TP < m4; i += 2 * TP) {
      const float4 x0 = xp[i], y0 = xq[i], x1 = xp[i + TP], y1 = xq[i + TP];
      a = fmaf(x0.x, x0.x, a);
      b = fmaf(y0.x, y0.x, b);
      gg = fmaf(x0.x, y0.x, gg);
      a1 = fmaf(x0.y, x0.y, a1);
      b1 = fmaf(y0.y, y0.y, b1);
      g1 = fmaf(x0.y, y0.y, g1);
      a = fmaf(x0.z, x0.z, a);
      b = fmaf(y0.z, y0.z, b);
      gg = fmaf(x0.z, y0.z, gg);
      a1 = fmaf(x0.w, x0.w, a1);
      b1 = fmaf(y0.w, y0.w, b1);
      g1 = fmaf(x0.w, y0.w, g1);
      a = fmaf(x1.x, x1.x, a);
      b = fmaf(y1.x, y1.x, b);
      gg = fmaf(x1.x, y1.x, gg);
      a1 = fmaf(x1.y, x1.y, a1);
      b1 = fmaf(y1.y, y1.y, b1);
      g1 = fmaf(x1.y, y1.y, g1);
      a = fmaf(x1.z, x1.z, a);
      b = fmaf(y1.z, y1.z, b);
      gg = fmaf(x1.z, y1.z, gg);
      a1 = fmaf(x1.w, x1.w, a1);
      b1 = fmaf(y1.w, y1.w, b1);
      g1 = fmaf(x1.w, y1.w, g1);
    }
    if (i < m4) {
      const float4 x0 = xp[i], y0 = xq[i];
      a = fmaf(x0.x, x0.x, a);
      b = fmaf(y0.x, y0.x, b);
      gg = fmaf(x0.x, y0.x, gg);
      a1 = fmaf(x0.y, x0.y, a1);
      b1 = fmaf(y0.y, y0.y, b1);
      g1 = fmaf(x0.y, y0.y, g1);
      a = fmaf(x0.z, x0.z, a);
      b = fmaf(y0.z, y0.z, b);
      gg = fmaf(x0.z, y0.z, gg);
      a1 = fmaf(x0.w, x0.w, a1);
      b1 = fmaf(y0.w, y0.w, b1);
      g1 = fmaf(x0.w, y0.w, g1);
    }
    a += a1;
    b += b1;
    gg += g1;
    a = jp_warp_sum(a);
    b = jp_warp_sum(b);
    gg = jp_warp_sum(gg);
    if constexpr (WPG > 1) {
      if (lane == 0) {
        red[(g * WPG + wg) * 3 + 0] = a;
        red[(g * WPG + wg) * 3 + 1] = b;
        red[(g * WPG + wg) * 3 + 2] = gg;
      }
      __syncthreads();
      a = 0.f;
      b = 0.f;
      gg = 0.f;
#pragma unroll
      for (int w = 0; w < WPG; ++w) {
        a += red[(g * WPG + w) * 3 + 0];
        b += red[(g * WPG + w) * 3 + 1];
        gg += red[(g * WPG + w) * 3 + 2];
      }
    }
    const bool rot = !(a <= amin || b <= amin || fabsf(gg) <= tol * sqrtf(a) * sqrtf(b));
    if (rot) {
      const float zeta = (b - a) / (2.f * gg);
      const float tt = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
      const float c = 1.f / sqrtf(1.f + tt * tt), sn = c * tt;
      for (int j = lt; j < m4; j += TP) {
        const float4 x = xp[j], y = xq[j];
        xp[j] = make_float4(c * x.x - sn * y.x, c * x.y - sn * y.y, c * x.z - sn * y.z, c * x.w - sn * y.w);
        xq[j] = make_float4(sn * x.x + c * y.x, sn * x.y + c * y.y, sn * x.z + c * y.z, sn * x.w + c * y.w);
      }
      if (lt < C2) {
        const float x = Q[lt + p * C2], y = Q[lt + q * C2];
        Q[lt + p * C2] = c * x - sn * y;
        Q[lt + q * C2] = sn * x + c * y;
      }
      if (lt == 0) {
        any = 1;
        if (a > amin_conv && b > amin_conv && fabsf(gg) > tol_conv * sqrtf(a) * sqrtf(b)) major = 1;
      }
    }
    __syncthreads();  // columns, Q and red are reused by the next round
  }
  if (!any) return;  // block-uniform (read after the last barrier)
#pragma unroll
  for (int c = 0; c < C2; ++c) {
    if (gcs[c] < 0) continue;
    const float4* src = cols4 + (int64_t)c * m4;
    float4* dst = W4 + (int64_t)gcs[c] * m4;
    for (int i = t; i < m4; i += THREADS) dst[i] = src[i];
  }
  __syncthreads();  // the column buffer now takes V's columns
  for (int i = t; i < n4; i += THREADS) {
    float4 v[C2];
#pragma unroll
    for (int c = 0; c < C2; ++c) v[c] = gcs[c] >= 0 ? V4[(int64_t)gcs[c] * n4 + i] : zero4;
#pragma unroll
    for (int c = 0; c < C2; ++c) cols4[(int64_t)c * n4 + i] = v[c];
  }
  __syncthreads();
  // V[:, cols] <- V[:, cols] Q: output columns 4 og .. 4 og + 3, rows 4 r4 .. 4 r4 + 3
  const int og = t % NG;
  int ogc[4];  // global columns of this thread's outputs (-1: none)
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = 4 * og + j;
    const int blk = c < WB ? bi : bj;
    const int gc = blk * WB + (c < WB ? c : c - WB);
    ogc[j] = (blk < nb && gc < n) ? gc : -1;
  }
  float qr[C2][4];
#pragma unroll
  for (int d = 0; d < C2; ++d)
#pragma unroll
    for (int j = 0; j < 4; ++j) qr[d][j] = Q[d + (4 * og + j) * C2];
  for (int r4 = t / NG; r4 < n4; r4 += THREADS / NG) {
    float4 acc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] = zero4;
#pragma unroll
    for (int d = 0; d < C2; ++d) {
      const float4 x = cols4[(int64_t)d * n4 + r4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc[j].x = fmaf(x.x, qr[d][j], acc[j].x);
        acc[j].y = fmaf(x.y, qr[d][j], acc[j].y);
        acc[j].z = fmaf(x.z, qr[d][j], acc[j].z);
        acc[j].w = fmaf(x.w, qr[d][j], acc[j].w);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (ogc[j] >= 0) V4[(int64_t)ogc[j] * n4 + r4] = acc[j];
  }
  if (t == 0 && major) *rotated = 1;
}

// Self-test of the grid barrier's timeout path: every block arrives at a
// barrier that counts one participant more than the grid has, so the count
// is never met; each block waits until the limit, the first to give up raises
// the status word and all of them leave.  No block spins past the limit.
__global__ void k_grid_barrier_selftest(int* aux, unsigned long long wait_ns) {
  const bool ok = jp_grid_sync((unsigned*)aux, (unsigned*)aux + 1, aux + 2, gridDim.x + 1, wait_ns);
  if (threadIdx.x == 0 && !ok) atomicAdd(aux + 3, 1);
}

}  // namespace

namespace itg {

int grid_barrier_selftest(itg_handle* h, int* status, int* blocks_out) {
  ITG_TRY(itg_scratch_reserve(h, 8 * sizeof(int)));
  int* aux = (int*)h->scratch;
  ITG_CUDA(h, cudaMemsetAsync(aux, 0, 8 * sizeof(int), h->stream));
  k_grid_barrier_selftest<<<2, 32, 0, h->stream>>>(aux, (unsigned long long)h->wait_ns);
  ITG_CHECK_LAUNCH(h);
  int* hp = (int*)h->pinned;
  ITG_CUDA(h, cudaMemcpyAsync(hp, aux, 4 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  *status = hp[2];
  *blocks_out = hp[3];
  return ITG_OK;
}

int jacobi_aux_ints(int max_sweeps) { return 8 + max_sweeps; }

// Runs up to max_sweeps sweeps on W (m x n) accumulating into V (n x n, set
// by the caller).  *sweeps = sweeps run; ITG_ERR_NOTCONVERGED when the limit
// was hit (results usable), ITG_ERR_UNSUPPORTED when the device cannot run a
// cooperative launch (the caller then uses per-step launches).
template <class T, int RC>
int launch_persist(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, T amin_conv, int max_sweeps,
                   int* aux) {
  const T tol_conv = conv_tol(tol);
  int per_sm = 0;
  ITG_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi_persist<T, RC>, JP_THREADS, 0));
  if (per_sm < 1) return ITG_ERR_UNSUPPORTED;
  if (per_sm > 4) per_sm = 4;  // fewer arrivals per barrier
  const int np = n + (n & 1);
  int64_t grid = (int64_t)h->num_sms * per_sm;
  if ((int64_t)np / 2 < grid) grid = np / 2;
  if (grid < 1) grid = 1;
  unsigned long long wait_ns = h->wait_ns;
  void* args[] = {(void*)&W,          (void*)&m,          (void*)&n,    (void*)&V,
                  (void*)&tol,        (void*)&tol_conv,   (void*)&amin, (void*)&amin_conv,
                  (void*)&max_sweeps, (void*)&aux,        (void*)&wait_ns};
  ITG_CUDA(h, cudaLaunchCooperativeKernel((const void*)k_jacobi_persist<T, RC>, dim3((unsigned)grid),
                                          dim3(JP_THREADS), args, 0, h->stream));
  return ITG_OK;
}

template <class T>
int jacobi_persistent(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, int max_sweeps, int* aux,
                      int* sweeps, T amin_conv) {
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device);
  if (!coop) return ITG_ERR_UNSUPPORTED;
  ITG_CUDA(h, cudaMemsetAsync(aux, 0, sizeof(int) * jacobi_aux_ints(max_sweeps), h->stream));
  int st;
  if (m <= 4 * JP_THREADS) st = launch_persist<T, 4>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, aux);
  else if (m <= 8 * JP_THREADS) st = launch_persist<T, 8>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, aux);
  else if (m <= 16 * JP_THREADS) st = launch_persist<T, 16>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, aux);
  else st = launch_persist<T, 0>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, aux);
  if (st != ITG_OK) return st;
  int* hp = (int*)h->pinned;
  ITG_CUDA(h, cudaMemcpyAsync(hp, aux, sizeof(int) * 4, cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (hp[2] != 0 || hp[3] < 0)
    return itg_fail(h, ITG_ERR_TIMEOUT, "Jacobi grid barrier timed out (n=%d)", n);
  *sweeps = hp[3] > max_sweeps ? max_sweeps : hp[3];
  return hp[3] > max_sweeps ? ITG_ERR_NOTCONVERGED : ITG_OK;
}

template <class T, int WB>
size_t jb_smem_bytes(int64_t m) {
  return sizeof(T) * ((size_t)2 * WB * m + (size_t)4 * WB * WB + (size_t)WB * (JB_THREADS / WB / 32) * 3);
}

template <class T, int WB, int THREADS>
int jb_run_t(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, T amin_conv, int max_sweeps, int* flag,
             int* sweeps) {
  const size_t smem = jb_smem_bytes<T, WB>(m);
  // FP32 with 16-byte aligned columns of W and V (and V's columns fitting in
  // the column buffer): the vectorised step
  const bool vec = std::is_same<T, float>::value && m % 4 == 0 && n % 4 == 0 && n <= m &&
                   ((uintptr_t)W % 16) == 0 && ((uintptr_t)V % 16) == 0;
  static bool attr = false;
  if (!attr) {
    ITG_CUDA(h, cudaFuncSetAttribute(k_jacobi_block_step<T, WB, THREADS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    if constexpr (std::is_same<T, float>::value)
      ITG_CUDA(h, cudaFuncSetAttribute(k_jacobi_block_step_f4<WB, THREADS>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  const int nb = (n + WB - 1) / WB, nbp = nb + (nb & 1);
  int* hp = (int*)h->pinned;
  for (int sw = 0; sw < max_sweeps; ++sw) {
    ITG_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
    for (int step = 0; step < nbp - 1; ++step) {
      if constexpr (std::is_same<T, float>::value) {
        if (vec) {
          k_jacobi_block_step_f4<WB, THREADS><<<nbp / 2, THREADS, smem, h->stream>>>(
              W, m, n, V, tol, conv_tol(tol), amin, amin_conv, step, step == 0, flag);
          continue;
        }
      }
      k_jacobi_block_step<T, WB, THREADS><<<nbp / 2, THREADS, smem, h->stream>>>(W, m, n, V, tol, conv_tol(tol),
                                                                                 amin, amin_conv, step, step == 0,
                                                                                 flag);
    }
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(hp, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hp[0] == 0) {
      *sweeps = sw + 1;
      return ITG_OK;
    }
  }
  *sweeps = max_sweeps;
  return ITG_ERR_NOTCONVERGED;
}

template <class T, int WB>
int jb_run(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, T amin_conv, int max_sweeps, int* flag,
           int* sweeps) {
  if (sizeof(T) == 8 && m <= JB_SMALL_M)
    return jb_run_t<T, WB, 32 * WB>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, flag, sweeps);
  return jb_run_t<T, WB, JB_THREADS>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, flag, sweeps);
}

// Blocked Jacobi with the widest block whose column pair fits in 200 KB of
// shared memory; ITG_ERR_UNSUPPORTED when not even 2 + 2 columns fit.
template <class T>
int jacobi_blocked(itg_handle* h, T* W, int64_t m, int n, T* V, T tol, T amin, int max_sweeps, int* flag,
                   int* sweeps, T amin_conv) {
  constexpr size_t LIM = 200 * 1024;
  if (n < 2) {
    *sweeps = 0;
    return ITG_OK;
  }
  // jacobi_mode 3 keeps the blocks at 4 columns (half the shared memory per CTA, more CTAs per SM)
  if (h->jacobi_mode != 3 && jb_smem_bytes<T, 8>(m) <= LIM && n >= 64)
    return jb_run<T, 8>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, flag, sweeps);
  if (jb_smem_bytes<T, 4>(m) <= LIM) return jb_run<T, 4>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, flag, sweeps);
  if (jb_smem_bytes<T, 2>(m) <= LIM) return jb_run<T, 2>(h, W, m, n, V, tol, amin, amin_conv, max_sweeps, flag, sweeps);
  return ITG_ERR_UNSUPPORTED;
}

template int jacobi_blocked<float>(itg_handle*, float*, int64_t, int, float*, float, float, int, int*, int*, float);
template int jacobi_blocked<double>(itg_handle*, double*, int64_t, int, double*, double, double, int, int*, int*,
                                     double);

template int jacobi_persistent<float>(itg_handle*, float*, int64_t, int, float*, float, float, int, int*, int*,
                                       float);
template int jacobi_persistent<double>(itg_handle*, double*, int64_t, int, double*, double, double, int, int*,
                                        int*, double);

}  // namespace itg
