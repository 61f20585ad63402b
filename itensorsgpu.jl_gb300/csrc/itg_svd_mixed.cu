// Large-matrix SVD by FP32 one-sided Jacobi plus FP64-accurate refinement.
//
// GB300 runs FP32 about 60x faster than FP64, so the O(n^3) scalar work of
// Jacobi is done in FP32 and every later O(n^3) step is a matrix product run by
// the contraction engine (FP64 gather-GEMM, or the split-precision tensor-core
// path, which is FP64-accurate):
//
//  1. W32 = float(A); one-sided Jacobi sweeps in FP32 (same rotation formula as
//     the FP64 kernels; block-cyclic in shared memory for large n) until
//     |w_p.w_q| <= 1e-5 |w_p||w_q|, skipping columns below FP32 resolution.
//  2. Refine X = double(V32) as eigenvectors of G = A^T A.  Per iteration
//       R = I - X^T X,  S = X^T (G X),  l_i = s_ii / (1 - r_ii),
//       e_ij = (s_ij + l_j r_ij) / (l_j - l_i)  (i != j, |l_j - l_i| > delta),
//       e_ij = r_ij / 2                          (diagonal and clustered pairs),
//       X <- X + X E.
//     These are the first-order conditions for X(I+E) to be orthonormal
//     (E + E^T = R) and to diagonalise S (s_ij + e_ji l_j + l_i e_ij = 0), the
//     scheme of Ogita & Aishima, "Iterative refinement for symmetric eigenvalue
//     decomposition", Japan J. Indust. Appl. Math. 35 (2018).  Convergence is
//     quadratic; clustered (degenerate) pairs only get their orthogonality
//     restored, which leaves any basis of a degenerate subspace.
//     Two Newton-Schulz steps then restore X's orthonormality to rounding.
//  3. sigma_i = sqrt(max(l_i, 0)), U = A X diag(1/sigma), then one Newton-
//     Schulz step U <- U + U (I - U^T U)/2 to restore orthonormality.
// Accuracy (measured on U diag(exp(-k/20)) V^T, n = 300 ... 2048): P = sigma^2
// (what truncation uses) to ~1e-13 P_max absolute, singular values and both
// factors to FP64 accuracy above ~1e-4 sigma_max.  Below that the FP32 start
// does not resolve the singular vectors well enough for the first-order
// refinement, so they are accurate only to ~1e-13 P_max / (their P gap): a
// value within ~1e-13 P_max of the truncation threshold may land on either
// side.  X (V) stays orthonormal to rounding for every column; U = A X / S
// only where S is resolved (itg_factorize_trunc never divides by S).
// itg_svd_trunc keeps the FP64 Jacobi path for callers that need LAPACK-level
// accuracy on tiny singular values.
#include "itg_internal.cuh"

#include <optional>

#include <cmath>

namespace itg {
int contract_f64(itg_handle* h, double alpha, const double* A, int rankA, const int64_t* dimsA,
                 const int32_t* modesA, const double* B, int rankB, const int64_t* dimsB,
                 const int32_t* modesB, double beta, double* C, int rankC, const int64_t* dimsC,
                 const int32_t* modesC, int precision);
}

namespace {

constexpr int ONECTA32_MAX_N = 192;  // larger problems: one launch per step

__device__ __forceinline__ int rr_player32(int pos, int step, int np) {
  if (pos == 0) return 0;
  return ((pos - 1 + step) % (np - 1)) + 1;
}

__device__ __forceinline__ float warp_sumf(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One round-robin step of FP32 one-sided Jacobi: one CTA per column pair.
__global__ void __launch_bounds__(256)
k_jacobi32_step(float* __restrict__ W, int64_t m, int n, float* __restrict__ V, float tol, float amin,
                int step, int* __restrict__ rotated) {
  __shared__ float sh[3][8];
  const int np = n + (n & 1);
  int p = rr_player32(blockIdx.x, step, np), q = rr_player32(np - 1 - blockIdx.x, step, np);
  if (p >= n || q >= n) return;
  if (p > q) { int t = p; p = q; q = t; }
  float* wp = W + (int64_t)p * m;
  float* wq = W + (int64_t)q * m;
  float a = 0.f, b = 0.f, g = 0.f;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    float x = wp[i], y = wq[i];
    a = fmaf(x, x, a);
    b = fmaf(y, y, b);
    g = fmaf(x, y, g);
  }
  a = warp_sumf(a); b = warp_sumf(b); g = warp_sumf(g);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sh[0][warp] = a; sh[1][warp] = b; sh[2][warp] = g; }
  __syncthreads();
  a = 0.f; b = 0.f; g = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += sh[0][w]; b += sh[1][w]; g += sh[2][w]; }
  if (a <= amin || b <= amin || fabsf(g) <= tol * sqrtf(a) * sqrtf(b)) return;
  const float zeta = (b - a) / (2.f * g);
  const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
  const float c = 1.f / sqrtf(1.f + t * t), s = c * t;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    float x = wp[i], y = wq[i];
    wp[i] = c * x - s * y;
    wq[i] = s * x + c * y;
  }
  float* vp = V + (int64_t)p * n;
  float* vq = V + (int64_t)q * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    float x = vp[i], y = vq[i];
    vp[i] = c * x - s * y;
    vq[i] = s * x + c * y;
  }
  if (threadIdx.x == 0) *rotated = 1;
}

// All sweeps in one CTA (n <= 512): warps take column pairs of each
// round-robin step; __syncthreads between steps.
__global__ void __launch_bounds__(1024)
k_jacobi32_onecta(float* __restrict__ W, int64_t m, int n, float* __restrict__ V, float tol, float amin,
                  int max_sweeps, int* __restrict__ sweeps_out) {
  __shared__ int rotated;
  const int np = n + (n & 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int step = 0; step < np - 1; ++step) {
      for (int pi = warp; pi < np / 2; pi += nw) {
        int p = rr_player32(pi, step, np), q = rr_player32(np - 1 - pi, step, np);
        if (p >= n || q >= n) continue;
        if (p > q) { const int t = p; p = q; q = t; }
        float* wp = W + (int64_t)p * m;
        float* wq = W + (int64_t)q * m;
        float a = 0.f, b = 0.f, g = 0.f;
        for (int64_t i = lane; i < m; i += 32) {
          const float x = wp[i], y = wq[i];
          a = fmaf(x, x, a);
          b = fmaf(y, y, b);
          g = fmaf(x, y, g);
        }
        a = warp_sumf(a); b = warp_sumf(b); g = warp_sumf(g);
        if (a <= amin || b <= amin || fabsf(g) <= tol * sqrtf(a) * sqrtf(b)) continue;
        const float zeta = (b - a) / (2.f * g);
        const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
        const float c = 1.f / sqrtf(1.f + t * t), s = c * t;
        for (int64_t i = lane; i < m; i += 32) {
          const float x = wp[i], y = wq[i];
          wp[i] = c * x - s * y;
          wq[i] = s * x + c * y;
        }
        float* vp = V + (int64_t)p * n;
        float* vq = V + (int64_t)q * n;
        for (int i = lane; i < n; i += 32) {
          const float x = vp[i], y = vq[i];
          vp[i] = c * x - s * y;
          vq[i] = s * x + c * y;
        }
        if (lane == 0) rotated = 1;
      }
      __syncthreads();
    }
    const int r = rotated;
    __syncthreads();
    if (!r) break;
  }
  if (threadIdx.x == 0) *sweeps_out = sweep;
}

__global__ void k_to_float(const double* __restrict__ A, int64_t lda, int64_t m, int64_t n, bool transpose,
                           float* __restrict__ W) {
  const int64_t total = m * n;  // W is (rows x cols) = transpose ? (n x m) : (m x n)
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (!transpose) {
      int64_t j = t / m, i = t - j * m;
      W[t] = (float)A[i + j * lda];
    } else {
      int64_t j = t / n, i = t - j * n;  // W[i, j] = A[j, i], W rows = n
      W[t] = (float)A[j + i * lda];
    }
  }
}

__global__ void k_identity32(int n, float* __restrict__ V) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
       i += (int64_t)gridDim.x * blockDim.x)
    V[i] = (i % (n + 1) == 0) ? 1.f : 0.f;
}

__global__ void k_to_double(const float* __restrict__ x, int64_t n, double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}

// lam[i] = s_ii / (1 - r_ii) with R = I - P (P = X^T X), S given.
__global__ void k_refine_lambda(const double* __restrict__ P, const double* __restrict__ S, int n,
                                double* __restrict__ lam) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double rii = 1.0 - P[i + (int64_t)i * n];
    lam[i] = S[i + (int64_t)i * n] / (1.0 - rii);
  }
}

// E (n x n) from P = X^T X and S = X^T G X; delta = cluster threshold (absolute).
__global__ void k_refine_E(const double* __restrict__ P, const double* __restrict__ S,
                           const double* __restrict__ lam, int n, double delta, double* __restrict__ E) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nn;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / n), i = (int)(t - (int64_t)j * n);
    const double rij = (i == j ? 1.0 : 0.0) - P[t];
    double e;
    if (i == j) {
      e = 0.5 * rij;
    } else {
      // A pair is resolved only when it is separated (gap > delta) and the
      // first-order correction is small against the gap from both sides (the
      // decision reads (i, j) and (j, i), so e_ij + e_ji = r_ij holds for
      // every pair); otherwise it is treated as part of a cluster and only
      // its orthogonality is restored.  This keeps a poor FP32 start (large
      // mixing between close eigenvalues) from driving the iteration away.
      const int64_t tt = (int64_t)j + (int64_t)i * n;
      const double rji = -P[tt];
      const double d = lam[j] - lam[i];
      const double nij = S[t] + lam[j] * rij, nji = S[tt] + lam[i] * rji;
      const bool ok = fabs(d) > delta && fabs(nij) <= 0.25 * fabs(d) && fabs(nji) <= 0.25 * fabs(d);
      e = ok ? nij / d : 0.5 * rij;
    }
    E[t] = e;
  }
}

// Q = I - P  (for Newton-Schulz: U <- U + U (I - U^T U)/2, written as 0.5*(I-P))
__global__ void k_half_identity_minus(const double* __restrict__ P, int n, double* __restrict__ Q) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nn;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / n), i = (int)(t - (int64_t)j * n);
    Q[t] = 0.5 * ((i == j ? 1.0 : 0.0) - P[t]);
  }
}

// inv[j] = 1/sigma_j, 0 when sigma is numerically zero.
__global__ void k_inv_sigma(const double* __restrict__ lam, int n, double floor_sig,
                            double* __restrict__ inv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double s = sqrt(fmax(lam[i], 0.0));
    inv[i] = (s > floor_sig) ? 1.0 / s : 0.0;
  }
}

// U[:, j] *= inv[j].
__global__ void k_scale_cols(double* __restrict__ U, int64_t m, int n, const double* __restrict__ inv) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    U[t] *= inv[t / m];
}

// part[block] = max |I - P| over the block's share of the n x n matrix P
// (+inf when a NaN was seen, so that the max over the partials keeps it);
// k_max_abs then reduces the partials.
__global__ void k_max_offident(const double* __restrict__ P, int n, double* __restrict__ part) {
  __shared__ double sh[32];
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  double mx = 0.0;
  const int64_t nn = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / n), i = (int)(t - (int64_t)j * n);
    const double v = fabs((i == j ? 1.0 : 0.0) - P[t]);
    if (!(v == v)) bad = 1;
    mx = fmax(mx, v);
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) b = fmax(b, sh[i]);
    part[blockIdx.x] = bad ? __longlong_as_double(0x7ff0000000000000ll) : b;
  }
}

__global__ void k_max_abs(const double* __restrict__ x, int n, double* __restrict__ out) {
  __shared__ double sh[32];
  double mx = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, fabs(x[i]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) b = fmax(b, sh[i]);
    *out = b;
  }
}

// C (rows x cols) = alpha * op(A) * B + beta * C for column-major square-ish blocks:
// tA = 1 uses A^T.  A is (ka x ra) when transposed, B is (k x cb).
int gemm(itg_handle* h, bool tA, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
         const double* B, double beta, double* C, int precision) {
  const int64_t dA[2] = {tA ? K : M, tA ? M : K};
  const int32_t mA[2] = {tA ? 3 : 1, tA ? 1 : 3};
  const int64_t dB[2] = {K, N};
  const int32_t mB[2] = {3, 2};
  const int64_t dC[2] = {M, N};
  const int32_t mC[2] = {1, 2};
  return itg::contract_f64(h, alpha, A, 2, dA, mA, B, 2, dB, mB, beta, C, 2, dC, mC, precision);
}

}  // namespace

namespace itg {

// Mixed-precision SVD of the working matrix (rows mm >= cols nn).  Outputs the
// unsorted right vectors X (nn x nn), lam (nn, = sigma^2) and the left vectors
// Uw (mm x nn).  `Awork` is the FP64 working matrix (mm x nn, ld = mm).
int svd_mixed_core(itg_handle* h, const double* Awork, int64_t mm, int64_t nn, int precision,
                   double* X, double* lam, double* Uw, double* ws, float* ws32, int* flag,
                   int* sweeps_out, bool need_u) {
  const int n = (int)nn;
  // 1. FP32 Jacobi
  std::optional<ProfScope> prof_jacobi;
  prof_jacobi.emplace(h, ITG_KERNEL_SVD_JACOBI);
  float* W32 = ws32;
  float* V32 = ws32 + mm * nn;
  k_to_float<<<itg_blocks_for(mm * nn, 256, h->num_sms * 16), 256, 0, h->stream>>>(Awork, mm, mm, nn, false, W32);
  k_identity32<<<itg_blocks_for(nn * nn, 256, h->num_sms * 16), 256, 0, h->stream>>>(n, V32);
  ITG_CHECK_LAUNCH(h);
  const int np = n + (n & 1);
  int* hp = (int*)h->pinned;
  int sweeps = 0;
  const float tol32 = 1e-5f;
  // Columns whose norm is below 1e-7 |A|_F are FP32 rounding noise (and their
  // squared norms underflow for graded inputs such as R^T); rotations that
  // involve them are skipped, otherwise the sweeps never settle.  Their
  // directions are resolved (as far as FP64 resolves them) by the refinement.
  double fro = 0.0;
  {
    // partial sums in the workspace tail (the handle's scratch holds the caller's buffers)
    const int64_t sq = nn * nn;
    double* red = ws + 5 * sq + ((mm * nn > sq) ? mm * nn : sq) + 64;
    ITG_TRY(itg::nrm2_dev(h, mm * nn, Awork, red + 520, red));
    ITG_CUDA(h, cudaMemcpyAsync(h->pinned, red + 520, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    fro = h->pinned[0];
  }
  const float amin = (float)(1e-14 * fro * fro);
  if (n <= ONECTA32_MAX_N) {
    k_jacobi32_onecta<<<1, 1024, 0, h->stream>>>(W32, mm, n, V32, tol32, amin, 30, flag);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(hp, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    sweeps = hp[0];
  } else {
    int st = ITG_ERR_UNSUPPORTED;
    if (h->jacobi_mode == 0 || h->jacobi_mode == 3)
      st = itg::jacobi_blocked<float>(h, W32, mm, n, V32, tol32, amin, 30, flag, &sweeps);
    else if (h->jacobi_mode == 2)
      st = itg::jacobi_persistent<float>(h, W32, mm, n, V32, tol32, amin, 30, flag, &sweeps);
    if (st != ITG_OK && st != ITG_ERR_NOTCONVERGED && st != ITG_ERR_UNSUPPORTED) return st;
    if (st == ITG_ERR_UNSUPPORTED) {
      // one launch per round-robin step (queued back to back)
      sweeps = 0;
      for (; sweeps < 30; ++sweeps) {
        ITG_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
        for (int step = 0; step < np - 1; ++step)
          k_jacobi32_step<<<np / 2, 256, 0, h->stream>>>(W32, mm, n, V32, tol32, amin, step, flag);
        ITG_CHECK_LAUNCH(h);
        ITG_CUDA(h, cudaMemcpyAsync(hp, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        ITG_CUDA(h, cudaStreamSynchronize(h->stream));
        if (hp[0] == 0) break;
      }
      sweeps++;
    }
  }
  *sweeps_out = sweeps;
  prof_jacobi.reset();
  ProfScope prof_refine(h, ITG_KERNEL_SVD_REFINE);
  // 2. refinement of X on G = A^T A
  // G P Q E Xn (nn^2 each) | S (max(mm*nn, nn^2), also the copy of U) | max slot
  double* G = ws;
  double* P = G + nn * nn;
  double* Q = P + nn * nn;
  double* E = Q + nn * nn;
  double* Xn = E + nn * nn;
  double* S = Xn + nn * nn;
  double* mx = S + ((mm * nn > nn * nn) ? mm * nn : nn * nn);
  k_to_double<<<itg_blocks_for(nn * nn, 256, h->num_sms * 16), 256, 0, h->stream>>>(V32, nn * nn, X);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(gemm(h, true, nn, nn, mm, 1.0, Awork, Awork, 0.0, G, precision));  // G = A^T A
  const int gb = itg_blocks_for(nn * nn, 256, h->num_sms * 16);
  for (int it = 0; it < 3; ++it) {
    ITG_TRY(gemm(h, true, nn, nn, nn, 1.0, X, X, 0.0, P, precision));   // P = X^T X
    ITG_TRY(gemm(h, false, nn, nn, nn, 1.0, G, X, 0.0, Q, precision));  // Q = G X
    ITG_TRY(gemm(h, true, nn, nn, nn, 1.0, X, Q, 0.0, S, precision));   // S = X^T G X
    k_refine_lambda<<<itg_blocks_for(nn, 256, 64), 256, 0, h->stream>>>(P, S, n, lam);
    k_max_abs<<<1, 1024, 0, h->stream>>>(lam, n, mx);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(h->pinned, mx, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    const double lmax = h->pinned[0] > 0.0 ? h->pinned[0] : 1.0;
    // pairs closer than the current eigenvector error are treated as one
    // cluster (only their orthogonality is restored): 1e-6 relative after the
    // FP32 start, then 1e-10
    const double delta = (it == 0 ? 1e-6 : 1e-10) * lmax;
    k_refine_E<<<gb, 256, 0, h->stream>>>(P, S, lam, n, delta, E);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(Xn, X, sizeof(double) * nn * nn, cudaMemcpyDeviceToDevice, h->stream));
    ITG_TRY(gemm(h, false, nn, nn, nn, 1.0, X, E, 1.0, Xn, precision));  // X <- X + X E
    ITG_CUDA(h, cudaMemcpyAsync(X, Xn, sizeof(double) * nn * nn, cudaMemcpyDeviceToDevice, h->stream));
  }
  // Newton-Schulz steps X <- X + X (I - X^T X)/2 until X^T X is the identity
  // to NS_TARGET (each step squares the deviation).  Pairs whose gap is below
  // the products' rounding (eigenvalues under ~1e-8 lambda_max) leave
  // first-order errors in E's antisymmetric part, hence second-order loss of
  // orthogonality (up to ~1e-5) after the refinement.  X is the orthonormal
  // factor of the bond split, and the sweep builds its environments on that
  // assumption: a deviation delta shows up as a relative energy error of about
  // delta times the chain length, so it is driven to rounding level here.
  constexpr int NS_MAX = 6;
  constexpr double NS_TARGET = 1e-14;
  const int64_t sq_ws = nn * nn;
  double* red = ws + 5 * sq_ws + ((mm * nn > sq_ws) ? mm * nn : sq_ws) + 64;
  double dev = 0.0;
  for (int it = 0;; ++it) {
    ITG_TRY(gemm(h, true, nn, nn, nn, 1.0, X, X, 0.0, P, precision));
    // partials in the workspace tail (512 blocks), then the max over them
    k_max_offident<<<512, 256, 0, h->stream>>>(P, n, red);
    k_max_abs<<<1, 1024, 0, h->stream>>>(red, 512, mx + 1);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(h->pinned, mx + 1, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    dev = h->pinned[0];
    if (!(dev > NS_TARGET) || it == NS_MAX) break;
    k_half_identity_minus<<<gb, 256, 0, h->stream>>>(P, n, Q);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(Xn, X, sizeof(double) * nn * nn, cudaMemcpyDeviceToDevice, h->stream));
    ITG_TRY(gemm(h, false, nn, nn, nn, 1.0, X, Q, 1.0, Xn, precision));
    ITG_CUDA(h, cudaMemcpyAsync(X, Xn, sizeof(double) * nn * nn, cudaMemcpyDeviceToDevice, h->stream));
  }
  // final eigenvalues from the refined X (P = X^T X is current)
  ITG_TRY(gemm(h, false, nn, nn, nn, 1.0, G, X, 0.0, Q, precision));
  ITG_TRY(gemm(h, true, nn, nn, nn, 1.0, X, Q, 0.0, S, precision));
  k_refine_lambda<<<itg_blocks_for(nn, 256, 64), 256, 0, h->stream>>>(P, S, n, lam);
  k_max_abs<<<1, 1024, 0, h->stream>>>(lam, n, mx);
  ITG_CHECK_LAUNCH(h);
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, mx, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  // Safeguard: the first-order refinement needs a start close enough to the
  // eigenvectors; when it was not (X not orthonormal to 1e-12 after the
  // Newton-Schulz steps, or not finite) the caller redoes the problem with
  // FP64 Jacobi.
  if (!(dev <= 1e-12) || !std::isfinite(h->pinned[0])) return ITG_ERR_NOTCONVERGED;
  if (!need_u) return ITG_OK;  // the caller keeps only the right vectors
  const double smax = sqrt(h->pinned[0] > 0.0 ? h->pinned[0] : 0.0);
  // 3. U = A X diag(1/sigma), one Newton-Schulz step
  ITG_TRY(gemm(h, false, mm, nn, nn, 1.0, Awork, X, 0.0, Uw, precision));
  double* inv = E;  // E is free after the refinement
  // columns with sigma < 1e-7 sigma_max are not resolved (A X / sigma is noise
  // there); they are left zero so that they cannot pollute the Newton-Schulz step
  k_inv_sigma<<<itg_blocks_for(nn, 256, 64), 256, 0, h->stream>>>(lam, n, 1e-7 * smax, inv);
  k_scale_cols<<<itg_blocks_for(mm * nn, 256, h->num_sms * 16), 256, 0, h->stream>>>(Uw, mm, n, inv);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(gemm(h, true, nn, nn, mm, 1.0, Uw, Uw, 0.0, P, precision));  // P = U^T U
  k_half_identity_minus<<<gb, 256, 0, h->stream>>>(P, n, Q);
  ITG_CHECK_LAUNCH(h);
  // Uw <- Uw + Uw Q  (through a copy: the product must not alias its operand)
  double* Ucp = S;  // S is free now; needs mm x nn: ensured by the caller's sizing
  ITG_CUDA(h, cudaMemcpyAsync(Ucp, Uw, sizeof(double) * mm * nn, cudaMemcpyDeviceToDevice, h->stream));
  ITG_TRY(gemm(h, false, mm, nn, nn, 1.0, Ucp, Q, 1.0, Uw, precision));
  return ITG_OK;
}

// One Newton-Schulz step on an isometry L (rows x cols, ld rows, rows >= cols):
// L <- L + L (I - L^T L) / 2, which squares its deviation from orthonormality.
// The factor that leaves the bond split (Q times the refined eigenvectors)
// carries the rounding of the Householder application, O(rows eps).  L^T L is
// measured with FP64 products: split products resolve it only to about
// 2^-48 sqrt(rows) (1e-13 at rows = 512), which is what this step removes;
// the correction L (I - L^T L) / 2 is of that size, so its own product may be
// split.  ws: 2 cols^2 doubles, tmp: rows x cols doubles (L's copy; the
// product must not alias its operand).
int ns_polish(itg_handle* h, double* L, int64_t rows, int64_t cols, double* ws, double* tmp, int precision) {
  if (rows <= 0 || cols <= 0) return ITG_OK;
  double* P = ws;
  double* Q = ws + cols * cols;
  // heuristic FP64 tiles: the shapes change from bond to bond, and timing the
  // three tile variants of each new shape would cost more than the product
  const bool tune = h->autotune;
  h->autotune = false;
  const int st = gemm(h, true, cols, cols, rows, 1.0, L, L, 0.0, P, ITG_PREC_FP64);
  h->autotune = tune;
  ITG_TRY(st);
  k_half_identity_minus<<<itg_blocks_for(cols * cols, 256, h->num_sms * 16), 256, 0, h->stream>>>(P, (int)cols, Q);
  ITG_CHECK_LAUNCH(h);
  ITG_CUDA(h, cudaMemcpyAsync(tmp, L, sizeof(double) * rows * cols, cudaMemcpyDeviceToDevice, h->stream));
  return gemm(h, false, rows, cols, cols, 1.0, tmp, Q, 1.0, L, precision);
}

size_t svd_mixed_ws_doubles(int64_t mm, int64_t nn) {
  const int64_t sq = nn * nn;
  const int64_t s_slot = (mm * nn > sq) ? mm * nn : sq;
  return (size_t)(5 * sq + s_slot + 64 + 528);
}

}  // namespace itg
