// Factorisations: on-device truncation (K6), one-sided Jacobi SVD (K5),
// symmetric eigendecomposition through the shifted SVD, and the thin Householder QR (K7).
#include "itg_internal.cuh"

#include <cmath>

// ============================================================== truncation
// One thread walks the spectrum in the same sequential order as the CPU
// rules it restates, so both give bit-identical sums.  n <= 2*chi is a few
// thousand values: tens of microseconds, once per bond.
__global__ void k_truncate(const double* __restrict__ P, int64_t n, int64_t maxdim,
                           int64_t mindim, double cutoff, int absoluteCutoff, int doRelCutoff,
                           int legacy, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int64_t origm = n;
  double truncerr = 0.0, docut = 0.0;
  int64_t keep = 1;
  if (origm == 0) {
    out[0] = 0; out[1] = 0; out[2] = 0;
    return;
  }
  if (maxdim <= 0 || maxdim > origm) maxdim = origm;
  if (!legacy) {
    // ITensors (NDTensors) CPU rule: cumulative discarded weight.
    if (origm == 1) {
      out[0] = 1; out[1] = 0.0; out[2] = fabs(P[0]) / 2;
      return;
    }
    const double sgn = (P[0] < 0.0) ? -1.0 : 1.0;
    // trailing negative weights count as zero
    int64_t lastpos = origm;  // values at index >= lastpos are treated as 0
    for (int64_t i = origm - 1; i >= 0; --i) {
      if (sgn * P[i] >= 0.0) break;
      lastpos = i;
    }
#define PV(i) ((i) >= lastpos ? 0.0 : sgn * P[(i)])
    if (mindim < 1) mindim = 1;
    int64_t nn = origm;
    while (nn > maxdim) { truncerr += PV(nn - 1); nn--; }
    if (absoluteCutoff) {
      while (PV(nn - 1) <= cutoff && nn > mindim) { truncerr += PV(nn - 1); nn--; }
    } else {
      double scale = 1.0;
      if (doRelCutoff) {
        scale = 0.0;
        for (int64_t i = 0; i < origm; ++i) scale += PV(i);
        if (scale == 0.0) scale = 1.0;
      }
      const double thr = __dmul_rn(cutoff, scale);
      while ((__dadd_rn(truncerr, PV(nn - 1)) <= thr) && nn > mindim) {
        truncerr += PV(nn - 1);
        nn--;
      }
      truncerr /= scale;
    }
    if (nn < 1) nn = 1;
    if (nn < origm) {
      docut = (PV(nn - 1) + PV(nn)) / 2;
      if (fabs(PV(nn - 1) - PV(nn)) < __dmul_rn(1e-3, PV(nn - 1)))
        docut = __dadd_rn(docut, __dmul_rn(1e-3, PV(nn - 1)));
    }
#undef PV
    keep = nn;
  } else {
    // src/tensor/cutruncate.jl:1-93, step by step.
    if (mindim < 1) mindim = 1;
    if (mindim > maxdim) mindim = maxdim;
    double maxP = P[0];
    for (int64_t i = 1; i < origm; ++i) maxP = fmax(maxP, P[i]);
    if (maxP == 0.0) {
      out[0] = 1; out[1] = 0.0; out[2] = 0.0;
      return;
    }
    if (origm == 1) {
      out[0] = 1; out[1] = 0.0; out[2] = maxP / 2;
      return;
    }
#define RP(i) (signbit(P[(i)]) ? 0.0 : P[(i)])
    int64_t nn = origm;
    if (nn > maxdim) {
      for (int64_t i = 0; i < nn - maxdim; ++i) truncerr += RP(i);  // head sum, as written
      nn = maxdim;
    }
    // cut_ind: first index whose value is strictly below the threshold
    // (cuBLAS iamax over the +-2/0 flag vector), 0 when there is none.
    int64_t cut_ind = 0;
    if (absoluteCutoff) {
      for (int64_t i = 0; i < origm; ++i)
        if (RP(i) - cutoff < 0.0) { cut_ind = i; break; }
      nn = min(maxdim, origm - cut_ind);
      nn = max(nn, mindim);
      for (int64_t i = cut_ind; i < origm; ++i) truncerr += RP(i);
    } else {
      double scale = 1.0;
      if (doRelCutoff) {
        scale = 0.0;
        for (int64_t i = 0; i < origm; ++i) scale += P[i];
        scale = scale > 0.0 ? scale : 1.0;
      }
      for (int64_t i = 0; i < origm; ++i)
        if (__dsub_rn(__dadd_rn(RP(i), truncerr), __dmul_rn(cutoff, scale)) < 0.0) { cut_ind = i; break; }
      if (cut_ind > 0) {
        for (int64_t i = cut_ind; i < origm; ++i) truncerr += RP(i);
      } else {
        for (int64_t i = 0; i < maxdim; ++i) truncerr += RP(i);
      }
      nn = min(maxdim, origm - cut_ind);
      nn = max(nn, mindim);
      truncerr = (scale == 0.0) ? 0.0 : truncerr / scale;
    }
#undef RP
    if (nn < 1) nn = 1;
    if (nn < origm) {
      docut = (P[nn - 1] + P[nn]) / 2;
      if (fabs(P[nn - 1] - P[nn]) < __dmul_rn(1e-3, P[nn - 1]))
        docut = __dadd_rn(docut, __dmul_rn(1e-3, P[nn - 1]));
    }
    keep = nn;
  }
  out[0] = (double)keep;
  out[1] = truncerr;
  out[2] = docut;
}

namespace itg {
int truncate_dev(itg_handle* h, const double* P, int64_t n, int64_t maxdim, int64_t mindim,
                 double cutoff, int absoluteCutoff, int doRelCutoff, int legacy_gpu, double* out3) {
  k_truncate<<<1, 32, 0, h->stream>>>(P, n, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff,
                                      legacy_gpu, out3);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}
}  // namespace itg

static int read_out3(itg_handle* h, const double* out3, int64_t* n_keep, double* truncerr,
                     double* docut) {
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, out3, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (n_keep) *n_keep = (int64_t)h->pinned[0];
  if (truncerr) *truncerr = h->pinned[1];
  if (docut) *docut = h->pinned[2];
  return ITG_OK;
}

extern "C" int itg_truncate(itg_handle* h, const double* P, int64_t n, int64_t maxdim,
                            int64_t mindim, double cutoff, int absoluteCutoff, int doRelCutoff,
                            int legacy_gpu, int64_t* n_keep, double* truncerr, double* docut) {
  if (!h || n < 0 || (n > 0 && !P)) return ITG_ERR_INVALID;
  ITG_TRY(itg_scratch_reserve(h, 4 * sizeof(double)));
  double* out3 = (double*)h->scratch;
  if (n == 0) {
    if (n_keep) *n_keep = 0;
    if (truncerr) *truncerr = 0;
    if (docut) *docut = 0;
    return ITG_OK;
  }
  ITG_TRY(itg::truncate_dev(h, P, n, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff, legacy_gpu, out3));
  return read_out3(h, out3, n_keep, truncerr, docut);
}

// ============================================================ Jacobi SVD
// One-sided Jacobi (Hestenes 1958; Demmel & Veselic 1992) on the columns of the
// m x n working matrix W (m >= n), accumulating the rotations in V (n x n).
// Pairs follow the round-robin ("circle") ordering of Brent & Luk, so each of
// the n'-1 steps of a sweep rotates n'/2 disjoint column pairs in parallel
// (n' = n rounded up to even; the extra slot is a bye).
//
// Rotation for the pair (p, q) with a = |w_p|^2, b = |w_q|^2, g = w_p.w_q:
//   zeta = (b - a) / (2g), t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)),
//   c = 1/sqrt(1 + t^2), s = c t;  w_p <- c w_p - s w_q,  w_q <- s w_p + c w_q.
// A pair is skipped when |g| <= tol * sqrt(a b).

__device__ __forceinline__ int rr_player(int pos, int step, int np) {
  if (pos == 0) return 0;
  return ((pos - 1 + step) % (np - 1)) + 1;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// A pair is rotated when |g| > tol sqrt(a b); the sweep counts as converged
// when no rotated pair had |g| > JACOBI_CONV * tol sqrt(a b).  Rotations in
// between polish pairs near the rounding floor of the dot product (about
// eps sqrt(m) relative, i.e. tol itself), where they can repeat without
// making progress; they must not keep the sweep loop running.
// Pairs involving a column with squared norm <= amin_conv (rounding noise of
// a rank-deficient input, see jacobi_run) are rotated like any other pair
// but never keep the loop running either.
constexpr double JACOBI_CONV = 4.0;

__device__ __forceinline__ bool jacobi_significant(double a, double b, double g, double tol, double amin_conv) {
  return a > amin_conv && b > amin_conv && fabs(g) > JACOBI_CONV * tol * sqrt(a) * sqrt(b);
}

__device__ __forceinline__ bool jacobi_rotation(double a, double b, double g, double tol, double& c, double& s) {
  if (a == 0.0 || b == 0.0) return false;
  if (fabs(g) <= tol * sqrt(a) * sqrt(b)) return false;
  double zeta = (b - a) / (2.0 * g);
  double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  c = 1.0 / sqrt(1.0 + t * t);
  s = c * t;
  return true;
}

// Small problems: the whole sweep loop in one CTA; warps take pairs.
__global__ void __launch_bounds__(1024)
k_jacobi_onecta(double* __restrict__ W, int64_t m, int n, double* __restrict__ V, double tol, double amin_conv,
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
        int p = rr_player(pi, step, np), q = rr_player(np - 1 - pi, step, np);
        if (p >= n || q >= n) continue;
        if (p > q) { int t = p; p = q; q = t; }
        double* wp = W + (int64_t)p * m;
        double* wq = W + (int64_t)q * m;
        double a = 0, b = 0, g = 0;
        for (int64_t i = lane; i < m; i += 32) {
          double x = wp[i], y = wq[i];
          a = fma(x, x, a);
          b = fma(y, y, b);
          g = fma(x, y, g);
        }
        a = warp_sum(a); b = warp_sum(b); g = warp_sum(g);
        double c, s;
        if (jacobi_rotation(a, b, g, tol, c, s)) {
          for (int64_t i = lane; i < m; i += 32) {
            double x = wp[i], y = wq[i];
            wp[i] = c * x - s * y;
            wq[i] = s * x + c * y;
          }
          double* vp = V + (int64_t)p * n;
          double* vq = V + (int64_t)q * n;
          for (int i = lane; i < n; i += 32) {
            double x = vp[i], y = vq[i];
            vp[i] = c * x - s * y;
            vq[i] = s * x + c * y;
          }
          if (lane == 0 && jacobi_significant(a, b, g, tol, amin_conv)) rotated = 1;
        }
      }
      __syncthreads();
    }
    int r = rotated;
    __syncthreads();
    if (!r) break;
  }
  if (threadIdx.x == 0) *sweeps_out = sweep;
}

// Large problems: one launch per round-robin step, one CTA per pair.
__global__ void __launch_bounds__(256)
k_jacobi_step(double* __restrict__ W, int64_t m, int n, double* __restrict__ V, double tol, double amin_conv,
              int step, int* __restrict__ rotated) {
  __shared__ double sh[3][8];
  const int np = n + (n & 1);
  const int pi = blockIdx.x;
  int p = rr_player(pi, step, np), q = rr_player(np - 1 - pi, step, np);
  if (p >= n || q >= n) return;
  if (p > q) { int t = p; p = q; q = t; }
  double* wp = W + (int64_t)p * m;
  double* wq = W + (int64_t)q * m;
  double a = 0, b = 0, g = 0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    double x = wp[i], y = wq[i];
    a = fma(x, x, a);
    b = fma(y, y, b);
    g = fma(x, y, g);
  }
  a = warp_sum(a); b = warp_sum(b); g = warp_sum(g);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sh[0][warp] = a; sh[1][warp] = b; sh[2][warp] = g; }
  __syncthreads();
  a = 0; b = 0; g = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += sh[0][w]; b += sh[1][w]; g += sh[2][w]; }
  double c, s;
  if (!jacobi_rotation(a, b, g, tol, c, s)) return;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    double x = wp[i], y = wq[i];
    wp[i] = c * x - s * y;
    wq[i] = s * x + c * y;
  }
  double* vp = V + (int64_t)p * n;
  double* vq = V + (int64_t)q * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double x = vp[i], y = vq[i];
    vp[i] = c * x - s * y;
    vq[i] = s * x + c * y;
  }
  if (threadIdx.x == 0 && jacobi_significant(a, b, g, tol, amin_conv)) *rotated = 1;
}

__global__ void k_identity(int n, double* __restrict__ V) {
  int64_t nn = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
       i += (int64_t)gridDim.x * blockDim.x)
    V[i] = (i % (n + 1) == 0) ? 1.0 : 0.0;
}

__global__ void k_col_norms(const double* __restrict__ W, int64_t m, double* __restrict__ sig) {
  __shared__ double sh[32];
  const double* w = W + (int64_t)blockIdx.x * m;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) s = fma(w[i], w[i], s);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
    sig[blockIdx.x] = sqrt(t);
  }
}

// Rescale every column of V (n x ncols) to unit norm: the accumulated plane
// rotations drift column norms by O(sweeps * n * eps).
__global__ void k_unit_cols(double* __restrict__ V, int64_t n) {
  __shared__ double sh[32];
  __shared__ double f;
  double* v = V + (int64_t)blockIdx.x * n;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma(v[i], v[i], s);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
    f = t > 0.0 ? 1.0 / sqrt(t) : 1.0;
  }
  __syncthreads();
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) v[i] *= f;
}

// Stable descending rank of each value (ties by index): order[rank] = j.
__global__ void k_rank_desc(const double* __restrict__ sig, int n, double shift,
                            int* __restrict__ order, double* __restrict__ S,
                            double* __restrict__ P, int square) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double v = sig[j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      double u = sig[i];
      r += (u > v) || (u == v && i < j);
    }
    order[r] = j;
    double sv = v - shift;
    S[r] = sv;
    P[r] = square ? sv * sv : sv;
  }
}

// out[:, r] = src[:, order[r]] * (scale_by_inv_sig ? 1/sig : 1) for r < ncols.
__global__ void k_gather_cols(const double* __restrict__ src, int64_t rows, const int* __restrict__ order,
                              const double* __restrict__ sig, int inv_scale, int ncols,
                              double* __restrict__ dst, int64_t ldd) {
  const int r = blockIdx.y;
  if (r >= ncols) return;
  const int j = order[r];
  double f = 1.0;
  if (inv_scale) {
    double sv = sig[j];
    f = (sv > 0.0) ? 1.0 / sv : 0.0;
  }
  const double* s = src + (int64_t)j * rows;
  double* d = dst + (int64_t)r * ldd;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = s[i] * f;
}

__global__ void k_copy_matrix(const double* __restrict__ A, int64_t lda, int64_t m, int64_t n,
                              double* __restrict__ W, double diag_shift) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = t / m, i = t - j * m;
    double v = A[i + j * lda];
    if (i == j) v += diag_shift;
    W[t] = v;
  }
}

// Row-sum bound of |A| (Gershgorin) for the eigen shift.
__global__ void k_gershgorin(const double* __restrict__ A, int64_t lda, int64_t n, double* out) {
  __shared__ double sh[32];
  double best = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double s = 0.0;
    for (int64_t j = 0; j < n; ++j) s += fabs(A[i + j * lda]);
    best = fmax(best, s);
  }
  for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) b = fmax(b, sh[i]);
    *out = b;
  }
}

namespace {

// ------------------------------------------------ QR preconditioning
// One-sided Jacobi converges in far fewer sweeps on R^T, where A = Q R, than on
// A itself when A's singular values are graded (the QR-preconditioned Jacobi
// of Drmac & Veselic, "New fast and accurate Jacobi SVD algorithm I", SIAM J.
// Matrix Anal. Appl. 29 (2008)): for A = U diag(exp(-k/20)) V^T, 10 sweeps
// instead of about 30.  With B = R^T = U_B S V_B^T: A = (Q V_B) S U_B^T.
//
// Householder step j of A (m x n, column-major): every CTA reads column j
// (never written during the step) and forms the same reflector
//   beta = -sign(alpha) |x|, tau = (beta - alpha) / beta, v = x / (alpha - beta), v_j = 1;
// CTA 0 stores v, tau and beta; CTA c > 0 applies I - tau v v^T to column j + c.
template <int T>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < T / 32; ++w) s += sh[w];
  __syncthreads();
  return s;
}

__global__ void __launch_bounds__(256)
k_house_step(double* __restrict__ A, int64_t m, int j, double* __restrict__ Vh, double* __restrict__ tau,
             double* __restrict__ rdiag) {
  __shared__ double sh[8];
  const double* x = A + (int64_t)j * m;
  const double alpha = x[j];
  double s2 = 0.0;
  for (int64_t i = j + 1 + threadIdx.x; i < m; i += 256) s2 = fma(x[i], x[i], s2);
  s2 = block_sum<256>(s2, sh);
  double tj = 0.0, beta = alpha, scale = 0.0;
  if (s2 > 0.0) {
    beta = -copysign(hypot(alpha, sqrt(s2)), alpha);
    tj = (beta - alpha) / beta;
    scale = 1.0 / (alpha - beta);
  }
  if (blockIdx.x == 0) {
    double* v = Vh + (int64_t)j * m;
    for (int64_t i = threadIdx.x; i < m; i += 256) v[i] = i < j ? 0.0 : (i == j ? 1.0 : x[i] * scale);
    if (threadIdx.x == 0) {
      tau[j] = tj;
      rdiag[j] = beta;
    }
    return;
  }
  if (tj == 0.0) return;
  double* col = A + (int64_t)(j + blockIdx.x) * m;
  double w = 0.0;
  for (int64_t i = j + 1 + threadIdx.x; i < m; i += 256) w = fma(x[i] * scale, col[i], w);
  w = block_sum<256>(w, sh) + col[j];
  const double f = tj * w;
  for (int64_t i = j + threadIdx.x; i < m; i += 256) col[i] -= f * (i == j ? 1.0 : x[i] * scale);
}

}  // namespace

namespace itg {
void house_step_launch(itg_handle* h, double* A, int64_t m, int j, int ncta, double* Vh, double* tau,
                       double* rdiag) {
  k_house_step<<<(unsigned)ncta, 256, 0, h->stream>>>(A, m, j, Vh, tau, rdiag);
}
}  // namespace itg

namespace {

// B = R^T (n x n, lower triangular) from the factored A (R above the diagonal, diagonal in rdiag).
__global__ void k_build_rt(const double* __restrict__ A, int64_t m, int n, const double* __restrict__ rdiag,
                           double* __restrict__ B) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / n), i = (int)(t - (int64_t)k * n);  // B(i, k) = R(k, i)
    B[t] = k < i ? A[k + (int64_t)i * m] : (k == i ? rdiag[i] : 0.0);
  }
}


constexpr int JACOBI_MAX_SWEEPS = 60;
constexpr int JACOBI_AUX_INTS = 8 + JACOBI_MAX_SWEEPS;
constexpr int64_t ONECTA_MAX_N = 192;

// Runs Jacobi on W (m x n, m >= n) with V = I.  Returns ITG_ERR_NOTCONVERGED
// (results still usable) when the sweep limit is hit.  flag_dev: at least
// JACOBI_AUX_INTS device ints.
int jacobi_run(itg_handle* h, double* W, int64_t m, int64_t n, double* V, int* flag_dev,
               int* sweeps_done) {
  k_identity<<<itg_blocks_for(n * n, 256, h->num_sms * 8), 256, 0, h->stream>>>((int)n, V);
  ITG_CHECK_LAUNCH(h);
  const double tol = 2.220446049250313e-16 * sqrt((double)m);
  if (n <= 1) { *sweeps_done = 0; return ITG_OK; }
  // Columns whose norm falls below 10 eps |W|_F carry only rounding noise of
  // the rotations that touched them (a rank-deficient W, e.g. the bond
  // matrices of a direct sum of two MPS): their pairs keep being rotated (so
  // that W's columns stay as orthogonal as rounding allows) but do not count
  // towards convergence, otherwise the sweeps never settle.
  ITG_TRY(itg::nrm2_dev(h, m * n, W, h->gemv_part + 1024, h->gemv_part));
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, h->gemv_part + 1024, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  const double fro = h->pinned[0];
  const double amin_conv = (10.0 * 2.220446049250313e-16 * fro) * (10.0 * 2.220446049250313e-16 * fro);
  if (n <= ONECTA_MAX_N) {
    k_jacobi_onecta<<<1, 1024, 0, h->stream>>>(W, m, (int)n, V, tol, amin_conv, JACOBI_MAX_SWEEPS, flag_dev);
    ITG_CHECK_LAUNCH(h);
    int* hp = (int*)h->pinned;
    ITG_CUDA(h, cudaMemcpyAsync(hp, flag_dev, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    *sweeps_done = hp[0];
    return hp[0] >= JACOBI_MAX_SWEEPS ? ITG_ERR_NOTCONVERGED : ITG_OK;
  }
  if (h->jacobi_mode == 0 || h->jacobi_mode == 3) {
    const int st = itg::jacobi_blocked<double>(h, W, m, (int)n, V, tol, 0.0, JACOBI_MAX_SWEEPS, flag_dev,
                                               sweeps_done, amin_conv);
    if (st != ITG_ERR_UNSUPPORTED) return st;
  } else if (h->jacobi_mode == 2) {
    const int st = itg::jacobi_persistent<double>(h, W, m, (int)n, V, tol, 0.0, JACOBI_MAX_SWEEPS, flag_dev,
                                                  sweeps_done, amin_conv);
    if (st != ITG_ERR_UNSUPPORTED) return st;
  }
  // per-step launches (devices without cooperative launch)
  const int np = (int)(n + (n & 1));
  int* hp = (int*)h->pinned;
  for (int sweep = 0; sweep < JACOBI_MAX_SWEEPS; ++sweep) {
    ITG_CUDA(h, cudaMemsetAsync(flag_dev, 0, sizeof(int), h->stream));
    for (int step = 0; step < np - 1; ++step)
      k_jacobi_step<<<np / 2, 256, 0, h->stream>>>(W, m, (int)n, V, tol, amin_conv, step, flag_dev);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(hp, flag_dev, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hp[0] == 0) { *sweeps_done = sweep + 1; return ITG_OK; }
  }
  *sweeps_done = JACOBI_MAX_SWEEPS;
  return ITG_ERR_NOTCONVERGED;
}

}  // namespace

namespace itg {
int svd_mixed_core(itg_handle* h, const double* Awork, int64_t mm, int64_t nn, int precision,
                   double* X, double* lam, double* Uw, double* ws, float* ws32, int* flag,
                   int* sweeps_out, bool need_u);
size_t svd_mixed_ws_doubles(int64_t mm, int64_t nn);
int ns_polish(itg_handle* h, double* L, int64_t rows, int64_t cols, double* ws, double* tmp, int precision);
}  // namespace itg

__global__ void k_sqrt_clamp(const double* __restrict__ lam, int n, double* __restrict__ sig) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    sig[i] = sqrt(fmax(lam[i], 0.0));
}

// Side of the working matrix that must come out exactly orthonormal (see svd_trunc_impl).
enum { ISO_NONE = -1, ISO_LEFT = 0, ISO_RIGHT = 1 };

static int svd_trunc_impl(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                          int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff,
                          int doRelCutoff, int legacy_gpu, double* U, double* S, double* V,
                          int64_t* k, double* truncerr, double* docut, int method, int precision,
                          int iso, bool want_other = true, bool square_t = false);

extern "C" int itg_svd_trunc(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                             int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff,
                             int doRelCutoff, int legacy_gpu, double* U, double* S, double* V,
                             int64_t* k, double* truncerr, double* docut) {
  return svd_trunc_impl(h, m, n, A, lda, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff,
                        legacy_gpu, U, S, V, k, truncerr, docut, ITG_SVD_JACOBI, ITG_PREC_FP64, ISO_NONE);
}

extern "C" int itg_svd_trunc_ex(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                                int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff,
                                int doRelCutoff, int legacy_gpu, double* U, double* S, double* V,
                                int64_t* k, double* truncerr, double* docut, int method,
                                int precision) {
  if (method != ITG_SVD_AUTO && method != ITG_SVD_JACOBI && method != ITG_SVD_MIXED)
    return itg_fail(h, ITG_ERR_INVALID, "unknown SVD method %d", method);
  if (precision != ITG_PREC_FP64 && precision != ITG_PREC_SPLIT)
    return itg_fail(h, ITG_ERR_INVALID, "unknown precision %d", precision);
  return svd_trunc_impl(h, m, n, A, lda, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff,
                        legacy_gpu, U, S, V, k, truncerr, docut, method, precision, ISO_NONE);
}


// iso: which side of the working matrix W (the tall orientation of A) must
// come out with exactly orthonormal columns when W is large:
//   ISO_LEFT : W = Q R, Jacobi on J = R^T;             W = (Q V_J) S U_J^T
//   ISO_RIGHT: W = Q1 R1, R1^T = Q2 R2, J = R2^T;      W = (Q1 U_J) S (Q2 V_J)^T
// V_J (the Jacobi rotations, or the refined eigenvectors of the mixed method)
// is orthonormal to rounding; U_J = J V_J / S is accurate only where S is
// resolved.  ISO_NONE uses ISO_LEFT when QR preconditioning is on.

static int svd_trunc_impl(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                          int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff,
                          int doRelCutoff, int legacy_gpu, double* U, double* S, double* V,
                          int64_t* k, double* truncerr, double* docut, int method, int precision,
                          int iso, bool want_other, bool square_t) {
  if (!h || m < 0 || n < 0 || lda < m || !A || !U || !S || !V) return ITG_ERR_INVALID;
  if (m == 0 || n == 0) {
    if (k) *k = 0;
    if (truncerr) *truncerr = 0;
    if (docut) *docut = 0;
    return ITG_OK;
  }
  // square_t: a square A is worked on as W = A^T (A's right side is W's left)
  const bool tr = m < n || (square_t && m == n);
  const int64_t mm = tr ? n : m, nn = tr ? m : n;  // working shape, mm >= nn
  if (nn > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "svd: min(m,n) too large");
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += itg_align256(bytes); return o; };
  const bool mixed = method == ITG_SVD_MIXED || (method == ITG_SVD_AUTO && nn > ONECTA_MAX_N);
  // QR preconditioning for large problems, and whenever a side must be
  // exactly orthonormal: that side is then Q times the rotations (or the
  // refined eigenvectors), never U_J = J V_J / S, which loses orthogonality
  // in columns whose S is small or rounding noise (rank-deficient inputs)
  const bool pre = (h->svd_qr_precond && nn > ONECTA_MAX_N) || iso != ISO_NONE;
  const bool two = pre && iso == ISO_RIGHT;
  // the Jacobi problem: W itself (mj = mm rows) or J (nn x nn)
  const int64_t mj = pre ? nn : mm;
  size_t oW = take(sizeof(double) * mm * nn), oV = take(sizeof(double) * nn * nn),
         oSig = take(sizeof(double) * nn), oP = take(sizeof(double) * nn),
         oOrd = take(sizeof(int) * nn), oOut = take(4 * sizeof(double)), oFlag = take(sizeof(int) * JACOBI_AUX_INTS);
  size_t oLam = 0, oUw = 0, oWs = 0, oWs32 = 0, oVh = 0, oTau = 0, oRd = 0, oB = 0, oVh2 = 0, oTau2 = 0,
         oRd2 = 0, oB2 = 0;
  if (mixed) {
    oLam = take(sizeof(double) * nn);
    oUw = take(sizeof(double) * mj * nn);
    oWs = take(sizeof(double) * itg::svd_mixed_ws_doubles(mj, nn));
    oWs32 = take(sizeof(float) * (mj * nn + nn * nn));
  }
  size_t oTq = 0, oTq2 = 0, oQws = 0;
  if (pre) {
    oVh = take(sizeof(double) * mm * nn);
    oTau = take(sizeof(double) * nn);
    oRd = take(sizeof(double) * nn);
    oB = take(sizeof(double) * nn * nn);
    oTq = take(sizeof(double) * itg::qr_blocked_t_doubles(nn));
    oQws = take(sizeof(double) * itg::qr_blocked_ws_doubles(nn));
  }
  if (two) {
    oVh2 = take(sizeof(double) * nn * nn);
    oTau2 = take(sizeof(double) * nn);
    oRd2 = take(sizeof(double) * nn);
    oB2 = take(sizeof(double) * nn * nn);
    oTq2 = take(sizeof(double) * itg::qr_blocked_t_doubles(nn));
  }
  ITG_TRY(itg_scratch_reserve(h, off));
  char* base = (char*)h->scratch;
  double* W = (double*)(base + oW);
  double* Vw = (double*)(base + oV);
  double* sig = (double*)(base + oSig);
  double* P = (double*)(base + oP);
  int* order = (int*)(base + oOrd);
  double* out3 = (double*)(base + oOut);
  int* flag = (int*)(base + oFlag);
  if (!tr) {
    k_copy_matrix<<<itg_blocks_for(m * n, 256, h->num_sms * 16), 256, 0, h->stream>>>(A, lda, m, n, W, 0.0);
    ITG_CHECK_LAUNCH(h);
  } else {
    if (lda != m) return itg_fail(h, ITG_ERR_UNSUPPORTED, "svd of a wide matrix needs lda == m");
    ITG_TRY(itg::transpose(h, m, n, A, lda, W));
  }
  int sweeps = 0;
  int st = ITG_OK;
  double* Uw_dst = tr ? V : U;  // rows mm
  double* Vw_dst = tr ? U : V;  // rows nn
  double* J = W;
  double *Vh = nullptr, *tau = nullptr, *Vh2 = nullptr, *tau2 = nullptr;
  double *Tq = nullptr, *Tq2 = nullptr, *Qws = nullptr;
  // products of the QR's trailing updates: FP64 (their depth is one 32-column
  // panel, too shallow for the split path's operand preparation to pay off)
  const int qr_prec = ITG_PREC_FP64;
  if (pre) {
    Vh = (double*)(base + oVh);
    tau = (double*)(base + oTau);
    double* rd = (double*)(base + oRd);
    J = (double*)(base + oB);
    Tq = (double*)(base + oTq);
    Qws = (double*)(base + oQws);
    ProfScope prof(h, ITG_KERNEL_SVD_QR);
    ITG_TRY(itg::qr_blocked(h, W, mm, nn, nn, Vh, tau, rd, Tq, Qws, qr_prec));
    k_build_rt<<<itg_blocks_for(nn * nn, 256, h->num_sms * 16), 256, 0, h->stream>>>(W, mm, (int)nn, rd, J);
    ITG_CHECK_LAUNCH(h);
    if (two) {
      Vh2 = (double*)(base + oVh2);
      tau2 = (double*)(base + oTau2);
      double* rd2 = (double*)(base + oRd2);
      double* J2 = (double*)(base + oB2);
      Tq2 = (double*)(base + oTq2);
      ITG_TRY(itg::qr_blocked(h, J, nn, nn, nn, Vh2, tau2, rd2, Tq2, Qws, qr_prec));
      k_build_rt<<<itg_blocks_for(nn * nn, 256, h->num_sms * 16), 256, 0, h->stream>>>(J, nn, (int)nn, rd2, J2);
      ITG_CHECK_LAUNCH(h);
      J = J2;
    }
  }
  // J's factors: left U_J (mj rows) and right V_J (nn rows), written where
  // they end up: without preconditioning W's left / right; with one QR, V_J
  // goes (zero-padded) to W's left slot and is rotated by Q; with two, U_J goes
  // to W's left slot (rotated by Q1) and V_J to the right slot (rotated by Q2).
  double* Jl_dst = !pre ? Uw_dst : (two ? Uw_dst : Vw_dst);
  double* Jr_dst = !pre ? Vw_dst : (two ? Vw_dst : Uw_dst);
  const int64_t ld_l = !pre ? mm : (two ? mm : nn);
  const int64_t ld_r = !pre ? nn : (two ? nn : mm);
  if (pre) ITG_CUDA(h, cudaMemsetAsync(Uw_dst, 0, sizeof(double) * mm * nn, h->stream));
  dim3 g1(itg_blocks_for(mj, 256, 64), (unsigned)nn), g2(itg_blocks_for(nn, 256, 64), (unsigned)nn);
  bool use_mixed = mixed;
  if (mixed) {
    double* lam = (double*)(base + oLam);
    double* Uw = (double*)(base + oUw);
    const int ms = itg::svd_mixed_core(h, J, mj, nn, precision, Vw, lam, Uw, (double*)(base + oWs),
                                       (float*)(base + oWs32), flag, &sweeps, want_other || !pre);
    if (ms == ITG_ERR_NOTCONVERGED) {
      use_mixed = false;  // refinement failed its check: FP64 Jacobi on the same J
      h->svd_fallbacks++;
    } else if (ms != ITG_OK) {
      return ms;
    }
  }
  if (use_mixed) {
    double* lam = (double*)(base + oLam);
    double* Uw = (double*)(base + oUw);
    k_sqrt_clamp<<<itg_blocks_for(nn, 256, 64), 256, 0, h->stream>>>(lam, (int)nn, sig);
    k_rank_desc<<<itg_blocks_for(nn, 256, 1024), 256, 0, h->stream>>>(sig, (int)nn, 0.0, order, S, P, 1);
    ITG_CHECK_LAUNCH(h);
    ITG_TRY(itg::truncate_dev(h, P, nn, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff, legacy_gpu, out3));
    if (want_other || !pre) k_gather_cols<<<g1, 256, 0, h->stream>>>(Uw, mj, order, sig, 0, (int)nn, Jl_dst, ld_l);
    k_gather_cols<<<g2, 256, 0, h->stream>>>(Vw, nn, order, sig, 0, (int)nn, Jr_dst, ld_r);
    ITG_CHECK_LAUNCH(h);
  } else {
    st = jacobi_run(h, J, mj, nn, Vw, flag, &sweeps);
    if (st != ITG_OK && st != ITG_ERR_NOTCONVERGED) return st;
    k_unit_cols<<<(unsigned)nn, 256, 0, h->stream>>>(Vw, nn);
    k_col_norms<<<(unsigned)nn, 256, 0, h->stream>>>(J, mj, sig);
    k_rank_desc<<<itg_blocks_for(nn, 256, 1024), 256, 0, h->stream>>>(sig, (int)nn, 0.0, order, S, P, 1);
    ITG_CHECK_LAUNCH(h);
    ITG_TRY(itg::truncate_dev(h, P, nn, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff, legacy_gpu, out3));
    // U_J = J[:, order] / sig; V_J = Vw[:, order].
    k_gather_cols<<<g1, 256, 0, h->stream>>>(J, mj, order, sig, 1, (int)nn, Jl_dst, ld_l);
    k_gather_cols<<<g2, 256, 0, h->stream>>>(Vw, nn, order, sig, 0, (int)nn, Jr_dst, ld_r);
    ITG_CHECK_LAUNCH(h);
  }
  h->last_sweeps = sweeps;
  h->last_mixed = use_mixed;
  ITG_TRY(read_out3(h, out3, k, truncerr, docut));
  if (pre) {
    // rotate the kept columns back
    const int64_t kk = (k && *k > 0) ? *k : nn;
    {
      ProfScope prof(h, ITG_KERNEL_SVD_QR);
      // with two QRs W's left slot holds the non-isometric factor
      if (!two || want_other) ITG_TRY(itg::q_apply_blocked(h, Uw_dst, mm, nn, kk, Vh, Tq, Qws));
      if (two) ITG_TRY(itg::q_apply_blocked(h, Vw_dst, nn, nn, kk, Vh2, Tq2, Qws));
    }
    // the mixed method's isometric factor: one Newton-Schulz step after the
    // Householder rotation (W, the QR's input, is free by now)
    if (use_mixed) {
      ProfScope prof(h, ITG_KERNEL_SVD_REFINE);
      ITG_TRY(itg::ns_polish(h, two ? Vw_dst : Uw_dst, two ? nn : mm, kk, (double*)(base + oWs), W, precision));
    }
  }
  if (st == ITG_ERR_NOTCONVERGED)
    return itg_fail(h, ITG_ERR_NOTCONVERGED, "Jacobi SVD did not converge in %d sweeps", sweeps);
  return ITG_OK;
}

extern "C" int itg_factorize_trunc(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda,
                                   int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff,
                                   int doRelCutoff, int legacy_gpu, int ortho, int method, int precision,
                                   double* L, double* S, double* C, int64_t* k, double* truncerr,
                                   double* docut) {
  if (!h || !A || !L || !S || !C || m < 0 || n < 0 || lda < m) return ITG_ERR_INVALID;
  if (ortho != ITG_ORTHO_LEFT && ortho != ITG_ORTHO_RIGHT) return itg_fail(h, ITG_ERR_INVALID, "unknown ortho %d", ortho);
  if (method != ITG_SVD_AUTO && method != ITG_SVD_JACOBI && method != ITG_SVD_MIXED)
    return itg_fail(h, ITG_ERR_INVALID, "unknown SVD method %d", method);
  if (precision != ITG_PREC_FP64 && precision != ITG_PREC_SPLIT)
    return itg_fail(h, ITG_ERR_INVALID, "unknown precision %d", precision);
  int64_t kk = 0;
  if (m == 0 || n == 0) {
    if (k) *k = 0;
    if (truncerr) *truncerr = 0;
    if (docut) *docut = 0;
    return ITG_OK;
  }
  if (lda != m) return itg_fail(h, ITG_ERR_UNSUPPORTED, "factorize needs lda == m");
  // the isometric factor in L's slot (U for ortho left, V for right); the other
  // SVD factor is scratch output in C's slot and replaced by the projection.
  // A square right-isometric split: the FP64 Jacobi keeps ISO_RIGHT's two QRs
  // (Jacobi on R2^T needs fewer sweeps; the FP64 N = 24 sweep at chi = 1024
  // took 20.6 s with two QRs and 26.9 s with one); the mixed method factors
  // A^T with its left side isometric, one QR (2048 x 2048: 0.153 s against
  // 0.178 s with two QRs).
  const bool tr = m < n;
  int iso = (ortho == ITG_ORTHO_LEFT) == !tr ? ISO_LEFT : ISO_RIGHT;
  const bool mixed_path = method == ITG_SVD_MIXED || (method == ITG_SVD_AUTO && (m < n ? m : n) > ONECTA_MAX_N);
  const bool square_t = mixed_path && m == n && iso == ISO_RIGHT;
  if (square_t) iso = ISO_LEFT;
  double* Ubuf = ortho == ITG_ORTHO_LEFT ? L : C;
  double* Vbuf = ortho == ITG_ORTHO_LEFT ? C : L;
  // the non-isometric factor is not needed: C is the projection below
  int st = svd_trunc_impl(h, m, n, A, lda, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff, legacy_gpu, Ubuf,
                          S, Vbuf, &kk, truncerr, docut, method, precision, iso, false, square_t);
  if (st != ITG_OK && st != ITG_ERR_NOTCONVERGED) return st;
  if (k) *k = kk;
  if (kk == 0) return st;
  // C = L^T A (kk x n) or C = A L (m x kk); C must not alias the GEMM operands,
  // so the scratch factor in C's slot is simply overwritten
  const int64_t dA[2] = {m, n};
  const int32_t mA[2] = {1, 2};
  if (ortho == ITG_ORTHO_LEFT) {
    const int64_t dL[2] = {m, kk}, dC[2] = {kk, n};
    const int32_t mL[2] = {1, 3}, mC[2] = {3, 2};
    ITG_TRY(itg::contract_f64(h, 1.0, L, 2, dL, mL, A, 2, dA, mA, 0.0, C, 2, dC, mC, precision));
  } else {
    const int64_t dR[2] = {n, kk}, dC[2] = {m, kk};
    const int32_t mR[2] = {2, 3}, mC[2] = {1, 3};
    ITG_TRY(itg::contract_f64(h, 1.0, A, 2, dA, mA, L, 2, dR, mR, 0.0, C, 2, dC, mC, precision));
  }
  return st == ITG_ERR_NOTCONVERGED ? itg_fail(h, st, "Jacobi SVD did not converge") : ITG_OK;
}

extern "C" int itg_eigh_trunc(itg_handle* h, int64_t n, const double* A, int64_t lda,
                              int64_t maxdim, int64_t mindim, double cutoff, int absoluteCutoff,
                              int doRelCutoff, int legacy_gpu, double* D, double* U, int64_t* k,
                              double* truncerr, double* docut) {
  if (!h || n < 0 || lda < n || !A || !D || !U) return ITG_ERR_INVALID;
  if (n == 0) {
    if (k) *k = 0;
    if (truncerr) *truncerr = 0;
    if (docut) *docut = 0;
    return ITG_OK;
  }
  if (n > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "eigh: n too large");
  // B = A + c I with c = max row sum of |A| is positive semidefinite, so its
  // one-sided Jacobi SVD B V = W with |w_j| = lambda_j + c and V the
  // eigenvectors; lambda_j = |w_j| - c.
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += itg_align256(bytes); return o; };
  size_t oW = take(sizeof(double) * n * n), oV = take(sizeof(double) * n * n),
         oSig = take(sizeof(double) * n), oP = take(sizeof(double) * n),
         oOrd = take(sizeof(int) * n), oOut = take(4 * sizeof(double)), oFlag = take(sizeof(int) * JACOBI_AUX_INTS),
         oC = take(sizeof(double));
  ITG_TRY(itg_scratch_reserve(h, off));
  char* base = (char*)h->scratch;
  double* W = (double*)(base + oW);
  double* Vw = (double*)(base + oV);
  double* sig = (double*)(base + oSig);
  double* P = (double*)(base + oP);
  int* order = (int*)(base + oOrd);
  double* out3 = (double*)(base + oOut);
  int* flag = (int*)(base + oFlag);
  double* cdev = (double*)(base + oC);
  k_gershgorin<<<1, 1024, 0, h->stream>>>(A, lda, n, cdev);
  ITG_CHECK_LAUNCH(h);
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, cdev, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  const double shift = h->pinned[0] > 0.0 ? h->pinned[0] : 1.0;
  k_copy_matrix<<<itg_blocks_for(n * n, 256, h->num_sms * 16), 256, 0, h->stream>>>(A, lda, n, n, W, shift);
  ITG_CHECK_LAUNCH(h);
  int sweeps = 0;
  int st = jacobi_run(h, W, n, n, Vw, flag, &sweeps);
  if (st != ITG_OK && st != ITG_ERR_NOTCONVERGED) return st;
  k_unit_cols<<<(unsigned)n, 256, 0, h->stream>>>(Vw, n);
  k_col_norms<<<(unsigned)n, 256, 0, h->stream>>>(W, n, sig);
  k_rank_desc<<<itg_blocks_for(n, 256, 1024), 256, 0, h->stream>>>(sig, (int)n, shift, order, D, P, 0);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::truncate_dev(h, P, n, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff, legacy_gpu, out3));
  dim3 g2(itg_blocks_for(n, 256, 64), (unsigned)n);
  k_gather_cols<<<g2, 256, 0, h->stream>>>(Vw, n, order, sig, 0, (int)n, U, n);
  ITG_CHECK_LAUNCH(h);
  h->last_sweeps = sweeps;
  ITG_TRY(read_out3(h, out3, k, truncerr, docut));
  if (st == ITG_ERR_NOTCONVERGED)
    return itg_fail(h, ITG_ERR_NOTCONVERGED, "Jacobi eigensolver did not converge in %d sweeps", sweeps);
  return ITG_OK;
}

// ================================================================== QR
// Householder QR through the blocked factorisation (itg_qr_blocked.cu), so Q
// has orthonormal columns for any A, rank-deficient included (a zero column
// gives a zero row of R and a unit column of Q).  A wide matrix (m < n) takes
// m reflectors applied to all n columns.  Rows of R and columns of Q are then
// sign-flipped together so that R's diagonal is non-negative.

// R (r x n) from the factored W: R(k, i) = s_k W(k, i) above the diagonal,
// |rd[k]| on it, 0 below, with s_k the sign of rd[k].
__global__ void k_extract_r(const double* __restrict__ W, int64_t m, int64_t r, int64_t n,
                            const double* __restrict__ rd, double* __restrict__ R) {
  const int64_t total = r * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / r, k = t - i * r;
    const double sk = rd[k] < 0.0 ? -1.0 : 1.0;
    R[t] = k < i ? sk * W[k + i * m] : (k == i ? fabs(rd[k]) : 0.0);
  }
}

// Q (m x r) = the first r columns of the identity.
__global__ void k_eye_cols(double* __restrict__ Q, int64_t m, int64_t r) {
  const int64_t total = m * r;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / m, i = t - j * m;
    Q[t] = i == j ? 1.0 : 0.0;
  }
}

__global__ void k_sign_cols(double* __restrict__ Q, int64_t m, int64_t r, const double* __restrict__ rd) {
  const int64_t total = m * r;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / m;
    if (rd[j] < 0.0) Q[t] = -Q[t];
  }
}

extern "C" int itg_qr(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda, double* Q,
                      double* R) {
  if (!h || m < 0 || n < 0 || lda < m || !A || !Q || !R) return ITG_ERR_INVALID;
  const int64_t r = m < n ? m : n;
  if (r == 0) return ITG_OK;
  if (r > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "qr: min(m,n) too large");
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  const size_t oW = take(sizeof(double) * m * n);
  const size_t oVh = take(sizeof(double) * m * r);
  const size_t oTau = take(sizeof(double) * r);
  const size_t oRd = take(sizeof(double) * r);
  const size_t oT = take(sizeof(double) * itg::qr_blocked_t_doubles(r));
  const size_t oWs = take(sizeof(double) * itg::qr_blocked_ws_doubles(n));
  ITG_TRY(itg_scratch_reserve(h, off));
  char* base = (char*)h->scratch;
  double* W = (double*)(base + oW);
  double* Vh = (double*)(base + oVh);
  double* tau = (double*)(base + oTau);
  double* rd = (double*)(base + oRd);
  double* Tq = (double*)(base + oT);
  double* ws = (double*)(base + oWs);
  k_copy_matrix<<<itg_blocks_for(m * n, 256, h->num_sms * 16), 256, 0, h->stream>>>(A, lda, m, n, W, 0.0);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::qr_blocked(h, W, m, n, r, Vh, tau, rd, Tq, ws, ITG_PREC_FP64));
  k_extract_r<<<itg_blocks_for(r * n, 256, h->num_sms * 16), 256, 0, h->stream>>>(W, m, r, n, rd, R);
  k_eye_cols<<<itg_blocks_for(m * r, 256, h->num_sms * 16), 256, 0, h->stream>>>(Q, m, r);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::q_apply_blocked(h, Q, m, r, r, Vh, Tq, ws));
  k_sign_cols<<<itg_blocks_for(m * r, 256, h->num_sms * 16), 256, 0, h->stream>>>(Q, m, r, rd);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_svd_info(itg_handle* h, int* sweeps, int* mixed_used, int64_t* mixed_fallbacks) {
  if (!h) return ITG_ERR_INVALID;
  if (sweeps) *sweeps = h->last_sweeps;
  if (mixed_used) *mixed_used = h->last_mixed ? 1 : 0;
  if (mixed_fallbacks) *mixed_fallbacks = h->svd_fallbacks;
  return ITG_OK;
}

extern "C" int itg_set_svd_options(itg_handle* h, int qr_precondition, int jacobi_mode) {
  if (!h || jacobi_mode < 0 || jacobi_mode > 3) return ITG_ERR_INVALID;
  h->svd_qr_precond = qr_precondition != 0;
  h->jacobi_mode = jacobi_mode;
  return ITG_OK;
}
