// Factorisations of complex (ITG_C64, interleaved re/im) matrices: truncated
// SVD and Hermitian eigendecomposition by one-sided complex Jacobi, thin QR
// by complex Gram-Schmidt with one full re-orthogonalisation.  Replace svd /
// eigen / qr on CuDenseTensor{ComplexF64} (src/tensor/culinearalgebra.jl:33-121,
// whose eigen takes the Hermitian route for complex input at :84-85;
// test/test_cuitensor.jl:100-130).
//
// Complex Jacobi rotation of the column pair (a_p, a_q) with alpha = |a_p|^2,
// beta = |a_q|^2, gamma = a_p^H a_q = |gamma| e^{i phi}: scaling a_q by
// e^{-i phi} makes the pair's inner product real and positive, after which
// the real rotation of the FP64 kernels applies:
//   zeta = (beta - alpha) / (2 |gamma|), t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)),
//   c = 1 / sqrt(1 + t^2), s = c t,
//   a_p <- c a_p - s e^{-i phi} a_q,  a_q <- s a_p + c e^{-i phi} a_q,
// and the same on V's columns.  At convergence W = A V has orthogonal
// columns, sigma_j = |w_j|, U = W / sigma and A = U diag(sigma) V^H.  Same
// skip rule (|gamma| <= tol sqrt(alpha beta)), convergence rule (4 tol, noise
// columns below 10 eps |A|_F ignored) and truncation (truncate_dev on P =
// sigma^2) as the real path.  One launch per round-robin step; these serve
// the complex tensors of the reference's tests, not the DMRG sweep.
#include "itg_internal.cuh"

#include <cmath>

namespace {

constexpr int ZJ_MAX_SWEEPS = 60;
constexpr double EPS = 2.220446049250313e-16;

__device__ __forceinline__ double zwarp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over a 256-thread block; every thread gets the result.
__device__ double zblock_sum(double v, double* sh) {
  v = zwarp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  return s;
}

__device__ __forceinline__ int zrr_player(int pos, int step, int np) {
  if (pos == 0) return 0;
  return 1 + (pos - 1 + step) % (np - 1);
}

// One round-robin step: one CTA per column pair.
__global__ void __launch_bounds__(256)
k_zjacobi_step(double* __restrict__ W, int64_t m, int n, double* __restrict__ V, double tol, double amin_conv,
               int step, int* __restrict__ rotated) {
  __shared__ double sh[4][8];
  const int np = n + (n & 1);
  int p = zrr_player(blockIdx.x, step, np), q = zrr_player(np - 1 - blockIdx.x, step, np);
  if (p >= n || q >= n) return;
  if (p > q) { const int t = p; p = q; q = t; }
  double* wp = W + 2 * (int64_t)p * m;
  double* wq = W + 2 * (int64_t)q * m;
  double a = 0, b = 0, gr = 0, gi = 0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    const double xr = wp[2 * i], xi = wp[2 * i + 1], yr = wq[2 * i], yi = wq[2 * i + 1];
    a = fma(xr, xr, fma(xi, xi, a));
    b = fma(yr, yr, fma(yi, yi, b));
    gr = fma(xr, yr, fma(xi, yi, gr));   // conj(x) y
    gi = fma(xr, yi, fma(-xi, yr, gi));
  }
  a = zblock_sum(a, sh[0]);
  b = zblock_sum(b, sh[1]);
  gr = zblock_sum(gr, sh[2]);
  gi = zblock_sum(gi, sh[3]);
  const double g = hypot(gr, gi);
  if (a == 0.0 || b == 0.0 || g <= tol * sqrt(a) * sqrt(b)) return;
  const double zeta = (b - a) / (2.0 * g);
  const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
  const double er = gr / g, ei = -gi / g;  // e^{-i phi}
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    const double xr = wp[2 * i], xi = wp[2 * i + 1];
    const double yr = er * wq[2 * i] - ei * wq[2 * i + 1], yi = er * wq[2 * i + 1] + ei * wq[2 * i];
    wp[2 * i] = c * xr - s * yr;
    wp[2 * i + 1] = c * xi - s * yi;
    wq[2 * i] = s * xr + c * yr;
    wq[2 * i + 1] = s * xi + c * yi;
  }
  double* vp = V + 2 * (int64_t)p * n;
  double* vq = V + 2 * (int64_t)q * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double xr = vp[2 * i], xi = vp[2 * i + 1];
    const double yr = er * vq[2 * i] - ei * vq[2 * i + 1], yi = er * vq[2 * i + 1] + ei * vq[2 * i];
    vp[2 * i] = c * xr - s * yr;
    vp[2 * i + 1] = c * xi - s * yi;
    vq[2 * i] = s * xr + c * yr;
    vq[2 * i + 1] = s * xi + c * yi;
  }
  if (threadIdx.x == 0 && a > amin_conv && b > amin_conv && g > 4.0 * tol * sqrt(a) * sqrt(b)) *rotated = 1;
}

// W (rows x cols) = A (or A^H when conj_tr), complex, A with leading dimension lda.
__global__ void k_zload(const double* __restrict__ A, int64_t lda, int64_t rows, int64_t cols, int conj_tr,
                        double* __restrict__ W) {
  const int64_t total = rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / rows, i = t - j * rows;
    const int64_t src = conj_tr ? (j + i * lda) : (i + j * lda);
    W[2 * t] = A[2 * src];
    W[2 * t + 1] = conj_tr ? -A[2 * src + 1] : A[2 * src + 1];
  }
}

__global__ void k_zidentity(int n, double* __restrict__ V) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
    V[2 * t] = (t % (n + 1) == 0) ? 1.0 : 0.0;
    V[2 * t + 1] = 0.0;
  }
}

__global__ void k_zcol_norms(const double* __restrict__ W, int64_t m, double* __restrict__ sig) {
  __shared__ double sh[8];
  const double* w = W + 2 * (int64_t)blockIdx.x * m;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < 2 * m; i += blockDim.x) s = fma(w[i], w[i], s);
  s = zblock_sum(s, sh);
  if (threadIdx.x == 0) sig[blockIdx.x] = sqrt(s);
}

__global__ void k_zrank(const double* __restrict__ sig, int n, int* __restrict__ order, double* __restrict__ S,
                        double* __restrict__ P) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const double v = sig[j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      const double u = sig[i];
      r += (u > v) || (u == v && i < j);
    }
    order[r] = j;
    S[r] = v;
    P[r] = v * v;
  }
}

// dst[:, r] = src[:, order[r]] (/ sig[order[r]] when inv), complex columns of `rows`.
__global__ void k_zgather(const double* __restrict__ src, int64_t rows, const int* __restrict__ order,
                          const double* __restrict__ sig, int inv, int ncols, double* __restrict__ dst) {
  const int r = blockIdx.y;
  if (r >= ncols) return;
  const int j = order[r];
  double f = 1.0;
  if (inv) f = sig[j] > 0.0 ? 1.0 / sig[j] : 0.0;
  const double* s = src + 2 * (int64_t)j * rows;
  double* d = dst + 2 * (int64_t)r * rows;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 2 * rows; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = s[i] * f;
}

// max over rows of sum_j |A_ij| (complex modulus): a bound on |eigenvalues|
__global__ void k_zgershgorin(const double* __restrict__ A, int64_t lda, int64_t n, double* out) {
  __shared__ double sh[32];
  double best = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double s = 0.0;
    for (int64_t j = 0; j < n; ++j) s += hypot(A[2 * (i + j * lda)], A[2 * (i + j * lda) + 1]);
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

// W[i, i] += shift (real part), complex n x n
__global__ void k_zshift_diag(double* __restrict__ W, int64_t n, double shift) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    W[2 * (i + i * n)] += shift;
}

// D[r] = sig[order[r]] - shift (descending), P = D
__global__ void k_zshift_rank(const double* __restrict__ sig, int n, double shift, int* __restrict__ order,
                              double* __restrict__ D, double* __restrict__ P) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const double v = sig[j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      const double u = sig[i];
      r += (u > v) || (u == v && i < j);
    }
    order[r] = j;
    D[r] = v - shift;
    P[r] = v - shift;
  }
}

// ---- complex CGS2 QR
// hc[i] = Q[:, i]^H q for i < blockIdx range (one block per i)
__global__ void __launch_bounds__(256)
k_zproj(const double* __restrict__ Q, int64_t m, const double* __restrict__ q, double* __restrict__ hc) {
  __shared__ double sh[2][8];
  const double* col = Q + 2 * (int64_t)blockIdx.x * m;
  double sr = 0.0, si = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    const double xr = col[2 * i], xi = col[2 * i + 1], yr = q[2 * i], yi = q[2 * i + 1];
    sr = fma(xr, yr, fma(xi, yi, sr));
    si = fma(xr, yi, fma(-xi, yr, si));
  }
  sr = zblock_sum(sr, sh[0]);
  si = zblock_sum(si, sh[1]);
  if (threadIdx.x == 0) {
    hc[2 * blockIdx.x] = sr;
    hc[2 * blockIdx.x + 1] = si;
  }
}

// q -= Q[:, :j] hc;  racc[:j] += hc (block 0)
__global__ void k_zcgs_update(const double* __restrict__ Q, int64_t m, int j, const double* __restrict__ hc,
                              double* __restrict__ q, double* __restrict__ racc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    double sr = q[2 * i], si = q[2 * i + 1];
    for (int c = 0; c < j; ++c) {
      const double qr = Q[2 * (i + (int64_t)c * m)], qi = Q[2 * (i + (int64_t)c * m) + 1];
      const double hr = hc[2 * c], hi = hc[2 * c + 1];
      sr -= qr * hr - qi * hi;
      si -= qr * hi + qi * hr;
    }
    q[2 * i] = sr;
    q[2 * i + 1] = si;
  }
  if (blockIdx.x == 0)
    for (int c = threadIdx.x; c < j; c += blockDim.x) {
      racc[2 * c] += hc[2 * c];
      racc[2 * c + 1] += hc[2 * c + 1];
    }
}

__global__ void __launch_bounds__(256) k_znormalize(double* __restrict__ q, int64_t m, double* __restrict__ rjj) {
  __shared__ double sh[8];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < 2 * m; i += blockDim.x) s = fma(q[i], q[i], s);
  s = zblock_sum(s, sh);
  const double nrm = sqrt(s);
  const double f = nrm > 0.0 ? 1.0 / nrm : 0.0;
  for (int64_t i = threadIdx.x; i < 2 * m; i += blockDim.x) q[i] *= f;
  if (threadIdx.x == 0) {
    rjj[0] = nrm;
    rjj[1] = 0.0;
  }
}

}  // namespace

extern "C" int itg_svd_trunc_z(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda, int64_t maxdim,
                               int64_t mindim, double cutoff, int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                               double* U, double* S, double* V, int64_t* k, double* truncerr, double* docut) {
  if (!h || m < 0 || n < 0 || lda < m || !A || !U || !S || !V) return ITG_ERR_INVALID;
  if (m == 0 || n == 0) {
    if (k) *k = 0;
    if (truncerr) *truncerr = 0;
    if (docut) *docut = 0;
    return ITG_OK;
  }
  const bool tr = m < n;
  const int64_t mm = tr ? n : m, nn = tr ? m : n;
  if (nn > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "complex svd: min(m,n) too large");
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += itg_align256(bytes); return o; };
  const size_t oW = take(16 * mm * nn), oV = take(16 * nn * nn), oSig = take(8 * nn), oP = take(8 * nn),
               oOrd = take(sizeof(int) * nn), oOut = take(4 * 8), oFlag = take(sizeof(int)), oRed = take(8 * 1024);
  ITG_TRY(itg_scratch_reserve(h, off));
  char* base = (char*)h->scratch;
  double* W = (double*)(base + oW);
  double* Vw = (double*)(base + oV);
  double* sig = (double*)(base + oSig);
  double* P = (double*)(base + oP);
  int* order = (int*)(base + oOrd);
  double* out3 = (double*)(base + oOut);
  int* flag = (int*)(base + oFlag);
  double* red = (double*)(base + oRed);
  k_zload<<<itg_blocks_for(mm * nn, 256, h->num_sms * 16), 256, 0, h->stream>>>(A, lda, mm, nn, tr ? 1 : 0, W);
  k_zidentity<<<itg_blocks_for(nn * nn, 256, h->num_sms * 8), 256, 0, h->stream>>>((int)nn, Vw);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::nrm2_dev(h, 2 * mm * nn, W, red + 1000, red));
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, red + 1000, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  const double fro = h->pinned[0];
  const double tol = EPS * sqrt((double)mm);
  const double amin_conv = (10.0 * EPS * fro) * (10.0 * EPS * fro);
  const int np = (int)(nn + (nn & 1));
  int* hp = (int*)h->pinned;
  int sweeps = ZJ_MAX_SWEEPS;
  for (int sw = 0; sw < ZJ_MAX_SWEEPS && nn > 1; ++sw) {
    ITG_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
    for (int step = 0; step < np - 1; ++step)
      k_zjacobi_step<<<np / 2, 256, 0, h->stream>>>(W, mm, (int)nn, Vw, tol, amin_conv, step, flag);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(hp, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hp[0] == 0) {
      sweeps = sw + 1;
      break;
    }
  }
  if (nn <= 1) sweeps = 0;
  k_zcol_norms<<<(unsigned)nn, 256, 0, h->stream>>>(W, mm, sig);
  k_zrank<<<itg_blocks_for(nn, 256, 1024), 256, 0, h->stream>>>(sig, (int)nn, order, S, P);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::truncate_dev(h, P, nn, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff, legacy_gpu, out3));
  // working left vectors W / sigma (mm rows), right vectors Vw (nn rows); A = U S V^H,
  // and for the conjugate-transposed problem A^H = Uw S Vw^H, i.e. U = Vw, V = Uw
  double* Lw_dst = tr ? V : U;
  double* Rw_dst = tr ? U : V;
  dim3 g1(itg_blocks_for(2 * mm, 256, 64), (unsigned)nn), g2(itg_blocks_for(2 * nn, 256, 64), (unsigned)nn);
  k_zgather<<<g1, 256, 0, h->stream>>>(W, mm, order, sig, 1, (int)nn, Lw_dst);
  k_zgather<<<g2, 256, 0, h->stream>>>(Vw, nn, order, sig, 0, (int)nn, Rw_dst);
  ITG_CHECK_LAUNCH(h);
  h->last_sweeps = sweeps;
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, out3, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (k) *k = (int64_t)h->pinned[0];
  if (truncerr) *truncerr = h->pinned[1];
  if (docut) *docut = h->pinned[2];
  if (sweeps >= ZJ_MAX_SWEEPS && nn > 1)
    return itg_fail(h, ITG_ERR_NOTCONVERGED, "complex Jacobi SVD did not converge in %d sweeps", sweeps);
  return ITG_OK;
}

// Hermitian eigendecomposition: B = A + c I with c = max row sum of |A| is
// positive semidefinite, so its one-sided Jacobi B V = W gives |w_j| =
// lambda_j + c with V the eigenvectors (the route of the real itg_eigh_trunc).
extern "C" int itg_eigh_trunc_z(itg_handle* h, int64_t n, const double* A, int64_t lda, int64_t maxdim,
                                int64_t mindim, double cutoff, int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                                double* D, double* U, int64_t* k, double* truncerr, double* docut) {
  if (!h || n < 0 || lda < n || !A || !D || !U) return ITG_ERR_INVALID;
  if (n == 0) {
    if (k) *k = 0;
    if (truncerr) *truncerr = 0;
    if (docut) *docut = 0;
    return ITG_OK;
  }
  if (n > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "complex eigh: n too large");
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += itg_align256(bytes); return o; };
  const size_t oW = take(16 * n * n), oV = take(16 * n * n), oSig = take(8 * n), oP = take(8 * n),
               oOrd = take(sizeof(int) * n), oOut = take(4 * 8), oFlag = take(sizeof(int)), oC = take(8),
               oRed = take(8 * 1024);
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
  double* red = (double*)(base + oRed);
  k_zgershgorin<<<1, 1024, 0, h->stream>>>(A, lda, n, cdev);
  ITG_CHECK_LAUNCH(h);
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, cdev, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  const double shift = h->pinned[0] > 0.0 ? h->pinned[0] : 1.0;
  k_zload<<<itg_blocks_for(n * n, 256, h->num_sms * 16), 256, 0, h->stream>>>(A, lda, n, n, 0, W);
  k_zshift_diag<<<itg_blocks_for(n, 256, 64), 256, 0, h->stream>>>(W, n, shift);
  k_zidentity<<<itg_blocks_for(n * n, 256, h->num_sms * 8), 256, 0, h->stream>>>((int)n, Vw);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::nrm2_dev(h, 2 * n * n, W, red + 1000, red));
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, red + 1000, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  const double fro = h->pinned[0];
  const double tol = EPS * sqrt((double)n);
  const double amin_conv = (10.0 * EPS * fro) * (10.0 * EPS * fro);
  const int np = (int)(n + (n & 1));
  int* hp = (int*)h->pinned;
  int sweeps = n > 1 ? ZJ_MAX_SWEEPS : 0;
  for (int sw = 0; sw < ZJ_MAX_SWEEPS && n > 1; ++sw) {
    ITG_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
    for (int step = 0; step < np - 1; ++step)
      k_zjacobi_step<<<np / 2, 256, 0, h->stream>>>(W, n, (int)n, Vw, tol, amin_conv, step, flag);
    ITG_CHECK_LAUNCH(h);
    ITG_CUDA(h, cudaMemcpyAsync(hp, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hp[0] == 0) {
      sweeps = sw + 1;
      break;
    }
  }
  k_zcol_norms<<<(unsigned)n, 256, 0, h->stream>>>(W, n, sig);
  k_zshift_rank<<<itg_blocks_for(n, 256, 1024), 256, 0, h->stream>>>(sig, (int)n, shift, order, D, P);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::truncate_dev(h, P, n, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff, legacy_gpu, out3));
  dim3 g2(itg_blocks_for(2 * n, 256, 64), (unsigned)n);
  k_zgather<<<g2, 256, 0, h->stream>>>(Vw, n, order, sig, 0, (int)n, U);
  ITG_CHECK_LAUNCH(h);
  h->last_sweeps = sweeps;
  ITG_CUDA(h, cudaMemcpyAsync(h->pinned, out3, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (k) *k = (int64_t)h->pinned[0];
  if (truncerr) *truncerr = h->pinned[1];
  if (docut) *docut = h->pinned[2];
  if (sweeps >= ZJ_MAX_SWEEPS)
    return itg_fail(h, ITG_ERR_NOTCONVERGED, "complex Jacobi eigensolver did not converge in %d sweeps", sweeps);
  return ITG_OK;
}

extern "C" int itg_qr_z(itg_handle* h, int64_t m, int64_t n, const double* A, int64_t lda, double* Q, double* R) {
  if (!h || m < 0 || n < 0 || lda < m || !A || !Q || !R) return ITG_ERR_INVALID;
  const int64_t r = m < n ? m : n;
  if (r == 0) return ITG_OK;
  if (r > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "complex qr: min(m,n) too large");
  ITG_CUDA(h, cudaMemsetAsync(R, 0, 16 * (size_t)r * n, h->stream));
  ITG_TRY(itg_scratch_reserve(h, 16 * (size_t)(r + 256)));
  double* hc = (double*)h->scratch;
  const int gb = itg_blocks_for(m, 256, h->num_sms * 4);
  for (int64_t j = 0; j < n; ++j) {
    const double* a = A + 2 * j * lda;
    double* rcol = R + 2 * j * r;
    if (j < r) {
      double* q = Q + 2 * j * m;
      ITG_CUDA(h, cudaMemcpyAsync(q, a, 16 * (size_t)m, cudaMemcpyDeviceToDevice, h->stream));
      if (j > 0) {
        for (int pass = 0; pass < 2; ++pass) {
          k_zproj<<<(unsigned)j, 256, 0, h->stream>>>(Q, m, q, hc);
          k_zcgs_update<<<gb, 256, 0, h->stream>>>(Q, m, (int)j, hc, q, rcol);
        }
      }
      k_znormalize<<<1, 256, 0, h->stream>>>(q, m, rcol + 2 * j);
    } else {
      k_zproj<<<(unsigned)r, 256, 0, h->stream>>>(Q, m, a, rcol);
    }
    ITG_CHECK_LAUNCH(h);
  }
  return ITG_OK;
}
