// Batched kernels for many independent small DMRG instances advanced in
// lockstep: one-CTA-per-instance Jacobi SVD with on-device truncation, and a
// lockstep Davidson whose H_eff chain runs as grouped contractions (one launch
// per chain step for all instances) and whose vector operations are segmented
// kernels over all instances' vectors at once.
#include "itg_internal.cuh"

#include <cmath>
#include <algorithm>
#include <vector>

namespace itg {
int contract_grouped_f64(itg_handle* h, int count, double alpha, const double* const* A, int rankA,
                         const int64_t* dimsA, const int32_t* modesA, const double* const* B, int rankB,
                         const int64_t* dimsB, const int32_t* modesB, double beta, double* const* C,
                         int rankC, const int64_t* dimsC, const int32_t* modesC);
}

namespace {

// ------------------------------------------------------------ batched SVD
struct SvdJob {
  const double* A;   // m x n input (ld = m)
  double* U;         // m x r out
  double* S;         // r out
  double* V;         // n x r out
  double* W;         // working mm x nn (transposed when m < n)
  double* Vw;        // nn x nn
  double* sig;       // nn
  double* P;         // nn
  int* order;        // nn
  double* out3;      // keep, truncerr, docut
  int m, n, mm, nn, tr;
  int64_t maxdim;
};

__device__ __forceinline__ int rr_p(int pos, int step, int np) {
  if (pos == 0) return 0;
  return ((pos - 1 + step) % (np - 1)) + 1;
}

__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One CTA per instance: copy, all Jacobi sweeps, norms, ranking.
__global__ void __launch_bounds__(1024)
k_svd_batched(SvdJob* __restrict__ jobs, double tol_eps, int max_sweeps, int* __restrict__ sweeps_out) {
  SvdJob J = jobs[blockIdx.x];
  const int mm = J.mm, nn = J.nn;
  // copy (transpose for wide inputs) and identity
  for (int t = threadIdx.x; t < mm * nn; t += blockDim.x) {
    const int j = t / mm, i = t - j * mm;
    J.W[t] = J.tr ? J.A[j + (int64_t)i * J.m] : J.A[i + (int64_t)j * J.m];
  }
  for (int t = threadIdx.x; t < nn * nn; t += blockDim.x) J.Vw[t] = (t % (nn + 1) == 0) ? 1.0 : 0.0;
  __syncthreads();
  __shared__ int rotated;
  const int np = nn + (nn & 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const double tol = tol_eps * sqrt((double)mm);
  int sweep = 0;
  for (; sweep < max_sweeps && nn > 1; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int step = 0; step < np - 1; ++step) {
      for (int pi = warp; pi < np / 2; pi += nw) {
        int p = rr_p(pi, step, np), q = rr_p(np - 1 - pi, step, np);
        if (p >= nn || q >= nn) continue;
        if (p > q) { const int t = p; p = q; q = t; }
        double* wp = J.W + (int64_t)p * mm;
        double* wq = J.W + (int64_t)q * mm;
        double a = 0, b = 0, g = 0;
        for (int i = lane; i < mm; i += 32) {
          const double x = wp[i], y = wq[i];
          a = fma(x, x, a);
          b = fma(y, y, b);
          g = fma(x, y, g);
        }
        a = wsum(a); b = wsum(b); g = wsum(g);
        if (a == 0.0 || b == 0.0 || fabs(g) <= tol * sqrt(a) * sqrt(b)) continue;
        const double zeta = (b - a) / (2.0 * g);
        const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        for (int i = lane; i < mm; i += 32) {
          const double x = wp[i], y = wq[i];
          wp[i] = c * x - s * y;
          wq[i] = s * x + c * y;
        }
        double* vp = J.Vw + (int64_t)p * nn;
        double* vq = J.Vw + (int64_t)q * nn;
        for (int i = lane; i < nn; i += 32) {
          const double x = vp[i], y = vq[i];
          vp[i] = c * x - s * y;
          vq[i] = s * x + c * y;
        }
        // converged once no pair above the rounding floor of the dot product
        // (4 tol, as in the single-matrix kernels) needed a rotation
        if (lane == 0 && fabs(g) > 4.0 * tol * sqrt(a) * sqrt(b)) rotated = 1;
      }
      __syncthreads();
    }
    const int r = rotated;
    __syncthreads();
    if (!r) break;
  }
  if (threadIdx.x == 0) sweeps_out[blockIdx.x] = sweep;
  // column norms of W, unit-norm V columns
  for (int j = warp; j < nn; j += nw) {
    double s = 0.0, v2 = 0.0;
    for (int i = lane; i < mm; i += 32) s = fma(J.W[i + (int64_t)j * mm], J.W[i + (int64_t)j * mm], s);
    for (int i = lane; i < nn; i += 32) v2 = fma(J.Vw[i + (int64_t)j * nn], J.Vw[i + (int64_t)j * nn], v2);
    s = wsum(s);
    v2 = wsum(v2);
    const double f = v2 > 0.0 ? 1.0 / sqrt(v2) : 1.0;
    for (int i = lane; i < nn; i += 32) J.Vw[i + (int64_t)j * nn] *= f;
    if (lane == 0) J.sig[j] = sqrt(s);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nn; j += blockDim.x) {
    const double v = J.sig[j];
    int r = 0;
    for (int i = 0; i < nn; ++i) {
      const double u = J.sig[i];
      r += (u > v) || (u == v && i < j);
    }
    J.order[r] = j;
    J.S[r] = v;
    J.P[r] = v * v;
  }
}

// Gather the sorted factors: U[:, r] = W[:, order[r]] / sigma (rows mm), V[:, r] = Vw[:, order[r]].
__global__ void k_svd_batched_gather(SvdJob* __restrict__ jobs) {
  const SvdJob J = jobs[blockIdx.x];
  const int mm = J.mm, nn = J.nn;
  double* Ud = J.tr ? J.V : J.U;  // rows mm
  double* Vd = J.tr ? J.U : J.V;  // rows nn
  for (int t = threadIdx.x; t < mm * nn; t += blockDim.x) {
    const int r = t / mm, i = t - r * mm;
    const int j = J.order[r];
    const double sv = J.sig[j];
    Ud[t] = sv > 0.0 ? J.W[i + (int64_t)j * mm] / sv : 0.0;
  }
  for (int t = threadIdx.x; t < nn * nn; t += blockDim.x) {
    const int r = t / nn, i = t - r * nn;
    Vd[t] = J.Vw[i + (int64_t)J.order[r] * nn];
  }
}

}  // namespace

namespace itg {
int truncate_dev(itg_handle* h, const double* P, int64_t n, int64_t maxdim, int64_t mindim,
                 double cutoff, int absoluteCutoff, int doRelCutoff, int legacy_gpu, double* out3);
}

extern "C" int itg_svd_trunc_batched(itg_handle* h, int count, const int64_t* m, const int64_t* n,
                                     const double* const* A, const int64_t* maxdim, int64_t mindim,
                                     double cutoff, int absoluteCutoff, int doRelCutoff, int legacy_gpu,
                                     double* const* U, double* const* S, double* const* V, int64_t* k,
                                     double* truncerr) {
  if (!h || count < 0 || (count > 0 && (!m || !n || !A || !maxdim || !U || !S || !V || !k || !truncerr)))
    return ITG_ERR_INVALID;
  if (count == 0) return ITG_OK;
  std::vector<SvdJob> jobs(count);
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off += itg_align256(b); return o; };
  std::vector<size_t> oW(count), oV(count), oSig(count), oP(count), oOrd(count), oOut(count);
  for (int i = 0; i < count; ++i) {
    if (m[i] <= 0 || n[i] <= 0) return itg_fail(h, ITG_ERR_SHAPE, "batched svd: empty matrix %d", i);
    const int64_t mm = m[i] >= n[i] ? m[i] : n[i], nn = m[i] >= n[i] ? n[i] : m[i];
    if (nn > 512 || mm > 8192)
      return itg_fail(h, ITG_ERR_UNSUPPORTED, "batched svd: instance %d (%lld x %lld) above 512 columns",
                      i, (long long)m[i], (long long)n[i]);
    oW[i] = take(sizeof(double) * mm * nn);
    oV[i] = take(sizeof(double) * nn * nn);
    oSig[i] = take(sizeof(double) * nn);
    oP[i] = take(sizeof(double) * nn);
    oOrd[i] = take(sizeof(int) * nn);
    oOut[i] = take(4 * sizeof(double));
  }
  const size_t oJobs = take(sizeof(SvdJob) * count), oSw = take(sizeof(int) * count);
  ITG_TRY(itg_scratch_reserve(h, off));
  char* base = (char*)h->scratch;
  for (int i = 0; i < count; ++i) {
    SvdJob& J = jobs[i];
    J.A = A[i];
    J.U = U[i];
    J.S = S[i];
    J.V = V[i];
    J.W = (double*)(base + oW[i]);
    J.Vw = (double*)(base + oV[i]);
    J.sig = (double*)(base + oSig[i]);
    J.P = (double*)(base + oP[i]);
    J.order = (int*)(base + oOrd[i]);
    J.out3 = (double*)(base + oOut[i]);
    J.m = (int)m[i];
    J.n = (int)n[i];
    J.tr = m[i] < n[i];
    J.mm = J.tr ? J.n : J.m;
    J.nn = J.tr ? J.m : J.n;
    J.maxdim = maxdim[i];
  }
  SvdJob* djobs = (SvdJob*)(base + oJobs);
  ITG_CUDA(h, cudaMemcpyAsync(djobs, jobs.data(), sizeof(SvdJob) * count, cudaMemcpyHostToDevice, h->stream));
  k_svd_batched<<<count, 1024, 0, h->stream>>>(djobs, 2.220446049250313e-16, 60, (int*)(base + oSw));
  ITG_CHECK_LAUNCH(h);
  for (int i = 0; i < count; ++i)
    ITG_TRY(itg::truncate_dev(h, jobs[i].P, jobs[i].nn, maxdim[i], mindim, cutoff, absoluteCutoff,
                              doRelCutoff, legacy_gpu, jobs[i].out3));
  k_svd_batched_gather<<<count, 512, 0, h->stream>>>(djobs);
  ITG_CHECK_LAUNCH(h);
  // read all truncation results (contiguous copies would need one buffer; the
  // out3 slots are 256 bytes apart, so copy them one by one into pinned memory)
  if (count * 3 > ITG_PINNED_DOUBLES) return itg_fail(h, ITG_ERR_UNSUPPORTED, "batched svd: too many instances");
  for (int i = 0; i < count; ++i)
    ITG_CUDA(h, cudaMemcpyAsync(h->pinned + 3 * i, jobs[i].out3, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int i = 0; i < count; ++i) {
    k[i] = (int64_t)h->pinned[3 * i];
    truncerr[i] = h->pinned[3 * i + 1];
  }
  return ITG_OK;
}

// ============================================================ batched Davidson
// Same algorithm as itg_davidson_heff2, run for many instances at once.  Each
// instance keeps its own state (basis size, restart count, convergence); every
// phase runs one launch over the instances that are in that phase.
namespace {

struct Seg {
  int64_t n;      // vector length chiL*d*d*chiR
  int64_t V;      // offset of basis (kmax columns of n) in the V / AV buffers
  int64_t v1;     // offset of one-vector buffers (X, HX, Rv, T, dg)
  int64_t t1, t3; // offsets of T1 / T3
  int64_t rows;   // chiL * chiR
  int64_t chiL, chiR;
};

__device__ __forceinline__ double bsum(double v, double* sh) {
  v = wsum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = wsum(v);
  __syncthreads();
  return v;
}

// G[i][a + kmax*b] = V_i[:, a] . AV_i[:, b]  for a, b < kk[i]
__global__ void k_seg_gram(const int* __restrict__ ids, const Seg* __restrict__ seg, const int* __restrict__ kk,
                           int kmax, const double* __restrict__ V, const double* __restrict__ AV,
                           double* __restrict__ G) {
  __shared__ double sh[32];
  const int i = ids[blockIdx.y];
  const int a = blockIdx.x % kmax, b = blockIdx.x / kmax;
  if (a >= kk[i] || b >= kk[i]) return;
  const Seg s = seg[i];
  const double* x = V + s.V + a * s.n;
  const double* y = AV + s.V + b * s.n;
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < s.n; e += blockDim.x) acc = fma(x[e], y[e], acc);
  acc = bsum(acc, sh);
  if (threadIdx.x == 0) G[(int64_t)i * kmax * kmax + a + kmax * b] = acc;
}

// X = V y, HX = AV y, Rv = HX - theta X
__global__ void k_seg_ritz(const int* __restrict__ ids, const Seg* __restrict__ seg, const int* __restrict__ kk,
                           int kmax, const double* __restrict__ V, const double* __restrict__ AV,
                           const double* __restrict__ y, const double* __restrict__ theta,
                           double* __restrict__ X, double* __restrict__ HX, double* __restrict__ Rv) {
  const int i = ids[blockIdx.y];
  const Seg s = seg[i];
  const int k = kk[i];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < s.n; e += (int64_t)gridDim.x * blockDim.x) {
    double xv = 0.0, hv = 0.0;
    for (int j = 0; j < k; ++j) {
      const double c = y[(int64_t)i * kmax + j];
      xv = fma(V[s.V + j * s.n + e], c, xv);
      hv = fma(AV[s.V + j * s.n + e], c, hv);
    }
    X[s.v1 + e] = xv;
    HX[s.v1 + e] = hv;
    Rv[s.v1 + e] = hv - theta[i] * xv;
  }
}

// out[i] = |buf_i| where buf_i starts at base + (col >= 0 ? V + col*n : v1)
__global__ void k_seg_nrm(const int* __restrict__ ids, const Seg* __restrict__ seg, const double* __restrict__ buf,
                          int col, const int* __restrict__ colv, double* __restrict__ out) {
  __shared__ double sh[32];
  const int i = ids[blockIdx.x];
  const Seg s = seg[i];
  const int c = colv ? colv[i] : col;
  const double* x = buf + (c >= 0 ? s.V + c * s.n : s.v1);
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < s.n; e += blockDim.x) acc = fma(x[e], x[e], acc);
  acc = bsum(acc, sh);
  if (threadIdx.x == 0) out[i] = sqrt(acc);
}

// t_i (basis column kk[i] of V) = Rv / (dg - theta), guarded; or = Rv (plain)
__global__ void k_seg_correction(const int* __restrict__ ids, const Seg* __restrict__ seg,
                                 const int* __restrict__ kk, const double* __restrict__ Rv,
                                 const double* __restrict__ dg, const double* __restrict__ theta, int plain,
                                 double* __restrict__ V) {
  const int i = ids[blockIdx.y];
  const Seg s = seg[i];
  double* t = V + s.V + kk[i] * s.n;
  const double th = theta[i];
  const double guard = 1e-8 * (fabs(th) > 1.0 ? fabs(th) : 1.0);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < s.n; e += (int64_t)gridDim.x * blockDim.x) {
    if (plain) {
      t[e] = Rv[s.v1 + e];
    } else {
      double den = dg[s.v1 + e] - th;
      if (fabs(den) < guard) den = den >= 0.0 ? guard : -guard;
      t[e] = Rv[s.v1 + e] / den;
    }
  }
}

// h[i][j] = V_i[:, j] . t_i (t_i = column kk[i]) for j < kk[i]
__global__ void k_seg_proj(const int* __restrict__ ids, const Seg* __restrict__ seg, const int* __restrict__ kk,
                           int kmax, const double* __restrict__ V, double* __restrict__ hcoef) {
  __shared__ double sh[32];
  const int i = ids[blockIdx.y];
  const int j = blockIdx.x;
  if (j >= kk[i]) return;
  const Seg s = seg[i];
  const double* x = V + s.V + j * s.n;
  const double* t = V + s.V + kk[i] * s.n;
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < s.n; e += blockDim.x) acc = fma(x[e], t[e], acc);
  acc = bsum(acc, sh);
  if (threadIdx.x == 0) hcoef[(int64_t)i * kmax + j] = acc;
}

// t_i -= sum_j V_i[:, j] h[i][j]
__global__ void k_seg_sub(const int* __restrict__ ids, const Seg* __restrict__ seg, const int* __restrict__ kk,
                          int kmax, double* __restrict__ V, const double* __restrict__ hcoef) {
  const int i = ids[blockIdx.y];
  const Seg s = seg[i];
  const int k = kk[i];
  double* t = V + s.V + k * s.n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < s.n; e += (int64_t)gridDim.x * blockDim.x) {
    double v = t[e];
    for (int j = 0; j < k; ++j) v = fma(-V[s.V + j * s.n + e], hcoef[(int64_t)i * kmax + j], v);
    t[e] = v;
  }
}

// dst_i = src_i * f[i]; src/dst given as (buffer, column or -1 for v1 slots).
__global__ void k_seg_scale(const int* __restrict__ ids, const Seg* __restrict__ seg, const double* __restrict__ src,
                            int scol, const int* __restrict__ scolv, double* __restrict__ dst, int dcol,
                            const double* __restrict__ f, double* const* __restrict__ extdst) {
  const int i = ids[blockIdx.y];
  const Seg s = seg[i];
  const int sc = scolv ? scolv[i] : scol;
  const double* x = src + (sc >= 0 ? s.V + sc * s.n : s.v1);
  double* y = extdst ? extdst[i] : dst + (dcol >= 0 ? s.V + dcol * s.n : s.v1);
  const double a = f[i];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < s.n; e += (int64_t)gridDim.x * blockDim.x)
    y[e] = x[e] * a;
}

struct HeffPtrs {
  const double* L;
  const double* W1;
  const double* W2;
  const double* R;
};

__global__ void k_seg_weff(const HeffPtrs* __restrict__ hp, int wL, int wM, int wR, int d, double* __restrict__ Weff) {
  const int i = blockIdx.x;
  const int nc = wL * d * d, nj = d * d * wR;
  const double* W1 = hp[i].W1;
  const double* W2 = hp[i].W2;
  for (int t = threadIdx.x; t < nc * nj; t += blockDim.x) {
    const int c = t % nc, j = t / nc;
    const int w = c % wL, s1 = (c / wL) % d, s2 = c / (wL * d);
    const int s1p = j % d, s2p = (j / d) % d, y = j / (d * d);
    double s = 0.0;
    for (int x = 0; x < wM; ++x)
      s = fma(W1[w + wL * (s1p + d * (s1 + d * x))], W2[x + wM * (s2p + d * (s2 + d * y))], s);
    Weff[(int64_t)i * nc * nj + t] = s;
  }
}

__global__ void k_seg_diag(const HeffPtrs* __restrict__ hp, const Seg* __restrict__ seg, int d, int wL, int wM,
                           int wR, double* __restrict__ dg) {
  extern __shared__ double wd[];
  const int i = blockIdx.y;
  const Seg s = seg[i];
  const double* W1 = hp[i].W1;
  const double* W2 = hp[i].W2;
  const int nwd = wL * d * d * wR;
  for (int t = threadIdx.x; t < nwd; t += blockDim.x) {
    const int w = t % wL, s1 = (t / wL) % d, s2 = (t / (wL * d)) % d, y = t / (wL * d * d);
    double acc = 0.0;
    for (int x = 0; x < wM; ++x)
      acc = fma(W1[w + wL * (s1 + d * (s1 + d * x))], W2[x + wM * (s2 + d * (s2 + d * y))], acc);
    wd[t] = acc;
  }
  __syncthreads();
  const double* L = hp[i].L;
  const double* R = hp[i].R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < s.n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = e % s.chiL;
    int64_t rest = e / s.chiL;
    const int s1 = (int)(rest % d);
    rest /= d;
    const int s2 = (int)(rest % d);
    const int64_t b = rest / d;
    double acc = 0.0;
    for (int w = 0; w < wL; ++w) {
      const double lv = L[a + s.chiL * (w + (int64_t)wL * a)];
      for (int y = 0; y < wR; ++y)
        acc = fma(lv * wd[w + wL * (s1 + d * (s2 + d * y))], R[b + s.chiR * (y + (int64_t)wR * b)], acc);
    }
    dg[s.v1 + e] = acc;
  }
}

__global__ void k_seg_mid(const int* __restrict__ ids, const Seg* __restrict__ seg, const double* __restrict__ T1,
                          const double* __restrict__ Weff, double* __restrict__ T3, int nc, int nj) {
  extern __shared__ double wsh[];
  const int i = ids[blockIdx.y];
  const Seg s = seg[i];
  for (int t = threadIdx.x; t < nc * nj; t += blockDim.x) wsh[t] = Weff[(int64_t)i * nc * nj + t];
  __syncthreads();
  const double* t1 = T1 + s.t1;
  double* t3 = T3 + s.t3;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < s.rows; r += (int64_t)gridDim.x * blockDim.x) {
    for (int j0 = 0; j0 < nj; j0 += 8) {
      double acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = 0.0;
      for (int c = 0; c < nc; ++c) {
        const double x = t1[r + s.rows * c];
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (j0 + q < nj) acc[q] = fma(x, wsh[c + nc * (j0 + q)], acc[q]);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (j0 + q < nj) t3[r + s.rows * (j0 + q)] = acc[q];
    }
  }
}

void small_lowest(int k, const double* Gin, int ld, double& theta, std::vector<double>& y) {
  std::vector<double> G(k * k), Vm(k * k, 0.0);
  for (int a = 0; a < k; ++a)
    for (int b = 0; b < k; ++b) G[a + k * b] = 0.5 * (Gin[a + ld * b] + Gin[b + ld * a]);
  for (int i = 0; i < k; ++i) Vm[i + k * i] = 1.0;
  auto g = [&](int i, int j) -> double& { return G[i + k * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) {
        tot += g(i, j) * g(i, j);
        if (i != j) off += g(i, j) * g(i, j);
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < k - 1; ++p)
      for (int q = p + 1; q < k; ++q) {
        const double apq = g(p, q);
        if (apq == 0.0) continue;
        const double tau = (g(q, q) - g(p, p)) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int r = 0; r < k; ++r) {
          const double x = g(r, p), z = g(r, q);
          g(r, p) = c * x - s * z;
          g(r, q) = s * x + c * z;
        }
        for (int r = 0; r < k; ++r) {
          const double x = g(p, r), z = g(q, r);
          g(p, r) = c * x - s * z;
          g(q, r) = s * x + c * z;
        }
        for (int r = 0; r < k; ++r) {
          const double x = Vm[r + k * p], z = Vm[r + k * q];
          Vm[r + k * p] = c * x - s * z;
          Vm[r + k * q] = s * x + c * z;
        }
      }
  }
  int best = 0;
  for (int i = 1; i < k; ++i)
    if (g(i, i) < g(best, best)) best = i;
  theta = g(best, best);
  y.assign(Vm.begin() + k * best, Vm.begin() + k * (best + 1));
  int im = 0;
  for (int i = 1; i < k; ++i)
    if (fabs(y[i]) > fabs(y[im])) im = i;
  if (y[im] < 0)
    for (auto& v : y) v = -v;
}

}  // namespace

extern "C" int itg_davidson_heff2_batched(itg_handle* h, int count, const int64_t* chiL, const int64_t* chiR,
                                          int64_t d, int64_t wL, int64_t wM, int64_t wR,
                                          const double* const* L, const double* const* W1,
                                          const double* const* W2, const double* const* R,
                                          double* const* psi, int krylovdim, int maxiter, double tol,
                                          double* energy, int* nmatvec) {
  if (!h || count < 0 || (count > 0 && (!chiL || !chiR || !L || !W1 || !W2 || !R || !psi || !energy)))
    return ITG_ERR_INVALID;
  if (count == 0) return ITG_OK;
  if (d <= 0 || wL <= 0 || wM <= 0 || wR <= 0) return itg_fail(h, ITG_ERR_SHAPE, "batched davidson: bad dims");
  const int nc = (int)(wL * d * d), nj = (int)(d * d * wR);
  if ((int64_t)nc * nj * 8 > 48 * 1024) return itg_fail(h, ITG_ERR_UNSUPPORTED, "batched davidson: MPO block too large");
  const int kmax = krylovdim < 2 ? 2 : (krylovdim > 16 ? 16 : krylovdim);
  if (maxiter < 1) maxiter = 1;
  if ((int64_t)count * kmax * kmax > ITG_PINNED_DOUBLES)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "batched davidson: count * krylovdim^2 too large");
  // ---- layout
  std::vector<Seg> seg(count);
  int64_t vtot = 0, v1tot = 0, t1tot = 0, t3tot = 0, nmax = 0;
  auto al = [](int64_t x) { return (x + 31) & ~(int64_t)31; };
  for (int i = 0; i < count; ++i) {
    if (chiL[i] <= 0 || chiR[i] <= 0) return itg_fail(h, ITG_ERR_SHAPE, "batched davidson: bad chi");
    Seg& s = seg[i];
    s.chiL = chiL[i];
    s.chiR = chiR[i];
    s.n = chiL[i] * d * d * chiR[i];
    s.rows = chiL[i] * chiR[i];
    s.V = vtot;
    vtot += al(s.n * kmax);
    s.v1 = v1tot;
    v1tot += al(s.n);
    s.t1 = t1tot;
    t1tot += al(s.rows * nc);
    s.t3 = t3tot;
    t3tot += al(s.rows * nj);
    nmax = s.n > nmax ? s.n : nmax;
  }
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off += itg_align256(b); return o; };
  const size_t oV = take(8 * vtot), oAV = take(8 * vtot), oX = take(8 * v1tot), oHX = take(8 * v1tot),
               oR = take(8 * v1tot), oDg = take(8 * v1tot), oT1 = take(8 * t1tot), oT3 = take(8 * t3tot),
               oW = take(8 * (size_t)count * nc * nj), oSeg = take(sizeof(Seg) * count),
               oHp = take(sizeof(HeffPtrs) * count), oIds = take(sizeof(int) * count),
               oKk = take(sizeof(int) * count), oG = take(8 * (size_t)count * kmax * kmax),
               oY = take(8 * (size_t)count * kmax), oTh = take(8 * (size_t)count), oHc = take(8 * (size_t)count * kmax),
               oNr = take(8 * (size_t)count), oF = take(8 * (size_t)count), oCol = take(sizeof(int) * count),
               oPsi = take(sizeof(double*) * count);
  ITG_TRY(itg_scratch_reserve(h, off));
  char* base = (char*)h->scratch;
  double* V = (double*)(base + oV);
  double* AV = (double*)(base + oAV);
  double* X = (double*)(base + oX);
  double* HX = (double*)(base + oHX);
  double* Rv = (double*)(base + oR);
  double* dg = (double*)(base + oDg);
  double* T1 = (double*)(base + oT1);
  double* T3 = (double*)(base + oT3);
  double* Weff = (double*)(base + oW);
  Seg* dseg = (Seg*)(base + oSeg);
  HeffPtrs* dhp = (HeffPtrs*)(base + oHp);
  int* dids = (int*)(base + oIds);
  int* dkk = (int*)(base + oKk);
  double* dG = (double*)(base + oG);
  double* dY = (double*)(base + oY);
  double* dTh = (double*)(base + oTh);
  double* dHc = (double*)(base + oHc);
  double* dNr = (double*)(base + oNr);
  double* dF = (double*)(base + oF);
  int* dCol = (int*)(base + oCol);
  double** dPsi = (double**)(base + oPsi);
  std::vector<HeffPtrs> hps(count);
  for (int i = 0; i < count; ++i) hps[i] = {L[i], W1[i], W2[i], R[i]};
  ITG_CUDA(h, cudaMemcpyAsync(dseg, seg.data(), sizeof(Seg) * count, cudaMemcpyHostToDevice, h->stream));
  ITG_CUDA(h, cudaMemcpyAsync(dhp, hps.data(), sizeof(HeffPtrs) * count, cudaMemcpyHostToDevice, h->stream));
  ITG_CUDA(h, cudaMemcpyAsync(dPsi, psi, sizeof(double*) * count, cudaMemcpyHostToDevice, h->stream));
  const int gx = (int)((nmax + 255) / 256 < 64 ? (nmax + 255) / 256 : 64);
  k_seg_weff<<<count, 256, 0, h->stream>>>(dhp, (int)wL, (int)wM, (int)wR, (int)d, Weff);
  k_seg_diag<<<dim3(gx, count), 256, sizeof(double) * wL * d * d * wR, h->stream>>>(dhp, dseg, (int)d, (int)wL,
                                                                                   (int)wM, (int)wR, dg);
  ITG_CHECK_LAUNCH(h);

  // ---- host-side state
  std::vector<int> kk(count, 1), restart(count, 0), nmv(count, 0), done(count, 0), phase(count, 0);
  std::vector<double> theta(count, 0.0), rn(count, 0.0);
  std::vector<int> ids;
  double* hpin = h->pinned;
  auto upload_ids = [&](const std::vector<int>& v) -> int {
    ITG_CUDA(h, cudaMemcpyAsync(dids, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice, h->stream));
    return ITG_OK;
  };
  auto upload_kk = [&]() -> int {
    ITG_CUDA(h, cudaMemcpyAsync(dkk, kk.data(), sizeof(int) * count, cudaMemcpyHostToDevice, h->stream));
    return ITG_OK;
  };
  auto read = [&](const double* src, size_t nd) -> int {
    ITG_CUDA(h, cudaMemcpyAsync(hpin, src, 8 * nd, cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    return ITG_OK;
  };
  // grouped H_eff matvec for the instances in `v`, from column kcol[i] of V into AV
  auto matvec = [&](const std::vector<int>& v, const std::vector<int>& kcol) -> int {
    const int c = (int)v.size();
    if (!c) return ITG_OK;
    std::vector<const double*> a1(c), b1(c), a3(c), b3(c);
    std::vector<double*> c1(c), c3(c);
    std::vector<int64_t> dA1(3 * c), dB1(4 * c), dC1(5 * c), dA3(5 * c), dB3(3 * c), dC3(4 * c);
    for (int q = 0; q < c; ++q) {
      const int i = v[q];
      const Seg& s = seg[i];
      a1[q] = L[i];
      b1[q] = V + s.V + (int64_t)kcol[i] * s.n;
      c1[q] = T1 + s.t1;
      a3[q] = T3 + s.t3;
      b3[q] = R[i];
      c3[q] = AV + s.V + (int64_t)kcol[i] * s.n;
      const int64_t A1[3] = {s.chiL, wL, s.chiL}, B1[4] = {s.chiL, d, d, s.chiR}, C1[5] = {s.chiL, s.chiR, wL, d, d};
      const int64_t A3[5] = {s.chiL, s.chiR, d, d, wR}, B3[3] = {s.chiR, wR, s.chiR}, C3[4] = {s.chiL, d, d, s.chiR};
      for (int z = 0; z < 3; ++z) dA1[3 * q + z] = A1[z];
      for (int z = 0; z < 4; ++z) dB1[4 * q + z] = B1[z];
      for (int z = 0; z < 5; ++z) dC1[5 * q + z] = C1[z];
      for (int z = 0; z < 5; ++z) dA3[5 * q + z] = A3[z];
      for (int z = 0; z < 3; ++z) dB3[3 * q + z] = B3[z];
      for (int z = 0; z < 4; ++z) dC3[4 * q + z] = C3[z];
    }
    const int32_t mL[3] = {1, 2, 3}, mP[4] = {1, 4, 5, 6}, mT1[5] = {3, 6, 2, 4, 5};
    const int32_t mT3[5] = {3, 6, 7, 9, 10}, mR[3] = {6, 10, 11}, mO[4] = {3, 7, 9, 11};
    ITG_TRY(itg::contract_grouped_f64(h, c, 1.0, a1.data(), 3, dA1.data(), mL, b1.data(), 4, dB1.data(), mP,
                                      0.0, c1.data(), 5, dC1.data(), mT1));
    ITG_TRY(upload_ids(v));
    int64_t rmax = 0;
    for (int i : v) rmax = seg[i].rows > rmax ? seg[i].rows : rmax;
    const int gr = (int)((rmax + 255) / 256 < 64 ? (rmax + 255) / 256 : 64);
    k_seg_mid<<<dim3(gr, c), 256, sizeof(double) * nc * nj, h->stream>>>(dids, dseg, T1, Weff, T3, nc, nj);
    ITG_CHECK_LAUNCH(h);
    ITG_TRY(itg::contract_grouped_f64(h, c, 1.0, a3.data(), 5, dA3.data(), mT3, b3.data(), 3, dB3.data(), mR,
                                      0.0, c3.data(), 4, dC3.data(), mO));
    for (int i : v) nmv[i]++;
    return ITG_OK;
  };

  // ---- start: V0 = psi / |psi|, AV0 = H V0
  std::vector<int> all(count);
  for (int i = 0; i < count; ++i) all[i] = i;
  {
    // X_i = psi_i (external pointers), then V0 = X / |X|
    ITG_TRY(upload_ids(all));
    for (int i = 0; i < count; ++i)
      ITG_CUDA(h, cudaMemcpyAsync(X + seg[i].v1, psi[i], 8 * seg[i].n, cudaMemcpyDeviceToDevice, h->stream));
    k_seg_nrm<<<count, 256, 0, h->stream>>>(dids, dseg, X, -1, nullptr, dNr);
    ITG_CHECK_LAUNCH(h);
    ITG_TRY(read(dNr, count));
    std::vector<double> inv(count);
    for (int i = 0; i < count; ++i) {
      if (!(hpin[i] > 0.0)) return itg_fail(h, ITG_ERR_INVALID, "batched davidson: zero start vector %d", i);
      inv[i] = 1.0 / hpin[i];
    }
    ITG_CUDA(h, cudaMemcpyAsync(dF, inv.data(), 8 * count, cudaMemcpyHostToDevice, h->stream));
    k_seg_scale<<<dim3(gx, count), 256, 0, h->stream>>>(dids, dseg, X, -1, nullptr, V, 0, dF, nullptr);
    ITG_CHECK_LAUNCH(h);
    std::vector<int> col0(count, 0);
    ITG_TRY(matvec(all, col0));
  }
  std::vector<double> Gh, yv;
  std::vector<double> ycoef((size_t)count * kmax, 0.0);
  for (;;) {
    // Rayleigh-Ritz for every instance still running
    ids.clear();
    for (int i = 0; i < count; ++i)
      if (!done[i]) ids.push_back(i);
    if (ids.empty()) break;
    const int c = (int)ids.size();
    ITG_TRY(upload_ids(ids));
    ITG_TRY(upload_kk());
    k_seg_gram<<<dim3(kmax * kmax, c), 256, 0, h->stream>>>(dids, dseg, dkk, kmax, V, AV, dG);
    ITG_CHECK_LAUNCH(h);
    ITG_TRY(read(dG, (size_t)count * kmax * kmax));
    for (int i : ids) {
      small_lowest(kk[i], hpin + (size_t)i * kmax * kmax, kmax, theta[i], yv);
      for (int j = 0; j < kmax; ++j) ycoef[(size_t)i * kmax + j] = j < kk[i] ? yv[j] : 0.0;
    }
    ITG_CUDA(h, cudaMemcpyAsync(dY, ycoef.data(), 8 * (size_t)count * kmax, cudaMemcpyHostToDevice, h->stream));
    ITG_CUDA(h, cudaMemcpyAsync(dTh, theta.data(), 8 * (size_t)count, cudaMemcpyHostToDevice, h->stream));
    k_seg_ritz<<<dim3(gx, c), 256, 0, h->stream>>>(dids, dseg, dkk, kmax, V, AV, dY, dTh, X, HX, Rv);
    k_seg_nrm<<<c, 256, 0, h->stream>>>(dids, dseg, Rv, -1, nullptr, dNr);
    ITG_CHECK_LAUNCH(h);
    ITG_TRY(read(dNr, count));
    std::vector<int> grow, stop;
    for (int i : ids) {
      rn[i] = hpin[i];
      if (rn[i] < tol || kk[i] == kmax) stop.push_back(i);
      else grow.push_back(i);
    }
    // correction vectors for the instances that grow their basis
    std::vector<int> accepted;
    std::vector<double> tscale(count, 0.0);
    if (!grow.empty()) {
      std::vector<int> cur = grow;
      for (int attempt = 0; attempt < 2 && !cur.empty(); ++attempt) {
        const int cc = (int)cur.size();
        ITG_TRY(upload_ids(cur));
        k_seg_correction<<<dim3(gx, cc), 256, 0, h->stream>>>(dids, dseg, dkk, Rv, dg, dTh, attempt, V);
        ITG_CHECK_LAUNCH(h);
        std::vector<int> colk(count, 0);
        for (int i = 0; i < count; ++i) colk[i] = kk[i];
        ITG_CUDA(h, cudaMemcpyAsync(dCol, colk.data(), sizeof(int) * count, cudaMemcpyHostToDevice, h->stream));
        k_seg_nrm<<<cc, 256, 0, h->stream>>>(dids, dseg, V, 0, dCol, dNr);
        ITG_CHECK_LAUNCH(h);
        ITG_TRY(read(dNr, count));
        std::vector<double> t0(count, 0.0);
        for (int i : cur) t0[i] = hpin[i];
        for (int pass = 0; pass < 2; ++pass) {
          k_seg_proj<<<dim3(kmax, cc), 256, 0, h->stream>>>(dids, dseg, dkk, kmax, V, dHc);
          k_seg_sub<<<dim3(gx, cc), 256, 0, h->stream>>>(dids, dseg, dkk, kmax, V, dHc);
        }
        k_seg_nrm<<<cc, 256, 0, h->stream>>>(dids, dseg, V, 0, dCol, dNr);
        ITG_CHECK_LAUNCH(h);
        ITG_TRY(read(dNr, count));
        std::vector<int> retry;
        for (int i : cur) {
          const double tn = hpin[i];
          if (tn > 1e-6 * t0[i]) {
            if (tn > 1e-14) {
              accepted.push_back(i);
              tscale[i] = 1.0 / tn;
            } else {
              stop.push_back(i);
            }
          } else if (attempt == 0) {
            retry.push_back(i);
          } else {
            stop.push_back(i);
          }
        }
        cur = retry;
      }
    }
    if (!accepted.empty()) {
      ITG_CUDA(h, cudaMemcpyAsync(dF, tscale.data(), 8 * count, cudaMemcpyHostToDevice, h->stream));
      // normalise column kk[i] in place; one launch per distinct kk value
      std::vector<int> kvals;
      for (int i : accepted)
        if (std::find(kvals.begin(), kvals.end(), kk[i]) == kvals.end()) kvals.push_back(kk[i]);
      for (int kv : kvals) {
        std::vector<int> sub;
        for (int i : accepted)
          if (kk[i] == kv) sub.push_back(i);
        ITG_TRY(upload_ids(sub));
        k_seg_scale<<<dim3(gx, (int)sub.size()), 256, 0, h->stream>>>(dids, dseg, V, kv, nullptr, V, kv, dF, nullptr);
        ITG_CHECK_LAUNCH(h);
      }
      ITG_TRY(matvec(accepted, kk));
      for (int i : accepted) kk[i]++;
    }
    // instances whose inner loop ended: restart or finish
    std::vector<int> rs, fin;
    for (int i : stop) {
      if (rn[i] < tol || restart[i] == maxiter - 1) fin.push_back(i);
      else rs.push_back(i);
    }
    auto normalise_into = [&](const std::vector<int>& v, bool to_psi) -> int {
      if (v.empty()) return ITG_OK;
      ITG_TRY(upload_ids(v));
      k_seg_nrm<<<(int)v.size(), 256, 0, h->stream>>>(dids, dseg, X, -1, nullptr, dNr);
      ITG_CHECK_LAUNCH(h);
      ITG_TRY(read(dNr, count));
      std::vector<double> f(count, 0.0);
      for (int i : v) f[i] = 1.0 / hpin[i];
      ITG_CUDA(h, cudaMemcpyAsync(dF, f.data(), 8 * count, cudaMemcpyHostToDevice, h->stream));
      if (to_psi) {
        k_seg_scale<<<dim3(gx, (int)v.size()), 256, 0, h->stream>>>(dids, dseg, X, -1, nullptr, nullptr, 0, dF, dPsi);
      } else {
        k_seg_scale<<<dim3(gx, (int)v.size()), 256, 0, h->stream>>>(dids, dseg, X, -1, nullptr, V, 0, dF, nullptr);
        k_seg_scale<<<dim3(gx, (int)v.size()), 256, 0, h->stream>>>(dids, dseg, HX, -1, nullptr, AV, 0, dF, nullptr);
      }
      ITG_CHECK_LAUNCH(h);
      return ITG_OK;
    };
    ITG_TRY(normalise_into(rs, false));
    for (int i : rs) {
      kk[i] = 1;
      restart[i]++;
    }
    ITG_TRY(normalise_into(fin, true));
    for (int i : fin) done[i] = 1;
  }
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int i = 0; i < count; ++i) {
    energy[i] = theta[i];
    if (nmatvec) nmatvec[i] = nmv[i];
  }
  return ITG_OK;
}
