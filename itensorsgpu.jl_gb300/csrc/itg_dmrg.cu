// Two-site DMRG kernels: the effective-Hamiltonian matvec chain (K8) and the
// Davidson eigensolver that drives it.
//
// H_eff psi = L . W1 . W2 . R . psi is evaluated as
//   step 1 (gather-GEMM, 2 wL d^2 chiL^2 chiR flop):
//       T1[a', b, w, s1, s2] = sum_a L[a, w, a'] psi[a, s1, s2, b]
//   step 2 (small dense block, 2 chiL chiR (wL d^2)(d^2 wR) flop):
//       T3[a', b, s1', s2', y] = sum_{w,s1,s2} T1[a', b, w, s1, s2] Weff[w,s1,s2; s1',s2',y]
//       with Weff = sum_x W1[w, s1', s1, x] W2[x, s2', s2, y] formed once per call
//   step 3 (gather-GEMM, 2 chiL d^2 chiR^2 wR flop):
//       out[a', s1', s2', b'] = sum_{b,y} T3[a', b, s1', s2', y] R[b, y, b']
// Steps 1 and 3 carry the chi^3 work; they go through the contraction engine
// (FP64 or split precision) with cached plans.  Step 2 merges the two MPO
// tensors, which the ITensors ProjMPO product applies one at a time.
#include "itg_internal.cuh"

#include <cmath>
#include <vector>

namespace itg {
int get_plan(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA, int rankB,
             const int64_t* dimsB, const int32_t* modesB, int rankC, const int64_t* dimsC,
             const int32_t* modesC, std::shared_ptr<ContractPlan>& plan);
int run_plan(itg_handle* h, const ContractPlan& p, double alpha, const double* A, const double* B,
             double beta, double* C, int precision);
int heff_mid_split(itg_handle* h, int64_t R, int nc, int nj, const double* T1, const double* Weff, double* T3);
}  // namespace itg

namespace {

struct HeffDims {
  int64_t chiL, chiR, d, wL, wM, wR;
  int64_t n() const { return chiL * d * d * chiR; }
  int64_t t1() const { return chiL * chiR * wL * d * d; }
  int64_t t3() const { return chiL * chiR * d * d * wR; }
  int64_t nc() const { return wL * d * d; }
  int64_t nj() const { return d * d * wR; }
};

// Weff[c + nc*j], c = w + wL*(s1 + d*s2), j = s1p + d*(s2p + d*y)
__global__ void k_weff(const double* __restrict__ W1, const double* __restrict__ W2, int wL, int wM,
                       int wR, int d, double* __restrict__ Weff) {
  const int nc = wL * d * d, nj = d * d * wR;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nc * nj; t += gridDim.x * blockDim.x) {
    int c = t % nc, j = t / nc;
    int w = c % wL, s1 = (c / wL) % d, s2 = c / (wL * d);
    int s1p = j % d, s2p = (j / d) % d, y = j / (d * d);
    double s = 0.0;
    for (int x = 0; x < wM; ++x)
      s = fma(W1[w + wL * (s1p + d * (s1 + d * x))], W2[x + wM * (s2p + d * (s2 + d * y))], s);
    Weff[t] = s;
  }
}

// T3[r + R*j] = sum_c T1[r + R*c] * Weff[c + nc*j]   (R = chiL*chiR rows)
__global__ void __launch_bounds__(256)
k_heff_mid(const double* __restrict__ T1, const double* __restrict__ Weff, double* __restrict__ T3,
           int64_t R, int nc, int nj) {
  extern __shared__ double wsh[];
  for (int i = threadIdx.x; i < nc * nj; i += blockDim.x) wsh[i] = Weff[i];
  __syncthreads();
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < R;
       r += (int64_t)gridDim.x * blockDim.x) {
    for (int j0 = 0; j0 < nj; j0 += 8) {
      double acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = 0.0;
      for (int c = 0; c < nc; ++c) {
        double x = T1[r + R * c];
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (j0 + q < nj) acc[q] = fma(x, wsh[c + nc * (j0 + q)], acc[q]);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (j0 + q < nj) T3[r + R * (j0 + q)] = acc[q];
    }
  }
}

// diag(H_eff)[a', s1', s2', b'] = sum_{w,y} L[a',w,a'] Wd[w,s1',s2',y] R[b',y,b']
// with Wd[w,s1,s2,y] = sum_x W1[w,s1,s1,x] W2[x,s2,s2,y] formed per block in smem.
__global__ void k_heff_diag(const double* __restrict__ L, const double* __restrict__ W1,
                            const double* __restrict__ W2, const double* __restrict__ Rt,
                            int64_t chiL, int64_t chiR, int d, int wL, int wM, int wR,
                            double* __restrict__ dg) {
  extern __shared__ double wd[];
  const int nwd = wL * d * d * wR;
  for (int t = threadIdx.x; t < nwd; t += blockDim.x) {
    int w = t % wL, s1 = (t / wL) % d, s2 = (t / (wL * d)) % d, y = t / (wL * d * d);
    double s = 0.0;
    for (int x = 0; x < wM; ++x)
      s = fma(W1[w + wL * (s1 + d * (s1 + d * x))], W2[x + wM * (s2 + d * (s2 + d * y))], s);
    wd[t] = s;
  }
  __syncthreads();
  const int64_t n = chiL * d * d * chiR;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t a = e % chiL;
    int64_t rest = e / chiL;
    int s1 = (int)(rest % d);
    rest /= d;
    int s2 = (int)(rest % d);
    int64_t b = rest / d;
    double s = 0.0;
    for (int w = 0; w < wL; ++w) {
      double lv = L[a + chiL * (w + (int64_t)wL * a)];
      for (int y = 0; y < wR; ++y)
        s = fma(lv * wd[w + wL * (s1 + d * (s2 + d * y))], Rt[b + chiR * (y + (int64_t)wR * b)], s);
    }
    dg[e] = s;
  }
}

struct HeffWork {
  double* T1;
  double* T3;
  double* Weff;
};

size_t heff_work_bytes(const HeffDims& D) {
  return itg_align256(sizeof(double) * D.t1()) + itg_align256(sizeof(double) * D.t3()) +
         itg_align256(sizeof(double) * D.nc() * D.nj());
}

HeffWork heff_carve(const HeffDims& D, char* base) {
  HeffWork w;
  w.T1 = (double*)base;
  base += itg_align256(sizeof(double) * D.t1());
  w.T3 = (double*)base;
  base += itg_align256(sizeof(double) * D.t3());
  w.Weff = (double*)base;
  return w;
}

int heff_validate(itg_handle* h, const HeffDims& D) {
  if (D.chiL <= 0 || D.chiR <= 0 || D.d <= 0 || D.wL <= 0 || D.wM <= 0 || D.wR <= 0)
    return itg_fail(h, ITG_ERR_SHAPE, "heff2: non-positive dimension");
  if (D.nc() * D.nj() * 8 > 48 * 1024)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "heff2: MPO block (%lld x %lld) too large",
                    (long long)D.nc(), (long long)D.nj());
  return ITG_OK;
}

// Weff must already be formed in w.Weff.
int heff_apply(itg_handle* h, const HeffDims& D, const double* L, const double* R, const double* psi,
               double* out, const HeffWork& w, int precision) {
  const int64_t dL[3] = {D.chiL, D.wL, D.chiL};
  const int32_t mL[3] = {1, 2, 3};
  const int64_t dP[4] = {D.chiL, D.d, D.d, D.chiR};
  const int32_t mP[4] = {1, 4, 5, 6};
  const int64_t dT1[5] = {D.chiL, D.chiR, D.wL, D.d, D.d};
  const int32_t mT1[5] = {3, 6, 2, 4, 5};
  const int64_t dT3[5] = {D.chiL, D.chiR, D.d, D.d, D.wR};
  const int32_t mT3[5] = {3, 6, 7, 9, 10};
  const int64_t dR[3] = {D.chiR, D.wR, D.chiR};
  const int32_t mR[3] = {6, 10, 11};
  const int64_t dO[4] = {D.chiL, D.d, D.d, D.chiR};
  const int32_t mO[4] = {3, 7, 9, 11};
  std::shared_ptr<ContractPlan> p1, p3;
  ITG_TRY(itg::get_plan(h, 3, dL, mL, 4, dP, mP, 5, dT1, mT1, p1));
  ITG_TRY(itg::get_plan(h, 5, dT3, mT3, 3, dR, mR, 4, dO, mO, p3));
  // inside one Davidson solve L and R are constant: the split path keeps their
  // digit slices (step 1's A operand, step 3's B operand) after the first matvec
  const bool keep = h->heff_keep_env_slices && precision == ITG_PREC_SPLIT;
  h->slice_keep[0] = keep;
  const int st1 = itg::run_plan(h, *p1, 1.0, L, psi, 0.0, w.T1, precision);
  h->slice_keep[0] = false;
  ITG_TRY(st1);
  const int64_t Rrows = D.chiL * D.chiR;
  const int nc = (int)D.nc(), nj = (int)D.nj();
  // split precision: the middle step on the tensor cores by the same exact
  // digit products (nc, nj <= 32); otherwise FP64 FMA
  int mid = ITG_ERR_UNSUPPORTED;
  if (precision == ITG_PREC_SPLIT) mid = itg::heff_mid_split(h, Rrows, nc, nj, w.T1, w.Weff, w.T3);
  if (mid == ITG_ERR_UNSUPPORTED) {
    ProfScope prof(h, ITG_KERNEL_HEFF_MID);
    k_heff_mid<<<itg_blocks_for(Rrows, 256, h->num_sms * 8), 256, sizeof(double) * nc * nj, h->stream>>>(
        w.T1, w.Weff, w.T3, Rrows, nc, nj);
    ITG_CHECK_LAUNCH(h);
  } else {
    ITG_TRY(mid);
  }
  h->slice_keep[1] = keep;
  const int st3 = itg::run_plan(h, *p3, 1.0, w.T3, R, 0.0, out, precision);
  h->slice_keep[1] = false;
  ITG_TRY(st3);
  return ITG_OK;
}

int form_weff(itg_handle* h, const HeffDims& D, const double* W1, const double* W2, double* Weff) {
  k_weff<<<1, 256, 0, h->stream>>>(W1, W2, (int)D.wL, (int)D.wM, (int)D.wR, (int)D.d, Weff);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

// ---------------------------------------------------------- small eigen
// Lowest eigenpair of a small symmetric matrix (k <= 32) by cyclic Jacobi,
// on the host in FP64.
void small_sym_lowest(int k, std::vector<double> G, double& theta, std::vector<double>& y) {
  std::vector<double> Vm(k * k, 0.0);
  for (int i = 0; i < k; ++i) Vm[i + k * i] = 1.0;
  auto a = [&](int i, int j) -> double& { return G[i + k * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) {
        tot += a(i, j) * a(i, j);
        if (i != j) off += a(i, j) * a(i, j);
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < k - 1; ++p)
      for (int q = p + 1; q < k; ++q) {
        double apq = a(p, q);
        if (apq == 0.0) continue;
        double tau = (a(q, q) - a(p, p)) / (2.0 * apq);
        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int r = 0; r < k; ++r) {  // columns
          double x = a(r, p), z = a(r, q);
          a(r, p) = c * x - s * z;
          a(r, q) = s * x + c * z;
        }
        for (int r = 0; r < k; ++r) {  // rows
          double x = a(p, r), z = a(q, r);
          a(p, r) = c * x - s * z;
          a(q, r) = s * x + c * z;
        }
        for (int r = 0; r < k; ++r) {
          double x = Vm[r + k * p], z = Vm[r + k * q];
          Vm[r + k * p] = c * x - s * z;
          Vm[r + k * q] = s * x + c * z;
        }
      }
  }
  int best = 0;
  for (int i = 1; i < k; ++i)
    if (a(i, i) < a(best, best)) best = i;
  theta = a(best, best);
  y.assign(Vm.begin() + k * best, Vm.begin() + k * (best + 1));
  // fix the sign: largest-magnitude component positive
  int im = 0;
  for (int i = 1; i < k; ++i)
    if (fabs(y[i]) > fabs(y[im])) im = i;
  if (y[im] < 0)
    for (auto& v : y) v = -v;
}

// t = r / (diag - theta), the denominator kept at least `guard` in magnitude.
__global__ void k_precond(int64_t n, const double* __restrict__ r, const double* __restrict__ dg,
                          double theta, double guard, double* __restrict__ t) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double den = dg[i] - theta;
    if (fabs(den) < guard) den = (den >= 0.0) ? guard : -guard;
    t[i] = r[i] / den;
  }
}

// Per-element features of the learned preconditioner (F = 5, float, element-major):
//   f0 = r_e sqrt(n) / |r|                      (normalised residual)
//   f1 = (diag_e - theta) / scale               (scale = mean |diag - theta|)
//   f2 = clamp(scale / (diag_e - theta), -10, 10) / 10
//   f3 = log10(max(lamL[a], 1e-12)) / 12 + 0.5  (left Schmidt value of the element's a)
//   f4 = log10(max(lamR[b], 1e-12)) / 12 + 0.5  (right Schmidt value of its b)
// and the multiplier m = f0 * 10 f2: the diagonally preconditioned residual
// (normalised, with the clipped inverse).  The learned correction is
// t = (1 + g) m, so a network with g = 0 is the diagonal preconditioner and
// training learns a per-element correction to it.
__global__ void k_features(int64_t n, int64_t chiL, int64_t dd, const double* __restrict__ r,
                           const double* __restrict__ dg, double theta, double rscale, double dscale,
                           const double* __restrict__ lamL, const double* __restrict__ lamR,
                           float* __restrict__ X, float* __restrict__ mult) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = e % chiL, b = e / (chiL * dd);
    const double dv = dg[e] - theta;
    double inv = dscale / (fabs(dv) > 1e-300 ? dv : 1e-300);
    inv = inv > 10.0 ? 10.0 : (inv < -10.0 ? -10.0 : inv);
    const double f0 = r[e] * rscale;
    X[e * 5 + 0] = (float)f0;
    X[e * 5 + 1] = (float)(dv / dscale);
    X[e * 5 + 2] = (float)(inv / 10.0);
    X[e * 5 + 3] = lamL ? (float)(log10(fmax(lamL[a], 1e-12)) / 12.0 + 0.5) : 0.f;
    X[e * 5 + 4] = lamR ? (float)(log10(fmax(lamR[b], 1e-12)) / 12.0 + 0.5) : 0.f;
    mult[e] = (float)(f0 * inv);
  }
}

// t = (1 + g) * mult (the learned correction, in FP64)
__global__ void k_learned_corr(int64_t n, const float* __restrict__ g, const float* __restrict__ mult,
                               double* __restrict__ t) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    t[e] = (1.0 + (double)g[e]) * (double)mult[e];
}

// out[0] = sum |diag - theta| (block partial sums, reduced on the host side)
__global__ void k_abs_diff_sum(int64_t n, const double* __restrict__ dg, double theta, double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    s += fabs(dg[e] - theta);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
    part[blockIdx.x] = t;
  }
}

// y = a*x + b*y with host scalars (x, y length n); b == 0 ignores y's old contents.
__global__ void k_lincomb(int64_t n, double a, const double* __restrict__ x, double b,
                          double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (b == 0.0) ? a * x[i] : a * x[i] + b * y[i];
}

}  // namespace

namespace itg {
// Pieces of the H_eff chain for entry points that bring their own buffers.
int heff_form_weff(itg_handle* h, int64_t d, int64_t wL, int64_t wM, int64_t wR, const double* W1,
                   const double* W2, double* Weff) {
  HeffDims D{1, 1, d, wL, wM, wR};
  return form_weff(h, D, W1, W2, Weff);
}
int heff_mid(itg_handle* h, int64_t rows, int nc, int nj, const double* T1, const double* Weff,
             double* T3) {
  k_heff_mid<<<itg_blocks_for(rows, 256, h->num_sms * 8), 256, sizeof(double) * nc * nj, h->stream>>>(
      T1, Weff, T3, rows, nc, nj);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}
}  // namespace itg

extern "C" int itg_heff2_apply(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d, int64_t wL,
                               int64_t wM, int64_t wR, const double* L, const double* W1,
                               const double* W2, const double* R, const double* psi, double* out,
                               int precision) {
  if (!h || !L || !W1 || !W2 || !R || !psi || !out) return ITG_ERR_INVALID;
  if (psi == out) return itg_fail(h, ITG_ERR_INVALID, "out must not alias psi");
  HeffDims D{chiL, chiR, d, wL, wM, wR};
  ITG_TRY(heff_validate(h, D));
  ITG_TRY(itg_scratch_reserve(h, heff_work_bytes(D)));
  HeffWork w = heff_carve(D, (char*)h->scratch);
  ITG_TRY(form_weff(h, D, W1, W2, w.Weff));
  return heff_apply(h, D, L, R, psi, out, w, precision);
}

extern "C" int itg_heff2_diag(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d, int64_t wL,
                              int64_t wM, int64_t wR, const double* L, const double* W1,
                              const double* W2, const double* R, double* diag) {
  if (!h || !L || !W1 || !W2 || !R || !diag) return ITG_ERR_INVALID;
  HeffDims D{chiL, chiR, d, wL, wM, wR};
  ITG_TRY(heff_validate(h, D));
  const int nwd = (int)(D.wL * D.d * D.d * D.wR);
  k_heff_diag<<<itg_blocks_for(D.n(), 256, h->num_sms * 8), 256, sizeof(double) * nwd, h->stream>>>(
      L, W1, W2, R, chiL, chiR, (int)d, (int)wL, (int)wM, (int)wR, diag);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

namespace itg {
int mlp_forward(itg_handle* h, void* mlp, int64_t n, const float* X, float* g);
}

static int davidson_impl(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d, int64_t wL, int64_t wM,
                         int64_t wR, const double* L, const double* W1, const double* W2, const double* R,
                         double* psi, int krylovdim, int maxiter, double tol, int precision, void* mlp,
                         const double* lamL, const double* lamR, double* energy, int* nmatvec,
                         int* fallbacks);

extern "C" int itg_davidson_heff2(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d, int64_t wL,
                                  int64_t wM, int64_t wR, const double* L, const double* W1,
                                  const double* W2, const double* R, double* psi, int krylovdim,
                                  int maxiter, double tol, int precision, double* energy,
                                  int* nmatvec) {
  return davidson_impl(h, chiL, chiR, d, wL, wM, wR, L, W1, W2, R, psi, krylovdim, maxiter, tol, precision,
                       nullptr, nullptr, nullptr, energy, nmatvec, nullptr);
}

extern "C" int itg_davidson_heff2_learned(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d, int64_t wL,
                                          int64_t wM, int64_t wR, const double* L, const double* W1,
                                          const double* W2, const double* R, double* psi, int krylovdim,
                                          int maxiter, double tol, int precision, void* mlp,
                                          const double* lamL, const double* lamR, double* energy,
                                          int* nmatvec, int* fallbacks) {
  if (!mlp) return itg_fail(h, ITG_ERR_INVALID, "learned davidson needs a network");
  return davidson_impl(h, chiL, chiR, d, wL, wM, wR, L, W1, W2, R, psi, krylovdim, maxiter, tol, precision,
                       mlp, lamL, lamR, energy, nmatvec, fallbacks);
}

extern "C" int itg_heff2_features(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d, const double* r,
                                  const double* diag, double theta, const double* lamL, const double* lamR,
                                  float* X, float* mult) {
  if (!h || !r || !diag || !X || !mult || chiL <= 0 || chiR <= 0 || d <= 0) return ITG_ERR_INVALID;
  const int64_t n = chiL * d * d * chiR;
  ITG_TRY(itg_scratch_reserve(h, sizeof(double) * 600));
  double* part = (double*)h->scratch;
  const int nb = itg_blocks_for(n, 256, 512);
  k_abs_diff_sum<<<nb, 256, 0, h->stream>>>(n, diag, theta, part);
  ITG_CHECK_LAUNCH(h);
  std::vector<double> hp(nb);
  ITG_CUDA(h, cudaMemcpyAsync(hp.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
  double rn = 0.0;
  ITG_TRY(itg_nrm2(h, n, r, &rn));
  double ds = 0.0;
  for (double x : hp) ds += x;
  ds = ds / (double)n;
  if (!(ds > 0.0)) ds = 1.0;
  const double rs = rn > 0.0 ? std::sqrt((double)n) / rn : 0.0;
  k_features<<<itg_blocks_for(n, 256, h->num_sms * 8), 256, 0, h->stream>>>(n, chiL, d * d, r, diag, theta, rs,
                                                                           ds, lamL, lamR, X, mult);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

static int davidson_impl(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d, int64_t wL, int64_t wM,
                         int64_t wR, const double* L, const double* W1, const double* W2, const double* R,
                         double* psi, int krylovdim, int maxiter, double tol, int precision, void* mlp,
                         const double* lamL, const double* lamR, double* energy, int* nmatvec,
                         int* fallbacks) {
  if (!h || !L || !W1 || !W2 || !R || !psi || !energy) return ITG_ERR_INVALID;
  HeffDims D{chiL, chiR, d, wL, wM, wR};
  ITG_TRY(heff_validate(h, D));
  // L and R do not change during the solve: let the split matvecs keep their
  // digit slices; forget them when the solve ends, however it ends
  struct EnvSliceScope {
    itg_handle* h;
    explicit EnvSliceScope(itg_handle* hh) : h(hh) { h->heff_keep_env_slices = true; }
    ~EnvSliceScope() {
      h->heff_keep_env_slices = false;
      h->slice_cache[0].valid = false;
      h->slice_cache[1].valid = false;
    }
  } env_scope(h);
  const int kmax = krylovdim < 2 ? 2 : (krylovdim > 32 ? 32 : krylovdim);
  if (maxiter < 1) maxiter = 1;
  const int64_t n = D.n();
  // scratch: heff work | V (n*kmax) | AV (n*kmax) | dg | X | HX | Rv | small | partials
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += itg_align256(bytes); return o; };
  size_t oH = take(heff_work_bytes(D));
  size_t oV = take(sizeof(double) * n * kmax), oAV = take(sizeof(double) * n * kmax);
  size_t oDg = take(sizeof(double) * n), oX = take(sizeof(double) * n), oHX = take(sizeof(double) * n),
         oR = take(sizeof(double) * n), oSm = take(sizeof(double) * (kmax * kmax + 4 * kmax + 8)),
         oPart = take(sizeof(double) * 1024);
  size_t oXg = take(h->use_graphs ? sizeof(double) * n : 0), oYg = take(h->use_graphs ? sizeof(double) * n : 0);
  size_t oFx = take(mlp ? sizeof(float) * n * 5 : 0), oFm = take(mlp ? sizeof(float) * n : 0),
         oFg = take(mlp ? sizeof(float) * n : 0), oFp = take(mlp ? sizeof(double) * 600 : 0);
  ITG_TRY(itg_scratch_reserve(h, off));
  char* base = (char*)h->scratch;
  HeffWork w = heff_carve(D, base + oH);
  double* V = (double*)(base + oV);
  double* AV = (double*)(base + oAV);
  double* dg = (double*)(base + oDg);
  double* X = (double*)(base + oX);
  double* HX = (double*)(base + oHX);
  double* Rv = (double*)(base + oR);
  double* sm = (double*)(base + oSm);
  double* part = (double*)(base + oPart);
  double* Xg = (double*)(base + oXg);
  double* Yg = (double*)(base + oYg);
  float* Fx = (float*)(base + oFx);
  float* Fm = (float*)(base + oFm);
  float* Fg = (float*)(base + oFg);
  double* Fp = (double*)(base + oFp);
  bool use_learned = mlp != nullptr;
  int nfallback = 0;
  double rn_prev = -1.0;
  bool last_was_learned = false;
  double* hp = h->pinned;
  const int gb = itg_blocks_for(n, 256, h->num_sms * 8);

  auto nrm = [&](const double* x, double& out) -> int {
    ITG_TRY(itg::nrm2_dev(h, n, x, sm + kmax * kmax + 4 * kmax, part));
    ITG_CUDA(h, cudaMemcpyAsync(hp, sm + kmax * kmax + 4 * kmax, sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    out = hp[0];
    return ITG_OK;
  };
  // With graphs on, the chain is captured once per call (after a first direct
  // matvec has built the plans and sized the workspaces) with fixed input and
  // output buffers, then replayed for every further matvec.
  cudaGraphExec_t gexec = nullptr;
  auto matvec_direct = [&](const double* x, double* y) -> int {
    return heff_apply(h, D, L, R, x, y, w, precision);
  };
  auto matvec = [&](const double* x, double* y) -> int {
    if (!h->use_graphs || !gexec) return matvec_direct(x, y);
    ITG_CUDA(h, cudaMemcpyAsync(Xg, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    ITG_CUDA(h, cudaGraphLaunch(gexec, h->stream));
    ITG_CUDA(h, cudaMemcpyAsync(y, Yg, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    return ITG_OK;
  };
  auto capture = [&]() -> int {
    if (!h->cap_stream) ITG_CUDA(h, cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaStream_t saved = h->stream;
    const bool prof = h->prof_on;
    h->prof_on = false;
    h->stream = h->cap_stream;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal);
    int st = ITG_OK;
    if (e == cudaSuccess) {
      st = matvec_direct(Xg, Yg);
      e = cudaStreamEndCapture(h->cap_stream, &graph);
    }
    h->stream = saved;
    h->prof_on = prof;
    if (st != ITG_OK) return st;
    if (e != cudaSuccess) return itg_fail(h, ITG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return itg_fail(h, ITG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    return ITG_OK;
  };
  struct GraphGuard {
    cudaGraphExec_t* g;
    ~GraphGuard() { if (*g) cudaGraphExecDestroy(*g); }
  } gguard{&gexec};

  ITG_TRY(form_weff(h, D, W1, W2, w.Weff));
  {
    int nwd = (int)(D.wL * D.d * D.d * D.wR);
    k_heff_diag<<<gb, 256, sizeof(double) * nwd, h->stream>>>(L, W1, W2, R, chiL, chiR, (int)d,
                                                             (int)wL, (int)wM, (int)wR, dg);
    ITG_CHECK_LAUNCH(h);
  }
  double pn = 0.0;
  ITG_TRY(nrm(psi, pn));
  if (!(pn > 0.0)) return itg_fail(h, ITG_ERR_INVALID, "davidson: zero start vector");
  k_lincomb<<<gb, 256, 0, h->stream>>>(n, 1.0 / pn, psi, 0.0, V);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(matvec_direct(V, AV));
  if (h->use_graphs) ITG_TRY(capture());
  int nmv = 1;
  int k = 1;
  double theta = 0.0, rn = 0.0;
  std::vector<double> G, y;
  for (int restart = 0; restart < maxiter; ++restart) {
    for (;;) {
      // Rayleigh-Ritz on span(V[:, :k])
      for (int j = 0; j < k; ++j) {
        ITG_TRY(itg_gemv_t(h, n, k, V, n, AV + (int64_t)j * n, sm + (int64_t)j * k));
      }
      ITG_CUDA(h, cudaMemcpyAsync(hp, sm, sizeof(double) * k * k, cudaMemcpyDeviceToHost, h->stream));
      ITG_CUDA(h, cudaStreamSynchronize(h->stream));
      G.assign(k * k, 0.0);
      for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) G[i + k * j] = 0.5 * (hp[i + k * j] + hp[j + k * i]);
      small_sym_lowest(k, G, theta, y);
      for (int i = 0; i < k; ++i) hp[i] = y[i];
      ITG_CUDA(h, cudaMemcpyAsync(sm + kmax * kmax, hp, sizeof(double) * k, cudaMemcpyHostToDevice,
                                  h->stream));
      ITG_TRY(itg_gemv_n(h, n, k, V, n, sm + kmax * kmax, 0.0, X));
      ITG_TRY(itg_gemv_n(h, n, k, AV, n, sm + kmax * kmax, 0.0, HX));
      ITG_CUDA(h, cudaMemcpyAsync(Rv, HX, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
      k_lincomb<<<gb, 256, 0, h->stream>>>(n, -theta, X, 1.0, Rv);
      ITG_CHECK_LAUNCH(h);
      ITG_TRY(nrm(Rv, rn));
      // stall rule: a learned correction that did not cut the residual by 10%
      // hands the rest of this solve to the diagonal preconditioner
      if (last_was_learned && rn_prev > 0.0 && rn > 0.9 * rn_prev) {
        use_learned = false;
        nfallback++;
      }
      rn_prev = rn;
      last_was_learned = false;
      if (rn < tol || k == kmax) break;
      // correction t = (diag - theta)^-1 r, orthogonalised twice against V.  When
      // the orthogonalisation cancels all but 1e-6 of it (the preconditioned
      // residual lies almost in span(V)), the plain residual is used instead.
      double* t = V + (int64_t)k * n;
      const double guard = 1e-8 * (fabs(theta) > 1.0 ? fabs(theta) : 1.0);
      double tn = 0.0;
      for (int attempt = 0; attempt < 2; ++attempt) {
        if (attempt == 0 && use_learned) {
          // learned correction t = (1 + g(features)) * (diagonally preconditioned r_hat)
          const int nb = itg_blocks_for(n, 256, 512);
          k_abs_diff_sum<<<nb, 256, 0, h->stream>>>(n, dg, theta, Fp);
          ITG_CHECK_LAUNCH(h);
          ITG_CUDA(h, cudaMemcpyAsync(hp, Fp, sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
          ITG_CUDA(h, cudaStreamSynchronize(h->stream));
          double ds = 0.0;
          for (int q = 0; q < nb; ++q) ds += hp[q];
          ds /= (double)n;
          if (!(ds > 0.0)) ds = 1.0;
          const double rs = rn > 0.0 ? std::sqrt((double)n) / rn : 0.0;
          k_features<<<gb, 256, 0, h->stream>>>(n, chiL, d * d, Rv, dg, theta, rs, ds, lamL, lamR, Fx, Fm);
          ITG_CHECK_LAUNCH(h);
          ITG_TRY(itg::mlp_forward(h, mlp, n, Fx, Fg));
          k_learned_corr<<<gb, 256, 0, h->stream>>>(n, Fg, Fm, t);
          ITG_CHECK_LAUNCH(h);
          last_was_learned = true;
        } else if (attempt == 0) {
          k_precond<<<gb, 256, 0, h->stream>>>(n, Rv, dg, theta, guard, t);
          ITG_CHECK_LAUNCH(h);
        } else {
          last_was_learned = false;
          ITG_CUDA(h, cudaMemcpyAsync(t, Rv, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
        }
        double t0 = 0.0;
        ITG_TRY(nrm(t, t0));
        for (int pass = 0; pass < 2; ++pass) {
          ITG_TRY(itg_gemv_t(h, n, k, V, n, t, sm + kmax * kmax + kmax));
          ITG_TRY(itg_scal(h, k, -1.0, sm + kmax * kmax + kmax));
          ITG_TRY(itg_gemv_n(h, n, k, V, n, sm + kmax * kmax + kmax, 1.0, t));
        }
        ITG_TRY(nrm(t, tn));
        if (tn > 1e-6 * t0) break;
        tn = 0.0;
      }
      if (!(tn > 1e-14)) break;
      ITG_TRY(itg_scal(h, n, 1.0 / tn, t));
      ITG_TRY(matvec(t, AV + (int64_t)k * n));
      nmv++;
      k++;
    }
    if (rn < tol || restart == maxiter - 1) break;
    double xn = 0.0;
    ITG_TRY(nrm(X, xn));
    k_lincomb<<<gb, 256, 0, h->stream>>>(n, 1.0 / xn, X, 0.0, V);
    k_lincomb<<<gb, 256, 0, h->stream>>>(n, 1.0 / xn, HX, 0.0, AV);
    ITG_CHECK_LAUNCH(h);
    k = 1;
  }
  double xn = 0.0;
  ITG_TRY(nrm(X, xn));
  k_lincomb<<<gb, 256, 0, h->stream>>>(n, 1.0 / xn, X, 0.0, psi);
  ITG_CHECK_LAUNCH(h);
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  *energy = theta;
  if (nmatvec) *nmatvec = nmv;
  if (fallbacks) *fallbacks = nfallback;
  return ITG_OK;
}
