// Complex FP64 tensors (ITG_C64) on the real engine.
//
// Storage is interleaved (re, im), the layout of Julia's ComplexF64, C99
// double _Complex and torch.complex128.  A complex tensor of dims D is the
// real tensor of dims (2, D...) whose first mode is re/im, so:
//   * permute, axpby and real-diagonal contractions with real scalars carry
//     the re/im mode along (itg_permute.cu, itg_diag.cu);
//   * complex x real: the complex operand's re/im mode passes through to C;
//   * complex x complex: the smaller operand X is expanded into its real
//     representation Xh[b, c, x] = sum_a M[a, b, c] X[a, x] with the complex
//     multiplication table M (M[0,0,0] = 1, M[1,1,0] = -1, M[0,1,1] =
//     M[1,0,1] = 1), i.e. Xh[0,0] = Xr, Xh[1,0] = -Xi, Xh[0,1] = Xi,
//     Xh[1,1] = Xr; then C[c, ...] = sum_{b, shared} Xh[b, c, ...] Y[b, ...]
//     is one real contraction with M' = 2M and K' = 2K: 8MNK real flops, the
//     work of four real GEMMs, on the FP64 or split-precision engine.
// Complex scalars other than real alpha / beta go through a temporary and
// k_zaxpby.  Replaces the ComplexF64 methods of the reference's storage
// overloads (src/tensor/cudense.jl contract!!, permute!, +/-; exercised by
// test/test_cucontract.jl:9, test/test_cudense.jl:9, test/test_cuitensor.jl:10).
#include "itg_internal.cuh"

#include <algorithm>
#include <vector>

namespace {

__global__ void k_realify(int64_t n, const double* __restrict__ X, double* __restrict__ Xh) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double re = X[2 * i], im = X[2 * i + 1];
    double* o = Xh + 4 * i;
    o[0] = re;   // (b=0, c=0)
    o[1] = -im;  // (b=1, c=0)
    o[2] = im;   // (b=0, c=1)
    o[3] = re;   // (b=1, c=1)
  }
}

// C = alpha * T + beta * C, complex scalars, n complex elements.
// T may alias C (itg_zscal).
__global__ void k_zaxpby(int64_t n, double ar, double ai, const double* T, double br, double bi, double* C,
                         int use_c) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double tr = T[2 * i], ti = T[2 * i + 1];
    double cr = ar * tr - ai * ti, ci = ar * ti + ai * tr;
    if (use_c) {
      const double xr = C[2 * i], xi = C[2 * i + 1];
      cr += br * xr - bi * xi;
      ci += br * xi + bi * xr;
    }
    C[2 * i] = cr;
    C[2 * i + 1] = ci;
  }
}

// Y may alias X.
__global__ void k_conj(int64_t n, const double* X, double* Y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    Y[2 * i] = X[2 * i];
    Y[2 * i + 1] = -X[2 * i + 1];
  }
}

__global__ void k_real_to_complex(int64_t n, const double* __restrict__ X, double* __restrict__ Z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    Z[2 * i] = X[i];
    Z[2 * i + 1] = 0.0;
  }
}

int64_t prod(int r, const int64_t* d) {
  int64_t p = 1;
  for (int i = 0; i < r; ++i) p *= d[i];
  return p;
}

// A label not used by any of the three mode lists, plus `k`.
int32_t free_label(int ra, const int32_t* ma, int rb, const int32_t* mb, int rc, const int32_t* mc, int k) {
  int32_t mx = 0;
  for (int i = 0; i < ra; ++i) mx = std::max(mx, ma[i]);
  for (int i = 0; i < rb; ++i) mx = std::max(mx, mb[i]);
  for (int i = 0; i < rc; ++i) mx = std::max(mx, mc[i]);
  return mx + 1 + k;
}

// (lead..., dims...) / (lead..., modes...)
void with_lead(std::vector<int64_t>& d, std::vector<int32_t>& m, std::initializer_list<int32_t> lead, int r,
               const int64_t* dims, const int32_t* modes) {
  d.clear();
  m.clear();
  for (int32_t l : lead) {
    d.push_back(2);
    m.push_back(l);
  }
  for (int i = 0; i < r; ++i) {
    d.push_back(dims[i]);
    m.push_back(modes[i]);
  }
}

int cplx_reserve(itg_handle* h, size_t bytes) {
  if (bytes <= h->cplx_buf_bytes) return ITG_OK;
  if (h->cplx_buf) {
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->cplx_buf);
    h->cplx_buf = nullptr;
    h->cplx_buf_bytes = 0;
  }
  const size_t want = itg_align256(bytes + bytes / 4);
  if (cudaMalloc(&h->cplx_buf, want) != cudaSuccess) {
    h->cplx_buf = nullptr;
    return itg_fail(h, ITG_ERR_ALLOC, "complex workspace of %zu bytes failed", want);
  }
  h->cplx_buf_bytes = want;
  return ITG_OK;
}

}  // namespace

namespace itg {

// Complex and mixed contraction: dtypeA / dtypeB in {ITG_F64, ITG_C64}; C is
// complex when either operand is.  alpha = (ar, ai), beta = (br, bi).
int contract_z(itg_handle* h, int dtA, int dtB, double ar, double ai, const double* A, int rankA,
               const int64_t* dimsA, const int32_t* modesA, const double* B, int rankB, const int64_t* dimsB,
               const int32_t* modesB, double br, double bi, double* C, int rankC, const int64_t* dimsC,
               const int32_t* modesC, int precision) {
  const bool ca = dtA == ITG_C64, cb = dtB == ITG_C64;
  if (!ca && !cb) {
    if (ai != 0.0 || bi != 0.0) return itg_fail(h, ITG_ERR_INVALID, "complex scalars on a real contraction");
    return contract_f64(h, ar, A, rankA, dimsA, modesA, B, rankB, dimsB, modesB, br, C, rankC, dimsC, modesC,
                        precision);
  }
  if (std::max(rankA, std::max(rankB, rankC)) + 2 > ITG_MAX_RANK)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "complex contraction of rank above %d", ITG_MAX_RANK - 2);
  const int64_t nA = prod(rankA, dimsA), nB = prod(rankB, dimsB), nC = prod(rankC, dimsC);
  const bool real_scalars = ai == 0.0 && bi == 0.0;
  // With complex scalars the product goes to a temporary T, then C = alpha T + beta C.
  const bool both = ca && cb;
  const bool expandA = both && nA <= nB;
  size_t off = 0;
  const size_t oX = off;
  if (both) off += itg_align256(sizeof(double) * 4 * (size_t)(expandA ? nA : nB));
  const size_t oT = off;
  if (!real_scalars) off += itg_align256(sizeof(double) * 2 * (size_t)nC);
  if (off) ITG_TRY(cplx_reserve(h, off));
  char* base = (char*)h->cplx_buf;
  double* target = real_scalars ? C : (double*)(base + oT);
  const double a0 = real_scalars ? ar : 1.0, b0 = real_scalars ? br : 0.0;
  const int32_t lc = free_label(rankA, modesA, rankB, modesB, rankC, modesC, 0);
  const int32_t lb = lc + 1;
  std::vector<int64_t> dA, dB, dC;
  std::vector<int32_t> mA, mB, mC;
  with_lead(dC, mC, {lc}, rankC, dimsC, modesC);
  if (!both) {
    if (ca) {
      with_lead(dA, mA, {lc}, rankA, dimsA, modesA);
      with_lead(dB, mB, {}, rankB, dimsB, modesB);
    } else {
      with_lead(dA, mA, {}, rankA, dimsA, modesA);
      with_lead(dB, mB, {lc}, rankB, dimsB, modesB);
    }
    ITG_TRY(contract_f64(h, a0, A, (int)dA.size(), dA.data(), mA.data(), B, (int)dB.size(), dB.data(), mB.data(),
                         b0, target, (int)dC.size(), dC.data(), mC.data(), precision));
  } else {
    double* Xh = (double*)(base + oX);
    const double* X = expandA ? A : B;
    const int64_t nX = expandA ? nA : nB;
    if (nX > 0) {
      k_realify<<<itg_blocks_for(nX, 256, h->num_sms * 16), 256, 0, h->stream>>>(nX, X, Xh);
      ITG_CHECK_LAUNCH(h);
    }
    if (expandA) {
      with_lead(dA, mA, {lb, lc}, rankA, dimsA, modesA);
      with_lead(dB, mB, {lb}, rankB, dimsB, modesB);
      ITG_TRY(contract_f64(h, a0, Xh, (int)dA.size(), dA.data(), mA.data(), B, (int)dB.size(), dB.data(),
                           mB.data(), b0, target, (int)dC.size(), dC.data(), mC.data(), precision));
    } else {
      with_lead(dA, mA, {lb}, rankA, dimsA, modesA);
      with_lead(dB, mB, {lb, lc}, rankB, dimsB, modesB);
      ITG_TRY(contract_f64(h, a0, A, (int)dA.size(), dA.data(), mA.data(), Xh, (int)dB.size(), dB.data(),
                           mB.data(), b0, target, (int)dC.size(), dC.data(), mC.data(), precision));
    }
  }
  if (!real_scalars && nC > 0) {
    k_zaxpby<<<itg_blocks_for(nC, 256, h->num_sms * 16), 256, 0, h->stream>>>(nC, ar, ai, target, br, bi, C,
                                                                           (br != 0.0 || bi != 0.0) ? 1 : 0);
    ITG_CHECK_LAUNCH(h);
  }
  return ITG_OK;
}

}  // namespace itg

extern "C" int itg_contract_z(itg_handle* h, int dtypeA, int dtypeB, const double* alpha, const void* A, int rankA,
                              const int64_t* dimsA, const int32_t* modesA, const void* B, int rankB,
                              const int64_t* dimsB, const int32_t* modesB, const double* beta, void* C, int rankC,
                              const int64_t* dimsC, const int32_t* modesC, int precision) {
  if (!h) return ITG_ERR_INVALID;
  if ((dtypeA != ITG_F64 && dtypeA != ITG_C64) || (dtypeB != ITG_F64 && dtypeB != ITG_C64))
    return itg_fail(h, ITG_ERR_INVALID, "dtypes %d, %d", dtypeA, dtypeB);
  if (!alpha || !beta) return itg_fail(h, ITG_ERR_INVALID, "null scalar");
  if (precision != ITG_PREC_FP64 && precision != ITG_PREC_SPLIT)
    return itg_fail(h, ITG_ERR_INVALID, "unknown precision %d", precision);
  if (rankA < 0 || rankB < 0 || rankC < 0 || rankA > ITG_MAX_RANK || rankB > ITG_MAX_RANK || rankC > ITG_MAX_RANK)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank outside 0..%d", ITG_MAX_RANK);
  if ((rankA && (!dimsA || !modesA)) || (rankB && (!dimsB || !modesB)) || (rankC && (!dimsC || !modesC)))
    return itg_fail(h, ITG_ERR_INVALID, "null dims/modes");
  if (!A || !B || !C) return itg_fail(h, ITG_ERR_INVALID, "null tensor pointer");
  if (C == A || C == B) return itg_fail(h, ITG_ERR_INVALID, "C must not alias A or B");
  for (int i = 0; i < rankA; ++i)
    if (dimsA[i] < 0) return itg_fail(h, ITG_ERR_SHAPE, "negative dimension");
  for (int i = 0; i < rankB; ++i)
    if (dimsB[i] < 0) return itg_fail(h, ITG_ERR_SHAPE, "negative dimension");
  for (int i = 0; i < rankC; ++i)
    if (dimsC[i] < 0) return itg_fail(h, ITG_ERR_SHAPE, "negative dimension");
  return itg::contract_z(h, dtypeA, dtypeB, alpha[0], alpha[1], (const double*)A, rankA, dimsA, modesA,
                         (const double*)B, rankB, dimsB, modesB, beta[0], beta[1], (double*)C, rankC, dimsC, modesC,
                         precision);
}

extern "C" int itg_conj(itg_handle* h, int64_t n, const double* x, double* y) {
  if (!h || n < 0 || (n > 0 && (!x || !y))) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_conj<<<itg_blocks_for(n, 256, h->num_sms * 16), 256, 0, h->stream>>>(n, x, y);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_real_to_complex(itg_handle* h, int64_t n, const double* x, double* z) {
  if (!h || n < 0 || (n > 0 && (!x || !z))) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  if ((const void*)x == (const void*)z) return itg_fail(h, ITG_ERR_INVALID, "z must not alias x");
  k_real_to_complex<<<itg_blocks_for(n, 256, h->num_sms * 16), 256, 0, h->stream>>>(n, x, z);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_zscal(itg_handle* h, int64_t n, const double* alpha, double* x) {
  if (!h || n < 0 || !alpha || (n > 0 && !x)) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_zaxpby<<<itg_blocks_for(n, 256, h->num_sms * 16), 256, 0, h->stream>>>(n, alpha[0], alpha[1], x, 0.0, 0.0, x, 0);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}
