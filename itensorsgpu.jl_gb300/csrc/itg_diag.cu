// Diagonal-tensor contractions (K4): gather/scale kernels instead of the
// densify-then-GEMM path of src/tensor/cudiag.jl:147-161.
//
// A Diag tensor D with modes (d_0 .. d_{r-1}) holds D[i, i, ..., i] = d[i]
// (or d[0] for every i when uniform).  Contracting it with a dense tensor T:
//   Dc = D's modes shared with T (summed), Df = D's modes that stay in C.
//   If Df is empty:  C[c] = alpha * sum_i d[i] * T[c's T-modes, Dc-modes = i]
//   else:            i is C's index on Df (all Df indices equal, else 0) and
//                    C[c] = alpha * d[i] * T[c's T-modes, Dc-modes = i]
// Every output element is written once; traffic is |C| + |T| + |d| doubles.
#include "itg_internal.cuh"

#include <algorithm>

namespace {

struct DiagDesc {
  int rankC;
  int64_t dimsC[ITG_MAX_RANK];
  int64_t strT[ITG_MAX_RANK];  // stride in T of C's mode (0 when it is a Df mode)
  int isDf[ITG_MAX_RANK];      // C's mode belongs to D
  int64_t sumDc;               // sum of T strides of Dc modes (index i along all of them)
  int64_t ndiag;               // diagonal length
  int hasDf;
};

__global__ void k_diag_dense(const double* __restrict__ d, int uniform, const double* __restrict__ T,
                             double* __restrict__ C, int64_t totalC, DiagDesc desc, double alpha,
                             double beta) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < totalC;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = c, toff = 0, di = -1;
    bool ok = true;
    for (int k = 0; k < desc.rankC; ++k) {
      int64_t dk = desc.dimsC[k];
      int64_t q = rem / dk;
      int64_t idx = rem - q * dk;
      rem = q;
      if (desc.isDf[k]) {
        if (di < 0) di = idx;
        else if (di != idx) ok = false;
      } else {
        toff += idx * desc.strT[k];
      }
    }
    double v = 0.0;
    if (desc.hasDf) {
      if (ok && di < desc.ndiag) {
        double dv = uniform ? d[0] : d[di];
        v = dv * T[toff + di * desc.sumDc];
      }
    } else {
      for (int64_t i = 0; i < desc.ndiag; ++i) {
        double dv = uniform ? d[0] : d[i];
        v = fma(dv, T[toff + i * desc.sumDc], v);
      }
    }
    v *= alpha;
    if (beta != 0.0) v = fma(beta, C[c], v);
    C[c] = v;
  }
}

// Row form of k_diag_dense for the usual shape (one Df mode in C): C is
// walked row by row along its mode 0, whose T stride is 1 (row_df = 0: the
// diagonal index is fixed along the row) or which is the Df mode itself with
// the diagonal's T stride sumDc (row_df = 1).  The index arithmetic runs
// once per row, so the element loop is a plain scaled stream.
struct RowDesc {
  int n;                        // C modes 1.. (the row index decomposition)
  int64_t dims[ITG_MAX_RANK];
  int64_t strT[ITG_MAX_RANK];
  int64_t strC[ITG_MAX_RANK];
  int df;                       // position among them of the Df mode, -1 when it is mode 0
};

__global__ void k_diag_rows(const double* __restrict__ d, int uniform, const double* __restrict__ T,
                            double* __restrict__ C, int64_t len, int64_t nrows, RowDesc r, int64_t sumDc,
                            int64_t ndiag, double alpha, double beta) {
  for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
    int64_t rem = row, toff = 0, coff = 0, di = -1;
    for (int k = 0; k < r.n; ++k) {
      const int64_t q = rem / r.dims[k];
      const int64_t idx = rem - q * r.dims[k];
      rem = q;
      coff += idx * r.strC[k];
      if (k == r.df) di = idx;
      else toff += idx * r.strT[k];
    }
    double* c = C + coff;
    if (r.df >= 0) {  // diagonal index fixed along the row, T contiguous
      const double dv = di < ndiag ? alpha * (uniform ? d[0] : d[di]) : 0.0;
      const double* t = T + toff + di * sumDc;
      for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
        double v = di < ndiag ? dv * t[i] : 0.0;
        if (beta != 0.0) v = fma(beta, c[i], v);
        c[i] = v;
      }
    } else {          // the row runs along the diagonal index
      const double* t = T + toff;
      for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
        double v = i < ndiag ? alpha * (uniform ? d[0] : d[i]) * t[i * sumDc] : 0.0;
        if (beta != 0.0) v = fma(beta, c[i], v);
        c[i] = v;
      }
    }
  }
}

__global__ void k_diag_diag(int64_t n, double alpha, const double* __restrict__ a, int au,
                            const double* __restrict__ b, int bu, double* __restrict__ c) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    c[i] = alpha * (au ? a[0] : a[i]) * (bu ? b[0] : b[i]);
}

__global__ void k_diag_scatter(const double* __restrict__ d, int uniform, int64_t ndiag,
                               int64_t step, double* __restrict__ T) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ndiag;
       i += (int64_t)gridDim.x * blockDim.x)
    T[i * step] = uniform ? d[0] : d[i];
}

}  // namespace

extern "C" int itg_diag_contract(itg_handle* h, int dtype, double alpha, const double* d,
                                 int uniform, int rankD, const int64_t* dimsD,
                                 const int32_t* modesD, const void* Tv, int rankT,
                                 const int64_t* dimsT, const int32_t* modesT, double beta, void* Cv,
                                 int rankC, const int64_t* dimsC, const int32_t* modesC) {
  if (!h) return ITG_ERR_INVALID;
  if (dtype != ITG_F64 && dtype != ITG_C64) return itg_fail(h, ITG_ERR_UNSUPPORTED, "dtype %d", dtype);
  if (!d || !Tv || !Cv) return itg_fail(h, ITG_ERR_INVALID, "null pointer");
  if (dtype == ITG_C64) {
    // real diagonal x complex dense: the re/im mode of T passes to C
    if (rankT + 1 > ITG_MAX_RANK || rankC + 1 > ITG_MAX_RANK || rankD < 1 || rankD > ITG_MAX_RANK || rankT < 0 ||
        rankC < 0)
      return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank out of range");
    int32_t c = 0;
    for (int i = 0; i < rankD; ++i) c = modesD[i] > c ? modesD[i] : c;
    for (int i = 0; i < rankT; ++i) c = modesT[i] > c ? modesT[i] : c;
    for (int i = 0; i < rankC; ++i) c = modesC[i] > c ? modesC[i] : c;
    ++c;
    int64_t dT[ITG_MAX_RANK], dC[ITG_MAX_RANK];
    int32_t mT[ITG_MAX_RANK], mC[ITG_MAX_RANK];
    dT[0] = dC[0] = 2;
    mT[0] = mC[0] = c;
    for (int i = 0; i < rankT; ++i) { dT[i + 1] = dimsT[i]; mT[i + 1] = modesT[i]; }
    for (int i = 0; i < rankC; ++i) { dC[i + 1] = dimsC[i]; mC[i + 1] = modesC[i]; }
    return itg_diag_contract(h, ITG_F64, alpha, d, uniform, rankD, dimsD, modesD, Tv, rankT + 1, dT, mT, beta, Cv,
                             rankC + 1, dC, mC);
  }
  if (rankD < 1 || rankD > ITG_MAX_RANK || rankT < 0 || rankT > ITG_MAX_RANK || rankC < 0 ||
      rankC > ITG_MAX_RANK)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank out of range");
  const double* T = (const double*)Tv;
  double* C = (double*)Cv;
  int64_t ndiag = dimsD[0];
  for (int i = 1; i < rankD; ++i) ndiag = dimsD[i] < ndiag ? dimsD[i] : ndiag;
  int64_t sT[ITG_MAX_RANK];
  {
    int64_t s = 1;
    for (int i = 0; i < rankT; ++i) { sT[i] = s; s *= dimsT[i]; }
  }
  auto pos = [](int r, const int32_t* m, int32_t x) {
    for (int i = 0; i < r; ++i)
      if (m[i] == x) return i;
    return -1;
  };
  DiagDesc desc;
  desc.rankC = rankC;
  desc.sumDc = 0;
  desc.ndiag = ndiag;
  desc.hasDf = 0;
  for (int i = 0; i < rankD; ++i) {
    int it = pos(rankT, modesT, modesD[i]);
    int ic = pos(rankC, modesC, modesD[i]);
    if (it >= 0 && ic >= 0)
      return itg_fail(h, ITG_ERR_UNSUPPORTED, "mode %d in D, T and C", modesD[i]);
    if (it < 0 && ic < 0) return itg_fail(h, ITG_ERR_SHAPE, "mode %d of D unused", modesD[i]);
    if (it >= 0) {
      if (dimsT[it] != dimsD[i]) return itg_fail(h, ITG_ERR_SHAPE, "dimension mismatch on mode %d", modesD[i]);
      desc.sumDc += sT[it];
    }
  }
  for (int i = 0; i < rankT; ++i)
    if (pos(rankD, modesD, modesT[i]) < 0 && pos(rankC, modesC, modesT[i]) < 0)
      return itg_fail(h, ITG_ERR_UNSUPPORTED, "mode %d of T is in neither D nor C", modesT[i]);
  int64_t totalC = 1;
  for (int k = 0; k < rankC; ++k) {
    desc.dimsC[k] = dimsC[k];
    totalC *= dimsC[k];
    int id = pos(rankD, modesD, modesC[k]);
    int it = pos(rankT, modesT, modesC[k]);
    if (id >= 0) {
      if (dimsD[id] != dimsC[k]) return itg_fail(h, ITG_ERR_SHAPE, "dimension mismatch on mode %d", modesC[k]);
      desc.isDf[k] = 1;
      desc.strT[k] = 0;
      desc.hasDf = 1;
    } else if (it >= 0) {
      if (dimsT[it] != dimsC[k]) return itg_fail(h, ITG_ERR_SHAPE, "dimension mismatch on mode %d", modesC[k]);
      desc.isDf[k] = 0;
      desc.strT[k] = sT[it];
    } else {
      return itg_fail(h, ITG_ERR_SHAPE, "mode %d of C in neither D nor T", modesC[k]);
    }
  }
  if (totalC == 0) return ITG_OK;
  // Row form: exactly one Df mode in C, and C's mode 0 either a T mode of
  // stride 1 or that Df mode itself.
  int ndf = 0;
  for (int k = 0; k < rankC; ++k) ndf += desc.isDf[k];
  const bool row0_t = rankC > 0 && !desc.isDf[0] && desc.strT[0] == 1;
  const bool row0_df = rankC > 0 && desc.isDf[0];
  if (ndf == 1 && (row0_t || row0_df) && dimsC[0] >= 32) {
    RowDesc r;
    r.n = 0;
    r.df = -1;
    int64_t sc = dimsC[0];
    for (int k = 1; k < rankC; ++k) {
      r.dims[r.n] = dimsC[k];
      r.strT[r.n] = desc.strT[k];
      r.strC[r.n] = sc;
      if (desc.isDf[k]) r.df = r.n;
      sc *= dimsC[k];
      r.n++;
    }
    const int64_t len = dimsC[0], nrows = totalC / len;
    const int threads = len >= 256 ? 256 : (len >= 64 ? 64 : 32);
    const int blocks = (int)std::min<int64_t>(nrows, (int64_t)h->num_sms * 64);
    k_diag_rows<<<blocks, threads, 0, h->stream>>>(d, uniform, T, C, len, nrows, r, desc.sumDc, ndiag, alpha, beta);
    ITG_CHECK_LAUNCH(h);
    return ITG_OK;
  }
  k_diag_dense<<<itg_blocks_for(totalC, 256, h->num_sms * 16), 256, 0, h->stream>>>(
      d, uniform, T, C, totalC, desc, alpha, beta);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_diag_diag(itg_handle* h, int64_t n, double alpha, const double* a, int au,
                             const double* b, int bu, double* c) {
  if (!h || n < 0 || !a || !b || !c) return ITG_ERR_INVALID;
  if (n == 0) return ITG_OK;
  k_diag_diag<<<itg_blocks_for(n, 256, h->num_sms * 8), 256, 0, h->stream>>>(n, alpha, a, au, b, bu, c);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

extern "C" int itg_diag_to_dense(itg_handle* h, const double* d, int uniform, int rank,
                                 const int64_t* dims, double* T) {
  if (!h || !d || !T || rank < 1 || rank > ITG_MAX_RANK || !dims) return ITG_ERR_INVALID;
  int64_t total = 1, step = 0, s = 1, nd = dims[0];
  for (int i = 0; i < rank; ++i) {
    total *= dims[i];
    step += s;
    s *= dims[i];
    nd = dims[i] < nd ? dims[i] : nd;
  }
  if (total == 0) return ITG_OK;
  ITG_CUDA(h, cudaMemsetAsync(T, 0, sizeof(double) * total, h->stream));
  k_diag_scatter<<<itg_blocks_for(nd, 256, h->num_sms * 4), 256, 0, h->stream>>>(d, uniform, nd, step, T);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}
