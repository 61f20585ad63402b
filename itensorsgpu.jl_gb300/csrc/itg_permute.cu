// Tensor permutation and permuted axpby (K2, K3).
//
// B[perm(i)] = alpha * A[i] (+ beta * Bin) for column-major tensors.  The host
// side first fuses modes that stay adjacent in both layouts, then picks one of
// two HBM-bound kernels:
//   * row copy  — A's fastest mode is also B's fastest: both sides stream
//                 contiguous rows; one div/mod chain per row.
//   * transpose — different fastest modes: 32x32 tiles staged through shared
//                 memory so that reads of A and writes of B are both coalesced.
#include "itg_internal.cuh"

namespace {

struct PermDesc {
  int rank;                        // after fusion
  int64_t dims[ITG_MAX_RANK];      // in A's order
  int64_t strA[ITG_MAX_RANK];      // stride of A's mode i in A
  int64_t strB[ITG_MAX_RANK];      // stride of A's mode i in B
};

// Remaining-mode decomposition used by both kernels: modes listed in `idx`.
struct RestDesc {
  int n;
  int64_t dims[ITG_MAX_RANK];
  int64_t strA[ITG_MAX_RANK];
  int64_t strB[ITG_MAX_RANK];
};

__device__ __forceinline__ void rest_offsets(const RestDesc& r, int64_t lin, int64_t& oa,
                                             int64_t& ob) {
  oa = 0;
  ob = 0;
  for (int i = 0; i < r.n; ++i) {
    int64_t d = r.dims[i];
    int64_t q = lin / d;
    int64_t c = lin - q * d;
    lin = q;
    oa += c * r.strA[i];
    ob += c * r.strB[i];
  }
}

// One CTA handles `rows_per_block` rows of length d0 (stride 1 in A and B).
__global__ void k_perm_rows(const double* __restrict__ A, double* __restrict__ B,
                            const double* __restrict__ Bin, double alpha, double beta,
                            int64_t d0, int64_t nrows, RestDesc rest) {
  for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
    int64_t oa, ob;
    rest_offsets(rest, row, oa, ob);
    const double* a = A + oa;
    double* b = B + ob;
    const double* bi = Bin ? Bin + ob : nullptr;
    for (int64_t i = threadIdx.x; i < d0; i += blockDim.x) {
      double v = alpha * a[i];
      if (bi) v = fma(beta, bi[i], v);
      b[i] = v;
    }
  }
}

// Tiled transpose between A's mode 0 (size n0, stride 1 in A, stride s0B in B)
// and A's mode q (size nq, stride sqA in A, stride 1 in B).  blockIdx.y walks
// the batches (the other modes), so their offsets are decomposed once per
// batch, and blockIdx.x the 32 x 32 tiles of one batch; the index arithmetic
// inside a batch is 32-bit.
#define TP 32
__global__ void __launch_bounds__(256)
k_perm_transpose(const double* __restrict__ A, double* __restrict__ B, const double* __restrict__ Bin,
                 double alpha, double beta, int64_t n0, int64_t nq, int64_t sqA, int64_t s0B, int64_t nbatch,
                 RestDesc rest) {
  __shared__ double tile[TP][TP + 1];
  const int t0 = (int)((n0 + TP - 1) / TP), tq = (int)((nq + TP - 1) / TP);
  const int tiles = t0 * tq;
  for (int64_t b = blockIdx.y; b < nbatch; b += gridDim.y) {
    int64_t oa, ob;
    rest_offsets(rest, b, oa, ob);
    for (int r = blockIdx.x; r < tiles; r += gridDim.x) {
      const int iq = r / t0, i0 = r - iq * t0;
      const int64_t base0 = (int64_t)i0 * TP, baseq = (int64_t)iq * TP;
      // read: threadIdx.x runs along mode 0 (contiguous in A); all loads first
      double v[TP / 8];
#pragma unroll
      for (int j = 0; j < TP / 8; ++j) {
        const int y = threadIdx.y + 8 * j;
        const int64_t i = base0 + threadIdx.x, k = baseq + y;
        v[j] = (i < n0 && k < nq) ? A[oa + i + k * sqA] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < TP / 8; ++j) tile[threadIdx.y + 8 * j][threadIdx.x] = v[j];
      __syncthreads();
      // write: threadIdx.x runs along mode q (contiguous in B)
#pragma unroll
      for (int j = 0; j < TP / 8; ++j) {
        const int y = threadIdx.y + 8 * j;
        const int64_t k = baseq + threadIdx.x, i = base0 + y;
        if (i < n0 && k < nq) {
          const int64_t o = ob + k + i * s0B;
          double w = alpha * tile[threadIdx.x][y];
          if (Bin) w = fma(beta, Bin[o], w);
          B[o] = w;
        }
      }
      __syncthreads();
    }
  }
}

// Resolve modesB as a permutation of modesA.  perm[j] = A-position of B's mode j.
int make_perm(itg_handle* h, int rank, const int32_t* modesA, const int32_t* modesB, int* perm) {
  for (int j = 0; j < rank; ++j) {
    perm[j] = -1;
    for (int i = 0; i < rank; ++i)
      if (modesA[i] == modesB[j]) {
        if (perm[j] >= 0) return itg_fail(h, ITG_ERR_SHAPE, "repeated mode %d", modesB[j]);
        perm[j] = i;
      }
    if (perm[j] < 0) return itg_fail(h, ITG_ERR_SHAPE, "mode %d of B not found in A", modesB[j]);
  }
  for (int i = 0; i < rank; ++i)
    for (int j = i + 1; j < rank; ++j)
      if (modesA[i] == modesA[j]) return itg_fail(h, ITG_ERR_SHAPE, "repeated mode %d in A", modesA[i]);
  return ITG_OK;
}

}  // namespace

// Shared host routine: Bin may be null (pure permute) or alias B.
static int permute_axpby(itg_handle* h, double alpha, const double* A, int rank,
                         const int64_t* dimsA, const int32_t* modesA, double beta,
                         const double* Bin, const int32_t* modesB, double* B) {
  if (rank < 0 || rank > ITG_MAX_RANK)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank %d outside 0..%d", rank, ITG_MAX_RANK);
  int perm[ITG_MAX_RANK];
  ITG_TRY(make_perm(h, rank, modesA, modesB, perm));
  int64_t total = 1;
  for (int i = 0; i < rank; ++i) {
    if (dimsA[i] < 0) return itg_fail(h, ITG_ERR_SHAPE, "negative dimension");
    total *= dimsA[i];
  }
  if (total == 0) return ITG_OK;
  // strides of A's modes in A and in B
  int64_t sA[ITG_MAX_RANK], sB[ITG_MAX_RANK];
  {
    int64_t s = 1;
    for (int i = 0; i < rank; ++i) { sA[i] = s; s *= dimsA[i]; }
    s = 1;
    for (int j = 0; j < rank; ++j) { sB[perm[j]] = s; s *= dimsA[perm[j]]; }
  }
  // Fuse: drop unit modes, then merge A-adjacent modes that are B-adjacent.
  PermDesc d;
  d.rank = 0;
  for (int i = 0; i < rank; ++i) {
    if (dimsA[i] == 1) continue;
    if (d.rank > 0) {
      int p = d.rank - 1;
      if (sA[i] == d.strA[p] * d.dims[p] && sB[i] == d.strB[p] * d.dims[p]) {
        d.dims[p] *= dimsA[i];
        continue;
      }
    }
    d.dims[d.rank] = dimsA[i];
    d.strA[d.rank] = sA[i];
    d.strB[d.rank] = sB[i];
    d.rank++;
  }
  const double* bin = (beta == 0.0) ? nullptr : Bin;
  if (d.rank == 0) {  // single element
    d.rank = 1;
    d.dims[0] = 1;
    d.strA[0] = 1;
    d.strB[0] = 1;
  }
  // find the fused mode that is fastest in B (strB == 1)
  int q = 0;
  for (int i = 0; i < d.rank; ++i)
    if (d.strB[i] == 1) q = i;
  RestDesc rest;
  if (q == 0) {
    rest.n = 0;
    for (int i = 1; i < d.rank; ++i) {
      rest.dims[rest.n] = d.dims[i];
      rest.strA[rest.n] = d.strA[i];
      rest.strB[rest.n] = d.strB[i];
      rest.n++;
    }
    int64_t nrows = total / d.dims[0];
    int threads = d.dims[0] >= 256 ? 256 : (d.dims[0] >= 64 ? 64 : 32);
    int blocks = (int)std::min<int64_t>(nrows, (int64_t)h->num_sms * 64);
    k_perm_rows<<<blocks, threads, 0, h->stream>>>(A, B, bin, alpha, beta, d.dims[0], nrows, rest);
  } else {
    rest.n = 0;
    for (int i = 1; i < d.rank; ++i) {
      if (i == q) continue;
      rest.dims[rest.n] = d.dims[i];
      rest.strA[rest.n] = d.strA[i];
      rest.strB[rest.n] = d.strB[i];
      rest.n++;
    }
    int64_t n0 = d.dims[0], nq = d.dims[q];
    int64_t nbatch = total / (n0 * nq);
    const int64_t tiles = ((n0 + TP - 1) / TP) * ((nq + TP - 1) / TP);
    if (tiles > (int64_t)INT32_MAX) return itg_fail(h, ITG_ERR_UNSUPPORTED, "permute: transpose too large");
    const int64_t want = (int64_t)h->num_sms * 32;  // resident CTAs
    const int64_t gx = std::min<int64_t>(tiles, want);
    const int64_t gy = std::min<int64_t>(std::min<int64_t>(nbatch, std::max<int64_t>(1, want / gx)), 65535);
    dim3 thr(TP, 8);
    k_perm_transpose<<<dim3((unsigned)gx, (unsigned)gy), thr, 0, h->stream>>>(A, B, bin, alpha, beta, n0, nq,
                                                                            d.strA[q], d.strB[0], nbatch, rest);
  }
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

namespace {
// Complex tensors (ITG_C64, interleaved re/im) are permuted as real tensors
// with one leading mode of length 2 that stays first.
struct C64View {
  int rank;
  int64_t dims[ITG_MAX_RANK];
  int32_t ma[ITG_MAX_RANK], mb[ITG_MAX_RANK];
};

int c64_view(itg_handle* h, int rank, const int64_t* dimsA, const int32_t* modesA, const int32_t* modesB,
             C64View& v) {
  if (rank + 1 > ITG_MAX_RANK) return itg_fail(h, ITG_ERR_UNSUPPORTED, "complex rank above %d", ITG_MAX_RANK - 1);
  int32_t c = 0;
  for (int i = 0; i < rank; ++i) c = modesA[i] > c ? modesA[i] : c;
  ++c;
  v.rank = rank + 1;
  v.dims[0] = 2;
  v.ma[0] = v.mb[0] = c;
  for (int i = 0; i < rank; ++i) {
    v.dims[i + 1] = dimsA[i];
    v.ma[i + 1] = modesA[i];
    v.mb[i + 1] = modesB[i];
  }
  return ITG_OK;
}
}  // namespace

extern "C" int itg_permute(itg_handle* h, int dtype, double alpha, const void* A, int rank,
                           const int64_t* dimsA, const int32_t* modesA, void* B,
                           const int32_t* modesB) {
  if (!h) return ITG_ERR_INVALID;
  if (dtype != ITG_F64 && dtype != ITG_C64) return itg_fail(h, ITG_ERR_UNSUPPORTED, "dtype %d", dtype);
  if (rank > 0 && (!dimsA || !modesA || !modesB)) return itg_fail(h, ITG_ERR_INVALID, "null array");
  if (!A || !B) return itg_fail(h, ITG_ERR_INVALID, "null tensor");
  if (dtype == ITG_C64) {
    C64View v;
    ITG_TRY(c64_view(h, rank, dimsA, modesA, modesB, v));
    return permute_axpby(h, alpha, (const double*)A, v.rank, v.dims, v.ma, 0.0, nullptr, v.mb, (double*)B);
  }
  return permute_axpby(h, alpha, (const double*)A, rank, dimsA, modesA, 0.0, nullptr, modesB,
                       (double*)B);
}

extern "C" int itg_axpby_permuted(itg_handle* h, int dtype, double alpha, const void* A, int rank,
                                  const int64_t* dimsA, const int32_t* modesA, double beta,
                                  const void* B, const int32_t* modesB, void* C) {
  if (!h) return ITG_ERR_INVALID;
  if (dtype != ITG_F64 && dtype != ITG_C64) return itg_fail(h, ITG_ERR_UNSUPPORTED, "dtype %d", dtype);
  if (rank > 0 && (!dimsA || !modesA || !modesB)) return itg_fail(h, ITG_ERR_INVALID, "null array");
  if (!A || !C || (beta != 0.0 && !B)) return itg_fail(h, ITG_ERR_INVALID, "null tensor");
  if (A == C) return itg_fail(h, ITG_ERR_INVALID, "C must not alias A");
  if (dtype == ITG_C64) {
    C64View v;
    ITG_TRY(c64_view(h, rank, dimsA, modesA, modesB, v));
    return permute_axpby(h, alpha, (const double*)A, v.rank, v.dims, v.ma, beta, (const double*)B, v.mb,
                         (double*)C);
  }
  return permute_axpby(h, alpha, (const double*)A, rank, dimsA, modesA, beta, (const double*)B,
                       modesB, (double*)C);
}

namespace itg {
int transpose(itg_handle* h, int64_t m, int64_t n, const double* in, int64_t lda, double* out) {
  if (lda != m) return itg_fail(h, ITG_ERR_UNSUPPORTED, "transpose needs lda == m");
  int64_t dims[2] = {m, n};
  int32_t ma[2] = {0, 1}, mb[2] = {1, 0};
  return permute_axpby(h, 1.0, in, 2, dims, ma, 0.0, nullptr, mb, out);
}
}  // namespace itg
