// Pairwise tensor contraction (K1): planner, plan cache and the FP64
// gather-GEMM kernel.
//
// A contraction C = alpha*A*B + beta*C is lowered to one GEMM
//     C[m, n] = alpha * sum_k A[m, k] * B[k, n] + beta * C[m, n]
// where m runs over A's free modes (in C's order), n over B's free modes (in
// C's order) and k over the contracted modes.  No tensor is permuted in memory:
// every operand is addressed through per-plan offset tables
//     A[m, k] = A[offAm[m] + offAk[k]],  B[k, n] = B[offBk[k] + offBn[n]],
//     C[m, n] = C[offCm[m] + offCn[n]],
// so the TTGT transposes are folded into the tile loads and the epilogue
// stores.  The scalar (rank 0) and outer-product (K = 1) cases of
// contract!! (src/tensor/cudense.jl:89-105) are the same GEMM with M, N or K
// equal to 1.  Plans are cached per (dims, modes) key like the reference's
// ContractionPlans (src/ITensorsGPU.jl:55, src/tensor/cudense.jl:284-294).
#include "itg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>



void itg_release_plans(itg_handle* h) { h->plans.clear(); }

// ------------------------------------------------------------ FP64 kernel
namespace {

constexpr int GBK = 16, GTHREADS = 256;
constexpr int SPAD = 4;  // shared-memory row padding (doubles)

// One BM x BN tile of C = alpha * A B + beta * C through the offset tables.
// 256 threads as 16 x 16, each computing (BM/16) x (BN/16) outputs split in
// two halves (rows ty*TM/2.. and BM/2 + ty*TM/2..) to keep shared-memory reads
// conflict-free.  AK / BK: the operand's k offsets are the fast ones (then a
// thread loads along k, otherwise along m / n).
template <int BM, int BN, bool AK, bool BK>
__device__ __forceinline__ void gemm_tile_f64(const double* __restrict__ A, const double* __restrict__ B,
                  double* __restrict__ C, const int64_t* __restrict__ offAm,
                  const int64_t* __restrict__ offAk, const int64_t* __restrict__ offBk,
                  const int64_t* __restrict__ offBn, const int64_t* __restrict__ offCm,
                  const int64_t* __restrict__ offCn, int64_t M, int64_t N, int64_t K,
                  double alpha, double beta, int64_t m0, int64_t n0, double* smem) {
  constexpr int RA = BM / 16, RB = BN / 16;   // loads per thread per k-tile
  constexpr int TM = BM / 16, TN = BN / 16;   // outputs per thread
  constexpr int SA = GTHREADS / BM, SB = GTHREADS / BN;  // k stride of the m/n-major loads
  double* As = smem;                              // [2][GBK][BM+SPAD]
  double* Bs = smem + 2 * GBK * (BM + SPAD);      // [2][GBK][BN+SPAD]
  const int t = threadIdx.x;

  int64_t aRow[RA];
  int64_t bCol[RB];
  if (AK) {
#pragma unroll
    for (int r = 0; r < RA; ++r) {
      int64_t m = m0 + (t >> 4) + 16 * r;
      aRow[r] = (m < M) ? offAm[m] : -1;
    }
  } else {
    int64_t m = m0 + (t % BM);
    aRow[0] = (m < M) ? offAm[m] : -1;
  }
  if (BK) {
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      int64_t n = n0 + (t >> 4) + 16 * r;
      bCol[r] = (n < N) ? offBn[n] : -1;
    }
  } else {
    int64_t n = n0 + (t % BN);
    bCol[0] = (n < N) ? offBn[n] : -1;
  }

  double ra[RA], rb[RB];
  auto load_tile = [&](int64_t k0) {
    if (AK) {
      int64_t k = k0 + (t & 15);
      int64_t ok = (k < K) ? offAk[k] : 0;
#pragma unroll
      for (int r = 0; r < RA; ++r) ra[r] = (k < K && aRow[r] >= 0) ? A[aRow[r] + ok] : 0.0;
    } else {
#pragma unroll
      for (int r = 0; r < RA; ++r) {
        int64_t k = k0 + (t / BM) + SA * r;
        ra[r] = (k < K && aRow[0] >= 0) ? A[aRow[0] + offAk[k]] : 0.0;
      }
    }
    if (BK) {
      int64_t k = k0 + (t & 15);
      int64_t ok = (k < K) ? offBk[k] : 0;
#pragma unroll
      for (int r = 0; r < RB; ++r) rb[r] = (k < K && bCol[r] >= 0) ? B[bCol[r] + ok] : 0.0;
    } else {
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        int64_t k = k0 + (t / BN) + SB * r;
        rb[r] = (k < K && bCol[0] >= 0) ? B[offBk[k] + bCol[0]] : 0.0;
      }
    }
  };
  auto store_tile = [&](int buf) {
    double* as = As + buf * GBK * (BM + SPAD);
    double* bs = Bs + buf * GBK * (BN + SPAD);
    if (AK) {
#pragma unroll
      for (int r = 0; r < RA; ++r) as[(t & 15) * (BM + SPAD) + (t >> 4) + 16 * r] = ra[r];
    } else {
#pragma unroll
      for (int r = 0; r < RA; ++r) as[((t / BM) + SA * r) * (BM + SPAD) + (t % BM)] = ra[r];
    }
    if (BK) {
#pragma unroll
      for (int r = 0; r < RB; ++r) bs[(t & 15) * (BN + SPAD) + (t >> 4) + 16 * r] = rb[r];
    } else {
#pragma unroll
      for (int r = 0; r < RB; ++r) bs[((t / BN) + SB * r) * (BN + SPAD) + (t % BN)] = rb[r];
    }
  };

  const int tx = t & 15, ty = t >> 4;
  double acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

  const int64_t nk = (K + GBK - 1) / GBK;
  if (nk > 0) {
    load_tile(0);
    store_tile(0);
  }
  __syncthreads();
  for (int64_t kt = 0; kt < nk; ++kt) {
    const int buf = (int)(kt & 1);
    if (kt + 1 < nk) load_tile((kt + 1) * GBK);
    const double* as = As + buf * GBK * (BM + SPAD);
    const double* bs = Bs + buf * GBK * (BN + SPAD);
#pragma unroll 4
    for (int kk = 0; kk < GBK; ++kk) {
      double a[TM], b[TN];
      const double* ap = as + kk * (BM + SPAD);
      const double* bp = bs + kk * (BN + SPAD);
#pragma unroll
      for (int i = 0; i < TM / 2; ++i) {
        a[i] = ap[ty * (TM / 2) + i];
        a[TM / 2 + i] = ap[BM / 2 + ty * (TM / 2) + i];
      }
#pragma unroll
      for (int j = 0; j < TN / 2; ++j) {
        b[j] = bp[tx * (TN / 2) + j];
        b[TN / 2 + j] = bp[BN / 2 + tx * (TN / 2) + j];
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (kt + 1 < nk) store_tile(buf ^ 1);
    __syncthreads();
  }

  // Epilogue: scatter to C's layout.
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    int64_t m = m0 + (i < TM / 2 ? ty * (TM / 2) + i : BM / 2 + ty * (TM / 2) + (i - TM / 2));
    if (m >= M) continue;
    int64_t cm = offCm[m];
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int64_t n = n0 + (j < TN / 2 ? tx * (TN / 2) + j : BN / 2 + tx * (TN / 2) + (j - TN / 2));
      if (n >= N) continue;
      double* c = C + cm + offCn[n];
      double v = alpha * acc[i][j];
      if (beta != 0.0) v = fma(beta, *c, v);
      *c = v;
    }
  }
}

template <int BM, int BN, bool AK, bool BK>
__global__ void __launch_bounds__(GTHREADS)
k_gemm_gather_f64(const double* __restrict__ A, const double* __restrict__ B,
                  double* __restrict__ C, const int64_t* __restrict__ offAm,
                  const int64_t* __restrict__ offAk, const int64_t* __restrict__ offBk,
                  const int64_t* __restrict__ offBn, const int64_t* __restrict__ offCm,
                  const int64_t* __restrict__ offCn, int64_t M, int64_t N, int64_t K,
                  double alpha, double beta) {
  extern __shared__ double smem[];
  gemm_tile_f64<BM, BN, AK, BK>(A, B, C, offAm, offAk, offBk, offBn, offCm, offCn, M, N, K, alpha, beta,
                                (int64_t)blockIdx.x * BM, (int64_t)blockIdx.y * BN, smem);
}

// Grouped launch: many contractions of one mode structure with different
// sizes.  CTA b finds its problem by binary search over tile_start.
struct GroupProb {
  const double* A;
  const double* B;
  double* C;
  const int64_t* tables;
  int64_t M, N, K;
  int64_t tile_start, tiles_n;
  int flags;  // bit 0: A K-major, bit 1: B K-major
};

template <int BM, int BN>
__global__ void __launch_bounds__(GTHREADS)
k_gemm_gather_f64_grouped(const GroupProb* __restrict__ probs, int count, double alpha, double beta) {
  extern __shared__ double smem[];
  const int64_t b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].tile_start <= b) lo = mid; else hi = mid - 1;
  }
  const GroupProb& p = probs[lo];
  const int64_t local = b - p.tile_start;
  const int64_t tm = local / p.tiles_n, tn = local - tm * p.tiles_n;
  const int64_t* T = p.tables;
  const int64_t *offAm = T, *offCm = T + p.M, *offBn = T + 2 * p.M, *offCn = T + 2 * p.M + p.N;
  const int64_t *offAk = T + 2 * p.M + 2 * p.N, *offBk = offAk + p.K;
  const int64_t m0 = tm * BM, n0 = tn * BN;
  switch (p.flags) {
    case 3: gemm_tile_f64<BM, BN, true, true>(p.A, p.B, p.C, offAm, offAk, offBk, offBn, offCm, offCn, p.M, p.N, p.K, alpha, beta, m0, n0, smem); break;
    case 1: gemm_tile_f64<BM, BN, true, false>(p.A, p.B, p.C, offAm, offAk, offBk, offBn, offCm, offCn, p.M, p.N, p.K, alpha, beta, m0, n0, smem); break;
    case 2: gemm_tile_f64<BM, BN, false, true>(p.A, p.B, p.C, offAm, offAk, offBk, offBn, offCm, offCn, p.M, p.N, p.K, alpha, beta, m0, n0, smem); break;
    default: gemm_tile_f64<BM, BN, false, false>(p.A, p.B, p.C, offAm, offAk, offBk, offBn, offCm, offCn, p.M, p.N, p.K, alpha, beta, m0, n0, smem); break;
  }
}

template <int BM, int BN>
constexpr size_t gemm_smem() { return sizeof(double) * 2 * GBK * ((BM + SPAD) + (BN + SPAD)); }

// Tile shape of each ITG_TILE_* variant.
inline int tile_bm(int tile) { return tile == ITG_TILE_64x64 ? 64 : 128; }
inline int tile_bn(int tile) { return tile == ITG_TILE_128x128 ? 128 : 64; }
inline int64_t tile_count(int tile, int64_t M, int64_t N) {
  const int bm = tile_bm(tile), bn = tile_bn(tile);
  return ((M + bm - 1) / bm) * ((N + bn - 1) / bn);
}

template <int BM, int BN, bool AK, bool BK>
int launch_gemm_t(itg_handle* h, const ContractPlan& p, const double* A, const double* B, double* C,
                  double alpha, double beta) {
  static bool attr_set = false;
  constexpr size_t smem = gemm_smem<BM, BN>();
  if (!attr_set) {
    ITG_CUDA(h, cudaFuncSetAttribute(k_gemm_gather_f64<BM, BN, AK, BK>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int64_t gx = (p.M + BM - 1) / BM, gy = (p.N + BN - 1) / BN;
  if (gy > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "N=%lld too large", (long long)p.N);
  dim3 grid((unsigned)gx, (unsigned)gy);
  ProfScope prof(h, ITG_KERNEL_GEMM_F64);
  k_gemm_gather_f64<BM, BN, AK, BK><<<grid, GTHREADS, smem, h->stream>>>(
      A, B, C, p.offAm(), p.offAk(), p.offBk(), p.offBn(), p.offCm(), p.offCn(), p.M, p.N, p.K,
      alpha, beta);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

template <bool AK, bool BK>
int launch_gemm_v(itg_handle* h, int tile, const ContractPlan& p, const double* A, const double* B, double* C,
                  double alpha, double beta) {
  switch (tile) {
    case ITG_TILE_64x64: return launch_gemm_t<64, 64, AK, BK>(h, p, A, B, C, alpha, beta);
    case ITG_TILE_128x64: return launch_gemm_t<128, 64, AK, BK>(h, p, A, B, C, alpha, beta);
    default: return launch_gemm_t<128, 128, AK, BK>(h, p, A, B, C, alpha, beta);
  }
}

int launch_gemm(itg_handle* h, int tile, const ContractPlan& p, const double* A, const double* B, double* C,
                double alpha, double beta) {
  if (p.a_kmaj && p.b_kmaj) return launch_gemm_v<true, true>(h, tile, p, A, B, C, alpha, beta);
  if (p.a_kmaj) return launch_gemm_v<true, false>(h, tile, p, A, B, C, alpha, beta);
  if (p.b_kmaj) return launch_gemm_v<false, true>(h, tile, p, A, B, C, alpha, beta);
  return launch_gemm_v<false, false>(h, tile, p, A, B, C, alpha, beta);
}

__global__ void k_scale_or_zero(int64_t n, double beta, double* __restrict__ C) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    C[i] = (beta == 0.0) ? 0.0 : beta * C[i];
}

// ------------------------------------------------------------ planning
struct ModeInfo {
  int32_t mode;
  int64_t dim;
  int64_t strA, strB, strC;  // -1 when absent
};

}  // namespace

namespace itg {

// Host half of planning: validates the modes and fills the offset tables
// (offAm, offCm, offBn, offCn, offAk, offBk) into `tab`; no device work.
int plan_tables_host(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA,
                     int rankB, const int64_t* dimsB, const int32_t* modesB, int rankC,
                     const int64_t* dimsC, const int32_t* modesC, ContractPlan& pl,
                     std::vector<int64_t>& tab, PlanTableDesc* desc) {
  auto strides = [](int r, const int64_t* d, int64_t* s) {
    int64_t x = 1;
    for (int i = 0; i < r; ++i) { s[i] = x; x *= d[i]; }
  };
  int64_t sA[ITG_MAX_RANK], sB[ITG_MAX_RANK], sC[ITG_MAX_RANK];
  strides(rankA, dimsA, sA);
  strides(rankB, dimsB, sB);
  strides(rankC, dimsC, sC);
  auto find = [](int r, const int32_t* m, int32_t x) {
    int pos = -1;
    for (int i = 0; i < r; ++i)
      if (m[i] == x) pos = (pos < 0) ? i : -2;
    return pos;
  };
  for (int i = 0; i < rankA; ++i)
    if (find(rankA, modesA, modesA[i]) == -2) return itg_fail(h, ITG_ERR_SHAPE, "repeated mode %d in A", modesA[i]);
  for (int i = 0; i < rankB; ++i)
    if (find(rankB, modesB, modesB[i]) == -2) return itg_fail(h, ITG_ERR_SHAPE, "repeated mode %d in B", modesB[i]);
  for (int i = 0; i < rankC; ++i)
    if (find(rankC, modesC, modesC[i]) == -2) return itg_fail(h, ITG_ERR_SHAPE, "repeated mode %d in C", modesC[i]);

  std::vector<ModeInfo> freeA, freeB, contr;
  // C's modes in C order
  for (int i = 0; i < rankC; ++i) {
    int ia = find(rankA, modesA, modesC[i]);
    int ib = find(rankB, modesB, modesC[i]);
    if (ia >= 0 && ib >= 0)
      return itg_fail(h, ITG_ERR_UNSUPPORTED, "mode %d appears in A, B and C (batch mode)", modesC[i]);
    if (ia < 0 && ib < 0) return itg_fail(h, ITG_ERR_SHAPE, "mode %d of C is in neither A nor B", modesC[i]);
    ModeInfo mi{modesC[i], dimsC[i], -1, -1, sC[i]};
    if (ia >= 0) {
      if (dimsA[ia] != dimsC[i]) return itg_fail(h, ITG_ERR_SHAPE, "dimension mismatch for mode %d", modesC[i]);
      mi.strA = sA[ia];
      freeA.push_back(mi);
    } else {
      if (dimsB[ib] != dimsC[i]) return itg_fail(h, ITG_ERR_SHAPE, "dimension mismatch for mode %d", modesC[i]);
      mi.strB = sB[ib];
      freeB.push_back(mi);
    }
  }
  for (int i = 0; i < rankA; ++i) {
    if (find(rankC, modesC, modesA[i]) >= 0) continue;
    int ib = find(rankB, modesB, modesA[i]);
    if (ib < 0) return itg_fail(h, ITG_ERR_UNSUPPORTED, "mode %d of A is in neither B nor C", modesA[i]);
    if (dimsA[i] != dimsB[ib]) return itg_fail(h, ITG_ERR_SHAPE, "dimension mismatch for contracted mode %d", modesA[i]);
    contr.push_back({modesA[i], dimsA[i], sA[i], sB[ib], -1});
  }
  for (int i = 0; i < rankB; ++i) {
    if (find(rankC, modesC, modesB[i]) >= 0) continue;
    if (find(rankA, modesA, modesB[i]) < 0)
      return itg_fail(h, ITG_ERR_UNSUPPORTED, "mode %d of B is in neither A nor C", modesB[i]);
  }
  // K order: A's order unless B's stride-1 mode is contracted and A's is not.
  bool aFirstContr = rankA > 0 && find(rankC, modesC, modesA[0]) < 0 && dimsA[0] > 1;
  bool bFirstContr = rankB > 0 && find(rankC, modesC, modesB[0]) < 0 && dimsB[0] > 1;
  if (!aFirstContr && bFirstContr)
    std::stable_sort(contr.begin(), contr.end(),
                     [](const ModeInfo& x, const ModeInfo& y) { return x.strB < y.strB; });

  ContractPlan* p = &pl;
  auto prod = [](const std::vector<ModeInfo>& v) {
    int64_t x = 1;
    for (auto& m : v) x *= m.dim;
    return x;
  };
  p->M = prod(freeA);
  p->N = prod(freeB);
  p->K = prod(contr);
  // Tables.
  tab.assign(2 * p->M + 2 * p->N + 2 * p->K, 0);
  auto fill = [](const std::vector<ModeInfo>& v, int64_t count, int which1, int which2,
                 int64_t* o1, int64_t* o2) {
    // which: 0 = strA, 1 = strB, 2 = strC
    auto st = [](const ModeInfo& m, int w) { return w == 0 ? m.strA : (w == 1 ? m.strB : m.strC); };
    std::vector<int64_t> idx(v.size(), 0);
    int64_t a = 0, b = 0;
    for (int64_t l = 0; l < count; ++l) {
      o1[l] = a;
      o2[l] = b;
      for (size_t i = 0; i < v.size(); ++i) {
        idx[i]++;
        a += st(v[i], which1);
        b += st(v[i], which2);
        if (idx[i] < v[i].dim) break;
        a -= st(v[i], which1) * v[i].dim;
        b -= st(v[i], which2) * v[i].dim;
        idx[i] = 0;
      }
    }
  };
  if (desc) {
    const std::vector<ModeInfo>* sec[3] = {&freeA, &freeB, &contr};
    const int w1[3] = {0, 1, 0}, w2[3] = {2, 2, 1};
    const int64_t cnt[3] = {p->M, p->N, p->K};
    auto st = [](const ModeInfo& m, int w) { return w == 0 ? m.strA : (w == 1 ? m.strB : m.strC); };
    for (int g = 0; g < 3; ++g) {
      desc->nmodes[g] = (int)sec[g]->size();
      desc->count[g] = cnt[g];
      for (int i = 0; i < desc->nmodes[g]; ++i) {
        desc->dim[g][i] = (*sec[g])[i].dim;
        desc->s1[g][i] = st((*sec[g])[i], w1[g]);
        desc->s2[g][i] = st((*sec[g])[i], w2[g]);
      }
    }
  }
  int64_t* t = tab.data();
  fill(freeA, p->M, 0, 2, t, t + p->M);
  fill(freeB, p->N, 1, 2, t + 2 * p->M, t + 2 * p->M + p->N);
  fill(contr, p->K, 0, 1, t + 2 * p->M + 2 * p->N, t + 2 * p->M + 2 * p->N + p->K);
  p->a_kmaj = p->K > 1 && (t[2 * p->M + 2 * p->N + 1] - t[2 * p->M + 2 * p->N] == 1);
  p->b_kmaj = p->K > 1 && (t[2 * p->M + 2 * p->N + p->K + 1] - t[2 * p->M + 2 * p->N + p->K] == 1);
  return ITG_OK;
}

}  // namespace itg

namespace {

int build_plan(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA, int rankB,
               const int64_t* dimsB, const int32_t* modesB, int rankC, const int64_t* dimsC,
               const int32_t* modesC, std::shared_ptr<ContractPlan>& out) {
  auto p = std::make_shared<ContractPlan>();
  std::vector<int64_t> tab;
  ITG_TRY(itg::plan_tables_host(h, rankA, dimsA, modesA, rankB, dimsB, modesB, rankC, dimsC, modesC,
                                *p, tab, nullptr));
  if (!tab.empty()) {
    cudaError_t e = cudaMalloc((void**)&p->tables, tab.size() * sizeof(int64_t));
    if (e != cudaSuccess)
      return itg_fail(h, ITG_ERR_ALLOC, "plan table allocation failed: %s", cudaGetErrorString(e));
    ITG_CUDA(h, cudaMemcpy(p->tables, tab.data(), tab.size() * sizeof(int64_t),
                           cudaMemcpyHostToDevice));
  }
  out = p;
  return ITG_OK;
}

std::string plan_key(int rankA, const int64_t* dimsA, const int32_t* modesA, int rankB,
                     const int64_t* dimsB, const int32_t* modesB, int rankC, const int64_t* dimsC,
                     const int32_t* modesC) {
  // Canonical labels: number modes by first appearance (C, then A, then B).
  std::vector<int32_t> seen;
  auto lab = [&](int32_t m) {
    for (size_t i = 0; i < seen.size(); ++i)
      if (seen[i] == m) return (int)i;
    seen.push_back(m);
    return (int)seen.size() - 1;
  };
  std::ostringstream os;
  for (int i = 0; i < rankC; ++i) os << lab(modesC[i]) << ',' << dimsC[i] << ',';
  os << '|';
  for (int i = 0; i < rankA; ++i) os << lab(modesA[i]) << ',' << dimsA[i] << ',';
  os << '|';
  for (int i = 0; i < rankB; ++i) os << lab(modesB[i]) << ',' << dimsB[i] << ',';
  return os.str();
}

}  // namespace

int itg_split_gemm(itg_handle* h, const ContractPlan& p, const double* A, const double* B, double* C,
                   double alpha, double beta, int bn);  // itg_split.cu

// ---------------------------------------------------------- autotuning
// Per-shape choice of the kernel variant, the counterpart of the reference's
// algorithm cache (src/cudense.jl:284-326), which times every cuTENSOR
// algorithm on the first contraction of a (mode, dim) key.  FP64 shapes whose
// 128x128 tiling under-fills the GPU are timed (larger ones take 128x128
// outright); split shapes wider than 128 columns time their three tcgen05
// variants.  The launches write into a throw-away buffer so C is untouched.
// Variants give bit-identical results.
namespace tune {

std::mutex mu;
std::unordered_map<std::string, int> cache;
bool loaded = false;

const char* file_path() { return std::getenv("ITG_TUNE_FILE"); }

void load_locked() {
  if (loaded) return;
  loaded = true;
  const char* f = file_path();
  if (!f) return;
  std::ifstream in(f);
  std::string line;
  while (std::getline(in, line)) {
    const size_t sp = line.rfind(' ');
    if (sp == std::string::npos) continue;
    cache[line.substr(0, sp)] = std::atoi(line.c_str() + sp + 1);
  }
}

bool lookup(const std::string& k, int& v) {
  std::lock_guard<std::mutex> g(mu);
  load_locked();
  auto it = cache.find(k);
  if (it == cache.end()) return false;
  v = it->second;
  return true;
}

void store(const std::string& k, int v) {
  std::lock_guard<std::mutex> g(mu);
  load_locked();
  cache[k] = v;
  if (const char* f = file_path()) {
    std::ofstream out(f, std::ios::app);
    out << k << ' ' << v << '\n';
  }
}

int64_t size() {
  std::lock_guard<std::mutex> g(mu);
  load_locked();
  return (int64_t)cache.size();
}

void clear() {
  std::lock_guard<std::mutex> g(mu);
  cache.clear();
  loaded = true;  // do not re-read the file after an explicit clear
}

bool capturing(itg_handle* h) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &st) != cudaSuccess) return true;
  return st != cudaStreamCaptureStatusNone;
}

int reserve(itg_handle* h, size_t bytes) {
  if (bytes <= h->tune_buf_bytes) return ITG_OK;
  if (h->tune_buf) {
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->tune_buf);
    h->tune_buf = nullptr;
    h->tune_buf_bytes = 0;
  }
  const size_t want = itg_align256(bytes);
  if (cudaMalloc(&h->tune_buf, want) != cudaSuccess) {
    h->tune_buf = nullptr;
    return itg_fail(h, ITG_ERR_ALLOC, "autotune buffer of %zu bytes", want);
  }
  h->tune_buf_bytes = want;
  return ITG_OK;
}

// Median-free timing: one warm launch, then the best of `reps` timed launches.
template <class F>
int time_variant(itg_handle* h, F&& launch, float& best_ms) {
  cudaEvent_t e0, e1;
  ITG_CUDA(h, cudaEventCreate(&e0));
  ITG_CUDA(h, cudaEventCreate(&e1));
  int st = launch();
  best_ms = 1e30f;
  for (int r = 0; r < 3 && st == ITG_OK; ++r) {
    cudaEventRecord(e0, h->stream);
    st = launch();
    cudaEventRecord(e1, h->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) st = itg_fail(h, ITG_ERR_CUDA, "autotune timing failed");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) best_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

int heuristic_tile(itg_handle* h, int64_t M, int64_t N) {
  if (tile_count(ITG_TILE_128x128, M, N) >= h->num_sms) return ITG_TILE_128x128;
  if (tile_count(ITG_TILE_128x64, M, N) >= h->num_sms) return ITG_TILE_128x64;
  return ITG_TILE_64x64;
}

int choose_f64(itg_handle* h, const ContractPlan& p, const double* A, const double* B, double alpha, int& tile) {
  if (p.tile >= 0) {
    tile = p.tile;
    return ITG_OK;
  }
  tile = heuristic_tile(h, p.M, p.N);
  const bool big = tile_count(ITG_TILE_128x128, p.M, p.N) >= 4 * (int64_t)h->num_sms;
  if (p.key.empty() || big) {
    if (!p.key.empty()) p.tile = tile;
    return ITG_OK;
  }
  const std::string k = "f64|" + p.key;
  int v = 0;
  if (lookup(k, v)) {
    tile = p.tile = v;
    return ITG_OK;
  }
  if (!h->autotune || capturing(h)) return ITG_OK;
  ITG_TRY(reserve(h, sizeof(double) * (size_t)(p.M * p.N)));
  double* out = (double*)h->tune_buf;
  const bool prof = h->prof_on;
  h->prof_on = false;
  float best = 1e30f;
  int best_tile = tile;
  int st = ITG_OK;
  for (int cand : {ITG_TILE_128x128, ITG_TILE_128x64, ITG_TILE_64x64}) {
    float ms = 0.f;
    st = time_variant(h, [&]() { return launch_gemm(h, cand, p, A, B, out, alpha, 0.0); }, ms);
    if (st != ITG_OK) break;
    if (ms < best) {
      best = ms;
      best_tile = cand;
    }
  }
  h->prof_on = prof;
  ITG_TRY(st);
  h->tune_runs++;
  store(k, best_tile);
  tile = p.tile = best_tile;
  return ITG_OK;
}

int choose_split(itg_handle* h, const ContractPlan& p, const double* A, const double* B, double alpha, int& bn) {
  if (p.split_bn) {
    bn = p.split_bn;
    return ITG_OK;
  }
  // heuristic: 128-wide tiles for narrow outputs, else 256-wide
  const bool narrow = p.N <= 128;
  bn = narrow ? ITG_SPLIT_BN_128 : ITG_SPLIT_BN_256;
  if (p.key.empty() || narrow) {
    if (!p.key.empty()) p.split_bn = bn;
    return ITG_OK;
  }
  const std::string k = "split|" + p.key;
  int v = 0;
  if (lookup(k, v)) {
    bn = p.split_bn = v;
    return ITG_OK;
  }
  if (!h->autotune || capturing(h)) return ITG_OK;
  ITG_TRY(reserve(h, sizeof(double) * (size_t)(p.M * p.N)));
  double* out = (double*)h->tune_buf;
  const bool prof = h->prof_on;
  h->prof_on = false;
  float best = 1e30f;
  int best_bn = bn;
  int st = ITG_OK;
  // one tile per CTA, or stream-K (persistent CTAs, the last partial wave
  // split at level boundaries): each wins on some shapes
  const int cands[] = {ITG_SPLIT_BN_256, ITG_SPLIT_BN_256 | ITG_SPLIT_STREAMK, ITG_SPLIT_BN_128,
                       ITG_SPLIT_BN_128 | ITG_SPLIT_STREAMK};
  for (int cand : cands) {
    float ms = 0.f;
    st = time_variant(h, [&]() { return itg_split_gemm(h, p, A, B, out, alpha, 0.0, cand); }, ms);
    if (st != ITG_OK) break;
    if (ms < best) {
      best = ms;
      best_bn = cand;
    }
  }
  h->prof_on = prof;
  ITG_TRY(st);
  h->tune_runs++;
  store(k, best_bn);
  bn = p.split_bn = best_bn;
  return ITG_OK;
}

}  // namespace tune

namespace itg {

int get_plan(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA, int rankB,
             const int64_t* dimsB, const int32_t* modesB, int rankC, const int64_t* dimsC,
             const int32_t* modesC, std::shared_ptr<ContractPlan>& plan) {
  std::string key = plan_key(rankA, dimsA, modesA, rankB, dimsB, modesB, rankC, dimsC, modesC);
  auto it = h->plans.find(key);
  if (it != h->plans.end()) {
    plan = it->second;
    return ITG_OK;
  }
  ITG_TRY(build_plan(h, rankA, dimsA, modesA, rankB, dimsB, modesB, rankC, dimsC, modesC, plan));
  plan->key = key;
  h->plans[key] = plan;
  return ITG_OK;
}

int run_plan(itg_handle* h, const ContractPlan& p, double alpha, const double* A, const double* B,
             double beta, double* C, int precision) {
  if (p.M == 0 || p.N == 0) return ITG_OK;
  if (p.K == 0) {
    int64_t n = p.M * p.N;  // C is dense with exactly M*N elements
    k_scale_or_zero<<<itg_blocks_for(n, 256, h->num_sms * 8), 256, 0, h->stream>>>(n, beta, C);
    ITG_CHECK_LAUNCH(h);
    return ITG_OK;
  }
  if (precision == ITG_PREC_SPLIT) {
    int bn = 0;
    ITG_TRY(tune::choose_split(h, p, A, B, alpha, bn));
    return itg_split_gemm(h, p, A, B, C, alpha, beta, bn);
  }
  int tile = ITG_TILE_128x128;
  ITG_TRY(tune::choose_f64(h, p, A, B, alpha, tile));
  return launch_gemm(h, tile, p, A, B, C, alpha, beta);
}

int contract_f64(itg_handle* h, double alpha, const double* A, int rankA, const int64_t* dimsA,
                 const int32_t* modesA, const double* B, int rankB, const int64_t* dimsB,
                 const int32_t* modesB, double beta, double* C, int rankC, const int64_t* dimsC,
                 const int32_t* modesC, int precision) {
  std::shared_ptr<ContractPlan> plan;
  ITG_TRY(get_plan(h, rankA, dimsA, modesA, rankB, dimsB, modesB, rankC, dimsC, modesC, plan));
  return run_plan(h, *plan, alpha, A, B, beta, C, precision);
}

}  // namespace itg

extern "C" int itg_contract(itg_handle* h, int dtype, double alpha, const void* A, int rankA,
                            const int64_t* dimsA, const int32_t* modesA, const void* B, int rankB,
                            const int64_t* dimsB, const int32_t* modesB, double beta, void* C,
                            int rankC, const int64_t* dimsC, const int32_t* modesC, int precision) {
  if (!h) return ITG_ERR_INVALID;
  if (dtype != ITG_F64 && dtype != ITG_C64) return itg_fail(h, ITG_ERR_UNSUPPORTED, "dtype %d not supported", dtype);
  if (dtype == ITG_C64) {
    const double al[2] = {alpha, 0.0}, be[2] = {beta, 0.0};
    return itg_contract_z(h, ITG_C64, ITG_C64, al, A, rankA, dimsA, modesA, B, rankB, dimsB, modesB, be, C, rankC,
                          dimsC, modesC, precision);
  }
  if (precision != ITG_PREC_FP64 && precision != ITG_PREC_SPLIT)
    return itg_fail(h, ITG_ERR_INVALID, "unknown precision %d", precision);
  if (rankA < 0 || rankB < 0 || rankC < 0 || rankA > ITG_MAX_RANK || rankB > ITG_MAX_RANK ||
      rankC > ITG_MAX_RANK)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank outside 0..%d", ITG_MAX_RANK);
  if ((rankA && (!dimsA || !modesA)) || (rankB && (!dimsB || !modesB)) ||
      (rankC && (!dimsC || !modesC)))
    return itg_fail(h, ITG_ERR_INVALID, "null dims/modes");
  if (!A || !B || !C) return itg_fail(h, ITG_ERR_INVALID, "null tensor pointer");
  if (C == A || C == B) return itg_fail(h, ITG_ERR_INVALID, "C must not alias A or B");
  for (int i = 0; i < rankA; ++i)
    if (dimsA[i] < 0) return itg_fail(h, ITG_ERR_SHAPE, "negative dimension");
  for (int i = 0; i < rankB; ++i)
    if (dimsB[i] < 0) return itg_fail(h, ITG_ERR_SHAPE, "negative dimension");
  for (int i = 0; i < rankC; ++i)
    if (dimsC[i] < 0) return itg_fail(h, ITG_ERR_SHAPE, "negative dimension");
  return itg::contract_f64(h, alpha, (const double*)A, rankA, dimsA, modesA, (const double*)B, rankB,
                           dimsB, modesB, beta, (double*)C, rankC, dimsC, modesC, precision);
}

namespace itg {
// Grouped FP64 contraction: `count` problems sharing ranks and mode labels,
// each with its own dims and pointers (dims arrays are concatenated per problem).
int contract_grouped_f64(itg_handle* h, int count, double alpha, const double* const* A, int rankA,
                         const int64_t* dimsA, const int32_t* modesA, const double* const* B, int rankB,
                         const int64_t* dimsB, const int32_t* modesB, double beta, double* const* C,
                         int rankC, const int64_t* dimsC, const int32_t* modesC) {
  if (count <= 0) return ITG_OK;
  std::vector<std::shared_ptr<ContractPlan>> plans(count);
  double sumM = 0, sumN = 0, sumK = 0;
  int64_t out_elems = 0;
  for (int i = 0; i < count; ++i) {
    ITG_TRY(get_plan(h, rankA, dimsA + (int64_t)i * rankA, modesA, rankB, dimsB + (int64_t)i * rankB,
                     modesB, rankC, dimsC + (int64_t)i * rankC, modesC, plans[i]));
    const ContractPlan& pl = *plans[i];
    if (pl.M == 0 || pl.N == 0 || pl.K == 0)
      return itg_fail(h, ITG_ERR_UNSUPPORTED, "grouped contraction with an empty problem");
    sumM += (double)pl.M;
    sumN += (double)pl.N;
    sumK += (double)pl.K;
    out_elems += (pl.M * pl.N + 31) / 32 * 32;
  }
  // descriptors for one tile variant, C_i taken from `outs`
  auto build = [&](int tile, double* const* outs, double* tune_out, std::vector<GroupProb>& probs) -> int64_t {
    const int bm = tile_bm(tile), bn = tile_bn(tile);
    probs.clear();
    probs.reserve(count);
    int64_t tiles = 0, off = 0;
    for (int i = 0; i < count; ++i) {
      const ContractPlan& pl = *plans[i];
      GroupProb g;
      g.A = A[i];
      g.B = B[i];
      if (tune_out) {
        g.C = tune_out + off;
        off += (pl.M * pl.N + 31) / 32 * 32;
      } else {
        g.C = outs[i];
      }
      g.tables = pl.tables;
      g.M = pl.M;
      g.N = pl.N;
      g.K = pl.K;
      g.tiles_n = (pl.N + bn - 1) / bn;
      g.tile_start = tiles;
      g.flags = (pl.a_kmaj ? 1 : 0) | (pl.b_kmaj ? 2 : 0);
      tiles += ((pl.M + bm - 1) / bm) * g.tiles_n;
      probs.push_back(g);
    }
    return tiles;
  };
  auto launch = [&](int tile, const GroupProb* dprobs, int64_t tiles, double bta) -> int {
    if (tiles > (int64_t)INT32_MAX) return itg_fail(h, ITG_ERR_UNSUPPORTED, "grouped: too many tiles");
    ProfScope prof(h, ITG_KERNEL_GEMM_F64);
    switch (tile) {
      case ITG_TILE_64x64: {
        static bool attr = false;
        if (!attr) {
          ITG_CUDA(h, cudaFuncSetAttribute(k_gemm_gather_f64_grouped<64, 64>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem<64, 64>()));
          attr = true;
        }
        k_gemm_gather_f64_grouped<64, 64><<<(unsigned)tiles, GTHREADS, gemm_smem<64, 64>(), h->stream>>>(
            dprobs, count, alpha, bta);
        break;
      }
      case ITG_TILE_128x64: {
        static bool attr = false;
        if (!attr) {
          ITG_CUDA(h, cudaFuncSetAttribute(k_gemm_gather_f64_grouped<128, 64>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem<128, 64>()));
          attr = true;
        }
        k_gemm_gather_f64_grouped<128, 64><<<(unsigned)tiles, GTHREADS, gemm_smem<128, 64>(), h->stream>>>(
            dprobs, count, alpha, bta);
        break;
      }
      default: {
        static bool attr = false;
        if (!attr) {
          ITG_CUDA(h, cudaFuncSetAttribute(k_gemm_gather_f64_grouped<128, 128>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)gemm_smem<128, 128>()));
          attr = true;
        }
        k_gemm_gather_f64_grouped<128, 128><<<(unsigned)tiles, GTHREADS, gemm_smem<128, 128>(), h->stream>>>(
            dprobs, count, alpha, bta);
        break;
      }
    }
    ITG_CHECK_LAUNCH(h);
    return ITG_OK;
  };
  // tile choice: cached per shape class (mode structure, log2 of the mean
  // M, N, K and of the count), timed on first use when the GPU is under-filled
  int64_t t128 = 0;
  for (int i = 0; i < count; ++i) t128 += tile_count(ITG_TILE_128x128, plans[i]->M, plans[i]->N);
  int tile = t128 >= h->num_sms ? ITG_TILE_128x128
             : (2 * t128 >= h->num_sms ? ITG_TILE_128x64 : ITG_TILE_64x64);
  std::vector<GroupProb> probs;
  if (t128 < 4 * (int64_t)h->num_sms) {
    std::vector<int64_t> ones(ITG_MAX_RANK, 1);
    auto lg = [](double x) { return (int)std::lround(std::log2(x > 1.0 ? x : 1.0)); };
    std::ostringstream os;
    os << "grp|" << plan_key(rankA, ones.data(), modesA, rankB, ones.data(), modesB, rankC, ones.data(), modesC)
       << '|' << lg(sumM / count) << ',' << lg(sumN / count) << ',' << lg(sumK / count) << ',' << lg(count);
    const std::string k = os.str();
    int v = 0;
    if (tune::lookup(k, v)) {
      tile = v;
    } else if (h->autotune && !tune::capturing(h)) {
      std::vector<GroupProb> tp;
      const size_t out_bytes = itg_align256(sizeof(double) * (size_t)out_elems);
      ITG_TRY(tune::reserve(h, out_bytes + itg_align256(sizeof(GroupProb) * count)));
      double* tout = (double*)h->tune_buf;
      GroupProb* tdesc = (GroupProb*)((char*)h->tune_buf + out_bytes);
      const bool prof = h->prof_on;
      h->prof_on = false;
      float best = 1e30f;
      int best_tile = tile, st = ITG_OK;
      for (int cand : {ITG_TILE_128x128, ITG_TILE_128x64, ITG_TILE_64x64}) {
        const int64_t tiles = build(cand, nullptr, tout, tp);
        if (cudaMemcpy(tdesc, tp.data(), sizeof(GroupProb) * tp.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
          st = itg_fail(h, ITG_ERR_CUDA, "autotune descriptor upload failed");
          break;
        }
        float ms = 0.f;
        st = tune::time_variant(h, [&]() { return launch(cand, tdesc, tiles, 0.0); }, ms);
        if (st != ITG_OK) break;
        if (ms < best) {
          best = ms;
          best_tile = cand;
        }
      }
      h->prof_on = prof;
      ITG_TRY(st);
      h->tune_runs++;
      tune::store(k, best_tile);
      tile = best_tile;
    }
  }
  const int64_t tiles = build(tile, C, nullptr, probs);
  const size_t bytes = sizeof(GroupProb) * probs.size();
  if (bytes > h->group_desc_bytes) {
    if (h->group_desc) {
      ITG_CUDA(h, cudaStreamSynchronize(h->stream));
      cudaFree(h->group_desc);
      h->group_desc = nullptr;
      h->group_desc_bytes = 0;
    }
    const size_t want = itg_align256(bytes * 2);
    if (cudaMalloc(&h->group_desc, want) != cudaSuccess)
      return itg_fail(h, ITG_ERR_ALLOC, "grouped descriptor allocation failed");
    h->group_desc_bytes = want;
  }
  // Pageable source: the copy is staged before the call returns, so `probs`
  // may go out of scope; the stream orders it before the kernel.
  ITG_CUDA(h, cudaMemcpyAsync(h->group_desc, probs.data(), bytes, cudaMemcpyHostToDevice, h->stream));
  return launch(tile, (const GroupProb*)h->group_desc, tiles, beta);
}
}  // namespace itg

extern "C" int itg_contract_grouped(itg_handle* h, int count, double alpha, const void* const* A,
                                    int rankA, const int64_t* dimsA, const int32_t* modesA,
                                    const void* const* B, int rankB, const int64_t* dimsB,
                                    const int32_t* modesB, double beta, void* const* C, int rankC,
                                    const int64_t* dimsC, const int32_t* modesC) {
  if (!h || count < 0 || (count > 0 && (!A || !B || !C || !dimsA || !dimsB || !dimsC)))
    return ITG_ERR_INVALID;
  if (rankA > ITG_MAX_RANK || rankB > ITG_MAX_RANK || rankC > ITG_MAX_RANK || rankA < 0 || rankB < 0 ||
      rankC < 0)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank outside 0..%d", ITG_MAX_RANK);
  for (int i = 0; i < count; ++i)
    if (!A[i] || !B[i] || !C[i] || C[i] == A[i] || C[i] == B[i])
      return itg_fail(h, ITG_ERR_INVALID, "grouped problem %d: null or aliased pointer", i);
  return itg::contract_grouped_f64(h, count, alpha, (const double* const*)A, rankA, dimsA, modesA,
                                   (const double* const*)B, rankB, dimsB, modesB, beta,
                                   (double* const*)C, rankC, dimsC, modesC);
}

extern "C" int itg_matmul(itg_handle* h, int64_t m, int64_t n, int64_t k, const double* A,
                          const double* B, double* C, int precision) {
  if (!h) return ITG_ERR_INVALID;
  int64_t dA[2] = {m, k}, dB[2] = {k, n}, dC[2] = {m, n};
  int32_t mA[2] = {0, 2}, mB[2] = {2, 1}, mC[2] = {0, 1};
  return itg_contract(h, ITG_F64, 1.0, A, 2, dA, mA, B, 2, dB, mB, 0.0, C, 2, dC, mC, precision);
}

extern "C" int itg_set_autotune(itg_handle* h, int enable) {
  if (!h) return ITG_ERR_INVALID;
  h->autotune = enable != 0;
  return ITG_OK;
}

extern "C" int itg_autotune_info(itg_handle* h, int64_t* entries, int64_t* tunings) {
  if (!h) return ITG_ERR_INVALID;
  if (entries) *entries = tune::size();
  if (tunings) *tunings = h->tune_runs;
  return ITG_OK;
}

extern "C" int itg_autotune_clear(itg_handle* h) {
  if (!h) return ITG_ERR_INVALID;
  tune::clear();
  for (auto& kv : h->plans) {
    kv.second->tile = -1;
    kv.second->split_bn = 0;
  }
  return ITG_OK;
}

extern "C" int itg_autotune_query(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA,
                                  int rankB, const int64_t* dimsB, const int32_t* modesB, int rankC,
                                  const int64_t* dimsC, const int32_t* modesC, int* tile, int* split_bn) {
  if (!h || !tile || !split_bn) return ITG_ERR_INVALID;
  if (rankA < 0 || rankB < 0 || rankC < 0 || rankA > ITG_MAX_RANK || rankB > ITG_MAX_RANK || rankC > ITG_MAX_RANK)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank outside 0..%d", ITG_MAX_RANK);
  std::shared_ptr<ContractPlan> plan;
  ITG_TRY(itg::get_plan(h, rankA, dimsA, modesA, rankB, dimsB, modesB, rankC, dimsC, modesC, plan));
  const ContractPlan& p = *plan;
  int v = 0;
  if (p.tile >= 0) *tile = p.tile;
  else if (tune::lookup("f64|" + p.key, v)) *tile = v;
  else *tile = tune::heuristic_tile(h, p.M, p.N);
  if (p.split_bn) *split_bn = p.split_bn;
  else if (tune::lookup("split|" + p.key, v)) *split_bn = v;
  else *split_bn = p.N <= 128 ? ITG_SPLIT_BN_128 : ITG_SPLIT_BN_256;
  return ITG_OK;
}

extern "C" int itg_autotune_force(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA,
                                  int rankB, const int64_t* dimsB, const int32_t* modesB, int rankC,
                                  const int64_t* dimsC, const int32_t* modesC, int tile, int split_bn) {
  if (!h) return ITG_ERR_INVALID;
  if (tile > ITG_TILE_64x64 ||
      (split_bn > 0 && (split_bn & ~ITG_SPLIT_STREAMK) != ITG_SPLIT_BN_128 &&
       (split_bn & ~ITG_SPLIT_STREAMK) != ITG_SPLIT_BN_256))
    return itg_fail(h, ITG_ERR_INVALID, "unknown variant (tile %d, split_bn %d)", tile, split_bn);
  if (rankA < 0 || rankB < 0 || rankC < 0 || rankA > ITG_MAX_RANK || rankB > ITG_MAX_RANK || rankC > ITG_MAX_RANK)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "rank outside 0..%d", ITG_MAX_RANK);
  std::shared_ptr<ContractPlan> plan;
  ITG_TRY(itg::get_plan(h, rankA, dimsA, modesA, rankB, dimsB, modesB, rankC, dimsC, modesC, plan));
  if (tile >= 0) {
    plan->tile = tile;
    tune::store("f64|" + plan->key, tile);
  }
  if (split_bn > 0) {
    plan->split_bn = split_bn;
    tune::store("split|" + plan->key, split_bn);
  }
  return ITG_OK;
}
