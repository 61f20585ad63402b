// itg_heff2_apply_noalloc: the two-site H_eff matvec without any device
// allocation by the library.
//
// Some callers cannot let a library call cudaMalloc: applications that own all
// device memory through their own pool with a fixed budget (the Julia side of
// ITensors keeps its tensors in the CUDA.jl pool), and callers for which the
// device-wide synchronisation cudaMalloc may cause is unacceptable.  This entry
// point takes its intermediates (T1, T3, the merged MPO block and the two
// contraction-plan index tables) from one file-scope __device__ array of fixed
// size; the caller still passes every input and output.
//
// Limits and rules (also in include/itg.h):
//  * capacity ITG_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB) per device, held by
//    every GPU that loads libitg.so until the process exits; a problem that does
//    not fit returns ITG_ERR_UNSUPPORTED with the required and available sizes
//    (the sizes are checked factor by factor before any product is formed, so
//    no dimensions can wrap around the check);
//  * FP64 arithmetic only (the split path needs a larger workspace);
//  * the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (once per device, under a mutex); make that first call
//    before any stream capture;
//  * the contraction plans' offset tables are written into the array by a
//    kernel from a small by-value descriptor, so a call issues no host-to-device
//    copy;
//  * every call reuses the same array, so calls that overlap on the GPU (two
//    streams, two host threads) race; the array keeps the last call's contents,
//    and nothing in it needs to start at zero because every intermediate is
//    fully overwritten before it is read.
#include "itg_internal.cuh"

#include <mutex>
#include <vector>

#define ITG_NOALLOC_SCRATCH_DOUBLES (4 * 1024 * 1024)

static __device__ __align__(256) double g_noalloc_scratch[ITG_NOALLOC_SCRATCH_DOUBLES];

namespace itg {
int plan_tables_host(itg_handle* h, int rankA, const int64_t* dimsA, const int32_t* modesA,
                     int rankB, const int64_t* dimsB, const int32_t* modesB, int rankC,
                     const int64_t* dimsC, const int32_t* modesC, ContractPlan& pl,
                     std::vector<int64_t>& tab, PlanTableDesc* desc);
int run_plan(itg_handle* h, const ContractPlan& p, double alpha, const double* A, const double* B,
             double beta, double* C, int precision);
int heff_form_weff(itg_handle* h, int64_t d, int64_t wL, int64_t wM, int64_t wR, const double* W1,
                   const double* W2, double* Weff);
int heff_mid(itg_handle* h, int64_t rows, int nc, int nj, const double* T1, const double* Weff,
             double* T3);
}  // namespace itg

namespace {

std::mutex g_setup_mu;
double* g_scratch_ptr[256] = {nullptr};

int scratch_address(itg_handle* h, double** out) {
  if (h->device < 0 || h->device >= 256) return itg_fail(h, ITG_ERR_INVALID, "device id out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[h->device]) {
    int cur = -1;
    ITG_CUDA(h, cudaGetDevice(&cur));
    if (cur != h->device) ITG_CUDA(h, cudaSetDevice(h->device));
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != h->device) cudaSetDevice(cur);
    if (e != cudaSuccess || !p)
      return itg_fail(h, ITG_ERR_CUDA, "cudaGetSymbolAddress(no-allocation scratch) failed: %s",
                      cudaGetErrorString(e));
    g_scratch_ptr[h->device] = (double*)p;
  }
  *out = g_scratch_ptr[h->device];
  return ITG_OK;
}

// The six offset tables of a plan (layout of ContractPlan::tables: offAm offCm
// | offBn offCn | offAk offBk) from their mixed-radix description.
__global__ void k_plan_tables(const PlanTableDesc d, int64_t* __restrict__ t) {
  const int64_t M = d.count[0], N = d.count[1], K = d.count[2];
  const int64_t total = M + N + K;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int g = i < M ? 0 : (i < M + N ? 1 : 2);
    const int64_t l = g == 0 ? i : (g == 1 ? i - M : i - M - N);
    int64_t* o1 = g == 0 ? t : (g == 1 ? t + 2 * M : t + 2 * M + 2 * N);
    int64_t* o2 = o1 + d.count[g];
    int64_t r = l, a = 0, b = 0;
    for (int m = 0; m < d.nmodes[g]; ++m) {
      const int64_t q = r / d.dim[g][m], digit = r - q * d.dim[g][m];
      a += digit * d.s1[g][m];
      b += digit * d.s2[g][m];
      r = q;
    }
    o1[l] = a;
    o2[l] = b;
  }
}

// a * b when it stays <= cap (a, b >= 1), else -1; never overflows.
int64_t mul_capped(int64_t a, int64_t b, int64_t cap) {
  if (a < 1 || b < 1 || a > cap / b) return -1;
  return a * b;
}

// A ContractPlan whose tables live in the static array: never freed.
struct BorrowedPlan : ContractPlan {
  ~BorrowedPlan() { tables = nullptr; }
};

int64_t align32(int64_t n) { return (n + 31) & ~(int64_t)31; }  // 256-byte steps, in doubles

}  // namespace

extern "C" int itg_heff2_apply_noalloc(itg_handle* h, int64_t chiL, int64_t chiR, int64_t d,
                                       int64_t wL, int64_t wM, int64_t wR, const double* L,
                                       const double* W1, const double* W2, const double* R,
                                       const double* psi, double* out) {
  if (!h || !L || !W1 || !W2 || !R || !psi || !out) return ITG_ERR_INVALID;
  if (psi == out) return itg_fail(h, ITG_ERR_INVALID, "out must not alias psi");
  if (chiL <= 0 || chiR <= 0 || d <= 0 || wL <= 0 || wM <= 0 || wR <= 0)
    return itg_fail(h, ITG_ERR_SHAPE, "heff2_noalloc: non-positive dimension");
  // Sizes, each checked against the capacity before it is formed: T1 and T3
  // hold chiL * chiR * nc and chiL * chiR * nj doubles, so once those fit every
  // other buffer (the merged MPO block and the plans' tables, whose lengths are
  // sums of factors of T1 and T3) is bounded by a small multiple of the cap.
  const int64_t CAP = ITG_NOALLOC_SCRATCH_DOUBLES;
  const int64_t dd = mul_capped(d, d, CAP);
  const int64_t nc = dd < 0 ? -1 : mul_capped(wL, dd, CAP), nj = dd < 0 ? -1 : mul_capped(dd, wR, CAP);
  const int64_t chi2 = mul_capped(chiL, chiR, CAP);
  const int64_t nT1 = (chi2 < 0 || nc < 0) ? -1 : mul_capped(chi2, nc, CAP);
  const int64_t nT3 = (chi2 < 0 || nj < 0) ? -1 : mul_capped(chi2, nj, CAP);
  if (nT1 < 0 || nT3 < 0)
    return itg_fail(h, ITG_ERR_UNSUPPORTED,
                    "heff2_noalloc: the intermediates exceed the fixed no-allocation array of %lld doubles "
                    "(use itg_heff2_apply)",
                    (long long)CAP);
  if (nc * nj * 8 > 48 * 1024)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "heff2_noalloc: MPO block too large");
  // table lengths of the two chi^3 steps: 2 (M + N + K) each
  const int64_t nTab1 = 2 * (wL * chiL + dd * chiR + chiL);
  const int64_t nTab3 = 2 * (chiL * dd + chiR + chiR * wR);
  // layout in doubles: T1 | T3 | Weff | tables of step 1 | tables of step 3
  const int64_t oT1 = 0, oT3 = oT1 + align32(nT1), oW = oT3 + align32(nT3);
  const int64_t oTab1 = oW + align32(nc * nj), oTab3 = oTab1 + align32(nTab1);
  const int64_t need = oTab3 + align32(nTab3);
  if (need > CAP)
    return itg_fail(h, ITG_ERR_UNSUPPORTED,
                    "heff2_noalloc: needs %lld doubles of scratch, the fixed no-allocation array "
                    "holds %lld (use itg_heff2_apply)",
                    (long long)need, (long long)CAP);
  const int64_t dL[3] = {chiL, wL, chiL};
  const int32_t mL[3] = {1, 2, 3};
  const int64_t dP[4] = {chiL, d, d, chiR};
  const int32_t mP[4] = {1, 4, 5, 6};
  const int64_t dT1[5] = {chiL, chiR, wL, d, d};
  const int32_t mT1[5] = {3, 6, 2, 4, 5};
  const int64_t dT3[5] = {chiL, chiR, d, d, wR};
  const int32_t mT3[5] = {3, 6, 7, 9, 10};
  const int64_t dR[3] = {chiR, wR, chiR};
  const int32_t mR[3] = {6, 10, 11};
  const int64_t dO[4] = {chiL, d, d, chiR};
  const int32_t mO[4] = {3, 7, 9, 11};
  BorrowedPlan p1, p3;
  std::vector<int64_t> tab1, tab3;
  PlanTableDesc desc1, desc3;
  ITG_TRY(itg::plan_tables_host(h, 3, dL, mL, 4, dP, mP, 5, dT1, mT1, p1, tab1, &desc1));
  ITG_TRY(itg::plan_tables_host(h, 5, dT3, mT3, 3, dR, mR, 4, dO, mO, p3, tab3, &desc3));
  if ((int64_t)tab1.size() != nTab1 || (int64_t)tab3.size() != nTab3)
    return itg_fail(h, ITG_ERR_INVALID, "heff2_noalloc: unexpected plan table size");
  double* base = nullptr;
  ITG_TRY(scratch_address(h, &base));
  double* T1 = base + oT1;
  double* T3 = base + oT3;
  double* Weff = base + oW;
  p1.tables = (int64_t*)(base + oTab1);
  p3.tables = (int64_t*)(base + oTab3);
  k_plan_tables<<<itg_blocks_for(nTab1 / 2, 256, h->num_sms * 4), 256, 0, h->stream>>>(desc1, p1.tables);
  k_plan_tables<<<itg_blocks_for(nTab3 / 2, 256, h->num_sms * 4), 256, 0, h->stream>>>(desc3, p3.tables);
  ITG_CHECK_LAUNCH(h);
  ITG_TRY(itg::heff_form_weff(h, d, wL, wM, wR, W1, W2, Weff));
  ITG_TRY(itg::run_plan(h, p1, 1.0, L, psi, 0.0, T1, ITG_PREC_FP64));
  ITG_TRY(itg::heff_mid(h, chi2, (int)nc, (int)nj, T1, Weff, T3));
  ITG_TRY(itg::run_plan(h, p3, 1.0, T3, R, 0.0, out, ITG_PREC_FP64));
  return ITG_OK;
}
