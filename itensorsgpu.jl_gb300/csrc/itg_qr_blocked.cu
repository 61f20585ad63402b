// Blocked Householder QR and the application of its Q, with the trailing
// updates as matrix products through the contraction engine (compact WY form
// of Schreiber & Van Loan, "A storage-efficient WY representation for
// products of Householder transformations", SIAM J. Sci. Stat. Comput. 10
// (1989); the T recurrence is LAPACK's larft, restated).
//
// Panel of QR_NB columns: the column steps of k_house_step (itg_factor.cu)
// restricted to the panel, then T (upper triangular, Q_p = I - V T V^T) from
// Y = V^T V, then the trailing columns A_t <- (I - V T^T V^T) A_t as three
// products: Z = V^T A_t (thin: split over K chunks), Z2 = T^T Z, A_t -= V Z2.  Q [X; 0] applies the panels
// in reverse order with Y <- Y - V (T (V^T Y)).  The products address
// submatrices in place through offset tables filled on the device, so they run
// on the FP64 gather-GEMM or on the split tensor-core path without copies.
#include "itg_internal.cuh"

namespace itg {
int run_plan(itg_handle* h, const ContractPlan& p, double alpha, const double* A, const double* B, double beta,
             double* C, int precision);
void house_step_launch(itg_handle* h, double* A, int64_t m, int j, int ncta, double* Vh, double* tau,
                       double* rdiag);
}  // namespace itg

namespace {

struct Aff {
  int64_t base, stride;
};

// offAm[M] offCm[M] offBn[N] offCn[N] offAk[K] offBk[K] (ContractPlan order)
__global__ void k_fill_tables(int64_t* __restrict__ T, int64_t M, int64_t N, int64_t K, Aff am, Aff cm, Aff bn,
                              Aff cn, Aff ak, Aff bk) {
  const int64_t tot = 2 * M + 2 * N + 2 * K;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i;
    Aff a;
    if (r < M) a = am;
    else if ((r -= M) < M) a = cm;
    else if ((r -= M) < N) a = bn;
    else if ((r -= N) < N) a = cn;
    else if ((r -= N) < K) a = ak;
    else { r -= K; a = bk; }
    T[i] = a.base + a.stride * r;
  }
}

struct TabPlan : ContractPlan {
  ~TabPlan() { tables = nullptr; }  // the tables live in the handle's buffer
};

// Both offset-table buffers hold at least `elems` entries.  Growing one waits
// for the whole device: the look-ahead stream may still read the old buffer.
int tab_reserve(itg_handle* h, int64_t elems) {
  if (elems <= h->tab_buf_elems && elems <= h->tab_buf2_elems) return ITG_OK;
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->qr_stream) ITG_CUDA(h, cudaStreamSynchronize(h->qr_stream));
  for (int b = 0; b < 2; ++b) {
    int64_t*& buf = b ? h->tab_buf2 : h->tab_buf;
    int64_t& cap = b ? h->tab_buf2_elems : h->tab_buf_elems;
    if (elems <= cap) continue;
    if (buf) cudaFree(buf);
    buf = nullptr;
    cap = 0;
    if (cudaMalloc((void**)&buf, sizeof(int64_t) * elems) != cudaSuccess)
      return itg_fail(h, ITG_ERR_ALLOC, "QR offset tables");
    cap = elems;
  }
  return ITG_OK;
}

// C[M x N] = alpha * A B + beta * C over submatrices described by affine
// offsets, on the handle's current stream with the offset tables in `tab`
// (tab_reserve'd: at least 2 (M + N + K) entries).
int strided_gemm(itg_handle* h, int64_t M, int64_t N, int64_t K, double alpha, const double* A, Aff am, Aff ak,
                 bool a_kmaj, const double* B, Aff bk, Aff bn, bool b_kmaj, double beta, double* C, Aff cm, Aff cn,
                 int precision, int64_t* tab) {
  if (M <= 0 || N <= 0 || K <= 0) return ITG_OK;
  const int64_t tot = 2 * M + 2 * N + 2 * K;
  k_fill_tables<<<itg_blocks_for(tot, 256, 64), 256, 0, h->stream>>>(tab, M, N, K, am, cm, bn, cn, ak, bk);
  ITG_CHECK_LAUNCH(h);
  TabPlan p;
  p.M = M;
  p.N = N;
  p.K = K;
  p.tables = tab;
  p.a_kmaj = a_kmaj;
  p.b_kmaj = b_kmaj;
  return itg::run_plan(h, p, alpha, A, B, beta, C, precision);
}

// T (nb x nb, leading dimension ldt, upper triangular) from Y = V^T V:
// T(j,j) = tau_j, T(0:j, j) = -tau_j T(0:j, 0:j) Y(0:j, j).
__global__ void k_larft(const double* __restrict__ Y, int ldy, const double* __restrict__ tau, int nb,
                        double* __restrict__ T, int ldt) {
  __shared__ double col[QR_NB_MAX];
  const int i = threadIdx.x;
  for (int q = i; q < nb * ldt; q += blockDim.x) T[q] = 0.0;
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const double tj = tau[j];
    double s = 0.0;
    if (i < j)
      for (int l = i; l < j; ++l) s = fma(T[i + (int64_t)l * ldt], Y[l + (int64_t)j * ldy], s);
    __syncthreads();  // every read of column j's inputs is done before the writes
    if (i < j) col[i] = -tj * s;
    __syncthreads();
    if (i < j) T[i + (int64_t)j * ldt] = col[i];
    if (i == j) T[j + (int64_t)j * ldt] = tj;
    __syncthreads();
  }
}

// C (bw x N, ld ldc) = V_p^T B for the panel's reflectors V_p (columns jb..jb+bw
// of Vh, rows jb..m) and N columns of B (ld ldb, rows jb..m): bw <= 32 rows of
// dot products of length K = m - jb.  The product is too thin for the tiled
// GEMM (it would run N / 64 CTAs), so the K range is split over gridDim.y
// chunks whose partial results are summed in chunk order by k_skinny_reduce.
constexpr int SK_TILE_K = 64;
constexpr int QR_PART_CHUNKS = 16;  // K chunks of the thin products (partials: 16 x 32 x N)
__global__ void __launch_bounds__(256)
k_skinny_partial(const double* __restrict__ Vh, int64_t m, int64_t jb, int bw, const double* __restrict__ B,
                 int64_t ldb, int64_t b0, int64_t N, int64_t kchunk, double* __restrict__ part) {
  __shared__ double vs[32][SK_TILE_K + 1];
  __shared__ double bs[32][SK_TILE_K + 1];
  const int t = threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.x * 32;
  const int64_t K = m - jb;
  const int64_t k_lo = (int64_t)blockIdx.y * kchunk;
  const int64_t k_hi = k_lo + kchunk < K ? k_lo + kchunk : K;
  const int r = t / 8, cq = (t % 8) * 4;  // each thread: row r, columns cq..cq+3
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t k0 = k_lo; k0 < k_hi; k0 += SK_TILE_K) {
    for (int i = t; i < 32 * SK_TILE_K; i += 256) {
      const int col = i / SK_TILE_K, kk = i % SK_TILE_K;
      const int64_t k = k0 + kk;
      const bool kin = k < k_hi;
      vs[col][kk] = (kin && col < bw) ? Vh[(jb + col) * m + jb + k] : 0.0;
      const int64_t c = c0 + col;
      bs[col][kk] = (kin && c < N) ? B[(b0 + c) * ldb + jb + k] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < SK_TILE_K; ++kk) {
      const double v = vs[r][kk];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(v, bs[cq + q][kk], acc[q]);
    }
    __syncthreads();
  }
  double* P = part + (int64_t)blockIdx.y * 32 * N;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t c = c0 + cq + q;
    if (c < N) P[r + 32 * c] = acc[q];
  }
}

__global__ void k_skinny_reduce(const double* __restrict__ part, int nchunk, int bw, int64_t N,
                                double* __restrict__ C, int64_t ldc) {
  const int64_t tot = 32 * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i % 32);
    const int64_t c = i / 32;
    if (r >= bw) continue;
    double s = 0.0;
    for (int q = 0; q < nchunk; ++q) s += part[(int64_t)q * tot + i];
    C[r + c * ldc] = s;
  }
}

int skinny_vt_b(itg_handle* h, const double* Vh, int64_t m, int64_t jb, int bw, const double* B, int64_t ldb,
                int64_t b0, int64_t N, double* C, int64_t ldc, double* part, int64_t part_doubles) {
  if (N <= 0) return ITG_OK;
  const int64_t K = m - jb;
  const int64_t ntile = (N + 31) / 32;
  int64_t nchunk = (4 * (int64_t)h->num_sms + ntile - 1) / ntile;
  const int64_t maxc = (K + SK_TILE_K - 1) / SK_TILE_K;
  if (nchunk > maxc) nchunk = maxc;
  if (nchunk > part_doubles / (32 * N)) nchunk = part_doubles / (32 * N);
  if (nchunk < 1) return itg_fail(h, ITG_ERR_INVALID, "skinny product: partial buffer too small");
  const int64_t kchunk = ((K + nchunk - 1) / nchunk + SK_TILE_K - 1) / SK_TILE_K * SK_TILE_K;
  nchunk = (K + kchunk - 1) / kchunk;
  k_skinny_partial<<<dim3((unsigned)ntile, (unsigned)nchunk), 256, 0, h->stream>>>(Vh, m, jb, bw, B, ldb, b0, N,
                                                                                   kchunk, part);
  k_skinny_reduce<<<itg_blocks_for(32 * N, 256, 1024), 256, 0, h->stream>>>(part, (int)nchunk, bw, N, C, ldc);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}

}  // namespace

namespace itg {

// Blocked Householder QR of W (m x n, ld m) in place with nref <= min(m, n)
// reflectors (nref = n for the tall case, m for a wide matrix): reflectors in
// Vh (m x nref, explicit unit diagonal, zeros above), tau, R's diagonal in rd,
// the rest of R's rows above the diagonal in W; Tbuf holds QR_NB^2 doubles
// per panel of reflectors and ws qr_blocked_ws_doubles(n) doubles.
//
// Look-ahead: the column steps of a panel are bound by their serial FP64
// scalar work and occupy few SMs.  They run on a stream of the greatest
// priority (qr_stream), so that their blocks are scheduled ahead of the
// trailing updates' product blocks, which run on the handle's stream: once
// panel p's reflectors and T are final, the panel stream updates the columns
// of panel p + 1 by them and factors panel p + 1 at once, while the handle's
// stream updates the rest of the trailing matrix by panel p.  The panel stream
// waits for that update before it applies the next panel's reflectors to the
// columns the update covers.  Each stream has its own Z, Z2, partial-sum and
// offset-table buffers.  Results are deterministic (the split of V^T A's K
// range into chunks depends only on the column counts).
namespace {
struct QrBufs {
  double *Z, *Z2, *part;
  int64_t part_doubles;
  int64_t* tab;
};

// A(:, c0 : c0 + nc) -= V_p (T_p^T (V_p^T A(:, c0 : c0 + nc))) on the handle's current stream
int qr_update_cols(itg_handle* h, double* W, int64_t m, int64_t jb, int64_t bw, const double* Vh, const double* Tp,
                   int64_t c0, int64_t nc, const QrBufs& b, int precision) {
  if (nc <= 0) return ITG_OK;
  const int NB = QR_NB;
  ITG_TRY(skinny_vt_b(h, Vh, m, jb, (int)bw, W, m, c0, nc, b.Z, bw, b.part, b.part_doubles));
  ITG_TRY(strided_gemm(h, bw, nc, bw, 1.0, Tp, Aff{0, NB}, Aff{0, 1}, true, b.Z, Aff{0, 1}, Aff{0, bw}, true, 0.0,
                       b.Z2, Aff{0, 1}, Aff{0, bw}, precision, b.tab));
  return strided_gemm(h, m - jb, nc, bw, -1.0, Vh, Aff{jb, 1}, Aff{jb * m, m}, false, b.Z2, Aff{0, 1}, Aff{0, bw},
                      true, 1.0, W, Aff{jb, 1}, Aff{c0 * m, m}, precision, b.tab);
}

// The handle's stream is swapped for the panel stream while this lives.
struct OnStream {
  itg_handle* h;
  cudaStream_t saved;
  OnStream(itg_handle* hh, cudaStream_t s) : h(hh), saved(hh->stream) { h->stream = s; }
  ~OnStream() { h->stream = saved; }
};

int qr_lookahead_init(itg_handle* h) {
  if (h->qr_stream) return ITG_OK;
  int least = 0, greatest = 0;
  ITG_CUDA(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
  ITG_CUDA(h, cudaStreamCreateWithPriority(&h->qr_stream, cudaStreamNonBlocking, greatest));
  ITG_CUDA(h, cudaEventCreateWithFlags(&h->qr_ev_ready, cudaEventDisableTiming));
  ITG_CUDA(h, cudaEventCreateWithFlags(&h->qr_ev_done, cudaEventDisableTiming));
  return ITG_OK;
}
}  // namespace

int qr_blocked(itg_handle* h, double* W, int64_t m, int64_t n, int64_t nref, double* Vh, double* tau, double* rd,
               double* Tbuf, double* ws, int precision) {
  const int NB = QR_NB;
  const int64_t part_doubles = QR_PART_CHUNKS * 32 * n;
  double* Ym = ws;
  QrBufs bp{ws + NB * NB, ws + NB * NB + (int64_t)NB * n, ws + NB * NB + 2 * (int64_t)NB * n, part_doubles,
            nullptr};  // panel stream
  double* ws2 = bp.part + part_doubles;
  QrBufs bu{ws2, ws2 + (int64_t)NB * n, ws2 + 2 * (int64_t)NB * n, part_doubles, nullptr};  // update stream
  ITG_TRY(qr_lookahead_init(h));
  ITG_TRY(tab_reserve(h, 2 * (m + n + NB)));
  bp.tab = h->tab_buf;
  bu.tab = h->tab_buf2;
  cudaStream_t main_stream = h->stream;
  // the panel stream starts after everything already queued on the handle's stream
  ITG_CUDA(h, cudaEventRecord(h->qr_ev_done, main_stream));
  {
    OnStream on(h, h->qr_stream);
    ITG_CUDA(h, cudaStreamWaitEvent(h->stream, h->qr_ev_done, 0));
    if (nref > 0)
      for (int64_t j = 0; j < (nref < NB ? nref : NB); ++j)
        house_step_launch(h, W, m, (int)j, (int)((nref < NB ? nref : NB) - j), Vh, tau, rd);
    ITG_CHECK_LAUNCH(h);
  }
  for (int64_t jb = 0, panel = 0; jb < nref; jb += NB, ++panel) {
    const int64_t bw = (nref - jb < NB) ? nref - jb : NB;
    const int64_t nt = n - jb - bw;
    double* Tp = Tbuf + panel * NB * NB;
    const int64_t jn = jb + bw;
    const int64_t nnext = nt > 0 && jn < nref ? ((nref - jn < NB) ? nref - jn : NB) : 0;
    const int64_t nrest = nt > 0 ? nt - nnext : 0;
    {
      OnStream on(h, h->qr_stream);
      // Y = V_p^T V_p (FP64: it defines T)
      ITG_TRY(skinny_vt_b(h, Vh, m, jb, (int)bw, Vh, m, jb, bw, Ym, bw, bp.part, part_doubles));
      k_larft<<<1, QR_NB_MAX, 0, h->stream>>>(Ym, (int)bw, tau + jb, (int)bw, Tp, NB);
      ITG_CHECK_LAUNCH(h);
      if (nt <= 0) continue;
      // V_p and T_p are final: the handle's stream may update the rest
      ITG_CUDA(h, cudaEventRecord(h->qr_ev_ready, h->stream));
      // panel p + 1's columns got panel p - 1's update on the handle's stream
      if (panel > 0) ITG_CUDA(h, cudaStreamWaitEvent(h->stream, h->qr_ev_done, 0));
      ITG_TRY(qr_update_cols(h, W, m, jb, bw, Vh, Tp, jn, nnext, bp, precision));
    }
    if (nrest > 0) {
      ITG_CUDA(h, cudaStreamWaitEvent(main_stream, h->qr_ev_ready, 0));
      ITG_TRY(qr_update_cols(h, W, m, jb, bw, Vh, Tp, jn + nnext, nrest, bu, precision));
    }
    ITG_CUDA(h, cudaEventRecord(h->qr_ev_done, main_stream));
    if (nnext > 0) {
      OnStream on(h, h->qr_stream);
      for (int64_t j = jn; j < jn + nnext; ++j) house_step_launch(h, W, m, (int)j, (int)(jn + nnext - j), Vh, tau, rd);
      ITG_CHECK_LAUNCH(h);
    }
  }
  // the handle's stream continues after the last panel's work
  ITG_CUDA(h, cudaEventRecord(h->qr_ev_ready, h->qr_stream));
  ITG_CUDA(h, cudaStreamWaitEvent(main_stream, h->qr_ev_ready, 0));
  return ITG_OK;
}

// Y <- Q Y on the first ncols columns of Y (m rows, ld m), Q from qr_blocked;
// FP64 products (Q's orthogonality is what the callers rely on).
int q_apply_blocked(itg_handle* h, double* Y, int64_t m, int64_t n, int64_t ncols, const double* Vh,
                    const double* Tbuf, double* ws) {
  if (ncols <= 0) return ITG_OK;
  const int NB = QR_NB;
  double* Z = ws + NB * NB;
  double* Z2 = Z + (int64_t)NB * ncols;
  double* part = Z2 + (int64_t)NB * ncols;
  const int64_t part_doubles = QR_PART_CHUNKS * 32 * ncols;
  ITG_TRY(tab_reserve(h, 2 * (m + ncols + NB)));
  const int64_t npanel = (n + NB - 1) / NB;
  for (int64_t panel = npanel - 1; panel >= 0; --panel) {
    const int64_t jb = panel * NB;
    const int64_t bw = (n - jb < NB) ? n - jb : NB;
    const double* Tp = Tbuf + panel * NB * NB;
    // Z = V_p^T Y(jb:m, :)
    ITG_TRY(skinny_vt_b(h, Vh, m, jb, (int)bw, Y, m, 0, ncols, Z, bw, part, part_doubles));
    // Z2 = T Z
    ITG_TRY(strided_gemm(h, bw, ncols, bw, 1.0, Tp, Aff{0, 1}, Aff{0, NB}, false, Z, Aff{0, 1}, Aff{0, bw}, true,
                         0.0, Z2, Aff{0, 1}, Aff{0, bw}, ITG_PREC_FP64, h->tab_buf));
    // Y(jb:m, :) -= V_p Z2
    ITG_TRY(strided_gemm(h, m - jb, ncols, bw, -1.0, Vh, Aff{jb, 1}, Aff{jb * m, m}, false, Z2, Aff{0, 1},
                         Aff{0, bw}, true, 1.0, Y, Aff{jb, 1}, Aff{0, m}, ITG_PREC_FP64, h->tab_buf));
  }
  return ITG_OK;
}

// Y, then Z, Z2 and the partial sums of the handle's stream, then those of the
// look-ahead stream.
size_t qr_blocked_ws_doubles(int64_t n) {
  return (size_t)QR_NB * QR_NB + 2 * (2 * (size_t)QR_NB * n + (size_t)QR_PART_CHUNKS * 32 * n);
}
size_t qr_blocked_t_doubles(int64_t n) { return (size_t)((n + QR_NB - 1) / QR_NB) * QR_NB * QR_NB; }

}  // namespace itg
