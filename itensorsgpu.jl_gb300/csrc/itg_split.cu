// Split-precision contraction path (ITG_PREC_SPLIT): FP64 GEMM through exact
// integer products of bf16 slices on the tcgen05 tensor cores.
//
// Method (error-free splitting after Ozaki, Ogita, Oishi & Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012); integer
// slices with exact low-precision accumulation as in Ootomo, Ozaki & Yokota,
// "DGEMM on integer matrix multiplication unit", IJHPCA 2024):
//
//   Row m of A is scaled by 2^-e_m (|A[m,k]| < 2^e_m) and written in S = 6
//   balanced base-2^8 digits:  A[m,k] ~ 2^e_m sum_{p<S} a_p[m,k] 2^-8(p+1)
//   with |a_0| <= 256 and |a_p| <= 128 (p >= 1); every digit is an exact bf16
//   (8 significant bits).  Column n of B likewise with exponent f_n, digits b_q.
//   C[m,n] ~ 2^(e_m+f_n-16) sum_{L<S} 2^-8L sum_{p+q=L} (a_p b_q)[m,n]:
//   21 digit products for 48 bits of each operand.
//
// Each a_p b_q product is an integer GEMM run by tcgen05.mma (kind::f16, bf16
// in, FP32 accumulate in TMEM).  Products of one level L are accumulated in a
// TMEM buffer only while the sum of |a||b| bounds stays <= 2^24, so every FP32
// partial sum (a "group") is an exact integer.  The epilogue warps read the
// buffer into int32 registers, summing the groups of one level exactly, and
// hand it back to the MMA warp, which meanwhile fills the other TMEM buffer;
// at each level end the int32 sums are shifted into an exact int64
// fixed-point accumulator (2^F scaling).  After the last level the int64
// accumulator is converted to FP64 with integer instructions (round to
// nearest) and C is scattered through the contraction plan's offset tables.
// No FP64 arithmetic runs in the inner loops (GB300's FP64 rate is a small
// fraction of its tensor rate).
//
// Kernel roles (10 warps per CTA; a CTA computes one 128 x BN output tile,
// or, persistent, a sequence of tiles and parts of tiles, see Part):
//   warp 0    TMA producer: A/B slice tiles (64 bf16 of K per stage, 128B
//             swizzle) into a 4-stage shared-memory ring, mbarrier complete_tx
//   warp 1    TMEM allocator and single-thread tcgen05.mma issuer
//   warps 2-9 TMEM drain / epilogue: warp w reads TMEM lanes 32*(w%4)..+31 and
//             owns half of the tile's columns
// Every mbarrier wait is bounded (%globaltimer; the handle's wait limit,
// itg_set_wait_limit_ns, 4 s by default); on timeout the kernel records
// ITG_ERR_TIMEOUT, stops issuing work, waits (bounded, regardless of the
// abort) for its own copies and MMAs still in flight, frees TMEM and returns.
#include "itg_internal.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>
#include <cmath>



namespace split {

constexpr int S_SLICES = 6;    // digits per operand (8 bits each)
constexpr int BM = 128;        // tile rows (TMEM lanes)
constexpr int BK = 64;         // K per pipeline stage (128 bytes of bf16)
constexpr int STAGES = 4;
constexpr int NUM_EPI_WARPS = 8;  // two per TMEM lane quarter, each owning half the columns
constexpr int NUM_THREADS = 64 + 32 * NUM_EPI_WARPS;

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait (wait_ns of %globaltimer); returns false when it runs out,
// recording ITG_ERR_TIMEOUT and raising the CTA's abort flag, or when another
// role of the CTA raised the flag first.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err,
                                          volatile int* abort_flag, uint64_t wait_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63) == 63) {
      if (*abort_flag) return false;
      if (globaltimer() - t0 > wait_ns) {
        atomicExch(err, ITG_ERR_TIMEOUT);
        *abort_flag = 1;
        return false;
      }
    }
  }
}
// Bounded wait that ignores the abort flag: on the way out, for this CTA's own
// TMA copies and MMAs still in flight (they complete by themselves; the bound
// only guards against a wait that can never end).
__device__ __forceinline__ bool mbar_drain(uint64_t* bar, uint32_t parity, uint64_t wait_ns) {
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63) == 63 && globaltimer() - t0 > wait_ns) return false;
  }
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_ld_32x32b_x32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_ld_32x32b_x32_nowait(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_ld_32x32b_x16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_ld_32x32b_x16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_st_32x32b_x16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
      "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_st_32x32b_x32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]),
      "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]),
      "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// core groups 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading-dimension offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride-dimension offset
  d |= (uint64_t)1 << 46;            // version
  d |= (uint64_t)2 << 61;            // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Digit magnitude bounds: 2^8 for the leading digit, 2^7 for the others.
__host__ __device__ __forceinline__ int digit_log2(int p) { return p == 0 ? 8 : 7; }

// Exact-accumulation schedule shared by every role.  Items are
// (level L, pair p, k-block kb) in level-major order; a group is a run of
// items of one level whose summed |product| bound stays <= 2^24.
struct Sched {
  int S, nkb;
  // iteration state
  int L, p, kb;
  int group;     // group index of the current item
  int64_t used;  // bound used in the current group (log-domain sums as integers)
  bool first_in_group;
  __host__ __device__ void begin(int S_, int nkb_) {
    S = S_;
    nkb = nkb_;
    L = 0;
    p = 0;
    kb = 0;
    group = 0;
    used = 0;
    first_in_group = true;
    used = cost();
  }
  // Jump to the first item of level L0 (a group always starts there).
  __host__ __device__ void seek(int L0) {
    L = L0;
    p = 0;
    kb = 0;
    first_in_group = true;
    used = L < S ? cost() : 0;
  }
  __host__ __device__ int q() const { return L - p; }
  __host__ __device__ int64_t cost() const {
    return (int64_t)BK << (digit_log2(p) + digit_log2(L - p));
  }
  __host__ __device__ bool valid() const { return L < S; }
  // Advance; reports whether the item just finished closed its group.
  __host__ __device__ bool advance() {
    int nL = L, np = p, nkb2 = kb + 1;
    if (nkb2 == nkb) {
      nkb2 = 0;
      np = p + 1;
      if (np > L) {
        np = 0;
        nL = L + 1;
      }
    }
    bool closes;
    if (nL >= S) {
      closes = true;
    } else if (nL != L) {
      closes = true;
    } else {
      int64_t c = (int64_t)BK << (digit_log2(np) + digit_log2(nL - np));
      closes = used + c > ((int64_t)1 << 24);
    }
    L = nL;
    p = np;
    kb = nkb2;
    if (closes) {
      group++;
      used = 0;
      first_in_group = true;
    } else {
      first_in_group = false;
    }
    if (L < S) used += cost();
    return closes;
  }
};

struct GemmArgs {
  int64_t M, N, K;
  int Mpad, Npad, Kpad, nkb, S, F, tiles_n;
  const int* eA;
  const int* eB;
  const int64_t* offCm;
  const int64_t* offCn;
  double* C;
  double alpha, beta;
  long long* acc;    // one private int64 tile accumulator per CTA
  long long* tacc;   // shared accumulators of tiles split between CTAs (one per CTA)
  int* cnt;          // contributions received by each shared accumulator
  int64_t W;         // tail work units: T * (tiles mod G)
  int G;             // CTAs in the grid
  int q;             // whole tiles per CTA before the tail
  uint64_t wait_ns;  // limit of every mbarrier wait (%globaltimer ns)
  int* err;
};

// Work partition over G persistent CTAs.  With q, r = divmod(tiles, G), CTA
// g first computes the whole tiles g, g + G, ..., g + (q - 1) G (in waves, so
// the tiles in flight at any time are neighbours and share operand panels in
// L2), then its share of the last r tiles: their units (tile ct, level L) in
// tile-major order, unit (ct, L) costing L + 1 (its k-blocks number
// (L + 1) * nkb) and starting at offset T * (ct - q G) + L (L + 1) / 2,
// T = S (S + 1) / 2.  CTA g owns the tail units whose start offset lies in
// [lo(g), lo(g + 1)), lo(g) = floor(g W / G), W = T r, so a tail tile may be
// shared by consecutive CTAs, always at a level boundary.  With G equal to
// the number of tiles every CTA computes exactly one whole tile.
struct Part {
  int64_t W;  // tail units
  int G, S, T, q;
  __host__ __device__ int base() const { return q * G; }  // first tail tile
  __host__ __device__ int64_t lo(int g) const { return (int64_t)g * W / G; }
  // first tail unit whose start offset is >= x
  __host__ __device__ void unit_at(int64_t x, int& ct, int& L) const {
    ct = (int)(x / T);
    const int r = (int)(x - (int64_t)T * ct);
    ct += base();
    L = 0;
    while (L < S && L * (L + 1) / 2 < r) ++L;
    if (L == S) {
      ++ct;
      L = 0;
    }
  }
  // CTA owning the tail unit that starts at offset s: the largest g with lo(g) <= s
  __host__ __device__ int owner(int64_t s) const {
    const int64_t g = ((s + 1) * G + W - 1) / W - 1;
    return g < 0 ? 0 : (g >= G ? G - 1 : (int)g);
  }
  // Segment idx of CTA g (tile ct, levels [L0, Le)); (tb, lb) and (te, le)
  // are unit_at(lo(g)) and unit_at(lo(g + 1)).  False past the last one.
  __host__ __device__ bool seg(int g, int idx, int tb, int lb, int te, int le, int& ct, int& L0, int& Le) const {
    if (idx < q) {
      ct = g + idx * G;
      L0 = 0;
      Le = S;
      return true;
    }
    const int j = idx - q;
    ct = tb + j;
    L0 = j == 0 ? lb : 0;
    if (!(ct < te || (ct == te && L0 < le))) return false;
    Le = ct == te ? le : S;
    return true;
  }
  // CTAs contributing to tile ct (the distinct owners of its units)
  __host__ __device__ int contributors(int ct, int& first) const {
    if (ct < base()) {
      first = 0;
      return 1;
    }
    const int64_t s0 = (int64_t)T * (ct - base());
    first = owner(s0);
    int n = 1;
    for (int L = 1, prev = first; L < S; ++L) {
      const int o = owner(s0 + L * (L + 1) / 2);
      n += o != prev;
      prev = o;
    }
    return n;
  }
};

// v * 2^exp2 rounded to nearest even, built with integer instructions.
__device__ __forceinline__ double i64_to_double_scaled(long long v, int exp2) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  unsigned long long u = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const int top = 63 - __clzll((long long)u);
  unsigned long long mant;
  int e2 = top + exp2;
  if (top <= 52) {
    mant = u << (52 - top);
  } else {
    const int sh = top - 52;
    const unsigned long long rem = u & ((1ull << sh) - 1);
    const unsigned long long half = 1ull << (sh - 1);
    mant = u >> sh;
    if (rem > half || (rem == half && (mant & 1ull))) {
      mant++;
      if (mant >> 53) {
        mant >>= 1;
        e2++;
      }
    }
  }
  const int be = e2 + 1023;
  if (be <= 0) return __longlong_as_double((long long)sgn);
  if (be >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
  return __longlong_as_double(
      (long long)(sgn | ((unsigned long long)be << 52) | (mant & ((1ull << 52) - 1))));
}

// Tile variants: BN = 256 keeps the int64 accumulators in global memory
// (two 256-column FP32 TMEM buffers fill the TMEM); BN = 128 keeps them in
// TMEM columns 256..511 (low / high words), so a drain never leaves the SM,
// and runs a 6-stage operand ring.
template <int BN>
struct Smem {
  static constexpr bool TACC = BN == 128;
  static constexpr int NSTAGE = TACC ? 6 : STAGES;
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int TOTAL = 1024 /*align slack*/ + NSTAGE * STAGE_BYTES + 256;
};

// 16 values of a CTA's private int64 accumulator (columns c0 .. c0 + 15 of
// this thread's row): TMEM columns 256 + c (low words) and 384 + c (high
// words) when TACC, else global memory.  Warp-collective when TACC.
template <bool TACC>
__device__ __forceinline__ void load_acc16(uint32_t lane_base, const long long* acc, int c0, int row,
                                           long long (&v)[16]) {
  if (TACC) {
    uint32_t lo[16], hi[16];
    const uint32_t tlo = lane_base + 256u + (uint32_t)c0;
    tc_ld_32x32b_x16_nowait(tlo, lo);
    tc_ld_32x32b_x16_nowait(tlo + 128u, hi);
    tc_wait_ld();
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = (long long)(((unsigned long long)hi[j] << 32) | lo[j]);
  } else {
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = acc[(size_t)(c0 + j) * BM + row];
  }
}

// A CTA walks its units (Part) tile segment by tile segment; the pipeline
// state (stage ring, TMEM buffers) carries over from one segment to the next.
// A tile owned by one CTA is converted to FP64 straight from the CTA's
// private accumulator.  A shared tile: every contributor adds its private
// accumulator into the tile's shared one with 64-bit integer atomics (exact,
// so the result does not depend on their order), then counts itself in; the
// last one to arrive converts.  Nobody waits for anybody else.
template <int BN>
__global__ void __launch_bounds__(NUM_THREADS, 1)
k_split_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
             GemmArgs args) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int NST = Smem<BN>::NSTAGE;
  constexpr bool TACC = Smem<BN>::TACC;
  uint8_t* stage_mem = base;
  uint64_t* bars = (uint64_t*)(base + NST * Smem<BN>::STAGE_BYTES);
  uint64_t* full = bars;                 // [NST]
  uint64_t* empty = bars + NST;          // [NST]
  uint64_t* acc_full = bars + 2 * NST;      // [2]
  uint64_t* acc_empty = bars + 2 * NST + 2; // [2]
  uint64_t* done_bar = bars + 2 * NST + 4;  // [1]
  volatile int* abort_flag = (volatile int*)(bars + 2 * NST + 5);
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * NST + 6);
  volatile int* decision = (volatile int*)(bars + 2 * NST + 7);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gcl = (int)blockIdx.x;  // this CTA's share of the work
  Part part;
  part.W = args.W;
  part.G = args.G;
  part.S = args.S;
  part.T = args.S * (args.S + 1) / 2;
  part.q = args.q;
  int tb, lb, te, le;  // tail units [ (tb, lb), (te, le) )
  part.unit_at(part.lo(gcl), tb, lb);
  part.unit_at(part.lo(gcl + 1), te, le);
  constexpr uint32_t TMEM_COLS = TACC ? 512 : 2 * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], NUM_EPI_WARPS);
    }
    mbar_init(done_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      int ct, L0, Le;
      for (int si = 0; ok && part.seg(gcl, si, tb, lb, te, le, ct, L0, Le); ++si) {
        const int m_grp = ct / args.tiles_n;
        const int n_tile = ct - m_grp * args.tiles_n;
        const int m0 = m_grp * BM, n0 = n_tile * BN;
        Sched sc;
        sc.begin(args.S, args.nkb);
        sc.seek(L0);
        while (sc.valid() && sc.L < Le) {
          if (*abort_flag) {
            ok = false;
            break;
          }
          const int s = it % NST;
          if (it >= NST) {
            if (!mbar_wait(&empty[s], ((it / NST) - 1) & 1, args.err, abort_flag, args.wait_ns)) {
              ok = false;
              break;
            }
          }
          uint8_t* sa = stage_mem + s * Smem<BN>::STAGE_BYTES;
          uint8_t* sb = sa + Smem<BN>::A_BYTES;
          mbar_arrive_expect_tx(&full[s], Smem<BN>::STAGE_BYTES);
          tma_load_2d(sa, &mapA, sc.kb * BK, sc.p * args.Mpad + m0, &full[s]);
          tma_load_2d(sb, &mapB, sc.kb * BK, sc.q() * args.Npad + n0, &full[s]);
          sc.advance();
          ++it;
        }
      }
      // make sure no copy is still landing in shared memory when we leave
      for (int j = std::max(0, it - NST); j < it; ++j) mbar_drain(&full[j % NST], (j / NST) & 1, args.wait_ns);
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(BM, BN);
      int it = 0, lg = 0;  // items and groups issued by this CTA
      bool ok = true;
      int ct, L0, Le;
      for (int si = 0; ok && part.seg(gcl, si, tb, lb, te, le, ct, L0, Le); ++si) {
        Sched sc;
        sc.begin(args.S, args.nkb);
        sc.seek(L0);
        while (sc.valid() && sc.L < Le) {
          const int b = lg & 1;
          const bool first = sc.first_in_group;
          if (first && lg >= 2) {
            ok = mbar_wait(&acc_empty[b], ((lg >> 1) - 1) & 1, args.err, abort_flag, args.wait_ns);
            tc_fence_after();
            if (!ok) break;
          }
          const int s = it % NST;
          ok = mbar_wait(&full[s], (it / NST) & 1, args.err, abort_flag, args.wait_ns);
          if (!ok) break;
          tc_fence_after();
          const uint32_t sa = smem_u32(stage_mem + s * Smem<BN>::STAGE_BYTES);
          const uint32_t sb = sa + Smem<BN>::A_BYTES;
          const uint64_t ad = sdesc_sw128(sa), bd = sdesc_sw128(sb);
          const uint32_t tmem_d = tmem_base + (uint32_t)(b * BN);
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            const uint32_t accum = (first && kk == 0) ? 0u : 1u;
            tc_mma_bf16(tmem_d, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), idesc, accum);
          }
          tc_commit(&empty[s]);
          if (sc.advance()) {
            tc_commit(&acc_full[b]);
            ++lg;
          }
          ++it;
        }
      }
      // all MMAs issued by this thread complete before TMEM is released
      tc_commit(done_bar);
      mbar_drain(done_bar, 0, args.wait_ns);
    }
  } else {
    // ------------------------------------------------------ drain/epilogue
    // Each thread owns one row and NCOL columns.  A group's FP32 values are
    // exact integers below 2^24 in magnitude; the groups of one level are
    // summed in int32 registers (exact for up to 127 groups) and only a level
    // end (or the 127th group) touches the int64 fixed-point accumulator.  The
    // TMEM buffer goes back to the MMA issuer as soon as it has been read,
    // except at a level end of the global-accumulator variant: there the int32
    // sums are parked in the drained buffer, which frees the registers for
    // FLUSH_BATCH accumulator loads in flight at a time, and the buffer is
    // handed back after the accumulator update.
    constexpr int NCOL = BN / 2;
    constexpr int NCH = NCOL / 32;
    constexpr int FLUSH_BATCH = 32;
    const int quarter = warp & 3;
    const int col_lo = ((warp - 2) / 4) * NCOL;
    const int row = quarter * 32 + lane;
    long long* acc = args.acc + (size_t)blockIdx.x * BN * BM;  // private: global (BN 256) or TMEM (BN 128)
    const uint32_t lane_base = tmem_base + ((uint32_t)(quarter * 32) << 16);
    int lg = 0;  // groups drained by this CTA
    int ct, L0, Le;
    for (int si = 0; part.seg(gcl, si, tb, lb, te, le, ct, L0, Le); ++si) {
      int32_t sum[NCOL];
#pragma unroll
      for (int j = 0; j < NCOL; ++j) sum[j] = 0;
      int nsum = 0;
      bool have_acc = false, complete = false;
      Sched sc;
      sc.begin(args.S, args.nkb);
      sc.seek(L0);
      while (sc.valid() && sc.L < Le) {
        const int L = sc.L;
        while (!sc.advance()) {
        }
        const bool seg_last = !sc.valid() || sc.L >= Le;
        const bool flush = seg_last || sc.L != L || nsum + 1 == 127;
        const int b = lg & 1;
        // every lane polls; the outcome is made warp-uniform because the TMEM
        // loads below are .sync.aligned
        const bool ok_lane = mbar_wait(&acc_full[b], (lg >> 1) & 1, args.err, abort_flag, args.wait_ns);
        if (!__all_sync(0xffffffffu, ok_lane)) break;
        tc_fence_after();
        const uint32_t tbuf = lane_base + (uint32_t)(b * BN + col_lo);
#pragma unroll
        for (int c = 0; c < NCOL / 16; ++c) {
          uint32_t r[16];
          tc_ld_32x32b_x16(tbuf + (uint32_t)(16 * c), r);
#pragma unroll
          for (int j = 0; j < 16; ++j) sum[16 * c + j] += __float2int_rn(__uint_as_float(r[j]));
        }
        ++lg;
        ++nsum;
        const int sh = args.F - 8 * L;
        if (!TACC && flush) {
          // park the level's sums in the drained buffer, then update the
          // global accumulator FLUSH_BATCH columns at a time
#pragma unroll
          for (int c = 0; c < NCOL / 16; ++c) {
            uint32_t r[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) r[j] = (uint32_t)sum[16 * c + j];
            tc_st_32x32b_x16(tbuf + (uint32_t)(16 * c), r);
          }
          tc_wait_st();
#pragma unroll
          for (int j = 0; j < NCOL; ++j) sum[j] = 0;
          long long* ap = acc + (size_t)col_lo * BM + row;
#pragma unroll 1
          for (int c0 = 0; c0 < NCOL; c0 += FLUSH_BATCH) {
            long long old[FLUSH_BATCH];
#pragma unroll
            for (int j = 0; j < FLUSH_BATCH; ++j) old[j] = have_acc ? ap[(size_t)(c0 + j) * BM] : 0ll;
#pragma unroll
            for (int h = 0; h < FLUSH_BATCH / 16; ++h) {
              uint32_t r[16];
              tc_ld_32x32b_x16(tbuf + (uint32_t)(c0 + 16 * h), r);
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                long long t = (long long)(int32_t)r[j];
                t = sh >= 0 ? (long long)((unsigned long long)t << sh) : (t >> (-sh));
                ap[(size_t)(c0 + 16 * h + j) * BM] = old[16 * h + j] + t;
              }
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[b]);
        if (TACC && flush) {
#pragma unroll
          for (int c = 0; c < NCH; ++c) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int c0 = col_lo + 32 * c + 16 * h;
              // int64 accumulator in TMEM: low words in columns 256 + c, high words in 384 + c
              const uint32_t tlo = lane_base + 256u + (uint32_t)c0, thi = tlo + 128u;
              uint32_t lo[16], hi[16];
              if (have_acc) {
                tc_ld_32x32b_x16_nowait(tlo, lo);
                tc_ld_32x32b_x16_nowait(thi, hi);
                tc_wait_ld();
              } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) lo[j] = hi[j] = 0u;
              }
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                long long t = (long long)sum[32 * c + 16 * h + j];
                t = sh >= 0 ? (long long)((unsigned long long)t << sh) : (t >> (-sh));
                const unsigned long long u = (((unsigned long long)hi[j] << 32) | lo[j]) + (unsigned long long)t;
                lo[j] = (uint32_t)(u & 0xFFFFFFFFull);
                hi[j] = (uint32_t)(u >> 32);
              }
              tc_st_32x32b_x16(tlo, lo);
              tc_st_32x32b_x16(thi, hi);
            }
          }
          tc_wait_st();
#pragma unroll
          for (int j = 0; j < NCOL; ++j) sum[j] = 0;
        }
        if (flush) {
          nsum = 0;
          have_acc = true;
          complete = seg_last;
        }
        if (__any_sync(0xffffffffu, *abort_flag != 0)) break;
      }
      // Segment end.  Every epilogue warp arrives here (a warp that stopped on
      // an abort included), so the decision below is the same for all of them.
      int first_owner;
      const int contributors = part.contributors(ct, first_owner);
      const bool shared_tile = contributors > 1;
      const int slot = first_owner;
      long long* tile_acc = args.tacc + (size_t)slot * BN * BM;
      if (shared_tile && complete) {
#pragma unroll 1
        for (int c0 = col_lo; c0 < col_lo + NCOL; c0 += 16) {
          long long v[16];
          load_acc16<TACC>(lane_base, acc, c0, row, v);
#pragma unroll
          for (int j = 0; j < 16; ++j)
            atomicAdd((unsigned long long*)(tile_acc + (size_t)(c0 + j) * BM + row), (unsigned long long)v[j]);
        }
        __threadfence();
      }
      asm volatile("bar.sync 1, %0;" ::"n"(32 * NUM_EPI_WARPS) : "memory");
      if (warp == 2 && lane == 0) {
        int d;
        if (*abort_flag || !complete) d = 2;
        else if (!shared_tile) d = 1;
        else d = atomicAdd(&args.cnt[slot], 1) == contributors - 1 ? 1 : 0;
        *decision = d;
      }
      asm volatile("bar.sync 1, %0;" ::"n"(32 * NUM_EPI_WARPS) : "memory");
      const int d = *decision;
      if (d == 2) break;
      if (d == 1) {
        // the int64 accumulator is complete: convert to FP64 with integer
        // instructions and scatter C through the plan's offset tables
        if (shared_tile) __threadfence();
        const int m_grp = ct / args.tiles_n;
        const int n0 = (ct - m_grp * args.tiles_n) * BN;
        const int64_t m = (int64_t)m_grp * BM + row;
        const int64_t cm = m < args.M ? args.offCm[m] : 0;
        const int em = m < args.M ? args.eA[m] - 1022 : 0;
        // FLUSH_BATCH accumulator values in flight at a time
#pragma unroll 1
        for (int c0 = col_lo; c0 < col_lo + NCOL; c0 += FLUSH_BATCH) {
          long long v[FLUSH_BATCH];
          if (shared_tile) {
#pragma unroll
            for (int j = 0; j < FLUSH_BATCH; ++j) v[j] = __ldcg(tile_acc + (size_t)(c0 + j) * BM + row);
          } else if (TACC) {
#pragma unroll
            for (int h = 0; h < FLUSH_BATCH / 16; ++h) {
              long long w[16];
              load_acc16<TACC>(lane_base, acc, c0 + 16 * h, row, w);
#pragma unroll
              for (int j = 0; j < 16; ++j) v[16 * h + j] = w[j];
            }
          } else {
#pragma unroll
            for (int j = 0; j < FLUSH_BATCH; ++j) v[j] = acc[(size_t)(c0 + j) * BM + row];
          }
          if (m < args.M) {
            // the column exponents and offsets are read-only for the whole
            // launch: read-only loads, issued 8 at a time ahead of the stores
            // (plain loads would be ordered after every store to C)
#pragma unroll
            for (int h = 0; h < FLUSH_BATCH / 8; ++h) {
              int eb[8];
              long long ocn[8];
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const int64_t n = (int64_t)n0 + c0 + 8 * h + j;
                const int64_t nc = n < args.N ? n : args.N - 1;
                eb[j] = __ldg(args.eB + nc);
                ocn[j] = __ldg((const long long*)args.offCn + nc);
              }
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const int64_t n = (int64_t)n0 + c0 + 8 * h + j;
                if (n >= args.N) continue;
                double x = i64_to_double_scaled(v[8 * h + j], em + eb[j] - 1022 - 16 - args.F);
                if (args.alpha != 1.0) x *= args.alpha;
                double* cp = args.C + cm + ocn[j];
                if (args.beta != 0.0) x = fma(args.beta, *cp, x);
                *cp = x;
              }
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TMEM_COLS));
  }
}

// Self-test of the mbarrier timeout path shared by every role of
// k_split_gemm: one thread waits, through mbar_wait, for phase 0 of a
// barrier that expects one arrival nobody makes; the wait runs out after the
// limit, records ITG_ERR_TIMEOUT in *err and raises the abort flag.
__global__ void k_mbar_selftest(int* err, uint64_t wait_ns) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const bool ok = mbar_wait(&bar, 0, err, (volatile int*)&abort_flag, wait_ns);
    if (ok) atomicExch(err, ITG_OK);
  }
  __syncthreads();
}

// ----------------------------------------------------------- slicing
// Exponent field (11 bits) of max_k |X[r,k]| for every row r < R.
__global__ void k_row_expfield(const double* __restrict__ X, const int64_t* __restrict__ offR,
                               const int64_t* __restrict__ offK, int64_t R, int64_t K,
                               int* __restrict__ efield) {
  {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); r < R; r += warps) {
      const double* x = X + offR[r];
      unsigned long long mx = 0;
      for (int64_t k = lane; k < K; k += 32) {
        unsigned long long b = (unsigned long long)__double_as_longlong(x[offK[k]]) & 0x7FFFFFFFFFFFFFFFull;
        mx = b > mx ? b : mx;
      }
      for (int o = 16; o > 0; o >>= 1) {
        unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = y > mx ? y : mx;
      }
      if (lane == 0) efield[r] = (int)((mx >> 52) & 0x7FF);
    }
  }
}

// Rows contiguous in memory: a 2-D grid, threads along rows, blockIdx.y over
// K chunks of 64; partial maxima meet through atomicMax on the exponent field
// (integer max, order independent).  efield must start at 0.
__global__ void k_row_expfield_mmajor(const double* __restrict__ X, const int64_t* __restrict__ offR,
                                      const int64_t* __restrict__ offK, int64_t R, int64_t K,
                                      int* __restrict__ efield) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int64_t k0 = (int64_t)blockIdx.y * 64, k1 = k0 + 64 < K ? k0 + 64 : K;
  const double* x = X + offR[r];
  unsigned long long mx = 0;
  for (int64_t k = k0; k < k1; ++k) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x[offK[k]]) & 0x7FFFFFFFFFFFFFFFull;
    mx = b > mx ? b : mx;
  }
  const int e = (int)((mx >> 52) & 0x7FF);
  if (e) atomicMax(&efield[r], e);
}

// Balanced base-2^8 digits of |X[r,k]| * 2^-e_r rounded to 48 fractional bits
// (S = 6 digits), and the sign of X[r,k]; the digits of X are the digits of
// |X| negated.  Y = |X| 2^(48 - e_r) (at most 2^48) splits into 24 + 24 bits
// whose bytes are the unbalanced digits u_p; one carry pass from the least
// significant digit makes them balanced (v = u_p + carry; v >= 128 -> digit
// v - 256, carry 1), so |d_0| <= 256 and |d_p| <= 128 for p >= 1, all exact
// in bf16.
__device__ __forceinline__ void make_digits_abs(double x, int efield_r, int (&d)[S_SLICES], bool& neg) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  neg = (bits >> 63) != 0;
  const int E = (int)((bits >> 52) & 0x7FF);
  unsigned long long M = bits & ((1ull << 52) - 1);
  if (E) M |= 1ull << 52;
  const int Ee = E ? E : 1;
  const int sh = Ee - 1075 - (efield_r - 1022) + 48;
  unsigned long long Y;
  if (M == 0 || E == 2047) {
    Y = 0;
  } else if (sh >= 0) {
    Y = M << sh;
  } else if (sh <= -60) {
    Y = 0;
  } else {
    Y = (M >> (-sh)) + ((M >> (-sh - 1)) & 1ull);
  }
  const uint32_t lo = (uint32_t)Y & 0x00FFFFFFu, hi = (uint32_t)(Y >> 24);
  const uint32_t u[6] = {hi >> 16, (hi >> 8) & 255u, hi & 255u, lo >> 16, (lo >> 8) & 255u, lo & 255u};
  int c = 0;
#pragma unroll
  for (int p = 5; p >= 1; --p) {
    const int v = (int)u[p] + c;
    c = v >= 128;
    d[p] = c ? v - 256 : v;
  }
  d[0] = (int)u[0] + c;
}

// ------------------------------------------------- H_eff middle step
// T3[r, j] = sum_c T1[r, c] Weff[c, j] for R rows r, c < nc <= 32, j < nj <= 32
// (the merged-MPO step of the two-site H_eff chain: K = nc = wL d^2, N = nj =
// d^2 wR), by the same exact digit products as k_split_gemm.  Persistent CTAs
// of 128 threads walk blocks of 128 rows.  Per block every thread loads its
// row of T1 (coalesced across the CTA per c), forms the row exponent and the
// 6 balanced digits of each element, and writes them K-major with the
// 128-byte swizzle into shared memory, two slices per 128-byte row (slice p
// at k offset 32 (p % 2) of tile p / 2); Weff's column digits are written the
// same way once per CTA.  One thread issues the 21 digit products (one or two
// K = 16 steps each) into six TMEM level accumulators of NJP columns; one
// group per level suffices because sum_{p+q=L} nc |a_p| |b_q| <= 32 (2 * 2^15
// + 4 * 2^14) = 2^22 keeps every FP32 partial sum an exact integer.  Each thread then reads
// its row's level sums, forms the int64 fixed-point value and converts it to
// FP64 with integer instructions: the same bits as k_split_gemm computes for
// this product (same digits, same fixed point, same rounding).
constexpr int MID_ROWS = 128;
constexpr int MID_THREADS = 128;
constexpr int MID_KSLICE = 32;  // padded K per slice (nc <= 32)
constexpr int MID_A_TILE = MID_ROWS * 128;     // bytes: 128 rows x 128 B (two slices)
constexpr int MID_NTILE = (S_SLICES + 1) / 2;  // 3 tiles hold the 6 slices

template <int NJP>
struct MidSmem {
  static constexpr int B_TILE = NJP * 128;
  static constexpr int A_OFF = 0;
  static constexpr int B_OFF = MID_NTILE * MID_A_TILE;
  static constexpr int TOTAL = 1024 /*align slack*/ + B_OFF + MID_NTILE * B_TILE + 256;
  static constexpr uint32_t TMEM_COLS = (S_SLICES * NJP <= 128) ? 128u : 256u;
};

// byte offset of element (row i, k) of a K-major 128-byte-swizzled tile
__device__ __forceinline__ uint32_t sw128_off(int i, int k) {
  return (uint32_t)(i * 128 + ((((k >> 3) ^ (i & 7))) << 4) + ((k & 7) << 1));
}

// bf16 bits of two small integers (|d| <= 2^8, exact in bf16) packed low | high:
// float(d) = (0x4B400000 + d as float bits) - 1.5 * 2^23 exactly, and the bf16
// of a float with at most 8 significant bits is its upper half.
__device__ __forceinline__ uint32_t pack_bf16x2(int lo, int hi) {
  const float fl = __int_as_float(0x4B400000 + lo) - 12582912.0f;
  const float fh = __int_as_float(0x4B400000 + hi) - 12582912.0f;
  return __byte_perm((uint32_t)__float_as_int(fl), (uint32_t)__float_as_int(fh), 0x7632);
}

// Writes the digits of 8 consecutive k (c0 .. c0 + 7 of slice p) of row i;
// sgn[q] holds the sign bits (0x8000 per half) of elements 2q, 2q + 1.
__device__ __forceinline__ void store_digit_chunk(uint8_t* tile, int i, int p, int c0, const int (&dg)[8],
                                                  const uint32_t (&sgn)[4]) {
  const int k = (p & 1) * MID_KSLICE + c0;
  uint4 v;
  v.x = pack_bf16x2(dg[0], dg[1]) ^ sgn[0];
  v.y = pack_bf16x2(dg[2], dg[3]) ^ sgn[1];
  v.z = pack_bf16x2(dg[4], dg[5]) ^ sgn[2];
  v.w = pack_bf16x2(dg[6], dg[7]) ^ sgn[3];
  *(uint4*)(tile + sw128_off(i, k)) = v;
}

// The 6 digits of 8 elements (x[c0 .. c0 + 7], row exponent field ef) into the
// 7 slices' chunks of row i.  A negative element's digits are the negated
// digits of its magnitude (bf16 sign bit; a zero digit may so become -0,
// which changes no product or sum).
__device__ __forceinline__ void digits8(uint8_t* tiles, int tile_bytes, int i, int c0, const double* x, int ef) {
  constexpr int S = S_SLICES;
  int dg[S][8];
  uint32_t sgn[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    int d[S];
    bool neg;
    make_digits_abs(x[e], ef, d, neg);
    if (neg) sgn[e >> 1] |= (e & 1) ? 0x80000000u : 0x00008000u;
#pragma unroll
    for (int p = 0; p < S; ++p) dg[p][e] = d[p];
  }
#pragma unroll
  for (int p = 0; p < S; ++p) store_digit_chunk(tiles + (p >> 1) * tile_bytes, i, p, c0, dg[p], sgn);
}

template <int NJP>
__global__ void __launch_bounds__(MID_THREADS)
k_heff_mid_split(const double* __restrict__ T1, const double* __restrict__ Weff, double* __restrict__ T3,
                 int64_t R, int nc, int nj, uint64_t wait_ns, int* err) {
  constexpr int S = S_SLICES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = base + MidSmem<NJP>::A_OFF;
  uint8_t* sB = base + MidSmem<NJP>::B_OFF;
  uint8_t* tail = sB + MID_NTILE * MidSmem<NJP>::B_TILE;
  uint64_t* done = (uint64_t*)tail;
  uint32_t* tmem_slot = (uint32_t*)(tail + 8);
  int* fB = (int*)(tail + 16);  // [NJP] column exponent fields of Weff
  volatile int* abort_flag = (volatile int*)(tail + 16 + 4 * 32);
  const int t = threadIdx.x, warp = t >> 5;
  const int ngrp = (nc + 7) >> 3;  // 8-element groups of c holding data

  if (t == 0) {
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(MidSmem<NJP>::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  // A chunks no block writes (k groups past nc): zero once
  {
    const int zero[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t nosign[4] = {0u, 0u, 0u, 0u};
    for (int cg = ngrp; cg < MID_KSLICE / 8; ++cg)
#pragma unroll
      for (int p = 0; p < S; ++p) store_digit_chunk(sA + (p >> 1) * MID_A_TILE, t, p, cg * 8, zero, nosign);
  }
  // B: digits of Weff's columns (row j of the B tiles, k = c), once per CTA
  {
    const int j = t >> 2, cg = t & 3;  // NJP * 4 <= 128 threads
    if (j < NJP) {
      int ef = 0;
      if (j < nj) {
        unsigned long long mx = 0;
        for (int c = 0; c < nc; ++c) {
          const unsigned long long b = (unsigned long long)__double_as_longlong(Weff[c + (int64_t)nc * j]) &
                                       0x7FFFFFFFFFFFFFFFull;
          mx = b > mx ? b : mx;
        }
        ef = (int)((mx >> 52) & 0x7FF);
      }
      if (cg == 0) fB[j] = ef;
      double w[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int c = cg * 8 + e;
        w[e] = (j < nj && c < nc) ? Weff[c + (int64_t)nc * j] : 0.0;
      }
      digits8(sB, MidSmem<NJP>::B_TILE, j, cg * 8, w, ef);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const uint32_t lane_base = tmem_base + ((uint32_t)(warp * 32) << 16);
  const int ksteps = nc > 16 ? 2 : 1;
  int lk = 0;
  while ((1 << lk) < nc) ++lk;
  const int F = 62 - 17 - lk;
  const int64_t nblk = (R + MID_ROWS - 1) / MID_ROWS;
  bool ok = true;
  uint32_t phase = 0;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x, phase ^= 1u) {
    const int64_t r = blk * MID_ROWS + t;
    // ---- A: this thread's row of T1 (all loads first)
    double x[MID_KSLICE];
#pragma unroll
    for (int c = 0; c < MID_KSLICE; ++c) x[c] = (c < nc && r < R) ? __ldcs(T1 + r + R * c) : 0.0;
    unsigned long long mx = 0;
#pragma unroll
    for (int c = 0; c < MID_KSLICE; ++c) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(x[c]) & 0x7FFFFFFFFFFFFFFFull;
      mx = b > mx ? b : mx;
    }
    const int eA = (int)((mx >> 52) & 0x7FF);
#pragma unroll
    for (int cg = 0; cg < MID_KSLICE / 8; ++cg)
      if (cg < ngrp) digits8(sA, MID_A_TILE, t, cg * 8, x + cg * 8, eA);
    // generic-proxy smem writes -> visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (t == 0) {
      constexpr uint32_t idesc = idesc_bf16(MID_ROWS, NJP);
      for (int L = 0; L < S; ++L) {
        for (int p = 0; p <= L; ++p) {
          const int q = L - p;
          const uint64_t ad = sdesc_sw128(smem_u32(sA + (p >> 1) * MID_A_TILE));
          const uint64_t bd = sdesc_sw128(smem_u32(sB + (q >> 1) * MidSmem<NJP>::B_TILE));
          for (int s = 0; s < ksteps; ++s) {
            const uint64_t ka = (uint64_t)(2 * (2 * (p & 1) + s)), kb = (uint64_t)(2 * (2 * (q & 1) + s));
            tc_mma_bf16(tmem_base + (uint32_t)(L * NJP), ad + ka, bd + kb, idesc, (p > 0 || s > 0) ? 1u : 0u);
          }
        }
      }
      tc_commit(done);
    }
    // every thread waits (bounded) for the products, then drains its row
    ok = mbar_wait(done, phase, err, abort_flag, wait_ns);
    tc_fence_after();
    // CTA-uniform decision: every thread reaches this barrier whatever its wait returned
    if (__syncthreads_or(!ok)) {
      ok = false;
      break;
    }
    // int64 fixed point: acc = sum_L s_L 2^(F - 8L) (F >= 40 here, so every
    // shift is a left shift), by Horner over the levels and one final shift
    long long acc[NJP];
#pragma unroll
    for (int L = 0; L < S; ++L) {
#pragma unroll
      for (int h = 0; h < NJP / 16; ++h) {
        if (16 * h < nj) {
          uint32_t v[16];
          tc_ld_32x32b_x16(lane_base + (uint32_t)(L * NJP + 16 * h), v);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            // exact integer of magnitude <= 2^22: float -> int by the 1.5 * 2^23 shift
            const long long tv = (long long)(__float_as_int(__uint_as_float(v[j]) + 12582912.0f) - 0x4B400000);
            acc[16 * h + j] = L == 0 ? tv : (long long)((unsigned long long)acc[16 * h + j] << 8) + tv;
          }
        }
      }
    }
    if (r < R) {
      const int em = eA - 1022;
#pragma unroll
      for (int j = 0; j < NJP; ++j)
        if (j < nj)
          __stcs(T3 + r + R * j, i64_to_double_scaled((long long)((unsigned long long)acc[j] << (F - 40)),
                                                      em + fB[j] - 1022 - 16 - F));
    }
    // the TMEM accumulators and the A tiles are reused by the next block
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) {
    // after a timeout the products may still be in flight: wait (bounded) before freeing TMEM
    if (!ok) mbar_drain(done, phase, wait_ns);
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(MidSmem<NJP>::TMEM_COLS));
  }
}

// out[p][r][k] (bf16, k contiguous, padded to Rpad x Kpad) for the gathered X.
template <bool KMAJ, int S>
__global__ void __launch_bounds__(256)
k_make_slices(const double* __restrict__ X, const int64_t* __restrict__ offR,
              const int64_t* __restrict__ offK, int64_t R, int64_t K, int64_t Rpad, int64_t Kpad,
              const int* __restrict__ efield, __nv_bfloat16* __restrict__ out) {
  __shared__ double tile[32][65];
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 64;
  const int t = threadIdx.x;
  if (KMAJ) {
    const int kk = t & 63;
    const int64_t k = k0 + kk;
    const int64_t ok = (k < K) ? offK[k] : 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int rr = (t >> 6) + 4 * i;
      const int64_t r = r0 + rr;
      tile[rr][kk] = (r < R && k < K) ? X[offR[r] + ok] : 0.0;
    }
  } else {
    const int rr = t & 31;
    const int64_t r = r0 + rr;
    const int64_t orr = (r < R) ? offR[r] : 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int kk = (t >> 5) + 8 * i;
      const int64_t k = k0 + kk;
      tile[rr][kk] = (r < R && k < K) ? X[orr + offK[k]] : 0.0;
    }
  }
  __syncthreads();
  // each thread: 8 consecutive k of one row -> one 16-byte store per slice
  static_assert(S == S_SLICES, "digit routine is written for 6 slices");
  const int rr = t >> 3, kc = t & 7;
  const int64_t r = r0 + rr;
  const int ef = (r < R) ? efield[r] : 0;
  int dg[S][8];
  uint32_t sgn[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    int d[S];
    bool neg;
    make_digits_abs(tile[rr][kc * 8 + e], ef, d, neg);
    if (neg) sgn[e >> 1] |= (e & 1) ? 0x80000000u : 0x00008000u;
#pragma unroll
    for (int p = 0; p < S; ++p) dg[p][e] = d[p];
  }
  const size_t plane = (size_t)Rpad * Kpad;
  const size_t o = (size_t)r * Kpad + k0 + kc * 8;
#pragma unroll
  for (int p = 0; p < S; ++p) {
    uint4 v;
    v.x = pack_bf16x2(dg[p][0], dg[p][1]) ^ sgn[0];
    v.y = pack_bf16x2(dg[p][2], dg[p][3]) ^ sgn[1];
    v.z = pack_bf16x2(dg[p][4], dg[p][5]) ^ sgn[2];
    v.w = pack_bf16x2(dg[p][6], dg[p][7]) ^ sgn[3];
    *(uint4*)(out + (size_t)p * plane + o) = v;
  }
}

// --------------------------------------------------------------- host
PFN_cuTensorMapEncodeTiled_v12000 get_encode(itg_handle* h) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  (void)h;
  return fn;
}

int make_map(itg_handle* h, CUtensorMap* map, void* base, int64_t inner, int64_t outer, int box_rows) {
  auto enc = get_encode(h);
  if (!enc) return itg_fail(h, ITG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  cuuint64_t strides[1] = {(cuuint64_t)(inner * 2)};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return itg_fail(h, ITG_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ITG_OK;
}

int ws_reserve(itg_handle* h, size_t bytes);

// CTAs of one variant that fit on the GPU at once (one per SM at this shared
// memory size), queried once per variant.
template <int BN>
int resident_ctas(itg_handle* h, int& out) {
  static int cached = 0;
  if (cached > 0) {
    out = cached;
    return ITG_OK;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_split_gemm<BN>, NUM_THREADS, Smem<BN>::TOTAL) !=
          cudaSuccess ||
      per_sm <= 0) {
    (void)cudaGetLastError();
    per_sm = 1;
  }
  const int n = per_sm * h->num_sms;
  cached = n > 0 ? n : 1;
  out = cached;
  return ITG_OK;
}

// streamk: one persistent CTA per resident slot sharing the work evenly
// (Part); otherwise one CTA per tile.
template <int BN>
int run(itg_handle* h, const ContractPlan& p, const double* A, const double* B, double* C,
        double alpha, double beta, bool streamk) {
  constexpr int S = S_SLICES;
  const int64_t Mpad = (p.M + BM - 1) / BM * BM;
  const int64_t Npad = (p.N + BN - 1) / BN * BN;
  const int64_t Kpad = (p.K + BK - 1) / BK * BK;
  if (Mpad * S > (int64_t)INT32_MAX || Npad * S > (int64_t)INT32_MAX || Kpad > (int64_t)INT32_MAX)
    return itg_fail(h, ITG_ERR_UNSUPPORTED, "split: problem too large");
  const int64_t tiles_m = Mpad / BM;
  const int64_t tiles = tiles_m * (Npad / BN);
  // F: fixed-point fraction bits of the int64 accumulator (keeps |acc| < 2^62).
  int lk = 0;
  while (((int64_t)1 << lk) < p.K) ++lk;
  const int F = 62 - 17 - lk;
  if (F < 8) return itg_fail(h, ITG_ERR_UNSUPPORTED, "split: contraction depth too large");
  if (tiles > (int64_t)INT32_MAX / 32) return itg_fail(h, ITG_ERR_UNSUPPORTED, "split: too many tiles");
  // the kernels need the attribute before the occupancy query
  static bool attr = false;
  if (!attr) {
    ITG_CUDA(h, cudaFuncSetAttribute(k_split_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     Smem<BN>::TOTAL));
    attr = true;
  }
  const int64_t nct = tiles;
  int64_t G = nct;
  if (streamk) {
    int res = 0;
    const int rst = resident_ctas<BN>(h, res);
    if (rst != ITG_OK) return rst;
    G = res;
  }
  const int64_t grid = G;
  const int64_t q = nct / G, r = nct % G;
  const bool shares = r != 0;  // the tail tiles are split between CTAs
  const size_t tile_bytes = sizeof(long long) * (size_t)BN * BM;
  // operands whose slices are kept (SliceCache): reuse on a match, else fill
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  ITG_CUDA(h, cudaStreamIsCapturing(h->stream, &cap));
  SliceCache* cache[2] = {nullptr, nullptr};
  bool hit[2] = {false, false};
  const double* srcs[2] = {A, B};
  const int64_t rpads[2] = {Mpad, Npad};
  for (int i = 0; i < 2; ++i) {
    if (!h->slice_keep[i]) continue;
    SliceCache& c = h->slice_cache[i];
    hit[i] = c.valid && c.src == srcs[i] && c.plan == (const void*)&p && c.rows_pad == rpads[i] && c.kpad == Kpad;
    if (hit[i]) {
      cache[i] = &c;
      continue;
    }
    if (cap != cudaStreamCaptureStatusNone) continue;  // no allocation inside a capture: plain path
    const size_t need = itg_align256(sizeof(int) * rpads[i]) + (size_t)2 * S * rpads[i] * Kpad;
    if (c.bytes < need) {
      ITG_CUDA(h, cudaStreamSynchronize(h->stream));
      if (c.buf) cudaFree(c.buf);
      c.buf = nullptr;
      c.bytes = 0;
      c.valid = false;
      if (cudaMalloc(&c.buf, need) != cudaSuccess) {
        (void)cudaGetLastError();
        c.buf = nullptr;
        continue;  // no room to keep them: plain path
      }
      c.bytes = need;
    }
    c.valid = false;
    cache[i] = &c;
  }
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off += itg_align256(b); return o; };
  const size_t oEA = take(cache[0] ? 0 : sizeof(int) * Mpad), oEB = take(cache[1] ? 0 : sizeof(int) * Npad);
  const size_t oSA = take(cache[0] ? 0 : (size_t)2 * S * Mpad * Kpad);
  const size_t oSB = take(cache[1] ? 0 : (size_t)2 * S * Npad * Kpad);
  const size_t oAcc = take(Smem<BN>::TACC ? 0 : tile_bytes * (size_t)grid);
  const size_t oTacc = take(shares ? tile_bytes * (size_t)grid : 0);
  const size_t oCnt = take(shares ? sizeof(int) * (size_t)grid : 0);
  const size_t oErr = take(sizeof(int));
  ITG_TRY(ws_reserve(h, off));
  char* ws = (char*)h->split_ws;
  int* eA = (int*)(ws + oEA);
  int* eB = (int*)(ws + oEB);
  __nv_bfloat16* sA = (__nv_bfloat16*)(ws + oSA);
  __nv_bfloat16* sB = (__nv_bfloat16*)(ws + oSB);
  if (cache[0]) {
    eA = (int*)cache[0]->buf;
    sA = (__nv_bfloat16*)((char*)cache[0]->buf + itg_align256(sizeof(int) * Mpad));
  }
  if (cache[1]) {
    eB = (int*)cache[1]->buf;
    sB = (__nv_bfloat16*)((char*)cache[1]->buf + itg_align256(sizeof(int) * Npad));
  }
  long long* acc = (long long*)(ws + oAcc);
  long long* tacc = (long long*)(ws + oTacc);
  int* cnt = (int*)(ws + oCnt);
  int* err = (int*)(ws + oErr);
  ITG_CUDA(h, cudaMemsetAsync(err, 0, sizeof(int), h->stream));
  if (shares) {
    ITG_CUDA(h, cudaMemsetAsync(tacc, 0, tile_bytes * (size_t)grid, h->stream));
    ITG_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)grid, h->stream));
  }
  // exponents
  {
    ProfScope prof(h, ITG_KERNEL_SPLIT_PREP);
    const int thr = 256;
    auto expo = [&](bool kmaj, const double* X, const int64_t* offR, const int64_t* offK, int64_t R,
                    int* ef) -> int {
      if (kmaj) {
        k_row_expfield<<<itg_blocks_for(R, thr / 32, h->num_sms * 16), thr, 0, h->stream>>>(
            X, offR, offK, R, p.K, ef);
      } else {
        ITG_CUDA(h, cudaMemsetAsync(ef, 0, sizeof(int) * R, h->stream));
        const int64_t ky = (p.K + 63) / 64;
        if (ky > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "split: contraction depth too large");
        dim3 g((unsigned)((R + thr - 1) / thr), (unsigned)ky);
        k_row_expfield_mmajor<<<g, thr, 0, h->stream>>>(X, offR, offK, R, p.K, ef);
      }
      return ITG_OK;
    };
    if (!hit[0]) ITG_TRY(expo(p.a_kmaj, A, p.offAm(), p.offAk(), p.M, eA));
    if (!hit[1]) ITG_TRY(expo(p.b_kmaj, B, p.offBn(), p.offBk(), p.N, eB));
    ITG_CHECK_LAUNCH(h);
  }
  // slices
  {
    ProfScope prof(h, ITG_KERNEL_SPLIT_PREP);
    dim3 gA((unsigned)(Kpad / 64), (unsigned)(Mpad / 32)), gB((unsigned)(Kpad / 64), (unsigned)(Npad / 32));
    if (gA.y > 65535 || gB.y > 65535) return itg_fail(h, ITG_ERR_UNSUPPORTED, "split: too many rows");
    if (!hit[0]) {
      if (p.a_kmaj)
        k_make_slices<true, S><<<gA, 256, 0, h->stream>>>(A, p.offAm(), p.offAk(), p.M, p.K, Mpad, Kpad, eA, sA);
      else
        k_make_slices<false, S><<<gA, 256, 0, h->stream>>>(A, p.offAm(), p.offAk(), p.M, p.K, Mpad, Kpad, eA, sA);
    }
    if (!hit[1]) {
      if (p.b_kmaj)
        k_make_slices<true, S><<<gB, 256, 0, h->stream>>>(B, p.offBn(), p.offBk(), p.N, p.K, Npad, Kpad, eB, sB);
      else
        k_make_slices<false, S><<<gB, 256, 0, h->stream>>>(B, p.offBn(), p.offBk(), p.N, p.K, Npad, Kpad, eB, sB);
    }
    ITG_CHECK_LAUNCH(h);
  }
  for (int i = 0; i < 2; ++i) {
    if (!cache[i] || hit[i]) continue;
    cache[i]->src = srcs[i];
    cache[i]->plan = (const void*)&p;
    cache[i]->rows_pad = rpads[i];
    cache[i]->kpad = Kpad;
    cache[i]->valid = true;
  }
  CUtensorMap mA, mB;
  ITG_TRY(make_map(h, &mA, sA, Kpad, Mpad * S, BM));
  ITG_TRY(make_map(h, &mB, sB, Kpad, Npad * S, BN));
  GemmArgs a;
  a.M = p.M;
  a.N = p.N;
  a.K = p.K;
  a.Mpad = (int)Mpad;
  a.Npad = (int)Npad;
  a.Kpad = (int)Kpad;
  a.nkb = (int)(Kpad / BK);
  a.S = S;
  a.F = F;
  a.tiles_n = (int)(Npad / BN);
  a.eA = eA;
  a.eB = eB;
  a.offCm = p.offCm();
  a.offCn = p.offCn();
  a.C = C;
  a.alpha = alpha;
  a.beta = beta;
  a.acc = acc;
  a.tacc = tacc;
  a.cnt = cnt;
  a.W = (int64_t)(S * (S + 1) / 2) * r;
  a.G = (int)G;
  a.q = (int)q;
  a.wait_ns = h->wait_ns;
  a.err = err;
  {
    ProfScope prof(h, ITG_KERNEL_GEMM_SPLIT);
    k_split_gemm<BN><<<(unsigned)grid, NUM_THREADS, Smem<BN>::TOTAL, h->stream>>>(mA, mB, a);
  }
  ITG_CHECK_LAUNCH(h);
  // surface a device-side timeout on the next synchronising call
  ITG_CUDA(h, cudaMemcpyAsync(h->dev_status, err, sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
  return ITG_OK;
}

// The H_eff middle step on the tensor cores (k_heff_mid_split); rows R =
// chiL chiR, T1 / T3 column-major with R rows.  ITG_ERR_UNSUPPORTED when nc or
// nj exceeds 32 (the caller then runs the FP64 kernel).
int heff_mid_split(itg_handle* h, int64_t R, int nc, int nj, const double* T1, const double* Weff, double* T3) {
  if (nc < 1 || nj < 1 || nc > MID_KSLICE || nj > 32) return ITG_ERR_UNSUPPORTED;
  const int64_t grid = (R + MID_ROWS - 1) / MID_ROWS;
  if (grid > (int64_t)INT32_MAX) return itg_fail(h, ITG_ERR_UNSUPPORTED, "heff mid: too many rows");
  ITG_TRY(ws_reserve(h, 256));
  int* err = (int*)h->split_ws;
  ITG_CUDA(h, cudaMemsetAsync(err, 0, sizeof(int), h->stream));
  auto launch = [&](auto njp_tag) -> int {
    constexpr int NJP = decltype(njp_tag)::value;
    static bool attr = false;
    if (!attr) {
      ITG_CUDA(h, cudaFuncSetAttribute(k_heff_mid_split<NJP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       MidSmem<NJP>::TOTAL));
      ITG_CUDA(h, cudaFuncSetAttribute(k_heff_mid_split<NJP>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
      attr = true;
    }
    // CTAs per SM: by shared memory (the carveout is set to its maximum) and by
    // TMEM (512 columns per SM)
    int smem_sm = 0;
    ITG_CUDA(h, cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device));
    int per_sm = smem_sm / (MidSmem<NJP>::TOTAL + 1024);
    const int tmem_cap = (int)(512u / MidSmem<NJP>::TMEM_COLS);
    if (per_sm > tmem_cap) per_sm = tmem_cap;
    if (per_sm < 1) per_sm = 1;
    const int64_t g = std::min<int64_t>(grid, (int64_t)per_sm * h->num_sms);
    k_heff_mid_split<NJP><<<(unsigned)g, MID_THREADS, MidSmem<NJP>::TOTAL, h->stream>>>(T1, Weff, T3, R, nc, nj,
                                                                                         h->wait_ns, err);
    ITG_CHECK_LAUNCH(h);
    return ITG_OK;
  };
  {
    ProfScope prof(h, ITG_KERNEL_HEFF_MID);
    if (nj <= 16) ITG_TRY(launch(std::integral_constant<int, 16>()));
    else ITG_TRY(launch(std::integral_constant<int, 32>()));
  }
  ITG_CUDA(h, cudaMemcpyAsync(h->dev_status, err, sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
  return ITG_OK;
}

int ws_reserve(itg_handle* h, size_t bytes) {
  if (bytes <= h->split_ws_bytes) return ITG_OK;
  size_t want = itg_align256(bytes + bytes / 8);
  if (h->split_ws) {
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->split_ws);
    h->split_ws = nullptr;
    h->split_ws_bytes = 0;
  }
  cudaError_t e = cudaMalloc(&h->split_ws, want);
  if (e != cudaSuccess) {
    h->split_ws = nullptr;
    return itg_fail(h, ITG_ERR_ALLOC, "split workspace of %zu bytes: %s", want, cudaGetErrorString(e));
  }
  h->split_ws_bytes = want;
  return ITG_OK;
}

}  // namespace split

namespace itg {
int heff_mid_split(itg_handle* h, int64_t R, int nc, int nj, const double* T1, const double* Weff, double* T3) {
  return split::heff_mid_split(h, R, nc, nj, T1, Weff, T3);
}
}  // namespace itg

// bn: tcgen05 tile variant: 128 or 256 columns, optionally | ITG_SPLIT_STREAMK
// (persistent CTAs sharing the work evenly); 0: 128 when N <= 128, else 256.
int itg_split_gemm(itg_handle* h, const ContractPlan& p, const double* A, const double* B, double* C,
                   double alpha, double beta, int bn) {
  if (bn == 0) bn = p.N <= 128 ? 128 : 256;
  const bool sk = (bn & ITG_SPLIT_STREAMK) != 0;
  bn &= ~ITG_SPLIT_STREAMK;
  if (bn == 128) return split::run<128>(h, p, A, B, C, alpha, beta, sk);
  return split::run<256>(h, p, A, B, C, alpha, beta, sk);
}

namespace itg {
int grid_barrier_selftest(itg_handle* h, int* status, int* blocks_out);  // itg_jacobi.cu
}

extern "C" int itg_set_wait_limit_ns(itg_handle* h, uint64_t ns) {
  if (!h) return ITG_ERR_INVALID;
  if (ns < 1000ull || ns > 60000000000ull)
    return itg_fail(h, ITG_ERR_INVALID, "wait limit %llu ns outside [1 us, 60 s]", (unsigned long long)ns);
  h->wait_ns = ns;
  return ITG_OK;
}

extern "C" int itg_wait_selftest(itg_handle* h, int which) {
  if (!h) return ITG_ERR_INVALID;
  if (which == 0) {
    int status = 0, blocks = 0;
    ITG_TRY(itg::grid_barrier_selftest(h, &status, &blocks));
    if (status != 0)
      return itg_fail(h, ITG_ERR_TIMEOUT, "grid barrier wait ran out after %llu ns (%d of 2 blocks gave up)",
                      (unsigned long long)h->wait_ns, blocks);
    return itg_fail(h, ITG_ERR_INVALID, "grid barrier self-test: the wait did not run out");
  }
  if (which == 1) {
    ITG_TRY(itg_scratch_reserve(h, 256));
    int* err = (int*)h->scratch;
    ITG_CUDA(h, cudaMemsetAsync(err, 0xFF, sizeof(int), h->stream));  // -1: not reported
    split::k_mbar_selftest<<<1, 32, 0, h->stream>>>(err, h->wait_ns);
    ITG_CHECK_LAUNCH(h);
    int* hp = (int*)h->pinned;
    ITG_CUDA(h, cudaMemcpyAsync(hp, err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hp[0] == ITG_ERR_TIMEOUT)
      return itg_fail(h, ITG_ERR_TIMEOUT, "mbarrier wait ran out after %llu ns", (unsigned long long)h->wait_ns);
    return itg_fail(h, ITG_ERR_INVALID, "mbarrier self-test: the wait did not run out (%d)", hp[0]);
  }
  return itg_fail(h, ITG_ERR_INVALID, "unknown self-test %d", which);
}

extern "C" int itg_split_partition(int64_t cluster_tiles, int clusters, int g, int32_t* seg, int cap,
                                   int* nseg) {
  if (cluster_tiles < 1 || clusters < 1 || g < 0 || g >= clusters || cap < 0 || !nseg || (cap > 0 && !seg) ||
      cluster_tiles > (int64_t)INT32_MAX / 32)
    return ITG_ERR_INVALID;
  split::Part part;
  part.S = split::S_SLICES;
  part.T = part.S * (part.S + 1) / 2;
  part.G = clusters;
  part.q = (int)(cluster_tiles / clusters);
  part.W = (int64_t)part.T * (cluster_tiles % clusters);
  int tb, lb, te, le;
  part.unit_at(part.lo(g), tb, lb);
  part.unit_at(part.lo(g + 1), te, le);
  int n = 0, ct, L0, Le;
  for (int si = 0; part.seg(g, si, tb, lb, te, le, ct, L0, Le); ++si, ++n) {
    if (n >= cap) continue;
    int first = 0;
    const int c = part.contributors(ct, first);
    int32_t* o = seg + 5 * n;
    o[0] = ct;
    o[1] = L0;
    o[2] = Le;
    o[3] = c;
    o[4] = first;
  }
  *nseg = n;
  return n > cap ? ITG_ERR_SHAPE : ITG_OK;
}

extern "C" double itg_split_error_bound(int64_t K) {
  // |C_split - C|_F <= 4 K 2^-8S (1 + (S+1)/4 * 1.02) |A|_F |B|_F + 2^-52 |C|_F
  // (digit truncation of both operands plus the dropped levels p + q >= S; the
  // 2^-52 term, bounded by |A|_F |B|_F, covers the final rounding to FP64).
  const int S = split::S_SLICES;
  const double k = (double)(K > 0 ? K : 1);
  return 4.0 * k * std::ldexp(1.0, -8 * S) * (1.0 + 0.255 * (S + 1)) + std::ldexp(1.0, -52);
}
