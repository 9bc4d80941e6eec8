// gemm_split.cu -- FP64-accurate GEMM on the BF16 tensor cores of sm_103a.
//
// C (M x N) = A (M x K) * B (K x N), all FP64 column-major, computed by error-
// free splitting (Ozaki, Ogita, Oishi & Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012):
//
//   A_ik = 2^{e_i - 60} sum_{s<S} a^s_ik 2^{53 - 8s},  B_kj likewise with f_j,
//
// e_i / f_j the row / column exponents (|A_ik| <= 2^{e_i}), so the scaled
// value is below 2^60 and every rounded digit satisfies |a^s|, |b^t| <= 128
// (exact in BF16).  Digit products are integers below 2^14; group g = s + t
// has g + 1 of them per k, so its partial sums over a K window of 128 stay
// below (g + 1) 2^21 < 2^24 for every g < S = 7: the FP32 tensor-core
// accumulation in TMEM is exact for all groups.  After each window the group
// sums are folded into two exact int64 accumulators per output,
//
//   H = acc_0 2^16 + acc_1 2^8 + acc_2,   L = acc_3 2^24 + acc_4 2^16 + acc_5 2^8 + acc_6,
//
// and the epilogue forms C_ij = 2^{e_i + f_j - 30} (H + 2^-32 L) with one FP64
// fma: the main loop issues no FP64 instruction (the FP64 pipe is the scarce
// unit on this part).  S = 7 planes carry 56 bits; the products dropped
// (s + t >= 7) weigh below 2^-56 of sum_k |A_ik||B_kj|.
//
// Kernels: k_split_a / k_split_b write the digit planes pre-tiled in the
// tcgen05 shared-memory image (K-major, no swizzle, 8x16-byte core matrices;
// B's planes stacked along N), so the GEMM stages each 16-deep K chunk with two
// cp.async.bulk (TMA) copies.  k_gemm_tc is persistent, one CTA per SM over
// 128 x 32 output tiles: a copy warp streams the chunks through six
// shared-memory stages, an MMA warp issues one tcgen05.mma.kind::f16 (BF16 x
// BF16 -> FP32) per A plane into one of two TMEM accumulator sets, and 8 warps
// drain a finished set with tcgen05.ld into exact int64 sums and write the
// tile.  Every mbarrier wait is bounded; a timeout sets an error flag and the
// CTA still waits for its copies and MMAs in flight and frees its TMEM.
#include <cuda_bf16.h>
#include <stdint.h>

#include <vector>

#include "hss_common.cuh"
#include "hss_gemm.h"
#include "hss_pool.h"

namespace hss {

constexpr int SP = 7;        // digit planes
constexpr int TM = 128;      // output tile rows (tcgen05 M)
constexpr int TN = 32;       // output tile cols (tcgen05 N)
constexpr int TK = 16;       // K per staged chunk (one MMA deep)
constexpr int KWIN = 128;    // exactness window for groups 0..2
constexpr int ATILE = TM * TK * 2;  // bytes of one A digit-plane tile (4 KB)
constexpr int BTILE = TN * TK * 2;  // bytes of one B digit-plane tile (1 KB)
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s bound on any wait

// ------------------------------------------------------------ splitting ---
// byte offset of element (r, k) inside a K-major no-swizzle tile with R rows:
// core matrix (r/8, k/8) is 128 contiguous bytes, rows of 16 bytes; core
// matrices adjacent in K are R*16 bytes apart (LBO), in R 128 bytes (SBO).
__device__ __forceinline__ int tile_off(int r, int k, int R) {
  return ((k >> 3) * (R >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Conversions between integer and floating types issue on the FP64 pipe of
// this part, which is its scarcest unit; the digit planes are built and read
// back with integer operations on the bit patterns instead.

// round(x * 2^(60 - e)) for |x| < 2^e by integer operations on the bits
__device__ __forceinline__ long long scaled_int(double x, int e) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  long long m = b & 0xFFFFFFFFFFFFFll;
  if (ex) m |= 1ll << 52;
  const int sh = (ex ? ex : 1) - 1015 - e;  // x = m 2^{(ex ? ex : 1) - 1075}
  long long q;
  if (sh >= 0) q = m << sh;  // sh <= 8 since |x| < 2^e
  else if (sh > -62) q = (m + (1ll << (-sh - 1))) >> (-sh);
  else q = 0;
  return b < 0 ? -q : q;
}

// BF16 bit pattern of an integer |d| <= 128 (exact)
__device__ __forceinline__ uint32_t bf16_of_int(int d) {
  const uint32_t a = (uint32_t)(d < 0 ? -d : d);
  const int e = 31 - __clz((int)(a | 1u));  // a in [2^e, 2^(e+1)), e <= 7
  const uint32_t bits = (d < 0 ? 0x8000u : 0u) | ((uint32_t)(e + 127) << 7) | ((a << (7 - e)) & 0x7Fu);
  return a ? bits : 0u;
}

// the value of an FP32 that holds an exact integer below 2^31 in magnitude
__device__ __forceinline__ int int_of_float(float v) {
  const int f = __float_as_int(v);
  const int E = ((f >> 23) & 0xFF) - 127;
  const int M = (f & 0x7FFFFF) | 0x800000;
  const int a = E < 0 ? 0 : (E >= 23 ? M << (E - 23) : M >> (23 - E));
  return f < 0 ? -a : a;
}

// (H + 2^-32 L) 2^e rounded to the nearest double (ties to even), from the
// exact 128-bit integer H 2^32 + L by integer operations; the FP64 pipe is
// used only when the result leaves the normal range.
__device__ __forceinline__ double exact_double(long long H, long long L, int e) {
  unsigned long long lo = (unsigned long long)H << 32;
  unsigned long long hi = (unsigned long long)(H >> 32);
  const unsigned long long l = (unsigned long long)L;
  const unsigned long long nlo = lo + l;
  hi += (unsigned long long)(L >> 63) + (nlo < lo ? 1ull : 0ull);
  lo = nlo;
  const bool neg = (long long)hi < 0;
  if (neg) {  // two's complement of the 128-bit value
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
  if ((hi | lo) == 0ull) return 0.0;
  const int n = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);  // bit length
  unsigned long long mant;
  int nn = n;
  if (n <= 53) {
    mant = lo << (53 - n);
  } else {
    const int sh = n - 53;  // 1 .. 75
    mant = sh < 64 ? (lo >> sh) | (sh ? hi << (64 - sh) : 0ull) : hi >> (sh - 64);
    const int hb = sh - 1;  // the rounding bit
    const unsigned long long half =
        hb < 64 ? (lo >> hb) & 1ull : (hi >> (hb - 64)) & 1ull;
    bool sticky;
    if (hb < 64) sticky = hb ? (lo & ((1ull << hb) - 1ull)) != 0ull : false;
    else sticky = lo != 0ull || (hb > 64 && (hi & ((1ull << (hb - 64)) - 1ull)) != 0ull);
    if (half && (sticky || (mant & 1ull))) {
      ++mant;
      if (mant == (1ull << 53)) { mant >>= 1; ++nn; }
    }
  }
  const int be = (nn - 1) + e - 32 + 1023;  // biased exponent of the leading bit
  if (be <= 0 || be >= 2047) {  // out of the normal range: scale in FP64
    const double v = ldexp((double)mant, nn - 53 + e - 32);
    return neg ? -v : v;
  }
  const unsigned long long bits = (neg ? 0x8000000000000000ull : 0ull) |
                                  ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

// the SP digits of q (|q| <= 2^60): d_s = round(q_s / 2^{53 - 8s}), |d_s| <= 128
__device__ __forceinline__ void split_digits(double x, int e, __nv_bfloat16 *dig) {
  long long q = scaled_int(x, e);
#pragma unroll
  for (int s = 0; s < SP; ++s) {
    const int sh = 53 - 8 * s;
    const long long d = (q + (1ll << (sh - 1))) >> sh;
    q -= d * (1ll << sh);
    dig[s] = __ushort_as_bfloat16((unsigned short)bf16_of_int((int)d));
  }
}

// frexp exponent of the largest |x| from its bit pattern (0 for zero)
__device__ __forceinline__ int bits_exp(unsigned long long b) {
  if (b == 0) return 0;
  const int ex = (int)(b >> 52);
  return ex ? ex - 1022 : (64 - __clzll((long long)b)) - 1074;
}


// The split runs over work items (operand, panel, chunk of SPLIT_KC k values):
// k_split_amax / k_split_bmax record the largest |x| of every row of A /
// column of B as its bit pattern (atomicMax on the sign-cleared bits, which
// order like |x|), then k_split_a / k_split_b write the digits of their chunk
// with the row / column exponents frexp(max|x|).  Many items per panel keep
// enough loads in flight for the long K of the large products.
constexpr int SPLIT_KC = 128;
constexpr int SPLIT_KT = SPLIT_KC / TK;  // k tiles per item

// the operand whose items contain flattened item b (operands sorted by w0)
__device__ __forceinline__ int split_operand(const SplitProb *__restrict__ probs, int nprob, int b) {
  int lo = 0, hi = nprob;
  while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (probs[mid].w0 <= b) lo = mid; else hi = mid; }
  return lo;
}

// A (M x K, lda): item = (row panel tm, chunk kc), tm fastest
__global__ void __launch_bounds__(256)
k_split_amax(const SplitProb *__restrict__ probs, int nprob) {
  const SplitProb P = probs[split_operand(probs, nprob, blockIdx.x)];
  if (P.ktiles <= SPLIT_KT) return;  // one chunk: k_split_a takes the maxima itself
  const int t = blockIdx.x - P.w0, ntm = (P.rows + TM - 1) / TM;
  const int tm = t % ntm, kc = t / ntm;
  const int tid = threadIdx.x, half = tid >> 7, r = tm * TM + (tid & 127);
  const int k1 = min(P.inner, (kc + 1) * SPLIT_KC);
  unsigned long long m = 0;
  if (r < P.rows) {
#pragma unroll 4
    for (int k = kc * SPLIT_KC + half; k < k1; k += 2) {
      const unsigned long long b =
          (unsigned long long)__double_as_longlong(P.src[(long long)k * P.ld + r]) & 0x7FFFFFFFFFFFFFFFull;
      m = b > m ? b : m;
    }
  }
  __shared__ unsigned long long sm[128];
  if (half) sm[tid & 127] = m;
  __syncthreads();
  if (!half && r < P.rows) {
    const unsigned long long o = sm[tid];
    atomicMax(P.mbits + r, o > m ? o : m);
  }
}

// A: planes [tile_m][tile_k][s] of TM x TK for the k tiles of chunk kc; the
// thread handles (row, 8 consecutive k) -> 16-byte rows of core matrices
__global__ void __launch_bounds__(256)
k_split_a(const SplitProb *__restrict__ probs, int nprob) {
  const SplitProb P = probs[split_operand(probs, nprob, blockIdx.x)];
  const int t = blockIdx.x - P.w0, ntm = (P.rows + TM - 1) / TM;
  const int tm = t % ntm, kc = t / ntm;
  const int tid = threadIdx.x;
  __shared__ int sexp[TM];
  __shared__ unsigned long long smx[8][TM];
  const bool single = P.ktiles <= SPLIT_KT;
  if (single) {  // one chunk: the row maxima here (warps over k, lanes over rows)
    const int lane = tid & 31, w = tid >> 5;
    unsigned long long mx[4] = {0, 0, 0, 0};
    for (int k = w; k < P.inner; k += 8)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = tm * TM + q * 32 + lane;
        if (r < P.rows) {
          const unsigned long long b =
              (unsigned long long)__double_as_longlong(P.src[(long long)k * P.ld + r]) & 0x7FFFFFFFFFFFFFFFull;
          mx[q] = b > mx[q] ? b : mx[q];
        }
      }
#pragma unroll
    for (int q = 0; q < 4; ++q) smx[w][q * 32 + lane] = mx[q];
    __syncthreads();
  }
  if (tid < TM) {
    const int r = tm * TM + tid;
    unsigned long long m = 0;
    if (single) {
      for (int i = 0; i < 8; ++i) m = smx[i][tid] > m ? smx[i][tid] : m;
    } else if (r < P.rows) {
      m = P.mbits[r];
    }
    const int e = r < P.rows ? bits_exp(m) : 0;
    sexp[tid] = e;
    if (kc == 0 && r < P.rows) P.expo[r] = e;
  }
  __syncthreads();
  const int kt0 = kc * SPLIT_KT, nkt = min(P.ktiles, kt0 + SPLIT_KT) - kt0;
  for (int v = tid; v < nkt * TM * (TK / 8); v += 256) {
    const int kt = kt0 + v / (TM * (TK / 8)), u = v % (TM * (TK / 8));
    char *tile = (char *)P.dst + ((long long)tm * P.ktiles + kt) * SP * ATILE;
    const int r = u % TM, k8 = u / TM;
    const int gr = tm * TM + r;
    __align__(16) __nv_bfloat16 dg[SP][8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int gk = kt * TK + k8 * 8 + c;
      const double x = (gr < P.rows && gk < P.inner) ? P.src[(long long)gk * P.ld + gr] : 0.0;
      __nv_bfloat16 d[SP];
      split_digits(x, sexp[r], d);
#pragma unroll
      for (int s = 0; s < SP; ++s) dg[s][c] = d[s];
    }
#pragma unroll
    for (int s = 0; s < SP; ++s)
      *reinterpret_cast<uint4 *>(tile + s * ATILE + tile_off(r, k8 * 8, TM)) =
          *reinterpret_cast<uint4 *>(dg[s]);
  }
}

// B (K x N, ldb; column gc holds k contiguously): item = (column panel tn,
// chunk kc); warp per column, lanes along k
__global__ void __launch_bounds__(256)
k_split_bmax(const SplitProb *__restrict__ probs, int nprob) {
  const SplitProb P = probs[split_operand(probs, nprob, blockIdx.x)];
  if (P.ktiles <= SPLIT_KT) return;  // one chunk: k_split_b takes the maxima itself
  const int t = blockIdx.x - P.w0, ntn = (P.rows + TN - 1) / TN;
  const int tn = t % ntn, kc = t / ntn;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k1 = min(P.inner, (kc + 1) * SPLIT_KC);
  for (int c = w; c < TN; c += 8) {
    const int gc = tn * TN + c;
    if (gc >= P.rows) break;
    unsigned long long m = 0;
    for (int k = kc * SPLIT_KC + lane; k < k1; k += 32) {
      const unsigned long long b =
          (unsigned long long)__double_as_longlong(P.src[(long long)gc * P.ld + k]) & 0x7FFFFFFFFFFFFFFFull;
      m = b > m ? b : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long v = __shfl_xor_sync(HSS_FULL, m, o);
      m = v > m ? v : m;
    }
    if (lane == 0) atomicMax(P.mbits + gc, m);
  }
}

// B: one K-major tile per (tile_n, tile_k) holding the SP planes stacked along
// N (plane p in rows p TN .. p TN + TN - 1, so the planes 0..P-1 form one
// operand of N = P TN rows), for the k tiles of chunk kc
__global__ void __launch_bounds__(256)
k_split_b(const SplitProb *__restrict__ probs, int nprob) {
  const SplitProb P = probs[split_operand(probs, nprob, blockIdx.x)];
  const int t = blockIdx.x - P.w0, ntn = (P.rows + TN - 1) / TN;
  const int tn = t % ntn, kc = t / ntn;
  const int tid = threadIdx.x;
  __shared__ int sexp[TN];
  if (P.ktiles <= SPLIT_KT) {  // one chunk: warp per column, max over k here
    const int lane = tid & 31, w = tid >> 5;
    for (int c = w; c < TN; c += 8) {
      const int gc = tn * TN + c;
      unsigned long long m = 0;
      if (gc < P.rows)
        for (int k = lane; k < P.inner; k += 32) {
          const unsigned long long b =
              (unsigned long long)__double_as_longlong(P.src[(long long)gc * P.ld + k]) & 0x7FFFFFFFFFFFFFFFull;
          m = b > m ? b : m;
        }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(HSS_FULL, m, o);
        m = v > m ? v : m;
      }
      if (lane == 0) {
        const int e = bits_exp(m);
        sexp[c] = e;
        if (gc < P.rows) P.expo[gc] = e;
      }
    }
  } else if (tid < TN) {
    const int gc = tn * TN + tid;
    const int e = gc < P.rows ? bits_exp(P.mbits[gc]) : 0;
    sexp[tid] = e;
    if (kc == 0 && gc < P.rows) P.expo[gc] = e;
  }
  __syncthreads();
  const int kt0 = kc * SPLIT_KT, nkt = min(P.ktiles, kt0 + SPLIT_KT) - kt0;
  for (int v = tid; v < nkt * TN * (TK / 8); v += 256) {
    const int kt = kt0 + v / (TN * (TK / 8)), u = v % (TN * (TK / 8));
    char *tile = (char *)P.dst + ((long long)tn * P.ktiles + kt) * SP * BTILE;
    const int c = u / (TK / 8), k8 = u % (TK / 8);
    const int gc = tn * TN + c;
    __align__(16) __nv_bfloat16 dg[SP][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int gk = kt * TK + k8 * 8 + q;
      const double x = (gc < P.rows && gk < P.inner) ? P.src[(long long)gc * P.ld + gk] : 0.0;
      __nv_bfloat16 d[SP];
      split_digits(x, sexp[c], d);
#pragma unroll
      for (int s = 0; s < SP; ++s) dg[s][q] = d[s];
    }
#pragma unroll
    for (int s = 0; s < SP; ++s)
      *reinterpret_cast<uint4 *>(tile + tile_off(s * TN + c, k8 * 8, SP * TN)) =
          *reinterpret_cast<uint4 *>(dg[s]);
  }
}

// ------------------------------------------------------- PTX wrappers -----
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  // base offset 0, relative LBO, swizzle none (bits 61-63 = 0)
  return d;
}

// kind::f16 instruction descriptor: D FP32, A/B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4)                     // D format FP32
         | (1u << 7)                   // A format BF16
         | (1u << 10)                  // B format BF16
         | ((uint32_t)(N >> 3) << 17)  // N / 8
         | ((uint32_t)(M >> 4) << 24); // M / 16
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// wait on phase parity, bounded by WAIT_NS of wall time; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity));
    if (done) return true;
    if (globaltimer_ns() - t0 > WAIT_NS) return false;
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes));
}

// bulk (non-tensor) TMA copy global -> shared, completion on an mbarrier
__device__ __forceinline__ void tma_load(void *sdst, const void *gsrc, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(sdst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                     uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------- GEMM ----
struct TcProb {
  const char *a_planes;  // [tm][kt][s] ATILE
  const char *b_planes;  // [tn][kt] SP * BTILE, planes stacked along N
  const int *ea, *eb;    // row / column exponents
  double *C;
  int ldc, M, N, ktiles, beta;
  int tile0;             // first flattened tile index
};

// Persistent kernel, one CTA per SM: warp 0 (one lane) streams the K chunks
// of the CTA's tiles through NST shared-memory stages with bulk copies;
// warp 1 (one lane) issues the 28 plane products of every chunk into one of
// two TMEM accumulator sets, alternating per 128-deep exactness window;
// warps 2..9 drain a finished set into exact int64 sums (the other set
// meanwhile takes the next window's MMAs) and write the tile's doubles.  So
// copies, MMAs and drains of consecutive tiles overlap.  Tiles t = blockIdx.x
// + i gridDim.x; tprob[t] names the tile's product.  Every wait is bounded;
// after a timeout every role stops, the CTA waits (bounded) for its copies
// and MMAs in flight, then frees its TMEM.
constexpr int NST = 6;                            // staged chunks in flight
constexpr int GTH = 320;                          // 10 warps
constexpr int ACC_SET = 256;                      // TMEM columns per accumulator set
constexpr int TMEM_TC = 2 * ACC_SET;
constexpr int STAGE_TC = SP * (ATILE + BTILE);    // one K chunk of both operands (35 KB)
constexpr int SMEM_TC = NST * STAGE_TC + 1024;
static_assert(SP * TN <= ACC_SET, "accumulator groups exceed a TMEM set");
static_assert(SMEM_TC <= 226 * 1024, "stages exceed the shared memory of a CTA");

__global__ void __launch_bounds__(GTH, 1)
k_gemm_tc(const TcProb *__restrict__ probs, const int *__restrict__ tprob, int ntiles,
          int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t full[NST], empty[NST], afull[2], aempty[2], fin;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_ok;
  __shared__ long long s_issued, s_consumed;
  __shared__ int s_skip;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // another CTA's wait already timed out: the launch is failing, skip the
  // work (one read, so the whole CTA leaves together)
  if (tid == 0) s_skip = *(volatile int *)err;
  __syncthreads();
  if (s_skip) return;
  auto sa = [&](int q) { return smem + q * STAGE_TC; };
  auto sb = [&](int q) { return smem + q * STAGE_TC + SP * ATILE; };
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(TMEM_TC));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int q = 0; q < NST; ++q) { mbar_init(&full[q], 1); mbar_init(&empty[q], 1); }
    for (int a = 0; a < 2; ++a) { mbar_init(&afull[a], 1); mbar_init(&aempty[a], 8); }
    mbar_init(&fin, 1);
    s_ok = 1;
    s_issued = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tbase = tmem_base;
  const int kwin = KWIN / TK;  // chunks per exactness window
  // Chunk g (counted over the CTA's tiles) lives in stage g % NST, that
  // stage's (g / NST)-th use: its "full" phase has parity (g / NST) & 1 and
  // the stage is free for it once "empty" of use g / NST - 1 completed.
  // Window w (counted likewise) accumulates in set w & 1, that set's
  // (w / 2)-th use, with the same parity rule for afull / aempty.
  if (warp == 0) {
    if (lane == 0) {  // copies
      long long g = 0;
      for (int t = blockIdx.x; t < ntiles && s_ok; t += gridDim.x) {
        const TcProb &P = probs[__ldg(tprob + t)];
        const int nk = P.ktiles, ntm = (P.M + TM - 1) / TM, tt = t - P.tile0;
        const char *ga0 = P.a_planes + (long long)(tt % ntm) * nk * SP * ATILE;
        const char *gb0 = P.b_planes + (long long)(tt / ntm) * nk * SP * BTILE;
        for (int kt = 0; kt < nk && s_ok; ++kt, ++g) {
          const int q = (int)(g % NST);
          if (g >= NST && !mbar_wait(&empty[q], (uint32_t)((g / NST) - 1) & 1)) {
            atomicOr(err, 1); s_ok = 0; break;
          }
          mbar_expect_tx(&full[q], STAGE_TC);
          tma_load(sa(q), ga0 + (long long)kt * SP * ATILE, SP * ATILE, &full[q]);
          tma_load(sb(q), gb0 + (long long)kt * SP * BTILE, SP * BTILE, &full[q]);
          s_issued = g + 1;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMAs
      long long g = 0, w = 0;
      for (int t = blockIdx.x; t < ntiles && s_ok; t += gridDim.x) {
        const int nk = probs[__ldg(tprob + t)].ktiles;
        for (int k0 = 0; k0 < nk && s_ok; k0 += kwin, ++w) {
          const int k1 = min(nk, k0 + kwin), a = (int)(w & 1);
          if (w >= 2 && !mbar_wait(&aempty[a], (uint32_t)((w / 2) - 1) & 1)) {
            atomicOr(err, 2); s_ok = 0; break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t acc = tbase + (uint32_t)(a * ACC_SET);
          for (int kt = k0; kt < k1 && s_ok; ++kt, ++g) {
            const int q = (int)(g % NST);
            if (!mbar_wait(&full[q], (uint32_t)(g / NST) & 1)) { atomicOr(err, 4); s_ok = 0; break; }
            s_consumed = g + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // descriptor(address + offset) = descriptor(address) + offset / 16.
            // A plane s2 times B planes 0 .. SP-1-s2 (stacked along N) is one
            // MMA of N = (SP - s2) TN whose column block p2 lands on group
            // s2 + p2; the window's first MMA (s2 = 0) overwrites every group
            const uint64_t ad0 = make_desc(smem_u32(sa(q)), TM * 16, 128);
            const uint64_t bd = make_desc(smem_u32(sb(q)), SP * TN * 16, 128);
            const uint32_t later = kt > k0 ? 1u : 0u;
#pragma unroll
            for (int s2 = 0; s2 < SP; ++s2)
              umma(acc + s2 * TN, ad0 + (uint64_t)((s2 * ATILE) >> 4), bd,
                   make_idesc(TM, (SP - s2) * TN), s2 > 0 ? 1u : later);
            umma_commit(&empty[q]);  // stage q is free once these MMAs completed
          }
          umma_commit(&afull[a]);    // the window's sums are complete
        }
      }
      // every MMA issued (also before an error) completes before TMEM is freed
      umma_commit(&fin);
      if (!mbar_wait(&fin, 0)) { atomicOr(err, 8); s_ok = 0; }
    }
  } else {  // warps 2..9: drain and write; TMEM lanes 32 (warp % 4) ..
    const int quarter = warp & 3, half = (warp - 2) >> 2;
    constexpr int TH = TN / 2;  // output columns per thread
    static_assert(TH == 16, "the drain reads 16 TMEM columns per group");
    long long w = 0;
    for (int t = blockIdx.x; t < ntiles && s_ok; t += gridDim.x) {
      const TcProb &P = probs[__ldg(tprob + t)];
      const int nk = P.ktiles, ntm = (P.M + TM - 1) / TM, tt = t - P.tile0;
      long long hacc[TH], lacc[TH];
#pragma unroll
      for (int j = 0; j < TH; ++j) { hacc[j] = 0; lacc[j] = 0; }
      bool okt = true;
      for (int k0 = 0; k0 < nk; k0 += kwin, ++w) {
        const int a = (int)(w & 1);
        // one lane waits, the warp follows its verdict (tcgen05.ld is warp-wide)
        int got = 0;
        if (lane == 0) got = mbar_wait(&afull[a], (uint32_t)(w / 2) & 1) ? 1 : 0;
        got = __shfl_sync(HSS_FULL, got, 0);
        if (!got) {
          if (lane == 0) { atomicOr(err, 16); s_ok = 0; }
          okt = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t lane_addr = tbase + (uint32_t)(a * ACC_SET) +
                                   ((uint32_t)(quarter * 32) << 16) + (uint32_t)(half * TH);
#pragma unroll
        for (int gq = 0; gq < SP; ++gq) {
          float v[16];
          tmem_ld16(lane_addr + gq * TN, v);
#pragma unroll
          for (int i = 0; i < TH; ++i) {
            const long long x = (long long)int_of_float(v[i]);
            if (gq < 3) hacc[i] += x * (1ll << (8 * (2 - gq)));
            else lacc[i] += x * (1ll << (8 * (6 - gq)));
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&aempty[a]);  // the set may take new MMAs
      }
      if (!okt) break;
      // C = 2^{e_i + f_j - 30} (H + 2^-32 L) (+ C)
      const int r = (tt % ntm) * TM + quarter * 32 + lane;
      if (r < P.M) {
        const int ei = P.ea[r];
#pragma unroll
        for (int j = 0; j < TH; ++j) {
          const int c = (tt / ntm) * TN + half * TH + j;
          if (c < P.N) {
            const double v = exact_double(hacc[j], lacc[j], ei + P.eb[c] - 30);
            double *dst = P.C + (long long)c * P.ldc + r;
            *dst = P.beta ? *dst + v : v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid == 0 && !s_ok) {
    // a bounded wait gave up: wait (bounded) for the copies still in flight
    // before the CTA's shared memory is released
    for (long long g = s_consumed; g < s_issued; ++g)
      if (!mbar_wait(&full[g % NST], (uint32_t)(g / NST) & 1)) break;
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(TMEM_TC));
}

// ------------------------------------------------- fused split GEMM -----
// Many small and medium products (the dense merge updates of the middle DC
// levels): each CTA splits its own FP64 A and B chunks into the SP digit
// planes directly in shared memory and issues the plane products on the
// tensor cores, so no plane buffer goes through global memory and no FP64
// instruction is spent on the splitting (the digits come from the operands'
// bit patterns; row / column exponents from a small pre-pass).  Tile 128 x 32,
// K chunks of 32 (56 MMAs of 128 x 32 x 16 each), 128-deep exactness windows
// drained into correctly rounded doubles (integer operations) and summed.
// About 100 KB of shared memory and 256 TMEM columns per CTA: two CTAs share
// an SM, so one's splitting overlaps the other's MMAs.  (Measured on the DC shapes it is issue bound -- every A
// element is split once per 32-column tile -- and slower than the staged
// planes, so it is the alternative, hss_config.gemm_path = 1.)
constexpr int FM = 128, FN = 32, FK = 32;
constexpr int FATILE = FM * FK * 2;  // 8 KB per A plane
constexpr int FBTILE = FN * FK * 2;  // 2 KB per B plane
constexpr int FSMEM = 100 * 1024;    // >= SP * (FATILE + FBTILE); caps residency at 2 CTAs per SM
static_assert(SP * (FATILE + FBTILE) + 1024 <= FSMEM, "fused GEMM tiles exceed the shared budget");

struct FusedProb {
  const double *A, *B;
  double *C;
  const int *ea, *eb;  // row / column exponents (frexp convention)
  int lda, ldb, ldc, M, N, K, beta;
  int tile0;
};
struct ExpJob {  // rows of A (stride = lda between k) or columns of B (contiguous k)
  const double *X;
  int ld, count, K;
  int *out;
  int off;       // first flattened item of this job
};


// the SP digits of q (|q| <= 2^60) as BF16 bit patterns, packed into the
// 16-byte core-matrix rows (element c of the 8 at half-word c)
__device__ __forceinline__ void digits_into(long long q, int c, uint32_t (*pk)[4]) {
#pragma unroll
  for (int s = 0; s < SP; ++s) {
    const int sh = 53 - 8 * s;
    const long long d = (q + (1ll << (sh - 1))) >> sh;
    q -= d * (1ll << sh);
    pk[s][c >> 1] |= bf16_of_int((int)d) << (16 * (c & 1));
  }
}

__global__ void k_row_exps(const ExpJob *__restrict__ jobs, int nj, int total) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int lo = 0, hi = nj;
  while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (jobs[mid].off <= t) lo = mid; else hi = mid; }
  const ExpJob J = jobs[lo];
  const int r = t - J.off;
  unsigned long long m = 0;
  for (int k = 0; k < J.K; ++k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(J.X[(long long)k * J.ld + r]) & 0x7FFFFFFFFFFFFFFFull;
    m = b > m ? b : m;
  }
  J.out[r] = bits_exp(m);
}

__global__ void k_col_exps(const ExpJob *__restrict__ jobs, int nj, int total) {
  const int w = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (w >= total) return;
  int lo = 0, hi = nj;
  while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (jobs[mid].off <= w) lo = mid; else hi = mid; }
  const ExpJob J = jobs[lo];
  const int c = w - J.off;
  unsigned long long m = 0;
  for (int k = lane; k < J.K; k += 32) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(J.X[(long long)c * J.ld + k]) & 0x7FFFFFFFFFFFFFFFull;
    m = b > m ? b : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(HSS_FULL, m, o);
    m = v > m ? v : m;
  }
  if (lane == 0) J.out[c] = bits_exp(m);
}

__global__ void __launch_bounds__(128, 2)
k_gemm_fused(const FusedProb *__restrict__ probs, int nprob, int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char fsm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  int lo = 0, hi = nprob;
  const int b = blockIdx.x;
  while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (probs[mid].tile0 <= b) lo = mid; else hi = mid; }
  __shared__ int s_skip;  // another CTA's wait timed out: the whole CTA skips the work
  if (threadIdx.x == 0) s_skip = *(volatile int *)err;
  __syncthreads();
  if (s_skip) return;
  const FusedProb P = probs[lo];
  const int t = b - P.tile0, ntm = (P.M + FM - 1) / FM;
  const int tm = t % ntm, tn = t / ntm;
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char *sa = fsm, *sb = fsm + SP * FATILE;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tbase = tmem_base;
  const uint32_t idesc = make_idesc(FM, FN);
  const int r = tm * FM + tid;
  const bool rok = r < P.M;
  const int er = rok ? P.ea[r] : 0;
  const int cb = tid >> 2, ko = tid & 3;  // this thread's B column and k octet
  const int gcb = tn * FN + cb;
  const bool cok = gcb < P.N;
  const int ecb = cok ? P.eb[gcb] : 0;
  __shared__ int s_eb[FN];
  if (tid < FN) s_eb[tid] = (tn * FN + tid < P.N) ? P.eb[tn * FN + tid] : 0;
  double acc[FN];
#pragma unroll
  for (int j = 0; j < FN; ++j) acc[j] = 0.0;
  uint32_t ph = 0;
  bool ok = true;
  for (int w0 = 0; w0 < P.K && ok; w0 += KWIN) {
    const int w1 = min(P.K, w0 + KWIN);
    for (int k0 = w0; k0 < w1; k0 += FK) {
      // split this thread's row of the A chunk (coalesced over the rows)
#pragma unroll 1
      for (int k8 = 0; k8 < FK / 8; ++k8) {
        uint32_t pk[SP][4];
#pragma unroll
        for (int s2 = 0; s2 < SP; ++s2) pk[s2][0] = pk[s2][1] = pk[s2][2] = pk[s2][3] = 0u;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int gk = k0 + k8 * 8 + c;
          const double x = (rok && gk < w1) ? P.A[(long long)gk * P.lda + r] : 0.0;
          digits_into(scaled_int(x, er), c, pk);
        }
#pragma unroll
        for (int s2 = 0; s2 < SP; ++s2)
          *reinterpret_cast<uint4 *>(sa + s2 * FATILE + tile_off(tid, k8 * 8, FM)) =
              make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
      }
      // split one k octet of one B column
      {
        uint32_t pk[SP][4];
#pragma unroll
        for (int s2 = 0; s2 < SP; ++s2) pk[s2][0] = pk[s2][1] = pk[s2][2] = pk[s2][3] = 0u;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int gk = k0 + ko * 8 + c;
          const double x = (cok && gk < w1) ? P.B[(long long)gcb * P.ldb + gk] : 0.0;
          digits_into(scaled_int(x, ecb), c, pk);
        }
#pragma unroll
        for (int s2 = 0; s2 < SP; ++s2)
          *reinterpret_cast<uint4 *>(sb + s2 * FBTILE + tile_off(cb, ko * 8, FN)) =
              make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
      }
      // generic-proxy stores -> visible to the tensor cores' async proxy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint64_t ad0 = make_desc(smem_u32(sa), FM * 16, 128);
        const uint64_t bd0 = make_desc(smem_u32(sb), FN * 16, 128);
        const uint32_t later = k0 > w0 ? 1u : 0u;
#pragma unroll
        for (int kk = 0; kk < FK / 16; ++kk)
#pragma unroll
          for (int s2 = 0; s2 < SP; ++s2)
#pragma unroll
            for (int q = 0; q + s2 < SP; ++q) {
              const uint32_t accum = (kk > 0 || s2 > 0) ? 1u : later;
              umma(tbase + (s2 + q) * FN, ad0 + (uint64_t)((s2 * FATILE + kk * 2 * (FM * 16)) >> 4),
                   bd0 + (uint64_t)((q * FBTILE + kk * 2 * (FN * 16)) >> 4), idesc, accum);
            }
        umma_commit(&bar);
      }
      __syncwarp();
      ok = __syncthreads_and(mbar_wait(&bar, ph));
      ph ^= 1;
      if (!ok) { if (tid == 0) atomicOr(err, 2); break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    if (!ok) break;
    // drain the window's exact group sums
    const uint32_t lane_addr = tbase + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int c = 0; c < FN; c += 16) {
      long long hv[16], lv[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) { hv[i] = 0; lv[i] = 0; }
#pragma unroll
      for (int g = 0; g < SP; ++g) {
        float v[16];
        tmem_ld16(lane_addr + g * FN + c, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const long long x = (long long)int_of_float(v[i]);
          if (g < 3) hv[i] += x * (1ll << (8 * (2 - g)));
          else lv[i] += x * (1ll << (8 * (6 - g)));
        }
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const double v = exact_double(hv[i], lv[i], er + s_eb[c + i] - 30);
        acc[c + i] = w0 == 0 ? v : acc[c + i] + v;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (ok && rok) {
#pragma unroll
    for (int j = 0; j < FN; ++j) {
      const int c = tn * FN + j;
      if (c < P.N) {
        double *dst = P.C + (long long)c * P.ldc + r;
        *dst = P.beta ? *dst + acc[j] : acc[j];
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(256));
}

// ----------------------------------------------------------------- host ---
void launch_gemm_split(const std::vector<GemmDesc> &probs, int *d_err, cudaStream_t st) {
  if (probs.empty()) return;
  // split every A and B operand
  std::vector<SplitProb> sa, sb;
  std::vector<TcProb> tc;
  long long abytes = 0, bbytes = 0, ea = 0, eb = 0, wa = 0, wb = 0;
  int tiles = 0;
  bool multi = false;  // some operand has more than one k chunk
  for (const auto &p : probs) {
    const int kt = (p.K + TK - 1) / TK;
    const int ntm = (p.M + TM - 1) / TM, ntn = (p.N + TN - 1) / TN;
    const int nkc = (kt + SPLIT_KT - 1) / SPLIT_KT;
    multi = multi || nkc > 1;
    SplitProb a{p.A, p.lda, p.M, p.K, kt, nullptr, nullptr, nullptr, (int)wa};
    SplitProb bb{p.B, p.ldb, p.N, p.K, kt, nullptr, nullptr, nullptr, (int)wb};
    a.dst = (void *)abytes; a.expo = (int *)ea; a.mbits = (unsigned long long *)ea;
    bb.dst = (void *)bbytes; bb.expo = (int *)eb; bb.mbits = (unsigned long long *)eb;
    abytes += (long long)ntm * kt * SP * ATILE;
    bbytes += (long long)ntn * kt * SP * BTILE;
    ea += ntm * TM;
    eb += ntn * TN;
    wa += (long long)ntm * nkc;
    wb += (long long)ntn * nkc;
    sa.push_back(a); sb.push_back(bb);
    TcProb t{nullptr, nullptr, nullptr, nullptr, p.C, p.ldc, p.M, p.N, kt, p.beta, tiles};
    tiles += ntm * ntn;
    tc.push_back(t);
  }
  if (tiles == 0) return;  // every product is empty
  char *A = pool<char>("gs_A", abytes + 1024), *B = pool<char>("gs_B", bbytes + 1024);
  int *EA = pool<int>("gs_ea", ea + 1), *EB = pool<int>("gs_eb", eb + 1);
  unsigned long long *MA = pool<unsigned long long>("gs_ma", ea + 1),
                     *MB = pool<unsigned long long>("gs_mb", eb + 1);
  for (size_t i = 0; i < probs.size(); ++i) {
    sa[i].dst = A + (long long)sa[i].dst; sa[i].expo = EA + (long long)sa[i].expo;
    sb[i].dst = B + (long long)sb[i].dst; sb[i].expo = EB + (long long)sb[i].expo;
    sa[i].mbits = MA + (long long)sa[i].mbits; sb[i].mbits = MB + (long long)sb[i].mbits;
    tc[i].a_planes = (const char *)sa[i].dst; tc[i].b_planes = (const char *)sb[i].dst;
    tc[i].ea = sa[i].expo; tc[i].eb = sb[i].expo;
  }
  SplitProb *dsa = pool<SplitProb>("gs_sa", sa.size()), *dsb = pool<SplitProb>("gs_sb", sb.size());
  TcProb *dtc = pool<TcProb>("gs_tc", tc.size());
  // tile -> product table for the persistent product kernel
  std::vector<int> tp(tiles);
  for (size_t i = 0; i < tc.size(); ++i) {
    const int nt = ((probs[i].M + TM - 1) / TM) * ((probs[i].N + TN - 1) / TN);
    for (int k = 0; k < nt; ++k) tp[tc[i].tile0 + k] = (int)i;
  }
  int *dtp = pool<int>("gs_tp", tp.size());
  stage_h2d(dsa, sa.data(), sa.size() * sizeof(SplitProb), st);
  stage_h2d(dsb, sb.data(), sb.size() * sizeof(SplitProb), st);
  stage_h2d(dtc, tc.data(), tc.size() * sizeof(TcProb), st);
  stage_h2d(dtp, tp.data(), tp.size() * sizeof(int), st);
  // operands of one k chunk (the DC's small products) take their maxima in
  // the digit kernels; the maxima pass (zeroed, then atomicMax) only runs when
  // some operand has several chunks.  Operands with K = 0 have no work item and
  // an unwritten exponent, which their all-zero sums never use.
  if (multi) {
    cudaMemsetAsync(MA, 0, sizeof(unsigned long long) * (ea + 1), st);
    cudaMemsetAsync(MB, 0, sizeof(unsigned long long) * (eb + 1), st);
    if (wa > 0) k_split_amax<<<(unsigned)wa, 256, 0, st>>>(dsa, (int)sa.size());
    if (wb > 0) k_split_bmax<<<(unsigned)wb, 256, 0, st>>>(dsb, (int)sb.size());
  }
  if (wa > 0) k_split_a<<<(unsigned)wa, 256, 0, st>>>(dsa, (int)sa.size());
  if (wb > 0) k_split_b<<<(unsigned)wb, 256, 0, st>>>(dsb, (int)sb.size());
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_TC);
    attr = true;
  }
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  k_gemm_tc<<<std::min(tiles, sms), GTH, SMEM_TC, st>>>(dtc, dtp, tiles, d_err);
}


void launch_gemm_fused(const std::vector<GemmDesc> &probs, int *d_err, cudaStream_t st) {
  if (probs.empty()) return;
  std::vector<ExpJob> rj, cj;
  std::vector<FusedProb> fp;
  int rows = 0, cols = 0, tiles = 0;
  for (const auto &p : probs) {
    rj.push_back({p.A, p.lda, p.M, p.K, nullptr, rows});
    cj.push_back({p.B, p.ldb, p.N, p.K, nullptr, cols});
    FusedProb f{p.A, p.B, p.C, nullptr, nullptr, p.lda, p.ldb, p.ldc, p.M, p.N, p.K, p.beta, tiles};
    fp.push_back(f);
    rows += p.M;
    cols += p.N;
    tiles += ((p.M + FM - 1) / FM) * ((p.N + FN - 1) / FN);
  }
  int *EA = pool<int>("gf_ea", rows + 1), *EB = pool<int>("gf_eb", cols + 1);
  for (size_t i = 0; i < probs.size(); ++i) {
    rj[i].out = EA + rj[i].off; cj[i].out = EB + cj[i].off;
    fp[i].ea = rj[i].out; fp[i].eb = cj[i].out;
  }
  ExpJob *drj = pool<ExpJob>("gf_rj", rj.size()), *dcj = pool<ExpJob>("gf_cj", cj.size());
  FusedProb *dfp = pool<FusedProb>("gf_fp", fp.size());
  stage_h2d(drj, rj.data(), rj.size() * sizeof(ExpJob), st);
  stage_h2d(dcj, cj.data(), cj.size() * sizeof(ExpJob), st);
  stage_h2d(dfp, fp.data(), fp.size() * sizeof(FusedProb), st);
  k_row_exps<<<(rows + 255) / 256, 256, 0, st>>>(drj, (int)rj.size(), rows);
  k_col_exps<<<(unsigned)(((long long)cols * 32 + 255) / 256), 256, 0, st>>>(dcj, (int)cj.size(), cols);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gemm_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, FSMEM);
    attr = true;
  }
  k_gemm_fused<<<tiles, 128, FSMEM, st>>>(dfp, (int)fp.size(), d_err);
}

}  // namespace hss
