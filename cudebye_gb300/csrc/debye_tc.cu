// debye_tc.cu — tensor-core Debye contraction on sm_103a (tcgen05 + TMEM).
//
// The reference sums, per species pair and per q (debyeRowSum,
// cuDebye-v15.cu:493-538),
//     S(q) = sum_k m_k sin(q r_k)/(q r_k),   r_k = k*rstep,
// with m_k = 2 n_k off the self distance (r_k > 0.0005) and n_k on it.
// Here the non-self part is rewritten as q*S'(q) = sum_k w_k sin(q r_k) with
// w_k = m_k / r_k = (2 / rstep) n_k / k, and the bins are cut into chunks of
// L = 256:
// k = k0 + j, k0 = ch*L, so sin(q r_k) = sin(q k0 dr) cos(q j dr)
//                                       + cos(q k0 dr) sin(q j dr).
// The j-basis [cos(q j dr) | sin(q j dr)] is the same for every chunk, so
// the sum becomes one real GEMM
//     D[row, n] = sum_j Basis[row, j] * W[n, j],   n = (pair, chunk)
// (rows: Qp cosine rows then Qp sine rows), followed by an epilogue that
// rotates each chunk by its twiddle (sin(q k0 dr) for cosine rows,
// cos(q k0 dr) for sine rows) and sums the chunks of a pair.
//
// Precision (<= 1e-6 relative on the intensity vs FP64): both operands are
// fixed-point integers split into four balanced base-256 digits, exact in
// bf16 (|digit| <= 128). Digit products are exact integers and a K = 256
// dot product of up to four digit pairs stays within 2^24, so the FP32
// tensor-core accumulation is error-free. The digit pairs with s + t <= 3
// (10 of 16) are accumulated into four TMEM accumulators by weight class;
// the epilogue recombines them exactly into a double-float, applies the
// per-chunk scale, the twiddle (double-float) and the chunk sum, and the
// pair and q sums run in FP64.
//
// Kernel shape: tiles of 128 rows x 64 columns, K = 256 in four slabs of 64
// stored pre-tiled in global memory in the canonical no-swizzle K-major
// core-matrix layout, so each slab is two contiguous bulk copies (TMA
// engine, cp.async.bulk) completing on an mbarrier. A persistent CTA per SM
// runs three roles: a producer thread streams slabs through two stages, an
// MMA thread issues tcgen05.mma (kind::f16, bf16 x bf16 -> f32, M=128,
// K=16) into one of two TMEM accumulator sets (4 classes x 64 f32 columns
// each) and commits, four epilogue warps drain the other set. One MMA
// multiplies digit s of A by all W digits t <= 3 - s at once (N = 256, 192,
// 128, 64): W's digit blocks lie one after another along N, and the classes
// one after another in TMEM, so product (s, t) lands in class s + t — four
// MMAs per K step instead of ten, and A read from shared memory once per
// digit.
// Every wait is bounded and reports a timeout through an error word.
//
// Two comparison forms share the kernel: BF16x3 (two 8-bit digits per
// operand, products (0,0), (0,1), (1,0)) and TF32x3: each operand's
// fixed-point value x is split into tf32 parts hi = tf32(x), lo =
// tf32(x - hi) (22 significant bits together), stored as fp32 in the same
// slab bytes (two 32-bit parts take the room of four 16-bit digits), and
// multiplied with tcgen05.mma kind::tf32 (K = 8) as hi*hi into one
// accumulator and hi*lo + lo*hi into another, with FP32 accumulation over
// the chunk's 256 bins; the lo*lo term and the FP32 rounding of the sums are
// its error. Neither form is exact; the exact split is the default.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "debye_tc.h"

namespace dbx {
namespace tc {

constexpr int kL = 256;             // bins per chunk = GEMM K
constexpr int kKS = 64;             // K per shared-memory slab
constexpr int kNSlab = kL / kKS;    // 4
constexpr int kTM = 128;            // rows per tile
constexpr int kTN = 64;             // columns (chunks) per tile
constexpr int kND = 4;              // digits per operand
constexpr int kABlock = kTM * kKS;  // elements per digit per slab (16 KB)
constexpr int kBBlock = kTN * kKS;  // 8 KB
constexpr int kASlabBytes = kND * kABlock * 2;  // 64 KB
constexpr int kBSlabBytes = kND * kBBlock * 2;  // 32 KB
constexpr int kTmemCols = 256;      // 4 classes x 64 columns
constexpr double kSelfR = 0.0005;   // cuDebye-v15.cu:508
// TF32 operands: two fp32 parts per value in the bytes of four bf16 digits.
constexpr int kNP32 = 2;
static_assert(kNP32 * kABlock * 4 == kASlabBytes, "tf32 A parts fill the slab");
static_assert(kNP32 * kBBlock * 4 == kBSlabBytes, "tf32 W parts fill the slab");

// Operand forms of the contraction (TcState::form).
constexpr int kFormExact = 0;   // 4 bf16 digits, 10 products: exact
constexpr int kFormBf16x3 = 1;  // 2 bf16 digits, 3 products
constexpr int kFormTf32x3 = 2;  // 2 tf32 parts, 3 products
__host__ __device__ constexpr int form_classes(int f) { return f == kFormExact ? 4 : 2; }
__host__ __device__ constexpr bool form_tf32(int f) { return f == kFormTf32x3; }

// Element offset of (row, k) inside a [rows x kKS] block stored as 8x8
// core matrices (8 rows x 16 bytes each, contiguous), row groups outermost:
// core (g, kc) at (g*kKS/8 + kc)*64 elements. Leading (K) byte offset 128,
// stride (row-group) byte offset kKS*16.
__host__ __device__ inline int tiled_off(int row, int k) {
  return (((row >> 3) * (kKS / 8) + (k >> 3)) << 6) + ((row & 7) << 3) + (k & 7);
}

// The same for 32-bit elements (8 rows x 4 elements per core matrix): core
// (g, kc) at (g*kKS/4 + kc)*32 elements. Leading byte offset 128, stride
// byte offset kKS*32.
__host__ __device__ inline int tiled_off32(int row, int k) {
  return (((row >> 3) * (kKS / 4) + (k >> 2)) << 5) + ((row & 7) << 2) + (k & 3);
}

// Nearest tf32 (10 explicit mantissa bits; ties away from zero) of a
// finite float: the tensor core reads only those bits of an fp32 operand.
__device__ inline float tf32_rn(float f) {
  return __uint_as_float((__float_as_uint(f) + 0x1000u) & 0xFFFFE000u);
}

// tf32 parts of the fixed-point value v 2^-24 (|v| < 2^31): hi + lo equals
// it to about 2^-22 relative. The scale 2^-24 makes the products' sums
// carry the weight of the exact form's top digit pair (2^48 over the
// product of two 31-bit fixed-point values), so the epilogue is shared.
__device__ inline void split_tf32(long long v, float &hi, float &lo) {
  const double x = (double)v * 0x1p-24;  // exact
  hi = tf32_rn((float)x);
  lo = tf32_rn((float)(x - (double)hi));
}

// Balanced base-256 digits of v, |v| <= 2^31 - 1, most significant first:
// v = d0*2^24 + d1*2^16 + d2*2^8 + d3, |d| <= 128.
__device__ inline void split4(long long v, float d[4]) {
  const int d3 = (int)(((v + 128) & 255) - 128);
  v = (v - d3) >> 8;
  const int d2 = (int)(((v + 128) & 255) - 128);
  v = (v - d2) >> 8;
  const int d1 = (int)(((v + 128) & 255) - 128);
  v = (v - d1) >> 8;
  d[0] = (float)v;
  d[1] = (float)d1;
  d[2] = (float)d2;
  d[3] = (float)d3;
}

__device__ inline long long fixed31(double v) {
  long long r = llrint(v * 2147483648.0);
  return r > 2147483647LL ? 2147483647LL : (r < -2147483647LL ? -2147483647LL : r);
}

// The basis and twiddle angles advance by a fixed step (dr or L dr per
// element), so each thread evaluates sincos (FP64, slow on this part) at
// the first of a run of kRun elements and at the step, and advances by
// rotation (two FP64 products and an FMA per component); the rotations
// add a few ulp over a run, far below the 2^-31 fixed-point resolution of
// the basis and the double-float twiddles' 2^-48.
constexpr int kRun = 16;

// Basis digits: rows [0,Qp) cos(K_q j dr), rows [Qp,2Qp) sin(K_q j dr).
// Layout: [row tile][slab][digit][tiled 128 x 64]. One thread per row and
// run of kRun columns; eight columns of a digit are one 16-byte store.
// TF32: [row tile][slab][part][tiled32 128 x 64] fp32, four columns of a
// part per 16-byte store.
template <bool TF32>
__global__ void basis_kernel(const double *__restrict__ K, int nq, int Qp,
                             double rstep, __nv_bfloat16 *__restrict__ A) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 2LL * Qp * (kL / kRun)) return;
  const int m = (int)(idx % (2 * Qp));
  const int j0 = (int)(idx / (2 * Qp)) * kRun;
  const bool sinrow = m >= Qp;
  const int q = sinrow ? m - Qp : m;
  double s = 0.0, c = 0.0, ss = 0.0, cs = 1.0;
  if (q < nq) {
    sincos(K[q] * ((double)j0 * rstep), &s, &c);
    sincos(K[q] * rstep, &ss, &cs);
  }
  const int mt = m / kTM, row = m % kTM;
  if (TF32) {
    float *A32 = reinterpret_cast<float *>(A);
#pragma unroll
    for (int g = 0; g < kRun; g += 4) {
      alignas(16) float part[kNP32][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        split_tf32(fixed31(sinrow ? s : c), part[0][i], part[1][i]);
        const double s2 = fma(s, cs, c * ss), c2 = fma(c, cs, -(s * ss));
        s = s2;
        c = c2;
      }
      const int j = j0 + g, ks = j / kKS, k = j % kKS;
      const size_t base =
          (size_t)(mt * kNSlab + ks) * kNP32 * kABlock + tiled_off32(row, k);
#pragma unroll
      for (int t = 0; t < kNP32; ++t)
        *reinterpret_cast<float4 *>(A32 + base + (size_t)t * kABlock) =
            *reinterpret_cast<const float4 *>(part[t]);
    }
    return;
  }
#pragma unroll
  for (int g = 0; g < kRun; g += 8) {
    alignas(16) __nv_bfloat16 dig[kND][8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float d[4];
      split4(fixed31(sinrow ? s : c), d);
#pragma unroll
      for (int t = 0; t < kND; ++t) dig[t][i] = __float2bfloat16_rn(d[t]);
      const double s2 = fma(s, cs, c * ss), c2 = fma(c, cs, -(s * ss));
      s = s2;
      c = c2;
    }
    const int j = j0 + g, ks = j / kKS, k = j % kKS;
    const size_t base = (size_t)(mt * kNSlab + ks) * kND * kABlock + tiled_off(row, k);
#pragma unroll
    for (int t = 0; t < kND; ++t)
      *reinterpret_cast<uint4 *>(A + base + (size_t)t * kABlock) =
          *reinterpret_cast<const uint4 *>(dig[t]);
  }
}

// Twiddles per (chunk, q): alpha = K_q * ch*L*dr, as double-floats in two
// planes: tw[ch*Qp + q] = (sin hi, sin lo), tw[(nch + ch)*Qp + q] = (cos hi,
// cos lo) (a cosine row of the contraction reads only the sine plane, a
// sine row only the cosine plane). One thread per q and run of kRun chunks.
__global__ void twiddle_kernel(const double *__restrict__ K, int nq, int Qp,
                               int nch, double rstep, float2 *__restrict__ tw) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)(nch / kRun) * Qp) return;
  const int q = (int)(idx % Qp);
  const int ch0 = (int)(idx / Qp) * kRun;
  double s = 0.0, c = 1.0, ss = 0.0, cs = 1.0;
  if (q < nq) {
    sincos(K[q] * ((double)ch0 * kL * rstep), &s, &c);
    sincos(K[q] * ((double)kL * rstep), &ss, &cs);
  }
#pragma unroll 4
  for (int i = 0; i < kRun; ++i) {
    const float sh = (float)s, ch_ = (float)c;
    tw[(size_t)(ch0 + i) * Qp + q] = make_float2(sh, (float)(s - (double)sh));
    tw[(size_t)(nch + ch0 + i) * Qp + q] = make_float2(ch_, (float)(c - (double)ch_));
    const double s2 = fma(s, cs, c * ss), c2 = fma(c, cs, -(s * ss));
    s = s2;
    c = c2;
  }
}

// Chunk weights as digits, one warp per (tile, column). The weight of bin
// k is w_k = m_k / r_k = (2 / rstep) (n_k / k) off the self distance
// (k >= kself, the first bin with k rstep > 0.0005); the common factor
// 2 / rstep is applied to the column sums (reduce_kernel), so the digits
// hold u_k = n_k / k, computed in integers: fixed31(u_k 2^-e) =
// round(n_k 2^(31-e) / k), with e the chunk's scale exponent (every
// u_k < 2^e). No FP64 arithmetic (slow on this part) is needed.
// Layout of W: [col tile][slab][digit][tiled 64 x 64]; E: per column,
// the chunk's scale exponent. TF32: [col tile][slab][part][tiled32 64 x 64]
// fp32 parts of the same fixed-point values.
template <bool TF32>
__global__ void weights_kernel(const TcTile *__restrict__ tiles, int ntiles,
                               const TcCol *__restrict__ cols, long long kself,
                               __nv_bfloat16 *__restrict__ W,
                               int *__restrict__ E,
                               int *__restrict__ nonself) {
  const int gw = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  const int nt = gw / kTN, n = gw % kTN;
  if (nt >= ntiles) return;
  const TcTile t = tiles[nt];
  const TcCol col = cols[t.col];
  const int ch = t.ch0 + n;
  unsigned long long cnt[8];
  float mx = 0.f;
  bool any = false;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const long long k = (long long)ch * kL + lane * 8 + i;
    unsigned long long c = 0;
    if (k < col.nbins && k >= kself && k > 0) c = col.hist[k];
    cnt[i] = c;
    any |= c != 0;
    if (c) mx = fmaxf(mx, (float)c / (float)k);  // estimate of u_k
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  any = __any_sync(0xffffffffu, any);
  int e = 0;
  if (any) {
    frexpf(mx, &e);  // mx < 2^e; exact check below, u_k < 2^e
    bool over = false;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const unsigned long long k = (unsigned long long)ch * kL + lane * 8 + i;
      // n >= k 2^e, exactly: floor(n / 2^e) >= k, or n 2^-e >= k for e < 0
      // (then n < k < 2^22, no overflow)
      if (cnt[i] && e < 64) over |= e >= 0 ? (cnt[i] >> e) >= k : (cnt[i] << -e) >= k;
    }
    if (__any_sync(0xffffffffu, over)) ++e;
  }
  const int j0 = lane * 8, ks = j0 / kKS, k0 = j0 % kKS;
  long long fx[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    long long f = 0;
    if (cnt[i]) {
      const unsigned long long k = (unsigned long long)ch * kL + lane * 8 + i;
      // n 2^(31-e) / k rounded; n < k 2^e keeps every operand below 2^53
      const unsigned long long num = e <= 31 ? cnt[i] << (31 - e) : cnt[i];
      const unsigned long long den = e <= 31 ? k : k << (e - 31);
      f = (long long)((num + den / 2) / den);
      f = f > 2147483647LL ? 2147483647LL : f;
    }
    fx[i] = f;
  }
  if (TF32) {
    float *W32 = reinterpret_cast<float *>(W);
    const size_t base = (size_t)(nt * kNSlab + ks) * kNP32 * kBBlock;
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // columns k0 + 4h .. k0 + 4h + 3
      alignas(16) float part[kNP32][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) split_tf32(fx[4 * h + i], part[0][i], part[1][i]);
#pragma unroll
      for (int t = 0; t < kNP32; ++t)
        *reinterpret_cast<float4 *>(W32 + base + (size_t)t * kBBlock +
                                    tiled_off32(n, k0 + 4 * h)) =
            *reinterpret_cast<const float4 *>(part[t]);
    }
  } else {
    const size_t base = (size_t)(nt * kNSlab + ks) * kND * kBBlock + tiled_off(n, k0);
    alignas(16) __nv_bfloat16 dig[kND][8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float d[4];
      split4(fx[i], d);
#pragma unroll
      for (int s = 0; s < kND; ++s) dig[s][i] = __float2bfloat16_rn(d[s]);
    }
#pragma unroll
    for (int s = 0; s < kND; ++s)
      *reinterpret_cast<uint4 *>(W + base + (size_t)s * kBBlock) =
          *reinterpret_cast<const uint4 *>(dig[s]);
  }
  if (lane == 0) {
    E[nt * kTN + n] = e;
    if (any) atomicOr(&nonself[t.col], 1);
  }
}

// ---- PTX helpers ------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  // Bounded wait: ~2^22 polls (seconds at most), then report a timeout.
  for (int it = 0; it < (1 << 22); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo,
                                              uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, no swizzle
}

// Instruction descriptor of kind::f16 (A/B bf16: format 1) or kind::tf32
// (A/B tf32: format 2): D f32, both operands K-major, M x N.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N, bool tf32 = false) {
  return (1u << 4) | ((tf32 ? 2u : 1u) << 7) | ((tf32 ? 2u : 1u) << 10) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t ad,
                                         uint64_t bd, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t ad,
                                         uint64_t bd, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,"
      "%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
        "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// Completes all prior tcgen05.ld of this thread. The loaded registers are
// passed through as in/out operands so that the compiler cannot use them
// before the wait.
__device__ __forceinline__ void tmem_wait16(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]),
                 "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]),
                 "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
                 "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

// ---- persistent, warp-specialised contraction ------------------------------
// One CTA per SM loops over tiles t = blockIdx.x + i * gridDim.x (row tile
// t % nrt, column tile t / nrt). Roles: warp 0 lane 0 streams the slabs of
// A and W through kPStages shared-memory stages (bulk copies on the TMA
// engine); warp 1 lane 0 issues the MMAs of a tile into one of two TMEM
// accumulator sets (2 x 256 columns); warps 4-7 (TMEM lanes 0-127) run the
// epilogue of the previous tile meanwhile. mbarriers: full[s] (copy landed),
// empty[s] (MMAs on stage s done), accf[b] (accumulator set b complete),
// acce[b] (set b drained by the epilogue). Every wait is bounded; a role that
// times out records the error and stops, and the others then time out too.
constexpr int kPThreads = 256;
constexpr int kPStageBytes = kASlabBytes + kBSlabBytes;
constexpr int kPStages = (192 * 1024) / kPStageBytes;  // 192 KB of stages
constexpr int kPSmemBytes = kPStages * kPStageBytes + 1024 + 256;

// Epilogue of one tile for TMEM lane `row` (0..127) of accumulator set at
// column offset acc_col: D = acc0 + acc1 2^-8 + acc2 2^-16 + acc3 2^-24,
// scaled, rotated by the chunk twiddle and summed over the tile's 64 chunks.
// The twiddle loads are the epilogue's long-latency step: the first group's
// 16 are issued before the thread waits for the tile's accumulators
// (epi_start), and each next group's while the current one is summed. The
// chunks' scale exponents are read once per tile, two per lane, and passed
// around by shuffles.
struct EpiTile {
  const float2 *twq;  // this row's twiddle plane, at chunk 0 of the grid
  int ch0;            // the tile's first chunk
  int e_lo, e_hi;     // scale exponents of chunks lane and lane + 32
  float2 t[16];       // twiddles of the next group to sum
};

__device__ __forceinline__ void epi_start(EpiTile &et, int row, int mt, int nt,
                                          const TcTile *__restrict__ tiles,
                                          const int *__restrict__ Ecol,
                                          const float2 *__restrict__ tw, int Qp,
                                          int nchc, int lane) {
  const int m = mt * kTM + row;
  const bool sinrow = m >= Qp;
  const int q = sinrow ? m - Qp : m;
  // cosine rows are rotated by sin(q k0 dr), sine rows by cos(q k0 dr)
  et.twq = tw + (sinrow ? (size_t)nchc * Qp : 0) + q;
  et.ch0 = __ldg(&tiles[nt].ch0);
  et.e_lo = __ldg(&Ecol[nt * kTN + lane]);
  et.e_hi = __ldg(&Ecol[nt * kTN + 32 + lane]);
#pragma unroll
  for (int i = 0; i < 16; ++i) et.t[i] = __ldg(&et.twq[(size_t)(et.ch0 + i) * Qp]);
}

// (h, l) += (p, pe): double-float accumulation with an exact two-sum of
// the leading parts.
__device__ __forceinline__ void dd_add(float &h, float &l, float p, float pe) {
  const float s = h + p;
  const float bb = s - h;
  const float e2 = (h - (s - bb)) + (p - bb);
  l += e2 + pe;
  h = s + l;
  l = l - (h - s);
}

template <int FORM>
__device__ __forceinline__ double tile_epilogue(uint32_t lane_base, EpiTile &et,
                                                int Qp) {
  constexpr int NCLS = form_classes(FORM);
  // weight of accumulator 1 against accumulator 0: one base-256 digit, or
  // none for the tf32 parts (hi*lo + lo*hi carry hi*hi's scale)
  constexpr float kC1 = form_tf32(FORM) ? 1.0f : 0x1p-8f;
  // two running sums (even and odd chunks) halve the dependent chain of
  // additions per tile; they are joined once at the end
  float sh[2] = {0.f, 0.f}, sl[2] = {0.f, 0.f};
#pragma unroll 1
  for (int cg = 0; cg < kTN / 16; ++cg) {
    uint32_t a0[16], a1[16], a2[16] = {}, a3[16] = {};
    tmem_ld16(lane_base + 0 * kTN + cg * 16, a0);
    tmem_ld16(lane_base + 1 * kTN + cg * 16, a1);
    if (NCLS > 2) {
      tmem_ld16(lane_base + 2 * kTN + cg * 16, a2);
      tmem_ld16(lane_base + 3 * kTN + cg * 16, a3);
    }
    float2 tc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) tc[i] = et.t[i];
    if (cg + 1 < kTN / 16) {  // the next group's twiddles, in flight meanwhile
#pragma unroll
      for (int i = 0; i < 16; ++i)
        et.t[i] = __ldg(&et.twq[(size_t)(et.ch0 + (cg + 1) * 16 + i) * Qp]);
    }
    tmem_wait16(a0);
    tmem_wait16(a1);
    if (NCLS > 2) {
      tmem_wait16(a2);
      tmem_wait16(a3);
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int n = cg * 16 + i;
      // exact two-sum of the top two classes, the rest rounded once
      const float c0 = __uint_as_float(a0[i]);
      const float c1 = __uint_as_float(a1[i]) * kC1;
      const float hi = c0 + c1;
      const float hb = hi - c0;
      const float lo = ((c0 - (hi - hb)) + (c1 - hb)) +
                       fmaf(__uint_as_float(a2[i]), 0x1p-16f,
                            __uint_as_float(a3[i]) * 0x1p-24f);
      const float th = tc[i].x, tl = tc[i].y;
      // (th + tl) * (hi + lo) as a double-float, scaled by 2^(E-14)
      float p = th * hi;
      float pe = fmaf(th, hi, -p);
      pe = fmaf(th, lo, fmaf(tl, hi, pe));
      const int e = __shfl_sync(0xffffffffu, n < 32 ? et.e_lo : et.e_hi, n & 31);
      const float sc = __int_as_float((e - 14 + 127) << 23);
      dd_add(sh[i & 1], sl[i & 1], p * sc, pe * sc);
    }
  }
  dd_add(sh[0], sl[0], sh[1], sl[1]);
  return (double)sh[0] + (double)sl[0];
}

// FORM kFormExact: the exact form (digit pairs with s + t <= 3, four
// accumulators). kFormBf16x3: only the pairs (0,0), (0,1), (1,0) — two 8-bit
// digits per operand and three products. kFormTf32x3: the same three
// products of tf32 parts (kind::tf32, K = 8). The last two are kept for
// precision comparisons.
template <int FORM>
__global__ void __launch_bounds__(kPThreads, 1)
    gemm_persistent_kernel(const __nv_bfloat16 *__restrict__ A,
                           const __nv_bfloat16 *__restrict__ W,
                           const TcTile *__restrict__ tiles,
                           const int *__restrict__ Ecol,
                           const float2 *__restrict__ tw, int Qp, int nchc,
                           int nrt, int ntiles, double *__restrict__ P,
                           int *__restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t *sbase = smem_raw + (base - raw);
  uint64_t *bars = reinterpret_cast<uint64_t *>(sbase + kPStages * kPStageBytes);
  // bars: full[kPStages], empty[kPStages], accf[2], acce[2]
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2 * kPStages + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  auto bar = [&](int i) { return smem_u32(&bars[i]); };
  const int FULL = 0, EMPTY = kPStages, ACCF = 2 * kPStages, ACCE = 2 * kPStages + 2;
  if (tid == 0) {
    for (int i = 0; i < 2 * kPStages + 2; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar(i)));
    for (int b = 0; b < 2; ++b)  // one arrival per epilogue warp
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(bar(ACCE + b)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
            smem_u32(tslot)),
        "r"(2 * kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tslot;
  const int total = nrt * ntiles;

  if (warp == 0 && lane == 0) {
    // producer
    int it = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
      const int mt = t % nrt, nt = t / nrt;
      const char *gA = reinterpret_cast<const char *>(A) +
                       (size_t)mt * kNSlab * kASlabBytes;
      const char *gW = reinterpret_cast<const char *>(W) +
                       (size_t)nt * kNSlab * kBSlabBytes;
      for (int ks = 0; ks < kNSlab; ++ks, ++it) {
        const int st = it % kPStages, use = it / kPStages;
        if (use > 0 && !mbar_wait(bar(EMPTY + st), (use - 1) & 1)) {
          ok = false;
          break;
        }
        const uint32_t sA = base + st * kPStageBytes, sB = sA + kASlabBytes;
        asm volatile(
            "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                bar(FULL + st)),
            "r"(kPStageBytes)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1], %2, [%3];" ::"r"(sA),
            "l"(gA + (size_t)ks * kASlabBytes), "r"(kASlabBytes), "r"(bar(FULL + st))
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1], %2, [%3];" ::"r"(sB),
            "l"(gW + (size_t)ks * kBSlabBytes), "r"(kBSlabBytes), "r"(bar(FULL + st))
            : "memory");
      }
    }
    if (!ok) atomicExch(err, 1);
    // let the copies still in flight land before the CTA can exit
    for (int k = it > kPStages ? it - kPStages : 0; k < it; ++k)
      mbar_wait(bar(FULL + k % kPStages), (k / kPStages) & 1);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr int NCLS = form_classes(FORM);
    constexpr bool TF32 = form_tf32(FORM);
    // bytes of one digit (part) block of A, and the MMA K step: 16 bf16 or
    // 8 tf32 elements, two core matrices (256 bytes) either way
    constexpr int kAPart = TF32 ? kABlock * 4 : kABlock * 2;
    constexpr int kSteps = TF32 ? kKS / 8 : kKS / 16;
    constexpr uint32_t kSbo = TF32 ? kKS * 32 : kKS * 16;
    int it = 0, tc = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < total && ok; t += gridDim.x, ++tc) {
      const int b = tc & 1, ub = tc >> 1;
      if (ub > 0 && !mbar_wait(bar(ACCE + b), (ub - 1) & 1)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t acc_base = tmem + b * kTmemCols;
      for (int ks = 0; ks < kNSlab; ++ks, ++it) {
        const int st = it % kPStages, use = it / kPStages;
        if (!mbar_wait(bar(FULL + st), use & 1)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t sA = base + st * kPStageBytes, sB = sA + kASlabBytes;
        // descriptors of the stage's first core matrices; the others differ
        // in the start-address field only (16-byte units, no carry out of
        // the field: shared addresses are below 256 KB), so each MMA needs
        // one add per operand instead of a descriptor build (the single
        // issuing thread limited the MMA rate)
        const uint64_t adb = make_desc(sA, 128, kSbo), bdb = make_desc(sB, 128, kSbo);
#pragma unroll
        for (int s = 0; s < NCLS; ++s) {
          // digit s of A against digits 0 .. NCLS-1-s of W in one MMA: the
          // W digit blocks follow one another along N with the same 8-row
          // stride, so N = (NCLS - s) * 64 columns read them all, and with
          // D at class s the block of digit t lands in class s + t
          const uint32_t idn = make_idesc(kTM, (NCLS - s) * kTN, TF32);
#pragma unroll
          for (int kk = 0; kk < kSteps; ++kk) {
            const uint64_t ad = adb + (uint64_t)((s * kAPart + kk * 256) >> 4);
            const uint64_t bd = bdb + (uint64_t)((kk * 256) >> 4);
            // the first MMA of a tile spans every class and starts them all
            const uint32_t acc = (ks > 0 || s > 0 || kk > 0) ? 1u : 0u;
            if (TF32)
              mma_tf32(acc_base + s * kTN, ad, bd, idn, acc);
            else
              mma_bf16(acc_base + s * kTN, ad, bd, idn, acc);
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
            "[%0];" ::"r"(bar(EMPTY + st))
            : "memory");
      }
      if (!ok) break;
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
          "[%0];" ::"r"(bar(ACCF + b))
          : "memory");
    }
    if (!ok) atomicExch(err, 1);
    // the MMAs issued so far finish before the CTA can exit
    if (it > 0) {
      const int k = it - 1;
      mbar_wait(bar(EMPTY + k % kPStages), (k / kPStages) & 1);
    }
  } else if (warp >= 4) {
    // epilogue: warp 4 + i reads TMEM lanes 32 i .. 32 i + 31
    const int row = (warp - 4) * 32 + lane;
    int tc = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x, ++tc) {
      const int b = tc & 1, ub = tc >> 1;
      const int mt = t % nrt, nt = t / nrt;
      EpiTile et;  // the first twiddles load while the MMAs run
      epi_start(et, row, mt, nt, tiles, Ecol, tw, Qp, nchc, lane);
      if (!mbar_wait(bar(ACCF + b), ub & 1)) {
        atomicExch(err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t lane_base =
          tmem + b * kTmemCols + ((uint32_t)((warp - 4) * 32) << 16);
      P[(size_t)nt * (2 * Qp) + mt * kTM + row] =
          tile_epilogue<FORM>(lane_base, et, Qp);
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar(ACCE + b))
                     : "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile(
        "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
        "r"(2 * kTmemCols));
}

// I[model][q] = sum over the model's columns (pair order) of
// ff[q] * (self + (2 / rstep) (sum of the column's tiles of P over both
// row halves) / K).
__global__ void reduce_kernel(const TcCol *__restrict__ cols, int ncols,
                              const int *__restrict__ model_col_begin,
                              int nmodels, const double *__restrict__ P,
                              const int *__restrict__ nonself,
                              const double *__restrict__ K, int nq, int Qp,
                              double wscale, double *__restrict__ I,
                              double *__restrict__ S_out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int mod = blockIdx.y;
  if (q >= nq || mod >= nmodels) return;
  const double Kq = K[q];
  double acc = 0.0;
  for (int c = model_col_begin[mod]; c < model_col_begin[mod + 1]; ++c) {
    const TcCol col = cols[c];
    double t = 0.0;
    for (int nt = col.tile_begin; nt < col.tile_end; ++nt)
      t += P[(size_t)nt * (2 * Qp) + q] + P[(size_t)nt * (2 * Qp) + Qp + q];
    double S;
    if (Kq == 0.0)  // sin(0)/0 of the reference (cuDebye-v15.cu:509)
      S = nonself[c] ? __longlong_as_double(0x7ff8000000000000LL) : col.self;
    else
      S = col.self + (t * wscale) / Kq;  // wscale = 2 / rstep
    if (S_out) S_out[(size_t)c * nq + q] = S;
    acc += S * col.ff[q];
  }
  I[(size_t)mod * nq + q] = acc;
}

// I[q] = sum over the columns of ff[c][q] * S[c][q], in column order: the
// same arithmetic as reduce_kernel's last step, for re-scoring resident row
// sums with new prefactors.
__global__ void combine_kernel(const double *__restrict__ ff,
                               const double *__restrict__ S, int ncols, int nq,
                               double *__restrict__ I) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double acc = 0.0;
  for (int c = 0; c < ncols; ++c) acc += S[(size_t)c * nq + q] * ff[(size_t)c * nq + q];
  I[q] = acc;
}

// Self-distance sum of each column: bins with r <= 0.0005 (m = n there).
__global__ void self_kernel(TcCol *cols, int ncols, double rstep) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  double s = 0.0;
  for (long long k = 0; k < cols[c].nbins && (double)k * rstep <= kSelfR; ++k)
    s += (double)cols[c].hist[k];
  cols[c].self = s;
}

}  // namespace tc

using namespace tc;

void tc_release(TcState *st) {
  for (DevBuf *b : {&st->basis, &st->twid, &st->W, &st->E, &st->P, &st->tiles,
                    &st->cols, &st->mcb, &st->nonself, &st->err})
    if (b->p) {
      cudaFree(b->p);
      b->p = nullptr;
      b->bytes = 0;
    }
  st->grid_K.clear();
}

size_t tc_bytes(const TcState *st) {
  size_t s = 0;
  for (const DevBuf *b : {&st->basis, &st->twid, &st->W, &st->E, &st->P,
                          &st->tiles, &st->cols, &st->mcb, &st->nonself, &st->err})
    s += b->bytes;
  return s;
}

Error tc_prepare(TcState *st, std::vector<TcCol> cols,
                 const std::vector<int> &model_col_begin, double rstep,
                 const double *h_K, const double *d_K, int nq,
                 cudaStream_t stream, size_t *delta) {
  const int ncols = (int)cols.size();
  const int nmodels = (int)model_col_begin.size() - 1;
  if (ncols == 0 || nq < 1) return fail(DBX_ERR_ARG, "empty Debye contraction");
  const int Qp = (nq + kTM - 1) / kTM * kTM;
  const int nrt = 2 * Qp / kTM;
  // Column tiles: each column (pair) gets ceil(nch/64) tiles of 64 chunks.
  std::vector<TcTile> tiles;
  int nch_max = 1;
  for (int c = 0; c < ncols; ++c) {
    const int nch = (int)((cols[c].nbins + kL - 1) / kL);
    nch_max = std::max(nch_max, nch);
    cols[c].tile_begin = (int)tiles.size();
    for (int ch0 = 0; ch0 < std::max(nch, 1); ch0 += kTN) tiles.push_back({c, ch0, 0, 0});
    cols[c].tile_end = (int)tiles.size();
  }
  const int nch_cap = (nch_max + kTN - 1) / kTN * kTN;  // twiddle rows
  const int ntiles = (int)tiles.size();
  // Plan data cached per (q grid, rstep, chunk count): basis and twiddles.
  const cudaStream_t as = st->alloc_stream;
  const bool tf32 = form_tf32(st->form);
  const bool same_grid = st->grid_K.size() == (size_t)nq && st->grid_rstep == rstep &&
                         st->grid_nch >= nch_cap && st->grid_tf32 == tf32 &&
                         std::memcmp(st->grid_K.data(), h_K, sizeof(double) * nq) == 0;
  DBX_TRY(buf_grow(&st->W, (size_t)ntiles * kNSlab * kBSlabBytes, delta, as));
  DBX_TRY(buf_grow(&st->E, sizeof(int) * ntiles * kTN, delta, as));
  DBX_TRY(buf_grow(&st->P, sizeof(double) * ntiles * 2 * Qp, delta, as));
  DBX_TRY(buf_grow(&st->tiles, sizeof(TcTile) * ntiles, delta, as));
  DBX_TRY(buf_grow(&st->cols, sizeof(TcCol) * ncols, delta, as));
  DBX_TRY(buf_grow(&st->mcb, sizeof(int) * (nmodels + 1), delta, as));
  DBX_TRY(buf_grow(&st->nonself, sizeof(int) * ncols, delta, as));
  DBX_TRY(buf_grow(&st->err, sizeof(int), delta, as));
  if (!same_grid) {
    DBX_TRY(buf_grow(&st->basis, (size_t)nrt * kNSlab * kASlabBytes, delta, as));
    DBX_TRY(buf_grow(&st->twid, 2 * sizeof(float2) * (size_t)nch_cap * Qp, delta, as));
    const long long nb = 2LL * Qp * (kL / kRun);
    auto bk = tf32 ? basis_kernel<true> : basis_kernel<false>;
    bk<<<(unsigned)((nb + 255) / 256), 256, 0, stream>>>(
        d_K, nq, Qp, rstep, (__nv_bfloat16 *)st->basis.p);
    const long long nt2 = (long long)(nch_cap / kRun) * Qp;  // nch_cap: multiple of 64
    twiddle_kernel<<<(unsigned)((nt2 + 255) / 256), 256, 0, stream>>>(
        d_K, nq, Qp, nch_cap, rstep, (float2 *)st->twid.p);
    DBX_CUDA_TRY(cudaGetLastError());
    st->grid_K.assign(h_K, h_K + nq);
    st->grid_rstep = rstep;
    st->grid_nch = nch_cap;
    st->grid_tf32 = tf32;
  }
  DBX_TRY(h2d_copy(st->tiles.p, tiles.data(), sizeof(TcTile) * ntiles, stream,
                   st->arena));
  DBX_TRY(h2d_copy(st->cols.p, cols.data(), sizeof(TcCol) * ncols, stream, st->arena));
  DBX_TRY(h2d_copy(st->mcb.p, model_col_begin.data(), sizeof(int) * (nmodels + 1),
                   stream, st->arena));
  st->h2d += sizeof(TcTile) * ntiles + sizeof(TcCol) * ncols + sizeof(int) * (nmodels + 1);
  if (!st->num_sms) {  // first use of this state: kernel attributes, SMs
    for (auto k : {gemm_persistent_kernel<kFormExact>, gemm_persistent_kernel<kFormBf16x3>,
                   gemm_persistent_kernel<kFormTf32x3>})
      DBX_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kPSmemBytes));
    int dev = 0;
    DBX_CUDA_TRY(cudaGetDevice(&dev));
    DBX_CUDA_TRY(cudaDeviceGetAttribute(&st->num_sms, cudaDevAttrMultiProcessorCount, dev));
  }
  ++st->prep_gen;
  st->ncols = ncols;
  st->nmodels = nmodels;
  st->ntiles = ntiles;
  st->nq = nq;
  st->Qp = Qp;
  st->rstep = rstep;
  return ok();
}

Error tc_execute(TcState *st, const double *d_K, double *d_I,
                 cudaStream_t stream, Timers *tm) {
  const int ncols = st->ncols, ntiles = st->ntiles, nq = st->nq, Qp = st->Qp;
  const int nrt = 2 * Qp / kTM;
  DBX_CUDA_TRY(cudaMemsetAsync(st->nonself.p, 0, sizeof(int) * ncols, stream));
  DBX_CUDA_TRY(cudaMemsetAsync(st->err.p, 0, sizeof(int), stream));
  self_kernel<<<(ncols + 127) / 128, 128, 0, stream>>>((TcCol *)st->cols.p, ncols,
                                                       st->rstep);
  const long long nwarps = (long long)ntiles * kTN;
  long long kself = 0;  // first bin beyond the self distance
  while ((double)kself * st->rstep <= kSelfR) ++kself;
  auto wk = form_tf32(st->form) ? weights_kernel<true> : weights_kernel<false>;
  wk<<<(unsigned)((nwarps * 32 + 255) / 256), 256, 0, stream>>>(
      (const TcTile *)st->tiles.p, ntiles, (const TcCol *)st->cols.p, kself,
      (__nv_bfloat16 *)st->W.p, (int *)st->E.p, (int *)st->nonself.p);
  DBX_CUDA_TRY(cudaGetLastError());
  tm->start(DBX_T_DEBYE, stream);
  const int total = nrt * ntiles;
  auto kern = st->form == kFormTf32x3   ? gemm_persistent_kernel<kFormTf32x3>
              : st->form == kFormBf16x3 ? gemm_persistent_kernel<kFormBf16x3>
                                        : gemm_persistent_kernel<kFormExact>;
  kern<<<std::min(total, st->num_sms), kPThreads, kPSmemBytes, stream>>>(
      (const __nv_bfloat16 *)st->basis.p, (const __nv_bfloat16 *)st->W.p,
      (const TcTile *)st->tiles.p, (const int *)st->E.p, (const float2 *)st->twid.p,
      Qp, st->grid_nch, nrt, ntiles, (double *)st->P.p, (int *)st->err.p);
  DBX_CUDA_TRY(cudaGetLastError());
  tm->stop(DBX_T_DEBYE, stream);
  dim3 rg((nq + 127) / 128, st->nmodels);
  reduce_kernel<<<rg, 128, 0, stream>>>(
      (const TcCol *)st->cols.p, ncols, (const int *)st->mcb.p, st->nmodels,
      (const double *)st->P.p, (const int *)st->nonself.p, d_K, nq, Qp,
      2.0 / st->rstep, d_I, st->S_out);
  DBX_CUDA_TRY(cudaGetLastError());
  return ok();
}

Error tc_combine(const double *d_ff, const double *d_S, int ncols, int nq,
                 double *d_I, cudaStream_t stream) {
  combine_kernel<<<(nq + 127) / 128, 128, 0, stream>>>(d_ff, d_S, ncols, nq, d_I);
  DBX_CUDA_TRY(cudaGetLastError());
  return ok();
}

Error tc_status(int herr) {
  if (herr)
    return fail(DBX_ERR_TIMEOUT, "tensor-core contraction: a bounded device wait ran out");
  return ok();
}

Error tc_check(TcState *st, cudaStream_t stream) {
  int herr = 0;
  DBX_CUDA_TRY(cudaMemcpyAsync(&herr, st->err.p, sizeof(int), cudaMemcpyDeviceToHost,
                               stream));
  DBX_CUDA_TRY(cudaStreamSynchronize(stream));
  st->d2h += sizeof(int);
  return tc_status(herr);
}

}  // namespace dbx
