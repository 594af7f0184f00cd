// FP64 block Gram products C = X^T Y on the 5th-generation tensor cores (tcgen05, sm_103a) by exact
// integer slicing (the Ozaki scheme).
//
// The eigensolver's B-orthogonalisation and Rayleigh-Ritz steps form C (a x b) = X^T Y for tall
// blocks X (n x a) and Y (n x b) with n up to ~1e6 and a, b <= 160. GB300 runs FP64 on its CUDA cores
// at ~1 TFLOP/s, against ~2 PFLOP/s of BF16 tensor throughput, so these products are FP64-bound by
// a wide margin. Here every FP64 value is written exactly as a sum of eight signed 7-bit digits
// relative to the largest magnitude of its column within a 128-row chunk:
//
//     x = 2^(E - 1022) * sum_{s<8} d_s 2^(-7(s+1)),   |d_s| <= 127   (56 bits, FP64 has 53)
//
// Digits are integers, so they are exact in BF16, and a digit product is an integer below 2^14.
// Products of digit pairs (s, t) with s + t = g are summed into one FP32 accumulator g in TMEM by
// tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulation); with at most 8 pairs per g and 128 rows
// per chunk every partial sum stays below 2^24, so the FP32 accumulation is exact. Pairs with
// s + t >= 8 are dropped: the truncation error is below 2^-52 of |x_max| |y_max| of the chunk, i.e.
// at FP64 rounding level in the normwise sense. After each chunk the eight exact accumulators are
// combined exactly into two int64 sums and added, scaled, into FP64 register accumulators. Cost per
// output element and chunk: 36 digit-pair MMAs on the tensor pipe, and on the FP64 pipe two
// conversions and two FMAs instead of 128 FMAs.
//
// A first, coalesced pass (chunk_exp_kernel) finds each column's exponent per 128-row chunk. Then one
// CTA (8 warps, two threads per row of C) owns a 128 x 32 tile of C and a range of rows of X and Y:
// per chunk, four 32-row sub-blocks are sliced into shared memory (8 digit planes per operand,
// K-major core-matrix layout without swizzle) and thread 0 issues the 72 MMAs of the sub-block,
// tracked by an mbarrier; the loads of a sub-block are issued before waiting on the previous
// sub-block's MMAs, so they overlap. Partial tiles of all CTAs are summed by a deterministic kernel.
//
// Every wait on the mbarrier is bounded (about one second of GPU time): on expiry the kernel raises
// an error flag, waits once more (bounded) for its MMAs in flight, frees its TMEM and returns.
#include <cuda_bf16.h>

#include <cstdint>
#include <mutex>

#include "device.h"
#include "ozaki.h"

namespace fem2d {

namespace {

constexpr int kDigits = 8;     // digits per FP64 value
constexpr int kChunk = 128;    // rows per exact accumulation
constexpr int kSub = 32;       // rows per shared-memory sub-block
constexpr int kM = 128;        // tile rows (columns of X)
constexpr int kN = 32;         // tile columns (columns of Y)
constexpr uint32_t kTmemCols = kDigits * kN;   // one FP32 accumulator of kN columns per digit sum
constexpr int kPlaneA = kM * kSub * 2;         // bytes of one digit plane of X (128 rows x 32 bf16)
constexpr int kPlaneB = kN * kSub * 2;         // bytes of one digit plane of Y
constexpr int kSmemBytes = kDigits * (kPlaneA + kPlaneB) + 1024;
constexpr uint64_t kWaitNs = 1000000000ull;    // bounded waits: 1 s

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// shared-memory matrix descriptor: no swizzle, K-major core matrices of 8 rows x 16 bytes;
// lbo = byte distance between core matrices adjacent in K, sbo = between 8-row groups
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version of the sm_100 family; base offset 0, no swizzle
  return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for the mbarrier phase; false when the time limit passed
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  if (mbar_try(mbar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try(mbar, parity))
    if (global_ns() - t0 > kWaitNs) return false;
  return true;
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int q = 0; q < 8; q++) v[q] = __uint_as_float(r[q]);
}

// the eight digits of v relative to the biased exponent E of its column's largest magnitude
__device__ __forceinline__ void digits8(double v, int E, float (&d)[kDigits]) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7FF);
  const int shift = E - ex;
  const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const unsigned long long A = (ex == 0 || shift > 55) ? 0ull : ((mant << 3) >> shift);
  const bool neg = (bits >> 63) != 0;
#pragma unroll
  for (int s = 0; s < kDigits; s++) {
    const int dg = (int)((A >> (49 - 7 * s)) & 0x7F);
    d[s] = (float)(neg ? -dg : dg);
  }
}

// digits8 with integer digit extraction on 32-bit halves and a float conversion by the 2^23 offset
// (no integer-to-float conversions); the same eight values as digits8
__device__ __forceinline__ void digits8_fast(double v, int E, float (&d)[kDigits]) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7FF);
  const int shift = E - ex;
  const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const unsigned long long A = (ex == 0 || shift > 55) ? 0ull : ((mant << 3) >> shift);
  const uint32_t hi = (uint32_t)(A >> 32), lo = (uint32_t)A;
  const float sg = (bits >> 63) ? -1.0f : 1.0f, off = -8388608.0f * sg;
  const uint32_t dg[kDigits] = {(hi >> 17) & 0x7Fu, (hi >> 10) & 0x7Fu, (hi >> 3) & 0x7Fu,
                                __funnelshift_r(lo, hi, 28) & 0x7Fu, (lo >> 21) & 0x7Fu, (lo >> 14) & 0x7Fu,
                                (lo >> 7) & 0x7Fu, lo & 0x7Fu};
#pragma unroll
  for (int s = 0; s < kDigits; s++) d[s] = fmaf(__uint_as_float(0x4B000000u | dg[s]), sg, off);
}

__device__ __forceinline__ int biased_exp(double v) {
  return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7FF);
}

// 2^e as a double (0 below the normal range)
__device__ __forceinline__ double pow2(int e) {
  if (e < -1022) return 0.0;
  if (e > 1023) e = 1023;
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// The two exact digit-sum halves T_hi (groups 0..3) and T_lo (groups 4..7, in units of 2^-28 of T_hi's)
// as one integer in units of 2^-SH of T_hi's: T_hi 2^SH + T_lo 2^(SH - 28) rounded to the nearest
// integer. The rounding error is at most 2^-(SH + 1) of a unit of T_hi, below one dropped digit pair
// (s + t >= 8) of a single product. The combination is integer work (GB300's FP64 pipe is the scarce
// unit): one int64 -> FP64 conversion per output follows. Each caller picks SH from its own bound on
// |T_hi| so that the result stays below 2^63: the Gram chunk and the operator-product item (|T_hi| < 2^42)
// take SH = 20, the block update (two chunks of K, |T_hi| < 2^43) SH = 19; |T_lo| < 2^46 everywhere.
template <int SH>
__device__ __forceinline__ long long fuse_digit_sums(long long th, long long tl) {
  return (long long)((unsigned long long)th << SH) + ((tl + (1ll << (27 - SH))) >> (28 - SH));
}
constexpr int kFuseGram = 20, kFuseGemm = 19, kFuseSpmm = 20;

// a 2^k, exact, by an integer add to a's exponent field when a and the result are normal; otherwise by
// an FP64 multiply
__device__ __forceinline__ double scale_pow2(double a, int k) {
  const long long bits = __double_as_longlong(a);
  const int e = (int)((bits >> 52) & 0x7FF);
  if (e != 0 && e + k >= 1 && e + k <= 2046) return __longlong_as_double(bits + ((long long)k << 52));
  return a * pow2(k);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// byte offset of core matrix (row group rg, k group kg) in a K-major tile with kSub columns
__device__ __forceinline__ int core_off(int rg, int kg) { return (rg * (kSub / 8) + kg) * 128; }

// E[c * a + j] = biased exponent of max |X[r][j]| over the 128-row chunk c (one pass, coalesced)
__global__ void __launch_bounds__(128) chunk_exp_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, int a,
                                                         int* __restrict__ E) {
  const int64_t c0 = (int64_t)blockIdx.x * kChunk;
  const int col = blockIdx.y * 128 + threadIdx.x;
  if (col >= a) return;
  const int rows = (int)min((int64_t)kChunk, n - c0);
  const double* xp = X + c0 * ldx + col;
  int e = 0, r = 0;
  for (; r + 16 <= rows; r += 16) {
    double v[16];
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __ldg(xp + (int64_t)(r + q) * ldx);
#pragma unroll
    for (int q = 0; q < 16; q++) e = max(e, biased_exp(v[q]));
  }
  for (; r < rows; r++) e = max(e, biased_exp(__ldg(xp + (int64_t)r * ldx)));
  E[(int64_t)blockIdx.x * a + col] = e;
}

// 8 warps per CTA: thread t owns row t % 128 of the C tile (the TMEM lane) and column half t / 128
// (16 FP64 accumulators), slices 16 of each sub-block's 32 rows of its column of X, and warps w and
// w + 4 read the two column halves of the same TMEM lanes back
constexpr int kGramThreads = 256;

__global__ void __launch_bounds__(kGramThreads, 2)
    ozaki_gram_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, int a, const double* __restrict__ Y,
                      int64_t ldy, int b, int64_t rows_per_cta, const int* __restrict__ EX, const int* __restrict__ EY,
                      double* __restrict__ P, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;                                   // kDigits planes of kM x kSub bf16
  uint8_t* sB = smem + kDigits * kPlaneA;               // kDigits planes of kN x kSub bf16
  int* eY = reinterpret_cast<int*>(sB + kDigits * kPlaneB);   // kN column exponents of Y in the chunk
  uint64_t* mbar = reinterpret_cast<uint64_t*>(eY + kN);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);

  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (kM - 1), half = tid >> 7;   // row of the C tile (TMEM lane), column half
  const int col0 = blockIdx.z * kM;    // first column of X in this tile
  const int cy0 = blockIdx.y * kN;     // first column of Y
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  const int64_t r1 = min(n, r0 + rows_per_cta);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the digit planes of X start zeroed: rows of the tile past column a of X are never written again
  for (int t = tid; t < kDigits * kPlaneA / 16; t += kGramThreads)
    reinterpret_cast<uint4*>(sA)[t] = make_uint4(0, 0, 0, 0);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t mb = smem_addr(mbar);
  uint32_t phase = 0;
  bool failed = false, pending = false;

  constexpr int kHalf = kN / 2;
  double acc[kHalf];
#pragma unroll
  for (int j = 0; j < kHalf; j++) acc[j] = 0.0;

  const int my_col = col0 + row;   // this thread's column of X (its row of C)
  const bool col_ok = my_col < a;
  // warps whose 32 rows of the tile all lie past column a of X skip their loads, slicing and readout
  const bool xw = col0 + 32 * (warp & 3) < a;
  const int yj = tid % kN, ykg = tid / kN;   // threads 0..127: a column of Y and its 8-row group
  const bool y_ok = tid < kN * (kSub / 8) && cy0 + yj < b;

  for (int64_t c0 = r0; c0 < r1 && !failed; c0 += kChunk) {
    const int64_t chunk = c0 / kChunk;
    const int Ex = col_ok ? EX[chunk * a + my_col] : 0;
    if (tid < kN) eY[tid] = (cy0 + tid < b) ? EY[chunk * b + cy0 + tid] : 0;
    __syncthreads();
    const int Ey = eY[yj];
    for (int sb = 0; sb < kChunk / kSub; sb++) {
      const int64_t s0 = c0 + sb * kSub + half * (kSub / 2);
      // this thread's 16 rows of the sub-block, loaded before waiting on the previous MMAs
      double xv[kSub / 2], yv[8];
      if (xw) {
#pragma unroll
        for (int r = 0; r < kSub / 2; r++) {
          const int64_t ra = s0 + r;
          xv[r] = (col_ok && ra < r1) ? __ldg(X + ra * ldx + my_col) : 0.0;
        }
      }
#pragma unroll
      for (int r = 0; r < 8; r++) {
        const int64_t ra = c0 + sb * kSub + ykg * 8 + r;
        yv[r] = (y_ok && ra < r1) ? __ldg(Y + ra * ldy + cy0 + yj) : 0.0;
      }
      if (pending) {   // the digit planes are free once the previous sub-block's MMAs have completed
        if (mbar_wait(mb, phase)) {
          phase ^= 1;
          pending = false;
        } else {
          failed = true;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      }
#pragma unroll
      for (int kh = 0; kh < kSub / 16; kh++) {
        if (!xw) break;
        const int kg = half * (kSub / 16) + kh;
        uint32_t pk[kDigits][4];
#pragma unroll
        for (int r8 = 0; r8 < 8; r8 += 2) {
          float d0[kDigits], d1[kDigits];
          digits8_fast(xv[kh * 8 + r8], Ex, d0);
          digits8_fast(xv[kh * 8 + r8 + 1], Ex, d1);
#pragma unroll
          for (int s2 = 0; s2 < kDigits; s2++) pk[s2][r8 >> 1] = pack_bf16(d0[s2], d1[s2]);
        }
        const int off = core_off(row >> 3, kg) + (row & 7) * 16;
#pragma unroll
        for (int s2 = 0; s2 < kDigits; s2++)
          *reinterpret_cast<uint4*>(sA + s2 * kPlaneA + off) = make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
      }
      if (tid < kN * (kSub / 8)) {
        uint32_t pk[kDigits][4];
#pragma unroll
        for (int r8 = 0; r8 < 8; r8 += 2) {
          float d0[kDigits], d1[kDigits];
          digits8_fast(yv[r8], Ey, d0);
          digits8_fast(yv[r8 + 1], Ey, d1);
#pragma unroll
          for (int s2 = 0; s2 < kDigits; s2++) pk[s2][r8 >> 1] = pack_bf16(d0[s2], d1[s2]);
        }
        const int off = core_off(yj >> 3, ykg) + (yj & 7) * 16;
#pragma unroll
        for (int s2 = 0; s2 < kDigits; s2++)
          *reinterpret_cast<uint4*>(sB + s2 * kPlaneB + off) = make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
      }
      // the generic-proxy stores above must be visible to the tensor core's (async) proxy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      if (__syncthreads_or(failed)) {   // a bounded wait expired somewhere: every thread leaves together
        failed = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (tid == 0) {
        const uint32_t aBase = smem_addr(sA), bBase = smem_addr(sB);
#pragma unroll 1
        // digit s2 of X against Y's digit planes 0 .. 7 - s2 stacked along N, written at TMEM column
        // 32 s2: the pair (s2, t) lands in accumulator g = s2 + t (one MMA per digit of X; an MMA costs
        // about the same for every N up to 64, so wide N pays)
#pragma unroll 1
        for (int s2 = 0; s2 < kDigits; s2++)
#pragma unroll
          for (int kk = 0; kk < kSub / 16; kk++) {
            const uint64_t da = smem_desc(aBase + s2 * kPlaneA + kk * 256, 128, (kSub / 8) * 128);
            const uint64_t db = smem_desc(bBase + kk * 256, 128, (kSub / 8) * 128);
            const uint32_t accum = (sb > 0 || s2 > 0 || kk > 0) ? 1u : 0u;
            mma_bf16(tmem + (uint32_t)(s2 * kN), da, db, instr_desc(kM, (kDigits - s2) * kN), accum);
          }
        mma_commit(mb);
      }
      pending = true;
    }
    if (failed) break;
    if (pending) {   // the chunk's last MMAs, before its accumulators are read
      if (mbar_wait(mb, phase)) {
        phase ^= 1;
        pending = false;
      } else {
        failed = true;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    // combine the eight exact digit-sum accumulators of this chunk (this thread's row and column half,
    // 8 columns at a time). acc_g <= (g + 1) 128 127^2 < 2^24; in int64, exactly,
    //   T_hi = sum_{g<4} acc_g 2^(7 (3 - g)) < 2^43,   T_lo = sum_{g>=4} acc_g 2^(7 (7 - g)) < 2^47,
    // and the chunk's contribution is (T_hi + T_lo 2^-28) 2^-35 2^(Ex - 1022) 2^(Ey - 1022), taken as
    // fuse_digit_sums(T_hi, T_lo) 2^-20 2^-35 2^(Ex - 1022) 2^(Ey - 1022): one conversion and one FMA
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
#pragma unroll
    for (int cb = 0; cb < kHalf; cb += 8) {
      if (!xw) break;
      const int jc = half * kHalf + cb;   // first column of this group in the C tile
      long long Th[8], Tl[8];
#pragma unroll
      for (int q = 0; q < 8; q++) Th[q] = Tl[q] = 0;
#pragma unroll
      for (int g = 0; g < kDigits; g++) {
        float v[8];
        tmem_ld8(lane_base + (uint32_t)(g * kN + jc), v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const long long iv = (long long)__float2int_rn(v[q]);
          if (g < 4) Th[q] += iv << (7 * (3 - g));
          else Tl[q] += iv << (7 * (7 - g));
        }
      }
#pragma unroll
      for (int q = 0; q < 8; q++)
        acc[cb + q] = fma((double)fuse_digit_sums<kFuseGram>(Th[q], Tl[q]),
                          pow2(Ex + eY[jc + q] - 2044 - 35 - kFuseGram), acc[cb + q]);
    }
    // every thread's TMEM reads are complete before the next chunk's MMAs overwrite the accumulators
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (failed && tid == 0) {   // every thread arrives here (uniform exits)
    atomicOr(err, 1);
    if (pending) mbar_wait(mb, phase);   // bounded: let MMAs still in flight finish before TMEM is freed
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  // this CTA's partial tile (kM x kN, row-major)
  const int64_t tile = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  double* out = P + tile * (kM * kN) + (int64_t)row * kN + half * kHalf;
#pragma unroll
  for (int j = 0; j < kHalf; j++) out[j] = acc[j];
}

// C[i * b + j] (row-major a x b) = sum over the CTAs of row range of the partial tiles
__global__ void ozaki_reduce_kernel(const double* __restrict__ P, int nrb, int ny, int a, int b, double* __restrict__ C) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a * b) return;
  const int i = e / b, j = e % b;
  const int mz = i / kM, nyi = j / kN;
  const int64_t base = (((int64_t)mz * ny + nyi) * nrb) * (kM * kN) + (int64_t)(i % kM) * kN + (j % kN);
  double s = 0.0;
  for (int k = 0; k < nrb; k++) s += P[base + (int64_t)k * (kM * kN)];
  C[e] = s;
}

// ---------------------------------------------------------------------------------------------------
// Z = beta Z + alpha X C for a tall X (n x a, a <= 256) and a small C (a x b, b <= 32): the block
// updates of the B-orthogonalisation and the Ritz-vector products. Each CTA owns 128-row tiles of X
// and Z (TMEM lane = row; 8 warps, two threads per row, each slicing 16 of a sub-block's 32 columns of
// X and owning 16 of the 32 columns of Z). X is sliced with one exponent per row (over its a entries)
// and C with one per column (over its a entries), so every K sub-block's digit sums share one scale:
// they are read from TMEM after each 128 columns of K (the exact-accumulation limit) and summed exactly
// in int64, fused into one integer (fuse_digit_sums) and converted to FP64 once per output element, with
// alpha and the power-of-two scale joined exactly in the exponent field. C's digit planes (K padded to
// kc) stay in shared memory for all tiles. Each 128 x 32 sub-block of X is brought in by coalesced
// asynchronous copies (cp.async, a whole row segment per warp instruction) into a padded staging
// buffer, one sub-block ahead of its slicing when two staging buffers fit. The row exponents come from
// a coalesced pre-pass (row_exp_kernel).
constexpr int kGemmKMax = 256;
constexpr int kGemmThreads = 256;
constexpr int kGemmPlanes = kDigits * kPlaneA;   // digit planes of one 128 x 32 sub-block of X (64 KB)
constexpr int kGemmRow = kSub + 1;               // staged doubles per row (padded: no bank conflicts)
constexpr int kGemmStage = kM * kGemmRow * 8;    // one staged 128 x 32 sub-block of X (33 KB)
constexpr int kGemmSmemMax = 227 * 1024;
// shared memory of the block update for K padded to kc, with `stages` staging buffers
__host__ __device__ constexpr int gemm_smem(int kc, int stages) {
  return kGemmPlanes + stages * kGemmStage + kDigits * kN * kc * 2 + 1024;
}

// byte offset of core matrix (row group rg, k group kg) in a K-major tile with kc columns
__device__ __forceinline__ int core_off_k(int rg, int kg, int kc) { return (rg * (kc / 8) + kg) * 128; }

// E[r] = biased exponent of max |X[r][k]| over k < a: a warp takes 4 rows at a time (lanes across the
// rows, four independent loads in flight per lane: the pass is bound by load latency)
constexpr int kRowExpRows = 4;
__global__ void __launch_bounds__(256) row_exp_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, int a,
                                                       int* __restrict__ E) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * kRowExpRows; r0 < n;
       r0 += nwarps * kRowExpRows) {
    int e[kRowExpRows];
#pragma unroll
    for (int u = 0; u < kRowExpRows; u++) e[u] = 0;
    for (int k = lane; k < a; k += 32)
#pragma unroll
      for (int u = 0; u < kRowExpRows; u++)
        if (r0 + u < n) e[u] = max(e[u], biased_exp(__ldg(X + (r0 + u) * ldx + k)));
#pragma unroll
    for (int u = 0; u < kRowExpRows; u++) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) e[u] = max(e[u], __shfl_xor_sync(0xffffffffu, e[u], off));
      if (lane == 0 && r0 + u < n) E[r0 + u] = e[u];
    }
  }
}

// rows of X tile `tile`, columns k0 .. k0 + 31, into the staging buffer sx (row r at r * kGemmRow);
// entries outside X are zero-filled
__device__ __forceinline__ void gemm_stage(const double* __restrict__ X, int64_t n, int64_t ldx, int a, int64_t tile,
                                           int k0, double* sx) {
#pragma unroll
  for (int i = 0; i < kM * kSub / kGemmThreads; i++) {
    const int e = threadIdx.x + kGemmThreads * i;
    const int r = e >> 5, q = e & 31;
    const int64_t row = tile * kM + r;
    const bool ok = row < n && k0 + q < a;
    const double* src = ok ? X + row * ldx + k0 + q : X;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_addr(sx + r * kGemmRow + q)), "l"(src),
                 "r"(ok ? 8 : 0)
                 : "memory");
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

__global__ void __launch_bounds__(kGemmThreads, 1)
    ozaki_gemm_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, int a, const double* __restrict__ C, int b,
                      double alpha, double beta, double* __restrict__ Z, int64_t ldz, const int* __restrict__ EXr,
                      int stages, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int kc = (a + kSub - 1) / kSub * kSub;     // K padded to whole sub-blocks
  const int planeC = kN * kc * 2;                  // one digit plane of C (32 x kc bf16, K-major)
  uint8_t* sA = smem;                              // digit planes of the current sub-block of X
  double* sX = reinterpret_cast<double*>(smem + kGemmPlanes);   // staging buffers
  uint8_t* sC = smem + kGemmPlanes + stages * kGemmStage;
  int* eC = reinterpret_cast<int*>(sC + kDigits * planeC);   // kN column exponents of C
  uint64_t* bar = reinterpret_cast<uint64_t*>(eC + kN);       // MMAs committed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int rl = tid & (kM - 1), half = tid >> 7;  // row of the tile (TMEM lane), column half
  const int64_t ntiles = (n + kM - 1) / kM;
  const int nsub = kc / kSub;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the first sub-block's copies, then C's column exponents and digit planes (row j of the B operand =
  // column j of C)
  if (blockIdx.x < ntiles) gemm_stage(X, n, ldx, a, blockIdx.x, 0, sX);
  if (tid < kN) {
    int e = 0;
    if (tid < b)
      for (int k = 0; k < a; k++) e = max(e, biased_exp(C[(int64_t)k * b + tid]));
    eC[tid] = e;
  }
  __syncthreads();
  for (int t = tid; t < kN * (kc / 8); t += kGemmThreads) {
    const int j = t % kN, kg = t / kN;
    uint32_t pk[kDigits][4];
#pragma unroll
    for (int r8 = 0; r8 < 8; r8 += 2) {
      float d0[kDigits], d1[kDigits];
      const int k0 = kg * 8 + r8;
      digits8((j < b && k0 < a) ? C[(int64_t)k0 * b + j] : 0.0, eC[j], d0);
      digits8((j < b && k0 + 1 < a) ? C[(int64_t)(k0 + 1) * b + j] : 0.0, eC[j], d1);
#pragma unroll
      for (int s2 = 0; s2 < kDigits; s2++) pk[s2][r8 >> 1] = pack_bf16(d0[s2], d1[s2]);
    }
    const int off = core_off_k(j >> 3, kg, kc) + (j & 7) * 16;
#pragma unroll
    for (int s2 = 0; s2 < kDigits; s2++)
      *reinterpret_cast<uint4*>(sC + s2 * planeC + off) = make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  bool failed = false;
  const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  const uint64_t dA = smem_desc(smem_addr(sA), 128, (kSub / 8) * 128);
  const uint64_t dC = smem_desc(smem_addr(sC), 128, (uint32_t)kc * 16u);
  uint32_t ph = 0u;
  bool pending = false;   // MMAs committed and not yet waited for (they read sA)
  int sbc = 0;            // sub-blocks staged so far (selects the staging buffer)

  for (int64_t tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
    const int64_t row = tile * kM + rl;
    const bool row_ok = row < n;
    const int Ex = row_ok ? EXr[row] : 0;
    long long Th[kN / 2], Tl[kN / 2];
#pragma unroll
    for (int j = 0; j < kN / 2; j++) Th[j] = Tl[j] = 0;
    for (int sb = 0; sb < nsub && !failed; sb++, sbc++) {
      const int k0 = sb * kSub;
      const double* sx = sX + (stages == 2 ? (sbc & 1) : 0) * (kGemmStage / 8);
      // the next sub-block's copies into the other staging buffer (with one buffer, after the slicing)
      int64_t nt = tile;
      int nk = k0 + kSub;
      if (nk >= kc) {
        nt = tile + gridDim.x;
        nk = 0;
      }
      const bool more = nt < ntiles;
      if (stages == 2 && more) {
        gemm_stage(X, n, ldx, a, nt, nk, sX + ((sbc + 1) & 1) * (kGemmStage / 8));
        asm volatile("cp.async.wait_group 1;" ::: "memory");
      } else {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
      }
      __syncthreads();   // every thread's copies of this sub-block have landed
      double xv[kSub / 2];
#pragma unroll
      for (int q = 0; q < kSub / 2; q++) xv[q] = sx[rl * kGemmRow + half * (kSub / 2) + q];
      if (pending) {   // the digit planes are free once the previous MMAs completed
        if (mbar_wait(smem_addr(bar), ph)) {
          ph ^= 1u;
          pending = false;
        } else {
          failed = true;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      }
#pragma unroll
      for (int kh = 0; kh < 2; kh++) {
        const int kg = half * 2 + kh;
        uint32_t pk[kDigits][4];
#pragma unroll
        for (int r8 = 0; r8 < 8; r8 += 2) {
          float d0[kDigits], d1[kDigits];
          digits8_fast(xv[kh * 8 + r8], Ex, d0);
          digits8_fast(xv[kh * 8 + r8 + 1], Ex, d1);
#pragma unroll
          for (int s2 = 0; s2 < kDigits; s2++) pk[s2][r8 >> 1] = pack_bf16(d0[s2], d1[s2]);
        }
        const int off = core_off(rl >> 3, kg) + (rl & 7) * 16;
#pragma unroll
        for (int s2 = 0; s2 < kDigits; s2++)
          *reinterpret_cast<uint4*>(sA + s2 * kPlaneA + off) = make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      if (__syncthreads_or(failed)) {   // a bounded wait expired somewhere: every thread leaves together
        failed = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // with one staging buffer the next sub-block's copies start now (its slot was read above)
      if (stages == 1 && more) gemm_stage(X, n, ldx, a, nt, nk, sX);
      const bool first = (k0 % kChunk) == 0;   // the accumulators restart every 128 columns of K
      if (tid == 0) {
#pragma unroll 1
        // digit s2 of X against C's digit planes 0 .. 7 - s2 stacked along N, written at TMEM column
        // 32 s2: the pair (s2, t) lands in accumulator g = s2 + t
#pragma unroll 1
        for (int s2 = 0; s2 < kDigits; s2++)
#pragma unroll
          for (int kk = 0; kk < kSub / 16; kk++) {
            const uint32_t accum = (!first || s2 > 0 || kk > 0) ? 1u : 0u;
            mma_bf16(tmem + (uint32_t)(s2 * kN), dA + (uint64_t)((s2 * kPlaneA + kk * 256) >> 4),
                     dC + (uint64_t)((((k0 / 8) + 2 * kk) * 128) >> 4), instr_desc(kM, (kDigits - s2) * kN), accum);
          }
        mma_commit(smem_addr(bar));
      }
      pending = true;
      const bool last = (k0 + kSub) % kChunk == 0 || k0 + kSub >= kc;
      if (last) {   // the accumulators are read back: wait for these MMAs now
        if (mbar_wait(smem_addr(bar), ph)) {
          ph ^= 1u;
          pending = false;
        } else {
          failed = true;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (__syncthreads_or(failed)) {
          failed = true;
          break;
        }
        // exact digit sums of these (at most 128) columns of K into the int64 accumulators
#pragma unroll
        for (int cb = 0; cb < kN / 2; cb += 8) {
          float v[kDigits][8];
#pragma unroll
          for (int g = 0; g < kDigits; g++) tmem_ld8(lane_base + (uint32_t)(g * kN + half * (kN / 2) + cb), v[g]);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int g = 0; g < kDigits; g++)
#pragma unroll
            for (int q = 0; q < 8; q++) {
              const long long iv = (long long)__float2int_rn(v[g][q]);
              if (g < 4) Th[cb + q] += iv << (7 * (3 - g));
              else Tl[cb + q] += iv << (7 * (7 - g));
            }
        }
        // every thread's reads of the accumulators precede the next MMAs
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      }
    }
    if (failed) break;
    if (row_ok) {
      // one conversion and one multiply (or FMA) per output: alpha and the power-of-two scale are
      // combined exactly in the exponent field
      double* zr = Z + row * ldz + half * (kN / 2);
#pragma unroll
      for (int q = 0; q < kN / 2; q++) {
        const int j = half * (kN / 2) + q;
        if (j >= b) break;
        const double t = (double)fuse_digit_sums<kFuseGemm>(Th[q], Tl[q]);
        const double m = scale_pow2(alpha, Ex + eC[j] - 2044 - 35 - kFuseGemm);
        zr[q] = beta == 0.0 ? t * m : fma(t, m, beta == 1.0 ? zr[q] : beta * zr[q]);
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");   // no copy outlives the kernel
  if (failed && tid == 0) {   // every thread arrives here (uniform exits)
    atomicOr(err, 1);
    if (pending) mbar_wait(smem_addr(bar), ph);   // bounded: MMAs in flight finish before TMEM is freed
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ---------------------------------------------------------------------------------------------------
// Operator products Y = coef M X for one matrix M (A or B) of the pencil, nb <= 32 columns of X.
//
// Rows of one Elem's interior functions share a column list (a run of R <= 64 rows); an item is one
// run and 64 consecutive columns of its list. M's values are sliced once per solve (spmm_slice_kernel)
// into the eight 7-bit digit planes of digits8 (one exponent per item row), in the K-major
// core-matrix layout the MMA reads. The product kernel gathers the item's 64 rows of X and slices them
// the same way (one exponent per column) into a sequence of digit planes of X, 16 or 32 rows (one per
// column) each, preceded by zero planes. The MMA's 128 rows are (digit-sum group g, column of X) and
// its N the run's rows: for the accumulator of group g, the MMA with digit plane t of M reads the
// window of X planes that starts at digit g - t, so each accumulator sums exactly the pairs (s, t) with
// s + t = g -- at most 8 pairs x 64 columns x 127^2 < 2^24, exact in FP32 -- and each TMEM lane holds
// one or two such sums per run row. With nb <= 16 the eight groups x 16 columns fill one 128-row
// operand (8 MMAs per plane step); with nb <= 32, groups 0..3 and 4..7 x 32 columns fill two (4 and 8
// MMAs). Sums are combined exactly in int64 across lanes and warps (fixed order), fused into one integer
// and converted once per item and output to FP64 (one conversion and one FMA) and summed per run in
// registers; every run is owned by one CTA, which writes
// its rows of Y once (no atomics, no zero fill, deterministic). Pairs with s + t >= 8 are dropped: below
// 2^-52 of max|m| max|x| of the item per term, FP64 rounding level in the normwise sense.
//
// Pipeline: two CTAs per SM, one shared-memory stage each, so one CTA's gathers and slicing overlap the
// other's MMAs and readout. Per item, thread 0 has its digit planes of M brought in by one bulk
// asynchronous copy while all threads gather and slice its rows of X (the next item's record, column
// indices and row exponents are loaded one item ahead, and its rows of X prefetched into L2). Every
// mbarrier wait is bounded (one second): on expiry the kernel raises the error flag, lets its copies
// and MMAs in flight finish (bounded), frees its TMEM and returns.
constexpr int kSpK = 64;                                // columns of a run's list per item
constexpr int kSpThreads = 256;
constexpr int kSpXPlaneW = 32 * kSpK * 2;               // a digit plane of X, 32 columns (4 KB)
constexpr int kSpXPlaneP = 16 * kSpK * 2;               // 16 columns (2 KB)
constexpr int kSpXBytes = 11 * kSpXPlaneW;              // 3 zero + 8 digit planes (wide); 7 + 8 (packed)
constexpr int kSpMBytes = 2 * kDigits * 64 * 64 + 2048; // planes of a 64-row item + row-block overrun
constexpr int kSpSmem = kSpXBytes + kSpMBytes + 1536;   // one stage; two CTAs per SM
constexpr uint32_t kSpTmemCols = 128;

// uint4 units of one item's digit planes: 2 sub-blocks of 32 K x 8 planes x R8 rows x 4 k-groups
__host__ __device__ constexpr int sp_item_units(int r8) { return 2 * kDigits * r8 * 4; }

__global__ void __launch_bounds__(256) spmm_slice_kernel(int nitems, const int4* __restrict__ items,
                                                          const int32_t* __restrict__ grp,
                                                          const int64_t* __restrict__ rp,
                                                          const int64_t* __restrict__ poff,
                                                          const int64_t* __restrict__ eoff,
                                                          const double* __restrict__ va, const double* __restrict__ vb,
                                                          double ca, double cb, uint4* __restrict__ planes,
                                                          int* __restrict__ ex) {
  // the sliced matrix's value at CSR position k: ca A + cb B, rounded as the FP64 product kernels do
  auto val = [&](int64_t k) {
    double x = 0.0;
    if (ca != 0.0) x += ca * va[k];
    if (cb != 0.0) x += cb * vb[k];
    return x;
  };
  __shared__ int erow[64];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 w = items[it];   // x: run, y: first column, z: rows R, w: columns Lc
    const int r0 = grp[w.x], R = w.z, R8 = (R + 7) & ~7, Lc = w.w;
    __syncthreads();
    if (threadIdx.x < 64) erow[threadIdx.x] = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < R * 4; t += blockDim.x) {   // row r, 16-column quarter
      const int r = t >> 2, q0 = (t & 3) * 16;
      const int64_t k0 = rp[r0 + r] + w.y;
      int e = 0;
      for (int q = q0; q < min(q0 + 16, Lc); q++) e = max(e, biased_exp(val(k0 + q)));
      atomicMax(&erow[r], e);
    }
    __syncthreads();
    if (threadIdx.x < R) ex[eoff[it] + threadIdx.x] = erow[threadIdx.x];
    // sub-block sb (32 columns), plane t, core matrix (r / 8, kg): 16 bytes at row r % 8
    uint4* pl = planes + poff[it];
    const int per_sub = kDigits * R8 * 4;
    for (int t = threadIdx.x; t < R8 * 8; t += blockDim.x) {
      const int r = t >> 3, kg8 = t & 7, sb = kg8 >> 2, kg = kg8 & 3;
      const int64_t k0 = r < R ? rp[r0 + r] + w.y : -1;
      const int E = r < R ? erow[r] : 0;
      uint32_t pk[kDigits][4];
#pragma unroll
      for (int r8 = 0; r8 < 8; r8 += 2) {
        const int q = kg8 * 8 + r8;
        float d0[kDigits], d1[kDigits];
        digits8((k0 >= 0 && q < Lc) ? val(k0 + q) : 0.0, E, d0);
        digits8((k0 >= 0 && q + 1 < Lc) ? val(k0 + q + 1) : 0.0, E, d1);
#pragma unroll
        for (int s2 = 0; s2 < kDigits; s2++) pk[s2][r8 >> 1] = pack_bf16(d0[s2], d1[s2]);
      }
      const int64_t cm = (int64_t)((r >> 3) * 4 + kg) * 8 + (r & 7);   // uint4 index within a plane
#pragma unroll
      for (int s2 = 0; s2 < kDigits; s2++)
        pl[(int64_t)sb * per_sub + (int64_t)s2 * R8 * 4 + cm] = make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
    }
  }
}

__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

// gather the item's 64 rows of X (their indices in cq, -1 past the item's columns), find each column's
// exponent (ecol: zeroed by the caller) and write the digit planes of X into xs (after its zero planes)
__device__ __forceinline__ void sp_stage_x(const int* cq, const double* __restrict__ X, int64_t ldx, int nb,
                                           bool packed, uint8_t* xs, int* ecol) {
  const int tid = threadIdx.x;
  if (!packed) {
    // thread: column j, rows q = 8 part .. 8 part + 7 (one core-matrix row of 8 K values per digit)
    const int j = tid & 31, part = tid >> 5;
    double xv[8];
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int c = cq[part * 8 + r];
      xv[r] = (j < nb && c >= 0) ? __ldg(X + (int64_t)c * ldx + j) : 0.0;
    }
    int e = 0;
#pragma unroll
    for (int r = 0; r < 8; r++) e = max(e, biased_exp(xv[r]));
    if (j < nb) atomicMax(&ecol[j], e);
    __syncthreads();
    const int E = ecol[j];
    uint32_t pk[kDigits][4];
#pragma unroll
    for (int r = 0; r < 8; r += 2) {
      float d0[kDigits], d1[kDigits];
      digits8_fast(xv[r], E, d0);
      digits8_fast(xv[r + 1], E, d1);
#pragma unroll
      for (int s = 0; s < kDigits; s++) pk[s][r >> 1] = pack_bf16(d0[s], d1[s]);
    }
    // digit s: plane 3 + s, row j
#pragma unroll
    for (int s = 0; s < kDigits; s++)
      *reinterpret_cast<uint4*>(xs + (3 + s) * kSpXPlaneW + (j >> 3) * 1024 + part * 128 + (j & 7) * 16) =
          make_uint4(pk[s][0], pk[s][1], pk[s][2], pk[s][3]);
  } else {
    // thread: column j < 16, rows q = 4 part .. 4 part + 3 (half a core-matrix row per digit)
    const int j = tid & 15, part = tid >> 4;
    double xv[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int c = cq[part * 4 + r];
      xv[r] = (j < nb && c >= 0) ? __ldg(X + (int64_t)c * ldx + j) : 0.0;
    }
    int e = 0;
#pragma unroll
    for (int r = 0; r < 4; r++) e = max(e, biased_exp(xv[r]));
    if (j < nb) atomicMax(&ecol[j], e);
    __syncthreads();
    const int E = ecol[j];
    uint32_t pk[kDigits][2];
#pragma unroll
    for (int r = 0; r < 4; r += 2) {
      float d0[kDigits], d1[kDigits];
      digits8_fast(xv[r], E, d0);
      digits8_fast(xv[r + 1], E, d1);
#pragma unroll
      for (int s = 0; s < kDigits; s++) pk[s][r >> 1] = pack_bf16(d0[s], d1[s]);
    }
    // digit s: plane 7 + s, row j
#pragma unroll
    for (int s = 0; s < kDigits; s++)
      *reinterpret_cast<uint2*>(xs + (7 + s) * kSpXPlaneP + (j >> 3) * 1024 + (part >> 1) * 128 + (j & 7) * 16 +
                                (part & 1) * 8) = make_uint2(pk[s][0], pk[s][1]);
  }
}

__global__ void __launch_bounds__(kSpThreads, 2)
    spmm_tc_kernel(const TcSpmmItem* __restrict__ items, const int32_t* __restrict__ cta_ptr,
                   const int2* __restrict__ zruns, int nzero, const int32_t* __restrict__ col,
                   const uint4* __restrict__ planes, const int* __restrict__ ex, double coef,
                   const double* __restrict__ X, int64_t ldx, int nb, double* __restrict__ Y, int64_t ldy,
                   int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* xs = smem;                          // zero planes + digit planes of X
  uint8_t* ms = smem + kSpXBytes;              // digit planes of M; the readout's partial sums afterwards
  int* ecol = reinterpret_cast<int*>(ms + kSpMBytes);   // [2][32] column exponents of X (by item parity)
  int* em = ecol + 64;                                   // [2][64] row exponents of M
  int* cq = em + 128;                                    // [2][64] the items' column indices (-1 past Lc)
  uint64_t* bar_full = reinterpret_cast<uint64_t*>(cq + 128);   // M planes arrived
  uint64_t* bar_mma = bar_full + 1;                              // MMAs committed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_mma + 1);
  int* sfail = reinterpret_cast<int*>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool packed = nb <= 16;

  // runs without columns: their rows of Y are zero
  for (int z = blockIdx.x; z < nzero; z += gridDim.x) {
    const int2 zr = zruns[z];
    for (int t = tid; t < zr.y * nb; t += kSpThreads) Y[(int64_t)(zr.x + t / nb) * ldy + t % nb] = 0.0;
  }
  // the buffers start zeroed: the zero planes of X stay so, and the MMAs read whole 8-row groups past
  // short runs
  for (int t = tid; t < (kSpXBytes + kSpMBytes) / 16; t += kSpThreads)
    reinterpret_cast<uint4*>(smem)[t] = make_uint4(0, 0, 0, 0);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(kSpTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar_full)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar_mma)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *sfail = 0;
  }
  const int i0 = cta_ptr[blockIdx.x], i1 = cta_ptr[blockIdx.x + 1];
  if (i0 < i1 && tid < 64) {   // the first item's exponent slots and column indices
    const TcSpmmItem f = items[i0];
    em[tid] = tid < f.R ? ex[f.eoff + tid] : 0;
    cq[tid] = tid < f.Lc ? __ldg(col + f.cbase + tid) : -1;
    if (tid < 32) ecol[tid] = 0;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t mbf = smem_addr(bar_full), mbm = smem_addr(bar_mma);
  const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  // descriptors of the X planes and of the M planes (address offsets are added in 16-byte units)
  const uint64_t dX = smem_desc(smem_addr(xs), 128, 1024);
  const uint64_t dM = smem_desc(smem_addr(ms), 128, 512);
  uint32_t ph_full = 0u, ph_mma = 0u;
  bool copy_out = false, failed = false;
  double acc[8];
#pragma unroll
  for (int o = 0; o < 8; o++) acc[o] = 0.0;

  // threads 0..63 hold the next item's record one iteration ahead, so the loads it addresses (column
  // indices, row exponents) start at the top of an iteration and are consumed after its gathers
  TcSpmmItem wn_next{};
  if (tid < 64 && i0 + 1 < i1) wn_next = items[i0 + 1];
  for (int idx = i0, k = 0; idx < i1; idx++, k++) {
    const TcSpmmItem w = items[idx];
    const bool more = idx + 1 < i1;
    const int R = w.R, R8 = (R + 7) & ~7, nrb = (R + 31) >> 5;
    int* ecs = ecol + 32 * (k & 1);
    int* ems = em + 64 * (k & 1);
    // the item's digit planes of M (the buffer's previous readers finished before the last barrier)
    if (tid == 0) {
      bulk_copy_g2s(smem_addr(ms), planes + w.poff, (uint32_t)sp_item_units(R8) * 16u, mbf);
      copy_out = true;
    }
    // the next item's column indices (used after this item's gathers for an L2 prefetch of its rows of
    // X, and by its own gathers), exponent slots of the other parity
    int nc = -1, emv = 0;
    TcSpmmItem wn_after{};
    if (more && tid < 64) {
      const TcSpmmItem wn = wn_next;
      nc = tid < wn.Lc ? __ldg(col + wn.cbase + tid) : -1;
      emv = tid < wn.R ? __ldg(ex + wn.eoff + tid) : 0;
      ecol[32 * ((k + 1) & 1) + (tid & 31)] = 0;
      if (idx + 2 < i1) wn_after = items[idx + 2];
    }
    sp_stage_x(cq + 64 * (k & 1), X, ldx, nb, packed, xs, ecs);
    if (nc >= 0) {
      const double* xr = X + (int64_t)nc * ldx;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(xr));
      if (nb > 16) asm volatile("prefetch.global.L2 [%0];" ::"l"(xr + 16));
    }
    if (more && tid < 64) {
      cq[64 * ((k + 1) & 1) + tid] = nc;
      em[64 * ((k + 1) & 1) + tid] = emv;
      wn_next = wn_after;
    }
    // the X planes (generic stores) are visible to the tensor core's async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
      if (mbar_wait(mbf, ph_full)) {
        ph_full ^= 1u;
        copy_out = false;
        const uint32_t plane = (uint32_t)R8 * 64u, sub = kDigits * plane;
        // all the run's rows in one MMA (N = R rounded up to 16, at most 64: an MMA costs about the
        // same for every N up to 64); TMEM column = run row
        const uint32_t idesc = instr_desc(128, (R + 15) & ~15);
#pragma unroll 1
        for (int ks = 0; ks < kSpK / 16; ks++) {
          const uint64_t db = dM + (((ks >> 1) * sub + (ks & 1) * 256u) >> 4);
          const uint64_t dx = dX + (uint64_t)(ks * 16);
          if (packed) {
            // lanes (group g, column j); plane t of M meets X digits g - t
#pragma unroll
            for (int t = 0; t < kDigits; t++)
              mma_bf16(tmem, dx + (uint64_t)((7 - t) * (kSpXPlaneP >> 4)), db + (uint64_t)(t * (plane >> 4)), idesc,
                       (ks > 0 || t > 0) ? 1u : 0u);
          } else {
            // groups 0..3 (t <= 3) at TMEM column 0 and 4..7 at column 64
#pragma unroll
            for (int t = 0; t < 4; t++)
              mma_bf16(tmem, dx + (uint64_t)((3 - t) * (kSpXPlaneW >> 4)), db + (uint64_t)(t * (plane >> 4)), idesc,
                       (ks > 0 || t > 0) ? 1u : 0u);
#pragma unroll
            for (int t = 0; t < kDigits; t++)
              mma_bf16(tmem + 64u, dx + (uint64_t)((7 - t) * (kSpXPlaneW >> 4)), db + (uint64_t)(t * (plane >> 4)),
                       idesc, (ks > 0 || t > 0) ? 1u : 0u);
          }
        }
      } else {
        *sfail = 1;
      }
      mma_commit(mbm);
    }
    const bool ok = mbar_wait(mbm, ph_mma);
    ph_mma ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (__syncthreads_or(!ok || (tid == 0 && *sfail))) {
      failed = true;
      break;
    }
    // readout into the M buffer (its planes are consumed): per lane (group g, column j) the exact int64
    // digit sums T_hi = sum_{g<4} D_g 2^(7 (3 - g)), T_lo = sum_{g>=4} D_g 2^(7 (7 - g)), one partial per
    // warp; D_g < 8 * 64 * 127^2 < 2^23, so the partials stay below 2^46. Lanes stay in integers: the FP64
    // conversion is done once per output by its owner (GB300's FP64 pipe is the scarce unit)
    long long* PH = reinterpret_cast<long long*>(ms);
    long long* PL = PH + 4096;
    const int rounds = packed ? 1 : nrb;
    for (int rb = 0; rb < rounds; rb++) {
      if (!packed) {
        // lane (r = warp % 4, column j = lane): groups r (block 0) and 4 + r (block 1) of row block rb;
        // warps 0-3 take the first half of its row groups, 4-7 the second
        const int r = warp & 3, j = lane;
        const int ngr = min(32, R - 32 * rb) > 16 ? 4 : 2;
        const int g0 = warp < 4 ? 0 : ngr / 2, g1 = warp < 4 ? ngr / 2 : ngr;
        for (int ig = g0; ig < g1; ig++) {
          float v0[8], v1[8];
          tmem_ld8(lane_base + (uint32_t)(rb * 32 + ig * 8), v0);
          tmem_ld8(lane_base + (uint32_t)(64 + rb * 32 + ig * 8), v1);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const int e = (r * 32 + ig * 8 + q) * 32 + j;
            PH[e] = (long long)__float2int_rn(v0[q]) << (7 * (3 - r));
            PL[e] = (long long)__float2int_rn(v1[q]) << (7 * (3 - r));
          }
        }
      } else {
        // lane (group g = 2 (warp % 4) + lane / 16, column j = lane % 16); the two groups of a warp are
        // both below 4 (warps 0, 1) or both above (2, 3) and are added by a shuffle; warps 0-3 and 4-7
        // split the row groups (the two row blocks, or the halves of one)
        const int g = 2 * (warp & 3) + (lane >> 4), j = lane & 15;
        const int sh = g < 4 ? 7 * (3 - g) : 7 * (7 - g);
        const int ngr_total = nrb == 2 ? 4 + ((R - 32) > 16 ? 4 : 2) : (R > 16 ? 4 : 2);
        const int first = warp < 4 ? 0 : (nrb == 2 ? 4 : ngr_total / 2);
        const int last = warp < 4 ? (nrb == 2 ? 4 : ngr_total / 2) : ngr_total;
        for (int gi = first; gi < last; gi++) {
          const int b = gi >> 2, ig = gi & 3;
          float v[8];
          tmem_ld8(lane_base + (uint32_t)(b * 32 + ig * 8), v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int q = 0; q < 8; q++) {
            long long t = (long long)__float2int_rn(v[q]) << sh;
            t += __shfl_xor_sync(0xffffffffu, t, 16);
            if (lane < 16) PH[((warp & 3) * 64 + b * 32 + ig * 8 + q) * 16 + j] = t;
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // convert: thread tid owns pairs p = tid + 256 o of the run (row p / 32 and column p % 32, or
      // row p / 16 and column p % 16 with nb <= 16); the partials are added in a fixed order
#pragma unroll
      for (int o = 0; o < 8; o++) {
        const int p = tid + 256 * o;
        const int i = packed ? p >> 4 : p >> 5, j = packed ? p & 15 : p & 31;
        const bool mine = packed ? o < 4 : (o >> 2) == rb;
        if (!mine || i >= R || j >= nb) continue;
        long long th, tl;
        if (packed) {
          th = PH[i * 16 + j] + PH[(64 + i) * 16 + j];
          tl = PH[(128 + i) * 16 + j] + PH[(192 + i) * 16 + j];
        } else {
          const int e = (i - 32 * rb) * 32 + j;
          th = PH[e] + PH[1024 + e] + PH[2048 + e] + PH[3072 + e];
          tl = PL[e] + PL[1024 + e] + PL[2048 + e] + PL[3072 + e];
        }
        acc[o] = fma((double)fuse_digit_sums<kFuseSpmm>(th, tl), pow2(ecs[j] + ems[i] - 2044 - 35 - kFuseSpmm), acc[o]);
      }
      if (rb + 1 < rounds) __syncthreads();
    }
    if (w.last) {   // the run is complete: its rows of Y
#pragma unroll
      for (int o = 0; o < 8; o++) {
        const int p = tid + 256 * o;
        const int i = packed ? p >> 4 : p >> 5, j = packed ? p & 15 : p & 31;
        if ((!packed || o < 4) && i < R && j < nb) Y[(int64_t)(w.r0 + i) * ldy + j] = coef * acc[o];
        acc[o] = 0.0;
      }
    }
    // the readout's generic accesses to the M buffer precede the next bulk copy into it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
  }
  if (failed && tid == 0) {
    atomicOr(err, 1);
    if (copy_out) mbar_wait(mbf, ph_full);   // bounded
    mbar_wait(mbm, ph_mma ^ 1u);             // bounded: MMAs still in flight finish before TMEM is freed
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kSpTmemCols) : "memory");
}

// The issue cost of tcgen05.mma (kind::f16, M = 128, K = 16) against N: one CTA per SM, thread 0 issues
// `reps` MMAs on zero operands into two alternating accumulators and waits (bounded) for their commit;
// the elapsed global time per MMA is written per CTA. The kernels above are shaped by this cost (one
// MMA costs about the same for every N up to 64).
__global__ void __launch_bounds__(128, 1) mma_cost_kernel(int N, int reps, unsigned long long* __restrict__ out,
                                                          int* __restrict__ err) {
  __shared__ __align__(1024) uint8_t A[128 * 16 * 2];
  __shared__ __align__(1024) uint8_t B[256 * 16 * 2];
  __shared__ uint64_t bar;
  __shared__ uint32_t slot;
  for (int t = threadIdx.x; t < 128 * 16; t += 128) reinterpret_cast<uint16_t*>(A)[t] = 0;
  for (int t = threadIdx.x; t < 256 * 16; t += 128) reinterpret_cast<uint16_t*>(B)[t] = 0;
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_addr(&slot)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = slot;
  if (threadIdx.x == 0) {
    // A: 128 rows x 16 K (row groups 256 bytes apart), B: N rows x 16 K
    const uint64_t da = smem_desc(smem_addr(A), 128, 256), db = smem_desc(smem_addr(B), 128, 256);
    const uint32_t idesc = instr_desc(128, N);
    uint32_t ph = 0;
    for (int pass = 0; pass < 2; pass++) {   // the first pass warms the pipe up
      const uint64_t t0 = global_ns();
      for (int r = 0; r < reps; r++) mma_bf16(tmem + (uint32_t)((r & 1) * 256), da, db, idesc, 1u);
      mma_commit(smem_addr(&bar));
      if (!mbar_wait(smem_addr(&bar), ph)) atomicOr(err, 1);
      ph ^= 1u;
      if (pass == 1) out[blockIdx.x] = global_ns() - t0;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

std::mutex g_attr_mu;
bool g_attr_done[256] = {};

}  // namespace

int ozaki_gram_partials(int64_t n, int a, int b, int num_sms) {
  const int tiles = ((a + kM - 1) / kM) * ((b + kN - 1) / kN);
  const int64_t chunks = std::max<int64_t>(1, (n + kChunk - 1) / kChunk);
  // two CTAs per SM (83 KB of shared memory and 256 TMEM columns each): one slices while the other
  // waits on its loads or MMAs
  const int64_t per = std::max<int64_t>(1, 2 * num_sms / tiles);
  return (int)std::min<int64_t>(per, chunks);
}

size_t ozaki_gram_workspace(int64_t n, int a, int b, int num_sms) {
  const int tiles = ((a + kM - 1) / kM) * ((b + kN - 1) / kN);
  const int64_t chunks = std::max<int64_t>(1, (n + kChunk - 1) / kChunk);
  // partial tiles, then the chunk exponents of X and Y (ints, two per double)
  return (size_t)ozaki_gram_partials(n, a, b, num_sms) * tiles * kM * kN + (size_t)(chunks * (a + b) + 1) / 2 + 1;
}

void ozaki_gemm(Ctx& c, int64_t n, const double* X, int64_t ldx, int a, const double* C, int b, double alpha,
                double beta, double* Z, int64_t ldz, int* rowexp, int* err) {
  if (n <= 0 || b <= 0) return;
  if (a < 1 || a > kGemmKMax || b > kN) fail(FEM2D_E_INVALID_ARG, "ozaki_gemm: a <= 256 and b <= 32");
  static std::mutex mu;
  static bool done[256] = {};
  {
    std::lock_guard<std::mutex> lk(mu);
    if (c.device >= 0 && c.device < 256 && !done[c.device]) {
      FEM2D_CUDA(cudaFuncSetAttribute(ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmemMax));
      done[c.device] = true;
    }
  }
  const int kc = (a + kSub - 1) / kSub * kSub;
  const int stages = gemm_smem(kc, 2) <= kGemmSmemMax ? 2 : 1;
  const int64_t ntiles = (n + kM - 1) / kM;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)c.num_sms));
  row_exp_kernel<<<(int)std::min<int64_t>((n * 32 + 255) / 256, (int64_t)c.num_sms * 16), 256, 0, c.stream>>>(
      n, X, ldx, a, rowexp);
  ozaki_gemm_kernel<<<grid, kGemmThreads, gemm_smem(kc, stages), c.stream>>>(n, X, ldx, a, C, b, alpha, beta, Z, ldz,
                                                                            rowexp, stages, err);
  FEM2D_CUDA(cudaGetLastError());
  c.launches += 2;
}

void TcSpmm::build(Ctx& c, int64_t n, const std::vector<int32_t>& grp_h, const std::vector<int64_t>& row_ptr) {
  std::vector<int4> it;
  std::vector<int64_t> po, eo;
  std::vector<int32_t> run_first;   // first item of each run
  std::vector<int2> zr;
  int64_t pcur = 0, ecur = 0;
  const int nruns = (int)grp_h.size() - 1;
  for (int g = 0; g < nruns; g++) {
    run_first.push_back((int32_t)it.size());
    const int r0 = grp_h[g], R = grp_h[g + 1] - r0;
    if (R <= 0) continue;
    if (R > 64) fail(FEM2D_E_INVALID_ARG, "tensor SpMM: a row run longer than 64 rows");
    const int64_t len = row_ptr[r0 + 1] - row_ptr[r0];
    if (len == 0) zr.push_back(make_int2(r0, R));
    const int R8 = (R + 7) & ~7;
    for (int64_t q0 = 0; q0 < len; q0 += kSpK) {
      it.push_back(make_int4(g, (int)q0, R, (int)std::min<int64_t>(kSpK, len - q0)));
      po.push_back(pcur);
      eo.push_back(ecur);
      pcur += sp_item_units(R8);
      ecur += R;
    }
  }
  run_first.push_back((int32_t)it.size());
  if (ecur > INT32_MAX) fail(FEM2D_E_TOO_LARGE, "tensor SpMM: too many row exponents");
  nitems = (int)it.size();
  plane_units = pcur;
  exp_count = ecur;
  nzero = (int)zr.size();
  // the product kernel's order: CTA b takes the runs b, b + grid, ... (two CTAs per SM)
  grid = std::max(1, std::min(std::max(nruns, 1), 2 * c.num_sms));
  std::vector<TcSpmmItem> ci;
  std::vector<int32_t> cp;
  ci.reserve(it.size());
  for (int b = 0; b < grid; b++) {
    cp.push_back((int32_t)ci.size());
    for (int g = b; g < nruns; g += grid)
      for (int q = run_first[g]; q < run_first[g + 1]; q++) {
        const int4 w = it[q];
        TcSpmmItem m;
        m.cbase = row_ptr[grp_h[g]] + w.y;
        m.poff = po[q];
        m.eoff = (int32_t)eo[q];
        m.r0 = grp_h[g];
        m.R = (int16_t)w.z;
        m.Lc = (int16_t)w.w;
        m.last = q + 1 == run_first[g + 1] ? 1 : 0;
        ci.push_back(m);
      }
  }
  cp.push_back((int32_t)ci.size());
  items.upload(it, c.stream);
  poff.upload(po, c.stream);
  eoff.upload(eo, c.stream);
  citems.upload(ci, c.stream);
  cta_ptr.upload(cp, c.stream);
  zruns.upload(zr.empty() ? std::vector<int2>{make_int2(0, 0)} : zr, c.stream);
  (void)n;
}

void TcSpmm::slice(Ctx& c, int k, const int32_t* grp, const int64_t* rp, const double* va, const double* vb,
                   double ca, double cb) {
  if (k < 0 || k >= kSlots) fail(FEM2D_E_INVALID_ARG, "tensor SpMM: slot out of range");
  Slot& sl = slot[k];
  if (sl.planes.n != (size_t)std::max<int64_t>(plane_units, 1)) sl.planes.alloc_on(std::max<int64_t>(plane_units, 1), c.stream);
  if (sl.exps.n != (size_t)std::max<int64_t>(exp_count, 1)) sl.exps.alloc_on(std::max<int64_t>(exp_count, 1), c.stream);
  sl.ca = ca;
  sl.cb = cb;
  sl.ready = true;
  if (nitems == 0) return;
  const int grid = std::max(1, std::min(nitems, c.num_sms * 8));
  spmm_slice_kernel<<<grid, 256, 0, c.stream>>>(nitems, items.p, grp, rp, poff.p, eoff.p, va, vb, ca, cb, sl.planes.p,
                                                 sl.exps.p);
  FEM2D_CUDA(cudaGetLastError());
  c.launches++;
}

int TcSpmm::find(double ca, double cb, double* coef) const {
  for (int k = 0; k < kSlots; k++) {
    const Slot& sl = slot[k];
    if (!sl.ready) continue;
    if (sl.ca == 1.0 && sl.cb == 0.0 && cb == 0.0 && ca != 0.0) {
      *coef = ca;
      return k;
    }
    if (sl.ca == 0.0 && sl.cb == 1.0 && ca == 0.0 && cb != 0.0) {
      *coef = cb;
      return k;
    }
    if (sl.ca == ca && sl.cb == cb) {
      *coef = 1.0;
      return k;
    }
  }
  return -1;
}

void TcSpmm::apply(Ctx& c, int k, double coef, const int32_t* grp, const int64_t* rp, const int32_t* col,
                   const double* X, int64_t ldx, int nb, double* Y, int64_t ldy, int* err) {
  if (nb < 1 || nb > 32) fail(FEM2D_E_INVALID_ARG, "tensor SpMM: 1..32 columns");
  if (k < 0 || k >= kSlots || !slot[k].ready) fail(FEM2D_E_INVALID_ARG, "tensor SpMM: matrix not sliced");
  static std::mutex mu;
  static bool done[256] = {};
  {
    std::lock_guard<std::mutex> lk(mu);
    if (c.device >= 0 && c.device < 256 && !done[c.device]) {
      FEM2D_CUDA(cudaFuncSetAttribute(spmm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSpSmem));
      done[c.device] = true;
    }
  }
  if (grid == 0) return;
  spmm_tc_kernel<<<grid, kSpThreads, kSpSmem, c.stream>>>(citems.p, cta_ptr.p, zruns.p, nzero, col, slot[k].planes.p,
                                                          slot[k].exps.p, coef, X, ldx, nb, Y, ldy, err);
  FEM2D_CUDA(cudaGetLastError());
  c.launches++;
}

void ozaki_gram(Ctx& c, int64_t n, const double* X, int64_t ldx, int a, const double* Y, int64_t ldy, int b,
                double* C, double* work, size_t work_doubles, int* err) {
  if (a <= 0 || b <= 0) return;
  if (a > 4 * kM || b > 8 * kN) fail(FEM2D_E_INVALID_ARG, "ozaki_gram: block wider than 512 x 256");
  {
    std::lock_guard<std::mutex> lk(g_attr_mu);
    if (c.device >= 0 && c.device < 256 && !g_attr_done[c.device]) {
      FEM2D_CUDA(cudaFuncSetAttribute(ozaki_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
      g_attr_done[c.device] = true;
    }
  }
  const int nrb = ozaki_gram_partials(n, a, b, c.num_sms);
  const int mz = (a + kM - 1) / kM, ny = (b + kN - 1) / kN;
  if (work_doubles < ozaki_gram_workspace(n, a, b, c.num_sms)) fail(FEM2D_E_INVALID_ARG, "ozaki_gram: workspace too small");
  const int64_t chunks = std::max<int64_t>(1, (n + kChunk - 1) / kChunk);
  int* EX = reinterpret_cast<int*>(work + (size_t)nrb * mz * ny * kM * kN);
  int* EY = EX + chunks * a;
  if (n > 0) {
    chunk_exp_kernel<<<dim3((unsigned)chunks, (a + 127) / 128), 128, 0, c.stream>>>(n, X, ldx, a, EX);
    chunk_exp_kernel<<<dim3((unsigned)chunks, (b + 127) / 128), 128, 0, c.stream>>>(n, Y, ldy, b, EY);
    FEM2D_CUDA(cudaGetLastError());
    c.launches += 2;
  }
  int64_t rpc = (std::max<int64_t>(n, 1) + nrb - 1) / nrb;
  rpc = (rpc + kChunk - 1) / kChunk * kChunk;
  dim3 grid(nrb, ny, mz);
  ozaki_gram_kernel<<<grid, kGramThreads, kSmemBytes, c.stream>>>(n, X, ldx, a, Y, ldy, b, rpc, EX, EY, work, err);
  FEM2D_CUDA(cudaGetLastError());
  ozaki_reduce_kernel<<<(a * b + 255) / 256, 256, 0, c.stream>>>(work, nrb, ny, a, b, C);
  FEM2D_CUDA(cudaGetLastError());
  c.launches += 2;
}


double measure_mma_ns(Ctx& c, int n) {
  if (n < 16 || n > 256 || n % 16 != 0) fail(FEM2D_E_INVALID_ARG, "MMA cost: N must be a multiple of 16 in 16..256");
  const int reps = 4096;
  DBuf<unsigned long long> out;
  DBuf<int> err;
  out.alloc(c.num_sms);
  err.alloc(1);
  FEM2D_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), c.stream));
  mma_cost_kernel<<<c.num_sms, 128, 0, c.stream>>>(n, reps, out.p, err.p);
  FEM2D_CUDA(cudaGetLastError());
  c.launches++;
  std::vector<unsigned long long> h(c.num_sms);
  int he = 0;
  FEM2D_CUDA(cudaMemcpyAsync(h.data(), out.p, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaMemcpyAsync(&he, err.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  if (he) fail(FEM2D_E_TIMEOUT, "MMA cost kernel: a bounded wait expired");
  double ns = 0.0;
  for (unsigned long long v : h) ns += (double)v;
  return ns / h.size() / reps;
}

}  // namespace fem2d
