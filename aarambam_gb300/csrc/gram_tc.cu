// Mode-bispectrum covariance QQ[n][m] = sum_t w_t Q_n(t) Q_m(t) on the
// tensor cores, FP64-accurate (the reference: compute_mode_bispectra_covariance,
// Aarambam/basis/tetrapyd.c:107-236, FP64 loops in C).
//
// The contraction is a GEMM of A = w Q [modes][points] with B = Q over the
// ~3e5 tetrapyd points.  FP64 products would run on GB300's FP64 units; here
// the operands are cut into bf16 digits and multiplied exactly on the bf16
// tensor pipe (a split-operand scheme after Ozaki et al., "Error-free
// transformations of matrix multiplication", 2012):
//
//   row scale   e_n = exponent of max_t |A[n][t]| (frexp), so that
//               v = rint(A 2^(62 - e_n)) is an integer with |v| <= 2^62;
//   digits      v = sum_{s=0..7} d_s 2^(8 (7 - s)), d_1..d_7 balanced in
//               [-128, 127], d_0 in [-64, 64]; stored as bf16 d_s 2^(-8 s)
//               (exact: at most 8 significant bits), so that
//               A = 2^(e_n - 6) sum_s Ahat_s up to 2^-63 of the row maximum;
//   products    QQ = 2^(eA_n + eB_m - 12) sum_{s + u <= 7} Ahat_s Bhat_u^T.
//               Every product Ahat_s Bhat_u is d_s d'_u 2^(-8 (s + u)): an
//               integer of at most 14 bits at the scale of its level
//               L = s + u.  Levels 0..5 each have their own FP32 accumulator
//               in tensor memory and stay below 2^24 over a group of 128
//               points, so they are exact; levels 6 and 7 share one (the only
//               rounding, at 2^-48 of the level-0 scale).  Levels above 7
//               are dropped (below the 2^-63 digit cut-off).
//   read-out    every 128 points the seven accumulators are read from tensor
//               memory and added, converted to integers, into two int64 fixed-
//               point sums per element (levels 0-2 in units of 2^-16 of the
//               level-0 scale, levels 3-7 in units of 2^-56, the low sum
//               normalised into the high one each time): the sum over the
//               points is exact integer arithmetic, so it does not depend on
//               the order, and the result is deterministic.
//
// Accuracy of the digit cut (the 20-mode basis on the 1536^3 case's 150-point
// grid, 300 modes, every level summed exactly, against a 96-bit evaluation):
// largest error 1.8e-16 of max |QQ|, 5.4e-15 of sqrt(QQ_nn QQ_mm); an FP64
// GEMM of the same operands gives 1.2e-15 and 4.4e-15.  The shared level-6/7
// accumulator adds one FP32 rounding per 128-point group at 2^-48 of the
// level-0 scale.
//
// Kernels:
//   k_tetra_modes   Q[n][t] in FP64 (kept by the caller for the stored-mode
//                   entry points; the stateless entry point makes it in its
//                   scratch), k_modes_rowmax the row maxima of |wQ| and |Q|;
//   k_tetra_digits  the bf16 digits of A (128-row tiles) and B (64-row tiles)
//                   in the tcgen05 no-swizzle K-major layout, 16 points per
//                   chunk, the eight digits of a (tile, chunk) contiguous;
//   k_gram_tc       one 128 x 64 tile of QQ (upper triangle only) over a range
//                   of point groups: 1D bulk copies (cp.async.bulk) into four
//                   48 KB stages tracked by mbarriers, one thread issuing the
//                   36 tcgen05.mma (M 128, N 64, K 16, bf16 -> FP32) per chunk
//                   into 7 x 64 tensor-memory columns, eight warps reading
//                   the accumulators out (tcgen05.ld) once per group;
//   k_gram_tc_reduce  the int64 sums of the point ranges, added in a fixed
//                   order, scaled to FP64 and mirrored.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/aarambam.h"
#include "tetra.cuh"

namespace aar {
namespace {

constexpr int kTM = 128;                   // A rows (modes n) per tile: MMA M
constexpr int kTN = 64;                    // B rows (modes m) per tile: MMA N
constexpr int kTK = 16;                    // points per chunk: MMA K
constexpr int kGroup = 8;                  // chunks per accumulator read-out
constexpr int kPts = kTK * kGroup;         // 128 points per group
constexpr int kDig = 8;                    // digits per value
constexpr int kAcc = 7;                    // accumulators: levels 0..5, 6 + 7
constexpr int kStages = 4;
constexpr int kABytes = kTM * kTK * 2;     // one digit of an A chunk: 4 KB
constexpr int kBBytes = kTN * kTK * 2;     // one digit of a B chunk: 2 KB
constexpr int kStageA = kDig * kABytes;    // 32 KB
constexpr int kStageB = kDig * kBBytes;    // 16 KB
constexpr int kStageBytes = kStageA + kStageB;
constexpr int kSmemBytes = kStages * kStageBytes + 1024;  // + alignment slack
constexpr int kEpiWarps = 8;
constexpr int kThreads = (kEpiWarps + 1) * 32;
constexpr uint32_t kTmemCols = 512;        // 7 x 64 used
constexpr int kTile = kTM * kTN;           // elements of one output tile
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait at most

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits
// 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 =
// 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase with the given parity to complete.  Bounded: gives up
// after kWaitNs (and 2^30 polls), or as soon as another thread of the block
// has given up (abort != 0, when `abort` is given); returns false then, after
// setting the block's abort flag.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort) {
  const unsigned long long t0 = globaltimer();
  for (uint32_t i = 0; i < (1u << 30); ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 63u) == 63u) {
      if (abort && *abort) return false;
      if (globaltimer() - t0 > kWaitNs) break;
    }
  }
  if (abort) *abort = 1;
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// 1D bulk copy global -> shared, completion counted on `bar` (16-byte
// aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, K-major without swizzle: core matrices
// of 8 rows x 16 bytes (8 bf16 along K) stored as 128 contiguous bytes, the
// next core matrix along K 128 bytes on (leading byte offset), the next
// group of 8 rows 256 bytes on (stride byte offset); descriptor version 1
// (bits 46-47), no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(256u >> 4) << 32) |
         (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

// arrive on `bar` once every tcgen05 operation this thread issued so far is complete
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---------------------------------------------------------------- operands
// Q[n][t] = Q_n(t) for t < npts, 0 for npts <= t < ldq (the mode bispectra
// kept by the caller for the stored-mode entry points).
__global__ void __launch_bounds__(256) k_tetra_modes(Tetra a, long long ldq, double* __restrict__ Q) {
  const int n = blockIdx.y;
  const double* r1 = a.f + a.p1[n] * a.nk;
  const double* r2 = a.f + a.p2[n] * a.nk;
  const double* r3 = a.f + a.p3[n] * a.nk;
  double* qrow = Q + (size_t)n * ldq;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ldq; t += (long long)gridDim.x * blockDim.x)
    qrow[t] = t < a.npts ? q_rows(r1, r2, r3, a.i1[t], a.i2[t], a.i3[t]) : 0.0;
}

// Row maxima of |w Q| (rowmax[n]) and |Q| (rowmax[nm + n]) over t < npts, as
// the bit patterns of non-negative doubles.
__global__ void __launch_bounds__(256) k_modes_rowmax(const double* __restrict__ Q, long long ldq,
                                                      const double* __restrict__ w, int npts, int nm,
                                                      unsigned long long* __restrict__ rowmax) {
  const int n = blockIdx.y;
  const double* qrow = Q + (size_t)n * ldq;
  double mA = 0.0, mB = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npts; t += gridDim.x * blockDim.x) {
    const double q = qrow[t];
    mB = fmax(mB, fabs(q));
    mA = fmax(mA, fabs(q * w[t]));
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    mA = fmax(mA, __shfl_xor_sync(0xffffffffu, mA, o));
    mB = fmax(mB, __shfl_xor_sync(0xffffffffu, mB, o));
  }
  __shared__ double sA[8], sB[8];
  if ((threadIdx.x & 31) == 0) {
    sA[threadIdx.x >> 5] = mA;
    sB[threadIdx.x >> 5] = mB;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      mA = fmax(mA, sA[i]);
      mB = fmax(mB, sB[i]);
    }
    atomicMax(rowmax + n, (unsigned long long)__double_as_longlong(mA));
    atomicMax(rowmax + nm + n, (unsigned long long)__double_as_longlong(mB));
  }
}

// The eight digits of x (|x| <= 2^e) as floats d_s 2^(-8 s), s = 0 most significant.
__device__ __forceinline__ void to_digits(double x, int e, float (&d)[kDig]) {
  long long v = __double2ll_rn(scalbn(x, 62 - e));
#pragma unroll
  for (int s = kDig - 1; s >= 1; --s) {
    const long long lo = ((v + 128) & 255) - 128;
    d[s] = scalbnf((float)lo, -8 * s);
    v = (v - lo) >> 8;
  }
  d[0] = (float)v;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ int row_exponent(unsigned long long bits) {
  int e = 0;
  const double m = __longlong_as_double((long long)bits);
  if (m > 0.0) frexp(m, &e);
  return e;
}

// One thread per (A tile I, chunk c, 16-byte unit u of the 4 KB block): row
// r = 8 (u / 16) + u % 8, points 8 ((u / 8) % 2) .. +7 of the chunk.  The
// unit index is the byte offset / 16 of that row's 8 points in the no-swizzle
// K-major layout ((r / 8) * 256 + kseg * 128 + (r % 8) * 16), so consecutive
// threads write consecutive 16 bytes; the same row's B digits go to the
// 64-row tile of the same row.
__global__ void __launch_bounds__(256) k_tetra_digits(const double* __restrict__ Q, long long ldq,
                                                      const double* __restrict__ w, int nm, int npts, int nch,
                                                      int rowsA, int rowsB,
                                                      const unsigned long long* __restrict__ rowmax,
                                                      uint4* __restrict__ adig, uint4* __restrict__ bdig,
                                                      int* __restrict__ expo) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long blk = gid >> 8;  // I * nch + c
  if (blk >= (long long)(rowsA / kTM) * nch) return;
  const int u = (int)(gid & 255);
  const int c = (int)(blk % nch), I = (int)(blk / nch);
  const int r = (u >> 4) * 8 + (u & 7), kseg = (u >> 3) & 1;
  const int n = I * kTM + r;
  const int t0 = c * kTK + kseg * 8;
  int eA = 0, eB = 0;
  double q[8];
  if (n < nm) {
    eA = row_exponent(rowmax[n]);
    eB = row_exponent(rowmax[nm + n]);
    const double2* src = reinterpret_cast<const double2*>(Q + (size_t)n * ldq + t0);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double2 v = src[j];
      q[2 * j] = v.x;
      q[2 * j + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) q[j] = 0.0;
  }
  if (c == 0 && kseg == 0) {
    expo[n] = eA;
    expo[rowsA + n] = eB;
  }
  uint32_t pk[kDig][4];
  // A = w Q (the product the FP64 form forms), 128-row tiles
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    const double x0 = (t0 + j < npts) ? q[j] * w[t0 + j] : 0.0;
    const double x1 = (t0 + j + 1 < npts) ? q[j + 1] * w[t0 + j + 1] : 0.0;
    float d0[kDig], d1[kDig];
    to_digits(x0, eA, d0);
    to_digits(x1, eA, d1);
#pragma unroll
    for (int s = 0; s < kDig; ++s) pk[s][j >> 1] = pack_bf16(d0[s], d1[s]);
  }
#pragma unroll
  for (int s = 0; s < kDig; ++s) adig[(blk * kDig + s) * (kABytes / 16) + u] = make_uint4(pk[s][0], pk[s][1], pk[s][2], pk[s][3]);
  if (n >= rowsB) return;
  // B = Q, 64-row tiles
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    float d0[kDig], d1[kDig];
    to_digits(q[j], eB, d0);
    to_digits(q[j + 1], eB, d1);
#pragma unroll
    for (int s = 0; s < kDig; ++s) pk[s][j >> 1] = pack_bf16(d0[s], d1[s]);
  }
  const int J = n / kTN, rb = n % kTN;
  const long long bblk = (long long)J * nch + c;
  const int ub = (rb >> 3) * 16 + kseg * 8 + (rb & 7);
#pragma unroll
  for (int s = 0; s < kDig; ++s) bdig[(bblk * kDig + s) * (kBBytes / 16) + ub] = make_uint4(pk[s][0], pk[s][1], pk[s][2], pk[s][3]);
}

// ---------------------------------------------------------------- the GEMM
struct GramArgs {
  const uint8_t* adig;  // [rowsA / 128][nch][8 digits][4 KB]
  const uint8_t* bdig;  // [rowsB / 64][nch][8 digits][2 KB]
  const int2* pairs;    // (A tile, B tile) per blockIdx.x
  int npairs, nch, ngroups, gps;  // gps: groups per blockIdx.y
  long long* part;      // [gridDim.y][npairs][2][64 cols][128 rows]
  int* err;
};

// Single thread: keeps kStages chunks in flight and issues the MMAs.
__device__ void gram_issue(const GramArgs& g, uint32_t base, uint32_t tmem, const uint8_t* asrc, const uint8_t* bsrc,
                           int nchunk, uint32_t full0, uint32_t empty0, uint32_t accf, uint32_t acce, uint32_t fin,
                           volatile int* abort) {
  int loaded = 0, waited = 0;
  auto load = [&](int c) {
    const int b = c % kStages;
    const uint32_t bar = full0 + 8u * b;
    const uint32_t sa = base + (uint32_t)(b * kStageBytes);
    mbar_expect_tx(bar, kStageBytes);
    bulk_g2s(sa, asrc + (size_t)c * kStageA, kStageA, bar);
    bulk_g2s(sa + kStageA, bsrc + (size_t)c * kStageB, kStageB, bar);
  };
  for (; loaded < kStages && loaded < nchunk; ++loaded) load(loaded);
  bool ok = true;
  for (int c = 0; c < nchunk; ++c) {
    const int b = c % kStages;
    if (c % kGroup == 0 && c > 0) {
      // the accumulators of the previous group have been read out
      if (!(ok = mbar_wait(acce, (uint32_t)((c / kGroup - 1) & 1), abort))) break;
      tc_fence_after();
    }
    if (!(ok = mbar_wait(full0 + 8u * b, (uint32_t)((c / kStages) & 1), abort))) break;
    waited = c + 1;
    tc_fence_after();
    const uint32_t sa = base + (uint32_t)(b * kStageBytes), sb = sa + kStageA;
    const bool first = (c % kGroup) == 0;
#pragma unroll
    for (int L = 0; L < kDig; ++L) {
#pragma unroll
      for (int s = 0; s <= L; ++s) {
        const int acc = L < kAcc - 1 ? L : kAcc - 1;
        const uint32_t fresh = (first && s == 0 && L < kAcc) ? 1u : 0u;
        mma_bf16(tmem + (uint32_t)(acc * kTN), sdesc(sa + (uint32_t)(s * kABytes)),
                 sdesc(sb + (uint32_t)((L - s) * kBBytes)), fresh ? 0u : 1u);
      }
    }
    mma_commit(empty0 + 8u * b);
    if (c % kGroup == kGroup - 1) mma_commit(accf);
    if (c >= 1 && loaded < nchunk) {
      const int pc = c - 1;  // its buffer takes chunk c - 1 + kStages
      if (!(ok = mbar_wait(empty0 + 8u * (pc % kStages), (uint32_t)((pc / kStages) & 1), abort))) break;
      load(loaded);
      ++loaded;
    }
  }
  if (!ok) {
    // drain what is in flight before the block frees its tensor memory
    mma_commit(fin);
    mbar_wait(fin, 0, nullptr);
    for (int c = waited; c < loaded; ++c) mbar_wait(full0 + 8u * (c % kStages), (uint32_t)((c / kStages) & 1), nullptr);
  }
}

// Warps 0-7: warp w reads tensor-memory lanes 32 (w % 4) .. +31 (tile rows)
// and columns 32 (w / 4) .. +31 of each accumulator.
__device__ void gram_epilogue(const GramArgs& g, uint32_t tmem, int gcnt, uint32_t accf, uint32_t acce,
                              volatile int* abort) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sp = warp & 3, half = warp >> 2;
  const uint32_t tb = tmem + ((uint32_t)(sp * 32) << 16) + (uint32_t)(half * 32);
  long long hi[32], lo[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) hi[j] = lo[j] = 0;
  for (int G = 0; G < gcnt; ++G) {
    const bool ok = __all_sync(0xffffffffu, mbar_wait(accf, (uint32_t)(G & 1), abort));
    if (!ok) return;
    tc_fence_after();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      uint32_t r[kAcc][4];
#pragma unroll
      for (int L = 0; L < kAcc; ++L) tmem_ld4(tb + (uint32_t)(L * kTN + q * 4), r[L]);
      tmem_wait_ld();
#pragma unroll
      for (int L = 0; L < kAcc; ++L)
#pragma unroll
        for (int j = 0; j < 4; ++j) asm volatile("" : "+r"(r[L][j]));  // no use before the wait
      if (q == 7) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float a0 = __uint_as_float(r[0][j]), a1 = __uint_as_float(r[1][j]), a2 = __uint_as_float(r[2][j]);
        const float a3 = __uint_as_float(r[3][j]), a4 = __uint_as_float(r[4][j]), a5 = __uint_as_float(r[5][j]);
        const float a67 = __uint_as_float(r[6][j]);
        // levels 0-2 in units of 2^-16, 3-7 in units of 2^-56 (of the level-0 scale)
        const long long h = (long long)__float2int_rn(a0) * 65536 + (long long)__float2int_rn(a1 * 0x1p8f) * 256 +
                            (long long)__float2int_rn(a2 * 0x1p16f);
        const long long l = (long long)__float2int_rn(a3 * 0x1p24f) * 4294967296ll +
                            (long long)__float2int_rn(a4 * 0x1p32f) * 16777216 +
                            (long long)__float2int_rn(a5 * 0x1p40f) * 65536 + __float2ll_rn(a67 * 0x1p56f);
        const int k = q * 4 + j;
        hi[k] += h;
        lo[k] += l;
        hi[k] += lo[k] >> 40;
        lo[k] &= 0xFFFFFFFFFFll;
      }
    }
  }
  long long* out = g.part + ((size_t)blockIdx.y * g.npairs + blockIdx.x) * 2 * kTile;
  const int row = sp * 32 + lane;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const int col = half * 32 + j;
    out[col * kTM + row] = hi[j];
    out[kTile + col * kTM + row] = lo[j];
  }
}

__global__ void __launch_bounds__(kThreads, 1) k_gram_tc(GramArgs g) {
  extern __shared__ uint8_t dsm[];
  __shared__ __align__(8) uint64_t bars[2 * kStages + 3];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[kStages]);
  const uint32_t accf = smem_u32(&bars[2 * kStages]), acce = accf + 8u, fin = accf + 16u;
  const int g0 = blockIdx.y * g.gps;
  const int gcnt = min(g.ngroups, g0 + g.gps) - g0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(full0 + 8u * i, 1);
      mbar_init(empty0 + 8u * i, 1);
    }
    mbar_init(accf, 1);
    mbar_init(acce, kEpiWarps);
    mbar_init(fin, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  if (gcnt > 0) {
    if (warp == kEpiWarps) {
      if (lane == 0) {
        const int2 tp = g.pairs[blockIdx.x];
        const size_t c0 = (size_t)g0 * kGroup;
        gram_issue(g, base, tmem, g.adig + ((size_t)tp.x * g.nch + c0) * kStageA,
                   g.bdig + ((size_t)tp.y * g.nch + c0) * kStageB, gcnt * kGroup, full0, empty0, accf, acce, fin,
                   &abort_flag);
      }
    } else {
      gram_epilogue(g, tmem, gcnt, accf, acce, &abort_flag);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
  if (threadIdx.x == 0 && abort_flag) atomicExch(g.err, 1);
}

// QQ[n][m] = QQ[m][n] for n <= m from the int64 sums of every point range,
// added in a fixed order
__global__ void k_gram_tc_reduce(const long long* __restrict__ part, int nsplit, int npairs,
                                 const int* __restrict__ pid, int ntB, const int* __restrict__ expo, int rowsA,
                                 int nm, double* __restrict__ qq) {
  const long long total = (long long)nm * nm;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(e / nm), m = (int)(e % nm);
    if (n > m) continue;
    const int p = pid[(n / kTM) * ntB + m / kTN];
    const size_t off = (size_t)(m % kTN) * kTM + (n % kTM);
    long long hi = 0, lo = 0;
    for (int s = 0; s < nsplit; ++s) {
      const long long* t = part + ((size_t)s * npairs + p) * 2 * kTile;
      hi += t[off];
      lo += t[kTile + off];
    }
    hi += lo >> 40;
    lo &= 0xFFFFFFFFFFll;
    const int sc = expo[n] + expo[rowsA + m];
    const double v = scalbn((double)hi, sc - 28) + scalbn((double)lo, sc - 68);
    qq[(size_t)n * nm + m] = v;
    qq[(size_t)m * nm + n] = v;
  }
}

// ---------------------------------------------------------------- host
struct GramPlan {
  int npts_pad, nch, ngroups, ntA, ntB, rowsA, rowsB, npairs, nsplit, gps;
  size_t off_max, off_exp, off_a, off_b, off_pairs, off_pid, off_part, off_err, total;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Q row stride of the stored-mode layout: npts rounded up to whole 128-point groups
long long modes_ld(int npts) { return (long long)align_up((size_t)npts, kPts); }

GramPlan gram_plan(int npts, int nm) {
  GramPlan p;
  p.npts_pad = (int)modes_ld(npts);
  p.nch = p.npts_pad / kTK;
  p.ngroups = p.npts_pad / kPts;
  p.ntA = (nm + kTM - 1) / kTM;
  p.ntB = (nm + kTN - 1) / kTN;
  p.rowsA = p.ntA * kTM;
  p.rowsB = p.ntB * kTN;
  p.npairs = 0;
  for (int I = 0; I < p.ntA; ++I) p.npairs += p.ntB - 2 * I;  // B tiles J >= 2 I reach the upper triangle
  // point ranges: about eight waves of one block per SM over the 152 SMs
  const int want = (8 * 152 + p.npairs - 1) / p.npairs;
  const int ns = want < 1 ? 1 : (want > p.ngroups ? p.ngroups : want);
  p.gps = (p.ngroups + ns - 1) / ns;
  p.nsplit = (p.ngroups + p.gps - 1) / p.gps;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o = align_up(o + bytes, 1024);
    return at;
  };
  p.off_max = take((size_t)2 * nm * sizeof(unsigned long long));
  p.off_exp = take((size_t)2 * p.rowsA * sizeof(int));
  p.off_a = take((size_t)p.ntA * p.nch * kStageA);
  p.off_b = take((size_t)p.ntB * p.nch * kStageB);
  p.off_pairs = take((size_t)p.npairs * sizeof(int2));
  p.off_pid = take((size_t)p.ntA * p.ntB * sizeof(int));
  p.off_part = take((size_t)p.nsplit * p.npairs * 2 * kTile * sizeof(long long));
  p.off_err = take(sizeof(int));
  p.total = o + 1024;  // the base is aligned up to 1 KB
  return p;
}

size_t q_bytes(int npts, int nm) { return align_up((size_t)nm * modes_ld(npts) * sizeof(double), 1024); }

int launch_modes(const Tetra& a, double* Q, long long ldq, cudaStream_t st) {
  const long long blocks = (ldq + 255) / 256;
  k_tetra_modes<<<dim3((unsigned)(blocks < 64 ? blocks : 64), a.nmodes), 256, 0, st>>>(a, ldq, Q);
  return tetra_status(cudaGetLastError());
}

// covariance from stored Q (row stride ldq, a multiple of 128 >= npts, zero
// beyond npts); d_scratch: gram_plan(npts, nm).total bytes
int gram_run(double* d_cov, const double* Q, long long ldq, const double* w, int npts, int nm, void* d_scratch,
             cudaStream_t st) {
  const GramPlan p = gram_plan(npts, nm);
  uint8_t* base = (uint8_t*)(((uintptr_t)d_scratch + 1023) & ~(uintptr_t)1023);
  unsigned long long* rowmax = (unsigned long long*)(base + p.off_max);
  int* expo = (int*)(base + p.off_exp);
  uint8_t* adig = base + p.off_a;
  uint8_t* bdig = base + p.off_b;
  int2* pairs = (int2*)(base + p.off_pairs);
  int* pid = (int*)(base + p.off_pid);
  long long* part = (long long*)(base + p.off_part);
  int* err = (int*)(base + p.off_err);
  // tile pairs reaching the upper triangle and their index table, made on the host
  std::vector<int2> hp;
  std::vector<int> hid((size_t)p.ntA * p.ntB, -1);
  for (int I = 0; I < p.ntA; ++I)
    for (int J = 2 * I; J < p.ntB; ++J) {
      hid[(size_t)I * p.ntB + J] = (int)hp.size();
      hp.push_back(make_int2(I, J));
    }
  cudaError_t e = cudaMemcpyAsync(pairs, hp.data(), sizeof(int2) * hp.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pid, hid.data(), sizeof(int) * hid.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(rowmax, 0, (size_t)2 * nm * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e != cudaSuccess) return tetra_status(e);
  const int gx = (npts + 255) / 256 < 64 ? (npts + 255) / 256 : 64;
  k_modes_rowmax<<<dim3(gx, nm), 256, 0, st>>>(Q, ldq, w, npts, nm, rowmax);
  const long long dthreads = (long long)p.ntA * p.nch * 256;
  k_tetra_digits<<<(unsigned)((dthreads + 255) / 256), 256, 0, st>>>(Q, ldq, w, nm, npts, p.nch, p.rowsA, p.rowsB,
                                                                     rowmax, (uint4*)adig, (uint4*)bdig, expo);
  if ((e = cudaGetLastError()) != cudaSuccess) return tetra_status(e);
  if ((e = cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes)) != cudaSuccess)
    return tetra_status(e);
  GramArgs g;
  g.adig = adig;
  g.bdig = bdig;
  g.pairs = pairs;
  g.npairs = p.npairs;
  g.nch = p.nch;
  g.ngroups = p.ngroups;
  g.gps = p.gps;
  g.part = part;
  g.err = err;
  k_gram_tc<<<dim3(p.npairs, p.nsplit), kThreads, kSmemBytes, st>>>(g);
  if ((e = cudaGetLastError()) != cudaSuccess) return tetra_status(e);
  k_gram_tc_reduce<<<1024, 256, 0, st>>>(part, p.nsplit, p.npairs, pid, p.ntB, expo, p.rowsA, nm, d_cov);
  if ((e = cudaGetLastError()) != cudaSuccess) return tetra_status(e);
  int herr = 0;
  e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return tetra_status(e);
  return herr ? AAR_ERR_CUDA : AAR_OK;
}

}  // namespace
}  // namespace aar

using namespace aar;

extern "C" {

int64_t aar_tetra_modes_ld(int32_t tetra_npts) { return tetra_npts > 0 ? modes_ld(tetra_npts) : 0; }

int aar_tetra_modes(double* d_Q, int64_t ldq, const int32_t* d_i1, const int32_t* d_i2, const int32_t* d_i3,
                    int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2, const int32_t* d_p3,
                    int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max, int32_t k_npts, void* stream) {
  if (!d_Q || !d_i1 || !d_i2 || !d_i3 || !d_p1 || !d_p2 || !d_p3 || !d_mode_evals || tetra_npts <= 0 ||
      n_modes <= 0 || mode_p_max <= 0 || k_npts <= 0 || ldq < tetra_npts)
    return AAR_ERR_ARG;
  const Tetra a = make_tetra(nullptr, d_i1, d_i2, d_i3, tetra_npts, d_p1, d_p2, d_p3, n_modes, d_mode_evals,
                             mode_p_max, k_npts);
  return launch_modes(a, d_Q, ldq, (cudaStream_t)stream);
}

size_t aar_modes_covariance_scratch_bytes(int32_t tetra_npts, int32_t n_modes) {
  if (tetra_npts <= 0 || n_modes <= 0) return 0;
  return gram_plan(tetra_npts, n_modes).total;
}

int aar_modes_covariance(double* d_cov, const double* d_Q, int64_t ldq, const double* d_tetra_weights,
                         int32_t tetra_npts, int32_t n_modes, void* d_scratch, size_t scratch_bytes, void* stream) {
  if (!d_cov || !d_Q || !d_tetra_weights || !d_scratch || tetra_npts <= 0 || n_modes <= 0) return AAR_ERR_ARG;
  if (ldq != modes_ld(tetra_npts) || ((uintptr_t)d_Q & 15)) return AAR_ERR_ARG;
  if (scratch_bytes < aar_modes_covariance_scratch_bytes(tetra_npts, n_modes)) return AAR_ERR_ARG;
  return gram_run(d_cov, d_Q, ldq, d_tetra_weights, tetra_npts, n_modes, d_scratch, (cudaStream_t)stream);
}

size_t aar_tetra_covariance_scratch_bytes(int32_t tetra_npts, int32_t n_modes) {
  if (tetra_npts <= 0 || n_modes <= 0) return 0;
  return q_bytes(tetra_npts, n_modes) + gram_plan(tetra_npts, n_modes).total + 1024;
}

int aar_tetra_covariance(double* d_cov, const double* d_tetra_weights, const int32_t* d_i1, const int32_t* d_i2,
                         const int32_t* d_i3, int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2,
                         const int32_t* d_p3, int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max,
                         int32_t k_npts, void* d_scratch, size_t scratch_bytes, void* stream) {
  const Tetra a = make_tetra(d_tetra_weights, d_i1, d_i2, d_i3, tetra_npts, d_p1, d_p2, d_p3, n_modes, d_mode_evals,
                             mode_p_max, k_npts);
  if (!d_cov || !d_scratch || !tetra_ok(a)) return AAR_ERR_ARG;
  if (scratch_bytes < aar_tetra_covariance_scratch_bytes(tetra_npts, n_modes)) return AAR_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  double* Q = (double*)(((uintptr_t)d_scratch + 1023) & ~(uintptr_t)1023);
  const long long ldq = modes_ld(tetra_npts);
  const int rc = launch_modes(a, Q, ldq, st);
  if (rc != AAR_OK) return rc;
  return gram_run(d_cov, Q, ldq, d_tetra_weights, tetra_npts, n_modes, (uint8_t*)Q + q_bytes(tetra_npts, n_modes),
                  st);
}

}  // extern "C"
