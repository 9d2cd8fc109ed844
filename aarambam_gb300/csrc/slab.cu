// Slab form of the FP32 path (AAR_SLAB_FP32): the fused form's arithmetic
// (FP32 fields, per-cell mode functions, compensated modal sum) for grids
// whose fused schedule does not fit one GPU -- at 1536^3 one field is
// 14.6 GB and the fused schedule holds the potential and max(M, 9) work
// fields, 21 x 14.6 = 308 GB at 20 modes.
//
// The modal sum and 2LPT are streamed over S strided real-space x-slabs
// {x = s + S j : j < L = N / S}.  With kx = k1 + L k2 (k1 < L, k2 < S):
//
//   inverse  f(s + S j, y, z) = sum e^{2 pi i (k1 j / L + (ky y + kz z) / N)} F_s(k1, ky, kz),
//            F_s(k1, ky, kz)  = sum_{k2} e^{+2 pi i kx s / N} X(kx, ky, kz),
//   forward  X(kx, ky, kz)    = sum_s e^{-2 pi i kx s / N} G_s(kx mod L, ky, kz),
//
// F_s an (L, N, N) half spectrum whose real inverse transform is the field
// at the slab's points, G_s the forward (L, N, N) transform of slab s.  So
// each real-space step (the products g_r = sum a'_{pqr} f_p f_q, the 2LPT
// source) runs on one slab at a time: the M filtered fields and R products
// exist as slab fields (1/S of a field each), and the transform stages are
// recomputed per slab -- every slab re-reads the whole potential for its
// fold, and its R forward transforms are folded back into one compensated
// accumulator (Neumaier, (sum, compensation) per component in two fields).
//
// Memory (F = one plan field, N^2 HP complex; F_s = L N (N/2+1) complex):
// the potential, then an arena of max(2F + (M + R) F_s, 7F + 6 F_s):
//   modal   acc sum, acc compensation, M slab f_p, R slab g_r
//   2LPT    six real displacement fields (the plan's work slots 0..5, the
//           layout every read-out entry point reads), the source spectrum S,
//           six slab fields (Hessians, then displacements)
// 1536^3, 20 modes, S = 8: 14.6 + 113 GB.
//
// The slab transforms are cuFFT FP32 C2R / R2C of size (L, N, N), in place
// on the [L][N][N/2+1] layout, with a work area the plan allocates: the
// fused form's own line FFTs are power-of-two kernels, and N = 1536 = 3 x
// 512 needs radix 3.  Folds, products, accumulations, the source and the
// scatter into the plan's fields are the kernels below.
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <algorithm>
#include <string>

#include "aar_internal.cuh"
#include "spectral.cuh"

namespace aar {

struct SlabState {
  int S = 0, L = 0, H = 0, M = 0, R = 0;
  int64_t sf = 0;  // float2 entries of one slab field: L N H
  int64_t ff = 0;  // float2 entries of one plan field: N N HP
  size_t arena = 0;  // float2 entries of the arena (the plan's d_work)
  cufftHandle c2r = 0, r2c = 0;
  bool have_c2r = false, have_r2c = false;
  void* fft_work = nullptr;
  size_t fft_need = 0, fft_alloc = 0;  // work area bytes the plans need / allocated
};

// Geometry of one slab pass.
struct SlabGeo {
  Grid g;
  int N, HP, H, L, S, s;  // s: the slab
  int64_t sf;
};

// Product terms of the slab kernels, by output slot (target r ascending).
struct SlabTerms {
  int M, nr;
  int begin[kMaxModes + 1];
  uint16_t p[kMaxTerms], q[kMaxTerms];
  float c[kMaxTerms];
};

__device__ __forceinline__ void slab_cell(int64_t t, const SlabGeo& a, int& k1, int& ky, int& kz) {
  kz = (int)(t % a.H);
  const int64_t r = t / a.H;
  ky = (int)(r % a.N);
  k1 = (int)(r / a.N);
}

// e^{-2 pi i kx s / N} from the plan's table twN[m] = e^{-2 pi i m / N}
__device__ __forceinline__ float2 slab_tw(const float2* __restrict__ twN, int kx, int s, int N) {
  return __ldg(twN + (int)(((int64_t)kx * s) % N));
}

__device__ __forceinline__ float2 mul_conj(float2 x, float2 w) {  // x conj(w)
  return make_float2(x.x * w.x + x.y * w.y, x.y * w.x - x.x * w.y);
}

// Hermitian projection of the kz = 0 and kz = N/2 planes of nf slab fields
// ((L, N) grids): X(k1, ky) <- (X(k1, ky) + conj X(-k1, -ky)) / 2.  FFTW's
// c2r -- the reference's, and the fused form's rows, which drop Im X_0 and
// Im X_{N/2} of a row after its x and y passes -- ignores the anti-Hermitian
// part of these planes, which factors odd in kz on the Nyquist plane (psi_z,
// d_xz, d_yz) create; cuFFT's C2R leaves the result for such input undefined
// (it differed with the transform size).  The projection commutes with the
// fold: conj of the twiddle at -kx is the twiddle at kx.
__global__ void __launch_bounds__(256) k_slab_herm(float2* F, int nf, int64_t sf, int L, int N, int H) {
  const int64_t plane = (int64_t)L * N;
  const int64_t total = (int64_t)nf * 2 * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int f = (int)(i / (2 * plane));
    const int64_t rem = i - (int64_t)f * 2 * plane;
    const int kz = rem < plane ? 0 : N / 2;
    const int64_t ij = rem < plane ? rem : rem - plane;
    const int k1 = (int)(ij / N), ky = (int)(ij - (int64_t)k1 * N);
    const int64_t me = ij, pa = (int64_t)((L - k1) % L) * N + (N - ky) % N;
    if (me > pa) continue;
    float2* a = F + (int64_t)f * sf + me * H + kz;
    if (me == pa) {
      a->y = 0.f;
      continue;
    }
    float2* b = F + (int64_t)f * sf + pa * H + kz;
    const float2 u = *a, v = *b;
    const float2 r = make_float2(0.5f * (u.x + v.x), 0.5f * (u.y - v.y));
    *a = r;
    *b = make_float2(r.x, -r.y);
  }
}

// Field filters q_p(k), p < M, at one cell (n2 = |k|^2 in grid units, > 0):
// the expressions of q_mode_cells (cells.cuh) with one Legendre recurrence
// for all modes (P_{p-1} for mode p > 3).
template <int MAXM>
__device__ __forceinline__ void q_all_modes(const RhoArgs& ra, int M, int n2, float* q) {
  const float lg = __log2f((float)n2);
  const float lk = fmaf(0.5f, lg, ra.log2kF);
#pragma unroll
  for (int p = 0; p < 4 && p < MAXM; ++p)
    if (p < M) q[p] = exp2f((ra.s * (float)(p - 3) + ra.e4) * lk);
  if constexpr (MAXM > 4) {
    if (M > 4) {
      const float kb = fmaf(ra.c1, exp2f(0.5f * ra.s * lg), -1.f - ra.c1);
      const float kp = exp2f(ra.e2 * lk);
      float P0 = 1.f, P1 = kb;
#pragma unroll
      for (int l = 2; l <= 3; ++l) {
        const float Pn = ra.A[l] * kb * P1 - ra.B[l] * P0;
        P0 = P1;
        P1 = Pn;
      }
      q[4] = (P1 - ra.x0[3]) * kp;
#pragma unroll
      for (int p = 5; p < MAXM; ++p) {
        if (p < M) {
          const float Pn = ra.A[p - 1] * kb * P1 - ra.B[p - 1] * P0;
          P0 = P1;
          P1 = Pn;
          q[p] = (P1 - ra.x0[p - 1]) * kp;
        }
      }
    }
  }
}

// ------------------------------------------------------------ modal stage
// F_p(k1, ky, kz) = sum_{k2} q_p(k) e^{+2 pi i kx s / N} phi(k), zero on the
// cut and at k = 0 (main.c:580-637), for all M filters in one read of phi.
template <int MAXM>
__global__ void __launch_bounds__(256) k_slab_fold_modal(SlabGeo a, RhoArgs ra, int M, const float2* __restrict__ phi,
                                                         const float2* __restrict__ twN, float2* __restrict__ out) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.sf; t += (int64_t)gridDim.x * blockDim.x) {
    int k1, ky, kz;
    slab_cell(t, a, k1, ky, kz);
    const int ys = sidx(ky, a.N);
    float2 F[MAXM];
#pragma unroll
    for (int p = 0; p < MAXM; ++p) F[p] = make_float2(0.f, 0.f);
    for (int k2 = 0; k2 < a.S; ++k2) {
      const int kx = k1 + a.L * k2, xs = sidx(kx, a.N);
      const int n2 = xs * xs + ys * ys + kz * kz;
      if (n2 == 0 || !keep_cell(a.g, xs, ys, kz)) continue;
      const float2 X = mul_conj(phi[row_of(kx, ky, a.N, kXB) * a.HP + kz], slab_tw(twN, kx, a.s, a.N));
      float q[MAXM];
      q_all_modes<MAXM>(ra, M, n2, q);
#pragma unroll
      for (int p = 0; p < MAXM; ++p)
        if (p < M) {
          F[p].x = fmaf(q[p], X.x, F[p].x);
          F[p].y = fmaf(q[p], X.y, F[p].y);
        }
    }
#pragma unroll
    for (int p = 0; p < MAXM; ++p)
      if (p < M) out[(int64_t)p * a.sf + t] = F[p];
  }
}

// g_r = sum_t c_t f_p f_q on the slab's real points (row length 2H, the
// first N values of a row), two neighbouring points per thread (N is even):
// the M pairs of a thread go to its own column of shared memory, the terms
// read them by index, one 8-byte load per factor.
constexpr int kProdThreads = 128;
__global__ void __launch_bounds__(kProdThreads) k_slab_products(SlabTerms tm, const float* __restrict__ f,
                                                                float* __restrict__ g, int64_t fsr, int N, int H,
                                                                int64_t rows) {
  __shared__ float2 fv[kMaxModes][kProdThreads];
  const int half = N / 2;
  const int64_t total = rows * half;
  const int tid = threadIdx.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + tid; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / half;
    const int64_t o = row * 2 * H + 2 * (i - row * half);
    for (int p = 0; p < tm.M; ++p) fv[p][tid] = *reinterpret_cast<const float2*>(f + (int64_t)p * fsr + o);
    for (int sl = 0; sl < tm.nr; ++sl) {
      float2 acc = make_float2(0.f, 0.f);
      for (int k = tm.begin[sl]; k < tm.begin[sl + 1]; ++k) {
        const float c = tm.c[k];
        const float2 a = fv[tm.p[k]][tid], b = fv[tm.q[k]][tid];
        acc.x += c * a.x * b.x;
        acc.y += c * a.y * b.y;
      }
      *reinterpret_cast<float2*>(g + (int64_t)sl * fsr + o) = acc;
    }
  }
}

// acc(k) += e^{-2 pi i kx s / N} sum_r rho_r(k) G_{r,s}(kx mod L, ky, kz):
// the slot sum Neumaier-compensated in the slab's frame, then rotated by the
// twiddle once and added to the running compensated sum (acc_s, acc_c) of
// the slabs.  rho_r per cell with k_modal_acc's expressions, its logarithm
// and exponentials in the base-2 hardware forms of q_mode_cells (every slab
// re-evaluates them; the bracket k^s / kmin^s - 1 of kbar is 0 or at least
// 0.42 for integer n2, no cancellation to guard).  The modes are walked in
// one unrolled pass r = 0 .. MAXM-1 with one Legendre recurrence and a
// bit mask of the active r: straight-line code (a walk over the slot list
// with a recurrence loop per slot stalled on instruction fetch, 900
// instructions per cell and slab at 11 slots).  Cut cells and k = 0 are not
// touched (the combine skips them).
struct SlotMap {
  uint32_t active;        // bit r: r has a product field
  int rmax;               // highest active r
  int slot[kMaxModes];    // its slab field
};

template <int MAXM>
__global__ void __launch_bounds__(256) k_slab_acc_modal(SlabGeo a, RhoArgs ra, SlotMap sm,
                                                        const float2* __restrict__ G, const float2* __restrict__ twN,
                                                        float2* acc_s, float2* acc_c, int first) {
  const int dm = (int)(((int64_t)a.L * a.s) % a.N);  // twiddle index step from kx to kx + L
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.sf; t += (int64_t)gridDim.x * blockDim.x) {
    int k1, ky, kz;
    slab_cell(t, a, k1, ky, kz);
    float2 v[MAXM];
#pragma unroll
    for (int r = 0; r < MAXM; ++r)
      v[r] = (sm.active >> r) & 1u ? __ldg(G + (int64_t)sm.slot[r] * a.sf + t) : make_float2(0.f, 0.f);
    const int ys = sidx(ky, a.N);
    int m = (int)(((int64_t)k1 * a.s) % a.N);
    for (int k2 = 0; k2 < a.S; ++k2, m = (m + dm >= a.N) ? m + dm - a.N : m + dm) {
      const int kx = k1 + a.L * k2, xs = sidx(kx, a.N);
      const int n2 = xs * xs + ys * ys + kz * kz;
      if (n2 == 0 || !keep_cell(a.g, xs, ys, kz)) continue;
      const int64_t e = row_of(kx, ky, a.N, kXB) * a.HP + kz;
      float2 s = first ? make_float2(0.f, 0.f) : acc_s[e];
      float2 c = first ? make_float2(0.f, 0.f) : acc_c[e];
      const float2 w = __ldg(twN + m);
      const float lg = __log2f((float)n2);
      const float Lk = fmaf(0.5f, lg, ra.log2kF);  // log2 k
      float2 ps = make_float2(0.f, 0.f), pc = make_float2(0.f, 0.f);
#pragma unroll
      for (int r = 0; r < 4 && r < MAXM; ++r)
        if ((sm.active >> r) & 1u) {
          const float rho = r == 3 ? 1.f : exp2f(ra.s * (float)(r - 3) * Lk);
          neumaier_add(ps.x, pc.x, v[r].x * rho);
          neumaier_add(ps.y, pc.y, v[r].y * rho);
        }
      if constexpr (MAXM > 4) {
        if (sm.rmax >= 4) {
          const float kbar = fmaf(ra.c1, exp2f(0.5f * ra.s * lg), -1.f - ra.c1);
          const float inv_k2 = ra.inv_kF2 / (float)n2;
          float P0 = 1.f, P1 = kbar;  // P_{l-1}, P_l with l = 1
#pragma unroll
          for (int r = 4; r < MAXM; ++r) {
            if (r > sm.rmax) break;
            // mode r takes P_{r-1}: one recurrence step (two for r = 4)
#pragma unroll
            for (int l = (r == 4 ? 2 : r - 1); l <= r - 1; ++l) {
              const float Pn = ra.A[l] * kbar * P1 - ra.B[l] * P0;
              P0 = P1;
              P1 = Pn;
            }
            if ((sm.active >> r) & 1u) {
              const float rho = (P1 - ra.x0[r - 1]) * inv_k2;
              neumaier_add(ps.x, pc.x, v[r].x * rho);
              neumaier_add(ps.y, pc.y, v[r].y * rho);
            }
          }
        }
      }
      const float2 u = cmul(ps, w), uc = cmul(pc, w);
      neumaier_add(s.x, c.x, u.x);
      neumaier_add(s.y, c.y, u.y);
      c.x += uc.x;
      c.y += uc.y;
      acc_s[e] = s;
      acc_c[e] = c;
    }
  }
}

// phi <- phi + fnl_n3 (sum + compensation) on kept cells, DC = 0
// (main.c:1101-1126, as k_modal_acc ends).
__global__ void __launch_bounds__(256) k_slab_combine(Grid g, int N, int HP, float2* phi, const float2* __restrict__ acc_s,
                                                      const float2* __restrict__ acc_c, float fnl_n3) {
  const int H = N / 2 + 1;
  const int64_t total = (int64_t)N * N * H;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / H;
    const int kz = (int)(i - row * H);
    const int64_t e = row * HP + kz;
    int x, y;
    row_xy(row, N, kXB, x, y);
    const int kx = sidx(x, N), ky = sidx(y, N);
    const int n2 = kx * kx + ky * ky + kz * kz;
    if (n2 == 0) {
      phi[e] = make_float2(0.f, 0.f);
      continue;
    }
    if (!keep_cell(g, kx, ky, kz)) continue;
    const float2 s = acc_s[e], c = acc_c[e];
    float2 ph = phi[e];
    ph.x += fnl_n3 * (s.x + c.x);
    ph.y += fnl_n3 * (s.y + c.y);
    phi[e] = ph;
  }
}

// ------------------------------------------------------------------ 2LPT
// Folded 2LPT spectra of slab s (lpt_factor, main.c:1180-1368).  KIND 0:
// the six Hessians -k_a k_b T/(D Beta) phi.  KIND 1: psi1_a = i k_a T/(D
// Beta) smth phi (0..2) and psi2_a = -i k_a / k^2 smth S (3..5).
template <int KIND>
__global__ void __launch_bounds__(256) k_slab_fold_lpt(SlabGeo a, LptArgs la, const float2* __restrict__ phi,
                                                       const float2* __restrict__ src, const float2* __restrict__ twN,
                                                       float2* __restrict__ out) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.sf; t += (int64_t)gridDim.x * blockDim.x) {
    int k1, ky, kz;
    slab_cell(t, a, k1, ky, kz);
    const int ys = sidx(ky, a.N);
    float2 F[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) F[c] = make_float2(0.f, 0.f);
    for (int k2 = 0; k2 < a.S; ++k2) {
      const int kx = k1 + a.L * k2, xs = sidx(kx, a.N);
      const int n2 = xs * xs + ys * ys + kz * kz;
      const int64_t e = row_of(kx, ky, a.N, kXB) * a.HP + kz;
      const float2 w = slab_tw(twN, kx, a.s, a.N);
      const float2 X = mul_conj(phi[e], w);
      if constexpr (KIND == 0) {
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const float f = lpt_factor<0>(la, c, kx, ky, kz, xs, ys, n2).x;
          F[c].x = fmaf(f, X.x, F[c].x);
          F[c].y = fmaf(f, X.y, F[c].y);
        }
      } else {
        const float2 Y = mul_conj(src[e], w);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float f = lpt_factor<1>(la, c, kx, ky, kz, xs, ys, n2).y;  // i f
          F[c].x = fmaf(-f, X.y, F[c].x);
          F[c].y = fmaf(f, X.x, F[c].y);
          const float h = lpt_factor<2>(la, c, kx, ky, kz, xs, ys, n2).y;
          F[3 + c].x = fmaf(-h, Y.y, F[3 + c].x);
          F[3 + c].y = fmaf(h, Y.x, F[3 + c].y);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) out[(int64_t)c * a.sf + t] = F[c];
  }
}

// 2LPT source on the slab's real points (main.c:1284-1294), into field 0
__global__ void __launch_bounds__(256) k_slab_source(float* d, int64_t fsr, int N, int H, int64_t rows) {
  const int64_t total = rows * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / N;
    const int64_t o = row * 2 * H + (i - row * N);
    float v[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] = d[(int64_t)c * fsr + o];
    d[o] = v[0] * (v[3] + v[5]) + v[3] * v[5] - v[1] * v[1] - v[2] * v[2] - v[4] * v[4];
  }
}

// S(kx, ky, kz) (+)= e^{-2 pi i kx s / N} S_s(kx mod L, ky, kz) on every cell
__global__ void __launch_bounds__(256) k_slab_acc_plain(SlabGeo a, const float2* __restrict__ G,
                                                        const float2* __restrict__ twN, float2* dst, int first) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.sf; t += (int64_t)gridDim.x * blockDim.x) {
    int k1, ky, kz;
    slab_cell(t, a, k1, ky, kz);
    const float2 v = __ldg(G + t);
    for (int k2 = 0; k2 < a.S; ++k2) {
      const int kx = k1 + a.L * k2;
      const int64_t e = row_of(kx, ky, a.N, kXB) * a.HP + kz;
      const float2 u = cmul(v, slab_tw(twN, kx, a.s, a.N));
      if (first) {
        dst[e] = u;
      } else {
        const float2 o = dst[e];
        dst[e] = make_float2(o.x + u.x, o.y + u.y);
      }
    }
  }
}

// The six real slab fields into the plan's displacement fields (work slots
// 0..5: real rows of 2 HP floats in the x-blocked row order).
__global__ void __launch_bounds__(256) k_slab_scatter(SlabGeo a, const float* __restrict__ src, int64_t sfr, float* dst,
                                                      int64_t ffr) {
  const int64_t per = (int64_t)a.L * a.N * a.N;
  const int64_t total = 6 * per;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / per);
    const int64_t rem = i - c * per;
    const int64_t row = rem / a.N;  // j N + y
    const int z = (int)(rem - row * a.N);
    const int j = (int)(row / a.N), y = (int)(row - (int64_t)j * a.N);
    const int x = a.s + a.S * j;
    dst[(int64_t)c * ffr + row_of(x, y, a.N, kXB) * 2 * a.HP + z] = src[(int64_t)c * sfr + row * 2 * a.H + z];
  }
}

// ------------------------------------------------------------------ host
static SlabState* st_of(Plan* p) { return (SlabState*)p->slab; }

void slab_free(Plan* p) {
  SlabState* s = st_of(p);
  if (!s) return;
  if (s->have_c2r) cufftDestroy(s->c2r);
  if (s->have_r2c) cufftDestroy(s->r2c);
  if (s->fft_work) {
    cudaFree(s->fft_work);
    p->used_bytes -= s->fft_alloc;
  }
  delete s;
  p->slab = nullptr;
}

static int cufft_err(Plan* p, const char* what, cufftResult r) {
  return set_err(p, std::string(what) + " failed (cufftResult " + std::to_string((int)r) + ")"), AAR_ERR_CUDA;
}

// Check the slab count of a plan's parameters (N even, N % S == 0, N / S >=
// 2, x-blocked rows: N % 4 == 0).
int slab_check(const aar_params& q, std::string& why) {
  const int N = q.nmesh, S = q.nslab;
  if (!(N >= 8 && N <= 2048 && N % kXB == 0)) return why = "slab form supports Nmesh = 8..2048, a multiple of 4", 1;
  if (S < 1 || N % S != 0 || N / S < 2) return why = "slab form: nslab must divide Nmesh with Nmesh / nslab >= 2", 1;
  return 0;
}

// The potential field, the arena (as the plan's work fields) and the cuFFT
// plans; redone when the mode or slot count changes the arena size.
int slab_setup(Plan* p) {
  const int N = p->N, S = p->prm.nslab, L = N / S, H = N / 2 + 1;
  const int M = p->M;
  const int R = (p->nr_active > 0 && p->prm.fnl != 0) ? p->nr_active : 0;
  const int64_t sf = (int64_t)L * N * H, ff = (int64_t)N * N * p->HP;
  const size_t modal = R ? (size_t)(2 * ff + (int64_t)(M + R) * sf) : 0;
  const size_t arena = std::max(modal, (size_t)(7 * ff + 6 * sf));
  SlabState* s = st_of(p);
  int rc;
  cufftResult r;
  if (!p->d_phik && (rc = plan_alloc(p, (void**)&p->d_phik, sizeof(float2) * (size_t)ff))) return rc;
  if (!s) {
    s = new SlabState();
    p->slab = s;
    s->S = S;
    s->L = L;
    s->H = H;
    s->sf = sf;
    s->ff = ff;
    size_t w1 = 0, w2 = 0;
    if ((r = cufftCreate(&s->c2r)) != CUFFT_SUCCESS) return cufft_err(p, "cufftCreate", r);
    s->have_c2r = true;
    if ((r = cufftCreate(&s->r2c)) != CUFFT_SUCCESS) return cufft_err(p, "cufftCreate", r);
    s->have_r2c = true;
    cufftSetAutoAllocation(s->c2r, 0);
    cufftSetAutoAllocation(s->r2c, 0);
    if ((r = cufftMakePlan3d(s->c2r, L, N, N, CUFFT_C2R, &w1)) != CUFFT_SUCCESS) return cufft_err(p, "cufftMakePlan3d C2R", r);
    if ((r = cufftMakePlan3d(s->r2c, L, N, N, CUFFT_R2C, &w2)) != CUFFT_SUCCESS) return cufft_err(p, "cufftMakePlan3d R2C", r);
    s->fft_need = std::max<size_t>(std::max(w1, w2), 256);
  }
  if (s->fft_work && s->fft_alloc < s->fft_need) {
    cudaFree(s->fft_work);
    p->used_bytes -= s->fft_alloc;
    s->fft_work = nullptr;
    s->fft_alloc = 0;
  }
  if (!s->fft_work) {
    if ((rc = plan_alloc(p, &s->fft_work, s->fft_need))) return rc;
    s->fft_alloc = s->fft_need;
    if ((r = cufftSetWorkArea(s->c2r, s->fft_work)) != CUFFT_SUCCESS) return cufft_err(p, "cufftSetWorkArea", r);
    if ((r = cufftSetWorkArea(s->r2c, s->fft_work)) != CUFFT_SUCCESS) return cufft_err(p, "cufftSetWorkArea", r);
  }
  if (!(s->arena == arena && p->d_work)) {
    if (p->d_work) {
      cudaFree(p->d_work);
      p->used_bytes -= sizeof(float2) * s->arena;
      p->d_work = nullptr;
      p->nwork = 0;
      s->arena = 0;
    }
    p->disp_real = false;
    if ((rc = plan_alloc(p, (void**)&p->d_work, sizeof(float2) * arena))) return rc;
    s->arena = arena;
  }
  s->M = M;
  s->R = R;
  p->nwork = 6;
  return AAR_OK;
}

#define SLAB_LAUNCH(name, ...)                 \
  do {                                         \
    ProfScope ps_(p, name, st);                \
    __VA_ARGS__;                               \
    AAR_CUDA_TRY(p, cudaGetLastError());       \
    p->last_launches += 1;                     \
  } while (0)

template <class F>
static int by_modes(int m, F&& f) {
  if (m <= 8) return f(std::integral_constant<int, 8>{});
  if (m <= 16) return f(std::integral_constant<int, 16>{});
  if (m <= 24) return f(std::integral_constant<int, 24>{});
  return f(std::integral_constant<int, 32>{});
}

// noise is in the potential (run_noise); leaves the total potential in
// d_phik and the six real displacement fields in work slots 0..5
int slab_run(Plan* p, cudaStream_t st) {
  int rc = slab_setup(p);
  if (rc) return rc;
  SlabState* s = st_of(p);
  const int N = p->N, S = s->S, L = s->L, H = s->H, M = p->M, R = s->R;
  const int64_t sf = s->sf, ff = s->ff;
  const unsigned nb = (unsigned)(p->num_sms * 8);
  cufftSetStream(s->c2r, st);
  cufftSetStream(s->r2c, st);
  auto c2r = [&](float2* x) -> int {
    ProfScope ps_(p, "slab_c2r", st);
    cufftResult r = cufftExecC2R(s->c2r, (cufftComplex*)x, (cufftReal*)x);
    return r == CUFFT_SUCCESS ? AAR_OK : cufft_err(p, "cufftExecC2R", r);
  };
  auto r2c = [&](float2* x) -> int {
    ProfScope ps_(p, "slab_r2c", st);
    cufftResult r = cufftExecR2C(s->r2c, (cufftReal*)x, (cufftComplex*)x);
    return r == CUFFT_SUCCESS ? AAR_OK : cufft_err(p, "cufftExecR2C", r);
  };
  // n consecutive slab fields from x, one (L, N, N) transform each (measured:
  // cuFFT's batched plans of the same transforms were slower -- 230 vs 159 ms
  // for the 256 C2R of a 1024^3 step -- and needed a larger work area)
  auto c2r_n = [&](float2* x, int n) -> int {
    for (int i = 0; i < n; ++i) {
      int rc2 = c2r(x + (int64_t)i * s->sf);
      if (rc2) return rc2;
    }
    return AAR_OK;
  };
  auto r2c_n = [&](float2* x, int n) -> int {
    for (int i = 0; i < n; ++i) {
      int rc2 = r2c(x + (int64_t)i * s->sf);
      if (rc2) return rc2;
    }
    return AAR_OK;
  };
  SlabGeo geo{p->grid, N, p->HP, H, L, S, 0, sf};
  auto herm = [&](float2* x, int nf) -> int {
    SLAB_LAUNCH("slab_herm", k_slab_herm<<<nb, 256, 0, st>>>(x, nf, sf, L, N, H));
    return AAR_OK;
  };
  float2* phi = p->d_phik;
  const float2* twN = p->d_twN;
  if (R > 0) {
    const RhoArgs ra = rho_args(p);
    float2* acc_s = p->d_work;
    float2* acc_c = acc_s + ff;
    float2* f = acc_c + ff;
    float2* g = f + (int64_t)M * sf;
    // product terms by target r (slot = ascending active r)
    static_assert(sizeof(SlabTerms) < 32000, "kernel parameter space");
    SlabTerms tm;
    SlotMap smap{};
    {
      const TermList& tl = *(const TermList*)p->host_terms.data();
      const Term* ft = (const Term*)(p->host_terms.data() + sizeof(TermList));
      tm.M = M;
      tm.nr = tl.nr;
      int k = 0;
      for (int j = 0; j < tl.nr; ++j) {
        const int r = tl.r_of_slot[j];
        smap.active |= 1u << r;
        smap.rmax = std::max(smap.rmax, r);
        smap.slot[r] = j;
        tm.begin[j] = k;
        for (int i = 0; i < tl.nterms; ++i)
          if (ft[i].r == r) {
            tm.p[k] = (uint16_t)ft[i].p;
            tm.q[k] = (uint16_t)ft[i].q;
            tm.c[k] = ft[i].c;
            ++k;
          }
      }
      tm.begin[tl.nr] = k;
    }
    for (int sl_i = 0; sl_i < S; ++sl_i) {
      geo.s = sl_i;
      rc = by_modes(M, [&](auto mc) {
        constexpr int MM = decltype(mc)::value;
        SLAB_LAUNCH("slab_fold", k_slab_fold_modal<MM><<<nb, 256, 0, st>>>(geo, ra, M, phi, twN, f));
        return AAR_OK;
      });
      if (rc) return rc;
      if ((rc = herm(f, M))) return rc;
      if ((rc = c2r_n(f, M))) return rc;
      SLAB_LAUNCH("slab_products", k_slab_products<<<2 * nb, kProdThreads, 0, st>>>(tm, (const float*)f, (float*)g,
                                                                                     2 * sf, N, H, (int64_t)L * N));
      if ((rc = r2c_n(g, R))) return rc;
      rc = by_modes(smap.rmax + 1, [&](auto mc) {
        constexpr int MM = decltype(mc)::value;
        SLAB_LAUNCH("slab_acc", k_slab_acc_modal<MM><<<nb, 256, 0, st>>>(geo, ra, smap, g, twN, acc_s, acc_c, sl_i == 0));
        return AAR_OK;
      });
      if (rc) return rc;
    }
    const float fnl_n3 = (float)(p->prm.fnl / ((double)N * N * N));
    SLAB_LAUNCH("slab_combine", k_slab_combine<<<nb, 256, 0, st>>>(p->grid, N, p->HP, phi, acc_s, acc_c, fnl_n3));
  }
  // 2LPT: source spectrum in slot 6, slab fields after it
  const LptArgs la = lpt_args(p);
  float2* Sk = p->d_work + 6 * ff;
  float2* h = Sk + ff;
  for (int sl_i = 0; sl_i < S; ++sl_i) {
    geo.s = sl_i;
    SLAB_LAUNCH("slab_lpt_fold_hess", k_slab_fold_lpt<0><<<nb, 256, 0, st>>>(geo, la, phi, nullptr, twN, h));
    if ((rc = herm(h, 6))) return rc;
    if ((rc = c2r_n(h, 6))) return rc;
    SLAB_LAUNCH("slab_lpt_source", k_slab_source<<<nb, 256, 0, st>>>((float*)h, 2 * sf, N, H, (int64_t)L * N));
    if ((rc = r2c(h))) return rc;
    SLAB_LAUNCH("slab_lpt_acc", k_slab_acc_plain<<<nb, 256, 0, st>>>(geo, h, twN, Sk, sl_i == 0));
  }
  for (int sl_i = 0; sl_i < S; ++sl_i) {
    geo.s = sl_i;
    SLAB_LAUNCH("slab_lpt_fold_disp", k_slab_fold_lpt<1><<<nb, 256, 0, st>>>(geo, la, phi, Sk, twN, h));
    if ((rc = herm(h, 6))) return rc;
    if ((rc = c2r_n(h, 6))) return rc;
    SLAB_LAUNCH("slab_scatter", k_slab_scatter<<<nb, 256, 0, st>>>(geo, (const float*)h, 2 * sf, (float*)p->d_work,
                                                                    2 * ff));
  }
  p->disp_real = true;
  return AAR_OK;
}

}  // namespace aar
