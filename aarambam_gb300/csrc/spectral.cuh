// Kernel parameter blocks and per-cell spectral factors shared by the
// forward passes (fused.cu) and the adjoint kernels (adjoint.cu).
#pragma once
#include "aar_internal.cuh"

namespace aar {

struct Term {      // one product f_p f_q with coefficient c into g_r
  int p, q, r;
  float c;
};

constexpr int kMaxTerms = 2048;

struct TermList {
  int nterms, nr;
  int r_of_slot[kMaxModes];       // active r values (ascending)
  int begin[kMaxModes + 1];       // terms of slot s: [begin[s], begin[s+1])
};

struct ModalArgs {
  Grid g;
  int M;
};

struct LptArgs {
  ModalArgs m;        // grid and k helpers
  float inv_Dbeta;    // 1 / (Dplus Beta)
  const float* twb;   // per n^2: T(k) / (Dplus Beta)
  const float* sinc;  // per grid index: sin(x)/x, x = k Box / 2N (1 at k = 0)
  const float* isinc2;  // per grid index: 1 / sinc^2
  float box_over_2n;
};

ModalArgs modal_args(Plan* p);
LptArgs lpt_args(Plan* p);

// The 2LPT spectral factors of main.c:1180-1368 at one cell (grid indices
// i, j of x, y; kz; signed kx, ky; n2 = |k|^2 in grid units), as complex
// multipliers of phi (or of the source S for MODE 2):
//   MODE 0  Hessian ab:   -k_a k_b T/(D Beta)          (comp 0..5 = 00 01 02 11 12 22)
//   MODE 1  ZA psi1_a:    i k_a T/(D Beta) smth
//   MODE 2  2LPT psi2_a: -i k_a / k^2 smth            (0 at k = 0)
// smth = [sinc_x sinc_y sinc_z]^-2 (CORRECT_CIC).  TWB = false leaves out
// the T/(D Beta) factor, for a phi that already carries it.
template <int MODE, bool TWB = true>
__device__ __forceinline__ float2 lpt_factor(const LptArgs& a, int comp, int i, int j, int kz, int kx, int ky, int n2) {
  const float kF = a.m.g.kF;
  const int ax = MODE == 0 ? (comp < 3 ? 0 : (comp < 5 ? 1 : 2)) : comp;
  const float ka = kF * (float)(ax == 0 ? kx : ax == 1 ? ky : kz);
  if (MODE == 0) {
    const int bx = comp == 0 ? 0 : comp == 1 ? 1 : comp == 2 ? 2 : comp == 3 ? 1 : 2;
    const float kb = kF * (float)(bx == 0 ? kx : bx == 1 ? ky : kz);
    return make_float2(TWB ? -ka * kb * __ldg(a.twb + n2) : -ka * kb, 0.f);
  }
  const float ff = 1.f / (__ldg(a.sinc + i) * __ldg(a.sinc + j) * __ldg(a.sinc + kz));
  const float smth = ff * ff;
  if (MODE == 1) return make_float2(0.f, TWB ? ka * __ldg(a.twb + n2) * smth : ka * smth);
  if (n2 == 0) return make_float2(0.f, 0.f);
  return make_float2(0.f, -ka / (kF * kF * (float)n2) * smth);
}

}  // namespace aar
