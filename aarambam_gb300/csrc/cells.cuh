// Per-cell geometry of the half spectrum, shared by the library's kernels
// and the run-time specialised ones (jit.cu, NVRTC): row order, signed
// wavenumbers, the reference's keep/cut rule and the per-cell mode
// functions of the modal accumulation.  Device code and plain structs only.
#pragma once
#include "fft.cuh"

namespace aar {

constexpr int kMaxModes = 32;  // modes of a plan (slots of the term list)

constexpr double kPi = 3.14159265358979323846;  // PI as the reference defines it

// signed wavenumber index of grid index i (main.c:410-423): N/2 -> -N/2
__host__ __device__ __forceinline__ int sidx(int i, int N) { return i < N / 2 ? i : i - N; }

// Row order of the fused form's fields.  A field (complex half-spectrum or
// real) is N^2 rows of HP complex / 2 HP real values, one row per (x, y);
// the row of (x, y) is row_of(x, y, N, xb), i.e. x is split into blocks of
// xb: [x / xb][y][x % xb].  With xb = kXB the N rows of an x line lie in
// N / kXB groups of kXB rows 4*HP bytes apart, instead of N rows N*HP*8 bytes
// apart: measured on GB300 at N = 1024, a tile copy with the x-pass pattern
// ran at 3.4 TB/s in natural order and 6.7 TB/s blocked (xb = 4 to 64),
// while the y-pass pattern stayed at 7.0-7.2 TB/s for xb <= 8.  xb = 1 is
// the natural [x][y] order of the reference and of the C-ABI's buffers.
constexpr int kXB = 4;
__host__ __device__ __forceinline__ int64_t row_of(int x, int y, int N, int xb) {
  return ((int64_t)(x / xb) * N + y) * xb + x % xb;
}
__host__ __device__ __forceinline__ void row_xy(int64_t m, int N, int xb, int& x, int& y) {
  const int64_t q = m / xb;
  x = (int)((q / N) * xb + m % xb);
  y = (int)(q % N);
}

// Geometry and scalars of one plan, passed by value to kernels.
struct Grid {
  int N;       // Nmesh
  int HP;      // padded half-spectrum row length (complex entries), >= N/2+1
  int kcut;    // cube mode: keep |k index| <= kcut on every axis
  int sphere;  // SphereMode
  int nsq_bnd; // sphere mode: (Nsample/2)^2, the only n^2 whose keep depends on rounding
  int nsample_half;
  double box;
  float kF;    // 2 pi / Box
};

// Keep / cut decision of the reference (main.c:428-441, :591-604), exact.
// Cube mode reduces to an integer bound on each axis (host-computed).  In
// sphere mode only n^2 == (Nsample/2)^2 sits on the rounding boundary; those
// cells repeat the reference's FP64 expression with unfused operations.
__device__ __forceinline__ bool keep_cell(const Grid& g, int kx, int ky, int kz) {
  if (!g.sphere) return abs(kx) <= g.kcut && abs(ky) <= g.kcut && abs(kz) <= g.kcut;
  int n2 = kx * kx + ky * ky + kz * kz;
  if (n2 != g.nsq_bnd) return n2 < g.nsq_bnd;
  double fx = __ddiv_rn(__dmul_rn((double)(2 * kx), kPi), g.box);
  double fy = __ddiv_rn(__dmul_rn((double)(2 * ky), kPi), g.box);
  double fz = __ddiv_rn(__dmul_rn((double)(2 * kz), kPi), g.box);
  double k2 = __dadd_rn(__dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fy, fy)), __dmul_rn(fz, fz));
  double km = __dsqrt_rn(k2);
  return !(__ddiv_rn(__dmul_rn(km, g.box), __dmul_rn(2.0, kPi)) > (double)g.nsample_half);
}

// rho_n(k) of the accumulation evaluated per cell (main.c:825-860):
// k^(s (n-3)) for n <= 3, (P_{n-1}(kbar) - X0[n-1]) / k^2 above, with
// kbar = -1 + 2 (k^s - kmin^s)/(kmax^s - kmin^s); kmin = kF, so
// k^s - kmin^s = kmin^s expm1(s ln(sqrt(n^2))) (no cancellation near kmin),
// and P_l by the Bonnet recurrence P_l = A_l kbar P_{l-1} - B_l P_{l-2}.
struct RhoArgs {
  float s, c1, log2kF, inv_kF2;  // c1 = 2 kmin^s / (kmax^s - kmin^s)
  float e4, e2;                  // 4 - ns, 2 - ns (exponents of the field filters)
  float x0[kMaxModes];
  float A[kMaxModes], B[kMaxModes];  // (2l-1)/l, (l-1)/l
};

// Field filter q_n(k) of main.c:580-637 at K cells (n2[i] = |k|^2 in grid
// units, > 0) in FP32: k^(s (n-3)) k^(4-ns) for n <= 3, (P_{n-1}(kbar) -
// X0[n-1]) k^(2-ns) above, with P_l as for rho_n (RhoArgs).  With k = kF
// sqrt(n2) and kmin = kF, kbar = -1 + c1 (n2^(s/2) - 1): for integer n2 >= 1
// the bracket is 0 or at least 2^(s/2) - 1 ~ 0.42, so it has no cancellation
// and the hardware base-2 logarithm and exponential (absolute error ~2^-22
// in the exponent; ~4e-7 relative in q) replace logf / expm1f: three
// special-function operations per cell.  The K recurrences run in lockstep
// (K independent chains per step).
template <int K>
__device__ __forceinline__ void q_mode_cells(const RhoArgs& ra, int n, const int* n2, float* out) {
  float lg[K];
#pragma unroll
  for (int i = 0; i < K; ++i) lg[i] = __log2f((float)n2[i]);  // log2 n2
  if (n <= 3) {
    const float e = ra.s * (float)(n - 3) + ra.e4;
#pragma unroll
    for (int i = 0; i < K; ++i) out[i] = exp2f(e * fmaf(0.5f, lg[i], ra.log2kF));
    return;
  }
  float kb[K], P0[K], P1[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    kb[i] = fmaf(ra.c1, exp2f(0.5f * ra.s * lg[i]), -1.f - ra.c1);
    P0[i] = 1.f;
    P1[i] = kb[i];
  }
  for (int l = 2; l < n; ++l) {
    const float A = ra.A[l], B = ra.B[l];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const float Pn = A * kb[i] * P1[i] - B * P0[i];
      P0[i] = P1[i];
      P1[i] = Pn;
    }
  }
  const float x0 = ra.x0[n - 1];
#pragma unroll
  for (int i = 0; i < K; ++i) out[i] = (P1[i] - x0) * exp2f(ra.e2 * fmaf(0.5f, lg[i], ra.log2kF));
}

// Neumaier's compensated step: s + c carries the running sum of the t's
__device__ __forceinline__ void neumaier_add(float& s, float& c, float t) {
  const float u = s + t;
  c += (fabsf(s) >= fabsf(t)) ? (s - u) + t : (t - u) + s;
  s = u;
}

}  // namespace aar
