// RANLUX as GSL's gsl_rng_ranlxd1 (the generator behind the reference's
// gsl_rng_uniform calls, Aarambam/LPT/Basis/main.c:317-349 and :392-403),
// for host and device, plus an exact skip-ahead.
//
// Generator: subtract-with-borrow over b = 2^48 with lags (12, 5):
//   x_n = x_{n-5} - x_{n-12} - c_{n-1} (mod b), c_n = borrow;
// after every 202 steps the 12 most recent values are delivered, oldest
// first, as x / 2^48.  Seeding: the low 31 seed bits drive
// bit_{n+31} = bit_n ^ bit_{n+18}; each of the 12 state words collects 48
// successive complemented bits, most significant first; carry 0.
//
// Skip-ahead.  With window W_t = (x_t .. x_{t+11}) and carry c_{t+11}, the
// integer K_t = P_t - b^5 Q_t - c_{t+11} b^12 (P_t = sum_{n<12} x_{t+n} b^n,
// Q_t = sum_{n<7} x_{t+n} b^n) satisfies K_{t+1} = K_t * b^{-1} (mod m),
// m = b^12 - b^5 + 1 (the b-adic number sum_n x_{t+n} b^n equals K_t / m),
// and K_t lies in [-m, 0] once t >= 13.  So the state after any number of
// steps follows from one modular product with a precomputed power of
// b^{-1}; the window digits come back as the b-adic digits of K_t / m
// (m = 1 mod b, so digit = (-V) mod b with V = -K_t) and the carry from the
// thirteenth digit.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define AAR_HD __host__ __device__ __forceinline__
#else
#define AAR_HD inline
#endif

namespace aar {

constexpr int kRlxLux = 202;  // ranlxd1
constexpr uint64_t kMask48 = (uint64_t(1) << 48) - 1;

struct Rlx {
  uint64_t x[12];  // canonical: x[0] oldest
  uint32_t carry;
  int pos;
};

AAR_HD void rlx_seed(Rlx& s, uint32_t seed) {
  if (seed == 0) seed = 1;
  uint32_t bits = seed & 0x7FFFFFFFu;  // 31-bit register, bit k = seed bit k
  int ib = 0, jb = 18;
  for (int w = 0; w < 12; ++w) {
    uint64_t word = 0;
    for (int l = 0; l < 48; ++l) {
      uint32_t bi = (bits >> ib) & 1u, bj = (bits >> jb) & 1u;
      word = (word << 1) | (bi ^ 1u);
      bits ^= (bj << ib);
      ib = (ib == 30) ? 0 : ib + 1;
      jb = (jb == 30) ? 0 : jb + 1;
    }
    s.x[w] = word;
  }
  s.carry = 0;
  s.pos = 12;
}

// 202 SWB steps on the canonical window, then rotate so x[0] is oldest.
// 202 = 16*12 + 10: sixteen full sweeps and a tail of 10 keep every index a
// compile-time constant (the state stays in registers).
AAR_HD void rlx_refill(Rlx& s) {
  uint64_t x0 = s.x[0], x1 = s.x[1], x2 = s.x[2], x3 = s.x[3], x4 = s.x[4], x5 = s.x[5], x6 = s.x[6],
           x7 = s.x[7], x8 = s.x[8], x9 = s.x[9], x10 = s.x[10], x11 = s.x[11];
  uint64_t c = s.carry;
#define AAR_SWB(a, b)                          \
  {                                            \
    uint64_t d = (b) - (a)-c;                  \
    c = d >> 63;                               \
    (a) = d & kMask48;                         \
  }
#pragma unroll 1
  for (int sweep = 0; sweep < 16; ++sweep) {
    AAR_SWB(x0, x7) AAR_SWB(x1, x8) AAR_SWB(x2, x9) AAR_SWB(x3, x10) AAR_SWB(x4, x11) AAR_SWB(x5, x0)
    AAR_SWB(x6, x1) AAR_SWB(x7, x2) AAR_SWB(x8, x3) AAR_SWB(x9, x4) AAR_SWB(x10, x5) AAR_SWB(x11, x6)
  }
  AAR_SWB(x0, x7) AAR_SWB(x1, x8) AAR_SWB(x2, x9) AAR_SWB(x3, x10) AAR_SWB(x4, x11) AAR_SWB(x5, x0)
  AAR_SWB(x6, x1) AAR_SWB(x7, x2) AAR_SWB(x8, x3) AAR_SWB(x9, x4)
#undef AAR_SWB
  // newest are x0..x9, oldest x10, x11
  s.x[0] = x10; s.x[1] = x11; s.x[2] = x0; s.x[3] = x1; s.x[4] = x2; s.x[5] = x3;
  s.x[6] = x4; s.x[7] = x5; s.x[8] = x6; s.x[9] = x7; s.x[10] = x8; s.x[11] = x9;
  s.carry = (uint32_t)c;
  s.pos = 0;
}

// raw 48-bit output; the uniform is raw * 2^-48
AAR_HD uint64_t rlx_next48(Rlx& s) {
  if (s.pos == 12) rlx_refill(s);
  return s.x[s.pos++];
}

// ------------------------------------------------------------ 576-bit math
struct U576 {
  uint64_t w[9];
};

AAR_HD void mul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
#ifdef __CUDA_ARCH__
  lo = a * b;
  hi = __umul64hi(a, b);
#else
  unsigned __int128 p = (unsigned __int128)a * b;
  lo = (uint64_t)p;
  hi = (uint64_t)(p >> 64);
#endif
}

// m = 2^576 - 2^240 + 1
AAR_HD U576 u576_m() {
  U576 m;
  m.w[0] = 1;
  m.w[1] = 0;
  m.w[2] = 0;
  m.w[3] = 0xFFFF000000000000ull;
  for (int i = 4; i < 9; ++i) m.w[i] = ~0ull;
  return m;
}

// r = a - b on n limbs, returns borrow
AAR_HD uint64_t limbs_sub(uint64_t* r, const uint64_t* a, const uint64_t* b, int n) {
  uint64_t br = 0;
  for (int i = 0; i < n; ++i) {
    uint64_t ai = a[i], bi = b[i];
    uint64_t d = ai - bi;
    uint64_t b1 = ai < bi;
    uint64_t d2 = d - br;
    uint64_t b2 = d < br;
    r[i] = d2;
    br = b1 | b2;
  }
  return br;
}
AAR_HD uint64_t limbs_add(uint64_t* r, const uint64_t* a, const uint64_t* b, int n) {
  uint64_t cy = 0;
  for (int i = 0; i < n; ++i) {
    uint64_t s = a[i] + b[i];
    uint64_t c1 = s < a[i];
    uint64_t s2 = s + cy;
    uint64_t c2 = s2 < s;
    r[i] = s2;
    cy = c1 | c2;
  }
  return cy;
}
AAR_HD bool limbs_geq(const uint64_t* a, const uint64_t* b, int n) {
  for (int i = n - 1; i >= 0; --i) {
    if (a[i] != b[i]) return a[i] > b[i];
  }
  return true;
}

// Fold a value given as 14 limbs (value < 2^896) modulo m using
// 2^576 = 2^240 - 1: v = L + H 2^576 -> L + (H << 240) - H.  Result < 2^577
// in 10 limbs (non-negative).
AAR_HD void fold576(const uint64_t* v, int nlimb, uint64_t* out10) {
  uint64_t L[14] = {0}, H[14] = {0}, S[14] = {0};
  for (int i = 0; i < 9 && i < nlimb; ++i) L[i] = v[i];
  for (int i = 9; i < nlimb; ++i) H[i - 9] = v[i];
  // S = H << 240 (240 = 3*64 + 48)
  for (int i = 0; i < 14; ++i) {
    uint64_t lo = (i - 3 >= 0 && i - 3 < 14) ? H[i - 3] : 0;
    uint64_t lo2 = (i - 4 >= 0 && i - 4 < 14) ? H[i - 4] : 0;
    S[i] = (lo << 48) | (lo2 >> 16);
  }
  uint64_t T[14];
  limbs_add(T, L, S, 14);
  limbs_sub(T, T, H, 14);  // T >= 0 since S >= H
  for (int i = 0; i < 10; ++i) out10[i] = T[i];
  // the caller guarantees T < 2^640 (10 limbs) for the inputs used below
}

// r = a * b mod m, a, b < m
AAR_HD U576 modmul576(const U576& a, const U576& b) {
  uint64_t P[18] = {0};
  for (int i = 0; i < 9; ++i) {
    uint64_t cy = 0;
    for (int j = 0; j < 9; ++j) {
      uint64_t lo, hi;
      mul64(a.w[i], b.w[j], lo, hi);
      uint64_t s = P[i + j] + lo;
      uint64_t c1 = s < lo;
      uint64_t s2 = s + cy;
      uint64_t c2 = s2 < s;
      P[i + j] = s2;
      cy = hi + c1 + c2;  // cannot overflow: hi <= 2^64 - 2
    }
    P[i + 9] = cy;
  }
  // first fold: P < 2^1152 -> T = L + (H << 240) - H < 2^817
  uint64_t L[14] = {0}, H[14] = {0}, S[14] = {0}, T[14];
  for (int i = 0; i < 9; ++i) {
    L[i] = P[i];
    H[i] = P[i + 9];
  }
  for (int i = 0; i < 14; ++i) {
    uint64_t lo = (i >= 3 && i - 3 < 9) ? H[i - 3] : 0;
    uint64_t lo2 = (i >= 4 && i - 4 < 9) ? H[i - 4] : 0;
    S[i] = (lo << 48) | (lo2 >> 16);
  }
  limbs_add(T, L, S, 14);
  limbs_sub(T, T, H, 14);
  // second fold: T < 2^817 -> < 2^577
  uint64_t L2[14] = {0}, H2[14] = {0}, S2[14] = {0}, U[14];
  for (int i = 0; i < 9; ++i) L2[i] = T[i];
  for (int i = 9; i < 14; ++i) H2[i - 9] = T[i];
  for (int i = 0; i < 14; ++i) {
    uint64_t lo = (i >= 3 && i - 3 < 5) ? H2[i - 3] : 0;
    uint64_t lo2 = (i >= 4 && i - 4 < 5) ? H2[i - 4] : 0;
    S2[i] = (lo << 48) | (lo2 >> 16);
  }
  limbs_add(U, L2, S2, 14);
  limbs_sub(U, U, H2, 14);
  // U < 2^577 + small; subtract m while U >= m
  U576 m = u576_m();
  uint64_t mm[10], u10[10];
  for (int i = 0; i < 9; ++i) mm[i] = m.w[i];
  mm[9] = 0;
  for (int i = 0; i < 10; ++i) u10[i] = U[i];
  for (int it = 0; it < 3; ++it)
    if (limbs_geq(u10, mm, 10)) limbs_sub(u10, u10, mm, 10);
  U576 r;
  for (int i = 0; i < 9; ++i) r.w[i] = u10[i];
  return r;
}

// K_0 mod m of a seeded window (carry 0): P - b^5 Q, reduced into [0, m).
AAR_HD U576 rlx_window_residue(const Rlx& s) {
  // P = sum x_n b^n packs 12 48-bit digits into 576 bits; Q: first 7 digits
  uint64_t P[10] = {0}, Q5[10] = {0};
  for (int n = 0; n < 12; ++n) {
    int bit = 48 * n, li = bit >> 6, sh = bit & 63;
    P[li] |= s.x[n] << sh;
    if (sh > 16) P[li + 1] |= s.x[n] >> (64 - sh);
  }
  for (int n = 0; n < 7; ++n) {  // b^5 Q: digit n at bit 48 (n + 5)
    int bit = 48 * (n + 5), li = bit >> 6, sh = bit & 63;
    Q5[li] |= s.x[n] << sh;
    if (sh > 16) Q5[li + 1] |= s.x[n] >> (64 - sh);
  }
  U576 m = u576_m();
  uint64_t mm[10];
  for (int i = 0; i < 9; ++i) mm[i] = m.w[i];
  mm[9] = 0;
  uint64_t R[10];
  if (limbs_geq(P, Q5, 10)) {
    limbs_sub(R, P, Q5, 10);  // in [0, 2^576)
    while (limbs_geq(R, mm, 10)) limbs_sub(R, R, mm, 10);
  } else {
    uint64_t D[10];
    limbs_sub(D, Q5, P, 10);  // -K in (0, 2^576)
    while (limbs_geq(D, mm, 10)) limbs_sub(D, D, mm, 10);
    // R = m - D (or 0)
    bool zero = true;
    for (int i = 0; i < 10; ++i) zero = zero && D[i] == 0;
    if (zero)
      for (int i = 0; i < 10; ++i) R[i] = 0;
    else
      limbs_sub(R, mm, D, 10);
  }
  U576 r;
  for (int i = 0; i < 9; ++i) r.w[i] = R[i];
  return r;
}

// Rebuild the window from the residue R of K_t (t >= 13): V = m - R = -K_t,
// digit = (-V) mod b, V <- (V + m digit) / b; carry from the 13th digit.
AAR_HD void rlx_from_residue(const U576& R, Rlx& s) {
  U576 m = u576_m();
  uint64_t V[10];
  {
    uint64_t mm[10], rr[10];
    for (int i = 0; i < 9; ++i) {
      mm[i] = m.w[i];
      rr[i] = R.w[i];
    }
    mm[9] = rr[9] = 0;
    limbs_sub(V, mm, rr, 10);
  }
  uint64_t dig[13];
  for (int n = 0; n < 13; ++n) {
    uint64_t d = (0 - V[0]) & kMask48;
    dig[n] = d;
    // V += m * d   (m * d = d 2^576 - d 2^240 + d)
    uint64_t md[10] = {0};
    for (int i = 0; i < 9; ++i) {
      uint64_t lo, hi;
      mul64(m.w[i], d, lo, hi);
      uint64_t s0 = md[i] + lo;
      uint64_t c0 = s0 < lo;
      md[i] = s0;
      md[i + 1] += hi + c0;
    }
    limbs_add(V, V, md, 10);
    // V >>= 48
    for (int i = 0; i < 9; ++i) V[i] = (V[i] >> 48) | (V[i + 1] << 16);
    V[9] >>= 48;
  }
  for (int n = 0; n < 12; ++n) s.x[n] = dig[n];
  // x_{t+12} = x_{t+7} - x_t - c_{t+11} + b c_{t+12}  =>  c_{t+11} = (x_{t+7} - x_t - x_{t+12}) mod b
  s.carry = (uint32_t)((dig[7] - dig[0] - dig[12]) & kMask48);
  s.pos = 12;
}

// b^{-1} mod m = m - b^11 + b^4  (b (b^11 - b^4) = b^12 - b^5 = -1 mod m)
AAR_HD U576 u576_binv() {
  U576 m = u576_m();
  uint64_t mm[10], t[10] = {0}, r[10];
  for (int i = 0; i < 9; ++i) mm[i] = m.w[i];
  mm[9] = 0;
  // b^11 = 2^528: limb 8 bit 16; b^4 = 2^192: limb 3 bit 0
  t[8] = uint64_t(1) << 16;
  limbs_sub(r, mm, t, 10);
  uint64_t b4[10] = {0};
  b4[3] = 1;
  limbs_add(r, r, b4, 10);
  U576 o;
  for (int i = 0; i < 9; ++i) o.w[i] = r[i];
  return o;
}

AAR_HD U576 u576_one() {
  U576 o;
  for (int i = 0; i < 9; ++i) o.w[i] = 0;
  o.w[0] = 1;
  return o;
}

AAR_HD U576 modpow576(U576 a, uint64_t e) {
  U576 r = u576_one();
  while (e) {
    if (e & 1) r = modmul576(r, a);
    a = modmul576(a, a);
    e >>= 1;
  }
  return r;
}

}  // namespace aar
