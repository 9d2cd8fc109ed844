// FP32 line FFTs for sm_103a: register DFTs of radix 2..32 with compile-time
// twiddles, composed into Stockham auto-sort stages that exchange through a
// padded shared-memory line buffer.  A line of length N is owned by T lanes of
// one warp (E = N / T values per lane); a warp may own several short lines.
//
// Stage formulation: Govindaraju et al., "High performance discrete Fourier
// transforms on graphics processors", SC'08, Fig. 2 (iteration j, radix R,
// span Ns: inputs x[j + r N/R], twiddle exp(s 2 pi i r (j mod Ns)/(Ns R)),
// outputs y[(j/Ns) Ns R + (j mod Ns) + r Ns]).
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#include <stdint.h>
#else
typedef long long int64_t;
typedef unsigned int uint32_t;
#endif

namespace aar {

// ---------------------------------------------------------------- complex
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// --------------------------------------------- compile-time trigonometry
// cos / sin of 2 pi k / n evaluated by quadrant reduction and Taylor series
// in double precision during compilation.
__host__ __device__ constexpr double ce_sin_small(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int n = 1; n < 14; ++n) {
    term *= -x2 / ((2.0 * n) * (2.0 * n + 1));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double ce_cos_small(double x) {
  double x2 = x * x, term = 1, sum = 1;
  for (int n = 1; n < 14; ++n) {
    term *= -x2 / ((2.0 * n - 1) * (2.0 * n));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double ce_cos2pi(long k, long n) {
  long t = ((k % n) + n) % n;
  long q = (4 * t) / n, r = 4 * t - q * n;
  double a = 1.5707963267948966192313216916397514 * (double)r / (double)n;
  double c = ce_cos_small(a), s = ce_sin_small(a);
  return q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}
__host__ __device__ constexpr double ce_sin2pi(long k, long n) {
  long t = ((k % n) + n) % n;
  long q = (4 * t) / n, r = 4 * t - q * n;
  double a = 1.5707963267948966192313216916397514 * (double)r / (double)n;
  double c = ce_cos_small(a), s = ce_sin_small(a);
  return q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
}

// multiply by exp(SIGN * 2 pi i K / R) with the trivial angles special-cased
template <int R, int K, int SIGN>
__device__ __forceinline__ float2 twiddle_ct(float2 v) {
  constexpr int k = ((K % R) + R) % R;
  if constexpr (k == 0) {
    return v;
  } else if constexpr (4 * k == R) {  // SIGN * i
    return SIGN < 0 ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  } else if constexpr (2 * k == R) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (4 * k == 3 * R) {  // -SIGN * i
    return SIGN < 0 ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  } else {
    constexpr float c = (float)ce_cos2pi(k, R);
    constexpr float s = (float)(SIGN * ce_sin2pi(k, R));
    return make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
  }
}

// ------------------------------------------------------ register DFTs
// In-place DFT of R values, natural order in and out: X_k = sum x_r w^{rk},
// w = exp(SIGN 2 pi i / R).  Radix-2 decimation in time, fully unrolled.
template <int R, int SIGN>
struct DFT {
  template <int K>
  static __device__ __forceinline__ void combine(float2* v, const float2* e, const float2* o) {
    if constexpr (K < R / 2) {
      float2 t = twiddle_ct<R, K, SIGN>(o[K]);
      v[K] = cadd(e[K], t);
      v[K + R / 2] = csub(e[K], t);
      combine<K + 1>(v, e, o);
    }
  }
  static __device__ __forceinline__ void run(float2* v) {
    if constexpr (R == 1) {
      return;
    } else if constexpr (R == 2) {
      float2 a = v[0], b = v[1];
      v[0] = cadd(a, b);
      v[1] = csub(a, b);
    } else if constexpr (R == 4) {
      float2 s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
      float2 s1 = cadd(v[1], v[3]), d1 = csub(v[1], v[3]);
      float2 rd1 = twiddle_ct<4, 1, SIGN>(d1);
      v[0] = cadd(s0, s1);
      v[2] = csub(s0, s1);
      v[1] = cadd(d0, rd1);
      v[3] = csub(d0, rd1);
    } else {
      float2 e[R / 2], o[R / 2];
#pragma unroll
      for (int i = 0; i < R / 2; ++i) {
        e[i] = v[2 * i];
        o[i] = v[2 * i + 1];
      }
      DFT<R / 2, SIGN>::run(e);
      DFT<R / 2, SIGN>::run(o);
      combine<0>(v, e, o);
    }
  }
};

// ------------------------------------------------------ stage planning
// Radix of stage s for a line of length N with E values per lane: the
// largest power of two <= E that divides what is left of N.
__host__ __device__ constexpr int stage_radix(int N, int E, int s) {
  int left = N, r = 1;
  for (int i = 0; i <= s; ++i) {
    r = 1;
    while (r * 2 <= E && left % (r * 2) == 0) r *= 2;
    if (i < s) left /= r;
  }
  return left == 1 ? 1 : r;
}
__host__ __device__ constexpr int stage_span(int N, int E, int s) {  // Ns before stage s
  int ns = 1;
  for (int i = 0; i < s; ++i) ns *= stage_radix(N, E, i);
  return ns;
}
__host__ __device__ constexpr int num_stages(int N, int E) {
  int s = 0;
  while (stage_span(N, E, s) < N) ++s;
  return s;
}

// padded shared-memory index: one spare slot per 16 entries, so that the
// first Stockham stage's stores (lane j writes j R + r, R = 8 or 16) and the
// natural-order loads both fall on distinct banks within a half-warp
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int spad_len(int n) { return n + n / 16 + 4; }

// Twiddle table for length N in global memory: tw[m] = exp(-2 pi i m / N).
// Runtime twiddle exp(SIGN 2 pi i m / N).
template <int SIGN>
__device__ __forceinline__ float2 tw_load(const float2* __restrict__ tw, int m) {
  float2 w = __ldg(tw + m);
  return SIGN < 0 ? w : make_float2(w.x, -w.y);
}

// ------------------------------------------------- lane twiddle tables
// Stage S >= 1 (span Ns, radix R) multiplies input r of the group of line
// index j by exp(SIGN 2 pi i r k (N / (Ns R)) / N), k = j mod Ns: per lane a
// function of k only, the same for every line.  A block keeps them in shared
// memory as lt[lt_off(S) + (r - 1) Ns + k] = exp(-2 pi i m / N), m = r k
// (N / (Ns R)), filled once per block (lt_fill), so a lane reads a stage's
// R - 1 factors as conflict-free shared loads (the lanes of one k
// broadcast) instead of R - 1 global loads per line at lane-scattered
// indices of the N-point table -- as many loads per lane and line as it has
// values, which made the twiddles the largest source of L1 wavefronts of the
// row kernel after its shared-memory stages.
__host__ __device__ constexpr int lt_off(int N, int E, int S) {
  int off = 0;
  for (int s = 1; s < S; ++s) off += (stage_radix(N, E, s) - 1) * stage_span(N, E, s);
  return off;
}
__host__ __device__ constexpr int lt_size(int N, int E) { return lt_off(N, E, num_stages(N, E)); }
// entry count rounded up to a whole 16 bytes (what follows stays aligned)
__host__ __device__ constexpr int lt_slots(int N, int E) { return (lt_size(N, E) + 1) / 2 * 2; }

// the exponent m of table entry i (0 <= i < lt_size(N, E))
template <int N, int E>
__device__ __forceinline__ int lt_exponent(int i) {
  int s = 1, off = 0;
  for (;;) {
    const int R = stage_radix(N, E, s), Ns = stage_span(N, E, s), n = (R - 1) * Ns;
    if (i < off + n) {
      const int rem = i - off;
      return (rem / Ns + 1) * (rem % Ns) * (N / (Ns * R));
    }
    off += n;
    ++s;
  }
}

// the table of an N-point line with E values per lane from tw (the table of
// a line TWS times longer), by the block's nthreads threads; ASYNC: as
// 8-byte cp.async copies (completed by the caller's cp.async wait), so the
// fill costs no round trip before the thread's other loads issue
template <int N, int E, int TWS, bool ASYNC = false>
__device__ __forceinline__ void lt_fill(float2* lt, const float2* __restrict__ tw, int tid, int nthreads) {
  for (int i = tid; i < lt_size(N, E); i += nthreads) {
    const float2* src = tw + lt_exponent<N, E>(i) * TWS;
    if constexpr (ASYNC) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(lt + i);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
    } else {
      lt[i] = __ldg(src);
    }
  }
}

// Shared-memory addresses of the stage loads and stores.  With the padding
// spad(i) = i + i/16, an index t-part + C (C a multiple of 16) pads to
// spad(t-part) + C + C/16, so a lane computes one padded base per stage and
// every other address is that base plus a compile-time constant.  This holds
// for the loads (t + T b + r N/R) when T and N/R are multiples of 16, and for
// the stores when the span Ns divides T (j/Ns = t/Ns + T b/Ns, j%Ns = t%Ns;
// the r Ns part never carries into the next 16-block together with t%Ns) or
// Ns = N/R (the last stage: base = j + r Ns).  Other shapes (short lines)
// use the plain formula.
template <int N, int T, int R>
struct LoadAddr {
  static constexpr bool kAffine = T % 16 == 0 && (N / R) % 16 == 0;
  static __device__ __forceinline__ int base(int t) { return t + (t >> 4); }
  template <int B, int RR>
  static __device__ __forceinline__ int at(int pb, int t) {
    constexpr int C = T * B + RR * (N / R);
    if constexpr (kAffine) return pb + C + C / 16;
    else return spad(t + C);
  }
};

template <int N, int T, int R, int Ns>
struct StoreAddr {
  static constexpr bool kLast = Ns * R == N;
  static constexpr bool kDivides = !kLast && T % Ns == 0 && Ns * R >= 16 && (T * R) % 16 == 0;
  static constexpr bool kAffine = kLast ? (T % 16 == 0 && Ns % 16 == 0) : kDivides;
  static __device__ __forceinline__ int base(int t) {
    if constexpr (kLast) {
      return t + (t >> 4);
    } else {
      const int u0 = (t / Ns) * Ns * R + (t % Ns);
      return u0 + (u0 >> 4);
    }
  }
  template <int B, int RR>
  static __device__ __forceinline__ int at(int pb, int t) {
    if constexpr (kAffine) {
      if constexpr (kLast) {
        constexpr int C = T * B + RR * Ns;
        return pb + C + C / 16;
      } else {
        constexpr int C = T * B * R;  // from j/Ns = t/Ns + T B/Ns
        constexpr int D = RR * Ns;
        return pb + C + C / 16 + D + (D >> 4);
      }
    } else {
      const int j = t + T * B;
      return spad((j / Ns) * Ns * R + (j % Ns) + RR * Ns);
    }
  }
};

// f.template operator()<B, RR>() for every group B < NB and RR < R
template <int B, int NB, int R, int RR = 0, class F>
__device__ __forceinline__ void unroll_br(F&& f) {
  if constexpr (B < NB) {
    if constexpr (RR < R) {
      f.template operator()<B, RR>();
      unroll_br<B, NB, R, RR + 1>(f);
    } else {
      unroll_br<B + 1, NB, R, 0>(f);
    }
  }
}

// One Stockham stage on the values a lane holds: v[b*R + r] = x[j + r N/R],
// j = t + T b.  On return v[b*R + r] = y[(j/Ns) Ns R + j%Ns + r Ns].  When Ns
// divides T the twiddle exponent k = j mod Ns = t mod Ns is the same for
// every group b, so the R - 1 twiddles are loaded once per stage.  The table
// tw holds exp(-2 pi i m / (N TWS)); TWS > 1 reads a longer line's table
// with stride TWS.
// LT: tw is the block's lane twiddle table (shared memory), LTO this
// stage's offset in it.
template <int N, int T, int R, int Ns, int SIGN, int TWS = 1, bool LT = false, int LTO = 0>
__device__ __forceinline__ float2 stage_twiddle(const float2* __restrict__ tw, int r, int k) {
  if constexpr (LT) {
    const float2 w = tw[LTO + (r - 1) * Ns + k];
    return SIGN < 0 ? w : make_float2(w.x, -w.y);
  } else {
    return tw_load<SIGN>(tw, r * k * (N / (Ns * R)) * TWS);
  }
}

template <int N, int T, int R, int Ns, int SIGN, int TWS = 1, bool LT = false, int LTO = 0>
__device__ __forceinline__ void stage_compute(float2* v, int t, const float2* __restrict__ tw) {
  constexpr int E = N / T;
  if constexpr (Ns > 1 && T % Ns == 0 && E / R > 1) {
    const int k = t % Ns;
    float2 w[R];
#pragma unroll
    for (int r = 1; r < R; ++r) w[r] = stage_twiddle<N, T, R, Ns, SIGN, TWS, LT, LTO>(tw, r, k);
#pragma unroll
    for (int b = 0; b < E / R; ++b) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], w[r]);
      DFT<R, SIGN>::run(v + b * R);
    }
  } else {
#pragma unroll
    for (int b = 0; b < E / R; ++b) {
      int j = t + T * b;
      if constexpr (Ns > 1) {
        int k = j % Ns;
#pragma unroll
        for (int r = 1; r < R; ++r)
          v[b * R + r] = cmul(v[b * R + r], stage_twiddle<N, T, R, Ns, SIGN, TWS, LT, LTO>(tw, r, k));
      }
      DFT<R, SIGN>::run(v + b * R);
    }
  }
}

// Write stage outputs into the line buffer (natural index, padded).
template <int N, int T, int R, int Ns>
__device__ __forceinline__ void stage_store(const float2* v, float2* s, int t) {
  using A = StoreAddr<N, T, R, Ns>;
  const int pb = A::base(t);
  unroll_br<0, N / T / R, R>([&]<int B, int RR>() { s[A::template at<B, RR>(pb, t)] = v[B * R + RR]; });
}

// Read the inputs of a stage of radix R from the line buffer.
template <int N, int T, int R>
__device__ __forceinline__ void stage_load(float2* v, const float2* s, int t) {
  using A = LoadAddr<N, T, R>;
  const int pb = A::base(t);
  unroll_br<0, N / T / R, R>([&]<int B, int RR>() { v[B * R + RR] = s[A::template at<B, RR>(pb, t)]; });
}

// Barrier among the T lanes that share a line: a warp barrier when the line
// lives in one warp, else the named barrier `bar_id` (1..15) over T threads.
template <int T>
__device__ __forceinline__ void line_sync(int bar_id) {
  if constexpr (T <= 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;\n" ::"r"(bar_id), "n"(T) : "memory");
  }
}

// Full line FFT.  On entry the line (natural order) is in the buffer s; on
// exit the transform is in s (natural order).  All T lanes of the line call
// this together; lanes with act == false (no line of their own) only take
// part in the barriers.  bar_id names the barrier of a line spread over
// several warps.
// SCALE multiplies the values of the first stage as they are loaded (line
// element t + T b + r N/R sits at v[b R + r]) by sc[b R + r] (SCALE 1) or by
// i sc[b R + r] (SCALE 2): a per-element filter folded into the transform.
// TWS: twiddle-table stride (tw of a line TWS times longer).  LT: tw is the
// block's lane twiddle table in shared memory (lt_fill<N, N/T, TWS>).
template <int N, int T, int SIGN, int S = 0, int SCALE = 0, int TWS = 1, bool LT = false>
__device__ __forceinline__ void line_fft_smem(float2* s, int t, const float2* __restrict__ tw, bool act,
                                              int bar_id = 1, const float* sc = nullptr) {
  constexpr int E = N / T;
  constexpr int NS = num_stages(N, E);
  if constexpr (S < NS) {
    constexpr int R = stage_radix(N, E, S);
    constexpr int Ns = stage_span(N, E, S);
    float2 v[E];
    if (act) stage_load<N, T, R>(v, s, t);
    if constexpr (S == 0 && SCALE != 0) {
#pragma unroll
      for (int i = 0; i < E; ++i)
        v[i] = SCALE == 1 ? make_float2(v[i].x * sc[i], v[i].y * sc[i]) : make_float2(-sc[i] * v[i].y, sc[i] * v[i].x);
    }
    line_sync<T>(bar_id);
    if (act) {
      stage_compute<N, T, R, Ns, SIGN, TWS, LT, lt_off(N, E, S)>(v, t, tw);
      stage_store<N, T, R, Ns>(v, s, t);
    }
    line_sync<T>(bar_id);
    line_fft_smem<N, T, SIGN, S + 1, 0, TWS, LT>(s, t, tw, act, bar_id);
  }
}

// Line index of the i-th value a lane holds after the first stage load.
template <int N, int T>
__host__ __device__ constexpr int first_load_index(int t, int i) {
  constexpr int E = N / T;
  constexpr int R = stage_radix(N, E, 0);
  return t + T * (i / R) + (i % R) * (N / R);
}

// lanes per line: 16 values per lane for N >= 512, 8 below
__host__ __device__ constexpr int lanes_for(int N) {
  return N >= 512 ? N / 16 : (N / 8 >= 1 ? (N / 8 < 32 ? N / 8 : 32) : 1);
}

// lanes per line of the strided (tile) passes: 32 values per lane for
// N >= 512, so that a 512- or 1024-point line is two Stockham stages
// (32 x 16, 32 x 32) instead of three, one warp per line.  (The row kernels
// keep lanes_for: their 512-point half lines with 32 values per lane were
// slower, 140 vs 95 ms at 1024^3.)
__host__ __device__ constexpr int lanes_for_tile(int N) { return N >= 512 ? N / 32 : lanes_for(N); }

}  // namespace aar
