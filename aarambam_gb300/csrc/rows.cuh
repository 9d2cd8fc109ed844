// Row (z) kernels: the real <-> half-complex transform of contiguous rows
// and the generic per-row "c2r, combine, r2c" body.  Device code only, so
// that it compiles both in this library and in the run-time specialised
// row kernel (jit.cu, NVRTC).
#pragma once
#include "fft.cuh"

namespace aar {

// asynchronous global -> shared copies (sm_80+ cp.async), 8 bytes each
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory");
}


// Per-axis real factor of the 2LPT y pass and c2r rows (index k along the
// axis; y uses the signed index, z the column index kz = 0..N/2): 0: 1,
// 1: k, 2: k^2, 3: 1/sinc^2, 4: kF k / sinc^2 (isinc2 = 1/sinc^2 per grid
// index gi).
__device__ __forceinline__ float axis_factor(int type, int k, float kF, const float* __restrict__ isinc2, int gi) {
  if (type == 0) return 1.f;
  if (type == 1) return (float)k;
  if (type == 2) return (float)k * (float)k;
  const float is2 = __ldg(isinc2 + gi);
  return type == 3 ? is2 : kF * (float)k * is2;
}

// z factor of a row's spectrum, applied as the c2r pre-step reads X_k
struct ZFac {
  int type;  // axis_factor type, 0 = none
  float kF;
  const float* isinc2;
  __device__ __forceinline__ float at(int k) const { return axis_factor(type, k, kF, isinc2, k); }
};

// Row layout: complex row X[0..N/2] at field + m HP, m the row's memory
// index (the plan's row order maps (x, y) to m); the real row x[0..N-1]
// occupies the same bytes (float2 z_n = (x_{2n}, x_{2n+1})).  The row steps
// are the same for every row, so the kernels run over memory rows.
template <int N>
struct RowCfg {
  static constexpr int H = N / 2;             // complex FFT length
  // 16 values per lane from H = 256 up (two stages of 16 x 16 at H = 256,
  // measured 6.2 vs 7.3 ms for the modal rows at 512^3; at H = 128 eight
  // lanes per line made the 256^3 batch slower, 139 vs 127 ms)
  static constexpr int T = H == 256 ? 16 : lanes_for(H);
  static constexpr int LPW = 32 / T;
  static constexpr int LS = spad_len(H);
};

// load X_k (k = 0..N/2) of a row and form Z_k = E_k + i O_k for the
// inverse half-length FFT (FFTW c2r semantics: Im X_0, Im X_{N/2} dropped)
template <int N>
__device__ __forceinline__ void row_c2r_pre(const float2* __restrict__ X, float2* line, int t, int T,
                                            const float2* __restrict__ twN, ZFac zf = ZFac{0, 0.f, nullptr}) {
  constexpr int H = N / 2;
  for (int k = t; k <= H / 2; k += T) {
    int k2 = H - k;
    float2 a = X[k], b = X[k2];
    if (zf.type) {
      a = cscale(a, zf.at(k));
      b = cscale(b, zf.at(k2));
    }
    if (k == 0) {
      a.y = 0.f;
      b.y = 0.f;
    }
    // E_k = X_k + conj(X_{H-k}); O_k = (X_k - conj(X_{H-k})) e^{+2 pi i k / N}
    float2 w = __ldg(twN + k);
    w.y = -w.y;
    float2 e = make_float2(a.x + b.x, a.y - b.y);
    float2 d = make_float2(a.x - b.x, a.y + b.y);
    float2 o = cmul(d, w);
    line[spad(k)] = make_float2(e.x - o.y, e.y + o.x);
    if (k2 != k && k2 < H) {
      // Z_{H-k}: E = X_{H-k} + conj(X_k), O = (X_{H-k} - conj(X_k)) e^{+2 pi i (H-k)/N}
      float2 w2 = __ldg(twN + k2);
      w2.y = -w2.y;
      float2 e2 = make_float2(b.x + a.x, b.y - a.y);
      float2 d2 = make_float2(b.x - a.x, b.y + a.y);
      float2 o2 = cmul(d2, w2);
      line[spad(k2)] = make_float2(e2.x - o2.y, e2.y + o2.x);
    }
  }
}

// The same pre-step in place, on X_0..X_{N/2} already staged in `line`
// (element k at spad(k)): each lane rewrites the pair (k, H - k) it reads.
template <int N>
__device__ __forceinline__ void row_c2r_pre_inplace(float2* line, int t, int T, const float2* __restrict__ twN,
                                                    ZFac zf = ZFac{0, 0.f, nullptr}) {
  constexpr int H = N / 2;
  for (int k = t; k <= H / 2; k += T) {
    int k2 = H - k;
    float2 a = line[spad(k)], b = line[spad(k2)];
    if (zf.type) {
      a = cscale(a, zf.at(k));
      b = cscale(b, zf.at(k2));
    }
    if (k == 0) {
      a.y = 0.f;
      b.y = 0.f;
    }
    float2 w = __ldg(twN + k);
    w.y = -w.y;
    float2 e = make_float2(a.x + b.x, a.y - b.y);
    float2 d = make_float2(a.x - b.x, a.y + b.y);
    float2 o = cmul(d, w);
    line[spad(k)] = make_float2(e.x - o.y, e.y + o.x);
    if (k2 != k && k2 < H) {
      float2 w2 = __ldg(twN + k2);
      w2.y = -w2.y;
      float2 e2 = make_float2(b.x + a.x, b.y - a.y);
      float2 d2 = make_float2(b.x - a.x, b.y + a.y);
      float2 o2 = cmul(d2, w2);
      line[spad(k2)] = make_float2(e2.x - o2.y, e2.y + o2.x);
    }
  }
}

// after the forward half-length FFT of z_n = (x_{2n}, x_{2n+1}) in `line`,
// write X_k = (Z_k + conj Z_{H-k})/2 - i e^{-2 pi i k/N} (Z_k - conj Z_{H-k})/2
template <int N>
__device__ __forceinline__ void row_r2c_post(const float2* line, float2* __restrict__ X, int t, int T,
                                             const float2* __restrict__ twN) {
  constexpr int H = N / 2;
  for (int k = t; k <= H; k += T) {
    float2 z = line[spad(k % H)], zc = line[spad((H - k) % H)];
    zc.y = -zc.y;
    float2 e = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
    float2 d = make_float2(0.5f * (z.x - zc.x), 0.5f * (z.y - zc.y));
    float2 w = (k < H) ? __ldg(twN + k) : make_float2(-1.f, 0.f);
    float2 od = cmul(d, w);  // e^{-2 pi i k/N} d
    X[k] = make_float2(e.x + od.y, e.y - od.x);  // e - i od
  }
}

// ---------------------------------------------------------------------
// Rows of N = 1024 (half-length H = 512) fold the radix-2 step of the
// half-length transform into the c2r pre-step and the r2c post-step, so a
// line takes two shared-memory stages (two H/2-point transforms of radix
// 16 x 16 on the half-warps) instead of three (16 x 16 x 2).  Lane `lane`
// of the warp owns the quads of positions k, h-k, h+k, H-k (h = H/2,
// k = lane + 32 i <= H/4); the quads partition 0..H, so the steps work in
// place without a barrier.
//
// Inverse: Z_n from X (the pre-step), then decimation in frequency:
// u_n = Z_n + Z_{n+h} to position n and (Z_n - Z_{n+h}) e^{2 pi i n/H} to
// n + h, n < h.  Inverse h-point transforms of the two halves leave z_{2m}
// at m and z_{2m+1} at h + m (z_n = (x_{2n}, x_{2n+1})): the line's samples
// in a permuted order, which the pointwise combine does not see.
// Forward, from that order: E_k (first half) and O_k (second half) after
// the h-point transforms, Z_k = E_k + e^{-2 pi i k/H} O_k and Z_{k+h} =
// E_k - e^{-2 pi i k/H} O_k, then the post-step X_k from Z_k, Z_{H-k}.
template <int N>
struct RowFold {
  static constexpr bool value = N == 1024;
};

// float2 slots of the lane twiddle table (fft.cuh) of the folded rows'
// H/2-point half-line transforms, at the start of their shared memory
// (filled once per block of M + R lines: the modal rows at 1024^3 with 20
// modes 67.9 -> 60.8 ms, the source rows 11.1 -> 10.6 ms)
template <int N>
__host__ __device__ constexpr int row_lt_slots() {
  return RowFold<N>::value ? lt_slots(N / 4, 16) : 0;
}

// Z_j of the c2r pre-step from a = X_j, b = X_{H-j}, w = e^{+2 pi i j/N}:
// E + i O with E = a + conj b, O = (a - conj b) w
__device__ __forceinline__ float2 pre1(float2 a, float2 b, float2 w) {
  const float2 e = make_float2(a.x + b.x, a.y - b.y);
  const float2 o = cmul(make_float2(a.x - b.x, a.y + b.y), w);
  return make_float2(e.x - o.y, e.y + o.x);
}
// X_j of the r2c post-step from z = Z_j, zr = Z_{H-j}, w = e^{-2 pi i j/N}
__device__ __forceinline__ float2 post1(float2 z, float2 zr, float2 w) {
  const float2 e = make_float2(0.5f * (z.x + zr.x), 0.5f * (z.y - zr.y));
  const float2 od = cmul(make_float2(0.5f * (z.x - zr.x), 0.5f * (z.y + zr.y)), w);
  return make_float2(e.x + od.y, e.y - od.x);
}

// The folded steps walk the quads k = lane + 32 it < Q in Q / 32 rounds; the
// quad k = Q, which has two outputs only (positions Q and H - Q, where its
// first and second output pairs coincide), rides with lane 0's first quad
// k = 0, which has no second pair: lane 0 computes that pair from the quad
// k = Q instead.  (With k = Q a round of its own, a fifth round ran a whole
// warp for one quad.)  At j = Q the twiddles of the two pair formulas agree:
// conj w_Q = i w_Q and -v_Q = conj v_Q (w_Q = e^{-i pi/4}, v_Q = -i).

// Inverse pre-step into the line buffer, from X in global memory (src):
// first pair (Z_k + Z_{k+h}, (Z_k - Z_{k+h}) e^{2 pi i k/H}) to positions k
// and h + k from the quad at k; second pair to positions h - k2 and H - k2
// from the quad at k2 (k2 = k, or Q for lane 0's first quad).
template <int N>
__device__ __forceinline__ void row_c2r_pre_fold(float2* line, int lane, const float2* __restrict__ twN,
                                                 const float2* __restrict__ twH, ZFac zf,
                                                 const float2* __restrict__ src) {
  constexpr int H = N / 2, h = H / 2, Q = H / 4;
  static_assert(Q % 32 == 0, "folded rows: whole rounds of quads");
  constexpr int NIT = Q / 32;
  // all of the lane's loads first (independent, in flight together), then
  // the quads: the loads of one quad do not wait for the previous quad's
  // arithmetic and stores
  float2 qa[NIT], qb[NIT], qc[NIT], qd[NIT];
#pragma unroll
  for (int it = 0; it < NIT; ++it) {
    const int k = lane + 32 * it;
    qa[it] = src[k];
    qb[it] = src[H - k];
    qc[it] = src[h - k];
    qd[it] = src[h + k];
  }
  const float2 xq = src[Q], x3q = src[H - Q];  // the quad k = Q: X_Q, X_{H-Q} (= X_{h-Q}, X_{h+Q})
  const float2 wQ = __ldg(twN + Q), vQ = __ldg(twH + Q);
#pragma unroll
  for (int it = 0; it < NIT; ++it) {
    const int k = lane + 32 * it;
    const bool l0 = it == 0 && lane == 0;
    float2 a = qa[it], b = qb[it], c = qc[it], d = qd[it];
    const int k2 = l0 ? Q : k;
    const float2 wk = __ldg(twN + k), vk = __ldg(twH + k);
    const float2 w2 = l0 ? wQ : wk, v2 = l0 ? vQ : vk;
    float2 a2 = l0 ? xq : a, b2 = l0 ? x3q : b, c2 = l0 ? xq : c, d2 = l0 ? x3q : d;
    if (zf.type) {
      a = cscale(a, zf.at(k));
      b = cscale(b, zf.at(H - k));
      c = cscale(c, zf.at(h - k));
      d = cscale(d, zf.at(h + k));
      a2 = l0 ? cscale(a2, zf.at(Q)) : a;
      b2 = l0 ? cscale(b2, zf.at(H - Q)) : b;
      c2 = l0 ? cscale(c2, zf.at(Q)) : c;
      d2 = l0 ? cscale(d2, zf.at(H - Q)) : d;
    }
    if (k == 0) {  // FFTW c2r: Im X_0, Im X_{N/2} dropped
      a.y = 0.f;
      b.y = 0.f;
    }
    // e^{+2 pi i j/N} at j = k, h+k: conj w, i conj w; at j = H-k2, h-k2: -w, i w
    const float2 zk = pre1(a, b, make_float2(wk.x, -wk.y));
    const float2 zhp = pre1(d, c, make_float2(wk.y, wk.x));
    const float2 zHk = pre1(b2, a2, make_float2(-w2.x, -w2.y));
    const float2 zhm = pre1(c2, d2, make_float2(-w2.y, w2.x));
    // butterflies n = k and n = h - k2; e^{2 pi i n/H}: conj v, -v
    line[spad(k)] = cadd(zk, zhp);
    line[spad(h + k)] = cmul(csub(zk, zhp), make_float2(vk.x, -vk.y));
    line[spad(h - k2)] = cadd(zhm, zHk);
    line[spad(H - k2)] = cmul(csub(zhm, zHk), make_float2(-v2.x, -v2.y));
  }
}

// Forward post-step from the line buffer to X (global): per quad k the four
// outputs X_k, X_{H-k}, X_{h-k}, X_{h+k}; lane 0's first quad gives X_0,
// X_H, X_h from k = 0 (Z_0 = E_0 + O_0 = Z_H, Z_h = E_0 - O_0) in the same
// three formulas with its operands selected, and X_Q, X_{H-Q} from the quad
// k = Q in the fourth and a fifth.
template <int N>
__device__ __forceinline__ void row_r2c_post_fold(const float2* line, float2* __restrict__ X, int lane,
                                                  const float2* __restrict__ twN, const float2* __restrict__ twH) {
  constexpr int H = N / 2, h = H / 2, Q = H / 4;
  static_assert(Q % 32 == 0, "folded rows: whole rounds of quads");
  constexpr int NIT = Q / 32;
  const float2 wQ = __ldg(twN + Q), vQ = __ldg(twH + Q);
#pragma unroll
  for (int it = 0; it < NIT; ++it) {
    const int k = lane + 32 * it;
    const bool l0 = it == 0 && lane == 0;
    const int k2 = l0 ? Q : k;
    const float2 wk = __ldg(twN + k), vk = __ldg(twH + k);
    const float2 v2 = l0 ? vQ : vk;
    const float2 ek = line[spad(k)], ok = cmul(line[spad(h + k)], vk);
    const float2 zk = cadd(ek, ok), zhp = csub(ek, ok);
    // Z_{h-k2} = E - conj(v) O, Z_{H-k2} = E + conj(v) O from positions h - k2, H - k2
    const float2 em = line[spad(h - k2)], om = cmul(line[spad(H - k2)], make_float2(v2.x, -v2.y));
    const float2 zhm = csub(em, om), zHk = cadd(em, om);
    // e^{-2 pi i j/N} at j = k, H-k, h-k, h+k: w, -conj w, -i conj w, -i w
    X[k] = post1(zk, l0 ? zk : zHk, wk);
    X[H - k] = post1(l0 ? zk : zHk, zk, make_float2(-wk.x, wk.y));
    X[h - k] = post1(l0 ? zhp : zhm, zhp, make_float2(-wk.y, -wk.x));
    if (l0) {
      X[Q] = post1(zhm, zHk, wQ);
      X[H - Q] = post1(zHk, zhm, make_float2(-wQ.x, wQ.y));
    } else {
      X[h + k] = post1(zhp, zhm, make_float2(wk.y, -wk.x));
    }
  }
}

// Generic row kernel.  For each memory row (blockIdx.x): c2r of `nin`
// input fields (slots in_slot[]), a per-position combine step Op, r2c of
// `nout` output lines into slots out_slot[].  One warp per line at a time.
// THREADS = 256 (the library's kernels; the NVRTC kernel may use 320) with
// two resident blocks per SM: while one block waits at a phase barrier (its
// last round of lines keeps only some warps busy) the other block's warps
// issue.
constexpr int kRowThreads = 256;
template <int N, class Op, int THREADS = kRowThreads>
__device__ __forceinline__ void rows_body(const Op& op, float2* work, int64_t fs, int HP,
                                          const float2* __restrict__ twN, const float2* __restrict__ twH) {
  using C = RowCfg<N>;
  constexpr int H = C::H;
  extern __shared__ float2 sm_all[];
  float2* sm = sm_all + row_lt_slots<N>();  // line buffers after the lane twiddles
  int64_t row = blockIdx.x;
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int nwarps = THREADS / 32;
  int sub = lane / C::T, t = lane % C::T;
  // phase 0: stage X_0..X_{N/2} of every input line at once (one exposed
  // memory latency per row instead of one per line; staging round by round
  // with a barrier per round measured slower: 148 vs 141 ms at 1024^3).
  // The folded rows read X in their pre-step straight from global memory
  // (staged: 83.6 vs 73.4 ms at 1024^3); the other sizes keep the staging
  // (reading in the pre-step: 7.44 vs 7.27 ms for the modal rows at 512^3
  // with 8 values per lane, 7.29 vs 6.21 ms with 16).
  if constexpr (!RowFold<N>::value) {
    for (int l = 0; l < op.nin(); ++l) {
      const float2* X = work + (int64_t)op.in_slot(l) * fs + row * HP;
      float2* line = sm + l * C::LS;
      for (int k = threadIdx.x; k <= H; k += THREADS) cp_async8(line + spad(k), X + k);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
  }
  if constexpr (RowFold<N>::value) {
    static_assert(C::T == 32 && H == 512, "folded rows: one warp per 512-point half line");
    constexpr int h = H / 2, HO = h + h / 16;  // spad(h + i) = spad(i) + HO
    const int half = lane >> 4, t16 = lane & 15;
    const float2* lt = sm_all;
    lt_fill<h, 16, 2>(sm_all, twH, threadIdx.x, THREADS);
    __syncthreads();
    for (int l = warp; l < op.nin(); l += nwarps) {
      float2* line = sm + l * C::LS;
      const float2* X = work + (int64_t)op.in_slot(l) * fs + row * HP;
      if constexpr (Op::kZfac) row_c2r_pre_fold<N>(line, lane, twN, twH, op.zfac(l), X);
      else row_c2r_pre_fold<N>(line, lane, twN, twH, ZFac{0, 0.f, nullptr}, X);
      __syncwarp();
      line_fft_smem<h, 16, +1, 0, 0, 2, true>(line + half * HO, t16, lt, true);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < H; n += (Op::kPairs ? 2 : 1) * THREADS) {
      if (Op::kPairs && n + THREADS < H) {
        const int pos[2] = {spad(n), spad(n + THREADS)};
        op.template combine<2>(sm, pos, C::LS);
      } else {
        const int pos[1] = {spad(n)};
        op.template combine<1>(sm, pos, C::LS);
      }
    }
    __syncthreads();
    for (int l = warp; l < op.nout(); l += nwarps) {
      float2* line = sm + op.out_line(l) * C::LS;
      line_fft_smem<h, 16, -1, 0, 0, 2, true>(line + half * HO, t16, lt, true);
      row_r2c_post_fold<N>(line, work + (int64_t)op.out_slot(l) * fs + row * HP, lane, twN, twH);
      __syncwarp();
    }
    return;
  }
  // phase 1: inverse transforms
  for (int l0 = warp * C::LPW; l0 < op.nin(); l0 += nwarps * C::LPW) {
    int l = l0 + sub;
    bool act = l < op.nin() && sub < C::LPW;
    float2* line = sm + (act ? l : 0) * C::LS;
    if (act) {
      if constexpr (Op::kZfac) row_c2r_pre_inplace<N>(line, t, C::T, twN, op.zfac(l));
      else row_c2r_pre_inplace<N>(line, t, C::T, twN);
    }
    __syncwarp();
    line_fft_smem<H, C::T, +1>(line, t, twH, act);
  }
  __syncthreads();
  // phase 2: per position combine (in place in the line buffers)
  for (int n = threadIdx.x; n < H; n += (Op::kPairs ? 2 : 1) * THREADS) {
    if (Op::kPairs && n + THREADS < H) {
      const int pos[2] = {spad(n), spad(n + THREADS)};
      op.template combine<2>(sm, pos, C::LS);
    } else {
      const int pos[1] = {spad(n)};
      op.template combine<1>(sm, pos, C::LS);
    }
  }
  __syncthreads();
  // phase 3: forward transforms of the output lines
  for (int l0 = warp * C::LPW; l0 < op.nout(); l0 += nwarps * C::LPW) {
    int l = l0 + sub;
    bool act = l < op.nout() && sub < C::LPW;
    float2* line = sm + (act ? op.out_line(l) : 0) * C::LS;
    line_fft_smem<H, C::T, -1>(line, t, twH, act);
    if (act) row_r2c_post<N>(line, work + (int64_t)op.out_slot(l) * fs + row * HP, t, C::T, twN);
    __syncwarp();
  }
}

}  // namespace aar
