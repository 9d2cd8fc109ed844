// Fused FP32 form of the Aarambam IC path on sm_103a.
//
// Fields live in HBM as complex half spectra float2 [N][N][HP] (HP >= N/2+1,
// a multiple of 8 so rows are 64-byte aligned); after a c2r the same buffer
// holds the real field as float [N][N][2 HP] (z fastest).  A 3-D transform is
// three passes, each reading and writing a field once:
//   x pass / y pass  -- strided complex FFTs on tiles of W consecutive kz
//                       columns x N rows, staged through shared memory;
//   z pass (rows)    -- the real<->half-complex transform of contiguous rows
//                       as an N/2-point complex FFT plus the usual
//                       even/odd split twiddle step.
// The reference's per-pass work is fused into these passes:
//   modal potential (Aarambam/LPT/Basis/main.c:564-1151) regrouped exactly by
//   linearity of the DFT: acc = sum_r rho_r(k) r2c[ g_r ],
//   g_r(x) = sum_{p<=q} a'_{pqr} f_p(x) f_q(x), f_p = c2r[ q_p(k) phi(k) ],
//   with a' = alpha on sorted triples plus the two counter-terms of
//   main.c:1045-1050.  The x pass that starts every f_p reads phi once and
//   applies q_p; one row kernel does all c2r's, products and r2c's of a row;
//   the last x pass applies rho_r, sums over r and adds Fnl acc / N^3.
//   2LPT (main.c:1156-1381): Hessians straight from phi (-k_a k_b T/(D Beta)),
//   the source in the row kernel, Poisson + CIC deconvolution fused into the
//   x pass that also starts the six displacement c2r's.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <stddef.h>

#include <algorithm>
#include <vector>

#include "aar_internal.cuh"
#include "fft.cuh"
#include "rows.cuh"
#include "spectral.cuh"

namespace aar {


// term list in plan-owned device memory (read uniformly by all threads)
struct DevTerms {
  TermList tl;
  Term t[kMaxTerms];
};
size_t terms_bytes() { return sizeof(DevTerms); }

// ----------------------------------------------------------- tile passes
// Line stride of a tile in shared memory: at least the padded line length,
// and = 2 (mod 16) float2 so that the 8 lines x 2 rows a half-warp touches
// while moving a tile between global and shared memory fall in 32 distinct
// banks.
__host__ __device__ constexpr int tile_ls(int N) {
  int base = N + N / 16;
  return base + ((2 - base % 16) + 16) % 16;
}

template <int N, int W>
struct AxisCfg {
  static constexpr int T = lanes_for_tile(N);  // lanes per line
  static constexpr int E = N / T;
  static constexpr int THREADS = ((W * T + 31) / 32) * 32;
  static constexpr int WARPS = THREADS / 32;
  static constexpr int LS = tile_ls(N);  // smem line stride (float2)
  static constexpr size_t SMEM = sizeof(float2) * (size_t)W * LS;
  static constexpr int PER = N * W / THREADS;  // tile elements per thread
  // resident blocks per SM aimed at: 32 values per lane need ~128 registers
  static constexpr int MINB = E >= 32 ? (THREADS >= 256 ? 2 : 4) : THREADS >= 512 ? 2 : 4;
};

// Tile indexing.  Axis 0 (x): rows n = x, other index o = y.  Axis 1 (y):
// rows n = y, o = x.  Column w covers kz = c0 + w.  Fields are in the
// x-blocked row order row_of(x, y, N, kXB).
// Tile element ownership: thread t owns column w = t % W and rows
// n = t / W + q THREADS/W, q < PER; with THREADS/W a multiple of 16 the
// padded shared index and the global offset are a per-thread base plus a
// compile-time (shared) or per-launch (global) stride times q.
template <int N, int W, int AXIS>
struct TileAddr {
  using C = AxisCfg<N, W>;
  static constexpr int DN = C::THREADS / W;  // row step between a thread's elements
  int w, n0, sbase;
  int64_t gbase, gstep;
  __device__ __forceinline__ TileAddr(int HP, int o, int c0) {
    w = threadIdx.x % W;
    n0 = threadIdx.x / W;
    sbase = w * C::LS + spad(n0);
    // a thread's rows n0 + q DN keep n0 % kXB, so the offsets stay affine in q
    static_assert(DN % kXB == 0, "row step of a tile thread must be a multiple of the x block");
    if (AXIS == 0) {
      gbase = row_of(n0, o, N, kXB) * HP + c0 + w;
      gstep = (int64_t)DN * N * HP;
    } else {
      gbase = row_of(o, n0, N, kXB) * HP + c0 + w;
      gstep = (int64_t)DN * kXB * HP;
    }
  }
  __device__ __forceinline__ int s(int q) const {
    if constexpr (DN % 16 == 0) return sbase + q * (DN + DN / 16);
    else return w * C::LS + spad(n0 + q * DN);
  }
  __device__ __forceinline__ int64_t g(int q) const { return gbase + q * gstep; }
};

// issue the asynchronous copy of a tile (rows along AXIS) into shared memory
template <int N, int W, int AXIS>
__device__ __forceinline__ void tile_load_async(float2* sm, const float2* __restrict__ f, int HP, int o, int c0) {
  using C = AxisCfg<N, W>;
  const TileAddr<N, W, AXIS> ta(HP, o, c0);
#pragma unroll 4
  for (int q = 0; q < C::PER; ++q) cp_async8(sm + ta.s(q), f + ta.g(q));
}

template <int N, int W, int AXIS>
__device__ __forceinline__ void tile_store(const float2* sm, float2* __restrict__ f, int HP, int o, int c0) {
  using C = AxisCfg<N, W>;
  const TileAddr<N, W, AXIS> ta(HP, o, c0);
#pragma unroll 4
  for (int q = 0; q < C::PER; ++q) f[ta.g(q)] = sm[ta.s(q)];
}

// run the W line FFTs of a tile held in shared memory (SCALE: optional
// per-element factors of the first stage, see line_fft_smem).  The second
// stage reads its twiddles from the global table: a per-block shared-memory
// lane table (fft.cuh, as the row kernels use) made every tile pass at
// 1024^3 slower (y pass 42.7 -> 46.7 ms with the table filled by cp.async
// while the tile loads, 49.6 filled by plain loads).
template <int N, int W, int SIGN, int SCALE = 0>
__device__ __forceinline__ void tile_fft(float2* sm, const float2* __restrict__ tw, const float* sc = nullptr) {
  using C = AxisCfg<N, W>;
  // lines spread over several warps synchronise on named barriers 1..W;
  // barrier ids stop at 15
  static_assert(C::T <= 32 || W <= 15, "too many multi-warp lines per tile for the named barriers");
  int line = threadIdx.x / C::T;
  int t = threadIdx.x % C::T;
  bool act = line < W;
  line_fft_smem<N, C::T, SIGN, 0, SCALE>(sm + (act ? line : 0) * C::LS, t, tw, act, 1 + (act ? line : 0), sc);
}

// Last modal step, after the forward x transform of every active slot r:
// acc = sum_r rho_r(k) g_r(k) (rho_r computed per cell in FP32, RhoArgs;
// Neumaier-compensated in registers), then phi <- phi + fnl_n3 * acc,
// DC = 0 (main.c:1101-1126).
// One thread per half-spectrum element (padding columns are not touched);
// cut cells keep phi as it is.  A streaming kernel: the R slot reads of a
// thread are independent, so many are in flight per SM.  (Measured: pairs of
// cells per thread with 16-byte loads were slower, 36.5 vs 30.8 ms at
// 1024^3; so was the slot list as a kernel parameter, 39.0 ms, and the rho
// row read with 16-byte loads into registers and the slots walked with
// compile-time indices, 38.0 ms.  Gathering rho_r from a per-|k|^2 table,
// one load per slot, left the kernel waiting on those loads: 31.4 ms.  The
// slot loads issued in chunks of eight ahead of their sums: 48 registers,
// five blocks per SM, 34.5 vs 28.9 ms.)
template <int N>
__global__ void __launch_bounds__(256) k_modal_acc(ModalArgs a, float2* phi, const float2* __restrict__ work,
                                                   int64_t fs, int HP, float fnl_n3, const DevTerms* __restrict__ dt,
                                                   const RhoArgs ra) {
  constexpr int K = N / 2 + 1;  // kz = 0 .. N/2 of a row
  constexpr int64_t total = (int64_t)N * N * K;
  // the active slots and their field bases, once per block
  __shared__ int rs[kMaxModes];
  __shared__ const float2* base[kMaxModes];
  const int nr = dt->tl.nr;
  if (threadIdx.x < nr) {
    const int r = dt->tl.r_of_slot[threadIdx.x];
    rs[threadIdx.x] = r;
    base[threadIdx.x] = work + (int64_t)r * fs;
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / K;
    const int kz = (int)(i - row * K);
    const int64_t e = row * HP + kz;
    int x, y;
    row_xy(row, N, kXB, x, y);
    const int kx = sidx(x, N), ky = sidx(y, N);
    const int n2 = kx * kx + ky * ky + kz * kz;
    if (n2 == 0) {
      phi[e] = make_float2(0.f, 0.f);
      continue;
    }
    if (!keep_cell(a.g, kx, ky, kz)) continue;
    const float lnn2 = logf((float)n2);
    const float kbar = -1.f + ra.c1 * expm1f(0.5f * ra.s * lnn2);
    const float L = ra.log2kF + lnn2 * 0.72134752044448170368f;  // log2 k = log2 kF + ln(n2) / (2 ln 2)
    const float inv_k2 = ra.inv_kF2 / (float)n2;
    float P0 = 1.f, P1 = kbar;  // P_{deg-1}, P_deg
    int deg = 1;
    float sx = 0.f, sy = 0.f, cx = 0.f, cy = 0.f;
#pragma unroll 4
    for (int k = 0; k < nr; ++k) {
      const int r = rs[k];
      const float2 v = __ldg(base[k] + e);
      float rho;
      if (r <= 3) {
        rho = r == 3 ? 1.f : exp2f(ra.s * (float)(r - 3) * L);
      } else {
        while (deg < r - 1) {
          ++deg;
          const float Pn = ra.A[deg] * kbar * P1 - ra.B[deg] * P0;
          P0 = P1;
          P1 = Pn;
        }
        rho = (P1 - ra.x0[r - 1]) * inv_k2;
      }
      const float tx = v.x * rho, ty = v.y * rho;
      const float ux = sx + tx, uy = sy + ty;
      cx += (fabsf(sx) >= fabsf(tx)) ? (sx - ux) + tx : (tx - ux) + sx;
      cy += (fabsf(sy) >= fabsf(ty)) ? (sy - uy) + ty : (ty - uy) + sy;
      sx = ux;
      sy = uy;
    }
    float2 ph = phi[e];
    ph.x += fnl_n3 * (sx + cx);
    ph.y += fnl_n3 * (sy + cy);
    phi[e] = ph;
  }
}

// phi_T = T(k)/(D Beta) phi on every half-spectrum cell (padding columns
// are not touched): the factor the Hessians and psi1 share.
template <int N>
__global__ void __launch_bounds__(256) k_scale_twb(const float2* __restrict__ phi, float2* out, int HP,
                                                   const float* __restrict__ twb) {
  constexpr int K = N / 2 + 1;
  constexpr int64_t total = (int64_t)N * N * K;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / K;
    const int kz = (int)(i - row * K);
    const int64_t e = row * HP + kz;
    int x, y;
    row_xy(row, N, kXB, x, y);
    const int kx = sidx(x, N), ky = sidx(y, N);
    const float t = __ldg(twb + kx * kx + ky * ky + kz * kz);
    const float2 v = phi[e];
    out[e] = make_float2(v.x * t, v.y * t);
  }
}

// ----------------------------------------------------------- row passes
// (rows.cuh: RowCfg, the c2r / r2c row steps and rows_body)
template <int N, class Op>
__global__ void __launch_bounds__(kRowThreads, Op::min_blocks(N)) k_rows(Op op, float2* work, int64_t fs, int HP,
                                                       const float2* __restrict__ twN, const float2* __restrict__ twH) {
  rows_body<N>(op, work, fs, HP, twN, twH);
}

// One product term of the row combine, as a kernel parameter: the shared-
// memory offsets of lines p and q, and bit 31 set for the counter-term that
// is evaluated early into g_1 (see ModalRowOp).
struct TermC {
  uint32_t off;  // p LS | (q LS) << 16 | early << 31
  float c;
};

// modal products: lines 0..M-1 hold f_p; line r is overwritten by g_r.  The
// term list travels in the kernel's parameter space, so every thread reads
// a term through the uniform constant path; each thread forms two positions
// per term.
struct ModalRowOp {
  // resident rows per SM: shared memory holds two at 1024^3 with 20 modes;
  // below that registers decide (three rows: 80 registers, no spill)
  static constexpr int min_blocks(int n) { return n >= 1024 ? 2 : 3; }
  static constexpr bool kZfac = false;
  static constexpr bool kPairs = true;
  int M, nr;
  int r_of_slot[kMaxModes];
  int begin[kMaxModes + 1];
  TermC t[kMaxTerms];
  __device__ int nin() const { return M; }
  __device__ int in_slot(int l) const { return l; }
  __device__ int nout() const { return nr; }
  __device__ int out_line(int l) const { return r_of_slot[l]; }
  __device__ int out_slot(int l) const { return r_of_slot[l]; }
  // Slots in descending r: g_r only needs f_p f_q with p <= q <= r, so once
  // g_r is formed nothing later reads f_r and it is stored over it at once.
  // (The counter-term f_0 f_2 -> g_1 reads f_2 after g_2 has replaced it;
  // that term is evaluated first, in the pass for r = 2, into a register.)
  template <int K>
  __device__ void combine(float2* sm, const int* pos, int LS) const {
    float2 g1_extra[K];
#pragma unroll
    for (int i = 0; i < K; ++i) g1_extra[i] = make_float2(0.f, 0.f);
    for (int s = nr - 1; s >= 0; --s) {
      const int r = r_of_slot[s];
      float2 acc[K];
#pragma unroll
      for (int i = 0; i < K; ++i) acc[i] = make_float2(0.f, 0.f);
      const int tb = begin[s], te = begin[s + 1];
#pragma unroll 2
      for (int ti = tb; ti < te; ++ti) {
        const TermC tm = t[ti];
        const int po = (int)(tm.off & 0xFFFFu), qo = (int)((tm.off >> 16) & 0x7FFFu);
        const bool early = (tm.off >> 31) != 0u;
#pragma unroll
        for (int i = 0; i < K; ++i) {
          const float2 fp = sm[po + pos[i]], fq = sm[qo + pos[i]];
          const float vx = tm.c * fp.x * fq.x, vy = tm.c * fp.y * fq.y;
          if (early) {
            g1_extra[i].x += vx;
            g1_extra[i].y += vy;
          } else {
            acc[i].x += vx;
            acc[i].y += vy;
          }
        }
      }
#pragma unroll
      for (int i = 0; i < K; ++i) {
        if (r == 1) {
          acc[i].x += g1_extra[i].x;
          acc[i].y += g1_extra[i].y;
        }
        sm[r * LS + pos[i]] = acc[i];
      }
    }
  }
};

// 2LPT source (main.c:1284-1294): lines 0..5 hold d00 d01 d02 d11 d12 d22;
// the source goes to line 0, written to slot `out`.
struct SourceRowOp {
  // seven lines per row (at 512^3 four blocks spill a few bytes with 16
  // values per lane and still ran faster than three: 2.33 vs 2.63 ms)
  static constexpr int min_blocks(int) { return 4; }
  static constexpr bool kPairs = true;
  static constexpr bool kZfac = true;  // z factors of the Hessians (1, 1, kz, 1, kz, kz^2)
  int out;
  float kF;
  const float* isinc2;
  __device__ ZFac zfac(int l) const { return ZFac{l == 2 || l == 4 ? 1 : l == 5 ? 2 : 0, kF, isinc2}; }
  __device__ int nin() const { return 6; }
  __device__ int in_slot(int l) const { return l; }
  __device__ int nout() const { return 1; }
  __device__ int out_line(int) const { return 0; }
  __device__ int out_slot(int) const { return out; }
  template <int K>
  __device__ void combine(float2* sm, const int* pos, int LS) const {
#pragma unroll
    for (int i = 0; i < K; ++i) {
      float2 d[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) d[c] = sm[c * LS + pos[i]];
      float2 s;
      s.x = d[0].x * (d[3].x + d[5].x) + d[3].x * d[5].x - d[1].x * d[1].x - d[2].x * d[2].x - d[4].x * d[4].x;
      s.y = d[0].y * (d[3].y + d[5].y) + d[3].y * d[5].y - d[1].y * d[1].y - d[2].y * d[2].y - d[4].y * d[4].y;
      sm[pos[i]] = s;
    }
  }
};

// c2r of one field per blockIdx.y (slot = first + blockIdx.y), each with
// its z factor (ZFac type ztype[blockIdx.y]; 0 = plain c2r)
struct ZTypes {
  int t[6];
  float kF;
  const float* isinc2;
  // t[i] by selects (a dynamic index into the parameter block would copy it
  // to local memory)
  __device__ __forceinline__ int at(int i) const {
    int r = t[0];
#pragma unroll
    for (int j = 1; j < 6; ++j) r = i == j ? t[j] : r;
    return i < 6 ? r : 0;
  }
};
template <int N>
__global__ void __launch_bounds__(256) k_rows_c2r(float2* work, int64_t fs, int HP, int first, int64_t nrows,
                                                  const float2* __restrict__ twN, const float2* __restrict__ twH,
                                                  ZTypes zt) {
  using C = RowCfg<N>;
  constexpr int H = C::H;
  extern __shared__ float2 sm[];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int sub = lane / C::T, t = lane % C::T;
  int lines_per_block = (blockDim.x >> 5) * C::LPW;
  int64_t row = (int64_t)blockIdx.x * lines_per_block + warp * C::LPW + sub;
  bool act = row < nrows && sub < C::LPW;
  float2* line = sm + (warp * C::LPW + sub) * C::LS;
  float2* f = work + (int64_t)(first + blockIdx.y) * fs + (act ? row : 0) * HP;
  const ZFac zf{zt.at(blockIdx.y), zt.kF, zt.isinc2};
  if constexpr (RowFold<N>::value) {
    // folded radix-2 (rows.cuh): the halves hold z_{2m} and z_{2m+1}; lane
    // t writes the pair (z_{2m}, z_{2m+1}) as one 16-byte store
    constexpr int h = H / 2, HO = h + h / 16;
    if (act) row_c2r_pre_fold<N>(line, lane, twN, twH, zf, f);
    __syncwarp();
    line_fft_smem<h, 16, +1, 0, 0, 2>(line + (lane >> 4) * HO, lane & 15, twH, act);
    if (act)
      for (int m = lane; m < h; m += 32) {
        const float2 e = line[spad(m)], o = line[spad(m) + HO];
        reinterpret_cast<float4*>(f)[m] = make_float4(e.x, e.y, o.x, o.y);
      }
    return;
  }
  if (act) row_c2r_pre<N>(f, line, t, C::T, twN, zf);
  __syncwarp();
  line_fft_smem<H, C::T, +1>(line, t, twH, act);
  if (act)
    for (int n = t; n < H; n += C::T) f[n] = line[spad(n)];
}

// ----------------------------------------------------------- 2LPT passes

__device__ __forceinline__ float sincf(float x) { return x == 0.f ? 1.f : sinf(x) / x; }

#include "passes.cuh"

// ----------------------------------------------------------- read-out
// Trilinear read-out (main.c:1440-1516).  Fields: slots 0..5 of `work` as
// real rows (float, row stride 2 HP); psi2 slots hold N^3 x the 2LPT field.
struct ReadArgs {
  int N, HP;
  int64_t fs;           // field stride in floats
  float box, inv_n3, vp1, vp2;
  float nb_hi, nb_lo;  // N / Box as a two-float sum
};

// Cell index and fraction of one coordinate: u = Pos N / Box
// (main.c:1444-1446) to ~1e-7 of a cell in FP32 -- the product with a
// two-float split of N/Box -- then the cell index and the fraction with the
// reference's clamps (main.c:1452-1463).
__device__ __forceinline__ void cell_coord(const ReadArgs& a, float p, int& i, float& f) {
  const int N = a.N;
  float hi = p * a.nb_hi;
  float lo = fmaf(p, a.nb_hi, -hi) + p * a.nb_lo;
  if (!(hi >= 0.f)) {  // also catches NaN: the cell index stays inside the grid
    hi = 0.f;
    lo = 0.f;
  }
  if (hi > (float)N) {
    hi = (float)N;
    lo = 0.f;
  }
  const float fl = floorf(hi);
  i = (int)fl;
  f = (hi - fl) + lo;  // hi - fl is exact
  if (f < 0.f) {
    i -= 1;
    f += 1.f;
  } else if (f >= 1.f) {
    i += 1;
    f -= 1.f;
  }
  if (i < 0) {  // (int) truncates: u in (-1, 0) reads cell 0 with a negative fraction
    f = (float)i + f;
    i = 0;
  }
  if (i >= N) {
    f += (float)(i - (N - 1));
    i = N - 1;
  }
}

// Position and velocity of a particle at Lagrangian coordinate p from its
// ZA and 2LPT displacements d1, d2 (main.c:1486-1509): Pos += dis - 3/7
// dis2 / N^3 with the periodic wrap, Vel = dis vp1 - 3/7 dis2 / N^3 vp2.
__device__ __forceinline__ void move_particle(const ReadArgs& a, const float* p, const float* dis, const float* dis2,
                                              float* op, float* ov) {
  for (int ax = 0; ax < 3; ++ax) {
    const float d1 = dis[ax], d2 = dis2[ax] * a.inv_n3;
    float d = d1 - (3.f / 7.f) * d2;
    float x = p[ax] + d;
    if (x < 0.f) x += a.box;
    if (x >= a.box) x -= a.box;
    op[ax] = x;
    ov[ax] = d1 * a.vp1 - (3.f / 7.f) * d2 * a.vp2;
  }
}

__device__ __forceinline__ void readout_one(const ReadArgs& a, const float* __restrict__ F, float px, float py,
                                            float pz, float* op, float* ov) {
  const int N = a.N;
  float p[3] = {px, py, pz};
  int ii[3], jj[3];
  float fr[3];
  for (int d = 0; d < 3; ++d) {
    cell_coord(a, p[d], ii[d], fr[d]);
    jj[d] = (ii[d] + 1 == N) ? 0 : ii[d] + 1;
  }
  const int64_t rs = 2 * (int64_t)a.HP;
  float u = fr[0], v = fr[1], w = fr[2];
  float dis[3], dis2[3];
  if (u == 0.f && v == 0.f && w == 0.f) {
    // on a grid point (a regular lattice whose spacing Box/N is a binary
    // fraction): weights f1 = 1, f2..f8 = 0, so the 8-point sum is the one
    // corner value exactly (finite fields) and the other 7 loads are skipped
    const int64_t o = row_of(ii[0], ii[1], N, kXB) * rs + ii[2];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      dis[ax] = F[ax * a.fs + o];
      dis2[ax] = F[(3 + ax) * a.fs + o];
    }
  } else {
    int64_t o000 = row_of(ii[0], ii[1], N, kXB) * rs, o010 = row_of(ii[0], jj[1], N, kXB) * rs;
    int64_t o100 = row_of(jj[0], ii[1], N, kXB) * rs, o110 = row_of(jj[0], jj[1], N, kXB) * rs;
    float f1 = (1 - u) * (1 - v) * (1 - w), f2 = (1 - u) * (1 - v) * w, f3 = (1 - u) * v * (1 - w),
          f4 = (1 - u) * v * w, f5 = u * (1 - v) * (1 - w), f6 = u * (1 - v) * w, f7 = u * v * (1 - w),
          f8 = u * v * w;
    int k0 = ii[2], k1 = jj[2];
    for (int ax = 0; ax < 3; ++ax) {
      const float* d1 = F + ax * a.fs;
      const float* d2 = F + (3 + ax) * a.fs;
      dis[ax] = d1[o000 + k0] * f1 + d1[o000 + k1] * f2 + d1[o010 + k0] * f3 + d1[o010 + k1] * f4 +
                d1[o100 + k0] * f5 + d1[o100 + k1] * f6 + d1[o110 + k0] * f7 + d1[o110 + k1] * f8;
      dis2[ax] = d2[o000 + k0] * f1 + d2[o000 + k1] * f2 + d2[o010 + k0] * f3 + d2[o010 + k1] * f4 +
                 d2[o100 + k0] * f5 + d2[o100 + k1] * f6 + d2[o110 + k0] * f7 + d2[o110 + k1] * f8;
    }
  }
  move_particle(a, p, dis, dis2, op, ov);
}

// One particle per thread.  (Measured at 1024^3 on a lattice: four
// particles per thread with 16-byte loads and stores, 79 registers and three
// blocks per SM, 27.0 vs 19.6 ms.)
__global__ void __launch_bounds__(256, 6) k_readout(ReadArgs a, const float* __restrict__ F, const float* __restrict__ lagr, int64_t np,
                          float* pos, float* vel) {
  int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
  float op[3], ov[3];
  readout_one(a, F, lagr[3 * n], lagr[3 * n + 1], lagr[3 * n + 2], op, ov);
  for (int d = 0; d < 3; ++d) {
    pos[3 * n + d] = op[d];
    vel[3 * n + d] = ov[d];
  }
}

// Lagrangian positions from a glass tiled tile^3 times (read_glass.c:129-214):
// Pos = glass / glass_box * (Box / tile) + t * (Box / tile) in FP64 with
// unfused operations, rounded to float.  The two products depend only on
// the glass particle and on the tile index, so k_glass_scale makes them once
// per call (3 nglass + tile doubles) and a particle costs one FP64 add per
// axis (GB300's FP64 rate is a small fraction of its FP32 rate).
__global__ void k_glass_scale(const float* __restrict__ glass, int64_t nglass, double glass_box, int tile,
                              double box_over_tile, double* __restrict__ gs) {
  const int64_t n = 3 * nglass + tile;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    gs[i] = i < 3 * nglass ? __dmul_rn(__ddiv_rn((double)glass[i], glass_box), box_over_tile)
                           : __dmul_rn((double)(i - 3 * nglass), box_over_tile);
}

// Particles n0 <= n < n1 (indices of the whole tiled set, particle order of
// read_glass.c:181-214: tile index outer, glass index inner).  A block's
// positions and velocities go through shared memory and out as 16-byte
// stores of whole lines: the outputs may be page-locked host memory written
// over the host link (4-byte stores 12 bytes apart: 37 GB/s at 1536^3; whole
// lines 41-47 GB/s, the rate the copy engines reach on the same link).
constexpr int kReadoutThreads = 256;
__global__ void __launch_bounds__(kReadoutThreads) k_readout_glass(ReadArgs a, const float* __restrict__ F,
                                                                   const double* __restrict__ gs, int64_t nglass,
                                                                   int tile, float* pos, float* vel, int* ids,
                                                                   int64_t n0, int64_t n1) {
  __shared__ float4 sp4[3 * kReadoutThreads / 4], sv4[3 * kReadoutThreads / 4];
  float* sp = (float*)sp4;
  float* sv = (float*)sv4;
  const int64_t base = n0 + (int64_t)blockIdx.x * kReadoutThreads;
  const int64_t n = base + threadIdx.x;
  if (n < n1) {
    int64_t gi = n % nglass, t = n / nglass;
    int ti = (int)(t / ((int64_t)tile * tile)), tj = (int)((t / tile) % tile), tk = (int)(t % tile);
    int tt[3] = {ti, tj, tk};
    const double* toff = gs + 3 * nglass;
    float lp[3];
    for (int d = 0; d < 3; ++d) lp[d] = (float)__dadd_rn(gs[3 * gi + d], toff[tt[d]]);
    float op[3], ov[3];
    readout_one(a, F, lp[0], lp[1], lp[2], op, ov);
    for (int d = 0; d < 3; ++d) {
      sp[3 * threadIdx.x + d] = op[d];
      sv[3 * threadIdx.x + d] = ov[d];
    }
    if (ids) ids[n] = (int)(n + 1);
  }
  __syncthreads();
  const int cnt = (int)min((int64_t)kReadoutThreads, n1 - base);
  float* po = pos + 3 * base;
  float* vo = vel + 3 * base;
  if (cnt == kReadoutThreads && ((reinterpret_cast<uintptr_t>(po) | reinterpret_cast<uintptr_t>(vo)) & 15) == 0) {
    for (int i = threadIdx.x; i < 3 * kReadoutThreads / 4; i += kReadoutThreads) {
      reinterpret_cast<float4*>(po)[i] = sp4[i];
      reinterpret_cast<float4*>(vo)[i] = sv4[i];
    }
  } else {
    for (int i = threadIdx.x; i < 3 * cnt; i += kReadoutThreads) {
      po[i] = sp[i];
      vo[i] = sv[i];
    }
  }
}

// ----------------------------------------------------------- lattice read-out
// Particles of the regular g^3 lattice glass (per-axis glass coordinate
// (float)(i * glass_box / g), the particle order of read_glass.c:181-214)
// tiled tile^3 times.  k_lattice_axis makes the Lagrangian coordinate of
// every lattice index of one axis with the operations of the general glass
// path (k_glass_scale + k_readout_glass) and flags any that is not exactly
// on its own grid point by the reference's own FP64 cell coordinate u = Pos
// / Box * Nmesh (main.c:1444-1446): u must equal the index.  When none is
// flagged and g tile = Nmesh, every particle sits on a grid point and reads
// just the grid value under it (the weights of the other seven corners are
// zero), so the read-out can be fused into the displacement rows:
// k_rows_lattice.  (The FP32 read-out's two-float coordinate can leave a
// fraction of ~1e-12 at such a point, which weights the neighbour by as
// much; the fused read-out takes the grid value, as the FP64 reference
// does.)
__global__ void k_lattice_axis(int N, double box, int g, double gsp, double glass_box, double bot, float* lpa,
                               int* off_grid) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int gi = i % g, ti = i / g;
  const float gc = (float)__dmul_rn((double)gi, gsp);
  const float lp = (float)__dadd_rn(__dmul_rn(__ddiv_rn((double)gc, glass_box), bot), __dmul_rn((double)ti, bot));
  lpa[i] = lp;
  const double u = __dmul_rn(__ddiv_rn((double)lp, box), (double)N);
  if (u != (double)i) atomicOr(off_grid, 1);
}

// The lattice glass itself (3 g^3 floats), for the general read-out.
__global__ void k_lattice_glass(int g, double gsp, float* glass) {
  const int64_t n = (int64_t)g * g * g;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ix = i / ((int64_t)g * g), iy = (i / g) % g, iz = i % g;
    glass[3 * i] = (float)__dmul_rn((double)ix, gsp);
    glass[3 * i + 1] = (float)__dmul_rn((double)iy, gsp);
    glass[3 * i + 2] = (float)__dmul_rn((double)iz, gsp);
  }
}

// The six displacement rows of RPB memory rows (c2r with the z factors, as
// k_rows_c2r; warp c takes field c), then the particles on the rows' grid
// points: Pos / Vel from the grid values (readout_one's on-grid branch,
// main.c:1486-1509) and IDs, written at their tiled-glass particle index.
// Rows [row0, row0 + nrows) of the x-blocked order.
template <int N>
struct LatticeCfg {
  static constexpr int RPB = RowFold<N>::value ? 1 : RowCfg<N>::LPW;  // rows per block
  static constexpr size_t SMEM = sizeof(float2) * (size_t)RPB * 6 * RowCfg<N>::LS;
};
template <int N>
__global__ void __launch_bounds__(192, 4) k_rows_lattice(const float2* __restrict__ work, int64_t fs, int HP,
                                                         const float2* __restrict__ twN, const float2* __restrict__ twH,
                                                         ZTypes zt, ReadArgs ra, int g, int tile,
                                                         const float* __restrict__ lpa, float* pos, float* vel,
                                                         int* ids, int64_t row0, int64_t nrows) {
  using C = RowCfg<N>;
  constexpr int H = C::H, RPB = LatticeCfg<N>::RPB;
  extern __shared__ float2 sm[];  // [RPB][6][LS]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t rbase = row0 + (int64_t)blockIdx.x * RPB, rend = row0 + nrows;
  const ZFac zf{zt.at(warp), zt.kF, zt.isinc2};
  if constexpr (RowFold<N>::value) {
    constexpr int h = H / 2, HO = h + h / 16;
    const bool act = rbase < rend;
    // (the lane twiddle table of rows_body cost more than it saved here:
    // one row per block, 13.1 -> 14.5 ms)
    float2* line = sm + warp * C::LS;
    if (act) row_c2r_pre_fold<N>(line, lane, twN, twH, zf, work + (int64_t)warp * fs + rbase * HP);
    __syncwarp();
    line_fft_smem<h, 16, +1, 0, 0, 2>(line + (lane >> 4) * HO, lane & 15, twH, act);
  } else {
    const int sub = lane / C::T, t = lane % C::T;
    const int64_t row = rbase + sub;
    const bool act = sub < RPB && row < rend;
    float2* line = sm + ((act ? sub : 0) * 6 + warp) * C::LS;
    if (act) row_c2r_pre<N>(work + (int64_t)warp * fs + row * HP, line, t, C::T, twN, zf);
    __syncwarp();
    line_fft_smem<H, C::T, +1>(line, t, twH, act);
  }
  __syncthreads();
  const int64_t g3 = (int64_t)g * g * g;
  for (int q = threadIdx.x; q < RPB * N; q += blockDim.x) {
    const int sub = q / N, z = q - sub * N;
    const int64_t row = rbase + sub;
    if (row >= rend) break;
    int x, y;
    row_xy(row, N, kXB, x, y);
    float d[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      float2 v;
      if constexpr (RowFold<N>::value) {
        // the folded transform leaves z_{2m} at m and z_{2m+1} at h + m
        // (z_j = (x_{2j}, x_{2j+1})): x_z sits in the pair of z / 4
        constexpr int h = H / 2, HO = h + h / 16;
        v = sm[c * C::LS + spad(z >> 2) + (((z >> 1) & 1) ? HO : 0)];
      } else {
        v = sm[(sub * 6 + c) * C::LS + spad(z >> 1)];
      }
      d[c] = (z & 1) ? v.y : v.x;
    }
    const float p[3] = {lpa[x], lpa[y], lpa[z]};
    float op[3], ov[3];
    move_particle(ra, p, d, d + 3, op, ov);
    const int ti = x / g, gi = x - ti * g, tj = y / g, gj = y - tj * g, tk = z / g, gk = z - tk * g;
    const int64_t n = (((int64_t)ti * tile + tj) * tile + tk) * g3 + ((int64_t)gi * g + gj) * g + gk;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      pos[3 * n + c] = op[c];
      vel[3 * n + c] = ov[c];
    }
    if (ids) ids[n] = (int)(n + 1);
  }
}

// ----------------------------------------------------------- host side
// Launch a persistent pass: as many blocks as fit on the device at once.
template <int N, class Op>
static int run_pass(Plan* p, const Op& op, int64_t nitems, cudaStream_t st, const char* name) {
  constexpr int W = 8;
  using A = AxisCfg<N, W>;
  auto kern = k_pass<N, W, Op>;
  const size_t smem = A::SMEM + ExtraSmem<Op>::value;
  AAR_CUDA_TRY(p, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (nitems < 1) return AAR_OK;
  if (nitems > 0x7fffffff) return set_err(p, std::string(name) + ": too many work items"), AAR_ERR_ARG;
  {
    ProfScope ps_(p, name, st);
    kern<<<(unsigned)nitems, A::THREADS, smem, st>>>(op, p->d_twN);
  }
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

RhoArgs rho_args(const Plan* p) {
  RhoArgs r{};
  const double ns = p->prm.primordial_index, box = p->prm.box;
  const double kF = 2 * kPi / box, kmin = kF, kmax = kF * p->prm.nmax;
  const double sx = (4 - ns) / 3, kmin_s = pow(kmin, sx), kmax_s = pow(kmax, sx);
  r.s = (float)sx;
  r.c1 = (float)(2 * kmin_s / (kmax_s - kmin_s));
  r.log2kF = (float)log2(kF);
  r.inv_kF2 = (float)(1 / (kF * kF));
  r.e4 = (float)(4 - ns);
  r.e2 = (float)(2 - ns);
  for (int n = 0; n < kMaxModes; ++n) r.x0[n] = n < (int)p->x0.size() ? (float)p->x0[n] : 0.f;
  for (int l = 1; l < kMaxModes; ++l) {
    r.A[l] = (float)((2.0 * l - 1) / l);
    r.B[l] = (float)((l - 1.0) / l);
  }
  return r;
}

template <int N>
struct Launch {
  static constexpr int W = 8;
  static int64_t tiles(Plan* p) { return (int64_t)N * (p->HP / W); }
  static int64_t fstride(Plan* p) { return (int64_t)N * N * p->HP; }
  static const int* slot_map(Plan* p) {
    return (const int*)((const char*)p->d_terms + offsetof(DevTerms, tl) + offsetof(TermList, r_of_slot));
  }
  static constexpr size_t row_smem(int nlines) {
    return sizeof(float2) * ((size_t)nlines * RowCfg<N>::LS + row_lt_slots<N>());
  }
  static int configure(Plan* p) {
    size_t sm_rows = row_smem(kMaxModes + 1);
    AAR_CUDA_TRY(p, cudaFuncSetAttribute(k_rows<N, ModalRowOp>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_rows));
    AAR_CUDA_TRY(p, cudaFuncSetAttribute(k_rows<N, SourceRowOp>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_rows));
    return AAR_OK;
  }
  // y transform of fields [first, first + nf) (or the active modal slots)
  template <int SIGN>
  static int ypass(Plan* p, float2* base, int nf, const int* map, cudaStream_t st, const char* name) {
    AxisOp<N, W, 1, SIGN> op{base, fstride(p), tiles(p), p->HP, map};
    return run_pass<N>(p, op, nf * tiles(p), st, name);
  }
  static int modal(Plan* p, const ModalArgs& a, cudaStream_t st) {
    int64_t fs = fstride(p);
    XinvOp<N, W> xo{a, p->d_phik, p->d_work, fs, tiles(p), p->HP, rho_args(p), p->xpass_group,
                    p->qcube_stale ? nullptr : p->d_qcube};
    int rc = run_pass<N>(p, xo, tiles(p) * a.M, st, "modal_xinv");
    if (rc) return rc;
    if ((rc = ypass<+1>(p, p->d_work, a.M, nullptr, st, "modal_ypass_inv"))) return rc;
    size_t sm_rows = row_smem(a.M + 1);
    if (p->jit) {
      if ((rc = jit_modal_rows(p, p->d_work, fs, st))) return rc;
      if ((rc = ypass<-1>(p, p->d_work, p->nr_active, slot_map(p), st, "modal_ypass_fwd"))) return rc;
      return modal_tail(p, a, fs, st);
    }
    static_assert(sizeof(ModalRowOp) < 32000, "kernel parameter space");
    ModalRowOp op;
    {
      const TermList& tl = *(const TermList*)p->host_terms.data();
      const Term* ft = (const Term*)(p->host_terms.data() + sizeof(TermList));
      constexpr int LS = RowCfg<N>::LS;
      static_assert(kMaxModes * LS < 0x8000, "line offsets fit 15 bits");
      op.M = a.M;
      op.nr = tl.nr;
      for (int i = 0; i < kMaxModes; ++i) op.r_of_slot[i] = tl.r_of_slot[i];
      for (int i = 0; i <= kMaxModes; ++i) op.begin[i] = tl.begin[i];
      for (int sl = 0; sl < tl.nr; ++sl)
        for (int i = tl.begin[sl]; i < tl.begin[sl + 1]; ++i) {
          const uint32_t early = ft[i].r != tl.r_of_slot[sl] ? 1u : 0u;
          op.t[i].off = (uint32_t)(ft[i].p * LS) | ((uint32_t)(ft[i].q * LS) << 16) | (early << 31);
          op.t[i].c = ft[i].c;
        }
    }
    {
      ProfScope ps_(p, "modal_rows", st);
      k_rows<N, ModalRowOp><<<(unsigned)((int64_t)N * N), kRowThreads, sm_rows, st>>>(op, p->d_work, fs, p->HP, p->d_twN,
                                                                               p->d_twH);
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    if ((rc = ypass<-1>(p, p->d_work, p->nr_active, slot_map(p), st, "modal_ypass_fwd"))) return rc;
    return modal_tail(p, a, fs, st);
  }
  // forward x of the active slots, then the accumulation into phi
  static int modal_tail(Plan* p, const ModalArgs& a, int64_t fs, cudaStream_t st) {
    int rc;
    {
      AxisOp<N, W, 0, -1> xf{p->d_work, fs, tiles(p), p->HP, slot_map(p)};
      if ((rc = run_pass<N>(p, xf, p->nr_active * tiles(p), st, "modal_xfwd"))) return rc;
    }
    float fnl_n3 = (float)(p->prm.fnl / ((double)N * N * N));
    if (jit_has_acc(p)) return jit_modal_acc(p, p->d_phik, p->d_work, fnl_n3, rho_args(p), st);
    {
      ProfScope ps_(p, "modal_acc", st);
      k_modal_acc<N><<<(unsigned)(p->num_sms * 8), 256, 0, st>>>(a, p->d_phik, p->d_work, fs, p->HP, fnl_n3,
                                                             (const DevTerms*)p->d_terms, rho_args(p));
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    return AAR_OK;
  }
  // 2LPT (main.c:1180-1431).  Work slots: 7 = T/(D Beta) phi; Hessians
  // d_ab in 0..5 (00 01 02 11 12 22) via x outputs P = -kF^2 kx^2 phi_T -> 0,
  // Q = -kF^2 kx phi_T -> 8, R = -kF^2 phi_T -> 6 and the y fan-out (xy, yz:
  // ky; yy: ky^2); the source rows apply the z factors (xz, yz: kz; zz:
  // kz^2) and write S to 6; psi1 (0..2) and psi2 (3..5) likewise from x
  // outputs in 0, 8 (psi1) and 3, 7 (psi2).
  static int lpt(Plan* p, const LptArgs& a, cudaStream_t st, bool rows = true) {
    int64_t fs = fstride(p);
    float2* phit = p->d_work + 7 * fs;  // T/(D Beta) phi, read by the Hessian and psi1 passes
    {
      ProfScope ps_(p, "lpt_scale_twb", st);
      k_scale_twb<N><<<(unsigned)(p->num_sms * 8), 256, 0, st>>>(p->d_phik, phit, p->HP, p->d_twb);
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    int rc;
    {
      LptXOp<N, W, 0> ho{a, phit, p->d_work, fs, tiles(p), p->HP, {0, 8, 6}, p->xpass_group};
      if ((rc = run_pass<N>(p, ho, tiles(p) * 3, st, "lpt_xinv_hess"))) return rc;
      YFanOp<N, W> yf{a, p->d_work, fs, tiles(p), p->HP, {0, 8, 8, 6, 6, 6}, {0, 1, 2, 3, 4, 5}, {0, 1, 0, 2, 1, 0}, 1};
      if ((rc = run_pass<N>(p, yf, tiles(p) * 6, st, "lpt_ypass_inv_hess"))) return rc;
    }
    size_t sm_rows = row_smem(7);
    SourceRowOp op{6, a.m.g.kF, a.isinc2};
    {
      ProfScope ps_(p, "lpt_rows_source", st);
      k_rows<N, SourceRowOp><<<(unsigned)((int64_t)N * N), kRowThreads, sm_rows, st>>>(op, p->d_work, fs, p->HP, p->d_twN,
                                                                                p->d_twH);
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    if ((rc = ypass<-1>(p, p->d_work + 6 * fs, 1, nullptr, st, "lpt_ypass_fwd_source"))) return rc;
    // forward x of the source in place with -1/k^2, then the displacement x passes
    {
      XfwdInvK2Op<N, W> xs{p->d_work + 6 * fs, tiles(p), p->HP, a.m.g.kF};
      if ((rc = run_pass<N>(p, xs, tiles(p), st, "lpt_xfwd_source"))) return rc;
    }
    {
      LptXOp<N, W, 1> m1{a, phit, p->d_work, fs, tiles(p), p->HP, {0, 8, 0}, p->xpass_group};
      if ((rc = run_pass<N>(p, m1, tiles(p) * 2, st, "lpt_xpsi1"))) return rc;
      LptXOp<N, W, 1> m2{a, p->d_work + 6 * fs, p->d_work, fs, tiles(p), p->HP, {3, 7, 0}, p->xpass_group};
      if ((rc = run_pass<N>(p, m2, tiles(p) * 2, st, "lpt_xpsi2"))) return rc;
      YFanOp<N, W> yf{a, p->d_work, fs, tiles(p), p->HP, {0, 8, 8, 3, 7, 7}, {0, 1, 2, 3, 4, 5}, {3, 4, 3, 3, 4, 3}, 1};
      if ((rc = run_pass<N>(p, yf, tiles(p) * 6, st, "lpt_ypass_inv_disp"))) return rc;
    }
    // the displacement rows: here, or fused with the lattice read-out
    // (fused_rows_lattice), which leaves no real fields behind
    p->disp_real = rows;
    if (!rows) return AAR_OK;
    using R = RowCfg<N>;
    int lines_per_block = 8 * R::LPW;
    int64_t nrows = (int64_t)N * N;
    dim3 grid((unsigned)((nrows + lines_per_block - 1) / lines_per_block), 6);
    const ZTypes zt{{3, 3, 4, 3, 3, 4}, a.m.g.kF, a.isinc2};
    {
      ProfScope ps_(p, "lpt_rows_c2r", st);
      k_rows_c2r<N><<<grid, 256, sizeof(float2) * lines_per_block * R::LS, st>>>(p->d_work, fs, p->HP, 0, nrows,
                                                                                p->d_twN, p->d_twH, zt);
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    return AAR_OK;
  }
};

template <class F>
static int dispatch_n(int N, F&& f) {
  switch (N) {
    case 16: return f(std::integral_constant<int, 16>{});
    case 32: return f(std::integral_constant<int, 32>{});
    case 64: return f(std::integral_constant<int, 64>{});
    case 128: return f(std::integral_constant<int, 128>{});
    case 256: return f(std::integral_constant<int, 256>{});
    case 512: return f(std::integral_constant<int, 512>{});
    case 1024: return f(std::integral_constant<int, 1024>{});
    default: return AAR_ERR_ARG;
  }
}

ModalArgs modal_args(Plan* p) {
  ModalArgs a;
  a.g = p->grid;
  a.M = p->M;
  return a;
}

// The regrouped term list by output slot: sorted triples p <= q <= r with
// alpha != 0 contribute a f_p f_q to g_r (main.c:833-867); the
// counter-terms of main.c:1045-1050 add -a012 t012 f_0 f_1 to g_2 and
// +a012 t012 f_0 f_2 to g_1.  The second one sits in the list of r = 2 (its
// target r stays 1): the row kernels form the slots in descending r and g_2
// replaces f_2 in place, so f_0 f_2 is taken before that.
std::vector<std::vector<Term>> regrouped_terms(const std::vector<double>& alpha, int M) {
  auto A = [&](int i, int j, int k) { return alpha[((size_t)i * M + j) * M + k]; };
  std::vector<std::vector<Term>> by_r(M);
  for (int i = 0; i < M; ++i)
    for (int j = i; j < M; ++j)
      for (int k = j; k < M; ++k)
        if (A(i, j, k) != 0) by_r[k].push_back(Term{i, j, k, (float)A(i, j, k)});
  if (M > 2 && A(0, 1, 2) != 0) {
    double t012 = -A(1, 1, 1) / A(0, 1, 2);
    double c = A(0, 1, 2) * t012;
    by_r[2].push_back(Term{0, 1, 2, (float)(-c)});
    by_r[2].push_back(Term{0, 2, 1, (float)(c)});
    if (by_r[1].empty()) by_r[1].push_back(Term{0, 0, 1, 0.f});  // keep a slot for r = 1
  }
  return by_r;
}

// Split of the active r over nparts cooperating plans, balanced by the
// number of product terms each g_r takes: the r in decreasing term count
// (ties: lower r first) each go to the part with the fewest terms so far
// (ties: lower part).  part_of_r[r] = -1 for an r without terms.
std::vector<int> modal_partition(const std::vector<std::vector<Term>>& by_r, int nparts) {
  const int M = (int)by_r.size();
  std::vector<int> cnt(M, 0), part(M, -1);
  for (const auto& lst : by_r)
    for (const Term& t : lst) cnt[t.r] += 1;
  std::vector<int> order;
  for (int r = 0; r < M; ++r)
    if (!by_r[r].empty() || cnt[r] > 0) order.push_back(r);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cnt[a] > cnt[b]; });
  std::vector<long> load(std::max(nparts, 1), 0);
  for (int r : order) {
    int best = 0;
    for (int q = 1; q < nparts; ++q)
      if (load[q] < load[best]) best = q;
    part[r] = best;
    load[best] += cnt[r];
  }
  return part;
}

// The plan's term list (device and host copies): the regrouped terms, or
// with a modal partition only the slots of the plan's part.  A split keeps
// the counter-term f_0 f_2 -> g_1 with the part of r = 1: as a term read
// before g_2 replaces f_2 when r = 2 is in the same part, else as an
// ordinary term of r = 1 (f_2 is never replaced in that part).
static int build_terms(Plan* p) {
  int M = p->M;
  std::vector<std::vector<Term>> by_r = regrouped_terms(p->alpha, M);
  if (p->modal_nparts > 1) {
    const std::vector<int> part = modal_partition(by_r, p->modal_nparts);
    const int me = p->modal_part;
    std::vector<std::vector<Term>> mine(M);
    for (int r = 0; r < M; ++r)
      for (const Term& t : by_r[r]) {
        if (part[t.r] != me) continue;
        if (t.r != r && part[r] != me) mine[t.r].push_back(t);  // counter-term moves to its own slot
        else mine[r].push_back(t);
      }
    by_r.swap(mine);
  }
  TermList tl{};
  std::vector<Term> flat;
  int nr = 0;
  for (int r = 0; r < M; ++r) {
    if (by_r[r].empty()) continue;
    tl.r_of_slot[nr] = r;
    tl.begin[nr] = (int)flat.size();
    for (auto& t : by_r[r]) flat.push_back(t);
    ++nr;
  }
  tl.begin[nr] = (int)flat.size();
  tl.nr = nr;
  tl.nterms = (int)flat.size();
  if (tl.nterms > kMaxTerms) return set_err(p, "too many alpha terms"), AAR_ERR_ARG;
  DevTerms* dt = (DevTerms*)p->d_terms;
  AAR_CUDA_TRY(p, cudaMemcpy(&dt->tl, &tl, sizeof(tl), cudaMemcpyHostToDevice));
  if (!flat.empty()) AAR_CUDA_TRY(p, cudaMemcpy(dt->t, flat.data(), sizeof(Term) * flat.size(), cudaMemcpyHostToDevice));
  p->host_terms.assign((const char*)&tl, (const char*)&tl + sizeof(tl));
  p->host_terms.insert(p->host_terms.end(), (const char*)flat.data(), (const char*)(flat.data() + flat.size()));
  p->nterms = tl.nterms;
  p->nr_active = nr;
  return AAR_OK;
}

// The filter cube of the first modal pass: q_p(|kx|, |ky|, kz) for
// 0 <= |kx|, |ky|, kz <= N/2 with q_mode_cells' arithmetic, zero on the cut
// and at k = 0 (keep_cell depends on |k_a| only).  Index ((p K + |ky|) K +
// kz) K + |kx|, K = N/2 + 1.
__global__ void __launch_bounds__(256) k_qcube(Grid g, RhoArgs ra, int M, float* __restrict__ q) {
  const int K = g.N / 2 + 1;
  const int64_t per = (int64_t)K * K * K;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < per; i += (int64_t)gridDim.x * blockDim.x) {
    const int ax = (int)(i % K);
    const int64_t r = i / K;
    const int kz = (int)(r % K), ay = (int)(r / K);
    int n2[1] = {ax * ax + ay * ay + kz * kz};
    const bool on = n2[0] != 0 && keep_cell(g, ax, ay, kz);
    if (!on) n2[0] = 1;
    for (int p = 0; p < M; ++p) {
      float v[1];
      q_mode_cells<1>(ra, p, n2, v);
      q[(int64_t)p * per + i] = on ? v[0] : 0.f;
    }
  }
}

int qcube_build(Plan* p) {
  if (!p->qcube_stale && p->d_qcube) return AAR_OK;
  const int64_t K = p->N / 2 + 1, per = K * K * K;
  if (!p->d_qcube || p->qcube_m != p->M) {
    if (p->d_qcube) cudaFree(p->d_qcube), p->used_bytes -= sizeof(float) * (size_t)per * p->qcube_m;
    p->d_qcube = nullptr;
    p->qcube_m = 0;
    int rc = plan_alloc(p, (void**)&p->d_qcube, sizeof(float) * (size_t)per * p->M);
    if (rc) return rc;
    p->qcube_m = p->M;
  }
  k_qcube<<<(unsigned)(p->num_sms * 8), 256>>>(p->grid, rho_args(p), p->M, p->d_qcube);
  AAR_CUDA_TRY(p, cudaGetLastError());
  // made on the legacy stream once per table set; runs on the caller's
  // streams read it afterwards
  AAR_CUDA_TRY(p, cudaDeviceSynchronize());
  p->qcube_stale = false;
  return AAR_OK;
}

int build_term_list(Plan* p) {
  if (p->M > kMaxModes) return set_err(p, "N_modes above 32 is not supported"), AAR_ERR_ARG;
  return build_terms(p);
}

int fused_prepare(Plan* p) {
  if (p->M > kMaxModes) return set_err(p, "N_modes above 32 is not supported"), AAR_ERR_ARG;
  int rc = build_terms(p);
  if (rc) return rc;
  if ((rc = dispatch_n(p->N, [&](auto nc) {
         p->row_ls = RowCfg<decltype(nc)::value>::LS;
         p->row_lt = row_lt_slots<decltype(nc)::value>();
         return Launch<decltype(nc)::value>::configure(p);
       })))
    return rc;
  return jit_prepare(p);
}

static_assert(kRowThreads == kRowThreadsHost, "row kernel block size");

// The plan's modal row kernel (NVRTC or generic) on nrows rows of caller
// fields laid out with field stride nrows * HP: a harness that profiles the
// row kernel on a few thousand rows without full-size fields.
int profile_modal_rows(Plan* p, float2* work, int64_t nrows, cudaStream_t st) {
  if (nrows < 1 || nrows > (int64_t)p->N * p->N) return set_err(p, "profile rows: 1 <= nrows <= N^2"), AAR_ERR_ARG;
  if (p->nr_active == 0) return set_err(p, "profile rows: no modal terms"), AAR_ERR_STATE;
  const int64_t fs = nrows * p->HP;
  if (p->jit) return jit_modal_rows(p, work, fs, st, nrows);
  return dispatch_n(p->N, [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    ModalRowOp op;
    const TermList& tl = *(const TermList*)p->host_terms.data();
    const Term* ft = (const Term*)(p->host_terms.data() + sizeof(TermList));
    constexpr int LS = RowCfg<N>::LS;
    op.M = p->M;
    op.nr = tl.nr;
    for (int i = 0; i < kMaxModes; ++i) op.r_of_slot[i] = tl.r_of_slot[i];
    for (int i = 0; i <= kMaxModes; ++i) op.begin[i] = tl.begin[i];
    for (int sl = 0; sl < tl.nr; ++sl)
      for (int i = tl.begin[sl]; i < tl.begin[sl + 1]; ++i) {
        const uint32_t early = ft[i].r != tl.r_of_slot[sl] ? 1u : 0u;
        op.t[i].off = (uint32_t)(ft[i].p * LS) | ((uint32_t)(ft[i].q * LS) << 16) | (early << 31);
        op.t[i].c = ft[i].c;
      }
    const size_t sm_rows = Launch<N>::row_smem(p->M + 1);
    {
      ProfScope ps_(p, "modal_rows", st);
      k_rows<N, ModalRowOp><<<(unsigned)nrows, kRowThreads, sm_rows, st>>>(op, work, fs, p->HP, p->d_twN, p->d_twH);
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    return AAR_OK;
  });
}

int fused_modal(Plan* p, cudaStream_t st) {
  ModalArgs a = modal_args(p);
  if (p->nr_active == 0 || p->prm.fnl == 0) return AAR_OK;  // no non-Gaussian term at all
  return dispatch_n(p->N, [&](auto nc) { return Launch<decltype(nc)::value>::modal(p, a, st); });
}

LptArgs lpt_args(Plan* p) {
  LptArgs a;
  a.m = modal_args(p);
  a.inv_Dbeta = (float)(1.0 / (p->Dplus * p->Beta));
  a.twb = p->d_twb;
  a.sinc = p->d_sinc;
  a.isinc2 = p->d_isinc2;
  a.box_over_2n = (float)(p->prm.box / 2 / p->N);
  return a;
}

int fused_lpt(Plan* p, cudaStream_t st, bool rows) {
  LptArgs a = lpt_args(p);
  return dispatch_n(p->N, [&](auto nc) { return Launch<decltype(nc)::value>::lpt(p, a, st, rows); });
}

static ReadArgs read_args(Plan* p) {
  ReadArgs a;
  a.N = p->N;
  a.HP = p->HP;
  a.fs = 2 * (int64_t)p->N * p->N * p->HP;
  a.box = (float)p->prm.box;
  unsigned int n3 = (unsigned int)p->N * (unsigned int)p->N * (unsigned int)p->N;
  a.inv_n3 = (float)(1.0 / (double)(float)n3);
  a.vp1 = (float)p->vel_prefac;
  a.vp2 = (float)p->vel_prefac2;
  const double nb = (double)p->N / p->prm.box;
  a.nb_hi = (float)nb;
  a.nb_lo = (float)(nb - (double)a.nb_hi);
  return a;
}

int fused_readout(Plan* p, const float* d_lagr, int64_t npart, float* d_pos, float* d_vel, cudaStream_t st) {
  if (npart == 0) return AAR_OK;
  int bs = 256;
  { ProfScope ps_(p, "readout", st);
  k_readout<<<(unsigned)((npart + bs - 1) / bs), bs, 0, st>>>(read_args(p), (const float*)p->d_work, d_lagr, npart,
                                                               d_pos, d_vel);
  }
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

// Lattice read-out set-up for (g, glass_box, tile): the per-axis Lagrangian
// coordinates and whether the rows can read out (see k_lattice_axis); made
// once per parameter set (one synchronisation), then cached.
int lattice_prepare(Plan* p, int g, double glass_box, int tile, cudaStream_t st, bool& fused) {
  fused = false;
  if ((int64_t)g * tile != p->N) return AAR_OK;
  if (p->lat_g == g && p->lat_box == glass_box && p->lat_tile == tile) {
    fused = p->lat_fused;
    return AAR_OK;
  }
  int rc;
  if (!p->d_lpa && (rc = plan_alloc(p, (void**)&p->d_lpa, sizeof(float) * (p->N + 1)))) return rc;
  int* d_flag = (int*)(p->d_lpa + p->N);
  AAR_CUDA_TRY(p, cudaMemsetAsync(d_flag, 0, sizeof(int), st));
  k_lattice_axis<<<(p->N + 255) / 256, 256, 0, st>>>(p->N, p->prm.box, g, glass_box / g, glass_box, p->prm.box / tile,
                                                      p->d_lpa, d_flag);
  AAR_CUDA_TRY(p, cudaGetLastError());
  int flag = 1;
  AAR_CUDA_TRY(p, cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
  p->lat_g = g;
  p->lat_box = glass_box;
  p->lat_tile = tile;
  p->lat_fused = flag == 0;
  fused = p->lat_fused;
  return AAR_OK;
}

int lattice_glass(Plan* p, int g, double glass_box, float* d_glass, cudaStream_t st) {
  const int64_t n = (int64_t)g * g * g;
  k_lattice_glass<<<(unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)p->num_sms * 8), 256, 0, st>>>(
      g, glass_box / g, d_glass);
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

// The displacement rows with the lattice read-out fused (rows [row0, row0 +
// nrows) of the x-blocked order; lattice_prepare said fused).
int fused_rows_lattice(Plan* p, int g, int tile, float* d_pos, float* d_vel, int* d_ids, int64_t row0, int64_t nrows,
                       cudaStream_t st) {
  if (nrows <= 0) return AAR_OK;
  const LptArgs la = lpt_args(p);
  const ZTypes zt{{3, 3, 4, 3, 3, 4}, la.m.g.kF, la.isinc2};
  return dispatch_n(p->N, [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    using L = LatticeCfg<N>;
    AAR_CUDA_TRY(p, cudaFuncSetAttribute(k_rows_lattice<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::SMEM));
    {
      ProfScope ps_(p, "lpt_rows_readout", st);
      k_rows_lattice<N><<<(unsigned)((nrows + L::RPB - 1) / L::RPB), 192, L::SMEM, st>>>(
          p->d_work, (int64_t)N * N * p->HP, p->HP, p->d_twN, p->d_twH, zt, read_args(p), g, tile, p->d_lpa, d_pos,
          d_vel, d_ids, row0, nrows);
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    return AAR_OK;
  });
}

int glass_prepare(Plan* p, const float* d_glass, int64_t nglass, double glass_box, int tile, cudaStream_t st) {
  const int64_t need = 3 * nglass + tile;
  if (need > p->gscale_cap) {
    AAR_CUDA_TRY(p, cudaDeviceSynchronize());  // an earlier read-out may still read the old buffer
    if (p->d_gscale) cudaFree(p->d_gscale), p->used_bytes -= sizeof(double) * (size_t)p->gscale_cap;
    p->d_gscale = nullptr;
    p->gscale_cap = 0;
    int rc = plan_alloc(p, (void**)&p->d_gscale, sizeof(double) * (size_t)need);
    if (rc) return rc;
    p->gscale_cap = need;
  }
  k_glass_scale<<<(unsigned)std::min<int64_t>((need + 255) / 256, (int64_t)p->num_sms * 8), 256, 0, st>>>(
      d_glass, nglass, glass_box, tile, p->prm.box / tile, p->d_gscale);
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

int fused_readout_glass(Plan* p, int64_t nglass, int tile, float* d_pos, float* d_vel, int* d_ids, cudaStream_t st,
                        int64_t n0, int64_t n1) {
  const int64_t np = nglass * tile * tile * tile;
  if (n1 < 0 || n1 > np) n1 = np;
  if (n1 <= n0) return AAR_OK;
  const int bs = kReadoutThreads;
  const int64_t cnt = n1 - n0;
  { ProfScope ps_(p, "readout_glass", st);
  k_readout_glass<<<(unsigned)((cnt + bs - 1) / bs), bs, 0, st>>>(read_args(p), (const float*)p->d_work, p->d_gscale,
                                                                   nglass, tile, d_pos, d_vel, d_ids, n0, n1);
  }
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

}  // namespace aar

// ----------------------------------------------------------- standalone 3-D transforms
namespace aar {

template <int N>
__global__ void __launch_bounds__(256) k_rows_r2c(float2* f, int HP, int64_t nrows, const float2* __restrict__ twN,
                                                  const float2* __restrict__ twH) {
  using C = RowCfg<N>;
  constexpr int H = C::H;
  extern __shared__ float2 sm[];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int sub = lane / C::T, t = lane % C::T;
  int lines_per_block = (blockDim.x >> 5) * C::LPW;
  int64_t row = (int64_t)blockIdx.x * lines_per_block + warp * C::LPW + sub;
  bool act = row < nrows && sub < C::LPW;
  float2* line = sm + (warp * C::LPW + sub) * C::LS;
  float2* r = f + (act ? row : 0) * HP;
  if (act)
    for (int n = t; n < H; n += C::T) line[spad(n)] = r[n];
  __syncwarp();
  line_fft_smem<H, C::T, -1>(line, t, twH, act);
  if (act) row_r2c_post<N>(line, r, t, C::T, twN);
}

template <int N>
struct Xform {
  static constexpr int W = 8;
  static int c2r(Plan* p, float2* slot, cudaStream_t st) {
    using R = RowCfg<N>;
    int64_t tiles = (int64_t)N * (p->HP / W);
    int rc = run_pass<N>(p, AxisOp<N, W, 0, +1>{slot, 0, tiles, p->HP, nullptr}, tiles, st, "xform_x");
    if (rc) return rc;
    if ((rc = run_pass<N>(p, AxisOp<N, W, 1, +1>{slot, 0, tiles, p->HP, nullptr}, tiles, st, "xform_y"))) return rc;
    int lpb = 8 * R::LPW;
    int64_t nrows = (int64_t)N * N;
    dim3 g2((unsigned)((nrows + lpb - 1) / lpb), 1);
    {
      ProfScope ps_(p, "xform_rows", st);
      k_rows_c2r<N><<<g2, 256, sizeof(float2) * lpb * R::LS, st>>>(slot, 0, p->HP, 0, nrows, p->d_twN, p->d_twH,
                                                                  ZTypes{{0, 0, 0, 0, 0, 0}, 0.f, nullptr});
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    return AAR_OK;
  }
  static int r2c(Plan* p, float2* slot, cudaStream_t st) {
    using R = RowCfg<N>;
    int lpb = 8 * R::LPW;
    int64_t nrows = (int64_t)N * N;
    dim3 g2((unsigned)((nrows + lpb - 1) / lpb), 1);
    {
      ProfScope ps_(p, "xform_rows", st);
      k_rows_r2c<N><<<g2, 256, sizeof(float2) * lpb * R::LS, st>>>(slot, p->HP, nrows, p->d_twN, p->d_twH);
    }
    AAR_CUDA_TRY(p, cudaGetLastError());
    p->last_launches += 1;
    int64_t tiles = (int64_t)N * (p->HP / W);
    int rc = run_pass<N>(p, AxisOp<N, W, 1, -1>{slot, 0, tiles, p->HP, nullptr}, tiles, st, "xform_y");
    if (rc) return rc;
    return run_pass<N>(p, AxisOp<N, W, 0, -1>{slot, 0, tiles, p->HP, nullptr}, tiles, st, "xform_x");
  }
};

// Row copy between row orders: row (x, y) of src (order src_xb, ld src_ld
// elements) to row (x, y) of dst, the first ncols elements of each row.
// Moves fields between the caller's natural [x][y] buffers and the plan's
// x-blocked ones.
template <class T>
__global__ void k_copy_rows(T* __restrict__ dst, int64_t dst_ld, int dst_xb, const T* __restrict__ src, int64_t src_ld,
                            int src_xb, int N, int ncols) {
  const int64_t total = (int64_t)N * N * ncols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / ncols;
    const int c = (int)(i - r * ncols);
    const int x = (int)(r / N), y = (int)(r % N);
    dst[row_of(x, y, N, dst_xb) * dst_ld + c] = src[row_of(x, y, N, src_xb) * src_ld + c];
  }
}

int copy_rows(Plan* p, void* dst, int64_t dst_ld, int dst_xb, const void* src, int64_t src_ld, int src_xb, int ncols,
              size_t elem, cudaStream_t st) {
  const unsigned nb = (unsigned)(p->num_sms * 8);
  if (elem == sizeof(float2))
    k_copy_rows<float2><<<nb, 256, 0, st>>>((float2*)dst, dst_ld, dst_xb, (const float2*)src, src_ld, src_xb, p->N,
                                            ncols);
  else
    k_copy_rows<float><<<nb, 256, 0, st>>>((float*)dst, dst_ld, dst_xb, (const float*)src, src_ld, src_xb, p->N,
                                           ncols);
  AAR_CUDA_TRY(p, cudaGetLastError());
  return AAR_OK;
}

// unnormalised FFTW-convention transforms through work slot 0
int fused_c2r(Plan* p, const float2* in, float* out, cudaStream_t st) {
  int N = p->N, H = N / 2 + 1;
  float2* slot = p->d_work;
  int rc = copy_rows(p, slot, p->HP, kXB, in, H, 1, H, sizeof(float2), st);
  if (rc) return rc;
  if ((rc = dispatch_n(N, [&](auto nc) { return Xform<decltype(nc)::value>::c2r(p, slot, st); }))) return rc;
  return copy_rows(p, out, N, 1, slot, 2 * p->HP, kXB, N, sizeof(float), st);
}

int fused_r2c(Plan* p, const float* in, float2* out, cudaStream_t st) {
  int N = p->N, H = N / 2 + 1;
  float2* slot = p->d_work;
  int rc = copy_rows(p, slot, 2 * p->HP, kXB, in, N, 1, N, sizeof(float), st);
  if (rc) return rc;
  if ((rc = dispatch_n(N, [&](auto nc) { return Xform<decltype(nc)::value>::r2c(p, slot, st); }))) return rc;
  return copy_rows(p, out, H, 1, slot, p->HP, kXB, H, sizeof(float2), st);
}

int fused_configure_xform(Plan* p) {
  return dispatch_n(p->N, [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    using R = RowCfg<N>;
    int lpb = 8 * R::LPW;
    AAR_CUDA_TRY(p, cudaFuncSetAttribute(k_rows_c2r<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(float2) * lpb * R::LS)));
    AAR_CUDA_TRY(p, cudaFuncSetAttribute(k_rows_r2c<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(float2) * lpb * R::LS)));
    return Launch<N>::configure(p);
  });
}

}  // namespace aar
