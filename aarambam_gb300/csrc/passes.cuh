// Strided FFT passes (included by fused.cu).
//
// A pass is a list of work items (tile x field / component), one block per
// item; several blocks share an SM, so one block's cp.async tile load
// overlaps the FFT work of the others.  (Measured at N = 512 and 1024: a
// persistent loop over items lets the compiler keep loop-invariant twiddles
// live across items and spill, and a second tile buffer for prefetching
// halves the resident blocks; both were slower.)  An Op supplies
//   early(f, item)    per-element filter factors (table lookups) for the
//                     values this thread loads in the first FFT stage,
//                     issued before the tile wait so that both latencies
//                     overlap; the factors are applied as the first stage
//                     loads its values (no separate pass over the tile)
//   load(buf, item)   issue the cp.async copy of the item's input tile
//   pre(buf, item, f) optional in-place prologue once the tile has landed
//                     (returns true when it wrote shared memory)
//   body(buf, item, tw, f)  the FFT(s) (ends with a barrier)
//   store(buf, item)  epilogue + store to global memory
// Consecutive items run at the same time on consecutive blocks, so items
// that share an input tile (one phi tile for the M filters, the six 2LPT
// components) are ordered next to each other and hit L2.
#pragma once
// (included inside namespace aar)

// shared memory an Op needs after its tile (Op::kExtraSmem, 0 when absent)
template <class Op, class = void>
struct ExtraSmem {
  static constexpr size_t value = 0;
};
template <class Op>
struct ExtraSmem<Op, decltype((void)Op::kExtraSmem)> {
  static constexpr size_t value = Op::kExtraSmem;
};

template <int N, int W, class Op>
__global__ void __launch_bounds__(AxisCfg<N, W>::THREADS, AxisCfg<N, W>::MINB) k_pass(Op op, const float2* __restrict__ tw) {
  extern __shared__ float2 sm[];
  const int64_t it = blockIdx.x;
  op.load(sm, it);
  cp_async_commit();
  typename Op::Early f;
  op.early(f, it);
  cp_async_wait<0>();
  __syncthreads();
  if (op.pre(sm, it, f)) __syncthreads();
  op.body(sm, it, tw, f);
  op.store(sm, it);
}

// The (row n, column w) of the i-th value this thread takes in the first FFT
// stage of a tile (line w = thread / T, lane t = thread % T); false for
// threads without a line.
template <int N, int W>
__device__ __forceinline__ bool fft_owned(int i, int& n, int& w) {
  using C = AxisCfg<N, W>;
  w = threadIdx.x / C::T;
  n = first_load_index<N, C::T>(threadIdx.x % C::T, i);
  return w < W;
}

// In-place complex FFT along AXIS of fields (slot_map[f] or f), items
// f * tiles + t.
template <int N, int W, int AXIS, int SIGN>
struct AxisOp {
  float2* base;
  int64_t fs, tiles;
  int HP;
  const int* slot_map;  // optional field indirection (active modal slots)
  __device__ float2* field(int64_t item) const {
    int64_t f = item / tiles;
    return base + (slot_map ? (int64_t)slot_map[f] : f) * fs;
  }
  __device__ void coords(int64_t item, int& o, int& c0) const {
    int64_t t = item % tiles;
    int ncol = HP / W;
    o = (int)(t / ncol);
    c0 = (int)(t % ncol) * W;
  }
  __device__ void load(float2* b, int64_t item) const {
    int o, c0;
    coords(item, o, c0);
    tile_load_async<N, W, AXIS>(b, field(item), HP, o, c0);
  }
  struct Early {};
  __device__ void early(Early&, int64_t) const {}
  __device__ bool pre(float2*, int64_t, const Early&) const { return false; }
  __device__ void body(float2* b, int64_t, const float2* tw, const Early&) const {
    tile_fft<N, W, SIGN>(b, tw);
    __syncthreads();
  }
  __device__ void store(const float2* b, int64_t item) const {
    int o, c0;
    coords(item, o, c0);
    tile_store<N, W, AXIS>(b, field(item), HP, o, c0);
  }
};

// Item order of the x passes that write several output fields from one
// input tile: groups of `grp` consecutive tiles, and within a group all
// tiles of output 0, then all of output 1, ...  The blocks resident at one
// time then write into a few fields instead of all of them (each tile of an
// x pass touches one address per x row, N rows 4 MB apart at N = 1024), and
// the group's input tiles stay in L2 while its outputs are produced.
__device__ __forceinline__ void group_order(int64_t item, int64_t tiles, int nc, int64_t grp, int64_t& t, int& c) {
  const int64_t span = grp * nc;
  const int64_t g = item / span, r = item - g * span;
  const int64_t gs = min(grp, tiles - g * grp);  // the last group may be short
  c = (int)(r / gs);
  t = g * grp + (r - (int64_t)c * gs);
}

// First modal pass: item = (tile group, p, tile) (group_order); phi tile
// times q_p(k) (zero on the cut, DC and padding columns), inverse x FFT,
// into field p.  The factors come from the plan's filter cube (qcube_build:
// q_p over (|ky|, kz, |kx|), made once per table set with q_mode_cells'
// arithmetic): a lane's 16 factors of one column are 16 coalesced loads,
// issued before the tile wait so that both latencies overlap.  Evaluated per
// cell (qcube null: q_mode_cells, the Legendre recurrence per cell and mode)
// the pass was issue-bound, 58 ms at 1024^3 with 20 modes; a gather from a
// per-|k|^2 table (3 MB per mode, scattered indices) was latency-bound.
template <int N, int W>
struct XinvOp {
  ModalArgs a;
  const float2* phi;
  float2* work;
  int64_t fs, tiles;
  int HP;
  RhoArgs ra;
  int64_t grp;
  const float* qcube;  // [M][N/2+1 |ky|][N/2+1 kz][N/2+1 |kx|], or null
  __device__ void coords(int64_t item, int& o, int& c0, int& p) const {
    int64_t t;
    group_order(item, tiles, a.M, grp, t, p);
    int ncol = HP / W;
    o = (int)(t / ncol);
    c0 = (int)(t % ncol) * W;
  }
  __device__ void load(float2* b, int64_t item) const {
    int o, c0, p;
    coords(item, o, c0, p);
    tile_load_async<N, W, 0>(b, phi, HP, o, c0);
  }
  struct Early {
    float f[AxisCfg<N, W>::E];
  };
  __device__ void early(Early& r, int64_t item) const {
    using C = AxisCfg<N, W>;
    int o, c0, p;
    coords(item, o, c0, p);
    const int ky = sidx(o, N);
    if constexpr (C::E == 32 && stage_radix(N, C::E, 0) == 32 && C::THREADS == W * C::T && 32 % C::T == 0) {
      // value i of lane t is line element n = t + T i.  For n >= N/2 the
      // filter depends on |kx| = N - n, which is element 31 - i of lane
      // (T - t) % T of the same line (same ky, kz): each lane evaluates its
      // 16 values below N/2 and takes the other 16 from its partner by
      // shuffle.  Lane t = 0 pairs with itself one place off: |kx| = T (16 -
      // j) is its own value 16 - j for j >= 1, and N/2 (j = 0) is one more
      // evaluation.
      const int t = threadIdx.x % C::T, w = threadIdx.x / C::T;
      const int kz = c0 + w;
      const bool col = kz <= N / 2;
      float g[16];
      float gn = 0.f;  // lane 0: the value at n = N/2 (kx = -N/2)
      if (qcube) {
        constexpr int K = N / 2 + 1;
        const float* qr = qcube + (((int64_t)p * K + (ky < 0 ? -ky : ky)) * K + (col ? kz : 0)) * K;
#pragma unroll
        for (int i = 0; i < 16; ++i) g[i] = col ? __ldg(qr + t + C::T * i) : 0.f;
        if (t == 0) gn = col ? __ldg(qr + N / 2) : 0.f;
      } else {
        const int c2 = ky * ky + kz * kz;
        int n2[16];
        bool on[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int kx = t + C::T * i;  // < N/2
          n2[i] = kx * kx + c2;
          on[i] = col && n2[i] != 0 && keep_cell(a.g, kx, ky, kz);
          if (!on[i]) n2[i] = 1;  // a harmless argument; the value is dropped
        }
        q_mode_cells<16>(ra, p, n2, g);
#pragma unroll
        for (int i = 0; i < 16; ++i) g[i] = on[i] ? g[i] : 0.f;
        if (t == 0) {
          const int kx = -N / 2;
          int m2[1] = {kx * kx + c2};
          float v[1];
          q_mode_cells<1>(ra, p, m2, v);
          gn = col && keep_cell(a.g, kx, ky, kz) ? v[0] : 0.f;
        }
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) r.f[i] = g[i];
      const int lane = threadIdx.x & 31;
      const int src = (lane - t) + (C::T - t) % C::T;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float v = __shfl_sync(0xffffffffu, g[15 - j], src);
        r.f[16 + j] = t != 0 ? v : (j == 0 ? gn : g[j == 0 ? 0 : 16 - j]);
      }
    } else if (qcube) {
      constexpr int K = N / 2 + 1;
      const float* qp = qcube + ((int64_t)p * K + (ky < 0 ? -ky : ky)) * K * K;
#pragma unroll
      for (int i = 0; i < C::E; ++i) {
        int n, w;
        const bool own = fft_owned<N, W>(i, n, w);
        const int kz = c0 + w, kx = sidx(n, N);
        r.f[i] = own && kz <= N / 2 ? __ldg(qp + (int64_t)kz * K + (kx < 0 ? -kx : kx)) : 0.f;
      }
    } else {
      int n2[C::E];
      bool on[C::E];
#pragma unroll
      for (int i = 0; i < C::E; ++i) {
        int n, w;
        const bool own = fft_owned<N, W>(i, n, w);
        const int kz = c0 + w, kx = sidx(n, N);
        n2[i] = kx * kx + ky * ky + kz * kz;
        on[i] = own && kz <= N / 2 && n2[i] != 0 && keep_cell(a.g, kx, ky, kz);
        if (!on[i]) n2[i] = 1;
      }
      q_mode_cells<C::E>(ra, p, n2, r.f);
#pragma unroll
      for (int i = 0; i < C::E; ++i) r.f[i] = on[i] ? r.f[i] : 0.f;
    }
  }
  __device__ bool pre(float2*, int64_t, const Early&) const { return false; }
  __device__ void body(float2* b, int64_t, const float2* tw, const Early& r) const {
    tile_fft<N, W, +1, 1>(b, tw, r.f);
    __syncthreads();
  }
  __device__ void store(const float2* b, int64_t item) const {
    int o, c0, p;
    coords(item, o, c0, p);
    tile_store<N, W, 0>(b, work + (int64_t)p * fs, HP, o, c0);
  }
};

// 2LPT x passes.  The spectral factors of main.c:1180-1368 are products of
// one factor per axis, except 1/k^2 of psi2, which the forward x pass of the
// source applies (XfwdInvK2Op); so an x pass writes one field per distinct
// x factor and a fan-out y pass (YFanOp) and the c2r rows (ZFac) apply the
// rest.  KIND 0, Hessians d_ab = -k_a k_b T/(D Beta) phi: x factors -kF^2 kx^2,
// -kF^2 kx, -kF^2 (3 outputs).  KIND 1, displacements i k_a smth on
// T/(D Beta) phi (psi1) or on -S/k^2 (psi2), smth = [sinc_x sinc_y sinc_z]^-2:
// x factors i kF kx / sinc_x^2 and i / sinc_x^2 (2 outputs).  Items in
// group_order over the outputs.
template <int N, int W, int KIND>
struct LptXOp {
  static constexpr size_t kExtraSmem = sizeof(float) * N;  // x factor per x index
  LptArgs a;
  const float2* src;
  float2* work;
  int64_t fs, tiles;
  int HP;
  int out[3];
  int64_t grp;
  static constexpr int NC = KIND == 0 ? 3 : 2;
  __device__ void coords(int64_t item, int& o, int& c0, int& comp) const {
    int64_t t;
    group_order(item, tiles, NC, grp, t, comp);
    int ncol = HP / W;
    o = (int)(t / ncol);
    c0 = (int)(t % ncol) * W;
  }
  __device__ static float* table(float2* b) { return (float*)(b + W * AxisCfg<N, W>::LS); }
  __device__ void load(float2* b, int64_t item) const {
    int o, c0, comp;
    coords(item, o, c0, comp);
    tile_load_async<N, W, 0>(b, src, HP, o, c0);
    float* tab = table(b);
    const float kF = a.m.g.kF;
    constexpr int TH = AxisCfg<N, W>::THREADS;
#pragma unroll
    for (int j = 0; j < (N + TH - 1) / TH; ++j) {
      const int n = threadIdx.x + j * TH;
      if (n >= N) break;
      const float kx = (float)sidx(n, N);
      float f;
      if (KIND == 0) {
        f = comp == 0 ? -kF * kF * kx * kx : comp == 1 ? -kF * kF * kx : -kF * kF;
      } else {
        const float is2 = __ldg(a.isinc2 + n);
        f = comp == 0 ? kF * kx * is2 : is2;
      }
      tab[n] = f;
    }
  }
  struct Early {};
  __device__ void early(Early&, int64_t) const {}
  __device__ bool pre(float2*, int64_t, const Early&) const { return false; }
  __device__ void body(float2* b, int64_t item, const float2* tw, const Early&) const {
    using C = AxisCfg<N, W>;
    int o, c0, comp;
    coords(item, o, c0, comp);
    const float* tab = table(b);
    float f[C::E];
#pragma unroll
    for (int i = 0; i < C::E; ++i) {
      int n, w;
      const bool own = fft_owned<N, W>(i, n, w);
      f[i] = own && c0 + w <= N / 2 ? tab[n] : 0.f;
    }
    tile_fft<N, W, +1, KIND == 0 ? 1 : 2>(b, tw, f);
    __syncthreads();
  }
  __device__ void store(const float2* b, int64_t item) const {
    int o, c0, comp;
    coords(item, o, c0, comp);
    tile_store<N, W, 0>(b, work + (int64_t)out[comp] * fs, HP, o, c0);
  }
};

// Inverse y pass fanning fields out: item (tile, c), c < NC: field in[c]
// times the y factor type[c] (axis_factor), inverse y FFT, into out[c].
// Outputs never alias an input that another item still reads (an in-place
// output reads only its own input).  The factor of every y index is put in
// shared memory (after the tile) while the tile loads and read after the
// barrier: per-value global loads in the first stage measured 18.3 vs 13.3
// ms at 1024^3 (their latency was exposed after the barrier).
template <int N, int W>
struct YFanOp {
  static constexpr int NC = 6;
  static constexpr size_t kExtraSmem = sizeof(float) * N;
  LptArgs a;
  float2* work;
  int64_t fs, tiles;
  int HP;
  int in[NC], out[NC], type[NC];
  int64_t grp;
  __device__ void coords(int64_t item, int& o, int& c0, int& c) const {
    int64_t t;
    group_order(item, tiles, NC, grp, t, c);
    int ncol = HP / W;
    o = (int)(t / ncol);
    c0 = (int)(t % ncol) * W;
  }
  __device__ static float* table(float2* b) { return (float*)(b + W * AxisCfg<N, W>::LS); }
  __device__ void load(float2* b, int64_t item) const {
    int o, c0, c;
    coords(item, o, c0, c);
    tile_load_async<N, W, 1>(b, work + (int64_t)in[c] * fs, HP, o, c0);
    float* tab = table(b);
    const int ty = type[c];
    constexpr int TH = AxisCfg<N, W>::THREADS;
#pragma unroll
    for (int j = 0; j < (N + TH - 1) / TH; ++j) {
      const int n = threadIdx.x + j * TH;
      if (n < N) tab[n] = axis_factor(ty, sidx(n, N), a.m.g.kF, a.isinc2, n);
    }
  }
  struct Early {};
  __device__ void early(Early&, int64_t) const {}
  __device__ bool pre(float2*, int64_t, const Early&) const { return false; }
  __device__ void body(float2* b, int64_t, const float2* tw, const Early&) const {
    using C = AxisCfg<N, W>;
    const float* tab = table(b);
    float f[C::E];
#pragma unroll
    for (int i = 0; i < C::E; ++i) {
      int n, w;
      fft_owned<N, W>(i, n, w);
      f[i] = tab[n];
    }
    tile_fft<N, W, +1, 1>(b, tw, f);
    __syncthreads();
  }
  __device__ void store(const float2* b, int64_t item) const {
    int o, c0, c;
    coords(item, o, c0, c);
    tile_store<N, W, 1>(b, work + (int64_t)out[c] * fs, HP, o, c0);
  }
};

// Forward x pass of the 2LPT source in place, then S <- -S / (kF^2 |k|^2)
// (0 at k = 0): the non-separable part of psi2 = -i k_a / k^2 S smth
// (main.c:1356-1363).
template <int N, int W>
struct XfwdInvK2Op {
  float2* f;
  int64_t tiles;
  int HP;
  float kF;
  __device__ void coords(int64_t item, int& o, int& c0) const {
    int ncol = HP / W;
    o = (int)(item / ncol);
    c0 = (int)(item % ncol) * W;
  }
  __device__ void load(float2* b, int64_t item) const {
    int o, c0;
    coords(item, o, c0);
    tile_load_async<N, W, 0>(b, f, HP, o, c0);
  }
  struct Early {};
  __device__ void early(Early&, int64_t) const {}
  __device__ bool pre(float2*, int64_t, const Early&) const { return false; }
  __device__ void body(float2* b, int64_t, const float2* tw, const Early&) const {
    tile_fft<N, W, -1>(b, tw);
    __syncthreads();
  }
  __device__ void store(const float2* b, int64_t item) const {
    using C = AxisCfg<N, W>;
    int o, c0;
    coords(item, o, c0);
    const TileAddr<N, W, 0> ta(HP, o, c0);
    const int ky = sidx(o, N), kz = c0 + ta.w;
#pragma unroll 4
    for (int q = 0; q < C::PER; ++q) {
      const int kx = sidx(ta.n0 + q * TileAddr<N, W, 0>::DN, N);
      const int n2 = kx * kx + ky * ky + kz * kz;
      const float g = n2 ? -1.f / (kF * kF * (float)n2) : 0.f;
      const float2 v = b[ta.s(q)];
      f[ta.g(q)] = make_float2(v.x * g, v.y * g);
    }
  }
};

