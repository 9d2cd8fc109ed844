// Seed table and Gaussian potential (white noise) kernels.
//
// Seed table (Aarambam/LPT/Basis/main.c:317-349): one ranlxd1 stream seeded
// with Seed delivers N^2 uniforms, stored as (unsigned)(0x7fffffff * u) in
// eight "shell" segments per i < N/2.  The stream is split into segments of
// rlx_seg refills; each thread rebuilds its segment's starting state with the
// exact skip-ahead of ranlux.cuh and scatters its draws (the shell order is a
// permutation of the table, so the scatter has no write conflicts).
//
// Noise (main.c:382-524): one thread per (i, j) column reseeds ranlxd1 with
// seedtable[i][j] and draws (phase, amplitude) pairs for k < N/2, skipping the
// Nyquist indices and DC after the draws, keeping the cube/sphere cut, and
// writing the k = 0 plane with its Hermitian partner.  The fused plan's
// spectrum is written in its x-blocked row order; the plain form and the
// caller's buffers in the natural one.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "aar_internal.cuh"
#include "ranlux.cuh"

namespace aar {

__device__ __forceinline__ int64_t shell_pos(int64_t d, int N) {
  // draws before shell i: 4 i^2; segment lengths i, i+1, i, i+1, ...
  int64_t i = (int64_t)sqrt((double)d) / 2;
  while (4 * (i + 1) * (i + 1) <= d) ++i;
  while (4 * i * i > d) --i;
  int64_t o = d - 4 * i * i;
  int64_t n = N;
  if (o < i) return i * n + o;
  o -= i;
  if (o < i + 1) return o * n + i;
  o -= i + 1;
  if (o < i) return (n - 1 - i) * n + o;
  o -= i;
  if (o < i + 1) return (n - 1 - o) * n + i;
  o -= i + 1;
  if (o < i) return i * n + (n - 1 - o);
  o -= i;
  if (o < i + 1) return o * n + (n - 1 - i);
  o -= i + 1;
  if (o < i) return (n - 1 - i) * n + (n - 1 - o);
  o -= i;
  return (n - 1 - o) * n + (n - 1 - i);
}

__global__ void k_seedtable(uint32_t seed, int N, int seg, const U576* __restrict__ pw, int npw,
                            uint32_t* __restrict__ table) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = (int64_t)N * N;
  int64_t d0 = g * 12 * seg;
  if (d0 >= total) return;
  Rlx s;
  rlx_seed(s, seed);
  if (g > 0) {
    U576 r = rlx_window_residue(s);
    for (int b = 0; b < npw; ++b)
      if ((g >> b) & 1) r = modmul576(r, pw[b]);
    rlx_from_residue(r, s);
  }
  int64_t d1 = d0 + 12 * (int64_t)seg;
  if (d1 > total) d1 = total;
  for (int64_t d = d0; d < d1; ++d) {
    double u = (double)rlx_next48(s) * 3.5527136788005009e-15;  // 2^-48
    table[shell_pos(d, N)] = __double2uint_rz(__dmul_rn(2147483647.0, u));
  }
}

int launch_seedtable(Plan* p, uint32_t seed, uint32_t* d_out, cudaStream_t st) {
  int64_t total = (int64_t)p->N * p->N;
  int64_t draws_per = 12 * (int64_t)p->rlx_seg;
  int64_t nthr = (total + draws_per - 1) / draws_per;
  int bs = 64;
  { ProfScope ps_(p, "seedtable", st);
  k_seedtable<<<(unsigned)((nthr + bs - 1) / bs), bs, 0, st>>>(seed, p->N, p->rlx_seg, (const U576*)p->d_rlxpow,
                                                                 32, d_out);
  }
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

// ------------------------------------------------------------ noise
struct NoiseArgs {
  Grid g;
  int xb;  // row order of the output: row_of(i, j, N, xb)
  int phase_flip, fixed_amp;
  int one_draw;  // every column one draw at a time (AAR_NOISE_ONE_DRAW=1: checks the six-cell blocks)
  // FP64 form: the reference's own formula
  double anorm, ns, fac, beta;
  aar_params prm;  // variant and ResBasis oscillation (noise_osc)
  // FP32 form: amplitude per n^2 = sqrt(Anorm k^ns osc) fac Beta / k^2
  const float* amp;
};

// -ln(u) for u = U 2^-48 in (0, 1), FP32 with the small-(1-u) branch exact
__device__ __forceinline__ float neg_log_u48(uint64_t U) {
  if (U < (uint64_t(1) << 47)) return -logf((float)U * 3.5527136788005009e-15f);  // u < 1/2
  float oneminus = (float)((uint64_t(1) << 48) - U) * 3.5527137e-15f;
  return -log1pf(-oneminus);
}

// cos / sin of 2 pi u (+ pi when flipped) for u = U 2^-48, FP32: the exact
// split U = H 2^24 + L gives sincospi(H 2^-23) plus a first-order correction.
__device__ __forceinline__ void sincos_u48(uint64_t U, bool flip, float& c, float& s) {
  uint32_t H = (uint32_t)(U >> 24), L = (uint32_t)(U & 0xFFFFFFu);
  float a = (float)H * 1.1920928955078125e-07f;  // H 2^-23 (exact)
  float s0, c0;
  sincospif(a, &s0, &c0);
  float d = (float)L * (float)(3.14159265358979323846 / 140737488355328.0);
  c = c0 - d * s0;
  s = s0 + d * c0;
  if (flip) {
    c = -c;
    s = -s;
  }
}

// One cell (i, j, k) of a column from its two uniforms U1 (phase), U2
// (amplitude): the Nyquist / DC skips after the draws, the cut, the
// Hermitian pair of the k = 0 plane (main.c:396-459).  FP64: the amplitude
// and phase by the reference's FP64 formula (main.c:443-459); OUT64: double2
// output (the plain forms), else float2 (the fused form, FP64 math rounded at
// the end when FP64).
template <bool FP64, bool OUT64>
__device__ __forceinline__ void noise_cell(const NoiseArgs& a, int i, int j, int k, uint64_t U1, uint64_t U2, double fx,
                                           double fy, void* __restrict__ out, int HP) {
  const int N = a.g.N;
  if (i == N / 2 || j == N / 2) return;
  if (i == 0 && j == 0 && k == 0) return;
  const int kx = sidx(i, N), ky = sidx(j, N);
  if (!keep_cell(a.g, kx, ky, k)) return;
  const double box = a.g.box;
  double re, im;
  float rf = 0.f, imf = 0.f;
  if (FP64) {
    double fz = __ddiv_rn(__dmul_rn((double)(2 * k), kPi), box);
    double k2 = __dadd_rn(__dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fy, fy)), __dmul_rn(fz, fz));
    double km = sqrt(k2);
    double phase = __dmul_rn(__dmul_rn((double)U1 * 3.5527136788005009e-15, 2.0), kPi);
    if (a.phase_flip) phase = __dadd_rn(phase, kPi);
    double ampl = (double)U2 * 3.5527136788005009e-15;
    double phig = noise_osc(a.prm, a.anorm * exp(a.ns * log(km)), km);
    if (!a.fixed_amp) phig *= -log(ampl);
    phig = sqrt(phig) * a.fac * a.beta / k2;
    double sn, cs;
    sincos(phase, &sn, &cs);
    re = phig * cs;
    im = phig * sn;
    rf = (float)re;
    imf = (float)im;
  } else {
    int n2 = kx * kx + ky * ky + k * k;
    float amp = __ldg(a.amp + n2);
    if (!a.fixed_amp) amp *= sqrtf(neg_log_u48(U2));
    float c, sn;
    sincos_u48(U1, a.phase_flip != 0, c, sn);
    rf = amp * c;
    imf = amp * sn;
    re = rf;
    im = imf;
  }
  int64_t c1 = -1, c2 = -1;
  if (k > 0) {
    c1 = row_of(i, j, N, a.xb) * HP + k;
  } else if (i == 0) {
    if (j >= N / 2) return;
    c1 = row_of(0, j, N, a.xb) * HP;
    c2 = row_of(0, N - j, N, a.xb) * HP;
  } else {
    if (i >= N / 2) return;
    int ii = N - i, jj = (N - j) % N;
    c1 = row_of(i, j, N, a.xb) * HP;
    c2 = row_of(ii, jj, N, a.xb) * HP;
  }
  if (OUT64) {
    double2* o = (double2*)out;
    o[c1] = make_double2(re, im);
    if (c2 >= 0) o[c2] = make_double2(re, -im);
  } else {
    float2* o = (float2*)out;
    o[c1] = make_float2(rf, imf);
    if (c2 >= 0) o[c2] = make_float2(rf, -imf);
  }
}

// The rest of a column from cell k on with the generator as it stands:
// draws one by one (U2 == 0 redrawn, main.c:401-403).  Taken from the
// start of the first refill block whose pairing a redraw would shift -- a
// zero U2 has probability 2^-48 -- and never otherwise.  Not inlined: the
// state indexed by its running position lives in local memory here only.
template <bool FP64, bool OUT64>
__device__ __noinline__ void noise_column_rest(NoiseArgs a, Rlx s, int i, int j, int k, double fx, double fy,
                                                void* __restrict__ out, int HP) {
  for (; k < a.g.N / 2; ++k) {
    const uint64_t U1 = rlx_next48(s);
    uint64_t U2;
    do U2 = rlx_next48(s);
    while (U2 == 0);
    noise_cell<FP64, OUT64>(a, i, j, k, U1, U2, fx, fy, out, HP);
  }
}

// One thread per (i, j) column.  A refill of ranlxd1 gives 12 uniforms, the
// (U1, U2) pairs of six cells while no U2 is zero: the column runs in blocks
// of six cells reading the refilled state at compile-time indices (it stays
// in registers), and a block with a zero U2 hands the column from its first
// draw to noise_column_rest.  Same draws, same cells as one draw at a time.
template <bool FP64, bool OUT64 = FP64>
__global__ void k_noise(NoiseArgs a, const uint32_t* __restrict__ seedtable, void* __restrict__ out, int HP) {
  const int N = a.g.N;
  int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= (int64_t)N * N) return;
  const int i = (int)(col / N), j = (int)(col % N);
  Rlx s;
  rlx_seed(s, seedtable[col]);
  double fx = 0, fy = 0;
  if (FP64) {
    fx = __ddiv_rn(__dmul_rn((double)(2 * sidx(i, N)), kPi), a.g.box);
    fy = __ddiv_rn(__dmul_rn((double)(2 * sidx(j, N)), kPi), a.g.box);
  }
  if (a.one_draw) {
    noise_column_rest<FP64, OUT64>(a, s, i, j, 0, fx, fy, out, HP);
    return;
  }
  for (int k = 0; k < N / 2; k += 6) {
    rlx_refill(s);  // every block consumes whole refills: the position is 12 here
    const int nk = min(6, N / 2 - k);
    bool zero = false;
#pragma unroll
    for (int c = 0; c < 6; ++c) zero |= c < nk && s.x[2 * c + 1] == 0;
    if (zero) {
      noise_column_rest<FP64, OUT64>(a, s, i, j, k, fx, fy, out, HP);
      return;
    }
#pragma unroll
    for (int c = 0; c < 6; ++c)
      if (c < nk) noise_cell<FP64, OUT64>(a, i, j, k + c, s.x[2 * c], s.x[2 * c + 1], fx, fy, out, HP);
  }
}

static NoiseArgs noise_args(Plan* p, int xb) {
  NoiseArgs a;
  a.g = p->grid;
  a.xb = xb;
  a.phase_flip = p->prm.phase_flip == 1;
  a.fixed_amp = p->prm.fixed_amplitude != 0;
  a.one_draw = p->noise_one_draw;
  a.anorm = p->Anorm;
  a.ns = p->prm.primordial_index;
  a.fac = pow(2 * kPi / p->prm.box, 1.5);
  a.beta = p->Beta;
  a.prm = p->prm;
  a.amp = p->d_amp;
  return a;
}

int launch_noise_fp32(Plan* p, const uint32_t* d_seed, float2* d_phik, cudaStream_t st) {
  size_t bytes = sizeof(float2) * (size_t)p->N * p->N * p->HP;
  AAR_CUDA_TRY(p, cudaMemsetAsync(d_phik, 0, bytes, st));
  int64_t cols = (int64_t)p->N * p->N;
  int bs = 128;
  { ProfScope ps_(p, "noise", st);
  if (p->prm.noise_fp64)
    k_noise<true, false><<<(unsigned)((cols + bs - 1) / bs), bs, 0, st>>>(noise_args(p, kXB), d_seed, d_phik, p->HP);
  else
    k_noise<false><<<(unsigned)((cols + bs - 1) / bs), bs, 0, st>>>(noise_args(p, kXB), d_seed, d_phik, p->HP);
  }
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

int launch_noise_fp64(Plan* p, const uint32_t* d_seed, double2* d_phik, int hp, cudaStream_t st) {
  size_t bytes = sizeof(double2) * (size_t)p->N * p->N * hp;
  AAR_CUDA_TRY(p, cudaMemsetAsync(d_phik, 0, bytes, st));
  int64_t cols = (int64_t)p->N * p->N;
  int bs = 128;
  { ProfScope ps_(p, "noise", st);
  k_noise<true><<<(unsigned)((cols + bs - 1) / bs), bs, 0, st>>>(noise_args(p, 1), d_seed, d_phik, hp);
  }
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches += 1;
  return AAR_OK;
}

// ------------------------------------------- no-allocation Gaussian spectrum
// Scratch of aar_gaussian_spectrum_noalloc: the seed table, one uint32 per
// (x, y) column of an Nmesh <= kNoAllocMaxN grid (4 MiB).  It is static
// device memory of this library, reserved when the CUDA module is loaded, so
// the call itself allocates nothing.  k_seedtable writes every entry before
// k_noise reads any, so nothing in it has to start at zero.  There is one
// scratch per device: calls that overlap on one device race on it.
constexpr int kNoAllocMaxN = 1024;
static __device__ __align__(256) uint32_t g_noalloc_seed[kNoAllocMaxN * kNoAllocMaxN];

// Address of the scratch on the plan's device, resolved once per device with
// cudaGetSymbolAddress (the first call on a device does this set-up).
static int noalloc_scratch(Plan* p, uint32_t** out) {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static uint32_t* addr[kMaxDev] = {};
  int dev = -1;
  AAR_CUDA_TRY(p, cudaGetDevice(&dev));
  if (dev != p->dev) return set_err(p, "the current device is not the plan's device"), AAR_ERR_ARG;
  if (dev < 0 || dev >= kMaxDev) return set_err(p, "device ordinal out of range"), AAR_ERR_ARG;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* a = nullptr;
    AAR_CUDA_TRY(p, cudaGetSymbolAddress(&a, g_noalloc_seed));
    addr[dev] = (uint32_t*)a;
  }
  *out = addr[dev];
  return AAR_OK;
}

// The Gaussian potential spectrum of the plan's seed straight into the
// caller's complex [N][N][N/2+1] buffer (float32 pairs for the fused form,
// float64 for the plain form), with the seed table in the static scratch
// instead of the plan's seed-table buffer.  Same kernels and arguments as
// launch_seedtable + launch_noise_fp32 / _fp64.
int noalloc_gaussian(Plan* p, void* d_out, cudaStream_t st) {
  const int N = p->N;
  if (N > kNoAllocMaxN)
    return set_err(p, "Nmesh " + std::to_string(N) + " exceeds the no-allocation scratch (Nmesh <= " +
                          std::to_string(kNoAllocMaxN) + ")"),
           AAR_ERR_ARG;
  uint32_t* seed = nullptr;
  int rc = noalloc_scratch(p, &seed);
  if (rc) return rc;
  const int64_t total = (int64_t)N * N;
  const int64_t draws_per = 12 * (int64_t)p->rlx_seg;
  const int64_t nthr = (total + draws_per - 1) / draws_per;
  k_seedtable<<<(unsigned)((nthr + 63) / 64), 64, 0, st>>>((uint32_t)p->prm.seed, N, p->rlx_seg,
                                                           (const U576*)p->d_rlxpow, 32, seed);
  AAR_CUDA_TRY(p, cudaGetLastError());
  const int hp = N / 2 + 1;
  const bool fp64 = is_plain(p->prm);
  AAR_CUDA_TRY(p, cudaMemsetAsync(d_out, 0, (fp64 ? sizeof(double2) : sizeof(float2)) * (size_t)total * hp, st));
  const unsigned nb = (unsigned)((total + 127) / 128);
  if (fp64)
    k_noise<true><<<nb, 128, 0, st>>>(noise_args(p, 1), seed, d_out, hp);
  else if (p->prm.noise_fp64)
    k_noise<true, false><<<nb, 128, 0, st>>>(noise_args(p, 1), seed, d_out, hp);
  else
    k_noise<false><<<nb, 128, 0, st>>>(noise_args(p, 1), seed, d_out, hp);
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches = 2;
  return AAR_OK;
}

}  // namespace aar
