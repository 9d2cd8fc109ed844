// Adjoint (reverse-mode) kernels of the fused FP32 path: white noise ->
// Gaussian potential -> modal non-Gaussian potential -> ZA + 2LPT
// displacements.  The transforms of the chain are the plan's own (aar_c2r /
// aar_r2c); these kernels are the per-cell spectral factors and the
// real-space products, forward (for recomputation) and transposed.
//
// Transposes of the FFTW-convention transforms on half spectra (kz = 0..N/2):
// a c2r sums w(kz) Re(X_k e^{i k.x}) with w = 1 on the kz = 0 and N/2 planes
// and 2 elsewhere, so c2r^T(G) = w r2c(G) (an unnormalised forward
// transform), and r2c^T(g) = c2r(g / w).  A complex factor F acting on
// (Re, Im) transposes to conj(F).
//
// Layouts (the C-ABI ones): complex [N][N][N/2+1] float2, real [N][N][N]
// float.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "aar_internal.cuh"
#include "fft.cuh"
#include "spectral.cuh"

namespace aar {

struct SpecArgs {
  LptArgs l;
  const float* amp;   // per n^2 noise amplitude
  const float* qtab;  // [M][nsq]
  const float* rtab;  // [nsq][rstride]
  int64_t nsq;
  int rstride;
  float fnl_n3;       // Fnl / N^3
};

// forward factor of op `op`, component / mode `comp`, at one cell
__device__ __forceinline__ float2 spec_factor(const SpecArgs& s, int op, int comp, int i, int j, int kz) {
  const Grid& g = s.l.m.g;
  const int N = g.N;
  const int kx = sidx(i, N), ky = sidx(j, N);
  const int n2 = kx * kx + ky * ky + kz * kz;
  switch (op) {
    case AAR_ADJ_OP_ONE:
      return make_float2(1.f, 0.f);
    case AAR_ADJ_OP_GAUSS: {
      // the cells the noise kernel writes (main.c:405-441): no Nyquist
      // index, no kz = N/2 plane, no DC, inside the cut
      const bool on = i != N / 2 && j != N / 2 && kz < N / 2 && n2 != 0 && keep_cell(g, kx, ky, kz);
      return make_float2(on ? __ldg(s.amp + n2) : 0.f, 0.f);
    }
    case AAR_ADJ_OP_Q: {
      const bool on = n2 != 0 && keep_cell(g, kx, ky, kz);
      return make_float2(on ? __ldg(s.qtab + (int64_t)comp * s.nsq + n2) : 0.f, 0.f);
    }
    case AAR_ADJ_OP_RHO: {
      const bool on = n2 != 0 && keep_cell(g, kx, ky, kz);
      return make_float2(on ? s.fnl_n3 * __ldg(s.rtab + (int64_t)n2 * s.rstride + comp) : 0.f, 0.f);
    }
    case AAR_ADJ_OP_HESS:
      return lpt_factor<0>(s.l, comp, i, j, kz, kx, ky, n2);
    case AAR_ADJ_OP_PSI1:
      return lpt_factor<1>(s.l, comp, i, j, kz, kx, ky, n2);
    case AAR_ADJ_OP_PSI2:
      return lpt_factor<2>(s.l, comp, i, j, kz, kx, ky, n2);
  }
  return make_float2(0.f, 0.f);
}

// out (+)= M(F) in, M(F) = F (mode 0), conj(F) w (1), conj(F) / w (2), conj(F) (3)
__global__ void __launch_bounds__(256) k_spec(SpecArgs s, int op, int comp, int mode, const float2* __restrict__ in,
                                              float2* out, int accumulate) {
  const int N = s.l.m.g.N, K = N / 2 + 1;
  const int64_t total = (int64_t)N * N * K;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = e / K;
    const int kz = (int)(e - row * K);
    const int i = (int)(row / N), j = (int)(row % N);
    float2 f = spec_factor(s, op, comp, i, j, kz);
    if (mode != 0) {
      f.y = -f.y;
      const float w = (kz == 0 || kz == N / 2) ? 1.f : 2.f;
      if (mode == 1) f = make_float2(f.x * w, f.y * w);
      if (mode == 2) f = make_float2(f.x / w, f.y / w);
    }
    const float2 r = cmul(in[e], f);
    if (accumulate) {
      const float2 o = out[e];
      out[e] = make_float2(o.x + r.x, o.y + r.y);
    } else {
      out[e] = r;
    }
  }
}

// Transpose of the 2LPT source S = d00 (d11 + d22) + d11 d22 - d01^2 - d02^2
// - d12^2 (main.c:1284-1294), fields in the order 00 01 02 11 12 22.
__global__ void __launch_bounds__(256) k_source_adj(const float* __restrict__ d, const float* __restrict__ gS, float* gd,
                                                    int64_t n) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const float g = gS[x];
    const float d00 = d[x], d01 = d[n + x], d02 = d[2 * n + x], d11 = d[3 * n + x], d12 = d[4 * n + x],
                d22 = d[5 * n + x];
    gd[x] = g * (d11 + d22);
    gd[n + x] = -2.f * g * d01;
    gd[2 * n + x] = -2.f * g * d02;
    gd[3 * n + x] = g * (d00 + d22);
    gd[4 * n + x] = -2.f * g * d12;
    gd[5 * n + x] = g * (d00 + d11);
  }
}

// Transposes of the modal products g_r = sum_t c_t f_p f_q (the plan's term
// list, counter-terms included):
//   gf_p = sum_t c_t gg_{r_t} (f_q [p = p_t] + f_p [p = q_t])
// and the coefficient sums  G_k = sum_x gg_r f_p f_q  for every triple k of
// `trip` (all sorted triples plus the counter-term product), accumulated per
// block in FP64 shared memory and added to gsum once per block.  Blocks loop
// over chunks of kChunk positions staged in shared memory.
constexpr int kChunk = 128;
constexpr int kLd = kChunk + 1;  // staged row stride (rows start on different banks)
struct AdjTerm {
  int p, q, r;
  float c;
};

__global__ void __launch_bounds__(kChunk) k_products_adj(const float* __restrict__ f, const float* __restrict__ gg,
                                                         float* gf, int M, int64_t n, const AdjTerm* __restrict__ terms,
                                                         int nterms, const int* __restrict__ trip, int ntrip,
                                                         double* gsum) {
  extern __shared__ double shd[];
  double* acc = shd;                          // [ntrip]
  float* sf = (float*)(shd + ntrip);          // [M][kLd]
  float* sg = sf + M * kLd;                   // [M][kLd]
  float* sgf = sg + M * kLd;                  // [M][kLd]
  const int t = threadIdx.x;
  for (int k = t; k < ntrip; k += kChunk) acc[k] = 0.0;
  for (int64_t x0 = (int64_t)blockIdx.x * kChunk; x0 < n; x0 += (int64_t)gridDim.x * kChunk) {
    const int64_t x = x0 + t;
    const bool in = x < n;
    __syncthreads();  // previous chunk's readers are done
    for (int m = 0; m < M; ++m) {
      sf[m * kLd + t] = in ? f[(int64_t)m * n + x] : 0.f;
      sg[m * kLd + t] = in ? gg[(int64_t)m * n + x] : 0.f;
      sgf[m * kLd + t] = 0.f;
    }
    __syncthreads();
    for (int k = 0; k < nterms; ++k) {
      const AdjTerm tm = terms[k];
      const float v = tm.c * sg[tm.r * kLd + t];
      const float fp = sf[tm.p * kLd + t], fq = sf[tm.q * kLd + t];
      sgf[tm.p * kLd + t] += v * fq;
      sgf[tm.q * kLd + t] += v * fp;
    }
    if (in)
      for (int m = 0; m < M; ++m) gf[(int64_t)m * n + x] = sgf[m * kLd + t];
    for (int k = t; k < ntrip; k += kChunk) {
      const int p = trip[3 * k], q = trip[3 * k + 1], r = trip[3 * k + 2];
      float s = 0.f;
      for (int u = 0; u < kChunk; ++u) s += sg[r * kLd + u] * sf[p * kLd + u] * sf[q * kLd + u];
      acc[k] += (double)s;
    }
  }
  __syncthreads();
  for (int k = t; k < ntrip; k += kChunk) atomicAdd(gsum + k, acc[k]);
}

static SpecArgs spec_args(Plan* p) {
  SpecArgs s;
  s.l = lpt_args(p);
  s.amp = p->d_amp;
  s.qtab = p->d_qtab;
  s.rtab = p->d_rtab;
  s.nsq = p->nsq;
  s.rstride = p->rtab_stride;
  s.fnl_n3 = (float)(p->prm.fnl / ((double)p->N * p->N * p->N));
  return s;
}

int adj_spectral(Plan* p, int op, int comp, int mode, const float2* in, float2* out, int accumulate,
                 cudaStream_t st) {
  if (op < AAR_ADJ_OP_ONE || op > AAR_ADJ_OP_PSI2 || mode < 0 || mode > 3) return set_err(p, "bad adjoint op"), AAR_ERR_ARG;
  const int lim = op == AAR_ADJ_OP_HESS ? 6 : (op == AAR_ADJ_OP_PSI1 || op == AAR_ADJ_OP_PSI2) ? 3
                  : (op == AAR_ADJ_OP_Q || op == AAR_ADJ_OP_RHO) ? p->M : 1;
  if (comp < 0 || comp >= lim) return set_err(p, "adjoint op component out of range"), AAR_ERR_ARG;
  k_spec<<<(unsigned)(p->num_sms * 8), 256, 0, st>>>(spec_args(p), op, comp, mode, in, out, accumulate);
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches = 1;
  return AAR_OK;
}

int adj_source(Plan* p, const float* d, const float* gS, float* gd, cudaStream_t st) {
  const int64_t n = (int64_t)p->N * p->N * p->N;
  k_source_adj<<<(unsigned)(p->num_sms * 8), 256, 0, st>>>(d, gS, gd, n);
  AAR_CUDA_TRY(p, cudaGetLastError());
  p->last_launches = 1;
  return AAR_OK;
}

// Term list of the forward products with explicit target r (counter-terms
// included), from the plan's host copy; triples = every sorted (p, q, r)
// followed by the counter-term product (0, 2, 1) when it exists.
int adj_products(Plan* p, const float* f, const float* gg, float* gf, double* galpha, cudaStream_t st) {
  const int M = p->M;
  if (p->host_terms.size() < sizeof(int) * 2) return set_err(p, "coefficient tables not set"), AAR_ERR_STATE;
  const TermList& tl = *(const TermList*)p->host_terms.data();
  const Term* ft = (const Term*)(p->host_terms.data() + sizeof(TermList));
  std::vector<AdjTerm> terms;
  for (int i = 0; i < tl.nterms; ++i)
    if (ft[i].c != 0.f) terms.push_back(AdjTerm{ft[i].p, ft[i].q, ft[i].r, ft[i].c});
  std::vector<int> trip;
  for (int a = 0; a < M; ++a)
    for (int b = a; b < M; ++b)
      for (int c = b; c < M; ++c) trip.insert(trip.end(), {a, b, c});
  const int nsorted = (int)trip.size() / 3;
  trip.insert(trip.end(), {0, 2, 1});
  const int ntrip = (int)trip.size() / 3;
  // device copies in plan-owned scratch (allocated once per size)
  const size_t off_trip = sizeof(AdjTerm) * terms.size();
  const size_t off_sum = (off_trip + sizeof(int) * trip.size() + 7) / 8 * 8;
  const size_t need = off_sum + sizeof(double) * ntrip;
  if (p->adj_scratch_bytes < need) {
    if (p->d_adj_scratch) cudaFree(p->d_adj_scratch), p->used_bytes -= p->adj_scratch_bytes;
    p->d_adj_scratch = nullptr;
    p->adj_scratch_bytes = 0;
    int rc = plan_alloc(p, &p->d_adj_scratch, need);
    if (rc) return rc;
    p->adj_scratch_bytes = need;
  }
  char* base = (char*)p->d_adj_scratch;
  AdjTerm* d_terms = (AdjTerm*)base;
  int* d_trip = (int*)(base + off_trip);
  double* d_sum = (double*)(base + off_sum);
  if (!terms.empty())
    AAR_CUDA_TRY(p, cudaMemcpyAsync(d_terms, terms.data(), sizeof(AdjTerm) * terms.size(), cudaMemcpyHostToDevice, st));
  AAR_CUDA_TRY(p, cudaMemcpyAsync(d_trip, trip.data(), sizeof(int) * trip.size(), cudaMemcpyHostToDevice, st));
  AAR_CUDA_TRY(p, cudaMemsetAsync(d_sum, 0, sizeof(double) * ntrip, st));
  const int64_t n = (int64_t)p->N * p->N * p->N;
  const size_t smem = sizeof(double) * ntrip + sizeof(float) * 3 * M * kLd;
  if (smem > 200 * 1024) return set_err(p, "too many modes for the adjoint products"), AAR_ERR_ARG;
  AAR_CUDA_TRY(p, cudaFuncSetAttribute(k_products_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t chunks = (n + kChunk - 1) / kChunk;
  const int64_t grid = std::min<int64_t>(chunks, (int64_t)p->num_sms * 8);
  k_products_adj<<<(unsigned)grid, kChunk, smem, st>>>(f, gg, gf, M, n, d_terms, (int)terms.size(), d_trip, ntrip,
                                                       d_sum);
  AAR_CUDA_TRY(p, cudaGetLastError());
  // coefficient gradient: sorted triples at [p][q][r]; the counter-terms
  // (+alpha111 on f0 f1 -> g2, -alpha111 on f0 f2 -> g1, present when
  // alpha012 != 0) add G(0,1,2) - G(0,2,1) to alpha111
  std::vector<double> sums(ntrip), g((size_t)M * M * M, 0.0);
  AAR_CUDA_TRY(p, cudaMemcpyAsync(sums.data(), d_sum, sizeof(double) * ntrip, cudaMemcpyDeviceToHost, st));
  AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
  for (int k = 0; k < nsorted; ++k) g[((size_t)trip[3 * k] * M + trip[3 * k + 1]) * M + trip[3 * k + 2]] = sums[k];
  if (M > 2 && p->alpha[(size_t)0 * M * M + 1 * M + 2] != 0) {
    int k012 = -1;
    for (int k = 0; k < nsorted; ++k)
      if (trip[3 * k] == 0 && trip[3 * k + 1] == 1 && trip[3 * k + 2] == 2) k012 = k;
    g[(size_t)1 * M * M + 1 * M + 1] += sums[k012] - sums[nsorted];
  }
  AAR_CUDA_TRY(p, cudaMemcpyAsync(galpha, g.data(), sizeof(double) * g.size(), cudaMemcpyHostToDevice, st));
  AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
  p->last_launches = 1;
  return AAR_OK;
}

}  // namespace aar
