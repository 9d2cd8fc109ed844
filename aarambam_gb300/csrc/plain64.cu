// Plain FP64 forms of the IC path: cuFFT Z2D / D2Z (in place, FFTW's padded
// layout [N][N][2(N/2+1)]) and separate pointwise kernels.
//
// AAR_PLAIN_FP64 keeps the loop structure of the reference 1:1
// (Aarambam/LPT/Basis/main.c:564-1516): one c2r per first index, c2r +
// product + r2c + accumulate per active pair, the 10 counter-term pair
// transforms, the four potential round-trip transforms, 6 + 1 + 6 transforms
// for 2LPT -- M + 2P + 41 in all.
//
// AAR_PLAIN_FP64_REGROUPED is the same arithmetic in FP64 with the modal sum
// regrouped exactly by linearity of the DFT, as the fused form does it:
// M filtered c2r f_p, then per active r the real-space product
// g_r = sum_{p<=q} a'_{pqr} f_p f_q (a' = alpha plus the counter-terms of
// main.c:1045-1050), one r2c and acc += rho_r g_r; then phi += Fnl acc / N^3
// without the potential round trips (main.c:1094-1150 are identities up to
// rounding when the potential is not saved) -- at most 2M + 13 transforms.
// It separates the gain of the regrouping from that of FP32 and fusion.
//
// cuFFT leaves the result of a Z2D on a half spectrum whose kz = 0 / N/2
// planes are not Hermitian undefined, while FFTW's rfftwnd drops the parts
// that break the symmetry; every Z2D here is preceded by the explicit
// projection X(k) <- (X(k) + conj X(-k)) / 2 on those two planes.
// The radial filters are FP64 tables per |k|^2 (index n^2 = i^2 + j^2 + k^2)
// evaluated on the host with the reference's formulas.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "aar_internal.cuh"

namespace aar {

struct PlainState {
  int N = 0, H = 0, M = 0;
  size_t nc = 0;                 // complex entries per field
  int nf = 0;                    // fields: 10 (reference structure) or max(10, M + 3) (regrouped)
  double2* f[kMaxModes + 3] = {};
  double2* disp[6] = {};         // after a run: ZA x, y, z and 2LPT x, y, z (real, padded rows)
  double* qin = nullptr;         // [M][nsq] field filters
  double* qout = nullptr;        // [M][nsq] radial parts rho_n
  double* twb = nullptr;         // [nsq] T(k) / (Dplus Beta)
  double* sinc = nullptr;        // [N] sin(x)/x of the CIC window per index
  cufftHandle z2d = 0, d2z = 0;
  bool plans = false;
  int64_t nsq = 0;
  size_t bytes = 0;              // device bytes allocated for this state (plan_alloc)
};

struct PArgs {
  Grid g;
  int N, H;
  int64_t nsq;
};

__device__ __forceinline__ void cell_of(int64_t c, int N, int H, int& i, int& j, int& k) {
  k = (int)(c % H);
  int64_t q = c / H;
  j = (int)(q % N);
  i = (int)(q / N);
}

// out = keep ? qin[n][n2] * phi : 0    (main.c:572-638, :666-731)
__global__ void kp_filter(PArgs a, const double* __restrict__ q, const double2* __restrict__ phi, double2* out) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)a.N * a.N * a.H) return;
  int i, j, k;
  cell_of(c, a.N, a.H, i, j, k);
  int kx = sidx(i, a.N), ky = sidx(j, a.N), kz = sidx(k, a.N);
  int n2 = kx * kx + ky * ky + kz * kz;
  double2 v = make_double2(0.0, 0.0);
  if (n2 != 0 && keep_cell(a.g, kx, ky, kz)) {
    double f = q[n2];
    double2 p = phi[c];
    v = make_double2(f * p.x, f * p.y);
  }
  out[c] = v;
}

// Hermitian projection of the kz = 0 and kz = N/2 planes (before a Z2D)
__global__ void kp_herm(PArgs a, double2* x) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t plane = (int64_t)a.N * a.N;
  if (t >= 2 * plane) return;
  int kz = t < plane ? 0 : a.N / 2;
  int64_t ij = t % plane;
  int i = (int)(ij / a.N), j = (int)(ij % a.N);
  int ii = (a.N - i) % a.N, jj = (a.N - j) % a.N;
  int64_t me = ((int64_t)i * a.N + j), pa = ((int64_t)ii * a.N + jj);
  if (me > pa) return;
  double2* p = x + me * a.H + kz;
  double2* q = x + pa * a.H + kz;
  if (me == pa) {
    p->y = 0.0;
    return;
  }
  double2 u = *p, v = *q;
  double2 r = make_double2(0.5 * (u.x + v.x), 0.5 * (u.y - v.y));
  *p = r;
  *q = make_double2(r.x, -r.y);
}

// g (=|+=) sum_t c_t f_{p_t} f_{q_t} on the padded real layout: the products
// of one output slot r of the regrouped modal sum (terms in chunks)
constexpr int kProdChunk = 48;
struct PTerms {
  int n;
  const double* fp[kProdChunk];
  const double* fq[kProdChunk];
  double c[kProdChunk];
};
__global__ void kp_products(PArgs a, PTerms t, double* g, int accumulate) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n3 = (int64_t)a.N * a.N * a.N;
  if (c >= n3) return;
  int64_t idx = (c / a.N) * 2 * a.H + c % a.N;
  double v = accumulate ? g[idx] : 0.0;
  for (int i = 0; i < t.n; ++i) v += t.c[i] * t.fp[i][idx] * t.fq[i][idx];
  g[idx] = v;
}

// phi <- phi + fnl acc / n3, DC = 0: the combination of main.c:1104-1126
// without the potential round trips
__global__ void kp_combine_regrouped(PArgs a, double2* phi, const double2* __restrict__ acc, double fnl, double n3) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)a.N * a.N * a.H) return;
  double2 p = phi[c], q = acc[c];
  p.x = p.x + fnl * q.x / n3;
  p.y = p.y + fnl * q.y / n3;
  if (c == 0) p = make_double2(0.0, 0.0);
  phi[c] = p;
}

// real [N][N][N] <- padded real rows [N][N][2H] (copy of a displacement field)
__global__ void kp_unpad(PArgs a, const double* __restrict__ in, double* out) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n3 = (int64_t)a.N * a.N * a.N;
  if (c >= n3) return;
  out[c] = in[(c / a.N) * 2 * a.H + c % a.N];
}

// real product fj <- fi * fj on the padded real layout (main.c:768-776)
__global__ void kp_mul(PArgs a, const double* __restrict__ fi, double* fj) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n3 = (int64_t)a.N * a.N * a.N;
  if (c >= n3) return;
  int64_t row = c / a.N, z = c % a.N;
  int64_t idx = row * 2 * a.H + z;
  fj[idx] = fi[idx] * fj[idx];
}

struct Coef {
  double c[32];
};

// acc += (sum_n w[n] qout[n][n2]) * g    (main.c:785-870, :1008-1058)
__global__ void kp_acc(PArgs a, Coef w, int n0, int n1, const double* __restrict__ qout, const double2* __restrict__ g,
                       double2* acc) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)a.N * a.N * a.H) return;
  int i, j, k;
  cell_of(c, a.N, a.H, i, j, k);
  int kx = sidx(i, a.N), ky = sidx(j, a.N), kz = sidx(k, a.N);
  int n2 = kx * kx + ky * ky + kz * kz;
  if (n2 == 0 || !keep_cell(a.g, kx, ky, kz)) return;
  double f = 0;
  for (int n = n0; n < n1; ++n)
    if (w.c[n] != 0) f += w.c[n] * qout[(int64_t)n * a.nsq + n2];
  double2 v = g[c], s = acc[c];
  acc[c] = make_double2(s.x + f * v.x, s.y + f * v.y);
}

__global__ void kp_scale(PArgs a, double2* x, double s) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)a.N * a.N * a.H) return;
  double2 v = x[c];
  x[c] = make_double2(v.x * s, v.y * s);
}

// phi <- phi / n3 + fnl acc / n3, DC = 0   (main.c:1104-1126)
__global__ void kp_combine(PArgs a, double2* phi, const double2* __restrict__ acc, double fnl, double n3) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)a.N * a.N * a.H) return;
  double2 p = phi[c], q = acc[c];
  p.x = p.x / n3 + fnl * q.x / n3;
  p.y = p.y / n3 + fnl * q.y / n3;
  if (c == 0) p = make_double2(0.0, 0.0);
  phi[c] = p;
}

// Hessians of the ZA displacement (main.c:1180-1277): d_ab = -k_a k_b twb phi
__global__ void kp_hess(PArgs a, double kF, const double* __restrict__ twb, const double2* __restrict__ phi,
                        double2* d0, double2* d1, double2* d2, double2* d3, double2* d4, double2* d5) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)a.N * a.N * a.H) return;
  int i, j, k;
  cell_of(c, a.N, a.H, i, j, k);
  int kv[3] = {sidx(i, a.N), sidx(j, a.N), sidx(k, a.N)};
  int n2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
  double t = twb[n2];
  double2 p = phi[c];
  double k0 = kF * kv[0], k1 = kF * kv[1], k2 = kF * kv[2];
  double2* out[6] = {d0, d1, d2, d3, d4, d5};
  double ka[6] = {k0, k0, k0, k1, k1, k2}, kb[6] = {k0, k1, k2, k1, k2, k2};
  for (int g = 0; g < 6; ++g) {
    double f = -ka[g] * kb[g] * t;
    out[g][c] = make_double2(f * p.x, f * p.y);
  }
}

// 2LPT source in place in d3 (main.c:1284-1294)
__global__ void kp_source(PArgs a, const double* d0, const double* d1, const double* d2, double* d3, const double* d4,
                          const double* d5) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n3 = (int64_t)a.N * a.N * a.N;
  if (c >= n3) return;
  int64_t idx = (c / a.N) * 2 * a.H + c % a.N;
  d3[idx] = d0[idx] * (d3[idx] + d5[idx]) + d3[idx] * d5[idx] - d1[idx] * d1[idx] - d2[idx] * d2[idx] -
            d4[idx] * d4[idx];
}

// ZA and 2LPT displacement spectra with the CIC deconvolution (main.c:1180-1216, 1311-1368)
__global__ void kp_disp(PArgs a, double kF, const double* __restrict__ twb, const double* __restrict__ sinc,
                        const double2* __restrict__ phi, const double2* __restrict__ S, double2* z0, double2* z1,
                        double2* z2, double2* s0, double2* s1, double2* s2) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)a.N * a.N * a.H) return;
  int i, j, k;
  cell_of(c, a.N, a.H, i, j, k);
  int kv[3] = {sidx(i, a.N), sidx(j, a.N), sidx(k, a.N)};
  int n2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
  double ff = 1.0 / (sinc[i] * sinc[j] * sinc[k]);
  double smth = ff * ff;
  double t = twb[n2];
  double2 p = phi[c], sv = S[c];
  double k2 = kF * kF * (double)n2;
  double2* za[3] = {z0, z1, z2};
  double2* lp[3] = {s0, s1, s2};
  for (int ax = 0; ax < 3; ++ax) {
    double kk = kF * kv[ax];
    za[ax][c] = make_double2(-kk * t * p.y * smth, kk * t * p.x * smth);
    if (n2 > 0)
      lp[ax][c] = make_double2(sv.y * kk / k2 * smth, -sv.x * kk / k2 * smth);
    else
      lp[ax][c] = make_double2(0.0, 0.0);
  }
}

struct PRead {
  int N, H;
  double box, vp1, vp2, n3f;
};

// read-out (main.c:1440-1516), FP64 arithmetic as the reference
__global__ void kp_readout(PRead a, const double* d0, const double* d1, const double* d2, const double* e0,
                           const double* e1, const double* e2, const float* __restrict__ lagr, int64_t np, float* pos,
                           float* vel) {
  int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= np) return;
  const int N = a.N;
  double pp[3] = {lagr[3 * n], lagr[3 * n + 1], lagr[3 * n + 2]};
  int ii[3], jj[3];
  double fr[3];
  for (int d = 0; d < 3; ++d) {
    double u = pp[d] / a.box * N;
    if (!(u >= 0.0)) u = 0.0;
    if (u > (double)N) u = (double)N;
    int i = (int)u;
    if (i == N) i = N - 1;
    fr[d] = u - i;
    ii[d] = i;
    jj[d] = (i + 1 == N) ? 0 : i + 1;
  }
  double u = fr[0], v = fr[1], w = fr[2];
  double f1 = (1 - u) * (1 - v) * (1 - w), f2 = (1 - u) * (1 - v) * (w), f3 = (1 - u) * (v) * (1 - w),
         f4 = (1 - u) * (v) * (w), f5 = (u) * (1 - v) * (1 - w), f6 = (u) * (1 - v) * (w), f7 = (u) * (v) * (1 - w),
         f8 = (u) * (v) * (w);
  const int64_t rs = 2 * (int64_t)a.H;
  int64_t o000 = ((int64_t)ii[0] * N + ii[1]) * rs, o010 = ((int64_t)ii[0] * N + jj[1]) * rs;
  int64_t o100 = ((int64_t)jj[0] * N + ii[1]) * rs, o110 = ((int64_t)jj[0] * N + jj[1]) * rs;
  int k0 = ii[2], k1 = jj[2];
  const double* D1[3] = {d0, d1, d2};
  const double* D2[3] = {e0, e1, e2};
  for (int ax = 0; ax < 3; ++ax) {
    const double* x = D1[ax];
    const double* y = D2[ax];
    double dis = x[o000 + k0] * f1 + x[o000 + k1] * f2 + x[o010 + k0] * f3 + x[o010 + k1] * f4 + x[o100 + k0] * f5 +
                 x[o100 + k1] * f6 + x[o110 + k0] * f7 + x[o110 + k1] * f8;
    double dis2 = y[o000 + k0] * f1 + y[o000 + k1] * f2 + y[o010 + k0] * f3 + y[o010 + k1] * f4 +
                  y[o100 + k0] * f5 + y[o100 + k1] * f6 + y[o110 + k0] * f7 + y[o110 + k1] * f8;
    dis2 /= a.n3f;
    float ps = (float)((double)(float)pp[ax] + (dis - 3. / 7. * dis2));
    double xw = fmod(fmod((double)ps, a.box) + a.box, a.box);
    pos[3 * n + ax] = (float)xw;
    vel[3 * n + ax] = (float)(dis * a.vp1 - 3. / 7. * dis2 * a.vp2);
  }
}

// ------------------------------------------------------------------ host
static PlainState* st_of(Plan* p) { return (PlainState*)p->plain; }

void plain_free(Plan* p) {
  PlainState* s = st_of(p);
  if (!s) return;
  for (int i = 0; i < s->nf; ++i)
    if (s->f[i]) cudaFree(s->f[i]);
  if (s->qin) cudaFree(s->qin);
  if (s->qout) cudaFree(s->qout);
  if (s->twb) cudaFree(s->twb);
  if (s->sinc) cudaFree(s->sinc);
  if (s->plans) {
    cufftDestroy(s->z2d);
    cufftDestroy(s->d2z);
  }
  p->used_bytes -= s->bytes;
  delete s;
  p->plain = nullptr;
}

double plain_transfer(const Plan* p, double k);  // capi.cu

static double legendre64(int l, double x) {
  if (l == 0) return 1.0;
  double p0 = 1.0, p1 = x;
  for (int n = 2; n <= l; ++n) {
    double p2 = ((2 * n - 1) * x * p1 - (n - 1) * p0) / n;
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

static bool regrouped(const Plan* p) { return p->prm.precision == AAR_PLAIN_FP64_REGROUPED; }

int plain_setup(Plan* p) {
  if (p->plain) return AAR_OK;
  if (!p->have_tables || !p->have_transfer) return set_err(p, "tables and transfer function must be set"), AAR_ERR_STATE;
  PlainState* s = new PlainState();
  p->plain = s;
  int N = p->N;
  s->N = N;
  s->H = N / 2 + 1;
  s->M = p->M;
  s->nc = (size_t)N * N * s->H;
  s->nsq = 3LL * (N / 2) * (N / 2) + 1;
  s->nf = regrouped(p) ? std::max(10, p->M + 3) : 10;
  int rc;
  auto alloc = [&](void** ptr, size_t bytes) {
    int r = plan_alloc(p, ptr, bytes);
    if (r == AAR_OK) s->bytes += bytes;
    return r;
  };
  for (int i = 0; i < s->nf; ++i)
    if ((rc = alloc((void**)&s->f[i], sizeof(double2) * s->nc))) return rc;
  if ((rc = alloc((void**)&s->qin, sizeof(double) * s->nsq * s->M))) return rc;
  if ((rc = alloc((void**)&s->qout, sizeof(double) * s->nsq * s->M))) return rc;
  if ((rc = alloc((void**)&s->twb, sizeof(double) * s->nsq))) return rc;
  if ((rc = alloc((void**)&s->sinc, sizeof(double) * N))) return rc;
  // host tables with the reference's formulas (main.c:580-637, :833-860)
  const double ns = p->prm.primordial_index, box = p->prm.box;
  const double kmin = 2 * kPi / box, kmax = 2 * kPi / box * p->prm.nmax;
  const double sx = (4 - ns) / 3;
  const double kmin_ns = pow(kmin, sx), kmax_ns = pow(kmax, sx);
  const double kF = 2 * kPi / box;
  std::vector<double> qin(s->nsq * s->M), qout(s->nsq * s->M), twb(s->nsq), sinc(N);
  for (int64_t n2 = 0; n2 < s->nsq; ++n2) {
    double k1 = kF * sqrt((double)n2), k2 = k1 * k1;
    double kbar = -1 + 2 * (pow(k1, sx) - kmin_ns) / (kmax_ns - kmin_ns);
    for (int n = 0; n < s->M; ++n) {
      double in, out;
      if (n2 == 0) {
        in = out = 0;
      } else if (n <= 3) {
        out = pow(k1, sx * (n - 3.));
        in = out * pow(k1, 4 - ns);
      } else {
        double d = legendre64(n - 1, kbar) - p->x0[n - 1];
        out = d / k2;
        in = d * pow(k1, 2 - ns);
      }
      qin[(size_t)n * s->nsq + n2] = in;
      qout[(size_t)n * s->nsq + n2] = out;
    }
    twb[n2] = plain_transfer(p, k1) / p->Dplus / p->Beta;
  }
  for (int i = 0; i < N; ++i) {
    double kv = sidx(i, N) * 2 * kPi / box;
    double f = 1;
    if (kv != 0) {
      f = (kv * box / 2) / N;
      f = sin(f) / f;
    }
    sinc[i] = f;
  }
  AAR_CUDA_TRY(p, cudaMemcpy(s->qin, qin.data(), sizeof(double) * qin.size(), cudaMemcpyHostToDevice));
  AAR_CUDA_TRY(p, cudaMemcpy(s->qout, qout.data(), sizeof(double) * qout.size(), cudaMemcpyHostToDevice));
  AAR_CUDA_TRY(p, cudaMemcpy(s->twb, twb.data(), sizeof(double) * twb.size(), cudaMemcpyHostToDevice));
  AAR_CUDA_TRY(p, cudaMemcpy(s->sinc, sinc.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  if (cufftPlan3d(&s->z2d, N, N, N, CUFFT_Z2D) != CUFFT_SUCCESS) return set_err(p, "cufftPlan3d Z2D failed"), AAR_ERR_CUDA;
  if (cufftPlan3d(&s->d2z, N, N, N, CUFFT_D2Z) != CUFFT_SUCCESS) {
    cufftDestroy(s->z2d);
    return set_err(p, "cufftPlan3d D2Z failed"), AAR_ERR_CUDA;
  }
  s->plans = true;
  return AAR_OK;
}

#define PL(name, grid, ...)                                   \
  do {                                                        \
    ProfScope ps_(p, name, st);                               \
    __VA_ARGS__;                                              \
    AAR_CUDA_TRY(p, cudaGetLastError());                      \
    p->last_launches += 1;                                    \
  } while (0)

// Regrouped modal sum (see the top of the file): per active r the sorted
// triples p <= q <= r with alpha != 0 give a f_p f_q; the counter-terms of
// main.c:1045-1050 add -a012 t012 f_0 f_1 to g_2 and +a012 t012 f_0 f_2 to
// g_1 (FP64 coefficients).
struct PlainTerm {
  int p, q;
  double c;
};
static std::vector<std::vector<PlainTerm>> plain_terms(const Plan* p) {
  const int M = p->M;
  auto A = [&](int i, int j, int k) { return p->alpha[((size_t)i * M + j) * M + k]; };
  std::vector<std::vector<PlainTerm>> by_r(M);
  for (int i = 0; i < M; ++i)
    for (int j = i; j < M; ++j)
      for (int k = j; k < M; ++k)
        if (A(i, j, k) != 0) by_r[k].push_back(PlainTerm{i, j, A(i, j, k)});
  if (M > 2 && A(0, 1, 2) != 0) {
    const double c = A(0, 1, 2) * (-A(1, 1, 1) / A(0, 1, 2));
    by_r[2].push_back(PlainTerm{0, 1, -c});
    by_r[1].push_back(PlainTerm{0, 2, c});
  }
  return by_r;
}

int plain_run(Plan* p, const float* d_lagr, int64_t npart, float* d_pos, float* d_vel, cudaStream_t st) {
  int rc = plain_setup(p);
  if (rc) return rc;
  PlainState* s = st_of(p);
  const int N = s->N, M = s->M;
  PArgs a{p->grid, N, s->H, s->nsq};
  const int bs = 256;
  unsigned gc = (unsigned)((s->nc + bs - 1) / bs);
  unsigned gr = (unsigned)(((int64_t)N * N * N + bs - 1) / bs);
  unsigned gh = (unsigned)((2LL * N * N + bs - 1) / bs);
  double2 *phi = s->f[0], *acc = s->f[1], *fi = s->f[2], *fj = s->f[3];
  cufftSetStream(s->z2d, st);
  cufftSetStream(s->d2z, st);
  auto z2d = [&](double2* x) -> int {
    PL("plain_herm", gh, kp_herm<<<gh, bs, 0, st>>>(a, x));
    ProfScope ps_(p, "plain_cufft_z2d", st);
    if (cufftExecZ2D(s->z2d, (cufftDoubleComplex*)x, (cufftDoubleReal*)x) != CUFFT_SUCCESS)
      return set_err(p, "cufftExecZ2D failed"), AAR_ERR_CUDA;
    return AAR_OK;
  };
  auto d2z = [&](double2* x) -> int {
    ProfScope ps_(p, "plain_cufft_d2z", st);
    if (cufftExecD2Z(s->d2z, (cufftDoubleReal*)x, (cufftDoubleComplex*)x) != CUFFT_SUCCESS)
      return set_err(p, "cufftExecD2Z failed"), AAR_ERR_CUDA;
    return AAR_OK;
  };
  // noise
  if ((rc = launch_seedtable(p, (uint32_t)p->prm.seed, p->d_seed, st))) return rc;
  if ((rc = launch_noise_fp64(p, p->d_seed, phi, s->H, st))) return rc;
  AAR_CUDA_TRY(p, cudaMemsetAsync(acc, 0, sizeof(double2) * s->nc, st));
  auto A = [&](int i, int j, int k) { return p->alpha[((size_t)i * M + j) * M + k]; };
  const double n3 = (double)((unsigned)N * (unsigned)N * (unsigned)N);
  if (regrouped(p)) {
    // M filtered c2r f_p into fields 3 .. M+2 (2 holds g_r)
    double2* g = s->f[2];
    double2** fp = s->f + 3;
    for (int m = 0; m < M; ++m) {
      PL("plain_filter", gc, kp_filter<<<gc, bs, 0, st>>>(a, s->qin + (size_t)m * s->nsq, phi, fp[m]));
      if ((rc = z2d(fp[m]))) return rc;
    }
    const auto by_r = plain_terms(p);
    for (int r = 0; r < M; ++r) {
      if (by_r[r].empty()) continue;
      const auto& T = by_r[r];
      for (size_t t0 = 0; t0 < T.size(); t0 += kProdChunk) {
        PTerms pt{};
        pt.n = (int)std::min(T.size() - t0, (size_t)kProdChunk);
        for (int i = 0; i < pt.n; ++i) {
          pt.fp[i] = (const double*)fp[T[t0 + i].p];
          pt.fq[i] = (const double*)fp[T[t0 + i].q];
          pt.c[i] = T[t0 + i].c;
        }
        PL("plain_products", gr, kp_products<<<gr, bs, 0, st>>>(a, pt, (double*)g, t0 > 0));
      }
      if ((rc = d2z(g))) return rc;
      Coef w{};
      w.c[r] = 1.0;
      PL("plain_acc", gc, kp_acc<<<gc, bs, 0, st>>>(a, w, r, r + 1, s->qout, g, acc));
    }
    PL("plain_combine", gc, kp_combine_regrouped<<<gc, bs, 0, st>>>(a, phi, acc, p->prm.fnl, n3));
  } else {
    // pair loop (main.c:564-880)
    for (int ni = 0; ni < M; ++ni) {
      PL("plain_filter", gc, kp_filter<<<gc, bs, 0, st>>>(a, s->qin + (size_t)ni * s->nsq, phi, fi));
      if ((rc = z2d(fi))) return rc;
      for (int nj = ni; nj < M; ++nj) {
        Coef w{};
        bool any = false;
        for (int nk = nj; nk < M; ++nk) {
          w.c[nk] = A(ni, nj, nk);
          any = any || fabs(A(ni, nj, nk)) > 0;
        }
        if (!any) continue;
        PL("plain_filter", gc, kp_filter<<<gc, bs, 0, st>>>(a, s->qin + (size_t)nj * s->nsq, phi, fj));
        if ((rc = z2d(fj))) return rc;
        PL("plain_mul", gr, kp_mul<<<gr, bs, 0, st>>>(a, (const double*)fi, (double*)fj));
        if ((rc = d2z(fj))) return rc;
        PL("plain_acc", gc, kp_acc<<<gc, bs, 0, st>>>(a, w, nj, M, s->qout, fj, acc));
      }
    }
    // counter-terms (main.c:888-1063): all ten pair transforms, weight on (0,1) and (0,2)
    double a012 = M > 2 ? A(0, 1, 2) : 0, t012 = (M > 2 && a012 != 0) ? -A(1, 1, 1) / a012 : 0;
    for (int ni = 0; ni <= 3; ++ni) {
      PL("plain_filter", gc, kp_filter<<<gc, bs, 0, st>>>(a, s->qin + (size_t)ni * s->nsq, phi, fi));
      if ((rc = z2d(fi))) return rc;
      for (int nj = ni; nj <= 3; ++nj) {
        PL("plain_filter", gc, kp_filter<<<gc, bs, 0, st>>>(a, s->qin + (size_t)nj * s->nsq, phi, fj));
        if ((rc = z2d(fj))) return rc;
        PL("plain_mul", gr, kp_mul<<<gr, bs, 0, st>>>(a, (const double*)fi, (double*)fj));
        if ((rc = d2z(fj))) return rc;
        Coef w{};
        if (ni == 0 && nj == 1) w.c[2] = -a012 * t012;
        if (ni == 0 && nj == 2) w.c[1] = a012 * t012;
        PL("plain_acc", gc, kp_acc<<<gc, bs, 0, st>>>(a, w, 0, M, s->qout, fj, acc));
      }
    }
    // combine (main.c:1094-1150): two real-space round trips
    if ((rc = z2d(phi))) return rc;
    if ((rc = d2z(phi))) return rc;
    PL("plain_combine", gc, kp_combine<<<gc, bs, 0, st>>>(a, phi, acc, p->prm.fnl, n3));
    if ((rc = z2d(phi))) return rc;
    if ((rc = d2z(phi))) return rc;
    PL("plain_scale", gc, kp_scale<<<gc, bs, 0, st>>>(a, phi, 1.0 / n3));
  }
  // 2LPT (main.c:1156-1381)
  double kF = 2 * kPi / p->prm.box;
  double2** d = s->f + 4;  // six Hessian fields: f[4..9]
  PL("plain_hess", gc, kp_hess<<<gc, bs, 0, st>>>(a, kF, s->twb, phi, d[0], d[1], d[2], d[3], d[4], d[5]));
  for (int g = 0; g < 6; ++g)
    if ((rc = z2d(d[g]))) return rc;
  PL("plain_source", gr, kp_source<<<gr, bs, 0, st>>>(a, (const double*)d[0], (const double*)d[1],
                                                    (const double*)d[2], (double*)d[3], (const double*)d[4],
                                                    (const double*)d[5]));
  if ((rc = d2z(d[3]))) return rc;
  // ZA spectra into acc, fi, fj; 2LPT spectra into d[0], d[1], d[2] (S stays in d[3])
  PL("plain_disp", gc, kp_disp<<<gc, bs, 0, st>>>(a, kF, s->twb, s->sinc, phi, d[3], acc, fi, fj, d[0], d[1], d[2]));
  double2* za[3] = {acc, fi, fj};
  for (int ax = 0; ax < 3; ++ax) {
    if ((rc = z2d(za[ax]))) return rc;
    if ((rc = z2d(d[ax]))) return rc;
  }
  for (int ax = 0; ax < 3; ++ax) {
    s->disp[ax] = za[ax];
    s->disp[3 + ax] = d[ax];
  }
  if (npart > 0) {
    PRead r{N, s->H, p->prm.box, p->vel_prefac, p->vel_prefac2,
            (double)(float)((unsigned)N * (unsigned)N * (unsigned)N)};
    unsigned gp = (unsigned)((npart + bs - 1) / bs);
    PL("plain_readout", gp, kp_readout<<<gp, bs, 0, st>>>(r, (const double*)acc, (const double*)fi, (const double*)fj,
                                                        (const double*)d[0], (const double*)d[1], (const double*)d[2],
                                                        d_lagr, npart, d_pos, d_vel));
  }
  return AAR_OK;
}

// Displacement field `which` of the last run (0..2 ZA, 3..5 2LPT before its
// 1/N^3) as float64 [N][N][N].
int plain_copy_field(Plan* p, int which, double* out, cudaStream_t st) {
  PlainState* s = st_of(p);
  if (!s || !s->disp[which]) return set_err(p, "no FP64 displacement fields: run the plan first"), AAR_ERR_STATE;
  PArgs a{p->grid, s->N, s->H, s->nsq};
  unsigned gr = (unsigned)(((int64_t)s->N * s->N * s->N + 255) / 256);
  kp_unpad<<<gr, 256, 0, st>>>(a, (const double*)s->disp[which], out);
  AAR_CUDA_TRY(p, cudaGetLastError());
  return AAR_OK;
}

// The potential spectrum of the last run (the total one once a run is
// done), complex float64 [N][N][N/2+1].
int plain_copy_spectrum(Plan* p, void* out, cudaStream_t st) {
  PlainState* s = st_of(p);
  if (!s) return set_err(p, "no FP64 spectrum: run the plan first"), AAR_ERR_STATE;
  AAR_CUDA_TRY(p, cudaMemcpyAsync(out, s->f[0], sizeof(double2) * s->nc, cudaMemcpyDeviceToDevice, st));
  return AAR_OK;
}

}  // namespace aar
