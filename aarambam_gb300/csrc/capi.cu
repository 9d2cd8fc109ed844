// C ABI of libaarambam_gpu.so: plan life cycle, host set-up and the run
// entry points.  Host scalars follow Aarambam/LPT/Basis/power.c:391-448
// (sigma8 normalisation and growth factors, by Romberg integration as in
// nrsrc/qromb.c), power.c:66-153 (transfer table), main.c:305-372.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "aar_internal.cuh"
#include "ranlux.cuh"
#include "spectral.cuh"

struct aar_plan {
  aar::Plan p;
};

namespace aar {

const char* set_err(Plan* p, const std::string& e) {
  p->err = e;
  return p->err.c_str();
}

int host_kcut(int nsample, double box) {
  // largest m with (m*2*PI/Box)*Box/(2*PI) <= Nsample/2 (integer division),
  // evaluated in the reference's operation order (main.c:410-441)
  int half = nsample / 2;
  int m = half + 1;
  while (m >= 0) {
    double kv = (double)(m * 2) * kPi / box;
    if (!(fabs(kv) * box / (2 * kPi) > half)) break;
    --m;
  }
  return m;
}

static cudaEvent_t pool_event(Plan* p) {
  if (!p->event_pool.empty()) {
    cudaEvent_t e = p->event_pool.back();
    p->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(Plan* pl, const char* name, cudaStream_t s) : p(pl), st(s) {
  if (!p->profiling) return;
  Plan::ProfRec r{name, pool_event(p), pool_event(p)};
  cudaEventRecord(r.a, st);
  p->prof.push_back(r);
  idx = (int)p->prof.size() - 1;
}
ProfScope::~ProfScope() {
  if (idx >= 0) cudaEventRecord(p->prof[idx].b, st);
}

// ------------------------------------------------------------ cosmology
struct Cosmo {
  const Plan* p;
  double norm;
  double transfer(double k) const {  // power.c:181-217
    k *= p->kconv;
    double lk = log10(k);
    const std::vector<double>& L = p->logk;
    if (lk < L.front() || lk > L.back()) return 0;
    int lo = 0, hi = (int)L.size() - 1;
    while (hi - lo > 1) {
      int mid = (hi + lo) / 2;
      if (lk < L[mid]) hi = mid;
      else lo = mid;
    }
    double u = (lk - L[lo]) / (L[hi] - L[lo]);
    return pow(10.0, (1 - u) * p->logT[lo] + u * p->logT[hi]);
  }
};

double plain_transfer(const Plan* p, double k) {
  Cosmo c{p, 1.0};
  return c.transfer(k);
}

// Romberg quadrature: trapezoid refinements extrapolated to zero step with
// Neville's algorithm over the last five estimates, relative tolerance 1e-8.
template <class F>
static double romberg(F&& f, double a, double b) {
  const int K = 5, JMAX = 40;
  std::vector<double> h(JMAX + 2), s(JMAX + 2);
  double trap = 0;
  h[1] = 1.0;
  for (int j = 1; j <= JMAX; ++j) {
    if (j == 1) {
      trap = 0.5 * (b - a) * (f(a) + f(b));
    } else {
      long it = 1L << (j - 2);
      double del = (b - a) / (double)it, x = a + 0.5 * del, sum = 0;
      for (long q = 0; q < it; ++q, x += del) sum += f(x);
      trap = 0.5 * (trap + (b - a) * sum / (double)it);
    }
    s[j] = trap;
    if (j >= K) {
      const double* xa = &h[j - K + 1];
      const double* ya = &s[j - K + 1];
      double c[5], d[5];
      int ns = 0;
      double dif = fabs(xa[0]);
      for (int i = 0; i < K; ++i) {
        if (fabs(xa[i]) < dif) {
          ns = i;
          dif = fabs(xa[i]);
        }
        c[i] = d[i] = ya[i];
      }
      double y = ya[ns--], dy = 0;
      for (int m = 1; m < K; ++m) {
        for (int i = 0; i < K - m; ++i) {
          double ho = xa[i], hp = xa[i + m], w = c[i + 1] - d[i], den = w / (ho - hp);
          d[i] = hp * den;
          c[i] = ho * den;
        }
        dy = (2 * (ns + 1) < (K - m)) ? c[ns + 1] : d[ns--];
        y += dy;
      }
      if (fabs(dy) <= 1e-8 * fabs(y)) return y;
    }
    h[j + 1] = 0.25 * h[j];
  }
  return NAN;
}

static double growth(double a, double Om, double OL) {  // power.c:587-598
  double ha = sqrt(Om / (a * a * a) + (1 - Om - OL) / (a * a) + OL);
  return ha * romberg([&](double x) { return pow(x / (Om + (1 - Om - OL) * x + OL * x * x * x), 1.5); }, 0, a);
}

static int set_transfer(Plan* p, const double* k, const double* t, int n) {
  if (n < 2 || !k || !t) return set_err(p, "transfer table needs at least 2 rows"), AAR_ERR_ARG;
  std::vector<std::pair<double, double>> rows(n);
  for (int i = 0; i < n; ++i) {
    if (!(k[i] > 0) || !(t[i] > 0)) return set_err(p, "transfer table needs positive k and T"), AAR_ERR_ARG;
    rows[i] = {log10(k[i]), log10(t[i])};
  }
  std::stable_sort(rows.begin(), rows.end(), [](auto& a, auto& b) { return a.first < b.first; });
  if (rows[0].first >= -4.6)
    return set_err(p, "klower of the transfer table is too large to normalise (first log10 k >= -4.6)"),
           AAR_ERR_TRANSFER;
  for (int i = 1; i < n; ++i)
    if (rows[i].first == rows[i - 1].first)
      return set_err(p, "two transfer rows share one k"), AAR_ERR_TRANSFER_DUP;
  p->logk.resize(n);
  p->logT.resize(n);
  for (int i = 0; i < n; ++i) {
    p->logk[i] = rows[i].first;
    p->logT[i] = rows[i].second - rows[0].second;
  }
  const aar_params& q = p->prm;
  p->kconv = q.input_spectrum_unit_length_in_cm / q.unit_length_in_cm;
  double UnitTime_in_s = q.unit_length_in_cm / q.unit_velocity_in_cm_per_s;
  p->Hubble = 3.2407789e-18 * UnitTime_in_s;
  p->InitTime = 1 / (1 + q.redshift);
  double R8 = 8 * (3.085678e24 / q.unit_length_in_cm);
  Cosmo cz{p, 1.0};
  double res = romberg(
      [&](double kk) {
        double kr = R8 * kk, kr2 = kr * kr, kr3 = kr2 * kr;
        if (kr < 1e-8) return 0.0;
        double w = 3 * (sin(kr) / kr3 - cos(kr) / kr2);
        double T = cz.transfer(kk);
        double P = 1.0 * exp(q.primordial_index * log(kk)) * power_osc(q, kk) * T * T;
        return 4 * kPi * kk * kk * w * w * P;
      },
      0, 500.0 * 1 / R8);
  p->Norm = q.sigma8 * q.sigma8 / res;
  p->Anorm = p->Norm;
  double Om = q.omega, OL = q.omega_lambda;
  p->D0 = growth(1.0, Om, OL) / growth(1.e-8, Om, OL) * 1.e-8;
  p->Dplus = growth(1.0, Om, OL) / growth(p->InitTime, Om, OL);
  double a = p->InitTime;
  double hubble_a = p->Hubble * sqrt(Om / pow(a, 3) + (1 - Om - OL) / pow(a, 2) + OL);
  double om_a = Om / (Om + a * (1 - Om - OL) + a * a * a * OL);
  p->vel_prefac = a * hubble_a * pow(om_a, 0.6) / sqrt(a);
  p->vel_prefac2 = a * hubble_a * (2 * pow(om_a, 4. / 7.)) / sqrt(a);
  p->Beta = 1.5 * Om / (2998. * 2998. / q.unit_length_in_cm / q.unit_length_in_cm * 3.085678e24 * 3.085678e24) /
            p->D0;
  p->have_transfer = true;

  // per-n^2 tables for the FP32 form: noise amplitude and T / (D Beta),
  // rewritten with synchronous copies (ordered only against the legacy
  // stream): runs in flight on other streams finish first
  if (is_fp32(p->prm)) {
    AAR_CUDA_TRY(p, cudaDeviceSynchronize());
    int N = p->N;
    int64_t nsq = 3LL * (N / 2) * (N / 2) + 1;
    std::vector<float> amp(nsq), twb(nsq);
    double kF = 2 * kPi / q.box;
    double fac = pow(2 * kPi / q.box, 1.5);
    for (int64_t n2 = 0; n2 < nsq; ++n2) {
      double km = kF * sqrt((double)n2), k2 = km * km;
      amp[n2] = n2 ? (float)(sqrt(noise_osc(q, p->Anorm * exp(q.primordial_index * log(km)), km)) * fac * p->Beta / k2)
                   : 0.f;
      twb[n2] = (float)(cz.transfer(km) / p->Dplus / p->Beta);
    }
    AAR_CUDA_TRY(p, cudaMemcpy(p->d_amp, amp.data(), sizeof(float) * nsq, cudaMemcpyHostToDevice));
    AAR_CUDA_TRY(p, cudaMemcpy(p->d_twb, twb.data(), sizeof(float) * nsq, cudaMemcpyHostToDevice));
  }
  return AAR_OK;
}

// ------------------------------------------------------------ allocation
int plan_alloc(Plan* p, void** ptr, size_t bytes) {
  if (p->prm.mem_limit_bytes > 0 && p->used_bytes + bytes > (size_t)p->prm.mem_limit_bytes)
    return set_err(p, "plan allocation above mem_limit_bytes"), AAR_ERR_OOM;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return set_err(p, std::string("cudaMalloc: ") + cudaGetErrorString(e)), AAR_ERR_OOM;
  }
  p->used_bytes += bytes;
  return AAR_OK;
}

static void plan_release(Plan* p) {
  for (auto& r : p->prof) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  p->prof.clear();
  for (auto e : p->event_pool) cudaEventDestroy(e);
  p->event_pool.clear();
  void* ptrs[] = {p->d_phik, p->d_work, p->d_seed, p->d_twN, p->d_twH, p->d_amp, p->d_twb, p->d_rlxpow, p->d_terms, p->d_io, p->d_qtab, p->d_rtab, p->d_sinc, p->d_isinc2, p->d_adj_scratch, p->d_qcube};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  p->d_phik = p->d_work = nullptr;
  p->d_seed = nullptr;
  p->d_twN = p->d_twH = nullptr;
  p->d_amp = p->d_twb = nullptr;
  p->d_rlxpow = p->d_terms = nullptr;
  p->d_qtab = p->d_rtab = nullptr;
  p->d_sinc = p->d_isinc2 = nullptr;
  p->d_qcube = nullptr;
  p->qcube_m = 0;
  p->qcube_stale = true;
  p->d_io = nullptr;
  p->io_cap = 0;
  p->d_adj_scratch = nullptr;
  p->adj_scratch_bytes = 0;
  jit_free(p);
  if (p->copy_stream) cudaStreamDestroy(p->copy_stream);
  if (p->copy_done) cudaEventDestroy(p->copy_done);
  if (p->copy_start) cudaEventDestroy(p->copy_start);
  p->copy_stream = nullptr;
  p->copy_done = p->copy_start = nullptr;
  for (int i = 0; i < 2; ++i) {
    if (p->out_stream[i]) cudaStreamDestroy(p->out_stream[i]);
    if (p->out_done[i]) cudaEventDestroy(p->out_done[i]);
    p->out_stream[i] = nullptr;
    p->out_done[i] = nullptr;
  }
  for (int i = 0; i < Plan::kOutChunks; ++i) {
    if (p->chunk_read[i]) cudaEventDestroy(p->chunk_read[i]);
    p->chunk_read[i] = nullptr;
  }
  for (int i = 0; i < Plan::kGlassChunks; ++i) {
    if (p->gchunk_read[i]) cudaEventDestroy(p->gchunk_read[i]);
    if (p->gchunk_free[i]) cudaEventDestroy(p->gchunk_free[i]);
    p->gchunk_read[i] = p->gchunk_free[i] = nullptr;
  }
  if (p->d_glass) cudaFree(p->d_glass);
  if (p->d_gout) cudaFree(p->d_gout);
  if (p->d_gscale) cudaFree(p->d_gscale);
  p->d_gscale = nullptr;
  p->gscale_cap = 0;
  p->d_glass = nullptr;
  p->d_gout = nullptr;
  p->glass_cap = p->gout_cap = 0;
  plain_free(p);
  slab_free(p);
}

static bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Work fields: the path needs max(M, 8) (2LPT: six Hessians, the source and
// T/(D Beta) phi); the standalone transforms (M = 0) need one.
static int alloc_fused(Plan* p, int M) {
  int N = p->N;
  size_t fbytes = sizeof(float2) * (size_t)N * N * p->HP;
  int nwork = M == 0 ? 1 : std::max(M, 9);  // the 2LPT schedule uses slots 0..8
  if (p->d_work && p->nwork >= nwork) return AAR_OK;
  if (p->d_work) {
    cudaFree(p->d_work);
    p->used_bytes -= fbytes * p->nwork;
    p->d_work = nullptr;
  }
  int rc = plan_alloc(p, (void**)&p->d_work, fbytes * nwork);
  if (rc) return rc;
  p->nwork = nwork;
  return AAR_OK;
}

// Per-|k|^2 tables of the mode functions, FP64 on the host with the
// reference's formulas, stored as float:
//   q_n (field filter, main.c:580-637):   k^{s(n-3)} k^{4-ns}           (n <= 3)
//                                         (P_{n-1}(kbar) - X0[n-1]) k^{2-ns}
//   rho_n (radial part, main.c:833-860):  k^{s(n-3)} (n <= 3),  (P_{n-1}(kbar) - X0[n-1]) / k^2
// with s = (4-ns)/3, kbar = -1 + 2 (k^s - kmin^s)/(kmax^s - kmin^s).
// q is stored per mode ([M][nsq]: a filter pass reads one mode); rho per
// |k|^2 ([nsq][rtab_stride], mode fastest: the accumulation reads every mode
// of one cell, a few sectors instead of one per mode).
static int mode_tables(Plan* p) {
  int N = p->N, M = p->M;
  int64_t nsq = 3LL * (N / 2) * (N / 2) + 1;
  if (p->d_qtab && p->nsq == nsq && p->qtab_m >= M) {
    // reuse the allocation
  } else {
    if (p->d_qtab) cudaFree(p->d_qtab), p->used_bytes -= sizeof(float) * p->nsq * p->qtab_m;
    if (p->d_rtab) cudaFree(p->d_rtab), p->used_bytes -= sizeof(float) * p->nsq * p->rtab_stride;
    p->d_qtab = p->d_rtab = nullptr;
    int rc;
    if ((rc = plan_alloc(p, (void**)&p->d_qtab, sizeof(float) * nsq * M))) return rc;
    p->rtab_stride = (M + 3) / 4 * 4;
    if ((rc = plan_alloc(p, (void**)&p->d_rtab, sizeof(float) * nsq * p->rtab_stride))) return rc;
    p->qtab_m = M;
  }
  p->nsq = nsq;
  const double ns = p->prm.primordial_index, box = p->prm.box;
  const double kmin = 2 * kPi / box, kmax = 2 * kPi / box * p->prm.nmax;
  const double sx = (4 - ns) / 3, kmin_ns = pow(kmin, sx), kmax_ns = pow(kmax, sx);
  const double kF = 2 * kPi / box;
  const int rs = p->rtab_stride;
  std::vector<float> qt((size_t)nsq * M), rt((size_t)nsq * rs, 0.f);
  std::vector<double> P(std::max(M, 2));
  for (int64_t n2 = 1; n2 < nsq; ++n2) {
    double k1 = kF * sqrt((double)n2), k2 = k1 * k1;
    double kbar = -1 + 2 * (pow(k1, sx) - kmin_ns) / (kmax_ns - kmin_ns);
    double pin = pow(k1, 4 - ns), p2n = pow(k1, 2 - ns);
    // P_l(kbar), l < M, by the Bonnet recurrence
    P[0] = 1;
    if (M > 1) P[1] = kbar;
    for (int l = 2; l < M; ++l) P[l] = ((2 * l - 1) * kbar * P[l - 1] - (l - 1) * P[l - 2]) / l;
    for (int n = 0; n < M; ++n) {
      double in, out;
      if (n <= 3) {
        out = pow(k1, sx * (n - 3.));
        in = out * pin;
      } else {
        double d = P[n - 1] - p->x0[n - 1];
        out = d / k2;
        in = d * p2n;
      }
      qt[(size_t)n * nsq + n2] = (float)in;
      rt[(size_t)n2 * rs + n] = (float)out;
    }
  }
  for (int n = 0; n < M; ++n) qt[(size_t)n * nsq] = 0.f;
  AAR_CUDA_TRY(p, cudaMemcpy(p->d_qtab, qt.data(), sizeof(float) * qt.size(), cudaMemcpyHostToDevice));
  AAR_CUDA_TRY(p, cudaMemcpy(p->d_rtab, rt.data(), sizeof(float) * rt.size(), cudaMemcpyHostToDevice));
  return AAR_OK;
}

static int create(Plan* p) {
  const aar_params& q = p->prm;
  int N = q.nmesh;
  if (q.nsample > q.nmax) return set_err(p, "Nmax must be >= Nsample (main.c:200)"), AAR_ERR_NMAX;
  if (!is_fp32(q) && !is_plain(q)) return set_err(p, "unknown precision"), AAR_ERR_ARG;
  if (q.precision == AAR_FUSED_FP32 && !(pow2(N) && N >= 16 && N <= 1024))
    return set_err(p, "fused FP32 form supports Nmesh = 16..1024, powers of two"), AAR_ERR_ARG;
  if (is_plain(q) && !(N >= 4 && N % 2 == 0 && N <= 2048))
    return set_err(p, "plain FP64 form supports even Nmesh up to 2048"), AAR_ERR_ARG;
  if (q.precision == AAR_SLAB_FP32) {
    std::string why;
    if (slab_check(q, why)) return set_err(p, why), AAR_ERR_ARG;
  }
  if (!(q.box > 0) || q.nsample <= 0) return set_err(p, "Box and Nsample must be positive"), AAR_ERR_ARG;
  if (q.seed < 0) return set_err(p, "Seed must be >= 0"), AAR_ERR_ARG;
  if (q.variant == AAR_VARIANT_BASIS) {
    if (q.which_spectrum != 0)
      return set_err(p, "2LPTBasis: only WhichSpectrum 0 (the tabulated transfer function) is supported"), AAR_ERR_ARG;
  } else if (q.variant == AAR_VARIANT_RESBASIS) {
    if (q.which_spectrum < 0 || q.which_spectrum > 2)
      return set_err(p, "2LPTResBasis: WhichSpectrum must be 0, 1 or 2"), AAR_ERR_ARG;
  } else {
    return set_err(p, "unknown variant"), AAR_ERR_ARG;
  }
  AAR_CUDA_TRY(p, cudaGetDevice(&p->dev));
  AAR_CUDA_TRY(p, cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->dev));
  if (const char* g = getenv("AAR_XPASS_GROUP")) p->xpass_group = std::max(1LL, atoll(g));
  if (const char* g = getenv("AAR_NOISE_ONE_DRAW")) p->noise_one_draw = atoi(g) == 1;
  if (const char* g = getenv("AAR_OUT_CHUNKS")) p->out_chunks = std::min(std::max(1, atoi(g)), (int)Plan::kOutChunks);
  p->N = N;
  p->HP = ((N / 2 + 1) + 7) / 8 * 8;
  p->grid.N = N;
  p->grid.HP = p->HP;
  p->grid.kcut = host_kcut(q.nsample, q.box);
  p->grid.sphere = q.sphere_mode == 1;
  p->grid.nsq_bnd = (q.nsample / 2) * (q.nsample / 2);
  p->grid.nsample_half = q.nsample / 2;
  p->grid.box = q.box;
  p->grid.kF = (float)(2 * kPi / q.box);

  int rc;
  if ((rc = plan_alloc(p, (void**)&p->d_seed, sizeof(uint32_t) * (size_t)N * N))) return rc;
  // ranlux skip-ahead: seed-table threads own rlx_seg refills; powers
  // (b^{-202 rlx_seg})^{2^i} mod m, i < 32
  p->rlx_seg = 8;
  {
    std::vector<U576> pw(32);
    U576 a = modpow576(u576_binv(), (uint64_t)kRlxLux * p->rlx_seg);
    for (int i = 0; i < 32; ++i) {
      pw[i] = a;
      a = modmul576(a, a);
    }
    if ((rc = plan_alloc(p, &p->d_rlxpow, sizeof(U576) * 32))) return rc;
    AAR_CUDA_TRY(p, cudaMemcpy(p->d_rlxpow, pw.data(), sizeof(U576) * 32, cudaMemcpyHostToDevice));
  }
  if (is_fp32(q)) {
    std::vector<float2> twN(N), twH(N / 2);
    for (int m = 0; m < N; ++m) {
      long double ang = -2.0L * 3.141592653589793238462643383279502884L * m / N;
      twN[m] = make_float2((float)cosl(ang), (float)sinl(ang));
    }
    for (int m = 0; m < N / 2; ++m) twH[m] = twN[2 * m];
    if ((rc = plan_alloc(p, (void**)&p->d_twN, sizeof(float2) * N))) return rc;
    if ((rc = plan_alloc(p, (void**)&p->d_twH, sizeof(float2) * (N / 2)))) return rc;
    AAR_CUDA_TRY(p, cudaMemcpy(p->d_twN, twN.data(), sizeof(float2) * N, cudaMemcpyHostToDevice));
    AAR_CUDA_TRY(p, cudaMemcpy(p->d_twH, twH.data(), sizeof(float2) * (N / 2), cudaMemcpyHostToDevice));
    int64_t nsq = 3LL * (N / 2) * (N / 2) + 1;
    if ((rc = plan_alloc(p, (void**)&p->d_amp, sizeof(float) * nsq))) return rc;
    if ((rc = plan_alloc(p, (void**)&p->d_twb, sizeof(float) * nsq))) return rc;
    // CIC window per grid index, the reference's expression (main.c:1334-1349)
    std::vector<float> sinc(N);
    for (int i = 0; i < N; ++i) {
      double kv = sidx(i, N) * 2 * kPi / q.box, f = 1;
      if (kv != 0) {
        f = (kv * q.box / 2) / N;
        f = sin(f) / f;
      }
      sinc[i] = (float)f;
    }
    if ((rc = plan_alloc(p, (void**)&p->d_sinc, sizeof(float) * N))) return rc;
    AAR_CUDA_TRY(p, cudaMemcpy(p->d_sinc, sinc.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    // its inverse square, the per-axis CIC deconvolution factor of the
    // separable 2LPT passes
    std::vector<float> is2(N);
    for (int i = 0; i < N; ++i) {
      double kv = sidx(i, N) * 2 * kPi / q.box, f = 1;
      if (kv != 0) {
        f = (kv * q.box / 2) / N;
        f = sin(f) / f;
      }
      is2[i] = (float)(1.0 / (f * f));
    }
    if ((rc = plan_alloc(p, (void**)&p->d_isinc2, sizeof(float) * N))) return rc;
    AAR_CUDA_TRY(p, cudaMemcpy(p->d_isinc2, is2.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
  }
  return AAR_OK;
}

static cudaStream_t S(void* s) { return (cudaStream_t)s; }

static int ready_tables(Plan* p) {
  if (!p->have_tables) return set_err(p, "coefficient tables not set"), AAR_ERR_STATE;
  if (!p->have_transfer) return set_err(p, "transfer function not set"), AAR_ERR_STATE;
  return AAR_OK;
}

// The fused form's fields (the potential spectrum and max(M, 9) work
// fields) are allocated on first use -- the first run, stage or
// aar_plan_prepare -- not when the plan is made or its tables are set, so a
// plan holds no field memory until it computes.
static int ensure_fields(Plan* p) {
  if (p->prm.precision == AAR_SLAB_FP32) return slab_setup(p);
  if (p->prm.precision != AAR_FUSED_FP32) return AAR_OK;
  if (!p->d_phik) {
    int rc = plan_alloc(p, (void**)&p->d_phik, sizeof(float2) * (size_t)p->N * p->N * p->HP);
    if (rc) return rc;
  }
  int rc = alloc_fused(p, p->M);
  if (rc) return rc;
  return qcube_build(p);
}

static int ready(Plan* p) {
  int rc = ready_tables(p);
  if (rc) return rc;
  return ensure_fields(p);
}

static int run_noise(Plan* p, cudaStream_t st) {
  int rc = launch_seedtable(p, (uint32_t)p->prm.seed, p->d_seed, st);
  if (rc) return rc;
  return launch_noise_fp32(p, p->d_seed, p->d_phik, st);
}

// The FP32 forms' field stages: noise, the modal sum and 2LPT, up to the six
// displacement fields (rows = false: the fused form stops before its
// displacement rows, which the lattice read-out then fuses).  The slab form
// always leaves the real fields.
static int field_stages(Plan* p, cudaStream_t st, bool rows = true) {
  int rc = run_noise(p, st);
  if (rc) return rc;
  if (p->prm.precision == AAR_SLAB_FP32) return slab_run(p, st);
  if ((rc = fused_modal(p, st))) return rc;
  return fused_lpt(p, st, rows);
}

}  // namespace aar

using namespace aar;

extern "C" {

int aar_version(void) { return 1; }

int aar_plan_create(const aar_params* prm, aar_plan** out) {
  if (!prm || !out) return AAR_ERR_ARG;
  *out = nullptr;
  aar_plan* h = new (std::nothrow) aar_plan();
  if (!h) return AAR_ERR_OOM;
  h->p.prm = *prm;
  int rc = create(&h->p);
  if (rc) {
    // keep the plan so the caller can read the message, but free device memory
    plan_release(&h->p);
    *out = h;
    return rc;
  }
  *out = h;
  return AAR_OK;
}

void aar_plan_destroy(aar_plan* h) {
  if (!h) return;
  plan_release(&h->p);
  delete h;
}

const char* aar_last_error(const aar_plan* h) { return h ? h->p.err.c_str() : "null plan"; }

int aar_last_launch_count(const aar_plan* h) { return h ? h->p.last_launches : 0; }

int64_t aar_plan_device_bytes(const aar_plan* h) { return h ? (int64_t)h->p.used_bytes : 0; }

int aar_set_tables(aar_plan* h, const double* alpha, const double* x0, int32_t M) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  if (M < 1 || M > 32 || !alpha || !x0) return set_err(p, "N_modes must be 1..32 with non-null tables"), AAR_ERR_ARG;
  size_t n3 = (size_t)M * M * M;
  for (size_t i = 0; i < n3; ++i)
    if (!isfinite(alpha[i])) return set_err(p, "non-finite alpha coefficient"), AAR_ERR_ARG;
  for (int i = 0; i < M; ++i)
    if (!isfinite(x0[i])) return set_err(p, "non-finite X0 coefficient"), AAR_ERR_ARG;
  ++p->generation;
  // the term list and the NVRTC module's coefficients are rewritten below
  // with synchronous copies that are ordered only against the legacy stream:
  // wait for runs still in flight on other streams (or in batch graphs)
  AAR_CUDA_TRY(p, cudaDeviceSynchronize());
  p->alpha.assign(alpha, alpha + n3);
  p->x0.assign(x0, x0 + M);
  p->M = M;
  plain_free(p);  // plain-form tables are rebuilt on the next run
  int rc;
  if (p->prm.precision == AAR_SLAB_FP32) {
    if (!p->d_terms && (rc = plan_alloc(p, &p->d_terms, terms_bytes()))) return rc;
    if ((rc = build_term_list(p))) return rc;
  }
  if (p->prm.precision == AAR_FUSED_FP32) {
    p->qcube_stale = true;  // rebuilt on first use (ensure_fields)
    if ((rc = mode_tables(p))) return rc;
    if (!p->d_terms && (rc = plan_alloc(p, &p->d_terms, terms_bytes()))) return rc;
    if ((rc = fused_prepare(p))) return rc;
    if ((rc = fused_configure_xform(p))) return rc;
  }
  p->have_tables = true;
  return AAR_OK;
}

int aar_plan_prepare(aar_plan* h) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  if (is_plain(p->prm)) return plain_setup(p);
  return AAR_OK;  // the fused form allocates its fields with the tables
}

int aar_set_transfer(aar_plan* h, const double* k, const double* t, int32_t n) {
  if (!h) return AAR_ERR_ARG;
  ++h->p.generation;
  plain_free(&h->p);
  return set_transfer(&h->p, k, t, n);
}

int aar_get_scalars(const aar_plan* h, aar_scalars* o) {
  if (!h || !o) return AAR_ERR_ARG;
  const Plan* p = &h->p;
  *o = aar_scalars{p->Norm, p->Anorm, p->D0, p->Dplus, p->InitTime, p->Hubble, p->Beta, p->vel_prefac, p->vel_prefac2};
  return AAR_OK;
}

int aar_set_seed(aar_plan* h, int32_t seed) {
  if (!h) return AAR_ERR_ARG;
  if (seed < 0) return set_err(&h->p, "Seed must be >= 0"), AAR_ERR_ARG;
  h->p.prm.seed = seed;
  ++h->p.generation;
  return AAR_OK;
}

int aar_seedtable(aar_plan* h, uint32_t* d_out, void* stream) {
  if (!h || !d_out) return AAR_ERR_ARG;
  h->p.last_launches = 0;
  return launch_seedtable(&h->p, (uint32_t)h->p.prm.seed, d_out, S(stream));
}

int aar_stage_noise(aar_plan* h, void* stream) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  p->last_launches = 0;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "stage calls are for the fused form"), AAR_ERR_ARG;
  return run_noise(p, S(stream));
}

int aar_stage_modal(aar_plan* h, void* stream) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  p->last_launches = 0;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "stage calls are for the fused form"), AAR_ERR_ARG;
  return fused_modal(p, S(stream));
}

int aar_stage_lpt(aar_plan* h, void* stream) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  p->last_launches = 0;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "stage calls are for the fused form"), AAR_ERR_ARG;
  return fused_lpt(p, S(stream));
}

int aar_stage_readout(aar_plan* h, const float* d_lagr, int64_t npart, float* d_pos, float* d_vel, void* stream) {
  if (!h || npart < 0 || (npart > 0 && (!d_lagr || !d_pos || !d_vel))) return AAR_ERR_ARG;
  Plan* p = &h->p;
  p->last_launches = 0;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "stage calls are for the fused form"), AAR_ERR_ARG;
  if (!p->d_work || p->nwork < 6 || !p->disp_real)
    return set_err(p, "no displacement fields: run the field stages first"), AAR_ERR_STATE;
  return fused_readout(p, d_lagr, npart, d_pos, d_vel, S(stream));
}

int aar_stage_readout_glass(aar_plan* h, const float* d_glass, int64_t nglass, double glass_box, int32_t tile,
                            float* d_pos, float* d_vel, int32_t* d_ids, void* stream) {
  if (!h || nglass < 0 || tile < 1 || !(glass_box > 0)) return AAR_ERR_ARG;
  Plan* p = &h->p;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "stage calls are for the fused form"), AAR_ERR_ARG;
  if (!p->d_work || p->nwork < 6 || !p->disp_real)
    return set_err(p, "no displacement fields: run the field stages first"), AAR_ERR_STATE;
  p->last_launches = 0;
  int rc = glass_prepare(p, d_glass, nglass, glass_box, tile, S(stream));
  if (rc) return rc;
  return fused_readout_glass(p, nglass, tile, d_pos, d_vel, d_ids, S(stream));
}

int aar_run(aar_plan* h, const float* d_lagr, int64_t npart, float* d_pos, float* d_vel, void* stream) {
  if (!h || npart < 0 || (npart > 0 && (!d_lagr || !d_pos || !d_vel))) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  p->last_launches = 0;
  cudaStream_t st = S(stream);
  if (is_plain(p->prm)) return plain_run(p, d_lagr, npart, d_pos, d_vel, st);
  if ((rc = field_stages(p, st))) return rc;
  return fused_readout(p, d_lagr, npart, d_pos, d_vel, st);
}

int aar_run_glass(aar_plan* h, const float* d_glass, int64_t nglass, double glass_box, int32_t tile, float* d_pos,
                  float* d_vel, int32_t* d_ids, void* stream) {
  if (!h || nglass < 0 || tile < 1 || !(glass_box > 0)) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  if (!is_fp32(p->prm)) return set_err(p, "aar_run_glass is for the FP32 forms"), AAR_ERR_ARG;
  p->last_launches = 0;
  cudaStream_t st = S(stream);
  if ((rc = field_stages(p, st))) return rc;
  if ((rc = glass_prepare(p, d_glass, nglass, glass_box, tile, st))) return rc;
  return fused_readout_glass(p, nglass, tile, d_pos, d_vel, d_ids, st);
}

static int run_glass_host(Plan* p, const float* h_glass, int64_t nglass, double glass_box, int tile, float* h_pos,
                          float* h_vel, int32_t* h_ids, cudaStream_t st, bool sync);


int aar_run_lattice(aar_plan* h, int32_t glass_n, double glass_box, int32_t tile, float* d_pos, float* d_vel,
                    int32_t* d_ids, void* stream) {
  if (!h || glass_n < 1 || tile < 1 || !(glass_box > 0) || !d_pos || !d_vel) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  if (!is_fp32(p->prm)) return set_err(p, "aar_run_lattice is for the FP32 forms"), AAR_ERR_ARG;
  cudaStream_t st = S(stream);
  bool fused = false;
  // the slab form keeps real displacement fields: the general read-out
  if (p->prm.precision == AAR_FUSED_FP32 && (rc = lattice_prepare(p, glass_n, glass_box, tile, st, fused))) return rc;
  p->last_launches = 0;
  if ((rc = field_stages(p, st, !fused))) return rc;
  if (fused) return fused_rows_lattice(p, glass_n, tile, d_pos, d_vel, d_ids, 0, (int64_t)p->N * p->N, st);
  // general read-out from the lattice glass made on the device
  const int64_t nglass = (int64_t)glass_n * glass_n * glass_n;
  if (nglass > p->glass_cap) {
    AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
    if (p->d_glass) cudaFree(p->d_glass), p->used_bytes -= sizeof(float) * 3 * (size_t)p->glass_cap;
    p->d_glass = nullptr;
    p->glass_cap = 0;
    if ((rc = plan_alloc(p, (void**)&p->d_glass, sizeof(float) * 3 * (size_t)nglass))) return rc;
    p->glass_cap = nglass;
  }
  if ((rc = lattice_glass(p, glass_n, glass_box, p->d_glass, st))) return rc;
  if ((rc = glass_prepare(p, p->d_glass, nglass, glass_box, tile, st))) return rc;
  return fused_readout_glass(p, nglass, tile, d_pos, d_vel, d_ids, st);
}

int aar_run_glass_host(aar_plan* h, const float* h_glass, int64_t nglass, double glass_box, int32_t tile,
                       float* h_pos, float* h_vel, int32_t* h_ids, void* stream) {
  if (!h || nglass < 0 || tile < 1 || !(glass_box > 0)) return AAR_ERR_ARG;
  return run_glass_host(&h->p, h_glass, nglass, glass_box, tile, h_pos, h_vel, h_ids, S(stream), true);
}

int aar_run_glass_host_async(aar_plan* h, const float* h_glass, int64_t nglass, double glass_box, int32_t tile,
                             float* h_pos, float* h_vel, int32_t* h_ids, void* stream) {
  if (!h || nglass < 0 || tile < 1 || !(glass_box > 0)) return AAR_ERR_ARG;
  return run_glass_host(&h->p, h_glass, nglass, glass_box, tile, h_pos, h_vel, h_ids, S(stream), false);
}

int aar_wait_host_copies(aar_plan* h) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  for (int i = 0; i < 2; ++i)
    if (p->out_done[i]) AAR_CUDA_TRY(p, cudaEventSynchronize(p->out_done[i]));
  return AAR_OK;
}

int aar_run_host(aar_plan* h, const float* h_lagr, int64_t npart, float* h_pos, float* h_vel, void* stream) {
  if (!h || npart < 0 || (npart > 0 && (!h_lagr || !h_pos || !h_vel))) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  cudaStream_t st = S(stream);
  size_t bytes = sizeof(float) * 3 * (size_t)npart;
  if (npart > p->io_cap) {  // plan-owned staging: in, pos, vel
    if (p->d_io) {
      cudaFree(p->d_io);
      p->used_bytes -= 3 * sizeof(float) * 3 * (size_t)p->io_cap;
      p->d_io = nullptr;
      p->io_cap = 0;
    }
    if ((rc = plan_alloc(p, (void**)&p->d_io, 3 * bytes))) return rc;
    p->io_cap = npart;
  }
  float* d_in = p->d_io;
  float* d_pos = d_in + 3 * (size_t)npart;
  float* d_vel = d_pos + 3 * (size_t)npart;
  if (is_plain(p->prm)) {
    if (npart > 0) AAR_CUDA_TRY(p, cudaMemcpyAsync(d_in, h_lagr, bytes, cudaMemcpyHostToDevice, st));
    if ((rc = aar_run(h, d_in, npart, d_pos, d_vel, stream))) return rc;
  } else {
    // the Lagrangian positions are needed only by the read-out: their copy
    // runs on a side stream while the fields are computed
    if (!p->copy_stream) {
      AAR_CUDA_TRY(p, cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking));
      AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->copy_done, cudaEventDisableTiming));
      AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->copy_start, cudaEventDisableTiming));
    }
    AAR_CUDA_TRY(p, cudaEventRecord(p->copy_start, st));  // after earlier work on the caller's stream
    AAR_CUDA_TRY(p, cudaStreamWaitEvent(p->copy_stream, p->copy_start, 0));
    if (npart > 0)
      AAR_CUDA_TRY(p, cudaMemcpyAsync(d_in, h_lagr, bytes, cudaMemcpyHostToDevice, p->copy_stream));
    AAR_CUDA_TRY(p, cudaEventRecord(p->copy_done, p->copy_stream));
    p->last_launches = 0;
    if ((rc = field_stages(p, st))) return rc;
    AAR_CUDA_TRY(p, cudaStreamWaitEvent(st, p->copy_done, 0));
    // read-out in chunks; each chunk's Pos/Vel go to the host on one of two
    // side streams while the next chunks are read out
    if (!p->out_stream[0]) {
      for (int i = 0; i < 2; ++i) {
        AAR_CUDA_TRY(p, cudaStreamCreateWithFlags(&p->out_stream[i], cudaStreamNonBlocking));
        AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->out_done[i], cudaEventDisableTiming));
      }
      for (int i = 0; i < Plan::kOutChunks; ++i)
        AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->chunk_read[i], cudaEventDisableTiming));
    }
    const int nchunk = npart >= (int64_t)p->out_chunks * 65536 ? p->out_chunks : 1;
    for (int c = 0; c < nchunk; ++c) {
      const int64_t a = npart * c / nchunk, b = npart * (c + 1) / nchunk, cnt = b - a;
      if ((rc = fused_readout(p, d_in + 3 * a, cnt, d_pos + 3 * a, d_vel + 3 * a, st))) return rc;
      if (cnt == 0) continue;
      cudaStream_t os = p->out_stream[c & 1];
      AAR_CUDA_TRY(p, cudaEventRecord(p->chunk_read[c], st));
      AAR_CUDA_TRY(p, cudaStreamWaitEvent(os, p->chunk_read[c], 0));
      const size_t cb = sizeof(float) * 3 * (size_t)cnt;
      AAR_CUDA_TRY(p, cudaMemcpyAsync(h_pos + 3 * a, d_pos + 3 * a, cb, cudaMemcpyDeviceToHost, os));
      AAR_CUDA_TRY(p, cudaMemcpyAsync(h_vel + 3 * a, d_vel + 3 * a, cb, cudaMemcpyDeviceToHost, os));
    }
    for (int i = 0; i < 2; ++i) {
      AAR_CUDA_TRY(p, cudaEventRecord(p->out_done[i], p->out_stream[i]));
      AAR_CUDA_TRY(p, cudaStreamWaitEvent(st, p->out_done[i], 0));
    }
    AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
    return AAR_OK;
  }
  if (npart > 0) {
    AAR_CUDA_TRY(p, cudaMemcpyAsync(h_pos, d_pos, bytes, cudaMemcpyDeviceToHost, st));
    AAR_CUDA_TRY(p, cudaMemcpyAsync(h_vel, d_vel, bytes, cudaMemcpyDeviceToHost, st));
  }
  AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
  return AAR_OK;
}

// Is the host glass the regular g^3 lattice with coordinates
// (float)(i * (glass_box / g)) in read_glass.c's particle order?
static bool host_lattice(const float* gl, int64_t n, double glass_box, int& g) {
  const int64_t c = llround(cbrt((double)n));
  if (c < 1 || c * c * c != n) return false;
  const double sp = glass_box / (double)c;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t ix = i / (c * c), iy = (i / c) % c, iz = i % c;
    if (gl[3 * i] != (float)((double)ix * sp) || gl[3 * i + 1] != (float)((double)iy * sp) ||
        gl[3 * i + 2] != (float)((double)iz * sp))
      return false;
  }
  g = (int)c;
  return true;
}

// Host-buffer glass run (aar_run_glass_host / _async).  Read-out in chunks
// of particles; chunk c goes to the host on side stream c % 2 as soon as it
// is read out.  Chunk c's staging is reused by the next call only after the
// event recorded behind its copy (gchunk_free[c]): a never-recorded event is
// already complete, so the first call waits for nothing.
static int run_glass_host(Plan* p, const float* h_glass, int64_t nglass, double glass_box, int tile, float* h_pos,
                          float* h_vel, int32_t* h_ids, cudaStream_t st, bool sync) {
  int rc = ready(p);
  if (rc) return rc;
  if (!is_fp32(p->prm)) return set_err(p, "aar_run_glass_host is for the FP32 forms"), AAR_ERR_ARG;
  const int64_t t3 = (int64_t)tile * tile * tile;
  const int64_t npart = nglass * t3;
  if (npart > 0 && (!h_glass || !h_pos || !h_vel)) return set_err(p, "null host buffer"), AAR_ERR_ARG;
  if (nglass > p->glass_cap) {
    // the previous call's read-out may still read the old glass buffer
    AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
    if (p->d_glass) cudaFree(p->d_glass), p->used_bytes -= sizeof(float) * 3 * (size_t)p->glass_cap;
    p->d_glass = nullptr;
    p->glass_cap = 0;
    if ((rc = plan_alloc(p, (void**)&p->d_glass, sizeof(float) * 3 * (size_t)nglass))) return rc;
    p->glass_cap = nglass;
  }
  const size_t per = sizeof(float) * 6 + sizeof(int32_t);
  if (npart > p->gout_cap) {
    // staging still being copied out by an earlier asynchronous call
    AAR_CUDA_TRY(p, cudaDeviceSynchronize());
    if (p->d_gout) cudaFree(p->d_gout), p->used_bytes -= per * (size_t)p->gout_cap;
    p->d_gout = nullptr;
    p->gout_cap = 0;
    if ((rc = plan_alloc(p, (void**)&p->d_gout, per * (size_t)npart))) return rc;
    p->gout_cap = npart;
  }
  if (!p->out_stream[0]) {
    for (int i = 0; i < 2; ++i) {
      AAR_CUDA_TRY(p, cudaStreamCreateWithFlags(&p->out_stream[i], cudaStreamNonBlocking));
      AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->out_done[i], cudaEventDisableTiming));
    }
    for (int i = 0; i < Plan::kOutChunks; ++i)
      AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->chunk_read[i], cudaEventDisableTiming));
  }
  if (!p->gchunk_read[0])
    for (int i = 0; i < Plan::kGlassChunks; ++i) {
      AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->gchunk_read[i], cudaEventDisableTiming));
      AAR_CUDA_TRY(p, cudaEventCreateWithFlags(&p->gchunk_free[i], cudaEventDisableTiming));
    }
  float* d_pos = p->d_gout;
  float* d_vel = d_pos + 3 * (size_t)npart;
  int32_t* d_ids = h_ids ? (int32_t*)(d_vel + 3 * (size_t)npart) : nullptr;
  p->last_launches = 0;
  // the chunk hand-over assumes the previous call's staging layout; with
  // another particle count, wait for all of its copies first
  if (npart != p->gout_last && p->out_done[0])
    for (int i = 0; i < 2; ++i) AAR_CUDA_TRY(p, cudaStreamWaitEvent(st, p->out_done[i], 0));
  p->gout_last = npart;
  // the reference's default glass is a regular lattice: when the host glass
  // is one and its tiling lands every particle on a grid point, the
  // read-out is fused into the displacement rows, chunk by chunk of tile
  // rows (the rows of tile index ti are contiguous for g a multiple of the
  // row block, and so are their particles)
  int g = 0;
  bool lat = false;
  if (p->prm.precision == AAR_FUSED_FP32 && host_lattice(h_glass, nglass, glass_box, g) && g % kXB == 0 &&
      (rc = lattice_prepare(p, g, glass_box, tile, st, lat)))
    return rc;
  if (nglass > 0 && !lat)
    AAR_CUDA_TRY(p, cudaMemcpyAsync(p->d_glass, h_glass, sizeof(float) * 3 * (size_t)nglass, cudaMemcpyHostToDevice, st));
  if ((rc = field_stages(p, st, !lat))) return rc;
  if (!lat && (rc = glass_prepare(p, p->d_glass, nglass, glass_box, tile, st))) return rc;
  const int nchunk = lat ? std::min(tile, (int)Plan::kGlassChunks)
                         : (npart >= (int64_t)Plan::kGlassChunks * 65536 ? Plan::kGlassChunks : 1);
  for (int c = 0; c < nchunk; ++c) {
    int64_t a, b;
    if (lat) {
      const int64_t t0 = (int64_t)tile * c / nchunk, t1 = (int64_t)tile * (c + 1) / nchunk;
      a = t0 * (int64_t)tile * tile * nglass;
      b = t1 * (int64_t)tile * tile * nglass;
    } else {
      a = npart * c / nchunk;
      b = npart * (c + 1) / nchunk;
    }
    const int64_t cnt = b - a;
    if (cnt == 0) continue;
    AAR_CUDA_TRY(p, cudaStreamWaitEvent(st, p->gchunk_free[c], 0));
    if (lat) {
      const int64_t t0 = (int64_t)tile * c / nchunk, t1 = (int64_t)tile * (c + 1) / nchunk;
      if ((rc = fused_rows_lattice(p, g, tile, d_pos, d_vel, d_ids, t0 * g * p->N, (t1 - t0) * g * p->N, st))) return rc;
    } else if ((rc = fused_readout_glass(p, nglass, tile, d_pos, d_vel, d_ids, st, a, b))) {
      return rc;
    }
    cudaStream_t os = p->out_stream[c & 1];
    AAR_CUDA_TRY(p, cudaEventRecord(p->gchunk_read[c], st));
    AAR_CUDA_TRY(p, cudaStreamWaitEvent(os, p->gchunk_read[c], 0));
    const size_t cb = sizeof(float) * 3 * (size_t)cnt;
    AAR_CUDA_TRY(p, cudaMemcpyAsync(h_pos + 3 * a, d_pos + 3 * a, cb, cudaMemcpyDeviceToHost, os));
    AAR_CUDA_TRY(p, cudaMemcpyAsync(h_vel + 3 * a, d_vel + 3 * a, cb, cudaMemcpyDeviceToHost, os));
    if (h_ids)
      AAR_CUDA_TRY(p, cudaMemcpyAsync(h_ids + a, d_ids + a, sizeof(int32_t) * (size_t)cnt, cudaMemcpyDeviceToHost, os));
    AAR_CUDA_TRY(p, cudaEventRecord(p->gchunk_free[c], os));
  }
  // the copies stay on the side streams: the caller's stream goes on with
  // the next realisation while they run (aar_wait_host_copies waits for them)
  for (int i = 0; i < 2; ++i) AAR_CUDA_TRY(p, cudaEventRecord(p->out_done[i], p->out_stream[i]));
  if (sync) {
    AAR_CUDA_TRY(p, cudaStreamSynchronize(st));
    for (int i = 0; i < 2; ++i) AAR_CUDA_TRY(p, cudaEventSynchronize(p->out_done[i]));
  }
  return AAR_OK;
}

int aar_copy_spectrum(aar_plan* h, void* d_out, void* stream) {
  if (!h || !d_out) return AAR_ERR_ARG;
  Plan* p = &h->p;
  if (is_plain(p->prm)) return plain_copy_spectrum(p, d_out, S(stream));
  if (!is_fp32(p->prm) || !p->d_phik) return set_err(p, "no FP32 spectrum in this plan"), AAR_ERR_STATE;
  const int H = p->N / 2 + 1;
  return copy_rows(p, d_out, H, 1, p->d_phik, p->HP, kXB, H, sizeof(float2), S(stream));
}

int aar_gaussian_spectrum_noalloc(aar_plan* h, void* d_out, void* stream) {
  if (!h || !d_out) return AAR_ERR_ARG;
  Plan* p = &h->p;
  if (!p->have_transfer) return set_err(p, "transfer function not set"), AAR_ERR_STATE;
  return noalloc_gaussian(p, d_out, S(stream));
}

static int need_work(Plan* p) {
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "transforms are for the fused form"), AAR_ERR_ARG;
  if (!p->d_work) {
    int rc = alloc_fused(p, 0);
    if (rc) return rc;
    if ((rc = fused_configure_xform(p))) return rc;
  }
  return AAR_OK;
}

int aar_c2r(aar_plan* h, const void* d_in, float* d_out, void* stream) {
  if (!h || !d_in || !d_out) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = need_work(p);
  if (rc) return rc;
  p->last_launches = 0;
  return fused_c2r(p, (const float2*)d_in, d_out, S(stream));
}

int aar_r2c(aar_plan* h, const float* d_in, void* d_out, void* stream) {
  if (!h || !d_in || !d_out) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = need_work(p);
  if (rc) return rc;
  p->last_launches = 0;
  return fused_r2c(p, d_in, (float2*)d_out, S(stream));
}

int aar_profile_enable(aar_plan* h, int32_t on) {
  if (!h) return AAR_ERR_ARG;
  h->p.profiling = on != 0;
  return AAR_OK;
}

int aar_profile_report(aar_plan* h, char* buf, int32_t len) {
  if (!h || !buf || len <= 0) return AAR_ERR_ARG;
  Plan* p = &h->p;
  AAR_CUDA_TRY(p, cudaDeviceSynchronize());
  std::vector<std::string> names;
  std::vector<double> ms;
  std::vector<int> cnt;
  for (auto& r : p->prof) {
    float t = 0;
    cudaEventElapsedTime(&t, r.a, r.b);
    size_t i = 0;
    while (i < names.size() && names[i] != r.name) ++i;
    if (i == names.size()) {
      names.push_back(r.name);
      ms.push_back(0);
      cnt.push_back(0);
    }
    ms[i] += t;
    cnt[i] += 1;
    p->event_pool.push_back(r.a);
    p->event_pool.push_back(r.b);
  }
  p->prof.clear();
  std::string out;
  for (size_t i = 0; i < names.size(); ++i) {
    char line[256];
    snprintf(line, sizeof(line), "%s,%d,%.6f\n", names[i].c_str(), cnt[i], ms[i]);
    out += line;
  }
  if ((int)out.size() + 1 > len) return set_err(p, "profile report buffer too small"), AAR_ERR_ARG;
  memcpy(buf, out.c_str(), out.size() + 1);
  return AAR_OK;
}

int aar_copy_field(aar_plan* h, int32_t which, void* d_out, void* stream) {
  if (!h || !d_out || which < 0 || which > 5) return AAR_ERR_ARG;
  Plan* p = &h->p;
  if (is_plain(p->prm)) return plain_copy_field(p, which, (double*)d_out, S(stream));
  if (!is_fp32(p->prm) || !p->d_work || which >= p->nwork || !p->disp_real)
    return set_err(p, "no FP32 displacement fields in this plan: run the field stages first"), AAR_ERR_STATE;
  int N = p->N;
  const float* src = (const float*)(p->d_work + (size_t)which * N * N * p->HP);
  return copy_rows(p, d_out, N, 1, src, 2 * p->HP, kXB, N, sizeof(float), S(stream));
}

int aar_profile_modal_rows(aar_plan* h, void* d_work, int64_t nrows, void* stream) {
  if (!h || !d_work) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready_tables(p);  // the caller's fields only: the plan's are not allocated
  if (rc) return rc;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "the row harness is for the fused form"), AAR_ERR_ARG;
  p->last_launches = 0;
  return profile_modal_rows(p, (float2*)d_work, nrows, S(stream));
}

// ------------------------------------------------------------- modal split
int aar_set_modal_partition(aar_plan* h, int32_t part, int32_t nparts) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  if (nparts < 1 || nparts > kMaxModes || part < 0 || part >= nparts)
    return set_err(p, "modal partition: need 0 <= part < nparts <= 32"), AAR_ERR_ARG;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "the modal split is for the fused form"), AAR_ERR_ARG;
  if (part == p->modal_part && nparts == p->modal_nparts) return AAR_OK;
  ++p->generation;
  p->modal_part = part;
  p->modal_nparts = nparts;
  if (!p->have_tables) return AAR_OK;
  AAR_CUDA_TRY(p, cudaDeviceSynchronize());  // the term list is rewritten below
  return fused_prepare(p);
}

int aar_modal_partition(const double* alpha, int32_t M, int32_t nparts, int32_t* part_of_r) {
  if (!alpha || !part_of_r || M < 1 || M > kMaxModes || nparts < 1 || nparts > kMaxModes) return AAR_ERR_ARG;
  std::vector<double> a(alpha, alpha + (size_t)M * M * M);
  const std::vector<int> part = modal_partition(regrouped_terms(a, M), nparts);
  for (int r = 0; r < M; ++r) part_of_r[r] = part[r];
  return AAR_OK;
}

// ------------------------------------------------------------- JIT rows
int aar_set_jit(aar_plan* h, int32_t mode) {
  if (!h || mode < 0 || mode > 2) return AAR_ERR_ARG;
  Plan* p = &h->p;
  p->jit_mode = mode;
  ++p->generation;
  if (!p->have_tables || p->prm.precision != AAR_FUSED_FP32) return AAR_OK;
  return jit_prepare(p);
}

const char* aar_jit_status(const aar_plan* h) { return h ? h->p.jit_status.c_str() : "null plan"; }

// ------------------------------------------------------------- autotuner
// Times the field stages (noise, modal, 2LPT) of this plan on its device for
// each schedule candidate and keeps the fastest: row kernel generic or
// NVRTC-specialised with 2 or 3 resident blocks per SM of 256 threads or 2
// of 320 (ten warps: one round of line transforms fewer when the plan has
// 17 to 20 modes), and the item
// grouping of the multi-output x passes (1, one y row of tiles, four rows).
// Each candidate runs twice (the first run compiles and warms up); the
// second is timed with CUDA events on the stream.  The plan's spectrum and
// fields are overwritten, as by a realisation.
int aar_autotune(aar_plan* h, char* report, int32_t len, void* stream) {
  if (!h) return AAR_ERR_ARG;
  Plan* p = &h->p;
  int rc = ready(p);
  if (rc) return rc;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "the autotuner is for the fused form"), AAR_ERR_ARG;
  cudaStream_t st = S(stream);
  struct Cand {
    int jit, minb, threads;
    int64_t grp;
    float ms;
  };
  const int64_t row_tiles = p->HP / 8;
  // (row kernel, blocks per SM, threads per block); 320 threads only where
  // ten warps take the M input lines in fewer rounds than eight
  std::vector<int3> rows = {{0, 2, 256}, {2, 2, 256}, {2, 3, 256}};
  if ((p->M + 9) / 10 < (p->M + 7) / 8) rows.push_back({2, 2, 320});
  std::vector<Cand> cands;
  for (const int3& r : rows)
    for (int64_t g : {(int64_t)1, row_tiles, 4 * row_tiles}) cands.push_back(Cand{r.x, r.y, r.z, g, -1.f});
  const int saved_mode = p->jit_mode, saved_minb = p->jit_minb, saved_threads = p->jit_threads;
  const int64_t saved_grp = p->xpass_group;
  // every candidate may unload and reload the NVRTC module (jit_prepare), so
  // graphs captured before this call are stale whatever the outcome
  ++p->generation;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  AAR_CUDA_TRY(p, cudaEventCreate(&e0));
  AAR_CUDA_TRY(p, cudaEventCreate(&e1));
  int best = -1;
  for (size_t i = 0; i < cands.size() && rc == AAR_OK; ++i) {
    Cand& c = cands[i];
    p->jit_mode = c.jit;
    p->jit_minb = c.minb;
    p->jit_threads = c.threads;
    p->xpass_group = c.grp;
    if ((rc = jit_prepare(p))) break;
    if (c.jit && p->jit == nullptr) continue;  // NVRTC unavailable: no such candidate
    for (int rep = 0; rep < 2 && rc == AAR_OK; ++rep) {
      if (rep == 1 && (rc = (cudaEventRecord(e0, st) == cudaSuccess ? AAR_OK : AAR_ERR_CUDA))) break;
      if ((rc = run_noise(p, st)) || (rc = fused_modal(p, st)) || (rc = fused_lpt(p, st))) break;
      if (rep == 1 && cudaEventRecord(e1, st) != cudaSuccess) rc = AAR_ERR_CUDA;
    }
    if (rc) break;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&c.ms, e0, e1) != cudaSuccess) {
      rc = AAR_ERR_CUDA;
      break;
    }
    if (best < 0 || c.ms < cands[best].ms) best = (int)i;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == AAR_ERR_CUDA) cudaGetLastError(), set_err(p, "autotune: a CUDA call failed");
  if (rc || best < 0) {
    p->jit_mode = saved_mode;
    p->jit_minb = saved_minb;
    p->jit_threads = saved_threads;
    p->xpass_group = saved_grp;
    jit_prepare(p);
    return rc ? rc : (set_err(p, "autotune: no candidate ran"), AAR_ERR_STATE);
  }
  p->jit_mode = cands[best].jit;
  p->jit_minb = cands[best].minb;
  p->jit_threads = cands[best].threads;
  p->xpass_group = cands[best].grp;
  if ((rc = jit_prepare(p))) return rc;
  if (report && len > 0) {
    std::string out;
    char line[160];
    for (size_t i = 0; i < cands.size(); ++i) {
      const Cand& c = cands[i];
      snprintf(line, sizeof(line), "%s rows=%s minb=%d threads=%d group=%lld %.3f ms\n", (int)i == best ? "*" : " ",
               c.jit ? "nvrtc" : "generic", c.jit ? c.minb : 0, c.threads, (long long)c.grp, c.ms);
      out += line;
    }
    if ((int)out.size() + 1 > len) return set_err(p, "autotune report buffer too small"), AAR_ERR_ARG;
    memcpy(report, out.c_str(), out.size() + 1);
  }
  return AAR_OK;
}

// ------------------------------------------------------------- adjoint
int aar_set_spectrum(aar_plan* h, const void* d_in, void* stream) {
  if (!h || !d_in) return AAR_ERR_ARG;
  Plan* p = &h->p;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "aar_set_spectrum is for the fused form"), AAR_ERR_ARG;
  if (!p->d_phik) {
    int rc = ensure_fields(p);
    if (rc) return rc;
  }
  const int H = p->N / 2 + 1;
  return copy_rows(p, p->d_phik, p->HP, kXB, d_in, H, 1, H, sizeof(float2), S(stream));
}

static int adj_ready(Plan* p) {
  int rc = ready(p);
  if (rc) return rc;
  if (p->prm.precision != AAR_FUSED_FP32) return set_err(p, "the adjoint is for the fused form"), AAR_ERR_ARG;
  return AAR_OK;
}

int aar_adj_spectral(aar_plan* h, int32_t op, int32_t comp, int32_t mode, const void* d_in, void* d_out,
                     int32_t accumulate, void* stream) {
  if (!h || !d_in || !d_out) return AAR_ERR_ARG;
  int rc = adj_ready(&h->p);
  if (rc) return rc;
  return adj_spectral(&h->p, op, comp, mode, (const float2*)d_in, (float2*)d_out, accumulate, S(stream));
}

int aar_adj_source(aar_plan* h, const float* d_hess, const float* d_gsource, float* d_out, void* stream) {
  if (!h || !d_hess || !d_gsource || !d_out) return AAR_ERR_ARG;
  int rc = adj_ready(&h->p);
  if (rc) return rc;
  return adj_source(&h->p, d_hess, d_gsource, d_out, S(stream));
}

int aar_adj_products(aar_plan* h, const float* d_f, const float* d_gg, float* d_gf, double* d_galpha, void* stream) {
  if (!h || !d_f || !d_gg || !d_gf || !d_galpha) return AAR_ERR_ARG;
  int rc = adj_ready(&h->p);
  if (rc) return rc;
  return adj_products(&h->p, d_f, d_gg, d_gf, d_galpha, S(stream));
}

// ------------------------------------------------------------- batches
// Several fused plans (realisations with their own seed, coefficient table,
// mode count and buffers) captured once into one CUDA graph: every plan's
// aar_run work is a branch of the graph on its own stream, so small kernels
// of different realisations overlap; later runs replay the graph with one
// launch.  The graph is captured again when the buffer pointers or particle
// counts change.
struct aar_batch {
  std::vector<aar_plan*> plans;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> done;
  cudaEvent_t fork = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uintptr_t> key;  // pointers and counts the graph was captured with
  std::string err;
  int launches = 0;
};

static int batch_err(aar_batch* b, const std::string& e, int code) {
  b->err = e;
  return code;
}

static void batch_drop_graph(aar_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->key.clear();
}

int aar_batch_create(aar_plan* const* plans, int32_t nplans, aar_batch** out) {
  if (!plans || nplans < 1 || !out) return AAR_ERR_ARG;
  *out = nullptr;
  aar_batch* b = new (std::nothrow) aar_batch();
  if (!b) return AAR_ERR_OOM;
  int dev = -1;
  for (int i = 0; i < nplans; ++i) {
    if (!plans[i] || plans[i]->p.prm.precision != AAR_FUSED_FP32 || (i > 0 && plans[i]->p.dev != dev)) {
      delete b;
      return AAR_ERR_ARG;
    }
    dev = plans[i]->p.dev;
    b->plans.push_back(plans[i]);
  }
  bool ok = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < nplans; ++i) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
    if (st) b->streams.push_back(st);
    if (ev) b->done.push_back(ev);
  }
  if (!ok) {
    aar_batch_destroy(b);
    return AAR_ERR_CUDA;
  }
  *out = b;
  return AAR_OK;
}

static int batch_capture(aar_batch* b, const float* const* d_lagr, const int64_t* npart, float* const* d_pos,
                         float* const* d_vel) {
  const int n = (int)b->plans.size();
  if (cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return batch_err(b, "cudaStreamBeginCapture failed", AAR_ERR_CUDA);
  int rc = AAR_OK;
  int launches = 0;
  if (cudaEventRecord(b->fork, b->cap) != cudaSuccess) rc = batch_err(b, "cudaEventRecord failed", AAR_ERR_CUDA);
  for (int i = 0; i < n && rc == AAR_OK; ++i) {
    Plan* p = &b->plans[i]->p;
    const bool prof = p->profiling;
    p->profiling = false;  // no event records inside the graph
    cudaStream_t st = b->streams[i];
    if (cudaStreamWaitEvent(st, b->fork, 0) != cudaSuccess) {
      rc = batch_err(b, "cudaStreamWaitEvent failed", AAR_ERR_CUDA);
    } else {
      rc = aar_run(b->plans[i], d_lagr[i], npart[i], d_pos[i], d_vel[i], st);
      if (rc) b->err = "plan " + std::to_string(i) + ": " + p->err;
      launches += p->last_launches;
    }
    p->profiling = prof;
    if (rc == AAR_OK && (cudaEventRecord(b->done[i], st) != cudaSuccess ||
                         cudaStreamWaitEvent(b->cap, b->done[i], 0) != cudaSuccess))
      rc = batch_err(b, "joining the plan streams failed", AAR_ERR_CUDA);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->cap, &g);
  if (rc == AAR_OK && e != cudaSuccess) rc = batch_err(b, std::string("capture: ") + cudaGetErrorString(e), AAR_ERR_CUDA);
  if (rc != AAR_OK) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
  }
  b->graph = g;
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) {
    batch_drop_graph(b);
    return batch_err(b, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e), AAR_ERR_CUDA);
  }
  b->launches = launches;
  return AAR_OK;
}

int aar_batch_run(aar_batch* b, const float* const* d_lagr, const int64_t* npart, float* const* d_pos,
                  float* const* d_vel, void* stream) {
  if (!b || !d_lagr || !npart || !d_pos || !d_vel) return AAR_ERR_ARG;
  const int n = (int)b->plans.size();
  std::vector<uintptr_t> key;
  for (int i = 0; i < n; ++i) {
    if (npart[i] < 0 || (npart[i] > 0 && (!d_lagr[i] || !d_pos[i] || !d_vel[i])))
      return batch_err(b, "bad particle arrays for plan " + std::to_string(i), AAR_ERR_ARG);
    int rc = ready(&b->plans[i]->p);
    if (rc) return batch_err(b, "plan " + std::to_string(i) + ": " + b->plans[i]->p.err, rc);
    key.insert(key.end(), {(uintptr_t)d_lagr[i], (uintptr_t)npart[i], (uintptr_t)d_pos[i], (uintptr_t)d_vel[i],
                           (uintptr_t)b->plans[i]->p.generation});
  }
  if (!b->exec || key != b->key) {
    batch_drop_graph(b);
    int rc = batch_capture(b, d_lagr, npart, d_pos, d_vel);
    if (rc) return rc;
    b->key = key;
  }
  cudaError_t e = cudaGraphLaunch(b->exec, S(stream));
  if (e != cudaSuccess) return batch_err(b, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e), AAR_ERR_CUDA);
  return AAR_OK;
}

int aar_batch_launch_count(const aar_batch* b) { return b ? b->launches : 0; }

const char* aar_batch_last_error(const aar_batch* b) { return b ? b->err.c_str() : "null batch"; }

void aar_batch_destroy(aar_batch* b) {
  if (!b) return;
  batch_drop_graph(b);
  for (auto st : b->streams) cudaStreamDestroy(st);
  for (auto ev : b->done) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap) cudaStreamDestroy(b->cap);
  delete b;
}

}  // extern "C"
