/*
 * CPU oracle for the Aarambam initial-condition path -- TEST INFRASTRUCTURE.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this code, and only as the checker.  It restates, in FP64 C, the algorithm
 * of the reference executable Aarambam/LPT/Basis (main.c, power.c,
 * read_glass.c, nrsrc/qromb.c); every function cites the lines it follows.
 *
 * The modal non-Gaussian potential keeps the reference's own loop structure
 * (one c2r per first index, one c2r + product + r2c per active pair, the
 * 10 counter-term pairs and the potential round trips, long double
 * accumulators), so that its cost stands in for the reference's CPU cost.
 */
#include "aar_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846
#define ORC_GRAVITY 6.672e-8
#define ORC_HUBBLE 3.2407789e-18

/* ========================================================================= */
/* RANLUX, GSL flavour (gsl_rng_ranlxd1 / ranlxd2).                           */
/* Subtract-with-borrow x_n = x_{n-5} - x_{n-12} - c_{n-1} (mod 2^48); after   */
/* every `luxury` steps the 12 most recent values are delivered in order.     */
/* Seeding: 31-bit seed bits drive the recurrence b_{n+31} = b_n ^ b_{n+18};  */
/* each state word takes 48 successive complemented bits, MSB first.          */
/* Call sites in the reference: main.c:317-349 (seed table), :392-403.        */
/* ========================================================================= */
void orc_rlx_seed(orc_rlx *s, unsigned long seed, int luxury) {
  if (seed == 0) seed = 1;
  uint32_t v = (uint32_t)(seed & 0xFFFFFFFFUL);
  int bits[31];
  for (int k = 0; k < 31; ++k) {
    bits[k] = (int)(v & 1u);
    v >>= 1;
  }
  int ib = 0, jb = 18;
  for (int w = 0; w < 12; ++w) {
    int64_t word = 0;
    for (int l = 0; l < 48; ++l) {
      word = 2 * word + (bits[ib] ^ 1);
      bits[ib] ^= bits[jb];
      ib = (ib + 1) % 31;
      jb = (jb + 1) % 31;
    }
    s->x[w] = word;
  }
  s->carry = 0;
  s->pos = 12; /* the seeded words themselves are never delivered */
  s->luxury = luxury;
}

static void orc_rlx_refill(orc_rlx *s) {
  int64_t *x = s->x;
  int64_t c = s->carry;
  for (int t = 0; t < s->luxury; ++t) {
    int a = t % 12, b = (t + 7) % 12;
    int64_t d = x[b] - x[a] - c;
    c = d < 0;
    if (d < 0) d += ((int64_t)1 << 48);
    x[a] = d;
  }
  int sh = s->luxury % 12; /* rotate so that x[0] is the oldest again */
  int64_t y[12];
  for (int k = 0; k < 12; ++k) y[k] = x[(k + sh) % 12];
  memcpy(x, y, sizeof(y));
  s->carry = c;
  s->pos = 0;
}

double orc_rlx_uniform(orc_rlx *s) {
  if (s->pos == 12) orc_rlx_refill(s);
  return (double)s->x[s->pos++] * (1.0 / 281474976710656.0);
}

unsigned long orc_rlx_get(orc_rlx *s) { return (unsigned long)(orc_rlx_uniform(s) * 4294967296.0); }

/* ========================================================================= */
/* Cosmology set-up                                                           */
/* ========================================================================= */

/* power.c:181-217 (tabulated transfer, log-log interpolation, 0 outside). */
double orc_transfer(const orc_params *p, double k) {
  k *= p->kconv;
  double lk = log10(k);
  if (lk < p->logk[0] || lk > p->logk[p->ntrans - 1]) return 0;
  int lo = 0, hi = p->ntrans - 1;
  while (hi - lo > 1) {
    int mid = (hi + lo) / 2;
    if (lk < p->logk[mid])
      hi = mid;
    else
      lo = mid;
  }
  double dl = p->logk[hi] - p->logk[lo];
  double u = (lk - p->logk[lo]) / dl;
  double lt = (1 - u) * p->logT[lo] + u * p->logT[hi];
  return pow(10.0, lt);
}

/* Romberg integration (nrsrc/qromb.c:2-26): trapezoid sums with step halving,
   extrapolated to zero step by Neville's scheme through the last 5 estimates;
   stops when the last correction is below 1e-8 of the estimate. */
typedef double (*orc_fn)(double, const void *);

static double orc_romberg(orc_fn f, const void *ctx, double a, double b) {
  enum { JMAX = 40, K = 5 };
  double s[JMAX + 2], h[JMAX + 2];
  double trap = 0;
  h[1] = 1.0;
  for (int j = 1; j <= JMAX; ++j) {
    if (j == 1) {
      trap = 0.5 * (b - a) * (f(a, ctx) + f(b, ctx));
    } else {
      long it = 1L << (j - 2);
      double del = (b - a) / (double)it, x = a + 0.5 * del, sum = 0;
      for (long q = 0; q < it; ++q, x += del) sum += f(x, ctx);
      trap = 0.5 * (trap + (b - a) * sum / (double)it);
    }
    s[j] = trap;
    if (j >= K) {
      /* Neville tableau at x=0 through points (h[j-K+1..j], s[...]) */
      const double *xa = &h[j - K + 1], *ya = &s[j - K + 1];
      double c[K], d[K];
      int ns = 0;
      double dif = fabs(xa[0]);
      for (int i = 0; i < K; ++i) {
        double dt = fabs(xa[i]);
        if (dt < dif) {
          ns = i;
          dif = dt;
        }
        c[i] = ya[i];
        d[i] = ya[i];
      }
      double y = ya[ns--], dy = 0;
      for (int m = 1; m < K; ++m) {
        for (int i = 0; i < K - m; ++i) {
          double ho = xa[i], hp = xa[i + m];
          double w = c[i + 1] - d[i];
          double den = w / (ho - hp);
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

typedef struct {
  const orc_params *p;
  double R;
} orc_sig_ctx;

/* PowerSpec (Basis/power.c:240-265 case 0; ResBasis/power.c:240-260, one
   case per WhichSpectrum, T^2 applied after the switch) */
static double orc_powerspec(const orc_params *p, double k) {
  double power = p->Norm * exp(p->ns * log(k));
  if (p->ResBasis && p->WhichSpectrum == 1)
    power = p->Norm * exp(p->ns * log(k)) * (1 + p->A_res * cos(p->w_res * k + p->phi_res));
  if (p->ResBasis && p->WhichSpectrum == 2)
    power = p->Norm * exp(p->ns * log(k)) * (1 + p->A_res * cos(p->w_res * log(k) + p->phi_res));
  double T = orc_transfer(p, k);
  power *= T * T;
  return power;
}

/* power.c:562-576 */
static double orc_sigma2_int(double k, const void *vctx) {
  const orc_sig_ctx *c = (const orc_sig_ctx *)vctx;
  double kr = c->R * k, kr2 = kr * kr, kr3 = kr2 * kr;
  if (kr < 1e-8) return 0;
  double w = 3 * (sin(kr) / kr3 - cos(kr) / kr2);
  double P = orc_powerspec(c->p, k);
  return 4 * ORC_PI * k * k * w * w * P;
}

typedef struct {
  double Om, OL;
} orc_gr_ctx;

/* power.c:579-598 */
static double orc_growth_int(double a, const void *vctx) {
  const orc_gr_ctx *c = (const orc_gr_ctx *)vctx;
  return pow(a / (c->Om + (1 - c->Om - c->OL) * a + c->OL * a * a * a), 1.5);
}
static double orc_growth(double a, double Om, double OL) {
  orc_gr_ctx c = {Om, OL};
  double ha = sqrt(Om / (a * a * a) + (1 - Om - OL) / (a * a) + OL);
  return ha * orc_romberg(orc_growth_int, &c, 0, a);
}

static int orc_cmp_pair(const void *a, const void *b) {
  const double *x = (const double *)a, *y = (const double *)b;
  return (x[0] > y[0]) - (x[0] < y[0]);
}

/* read_transfer_table (power.c:66-153), set_units (main.c:1547-1552),
   initialize_powerspectrum (power.c:391-448), main.c:305-307 and :372. */
int orc_setup(orc_params *p, const orc_cosmo *c, int ntrans, const double *k, const double *T) {
  if (ntrans < 2) return 17;
  double *tab = (double *)malloc(sizeof(double) * 2 * ntrans);
  for (int i = 0; i < ntrans; ++i) {
    tab[2 * i] = log10(k[i]);
    tab[2 * i + 1] = log10(T[i]);
  }
  qsort(tab, ntrans, 2 * sizeof(double), orc_cmp_pair);
  if (tab[0] >= -4.6) {
    free(tab);
    return 1111;
  }
  p->ntrans = ntrans;
  p->logk = (double *)malloc(sizeof(double) * ntrans);
  p->logT = (double *)malloc(sizeof(double) * ntrans);
  double t0 = tab[1];
  for (int i = 0; i < ntrans; ++i) {
    p->logk[i] = tab[2 * i];
    p->logT[i] = tab[2 * i + 1] - t0;
  }
  free(tab);
  p->kconv = c->InputSpectrum_UnitLength_in_cm / c->UnitLength_in_cm;
  p->ns = c->PrimordialIndex;

  double UnitTime_in_s = c->UnitLength_in_cm / c->UnitVelocity_in_cm_per_s;
  p->Hubble = ORC_HUBBLE * UnitTime_in_s;
  p->InitTime = 1 / (1 + c->Redshift);
  double R8 = 8 * (3.085678e24 / c->UnitLength_in_cm);
  p->Norm = 1.0;
  orc_sig_ctx sc = {p, R8};
  double res = orc_romberg(orc_sigma2_int, &sc, 0, 500.0 * 1 / R8);
  p->Norm = c->Sigma8 * c->Sigma8 / res;
  p->Anorm = p->Norm;
  double Om = c->Omega, OL = c->OmegaLambda;
  p->D0 = orc_growth(1.0, Om, OL) / orc_growth(1.e-8, Om, OL) * 1.e-8;
  p->Dplus = orc_growth(1.0, Om, OL) / orc_growth(p->InitTime, Om, OL);
  double a = p->InitTime;
  double hubble_a = p->Hubble * sqrt(Om / pow(a, 3) + (1 - Om - OL) / pow(a, 2) + OL);
  double om_a = Om / (Om + a * (1 - Om - OL) + a * a * a * OL);
  p->vel_prefac = a * hubble_a * pow(om_a, 0.6) / sqrt(a);
  p->vel_prefac2 = a * hubble_a * (2 * pow(om_a, 4. / 7.)) / sqrt(a);
  p->Beta = 1.5 * Om /
            (2998. * 2998. / c->UnitLength_in_cm / c->UnitLength_in_cm * 3.085678e24 * 3.085678e24) /
            p->D0;
  return 0;
}

void orc_free(orc_params *p) {
  free(p->logk);
  free(p->logT);
  p->logk = p->logT = NULL;
}

/* ========================================================================= */
/* FFT: Stockham auto-sort, radices 4/2/3/5, FP64 (FFTW2 stand-in).           */
/* Iteration per Govindaraju et al., SC'08 ("High performance discrete        */
/* Fourier transforms on graphics processors"), Fig. 2.                       */
/* ========================================================================= */
typedef struct {
  int n, nf;
  int f[64];
  double *tw; /* exp(-2 pi i t / n), t = 0..n-1 */
} orc_fft;

static void orc_fft_init(orc_fft *pl, int n) {
  pl->n = n;
  pl->nf = 0;
  int m = n;
  while (m % 4 == 0) {
    pl->f[pl->nf++] = 4;
    m /= 4;
  }
  while (m % 2 == 0) {
    pl->f[pl->nf++] = 2;
    m /= 2;
  }
  while (m % 3 == 0) {
    pl->f[pl->nf++] = 3;
    m /= 3;
  }
  while (m % 5 == 0) {
    pl->f[pl->nf++] = 5;
    m /= 5;
  }
  if (m != 1) pl->f[pl->nf++] = m; /* generic odd factor, slow DFT */
  pl->tw = (double *)malloc(sizeof(double) * 2 * n);
  for (int t = 0; t < n; ++t) {
    long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)n;
    pl->tw[2 * t] = (double)cosl(ang);
    pl->tw[2 * t + 1] = (double)sinl(ang);
  }
}

static void orc_fft_free(orc_fft *pl) { free(pl->tw); }

/* in-place 1-D complex DFT of x (n complex), sign -1 forward, +1 inverse;
   work must hold n complex. */
static void orc_fft_1d(const orc_fft *pl, double *x, double *work, int sign) {
  int n = pl->n;
  double *src = x, *dst = work;
  int Ns = 1;
  for (int s = 0; s < pl->nf; ++s) {
    int R = pl->f[s];
    int stride = n / R;
    for (int j = 0; j < stride; ++j) {
      int k = j % Ns;
      double vr[64], vi[64];
      for (int r = 0; r < R; ++r) {
        double ar = src[2 * (j + r * stride)], ai = src[2 * (j + r * stride) + 1];
        long t = ((long)r * k * (n / (Ns * R))) % n;
        double wr = pl->tw[2 * t], wi = sign < 0 ? pl->tw[2 * t + 1] : -pl->tw[2 * t + 1];
        vr[r] = ar * wr - ai * wi;
        vi[r] = ar * wi + ai * wr;
      }
      double yr[64], yi[64];
      if (R == 2) {
        yr[0] = vr[0] + vr[1];
        yi[0] = vi[0] + vi[1];
        yr[1] = vr[0] - vr[1];
        yi[1] = vi[0] - vi[1];
      } else if (R == 4) {
        double s0r = vr[0] + vr[2], s0i = vi[0] + vi[2];
        double d0r = vr[0] - vr[2], d0i = vi[0] - vi[2];
        double s1r = vr[1] + vr[3], s1i = vi[1] + vi[3];
        double d1r = vr[1] - vr[3], d1i = vi[1] - vi[3];
        /* rotate d1 by sign*i */
        double rr = sign < 0 ? d1i : -d1i, ri = sign < 0 ? -d1r : d1r;
        yr[0] = s0r + s1r;
        yi[0] = s0i + s1i;
        yr[2] = s0r - s1r;
        yi[2] = s0i - s1i;
        yr[1] = d0r + rr;
        yi[1] = d0i + ri;
        yr[3] = d0r - rr;
        yi[3] = d0i - ri;
      } else {
        for (int q = 0; q < R; ++q) {
          double ar = 0, ai = 0;
          for (int r = 0; r < R; ++r) {
            long t = ((long)q * r % R) * (n / R);
            double wr = pl->tw[2 * t], wi = sign < 0 ? pl->tw[2 * t + 1] : -pl->tw[2 * t + 1];
            ar += vr[r] * wr - vi[r] * wi;
            ai += vr[r] * wi + vi[r] * wr;
          }
          yr[q] = ar;
          yi[q] = ai;
        }
      }
      int base = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; ++r) {
        dst[2 * (base + r * Ns)] = yr[r];
        dst[2 * (base + r * Ns) + 1] = yi[r];
      }
    }
    double *t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  if (src != x) memcpy(x, src, sizeof(double) * 2 * n);
}

/* complex pass along one axis of a [N][N][H] complex array */
static void orc_pass_axis(const orc_fft *pl, double *c, int N, int H, int axis, int sign) {
  size_t sN = (size_t)N;
#pragma omp parallel
  {
    double *line = (double *)malloc(sizeof(double) * 2 * N);
    double *work = (double *)malloc(sizeof(double) * 2 * N);
#pragma omp for schedule(static)
    for (long q = 0; q < (long)N * H; ++q) {
      size_t a = (size_t)(q / H), kz = (size_t)(q % H), base, stride;
      if (axis == 0) { /* along x: fixed (y=a, kz) */
        base = (a * H + kz);
        stride = sN * H;
      } else { /* along y: fixed (x=a, kz) */
        base = a * sN * H + kz;
        stride = H;
      }
      for (int t = 0; t < N; ++t) {
        line[2 * t] = c[2 * (base + t * stride)];
        line[2 * t + 1] = c[2 * (base + t * stride) + 1];
      }
      orc_fft_1d(pl, line, work, sign);
      for (int t = 0; t < N; ++t) {
        c[2 * (base + t * stride)] = line[2 * t];
        c[2 * (base + t * stride) + 1] = line[2 * t + 1];
      }
    }
    free(line);
    free(work);
  }
}

/* c2r: x and y complex inverse passes, then the Hermitian 1-D c2r along z in
   which the imaginary parts of the kz=0 and kz=N/2 entries are dropped. */
void orc_c2r_3d(int N, const double *cin, double *rout) {
  int H = N / 2 + 1;
  size_t nc = (size_t)N * N * H;
  double *c = (double *)malloc(sizeof(double) * 2 * nc);
  memcpy(c, cin, sizeof(double) * 2 * nc);
  orc_fft pl;
  orc_fft_init(&pl, N);
  orc_pass_axis(&pl, c, N, H, 0, +1);
  orc_pass_axis(&pl, c, N, H, 1, +1);
#pragma omp parallel
  {
    double *line = (double *)malloc(sizeof(double) * 2 * N);
    double *work = (double *)malloc(sizeof(double) * 2 * N);
#pragma omp for schedule(static)
    for (long q = 0; q < (long)N * N; ++q) {
      const double *row = c + 2 * (size_t)q * H;
      line[0] = row[0];
      line[1] = 0;
      for (int kz = 1; kz < N / 2; ++kz) {
        line[2 * kz] = row[2 * kz];
        line[2 * kz + 1] = row[2 * kz + 1];
        line[2 * (N - kz)] = row[2 * kz];
        line[2 * (N - kz) + 1] = -row[2 * kz + 1];
      }
      line[2 * (N / 2)] = row[2 * (N / 2)];
      line[2 * (N / 2) + 1] = 0;
      orc_fft_1d(&pl, line, work, +1);
      double *out = rout + (size_t)q * N;
      for (int z = 0; z < N; ++z) out[z] = line[2 * z];
    }
    free(line);
    free(work);
  }
  orc_fft_free(&pl);
  free(c);
}

void orc_r2c_3d(int N, const double *rin, double *cout) {
  int H = N / 2 + 1;
  orc_fft pl;
  orc_fft_init(&pl, N);
#pragma omp parallel
  {
    double *line = (double *)malloc(sizeof(double) * 2 * N);
    double *work = (double *)malloc(sizeof(double) * 2 * N);
#pragma omp for schedule(static)
    for (long q = 0; q < (long)N * N; ++q) {
      const double *in = rin + (size_t)q * N;
      for (int z = 0; z < N; ++z) {
        line[2 * z] = in[z];
        line[2 * z + 1] = 0;
      }
      orc_fft_1d(&pl, line, work, -1);
      memcpy(cout + 2 * (size_t)q * H, line, sizeof(double) * 2 * H);
    }
    free(line);
    free(work);
  }
  orc_pass_axis(&pl, cout, N, H, 1, -1);
  orc_pass_axis(&pl, cout, N, H, 0, -1);
  orc_fft_free(&pl);
}

/* ========================================================================= */
/* Seed table (main.c:317-349): one ranlxd1 stream seeded with Seed fills the */
/* N x N table in 8 "shell" segments per i < N/2.                             */
/* ========================================================================= */
void orc_seedtable(int seed, int N, uint32_t *t) {
  orc_rlx r;
  orc_rlx_seed(&r, (unsigned long)seed, 202);
#define ORC_DRAW ((uint32_t)(0x7fffffff * orc_rlx_uniform(&r)))
  for (int i = 0; i < N / 2; ++i) {
    for (int j = 0; j < i; ++j) t[(size_t)i * N + j] = ORC_DRAW;
    for (int j = 0; j < i + 1; ++j) t[(size_t)j * N + i] = ORC_DRAW;
    for (int j = 0; j < i; ++j) t[(size_t)(N - 1 - i) * N + j] = ORC_DRAW;
    for (int j = 0; j < i + 1; ++j) t[(size_t)(N - 1 - j) * N + i] = ORC_DRAW;
    for (int j = 0; j < i; ++j) t[(size_t)i * N + (N - 1 - j)] = ORC_DRAW;
    for (int j = 0; j < i + 1; ++j) t[(size_t)j * N + (N - 1 - i)] = ORC_DRAW;
    for (int j = 0; j < i; ++j) t[(size_t)(N - 1 - i) * N + (N - 1 - j)] = ORC_DRAW;
    for (int j = 0; j < i + 1; ++j) t[(size_t)(N - 1 - j) * N + (N - 1 - i)] = ORC_DRAW;
  }
#undef ORC_DRAW
}

/* cube / sphere cut (main.c:428-441) */
static inline int orc_cut(const orc_params *p, double kx, double ky, double kz, double kmag) {
  /* same operation order as the reference: the Nyquist index sits exactly on
     the boundary, so the rounding of |k| Box / (2 PI) decides inclusion */
  if (p->SphereMode == 1) return kmag * p->Box / (2 * ORC_PI) > p->Nsample / 2;
  return fabs(kx) * p->Box / (2 * ORC_PI) > p->Nsample / 2 ||
         fabs(ky) * p->Box / (2 * ORC_PI) > p->Nsample / 2 ||
         fabs(kz) * p->Box / (2 * ORC_PI) > p->Nsample / 2;
}

/* ========================================================================= */
/* Gaussian potential (main.c:354-524)                                        */
/* ========================================================================= */
void orc_gauss_potential(const orc_params *p, const uint32_t *seedtable, double *phik) {
  int N = p->N, H = N / 2 + 1;
  double fac = pow(2 * ORC_PI / p->Box, 1.5);
  double shift = p->PhaseFlip == 1 ? ORC_PI : 0.0;
  memset(phik, 0, sizeof(double) * 2 * (size_t)N * N * H);
#pragma omp parallel for schedule(dynamic, 16)
  for (long col = 0; col < (long)N * N; ++col) {
    int i = (int)(col / N), j = (int)(col % N);
    orc_rlx r;
    orc_rlx_seed(&r, seedtable[(size_t)i * N + j], 202);
    for (int k = 0; k < N / 2; ++k) {
      double phase = orc_rlx_uniform(&r) * 2 * ORC_PI;
      phase += shift;
      double ampl;
      do
        ampl = orc_rlx_uniform(&r);
      while (ampl == 0);
      if (i == N / 2 || j == N / 2 || k == N / 2) continue;
      if (i == 0 && j == 0 && k == 0) continue;
      /* the reference forms kvec as index*2*PI/Box; reproduce that rounding */
      double kx, ky, kz;
      kx = (i < N / 2) ? i * 2 * ORC_PI / p->Box : -(N - i) * 2 * ORC_PI / p->Box;
      ky = (j < N / 2) ? j * 2 * ORC_PI / p->Box : -(N - j) * 2 * ORC_PI / p->Box;
      kz = (k < N / 2) ? k * 2 * ORC_PI / p->Box : -(N - k) * 2 * ORC_PI / p->Box;
      double k2 = kx * kx + ky * ky + kz * kz, km = sqrt(k2);
      if (orc_cut(p, kx, ky, kz, km)) continue;
      double phig = p->Anorm * exp(p->ns * log(km));
      if (p->ResBasis) {
        /* ResBasis/main.c:445-455: the switch has no break statements */
        switch (p->WhichSpectrum) {
          case 0:
            phig *= 1.0;
            /* fall through */
          case 1:
            phig *= (1.0 + p->A_res * cos(p->w_res * km + p->phi_res));
            /* fall through */
          case 2:
            phig *= (1.0 + p->A_res * cos(p->w_res * log(km) + p->phi_res));
        }
      }
      if (!p->FixedAmplitude) phig *= -log(ampl);
      phig = sqrt(phig) * fac * p->Beta / k2;
      double re = phig * cos(phase), im = phig * sin(phase);
      if (k > 0) {
        size_t c = ((size_t)i * N + j) * H + k;
        phik[2 * c] = re;
        phik[2 * c + 1] = im;
      } else if (i == 0) {
        if (j >= N / 2) continue;
        size_t c = ((size_t)0 * N + j) * H, cc = ((size_t)0 * N + (N - j)) * H;
        phik[2 * c] = re;
        phik[2 * c + 1] = im;
        phik[2 * cc] = re;
        phik[2 * cc + 1] = -im;
      } else {
        if (i >= N / 2) continue;
        int ii = N - i, jj = (N - j) % N;
        size_t c = ((size_t)i * N + j) * H, cc = ((size_t)ii * N + jj) * H;
        phik[2 * c] = re;
        phik[2 * c + 1] = im;
        phik[2 * cc] = re;
        phik[2 * cc + 1] = -im;
      }
    }
  }
}

/* ========================================================================= */
/* Modal non-Gaussian potential, reference structure (main.c:564-1063)        */
/* ========================================================================= */

/* per-cell wavenumber quantities shared by the filters */
typedef struct {
  double k1, kbar;
  int skip; /* DC or outside the cut */
} orc_kcell;

static void orc_kgrid(const orc_params *p, orc_kcell *kc) {
  int N = p->N, H = N / 2 + 1;
  double kmin = 2 * ORC_PI / p->Box, kmax = 2 * ORC_PI / p->Box * p->Nmax;
  double s = (4 - p->ns) / 3;
  double kmin_ns = pow(kmin, s), kmax_ns = pow(kmax, s);
#pragma omp parallel for schedule(static)
  for (long q = 0; q < (long)N * N; ++q) {
    int i = (int)(q / N), j = (int)(q % N);
    for (int k = 0; k < H; ++k) {
      double kx = (i < N / 2) ? i * 2 * ORC_PI / p->Box : -(N - i) * 2 * ORC_PI / p->Box;
      double ky = (j < N / 2) ? j * 2 * ORC_PI / p->Box : -(N - j) * 2 * ORC_PI / p->Box;
      double kz = (k < N / 2) ? k * 2 * ORC_PI / p->Box : -(N - k) * 2 * ORC_PI / p->Box;
      double k2 = kx * kx + ky * ky + kz * kz, k1 = sqrt(k2);
      orc_kcell *c = &kc[(size_t)q * H + k];
      c->k1 = k1;
      c->kbar = -1 + 2 * (pow(k1, s) - kmin_ns) / (kmax_ns - kmin_ns);
      c->skip = (i + j + k == 0) || orc_cut(p, kx, ky, kz, k1);
    }
  }
}

/* Legendre P_l(x), Bonnet recurrence (stands in for gsl_sf_legendre_Pl) */
static double orc_legendre(int l, double x) {
  if (l == 0) return 1.0;
  double p0 = 1.0, p1 = x;
  for (int n = 2; n <= l; ++n) {
    double p2 = ((2 * n - 1) * x * p1 - (n - 1) * p0) / n;
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

/* radial part of mode n: k^{s(n-3)} for n <= 3, (P_{n-1}(kbar) - X0[n-1]) / k^2
   for n >= 4 (main.c:833-860); the field filter is this times k^{4-ns}
   (main.c:606-637 writes it as k^{s(n-3)} k^{4-ns} and
   (P_{n-1} - X0) k^{2-ns}). */
static double orc_mode_out(int n, double k1, double kbar, double s, const double *x0) {
  if (n <= 3) return pow(k1, s * (n - 3.));
  return (orc_legendre(n - 1, kbar) - x0[n - 1]) / (k1 * k1);
}
static double orc_mode_in(int n, double k1, double kbar, double s, double ns, const double *x0) {
  if (n <= 3) return pow(k1, s * (n - 3.)) * pow(k1, 4 - ns);
  return (orc_legendre(n - 1, kbar) - x0[n - 1]) * pow(k1, 2 - ns);
}

static void orc_filter(const orc_params *p, const orc_kcell *kc, int n, const double *x0,
                       const double *phik, double *out) {
  int N = p->N, H = N / 2 + 1;
  double s = (4 - p->ns) / 3;
  size_t nc = (size_t)N * N * H;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)nc; ++c) {
    if (kc[c].skip) {
      out[2 * c] = out[2 * c + 1] = 0;
      continue;
    }
    double f = orc_mode_in(n, kc[c].k1, kc[c].kbar, s, p->ns, x0);
    out[2 * c] = f * phik[2 * c];
    out[2 * c + 1] = f * phik[2 * c + 1];
  }
}

void orc_modal_acc(const orc_params *p, int M, const double *alpha, const double *x0,
                   const double *phik, double *acc) {
  int N = p->N, H = N / 2 + 1;
  size_t nc = (size_t)N * N * H, nr = (size_t)N * N * N;
  double s = (4 - p->ns) / 3;
#define A3(a, b, c) alpha[((size_t)(a) * M + (b)) * M + (c)]
  orc_kcell *kc = (orc_kcell *)malloc(sizeof(orc_kcell) * nc);
  orc_kgrid(p, kc);
  long double *acc_re = (long double *)calloc(nc, sizeof(long double));
  long double *acc_im = (long double *)calloc(nc, sizeof(long double));
  double *spec = (double *)malloc(sizeof(double) * 2 * nc);
  double *fi = (double *)malloc(sizeof(double) * nr);
  double *fj = (double *)malloc(sizeof(double) * nr);
  double *prod = (double *)malloc(sizeof(double) * nr);
  double *g = (double *)malloc(sizeof(double) * 2 * nc);

  for (int ni = 0; ni < M; ++ni) {
    orc_filter(p, kc, ni, x0, phik, spec);
    orc_c2r_3d(N, spec, fi);
    for (int nj = ni; nj < M; ++nj) {
      int any = 0;
      for (int nk = nj; nk < M; ++nk)
        if (fabs(A3(ni, nj, nk)) > 0) any = 1;
      if (!any) continue; /* main.c:745-759 */
      orc_filter(p, kc, nj, x0, phik, spec);
      orc_c2r_3d(N, spec, fj);
#pragma omp parallel for schedule(static)
      for (long c = 0; c < (long)nr; ++c) prod[c] = fi[c] * fj[c];
      orc_r2c_3d(N, prod, g);
#pragma omp parallel for schedule(static)
      for (long c = 0; c < (long)nc; ++c) {
        if (kc[c].skip) continue;
        double w = 0;
        for (int nk = nj; nk < M; ++nk) w += A3(ni, nj, nk) * orc_mode_out(nk, kc[c].k1, kc[c].kbar, s, x0);
        acc_re[c] += (long double)(w * g[2 * c]);
        acc_im[c] += (long double)(w * g[2 * c + 1]);
      }
    }
  }
  /* counter-terms (main.c:888-1063): only (0,1) and (0,2) carry weight */
  double t012 = (M > 2 && A3(0, 1, 2) != 0) ? -A3(1, 1, 1) / A3(0, 1, 2) : 0;
  for (int ni = 0; ni <= 3; ++ni) {
    orc_filter(p, kc, ni, x0, phik, spec); /* n <= 3 filters need no X0 */
    orc_c2r_3d(N, spec, fi);
    for (int nj = ni; nj <= 3; ++nj) {
      orc_filter(p, kc, nj, x0, phik, spec);
      orc_c2r_3d(N, spec, fj);
#pragma omp parallel for schedule(static)
      for (long c = 0; c < (long)nr; ++c) prod[c] = fi[c] * fj[c];
      orc_r2c_3d(N, prod, g);
      double a012 = M > 2 ? A3(0, 1, 2) : 0;
#pragma omp parallel for schedule(static)
      for (long c = 0; c < (long)nc; ++c) {
        if (kc[c].skip) continue;
        double w = 0;
        if (ni == 0 && nj == 1) w += -a012 * t012 * pow(kc[c].k1, s * (2 - 3.0));
        if (ni == 0 && nj == 2) w += a012 * t012 * pow(kc[c].k1, s * (1 - 3.0));
        acc_re[c] += (long double)(w * g[2 * c]);
        acc_im[c] += (long double)(w * g[2 * c + 1]);
      }
    }
  }
  for (size_t c = 0; c < nc; ++c) {
    acc[2 * c] = (double)acc_re[c];
    acc[2 * c + 1] = (double)acc_im[c];
  }
  acc[0] = acc[1] = 0;
#undef A3
  free(kc);
  free(acc_re);
  free(acc_im);
  free(spec);
  free(fi);
  free(fj);
  free(prod);
  free(g);
}

/* The same accumulation regrouped by linearity of the DFT, restricted to the
   radial modes r with r_on[r] != 0 (the share of one part of a modal sum
   split over r): acc = sum_r rho_r r2c(g_r), g_r = sum_{p<=q<=r}
   alpha'_{pqr} f_p f_q, where alpha' is alpha on sorted triples plus the
   two counter-terms of main.c:1045-1050 (-a012 t012 f_0 f_1 into g_2,
   +a012 t012 f_0 f_2 into g_1).  Summed over all r it equals orc_modal_acc
   up to rounding; the sum over a partition of the r equals the unsplit
   one.  Checker of the split only (FP64, this file's own FFT). */
void orc_modal_acc_regrouped(const orc_params *p, int M, const double *alpha, const double *x0,
                             const double *phik, const int *r_on, double *acc) {
  int N = p->N, H = N / 2 + 1;
  size_t nc = (size_t)N * N * H, nr = (size_t)N * N * N;
  double s = (4 - p->ns) / 3;
#define A3(a, b, c) alpha[((size_t)(a) * M + (b)) * M + (c)]
  orc_kcell *kc = (orc_kcell *)malloc(sizeof(orc_kcell) * nc);
  orc_kgrid(p, kc);
  double *spec = (double *)malloc(sizeof(double) * 2 * nc);
  double *f = (double *)malloc(sizeof(double) * nr * M);
  double *gr = (double *)malloc(sizeof(double) * nr);
  double *G = (double *)malloc(sizeof(double) * 2 * nc);
  for (int n = 0; n < M; ++n) {
    orc_filter(p, kc, n, x0, phik, spec);
    orc_c2r_3d(N, spec, f + (size_t)n * nr);
  }
  double a012 = M > 2 ? A3(0, 1, 2) : 0, t012 = (M > 2 && a012 != 0) ? -A3(1, 1, 1) / a012 : 0;
  memset(acc, 0, sizeof(double) * 2 * nc);
  for (int r = 0; r < M; ++r) {
    if (!r_on[r]) continue;
    memset(gr, 0, sizeof(double) * nr);
    int any = 0;
    for (int a = 0; a <= r; ++a)
      for (int b = a; b <= r; ++b) {
        double c = A3(a, b, r);
        if (r == 2 && a == 0 && b == 1) c += -a012 * t012;
        if (c == 0) continue;
        any = 1;
        const double *fa = f + (size_t)a * nr, *fb = f + (size_t)b * nr;
#pragma omp parallel for schedule(static)
        for (long x = 0; x < (long)nr; ++x) gr[x] += c * fa[x] * fb[x];
      }
    if (r == 1 && a012 * t012 != 0) { /* +a012 t012 f_0 f_2 into g_1 */
      any = 1;
      const double c = a012 * t012, *fa = f, *fb = f + 2 * nr;
#pragma omp parallel for schedule(static)
      for (long x = 0; x < (long)nr; ++x) gr[x] += c * fa[x] * fb[x];
    }
    if (!any) continue;
    orc_r2c_3d(N, gr, G);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)nc; ++c) {
      if (kc[c].skip) continue;
      double w = orc_mode_out(r, kc[c].k1, kc[c].kbar, s, x0);
      acc[2 * c] += w * G[2 * c];
      acc[2 * c + 1] += w * G[2 * c + 1];
    }
  }
  acc[0] = acc[1] = 0;
#undef A3
  free(kc);
  free(spec);
  free(f);
  free(gr);
  free(G);
}

/* main.c:1094-1150 */
void orc_combine(const orc_params *p, double *phik, const double *acc, double *pot_gauss,
                 double *pot_ng) {
  int N = p->N, H = N / 2 + 1;
  size_t nc = (size_t)N * N * H, nr = (size_t)N * N * N;
  double *r = (double *)malloc(sizeof(double) * nr);
  double n3 = (double)((unsigned int)N * (unsigned int)N * (unsigned int)N);
  orc_c2r_3d(N, phik, r);
  if (pot_gauss) memcpy(pot_gauss, r, sizeof(double) * nr);
  orc_r2c_3d(N, r, phik);
  for (size_t c = 0; c < nc; ++c) {
    phik[2 * c] /= n3;
    phik[2 * c + 1] /= n3;
    phik[2 * c] += p->Fnl * acc[2 * c] / n3;
    phik[2 * c + 1] += p->Fnl * acc[2 * c + 1] / n3;
  }
  phik[0] = phik[1] = 0;
  orc_c2r_3d(N, phik, r);
  if (pot_ng) memcpy(pot_ng, r, sizeof(double) * nr);
  orc_r2c_3d(N, r, phik);
  for (size_t c = 0; c < 2 * nc; ++c) phik[c] /= n3;
  free(r);
}

/* ZA, 2LPT source, Poisson solve, CIC deconvolution, 6 c2r (main.c:1158-1381) */
void orc_lpt_fields(const orc_params *p, const double *phik, double *disp) {
  int N = p->N, H = N / 2 + 1;
  size_t nc = (size_t)N * N * H, nr = (size_t)N * N * N;
  double *cd = (double *)malloc(sizeof(double) * 2 * nc * 3);  /* cdisp[3] */
  double *cg = (double *)malloc(sizeof(double) * 2 * nc * 6);  /* cdigrad[6] */
  double *dg = (double *)malloc(sizeof(double) * nr * 6);
#pragma omp parallel for schedule(static)
  for (long q = 0; q < (long)N * N; ++q) {
    int i = (int)(q / N), j = (int)(q % N);
    for (int k = 0; k < H; ++k) {
      size_t c = (size_t)q * H + k;
      double kv[3];
      kv[0] = (i < N / 2) ? i * 2 * ORC_PI / p->Box : -(N - i) * 2 * ORC_PI / p->Box;
      kv[1] = (j < N / 2) ? j * 2 * ORC_PI / p->Box : -(N - j) * 2 * ORC_PI / p->Box;
      kv[2] = (k < N / 2) ? k * 2 * ORC_PI / p->Box : -(N - k) * 2 * ORC_PI / p->Box;
      double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2], km = sqrt(k2);
      double twb = orc_transfer(p, km) / p->Dplus / p->Beta;
      for (int a = 0; a < 3; ++a) {
        cd[2 * (a * nc + c) + 1] = kv[a] * twb * phik[2 * c];
        cd[2 * (a * nc + c)] = -kv[a] * twb * phik[2 * c + 1];
      }
      static const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
      for (int g = 0; g < 6; ++g) {
        const double *src = cd + 2 * (pa[g] * nc + c);
        cg[2 * (g * nc + c)] = -src[1] * kv[pb[g]];
        cg[2 * (g * nc + c) + 1] = src[0] * kv[pb[g]];
      }
    }
  }
  for (int g = 0; g < 6; ++g) orc_c2r_3d(N, cg + 2 * g * nc, dg + g * nr);
  double *src = dg + 3 * nr;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)nr; ++c) {
    double d0 = dg[c], d1 = dg[nr + c], d2 = dg[2 * nr + c], d3 = dg[3 * nr + c], d4 = dg[4 * nr + c],
           d5 = dg[5 * nr + c];
    src[c] = d0 * (d3 + d5) + d3 * d5 - d1 * d1 - d2 * d2 - d4 * d4;
  }
  double *cs = cg; /* reuse slot 0 for the source spectrum */
  orc_r2c_3d(N, src, cs);
  double *cd2 = cg + 2 * nc; /* slots 1..3 */
#pragma omp parallel for schedule(static)
  for (long q = 0; q < (long)N * N; ++q) {
    int i = (int)(q / N), j = (int)(q % N);
    for (int k = 0; k < H; ++k) {
      size_t c = (size_t)q * H + k;
      double kv[3];
      kv[0] = (i < N / 2) ? i * 2 * ORC_PI / p->Box : -(N - i) * 2 * ORC_PI / p->Box;
      kv[1] = (j < N / 2) ? j * 2 * ORC_PI / p->Box : -(N - j) * 2 * ORC_PI / p->Box;
      kv[2] = (k < N / 2) ? k * 2 * ORC_PI / p->Box : -(N - k) * 2 * ORC_PI / p->Box;
      double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
      double fx = 1, fy = 1, fz = 1;
      if (kv[0] != 0) {
        fx = (kv[0] * p->Box / 2) / N;
        fx = sin(fx) / fx;
      }
      if (kv[1] != 0) {
        fy = (kv[1] * p->Box / 2) / N;
        fy = sin(fy) / fy;
      }
      if (kv[2] != 0) {
        fz = (kv[2] * p->Box / 2) / N;
        fz = sin(fz) / fz;
      }
      double ff = 1 / (fx * fy * fz), smth = ff * ff;
      double sre = cs[2 * c], sim = cs[2 * c + 1];
      for (int a = 0; a < 3; ++a) {
        double *o = cd2 + 2 * (a * nc + c);
        if (k2 > 0.0) {
          o[0] = sim * kv[a] / k2;
          o[1] = -sre * kv[a] / k2;
        } else
          o[0] = o[1] = 0.0;
        cd[2 * (a * nc + c)] *= smth;
        cd[2 * (a * nc + c) + 1] *= smth;
        o[0] *= smth;
        o[1] *= smth;
      }
    }
  }
  for (int a = 0; a < 3; ++a) {
    orc_c2r_3d(N, cd + 2 * a * nc, disp + a * nr);
    orc_c2r_3d(N, cd2 + 2 * a * nc, disp + (3 + a) * nr);
  }
  free(cd);
  free(cg);
  free(dg);
}

/* main.c:1436-1516 and periodic_wrap main.c:1534-1536 */
void orc_readout(const orc_params *p, const double *disp, int64_t npart, float *pos, float *vel) {
  int N = p->N;
  size_t nr = (size_t)N * N * N;
  unsigned int nmesh3 = (unsigned int)N * (unsigned int)N * (unsigned int)N;
  double Box = p->Box;
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < npart; ++n) {
    double u = pos[3 * n] / Box * N, v = pos[3 * n + 1] / Box * N, w = pos[3 * n + 2] / Box * N;
    int i = (int)u, j = (int)v, k = (int)w;
    if (i == N) i = N - 1;
    if (i < 0) i = 0;
    if (j == N) j = N - 1;
    if (k == N) k = N - 1;
    u -= i;
    v -= j;
    w -= k;
    int ii = (i + 1) % N, jj = j + 1, kk = k + 1;
    if (jj >= N) jj -= N;
    if (kk >= N) kk -= N;
    double f1 = (1 - u) * (1 - v) * (1 - w), f2 = (1 - u) * (1 - v) * (w), f3 = (1 - u) * (v) * (1 - w),
           f4 = (1 - u) * (v) * (w), f5 = (u) * (1 - v) * (1 - w), f6 = (u) * (1 - v) * (w),
           f7 = (u) * (v) * (1 - w), f8 = (u) * (v) * (w);
#define ORC_AT(f, a, b, c) (f)[((size_t)(a) * N + (b)) * N + (c)]
    for (int ax = 0; ax < 3; ++ax) {
      const double *d1 = disp + ax * nr, *d2 = disp + (3 + ax) * nr;
      double dis = ORC_AT(d1, i, j, k) * f1 + ORC_AT(d1, i, j, kk) * f2 + ORC_AT(d1, i, jj, k) * f3 +
                   ORC_AT(d1, i, jj, kk) * f4 + ORC_AT(d1, ii, j, k) * f5 + ORC_AT(d1, ii, j, kk) * f6 +
                   ORC_AT(d1, ii, jj, k) * f7 + ORC_AT(d1, ii, jj, kk) * f8;
      double dis2 = ORC_AT(d2, i, j, k) * f1 + ORC_AT(d2, i, j, kk) * f2 + ORC_AT(d2, i, jj, k) * f3 +
                    ORC_AT(d2, i, jj, kk) * f4 + ORC_AT(d2, ii, j, k) * f5 + ORC_AT(d2, ii, j, kk) * f6 +
                    ORC_AT(d2, ii, jj, k) * f7 + ORC_AT(d2, ii, jj, kk) * f8;
      dis2 /= (float)nmesh3;
      pos[3 * n + ax] += dis - 3. / 7. * dis2;
      vel[3 * n + ax] = dis * p->vel_prefac - 3. / 7. * dis2 * p->vel_prefac2;
      double x = pos[3 * n + ax];
      pos[3 * n + ax] = fmod(fmod(x, Box) + Box, Box);
    }
#undef ORC_AT
  }
  (void)nr;
}

/* read_glass.c:181-214 (single task: every slab is local) */
void orc_tile_glass(const orc_params *p, const float *glass, int64_t nglass, double glass_box,
                    int tile, float *pos, int *ids) {
  int64_t count = 0;
  double Box = p->Box;
  for (int i = 0; i < tile; ++i)
    for (int j = 0; j < tile; ++j)
      for (int k = 0; k < tile; ++k)
        for (int64_t n = 0; n < nglass; ++n, ++count) {
          float x = glass[3 * n] / glass_box * (Box / tile) + i * (Box / tile);
          float y = glass[3 * n + 1] / glass_box * (Box / tile) + j * (Box / tile);
          float z = glass[3 * n + 2] / glass_box * (Box / tile) + k * (Box / tile);
          pos[3 * count] = x;
          pos[3 * count + 1] = y;
          pos[3 * count + 2] = z;
          if (ids) ids[count] = (int)(count + 1);
        }
}

int orc_run(const orc_params *p, int M, const double *alpha, const double *x0, int64_t npart,
            float *pos, float *vel, double *phik_out) {
  int N = p->N, H = N / 2 + 1;
  size_t nc = (size_t)N * N * H, nr = (size_t)N * N * N;
  if (p->Nmax < p->Nsample) return 200; /* main.c:200 */
  uint32_t *st = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)N * N);
  double *phik = (double *)malloc(sizeof(double) * 2 * nc);
  double *acc = (double *)malloc(sizeof(double) * 2 * nc);
  orc_seedtable(p->Seed, N, st);
  orc_gauss_potential(p, st, phik);
  orc_modal_acc(p, M, alpha, x0, phik, acc);
  orc_combine(p, phik, acc, NULL, NULL);
  free(acc);
  free(st);
  if (phik_out) memcpy(phik_out, phik, sizeof(double) * 2 * nc);
  double *disp = (double *)malloc(sizeof(double) * nr * 6);
  orc_lpt_fields(p, phik, disp);
  free(phik);
  orc_readout(p, disp, npart, pos, vel);
  free(disp);
  return 0;
}
