/*
 * CPU oracle for the Aarambam initial-condition path (test infrastructure only).
 *
 * A plain-C, FP64 restatement of the reference 2LPT executable's algorithm
 * (Aarambam/LPT/Basis/main.c:149-1532, power.c, read_glass.c) used as the
 * checker for the CUDA implementation and as the timed CPU baseline.  It is
 * never linked into, loaded by, or called from the product library.
 *
 * Third-party arithmetic the reference takes from libraries that are not part
 * of the reference checkout is restated here from the published algorithms:
 *   - GSL gsl_rng_ranlxd1 (RANLUX, Luscher 1994; GSL's double-precision
 *     variant with base 2^48, lags (12,5), luxury 202), pinned by GSL's
 *     known-answer values (seed 1, 10000th output);
 *   - GSL gsl_sf_legendre_Pl (Bonnet recurrence);
 *   - FFTW 2.1.5 rfftwnd c2r / r2c (unnormalised 3D real DFT, complex axes
 *     first for c2r, imaginary parts of the kz=0 and kz=N/2 entries dropped by
 *     the final 1-D complex-to-real step).
 */
#ifndef AAR_ORACLE_H
#define AAR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RANLUX (GSL ranlxd1 / ranlxd2) ---- */
typedef struct {
  int64_t x[12]; /* 48-bit integers, x[0] oldest after each refill */
  int64_t carry;
  int pos;
  int luxury; /* 202 for ranlxd1, 397 for ranlxd2 */
} orc_rlx;

void orc_rlx_seed(orc_rlx *s, unsigned long seed, int luxury);
double orc_rlx_uniform(orc_rlx *s);          /* gsl_rng_uniform */
unsigned long orc_rlx_get(orc_rlx *s);       /* gsl_rng_get */

/* ---- cosmology / host scalar set-up (power.c:391-448, main.c:305-372) ---- */
typedef struct {
  double Omega, OmegaLambda, HubbleParam, Sigma8, PrimordialIndex, Redshift;
  double UnitLength_in_cm, UnitMass_in_g, UnitVelocity_in_cm_per_s;
  double InputSpectrum_UnitLength_in_cm;
} orc_cosmo;

typedef struct {
  int N, Nsample, Nmax, Seed;
  double Box, ns, Fnl;
  int FixedAmplitude, PhaseFlip, SphereMode;
  /* derived scalars */
  double Norm, Anorm, D0, Dplus, InitTime, Hubble, Beta, vel_prefac, vel_prefac2;
  double kconv; /* InputSpectrum_UnitLength_in_cm / UnitLength_in_cm */
  int ntrans;
  double *logk, *logT; /* sorted, logT normalised to the first entry */
  /* 2LPTResBasis (LPT/ResBasis): ResBasis = 1 adds the oscillation
     A_res, w_res, phi_res selected by WhichSpectrum; 0 = 2LPTBasis */
  int ResBasis, WhichSpectrum;
  double A_res, w_res, phi_res;
} orc_params;

/* Returns 0 on success, nonzero error code on a bad transfer table. */
int orc_setup(orc_params *p, const orc_cosmo *c, int ntrans, const double *k, const double *T);
void orc_free(orc_params *p);
double orc_transfer(const orc_params *p, double k);

/* ---- FFT (FP64, unnormalised) ---- */
/* real: [N][N][N] unpadded; complex: [N][N][N/2+1] interleaved re,im */
void orc_c2r_3d(int N, const double *cin, double *rout);
void orc_r2c_3d(int N, const double *rin, double *cout);

/* ---- the path ---- */
void orc_seedtable(int seed, int N, uint32_t *table);
/* Gaussian potential: complex [N][N][N/2+1] */
void orc_gauss_potential(const orc_params *p, const uint32_t *seedtable, double *phik);
/* Non-Gaussian accumulator (reference pair-loop structure), complex [N][N][N/2+1].
   alpha: symmetric [M][M][M]; x0: [M]. */
void orc_modal_acc(const orc_params *p, int M, const double *alpha, const double *x0,
                   const double *phik, double *acc);
void orc_modal_acc_regrouped(const orc_params *p, int M, const double *alpha, const double *x0,
                             const double *phik, const int *r_on, double *acc);
/* Total potential in place: phik <- phik + Fnl*acc/N^3 with the reference's
   two real-space round trips; DC zeroed.  If pot_gauss / pot_ng are non-null
   they receive the real-space fields the reference dumps (write_phi). */
void orc_combine(const orc_params *p, double *phik, const double *acc, double *pot_gauss,
                 double *pot_ng);
/* ZA + 2LPT displacement fields: disp[6][N][N][N] (psi1 x,y,z then psi2
   x,y,z; psi2 is the unnormalised c2r output as in the reference). */
void orc_lpt_fields(const orc_params *p, const double *phik, double *disp);
/* Trilinear read-out of particles (main.c:1440-1516); pos/vel float[3*n]. */
void orc_readout(const orc_params *p, const double *disp, int64_t npart, float *pos, float *vel);
/* Lagrangian positions from a glass tiled tile^3 times (read_glass.c:129-214) */
void orc_tile_glass(const orc_params *p, const float *glass, int64_t nglass, double glass_box,
                    int tile, float *pos, int *ids);

/* Convenience: the whole path.  pos is input (Lagrangian) and output. */
int orc_run(const orc_params *p, int M, const double *alpha, const double *x0, int64_t npart,
            float *pos, float *vel, double *phik_out /* optional: total potential */);

#ifdef __cplusplus
}
#endif
#endif
