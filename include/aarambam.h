/*
 * aarambam.h -- C ABI of libaarambam_gpu.so, the GB300 (sm_103a) implementation
 * of Aarambam's initial-condition path: seed-table white noise -> modal
 * non-Gaussian potential -> ZA + 2LPT displacements -> particles.
 *
 * The reference exposes this path as a process: `Aarambam-2LPT-Basis
 * <paramfile>` (Aarambam/LPT/Basis/cli.py:5-10) runs the C/MPI executable
 * whose work happens in main() (Aarambam/LPT/Basis/main.c:53-102) and
 * displacement_fields() (main.c:149-1532).  Each entry point below replaces
 * one piece of that executable; the comment names the piece.  The reference
 * has no in-process library interface, so the binding a maintainer adds is
 * the ctypes layer of the Python package (aarambam_gb300/_lib.py) behind the
 * same CLI name.
 *
 * Conventions: every call returns AAR_OK (0) or an error code (never exits);
 * aar_last_error() gives the message.  Device pointers are caller-owned CUDA
 * allocations on the plan's device, or page-locked host memory
 * (cudaHostAlloc / cudaHostRegister), which the kernels address directly over
 * the host link -- how the slab form writes 1536^3 particles that do not fit
 * beside its fields; `stream` is a cudaStream_t (NULL = the legacy default
 * stream).  A plan owns its scratch and is not thread-safe;
 * distinct plans may run concurrently on distinct streams.
 */
#ifndef AARAMBAM_H
#define AARAMBAM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AAR_OK 0
#define AAR_ERR_ARG 1           /* invalid argument or unsupported size */
#define AAR_ERR_CUDA 2          /* a CUDA call failed */
#define AAR_ERR_OOM 3           /* device allocation refused (or over mem_limit_bytes) */
#define AAR_ERR_STATE 4         /* tables / transfer function not set */
#define AAR_ERR_NMAX 200        /* Nmax < Nsample (main.c:200 assert) */
#define AAR_ERR_TRANSFER 1111   /* first log10 k of the transfer table >= -4.6 (power.c:117-122) */
#define AAR_ERR_TRANSFER_DUP 777 /* two transfer rows with equal k (power.c:205-206) */

/* Arithmetic of the run. */
#define AAR_FUSED_FP32 0  /* own FFTs, fused filters/products/accumulation, FP32 */
#define AAR_PLAIN_FP64 1  /* cuFFT Z2D/D2Z + separate pointwise kernels, FP64, the reference's
                             loop structure (M + 2P + 41 transforms) */
#define AAR_PLAIN_FP64_REGROUPED 2 /* as AAR_PLAIN_FP64 with the modal sum regrouped by linearity
                                      (M c2r + R r2c; <= 2M + 13 transforms in all) */
#define AAR_SLAB_FP32 3  /* the fused form's FP32 arithmetic streamed over nslab strided real-space
                            x-slabs, for grids whose fused fields do not fit one GPU (1536^3): the
                            filtered fields and products exist per slab, the transform stages are
                            recomputed per slab ((Nmesh/nslab, Nmesh, Nmesh) cuFFT FP32 transforms
                            of spectra folded along x), the modal sum is accumulated compensated
                            across slabs; even Nmesh = 8..2048, a multiple of 4 */

/* Which executable's power spectrum the plan follows. */
#define AAR_VARIANT_BASIS 0    /* 2LPTBasis: P(k) = Norm k^ns T^2 (LPT/Basis/power.c:240-265) */
#define AAR_VARIANT_RESBASIS 1 /* 2LPTResBasis: P(k) with the oscillation A_res, w_res, phi_res
                                  (LPT/ResBasis/power.c:240-260, main.c:445-455) */

/* The parameter-file values the path uses (read_param.c:25-184). */
typedef struct aar_params {
  int32_t nmesh, nsample, nmax, seed;
  double box;
  double omega, omega_lambda, hubble_param, sigma8, primordial_index, redshift, fnl;
  double unit_length_in_cm, unit_mass_in_g, unit_velocity_in_cm_per_s;
  double input_spectrum_unit_length_in_cm;
  int32_t fixed_amplitude, phase_flip, sphere_mode;
  int32_t precision;        /* AAR_FUSED_FP32, AAR_PLAIN_FP64, AAR_PLAIN_FP64_REGROUPED or AAR_SLAB_FP32 */
  int64_t mem_limit_bytes;  /* refuse plan allocations beyond this (0 = no cap) */
  int32_t variant;          /* AAR_VARIANT_BASIS or AAR_VARIANT_RESBASIS */
  int32_t which_spectrum;   /* WhichSpectrum: 0 for Basis; 0, 1 or 2 for ResBasis */
  double a_res, w_res, phi_res; /* ResBasis oscillation (ResBasis/read_param.c:88-99) */
  int32_t noise_fp64;       /* fused form: 1 = RNG-to-amplitude step (phase, -ln u, sqrt, amplitude)
                               in FP64 with the reference's formula, rounded to float at the end;
                               0 (default) = FP32 from the exact 48-bit uniforms */
  int32_t nslab;            /* AAR_SLAB_FP32: number of x-slabs S (Nmesh % S == 0, Nmesh / S >= 2);
                               device memory ~ 1 + max(2 + (M+R)/S, 7 + 6/S) fields of Nmesh^2
                               (Nmesh/2+1) complex floats (M modes, R active r): 8.75 fields, 128 GB
                               at 1536^3 with 20 modes and S = 8; ignored by the other forms */
} aar_params;

/* Host scalars of the set-up: power.c:391-448 (Norm = sigma8 normalisation,
   Anorm, D0, Dplus), set_units main.c:1547-1552 (Hubble), main.c:305-307
   (velocity prefactors), main.c:372 (Beta). */
typedef struct aar_scalars {
  double norm, anorm, d0, dplus, init_time, hubble, beta, vel_prefac, vel_prefac2;
} aar_scalars;

typedef struct aar_plan aar_plan;

/* Create a plan for one grid size on the current CUDA device
   (replaces initialize_ffts main.c:1556-1599 and the parameter broadcast). */
int aar_plan_create(const aar_params* prm, aar_plan** out);

/* Allocate now what the plan's runs need (the plain forms' FP64 fields,
   tables and cuFFT plans, the fused form's work fields), so that the first
   run does no set-up.  Needs tables and transfer function.  Optional: a run
   without it prepares itself.  (The reference sets up inside
   displacement_fields, main.c:149-212, 1556-1599.) */
int aar_plan_prepare(aar_plan* plan);

/* Coefficient tables: alpha as a symmetric [M][M][M] array (as the reference
   stores it after reading AlphaTable.dat, main.c:213-247), X0 as [M] (first
   value column of AiTable.dat, main.c:249-289).  aar_set_tables and
   aar_set_transfer synchronise the device before they rewrite the plan's
   device tables, so runs of the plan still in flight finish with the old
   values. */
int aar_set_tables(aar_plan* plan, const double* alpha_sym, const double* x0, int32_t n_modes);

/* Tabulated transfer function, raw (k, T) rows in h/Mpc (read_transfer_table
   power.c:66-153 plus initialize_powerspectrum power.c:391-448, which needs
   the table for the sigma8 normalisation).  Computes the host scalars. */
int aar_set_transfer(aar_plan* plan, const double* k, const double* t, int32_t n);

int aar_get_scalars(const aar_plan* plan, aar_scalars* out);

/* Change the realisation seed (the parameter-file Seed). */
int aar_set_seed(aar_plan* plan, int32_t seed);

/* The whole of displacement_fields() (main.c:149-1532): particles at the
   Lagrangian positions d_lagr_pos (float32 [npart][3]) are moved; positions
   and velocities (float32 [npart][3]) are written to d_pos / d_vel, which may
   alias d_lagr_pos. */
int aar_run(aar_plan* plan, const float* d_lagr_pos, int64_t npart, float* d_pos, float* d_vel, void* stream);

/* As aar_run, with the Lagrangian positions made on the device from a glass
   tiled tile^3 times (read_glass.c:129-214); also writes the particle IDs
   (int32, 1-based, read_glass.c:183-211).  npart = nglass * tile^3. */
int aar_run_glass(aar_plan* plan, const float* d_glass_pos, int64_t nglass, double glass_box, int32_t tile,
                  float* d_pos, float* d_vel, int32_t* d_ids, void* stream);

/* As aar_run_glass for the regular glass_n^3 lattice glass -- per-axis
   coordinates (float)(i * glass_box / glass_n), the particle order of
   read_glass.c:181-214, the layout of the reference's default glass
   (defaults/dummy_glass_dmonly_64.dat, 64^3) -- tiled tile^3 times, with no
   glass array.  When glass_n * tile == Nmesh and every tiled coordinate
   falls exactly on a grid point by the reference's FP64 cell coordinate
   u = Pos / Box * Nmesh (main.c:1444-1446; checked on the device once per
   parameter set, one synchronisation), each particle reads only the grid
   value under it, as the reference does, and the read-out is fused into the
   displacement rows: the real displacement fields are then not kept
   (aar_copy_field / aar_stage_readout need aar_stage_lpt).  The general
   read-out's FP32 two-float coordinate can leave fractions of ~1e-7 at
   such points; its results agree with the fused ones to float rounding.
   Otherwise the general read-out runs.  Positions, velocities and IDs as
   aar_run_glass (d_ids may be NULL). */
int aar_run_lattice(aar_plan* plan, int32_t glass_n, double glass_box, int32_t tile, float* d_pos, float* d_vel,
                    int32_t* d_ids, void* stream);

/* aar_run with HOST buffers: copies in, runs on `stream`, copies out and
   synchronises.  The device staging buffers are owned by the plan (allocated
   on first use, grown when npart grows, freed with the plan). */
int aar_run_host(aar_plan* plan, const float* h_lagr_pos, int64_t npart, float* h_pos, float* h_vel, void* stream);

/* aar_run_glass with HOST buffers, on the reference's own dataflow: the
   glass (nglass float32 [3] positions as read from the GlassFile,
   read_glass.c:43-84) is copied in, the Lagrangian positions are made on the
   device from it tiled tile^3 times (read_glass.c:129-214), and the
   particles are read out in chunks whose positions, velocities and (when
   h_ids is not NULL) IDs go to the host while later chunks are read out --
   no N^3 Lagrangian array crosses to the GPU.  A glass that is the regular
   lattice (as aar_run_lattice describes) gets aar_run_lattice's fused
   read-out, in chunks of tile rows.  npart = nglass * tile^3;
   h_pos / h_vel float32 [npart][3], h_ids int32 [npart].  Returns when the
   results are in the host buffers.  The plan owns the device staging
   (grown on demand, freed with the plan).  Fused form only. */
int aar_run_glass_host(aar_plan* plan, const float* h_glass, int64_t nglass, double glass_box, int32_t tile,
                       float* h_pos, float* h_vel, int32_t* h_ids, void* stream);

/* aar_run_glass_host without the wait: the fields and the read-out are
   enqueued behind earlier work on `stream`, the copies to the host on the
   plan's own two side streams, and the call returns.  The host buffers hold
   the results once aar_wait_host_copies(plan) has returned; until then they
   must stay valid and must not be read.  A following call on the same plan
   computes the next realisation's fields on `stream` while this one's
   particles are still on their way out; each staging chunk is handed over by
   an event, so the next read-out of a chunk waits only for that chunk's
   copy.  Use pinned host memory (cudaHostAlloc / cudaHostRegister): copies
   from pageable memory are not asynchronous. */
int aar_run_glass_host_async(aar_plan* plan, const float* h_glass, int64_t nglass, double glass_box, int32_t tile,
                             float* h_pos, float* h_vel, int32_t* h_ids, void* stream);
/* Block until every copy to the host that the plan's aar_run_glass_host*
   calls have enqueued is done. */
int aar_wait_host_copies(aar_plan* plan);

/* ---- stage entry points (the same work as aar_run, split; used by tests) ---- */

/* Seed table of main.c:317-349 (uint32 [N][N]) for the plan's seed. */
int aar_seedtable(aar_plan* plan, uint32_t* d_out, void* stream);
/* Gaussian potential spectrum (main.c:354-524) into the plan's spectrum. */
int aar_stage_noise(aar_plan* plan, void* stream);
/* Modal non-Gaussian potential and combination (main.c:564-1151). */
int aar_stage_modal(aar_plan* plan, void* stream);
/* ZA + 2LPT displacement fields (main.c:1156-1381). */
int aar_stage_lpt(aar_plan* plan, void* stream);
/* Particle read-out (main.c:1436-1516). */
int aar_stage_readout(aar_plan* plan, const float* d_lagr_pos, int64_t npart, float* d_pos, float* d_vel,
                      void* stream);
/* Read-out with the Lagrangian positions made from a tiled glass, as in
   aar_run_glass (read_glass.c:129-214, main.c:1436-1516). */
int aar_stage_readout_glass(aar_plan* plan, const float* d_glass_pos, int64_t nglass, double glass_box, int32_t tile,
                            float* d_pos, float* d_vel, int32_t* d_ids, void* stream);
/* Copy the plan's current potential spectrum to d_out as complex
   [N][N][N/2+1] (interleaved re, im; float32 for AAR_FUSED_FP32, float64
   for the plain forms, whose spectrum is the total one after a run). */
int aar_copy_spectrum(aar_plan* plan, void* d_out, void* stream);
/* Copy displacement field `which` (0..2: ZA x,y,z; 3..5: 2LPT x,y,z as the
   reference holds them before its 1/N^3, main.c:1378-1431) to d_out, real
   [N][N][N]: float32 for AAR_FUSED_FP32, float64 for the plain forms (after
   a run). */
int aar_copy_field(aar_plan* plan, int32_t which, void* d_out, void* stream);

/* No counterpart in the reference.  The Gaussian potential spectrum of the
   plan's seed (what aar_stage_noise + aar_copy_spectrum give for the fused
   form) written straight into the caller's buffer d_out, complex
   [N][N][N/2+1]: float32 pairs for AAR_FUSED_FP32 plans, float64 pairs for
   the plain FP64 plans.  Needs the transfer function set (aar_set_transfer);
   the coefficient tables are not used.
   The call allocates nothing: no cudaMalloc / cudaFree and no allocating
   library.  It is for callers that own the device-memory budget themselves,
   such as a simulation code that reserved HBM for its particle and mesh
   arrays up front, or a framework whose caching allocator holds the device
   memory: there a library cudaMalloc can fail once the memory is reserved,
   and a cudaFree synchronises the whole device and stalls the caller's other
   streams.  The seed table it needs between its two kernels lives in a
   static 4 MiB device array of the library (Nmesh <= 1024); larger Nmesh is
   rejected with AAR_ERR_ARG and a message.  The plan's own spectrum and
   seed-table buffers are not touched.  d_out need not be zeroed (the call
   clears it on the stream) and nothing in the scratch has to start at zero.
   The first call on a device resolves the scratch address
   (cudaGetSymbolAddress); make that first call before any stream capture
   begins.  Under CUDA's lazy module loading, that first call may also be
   the one that loads the library's noise module on the device, which
   reserves the 4 MiB array and the module's code: that one-time load is the
   only device memory the entry point ever causes to be reserved, so make
   the first call during set-up (or run any other call of the library on the
   device first).  The cached address belongs to the device's primary
   context and stays valid for the life of the process; after
   cudaDeviceReset, or from a non-primary context, it is stale.  There is
   one scratch per device, so calls that overlap on one device (other
   streams or host threads) race on it: serialise them. */
int aar_gaussian_spectrum_noalloc(aar_plan* plan, void* d_out, void* stream);

/* The plan's own 3-D transforms with FFTW's rfftwnd conventions
   (unnormalised; c2r drops the imaginary parts that the kz = 0 and kz = N/2
   planes would need to be Hermitian), as used on every rfftwnd_mpi call site
   of main.c.  Fused form only; complex data as in aar_copy_spectrum, real
   data float32 [N][N][N].  The plan's first work field is used as scratch. */
int aar_c2r(aar_plan* plan, const void* d_in, float* d_out, void* stream);
int aar_r2c(aar_plan* plan, const float* d_in, void* d_out, void* stream);

/* ---- modal decomposition (the Decomposer's dense FP64 work) ----
   Stateless entry points on device pointers, with the arguments of the
   reference's C kernels (Aarambam/basis/tetrapyd.h, bound from
   cmbbest.pyx:35-47): tetrapyd points (weights, i1 >= i2 >= i3 indices into
   the 1D k grid), 3D mode indices p1 >= p2 >= p3, and the 1D mode functions
   mode_evals[mode_p_max][k_npts] (mode_p_max * k_npts * 8 <= 160 KiB).
   Q_n(t) is the symmetrised product of tetrapyd.c:136-152.  Return AAR_OK,
   AAR_ERR_ARG or AAR_ERR_CUDA. */

/* Scratch bytes aar_tetra_covariance needs (the mode bispectra, their bf16
   digit tiles and the per-range int64 sums). */
size_t aar_tetra_covariance_scratch_bytes(int32_t tetra_npts, int32_t n_modes);

/* cov[n][m] = sum_t w_t Q_n(t) Q_m(t), [n_modes][n_modes], symmetric,
   FP64-accurate on the bf16 tensor cores (the operands cut into eight 8-bit
   digits, exact level sums, int64 fixed-point accumulation; deterministic).
   Synchronises the stream.  Replaces compute_mode_bispectra_covariance
   (tetrapyd.c:107-236). */
int aar_tetra_covariance(double* d_cov, const double* d_tetra_weights, const int32_t* d_i1, const int32_t* d_i2,
                         const int32_t* d_i3, int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2,
                         const int32_t* d_p3, int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max,
                         int32_t k_npts, void* d_scratch, size_t scratch_bytes, void* stream);

/* QS[s][n] = sum_t S[s][t] w_t Q_n(t), S [n_shapes][tetra_npts].
   Replaces compute_QS (tetrapyd.c:238-305). */
int aar_tetra_QS(double* d_QS, const double* d_S, int32_t n_shapes, const double* d_tetra_weights,
                 const int32_t* d_i1, const int32_t* d_i2, const int32_t* d_i3, int32_t tetra_npts,
                 const int32_t* d_p1, const int32_t* d_p2, const int32_t* d_p3, int32_t n_modes,
                 const double* d_mode_evals, int32_t mode_p_max, int32_t k_npts, void* stream);

/* R[t] = S[t] - sum_j coef[j] Q_{sel[j]}(t), j ascending: the matching-
   pursuit residual (cmbbest.pyx:433) without storing Q. */
int aar_tetra_residual(double* d_R, const double* d_S, const int32_t* d_sel, const double* d_coef, int32_t n_sel,
                       const double* d_tetra_weights, const int32_t* d_i1, const int32_t* d_i2, const int32_t* d_i3,
                       int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2, const int32_t* d_p3,
                       int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max, int32_t k_npts,
                       void* stream);

/* Stored mode bispectra: Q[n][t] = Q_n(t) made once per basis and kept by
   the caller ([n_modes][ldq] doubles, ldq = aar_tetra_modes_ld(tetra_npts),
   the point count rounded up to a multiple of 128; zeros beyond tetra_npts,
   16-byte aligned), read by the aar_modes_* entry points instead of
   evaluating Q_n(t) again (the matching pursuit projects on every mode at
   every step). */
int64_t aar_tetra_modes_ld(int32_t tetra_npts);
int aar_tetra_modes(double* d_Q, int64_t ldq, const int32_t* d_i1, const int32_t* d_i2, const int32_t* d_i3,
                    int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2, const int32_t* d_p3,
                    int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max, int32_t k_npts, void* stream);

/* aar_tetra_covariance from stored mode bispectra (ldq as above). */
size_t aar_modes_covariance_scratch_bytes(int32_t tetra_npts, int32_t n_modes);
int aar_modes_covariance(double* d_cov, const double* d_Q, int64_t ldq, const double* d_tetra_weights,
                         int32_t tetra_npts, int32_t n_modes, void* d_scratch, size_t scratch_bytes, void* stream);

/* aar_tetra_QS and aar_tetra_residual from stored mode bispectra: the same
   terms, order and reductions, so the same results. */
int aar_modes_project(double* d_out, const double* d_X, int32_t n_shapes, const double* d_tetra_weights,
                      const double* d_Q, int64_t ldq, int32_t tetra_npts, int32_t n_modes, void* stream);
int aar_modes_residual(double* d_R, const double* d_S, const int32_t* d_sel, const double* d_coef, int32_t n_sel,
                       const double* d_Q, int64_t ldq, int32_t tetra_npts, void* stream);

/* Condition numbers lambda_max / lambda_min of the bordered symmetric
   matrices [[A, b_i], [b_i^T, c_i]], i < n_cand, given the eigenvalues lam
   (ascending, k of them) of the PSD matrix A = V diag(lam) V^T, the rows
   Z[i] = (V^T b_i)^T [n_cand][k] and c.  Replaces the per-candidate
   np.linalg.cond of get_cond (cmbbest.pyx:44-47, :443-446). */
int aar_bordered_cond(double* d_cond, const double* d_lam, int32_t k, const double* d_Z, const double* d_c,
                      int32_t n_cand, void* stream);

/* ---- adjoint of the fused chain (no counterpart in the reference) ----
   Building blocks of a reverse-mode pass over white noise w -> Gaussian
   potential -> modal non-Gaussian potential -> ZA + 2LPT displacements
   (aarambam_gb300/adjoint.py drives them with aar_c2r / aar_r2c).  Complex
   data are [N][N][N/2+1] float2, real fields [N][N][N] float. */
#define AAR_ADJ_OP_ONE 0    /* 1 */
#define AAR_ADJ_OP_GAUSS 1  /* noise amplitude on the cells the noise draw writes (main.c:405-459) */
#define AAR_ADJ_OP_Q 2      /* field filter q_comp(k) of mode comp (main.c:580-637) */
#define AAR_ADJ_OP_RHO 3    /* Fnl/N^3 rho_comp(k) of mode comp (main.c:825-867, 1111-1116) */
#define AAR_ADJ_OP_HESS 4   /* -k_a k_b T/(D Beta), comp 0..5 = 00 01 02 11 12 22 (main.c:1238-1277) */
#define AAR_ADJ_OP_PSI1 5   /* i k_a T/(D Beta) smth, comp = axis (main.c:1180-1216, 1332-1367) */
#define AAR_ADJ_OP_PSI2 6   /* -i k_a/k^2 smth, comp = axis (main.c:1311-1368) */
/* Write d_in into the plan's potential spectrum (what aar_stage_noise
   would have written), so that aar_stage_modal / aar_stage_lpt continue from
   a caller-made Gaussian potential. */
int aar_set_spectrum(aar_plan* plan, const void* d_in, void* stream);
/* d_out (+)= M(F) d_in per cell, F the factor of (op, comp); mode 0: F,
   1: conj(F) w, 2: conj(F)/w, 3: conj(F), with w = 1 on the kz = 0 and N/2
   planes and 2 elsewhere (c2r^T = w r2c, r2c^T = c2r(./w)). */
int aar_adj_spectral(aar_plan* plan, int32_t op, int32_t comp, int32_t mode, const void* d_in, void* d_out,
                     int32_t accumulate, void* stream);
/* Transpose of the 2LPT source: d_hess and d_out are 6 real fields
   (00 01 02 11 12 22), d_gsource the source gradient. */
int aar_adj_source(aar_plan* plan, const float* d_hess, const float* d_gsource, float* d_out, void* stream);
/* Transpose of the modal products g_r = sum alpha' f_p f_q: d_f the M fields
   f_p, d_gg the M gradients of g_r (zero for unused r), d_gf (out) the M
   gradients of f_p, d_galpha (out, FP64 [M][M][M]) the gradient with respect
   to alpha at every sorted index p <= q <= r (the counter-terms of
   main.c:1045-1050 included); synchronises the stream. */
int aar_adj_products(aar_plan* plan, const float* d_f, const float* d_gg, float* d_gf, double* d_galpha, void* stream);

/* ---- batches (no counterpart in the reference, whose executable makes one
   realisation per process) ----
   Several fused plans (realisations with their own seed, coefficient table,
   mode count and buffers; one device) run as one CUDA graph.  The first
   aar_batch_run captures every plan's aar_run work as a branch of the graph
   (one stream per plan, so small kernels of different realisations overlap);
   later runs replay it with one graph launch on `stream`.  The graph is
   captured again when a buffer pointer, a particle count or a plan
   (aar_set_seed / aar_set_tables / aar_set_transfer) changes.  Arrays are
   indexed by plan; the plans' profiling is suspended while capturing. */
typedef struct aar_batch aar_batch;
int aar_batch_create(aar_plan* const* plans, int32_t nplans, aar_batch** out);
int aar_batch_run(aar_batch* batch, const float* const* d_lagr_pos, const int64_t* npart, float* const* d_pos,
                  float* const* d_vel, void* stream);
/* Kernels in one replay of the batch graph. */
int aar_batch_launch_count(const aar_batch* batch);
const char* aar_batch_last_error(const aar_batch* batch);
void aar_batch_destroy(aar_batch* batch);

/* ---- the modal sum split over radial modes (no counterpart in the
   reference, which splits the grid into x-slabs over MPI ranks instead,
   main.c:1556-1599) ----
   acc = sum_r rho_r r2c(g_r) is a sum of independent terms once the Gaussian
   potential is known, so nparts cooperating plans (one per GPU) each
   regenerate the Gaussian potential from the seed and sum their own share
   of the r; the shares add up to the unsplit sum.
   aar_modal_partition: which part each r goes to (-1: r without terms),
   balanced by the number of product terms per r; host only.
   aar_set_modal_partition: this plan's part; its aar_stage_modal then adds
   only its share, Fnl / N^3 sum_{r in part} rho_r r2c(g_r), to the Gaussian
   potential.  The caller sums (spectrum after the modal stage - Gaussian
   spectrum) over the parts, adds it to the Gaussian spectrum on one plan
   (aar_set_spectrum) and continues there with aar_stage_lpt (see
   aarambam_gb300/modal_split.py).  Fused form; (0, 1) is the unsplit sum. */
int aar_modal_partition(const double* alpha_sym, int32_t n_modes, int32_t nparts, int32_t* part_of_r);
int aar_set_modal_partition(aar_plan* plan, int32_t part, int32_t nparts);

/* Run-time specialised modal row and accumulation kernels (no counterpart
   in the reference): mode 0 off, 1 (default) for Nmesh >= 256, 2 always.
   Both are compiled with NVRTC for the plan's alpha-term structure when the tables
   are set (a new table with the same nonzero pattern only updates its
   coefficients); when compiling or loading fails the generic kernel stays
   in use and aar_jit_status says why ("on", "off" or the reason). */
int aar_set_jit(aar_plan* plan, int32_t mode);
const char* aar_jit_status(const aar_plan* plan);

/* Schedule autotuner (no counterpart in the reference): times the field
   stages of this plan on its device for each candidate schedule -- the row
   kernel generic or NVRTC-specialised with 2 or 3 resident blocks per SM of
   256 threads (or 2 of 320 where ten warps need fewer rounds over the modes),
   and the item grouping of the multi-output x passes -- and keeps the
   fastest for the plan's later runs.  Needs tables and transfer function;
   overwrites the plan's spectrum and fields.  `report` (may be NULL)
   receives one line per candidate, the chosen one marked '*'. */
int aar_autotune(aar_plan* plan, char* report, int32_t len, void* stream);

/* Profiling harness (no counterpart in the reference): the plan's modal row
   kernel (the NVRTC one when in use) on nrows rows of caller fields, d_work
   = M + 1 fields of nrows rows of HP = round_up(N/2+1, 8) complex float
   each, field stride nrows * HP.  What a full modal stage runs on N^2 rows,
   on a case small enough for a counter capture. */
int aar_profile_modal_rows(aar_plan* plan, void* d_work, int64_t nrows, void* stream);

/* Per-kernel timing: when enabled, CUDA events are recorded on the launching
   stream around every kernel; aar_profile_report synchronises the device and
   writes "kernel,launches,total_ms" lines for everything recorded since the
   last report into buf (NUL-terminated). */
int aar_profile_enable(aar_plan* plan, int32_t on);
int aar_profile_report(aar_plan* plan, char* buf, int32_t len);

/* Device bytes the plan holds now: fields, tables, staging and scratch it
   allocated (not the caller's buffers). */
int64_t aar_plan_device_bytes(const aar_plan* plan);

/* Number of kernels the last aar_run* / stage call launched. */
int aar_last_launch_count(const aar_plan* plan);
const char* aar_last_error(const aar_plan* plan);
void aar_plan_destroy(aar_plan* plan);
int aar_version(void);

#ifdef __cplusplus
}
#endif
#endif
