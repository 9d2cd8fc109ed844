// Internal declarations shared by the CUDA translation units of
// libaarambam_gpu.so (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/aarambam.h"
#include "cells.cuh"

namespace aar {

constexpr int kRowThreadsHost = 256;  // block size of the row kernels (rows.cuh kRowThreads)

// Host twin of keep_cell's cube bound.
int host_kcut(int nsample, double box);

// ----------------------------------------------------------- plan state
// ResBasis oscillation of the primordial spectrum.  power_osc: the factor
// in PowerSpec (ResBasis/power.c:240-260), used by the sigma8
// normalisation; one case per WhichSpectrum.  noise_osc: the factors on the
// per-cell power phig of the Gaussian potential (ResBasis/main.c:445-455),
// where the switch has no break, so WhichSpectrum 0 and 1 apply the linear
// and then the log oscillation and 2 the log one only.  Basis: no factor.
__host__ __device__ inline double power_osc(const aar_params& q, double k) {
  if (q.variant != AAR_VARIANT_RESBASIS) return 1.0;
  if (q.which_spectrum == 1) return 1 + q.a_res * cos(q.w_res * k + q.phi_res);
  if (q.which_spectrum == 2) return 1 + q.a_res * cos(q.w_res * log(k) + q.phi_res);
  return 1.0;
}
__host__ __device__ inline double noise_osc(const aar_params& q, double phig, double kmag) {
  if (q.variant != AAR_VARIANT_RESBASIS) return phig;
  if (q.which_spectrum <= 1) phig *= (1.0 + q.a_res * cos(q.w_res * kmag + q.phi_res));
  phig *= (1.0 + q.a_res * cos(q.w_res * log(kmag) + q.phi_res));
  return phig;
}

struct Plan {
  aar_params prm;
  std::string err;
  int N = 0, HP = 0, M = 0;
  Grid grid{};
  // host scalars (power.c:391-448, main.c:305-372)
  double Norm = 0, Anorm = 0, D0 = 0, Dplus = 0, InitTime = 0, Hubble = 0, Beta = 0;
  double vel_prefac = 0, vel_prefac2 = 0, kconv = 1;
  std::vector<double> logk, logT;  // sorted, normalised transfer table
  std::vector<double> alpha;       // M^3 symmetric
  std::vector<double> x0;          // M
  bool have_tables = false, have_transfer = false;
  // device resources (fused FP32 form)
  int dev = -1;
  int num_sms = 0;            // multiprocessors of the plan's device
  float2* d_phik = nullptr;   // Gaussian / total potential spectrum [N][N][HP]
  float2* d_work = nullptr;   // nwork fields [N][N][HP]
  int nwork = 0;
  uint32_t* d_seed = nullptr; // seed table [N][N]
  float2* d_twN = nullptr;    // exp(-2 pi i m / N), m < N
  float2* d_twH = nullptr;    // exp(-2 pi i m / (N/2)), m < N/2
  float* d_amp = nullptr;     // per n^2 noise amplitude
  float* d_twb = nullptr;     // per n^2 T(k) / (Dplus Beta)
  float* d_sinc = nullptr;    // per grid index: CIC window sin(x)/x
  float* d_isinc2 = nullptr;  // per grid index: 1 / (sin(x)/x)^2
  float* d_qtab = nullptr;    // [M][nsq] field filters q_p per n^2
  float* d_rtab = nullptr;    // [nsq][rtab_stride] radial parts rho_r per n^2 (r fastest)
  int rtab_stride = 0;
  int64_t nsq = 0;            // 3 (N/2)^2 + 1
  int qtab_m = 0;             // modes the tables were allocated for
  // field filters of the first modal pass over (|ky|, kz, |kx|), M (N/2+1)^3
  // floats (qcube_build); made on first use after each table change
  float* d_qcube = nullptr;
  int qcube_m = 0;
  bool qcube_stale = true;
  void* d_rlxpow = nullptr;   // skip-ahead powers (U576[32])
  int rlx_seg = 0;            // refills per seed-table thread
  // modal term list (device)
  void* d_terms = nullptr;
  std::vector<char> host_terms;  // the same term list on the host (kernel parameter of the row combine)
  int row_ls = 0;                // row-kernel line stride (float2) of this grid size
  int row_lt = 0;                // float2 slots of the row kernels' lane twiddle table
  void* jit = nullptr;           // run-time specialised modal row kernel (jit.cu), or null
  int jit_mode = 1;              // 0 off, 1 for N >= 256, 2 always
  int jit_minb = 0;              // resident row blocks per SM of the NVRTC kernel (0: by N)
  int jit_threads = 0;           // threads per block of the NVRTC row kernel (0: 256)
  int64_t xpass_group = 1;       // tiles per item group of the multi-output x passes (passes.cuh)
  int noise_one_draw = 0;        // noise columns one draw at a time (AAR_NOISE_ONE_DRAW=1, a check)
  std::string jit_status = "off";
  int nterms = 0, nr_active = 0;
  int modal_part = 0, modal_nparts = 1;  // split of the modal sum over r (this plan's part)
  // plain FP64 form
  void* plain = nullptr;
  // slab form (slab.cu)
  void* slab = nullptr;
  int last_launches = 0;      // kernels launched by the last run
  uint64_t generation = 0;    // bumped by every set_* call (captured graphs of the plan go stale)
  size_t used_bytes = 0;      // device bytes this plan holds
  // optional per-kernel timing: events recorded around every launch
  bool profiling = false;
  struct ProfRec {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<ProfRec> prof;
  std::vector<cudaEvent_t> event_pool;
  // adjoint: term / triple tables and coefficient sums (grown on demand)
  void* d_adj_scratch = nullptr;
  size_t adj_scratch_bytes = 0;
  // staging buffers of aar_run_host (grown on demand, kept for reuse)
  float* d_io = nullptr;
  int64_t io_cap = 0;
  cudaStream_t copy_stream = nullptr;  // side stream of the host-to-device copy
  cudaEvent_t copy_start = nullptr, copy_done = nullptr;
  // device-to-host of the particles, chunk by chunk behind the read-out
  static constexpr int kOutChunks = 8;
  int out_chunks = kOutChunks;  // chunks of the host read-out (1: one copy after the read-out)
  cudaStream_t out_stream[2] = {nullptr, nullptr};
  cudaEvent_t chunk_read[kOutChunks] = {}, out_done[2] = {nullptr, nullptr};
  // host-buffer glass runs: device glass, full-size Pos/Vel/ID staging, and
  // per chunk the event after its copy-out (the next read-out of the chunk
  // waits for it)
  float* d_glass = nullptr;
  int64_t glass_cap = 0;
  double* d_gscale = nullptr;  // glass_prepare: 3 nglass + tile products (read_glass.c:129-214)
  int64_t gscale_cap = 0;
  // lattice read-out (lattice_prepare): per-axis Lagrangian coordinates (+ a
  // flag word) and the parameter set they were made for
  float* d_lpa = nullptr;
  int lat_g = 0, lat_tile = 0;
  double lat_box = 0;
  bool lat_fused = false;
  bool disp_real = false;  // the work slots 0..5 hold the real displacement fields
  float* d_gout = nullptr;  // [npart][3] pos, then [npart][3] vel, then npart int32 ids
  int64_t gout_cap = 0;
  int64_t gout_last = -1;   // particle count of the last host-buffer glass call
  static constexpr int kGlassChunks = 16;
  cudaEvent_t gchunk_read[kGlassChunks] = {}, gchunk_free[kGlassChunks] = {};
};

// Records CUDA events around the kernels launched in its scope (when the
// plan's profiling is on), on the launching stream.
struct ProfScope {
  Plan* p;
  int idx = -1;
  cudaStream_t st;
  ProfScope(Plan* pl, const char* name, cudaStream_t s);
  ~ProfScope();
};

int plan_alloc(Plan* p, void** ptr, size_t bytes);
size_t terms_bytes();

const char* set_err(Plan* p, const std::string& e);

// launchers (return 0 or an error code; errors leave a message on the plan)
int launch_seedtable(Plan* p, uint32_t seed, uint32_t* d_out, cudaStream_t st);
int launch_noise_fp32(Plan* p, const uint32_t* d_seed, float2* d_phik, cudaStream_t st);
int launch_noise_fp64(Plan* p, const uint32_t* d_seed, double2* d_phik, int hp, cudaStream_t st);
int fused_prepare(Plan* p);
int qcube_build(Plan* p);
struct Term;
std::vector<std::vector<Term>> regrouped_terms(const std::vector<double>& alpha, int M);
std::vector<int> modal_partition(const std::vector<std::vector<Term>>& by_r, int nparts);
int fused_modal(Plan* p, cudaStream_t st);
// rows = false stops before the displacement rows (fused_rows_lattice does them)
int fused_lpt(Plan* p, cudaStream_t st, bool rows = true);
int lattice_prepare(Plan* p, int g, double glass_box, int tile, cudaStream_t st, bool& fused);
int lattice_glass(Plan* p, int g, double glass_box, float* d_glass, cudaStream_t st);
int fused_rows_lattice(Plan* p, int g, int tile, float* d_pos, float* d_vel, int* d_ids, int64_t row0, int64_t nrows,
                       cudaStream_t st);
int fused_readout(Plan* p, const float* d_lagr, int64_t npart, float* d_pos, float* d_vel, cudaStream_t st);
// glass_prepare makes the per-glass-particle and per-tile products of the
// Lagrangian positions (plan-owned scratch); fused_readout_glass then reads
// out particles n0 <= n < n1 (n1 < 0: all)
int glass_prepare(Plan* p, const float* d_glass, int64_t nglass, double glass_box, int tile, cudaStream_t st);
int fused_readout_glass(Plan* p, int64_t nglass, int tile, float* d_pos, float* d_vel, int* d_ids, cudaStream_t st,
                        int64_t n0 = 0, int64_t n1 = -1);
int plain_run(Plan* p, const float* d_lagr, int64_t npart, float* d_pos, float* d_vel, cudaStream_t st);
int plain_setup(Plan* p);
int plain_copy_field(Plan* p, int which, double* out, cudaStream_t st);
int plain_copy_spectrum(Plan* p, void* out, cudaStream_t st);
void plain_free(Plan* p);
inline bool is_plain(const aar_params& q) {
  return q.precision == AAR_PLAIN_FP64 || q.precision == AAR_PLAIN_FP64_REGROUPED;
}
// the FP32 forms share the plan's field layout (x-blocked rows of HP complex)
inline bool is_fp32(const aar_params& q) { return q.precision == AAR_FUSED_FP32 || q.precision == AAR_SLAB_FP32; }
int build_term_list(Plan* p);  // the regrouped term list (fused.cu)
RhoArgs rho_args(const Plan* p);
int slab_check(const aar_params& q, std::string& why);
int slab_setup(Plan* p);
int slab_run(Plan* p, cudaStream_t st);
void slab_free(Plan* p);
int fused_c2r(Plan* p, const float2* in, float* out, cudaStream_t st);
int fused_r2c(Plan* p, const float* in, float2* out, cudaStream_t st);
int fused_configure_xform(Plan* p);
// row copy between row orders (row_of), ncols elements of `elem` bytes per row
int copy_rows(Plan* p, void* dst, int64_t dst_ld, int dst_xb, const void* src, int64_t src_ld, int src_xb, int ncols,
              size_t elem, cudaStream_t st);
int noalloc_gaussian(Plan* p, void* d_out, cudaStream_t st);
int jit_prepare(Plan* p);
int jit_modal_rows(Plan* p, float2* work, int64_t fs, cudaStream_t st, int64_t nrows = -1);
int profile_modal_rows(Plan* p, float2* work, int64_t nrows, cudaStream_t st);
// the specialised modal accumulation of the same module; false when the
// plan has none (the generic k_modal_acc runs)
bool jit_has_acc(const Plan* p);
int jit_modal_acc(Plan* p, float2* phi, const float2* work, float fnl_n3, const RhoArgs& ra, cudaStream_t st);
void jit_free(Plan* p);
int adj_spectral(Plan* p, int op, int comp, int mode, const float2* in, float2* out, int accumulate,
                 cudaStream_t st);
int adj_source(Plan* p, const float* d, const float* gS, float* gd, cudaStream_t st);
int adj_products(Plan* p, const float* f, const float* gg, float* gf, double* galpha, cudaStream_t st);

}  // namespace aar

#define AAR_CUDA_TRY(p, call)                                                                  \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) {                                                                   \
      aar::set_err((p), std::string(#call) + ": " + cudaGetErrorString(e_));                  \
      return AAR_ERR_CUDA;                                                                     \
    }                                                                                          \
  } while (0)
