// Modal decomposition (the Decomposer's dense work) on the GPU, FP64.
//
// The reference builds the mode-bispectrum covariance ("QQ") and the
// shape projections ("QS") in C with OpenMP over modes
// (Aarambam/basis/tetrapyd.c:107-236 compute_mode_bispectra_covariance,
// :238-305 compute_QS) and does the rest of its orthogonal matching pursuit
// in numpy (Aarambam/basis/cmbbest.pyx:320-490), including one condition
// number per candidate mode and iteration through a full SVD
// (cmbbest.pyx:44-47, :443-446).  Here (the covariance is in gram_tc.cu,
// on the tensor cores):
//
//   k_tetra_project out[s][n] = sum_t X_s(t) w_t Q_n(t) (QS for the shape, QR for
//                  the residual), one warp per (mode, shape);
//   k_tetra_residual R(t) = S(t) - sum_j c_j Q_{n_j}(t) over the selected modes;
//   k_modes_project, k_modes_residual  the same from the mode bispectra Q[n][t]
//                  stored once per basis (aar_tetra_modes, gram_tc.cu): the
//                  pursuit's per-step projection reads 8 bytes per (mode,
//                  point) instead of evaluating the 3 x 3 permanent in FP64;
//   k_bordered_cond  cond of [[A, b_i], [b_i^T, c_i]] for every candidate i
//                  from the eigen-decomposition A = V diag(lam) V^T of the
//                  selected block: with z = V^T b_i the extreme eigenvalues
//                  are the outer roots of the secular equation
//                  c_i - mu - sum_j z_j^2 / (lam_j - mu) = 0, found by
//                  bisection (one warp per candidate).
//
// Q_n(t) is evaluated on the fly from the 1D mode functions (tetra.cuh).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/aarambam.h"
#include "tetra.cuh"

namespace aar {
namespace {

// out[s][n] = sum_t X_s(t) w_t Q_n(t); one warp per (n, s)
__global__ void k_tetra_project(Tetra a, const double* __restrict__ X, int nshapes, double* __restrict__ out) {
  extern __shared__ double f[];
  for (int i = threadIdx.x; i < a.pmax * a.nk; i += blockDim.x) f[i] = a.f[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wid >= (int64_t)a.nmodes * nshapes) return;
  const int n = (int)(wid % a.nmodes), s = (int)(wid / a.nmodes);
  const int p1 = a.p1[n], p2 = a.p2[n], p3 = a.p3[n];
  const double* x = X + (int64_t)s * a.npts;
  double acc = 0.0;
  for (int t = lane; t < a.npts; t += 32)
    acc = fma(x[t] * a.w[t], q_eval(f, a.nk, p1, p2, p3, a.i1[t], a.i2[t], a.i3[t]), acc);
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[(int64_t)s * a.nmodes + n] = acc;
}

// R(t) = S(t) - sum_j coef[j] Q_{sel[j]}(t), j ascending
__global__ void k_tetra_residual(Tetra a, const double* __restrict__ S, const int* __restrict__ sel,
                                 const double* __restrict__ coef, int nsel, double* __restrict__ R) {
  extern __shared__ double f[];
  for (int i = threadIdx.x; i < a.pmax * a.nk; i += blockDim.x) f[i] = a.f[i];
  __syncthreads();
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < a.npts; t += gridDim.x * blockDim.x) {
    const int x = a.i1[t], y = a.i2[t], z = a.i3[t];
    double sum = 0.0;
    for (int j = 0; j < nsel; ++j) {
      const int n = sel[j];
      sum += coef[j] * q_eval(f, a.nk, a.p1[n], a.p2[n], a.p3[n], x, y, z);
    }
    R[t] = S[t] - sum;
  }
}

// The same two sums from stored mode bispectra Q[n][t] (row stride ldq):
// the terms, their order and the warp reduction of k_tetra_project and
// k_tetra_residual, with Q read instead of evaluated.  Projection: one warp
// per mode, a block of ceil(modes / SMs) warps (one wave of blocks, the rows
// spread evenly: the sum is FP64-bound on GB300, about 2 FP64 multiply-adds
// per clock per SM); per tile of 512 points the products x_t w_t are formed
// once into shared memory for the block's rows and every lane issues its 16
// loads of Q before their multiply-adds (lane l adds the points l, l + 32,
// ... in ascending order, as k_tetra_project).
constexpr int kProjTile = 512;

__global__ void __launch_bounds__(1024) k_modes_project(const double* __restrict__ Q, long long ldq,
                                                        const double* __restrict__ w, int npts, int nmodes,
                                                        const double* __restrict__ X, double* __restrict__ out) {
  __shared__ double xw[2][kProjTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = blockIdx.x * (int)(blockDim.x >> 5) + warp, s = blockIdx.y;
  const bool row = n < nmodes;
  const double* q = Q + (size_t)(row ? n : 0) * ldq;
  const double* x = X + (int64_t)s * npts;
  double acc = 0.0;
  int buf = 0;
  for (int t0 = 0; t0 < npts; t0 += kProjTile, buf ^= 1) {
    for (int i = threadIdx.x; i < kProjTile; i += blockDim.x) {
      const int t = t0 + i;
      xw[buf][i] = t < npts ? x[t] * w[t] : 0.0;
    }
    __syncthreads();  // xw[buf] complete; xw[buf ^ 1] is rewritten only after the next barrier
    if (row) {
      if (t0 + kProjTile <= npts) {
        double qv[kProjTile / 32];
#pragma unroll
        for (int j = 0; j < kProjTile / 32; ++j) qv[j] = q[t0 + lane + 32 * j];
#pragma unroll
        for (int j = 0; j < kProjTile / 32; ++j) acc = fma(xw[buf][lane + 32 * j], qv[j], acc);
      } else {
        for (int j = 0; t0 + lane + 32 * j < npts; ++j) acc = fma(xw[buf][lane + 32 * j], q[t0 + lane + 32 * j], acc);
      }
    }
  }
  if (!row) return;
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[(int64_t)s * nmodes + n] = acc;
}

__global__ void k_modes_residual(const double* __restrict__ Q, long long ldq, int npts, const double* __restrict__ S,
                                 const int* __restrict__ sel, const double* __restrict__ coef, int nsel,
                                 double* __restrict__ R) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npts; t += gridDim.x * blockDim.x) {
    double sum = 0.0;
    for (int j = 0; j < nsel; ++j) sum += coef[j] * Q[(size_t)sel[j] * ldq + t];
    R[t] = S[t] - sum;
  }
}

// g(mu) = c - mu - sum_j z_j^2 / (lam_j - mu), warp-reduced.  `pole` is the
// index of the bracket end that is an eigenvalue of A (its term is skipped
// when evaluating at that end and z_pole = 0).
__device__ __forceinline__ double secular(const double* lam, const double* z, int k, double c, double mu) {
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  for (int j = lane; j < k; j += 32) {
    const double d = lam[j] - mu;
    const double zz = z[j] * z[j];
    if (zz != 0.0) s += zz / d;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return c - mu - s;
}

// cond_i = lambda_max / lambda_min of the bordered matrix of candidate i.
// lam: eigenvalues of A ascending [k]; Z: V^T b_i, column i at Z + i*k;
// c: diagonal entries c_i.  One warp per candidate.
__global__ void k_bordered_cond(const double* __restrict__ lam, int k, const double* __restrict__ Z,
                                const double* __restrict__ c, int ncand, double* __restrict__ cond) {
  const int lane = threadIdx.x & 31;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= ncand) return;
  const double* z = Z + i * k;
  const double ci = c[i];
  double zn = 0.0;
  for (int j = lane; j < k; j += 32) zn += z[j] * z[j];
#pragma unroll
  for (int o = 16; o; o >>= 1) zn += __shfl_xor_sync(0xffffffffu, zn, o);
  zn = sqrt(zn);
  const double l1 = lam[0], lk = lam[k - 1];
  const double z1 = z[0], zk = z[k - 1];
  // smallest eigenvalue: root of g below l1 (g decreasing there); none when
  // z_1 = 0 and g(l1) >= 0, then l1 itself
  double lmin;
  if (z1 == 0.0 && secular(lam, z, k, ci, l1) >= 0.0) {
    lmin = l1;
  } else {
    double lo = fmin(l1, ci) - zn - 1e-300, hi = l1;
    for (int it = 0; it < 2000; ++it) {
      const double mid = 0.5 * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      if (secular(lam, z, k, ci, mid) > 0.0) lo = mid;
      else hi = mid;
    }
    lmin = 0.5 * (lo + hi);
  }
  // largest eigenvalue: root of g above lk; none when z_k = 0 and g(lk) <= 0
  double lmax;
  if (zk == 0.0 && secular(lam, z, k, ci, lk) <= 0.0) {
    lmax = lk;
  } else {
    double lo = lk, hi = fmax(lk, ci) + zn + 1e-300;
    for (int it = 0; it < 2000; ++it) {
      const double mid = 0.5 * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      if (secular(lam, z, k, ci, mid) > 0.0) lo = mid;
      else hi = mid;
    }
    lmax = 0.5 * (lo + hi);
  }
  if (lane == 0) cond[i] = lmin > 0.0 ? lmax / lmin : INFINITY;
}

}  // namespace
}  // namespace aar

using namespace aar;

extern "C" {

int aar_tetra_QS(double* d_QS, const double* d_S, int32_t n_shapes, const double* d_tetra_weights, const int32_t* d_i1,
                 const int32_t* d_i2, const int32_t* d_i3, int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2,
                 const int32_t* d_p3, int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max, int32_t k_npts,
                 void* stream) {
  const Tetra a = make_tetra(d_tetra_weights, d_i1, d_i2, d_i3, tetra_npts, d_p1, d_p2, d_p3, n_modes, d_mode_evals,
                             mode_p_max, k_npts);
  if (!d_QS || !d_S || n_shapes < 1 || !tetra_ok(a)) return AAR_ERR_ARG;
  const size_t smem = sizeof(double) * (size_t)mode_p_max * k_npts;
  cudaError_t e = cudaFuncSetAttribute(k_tetra_project, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return tetra_status(e);
  const int64_t warps = (int64_t)n_modes * n_shapes;
  k_tetra_project<<<(unsigned)((warps * 32 + 255) / 256), 256, smem, (cudaStream_t)stream>>>(a, d_S, n_shapes, d_QS);
  return tetra_status(cudaGetLastError());
}

int aar_tetra_residual(double* d_R, const double* d_S, const int32_t* d_sel, const double* d_coef, int32_t n_sel,
                       const double* d_tetra_weights, const int32_t* d_i1, const int32_t* d_i2, const int32_t* d_i3,
                       int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2, const int32_t* d_p3,
                       int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max, int32_t k_npts, void* stream) {
  const Tetra a = make_tetra(d_tetra_weights, d_i1, d_i2, d_i3, tetra_npts, d_p1, d_p2, d_p3, n_modes, d_mode_evals,
                             mode_p_max, k_npts);
  if (!d_R || !d_S || n_sel < 0 || (n_sel > 0 && (!d_sel || !d_coef)) || !tetra_ok(a)) return AAR_ERR_ARG;
  const size_t smem = sizeof(double) * (size_t)mode_p_max * k_npts;
  cudaError_t e = cudaFuncSetAttribute(k_tetra_residual, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return tetra_status(e);
  k_tetra_residual<<<(unsigned)((tetra_npts + 255) / 256), 256, smem, (cudaStream_t)stream>>>(a, d_S, d_sel, d_coef,
                                                                                                n_sel, d_R);
  return tetra_status(cudaGetLastError());
}

int aar_modes_project(double* d_out, const double* d_X, int32_t n_shapes, const double* d_tetra_weights,
                      const double* d_Q, int64_t ldq, int32_t tetra_npts, int32_t n_modes, void* stream) {
  if (!d_out || !d_X || !d_tetra_weights || !d_Q || n_shapes < 1 || tetra_npts < 1 || n_modes < 1 ||
      ldq < tetra_npts)
    return AAR_ERR_ARG;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms < 1)
      sms = 1;
  }
  int wpb = (n_modes + sms - 1) / sms;  // warps (modes) per block
  wpb = wpb < 1 ? 1 : (wpb > 32 ? 32 : wpb);
  k_modes_project<<<dim3((n_modes + wpb - 1) / wpb, n_shapes), wpb * 32, 0, (cudaStream_t)stream>>>(
      d_Q, ldq, d_tetra_weights, tetra_npts, n_modes, d_X, d_out);
  return tetra_status(cudaGetLastError());
}

int aar_modes_residual(double* d_R, const double* d_S, const int32_t* d_sel, const double* d_coef, int32_t n_sel,
                       const double* d_Q, int64_t ldq, int32_t tetra_npts, void* stream) {
  if (!d_R || !d_S || !d_Q || n_sel < 0 || (n_sel > 0 && (!d_sel || !d_coef)) || tetra_npts < 1 || ldq < tetra_npts)
    return AAR_ERR_ARG;
  k_modes_residual<<<(unsigned)((tetra_npts + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      d_Q, ldq, tetra_npts, d_S, d_sel, d_coef, n_sel, d_R);
  return tetra_status(cudaGetLastError());
}

int aar_bordered_cond(double* d_cond, const double* d_lam, int32_t k, const double* d_Z, const double* d_c,
                      int32_t n_cand, void* stream) {
  if (!d_cond || !d_lam || !d_Z || !d_c || k < 1 || n_cand < 0) return AAR_ERR_ARG;
  if (n_cand == 0) return AAR_OK;
  k_bordered_cond<<<(unsigned)(((int64_t)n_cand * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_lam, k, d_Z, d_c,
                                                                                                     n_cand, d_cond);
  return tetra_status(cudaGetLastError());
}

}  // extern "C"
