// Modal decomposition (the Decomposer's dense work) on the GPU, FP64.
//
// The reference builds the mode-bispectrum covariance ("QQ") and the
// shape projections ("QS") in C with OpenMP over modes
// (Aarambam/basis/tetrapyd.c:107-236 compute_mode_bispectra_covariance,
// :238-305 compute_QS) and does the rest of its orthogonal matching pursuit
// in numpy (Aarambam/basis/cmbbest.pyx:320-490), including one condition
// number per candidate mode and iteration through a full SVD
// (cmbbest.pyx:44-47, :443-446).  Here:
//
//   k_tetra_gram   QQ[n][m] = sum_t w_t Q_n(t) Q_m(t) as a tiled FP64 GEMM whose
//                  operand tiles are generated in shared memory from the
//                  1D mode functions (Q is never stored): a block owns a
//                  64 x 64 tile of QQ (upper triangle only) and one slice of
//                  the tetrapyd points; slices are summed by k_gram_reduce in
//                  a fixed order, so the result is deterministic;
//   k_tetra_project out[s][n] = sum_t X_s(t) w_t Q_n(t) (QS for the shape, QR for
//                  the residual), one warp per (mode, shape);
//   k_tetra_residual R(t) = S(t) - sum_j c_j Q_{n_j}(t) over the selected modes;
//   k_bordered_cond  cond of [[A, b_i], [b_i^T, c_i]] for every candidate i
//                  from the eigen-decomposition A = V diag(lam) V^T of the
//                  selected block: with z = V^T b_i the extreme eigenvalues
//                  are the outer roots of the secular equation
//                  c_i - mu - sum_j z_j^2 / (lam_j - mu) = 0, found by
//                  bisection (one warp per candidate).
//
// Q_n(t) for mode n = (p1, p2, p3) and point t = (i1, i2, i3) is the
// symmetrised product (1/6) sum over the permutations (a, b, c) of
// (i1, i2, i3) of f_p1(k_a) f_p2(k_b) f_p3(k_c), as tetrapyd.c:136-152.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/aarambam.h"

namespace aar {
namespace {

struct Tetra {
  const double* w;  // point weights
  const int *i1, *i2, *i3;
  int npts;
  const int *p1, *p2, *p3;
  int nmodes;
  const double* f;  // mode functions [p][k]
  int pmax, nk;
};

// Q_n at a point from the mode-function table in shared memory
__device__ __forceinline__ double q_eval(const double* f, int nk, int p1, int p2, int p3, int a, int b, int c) {
  const double* r1 = f + p1 * nk;
  const double* r2 = f + p2 * nk;
  const double* r3 = f + p3 * nk;
  const double m11 = r1[a], m12 = r1[b], m13 = r1[c];
  const double m21 = r2[a], m22 = r2[b], m23 = r2[c];
  const double m31 = r3[a], m32 = r3[b], m33 = r3[c];
  return (m11 * m22 * m33 + m11 * m23 * m32 + m12 * m21 * m33 + m12 * m23 * m31 + m13 * m21 * m32 +
          m13 * m22 * m31) /
         6.0;
}

constexpr int kGT = 64;   // modes per tile side
constexpr int kGC = 16;   // points per staged chunk
constexpr int kGThreads = 256;

// Grid: x = upper-triangular tile pair, y = point slice.  Output: partial
// sums part[slice][n][m] for the block's tile (n tile <= m tile).
__global__ void __launch_bounds__(kGThreads) k_tetra_gram(Tetra a, const int2* __restrict__ pairs, int slice_len,
                                                          double* __restrict__ part) {
  extern __shared__ double sm[];
  double* f = sm;                              // [pmax][nk]
  double* qa = f + a.pmax * a.nk;              // [kGC][kGT]  w_t Q_n(t)
  double* qb = qa + kGC * kGT;                 // [kGC][kGT]  Q_m(t)
  int* ti = (int*)(qb + kGC * kGT);            // [3][kGC]
  for (int i = threadIdx.x; i < a.pmax * a.nk; i += kGThreads) f[i] = a.f[i];
  const int2 tp = pairs[blockIdx.x];
  const int n0 = tp.x * kGT, m0 = tp.y * kGT;
  const int t0 = blockIdx.y * slice_len;
  const int t1 = min(a.npts, t0 + slice_len);
  // each thread: a 4 x 4 block of the tile (rows ty*4.., cols tx*4..)
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  // operand generation: thread -> (mode r, points) pairs
  for (int tc = t0; tc < t1; tc += kGC) {
    __syncthreads();  // previous chunk consumed (and f loaded on the first pass)
    if (threadIdx.x < kGC) {
      const int t = tc + threadIdx.x;
      const bool in = t < t1;
      ti[threadIdx.x] = in ? a.i1[t] : -1;
      ti[kGC + threadIdx.x] = in ? a.i2[t] : 0;
      ti[2 * kGC + threadIdx.x] = in ? a.i3[t] : 0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * kGT * kGC; e += kGThreads) {
      const int side = e / (kGT * kGC);
      const int r = e % kGT, c = (e / kGT) % kGC;
      const int n = (side ? m0 : n0) + r;
      double v = 0.0;
      const int x = ti[c];
      if (x >= 0 && n < a.nmodes) {
        v = q_eval(f, a.nk, a.p1[n], a.p2[n], a.p3[n], x, ti[kGC + c], ti[2 * kGC + c]);
        if (!side) v *= a.w[tc + c];
      }
      (side ? qb : qa)[c * kGT + r] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int c = 0; c < kGC; ++c) {
      double u[4], v[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) u[i] = qa[c * kGT + ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = qb[c * kGT + tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(u[i], v[j], acc[i][j]);
    }
  }
  const int64_t nm = a.nmodes;
  double* out = part + (int64_t)blockIdx.y * nm * nm;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + ty * 4 + i, m = m0 + tx * 4 + j;
      if (n < a.nmodes && m < a.nmodes) out[(int64_t)n * nm + m] = acc[i][j];
    }
}

// QQ = sum over slices (slice order fixed), mirrored into the lower triangle
__global__ void k_gram_reduce(const double* __restrict__ part, int nslices, int nmodes, double* __restrict__ qq) {
  const int64_t nm = nmodes;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nm * nm; e += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(e / nm), m = (int)(e % nm);
    if (n > m) continue;  // the lower triangle is the mirror
    double s = 0.0;
    for (int k = 0; k < nslices; ++k) s += part[(int64_t)k * nm * nm + e];
    qq[e] = s;
    qq[(int64_t)m * nm + n] = s;
  }
}

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

Tetra make_tetra(const double* w, const int* i1, const int* i2, const int* i3, int npts, const int* p1, const int* p2,
                 const int* p3, int nmodes, const double* f, int pmax, int nk) {
  Tetra a;
  a.w = w;
  a.i1 = i1;
  a.i2 = i2;
  a.i3 = i3;
  a.npts = npts;
  a.p1 = p1;
  a.p2 = p2;
  a.p3 = p3;
  a.nmodes = nmodes;
  a.f = f;
  a.pmax = pmax;
  a.nk = nk;
  return a;
}

bool tetra_ok(const Tetra& a) {
  return a.w && a.i1 && a.i2 && a.i3 && a.p1 && a.p2 && a.p3 && a.f && a.npts > 0 && a.nmodes > 0 && a.pmax > 0 &&
         a.nk > 0 && (size_t)a.pmax * a.nk * sizeof(double) <= 160 * 1024;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return AAR_OK;
  cudaGetLastError();
  return AAR_ERR_CUDA;
}

}  // namespace
}  // namespace aar

using namespace aar;

extern "C" {

size_t aar_tetra_covariance_scratch_bytes(int32_t tetra_npts, int32_t n_modes) {
  const int64_t slices = (tetra_npts + 65535) / 65536;
  const int64_t ntile = (n_modes + kGT - 1) / kGT;
  return (size_t)slices * n_modes * n_modes * sizeof(double) + (size_t)ntile * (ntile + 1) / 2 * sizeof(int2);
}

int aar_tetra_covariance(double* d_cov, const double* d_tetra_weights, const int32_t* d_i1, const int32_t* d_i2,
                         const int32_t* d_i3, int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2,
                         const int32_t* d_p3, int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max,
                         int32_t k_npts, void* d_scratch, size_t scratch_bytes, void* stream) {
  const Tetra a = make_tetra(d_tetra_weights, d_i1, d_i2, d_i3, tetra_npts, d_p1, d_p2, d_p3, n_modes, d_mode_evals,
                             mode_p_max, k_npts);
  if (!d_cov || !d_scratch || !tetra_ok(a)) return AAR_ERR_ARG;
  if (scratch_bytes < aar_tetra_covariance_scratch_bytes(tetra_npts, n_modes)) return AAR_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int slice_len = 65536;
  const int nslices = (tetra_npts + slice_len - 1) / slice_len;
  const int ntile = (n_modes + kGT - 1) / kGT;
  const int npairs = ntile * (ntile + 1) / 2;
  double* part = (double*)d_scratch;
  int2* pairs = (int2*)(part + (size_t)nslices * n_modes * n_modes);
  // tile pairs (n tile <= m tile), made on the host
  int2* hp = new int2[npairs];
  int q = 0;
  for (int x = 0; x < ntile; ++x)
    for (int y = x; y < ntile; ++y) hp[q++] = make_int2(x, y);
  cudaError_t e = cudaMemcpyAsync(pairs, hp, sizeof(int2) * npairs, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  delete[] hp;
  if (e != cudaSuccess) return cuda_status(e);
  const size_t smem = sizeof(double) * ((size_t)mode_p_max * k_npts + 2 * kGC * kGT) + sizeof(int) * 3 * kGC;
  if ((e = cudaFuncSetAttribute(k_tetra_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
    return cuda_status(e);
  k_tetra_gram<<<dim3(npairs, nslices), kGThreads, smem, st>>>(a, pairs, slice_len, part);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
  k_gram_reduce<<<1024, 256, 0, st>>>(part, nslices, n_modes, d_cov);
  return cuda_status(cudaGetLastError());
}

int aar_tetra_QS(double* d_QS, const double* d_S, int32_t n_shapes, const double* d_tetra_weights, const int32_t* d_i1,
                 const int32_t* d_i2, const int32_t* d_i3, int32_t tetra_npts, const int32_t* d_p1, const int32_t* d_p2,
                 const int32_t* d_p3, int32_t n_modes, const double* d_mode_evals, int32_t mode_p_max, int32_t k_npts,
                 void* stream) {
  const Tetra a = make_tetra(d_tetra_weights, d_i1, d_i2, d_i3, tetra_npts, d_p1, d_p2, d_p3, n_modes, d_mode_evals,
                             mode_p_max, k_npts);
  if (!d_QS || !d_S || n_shapes < 1 || !tetra_ok(a)) return AAR_ERR_ARG;
  const size_t smem = sizeof(double) * (size_t)mode_p_max * k_npts;
  cudaError_t e = cudaFuncSetAttribute(k_tetra_project, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  const int64_t warps = (int64_t)n_modes * n_shapes;
  k_tetra_project<<<(unsigned)((warps * 32 + 255) / 256), 256, smem, (cudaStream_t)stream>>>(a, d_S, n_shapes, d_QS);
  return cuda_status(cudaGetLastError());
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
  if (e != cudaSuccess) return cuda_status(e);
  k_tetra_residual<<<(unsigned)((tetra_npts + 255) / 256), 256, smem, (cudaStream_t)stream>>>(a, d_S, d_sel, d_coef,
                                                                                                n_sel, d_R);
  return cuda_status(cudaGetLastError());
}

int aar_bordered_cond(double* d_cond, const double* d_lam, int32_t k, const double* d_Z, const double* d_c,
                      int32_t n_cand, void* stream) {
  if (!d_cond || !d_lam || !d_Z || !d_c || k < 1 || n_cand < 0) return AAR_ERR_ARG;
  if (n_cand == 0) return AAR_OK;
  k_bordered_cond<<<(unsigned)(((int64_t)n_cand * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_lam, k, d_Z, d_c,
                                                                                                     n_cand, d_cond);
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
