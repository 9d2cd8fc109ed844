// Tetrapyd points and separable mode bispectra shared by the Decomposer's
// kernels (decomp.cu: projections, residual, condition numbers; gram_tc.cu:
// the covariance on the tensor cores).
//
// Q_n(t) for mode n = (p1, p2, p3) and point t = (i1, i2, i3) is the
// symmetrised product (1/6) sum over the permutations (a, b, c) of
// (i1, i2, i3) of f_p1(k_a) f_p2(k_b) f_p3(k_c), as tetrapyd.c:136-152.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/aarambam.h"

namespace aar {

struct Tetra {
  const double* w;  // point weights
  const int *i1, *i2, *i3;
  int npts;
  const int *p1, *p2, *p3;
  int nmodes;
  const double* f;  // mode functions [p][k]
  int pmax, nk;
};

// Q_n at a point from three rows of the mode-function table
__device__ __forceinline__ double q_rows(const double* r1, const double* r2, const double* r3, int a, int b, int c) {
  const double m11 = r1[a], m12 = r1[b], m13 = r1[c];
  const double m21 = r2[a], m22 = r2[b], m23 = r2[c];
  const double m31 = r3[a], m32 = r3[b], m33 = r3[c];
  return (m11 * m22 * m33 + m11 * m23 * m32 + m12 * m21 * m33 + m12 * m23 * m31 + m13 * m21 * m32 +
          m13 * m22 * m31) /
         6.0;
}

__device__ __forceinline__ double q_eval(const double* f, int nk, int p1, int p2, int p3, int a, int b, int c) {
  return q_rows(f + p1 * nk, f + p2 * nk, f + p3 * nk, a, b, c);
}

inline Tetra make_tetra(const double* w, const int* i1, const int* i2, const int* i3, int npts, const int* p1,
                        const int* p2, const int* p3, int nmodes, const double* f, int pmax, int nk) {
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

inline bool tetra_ok(const Tetra& a) {
  return a.w && a.i1 && a.i2 && a.i3 && a.p1 && a.p2 && a.p3 && a.f && a.npts > 0 && a.nmodes > 0 && a.pmax > 0 &&
         a.nk > 0 && (size_t)a.pmax * a.nk * sizeof(double) <= 160 * 1024;
}

inline int tetra_status(cudaError_t e) {
  if (e == cudaSuccess) return AAR_OK;
  cudaGetLastError();
  return AAR_ERR_CUDA;
}

}  // namespace aar
