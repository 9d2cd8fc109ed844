// Run-time specialised modal row kernel.
//
// The generic row kernel (fused.cu, ModalRowOp) reads its term list at run
// time, so every term costs four shared-memory loads (f_p and f_q at two
// positions).  Here the kernel is generated for the plan's term structure
// and compiled with NVRTC for sm_103a: a thread loads the M values f_p of
// its positions into registers once and every term is two multiply-adds with
// compile-time register indices; the coefficients sit in the module's
// __constant__ memory, so a new alpha table with the same nonzero pattern
// (same terms) only rewrites them.  The FFT and row code are the same
// headers the library is built from (fft.cuh, rows.cuh, embedded at build
// time).  If NVRTC or the module load fails, the plan keeps the generic
// kernel and records why.
#include <cuda_runtime.h>
#include <nvrtc.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "aar_internal.cuh"
#include "jit_embed.h"  // kEmbedFft, kEmbedRows, kEmbedCells (generated by build.py)
#include "spectral.cuh"

namespace aar {

struct JitState {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kern = nullptr;
  float* coef = nullptr;  // the module's __constant__ coefficients
  std::string key;        // N, M and the term structure the module was made for
  size_t smem = 0;
  int nterms = 0;
  int threads = kRowThreadsHost;  // block size the module was compiled for
  cudaKernel_t acc = nullptr;      // aar_modal_acc_jit, or null
  int acc_blocks = 0;              // its resident blocks per SM
  int64_t acc_fs = 0;              // field stride it was compiled for
};

static std::string gen_source(int N, int M, int minb, int threads, int pairs, const TermList& tl,
                              const std::vector<Term>& terms) {
  std::string s;
  // kCoef at global scope: its symbol name is not mangled (cudaLibraryGetGlobal)
  s += "#include \"rows.cuh\"\n";
  s += "__constant__ float kCoef[" + std::to_string(terms.empty() ? 1 : terms.size()) + "];\n";
  s += "namespace aar {\n";
  s += "struct JitRowOp {\n";
  s += "  static constexpr int min_blocks(int) { return " + std::to_string(minb) + "; }\n";
  s += "  static constexpr bool kPairs = " + std::string(pairs ? "true" : "false") + ";\n";
  s += "  static constexpr bool kZfac = false;\n";
  s += "  __device__ int nin() const { return " + std::to_string(M) + "; }\n";
  s += "  __device__ int in_slot(int l) const { return l; }\n";
  s += "  __device__ int nout() const { return " + std::to_string(tl.nr) + "; }\n";
  s += "  __device__ int out_line(int l) const {\n    switch (l) {\n";
  for (int i = 0; i < tl.nr; ++i) s += "      case " + std::to_string(i) + ": return " + std::to_string(tl.r_of_slot[i]) + ";\n";
  s += "    }\n    return 0;\n  }\n";
  s += "  __device__ int out_slot(int l) const { return out_line(l); }\n";
  s += "  template <int K>\n  __device__ __forceinline__ void combine(float2* sm, const int* pos, int LS) const {\n";
  s += "    float2 f[" + std::to_string(M) + "][K];\n";
  s += "#pragma unroll\n    for (int p = 0; p < " + std::to_string(M) + "; ++p)\n";
  s += "#pragma unroll\n      for (int i = 0; i < K; ++i) f[p][i] = sm[p * LS + pos[i]];\n";
  // one block per output slot (the counter-term f0 f2 -> g1 with its own
  // target r).  The slot's terms are factored: greedily, the field that
  // occurs in most remaining terms is taken out, g_r += f_F (sum_t c_t f_t),
  // so a term costs one multiply-add and a group one more (at 20 modes 212
  // operations for the 134 terms instead of 268).
  for (int sl = 0; sl < tl.nr; ++sl) {
    const int r = tl.r_of_slot[sl];
    s += "    {\n      float2 a[K];\n#pragma unroll\n      for (int i = 0; i < K; ++i) a[i] = make_float2(0.f, 0.f);\n";
    std::vector<size_t> rem;
    for (size_t t = 0; t < terms.size(); ++t)
      if (terms[t].r == r) rem.push_back(t);
    while (!rem.empty()) {
      std::vector<int> cnt(M, 0);
      for (size_t t : rem) {
        cnt[terms[t].p] += 1;
        if (terms[t].q != terms[t].p) cnt[terms[t].q] += 1;
      }
      const int F = (int)(std::max_element(cnt.begin(), cnt.end()) - cnt.begin());
      std::vector<size_t> keep;
      bool first = true;
      for (size_t t : rem) {
        if (terms[t].p != F && terms[t].q != F) {
          keep.push_back(t);
          continue;
        }
        const int o = terms[t].p == F ? terms[t].q : terms[t].p;
        const std::string c = "kCoef[" + std::to_string(t) + "]", fo = "f[" + std::to_string(o) + "][i]";
        if (first)
          s += "      {\n      float2 h[K];\n#pragma unroll\n      for (int i = 0; i < K; ++i) h[i] = make_float2(" + c + " * " +
               fo + ".x, " + c + " * " + fo + ".y);\n";
        else
          s += "#pragma unroll\n      for (int i = 0; i < K; ++i) { h[i].x = fmaf(" + c + ", " + fo + ".x, h[i].x); h[i].y = fmaf(" +
               c + ", " + fo + ".y, h[i].y); }\n";
        first = false;
      }
      const std::string fF = "f[" + std::to_string(F) + "][i]";
      s += "#pragma unroll\n      for (int i = 0; i < K; ++i) { a[i].x = fmaf(" + fF + ".x, h[i].x, a[i].x); a[i].y = fmaf(" + fF +
           ".y, h[i].y, a[i].y); }\n      }\n";
      rem.swap(keep);
    }
    s += "#pragma unroll\n      for (int i = 0; i < K; ++i) sm[" + std::to_string(r) + " * LS + pos[i]] = a[i];\n    }\n";
  }
  s += "  }\n};\n}  // namespace aar\n";
  s += "extern \"C\" __global__ void __launch_bounds__(" + std::to_string(threads) + ", " + std::to_string(minb) +
       ") aar_modal_rows_jit(float2* work, long long fs, int HP, const float2* __restrict__ twN, "
       "const float2* __restrict__ twH) {\n";
  s += "  aar::rows_body<" + std::to_string(N) + ", aar::JitRowOp, " + std::to_string(threads) +
       ">(aar::JitRowOp{}, work, fs, HP, twN, twH);\n}\n";
  return s;
}

// The modal accumulation of k_modal_acc (fused.cu) for this plan's active
// slots: the slot list, the recurrence steps between slots and the field
// offsets are compile-time, so the slot loop is straight-line code whose
// loads all issue before the sums (the generic kernel reads the slot list
// from shared memory and walks it with a runtime loop).  Same arithmetic in
// the same order as the generic kernel.
static std::string gen_acc(int N, int HP, const TermList& tl) {
  const long long fs = (long long)N * N * HP;
  std::string s;
  s += "extern \"C\" __global__ void __launch_bounds__(256) aar_modal_acc_jit(aar::Grid g, float2* phi, "
       "const float2* __restrict__ work, float fnl_n3, aar::RhoArgs ra) {\n";
  s += "  constexpr int N = " + std::to_string(N) + ", K = N / 2 + 1, HP = " + std::to_string(HP) + ";\n";
  s += "  constexpr long long total = (long long)N * N * K;\n";
  s += "  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;"
       " i += (long long)gridDim.x * blockDim.x) {\n";
  s += "    const long long row = i / K;\n    const int kz = (int)(i - row * K);\n    const long long e = row * HP + kz;\n";
  s += "    int x, y;\n    aar::row_xy(row, N, aar::kXB, x, y);\n";
  s += "    const int kx = aar::sidx(x, N), ky = aar::sidx(y, N);\n    const int n2 = kx * kx + ky * ky + kz * kz;\n";
  s += "    if (n2 == 0) {\n      phi[e] = make_float2(0.f, 0.f);\n      continue;\n    }\n";
  s += "    if (!aar::keep_cell(g, kx, ky, kz)) continue;\n";
  s += "    const float2* w = work + e;\n";
  for (int j = 0; j < tl.nr; ++j)
    s += "    const float2 v" + std::to_string(j) + " = __ldg(w + " + std::to_string((long long)tl.r_of_slot[j] * fs) +
         "LL);\n";
  s += "    const float lnn2 = logf((float)n2);\n";
  s += "    const float kbar = -1.f + ra.c1 * expm1f(0.5f * ra.s * lnn2);\n";
  s += "    const float L = ra.log2kF + lnn2 * 0.72134752044448170368f;\n";
  s += "    const float inv_k2 = ra.inv_kF2 / (float)n2;\n";
  s += "    float P0 = 1.f, P1 = kbar, Pn, rho;\n    float sx = 0.f, sy = 0.f, cx = 0.f, cy = 0.f;\n";
  int deg = 1;
  for (int j = 0; j < tl.nr; ++j) {
    const int r = tl.r_of_slot[j];
    if (r <= 3) {
      s += r == 3 ? "    rho = 1.f;\n" : "    rho = exp2f(ra.s * (float)(" + std::to_string(r - 3) + ") * L);\n";
    } else {
      for (; deg < r - 1; ) {
        ++deg;
        const std::string d = std::to_string(deg);
        s += "    Pn = ra.A[" + d + "] * kbar * P1 - ra.B[" + d + "] * P0;\n    P0 = P1;\n    P1 = Pn;\n";
      }
      s += "    rho = (P1 - ra.x0[" + std::to_string(r - 1) + "]) * inv_k2;\n";
    }
    s += "    aar::neumaier_add(sx, cx, v" + std::to_string(j) + ".x * rho);\n";
    s += "    aar::neumaier_add(sy, cy, v" + std::to_string(j) + ".y * rho);\n";
  }
  s += "    float2 ph = phi[e];\n    ph.x += fnl_n3 * (sx + cx);\n    ph.y += fnl_n3 * (sy + cy);\n    phi[e] = ph;\n";
  s += "  }\n}\n";
  return s;
}

static void jit_release(JitState* j) {
  if (!j) return;
  if (j->lib) cudaLibraryUnload(j->lib);
  delete j;
}

void jit_free(Plan* p) {
  jit_release((JitState*)p->jit);
  p->jit = nullptr;
}

// Build (or reuse) the specialised kernel for the plan's current term list.
// Returns AAR_OK with p->jit set, or AAR_OK with p->jit == nullptr and the
// reason in p->jit_status when the generic kernel stays in use.
int jit_prepare(Plan* p) {
  const bool want = p->jit_mode == 2 || (p->jit_mode == 1 && p->N >= 256);
  if (!want || p->prm.precision != AAR_FUSED_FP32 || p->nr_active == 0) {
    jit_free(p);
    p->jit_status = want ? "no modal terms" : "off";
    return AAR_OK;
  }
  const TermList& tl = *(const TermList*)p->host_terms.data();
  const Term* ft = (const Term*)(p->host_terms.data() + sizeof(TermList));
  std::vector<Term> terms(ft, ft + tl.nterms);
  const int N = p->N, M = p->M;
  const int minb = p->jit_minb > 0 ? p->jit_minb : (N >= 1024 ? 2 : 3);
  // default block size: 320 threads (ten warps) at N = 1024 where they take
  // the M input lines in fewer rounds than eight warps (measured at 1024^3,
  // 20 modes: 362 vs 372 ms per step); the autotuner may choose otherwise
  const int threads = p->jit_threads > 0                                   ? p->jit_threads
                      : (N >= 1024 && (M + 9) / 10 < (M + 7) / 8) ? 320
                                                                       : kRowThreadsHost;
  const int regcap = 65536 / (threads * minb);
  const int pairs = 2 * 2 * M + 16 <= regcap * 3 / 4;  // f values of two positions fit the register budget
  std::string key = std::to_string(N) + ":" + std::to_string(M) + ":" + std::to_string(minb) + ":" +
                    std::to_string(threads) + ":" + std::to_string(pairs) + ":";
  for (const Term& t : terms) key += std::to_string(t.p) + "," + std::to_string(t.q) + "," + std::to_string(t.r) + ";";
  std::vector<float> coef(terms.size());
  for (size_t i = 0; i < terms.size(); ++i) coef[i] = terms[i].c;
  JitState* j = (JitState*)p->jit;
  if (!j || j->key != key) {
    jit_free(p);
    const std::string src = "#include \"cells.cuh\"\n" + gen_source(N, M, minb, threads, pairs, tl, terms) +
                            gen_acc(N, p->HP, tl);
    nvrtcProgram prog;
    const char* hdrs[3] = {kEmbedFft, kEmbedRows, kEmbedCells};
    const char* names[3] = {"fft.cuh", "rows.cuh", "cells.cuh"};
    if (nvrtcCreateProgram(&prog, src.c_str(), "aar_modal_rows_jit.cu", 3, hdrs, names) != NVRTC_SUCCESS) {
      p->jit_status = "nvrtcCreateProgram failed";
      return AAR_OK;
    }
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++20", "-lineinfo", "-default-device"};
    nvrtcResult cr = nvrtcCompileProgram(prog, 4, opts);
    if (cr != NVRTC_SUCCESS) {
      size_t n = 0;
      nvrtcGetProgramLogSize(prog, &n);
      std::string log(n, '\0');
      if (n) nvrtcGetProgramLog(prog, &log[0]);
      nvrtcDestroyProgram(&prog);
      p->jit_status = "NVRTC: " + log.substr(0, 2000);
      return AAR_OK;
    }
    size_t nbin = 0;
    nvrtcGetCUBINSize(prog, &nbin);
    std::vector<char> bin(nbin);
    nvrtcGetCUBIN(prog, bin.data());
    nvrtcDestroyProgram(&prog);
    j = new JitState();
    if (cudaLibraryLoadData(&j->lib, bin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess ||
        cudaLibraryGetKernel(&j->kern, j->lib, "aar_modal_rows_jit") != cudaSuccess) {
      cudaGetLastError();
      jit_release(j);
      p->jit_status = "module load failed";
      return AAR_OK;
    }
    size_t csize = 0;
    if (cudaLibraryGetGlobal((void**)&j->coef, &csize, j->lib, "kCoef") != cudaSuccess) {
      cudaGetLastError();
      jit_release(j);
      p->jit_status = "coefficient symbol missing";
      return AAR_OK;
    }
    j->key = key;
    j->nterms = (int)terms.size();
    j->threads = threads;
    // the accumulation kernel is optional: without it the generic one runs
    if (cudaLibraryGetKernel(&j->acc, j->lib, "aar_modal_acc_jit") != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&j->acc_blocks, (const void*)j->acc, 256, 0) != cudaSuccess ||
        j->acc_blocks < 1) {
      cudaGetLastError();
      j->acc = nullptr;
    }
    j->acc_fs = (int64_t)N * N * p->HP;
    p->jit = j;
  }
  j->smem = sizeof(float2) * ((size_t)(M + 1) * p->row_ls + p->row_lt);
  if (cudaFuncSetAttribute((const void*)j->kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)j->smem) !=
      cudaSuccess) {
    cudaGetLastError();
    jit_free(p);
    p->jit_status = "shared-memory attribute refused";
    return AAR_OK;
  }
  if (!coef.empty()) AAR_CUDA_TRY(p, cudaMemcpy(j->coef, coef.data(), sizeof(float) * coef.size(), cudaMemcpyHostToDevice));
  p->jit_status = "on";
  return AAR_OK;
}

int jit_modal_rows(Plan* p, float2* work, int64_t fs, cudaStream_t st, int64_t nrows) {
  JitState* j = (JitState*)p->jit;
  long long fsl = fs;
  int hp = p->HP;
  void* args[] = {&work, &fsl, &hp, &p->d_twN, &p->d_twH};
  if (nrows < 0) nrows = (int64_t)p->N * p->N;
  {
    ProfScope ps_(p, "modal_rows", st);
    AAR_CUDA_TRY(p, cudaLaunchKernel((const void*)j->kern, dim3((unsigned)nrows), dim3(j->threads), args, j->smem, st));
  }
  p->last_launches += 1;
  return AAR_OK;
}

bool jit_has_acc(const Plan* p) {
  const JitState* j = (const JitState*)p->jit;
  return j && j->acc && j->acc_fs == (int64_t)p->N * p->N * p->HP;
}

int jit_modal_acc(Plan* p, float2* phi, const float2* work, float fnl_n3, const RhoArgs& ra, cudaStream_t st) {
  JitState* j = (JitState*)p->jit;
  Grid g = p->grid;
  RhoArgs r = ra;
  void* args[] = {&g, &phi, &work, &fnl_n3, &r};
  {
    ProfScope ps_(p, "modal_acc", st);
    AAR_CUDA_TRY(p, cudaLaunchKernel((const void*)j->acc, dim3((unsigned)(p->num_sms * j->acc_blocks)), dim3(256), args,
                                     0, st));
  }
  p->last_launches += 1;
  return AAR_OK;
}

}  // namespace aar
