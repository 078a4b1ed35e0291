// Batched generalised Hermitian eigen-solver for small n, one CTA per k-point,
// everything in shared memory (FP64).
//
// Same mathematical steps as LAPACK zhegv (itype 1, 'V', 'U'), the routine the
// reference calls in solveZHEGV (src/olcao/interfaces.F90:73-120):
//   1. S = U^H U                      (zpotrf 'U'; info = n + j when the
//                                      leading minor j is not positive)
//   2. C = U^{-H} H U^{-1}            (zhegst itype 1)
//   3. C = V diag(w) V^H              here: two-sided cyclic Jacobi with a
//                                      parallel (round-robin) pair ordering
//   4. X = U^{-1} V                   (back-transform, X^H S X = I)
// Eigenvalues are returned in ascending order with their vectors.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "olc_common.h"
#include "olc_jacobi.cuh"

namespace olc {

namespace {

constexpr int kSmallMaxN = jac::kMaxN;
constexpr int kThreads = 256;
using jac::cd;
using jac::cmul;
using jac::csub;

__global__ void __launch_bounds__(kThreads) small_hegv_kernel(
    const double* __restrict__ hin, const double* __restrict__ sin_, int n, int num_states,
    int s_factored, double* __restrict__ eig_out, double* __restrict__ vec_out,
    int32_t* __restrict__ info_out, double* __restrict__ trace_out) {
  extern __shared__ double smem[];
  const int k = blockIdx.x;
  const int tid = threadIdx.x;
  const size_t nn = (size_t)n * n;
  cd* U = reinterpret_cast<cd*>(smem);          // n*n, column-major U[col*n+row]
  cd* C = U + nn;
  cd* V = C + nn;
  double* w = reinterpret_cast<double*>(V + nn);     // n
  int* order = reinterpret_cast<int*>(w + n);       // n
  __shared__ jac::Shared sh;

  const cd* Hg = reinterpret_cast<const cd*>(hin) + (size_t)k * nn;
  const cd* Sg = reinterpret_cast<const cd*>(sin_) + (size_t)k * nn;
  for (size_t i = tid; i < nn; i += blockDim.x) {
    U[i] = Sg[i];
    C[i] = Hg[i];
  }
  jac::hegv_inplace(U, C, V, n, s_factored != 0, sh, trace_out ? trace_out + (size_t)k * 82 : nullptr);
  if (sh.fail) {
    if (tid == 0 && info_out) info_out[k] = sh.fail;
    for (int i = tid; i < num_states; i += blockDim.x) eig_out[(size_t)k * num_states + i] = 0.0;
    return;
  }
  // ---- 4. eigenvalues, sort, back-transform X = U^{-1} V ------------------
  jac::sorted_order(C, n, w, order);
  for (int i = tid; i < num_states; i += blockDim.x) eig_out[(size_t)k * num_states + i] = w[order[i]];
  if (vec_out) {
    cd* X = reinterpret_cast<cd*>(vec_out) + (size_t)k * n * num_states;
    // back substitution per output column
    for (int col = tid; col < num_states; col += blockDim.x) {
      const int src = order[col];
      for (int r = n - 1; r >= 0; --r) {
        cd acc = V[(size_t)src * n + r];
        for (int q = r + 1; q < n; ++q) acc = csub(acc, cmul(U[(size_t)q * n + r], X[(size_t)col * n + q]));
        const double inv = 1.0 / U[(size_t)r * n + r].x;
        X[(size_t)col * n + r] = {acc.x * inv, acc.y * inv};
      }
    }
  }
  if (tid == 0 && info_out) info_out[k] = 0;
}

}  // namespace

// Largest n sent to the batched in-shared-memory solver.  OLC_SMALL_SOLVER_MAX_N
// lowers it (0 routes every size to the library path; used to cross-check the
// two solvers on the same matrices).
int small_solver_max_n() {
  static int v = -1;
  if (v < 0) {
    v = kSmallMaxN;
    if (const char* e = std::getenv("OLC_SMALL_SOLVER_MAX_N")) v = std::min(kSmallMaxN, std::atoi(e));
  }
  return v;
}

int solve_small_batched(olc_context* ctx, const double* h_full, const double* s_full, int n,
                        int num_states, double* eigenvalues, double* vectors, int32_t* info_host,
                        bool s_is_factored) {
  const int nk = ctx->dims.num_kpoints;
  const size_t smem = sizeof(double) * 2 * 3 * (size_t)n * n + sizeof(double) * n + sizeof(int) * n;
  int st;
  if ((st = cuda_check(cudaFuncSetAttribute(small_hegv_kernel,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "smem attribute"))) return st;
  int32_t* dinfo = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&dinfo, sizeof(int32_t) * nk, ctx->stream), "malloc info"))) return st;
  StageScope scope(ctx, OLC_STAGE_SOLVE);
  // OLC_SMALL_SOLVER_TRACE=1 prints each k-point's Jacobi convergence history
  double* dtrace = nullptr;
  static const bool trace = std::getenv("OLC_SMALL_SOLVER_TRACE") != nullptr;
  if (trace) {
    const size_t tl = 82 * (size_t)nk;
    cudaMalloc(&dtrace, sizeof(double) * tl);
    cudaMemset(dtrace, 0, sizeof(double) * tl);
  }
  small_hegv_kernel<<<nk, kThreads, smem, ctx->stream>>>(h_full, s_full, n, num_states,
                                                         s_is_factored ? 1 : 0, eigenvalues,
                                                         vectors, dinfo, dtrace);
  if (dtrace) {
    std::vector<double> ht(82 * (size_t)nk);
    cudaMemcpy(ht.data(), dtrace, sizeof(double) * ht.size(), cudaMemcpyDeviceToHost);
    for (int k = 0; k < nk; ++k) {
      std::fprintf(stderr, "k=%d", k);
      for (int q = 0; q < 40 && ht[82 * k + 2 * q + 1] != 0.0; ++q)
        std::fprintf(stderr, " %.2e", ht[82 * k + 2 * q] / ht[82 * k + 2 * q + 1]);
      std::fprintf(stderr, "\n");
    }
    cudaFree(dtrace);
  }
  st = cuda_check(cudaGetLastError(), "small_hegv_kernel");
  std::vector<int32_t> hinfo(nk, 0);
  cudaMemcpyAsync(hinfo.data(), dinfo, sizeof(int32_t) * nk, cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(dinfo, ctx->stream);
  int s2 = cuda_check(cudaStreamSynchronize(ctx->stream), "small solve sync");
  if (st) return st;
  if (s2) return s2;
  int worst = 0;
  for (int k = 0; k < nk; ++k) {
    if (info_host) info_host[k] = hinfo[k];
    if (hinfo[k] && !worst) worst = hinfo[k];
  }
  if (worst > n) return fail(OLC_ERR_NOT_PD, "ZHEGV: overlap matrix not positive definite");
  if (worst) return fail(OLC_ERR_EIGEN, "eigen-solver did not converge");
  return OLC_OK;
}

// Launches the batched solver on full Hermitian h, s [nk][n][n] with no
// allocation and no synchronisation (info is device memory).
int launch_small_hegv_raw(cudaStream_t stream, const double* h_full, const double* s_full, int n,
                          int nk, int num_states, double* eigenvalues, double* vectors,
                          int32_t* info_dev) {
  const size_t smem = sizeof(double) * 2 * 3 * (size_t)n * n + sizeof(double) * n + sizeof(int) * n;
  int st;
  if ((st = cuda_check(cudaFuncSetAttribute(small_hegv_kernel,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "smem attribute"))) return st;
  count_launch();
  small_hegv_kernel<<<nk, kThreads, smem, stream>>>(h_full, s_full, n, num_states, 0, eigenvalues,
                                                    vectors, info_dev, nullptr);
  return cuda_check(cudaGetLastError(), "small_hegv_kernel");
}

int small_solver_capacity_n() { return kSmallMaxN; }

}  // namespace olc
