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

namespace olc {

namespace {

constexpr int kSmallMaxN = 64;
constexpr int kThreads = 256;

struct cd { double x, y; };
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd cmulc(cd a, cd b) { return {a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x}; }  // conj(a)*b
__device__ __forceinline__ cd csub(cd a, cd b) { return {a.x - b.x, a.y - b.y}; }

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
  __shared__ int s_fail;
  __shared__ double s_red[kThreads / 32];
  __shared__ double s_off, s_diag;
  __shared__ int s_p[kSmallMaxN / 2], s_q[kSmallMaxN / 2];
  __shared__ double s_c[kSmallMaxN / 2], s_s[kSmallMaxN / 2], s_phx[kSmallMaxN / 2],
      s_phy[kSmallMaxN / 2];

  const cd* Hg = reinterpret_cast<const cd*>(hin) + (size_t)k * nn;
  const cd* Sg = reinterpret_cast<const cd*>(sin_) + (size_t)k * nn;
  for (size_t i = tid; i < nn; i += blockDim.x) {
    U[i] = Sg[i];
    C[i] = Hg[i];
  }
  if (tid == 0) s_fail = 0;
  __syncthreads();

  // ---- 1. Cholesky S = U^H U (right-looking, upper) ----------------------
  if (!s_factored) {
    for (int j = 0; j < n; ++j) {
      if (tid == 0) {
        const double d = U[(size_t)j * n + j].x;
        if (!(d > 0.0)) s_fail = n + j + 1;
        U[(size_t)j * n + j] = {sqrt(fmax(d, 1e-300)), 0.0};
      }
      __syncthreads();
      if (s_fail) break;
      const double inv = 1.0 / U[(size_t)j * n + j].x;
      for (int i = j + 1 + tid; i < n; i += blockDim.x) {   // row j, columns i > j
        cd& u = U[(size_t)i * n + j];
        u.x *= inv;
        u.y *= inv;
      }
      __syncthreads();
      // trailing update S(r,c) -= conj(U(j,r)) U(j,c) for j < r <= c
      const int m = n - j - 1;
      for (int e = tid; e < m * m; e += blockDim.x) {
        const int r = j + 1 + e % m, c = j + 1 + e / m;
        if (r <= c) {
          const cd a = U[(size_t)r * n + j], b = U[(size_t)c * n + j];
          cd& t = U[(size_t)c * n + r];
          t = csub(t, cmulc(a, b));
        }
      }
      __syncthreads();
    }
    // clear the strict lower triangle
    for (size_t e = tid; e < nn; e += blockDim.x) {
      const int r = (int)(e % n), c = (int)(e / n);
      if (r > c) U[e] = {0.0, 0.0};
    }
    __syncthreads();
  }
  if (s_fail) {
    if (tid == 0 && info_out) info_out[k] = s_fail;
    for (int i = tid; i < num_states; i += blockDim.x) eig_out[(size_t)k * num_states + i] = 0.0;
    return;
  }

  // ---- 2. C = U^{-H} H U^{-1} --------------------------------------------
  // Y = U^{-H} H : row by row (forward substitution), in place in C
  for (int i = 0; i < n; ++i) {
    const double inv = 1.0 / U[(size_t)i * n + i].x;
    for (int c = tid; c < n; c += blockDim.x) {
      cd acc = C[(size_t)c * n + i];
      for (int q = 0; q < i; ++q) acc = csub(acc, cmulc(U[(size_t)i * n + q], C[(size_t)c * n + q]));
      C[(size_t)c * n + i] = {acc.x * inv, acc.y * inv};
    }
    __syncthreads();
  }
  // C = Y U^{-1} : column by column, in place
  for (int j = 0; j < n; ++j) {
    const double inv = 1.0 / U[(size_t)j * n + j].x;
    for (int r = tid; r < n; r += blockDim.x) {
      cd acc = C[(size_t)j * n + r];
      for (int q = 0; q < j; ++q) acc = csub(acc, cmul(C[(size_t)q * n + r], U[(size_t)j * n + q]));
      C[(size_t)j * n + r] = {acc.x * inv, acc.y * inv};
    }
    __syncthreads();
  }
  if (trace_out) {
    double* d0 = trace_out + (size_t)gridDim.x * 82 + (size_t)k * 6 * nn;
    for (size_t e = tid; e < nn; e += blockDim.x) { d0[2 * e] = C[e].x; d0[2 * e + 1] = C[e].y; }
  }
  // V = I
  for (size_t e = tid; e < nn; e += blockDim.x) {
    const int r = (int)(e % n), c = (int)(e / n);
    V[e] = {r == c ? 1.0 : 0.0, 0.0};
  }
  __syncthreads();

  // ---- 3. cyclic Jacobi with round-robin pairs ---------------------------
  const int m = (n % 2) ? n + 1 : n;
  const int half = m / 2;
  for (int sweep = 0; sweep < 40; ++sweep) {
    // convergence: off-diagonal vs diagonal mass
    double off = 0.0, dg = 0.0;
    for (size_t e = tid; e < nn; e += blockDim.x) {
      const int r = (int)(e % n), c = (int)(e / n);
      const double a2 = C[e].x * C[e].x + C[e].y * C[e].y;
      if (r == c) dg += a2; else off += a2;
    }
    for (int o = 16; o; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dg += __shfl_xor_sync(0xffffffffu, dg, o);
    }
    if ((tid & 31) == 0) s_red[tid >> 5] = off;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < (int)(blockDim.x / 32); ++q) t += s_red[q];
      s_off = t;
    }
    __syncthreads();
    if ((tid & 31) == 0) s_red[tid >> 5] = dg;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < (int)(blockDim.x / 32); ++q) t += s_red[q];
      s_diag = t;
    }
    __syncthreads();
    if (trace_out && tid == 0 && sweep < 40) {
      trace_out[(size_t)k * 82 + 2 * sweep] = s_off;
      trace_out[(size_t)k * 82 + 2 * sweep + 1] = s_diag;
    }
    if (s_off <= 1e-28 * s_diag || s_off == 0.0) break;
    for (int round = 0; round < m - 1; ++round) {
      // rotation parameters of this round's disjoint pairs, from the
      // pre-round matrix: J = D R with D = diag(1, e^{-i phi}), R real
      if (tid < half) {
        const int pi = tid;
        int p, q;
        if (pi == 0) { p = round % (m - 1); q = m - 1; }
        else { p = (round + pi) % (m - 1); q = (round - pi + (m - 1)) % (m - 1); }
        if (p > q) { const int t = p; p = q; q = t; }
        double c = 1.0, s = 0.0, phx = 1.0, phy = 0.0;
        if (q < n) {
          const cd cpq = C[(size_t)q * n + p];
          // hypot keeps |e^{-i phi}| = 1 when the entry is tiny (x*x + y*y
          // would drop into denormals and make the rotation non-unitary);
          // entries below 1e-18 of the diagonal scale are left alone
          const double b = hypot(cpq.x, cpq.y);
          const double app = C[(size_t)p * n + p].x, aqq = C[(size_t)q * n + q].x;
          if (b > 1e-300 && b > 1e-18 * (fabs(app) + fabs(aqq))) {
            const double th = (aqq - app) / (2.0 * b);
            const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
            phx = cpq.x / b;
            phy = -cpq.y / b;
          }
        }
        s_p[pi] = p; s_q[pi] = q; s_c[pi] = c; s_s[pi] = s; s_phx[pi] = phx; s_phy[pi] = phy;
      }
      __syncthreads();
      // columns: C <- C J, V <- V J
      //   col_p' = c col_p - s e^{-i phi} col_q ; col_q' = s col_p + c e^{-i phi} col_q
      for (int e = tid; e < half * n; e += blockDim.x) {
        const int pi = e / n, r = e % n;
        const int p = s_p[pi], q = s_q[pi];
        if (q >= n || s_s[pi] == 0.0) continue;
        const double c = s_c[pi], s = s_s[pi];
        const cd ph = {s_phx[pi], s_phy[pi]};
        {
          const cd xp = C[(size_t)p * n + r], eq = cmul(ph, C[(size_t)q * n + r]);
          C[(size_t)p * n + r] = {c * xp.x - s * eq.x, c * xp.y - s * eq.y};
          C[(size_t)q * n + r] = {s * xp.x + c * eq.x, s * xp.y + c * eq.y};
        }
        {
          const cd xp = V[(size_t)p * n + r], eq = cmul(ph, V[(size_t)q * n + r]);
          V[(size_t)p * n + r] = {c * xp.x - s * eq.x, c * xp.y - s * eq.y};
          V[(size_t)q * n + r] = {s * xp.x + c * eq.x, s * xp.y + c * eq.y};
        }
      }
      __syncthreads();
      // rows: C <- J^H C
      //   row_p' = c row_p - s e^{i phi} row_q ; row_q' = s row_p + c e^{i phi} row_q
      for (int e = tid; e < half * n; e += blockDim.x) {
        const int pi = e / n, col = e % n;
        const int p = s_p[pi], q = s_q[pi];
        if (q >= n || s_s[pi] == 0.0) continue;
        const double c = s_c[pi], s = s_s[pi];
        const cd phc = {s_phx[pi], -s_phy[pi]};
        const cd xp = C[(size_t)col * n + p], eq = cmul(phc, C[(size_t)col * n + q]);
        C[(size_t)col * n + p] = {c * xp.x - s * eq.x, c * xp.y - s * eq.y};
        C[(size_t)col * n + q] = {s * xp.x + c * eq.x, s * xp.y + c * eq.y};
      }
      __syncthreads();
    }
  }
  if (trace_out) {
    double* d1 = trace_out + (size_t)gridDim.x * 82 + (size_t)k * 6 * nn + 2 * nn;
    for (size_t e = tid; e < nn; e += blockDim.x) {
      d1[2 * e] = C[e].x; d1[2 * e + 1] = C[e].y;
      d1[2 * nn + 2 * e] = V[e].x; d1[2 * nn + 2 * e + 1] = V[e].y;
    }
  }
  __syncthreads();
  // ---- 4. eigenvalues, sort, back-transform X = U^{-1} V ------------------
  for (int i = tid; i < n; i += blockDim.x) {
    w[i] = C[(size_t)i * n + i].x;
    order[i] = i;
  }
  __syncthreads();
  if (tid == 0) {
    for (int i = 1; i < n; ++i) {   // insertion sort, ascending
      const int oi = order[i];
      const double wi = w[oi];
      int j = i - 1;
      while (j >= 0 && w[order[j]] > wi) { order[j + 1] = order[j]; --j; }
      order[j + 1] = oi;
    }
  }
  __syncthreads();
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
  if ((st = cuda_check(cudaMallocAsync((void**)&dinfo, sizeof(int32_t) * nk, ctx->stream), "malloc info"))) return st;
  StageScope scope(ctx, OLC_STAGE_SOLVE);
  // OLC_SMALL_SOLVER_TRACE=1 prints each k-point's Jacobi convergence history
  double* dtrace = nullptr;
  static const bool trace = std::getenv("OLC_SMALL_SOLVER_TRACE") != nullptr;
  if (trace) {
    const size_t tl = 82 * (size_t)nk + 6 * (size_t)n * n * nk;
    cudaMalloc(&dtrace, sizeof(double) * tl);
    cudaMemset(dtrace, 0, sizeof(double) * tl);
  }
  small_hegv_kernel<<<nk, kThreads, smem, ctx->stream>>>(h_full, s_full, n, num_states,
                                                         s_is_factored ? 1 : 0, eigenvalues,
                                                         vectors, dinfo, dtrace);
  if (dtrace) {
    std::vector<double> ht(82 * (size_t)nk + 6 * (size_t)n * n * nk);
    cudaMemcpy(ht.data(), dtrace, sizeof(double) * ht.size(), cudaMemcpyDeviceToHost);
    if (const char* f = std::getenv("OLC_SMALL_SOLVER_TRACE_FILE")) {
      FILE* fp = std::fopen(f, "wb");
      if (fp) { std::fwrite(ht.data() + 82 * (size_t)nk, sizeof(double), 6 * (size_t)n * n * nk, fp); std::fclose(fp); }
    }
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
