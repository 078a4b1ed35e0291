// Dense stages of the hot path: valence-core orthogonalisation and packing,
// Hamiltonian assembly, and the per-k generalised Hermitian eigen-solve.
//
//   ortho + pack     intgOrtho.F90:23-187 with integrals.F90:2601-2853:
//                    O' = O_vv - (S_cv^H O_cv + O_cv^H S_cv) + S_cv^H O_cc S_cv
//                    (S' = S_vv - 2 S_cv^H S_cv + S_cv^H S_cc S_cv), upper
//                    triangle, diagonal made real as zherk/zher2k do, packed
//                    column by column with |x| < 1e-10 flushed when core_dim > 0.
//   assembly         secularEqn.F90:128-166, matrixSubs.F90:248-355.
//   solve            solveZHEGV, interfaces.F90:73-120 (itype 1, 'V', 'U').
// The orthogonalisation's products are FP64-accurate split-digit products on
// the tcgen05 kernel (olc_tcgemm.cu, through olc_ozaki.cu); the epilogue that
// combines, flushes and packs is a hand-written kernel.  The FP64 solve (the
// reference-equivalent path) uses a batched in-shared-memory kernel for
// n <= 64 (olc_eigen_small.cu) and cuSOLVER zhegvd per k above.
#include <cstdlib>
#include <algorithm>
#include <cstdio>

#include "olc_common.h"

namespace olc {

int solve_small_batched(olc_context* ctx, const double* h_full, const double* s_full, int n,
                        int num_states, double* eigenvalues, double* vectors, int32_t* info_host,
                        bool s_is_factored);
int small_solver_max_n();

namespace {

// combine, flush and pack; optionally also emit the full upper matrix (+ add)
struct PackArgs {
  const double* vv;      // [nk][nv][nv]
  const double* X;       // S_cv^H O_cv          (nullptr when nc == 0)
  const double* Y;       // S_cv^H O_cc S_cv
  const double* add;     // optional full upper matrix added after the flush
  double* packed;        // [nk][plen][2] or nullptr
  double* full;          // [nk][nv][nv] upper, or nullptr
  int nv;
  int nk;
  int nc;
  int is_overlap;
};

__global__ void ortho_pack_kernel(PackArgs a) {
  const size_t plen = (size_t)a.nv * (a.nv + 1) / 2;
  const size_t total = plen * a.nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / plen);
    const size_t r = idx % plen;
    // column i, row j <= i with r = i(i+1)/2 + j
    int i = (int)((sqrt(8.0 * (double)r + 1.0) - 1.0) * 0.5);
    while ((size_t)i * (i + 1) / 2 > r) --i;
    while ((size_t)(i + 1) * (i + 2) / 2 <= r) ++i;
    const int j = (int)(r - (size_t)i * (i + 1) / 2);
    const size_t nn = (size_t)a.nv * a.nv;
    const size_t off = (size_t)k * nn + (size_t)i * a.nv + j;   // (row j, col i)
    double re = a.vv[2 * off], im = a.vv[2 * off + 1];
    if (a.nc) {
      const double xr = a.X[2 * off], xi = a.X[2 * off + 1];
      if (a.is_overlap) {   // zherk('U','C',-2)
        re -= 2.0 * xr;
        im -= 2.0 * xi;
      } else {              // zher2k('U','C',-1): X + X^H
        const size_t offT = (size_t)k * nn + (size_t)j * a.nv + i;
        re -= xr + a.X[2 * offT];
        im -= xi - a.X[2 * offT + 1];
      }
      if (i == j) im = 0.0;
      re += a.Y[2 * off];
      im += a.Y[2 * off + 1];
      if (fabs(re) < 1.0e-10) re = 0.0;
      if (fabs(im) < 1.0e-10) im = 0.0;
    }
    if (a.packed) {
      a.packed[2 * idx] = re;
      a.packed[2 * idx + 1] = im;
    }
    if (a.full) {
      if (a.add) {
        re += a.add[2 * off];
        im += a.add[2 * off + 1];
      }
      a.full[2 * off] = re;
      a.full[2 * off + 1] = im;
    }
  }
}

// packed [nk][plen][2] -> full Hermitian [nk][n][n] (both triangles)
__global__ void unpack_kernel(const double* packed, double* full, int n, int nk) {
  const size_t nn = (size_t)n * n;
  const size_t total = nn * nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / nn);
    const size_t r = idx % nn;
    const int col = (int)(r / n), row = (int)(r % n);
    const int i = max(row, col), j = min(row, col);
    const size_t p = (size_t)k * ((size_t)n * (n + 1) / 2) + (size_t)i * (i + 1) / 2 + j;
    double re = packed[2 * p], im = packed[2 * p + 1];
    if (row > col) im = -im;
    if (row == col) im = 0.0;
    full[2 * idx] = re;
    full[2 * idx + 1] = im;
  }
}

// upper-only full matrix -> Hermitian (fill the strict lower triangle)
__global__ void hermitize_kernel(double* full, int n, int nk) {
  const size_t nn = (size_t)n * n;
  const size_t total = nn * nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / nn);
    const size_t r = idx % nn;
    const int col = (int)(r / n), row = (int)(r % n);
    if (row > col) {
      const size_t src = (size_t)k * nn + (size_t)row * n + col;
      full[2 * idx] = full[2 * src];
      full[2 * idx + 1] = -full[2 * src + 1];
    } else if (row == col) {
      full[2 * idx + 1] = 0.0;
    }
  }
}

// H packed = NP + KE + sum c_j V_j (zero multiplier adds unscaled)
__global__ void assemble_kernel(const double* const* terms, const double* coeffs, int nterm,
                                size_t len, double* out) {
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < len;
       idx += (size_t)gridDim.x * blockDim.x) {
    double acc = terms[0][idx];
    for (int t = 1; t < nterm; ++t) {
      const double c = coeffs[t];
      const double x = terms[t][idx];
      acc = (c == 0.0) ? acc + x : acc + x * c;
    }
    out[idx] = acc;
  }
}

// multipliers: leading `off` terms (NP, KE) weigh 1; an exact 0 counts as 1
__global__ void fix_coeff_kernel(double* c, int n, int off) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (i < off) c[i] = 1.0;
    else if (c[i] == 0.0) c[i] = 1.0;
  }
}

__global__ void gather_eigs_kernel(const double* w, int n, int nstates, int k, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nstates) out[(size_t)k * nstates + i] = w[i];
}

int grid_for(size_t n) {
  size_t g = (n + 255) / 256;
  return (int)std::min<size_t>(g, 152 * 32);
}

}  // namespace

// Orthogonalise one operator for all k.  vv/cv/cc are the operator's blocks,
// scv is S_cv.  Writes packed and/or full (upper, with `add` added).
int ortho_pack_ex(olc_context* ctx, bool is_overlap, const double* vv, const double* cv,
                  const double* cc, const double* scv, double* packed, double* full,
                  const double* add) {
  const int nv = ctx->dims.vale_dim, nc = ctx->dims.core_dim, nk = ctx->dims.num_kpoints;
  int st;
  if (nc) {
    const size_t nn = (size_t)nv * nv;
    if (!ctx->d_work_x) {
      if ((st = dalloc(ctx, &ctx->d_work_x, 2 * nn * nk))) return st;
      if ((st = dalloc(ctx, &ctx->d_work_y, 2 * nn * nk))) return st;
      if ((st = dalloc(ctx, &ctx->d_work_w, 2 * (size_t)nv * nc * nk))) return st;
    }
    // the three products on the tensor cores, FP64-accurate (split digits,
    // olc_ozaki.cu); OLC_ORTHO_BITS lowers the bits kept per operand
    int bits = 53;
    if (const char* v = std::getenv("OLC_ORTHO_BITS")) bits = std::max(24, std::min(53, std::atoi(v)));
    const long long sCV = 2LL * nc * nv, sCC = 2LL * nc * nc, sW = 2LL * nv * nc;
    // X = S_cv^H O_cv
    if ((st = ozaki_zgemm<double, double>(ctx, nv, nv, nc, scv, sCV, nc, true, bits, is_overlap ? scv : cv,
                                          sCV, nc, bits, ctx->d_work_x, nk, OLC_STAGE_ORTHO))) return st;
    // W = S_cv^H O_cc
    if ((st = ozaki_zgemm<double, double>(ctx, nv, nc, nc, scv, sCV, nc, true, bits, cc, sCC, nc, bits,
                                          ctx->d_work_w, nk, OLC_STAGE_ORTHO))) return st;
    // Y = W S_cv
    if ((st = ozaki_zgemm<double, double>(ctx, nv, nv, nc, ctx->d_work_w, sW, nv, false, bits, scv, sCV, nc,
                                          bits, ctx->d_work_y, nk, OLC_STAGE_ORTHO))) return st;
  }
  PackArgs a;
  a.vv = vv;
  a.X = ctx->d_work_x;
  a.Y = ctx->d_work_y;
  a.add = add;
  a.packed = packed;
  a.full = full;
  a.nv = nv;
  a.nk = nk;
  a.nc = nc;
  a.is_overlap = is_overlap ? 1 : 0;
  const size_t total = (size_t)nv * (nv + 1) / 2 * nk;
  StageScope scope(ctx, OLC_STAGE_ORTHO);
  ortho_pack_kernel<<<grid_for(total), 256, 0, ctx->stream>>>(a);
  return cuda_check(cudaGetLastError(), "ortho_pack_kernel");
}

int ortho_pack(olc_context* ctx, bool is_overlap, double* vv, const double* cv, const double* cc,
               const double* scv, double* packed, double* full_out) {
  return ortho_pack_ex(ctx, is_overlap, vv, cv, cc, is_overlap ? cv : scv, packed, full_out,
                       nullptr);
}

int assemble_packed(olc_context* ctx, const double* const* terms, const double* coeffs, int nterm,
                    double* out) {
  if (nterm < 1) return fail(OLC_ERR_ARG, "assemble: need at least one term");
  const size_t len = 2 * (size_t)ctx->dims.packed_len * ctx->dims.num_kpoints;
  const double** dterms = nullptr;
  double* dco = nullptr;
  int st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&dterms, sizeof(double*) * nterm, ctx->stream), "malloc"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&dco, sizeof(double) * nterm, ctx->stream), "malloc"))) return st;
  cudaMemcpyAsync(dterms, terms, sizeof(double*) * nterm, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(dco, coeffs, sizeof(double) * nterm, cudaMemcpyHostToDevice, ctx->stream);
  {
    StageScope scope(ctx, OLC_STAGE_ASSEMBLE);
    assemble_kernel<<<grid_for(len), 256, 0, ctx->stream>>>(dterms, dco, nterm, len, out);
  }
  st = cuda_check(cudaGetLastError(), "assemble_kernel");
  cudaFreeAsync(dterms, ctx->stream);
  cudaFreeAsync(dco, ctx->stream);
  if (!st) st = cuda_check(cudaStreamSynchronize(ctx->stream), "assemble sync");
  return st;
}

// Generalised eigen-problem per k on full Hermitian matrices h, s (both
// overwritten).  Library path: cuSOLVER zhegvd (the algorithm of LAPACK
// zhegv: Cholesky, reduction, tridiagonal solve, back-transform).  The k-points
// are independent problems, so they are spread over concurrent sub-streams,
// each with its own solver handle and workspace.
int solve_full_library(olc_context* ctx, double* h, double* s, int num_states,
                       double* eigenvalues, int eig_on_device, double* vectors, int32_t* info) {
  const int n = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  const size_t nn = (size_t)n * n;
  int st;
  const int nsub = std::max(1, std::min(nk, 16));
  if ((int)ctx->sub_streams.size() != nsub || ctx->sub_n != n) {
    for (size_t i = 0; i < ctx->sub_streams.size(); ++i) {
      cudaStreamSynchronize(ctx->sub_streams[i]);
      cusolverDnDestroy(ctx->sub_solvers[i]);
      cudaFree(ctx->sub_work[i]);
      cudaFree(ctx->sub_eval[i]);
      cudaStreamDestroy(ctx->sub_streams[i]);
      cudaEventDestroy(ctx->ev_join[i]);
    }
    ctx->sub_streams.clear(); ctx->sub_solvers.clear(); ctx->sub_work.clear();
    ctx->sub_eval.clear(); ctx->ev_join.clear();
    if (!ctx->ev_fork) cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    int lwork = 0;
    cusolverDnHandle_t h0;
    if (cusolverDnCreate(&h0) != CUSOLVER_STATUS_SUCCESS) return fail(OLC_ERR_CUDA, "cusolverDnCreate failed");
    cusolverStatus_t ss = cusolverDnZhegvd_bufferSize(
        h0, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n,
        reinterpret_cast<cuDoubleComplex*>(h), n, reinterpret_cast<cuDoubleComplex*>(s), n,
        nullptr, &lwork);
    cusolverDnDestroy(h0);
    if (ss != CUSOLVER_STATUS_SUCCESS) return fail(OLC_ERR_CUDA, "zhegvd_bufferSize failed");
    ctx->sub_work_bytes = sizeof(cuDoubleComplex) * (size_t)lwork;
    for (int i = 0; i < nsub; ++i) {
      cudaStream_t sm;
      cusolverDnHandle_t hs;
      void* w = nullptr;
      double* ev = nullptr;
      cudaEvent_t ej;
      if ((st = cuda_check(cudaStreamCreateWithFlags(&sm, cudaStreamNonBlocking), "sub stream"))) return st;
      if (cusolverDnCreate(&hs) != CUSOLVER_STATUS_SUCCESS) return fail(OLC_ERR_CUDA, "cusolverDnCreate failed");
      cusolverDnSetStream(hs, sm);
      if ((st = cuda_check(cudaMalloc(&w, ctx->sub_work_bytes), "solver work"))) return st;
      if ((st = cuda_check(cudaMalloc((void**)&ev, sizeof(double) * n), "solver eval"))) return st;
      cudaEventCreateWithFlags(&ej, cudaEventDisableTiming);
      ctx->sub_streams.push_back(sm);
      ctx->sub_solvers.push_back(hs);
      ctx->sub_work.push_back(w);
      ctx->sub_eval.push_back(ev);
      ctx->ev_join.push_back(ej);
    }
    ctx->sub_n = n;
  }
  if (!ctx->d_info && (st = dalloc(ctx, &ctx->d_info, (size_t)nk))) return st;
  double* eig_dev = eigenvalues;
  double* tmp_eigs = nullptr;
  if (!eig_on_device) {
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&tmp_eigs, sizeof(double) * (size_t)num_states * nk,
                                         ctx->stream), "malloc eigs"))) return st;
    eig_dev = tmp_eigs;
  }
  const int lwork = (int)(ctx->sub_work_bytes / sizeof(cuDoubleComplex));
  StageScope scope(ctx, OLC_STAGE_SOLVE, 0);
  cudaEventRecord(ctx->ev_fork, ctx->stream);
  for (int i = 0; i < nsub; ++i) cudaStreamWaitEvent(ctx->sub_streams[i], ctx->ev_fork, 0);
  st = parallel_host(nsub, ctx->device, [&](int i) -> int {
    cudaStream_t sm = ctx->sub_streams[i];
    for (int k = i; k < nk; k += nsub) {
      auto* H = reinterpret_cast<cuDoubleComplex*>(h) + (size_t)k * nn;
      auto* S = reinterpret_cast<cuDoubleComplex*>(s) + (size_t)k * nn;
      cusolverStatus_t ss = cusolverDnZhegvd(ctx->sub_solvers[i], CUSOLVER_EIG_TYPE_1,
                                             CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n,
                                             H, n, S, n, ctx->sub_eval[i],
                                             reinterpret_cast<cuDoubleComplex*>(ctx->sub_work[i]),
                                             lwork, ctx->d_info + k);
      if (ss != CUSOLVER_STATUS_SUCCESS) return OLC_ERR_CUDA;
      gather_eigs_kernel<<<(num_states + 127) / 128, 128, 0, sm>>>(ctx->sub_eval[i], n, num_states,
                                                                   k, eig_dev);
      if (vectors)
        cudaMemcpyAsync(vectors + 2 * (size_t)k * n * num_states, H,
                        sizeof(cuDoubleComplex) * (size_t)n * num_states, cudaMemcpyDeviceToDevice, sm);
    }
    return 0;
  });
  scope.add_launches(nk);
  if (st) return fail(st, "cusolverDnZhegvd failed");
  for (int i = 0; i < nsub; ++i) {
    cudaEventRecord(ctx->ev_join[i], ctx->sub_streams[i]);
    cudaStreamWaitEvent(ctx->stream, ctx->ev_join[i], 0);
  }
  if (!eig_on_device) {
    cudaMemcpyAsync(eigenvalues, tmp_eigs, sizeof(double) * (size_t)num_states * nk,
                    cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(tmp_eigs, ctx->stream);
  }
  std::vector<int> hinfo(nk);
  cudaMemcpyAsync(hinfo.data(), ctx->d_info, sizeof(int) * nk, cudaMemcpyDeviceToHost, ctx->stream);
  if ((st = cuda_check(cudaStreamSynchronize(ctx->stream), "solve sync"))) return st;
  int worst = 0;
  for (int k = 0; k < nk; ++k) {
    if (info) info[k] = hinfo[k];
    if (hinfo[k] != 0 && worst == 0) worst = hinfo[k];
  }
  if (worst > n) return fail(OLC_ERR_NOT_PD, "ZHEGV: overlap matrix not positive definite");
  if (worst != 0) return fail(OLC_ERR_EIGEN, "ZHEGV: eigen-solver did not converge");
  return OLC_OK;
}

int solve_full_mixed(olc_context* ctx, const double* h, const double* s, int num_states,
                     double* eig_dev, double* vectors, bool check = true, bool s_prepared = false);

int solve_full(olc_context* ctx, double* h, double* s, int num_states, double* eigenvalues,
               int eig_on_device, double* vectors, int32_t* info, int precision = OLC_PREC_FP64,
               bool s_prepared = false) {
  const int n = ctx->dims.vale_dim;
  if (precision == OLC_PREC_MIXED && n > small_solver_max_n()) {
    int st;
    double* eig_dev = eigenvalues;
    double* tmp = nullptr;
    const int nk = ctx->dims.num_kpoints;
    if (!eig_on_device) {
      if ((st = cuda_check(ctx_malloc(ctx, (void**)&tmp, sizeof(double) * (size_t)num_states * nk,
                                           ctx->stream), "malloc eigs"))) return st;
      eig_dev = tmp;
    }
    st = solve_full_mixed(ctx, h, s, num_states, eig_dev, vectors, true, s_prepared);
    if (!eig_on_device) {
      cudaMemcpyAsync(eigenvalues, tmp, sizeof(double) * (size_t)num_states * nk,
                      cudaMemcpyDeviceToHost, ctx->stream);
      cudaFreeAsync(tmp, ctx->stream);
      int s2 = cuda_check(cudaStreamSynchronize(ctx->stream), "eig copy");
      if (!st) st = s2;
    }
    if (info)
      for (int k = 0; k < nk; ++k) info[k] = 0;
    return st;
  }
  if (n <= small_solver_max_n()) {
    int st;
    double* eig_dev = eigenvalues;
    double* tmp = nullptr;
    const int nk = ctx->dims.num_kpoints;
    if (!eig_on_device) {
      if ((st = cuda_check(ctx_malloc(ctx, (void**)&tmp, sizeof(double) * (size_t)num_states * nk,
                                           ctx->stream), "malloc eigs"))) return st;
      eig_dev = tmp;
    }
    st = solve_small_batched(ctx, h, s, n, num_states, eig_dev, vectors, info, false);
    if (!eig_on_device) {
      cudaMemcpyAsync(eigenvalues, tmp, sizeof(double) * (size_t)num_states * nk,
                      cudaMemcpyDeviceToHost, ctx->stream);
      cudaFreeAsync(tmp, ctx->stream);
      int s2 = cuda_check(cudaStreamSynchronize(ctx->stream), "eig copy");
      if (!st) st = s2;
    }
    return st;
  }
  return solve_full_library(ctx, h, s, num_states, eigenvalues, eig_on_device, vectors, info);
}

int solve_packed(olc_context* ctx, const double* packed_h, const double* packed_s, int num_states,
                 double* eigenvalues, double* vectors, int32_t* info) {
  const int n = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  if (num_states < 1 || num_states > n) return fail(OLC_ERR_ARG, "num_states out of range");
  const size_t nn = (size_t)n * n;
  double *h = nullptr, *s = nullptr;
  int st;
  if ((st = cuda_check(cudaMalloc(&h, 16 * nn * nk), "malloc h"))) return st;
  if ((st = cuda_check(cudaMalloc(&s, 16 * nn * nk), "malloc s"))) { cudaFree(h); return st; }
  {
    StageScope scope(ctx, OLC_STAGE_ASSEMBLE, 2);
    unpack_kernel<<<grid_for(nn * nk), 256, 0, ctx->stream>>>(packed_h, h, n, nk);
    unpack_kernel<<<grid_for(nn * nk), 256, 0, ctx->stream>>>(packed_s, s, n, nk);
  }
  st = cuda_check(cudaGetLastError(), "unpack_kernel");
  if (!st) st = solve_full(ctx, h, s, num_states, eigenvalues, 1, vectors, info);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(h);
  cudaFree(s);
  return st;
}

// ---------------------------------------------------------------------------
// SCF pass
// ---------------------------------------------------------------------------
namespace {

// Stored form: H(k) = NP + KE + sum_j c_j V_j from the resident packed terms,
// written straight into the full Hermitian matrix the solver consumes (the
// packed read, readPackedMatrixAccum and unpackMatrix in one pass).
__global__ void assemble_full_kernel(const double* __restrict__ terms, const double* __restrict__ c,
                                     int nterm, int n, int nk, double* __restrict__ full) {
  const size_t plen = (size_t)n * (n + 1) / 2;
  const size_t total = plen * nk;
  const size_t tstride = 2 * plen * nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / plen);
    const size_t r = idx % plen;
    int i = (int)((sqrt(8.0 * (double)r + 1.0) - 1.0) * 0.5);
    while ((size_t)i * (i + 1) / 2 > r) --i;
    while ((size_t)(i + 1) * (i + 2) / 2 <= r) ++i;
    const int j = (int)(r - (size_t)i * (i + 1) / 2);
    const double2* t2 = reinterpret_cast<const double2*>(terms);
    double2 acc = t2[idx];
    for (int t = 1; t < nterm; ++t) {
      const double2 x = t2[(size_t)t * (tstride / 2) + idx];
      const double w = c[t];
      acc.x += w * x.x;
      acc.y += w * x.y;
    }
    double2* f = reinterpret_cast<double2*>(full) + (size_t)k * n * n;
    if (i == j) {
      f[(size_t)i * n + i] = make_double2(acc.x, 0.0);
    } else {
      f[(size_t)i * n + j] = acc;                               // (row j, col i)
      f[(size_t)j * n + i] = make_double2(acc.x, -acc.y);       // (row i, col j)
    }
  }
}

}  // namespace

int scf_prepare(olc_context* ctx, int precision, int form) {
  const int nv = ctx->dims.vale_dim, nc = ctx->dims.core_dim, nk = ctx->dims.num_kpoints;
  const int pd = ctx->dims.pot_dim;
  const size_t nn = (size_t)nv * nv;
  const size_t plen2 = 2 * (size_t)ctx->dims.packed_len * nk;   // doubles per packed term
  int st;
  if (!ctx->d_work_vv) {
    if ((st = dalloc(ctx, &ctx->d_work_vv, 2 * nn * nk))) return st;
    if (nc) {
      if ((st = dalloc(ctx, &ctx->d_work_cv, 2 * (size_t)nc * nv * nk))) return st;
      if ((st = dalloc(ctx, &ctx->d_work_cc, 2 * (size_t)nc * nc * nk))) return st;
      if ((st = dalloc(ctx, &ctx->d_scv, 2 * (size_t)nc * nv * nk))) return st;
    }
    if ((st = dalloc(ctx, &ctx->d_chol, 2 * nn * nk))) return st;   // orthogonalised S
  }
  // S: overlap integrals, keep S_cv, orthogonalise
  if ((st = run_primitives(ctx, OLC_OP_OVERLAP, 0, nullptr, OLC_PREC_FP64, false))) return st;
  if ((st = run_contract_bloch(ctx, ctx->d_work_vv, nc ? ctx->d_scv : nullptr, ctx->d_work_cc))) return st;
  if ((st = ortho_pack_ex(ctx, true, ctx->d_work_vv, ctx->d_scv, ctx->d_work_cc, ctx->d_scv,
                          nullptr, ctx->d_chol, nullptr))) return st;
  count_launch();
  hermitize_kernel<<<grid_for(nn * nk), 256, 0, ctx->stream>>>(ctx->d_chol, nv, nk);
  const int nfix = 2 + ctx->rel;          // NP, KE (, MV) ahead of the V_j
  if (form == OLC_FORM_STORED) {
    if (!ctx->d_terms && (st = dalloc(ctx, &ctx->d_terms, plen2 * (nfix + pd)))) return st;
    // term 0 = NP, 1 = KE, 2 = MV when rel = 1, then V_j (the order the
    // reference sums them, secularEqn.F90:128-150)
    const int ops[3] = {OLC_OP_NUCLEAR, OLC_OP_KINETIC, OLC_OP_MASSVEL};
    for (int t = 0; t < nfix + pd; ++t) {
      const int op = t < nfix ? ops[t] : OLC_OP_ELECPOT;
      if ((st = run_primitives(ctx, op, t < nfix ? 0 : t - nfix, nullptr, OLC_PREC_FP64, false))) return st;
      if ((st = run_contract_bloch(ctx, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc))) return st;
      if ((st = ortho_pack_ex(ctx, false, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc,
                              ctx->d_scv, ctx->d_terms + (size_t)t * plen2, nullptr, nullptr))) return st;
    }
  } else {
    if (!ctx->d_h0 && (st = dalloc(ctx, &ctx->d_h0, 2 * nn * nk))) return st;
    // H0 = KE + NP (+ MV) in one pass
    if ((st = run_primitives(ctx, OLC_OP_KINETIC, 0, nullptr, OLC_PREC_FP64, false))) return st;
    if ((st = run_primitives(ctx, OLC_OP_NUCLEAR, 0, nullptr, OLC_PREC_FP64, true))) return st;
    if (ctx->rel && (st = run_primitives(ctx, OLC_OP_MASSVEL, 0, nullptr, OLC_PREC_FP64, true))) return st;
    if ((st = run_contract_bloch(ctx, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc))) return st;
    if ((st = ortho_pack_ex(ctx, false, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc, ctx->d_scv,
                            nullptr, ctx->d_h0, nullptr))) return st;
  }
  ctx->prepared = true;
  ctx->w32_valid = false;
  ctx->prep_precision = precision;
  ctx->prep_form = form;
  return cuda_check(cudaStreamSynchronize(ctx->stream), "prepare sync");
}

// Builds H(k) (full Hermitian, all k) for the prepared form into h.
int build_hamiltonian(olc_context* ctx, const double* coeffs, int precision, int flags, double* h);

int scf_matrices(olc_context* ctx, const double* coeffs, int kpoint, double* h, double* s,
                 int on_device) {
  if (!ctx->prepared) return fail(OLC_ERR_ARG, "olc_scf_matrices before olc_scf_prepare");
  const int nv = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  if (kpoint < 0 || kpoint >= nk) return fail(OLC_ERR_ARG, "k-point out of range");
  const size_t nn = (size_t)nv * nv;
  double* hall = nullptr;
  int st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&hall, 16 * nn * nk, ctx->stream), "malloc h"))) return st;
  st = build_hamiltonian(ctx, coeffs, ctx->prep_precision, 0, hall);
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (!st && h) st = cuda_check(cudaMemcpyAsync(h, hall + 2 * nn * kpoint, 16 * nn, kind, ctx->stream), "copy h");
  if (!st && s) st = cuda_check(cudaMemcpyAsync(s, ctx->d_chol + 2 * nn * kpoint, 16 * nn, kind, ctx->stream), "copy s");
  cudaFreeAsync(hall, ctx->stream);
  int s2 = cuda_check(cudaStreamSynchronize(ctx->stream), "matrices sync");
  return st ? st : s2;
}

// The mixed, stored-form pass queued on the context stream without any host
// synchronisation (the part a CUDA graph captures): H(k) from the resident
// terms with the device coefficients, then the mixed solve.
static int enqueue_mixed_pass(olc_context* ctx, const double* dcoeffs, int num_states, double* eig_dev,
                              double* vectors) {
  const int nv = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  const size_t nn = (size_t)nv * nv;
  int st;
  double* h = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&h, 16 * nn * nk, ctx->stream), "malloc h"))) return st;
  if ((st = build_hamiltonian(ctx, dcoeffs, OLC_PREC_MIXED, OLC_ITER_COEFF_DEVICE, h))) return st;
  // the mixed solve reads S without modifying it: the prepared S directly
  st = solve_full_mixed(ctx, h, ctx->d_chol, num_states, eig_dev, vectors, false, true);
  cudaFreeAsync(h, ctx->stream);
  return st;
}

// OLC_ITER_GRAPH: the mixed stored-form pass as a CUDA graph.  Inputs and
// outputs go through fixed context buffers; the first call for a given
// (num_states, vectors) runs the pass directly (library workspaces get
// allocated), the second captures it, later calls replay it.  If the capture
// is refused, the context keeps running the pass directly.
static int scf_iteration_graph(olc_context* ctx, const double* coeffs, int num_states,
                               double* eigenvalues, int flags, double* vectors) {
  const int nv = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints, pd = ctx->dims.pot_dim;
  cudaStream_t stream = ctx->stream;
  int st;
  if (!ctx->g_coeff && (st = dalloc(ctx, &ctx->g_coeff, (size_t)std::max(1, pd)))) return st;
  if (!ctx->g_eig && (st = dalloc(ctx, &ctx->g_eig, (size_t)nv * nk))) return st;
  if (vectors && !ctx->g_vec && (st = dalloc(ctx, &ctx->g_vec, 2 * (size_t)nv * nv * nk))) return st;
  cudaMemcpyAsync(ctx->g_coeff, coeffs, sizeof(double) * pd,
                  (flags & OLC_ITER_COEFF_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream);
  double* vout = vectors ? ctx->g_vec : nullptr;
  const int key = num_states * 2 + (vectors ? 1 : 0);
  if (ctx->graph_exec && ctx->graph_key != key) {
    cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
  }
  if (!ctx->graph_exec) {
    if (ctx->graph_warm != key || ctx->graph_broken) {
      // direct pass (first call for this key, or capture refused before)
      if ((st = enqueue_mixed_pass(ctx, ctx->g_coeff, num_states, ctx->g_eig, vout))) return st;
      ctx->graph_warm = key;
    } else {
      const int64_t l0 = olc_launch_count();
      ctx->capturing = true;
      cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
      int sq = e == cudaSuccess ? enqueue_mixed_pass(ctx, ctx->g_coeff, num_states, ctx->g_eig, vout) : 1;
      cudaGraph_t g = nullptr;
      if (e == cudaSuccess) e = cudaStreamEndCapture(stream, &g);
      ctx->capturing = false;
      const int64_t captured = olc_launch_count() - l0;
      count_launch(-(int)captured);      // nothing ran yet
      if (!sq && e == cudaSuccess && g) e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (sq || e != cudaSuccess || !ctx->graph_exec) {
        cudaGetLastError();
        ctx->graph_exec = nullptr;
        ctx->graph_broken = true;
        if ((st = enqueue_mixed_pass(ctx, ctx->g_coeff, num_states, ctx->g_eig, vout))) return st;
      } else {
        ctx->graph_key = key;
        ctx->graph_launches = captured;
      }
    }
  }
  if (ctx->graph_exec) {
    if ((st = cuda_check(cudaGraphLaunch(ctx->graph_exec, stream), "graph launch"))) return st;
    count_launch((int)ctx->graph_launches);
  }
  if ((st = mixed_check_info(ctx))) return st;
  const size_t ebytes = sizeof(double) * (size_t)num_states * nk;
  cudaMemcpyAsync(eigenvalues, ctx->g_eig, ebytes,
                  (flags & OLC_ITER_EIG_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream);
  if (vectors)
    cudaMemcpyAsync(vectors, ctx->g_vec, 16 * (size_t)nv * num_states * nk, cudaMemcpyDeviceToDevice, stream);
  return cuda_check(cudaStreamSynchronize(stream), "graph pass sync");
}

int scf_iteration(olc_context* ctx, const double* coeffs, int precision, int num_states,
                  double* eigenvalues, int flags, double* vectors) {
  if (!ctx->prepared) return fail(OLC_ERR_ARG, "olc_scf_iteration before olc_scf_prepare");
  const int nv = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  if (num_states < 1 || num_states > nv) return fail(OLC_ERR_ARG, "num_states out of range");
  if ((flags & OLC_ITER_GRAPH) && precision == OLC_PREC_MIXED && ctx->prep_form == OLC_FORM_STORED &&
      nv > small_solver_max_n())
    return scf_iteration_graph(ctx, coeffs, num_states, eigenvalues, flags, vectors);
  const size_t nn = (size_t)nv * nv;
  int st;
  // the FP64 solvers overwrite S with its factor and need a copy; the mixed
  // solver (n above the small solver's limit) reads the prepared S directly
  const bool mixed = precision == OLC_PREC_MIXED && nv > small_solver_max_n();
  double *h = nullptr, *s = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&h, 16 * nn * nk, ctx->stream), "malloc h"))) return st;
  if (!mixed && (st = cuda_check(ctx_malloc(ctx, (void**)&s, 16 * nn * nk, ctx->stream), "malloc s"))) return st;
  if ((st = build_hamiltonian(ctx, coeffs, precision, flags, h))) return st;
  if (!mixed) cudaMemcpyAsync(s, ctx->d_chol, 16 * nn * nk, cudaMemcpyDeviceToDevice, ctx->stream);
  st = solve_full(ctx, h, mixed ? ctx->d_chol : s, num_states, eigenvalues,
                  (flags & OLC_ITER_EIG_DEVICE) ? 1 : 0, vectors, nullptr, precision, mixed);
  cudaFreeAsync(h, ctx->stream);
  if (s) cudaFreeAsync(s, ctx->stream);
  int s2 = cuda_check(cudaStreamSynchronize(ctx->stream), "iteration sync");
  return st ? st : s2;
}

int build_hamiltonian(olc_context* ctx, const double* coeffs, int precision, int flags, double* h) {
  const int nv = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints, pd = ctx->dims.pot_dim;
  const size_t nn = (size_t)nv * nv;
  int st;
  // coefficients on the device; the reference adds a term whose multiplier
  // is exactly 0 unscaled (matrixSubs.F90:278-282)
  double* dco = nullptr;
  const int off = ctx->prep_form == OLC_FORM_STORED ? 2 + ctx->rel : 0;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&dco, sizeof(double) * (pd + 3), ctx->stream), "malloc coeffs"))) return st;
  if (flags & OLC_ITER_COEFF_DEVICE) {
    cudaMemcpyAsync(dco + off, coeffs, sizeof(double) * pd, cudaMemcpyDeviceToDevice, ctx->stream);
  } else {
    cudaMemcpyAsync(dco + off, coeffs, sizeof(double) * pd, cudaMemcpyHostToDevice, ctx->stream);
  }
  count_launch();
  fix_coeff_kernel<<<1, 64, 0, ctx->stream>>>(dco, pd + off, off);
  if (ctx->prep_form == OLC_FORM_STORED) {
    const size_t plen = (size_t)ctx->dims.packed_len;
    StageScope scope(ctx, OLC_STAGE_ASSEMBLE);
    assemble_full_kernel<<<grid_for(plen * nk), 256, 0, ctx->stream>>>(ctx->d_terms, dco, pd + off,
                                                                        nv, nk, h);
    if ((st = cuda_check(cudaGetLastError(), "assemble_full_kernel"))) return st;
  } else {
    st = run_primitives(ctx, OLC_OP_ELECPOT, 0, dco, precision, false);
    if (st) { cudaFreeAsync(dco, ctx->stream); return st; }
    if ((st = run_contract_bloch(ctx, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc))) return st;
    // H' = ortho(V) + H0, upper, then mirrored
    if ((st = ortho_pack_ex(ctx, false, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc, ctx->d_scv,
                            nullptr, h, ctx->d_h0))) return st;
    StageScope scope(ctx, OLC_STAGE_ASSEMBLE);
    hermitize_kernel<<<grid_for(nn * nk), 256, 0, ctx->stream>>>(h, nv, nk);
  }
  cudaFreeAsync(dco, ctx->stream);
  return cuda_check(cudaGetLastError(), "hamiltonian kernels");
}

}  // namespace olc
