// Valence charge density and its traces with the stored operators: the step
// after the eigen-solve in an SCF iteration (makeValenceRho,
// src/olcao/valeCharge.F90:34-420; matrixElementMult, matrixSubs.F90:10-53).
//
// The reference, per k and spin channel, adds f(n) x_n x_n^H to the upper
// triangle of rho one zher per occupied state (valeCharge.F90:232-241),
// packs it (packMatrix), turns the two channels into total and difference
// when spin = 2 (:307-313), and forms for every stored operator T (overlap,
// nuclear, kinetic, mass velocity when rel = 1, each potential term)
//     sum_{j<i} 2 (Re T_ji Re rho_ji + Im T_ji Im rho_ji) + sum_i Re T_ii Re rho_ii
// accumulated over k (:321-395).
//
// Here, for all k at once:
//  * the occupied states of each k (sum over spin of |f| >= 1e-8, the
//    reference's smallThresh test) are gathered into A = X_occ diag(f) and
//    B = X_occ^H, zero-padded to the largest occupied count over k;
//  * rho(k) = A B is one batched FP64-accurate split product on the tensor
//    cores (olc_ozaki.cu, 53 bits per operand);
//  * one HBM-bound pass reads every operator's upper triangle once against
//    rho's and writes per-block partial traces, which a second kernel sums
//    in a fixed order (bitwise reproducible from run to run).
// The overlap comes from the prepared full S; NP, KE and V_j from the stored
// packed terms, or, for a context prepared in the fused form, recomputed one
// operator at a time into a scratch packed buffer.
#include <algorithm>
#include <cmath>
#include <vector>

#include "olc_common.h"

namespace olc {

namespace {

constexpr double kSmallThresh = 1.0e-8;   // smallThresh, src/constants.f90:49
constexpr int kTraceThreads = 256;
constexpr int kTraceEpt = 4;               // packed elements per thread per tile
constexpr int kTraceChunk = 24;            // operators per trace launch (48 KB of accumulators)

int grid_of(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

// A[k] (n x nocc) = X_occ diag(f), B[k] (nocc x n) = X_occ^H, column-major.
// idx[k][c] < 0 marks a padding column (f = 0, x = 0).
__global__ void gather_occupied_kernel(const double* __restrict__ X, int n, int ns, int nk, int nocc,
                                       const int* __restrict__ idx, const double* __restrict__ f,
                                       double* __restrict__ A, double* __restrict__ B) {
  const size_t total = (size_t)nk * nocc * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % n);
    const size_t kc = e / n;                 // k * nocc + c
    const int c = (int)(kc % nocc), k = (int)(kc / nocc);
    const int q = idx[kc];
    double xr = 0.0, xi = 0.0;
    if (q >= 0) {
      const size_t off = ((size_t)k * ns + q) * n + r;
      xr = X[2 * off];
      xi = X[2 * off + 1];
    }
    const double w = f[kc];
    A[2 * e] = w * xr;
    A[2 * e + 1] = w * xi;
    const size_t ob = ((size_t)k * n + r) * nocc + c;
    B[2 * ob] = xr;
    B[2 * ob + 1] = -xi;
  }
}

// spin = 2: (up, down) -> (up + down, up - down) over the upper triangles
// (valeCharge.F90:307-313).
__global__ void spin_sum_diff_kernel(double* __restrict__ r0, double* __restrict__ r1, int n, int nk) {
  const size_t total = (size_t)nk * n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t m = e % ((size_t)n * n);
    const int i = (int)(m / n), j = (int)(m % n);
    if (j > i) continue;
    const double ar = r0[2 * e], ai = r0[2 * e + 1], br = r1[2 * e], bi = r1[2 * e + 1];
    r0[2 * e] = ar + br;
    r0[2 * e + 1] = ai + bi;
    r1[2 * e] = ar - br;
    r1[2 * e + 1] = ai - bi;
  }
}

// packMatrix of every k (matrixSubs.F90:400-425): full [nk][n][n] -> packed
// [nk][plen][2], index j + i(i+1)/2 for row j <= column i.
__global__ void pack_rho_kernel(const double* __restrict__ full, int n, int nk, double* __restrict__ packed) {
  const size_t plen = (size_t)n * (n + 1) / 2, total = plen * nk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e / plen);
    const size_t r = e % plen;
    int i = (int)((sqrt(8.0 * (double)r + 1.0) - 1.0) * 0.5);
    while ((size_t)i * (i + 1) / 2 > r) --i;
    while ((size_t)(i + 1) * (i + 2) / 2 <= r) ++i;
    const int j = (int)(r - (size_t)i * (i + 1) / 2);
    const size_t off = (size_t)k * n * n + (size_t)i * n + j;
    packed[2 * e] = full[2 * off];
    packed[2 * e + 1] = full[2 * off + 1];
  }
}

// Element-wise traces of rho against nt operators.  Operator 0 is the full
// S [nk][n][n] when sfull != nullptr; the others are packed terms
// [nt'][nk][plen][2] (term stride tstride doubles).  Block (b, k) walks tiles
// b, b + gridDim.x, ... of k's packed index range.  Every thread keeps one
// running sum per operator in shared memory (sacc[t][thread]), so the inner
// loop has no cross-thread traffic; the block reduces them once at the end
// and writes partial[(k * gridDim.x + b) * nt + t].  Each pass over a tile
// has the loads of two operators in flight.
__global__ void __launch_bounds__(kTraceThreads) trace_kernel(
    const double* __restrict__ rho, const double* __restrict__ sfull, const double* __restrict__ terms,
    long long tstride, int nt, int n, long long plen, double* __restrict__ partial) {
  extern __shared__ double sacc[];           // [nt][kTraceThreads]
  const int k = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int t = 0; t < nt; ++t) sacc[t * kTraceThreads + tid] = 0.0;
  const size_t nn = (size_t)n * n;
  const double2* rk = reinterpret_cast<const double2*>(rho) + (size_t)k * nn;
  const double2* sk = sfull ? reinterpret_cast<const double2*>(sfull) + (size_t)k * nn : nullptr;
  const int npk = sfull ? 1 : 0;
  const long long tile = (long long)kTraceThreads * kTraceEpt;
  for (long long base = (long long)blockIdx.x * tile; base < plen; base += (long long)gridDim.x * tile) {
    double wr[kTraceEpt], wi[kTraceEpt];
    size_t foff[kTraceEpt];
    long long pr[kTraceEpt];
#pragma unroll
    for (int e = 0; e < kTraceEpt; ++e) {
      const long long r = base + (long long)e * kTraceThreads + tid;
      pr[e] = r < plen ? r : plen - 1;       // clamped: in bounds, weight 0
      int i = (int)((sqrtf(8.0f * (float)pr[e] + 1.0f) - 1.0f) * 0.5f);
      while ((long long)i * (i + 1) / 2 > pr[e]) --i;
      while ((long long)(i + 1) * (i + 2) / 2 <= pr[e]) ++i;
      const int j = (int)(pr[e] - (long long)i * (i + 1) / 2);
      foff[e] = (size_t)i * n + j;
      const double2 x = rk[foff[e]];
      // the diagonal counts once and only its real part; off-diagonal
      // elements stand for themselves and their mirror image
      const double g = r < plen ? (i == j ? 1.0 : 2.0) : 0.0;
      wr[e] = g * x.x;
      wi[e] = (i == j) ? 0.0 : g * x.y;
    }
    int t = 0;
    if (npk) {
      double a = 0.0;
#pragma unroll
      for (int e = 0; e < kTraceEpt; ++e) {
        const double2 v = sk[foff[e]];
        a += v.x * wr[e] + v.y * wi[e];
      }
      sacc[tid] += a;
      t = 1;
    }
    for (; t + 1 < nt; t += 2) {
      const double2* t0 = reinterpret_cast<const double2*>(terms + (size_t)(t - npk) * tstride) + (size_t)k * plen;
      const double2* t1 = reinterpret_cast<const double2*>(terms + (size_t)(t + 1 - npk) * tstride) + (size_t)k * plen;
      double2 v0[kTraceEpt], v1[kTraceEpt];
#pragma unroll
      for (int e = 0; e < kTraceEpt; ++e) {
        v0[e] = t0[pr[e]];
        v1[e] = t1[pr[e]];
      }
      double a0 = 0.0, a1 = 0.0;
#pragma unroll
      for (int e = 0; e < kTraceEpt; ++e) {
        a0 += v0[e].x * wr[e] + v0[e].y * wi[e];
        a1 += v1[e].x * wr[e] + v1[e].y * wi[e];
      }
      sacc[t * kTraceThreads + tid] += a0;
      sacc[(t + 1) * kTraceThreads + tid] += a1;
    }
    if (t < nt) {
      const double2* t0 = reinterpret_cast<const double2*>(terms + (size_t)(t - npk) * tstride) + (size_t)k * plen;
      double a0 = 0.0;
#pragma unroll
      for (int e = 0; e < kTraceEpt; ++e) {
        const double2 v = t0[pr[e]];
        a0 += v.x * wr[e] + v.y * wi[e];
      }
      sacc[t * kTraceThreads + tid] += a0;
    }
  }
  __syncthreads();
  for (int t = warp; t < nt; t += kTraceThreads / 32) {
    double a = 0.0;
    for (int q = lane; q < kTraceThreads; q += 32) a += sacc[t * kTraceThreads + q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) partial[((size_t)k * gridDim.x + blockIdx.x) * nt + t] = a;
  }
}

// out[t] = sum over the np partial rows of partial[row * nt + t], in a fixed
// order: one block per t.
__global__ void reduce_partials_kernel(const double* __restrict__ partial, int np, int nt,
                                       double* __restrict__ out) {
  __shared__ double s[256];
  const int t = blockIdx.x;
  double a = 0.0;
  for (int q = threadIdx.x; q < np; q += blockDim.x) a += partial[(size_t)q * nt + t];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[t] = s[0];
}

struct Scratch {
  olc_context* ctx;
  std::vector<void*> ptrs;
  template <class T>
  int get(T** p, size_t bytes, const char* what) {
    void* q = nullptr;
    int st = cuda_check(ctx_malloc(ctx, &q, std::max<size_t>(bytes, 16), ctx->stream), what);
    if (st) return st;
    ptrs.push_back(q);
    *p = static_cast<T*>(q);
    return OLC_OK;
  }
  ~Scratch() {
    for (void* q : ptrs) cudaFreeAsync(q, ctx->stream);
  }
};

// Traces of rho (all k) against nt operators into out[nt] (device), in
// chunks of at most kTraceChunk operators (per-thread accumulators of one
// chunk fill 48 KB of shared memory).
int launch_traces(olc_context* ctx, const double* rho, const double* sfull, const double* terms,
                  long long tstride, int nt, double* partial, int bx, double* out) {
  const int n = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  const long long plen = ctx->dims.packed_len;
  StageScope scope(ctx, OLC_STAGE_DENSITY, 0);
  for (int t0 = 0; t0 < nt; t0 += kTraceChunk) {
    const int c = std::min(kTraceChunk, nt - t0);
    const bool with_s = sfull && t0 == 0;
    const double* tp = terms ? terms + (size_t)(t0 - (sfull && t0 > 0 ? 1 : 0)) * tstride : nullptr;
    const size_t smem = sizeof(double) * kTraceThreads * c;
    trace_kernel<<<dim3(bx, nk), kTraceThreads, smem, ctx->stream>>>(rho, with_s ? sfull : nullptr, tp, tstride, c,
                                                                      n, plen, partial);
    reduce_partials_kernel<<<c, 256, 0, ctx->stream>>>(partial, bx * nk, c, out + t0);
    scope.add_launches(2);
  }
  return cuda_check(cudaGetLastError(), "trace kernels");
}

}  // namespace

int make_valence_rho(olc_context* ctx, int num_states, int spin, const double* occupation,
                     const double* eigenvalues, const double* vectors, double* traces,
                     double* electron_energy, double* rho_packed) {
  if (!ctx->prepared || !ctx->d_chol)
    return fail(OLC_ERR_ARG, "olc_make_valence_rho: call olc_scf_prepare first");
  const int n = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints, pd = ctx->dims.pot_dim;
  if (spin != 1 && spin != 2) return fail(OLC_ERR_ARG, "olc_make_valence_rho: spin must be 1 or 2");
  if (num_states < 1 || num_states > n) return fail(OLC_ERR_ARG, "olc_make_valence_rho: num_states out of range");
  if (!occupation || !vectors || !traces)
    return fail(OLC_ERR_ARG, "olc_make_valence_rho: occupation, vectors and traces are required");
  if (electron_energy && !eigenvalues)
    return fail(OLC_ERR_ARG, "olc_make_valence_rho: electron_energy needs eigenvalues");
  const int nfix = 2 + ctx->rel;            // NP, KE (, MV) ahead of the V_j
  const int nt = 1 + nfix + pd;
  const size_t nn = (size_t)n * n;
  auto occ = [&](int s, int k, int j) { return occupation[j + (size_t)num_states * (k + (size_t)nk * s)]; };

  // occupied states of every k (valeCharge.F90:232-234) and the electron
  // energy sum f * lambda in the reference's order (k, then state)
  std::vector<std::vector<int>> kept(nk);
  int nocc = 0;
  std::vector<double> energy(spin, 0.0);
  for (int k = 0; k < nk; ++k) {
    for (int j = 0; j < num_states; ++j) {
      double a = 0.0;
      for (int s = 0; s < spin; ++s) a += std::fabs(occ(s, k, j));
      if (a < kSmallThresh) continue;
      kept[k].push_back(j);
      if (eigenvalues)
        for (int s = 0; s < spin; ++s)
          energy[s] += occ(s, k, j) * eigenvalues[j + (size_t)num_states * (k + (size_t)nk * s)];
    }
    nocc = std::max<int>(nocc, (int)kept[k].size());
  }
  if (electron_energy)
    for (int s = 0; s < spin; ++s) electron_energy[s] = energy[s];
  std::fill(traces, traces + (size_t)nt * spin, 0.0);
  cudaStream_t st = ctx->stream;
  int rc;
  if (nocc == 0) {
    if (rho_packed)
      return cuda_check(cudaMemsetAsync(rho_packed, 0, 16 * (size_t)ctx->dims.packed_len * nk * spin, st),
                        "clear rho");
    return OLC_OK;
  }
  std::vector<int> hidx((size_t)nk * nocc, -1);
  std::vector<double> hf((size_t)spin * nk * nocc, 0.0);
  for (int k = 0; k < nk; ++k)
    for (size_t c = 0; c < kept[k].size(); ++c) {
      hidx[(size_t)k * nocc + c] = kept[k][c];
      for (int s = 0; s < spin; ++s) hf[((size_t)s * nk + k) * nocc + c] = occ(s, k, kept[k][c]);
    }

  Scratch sc{ctx, {}};
  int* didx = nullptr;
  double *df = nullptr, *A = nullptr, *B = nullptr, *rho = nullptr, *dtr = nullptr, *partial = nullptr;
  if ((rc = sc.get(&didx, sizeof(int) * hidx.size(), "malloc occupied index"))) return rc;
  if ((rc = sc.get(&df, sizeof(double) * hf.size(), "malloc occupations"))) return rc;
  if ((rc = sc.get(&A, 16 * (size_t)nk * nocc * n, "malloc X f"))) return rc;
  if ((rc = sc.get(&B, 16 * (size_t)nk * nocc * n, "malloc X^H"))) return rc;
  if ((rc = sc.get(&rho, 16 * nn * nk * spin, "malloc rho"))) return rc;
  if ((rc = sc.get(&dtr, sizeof(double) * nt * spin, "malloc traces"))) return rc;
  if ((rc = cuda_check(cudaMemcpyAsync(didx, hidx.data(), sizeof(int) * hidx.size(), cudaMemcpyHostToDevice, st),
                       "copy index"))) return rc;
  if ((rc = cuda_check(cudaMemcpyAsync(df, hf.data(), sizeof(double) * hf.size(), cudaMemcpyHostToDevice, st),
                       "copy occupations"))) return rc;

  // rho_s(k) = X_occ diag(f_s) X_occ^H for every spin channel
  for (int s = 0; s < spin; ++s) {
    {
      StageScope scope(ctx, OLC_STAGE_DENSITY);
      gather_occupied_kernel<<<grid_of((size_t)nk * nocc * n), 256, 0, st>>>(
          vectors + 2 * (size_t)s * n * num_states * nk, n, num_states, nk, nocc, didx,
          df + (size_t)s * nk * nocc, A, B);
    }
    if ((rc = ozaki_zgemm<double, double>(ctx, n, n, nocc, A, 2LL * n * nocc, n, false, 53, B, 2LL * nocc * n,
                                          nocc, 53, rho + 2 * (size_t)s * nn * nk, nk, OLC_STAGE_DENSITY,
                                          true)))
      return rc;
  }
  double* rho1 = rho + 2 * nn * nk;
  if (spin == 2) {
    StageScope scope(ctx, OLC_STAGE_DENSITY);
    spin_sum_diff_kernel<<<grid_of(nn * nk), 256, 0, st>>>(rho, rho1, n, nk);
  }
  if (rho_packed) {
    StageScope scope(ctx, OLC_STAGE_DENSITY, spin);
    const size_t pl2 = 2 * (size_t)ctx->dims.packed_len * nk;
    for (int s = 0; s < spin; ++s)
      pack_rho_kernel<<<grid_of(pl2 / 2), 256, 0, st>>>(rho + 2 * (size_t)s * nn * nk, n, nk, rho_packed + s * pl2);
  }

  // element-wise traces: S from the prepared full overlap, then NP, KE, V_j
  const long long plen = ctx->dims.packed_len;
  const long long tiles = (plen + (long long)kTraceThreads * kTraceEpt - 1) / ((long long)kTraceThreads * kTraceEpt);
  const int bx = (int)std::max<long long>(1, std::min<long long>(tiles, (152LL * 8 + nk - 1) / nk));
  if ((rc = sc.get(&partial, sizeof(double) * (size_t)bx * nk * nt, "malloc partial traces"))) return rc;
  const long long tstride = 2 * plen * nk;
  if (ctx->prep_form == OLC_FORM_STORED && ctx->d_terms) {
    // d_terms holds NP, KE, (MV,) V_j in the trace order of the reference
    for (int s = 0; s < spin; ++s)
      if ((rc = launch_traces(ctx, rho + 2 * (size_t)s * nn * nk, ctx->d_chol, ctx->d_terms, tstride, nt, partial,
                              bx, dtr + (size_t)s * nt))) return rc;
  } else {
    // fused form: no operator is kept apart, so each is recomputed,
    // orthogonalised and packed once into scratch (as olc_scf_prepare's
    // stored form builds them) and traced for every spin channel
    double* tmp = nullptr;
    if ((rc = sc.get(&tmp, 8 * (size_t)tstride, "malloc packed operator"))) return rc;
    for (int s = 0; s < spin; ++s)
      if ((rc = launch_traces(ctx, rho + 2 * (size_t)s * nn * nk, ctx->d_chol, nullptr, 0, 1, partial, bx,
                              dtr + (size_t)s * nt))) return rc;
    const int ops[3] = {OLC_OP_NUCLEAR, OLC_OP_KINETIC, OLC_OP_MASSVEL};
    for (int t = 0; t < nfix + pd; ++t) {
      const int op = t < nfix ? ops[t] : OLC_OP_ELECPOT;
      if ((rc = run_primitives(ctx, op, t < nfix ? 0 : t - nfix, nullptr, OLC_PREC_FP64, false))) return rc;
      if ((rc = run_contract_bloch(ctx, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc))) return rc;
      if ((rc = ortho_pack(ctx, false, ctx->d_work_vv, ctx->d_work_cv, ctx->d_work_cc, ctx->d_scv, tmp, nullptr)))
        return rc;
      for (int s = 0; s < spin; ++s)
        if ((rc = launch_traces(ctx, rho + 2 * (size_t)s * nn * nk, nullptr, tmp, tstride, 1, partial, bx,
                                dtr + (size_t)s * nt + 1 + t))) return rc;
    }
  }
  if ((rc = cuda_check(cudaMemcpyAsync(traces, dtr, sizeof(double) * nt * spin, cudaMemcpyDeviceToHost, st),
                       "copy traces"))) return rc;
  return cuda_check(cudaStreamSynchronize(st), "valence rho sync");
}

}  // namespace olc
