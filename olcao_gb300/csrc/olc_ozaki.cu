// FP64-accurate complex products from BF16 tensor-core GEMMs (the splitting
// of Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59 (2012) 95-118).
//
// C[b] = op(A[b]) B[b], A logical m x k (op = identity or conjugate
// transpose), B k x n, C m x n complex FP64, column-major, for a batch.
//
//  * Every row of A (column of B) gets an exponent e with max |x| < 2^e over
//    the row; x 2^(W-e) truncated to an integer N with W = nd * beta bits is
//    cut into nd signed digits of beta bits, most significant first.  The
//    digits are read straight off the IEEE bit pattern (integer arithmetic
//    only) and stored as BF16, which holds them exactly.
//  * Complex products use planar operands: A's digits as [Ar; Ai] (2m x k),
//    B's as [Br, Bi] (k x 2n).  One real GEMM gives the four blocks
//    ArBr, ArBi, AiBr, AiBi; Re = ArBr - AiBi, Im = ArBi + AiBr.
//  * Digit pairs (s, t) with equal s + t = d share the scale 2^(-beta d).
//    They are summed by ONE GEMM over the concatenated K dimension (A's
//    digit blocks are consecutive columns, B's are stored in reverse digit
//    order so that the matching blocks are consecutive rows).  beta is the
//    largest width for which pairs * k * (2^beta - 1)^2 < 2^24, so every FP32
//    sum in the GEMM is an exact integer.
//  * One pass combines all groups per element in 64-bit integer fixed point
//    (groups converted to int32 exactly) and scales by 2^(e_row + f_col).
#include <algorithm>
#include <cuda_bf16.h>

#include <cstdlib>
#include <cstring>

#include "olc_common.h"
#include "olc_tcgemm.h"

namespace olc {

namespace {

__device__ __forceinline__ int expo_field(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff);
}
__device__ __forceinline__ int expo_field(float x) { return (int)((__float_as_uint(x) >> 23) & 0xff); }
// 2^e bounds |x| for a normal number with exponent field E
__device__ __forceinline__ int bound_expo(double, int E) { return E ? E - 1022 : -100000; }
__device__ __forceinline__ int bound_expo(float, int E) { return E ? E - 126 : -100000; }

// trunc(|x| 2^(W - e)) for |x| < 2^e, W <= 62; subnormals count as zero
__device__ __forceinline__ unsigned long long fixed_bits(double x, int e, int W) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  const int E = (int)(u >> 52);
  if (E == 0) return 0ULL;
  const unsigned long long mant = (u & 0xfffffffffffffULL) | (1ULL << 52);
  const int sh = E - 1075 + W - e;
  if (sh >= 0) return mant << sh;
  if (sh <= -64) return 0ULL;
  return mant >> (-sh);
}
__device__ __forceinline__ unsigned long long fixed_bits(float x, int e, int W) {
  const unsigned u = __float_as_uint(x) & 0x7fffffffu;
  const int E = (int)(u >> 23);
  if (E == 0) return 0ULL;
  const unsigned long long mant = (unsigned long long)((u & 0x7fffffu) | (1u << 23));
  const int sh = E - 150 + W - e;
  if (sh >= 0) return mant << sh;
  if (sh <= -64) return 0ULL;
  return mant >> (-sh);
}

__device__ __forceinline__ double exp2_int(int p) {
  if (p < -1022) return 0.0;
  return __longlong_as_double((long long)(p + 1023) << 52);
}

// Row exponents of a column-major source read down its rows (thread per row,
// coalesced across rows): used for the left operand without transpose.
template <class T>
__global__ void row_expo_kernel(const T* __restrict__ src, long long sstride, int ld, int rows,
                                int cols, int nb, int* __restrict__ expo) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)rows * nb) return;
  const int b = (int)(t / rows), r = (int)(t % rows);
  const T* s = src + (size_t)b * sstride;
  int E = 0;
  for (int c = 0; c < cols; ++c) {
    E = max(E, expo_field(s[2 * ((size_t)c * ld + r)]));
    E = max(E, expo_field(s[2 * ((size_t)c * ld + r) + 1]));
  }
  expo[t] = bound_expo(T(0), E);
}

// Exponents of source columns (warp per column, contiguous): the right
// operand's columns, or the rows of a conjugate-transposed left operand.
template <class T>
__global__ void col_expo_kernel(const T* __restrict__ src, long long sstride, int ld, int len,
                                int lines, int nb, int* __restrict__ expo) {
  const size_t gw = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= (size_t)lines * nb) return;
  const int b = (int)(gw / lines), line = (int)(gw % lines);
  const T* s = src + (size_t)b * sstride + 2 * (size_t)line * ld;
  int E = 0;
  for (int i = lane; i < 2 * len; i += 32) E = max(E, expo_field(s[i]));
  for (int o = 16; o; o >>= 1) E = max(E, __shfl_xor_sync(0xffffffffu, E, o));
  if (lane == 0) expo[gw] = bound_expo(T(0), E);
}

// Left operand digits: out[b][s][c][r'] (kp columns of 2 mp rows, the
// padding zero) with r' < mp the digits of Re A(r,c), r' >= mp those of
// Im A(r,c); A = src or src^H.  32 x 32 tiles through shared
// memory so that reads and writes both coalesce.
template <class T>
__global__ void __launch_bounds__(256) slice_left_kernel(const T* __restrict__ src, long long sstride,
                                                         int ld, bool conj, int m, int k, int mp, int kp,
                                                         const int* __restrict__ ea, int na, int beta,
                                                         __nv_bfloat16* __restrict__ out) {
  __shared__ T tre[32][33], tim[32][33];
  const int b = blockIdx.z;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const T* s = src + (size_t)b * sstride;
  for (int j = ty; j < 32; j += 8) {
    if (!conj) {
      const int r = r0 + tx, c = c0 + j;
      if (r < m && c < k) {
        tre[j][tx] = s[2 * ((size_t)c * ld + r)];
        tim[j][tx] = s[2 * ((size_t)c * ld + r) + 1];
      }
    } else {
      const int c = c0 + tx, r = r0 + j;
      if (r < m && c < k) {
        tre[tx][j] = s[2 * ((size_t)r * ld + c)];
        tim[tx][j] = -s[2 * ((size_t)r * ld + c) + 1];
      }
    }
  }
  __syncthreads();
  const int W = na * beta;
  const unsigned long long mask = (1ULL << beta) - 1ULL;
  const size_t slice = (size_t)kp * 2 * mp;
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + tx, c = c0 + j;
    if (r >= m || c >= k) continue;
    const T xr = tre[j][tx], xi = tim[j][tx];
    const int e = ea[(size_t)b * m + r];
    const unsigned long long Nr = fixed_bits(xr, e, W), Ni = fixed_bits(xi, e, W);
    const bool sr = xr < T(0), si = xi < T(0);
    __nv_bfloat16* o = out + ((size_t)b * na * kp + c) * 2 * mp;
    for (int d = 0; d < na; ++d) {
      const int sh = W - beta * (d + 1);
      const int dr = (int)((Nr >> sh) & mask), di = (int)((Ni >> sh) & mask);
      o[(size_t)d * slice + r] = __float2bfloat16_rn((float)(sr ? -dr : dr));
      o[(size_t)d * slice + r + mp] = __float2bfloat16_rn((float)(si ? -di : di));
    }
  }
}

// Right operand digits: out[b][c'][row] (2 np columns, the padding zero),
// c' < np the digits of Re B(r,c), c' >= np those of Im B(r,c); digit t at
// rows (nbs-1-t)*kp + r (ld nbs*kp).
template <class T>
__global__ void slice_right_kernel(const T* __restrict__ src, long long sstride, int ld, int k,
                                   int n, int kp, int np, const int* __restrict__ fb, int nbs,
                                   int beta, int nb, __nv_bfloat16* __restrict__ out) {
  const size_t per = (size_t)k * n, total = per * nb;
  const int W = nbs * beta;
  const unsigned long long mask = (1ULL << beta) - 1ULL;
  const size_t ldo = (size_t)nbs * kp;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(idx / per);
    const size_t q = idx % per;
    const int r = (int)(q % k), c = (int)(q / k);
    const T* s = src + (size_t)b * sstride;
    const T xr = s[2 * ((size_t)c * ld + r)], xi = s[2 * ((size_t)c * ld + r) + 1];
    const int e = fb[(size_t)b * n + c];
    const unsigned long long Nr = fixed_bits(xr, e, W), Ni = fixed_bits(xi, e, W);
    const bool sr = xr < T(0), si = xi < T(0);
    __nv_bfloat16* o = out + (size_t)b * 2 * np * ldo;
    for (int t = 0; t < nbs; ++t) {
      const int sh = W - beta * (t + 1);
      const int dr = (int)((Nr >> sh) & mask), di = (int)((Ni >> sh) & mask);
      const size_t row = (size_t)(nbs - 1 - t) * kp + r;
      o[(size_t)c * ldo + row] = __float2bfloat16_rn((float)(sr ? -dr : dr));
      o[(size_t)(c + np) * ldo + row] = __float2bfloat16_rn((float)(si ? -di : di));
    }
  }
}

// Combine the group products: G[d][b] is the 2mp x 2np FP32 product of group d
// (exact integers).  Group values (int32, exact) are added in 64-bit fixed
// point, `per_acc` groups per accumulator; the accumulators are combined in
// FP64 and scaled by 2^(e_r + f_c - 2 beta).  One thread per 4 consecutive
// rows of one column (16-byte loads; mp is a multiple of 8).
__global__ void combine_kernel(const float* __restrict__ G, int ngroups, size_t gstride,
                               const int* __restrict__ ea, const int* __restrict__ fb, int m, int n,
                               int mp, int np, int beta, int per_acc, int nb, double* __restrict__ C) {
  const int mq = (m + 3) >> 2;                 // row quads per column
  const size_t per = (size_t)mq * n, total = per * nb;
  const size_t m2 = 2 * (size_t)mp;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(idx / per);
    const size_t q = idx % per;
    const int r0 = 4 * (int)(q % mq), c = (int)(q / mq);
    const float* g = G + (size_t)b * 4 * mp * np;
    double accr[4] = {0.0, 0.0, 0.0, 0.0}, acci[4] = {0.0, 0.0, 0.0, 0.0};
    for (int d0 = 0; d0 < ngroups; d0 += per_acc) {
      const int d1 = min(ngroups, d0 + per_acc);
      long long ar[4] = {0, 0, 0, 0}, ai[4] = {0, 0, 0, 0};
      for (int d = d0; d < d1; ++d) {
        const float* gd = g + (size_t)d * gstride;
        const float4 rr = *reinterpret_cast<const float4*>(gd + (size_t)c * m2 + r0);
        const float4 ii = *reinterpret_cast<const float4*>(gd + (size_t)(c + np) * m2 + r0 + mp);
        const float4 ri = *reinterpret_cast<const float4*>(gd + (size_t)(c + np) * m2 + r0);
        const float4 ir = *reinterpret_cast<const float4*>(gd + (size_t)c * m2 + r0 + mp);
        ar[0] = (ar[0] << beta) + (long long)(__float2int_rn(rr.x) - __float2int_rn(ii.x));
        ar[1] = (ar[1] << beta) + (long long)(__float2int_rn(rr.y) - __float2int_rn(ii.y));
        ar[2] = (ar[2] << beta) + (long long)(__float2int_rn(rr.z) - __float2int_rn(ii.z));
        ar[3] = (ar[3] << beta) + (long long)(__float2int_rn(rr.w) - __float2int_rn(ii.w));
        ai[0] = (ai[0] << beta) + (long long)(__float2int_rn(ri.x) + __float2int_rn(ir.x));
        ai[1] = (ai[1] << beta) + (long long)(__float2int_rn(ri.y) + __float2int_rn(ir.y));
        ai[2] = (ai[2] << beta) + (long long)(__float2int_rn(ri.z) + __float2int_rn(ir.z));
        ai[3] = (ai[3] << beta) + (long long)(__float2int_rn(ri.w) + __float2int_rn(ir.w));
      }
      const double w = exp2_int(-beta * (d1 - 1));
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        accr[u] = fma((double)ar[u], w, accr[u]);
        acci[u] = fma((double)ai[u], w, acci[u]);
      }
    }
    const int fc = fb[(size_t)b * n + c];
    double* o = C + 2 * ((size_t)b * m * n + (size_t)c * m);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = r0 + u;
      if (r >= m) break;
      const double sc = exp2_int(ea[(size_t)b * m + r] + fc - 2 * beta);
      o[2 * r] = accr[u] * sc;
      o[2 * r + 1] = acci[u] * sc;
    }
  }
}

int grid_of(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

}  // namespace

// Digit width for a K-length product of na x nbs digits (see the file comment).
void ozaki_plan(int k, int bits_a, int bits_b, int* beta, int* na, int* nbs) {
  for (int bt = 8; bt >= 2; --bt) {
    const int a = (bits_a + bt - 1) / bt, b = (bits_b + bt - 1) / bt;
    const double g = std::min(a, b);
    const double mx = (double)((1 << bt) - 1);
    if (g * (double)k * mx * mx < 16777216.0) {
      *beta = bt; *na = a; *nbs = b;
      return;
    }
  }
  *beta = 1; *na = bits_a; *nbs = bits_b;
}

template <class TA, class TB>
int ozaki_zgemm(olc_context* ctx, int m, int n, int k, const TA* A, long long sA, int lda,
                bool conjA, int bits_a, const TB* B, long long sB, int ldb, int bits_b, double* C,
                int nb, int stage, bool hermitian) {
  // the hand-written tcgen05 kernel (olc_tcgemm.cu) unless OLC_SPLIT_GEMM=cublas
  // selects the library GEMM path below
  const char* path = std::getenv("OLC_SPLIT_GEMM");
  if (!(path && std::strcmp(path, "cublas") == 0))
    return tc::zgemm_fixed<TA, TB>(ctx, m, n, k, A, sA, lda, conjA, bits_a, B, sB, ldb, bits_b, C, nb, stage,
                                   hermitian);
  cudaStream_t st = ctx->stream;
  int beta, na, nbs;
  ozaki_plan(k, bits_a, bits_b, &beta, &na, &nbs);
  const int ngroups = na + nbs - 1;
  // fixed-point accumulators: (int32 group values < 2^25) << beta * groups <= 2^62
  const int per_acc = std::max(1, (62 - 26 - 3) / beta + 1);
  // GEMM dimensions padded to multiples of 8 (16-byte aligned BF16 rows and
  // FP32 output columns); the padding digits are zero
  const int mp = (m + 7) & ~7, np = (n + 7) & ~7, kp = (k + 7) & ~7;
  const bool padded = mp != m || np != n || kp != k;
  // batch chunk so that the group products stay below ~8 GB
  const size_t gbytes = (size_t)ngroups * 16 * (size_t)mp * np;
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(nb, (8ULL << 30) / std::max<size_t>(gbytes, 1)));
  __nv_bfloat16 *wa = nullptr, *wb = nullptr;
  float* G = nullptr;
  int *ea = nullptr, *fb = nullptr;
  int s;
  const size_t abytes = 2ULL * chunk * na * kp * 2 * mp, bbytes = 2ULL * chunk * 2 * np * nbs * kp;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&wa, abytes, st), "malloc digits A"))) return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&wb, bbytes, st), "malloc digits B"))) return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&G, gbytes * chunk, st), "malloc group products"))) return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&ea, 4ULL * chunk * m, st), "malloc ea"))) return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&fb, 4ULL * chunk * n, st), "malloc fb"))) return s;
  StageScope scope(ctx, stage, 0);
  const float one = 1.0f, zero = 0.0f;
  for (int b0 = 0; b0 < nb; b0 += chunk) {
    const int cb = std::min(chunk, nb - b0);
    const TA* Ab = A + (size_t)b0 * sA;
    const TB* Bb = B + (size_t)b0 * sB;
    if (padded) {
      if ((s = cuda_check(cudaMemsetAsync(wa, 0, abytes, st), "clear digits A"))) return s;
      if ((s = cuda_check(cudaMemsetAsync(wb, 0, bbytes, st), "clear digits B"))) return s;
    }
    if (conjA) col_expo_kernel<TA><<<(int)(((size_t)m * cb * 32 + 255) / 256), 256, 0, st>>>(Ab, sA, lda, k, m, cb, ea);
    else row_expo_kernel<TA><<<(int)(((size_t)m * cb + 255) / 256), 256, 0, st>>>(Ab, sA, lda, m, k, cb, ea);
    col_expo_kernel<TB><<<(int)(((size_t)n * cb * 32 + 255) / 256), 256, 0, st>>>(Bb, sB, ldb, k, n, cb, fb);
    slice_left_kernel<TA><<<dim3((m + 31) / 32, (k + 31) / 32, cb), dim3(32, 8), 0, st>>>(
        Ab, sA, lda, conjA, m, k, mp, kp, ea, na, beta, wa);
    slice_right_kernel<TB><<<grid_of((size_t)k * n * cb), 256, 0, st>>>(Bb, sB, ldb, k, n, kp, np, fb, nbs, beta,
                                                                       cb, wb);
    scope.add_launches(4);
    const size_t gstride = (size_t)cb * 4 * mp * np;
    for (int d = 0; d < ngroups; ++d) {
      const int s_lo = std::max(0, d - (nbs - 1)), s_hi = std::min(na - 1, d);
      const int t_hi = d - s_lo;
      const int pairs = s_hi - s_lo + 1;
      cublasStatus_t bs = cublasGemmStridedBatchedEx(
          ctx->blas, CUBLAS_OP_N, CUBLAS_OP_N, 2 * mp, 2 * np, pairs * kp, &one,
          wa + (size_t)s_lo * kp * 2 * mp, CUDA_R_16BF, 2 * mp, (long long)na * kp * 2 * mp,
          wb + (size_t)(nbs - 1 - t_hi) * kp, CUDA_R_16BF, nbs * kp, (long long)2 * np * nbs * kp, &zero,
          G + (size_t)d * gstride, CUDA_R_32F, 2 * mp, 4LL * mp * np, cb, CUBLAS_COMPUTE_32F,
          CUBLAS_GEMM_DEFAULT);
      if (bs != CUBLAS_STATUS_SUCCESS) return fail(OLC_ERR_CUDA, "BF16 digit GEMM failed");
    }
    combine_kernel<<<grid_of((size_t)((m + 3) / 4) * n * cb), 256, 0, st>>>(G, ngroups, gstride, ea, fb, m, n, mp, np, beta,
                                                               per_acc, cb, C + 2 * (size_t)b0 * m * n);
    scope.add_launches(1);
  }
  cudaFreeAsync(wa, st);
  cudaFreeAsync(wb, st);
  cudaFreeAsync(G, st);
  cudaFreeAsync(ea, st);
  cudaFreeAsync(fb, st);
  return cuda_check(cudaGetLastError(), "split-product kernels");
}

template int ozaki_zgemm<double, float>(olc_context*, int, int, int, const double*, long long, int, bool,
                                        int, const float*, long long, int, int, double*, int, int, bool);
template int ozaki_zgemm<float, double>(olc_context*, int, int, int, const float*, long long, int, bool,
                                        int, const double*, long long, int, int, double*, int, int, bool);
template int ozaki_zgemm<double, double>(olc_context*, int, int, int, const double*, long long, int, bool,
                                         int, const double*, long long, int, int, double*, int, int, bool);

}  // namespace olc
