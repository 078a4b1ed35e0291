// Batched FP32 generalised Hermitian eigen-solve of every k at once: the FP32
// stage of the mixed-precision solver (the role LAPACK chegv plays, restated
// for one GPU and all k-points together).
//
//   1. C = W^H H W with W = U^{-1}, S = U^H U: W comes from
//      inverse_factors (FP64 Cholesky and triangular inverse, rounded to
//      FP32, computed once per prepared S); the two products run on the
//      tensor cores (three BF16 pieces per FP32 operand, olc_tcgemm.cu).
//   2. C = Q T Q^H by Householder reflectors H_i = I - tau_i v_i v_i^H, the
//      lower-triangle reduction of LAPACK chetrd in its blocked form: panels
//      of 32 reflectors, one thread-block cluster per k whose CTAs own
//      interleaved columns and rows.  Inside a panel every step reads the
//      trailing matrix once (no write-back: the panel's updates are held back
//      as V, W and applied to the vectors, LAPACK clatrd); the reflector
//      columns and the partial products cross CTAs through distributed shared
//      memory, the cluster barrier orders the steps.  Between panels the
//      trailing matrix takes the panel's rank-64 update on the tensor cores.
//   3. T z = lambda z in FP64: eigenvalues by bisection on FP32 Sturm counts,
//      eigenvectors by FP64 inverse iteration (LU with partial pivoting of
//      T - sigma I, as LAPACK dstein), then modified Gram-Schmidt inside every
//      group of eigenvalues too close for inverse iteration to separate.
//   4. Back-transform Z = Q Z_T in blocks of 128 reflectors written as
//      I - V T V^H (compact WY, LAPACK clarft), four tensor-core products per
//      block.
//   5. X = W Z (tensor-core product).
// X is S-orthonormal and diagonalises H to FP32 accuracy; the Rayleigh-Ritz
// step of the mixed solver takes it from there.
#include <algorithm>
#include <cfloat>
#include <cooperative_groups.h>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "olc_common.h"
#include "olc_tcgemm.h"

namespace cg = cooperative_groups;

namespace olc {

namespace {

constexpr int kWyBlock = 128;        // reflectors per compact-WY block

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// Sum over the CTA in FP64 (red: >= 33 doubles of shared memory).
__device__ __forceinline__ double block_sum_d(double v, double* red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// Two sums over the CTA in FP64 (red: >= 66 doubles).
__device__ __forceinline__ void block_sum2_d(double& a, double& b, double* red) {
  for (int o = 16; o; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5] = a;
    red[32 + (threadIdx.x >> 5)] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0, t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { s += red[q]; t += red[32 + q]; }
    red[64] = s;
    red[65] = t;
  }
  __syncthreads();
  a = red[64];
  b = red[65];
}

// ---------------------------------------------------------------------------
// 2. Householder tridiagonalisation in panels, one cluster of G CTAs per k
// ---------------------------------------------------------------------------
// The lower-triangle reduction of LAPACK chetrd in its blocked form.  A panel
// of kTrdNb reflectors is formed by one hetrd_panel_kernel launch against the
// matrix A_s as it stood at the panel's start, the panel's rank-2 updates held
// back as V, W (A_cur = A_s - V W^H - W V^H, LAPACK clatrd); between panels
// the trailing matrix receives them at once, A22 -= [V W] [W V]^H, an
// FP32-accurate tensor-core product (olc_tcgemm.cu, lower tiles only).
// While a panel runs, A is only read (and column i receives v_i), so the
// HBM stream of each step is one read of the trailing lower triangle.
//
// A: [nk][n][ld] complex FP32, column-major; only the lower triangle is read
// (the upper one holds stale values).  On return column i holds v_i in rows
// i+1..n-1 (v_i(i+1) = 1), d[k][i] the diagonal of T, e[k][i] its (real)
// off-diagonal, tau[k][i] the reflector factors.
// XH, YH: [nk][n][2 kTrdNb]: row r of XH is [conj V(r, :) | conj W(r, :)],
// of YH [conj W(r, :) | conj V(r, :)] -- the operands of the trailing update
// in the K-major layout the tensor-core product reads as op(A) = A^H.
//
// Inside a cluster, column r and row r belong to CTA r % G.  Step i
// (t = i - p0 within the panel):
//  (a) each CTA forms the rows r >= i it owns of column i of A_cur (A_s(r, i)
//      minus the held-back updates: a warp per row, a lane per reflector of
//      the panel) and writes them into every CTA's copy of the column
//      (distributed shared memory), with its share of ||x||^2;  cluster barrier
//  (b) every CTA forms the reflector (v_i, tau_i) from the whole column and
//      stores the rows it owns of v_i into column i of A; streams its columns
//      r > i of A_s once, read only: conj(a) v_i(c) adds to (A_s v_i)(r) and,
//      for c > r, a v_i(r) to (A_s v_i)(c) (shared-memory atomics); forms its
//      rows' share of V^H v_i and W^H v_i (a warp per four columns of XH);
//                                                                cluster barrier
//  (c) sums the cluster's partial products for its rows:
//      p = tau_i (A_s v_i - V (W^H v_i) - W (V^H v_i)), with its share of
//      p^H v_i;                                                   cluster barrier
//  (d) w_i = p - tau_i/2 (p^H v_i) v_i for its rows, into XH and YH.
// Every CTA keeps the panel rows p0..p1-1 of V and W in shared memory: row i
// of both gives the coefficients of column i in (a), so it forms p for the
// panel rows itself.  The column buffer alternates between steps, so that the
// writes of step i+1 into another CTA's buffer never meet that CTA's reads of
// step i.
//
// Deterministic variant (DET): the partial products are accumulated in
// 64-bit fixed point with integer shared-memory atomics, whose sum does not
// depend on the order in which the warps add; the unit of step i is
// 2^-60 of a bound on every partial sum, ||A||_F ||v_i|| (the Frobenius norm
// of the whole matrix bounds every trailing matrix: the reflectors are
// unitary).  Every other sum runs in a fixed order, so a rerun gives
// bit-identical reflectors.  It needs 32 bytes of shared memory per row (the
// float variant 24), so the largest n run the float variant.
constexpr int kTrdThreads = 512;
constexpr int kTrdWarps = kTrdThreads / 32;
constexpr int kTrdNb = 32;        // reflectors per panel: one lane per reflector
constexpr int kTrdXW = 2 * kTrdNb;  // row length of XH, YH
constexpr int kTrdPanel = 8;      // owned columns per warp and pass of the product
constexpr int kTrdMaxG = 16;
static_assert(4 * kTrdWarps == kTrdXW, "a warp per four columns of XH");

// Destination of the partial products A v_i of one CTA.  The sums of row c
// live in four planes of ld/2 words -- (re, even rows), (re, odd rows),
// (im, even rows), (im, odd rows) -- at word c/2, so that the lanes of a warp,
// which add to consecutive row pairs, touch consecutive words.
struct TrdAcc {
  float* f;                       // float variant: shared-memory float sums
  unsigned long long* q;          // DET: fixed-point sums
  float scale;                    // DET: 1 / unit (a power of two)
  int h;                          // words per plane (ld / 2)
};

__device__ __forceinline__ int acc_re(int c, int h) { return (c & 1) * h + (c >> 1); }
__device__ __forceinline__ int acc_im(int c, int h) { return (2 + (c & 1)) * h + (c >> 1); }

template <bool DET>
__device__ __forceinline__ void acc_add(const TrdAcc& a, int c, float x, float y) {
  if (DET) {
    atomicAdd(&a.q[acc_re(c, a.h)], (unsigned long long)__float2ll_rn(x * a.scale));
    atomicAdd(&a.q[acc_im(c, a.h)], (unsigned long long)__float2ll_rn(y * a.scale));
  } else {
    atomicAdd(&a.f[acc_re(c, a.h)], x);
    atomicAdd(&a.f[acc_im(c, a.h)], y);
  }
}

// One row pair (2q, 2q+1) of a set of owned columns cb + t G (t < kTrdPanel;
// a column >= n is an empty slot), the matrix values already loaded: the
// columns' products and the pair's mirrored products.  MASK: the pair may lie
// on or above a column's diagonal.
template <bool DET, bool MASK>
__device__ __forceinline__ void trd_pair(const float4 (&a4)[kTrdPanel], int n, int q, int cb, int G,
                                         const float2 (&vr)[kTrdPanel], float (&ax)[kTrdPanel],
                                         float (&ay)[kTrdPanel], const float4 vc, const TrdAcc& acc) {
  const int c0 = 2 * q;
  float s0x = 0.f, s0y = 0.f, s1x = 0.f, s1y = 0.f;
#pragma unroll
  for (int t = 0; t < kTrdPanel; ++t) {
    const int c = cb + t * G;
    if (c >= n || (MASK && c > c0 + 1)) continue;
    float2 a0 = make_float2(a4[t].x, a4[t].y), a1 = make_float2(a4[t].z, a4[t].w);
    if (MASK) {                     // the diagonal is real
      if (c0 == c) a0.y = 0.f;
      if (c0 + 1 == c) a1.y = 0.f;
    }
    // complex multiply-adds as chains of two fused multiply-adds each
    if (!MASK || c0 >= c) {
      ax[t] = fmaf(a0.x, vc.x, fmaf(a0.y, vc.y, ax[t]));     // conj(a) v
      ay[t] = fmaf(a0.x, vc.y, fmaf(-a0.y, vc.x, ay[t]));
    }
    ax[t] = fmaf(a1.x, vc.z, fmaf(a1.y, vc.w, ax[t]));
    ay[t] = fmaf(a1.x, vc.w, fmaf(-a1.y, vc.z, ay[t]));
    if (!MASK || c0 > c) {
      s0x = fmaf(a0.x, vr[t].x, fmaf(-a0.y, vr[t].y, s0x));
      s0y = fmaf(a0.x, vr[t].y, fmaf(a0.y, vr[t].x, s0y));
    }
    if (!MASK || c0 + 1 > c) {
      s1x = fmaf(a1.x, vr[t].x, fmaf(-a1.y, vr[t].y, s1x));
      s1y = fmaf(a1.x, vr[t].y, fmaf(a1.y, vr[t].x, s1y));
    }
  }
  if (!MASK || s0x != 0.f || s0y != 0.f) acc_add<DET>(acc, c0, s0x, s0y);
  if (!MASK || s1x != 0.f || s1y != 0.f) acc_add<DET>(acc, c0 + 1, s1x, s1y);
}

// One set of kTrdPanel owned columns cb + t G (slots past the last column are
// empty): the pairs touching the diagonals first, then the bulk unmasked
// with two pairs per lane in flight.  A_s is read through the non-coherent
// path: the kernel writes only column i, which no product reads.  Column
// indices and offsets are formed from cb and G where they are used, which
// keeps the loads of both pairs in registers.
template <bool DET>
__device__ __noinline__ void trd_columns(const float2* __restrict__ Ak, int n, int ld, int r0, int G, int pn,
                                            int lane, const float2* vC, const TrdAcc& acc) {
  const int cb = r0 + pn * kTrdPanel * G;       // first column of the set
  float2 vr[kTrdPanel];
  float ax[kTrdPanel], ay[kTrdPanel];
#pragma unroll
  for (int t = 0; t < kTrdPanel; ++t) {
    vr[t] = vC[min(cb + t * G, n - 1)];
    ax[t] = 0.f;
    ay[t] = 0.f;
  }
  const int h = ld >> 1;                        // float4 per column
  const float4* A4 = reinterpret_cast<const float4*>(Ak) + (size_t)cb * h;
  const int hs = G * h;                         // float4 between the set's columns
  const float4* vC4 = reinterpret_cast<const float4*>(vC);
  const int c_last = min(cb + (kTrdPanel - 1) * G, n - 1 - (n - 1 - cb) % G);
  const int q1 = h;                             // the last pair may hold the zero padding row
  const int qd = min(q1, (c_last >> 1) + 1);    // pairs from qd on lie below every diagonal
  int q = (cb >> 1) + lane;
  for (; q < qd; q += 32) {
    float4 a4[kTrdPanel];
#pragma unroll
    for (int t = 0; t < kTrdPanel; ++t) {
      const int c = cb + t * G;
      a4[t] = (c < n && c <= 2 * q + 1) ? __ldg(A4 + (size_t)t * hs + q) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    trd_pair<DET, true>(a4, n, q, cb, G, vr, ax, ay, vC4[q], acc);
  }
  for (; q + 32 < q1; q += 64) {
    float4 a4[kTrdPanel], b4[kTrdPanel];
#pragma unroll
    for (int t = 0; t < kTrdPanel; ++t) {
      const bool ok = cb + t * G < n;
      a4[t] = ok ? __ldg(A4 + (size_t)t * hs + q) : make_float4(0.f, 0.f, 0.f, 0.f);
      b4[t] = ok ? __ldg(A4 + (size_t)t * hs + q + 32) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    trd_pair<DET, false>(a4, n, q, cb, G, vr, ax, ay, vC4[q], acc);
    trd_pair<DET, false>(b4, n, q + 32, cb, G, vr, ax, ay, vC4[q + 32], acc);
  }
  if (q < q1) {
    float4 a4[kTrdPanel];
#pragma unroll
    for (int t = 0; t < kTrdPanel; ++t)
      a4[t] = cb + t * G < n ? __ldg(A4 + (size_t)t * hs + q) : make_float4(0.f, 0.f, 0.f, 0.f);
    trd_pair<DET, false>(a4, n, q, cb, G, vr, ax, ay, vC4[q], acc);
  }
#pragma unroll
  for (int t = 0; t < kTrdPanel; ++t) {
    float x = ax[t], y = ay[t];
    for (int o = 16; o; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if (lane == 0 && cb + t * G < n) acc_add<DET>(acc, cb + t * G, x, y);
  }
}

// Cluster sum of the partial products of row c (in rank order; the remote
// loads of all CTAs are issued together).
template <bool DET>
__device__ __forceinline__ float2 trd_row_sum(cg::cluster_group& cl, int G, int c, const TrdAcc& a, double unit) {
  const int jr = acc_re(c, a.h), ji = acc_im(c, a.h);
  if constexpr (DET) {
    long long qr = 0, qi = 0;     // integer sums: the same in any order
#pragma unroll
    for (int g = 0; g < kTrdMaxG; ++g)
      if (g < G) {
        const unsigned long long* qg = cl.map_shared_rank(a.q, g);
        qr += (long long)qg[jr];
        qi += (long long)qg[ji];
      }
    return make_float2((float)((double)qr * unit), (float)((double)qi * unit));
  } else {
  float ur[kTrdMaxG], ui[kTrdMaxG];
#pragma unroll
  for (int g = 0; g < kTrdMaxG; ++g) {
    ur[g] = 0.f;
    ui[g] = 0.f;
    if (g < G) {
      const float* fg = cl.map_shared_rank(a.f, g);
      ur[g] = fg[jr];
      ui[g] = fg[ji];
    }
  }
  float2 u = make_float2(0.f, 0.f);
#pragma unroll
  for (int g = 0; g < kTrdMaxG; ++g) {
    u.x += ur[g];
    u.y += ui[g];
  }
  return u;
  }
}

// The product p of an owned row past the panel, kept in the row's own sum
// words (only the owner reads the sums of such a row).
template <bool DET>
__device__ __forceinline__ void trd_keep(const TrdAcc& a, int c, float2 p) {
  if (DET) {
    a.q[acc_re(c, a.h)] = __float_as_uint(p.x);
    a.q[acc_im(c, a.h)] = __float_as_uint(p.y);
  } else {
    a.f[acc_re(c, a.h)] = p.x;
    a.f[acc_im(c, a.h)] = p.y;
  }
}
template <bool DET>
__device__ __forceinline__ float2 trd_kept(const TrdAcc& a, int c) {
  if (DET) return make_float2(__uint_as_float((unsigned)a.q[acc_re(c, a.h)]), __uint_as_float((unsigned)a.q[acc_im(c, a.h)]));
  return make_float2(a.f[acc_re(c, a.h)], a.f[acc_im(c, a.h)]);
}

__device__ __forceinline__ float2 warp_sum2(float2 s) {
  for (int o = 16; o; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  return s;
}

// First row >= x owned by CTA `rank` of G.
__device__ __forceinline__ int trd_first_owned(int x, int rank, int G) { return x + ((rank - x) % G + G) % G; }

struct TrdArgs {
  float2* A;
  float2* XH;
  float2* YH;
  double* d;
  double* e;
  float2* tau;
  double* fro;          // [nk] ||A||_F of the matrix entering the first panel
  int n, ld, p0, nbp;   // panel: steps p0 .. p0 + nbp - 1
};

template <bool DET>
__global__ void __launch_bounds__(kTrdThreads, 1) hetrd_panel_kernel(const __grid_constant__ TrdArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int G = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int k = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = a.n, ld = a.ld, p0 = a.p0, p1 = a.p0 + a.nbp;
  float2* Ak = a.A + (size_t)k * n * ld;
  float2* XHk = a.XH + (size_t)k * n * kTrdXW;
  float2* YHk = a.YH + (size_t)k * n * kTrdXW;
  extern __shared__ float4 trd_sm4[];
  float2* vbuf = reinterpret_cast<float2*>(trd_sm4);                 // [2][ld] column / reflector
  float* fsum = reinterpret_cast<float*>(vbuf + 2 * (size_t)ld);       // float variant: [4][ld / 2]
  unsigned long long* qsum = reinterpret_cast<unsigned long long*>(fsum);   // DET: [4][ld / 2]
  __shared__ float2 Vp[kTrdNb][kTrdNb], Wp[kTrdNb][kTrdNb];   // panel rows of V, W: [row - p0][t]
  __shared__ float2 ypart[kTrdXW], ysum[kTrdXW], pp[kTrdNb];
  __shared__ double s_nrm[kTrdMaxG], s_frp[kTrdMaxG];
  __shared__ double2 s_dot[kTrdMaxG];
  __shared__ double red[72];
  __shared__ float2 s_tau, s_scale, s_al2;
  __shared__ float s_diag, s_beta, s_qscale;
  __shared__ double s_unit, s_fro;
  for (int x = tid; x < (DET ? 4 : 3) * ld; x += blockDim.x) vbuf[x] = make_float2(0.f, 0.f);
  for (int x = tid; x < kTrdNb * kTrdNb; x += blockDim.x) {
    (&Vp[0][0])[x] = make_float2(0.f, 0.f);
    (&Wp[0][0])[x] = make_float2(0.f, 0.f);
  }
  if (DET && p0 == 0) {
    // ||A||_F of the lower-triangle storage (off-diagonal entries twice)
    double part = 0.0;
    for (int c = rank; c < n; c += G) {
      const float2* colc = Ak + (size_t)c * ld;
      for (int r = c + tid; r < n; r += blockDim.x) {
        const float2 v = colc[r];
        part += (r == c ? 1.0 : 2.0) * ((double)v.x * v.x + (double)v.y * v.y);
      }
    }
    const double f2 = block_sum_d(part, red);
    if (tid < G) cl.map_shared_rank(s_frp, tid)[rank] = f2;
  }
  __syncthreads();
  cl.sync();
  if (DET && tid == 0) {
    if (p0 == 0) {
      double f2 = 0.0;
      for (int g = 0; g < G; ++g) f2 += s_frp[g];
      s_fro = sqrt(f2);
      if (rank == 0) a.fro[k] = s_fro;
    } else {
      s_fro = a.fro[k];
    }
  }
  int cur = 0;
  for (int i = p0; i < p1; ++i) {
    const int t = i - p0;
    float2* vC = vbuf + (size_t)cur * ld;
    // ---- (a) the owned rows of column i of A_cur, broadcast ---------------------
    {
      // thread per owned row: x = A_s(r, i) - sum_u V(r, u) conj W(i, u) + W(r, u) conj V(i, u)
      //                         = A_s(r, i) - conj(sum_u xv(u) W(i, u) + xw(u) V(i, u))
      double part = 0.0;
      for (int r = trd_first_owned(i, rank, G) + tid * G; r < n; r += blockDim.x * G) {
        float2 x = Ak[(size_t)i * ld + r];
        const float2* xr = XHk + (size_t)r * kTrdXW;
        float sx = 0.f, sy = 0.f;
#pragma unroll 4
        for (int u = 0; u < t; ++u) {
          const float2 xv = xr[u], xw = xr[kTrdNb + u], wq = Wp[t][u], vq = Vp[t][u];
          sx += (xv.x * wq.x - xv.y * wq.y) + (xw.x * vq.x - xw.y * vq.y);
          sy += (xv.x * wq.y + xv.y * wq.x) + (xw.x * vq.y + xw.y * vq.x);
        }
        x.x -= sx;
        x.y += sy;
#pragma unroll
        for (int g = 0; g < kTrdMaxG; ++g)
          if (g < G) cl.map_shared_rank(vC, g)[r] = x;
        if (r >= i + 2) part += (double)x.x * x.x + (double)x.y * x.y;
      }
      const double xn2 = block_sum_d(part, red);
      if (tid < G) cl.map_shared_rank(s_nrm, tid)[rank] = xn2;
    }
    __syncthreads();
    cl.sync();
    // ---- (b) reflector; v_i into column i; products with A_s, V, W ------------------
    if (tid == 0) {
      double xn2 = 0.0;
      for (int g = 0; g < G; ++g) xn2 += s_nrm[g];
      s_diag = vC[i].x;
      const float2 al = vC[i + 1];
      float2 tau = make_float2(0.f, 0.f), scale = make_float2(0.f, 0.f);
      float beta = al.x;
      double vnorm2 = 1.0;
      if (!(xn2 == 0.0 && al.y == 0.f)) {
        const float an = sqrtf(al.x * al.x + al.y * al.y + (float)xn2);
        beta = (al.x >= 0.f) ? -an : an;
        tau = make_float2((beta - al.x) / beta, -al.y / beta);
        const float dr = al.x - beta, di = al.y, den = dr * dr + di * di;
        scale = make_float2(dr / den, -di / den);
        vnorm2 = 1.0 + xn2 / (double)den;
      }
      s_tau = tau;
      s_scale = scale;
      s_beta = beta;
      if (DET) {
        // unit 2^(E - 60) with 2^E >= 2 ||A||_F ||v_i||
        int E;
        frexp(2.0 * s_fro * sqrt(vnorm2) + 1e-300, &E);
        E = max(E, -60);
        s_unit = ldexp(1.0, E - 60);
        s_qscale = ldexpf(1.f, 60 - E);
      }
    }
    __syncthreads();
    {
      const float2 scale = s_scale;
      for (int r = i + 1 + tid; r < n; r += blockDim.x)
        vC[r] = (r == i + 1) ? make_float2(1.f, 0.f) : cmul(vC[r], scale);
      if (tid == 0) vC[i] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int r0 = trd_first_owned(i + 1, rank, G);
    for (int r = r0 + tid * G; r < n; r += blockDim.x * G) Ak[(size_t)i * ld + r] = vC[r];
    {
      const TrdAcc acc{fsum, qsum, DET ? s_qscale : 1.f, ld >> 1};
      const int nown = r0 < n ? (n - r0 + G - 1) / G : 0;
      const int npanel = (nown + kTrdPanel - 1) / kTrdPanel;
      for (int pn = warp; pn < npanel; pn += kTrdWarps) trd_columns<DET>(Ak, n, ld, r0, G, pn, lane, vC, acc);
    }
    {
      // this CTA's share of XH^T v over its rows r > i: warp w takes columns 4w..4w+3
      const int c4 = 4 * warp, u0 = c4 % kTrdNb;
      float2 y[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) y[j] = make_float2(0.f, 0.f);
      if (u0 < t) {
#pragma unroll 4
        for (int r = r0 + lane * G; r < n; r += 32 * G) {
          const float4* xr = reinterpret_cast<const float4*>(XHk + (size_t)r * kTrdXW + c4);
          const float4 q0 = xr[0], q1 = xr[1];
          const float2 vr = vC[r];
          const float2 z[4] = {make_float2(q0.x, q0.y), make_float2(q0.z, q0.w), make_float2(q1.x, q1.y),
                               make_float2(q1.z, q1.w)};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float2 m = cmul(z[j], vr);
            y[j].x += m.x;
            y[j].y += m.y;
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) y[j] = warp_sum2(y[j]);
      }
      if (lane == 0)
#pragma unroll
        for (int j = 0; j < 4; ++j) ypart[c4 + j] = (u0 + j < t) ? y[j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    cl.sync();
    // ---- (c) p = tau (A_s v - V (W^H v) - W (V^H v)) ------------------------------
    if (tid < kTrdXW) {
      float2 u[kTrdMaxG];
#pragma unroll
      for (int g = 0; g < kTrdMaxG; ++g) u[g] = g < G ? cl.map_shared_rank(ypart, g)[tid] : make_float2(0.f, 0.f);
      float2 s = make_float2(0.f, 0.f);
#pragma unroll
      for (int g = 0; g < kTrdMaxG; ++g) {
        s.x += u[g].x;
        s.y += u[g].y;
      }
      ysum[tid] = s;
    }
    __syncthreads();
    {
      const float2 tau = s_tau;
      const double unit = DET ? s_unit : 0.0;
      const TrdAcc sums{fsum, qsum, 1.f, ld >> 1};
      // ysum[nb + u] = (W^H v)(u), ysum[u] = (V^H v)(u)
      double sx = 0.0, sy = 0.0;
      // thread per row.  Panel rows (every CTA): V, W from the tables
      for (int c = i + 1 + tid; c < p1; c += blockDim.x) {
        const float2 P = trd_row_sum<DET>(cl, G, c, sums, unit);
        float qx = 0.f, qy = 0.f;
        for (int u = 0; u < t; ++u) {
          const float2 t1 = cmul(Vp[c - p0][u], ysum[kTrdNb + u]), t2 = cmul(Wp[c - p0][u], ysum[u]);
          qx += t1.x + t2.x;
          qy += t1.y + t2.y;
        }
        const float2 p = cmul(tau, make_float2(P.x - qx, P.y - qy));
        pp[c - p0] = p;
        if (c % G == rank) {
          const float2 v = vC[c];
          sx += (double)p.x * v.x + (double)p.y * v.y;
          sy += (double)p.x * v.y - (double)p.y * v.x;
        }
      }
      // owned rows past the panel: V, W from XH; p kept in the row's own sum
      // slot (only the owner reads the sums of a row past the panel)
      for (int c = trd_first_owned(max(i + 1, p1), rank, G) + tid * G; c < n; c += blockDim.x * G) {
        const float2 P = trd_row_sum<DET>(cl, G, c, sums, unit);
        const float2* xr = XHk + (size_t)c * kTrdXW;
        float qx = 0.f, qy = 0.f;
#pragma unroll 4
        for (int u = 0; u < t; ++u) {
          // V(c, u) (W^H v)(u) + W(c, u) (V^H v)(u), V = conj(xv), W = conj(xw)
          const float2 t1 = cmul(conjf2(xr[u]), ysum[kTrdNb + u]), t2 = cmul(conjf2(xr[kTrdNb + u]), ysum[u]);
          qx += t1.x + t2.x;
          qy += t1.y + t2.y;
        }
        const float2 p = cmul(tau, make_float2(P.x - qx, P.y - qy));
        trd_keep<DET>(sums, c, p);
        const float2 v = vC[c];
        sx += (double)p.x * v.x + (double)p.y * v.y;
        sy += (double)p.x * v.y - (double)p.y * v.x;
      }
      block_sum2_d(sx, sy, red);
      if (tid < G) cl.map_shared_rank(s_dot, tid)[rank] = make_double2(sx, sy);
    }
    __syncthreads();
    cl.sync();
    // ---- (d) w = p + alpha v with alpha = -tau/2 p^H v ------------------------------
    if (tid == 0) {
      const float2 tau = s_tau;
      double sx = 0.0, sy = 0.0;
      for (int g = 0; g < G; ++g) {
        sx += s_dot[g].x;
        sy += s_dot[g].y;
      }
      s_al2 = make_float2((float)(-0.5 * (tau.x * sx - tau.y * sy)), (float)(-0.5 * (tau.x * sy + tau.y * sx)));
      if (rank == 0) {
        a.d[(size_t)k * n + i] = s_diag;
        a.e[(size_t)k * (n - 1) + i] = s_beta;
        a.tau[(size_t)k * (n - 1) + i] = tau;
      }
    }
    __syncthreads();
    {
      const float2 al2 = s_al2;
      const TrdAcc sums{fsum, qsum, 1.f, ld >> 1};
      for (int c = trd_first_owned(p0, rank, G) + tid * G; c < n; c += blockDim.x * G) {
        float2 xv = make_float2(0.f, 0.f), xw = xv;     // conj v(c), conj w(c)
        if (c > i) {
          const float2 v = vC[c];
          const float2 p = c < p1 ? pp[c - p0] : trd_kept<DET>(sums, c);
          const float2 m = cmul(al2, v);
          xv = conjf2(v);
          xw = make_float2(p.x + m.x, -(p.y + m.y));
        }
        XHk[(size_t)c * kTrdXW + t] = xv;
        XHk[(size_t)c * kTrdXW + kTrdNb + t] = xw;
        YHk[(size_t)c * kTrdXW + t] = xw;
        YHk[(size_t)c * kTrdXW + kTrdNb + t] = xv;
      }
      for (int c = i + 1 + tid; c < p1; c += blockDim.x) {
        const float2 v = vC[c], m = cmul(al2, v), p = pp[c - p0];
        Vp[c - p0][t] = v;
        Wp[c - p0][t] = make_float2(p.x + m.x, p.y + m.y);
      }
    }
    __syncthreads();
    // every CTA has read this CTA's sums (cluster barrier above)
    for (int c = i + tid; c < ld; c += blockDim.x) {
      if (DET) {
        qsum[acc_re(c, ld >> 1)] = 0ULL;
        qsum[acc_im(c, ld >> 1)] = 0ULL;
      } else {
        fsum[acc_re(c, ld >> 1)] = 0.f;
        fsum[acc_im(c, ld >> 1)] = 0.f;
      }
    }
    __syncthreads();
    cur ^= 1;
  }
  // last diagonal element: A_s(n-1, n-1) - 2 Re sum_u V(n-1, u) conj W(n-1, u)
  if (p1 == n - 1 && rank == (n - 1) % G && warp == 0) {
    float s = 0.f;
    if (lane < a.nbp) {
      const float2 xv = XHk[(size_t)(n - 1) * kTrdXW + lane], xw = XHk[(size_t)(n - 1) * kTrdXW + kTrdNb + lane];
      s = xv.x * xw.x + xv.y * xw.y;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) a.d[(size_t)k * n + n - 1] = Ak[(size_t)(n - 1) * ld + n - 1].x - 2.f * s;
  }
  cl.sync();
}
// ---------------------------------------------------------------------------
// 3. tridiagonal eigen-solve
// ---------------------------------------------------------------------------
// FP32 copies of T_k for the Sturm counts: df = d, ef = |e| (ef[n-1] = 0).
__global__ void tri_prep_kernel(const double* __restrict__ d, const double* __restrict__ e, int n,
                                int nk, float* __restrict__ df, float* __restrict__ ef) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * nk) return;
  const int k = (int)(t / n), i = (int)(t % n);
  df[t] = (float)d[t];
  ef[t] = i < n - 1 ? fabsf((float)e[(size_t)k * (n - 1) + i]) : 0.f;
}

// Eigenvalue j (ascending) of T_k by multisection on Sturm counts (FP32): the
// count of eigenvalues below x is the number of negative pivots of the LDL^T
// factorisation of T - x I (q_i = d_i - x - e_{i-1}^2 / q_{i-1}, pivots below
// pivmin replaced by -pivmin as in LAPACK dstebz).  Four shifts per pass
// (four independent recurrences in flight) cut the interval five-fold.
__global__ void bisect_kernel(const float* __restrict__ df, const float* __restrict__ ef, int n,
                              int nk, double* __restrict__ lam) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * nk) return;
  const int k = t / n, j = t % n;
  const float* dk = df + (size_t)k * n;
  const float* ek = ef + (size_t)k * n;
  float lo = FLT_MAX, hi = -FLT_MAX, emax2 = 0.f, el = 0.f;
  for (int i = 0; i < n; ++i) {
    const float er = ek[i], di = dk[i];
    lo = fminf(lo, di - el - er);
    hi = fmaxf(hi, di + el + er);
    emax2 = fmaxf(emax2, er * er);
    el = er;
  }
  const float pivmin = 1e-30f * fmaxf(1.f, emax2);
  const float w = fmaxf(fabsf(lo), fabsf(hi));
  lo -= 4e-6f * w + 2.f * pivmin;
  hi += 4e-6f * w + 2.f * pivmin;
  for (int it = 0; it < 40; ++it) {
    if (hi - lo <= 2.f * FLT_EPSILON * fmaxf(fabsf(lo), fabsf(hi)) + pivmin) break;
    const float h = 0.2f * (hi - lo);
    float x[4], q[4];
    int c[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      x[s] = lo + h * (float)(s + 1);
      q[s] = dk[0] - x[s];
      if (fabsf(q[s]) < pivmin) q[s] = -pivmin;
      c[s] = q[s] < 0.f;
    }
    for (int i = 1; i < n; ++i) {
      const float e2 = ek[i - 1] * ek[i - 1], di = dk[i];
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        q[s] = di - x[s] - e2 / q[s];
        if (fabsf(q[s]) < pivmin) q[s] = -pivmin;
        c[s] += q[s] < 0.f;
      }
    }
    float nlo = lo, nhi = hi;
#pragma unroll
    for (int s = 3; s >= 0; --s)
      if (c[s] > j) nhi = x[s];
#pragma unroll
    for (int s = 0; s < 4; ++s)
      if (c[s] <= j) nlo = x[s];
    if (nlo == lo && nhi == hi) break;
    lo = nlo;
    hi = nhi;
  }
  lam[t] = 0.5 * ((double)lo + (double)hi);
}

// Inverse iteration in FP64 for eigenvalue j of T_k (one thread each):
// T - sigma I = P L U with partial pivoting (U has two super-diagonals), tiny
// pivots replaced by eps * ||T||, three solves from a pseudo-random start.
// Work arrays are interleaved ([i][thread]) so that a warp's accesses
// coalesce.  Z: [nk][n][n] FP64, column j = eigenvector j.
__global__ void invit_kernel(const double* __restrict__ d, const double* __restrict__ e,
                             const double* __restrict__ lam, int n, int nk,
                             double* __restrict__ work, unsigned char* __restrict__ piv,
                             double* __restrict__ Z) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int T = n * nk;
  if (t >= T) return;
  const int k = t / n, j = t % n;
  const double* dk = d + (size_t)k * n;
  const double* ek = e + (size_t)k * (n - 1);
  double* Lm = work;                      // multipliers
  double* U0 = work + (size_t)n * T;      // 1 / diagonal of U
  double* U1 = work + (size_t)2 * n * T;  // first super-diagonal
  double* U2 = work + (size_t)3 * n * T;  // second super-diagonal
  double* x = work + (size_t)4 * n * T;   // iterate
  const double sigma = lam[t];
  double tn = 0.0;
  for (int i = 0; i < n; ++i) tn = fmax(tn, fabs(dk[i]) + (i > 0 ? fabs(ek[i - 1]) : 0.0) + (i < n - 1 ? fabs(ek[i]) : 0.0));
  const double tiny = 2.2e-16 * fmax(tn, 1e-300);
  // factorisation
  double a = dk[0] - sigma, b = n > 1 ? ek[0] : 0.0;
  for (int i = 0; i < n - 1; ++i) {
    const double sub = ek[i], nd = dk[i + 1] - sigma, ns = (i + 1 < n - 1) ? ek[i + 1] : 0.0;
    const size_t o = (size_t)i * T + t;
    if (fabs(a) >= fabs(sub)) {
      if (fabs(a) < tiny) a = a >= 0.0 ? tiny : -tiny;
      const double inv = 1.0 / a, m = sub * inv;
      U0[o] = inv; U1[o] = b; U2[o] = 0.0; Lm[o] = m; piv[o] = 0;
      a = nd - m * b;
      b = ns;
    } else {
      const double inv = 1.0 / sub, m = a * inv;
      U0[o] = inv; U1[o] = nd; U2[o] = ns; Lm[o] = m; piv[o] = 1;
      a = b - m * nd;
      b = -m * ns;
    }
  }
  if (fabs(a) < tiny) a = a >= 0.0 ? tiny : -tiny;
  U0[(size_t)(n - 1) * T + t] = 1.0 / a;
  // start vector: a fixed pseudo-random sequence per (j, i)
  unsigned s = 0x9e3779b9u * (unsigned)(j + 1) ^ 0x85ebca6bu;
  for (int i = 0; i < n; ++i) {
    s ^= s << 13; s ^= s >> 17; s ^= s << 5;
    x[(size_t)i * T + t] = (double)(s & 0xffffff) / 16777216.0 - 0.5;
  }
  // the sweeps load their coefficients kInvChunk rows ahead of the
  // dependent arithmetic (one memory latency per chunk instead of per row)
  constexpr int kInvChunk = 8;
  for (int it = 0; it < 3; ++it) {
    // forward: apply P and L; yi carries the current row
    double yi = x[t];
    for (int i0 = 0; i0 < n - 1; i0 += kInvChunk) {
      const int c = min(kInvChunk, n - 1 - i0);
      double Lc[kInvChunk], yn[kInvChunk];
      unsigned char pv[kInvChunk];
#pragma unroll
      for (int u = 0; u < kInvChunk; ++u)
        if (u < c) {
          const size_t o = (size_t)(i0 + u) * T + t;
          Lc[u] = Lm[o];
          pv[u] = piv[o];
          yn[u] = x[o + T];
        }
#pragma unroll
      for (int u = 0; u < kInvChunk; ++u)
        if (u < c) {
          double top = yi, bot = yn[u];
          if (pv[u]) { top = yn[u]; bot = yi; }
          x[(size_t)(i0 + u) * T + t] = top;
          yi = bot - Lc[u] * top;
        }
    }
    x[(size_t)(n - 1) * T + t] = yi;
    // back substitution with U, scaled to max |x| = 1
    double x1 = 0.0, x2 = 0.0, amax = 0.0;
    for (int i0 = n - 1; i0 >= 0; i0 -= kInvChunk) {
      const int c = min(kInvChunk, i0 + 1);
      double xv[kInvChunk], u0[kInvChunk], u1[kInvChunk], u2[kInvChunk];
#pragma unroll
      for (int u = 0; u < kInvChunk; ++u)
        if (u < c) {
          const size_t o = (size_t)(i0 - u) * T + t;
          xv[u] = x[o];
          u0[u] = U0[o];
          u1[u] = U1[o];
          u2[u] = U2[o];
        }
#pragma unroll
      for (int u = 0; u < kInvChunk; ++u)
        if (u < c) {
          const double xi = (xv[u] - u1[u] * x1 - u2[u] * x2) * u0[u];
          x[(size_t)(i0 - u) * T + t] = xi;
          x2 = x1;
          x1 = xi;
          amax = fmax(amax, fabs(xi));
        }
    }
    const double sc = amax > 0.0 ? 1.0 / amax : 1.0;
    for (int i = 0; i < n; ++i) x[(size_t)i * T + t] *= sc;
  }
  double nrm = 0.0;
  for (int i = 0; i < n; ++i) { const double v = x[(size_t)i * T + t]; nrm += v * v; }
  const double sc = 1.0 / sqrt(nrm);
  double* z = Z + ((size_t)k * n + j) * n;
  for (int i = 0; i < n; ++i) z[i] = x[(size_t)i * T + t] * sc;
}

// Modified Gram-Schmidt (twice) inside every group of consecutive
// eigenvalues closer than tol * max|lambda|: inverse iteration cannot separate
// those, any orthonormal basis of their span serves.  Grid (nk, kMgsCtas):
// thread 0 of every CTA lists the k's groups, warp w of CTA c takes groups
// w + 8 c, w + 8 c + 8 kMgsCtas, ...
constexpr int kMgsCtas = 16;
__global__ void __launch_bounds__(256) group_mgs_kernel(const double* __restrict__ lam,
                                                        double* __restrict__ Z, int n, double tol) {
  extern __shared__ int gstart[];
  __shared__ int ng;
  const int k = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
  const int gw = blockIdx.y * (blockDim.x >> 5) + (tid >> 5), nw = gridDim.y * (blockDim.x >> 5);
  const double* lk = lam + (size_t)k * n;
  if (tid == 0) {
    double amax = 0.0;
    for (int j = 0; j < n; ++j) amax = fmax(amax, fabs(lk[j]));
    const double thr = tol * fmax(amax, 1e-300);
    int c = 0, s0 = 0;
    for (int j = 1; j <= n; ++j) {
      if (j == n || lk[j] - lk[j - 1] > thr) {
        if (j - s0 > 1) { gstart[2 * c] = s0; gstart[2 * c + 1] = j; ++c; }
        s0 = j;
      }
    }
    ng = c;
  }
  __syncthreads();
  double* Zk = Z + (size_t)k * n * n;
  for (int g = gw; g < ng; g += nw) {
    const int s0 = gstart[2 * g], s1 = gstart[2 * g + 1];
    for (int m = s0 + 1; m < s1; ++m) {
      double* zm = Zk + (size_t)m * n;
      for (int pass = 0; pass < 2; ++pass) {
        for (int q = s0; q < m; ++q) {
          const double* zq = Zk + (size_t)q * n;
          double dt = 0.0;
          for (int i = lane; i < n; i += 32) dt += zq[i] * zm[i];
          for (int o = 16; o; o >>= 1) dt += __shfl_xor_sync(0xffffffffu, dt, o);
          for (int i = lane; i < n; i += 32) zm[i] -= dt * zq[i];
          __syncwarp();
        }
        double nr = 0.0;
        for (int i = lane; i < n; i += 32) nr += zm[i] * zm[i];
        for (int o = 16; o; o >>= 1) nr += __shfl_xor_sync(0xffffffffu, nr, o);
        const double sc = nr > 0.0 ? 1.0 / sqrt(nr) : 0.0;
        for (int i = lane; i < n; i += 32) zm[i] *= sc;
        __syncwarp();
      }
    }
  }
}

// The tridiagonal eigenvectors as complex FP32 columns of even length
// (Zc [nk][n][ld], a zero padding row for odd n).
__global__ void z_to_c32_kernel(const double* __restrict__ Z, int n, int ld, int nk, float2* __restrict__ Zc) {
  const size_t total = (size_t)nk * n * ld;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % ld);
    const size_t kc = e / ld;          // k * n + column
    Zc[e] = make_float2(r < n ? (float)Z[kc * n + r] : 0.f, 0.f);
  }
}

// ---------------------------------------------------------------------------
// 4. compact-WY back-transform
// ---------------------------------------------------------------------------
// V block: reflectors j0..j0+nb-1 on rows j0..n-1 (L rows; row j0 and the
// rows above each reflector's leading 1 are zero, so that with j0 and n even
// every GEMM operand starts on a 16-byte boundary).  V: [nk][nb][L] complex,
// column-major.
__global__ void build_v_kernel(const float2* __restrict__ A, int n, int ld, int j0, int nb, int L,
                               int nk, float2* __restrict__ V) {
  const size_t total = (size_t)nk * nb * L;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int rr = (int)(e % L);
    const int tcol = (int)((e / L) % nb);
    const int k = (int)(e / ((size_t)L * nb));
    const int r = j0 + rr, j = j0 + tcol;
    V[e] = (r >= j + 1 && r < n) ? A[(size_t)k * n * ld + (size_t)j * ld + r] : make_float2(0.f, 0.f);
  }
}

// T factor of the block (LAPACK clarft, forward, columnwise), one CTA per k:
// T(s,s) = tau_s, T(s,t) = -tau_t sum_{u=s}^{t-1} T(s,u) (V^H V)(u,t); thread s
// owns row s.  Gm: [nk][nb][nb] = V^H V; Tm: [nk][nb][nb] column-major.
__global__ void tfactor_kernel(const float2* __restrict__ Gm, const float2* __restrict__ tau, int n,
                               int j0, int nb, float2* __restrict__ Tm) {
  const int k = blockIdx.x, s = threadIdx.x;
  if (s >= nb) return;
  const float2* G = Gm + (size_t)k * nb * nb;
  const float2* tk = tau + (size_t)k * (n - 1) + j0;
  float2* T = Tm + (size_t)k * nb * nb;
  for (int t = 0; t < nb; ++t) {
    float2 v = make_float2(0.f, 0.f);
    if (t == s) {
      v = tk[s];
    } else if (t > s) {
      float2 acc = make_float2(0.f, 0.f);
      for (int u = s; u < t; ++u) {
        const float2 p = cmul(T[(size_t)u * nb + s], G[(size_t)t * nb + u]);
        acc.x += p.x;
        acc.y += p.y;
      }
      const float2 q = cmul(tk[t], acc);
      v = make_float2(-q.x, -q.y);
    }
    T[(size_t)t * nb + s] = v;
  }
}

// Upper triangle of the FP64 factor (row-major-free: column-major [nk][n][n])
// rounded to FP32, the strictly lower part zero (potrf and trtri leave the
// input's lower triangle in place).
__global__ void upper_to_f32_kernel(const double* __restrict__ in, int n, size_t total, float* __restrict__ out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t r2 = e % ((size_t)n * n);
    const int r = (int)(r2 % n), c = (int)(r2 / n);
    out[2 * e] = r <= c ? (float)in[2 * e] : 0.f;
    out[2 * e + 1] = r <= c ? (float)in[2 * e + 1] : 0.f;
  }
}

}  // namespace

static int max_smem_optin() {
  int dev = 0, smem = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return smem;
}

// Static shared memory of a panel kernel variant.
static size_t trd_static_smem(bool det) {
  cudaFuncAttributes fa{};
  if ((det ? cudaFuncGetAttributes(&fa, hetrd_panel_kernel<true>)
           : cudaFuncGetAttributes(&fa, hetrd_panel_kernel<false>)) != cudaSuccess) {
    cudaGetLastError();
    return 32768;
  }
  return fa.sharedSizeBytes;
}

// Dynamic shared memory of the panel kernel: the two column buffers and the
// partial products, 32 (DET) or 24 (float) bytes per row.
static size_t hetrd_smem(int ld, bool det) { return (det ? 32 : 24) * (size_t)ld; }

// The deterministic variant up to n = kTrdDetMaxN (where its shared memory
// fits too); above, the FP32-atomic variant, whose half-width atomics stream
// the large matrices faster (Si512: 1.86 against 2.27 s per pass).
// OLC_TRD_DET=0 / 1 selects a variant wherever it fits.
constexpr int kTrdDetMaxN = 4096;
static bool hetrd_det(int ld) {
  bool want = ld <= kTrdDetMaxN;
  if (const char* v = std::getenv("OLC_TRD_DET")) want = v[0] != '0';
  if (!want) return false;
  return hetrd_smem(ld, true) + trd_static_smem(true) <= (size_t)max_smem_optin();
}

int hetrd_max_n() {
  return (int)(((size_t)max_smem_optin() - trd_static_smem(false)) / 24) & ~1;
}

// One panel launch with clusters of G CTAs (one cluster per k); G = 16 is a
// non-portable cluster size (allowed explicitly).
static int launch_panel(olc_context* ctx, int G, const TrdArgs& args, int nk, size_t smem, bool det) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(G, nk, 1);
  cfg.blockDim = dim3(kTrdThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (det) return cuda_check(cudaLaunchKernelEx(&cfg, hetrd_panel_kernel<true>, args), "hetrd panel launch");
  return cuda_check(cudaLaunchKernelEx(&cfg, hetrd_panel_kernel<false>, args), "hetrd panel launch");
}

// How many clusters of G CTAs of the panel kernel with this shared memory can
// be resident at once (0: none; 16 exceeds the portable limit and may not fit
// a GPC).
static int max_clusters(int G, size_t smem, bool det) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(G, 1, 1);
  cfg.blockDim = dim3(kTrdThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  const cudaError_t r = det ? cudaOccupancyMaxActiveClusters(&nclusters, hetrd_panel_kernel<true>, &cfg)
                            : cudaOccupancyMaxActiveClusters(&nclusters, hetrd_panel_kernel<false>, &cfg);
  if (r != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nclusters;
}

// The whole reduction: a panel launch per kTrdNb reflectors, the trailing
// update A22 -= [V W] [W V]^H between panels (lower tiles only; the panel
// kernel reads nothing above the diagonal).  first_only: the first panel
// alone (the tuner's sample).
static int hetrd_run(olc_context* ctx, int G, float2* H, int n, int ld, int nk, size_t smem, bool det, double* d,
                     double* e, float2* tau, float2* XH, float2* YH, double* fro, bool first_only) {
  const long long sX = 2LL * n * kTrdXW;          // floats per k of XH, YH
  for (int p0 = 0; p0 < n - 1; p0 += kTrdNb) {
    const int nbp = std::min(kTrdNb, n - 1 - p0);
    const TrdArgs args{H, XH, YH, d, e, tau, fro, n, ld, p0, nbp};
    int st;
    {
      StageScope scope(ctx, OLC_STAGE_TRIDIAG, 1);
      if ((st = launch_panel(ctx, G, args, nk, smem, det))) return st;
    }
    if (first_only) return OLC_OK;
    const int p1 = p0 + nbp;
    if (p1 < n - 1) {
      const int m = n - p1;
      const float* Xf = reinterpret_cast<const float*>(XH) + 2LL * p1 * kTrdXW;
      const float* Yf = reinterpret_cast<const float*>(YH) + 2LL * p1 * kTrdXW;
      float* C = reinterpret_cast<float*>(H) + 2 * ((size_t)p1 * ld + p1);
      if ((st = tc::cgemm_f32(ctx, m, m, kTrdXW, Xf, sX, kTrdXW, true, Yf, sX, kTrdXW, -1.f, 1.f, C, 2LL * n * ld, ld,
                              nk, OLC_STAGE_TRIDIAG, /*lower=*/true)))
        return st;
    }
  }
  return OLC_OK;
}

// Autotuner of the CTAs per k: the first pass of a context for a given
// (n, nk) times the first panel (the longest product of the reduction) with
// every candidate cluster size that keeps the launch within two waves, on a
// copy of the reduced matrices, and keeps the fastest.
static int tune_cluster(olc_context* ctx, const float2* H, int n, int ld, int nk, size_t smem, bool det, double* d,
                        double* e, float2* tau, float2* XH, float2* YH, double* fro, int* G) {
  if (ctx->trd_tuned_n == n && ctx->trd_tuned_nk == nk) {
    *G = ctx->trd_tuned_g;
    return OLC_OK;
  }
  // candidates: the powers of two within two waves, and the largest cluster
  // size whose nk clusters are all resident at once (one wave, which need
  // not be a power of two: a 16-CTA cluster takes a whole GPC)
  int cand[6], nc = 0;
  for (int g = 1; g <= kTrdMaxG; g *= 2)
    if (g * nk <= 2 * 152 && (g * nk >= 38 || g == 8) && max_clusters(g, smem, det) > 0) cand[nc++] = g;
  for (int g = kTrdMaxG; g > 1; --g)
    if (max_clusters(g, smem, det) >= nk) {
      bool have = false;
      for (int j = 0; j < nc; ++j) have |= cand[j] == g;
      if (!have) cand[nc++] = g;
      break;
    }
  if (!nc) cand[nc++] = 1;
  int best = cand[0];
  if (nc > 1) {
    const size_t bytes = sizeof(float2) * (size_t)n * ld * nk;
    float2* scratch = nullptr;
    int st;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&scratch, bytes, ctx->stream), "malloc tuning copy"))) return st;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best_ms = 1e30f;
    for (int i = 0; i < nc; ++i) {
      cudaMemcpyAsync(scratch, H, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
      cudaEventRecord(a, ctx->stream);
      st = hetrd_run(ctx, cand[i], scratch, n, ld, nk, smem, det, d, e, tau, XH, YH, fro, true);
      cudaEventRecord(b, ctx->stream);
      if (!st) st = cuda_check(cudaEventSynchronize(b), "tuning sync");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      if (st) break;
      if (ms < best_ms) { best_ms = ms; best = cand[i]; }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFreeAsync(scratch, ctx->stream);
    if (st) return st;
  }
  ctx->trd_tuned_n = n;
  ctx->trd_tuned_nk = nk;
  ctx->trd_tuned_g = best;
  *G = best;
  return OLC_OK;
}

// W = U^{-1} (S = U^H U) of every k in FP64 -- the Cholesky factorisation
// of S(k) stays in FP64 because diffuse Gaussians make S ill-conditioned --
// rounded to FP32 into w32 ([nk][n][n] complex, upper triangular).
// ctx->d_info receives potrf's info per k (> 0: not positive definite).
// s64: full Hermitian FP64 [nk][n][n], not modified.
int inverse_factors(olc_context* ctx, int n, int nk, const double* s64, float* w32) {
  cudaStream_t stream = ctx->stream;
  const size_t nn = (size_t)n * n;
  int st;
  double* Sd = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&Sd, 16 * nn * nk, stream), "malloc FP64 factor"))) return st;
  if ((st = cuda_check(cudaMemcpyAsync(Sd, s64, 16 * nn * nk, cudaMemcpyDeviceToDevice, stream), "copy S")))
    return st;
  if (!ctx->d_info && (st = dalloc(ctx, &ctx->d_info, (size_t)nk))) return st;
  StageScope scope(ctx, OLC_STAGE_SOLVE, 0);
  cusolverDnSetStream(ctx->solver, stream);
  cusolverDnParams_t params;
  if (cusolverDnCreateParams(&params) != CUSOLVER_STATUS_SUCCESS) return fail(OLC_ERR_CUDA, "cusolver params");
  size_t dws = 0, hws = 0, dws2 = 0, hws2 = 0;
  if (cusolverDnXpotrf_bufferSize(ctx->solver, params, CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, Sd, n, CUDA_C_64F,
                                  &dws, &hws) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnXtrtri_bufferSize(ctx->solver, CUBLAS_FILL_MODE_UPPER, CUBLAS_DIAG_NON_UNIT, n, CUDA_C_64F, Sd, n,
                                  &dws2, &hws2) != CUSOLVER_STATUS_SUCCESS) {
    cusolverDnDestroyParams(params);
    return fail(OLC_ERR_CUDA, "potrf/trtri buffer size");
  }
  dws = std::max(dws, dws2);
  hws = std::max(hws, hws2);
  void* dwork = nullptr;
  int* tinfo = nullptr;        // trtri's info (cannot fail after a successful potrf)
  std::vector<char> hwork(std::max<size_t>(hws, 1));
  if ((st = cuda_check(ctx_malloc(ctx, &dwork, std::max<size_t>(dws, 16), stream), "malloc factor work")) ||
      (st = cuda_check(ctx_malloc(ctx, (void**)&tinfo, sizeof(int) * nk, stream), "malloc trtri info"))) {
    cusolverDnDestroyParams(params);
    return st;
  }
  for (int k = 0; k < nk && !st; ++k) {
    double* Ak = Sd + 2 * nn * k;
    if (cusolverDnXpotrf(ctx->solver, params, CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, Ak, n, CUDA_C_64F, dwork, dws,
                         hwork.data(), hws, ctx->d_info + k) != CUSOLVER_STATUS_SUCCESS)
      st = fail(OLC_ERR_CUDA, "cusolverDnXpotrf failed");
    else if (cusolverDnXtrtri(ctx->solver, CUBLAS_FILL_MODE_UPPER, CUBLAS_DIAG_NON_UNIT, n, CUDA_C_64F, Ak, n, dwork,
                              dws, hwork.data(), hws, tinfo + k) != CUSOLVER_STATUS_SUCCESS)
      st = fail(OLC_ERR_CUDA, "cusolverDnXtrtri failed");
  }
  // d_info keeps potrf's info: a failed factor is refused by mixed_check_info
  ctx->info_potrf = true;
  cusolverDnDestroyParams(params);
  if (st) return st;
  upper_to_f32_kernel<<<(int)std::min<size_t>((nn * nk + 255) / 256, 152 * 16), 256, 0, stream>>>(Sd, n, nn * nk,
                                                                                                 w32);
  scope.add_launches(1);
  cudaFreeAsync(dwork, stream);
  cudaFreeAsync(tinfo, stream);
  cudaFreeAsync(Sd, stream);
  return cuda_check(cudaGetLastError(), "inverse factors");
}

// FP32 eigenvectors X (S-orthonormal, [nk][n][n] complex column-major) of
// every pencil (h32, S) with w32 = U^{-1} from inverse_factors.  h32 is not
// modified.
int solve_fp32_batched(olc_context* ctx, int n, int nk, const float* h32, const float* w32, float* X) {
  cudaStream_t stream = ctx->stream;
  int st;
  if (n < 2) return fail(OLC_ERR_UNSUPPORTED, "batched FP32 solver needs n >= 2");
  if (n > hetrd_max_n()) return fail(OLC_ERR_UNSUPPORTED, "batched FP32 solver: n above the shared-memory limit");
  // the reduced matrix and the tridiagonal eigenvectors keep columns of even
  // length (a zero row for odd n) so that every column starts on a 16-byte
  // boundary; nn = batch stride of those, n2 = batch stride of h32, w32, X
  const int ld = n + (n & 1);
  const size_t nn = (size_t)n * ld, n2 = (size_t)n * n;
  float2 *C = nullptr, *Zc = nullptr;
  float* T = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&C, 8 * nn * nk, stream), "malloc reduced matrix"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&Zc, 8 * nn * nk, stream), "malloc Z"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&T, 8 * n2 * nk, stream), "malloc H W"))) return st;
  if (ld != n && (st = cuda_check(cudaMemsetAsync(C, 0, 8 * nn * nk, stream), "clear padding"))) return st;
  // ---- 1. C = W^H (H W) ------------------------------------------------------
  // W is upper triangular: H W skips the K blocks below each column, W^H (H W)
  // those right of each row
  if ((st = tc::cgemm_f32(ctx, n, n, n, h32, 2 * (long long)n2, n, false, w32, 2 * (long long)n2, n, 1.f, 0.f, T,
                          2 * (long long)n2, n, nk, OLC_STAGE_SOLVE, false, tc::kTriBUpper)))
    return st;
  if ((st = tc::cgemm_f32(ctx, n, n, n, w32, 2 * (long long)n2, n, true, T, 2 * (long long)n2, n, 1.f, 0.f,
                          reinterpret_cast<float*>(C), 2 * (long long)nn, ld, nk, OLC_STAGE_SOLVE, false,
                          tc::kTriALower)))
    return st;
  cudaFreeAsync(T, stream);
  float2* H = C;
  float2* Xc = Zc;
  // ---- 2. tridiagonalisation ----------------------------------------------
  double *d = nullptr, *e = nullptr, *lam = nullptr, *work = nullptr, *Z = nullptr;
  float2* tau = nullptr;
  unsigned char* piv = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&d, 8ULL * n * nk, stream), "malloc d"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&e, 8ULL * (n - 1) * nk, stream), "malloc e"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&tau, 8ULL * (n - 1) * nk, stream), "malloc tau"))) return st;
  {
    // algorithmic traffic: every step reads the trailing lower triangle once;
    // every trailing update reads and writes the lower triangle it changes
    double bytes = 8.0 * ((double)n * n * n - n) / 6.0;
    for (int p1 = kTrdNb; p1 < n - 1; p1 += kTrdNb) bytes += 16.0 * (double)(n - p1) * (n - p1 + 1) / 2.0;
    add_work(ctx, OLC_STAGE_TRIDIAG, 0.0, bytes * nk);
    const bool det = hetrd_det(ld);
    const size_t smem = hetrd_smem(ld, det);
    if ((st = cuda_check(cudaFuncSetAttribute(det ? hetrd_panel_kernel<true> : hetrd_panel_kernel<false>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "hetrd smem"))) return st;
    if ((st = cuda_check(cudaFuncSetAttribute(det ? hetrd_panel_kernel<true> : hetrd_panel_kernel<false>,
                                              cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                         "hetrd cluster size"))) return st;
    float2 *XH = nullptr, *YH = nullptr;
    double* fro = nullptr;
    const size_t xbytes = sizeof(float2) * (size_t)kTrdXW * n * nk;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&XH, xbytes, stream), "malloc XH"))) return st;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&YH, xbytes, stream), "malloc YH"))) return st;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&fro, 8ULL * nk, stream), "malloc fro"))) return st;
    int G = 0;
    if (const char* v = std::getenv("OLC_TRD_CLUSTER")) {
      const int g = std::atoi(v);
      if (g >= 1 && g <= kTrdMaxG) G = g;
    }
    if (!G && (st = tune_cluster(ctx, H, n, ld, nk, smem, det, d, e, tau, XH, YH, fro, &G))) return st;
    if ((st = hetrd_run(ctx, G, H, n, ld, nk, smem, det, d, e, tau, XH, YH, fro, false))) return st;
    cudaFreeAsync(XH, stream);
    cudaFreeAsync(YH, stream);
    cudaFreeAsync(fro, stream);
  }
  // ---- 3. tridiagonal eigen-solve -------------------------------------------
  const size_t TT = (size_t)n * nk;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&lam, 8ULL * TT, stream), "malloc lam"))) return st;
  float *df = nullptr, *ef = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&df, 4ULL * TT, stream), "malloc df"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&ef, 4ULL * TT, stream), "malloc ef"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&work, 8ULL * 5 * n * TT, stream), "malloc invit work"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&piv, (size_t)n * TT, stream), "malloc piv"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&Z, 8ULL * n * n * nk, stream), "malloc Z"))) return st;
  {
    StageScope scope(ctx, OLC_STAGE_SOLVE, 4);
    tri_prep_kernel<<<(int)((TT + 255) / 256), 256, 0, stream>>>(d, e, n, nk, df, ef);
    bisect_kernel<<<(int)((TT + 127) / 128), 128, 0, stream>>>(df, ef, n, nk, lam);
    invit_kernel<<<(int)((TT + 127) / 128), 128, 0, stream>>>(d, e, lam, n, nk, work, piv, Z);
    const size_t gsm = sizeof(int) * 2 * (size_t)(n / 2 + 1);
    if ((st = cuda_check(cudaFuncSetAttribute(group_mgs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)gsm), "mgs smem"))) return st;
    group_mgs_kernel<<<dim3(nk, kMgsCtas), 256, gsm, stream>>>(lam, Z, n, 1e-5);
    z_to_c32_kernel<<<152 * 16, 256, 0, stream>>>(Z, n, ld, nk, Xc);
    scope.add_launches(1);
  }
  cudaFreeAsync(work, stream);
  cudaFreeAsync(piv, stream);
  cudaFreeAsync(df, stream);
  cudaFreeAsync(ef, stream);
  // ---- 4. back-transform Z = Q Z_T ------------------------------------------
  {
    const int nblk = (n - 1 + kWyBlock - 1) / kWyBlock;
    float2 *V = nullptr, *Gm = nullptr, *Tm = nullptr, *W1 = nullptr, *W2 = nullptr;
    const size_t nb = kWyBlock;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&V, 8ULL * nb * n * nk, stream), "malloc V"))) return st;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&Gm, 8ULL * nb * nb * nk, stream), "malloc G"))) return st;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&Tm, 8ULL * nb * nb * nk, stream), "malloc T"))) return st;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&W1, 8ULL * nb * n * nk, stream), "malloc W1"))) return st;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&W2, 8ULL * nb * n * nk, stream), "malloc W2"))) return st;
    float* Vf = reinterpret_cast<float*>(V);
    float* Zf = reinterpret_cast<float*>(Xc);
    for (int b = nblk - 1; b >= 0; --b) {
      const int j0 = b * kWyBlock;
      const int nbb = std::min(kWyBlock, n - 1 - j0);
      const int L = n - j0;
      const long long sV = 2LL * nbb * L, sG = 2LL * nbb * nbb, sW = 2LL * nbb * n;
      {
        StageScope scope(ctx, OLC_STAGE_BACKTRANSFORM, 1);
        build_v_kernel<<<std::min<size_t>((size_t)nbb * L * nk / 256 + 1, 152 * 16), 256, 0, stream>>>(
            H, n, ld, j0, nbb, L, nk, V);
      }
      // G = V^H V, T (clarft), W1 = V^H Z, W2 = T W1, Z -= V W2
      if ((st = tc::cgemm_f32(ctx, nbb, nbb, L, Vf, sV, L, true, Vf, sV, L, 1.f, 0.f,
                              reinterpret_cast<float*>(Gm), sG, nbb, nk, OLC_STAGE_BACKTRANSFORM)))
        return st;
      {
        StageScope scope(ctx, OLC_STAGE_BACKTRANSFORM, 1);
        tfactor_kernel<<<nk, kWyBlock, 0, stream>>>(Gm, tau, n, j0, nbb, Tm);
      }
      if ((st = tc::cgemm_f32(ctx, nbb, n, L, Vf, sV, L, true, Zf + 2 * j0, 2 * (long long)nn, ld, 1.f, 0.f,
                              reinterpret_cast<float*>(W1), sW, nbb, nk, OLC_STAGE_BACKTRANSFORM)))
        return st;
      if ((st = tc::cgemm_f32(ctx, nbb, n, nbb, reinterpret_cast<float*>(Tm), sG, nbb, false,
                              reinterpret_cast<float*>(W1), sW, nbb, 1.f, 0.f, reinterpret_cast<float*>(W2), sW, nbb,
                              nk, OLC_STAGE_BACKTRANSFORM)))
        return st;
      if ((st = tc::cgemm_f32(ctx, L, n, nbb, Vf, sV, L, false, reinterpret_cast<float*>(W2), sW, nbb, -1.f, 1.f,
                              Zf + 2 * j0, 2 * (long long)nn, ld, nk, OLC_STAGE_BACKTRANSFORM)))
        return st;
    }
    cudaFreeAsync(V, stream);
    cudaFreeAsync(Gm, stream);
    cudaFreeAsync(Tm, stream);
    cudaFreeAsync(W1, stream);
    cudaFreeAsync(W2, stream);
  }
  // ---- 5. X = W Z ---------------------------------------------------------------
  if ((st = tc::cgemm_f32(ctx, n, n, n, w32, 2 * (long long)n2, n, false, reinterpret_cast<float*>(Xc),
                          2 * (long long)nn, ld, 1.f, 0.f, X, 2 * (long long)n2, n, nk, OLC_STAGE_BACKTRANSFORM, false,
                          tc::kTriAUpper)))
    return st;
  cudaFreeAsync(C, stream);
  cudaFreeAsync(Zc, stream);
  cudaFreeAsync(d, stream);
  cudaFreeAsync(e, stream);
  cudaFreeAsync(tau, stream);
  cudaFreeAsync(lam, stream);
  cudaFreeAsync(Z, stream);
  return cuda_check(cudaGetLastError(), "batched FP32 solve");
}

}  // namespace olc
