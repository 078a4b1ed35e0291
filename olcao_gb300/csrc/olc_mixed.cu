// Mixed-precision generalised eigen-solve (OLC_PREC_MIXED), for all k at once.
//
// The reference solves every H(k) x = e S(k) x with LAPACK zhegv in FP64
// (solveZHEGV, interfaces.F90:73-120).  On GB300 FP64 arithmetic runs at about
// 1 TFLOP/s while BF16 tensor-core products run above 1 PFLOP/s, so the
// FP64-accurate answer is recovered from an FP32 solve instead:
//
//   1. FP32 pencil: X (n x n, S-orthonormal to FP32 accuracy) from the
//      batched FP32 solver of olc_tridiag.cu (all k in one set of launches).
//   2. Rayleigh-Ritz in that basis with FP64-accurate products:
//        Hh = X^H (H X),  Sh = X^H (S X),
//      each formed error-free from BF16 digits on the tensor cores
//      (olc_tcgemm.cu fixed mode).
//   3. Sh = I + E with E ~ 1e-5: the Loewdin transform (I+F)^H Hh (I+F),
//      F = -E/2 + 3E^2/8, makes the pencil standard to O(E^3); since F is
//      small its products need only FP32 GEMMs.  The basis becomes X (I+F).
//   4. The pencil is now standard and diagonal up to the FP32 error of X.
//      States are grouped into clusters of close diagonal values (gap
//      < 5e-3 Ha, at most 64 states); the rest of the spectrum is folded into
//      each cluster to second order with its first-order energy dependence.
//      A single state gets its shifted energy in closed form; a larger
//      cluster is diagonalised by an FP32 Jacobi solver after the shift by
//      its mean energy (the shifted block's norm is the cluster width, so
//      FP32 rounding stays near 1e-8 Ha).  Eigenvectors are X z.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <cuda_bf16.h>

#include "olc_common.h"
#include "olc_tcgemm.h"

namespace olc {

namespace {

constexpr double kClusterGap = 5e-3;
constexpr int kSortMax = 8192;      // n limit of the in-shared-memory sort

// ---------------------------------------------------------------------------
// conversions
// ---------------------------------------------------------------------------
__global__ void to_c64_kernel(const double* __restrict__ in, float* __restrict__ out, size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 32); }

// Bits per slice so that a length-2k sum of slice products stays below 2^24
// (exact in FP32): 2 beta + ceil(log2(2k)) <= 24.

// ---------------------------------------------------------------------------
// extraction
// ---------------------------------------------------------------------------
constexpr int kMaxCluster = 64;     // states per exactly-solved block
constexpr int kMaxCore = 48;        // core of a cluster cut out of a longer run
constexpr int kBuffer = 8;          // neighbours solved with a cut core on each cut side
constexpr int kSmallCluster = 16;   // blocks up to this size use the small kernel

struct ClusterLists {
  int* order;      // [nk][n] state held by each sorted slot
  int* pos;        // [nk][n] sorted slot of each state
  double* diag;    // [nk][n] a_j = Hh_jj
  int* csize;      // [nk][n] size of the cluster holding each slot
  int4* small;     // (k, first slot, size, cut flags): blocks of up to kSmallCluster states
  int4* large;     // larger blocks; flags bit 0 / 1: cut on the low / high side
  int* counters;   // [4] small count, large count, small next, large next
  int cap;         // capacity of each list
};

// Per k (one CTA): a_j = Re Hh_jj (the basis is orthonormal after the Loewdin
// step), sorted ascending (bitonic sort in shared memory); fills order, pos
// and diag of L.
__global__ void __launch_bounds__(1024) cluster_sort_kernel(const double* __restrict__ Hh, int n,
                                                            ClusterLists L) {
  extern __shared__ double sortmem[];
  int P = 1;
  while (P < n) P <<= 1;
  double* key = sortmem;
  int* idx = reinterpret_cast<int*>(sortmem + P);
  const int k = blockIdx.x, tid = threadIdx.x;
  const size_t nn = (size_t)n * n;
  for (int i = tid; i < P; i += blockDim.x) {
    if (i < n) {
      const double h = Hh[2 * ((size_t)k * nn + (size_t)i * n + i)];
      key[i] = h;
      L.diag[(size_t)k * n + i] = h;
    } else {
      key[i] = 1e300;
    }
    idx[i] = i;
  }
  __syncthreads();
  for (int size = 2; size <= P; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = tid; i < P; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const bool greater = key[i] > key[j] || (key[i] == key[j] && idx[i] > idx[j]);
          if (greater == up) {
            const double t = key[i]; key[i] = key[j]; key[j] = t;
            const int u = idx[i]; idx[i] = idx[j]; idx[j] = u;
          }
        }
      }
      __syncthreads();
    }
  for (int i = tid; i < n; i += blockDim.x) {
    L.order[(size_t)k * n + i] = idx[i];
    L.pos[(size_t)k * n + idx[i]] = i;
  }
}

// Strong couplings, one warp per (k, state p): the second-order fold treats
// the coupling A_jp of p to a state j of another cluster only approximately
// (its neglected terms grow with |A_jp| / |a_p - a_j|).  Where that ratio
// exceeds kCoupleRatio (and |A_jp| exceeds kCoupleFloor) the two states must
// be solved exactly in one cluster: reach[k][pos p] receives the largest
// sorted slot of such a partner above p (integer maximum: the result does not
// depend on the order of the warps).
constexpr double kCoupleRatio = 1e-2;
constexpr double kCoupleFloor = 1e-9;
__global__ void __launch_bounds__(256) coupling_reach_kernel(const double* __restrict__ Hh, int n, int nk,
                                                             ClusterLists L, double ratio,
                                                             int* __restrict__ reach) {
  const int gw = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (gw >= n * nk) return;
  const int k = gw / n, p = gw % n;
  const size_t nn = (size_t)n * n;
  const double* diag = L.diag + (size_t)k * n;
  const int* pos = L.pos + (size_t)k * n;
  const double ap = diag[p];
  const int pp = pos[p];
  const double* col = Hh + 2 * ((size_t)k * nn + (size_t)p * n);
  int far = -1;
  for (int j = lane; j < n; j += 32) {
    const int pj = pos[j];
    if (pj <= pp) continue;
    const double ar = col[2 * j], ai = col[2 * j + 1];
    const double a2 = ar * ar + ai * ai;
    const double dlt = fabs(ap - diag[j]);
    if (a2 > kCoupleFloor * kCoupleFloor && a2 > ratio * ratio * dlt * dlt) far = max(far, pj);
  }
  for (int o = 16; o; o >>= 1) far = max(far, __shfl_xor_sync(0xffffffffu, far, o));
  if (lane == 0 && far >= 0) atomicMax(&reach[(size_t)k * n + pp], far);
}

// Clusters, one CTA per k (sorted values and reaches staged in shared memory,
// one thread scans): runs of sorted values closer than kClusterGap,
// joined across a boundary when a strong coupling (reach) crosses it.  A run
// longer than kMaxCluster is cut into cores of at most kMaxCore states at its
// widest gaps; a core is later solved together with kBuffer neighbours on
// each cut side (only its own eigenpairs are kept), so that the strongly
// coupled states across a cut are treated exactly.  Appends every cluster
// except clean single states to a work list.
__global__ void __launch_bounds__(256) cluster_form_kernel(int n, ClusterLists L, const int* __restrict__ reach,
                                                           double gap) {
  extern __shared__ double formmem[];
  double* keys = formmem;
  int* rk = reinterpret_cast<int*>(formmem + n);
  const int k = blockIdx.x;
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    keys[s] = L.diag[(size_t)k * n + L.order[(size_t)k * n + s]];
    rk[s] = reach[(size_t)k * n + s];
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  auto key = [&](int s) { return keys[s]; };
  // a cluster [s0, s1) with cut flags; clean singletons go to the warp kernel
  auto close = [&](int s0, int s1, int flags) {
    const int m = s1 - s0;
    for (int s = s0; s < s1; ++s) L.csize[(size_t)k * n + s] = flags ? -m : m;
    if (m > 1 || flags) {
      const int ext = m + ((flags & 1) ? min(kBuffer, s0) : 0) + ((flags & 2) ? min(kBuffer, n - s1) : 0);
      const bool sm = ext <= kSmallCluster;
      const int at = atomicAdd(L.counters + (sm ? 0 : 1), 1);
      if (at < L.cap) (sm ? L.small : L.large)[at] = make_int4(k, s0, m, flags);
    }
  };
  int s0 = 0, span = rk[0];
  for (int i = 1; i <= n; ++i) {
    if (i < n && (key(i) - key(i - 1) < gap || span >= i)) {
      span = max(span, rk[i]);
      continue;
    }
    // run [s0, i)
    if (i - s0 <= kMaxCluster) {
      close(s0, i, 0);
    } else {
      // cores of at most kMaxCore states, each ending at the widest gap
      // it can reach; cut sides are solved with buffer states
      int cur = s0, cutl = 0;
      while (i - cur > kMaxCore) {
        int g = cur + 1;
        for (int t = cur + 2; t <= cur + kMaxCore; ++t)
          if (key(t) - key(t - 1) > key(g) - key(g - 1)) g = t;
        close(cur, g, cutl | 2);
        cur = g;
        cutl = 1;
      }
      close(cur, i, cutl);
    }
    s0 = i;
    if (i < n) span = rk[i];
  }
}

// One warp per single-state cluster: the rest of the spectrum folded in to
// second order with its first-order energy dependence,
//   E = a_p + F1 (1 - D2),  F1 = sum_j |A_jp|^2 / (a_p - a_j),
//                           D2 = sum_j |A_jp|^2 / (a_p - a_j)^2,
// and the basis vector as eigenvector.  The couplings A_jp are ~1e-6 of H
// (the basis diagonalises H to FP32 accuracy), so F1 and D2 need only FP32.
__global__ void __launch_bounds__(256) singleton_kernel(const double* __restrict__ Hh,
                                                        const float* __restrict__ X,
                                                        ClusterLists L, int n, int nk,
                                                        double* __restrict__ w_slot,
                                                        double* __restrict__ v_slot) {
  const int gw = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (gw >= n * nk) return;
  const int k = gw / n, slot = gw % n;
  if (L.csize[(size_t)k * n + slot] != 1) return;
  const size_t nn = (size_t)n * n;
  const int p = L.order[(size_t)k * n + slot];
  const double* diag = L.diag + (size_t)k * n;
  const double ap = diag[p];
  const double* col = Hh + 2 * ((size_t)k * nn + (size_t)p * n);
  float f1 = 0.f, d2 = 0.f;
  for (int j = lane; j < n; j += 32) {
    const double dlt = ap - diag[j];
    if (j == p || fabs(dlt) < 1e-9) continue;
    const float w = 1.0f / (float)dlt;
    const float ar = (float)col[2 * j], ai = (float)col[2 * j + 1];
    const float a2 = ar * ar + ai * ai;
    f1 += a2 * w;
    d2 += a2 * w * w;
  }
  for (int o = 16; o; o >>= 1) {
    f1 += __shfl_xor_sync(0xffffffffu, f1, o);
    d2 += __shfl_xor_sync(0xffffffffu, d2, o);
  }
  if (lane == 0) w_slot[(size_t)k * n + slot] = ap + (double)f1 * (1.0 - (double)d2);
  if (!v_slot) return;
  const float* x = X + 2 * ((size_t)k * nn + (size_t)p * n);
  double* o = v_slot + 2 * ((size_t)k * nn + (size_t)slot * n);
  for (int r = lane; r < n; r += 32) {
    const float2 v = reinterpret_cast<const float2*>(x)[r];
    o[2 * r] = v.x;
    o[2 * r + 1] = v.y;
  }
}

template <int MAXM>
struct ClusterSmem {
  float2 C[MAXM * MAXM];     // A - lc I + F1, then diag = eigenvalue shifts
  float2 V[MAXM * MAXM];     // eigenvectors z
  float2 D[MAXM * MAXM];     // D2
  float2 Cp[32 * MAXM];      // [32][m] couplings A_jp of one chunk of j
  float w[32];               // 1 / (lc - a_j) of the chunk (0 inside the cluster)
  int cidx[MAXM];
  int sel[MAXM];             // block eigenpair of each core slot
  float red[32];
  float off, fro;
  int item, rotated;
  double lc;
  int pp[MAXM / 2], qq[MAXM / 2];
  float c[MAXM / 2], s[MAXM / 2], phx[MAXM / 2], phy[MAXM / 2];
};

__device__ __forceinline__ float block_sum(float v, float* red, float* out) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    *out = t;
  }
  __syncthreads();
  return *out;
}

// Standard Hermitian eigen-solve of the m x m FP32 block S.C by parallel
// cyclic Jacobi (round-robin pairs, the rotation of LAPACK's zheev-free
// two-sided scheme: J = diag(1, e^{-i phi}) R(theta)); S.V accumulates the
// rotations.  The block is a shift of a cluster of nearly equal energies, so
// its norm is the cluster width: entries below 3e-8 of the Frobenius norm are
// left alone and the sweeps stop once no rotation is applied.
template <int MAXM>
__device__ void jacobi_f32(ClusterSmem<MAXM>& S, int m) {
  const int tid = threadIdx.x;
  for (int e = tid; e < m * m; e += blockDim.x) S.V[e] = make_float2((e % m) == (e / m) ? 1.f : 0.f, 0.f);
  float fro = 0.f;
  for (int e = tid; e < m * m; e += blockDim.x) fro += S.C[e].x * S.C[e].x + S.C[e].y * S.C[e].y;
  fro = sqrtf(block_sum(fro, S.red, &S.fro));
  const float tiny = 3e-8f * fro + 1e-30f;
  const int mm = (m % 2) ? m + 1 : m;
  const int half = mm / 2;
  for (int sweep = 0; sweep < 30; ++sweep) {
    if (tid == 0) S.rotated = 0;
    __syncthreads();
    for (int round = 0; round < mm - 1; ++round) {
      if (tid < half) {
        const int pi = tid;
        int p, q;
        if (pi == 0) { p = round % (mm - 1); q = mm - 1; }
        else { p = (round + pi) % (mm - 1); q = (round - pi + (mm - 1)) % (mm - 1); }
        if (p > q) { const int t = p; p = q; q = t; }
        float c = 1.f, s = 0.f, phx = 1.f, phy = 0.f;
        if (q < m) {
          const float2 cpq = S.C[q * m + p];
          const float b = hypotf(cpq.x, cpq.y);
          if (b > tiny) {
            const float app = S.C[p * m + p].x, aqq = S.C[q * m + q].x;
            const float th = (aqq - app) / (2.f * b);
            const float t = (th >= 0.f ? 1.f : -1.f) / (fabsf(th) + sqrtf(th * th + 1.f));
            c = rsqrtf(t * t + 1.f);
            s = t * c;
            phx = cpq.x / b;
            phy = -cpq.y / b;
            S.rotated = 1;
          }
        }
        S.pp[pi] = p; S.qq[pi] = q; S.c[pi] = c; S.s[pi] = s; S.phx[pi] = phx; S.phy[pi] = phy;
      }
      __syncthreads();
      // columns: C <- C J, V <- V J
      for (int e = tid; e < half * m; e += blockDim.x) {
        const int pi = e / m, r = e % m;
        const int p = S.pp[pi], q = S.qq[pi];
        if (q >= m || S.s[pi] == 0.f) continue;
        const float c = S.c[pi], s = S.s[pi], hx = S.phx[pi], hy = S.phy[pi];
        {
          const float2 xp = S.C[p * m + r], xq = S.C[q * m + r];
          const float eqx = hx * xq.x - hy * xq.y, eqy = hx * xq.y + hy * xq.x;
          S.C[p * m + r] = make_float2(c * xp.x - s * eqx, c * xp.y - s * eqy);
          S.C[q * m + r] = make_float2(s * xp.x + c * eqx, s * xp.y + c * eqy);
        }
        {
          const float2 xp = S.V[p * m + r], xq = S.V[q * m + r];
          const float eqx = hx * xq.x - hy * xq.y, eqy = hx * xq.y + hy * xq.x;
          S.V[p * m + r] = make_float2(c * xp.x - s * eqx, c * xp.y - s * eqy);
          S.V[q * m + r] = make_float2(s * xp.x + c * eqx, s * xp.y + c * eqy);
        }
      }
      __syncthreads();
      // rows: C <- J^H C
      for (int e = tid; e < half * m; e += blockDim.x) {
        const int pi = e / m, col = e % m;
        const int p = S.pp[pi], q = S.qq[pi];
        if (q >= m || S.s[pi] == 0.f) continue;
        const float c = S.c[pi], s = S.s[pi], hx = S.phx[pi], hy = -S.phy[pi];
        const float2 xp = S.C[col * m + p], xq = S.C[col * m + q];
        const float eqx = hx * xq.x - hy * xq.y, eqy = hx * xq.y + hy * xq.x;
        S.C[col * m + p] = make_float2(c * xp.x - s * eqx, c * xp.y - s * eqy);
        S.C[col * m + q] = make_float2(s * xp.x + c * eqx, s * xp.y + c * eqy);
      }
      __syncthreads();
    }
    const int rotated = S.rotated;
    __syncthreads();
    if (!rotated) break;
  }
}

// Clusters other than clean single states, one work item per CTA at a time
// (items taken from an atomic counter); a cut core is extended by its buffer
// states and keeps the eigenpairs ranked at its own positions.  With lc the cluster's mean energy and
// F1 = sum_j A_.j A_j. / (lc - a_j), D2 = sum_j A_.j A_j. / (lc - a_j)^2 over
// the states j outside the cluster, the folded pencil is
//   (A - lc I + F1) y = (E - lc) (I + D2) y,
// solved as the standard problem (A - lc I + F1) z = mu z in FP32 (its norm is
// the cluster width, so FP32 rounding stays below 1e-8 Ha) with the
// first-order effect of D2, E = lc + mu (1 - z^H D2 z).  Eigenvectors X z.
template <int MAXM>
__global__ void cluster_solve_kernel(const double* __restrict__ Hh, const float* __restrict__ X,
                                     ClusterLists L, const int4* __restrict__ list,
                                     const int* __restrict__ count, int* __restrict__ next, int n,
                                     double* __restrict__ w_slot, double* __restrict__ v_slot) {
  extern __shared__ __align__(16) unsigned char smraw[];
  ClusterSmem<MAXM>& S = *reinterpret_cast<ClusterSmem<MAXM>*>(smraw);
  const int tid = threadIdx.x;
  const size_t nn = (size_t)n * n;
  const int total = min(*count, L.cap);
  constexpr int TP = (MAXM + 3) / 4;          // 4 x 4 tiles per side
  for (;;) {
    if (tid == 0) S.item = atomicAdd(next, 1);
    __syncthreads();
    const int item = S.item;
    if (item >= total) break;
    const int4 it = list[item];
    const int k = it.x, s0c = it.y, mc = it.z;
    // the block: the core [s0c, s0c + mc) and buffer states on cut sides
    const int bl = (it.w & 1) ? min(kBuffer, s0c) : 0;
    const int br = (it.w & 2) ? min(kBuffer, n - s0c - mc) : 0;
    const int s0 = s0c - bl, m = mc + bl + br;
    const double* H = Hh + 2 * (size_t)k * nn;
    const double* diag = L.diag + (size_t)k * n;
    const int* pos = L.pos + (size_t)k * n;
    for (int p = tid; p < m; p += blockDim.x) S.cidx[p] = L.order[(size_t)k * n + s0 + p];
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int p = bl; p < bl + mc; ++p) t += diag[S.cidx[p]];
      S.lc = t / mc;
    }
    __syncthreads();
    const double lc = S.lc;
    // ---- fold the outside states: 4 x 4 tile of (p, q) per thread -----------
    const int tp = tid % TP, tq = tid / TP;
    const bool own = tq < TP && 4 * tp < m && 4 * tq < m;
    float fr[4][4], fi[4][4], dr[4][4], di[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) fr[a][b] = fi[a][b] = dr[a][b] = di[a][b] = 0.f;
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int J = min(32, n - j0);
      for (int e = tid; e < 32 * m; e += blockDim.x) {
        const int jj = e % 32, p = e / 32;
        float2 v = make_float2(0.f, 0.f);
        if (jj < J) {
          const int j = j0 + jj;
          if ((unsigned)(pos[j] - s0) >= (unsigned)m) {
            const double* src = H + 2 * ((size_t)S.cidx[p] * n + j);   // A(j, p)
            v = make_float2((float)src[0], (float)src[1]);
          }
        }
        S.Cp[jj * MAXM + p] = v;
      }
      for (int jj = tid; jj < 32; jj += blockDim.x) {
        float w = 0.f;
        if (jj < J) {
          const int j = j0 + jj;
          const double dlt = lc - diag[j];
          if ((unsigned)(pos[j] - s0) >= (unsigned)m && fabs(dlt) >= 1e-9) w = 1.0f / (float)dlt;
        }
        S.w[jj] = w;
      }
      __syncthreads();
      if (own) {
        for (int jj = 0; jj < J; ++jj) {
          const float w = S.w[jj], w2 = w * w;
          float2 x[4], y[4];
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            x[a] = S.Cp[jj * MAXM + min(4 * tp + a, MAXM - 1)];
            y[a] = S.Cp[jj * MAXM + min(4 * tq + a, MAXM - 1)];
          }
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
              // conj(A(j,p)) A(j,q) = A(p,j) A(j,q)
              const float tr = x[a].x * y[b].x + x[a].y * y[b].y;
              const float ti = x[a].x * y[b].y - x[a].y * y[b].x;
              fr[a][b] += w * tr;
              fi[a][b] += w * ti;
              dr[a][b] += w2 * tr;
              di[a][b] += w2 * ti;
            }
        }
      }
      __syncthreads();
    }
    // ---- the shifted block and D2 ------------------------------------------
    if (own) {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int p = 4 * tp + a, q = 4 * tq + b;
          if (p < m && q < m) {
            const double* src = H + 2 * ((size_t)S.cidx[q] * n + S.cidx[p]);   // A(p, q)
            const double re = src[0] - (p == q ? lc : 0.0);
            S.C[q * m + p] = make_float2((float)re + fr[a][b], (p == q) ? 0.f : (float)src[1] + fi[a][b]);
            S.D[q * m + p] = make_float2(dr[a][b], (p == q) ? 0.f : di[a][b]);
          }
        }
    }
    __syncthreads();
    jacobi_f32<MAXM>(S, m);
    // ---- the core's eigenpairs: block eigenvalues ranked bl .. bl + mc - 1 ----
    for (int i = tid; i < m; i += blockDim.x) {
      const float mi = S.C[i * m + i].x;
      int rank = 0;
      for (int j = 0; j < m; ++j) {
        const float mj = S.C[j * m + j].x;
        rank += (mj < mi) || (mj == mi && j < i);
      }
      if (rank >= bl && rank < bl + mc) S.sel[rank - bl] = i;
    }
    __syncthreads();
    // ---- eigenvalues: E = lc + mu (1 - z^H D2 z) ------------------------------
    for (int t = tid; t < mc; t += blockDim.x) {
      const int i = S.sel[t];
      float dre = 0.f;
      for (int q = 0; q < m; ++q) {
        float2 acc = make_float2(0.f, 0.f);      // (D2 z)_q
        for (int p = 0; p < m; ++p) {
          const float2 d = S.D[p * m + q], z = S.V[i * m + p];
          acc.x += d.x * z.x - d.y * z.y;
          acc.y += d.x * z.y + d.y * z.x;
        }
        const float2 zq = S.V[i * m + q];
        dre += zq.x * acc.x + zq.y * acc.y;      // Re conj(z_q) (D z)_q
      }
      const double mu = S.C[i * m + i].x;
      w_slot[(size_t)k * n + s0c + t] = lc + mu * (1.0 - (double)dre);
    }
    // ---- eigenvectors x_i = X z_i ---------------------------------------------
    if (v_slot) {
      const float2* Xk = reinterpret_cast<const float2*>(X) + (size_t)k * nn;
      for (int i0 = 0; i0 < mc; i0 += 8) {
        const int I = min(8, mc - i0);
        for (int row = tid; row < n; row += blockDim.x) {
          float ar[8], ai[8];
#pragma unroll
          for (int b = 0; b < 8; ++b) ar[b] = ai[b] = 0.f;
          for (int p = 0; p < m; ++p) {
            const float2 xv = Xk[(size_t)S.cidx[p] * n + row];
#pragma unroll
            for (int b = 0; b < 8; ++b) {
              const float2 z = S.V[S.sel[min(i0 + b, mc - 1)] * m + p];
              ar[b] += xv.x * z.x - xv.y * z.y;
              ai[b] += xv.x * z.y + xv.y * z.x;
            }
          }
          for (int b = 0; b < I; ++b) {
            double* o = v_slot + 2 * ((size_t)k * nn + (size_t)(s0c + i0 + b) * n + row);
            o[0] = ar[b];
            o[1] = ai[b];
          }
        }
      }
    }
    __syncthreads();
  }
}

// Final ascending order over all clusters (one CTA per k): the eigenvalues,
// and the slot of each output column in perm [nk][n] for gather_vectors_kernel.
__global__ void __launch_bounds__(1024) final_sort_kernel(const double* __restrict__ w_slot,
                                                          int n, int num_states,
                                                          double* __restrict__ eig,
                                                          int* __restrict__ perm) {
  extern __shared__ double sortmem[];
  int P0 = 1;
  while (P0 < n) P0 <<= 1;
  double* key = sortmem;
  int* idx = reinterpret_cast<int*>(sortmem + P0);
  const int k = blockIdx.x, tid = threadIdx.x;
  int P = 1;
  while (P < n) P <<= 1;
  for (int i = tid; i < P; i += blockDim.x) {
    key[i] = i < n ? w_slot[(size_t)k * n + i] : 1e300;
    idx[i] = i;
  }
  __syncthreads();
  for (int size = 2; size <= P; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = tid; i < P; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          if ((key[i] > key[j]) == up) {
            const double t = key[i]; key[i] = key[j]; key[j] = t;
            const int u = idx[i]; idx[i] = idx[j]; idx[j] = u;
          }
        }
      }
      __syncthreads();
    }
  for (int i = tid; i < num_states; i += blockDim.x) {
    eig[(size_t)k * num_states + i] = key[i];
    perm[(size_t)k * n + i] = idx[i];
  }
}

// Eigenvectors in the sorted order, every k at once (grid-stride over
// [nk][num_states][n] complex).
__global__ void gather_vectors_kernel(const double2* __restrict__ v_slot, const int* __restrict__ perm, int n,
                                      int num_states, int nk, double2* __restrict__ vec) {
  const size_t per = (size_t)n * num_states, total = per * nk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t k = e / per, r = e % per;
    const int row = (int)(r % n), col = (int)(r / n);
    vec[e] = v_slot[(k * n + (size_t)perm[k * n + col]) * n + row];
  }
}

}  // namespace

namespace {

// E = Sh - I (FP32), and the FP32 copy of Hh
__global__ void loewdin_prep_kernel(const double* __restrict__ Hh, const double* __restrict__ Sh,
                                    int n, size_t total, float* __restrict__ E,
                                    float* __restrict__ H32) {
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const size_t r = idx % ((size_t)n * n);
    const int row = (int)(r % n), col = (int)(r / n);
    E[2 * idx] = (float)(Sh[2 * idx] - (row == col ? 1.0 : 0.0));
    E[2 * idx + 1] = (float)Sh[2 * idx + 1];
    H32[2 * idx] = (float)Hh[2 * idx];
    H32[2 * idx + 1] = (float)Hh[2 * idx + 1];
  }
}

// F = -E/2 + (3/8) E2   (in place in E2)
__global__ void loewdin_f_kernel(const float* __restrict__ E, float* __restrict__ E2, size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x)
    E2[i] = -0.5f * E[i] + 0.375f * E2[i];
}

// out (FP64) = base (FP64) + add (FP32); optional FP32 copy of the sum
__global__ void add_f32_kernel(double* __restrict__ out, const double* __restrict__ base,
                               const float* __restrict__ add, float* __restrict__ copy32,
                               size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x) {
    const double v = base[i] + (double)add[i];
    out[i] = v;
    if (copy32) copy32[i] = (float)v;
  }
}

// Sh := I (the transformed pencil is standard)
__global__ void set_identity_kernel(double* __restrict__ S, int n, size_t total) {
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const size_t r = idx % ((size_t)n * n);
    S[2 * idx] = ((int)(r % n) == (int)(r / n)) ? 1.0 : 0.0;
    S[2 * idx + 1] = 0.0;
  }
}


}  // namespace

// Hh := (I+F)^H Hh (I+F), Sh := I, X := X (I+F) with F = -E/2 + 3E^2/8, E = Sh - I.
// The products with the small F run as FP32-accurate tensor-core products
// (olc_tcgemm.cu): their relative error times |F| ~ 1e-5 is far below FP64
// needs.
int loewdin(olc_context* ctx, int n, int nk, double* Hh, double* Sh, float* X) {
  cudaStream_t stream = ctx->stream;
  const size_t nn = (size_t)n * n, total = nn * nk;
  const long long s2 = 2 * (long long)nn;     // batch stride in floats
  float *E = nullptr, *F = nullptr, *H32 = nullptr, *T = nullptr;
  int st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&E, 8 * total, stream), "malloc E"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&F, 8 * total, stream), "malloc F"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&H32, 8 * total, stream), "malloc H32"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&T, 8 * total, stream), "malloc T"))) return st;
  {
    StageScope scope(ctx, OLC_STAGE_REFINE, 1);
    loewdin_prep_kernel<<<grid_for(total), 256, 0, stream>>>(Hh, Sh, n, total, E, H32);
  }
  auto gemm = [&](const float* A, bool conjA, const float* B, float beta, float* C) {
    return tc::cgemm_f32(ctx, n, n, n, A, s2, n, conjA, B, s2, n, 1.f, beta, C, s2, n, nk, OLC_STAGE_REFINE);
  };
  if ((st = gemm(E, false, E, 0.f, F))) return st;                 // F = E^2
  {
    StageScope scope(ctx, OLC_STAGE_REFINE, 1);
    loewdin_f_kernel<<<grid_for(2 * total), 256, 0, stream>>>(E, F, 2 * total);
  }
  // W = Hh + Hh F  (into Hh, FP32 copy into H32)
  if ((st = gemm(H32, false, F, 0.f, T))) return st;
  {
    StageScope scope(ctx, OLC_STAGE_REFINE, 1);
    add_f32_kernel<<<grid_for(2 * total), 256, 0, stream>>>(Hh, Hh, T, H32, 2 * total);
  }
  // Hh' = W + F^H W
  if ((st = gemm(F, true, H32, 0.f, T))) return st;
  {
    StageScope scope(ctx, OLC_STAGE_REFINE, 2);
    add_f32_kernel<<<grid_for(2 * total), 256, 0, stream>>>(Hh, Hh, T, nullptr, 2 * total);
    set_identity_kernel<<<grid_for(total), 256, 0, stream>>>(Sh, n, total);
  }
  // X' = X + X F (the operand is split into BF16 pieces before the product
  // writes, so X may be both operand and output)
  if ((st = gemm(X, false, F, 1.f, X))) return st;
  cudaFreeAsync(E, stream);
  cudaFreeAsync(F, stream);
  cudaFreeAsync(H32, stream);
  cudaFreeAsync(T, stream);
  return cuda_check(cudaGetLastError(), "loewdin kernels");
}



// Solve every k with the mixed-precision scheme; h, s are full Hermitian
// FP64 [nk][n][n] (not modified).
int solve_full_mixed(olc_context* ctx, const double* h, const double* s, int num_states,
                     double* eig_dev, double* vectors, bool check, bool s_prepared) {
  const int n = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  if (n > kSortMax) return fail(OLC_ERR_UNSUPPORTED, "mixed solver: n above 8192");
  const size_t nn = (size_t)n * n;
  int st;
  cudaStream_t stream = ctx->stream;
  // ---- 1. FP32 generalised solve per k -----------------------------------
  // W = U^{-1} (S = U^H U, FP64 factorisation rounded to FP32); the prepared
  // S(k) does not change between passes, so its factors are kept from the
  // first pass
  if (n < 2 || n > hetrd_max_n())
    return fail(OLC_ERR_UNSUPPORTED, "mixed solver: n outside the batched FP32 solver's range");
  float* h32 = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&h32, 8 * nn * nk, stream), "malloc h32"))) return st;
  {
    StageScope scope(ctx, OLC_STAGE_SOLVE, 1);
    to_c64_kernel<<<grid_for(2 * nn * nk), 256, 0, stream>>>(h, h32, 2 * nn * nk);
  }
  float* X = nullptr;      // FP32 eigenvectors, [nk][n][n] complex
  float* w32 = nullptr;
  if (s_prepared) {
    if (!ctx->w32 && (st = dalloc(ctx, &ctx->w32, 2 * nn * nk))) return st;
    w32 = ctx->w32;
    if (!ctx->w32_valid) {
      if ((st = inverse_factors(ctx, n, nk, s, w32))) return st;
      ctx->w32_valid = true;
    } else if ((st = cuda_check(cudaMemsetAsync(ctx->d_info, 0, sizeof(int) * nk, stream), "clear info"))) {
      return st;
    }
  } else {
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&w32, 8 * nn * nk, stream), "malloc w32"))) return st;
    if ((st = inverse_factors(ctx, n, nk, s, w32))) return st;
  }
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&X, 8 * nn * nk, stream), "malloc X"))) return st;
  if ((st = solve_fp32_batched(ctx, n, nk, h32, w32, X))) return st;
  if (!s_prepared) cudaFreeAsync(w32, stream);
  cudaFreeAsync(h32, stream);
  // ---- 2. Rayleigh-Ritz with error-free split products ---------------------
  double *Y = nullptr, *Hh = nullptr, *Sh = nullptr;
  // bits kept of FP64 and FP32 operands (OLC_SPLIT_BITS overrides the FP64 count)
  int b64 = 48;
  const int b32 = 24;
  if (const char* v = std::getenv("OLC_SPLIT_BITS")) b64 = std::max(24, std::min(53, std::atoi(v)));
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&Y, 16ULL * nn * nk, stream), "malloc Y"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&Hh, 16ULL * nn * nk, stream), "malloc Hh"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&Sh, 16ULL * nn * nk, stream), "malloc Sh"))) return st;
  const long long snn = (long long)nn * 2;
  // Y = H X ; Hh = X^H Y
  if ((st = ozaki_zgemm<double, float>(ctx, n, n, n, h, snn, n, false, b64, X, snn, n, b32, Y, nk,
                                       OLC_STAGE_SPLIT))) return st;
  if ((st = ozaki_zgemm<float, double>(ctx, n, n, n, X, snn, n, true, b32, Y, snn, n, b64, Hh, nk,
                                       OLC_STAGE_SPLIT, true))) return st;
  // Y = S X ; Sh = X^H Y
  if ((st = ozaki_zgemm<double, float>(ctx, n, n, n, s, snn, n, false, b64, X, snn, n, b32, Y, nk,
                                       OLC_STAGE_SPLIT))) return st;
  if ((st = ozaki_zgemm<float, double>(ctx, n, n, n, X, snn, n, true, b32, Y, snn, n, b64, Sh, nk,
                                       OLC_STAGE_SPLIT, true))) return st;
  cudaFreeAsync(Y, stream);
  // ---- 3. Loewdin transform: Sh = I + E  ->  (I+F)^H Hh (I+F), F = -E/2 + 3E^2/8
  // so that the pencil is standard; the products with the small F need only
  // FP32 (their relative error times |F| ~ 1e-5 is far below FP64 needs)
  if ((st = loewdin(ctx, n, nk, Hh, Sh, X))) return st;
  // ---- 4. clusters and their exact solves -----------------------------------
  ClusterLists L{};
  L.cap = n * nk;                 // every cluster holds at least one state
  double *w_slot = nullptr, *v_slot = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&L.order, 4ULL * n * nk, stream), "malloc order"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&L.pos, 4ULL * n * nk, stream), "malloc pos"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&L.csize, 4ULL * n * nk, stream), "malloc csize"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&L.diag, 8ULL * n * nk, stream), "malloc diag"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&L.small, sizeof(int4) * (size_t)L.cap, stream), "malloc list"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&L.large, sizeof(int4) * (size_t)L.cap, stream), "malloc list"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&L.counters, 4 * sizeof(int), stream), "malloc counters"))) return st;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&w_slot, 8ULL * n * nk, stream), "malloc w"))) return st;
  int* reach = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&reach, 4ULL * n * nk, stream), "malloc reach"))) return st;
  if (vectors && (st = cuda_check(ctx_malloc(ctx, (void**)&v_slot, 16ULL * nn * nk, stream), "malloc v"))) return st;
  {
    StageScope scope(ctx, OLC_STAGE_REFINE, 5);
    int P = 1;
    while (P < n) P <<= 1;
    const size_t sortmem = (size_t)P * (sizeof(double) + sizeof(int));
    if ((st = cuda_check(cudaFuncSetAttribute(cluster_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sortmem), "smem attribute"))) return st;
    if ((st = cuda_check(cudaFuncSetAttribute(final_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sortmem), "smem attribute"))) return st;
    if ((st = cuda_check(cudaMemsetAsync(L.counters, 0, 4 * sizeof(int), stream), "memset"))) return st;
    cluster_sort_kernel<<<nk, 1024, sortmem, stream>>>(Hh, n, L);
    if ((st = cuda_check(cudaMemsetAsync(reach, 0xff, 4ULL * n * nk, stream), "memset reach"))) return st;
    // OLC_COUPLE_RATIO overrides the coupling ratio (0: gaps alone form the clusters)
    double ratio = kCoupleRatio;
    if (const char* v = std::getenv("OLC_COUPLE_RATIO")) ratio = std::atof(v);
    if (ratio > 0.0) {
      coupling_reach_kernel<<<(int)(((size_t)n * nk * 32 + 255) / 256), 256, 0, stream>>>(Hh, n, nk, L, ratio,
                                                                                          reach);
      scope.add_launches(1);
    }
    const size_t formmem = (size_t)n * (sizeof(double) + sizeof(int));
    if ((st = cuda_check(cudaFuncSetAttribute(cluster_form_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)formmem), "smem attribute"))) return st;
    // OLC_CLUSTER_GAP overrides the gap that separates clusters (Hartree)
    double gap = kClusterGap;
    if (const char* v = std::getenv("OLC_CLUSTER_GAP")) gap = std::atof(v);
    cluster_form_kernel<<<nk, 256, formmem, stream>>>(n, L, reach, gap);
    singleton_kernel<<<(int)(((size_t)n * nk * 32 + 255) / 256), 256, 0, stream>>>(Hh, X, L, n, nk, w_slot,
                                                                                  v_slot);
    const size_t sm_small = sizeof(ClusterSmem<kSmallCluster>), sm_large = sizeof(ClusterSmem<kMaxCluster>);
    if ((st = cuda_check(cudaFuncSetAttribute(cluster_solve_kernel<kSmallCluster>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_small),
                         "smem attribute"))) return st;
    if ((st = cuda_check(cudaFuncSetAttribute(cluster_solve_kernel<kMaxCluster>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_large),
                         "smem attribute"))) return st;
    cluster_solve_kernel<kSmallCluster><<<152 * 8, 128, sm_small, stream>>>(
        Hh, X, L, L.small, L.counters + 0, L.counters + 2, n, w_slot, v_slot);
    cluster_solve_kernel<kMaxCluster><<<152 * 2, 256, sm_large, stream>>>(
        Hh, X, L, L.large, L.counters + 1, L.counters + 3, n, w_slot, v_slot);
  }
  if ((st = cuda_check(cudaGetLastError(), "extraction kernels"))) return st;
  {
    StageScope scope(ctx, OLC_STAGE_REFINE, 1);
    int P = 1;
    while (P < n) P <<= 1;
    const size_t sortmem = (size_t)P * (sizeof(double) + sizeof(int));
    // L.order is free once the clusters are solved: it takes the permutation
    final_sort_kernel<<<nk, 1024, sortmem, stream>>>(w_slot, n, num_states, eig_dev, L.order);
    if (vectors) {
      gather_vectors_kernel<<<152 * 16, 256, 0, stream>>>(reinterpret_cast<const double2*>(v_slot), L.order, n,
                                                          num_states, nk, reinterpret_cast<double2*>(vectors));
      scope.add_launches(1);
    }
  }
  st = cuda_check(cudaGetLastError(), "final sort");
  cudaFreeAsync(L.order, stream);
  cudaFreeAsync(L.pos, stream);
  cudaFreeAsync(L.csize, stream);
  cudaFreeAsync(L.diag, stream);
  cudaFreeAsync(L.small, stream);
  cudaFreeAsync(L.large, stream);
  cudaFreeAsync(L.counters, stream);
  cudaFreeAsync(w_slot, stream);
  cudaFreeAsync(reach, stream);
  if (v_slot) cudaFreeAsync(v_slot, stream);
  cudaFreeAsync(Hh, stream);
  cudaFreeAsync(Sh, stream);
  cudaFreeAsync(X, stream);
  if (st || !check) return st;
  return mixed_check_info(ctx);
}

// Waits for the queued mixed solve and turns the FP32 factorisation's info
// codes into a status.
int mixed_check_info(olc_context* ctx) {
  const int n = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints;
  std::vector<int> hinfo(nk);
  cudaMemcpyAsync(hinfo.data(), ctx->d_info, sizeof(int) * nk, cudaMemcpyDeviceToHost, ctx->stream);
  int st = cuda_check(cudaStreamSynchronize(ctx->stream), "mixed solve sync");
  if (st) return st;
  for (int k = 0; k < nk; ++k) {
    if (hinfo[k] != 0) ctx->w32_valid = false;
    // potrf: info in 1..n = leading minor not positive definite; chegvd:
    // info > n the same, info <= n = no convergence
    if (hinfo[k] > n || (hinfo[k] > 0 && ctx->info_potrf))
      return fail(OLC_ERR_NOT_PD, "overlap matrix not positive definite");
    if (hinfo[k] != 0) return fail(OLC_ERR_EIGEN, "FP32 eigen-solver did not converge");
  }
  return OLC_OK;
}

// Error-free product check entry (tests): C = A B for one complex FP64 pair.
int ozaki_selftest(olc_context* ctx, int m, int n, int k, const double* A, const double* B,
                   double* C) {
  int st = ozaki_zgemm<double, double>(ctx, m, n, k, A, 0, m, false, 53, B, 0, k, 53, C, 1);
  int s2 = cuda_check(cudaStreamSynchronize(ctx->stream), "split product selftest sync");
  return st ? st : s2;
}

}  // namespace olc
