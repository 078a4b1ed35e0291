// Generalised Hermitian eigen-solve of one small pencil by one CTA, all in
// shared memory (FP64): the steps of LAPACK zhegv (itype 1, upper) with a
// two-sided cyclic Jacobi eigensolver for the reduced problem.
//   1. B = U^H U (right-looking Cholesky; failure n + j + 1 as zpotrf/zhegv)
//   2. C = U^{-H} A U^{-1}
//   3. C = V diag(w) V^H by parallel (round-robin) cyclic Jacobi rotations
// The caller loads U = B and C = A (column-major, full Hermitian), calls
// hegv_inplace, then reads the eigenvalues off diag(C), the reduced
// eigenvectors from V, and back-transforms with U (x = U^{-1} v).
#pragma once

#include <cuda_runtime.h>

namespace olc {
namespace jac {

constexpr int kMaxN = 64;

struct cd { double x, y; };
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd cmulc(cd a, cd b) { return {a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x}; }  // conj(a)*b
__device__ __forceinline__ cd csub(cd a, cd b) { return {a.x - b.x, a.y - b.y}; }

struct Shared {
  int fail;
  double red[32];
  double off, diag;
  int p[kMaxN / 2], q[kMaxN / 2];
  double c[kMaxN / 2], s[kMaxN / 2], phx[kMaxN / 2], phy[kMaxN / 2];
};

// All threads of the CTA must call this; sh.fail != 0 on return when B is not
// positive definite.  trace (nullable) receives (off, diag) per sweep.
static __device__ __noinline__ void hegv_inplace(cd* U, cd* C, cd* V, int n, bool u_factored,
                                          Shared& sh, double* trace) {
  const int tid = threadIdx.x;
  const size_t nn = (size_t)n * n;
  if (tid == 0) sh.fail = 0;
  __syncthreads();
  // ---- 1. Cholesky S = U^H U (right-looking, upper) ----------------------
  if (!u_factored) {
    for (int j = 0; j < n; ++j) {
      if (tid == 0) {
        const double d = U[(size_t)j * n + j].x;
        if (!(d > 0.0)) sh.fail = n + j + 1;
        U[(size_t)j * n + j] = {sqrt(fmax(d, 1e-300)), 0.0};
      }
      __syncthreads();
      if (sh.fail) break;
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
  if (sh.fail) return;

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
    if ((tid & 31) == 0) sh.red[tid >> 5] = off;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < (int)(blockDim.x / 32); ++q) t += sh.red[q];
      sh.off = t;
    }
    __syncthreads();
    if ((tid & 31) == 0) sh.red[tid >> 5] = dg;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < (int)(blockDim.x / 32); ++q) t += sh.red[q];
      sh.diag = t;
    }
    __syncthreads();
    if (trace && tid == 0 && sweep < 40) {
      trace[2 * sweep] = sh.off;
      trace[2 * sweep + 1] = sh.diag;
    }
    if (sh.off <= 1e-28 * sh.diag || sh.off == 0.0) break;
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
        sh.p[pi] = p; sh.q[pi] = q; sh.c[pi] = c; sh.s[pi] = s; sh.phx[pi] = phx; sh.phy[pi] = phy;
      }
      __syncthreads();
      // columns: C <- C J, V <- V J
      //   col_p' = c col_p - s e^{-i phi} col_q ; col_q' = s col_p + c e^{-i phi} col_q
      for (int e = tid; e < half * n; e += blockDim.x) {
        const int pi = e / n, r = e % n;
        const int p = sh.p[pi], q = sh.q[pi];
        if (q >= n || sh.s[pi] == 0.0) continue;
        const double c = sh.c[pi], s = sh.s[pi];
        const cd ph = {sh.phx[pi], sh.phy[pi]};
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
        const int p = sh.p[pi], q = sh.q[pi];
        if (q >= n || sh.s[pi] == 0.0) continue;
        const double c = sh.c[pi], s = sh.s[pi];
        const cd phc = {sh.phx[pi], -sh.phy[pi]};
        const cd xp = C[(size_t)col * n + p], eq = cmul(phc, C[(size_t)col * n + q]);
        C[(size_t)col * n + p] = {c * xp.x - s * eq.x, c * xp.y - s * eq.y};
        C[(size_t)col * n + q] = {s * xp.x + c * eq.x, s * xp.y + c * eq.y};
      }
      __syncthreads();
    }
  }
  __syncthreads();
}

// Ascending order of the eigenvalues diag(C) into order[] (thread 0 sorts).
static __device__ __forceinline__ void sorted_order(const cd* C, int n, double* w, int* order) {
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += blockDim.x) {
    w[i] = C[(size_t)i * n + i].x;
    order[i] = i;
  }
  __syncthreads();
  if (tid == 0) {
    for (int i = 1; i < n; ++i) {
      const int oi = order[i];
      const double wi = w[oi];
      int j = i - 1;
      while (j >= 0 && w[order[j]] > wi) { order[j + 1] = order[j]; --j; }
      order[j + 1] = oi;
    }
  }
  __syncthreads();
}

}  // namespace jac
}  // namespace olc
