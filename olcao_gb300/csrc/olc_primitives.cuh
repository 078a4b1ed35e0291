// Device Gaussian primitives for l <= 3 per centre (s, p, d, f Cartesians and
// the unnormalised real harmonics of gaussIntegrals.f90:33-39).
//
// All primitives are Obara-Saika recurrences (Obara & Saika, J. Chem. Phys.
// 84, 3963 (1986)) held in registers, specialised at compile time on the
// angular class (L1, L2) so that every loop is unrolled:
//   overlap      == overlap2CIntg   (gaussIntegrals.f90:26-4420)
//   kinetic      == kinetic2CIntg   (gaussIntegrals.f90:4422-11622)
//   mass velocity== massvel2CIntg   (gaussIntegrals.f90:39070-49402)
//   elec 3-centre== electron3CIntg  (gaussIntegrals.f90:11624-16023)
//   nuclear      == nuclear3CIntg   (gaussIntegrals.f90:16223-23039)
// with the Boys function evaluated in the reference's formulation
// (gaussIntegrals.f90:16080-16221, see boys_reference below).
#pragma once

#include <cuda_runtime.h>

namespace olc {

__host__ __device__ constexpr int ncart(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ constexpr int nharm(int L) { return (L + 1) * (L + 1); }

// Cartesian functions s; x y z; xx yy zz xy xz yz;
// xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz
__host__ __device__ constexpr int cex(int c) {
  return c == 1 ? 1 : c == 4 ? 2 : c == 7 ? 1 : c == 8 ? 1 : c == 10 ? 3 : c == 13 ? 2 : c == 14 ? 2
       : c == 15 ? 1 : c == 17 ? 1 : c == 19 ? 1 : 0;
}
__host__ __device__ constexpr int cey(int c) {
  return c == 2 ? 1 : c == 5 ? 2 : c == 7 ? 1 : c == 9 ? 1 : c == 11 ? 3 : c == 13 ? 1 : c == 15 ? 2
       : c == 16 ? 2 : c == 18 ? 1 : c == 19 ? 1 : 0;
}
__host__ __device__ constexpr int cez(int c) {
  return c == 3 ? 1 : c == 6 ? 2 : c == 8 ? 1 : c == 9 ? 1 : c == 12 ? 3 : c == 14 ? 1 : c == 16 ? 1
       : c == 17 ? 2 : c == 18 ? 2 : c == 19 ? 1 : 0;
}

// Real harmonic p (0-based lm) as a combination of Cartesians (the
// unnormalised functions of the reference's sh order):
// s; x y z; xy xz yz; xx-yy; 2zz-xx-yy;
// xyz; xxz-yyz; xxx-3yyx; 3xxy-yyy; 2zzz-3xxz-3yyz; 4zzx-xxx-yyx; 4zzy-xxy-yyy
__host__ __device__ constexpr int hn(int p) {
  return p == 7 ? 2 : p == 8 ? 3 : (p >= 10 && p <= 12) ? 2 : p >= 13 ? 3 : 1;
}
__host__ __device__ constexpr int hc(int p, int t) {  // cartesian index of term t
  return p <= 3 ? p : p == 4 ? 7 : p == 5 ? 8 : p == 6 ? 9
       : p == 7 ? (t == 0 ? 4 : 5)
       : p == 8 ? (t == 0 ? 6 : t == 1 ? 4 : 5)
       : p == 9 ? 19
       : p == 10 ? (t == 0 ? 14 : 16)
       : p == 11 ? (t == 0 ? 10 : 15)
       : p == 12 ? (t == 0 ? 13 : 11)
       : p == 13 ? (t == 0 ? 12 : t == 1 ? 14 : 16)
       : p == 14 ? (t == 0 ? 17 : t == 1 ? 10 : 15)
       : (t == 0 ? 18 : t == 1 ? 13 : 11);
}
__host__ __device__ constexpr double hw(int p, int t) {  // coefficient of term t
  return p == 7 ? (t == 0 ? 1.0 : -1.0)
       : p == 8 ? (t == 0 ? 2.0 : -1.0)
       : p == 10 ? (t == 0 ? 1.0 : -1.0)
       : p == 11 ? (t == 0 ? 1.0 : -3.0)
       : p == 12 ? (t == 0 ? 3.0 : -1.0)
       : p == 13 ? (t == 0 ? 2.0 : -3.0)
       : (p == 14 || p == 15) ? (t == 0 ? 4.0 : -1.0)
       : 1.0;
}

// 1-D Obara-Saika overlap recurrence with unit prefactor:
// s[i+1][j] = PA s[i][j] + (i s[i-1][j] + j s[i][j-1]) / (2 zeta), and the
// same along j with PB.
template <int LI, int LJ, class R>
__device__ __forceinline__ void os1d(R pa, R pb, R inv2z, R (&s)[LI + 1][LJ + 1]) {
  s[0][0] = R(1);
#pragma unroll
  for (int i = 0; i <= LI; ++i) {
    if (i > 0) {
      R v = pa * s[i - 1][0];
      if (i > 1) v += R(i - 1) * inv2z * s[i - 2][0];
      s[i][0] = v;
    }
#pragma unroll
    for (int j = 1; j <= LJ; ++j) {
      R v = pb * s[i][j - 1];
      if (i > 0) v += R(i) * inv2z * s[i - 1][j - 1];
      if (j > 1) v += R(j - 1) * inv2z * s[i][j - 2];
      s[i][j] = v;
    }
  }
}

// Write the harmonic block of a Cartesian accumulator:
// out[q * NS1 + p] (=|+=) sum of hw * cart[c1 * N2 + c2].
template <int L1, int L2, class R>
__device__ __forceinline__ void store_harmonic(const R* cart, double* out, bool accumulate,
                                               double scale) {
  constexpr int N2 = ncart(L2), NS1 = nharm(L1), NS2 = nharm(L2);
#pragma unroll
  for (int q = 0; q < NS2; ++q)
#pragma unroll
    for (int p = 0; p < NS1; ++p) {
      double v = 0.0;
#pragma unroll
      for (int t = 0; t < hn(p); ++t)
#pragma unroll
        for (int u = 0; u < hn(q); ++u)
          v += hw(p, t) * hw(q, u) * (double)cart[hc(p, t) * N2 + hc(q, u)];
      v *= scale;
      if (accumulate) out[q * NS1 + p] += v;
      else out[q * NS1 + p] = v;
    }
}

// ---------------------------------------------------------------------------
// two-centre overlap and kinetic energy (added into cart[] with weight w)
// ---------------------------------------------------------------------------
template <int L1, int L2>
__device__ __forceinline__ void add_overlap(double a1, double a2, const double* A,
                                            const double* B, double w, double* cart) {
  constexpr int N1 = ncart(L1), N2 = ncart(L2);
  const double z = a1 + a2, inv2z = 1.0 / (2.0 * z), xi = a1 * a2 / z;
  double s[3][L1 + 1][L2 + 1];
  double d2 = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double P = (a1 * A[c] + a2 * B[c]) / z;
    d2 += (A[c] - B[c]) * (A[c] - B[c]);
    os1d<L1, L2>(P - A[c], P - B[c], inv2z, s[c]);
  }
  const double r = kPi / z;
  const double pref = w * r * sqrt(r) * exp(-xi * d2);
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b)
      cart[a * N2 + b] += pref * s[0][cex(a)][cex(b)] * s[1][cey(a)][cey(b)] * s[2][cez(a)][cez(b)];
}

// Cartesian index of exponents (x, y, z), |e| <= 2, in the order above.
__host__ __device__ constexpr int cidx(int x, int y, int z) {
  return (x + y + z) == 0 ? 0
         : (x + y + z) == 1 ? (x ? 1 : y ? 2 : 3)
         : (x == 2 ? 4 : y == 2 ? 5 : z == 2 ? 6 : (x && y) ? 7 : (x && z) ? 8 : 9);
}
__host__ __device__ constexpr int cexp(int c, int i) { return i == 0 ? cex(c) : i == 1 ? cey(c) : cez(c); }
// last non-zero direction of Cartesian c (the direction the recurrence lowers)
__host__ __device__ constexpr int clast(int c) { return cez(c) ? 2 : cey(c) ? 1 : 0; }
__host__ __device__ constexpr int clower(int c, int i) {
  return cidx(cex(c) - (i == 0), cey(c) - (i == 1), cez(c) - (i == 2));
}

// Kinetic energy by the three-dimensional Obara-Saika kinetic recurrence
//   (a+1_i|T|b) = PA_i (a|T|b) + [N_i(a)(a-1_i|T|b) + N_i(b)(a|T|b-1_i)]/(2 zeta)
//                 + 2 xi [(a+1_i|b) - N_i(a)/(2 a1) (a-1_i|b)]
// (likewise on b with PB and a2) from (0|T|0) = xi (3 - 2 xi |AB|^2) (0|0).
template <int L1, int L2>
__device__ __forceinline__ void add_kinetic(double a1, double a2, const double* A,
                                            const double* B, double w, double* cart) {
  constexpr int N1 = ncart(L1), N2 = ncart(L2);
  const double z = a1 + a2, inv2z = 1.0 / (2.0 * z), xi = a1 * a2 / z;
  const double x2 = 2.0 * xi, inv2a1 = 1.0 / (2.0 * a1), inv2a2 = 1.0 / (2.0 * a2);
  double s[3][L1 + 1][L2 + 1], PA[3], PB[3];
  double d2 = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double P = (a1 * A[c] + a2 * B[c]) / z;
    PA[c] = P - A[c];
    PB[c] = P - B[c];
    d2 += (A[c] - B[c]) * (A[c] - B[c]);
    os1d<L1, L2>(PA[c], PB[c], inv2z, s[c]);
  }
  const double r = kPi / z;
  const double pref = r * sqrt(r) * exp(-xi * d2);
  double S[N1][N2], T[N1][N2];
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b)
      S[a][b] = pref * s[0][cex(a)][cex(b)] * s[1][cey(a)][cey(b)] * s[2][cez(a)][cez(b)];
  T[0][0] = xi * (3.0 - 2.0 * xi * d2) * pref;
#pragma unroll
  for (int b = 1; b < N2; ++b) {
    const int i = clast(b), bp = clower(b, i), n = cexp(bp, i);
    double v = PB[i] * T[0][bp] + x2 * S[0][b];
    if (n > 0) {
      const int bq = clower(bp, i);
      v += n * inv2z * T[0][bq] - x2 * n * inv2a2 * S[0][bq];
    }
    T[0][b] = v;
  }
#pragma unroll
  for (int a = 1; a < N1; ++a) {
    const int i = clast(a), ap = clower(a, i), n = cexp(ap, i);
#pragma unroll
    for (int b = 0; b < N2; ++b) {
      double v = PA[i] * T[ap][b] + x2 * S[a][b];
      if (n > 0) {
        const int aq = clower(ap, i);
        v += n * inv2z * T[aq][b] - x2 * n * inv2a1 * S[aq][b];
      }
      if (cexp(b, i) > 0) v += cexp(b, i) * inv2z * T[ap][clower(b, i)];
      T[a][b] = v;
    }
  }
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b) cart[a * N2 + b] += w * T[a][b];
}

// Mass velocity: w (alpha^2 / 8) <a| nabla^4 |b> with alpha = fineStructure
// x 1e-3 (constants.f90:47), the quantity massvel2CIntg returns
// (gaussIntegrals.f90:39070-49402).  nabla^4 = sum_i d4_i + 2 sum_{i<j} d2_i d2_j
// acts on b; per direction, on x^l exp(-a2 x^2),
//   d2 -> l(l-1) x^(l-2) - 2 a2 (2l+1) x^l + 4 a2^2 x^(l+2)   (times the Gaussian)
// and d4 is d2 applied twice, so every factor is a short combination of
// 1-D overlaps with b's power raised by at most 4.
constexpr double kFineStructure = 7.2973525693e-3;
template <int LI, int LJ>
__device__ __forceinline__ double lap1d(const double (&s)[LI + 1][LJ + 5], int i, int j, double a2) {
  double v = -2.0 * a2 * (2 * j + 1) * s[i][j] + 4.0 * a2 * a2 * s[i][j + 2];
  if (j >= 2) v += j * (j - 1) * s[i][j - 2];
  return v;
}
template <int LI, int LJ>
__device__ __forceinline__ double lap2d(const double (&s)[LI + 1][LJ + 5], int i, int j, double a2) {
  double v = -2.0 * a2 * (2 * j + 1) * lap1d<LI, LJ>(s, i, j, a2) +
             4.0 * a2 * a2 * lap1d<LI, LJ>(s, i, j + 2, a2);
  if (j >= 2) v += j * (j - 1) * lap1d<LI, LJ>(s, i, j - 2, a2);
  return v;
}

// Momentum (momentum2CIntg): component `comp` of <a| d/dr_comp |b>, the
// derivative acting on b: d/dx [x^l e^{-a2 x^2}] = (l x^{l-1} - 2 a2 x^{l+1})
// e^{-a2 x^2}, a 1-D overlap with b's power lowered or raised by one in that
// direction times the plain overlaps of the other two.
template <int L1, int L2>
__device__ __forceinline__ void add_momentum(double a1, double a2, const double* A, const double* B, int comp,
                                             double w, double* cart) {
  constexpr int N1 = ncart(L1), N2 = ncart(L2);
  const double z = a1 + a2, inv2z = 1.0 / (2.0 * z), xi = a1 * a2 / z;
  double s[3][L1 + 1][L2 + 2];
  double d2 = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double P = (a1 * A[c] + a2 * B[c]) / z;
    d2 += (A[c] - B[c]) * (A[c] - B[c]);
    os1d<L1, L2 + 1>(P - A[c], P - B[c], inv2z, s[c]);
  }
  const double r = kPi / z;
  const double pref = w * r * sqrt(r) * exp(-xi * d2);
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b) {
      double v = pref;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int ia = cexp(a, c), jb = cexp(b, c);
        if (c == comp) {
          double d = -2.0 * a2 * s[c][ia][jb + 1];
          if (jb > 0) d += jb * s[c][ia][jb - 1];
          v *= d;
        } else {
          v *= s[c][ia][jb];
        }
      }
      cart[a * N2 + b] += v;
    }
}

template <int L1, int L2>
__device__ __forceinline__ void add_massvel(double a1, double a2, const double* A,
                                            const double* B, double w, double* cart) {
  constexpr int N1 = ncart(L1), N2 = ncart(L2);
  const double z = a1 + a2, inv2z = 1.0 / (2.0 * z), xi = a1 * a2 / z;
  double s[3][L1 + 1][L2 + 5];
  double d2 = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double P = (a1 * A[c] + a2 * B[c]) / z;
    d2 += (A[c] - B[c]) * (A[c] - B[c]);
    os1d<L1, L2 + 4>(P - A[c], P - B[c], inv2z, s[c]);
  }
  const double r = kPi / z;
  const double pref = w * (kFineStructure * kFineStructure / 8.0) * r * sqrt(r) * exp(-xi * d2);
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b) {
      double i0[3], i2[3], i4[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int ia = cexp(a, c), jb = cexp(b, c);
        i0[c] = s[c][ia][jb];
        i2[c] = lap1d<L1, L2>(s[c], ia, jb, a2);
        i4[c] = lap2d<L1, L2>(s[c], ia, jb, a2);
      }
      cart[a * N2 + b] += pref * (i4[0] * i0[1] * i0[2] + i0[0] * i4[1] * i0[2] + i0[0] * i0[1] * i4[2] +
                                  2.0 * (i2[0] * i2[1] * i0[2] + i2[0] * i0[1] * i2[2] + i0[0] * i2[1] * i2[2]));
    }
}

// ---------------------------------------------------------------------------
// three-centre overlap with an s-type Gaussian exp(-a3 |r - C|^2)
// ---------------------------------------------------------------------------
template <int L1, int L2, class R>
__device__ __forceinline__ void add_elec3c(double a1, double a2, double a3, const double* A,
                                           const double* B, const double* Cc, double expAB,
                                           double w, R* cart) {
  constexpr int N1 = ncart(L1), N2 = ncart(L2);
  const double z = a1 + a2, z3 = z + a3;
  R s[3][L1 + 1][L2 + 1];
  double pc2 = 0.0;
  const double inv2z3 = 1.0 / (2.0 * z3);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double P = (a1 * A[c] + a2 * B[c]) / z;
    const double G = (a1 * A[c] + a2 * B[c] + a3 * Cc[c]) / z3;
    pc2 += (P - Cc[c]) * (P - Cc[c]);
    os1d<L1, L2, R>(R(G - A[c]), R(G - B[c]), R(inv2z3), s[c]);
  }
  const double r = kPi / z3;
  const R pref = R(w * r * sqrt(r) * expAB * exp(-(z * a3 / z3) * pc2));
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b)
      cart[a * N2 + b] += pref * s[0][cex(a)][cex(b)] * s[1][cey(a)][cey(b)] * s[2][cez(a)][cez(b)];
}

// Far-shell split of add_elec3c.  With rho = z a3 / z3 |P - C|^2 an image
// enters with the suppression exp(-rho); images past kFarRho (exp(-22) =
// 2.8e-10) may run in FP32 (GB300's FP32 rate is 64x its FP64 rate).  Their
// FP32 rounding, 6e-8 of a term that the suppression and the recurrence's
// polynomial in the image distance (up to 25^4 for d-d at the cut-off
// radius) keep below ~3e-6 of the block scale, stays near 2e-13 of it.
constexpr double kFarRho = 22.0;

__device__ __forceinline__ double elec3c_rho(double a1, double a2, double a3, const double* A,
                                             const double* B, const double* Cc) {
  const double z = a1 + a2;
  double pc2 = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double P = (a1 * A[c] + a2 * B[c]) / z;
    pc2 += (P - Cc[c]) * (P - Cc[c]);
  }
  return z * a3 / (z + a3) * pc2;
}

// add_elec3c for a far image, in FP32 (rho from elec3c_rho).
template <int L1, int L2>
__device__ __forceinline__ void add_elec3c_f32(double a1, double a2, double a3, const double* A,
                                               const double* B, const double* Cc, double expAB,
                                               double w, double rho, float* cart) {
  constexpr int N1 = ncart(L1), N2 = ncart(L2);
  const float iz3 = 1.0f / (float)(a1 + a2 + a3);
  float s[3][L1 + 1][L2 + 1];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    // G - A = (a2 (B - A) + a3 (C - A)) / z3, G - B = (-a1 (B - A) + a3 (C - B)) / z3
    const float ba = (float)(B[c] - A[c]), ca = (float)(Cc[c] - A[c]), cb = (float)(Cc[c] - B[c]);
    const float ga = ((float)a2 * ba + (float)a3 * ca) * iz3;
    const float gb = (-(float)a1 * ba + (float)a3 * cb) * iz3;
    os1d<L1, L2, float>(ga, gb, 0.5f * iz3, s[c]);
  }
  const float r = 3.14159265358979f * iz3;
  const float pref = (float)(w * expAB) * r * sqrtf(r) * expf(-(float)rho);
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b)
      cart[a * N2 + b] += pref * s[0][cex(a)][cex(b)] * s[1][cey(a)][cey(b)] * s[2][cez(a)][cez(b)];
}

// ---------------------------------------------------------------------------
// Boys function F_0..F_n in the reference's formulation
// ---------------------------------------------------------------------------
// Gamma(k + 1/2) rounded to binary32: the reference's gfortran build stores
// its series constants as default-kind REAL literals.
__host__ __device__ constexpr double gamma_half_f32(int k) {
  double r = 1.7724538509055160273;
  for (int i = 1; i <= k; ++i) r *= (i - 0.5);
  return (double)(float)r;
}

template <int NMAX>
__device__ __forceinline__ void boys_reference(double T, double (&F)[NMAX + 1]) {
  const double thr = (double)0.1f;
  const double eT = exp(-T);
  if (T <= thr) {
    // F_N = 1/2 e^-T Gamma(N+1/2) sum_{i=1..7} T^(i-1) / Gamma(N+i+1/2)
#pragma unroll
    for (int N = 0; N <= NMAX; ++N) {
      double acc = 1.0 / gamma_half_f32(N + 1);
      double tp = 1.0;
#pragma unroll
      for (int i = 2; i <= 7; ++i) {
        tp *= T;
        acc += tp / gamma_half_f32(N + i);
      }
      F[N] = 0.5 * eT * gamma_half_f32(N) * acc;
    }
    return;
  }
  // closed forms: F_n = (2n-1)!!/2^(n+1) [ sqrt(pi) erf(sqrt T) / T^(n+1/2)
  //                     - e^-T sum_{k<n} 2^(k+1) / ((2k+1)!! T^(n-k)) ]
  const double rt = sqrt(T);
  const double spe = 1.7724538509055160273 * erf(rt);
  const double invT = 1.0 / T;
#pragma unroll
  for (int n = 0; n <= NMAX; ++n) {
    double dfn = 1.0;
    for (int q = 2 * n - 1; q > 1; q -= 2) dfn *= q;
    double sum = 0.0, dfk = 1.0, p2 = 2.0;
#pragma unroll
    for (int k = 0; k < n; ++k) {
      if (k > 0) dfk *= (2 * k + 1);
      double tp = 1.0;
      for (int q = 0; q < n - k; ++q) tp *= invT;
      sum += p2 / dfk * tp;
      p2 *= 2.0;
    }
    double tn = rt;
    for (int q = 0; q < n; ++q) tn *= T;
    double two = 1.0;
    for (int q = 0; q <= n; ++q) two *= 2.0;
    F[n] = dfn / two * (spe / tn - eT * sum);
  }
}

// ---------------------------------------------------------------------------
// nuclear attraction  int phi_a phi_b exp(-a3 |r-C|^2) / |r-C|  (added with
// weight w into cart[]).  Vertical Obara-Saika recurrence on centre A with
// auxiliary order m, then the horizontal transfer
// (a|b) = sum_k C(b,k) AB^(b-k) [a+k] applied per dimension.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int binom(int n, int k) {
  return (k == 0 || k == n) ? 1 : (n == 2 && k == 1) ? 2 : (n == 3 && (k == 1 || k == 2)) ? 3 : 1;
}

template <int L1, int L2>
__device__ __forceinline__ void add_nuclear(double a1, double a2, double a3, const double* A,
                                            const double* B, const double* Cc, double w,
                                            double* cart) {
  constexpr int LT = L1 + L2;
  constexpr int E = LT + 1;
  constexpr int N1 = ncart(L1), N2 = ncart(L2);
  const double z3 = a1 + a2 + a3, inv2z3 = 1.0 / (2.0 * z3);
  double GA[3], GC[3], AB[3];
  double gc2 = 0.0, ex = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double G = (a1 * A[c] + a2 * B[c] + a3 * Cc[c]) / z3;
    GA[c] = G - A[c];
    GC[c] = G - Cc[c];
    AB[c] = A[c] - B[c];
    gc2 += GC[c] * GC[c];
    const double d1 = A[c] - B[c], d2 = A[c] - Cc[c], d3 = B[c] - Cc[c];
    ex += a1 * a2 * d1 * d1 + a1 * a3 * d2 * d2 + a2 * a3 * d3 * d3;
  }
  double F[LT + 1];
  boys_reference<LT>(z3 * gc2, F);
  const double pre = w * 2.0 * (kPi / z3) * exp(-ex / z3);
  // V[x][y][z][m], |e| <= LT, m <= LT - |e|
  double V[E][E][E][E];
#pragma unroll
  for (int m = 0; m <= LT; ++m) V[0][0][0][m] = pre * F[m];
#pragma unroll
  for (int s = 1; s <= LT; ++s)
#pragma unroll
    for (int x = s; x >= 0; --x)
#pragma unroll
      for (int y = s - x; y >= 0; --y) {
        const int zz = s - x - y;
        // lower along the first non-zero direction
        const int d = x > 0 ? 0 : (y > 0 ? 1 : 2);
        const int px = x - (d == 0), py = y - (d == 1), pz = zz - (d == 2);
        const int pe = d == 0 ? px : d == 1 ? py : pz;   // exponent of parent along d
#pragma unroll
        for (int m = 0; m <= LT - s; ++m) {
          double v = GA[d] * V[px][py][pz][m] - GC[d] * V[px][py][pz][m + 1];
          if (pe > 0) {
            const int qx = px - (d == 0), qy = py - (d == 1), qz = pz - (d == 2);
            v += pe * inv2z3 * (V[qx][qy][qz][m] - V[qx][qy][qz][m + 1]);
          }
          V[x][y][zz][m] = v;
        }
      }
#pragma unroll
  for (int a = 0; a < N1; ++a)
#pragma unroll
    for (int b = 0; b < N2; ++b) {
      const int ax = cex(a), ay = cey(a), az = cez(a);
      const int bx = cex(b), by = cey(b), bz = cez(b);
      double acc = 0.0;
#pragma unroll
      for (int kx = 0; kx <= bx; ++kx) {
        double fx = binom(bx, kx);
        for (int q = 0; q < bx - kx; ++q) fx *= AB[0];
#pragma unroll
        for (int ky = 0; ky <= by; ++ky) {
          double fy = binom(by, ky);
          for (int q = 0; q < by - ky; ++q) fy *= AB[1];
#pragma unroll
          for (int kz = 0; kz <= bz; ++kz) {
            double fz = binom(bz, kz);
            for (int q = 0; q < bz - kz; ++q) fz *= AB[2];
            acc += fx * fy * fz * V[ax + kx][ay + ky][az + kz][0];
          }
        }
      }
      cart[a * N2 + b] += acc;
    }
}

}  // namespace olc
