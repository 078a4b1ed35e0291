// Primitive-stage device code shared by the translation units of the
// integral kernels (olc_integrals.cu: s, p, d classes; olc_integrals_f*.cu:
// the classes with an f function, compiled apart because their
// recurrences are large).
#pragma once

#include <type_traits>

#include "olc_common.h"
#include "olc_primitives.cuh"

namespace olc {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double elem_alpha(const SysView& v, int e, int a) {
  return v.elem_alpha[e * OLC_MAX_ALPHAS + a];
}

// alphaDist(a1, a2, e1, e2) of gaussRelations.f90:64-135 (same operation order)
__device__ __forceinline__ double alpha_dist(const SysView& v, int a1, int a2, int e1, int e2) {
  const double al = elem_alpha(v, e1, a1), ak = elem_alpha(v, e2, a2);
  return v.log_thresh / ak / (al / (al + ak));
}

// Reduce v by the lattice vector obtained from rounding its fractional
// coordinates (the first step of findLatticeVector, lattice.f90:777-793).
__device__ __forceinline__ void round_reduce(const SysView& v, const double* in, double* out) {
  double L[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double f = in[0] * v.inv_real[i * 3] + in[1] * v.inv_real[i * 3 + 1] +
                     in[2] * v.inv_real[i * 3 + 2];
    double r = floor(fabs(f) + 0.5);
    if (f < 0.0) r = -r;
#pragma unroll
    for (int c = 0; c < 3; ++c) L[c] += v.real_vec[i * 3 + c] * r;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c] = in[c] - L[c];
}

struct ItemGeom {
  double A[3], B[3];
  double a1, a2, sep;
  int e1, e2, ia1, ia2;
};

__device__ __forceinline__ void load_item(const SysView& v, int task, int ab, ItemGeom& g) {
  const DevTask tk = v.tasks[task];
  const DevPair p = v.pairs[tk.pair];
  const DevType& t1 = v.types[v.site_type[p.i]];
  const DevType& t2 = v.types[v.site_type[p.j]];
  g.ia1 = ab & 255;
  g.ia2 = ab >> 8;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    g.A[c] = v.site_pos[3 * p.i + c];
    g.B[c] = v.site_pos[3 * p.j + c] + p.L[c] + v.cells[4 * tk.cell + c];
  }
  g.a1 = t1.alphas[g.ia1];
  g.a2 = t2.alphas[g.ia2];
  g.e1 = t1.element;
  g.e2 = t2.element;
  g.sep = tk.sep;
}

// Visit every lattice image C' = C + T of a site with |P - C'|^2 <= tad.
// The image set equals the reference's {cells of the nearest-origin loop},
// integrals.F90:2374-2418 / 2533-2594.
template <class F>
__device__ __forceinline__ void for_images(const SysView& v, const double* P, const double* C,
                                           double tad, F&& f) {
  double d[3] = {P[0] - C[0], P[1] - C[1], P[2] - C[2]};
  double r[3];
  round_reduce(v, d, r);
  const double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  const double lim = rn + sqrt(tad);
  const double lim2 = lim * lim;
  // base image of C: C + (d - r)
  const double base[3] = {C[0] + (d[0] - r[0]), C[1] + (d[1] - r[1]), C[2] + (d[2] - r[2])};
  for (int n = 0; n < v.ncells; ++n) {
    const double4 cell = reinterpret_cast<const double4*>(v.cells)[n];
    if (cell.w > lim2) break;
    const double x = r[0] - cell.x, y = r[1] - cell.y, z = r[2] - cell.z;
    const double d2 = x * x + y * y + z * z;
    if (d2 > tad) continue;
    const double Cp[3] = {base[0] + cell.x, base[1] + cell.y, base[2] + cell.z};
    f(Cp, d2);
  }
}

// ---------------------------------------------------------------------------
// stage 1: primitive kernels
// ---------------------------------------------------------------------------
struct PrimArgs {
  const int32_t* task;
  const int32_t* ab;
  int n;
  double* out;              // class block of the sh scratch
  const double* coeffs;     // device [pot_dim] (EP) or nullptr
  int accumulate;
  int ep_type;              // EP: potential type of a single term, -1 = all types
  int ep_alpha;             // EP: exponent index of a single term
};

// MODE 0: every term in FP64.  Mixed precision splits the electronic
// potential into two passes: MODE 1 the near images (FP64), MODE 2 the images
// past the far-shell cut (FP32 accumulator), added to the same blocks.
template <int OP, int L1, int L2, int MODE>
__global__ void __launch_bounds__(128) prim_kernel(SysView v, PrimArgs a) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= a.n) return;
  constexpr int N1 = ncart(L1), N2 = ncart(L2), NS = nharm(L1) * nharm(L2);
  ItemGeom g;
  load_item(v, a.task[idx], a.ab[idx], g);
  using R = typename std::conditional<MODE == 2, float, double>::type;
  R cart[N1 * N2];
#pragma unroll
  for (int q = 0; q < N1 * N2; ++q) cart[q] = R(0);
  double scale = 1.0;
  if constexpr (OP == OLC_OP_OVERLAP) {
    add_overlap<L1, L2>(g.a1, g.a2, g.A, g.B, 1.0, cart);
  } else if constexpr (OP == OLC_OP_KINETIC) {
    add_kinetic<L1, L2>(g.a1, g.a2, g.A, g.B, 1.0, cart);
  } else if constexpr (OP == OLC_OP_MASSVEL) {
    // gaussOverlapMV accumulates the primitive with a minus sign
    // (integrals.F90:1228-1236): the mass-velocity term lowers H
    add_massvel<L1, L2>(g.a1, g.a2, g.A, g.B, -1.0, cart);
  } else {
    // centre of the alpha-pair overlap (alphaCenter, gaussRelations.f90:122)
    const double al = elem_alpha(v, g.e1, g.ia1), ak = elem_alpha(v, g.e2, g.ia2);
    const double cen = al / (al + ak);
    double P[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) P[c] = cen * (g.A[c] - g.B[c]) + g.B[c];
    const double frac = 1.0 - g.sep / alpha_dist(v, g.ia1, g.ia2, g.e1, g.e2);
    const double T = v.log_thresh;
    if constexpr (OP == OLC_OP_NUCLEAR) {
      for (int m = 0; m < v.num_pot_sites; ++m) {
        const DevPotType& pt = v.pot_types[v.pot_site_type[m]];
        if (pt.nuc_charge < 1.0e-8) continue;
        const double an = v.elem_nuc_alpha[pt.element];
        const double tad = frac * (T * (al + ak + an) / (al + ak) / an);
        const double nz = -pt.nuc_charge, nalpha = pt.nuc_alpha;
        for_images(v, P, &v.pot_site_pos[3 * m], tad, [&](const double* Cp, double) {
          add_nuclear<L1, L2>(g.a1, g.a2, nalpha, g.A, g.B, Cp, nz, cart);
        });
      }
    } else {  // electronic potential: single term or sum_j c_j V_j
      double d2 = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) d2 += (g.A[c] - g.B[c]) * (g.A[c] - g.B[c]);
      const double expAB = exp(-(g.a1 * g.a2 / (g.a1 + g.a2)) * d2);
      const int t0 = a.ep_type < 0 ? 0 : a.ep_type;
      const int t1 = a.ep_type < 0 ? v.num_pot_types : a.ep_type + 1;
      for (int t = t0; t < t1; ++t) {
        const DevPotType& pt = v.pot_types[t];
        const double* pe = &v.elem_pot_alpha[pt.element * OLC_MAX_POT_ALPHAS];
        const int j0 = a.ep_type < 0 ? 0 : a.ep_alpha;
        const int j1 = a.ep_type < 0 ? pt.num_alphas : a.ep_alpha + 1;
        // largest radius first: alphaPotDist decreases with the exponent
        const double tad0 = frac * (T * (al + ak + pe[j0]) / (al + ak) / pe[j0]);
        for (int m = 0; m < pt.multiplicity; ++m) {
          const double* C = &v.pot_site_pos[3 * (pt.first_site + m)];
          for_images(v, P, C, tad0, [&](const double* Cp, double dd) {
            for (int j = j0; j < j1; ++j) {
              const double tad = frac * (T * (al + ak + pe[j]) / (al + ak) / pe[j]);
              if (dd > tad) break;
              const double w = a.coeffs ? a.coeffs[pt.cumul_alpha + j] : 1.0;
              if constexpr (MODE == 0) {
                add_elec3c<L1, L2, double>(g.a1, g.a2, pt.alphas[j], g.A, g.B, Cp, expAB, w, cart);
              } else {
                const double rho = elec3c_rho(g.a1, g.a2, pt.alphas[j], g.A, g.B, Cp);
                if constexpr (MODE == 1) {
                  if (rho <= kFarRho)
                    add_elec3c<L1, L2, double>(g.a1, g.a2, pt.alphas[j], g.A, g.B, Cp, expAB, w, cart);
                } else {
                  if (rho > kFarRho)
                    add_elec3c_f32<L1, L2>(g.a1, g.a2, pt.alphas[j], g.A, g.B, Cp, expAB, w, rho, cart);
                }
              }
            }
          });
        }
      }
    }
  }
  store_harmonic<L1, L2, R>(cart, a.out + (size_t)idx * NS, a.accumulate != 0, scale);
}

// One primitive of explicit inputs (the testing entry olc_primitive_batch).
template <int L1, int L2>
__device__ __forceinline__ void prim_one(int kind, const double* in, double* out) {
  constexpr int N1 = ncart(L1), N2 = ncart(L2), NS1 = nharm(L1), NS2 = nharm(L2);
  double cart[N1 * N2];
#pragma unroll
  for (int q = 0; q < N1 * N2; ++q) cart[q] = 0.0;
  const double *A = in + 3, *B = in + 6, *C = in + 9;
  if (kind == 1) add_overlap<L1, L2>(in[0], in[1], A, B, 1.0, cart);
  else if (kind == 2) add_kinetic<L1, L2>(in[0], in[1], A, B, 1.0, cart);
  else if (kind == 3) add_nuclear<L1, L2>(in[0], in[1], in[2], A, B, C, 1.0, cart);
  else if (kind == 5) add_massvel<L1, L2>(in[0], in[1], A, B, 1.0, cart);
  else if (kind >= 6) add_momentum<L1, L2>(in[0], in[1], A, B, kind - 6, 1.0, cart);
  else {
    double d2 = 0.0;
    for (int c = 0; c < 3; ++c) d2 += (A[c] - B[c]) * (A[c] - B[c]);
    const double expAB = exp(-(in[0] * in[1] / (in[0] + in[1])) * d2);
    add_elec3c<L1, L2, double>(in[0], in[1], in[2], A, B, C, expAB, 1.0, cart);
  }
  double sh[NS1 * NS2];
  store_harmonic<L1, L2, double>(cart, sh, false, 1.0);
  for (int q = 0; q < NS2; ++q)
    for (int p2 = 0; p2 < NS1; ++p2) out[q * 16 + p2] = sh[q * NS1 + p2];
}


// f classes (olc_integrals_f*.cu): launches of prim_kernel for the 7 classes
// with l1 = 3 or l2 = 3, one function per operator; mode as prim_kernel.
int launch_prim_f_overlap(cudaStream_t st, const SysView& v, const PrimArgs& a, int l1, int l2, dim3 g, dim3 b);
int launch_prim_f_kinetic(cudaStream_t st, const SysView& v, const PrimArgs& a, int l1, int l2, dim3 g, dim3 b);
int launch_prim_f_massvel(cudaStream_t st, const SysView& v, const PrimArgs& a, int l1, int l2, dim3 g, dim3 b);
int launch_prim_f_nuclear(cudaStream_t st, const SysView& v, const PrimArgs& a, int l1, int l2, dim3 g, dim3 b);
int launch_prim_f_elecpot(cudaStream_t st, const SysView& v, const PrimArgs& a, int l1, int l2, int mode, dim3 g,
                          dim3 b);
// primitive batch entries of the f classes, one per kind (1 overlap,
// 2 kinetic, 3 nuclear, 4 three-centre, 5 mass velocity, 6-8 momentum x, y,
// z with the overlap), in the same translation units
void launch_prim_batch_f_overlap(int n, const double* in, const int32_t* lm, double* out);
void launch_prim_batch_f_kinetic(int n, const double* in, const int32_t* lm, double* out);
void launch_prim_batch_f_nuclear(int n, const double* in, const int32_t* lm, double* out);
void launch_prim_batch_f_elecpot(int n, const double* in, const int32_t* lm, double* out);
void launch_prim_batch_f_massvel(int n, const double* in, const int32_t* lm, double* out);
void launch_prim_batch_f_momentum(int kind, int n, const double* in, const int32_t* lm, double* out);

// Primitive batch kernel of one kind and one f class (a kernel per class
// keeps each recurrence's register allocation separate).
template <int KIND, int L1, int L2>
__global__ void prim_batch_f_kernel(int n, const double* in, const int32_t* lm, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto lof = [](int lma) { return lma == 1 ? 0 : lma == 4 ? 1 : lma == 9 ? 2 : 3; };
  if (lof(lm[2 * i]) != L1 || lof(lm[2 * i + 1]) != L2) return;
  prim_one<L1, L2>(KIND, in + 12 * i, out + 256 * i);
}

template <int KIND>
void launch_prim_batch_f_kind(int n, const double* in, const int32_t* lm, double* out) {
  const int g = (n + 63) / 64;
  prim_batch_f_kernel<KIND, 0, 3><<<g, 64>>>(n, in, lm, out);
  prim_batch_f_kernel<KIND, 1, 3><<<g, 64>>>(n, in, lm, out);
  prim_batch_f_kernel<KIND, 2, 3><<<g, 64>>>(n, in, lm, out);
  prim_batch_f_kernel<KIND, 3, 0><<<g, 64>>>(n, in, lm, out);
  prim_batch_f_kernel<KIND, 3, 1><<<g, 64>>>(n, in, lm, out);
  prim_batch_f_kernel<KIND, 3, 2><<<g, 64>>>(n, in, lm, out);
  prim_batch_f_kernel<KIND, 3, 3><<<g, 64>>>(n, in, lm, out);
}

}  // namespace olc
