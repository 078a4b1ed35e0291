// Integral stages of the hot path on sm_103a.
//
// Stage 1 (primitive kernels, one thread per alpha-pair item, one launch per
//   angular class so a warp runs one straight-line recurrence):  the reference's
//   alpha loop body -- overlap2CIntg / kinetic2CIntg / massvel2CIntg
//   (integrals.F90:312-416, 1150-1236)
//   and the third-centre sums of nuclearPE / electronicPE (integrals.F90:
//   2275-2598) -- producing the harmonic block sh(lm1, lm2) of each item in
//   a scratch buffer.
// Stage 2 (contraction, one warp per (pair, cell) task): the accumulation
//   into pairXBasisFn2 and multWithBasisFn1 (integrals.F90:402-410,
//   intgSaving.F90:56-89) as one sum over the task's items,
//   block(m1,m2) = sum c1(a1,m1) c2(a2,m2) sh(lm(m1), lm(m2)).
// Stage 3 (Bloch sum + scatter, one CTA per (pair, k range)):
//   applyPhaseFactors, kPointLatticeOriginShift and saveCurrentPair
//   (intgSaving.F90:95-505) -- out(m1,m2,k) = e^{ik.L} sum_R e^{ik.R} block_R
//   written straight into valeVale / coreVale / coreCore.
#include <cstdio>

#include "olc_prim_kernel.cuh"

namespace olc {

// ---------------------------------------------------------------------------
// stage 1: primitive kernels
// ---------------------------------------------------------------------------
template <int OP, int MODE>
int launch_class(olc_context* ctx, int cls, const double* coeffs, int ep_type, int ep_alpha,
                 bool accumulate) {
  const ItemLists& it = ctx->items;
  PrimArgs a;
  a.task = it.task[cls];
  a.ab = it.ab[cls];
  a.n = it.count[cls];
  a.out = ctx->d_sh + it.sh_offset[cls];
  a.coeffs = coeffs;
  a.accumulate = accumulate ? 1 : 0;
  a.ep_type = ep_type;
  a.ep_alpha = ep_alpha;
  if (a.n == 0) return OLC_OK;
  const dim3 block(128), grid((a.n + 127) / 128);
  StageScope scope(ctx, OLC_STAGE_PRIMITIVES);
  const int l1 = cls / (kMaxL + 1), l2 = cls % (kMaxL + 1);
  if (l1 == 3 || l2 == 3) {
    switch (OP) {
      case OLC_OP_OVERLAP: return launch_prim_f_overlap(ctx->stream, ctx->view, a, l1, l2, grid, block);
      case OLC_OP_KINETIC: return launch_prim_f_kinetic(ctx->stream, ctx->view, a, l1, l2, grid, block);
      case OLC_OP_MASSVEL: return launch_prim_f_massvel(ctx->stream, ctx->view, a, l1, l2, grid, block);
      case OLC_OP_NUCLEAR: return launch_prim_f_nuclear(ctx->stream, ctx->view, a, l1, l2, grid, block);
      default: return launch_prim_f_elecpot(ctx->stream, ctx->view, a, l1, l2, MODE, grid, block);
    }
  }
  switch (l1 * 3 + l2) {
#define OLC_CASE(c, l1, l2) \
  case c: prim_kernel<OP, l1, l2, MODE><<<grid, block, 0, ctx->stream>>>(ctx->view, a); break;
    OLC_CASE(0, 0, 0) OLC_CASE(1, 0, 1) OLC_CASE(2, 0, 2)
    OLC_CASE(3, 1, 0) OLC_CASE(4, 1, 1) OLC_CASE(5, 1, 2)
    OLC_CASE(6, 2, 0) OLC_CASE(7, 2, 1) OLC_CASE(8, 2, 2)
#undef OLC_CASE
  }
  return cuda_check(cudaGetLastError(), "prim_kernel launch");
}

int run_primitives(olc_context* ctx, int op, int term, const double* coeffs, int precision,
                   bool accumulate) {
  int ep_type = -1, ep_alpha = 0;
  if (op == OLC_OP_ELECPOT && !coeffs) {
    ep_type = -2;
    for (size_t t = 0; t < ctx->hpots.size(); ++t)
      if (term >= ctx->hpots[t].cumul_alpha &&
          term < ctx->hpots[t].cumul_alpha + ctx->hpots[t].num_alphas) {
        ep_type = (int)t;
        ep_alpha = term - ctx->hpots[t].cumul_alpha;
      }
    if (ep_type < 0) return fail(OLC_ERR_ARG, "potential term index out of range");
  }
  // OLC_PREC_MIXED: far-shell electronic-potential images in FP32
  const bool far32 = precision == OLC_PREC_MIXED;
  for (int cls = 0; cls < kNumClasses; ++cls) {
    int st = 0;
    switch (op) {
      case OLC_OP_OVERLAP: st = launch_class<OLC_OP_OVERLAP, 0>(ctx, cls, nullptr, -1, 0, accumulate); break;
      case OLC_OP_KINETIC: st = launch_class<OLC_OP_KINETIC, 0>(ctx, cls, nullptr, -1, 0, accumulate); break;
      case OLC_OP_MASSVEL: st = launch_class<OLC_OP_MASSVEL, 0>(ctx, cls, nullptr, -1, 0, accumulate); break;
      case OLC_OP_NUCLEAR: st = launch_class<OLC_OP_NUCLEAR, 0>(ctx, cls, nullptr, -1, 0, accumulate); break;
      case OLC_OP_ELECPOT:
        if (far32) {
          st = launch_class<OLC_OP_ELECPOT, 1>(ctx, cls, coeffs, ep_type, ep_alpha, accumulate);
          if (!st) st = launch_class<OLC_OP_ELECPOT, 2>(ctx, cls, coeffs, ep_type, ep_alpha, true);
        } else {
          st = launch_class<OLC_OP_ELECPOT, 0>(ctx, cls, coeffs, ep_type, ep_alpha, accumulate);
        }
        break;
      default: return fail(OLC_ERR_ARG, "unknown integral operator");
    }
    if (st) return st;
  }
  return OLC_OK;
}

// ---------------------------------------------------------------------------
// stage 2: contraction with the basis coefficients, one warp per task
// ---------------------------------------------------------------------------
struct ContractArgs {
  const int32_t* ab[kNumClasses];
  const int32_t* start[kNumClasses];
  const double* sh[kNumClasses];
  int ntasks;
  int ms;                   // block stride (max states)
  double* block;            // [task][m2*ms + m1]
};

__global__ void __launch_bounds__(256) contract_kernel(SysView v, ContractArgs a) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= a.ntasks) return;
  const DevTask tk = v.tasks[warp];
  const DevPair p = v.pairs[tk.pair];
  const DevType& t1 = v.types[v.site_type[p.i]];
  const DevType& t2 = v.types[v.site_type[p.j]];
  const int M1 = t1.nstates, M2 = t2.nstates;
  double* out = a.block + (size_t)warp * a.ms * a.ms;
  for (int e = lane; e < M1 * M2; e += 32) {
    const int m1 = e % M1, m2 = e / M1;
    const int lm1 = t1.lm_index[m1] - 1, lm2 = t2.lm_index[m2] - 1;
    double acc = 0.0;
#pragma unroll
    for (int cls = 0; cls < kNumClasses; ++cls) {
      const int l1 = cls / (kMaxL + 1), l2 = cls % (kMaxL + 1);
      const int ns1 = (l1 + 1) * (l1 + 1), ns2 = (l2 + 1) * (l2 + 1);
      if (lm1 >= ns1 || lm2 >= ns2) continue;
      const int b = a.start[cls][warp], en = a.start[cls][warp + 1];
      const double* sh = a.sh[cls];
      for (int q = b; q < en; ++q) {
        const int ab = a.ab[cls][q];
        const int a1 = ab & 255, a2 = ab >> 8;
        acc += t1.basis[a1 * OLC_MAX_STATES + m1] * t2.basis[a2 * OLC_MAX_STATES + m2] *
               sh[(size_t)q * ns1 * ns2 + lm2 * ns1 + lm1];
      }
    }
    out[m2 * a.ms + m1] = acc;
  }
}

// ---------------------------------------------------------------------------
// stage 3: Bloch sum, lattice-origin phase and scatter
// ---------------------------------------------------------------------------
__global__ void phase_table_kernel(SysView v, double* phase) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= v.nk * v.ncells) return;
  const int k = idx / v.ncells, n = idx % v.ncells;
  const double kr = v.kxyz[3 * k] * v.cells[4 * n] + v.kxyz[3 * k + 1] * v.cells[4 * n + 1] +
                    v.kxyz[3 * k + 2] * v.cells[4 * n + 2];
  double s, c;
  sincos(kr, &s, &c);
  phase[2 * idx] = c;
  phase[2 * idx + 1] = s;
}

struct BlochArgs {
  const double* block;
  int ms;
  int kchunk;
  double* vv;
  double* cv;
  double* cc;
};

__global__ void __launch_bounds__(256) bloch_scatter_kernel(SysView v, BlochArgs a) {
  const DevPair p = v.pairs[blockIdx.x];
  const DevType& t1 = v.types[v.site_type[p.i]];
  const DevType& t2 = v.types[v.site_type[p.j]];
  const int M1 = t1.nstates, M2 = t2.nstates;
  const int k0 = blockIdx.y * a.kchunk;
  const int k1 = min(v.nk, k0 + a.kchunk);
  const int per_k = M1 * M2;
  const int total = per_k * (k1 - k0);
  const size_t nv = v.vale_dim, nc = v.core_dim;
  const bool same = (p.i == p.j);
  const int vi1 = v.cum_vale[p.i], vi2 = v.cum_vale[p.j];
  const int ci1 = v.cum_core[p.i], ci2 = v.cum_core[p.j];
  const int vn1 = t1.nvale, vn2 = t2.nvale;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int k = k0 + e / per_k;
    const int r = e % per_k;
    const int m1 = r % M1, m2 = r / M1;
    double re = 0.0, im = 0.0;
    const double* ph = v.phase + 2 * (size_t)k * v.ncells;
    for (int t = p.task_begin; t < p.task_end; ++t) {
      const int cell = v.tasks[t].cell;
      const double b = a.block[(size_t)t * a.ms * a.ms + m2 * a.ms + m1];
      re += ph[2 * cell] * b;
      im += ph[2 * cell + 1] * b;
    }
    const double kl = v.kxyz[3 * k] * p.L[0] + v.kxyz[3 * k + 1] * p.L[1] + v.kxyz[3 * k + 2] * p.L[2];
    if (kl != 0.0) {
      double s, c;
      sincos(kl, &s, &c);
      const double nr = c * re - s * im, ni = s * re + c * im;
      re = nr;
      im = ni;
    }
    // saveCurrentPair (intgSaving.F90:201-505)
    if (m1 < vn1 && m2 < vn2) {
      const size_t row = vi1 + m1, col = vi2 + m2;
      double* d = a.vv + 2 * ((size_t)k * nv * nv + col * nv + row);
      if (same && m1 > m2) { d[0] = 0.0; d[1] = 0.0; }
      else { d[0] = re; d[1] = im; }
    } else if (m1 >= vn1 && m2 < vn2) {
      if (!same) {
        double* d = a.cv + 2 * ((size_t)k * nc * nv + (size_t)(vi2 + m2) * nc + ci1 + (m1 - vn1));
        d[0] = re;
        d[1] = im;
      }
    } else if (m1 < vn1 && m2 >= vn2) {
      double* d = a.cv + 2 * ((size_t)k * nc * nv + (size_t)(vi1 + m1) * nc + ci2 + (m2 - vn2));
      d[0] = re;
      d[1] = -im;
    } else {
      const int c1 = m1 - vn1, c2 = m2 - vn2;
      double* d = a.cc + 2 * ((size_t)k * nc * nc + (size_t)(ci2 + c2) * nc + ci1 + c1);
      d[0] = re;
      d[1] = im;
      if (!same) {
        double* e2 = a.cc + 2 * ((size_t)k * nc * nc + (size_t)(ci1 + c1) * nc + ci2 + c2);
        e2[0] = re;
        e2[1] = -im;
      }
    }
  }
}

int run_contract_bloch(olc_context* ctx, double* vv, double* cv, double* cc) {
  const SysView& v = ctx->view;
  const int ntasks = ctx->dims.num_pair_tasks;
  const size_t nv = v.vale_dim, nc = v.core_dim, nk = v.nk;
  int st;
  if ((st = cuda_check(cudaMemsetAsync(vv, 0, 16 * nv * nv * nk, ctx->stream), "memset vv"))) return st;
  if (nc) {
    if (!cv || !cc) return fail(OLC_ERR_ARG, "core outputs required when core_dim > 0");
    if ((st = cuda_check(cudaMemsetAsync(cv, 0, 16 * nc * nv * nk, ctx->stream), "memset cv"))) return st;
    if ((st = cuda_check(cudaMemsetAsync(cc, 0, 16 * nc * nc * nk, ctx->stream), "memset cc"))) return st;
  }
  if (ntasks == 0) return OLC_OK;
  ContractArgs ca;
  for (int c = 0; c < kNumClasses; ++c) {
    ca.ab[c] = ctx->items.ab[c];
    ca.start[c] = ctx->items.task_start[c];
    ca.sh[c] = ctx->d_sh + ctx->items.sh_offset[c];
  }
  ca.ntasks = ntasks;
  ca.ms = ctx->max_states;
  ca.block = ctx->d_block;
  {
    StageScope scope(ctx, OLC_STAGE_CONTRACT);
    contract_kernel<<<(ntasks + 7) / 8, 256, 0, ctx->stream>>>(v, ca);
  }
  if ((st = cuda_check(cudaGetLastError(), "contract_kernel"))) return st;
  BlochArgs ba;
  const int per_k_cap = 256;
  ba.block = ctx->d_block;
  ba.ms = ctx->max_states;
  const int per_k = ctx->max_states * ctx->max_states;
  ba.kchunk = std::max(1, std::min((int)nk, per_k_cap * 4 / std::max(1, per_k)));
  ba.vv = vv;
  ba.cv = cv;
  ba.cc = cc;
  dim3 grid((unsigned)ctx->hpairs.size(), (unsigned)((nk + ba.kchunk - 1) / ba.kchunk));
  StageScope scope(ctx, OLC_STAGE_BLOCH);
  bloch_scatter_kernel<<<grid, 256, 0, ctx->stream>>>(v, ba);
  return cuda_check(cudaGetLastError(), "bloch_scatter_kernel");
}

int build_phase_table(olc_context* ctx) {
  const SysView& v = ctx->view;
  const int n = v.nk * v.ncells;
  count_launch();
  phase_table_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(v, const_cast<double*>(v.phase));
  return cuda_check(cudaGetLastError(), "phase_table_kernel");
}

// ---------------------------------------------------------------------------
// primitive batch (testing entry): explicit inputs, one thread per primitive
// ---------------------------------------------------------------------------
__global__ void prim_batch_kernel(int kind, int n, const double* in, const int32_t* lm,
                                  double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto lof = [](int lma) { return lma == 1 ? 0 : lma == 4 ? 1 : 2; };
  if (lm[2 * i] == 16 || lm[2 * i + 1] == 16) return;      // f classes: prim_batch_f_kernel
  const int c = lof(lm[2 * i]) * 3 + lof(lm[2 * i + 1]);
  const double* x = in + 12 * i;
  double* o = out + 256 * i;
  switch (c) {
    case 0: prim_one<0, 0>(kind, x, o); break;
    case 1: prim_one<0, 1>(kind, x, o); break;
    case 2: prim_one<0, 2>(kind, x, o); break;
    case 3: prim_one<1, 0>(kind, x, o); break;
    case 4: prim_one<1, 1>(kind, x, o); break;
    case 5: prim_one<1, 2>(kind, x, o); break;
    case 6: prim_one<2, 0>(kind, x, o); break;
    case 7: prim_one<2, 1>(kind, x, o); break;
    case 8: prim_one<2, 2>(kind, x, o); break;
  }
}

int primitive_batch_device(int kind, int n, const double* in, const int32_t* lmalpha,
                           double* out) {
  if (kind < 1 || kind > 8 || n < 0) return fail(OLC_ERR_ARG, "olc_primitive_batch: bad kind");
  for (int i = 0; i < n; ++i) {
    for (int s = 0; s < 2; ++s) {
      int l = lmalpha[2 * i + s];
      if (l != 1 && l != 4 && l != 9 && l != 16)
        return fail(OLC_ERR_ARG, "lmalpha must be 1, 4, 9 or 16");
    }
  }
  if (n == 0) return OLC_OK;
  double *din = nullptr, *dout = nullptr;
  int32_t* dlm = nullptr;
  int st = OLC_OK;
  if ((st = cuda_check(cudaMalloc(&din, sizeof(double) * 12 * n), "malloc"))) return st;
  if ((st = cuda_check(cudaMalloc(&dout, sizeof(double) * 256 * n), "malloc"))) { cudaFree(din); return st; }
  if ((st = cuda_check(cudaMalloc(&dlm, sizeof(int32_t) * 2 * n), "malloc"))) { cudaFree(din); cudaFree(dout); return st; }
  st = cuda_check(cudaMemcpy(din, in, sizeof(double) * 12 * n, cudaMemcpyHostToDevice), "copy");
  if (!st) st = cuda_check(cudaMemcpy(dlm, lmalpha, sizeof(int32_t) * 2 * n, cudaMemcpyHostToDevice), "copy");
  if (!st) st = cuda_check(cudaMemset(dout, 0, sizeof(double) * 256 * n), "memset");
  if (!st) {
    count_launch();
    prim_batch_kernel<<<(n + 63) / 64, 64>>>(kind, n, din, dlm, dout);
    switch (kind) {
      case 1: launch_prim_batch_f_overlap(n, din, dlm, dout); break;
      case 2: launch_prim_batch_f_kinetic(n, din, dlm, dout); break;
      case 3: launch_prim_batch_f_nuclear(n, din, dlm, dout); break;
      case 4: launch_prim_batch_f_elecpot(n, din, dlm, dout); break;
      case 5: launch_prim_batch_f_massvel(n, din, dlm, dout); break;
      default: launch_prim_batch_f_momentum(kind, n, din, dlm, dout); break;
    }
    count_launch(7);
    st = cuda_check(cudaGetLastError(), "prim_batch_kernel");
  }
  if (!st) st = cuda_check(cudaMemcpy(out, dout, sizeof(double) * 256 * n, cudaMemcpyDeviceToHost), "copy back");
  cudaFree(din);
  cudaFree(dout);
  cudaFree(dlm);
  return st;
}

}  // namespace olc
