// Host-side set-up of a context: lattice, k-points, basis, screening tables,
// the (atom pair, lattice cell) task list and the alpha-pair work items.
//
// Restates, for the device data layout:
//   getRecipCellVectors / setCutoffThresh / initializeLattice / makeLattice /
//   cellBorderCheck        src/olcao/lattice.f90:180-215, 229-286, 300-432, 456-747
//   convertKPointsToXYZ    src/olcao/kpoints.f90:251-281
//   renormalizeBasis       src/olcao/basis.f90:55-243
//   makeAlpha*Dist         src/olcao/gaussRelations.f90:64-278
//   pair / cell screening  src/olcao/integrals.F90:199-286
//   alpha-pair traversal   src/olcao/integrals.F90:312-416 (as the staircase set
//                          {(a1, a2) : alphaDist(a1, a2) >= |A - B'|^2}, which
//                          the reference's diagonal/mode walk enumerates because
//                          the exponents ascend)
#include <algorithm>
#include <cmath>
#include <cstring>

#include "olc_common.h"

namespace olc {
namespace {

const double kAngNorm[16] = {
    0.2820947917738782, 0.4886025119029199, 0.4886025119029199, 0.4886025119029199,
    1.0925484305920790, 1.0925484305920790, 1.0925484305920790, 0.5462742152960396,
    0.3153915652525200, 2.8906114426405543, 1.4453057213202771, 0.5900435899266435,
    0.5900435899266435, 0.3731763325901154, 0.4570457994644657, 0.4570457994644657};

struct Lattice {
  double rv[3][3];        // [abc][xyz]
  double recip[3][3];     // [abc][xyz]
  double inv[3][3];
  double maxSq = 0;
  std::vector<double> cells;   // x, y, z, |R|^2
  int nnear = 0;

  void nearest(const double* v, double* L) const {
    double base[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i) {
      double f = v[0] * inv[i][0] + v[1] * inv[i][1] + v[2] * inv[i][2];
      double r = std::floor(std::fabs(f) + 0.5);
      if (f < 0) r = -r;
      for (int c = 0; c < 3; ++c) base[c] += rv[i][c] * r;
    }
    double best = 0;
    for (int c = 0; c < 3; ++c) best += (v[c] - base[c]) * (v[c] - base[c]);
    int bi = -1;
    for (int n = 1; n < nnear; ++n) {
      double d = 0;
      for (int c = 0; c < 3; ++c) {
        double x = v[c] - base[c] - cells[4 * n + c];
        d += x * x;
      }
      if (d < best) { best = d; bi = n; }
    }
    for (int c = 0; c < 3; ++c) L[c] = base[c] + (bi >= 0 ? cells[4 * bi + c] : 0.0);
  }
};

void make_lattice(Lattice& lat, double negl) {
  int reps[3];
  for (int i = 0; i < 3; ++i) {
    double len = std::sqrt(lat.rv[i][0] * lat.rv[i][0] + lat.rv[i][1] * lat.rv[i][1] +
                           lat.rv[i][2] * lat.rv[i][2]);
    reps[i] = 2 * (int)std::ceil(std::sqrt(negl) / len) + 1;
  }
  double shifts[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) shifts[c] += lat.rv[i][c];
  std::vector<std::pair<double, int>> order;
  std::vector<double> dims;
  for (int i = 1; i <= reps[0]; ++i)
    for (int j = 1; j <= reps[1]; ++j)
      for (int k = 1; k <= reps[2]; ++k) {
        int rep[3] = {i - (1 + reps[0]) / 2, j - (1 + reps[1]) / 2, k - (1 + reps[2]) / 2};
        double d[3] = {0, 0, 0};
        for (int l = 0; l < 3; ++l)
          for (int c = 0; c < 3; ++c) d[c] += lat.rv[l][c] * rep[l];
        double sq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (sq > negl) {
          // a cell is kept when one of seven further corners lies inside
          static const int walk[7][2] = {{0, 1}, {1, 1}, {0, -1}, {2, 1}, {0, 1}, {1, -1}, {0, -1}};
          double t[3] = {d[0], d[1], d[2]};
          bool in = false;
          for (int q = 0; q < 7 && !in; ++q) {
            t[walk[q][0]] += walk[q][1] * shifts[walk[q][0]];
            in = (t[0] * t[0] + t[1] * t[1] + t[2] * t[2] < negl);
          }
          if (!in) continue;
        }
        order.push_back({sq, (int)dims.size() / 3});
        dims.insert(dims.end(), d, d + 3);
      }
  std::stable_sort(order.begin(), order.end(),
                   [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
                     return a.first < b.first;
                   });
  lat.cells.resize(4 * order.size());
  for (size_t n = 0; n < order.size(); ++n) {
    for (int c = 0; c < 3; ++c) lat.cells[4 * n + c] = dims[3 * order[n].second + c];
    lat.cells[4 * n + 3] = order[n].first;
  }
  lat.nnear = 0;
  while (lat.nnear < (int)order.size() && lat.cells[4 * lat.nnear + 3] <= 3.0 * lat.maxSq * (1 + 1e-12))
    ++lat.nnear;
}

template <class T>
int upload(olc_context* ctx, T** dst, const std::vector<T>& src) {
  if (src.empty()) { *dst = nullptr; return OLC_OK; }
  int st = dalloc(ctx, dst, src.size());
  if (st) return st;
  return cuda_check(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice),
                    "upload");
}

int lmax_of_alpha(const olc_atom_type_t& t, int a /*0-based*/) {
  int j = a + 1;
  if (j <= t.num_orb_alphas[3]) return 3;
  if (j <= t.num_orb_alphas[2]) return 2;
  if (j <= t.num_orb_alphas[1]) return 1;
  return 0;
}

}  // namespace

int build_system(olc_context* ctx, const olc_system_t* s) {
  if (!s || s->num_atom_types <= 0 || s->num_atom_sites <= 0 || s->num_kpoints <= 0 ||
      !s->atom_types || !s->site_type || !s->site_pos || !s->kpoints_abc)
    return fail(OLC_ERR_ARG, "olc_create: incomplete system description");
  if (!(s->basis_fn_thresh > 0.0 && s->basis_fn_thresh < 1.0))
    return fail(OLC_ERR_ARG, "olc_create: basis_fn_thresh must be in (0,1)");
  if (s->rel != 0 && s->rel != 1) return fail(OLC_ERR_ARG, "olc_create: rel must be 0 or 1");
  ctx->rel = s->rel;
  Lattice lat;
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) lat.rv[i][c] = s->real_vectors[i * 3 + c];
  for (int i = 0; i < 3; ++i) {
    int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
    for (int j = 0; j < 3; ++j) {
      int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      lat.recip[i][j] = lat.rv[i1][j1] * lat.rv[i2][j2] - lat.rv[i1][j2] * lat.rv[i2][j1];
    }
  }
  double vol = 0;
  for (int j = 0; j < 3; ++j) vol += lat.recip[0][j] * lat.rv[0][j];
  if (std::fabs(vol) < 1e-12) return fail(OLC_ERR_ARG, "olc_create: singular lattice");
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      lat.recip[i][j] = 2.0 * kPi * lat.recip[i][j] / vol;
      lat.inv[i][j] = lat.recip[i][j] / (2.0 * kPi);
    }
  const double T = -std::log(s->basis_fn_thresh);

  // ---- atom types --------------------------------------------------------
  int nelem = 0;
  double minAtomicAlpha = 100.0, minPotAlpha = 10000.0;
  ctx->htypes.assign(s->num_atom_types, DevType{});
  int maxStates = 0;
  for (int t = 0; t < s->num_atom_types; ++t) {
    const olc_atom_type_t& at = s->atom_types[t];
    DevType& d = ctx->htypes[t];
    if (at.element < 1) return fail(OLC_ERR_ARG, "atom type element ids are 1-based");
    nelem = std::max(nelem, at.element);
    d.element = at.element - 1;
    d.nalpha = at.num_orb_alphas[0];
    if (d.nalpha < 1 || d.nalpha > OLC_MAX_ALPHAS)
      return fail(OLC_ERR_ARG, "num_orb_alphas[0] out of range");
    for (int l = 1; l < 4; ++l)
      if (at.num_orb_alphas[l] > at.num_orb_alphas[l - 1])
        return fail(OLC_ERR_ARG, "numOrbAlphas must not increase with l");
    for (int a = 0; a < d.nalpha; ++a) {
      d.alphas[a] = at.alphas[a];
      if (a > 0 && !(at.alphas[a] > at.alphas[a - 1]))
        return fail(OLC_ERR_ARG, "atomic exponents must ascend");
      d.lmax_alpha[a] = lmax_of_alpha(at, a);
    }
    minAtomicAlpha = std::min(minAtomicAlpha, at.alphas[0]);
    int m = 0, nrad = at.num_vale_radial + at.num_core_radial;
    if (nrad > OLC_MAX_RADIAL) return fail(OLC_ERR_ARG, "too many radial functions");
    for (int r = 0; r < nrad; ++r) {
      int l = at.radial_l[r];
      if (l < 0 || l > kMaxL) return fail(OLC_ERR_ARG, "radial functions have l = 0..3 (s, p, d, f)");
      int na = at.num_orb_alphas[l];
      for (int k = 1; k <= 2 * l + 1; ++k) {
        if (m >= OLC_MAX_STATES) return fail(OLC_ERR_ARG, "too many states per type");
        d.lm_index[m] = l * l + k;
        for (int a = 0; a < na; ++a)
          d.basis[a * OLC_MAX_STATES + m] = at.radial_coeff[r][a] * kAngNorm[l * l + k - 1];
        ++m;
      }
      if (r + 1 == at.num_vale_radial) d.nvale = m;
    }
    d.nstates = m;
    d.ncore = m - d.nvale;
    maxStates = std::max(maxStates, m);
  }
  ctx->max_states = maxStates;

  // ---- potential types / sites --------------------------------------------
  const int npt = s->num_pot_types;
  ctx->hpots.assign(npt, DevPotType{});
  int potDim = 0;
  for (int t = 0; t < npt; ++t) {
    const olc_pot_type_t& p = s->pot_types[t];
    DevPotType& d = ctx->hpots[t];
    if (p.element < 1) return fail(OLC_ERR_ARG, "potential element ids are 1-based");
    if (p.num_alphas < 1 || p.num_alphas > OLC_MAX_POT_ALPHAS)
      return fail(OLC_ERR_ARG, "potential num_alphas out of range");
    nelem = std::max(nelem, p.element);
    d.element = p.element - 1;
    d.num_alphas = p.num_alphas;
    d.nuc_charge = p.nuc_charge;
    d.nuc_alpha = p.nuc_alpha;
    for (int a = 0; a < p.num_alphas; ++a) d.alphas[a] = p.alphas[a];
    d.cumul_alpha = potDim;
    potDim += p.num_alphas;
    d.first_site = -1;
    minPotAlpha = std::min(minPotAlpha, p.alphas[0]);
  }
  for (int m = 0; m < s->num_pot_sites; ++m) {
    int t = s->pot_site_type[m];
    if (t < 0 || t >= npt) return fail(OLC_ERR_ARG, "pot_site_type out of range");
    DevPotType& d = ctx->hpots[t];
    if (d.first_site < 0) d.first_site = m;
    else if (d.first_site + d.multiplicity != m)
      return fail(OLC_ERR_ARG, "potential sites of one type must be consecutive");
    d.multiplicity++;
  }
  ctx->nelem = nelem;
  std::vector<double> elemAlpha((size_t)nelem * OLC_MAX_ALPHAS, 0.0);
  std::vector<double> elemPot((size_t)nelem * OLC_MAX_POT_ALPHAS, 0.0);
  std::vector<double> elemNuc(nelem, 0.0);
  std::vector<int> elemHasAlpha(nelem, 0), elemHasPot(nelem, 0);
  for (auto& d : ctx->htypes)
    if (!elemHasAlpha[d.element]) {
      elemHasAlpha[d.element] = 1;
      for (int a = 0; a < d.nalpha; ++a) elemAlpha[(size_t)d.element * OLC_MAX_ALPHAS + a] = d.alphas[a];
    }
  for (auto& d : ctx->hpots) {
    if (!elemHasPot[d.element]) {
      elemHasPot[d.element] = 1;
      for (int a = 0; a < d.num_alphas; ++a)
        elemPot[(size_t)d.element * OLC_MAX_POT_ALPHAS + a] = d.alphas[a];
    }
    if (elemNuc[d.element] == 0.0) elemNuc[d.element] = d.nuc_alpha;
  }
  auto alphaDist = [&](int a1, int a2, int e1, int e2) {
    double al = elemAlpha[(size_t)e1 * OLC_MAX_ALPHAS + a1];
    double ak = elemAlpha[(size_t)e2 * OLC_MAX_ALPHAS + a2];
    return T / ak / (al / (al + ak));
  };

  // ---- lattice (initializeLattice) -----------------------------------------
  double negl = T * std::max(2.0 / minAtomicAlpha, 1.0 / minPotAlpha + 0.5 / minAtomicAlpha);
  for (int i = 0; i < 3; ++i) {
    double sq = lat.rv[i][0] * lat.rv[i][0] + lat.rv[i][1] * lat.rv[i][1] + lat.rv[i][2] * lat.rv[i][2];
    lat.maxSq = std::max(lat.maxSq, sq);
  }
  const double neglBase = negl;
  negl = negl + 0.75 * lat.maxSq + std::sqrt(3.0 * lat.maxSq * negl);
  negl = std::max(negl, 2.0 * T / minAtomicAlpha);
  // The reference's cell list (its last |R|^2 bounds the pair loops and gives
  // the "More lattice points needed" stop).  The device list is extended so
  // that third-centre images found from a rounded (not nearest) origin are
  // always covered: |r| <= (|a|+|b|+|c|)/2 for the rounding residual.
  make_lattice(lat, negl);
  const double refMaxCell = lat.cells[lat.cells.size() - 1];
  double half = 0.0;
  for (int i = 0; i < 3; ++i)
    half += 0.5 * std::sqrt(lat.rv[i][0] * lat.rv[i][0] + lat.rv[i][1] * lat.rv[i][1] +
                            lat.rv[i][2] * lat.rv[i][2]);
  const double ext = std::pow(std::sqrt(neglBase) + half, 2) * (1.0 + 1e-9);
  if (ext > negl) make_lattice(lat, ext);
  const int ncells = (int)(lat.cells.size() / 4);

  // ---- sites ----------------------------------------------------------------
  const int ns = s->num_atom_sites;
  std::vector<int32_t> siteType(s->site_type, s->site_type + ns);
  std::vector<double> sitePos(s->site_pos, s->site_pos + 3 * ns);
  std::vector<int32_t> cumVale(ns), cumCore(ns);
  int valeDim = 0, coreDim = 0;
  for (int i = 0; i < ns; ++i) {
    if (siteType[i] < 0 || siteType[i] >= s->num_atom_types)
      return fail(OLC_ERR_ARG, "site_type out of range");
    cumVale[i] = valeDim;
    cumCore[i] = coreDim;
    valeDim += ctx->htypes[siteType[i]].nvale;
    coreDim += ctx->htypes[siteType[i]].ncore;
  }

  // ---- pairs, tasks ---------------------------------------------------------
  ctx->hpairs.clear();
  ctx->htasks.clear();
  const double maxCell = refMaxCell;
  for (int i = 0; i < ns; ++i) {
    const DevType& t1 = ctx->htypes[siteType[i]];
    const double* A = &sitePos[3 * i];
    for (int j = i; j < ns; ++j) {
      const DevType& t2 = ctx->htypes[siteType[j]];
      const double* B = &sitePos[3 * j];
      double dv[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
      double L[3];
      lat.nearest(dv, L);
      double sepSq = 0;
      for (int c = 0; c < 3; ++c) sepSq += (dv[c] - L[c]) * (dv[c] - L[c]);
      double nl = alphaDist(0, 0, t1.element, t2.element);
      if (sepSq > nl) continue;
      double maxR = sepSq + nl + 2.0 * std::sqrt(sepSq * nl);
      if (maxR > maxCell)
        return fail(OLC_ERR_LATTICE, "More lattice points needed for this atom overlap pair");
      DevPair p{};
      p.i = i;
      p.j = j;
      for (int c = 0; c < 3; ++c) p.L[c] = L[c];
      p.task_begin = (int)ctx->htasks.size();
      for (int n = 0; n < ncells; ++n) {
        if (lat.cells[4 * n + 3] > maxR) break;
        double sep = 0;
        for (int c = 0; c < 3; ++c) {
          double x = A[c] - (B[c] + L[c] + lat.cells[4 * n + c]);
          sep += x * x;
        }
        if (sep > nl) continue;
        ctx->htasks.push_back(DevTask{(int32_t)ctx->hpairs.size(), n, sep});
      }
      p.task_end = (int)ctx->htasks.size();
      if (p.task_end > p.task_begin) ctx->hpairs.push_back(p);
    }
  }
  const int ntasks = (int)ctx->htasks.size();

  // ---- alpha-pair items grouped by (l1, l2) class -------------------------
  std::vector<int32_t> itTask[kNumClasses], itAB[kNumClasses], itStart[kNumClasses];
  for (int c = 0; c < kNumClasses; ++c) itStart[c].assign(ntasks + 1, 0);
  for (int q = 0; q < ntasks; ++q) {
    const DevTask& tk = ctx->htasks[q];
    const DevPair& p = ctx->hpairs[tk.pair];
    const DevType& t1 = ctx->htypes[siteType[p.i]];
    const DevType& t2 = ctx->htypes[siteType[p.j]];
    for (int c = 0; c < kNumClasses; ++c) itStart[c][q] = (int32_t)itTask[c].size();
    for (int a1 = 0; a1 < t1.nalpha; ++a1) {
      for (int a2 = 0; a2 < t2.nalpha; ++a2) {
        if (alphaDist(a1, a2, t1.element, t2.element) < tk.sep) break;
        int cls = t1.lmax_alpha[a1] * (kMaxL + 1) + t2.lmax_alpha[a2];
        itTask[cls].push_back(q);
        itAB[cls].push_back(a1 | (a2 << 8));
      }
    }
  }
  for (int c = 0; c < kNumClasses; ++c) itStart[c][ntasks] = (int32_t)itTask[c].size();

  // ---- k-points ---------------------------------------------------------------
  const int nk = s->num_kpoints;
  std::vector<double> kxyz(3 * nk);
  for (int q = 0; q < nk; ++q)
    for (int c = 0; c < 3; ++c) {
      double v = 0;
      for (int i = 0; i < 3; ++i) v += s->kpoints_abc[3 * q + i] * lat.recip[i][c];
      kxyz[3 * q + c] = v;
    }

  // ---- upload ------------------------------------------------------------------
  SysView& v = ctx->view;
  int st = 0;
  DevType* dTypes;
  if ((st = upload(ctx, &dTypes, ctx->htypes))) return st;
  v.types = dTypes;
  int32_t* dst;
  double* dd;
  if ((st = upload(ctx, &dst, siteType))) return st;
  v.site_type = dst;
  if ((st = upload(ctx, &dd, sitePos))) return st;
  v.site_pos = dd;
  if ((st = upload(ctx, &dst, cumVale))) return st;
  v.cum_vale = dst;
  if ((st = upload(ctx, &dst, cumCore))) return st;
  v.cum_core = dst;
  DevPair* dPairs;
  if ((st = upload(ctx, &dPairs, ctx->hpairs))) return st;
  v.pairs = dPairs;
  DevTask* dTasks;
  if ((st = upload(ctx, &dTasks, ctx->htasks))) return st;
  v.tasks = dTasks;
  if ((st = upload(ctx, &dd, lat.cells))) return st;
  v.cells = dd;
  v.ncells = ncells;
  ctx->hcells = lat.cells;
  DevPotType* dPots;
  if ((st = upload(ctx, &dPots, ctx->hpots))) return st;
  v.pot_types = dPots;
  v.num_pot_types = npt;
  std::vector<double> potPos(s->pot_site_pos, s->pot_site_pos + 3 * s->num_pot_sites);
  std::vector<int32_t> potType(s->pot_site_type, s->pot_site_type + s->num_pot_sites);
  if ((st = upload(ctx, &dd, potPos))) return st;
  v.pot_site_pos = dd;
  if ((st = upload(ctx, &dst, potType))) return st;
  v.pot_site_type = dst;
  v.num_pot_sites = s->num_pot_sites;
  if ((st = upload(ctx, &dd, elemAlpha))) return st;
  v.elem_alpha = dd;
  if ((st = upload(ctx, &dd, elemNuc))) return st;
  v.elem_nuc_alpha = dd;
  if ((st = upload(ctx, &dd, elemPot))) return st;
  v.elem_pot_alpha = dd;
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) {
      v.inv_real[i * 3 + c] = lat.inv[i][c];
      v.real_vec[i * 3 + c] = lat.rv[i][c];
    }
  v.log_thresh = T;
  v.vale_dim = valeDim;
  v.core_dim = coreDim;
  v.nk = nk;
  if ((st = upload(ctx, &dd, kxyz))) return st;
  v.kxyz = dd;
  double* dphase;
  if ((st = dalloc(ctx, &dphase, (size_t)2 * nk * ncells))) return st;
  v.phase = dphase;

  ItemLists& it = ctx->items;
  int64_t shOff = 0;
  for (int c = 0; c < kNumClasses; ++c) {
    int l1 = c / (kMaxL + 1), l2 = c % (kMaxL + 1);
    it.count[c] = (int32_t)itTask[c].size();
    it.sh_offset[c] = shOff;
    shOff += (int64_t)it.count[c] * (l1 + 1) * (l1 + 1) * (l2 + 1) * (l2 + 1);
    if ((st = upload(ctx, &it.task[c], itTask[c]))) return st;
    if ((st = upload(ctx, &it.ab[c], itAB[c]))) return st;
    if ((st = upload(ctx, &it.task_start[c], itStart[c]))) return st;
  }
  it.total_sh = shOff;
  if ((st = dalloc(ctx, &ctx->d_sh, (size_t)std::max<int64_t>(shOff, 1)))) return st;
  ctx->block_stride = (int64_t)maxStates * maxStates;
  if ((st = dalloc(ctx, &ctx->d_block, (size_t)std::max(1, ntasks) * ctx->block_stride))) return st;

  olc_dims_t& dm = ctx->dims;
  dm.vale_dim = valeDim;
  dm.core_dim = coreDim;
  dm.pot_dim = potDim;
  dm.num_kpoints = nk;
  dm.num_cells = ncells;
  dm.num_pair_tasks = ntasks;
  dm.packed_len = (int64_t)valeDim * (valeDim + 1) / 2;
  return OLC_OK;
}

}  // namespace olc
