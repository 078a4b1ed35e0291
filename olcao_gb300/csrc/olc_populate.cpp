// Occupation of the eigenstates: populateStates (src/olcao/populate.F90:132-578).
//
// Host code: the input is numStates x numKPoints x spin eigenvalues (tens of
// thousands of numbers per SCF iteration), the work a sort and a bisection,
// so it runs where the reference runs it, on the host, between the eigen-
// solve and the valence density.
//
//  * The eigenvalues are listed k-point by k-point, spin by spin, state by
//    state (populate.F90:224-232) and sorted by the reference's bottom-up
//    merge of adjacent runs (sortSubs.f90:18-175).  On equal values that
//    merge takes the element of the second run first; it is restated here
//    step for step so that ties are broken the same way.
//  * populateStandard (:172-415): fill the sorted states with kPointWeight(k)
//    / spin electrons each until numElectrons are placed (the last one
//    partially), then spread the charge of the highest occupied level evenly
//    over the states within smallThresh of its energy.
//  * populateSmearing (:418-578), when thermal_sigma != 0: bisection for the
//    Fermi energy between (highest occupied - fermiSearchLimit) and (next
//    state + fermiSearchLimit), populations weighted by the step function
//    1 / (1 + exp((e - eF) / sigma)) cut at +-maxThermalRange
//    (mathSubs.f90:164-185), at most 500 steps, stopping when the charge is
//    within smallThresh of numElectrons.
// XANES core holes (excitedQN_n, correctCorePopulation) are not handled.
#include <cmath>
#include <vector>

#include "olc_common.h"

namespace olc {

namespace {

constexpr double kSmallThresh = 1.0e-8;   // smallThresh, src/constants.f90:49

// One pass of the bottom-up merge over the current runs (borders[0..nseg]).
void merge_runs(const std::vector<double>& fd, std::vector<double>& td, const std::vector<int>& fo,
                std::vector<int>& to, std::vector<int>& borders, int nseg) {
  size_t tp = 0;
  for (int i = 0; i < nseg / 2; ++i) {
    size_t p1 = borders[2 * i], p2 = borders[2 * i + 1];
    const size_t e1 = borders[2 * i + 1], e2 = borders[2 * i + 2];
    while (tp < e2) {
      if (p1 < e1 && (p2 >= e2 || fd[p1] < fd[p2])) {
        td[tp] = fd[p1];
        to[tp++] = fo[p1++];
      } else {
        td[tp] = fd[p2];
        to[tp++] = fo[p2++];
      }
    }
    borders[i + 1] = (int)e2;
  }
  if (nseg % 2) {
    for (size_t q = tp; q < (size_t)borders[nseg]; ++q) {
      td[q] = fd[q];
      to[q] = fo[q];
    }
    borders[nseg / 2 + 1] = borders[nseg];
  }
}

// Sorted values and, for each, its index in the unsorted list.
void merge_sort(const std::vector<double>& in, std::vector<double>& sorted, std::vector<int>& order) {
  const int n = (int)in.size();
  std::vector<double> a(in), b(n);
  std::vector<int> oa(n), ob(n), borders(n + 1);
  for (int i = 0; i < n; ++i) oa[i] = i;
  for (int i = 0; i <= n; ++i) borders[i] = i;
  int nseg = n;
  bool in_a = true;
  while (nseg > 1) {
    if (in_a) merge_runs(a, b, oa, ob, borders, nseg);
    else merge_runs(b, a, ob, oa, borders, nseg);
    in_a = !in_a;
    nseg = nseg / 2 + nseg % 2;
  }
  sorted = in_a ? a : b;
  order = in_a ? oa : ob;
}

double step_function(double x, double range) {
  if (x > range) return 0.0;
  if (x < -range) return 1.0;
  return 1.0 / (1.0 + std::exp(x));
}

}  // namespace

int populate_states(int num_states, int nk, int spin, const double* eig, const double* kweight,
                    double num_electrons, double thermal_sigma, double fermi_search_limit,
                    double max_thermal_range, double* occupation, double* occupied_energy) {
  const int nseg = num_states * nk * spin;
  // grouped by k-point, then spin, then state (populate.F90:224-232)
  std::vector<double> list(nseg);
  std::vector<int> kpt(nseg);
  int q = 0;
  for (int k = 0; k < nk; ++k)
    for (int s = 0; s < spin; ++s)
      for (int j = 0; j < num_states; ++j) {
        list[q] = eig[j + (size_t)num_states * (k + (size_t)nk * s)];
        kpt[q++] = k;
      }
  std::vector<double> sorted;
  std::vector<int> order;
  merge_sort(list, sorted, order);
  auto weight = [&](int i) { return kweight[kpt[order[i]]] / spin; };

  std::vector<double> pop(nseg, 0.0);
  double placed = 0.0;
  int occ = -1;
  for (int i = 0; i < nseg; ++i) {
    pop[order[i]] = weight(i);
    placed += pop[order[i]];
    if (placed > num_electrons) {
      pop[order[i]] = weight(i) + num_electrons - placed;
      placed = num_electrons;
    }
    if (std::fabs(num_electrons - placed) < kSmallThresh) {
      occ = i;
      break;
    }
  }
  if (occ < 0)
    return fail(OLC_ERR_ARG, "olc_populate_states: the states hold fewer electrons than num_electrons");
  double eocc = sorted[occ];
  // spread the highest occupied level's charge over its degenerate states
  int lo = occ, hi = occ;
  double charge = pop[order[occ]], possible = weight(occ);
  while (hi + 1 < nseg && std::fabs(eocc - sorted[hi + 1]) <= kSmallThresh) {
    ++hi;
    possible += weight(hi);
  }
  while (lo > 0 && std::fabs(eocc - sorted[lo - 1]) <= kSmallThresh) {
    --lo;
    possible += weight(lo);
    charge += weight(lo);
  }
  for (int i = lo; i <= hi; ++i) pop[order[i]] = charge / possible * weight(i);
  occ = hi;
  eocc = sorted[occ];

  if (thermal_sigma != 0.0) {
    double emin = sorted[occ] - fermi_search_limit;
    double emax = sorted[std::min(occ + 1, nseg - 1)] + fermi_search_limit;
    for (int it = 0; it < 500; ++it) {
      eocc = 0.5 * (emin + emax);
      double sum = 0.0;
      std::fill(pop.begin(), pop.end(), 0.0);
      for (int i = 0; i < nseg; ++i) {
        const double f = step_function((sorted[i] - eocc) / thermal_sigma, max_thermal_range);
        if (f == 0.0) break;
        pop[order[i]] = weight(i) * f;
        sum += pop[order[i]];
      }
      if (std::fabs(sum - num_electrons) < kSmallThresh) break;
      if (sum < num_electrons) emin = eocc;
      else emax = eocc;
    }
  }
  // structuredElectronPopulation(state, k, spin) (valeCharge.F90:160-170)
  q = 0;
  for (int k = 0; k < nk; ++k)
    for (int s = 0; s < spin; ++s)
      for (int j = 0; j < num_states; ++j)
        occupation[j + (size_t)num_states * (k + (size_t)nk * s)] = pop[q++];
  if (occupied_energy) *occupied_energy = eocc;
  return OLC_OK;
}

}  // namespace olc
