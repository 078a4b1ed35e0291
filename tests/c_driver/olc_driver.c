/* Plain-C driver of the libolcao_gb300 C-ABI (include/olcao_gpu.h): what a C or
 * Fortran host sees, without Python in between.
 *
 *   olc_driver host   host-only entries: version, argument refusal with the
 *                     error text, populateStates on a two-k insulator
 *   olc_driver gpu    additionally one primitive batch on the device: the s-s
 *                     overlap of two Gaussians against its closed form
 *                     (pi / (a1 + a2))^(3/2) exp(-a1 a2 / (a1 + a2) |A - B|^2)
 *
 * Exit status 0 when every check holds. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "olcao_gpu.h"

static int failures = 0;

static void check(int ok, const char* what) {
  printf("%-58s %s\n", what, ok ? "ok" : "FAILED");
  if (!ok) ++failures;
}

int main(int argc, char** argv) {
  const int gpu = argc > 1 && strcmp(argv[1], "gpu") == 0;
  char msg[256];
  check(olc_version() != NULL && strlen(olc_version()) > 0, "olc_version");

  /* a null system is refused with OLC_ERR_ARG and a message */
  olc_context_t* ctx = NULL;
  const int st = olc_create(NULL, NULL, &ctx);
  olc_last_error(msg, sizeof msg);
  check(st == OLC_ERR_ARG && ctx == NULL && strlen(msg) > 0, "olc_create(NULL) refused");

  /* populateStates: 3 states, 2 k-points (weights 1, spin 1), 2 electrons
   * per k-weight unit: the lowest state of each k is filled (1 each), the
   * highest occupied energy is the larger of the two lowest eigenvalues */
  const double eig[6] = {-0.5, 0.1, 0.3, -0.4, 0.2, 0.4};
  const double w[2] = {1.0, 1.0};
  double occ[6], ef = 0.0;
  int sp = olc_populate_states(3, 2, 1, eig, w, 2.0, 0.0, 0.1, 10.0, occ, &ef);
  check(sp == OLC_OK && fabs(occ[0] - 1.0) < 1e-14 && fabs(occ[3] - 1.0) < 1e-14 &&
            fabs(occ[1]) < 1e-14 && fabs(occ[4]) < 1e-14 && fabs(ef + 0.4) < 1e-14,
        "olc_populate_states (insulator, 2 k)");
  /* too few states for the electrons */
  sp = olc_populate_states(3, 2, 1, eig, w, 100.0, 0.0, 0.1, 10.0, occ, &ef);
  check(sp == OLC_ERR_ARG, "olc_populate_states refuses 100 electrons");

  if (gpu) {
    /* s-s overlap primitive, three separations */
    double in[36] = {0}, out[3 * 256];
    int32_t lm[6] = {1, 1, 1, 1, 1, 1};
    const double a1 = 0.7, a2 = 2.3, d[3] = {0.0, 0.8, 2.5};
    for (int q = 0; q < 3; ++q) {
      in[12 * q + 0] = a1;
      in[12 * q + 1] = a2;
      in[12 * q + 6] = d[q];      /* B = (d, 0, 0), A = 0 */
    }
    const int pr = olc_primitive_batch(1, 3, in, lm, out);
    double worst = 0.0;
    for (int q = 0; q < 3; ++q) {
      const double z = a1 + a2;
      const double ref = pow(3.14159265358979323846 / z, 1.5) * exp(-a1 * a2 / z * d[q] * d[q]);
      worst = fmax(worst, fabs(out[256 * q] - ref) / ref);
    }
    check(pr == OLC_OK && worst < 1e-14, "olc_primitive_batch s-s overlap on the GPU");
  }
  printf("%d failure(s)\n", failures);
  return failures ? 1 : 0;
}
