/* A plain C99 client of include/hqcgb.h, built and run by
 * tests/test_cpu_library.py: the header compiles as C and the library links
 * and answers through the C ABI alone, with no Python and no torch.  Only
 * entry points that need no GPU are called (argument validation, the
 * error-message channel, the host-side DIIS solve and tile plan). */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "hqcgb.h"

static int fail(const char *what) {
  fprintf(stderr, "c_client: %s\n", what);
  return 1;
}

int main(void) {
  /* a plan with no atoms is rejected before any device call */
  hqcgb_params P;
  memset(&P, 0, sizeof(P));
  hqcgb_plan *plan = NULL;
  if (hqcgb_plan_create(&P, &plan) != HQCGB_BAD_ARG) return fail("plan_create accepted n_atoms = 0");
  if (!strstr(hqcgb_last_error(), "n_atoms")) return fail("last_error does not name the bad field");

  /* DIIS on a 2-vector history with B = diag(1, 4): c = (0.8, 0.2) up to the
   * eta regularisation (B stored as interleaved complex) */
  double B[8] = {1, 0, 0, 0, 0, 0, 4, 0}, c[4];
  if (hqcgb_diis_coefficients(2, B, c) != HQCGB_OK) return fail("diis_coefficients failed");
  if (fabs(c[0] - 0.8) > 1e-9 || fabs(c[2] - 0.2) > 1e-9 || fabs(c[1]) > 1e-12 || fabs(c[3]) > 1e-12)
    return fail("diis coefficients wrong");

  /* the quadrature tile plan of 270 AOs (2 full blocks + 14), symmetric: the
   * persistent form, 3 full tiles + (0, last), (1, last) and the corner in
   * one launch */
  int tiles[64 * 7], count = 0, launches = 0;
  if (hqcgb_tc_quad_tiles(270, 1, 64, tiles, &count, &launches) != HQCGB_OK) return fail("tile plan failed");
  if (count != 6 || launches != 1) return fail("unexpected tile plan for 270 AOs");

  printf("c_client ok\n");
  return 0;
}
