/* A C99 caller of include/awigner.h: the header compiles as plain C and the library is usable
 * without Python.  Runs on a machine without a GPU (aw_check_config makes no CUDA runtime call):
 * a harmonic Wigner-Moyal configuration with the Ehrenfest observables is checked, then the same
 * configuration with an expression that does not compile, with observable terms outside their
 * history row or without an expression, and with a grid that is too small.
 * Prints one line per check and exits non-zero on the first unexpected status. */
#include <stdio.h>
#include <string.h>

#include "awigner.h"

static int expect(const char* what, int got, int want) {
  printf("%s: %d%s%s\n", what, got, got ? " " : "", got ? aw_last_error() : "");
  if (got != want) {
    printf("unexpected status for %s (wanted %d)\n", what, want);
    return 1;
  }
  return 0;
}

int main(void) {
  const int n = 64;
  const double xa = 6.0, pa = 6.0;
  aw_config c;
  memset(&c, 0, sizeof c);
  c.kind = AW_WIGNER_MOYAL;
  c.precision = AW_C128;
  c.x_grid_dim = n;
  c.p_grid_dim = n;
  c.dX = 2.0 * xa / n;
  c.dP = 2.0 * pa / n;
  c.dt = 0.01;
  c.dXdP = c.dX * c.dP;
  c.cuda_consts = "#define X_gridDIM 64\n#define omega 1.000000000000000e+00\n";
  c.V = "0.5 * omega * omega * X * X";
  c.K = "0.5 * P * P";
  /* Ehrenfest slots of wigner_moyal_cuda_1d.py:584-606: <X>, <diff_K>, <P>, -<diff_V>, <K> + <V> */
  const char* obs_x[] = {"X", "omega * omega * X", "0.5 * omega * omega * X * X"};
  const char* obs_p[] = {"P", "0.5 * P * P"};
  const int32_t slot[] = {0, 1, 2, 3, 4, 4};
  const int32_t kind[] = {AW_TERM_X, AW_TERM_P, AW_TERM_P, AW_TERM_X, AW_TERM_P, AW_TERM_X};
  const int32_t index[] = {0, 0, 0, 1, 1, 2};
  const double coef[] = {1.0, 1.0, 1.0, -1.0, 1.0, 1.0};
  c.ehrenfest = 1;
  c.n_obs_x = 3;
  c.obs_x = obs_x;
  c.n_obs_p = 2;
  c.obs_p = obs_p;
  c.n_terms = 6;
  c.term_slot = slot;
  c.term_kind = kind;
  c.term_index = index;
  c.term_coef = coef;
  c.n_slots = 5;

  int bad = 0;
  printf("aw_version: %d\n", aw_version());
  bad |= expect("valid configuration", aw_check_config(&c, "sm_103a"), AW_OK);
  c.V = "0.5 * omega * omega * X * X + no_such_name";
  bad |= expect("undefined name in V", aw_check_config(&c, NULL), AW_E_JIT);
  c.V = "0.5 * omega * omega * X * X";
  const int32_t slot_out[] = {0, 1, 2, 3, 4, 5};
  c.term_slot = slot_out;
  bad |= expect("term slot outside the row", aw_check_config(&c, NULL), AW_E_ARG);
  c.term_slot = slot;
  const int32_t index_out[] = {0, 0, 0, 1, 2, 2};
  c.term_index = index_out;
  bad |= expect("term without an expression", aw_check_config(&c, NULL), AW_E_ARG);
  c.term_index = index;
  c.x_grid_dim = 16;
  bad |= expect("16-point grid", aw_check_config(&c, NULL), AW_E_ARG);
  bad |= expect("null configuration", aw_check_config(NULL, NULL), AW_E_ARG);
  return bad;
}
