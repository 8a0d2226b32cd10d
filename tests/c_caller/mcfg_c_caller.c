/*
 * mcfg_c_caller.c -- a plain C99 caller of the C-ABI (include/mcfg.h), the
 * way MCF's iso_c_binding module or any other host code binds it: fill
 * mcfg_params, create a handle, upload MCF-layout arrays, step with the
 * state in host arrays, read the statistics, destroy.  Every status is
 * checked (MCF's stat_info convention); on an error the routine and the
 * library's message go to stderr and the program exits with status 2.
 *
 * usage: mcfg_c_caller OUT N_SIDE STEPS PRECISION REUSE
 *   a periodic N_SIDE^3 lattice (dx = 1, jittered by a 64-bit LCG that the
 *   Python test reproduces), C2's physics (quintic rc = 3, Hu-Adams, Morris
 *   EOS with gamma 1, c = 10, eta = 1, kT = 1e-3, Wiener noise), dt = 1e-3;
 *   OUT receives n, then x[n*3], v[n*3] (doubles) and ke, momentum[3].
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mcfg.h"

static uint64_t lcg_state = 20261203u;

/* uniform in [0, 1) from the top 53 bits of Knuth's MMIX LCG */
static double lcg_uniform(void) {
  lcg_state = lcg_state * 6364136223846793005ull + 1442695040888963407ull;
  return (double)(lcg_state >> 11) * (1.0 / 9007199254740992.0);
}

static void fail(const char* routine, const char* msg) {
  fprintf(stderr, "mcfg error: %s: %s\n", routine, msg ? msg : "(no message)");
  exit(2);
}

#define CHECK(h, call, routine)                                \
  do {                                                         \
    if ((call) != MCFG_OK) fail(routine, mcfg_last_error(h)); \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s OUT N_SIDE STEPS PRECISION REUSE\n", argv[0]);
    return 1;
  }
  const char* out_path = argv[1];
  const int ns = atoi(argv[2]), steps = atoi(argv[3]);
  const int precision = atoi(argv[4]), reuse = atoi(argv[5]);
  if (ns < 9 || steps < 1) {
    fprintf(stderr, "N_SIDE >= 9 and STEPS >= 1\n");
    return 1;
  }
  if (mcfg_sizeof_params() != (int64_t)sizeof(mcfg_params)) {
    fprintf(stderr, "mcfg_params layout differs from the library's\n");
    return 1;
  }

  mcfg_params p;
  memset(&p, 0, sizeof p);
  p.num_dim = 3;
  for (int f = 0; f < 6; ++f) p.bcdef[f] = MCFG_BC_PERIODIC;
  for (int a = 0; a < 3; ++a) {
    p.min_phys[a] = p.min_phys_t[a] = 0.0;
    p.max_phys[a] = p.max_phys_t[a] = (double)ns;
  }
  p.cut_off = 3.0;
  p.cell_factor = 1.0001;
  p.kernel_type = 1;
  p.rhs_density_type = 2;
  p.rhs_force_type = 3;
  p.stateEquation_type = 1;
  p.c = 10.0;
  p.rho = 1.0;
  p.rho_ref = 1.0;
  p.gamma = 1.0;
  p.eta = 1.0;
  p.eta_coef = 1.0;
  p.kt = 1e-3;
  p.dt = 1e-3;
  p.Brownian = 1;
  p.symmetry = 1;
  p.wall_noslip_type = 2;
  p.init_density = 1.0;
  p.Newtonian = 1;
  p.precision = precision;
  p.seed = 42;
  p.device = 0;
  p.reserved[1] = reuse;

  const int64_t n = (int64_t)ns * ns * ns;
  double* x = malloc(sizeof(double) * 3 * (size_t)n);
  double* v = malloc(sizeof(double) * 3 * (size_t)n);
  double* m = malloc(sizeof(double) * (size_t)n);
  int32_t* id = malloc(sizeof(int32_t) * 2 * (size_t)n);
  if (!x || !v || !m || !id) {
    fprintf(stderr, "out of host memory\n");
    return 1;
  }
  int64_t q = 0;
  for (int i = 0; i < ns; ++i)
    for (int j = 0; j < ns; ++j)
      for (int k = 0; k < ns; ++k, ++q) {
        const double c[3] = {i + 0.5, j + 0.5, k + 0.5};
        for (int a = 0; a < 3; ++a) {
          x[3 * q + a] = c[a] + 0.1 * (lcg_uniform() - 0.5);
          v[3 * q + a] = 0.02 * (lcg_uniform() - 0.5);
        }
        m[q] = 1.0; /* number density: m = rho dx^3 */
        id[2 * q] = (int32_t)(q + 1);
        id[2 * q + 1] = 0;
      }

  mcfg_handle* h = NULL;
  if (mcfg_create(&p, &h) != MCFG_OK) fail("mcfg_create", mcfg_create_error());
  CHECK(h, mcfg_upload(h, n, x, v, m, id, NULL), "mcfg_upload");
  CHECK(h, mcfg_init_force(h, 0), "mcfg_init_force");
  for (int s = 1; s <= steps; ++s)
    CHECK(h, mcfg_step_vv_host(h, s, p.dt, x, v), "mcfg_step_vv_host");
  double ke = 0.0, mom[3] = {0, 0, 0};
  CHECK(h, mcfg_statistics(h, &ke, mom, NULL), "mcfg_statistics");
  CHECK(h, mcfg_destroy(h), "mcfg_destroy");

  FILE* fo = fopen(out_path, "wb");
  if (!fo) {
    fprintf(stderr, "cannot open %s\n", out_path);
    return 1;
  }
  const size_t nd = 3 * (size_t)n;
  const int ok = fwrite(&n, sizeof n, 1, fo) == 1 && fwrite(x, sizeof(double), nd, fo) == nd &&
                 fwrite(v, sizeof(double), nd, fo) == nd && fwrite(&ke, sizeof ke, 1, fo) == 1 &&
                 fwrite(mom, sizeof(double), 3, fo) == 3;
  fclose(fo);
  free(x);
  free(v);
  free(m);
  free(id);
  if (!ok) {
    fprintf(stderr, "write failed\n");
    return 1;
  }
  printf("ok n=%lld ke=%.17g\n", (long long)n, ke);
  return 0;
}
