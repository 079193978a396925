/* A plain C11 consumer of include/gturbo_gb.h, as a Fortran driver's
 * iso_c_binding interface sees the library: it prints the layout of the
 * public structs and the results of the host-only entry points as one JSON
 * object, which tests/test_c_consumer.py compares with the Python mirror and
 * the oracle.  Usage: c_consumer <params.dat path> */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

#include "gturbo_gb.h"

#define FIELD(T, f) printf("\"%s\": [%zu, %zu], ", #f, offsetof(T, f), sizeof(((T*)0)->f))

int main(int argc, char** argv) {
  printf("{\"gt_params\": {\"size\": %zu, ", sizeof(gt_params));
  FIELD(gt_params, nx); FIELD(gt_params, ny); FIELD(gt_params, nz);
  FIELD(gt_params, xlx); FIELD(gt_params, xly); FIELD(gt_params, xlz);
  FIELD(gt_params, nu); FIELD(gt_params, alpnu); FIELD(gt_params, mu); FIELD(gt_params, alpmu);
  FIELD(gt_params, dt); FIELD(gt_params, omega); FIELD(gt_params, rtrunc);
  FIELD(gt_params, truncate); FIELD(gt_params, famp); FIELD(gt_params, k1f); FIELD(gt_params, k2f);
  FIELD(gt_params, forcing); FIELD(gt_params, dt2_mode); FIELD(gt_params, precision);
  printf("\"device\": [%zu, %zu]}, ", offsetof(gt_params, device), sizeof(((gt_params*)0)->device));
  printf("\"gt_diag\": {\"size\": %zu, ", sizeof(gt_diag));
  FIELD(gt_diag, energy); FIELD(gt_diag, enstrophy); FIELD(gt_diag, helicity);
  FIELD(gt_diag, inpe); FIELD(gt_diag, inpz);
  printf("\"nonfinite\": [%zu, %zu]}, ", offsetof(gt_diag, nonfinite), sizeof(((gt_diag*)0)->nonfinite));

  gt_params p;
  int rc = gt_params_default(&p);
  printf("\"default_rc\": %d, \"default_nx\": %d, \"default_nu\": %.17g, ", rc, p.nx, p.nu);
  rc = gt_params_read(argc > 1 ? argv[1] : "", &p);
  printf("\"read_rc\": %d, \"read_nu\": %.17g, \"read_dt\": %.17g, \"read_omega\": %.17g, ", rc, p.nu,
         p.dt, p.omega);
  p.nx = p.ny = p.nz = 32;
  p.forcing = GT_FORCING_3D3C;
  p.famp = 0.05;
  printf("\"validate_rc\": %d, ", gt_params_validate(&p));
  size_t bytes = 0;
  rc = gt_memory_estimate(&p, &bytes);
  printf("\"estimate_rc\": %d, \"estimate_bytes\": %zu, ", rc, bytes);

  int32_t irand = 8299396;
  float r[5];
  rc = gt_rann(&irand, 5, r);
  printf("\"rann_rc\": %d, \"rann_state\": %d, \"rann\": [%.9g, %.9g, %.9g, %.9g, %.9g], ", rc, irand,
         (double)r[0], (double)r[1], (double)r[2], (double)r[3], (double)r[4]);

  int32_t nf = 0;
  int32_t* ix = malloc(sizeof(int32_t) * 2 * GT_NFORC);
  int32_t* iy = malloc(sizeof(int32_t) * 2 * GT_NFORC);
  int32_t* iz = malloc(sizeof(int32_t) * 2 * GT_NFORC);
  double* dF = malloc(sizeof(double) * 6 * 2 * GT_NFORC);
  double inpe = 0, inpz = 0;
  rc = gt_forced_modes(&p, &nf, ix, iy, iz, NULL, &inpe, &inpz);
  printf("\"modes_rc\": %d, \"nf\": %d, \"first_mode\": [%d, %d, %d], \"inpe\": %.17g, ", rc, nf, iz[0],
         iy[0], ix[0], inpe);
  int32_t seed = 8299396, n = 0;
  rc = gt_forcing_increments(&p, &seed, 2 * GT_NFORC, &n, ix, iy, iz, dF);
  double sum = 0;
  for (int e = 0; e < 6 * n; ++e) sum += dF[e];
  printf("\"incr_rc\": %d, \"n\": %d, \"seed_after\": %d, \"dF0\": [%.17g, %.17g], \"dF_sum\": %.17g, ", rc, n,
         seed, dF[0], dF[1], sum);

  p.nx = 12;   /* not a power of two */
  printf("\"bad_grid_rc\": %d, \"strerror_einval\": \"%s\"}\n", gt_params_validate(&p), gt_strerror(GT_EINVAL));
  free(ix);
  free(iy);
  free(iz);
  free(dF);
  return 0;
}
