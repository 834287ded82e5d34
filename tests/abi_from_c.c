/* abi_from_c.c -- test helper: the C ABI compiled as C99 and called from C.  Uses only host
 * entry points (no device): the Förster-form table, the chirality labeller in its neutral case,
 * and the device-less context creation.  Prints "ok" and exits 0 on success. */
#include <math.h>
#include <stdio.h>

#include "cntkmc.h"

int main(void) {
  double dist_spec[3] = {0.5e-9, 10e-9, 20}, theta_spec[3] = {0.0, 90.0, 7};
  double dist[20], theta[7], rate[20 * 7];
  if (kmc_forster2d_table(1e15, dist_spec, theta_spec, dist, theta, rate) != KMC_OK) return 1;
  /* the labeller with equal chiralities, no floor and no near field is the same table */
  double e = 0.0, d = 1.0;
  kmc_species_model m = {1, 1e15, &e, &d, 1.0, 1.0, 1.0, 0.0, 0.0};
  double dd[20 * 7], tt[20 * 7], r[20 * 7];
  int32_t z[20 * 7];
  for (int i = 0; i < 20; ++i)
    for (int k = 0; k < 7; ++k) {
      dd[i * 7 + k] = dist[i];
      tt[i * 7 + k] = theta[k];
      z[i * 7 + k] = 0;
    }
  if (kmc_species_rates(&m, 20 * 7, dd, tt, z, z, r) != KMC_OK) return 2;
  for (int i = 0; i < 20 * 7; ++i)
    if (r[i] != rate[i]) return 3;
  /* bad arguments are refused with a status, not a crash */
  int32_t bad = 5;
  if (kmc_species_rates(&m, 1, dd, tt, &bad, z, r) != KMC_ERR_ARG) return 4;
  if (KMC_MLP_PARAMS(4) != 4580) return 5;
  int st = 0;
  kmc_ctx* c = kmc_create(0, &st);
  if (c) kmc_destroy(c); /* a device is present: nothing more to check here */
  else if (st != KMC_ERR_NO_DEVICE) return 6;
  printf("ok %s\n", kmc_version());
  return 0;
}
