/*
 * Drop-in driver: a libdft imaginary-time relaxation written against the
 * libgrid / libdft call signatures, linked against libdftgpu instead.
 *
 * Plain OT on a 64^3 periodic grid (step 1 bohr), a repulsive Gaussian
 * impurity 10 K exp(-r^2 / (2 * 3^2)) at the centre, initial state
 * sqrt(rho0) (1 - exp(-r^2 / (2 * 5^2))), predict-correct imaginary-time
 * steps of 10 fs with the particle number held at its initial value.
 * The loop body is the one libdft's examples use
 * (examples/imag_time/imag_time.c:231-239).  With "hd" the functional is the
 * one that example allocates, DFT_OT_PLAIN | DFT_OT_KC | DFT_OT_HD
 * (examples/imag_time/imag_time.c:204).
 *
 *   usage: imag_time [steps] [fp32|fp64] [hd]
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dftgpu.h"

#define NX 64
#define NY 64
#define NZ 64
#define STEP 1.0
#define TS 10.0   /* fs */

static REAL impurity(void *arg, REAL x, REAL y, REAL z) {
  (void) arg;
  return 10.0 / GRID_AUTOK * exp(-(x * x + y * y + z * z) / (2.0 * 3.0 * 3.0));
}

static REAL complex initial(void *arg, REAL x, REAL y, REAL z) {
  REAL rho0 = *(REAL *) arg;
  return sqrt(rho0) * (1.0 - exp(-(x * x + y * y + z * z) / (2.0 * 5.0 * 5.0)));
}

int main(int argc, char **argv) {
  int steps = argc > 1 ? atoi(argv[1]) : 200;
  int gpus[] = { 0 };
  cuda_enable(1, 1, gpus);
  if (argc > 2 && !strcmp(argv[2], "fp32")) dftgpu_set_precision(DFTGPU_FP32);

  wf *gwf = grid_wf_alloc(NX, NY, NZ, STEP, DFT_HELIUM_MASS, WF_PERIODIC_BOUNDARY, WF_2ND_ORDER_FFT, "gwf");
  if (!gwf) { fprintf(stderr, "grid_wf_alloc: %s\n", dftgpu_last_error_message()); return 1; }
  wf *gwfp = grid_wf_clone(gwf, "gwfp");
  const INT model = (argc > 3 && !strcmp(argv[3], "hd")) ? (DFT_OT_PLAIN | DFT_OT_KC | DFT_OT_HD) : DFT_OT_PLAIN;
  dft_ot_functional *otf = dft_ot_alloc(model, gwf, DFT_MIN_SUBSTEPS, DFT_MAX_SUBSTEPS);
  if (!otf) { fprintf(stderr, "dft_ot_alloc: %s\n", dftgpu_last_error_message()); return 1; }
  REAL rho0 = dft_ot_bulk_density_pressurized(otf, 0.0);
  REAL mu0 = dft_ot_bulk_chempot_pressurized(otf, 0.0);
  printf("mu0 = %.6f K/atom, rho0 = %.6f Angs^-3\n", mu0 * GRID_AUTOK, rho0 / (GRID_AUTOANG * GRID_AUTOANG * GRID_AUTOANG));

  rgrid *ext_pot = rgrid_clone(otf->density, "ext_pot");
  cgrid *potential_store = cgrid_clone(gwf->grid, "potential_store");
  rgrid_map(ext_pot, impurity, NULL);
  grid_wf_map(gwf, initial, &rho0);
  gwf->norm = grid_wf_norm(gwf);

  for (int iter = 0; iter < steps; iter++) {
    grid_real_to_complex_re(potential_store, ext_pot);
    dft_ot_potential(otf, potential_store, gwf);
    cgrid_add(potential_store, -mu0);
    grid_wf_propagate_predict(gwf, gwfp, potential_store, -I * TS / GRID_AUTOFS);
    grid_add_real_to_complex_re(potential_store, ext_pot);
    dft_ot_potential(otf, potential_store, gwfp);
    cgrid_add(potential_store, -mu0);
    cgrid_multiply(potential_store, 0.5);
    grid_wf_propagate_correct(gwf, potential_store, -I * TS / GRID_AUTOFS);
    grid_wf_normalize(gwf);
  }
  double energy, natoms, mu;
  if (dftgpu_energy_report(otf, gwf, ext_pot, &energy, &natoms, &mu)) {
    fprintf(stderr, "energy report: %s\n", dftgpu_last_error_message());
    return 1;
  }
  printf("steps %d  N = %.10f  E = %.10e K  E/N = %.10f K  mu = %.10f K\n", steps, natoms, energy * GRID_AUTOK,
         energy / natoms * GRID_AUTOK, mu * GRID_AUTOK);
  int err = dftgpu_last_error();
  dft_ot_free(otf);
  rgrid_free(ext_pot);
  cgrid_free(potential_store);
  grid_wf_free(gwfp);
  grid_wf_free(gwf);
  return err ? 1 : 0;
}
