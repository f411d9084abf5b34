/*
 * Drop-in driver: a bubble held fixed on the grid while the liquid flows past
 * it (moving background), written against the libgrid / libdft call
 * signatures and linked against libdftgpu.  The loop follows libdft's
 * gas-bubble example (examples/gas-bubble/bubble.c:104-206): the background
 * momentum k0 = m v / hbar is set on both wave functions with
 * cgrid_set_momentum, the velocity rounded to a multiple of 2 pi hbar /
 * (m NZ STEP) so that the boosted state is periodic; warm-up imaginary-time
 * predict-correct steps with the chemical potential in the external
 * potential; then real-time steps with a small imaginary part of the time
 * step (the example's FFT_STAB).
 *
 * Plain OT on a 64 x 64 x 128 grid (step 2 bohr); the bubble is a repulsive
 * Gaussian of 500 K and width 6 bohr at the centre (this driver's choice);
 * background velocity 50 m/s along z.
 *
 *   usage: moving_bubble [warmup_steps] [real_steps] [fp32]
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dftgpu.h"

#define NX 64
#define NY 64
#define NZ 128
#define STEP 2.0
#define TS 5.0            /* fs */
#define FFT_STAB 0.005    /* fraction of imaginary time in the real-time steps */
#define VZ (50.0 / GRID_AUTOMPS)

static REAL bubble(void *arg, REAL x, REAL y, REAL z) {
  REAL mu0 = *(REAL *) arg;
  return 500.0 / GRID_AUTOK * exp(-(x * x + y * y + z * z) / (2.0 * 6.0 * 6.0)) - mu0;
}

/* nearest velocity whose momentum m v / hbar is a reciprocal-grid vector along z */
static REAL round_veloc(REAL v) {
  REAL q = 2.0 * M_PI / (DFT_HELIUM_MASS * NZ * STEP);   /* hbar = 1 */
  return q * floor(v / q + 0.5);
}

int main(int argc, char **argv) {
  int warm = argc > 1 ? atoi(argv[1]) : 100, steps = argc > 2 ? atoi(argv[2]) : 100;
  int gpus[] = { 0 };
  cuda_enable(1, 1, gpus);
  if (argc > 3 && !strcmp(argv[3], "fp32")) dftgpu_set_precision(DFTGPU_FP32);

  wf *gwf = grid_wf_alloc(NX, NY, NZ, STEP, DFT_HELIUM_MASS, WF_PERIODIC_BOUNDARY, WF_2ND_ORDER_FFT, "gwf");
  if (!gwf) { fprintf(stderr, "grid_wf_alloc: %s\n", dftgpu_last_error_message()); return 1; }
  wf *gwfp = grid_wf_clone(gwf, "gwfp");
  cgrid *cworkspace = cgrid_clone(gwf->grid, "cworkspace");
  dft_ot_functional *otf = dft_ot_alloc(DFT_OT_PLAIN, gwf, DFT_MIN_SUBSTEPS, DFT_MAX_SUBSTEPS);
  if (!otf) { fprintf(stderr, "dft_ot_alloc: %s\n", dftgpu_last_error_message()); return 1; }
  REAL rho0 = dft_ot_bulk_density_pressurized(otf, 0.0);
  REAL mu0 = dft_ot_bulk_chempot_pressurized(otf, 0.0);
  rgrid *ext_pot = rgrid_clone(otf->density, "ext_pot");
  rgrid_map(ext_pot, bubble, &mu0);                  /* external potential - mu0 */

  REAL vz = round_veloc(VZ), kz = DFT_HELIUM_MASS * vz;
  printf("background velocity %.3f m/s, kz = %.6e bohr^-1\n", vz * GRID_AUTOMPS, kz);
  cgrid_set_momentum(gwf->grid, 0.0, 0.0, kz);
  cgrid_set_momentum(gwfp->grid, 0.0, 0.0, kz);
  grid_wf_constant(gwf, sqrt(rho0));

  for (int iter = 0; iter < warm + steps; iter++) {
    REAL complex dt = iter < warm ? -I * TS / GRID_AUTOFS : TS / GRID_AUTOFS - I * FFT_STAB * TS / GRID_AUTOFS;
    grid_real_to_complex_re(cworkspace, ext_pot);
    dft_ot_potential(otf, cworkspace, gwf);
    grid_wf_propagate_predict(gwf, gwfp, cworkspace, dt);
    grid_add_real_to_complex_re(cworkspace, ext_pot);
    dft_ot_potential(otf, cworkspace, gwfp);
    cgrid_multiply(cworkspace, 0.5);
    grid_wf_propagate_correct(gwf, cworkspace, dt);
  }
  double energy, natoms, mu;
  if (dftgpu_energy_report(otf, gwf, ext_pot, &energy, &natoms, &mu)) {
    fprintf(stderr, "energy report: %s\n", dftgpu_last_error_message());
    return 1;
  }
  printf("warm-up %d + real-time %d steps  N = %.6f  E = %.6e K  kinetic (moving frame) = %.6e K\n", warm, steps,
         natoms, energy * GRID_AUTOK, grid_wf_kinetic_energy(gwf) * GRID_AUTOK);
  int err = dftgpu_last_error();
  dft_ot_free(otf);
  rgrid_free(ext_pot);
  cgrid_free(cworkspace);
  grid_wf_free(gwfp);
  grid_wf_free(gwf);
  return err ? 1 : 0;
}
