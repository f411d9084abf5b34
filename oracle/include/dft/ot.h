/*
 * CPU oracle: restatement of libdft's Orsay-Trento interface (FP64).
 * TEST INFRASTRUCTURE ONLY.
 *
 * The model bit flags, the functional structure's public field names and the
 * exported function names are kept identical to libdft (src/ot.h:37-202,
 * src/dft.h:18-56) because they are the interface under test; the code
 * behind them (oracle/ot_port.c) is this project's own.
 */
#ifndef ORACLE_DFT_OT_H
#define ORACLE_DFT_OT_H

#include "grid/grid.h"
#include "grid/au.h"

/* Model flags (src/ot.h:37-60). */
#define DFT_OT_PLAIN    0
#define DFT_OT_KC       1
#define DFT_OT_HD       2
#define DFT_OT_HD2      4
#define DFT_OT_BACKFLOW 8
#define DFT_OT_T0MK    16
#define DFT_OT_T400MK  32
#define DFT_OT_T600MK  64
#define DFT_OT_T800MK  128
#define DFT_OT_T1200MK 256
#define DFT_OT_T1400MK 512
#define DFT_OT_T1600MK 1024
#define DFT_OT_T1800MK 2048
#define DFT_OT_T2000MK 4096
#define DFT_OT_T2100MK 8192
#define DFT_OT_T2200MK 16384
#define DFT_OT_T2400MK 32768
#define DFT_OT_T2600MK 65536
#define DFT_OT_T2800MK 131072
#define DFT_OT_T3000MK 262144
#define DFT_GP         524288
#define DFT_DR         1048576
#define DFT_ZERO       2097152
#define DFT_GP2        4194304

/* Models the oracle restates: the OT functional (0 K and the thermal
 * parameter sets with their ideal Bose gas term) with optional KC, BF and the
 * high-density terms (HD, HD2). */
#define ORACLE_THERMAL_MODELS (DFT_OT_T0MK | DFT_OT_T400MK | DFT_OT_T600MK | DFT_OT_T800MK | DFT_OT_T1200MK | \
                               DFT_OT_T1400MK | DFT_OT_T1600MK | DFT_OT_T1800MK | DFT_OT_T2000MK | DFT_OT_T2100MK | \
                               DFT_OT_T2200MK | DFT_OT_T2400MK | DFT_OT_T2600MK | DFT_OT_T2800MK | DFT_OT_T3000MK)
#define ORACLE_SUPPORTED_MODELS (DFT_OT_KC | DFT_OT_HD | DFT_OT_HD2 | DFT_OT_BACKFLOW | ORACLE_THERMAL_MODELS)

#define DFT_HELIUM_MASS (4.002602 / GRID_AUTOAMU)
#define DFT_MIN_SUBSTEPS 4
#define DFT_MAX_SUBSTEPS 32
#define DFT_EPS 1E-4

typedef struct lj_struct {
  REAL h, sigma, epsilon, cval;
} dft_common_lj;

typedef struct bf_struct {
  REAL g11, g12, g21, g22, a1, a2;
} dft_ot_bf;

typedef struct {
  REAL kx, ky, kz;
  REAL a;
  REAL rho;
} dft_plane_wave;

typedef struct dft_ot_functional_struct {
  INT model;
  REAL b, c2, c2_exp, c3, c3_exp, c4;
  REAL rho_0s, alpha_s, l_g, mass, rho0, temp;
  dft_common_lj lj_params;
  dft_ot_bf bf_params;
  rgrid *lennard_jones, *spherical_avg;
  rgrid *gaussian_tf, *gaussian_x_tf, *gaussian_y_tf, *gaussian_z_tf;
  rgrid *backflow_pot;
  REAL beta, rhom, C, mu0, xi, rhobf;
  REAL div_epsilon, max_veloc, max_bfpot, c_bfpot;
  rgrid *workspace1, *workspace2, *workspace3, *workspace4, *workspace5;
  rgrid *workspace6, *workspace7, *workspace8, *workspace9;
  rgrid *density;
} dft_ot_functional;

/* kernel shape functions (src/common.c:53-200, src/ot-private.h:10-21) */
REAL dft_common_lj_func(REAL r2, REAL sig, REAL eps);
REAL dft_common_lennard_jones(void *arg, REAL x, REAL y, REAL z);
REAL dft_common_spherical_avg(void *arg, REAL x, REAL y, REAL z);
REAL dft_common_gaussian(void *arg, REAL x, REAL y, REAL z);
REAL dft_ot_backflow_pot(void *arg, REAL x, REAL y, REAL z);
REAL complex dft_common_planewave(void *arg, REAL x, REAL y, REAL z);

/* functional (src/ot.c, src/ot-energy.c) */
void dft_ot_init_params(dft_ot_functional *otf, INT model);
dft_ot_functional *dft_ot_alloc(INT model, wf *gwf, INT min_substeps, INT max_substeps);
void dft_ot_free(dft_ot_functional *otf);
void dft_ot_potential(dft_ot_functional *otf, cgrid *potential, wf *gwf);
void dft_ot_energy_density(dft_ot_functional *otf, rgrid *energy_density, wf *gwf);

/* bulk (src/helium-ot-bulk.c) */
REAL dft_ot_bulk_energy(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_dEdRho(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_pressure(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_dPdRho(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_density_pressurized(dft_ot_functional *otf, REAL pressure);
REAL dft_ot_bulk_chempot_pressurized(dft_ot_functional *otf, REAL pressure);
REAL dft_ot_bulk_density(dft_ot_functional *otf);
REAL dft_ot_bulk_chempot(dft_ot_functional *otf);
REAL dft_ot_bulk_chempot2(dft_ot_functional *otf);
REAL dft_ot_bulk_compressibility(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_sound_speed(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_dispersion(dft_ot_functional *otf, REAL *k, REAL rho0);

#endif
