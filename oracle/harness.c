/*
 * CPU oracle: flat C entry points for the Python test harness (ctypes).
 * TEST INFRASTRUCTURE ONLY.
 *
 * The same source is compiled twice: into liboracle.so against the oracle's
 * own restatement (oracle/ot_port.c) and, when the reference tree is present,
 * into _ref/libdft_ref.so against libdft's unmodified src/ot.c, ot-energy.c,
 * common.c and helium-ot-bulk.c (-DORACLE_REF).  Both libraries link the same
 * libgrid-subset restatement (oracle/grid_shim.c), so the two can be compared
 * call for call.  Buffers crossing this boundary are contiguous FP64 arrays in
 * [x][y][z] order (complex values interleaved re, im).
 */
#include <string.h>
#include "grid/grid.h"
#include "grid/au.h"
#ifdef ORACLE_REF
#include "dft.h"
#include "ot.h"
#else
#include "dft/ot.h"
#endif

int orc_kind(void) {
#ifdef ORACLE_REF
  return 2;
#else
  return 1;
#endif
}

int orc_sizeof_real(void) { return (int) sizeof(REAL); }

/* ---------------- grids ---------------- */

wf *orc_wf_new(long nx, long ny, long nz, double step, double mass) {
  return grid_wf_alloc(nx, ny, nz, step, mass, WF_PERIODIC_BOUNDARY, WF_2ND_ORDER_FFT, "oracle wf");
}
void orc_wf_free(wf *g) { grid_wf_free(g); }
cgrid *orc_wf_grid(wf *g) { return g->grid; }
void orc_wf_set_norm(wf *g, double n) { g->norm = n; }
double orc_wf_norm(wf *g) { return grid_wf_norm(g); }
double orc_wf_normalize(wf *g) { return grid_wf_normalize(g); }
double orc_wf_kinetic_energy(wf *g) { return grid_wf_energy(g, NULL); }
void orc_wf_density(wf *g, rgrid *d) { grid_wf_density(g, d); }
void orc_wf_velocity(wf *g, rgrid *vx, rgrid *vy, rgrid *vz, double eps) { grid_wf_velocity(g, vx, vy, vz, eps); }
void orc_wf_set_momentum(wf *g, double kx0, double ky0, double kz0) { cgrid_set_momentum(g->grid, kx0, ky0, kz0); }
void orc_wf_set_propagator(wf *g, int propagator) { g->propagator = (char) propagator; }
void orc_wf_boundary(wf *g, wf *gp, double amp, double rho0, long lx, long hx, long ly, long hy, long lz, long hz) {
  grid_wf_boundary(g, gp, amp, rho0, lx, hx, ly, hy, lz, hz);
}
void orc_wf_absorb_potential(wf *g, cgrid *pot, double amp, double rho0) { grid_wf_absorb_potential(g, pot, amp, rho0); }

cgrid *orc_cgrid_new(long nx, long ny, long nz, double step) {
  return cgrid_alloc(nx, ny, nz, step, CGRID_PERIODIC_BOUNDARY, NULL, "oracle cgrid");
}
void orc_cgrid_free(cgrid *g) { cgrid_free(g); }

void orc_cgrid_set(cgrid *g, const double *buf) {
  memcpy(g->value, buf, sizeof(REAL complex) * (size_t) (g->nx * g->ny * g->nz));
}
void orc_cgrid_get(cgrid *g, double *buf) {
  memcpy(buf, g->value, sizeof(REAL complex) * (size_t) (g->nx * g->ny * g->nz));
}

rgrid *orc_rgrid_new(long nx, long ny, long nz, double step) {
  return rgrid_alloc(nx, ny, nz, step, RGRID_PERIODIC_BOUNDARY, NULL, "oracle rgrid");
}
void orc_rgrid_free(rgrid *g) { rgrid_free(g); }

void orc_rgrid_set(rgrid *g, const double *buf) {
  for (INT ij = 0; ij < g->nx * g->ny; ij++)
    memcpy(g->value + ij * g->nz2, buf + ij * g->nz, sizeof(REAL) * (size_t) g->nz);
}
void orc_rgrid_get(rgrid *g, double *buf) {
  for (INT ij = 0; ij < g->nx * g->ny; ij++)
    memcpy(buf + ij * g->nz, g->value + ij * g->nz2, sizeof(REAL) * (size_t) g->nz);
}
/* half spectrum (nx * ny * (nz/2+1) complex) of a transformed rgrid */
void orc_rgrid_get_spectrum(rgrid *g, double *buf) {
  memcpy(buf, g->value, sizeof(REAL complex) * (size_t) (g->nx * g->ny * (g->nz / 2 + 1)));
}
double orc_rgrid_integral(rgrid *g) { return rgrid_integral(g); }
void orc_rgrid_fft(rgrid *g) { rgrid_fft(g); }
void orc_rgrid_inverse_fft_norm(rgrid *g) { rgrid_inverse_fft_norm(g); }
void orc_cgrid_fft(cgrid *g) { cgrid_fft(g); }
void orc_cgrid_inverse_fft_norm(cgrid *g) { cgrid_inverse_fft_norm(g); }
void orc_fft1d(double *data, long n, int sign) { oracle_fft1d((REAL complex *) data, n, 1, sign); }

/* ---------------- functional ---------------- */

/* Allocate the functional; lg_bohr > 0 replaces the KC Gaussian width and
 * regenerates the F and dF kernels the way src/ot.c:184-200 builds them. */
dft_ot_functional *orc_ot_new(long model, wf *gwf, long min_ns, long max_ns, double lg_bohr) {
  dft_ot_functional *otf = dft_ot_alloc(model, gwf, min_ns, max_ns);
  if (!otf) return NULL;
  if (lg_bohr > 0.0 && (model & DFT_OT_KC) && lg_bohr != otf->l_g) {
    REAL iw = 1.0 / lg_bohr;
    otf->l_g = lg_bohr;
    rgrid_adaptive_map(otf->gaussian_tf, dft_common_gaussian, &iw, min_ns, max_ns, 0.01 / GRID_AUTOK);
    rgrid_gradient(otf->gaussian_tf, otf->gaussian_x_tf, otf->gaussian_y_tf, otf->gaussian_z_tf);
    rgrid_fft(otf->gaussian_x_tf);
    rgrid_fft(otf->gaussian_y_tf);
    rgrid_fft(otf->gaussian_z_tf);
    rgrid_fft(otf->gaussian_tf);
  }
  return otf;
}
void orc_ot_free(dft_ot_functional *otf) { dft_ot_free(otf); }

/* parameter vector, fixed order:
 * b c2 c2_exp c3 c3_exp rho0 h sigma epsilon rho_0s alpha_s l_g mass
 * g11 g12 g21 g22 a1 a2 div_epsilon max_veloc max_bfpot c_bfpot */
int orc_ot_params(dft_ot_functional *o, double *out) {
  double v[] = { o->b, o->c2, o->c2_exp, o->c3, o->c3_exp, o->rho0, o->lj_params.h, o->lj_params.sigma,
                 o->lj_params.epsilon, o->rho_0s, o->alpha_s, o->l_g, o->mass, o->bf_params.g11,
                 o->bf_params.g12, o->bf_params.g21, o->bf_params.g22, o->bf_params.a1, o->bf_params.a2,
                 o->div_epsilon, o->max_veloc, o->max_bfpot, o->c_bfpot };
  int n = (int) (sizeof(v) / sizeof(v[0]));
  memcpy(out, v, sizeof(v));
  return n;
}

void orc_ot_set_limits(dft_ot_functional *o, double div_epsilon, double max_veloc, double max_bfpot, double c_bfpot) {
  o->div_epsilon = div_epsilon; o->max_veloc = max_veloc; o->max_bfpot = max_bfpot; o->c_bfpot = c_bfpot;
}

/* which: 0 LJ, 1 SA, 2 F, 3 dF/dx, 4 dF/dy, 5 dF/dz, 6 V_j.  Returns 0 if absent. */
int orc_ot_kernel(dft_ot_functional *o, int which, double *out) {
  rgrid *g[] = { o->lennard_jones, o->spherical_avg, o->gaussian_tf, o->gaussian_x_tf, o->gaussian_y_tf,
                 o->gaussian_z_tf, o->backflow_pot };
  if (which < 0 || which > 6 || !g[which]) return 0;
  orc_rgrid_get_spectrum(g[which], out);
  return 1;
}

void orc_ot_potential(dft_ot_functional *o, cgrid *P, wf *g) { dft_ot_potential(o, P, g); }
void orc_ot_energy_density(dft_ot_functional *o, rgrid *ed, wf *g) { dft_ot_energy_density(o, ed, g); }

/* ---------------- propagation ---------------- */

void orc_propagate(wf *g, cgrid *P, double dtr, double dti) { grid_wf_propagate(g, P, dtr + I * dti); }
void orc_predict(wf *g, wf *gp, cgrid *P, double dtr, double dti) { grid_wf_propagate_predict(g, gp, P, dtr + I * dti); }
void orc_correct(wf *g, cgrid *P, double dtr, double dti) { grid_wf_propagate_correct(g, P, dtr + I * dti); }

/* One predict-correct step in the form every libdft dynamics example uses
 * (examples/imag_time/imag_time.c:231-239): vext may be NULL. */
void orc_pc_step(dft_ot_functional *otf, wf *g, wf *gp, cgrid *P, rgrid *vext, double mu0, double dtr, double dti) {
  REAL complex dt = dtr + I * dti;
  if (vext) grid_real_to_complex_re(P, vext); else cgrid_zero(P);
  dft_ot_potential(otf, P, g);
  cgrid_add(P, -mu0);
  grid_wf_propagate_predict(g, gp, P, dt);
  if (vext) grid_add_real_to_complex_re(P, vext);
  dft_ot_potential(otf, P, gp);
  cgrid_add(P, -mu0);
  cgrid_multiply(P, 0.5);
  grid_wf_propagate_correct(g, P, dt);
}

/* E = <T> + int eps[psi] + int rho V_ext (examples/imag_time/imag_time.c:251-253) */
double orc_total_energy(dft_ot_functional *otf, wf *g, rgrid *vext, rgrid *work) {
  dft_ot_energy_density(otf, work, g);
  if (vext) rgrid_add_scaled_product(work, 1.0, otf->density, vext);
  return grid_wf_energy(g, NULL) + rgrid_integral(work);
}

/* ---------------- bulk ---------------- */
double orc_bulk_density(dft_ot_functional *o, double p) { return dft_ot_bulk_density_pressurized(o, p); }
double orc_bulk_chempot(dft_ot_functional *o, double p) { return dft_ot_bulk_chempot_pressurized(o, p); }
double orc_bulk_dEdRho(dft_ot_functional *o, double rho) { return dft_ot_bulk_dEdRho(o, rho); }
double orc_bulk_energy(dft_ot_functional *o, double rho) { return dft_ot_bulk_energy(o, rho); }
double orc_bulk_sound_speed(dft_ot_functional *o, double rho) { return dft_ot_bulk_sound_speed(o, rho); }
double orc_bulk_dispersion(dft_ot_functional *o, double k, double rho0) { return dft_ot_bulk_dispersion(o, &k, rho0); }

double orc_const(int which) {
  switch (which) {
  case 0: return GRID_AUTOANG;
  case 1: return GRID_AUTOK;
  case 2: return GRID_AUTOFS;
  case 3: return GRID_AUTOAMU;
  case 4: return GRID_AUTOBAR;
  case 5: return GRID_AUTOMPS;
  default: return 0.0;
  }
}

#ifdef ORACLE_REF
/* ---------------- reference-only entry points (golden fixtures) ----------------
 * Term-level and density-driven calls of libdft (src/ot.c:431, 524, 547, 840;
 * src/ot-energy.c:123, 202), available only when libdft's own sources are
 * linked.  The work grids are allocated per call. */
static rgrid *ref_ws(rgrid *like) { return rgrid_clone(like, "oracle ref workspace"); }

void orc_ref_potential2(dft_ot_functional *o, cgrid *P, rgrid *rho, rgrid *vx, rgrid *vy, rgrid *vz) {
  dft_ot_potential2(o, P, rho, vx, vy, vz);
}
void orc_ref_add_lj(dft_ot_functional *o, cgrid *P, rgrid *rho) {
  rgrid *w1 = ref_ws(rho), *w2 = ref_ws(rho);
  dft_ot_add_lennard_jones_potential(o, P, rho, w1, w2);
  rgrid_free(w1); rgrid_free(w2);
}
void orc_ref_add_local(dft_ot_functional *o, cgrid *P, rgrid *rho) {
  /* rho_tf = FFT(rho), as dft_ot_add_lennard_jones_potential leaves it (src/ot.c:526-527) */
  rgrid *tf = ref_ws(rho), *w1 = ref_ws(rho), *w2 = ref_ws(rho);
  rgrid_copy(tf, rho);
  rgrid_fft(tf);
  dft_ot_add_local_correlation_potential(o, P, rho, tf, w1, w2);
  rgrid_free(tf); rgrid_free(w1); rgrid_free(w2);
}
void orc_ref_backflow(dft_ot_functional *o, cgrid *P, rgrid *rho, rgrid *vx, rgrid *vy, rgrid *vz) {
  rgrid *w[6];
  for (int i = 0; i < 6; i++) w[i] = ref_ws(rho);
  dft_ot_backflow_potential(o, P, rho, vx, vy, vz, w[0], w[1], w[2], w[3], w[4], w[5]);
  for (int i = 0; i < 6; i++) rgrid_free(w[i]);
}
void orc_ref_energy_density_kc(dft_ot_functional *o, rgrid *ed, wf *g, rgrid *rho) {
  dft_ot_energy_density_kc(o, ed, g, rho);
}
void orc_ref_energy_density_bf(dft_ot_functional *o, rgrid *ed, wf *g, rgrid *rho) {
  dft_ot_energy_density_bf(o, ed, g, rho);
}
#endif
