/*
 * CPU oracle: FP64 restatement of libdft's Orsay-Trento hot path.
 * TEST INFRASTRUCTURE ONLY -- it is the checker (and the timed CPU baseline)
 * for the GB300 library, never part of the shipped product.
 *
 * Covers the 0 K OT functional with optional kinetic correlation (KC) and
 * backflow (BF) on 3-D grids: parameters, kernel generation, potential,
 * energy density and the bulk (uniform-liquid) relations.  The arithmetic is
 * organised as a few fused per-point loops around FFT convolutions; every
 * term cites the reference line it restates.  The high-density terms (HD,
 * HD2) use the shim's restatement of libgrid's grid_func1..5 (grid_shim.c).
 * Unsupported models (thermal, GP, DR) are rejected with an error
 * message.
 */
#include <string.h>
#include "grid/grid.h"
#include "grid/au.h"
#include "dft/ot.h"

/* ------------------------------------------------------------------ */
/* kernel shape functions                                               */
/* ------------------------------------------------------------------ */

/* 4 eps ((s/r)^12 - (s/r)^6) given r^2 (src/common.c:31-39). */
REAL dft_common_lj_func(REAL r2, REAL sig, REAL eps) {
  REAL s2 = sig * sig / r2;
  REAL s6 = s2 * s2 * s2;
  return 4.0 * eps * s6 * (s6 - 1.0);
}

/* LJ with constant core for r <= h (src/common.c:53-66). */
REAL dft_common_lennard_jones(void *arg, REAL x, REAL y, REAL z) {
  const dft_common_lj *p = (const dft_common_lj *) arg;
  REAL r2 = x * x + y * y + z * z;
  if (r2 <= p->h * p->h) return p->cval;
  return dft_common_lj_func(r2, p->sigma, p->epsilon);
}

/* Normalised sphere indicator of radius h (src/common.c:131-138). */
REAL dft_common_spherical_avg(void *arg, REAL x, REAL y, REAL z) {
  REAL h = *(const REAL *) arg;
  if (x * x + y * y + z * z <= h * h) return 3.0 / (4.0 * M_PI * h * h * h);
  return 0.0;
}

/* Normalised 3-D Gaussian with inverse width arg (src/common.c:193-200). */
REAL dft_common_gaussian(void *arg, REAL x, REAL y, REAL z) {
  REAL iw = *(const REAL *) arg;
  REAL nrm = iw / sqrt(M_PI);
  return nrm * nrm * nrm * exp(-(x * x + y * y + z * z) * iw * iw);
}

/* Backflow kernel V_j(r) (src/ot-private.h:10-21). */
REAL dft_ot_backflow_pot(void *arg, REAL x, REAL y, REAL z) {
  const dft_ot_bf *p = (const dft_ot_bf *) arg;
  REAL r2 = x * x + y * y + z * z;
  return (p->g11 + p->g12 * r2) * exp(-p->a1 * r2) + (p->g21 + p->g22 * r2) * exp(-p->a2 * r2);
}

/* 1-D effective kernels of a grid with nx = ny = 1, already integrated over
 * the x-y plane (src/ot.c:133-217 with DFT_OT_1D, src/ot.h:146): LJ with the
 * core |z| < h evaluated at h (src/common.c:80-91), the sphere's cross-section
 * (src/common.c:152-158), the Gaussian's line density (src/common.c:214-220),
 * and the backflow kernel integrated over the plane (src/ot-private.h:29-41). */
REAL dft_common_lennard_jones_1d(void *arg, REAL x, REAL y, REAL z) {
  const dft_common_lj *p = (const dft_common_lj *) arg;
  REAL s6 = pow(p->sigma, 6.0);
  (void) x; (void) y;
  z = fabs(z);
  if (z < p->h) z = p->h;
  return 2.0 * M_PI * p->epsilon * s6 * (2.0 * s6 - 5.0 * pow(z, 6.0)) / (5.0 * pow(z, 10.0));
}

REAL dft_common_spherical_avg_1d(void *arg, REAL x, REAL y, REAL z) {
  REAL h = *(const REAL *) arg, h2 = h * h;
  (void) x; (void) y;
  z = fabs(z);
  if (z > h) return 0.0;
  return 3.0 * (h2 - z * z) / (4.0 * h2 * h);
}

REAL dft_common_gaussian_1d(void *arg, REAL x, REAL y, REAL z) {
  REAL iw = *(const REAL *) arg;
  (void) x; (void) y;
  return iw / sqrt(M_PI) * exp(-z * z * iw * iw);
}

REAL dft_ot_backflow_pot_1d(void *arg, REAL x, REAL y, REAL z) {
  const dft_ot_bf *p = (const dft_ot_bf *) arg;
  REAL z2 = z * z;
  (void) x; (void) y;
  return M_PI * ((p->g11 + p->g12 * (1.0 + p->a1 * z2) / p->a1) * exp(-p->a1 * z2) / p->a1
               + (p->g21 + p->g22 * (1.0 + p->a2 * z2) / p->a2) * exp(-p->a2 * z2) / p->a2);
}

/* sqrt(rho) (1 + a cos(k.r)) (src/common.c:1214-1224). */
REAL complex dft_common_planewave(void *arg, REAL x, REAL y, REAL z) {
  const dft_plane_wave *w = (const dft_plane_wave *) arg;
  REAL amp = sqrt(w->rho);
  return amp + w->a * amp * cos(w->kx * x + w->ky * y + w->kz * z);
}

/* ------------------------------------------------------------------ */
/* parameters                                                           */
/* ------------------------------------------------------------------ */

/* 0 K OT parameters (src/ot.c:1026-1036) and the shared constants and
 * atomic-unit conversions (src/ot.c:1234-1270). */
void dft_ot_init_params(dft_ot_functional *otf, INT model) {
  REAL a3 = GRID_AUTOANG * GRID_AUTOANG * GRID_AUTOANG;
  /* as src/ot.c:1002-1012: the model field is the caller's (dft_ot_alloc sets
   * it, src/ot.c:81); its high-density bits select the HD parameters */
  if (otf->model & (DFT_OT_HD | DFT_OT_HD2)) {
    otf->beta = (40.0 / (GRID_AUTOANG * GRID_AUTOANG * GRID_AUTOANG));
    otf->rhom = (0.37 * GRID_AUTOANG * GRID_AUTOANG * GRID_AUTOANG);
    otf->C = 0.1;
  } else {
    otf->beta = otf->rhom = otf->C = 0.0;
  }
  otf->b = -718.99;
  otf->c2 = -2.411857E4;
  otf->c2_exp = 2.0;
  otf->c3 = 1.858496E6;
  otf->c3_exp = 3.0;
  otf->c4 = 0.0;
  otf->temp = 0.0;
  otf->rho0 = 0.0218360;
  otf->lj_params.h = 2.1903;
  /* the thermal parameter sets (src/ot.c:1038-1222), each selected by its
   * bit; a later bit overrides an earlier one as in the reference */
  static const struct { INT bit; REAL b, c2, c3, c4, temp, rho0, h; } tset[] = {
    { DFT_OT_T0MK, -719.2435, -24258.88, 1865257.0, 0.0, 0.0, 0.0218354, 2.19035 },
    { DFT_OT_T400MK, -714.2174, -24566.29, 1873203.0, 0.98004, 0.4, 0.0218351, 2.18982 },
    { DFT_OT_T600MK, -705.1319, -25124.17, 1887707.0, 0.99915, 0.6, 0.0218346, 2.18887 },
    { DFT_OT_T800MK, -690.4745, -26027.12, 1911283.0, 0.99548, 0.8, 0.0218331, 2.18735 },
    { DFT_OT_T1200MK, -646.5135, -28582.81, 1973737.0, 0.99666, 1.2, 0.0218298, 2.18287 },
    { DFT_OT_T1400MK, -625.8123, -29434.03, 1984068.0, 0.99829, 1.4, 0.0218332, 2.18080 },
    { DFT_OT_T1600MK, -605.9788, -30025.96, 1980898.0, 1.00087, 1.6, 0.0218453, 2.17885 },
    { DFT_OT_T1800MK, -593.8289, -29807.56, 1945685.0, 1.00443, 1.8, 0.0218703, 2.17766 },
    { DFT_OT_T2000MK, -600.8313, -27850.96, 1847407.0, 1.00919, 2.0, 0.0219153, 2.17834 },
    { DFT_OT_T2100MK, -620.9129, -25418.15, 1747494.0, 1.01156, 2.1, 0.0219500, 2.18032 },
    { DFT_OT_T2200MK, -619.2016, -25096.68, 1720802.0, 1.01436, 2.2, 0.0219859, 2.18015 },
    { DFT_OT_T2400MK, -609.0757, -26009.98, 1747943.0, 1.02130, 2.4, 0.0218748, 2.17915 },
    { DFT_OT_T2600MK, -634.0664, -23790.66, 1670707.0, 1.02770, 2.6, 0.0217135, 2.18162 },
    { DFT_OT_T2800MK, -663.9942, -21046.37, 1574611.0, 1.03429, 2.8, 0.0215090, 2.18463 },
    { DFT_OT_T3000MK, -673.6543, -20022.76, 1535887.0, 1.04271, 3.0, 0.0212593, 2.18562 },
  };
  for (unsigned i = 0; i < sizeof(tset) / sizeof(tset[0]); i++)
    if (model & tset[i].bit) {
      otf->b = tset[i].b; otf->c2 = tset[i].c2; otf->c3 = tset[i].c3; otf->c4 = tset[i].c4;
      otf->temp = tset[i].temp; otf->rho0 = tset[i].rho0; otf->lj_params.h = tset[i].h;
    }
  otf->mu0 = 0.0;
  otf->xi = 1E4 / a3;
  otf->rhobf = 0.033 * a3;
  /* K, Angstrom -> hartree, bohr */
  otf->b /= GRID_AUTOK * a3;
  otf->c2 /= GRID_AUTOK * pow(GRID_AUTOANG, 3.0 * otf->c2_exp);
  otf->c3 /= GRID_AUTOK * pow(GRID_AUTOANG, 3.0 * otf->c3_exp);
  otf->rho0 *= a3;
  otf->lj_params.h /= GRID_AUTOANG;
  otf->lj_params.sigma = 2.556 / GRID_AUTOANG;
  otf->lj_params.epsilon = 10.22 / GRID_AUTOK;
  otf->lj_params.cval = 0.0;
  otf->rho_0s = 0.04 * GRID_AUTOANG * GRID_AUTOANG * GRID_AUTOANG;   /* the product order of src/ot.c:1248 */
  otf->alpha_s = 54.31 / a3;
  otf->l_g = 1.0 / GRID_AUTOANG;
  otf->mass = 4.0026 / GRID_AUTOAMU;
  otf->bf_params.g11 = -19.7544;
  otf->bf_params.g12 = 12.5616 * GRID_AUTOANG * GRID_AUTOANG;
  otf->bf_params.a1 = 1.023 * GRID_AUTOANG * GRID_AUTOANG;
  otf->bf_params.g21 = -0.2395;
  otf->bf_params.g22 = 0.0312 * GRID_AUTOANG * GRID_AUTOANG;
  otf->bf_params.a2 = 0.14912 * GRID_AUTOANG * GRID_AUTOANG;
  otf->div_epsilon = DFT_EPS;
  otf->max_veloc = 999.0 / GRID_AUTOMPS;
  otf->max_bfpot = 10000.0 / GRID_AUTOK;
  otf->c_bfpot = 1.0;
}

/* ------------------------------------------------------------------ */
/* helpers                                                              */
/* ------------------------------------------------------------------ */

#define NRM(g) ((g)->nx * (g)->ny)
#define V(g, ij, k) ((g)->value[(ij) * (g)->nz2 + (k)])

static REAL ipow(REAL v, INT n) {
  REAL r = 1.0;
  for (INT m = 0; m < n; m++) r *= v;
  return r;
}

/* dst(real) = (kernel * src)(r): both spectra already transformed. */
static void convolve(rgrid *dst, rgrid *spec, rgrid *kernel) {
  rgrid_fft_convolute(dst, spec, kernel);
  rgrid_inverse_fft_norm2(dst);
}

/* central difference of src along axis at (i,j,k), periodic */
static inline REAL fd(const rgrid *s, INT i, INT j, INT k, int axis) {
  INT nx = s->nx, ny = s->ny, nz = s->nz;
  REAL p, m;
  if (axis == 0) {
    if (nx == 1) return 0.0;
    p = s->value[(((i + 1) % nx) * ny + j) * s->nz2 + k];
    m = s->value[(((i - 1 + nx) % nx) * ny + j) * s->nz2 + k];
  } else if (axis == 1) {
    if (ny == 1) return 0.0;
    p = s->value[(i * ny + (j + 1) % ny) * s->nz2 + k];
    m = s->value[(i * ny + (j - 1 + ny) % ny) * s->nz2 + k];
  } else {
    if (nz == 1) return 0.0;
    p = s->value[(i * ny + j) * s->nz2 + (k + 1) % nz];
    m = s->value[(i * ny + j) * s->nz2 + (k - 1 + nz) % nz];
  }
  return (p - m) / (2.0 * s->step);
}

static int check_model(INT model, const char *who) {
  if (model & ~((INT) ORACLE_SUPPORTED_MODELS)) {
    fprintf(stderr, "oracle: %s: model " FMT_I " is outside the restated subset (OT 0 K, KC, HD, BF).\n", who, model);
    return 0;
  }
  return 1;
}

/* ------------------------------------------------------------------ */
/* allocation and kernel generation (src/ot.c:66-258)                   */
/* ------------------------------------------------------------------ */

static rgrid *new_grid(wf *gwf, char *id) {
  cgrid *c = gwf->grid;
  rgrid *g = rgrid_alloc(c->nx, c->ny, c->nz, c->step, RGRID_PERIODIC_BOUNDARY, NULL, id);
  rgrid_set_origin(g, c->x0, c->y0, c->z0);
  return g;
}

dft_ot_functional *dft_ot_alloc(INT model, wf *gwf, INT min_ns, INT max_ns) {
  cgrid *c = gwf->grid;
  REAL step = c->step, tol = 0.01 / GRID_AUTOK, radius, iw;

  const int one_d = c->nx == 1 && c->ny == 1;   /* the 1-D effective model (src/ot.c:133-217) */
  if (!check_model(model, "dft_ot_alloc")) return NULL;
  dft_ot_functional *otf = (dft_ot_functional *) calloc(1, sizeof(dft_ot_functional));
  if (!otf) return NULL;
  otf->model = model;
  dft_ot_init_params(otf, model);

  /* LJ kernel, rescaled so that its integral is b (src/ot.c:150-161) */
  otf->lennard_jones = new_grid(gwf, "OT LJ");
  rgrid_adaptive_map(otf->lennard_jones, one_d ? dft_common_lennard_jones_1d : dft_common_lennard_jones,
                     &otf->lj_params, min_ns, max_ns, tol);
  rgrid_fft(otf->lennard_jones);
  if (!one_d)   /* the 1-D kernels are not rescaled (src/ot.c:159-160, 180-181) */
    rgrid_fft_multiply(otf->lennard_jones, otf->b / (step * step * step * creal(rgrid_cvalue_at_index(otf->lennard_jones, 0, 0, 0))));

  /* spherical average of radius h (HD2: 1.065 h), integral 1 (src/ot.c:164-181) */
  radius = (model & DFT_OT_HD2) ? otf->lj_params.h * 1.065 : otf->lj_params.h;
  otf->spherical_avg = new_grid(gwf, "OT SA");
  rgrid_adaptive_map(otf->spherical_avg, one_d ? dft_common_spherical_avg_1d : dft_common_spherical_avg, &radius,
                     min_ns, max_ns, tol);
  rgrid_fft(otf->spherical_avg);
  if (!one_d)
    rgrid_fft_multiply(otf->spherical_avg, 1.0 / (step * step * step * creal(rgrid_cvalue_at_index(otf->spherical_avg, 0, 0, 0))));

  /* KC Gaussian F and its finite-difference gradient (src/ot.c:184-200) */
  if (model & DFT_OT_KC) {
    iw = 1.0 / otf->l_g;
    otf->gaussian_tf = new_grid(gwf, "OT F");
    otf->gaussian_x_tf = new_grid(gwf, "OT dF/dx");
    otf->gaussian_y_tf = new_grid(gwf, "OT dF/dy");
    otf->gaussian_z_tf = new_grid(gwf, "OT dF/dz");
    rgrid_adaptive_map(otf->gaussian_tf, one_d ? dft_common_gaussian_1d : dft_common_gaussian, &iw, min_ns, max_ns, tol);
    rgrid_gradient(otf->gaussian_tf, otf->gaussian_x_tf, otf->gaussian_y_tf, otf->gaussian_z_tf);
    rgrid_fft(otf->gaussian_x_tf);
    rgrid_fft(otf->gaussian_y_tf);
    rgrid_fft(otf->gaussian_z_tf);
    rgrid_fft(otf->gaussian_tf);
  }

  /* backflow kernel V_j (src/ot.c:207-217) */
  if (model & DFT_OT_BACKFLOW) {
    otf->backflow_pot = new_grid(gwf, "OT Vj");
    rgrid_adaptive_map(otf->backflow_pot, one_d ? dft_ot_backflow_pot_1d : dft_ot_backflow_pot, &otf->bf_params,
                       min_ns, max_ns, tol);
    rgrid_fft(otf->backflow_pot);
  }

  otf->density = new_grid(gwf, "OT density");
  rgrid **ws[9] = { &otf->workspace1, &otf->workspace2, &otf->workspace3, &otf->workspace4, &otf->workspace5,
                    &otf->workspace6, &otf->workspace7, &otf->workspace8, &otf->workspace9 };
  for (int i = 0; i < 9; i++) *ws[i] = new_grid(gwf, "OT workspace");
  return otf;
}

void dft_ot_free(dft_ot_functional *otf) {
  if (!otf) return;
  rgrid *g[] = { otf->lennard_jones, otf->spherical_avg, otf->gaussian_tf, otf->gaussian_x_tf, otf->gaussian_y_tf,
                 otf->gaussian_z_tf, otf->backflow_pot, otf->density, otf->workspace1, otf->workspace2,
                 otf->workspace3, otf->workspace4, otf->workspace5, otf->workspace6, otf->workspace7,
                 otf->workspace8, otf->workspace9 };
  for (size_t i = 0; i < sizeof(g) / sizeof(g[0]); i++) if (g[i]) rgrid_free(g[i]);
  free(otf);
}

/* ------------------------------------------------------------------ */
/* potential (src/ot.c:314-408)                                         */
/* ------------------------------------------------------------------ */

/* KC potential (src/ot.c:604-797).  rk = FFT(rho) on entry. */
static void kc_potential(dft_ot_functional *otf, cgrid *P, rgrid *rho, rgrid *rk) {
  rgrid *rst = otf->workspace2, *g = otf->workspace3, *s = otf->workspace4, *t1 = otf->workspace5;
  rgrid *J = otf->workspace6, *h = otf->workspace7, *d = otf->workspace8;
  rgrid *dF[3] = { otf->gaussian_x_tf, otf->gaussian_y_tf, otf->gaussian_z_tf };
  INT nx = rho->nx, ny = rho->ny, nz = rho->nz;
  REAL c = otf->alpha_s / (2.0 * otf->mass);

  /* rho_st = 1 - (F * rho) / rho_0s  (src/ot.c:608-612) */
  convolve(rst, rk, otf->gaussian_tf);
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < NRM(rho); ij++)
    for (INT k = 0; k < nz; k++) V(rst, ij, k) = 1.0 - V(rst, ij, k) / otf->rho_0s;

  for (int a = 0; a < 3; a++) {
    if ((a == 0 && nx == 1) || (a == 1 && ny == 1)) continue;   /* src/ot.c:614-616 */
    /* g = d_a rho ; s = g rho_st ; G_a = FFT(s)  (src/ot.c:632-638) */
#pragma omp parallel for schedule(static)
    for (INT ij = 0; ij < NRM(rho); ij++) {
      INT i = ij / ny, j = ij % ny;
      for (INT k = 0; k < nz; k++) {
        REAL gv = fd(rho, i, j, k, a);
        V(g, ij, k) = gv;
        V(s, ij, k) = gv * V(rst, ij, k);
      }
    }
    rgrid_fft(s);
    convolve(t1, s, dF[a]);                    /* (dF_a * G_a)     src/ot.c:641-642 */
    convolve(J, s, otf->gaussian_tf);          /* J = F * G_a      src/ot.c:652-653 */
#pragma omp parallel for schedule(static)
    for (INT ij = 0; ij < NRM(rho); ij++)
      for (INT k = 0; k < nz; k++) V(h, ij, k) = V(g, ij, k) * V(J, ij, k);   /* H = g J  src/ot.c:656-657 */
    rgrid_fft(h);
    rgrid_fft_convolute(h, h, otf->gaussian_tf);  /* F * H          src/ot.c:661-662 */
    rgrid_inverse_fft_norm2(h);
    convolve(d, rk, dF[a]);                    /* dF_a * rho       src/ot.c:671-672 */
    /* P += c rho_st (dF_a*G_a) + c (F*H) - c J (dF_a*rho)  (src/ot.c:643-645,663-664,673-675) */
#pragma omp parallel for schedule(static)
    for (INT ij = 0; ij < NRM(rho); ij++)
      for (INT k = 0; k < nz; k++) {
        REAL add = c * V(rst, ij, k) * V(t1, ij, k) + c * V(h, ij, k) - c * V(J, ij, k) * V(d, ij, k);
        P->value[ij * nz + k] += add;
      }
  }
}

/* BF potential (src/ot.c:380-400 and 840-991); rk = FFT(rho).  With HD / HD2
 * the backflow sees the cut-off density rho G(rho) (src/ot.c:843-886) and its
 * real part is multiplied by d(rho G)/drho (src/ot.c:907-908), the imaginary
 * part's gradients by G (src/ot.c:934-982). */
static void bf_potential(dft_ot_functional *otf, cgrid *P, wf *gwf, rgrid *rho, rgrid *rk) {
  rgrid *vx = otf->workspace2, *vy = otf->workspace3, *vz = otf->workspace4;
  rgrid *A = otf->workspace5, *C = otf->workspace6, *Bx = otf->workspace7, *By = otf->workspace8, *Bz = otf->workspace9;
  rgrid *v[3] = { vx, vy, vz }, *B[3] = { Bx, By, Bz };
  INT ny = rho->ny, nz = rho->nz;
  REAL m = otf->mass, cap = otf->max_veloc, bcap = otf->max_bfpot, eps = otf->div_epsilon;
  int clamp_v = otf->max_veloc < (999.0 / GRID_AUTOMPS);
  int clamp_p = otf->max_bfpot < (10000.0 / GRID_AUTOK);
  int hd = (otf->model & (DFT_OT_HD | DFT_OT_HD2)) != 0;
  rgrid *rt = rho, *gfac = NULL, *dfac = NULL;                 /* rho G, G, d(rho G)/drho */

  grid_wf_velocity(gwf, vx, vy, vz, otf->div_epsilon);       /* src/ot.c:390 */
  if (clamp_v)                                                 /* src/ot.c:391-395 */
    for (int a = 0; a < 3; a++) rgrid_threshold_clear(v[a], v[a], cap, -cap, cap, -cap);

  if (hd) {
    rt = rgrid_clone(rho, "rho G");
    gfac = rgrid_clone(rho, "G");
    dfac = rgrid_clone(rho, "d(rho G)");
    rgrid_constant(gfac, 1.0);
    rgrid_constant(dfac, 1.0);
    grid_func2_operate_one(rt, rho, otf->xi, otf->rhobf);
    grid_func1_operate_one_product(gfac, gfac, rho, otf->xi, otf->rhobf);
    grid_func3_operate_one_product(dfac, dfac, rho, otf->xi, otf->rhobf);
    rgrid_copy(A, rt);
    rgrid_fft(A);
    rgrid_fft_convolute(A, A, otf->backflow_pot);              /* A = V_j * (rho G)  src/ot.c:843-849 */
    rgrid_inverse_fft_norm2(A);
  } else
    convolve(A, rk, otf->backflow_pot);                        /* A = V_j * rho   src/ot.c:842-849 */
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < NRM(rho); ij++)
    for (INT k = 0; k < nz; k++) {
      REAL r = V(rt, ij, k), x = V(vx, ij, k), y = V(vy, ij, k), z = V(vz, ij, k);
      V(C, ij, k) = (z * z + y * y + x * x) * r;               /* rho |v|^2   src/ot.c:852-860 */
      V(Bx, ij, k) = x * r;                                    /* rho v_a     src/ot.c:871,879,888 */
      V(By, ij, k) = y * r;
      V(Bz, ij, k) = z * r;
    }
  rgrid_fft(C);
  rgrid_fft_convolute(C, C, otf->backflow_pot);
  rgrid_inverse_fft_norm2(C);
  for (int a = 0; a < 3; a++) {
    rgrid_fft(B[a]);
    rgrid_fft_convolute(B[a], B[a], otf->backflow_pot);
    rgrid_inverse_fft_norm2(B[a]);
  }
  /* real part -(m/2)[A v^2 - 2 v.B + C] (src/ot.c:895-915); then v_a <- v_a A - B_a (src/ot.c:924-931) */
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < NRM(rho); ij++)
    for (INT k = 0; k < nz; k++) {
      REAL x = V(vx, ij, k), y = V(vy, ij, k), z = V(vz, ij, k), a = V(A, ij, k);
      REAL re = -0.5 * m * (a * (z * z + y * y + x * x) - 2.0 * (x * V(Bx, ij, k) + y * V(By, ij, k) + z * V(Bz, ij, k)) + V(C, ij, k));
      if (hd) re *= V(dfac, ij, k);
      if (clamp_p) { if (re > bcap) re = bcap; else if (re < -bcap) re = -bcap; }
      re *= otf->c_bfpot;
      P->value[ij * nz + k] += re;
      V(vx, ij, k) = x * a - V(Bx, ij, k);
      V(vy, ij, k) = y * a - V(By, ij, k);
      V(vz, ij, k) = z * a - V(Bz, ij, k);
    }
  /* imaginary part (1/2) sum_a [ (d_a rho / rho) w_a + d_a w_a ] (src/ot.c:933-990) */
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < NRM(rho); ij++) {
    INT i = ij / ny, j = ij % ny;
    for (INT k = 0; k < nz; k++) {
      REAL r = V(rho, ij, k), im = 0.0;
      if (r < eps) r = eps;
      for (int a = 0; a < 3; a++) im += 0.5 * (fd(rt, i, j, k, a) / r) * V(v[a], ij, k);
      for (int a = 0; a < 3; a++) im += 0.5 * fd(v[a], i, j, k, a) * (hd ? V(gfac, ij, k) : 1.0);
      if (clamp_p) { if (im > bcap) im = bcap; else if (im < -bcap) im = -bcap; }
      im *= otf->c_bfpot;
      P->value[ij * nz + k] += I * im;
    }
  }
  if (hd) {
    rgrid_free(rt);
    rgrid_free(gfac);
    rgrid_free(dfac);
  }
}

void dft_ot_potential(dft_ot_functional *otf, cgrid *P, wf *gwf) {
  rgrid *rho = otf->density, *rk = otf->workspace1, *u = otf->workspace2, *rb = otf->workspace3, *q = otf->workspace4;
  INT nz = rho->nz;
  REAL c2 = otf->c2, c3 = otf->c3;
  INT e2 = (INT) otf->c2_exp, e3 = (INT) otf->c3_exp;

  if (!check_model(otf->model, "dft_ot_potential")) abort();
  grid_wf_density(gwf, rho);                                   /* src/ot.c:320 */
  rgrid_copy(rk, rho);
  rgrid_fft(rk);                                               /* src/ot.c:526-527 */
  convolve(u, rk, otf->lennard_jones);                         /* src/ot.c:528-529 */
  convolve(rb, rk, otf->spherical_avg);                        /* rho_bar  src/ot.c:550-551 */
  /* P += V_LJ*rho + c2/2 rb^2 + c3/3 rb^3 ; q = (c2 e2/2 rb^(e2-1) + c3 e3/3 rb^(e3-1)) rho
   * (src/ot.c:530, 557-559, 565-567, 574-581) */
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < NRM(rho); ij++)
    for (INT k = 0; k < nz; k++) {
      REAL b = V(rb, ij, k);
      P->value[ij * nz + k] += V(u, ij, k) + (c2 / 2.0) * ipow(b, e2) + (c3 / 3.0) * ipow(b, e3);
      V(q, ij, k) = ((c2 * (REAL) e2 / 2.0) * ipow(b, e2 - 1) + (c3 * (REAL) e3 / 3.0) * ipow(b, e3 - 1)) * V(rho, ij, k);
    }
  rgrid_fft(q);                                                /* src/ot.c:582-585 */
  rgrid_fft_convolute(q, q, otf->spherical_avg);
  rgrid_inverse_fft_norm2(q);
  grid_add_real_to_complex_re(P, q);

  if (otf->model & DFT_OT_KC) kc_potential(otf, P, rho, rk);
  if (otf->model & (DFT_OT_HD | DFT_OT_HD2)) {                 /* Barranco penalty  src/ot.c:374-378, 815-819 */
    grid_func4_operate_one(q, rho, otf->beta, otf->rhom, otf->C);
    grid_add_real_to_complex_re(P, q);
  }
  if (otf->model & DFT_OT_BACKFLOW) bf_potential(otf, P, gwf, rho, rk);
  if (otf->model >= DFT_OT_T400MK) {                           /* ideal Bose gas  src/ot.c:402-407, 804-809 */
    grid_func6a_operate_one(q, rho, otf->mass, otf->temp, otf->c4);
    grid_add_real_to_complex_re(P, q);
  }
}

/* ------------------------------------------------------------------ */
/* energy density (src/ot-energy.c:38-288)                              */
/* ------------------------------------------------------------------ */

void dft_ot_energy_density(dft_ot_functional *otf, rgrid *ed, wf *gwf) {
  rgrid *rho = otf->density, *rk = otf->workspace1, *u = otf->workspace2, *rb = otf->workspace3;
  INT nx = rho->nx, ny = rho->ny, nz = rho->nz;
  REAL c2 = otf->c2, c3 = otf->c3;
  INT e2 = (INT) otf->c2_exp, e3 = (INT) otf->c3_exp;

  if (!check_model(otf->model, "dft_ot_energy_density")) abort();
  grid_wf_density(gwf, rho);
  rgrid_copy(rk, rho);
  rgrid_fft(rk);
  convolve(u, rk, otf->lennard_jones);
  convolve(rb, rk, otf->spherical_avg);
  /* (1/2) rho (V_LJ*rho) + c2/2 rb^e2 rho + c3/3 rb^e3 rho  (src/ot-energy.c:70-93) */
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < NRM(rho); ij++)
    for (INT k = 0; k < nz; k++) {
      REAL r = V(rho, ij, k), b = V(rb, ij, k);
      V(ed, ij, k) = 0.5 * r * V(u, ij, k) + (c2 / 2.0) * (ipow(b, e2) * r) + (c3 / 3.0) * (ipow(b, e3) * r);
    }
  if (otf->model & (DFT_OT_HD | DFT_OT_HD2)) {                 /* Barranco  src/ot-energy.c:96-99 */
    grid_func5_operate_one(u, rho, otf->beta, otf->rhom, otf->C);
    rgrid_sum(ed, ed, u);
  }
  if (otf->model >= DFT_OT_T400MK) {                           /* ideal Bose gas  src/ot-energy.c:101-105 */
    grid_func6b_operate_one(u, rho, otf->mass, otf->temp, otf->c4);
    rgrid_sum(ed, ed, u);
  }

  if (otf->model & DFT_OT_KC) {
    /* -(alpha_s / 4m) sum_a g_a rho_st [F * (g_a rho_st)]  (src/ot-energy.c:144-190) */
    rgrid *rst = otf->workspace2, *s = otf->workspace3;
    REAL f = -otf->alpha_s / (4.0 * otf->mass);
    convolve(rst, rk, otf->gaussian_tf);
#pragma omp parallel for schedule(static)
    for (INT ij = 0; ij < NRM(rho); ij++)
      for (INT k = 0; k < nz; k++) V(rst, ij, k) = V(rst, ij, k) * (-1.0 / otf->rho_0s) + 1.0;
    for (int a = 0; a < 3; a++) {
#pragma omp parallel for schedule(static)
      for (INT ij = 0; ij < NRM(rho); ij++) {
        INT i = ij / ny, j = ij % ny;
        for (INT k = 0; k < nz; k++) V(s, ij, k) = fd(rho, i, j, k, a) * V(rst, ij, k);
      }
      rgrid_fft(s);
      rgrid_fft_convolute(s, s, otf->gaussian_tf);
      rgrid_inverse_fft_norm2(s);
#pragma omp parallel for schedule(static)
      for (INT ij = 0; ij < NRM(rho); ij++) {
        INT i = ij / ny, j = ij % ny;
        for (INT k = 0; k < nz; k++) V(ed, ij, k) += f * (V(s, ij, k) * fd(rho, i, j, k, a) * V(rst, ij, k));
      }
    }
  }

  if (otf->model & DFT_OT_BACKFLOW) {
    /* (src/ot-energy.c:221-287); with HD / HD2 every density of the backflow
     * energy is the cut-off density rho G(rho) (src/ot-energy.c:221-227) */
    rgrid *vx = otf->workspace2, *vy = otf->workspace3, *vz = otf->workspace4, *t = otf->workspace5;
    rgrid *v[3] = { vx, vy, vz };
    REAL cm = otf->c_bfpot * otf->mass;
    int hd = (otf->model & (DFT_OT_HD | DFT_OT_HD2)) != 0;
    rgrid *rho_in = rho;
    if (hd) {
      rho = rgrid_clone(rho_in, "rho G");
      grid_func2_operate_one(rho, rho_in, otf->xi, otf->rhobf);
    }
    grid_wf_velocity(gwf, vx, vy, vz, DFT_EPS);
    if (hd) {
      rgrid_copy(t, rho);
      rgrid_fft(t);
      rgrid_fft_convolute(t, t, otf->backflow_pot);
      rgrid_inverse_fft_norm2(t);
    } else
      convolve(t, rk, otf->backflow_pot);
#pragma omp parallel for schedule(static)
    for (INT ij = 0; ij < NRM(rho); ij++)
      for (INT k = 0; k < nz; k++) {
        REAL x = V(vx, ij, k), y = V(vy, ij, k), z = V(vz, ij, k);
        V(ed, ij, k) += -(cm / 4.0) * (V(t, ij, k) * (x * x + y * y + z * z) * V(rho, ij, k));
      }
    for (int a = 0; a < 3; a++) {
#pragma omp parallel for schedule(static)
      for (INT ij = 0; ij < NRM(rho); ij++)
        for (INT k = 0; k < nz; k++) V(t, ij, k) = V(rho, ij, k) * V(v[a], ij, k);
      rgrid_fft(t);
      rgrid_fft_convolute(t, t, otf->backflow_pot);
      rgrid_inverse_fft_norm2(t);
#pragma omp parallel for schedule(static)
      for (INT ij = 0; ij < NRM(rho); ij++)
        for (INT k = 0; k < nz; k++) V(ed, ij, k) += (cm / 2.0) * (V(t, ij, k) * V(rho, ij, k) * V(v[a], ij, k));
    }
#pragma omp parallel for schedule(static)
    for (INT ij = 0; ij < NRM(rho); ij++)
      for (INT k = 0; k < nz; k++) {
        REAL x = V(vx, ij, k), y = V(vy, ij, k), z = V(vz, ij, k);
        V(t, ij, k) = V(rho, ij, k) * (x * x + y * y + z * z);
      }
    rgrid_fft(t);
    rgrid_fft_convolute(t, t, otf->backflow_pot);
    rgrid_inverse_fft_norm2(t);
#pragma omp parallel for schedule(static)
    for (INT ij = 0; ij < NRM(rho); ij++)
      for (INT k = 0; k < nz; k++) V(ed, ij, k) += -(cm / 4.0) * (V(t, ij, k) * V(rho, ij, k));
    if (hd) {
      rgrid_free(rho);
      rho = rho_in;
    }
  }
  (void) nx;
}

/* ------------------------------------------------------------------ */
/* bulk liquid (src/helium-ot-bulk.c:21-434)                            */
/* ------------------------------------------------------------------ */

/* E/V = b/2 rho^2 + c2/2 rho^3 + c3/3 rho^4 (+ the ideal Bose gas when c4 != 0)
 * (src/helium-ot-bulk.c:21-33) */
REAL dft_ot_bulk_energy(dft_ot_functional *otf, REAL rho) {
  REAL e = 0.5 * otf->b * rho * rho + 0.5 * otf->c2 * rho * rho * rho + (1.0 / 3.0) * otf->c3 * rho * rho * rho * rho;
  if (otf->c4 != 0.0) e += oracle_bose_energy(rho, otf->mass, otf->temp, otf->c4);
  return e;
}

/* dE/drho (src/helium-ot-bulk.c:45-57) */
REAL dft_ot_bulk_dEdRho(dft_ot_functional *otf, REAL rho) {
  REAL d = otf->b * rho + 1.5 * otf->c2 * rho * rho + (4.0 / 3.0) * otf->c3 * rho * rho * rho;
  if (otf->c4 != 0.0) d += oracle_bose_dEdRho(rho, otf->mass, otf->temp, otf->c4);
  return d;
}

/* P = rho dE/drho - E (src/helium-ot-bulk.c:143-146) */
REAL dft_ot_bulk_pressure(dft_ot_functional *otf, REAL rho) {
  return rho * dft_ot_bulk_dEdRho(otf, rho) - dft_ot_bulk_energy(otf, rho);
}

/* central difference with step 1e-7 (src/helium-ot-bulk.c:157-172) */
REAL dft_ot_bulk_dPdRho(dft_ot_functional *otf, REAL rho) {
  const REAL h = 1E-7;
  return (dft_ot_bulk_pressure(otf, rho + h) - dft_ot_bulk_pressure(otf, rho - h)) / (2.0 * h);
}

/* Newton iteration from rho = 1 a.u., |P - P0| < 1e-12 (src/helium-ot-bulk.c:185-211) */
REAL dft_ot_bulk_density_pressurized(dft_ot_functional *otf, REAL pressure) {
  REAL rho = 1.0, miss = dft_ot_bulk_pressure(otf, rho) - pressure;
  for (int it = 0; it < 1000; it++) {
    if (fabs(miss) < 1.0E-12) return rho;
    rho -= miss / dft_ot_bulk_dPdRho(otf, rho);
    miss = dft_ot_bulk_pressure(otf, rho) - pressure;
  }
  fprintf(stderr, "oracle: bulk density Newton iteration did not converge.\n");
  return NAN;
}

REAL dft_ot_bulk_chempot_pressurized(dft_ot_functional *otf, REAL pressure) {
  return dft_ot_bulk_dEdRho(otf, dft_ot_bulk_density_pressurized(otf, pressure));
}

REAL dft_ot_bulk_density(dft_ot_functional *otf) { return dft_ot_bulk_density_pressurized(otf, 0.0); }
REAL dft_ot_bulk_chempot(dft_ot_functional *otf) { return dft_ot_bulk_dEdRho(otf, dft_ot_bulk_density(otf)); }
REAL dft_ot_bulk_chempot2(dft_ot_functional *otf) { return dft_ot_bulk_dEdRho(otf, otf->rho0); }

REAL dft_ot_bulk_compressibility(dft_ot_functional *otf, REAL rho) {
  return 1.0 / (rho * dft_ot_bulk_dPdRho(otf, rho));
}

REAL dft_ot_bulk_sound_speed(dft_ot_functional *otf, REAL rho) {
  return 1.0 / sqrt(otf->mass * rho * dft_ot_bulk_compressibility(otf, rho));
}

/* Fourier transform of the core-cut LJ by midpoint-free rectangle sum
 * (src/helium-ot-bulk.c:379-388). */
static REAL bulk_ft_lj(dft_ot_functional *otf, REAL k) {
  REAL sg = otf->lj_params.sigma, ks = k * sg, acc = 0.0;
  for (REAL x = otf->lj_params.h / sg; x < 1E3; x += 1.0E-2) acc += sin(ks * x) * (pow(x, -11.0) - pow(x, -5.0));
  return acc * 1.0E-2 * 16.0 * M_PI * otf->lj_params.epsilon * sg * sg * sg / ks;
}

static REAL bulk_ft_sphere(dft_ot_functional *otf, REAL k) {
  REAL kh = k * otf->lj_params.h;
  return (3.0 / (kh * kh * kh)) * (sin(kh) - kh * cos(kh));
}

static REAL bulk_ft_vj(dft_ot_functional *otf, REAL k) {
  const dft_ot_bf *p = &otf->bf_params;
  REAL k2 = k * k, pi32 = pow(M_PI, 1.5);
  REAL t1 = (p->g11 * pow(M_PI / p->a1, 1.5) + p->g12 * (6.0 * p->a1 - k2) * pi32 / (4.0 * pow(p->a1, 3.5))) * exp(-k2 / (4.0 * p->a1));
  REAL t2 = (p->g21 * pow(M_PI / p->a2, 1.5) + p->g22 * (6.0 * p->a2 - k2) * pi32 / (4.0 * pow(p->a2, 3.5))) * exp(-k2 / (4.0 * p->a2));
  return t1 + t2;
}

/* Semi-analytic bulk dispersion omega(k) (src/helium-ot-bulk.c:411-434). */
REAL dft_ot_bulk_dispersion(dft_ot_functional *otf, REAL *k, REAL rho0) {
  REAL kk = *k;
  if (rho0 < 0.0 || kk < 1E-3) return 0.0;
  REAL lj = bulk_ft_lj(otf, kk), pi = bulk_ft_sphere(otf, kk);
  REAL t = HBAR * HBAR * kk * kk / otf->mass;
  REAL chi = t / 4.0 + rho0 * lj + otf->c2 * (2.0 * pi + pi * pi) * rho0 * rho0 + 2.0 * otf->c3 * (pi + pi * pi) * rho0 * rho0 * rho0;
  if (otf->model & DFT_OT_KC) {
    REAL f = 1.0 - rho0 / otf->rho_0s;
    chi += -(t / 2.0) * otf->alpha_s * rho0 * f * f * exp(-kk * kk * otf->l_g * otf->l_g / 4.0);
  }
  if (otf->model & DFT_OT_BACKFLOW)
    return sqrt(t * chi * (1.0 - rho0 * (bulk_ft_vj(otf, 0.0) - bulk_ft_vj(otf, kk))));
  return sqrt(t * chi);
}
