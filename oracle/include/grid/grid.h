/*
 * CPU oracle: FP64 restatement of the libgrid subset that libdft's hot path
 * calls.  TEST INFRASTRUCTURE ONLY -- this is the checker that the GB300
 * library is compared against, never part of the shipped product.
 *
 * libdft includes <grid/grid.h> (src/ot.c:12) from jmeloranta/libgrid
 * ("multi-GPU branch", README:17-18; no version pinned, not vendored).  That
 * library is absent, so every function here is restated from its name, its
 * call sites in libdft and the mathematics it has to compute.  The semantics
 * chosen where libgrid's own choice cannot be seen ("parity unpinned at the
 * libgrid boundary") are:
 *
 *  - grid coordinates: x_i = (i - nx/2) * step - x0 (integer nx/2), the form
 *    libdft itself uses at src/common.c:1183-1187;
 *  - rgrid storage: real value (i,j,k) at (i*ny + j)*nz2 + k with
 *    nz2 = 2*(nz/2+1), so the r2c half spectrum fits in place; k-space value
 *    (i,j,kz) is complex element (i*ny + j)*(nz/2+1) + kz;
 *  - rgrid_fft / cgrid_fft: unnormalised forward DFT, exp(-2 pi i k.n/N);
 *    rgrid_inverse_fft_norm: scaled 1/N; rgrid_inverse_fft_norm2: scaled
 *    step^3/N (the convolution normalisation implied by src/ot.c:160,181);
 *  - rgrid_fft_convolute: product of two spectra times the phase that moves
 *    a kernel sampled about index n/2 of each axis to index 0:
 *    exp(2 pi i k (n/2) / n) per axis, i.e. (-1)^(i+j+k) for even sizes and a
 *    rotation for odd x / y sizes;
 *  - finite differences: second-order central, periodic;
 *  - rgrid_adaptive_map: cell average over s^3 cell-centred sub-points,
 *    s = min_ns, 2 min_ns, ... <= max_ns, stopping when two successive
 *    averages differ by less than tol;
 *  - grid_wf_velocity: v = (hbar/m) Im(psi^* D psi) / max(|psi|^2, eps);
 *    rgrid_division_eps: a / max(b, eps);
 *  - propagation (WF_2ND_ORDER_FFT, periodic): one step
 *    S(V,dt) = exp(-i V dt/2) F^-1 exp(-i hbar k^2 dt / 2m) F exp(-i V dt/2),
 *    complex dt allowed; predict: psi_p = S(V,dt) psi, correct:
 *    psi = S(V,dt) psi with the caller's averaged V;
 *  - WF_2ND_ORDER_CN (periodic): the same S with the kinetic factor replaced
 *    by Crank-Nicolson on the 3-point finite-difference operator, axis by
 *    axis, prod_a (1 - i hbar Q_a dt / 4m) / (1 + i hbar Q_a dt / 4m) with
 *    Q_a = (2 sin((k_a - k0_a) step / 2) / step)^2 (each axis operator is
 *    diagonal in k); the kinetic energy of such a wave function uses Q_a in
 *    place of (k_a - k0_a)^2.
 */
#ifndef ORACLE_GRID_GRID_H
#define ORACLE_GRID_GRID_H

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#define REAL double   /* a macro, so that "REAL complex" is a valid type */
#define INT long

#define FMT_R "%le"
#define FMT_I "%ld"

#define EXP(x) exp(x)
#define POW(x, y) pow(x, y)
#define SQRT(x) sqrt(x)
#define FABS(x) fabs(x)
#define SIN(x) sin(x)
#define COS(x) cos(x)
#define TAN(x) tan(x)
#define LOG(x) log(x)
#define ACOS(x) acos(x)
#define ASIN(x) asin(x)
#define ATAN(x) atan(x)
#define ATAN2(y, x) atan2(y, x)
#define TANH(x) tanh(x)
#define CEXP(x) cexp(x)
#define CABS(x) cabs(x)
#define CREAL(x) creal(x)
#define CIMAG(x) cimag(x)
#define CARG(x) carg(x)
#define CONJ(x) conj(x)
#define CSQRT(x) csqrt(x)
#define ABS(x) labs(x)
#define HBAR 1.0

/* Boundary / propagator selectors.  Only periodic + 2nd-order FFT exist. */
#define WF_DIRICHLET_BOUNDARY  1
#define WF_NEUMANN_BOUNDARY    2
#define WF_PERIODIC_BOUNDARY   3
#define WF_2ND_ORDER_FFT       1
#define WF_4TH_ORDER_FFT       2
#define WF_2ND_ORDER_CN        3
#define WF_4TH_ORDER_CN        4

typedef struct rgrid_struct rgrid;
typedef struct cgrid_struct cgrid;

struct rgrid_struct {
  REAL *value;               /* nx * ny * nz2 doubles */
  INT nx, ny, nz, nz2;
  REAL step;
  REAL x0, y0, z0;
  char id[32];
  char flag;                 /* claim flag (rgrid_claim/release) */
};

struct cgrid_struct {
  REAL complex *value;       /* nx * ny * nz complex */
  INT nx, ny, nz;
  REAL step;
  REAL x0, y0, z0;
  REAL kx0, ky0, kz0;        /* moving-background momentum (always 0 here) */
  char id[32];
  char flag;
};

typedef struct wf_struct {
  cgrid *grid;
  REAL mass;
  REAL norm;                 /* target norm for grid_wf_normalize() */
  char boundary;
  char propagator;
  cgrid *cworkspace;         /* scratch for propagation / kinetic energy */
  /* absorbing boundary (grid_wf_boundary): layer outside [lo, hi) per axis */
  int abs_on;
  REAL abs_amp, abs_rho0;
  INT abs_lo[3], abs_hi[3];
} wf;

typedef struct grid_timer_struct {
  double start;
} grid_timer;

typedef struct rfunction_struct rfunction;   /* opaque; not implemented */

/* Periodic boundary sentinel accepted by rgrid_alloc / cgrid_alloc. */
REAL rgrid_value_outside_periodic(rgrid *grid, INT i, INT j, INT k);
REAL complex cgrid_value_outside_periodic(cgrid *grid, INT i, INT j, INT k);
#define RGRID_PERIODIC_BOUNDARY rgrid_value_outside_periodic
#define CGRID_PERIODIC_BOUNDARY cgrid_value_outside_periodic

/* sizes (src/ot.c:75) */
char grid_sizeof_real(void);
char grid_sizeof_real_complex(void);
char grid_sizeof_int(void);

/* threads / timers / misc (examples only) */
void grid_threads_init(INT threads);
void grid_set_fftw_flags(char flags);
void grid_fft_read_wisdom(char *file);
void grid_fft_write_wisdom(char *file);
void grid_timer_start(grid_timer *timer);
REAL grid_timer_wall_clock_time(grid_timer *timer);

/* rgrid */
rgrid *rgrid_alloc(INT nx, INT ny, INT nz, REAL step, REAL (*value_outside)(rgrid *, INT, INT, INT), void *outside_params_ptr, char *id);
void rgrid_free(rgrid *grid);
rgrid *rgrid_clone(rgrid *grid, char *id);
void rgrid_set_origin(rgrid *grid, REAL x0, REAL y0, REAL z0);
void rgrid_claim(rgrid *grid);
void rgrid_release(rgrid *grid);
void rgrid_zero(rgrid *grid);
void rgrid_constant(rgrid *grid, REAL c);
void rgrid_copy(rgrid *dst, rgrid *src);
void rgrid_map(rgrid *grid, REAL (*func)(void *arg, REAL x, REAL y, REAL z), void *farg);
void rgrid_smooth_map(rgrid *grid, REAL (*func)(void *arg, REAL x, REAL y, REAL z), void *farg, INT ns);
INT rgrid_adaptive_map(rgrid *grid, REAL (*func)(void *arg, REAL x, REAL y, REAL z), void *farg, INT min_ns, INT max_ns, REAL tol);
REAL rgrid_value_at_index(rgrid *grid, INT i, INT j, INT k);
void rgrid_value_to_index(rgrid *grid, INT i, INT j, INT k, REAL value);
REAL complex rgrid_cvalue_at_index(rgrid *grid, INT i, INT j, INT k);
REAL rgrid_integral(rgrid *grid);
void rgrid_sum(rgrid *dst, rgrid *a, rgrid *b);
void rgrid_difference(rgrid *dst, rgrid *a, rgrid *b);
void rgrid_product(rgrid *dst, rgrid *a, rgrid *b);
void rgrid_multiply(rgrid *grid, REAL c);
void rgrid_add(rgrid *grid, REAL c);
void rgrid_multiply_and_add(rgrid *grid, REAL c, REAL a);
void rgrid_add_scaled(rgrid *dst, REAL c, rgrid *src);
void rgrid_add_scaled_product(rgrid *dst, REAL c, rgrid *a, rgrid *b);
void rgrid_power(rgrid *dst, rgrid *src, REAL x);
void rgrid_ipower(rgrid *dst, rgrid *src, INT n);
void rgrid_division_eps(rgrid *dst, rgrid *a, rgrid *b, REAL eps);
void rgrid_threshold_clear(rgrid *dst, rgrid *src, REAL ul, REAL ll, REAL uval, REAL lval);
void rgrid_gradient_x(rgrid *src, rgrid *dst);
void rgrid_gradient_y(rgrid *src, rgrid *dst);
void rgrid_gradient_z(rgrid *src, rgrid *dst);
void rgrid_gradient(rgrid *src, rgrid *dx, rgrid *dy, rgrid *dz);
void rgrid_fft(rgrid *grid);
void rgrid_inverse_fft(rgrid *grid);
void rgrid_inverse_fft_norm(rgrid *grid);
void rgrid_inverse_fft_norm2(rgrid *grid);
void rgrid_fft_convolute(rgrid *dst, rgrid *a, rgrid *b);
void rgrid_fft_multiply(rgrid *grid, REAL c);

/* cgrid */
cgrid *cgrid_alloc(INT nx, INT ny, INT nz, REAL step, REAL complex (*value_outside)(cgrid *, INT, INT, INT), void *outside_params_ptr, char *id);
void cgrid_free(cgrid *grid);
cgrid *cgrid_clone(cgrid *grid, char *id);
void cgrid_set_origin(cgrid *grid, REAL x0, REAL y0, REAL z0);
void cgrid_set_momentum(cgrid *grid, REAL kx0, REAL ky0, REAL kz0);
void cgrid_zero(cgrid *grid);
void cgrid_constant(cgrid *grid, REAL complex c);
void cgrid_copy(cgrid *dst, cgrid *src);
void cgrid_add(cgrid *grid, REAL complex c);
void cgrid_multiply(cgrid *grid, REAL complex c);
void cgrid_sum(cgrid *dst, cgrid *a, cgrid *b);
void cgrid_map(cgrid *grid, REAL complex (*func)(void *arg, REAL x, REAL y, REAL z), void *farg);
REAL complex cgrid_value_at_index(cgrid *grid, INT i, INT j, INT k);
void cgrid_value_to_index(cgrid *grid, INT i, INT j, INT k, REAL complex value);
REAL complex cgrid_integral(cgrid *grid);
void cgrid_fft(cgrid *grid);
void cgrid_inverse_fft(cgrid *grid);
void cgrid_inverse_fft_norm(cgrid *grid);

/* real <-> complex */
void grid_real_to_complex_re(cgrid *dst, rgrid *src);
void grid_add_real_to_complex_re(cgrid *dst, rgrid *src);
void grid_add_real_to_complex_im(cgrid *dst, rgrid *src);
void grid_complex_re_to_real(rgrid *dst, cgrid *src);
void grid_complex_im_to_real(rgrid *dst, cgrid *src);

/* wave functions */
wf *grid_wf_alloc(INT nx, INT ny, INT nz, REAL step, REAL mass, char boundary, char propagator, char *id);
wf *grid_wf_clone(wf *gwf, char *id);
void grid_wf_free(wf *gwf);
void grid_wf_map(wf *gwf, REAL complex (*func)(void *arg, REAL x, REAL y, REAL z), void *farg);
void grid_wf_constant(wf *gwf, REAL complex c);
void grid_wf_density(wf *gwf, rgrid *density);
REAL grid_wf_norm(wf *gwf);
REAL grid_wf_normalize(wf *gwf);
REAL grid_wf_energy(wf *gwf, rgrid *potential);
REAL grid_wf_kinetic_energy(wf *gwf);
REAL grid_wf_potential_energy(wf *gwf, rgrid *potential);
void grid_wf_velocity(wf *gwf, rgrid *vx, rgrid *vy, rgrid *vz, REAL eps);
void grid_wf_velocity_x(wf *gwf, rgrid *vx, REAL eps);
void grid_wf_velocity_y(wf *gwf, rgrid *vy, REAL eps);
void grid_wf_velocity_z(wf *gwf, rgrid *vz, REAL eps);
void grid_wf_propagate(wf *gwf, cgrid *potential, REAL complex time);
void grid_wf_propagate_predict(wf *gwf, wf *gwfp, cgrid *potential, REAL complex time);
void grid_wf_propagate_correct(wf *gwf, cgrid *potential, REAL complex time);
void grid_wf_propagate_potential(wf *gwf, REAL complex time, cgrid *potential, REAL cons);
void grid_wf_propagate_kinetic_fft(wf *gwf, REAL complex time);

/* libgrid routines that libdft's non-hot code references (HD / thermal
 * functionals, spline and file-driven potentials).  Not restated: they print
 * an error and abort if called. */
void grid_wf_boundary(wf *gwf, wf *gwfp, REAL amp, REAL rho0, INT lx, INT hx, INT ly, INT hy, INT lz, INT hz);
void grid_wf_absorb_potential(wf *gwf, cgrid *potential, REAL amp, REAL rho0);
void grid_func1_operate_one_product(rgrid *dst, rgrid *a, rgrid *b, REAL xi, REAL rhobf);
void grid_func2_operate_one(rgrid *dst, rgrid *src, REAL xi, REAL rhobf);
void grid_func2_operate_one_product(rgrid *dst, rgrid *a, rgrid *b, REAL xi, REAL rhobf);
void grid_func3_operate_one_product(rgrid *dst, rgrid *a, rgrid *b, REAL xi, REAL rhobf);
void grid_func4_operate_one(rgrid *dst, rgrid *src, REAL beta, REAL rhom, REAL C);
void grid_func5_operate_one(rgrid *dst, rgrid *src, REAL beta, REAL rhom, REAL C);
void grid_func6a_operate_one(rgrid *dst, rgrid *src, REAL mass, REAL temp, REAL c4);
void grid_func6b_operate_one(rgrid *dst, rgrid *src, REAL mass, REAL temp, REAL c4);
/* ideal Bose gas (the shim's restatement behind grid_func6a / 6b) */
REAL oracle_lwl3(REAL mass, REAL temp);
REAL oracle_bose_energy(REAL rho, REAL mass, REAL temp, REAL c4);
REAL oracle_bose_dEdRho(REAL rho, REAL mass, REAL temp, REAL c4);
void grid_spline_ypp(REAL *x, REAL *y, INT n, REAL yp1, REAL ypn, REAL *y2);
REAL grid_spline_interpolate(REAL *xa, REAL *ya, REAL *y2a, INT n, REAL x);
REAL grid_polynomial_interpolate(REAL *xa, REAL *ya, INT n, REAL x, REAL *dy);

/* 1-D complex FFT used by the oracle (also exported for tests). */
void oracle_fft1d(REAL complex *data, INT n, INT stride, int sign);

#endif
