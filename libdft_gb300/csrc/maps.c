/*
 * Host-side helpers libdft's drivers call around the time step: the map
 * callbacks of libdft's src/common.c and src/initial.c (shape functions and
 * initial states for rgrid_map / cgrid_map / grid_wf_map), libgrid's timer,
 * and libgrid's FFTW planning calls (no-ops here).
 *
 * The callbacks return the values the reference computes for the same
 * arguments: each evaluates its formula with the same operations in the same
 * order (compiled without FMA contraction), so results agree bit for bit with
 * libdft's own build.
 */
#define _DEFAULT_SOURCE   /* clock_gettime, M_PI */
#include <complex.h>
#include <math.h>
#include <time.h>

#include "dftgpu.h"

/* vortex-core cut-off of src/common.c:1238 and src/initial.c:29 (bohr) */
#define CORE_CUT 0.05

/* ------------------------------------------------------ shape functions */

/* 4 eps ((sig/r)^12 - (sig/r)^6) with r2 = r^2 -- src/common.c:31-39 */
REAL dft_common_lj_func(REAL r2, REAL sig, REAL eps) {
  REAL s = sig * sig / r2;
  s = s * s * s;
  return 4.0 * eps * s * (s - 1.0);
}

/* LJ with a constant core cval for r <= h -- src/common.c:53-65 */
REAL dft_common_lennard_jones(void *arg, REAL x, REAL y, REAL z) {
  const dft_common_lj *p = (const dft_common_lj *) arg;
  REAL r2 = x * x + y * y + z * z;
  if (r2 <= p->h * p->h) return p->cval;
  return dft_common_lj_func(r2, p->sigma, p->epsilon);
}

/* LJ integrated over the plane perpendicular to z, for a 1-D grid along z:
 * 2 pi eps s^6 (2 s^6 - 5 z^6) / (5 z^10), |z| clamped at h -- src/common.c:80-91 */
REAL dft_common_lennard_jones_1d(void *arg, REAL x, REAL y, REAL z) {
  const dft_common_lj *p = (const dft_common_lj *) arg;
  REAL s6 = pow(p->sigma, 6.0);
  (void) x; (void) y;
  z = fabs(z);
  if (z < p->h) z = p->h;
  return 2.0 * M_PI * p->epsilon * s6 * (2.0 * s6 - 5.0 * pow(z, 6.0)) / (5.0 * pow(z, 10.0));
}

/* LJ with the core replaced by U(h) (r/h)^4 -- src/common.c:104-116 */
REAL dft_common_lennard_jones_smooth(void *arg, REAL x, REAL y, REAL z) {
  const dft_common_lj *p = (const dft_common_lj *) arg;
  REAL h2 = p->h * p->h, r2 = x * x + y * y + z * z;
  if (r2 < h2) return dft_common_lj_func(h2, p->sigma, p->epsilon) * r2 * r2 / (h2 * h2);
  return dft_common_lj_func(r2, p->sigma, p->epsilon);
}

/* normalised step function of a sphere of radius h -- src/common.c:131-138 */
REAL dft_common_spherical_avg(void *arg, REAL x, REAL y, REAL z) {
  REAL h = *(const REAL *) arg, h2 = h * h;
  if (x * x + y * y + z * z <= h2) return 3.0 / (4.0 * M_PI * h * h2);
  return 0.0;
}

/* the sphere's step function integrated over the plane perpendicular to z:
 * 3 (h^2 - z^2) / (4 h^3) inside |z| <= h -- src/common.c:152-159 */
REAL dft_common_spherical_avg_1d(void *arg, REAL x, REAL y, REAL z) {
  REAL h = *(const REAL *) arg, h2 = h * h;
  (void) x; (void) y;
  z = fabs(z);
  if (z > h) return 0.0;
  return 3.0 * (h2 - z * z) / (4.0 * h2 * h);
}

/* its Fourier transform 3 (sin(hk) - hk cos(hk)) / (hk)^3, with the
 * second-order series below hk = 1e-5 -- src/common.c:173-180 */
REAL dft_common_spherical_avg_k(void *arg, REAL kx, REAL ky, REAL kz) {
  REAL hk = *(const REAL *) arg * sqrt(kx * kx + ky * ky + kz * kz);
  if (hk < 1.e-5) return 1.0 - 0.1 * hk * hk;
  return 3.0 * (sin(hk) - hk * cos(hk)) / (hk * hk * hk);
}

/* unit-integral Gaussian (a / sqrt(pi))^3 exp(-a^2 r^2), a = inverse width
 * -- src/common.c:193-200 */
REAL dft_common_gaussian(void *arg, REAL x, REAL y, REAL z) {
  REAL a = *(const REAL *) arg, c = 0.5 * M_2_SQRTPI * a;
  c = c * c * c;
  return c * exp(-(x * x + y * y + z * z) * a * a);
}

/* the Gaussian integrated over the plane perpendicular to z:
 * (a / sqrt(pi)) exp(-a^2 z^2) -- src/common.c:214-220 */
REAL dft_common_gaussian_1d(void *arg, REAL x, REAL y, REAL z) {
  REAL a = *(const REAL *) arg, c = 0.5 * M_2_SQRTPI * a;
  (void) x; (void) y;
  return c * exp(-z * z * a * a);
}

/* the same as a complex value -- src/common.c:235-242 */
REAL complex dft_common_cgaussian(void *arg, REAL x, REAL y, REAL z) {
  return (REAL complex) dft_common_gaussian(arg, x, y, z);
}

/* sqrt(rho) (1 + a cos(k.r)) -- src/common.c:1214-1225 */
REAL complex dft_common_planewave(void *arg, REAL x, REAL y, REAL z) {
  const dft_plane_wave *p = (const dft_plane_wave *) arg;
  REAL amp = sqrt(p->rho);
  return amp + p->a * amp * cos(p->kx * x + p->ky * y + p->kz * z);
}

/* Feynman-Onsager line potential 1 / (2 m r_perp^2), r_perp clamped at the
 * core cut-off -- src/common.c:1240-1292 (param: REAL *mass) */
static REAL line_potential(const void *param, REAL rp2) {
  if (rp2 < CORE_CUT * CORE_CUT) rp2 = CORE_CUT * CORE_CUT;
  return 1.0 / (2.0 * *(const REAL *) param * rp2);
}
REAL dft_common_vortex_x(void *param, REAL x, REAL y, REAL z) { (void) x; return line_potential(param, y * y + z * z); }
REAL dft_common_vortex_y(void *param, REAL x, REAL y, REAL z) { (void) y; return line_potential(param, x * x + z * z); }
REAL dft_common_vortex_z(void *param, REAL x, REAL y, REAL z) { (void) z; return line_potential(param, x * x + y * y); }

/* --------------------------------------------------------- initial states */

/* one quantum of circulation around an axis: (u + i v) / |(u, v)|, zero in
 * the core -- src/initial.c:31-85 */
static REAL complex vortex_n1(REAL u, REAL v) {
  REAL d = sqrt(u * u + v * v);
  if (d < CORE_CUT) return 0.0;
  return (u + I * v) / d;
}
REAL complex dft_initial_vortex_x_n1(void *na, REAL x, REAL y, REAL z) { (void) na; (void) x; return vortex_n1(y, z); }
REAL complex dft_initial_vortex_y_n1(void *na, REAL x, REAL y, REAL z) { (void) na; (void) y; return vortex_n1(x, z); }
REAL complex dft_initial_vortex_z_n1(void *na, REAL x, REAL y, REAL z) { (void) na; (void) z; return vortex_n1(x, y); }

/* two quanta: (u + i v)^2 / (u^2 + v^2).  The core test uses |(x, y)| for
 * every axis, as src/initial.c:94,115,136 do, so the x and y variants have
 * the reference's zeros. */
static REAL complex vortex_n2(REAL u, REAL v, REAL x, REAL y) {
  REAL u2 = u * u, v2 = v * v;
  REAL d = sqrt(x * x + y * y);
  if (d < CORE_CUT) return 0.0;
  return ((u2 - v2) + I * 2 * u * v) / (u2 + v2);
}
REAL complex dft_initial_vortex_x_n2(void *na, REAL x, REAL y, REAL z) { (void) na; return vortex_n2(y, z, x, y); }
REAL complex dft_initial_vortex_y_n2(void *na, REAL x, REAL y, REAL z) { (void) na; return vortex_n2(x, z, x, y); }
REAL complex dft_initial_vortex_z_n2(void *na, REAL x, REAL y, REAL z) { (void) na; return vortex_n2(x, y, x, y); }

/* 0 inside a sphere of the given radius, 1 outside -- src/initial.c:154-161 */
REAL complex dft_initial_bubble(void *prm, REAL x, REAL y, REAL z) {
  REAL r = sqrt(x * x + y * y + z * z);
  if (r < *(const REAL *) prm) return 0.0;
  return 1.0;
}

/* ------------------------------------------------------ timer, FFTW calls */

static double now_wall(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double) t.tv_sec + 1e-9 * (double) t.tv_nsec;
}

void grid_timer_start(grid_timer *timer) {
  timer->wall0 = now_wall();
  timer->cpu0 = (double) clock() / CLOCKS_PER_SEC;
}
REAL grid_timer_wall_clock_time(grid_timer *timer) { return now_wall() - timer->wall0; }
REAL grid_timer_cpu_time(grid_timer *timer) { return (double) clock() / CLOCKS_PER_SEC - timer->cpu0; }

void grid_set_fftw_flags(INT flags) { (void) flags; }
void grid_threads_init(INT threads) { (void) threads; }
void grid_fft_read_wisdom(char *file) { (void) file; }
void grid_fft_write_wisdom(char *file) { (void) file; }
