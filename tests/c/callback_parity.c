/*
 * Test helper (CPU): evaluates libdft's map callbacks from two shared
 * libraries -- libdftgpu.so and the reference-built oracle library -- at the
 * same points and reports any value whose bits differ.
 *
 *   callback_parity <libA.so> <libB.so>   -> prints "compared N values", exit 0
 *                                            when every value is bit-identical
 *
 * The libraries export the same names, so each is opened with RTLD_LOCAL and
 * its functions looked up by dlsym.
 */
#define _DEFAULT_SOURCE
#include <complex.h>
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef double (*rfn)(void *, double, double, double);
typedef double complex (*cfn)(void *, double, double, double);
typedef double (*ljfn)(double, double, double);

typedef struct { double h, sigma, epsilon, cval; } lj_params;          /* libdft dft_common_lj */
typedef struct { double kx, ky, kz, a, rho; } plane_wave;              /* libdft dft_plane_wave */

static void *lib[2];
static long compared, failed;

static void *sym(int which, const char *name) {
  void *p = dlsym(lib[which], name);
  if (!p) { fprintf(stderr, "missing %s in library %d\n", name, which); exit(2); }
  return p;
}

static int same_bits(double a, double b) { return memcmp(&a, &b, sizeof a) == 0; }

static void check(const char *name, double a, double b, double x, double y, double z) {
  compared++;
  if (!same_bits(a, b)) {
    failed++;
    if (failed < 20) fprintf(stderr, "%s(%.17g, %.17g, %.17g): %.17g vs %.17g\n", name, x, y, z, a, b);
  }
}

/* points: a lattice through the origin plus points on the core radii */
#define NP 4096
static double px[NP], py[NP], pz[NP];
static int np_used;

static void make_points(void) {
  int n = 0;
  for (int i = -7; i <= 7 && n < NP; i++)
    for (int j = -7; j <= 7 && n < NP; j++)
      for (int k = -7; k <= 7 && n < NP; k += 2) {
        px[n] = 0.73 * i; py[n] = 0.61 * j; pz[n] = 0.57 * k; n++;
      }
  const double radii[] = { 0.0, 0.05, 0.0499999, 0.0500001, 1.0, 4.1396, 4.8302, 3.5 };
  for (unsigned r = 0; r < sizeof radii / sizeof radii[0] && n + 3 <= NP; r++) {
    px[n] = radii[r]; py[n] = 0.0; pz[n] = 0.0; n++;
    px[n] = 0.0; py[n] = radii[r]; pz[n] = 0.0; n++;
    px[n] = 0.0; py[n] = 0.0; pz[n] = radii[r]; n++;
  }
  np_used = n;
}

static void real_cb(const char *name, void *arg) {
  rfn f0 = (rfn) sym(0, name), f1 = (rfn) sym(1, name);
  for (int i = 0; i < np_used; i++) check(name, f0(arg, px[i], py[i], pz[i]), f1(arg, px[i], py[i], pz[i]), px[i], py[i], pz[i]);
}

static void complex_cb(const char *name, void *arg) {
  cfn f0 = (cfn) sym(0, name), f1 = (cfn) sym(1, name);
  for (int i = 0; i < np_used; i++) {
    double complex a = f0(arg, px[i], py[i], pz[i]), b = f1(arg, px[i], py[i], pz[i]);
    check(name, creal(a), creal(b), px[i], py[i], pz[i]);
    check(name, cimag(a), cimag(b), px[i], py[i], pz[i]);
  }
}

int main(int argc, char **argv) {
  if (argc != 3) { fprintf(stderr, "usage: %s libA.so libB.so\n", argv[0]); return 2; }
  for (int i = 0; i < 2; i++) {
    lib[i] = dlopen(argv[1 + i], RTLD_NOW | RTLD_LOCAL);
    if (!lib[i]) { fprintf(stderr, "dlopen %s: %s\n", argv[1 + i], dlerror()); return 2; }
  }
  make_points();

  /* OT parameters in bohr / hartree (libdft src/ot.c:1026-1036 converted) */
  lj_params lj = { 2.1903 / 0.529177210903, 2.556 / 0.529177210903, 10.22 / 3.1577502480407E5, 0.0 };
  lj_params lj_core = lj;
  lj_core.cval = -1.5e-5;
  double radius = 2.1903 / 0.529177210903, inv_width = 1.0 / 1.1, mass = 7296.297, bubble = 3.5;
  plane_wave pw = { 0.3, -0.2, 0.45, 1e-3, 0.0218360 * 0.529177210903 * 0.529177210903 * 0.529177210903 };

  ljfn g0 = (ljfn) sym(0, "dft_common_lj_func"), g1 = (ljfn) sym(1, "dft_common_lj_func");
  for (int i = 1; i < np_used; i++) {
    double r2 = px[i] * px[i] + py[i] * py[i] + pz[i] * pz[i] + 0.25;
    check("dft_common_lj_func", g0(r2, lj.sigma, lj.epsilon), g1(r2, lj.sigma, lj.epsilon), r2, 0, 0);
  }
  real_cb("dft_common_lennard_jones", &lj);
  real_cb("dft_common_lennard_jones", &lj_core);
  real_cb("dft_common_lennard_jones_smooth", &lj);
  real_cb("dft_common_lennard_jones_1d", &lj);
  real_cb("dft_common_spherical_avg_1d", &radius);
  real_cb("dft_common_gaussian_1d", &inv_width);
  real_cb("dft_common_spherical_avg", &radius);
  real_cb("dft_common_spherical_avg_k", &radius);
  real_cb("dft_common_gaussian", &inv_width);
  real_cb("dft_common_vortex_x", &mass);
  real_cb("dft_common_vortex_y", &mass);
  real_cb("dft_common_vortex_z", &mass);
  complex_cb("dft_common_cgaussian", &inv_width);
  complex_cb("dft_common_planewave", &pw);
  complex_cb("dft_initial_vortex_x_n1", NULL);
  complex_cb("dft_initial_vortex_y_n1", NULL);
  complex_cb("dft_initial_vortex_z_n1", NULL);
  complex_cb("dft_initial_vortex_x_n2", NULL);
  complex_cb("dft_initial_vortex_y_n2", NULL);
  complex_cb("dft_initial_vortex_z_n2", NULL);
  complex_cb("dft_initial_bubble", &bubble);

  printf("compared %ld values, %ld differ\n", compared, failed);
  return failed ? 1 : 0;
}
