/*
 * CPU oracle, libgrid subset (FP64, OpenMP).  TEST INFRASTRUCTURE ONLY.
 *
 * Restates, from its mathematics, the part of jmeloranta/libgrid that
 * libdft's hot path calls (src/ot.c, src/ot-energy.c, src/helium-ot-bulk.c).
 * libgrid is not vendored in the reference and no version is pinned, so the
 * semantics are the documented choices listed in include/grid/grid.h.
 *
 * Reductions are deterministic: every row is summed sequentially and the row
 * sums are added in a fixed order, independent of the OpenMP thread count.
 * Build with -ffp-contract=off so x86 and Arm hosts round identically.
 */
#include <string.h>
#include <time.h>
#include <omp.h>
#include "grid/grid.h"
#include "grid/au.h"

/* ------------------------------------------------------------------ */
/* 1-D mixed-radix Stockham FFT                                         */
/* ------------------------------------------------------------------ */

#define MAXFAC 48
#define MAXRADIX 64

typedef struct {
  INT n;
  int nf;
  int fac[MAXFAC];
  REAL complex *tw;           /* tw[t] = exp(-2 pi i t / n) */
} fft_plan;

#define NPLANS 512   /* distinct lengths in one process (a test session visits many) */
static fft_plan plans[NPLANS];
static int nplans = 0;

static void plan_init(fft_plan *p, INT n) {
  INT m = n;
  p->n = n;
  p->nf = 0;
  while (m % 4 == 0) { p->fac[p->nf++] = 4; m /= 4; }
  while (m % 2 == 0) { p->fac[p->nf++] = 2; m /= 2; }
  while (m % 3 == 0) { p->fac[p->nf++] = 3; m /= 3; }
  while (m % 5 == 0) { p->fac[p->nf++] = 5; m /= 5; }
  for (INT f = 7; m > 1; f += 2)
    while (m % f == 0) {
      if (f > MAXRADIX) { fprintf(stderr, "oracle: FFT length " FMT_I " has a prime factor > %d\n", n, MAXRADIX); abort(); }
      p->fac[p->nf++] = (int) f; m /= f;
    }
  p->tw = (REAL complex *) malloc(sizeof(REAL complex) * (size_t) n);
  for (INT t = 0; t < n; t++) {
    /* angle reduced to [-pi, pi] before cos/sin for accuracy */
    INT tt = (t <= n / 2) ? t : t - n;
    REAL a = -2.0 * M_PI * (REAL) tt / (REAL) n;
    p->tw[t] = cos(a) + I * sin(a);
  }
}

static const fft_plan *get_plan(INT n) {
  const fft_plan *res = NULL;
#pragma omp critical(oracle_fft_plan)
  {
    for (int i = 0; i < nplans; i++)
      if (plans[i].n == n) { res = &plans[i]; break; }
    if (!res) {
      if (nplans == NPLANS) { fprintf(stderr, "oracle: too many FFT plans\n"); abort(); }
      plan_init(&plans[nplans], n);
      res = &plans[nplans];
      nplans++;
    }
  }
  return res;
}

/* In-place small DFT of length r with sign = -1 (forward) or +1 (inverse). */
static void small_dft(REAL complex *u, int r, int sign, const fft_plan *pl) {
  REAL complex a, b, c, d, e;
  REAL s = (REAL) sign;
  switch (r) {
  case 2:
    a = u[0]; b = u[1];
    u[0] = a + b; u[1] = a - b;
    return;
  case 3: {
    const REAL s3 = 0.86602540378443864676;
    a = u[0]; b = u[1]; c = u[2];
    REAL complex m = a - 0.5 * (b + c);
    REAL complex n = s3 * (b - c);
    u[0] = a + b + c;
    u[1] = m + I * s * n;
    u[2] = m - I * s * n;
    return;
  }
  case 4: {
    a = u[0]; b = u[1]; c = u[2]; d = u[3];
    REAL complex t0 = a + c, t1 = a - c, t2 = b + d, t3 = b - d;
    u[0] = t0 + t2;
    u[1] = t1 + I * s * t3;
    u[2] = t0 - t2;
    u[3] = t1 - I * s * t3;
    return;
  }
  case 5: {
    const REAL c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;
    const REAL s1 = 0.95105651629515357212, s2 = 0.58778525229247312917;
    a = u[0]; b = u[1]; c = u[2]; d = u[3]; e = u[4];
    REAL complex t1 = b + e, t2 = c + d, t3 = b - e, t4 = c - d;
    REAL complex m1 = a + c1 * t1 + c2 * t2;
    REAL complex m2 = a + c2 * t1 + c1 * t2;
    REAL complex n1 = s1 * t3 + s2 * t4;
    REAL complex n2 = s2 * t3 - s1 * t4;
    u[0] = a + t1 + t2;
    u[1] = m1 + I * s * n1;
    u[4] = m1 - I * s * n1;
    u[2] = m2 + I * s * n2;
    u[3] = m2 - I * s * n2;
    return;
  }
  default: {
    REAL complex v[MAXRADIX];
    INT step = pl->n / r;
    for (int q = 0; q < r; q++) {
      REAL complex acc = 0.0;
      for (int m = 0; m < r; m++) {
        REAL complex w = pl->tw[((INT) ((q * m) % r)) * step];
        if (sign > 0) w = conj(w);
        acc += u[m] * w;
      }
      v[q] = acc;
    }
    for (int q = 0; q < r; q++) u[q] = v[q];
    return;
  }
  }
}

/* x: n contiguous values; w: n scratch. sign -1 forward, +1 inverse. */
static void fft_contig(const fft_plan *pl, REAL complex *x, REAL complex *w, int sign) {
  INT n = pl->n, p = 1;
  REAL complex *in = x, *out = w, *tmp;
  if (n == 1) return;
  for (int s = 0; s < pl->nf; s++) {
    int r = pl->fac[s];
    INT nr = n / r, twstep = n / (p * r);
    for (INT i = 0; i < nr; i++) {
      INT k = i % p;
      REAL complex u[MAXRADIX];
      for (int q = 0; q < r; q++) {
        REAL complex v = in[i + q * nr];
        if (q && k) {
          REAL complex t = pl->tw[(q * k * twstep) % n];
          if (sign > 0) t = conj(t);
          v *= t;
        }
        u[q] = v;
      }
      small_dft(u, r, sign, pl);
      INT j = (i - k) * r + k;
      for (int q = 0; q < r; q++) out[j + q * p] = u[q];
    }
    p *= r;
    tmp = in; in = out; out = tmp;
  }
  if (in != x) memcpy(x, in, sizeof(REAL complex) * (size_t) n);
}

void oracle_fft1d(REAL complex *data, INT n, INT stride, int sign) {
  const fft_plan *pl = get_plan(n);
  REAL complex *buf = malloc(sizeof(REAL complex) * 2 * (size_t) n);
  for (INT i = 0; i < n; i++) buf[i] = data[i * stride];
  fft_contig(pl, buf, buf + n, sign);
  for (INT i = 0; i < n; i++) data[i * stride] = buf[i];
  free(buf);
}

/* Transform along one axis of a [n0][n1][n2] complex array. */
static void fft_axis(REAL complex *data, INT n0, INT n1, INT n2, int axis, int sign) {
  INT n = (axis == 0) ? n0 : (axis == 1) ? n1 : n2;
  if (n == 1) return;
  const fft_plan *pl = get_plan(n);
  INT stride = (axis == 0) ? n1 * n2 : (axis == 1) ? n2 : 1;
  INT nlines = n0 * n1 * n2 / n;
#pragma omp parallel
  {
    REAL complex *buf = malloc(sizeof(REAL complex) * 2 * (size_t) n);
#pragma omp for schedule(static)
    for (INT l = 0; l < nlines; l++) {
      INT base;
      if (axis == 2) base = l * n2;
      else if (axis == 1) base = (l / n2) * n1 * n2 + (l % n2);
      else base = l;
      REAL complex *p = data + base;
      for (INT i = 0; i < n; i++) buf[i] = p[i * stride];
      fft_contig(pl, buf, buf + n, sign);
      for (INT i = 0; i < n; i++) p[i * stride] = buf[i];
    }
    free(buf);
  }
}

/* ------------------------------------------------------------------ */
/* misc                                                                 */
/* ------------------------------------------------------------------ */

REAL rgrid_value_outside_periodic(rgrid *grid, INT i, INT j, INT k) {
  INT nx = grid->nx, ny = grid->ny, nz = grid->nz;
  i %= nx; if (i < 0) i += nx;
  j %= ny; if (j < 0) j += ny;
  k %= nz; if (k < 0) k += nz;
  return grid->value[(i * ny + j) * grid->nz2 + k];
}

REAL complex cgrid_value_outside_periodic(cgrid *grid, INT i, INT j, INT k) {
  INT nx = grid->nx, ny = grid->ny, nz = grid->nz;
  i %= nx; if (i < 0) i += nx;
  j %= ny; if (j < 0) j += ny;
  k %= nz; if (k < 0) k += nz;
  return grid->value[(i * ny + j) * nz + k];
}

char grid_sizeof_real(void) { return (char) sizeof(REAL); }
char grid_sizeof_real_complex(void) { return (char) sizeof(REAL complex); }
char grid_sizeof_int(void) { return (char) sizeof(INT); }
void grid_threads_init(INT threads) { if (threads > 0) omp_set_num_threads((int) threads); }
void grid_set_fftw_flags(char flags) { (void) flags; }
void grid_fft_read_wisdom(char *file) { (void) file; }
void grid_fft_write_wisdom(char *file) { (void) file; }

void grid_timer_start(grid_timer *timer) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  timer->start = (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

REAL grid_timer_wall_clock_time(grid_timer *timer) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec - timer->start;
}

static void not_restated(const char *name) {
  fprintf(stderr, "oracle: %s is outside the restated libgrid subset.\n", name);
  abort();
}


void grid_spline_ypp(REAL *x, REAL *y, INT n, REAL yp1, REAL ypn, REAL *y2) { (void) x; (void) y; (void) n; (void) yp1; (void) ypn; (void) y2; not_restated("grid_spline_ypp"); }
REAL grid_spline_interpolate(REAL *xa, REAL *ya, REAL *y2a, INT n, REAL x) { (void) xa; (void) ya; (void) y2a; (void) n; (void) x; not_restated("grid_spline_interpolate"); return 0.0; }
REAL grid_polynomial_interpolate(REAL *xa, REAL *ya, INT n, REAL x, REAL *dy) { (void) xa; (void) ya; (void) n; (void) x; (void) dy; not_restated("grid_polynomial_interpolate"); return 0.0; }

/* ------------------------------------------------------------------ */
/* rgrid                                                                */
/* ------------------------------------------------------------------ */

#define RIDX(g, i, j, k) ((((i) * (g)->ny + (j)) * (g)->nz2) + (k))

rgrid *rgrid_alloc(INT nx, INT ny, INT nz, REAL step, REAL (*value_outside)(rgrid *, INT, INT, INT), void *outside_params_ptr, char *id) {
  (void) value_outside; (void) outside_params_ptr;
  rgrid *g = (rgrid *) calloc(1, sizeof(rgrid));
  if (!g) return NULL;
  g->nx = nx; g->ny = ny; g->nz = nz;
  g->nz2 = 2 * (nz / 2 + 1);
  g->step = step;
  g->value = (REAL *) calloc((size_t) (nx * ny * g->nz2), sizeof(REAL));
  if (!g->value) { free(g); return NULL; }
  if (id) { strncpy(g->id, id, sizeof(g->id) - 1); }
  return g;
}

void rgrid_free(rgrid *g) { if (g) { free(g->value); free(g); } }

rgrid *rgrid_clone(rgrid *g, char *id) {
  rgrid *c = rgrid_alloc(g->nx, g->ny, g->nz, g->step, RGRID_PERIODIC_BOUNDARY, NULL, id);
  if (c) { c->x0 = g->x0; c->y0 = g->y0; c->z0 = g->z0; }
  return c;
}

void rgrid_set_origin(rgrid *g, REAL x0, REAL y0, REAL z0) { g->x0 = x0; g->y0 = y0; g->z0 = z0; }
void rgrid_claim(rgrid *g) { if (g->flag) { fprintf(stderr, "oracle: grid %s claimed twice.\n", g->id); abort(); } g->flag = 1; }
void rgrid_release(rgrid *g) { g->flag = 0; }

void rgrid_zero(rgrid *g) { memset(g->value, 0, sizeof(REAL) * (size_t) (g->nx * g->ny * g->nz2)); }

#define RLOOP(g) \
  _Pragma("omp parallel for schedule(static)") \
  for (INT ij = 0; ij < (g)->nx * (g)->ny; ij++) \
    for (INT k = 0; k < (g)->nz; k++)

#define RAT(g) ((g)->value[ij * (g)->nz2 + k])

void rgrid_constant(rgrid *g, REAL c) { RLOOP(g) RAT(g) = c; }

/* High-density terms (libgrid grid_func1..5; not in the reference tree).
 * Restated from the published functional -- a documented choice, parity is
 * unpinned at this boundary:
 *   Barranco et al., PRB 72, 214522 (2005) (cited at src/ot.h:142-146):
 *     E_HD(rho) = C rho [1 + tanh(beta (rho - rho_m))]                   (func5)
 *     V_HD(rho) = dE_HD/drho = C [1 + tanh(t)] + C beta rho sech^2(t),
 *                 t = beta (rho - rho_m)                                  (func4)
 *   backflow density cut-off (src/ot.c:1234-1236): rho -> rho G(rho),
 *     G(rho) = [1 - tanh(xi (rho - rho_bf))] / 2  (1 below rho_bf, 0 above),
 *     func1 = G, func2 = rho G, func3 = d(rho G)/drho = G + rho G'. */
static REAL hd_sech2(REAL t) { REAL c = cosh(t); return 1.0 / (c * c); }   /* 0 once cosh overflows */
static REAL bf_cut(REAL r, REAL xi, REAL rbf) { return 0.5 * (1.0 - tanh(xi * (r - rbf))); }
static REAL bf_cut_d(REAL r, REAL xi, REAL rbf) { return -0.5 * xi * hd_sech2(xi * (r - rbf)); }

void grid_func1_operate_one_product(rgrid *d, rgrid *a, rgrid *b, REAL xi, REAL rbf) {
  RLOOP(d) RAT(d) = RAT(a) * bf_cut(RAT(b), xi, rbf);
}
void grid_func2_operate_one(rgrid *d, rgrid *s, REAL xi, REAL rbf) {
  RLOOP(d) { REAL r = RAT(s); RAT(d) = r * bf_cut(r, xi, rbf); }
}
void grid_func2_operate_one_product(rgrid *d, rgrid *a, rgrid *b, REAL xi, REAL rbf) {
  RLOOP(d) { REAL r = RAT(b); RAT(d) = RAT(a) * (r * bf_cut(r, xi, rbf)); }
}
void grid_func3_operate_one_product(rgrid *d, rgrid *a, rgrid *b, REAL xi, REAL rbf) {
  RLOOP(d) { REAL r = RAT(b); RAT(d) = RAT(a) * (bf_cut(r, xi, rbf) + r * bf_cut_d(r, xi, rbf)); }
}
void grid_func4_operate_one(rgrid *d, rgrid *s, REAL beta, REAL rhom, REAL C) {
  RLOOP(d) { REAL r = RAT(s), t = beta * (r - rhom); RAT(d) = C * (1.0 + tanh(t)) + C * beta * r * hd_sech2(t); }
}
void grid_func5_operate_one(rgrid *d, rgrid *s, REAL beta, REAL rhom, REAL C) {
  RLOOP(d) { REAL r = RAT(s); RAT(d) = C * r * (1.0 + tanh(beta * (r - rhom))); }
}
void rgrid_copy(rgrid *dst, rgrid *src) { memcpy(dst->value, src->value, sizeof(REAL) * (size_t) (src->nx * src->ny * src->nz2)); }
void rgrid_sum(rgrid *d, rgrid *a, rgrid *b) { RLOOP(d) RAT(d) = RAT(a) + RAT(b); }
void rgrid_difference(rgrid *d, rgrid *a, rgrid *b) { RLOOP(d) RAT(d) = RAT(a) - RAT(b); }
void rgrid_product(rgrid *d, rgrid *a, rgrid *b) { RLOOP(d) RAT(d) = RAT(a) * RAT(b); }
void rgrid_multiply(rgrid *g, REAL c) { RLOOP(g) RAT(g) *= c; }
void rgrid_add(rgrid *g, REAL c) { RLOOP(g) RAT(g) += c; }
void rgrid_multiply_and_add(rgrid *g, REAL c, REAL a) { RLOOP(g) RAT(g) = RAT(g) * c + a; }
void rgrid_add_scaled(rgrid *d, REAL c, rgrid *s) { RLOOP(d) RAT(d) += c * RAT(s); }
void rgrid_add_scaled_product(rgrid *d, REAL c, rgrid *a, rgrid *b) { RLOOP(d) RAT(d) += c * RAT(a) * RAT(b); }
void rgrid_power(rgrid *d, rgrid *s, REAL x) { RLOOP(d) RAT(d) = pow(RAT(s), x); }

void rgrid_ipower(rgrid *d, rgrid *s, INT n) {
  RLOOP(d) {
    REAL v = RAT(s), r = 1.0;
    if (n >= 0) { for (INT m = 0; m < n; m++) r *= v; }
    else { for (INT m = 0; m < -n; m++) r *= v; r = 1.0 / r; }
    RAT(d) = r;
  }
}

void rgrid_division_eps(rgrid *d, rgrid *a, rgrid *b, REAL eps) {
  RLOOP(d) { REAL den = RAT(b); if (den < eps) den = eps; RAT(d) = RAT(a) / den; }
}

void rgrid_threshold_clear(rgrid *d, rgrid *s, REAL ul, REAL ll, REAL uval, REAL lval) {
  RLOOP(d) { REAL v = RAT(s); if (v > ul) v = uval; else if (v < ll) v = lval; RAT(d) = v; }
}

REAL rgrid_value_at_index(rgrid *g, INT i, INT j, INT k) { return rgrid_value_outside_periodic(g, i, j, k); }
void rgrid_value_to_index(rgrid *g, INT i, INT j, INT k, REAL v) { g->value[RIDX(g, i, j, k)] = v; }

REAL complex rgrid_cvalue_at_index(rgrid *g, INT i, INT j, INT k) {
  REAL complex *c = (REAL complex *) g->value;
  return c[(i * g->ny + j) * (g->nz / 2 + 1) + k];
}

static REAL row_sum_det(const REAL *rowsums, INT n) {
  REAL s = 0.0;
  for (INT i = 0; i < n; i++) s += rowsums[i];
  return s;
}

REAL rgrid_integral(rgrid *g) {
  INT nr = g->nx * g->ny;
  REAL *rs = malloc(sizeof(REAL) * (size_t) nr);
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nr; ij++) {
    REAL s = 0.0;
    for (INT k = 0; k < g->nz; k++) s += g->value[ij * g->nz2 + k];
    rs[ij] = s;
  }
  REAL s = row_sum_det(rs, nr);
  free(rs);
  return s * g->step * g->step * g->step;
}

void rgrid_map(rgrid *g, REAL (*func)(void *, REAL, REAL, REAL), void *farg) {
  INT nx = g->nx, ny = g->ny, nz = g->nz;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL x = (REAL) (i - nx / 2) * g->step - g->x0;
    REAL y = (REAL) (j - ny / 2) * g->step - g->y0;
    for (INT k = 0; k < nz; k++) {
      REAL z = (REAL) (k - nz / 2) * g->step - g->z0;
      g->value[ij * g->nz2 + k] = func(farg, x, y, z);
    }
  }
}

/* Average of func over ns^3 cell-centred sub-points of the cell at (x,y,z). */
static REAL cell_average(REAL (*func)(void *, REAL, REAL, REAL), void *farg, REAL x, REAL y, REAL z, REAL step, INT ns) {
  REAL sum = 0.0, h = step / (REAL) ns;
  for (INT a = 0; a < ns; a++) {
    REAL xs = x + ((REAL) a + 0.5) * h - 0.5 * step;
    for (INT b = 0; b < ns; b++) {
      REAL ys = y + ((REAL) b + 0.5) * h - 0.5 * step;
      for (INT c = 0; c < ns; c++) {
        REAL zs = z + ((REAL) c + 0.5) * h - 0.5 * step;
        sum += func(farg, xs, ys, zs);
      }
    }
  }
  return sum / (REAL) (ns * ns * ns);
}

void rgrid_smooth_map(rgrid *g, REAL (*func)(void *, REAL, REAL, REAL), void *farg, INT ns) {
  INT nx = g->nx, ny = g->ny, nz = g->nz;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL x = (REAL) (i - nx / 2) * g->step - g->x0;
    REAL y = (REAL) (j - ny / 2) * g->step - g->y0;
    for (INT k = 0; k < nz; k++) {
      REAL z = (REAL) (k - nz / 2) * g->step - g->z0;
      g->value[ij * g->nz2 + k] = cell_average(func, farg, x, y, z, g->step, ns);
    }
  }
}

INT rgrid_adaptive_map(rgrid *g, REAL (*func)(void *, REAL, REAL, REAL), void *farg, INT min_ns, INT max_ns, REAL tol) {
  INT nx = g->nx, ny = g->ny, nz = g->nz, maxused = min_ns;
#pragma omp parallel for schedule(dynamic, 4) reduction(max:maxused)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL x = (REAL) (i - nx / 2) * g->step - g->x0;
    REAL y = (REAL) (j - ny / 2) * g->step - g->y0;
    for (INT k = 0; k < nz; k++) {
      REAL z = (REAL) (k - nz / 2) * g->step - g->z0;
      INT ns = min_ns;
      REAL v = cell_average(func, farg, x, y, z, g->step, ns);
      while (2 * ns <= max_ns) {
        REAL v2 = cell_average(func, farg, x, y, z, g->step, 2 * ns);
        ns *= 2;
        REAL diff = v2 - v;
        v = v2;
        if (fabs(diff) < tol) break;
      }
      if (ns > maxused) maxused = ns;
      g->value[ij * g->nz2 + k] = v;
    }
  }
  return maxused;
}

/* Second-order central difference along one axis, periodic. */
static void rgrid_fd(rgrid *src, rgrid *dst, int axis) {
  INT nx = src->nx, ny = src->ny, nz = src->nz;
  REAL inv2h = 1.0 / (2.0 * src->step);
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    for (INT k = 0; k < nz; k++) {
      REAL p, m;
      if (axis == 0) {
        p = src->value[RIDX(src, (i + 1) % nx, j, k)];
        m = src->value[RIDX(src, (i - 1 + nx) % nx, j, k)];
      } else if (axis == 1) {
        p = src->value[RIDX(src, i, (j + 1) % ny, k)];
        m = src->value[RIDX(src, i, (j - 1 + ny) % ny, k)];
      } else {
        p = src->value[RIDX(src, i, j, (k + 1) % nz)];
        m = src->value[RIDX(src, i, j, (k - 1 + nz) % nz)];
      }
      dst->value[RIDX(dst, i, j, k)] = (p - m) * inv2h;
    }
  }
}

void rgrid_gradient_x(rgrid *s, rgrid *d) { if (s->nx == 1) rgrid_zero(d); else rgrid_fd(s, d, 0); }
void rgrid_gradient_y(rgrid *s, rgrid *d) { if (s->ny == 1) rgrid_zero(d); else rgrid_fd(s, d, 1); }
void rgrid_gradient_z(rgrid *s, rgrid *d) { if (s->nz == 1) rgrid_zero(d); else rgrid_fd(s, d, 2); }
void rgrid_gradient(rgrid *s, rgrid *dx, rgrid *dy, rgrid *dz) { rgrid_gradient_x(s, dx); rgrid_gradient_y(s, dy); rgrid_gradient_z(s, dz); }

/* r2c along z in place, then c2c along y and x on the half spectrum. */
void rgrid_fft(rgrid *g) {
  INT nx = g->nx, ny = g->ny, nz = g->nz, nzh = nz / 2 + 1;
  const fft_plan *pl = get_plan(nz);
#pragma omp parallel
  {
    REAL complex *buf = malloc(sizeof(REAL complex) * 2 * (size_t) nz);
#pragma omp for schedule(static)
    for (INT ij = 0; ij < nx * ny; ij++) {
      REAL *row = g->value + ij * g->nz2;
      for (INT k = 0; k < nz; k++) buf[k] = row[k];
      fft_contig(pl, buf, buf + nz, -1);
      REAL complex *crow = (REAL complex *) row;
      for (INT k = 0; k < nzh; k++) crow[k] = buf[k];
    }
    free(buf);
  }
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 1, -1);
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 0, -1);
}

void rgrid_inverse_fft(rgrid *g) {
  INT nx = g->nx, ny = g->ny, nz = g->nz, nzh = nz / 2 + 1;
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 0, +1);
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 1, +1);
  const fft_plan *pl = get_plan(nz);
#pragma omp parallel
  {
    REAL complex *buf = malloc(sizeof(REAL complex) * 2 * (size_t) nz);
#pragma omp for schedule(static)
    for (INT ij = 0; ij < nx * ny; ij++) {
      REAL complex *crow = (REAL complex *) (g->value + ij * g->nz2);
      for (INT k = 0; k < nzh; k++) buf[k] = crow[k];
      for (INT k = nzh; k < nz; k++) buf[k] = conj(buf[nz - k]);
      fft_contig(pl, buf, buf + nz, +1);
      REAL *row = (REAL *) crow;
      for (INT k = 0; k < nz; k++) row[k] = creal(buf[k]);
    }
    free(buf);
  }
}

static void rgrid_scale_real(rgrid *g, REAL c) { RLOOP(g) RAT(g) *= c; }

void rgrid_inverse_fft_norm(rgrid *g) {
  rgrid_inverse_fft(g);
  rgrid_scale_real(g, 1.0 / (REAL) (g->nx * g->ny * g->nz));
}

/* Inverse transform of a convolution, times the volume element over N.  A
 * grid with one point across x and y (libdft's 1-D effective model, whose
 * kernels are already integrated over the x-y plane, src/ot.c:133-217) takes
 * the line element dz = step instead of step^3: this is the measure under
 * which the uniform liquid keeps its bulk chemical potential. */
void rgrid_inverse_fft_norm2(rgrid *g) {
  rgrid_inverse_fft(g);
  const REAL dv = (g->nx == 1 && g->ny == 1) ? g->step : g->step * g->step * g->step;
  rgrid_scale_real(g, dv / (REAL) (g->nx * g->ny * g->nz));
}

/* Product of two spectra times the centring phase: the kernel operand was
 * sampled about index c = n/2 of each axis (x_i = (i - n/2) step), and the
 * kernel about index 0 has the spectrum times exp(2 pi i k c / n) per axis --
 * the sign (-1)^k for even n, a rotation for odd n (odd x and y sizes). */
static REAL complex centring_phase(INT k, INT n) {
  if (!(n & 1)) return (k & 1) ? -1.0 : 1.0;
  const REAL ang = 2.0 * M_PI * (REAL) ((k * (n / 2)) % n) / (REAL) n;
  return cos(ang) + I * sin(ang);
}

void rgrid_fft_convolute(rgrid *d, rgrid *a, rgrid *b) {
  INT nx = d->nx, ny = d->ny, nzh = d->nz / 2 + 1;
  REAL complex *cd = (REAL complex *) d->value, *ca = (REAL complex *) a->value, *cb = (REAL complex *) b->value;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL complex pxy = centring_phase(i, nx) * centring_phase(j, ny);
    for (INT k = 0; k < nzh; k++) {
      INT idx = ij * nzh + k;
      REAL complex v = ca[idx] * cb[idx] * pxy;
      cd[idx] = (k & 1) ? -v : v;
    }
  }
}

void rgrid_fft_multiply(rgrid *g, REAL c) {
  INT n = g->nx * g->ny * (g->nz / 2 + 1);
  REAL complex *cv = (REAL complex *) g->value;
#pragma omp parallel for schedule(static)
  for (INT i = 0; i < n; i++) cv[i] *= c;
}

/* ------------------------------------------------------------------ */
/* cgrid                                                                */
/* ------------------------------------------------------------------ */

cgrid *cgrid_alloc(INT nx, INT ny, INT nz, REAL step, REAL complex (*value_outside)(cgrid *, INT, INT, INT), void *outside_params_ptr, char *id) {
  (void) value_outside; (void) outside_params_ptr;
  cgrid *g = (cgrid *) calloc(1, sizeof(cgrid));
  if (!g) return NULL;
  g->nx = nx; g->ny = ny; g->nz = nz; g->step = step;
  g->value = (REAL complex *) calloc((size_t) (nx * ny * nz), sizeof(REAL complex));
  if (!g->value) { free(g); return NULL; }
  if (id) strncpy(g->id, id, sizeof(g->id) - 1);
  return g;
}

void cgrid_free(cgrid *g) { if (g) { free(g->value); free(g); } }

cgrid *cgrid_clone(cgrid *g, char *id) {
  cgrid *c = cgrid_alloc(g->nx, g->ny, g->nz, g->step, CGRID_PERIODIC_BOUNDARY, NULL, id);
  if (c) { c->x0 = g->x0; c->y0 = g->y0; c->z0 = g->z0; c->kx0 = g->kx0; c->ky0 = g->ky0; c->kz0 = g->kz0; }
  return c;
}

void cgrid_set_origin(cgrid *g, REAL x0, REAL y0, REAL z0) { g->x0 = x0; g->y0 = y0; g->z0 = z0; }

/* Moving background (called by examples/gas-bubble/bubble.c:104,173,
 * examples/added_mass/added_mass.c:78, examples/1d-bubble/bubble-1d.c:136).
 * Restated semantics: the wave function is stored in the frame moving with
 * momentum hbar k0, where the kinetic operator is hbar^2 |k - k0|^2 / 2m; it
 * enters the kinetic propagator and the kinetic energy of the wave function
 * whose grid carries it, and nothing else (the OT terms depend on the density
 * and on velocity differences only). */
void cgrid_set_momentum(cgrid *g, REAL kx0, REAL ky0, REAL kz0) {
  g->kx0 = kx0; g->ky0 = ky0; g->kz0 = kz0;
}

#define CN(g) ((g)->nx * (g)->ny * (g)->nz)
#define CLOOP(g) _Pragma("omp parallel for schedule(static)") for (INT ii = 0; ii < CN(g); ii++)

void cgrid_zero(cgrid *g) { memset(g->value, 0, sizeof(REAL complex) * (size_t) CN(g)); }
void cgrid_constant(cgrid *g, REAL complex c) { CLOOP(g) g->value[ii] = c; }
void cgrid_copy(cgrid *d, cgrid *s) { memcpy(d->value, s->value, sizeof(REAL complex) * (size_t) CN(s)); }
void cgrid_add(cgrid *g, REAL complex c) { CLOOP(g) g->value[ii] += c; }
void cgrid_multiply(cgrid *g, REAL complex c) { CLOOP(g) g->value[ii] *= c; }
void cgrid_sum(cgrid *d, cgrid *a, cgrid *b) { CLOOP(d) d->value[ii] = a->value[ii] + b->value[ii]; }

void cgrid_map(cgrid *g, REAL complex (*func)(void *, REAL, REAL, REAL), void *farg) {
  INT nx = g->nx, ny = g->ny, nz = g->nz;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL x = (REAL) (i - nx / 2) * g->step - g->x0;
    REAL y = (REAL) (j - ny / 2) * g->step - g->y0;
    for (INT k = 0; k < nz; k++) {
      REAL z = (REAL) (k - nz / 2) * g->step - g->z0;
      g->value[ij * nz + k] = func(farg, x, y, z);
    }
  }
}

REAL complex cgrid_value_at_index(cgrid *g, INT i, INT j, INT k) { return cgrid_value_outside_periodic(g, i, j, k); }
void cgrid_value_to_index(cgrid *g, INT i, INT j, INT k, REAL complex v) { g->value[(i * g->ny + j) * g->nz + k] = v; }

REAL complex cgrid_integral(cgrid *g) {
  INT nr = g->nx * g->ny, nz = g->nz;
  REAL *rs = malloc(sizeof(REAL) * 2 * (size_t) nr);
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nr; ij++) {
    REAL sr = 0.0, si = 0.0;
    for (INT k = 0; k < nz; k++) { sr += creal(g->value[ij * nz + k]); si += cimag(g->value[ij * nz + k]); }
    rs[2 * ij] = sr; rs[2 * ij + 1] = si;
  }
  REAL sr = 0.0, si = 0.0;
  for (INT ij = 0; ij < nr; ij++) { sr += rs[2 * ij]; si += rs[2 * ij + 1]; }
  free(rs);
  REAL dv = g->step * g->step * g->step;
  return (sr + I * si) * dv;
}

void cgrid_fft(cgrid *g) {
  fft_axis(g->value, g->nx, g->ny, g->nz, 2, -1);
  fft_axis(g->value, g->nx, g->ny, g->nz, 1, -1);
  fft_axis(g->value, g->nx, g->ny, g->nz, 0, -1);
}

void cgrid_inverse_fft(cgrid *g) {
  fft_axis(g->value, g->nx, g->ny, g->nz, 0, +1);
  fft_axis(g->value, g->nx, g->ny, g->nz, 1, +1);
  fft_axis(g->value, g->nx, g->ny, g->nz, 2, +1);
}

void cgrid_inverse_fft_norm(cgrid *g) {
  cgrid_inverse_fft(g);
  REAL c = 1.0 / (REAL) CN(g);
  CLOOP(g) g->value[ii] *= c;
}

/* ------------------------------------------------------------------ */
/* real <-> complex                                                     */
/* ------------------------------------------------------------------ */

void grid_real_to_complex_re(cgrid *d, rgrid *s) {
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < s->nx * s->ny; ij++)
    for (INT k = 0; k < s->nz; k++) d->value[ij * d->nz + k] = s->value[ij * s->nz2 + k];
}

void grid_add_real_to_complex_re(cgrid *d, rgrid *s) {
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < s->nx * s->ny; ij++)
    for (INT k = 0; k < s->nz; k++) d->value[ij * d->nz + k] += s->value[ij * s->nz2 + k];
}

void grid_add_real_to_complex_im(cgrid *d, rgrid *s) {
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < s->nx * s->ny; ij++)
    for (INT k = 0; k < s->nz; k++) d->value[ij * d->nz + k] += I * s->value[ij * s->nz2 + k];
}

void grid_complex_re_to_real(rgrid *d, cgrid *s) {
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < s->nx * s->ny; ij++)
    for (INT k = 0; k < s->nz; k++) d->value[ij * d->nz2 + k] = creal(s->value[ij * s->nz + k]);
}

void grid_complex_im_to_real(rgrid *d, cgrid *s) {
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < s->nx * s->ny; ij++)
    for (INT k = 0; k < s->nz; k++) d->value[ij * d->nz2 + k] = cimag(s->value[ij * s->nz + k]);
}

/* ------------------------------------------------------------------ */
/* wave functions                                                       */
/* ------------------------------------------------------------------ */

wf *grid_wf_alloc(INT nx, INT ny, INT nz, REAL step, REAL mass, char boundary, char propagator, char *id) {
  if (boundary != WF_PERIODIC_BOUNDARY || (propagator != WF_2ND_ORDER_FFT && propagator != WF_2ND_ORDER_CN)) {
    fprintf(stderr, "oracle: only periodic boundaries with the 2nd-order FFT or CN propagator are restated.\n");
    return NULL;
  }
  wf *w = (wf *) calloc(1, sizeof(wf));
  if (!w) return NULL;
  w->grid = cgrid_alloc(nx, ny, nz, step, CGRID_PERIODIC_BOUNDARY, NULL, id);
  if (!w->grid) { free(w); return NULL; }
  w->mass = mass;
  w->norm = 1.0;
  w->boundary = boundary;
  w->propagator = propagator;
  w->cworkspace = NULL;
  return w;
}

wf *grid_wf_clone(wf *g, char *id) {
  wf *w = grid_wf_alloc(g->grid->nx, g->grid->ny, g->grid->nz, g->grid->step, g->mass, g->boundary, g->propagator, id);
  if (!w) return NULL;
  w->norm = g->norm;
  cgrid_set_origin(w->grid, g->grid->x0, g->grid->y0, g->grid->z0);
  return w;
}

void grid_wf_free(wf *g) {
  if (!g) return;
  cgrid_free(g->grid);
  if (g->cworkspace) cgrid_free(g->cworkspace);
  free(g);
}

void grid_wf_map(wf *g, REAL complex (*func)(void *, REAL, REAL, REAL), void *farg) { cgrid_map(g->grid, func, farg); }
void grid_wf_constant(wf *g, REAL complex c) { cgrid_constant(g->grid, c); }

void grid_wf_density(wf *g, rgrid *d) {
  cgrid *c = g->grid;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < c->nx * c->ny; ij++)
    for (INT k = 0; k < c->nz; k++) {
      REAL complex v = c->value[ij * c->nz + k];
      d->value[ij * d->nz2 + k] = creal(v) * creal(v) + cimag(v) * cimag(v);
    }
}

REAL grid_wf_norm(wf *g) {
  cgrid *c = g->grid;
  INT nr = c->nx * c->ny;
  REAL *rs = malloc(sizeof(REAL) * (size_t) nr);
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nr; ij++) {
    REAL s = 0.0;
    for (INT k = 0; k < c->nz; k++) {
      REAL complex v = c->value[ij * c->nz + k];
      s += creal(v) * creal(v) + cimag(v) * cimag(v);
    }
    rs[ij] = s;
  }
  REAL s = row_sum_det(rs, nr);
  free(rs);
  return s * c->step * c->step * c->step;
}

REAL grid_wf_normalize(wf *g) {
  REAL n = grid_wf_norm(g);
  REAL f = sqrt(g->norm / n);
  cgrid_multiply(g->grid, f);
  return f;
}

static cgrid *wf_workspace(wf *g) {
  if (!g->cworkspace) g->cworkspace = cgrid_clone(g->grid, "wf workspace");
  return g->cworkspace;
}

/* k_i = 2 pi (i or i - n) / (n step), with the Nyquist index i = n/2 taken as -n/2. */
static inline REAL kval(INT i, INT n, REAL step) {
  INT m = (i < (n + 1) / 2) ? i : i - n;
  return 2.0 * M_PI * (REAL) m / ((REAL) n * step);
}

/* The kinetic operator's value along one axis at wave number k: k^2 for the
 * FFT propagator; for WF_2ND_ORDER_CN the eigenvalue (2 sin(k h / 2) / h)^2 of
 * the periodic second difference -(f[j+1] - 2 f[j] + f[j-1]) / h^2, the
 * finite-difference operator that propagator steps with (libgrid's CN
 * propagator is absent; this is the restatement both sides share). */
static inline REAL kin_axis(REAL k, REAL h, int cn) {
  if (!cn) return k * k;
  REAL s = 2.0 * sin(0.5 * k * h) / h;
  return s * s;
}

REAL grid_wf_kinetic_energy(wf *g) {
  cgrid *c = g->grid, *w = wf_workspace(g);
  INT nx = c->nx, ny = c->ny, nz = c->nz, nr = nx * ny;
  int cn = g->propagator == WF_2ND_ORDER_CN;
  REAL h = c->step;
  cgrid_copy(w, c);
  cgrid_fft(w);
  REAL *rs = malloc(sizeof(REAL) * (size_t) nr);
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nr; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL qxy = kin_axis(kval(i, nx, h) - c->kx0, h, cn) + kin_axis(kval(j, ny, h) - c->ky0, h, cn), s = 0.0;
    for (INT k = 0; k < nz; k++) {
      REAL q = qxy + kin_axis(kval(k, nz, h) - c->kz0, h, cn);
      REAL complex v = w->value[ij * nz + k];
      s += q * (creal(v) * creal(v) + cimag(v) * cimag(v));
    }
    rs[ij] = s;
  }
  REAL s = row_sum_det(rs, nr);
  free(rs);
  REAL dv = c->step * c->step * c->step;
  return HBAR * HBAR / (2.0 * g->mass) * s * dv / (REAL) (nx * ny * nz);
}

REAL grid_wf_potential_energy(wf *g, rgrid *pot) {
  cgrid *c = g->grid;
  INT nr = c->nx * c->ny;
  REAL *rs = malloc(sizeof(REAL) * (size_t) nr);
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nr; ij++) {
    REAL s = 0.0;
    for (INT k = 0; k < c->nz; k++) {
      REAL complex v = c->value[ij * c->nz + k];
      s += (creal(v) * creal(v) + cimag(v) * cimag(v)) * pot->value[ij * pot->nz2 + k];
    }
    rs[ij] = s;
  }
  REAL s = row_sum_det(rs, nr);
  free(rs);
  return s * c->step * c->step * c->step;
}

REAL grid_wf_energy(wf *g, rgrid *pot) {
  REAL e = grid_wf_kinetic_energy(g);
  if (pot) e += grid_wf_potential_energy(g, pot);
  return e;
}

static void wf_velocity_axis(wf *g, rgrid *v, REAL eps, int axis) {
  cgrid *c = g->grid;
  INT nx = c->nx, ny = c->ny, nz = c->nz;
  REAL f = HBAR / (g->mass * 2.0 * c->step);
  INT n = (axis == 0) ? nx : (axis == 1) ? ny : nz;
  if (n == 1) { rgrid_zero(v); return; }
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    for (INT k = 0; k < nz; k++) {
      REAL complex p, m, z = c->value[ij * nz + k];
      if (axis == 0) { p = c->value[(((i + 1) % nx) * ny + j) * nz + k]; m = c->value[(((i - 1 + nx) % nx) * ny + j) * nz + k]; }
      else if (axis == 1) { p = c->value[(i * ny + (j + 1) % ny) * nz + k]; m = c->value[(i * ny + (j - 1 + ny) % ny) * nz + k]; }
      else { p = c->value[ij * nz + (k + 1) % nz]; m = c->value[ij * nz + (k - 1 + nz) % nz]; }
      REAL complex d = p - m;
      REAL flux = creal(z) * cimag(d) - cimag(z) * creal(d);   /* Im(conj(z) d) */
      REAL rho = creal(z) * creal(z) + cimag(z) * cimag(z);
      if (rho < eps) rho = eps;
      v->value[ij * v->nz2 + k] = f * flux / rho;
    }
  }
}

void grid_wf_velocity_x(wf *g, rgrid *v, REAL eps) { wf_velocity_axis(g, v, eps, 0); }
void grid_wf_velocity_y(wf *g, rgrid *v, REAL eps) { wf_velocity_axis(g, v, eps, 1); }
void grid_wf_velocity_z(wf *g, rgrid *v, REAL eps) { wf_velocity_axis(g, v, eps, 2); }
void grid_wf_velocity(wf *g, rgrid *vx, rgrid *vy, rgrid *vz, REAL eps) {
  wf_velocity_axis(g, vx, eps, 0); wf_velocity_axis(g, vy, eps, 1); wf_velocity_axis(g, vz, eps, 2);
}

/* dst = exp(-i V dt / 2) src, elementwise */
static void apply_potential_half(cgrid *dst, cgrid *src, cgrid *pot, REAL complex dt) {
  INT n = CN(src);
#pragma omp parallel for schedule(static)
  for (INT ii = 0; ii < n; ii++)
    dst->value[ii] = src->value[ii] * cexp(-I * pot->value[ii] * dt / (2.0 * HBAR));
}

/* The Crank-Nicolson factor of one axis: (1 - i hbar Q dt / 4m) / (1 + i hbar Q dt / 4m),
 * Q = kin_axis(k, h, 1).  Crank-Nicolson applied axis by axis (x, y, z) to
 * the periodic finite-difference operator multiplies each k by the product
 * of the three factors (every axis operator is diagonal in k). */
static inline REAL complex cn_axis(REAL k, REAL h, REAL mass, REAL complex dt) {
  REAL complex a = I * HBAR * kin_axis(k, h, 1) * dt / (4.0 * mass);
  return (1.0 - a) / (1.0 + a);
}

/* psi(k) *= exp(-i hbar |k - k0|^2 dt / 2m) / N, k0 = the momentum of grid m
 * (the Crank-Nicolson factors instead for a WF_2ND_ORDER_CN wave function) */
static void apply_kinetic(cgrid *c, const cgrid *m, REAL mass, REAL complex dt, int normalize, int cn) {
  INT nx = c->nx, ny = c->ny, nz = c->nz;
  REAL inv_n = normalize ? 1.0 / (REAL) (nx * ny * nz) : 1.0, h = c->step;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL kx = kval(i, nx, h) - m->kx0, ky = kval(j, ny, h) - m->ky0;
    for (INT k = 0; k < nz; k++) {
      REAL kz = kval(k, nz, h) - m->kz0;
      if (cn) {
        c->value[ij * nz + k] *= cn_axis(kx, h, mass, dt) * cn_axis(ky, h, mass, dt) * cn_axis(kz, h, mass, dt) * inv_n;
        continue;
      }
      REAL k2 = kx * kx + ky * ky + kz * kz;
      c->value[ij * nz + k] *= cexp(-I * HBAR * k2 * dt / (2.0 * mass)) * inv_n;
    }
  }
}

/* dst = S(V, dt) src ; dst may equal src */
static void strang_step(wf *g, cgrid *dst, cgrid *src, cgrid *pot, REAL complex dt) {
  apply_potential_half(dst, src, pot, dt);
  cgrid_fft(dst);
  apply_kinetic(dst, g->grid, g->mass, dt, 1, g->propagator == WF_2ND_ORDER_CN);
  cgrid_inverse_fft(dst);
  apply_potential_half(dst, dst, pot, dt);
}

/* Absorbing boundary (libgrid grid_wf_boundary / grid_wf_absorb_potential,
 * call sites examples/gas-bubble/bubble.c:149-157, examples/1d-bubble/
 * bubble-1d.c:192,222).  libgrid's arithmetic is not in the reference tree;
 * the restatement (a documented choice, shared with the GPU library): the
 * layer outside [lx, hx) x [ly, hy) x [lz, hz) has the weight
 * lambda = max over the axes of (l - i) / l below l and (i - h + 1) / (n - h)
 * from h on, and the absorbing potential is -i amp lambda (|psi|^2 / rho0 - 1).
 * Predict / correct steps of a wave function with a boundary add it,
 * evaluated from the step's input, to their potential; grid_wf_propagate does
 * not (single-step callers add it with grid_wf_absorb_potential). */
static REAL abs_ramp(INT i, INT l, INT h, INT n) {
  if (i < l) return (REAL) (l - i) / (REAL) l;
  if (i >= h) return (REAL) (i - h + 1) / (REAL) (n - h);
  return 0.0;
}

void grid_wf_boundary(wf *gwf, wf *gwfp, REAL amp, REAL rho0, INT lx, INT hx, INT ly, INT hy, INT lz, INT hz) {
  wf *w[2] = { gwf, gwfp };
  for (int n = 0; n < 2; n++) {
    if (!w[n]) continue;
    w[n]->abs_on = 1;
    w[n]->abs_amp = amp;
    w[n]->abs_rho0 = rho0;
    w[n]->abs_lo[0] = lx; w[n]->abs_hi[0] = hx;
    w[n]->abs_lo[1] = ly; w[n]->abs_hi[1] = hy;
    w[n]->abs_lo[2] = lz; w[n]->abs_hi[2] = hz;
  }
}

/* dst = pot - i amp lambda (|psi|^2 / rho0 - 1) (dst may be pot) */
static void absorb_add(wf *g, cgrid *dst, const cgrid *pot, REAL amp, REAL rho0) {
  cgrid *c = g->grid;
  INT nx = c->nx, ny = c->ny, nz = c->nz;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < nx * ny; ij++) {
    INT i = ij / ny, j = ij % ny;
    REAL lij = abs_ramp(i, g->abs_lo[0], g->abs_hi[0], nx);
    REAL ly = abs_ramp(j, g->abs_lo[1], g->abs_hi[1], ny);
    if (ly > lij) lij = ly;
    for (INT k = 0; k < nz; k++) {
      REAL lam = abs_ramp(k, g->abs_lo[2], g->abs_hi[2], nz);
      if (lij > lam) lam = lij;
      REAL complex v = pot->value[ij * nz + k];
      if (lam > 0.0) {
        REAL complex a = c->value[ij * nz + k];
        v -= I * amp * lam * ((creal(a) * creal(a) + cimag(a) * cimag(a)) / rho0 - 1.0);
      }
      dst->value[ij * nz + k] = v;
    }
  }
}

void grid_wf_absorb_potential(wf *gwf, cgrid *potential, REAL amp, REAL rho0) {
  if (!gwf->abs_on) {
    fprintf(stderr, "oracle: grid_wf_absorb_potential without grid_wf_boundary.\n");
    abort();
  }
  absorb_add(gwf, potential, potential, amp, rho0);
}

static void strang_step_pc(wf *g, cgrid *dst, cgrid *src, cgrid *pot, REAL complex dt) {
  if (!g->abs_on) { strang_step(g, dst, src, pot, dt); return; }
  cgrid *v = cgrid_clone(pot, "absorbing potential");
  absorb_add(g, v, pot, g->abs_amp, g->abs_rho0);
  strang_step(g, dst, src, v, dt);
  cgrid_free(v);
}

void grid_wf_propagate(wf *g, cgrid *pot, REAL complex dt) { strang_step(g, g->grid, g->grid, pot, dt); }
void grid_wf_propagate_predict(wf *g, wf *gp, cgrid *pot, REAL complex dt) { strang_step_pc(g, gp->grid, g->grid, pot, dt); }
void grid_wf_propagate_correct(wf *g, cgrid *pot, REAL complex dt) { strang_step_pc(g, g->grid, g->grid, pot, dt); }

void grid_wf_propagate_potential(wf *g, REAL complex dt, cgrid *pot, REAL cons) {
  INT n = CN(g->grid);
#pragma omp parallel for schedule(static)
  for (INT ii = 0; ii < n; ii++)
    g->grid->value[ii] *= cexp(-I * (pot->value[ii] + cons) * dt / HBAR);
}

void grid_wf_propagate_kinetic_fft(wf *g, REAL complex dt) { apply_kinetic(g->grid, g->grid, g->mass, dt, 0, 0); }

/* ------------------------------------------------------------------ */
/* ideal Bose gas of the thermal OT models (grid_func6a / 6b)            */
/* ------------------------------------------------------------------ */
/* libgrid's grid_func6a / 6b (src/ot.c:804-809, src/ot-energy.c:103) are
 * absent; they are restated as libdft's own host forms of the same term,
 * which its bulk relations use (src/common.c:253-529, src/helium-ot-bulk.c:
 * 30-31, 54-55): thermal wavelength lambda^3 = (2 pi hbar^2 / (m kB T))^(3/2);
 * the polylogarithms g_s(z) = sum_{k=1}^{256} z^k / k^s; z solving
 * g_{3/2}(z) = rho lambda^3 by golden-section search to a bracket of 1e-6
 * (z = 1 from g_{3/2}(1) on);
 *   f(rho)  = c4 kB T (rho ln z - g_{5/2}(z) / lambda^3),
 *   mu(rho) = c4 kB T (ln z + rho lambda^3 / g_{1/2}(z) - g_{3/2}(z) / g_{1/2}(z)),
 *             and -c4 kB T g_{3/2}(1) / lambda^3 for rho lambda^3 >= g_{3/2}(1). */
REAL oracle_lwl3(REAL mass, REAL temp) {
  REAL lwl = sqrt(2.0 * M_PI * HBAR * HBAR / (mass * GRID_AUKB * temp));
  return lwl * lwl * lwl;
}

static REAL oracle_polylog(REAL z, REAL s) {
  REAL val = 0.0, zk = 1.0;
  for (INT k = 1; k <= 256; k++) {
    zk *= z;
    val += zk / pow((REAL) k, s);
  }
  return val;
}

static REAL oracle_bose_z(REAL val) {
  const REAL golden = (sqrt(5.0) + 1.0) / 2.0;
  if (val >= oracle_polylog(1.0, 1.5)) return 1.0;
  REAL a = 0.0, b = 1.0, c = b - (b - a) / golden, d = a + (b - a) / golden;
  while (fabs(c - d) > 1E-6) {
    REAL t = val - oracle_polylog(c, 1.5), fc = t * t;
    t = val - oracle_polylog(d, 1.5);
    REAL fd = t * t;
    if (fc < fd) b = d; else a = c;
    c = b - (b - a) / golden;
    d = a + (b - a) / golden;
  }
  return (b + a) / 2.0;
}

REAL oracle_bose_energy(REAL rho, REAL mass, REAL temp, REAL c4) {
  REAL l3 = oracle_lwl3(mass, temp), z = oracle_bose_z(rho * l3);
  return c4 * GRID_AUKB * temp * (rho * log(z) - oracle_polylog(z, 2.5) / l3);
}

REAL oracle_bose_dEdRho(REAL rho, REAL mass, REAL temp, REAL c4) {
  REAL l3 = oracle_lwl3(mass, temp), rl3 = rho * l3, g32_1 = oracle_polylog(1.0, 1.5);
  if (rl3 >= g32_1) return -c4 * GRID_AUKB * (temp / l3) * g32_1;
  REAL z0 = oracle_bose_z(rl3), g12 = oracle_polylog(z0, 0.5), g32 = oracle_polylog(z0, 1.5);
  return c4 * GRID_AUKB * temp * (log(z0) + rl3 / g12 - g32 / g12);
}

void grid_func6a_operate_one(rgrid *d, rgrid *s, REAL mass, REAL temp, REAL c4) {
  INT nz = s->nz;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < s->nx * s->ny; ij++)
    for (INT k = 0; k < nz; k++) d->value[ij * d->nz2 + k] = oracle_bose_dEdRho(s->value[ij * s->nz2 + k], mass, temp, c4);
}

void grid_func6b_operate_one(rgrid *d, rgrid *s, REAL mass, REAL temp, REAL c4) {
  INT nz = s->nz;
#pragma omp parallel for schedule(static)
  for (INT ij = 0; ij < s->nx * s->ny; ij++)
    for (INT k = 0; k < nz; k++) d->value[ij * d->nz2 + k] = oracle_bose_energy(s->value[ij * s->nz2 + k], mass, temp, c4);
}
