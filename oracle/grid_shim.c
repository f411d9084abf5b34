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
/* 1-D mixed-radix Stockham FFT, batched over lines                     */
/* ------------------------------------------------------------------ */
/*
 * A batch holds V lines of length n in split form, re[i * V + v] and
 * im[i * V + v] for element i of line v, so each butterfly applies one set of
 * twiddles to V contiguous values.  Stage s has radix r and p = the product
 * of the earlier radices: it reads elements i + q n / r (q < r), multiplies
 * element q by exp(-+2 pi i q k / (p r)) with k = i mod p, takes the r-point
 * DFT and writes element (i - k) r + k + q p of the other buffer (Stockham
 * autosort: no bit reversal).  The stage twiddles are copied from the
 * length-n table, whose angles are reduced to [-pi, pi] before cos / sin.
 */

#define MAXFAC 48
#define MAXRADIX 64
#define FFT_BATCH 8   /* lines per batch */

typedef struct {
  INT n;
  int nf;
  int fac[MAXFAC];
  REAL complex *tw;        /* tw[t] = exp(-2 pi i t / n) */
  REAL *stw[MAXFAC];       /* stage s: (re, im) of tw[q k n / (p r)] at [2 (k (r - 1) + q - 1)], k < p, 1 <= q < r */
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
  INT pp = 1;
  for (int s = 0; s < p->nf; s++) {
    const int r = p->fac[s];
    const INT twstep = n / (pp * r);
    REAL *t = (REAL *) malloc(sizeof(REAL) * 2 * (size_t) (pp * (r - 1)));
    for (INT k = 0; k < pp; k++)
      for (int q = 1; q < r; q++) {
        const REAL complex w = p->tw[(q * k * twstep) % n];
        t[2 * (k * (r - 1) + q - 1)] = creal(w);
        t[2 * (k * (r - 1) + q - 1) + 1] = cimag(w);
      }
    p->stw[s] = t;
    pp *= r;
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

/* One stage's butterflies at input index i, output index j, for the V lines
 * of a batch.  tw: the stage twiddles of this k; sg = sign (-1 forward, +1
 * inverse): the inverse uses the conjugate twiddles. */
static void bfly2(const REAL *ir, const REAL *ii, REAL *orr, REAL *oi, INT i, INT j, INT nr, INT p, int V,
                  const REAL *tw, REAL sg) {
  const REAL wr = tw[0], wi = -sg * tw[1];
  const REAL *ar = ir + i * V, *ai = ii + i * V, *br = ir + (i + nr) * V, *bi = ii + (i + nr) * V;
  REAL *o0r = orr + j * V, *o0i = oi + j * V, *o1r = orr + (j + p) * V, *o1i = oi + (j + p) * V;
  for (int v = 0; v < V; v++) {
    const REAL xr = br[v] * wr - bi[v] * wi, xi = br[v] * wi + bi[v] * wr;
    o0r[v] = ar[v] + xr; o0i[v] = ai[v] + xi;
    o1r[v] = ar[v] - xr; o1i[v] = ai[v] - xi;
  }
}

static void bfly3(const REAL *ir, const REAL *ii, REAL *orr, REAL *oi, INT i, INT j, INT nr, INT p, int V,
                  const REAL *tw, REAL sg) {
  const REAL s3 = 0.86602540378443864676;
  const REAL w1r = tw[0], w1i = -sg * tw[1], w2r = tw[2], w2i = -sg * tw[3];
  const REAL *ar = ir + i * V, *ai = ii + i * V, *br = ir + (i + nr) * V, *bi = ii + (i + nr) * V;
  const REAL *cr = ir + (i + 2 * nr) * V, *ci = ii + (i + 2 * nr) * V;
  REAL *o0r = orr + j * V, *o0i = oi + j * V, *o1r = orr + (j + p) * V, *o1i = oi + (j + p) * V;
  REAL *o2r = orr + (j + 2 * p) * V, *o2i = oi + (j + 2 * p) * V;
  for (int v = 0; v < V; v++) {
    const REAL xr = br[v] * w1r - bi[v] * w1i, xi = br[v] * w1i + bi[v] * w1r;
    const REAL yr = cr[v] * w2r - ci[v] * w2i, yi = cr[v] * w2i + ci[v] * w2r;
    const REAL mr = ar[v] - 0.5 * (xr + yr), mi = ai[v] - 0.5 * (xi + yi);
    const REAL nr_ = s3 * (xr - yr), ni = s3 * (xi - yi);
    o0r[v] = ar[v] + xr + yr; o0i[v] = ai[v] + xi + yi;
    o1r[v] = mr - sg * ni; o1i[v] = mi + sg * nr_;     /* m + i sg n */
    o2r[v] = mr + sg * ni; o2i[v] = mi - sg * nr_;     /* m - i sg n */
  }
}

static void bfly4(const REAL *ir, const REAL *ii, REAL *orr, REAL *oi, INT i, INT j, INT nr, INT p, int V,
                  const REAL *tw, REAL sg) {
  const REAL w1r = tw[0], w1i = -sg * tw[1], w2r = tw[2], w2i = -sg * tw[3], w3r = tw[4], w3i = -sg * tw[5];
  const REAL *ar = ir + i * V, *ai = ii + i * V, *br = ir + (i + nr) * V, *bi = ii + (i + nr) * V;
  const REAL *cr = ir + (i + 2 * nr) * V, *ci = ii + (i + 2 * nr) * V;
  const REAL *dr = ir + (i + 3 * nr) * V, *di = ii + (i + 3 * nr) * V;
  REAL *o0r = orr + j * V, *o0i = oi + j * V, *o1r = orr + (j + p) * V, *o1i = oi + (j + p) * V;
  REAL *o2r = orr + (j + 2 * p) * V, *o2i = oi + (j + 2 * p) * V, *o3r = orr + (j + 3 * p) * V, *o3i = oi + (j + 3 * p) * V;
  for (int v = 0; v < V; v++) {
    const REAL xr = br[v] * w1r - bi[v] * w1i, xi = br[v] * w1i + bi[v] * w1r;
    const REAL yr = cr[v] * w2r - ci[v] * w2i, yi = cr[v] * w2i + ci[v] * w2r;
    const REAL zr = dr[v] * w3r - di[v] * w3i, zi = dr[v] * w3i + di[v] * w3r;
    const REAL t0r = ar[v] + yr, t0i = ai[v] + yi, t1r = ar[v] - yr, t1i = ai[v] - yi;
    const REAL t2r = xr + zr, t2i = xi + zi, t3r = xr - zr, t3i = xi - zi;
    o0r[v] = t0r + t2r; o0i[v] = t0i + t2i;
    o1r[v] = t1r - sg * t3i; o1i[v] = t1i + sg * t3r;  /* t1 + i sg t3 */
    o2r[v] = t0r - t2r; o2i[v] = t0i - t2i;
    o3r[v] = t1r + sg * t3i; o3i[v] = t1i - sg * t3r;  /* t1 - i sg t3 */
  }
}

static void bfly5(const REAL *ir, const REAL *ii, REAL *orr, REAL *oi, INT i, INT j, INT nr, INT p, int V,
                  const REAL *tw, REAL sg) {
  const REAL c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;
  const REAL s1 = 0.95105651629515357212, s2 = 0.58778525229247312917;
  REAL wr[4], wi[4];
  for (int q = 0; q < 4; q++) { wr[q] = tw[2 * q]; wi[q] = -sg * tw[2 * q + 1]; }
  const REAL *ar = ir + i * V, *ai = ii + i * V;
  REAL *o0r = orr + j * V, *o0i = oi + j * V, *o1r = orr + (j + p) * V, *o1i = oi + (j + p) * V;
  REAL *o2r = orr + (j + 2 * p) * V, *o2i = oi + (j + 2 * p) * V, *o3r = orr + (j + 3 * p) * V, *o3i = oi + (j + 3 * p) * V;
  REAL *o4r = orr + (j + 4 * p) * V, *o4i = oi + (j + 4 * p) * V;
  for (int v = 0; v < V; v++) {
    REAL ur[4], ui[4];
    for (int q = 0; q < 4; q++) {
      const REAL xr = ir[(i + (q + 1) * nr) * V + v], xi = ii[(i + (q + 1) * nr) * V + v];
      ur[q] = xr * wr[q] - xi * wi[q];
      ui[q] = xr * wi[q] + xi * wr[q];
    }
    const REAL t1r = ur[0] + ur[3], t1i = ui[0] + ui[3], t2r = ur[1] + ur[2], t2i = ui[1] + ui[2];
    const REAL t3r = ur[0] - ur[3], t3i = ui[0] - ui[3], t4r = ur[1] - ur[2], t4i = ui[1] - ui[2];
    const REAL m1r = ar[v] + c1 * t1r + c2 * t2r, m1i = ai[v] + c1 * t1i + c2 * t2i;
    const REAL m2r = ar[v] + c2 * t1r + c1 * t2r, m2i = ai[v] + c2 * t1i + c1 * t2i;
    const REAL n1r = s1 * t3r + s2 * t4r, n1i = s1 * t3i + s2 * t4i;
    const REAL n2r = s2 * t3r - s1 * t4r, n2i = s2 * t3i - s1 * t4i;
    o0r[v] = ar[v] + t1r + t2r; o0i[v] = ai[v] + t1i + t2i;
    o1r[v] = m1r - sg * n1i; o1i[v] = m1i + sg * n1r;  /* m1 + i sg n1 */
    o4r[v] = m1r + sg * n1i; o4i[v] = m1i - sg * n1r;
    o2r[v] = m2r - sg * n2i; o2i[v] = m2i + sg * n2r;  /* m2 + i sg n2 */
    o3r[v] = m2r + sg * n2i; o3i[v] = m2i - sg * n2r;
  }
}

/* any radix r <= MAXRADIX: the r-point DFT as a sum, roots of unity from the
 * length-n table */
static void bfly_any(const fft_plan *pl, int r, const REAL *ir, const REAL *ii, REAL *orr, REAL *oi, INT i, INT j,
                     INT nr, INT p, int V, const REAL *tw, REAL sg) {
  const INT step = pl->n / r;
  for (int v = 0; v < V; v++) {
    REAL ur[MAXRADIX], ui[MAXRADIX];
    ur[0] = ir[i * V + v]; ui[0] = ii[i * V + v];
    for (int q = 1; q < r; q++) {
      const REAL xr = ir[(i + q * nr) * V + v], xi = ii[(i + q * nr) * V + v];
      const REAL wr = tw[2 * (q - 1)], wi = -sg * tw[2 * (q - 1) + 1];
      ur[q] = xr * wr - xi * wi;
      ui[q] = xr * wi + xi * wr;
    }
    for (int q = 0; q < r; q++) {
      REAL accr = 0.0, acci = 0.0;
      for (int m = 0; m < r; m++) {
        const REAL complex w = pl->tw[((INT) ((q * m) % r)) * step];
        const REAL wr = creal(w), wi = -sg * cimag(w);
        accr += ur[m] * wr - ui[m] * wi;
        acci += ur[m] * wi + ui[m] * wr;
      }
      orr[(j + q * p) * V + v] = accr;
      oi[(j + q * p) * V + v] = acci;
    }
  }
}

/* V lines in (xr, xi), scratch (wr, wi) of the same size; the result ends in
 * (xr, xi).  sign -1 forward, +1 inverse (unnormalised). */
static void fft_batch(const fft_plan *pl, REAL *xr, REAL *xi, REAL *wr, REAL *wi, int V, int sign) {
  const INT n = pl->n;
  const REAL sg = (REAL) sign;
  REAL *ir = xr, *ii = xi, *orr = wr, *oi = wi, *t;
  INT p = 1;
  if (n == 1) return;
  for (int s = 0; s < pl->nf; s++) {
    const int r = pl->fac[s];
    const INT nr = n / r;
    const REAL *st = pl->stw[s];
    for (INT m = 0; m < nr / p; m++)
      for (INT k = 0; k < p; k++) {
        const INT i = m * p + k, j = m * p * r + k;
        const REAL *tw = st + 2 * k * (r - 1);
        switch (r) {
        case 2: bfly2(ir, ii, orr, oi, i, j, nr, p, V, tw, sg); break;
        case 3: bfly3(ir, ii, orr, oi, i, j, nr, p, V, tw, sg); break;
        case 4: bfly4(ir, ii, orr, oi, i, j, nr, p, V, tw, sg); break;
        case 5: bfly5(ir, ii, orr, oi, i, j, nr, p, V, tw, sg); break;
        default: bfly_any(pl, r, ir, ii, orr, oi, i, j, nr, p, V, tw, sg); break;
        }
      }
    p *= r;
    t = ir; ir = orr; orr = t;
    t = ii; ii = oi; oi = t;
  }
  if (ir != xr) {
    memcpy(xr, ir, sizeof(REAL) * (size_t) (n * V));
    memcpy(xi, ii, sizeof(REAL) * (size_t) (n * V));
  }
}

/* work space of one thread for batches of V lines of length n */
typedef struct { REAL *xr, *xi, *wr, *wi; } fft_work;

static fft_work work_alloc(INT n, int V) {
  fft_work w;
  w.xr = (REAL *) malloc(sizeof(REAL) * 4 * (size_t) (n * V));
  w.xi = w.xr + n * V;
  w.wr = w.xi + n * V;
  w.wi = w.wr + n * V;
  return w;
}

void oracle_fft1d(REAL complex *data, INT n, INT stride, int sign) {
  const fft_plan *pl = get_plan(n);
  fft_work w = work_alloc(n, 1);
  for (INT i = 0; i < n; i++) { w.xr[i] = creal(data[i * stride]); w.xi[i] = cimag(data[i * stride]); }
  fft_batch(pl, w.xr, w.xi, w.wr, w.wi, 1, sign);
  for (INT i = 0; i < n; i++) data[i * stride] = w.xr[i] + I * w.xi[i];
  free(w.xr);
}

/* Transform along one axis of a [n0][n1][n2] complex array, FFT_BATCH lines
 * at a time: along x and y the batch is FFT_BATCH neighbouring lines (adjacent
 * in z, so each element index reads one contiguous run); along z it is
 * FFT_BATCH consecutive rows. */
static void fft_axis(REAL complex *data, INT n0, INT n1, INT n2, int axis, int sign) {
  const INT n = (axis == 0) ? n0 : (axis == 1) ? n1 : n2;
  if (n == 1) return;
  const fft_plan *pl = get_plan(n);
  REAL *d = (REAL *) data;
  const INT stride = (axis == 0) ? n1 * n2 : (axis == 1) ? n2 : 1;
  /* lines come in runs of `inner` neighbours (consecutive line starts one
   * complex value apart for x / y, one row apart for z), `outer` runs */
  const INT outer = (axis == 1) ? n0 : 1;
  const INT inner = (axis == 0) ? n1 * n2 : (axis == 1) ? n2 : n0 * n1;
  const INT nbat = (inner + FFT_BATCH - 1) / FFT_BATCH;
#pragma omp parallel
  {
    fft_work w = work_alloc(n, FFT_BATCH);
#pragma omp for schedule(static)
    for (INT b = 0; b < outer * nbat; b++) {
      const INT o = b / nbat, c0 = (b % nbat) * FFT_BATCH;
      const int V = (int) ((inner - c0 < FFT_BATCH) ? inner - c0 : FFT_BATCH);
      if (axis == 2) {
        for (int v = 0; v < V; v++) {
          const REAL *row = d + 2 * (c0 + v) * n2;
          for (INT i = 0; i < n; i++) { w.xr[i * V + v] = row[2 * i]; w.xi[i * V + v] = row[2 * i + 1]; }
        }
      } else {
        const REAL *base = d + 2 * (o * n1 * n2 + c0);
        for (INT i = 0; i < n; i++)
          for (int v = 0; v < V; v++) {
            w.xr[i * V + v] = base[2 * (i * stride + v)];
            w.xi[i * V + v] = base[2 * (i * stride + v) + 1];
          }
      }
      fft_batch(pl, w.xr, w.xi, w.wr, w.wi, V, sign);
      if (axis == 2) {
        for (int v = 0; v < V; v++) {
          REAL *row = d + 2 * (c0 + v) * n2;
          for (INT i = 0; i < n; i++) { row[2 * i] = w.xr[i * V + v]; row[2 * i + 1] = w.xi[i * V + v]; }
        }
      } else {
        REAL *base = d + 2 * (o * n1 * n2 + c0);
        for (INT i = 0; i < n; i++)
          for (int v = 0; v < V; v++) {
            base[2 * (i * stride + v)] = w.xr[i * V + v];
            base[2 * (i * stride + v) + 1] = w.xi[i * V + v];
          }
      }
    }
    free(w.xr);
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

/* r2c along z in place, then c2c along y and x on the half spectrum.  An even
 * nz = 2h takes a length-h complex transform of z[m] = x[2m] + i x[2m+1]:
 * with Z its transform, E[k] = (Z[k] + conj Z[h-k]) / 2 and
 * O[k] = (Z[k] - conj Z[h-k]) / (2i) are the transforms of the even and odd
 * samples, and X[k] = E[k] + w^k O[k], w = exp(-2 pi i / nz), for k <= h
 * (X[0] and X[h] real).  An odd nz is transformed as a complex line. */
void rgrid_fft(rgrid *g) {
  const INT nx = g->nx, ny = g->ny, nz = g->nz, nzh = nz / 2 + 1, rows = nx * ny;
  const int half = !(nz & 1);
  const INT nl = half ? nz / 2 : nz;
  const fft_plan *pl = get_plan(nl);
  const fft_plan *pw = get_plan(nz);   /* w^k = pw->tw[k] */
  const INT nbat = (rows + FFT_BATCH - 1) / FFT_BATCH;
#pragma omp parallel
  {
    fft_work w = work_alloc(nl, FFT_BATCH);
#pragma omp for schedule(static)
    for (INT b = 0; b < nbat; b++) {
      const INT r0 = b * FFT_BATCH;
      const int V = (int) ((rows - r0 < FFT_BATCH) ? rows - r0 : FFT_BATCH);
      for (int v = 0; v < V; v++) {
        const REAL *row = g->value + (r0 + v) * g->nz2;
        if (half)
          for (INT m = 0; m < nl; m++) { w.xr[m * V + v] = row[2 * m]; w.xi[m * V + v] = row[2 * m + 1]; }
        else
          for (INT m = 0; m < nl; m++) { w.xr[m * V + v] = row[m]; w.xi[m * V + v] = 0.0; }
      }
      fft_batch(pl, w.xr, w.xi, w.wr, w.wi, V, -1);
      for (int v = 0; v < V; v++) {
        REAL *row = g->value + (r0 + v) * g->nz2;
        if (!half) {
          for (INT k = 0; k < nzh; k++) { row[2 * k] = w.xr[k * V + v]; row[2 * k + 1] = w.xi[k * V + v]; }
          continue;
        }
        const INT h = nl;
        const REAL z0r = w.xr[v], z0i = w.xi[v];
        for (INT k = 1; k < h; k++) {
          const REAL zr = w.xr[k * V + v], zi = w.xi[k * V + v];
          const REAL cr = w.xr[(h - k) * V + v], ci = -w.xi[(h - k) * V + v];   /* conj Z[h-k] */
          const REAL er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
          const REAL or_ = 0.5 * (zi - ci), oi = -0.5 * (zr - cr);
          const REAL wr = creal(pw->tw[k]), wi = cimag(pw->tw[k]);
          row[2 * k] = er + (wr * or_ - wi * oi);
          row[2 * k + 1] = ei + (wr * oi + wi * or_);
        }
        row[0] = z0r + z0i; row[1] = 0.0;
        row[2 * h] = z0r - z0i; row[2 * h + 1] = 0.0;
      }
    }
    free(w.xr);
  }
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 1, -1);
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 0, -1);
}

/* Inverse of rgrid_fft (unnormalised): c2c along x and y, then c2r along z.
 * An even nz = 2h forms Z[k] = A[k] + i B[k] (k < h) with
 * A[k] = X[k] + conj X[h-k] and B[k] = (X[k] - conj X[h-k]) conj(w^k), whose
 * length-h inverse is nz (x[2m] + i x[2m+1]).  The imaginary parts of X[0]
 * and X[h], which a real field's spectrum does not have, are dropped. */
void rgrid_inverse_fft(rgrid *g) {
  const INT nx = g->nx, ny = g->ny, nz = g->nz, nzh = nz / 2 + 1, rows = nx * ny;
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 0, +1);
  fft_axis((REAL complex *) g->value, nx, ny, nzh, 1, +1);
  const int half = !(nz & 1);
  const INT nl = half ? nz / 2 : nz;
  const fft_plan *pl = get_plan(nl);
  const fft_plan *pw = get_plan(nz);
  const INT nbat = (rows + FFT_BATCH - 1) / FFT_BATCH;
#pragma omp parallel
  {
    fft_work w = work_alloc(nl, FFT_BATCH);
#pragma omp for schedule(static)
    for (INT b = 0; b < nbat; b++) {
      const INT r0 = b * FFT_BATCH;
      const int V = (int) ((rows - r0 < FFT_BATCH) ? rows - r0 : FFT_BATCH);
      for (int v = 0; v < V; v++) {
        const REAL *row = g->value + (r0 + v) * g->nz2;
        if (!half) {
          for (INT k = 0; k < nzh; k++) { w.xr[k * V + v] = row[2 * k]; w.xi[k * V + v] = row[2 * k + 1]; }
          for (INT k = nzh; k < nz; k++) { w.xr[k * V + v] = row[2 * (nz - k)]; w.xi[k * V + v] = -row[2 * (nz - k) + 1]; }
          continue;
        }
        const INT h = nl;
        for (INT k = 0; k < h; k++) {
          const REAL xr = row[2 * k], xi = k ? row[2 * k + 1] : 0.0;
          const REAL cr = row[2 * (h - k)], ci = k ? -row[2 * (h - k) + 1] : 0.0;   /* conj X[h-k] */
          const REAL ar = xr + cr, ai = xi + ci;
          const REAL dr = xr - cr, di = xi - ci;
          const REAL wr = creal(pw->tw[k]), wi = -cimag(pw->tw[k]);                 /* conj w^k */
          const REAL br = dr * wr - di * wi, bi = dr * wi + di * wr;
          w.xr[k * V + v] = ar - bi;
          w.xi[k * V + v] = ai + br;
        }
      }
      fft_batch(pl, w.xr, w.xi, w.wr, w.wi, V, +1);
      for (int v = 0; v < V; v++) {
        REAL *row = g->value + (r0 + v) * g->nz2;
        if (half)
          for (INT m = 0; m < nl; m++) { row[2 * m] = w.xr[m * V + v]; row[2 * m + 1] = w.xi[m * V + v]; }
        else
          for (INT m = 0; m < nl; m++) row[m] = w.xr[m * V + v];
      }
    }
    free(w.xr);
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
