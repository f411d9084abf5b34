// extern "C" entry points of libdftgpu (declared in include/dftgpu.h).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "grid_internal.cuh"
#include "ot_internal.cuh"
#include "ot_thermal.cuh"

using namespace dftgpu;

namespace {

rgrid *rgrid_new(INT nx, INT ny, INT nz, REAL step, int prec, const char *id) {
  if (ensure_device() != DFTGPU_OK) return nullptr;
  if (check_dims(nx, ny, nz) != DFTGPU_OK) return nullptr;
  rgrid *g = (rgrid *) calloc(1, sizeof(rgrid));
  g->nx = nx; g->ny = ny; g->nz = nz; g->step = step; g->prec = prec;
  if (id) strncpy(g->id, id, sizeof(g->id) - 1);
  g->value = dev_alloc(gsize(g) * elem_size(prec));
  if (!g->value) { free(g); return nullptr; }
  if (cudaMemsetAsync(g->value, 0, gsize(g) * elem_size(prec), rt().stream) != cudaSuccess) {
    dev_free(g->value); free(g); set_error(DFTGPU_ERR_CUDA, "memset"); return nullptr;
  }
  return g;
}

cgrid *cgrid_new(INT nx, INT ny, INT nz, REAL step, int prec, const char *id) {
  if (ensure_device() != DFTGPU_OK) return nullptr;
  if (check_dims(nx, ny, nz) != DFTGPU_OK) return nullptr;
  cgrid *g = (cgrid *) calloc(1, sizeof(cgrid));
  g->nx = nx; g->ny = ny; g->nz = nz; g->step = step; g->prec = prec;
  if (id) strncpy(g->id, id, sizeof(g->id) - 1);
  g->value = dev_alloc(gsize(g) * 2 * elem_size(prec));
  if (!g->value) { free(g); return nullptr; }
  if (cudaMemsetAsync(g->value, 0, gsize(g) * 2 * elem_size(prec), rt().stream) != cudaSuccess) {
    dev_free(g->value); free(g); set_error(DFTGPU_ERR_CUDA, "memset"); return nullptr;
  }
  return g;
}

template <class G> bool same_shape(const G *a, const G *b) {
  return a && b && a->nx == b->nx && a->ny == b->ny && a->nz == b->nz && a->prec == b->prec;
}

bool rc_shape(const cgrid *c, const rgrid *r) {
  return c && r && c->nx == r->nx && c->ny == r->ny && c->nz == r->nz && c->prec == r->prec;
}

int bad_arg(const char *what) { set_error(DFTGPU_ERR_ARG, "%s", what); return DFTGPU_ERR_ARG; }

// NULL grids / wave functions are refused with DFTGPU_ERR_ARG before any device work
#define NEED(cond, what, ...)                                 \
  do {                                                        \
    if (!(cond)) { bad_arg(what ": NULL argument"); return __VA_ARGS__; } \
  } while (0)

// Instantiated graph of one predict-correct step, replayed by dftgpu_run when
// it is called again with the same arguments.  Any free of a grid, wave
// function or functional bumps g_generation and so invalidates it.
unsigned long g_generation = 1;
struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr, user = nullptr;
  cudaEvent_t ev = nullptr;
  unsigned long gen = 0;
  dft_ot_functional *otf = nullptr;
  wf *g = nullptr, *gp = nullptr;
  cgrid *P = nullptr;
  rgrid *vext = nullptr;
  double mu0 = 0, dr = 0, di = 0;
  double k0[3] = { 0, 0, 0 };   // moving-background momentum captured in the kinetic passes
  int renorm = 0;
} g_graph;

}  // namespace

extern "C" {

// ------------------------------------------------------------------ runtime
int dftgpu_init(int device) {
  Runtime &R = rt();
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error(DFTGPU_ERR_NODEVICE, "no CUDA device available");
    return DFTGPU_ERR_NODEVICE;
  }
  if (device < 0 || device >= n) return bad_arg("dftgpu_init: device index out of range");
  DFT_CUDA(cudaSetDevice(device));
  cudaDeviceProp p;
  DFT_CUDA(cudaGetDeviceProperties(&p, device));
  R.device = device;
  R.num_sms = p.multiProcessorCount;
  R.max_smem_optin = p.sharedMemPerBlockOptin;
  return DFTGPU_OK;
}

void cuda_enable(char value, INT ngpus, int *gpus) {
  if (!value) return;
  if (ngpus != 1) set_error(DFTGPU_ERR_UNSUPPORTED, "cuda_enable: one GPU per process (got %ld); using the first", (long) ngpus);
  dftgpu_init(gpus ? gpus[0] : 0);
}

int dftgpu_set_precision(int prec) {
  if (prec != DFTGPU_FP32 && prec != DFTGPU_FP64) return bad_arg("dftgpu_set_precision: FP32 or FP64");
  rt().precision = prec;
  return DFTGPU_OK;
}
int dftgpu_get_precision(void) { return rt().precision; }

int dftgpu_last_error(void) { int e = g_last_error; g_last_error = 0; return e; }
const char *dftgpu_last_error_message(void);

int dftgpu_synchronize(void) {
  if (ensure_device() != DFTGPU_OK) return DFTGPU_ERR_NODEVICE;
  DFT_CUDA(cudaStreamSynchronize(rt().stream));
  return fused_zy_fault();
}
int dftgpu_set_stream(void *stream) { rt().stream = (cudaStream_t) stream; return DFTGPU_OK; }
int dftgpu_profile(int enable) { return prof_enable(enable); }
int dftgpu_profile_report(char *buf, size_t len) {
  if (!buf || !len) return bad_arg("dftgpu_profile_report: buffer");
  return prof_report(buf, len);
}
void *dftgpu_get_stream(void) { return (void *) rt().stream; }

REAL rgrid_value_outside_periodic(rgrid *grid, INT i, INT j, INT k) {
  (void) grid; (void) i; (void) j; (void) k;
  return 0.0;   // sentinel only: the library evaluates periodic boundaries itself
}

// ------------------------------------------------------------------ rgrid
rgrid *rgrid_alloc(INT nx, INT ny, INT nz, REAL step, rgrid_outside_fn value_outside, void *outside_params_ptr, char *id) {
  (void) outside_params_ptr;
  if (value_outside && value_outside != rgrid_value_outside_periodic) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "rgrid_alloc: only periodic boundaries");
    return nullptr;
  }
  return rgrid_new(nx, ny, nz, step, rt().precision, id);
}

void rgrid_free(rgrid *g) { if (g) { g_generation++; dev_free(g->value); free(g); } }

rgrid *rgrid_clone(rgrid *g, char *id) {
  if (!g) return nullptr;
  rgrid *c = rgrid_new(g->nx, g->ny, g->nz, g->step, g->prec, id);
  if (c) { c->x0 = g->x0; c->y0 = g->y0; c->z0 = g->z0; }
  return c;
}

void rgrid_set_origin(rgrid *g, REAL x0, REAL y0, REAL z0) { NEED(g, "rgrid_set_origin"); g->x0 = x0; g->y0 = y0; g->z0 = z0; }
void rgrid_zero(rgrid *g) { NEED(g, "rgrid_zero"); rfill(g, 0.0); }
void rgrid_constant(rgrid *g, REAL c) { NEED(g, "rgrid_constant"); rfill(g, c); }
void rgrid_copy(rgrid *d, rgrid *s) {
  if (!same_shape(d, s)) { bad_arg("rgrid_copy: shape mismatch"); return; }
  if (cudaMemcpyAsync(d->value, s->value, gsize(s) * elem_size(s->prec), cudaMemcpyDeviceToDevice, rt().stream) != cudaSuccess)
    set_error(DFTGPU_ERR_CUDA, "rgrid_copy");
}
void rgrid_add(rgrid *g, REAL c) { NEED(g, "rgrid_add"); raxpb(g, 1.0, c); }
void rgrid_multiply(rgrid *g, REAL c) { NEED(g, "rgrid_multiply"); raxpb(g, c, 0.0); }
void rgrid_sum(rgrid *d, rgrid *a, rgrid *b) {
  if (!same_shape(d, a) || !same_shape(d, b)) { bad_arg("rgrid_sum: shape mismatch"); return; }
  rbinary(d, a, b, 0.0, 0);
}
void rgrid_product(rgrid *d, rgrid *a, rgrid *b) {
  if (!same_shape(d, a) || !same_shape(d, b)) { bad_arg("rgrid_product: shape mismatch"); return; }
  rbinary(d, a, b, 0.0, 1);
}
void rgrid_add_scaled(rgrid *d, REAL c, rgrid *s) {
  if (!same_shape(d, s)) { bad_arg("rgrid_add_scaled: shape mismatch"); return; }
  rbinary(d, s, nullptr, c, 2);
}
void rgrid_add_scaled_product(rgrid *d, REAL c, rgrid *a, rgrid *b) {
  if (!same_shape(d, a) || !same_shape(d, b)) { bad_arg("rgrid_add_scaled_product: shape mismatch"); return; }
  rbinary(d, a, b, c, 3);
}
void rgrid_power(rgrid *d, rgrid *s, REAL exponent) {
  if (!same_shape(d, s)) { bad_arg("rgrid_power: shape mismatch"); return; }
  rpower(d, s, exponent);
}
REAL rgrid_integral(rgrid *g) {
  NEED(g, "rgrid_integral", NAN);
  double v = NAN;
  rintegral(g, &v);
  return v;
}

void rgrid_map(rgrid *g, rgrid_map_fn func, void *farg) {
  NEED(g && func, "rgrid_map");
  const INT nx = g->nx, ny = g->ny, nz = g->nz;
  std::vector<double> h(gsize(g));
  for (INT i = 0; i < nx; i++) {
    const REAL x = (REAL) (i - nx / 2) * g->step - g->x0;
    for (INT j = 0; j < ny; j++) {
      const REAL y = (REAL) (j - ny / 2) * g->step - g->y0;
      for (INT k = 0; k < nz; k++) {
        const REAL z = (REAL) (k - nz / 2) * g->step - g->z0;
        h[(i * ny + j) * nz + k] = func(farg, x, y, z);
      }
    }
  }
  copy_values_in(g->prec, g->value, h.data(), h.size());
}

// n consecutive values of precision prec from element idx of a device grid,
// read on the work stream after the work queued on it
static int read_values(int prec, const void *dev, size_t idx, int n, double *out) {
  if (prec == DFTGPU_FP32) {
    float f[2];
    DFT_CUDA(cudaMemcpyAsync(f, (const float *) dev + idx, n * sizeof(float), cudaMemcpyDeviceToHost, rt().stream));
    DFT_CUDA(cudaStreamSynchronize(rt().stream));
    for (int i = 0; i < n; i++) out[i] = f[i];
  } else {
    DFT_CUDA(cudaMemcpyAsync(out, (const double *) dev + idx, n * sizeof(double), cudaMemcpyDeviceToHost, rt().stream));
    DFT_CUDA(cudaStreamSynchronize(rt().stream));
  }
  return DFTGPU_OK;
}

static size_t wrapped_index(INT nx, INT ny, INT nz, INT i, INT j, INT k) {
  i = ((i % nx) + nx) % nx; j = ((j % ny) + ny) % ny; k = ((k % nz) + nz) % nz;
  return ((size_t) i * ny + j) * nz + k;
}

REAL rgrid_value_at_index(rgrid *g, INT i, INT j, INT k) {
  if (!g) { bad_arg("rgrid_value_at_index: NULL grid"); return NAN; }
  double v = NAN;
  if (read_values(g->prec, g->value, wrapped_index(g->nx, g->ny, g->nz, i, j, k), 1, &v) != DFTGPU_OK) return NAN;
  return v;
}

int cgrid_value_at_index_re_im(cgrid *g, INT i, INT j, INT k, REAL *re, REAL *im) {
  if (!g || !re || !im) return bad_arg("cgrid_value_at_index: NULL argument");
  double v[2] = { NAN, NAN };
  const int rc = read_values(g->prec, g->value, 2 * wrapped_index(g->nx, g->ny, g->nz, i, j, k), 2, v);
  *re = v[0];
  *im = v[1];
  return rc;
}

int rgrid_copy_to_host(rgrid *g, double *host) { NEED(g && host, "rgrid_copy_to_host", DFTGPU_ERR_ARG); return copy_values_out(g->prec, g->value, host, gsize(g)); }
int rgrid_copy_from_host(rgrid *g, const double *host) { NEED(g && host, "rgrid_copy_from_host", DFTGPU_ERR_ARG); return copy_values_in(g->prec, g->value, host, gsize(g)); }
int rgrid_copy_to_host_raw(rgrid *g, void *host) {
  NEED(g && host, "rgrid_copy_to_host_raw", DFTGPU_ERR_ARG);
  DFT_CUDA(cudaMemcpyAsync(host, g->value, gsize(g) * elem_size(g->prec), cudaMemcpyDeviceToHost, rt().stream));
  DFT_CUDA(cudaStreamSynchronize(rt().stream));
  return DFTGPU_OK;
}
int rgrid_copy_from_host_raw(rgrid *g, const void *host) {
  NEED(g && host, "rgrid_copy_from_host_raw", DFTGPU_ERR_ARG);
  DFT_CUDA(cudaMemcpyAsync(g->value, host, gsize(g) * elem_size(g->prec), cudaMemcpyHostToDevice, rt().stream));
  return DFTGPU_OK;
}

// ------------------------------------------------------------------ cgrid
cgrid *cgrid_alloc(INT nx, INT ny, INT nz, REAL step, void *value_outside, void *outside_params_ptr, char *id) {
  (void) value_outside; (void) outside_params_ptr;
  return cgrid_new(nx, ny, nz, step, rt().precision, id);
}
void cgrid_free(cgrid *g) { if (g) { g_generation++; dev_free(g->value); free(g); } }
cgrid *cgrid_clone(cgrid *g, char *id) {
  if (!g) return nullptr;
  cgrid *c = cgrid_new(g->nx, g->ny, g->nz, g->step, g->prec, id);
  if (c) { c->x0 = g->x0; c->y0 = g->y0; c->z0 = g->z0; c->kx0 = g->kx0; c->ky0 = g->ky0; c->kz0 = g->kz0; }
  return c;
}
// Moving background: the wave function on this grid lives in the frame moving
// with momentum hbar k0, where the kinetic operator is hbar^2 |k - k0|^2 / 2m
// (callers: examples/gas-bubble/bubble.c:104,173,
// examples/added_mass/added_mass.c:78, examples/1d-bubble/bubble-1d.c:136).
void cgrid_set_momentum(cgrid *g, REAL kx0, REAL ky0, REAL kz0) {
  NEED(g, "cgrid_set_momentum");
  g->kx0 = kx0; g->ky0 = ky0; g->kz0 = kz0;
}
void cgrid_zero(cgrid *g) { NEED(g, "cgrid_zero"); cfill(g, 0.0, 0.0); }
void cgrid_constant_re_im(cgrid *g, REAL re, REAL im) { NEED(g, "cgrid_constant"); cfill(g, re, im); }
void cgrid_add_re_im(cgrid *g, REAL re, REAL im) { NEED(g, "cgrid_add"); cmuladd(g, 1.0, 0.0, re, im); }
void cgrid_multiply_re_im(cgrid *g, REAL re, REAL im) { NEED(g, "cgrid_multiply"); cmuladd(g, re, im, 0.0, 0.0); }
void cgrid_copy(cgrid *d, cgrid *s) {
  if (!same_shape(d, s)) { bad_arg("cgrid_copy: shape mismatch"); return; }
  if (cudaMemcpyAsync(d->value, s->value, gsize(s) * 2 * elem_size(s->prec), cudaMemcpyDeviceToDevice, rt().stream) != cudaSuccess)
    set_error(DFTGPU_ERR_CUDA, "cgrid_copy");
}
void cgrid_map_re_im(cgrid *g, cgrid_map_fn func, void *farg) {
  NEED(g && func, "cgrid_map");
  const INT nx = g->nx, ny = g->ny, nz = g->nz;
  std::vector<double> h(2 * gsize(g));
  for (INT i = 0; i < nx; i++) {
    const REAL x = (REAL) (i - nx / 2) * g->step - g->x0;
    for (INT j = 0; j < ny; j++) {
      const REAL y = (REAL) (j - ny / 2) * g->step - g->y0;
      for (INT k = 0; k < nz; k++) {
        const REAL z = (REAL) (k - nz / 2) * g->step - g->z0;
        const size_t idx = (size_t) ((i * ny + j) * nz + k);
        func(farg, x, y, z, &h[2 * idx], &h[2 * idx + 1]);
      }
    }
  }
  copy_values_in(g->prec, g->value, h.data(), h.size());
}
int cgrid_copy_to_host(cgrid *g, double *host) { NEED(g && host, "cgrid_copy_to_host", DFTGPU_ERR_ARG); return copy_values_out(g->prec, g->value, host, 2 * gsize(g)); }
int cgrid_copy_from_host(cgrid *g, const double *host) { NEED(g && host, "cgrid_copy_from_host", DFTGPU_ERR_ARG); return copy_values_in(g->prec, g->value, host, 2 * gsize(g)); }
int cgrid_copy_to_host_raw(cgrid *g, void *host) {
  NEED(g && host, "cgrid_copy_to_host_raw", DFTGPU_ERR_ARG);
  DFT_CUDA(cudaMemcpyAsync(host, g->value, gsize(g) * 2 * elem_size(g->prec), cudaMemcpyDeviceToHost, rt().stream));
  DFT_CUDA(cudaStreamSynchronize(rt().stream));
  return DFTGPU_OK;
}
int cgrid_copy_from_host_raw(cgrid *g, const void *host) {
  NEED(g && host, "cgrid_copy_from_host_raw", DFTGPU_ERR_ARG);
  DFT_CUDA(cudaMemcpyAsync(g->value, host, gsize(g) * 2 * elem_size(g->prec), cudaMemcpyHostToDevice, rt().stream));
  return DFTGPU_OK;
}

void grid_real_to_complex_re(cgrid *d, rgrid *s) { if (!rc_shape(d, s)) { bad_arg("grid_real_to_complex_re"); return; } real_to_complex(d, s, 0); }
void grid_add_real_to_complex_re(cgrid *d, rgrid *s) { if (!rc_shape(d, s)) { bad_arg("grid_add_real_to_complex_re"); return; } real_to_complex(d, s, 1); }
void grid_add_real_to_complex_im(cgrid *d, rgrid *s) { if (!rc_shape(d, s)) { bad_arg("grid_add_real_to_complex_im"); return; } real_to_complex(d, s, 2); }

// ------------------------------------------------------------------ wave functions
wf *grid_wf_alloc(INT nx, INT ny, INT nz, REAL step, REAL mass, char boundary, char propagator, char *id) {
  if (boundary != WF_PERIODIC_BOUNDARY || (propagator != WF_2ND_ORDER_FFT && propagator != WF_2ND_ORDER_CN)) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "grid_wf_alloc: periodic boundary with WF_2ND_ORDER_FFT or WF_2ND_ORDER_CN only");
    return nullptr;
  }
  cgrid *c = cgrid_new(nx, ny, nz, step, rt().precision, id);
  if (!c) return nullptr;
  wf *w = (wf *) calloc(1, sizeof(wf));
  if (!w) { cgrid_free(c); set_error(DFTGPU_ERR_NOMEM, "grid_wf_alloc"); return nullptr; }
  w->grid = c;
  w->mass = mass;
  w->norm = 1.0;
  w->boundary = boundary;
  w->propagator = propagator;
  w->priv = new WfPriv();
  return w;
}

wf *grid_wf_clone(wf *g, char *id) {
  if (!g) return nullptr;
  int save = rt().precision;
  rt().precision = g->grid->prec;
  wf *w = grid_wf_alloc(g->grid->nx, g->grid->ny, g->grid->nz, g->grid->step, g->mass, g->boundary, g->propagator, id);
  rt().precision = save;
  if (w) {
    w->norm = g->norm;
    w->grid->x0 = g->grid->x0; w->grid->y0 = g->grid->y0; w->grid->z0 = g->grid->z0;
    w->grid->kx0 = g->grid->kx0; w->grid->ky0 = g->grid->ky0; w->grid->kz0 = g->grid->kz0;
  }
  return w;
}

void grid_wf_free(wf *g) {
  if (!g) return;
  WfPriv *p = (WfPriv *) g->priv;
  if (p) {
    dev_free(p->spec);
    if (p->vtot) { dev_free(p->vtot->value); free(p->vtot); }
    delete p;
  }
  cgrid_free(g->grid);
  free(g);
}

// Absorbing boundary (libgrid; call sites examples/gas-bubble/bubble.c:149-157,
// examples/1d-bubble/bubble-1d.c:192,222).  libgrid's arithmetic is not in the
// reference tree; the form here is this library's (AbsBoundary in
// grid_internal.cuh): outside [lx, hx) x [ly, hy) x [lz, hz) the weight lambda
// rises linearly to 1 at the grid's edge, and the absorbing potential is
// -i amp lambda (|psi|^2 / rho0 - 1), which drives the density there towards
// rho0.  grid_wf_propagate_predict / _correct (and dftgpu_pc_step /
// dftgpu_run) add it, evaluated from the step's input, to the potential of
// the wave function that has the boundary; grid_wf_propagate does not (a
// single-step caller adds it with grid_wf_absorb_potential).
static int set_boundary(wf *g, REAL amp, REAL rho0, const INT lo[3], const INT hi[3]) {
  const INT n[3] = { g->grid->nx, g->grid->ny, g->grid->nz };
  for (int a = 0; a < 3; a++)
    if (lo[a] < 0 || hi[a] > n[a] || lo[a] > hi[a]) return bad_arg("grid_wf_boundary: layer outside the grid");
  if (!(rho0 > 0.0)) return bad_arg("grid_wf_boundary: rho0 must be positive");
  AbsBoundary &b = ((WfPriv *) g->priv)->abs;
  b.on = 1;
  b.amp = amp;
  b.rho0 = rho0;
  for (int a = 0; a < 3; a++) { b.lo[a] = (int) lo[a]; b.hi[a] = (int) hi[a]; }
  g_generation++;   // a captured step graph of this wave function is stale
  return DFTGPU_OK;
}

void grid_wf_boundary(wf *gwf, wf *gwfp, REAL amp, REAL rho0, INT lx, INT hx, INT ly, INT hy, INT lz, INT hz) {
  NEED(gwf, "grid_wf_boundary");
  const INT lo[3] = { lx, ly, lz }, hi[3] = { hx, hy, hz };
  if (set_boundary(gwf, amp, rho0, lo, hi)) return;
  if (gwfp) set_boundary(gwfp, amp, rho0, lo, hi);
}

void grid_wf_absorb_potential(wf *gwf, cgrid *potential, REAL amp, REAL rho0) {
  NEED(gwf && potential, "grid_wf_absorb_potential");
  if (!same_shape(gwf->grid, potential) || potential->prec != gwf->grid->prec) {
    bad_arg("grid_wf_absorb_potential: grid mismatch");
    return;
  }
  const AbsBoundary &b = ((WfPriv *) gwf->priv)->abs;
  if (!b.on) { bad_arg("grid_wf_absorb_potential: no absorbing boundary set (grid_wf_boundary)"); return; }
  if (!(rho0 > 0.0)) { bad_arg("grid_wf_absorb_potential: rho0 must be positive"); return; }
  absorb_add(potential, potential, gwf->grid, b, amp, rho0);
}

void grid_wf_constant_re_im(wf *g, REAL re, REAL im) { NEED(g, "grid_wf_constant"); cfill(g->grid, re, im); }

void grid_wf_density(wf *g, rgrid *d) {
  NEED(g, "grid_wf_density");
  if (!rc_shape(g->grid, d)) { bad_arg("grid_wf_density: shape mismatch"); return; }
  density(g->grid, d);
}

REAL grid_wf_norm(wf *g) {
  NEED(g, "grid_wf_norm", NAN);
  double v = NAN;
  double *slot = reduce_slots();
  if (norm_dev(g->grid, slot + 1) != DFTGPU_OK) return NAN;
  if (cudaMemcpyAsync(&v, slot + 1, sizeof(double), cudaMemcpyDeviceToHost, rt().stream) != cudaSuccess ||
      cudaStreamSynchronize(rt().stream) != cudaSuccess) { set_error(DFTGPU_ERR_CUDA, "grid_wf_norm"); return NAN; }
  if (!isfinite(v)) set_error(DFTGPU_ERR_NONFINITE, "grid_wf_norm: non-finite norm");
  return v;
}

REAL grid_wf_normalize(wf *g) {
  NEED(g, "grid_wf_normalize", NAN);
  double *slot = reduce_slots();
  if (norm_dev(g->grid, slot + 2) != DFTGPU_OK) return NAN;
  if (scale_by_norm(g->grid, slot + 2, g->norm) != DFTGPU_OK) return NAN;
  double v = NAN;
  if (cudaMemcpyAsync(&v, slot + 2, sizeof(double), cudaMemcpyDeviceToHost, rt().stream) != cudaSuccess ||
      cudaStreamSynchronize(rt().stream) != cudaSuccess) { set_error(DFTGPU_ERR_CUDA, "grid_wf_normalize"); return NAN; }
  if (!isfinite(v) || v <= 0.0) set_error(DFTGPU_ERR_NONFINITE, "grid_wf_normalize: norm %g", v);
  return sqrt(g->norm / v);
}

REAL grid_wf_kinetic_energy(wf *g) {
  NEED(g, "grid_wf_kinetic_energy", NAN);
  double v = NAN;
  kinetic_energy(g, &v);
  return v;
}

REAL grid_wf_energy(wf *g, rgrid *pot) {
  NEED(g, "grid_wf_energy", NAN);
  double e = grid_wf_kinetic_energy(g);
  if (pot) {
    rgrid *d = rgrid_new(g->grid->nx, g->grid->ny, g->grid->nz, g->grid->step, g->grid->prec, "tmp");
    if (!d) return NAN;
    density(g->grid, d);
    rbinary(d, d, pot, 0.0, 1);
    double v = NAN;
    rintegral(d, &v);
    rgrid_free(d);
    e += v;
  }
  return e;
}

void grid_wf_velocity(wf *g, rgrid *vx, rgrid *vy, rgrid *vz, REAL eps) {
  NEED(g, "grid_wf_velocity");
  if (!rc_shape(g->grid, vx) || !rc_shape(g->grid, vy) || !rc_shape(g->grid, vz)) { bad_arg("grid_wf_velocity"); return; }
  velocity(g, vx, vy, vz, eps);
}

int dftgpu_wf_propagate(wf *g, cgrid *pot, double dr, double di) { NEED(g, "propagate", DFTGPU_ERR_ARG); return propagate(g, g->grid, g->grid, pot, dr, di); }
int dftgpu_wf_propagate_predict(wf *g, wf *gp, cgrid *pot, double dr, double di) {
  NEED(g, "propagate_predict", DFTGPU_ERR_ARG);
  if (!gp || !same_shape(g->grid, gp->grid)) return bad_arg("propagate_predict: wave function mismatch");
  return propagate_pc(g, gp->grid, g->grid, pot, dr, di);
}
int dftgpu_wf_propagate_correct(wf *g, cgrid *pot, double dr, double di) { NEED(g, "propagate_correct", DFTGPU_ERR_ARG); return propagate_pc(g, g->grid, g->grid, pot, dr, di); }

// ------------------------------------------------------------------ OT functional
// 0 K OT parameters and unit conversions (src/ot.c:1026-1036, 1234-1270)
void dft_ot_init_params(dft_ot_functional *otf, INT model) {
  const double a3 = GRID_AUTOANG * GRID_AUTOANG * GRID_AUTOANG;
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
  // the thermal parameter sets (src/ot.c:1038-1222): b, c2, c3 (K, Angstrom),
  // c4, T (K), rho0, h; each selected by its bit, a later bit overriding an
  // earlier one as in the reference
  static const struct { INT bit; double b, c2, c3, c4, temp, rho0, h; } tset[] = {
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
  for (const auto &t : tset)
    if (model & t.bit) {
      otf->b = t.b; otf->c2 = t.c2; otf->c3 = t.c3; otf->c4 = t.c4;
      otf->temp = t.temp; otf->rho0 = t.rho0; otf->lj_params.h = t.h;
    }
  otf->mu0 = 0.0;
  otf->xi = 1E4 / a3;
  otf->rhobf = 0.033 * a3;
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

dft_ot_functional *dft_ot_alloc(INT model, wf *gwf, INT min_substeps, INT max_substeps) {
  if (!gwf) { bad_arg("dft_ot_alloc: NULL wave function"); return nullptr; }
  if (model & ~((INT) (DFT_OT_KC | DFT_OT_HD | DFT_OT_HD2 | DFT_OT_BACKFLOW | (2 * DFT_OT_T3000MK - DFT_OT_T0MK)))) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "dft_ot_alloc: model %ld outside {PLAIN, KC, HD, HD2, BACKFLOW, T0MK..T3000MK}",
              (long) model);
    return nullptr;
  }
  cgrid *c = gwf->grid;
  dft_ot_functional *otf = (dft_ot_functional *) calloc(1, sizeof(dft_ot_functional));
  if (!otf) return nullptr;
  otf->model = model;
  dft_ot_init_params(otf, model);
  OtPriv *P = new OtPriv();
  P->prec = c->prec;
  P->nx = (int) c->nx; P->ny = (int) c->ny; P->nz = (int) c->nz;
  P->step = c->step; P->x0 = c->x0; P->y0 = c->y0; P->z0 = c->z0;
  P->oct_n = (size_t) (P->nz / 2 + 1) * (P->nx / 2 + 1) * (P->ny / 2 + 1);
  otf->priv = P;
  otf->density = rgrid_new(c->nx, c->ny, c->nz, c->step, c->prec, "OT density");
  if (!otf->density || ot_generate_kernels(otf, (int) min_substeps, (int) max_substeps) != DFTGPU_OK) {
    dft_ot_free(otf);
    return nullptr;
  }
  return otf;
}

int dft_ot_update_kernels(dft_ot_functional *otf, INT min_substeps, INT max_substeps) {
  if (!otf) return bad_arg("dft_ot_update_kernels: NULL");
  return ot_generate_kernels(otf, (int) min_substeps, (int) max_substeps);
}

void dft_ot_free(dft_ot_functional *otf) {
  if (!otf) return;
  g_generation++;
  OtPriv *P = (OtPriv *) otf->priv;
  if (P) {
    for (int i = 0; i < OT_NKER; i++) dev_free(P->ker[i]);
    for (int i = 0; i < OT_MAX_REAL; i++) dev_free(P->real[i]);
    for (int i = 0; i < OT_MAX_SPEC; i++) dev_free(P->spec[i]);
    cgrid_free(P->pot_tmp);
    rgrid_free(P->ed_tmp);
    adj_free(P);
    delete P;
  }
  rgrid_free(otf->density);
  free(otf);
}

static bool ot_matches(dft_ot_functional *otf, const cgrid *c) {
  OtPriv *P = (OtPriv *) otf->priv;
  return c && P && c->nx == P->nx && c->ny == P->ny && c->nz == P->nz && c->prec == P->prec;
}

void dft_ot_potential(dft_ot_functional *otf, cgrid *potential, wf *gwf) {
  if (!otf || !gwf || !ot_matches(otf, potential) || !ot_matches(otf, gwf->grid)) { bad_arg("dft_ot_potential: grid mismatch"); return; }
  ot_potential(otf, potential, gwf);
}

static bool ot_matches_r(dft_ot_functional *otf, const rgrid *r) {
  OtPriv *P = otf ? (OtPriv *) otf->priv : nullptr;
  return r && P && r->nx == P->nx && r->ny == P->ny && r->nz == P->nz && r->prec == P->prec;
}

static void potential_from_fields(const char *what, dft_ot_functional *otf, cgrid *potential, rgrid *density,
                                  rgrid *vx, rgrid *vy, rgrid *vz, int terms, bool vclamp) {
  if (!otf || !ot_matches(otf, potential) || !ot_matches_r(otf, density)) { bad_arg(what); return; }
  PotSrc src;
  src.terms = terms;
  src.dens = density->value;
  src.vclamp = vclamp;
  if ((terms & POT_BF) && (otf->model & DFT_OT_BACKFLOW)) {
    if (!ot_matches_r(otf, vx) || !ot_matches_r(otf, vy) || !ot_matches_r(otf, vz)) { bad_arg(what); return; }
    src.vel[0] = vx->value; src.vel[1] = vy->value; src.vel[2] = vz->value;
    src.wout[0] = vx->value; src.wout[1] = vy->value; src.wout[2] = vz->value;
  }
  ot_potential_src(otf, potential, nullptr, 0, nullptr, 0.0, 1.0, src);
}

void dft_ot_potential2(dft_ot_functional *otf, cgrid *potential, rgrid *density, rgrid *veloc_x, rgrid *veloc_y,
                       rgrid *veloc_z) {
  potential_from_fields("dft_ot_potential2: grid mismatch", otf, potential, density, veloc_x, veloc_y, veloc_z,
                        POT_ALL, true);
}

void dft_ot_add_lennard_jones_potential(dft_ot_functional *otf, cgrid *potential, rgrid *density, rgrid *workspace1,
                                        rgrid *workspace2) {
  (void) workspace1; (void) workspace2;
  potential_from_fields("dft_ot_add_lennard_jones_potential: grid mismatch", otf, potential, density, nullptr,
                        nullptr, nullptr, POT_LJ, true);
}

void dft_ot_add_local_correlation_potential(dft_ot_functional *otf, cgrid *potential, rgrid *rho, rgrid *rho_tf,
                                            rgrid *workspace1, rgrid *workspace2) {
  (void) rho_tf; (void) workspace1; (void) workspace2;
  potential_from_fields("dft_ot_add_local_correlation_potential: grid mismatch", otf, potential, rho, nullptr,
                        nullptr, nullptr, POT_LOCAL, true);
}

void dft_ot_backflow_potential(dft_ot_functional *otf, cgrid *potential, rgrid *density, rgrid *veloc_x,
                               rgrid *veloc_y, rgrid *veloc_z, rgrid *workspace1, rgrid *workspace2,
                               rgrid *workspace3, rgrid *workspace4, rgrid *workspace5, rgrid *workspace6) {
  (void) workspace1; (void) workspace2; (void) workspace3; (void) workspace4; (void) workspace5; (void) workspace6;
  if (otf && !(otf->model & DFT_OT_BACKFLOW)) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "dft_ot_backflow_potential: functional allocated without DFT_OT_BACKFLOW");
    return;
  }
  potential_from_fields("dft_ot_backflow_potential: grid mismatch", otf, potential, density, veloc_x, veloc_y,
                        veloc_z, POT_BF, false);
}

static void energy_density_part(const char *what, dft_ot_functional *otf, rgrid *ed, wf *gwf, rgrid *density,
                                int terms, int model_bit) {
  if (!otf || !gwf || !ot_matches(otf, gwf->grid) || !ot_matches_r(otf, ed) || !ot_matches_r(otf, density)) {
    bad_arg(what);
    return;
  }
  if (!(otf->model & model_bit)) { set_error(DFTGPU_ERR_UNSUPPORTED, "%s: term not in the functional's model", what); return; }
  ot_energy_density_terms(otf, ed, gwf, terms, density, true);
}

void dft_ot_energy_density_kc(dft_ot_functional *otf, rgrid *ed, wf *gwf, rgrid *density) {
  energy_density_part("dft_ot_energy_density_kc", otf, ed, gwf, density, POT_KC, DFT_OT_KC);
}

void dft_ot_energy_density_bf(dft_ot_functional *otf, rgrid *ed, wf *gwf, rgrid *density) {
  energy_density_part("dft_ot_energy_density_bf", otf, ed, gwf, density, POT_BF, DFT_OT_BACKFLOW);
}

void dft_ot_energy_density(dft_ot_functional *otf, rgrid *ed, wf *gwf) {
  OtPriv *P = otf ? (OtPriv *) otf->priv : nullptr;
  if (!P || !gwf || !ot_matches(otf, gwf->grid) || !ed || ed->nx != P->nx || ed->ny != P->ny || ed->nz != P->nz || ed->prec != P->prec) {
    bad_arg("dft_ot_energy_density: grid mismatch");
    return;
  }
  ot_energy_density(otf, ed, gwf);
}

int dftgpu_rgrid_spectrum(rgrid *g, double *host) {
  if (!g || !host) return bad_arg("dftgpu_rgrid_spectrum: NULL");
  return rspectrum(g, host);
}

int dftgpu_ot_kernel(dft_ot_functional *otf, int which, double *host) {
  if (!otf || !host || which < 0 || which >= OT_NKER) return bad_arg("dftgpu_ot_kernel: argument");
  OtPriv *P = (OtPriv *) otf->priv;
  if (which >= OT_F && which <= OT_FZ && !(otf->model & DFT_OT_KC)) return bad_arg("dftgpu_ot_kernel: no KC kernels");
  if (which == OT_VJ && !(otf->model & DFT_OT_BACKFLOW)) return bad_arg("dftgpu_ot_kernel: no backflow kernel");
  return copy_values_out(P->prec, P->ker[which], host, P->oct_n);
}

}  // extern "C"

// ------------------------------------------------------------------ ideal Bose gas (host)
// libdft's host forms (src/common.c:253-529): lambda^3, the 256-term
// polylogarithms, z from golden-section search to a bracket of 1e-6, and the
// free energy / its density derivative; the bulk relations use them when
// c4 != 0 (src/helium-ot-bulk.c:30-31, 54-55).  The device form of the same
// term is ot_thermal.cuh.
namespace {
double polylog256(double z, double s) {
  double val = 0.0, zk = 1.0;
  for (int k = 1; k <= 256; k++) {
    zk *= z;
    val += zk / pow((double) k, s);
  }
  return val;
}
double golden_z(double val) {
  const double g = (sqrt(5.0) + 1.0) / 2.0;
  if (val >= polylog256(1.0, 1.5)) return 1.0;
  double a = 0.0, b = 1.0, c = b - (b - a) / g, d = a + (b - a) / g;
  while (fabs(c - d) > 1E-6) {
    double t = val - polylog256(c, 1.5);
    const double fc = t * t;
    t = val - polylog256(d, 1.5);
    const double fd = t * t;
    if (fc < fd) b = d; else a = c;
    c = b - (b - a) / g;
    d = a + (b - a) / g;
  }
  return (b + a) / 2.0;
}
double bose_energy(const dft_ot_functional *o, double rho) {
  const double l3 = dftgpu::bose_lwl3(o->mass, o->temp), z = golden_z(rho * l3);
  return o->c4 * GRID_AUKB * o->temp * (rho * log(z) - polylog256(z, 2.5) / l3);
}
double bose_dEdRho(const dft_ot_functional *o, double rho) {
  const double l3 = dftgpu::bose_lwl3(o->mass, o->temp), rl3 = rho * l3, g32_1 = polylog256(1.0, 1.5);
  if (rl3 >= g32_1) return -o->c4 * GRID_AUKB * (o->temp / l3) * g32_1;
  const double z0 = golden_z(rl3), g12 = polylog256(z0, 0.5), g32 = polylog256(z0, 1.5);
  return o->c4 * GRID_AUKB * o->temp * (log(z0) + rl3 / g12 - g32 / g12);
}
}  // namespace

namespace dftgpu {
bool bose_model(const dft_ot_functional *otf) { return otf->model >= DFT_OT_T400MK && otf->c4 != 0.0; }
double bose_lwl3(double mass, double temp) {
  const double lwl = sqrt(2.0 * M_PI * HBAR * HBAR / (mass * GRID_AUKB * temp));
  return lwl * lwl * lwl;
}
double bose_g32_one() { return polylog256(1.0, 1.5); }
double bose_zmin() { return golden_z(0.0); }
}  // namespace dftgpu

extern "C" {

// ------------------------------------------------------------------ bulk (host)
// src/helium-ot-bulk.c:21-33, 45-57, 143-172, 185-258, 376-434
REAL dft_ot_bulk_energy(dft_ot_functional *o, REAL rho) {
  double e = 0.5 * o->b * rho * rho + 0.5 * o->c2 * rho * rho * rho + (1.0 / 3.0) * o->c3 * rho * rho * rho * rho;
  if (o->c4 != 0.0) e += bose_energy(o, rho);
  return e;
}
REAL dft_ot_bulk_dEdRho(dft_ot_functional *o, REAL rho) {
  double d = o->b * rho + 1.5 * o->c2 * rho * rho + (4.0 / 3.0) * o->c3 * rho * rho * rho;
  if (o->c4 != 0.0) d += bose_dEdRho(o, rho);
  return d;
}
REAL dft_ot_bulk_pressure(dft_ot_functional *o, REAL rho) { return rho * dft_ot_bulk_dEdRho(o, rho) - dft_ot_bulk_energy(o, rho); }
REAL dft_ot_bulk_dPdRho(dft_ot_functional *o, REAL rho) {
  const double h = 1E-7;
  return (dft_ot_bulk_pressure(o, rho + h) - dft_ot_bulk_pressure(o, rho - h)) / (2.0 * h);
}
REAL dft_ot_bulk_density_pressurized(dft_ot_functional *o, REAL pressure) {
  double rho = 1.0, miss = dft_ot_bulk_pressure(o, rho) - pressure;
  for (int it = 0; it < 1000; it++) {
    if (fabs(miss) < 1.0E-12) return rho;
    rho -= miss / dft_ot_bulk_dPdRho(o, rho);
    miss = dft_ot_bulk_pressure(o, rho) - pressure;
  }
  set_error(DFTGPU_ERR_NONFINITE, "bulk density: Newton iteration did not converge");
  return NAN;
}
REAL dft_ot_bulk_chempot_pressurized(dft_ot_functional *o, REAL p) { return dft_ot_bulk_dEdRho(o, dft_ot_bulk_density_pressurized(o, p)); }
REAL dft_ot_bulk_density(dft_ot_functional *o) { return dft_ot_bulk_density_pressurized(o, 0.0); }
REAL dft_ot_bulk_chempot(dft_ot_functional *o) { return dft_ot_bulk_dEdRho(o, dft_ot_bulk_density(o)); }
REAL dft_ot_bulk_chempot2(dft_ot_functional *o) { return dft_ot_bulk_dEdRho(o, o->rho0); }
REAL dft_ot_bulk_compressibility(dft_ot_functional *o, REAL rho) { return 1.0 / (rho * dft_ot_bulk_dPdRho(o, rho)); }
REAL dft_ot_bulk_sound_speed(dft_ot_functional *o, REAL rho) { return 1.0 / sqrt(o->mass * rho * dft_ot_bulk_compressibility(o, rho)); }

REAL dft_ot_bulk_chempot3(dft_ot_functional *o, REAL rho0) { return dft_ot_bulk_dEdRho(o, rho0); }

// Fourier transform of the cored LJ potential at k, by the rectangle rule in
// x = r / sigma from h / sigma to 1000 in steps of 0.01 (src/helium-ot-bulk.c:382-392)
static double lj_transform(const dft_ot_functional *o, double k) {
  const double sg = o->lj_params.sigma, ks = k * sg;
  double lj = 0.0;
  for (double x = o->lj_params.h / sg; x < 1E3; x += 1.0E-2) lj += sin(ks * x) * (pow(x, -11.0) - pow(x, -5.0));
  return lj * (1.0E-2 * 16.0 * M_PI * o->lj_params.epsilon * sg * sg * sg / ks);
}

// kinetic term kin + rho V_LJ(k) + the correlation terms of the uniform
// liquid, summed in this order (src/helium-ot-bulk.c:419-422, 456-459)
static double response_terms(const dft_ot_functional *o, double kin, double k, double rho0) {
  const double kh = k * o->lj_params.h, pi = (3.0 / (kh * kh * kh)) * (sin(kh) - kh * cos(kh));
  return kin + rho0 * lj_transform(o, k) + o->c2 * (2.0 * pi + pi * pi) * rho0 * rho0 +
         2.0 * o->c3 * (pi + pi * pi) * rho0 * rho0 * rho0;
}

// the KC term with prefactor c: c alpha_s rho0 (1 - rho0/rho_0s)^2 exp(-k^2 l_g^2 / 4)
static double kc_term(const dft_ot_functional *o, double c, double k, double rho0) {
  const double f = 1.0 - rho0 / o->rho_0s;
  return c * o->alpha_s * rho0 * f * f * exp(-k * k * o->l_g * o->l_g / 4.0);
}

REAL dft_ot_bulk_istatic(dft_ot_functional *o, REAL *kp, REAL rho0) {
  if (rho0 < 0.0) return 0.0;
  const double k = *kp;
  if (k < 1E-2) return 1E-2;
  double chi = response_terms(o, k * k / (4.0 * o->mass), k, rho0);
  // src/helium-ot-bulk.c:462-463: the KC prefactor is hbar^2 / 2m (no k^2 here)
  if (o->model & DFT_OT_KC) chi += kc_term(o, -(1.0 / (2.0 * o->mass)), k, rho0);
  return chi;
}

REAL dft_ot_bulk_dispersion(dft_ot_functional *o, REAL *kp, REAL rho0) {
  const double k = *kp;
  if (rho0 < 0.0 || k < 1E-3) return 0.0;
  const double t = k * k / o->mass;
  double chi = response_terms(o, t / 4.0, k, rho0);
  if (o->model & DFT_OT_KC) chi += kc_term(o, -(t / 2.0), k, rho0);
  if (o->model & DFT_OT_BACKFLOW) {
    const dft_ot_bf &p = o->bf_params;
    auto vj = [&](double q) {
      const double q2 = q * q, pi32 = pow(M_PI, 1.5);
      return (p.g11 * pow(M_PI / p.a1, 1.5) + p.g12 * (6.0 * p.a1 - q2) * pi32 / (4.0 * pow(p.a1, 3.5))) * exp(-q2 / (4.0 * p.a1)) +
             (p.g21 * pow(M_PI / p.a2, 1.5) + p.g22 * (6.0 * p.a2 - q2) * pi32 / (4.0 * pow(p.a2, 3.5))) * exp(-q2 / (4.0 * p.a2));
    };
    return sqrt(t * chi * (1.0 - rho0 * (vj(0.0) - vj(k))));
  }
  return sqrt(t * chi);
}

// ------------------------------------------------------------------ fused step
static int pc_step_impl(dft_ot_functional *otf, wf *gwf, wf *gwfp, cgrid *P, rgrid *vext, double mu0, double dr, double di) {
  // P = Vext + V_OT[psi] - mu0   (the fills and shifts run inside the potential's pointwise passes)
  DFT_TRY(ot_potential_ex(otf, P, gwf, 1, vext, -mu0, 1.0));
  DFT_TRY(propagate_pc(gwf, gwfp->grid, gwf->grid, P, dr, di));
  // P = (P + Vext + V_OT[psi_p] - mu0) / 2
  DFT_TRY(ot_potential_ex(otf, P, gwfp, 0, vext, -mu0, 0.5));
  return propagate_pc(gwf, gwf->grid, gwf->grid, P, dr, di);
}

static int check_step_args(dft_ot_functional *otf, wf *gwf, wf *gwfp, cgrid *P, rgrid *vext) {
  if (!otf || !gwf || !gwfp || !P) return bad_arg("pc step: NULL argument");
  if (!ot_matches(otf, gwf->grid) || !ot_matches(otf, gwfp->grid) || !ot_matches(otf, P)) return bad_arg("pc step: grid mismatch");
  if (vext && !rc_shape(P, vext)) return bad_arg("pc step: vext mismatch");
  return DFTGPU_OK;
}

int dftgpu_pc_step(dft_ot_functional *otf, wf *gwf, wf *gwfp, cgrid *P, rgrid *vext, double mu0, double dr, double di) {
  DFT_TRY(check_step_args(otf, gwf, gwfp, P, vext));
  return pc_step_impl(otf, gwf, gwfp, P, vext, mu0, dr, di);
}

static int step_with_renorm(dft_ot_functional *otf, wf *gwf, wf *gwfp, cgrid *P, rgrid *vext, double mu0, double dr, double di, int renorm) {
  DFT_TRY(pc_step_impl(otf, gwf, gwfp, P, vext, mu0, dr, di));
  if (renorm) {
    double *slot = reduce_slots();
    DFT_TRY(norm_dev(gwf->grid, slot + 3));
    DFT_TRY(scale_by_norm(gwf->grid, slot + 3, gwf->norm));
  }
  return DFTGPU_OK;
}

int dftgpu_run(dft_ot_functional *otf, wf *gwf, wf *gwfp, cgrid *P, rgrid *vext, double mu0, double dr, double di,
               INT nsteps, int renorm) {
  DFT_TRY(check_step_args(otf, gwf, gwfp, P, vext));
  if (nsteps <= 0) return DFTGPU_OK;
  if (getenv("DFTGPU_NO_GRAPH")) {
    for (INT s = 0; s < nsteps; s++) DFT_TRY(step_with_renorm(otf, gwf, gwfp, P, vext, mu0, dr, di, renorm));
    return DFTGPU_OK;
  }
  GraphCache &G = g_graph;
  const bool hit = G.exec && G.gen == g_generation && G.otf == otf && G.g == gwf && G.gp == gwfp && G.P == P &&
                   G.vext == vext && G.mu0 == mu0 && G.dr == dr && G.di == di && G.renorm == renorm &&
                   G.user == rt().stream && G.k0[0] == gwf->grid->kx0 && G.k0[1] == gwf->grid->ky0 &&
                   G.k0[2] == gwf->grid->kz0;
  if (!hit) {
    // one step eagerly: allocates work buffers and FFT tables outside capture
    DFT_TRY(step_with_renorm(otf, gwf, gwfp, P, vext, mu0, dr, di, renorm));
    if (--nsteps == 0) return DFTGPU_OK;
    if (G.exec) { cudaGraphExecDestroy(G.exec); G.exec = nullptr; }
    if (!G.cap) DFT_CUDA(cudaStreamCreateWithFlags(&G.cap, cudaStreamNonBlocking));
    if (!G.ev) DFT_CUDA(cudaEventCreateWithFlags(&G.ev, cudaEventDisableTiming));
  }
  cudaStream_t user = rt().stream;
  DFT_CUDA(cudaEventRecord(G.ev, user));
  DFT_CUDA(cudaStreamWaitEvent(G.cap, G.ev, 0));
  int rc = DFTGPU_OK;
  if (!hit) {
    cudaGraph_t graph = nullptr;
    rt().stream = G.cap;
    if (cudaStreamBeginCapture(G.cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = DFTGPU_ERR_CUDA;
    if (!rc) {
      rc = step_with_renorm(otf, gwf, gwfp, P, vext, mu0, dr, di, renorm);
      cudaError_t e = cudaStreamEndCapture(G.cap, &graph);
      if (!rc && e != cudaSuccess) { rc = DFTGPU_ERR_CUDA; set_error(rc, "graph capture: %s", cudaGetErrorString(e)); }
    }
    rt().stream = user;
    if (!rc && cudaGraphInstantiate(&G.exec, graph, 0) != cudaSuccess) {
      rc = DFTGPU_ERR_CUDA;
      set_error(rc, "graph instantiate");
      G.exec = nullptr;
    }
    if (graph) cudaGraphDestroy(graph);
    if (!rc) {
      G.gen = g_generation; G.otf = otf; G.g = gwf; G.gp = gwfp; G.P = P; G.vext = vext;
      G.mu0 = mu0; G.dr = dr; G.di = di; G.renorm = renorm; G.user = user;
      G.k0[0] = gwf->grid->kx0; G.k0[1] = gwf->grid->ky0; G.k0[2] = gwf->grid->kz0;
    }
  }
  for (INT s = 0; !rc && s < nsteps; s++)
    if (cudaGraphLaunch(G.exec, G.cap) != cudaSuccess) { rc = DFTGPU_ERR_CUDA; set_error(rc, "graph launch"); }
  cudaEventRecord(G.ev, G.cap);
  cudaStreamWaitEvent(user, G.ev, 0);
  return rc;
}

int dftgpu_energy_report(dft_ot_functional *otf, wf *gwf, rgrid *vext, double *energy, double *natoms, double *mu) {
  if (!otf || !gwf || !ot_matches(otf, gwf->grid)) return bad_arg("energy report: grid mismatch");
  OtPriv *Pv = (OtPriv *) otf->priv;
  cgrid *c = gwf->grid;
  if (!Pv->ed_tmp) Pv->ed_tmp = rgrid_new(c->nx, c->ny, c->nz, c->step, c->prec, "ed");
  if (!Pv->pot_tmp) Pv->pot_tmp = cgrid_new(c->nx, c->ny, c->nz, c->step, c->prec, "pot");
  if (!Pv->ed_tmp || !Pv->pot_tmp) return DFTGPU_ERR_NOMEM;
  double ekin = 0, eint = 0, evx = 0, n = 0, epot = 0;
  DFT_TRY(kinetic_energy(gwf, &ekin));
  DFT_TRY(ot_energy_density(otf, Pv->ed_tmp, gwf));
  DFT_TRY(rintegral(Pv->ed_tmp, &eint));
  if (vext) {   // density is current after ot_energy_density
    DFT_TRY(rbinary(Pv->ed_tmp, otf->density, vext, 0.0, 1));
    DFT_TRY(rintegral(Pv->ed_tmp, &evx));
  }
  n = grid_wf_norm(gwf);
  DFT_TRY(cfill(Pv->pot_tmp, 0.0, 0.0));
  DFT_TRY(ot_potential(otf, Pv->pot_tmp, gwf));          // also refreshes otf->density
  double e_rho_v = 0.0;
  DFT_TRY(rho_dot_re(otf->density, Pv->pot_tmp, &e_rho_v));
  epot = e_rho_v;
  if (energy) *energy = ekin + eint + evx;
  if (natoms) *natoms = n;
  if (mu) *mu = (ekin + epot + evx) / n;
  if (!isfinite(ekin + eint + evx) || !isfinite(n)) { set_error(DFTGPU_ERR_NONFINITE, "energy report: non-finite"); return DFTGPU_ERR_NONFINITE; }
  return DFTGPU_OK;
}

}  // extern "C"
