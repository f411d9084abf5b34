// Runtime control, grid objects, elementwise operations, FP64 reductions and
// the split-operator wave-function propagator.
//
// The libgrid functions restated here have no source in the reference tree;
// their meaning follows their libdft call sites (cited per entry point in
// include/dftgpu.h) and the conventions below:
//   x_i = (i - nx/2) step - x0;  k_i = 2 pi (i or i - n) / (n step)
//   S(V, dt) = exp(-i V dt/2) F^-1 exp(-i hbar k^2 dt / 2m) F exp(-i V dt/2)
//   v = (hbar/m) Im(psi^* D psi) / max(|psi|^2, eps), D = central difference.
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ops.cuh"
#include "grid_internal.cuh"

namespace dftgpu {

thread_local int g_last_error = 0;
static thread_local char g_last_msg[512] = "";

void set_error(int code, const char *fmt, ...) {
  g_last_error = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_msg, sizeof(g_last_msg), fmt, ap);
  va_end(ap);
  if (getenv("DFTGPU_VERBOSE")) fprintf(stderr, "libdftgpu: error %d: %s\n", code, g_last_msg);
}

}  // namespace dftgpu

extern "C" const char *dftgpu_last_error_message(void) { return dftgpu::g_last_msg; }

namespace dftgpu {

Runtime &rt() {
  static Runtime r;
  return r;
}

int ensure_device() {
  Runtime &R = rt();
  if (R.device >= 0) return DFTGPU_OK;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error(DFTGPU_ERR_NODEVICE, "no CUDA device available");
    return DFTGPU_ERR_NODEVICE;
  }
  DFT_CUDA(cudaSetDevice(0));
  R.device = 0;
  cudaDeviceProp p;
  DFT_CUDA(cudaGetDeviceProperties(&p, 0));
  R.num_sms = p.multiProcessorCount;
  R.max_smem_optin = p.sharedMemPerBlockOptin;
  return DFTGPU_OK;
}

// ------------------------------------------------------------------ parallel branches
// Auxiliary streams for independent transforms (par_for in ops.cuh).  The
// number of streams used (work stream included) is DFTGPU_STREAMS, default 2.
int par_streams(cudaStream_t **aux, cudaEvent_t **ev) {
  static int n = -1;
  static cudaStream_t s[PAR_MAX - 1];
  static cudaEvent_t e[PAR_MAX];
  if (n < 0) {
    const char *v = getenv("DFTGPU_STREAMS");
    int want = v ? atoi(v) : 2;
    if (want < 1) want = 1;
    if (want > PAR_MAX) want = PAR_MAX;
    for (int i = 0; i < want - 1; i++)
      if (cudaStreamCreateWithFlags(&s[i], cudaStreamNonBlocking) != cudaSuccess) { want = i + 1; break; }
    for (int i = 0; i < want; i++)
      if (cudaEventCreateWithFlags(&e[i], cudaEventDisableTiming) != cudaSuccess) { want = 1; break; }
    n = want;
  }
  *aux = s;
  *ev = e;
  return n;
}

// ------------------------------------------------------------------ profiler
namespace {
struct ProfRec { cudaEvent_t a, b; const char *name; double bytes; int kernels; };
bool g_prof = false;
std::vector<ProfRec> g_recs;      // records of the current profile window
std::vector<cudaEvent_t> g_pool;  // spare events
size_t g_used = 0;

cudaEvent_t pool_event() {
  if (g_used < g_pool.size()) return g_pool[g_used++];
  cudaEvent_t e;
  cudaEventCreate(&e);
  g_pool.push_back(e);
  g_used++;
  return e;
}
}  // namespace

bool prof_on() { return g_prof; }

int prof_begin() {
  ProfRec r;
  r.a = pool_event();
  r.b = pool_event();
  r.name = nullptr;
  r.bytes = 0;
  r.kernels = 0;
  cudaEventRecord(r.a, rt().stream);
  g_recs.push_back(r);
  return (int) g_recs.size() - 1;
}

void prof_end(int id, const char *name, double bytes, int kernels) {
  ProfRec &r = g_recs[id];
  r.name = name;
  r.bytes = bytes;
  r.kernels = kernels;
  cudaEventRecord(r.b, rt().stream);
}

int prof_enable(int on) {
  DFT_TRY(ensure_device());
  g_prof = on != 0;
  g_recs.clear();
  g_used = 0;
  return DFTGPU_OK;
}

// JSON {"class": {"launches": n, "ms": t, "bytes": b}, ...}; launches counts
// kernel launches (a scope may hold several, e.g. the two-kernel reduction)
int prof_report(char *buf, size_t len) {
  DFT_CUDA(cudaDeviceSynchronize());
  struct Acc { const char *name; long n; double ms, bytes; };
  std::vector<Acc> acc;
  for (const ProfRec &r : g_recs) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) { cudaGetLastError(); continue; }
    size_t k = 0;
    while (k < acc.size() && strcmp(acc[k].name, r.name)) k++;
    if (k == acc.size()) acc.push_back({r.name, 0, 0.0, 0.0});
    acc[k].n += r.kernels;
    acc[k].ms += ms;
    acc[k].bytes += r.bytes;
  }
  size_t off = (size_t) snprintf(buf, len, "{");
  for (size_t k = 0; k < acc.size() && off < len; k++)
    off += (size_t) snprintf(buf + off, len - off, "%s\"%s\": {\"launches\": %ld, \"ms\": %.6f, \"bytes\": %.0f}",
                             k ? ", " : "", acc[k].name, acc[k].n, acc[k].ms, acc[k].bytes);
  if (off < len) snprintf(buf + off, len - off, "}");
  return DFTGPU_OK;
}

static double *g_slots = nullptr;
static double *g_partials = nullptr;

double *reduce_slots() {
  if (!g_slots) {
    if (cudaMalloc(&g_slots, 64 * sizeof(double)) != cudaSuccess) return nullptr;
    cudaMemset(g_slots, 0, 64 * sizeof(double));
  }
  return g_slots;
}

int reduce_partials(double **buf, size_t *n) {
  if (!g_partials) DFT_CUDA(cudaMalloc(&g_partials, 8 * RED_BLOCKS * sizeof(double)));
  if (!reduce_slots()) { set_error(DFTGPU_ERR_NOMEM, "reduction slots"); return DFTGPU_ERR_NOMEM; }
  *buf = g_partials;
  *n = 8 * RED_BLOCKS;
  return DFTGPU_OK;
}

// ------------------------------------------------------------------ buffers
void *dev_alloc(size_t bytes) {
  void *p = nullptr;
  if (ensure_device() != DFTGPU_OK) return nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
    cudaGetLastError();
    set_error(DFTGPU_ERR_NOMEM, "cudaMalloc(%zu) failed", bytes);
    return nullptr;
  }
  return p;
}

void dev_free(void *p) { if (p) cudaFree(p); }

// Grid dimensions: 2^a 3^b 5^c in [2, FFT_MAX_N]; x and y may be odd (libdft's
// largest production grid is 729 x 384 x 384, examples/gas-bubble/config.h:56),
// z must be even (real fields are transformed as packed pairs along z).  A 1-D
// grid, nx = ny = 1 (libdft's 1-D effective model, src/ot.c:133-217; its
// driver examples/1d-bubble/bubble-1d.c:25 runs nz = 4096), takes nz up to
// FFT_MAX_LINE.
int check_dims(INT nx, INT ny, INT nz) {
  const bool one_d = nx == 1 && ny == 1;
  INT d[3] = { nx, ny, nz };
  for (int i = 0; i < 3; i++) {
    INT m = d[i];
    const INT lo = one_d && i < 2 ? 1 : 2, hi = one_d ? FFT_MAX_LINE : FFT_MAX_N;
    if (m < lo || m > hi || (i == 2 && (m & 1))) {
      set_error(DFTGPU_ERR_SIZE, "grid dimension %ld must be in [2, %d] (nz up to %d with nx = ny = 1)%s", (long) m,
                FFT_MAX_N, FFT_MAX_LINE, i == 2 ? " and even along z" : "");
      return DFTGPU_ERR_SIZE;
    }
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    while (m % 5 == 0) m /= 5;
    if (m != 1) {
      set_error(DFTGPU_ERR_SIZE, "grid dimension %ld is not of the form 2^a 3^b 5^c", (long) d[i]);
      return DFTGPU_ERR_SIZE;
    }
  }
  return DFTGPU_OK;
}

// ------------------------------------------------------------------ elementwise
template <typename T> int k_fill(T *p, size_t n, T v) {
  return launch_each(n, [=] __device__(size_t i) { p[i] = v; });
}
template <typename T> int k_axpb(T *p, size_t n, T a, T b) {   // p = a p + b
  return launch_each(n, [=] __device__(size_t i) { p[i] = a * p[i] + b; });
}

// ------------------------------------------------------------------ propagation
// The propagation passes' functors use the split interface of the line
// kernels: PhaseLoad fetches psi and V of all of a thread's elements before
// any phase factor is formed; PhaseStore prefetches its V lines into L2
// before the transform, so the loads after it do not wait on DRAM.
template <typename T> struct PhaseLoad {   // psi * exp(-i V dt / 2)
  typedef typename cplx_t<T>::type C;
  static constexpr bool kSplit = true, kAhead = true;
  struct Raw { C p, v; };
  const C *psi; const C *V; int ny, nz; T hr, hi;   // (hr, hi) = dt / 2
  __device__ void prefetch_lines(int x, int y0, int nl, int) const {
    const size_t o = ((size_t) x * ny + y0) * nz, n = (size_t) nl * nz * sizeof(C);
    if (threadIdx.x == 0) prefetch_bulk_l2(psi + o, n);
    if (threadIdx.x == 32) prefetch_bulk_l2(V + o, n);
  }
  __device__ Raw fetch(int x, int y, int e) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    return Raw{ psi[i], V[i] };
  }
  __device__ C cook(const Raw &r) const {
    // -i V dt/2 = (Im(V dt/2), -Re(V dt/2))
    const C z = mk<T>(r.v.x * hi + r.v.y * hr, -(r.v.x * hr - r.v.y * hi));
    return mul_cexp(r.p, z);
  }
  __device__ C operator()(int x, int y, int e) const { return cook(fetch(x, y, e)); }
};
template <typename T> struct PhaseStore {
  typedef typename cplx_t<T>::type C;
  static constexpr bool kSplit = true, kBoundedStore = true;
  C *psi; const C *V; int ny, nz; T hr, hi;
  __device__ void prefetch(int x, int y, int e) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    if ((i * sizeof(C)) % 32 == 0) prefetch_l2(V + i);   // one per 32-byte sector
  }
  __device__ void operator()(int x, int y, int e, C val) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    const C v = __ldg(V + i);   // read-only path: the loads may move ahead of the psi stores
    C z = mk<T>(v.x * hi + v.y * hr, -(v.x * hr - v.y * hi));
    psi[i] = mul_cexp(val, z);
  }
};

// Functors of the factorised kinetic passes (FP32 register FFTs): the wave
// function stays in its [x][y][z] layout; (a, b, e) = (x, y, z) for the z
// rows, (x, z, y) for the y lines and (y, z, x) for the x lines.
struct RowStoreF {   // z rows
  float2 *f; int ny, nz;
  __device__ void operator()(int x, int y, int z, float2 v) const { f[((size_t) x * ny + y) * nz + z] = v; }
};
// (32-bit element offsets: grids of up to 2^31 points; a 64-bit address per
// element of a strided line costs two registers each across the transform)
struct LineYF {      // y lines, B consecutive z per CTA
  static constexpr bool kAhead = true;
  float2 *f; int ny, nz;
  __device__ void prefetch_lines(int x, int z0, int nl, int ne) const {   // one run of nl values per y
    for (int y = threadIdx.x; y < ne; y += blockDim.x) prefetch_bulk_l2(f + ((unsigned) (x * ny + y) * (unsigned) nz + z0), (size_t) nl * sizeof(float2));
  }
  __device__ float2 operator()(int x, int z, int y) const { return f[(unsigned) (x * ny + y) * (unsigned) nz + z]; }
  __device__ void operator()(int x, int z, int y, float2 v) const { f[(unsigned) (x * ny + y) * (unsigned) nz + z] = v; }
};
struct LineXF {      // x lines, B consecutive z per CTA
  static constexpr bool kAhead = true;
  const float2 *f; int nx, ny, nz;
  __device__ void prefetch_lines(int y, int z0, int nl, int ne) const {   // one run of nl values per x
    for (int x = threadIdx.x; x < ne; x += blockDim.x) prefetch_bulk_l2(f + ((unsigned) (x * ny + y) * (unsigned) nz + z0), (size_t) nl * sizeof(float2));
  }
  __device__ float2 operator()(int y, int z, int x) const { return f[(unsigned) (x * ny + y) * (unsigned) nz + z]; }
};
struct PhaseStoreXF {   // x lines: psi <- v exp(-i V dt / 2)
  static constexpr bool kSplit = true, kBoundedStore = true;
  float2 *psi; const float2 *V; int ny, nz; float hr, hi;
  __device__ void prefetch(int y, int z, int x) const {
    const unsigned i = (unsigned) (x * ny + y) * (unsigned) nz + z;
    if ((i & 3) == 0) prefetch_l2(V + i);   // one per 32-byte sector
  }
  __device__ void operator()(int y, int z, int x, float2 val) const {
    const unsigned i = (unsigned) (x * ny + y) * (unsigned) nz + z;
    const float2 v = __ldg(V + i);
    psi[i] = mul_cexp(val, make_float2(v.x * hi + v.y * hr, -(v.x * hr - v.y * hi)));
  }
};

// The factorised kinetic passes fit when every axis is a register-FFT length
// and each pass's line count is a multiple of its CTA's lines.
static bool kin_fits(int nx, int ny, int nz) {
  auto ok = [](int n) { return n == 64 || n == 128 || n == 256 || n == 512; };
  auto lines = [](int n) { return n == 64 ? 32 : 256 / (n / 16); };   // ff::Shape<n>::B
  return !generic_fft_only() && ok(nx) && ok(ny) && ok(nz) && ny % lines(nz) == 0 && nz % lines(ny) == 0 &&
         nz % lines(nx) == 0;
}

// dst = S(V, dt) src in three passes (FP32, register-FFT lengths):
//   z: rows of src times exp(-i V dt/2), FFT_z, exp(cdt (kz - kz0)^2)/nz, FFT_z^-1 -> dst
//   y: FFT_y, exp(cdt (ky - ky0)^2)/ny, FFT_y^-1 (in place)
//   x: FFT_x, exp(cdt (kx - kx0)^2)/nx, FFT_x^-1, times exp(-i V dt/2) (in place)
// The same operator as the five-pass form below (F^-1 K F factorises per
// axis); it moves the wave function through HBM three times instead of five,
// but its strided y and x passes (128-byte runs, every run in another DRAM
// page) run at 2.6-3.4 TB/s against 5-6.7 for the contiguous passes of the
// five-pass form: 317 against 300 us per propagation at 256^3, so it is
// opt-in (DFTGPU_FACTORISED_PROP=1).
static int strang_factorised(wf *g, cgrid *dst, cgrid *src, cgrid *V, double dr, double di) {
  const int nx = (int) src->nx, ny = (int) src->ny, nz = (int) src->nz;
  const double m = g->mass, step = src->step;
  const cgrid *mg = g->grid;   // moving-background momentum of the wave function
  const float2 cdt = make_float2((float) (di / (2.0 * m)), (float) (-dr / (2.0 * m)));   // -i dt / 2m
  const float hr = (float) (0.5 * dr), hi = (float) (0.5 * di);
  const double nb = (double) nx * ny * nz * sizeof(float2);
  float2 *out = (float2 *) dst->value;
  const float2 *pot = (const float2 *) V->value;
  PhaseLoad<float> ld{(const float2 *) src->value, pot, ny, nz, hr, hi};
  RowStoreF sz{out, ny, nz};
  DFT_TRY(launch_kin_pass<ff::MAP_E>(nz, nx, ny, cdt, (float) (2.0 * M_PI / (nz * step)), (float) mg->kz0, ld, sz,
                                     "prop_kin_z", 3.0 * nb));
  LineYF ly{out, ny, nz};
  DFT_TRY(launch_kin_pass<ff::MAP_L>(ny, nx, nz, cdt, (float) (2.0 * M_PI / (ny * step)), (float) mg->ky0, ly, ly,
                                     "prop_kin_y", 2.0 * nb));
  LineXF lx{out, nx, ny, nz};
  PhaseStoreXF sx{out, pot, ny, nz, hr, hi};
  return launch_kin_pass<ff::MAP_L>(nx, ny, nz, cdt, (float) (2.0 * M_PI / (nx * step)), (float) mg->kx0, lx, sx,
                                    "prop_kin_x", 3.0 * nb);
}

// dst = S(V, dt) src, through the wave function's spectral scratch buffer
template <typename T> int strang(wf *g, cgrid *dst, cgrid *src, cgrid *V, double dr, double di) {
  typedef typename cplx_t<T>::type C;
  const int nx = (int) src->nx, ny = (int) src->ny, nz = (int) src->nz;
  const int cn = g->propagator == WF_2ND_ORDER_CN;
  if constexpr (std::is_same<T, float>::value) {
    if (!cn && factorised_propagation() && kin_fits(nx, ny, nz)) return strang_factorised(g, dst, src, V, dr, di);
  }
  C *spec = (C *) wf_spec(g);
  if (!spec) return DFTGPU_ERR_NOMEM;
  const T hr = (T) (0.5 * dr), hi = (T) (0.5 * di);
  PhaseLoad<T> ld{(const C *) src->value, (const C *) V->value, ny, nz, hr, hi};
  SpecStoreZ<T> sz{spec, nx, ny};
  DFT_TRY((launch_lines<T, LINE_C2C, 1, 0>(nz, nx, ny, (T) -1, ld, sz)));
  DFT_TRY(ypass<T>(spec, nx, ny, nz, (T) -1));
  KinArgs<T> K;
  const double m = g->mass;
  const cgrid *mg = g->grid;   // moving-background momentum of the wave function
  kin_args<T>(K, nx, ny, nz, src->step, make_double2(di / (2.0 * m), -dr / (2.0 * m)),   // -i dt / 2m
              mg->kx0, mg->ky0, mg->kz0, spec);
  K.cn = cn;
  DFT_TRY(launch_xkinetic<T>(K));
  DFT_TRY(ypass<T>(spec, nx, ny, nz, (T) 1));
  SpecLoadZ<T> lz{spec, nx, ny};
  PhaseStore<T> st{(C *) dst->value, (const C *) V->value, ny, nz, hr, hi};
  return launch_lines<T, LINE_C2C, 0, 1>(nz, nx, ny, (T) 1, lz, st);
}

int propagate(wf *g, cgrid *dst, cgrid *src, cgrid *V, double dr, double di) {
  if (!g || !dst || !src || !V) { set_error(DFTGPU_ERR_ARG, "propagate: NULL argument"); return DFTGPU_ERR_ARG; }
  if (V->prec != src->prec || dst->prec != src->prec || V->nx != src->nx || V->ny != src->ny || V->nz != src->nz) {
    set_error(DFTGPU_ERR_ARG, "propagate: potential / wave function mismatch");
    return DFTGPU_ERR_ARG;
  }
  return src->prec == DFTGPU_FP32 ? strang<float>(g, dst, src, V, dr, di) : strang<double>(g, dst, src, V, dr, di);
}

// ------------------------------------------------------------------ absorbing boundary
// weight of the boundary layer along one axis: (l - i) / l below l, (i - h + 1) / (n - h) from h on
__device__ __forceinline__ double abs_ramp(int i, int l, int h, int n) {
  if (i < l) return (double) (l - i) / (double) l;
  if (i >= h) return (double) (i - h + 1) / (double) (n - h);
  return 0.0;
}

template <typename T> static int absorb_add_t(cgrid *dst, const cgrid *pot, const cgrid *psi, const AbsBoundary &b,
                                              double amp, double rho0) {
  typedef typename cplx_t<T>::type C;
  C *d = (C *) dst->value;
  const C *p = (const C *) pot->value, *w = (const C *) psi->value;
  const int nx = (int) psi->nx, ny = (int) psi->ny, nz = (int) psi->nz;
  const int lx = b.lo[0], hx = b.hi[0], ly = b.lo[1], hy = b.hi[1], lz = b.lo[2], hz = b.hi[2];
  const double irho = 1.0 / rho0;
  return launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
    double lam = abs_ramp(x, lx, hx, nx);
    lam = fmax(lam, abs_ramp(y, ly, hy, ny));
    lam = fmax(lam, abs_ramp(z, lz, hz, nz));
    C v = p[i];
    if (lam > 0.0) {
      const C a = w[i];
      v.y -= (T) (amp * lam * (((double) a.x * a.x + (double) a.y * a.y) * irho - 1.0));
    }
    d[i] = v;
  }, 5.0 * gsize(psi) * sizeof(T), "absorb");
}

int absorb_add(cgrid *dst, const cgrid *pot, const cgrid *psi, const AbsBoundary &b, double amp, double rho0) {
  return psi->prec == DFTGPU_FP32 ? absorb_add_t<float>(dst, pot, psi, b, amp, rho0)
                                  : absorb_add_t<double>(dst, pot, psi, b, amp, rho0);
}

int propagate_pc(wf *g, cgrid *dst, cgrid *src, cgrid *V, double dr, double di) {
  WfPriv *p = (WfPriv *) g->priv;
  if (!p || !p->abs.on) return propagate(g, dst, src, V, dr, di);
  if (!p->vtot) {
    const cgrid *c = g->grid;
    p->vtot = (cgrid *) calloc(1, sizeof(cgrid));
    if (!p->vtot) return DFTGPU_ERR_NOMEM;
    *p->vtot = *c;
    p->vtot->value = dev_alloc(gsize(c) * 2 * elem_size(c->prec));
    if (!p->vtot->value) { free(p->vtot); p->vtot = nullptr; return DFTGPU_ERR_NOMEM; }
  }
  DFT_TRY(absorb_add(p->vtot, V, src, p->abs, p->abs.amp, p->abs.rho0));
  return propagate(g, dst, src, p->vtot, dr, di);
}

// ------------------------------------------------------------------ spectra of psi
template <typename T> int cfft3_forward(cgrid *src, typename cplx_t<T>::type *spec) {
  const int nx = (int) src->nx, ny = (int) src->ny, nz = (int) src->nz;
  CplxLoad<T> ld{(const typename cplx_t<T>::type *) src->value, ny, nz};
  SpecStoreZ<T> sz{spec, nx, ny};
  DFT_TRY((launch_lines<T, LINE_C2C, 1, 0>(nz, nx, ny, (T) -1, ld, sz)));
  DFT_TRY(ypass<T>(spec, nx, ny, nz, (T) -1));
  SpecLineXT<T> io{spec, nx, ny};
  return launch_lines<T, LINE_C2C, 0, 0>(nx, nz, ny, (T) -1, io, io);
}

template <typename T> int kinetic_energy_t(wf *g, double *out) {
  typedef typename cplx_t<T>::type C;
  cgrid *c = g->grid;
  C *spec = (C *) wf_spec(g);
  if (!spec) return DFTGPU_ERR_NOMEM;
  DFT_TRY(cfft3_forward<T>(c, spec));
  const int nx = (int) c->nx, ny = (int) c->ny, nz = (int) c->nz;
  const double dkx = 2.0 * M_PI / (nx * c->step), dky = 2.0 * M_PI / (ny * c->step), dkz = 2.0 * M_PI / (nz * c->step);
  const double k0x = c->kx0, k0y = c->ky0, k0z = c->kz0;   // kinetic energy in the moving frame
  const double dv = c->step * c->step * c->step;
  const double scale = 1.0 / (2.0 * g->mass) * dv / ((double) nx * ny * nz);
  const size_t n = (size_t) nx * ny * nz;
  const double h = c->step;
  // spectral layout [kz][kx][ky]; Crank-Nicolson wave functions: the
  // finite-difference kinetic operator that propagator steps with,
  // (2 sin(k h / 2) / h)^2 per axis in place of k^2
  if (g->propagator == WF_2ND_ORDER_CN)
    return reduce_host<1>(n, [=] __device__(size_t i, double *v) {
      const int ky = (int) (i % ny), kx = (int) ((i / ny) % nx), kz = (int) (i / ((size_t) nx * ny));
      const double a = 2.0 * sin(0.5 * h * (kfreq(kx, nx, dkx) - k0x)) / h;
      const double b = 2.0 * sin(0.5 * h * (kfreq(ky, ny, dky) - k0y)) / h;
      const double cc = 2.0 * sin(0.5 * h * (kfreq(kz, nz, dkz) - k0z)) / h;
      const C s = spec[i];
      v[0] = (a * a + b * b + cc * cc) * ((double) s.x * s.x + (double) s.y * s.y);
    }, out, scale);
  return reduce_host<1>(n, [=] __device__(size_t i, double *v) {
    const int ky = (int) (i % ny), kx = (int) ((i / ny) % nx), kz = (int) (i / ((size_t) nx * ny));
    const double a = kfreq(kx, nx, dkx) - k0x, b = kfreq(ky, ny, dky) - k0y, cc = kfreq(kz, nz, dkz) - k0z;
    const C s = spec[i];
    v[0] = (a * a + b * b + cc * cc) * ((double) s.x * s.x + (double) s.y * s.y);
  }, out, scale);
}

int kinetic_energy(wf *g, double *out) {
  return g->grid->prec == DFTGPU_FP32 ? kinetic_energy_t<float>(g, out) : kinetic_energy_t<double>(g, out);
}

// sum |psi|^2 dV: each reduction item is a run of 8 consecutive values summed
// in the grid's precision (FP32: within 8 ulps of the run's sum), runs are
// accumulated in FP64 -- one FP64 add per 8 values instead of per value.  The
// last run is short when 8 does not divide the count (odd x and y sizes).
template <typename T> int norm_dev_t(cgrid *c, double *slot) {
  typedef typename cplx_t<T>::type C;
  const C *p = (const C *) c->value;
  const double dv = c->step * c->step * c->step;
  const size_t n = gsize(c), runs = (n + 7) / 8;
  return reduce_dev<1>(runs, [=] __device__(size_t r, double *v) {
    const C *q = p + 8 * r;
    T s = (T) 0;
    if (8 * r + 8 <= n) {
#pragma unroll
      for (int k = 0; k < 8; k++) { const C z = q[k]; s += z.x * z.x + z.y * z.y; }
    } else {
      for (size_t k = 0; 8 * r + k < n; k++) { const C z = q[k]; s += z.x * z.x + z.y * z.y; }
    }
    v[0] = (double) s;
  }, slot, dv);
}

int norm_dev(cgrid *c, double *slot) {
  return c->prec == DFTGPU_FP32 ? norm_dev_t<float>(c, slot) : norm_dev_t<double>(c, slot);
}

// psi *= sqrt(target / norm) with norm read from the device slot
// factor sqrt(target / norm) computed once in FP64, stored in the grid's precision
template <typename T> __global__ void norm_factor_kernel(const double *slot, double target, T *factor) {
  *factor = (T) sqrt(target / slot[0]);
}

template <typename T> int scale_by_norm_t(cgrid *c, const double *slot, double target) {
  typedef typename cplx_t<T>::type C;
  C *p = (C *) c->value;
  T *factor = (T *) (reduce_slots() + 48);   // scratch slot, written here and read below on the same stream
  {
    ProfScope prof("reduce_fp64", 0.0);
    norm_factor_kernel<T><<<1, 1, 0, rt().stream>>>(slot, target, factor);
    DFT_CHECK_LAUNCH();
  }
  return launch_each(gsize(c), [=] __device__(size_t i) {
    const T f = *factor;
    C z = p[i];
    z.x *= f; z.y *= f;
    p[i] = z;
  }, 4.0 * gsize(c) * sizeof(T), "normalize");
}

int scale_by_norm(cgrid *c, const double *slot, double target) {
  return c->prec == DFTGPU_FP32 ? scale_by_norm_t<float>(c, slot, target) : scale_by_norm_t<double>(c, slot, target);
}

template <typename T> int velocity_t(wf *g, rgrid *vx, rgrid *vy, rgrid *vz, double eps) {
  typedef typename cplx_t<T>::type C;
  cgrid *c = g->grid;
  const C *p = (const C *) c->value;
  T *out[3] = { (T *) vx->value, (T *) vy->value, (T *) vz->value };
  T *ox = out[0], *oy = out[1], *oz = out[2];
  const int nx = (int) c->nx, ny = (int) c->ny, nz = (int) c->nz;
  const double f = 1.0 / (g->mass * 2.0 * c->step);
  return launch_each(gsize(c), [=] __device__(size_t i) {
    const int k = (int) (i % nz), j = (int) ((i / nz) % ny), x = (int) (i / ((size_t) ny * nz));
    const C z = p[i];
    double rho = (double) z.x * z.x + (double) z.y * z.y;
    if (rho < eps) rho = eps;
    const double g0 = f / rho;
    const size_t ixp = ((size_t) ((x + 1) % nx) * ny + j) * nz + k, ixm = ((size_t) ((x - 1 + nx) % nx) * ny + j) * nz + k;
    const size_t iyp = ((size_t) x * ny + (j + 1) % ny) * nz + k, iym = ((size_t) x * ny + (j - 1 + ny) % ny) * nz + k;
    const size_t izp = ((size_t) x * ny + j) * nz + (k + 1) % nz, izm = ((size_t) x * ny + j) * nz + (k - 1 + nz) % nz;
    C d;
    d = p[ixp] - p[ixm]; ox[i] = (T) (g0 * ((double) z.x * d.y - (double) z.y * d.x));
    d = p[iyp] - p[iym]; oy[i] = (T) (g0 * ((double) z.x * d.y - (double) z.y * d.x));
    d = p[izp] - p[izm]; oz[i] = (T) (g0 * ((double) z.x * d.y - (double) z.y * d.x));
  });
}

// forward r2c of a real grid to the host, in the oracle's [x][y][kz] order
template <typename T> static int rspectrum_t(rgrid *g, double *host) {
  typedef typename cplx_t<T>::type C;
  const int nx = (int) g->nx, ny = (int) g->ny, nz = (int) g->nz, nzh = nz / 2 + 1;
  const size_t ns = (size_t) nzh * nx * ny;
  C *spec = (C *) dev_alloc(ns * sizeof(C));
  if (!spec) return DFTGPU_ERR_NOMEM;
  RealPairLoad<T> ld{(const T *) g->value, ny, nz};
  int rc = rfft_zy<T>(ld, spec, nx, ny, nz);
  SpecLineXT<T> io{spec, nx, ny};
  if (!rc) rc = launch_lines<T, LINE_C2C, 0, 0>(nx, nzh, ny, (T) -1, io, io);
  std::vector<C> h(ns);
  if (!rc && (cudaMemcpyAsync(h.data(), spec, ns * sizeof(C), cudaMemcpyDeviceToHost, rt().stream) != cudaSuccess ||
              cudaStreamSynchronize(rt().stream) != cudaSuccess)) rc = DFTGPU_ERR_CUDA;
  dev_free(spec);
  if (rc) return rc;
  for (int kz = 0; kz < nzh; kz++)
    for (int x = 0; x < nx; x++)
      for (int y = 0; y < ny; y++) {
        const C v = h[((size_t) kz * nx + x) * ny + y];
        const size_t o = ((size_t) x * ny + y) * nzh + kz;
        host[2 * o] = v.x; host[2 * o + 1] = v.y;
      }
  return DFTGPU_OK;
}

int rspectrum(rgrid *g, double *host) {
  return g->prec == DFTGPU_FP32 ? rspectrum_t<float>(g, host) : rspectrum_t<double>(g, host);
}

int velocity(wf *g, rgrid *vx, rgrid *vy, rgrid *vz, double eps) {
  return g->grid->prec == DFTGPU_FP32 ? velocity_t<float>(g, vx, vy, vz, eps) : velocity_t<double>(g, vx, vy, vz, eps);
}

// ------------------------------------------------------------------ host copies
template <typename T> static int copy_out(const void *dev, double *host, size_t n) {
  if (sizeof(T) == 8) { DFT_CUDA(cudaMemcpyAsync(host, dev, n * 8, cudaMemcpyDeviceToHost, rt().stream)); }
  else {
    std::vector<float> tmp(n);
    DFT_CUDA(cudaMemcpyAsync(tmp.data(), dev, n * 4, cudaMemcpyDeviceToHost, rt().stream));
    DFT_CUDA(cudaStreamSynchronize(rt().stream));
    for (size_t i = 0; i < n; i++) host[i] = tmp[i];
  }
  DFT_CUDA(cudaStreamSynchronize(rt().stream));
  return DFTGPU_OK;
}

template <typename T> static int copy_in(void *dev, const double *host, size_t n) {
  if (sizeof(T) == 8) { DFT_CUDA(cudaMemcpyAsync(dev, host, n * 8, cudaMemcpyHostToDevice, rt().stream)); }
  else {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; i++) tmp[i] = (float) host[i];
    DFT_CUDA(cudaMemcpyAsync(dev, tmp.data(), n * 4, cudaMemcpyHostToDevice, rt().stream));
  }
  DFT_CUDA(cudaStreamSynchronize(rt().stream));
  return DFTGPU_OK;
}

int copy_values_out(int prec, const void *dev, double *host, size_t n) {
  DFT_TRY(prec == DFTGPU_FP32 ? copy_out<float>(dev, host, n) : copy_out<double>(dev, host, n));
  return fused_zy_fault();
}
int copy_values_in(int prec, void *dev, const double *host, size_t n) {
  return prec == DFTGPU_FP32 ? copy_in<float>(dev, host, n) : copy_in<double>(dev, host, n);
}

// ------------------------------------------------------------------ generic real ops
int rfill(rgrid *g, double v) {
  return g->prec == DFTGPU_FP32 ? k_fill<float>((float *) g->value, gsize(g), (float) v) : k_fill<double>((double *) g->value, gsize(g), v);
}
int raxpb(rgrid *g, double a, double b) {
  return g->prec == DFTGPU_FP32 ? k_axpb<float>((float *) g->value, gsize(g), (float) a, (float) b)
                                : k_axpb<double>((double *) g->value, gsize(g), a, b);
}
int cfill(cgrid *g, double re, double im) {
  if (g->prec == DFTGPU_FP32) { float2 v = make_float2((float) re, (float) im); float2 *p = (float2 *) g->value;
    return launch_each(gsize(g), [=] __device__(size_t i) { p[i] = v; }); }
  double2 v = make_double2(re, im); double2 *p = (double2 *) g->value;
  return launch_each(gsize(g), [=] __device__(size_t i) { p[i] = v; });
}
template <typename T> static int cmuladd_t(cgrid *g, double mr, double mi, double ar, double ai) {
  typedef typename cplx_t<T>::type C;
  C *p = (C *) g->value;
  const C m = mk<T>((T) mr, (T) mi), a = mk<T>((T) ar, (T) ai);
  return launch_each(gsize(g), [=] __device__(size_t i) { p[i] = cmul(p[i], m) + a; }, 4.0 * gsize(g) * sizeof(T),
                     "cgrid_muladd");
}
int cmuladd(cgrid *g, double mr, double mi, double ar, double ai) {
  return g->prec == DFTGPU_FP32 ? cmuladd_t<float>(g, mr, mi, ar, ai) : cmuladd_t<double>(g, mr, mi, ar, ai);
}

// mode 0: dst.re = src (im = 0); 1: dst.re += src; 2: dst.im += src
template <typename T> static int r2c_t(cgrid *d, rgrid *s, int mode) {
  typedef typename cplx_t<T>::type C;
  C *p = (C *) d->value;
  const T *q = (const T *) s->value;
  return launch_each(gsize(d), [=] __device__(size_t i) {
    C v = p[i];
    if (mode == 0) { v.x = q[i]; v.y = (T) 0; }
    else if (mode == 1) v.x += q[i];
    else v.y += q[i];
    p[i] = v;
  }, (mode == 0 ? 3.0 : 5.0) * gsize(d) * sizeof(T), "real_to_complex");
}
int real_to_complex(cgrid *d, rgrid *s, int mode) {
  return d->prec == DFTGPU_FP32 ? r2c_t<float>(d, s, mode) : r2c_t<double>(d, s, mode);
}

// op 0: d = a + b; 1: d = a * b; 2: d += c a; 3: d += c a b
template <typename T> static int rbin_t(rgrid *d, rgrid *a, rgrid *b, double c, int op) {
  T *pd = (T *) d->value;
  const T *pa = (const T *) a->value, *pb = b ? (const T *) b->value : nullptr;
  const T cc = (T) c;
  return launch_each(gsize(d), [=] __device__(size_t i) {
    if (op == 0) pd[i] = pa[i] + pb[i];
    else if (op == 1) pd[i] = pa[i] * pb[i];
    else if (op == 2) pd[i] += cc * pa[i];
    else pd[i] += cc * pa[i] * pb[i];
  });
}
int rbinary(rgrid *d, rgrid *a, rgrid *b, double c, int op) {
  return d->prec == DFTGPU_FP32 ? rbin_t<float>(d, a, b, c, op) : rbin_t<double>(d, a, b, c, op);
}

// d = s^e (pow of the grid's precision)
template <typename T> static int rpow_t(rgrid *d, rgrid *s, double e) {
  T *pd = (T *) d->value;
  const T *ps = (const T *) s->value;
  const T ee = (T) e;
  return launch_each(gsize(d), [=] __device__(size_t i) { pd[i] = pow(ps[i], ee); }, 2.0 * gsize(d) * sizeof(T),
                     "rgrid_power");
}
int rpower(rgrid *d, rgrid *s, double e) {
  return d->prec == DFTGPU_FP32 ? rpow_t<float>(d, s, e) : rpow_t<double>(d, s, e);
}

template <typename T> static int rsum_t(rgrid *g, double *out) {
  const T *p = (const T *) g->value;
  const double dv = g->step * g->step * g->step;
  return reduce_host<1>(gsize(g), [=] __device__(size_t i, double *v) { v[0] = (double) p[i]; }, out, dv);
}
int rintegral(rgrid *g, double *out) {
  return g->prec == DFTGPU_FP32 ? rsum_t<float>(g, out) : rsum_t<double>(g, out);
}

template <typename T> static int density_t(cgrid *c, rgrid *d) {
  typedef typename cplx_t<T>::type C;
  const C *p = (const C *) c->value;
  T *q = (T *) d->value;
  return launch_each(gsize(c), [=] __device__(size_t i) { const C z = p[i]; q[i] = z.x * z.x + z.y * z.y; },
                     3.0 * gsize(c) * sizeof(T), "density");
}
int density(cgrid *c, rgrid *d) {
  return c->prec == DFTGPU_FP32 ? density_t<float>(c, d) : density_t<double>(c, d);
}

template <typename T> static int rho_dot_re_t(rgrid *r, cgrid *P, double *out) {
  typedef typename cplx_t<T>::type C;
  const T *a = (const T *) r->value;
  const C *b = (const C *) P->value;
  const double dv = r->step * r->step * r->step;
  return reduce_host<1>(gsize(r), [=] __device__(size_t i, double *v) { v[0] = (double) a[i] * (double) b[i].x; }, out, dv);
}
int rho_dot_re(rgrid *r, cgrid *P, double *out) {
  return r->prec == DFTGPU_FP32 ? rho_dot_re_t<float>(r, P, out) : rho_dot_re_t<double>(r, P, out);
}

}  // namespace dftgpu
