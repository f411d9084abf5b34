// Allocation-free variant of the split-operator wave-function step.
//
// Some callers cannot call cudaMalloc at all: code that runs while a CUDA
// graph is being captured by someone else, host frameworks that own every
// byte of device memory through their own pool (and forbid side allocations
// behind their back), or long-running services that must never grow their
// footprint after start-up.  dftgpu_wf_propagate_noalloc() serves them: the
// caller passes device pointers it owns for the input, the output and the
// potential, and the only work memory is the file-scope device array below,
// which exists in every GPU that loads this library until the process exits.
//
// The array holds the spectral scratch of one step (nx*ny*nz complex values in
// the requested precision) and the FFT twiddle tables, so the grid is limited
// to NOALLOC_SCRATCH_BYTES / (2 * sizeof(real)) points: 2,097,152 in FP64
// (e.g. 128^3), 4,194,304 in FP32 (e.g. 128 x 128 x 256).
//
// Every call shares the one array and leaves the last call's contents in it;
// nothing in it has to start at zero (each call rewrites the twiddle tables it
// uses and overwrites the whole scratch before reading it).  Calls whose work
// overlaps on the GPU (different streams, or different host threads) race on
// the array: serialise them.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (the name is only a host-side stand-in in host code);
// make that first call before any stream capture.
#include <math.h>

#include "ops.cuh"
#include "grid_internal.cuh"

namespace dftgpu {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t) 32 << 20;   // spectral scratch, 32 MiB
// the z, y and x twiddle tables one after the other, each starting on a
// 256-byte boundary: nz + ny + nx complex values plus padding, at most
// 4096 + 32 + 1 (a 1-D grid) or 3 * 1024 (a 3-D grid) complex doubles
constexpr size_t NOALLOC_TW_BYTES = (size_t) 128 << 10;
constexpr int TW_ALIGN = 32;   // table offsets in complex values (256 bytes in FP64)

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES + NOALLOC_TW_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
unsigned char *g_scratch_addr[NOALLOC_MAX_DEVICES] = {};    // device address per device, set once

int scratch_address(int device, unsigned char **out) {
  if (device < 0 || device >= NOALLOC_MAX_DEVICES) {
    set_error(DFTGPU_ERR_ARG, "noalloc: device index %d out of range", device);
    return DFTGPU_ERR_ARG;
  }
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(DFTGPU_ERR_CUDA, "noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return DFTGPU_ERR_CUDA;
    }
    g_scratch_addr[device] = (unsigned char *) p;
  }
  *out = g_scratch_addr[device];
  return DFTGPU_OK;
}

// radices for a 2^a 3^b 5^c length, largest power-of-two radix first
bool radices_for(int n, int *radix, int *nst) {
  int m = n, k = 0;
  while (m % 8 == 0 && k < FFT_MAX_STAGES) { radix[k++] = 8; m /= 8; }
  while (m % 4 == 0 && k < FFT_MAX_STAGES) { radix[k++] = 4; m /= 4; }
  while (m % 2 == 0 && k < FFT_MAX_STAGES) { radix[k++] = 2; m /= 2; }
  while (m % 3 == 0 && k < FFT_MAX_STAGES) { radix[k++] = 3; m /= 3; }
  while (m % 5 == 0 && k < FFT_MAX_STAGES) { radix[k++] = 5; m /= 5; }
  *nst = k;
  return m == 1;
}

// tw[t] = exp(-2 pi i t / n), evaluated in FP64 and rounded once.  In FP32
// the pair is the one, among the float pairs within one ulp of (cos, sin),
// whose x^2 + y^2 is closest to 1 (the rule of the library's own tables):
// independently rounded pairs leave |w|^2 off 1 by up to 1.2e-7 in a fixed
// pattern, which drifts the norm of a real-time step.
__device__ __forceinline__ void round_unit(double c, double s, float2 &w) {
  const float fx = (float) c, fy = (float) s;
  const float xs[2] = { fx, nextafterf(fx, c > (double) fx ? 2.f : -2.f) };
  const float ys[2] = { fy, nextafterf(fy, s > (double) fy ? 2.f : -2.f) };
  double best = -1.0;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      const double dev = fabs((double) xs[a] * xs[a] + (double) ys[b] * ys[b] - 1.0);
      if (best < 0.0 || dev < best) { best = dev; w = make_float2(xs[a], ys[b]); }
    }
}
__device__ __forceinline__ void round_unit(double c, double s, double2 &w) { w = make_double2(c, s); }

template <typename T> __global__ void twiddle_kernel(typename cplx_t<T>::type *tw, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int tt = (t <= n / 2) ? t : t - n;
    double s, c;
    sincospi(-2.0 * (double) tt / (double) n, &s, &c);
    round_unit(c, s, tw[t]);
  }
}

template <typename T> int make_plan(int n, typename cplx_t<T>::type *tw, cudaStream_t s, FftPlan<T> *pl) {
  if (!radices_for(n, pl->radix, &pl->nst)) {
    set_error(DFTGPU_ERR_SIZE, "noalloc: length %d is not of the form 2^a 3^b 5^c", n);
    return DFTGPU_ERR_SIZE;
  }
  pl->n = n;
  pl->tw = tw;
  twiddle_kernel<T><<<(n + 255) / 256, 256, 0, s>>>(tw, n);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// psi * exp(-i V dt / 2) on load and on store (the potential half steps)
template <typename T> struct HalfStepLoad {
  typedef typename cplx_t<T>::type C;
  const C *psi; const C *V; int ny, nz; T hr, hi;   // (hr, hi) = dt / 2
  __device__ C operator()(int x, int y, int e) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    const C v = V[i];
    return mul_cexp(psi[i], mk<T>(v.x * hi + v.y * hr, -(v.x * hr - v.y * hi)));
  }
};
template <typename T> struct HalfStepStore {
  typedef typename cplx_t<T>::type C;
  C *psi; const C *V; int ny, nz; T hr, hi;
  __device__ void operator()(int x, int y, int e, C val) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    const C v = V[i];
    psi[i] = mul_cexp(val, mk<T>(v.x * hi + v.y * hr, -(v.x * hr - v.y * hi)));
  }
};

template <typename T, int MODE, class Ld, class St>
int run_lines(const FftPlan<T> &pl, int na, int nb, T sign, int e_fast, int e_fast_store, const Ld &ld, const St &st,
              cudaStream_t s) {
  typedef typename cplx_t<T>::type C;
  LineArgs<T> args;
  args.plan = pl;
  args.sign = sign;
  args.nb = nb;
  args.e_fast = e_fast;
  args.e_fast_store = e_fast_store;
  args.tw2 = nullptr;
  int B; size_t smem;
  DFT_TRY(choose_tile(pl.n, nb, sizeof(C), 2, &B, &smem));
  args.B = B;
  auto kfn = line_fft_kernel<T, MODE, Ld, St>;
  if (smem > 48 * 1024) DFT_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
  kfn<<<dim3(nb / B, na), FFT_THREADS, smem, s>>>(args, ld, st);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

template <typename T>
int propagate_noalloc_t(void *out, const void *in, const void *pot, int nx, int ny, int nz, double step, double mass,
                        double dr, double di, cudaStream_t s, unsigned char *base) {
  typedef typename cplx_t<T>::type C;
  C *spec = (C *) base;
  C *tw = (C *) (base + NOALLOC_SCRATCH_BYTES);
  // tables placed by the lengths they hold (a 1-D grid's z line is up to 4096 long)
  const size_t oy = (size_t) (nz + TW_ALIGN - 1) / TW_ALIGN * TW_ALIGN;
  const size_t ox = oy + (size_t) (ny + TW_ALIGN - 1) / TW_ALIGN * TW_ALIGN;
  if ((ox + nx) * sizeof(C) > NOALLOC_TW_BYTES) {
    set_error(DFTGPU_ERR_SIZE, "noalloc: twiddle tables for %dx%dx%d exceed %zu bytes", nx, ny, nz, NOALLOC_TW_BYTES);
    return DFTGPU_ERR_SIZE;
  }
  FftPlan<T> pz, py, px;
  DFT_TRY(make_plan<T>(nz, tw, s, &pz));
  DFT_TRY(make_plan<T>(ny, tw + oy, s, &py));
  DFT_TRY(make_plan<T>(nx, tw + ox, s, &px));
  const T hr = (T) (0.5 * dr), hi = (T) (0.5 * di);
  HalfStepLoad<T> ld{(const C *) in, (const C *) pot, ny, nz, hr, hi};
  SpecStoreZ<T> sz{spec, nx, ny};
  DFT_TRY((run_lines<T, LINE_C2C>(pz, nx, ny, (T) -1, 1, 0, ld, sz, s)));
  SpecLineY<T> ioy{spec, nx, ny};
  DFT_TRY((run_lines<T, LINE_C2C>(py, nz, nx, (T) -1, 1, 1, ioy, ioy, s)));
  KinArgs<T> K;
  K.plan = px;
  kin_args<T>(K, nx, ny, nz, step, make_double2(di / (2.0 * mass), -dr / (2.0 * mass)), 0.0, 0.0, 0.0, spec);
  int B; size_t smem;
  DFT_TRY(choose_tile(nx, ny, sizeof(C), 2, &B, &smem));
  smem = kin_smem(nx, B, sizeof(C));
  K.B = B;
  int optin = 0, dev = 0;
  DFT_CUDA(cudaGetDevice(&dev));
  DFT_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem > (size_t) optin) {
    set_error(DFTGPU_ERR_SIZE, "noalloc: kinetic pass for nx=%d needs %zu bytes of shared memory (limit %d)", nx, smem,
              optin);
    return DFTGPU_ERR_SIZE;
  }
  if (smem > 48 * 1024)
    DFT_CUDA(cudaFuncSetAttribute(xkinetic_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
  xkinetic_kernel<T><<<dim3(ny / B, nz), FFT_THREADS, smem, s>>>(K);
  DFT_CHECK_LAUNCH();
  DFT_TRY((run_lines<T, LINE_C2C>(py, nz, nx, (T) 1, 1, 1, ioy, ioy, s)));
  SpecLoadZ<T> lz{spec, nx, ny};
  HalfStepStore<T> st{(C *) out, (const C *) pot, ny, nz, hr, hi};
  return run_lines<T, LINE_C2C>(pz, nx, ny, (T) 1, 0, 1, lz, st, s);
}

}  // namespace
}  // namespace dftgpu

using namespace dftgpu;

extern "C" int dftgpu_wf_propagate_noalloc(void *psi_out, const void *psi_in, const void *potential, INT nx, INT ny,
                                           INT nz, REAL step, REAL mass, double dt_re, double dt_im, int prec,
                                           void *stream) {
  if (!psi_out || !psi_in || !potential) { set_error(DFTGPU_ERR_ARG, "noalloc: NULL pointer"); return DFTGPU_ERR_ARG; }
  if (prec != DFTGPU_FP32 && prec != DFTGPU_FP64) { set_error(DFTGPU_ERR_ARG, "noalloc: precision"); return DFTGPU_ERR_ARG; }
  if (!(step > 0.0) || !(mass > 0.0)) { set_error(DFTGPU_ERR_ARG, "noalloc: step and mass must be positive"); return DFTGPU_ERR_ARG; }
  DFT_TRY(check_dims(nx, ny, nz));
  const size_t need = (size_t) nx * ny * nz * 2 * elem_size(prec);
  if (need > NOALLOC_SCRATCH_BYTES) {
    set_error(DFTGPU_ERR_SIZE, "noalloc: grid %ldx%ldx%ld needs %zu bytes of scratch; the static scratch holds %zu",
              (long) nx, (long) ny, (long) nz, need, NOALLOC_SCRATCH_BYTES);
    return DFTGPU_ERR_SIZE;
  }
  int device = 0;
  DFT_CUDA(cudaGetDevice(&device));
  unsigned char *base = nullptr;
  DFT_TRY(scratch_address(device, &base));
  cudaStream_t s = (cudaStream_t) stream;
  return prec == DFTGPU_FP32
             ? propagate_noalloc_t<float>(psi_out, psi_in, potential, (int) nx, (int) ny, (int) nz, step, mass, dt_re, dt_im, s, base)
             : propagate_noalloc_t<double>(psi_out, psi_in, potential, (int) nx, (int) ny, (int) nz, step, mass, dt_re, dt_im, s, base);
}
