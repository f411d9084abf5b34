// FFT plans, twiddle tables and launchers for the x-pencil kernels.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <map>
#include <mutex>
#include <utility>

#include <cudaTypedefs.h>

#include "fft.cuh"
#include "ops.cuh"

namespace dftgpu {

namespace {
struct PlanEntry {
  int nst;
  int radix[FFT_MAX_STAGES];
  void *tw;
};
std::map<std::pair<int, int>, PlanEntry> g_plans;   // (n, sizeof(T)) -> plan
std::mutex g_plan_mu;

// FP64: radices up to 8 (the FP64 kernels compile for those only)
int factorize_small(int n, int *radix, int *nst) {
  int m = n, k = 0;
  while (m % 8 == 0 && m > 8) { radix[k++] = 8; m /= 8; }
  if (m % 8 == 0) { radix[k++] = 8; m /= 8; }
  if (m % 4 == 0) { radix[k++] = 4; m /= 4; }
  if (m % 2 == 0) { radix[k++] = 2; m /= 2; }
  while (m % 3 == 0) { radix[k++] = 3; m /= 3; }
  while (m % 5 == 0) { radix[k++] = 5; m /= 5; }
  if (m != 1 || k > FFT_MAX_STAGES) return DFTGPU_ERR_SIZE;
  *nst = k;
  return DFTGPU_OK;
}

// FP32
int factorize(int n, int *radix, int *nst) {
  int m = n, k = 0, a = 0, b = 0, c = 0;
  while (m % 2 == 0) { m /= 2; a++; }
  while (m % 3 == 0) { m /= 3; b++; }
  while (m % 5 == 0) { m /= 5; c++; }
  if (m != 1) return DFTGPU_ERR_SIZE;
  // few stages: radix 16 for the power of two, one 8 / 4 / 2 for its rest;
  // 15 = 3 x 5 and 9 = 3 x 3 for the odd part; a rest of 2 or 4 merged with
  // a rest of 3 (6, 12) or 2 with a 5 (10)
  while (a >= 4) { radix[k++] = 16; a -= 4; }
  int r2 = 1 << a;
  while (b >= 1 && c >= 1) { radix[k++] = 15; b--; c--; }
  while (b >= 2) { radix[k++] = 9; b -= 2; }
  if ((r2 == 2 || r2 == 4) && b == 1) { radix[k++] = 3 * r2; r2 = 1; b = 0; }
  else if (r2 == 2 && c >= 1) { radix[k++] = 10; r2 = 1; c--; }
  if (r2 > 1) radix[k++] = r2;
  if (b == 1) radix[k++] = 3;
  while (c-- > 0) radix[k++] = 5;
  if (k > FFT_MAX_STAGES) return DFTGPU_ERR_SIZE;
  *nst = k;
  return DFTGPU_OK;
}
}  // namespace

template <typename T> int get_plan(int n, FftPlan<T> *plan) {
  typedef typename cplx_t<T>::type C;
  if (n < 1 || n > FFT_MAX_LINE) {
    set_error(DFTGPU_ERR_SIZE, "FFT length %d outside [1, %d]", n, FFT_MAX_LINE);
    return DFTGPU_ERR_SIZE;
  }
  std::lock_guard<std::mutex> lock(g_plan_mu);
  auto key = std::make_pair(n, (int) sizeof(T));
  auto it = g_plans.find(key);
  if (it == g_plans.end()) {
    PlanEntry e;
    if (n == 1) { e.nst = 0; }
    else if ((sizeof(T) == 4 ? factorize(n, e.radix, &e.nst) : factorize_small(n, e.radix, &e.nst)) != DFTGPU_OK) {
      set_error(DFTGPU_ERR_SIZE, "FFT length %d is not of the form 2^a 3^b 5^c", n);
      return DFTGPU_ERR_SIZE;
    }
    C *h = (C *) malloc(sizeof(C) * (size_t) n);
    for (int t = 0; t < n; t++) {
      // reduce the angle to [-pi, pi] and evaluate in long double, round once
      long tt = (t <= n / 2) ? t : (long) t - n;
      long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double) tt / (long double) n;
      const long double cr = cosl(ang), ci = sinl(ang);
      h[t].x = (T) cr;
      h[t].y = (T) ci;
      if (sizeof(T) == 4) {
        // of the float pairs within one ulp of (cos, sin), take the one
        // closest to the unit circle: independent rounding leaves |w|^2 off 1
        // by up to 1.2e-7, a fixed pattern that biases the norm
        const float fx = (float) cr, fy = (float) ci;
        const float xs[2] = { fx, nextafterf(fx, cr > (long double) fx ? 2.f : -2.f) };
        const float ys[2] = { fy, nextafterf(fy, ci > (long double) fy ? 2.f : -2.f) };
        long double best = -1.0L;
        for (float x : xs)
          for (float y : ys) {
            const long double dev = fabsl((long double) x * x + (long double) y * y - 1.0L);
            if (best < 0 || dev < best) { best = dev; h[t].x = (T) x; h[t].y = (T) y; }
          }
      }
    }
    void *d = nullptr;
    cudaError_t err = cudaMalloc(&d, sizeof(C) * (size_t) n);
    if (err == cudaSuccess) err = cudaMemcpy(d, h, sizeof(C) * (size_t) n, cudaMemcpyHostToDevice);
    // the table is complete on the device before any stream (also a
    // non-blocking one: a caller's, or a parallel branch) reads it
    if (err == cudaSuccess) err = cudaDeviceSynchronize();
    free(h);
    if (err != cudaSuccess) {
      set_error(DFTGPU_ERR_CUDA, "twiddle table: %s", cudaGetErrorString(err));
      return DFTGPU_ERR_CUDA;
    }
    e.tw = d;
    it = g_plans.emplace(key, e).first;
  }
  plan->n = n;
  plan->nst = it->second.nst;
  for (int i = 0; i < it->second.nst; i++) plan->radix[i] = it->second.radix[i];
  plan->tw = (const C *) it->second.tw;
  return DFTGPU_OK;
}

template int get_plan<float>(int, FftPlan<float> *);
template int get_plan<double>(int, FftPlan<double> *);

int choose_tile(int n, int nb, size_t cplx_bytes, int nbufs, int *B, size_t *smem, bool partial) {
  const size_t budget = 113 * 1024, hard = 225 * 1024;
  const int cand[5] = { 16, 8, 4, 2, 1 };
  for (int pass = 0; pass < 2; pass++) {
    for (int c = 0; c < 5; c++) {
      int b = cand[c];
      if (nb % b && !partial) continue;
      if (b > nb && b > 1) continue;
      size_t s = (size_t) nbufs * (size_t) n * (size_t) tile_pitch(b) * cplx_bytes;
      if (s <= (pass == 0 ? budget : hard)) { *B = b; *smem = s; return DFTGPU_OK; }
    }
  }
  set_error(DFTGPU_ERR_SIZE, "FFT tile for n=%d does not fit in shared memory", n);
  return DFTGPU_ERR_SIZE;
}

bool fused_zy_off() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("DFTGPU_FUSED_ZY");
    v = (e && e[0] == '1') ? 0 : 1;
  }
  return v == 1;
}

bool prefetch_ahead_on() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("DFTGPU_PREFETCH_AHEAD");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}

bool factorised_propagation() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("DFTGPU_FACTORISED_PROP");
    v = (e && e[0] == '1') ? 1 : 0;
  }
  return v == 1;
}

bool march_on() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("DFTGPU_MARCH");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}

namespace {
int g_tma = -1;
}
bool tma_on() {
  if (g_tma < 0) {
    const char *e = getenv("DFTGPU_TMA");
    g_tma = (e && e[0] == '0') ? 0 : 1;
  }
  return g_tma == 1;
}
void tma_disable() { g_tma = 0; }

namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
}

int encode_spec_map(CUtensorMap *map, const void *spec, int nx, int ny, int rows) {
  if (!g_encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaGetLastError();
      set_error(DFTGPU_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
      return DFTGPU_ERR_CUDA;
    }
    g_encode = (PFN_cuTensorMapEncodeTiled_v12000) fn;
  }
  // [rows][nx][ny] of 8-byte elements; box {16 y, 1 x, rows}: 128-byte rows
  const cuuint64_t dims[3] = { (cuuint64_t) ny, (cuuint64_t) nx, (cuuint64_t) rows };
  const cuuint64_t strides[2] = { (cuuint64_t) ny * 8, (cuuint64_t) nx * ny * 8 };
  const cuuint32_t box[3] = { 16, 1, (cuuint32_t) rows }, estr[3] = { 1, 1, 1 };
  const CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void *>(spec), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(DFTGPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) for a %d x %d x %d spectrum", (int) r, rows, nx, ny);
    return DFTGPU_ERR_CUDA;
  }
  return DFTGPU_OK;
}

bool generic_fft_only() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("DFTGPU_GENERIC_FFT");
    v = (e && e[0] == '1') ? 1 : 0;
  }
  return v == 1;
}

namespace {

double xconv_bytes(const XConvArgs<float> &A, int kxh, int kyh) {
  const double spec = (double) A.nkz * A.nx * A.ny * sizeof(float2);
  double bytes = spec * A.nin;
  for (int o = 0; o < A.nout; o++) bytes += spec * (A.out[o].accumulate ? 2 : 1);
  const float *seen[XC_MAX_TERMS];
  int nseen = 0;
  for (int t = 0; t < XC_MAX_TERMS; t++) {
    const float *k = A.term[t].ker;
    if (!k || A.term[t].kind == KER_UNIT) continue;
    bool dup = false;
    for (int s = 0; s < nseen; s++) dup |= seen[s] == k;
    if (!dup) { seen[nseen++] = k; bytes += (double) A.nkz * kxh * kyh * sizeof(float); }
  }
  return bytes;
}

template <int N> int fast_xconv(const XConvArgs<float> &A) {
  constexpr int B = ff::Shape<N>::B;
  if (A.ny % B || (A.ny / 2) % B || A.nin > 4 || A.nout > 8) return -1;
  ff::XArgsF F;
  memset(&F, 0, sizeof(F));
  F.nx = A.nx; F.ny = A.ny; F.kxh = A.nx / 2 + 1; F.kyh = A.ny / 2 + 1;
  F.nin = A.nin; F.nout = A.nout;
  for (int i = 0; i < A.nin; i++) F.src[i] = A.src[i];
  int multi = -1, nt = 0;
  for (int o = 0; o < A.nout; o++) {
    F.dst[o] = A.out[o].dst;
    F.acc_out[o] = A.out[o].accumulate;
    F.t0[o] = A.out[o].t0;
    F.nterm[o] = A.out[o].nt;
    if (A.out[o].nt > 1) {
      if (multi >= 0) return -1;   // at most one output accumulated in registers
      multi = o;
    }
    if (A.out[o].nt < 1) return -1;
    nt = A.out[o].t0 + A.out[o].nt > nt ? A.out[o].t0 + A.out[o].nt : nt;
  }
  if (nt > 16) return -1;
  F.nslice = 0;
  for (int t = 0; t < nt; t++) {
    F.kind[t] = A.term[t].kind; F.in[t] = A.term[t].in; F.coef[t] = A.term[t].coef;
    F.slot[t] = -1;
    if (A.term[t].kind == KER_UNIT) continue;
    for (int s = 0; s < F.nslice; s++)
      if (F.slice_src[s] == A.term[t].ker) F.slot[t] = s;
    if (F.slot[t] < 0) {
      if (F.nslice == 8) return -1;
      F.slice_src[F.nslice] = A.term[t].ker;
      F.slot[t] = F.nslice++;
    }
  }
  FftPlan<float> p;
  DFT_TRY(get_plan<float>(N, &p));
  const int smem = ff::xconv_smem<N>(F.nslice);
  // request exactly the dynamic shared memory this launch needs (the kernel
  // also has static shared memory, so the opt-in maximum itself is not valid)
  // MODE 2: one output summing every term; 1: mixed with one multi-term output; 0: single-term outputs
  const int mode = (A.nout == 1 && multi == 0) ? 2 : (multi >= 0 ? 1 : 0);
  static int granted[3] = { 48 * 1024, 48 * 1024, 48 * 1024 };
  if (smem > granted[mode]) {
    if (mode == 2) DFT_CUDA(cudaFuncSetAttribute(ff::xconv_kernel<N, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    else if (mode == 1) DFT_CUDA(cudaFuncSetAttribute(ff::xconv_kernel<N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    else DFT_CUDA(cudaFuncSetAttribute(ff::xconv_kernel<N, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    granted[mode] = smem;
  }
  ProfScope prof("fft_x_conv", xconv_bytes(A, F.kxh, F.kyh));
  const dim3 grid(A.ny / B, A.nkz);
  if (mode == 2) ff::xconv_kernel<N, 2><<<grid, 256, smem, rt().stream>>>(p.tw, F, multi);
  else if (mode == 1) ff::xconv_kernel<N, 1><<<grid, 256, smem, rt().stream>>>(p.tw, F, multi);
  else ff::xconv_kernel<N, 0><<<grid, 256, smem, rt().stream>>>(p.tw, F, multi);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

template <int N> int fast_xkinetic(const KinArgs<float> &A) {
  constexpr int B = ff::Shape<N>::B;
  if (A.ny % B) return -1;
  FftPlan<float> p;
  DFT_TRY(get_plan<float>(N, &p));
  ProfScope prof("fft_x_kinetic", 2.0 * A.nx * A.ny * A.nz * sizeof(float2));
  auto k = A.cn ? ff::xkinetic_kernel<N, true> : ff::xkinetic_kernel<N, false>;
  k<<<dim3(A.ny / B, A.nz), 256, 0, rt().stream>>>(
      p.tw, A.data, A.ny, A.nz, make_float2((float) A.cdt.x, (float) A.cdt.y), (float) A.inv_n, (float) A.dkx,
      (float) A.dky, (float) A.dkz, (float) A.kx0, (float) A.ky0, (float) A.kz0, (float) A.h);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

}  // namespace

template <typename T> int launch_xconv(XConvArgs<T> &A) {
  typedef typename cplx_t<T>::type C;
  if constexpr (std::is_same<T, float>::value) {
    if (!generic_fft_only()) {
      int rc = -1;
      switch (A.nx) {
        case 64: rc = fast_xconv<64>(A); break;
        case 128: rc = fast_xconv<128>(A); break;
        case 256: rc = fast_xconv<256>(A); break;
        case 512: rc = fast_xconv<512>(A); break;
        case 96: rc = fast_xconv<96>(A); break;
        case 192: rc = fast_xconv<192>(A); break;
        case 384: rc = fast_xconv<384>(A); break;
        default: break;
      }
      if (rc >= 0) return rc;
    }
  }
  DFT_TRY(get_plan<T>(A.nx, &A.plan));
  int B; size_t smem;
  DFT_TRY(choose_tile(A.nx, A.ny, sizeof(C), 3, &B, &smem));   // three tiles (xconv_kernel)
  A.B = B;
  A.kxh = A.nx / 2 + 1;
  A.kyh = A.ny / 2 + 1;
  static bool attr = false;
  if (!attr) {
    DFT_CUDA(cudaFuncSetAttribute(xconv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) rt().max_smem_optin));
    attr = true;
  }
  dim3 grid(A.ny / B, A.nkz);
  double bytes = 0.0;
  {
    const double spec = (double) A.nkz * A.nx * A.ny * sizeof(C);
    bytes = spec * A.nin;
    for (int o = 0; o < A.nout; o++) bytes += spec * (A.out[o].accumulate ? 2 : 1);
    const T *seen[XC_MAX_TERMS];
    int nseen = 0;
    for (int t = 0; t < XC_MAX_TERMS; t++) {
      const T *k = A.term[t].ker;
      if (!k || A.term[t].kind == KER_UNIT) continue;
      bool dup = false;
      for (int s = 0; s < nseen; s++) dup |= seen[s] == k;
      if (!dup) { seen[nseen++] = k; bytes += (double) A.nkz * A.kxh * A.kyh * sizeof(T); }
    }
  }
  ProfScope prof("fft_x_conv", bytes);
  xconv_kernel<T><<<grid, FFT_THREADS, smem, rt().stream>>>(A);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

template <typename T> int launch_xkinetic(KinArgs<T> &A) {
  typedef typename cplx_t<T>::type C;
  if constexpr (std::is_same<T, float>::value) {
    if (!generic_fft_only()) {
      int rc = -1;
      switch (A.nx) {
        case 64: rc = fast_xkinetic<64>(A); break;
        case 128: rc = fast_xkinetic<128>(A); break;
        case 256: rc = fast_xkinetic<256>(A); break;
        case 512: rc = fast_xkinetic<512>(A); break;
        case 96: rc = fast_xkinetic<96>(A); break;
        case 192: rc = fast_xkinetic<192>(A); break;
        case 384: rc = fast_xkinetic<384>(A); break;
        default: break;
      }
      if (rc >= 0) return rc;
    }
  }
  DFT_TRY(get_plan<T>(A.nx, &A.plan));
  int B; size_t smem;
  DFT_TRY(choose_tile(A.nx, A.ny, sizeof(C), 2, &B, &smem));
  smem = kin_smem(A.nx, B, sizeof(C));
  if (smem > rt().max_smem_optin) {
    set_error(DFTGPU_ERR_SIZE, "kinetic pass for nx=%d does not fit in shared memory", A.nx);
    return DFTGPU_ERR_SIZE;
  }
  A.B = B;
  static bool attr = false;
  if (!attr) {
    DFT_CUDA(cudaFuncSetAttribute(xkinetic_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) rt().max_smem_optin));
    attr = true;
  }
  dim3 grid(A.ny / B, A.nz);
  ProfScope prof("fft_x_kinetic", 2.0 * A.nx * A.ny * A.nz * sizeof(C));
  xkinetic_kernel<T><<<grid, FFT_THREADS, smem, rt().stream>>>(A);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

template int launch_xconv<float>(XConvArgs<float> &);
template int launch_xconv<double>(XConvArgs<double> &);
template int launch_xkinetic<float>(KinArgs<float> &);
template int launch_xkinetic<double>(KinArgs<double> &);

// ------------------------------------------------------------------ fused z + y passes
namespace {

int *g_zy_fault = nullptr;   // set by a kernel whose wait on an asynchronous copy gave up

template <int NY, int NZ, int CL, bool FWD, class Kern, class... Args>
int launch_zy_cluster(Kern kfn, int nx, Args... args) {
  typedef ff::ZYPlane<NY, NZ, CL> Z;
  static bool attr_done = false;
  if (!attr_done) {
    DFT_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, Z::SMEM));
    attr_done = true;
  }
  if (!async_fault_flag()) return DFTGPU_ERR_CUDA;
  FftPlan<float> pz, p2, py;
  DFT_TRY(get_plan<float>(Z::NZC, &pz));
  DFT_TRY(get_plan<float>(NZ, &p2));
  DFT_TRY(get_plan<float>(NY, &py));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL, nx);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = Z::SMEM;
  cfg.stream = rt().stream;
  cudaLaunchAttribute at[1];
  memset(at, 0, sizeof(at));
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kfn, (const float2 *) pz.tw, (const float2 *) p2.tw,
                                           (const float2 *) py.tw, args..., nx, g_zy_fault);
  if (e != cudaSuccess) {
    cudaFuncAttributes fa = {};
    cudaFuncGetAttributes(&fa, kfn);
    set_error(DFTGPU_ERR_CUDA, "fused %s pass %dx%d (cluster %d, %d B shared, nx %d): %s; function: %d regs, "
              "max dynamic shared %d B", FWD ? "zy r2c" : "yz c2r", NY, NZ, CL, Z::SMEM, nx, cudaGetErrorString(e),
              fa.numRegs, fa.maxDynamicSharedSizeBytes);
    return DFTGPU_ERR_CUDA;
  }
  return DFTGPU_OK;
}

bool fused_shape(int ny, int nz) {
  return !generic_fft_only() && !fused_zy_off() && ny == nz && (ny == 128 || ny == 256);
}

}  // namespace

int *async_fault_flag() {
  if (!g_zy_fault) {
    if (cudaMalloc(&g_zy_fault, sizeof(int)) != cudaSuccess || cudaMemset(g_zy_fault, 0, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      g_zy_fault = nullptr;
      set_error(DFTGPU_ERR_CUDA, "asynchronous-copy fault flag");
      return nullptr;
    }
  }
  return g_zy_fault;
}

int fused_zy_fault() {
  if (!g_zy_fault) return DFTGPU_OK;
  int v = 0;
  DFT_CUDA(cudaMemcpy(&v, g_zy_fault, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) {
    cudaMemset(g_zy_fault, 0, sizeof(int));
    set_error(DFTGPU_ERR_CUDA, "a wait on an asynchronous copy (TMA or fused plane pass) timed out");
    return DFTGPU_ERR_CUDA;
  }
  return DFTGPU_OK;
}

int launch_zy_r2c(const RealPairLoad<float> &ld, float2 *spec, int nx, int ny, int nz) {
  if (!fused_shape(ny, nz)) return -1;
  ProfScope prof("fft_zy_r2c", (double) nx * ny * nz * 4.0 + (double) nx * ny * (nz / 2 + 1) * 8.0);
  if (ny == 128) return launch_zy_cluster<128, 128, 2, true>(ff::zy_r2c_kernel<128, 128, 2>, nx, ld.f, spec);
  return launch_zy_cluster<256, 256, 8, true>(ff::zy_r2c_kernel<256, 256, 8>, nx, ld.f, spec);
}

int launch_yz_c2r(const float2 *spec, const RealPairStore<float> &st, int nx, int ny, int nz) {
  if (!fused_shape(ny, nz)) return -1;
  ProfScope prof("fft_yz_c2r", (double) nx * ny * nz * 4.0 + (double) nx * ny * (nz / 2 + 1) * 8.0);
  if (ny == 128) return launch_zy_cluster<128, 128, 2, false>(ff::yz_c2r_kernel<128, 128, 2>, nx, spec, st.f, st.scale);
  return launch_zy_cluster<256, 256, 8, false>(ff::yz_c2r_kernel<256, 256, 8>, nx, spec, st.f, st.scale);
}

}  // namespace dftgpu
