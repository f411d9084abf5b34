// Elementwise launch, FP64 reductions and 3-D transform sequences shared by
// the grid and OT translation units.
#pragma once

#include "fft.cuh"

namespace dftgpu {

// grid-stride elementwise launch of a device lambda f(i), i < n
template <class F> __global__ void each_kernel(size_t n, F f) {
  for (size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x) f(i);
}

// f(0..n-1), independent of one another, spread round-robin over the work
// stream and the auxiliary streams with event fork / join, so that a CUDA
// graph captured from the work stream gets them as parallel branches.  Runs
// on the work stream alone while the profiler is on (per-launch timings).
template <class F> int par_for(int n, F f) {
  cudaStream_t *aux;
  cudaEvent_t *ev;
  const int ns = prof_on() || n < 2 ? 1 : par_streams(&aux, &ev);
  if (ns < 2) {
    for (int i = 0; i < n; i++) DFT_TRY(f(i));
    return DFTGPU_OK;
  }
  const cudaStream_t main = rt().stream;
  const int use = ns < n ? ns : n;
  DFT_CUDA(cudaEventRecord(ev[0], main));
  for (int k = 0; k < use - 1; k++) DFT_CUDA(cudaStreamWaitEvent(aux[k], ev[0], 0));
  int rc = DFTGPU_OK;
  for (int i = 0; i < n && rc == DFTGPU_OK; i++) {
    rt().stream = i % use == 0 ? main : aux[i % use - 1];
    rc = f(i);
  }
  rt().stream = main;
  for (int k = 0; k < use - 1; k++) {
    DFT_CUDA(cudaEventRecord(ev[k + 1], aux[k]));
    DFT_CUDA(cudaStreamWaitEvent(main, ev[k + 1], 0));
  }
  return rc;
}

// bytes: algorithmic bytes the lambda reads and writes (0 if not stated)
template <class F> int launch_each(size_t n, F f, double bytes = 0.0, const char *name = "pointwise") {
  if (n == 0) return DFTGPU_OK;
  int blocks = (int) ((n + 255) / 256);
  int cap = rt().num_sms * 8;
  if (blocks > cap) blocks = cap;
  ProfScope prof(name, bytes);
  each_kernel<<<blocks, 256, 0, rt().stream>>>(n, f);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// One CTA per (x, y) row of an [nx][ny][nz] grid, threads along z: the
// lambda gets f(x, y, z, i) with i the linear index, no index division.
template <class F> __global__ void rows_kernel(int ny, int nz, F f) {
  const int y = blockIdx.x, x = blockIdx.y;
  const int base = (x * ny + y) * nz;
  for (int z = threadIdx.x; z < nz; z += blockDim.x) f(x, y, z, base + z);
}

template <class F> int launch_rows(int nx, int ny, int nz, F f, double bytes = 0.0, const char *name = "pointwise") {
  int bd = nz < 256 ? ((nz + 31) / 32) * 32 : 256;
  ProfScope prof(name, bytes);
  rows_kernel<<<dim3(ny, nx), bd, 0, rt().stream>>>(ny, nz, f);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// The same with a register budget for MINB resident 256-thread CTAs per SM:
// for latency-bound passes with many independent loads per element.
template <int MINB, class F> __global__ void __launch_bounds__(256, MINB) rows_kernel_b(int ny, int nz, F f) {
  const int y = blockIdx.x, x = blockIdx.y;
  const int base = (x * ny + y) * nz;
  for (int z = threadIdx.x; z < nz; z += blockDim.x) f(x, y, z, base + z);
}
template <int MINB, class F>
int launch_rows_b(int nx, int ny, int nz, F f, double bytes = 0.0, const char *name = "pointwise") {
  int bd = nz < 256 ? ((nz + 31) / 32) * 32 : 256;
  ProfScope prof(name, bytes);
  rows_kernel_b<MINB><<<dim3(ny, nx), bd, 0, rt().stream>>>(ny, nz, f);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// periodic neighbours of (x, y, z) along axis a, by comparison (no division)
struct Stencil3 {
  int nx, ny, nz;
  __device__ __forceinline__ void nb(int x, int y, int z, int i, int a, int &ip, int &im) const {
    if (a == 0) {
      const int s = ny * nz;
      ip = x + 1 < nx ? i + s : i + s - nx * s;
      im = x > 0 ? i - s : i - s + nx * s;
    } else if (a == 1) {
      ip = y + 1 < ny ? i + nz : i + nz - ny * nz;
      im = y > 0 ? i - nz : i - nz + ny * nz;
    } else {
      ip = z + 1 < nz ? i + 1 : i + 1 - nz;
      im = z > 0 ? i - 1 : i - 1 + nz;
    }
  }
};

// ---------------------------------------------------------------- reductions
// Deterministic FP64 sum of f(i) over i < n: a fixed grid of RED_BLOCKS
// blocks each sums a fixed strided subset, block partials are combined by a
// single block in a fixed order.  Result left in *slot (device).
constexpr int RED_BLOCKS = 1024;
constexpr int RED_THREADS = 256;

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[RED_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (int) (blockDim.x >> 5)) ? sh[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

template <int NV, class F> __global__ void reduce_partial_kernel(size_t n, F f, double *partial) {
  double acc[NV];
#pragma unroll
  for (int j = 0; j < NV; j++) acc[j] = 0.0;
  for (size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x) {
    double v[NV];
    f(i, v);
#pragma unroll
    for (int j = 0; j < NV; j++) acc[j] += v[j];
  }
#pragma unroll
  for (int j = 0; j < NV; j++) {
    double s = block_sum(acc[j]);
    if (threadIdx.x == 0) partial[j * RED_BLOCKS + blockIdx.x] = s;
  }
}

template <int NV> __global__ void reduce_final_kernel(const double *partial, double *slot, double scale) {
#pragma unroll
  for (int j = 0; j < NV; j++) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < RED_BLOCKS; i += blockDim.x) acc += partial[j * RED_BLOCKS + i];
    double s = block_sum(acc);
    if (threadIdx.x == 0) slot[j] = s * scale;
  }
}

// f(i, double v[NV]); results (times scale) to slot[0..NV) on the device.
template <int NV, class F> int reduce_dev(size_t n, F f, double *slot, double scale) {
  double *part; size_t np;
  DFT_TRY(reduce_partials(&part, &np));
  ProfScope prof("reduce_fp64", 0.0, 2);
  reduce_partial_kernel<NV><<<RED_BLOCKS, RED_THREADS, 0, rt().stream>>>(n, f, part);
  DFT_CHECK_LAUNCH();
  reduce_final_kernel<NV><<<1, RED_THREADS, 0, rt().stream>>>(part, slot, scale);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// Same, result copied to the host (synchronises the stream).
template <int NV, class F> int reduce_host(size_t n, F f, double *out, double scale) {
  double *slot = reduce_slots();
  DFT_TRY(reduce_dev<NV>(n, f, slot, scale));
  DFT_CUDA(cudaMemcpyAsync(out, slot, sizeof(double) * NV, cudaMemcpyDeviceToHost, rt().stream));
  DFT_CUDA(cudaStreamSynchronize(rt().stream));
  return DFTGPU_OK;
}

// ---------------------------------------------------------------- functors
// Spectral layout [kz][x][y]; real / complex grids [x][y][z].
template <typename T> struct SpecStoreZ {           // z pass output
  static constexpr bool kSpecZ = true;
  typename cplx_t<T>::type *spec; int nx, ny;
  __device__ void operator()(int x, int y, int k, typename cplx_t<T>::type v) const {
    spec[((size_t) k * nx + x) * ny + y] = v;
  }
};
// Load functors with kAhead provide prefetch_lines(a, b0, nl, ne), called by
// every thread of a CTA of the line kernels: bring the input of lines
// (a, b0 .. b0+nl-1), elements 0 .. ne-1, into L2 (bulk prefetches).
template <typename T> struct SpecLoadZ {            // z pass input (inverse); its tiles are one short
  typedef typename cplx_t<T>::type C;                // run per plane, not prefetched ahead
  static constexpr bool kSpecZ = true;
  const C *spec; int nx, ny;
  __device__ C operator()(int x, int y, int k) const {
    return spec[((size_t) k * nx + x) * ny + y];
  }
};
template <typename T> struct SpecLineY {            // y pass in place: line (kz, x), element y
  typedef typename cplx_t<T>::type C;
  static constexpr bool kAhead = true;
  typename cplx_t<T>::type *spec; int nx, ny;
  __device__ void prefetch_lines(int kz, int x0, int nl, int) const {     // nl whole lines, contiguous
    if (threadIdx.x == 0) prefetch_bulk_l2(spec + ((size_t) kz * nx + x0) * ny, (size_t) nl * ny * sizeof(C));
  }
  __device__ typename cplx_t<T>::type operator()(int kz, int x, int y) const {
    return spec[((size_t) kz * nx + x) * ny + y];
  }
  __device__ void operator()(int kz, int x, int y, typename cplx_t<T>::type v) const {
    spec[((size_t) kz * nx + x) * ny + y] = v;
  }
};
template <typename T> struct RealPairLoad {         // packed (f[2e], f[2e+1]) of a real row
  static constexpr bool kAhead = true;
  const T *f; int ny, nz;
  __device__ void prefetch_lines(int x, int y0, int nl, int) const {      // nl whole rows, contiguous
    if (threadIdx.x == 0) prefetch_bulk_l2(f + ((size_t) x * ny + y0) * nz, (size_t) nl * nz * sizeof(T));
  }
  // one vector access per pair: rows start on a multiple of nz (even) values
  __device__ typename cplx_t<T>::type operator()(int x, int y, int e) const {
    const T *row = f + ((size_t) x * ny + y) * nz;
    return *reinterpret_cast<const typename cplx_t<T>::type *>(row + 2 * e);
  }
};
template <typename T> struct RealPairStore {        // real row <- scale * (re, im)
  T *f; int ny, nz; T scale;
  __device__ void operator()(int x, int y, int e, typename cplx_t<T>::type v) const {
    T *row = f + ((size_t) x * ny + y) * nz;
    *reinterpret_cast<typename cplx_t<T>::type *>(row + 2 * e) = mk<T>(v.x * scale, v.y * scale);
  }
};
// (|psi[2e]|^2, |psi[2e+1]|^2) of a wave-function row, also stored into the
// density grid: the density pass (src/ot.c:320) done by the first z pass of rho.
// Algorithmic bytes beyond a real-row load: the psi row is twice as wide, and
// the density row is written (2 real fields).
// Split (fetch / cook): the density stores could alias psi for the compiler,
// so without the split every element's psi loads would wait for the previous
// element's store.
template <typename T> struct DensityPairLoad {
  typedef typename cplx_t<T>::type C;
  static constexpr bool kAhead = true, kSplit = true;
  struct Raw { C a, b; T *dst; };
  const C *psi; T *rho; int ny, nz;
  __device__ void prefetch_lines(int x, int y0, int nl, int) const {
    if (threadIdx.x == 0) prefetch_bulk_l2(psi + ((size_t) x * ny + y0) * nz, (size_t) nl * nz * sizeof(C));
  }
  __device__ Raw fetch(int x, int y, int e) const {
    const size_t r = ((size_t) x * ny + y) * nz + 2 * e;
    if constexpr (std::is_same<T, float>::value) {   // the pair as one 16-byte load (r even)
      const float4 q = *reinterpret_cast<const float4 *>(psi + r);
      return Raw{ make_float2(q.x, q.y), make_float2(q.z, q.w), rho + r };
    } else {
      return Raw{ psi[r], psi[r + 1], rho + r };
    }
  }
  __device__ C cook(const Raw &w) const {
    const C d = mk<T>(w.a.x * w.a.x + w.a.y * w.a.y, w.b.x * w.b.x + w.b.y * w.b.y);
    *reinterpret_cast<C *>(w.dst) = d;     // rows hold an even number of values
    return d;
  }
  __device__ C operator()(int x, int y, int e) const { return cook(fetch(x, y, e)); }
};
// P <- scale * (P + (re, im) added to the real parts of P[2e], P[2e+1]): the
// last c2r z pass of the potential adds the merged linear part into P and
// applies the predict-correct scale.  Algorithmic bytes beyond a real-row
// store: P is read and written (3 real fields).
template <typename T> struct PotAddPairStore {
  typedef typename cplx_t<T>::type C;
  static constexpr bool kSplit = true;
  C *pot; int ny, nz; T scale;
  __device__ void prefetch(int x, int y, int e) const {
    const size_t r = ((size_t) x * ny + y) * nz + 2 * e;
    if ((r * sizeof(C)) % 32 == 0) prefetch_l2(pot + r);   // one per 32-byte sector
  }
  __device__ void operator()(int x, int y, int e, C v) const {
    const size_t r = ((size_t) x * ny + y) * nz + 2 * e;
    if constexpr (std::is_same<T, float>::value) {   // the pair as one 16-byte access (r even)
      float4 q = *reinterpret_cast<const float4 *>(pot + r);
      q.x += v.x;
      q.z += v.y;
      *reinterpret_cast<float4 *>(pot + r) = make_float4(q.x * scale, q.y * scale, q.z * scale, q.w * scale);
    } else {
      C p0 = pot[r], p1 = pot[r + 1];
      p0.x += v.x;
      p1.x += v.y;
      pot[r] = mk<T>(p0.x * scale, p0.y * scale);
      pot[r + 1] = mk<T>(p1.x * scale, p1.y * scale);
    }
  }
};
template <typename T> struct CplxLoad {
  const typename cplx_t<T>::type *f; int ny, nz;
  __device__ typename cplx_t<T>::type operator()(int x, int y, int e) const {
    return f[((size_t) x * ny + y) * nz + e];
  }
};

// Fused z + y passes of a real field (fft.cu; the cluster kernels are
// instantiated in that one translation unit).  Return -1 when no fused
// instantiation fits the shape (the caller runs the separate passes).
int launch_zy_r2c(const RealPairLoad<float> &ld, float2 *spec, int nx, int ny, int nz);
int launch_yz_c2r(const float2 *spec, const RealPairStore<float> &st, int nx, int ny, int nz);

// y passes over nkz planes of a spectral buffer
template <typename T> int ypass(typename cplx_t<T>::type *spec, int nx, int ny, int nkz, T sign) {
  SpecLineY<T> io{spec, nx, ny};
  return launch_lines<T, LINE_C2C, 1, 1>(ny, nkz, nx, sign, io, io);
}

// forward r2c of a real field through its z and y passes, with a custom
// packed-pair loader (fused producer); spec is [nz/2+1][nx][ny]
// extra_bytes: algorithmic bytes of the load / store functor beyond one real field
template <typename T, class Ld>
int rfft_zy(const Ld &ld, typename cplx_t<T>::type *spec, int nx, int ny, int nz, double extra_bytes = 0.0) {
  if constexpr (std::is_same<Ld, RealPairLoad<float>>::value) {
    const int rc = launch_zy_r2c(ld, spec, nx, ny, nz);
    if (rc >= 0) return rc;
  }
  SpecStoreZ<T> st{spec, nx, ny};
  DFT_TRY((launch_lines<T, LINE_R2C, 1, 0>(nz / 2, nx, ny, (T) -1, ld, st, extra_bytes)));
  return ypass<T>(spec, nx, ny, nz / 2 + 1, (T) -1);
}

// inverse: y passes then c2r z pass into a custom consumer st(x, y, e, (v[2e], v[2e+1]))
template <typename T, class St>
int irfft_yz(typename cplx_t<T>::type *spec, const St &st, int nx, int ny, int nz, double extra_bytes = 0.0) {
  if constexpr (std::is_same<St, RealPairStore<float>>::value) {
    const int rc = launch_yz_c2r(spec, st, nx, ny, nz);
    if (rc >= 0) return rc;
  }
  DFT_TRY(ypass<T>(spec, nx, ny, nz / 2 + 1, (T) 1));
  SpecLoadZ<T> ld{spec, nx, ny};
  return launch_lines<T, LINE_C2R, 0, 1>(nz / 2, nx, ny, (T) 1, ld, st, extra_bytes);
}

}  // namespace dftgpu
