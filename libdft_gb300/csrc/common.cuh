// Shared definitions for the GB300 OT-DFT library (sm_103a).
//
// Precision model: a grid stores either FP32 or FP64 values (the "bulk"
// precision).  Reductions (norms, energies, chemical potential) always
// accumulate in FP64; the k-space convolution kernels are generated in FP64
// and stored in the bulk precision.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "dftgpu.h"

namespace dftgpu {

// ------------------------------------------------------------------ complex
template <typename T> struct cplx_t;
template <> struct cplx_t<float> { typedef float2 type; };
template <> struct cplx_t<double> { typedef double2 type; };

template <typename T> __host__ __device__ __forceinline__ typename cplx_t<T>::type mk(T re, T im) {
  typename cplx_t<T>::type r; r.x = re; r.y = im; return r;
}
__host__ __device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 operator*(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 operator*(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
  C r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
// multiply by +i (s = +1) or -i (s = -1)
template <typename C, typename T> __host__ __device__ __forceinline__ C imul(C a, T s) {
  C r; r.x = -s * a.y; r.y = s * a.x; return r;
}
template <typename C> __host__ __device__ __forceinline__ C conjc(C a) { C r; r.x = a.x; r.y = -a.y; return r; }

// exp(z) for complex z, in the precision of C
__device__ __forceinline__ float2 cexp_dev(float2 z) {
  float e = expf(z.x), s, c; sincosf(z.y, &s, &c); return make_float2(e * c, e * s);
}
__device__ __forceinline__ double2 cexp_dev(double2 z) {
  double e = exp(z.x), s, c; sincos(z.y, &s, &c); return make_double2(e * c, e * s);
}

// Bring the line holding p into L2 (generic address; no register result).
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.L2 [%0];" ::"l"(p)); }
// Bring [p, p + bytes) into L2 with one bulk prefetch; skipped unless p and
// bytes are multiples of 16 (the instruction's requirement).
__device__ __forceinline__ void prefetch_bulk_l2(const void *p, size_t bytes) {
  if ((((size_t) p) | bytes) & 15 || bytes == 0 || bytes > 0xffffffffull) return;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"((unsigned) bytes));
}

// exp(z) - 1 for |Re z| + |Im z| < 0.25 from the Taylor series of e^x - 1,
// sin y and cos y - 1 (Horner), each truncated where the next term is below
// 2e-9 of the result on that interval (e^x - 1 to x^7, sin y to y^7,
// cos y - 1 to y^8): no range reduction, and cos y - 1 keeps its full relative
// precision, so |exp(i y)| = 1 to the rounding of y.
__device__ __forceinline__ float2 cexpm1_small(float2 z) {
  const float x = z.x, y = z.y, y2 = y * y;
  float em = fmaf(x, 1.f / 5040.f, 1.f / 720.f);
  em = fmaf(x, em, 1.f / 120.f);
  em = fmaf(x, em, 1.f / 24.f);
  em = fmaf(x, em, 1.f / 6.f);
  em = fmaf(x, em, 0.5f);
  em = fmaf(x, em, 1.f);
  em *= x;                                         // e^x - 1
  float sy = fmaf(y2, -1.f / 5040.f, 1.f / 120.f);
  sy = fmaf(y2, sy, -1.f / 6.f);
  sy = fmaf(y2, sy, 1.f);
  sy *= y;                                         // sin y
  float cm = fmaf(y2, 1.f / 40320.f, -1.f / 720.f);
  cm = fmaf(y2, cm, 1.f / 24.f);
  cm = fmaf(y2, cm, -0.5f);
  cm *= y2;                                        // cos y - 1
  return make_float2(fmaf(em, cm, em + cm), fmaf(em, sy, sy));   // (e^x cos y - 1, e^x sin y)
}

// exp(z) - 1, so that a factor near 1 keeps the full relative precision of
// its difference from 1: the polynomials above for small |z|, otherwise
// expm1 and the half-angle sine (cos y - 1 = -2 sin^2(y/2)).
__device__ __forceinline__ float2 cexpm1(float2 z) {
  if (fabsf(z.x) + fabsf(z.y) < 0.25f) return cexpm1_small(z);
  float sh, ch;
  sincosf(0.5f * z.y, &sh, &ch);
  const float em = expm1f(z.x), s2 = 2.f * sh * sh;
  return make_float2(em * (1.f - s2) - s2, (1.f + em) * (2.f * sh * ch));
}
__device__ __forceinline__ double2 cexpm1(double2 z) {
  double sh, ch;
  sincos(0.5 * z.y, &sh, &ch);
  const double em = expm1(z.x), s2 = 2.0 * sh * sh;
  return make_double2(em * (1.0 - s2) - s2, (1.0 + em) * (2.0 * sh * ch));
}

// a (1 + d) evaluated as a + a d
__device__ __forceinline__ float2 mul_1p(float2 a, float2 d) {
  return make_float2(a.x + (a.x * d.x - a.y * d.y), a.y + (a.x * d.y + a.y * d.x));
}
__device__ __forceinline__ double2 mul_1p(double2 a, double2 d) {
  return make_double2(a.x + (a.x * d.x - a.y * d.y), a.y + (a.x * d.y + a.y * d.x));
}

// (1 + p)(1 + q) - 1
template <typename C> __device__ __forceinline__ C cprod1p(C p, C q) {
  C r;
  r.x = p.x + q.x + (p.x * q.x - p.y * q.y);
  r.y = p.y + q.y + (p.x * q.y + p.y * q.x);
  return r;
}

// One axis of the Crank-Nicolson kinetic step, minus one:
//   (1 + c Q / 2) / (1 - c Q / 2) - 1 = c Q / (1 - c Q / 2),
// Q = (2 sin(k h / 2) / h)^2 the eigenvalue of the periodic second difference
// -(f[j+1] - 2 f[j] + f[j-1]) / h^2 at wave number k, c = -i dt / 2m.  For
// Re c <= 0 (real or imaginary time) |1 - c Q / 2| >= 1.
__device__ __forceinline__ float2 cn_m1(float2 c, float k, float h) {
  const float s = 2.f * sinf(0.5f * k * h) / h, q = s * s;
  const float nx = c.x * q, ny = c.y * q, dx = 1.f - 0.5f * nx, dy = -0.5f * ny;
  const float id = 1.f / (dx * dx + dy * dy);
  return make_float2((nx * dx + ny * dy) * id, (ny * dx - nx * dy) * id);
}
__device__ __forceinline__ double2 cn_m1(double2 c, double k, double h) {
  const double s = 2.0 * sin(0.5 * k * h) / h, q = s * s;
  const double nx = c.x * q, ny = c.y * q, dx = 1.0 - 0.5 * nx, dy = -0.5 * ny;
  const double id = 1.0 / (dx * dx + dy * dy);
  return make_double2((nx * dx + ny * dy) * id, (ny * dx - nx * dy) * id);
}

// a * exp(z).  For small |z| the factor is applied as a + a (exp(z) - 1): a
// factor rounded as a whole has |exp(i theta)|^2 = c^2 + s^2 off 1 by the
// rounding of c near 1, which is biased for small angles and changed the norm
// by ~7e-8 (FP32) at every real-time step; the split form keeps
// |exp(i theta)| = 1 to the rounding of theta.  Large |z| (strongly damped
// modes) uses the factor directly, so a damped value keeps its own relative
// precision.
__device__ __forceinline__ float2 mul_cexp(float2 a, float2 z) {
  if (fabsf(z.x) + fabsf(z.y) < 0.25f) return mul_1p(a, cexpm1_small(z));
  return cmul(a, cexp_dev(z));
}
__device__ __forceinline__ double2 mul_cexp(double2 a, double2 z) {
  if (fabs(z.x) + fabs(z.y) < 0.25) return mul_1p(a, cexpm1(z));
  return cmul(a, cexp_dev(z));
}

// ------------------------------------------------------------------ errors
extern thread_local int g_last_error;
void set_error(int code, const char *fmt, ...);

#define DFT_CUDA(call)                                                         \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) {                                                   \
      ::dftgpu::set_error(DFTGPU_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, \
                          #call, cudaGetErrorString(_e));                      \
      return DFTGPU_ERR_CUDA;                                                  \
    }                                                                          \
  } while (0)

#define DFT_CHECK_LAUNCH()                                                     \
  do {                                                                         \
    cudaError_t _e = cudaGetLastError();                                       \
    if (_e != cudaSuccess) {                                                   \
      ::dftgpu::set_error(DFTGPU_ERR_CUDA, "%s:%d launch: %s", __FILE__,       \
                          __LINE__, cudaGetErrorString(_e));                   \
      return DFTGPU_ERR_CUDA;                                                  \
    }                                                                          \
  } while (0)

#define DFT_TRY(expr)                                                          \
  do { int _r = (expr); if (_r != DFTGPU_OK) return _r; } while (0)

// ------------------------------------------------------------------ runtime
struct Runtime {
  int device = -1;
  int num_sms = 0;
  int precision = DFTGPU_FP64;
  cudaStream_t stream = 0;
  size_t max_smem_optin = 0;
};
Runtime &rt();
int ensure_device();

// Streams for parallel graph branches: returns how many streams to use (the
// work stream included); aux[0..n-2] are the others, ev[0..n-1] fork / join
// events.
constexpr int PAR_MAX = 4;
int par_streams(cudaStream_t **aux, cudaEvent_t **ev);

// Device-resident FP64 accumulator slots used by reductions.
double *reduce_slots();
int reduce_partials(double **buf, size_t *n);

// ------------------------------------------------------------------ profiler
// When enabled (dftgpu_profile), every kernel launch is bracketed by CUDA
// events on the launching stream and tagged with a class name and its
// algorithmic bytes (each input read once, each output written once).
bool prof_on();
int prof_begin();                                     // returns a record id or -1
void prof_end(int id, const char *name, double bytes, int kernels = 1);

struct ProfScope {      // kernels: kernel launches inside the scope
  int id;
  const char *name;
  double bytes;
  int kernels;
  ProfScope(const char *n, double b, int k = 1) : id(prof_on() ? prof_begin() : -1), name(n), bytes(b), kernels(k) {}
  ~ProfScope() { if (id >= 0) prof_end(id, name, bytes, kernels); }
};

inline size_t elem_size(int prec) { return prec == DFTGPU_FP32 ? 4 : 8; }

}  // namespace dftgpu
