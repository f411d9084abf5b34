// Register-resident line FFTs for FP32 power-of-two lengths N = 64..512.
//
// Each thread owns E = 8 or 16 elements of one line; TL = N / E threads work
// on a line and a CTA of 256 threads holds B = 256 / TL lines.  A length-N
// transform is 2 or 3 Stockham stages with compile-time radices
//   N = 64: 8 x 8     N = 128: 16 x 8     N = 256: 16 x 16     N = 512: 16 x 16 x 2
// computed entirely in registers; only the stage boundaries exchange data
// through shared memory (one store + one load per element; the line pitch and
// skew of Shape<N>::LP / sidx() keep both mappings below free of bank
// conflicts).  The first stage reads
// element t + TL*q of its line and the last stage produces elements
// t + TL*j, so loads and stores go straight between HBM and registers:
//   EFAST mapping (thread t fast within a line): lines contiguous in memory
//     (y lines of the spectral layout, rows of real space);
//   LFAST mapping (line index fast): pencils strided in memory with adjacent
//     lines adjacent (x pencils) -- B lines give one contiguous run per element.
// Passes whose other side is transposed (the z pass writes [kz][x][y]) stage
// that side through shared memory with a cooperative line-fast loop.  The
// forward transform's output layout equals the inverse's input layout, so the
// x-pencil kernels apply k-space factors in registers between the two.
// Load / store functors may opt into split loads, store-side L2 prefetch,
// bounded entry points and a one-wave-ahead bulk L2 prefetch (see the traits
// before line_body).
#pragma once

#include <cooperative_groups.h>
#include <cuda.h>

#include "common.cuh"

namespace dftgpu {
namespace ff {

typedef float2 C;

// smallest value >= lo that is r (mod 16)
constexpr int pitch_mod_16(int lo, int r) { return lo % 16 <= r ? lo - lo % 16 + r : lo - lo % 16 + 16 + r; }

// Lengths 3 * 2^k (96, 192, 384) hold 12 elements per thread (radix 12 =
// 4 x 3 first, then 4 and 2); the powers of two 16 (8 for N = 64).
template <int N> struct Shape {
  static constexpr bool THREE = N % 3 == 0;
  static constexpr int E = THREE ? 12 : (N == 64) ? 8 : 16;
  static constexpr int NS = (N == 512 || N == 96 || N == 192) ? 3 : (N == 384) ? 4 : 2;
  static constexpr int TL = N / E;           // threads per line
  static constexpr int B = 256 / TL;         // lines per CTA
  // padded line pitch in shared memory (8-byte words; 16 bank pairs), chosen
  // with the skew e/16 of sidx() so that each access pattern of the line
  // kernels hits 16 different bank pairs per half-warp:
  //  TL = 16: a half-warp is 16 elements of one line, or 16 lines at one
  //           element: an odd pitch;
  //  TL = 8:  two lines x 8 elements, or 16 lines: pitch = 8 (mod 16) plus
  //           the line offset (l / 2) mod 16 of sidx() (the two lines' windows
  //           in opposite halves, 16 consecutive lines on 16 bank pairs);
  //  TL = 32: 8 lines x 2 adjacent elements (B = 8): pitch = 2 (mod 16).
  static constexpr int LP0 = N + N / 16 + 1;
  static constexpr int LP = TL == 8 ? pitch_mod_16(LP0 + 15, 8) : TL == 32 ? pitch_mod_16(LP0, 2) : LP0;
  static constexpr int SMEM = B * LP * (int) sizeof(C);
  template <int S> __host__ __device__ static constexpr int R() {
    // the first stage takes all E elements of a thread (one butterfly): the
    // loads fill slot q with element t + TL q, the first stage's input order
    if constexpr (N == 96) return S == 0 ? 12 : S == 1 ? 4 : 2;
    else if constexpr (N == 192) return S == 0 ? 12 : 4;
    else if constexpr (N == 384) return S == 0 ? 12 : S < 3 ? 4 : 2;
    else return N == 64 ? 8 : N == 128 ? (S == 0 ? 16 : 8) : N == 256 ? 16 : (S < 2 ? 16 : 2);
  }
  template <int S> __host__ __device__ static constexpr int P() {   // product of the radices before stage S
    if constexpr (S == 0) return 1;
    else return P<S - 1>() * R<S - 1>();
  }
};

template <int N> constexpr bool supported() {
  return N == 64 || N == 128 || N == 256 || N == 512 || N == 96 || N == 192 || N == 384;
}

__host__ __device__ constexpr int sidx(int l, int e, int LP) {
  return l * LP + e + (e >> 4) + ((LP & 15) == 8 ? ((l >> 1) & 15) : 0);
}

// --------------------------------------------------------------- butterflies
__device__ __forceinline__ C rot(C a, float s) { return make_float2(-s * a.y, s * a.x); }   // * (s i)

__device__ __forceinline__ void bf2(C *u) { C a = u[0]; u[0] = a + u[1]; u[1] = a - u[1]; }

__device__ __forceinline__ void bf4(C &a, C &b, C &c, C &d, float s) {   // in place, natural order
  C t0 = a + c, t1 = a - c, t2 = b + d, t3 = b - d;
  a = t0 + t2; c = t0 - t2; b = t1 + rot(t3, s); d = t1 - rot(t3, s);
}

// Rotation constants.  No float pair (c, s) has c^2 + s^2 = 1 exactly; the
// rounded 1/sqrt(2) gives 2 h^2 = 1 - 3.4e-8 and the rounded (cos, sin)(pi/8)
// 1 - 5.7e-8, a bias that lowers the norm at every stage.  Half of the
// rotations use the neighbouring float instead (hb: h^2 + hb^2 = 1 + 5.0e-8;
// c1b: c1b^2 + s1^2 = 1 + 5.3e-8), so that the deviations cancel on average
// (each constant stays within one ulp of its value).
constexpr float FF_H = 0.70710678118654752440f, FF_HB = 0.70710682868957519531f;
constexpr float FF_C1 = 0.92387953251128675613f, FF_C1B = 0.92387956380844116211f, FF_S1 = 0.38268343236508977173f;

__device__ __forceinline__ void bf8(C *u, float s) {
  const float h = FF_H, hb = FF_HB;
  C a0 = u[0] + u[4], a1 = u[0] - u[4], b0 = u[2] + u[6], b1 = u[2] - u[6];
  C c0 = u[1] + u[5], c1 = u[1] - u[5], d0 = u[3] + u[7], d1 = u[3] - u[7];
  C e0 = a0 + b0, e1 = a0 - b0, f0 = c0 + d0, f1 = c0 - d0;
  u[0] = e0 + f0; u[4] = e0 - f0; u[2] = e1 + rot(f1, s); u[6] = e1 - rot(f1, s);
  C b1w = rot(b1, s);
  C c1w = make_float2(h * (c1.x - s * c1.y), h * (c1.y + s * c1.x));
  C d1w = make_float2(-h * d1.x - hb * (s * d1.y), -h * d1.y + hb * (s * d1.x));
  C g0 = a1 + b1w, g1 = a1 - b1w, k0 = c1w + d1w, k1 = c1w - d1w;
  u[1] = g0 + k0; u[5] = g0 - k0; u[3] = g1 + rot(k1, s); u[7] = g1 - rot(k1, s);
}

// 16-point DFT as 4 x 4 with W16 twiddles; output in natural order
__device__ __forceinline__ void bf16(C *u, float s) {
  const float c1 = FF_C1, c1b = FF_C1B, s1 = FF_S1, h = FF_H, hb = FF_HB;
  // step 1: for n2 = 0..3, 4-point DFT over n1 of x[4 n1 + n2] -> y[n2][k1]
#pragma unroll
  for (int n2 = 0; n2 < 4; n2++) bf4(u[n2], u[4 + n2], u[8 + n2], u[12 + n2], s);
  // now u[4 k1 + n2] = y[n2][k1]; step 2: y[n2][k1] *= W16^(n2 k1), W16 = exp(s 2 pi i / 16)
  // n2 = 1: k1 = 1,2,3 -> W^1, W^2, W^3 ; n2 = 2 -> W^2, W^4, W^6 ; n2 = 3 -> W^3, W^6, W^9
  auto tw = [&](C &v, float cr, float ci) {   // v *= (cr + s i ci)
    const float im = s * ci;
    v = make_float2(v.x * cr - v.y * im, v.x * im + v.y * cr);
  };
  tw(u[4 + 1], c1b, s1); tw(u[8 + 1], h, hb);    tw(u[12 + 1], s1, c1);
  tw(u[4 + 2], h, h);    u[8 + 2] = rot(u[8 + 2], s); tw(u[12 + 2], -h, hb);
  tw(u[4 + 3], s1, c1);  tw(u[8 + 3], -h, h);    tw(u[12 + 3], -c1b, -s1);
  // step 3: for k1 = 0..3, 4-point DFT over n2 of y[n2][k1] = u[4 k1 + n2] -> X[k1 + 4 k2]
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) bf4(u[4 * k1 + 0], u[4 * k1 + 1], u[4 * k1 + 2], u[4 * k1 + 3], s);
  // u[4 k1 + k2] = X[k1 + 4 k2]: transpose the 4 x 4 block into natural order
  C t[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) t[k1 + 4 * k2] = u[4 * k1 + k2];
#pragma unroll
  for (int i = 0; i < 16; i++) u[i] = t[i];
}

__device__ __forceinline__ void bf3(C *u, float s) {
  const float s3 = 0.86602540378443864676f;
  const C a = u[0], b = u[1], c = u[2];
  const C m = a - (b + c) * 0.5f, d = (b - c) * s3;
  u[0] = a + b + c;
  u[1] = m + rot(d, s);
  u[2] = m - rot(d, s);
}

// 12 = 4 x 3 by the prime-factor map: input (3 n1 + 4 n2) mod 12, output
// (9 k1 + 4 k2) mod 12, no twiddles between the layers
__device__ __forceinline__ void bf12(C *u, float s) {
  C y[3][4];
#pragma unroll
  for (int n2 = 0; n2 < 3; n2++) {
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) y[n2][n1] = u[(3 * n1 + 4 * n2) % 12];
    bf4(y[n2][0], y[n2][1], y[n2][2], y[n2][3], s);
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    C z[3] = { y[0][k1], y[1][k1], y[2][k1] };
    bf3(z, s);
#pragma unroll
    for (int k2 = 0; k2 < 3; k2++) u[(9 * k1 + 4 * k2) % 12] = z[k2];
  }
}

template <int R> __device__ __forceinline__ void bfR(C *u, float s) {
  if constexpr (R == 2) bf2(u);
  else if constexpr (R == 4) bf4(u[0], u[1], u[2], u[3], s);
  else if constexpr (R == 8) bf8(u, s);
  else if constexpr (R == 12) bf12(u, s);
  else bf16(u, s);
}

// --------------------------------------------------------------- stages
// Register slot m*R + q of a thread holds input q of its butterfly m before a
// stage and output q after it; butterfly m of thread t is i = t + m*TL.
template <int N, int S>
__device__ __forceinline__ void stage(C (&v)[Shape<N>::E], int t, float s, const C *__restrict__ tw) {
  constexpr int E = Shape<N>::E, TL = Shape<N>::TL;
  constexpr int R = Shape<N>::template R<S>(), P = Shape<N>::template P<S>(), NB = E / R;
  constexpr int TWS = N / (P * R);
#pragma unroll
  for (int m = 0; m < NB; m++) {
    const int i = t + m * TL, k = i % P;
    if (P > 1) {
#pragma unroll
      for (int q = 1; q < R; q++) {
        C w = __ldg(&tw[q * k * TWS]);
        w.y *= -s;
        v[m * R + q] = cmul(v[m * R + q], w);
      }
    }
    bfR<R>(&v[m * R], s);
  }
}

// output position of register slot m*R + q after stage S
template <int N, int S> __host__ __device__ constexpr int out_pos(int t, int slot) {
  constexpr int TL = Shape<N>::TL, R = Shape<N>::template R<S>(), P = Shape<N>::template P<S>();
  const int m = slot / R, q = slot % R, i = t + m * TL, k = i % P;
  return (i - k) * R + k + q * P;
}
// input position of register slot m*R + q before stage S
template <int N, int S> __host__ __device__ constexpr int in_pos(int t, int slot) {
  constexpr int TL = Shape<N>::TL, R = Shape<N>::template R<S>();
  const int m = slot / R, q = slot % R;
  return t + m * TL + q * (N / R);
}

// Full transform in registers: on entry v[q] = x[t + TL q]; on exit v[slot]
// = X[out_pos<N, NS-1>(t, slot)], which is t + TL * j(slot).  A line's
// exchange touches only its own row of sm, so when its TL threads are lanes
// of one warp (WARP: the element-fast mapping, t = threadIdx % TL) the
// exchange needs a warp barrier only; otherwise the CTA barrier.
template <int N, int S = 0, bool WARP = false>
__device__ __forceinline__ void transform(C (&v)[Shape<N>::E], int t, int l, float s, const C *__restrict__ tw,
                                          C *__restrict__ sm) {
  constexpr int E = Shape<N>::E, LP = Shape<N>::LP;
  static_assert(!WARP || 32 % Shape<N>::TL == 0, "a line within one warp");
  stage<N, S>(v, t, s, tw);
  if constexpr (S + 1 < Shape<N>::NS) {
#pragma unroll
    for (int j = 0; j < E; j++) sm[sidx(l, out_pos<N, S>(t, j), LP)] = v[j];
    if constexpr (WARP) __syncwarp(); else __syncthreads();
#pragma unroll
    for (int j = 0; j < E; j++) v[j] = sm[sidx(l, in_pos<N, S + 1>(t, j), LP)];
    if constexpr (WARP) __syncwarp(); else __syncthreads();
    transform<N, S + 1, WARP>(v, t, l, s, tw, sm);
  }
}

// element index held by register slot j after a full transform (= t + TL * jj)
template <int N> __host__ __device__ constexpr int final_pos(int t, int j) { return out_pos<N, Shape<N>::NS - 1>(t, j); }

// register slot that holds element t + TL*q after a forward transform (the
// inverse transform wants element t + TL*q in slot q)
template <int N> __host__ __device__ constexpr int slot_of(int q) {
  // final_pos(t, j) = t + TL * jj(j) independent of t; invert jj
  for (int j = 0; j < Shape<N>::E; j++)
    if (out_pos<N, Shape<N>::NS - 1>(0, j) == Shape<N>::TL * q) return j;
  return 0;
}

template <int N> __device__ __forceinline__ void to_input_order(C (&v)[Shape<N>::E]) {
  constexpr int E = Shape<N>::E;
  C t[E];
#pragma unroll
  for (int q = 0; q < E; q++) t[q] = v[slot_of<N>(q)];
#pragma unroll
  for (int q = 0; q < E; q++) v[q] = t[q];
}

// --------------------------------------------------------------- asynchronous copies
__device__ __forceinline__ unsigned su32(const void *p) { return (unsigned) __cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned cl_addr(unsigned a, unsigned rank) {   // shared::cluster address in CTA rank
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for the completion of phase `parity`; after 0.5 s the wait gives up,
// records the failure in *fault (read by the host after the launch) and
// returns false.  A thread whose wait gave up skips its global stores, and
// every CTA ends with a cluster barrier, so no CTA exits before each peer has
// passed its own bounded waits.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int *fault) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (!mbar_try_wait(bar, parity)) {
    if (gtimer() - t0 > 500000000ull) { atomicExch(fault, 1); return false; }
  }
  return true;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_g2s(unsigned dst, const void *src, unsigned bytes, unsigned bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void bulk_s2c(unsigned dst, unsigned src, unsigned bytes, unsigned bar) {
  asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "r"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// TMA (cp.async.bulk.tensor) of one 3-D box of a tensor map: load into shared
// memory completing on an mbarrier, store from shared memory as a bulk group.
// The tensor map is a __grid_constant__ kernel parameter (its generic address).
__device__ __forceinline__ void tma_load_3d(unsigned dst, const void *tmap, int c0, int c1, int c2, unsigned bar) {
  asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
               ::"r"(dst), "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void tma_store_3d(const void *tmap, int c0, int c1, int c2, unsigned src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];"
               ::"l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(src)
               : "memory");
}
// Byte offset of 8-byte element (row, col) of a box stored with the 128-byte
// swizzle (16 elements per 128-byte row; the 16-byte chunk index is XORed
// with the row index mod 8; the box starts on a 1024-byte boundary).
__device__ __forceinline__ int swz128(int row, int col) {
  return row * 128 + ((((col >> 1) ^ (row & 7)) << 4) | ((col & 1) << 3));
}

// --------------------------------------------------------------- line pass
enum { MAP_E = 0, MAP_L = 1 };

// Optional split interface of the load / store functors, detected by a
// member kSplit: a split load functor separates fetch(a, b, e) -> Raw from
// cook(Raw) -> C, so that all global loads of a thread are in flight before
// the first value is combined; a split store functor has prefetch(a, b, e),
// called before the transform for the elements it will store.
template <class F> __host__ __device__ constexpr auto split_of(int) -> decltype(F::kSplit, bool()) { return F::kSplit; }
template <class F> __host__ __device__ constexpr bool split_of(long) { return false; }
// Load functors with kAhead: each CTA prefetches into L2 the input of the CTA
// `ahead` places after it (one wave of resident CTAs later), whose loads then
// hit L2 instead of waiting on DRAM.
template <class F> __host__ __device__ constexpr auto bounded_store_of(int) -> decltype(F::kBoundedStore, bool()) { return F::kBoundedStore; }
template <class F> __host__ __device__ constexpr bool bounded_store_of(long) { return false; }
template <class F> __host__ __device__ constexpr auto ahead_of(int) -> decltype(F::kAhead, bool()) { return F::kAhead; }
template <class F> __host__ __device__ constexpr bool ahead_of(long) { return false; }
template <int N, int MODE, int B, class Ld> __device__ __forceinline__ void prefetch_ahead(const Ld &ld, int ahead) {
  if constexpr (ahead_of<Ld>(0)) {
    const int id = blockIdx.y * gridDim.x + blockIdx.x + ahead;
    if (ahead > 0 && id < (int) (gridDim.x * gridDim.y)) {
      const int a2 = id / gridDim.x, b2 = (id - a2 * gridDim.x) * B;
      ld.prefetch_lines(a2, b2, B, MODE == 2 ? N + 1 : N);
    }
  }
}

// TMA staging of the transposed side of a z pass: the [kz][x][y] tile of a
// CTA (its B lines, the N or N+1 kz values) moves as B/16 boxes {16 y, 1 x,
// rows kz} of a 3-D tensor map over the spectral buffer, with the 128-byte
// swizzle; each box starts on a 1024-byte boundary of shared memory.
struct alignas(64) TmaMaps {
  CUtensorMap load, store;   // the staged load / store side (the unused one is not read)
};
template <int N, int MODE> struct TmaTile {
  static constexpr int ROWS = MODE == 0 ? N : N + 1;           // kz values of the tile
  static constexpr int NBOX = Shape<N>::B / 16;
  static constexpr int BOXB = ((ROWS * 128 + 1023) / 1024) * 1024;
  static constexpr int BYTES = NBOX * BOXB;
  static constexpr bool OK = ROWS <= 256 && Shape<N>::B % 16 == 0;
};
// Shared memory of a line pass: the transform's exchange buffer, which also
// holds the TMA boxes (1024-byte aligned) when TMA is on.
template <int N, int MODE, int TMA> struct LineSmem {
  static constexpr int XB = Shape<N>::B * Shape<N>::LP * (int) sizeof(C);
  static constexpr int TB = TMA ? TmaTile<N, MODE>::BYTES : 0;
  static constexpr int BYTES = (XB > TB ? XB : TB) + (TMA ? 1024 : 0);
};

// MODE 0 C2C, 1 R2C (N = nz/2, post-processed to N+1 outputs), 2 C2R.
// LDS / STS: stage the load / store side through shared memory with a
// line-fast cooperative loop (used for the transposed side of z passes).
// TMA: the staged side moves by TMA instead (tensor maps in tm, bounded wait
// recorded in *fault; a thread whose wait gave up skips its global stores).
template <int N, int MODE, int MAP, int LDS, int STS, int TMA, class Ld, class St>
__device__ __forceinline__ void line_body(const C *__restrict__ tw, const C *__restrict__ tw2, float sign,
                                          const Ld &ld, const St &st, int ahead, const TmaMaps *tm, int *fault) {
  constexpr int E = Shape<N>::E, TL = Shape<N>::TL, B = Shape<N>::B, LP = Shape<N>::LP;
  typedef TmaTile<N, MODE> TT;
  static_assert(!TMA || TT::OK, "TMA tile");
  __shared__ __align__(16) unsigned char smraw[LineSmem<N, MODE, TMA>::BYTES];
  __shared__ unsigned long long tbar;
  unsigned char *smb = smraw;
  if constexpr (TMA) smb += (1024 - (su32(smraw) & 1023)) & 1023;
  C *sm = reinterpret_cast<C *>(smb);
  const int a = blockIdx.y, b0 = blockIdx.x * B;
  const int t = MAP == MAP_E ? threadIdx.x % TL : threadIdx.x / B;
  const int l = MAP == MAP_E ? threadIdx.x / TL : threadIdx.x % B;
  bool ok = true;
  C v[E];
  if constexpr (LDS == 0 && split_of<Ld>(0)) {
    typename Ld::Raw raw[E];
#pragma unroll
    for (int q = 0; q < E; q++) raw[q] = ld.fetch(a, b0 + l, t + TL * q);
    prefetch_ahead<N, MODE, B>(ld, ahead);   // after the own loads: issued before it, they are not delayed
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = ld.cook(raw[q]);
  } else if constexpr (LDS == 0) {
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = ld(a, b0 + l, t + TL * q);
    prefetch_ahead<N, MODE, B>(ld, ahead);
  } else {
    if constexpr (TMA) {
      // the tile's boxes by TMA (one thread), completion on an mbarrier
      const unsigned sb = su32(smb), mb = su32(&tbar);
      if (threadIdx.x == 0) {
        mbar_init(mb, 1);
        fence_mbar_init();
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        mbar_expect_tx(mb, TT::NBOX * TT::ROWS * 128);
#pragma unroll
        for (int h = 0; h < TT::NBOX; h++) tma_load_3d(sb + h * TT::BOXB, &tm->load, b0 + 16 * h, a, 0, mb);
      }
      ok = mbar_wait(mb, 0, fault);
      prefetch_ahead<N, MODE, B>(ld, ahead);
    } else {
      // line-fast cooperative load of the whole tile (C2R: also the Nyquist
      // element N, which lands in the pitch's spare slot), fully unrolled so
      // that every load is in flight before the first shared-memory store
      constexpr int NE = MODE == 2 ? N + 1 : N, TOT = B * NE, IT = (TOT + 255) / 256;
#pragma unroll
      for (int it = 0; it < IT; it++) {
        const int idx = threadIdx.x + it * 256;
        if (TOT % 256 == 0 || idx < TOT) {
          const int ll = idx % B, e = idx / B;
          sm[sidx(ll, e, LP)] = ld(a, b0 + ll, e);
        }
      }
      prefetch_ahead<N, MODE, B>(ld, ahead);
      __syncthreads();
    }
    // element e of this thread's line from the staged tile
    auto staged = [&](int e) -> C {
      if constexpr (TMA) return *reinterpret_cast<const C *>(smb + (l >> 4) * TT::BOXB + swz128(e, l & 15));
      else return sm[sidx(l, e, LP)];
    };
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int e = t + TL * q;
      if constexpr (MODE == 2) {
        // Z[k] = (X[k] + X*[N-k]) + i w^-k (X[k] - X*[N-k]),  w = exp(-2 pi i / 2N)
        C xk = staged(e), xm = staged(N - e);
        if (e == 0) { xk.y = 0.f; xm.y = 0.f; }
        const C sum = make_float2(xk.x + xm.x, xk.y - xm.y), dif = make_float2(xk.x - xm.x, xk.y + xm.y);
        C w = __ldg(&tw2[e]);
        w.y = -w.y;
        const C tt = cmul(dif, w);
        v[q] = make_float2(sum.x - tt.y, sum.y + tt.x);
      } else {
        v[q] = staged(e);
      }
    }
    __syncthreads();
  }
  if constexpr (STS == 0 && split_of<St>(0)) {
#pragma unroll
    for (int j = 0; j < E; j++) st.prefetch(a, b0 + l, final_pos<N>(t, j));
  }
  transform<N, 0, MAP == MAP_E>(v, t, l, sign, tw, sm);
  if constexpr (STS == 0) {
    if (ok) {
#pragma unroll
      for (int j = 0; j < E; j++) st(a, b0 + l, final_pos<N>(t, j), v[j]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < E; j++) sm[sidx(l, final_pos<N>(t, j), LP)] = v[j];
    __syncthreads();
    if constexpr (TMA) {
      // the output tile in registers first (the boxes overlay the exchange
      // buffer), then into the swizzled boxes and out by TMA
      constexpr int TOT = MODE == 1 ? B * (N / 2 + 1) : B * N, IT = (TOT + 255) / 256;
      C xa[IT], xb[IT];
#pragma unroll
      for (int it = 0; it < IT; it++) {
        const int idx = threadIdx.x + it * 256;
        if (idx < TOT) {
          const int ll = idx % B, k = idx / B;
          if constexpr (MODE == 1) {
            const C zk = sm[sidx(ll, k, LP)], zm = sm[sidx(ll, k == 0 ? 0 : N - k, LP)];
            const C sum = make_float2(zk.x + zm.x, zk.y - zm.y), dif = make_float2(zk.x - zm.x, zk.y + zm.y);
            const C tt = cmul(dif, __ldg(&tw2[k]));
            xa[it] = make_float2(0.5f * (sum.x + tt.y), 0.5f * (sum.y - tt.x));
            xb[it] = make_float2(0.5f * (sum.x - tt.y), -0.5f * (sum.y + tt.x));
          } else {
            xa[it] = sm[sidx(ll, k, LP)];
          }
        }
      }
      __syncthreads();
#pragma unroll
      for (int it = 0; it < IT; it++) {
        const int idx = threadIdx.x + it * 256;
        if (idx < TOT) {
          const int ll = idx % B, k = idx / B;
          unsigned char *box = smb + (ll >> 4) * TT::BOXB;
          *reinterpret_cast<C *>(box + swz128(k, ll & 15)) = xa[it];
          if (MODE == 1 && k != N / 2) *reinterpret_cast<C *>(box + swz128(N - k, ll & 15)) = xb[it];
        }
      }
      fence_proxy_async();   // the generic-proxy writes above, visible to the TMA store
      __syncthreads();
      if (threadIdx.x == 0) {
#pragma unroll
        for (int h = 0; h < TT::NBOX; h++) tma_store_3d(&tm->store, b0 + 16 * h, a, 0, su32(smb) + h * TT::BOXB);
        bulk_commit();
        bulk_wait_read();   // the boxes have been read before the CTA's shared memory is released
      }
    } else if constexpr (MODE == 1) {
      // X[k] = (Z[k] + Z*[N-k]) / 2 - (i/2) w^k (Z[k] - Z*[N-k]),  k = 0..N, in
      // pairs: with sum = Z[k] + Z*[N-k] and tt = w^k (Z[k] - Z*[N-k]),
      // X[k] = (sum - i tt) / 2 and X[N-k] = conj(sum + i tt) / 2 (w^N = -1),
      // so one read of Z[k], Z[N-k] gives both outputs (k = 0: X[0] and X[N];
      // k = N/2 pairs with itself)
      constexpr int TOT = B * (N / 2 + 1), IT = (TOT + 255) / 256;
#pragma unroll
      for (int it = 0; it < IT; it++) {
        const int idx = threadIdx.x + it * 256;
        if (idx < TOT) {
          const int ll = idx % B, k = idx / B;
          const C zk = sm[sidx(ll, k, LP)], zm = sm[sidx(ll, k == 0 ? 0 : N - k, LP)];
          const C sum = make_float2(zk.x + zm.x, zk.y - zm.y), dif = make_float2(zk.x - zm.x, zk.y + zm.y);
          const C tt = cmul(dif, __ldg(&tw2[k]));
          st(a, b0 + ll, k, make_float2(0.5f * (sum.x + tt.y), 0.5f * (sum.y - tt.x)));
          if (k != N / 2) st(a, b0 + ll, N - k, make_float2(0.5f * (sum.x - tt.y), -0.5f * (sum.y + tt.x)));
        }
      }
    } else {
      constexpr int IT = B * N / 256;
#pragma unroll
      for (int it = 0; it < IT; it++) {
        const int idx = threadIdx.x + it * 256;
        const int ll = idx % B, e = idx / B;
        st(a, b0 + ll, e, sm[sidx(ll, e, LP)]);
      }
    }
  }
}

template <int N, int MODE, int MAP, int LDS, int STS, int TMA, class Ld, class St>
__global__ void __launch_bounds__(256) line_kernel(const C *__restrict__ tw, const C *__restrict__ tw2, float sign,
                                                   const Ld ld, const St st, int ahead,
                                                   const __grid_constant__ TmaMaps tm, int *fault) {
  line_body<N, MODE, MAP, LDS, STS, TMA>(tw, tw2, sign, ld, st, ahead, &tm, fault);
}
// Passes whose store functor asks for it (kBoundedStore: the inverse phase
// pass, whose operand loads follow the transform): bounded to 48 registers,
// 5 CTAs per SM, to hide their latency.
template <int N, int MODE, int MAP, int LDS, int STS, int TMA, class Ld, class St>
__global__ void __launch_bounds__(256, 5) line_kernel_stsplit(const C *__restrict__ tw, const C *__restrict__ tw2,
                                                              float sign, const Ld ld, const St st, int ahead,
                                                              const __grid_constant__ TmaMaps tm, int *fault) {
  line_body<N, MODE, MAP, LDS, STS, TMA>(tw, tw2, sign, ld, st, ahead, &tm, fault);
}
// Split loads hold all of a thread's operands (two complex per element) at
// once; the bound keeps them to 80 registers, 3 CTAs per SM, without spills.
template <int N, int MODE, int MAP, int LDS, int STS, int TMA, class Ld, class St>
__global__ void __launch_bounds__(256, 3) line_kernel_split(const C *__restrict__ tw, const C *__restrict__ tw2,
                                                            float sign, const Ld ld, const St st, int ahead,
                                                            const __grid_constant__ TmaMaps tm, int *fault) {
  line_body<N, MODE, MAP, LDS, STS, TMA>(tw, tw2, sign, ld, st, ahead, &tm, fault);
}

// --------------------------------------------------------------- x pencils
// LFAST pencils of the spectral layout [kz][x][y]: line (kz, y), element x.
struct XArgsF {
  int nx, ny, kxh, kyh;
  int nin, nout, nslice, pad_;
  const C *src[4];
  C *dst[8];
  int acc_out[8];             // 1: dst += result
  int nterm[8], t0[8];        // terms of each output
  int kind[16], in[16];       // kernel symmetry (0 even, 1 odd x, 2 odd y, 3 odd z, 4 unit), input
  int slot[16];               // kernel slice used by the term (-1: unit)
  float coef[16];
  const float *slice_src[8];  // distinct kernel octants of this launch
};

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned s = (unsigned) __cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::); }

// w[j] (+)= K_tm(kx_j, ky) v[j] for all of a thread's elements (x = the
// element's final position): the term's kind, coefficient and kernel slice
// are read once per call and each symmetry kind has its own loop.
template <int N, bool ACC>
__device__ __forceinline__ void kmul_all(const XArgsF &A, const float *ks, int tm, const C (&v)[Shape<N>::E],
                                         C (&w)[Shape<N>::E], int t, int y, int iyo) {
  constexpr int E = Shape<N>::E, B = Shape<N>::B, KXH = N / 2 + 1;
  const int kind = A.kind[tm];
  const float coef = A.coef[tm];
  if (kind == 4) {
#pragma unroll
    for (int j = 0; j < E; j++) w[j] = ACC ? w[j] + v[j] * coef : v[j] * coef;
    return;
  }
  const float *kk = ks + A.slot[tm] * KXH * B + iyo;
  if (kind == 0) {
#pragma unroll
    for (int j = 0; j < E; j++) {
      const int x = final_pos<N>(t, j), ix = x <= N / 2 ? x : N - x;
      const C r = v[j] * (kk[ix * B] * coef);
      w[j] = ACC ? w[j] + r : r;
    }
    return;
  }
  // odd kernels: (i sg kv) v, sg = -1 on the negative-frequency half of the odd axis
  const float sgy = (kind == 2 && y > A.ny / 2) ? -coef : coef;
#pragma unroll
  for (int j = 0; j < E; j++) {
    const int x = final_pos<N>(t, j), ix = x <= N / 2 ? x : N - x;
    const float sg = kind == 1 ? (x > N / 2 ? -coef : coef) : sgy;
    const float kv = kk[ix * B] * sg;
    const C r = make_float2(-kv * v[j].y, kv * v[j].x);
    w[j] = ACC ? w[j] + r : r;
  }
}

template <int N> constexpr int xconv_smem(int nslice) {
  return Shape<N>::B * Shape<N>::LP * (int) sizeof(C) + nslice * (N / 2 + 1) * Shape<N>::B * (int) sizeof(float);
}

// Inputs are processed one after the other (forward FFT in registers).
// MODE 0: every output has one term and is produced right after its input.
// MODE 1: as 0, plus at most one output with several terms (index `multi`)
//         accumulated in registers and produced at the end.
// MODE 2: a single output, the sum of all terms, accumulated in registers;
//         while one input is transformed, the CTA's pencils of the next
//         input are bulk-prefetched into L2 (128-byte runs, one per thread).
// The launch parameters are staged in shared memory, and this CTA's slice of
// every kernel octant (all kx, the B ky of its pencils) is fetched with
// cp.async while the first input is loaded and transformed.
// Requires B | ny/2 so that a CTA's pencils lie on one side of ny/2.
template <int N, int MODE>
__global__ void __launch_bounds__(256, MODE == 1 ? 1 : (MODE == 0 ? 3 : 2)) xconv_kernel(const C *__restrict__ tw, const XArgsF A, int multi) {
  constexpr bool MULTI = MODE == 1;
  constexpr int E = Shape<N>::E, TL = Shape<N>::TL, B = Shape<N>::B, LP = Shape<N>::LP, KXH = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  float *ks = reinterpret_cast<float *>(sm + B * LP);
  __shared__ XArgsF sA;
  {
    const int *sw = reinterpret_cast<const int *>(&A);
    int *dw = reinterpret_cast<int *>(&sA);
    for (int i = threadIdx.x; i < (int) (sizeof(XArgsF) / sizeof(int)); i += 256) dw[i] = sw[i];
  }
  const int kz = blockIdx.y, y0 = blockIdx.x * B, l = threadIdx.x % B, t = threadIdx.x / B, y = y0 + l;
  const int half = A.ny / 2;
  const int iylo = y0 < half ? y0 : A.ny - (y0 + B - 1);
  const int iyo = (y <= half ? y : A.ny - y) - iylo;
  for (int idx = threadIdx.x; idx < A.nslice * KXH * B; idx += 256) {
    const int s = idx / (KXH * B), r = idx % (KXH * B), ix = r / B, c = r % B;
    cp_async4(&ks[idx], A.slice_src[s] + ((size_t) kz * A.kxh + ix) * A.kyh + iylo + c);
  }
  cp_async_commit();
  const size_t plane = (size_t) A.nx * A.ny;
  if constexpr (MODE == 2) {
    C acc[E], v[E];
#pragma unroll
    for (int j = 0; j < E; j++) acc[j] = make_float2(0.f, 0.f);
    {
      const C *src = A.src[0] + kz * plane + y;
#pragma unroll
      for (int q = 0; q < E; q++) v[q] = src[(size_t) (t + TL * q) * A.ny];
    }
    __syncthreads();   // sA ready
    for (int in = 0; in < sA.nin; in++) {
      if (in > 0) {
        const C *src = sA.src[in] + kz * plane + y;
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = src[(size_t) (t + TL * q) * A.ny];
      }
      if (in + 1 < sA.nin) {   // the next input's pencils of this CTA into L2 while this one is transformed
        const C *nsrc = sA.src[in + 1] + kz * plane + y0;
        for (int x = threadIdx.x; x < N; x += 256) prefetch_bulk_l2(nsrc + (size_t) x * A.ny, B * sizeof(C));
      }
      transform<N>(v, t, l, -1.f, tw, sm);
      if (in == 0) {
        cp_async_wait_all();
        __syncthreads();   // kernel slices visible to all threads
      }
      for (int tm = 0; tm < sA.nterm[0]; tm++) {
        if (sA.in[tm] != in) continue;
        kmul_all<N, true>(sA, ks, tm, v, acc, t, y, iyo);
      }
    }
    to_input_order<N>(acc);
    transform<N>(acc, t, l, 1.f, tw, sm);
    C *dst = sA.dst[0] + kz * plane + y;
#pragma unroll
    for (int j = 0; j < E; j++) {
      C r = acc[j];
      const size_t off = (size_t) final_pos<N>(t, j) * A.ny;
      if (sA.acc_out[0]) r = r + dst[off];
      dst[off] = r;
    }
    return;
  }
  C acc[MULTI ? E : 1];
  if constexpr (MULTI) {
#pragma unroll
    for (int j = 0; j < E; j++) acc[j] = make_float2(0.f, 0.f);
  }
  __syncthreads();   // sA ready
  for (int in = 0; in < sA.nin; in++) {
    const C *src = sA.src[in] + kz * plane + y;
    C v[E];
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = src[(size_t) (t + TL * q) * A.ny];
    if (in + 1 < sA.nin) {   // the next input's pencils of this CTA into L2 (as MODE 2)
      const C *nsrc = sA.src[in + 1] + kz * plane + y0;
      for (int x = threadIdx.x; x < N; x += 256) prefetch_bulk_l2(nsrc + (size_t) x * A.ny, B * sizeof(C));
    }
    transform<N>(v, t, l, -1.f, tw, sm);
    if (in == 0) {
      cp_async_wait_all();
      __syncthreads();   // kernel slices visible to all threads
    }
    for (int o = 0; o < sA.nout; o++) {
      if constexpr (MULTI) {
        if (o == multi) {
          for (int tm = sA.t0[o]; tm < sA.t0[o] + sA.nterm[o]; tm++) {
            if (sA.in[tm] != in) continue;
            kmul_all<N, true>(sA, ks, tm, v, acc, t, y, iyo);
          }
          continue;
        }
      }
      const int tm = sA.t0[o];
      if (sA.in[tm] != in) continue;
      C w[E];
      kmul_all<N, false>(sA, ks, tm, v, w, t, y, iyo);
      to_input_order<N>(w);
      transform<N>(w, t, l, 1.f, tw, sm);
      C *dst = sA.dst[o] + kz * plane + y;
      const bool accum = sA.acc_out[o];
#pragma unroll
      for (int j = 0; j < E; j++) {
        C r = w[j];
        const size_t off = (size_t) final_pos<N>(t, j) * A.ny;
        if (accum) r = r + dst[off];
        dst[off] = r;
      }
    }
  }
  if constexpr (MULTI) {
    if (multi >= 0) {
      to_input_order<N>(acc);
      transform<N>(acc, t, l, 1.f, tw, sm);
      C *dst = sA.dst[multi] + kz * plane + y;
#pragma unroll
      for (int j = 0; j < E; j++) {
        C r = acc[j];
        const size_t off = (size_t) final_pos<N>(t, j) * A.ny;
        if (sA.acc_out[multi]) r = r + dst[off];
        dst[off] = r;
      }
    }
  }
}

// psi(k) *= exp(cdt k^2) / N between forward and inverse x transforms; CN:
// the Crank-Nicolson factor of the finite-difference kinetic operator, one per
// axis (cn_m1; h the grid step)
template <int N, bool CN>
__global__ void __launch_bounds__(256) xkinetic_kernel(const C *__restrict__ tw, C *data, int ny, int nz, float2 cdt,
                                                      float inv_n, float dkx, float dky, float dkz, float kx0,
                                                      float ky0, float kz0, float h) {
  constexpr int E = Shape<N>::E, TL = Shape<N>::TL, B = Shape<N>::B, LP = Shape<N>::LP;
  __shared__ C sm[B * LP];
  __shared__ C fx[N];   // exp(cdt (kx - kx0)^2) - 1
  const int kz = blockIdx.y, l = threadIdx.x % B, t = threadIdx.x / B, y = blockIdx.x * B + l;
  for (int e = threadIdx.x; e < N; e += 256) {
    const float k = (float) (e < (N + 1) / 2 ? e : e - N) * dkx - kx0;
    fx[e] = CN ? cn_m1(cdt, k, h) : cexpm1(make_float2(cdt.x * (k * k), cdt.y * (k * k)));
  }
  C fyz;                // exp(cdt ((ky - ky0)^2 + (kz - kz0)^2)) - 1 of this thread's line
  {
    const float kzv = (float) (kz < (nz + 1) / 2 ? kz : kz - nz) * dkz - kz0;
    const float kyv = (float) (y < (ny + 1) / 2 ? y : y - ny) * dky - ky0;
    const float q = kyv * kyv + kzv * kzv;
    fyz = CN ? cprod1p(cn_m1(cdt, kyv, h), cn_m1(cdt, kzv, h)) : cexpm1(make_float2(cdt.x * q, cdt.y * q));
  }
  C *base = data + kz * (size_t) N * ny + y;
  C v[E];
#pragma unroll
  for (int q = 0; q < E; q++) v[q] = base[(size_t) (t + TL * q) * ny];
  transform<N>(v, t, l, -1.f, tw, sm);
  __syncthreads();      // fx complete (the transform's own barriers do not cover the last writes)
#pragma unroll
  for (int j = 0; j < E; j++)
    v[j] = mul_1p(make_float2(v[j].x * inv_n, v[j].y * inv_n), cprod1p(fx[final_pos<N>(t, j)], fyz));
  to_input_order<N>(v);
  transform<N>(v, t, l, 1.f, tw, sm);
#pragma unroll
  for (int j = 0; j < E; j++) base[(size_t) final_pos<N>(t, j) * ny] = v[j];
}

// --------------------------------------------------------------- factorised kinetic passes
// exp(cdt |k - k0|^2) is a product of one factor per axis, and the 3-D DFT is
// the product of the three 1-D DFTs, so F^-1 K F = prod_a (F_a^-1 K_a F_a):
// the kinetic step of the split-operator propagator runs as one pass per axis,
// each a line FFT, the factor exp(cdt (k_a - k0_a)^2) / n_a applied as
// v + v f (f = exp(.) - 1, tabulated per CTA in shared memory), and the
// inverse line FFT.  Every pass reads and writes the wave function in its own
// [x][y][z] layout (no transposed spectra): z rows (element-fast), y and x
// lines strided with B consecutive z per CTA (line-fast).  The potential
// half steps are the load functor of the z pass and the store functor of the
// x pass.  Bounds: MINB CTAs per SM (split load / bounded store variants).
template <int N, int MAP, int MINB, class Ld, class St>
__global__ void __launch_bounds__(256, MINB) line_kin_kernel(const C *__restrict__ tw, float2 cdt, float inv_n, float dk,
                                                             float k0, const Ld ld, const St st, int ahead) {
  constexpr int E = Shape<N>::E, TL = Shape<N>::TL, B = Shape<N>::B, LP = Shape<N>::LP;
  __shared__ C sm[B * LP];
  __shared__ C fk[N];   // exp(cdt (k - k0)^2) - 1
  const int a = blockIdx.y, b0 = blockIdx.x * B;
  const int t = MAP == MAP_E ? threadIdx.x % TL : threadIdx.x / B;
  const int l = MAP == MAP_E ? threadIdx.x / TL : threadIdx.x % B;
  C v[E];
  if constexpr (split_of<Ld>(0)) {
    typename Ld::Raw raw[E];
#pragma unroll
    for (int q = 0; q < E; q++) raw[q] = ld.fetch(a, b0 + l, t + TL * q);
    prefetch_ahead<N, 0, B>(ld, ahead);
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = ld.cook(raw[q]);
  } else {
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = ld(a, b0 + l, t + TL * q);
    prefetch_ahead<N, 0, B>(ld, ahead);
  }
  for (int e = threadIdx.x; e < N; e += 256) {
    const float k = (float) (e < (N + 1) / 2 ? e : e - N) * dk - k0;
    fk[e] = cexpm1(make_float2(cdt.x * (k * k), cdt.y * (k * k)));
  }
  if constexpr (split_of<St>(0)) {
#pragma unroll
    for (int j = 0; j < E; j++) st.prefetch(a, b0 + l, final_pos<N>(t, j));
  }
  transform<N>(v, t, l, -1.f, tw, sm);
  __syncthreads();      // fk complete (the transform's own barriers precede its last stage)
#pragma unroll
  for (int j = 0; j < E; j++) v[j] = mul_1p(make_float2(v[j].x * inv_n, v[j].y * inv_n), fk[final_pos<N>(t, j)]);
  to_input_order<N>(v);
  transform<N>(v, t, l, 1.f, tw, sm);
#pragma unroll
  for (int j = 0; j < E; j++) st(a, b0 + l, final_pos<N>(t, j), v[j]);
}

// --------------------------------------------------------------- fused z + y plane passes
// The z and y passes of a real field's 3-D transform done by one cluster of
// CL CTAs per x plane, so the half spectrum crosses HBM once instead of
// three times.  CTA r of a cluster owns rows y = r*RY .. r*RY+RY-1 of the
// (y, kz) plane and the KC column lines c = r*KC .. r*KC+KC-1.  Data move by
// bulk asynchronous copies that complete on mbarriers: rows / columns from
// global memory into a staging area, and the plane exchange between the
// CTAs as one contiguous block per (source, destination) pair, laid out
// [kz][row] on one side and [source][column][row] on the other.  The z = 0
// and z = NZC (Nyquist) columns are real in y space; they travel as one
// complex column X_0 + i X_NZC, so the NZC column lines split evenly.
template <int NY, int NZ, int CL> struct ZYPlane {
  static constexpr int NZC = NZ / 2;            // packed complex z length
  static constexpr int BY = Shape<NY>::B;       // column lines per batch
  static constexpr int BZ = Shape<NZC>::B;      // rows per batch
  static constexpr int RY = NY / CL;            // rows per CTA
  static constexpr int KC = NZC / CL;           // column lines per CTA
  static constexpr int CB = KC / BY;            // column batches per CTA
  static constexpr int RB = RY / BZ;            // row batches per CTA
  static constexpr int PRW = NZC + 8;           // staged row pitch (complex pairs)
  static constexpr int PC = NY + 8;             // staged column pitch
  static constexpr int PLT = (NZC + 2) * RY;    // plane [kz][row]
  static constexpr int IN = CL * KC * RY;       // exchange blocks [source or destination][column][row]
  static constexpr int STF = RY * PRW, STI = KC * PC;
  static constexpr int A1 = IN > STF ? (IN > STI ? IN : STI) : (STF > STI ? STF : STI);
  static constexpr int NQ = CL * RY;            // Nyquist row blocks
  static constexpr int NQS = NY;                // staged Nyquist column (inverse, rank 0)
  static constexpr int SCRY = BY * Shape<NY>::LP, SCRZ = BZ * Shape<NZC>::LP;
  static constexpr int SCR = SCRY > SCRZ ? SCRY : SCRZ;
  static constexpr int SMEM = (PLT + A1 + NQ + NQS + SCR) * (int) sizeof(C) + 16;
  static_assert(supported<NY>() && supported<NZC>(), "fused plane pass lengths");
  static_assert(CB == 1 && KC == BY && RB >= 1 && RY % BZ == 0 && NY % CL == 0 && NZC % CL == 0,
                "fused plane split");
  static_assert(NZC % 16 == 0 && NY % 16 == 0, "staged pitches stay 16-byte multiples");
};


// forward: real field f[x][y][z] -> spec[kz][x][y], kz = 0..NZC
template <int NY, int NZ, int CL>
__global__ void __launch_bounds__(256, 2) zy_r2c_kernel(const C *__restrict__ twz, const C *__restrict__ tw2z,
                                                        const C *__restrict__ twy, const float *__restrict__ f,
                                                        C *__restrict__ spec, int nx, int *fault) {
  typedef ZYPlane<NY, NZ, CL> Z;
  namespace cg = cooperative_groups;
  extern __shared__ __align__(128) unsigned char smraw[];
  C *plt = reinterpret_cast<C *>(smraw);   // [NZC+2][RY]
  C *a1 = plt + Z::PLT;                    // staged rows [RY][PRW], then incoming [CL][KC][RY]
  C *nq = a1 + Z::A1;                      // incoming Nyquist rows [CL][RY] (rank 0)
  C *scr = nq + Z::NQ + Z::NQS;
  unsigned long long *bars = reinterpret_cast<unsigned long long *>(scr + Z::SCR);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int) cluster.block_rank(), x = blockIdx.y, tid = threadIdx.x;
  const unsigned bar_ld = su32(&bars[0]), bar_in = su32(&bars[1]);
  if (tid == 0) {
    mbar_init(bar_ld, 1);
    mbar_init(bar_in, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(bar_ld, Z::RY * NZ * 4);
    mbar_expect_tx(bar_in, (Z::IN + (rank == 0 ? Z::NQ : 0)) * 8);
  }
  __syncthreads();
  if (tid < Z::RY) bulk_g2s(su32(a1 + tid * Z::PRW), f + ((size_t) x * NY + rank * Z::RY + tid) * NZ, NZ * 4, bar_ld);
  bool ok = mbar_wait(bar_ld, 0, fault);
  {  // z pass of this CTA's rows into the plane [kz][row]
    constexpr int N = Z::NZC, E = Shape<N>::E, TL = Shape<N>::TL, B = Shape<N>::B, LP = Shape<N>::LP;
    const int t = tid % TL, l = tid / TL;
#pragma unroll 1
    for (int rb = 0; rb < Z::RB; rb++) {
      const C *row = a1 + (rb * B + l) * Z::PRW;
      C v[E];
#pragma unroll
      for (int q = 0; q < E; q++) v[q] = row[t + TL * q];
      transform<N>(v, t, l, -1.f, twz, scr);
#pragma unroll
      for (int j = 0; j < E; j++) scr[sidx(l, final_pos<N>(t, j), LP)] = v[j];
      __syncthreads();
      // X[k] = (Z[k] + Z*[N-k]) / 2 - (i/2) w^k (Z[k] - Z*[N-k]),  k = 0..N
      constexpr int TOT = B * (N + 1), IT = (TOT + 255) / 256;
#pragma unroll
      for (int it = 0; it < IT; it++) {
        const int idx = tid + it * 256;
        if (idx < TOT) {
          const int ll = idx % B, k = idx / B;
          const C zk = scr[sidx(ll, k == N ? 0 : k, LP)], zm = scr[sidx(ll, k == 0 ? 0 : N - k, LP)];
          const C sum = make_float2(zk.x + zm.x, zk.y - zm.y), dif = make_float2(zk.x - zm.x, zk.y + zm.y);
          const C w = k == N ? make_float2(-1.f, 0.f) : __ldg(&tw2z[k]);
          const C tt = cmul(dif, w);
          plt[k * Z::RY + rb * B + ll] = make_float2(0.5f * (sum.x + tt.y), 0.5f * (sum.y - tt.x));
        }
      }
      __syncthreads();
    }
  }
  fence_proxy_async();
  cluster.sync();   // planes complete, staging areas free, barriers armed in every CTA
  if (tid < CL) {
    bulk_s2c(cl_addr(su32(a1 + rank * Z::KC * Z::RY), tid), su32(plt + tid * Z::KC * Z::RY), Z::KC * Z::RY * 8,
             cl_addr(bar_in, tid));
  } else if (tid == CL) {
    bulk_s2c(cl_addr(su32(nq + rank * Z::RY), 0), su32(plt + Z::NZC * Z::RY), Z::RY * 8, cl_addr(bar_in, 0));
  }
  if (tid <= CL) bulk_commit();
  ok = mbar_wait(bar_in, 0, fault) && ok;
  {  // y pass of this CTA's column lines
    constexpr int N = NY, E = Shape<N>::E, TL = Shape<N>::TL;
    const int t = tid % TL, l = tid / TL, c = rank * Z::KC + l;
    C v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int y = t + TL * q, sr = y / Z::RY, r = y % Z::RY;
      v[q] = c == 0 ? make_float2(a1[(sr * Z::KC) * Z::RY + r].x, nq[sr * Z::RY + r].x)
                    : a1[(sr * Z::KC + l) * Z::RY + r];
    }
    transform<N>(v, t, l, -1.f, twy, scr);
    if (c != 0 && ok) {
#pragma unroll
      for (int j = 0; j < E; j++) spec[((size_t) c * nx + x) * NY + final_pos<N>(t, j)] = v[j];
    }
    if (rank == 0) {   // CTA-uniform: separate the z = 0 and z = NZC columns
      if (l == 0) {
#pragma unroll
        for (int j = 0; j < E; j++) scr[final_pos<N>(t, j)] = v[j];
      }
      __syncthreads();
      if (l == 0 && ok) {
#pragma unroll
        for (int j = 0; j < E; j++) {
          const int k = final_pos<N>(t, j);
          const C zk = scr[k], zm = scr[(N - k) & (N - 1)];
          // S_0 = (Z[k] + Z*[-k]) / 2 ; S_NZC = (Z[k] - Z*[-k]) / (2i)
          spec[(size_t) x * NY + k] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
          spec[((size_t) Z::NZC * nx + x) * NY + k] = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
        }
      }
    }
  }
  if (tid <= CL) bulk_wait_read();   // own outgoing copies have read the plane
  cluster.sync();                    // no CTA leaves while a peer may still be copying into it
}

// inverse: spec[kz][x][y] -> real field f[x][y][z] * scale
template <int NY, int NZ, int CL>
__global__ void __launch_bounds__(256, 2) yz_c2r_kernel(const C *__restrict__ twz, const C *__restrict__ tw2z,
                                                        const C *__restrict__ twy, const C *__restrict__ spec,
                                                        float *__restrict__ f, float scale, int nx, int *fault) {
  typedef ZYPlane<NY, NZ, CL> Z;
  namespace cg = cooperative_groups;
  extern __shared__ __align__(128) unsigned char smraw[];
  C *plt = reinterpret_cast<C *>(smraw);   // incoming plane [NZC+2][RY]
  C *a1 = plt + Z::PLT;                    // staged columns [KC][PC], then outgoing [CL][KC][RY]
  C *nq = a1 + Z::A1;                      // outgoing Nyquist rows [CL][RY] (rank 0)
  C *nqs = nq + Z::NQ;                     // staged Nyquist column [NY] (rank 0)
  C *scr = nqs + Z::NQS;
  unsigned long long *bars = reinterpret_cast<unsigned long long *>(scr + Z::SCR);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int) cluster.block_rank(), x = blockIdx.y, tid = threadIdx.x;
  const unsigned bar_ld = su32(&bars[0]), bar_in = su32(&bars[1]);
  if (tid == 0) {
    mbar_init(bar_ld, 1);
    mbar_init(bar_in, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(bar_ld, (Z::KC + (rank == 0 ? 1 : 0)) * NY * 8);
    mbar_expect_tx(bar_in, (Z::IN + Z::RY) * 8);
  }
  __syncthreads();
  if (tid < Z::KC) {
    bulk_g2s(su32(a1 + tid * Z::PC), spec + ((size_t) (rank * Z::KC + tid) * nx + x) * NY, NY * 8, bar_ld);
  } else if (tid == Z::KC && rank == 0) {
    bulk_g2s(su32(nqs), spec + ((size_t) Z::NZC * nx + x) * NY, NY * 8, bar_ld);
  }
  bool ok = mbar_wait(bar_ld, 0, fault);
  {  // y pass of this CTA's column lines into the outgoing blocks
    constexpr int N = NY, E = Shape<N>::E, TL = Shape<N>::TL;
    const int t = tid % TL, l = tid / TL, c = rank * Z::KC + l;
    C v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int y = t + TL * q;
      if (c == 0) {   // X_0 + i X_NZC
        const C a = a1[y], b = nqs[y];
        v[q] = make_float2(a.x - b.y, a.y + b.x);
      } else {
        v[q] = a1[l * Z::PC + y];
      }
    }
    transform<N>(v, t, l, 1.f, twy, scr);   // its barriers order every staged read before the writes below
#pragma unroll
    for (int j = 0; j < E; j++) {
      const int y = final_pos<N>(t, j), sr = y / Z::RY, r = y % Z::RY;
      if (c == 0) {
        a1[(sr * Z::KC) * Z::RY + r] = make_float2(v[j].x, 0.f);
        nq[sr * Z::RY + r] = make_float2(v[j].y, 0.f);
      } else {
        a1[(sr * Z::KC + l) * Z::RY + r] = v[j];
      }
    }
  }
  fence_proxy_async();
  cluster.sync();   // outgoing blocks complete, barriers armed in every CTA
  if (tid < CL) {
    bulk_s2c(cl_addr(su32(plt + rank * Z::KC * Z::RY), tid), su32(a1 + tid * Z::KC * Z::RY), Z::KC * Z::RY * 8,
             cl_addr(bar_in, tid));
  } else if (tid < 2 * CL && rank == 0) {
    bulk_s2c(cl_addr(su32(plt + Z::NZC * Z::RY), tid - CL), su32(nq + (tid - CL) * Z::RY), Z::RY * 8,
             cl_addr(bar_in, tid - CL));
  }
  if (tid < 2 * CL) bulk_commit();
  ok = mbar_wait(bar_in, 0, fault) && ok;
  {  // c2r z pass of this CTA's rows (line-fast), rows stored through shared memory
    constexpr int N = Z::NZC, E = Shape<N>::E, TL = Shape<N>::TL, B = Shape<N>::B, LP = Shape<N>::LP;
    const int t = tid / B, l = tid % B;
#pragma unroll 1
    for (int rb = 0; rb < Z::RB; rb++) {
      const int r = rb * B + l;
      C v[E];
#pragma unroll
      for (int q = 0; q < E; q++) {
        // Z[k] = (X[k] + X*[N-k]) + i w^-k (X[k] - X*[N-k]),  w = exp(-2 pi i / 2N)
        const int e = t + TL * q;
        const C xk = plt[e * Z::RY + r], xm = plt[(N - e) * Z::RY + r];
        const C sum = make_float2(xk.x + xm.x, xk.y - xm.y), dif = make_float2(xk.x - xm.x, xk.y + xm.y);
        C w = __ldg(&tw2z[e]);
        w.y = -w.y;
        const C tt = cmul(dif, w);
        v[q] = make_float2(sum.x - tt.y, sum.y + tt.x);
      }
      transform<N>(v, t, l, 1.f, twz, scr);
#pragma unroll
      for (int j = 0; j < E; j++) scr[sidx(l, final_pos<N>(t, j), LP)] = v[j];
      __syncthreads();
      constexpr int IT = B * N / 256;
#pragma unroll
      for (int it = 0; it < IT; it++) {
        const int idx = tid + it * 256, e = idx % N, ll = idx / N;
        const C val = scr[sidx(ll, e, LP)];
        C *row = reinterpret_cast<C *>(f + ((size_t) x * NY + rank * Z::RY + rb * B + ll) * NZ);
        if (ok) row[e] = make_float2(val.x * scale, val.y * scale);
      }
      __syncthreads();
    }
  }
  if (tid < 2 * CL) bulk_wait_read();   // own outgoing copies have read their blocks
  cluster.sync();                        // no CTA leaves while a peer may still be copying into it
}

}  // namespace ff
}  // namespace dftgpu
