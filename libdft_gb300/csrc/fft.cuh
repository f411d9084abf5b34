// 3-D FFT building blocks for sm_103a (header-only templates).
//
// A 3-D transform of an [nx][ny][nz] grid runs as three line passes:
//   z pass  rows (x,y) are contiguous in real space; the output is written
//           transposed into the spectral layout [kz][x][y]
//   y pass  lines along y are contiguous in [kz][x][y]
//   x pass  pencils along x (stride ny); B consecutive y per CTA, so every
//           global access is a contiguous run of B complex values.
// Real fields use the half spectrum (kz = 0..nz/2) produced by packing a real
// row of length nz into nz/2 complex values (even + i odd), one FFT of length
// nz/2 and a twiddle post-processing step; the inverse does the reverse.
//
// The generic line pass (any 2^a 3^b 5^c length, and all of FP64) stages a
// tile of B lines in shared memory as [n][B+1] (element-major, padded), runs
// a Stockham autosort FFT (ping-pong buffers; radices {16, 15, 12, 10, 9, 8,
// 6, 5, 4, 3, 2} in FP32, {8, 5, 4, 3, 2} in FP64) and streams the tile back.  Loads and
// stores go through functors, which is where pointwise producers (|psi|^2,
// products of fields, phase factors) and consumers (accumulate into the
// potential) are fused.  Twiddles come from per-length tables computed in
// FP64 on the host and rounded once to the bulk precision.
#pragma once

#include <string.h>

#include <type_traits>

#include "common.cuh"
#include "fast_fft.cuh"

namespace dftgpu {

constexpr int FFT_THREADS = 256;
constexpr int FFT_MAX_STAGES = 16;
constexpr int FFT_MAX_N = 1024;      // grid dimension (3-D grids)
constexpr int FFT_MAX_LINE = 4096;   // z of a 1-D grid (nx = ny = 1); transform lengths up to this

template <typename T> struct FftPlan {
  int n;                       // transform length
  int nst;                     // number of stages
  int radix[FFT_MAX_STAGES];
  const typename cplx_t<T>::type *tw;   // tw[t] = exp(-2 pi i t / n), t < n
};

// Host: build (and cache) the plan for length n in precision T.
template <typename T> int get_plan(int n, FftPlan<T> *plan);

// ------------------------------------------------------------ butterflies
template <typename C, typename T>
__device__ __forceinline__ void dft2(C &a, C &b) { C t = a; a = t + b; b = t - b; }

// v * exp(s i 2 pi m / R) given (cos, sin) of 2 pi m / R
template <typename C, typename T> __device__ __forceinline__ C rot_cs(C v, T c, T sn, T s) {
  const T si = s * sn;
  C r; r.x = v.x * c - v.y * si; r.y = v.x * si + v.y * c;
  return r;
}

template <int R, typename C, typename T> __device__ __forceinline__ void small_dft(C *u, T s);

// Prime-factor radix R = R1 R2 (gcd 1, Good-Thomas): input n = (A1 n1 + A2 n2)
// mod R, output k = (K1 k1 + K2 k2) mod R with K1 = 1 (mod R1), 0 (mod R2)
// and K2 = 0 (mod R1), 1 (mod R2); no twiddles between the two layers.
template <int R1, int R2, int A1, int A2, int K1, int K2, typename C, typename T>
__device__ __forceinline__ void pfa_dft(C *u, T s) {
  constexpr int R = R1 * R2;
  C y[R2][R1];
#pragma unroll
  for (int n2 = 0; n2 < R2; n2++) {
#pragma unroll
    for (int n1 = 0; n1 < R1; n1++) y[n2][n1] = u[(A1 * n1 + A2 * n2) % R];
    small_dft<R1, C, T>(y[n2], s);
  }
#pragma unroll
  for (int k1 = 0; k1 < R1; k1++) {
    C z[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; n2++) z[n2] = y[n2][k1];
    small_dft<R2, C, T>(z, s);
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) u[(K1 * k1 + K2 * k2) % R] = z[k2];
  }
}

// R-point DFT in place, natural order; s = -1 forward, +1 inverse.
// Radices 2, 3, 4, 5, 8 directly; 16 and 9 as 4 x 4 and 3 x 3 with their
// internal twiddles; 6, 10, 12, 15 as prime-factor pairs.
template <int R, typename C, typename T>
__device__ __forceinline__ void small_dft(C *u, T s) {
  if constexpr (R == 2) {
    dft2<C, T>(u[0], u[1]);
  } else if constexpr (R == 3) {
    const T s3 = (T) 0.86602540378443864676;
    C a = u[0], b = u[1], c = u[2];
    C m = a - (b + c) * (T) 0.5;
    C d = (b - c) * s3;
    u[0] = a + b + c;
    u[1] = m + imul<C, T>(d, s);
    u[2] = m - imul<C, T>(d, s);
  } else if constexpr (R == 4) {
    C t0 = u[0] + u[2], t1 = u[0] - u[2], t2 = u[1] + u[3], t3 = u[1] - u[3];
    u[0] = t0 + t2;
    u[2] = t0 - t2;
    u[1] = t1 + imul<C, T>(t3, s);
    u[3] = t1 - imul<C, T>(t3, s);
  } else if constexpr (R == 5) {
    const T c1 = (T) 0.30901699437494742410, c2 = (T) -0.80901699437494742410;
    const T s1 = (T) 0.95105651629515357212, s2 = (T) 0.58778525229247312917;
    C a = u[0];
    C t1 = u[1] + u[4], t2 = u[2] + u[3], t3 = u[1] - u[4], t4 = u[2] - u[3];
    C m1 = a + t1 * c1 + t2 * c2;
    C m2 = a + t1 * c2 + t2 * c1;
    C n1 = t3 * s1 + t4 * s2;
    C n2 = t3 * s2 - t4 * s1;
    u[0] = a + t1 + t2;
    u[1] = m1 + imul<C, T>(n1, s);
    u[4] = m1 - imul<C, T>(n1, s);
    u[2] = m2 + imul<C, T>(n2, s);
    u[3] = m2 - imul<C, T>(n2, s);
  } else if constexpr (R == 8) {
    const T h = (T) 0.70710678118654752440;
    // radix-2 over stride 4, then two radix-4 with the W8 twiddles
    C a0 = u[0] + u[4], a1 = u[0] - u[4];
    C b0 = u[2] + u[6], b1 = u[2] - u[6];
    C c0 = u[1] + u[5], c1 = u[1] - u[5];
    C d0 = u[3] + u[7], d1 = u[3] - u[7];
    // even outputs: 4-point DFT of (a0, c0, b0, d0)
    C e0 = a0 + b0, e1 = a0 - b0, f0 = c0 + d0, f1 = c0 - d0;
    u[0] = e0 + f0;
    u[4] = e0 - f0;
    u[2] = e1 + imul<C, T>(f1, s);
    u[6] = e1 - imul<C, T>(f1, s);
    // odd outputs: 4-point DFT of (a1, W c1, W^2 b1, W^3 d1), W = exp(s i pi/4)
    C b1w = imul<C, T>(b1, s);                       // W^2 b1
    C c1w, d1w;
    c1w.x = h * (c1.x - s * c1.y); c1w.y = h * (c1.y + s * c1.x);      // W c1
    d1w.x = h * (-d1.x - s * d1.y); d1w.y = h * (-d1.y + s * d1.x);    // W^3 d1
    C g0 = a1 + b1w, g1 = a1 - b1w, k0 = c1w + d1w, k1 = c1w - d1w;
    u[1] = g0 + k0;
    u[5] = g0 - k0;
    u[3] = g1 + imul<C, T>(k1, s);
    u[7] = g1 - imul<C, T>(k1, s);
  } else if constexpr (R == 16) {
    // 4 x 4: 4-point DFTs over n1 of x[4 n1 + n2], twiddles W16^(n2 k1),
    // 4-point DFTs over n2; X[k1 + 4 k2]
    const T c1 = (T) 0.923879532511286756128, s1 = (T) 0.382683432365089771728, h = (T) 0.707106781186547524401;
    C y[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
#pragma unroll
      for (int n1 = 0; n1 < 4; n1++) y[n2][n1] = u[4 * n1 + n2];
      small_dft<4, C, T>(y[n2], s);
    }
    y[1][1] = rot_cs<C, T>(y[1][1], c1, s1, s); y[1][2] = rot_cs<C, T>(y[1][2], h, h, s);
    y[1][3] = rot_cs<C, T>(y[1][3], s1, c1, s);
    y[2][1] = rot_cs<C, T>(y[2][1], h, h, s); y[2][2] = imul<C, T>(y[2][2], s);
    y[2][3] = rot_cs<C, T>(y[2][3], -h, h, s);
    y[3][1] = rot_cs<C, T>(y[3][1], s1, c1, s); y[3][2] = rot_cs<C, T>(y[3][2], -h, h, s);
    y[3][3] = rot_cs<C, T>(y[3][3], -c1, -s1, s);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
      C z[4] = { y[0][k1], y[1][k1], y[2][k1], y[3][k1] };
      small_dft<4, C, T>(z, s);
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++) u[k1 + 4 * k2] = z[k2];
    }
  } else if constexpr (R == 9) {
    // 3 x 3 with twiddles W9^(n2 k1): (n2, k1) = (1,1), (1,2), (2,1): m = 1, 2; (2,2): m = 4
    const T ca = (T) 0.766044443118978035202, sa = (T) 0.642787609686539326323;
    const T cb = (T) 0.173648177666930348852, sb = (T) 0.984807753012208059367;
    const T cd = (T) -0.939692620785908384054, sd = (T) 0.342020143325668733044;
    C y[3][3];
#pragma unroll
    for (int n2 = 0; n2 < 3; n2++) {
#pragma unroll
      for (int n1 = 0; n1 < 3; n1++) y[n2][n1] = u[3 * n1 + n2];
      small_dft<3, C, T>(y[n2], s);
    }
    y[1][1] = rot_cs<C, T>(y[1][1], ca, sa, s); y[1][2] = rot_cs<C, T>(y[1][2], cb, sb, s);
    y[2][1] = rot_cs<C, T>(y[2][1], cb, sb, s); y[2][2] = rot_cs<C, T>(y[2][2], cd, sd, s);
#pragma unroll
    for (int k1 = 0; k1 < 3; k1++) {
      C z[3] = { y[0][k1], y[1][k1], y[2][k1] };
      small_dft<3, C, T>(z, s);
#pragma unroll
      for (int k2 = 0; k2 < 3; k2++) u[k1 + 3 * k2] = z[k2];
    }
  } else if constexpr (R == 6) {
    pfa_dft<2, 3, 3, 2, 3, 4, C, T>(u, s);
  } else if constexpr (R == 10) {
    pfa_dft<2, 5, 5, 2, 5, 6, C, T>(u, s);
  } else if constexpr (R == 12) {
    pfa_dft<4, 3, 3, 4, 9, 4, C, T>(u, s);
  } else if constexpr (R == 15) {
    pfa_dft<3, 5, 5, 3, 10, 6, C, T>(u, s);
  }
}

// One radix-R Stockham stage over a tile of B lines in [n][ldb] layout.
// FP32: thread t on line t % B, butterflies t / B + j blockDim.x / B; FP64:
// butterfly (line, index) = (idx % B, idx / B) for idx = t + j blockDim.x,
// twiddle index mod n.  Each form is the faster one for its precision: the
// first took the FP32 2.3.5 steps from 94 to 119 steps/s at 240^3, the
// second the FP64 256^3 step from 99 to 91 ms.
template <int R, typename T>
__device__ __forceinline__ void stockham_stage(const typename cplx_t<T>::type *__restrict__ in,
                                               typename cplx_t<T>::type *__restrict__ out,
                                               int n, int B, int ldb, int p,
                                               const typename cplx_t<T>::type *__restrict__ tw, T s) {
  typedef typename cplx_t<T>::type C;
  const int nR = n / R, twstep = n / (p * R);
  auto butterfly = [&](int l, int i, int k, int tq) {
    C u[R];
#pragma unroll
    for (int q = 0; q < R; q++) {
      C v = in[(i + q * nR) * ldb + l];
      if (q > 0 && k > 0) {
        C w = __ldg(&tw[tq ? (q * k * twstep) % n : q * k * twstep]);   // q k twstep < n
        w.y *= -s;   // tw holds exp(-i...); inverse (s=+1) uses the conjugate
        v = cmul(v, w);
      }
      u[q] = v;
    }
    small_dft<R, C, T>(u, s);
    const int j = (i - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; q++) out[(j + q * p) * ldb + l] = u[q];
  };
  if constexpr (sizeof(T) == 4) {
    const int l = threadIdx.x % B, istep = blockDim.x / B;
    for (int i = threadIdx.x / B; i < nR; i += istep) butterfly(l, i, i % p, 0);
  } else {
    for (int idx = threadIdx.x; idx < nR * B; idx += blockDim.x) {
      const int l = idx % B, i = idx / B;
      butterfly(l, i, i % p, 1);
    }
  }
}

// Runs all stages; returns the buffer holding the result (a or b).
template <typename T>
__device__ __forceinline__ typename cplx_t<T>::type *tile_fft(typename cplx_t<T>::type *a,
                                                              typename cplx_t<T>::type *b,
                                                              const FftPlan<T> &pl, int B, int ldb, T s) {
  typedef typename cplx_t<T>::type C;
  C *in = a, *out = b;
  int p = 1;
  for (int st = 0; st < pl.nst; st++) {
    const int R = pl.radix[st];
    // FP64 plans use radices up to 8 only (the larger ones would raise the
    // kernels' register count, and FP64 occupancy with it, for every length)
    switch (R) {
      case 8: stockham_stage<8, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
      case 4: stockham_stage<4, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
      case 2: stockham_stage<2, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
      case 3: stockham_stage<3, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
      case 5: stockham_stage<5, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
      default:
        if constexpr (sizeof(T) == 4) {
          switch (R) {
            case 16: stockham_stage<16, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
            case 6: stockham_stage<6, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
            case 9: stockham_stage<9, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
            case 10: stockham_stage<10, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
            case 12: stockham_stage<12, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
            default: stockham_stage<15, T>(in, out, pl.n, B, ldb, p, pl.tw, s); break;
          }
        }
        break;
    }
    __syncthreads();
    p *= R;
    C *t = in; in = out; out = t;
  }
  return in;
}

// ------------------------------------------------------------ line pass
enum { LINE_C2C = 0, LINE_R2C = 1, LINE_C2R = 2 };

template <typename T> struct LineArgs {
  FftPlan<T> plan;       // length of the complex FFT actually run
  int B;                 // lines per CTA (divides nb)
  int nb;                // extent of the fast line index b
  T sign;                // -1 forward, +1 inverse
  const typename cplx_t<T>::type *tw2;  // R2C/C2R: table of length 2n
  int e_fast;            // 1: the load functor's fast address index is the element
  int e_fast_store;      // 1: the store functor's fast address index is the element
};

// Element pitch of a tile of B lines: padded against bank conflicts between
// lines; a single line (long lines of 1-D grids) needs no padding.
__host__ __device__ __forceinline__ int tile_pitch(int B) { return B == 1 ? 1 : B + 1; }

// Visits the (line l, element e) pairs of this thread, e < n: element-fast
// (each line in turn, elements across the threads) or line-fast (thread t
// on line t % B, elements t / B + j blockDim.x / B); in batches of U whose
// fetches are all issued before the first put, so that U global loads per
// thread are in flight together.
// Element-fast mapping of the threads over a tile's (line, element) pairs:
// lines shorter than the CTA take several lines per pass (thread t on line
// t / n + j lpp, element t % n), so that no thread idles for n < blockDim.
struct EFastMap {
  int l0, lstep, e0, estep;
  __device__ __forceinline__ EFastMap(int n) {
    const int tid = threadIdx.x, nth = blockDim.x;
    if (n < nth) {
      lstep = nth / n;
      l0 = tid / n;
      e0 = tid - l0 * n;
      estep = n;
      if (l0 >= lstep) l0 = 1 << 30;   // the threads past lstep * n have no pair
    } else {
      l0 = 0; lstep = 1; e0 = tid; estep = nth;
    }
  }
};

template <int U, class Fetch, class Put>
__device__ __forceinline__ void batched_tile(int efast, int n, int B, Fetch fetch, Put put) {
  typedef decltype(fetch(0, 0)) R;
  const int tid = threadIdx.x, nth = blockDim.x;
  if (efast) {
    const EFastMap m(n);
    for (int e = m.e0; e < n; e += m.estep)
      for (int l0 = m.l0; l0 < B; l0 += U * m.lstep) {
        R r[U];
#pragma unroll
        for (int u = 0; u < U; u++)
          if (l0 + u * m.lstep < B) r[u] = fetch(l0 + u * m.lstep, e);
#pragma unroll
        for (int u = 0; u < U; u++)
          if (l0 + u * m.lstep < B) put(l0 + u * m.lstep, e, r[u]);
      }
  } else {
    const int l = tid % B, est = nth / B;
    for (int e0 = tid / B; e0 < n; e0 += U * est) {
      R r[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int e = e0 + u * est;
        if (e < n) r[u] = fetch(l, e);
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int e = e0 + u * est;
        if (e < n) put(l, e, r[u]);
      }
    }
  }
}

template <typename C> struct CPair { C a, b; };

// Line (a, b) = (blockIdx.y, blockIdx.x * B + l), element e.
//   LINE_C2C: X = FFT(ld(a,b,e)), st(a,b,e,X[e]) for e < n
//   LINE_R2C: z = ld(a,b,e) (packed even/odd reals), st(a,b,k,X[k]) for k <= n
//   LINE_C2R: X[k] = ld(a,b,k) for k <= n, st(a,b,e, (x[2e], x[2e+1]))
template <typename T, int MODE, class Ld, class St>
__global__ void __launch_bounds__(FFT_THREADS) line_fft_kernel(const LineArgs<T> args, const Ld ld, const St st) {
  typedef typename cplx_t<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = args.plan.n, B = args.B, ldb = tile_pitch(B);
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + n * ldb;
  const int a = blockIdx.y, b0 = blockIdx.x * B;
  // element-fast side: each line in turn, elements across the threads;
  // line-fast side: thread t on line t % B, elements t / B + j (blockDim / B)
  const int tid = threadIdx.x, nth = blockDim.x, lt = tid % B, et0 = tid / B, est = nth / B;
  (void) lt; (void) et0; (void) est;
  // the last tile may be partial (B need not divide nb): its missing lines
  // are transformed as zeros and not stored
  const int nb = args.nb;
  const C zero = mk<T>((T) 0, (T) 0);

  // ---- load
  if (MODE == LINE_C2R) {
    // Z[k] = (X[k] + X*[n-k]) + i w^{-k} (X[k] - X*[n-k]),  w = exp(-2 pi i / 2n)
    batched_tile<sizeof(T) == 4 ? 4 : 1>(args.e_fast, n, B,
        [&](int l, int k) {
          if (b0 + l >= nb) return CPair<C>{ zero, zero };
          return CPair<C>{ ld(a, b0 + l, k), ld(a, b0 + l, n - k) };
        },
        [&](int l, int k, CPair<C> x) {
          C xk = x.a, xm = x.b;
          if (k == 0) { xk.y = (T) 0; xm.y = (T) 0; }   // DC / Nyquist are real
          C sum = xk + conjc(xm), dif = xk - conjc(xm);
          C w = __ldg(&args.tw2[k]);
          w.y = -w.y;                                    // w^{-k}
          C t = cmul(dif, w);
          C z; z.x = sum.x - t.y; z.y = sum.y + t.x;     // sum + i t
          buf0[k * ldb + l] = z;
        });
  } else {
    batched_tile<sizeof(T) == 4 ? 8 : 1>(args.e_fast, n, B, [&](int l, int e) { return b0 + l < nb ? ld(a, b0 + l, e) : zero; },
                                         [&](int l, int e, C v) { buf0[e * ldb + l] = v; });
  }
  __syncthreads();

  C *res = tile_fft<T>(buf0, buf1, args.plan, B, ldb, args.sign);

  // ---- store
  if (MODE == LINE_R2C) {
    // X[k] = (Z[k] + Z*[n-k]) / 2 - (i/2) w^k (Z[k] - Z*[n-k]),  k = 0..n
    auto one = [&](int k, int l) {
      C zk = res[(k == n ? 0 : k) * ldb + l];
      C zm = res[(k == 0 ? 0 : n - k) * ldb + l];
      C sum = zk + conjc(zm), dif = zk - conjc(zm);
      C w = __ldg(&args.tw2[k == n ? 0 : k]);
      if (k == n) { w.x = (T) -1; w.y = (T) 0; }
      C t = cmul(dif, w);
      C x; x.x = (T) 0.5 * (sum.x + t.y); x.y = (T) 0.5 * (sum.y - t.x);   // (sum - i t)/2
      if (b0 + l < nb) st(a, b0 + l, k, x);
    };
    if (args.e_fast_store) {
      const EFastMap m(n + 1);
      for (int k = m.e0; k <= n; k += m.estep)
        for (int l = m.l0; l < B; l += m.lstep) one(k, l);
    } else {
      for (int k = et0; k <= n; k += est) one(k, lt);
    }
  } else {
    if (args.e_fast_store) {
      const EFastMap m(n);
      for (int e = m.e0; e < n; e += m.estep)
        for (int l = m.l0; l < B; l += m.lstep)
          if (b0 + l < nb) st(a, b0 + l, e, res[e * ldb + l]);
    } else {
      if (b0 + lt < nb)
        for (int e = et0; e < n; e += est) st(a, b0 + lt, e, res[e * ldb + lt]);
    }
  }
}

// ------------------------------------------------------------ x-pencil convolution
// Kernel spectra are stored for the non-negative octant only, in layout
// [kz][kx][ky] with extents (nz/2+1, nx/2+1, ny/2+1), already multiplied by the
// centring phase (-1)^(kx+ky+kz) and the convolution normalisation step^3/N.
enum { KER_EVEN = 0, KER_ODD_X = 1, KER_ODD_Y = 2, KER_ODD_Z = 3, KER_UNIT = 4 };

constexpr int XC_MAX_IN = 4;
constexpr int XC_MAX_OUT = 8;
constexpr int XC_MAX_TERMS = 16;

template <typename T> struct XTerm {
  const T *ker;   // octant spectrum (real part for KER_EVEN, imaginary part for KER_ODD_*)
  int kind;
  int in;         // input index
  T coef;
};

template <typename T> struct XOut {
  typename cplx_t<T>::type *dst;   // spectral buffer [kz][x][y]
  int t0, nt;                      // terms [t0, t0+nt)
  int accumulate;                  // 1: dst += result
};

template <typename T> struct XConvArgs {
  FftPlan<T> plan;                 // length nx
  int B, nx, ny, nkz;              // tile width, grid dims, number of kz planes
  int kxh, kyh;                    // octant extents nx/2+1, ny/2+1
  int nin, nout;
  const typename cplx_t<T>::type *src[XC_MAX_IN];
  XOut<T> out[XC_MAX_OUT];
  XTerm<T> term[XC_MAX_TERMS];
};

template <typename T>
__device__ __forceinline__ typename cplx_t<T>::type apply_kernel(const XTerm<T> &t, typename cplx_t<T>::type v,
                                                                 int kx, int ky, int kz, const XConvArgs<T> &A) {
  typedef typename cplx_t<T>::type C;
  if (t.kind == KER_UNIT) return v * t.coef;
  const int ix = kx <= A.nx / 2 ? kx : A.nx - kx;
  const int iy = ky <= A.ny / 2 ? ky : A.ny - ky;
  const T kv = __ldg(&t.ker[((size_t) kz * A.kxh + ix) * A.kyh + iy]) * t.coef;
  if (t.kind == KER_EVEN) return v * kv;
  T sgn = (T) 1;
  if (t.kind == KER_ODD_X && kx > A.nx / 2) sgn = (T) -1;
  if (t.kind == KER_ODD_Y && ky > A.ny / 2) sgn = (T) -1;
  C r; r.x = -sgn * kv * v.y; r.y = sgn * kv * v.x;   // (i sgn kv) v
  return r;
}

// grid (ny / B, nkz); one CTA = B consecutive y pencils of one kz plane.
// One input: its spectrum is computed once into a tile and every output is
// formed from it (3 tiles).  Several inputs: the outputs one after the other,
// each summing its terms into an accumulator tile, the input of each term
// transformed when the term is reached (3 tiles instead of inputs + 2, so a
// CTA holds more pencils; the transforms are the same in number when each
// input feeds one output).
template <typename T>
__global__ void __launch_bounds__(FFT_THREADS) xconv_kernel(const XConvArgs<T> A) {
  typedef typename cplx_t<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = A.plan.n, B = A.B, ldb = tile_pitch(B), tile = n * ldb;   // as choose_tile
  C *bufs = reinterpret_cast<C *>(smem_raw);
  const int kz = blockIdx.y, y0 = blockIdx.x * B;
  const size_t plane = (size_t) A.nx * A.ny;
  const int l = threadIdx.x % B, e0 = threadIdx.x / B, est = blockDim.x / B;   // thread: one pencil
  constexpr int LU = sizeof(T) == 4 ? 8 : 1;   // loads in flight per thread (FP32)

  // forward transform of input `in` into tile `tin` (scratch `tsc`); returns the result's tile
  auto forward = [&](int in, C *tin, C *tsc) -> C * {
    const C *src = A.src[in] + kz * plane + y0;
    batched_tile<LU>(0, n, B, [&](int ll, int e) { return src[(size_t) e * A.ny + ll]; },
                     [&](int ll, int e, C v) { tin[e * ldb + ll] = v; });
    __syncthreads();
    return tile_fft<T>(tin, tsc, A.plan, B, ldb, (T) -1);
  };
  // inverse transform of tile `acc` (scratch `tsc`) and the store of output `out`
  auto emit = [&](const XOut<T> &out, C *acc, C *tsc) {
    C *r = tile_fft<T>(acc, tsc, A.plan, B, ldb, (T) 1);
    C *dst = out.dst + kz * plane + y0;
    if (out.accumulate) {
      batched_tile<LU>(0, n, B, [&](int ll, int e) { return dst[(size_t) e * A.ny + ll]; },
                       [&](int ll, int e, C v) { dst[(size_t) e * A.ny + ll] = v + r[e * ldb + ll]; });
    } else {
      for (int e = e0; e < n; e += est) dst[(size_t) e * A.ny + l] = r[e * ldb + l];
    }
    __syncthreads();
  };

  if (A.nin == 1) {
    C *X = bufs, *scr0 = bufs + tile, *scr1 = scr0 + tile;
    C *r = forward(0, X, scr0);
    if (r != X) {   // an odd number of stages ends in the scratch tile
      for (int idx = threadIdx.x; idx < tile; idx += blockDim.x) X[idx] = r[idx];
      __syncthreads();
    }
    for (int o = 0; o < A.nout; o++) {
      const XOut<T> &out = A.out[o];
      constexpr int U = sizeof(T) == 4 ? 4 : 1;   // elements per batch (FP32): their kernel values loaded together
      for (int eb = e0; eb < n; eb += U * est) {
        C acc[U];
#pragma unroll
        for (int u = 0; u < U; u++) acc[u] = mk<T>((T) 0, (T) 0);
        for (int t = out.t0; t < out.t0 + out.nt; t++) {
          const XTerm<T> &tm = A.term[t];
#pragma unroll
          for (int u = 0; u < U; u++) {
            const int e = eb + u * est;
            if (e < n) acc[u] = acc[u] + apply_kernel<T>(tm, X[e * ldb + l], e, y0 + l, kz, A);
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = eb + u * est;
          if (e < n) scr0[e * ldb + l] = acc[u];
        }
      }
      __syncthreads();
      emit(out, scr0, scr1);
    }
    return;
  }

  C *X = bufs, *Y = bufs + tile, *ACC = bufs + 2 * tile;
  for (int o = 0; o < A.nout; o++) {
    const XOut<T> &out = A.out[o];
    if (out.nt == 0) {   // no term: a zero output (added: no change)
      for (int e = e0; e < n; e += est) ACC[e * ldb + l] = mk<T>((T) 0, (T) 0);
      __syncthreads();
    }
    for (int t = out.t0; t < out.t0 + out.nt; t++) {
      const XTerm<T> &tm = A.term[t];
      const C *r = forward(tm.in, X, Y);
      for (int e = e0; e < n; e += est) {   // each thread its own elements: no barrier before the sum
        const C v = apply_kernel<T>(tm, r[e * ldb + l], e, y0 + l, kz, A);
        ACC[e * ldb + l] = t == out.t0 ? v : ACC[e * ldb + l] + v;
      }
      __syncthreads();   // the tiles X / Y are free for the next term's input
    }
    emit(out, ACC, X);
  }
}

// ------------------------------------------------------------ kinetic x pass
// psi(k) *= exp(-i hbar |k - k0|^2 dt / 2m) / N in the middle of an x-pencil
// FFT pair; k0 is the moving-background momentum of the wave function's grid.
// The factor separates, exp(c |k - k0|^2) = (1 + fx(kx)) (1 + fyz(ky, kz)),
// so each CTA tabulates fx for its line length and fyz for its lines (two
// transcendental evaluations per thread instead of one per element) and
// applies psi + psi ((1 + fx)(1 + fyz) - 1), which keeps |factor| = 1 to the
// rounding of the exponent in real time.  With cn set the factor is the
// Crank-Nicolson one of the finite-difference kinetic operator, one per axis
// (cn_m1), and separates the same way: (1 + fx)(1 + fy)(1 + fz).
template <typename T> struct KinArgs {
  FftPlan<T> plan;
  int B, nx, ny, nz;
  double2 cdt;          // -i dt / (2 m): factor = exp(cdt |k - k0|^2)
  double inv_n;
  double dkx, dky, dkz; // 2 pi / (n step)
  double kx0, ky0, kz0; // moving-background momentum
  double h;             // grid step
  int cn;               // Crank-Nicolson factors instead of exp(cdt |k - k0|^2)
  typename cplx_t<T>::type *data;
};

template <typename T>
inline void kin_args(KinArgs<T> &K, int nx, int ny, int nz, double step, double2 cdt, double kx0, double ky0,
                     double kz0, typename cplx_t<T>::type *data) {
  K.nx = nx; K.ny = ny; K.nz = nz;
  K.data = data;
  K.cdt = cdt;
  K.inv_n = 1.0 / ((double) nx * ny * nz);
  K.dkx = 2.0 * M_PI / (nx * step);
  K.dky = 2.0 * M_PI / (ny * step);
  K.dkz = 2.0 * M_PI / (nz * step);
  K.kx0 = kx0; K.ky0 = ky0; K.kz0 = kz0;
  K.h = step;
  K.cn = 0;
}

// shared memory of the generic kinetic kernel: two tiles + the factor tables
inline size_t kin_smem(int n, int B, size_t cplx_bytes) {
  return 2 * (size_t) n * (B + 1) * cplx_bytes + (size_t) (n + B) * cplx_bytes;
}

__device__ __forceinline__ double kfreq(int i, int n, double dk) {
  return (double) (i < (n + 1) / 2 ? i : i - n) * dk;
}

template <typename T>
__global__ void __launch_bounds__(FFT_THREADS) xkinetic_kernel(const KinArgs<T> A) {
  typedef typename cplx_t<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = A.plan.n, B = A.B, ldb = B + 1, tile = n * ldb;
  C *s0 = reinterpret_cast<C *>(smem_raw), *s1 = s0 + tile, *fx = s1 + tile, *fyz = fx + n;
  const int kz = blockIdx.y, y0 = blockIdx.x * B;
  const size_t plane = (size_t) A.nx * A.ny;
  C *base = A.data + kz * plane + y0;
  const C c = mk<T>((T) A.cdt.x, (T) A.cdt.y);
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const double k = kfreq(e, A.nx, A.dkx) - A.kx0, q = k * k;
    fx[e] = A.cn ? cn_m1(c, (T) k, (T) A.h) : cexpm1(mk<T>((T) (A.cdt.x * q), (T) (A.cdt.y * q)));
  }
  const double kzv = kfreq(kz, A.nz, A.dkz) - A.kz0;
  for (int l = threadIdx.x; l < B; l += blockDim.x) {
    const double k = kfreq(y0 + l, A.ny, A.dky) - A.ky0, q = k * k + kzv * kzv;
    fyz[l] = A.cn ? cprod1p(cn_m1(c, (T) k, (T) A.h), cn_m1(c, (T) kzv, (T) A.h))
                  : cexpm1(mk<T>((T) (A.cdt.x * q), (T) (A.cdt.y * q)));
  }
  for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) {
    const int l = idx % B, e = idx / B;
    s0[e * ldb + l] = base[(size_t) e * A.ny + l];
  }
  __syncthreads();
  C *r = tile_fft<T>(s0, s1, A.plan, B, ldb, (T) -1);
  for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) {
    const int l = idx % B, e = idx / B;
    const C a = r[e * ldb + l];
    r[e * ldb + l] = mul_1p(mk<T>(a.x * (T) A.inv_n, a.y * (T) A.inv_n), cprod1p(fx[e], fyz[l]));
  }
  __syncthreads();
  C *other = (r == s0) ? s1 : s0;
  C *r2 = tile_fft<T>(r, other, A.plan, B, ldb, (T) 1);
  for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) {
    const int l = idx % B, e = idx / B;
    base[(size_t) e * A.ny + l] = r2[e * ldb + l];
  }
}

// ------------------------------------------------------------ launch helpers
// partial: B need not divide nb (the kernel skips the missing lines of the last tile)
int choose_tile(int n, int nb, size_t cplx_bytes, int nbufs, int *B, size_t *smem, bool partial = false);

// "Opt-in shared memory already requested" flag per kernel instantiation.
// It lives in an anonymous namespace so that every translation unit keeps its
// own flag: without relocatable device code each translation unit registers
// its own copy of a template kernel, and the attribute must be set on each.
namespace {
template <class Kernel> struct SmemOptIn { static bool done; };
template <class Kernel> bool SmemOptIn<Kernel>::done = false;
}  // namespace

bool generic_fft_only();   // DFTGPU_GENERIC_FFT=1 disables the register kernels
bool prefetch_ahead_on();  // DFTGPU_PREFETCH_AHEAD=0 disables the one-wave-ahead L2 prefetch
bool factorised_propagation();  // DFTGPU_FACTORISED_PROP=1: FP32 propagation by one kinetic pass per axis
bool march_on();  // DFTGPU_MARCH=0: the second OT pointwise pass one CTA per row instead of x-marching

// CTAs of a 256-thread kernel resident on the whole GPU at once (the distance
// of the line kernels' one-wave-ahead prefetch); 0 when prefetching is off.
template <class K> int resident_ctas(K kernel) {
  static int n = -1;
  if (n < 0) {
    int per_sm = 0;
    if (!prefetch_ahead_on() || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess)
      per_sm = 0;
    n = per_sm * rt().num_sms;
  }
  return n;
}

// TMA for the transposed side of the z passes (DFTGPU_TMA=0 turns it off)
bool tma_on();
void tma_disable();
// Tensor map over a spectral buffer [rows][nx][ny] of complex FP32 values
// (8-byte elements) with boxes {16 y, 1 x, rows} and the 128-byte swizzle.
int encode_spec_map(CUtensorMap *map, const void *spec, int nx, int ny, int rows);
// Device flag set by a kernel whose bounded wait on an asynchronous copy gave
// up (read and cleared by dftgpu_synchronize and the device-to-host copies).
int *async_fault_flag();

// Functors of the spectral layout [kz][x][y] used by z passes (kSpecZ: members
// spec, nx, ny), whose staged side may move by TMA.
template <class F> __host__ __device__ constexpr auto spec_z_of(int) -> decltype(F::kSpecZ, bool()) { return F::kSpecZ; }
template <class F> __host__ __device__ constexpr bool spec_z_of(long) { return false; }

template <int N, int MODE, int MAP, int LDS, int STS, int TMA, class Ld, class St>
void launch_line_kernel(int na, int nb, const float2 *tw, const float2 *tw2, float sign, const Ld &ld, const St &st,
                        const ff::TmaMaps &tm, int *fault) {
  constexpr int B = ff::Shape<N>::B;
  if constexpr (LDS == 0 && ff::split_of<Ld>(0)) {
    auto k = ff::line_kernel_split<N, MODE, MAP, LDS, STS, TMA, Ld, St>;
    k<<<dim3(nb / B, na), 256, 0, rt().stream>>>(tw, tw2, sign, ld, st, resident_ctas(k), tm, fault);
  } else if constexpr (STS == 0 && ff::bounded_store_of<St>(0)) {
    auto k = ff::line_kernel_stsplit<N, MODE, MAP, LDS, STS, TMA, Ld, St>;
    k<<<dim3(nb / B, na), 256, 0, rt().stream>>>(tw, tw2, sign, ld, st, resident_ctas(k), tm, fault);
  } else {
    auto k = ff::line_kernel<N, MODE, MAP, LDS, STS, TMA, Ld, St>;
    k<<<dim3(nb / B, na), 256, 0, rt().stream>>>(tw, tw2, sign, ld, st, resident_ctas(k), tm, fault);
  }
}

// FP32 power-of-two lengths: register-resident kernel.  EF / EFS: the fast
// address index of the load / store side is the element (1) or the line (0).
// Returns -1 when the shape does not fit the kernel (caller falls back).
template <int N, int MODE, int EF, int EFS, class Ld, class St>
int launch_fast_lines(int na, int nb, float sign, const Ld &ld, const St &st) {
  static_assert(MODE != LINE_R2C || (EF == 1 && EFS == 0), "r2c z pass: element-fast load, line-fast store");
  static_assert(MODE != LINE_C2R || (EF == 0 && EFS == 1), "c2r z pass: line-fast load, element-fast store");
  constexpr int MAP = (EF == 0 && EFS == 0) ? ff::MAP_L : ff::MAP_E;
  constexpr int LDS = (EF == 0 && EFS == 1) ? 1 : 0;
  constexpr int STS = (EF == 1 && EFS == 0) ? 1 : 0;
  constexpr int B = ff::Shape<N>::B;
  if (nb % B) return -1;
  FftPlan<float> p1, p2;
  DFT_TRY(get_plan<float>(N, &p1));
  p2.tw = nullptr;
  if (MODE != LINE_C2C) DFT_TRY(get_plan<float>(2 * N, &p2));
  ff::TmaMaps tm;
  memset(&tm, 0, sizeof(tm));
  // TMA on the spectral side of the z passes: loads of the c2r / c2c passes,
  // stores of the c2c passes.  The r2c passes keep their store loop: with a
  // TMA store the 256^3 step ran at the same rate (235.4 against 236.6 steps/s).
  constexpr bool TMA_LD = LDS && spec_z_of<Ld>(0) && ff::TmaTile<N, MODE>::OK;
  constexpr bool TMA_ST = STS && MODE == LINE_C2C && spec_z_of<St>(0) && ff::TmaTile<N, MODE>::OK;
  if constexpr (TMA_LD || TMA_ST) {
    if (tma_on()) {
      constexpr int ROWS = ff::TmaTile<N, MODE>::ROWS;
      int rc = DFTGPU_OK;
      if constexpr (TMA_LD) rc = encode_spec_map(&tm.load, ld.spec, ld.nx, ld.ny, ROWS);
      if constexpr (TMA_ST) if (!rc) rc = encode_spec_map(&tm.store, st.spec, st.nx, st.ny, ROWS);
      int *fault = rc ? nullptr : async_fault_flag();
      if (fault) {
        launch_line_kernel<N, MODE, MAP, LDS, STS, 1>(na, nb, p1.tw, p2.tw, sign, ld, st, tm, fault);
        DFT_CHECK_LAUNCH();
        return DFTGPU_OK;
      }
      tma_disable();   // no tensor maps here: the load / store loops from now on
      g_last_error = 0;   // the encode failure is not the caller's error
    }
  }
  launch_line_kernel<N, MODE, MAP, LDS, STS, 0>(na, nb, p1.tw, p2.tw, sign, ld, st, tm, nullptr);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// One factorised kinetic pass (ff::line_kin_kernel) over na x nb lines of
// length N: line-fast (MAP_L) when the lines are strided with consecutive
// lines adjacent, element-fast (MAP_E) for contiguous rows.  Returns -1 when
// the shape does not fit (nb not a multiple of the CTA's line count).
template <int N, int MAP, class Ld, class St>
int launch_kin_lines(int na, int nb, float2 cdt, float inv_n, float dk, float k0, const Ld &ld, const St &st) {
  constexpr int B = ff::Shape<N>::B;
  if (nb % B) return -1;
  FftPlan<float> p;
  DFT_TRY(get_plan<float>(N, &p));
  // two transforms and the factor table: rows bounded to 80 registers (3 CTAs
  // per SM); strided lines keep a runtime-stride address per element and get
  // 128 (2 CTAs per SM) so that they do not spill
  auto k = ff::line_kin_kernel<N, MAP, (MAP == ff::MAP_E || !ff::bounded_store_of<St>(0)) ? 3 : 2, Ld, St>;
  k<<<dim3(nb / B, na), 256, 0, rt().stream>>>(p.tw, cdt, inv_n, dk, k0, ld, st, resident_ctas(k));
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

template <int MAP, class Ld, class St>
int launch_kin_pass(int n, int na, int nb, float2 cdt, float dk, float k0, const Ld &ld, const St &st, const char *name,
                    double bytes) {
  if (generic_fft_only()) return -1;
  if (n != 64 && n != 128 && n != 256 && n != 512) return -1;
  ProfScope prof(name, bytes);
  const float inv_n = 1.f / (float) n;
  switch (n) {
    case 64: return launch_kin_lines<64, MAP>(na, nb, cdt, inv_n, dk, k0, ld, st);
    case 128: return launch_kin_lines<128, MAP>(na, nb, cdt, inv_n, dk, k0, ld, st);
    case 256: return launch_kin_lines<256, MAP>(na, nb, cdt, inv_n, dk, k0, ld, st);
    default: return launch_kin_lines<512, MAP>(na, nb, cdt, inv_n, dk, k0, ld, st);
  }
}

// extra_bytes: algorithmic bytes read / written by the fused functors beyond
// the transformed line data itself (e.g. the potential read by a phase load).
template <typename T, int MODE, int EF, int EFS, class Ld, class St>
int launch_lines(int n_fft, int na, int nb, T sign, const Ld &ld, const St &st, double extra_bytes = 0.0) {
  typedef typename cplx_t<T>::type C;
  const double lines = (double) na * nb;
  const double data = MODE == LINE_C2C ? 2.0 * n_fft : (2.0 * n_fft + 1.0);
  ProfScope prof(MODE == LINE_C2C ? "fft_line_c2c" : (MODE == LINE_R2C ? "fft_line_r2c" : "fft_line_c2r"),
                 lines * data * sizeof(C) + extra_bytes);
  if constexpr (std::is_same<T, float>::value) {
    if (!generic_fft_only()) {
      int rc = -1;
      switch (n_fft) {
        case 64: rc = launch_fast_lines<64, MODE, EF, EFS>(na, nb, sign, ld, st); break;
        case 128: rc = launch_fast_lines<128, MODE, EF, EFS>(na, nb, sign, ld, st); break;
        case 256: rc = launch_fast_lines<256, MODE, EF, EFS>(na, nb, sign, ld, st); break;
        case 512: rc = launch_fast_lines<512, MODE, EF, EFS>(na, nb, sign, ld, st); break;
        case 96: rc = launch_fast_lines<96, MODE, EF, EFS>(na, nb, sign, ld, st); break;
        case 192: rc = launch_fast_lines<192, MODE, EF, EFS>(na, nb, sign, ld, st); break;
        case 384: rc = launch_fast_lines<384, MODE, EF, EFS>(na, nb, sign, ld, st); break;
        default: break;
      }
      if (rc >= 0) return rc;
    }
  }
  LineArgs<T> args;
  DFT_TRY(get_plan<T>(n_fft, &args.plan));
  args.sign = sign;
  args.nb = nb;
  args.e_fast = EF;
  args.e_fast_store = EFS;
  args.tw2 = nullptr;
  if (MODE != LINE_C2C) {
    FftPlan<T> p2;
    DFT_TRY(get_plan<T>(2 * n_fft, &p2));
    args.tw2 = p2.tw;
  }
  int B; size_t smem;
  DFT_TRY(choose_tile(n_fft, nb, sizeof(C), 2, &B, &smem, true));
  args.B = B;
  auto kfn = line_fft_kernel<T, MODE, Ld, St>;
  typedef SmemOptIn<LineArgs<T> (*)(Ld *, St *, int (*)[MODE + 1])> Flag;
  if (smem > 48 * 1024 && !Flag::done) {
    DFT_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) rt().max_smem_optin));
    Flag::done = true;
  }
  if (smem > rt().max_smem_optin) {
    set_error(DFTGPU_ERR_SIZE, "line FFT n=%d needs %zu bytes of shared memory", n_fft, smem);
    return DFTGPU_ERR_SIZE;
  }
  dim3 grid((nb + B - 1) / B, na);
  kfn<<<grid, FFT_THREADS, smem, rt().stream>>>(args, ld, st);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

template <typename T> int launch_xconv(XConvArgs<T> &A);
template <typename T> int launch_xkinetic(KinArgs<T> &A);

// ------------------------------------------------------------ fused z + y passes
// The fused z + y plane passes (cluster kernels, fast_fft.cuh) are selected
// with DFTGPU_FUSED_ZY=1; by default the separate passes run (measured
// faster at 256^3: 60-64 us against 73-83 us per real transform).
bool fused_zy_off();

}  // namespace dftgpu
