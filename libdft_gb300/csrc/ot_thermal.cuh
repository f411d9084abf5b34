// Ideal Bose gas term of the thermal OT models (DFT_OT_T400MK ... T3000MK).
//
// libdft adds it through libgrid's grid_func6a / 6b (src/ot.c:402-407,
// 804-809; src/ot-energy.c:101-105), which are absent; the form is libdft's
// own host one (src/common.c:253-529, used by its bulk relations
// src/helium-ot-bulk.c:30-31, 54-55):
//   lambda^3 = (2 pi hbar^2 / (m kB T))^(3/2),  x = rho lambda^3,
//   g_s(z) = sum_{k=1}^{256} z^k / k^s,  z: g_{3/2}(z) = x  (z = 1 for x >= g_{3/2}(1)),
//   f(rho)  = c4 kB T (rho ln z - g_{5/2}(z) / lambda^3),
//   mu(rho) = c4 kB T (ln z + x / g_{1/2}(z) - g_{3/2}(z) / g_{1/2}(z)),
//             -c4 kB T g_{3/2}(1) / lambda^3 for x >= g_{3/2}(1).
// libdft finds z by golden-section search to a bracket of 1e-6; here z is the
// root of the same truncated series to the working precision (safeguarded
// Newton steps, dg_{3/2}/dz = g_{1/2}(z) / z), so the two agree within the
// resolution of that search.  Below it the search cannot go: its z for a
// vanishing density is zmin (about 2e-6, the last bracket's midpoint), and so
// z is taken no smaller than zmin here (instead of ln z -> -inf as rho -> 0).
// The series stop once a term no longer changes the sum.
#pragma once

#include "common.cuh"

namespace dftgpu {

constexpr int BOSE_TERMS = 256;

template <typename T> struct BoseGas {
  T l3, kt, c4, g32_1, zmin;   // lambda^3, kB T, c4, g_{3/2}(1) of the truncated series, z floor

  // g_{1/2}, g_{3/2} (and g_{5/2} when asked) at z in [0, 1]
  __device__ __forceinline__ void series(T z, T &g12, T &g32, T *g52) const {
    T zk = (T) 1, a = 0, b = 0, c = 0;
    for (int k = 1; k <= BOSE_TERMS; k++) {
      zk *= z;
      const T kk = (T) k, ik = (T) 1 / kk, ta = zk * rsqrt(kk);   // z^k k^(-1/2)
      if (ta <= a * (T) 1e-17 && k > 1) break;   // every later term is smaller still
      a += ta;
      b += ta * ik;                                // z^k k^(-3/2)
      if (g52) c += ta * ik * ik;                  // z^k k^(-5/2)
    }
    g12 = a;
    g32 = b;
    if (g52) *g52 = c;
  }

  __device__ __forceinline__ T root(T x) const {   // g_{3/2}(z) = x, x < g_{3/2}(1); z >= zmin
    T g12m, g32m;
    series(zmin, g12m, g32m, nullptr);
    if (x <= g32m) return zmin;
    T lo = zmin, hi = 1, z = x < (T) 0.5 ? x : (T) 0.5;
    for (int it = 0; it < 100; it++) {
      T g12, g32;
      series(z, g12, g32, nullptr);
      const T f = g32 - x;
      if (f > 0) hi = z; else lo = z;
      T zn = z - f * z / g12;
      if (!(zn > lo && zn < hi)) zn = (T) 0.5 * (lo + hi);
      const T dz = zn - z;
      z = zn;
      if (fabs(dz) <= (T) 4 * (sizeof(T) == 4 ? (T) 1.2e-7 : (T) 2.3e-16) * z) break;
    }
    return z;
  }

  __device__ __forceinline__ T dEdRho(T rho) const {
    const T x = rho * l3;
    if (x >= g32_1) return -c4 * kt * g32_1 / l3;
    const T z = root(x);
    T g12, g32;
    series(z, g12, g32, nullptr);
    return c4 * kt * (log(z) + x / g12 - g32 / g12);
  }

  __device__ __forceinline__ T energy(T rho) const {
    const T x = rho * l3;
    T z = 1, g12, g32, g52;
    if (x < g32_1) z = root(x);
    series(z, g12, g32, &g52);
    return c4 * kt * (rho * log(z) - g52 / l3);
  }
};

// host (api.cu): whether the potential / energy density carry the term
// (src/ot.c:402, src/ot-energy.c:101); lambda^3; g_{3/2}(1) of the truncated
// series; the search's z for a vanishing density
bool bose_model(const dft_ot_functional *otf);
double bose_lwl3(double mass, double temp);
double bose_g32_one();
double bose_zmin();

template <typename T> inline BoseGas<T> bose_par(const dft_ot_functional *otf) {
  return BoseGas<T>{(T) bose_lwl3(otf->mass, otf->temp), (T) (GRID_AUKB * otf->temp), (T) otf->c4,
                    (T) bose_g32_one(), (T) bose_zmin()};
}

}  // namespace dftgpu
