// Work-buffer helpers shared by the OT potential (ot.cu) and its adjoint
// (adjoint.cu): real-field / half-spectrum slots, forward and inverse real
// transforms, and builders for the x-pencil convolution arguments.
#pragma once

#include <string.h>

#include "ops.cuh"
#include "ot_internal.cuh"

namespace dftgpu {

// Real-field slots written by the potential evaluation (potential_t).  After a
// potential evaluation they hold, for the wave function it was evaluated on:
// R_RB rho_bar, R_RT F*rho, R_A V_j*rho,
// R_Q (c2 rb + c3 rb^2) rho, R_RST rho_st (energy density only: the potential and
// its adjoint recompute rho_st = 1 - R_RT / rho_0s), R_S0..2 G_a = (d_a rho) rho_st,
// R_V0..2 the velocity v_a (BF),
// R_E rho|v|^2, R_B0..2 rho v_a, R_J0..2 J_a = F*G_a,
// R_C V_j*(rho|v|^2) (only with a clamped backflow potential),
// R_BB0..2 B_a = V_j*(rho v_a), R_H sum_a (d_a rho) J_a.  R_U is not used
// by the potential (the merged linear part LJ*rho + w*q + c F*h
// - m/2 V_j*(rho|v|^2) is added into P by its inverse transform); the energy
// density uses slot 0 as scratch.  Slots from R_NREAL on are free.
// R_RG rho G(rho), the backflow's cut-off density of the high-density models.
enum PotSlot {
  R_U, R_RB, R_RT, R_A, R_Q, R_RST, R_S0, R_S1, R_S2, R_V0, R_V1, R_V2, R_E,
  R_B0, R_B1, R_B2, R_J0, R_J1, R_J2, R_C, R_BB0, R_BB1, R_BB2, R_H, R_RG, R_NREAL
};

template <typename T> struct Fields {
  typedef typename cplx_t<T>::type C;
  OtPriv *P;
  int nx, ny, nz;
  T *r(int i) { return (T *) ot_real(P, i); }
  C *s(int i) { return (C *) ot_spec(P, i); }
  const T *k(int i) { return (const T *) P->ker[i]; }
  int fwd(const T *f, C *spec) {
    RealPairLoad<T> ld{f, ny, nz};
    return rfft_zy<T>(ld, spec, nx, ny, nz);
  }
  int inv(C *spec, T *f) {
    RealPairStore<T> st{f, ny, nz, (T) 1};
    return irfft_yz<T>(spec, st, nx, ny, nz);
  }
};

template <typename T> inline void xc_init(XConvArgs<T> &A, const OtPriv *P) {
  memset(&A, 0, sizeof(A));
  A.nx = P->nx; A.ny = P->ny; A.nkz = P->nz / 2 + 1;
}
template <typename T> inline void xc_in(XConvArgs<T> &A, const typename cplx_t<T>::type *s) { A.src[A.nin++] = s; }
template <typename T> inline void xc_out(XConvArgs<T> &A, typename cplx_t<T>::type *dst, int acc = 0) {
  XOut<T> &o = A.out[A.nout++];
  o.dst = dst; o.accumulate = acc;
  o.t0 = A.nout > 1 ? A.out[A.nout - 2].t0 + A.out[A.nout - 2].nt : 0;
  o.nt = 0;
}
template <typename T> inline void xc_term(XConvArgs<T> &A, int in, const T *ker, int kind, T coef) {
  XOut<T> &o = A.out[A.nout - 1];
  XTerm<T> &t = A.term[o.t0 + o.nt];
  t.ker = ker; t.kind = kind; t.in = in; t.coef = coef;
  o.nt++;
}

template <typename T> __device__ __forceinline__ T clampv(T v, T cap) { return v > cap ? cap : (v < -cap ? -cap : v); }

// High-density terms of the HD / HD2 models (libgrid's grid_func1..5, which
// the reference tree does not contain, restated from the published
// functional):
//   Barranco et al., PRB 72, 214522 (2005) (src/ot.h:142-146):
//     E_HD = C rho [1 + tanh(beta (rho - rho_m))],
//     V_HD = dE_HD/drho = C [1 + tanh(t)] + C beta rho sech^2(t), t = beta (rho - rho_m);
//   backflow density cut-off (src/ot.c:1234-1236): rho -> rho G(rho),
//     G(rho) = [1 - tanh(xi (rho - rho_bf))] / 2, and d(rho G)/drho = G + rho G'.
// sech^2 as 1 / cosh^2, which is 0 once cosh overflows.
template <typename T> struct HdPar {
  T beta, rhom, C, xi, rbf;
  __device__ __forceinline__ T vhd(T r) const {
    const T t = beta * (r - rhom), ch = cosh(t);
    return C * ((T) 1 + tanh(t)) + C * beta * r / (ch * ch);
  }
  __device__ __forceinline__ T ehd(T r) const { return C * r * ((T) 1 + tanh(beta * (r - rhom))); }
  __device__ __forceinline__ T g(T r) const { return (T) 0.5 * ((T) 1 - tanh(xi * (r - rbf))); }
  __device__ __forceinline__ T rg(T r) const { return r * g(r); }
  __device__ __forceinline__ T drg(T r) const {
    const T ch = cosh(xi * (r - rbf));
    return g(r) - r * ((T) 0.5 * xi) / (ch * ch);
  }
};
template <typename T> inline HdPar<T> hd_par(const dft_ot_functional *otf) {
  return HdPar<T>{(T) otf->beta, (T) otf->rhom, (T) otf->C, (T) otf->xi, (T) otf->rhobf};
}
inline bool hd_model(const dft_ot_functional *otf) { return (otf->model & (DFT_OT_HD | DFT_OT_HD2)) != 0; }

}  // namespace dftgpu
