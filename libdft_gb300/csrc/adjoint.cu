// Hand-written adjoint (vector-Jacobian products) of the OT potential, the
// split-operator step and the predict-correct step, and the checkpointed
// reverse sweep for the gradient of an end-of-trajectory objective with
// respect to the external potential.
//
// Convention: for a real objective J of complex fields, a cotangent g of psi
// means dJ = Re sum conj(g) dpsi (g = 2 dJ/dpsi^*); a cotangent of a complex
// potential V = Vr + i Vi is stored as gamma = gamma_r + i gamma_i with
// dJ = sum gamma_r dVr + gamma_i dVi.  Sums run over grid points (no volume
// factor); convolutions with the even OT kernels are self-adjoint, those with
// the odd kernels dF_a and the central differences D_a are anti-self-adjoint.
//
// Forward maps (the GPU forward path, which follows src/ot.c:314-991):
//   V_OT[psi]: LJ*rho + c2/2 rb^2 + c3/3 rb^3 + w*[(c2 rb + c3 rb^2) rho]
//     + c sum_a [rho_st (dF_a*G_a) + F*(g_a J_a) - J_a (dF_a*rho)]          (KC)
//     + R + i I  (BF real / imaginary parts)
//   S(V, dt) psi = D F^-1 K F D psi,  D = exp(-i V dt/2), K = exp(-i k^2 dt/2m)
//   PC step: V1 = Vext + V_OT[psi] - mu0, psi_p = S(V1) psi,
//            V2 = (V1 + Vext + V_OT[psi_p] - mu0)/2, psi' = S(V2) psi.
// Adjoints:
//   S^H = S(conj V, -conj dt); dJ/dV = (-i dt/2)(conj(g') psi' + conj(h) u)
//   with u = D psi and h = F^-1 K^H F (D^H g').
// Backflow clamps (max_veloc, max_bfpot) and c_bfpot != 1 are not
// differentiated (rejected).
#include <math.h>

#include <vector>

#include "grid_internal.cuh"
#include "ot_thermal.cuh"
#include "ot_work.cuh"

namespace dftgpu {

enum AdjSlot {
  A_GR = R_NREAL, A_GI, A_WG, A_GAM, A_X, A_Y, A_Z0, A_Z1, A_Z2, A_LJ0, A_LJ1, A_LJ2, A_Q0, A_Q1, A_Q2,
  A_FLJ0, A_FLJ1, A_FLJ2, A_LG0, A_LG1, A_LG2, A_LST, A_LOC, A_LCONV, A_LA, A_LC, A_LB0, A_LB1, A_LB2,
  A_MU0, A_MU1, A_MU2, A_LCIN, A_LBIN0, A_LBIN1, A_LBIN2, A_VX, A_VY, A_VZ, A_K0R, A_K0I, A_K1R, A_K1I,
  A_K2R, A_K2I, A_END
};
static_assert(A_END <= OT_MAX_REAL, "adjoint work slots");

// ------------------------------------------------------------------ OT VJP
// g += (dV_OT/dpsi)^H (gscale * gam).  fresh != 0: the potential work slots
// and otf->density already hold the intermediates of this psi (the last
// potential evaluation was on it), otherwise they are recomputed first.
template <typename T>
static int ot_vjp_t(dft_ot_functional *otf, wf *gwf, const typename cplx_t<T>::type *gam, T gscale,
                    typename cplx_t<T>::type *g, int fresh) {
  typedef typename cplx_t<T>::type C;
  OtPriv *P = (OtPriv *) otf->priv;
  const bool kc = otf->model & DFT_OT_KC, bf = otf->model & DFT_OT_BACKFLOW;
  if (bf && (otf->max_veloc < (999.0 / GRID_AUTOMPS) || otf->max_bfpot < (10000.0 / GRID_AUTOK) || otf->c_bfpot != 1.0)) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "adjoint: backflow clamps / weight are not differentiated");
    return DFTGPU_ERR_UNSUPPORTED;
  }
  if (hd_model(otf)) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "adjoint: the high-density terms (HD, HD2) are not differentiated");
    return DFTGPU_ERR_UNSUPPORTED;
  }
  // forward intermediates for this psi (potential into scratch)
  cgrid *c = gwf->grid;
  if (!fresh) {
    if (!P->pot_tmp) {
      P->pot_tmp = ::cgrid_clone(c, (char *) "pot");
      if (!P->pot_tmp) return DFTGPU_ERR_NOMEM;
    }
    DFT_TRY(ot_potential_ex(otf, P->pot_tmp, gwf, 1, nullptr, 0.0, 1.0));
  }

  Fields<T> F{P, P->nx, P->ny, P->nz};
  const int nx = P->nx, ny = P->ny, nz = P->nz;
  const Stencil3 S{nx, ny, nz};
  std::vector<T *> r(A_END);
  for (int i = 0; i < A_END; i++) { r[i] = F.r(i); if (!r[i]) return DFTGPU_ERR_NOMEM; }
  C *s[OT_MAX_SPEC];
  for (int i = 0; i < OT_MAX_SPEC; i++) { s[i] = F.s(i); if (!s[i]) return DFTGPU_ERR_NOMEM; }
  C *lacc = s[11];                        // spectral accumulator of the convolution parts of lambda_rho
  const C *psi = (const C *) c->value;
  const T *rho = (const T *) otf->density->value;
  const T inv2h = (T) (1.0 / (2.0 * P->step));

  // gamma split
  {
    T *gr = r[A_GR], *gi = r[A_GI];
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      gr[i] = gscale * gam[i].x;
      gi[i] = gscale * gam[i].y;
    }, 0.0, "adj_split"));
  }
  // stage 1: LJ*gamma (into the accumulator), w*gamma, F*gamma
  DFT_TRY(F.fwd(r[A_GR], s[0]));
  {
    XConvArgs<T> A; xc_init(A, P); xc_in(A, (const C *) s[0]);
    xc_out(A, lacc); xc_term(A, 0, F.k(OT_LJ), KER_EVEN, (T) 1);
    xc_out(A, s[1]); xc_term(A, 0, F.k(OT_SA), KER_EVEN, (T) 1);
    if (kc) { xc_out(A, s[2]); xc_term(A, 0, F.k(OT_F), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(A));
    DFT_TRY(F.inv(s[1], r[A_WG]));
    if (kc) DFT_TRY(F.inv(s[2], r[A_GAM]));
  }
  // pointwise 1: X = gamma (c2 rb + c3 rb^2) + Wg (c2 + 2 c3 rb) rho ; lambda_loc = Wg (c2 rb + c3 rb^2)
  //   KC: Y = gamma rho_st, divZ = sum_a D_a (gamma J_a), lJ_a = c (Gam g_a - gamma D_a (F*rho))
  //   (dF_a = D_a F, so sum_a dF_a*(gamma J_a) = F*divZ and dF_a*rho = D_a (F*rho))
  {
    const T c2 = (T) otf->c2, c3 = (T) otf->c3, ck = (T) (otf->alpha_s / (2.0 * otf->mass));
    T *gr = r[A_GR], *wg = r[A_WG], *gm = r[A_GAM], *X = r[A_X], *loc = r[A_LOC], *Y = r[A_Y];
    T *rb = r[R_RB], *rt = r[R_RT], *dz = r[A_Z0];
    const T irs = (T) (1.0 / otf->rho_0s);
    T *L0 = r[A_LJ0], *L1 = r[A_LJ1], *L2 = r[A_LJ2];
    T *J0 = r[R_J0], *J1 = r[R_J1], *J2 = r[R_J2];
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const T b = rb[i], ga = gr[i], w = wg[i], q1 = c2 * b + c3 * b * b;
      X[i] = ga * q1 + w * (c2 + (T) 2 * c3 * b) * rho[i];
      loc[i] = w * q1;
      if (kc) {
        Y[i] = ga * ((T) 1 - rt[i] * irs);   // rho_st as the potential forms it
        const T *Ja[3] = { J0, J1, J2 };
        T *La[3] = { L0, L1, L2 };
        T dv = 0;
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          const T ga_ = (rho[ip] - rho[im]) * inv2h;
          dv += (gr[ip] * Ja[a][ip] - gr[im] * Ja[a][im]) * inv2h;
          La[a][i] = ck * (gm[i] * ga_ - ga * ((rt[ip] - rt[im]) * inv2h));
        }
        dz[i] = dv;
      }
    }, 0.0, "adj_pointwise_1"));
  }
  DFT_TRY(F.fwd(r[A_X], s[3]));
  {
    XConvArgs<T> A; xc_init(A, P); xc_in(A, (const C *) s[3]);
    xc_out(A, lacc, 1); xc_term(A, 0, F.k(OT_SA), KER_EVEN, (T) 1);        // + w*X
    DFT_TRY(launch_xconv<T>(A));
  }
  if (kc) {
    const T ck = (T) (otf->alpha_s / (2.0 * otf->mass));
    DFT_TRY(F.fwd(r[A_Y], s[4]));
    DFT_TRY(F.fwd(r[A_Z0], s[5]));
    for (int a = 0; a < 3; a++) DFT_TRY(F.fwd(r[A_LJ0 + a], s[8 + a]));
    XConvArgs<T> A; xc_init(A, P);                                          // F*Y ; lacc += c F*divZ
    xc_in(A, (const C *) s[4]);
    xc_in(A, (const C *) s[5]);
    xc_out(A, s[4]); xc_term(A, 0, F.k(OT_F), KER_EVEN, (T) 1);
    xc_out(A, lacc, 1); xc_term(A, 1, F.k(OT_F), KER_EVEN, ck);
    DFT_TRY(launch_xconv<T>(A));
    XConvArgs<T> D; xc_init(D, P);                                          // F * lJ_a
    for (int a = 0; a < 3; a++) xc_in(D, (const C *) s[8 + a]);
    for (int a = 0; a < 3; a++) { xc_out(D, s[8 + a]); xc_term(D, a, F.k(OT_F), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(D));
    DFT_TRY(F.inv(s[4], r[A_Q0]));
    for (int a = 0; a < 3; a++) DFT_TRY(F.inv(s[8 + a], r[A_FLJ0 + a]));
    // pointwise 2: Q_a = dF_a*Y = D_a (F*Y) ; lG_a = -c Q_a + F*lJ_a ; lg_a = c Gam J_a + lG_a rho_st ;
    //              lst = c gamma sum_a D_a J_a + sum lG_a g_a
    {
      T *gr = r[A_GR], *gm = r[A_GAM], *rt = r[R_RT], *lst = r[A_LST], *fy = r[A_Q0];
      const T irs = (T) (1.0 / otf->rho_0s);
      T *F0 = r[A_FLJ0], *F1 = r[A_FLJ1], *F2 = r[A_FLJ2];
      T *J0 = r[R_J0], *J1 = r[R_J1], *J2 = r[R_J2], *G0 = r[A_LG0], *G1 = r[A_LG1], *G2 = r[A_LG2];
      DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
        const T *Fa[3] = { F0, F1, F2 }, *Ja[3] = { J0, J1, J2 };
        T *Ga[3] = { G0, G1, G2 };
        T acc = 0, t1 = 0;
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          const T ga_ = (rho[ip] - rho[im]) * inv2h;
          const T lG = -ck * ((fy[ip] - fy[im]) * inv2h) + Fa[a][i];
          Ga[a][i] = ck * gm[i] * Ja[a][i] + lG * ((T) 1 - rt[i] * irs);
          acc += lG * ga_;
          t1 += (Ja[a][ip] - Ja[a][im]) * inv2h;
        }
        lst[i] = acc + ck * gr[i] * t1;
      }, 0.0, "adj_pointwise_2"));
    }
    // pointwise 3: lambda_loc -= sum_a D_a(lg_a)
    {
      T *loc = r[A_LOC], *G0 = r[A_LG0], *G1 = r[A_LG1], *G2 = r[A_LG2];
      DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
        const T *Ga[3] = { G0, G1, G2 };
        T acc = 0;
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          acc += (Ga[a][ip] - Ga[a][im]) * inv2h;
        }
        loc[i] -= acc;
      }));
    }
    DFT_TRY(F.fwd(r[A_LST], s[3]));
    XConvArgs<T> E; xc_init(E, P); xc_in(E, (const C *) s[3]);
    xc_out(E, lacc, 1); xc_term(E, 0, F.k(OT_F), KER_EVEN, (T) (-1.0 / otf->rho_0s));
    DFT_TRY(launch_xconv<T>(E));
  }
  if (bf) {
    const T m = (T) otf->mass, eps = (T) otf->div_epsilon;
    const T vf = (T) (1.0 / (gwf->mass * 2.0 * P->step)), invm = (T) (1.0 / gwf->mass);
    T *gr = r[A_GR], *gi = r[A_GI], *Aa = r[R_A];
    T *B0 = r[R_BB0], *B1 = r[R_BB1], *B2 = r[R_BB2];
    T *vx = r[A_VX], *vy = r[A_VY], *vz = r[A_VZ], *lA = r[A_LA], *lC = r[A_LC];
    T *lB0 = r[A_LB0], *lB1 = r[A_LB1], *lB2 = r[A_LB2], *mu0 = r[A_MU0], *mu1 = r[A_MU1], *mu2 = r[A_MU2];
    T *loc = r[A_LOC], *p0 = r[A_Q0], *p1 = r[A_Q1], *p2 = r[A_Q2];
    // B1: velocity, lambda_w, lambda_A, lambda_B, lambda_C, mu (first parts), rho_eps terms
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const C pz = psi[i];
      T rr = pz.x * pz.x + pz.y * pz.y;
      if (rr < eps) rr = eps;
      const T g0 = vf / rr;
      T v[3];
      const T *Ba[3] = { B0, B1, B2 };
      T *lBa[3] = { lB0, lB1, lB2 }, *mua[3] = { mu0, mu1, mu2 }, *pa[3] = { p0, p1, p2 };
      for (int a = 0; a < 3; a++) {
        int ip, im; S.nb(x, y, z, i, a, ip, im);
        const C d = psi[ip] - psi[im];
        v[a] = g0 * (pz.x * d.y - pz.y * d.x);
      }
      vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
      const T ga = gr[i], gb = gi[i], A = Aa[i], rh = rho[i];
      const T re = rh < eps ? eps : rh;
      T la = -(T) 0.5 * m * ga * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      T lrho = 0;
      for (int a = 0; a < 3; a++) {
        int ip, im; S.nb(x, y, z, i, a, ip, im);
        const T drho = (rho[ip] - rho[im]) * inv2h;
        const T dgi = (gi[ip] - gi[im]) * inv2h;
        const T lw = (T) 0.5 * gb * drho / re - (T) 0.5 * dgi;        // lambda_w_a
        la += lw * v[a];
        lBa[a][i] = m * ga * v[a] - lw;
        mua[a][i] = -m * ga * (A * v[a] - Ba[a][i]) + lw * A;
        const T wa = v[a] * A - Ba[a][i];                                 // w_a = v_a A - B_a
        pa[a][i] = (T) 0.5 * gb * wa / re;                               // for - D_a(1/2 gamma_i w_a / rho_eps)
        if (rh > eps) lrho -= (T) 0.5 * gb * drho * wa / (re * re);
      }
      lA[i] = la;
      lC[i] = -(T) 0.5 * m * ga;
      loc[i] += lrho;
    }));
    // B2: lambda_loc -= sum_a D_a(p_a)
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const T *pa[3] = { p0, p1, p2 };
      T acc = 0;
      for (int a = 0; a < 3; a++) {
        int ip, im; S.nb(x, y, z, i, a, ip, im);
        acc += (pa[a][ip] - pa[a][im]) * inv2h;
      }
      loc[i] -= acc;
    }));
    DFT_TRY(F.fwd(r[A_LA], s[3]));
    DFT_TRY(F.fwd(r[A_LC], s[4]));
    for (int a = 0; a < 3; a++) DFT_TRY(F.fwd(r[A_LB0 + a], s[5 + a]));
    {
      XConvArgs<T> A; xc_init(A, P); xc_in(A, (const C *) s[3]);
      xc_out(A, lacc, 1); xc_term(A, 0, F.k(OT_VJ), KER_EVEN, (T) 1);    // + V_j * lambda_A
      DFT_TRY(launch_xconv<T>(A));
      XConvArgs<T> B; xc_init(B, P);
      for (int a = 0; a < 4; a++) xc_in(B, (const C *) s[4 + a]);
      for (int a = 0; a < 4; a++) { xc_out(B, s[4 + a]); xc_term(B, a, F.k(OT_VJ), KER_EVEN, (T) 1); }
      DFT_TRY(launch_xconv<T>(B));
      DFT_TRY(F.inv(s[4], r[A_LCIN]));
      for (int a = 0; a < 3; a++) DFT_TRY(F.inv(s[5 + a], r[A_LBIN0 + a]));
    }
    // B3: lambda_loc += lCin |v|^2 + sum lBin_a v_a ; mu_a += 2 lCin rho v_a + lBin_a rho ;
    //     velocity adjoint: g += -i kappa_a D_a psi + 2 lrho_v psi, K_a = kappa_a psi stored
    T *lCin = r[A_LCIN], *lb0 = r[A_LBIN0], *lb1 = r[A_LBIN1], *lb2 = r[A_LBIN2];
    T *k0r = r[A_K0R], *k0i = r[A_K0I], *k1r = r[A_K1R], *k1i = r[A_K1I], *k2r = r[A_K2R], *k2i = r[A_K2I];
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const T v[3] = { vx[i], vy[i], vz[i] };
      const T *lba[3] = { lb0, lb1, lb2 }, *mua[3] = { mu0, mu1, mu2 };
      T *kr[3] = { k0r, k1r, k2r }, *ki[3] = { k0i, k1i, k2i };
      const T rh = rho[i], lc = lCin[i];
      loc[i] += lc * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) + lba[0][i] * v[0] + lba[1][i] * v[1] + lba[2][i] * v[2];
      const C pz = psi[i];
      const T r2 = pz.x * pz.x + pz.y * pz.y;
      const T rv = r2 < eps ? eps : r2;
      C gg = g[i];
      T lrv = 0;
      for (int a = 0; a < 3; a++) {
        const T mu = mua[a][i] + (T) 2 * lc * rh * v[a] + lba[a][i] * rh;
        const T kap = mu * invm / rv;
        int ip, im; S.nb(x, y, z, i, a, ip, im);
        const C d = psi[ip] - psi[im];
        const C dpsi = mk<T>(d.x * inv2h, d.y * inv2h);
        gg.x += kap * dpsi.y;             // -i kappa D psi
        gg.y -= kap * dpsi.x;
        kr[a][i] = kap * pz.x;
        ki[a][i] = kap * pz.y;
        if (r2 > eps) lrv -= mu * v[a] / rv;
      }
      gg.x += (T) 2 * lrv * pz.x;
      gg.y += (T) 2 * lrv * pz.y;
      g[i] = gg;
    }));
    // B4: g += -i sum_a D_a(K_a)
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const T *kr[3] = { k0r, k1r, k2r }, *ki[3] = { k0i, k1i, k2i };
      C gg = g[i];
      for (int a = 0; a < 3; a++) {
        int ip, im; S.nb(x, y, z, i, a, ip, im);
        const T dr = (kr[a][ip] - kr[a][im]) * inv2h, di = (ki[a][ip] - ki[a][im]) * inv2h;
        gg.x += di;                        // -i (dr + i di) = di - i dr
        gg.y -= dr;
      }
      g[i] = gg;
    }));
  }
  // lambda_rho = lambda_loc + (convolution parts); g += 2 lambda_rho psi
  DFT_TRY(F.inv(lacc, r[A_LCONV]));
  {
    T *loc = r[A_LOC], *lcv = r[A_LCONV];
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const T l = (T) 2 * (loc[i] + lcv[i]);
      const C pz = psi[i];
      C gg = g[i];
      gg.x += l * pz.x;
      gg.y += l * pz.y;
      g[i] = gg;
    }));
  }
  return DFTGPU_OK;
}

static int ot_vjp(dft_ot_functional *otf, wf *gwf, cgrid *gam, double gscale, cgrid *g, int fresh) {
  return g->prec == DFTGPU_FP32
             ? ot_vjp_t<float>(otf, gwf, (const float2 *) gam->value, (float) gscale, (float2 *) g->value, fresh)
             : ot_vjp_t<double>(otf, gwf, (const double2 *) gam->value, gscale, (double2 *) g->value, fresh);
}

// ------------------------------------------------------------------ split-operator VJP
// exponent a = -i V dt/2 as (re, im)
template <typename T> __device__ __forceinline__ typename cplx_t<T>::type half_exponent(typename cplx_t<T>::type v, T hr, T hi) {
  return mk<T>(v.x * hi + v.y * hr, -(v.x * hr - v.y * hi));
}

// Split functors of the line kernels (as the forward propagation's): AdjLoad
// fetches all of a thread's operands before combining them, AdjStore
// prefetches its operand lines into L2 before the transform.
template <typename T> struct AdjLoad {   // D^H g' = exp(conj a) g'
  typedef typename cplx_t<T>::type C;
  static constexpr bool kSplit = true, kAhead = true;
  struct Raw { C g, v; };
  const C *gp; const C *V; int ny, nz; T hr, hi;
  __device__ void prefetch_lines(int x, int y0, int nl, int) const {
    const size_t o = ((size_t) x * ny + y0) * nz, n = (size_t) nl * nz * sizeof(C);
    if (threadIdx.x == 0) prefetch_bulk_l2(gp + o, n);
    if (threadIdx.x == 32) prefetch_bulk_l2(V + o, n);
  }
  __device__ Raw fetch(int x, int y, int e) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    return Raw{ gp[i], V[i] };
  }
  __device__ C cook(const Raw &r) const {
    C a = half_exponent<T>(r.v, hr, hi);
    a.y = -a.y;
    return mul_cexp(r.g, a);
  }
  __device__ C operator()(int x, int y, int e) const { return cook(fetch(x, y, e)); }
};
// h -> g_out = D^H h ; gamma_V += scale * (Re c, -Im c), c = (-i dt/2)(conj(g') psi' + conj(h) D psi)
template <typename T> struct AdjStore {
  typedef typename cplx_t<T>::type C;
  static constexpr bool kSplit = true;
  C *gout; const C *gp; const C *psi; const C *psio; const C *V; C *gamV; int ny, nz; T hr, hi, dr2, di2, scale; int acc;
  __device__ void prefetch(int x, int y, int e) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    if ((i * sizeof(C)) % 32) return;                    // one per 32-byte sector
    prefetch_l2(V + i); prefetch_l2(psi + i); prefetch_l2(psio + i); prefetch_l2(gp + i); prefetch_l2(gamV + i);
    if (acc) prefetch_l2(gout + i);
  }
  __device__ void operator()(int x, int y, int e, C h) const {
    const size_t i = ((size_t) x * ny + y) * nz + e;
    // operands this kernel never writes through the read-only path (their
    // loads may move ahead of the previous elements' stores); gp may be gout
    const C a = half_exponent<T>(__ldg(V + i), hr, hi);
    const C u = mul_cexp(__ldg(psi + i), a);
    const C Y = cmulc(__ldg(psio + i), gp[i]) + cmulc(u, h);   // conj(g') psi' + conj(h) u
    // c = (-i dt/2) Y with dt/2 = (dr2, di2): (-i)(dr2 + i di2) = di2 - i dr2
    const C cc = mk<T>(di2 * Y.x + dr2 * Y.y, di2 * Y.y - dr2 * Y.x);
    C gv = gamV[i];
    gv.x += scale * cc.x;
    gv.y -= scale * cc.y;
    gamV[i] = gv;
    const C o = mul_cexp(h, conjc(a));
    gout[i] = acc ? gout[i] + o : o;
  }
};

// g_out (+)= S(V,dt)^H g_in and gamV += scale * dJ/dV, given psi (step input)
// and psio = S(V,dt) psi; acc selects g_out += instead of =.  g_out may alias
// g_in when acc == 0.  Uses the wave function's spectral scratch.
template <typename T>
static int strang_vjp_t(wf *g, cgrid *V, double dr, double di, const cgrid *psi, const cgrid *psio, const cgrid *gin,
                        cgrid *gout, cgrid *gamV, double scale, int acc) {
  typedef typename cplx_t<T>::type C;
  const int nx = (int) V->nx, ny = (int) V->ny, nz = (int) V->nz;
  C *spec = (C *) wf_spec(g);
  if (!spec) return DFTGPU_ERR_NOMEM;
  const T hr = (T) (0.5 * dr), hi = (T) (0.5 * di);
  AdjLoad<T> ld{(const C *) gin->value, (const C *) V->value, ny, nz, hr, hi};
  SpecStoreZ<T> sz{spec, nx, ny};
  DFT_TRY((launch_lines<T, LINE_C2C, 1, 0>(nz, nx, ny, (T) -1, ld, sz)));
  DFT_TRY(ypass<T>(spec, nx, ny, nz, (T) -1));
  KinArgs<T> K;
  kin_args<T>(K, nx, ny, nz, V->step, make_double2(di / (2.0 * g->mass), dr / (2.0 * g->mass)),   // conj(-i dt / 2m)
              g->grid->kx0, g->grid->ky0, g->grid->kz0, spec);
  K.cn = g->propagator == WF_2ND_ORDER_CN;   // real Q: the conjugate factor is the factor of conj(c)
  DFT_TRY(launch_xkinetic<T>(K));
  DFT_TRY(ypass<T>(spec, nx, ny, nz, (T) 1));
  SpecLoadZ<T> lz{spec, nx, ny};
  AdjStore<T> st{(C *) gout->value, (const C *) gin->value, (const C *) psi->value, (const C *) psio->value,
                 (const C *) V->value, (C *) gamV->value, ny, nz, hr, hi, (T) (0.5 * dr), (T) (0.5 * di), (T) scale, acc};
  return launch_lines<T, LINE_C2C, 0, 1>(nz, nx, ny, (T) 1, lz, st);
}

static int strang_vjp(wf *g, cgrid *V, double dr, double di, const cgrid *psi, const cgrid *psio, const cgrid *gin,
                      cgrid *gout, cgrid *gamV, double scale, int acc) {
  return V->prec == DFTGPU_FP32 ? strang_vjp_t<float>(g, V, dr, di, psi, psio, gin, gout, gamV, scale, acc)
                                : strang_vjp_t<double>(g, V, dr, di, psi, psio, gin, gout, gamV, scale, acc);
}

// ------------------------------------------------------------------ predict-correct step VJP
// Work state kept with the functional: the recorded step (V1, psi_p, V2,
// psi') and the cotangent buffers.  wk / wp are wave functions (mass, spectral
// scratch) whose grids hold the step input psi_k and the predicted psi_p.
struct AdjWork {
  wf *wk = nullptr, *wp = nullptr;
  cgrid *V1 = nullptr, *V2 = nullptr, *psio = nullptr, *gV1 = nullptr, *gV2 = nullptr, *gp = nullptr, *gt = nullptr,
        *g = nullptr;
};

static void work_free(AdjWork *W) {
  if (!W) return;
  grid_wf_free(W->wk); grid_wf_free(W->wp);
  cgrid *c[] = { W->V1, W->V2, W->psio, W->gV1, W->gV2, W->gp, W->gt, W->g };
  for (cgrid *x : c) cgrid_free(x);
  delete W;
}

void adj_free(OtPriv *P) {
  work_free((AdjWork *) P->adj);
  P->adj = nullptr;
}

static void same_momentum(wf *dst, const wf *src) {
  dst->grid->kx0 = src->grid->kx0; dst->grid->ky0 = src->grid->ky0; dst->grid->kz0 = src->grid->kz0;
}

static AdjWork *work_get(OtPriv *P, wf *gwf) {
  AdjWork *W = (AdjWork *) P->adj;
  if (W && W->wk->mass == gwf->mass && W->wk->propagator == gwf->propagator) {
    same_momentum(W->wk, gwf); same_momentum(W->wp, gwf);
    return W;
  }
  adj_free(P);
  W = new AdjWork();
  W->wk = grid_wf_clone(gwf, (char *) "adj_psi");   // the clones carry gwf's momentum
  W->wp = grid_wf_clone(gwf, (char *) "adj_psip");
  cgrid *c = gwf->grid;
  cgrid **f[] = { &W->V1, &W->V2, &W->psio, &W->gV1, &W->gV2, &W->gp, &W->gt, &W->g };
  bool ok = W->wk && W->wp;
  for (cgrid **x : f) { *x = ::cgrid_clone(c, (char *) "adj"); ok = ok && *x; }
  if (!ok) { work_free(W); set_error(DFTGPU_ERR_NOMEM, "adjoint work buffers"); return nullptr; }
  P->adj = W;
  return W;
}

static int ccopy(cgrid *d, const cgrid *s) {
  DFT_CUDA(cudaMemcpyAsync(d->value, s->value, gsize(s) * 2 * elem_size(s->prec), cudaMemcpyDeviceToDevice, rt().stream));
  return DFTGPU_OK;
}

// The forward predict-correct step from psi_k (in W->wk), with the same
// kernels as dftgpu_pc_step: V1, psi_p, V2 and psi' (before renormalisation)
// are left in W.  Afterwards the potential work slots hold psi_p's intermediates.
static int record_step(dft_ot_functional *otf, AdjWork *W, rgrid *vext, double mu0, double dr, double di) {
  DFT_TRY(ot_potential_ex(otf, W->V1, W->wk, 1, vext, -mu0, 1.0));
  DFT_TRY(propagate(W->wk, W->wp->grid, W->wk->grid, W->V1, dr, di));
  DFT_TRY(ccopy(W->V2, W->V1));
  DFT_TRY(ot_potential_ex(otf, W->V2, W->wp, 0, vext, -mu0, 0.5));
  return propagate(W->wk, W->psio, W->wk->grid, W->V2, dr, di);
}

// dst = one step (with renormalisation to norm when renorm) from src
static int fwd_step(dft_ot_functional *otf, AdjWork *W, const cgrid *src, cgrid *dst, rgrid *vext, double mu0, double dr,
                    double di, int renorm, double norm) {
  DFT_TRY(ccopy(W->wk->grid, src));
  DFT_TRY(record_step(otf, W, vext, mu0, dr, di));
  if (renorm) {
    double *slot = reduce_slots();
    DFT_TRY(norm_dev(W->psio, slot + 4));
    DFT_TRY(scale_by_norm(W->psio, slot + 4, norm));
  }
  return ccopy(dst, W->psio);
}

// g <- s g - (s/n) Re<g, psi'> dV psi' for psi'' = s psi', s = sqrt(norm / n),
// n = int |psi'|^2 (the VJP of the renormalisation)
template <typename T> static int renorm_vjp_t(cgrid *psio, cgrid *g, double norm) {
  typedef typename cplx_t<T>::type C;
  const C *p = (const C *) psio->value;
  C *gv = (C *) g->value;
  const size_t n = gsize(psio);
  const double dv = psio->step * psio->step * psio->step;
  double r[2];
  DFT_TRY(reduce_host<2>(n, [=] __device__(size_t i, double *v) {
    const C a = p[i], b = gv[i];
    v[0] = (double) a.x * a.x + (double) a.y * a.y;
    v[1] = (double) a.x * b.x + (double) a.y * b.y;
  }, r, dv));
  if (!(r[0] > 0.0)) { set_error(DFTGPU_ERR_NONFINITE, "adjoint: zero norm"); return DFTGPU_ERR_NONFINITE; }
  const double s = sqrt(norm / r[0]);
  const T a = (T) s, b = (T) (-s / r[0] * r[1]);
  return launch_each(n, [=] __device__(size_t i) { gv[i] = gv[i] * a + p[i] * b; });
}

template <typename T> static int gvext_acc_t(rgrid *gv, const cgrid *g1, const cgrid *g2) {
  typedef typename cplx_t<T>::type C;
  T *o = (T *) gv->value;
  const C *a = (const C *) g1->value, *b = (const C *) g2->value;
  return launch_each(gsize(g1), [=] __device__(size_t i) { o[i] += a[i].x + (T) 0.5 * b[i].x; });
}
template <typename T> static int half_copy_t(cgrid *d, const cgrid *s) {
  typedef typename cplx_t<T>::type C;
  C *o = (C *) d->value;
  const C *a = (const C *) s->value;
  return launch_each(gsize(s), [=] __device__(size_t i) { o[i] = a[i] * (T) 0.5; });
}

// g (cotangent of the step output) <- cotangent of its input psi_k (in W->wk);
// gvext += the step's contribution to dJ/dVext.
static int step_vjp(dft_ot_functional *otf, AdjWork *W, rgrid *vext, double mu0, double dr, double di, int renorm,
                    double norm, cgrid *g, rgrid *gvext) {
  const bool f32 = g->prec == DFTGPU_FP32;
  DFT_TRY(record_step(otf, W, vext, mu0, dr, di));
  if (renorm) DFT_TRY(f32 ? renorm_vjp_t<float>(W->psio, g, norm) : renorm_vjp_t<double>(W->psio, g, norm));
  // psi' = S(V2) psi_k
  DFT_TRY(cfill(W->gV2, 0.0, 0.0));
  DFT_TRY(strang_vjp(W->wk, W->V2, dr, di, W->wk->grid, W->psio, g, W->gt, W->gV2, 1.0, 0));
  // V2 = (V1 + Vext + V_OT[psi_p] - mu0) / 2
  DFT_TRY(f32 ? half_copy_t<float>(W->gV1, W->gV2) : half_copy_t<double>(W->gV1, W->gV2));
  DFT_TRY(cfill(W->gp, 0.0, 0.0));
  DFT_TRY(ot_vjp(otf, W->wp, W->gV2, 0.5, W->gp, 1));
  // psi_p = S(V1) psi_k
  DFT_TRY(strang_vjp(W->wk, W->V1, dr, di, W->wk->grid, W->wp->grid, W->gp, W->gt, W->gV1, 1.0, 1));
  // V1 = Vext + V_OT[psi_k] - mu0
  if (gvext) DFT_TRY(f32 ? gvext_acc_t<float>(gvext, W->gV1, W->gV2) : gvext_acc_t<double>(gvext, W->gV1, W->gV2));
  DFT_TRY(ot_vjp(otf, W->wk, W->gV1, 1.0, W->gt, 0));
  return ccopy(g, W->gt);
}

// J = int (|psi|^2 - rho_t)^2 dV and g = 2 dJ/dpsi^* = 4 (|psi|^2 - rho_t) dV psi
template <typename T> static int objective_t(const cgrid *psi, const rgrid *rt_, cgrid *g, double *J) {
  typedef typename cplx_t<T>::type C;
  const C *p = (const C *) psi->value;
  const T *t = (const T *) rt_->value;
  C *gv = (C *) g->value;
  const size_t n = gsize(psi);
  const double dv = psi->step * psi->step * psi->step;
  DFT_TRY(reduce_host<1>(n, [=] __device__(size_t i, double *v) {
    const C a = p[i];
    const double d = (double) a.x * a.x + (double) a.y * a.y - (double) t[i];
    v[0] = d * d;
  }, J, dv));
  const T f = (T) (4.0 * dv);
  return launch_each(n, [=] __device__(size_t i) {
    const C a = p[i];
    gv[i] = a * (f * (a.x * a.x + a.y * a.y - t[i]));
  });
}

}  // namespace dftgpu

// ------------------------------------------------------------------ C entry points
using namespace dftgpu;

namespace {

int adj_arg(const char *what) { set_error(DFTGPU_ERR_ARG, "%s", what); return DFTGPU_ERR_ARG; }

bool fits(dft_ot_functional *otf, const cgrid *c) {
  OtPriv *P = otf ? (OtPriv *) otf->priv : nullptr;
  return c && P && c->nx == P->nx && c->ny == P->ny && c->nz == P->nz && c->prec == P->prec;
}
bool fits_r(dft_ot_functional *otf, const rgrid *r) {
  OtPriv *P = otf ? (OtPriv *) otf->priv : nullptr;
  return r && P && r->nx == P->nx && r->ny == P->ny && r->nz == P->nz && r->prec == P->prec;
}

// The potential evaluations leave every intermediate the VJP reads in its
// work slot (rho_st excepted, which the VJP recomputes from F*rho).
// The high-density terms and the absorbing boundary are not differentiated:
// refused before any work.
int hd_refused(dft_ot_functional *otf, wf *gwf = nullptr) {
  if (gwf && ((WfPriv *) gwf->priv)->abs.on) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "adjoint: the absorbing boundary is not differentiated");
    return DFTGPU_ERR_UNSUPPORTED;
  }
  if (bose_model(otf)) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "adjoint: the thermal models' ideal Bose gas term is not differentiated");
    return DFTGPU_ERR_UNSUPPORTED;
  }
  if (!hd_model(otf)) return DFTGPU_OK;
  set_error(DFTGPU_ERR_UNSUPPORTED, "adjoint: the high-density terms (HD, HD2) are not differentiated");
  return DFTGPU_ERR_UNSUPPORTED;
}

}  // namespace

extern "C" {

int dftgpu_ot_potential_vjp(dft_ot_functional *otf, wf *gwf, cgrid *cot, cgrid *grad_psi) {
  if (!otf || !gwf || !fits(otf, gwf->grid) || !fits(otf, cot) || !fits(otf, grad_psi))
    return adj_arg("dftgpu_ot_potential_vjp: grid mismatch");
  DFT_TRY(hd_refused(otf));
  return ot_vjp(otf, gwf, cot, 1.0, grad_psi, 0);
}

int dftgpu_wf_propagate_vjp(wf *gwf, cgrid *pot, double dt_re, double dt_im, cgrid *psi_in, cgrid *psi_out,
                            cgrid *cot_out, cgrid *cot_in, cgrid *cot_pot) {
  if (!gwf || !pot || !psi_in || !psi_out || !cot_out || !cot_in || !cot_pot)
    return adj_arg("dftgpu_wf_propagate_vjp: NULL argument");
  const cgrid *c[] = { pot, psi_in, psi_out, cot_out, cot_in, cot_pot };
  for (const cgrid *x : c)
    if (x->nx != gwf->grid->nx || x->ny != gwf->grid->ny || x->nz != gwf->grid->nz || x->prec != gwf->grid->prec)
      return adj_arg("dftgpu_wf_propagate_vjp: grid mismatch");
  return strang_vjp(gwf, pot, dt_re, dt_im, psi_in, psi_out, cot_out, cot_in, cot_pot, 1.0, 0);
}

int dftgpu_pc_step_vjp(dft_ot_functional *otf, wf *gwf, rgrid *vext, double mu0, double dt_re, double dt_im, int renorm,
                       cgrid *cot, rgrid *grad_vext) {
  if (!otf || !gwf || !fits(otf, gwf->grid) || !fits(otf, cot)) return adj_arg("dftgpu_pc_step_vjp: grid mismatch");
  if ((vext && !fits_r(otf, vext)) || (grad_vext && !fits_r(otf, grad_vext)))
    return adj_arg("dftgpu_pc_step_vjp: vext mismatch");
  DFT_TRY(hd_refused(otf, gwf));
  AdjWork *W = work_get((OtPriv *) otf->priv, gwf);
  if (!W) return DFTGPU_ERR_NOMEM;
  DFT_TRY(ccopy(W->wk->grid, gwf->grid));
  return step_vjp(otf, W, vext, mu0, dt_re, dt_im, renorm, gwf->norm, cot, grad_vext);
}

int dftgpu_adjoint_run(dft_ot_functional *otf, wf *gwf, rgrid *vext, double mu0, double dt_re, double dt_im, INT nsteps,
                       int renorm, INT checkpoint_every, rgrid *rho_target, double *J, rgrid *grad_vext,
                       cgrid *grad_psi0) {
  if (!otf || !gwf || !fits(otf, gwf->grid) || !fits_r(otf, rho_target) || !J)
    return adj_arg("dftgpu_adjoint_run: grid mismatch");
  if ((vext && !fits_r(otf, vext)) || (grad_vext && !fits_r(otf, grad_vext)) || (grad_psi0 && !fits(otf, grad_psi0)))
    return adj_arg("dftgpu_adjoint_run: grid mismatch");
  if (nsteps < 0) return adj_arg("dftgpu_adjoint_run: nsteps < 0");
  DFT_TRY(hd_refused(otf, gwf));
  AdjWork *W = work_get((OtPriv *) otf->priv, gwf);
  if (!W) return DFTGPU_ERR_NOMEM;
  const bool f32 = gwf->grid->prec == DFTGPU_FP32;
  INT K = checkpoint_every > 0 ? checkpoint_every : (INT) ceil(sqrt((double) (nsteps > 0 ? nsteps : 1)));
  if (K > nsteps && nsteps > 0) K = nsteps;
  const bool want = grad_vext || grad_psi0;              // else: forward sweep and J only
  const INT nck = nsteps > 0 && want ? (nsteps + K - 1) / K : 0;
  std::vector<cgrid *> ck, seg;
  int rc = DFTGPU_OK;
  for (INT c = 0; c < nck && !rc; c++) { ck.push_back(::cgrid_clone(gwf->grid, (char *) "adj_ck")); if (!ck.back()) rc = DFTGPU_ERR_NOMEM; }
  for (INT j = 1; j < K && nck > 0 && !rc; j++) { seg.push_back(::cgrid_clone(gwf->grid, (char *) "adj_seg")); if (!seg.back()) rc = DFTGPU_ERR_NOMEM; }
  if (!rc && grad_vext) rc = rfill(grad_vext, 0.0);
  // forward sweep: checkpoints psi_0, psi_K, psi_2K, ...; gwf ends at psi_T
  for (INT s = 0; s < nsteps && !rc; s++) {
    if (want && s % K == 0) rc = ccopy(ck[s / K], gwf->grid);
    if (!rc) rc = fwd_step(otf, W, gwf->grid, gwf->grid, vext, mu0, dt_re, dt_im, renorm, gwf->norm);
  }
  if (!rc) rc = f32 ? objective_t<float>(gwf->grid, rho_target, W->g, J) : objective_t<double>(gwf->grid, rho_target, W->g, J);
  if (!rc && !isfinite(*J)) { rc = DFTGPU_ERR_NONFINITE; set_error(rc, "dftgpu_adjoint_run: non-finite objective"); }
  // reverse sweep, one checkpoint segment at a time
  for (INT c = nck - 1; c >= 0 && !rc; c--) {
    const INT s0 = c * K, len = (s0 + K < nsteps ? K : nsteps - s0);
    std::vector<cgrid *> st(len);
    st[0] = ck[c];
    for (INT j = 1; j < len && !rc; j++) {
      st[j] = seg[j - 1];
      rc = fwd_step(otf, W, st[j - 1], st[j], vext, mu0, dt_re, dt_im, renorm, gwf->norm);
    }
    for (INT j = len - 1; j >= 0 && !rc; j--) {
      rc = ccopy(W->wk->grid, st[j]);
      if (!rc) rc = step_vjp(otf, W, vext, mu0, dt_re, dt_im, renorm, gwf->norm, W->g, grad_vext);
    }
  }
  if (!rc && grad_psi0) rc = ccopy(grad_psi0, W->g);
  if (!rc && cudaStreamSynchronize(rt().stream) != cudaSuccess) { rc = DFTGPU_ERR_CUDA; set_error(rc, "dftgpu_adjoint_run"); }
  for (cgrid *x : ck) cgrid_free(x);
  for (cgrid *x : seg) cgrid_free(x);
  return rc;
}

}  // extern "C"
