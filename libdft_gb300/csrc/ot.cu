// Orsay-Trento functional on the GPU: kernel generation, potential and
// energy density (libdft src/ot.c:66-991, src/ot-energy.c:38-288).
//
// Potential dataflow (full model), one forward r2c per produced field and
// one inverse c2r per needed real field; linearity merges the reference's
// per-axis KC transforms and every term that enters the potential linearly:
//   rho = |psi|^2 ;  rho^ = F rho
//   x pass 1 (one input): w rho^, F rho^, V_j rho^
//   pointwise 1: P.re += c2/2 rb^2 + c3/3 rb^3 ; q = (c2 rb + c3 rb^2) rho
//             KC: rho_st, s_a = (d_a rho) rho_st ;  BF: v, rho|v|^2, rho v_a
//   x pass 2: F s_a^ (-> J_a) ; V_j (rho v_a)^ (-> B_a)
//   pointwise 2: P.re += c rho_st sum_a D_a J_a - c sum_a J_a D_a(F*rho)
//             (dF_a = D_a F: the derivative kernels are central differences)
//             KC: h = sum_a (d_a rho) J_a ;  BF: -m/2 (A|v|^2 - 2 v.B) and the
//             imaginary part from w_a = v_a A - B_a (formed at each stencil point)
//   x pass 3: V_LJ rho^ + w q^ + c F h^ - m/2 V_j (rho|v|^2)^  (one output)
//   pointwise 3: P.re += that linear part.
// Full model: 10 forward and 10 inverse real transforms (src/ot.c: 34).
#include <math.h>
#include <string.h>

#include "grid_internal.cuh"
#include "ot_march.cuh"
#include "ot_thermal.cuh"
#include "ot_work.cuh"

namespace dftgpu {

// ------------------------------------------------------------------ shapes
// (src/common.c:31-66, 131-138, 193-200; src/ot-private.h:10-21)
struct ShapeLJ {
  double h, sig, eps, cval;
  __device__ double operator()(double x, double y, double z) const {
    const double r2 = x * x + y * y + z * z;
    if (r2 <= h * h) return cval;
    const double s2 = sig * sig / r2, s6 = s2 * s2 * s2;
    return 4.0 * eps * s6 * (s6 - 1.0);
  }
};
struct ShapeSA {
  double h;
  __device__ double operator()(double x, double y, double z) const {
    return (x * x + y * y + z * z <= h * h) ? 3.0 / (4.0 * M_PI * h * h * h) : 0.0;
  }
};
struct ShapeGauss {
  double iw;
  __device__ double operator()(double x, double y, double z) const {
    const double nrm = iw / sqrt(M_PI);
    return nrm * nrm * nrm * exp(-(x * x + y * y + z * z) * iw * iw);
  }
};
struct ShapeBF {
  double g11, g12, g21, g22, a1, a2;
  __device__ double operator()(double x, double y, double z) const {
    const double r2 = x * x + y * y + z * z;
    return (g11 + g12 * r2) * exp(-a1 * r2) + (g21 + g22 * r2) * exp(-a2 * r2);
  }
};

// 1-D effective kernels of a grid with nx = ny = 1 (libdft's DFT_OT_1D branch,
// src/ot.c:133-217, src/ot.h:146), integrated over the x-y plane: LJ with the
// core |z| < h evaluated at h (src/common.c:80-91), the sphere's
// cross-section (src/common.c:152-158), the Gaussian's line density
// (src/common.c:214-220), the backflow kernel (src/ot-private.h:29-41)
struct ShapeLJ1D {
  double h, sig, eps;
  __device__ double operator()(double, double, double z) const {
    const double s6 = pow(sig, 6.0);
    double a = fabs(z);
    if (a < h) a = h;
    return 2.0 * M_PI * eps * s6 * (2.0 * s6 - 5.0 * pow(a, 6.0)) / (5.0 * pow(a, 10.0));
  }
};
struct ShapeSA1D {
  double h;
  __device__ double operator()(double, double, double z) const {
    const double a = fabs(z);
    return a > h ? 0.0 : 3.0 * (h * h - a * a) / (4.0 * h * h * h);
  }
};
struct ShapeGauss1D {
  double iw;
  __device__ double operator()(double, double, double z) const { return iw / sqrt(M_PI) * exp(-z * z * iw * iw); }
};
struct ShapeBF1D {
  double g11, g12, g21, g22, a1, a2;
  __device__ double operator()(double, double, double z) const {
    const double z2 = z * z;
    return M_PI * ((g11 + g12 * (1.0 + a1 * z2) / a1) * exp(-a1 * z2) / a1 +
                   (g21 + g22 * (1.0 + a2 * z2) / a2) * exp(-a2 * z2) / a2);
  }
};

template <class S>
__device__ double cell_average(const S &f, double x, double y, double z, double step, int ns) {
  double sum = 0.0;
  const double h = step / (double) ns;
  for (int a = 0; a < ns; a++) {
    const double xs = x + ((double) a + 0.5) * h - 0.5 * step;
    for (int b = 0; b < ns; b++) {
      const double ys = y + ((double) b + 0.5) * h - 0.5 * step;
      for (int c = 0; c < ns; c++) {
        const double zs = z + ((double) c + 0.5) * h - 0.5 * step;
        sum += f(xs, ys, zs);
      }
    }
  }
  return sum / (double) (ns * ns * ns);
}

// Cell averages over ns^3 sub-points, ns doubling from min_ns until two
// successive averages differ by less than tol or ns would exceed max_ns.
template <class S>
__global__ void adaptive_map_kernel(double *out, int nx, int ny, int nz, double step, double x0, double y0,
                                    double z0, int min_ns, int max_ns, double tol, S f) {
  const size_t n = (size_t) nx * ny * nz;
  for (size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x) {
    const int k = (int) (i % nz), j = (int) ((i / nz) % ny), ii = (int) (i / ((size_t) ny * nz));
    const double x = (double) (ii - nx / 2) * step - x0;
    const double y = (double) (j - ny / 2) * step - y0;
    const double z = (double) (k - nz / 2) * step - z0;
    int ns = min_ns;
    double v = cell_average(f, x, y, z, step, ns);
    while (2 * ns <= max_ns) {
      const double v2 = cell_average(f, x, y, z, step, 2 * ns);
      ns *= 2;
      const double d = v2 - v;
      v = v2;
      if (fabs(d) < tol) break;
    }
    out[i] = v;
  }
}

template <class S> static int adaptive_map(double *out, const OtPriv *P, int min_ns, int max_ns, double tol, const S &f) {
  const size_t n = (size_t) P->nx * P->ny * P->nz;
  int blocks = (int) ((n + 127) / 128);
  adaptive_map_kernel<S><<<blocks, 128, 0, rt().stream>>>(out, P->nx, P->ny, P->nz, P->step, P->x0, P->y0, P->z0,
                                                          min_ns, max_ns, tol, f);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// central difference along axis of an FP64 field, periodic
static int fd_field(const double *src, double *dst, const OtPriv *P, int axis) {
  const int nx = P->nx, ny = P->ny, nz = P->nz;
  const double inv2h = 1.0 / (2.0 * P->step);
  return launch_each((size_t) nx * ny * nz, [=] __device__(size_t i) {
    const int k = (int) (i % nz), j = (int) ((i / nz) % ny), x = (int) (i / ((size_t) ny * nz));
    size_t ip, im;
    if (axis == 0) { ip = ((size_t) ((x + 1) % nx) * ny + j) * nz + k; im = ((size_t) ((x - 1 + nx) % nx) * ny + j) * nz + k; }
    else if (axis == 1) { ip = ((size_t) x * ny + (j + 1) % ny) * nz + k; im = ((size_t) x * ny + (j - 1 + ny) % ny) * nz + k; }
    else { ip = ((size_t) x * ny + j) * nz + (k + 1) % nz; im = ((size_t) x * ny + j) * nz + (k - 1 + nz) % nz; }
    dst[i] = (src[ip] - src[im]) * inv2h;
  });
}

// FP64 r2c of a real field into the half spectrum [kz][kx][ky]
static int rfft3_fp64(const double *f, double2 *spec, const OtPriv *P) {
  RealPairLoad<double> ld{f, P->ny, P->nz};
  DFT_TRY((rfft_zy<double>(ld, spec, P->nx, P->ny, P->nz)));
  SpecLineXT<double> io{spec, P->nx, P->ny};
  return launch_lines<double, LINE_C2C, 0, 0>(P->nx, P->nz / 2 + 1, P->ny, -1.0, io, io);
}

// Octant [kz][kx][ky] of the (re or im) kernel spectrum, times scale.  The
// kernel was sampled about index c = n/2 of each axis (x_i = (i - n/2) step);
// the kernel about index 0 has the spectrum S(k) exp(2 pi i k c / n) per axis,
// which is the sign (-1)^k for even n and a rotation for odd n.
template <typename T> static int extract_octant(const double2 *spec, T *oct, const OtPriv *P, int imag, double scale) {
  const int nx = P->nx, ny = P->ny, nz = P->nz, kxh = nx / 2 + 1, kyh = ny / 2 + 1, kzh = nz / 2 + 1;
  return launch_each((size_t) kzh * kxh * kyh, [=] __device__(size_t i) {
    const int iy = (int) (i % kyh), ix = (int) ((i / kyh) % kxh), iz = (int) (i / ((size_t) kxh * kyh));
    double2 v = spec[((size_t) iz * nx + ix) * ny + iy];
    const int k[3] = { ix, iy, iz }, n[3] = { nx, ny, nz };
    for (int a = 0; a < 3; a++) {
      if (!(n[a] & 1)) {
        if (k[a] & 1) v = make_double2(-v.x, -v.y);
      } else {   // exp(2 pi i k c / n), c = (n - 1) / 2, reduced modulo n
        double s, c;
        sincospi(2.0 * (double) (((long) k[a] * (n[a] / 2)) % n[a]) / (double) n[a], &s, &c);
        v = make_double2(v.x * c - v.y * s, v.x * s + v.y * c);
      }
    }
    oct[i] = (T) ((imag ? v.y : v.x) * scale);
  });
}

int ot_generate_kernels(dft_ot_functional *otf, int min_ns, int max_ns) {
  OtPriv *P = (OtPriv *) otf->priv;
  const size_t n = (size_t) P->nx * P->ny * P->nz;
  const size_t nspec = (size_t) (P->nz / 2 + 1) * P->nx * P->ny;
  const double tol = 0.01 / GRID_AUTOK;
  // the convolution measure: the volume element, or on a 1-D grid (nx = ny = 1)
  // the line element dz, its kernels being integrated over the x-y plane
  const bool one_d = P->nx == 1 && P->ny == 1;
  const double dv = one_d ? P->step : P->step * P->step * P->step, inv_n = 1.0 / (double) n;
  double *f = (double *) dev_alloc(n * sizeof(double));
  double *g = (double *) dev_alloc(n * sizeof(double));
  double2 *spec = (double2 *) dev_alloc(nspec * sizeof(double2));
  int rc = DFTGPU_OK;
  if (!f || !g || !spec) { rc = DFTGPU_ERR_NOMEM; goto done; }

  for (int kk = 0; kk < OT_NKER; kk++) {
    if (!P->ker[kk]) P->ker[kk] = dev_alloc(P->oct_n * elem_size(P->prec));
    if (!P->ker[kk]) { rc = DFTGPU_ERR_NOMEM; goto done; }
  }

  {
    // LJ with integral b (src/ot.c:150-161), spherical average with integral 1 (src/ot.c:164-181)
    for (int which = 0; which < 2; which++) {
      const double radius = (otf->model & DFT_OT_HD2) ? otf->lj_params.h * 1.065 : otf->lj_params.h;
      if (which == 0 && one_d) {
        rc = adaptive_map(f, P, min_ns, max_ns, tol, ShapeLJ1D{otf->lj_params.h, otf->lj_params.sigma, otf->lj_params.epsilon});
      } else if (which == 0) {
        ShapeLJ s{otf->lj_params.h, otf->lj_params.sigma, otf->lj_params.epsilon, otf->lj_params.cval};
        rc = adaptive_map(f, P, min_ns, max_ns, tol, s);
      } else if (one_d) {
        rc = adaptive_map(f, P, min_ns, max_ns, tol, ShapeSA1D{radius});
      } else {   // HD2: radius 1.065 h (src/ot.c:164-166, PRB 72, 214522)
        rc = adaptive_map(f, P, min_ns, max_ns, tol, ShapeSA{radius});
      }
      if (rc) goto done;
      if ((rc = rfft3_fp64(f, spec, P))) goto done;
      double2 k0;
      if (cudaMemcpyAsync(&k0, spec, sizeof(k0), cudaMemcpyDeviceToHost, rt().stream) != cudaSuccess ||
          cudaStreamSynchronize(rt().stream) != cudaSuccess) { rc = DFTGPU_ERR_CUDA; goto done; }
      // 1-D kernels are not rescaled to their integrals (src/ot.c:159-160, 180-181)
      const double target = which == 0 ? otf->b : 1.0;
      const double scale = one_d ? dv * inv_n : target / (dv * k0.x) * dv * inv_n;
      rc = P->prec == DFTGPU_FP32 ? extract_octant<float>(spec, (float *) P->ker[which], P, 0, scale)
                                  : extract_octant<double>(spec, (double *) P->ker[which], P, 0, scale);
      if (rc) goto done;
    }
    if (otf->model & DFT_OT_KC) {
      // Gaussian F and its central-difference gradient (src/ot.c:184-200)
      rc = one_d ? adaptive_map(f, P, min_ns, max_ns, tol, ShapeGauss1D{1.0 / otf->l_g})
                 : adaptive_map(f, P, min_ns, max_ns, tol, ShapeGauss{1.0 / otf->l_g});
      if (rc) goto done;
      for (int which = 2; which < 6; which++) {
        const double *src = f;
        if (which > 2) { if ((rc = fd_field(f, g, P, which - 3))) goto done; src = g; }
        if ((rc = rfft3_fp64(src, spec, P))) goto done;
        rc = P->prec == DFTGPU_FP32 ? extract_octant<float>(spec, (float *) P->ker[which], P, which > 2, dv * inv_n)
                                    : extract_octant<double>(spec, (double *) P->ker[which], P, which > 2, dv * inv_n);
        if (rc) goto done;
      }
    }
    if (otf->model & DFT_OT_BACKFLOW) {
      // V_j (src/ot.c:207-217)
      const dft_ot_bf &b = otf->bf_params;
      rc = one_d ? adaptive_map(f, P, min_ns, max_ns, tol, ShapeBF1D{b.g11, b.g12, b.g21, b.g22, b.a1, b.a2})
                 : adaptive_map(f, P, min_ns, max_ns, tol, ShapeBF{b.g11, b.g12, b.g21, b.g22, b.a1, b.a2});
      if (rc) goto done;
      if ((rc = rfft3_fp64(f, spec, P))) goto done;
      rc = P->prec == DFTGPU_FP32 ? extract_octant<float>(spec, (float *) P->ker[6], P, 0, dv * inv_n)
                                  : extract_octant<double>(spec, (double *) P->ker[6], P, 0, dv * inv_n);
      if (rc) goto done;
    }
    if (cudaStreamSynchronize(rt().stream) != cudaSuccess) rc = DFTGPU_ERR_CUDA;
  }
done:
  dev_free(f);
  dev_free(g);
  dev_free(spec);
  if (rc && !g_last_error) set_error(rc, "kernel generation failed");
  return rc;
}


// ------------------------------------------------------------------ potential
// P <- scale * ((overwrite ? 0 : P) + base + add + V_OT[psi]); base may be NULL.
// dft_ot_potential is overwrite = 0, base = NULL, add = 0, scale = 1 (src/ot.c:296:
// the potential is added to P); the predict-correct step folds its
// P = Vext, -mu0 and *0.5 (examples/imag_time/imag_time.c:231-238) in here.
//
// Spectral slots: s0 rho^, s1-3 s_a^ -> J_a^, s4 (rho|v|^2)^, s5-7 (rho v_a)^ ->
// B_a^, s8 sum_a dF_a s_a^, s9 q^, s10 h^ (or V_j (rho|v|^2)^ when the backflow
// potential is clamped), s11 the merged linear part.
//
// src selects the terms (LJ, local correlation, KC, BF) and where rho and v
// come from: psi (dft_ot_potential) or given grids (dft_ot_potential2 and the
// per-term entry points, src/ot.c:431-507, 524-586, 840-991).
template <typename T> static int potential_t(dft_ot_functional *otf, cgrid *Pg, wf *gwf, int overwrite, const T *base,
                                             double add_d, double scale_d, const PotSrc &src) {
  const T add = (T) add_d, scale = (T) scale_d;
  typedef typename cplx_t<T>::type C;
  OtPriv *P = (OtPriv *) otf->priv;
  Fields<T> F{P, P->nx, P->ny, P->nz};
  const int nx = P->nx, ny = P->ny, nz = P->nz;
  const double nb = (double) nx * ny * nz * sizeof(T);   // bytes of one real field
  const bool lj = src.terms & POT_LJ, loc = src.terms & POT_LOCAL;
  const bool kc = (src.terms & POT_KC) && (otf->model & DFT_OT_KC);
  const bool bf = (src.terms & POT_BF) && (otf->model & DFT_OT_BACKFLOW);
  // high-density models: the Barranco penalty (a local term) and the
  // backflow's cut-off density rho G(rho) (src/ot.c:374-378, 843-982)
  const bool hd = hd_model(otf), hdp = hd && (src.terms & POT_HD), bfhd = bf && hd;
  const HdPar<T> hp = hd_par<T>(otf);
  // the backflow real part is merged into the linear part unless it is
  // clamped or multiplied by d(rho G)/drho
  const bool clampp = otf->max_bfpot < (10000.0 / GRID_AUTOK);
  const bool cmerge = bf && !clampp && !bfhd;
  const Stencil3 S{nx, ny, nz};
  C *pot = (C *) Pg->value;
  const C *psi = gwf ? (const C *) gwf->grid->value : nullptr;
  T *rho = (T *) otf->density->value;
  const T *vin0 = (const T *) src.vel[0], *vin1 = (const T *) src.vel[1], *vin2 = (const T *) src.vel[2];
  const bool vgiven = vin0 != nullptr;
  if ((!src.dens || (bf && !vgiven)) && !gwf) {
    set_error(DFTGPU_ERR_ARG, "OT potential: no wave function for the density / velocity");
    return DFTGPU_ERR_ARG;
  }

  // real-field slots
  T *r[R_NREAL];   // slots of PotSlot (ot_work.cuh)
  for (int i = 0; i < R_NREAL; i++) {
    r[i] = nullptr;
    if (i == R_U) continue;   // not used here: the linear part goes into P in its inverse transform
    r[i] = F.r(i);
    if (!r[i]) return DFTGPU_ERR_NOMEM;
  }
  C *s[OT_MAX_SPEC];
  for (int i = 0; i < OT_MAX_SPEC; i++) { s[i] = F.s(i); if (!s[i]) return DFTGPU_ERR_NOMEM; }

  if (src.dens) {
    if (src.dens != otf->density->value)
      DFT_CUDA(cudaMemcpyAsync(rho, src.dens, nb, cudaMemcpyDeviceToDevice, rt().stream));
    DFT_TRY(F.fwd(rho, s[0]));
  } else {   // rho = |psi|^2 (src/ot.c:320), formed and stored by the first z pass
    DensityPairLoad<T> ld{psi, rho, ny, nz};
    DFT_TRY(rfft_zy<T>(ld, s[0], nx, ny, nz, 2.0 * nb));
  }
  // HD backflow: A = V_j * (rho G) (src/ot.c:843-849) convolves the cut-off density, s10
  const C *sA = s[0];
  if (bfhd) {
    T *rg = r[R_RG];
    DFT_TRY(launch_each((size_t) nx * ny * nz, [=] __device__(size_t i) { rg[i] = hp.rg(rho[i]); }, 2.0 * nb, "ot_hd_density"));
    DFT_TRY(F.fwd(rg, s[10]));
    sA = s[10];
  }

  // x pass 1: one input, kernels SA (+F) (+V_j); rho^ stays in s0.  The
  // derivative kernels dF_a are the central-difference gradient of the
  // sampled F (src/ot.c:195-196), so dF_a*f = D_a (F*f) on the periodic grid:
  // dF_a*rho and sum_a dF_a*G_a are taken as stencils of F*rho and J_a.
  if (loc || kc || bf) {
    XConvArgs<T> A; xc_init(A, P); xc_in(A, (const C *) s[0]);
    if (bfhd) xc_in(A, sA);
    if (loc) { xc_out(A, s[2]); xc_term(A, 0, F.k(OT_SA), KER_EVEN, (T) 1); }
    if (kc) { xc_out(A, s[3]); xc_term(A, 0, F.k(OT_F), KER_EVEN, (T) 1); }
    if (bf) { xc_out(A, s[7]); xc_term(A, bfhd ? 1 : 0, F.k(OT_VJ), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(A));
    C *sp[3]; T *dst[3]; int n = 0;
    if (loc) { sp[n] = s[2]; dst[n++] = r[R_RB]; }
    if (kc) { sp[n] = s[3]; dst[n++] = r[R_RT]; }
    if (bf) { sp[n] = s[7]; dst[n++] = r[R_A]; }
    DFT_TRY(par_for(n, [&](int i) { return F.inv(sp[i], dst[i]); }));
  }

  // pointwise 1
  {
    const T c2 = (T) otf->c2, c3 = (T) otf->c3, irs = (T) (1.0 / otf->rho_0s);
    T *rb = r[R_RB], *rt = r[R_RT], *q = r[R_Q];
    T *s0 = r[R_S0], *s1 = r[R_S1], *s2 = r[R_S2];
    T *v0 = r[R_V0], *v1 = r[R_V1], *v2 = r[R_V2], *e = r[R_E], *b0 = r[R_B0], *b1 = r[R_B1], *b2 = r[R_B2];
    const T inv2h = (T) (1.0 / (2.0 * P->step));
    const double vf = gwf ? 1.0 / (gwf->mass * 2.0 * P->step) : 0.0, deps = otf->div_epsilon;
    const bool clampv_on = src.vclamp && otf->max_veloc < (999.0 / GRID_AUTOMPS);
    const T vcap = (T) otf->max_veloc;
    // every load is issued before the first store (stores through the other
    // pointers could alias the loaded arrays, so the compiler keeps the order)
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const T b = loc ? rb[i] : (T) 0, rh = rho[i];
      C p = overwrite ? mk<T>((T) 0, (T) 0) : pot[i];
      if (base) p.x += base[i];
      T st = 0, dr[3] = { 0, 0, 0 };
      if (kc) {
        st = (T) 1 - rt[i] * irs;
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          dr[a] = (rho[ip] - rho[im]) * inv2h;
        }
      }
      T va[3] = { 0, 0, 0 };
      if (bf && vgiven) {   // given velocity (clamped as src/ot.c:494-497 when asked)
        va[0] = vin0[i]; va[1] = vin1[i]; va[2] = vin2[i];
        if (clampv_on) for (int a = 0; a < 3; a++) va[a] = clampv<T>(va[a], vcap);
      } else if (bf) {  // velocity src/ot.c:390-395
        const C pz = psi[i];
        C d[3];
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          d[a] = psi[ip] - psi[im];
        }
        T rr = pz.x * pz.x + pz.y * pz.y;             // velocity in the grid's precision
        if (rr < (T) deps) rr = (T) deps;
        const T g0 = (T) vf / rr;
        for (int a = 0; a < 3; a++) {
          T vv = g0 * (pz.x * d[a].y - pz.y * d[a].x);
          if (clampv_on) vv = clampv<T>(vv, vcap);
          va[a] = vv;
        }
      }
      // src/ot.c:557-567 (the LJ term src/ot.c:530 is in the merged linear part)
      p.x += add;
      if (loc) p.x += (c2 / (T) 2) * (b * b) + (c3 / (T) 3) * (b * b * b);
      if (hdp) p.x += hp.vhd(rh);   // Barranco penalty src/ot.c:374-378, 815-819
      pot[i] = p;
      if (loc) q[i] = (c2 * b + c3 * (b * b)) * rh;
      if (kc) {  // src/ot.c:608-612, 632-637 (rho_st itself is recomputed from rt where needed)
        s0[i] = dr[0] * st; s1[i] = dr[1] * st; s2[i] = dr[2] * st;
      }
      if (bf) {  // C, B_a inputs src/ot.c:852-888 (HD: the cut-off density rho G)
        const T rb_ = bfhd ? hp.rg(rh) : rh;
        v0[i] = va[0]; v1[i] = va[1]; v2[i] = va[2];
        e[i] = (va[2] * va[2] + va[1] * va[1] + va[0] * va[0]) * rb_;
        b0[i] = va[0] * rb_; b1[i] = va[1] * rb_; b2[i] = va[2] * rb_;
      }
    }, nb * (5 + (kc ? 4 : 0) + (bf ? 9 : 0)), "ot_pointwise_1"));
  }

  // ideal Bose gas of the thermal models (src/ot.c:402-407, 804-809): its own
  // pass, so that the other models' pointwise passes carry none of its code
  if (bose_model(otf) && (src.terms & POT_THERMAL)) {
    const BoseGas<T> bg = bose_par<T>(otf);
    DFT_TRY(launch_each((size_t) nx * ny * nz, [=] __device__(size_t i) { pot[i].x += bg.dEdRho(rho[i]); },
                        3.0 * nb, "ot_thermal"));
  }

  // forward transforms of the produced fields (independent: parallel branches)
  {
    const T *in[8]; C *sp[8]; int n = 0;
    if (loc) { in[n] = r[R_Q]; sp[n++] = s[9]; }
    if (kc) for (int a = 0; a < 3; a++) { in[n] = r[R_S0 + a]; sp[n++] = s[1 + a]; }
    if (bf) {
      in[n] = r[R_E]; sp[n++] = s[4];
      for (int a = 0; a < 3; a++) { in[n] = r[R_B0 + a]; sp[n++] = s[5 + a]; }
    }
    DFT_TRY(par_for(n, [&](int i) { return F.fwd(in[i], sp[i]); }));
  }

  // x pass 2: the KC and BF chains are independent
  auto kc_chain = [&]() -> int {
    // J_a = F s_a^ in place (src/ot.c:652)
    XConvArgs<T> B; xc_init(B, P);
    for (int a = 0; a < 3; a++) xc_in(B, (const C *) s[1 + a]);
    for (int a = 0; a < 3; a++) { xc_out(B, s[1 + a]); xc_term(B, a, F.k(OT_F), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(B));
    for (int a = 0; a < 3; a++) DFT_TRY(F.inv(s[1 + a], r[R_J0 + a]));
    return DFTGPU_OK;
  };
  auto bf_chain = [&]() -> int {   // B_a = V_j (rho v_a)^ in place (+ C = V_j (rho|v|^2)^ when clamped)
    XConvArgs<T> A; xc_init(A, P);
    for (int a = 0; a < 3; a++) xc_in(A, (const C *) s[5 + a]);
    for (int a = 0; a < 3; a++) { xc_out(A, s[5 + a]); xc_term(A, a, F.k(OT_VJ), KER_EVEN, (T) 1); }
    if (!cmerge) { xc_in(A, (const C *) s[4]); xc_out(A, s[10]); xc_term(A, 3, F.k(OT_VJ), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(A));
    if (!cmerge) DFT_TRY(F.inv(s[10], r[R_C]));
    for (int a = 0; a < 3; a++) DFT_TRY(F.inv(s[5 + a], r[R_BB0 + a]));
    return DFTGPU_OK;
  };
  if (kc && bf) DFT_TRY(par_for(2, [&](int i) { return i == 0 ? kc_chain() : bf_chain(); }));
  else if (kc) DFT_TRY(kc_chain());
  else if (bf) DFT_TRY(bf_chain());

  // pointwise 2
  if (kc || bf) {
    const T c = (T) (otf->alpha_s / (2.0 * otf->mass)), hm = (T) (-0.5 * otf->mass), cbf = (T) otf->c_bfpot;
    const T pcap = (T) otf->max_bfpot, inv2h = (T) (1.0 / (2.0 * P->step));
    const T eps = (T) otf->div_epsilon, irs = (T) (1.0 / otf->rho_0s);
    T *rt = r[R_RT], *J0 = r[R_J0], *J1 = r[R_J1], *J2 = r[R_J2], *h = r[R_H];
    T *v0 = r[R_V0], *v1 = r[R_V1], *v2 = r[R_V2], *A = r[R_A], *Cc = r[R_C], *B0 = r[R_BB0], *B1 = r[R_BB1], *B2 = r[R_BB2];
    T *wo0 = (T *) src.wout[0], *wo1 = (T *) src.wout[1], *wo2 = (T *) src.wout[2];
    const double pw2_bytes = nb * (2 + (kc ? 6 : 0) + (bf ? (cmerge ? 8 : 9) : 0));
    bool marched = false;
    if constexpr (std::is_same<T, float>::value) {   // x-marching form (ot_march.cuh)
      if (march_on() && march2_fits(nx, ny, nz)) {
        March2Args M;
        M.pot = pot; M.rho = rho; M.rt = rt; M.J0 = J0; M.J1 = J1; M.J2 = J2;
        M.v0 = v0; M.v1 = v1; M.v2 = v2; M.A = A; M.Cc = Cc; M.B0 = B0; M.B1 = B1; M.B2 = B2;
        M.h = h; M.wo0 = wo0; M.wo1 = wo1; M.wo2 = wo2;
        M.nx = nx; M.ny = ny; M.nz = nz; M.lx = 0;
        M.c = c; M.hm = hm; M.cbf = cbf; M.pcap = pcap; M.inv2h = inv2h; M.eps = eps; M.irs = irs;
        M.cmerge = cmerge; M.bfhd = bfhd; M.clampp = clampp; M.hp = hp;
        ProfScope prof("ot_pointwise_2", pw2_bytes);
        DFT_TRY(launch_march2(M, kc, bf));
        marched = true;
      }
    }
    // per-row form.  FP32: 6 CTAs per SM (42 registers, no spills) keep more
    // of its ~40 loads per element in flight; the FP64 variant would spill
    constexpr int kMinBlocks = std::is_same<T, float>::value ? 6 : 1;
    if (!marched) DFT_TRY(launch_rows_b<kMinBlocks>(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      C p = pot[i];
      T hval = 0, wv[3] = { 0, 0, 0 };   // stores last: every load is issued before them
      if (kc) {  // src/ot.c:641-645, 656-657, 673-675 summed over axes
        const T *Ja[3] = { J0, J1, J2 };
        T hv = 0, t1 = 0, jd = 0;
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          const T ja = Ja[a][i];
          hv += (rho[ip] - rho[im]) * inv2h * ja;        // (d_a rho) J_a
          t1 += (Ja[a][ip] - Ja[a][im]) * inv2h;         // dF_a * G_a = D_a J_a
          jd += ja * ((rt[ip] - rt[im]) * inv2h);        // J_a (dF_a * rho) = J_a D_a (F*rho)
        }
        const T st = (T) 1 - rt[i] * irs;   // rho_st (src/ot.c:608-612)
        p.x += c * st * t1 - c * jd;
        hval = hv;
      }
      if (bf) {
        // real part src/ot.c:895-915 (V_j*(rho|v|^2) is in the linear part unless clamped)
        const T *va[3] = { v0, v1, v2 }, *Ba[3] = { B0, B1, B2 };
        const T a = A[i];
        T vv = 0, vb = 0;
        for (int k = 0; k < 3; k++) { vv += va[k][i] * va[k][i]; vb += va[k][i] * Ba[k][i]; }
        T re = hm * (a * vv - (T) 2 * vb);
        if (!cmerge) re += hm * Cc[i];
        if (bfhd) re *= hp.drg(rho[i]);       // d(rho G)/drho  src/ot.c:907-908
        if (clampp) re = clampv<T>(re, pcap);
        p.x += re * cbf;
        // imaginary part src/ot.c:924-990 with w_a = v_a A - B_a (src/ot.c:924-931);
        // HD: the gradient of rho G, and G times the gradient of w_a (src/ot.c:934-982)
        T rr = rho[i];
        const T gw = bfhd ? hp.g(rr) : (T) 1;
        if (rr < eps) rr = eps;
        T im = 0;
        for (int k = 0; k < 3; k++) {
          int ip, imm; S.nb(x, y, z, i, k, ip, imm);
          const T w = va[k][i] * a - Ba[k][i];
          wv[k] = w;
          const T wp = va[k][ip] * A[ip] - Ba[k][ip], wm = va[k][imm] * A[imm] - Ba[k][imm];
          const T dr = bfhd ? hp.rg(rho[ip]) - hp.rg(rho[imm]) : rho[ip] - rho[imm];
          im += (T) 0.5 * ((dr * inv2h) / rr) * w + (T) 0.5 * ((wp - wm) * inv2h) * gw;
        }
        if (clampp) im = clampv<T>(im, pcap);
        p.y += im * cbf;
      }
      if (kc) h[i] = hval;
      if (bf && wo0) { wo0[i] = wv[0]; wo1[i] = wv[1]; wo2[i] = wv[2]; }   // src/ot.c:924-931
      pot[i] = p;
    }, pw2_bytes, "ot_pointwise_2"));
  }

  // merged linear part (one inverse transform):
  //   V_LJ rho^ + w q^ (src/ot.c:530, 582-585) + c F h^ (KC, src/ot.c:656-664)
  //   + c_bf (-m/2) V_j (rho|v|^2)^ (BF, src/ot.c:895-915)
  const bool linear = lj || loc || kc || cmerge;
  if (kc) DFT_TRY(F.fwd(r[R_H], s[10]));
  if (linear) {
    XConvArgs<T> A; xc_init(A, P);
    int nin = 0;
    xc_out(A, s[11]);
    if (lj) { xc_in(A, (const C *) s[0]); xc_term(A, nin++, F.k(OT_LJ), KER_EVEN, (T) 1); }
    if (loc) { xc_in(A, (const C *) s[9]); xc_term(A, nin++, F.k(OT_SA), KER_EVEN, (T) 1); }
    if (kc) { xc_in(A, (const C *) s[10]); xc_term(A, nin++, F.k(OT_F), KER_EVEN, (T) (otf->alpha_s / (2.0 * otf->mass))); }
    if (cmerge) {
      xc_in(A, (const C *) s[4]);
      xc_term(A, nin++, F.k(OT_VJ), KER_EVEN, (T) (-0.5 * otf->mass * otf->c_bfpot));
    }
    DFT_TRY(launch_xconv<T>(A));
    // P.re += linear part, P *= scale, in the store of the inverse transform
    PotAddPairStore<T> st{pot, ny, nz, scale};
    return irfft_yz<T>(s[11], st, nx, ny, nz, 3.0 * nb);
  }

  // pointwise 3 (no linear term): P *= scale
  if (scale != (T) 1) {
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      C p = pot[i];
      p.x *= scale; p.y *= scale;
      pot[i] = p;
    }, nb * 4, "ot_pointwise_3"));
  }
  return DFTGPU_OK;
}

int ot_potential(dft_ot_functional *otf, cgrid *P, wf *gwf) {
  return ot_potential_ex(otf, P, gwf, 0, nullptr, 0.0, 1.0);
}

int ot_potential_ex(dft_ot_functional *otf, cgrid *P, wf *gwf, int overwrite, rgrid *base, double add, double scale) {
  return ot_potential_src(otf, P, gwf, overwrite, base, add, scale, PotSrc());
}

int ot_potential_src(dft_ot_functional *otf, cgrid *P, wf *gwf, int overwrite, rgrid *base, double add, double scale,
                     const PotSrc &src) {
  return P->prec == DFTGPU_FP32
             ? potential_t<float>(otf, P, gwf, overwrite, base ? (const float *) base->value : nullptr, add, scale, src)
             : potential_t<double>(otf, P, gwf, overwrite, base ? (const double *) base->value : nullptr, add, scale, src);
}

// ------------------------------------------------------------------ energy density
// terms: POT_LJ | POT_LOCAL (the plain part), POT_KC, POT_BF; dens: rho grid
// to use instead of |psi|^2; add: ed += instead of ed = (the _kc / _bf entry
// points add to the plain part, src/ot-energy.c:108-109).
template <typename T> static int energy_density_t(dft_ot_functional *otf, rgrid *edg, wf *gwf, int terms,
                                                  const rgrid *dens, bool add) {
  typedef typename cplx_t<T>::type C;
  OtPriv *P = (OtPriv *) otf->priv;
  Fields<T> F{P, P->nx, P->ny, P->nz};
  const int nx = P->nx, ny = P->ny, nz = P->nz;
  const double nb = (double) nx * ny * nz * sizeof(T);   // bytes of one real field
  const bool plain = terms & (POT_LJ | POT_LOCAL);
  const bool kc = (terms & POT_KC) && (otf->model & DFT_OT_KC), bf = (terms & POT_BF) && (otf->model & DFT_OT_BACKFLOW);
  // high-density models: Barranco's energy with the plain part
  // (src/ot-energy.c:96-99), the backflow with rho G(rho) (src/ot-energy.c:221-227)
  const bool hd = hd_model(otf), hde = hd && (terms & POT_HD), bfhd = bf && hd;
  const bool bosee = bose_model(otf) && (terms & POT_THERMAL);
  const BoseGas<T> bg = bose_par<T>(otf);
  const HdPar<T> hp = hd_par<T>(otf);
  const Stencil3 S{nx, ny, nz};
  const C *psi = (const C *) gwf->grid->value;
  T *rho = (T *) otf->density->value, *ed = (T *) edg->value;
  enum { R_U, R_RB, R_RT, R_A, R_RST, R_S0, R_S1, R_S2, R_V0, R_V1, R_V2, R_E, R_B0, R_B1, R_B2, R_RG, R_NREAL };
  T *r[R_NREAL];
  for (int i = 0; i < R_NREAL; i++) { r[i] = F.r(i); if (!r[i]) return DFTGPU_ERR_NOMEM; }
  C *s[9];
  for (int i = 0; i < 9; i++) { s[i] = F.s(i); if (!s[i]) return DFTGPU_ERR_NOMEM; }

  const bool any = plain || kc || bf || hde;
  if (dens) {
    if (dens != otf->density) DFT_CUDA(cudaMemcpyAsync(rho, dens->value, nb, cudaMemcpyDeviceToDevice, rt().stream));
    if (!any) return add ? DFTGPU_OK : rfill(edg, 0.0);
    DFT_TRY(F.fwd(rho, s[0]));
  } else if (!any) {
    DFT_TRY(density(gwf->grid, otf->density));
    return add ? DFTGPU_OK : rfill(edg, 0.0);
  } else {   // rho = |psi|^2 (src/ot-energy.c:44), formed and stored by the first z pass
    DensityPairLoad<T> ld{psi, rho, ny, nz};
    DFT_TRY(rfft_zy<T>(ld, s[0], nx, ny, nz, 2.0 * nb));
  }
  T *rg = r[R_RG];   // the backflow's density: rho G(rho) (HD) or rho
  if (bfhd) {
    DFT_TRY(launch_each((size_t) nx * ny * nz, [=] __device__(size_t i) { rg[i] = hp.rg(rho[i]); }, 2.0 * nb, "ot_hd_density"));
    DFT_TRY(F.fwd(rg, s[8]));
  }
  const T *rbf = bfhd ? rg : rho;
  if (plain || kc || bf) {
    XConvArgs<T> A; xc_init(A, P); xc_in(A, (const C *) s[0]);
    if (bfhd) xc_in(A, (const C *) s[8]);
    if (plain) {
      xc_out(A, s[1]); xc_term(A, 0, F.k(OT_LJ), KER_EVEN, (T) 1);
      xc_out(A, s[2]); xc_term(A, 0, F.k(OT_SA), KER_EVEN, (T) 1);
    }
    if (kc) { xc_out(A, s[3]); xc_term(A, 0, F.k(OT_F), KER_EVEN, (T) 1); }
    if (bf) { xc_out(A, s[4]); xc_term(A, bfhd ? 1 : 0, F.k(OT_VJ), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(A));
    if (plain) {
      DFT_TRY(F.inv(s[1], r[R_U]));
      DFT_TRY(F.inv(s[2], r[R_RB]));
    }
    if (kc) DFT_TRY(F.inv(s[3], r[R_RT]));
    if (bf) DFT_TRY(F.inv(s[4], r[R_A]));
  }
  {
    const T c2 = (T) otf->c2, c3 = (T) otf->c3, irs = (T) (1.0 / otf->rho_0s), inv2h = (T) (1.0 / (2.0 * P->step));
    const T cm = (T) (otf->c_bfpot * otf->mass);
    const double vf = 1.0 / (gwf->mass * 2.0 * P->step);
    T *u = r[R_U], *rb = r[R_RB], *rt = r[R_RT], *A = r[R_A], *rst = r[R_RST], *s0 = r[R_S0], *s1 = r[R_S1], *s2 = r[R_S2];
    T *v0 = r[R_V0], *v1 = r[R_V1], *v2 = r[R_V2], *e = r[R_E], *b0 = r[R_B0], *b1 = r[R_B1], *b2 = r[R_B2];
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      const T rh = rho[i];
      T acc = add ? ed[i] : (T) 0;
      if (plain) {  // src/ot-energy.c:70-93
        const T b = rb[i];
        acc += (T) 0.5 * rh * u[i] + (c2 / (T) 2) * ((b * b) * rh) + (c3 / (T) 3) * ((b * b * b) * rh);
      }
      if (hde) acc += hp.ehd(rh);   // src/ot-energy.c:96-99
      if (bosee) acc += bg.energy(rh);   // src/ot-energy.c:101-105
      if (kc) {  // src/ot-energy.c:144-161
        const T st = rt[i] * (-irs) + (T) 1;
        rst[i] = st;
        T *sa[3] = { s0, s1, s2 };
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          sa[a][i] = (rho[ip] - rho[im]) * inv2h * st;
        }
      }
      if (bf) {  // src/ot-energy.c:231-251 (velocity regularised with DFT_EPS)
        const C pz = psi[i];
        T rr = pz.x * pz.x + pz.y * pz.y;
        if (rr < (T) DFT_EPS) rr = (T) DFT_EPS;
        const T g0 = (T) vf / rr;
        T va[3];
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          const C d = psi[ip] - psi[im];
          va[a] = g0 * (pz.x * d.y - pz.y * d.x);
        }
        v0[i] = va[0]; v1[i] = va[1]; v2[i] = va[2];
        const T vv = va[0] * va[0] + va[1] * va[1] + va[2] * va[2], rhb = rbf[i];
        acc += -(cm / (T) 4) * (A[i] * vv * rhb);
        e[i] = rhb * vv;
        b0[i] = rhb * va[0]; b1[i] = rhb * va[1]; b2[i] = rhb * va[2];
      }
      ed[i] = acc;
    }, nb * (4 + (kc ? 5 : 0) + (bf ? 10 : 0)), "ed_pointwise_1"));
  }
  if (kc) {
    for (int a = 0; a < 3; a++) DFT_TRY(F.fwd(r[R_S0 + a], s[1 + a]));
    XConvArgs<T> A; xc_init(A, P);
    for (int a = 0; a < 3; a++) xc_in(A, (const C *) s[1 + a]);
    for (int a = 0; a < 3; a++) { xc_out(A, s[1 + a]); xc_term(A, a, F.k(OT_F), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(A));
    for (int a = 0; a < 3; a++) DFT_TRY(F.inv(s[1 + a], r[R_S0 + a]));   // s_a <- F * s_a
  }
  if (bf) {
    DFT_TRY(F.fwd(r[R_E], s[4]));
    for (int a = 0; a < 3; a++) DFT_TRY(F.fwd(r[R_B0 + a], s[5 + a]));
    XConvArgs<T> A; xc_init(A, P);
    for (int a = 0; a < 4; a++) xc_in(A, (const C *) s[4 + a]);
    for (int a = 0; a < 4; a++) { xc_out(A, s[4 + a]); xc_term(A, a, F.k(OT_VJ), KER_EVEN, (T) 1); }
    DFT_TRY(launch_xconv<T>(A));
    DFT_TRY(F.inv(s[4], r[R_E]));
    for (int a = 0; a < 3; a++) DFT_TRY(F.inv(s[5 + a], r[R_B0 + a]));
  }
  if (kc || bf) {
    const T f = (T) (-otf->alpha_s / (4.0 * otf->mass)), cm = (T) (otf->c_bfpot * otf->mass);
    const T inv2h = (T) (1.0 / (2.0 * P->step));
    T *rst = r[R_RST], *t0 = r[R_S0], *t1 = r[R_S1], *t2 = r[R_S2];
    T *v0 = r[R_V0], *v1 = r[R_V1], *v2 = r[R_V2], *cc = r[R_E], *B0 = r[R_B0], *B1 = r[R_B1], *B2 = r[R_B2];
    DFT_TRY(launch_rows(nx, ny, nz, [=] __device__(int x, int y, int z, int i) {
      T acc = ed[i];
      const T rh = rho[i];
      if (kc) {  // src/ot-energy.c:176-190
        const T *ta[3] = { t0, t1, t2 };
        for (int a = 0; a < 3; a++) {
          int ip, im; S.nb(x, y, z, i, a, ip, im);
          acc += f * (ta[a][i] * ((rho[ip] - rho[im]) * inv2h) * rst[i]);
        }
      }
      if (bf) {  // src/ot-energy.c:253-287
        const T rhb = rbf[i];
        acc += (cm / (T) 2) * (B0[i] * rhb * v0[i]);
        acc += (cm / (T) 2) * (B1[i] * rhb * v1[i]);
        acc += (cm / (T) 2) * (B2[i] * rhb * v2[i]);
        acc += -(cm / (T) 4) * (cc[i] * rhb);
      }
      ed[i] = acc;
    }, nb * (3 + (kc ? 5 : 0) + (bf ? 8 : 0)), "ed_pointwise_2"));
  }
  return DFTGPU_OK;
}

int ot_energy_density(dft_ot_functional *otf, rgrid *ed, wf *gwf) {
  return ot_energy_density_terms(otf, ed, gwf, POT_ALL, nullptr, false);
}

int ot_energy_density_terms(dft_ot_functional *otf, rgrid *ed, wf *gwf, int terms, const rgrid *dens, bool add) {
  return ed->prec == DFTGPU_FP32 ? energy_density_t<float>(otf, ed, gwf, terms, dens, add)
                                 : energy_density_t<double>(otf, ed, gwf, terms, dens, add);
}

}  // namespace dftgpu
