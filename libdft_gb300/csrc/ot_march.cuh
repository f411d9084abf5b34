// Second pointwise pass of the OT potential as an x-marching stencil kernel
// (FP32): the kinetic-correlation stencil terms and the backflow real and
// imaginary parts, src/ot.c:641-675 and 895-990, with the same per-element
// arithmetic as the one-CTA-per-row form in ot.cu.
//
// The per-row form loads every stencil neighbour from L2: about 45 loads per
// element, most of them rows of other CTAs.  Here a CTA owns TY adjacent y
// rows and all nz points of each (one thread per z) and walks a run of x
// planes.  Per plane it loads each field once:
//   x neighbours  - the fields of the stencils along x (rho, F*rho, J_x and
//                   the backflow w_x = v_x A - B_x) are carried in registers
//                   from plane to plane, the next plane loaded one step ahead;
//   y neighbours  - the CTA's own rows, plus one halo row on each side;
//   z neighbours  - the neighbouring threads, through a double-buffered
//                   shared-memory plane (one barrier per x plane).
// About 20 loads per element at TY = 2, each field read once from DRAM.
#pragma once

#include "ot_work.cuh"

namespace dftgpu {

struct March2Args {
  float2 *pot;                          // potential, updated in place
  const float *rho, *rt;                // rho, F*rho
  const float *J0, *J1, *J2;            // J_a = F * G_a (KC)
  const float *v0, *v1, *v2;            // velocity (BF)
  const float *A, *Cc, *B0, *B1, *B2;   // V_j*rho, V_j*(rho|v|^2) (unmerged only), V_j*(rho v_a)
  float *h;                             // sum_a (d_a rho) J_a (KC)
  float *wo0, *wo1, *wo2;               // w_a = v_a A - B_a (BF, optional)
  int nx, ny, nz, lx;                   // lx: x planes per CTA
  float c, hm, cbf, pcap, inv2h, eps, irs;
  int cmerge, bfhd, clampp;
  HdPar<float> hp;
};

// Resident CTAs per SM the kernel is compiled for (per 256 threads): 3 for the
// full model (80 registers, no spills; unbounded it took 124 and ran 2), 4 for
// one term (56-64 registers)
constexpr int march2_minb(int nt, bool kc, bool bf) { return nt >= 512 ? 1 : (kc && bf ? 3 : 4) * (256 / nt); }

// NT threads = nz; TY rows per CTA; KC / BF: the terms present
template <int NT, int TY, bool KC, bool BF>
__global__ void __launch_bounds__(NT, march2_minb(NT, KC, BF)) march2_kernel(const March2Args a) {
  static_assert(KC || BF, "one of the terms");
  // z-exchange plane, double-buffered: rho, F*rho, J_z, w_z of each row
  __shared__ float zx[2][4][TY][NT];
  const int z = threadIdx.x, nz = a.nz, ny = a.ny, nx = a.nx;
  const int zp = z + 1 < nz ? z + 1 : 0, zm = z > 0 ? z - 1 : nz - 1;
  const int y0 = blockIdx.x * TY;
  const int xb = blockIdx.y * a.lx, xe = min(xb + a.lx, nx);
  const int yh0 = y0 > 0 ? y0 - 1 : ny - 1, yh1 = y0 + TY < ny ? y0 + TY : 0;   // halo rows
  const float inv2h = a.inv2h;
  auto at = [&](int x, int y) { return (x * ny + y) * nz + z; };

  // carried state per row: plane x-1 (m), x (c); the x+1 plane (p) is loaded each step
  float m_rho[TY], m_rt[TY], m_j[TY], m_w[TY];
  float c_rho[TY], c_rt[TY], c_j[TY], c_v[TY], c_a[TY], c_b[TY];
  {
    const int xm = xb > 0 ? xb - 1 : nx - 1;
#pragma unroll
    for (int r = 0; r < TY; r++) {
      const int im = at(xm, y0 + r), ic = at(xb, y0 + r);
      m_rho[r] = a.rho[im]; c_rho[r] = a.rho[ic];
      if (KC) { m_rt[r] = a.rt[im]; m_j[r] = a.J0[im]; c_rt[r] = a.rt[ic]; c_j[r] = a.J0[ic]; }
      if (BF) {
        m_w[r] = a.v0[im] * a.A[im] - a.B0[im];
        c_v[r] = a.v0[ic]; c_a[r] = a.A[ic]; c_b[r] = a.B0[ic];
      }
    }
  }

  int buf = 0;
  for (int x = xb; x < xe; x++, buf ^= 1) {
    const int xp = x + 1 < nx ? x + 1 : 0;
    // plane x+1 (the x neighbours of this plane, the centre of the next)
    float p_rho[TY], p_rt[TY], p_j[TY], p_v[TY], p_a[TY], p_b[TY];
#pragma unroll
    for (int r = 0; r < TY; r++) {
      const int ip = at(xp, y0 + r);
      p_rho[r] = a.rho[ip];
      if (KC) { p_rt[r] = a.rt[ip]; p_j[r] = a.J0[ip]; }
      if (BF) { p_v[r] = a.v0[ip]; p_a[r] = a.A[ip]; p_b[r] = a.B0[ip]; }
    }
    // this plane's centre-only fields
    float2 pot[TY];
    float j1[TY], j2[TY], v1[TY], v2[TY], b1[TY], b2[TY], cc[TY];
#pragma unroll
    for (int r = 0; r < TY; r++) {
      const int i = at(x, y0 + r);
      pot[r] = a.pot[i];
      if (KC) { j1[r] = a.J1[i]; j2[r] = a.J2[i]; }
      if (BF) {
        v1[r] = a.v1[i]; v2[r] = a.v2[i]; b1[r] = a.B1[i]; b2[r] = a.B2[i];
        cc[r] = a.cmerge ? 0.0f : a.Cc[i];
      }
    }
    // halo rows y0-1, y0+TY of this plane (y stencils of the edge rows)
    float h_rho[2], h_rt[2], h_j[2], h_w[2];
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const int i = at(x, s == 0 ? yh0 : yh1);
      h_rho[s] = a.rho[i];
      if (KC) { h_rt[s] = a.rt[i]; h_j[s] = a.J1[i]; }
      if (BF) h_w[s] = a.v1[i] * a.A[i] - a.B1[i];
    }
    float w1[TY], w2[TY];
#pragma unroll
    for (int r = 0; r < TY; r++) {
      if (BF) { w1[r] = v1[r] * c_a[r] - b1[r]; w2[r] = v2[r] * c_a[r] - b2[r]; }
      zx[buf][0][r][z] = c_rho[r];
      if (KC) { zx[buf][1][r][z] = c_rt[r]; zx[buf][2][r][z] = j2[r]; }
      if (BF) zx[buf][3][r][z] = w2[r];
    }
    __syncthreads();

#pragma unroll
    for (int r = 0; r < TY; r++) {
      const int i = at(x, y0 + r);
      // neighbours (ip, im) along x, y, z
      const float rho_p[3] = { p_rho[r], r + 1 < TY ? c_rho[r + 1] : h_rho[1], zx[buf][0][r][zp] };
      const float rho_m[3] = { m_rho[r], r > 0 ? c_rho[r - 1] : h_rho[0], zx[buf][0][r][zm] };
      float2 p = pot[r];
      float hval = 0.0f;
      if (KC) {  // src/ot.c:641-645, 656-657, 673-675 summed over axes
        const float ja[3] = { c_j[r], j1[r], j2[r] };
        const float j_p[3] = { p_j[r], r + 1 < TY ? j1[r + 1] : h_j[1], zx[buf][2][r][zp] };
        const float j_m[3] = { m_j[r], r > 0 ? j1[r - 1] : h_j[0], zx[buf][2][r][zm] };
        const float t_p[3] = { p_rt[r], r + 1 < TY ? c_rt[r + 1] : h_rt[1], zx[buf][1][r][zp] };
        const float t_m[3] = { m_rt[r], r > 0 ? c_rt[r - 1] : h_rt[0], zx[buf][1][r][zm] };
        float hv = 0.0f, t1 = 0.0f, jd = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; d++) {
          hv += (rho_p[d] - rho_m[d]) * inv2h * ja[d];
          t1 += (j_p[d] - j_m[d]) * inv2h;
          jd += ja[d] * ((t_p[d] - t_m[d]) * inv2h);
        }
        const float st = 1.0f - c_rt[r] * a.irs;
        p.x += a.c * st * t1 - a.c * jd;
        hval = hv;
      }
      float w[3] = { 0.0f, 0.0f, 0.0f };
      if (BF) {  // src/ot.c:895-915 (real), 924-990 (imaginary)
        const float av = c_a[r];
        const float va[3] = { c_v[r], v1[r], v2[r] }, ba[3] = { c_b[r], b1[r], b2[r] };
        float vv = 0.0f, vb = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) { vv += va[k] * va[k]; vb += va[k] * ba[k]; }
        float re = a.hm * (av * vv - 2.0f * vb);
        if (!a.cmerge) re += a.hm * cc[r];
        if (a.bfhd) re *= a.hp.drg(c_rho[r]);
        if (a.clampp) re = clampv<float>(re, a.pcap);
        p.x += re * a.cbf;
        float rr = c_rho[r];
        const float gw = a.bfhd ? a.hp.g(rr) : 1.0f;
        if (rr < a.eps) rr = a.eps;
        const float w_p[3] = { p_v[r] * p_a[r] - p_b[r], r + 1 < TY ? w1[r + 1] : h_w[1], zx[buf][3][r][zp] };
        const float w_m[3] = { m_w[r], r > 0 ? w1[r - 1] : h_w[0], zx[buf][3][r][zm] };
        float im = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const float wk = va[k] * av - ba[k];
          w[k] = wk;
          const float dr = a.bfhd ? a.hp.rg(rho_p[k]) - a.hp.rg(rho_m[k]) : rho_p[k] - rho_m[k];
          im += 0.5f * ((dr * inv2h) / rr) * wk + 0.5f * ((w_p[k] - w_m[k]) * inv2h) * gw;
        }
        if (a.clampp) im = clampv<float>(im, a.pcap);
        p.y += im * a.cbf;
      }
      if (KC) a.h[i] = hval;
      if (BF && a.wo0) { a.wo0[i] = w[0]; a.wo1[i] = w[1]; a.wo2[i] = w[2]; }
      a.pot[i] = p;
    }

    // carry: x -> x-1, x+1 -> x
#pragma unroll
    for (int r = 0; r < TY; r++) {
      m_rho[r] = c_rho[r]; c_rho[r] = p_rho[r];
      if (KC) { m_rt[r] = c_rt[r]; m_j[r] = c_j[r]; c_rt[r] = p_rt[r]; c_j[r] = p_j[r]; }
      if (BF) {
        m_w[r] = c_v[r] * c_a[r] - c_b[r];
        c_v[r] = p_v[r]; c_a[r] = p_a[r]; c_b[r] = p_b[r];
      }
    }
  }
}

// x planes per CTA: about four waves of resident CTAs, at least 4 planes
inline int march_lx(int nx, int ytiles, int resident) {
  const int want = 4 * resident;
  int chunks = (want + ytiles - 1) / ytiles;
  if (chunks > nx / 4) chunks = nx / 4;
  if (chunks < 1) chunks = 1;
  return (nx + chunks - 1) / chunks;
}

template <int NT, int TY, bool KC, bool BF> int launch_march2_t(March2Args &A) {
  auto k = march2_kernel<NT, TY, KC, BF>;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NT, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  A.lx = march_lx(A.nx, A.ny / TY, per_sm * rt().num_sms);
  dim3 grid(A.ny / TY, (A.nx + A.lx - 1) / A.lx);
  k<<<grid, NT, 0, rt().stream>>>(A);
  DFT_CHECK_LAUNCH();
  return DFTGPU_OK;
}

// whether the marching form takes this grid (else the per-row form runs)
inline bool march2_fits(int nx, int ny, int nz) {
  (void) nx;
  return (nz == 128 || nz == 256 || nz == 512) && ny % 2 == 0 && ny >= 2;
}

template <int NT> int launch_march2_nt(March2Args &A, bool kc, bool bf) {
  if (kc && bf) return launch_march2_t<NT, 2, true, true>(A);
  if (kc) return launch_march2_t<NT, 2, true, false>(A);
  return launch_march2_t<NT, 2, false, true>(A);
}

inline int launch_march2(March2Args &A, bool kc, bool bf) {
  switch (A.nz) {
    case 128: return launch_march2_nt<128>(A, kc, bf);
    case 256: return launch_march2_nt<256>(A, kc, bf);
    default: return launch_march2_nt<512>(A, kc, bf);
  }
}

}  // namespace dftgpu
