// Internal grid helpers shared by grid.cu, ot.cu and api.cu.
#pragma once

#include "common.cuh"

namespace dftgpu {

inline size_t gsize(const rgrid *g) { return (size_t) g->nx * g->ny * g->nz; }
inline size_t gsize(const cgrid *g) { return (size_t) g->nx * g->ny * g->nz; }

// Absorbing boundary of a wave function (grid_wf_boundary): the layer outside
// [lx, hx) x [ly, hy) x [lz, hz) (grid indices) with the weight
// lambda = max over the axes of the linear ramp from 0 at the inner edge to 1
// at the grid's edge, and the potential -i amp lambda (|psi|^2 / rho0 - 1).
struct AbsBoundary {
  int on = 0;
  double amp = 0, rho0 = 0;
  int lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
};

struct WfPriv {
  void *spec = nullptr;        // nx*ny*nz complex spectral scratch
  AbsBoundary abs;
  cgrid *vtot = nullptr;       // potential plus the absorbing term (predict-correct steps)
};

// dst = pot + (-i) amp lambda (|psi|^2 / rho0 - 1) over the boundary layer
// (dst may be pot); grid.cu
int absorb_add(cgrid *dst, const cgrid *pot, const cgrid *psi, const AbsBoundary &b, double amp, double rho0);
// The predict / correct propagation: S(V + V_abs(src)) when the wave function
// has an absorbing boundary, else S(V)
int propagate_pc(wf *g, cgrid *dst, cgrid *src, cgrid *V, double dr, double di);

void *dev_alloc(size_t bytes);
void dev_free(void *p);
int check_dims(INT nx, INT ny, INT nz);

inline void *wf_spec(wf *g) {
  WfPriv *p = (WfPriv *) g->priv;
  if (!p->spec) p->spec = dev_alloc(gsize(g->grid) * 2 * elem_size(g->grid->prec));
  return p->spec;
}

// x pencils of a spectral buffer [kz][x][y] as plain lines: line (kz, y), element x
template <typename T> struct SpecLineXT {
  typename cplx_t<T>::type *spec; int nx, ny;
  __device__ typename cplx_t<T>::type operator()(int kz, int y, int x) const {
    return spec[((size_t) kz * nx + x) * ny + y];
  }
  __device__ void operator()(int kz, int y, int x, typename cplx_t<T>::type v) const {
    spec[((size_t) kz * nx + x) * ny + y] = v;
  }
};

int propagate(wf *g, cgrid *dst, cgrid *src, cgrid *V, double dr, double di);
int kinetic_energy(wf *g, double *out);
int norm_dev(cgrid *c, double *slot);
int scale_by_norm(cgrid *c, const double *slot, double target);
int velocity(wf *g, rgrid *vx, rgrid *vy, rgrid *vz, double eps);
int copy_values_out(int prec, const void *dev, double *host, size_t n);
int copy_values_in(int prec, void *dev, const double *host, size_t n);
int rfill(rgrid *g, double v);
int raxpb(rgrid *g, double a, double b);
int cfill(cgrid *g, double re, double im);
int cmuladd(cgrid *g, double mr, double mi, double ar, double ai);
int real_to_complex(cgrid *d, rgrid *s, int mode);
int rbinary(rgrid *d, rgrid *a, rgrid *b, double c, int op);
int rpower(rgrid *d, rgrid *s, double e);
int rintegral(rgrid *g, double *out);
int density(cgrid *c, rgrid *d);
int rspectrum(rgrid *g, double *host);
int prof_enable(int on);
int prof_report(char *buf, size_t len);
int rho_dot_re(rgrid *rho, cgrid *P, double *out);   // sum rho Re(P) dV
// DFTGPU_ERR_CUDA (with a message) if a fused plane pass's barrier wait timed
// out since the last call (fft.cu); synchronous.
int fused_zy_fault();

}  // namespace dftgpu
