// Private state of a GPU OT functional.
#pragma once

#include "common.cuh"

namespace dftgpu {

enum { OT_LJ = 0, OT_SA = 1, OT_F = 2, OT_FX = 3, OT_FY = 4, OT_FZ = 5, OT_VJ = 6, OT_NKER = 7 };
constexpr int OT_MAX_REAL = 80;
constexpr int OT_MAX_SPEC = 12;

struct OtPriv {
  int prec = DFTGPU_FP64;
  int nx = 0, ny = 0, nz = 0;
  double step = 0, x0 = 0, y0 = 0, z0 = 0;
  size_t oct_n = 0;                 // (nz/2+1)(nx/2+1)(ny/2+1)
  void *ker[OT_NKER] = {};          // octant spectra, bulk precision
  void *real[OT_MAX_REAL] = {};     // nx*ny*nz real work fields
  void *spec[OT_MAX_SPEC] = {};     // (nz/2+1)*nx*ny complex half spectra
  cgrid *pot_tmp = nullptr;         // energy report scratch
  rgrid *ed_tmp = nullptr;
  void *adj = nullptr;              // adjoint work state (adjoint.cu)
};

void *dev_alloc(size_t bytes);

inline void *ot_real(OtPriv *P, int i) {
  if (!P->real[i]) P->real[i] = dev_alloc((size_t) P->nx * P->ny * P->nz * elem_size(P->prec));
  return P->real[i];
}
inline void *ot_spec(OtPriv *P, int i) {
  if (!P->spec[i]) P->spec[i] = dev_alloc((size_t) (P->nz / 2 + 1) * P->nx * P->ny * 2 * elem_size(P->prec));
  return P->spec[i];
}

// Terms of the OT potential and the sources of rho and v (default: every
// term of the model, rho and v from the wave function).
// POT_HD: Barranco penalty; POT_THERMAL: the ideal Bose gas of the thermal models
enum { POT_LJ = 1, POT_LOCAL = 2, POT_KC = 4, POT_BF = 8, POT_HD = 16, POT_THERMAL = 32, POT_ALL = 63 };
struct PotSrc {
  int terms = POT_ALL;
  const void *dens = nullptr;                      // rho grid (bulk precision) instead of |psi|^2
  const void *vel[3] = { nullptr, nullptr, nullptr };   // velocity grids instead of the psi stencil
  void *wout[3] = { nullptr, nullptr, nullptr };   // receive w_a = v_a A - B_a (BF)
  bool vclamp = true;                              // apply max_veloc to the velocities
};

int ot_generate_kernels(dft_ot_functional *otf, int min_ns, int max_ns);
int ot_potential(dft_ot_functional *otf, cgrid *P, wf *gwf);
int ot_potential_ex(dft_ot_functional *otf, cgrid *P, wf *gwf, int overwrite, rgrid *base, double add, double scale);
int ot_potential_src(dft_ot_functional *otf, cgrid *P, wf *gwf, int overwrite, rgrid *base, double add, double scale,
                     const PotSrc &src);
int ot_energy_density(dft_ot_functional *otf, rgrid *ed, wf *gwf);
int ot_energy_density_terms(dft_ot_functional *otf, rgrid *ed, wf *gwf, int terms, const rgrid *dens, bool add);
void adj_free(OtPriv *P);

}  // namespace dftgpu
