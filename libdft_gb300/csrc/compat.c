/*
 * C-only entry points of libdftgpu: the forms of the libgrid / libdft calls
 * that take or return REAL complex (C99 complex cannot cross the CUDA C++
 * translation units portably, so these wrappers split it into re, im).
 * Signatures follow the call sites in libdft's examples
 * (examples/imag_time/imag_time.c:221-239, src/helium-ot-bulk.c:331-347).
 */
#include <complex.h>
#include <stdlib.h>

#include "dftgpu.h"

void grid_wf_propagate(wf *gwf, cgrid *potential, REAL complex time) {
  dftgpu_wf_propagate(gwf, potential, creal(time), cimag(time));
}

void grid_wf_propagate_predict(wf *gwf, wf *gwfp, cgrid *potential, REAL complex time) {
  dftgpu_wf_propagate_predict(gwf, gwfp, potential, creal(time), cimag(time));
}

void grid_wf_propagate_correct(wf *gwf, cgrid *potential, REAL complex time) {
  dftgpu_wf_propagate_correct(gwf, potential, creal(time), cimag(time));
}

void grid_wf_constant(wf *gwf, REAL complex c) { grid_wf_constant_re_im(gwf, creal(c), cimag(c)); }
void cgrid_add(cgrid *grid, REAL complex c) { cgrid_add_re_im(grid, creal(c), cimag(c)); }
void cgrid_multiply(cgrid *grid, REAL complex c) { cgrid_multiply_re_im(grid, creal(c), cimag(c)); }
void cgrid_constant(cgrid *grid, REAL complex c) { cgrid_constant_re_im(grid, creal(c), cimag(c)); }

/* grid_wf_map / cgrid_map with a REAL complex callback (src/helium-ot-bulk.c:331) */
typedef REAL complex (*cmap_fn)(void *arg, REAL x, REAL y, REAL z);
struct cmap_ctx { cmap_fn f; void *arg; };

static void cmap_adapter(void *arg, REAL x, REAL y, REAL z, REAL *re, REAL *im) {
  struct cmap_ctx *c = (struct cmap_ctx *) arg;
  REAL complex v = c->f(c->arg, x, y, z);
  *re = creal(v);
  *im = cimag(v);
}

void cgrid_map(cgrid *grid, cmap_fn func, void *farg) {
  struct cmap_ctx c = { func, farg };
  cgrid_map_re_im(grid, cmap_adapter, &c);
}

void grid_wf_map(wf *gwf, cmap_fn func, void *farg) { cgrid_map(gwf->grid, func, farg); }

/* cgrid_value_at_index (src/helium-ot-bulk.c:353); NAN + NAN i on error */
REAL complex cgrid_value_at_index(cgrid *grid, INT i, INT j, INT k) {
  REAL re = NAN, im = NAN;
  cgrid_value_at_index_re_im(grid, i, j, k, &re, &im);
  return re + I * im;
}
