/*
 * libdftgpu -- GB300 (sm_103a) implementation of libdft's per-time-step hot
 * path: the Orsay-Trento (OT) potential and energy density and the
 * split-operator wave-function step, behind the call signatures libdft and
 * libgrid expose for that path.
 *
 * Grids live in GPU memory.  A grid's values are FP64 or FP32 ("bulk"
 * precision, chosen with dftgpu_set_precision() before allocation);
 * reductions (norm, energies) accumulate in FP64 and the k-space convolution
 * kernels are generated in FP64.  Host data moves only through the explicit
 * *_to_host / *_from_host copies (libgrid's CUDA mode has the same rule:
 * *_host_lock, libdft src/spectroscopy1a.c:53).
 *
 * Reference citations are paths inside jmeloranta/libdft.  libgrid functions
 * (grid_wf_*, rgrid_*, cgrid_*) are not in that tree; their citations are the
 * libdft call sites that define how they are used.
 *
 * Error convention: the drop-in entry points keep libdft's void / pointer
 * returns; a failure sets a code readable with dftgpu_last_error() (and
 * allocation returns NULL, as src/ot.c:82-85 does).  The dftgpu_* entry points
 * return the code directly.  The library never calls exit().
 */
#ifndef DFTGPU_H
#define DFTGPU_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef REAL
#define REAL double
#endif
#ifndef INT
#define INT long
#endif

/* ---------------------------------------------------------------- status */
#define DFTGPU_OK               0
#define DFTGPU_ERR_ARG          1   /* invalid argument / grid mismatch */
#define DFTGPU_ERR_SIZE         2   /* unsupported grid size */
#define DFTGPU_ERR_NOMEM        3   /* device allocation failed */
#define DFTGPU_ERR_CUDA         4   /* CUDA runtime error */
#define DFTGPU_ERR_NONFINITE    5   /* NaN / Inf detected by an FP64 reduction */
#define DFTGPU_ERR_UNSUPPORTED  6   /* model / boundary / propagator not provided */
#define DFTGPU_ERR_NODEVICE     7   /* no CUDA device */
#define DFTGPU_ERR_IO           8   /* file could not be opened, read or written */

/* precision of newly allocated grids */
#define DFTGPU_FP64 0
#define DFTGPU_FP32 1

/* -------------------------------------------------------- OT model flags
 * Same values as libdft src/ot.h:37-60.  Provided: DFT_OT_PLAIN, DFT_OT_KC,
 * DFT_OT_BACKFLOW and their combinations; the others are rejected with
 * DFTGPU_ERR_UNSUPPORTED. */
#define DFT_OT_PLAIN    0
#define DFT_OT_KC       1
#define DFT_OT_HD       2
#define DFT_OT_HD2      4
#define DFT_OT_BACKFLOW 8
#define DFT_OT_T0MK    16
#define DFT_OT_T400MK  32        /* thermal models: their parameter sets (src/ot.c:1038-1222) */
#define DFT_OT_T600MK  64        /* and the ideal Bose gas term (src/ot.c:402-407, 804-809)   */
#define DFT_OT_T800MK  128
#define DFT_OT_T1200MK 256
#define DFT_OT_T1400MK 512
#define DFT_OT_T1600MK 1024
#define DFT_OT_T1800MK 2048
#define DFT_OT_T2000MK 4096
#define DFT_OT_T2100MK 8192
#define DFT_OT_T2200MK 16384
#define DFT_OT_T2400MK 32768
#define DFT_OT_T2600MK 65536
#define DFT_OT_T2800MK 131072
#define DFT_OT_T3000MK 262144
#define DFT_GP         524288
#define DFT_DR         1048576
#define DFT_ZERO       2097152
#define DFT_GP2        4194304

/* wave-function options (libgrid; used at examples/imag_time/imag_time.c:197) */
#define WF_DIRICHLET_BOUNDARY  1
#define WF_NEUMANN_BOUNDARY    2
#define WF_PERIODIC_BOUNDARY   3
#define WF_2ND_ORDER_FFT       1
#define WF_4TH_ORDER_FFT       2
#define WF_2ND_ORDER_CN        3

#define DFT_MIN_SUBSTEPS 4      /* src/ot.h:140 */
#define DFT_MAX_SUBSTEPS 32     /* src/ot.h:141 */
#define DFT_EPS 1E-4            /* src/ot.h:147 */

/* atomic units (libgrid au.h, restated from CODATA 2018) */
#define GRID_AUTOANG   0.529177210903
#define GRID_AUTOK     3.1577502480407E5
#define GRID_AUTOFS    0.024188843265857
#define GRID_AUTOAMU   (1.0 / 1822.888486209)
#define GRID_AUTOMPS   2.18769126364E6
#define GRID_AUTOBAR   2.9421015697E8
#define DFT_HELIUM_MASS (4.002602 / GRID_AUTOAMU)   /* src/ot.h:137 */

/* ----------------------------------------------------------------- types */
typedef struct rgrid_struct rgrid;
typedef struct cgrid_struct cgrid;

/* Real grid.  value is a DEVICE pointer to nx*ny*nz values in [x][y][z]
 * order (FP32 or FP64 per prec).  Coordinates: x_i = (i - nx/2) step - x0. */
struct rgrid_struct {
  void *value;
  INT nx, ny, nz;
  REAL step;
  REAL x0, y0, z0;
  int prec;
  char id[32];
};

/* Complex grid, same layout with interleaved (re, im). */
struct cgrid_struct {
  void *value;
  INT nx, ny, nz;
  REAL step;
  REAL x0, y0, z0;
  REAL kx0, ky0, kz0;
  int prec;
  char id[32];
};

/* Wave function (libgrid wf: grid, mass, norm, boundary, propagator). */
typedef struct wf_struct {
  cgrid *grid;
  REAL mass;
  REAL norm;          /* target particle number for grid_wf_normalize() */
  char boundary;
  char propagator;
  void *priv;
} wf;

typedef struct {      /* src/dft.h:23-28 */
  REAL h, sigma, epsilon, cval;
} dft_common_lj;

typedef struct {      /* src/ot.h:69-71 */
  REAL g11, g12, g21, g22, a1, a2;
} dft_ot_bf;

/* OT functional; public fields as in src/ot.h:159-202.  The kernel and
 * workspace fields of libdft are replaced by the opaque priv state (device
 * kernel spectra and work buffers); density is kept (device grid). */
typedef struct dft_ot_functional_struct {
  INT model;
  REAL b, c2, c2_exp, c3, c3_exp, c4;
  REAL rho_0s, alpha_s, l_g, mass, rho0, temp;
  dft_common_lj lj_params;
  dft_ot_bf bf_params;
  REAL beta, rhom, C, mu0, xi, rhobf;
  REAL div_epsilon, max_veloc, max_bfpot, c_bfpot;
  rgrid *density;
  void *priv;
} dft_ot_functional;

typedef REAL (*rgrid_outside_fn)(rgrid *grid, INT i, INT j, INT k);
typedef REAL (*rgrid_map_fn)(void *arg, REAL x, REAL y, REAL z);
typedef void (*cgrid_map_fn)(void *arg, REAL x, REAL y, REAL z, REAL *re, REAL *im);

/* periodic boundary sentinel (libgrid RGRID_PERIODIC_BOUNDARY, src/ot.c:95) */
REAL rgrid_value_outside_periodic(rgrid *grid, INT i, INT j, INT k);
#define RGRID_PERIODIC_BOUNDARY rgrid_value_outside_periodic

/* ------------------------------------------------------- runtime control */
/* Select the GPU.  libgrid: cuda_enable(1, NGPUS, gpus)
 * (examples/imag_time/imag_time.c:185-189).  One GPU only: ngpus must be 1.
 * One device per process: call this before allocating any grid and do not
 * switch devices afterwards.  The FP64 reduction slots and partial sums, the
 * FFT twiddle tables and the parallel-branch streams are process-global and
 * are allocated on that device at first use; a functional's and a wave
 * function's work buffers belong to that object.  Like libgrid's CPU calls,
 * the library is not reentrant: issue all calls from one host thread, on the
 * one work stream (dftgpu_set_stream) -- two functionals or wave functions
 * stepped concurrently on different streams would race on the reduction
 * slots. */
void cuda_enable(char value, INT ngpus, int *gpus);
int dftgpu_init(int device);
/* Precision for grids allocated from now on (DFTGPU_FP64 / DFTGPU_FP32). */
int dftgpu_set_precision(int prec);
int dftgpu_get_precision(void);
/* Last error code of this thread (0 = none) and its message; clears it. */
int dftgpu_last_error(void);
const char *dftgpu_last_error_message(void);
int dftgpu_synchronize(void);
/* CUDA stream (cudaStream_t) all work is issued on; NULL = legacy default. */
int dftgpu_set_stream(void *stream);
void *dftgpu_get_stream(void);
/* Kernel profiler (no libdft counterpart; libdft times whole iterations with
 * grid_timer_*, examples/imag_time/imag_time.c:228,242).  While enabled,
 * every launch is bracketed by CUDA events on the work stream; the report is
 * JSON {"class": {"launches": n, "ms": total, "bytes": algorithmic bytes}}.
 * Enabling clears previous records.  Not usable inside graph capture. */
int dftgpu_profile(int enable);
int dftgpu_profile_report(char *buf, size_t len);

/* ------------------------------------------------------------ real grids
 * libgrid rgrid API as used by libdft (src/ot.c:95-244, ot-energy.c:59-72,
 * examples/imag_time/imag_time.c:213-253). */
rgrid *rgrid_alloc(INT nx, INT ny, INT nz, REAL step, rgrid_outside_fn value_outside, void *outside_params_ptr, char *id);
void rgrid_free(rgrid *grid);
rgrid *rgrid_clone(rgrid *grid, char *id);
void rgrid_set_origin(rgrid *grid, REAL x0, REAL y0, REAL z0);
void rgrid_zero(rgrid *grid);
void rgrid_constant(rgrid *grid, REAL c);
void rgrid_copy(rgrid *dst, rgrid *src);
void rgrid_add(rgrid *grid, REAL c);
void rgrid_multiply(rgrid *grid, REAL c);
void rgrid_sum(rgrid *dst, rgrid *a, rgrid *b);
void rgrid_product(rgrid *dst, rgrid *a, rgrid *b);
void rgrid_add_scaled(rgrid *dst, REAL c, rgrid *src);
void rgrid_add_scaled_product(rgrid *dst, REAL c, rgrid *a, rgrid *b);
/* dst = src^exponent at every point (pow; examples/soliton/soliton.c:96,
 * examples/1d-soliton/soliton-1d.c:105: the amplitude sqrt(rho)) */
void rgrid_power(rgrid *dst, rgrid *src, REAL exponent);
REAL rgrid_integral(rgrid *grid);
/* Host callback evaluated in FP64 on the host at every grid point, then copied
 * to the device (setup only; examples/imag_time/imag_time.c:218). */
void rgrid_map(rgrid *grid, rgrid_map_fn func, void *farg);
REAL rgrid_value_at_index(rgrid *grid, INT i, INT j, INT k);
/* Host copies: buffers are FP64, nx*ny*nz values in [x][y][z] order. */
int rgrid_copy_to_host(rgrid *grid, double *host);
int rgrid_copy_from_host(rgrid *grid, const double *host);
/* Raw copies in the grid's own precision (4 or 8 bytes per value). */
int rgrid_copy_to_host_raw(rgrid *grid, void *host);
int rgrid_copy_from_host_raw(rgrid *grid, const void *host);

/* --------------------------------------------------------- complex grids */
cgrid *cgrid_alloc(INT nx, INT ny, INT nz, REAL step, void *value_outside, void *outside_params_ptr, char *id);
void cgrid_free(cgrid *grid);
cgrid *cgrid_clone(cgrid *grid, char *id);
void cgrid_zero(cgrid *grid);                             /* src/helium-ot-bulk.c:335 */
void cgrid_constant_re_im(cgrid *grid, REAL re, REAL im);
void cgrid_add_re_im(cgrid *grid, REAL re, REAL im);      /* cgrid_add(P, -mu0), imag_time.c:233 */
void cgrid_multiply_re_im(cgrid *grid, REAL re, REAL im); /* cgrid_multiply(P, 0.5), imag_time.c:238 */
void cgrid_copy(cgrid *dst, cgrid *src);
/* Moving background (examples/gas-bubble/bubble.c:104,173,
 * examples/added_mass/added_mass.c:78): a wave function on this grid is
 * propagated with the kinetic operator hbar^2 |k - k0|^2 / 2m and its kinetic
 * energy is <hbar^2 |k - k0|^2 / 2m>.  Clones copy the momentum. */
void cgrid_set_momentum(cgrid *grid, REAL kx0, REAL ky0, REAL kz0);
void cgrid_map_re_im(cgrid *grid, cgrid_map_fn func, void *farg);
int cgrid_copy_to_host(cgrid *grid, double *host);        /* interleaved re, im */
int cgrid_copy_from_host(cgrid *grid, const double *host);
int cgrid_copy_to_host_raw(cgrid *grid, void *host);
int cgrid_copy_from_host_raw(cgrid *grid, const void *host);

/* grid_real_to_complex_re / grid_add_real_to_complex_re / _im
 * (imag_time.c:231,235; src/ot.c:530,990) */
void grid_real_to_complex_re(cgrid *dst, rgrid *src);
void grid_add_real_to_complex_re(cgrid *dst, rgrid *src);
void grid_add_real_to_complex_im(cgrid *dst, rgrid *src);

/* -------------------------------------------------------- wave functions
 * libgrid wf API as called by libdft and its examples. */
/* grid_wf_alloc (imag_time.c:197): periodic boundary with WF_2ND_ORDER_FFT or
 * WF_2ND_ORDER_CN (examples/gas-bubble/config.h:66).  The CN wave function
 * steps its kinetic part by Crank-Nicolson on the 3-point finite-difference
 * operator, axis by axis (x, y, z); on the periodic grid each axis factor is
 * diagonal in k, (1 - i dt Q / 4m) / (1 + i dt Q / 4m) with
 * Q = (2 sin((k - k0) h / 2) / h)^2, and is applied there.  grid_wf_energy of
 * a CN wave function uses the same finite-difference kinetic operator.
 * Dimensions 2^a 3^b 5^c in [2, 1024], x and y may be odd, z even; a 1-D grid
 * (nx = ny = 1, examples/1d-bubble/bubble-1d.c:126) takes nz up to 4096 and the
 * OT functional's 1-D effective model (src/ot.c:133-217).  Other sizes return
 * NULL with DFTGPU_ERR_SIZE (the same rule for rgrid_alloc / cgrid_alloc). */
wf *grid_wf_alloc(INT nx, INT ny, INT nz, REAL step, REAL mass, char boundary, char propagator, char *id);
wf *grid_wf_clone(wf *gwf, char *id);                     /* imag_time.c:201 */
void grid_wf_free(wf *gwf);
void grid_wf_constant_re_im(wf *gwf, REAL re, REAL im);   /* grid_wf_constant, imag_time.c:221 */
void grid_wf_density(wf *gwf, rgrid *density);            /* src/ot.c:320 */
REAL grid_wf_norm(wf *gwf);                               /* imag_time.c:254 */
REAL grid_wf_normalize(wf *gwf);                          /* examples/imag_time_rot/imag_time.c:208 */
REAL grid_wf_energy(wf *gwf, rgrid *potential);           /* kinetic (+ <V>), imag_time.c:253 */
REAL grid_wf_kinetic_energy(wf *gwf);
void grid_wf_velocity(wf *gwf, rgrid *vx, rgrid *vy, rgrid *vz, REAL eps);  /* src/ot.c:390 */
/* propagation with complex time step split into (re, im)
 * (grid_wf_propagate / _predict / _correct: imag_time.c:234,239,
 * src/helium-ot-bulk.c:340-347); the REAL complex forms are below. */
int dftgpu_wf_propagate(wf *gwf, cgrid *potential, double dt_re, double dt_im);
int dftgpu_wf_propagate_predict(wf *gwf, wf *gwfp, cgrid *potential, double dt_re, double dt_im);
int dftgpu_wf_propagate_correct(wf *gwf, cgrid *potential, double dt_re, double dt_im);

/* Absorbing boundary (libgrid; examples/gas-bubble/bubble.c:149-157,
 * examples/1d-bubble/bubble-1d.c:192): the layer of grid points outside
 * [lx, hx) x [ly, hy) x [lz, hz) absorbs, with a weight lambda that rises
 * linearly from 0 at the layer's inner edge to 1 at the grid's edge.  Set on
 * gwf and, when given, gwfp.  From then on the predict / correct steps of that
 * wave function (grid_wf_propagate_predict / _correct, dftgpu_pc_step,
 * dftgpu_run) add -i amp lambda (|psi|^2 / rho0 - 1), evaluated from the step's
 * input, to their potential, which drives the density in the layer towards
 * rho0.  libgrid's own arithmetic is not in the reference tree: this form is
 * this library's.  The adjoint entry points refuse a wave function that has a
 * boundary (DFTGPU_ERR_UNSUPPORTED). */
void grid_wf_boundary(wf *gwf, wf *gwfp, REAL amp, REAL rho0, INT lx, INT hx, INT ly, INT hy, INT lz, INT hz);
/* potential += -i amp lambda (|psi|^2 / rho0 - 1) over gwf's absorbing layer
 * (examples/1d-bubble/bubble-1d.c:222; single-step callers, whose
 * grid_wf_propagate does not add it). */
void grid_wf_absorb_potential(wf *gwf, cgrid *potential, REAL amp, REAL rho0);

/* Allocation-free form of dftgpu_wf_propagate (no counterpart in the
 * reference: libgrid allocates its own work grids).  For callers that may not
 * call cudaMalloc -- code running inside someone else's stream capture, hosts
 * whose memory pool owns all device memory, services that must not grow after
 * start-up.  The caller passes device pointers it owns: psi_in and potential
 * (nx*ny*nz interleaved complex values of precision prec, [x][y][z] order) and
 * psi_out (same size; may equal psi_in); one step psi_out = S(V, dt) psi_in on
 * `stream` (NULL = legacy default stream), with the FFT propagator's kinetic
 * step and no moving background.  Work memory is a static 32 MiB
 * device array plus twiddle tables, held by every GPU that loads the library
 * until exit: grids up to 2,097,152 points in FP64 or 4,194,304 in FP32;
 * larger ones are rejected with DFTGPU_ERR_SIZE.  All calls share that array
 * (overlapping calls on the GPU race); the first call on a device resolves
 * its address and should come before any stream capture. */
int dftgpu_wf_propagate_noalloc(void *psi_out, const void *psi_in, const void *potential, INT nx, INT ny, INT nz,
                                REAL step, REAL mass, double dt_re, double dt_im, int prec, void *stream);

/* ---------------------------------------------------------- OT functional */
/* src/ot.c:66.  Models: PLAIN, KC, HD, HD2, BACKFLOW and the thermal sets
 * T0MK..T3000MK (combinations as in libdft); GP and DR get NULL with
 * DFTGPU_ERR_UNSUPPORTED.  On a 1-D grid (nx = ny = 1) the 1-D effective kernels. */
dft_ot_functional *dft_ot_alloc(INT model, wf *gwf, INT min_substeps, INT max_substeps);
void dft_ot_free(dft_ot_functional *otf);                                                   /* src/ot.c:268 */
void dft_ot_potential(dft_ot_functional *otf, cgrid *potential, wf *gwf);                    /* src/ot.c:314 */
void dft_ot_energy_density(dft_ot_functional *otf, rgrid *energy_density, wf *gwf);         /* src/ot-energy.c:38 */
/* The potential from a given density and velocity field instead of a wave
 * function (src/ot.c:431).  With backflow the velocity grids are clamped to
 * max_veloc and overwritten with w_a = v_a (V_j*rho) - V_j*(rho v_a), as the
 * reference does (src/ot.c:494-497, 924-931). */
void dft_ot_potential2(dft_ot_functional *otf, cgrid *potential, rgrid *density, rgrid *veloc_x,
                       rgrid *veloc_y, rgrid *veloc_z);                                    /* src/ot.c:431 */
/* Single terms, added to potential from the given density (src/ot.c:524, 547,
 * 840; "usually not called directly").  The workspace / rho_tf arguments are
 * accepted for signature compatibility and not used: the library keeps its
 * spectra in its own work buffers, so rho_tf does not receive FFT(rho). */
void dft_ot_add_lennard_jones_potential(dft_ot_functional *otf, cgrid *potential, rgrid *density,
                                        rgrid *workspace1, rgrid *workspace2);             /* src/ot.c:524 */
void dft_ot_add_local_correlation_potential(dft_ot_functional *otf, cgrid *potential, rgrid *rho,
                                            rgrid *rho_tf, rgrid *workspace1,
                                            rgrid *workspace2);                            /* src/ot.c:547 */
void dft_ot_backflow_potential(dft_ot_functional *otf, cgrid *potential, rgrid *density, rgrid *veloc_x,
                               rgrid *veloc_y, rgrid *veloc_z, rgrid *workspace1, rgrid *workspace2,
                               rgrid *workspace3, rgrid *workspace4, rgrid *workspace5,
                               rgrid *workspace6);                                         /* src/ot.c:840 */
/* KC and backflow parts of the energy density, added to energy_density, with
 * the given density (src/ot-energy.c:123, 202). */
void dft_ot_energy_density_kc(dft_ot_functional *otf, rgrid *energy_density, wf *gwf,
                              rgrid *density);                                             /* src/ot-energy.c:123 */
void dft_ot_energy_density_bf(dft_ot_functional *otf, rgrid *energy_density, wf *gwf,
                              rgrid *density);                                             /* src/ot-energy.c:202 */
void dft_ot_init_params(dft_ot_functional *otf, INT model);                                 /* src/ot.c:1002 */
/* Regenerate the k-space kernels after changing otf parameters such as l_g
 * (src/ot.c:138-217 run again); libdft has no separate entry for this. */
int dft_ot_update_kernels(dft_ot_functional *otf, INT min_substeps, INT max_substeps);

/* Inspection: the k-space kernel `which` (0 LJ, 1 spherical average, 2 F,
 * 3-5 dF/dx,dy,dz, 6 V_j) as stored: the non-negative octant
 * [kz][kx][ky] (extents nz/2+1, nx/2+1, ny/2+1) of its spectrum (real part;
 * imaginary part for dF), times (-1)^(kx+ky+kz) step^3/N (LJ and the
 * spherical average additionally rescaled to integrals b and 1, src/ot.c:160,181).
 * host receives FP64 values.  No libdft counterpart (libdft keeps the full
 * spectra in otf->lennard_jones etc., src/ot.h:174-180). */
int dftgpu_ot_kernel(dft_ot_functional *otf, int which, double *host);
/* Inspection: unnormalised forward r2c 3-D FFT of a real grid, written to
 * host as nx*ny*(nz/2+1) complex values in [x][y][kz] order (libgrid
 * rgrid_fft, src/ot.c:527, but out of place). */
int dftgpu_rgrid_spectrum(rgrid *grid, double *host);

/* bulk liquid relations, host-only (src/helium-ot-bulk.c:21-434) */
REAL dft_ot_bulk_energy(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_dEdRho(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_pressure(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_dPdRho(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_density_pressurized(dft_ot_functional *otf, REAL pressure);
REAL dft_ot_bulk_chempot_pressurized(dft_ot_functional *otf, REAL pressure);
REAL dft_ot_bulk_density(dft_ot_functional *otf);
REAL dft_ot_bulk_chempot(dft_ot_functional *otf);
REAL dft_ot_bulk_chempot2(dft_ot_functional *otf);
REAL dft_ot_bulk_compressibility(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_sound_speed(dft_ot_functional *otf, REAL rho);
REAL dft_ot_bulk_dispersion(dft_ot_functional *otf, REAL *k, REAL rho0);
REAL dft_ot_bulk_chempot3(dft_ot_functional *otf, REAL rho0);                 /* src/helium-ot-bulk.c:128 */
/* -1/X(k) of the uniform liquid (src/helium-ot-bulk.c:445); as there, k below
 * 0.01 bohr^-1 returns 0.01. */
REAL dft_ot_bulk_istatic(dft_ot_functional *otf, REAL *k, REAL rho0);

/* ------------------------------------------- driver compatibility
 * Names libdft's example drivers take from libgrid's <grid/grid.h> and
 * <grid/au.h> and from libdft's <dft/dft.h> besides the entry points above.
 * include/grid/grid.h, grid/au.h, dft/dft.h and dft/ot.h include this file,
 * so a driver builds with its own #include lines and -I<repo>/include. */
#define HBAR           1.0                    /* atomic units */
#define GRID_AUTOM     0.529177210903E-10     /* bohr -> m (CODATA 2018) */
#define GRID_AUTOS     2.4188843265857E-17    /* a.u. time -> s */
#define GRID_AUTOPA    2.9421015697E13        /* a.u. pressure -> Pa */
#define GRID_AUKB      (1.0 / GRID_AUTOK)     /* Boltzmann constant, hartree / K */
#define GRID_HZTOCM1   3.33564095198152E-11   /* Hz -> cm^-1 (1 / c in cm/s) */
#define FMT_R "%le"
#define FMT_I "%ld"

typedef struct {      /* src/dft.h:55-60 */
  REAL kx, ky, kz;    /* wave vector */
  REAL a;             /* relative amplitude */
  REAL rho;           /* background density */
} dft_plane_wave;

/* 1-D potential tables read from "r value" text files (src/dft.h:16-54):
 * equidistant r from begin in steps of step, length values. */
#define DFT_MAX_POTENTIAL_POINTS 8192
typedef struct extpot {
  REAL points[DFT_MAX_POTENTIAL_POINTS];
  REAL begin;
  INT length;
  REAL step;
} dft_extpot;
/* tables along x, y, z, averaging mode (0 none, 1 xy, 2 yz, 3 xz, 4 all),
 * orientation (theta0, phi0) and origin of the mapped potential */
typedef struct extpot_set {
  dft_extpot *x, *y, *z;
  char average;
  REAL theta0, phi0;
  REAL x0, y0, z0;
} dft_extpot_set;
/* Read a table (src/common.c:541-576).  Where libdft exits, this records
 * DFTGPU_ERR_IO (file not readable) or DFTGPU_ERR_ARG (distances decreasing or
 * not equidistant) and leaves the table as read so far. */
void dft_common_read_pot(char *file, dft_extpot *pot);
/* rgrid_map callback of a dft_extpot_set (src/common.c:588-668). */
REAL dft_common_extpot(void *arg, REAL x, REAL y, REAL z);
/* Read the three tables and map them onto potential (src/common.c:689-709);
 * nothing is mapped if a table cannot be read. */
void dft_common_potential_map(char average, char *filex, char *filey, char *filez, rgrid *potential, REAL theta0,
                              REAL phi0, REAL x0, REAL y0, REAL z0);

/* Wall-clock and CPU timer (examples/imag_time/imag_time.c:228,242). */
typedef struct grid_timer_struct {
  double wall0, cpu0;
} grid_timer;
void grid_timer_start(grid_timer *timer);
REAL grid_timer_wall_clock_time(grid_timer *timer);   /* seconds since grid_timer_start */
REAL grid_timer_cpu_time(grid_timer *timer);

/* FFTW planning and host threads (examples/imag_time/imag_time.c:192-194,226):
 * accepted and ignored -- the GPU transforms need no plans or wisdom and the
 * host does no grid arithmetic. */
void grid_set_fftw_flags(INT flags);
void grid_threads_init(INT threads);
void grid_fft_read_wisdom(char *file);
void grid_fft_write_wisdom(char *file);

/* Map callbacks of libdft (src/common.c, src/initial.c) for rgrid_map /
 * cgrid_map / grid_wf_map: host functions, same arguments and values. */
REAL dft_common_lj_func(REAL r2, REAL sig, REAL eps);                      /* src/common.c:31 */
REAL dft_common_lennard_jones(void *arg, REAL x, REAL y, REAL z);          /* src/common.c:53 (dft_common_lj *) */
REAL dft_common_lennard_jones_smooth(void *arg, REAL x, REAL y, REAL z);   /* src/common.c:104 */
/* the 1-D forms (integrated over the x-y plane, for grids along z) */
REAL dft_common_lennard_jones_1d(void *arg, REAL x, REAL y, REAL z);       /* src/common.c:80 */
REAL dft_common_spherical_avg_1d(void *arg, REAL x, REAL y, REAL z);       /* src/common.c:152 */
REAL dft_common_gaussian_1d(void *arg, REAL x, REAL y, REAL z);            /* src/common.c:214 */
REAL dft_common_spherical_avg(void *arg, REAL x, REAL y, REAL z);          /* src/common.c:131 (REAL *radius) */
REAL dft_common_spherical_avg_k(void *arg, REAL kx, REAL ky, REAL kz);     /* src/common.c:173 */
REAL dft_common_gaussian(void *arg, REAL x, REAL y, REAL z);               /* src/common.c:193 (REAL *inv_width) */
REAL dft_common_vortex_x(void *param, REAL x, REAL y, REAL z);             /* src/common.c:1240 (REAL *mass) */
REAL dft_common_vortex_y(void *param, REAL x, REAL y, REAL z);             /* src/common.c:1260 */
REAL dft_common_vortex_z(void *param, REAL x, REAL y, REAL z);             /* src/common.c:1280 */

/* Grid files.  <base>.grd holds the whole grid (FP64, with its shape, step,
 * origin and, for complex grids, momentum); <base>.x, .y, .z are text cuts
 * along each axis through (nx/2, ny/2, nz/2): "coordinate value" lines
 * (complex: "coordinate re im").  The file names follow libdft's drivers
 * (examples/imag_time/imag_time.c:248-250, examples/imag_time/Makefile:16);
 * the .grd layout is this library's own, written out below, because
 * libgrid's is not part of libdft -- files written by libgrid are refused
 * (DFTGPU_ERR_UNSUPPORTED).  Writers take a base name and add the
 * extensions; readers take the file's whole name, as libdft's drivers pass it
 * (argv[1] = "bubble-100.grd", examples/gas-bubble/bubble.c:143; a renamed
 * copy, "restart.chk", examples/electron/electron.c:163): a name that is an
 * existing regular file is read as it is, any other as <name>.grd.  Reading
 * requires the grid's shape (DFTGPU_ERR_SIZE otherwise) and sets its values,
 * origin and momentum; an FP32 grid receives the values rounded to FP32.
 *   .grd layout, little-endian: char magic[8] = "DFTGPUG1"; int64 kind
 *   (0 real, 1 complex); int64 nx, ny, nz; double step, x0, y0, z0, kx0,
 *   ky0, kz0; then nx*ny*nz doubles (complex: re, im pairs) in [x][y][z]
 *   order. */
void rgrid_write_grid(char *base, rgrid *grid);            /* examples/imag_time/imag_time.c:248 */
void cgrid_write_grid(char *base, cgrid *grid);            /* examples/imag_time/imag_time.c:250 */
void rgrid_read_grid(rgrid *grid, char *file);             /* examples/added_mass_viscosity/added_mass2.c:368 */
void cgrid_read_grid(cgrid *grid, char *file);             /* examples/added_mass/added_mass.c:111 */
/* The same on host buffers (nx*ny*nz FP64 values, complex interleaved):
 * meta = { step, x0, y0, z0, kx0, ky0, kz0 }.  Return a DFTGPU_* code. */
int dftgpu_grid_file_write(const char *base, int is_complex, INT nx, INT ny, INT nz, const double *meta,
                           const double *values);
int dftgpu_grid_file_read(const char *name, int is_complex, INT nx, INT ny, INT nz, double *meta, double *values);
/* The .grd layout on a stream the caller opened and closes (a checkpoint read
 * as libdft's 1-D drivers do: fopen(argv[1]); cgrid_read(gwf->grid, fp),
 * examples/1d-bubble/bubble-1d.c:164-170, examples/1d-soliton/soliton-1d.c:93-99).
 * A NULL grid is allocated with the file's shape and step (in the current
 * precision; tmp = cgrid_read(NULL, fp), examples/vortex-trace/trace.c:155);
 * a given grid must have the file's shape.  A body of the other
 * kind (a real grid's body read by cgrid_read) is refused with DFTGPU_ERR_ARG:
 * how libgrid would turn a density into a wave function is not in the
 * reference tree.  The read functions return the grid, or NULL with the error
 * recorded. */
cgrid *cgrid_read(cgrid *grid, FILE *in);
rgrid *rgrid_read(rgrid *grid, FILE *in);
void cgrid_write(cgrid *grid, FILE *out);
void rgrid_write(rgrid *grid, FILE *out);
/* one value of a complex grid (cgrid_value_at_index; indices wrap periodically) */
int cgrid_value_at_index_re_im(cgrid *grid, INT i, INT j, INT k, REAL *re, REAL *im);

/* ----------------------------------------------- fused step and reports */
/* One predict-correct step exactly as the libdft dynamics examples write it
 * (examples/imag_time/imag_time.c:231-239):
 *   P = Vext; P += V_OT[psi]; P -= mu0; psi_p = S(P,dt) psi;
 *   P += Vext; P += V_OT[psi_p]; P -= mu0; P *= 1/2; psi = S(P,dt) psi.
 * vext may be NULL (zero).  P is left holding the averaged potential. */
int dftgpu_pc_step(dft_ot_functional *otf, wf *gwf, wf *gwfp, cgrid *potential, rgrid *vext,
                   double mu0, double dt_re, double dt_im);
/* nsteps predict-correct steps; if renorm != 0, grid_wf_normalize(gwf) after
 * each (examples/imag_time_rot/imag_time.c:208).  The loop is captured once
 * in a CUDA graph and replayed. */
int dftgpu_run(dft_ot_functional *otf, wf *gwf, wf *gwfp, cgrid *potential, rgrid *vext,
               double mu0, double dt_re, double dt_im, INT nsteps, int renorm);
/* E = <T> + int eps[psi] + int rho Vext, N = int |psi|^2 and the chemical
 * potential mu = (<T> + int rho (V_OT + Vext)) / N, all FP64
 * (examples/imag_time/imag_time.c:251-257).  vext may be NULL. */
int dftgpu_energy_report(dft_ot_functional *otf, wf *gwf, rgrid *vext, double *energy,
                         double *natoms, double *mu);

/* ---- Reverse mode (no reference counterpart: libdft has no adjoint) ----
 * Cotangent convention: for a real objective J, the cotangent of a complex
 * field psi is g = 2 dJ/dpsi^* (dJ = Re sum conj(g) dpsi); the cotangent of a
 * complex potential V is gamma with dJ = sum Re(gamma) dRe V + Im(gamma) dIm V.
 * Sums run over grid points.  Backflow with max_veloc / max_bfpot limits or
 * c_bfpot != 1 is not differentiated (DFTGPU_ERR_UNSUPPORTED). */
/* grad_psi += (d dft_ot_potential / d psi)^H cot (vector-Jacobian product of
 * the OT potential, src/ot.c:296, with respect to the wave function). */
int dftgpu_ot_potential_vjp(dft_ot_functional *otf, wf *gwf, cgrid *cot, cgrid *grad_psi);
/* Adjoint of psi_out = S(pot, dt) psi_in (grid_wf_propagate, libgrid wf
 * propagation): cot_in = S^H cot_out (cot_in may alias cot_out), cot_pot +=
 * dJ/dpot.  psi_out must hold S(pot, dt) psi_in. */
int dftgpu_wf_propagate_vjp(wf *gwf, cgrid *pot, double dt_re, double dt_im, cgrid *psi_in,
                            cgrid *psi_out, cgrid *cot_out, cgrid *cot_in, cgrid *cot_pot);
/* Adjoint of one dftgpu_pc_step from psi = gwf (unchanged), followed by
 * grid_wf_normalize when renorm: on entry cot is the cotangent of the step's
 * output, on return that of its input; grad_vext (may be NULL) += dJ/dVext. */
int dftgpu_pc_step_vjp(dft_ot_functional *otf, wf *gwf, rgrid *vext, double mu0, double dt_re,
                       double dt_im, int renorm, cgrid *cot, rgrid *grad_vext);
/* J = int (|psi_T|^2 - rho_target)^2 dV after nsteps predict-correct steps
 * from psi_0 = gwf (gwf is left at psi_T, as dftgpu_run), and its gradient
 * with respect to every Vext grid value (grad_vext, overwritten) and psi_0
 * (grad_psi0, cotangent convention above); either may be NULL.  The reverse
 * sweep recomputes each segment of checkpoint_every steps from a stored
 * checkpoint (0: ceil(sqrt(nsteps))), holding about 2 sqrt(nsteps) wave
 * functions on the device.  With both gradients NULL only the forward
 * sweep and J are computed. */
int dftgpu_adjoint_run(dft_ot_functional *otf, wf *gwf, rgrid *vext, double mu0, double dt_re,
                       double dt_im, INT nsteps, int renorm, INT checkpoint_every,
                       rgrid *rho_target, double *J, rgrid *grad_vext, cgrid *grad_psi0);

#ifndef __cplusplus
#include <complex.h>
#include <math.h>
#include <stdlib.h>
/* libgrid's math names for REAL = double, as libdft's drivers use them */
#define SQRT(x) sqrt(x)
#define EXP(x) exp(x)
#define POW(x, y) pow(x, y)
#define FABS(x) fabs(x)
#define SIN(x) sin(x)
#define COS(x) cos(x)
#define TAN(x) tan(x)
#define TANH(x) tanh(x)
#define LOG(x) log(x)
#define ACOS(x) acos(x)
#define ASIN(x) asin(x)
#define ATAN(x) atan(x)
#define ATAN2(y, x) atan2(y, x)
#define CEXP(x) cexp(x)
#define CABS(x) cabs(x)
#define CREAL(x) creal(x)
#define CIMAG(x) cimag(x)
#define CARG(x) carg(x)
#define CONJ(x) conj(x)
#define CSQRT(x) csqrt(x)
#define ABS(x) labs(x)

/* REAL complex forms of the libgrid / libdft entry points (C only). */
void grid_wf_propagate(wf *gwf, cgrid *potential, REAL complex time);
void grid_wf_propagate_predict(wf *gwf, wf *gwfp, cgrid *potential, REAL complex time);
void grid_wf_propagate_correct(wf *gwf, cgrid *potential, REAL complex time);
void grid_wf_constant(wf *gwf, REAL complex c);
void cgrid_add(cgrid *grid, REAL complex c);
void cgrid_multiply(cgrid *grid, REAL complex c);
void cgrid_constant(cgrid *grid, REAL complex c);
void cgrid_map(cgrid *grid, REAL complex (*func)(void *arg, REAL x, REAL y, REAL z), void *farg);
void grid_wf_map(wf *gwf, REAL complex (*func)(void *arg, REAL x, REAL y, REAL z), void *farg);  /* src/helium-ot-bulk.c:331 */
REAL complex cgrid_value_at_index(cgrid *grid, INT i, INT j, INT k);  /* src/helium-ot-bulk.c:353 */

/* complex map callbacks of libdft (src/common.c, src/initial.c) */
REAL complex dft_common_cgaussian(void *arg, REAL x, REAL y, REAL z);       /* src/common.c:235 (REAL *inv_width) */
REAL complex dft_common_planewave(void *arg, REAL x, REAL y, REAL z);       /* src/common.c:1214 (dft_plane_wave *) */
REAL complex dft_initial_vortex_x_n1(void *na, REAL x, REAL y, REAL z);     /* src/initial.c:31 */
REAL complex dft_initial_vortex_y_n1(void *na, REAL x, REAL y, REAL z);     /* src/initial.c:51 */
REAL complex dft_initial_vortex_z_n1(void *na, REAL x, REAL y, REAL z);     /* src/initial.c:71 */
REAL complex dft_initial_vortex_x_n2(void *na, REAL x, REAL y, REAL z);     /* src/initial.c:91 */
REAL complex dft_initial_vortex_y_n2(void *na, REAL x, REAL y, REAL z);     /* src/initial.c:112 */
REAL complex dft_initial_vortex_z_n2(void *na, REAL x, REAL y, REAL z);     /* src/initial.c:133 */
REAL complex dft_initial_bubble(void *prm, REAL x, REAL y, REAL z);         /* src/initial.c:154 (REAL *radius) */

/* Drivers of libdft built on the entry points above (src/helium-ot-bulk.c):
 * the period of a small density wave of wave vector k (rounded to the grid)
 * propagated from the plane wave of amplitude amp, as an energy in hartree
 * (k is updated to the value used; pred selects predict-correct steps; dir 0,
 * 1, 2 = x, y, z) -- src/helium-ot-bulk.c:274; and the surface tension of a
 * slab of the given width relaxed with time step ts -- src/helium-ot-bulk.c:486.
 * Where the reference calls exit(1) (bad direction, one point along it),
 * these record DFTGPU_ERR_ARG and return NAN. */
REAL dft_ot_dispersion(wf *gwf, dft_ot_functional *otf, REAL ts, REAL *k, REAL amp, char pred, char dir);
REAL dft_ot_bulk_surface_tension(wf *gwf, dft_ot_functional *otf, REAL ts, REAL width);
#endif

#ifdef __cplusplus
}
#endif
#endif
