// Host-side parts of libdft's drivers around the time step: grid files
// (rgrid_write_grid / cgrid_read_grid ...) and the two libdft drivers that
// run the time step themselves, dft_ot_dispersion and
// dft_ot_bulk_surface_tension (src/helium-ot-bulk.c:274-369, 486-518).  Both
// drivers are written on the library's public entry points, so every step they
// take is the GPU step the rest of the library provides.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <string>
#include <vector>

#include "grid_internal.cuh"

using namespace dftgpu;

namespace {

const char kMagic[8] = { 'D', 'F', 'T', 'G', 'P', 'U', 'G', '1' };

struct File {
  FILE *f;
  explicit File(const std::string &path, const char *mode) : f(fopen(path.c_str(), mode)) {}
  ~File() { if (f) fclose(f); }
  int close() { int rc = f ? fclose(f) : 0; f = nullptr; return rc; }
};

// The file a read takes: libdft's drivers write with a base name (the
// writer adds .grd, examples/gas-bubble/bubble.c:182) and read with the
// file's whole name, often renamed ("restart.chk", examples/electron/electron.c:163;
// "liquid_input", examples/added_mass/added_mass.c:111 and its README).  A
// name that is an existing regular file is read as it is, any other as
// <name>.grd.
std::string read_path(const char *name) {
  struct stat st;
  if (stat(name, &st) == 0 && S_ISREG(st.st_mode)) return std::string(name);
  return std::string(name) + ".grd";
}

// "coordinate value" lines along each axis through (nx/2, ny/2, nz/2)
int write_cuts(const std::string &base, int cplx, const INT n[3], const double *meta, const double *v) {
  static const char *ext[3] = { ".x", ".y", ".z" };
  for (int a = 0; a < 3; a++) {
    File out(base + ext[a], "w");
    if (!out.f) { set_error(DFTGPU_ERR_IO, "grid file: cannot open %s%s", base.c_str(), ext[a]); return DFTGPU_ERR_IO; }
    INT at[3] = { n[0] / 2, n[1] / 2, n[2] / 2 };
    for (INT i = 0; i < n[a]; i++) {
      at[a] = i;
      const size_t idx = ((size_t) at[0] * n[1] + at[1]) * n[2] + at[2];
      const double c = (double) (i - n[a] / 2) * meta[0] - meta[1 + a];
      if (cplx) fprintf(out.f, "%le %le %le\n", c, v[2 * idx], v[2 * idx + 1]);
      else fprintf(out.f, "%le %le\n", c, v[idx]);
    }
    if (out.close()) { set_error(DFTGPU_ERR_IO, "grid file: write error on %s%s", base.c_str(), ext[a]); return DFTGPU_ERR_IO; }
  }
  return DFTGPU_OK;
}

bool dims_ok(INT nx, INT ny, INT nz) { return nx > 0 && ny > 0 && nz > 0; }

// The .grd body on an open stream: magic, kind, shape, the 7 meta values
// (step, origin, momentum), then the values.
bool write_body(FILE *f, int is_complex, INT nx, INT ny, INT nz, const double *meta, const double *values) {
  const size_t count = (size_t) nx * ny * nz * (is_complex ? 2 : 1);
  const int64_t head[4] = { is_complex ? 1 : 0, (int64_t) nx, (int64_t) ny, (int64_t) nz };
  return fwrite(kMagic, 1, 8, f) == 8 && fwrite(head, sizeof(int64_t), 4, f) == 4 &&
         fwrite(meta, sizeof(double), 7, f) == 7 && fwrite(values, sizeof(double), count, f) == count;
}

struct GrdHead {
  int64_t kind, nx, ny, nz;
  double meta[7];
};

// magic, kind, shape and meta of a .grd body; `what` names the source in messages
int read_head(FILE *f, const char *what, GrdHead *h) {
  char magic[8];
  int64_t head[4];
  if (fread(magic, 1, 8, f) != 8 || memcmp(magic, kMagic, 8) != 0) {
    set_error(DFTGPU_ERR_UNSUPPORTED, "grid file: %s is not in this library's grid layout", what);
    return DFTGPU_ERR_UNSUPPORTED;
  }
  if (fread(head, sizeof(int64_t), 4, f) != 4 || fread(h->meta, sizeof(double), 7, f) != 7) {
    set_error(DFTGPU_ERR_IO, "grid file: %s truncated", what);
    return DFTGPU_ERR_IO;
  }
  h->kind = head[0]; h->nx = head[1]; h->ny = head[2]; h->nz = head[3];
  return DFTGPU_OK;
}

// the body's kind and shape against the grid it is read into
int check_head(const GrdHead &h, const char *what, int is_complex, INT nx, INT ny, INT nz) {
  if (h.kind != (is_complex ? 1 : 0)) {
    set_error(DFTGPU_ERR_ARG, "grid file: %s holds a %s grid", what, h.kind ? "complex" : "real");
    return DFTGPU_ERR_ARG;
  }
  if (h.nx != nx || h.ny != ny || h.nz != nz) {
    set_error(DFTGPU_ERR_SIZE, "grid file: %s is %lldx%lldx%lld, the grid %ldx%ldx%ld", what, (long long) h.nx,
              (long long) h.ny, (long long) h.nz, (long) nx, (long) ny, (long) nz);
    return DFTGPU_ERR_SIZE;
  }
  return DFTGPU_OK;
}

int read_vals(FILE *f, const char *what, size_t count, double *values) {
  if (fread(values, sizeof(double), count, f) != count) {
    set_error(DFTGPU_ERR_IO, "grid file: %s truncated", what);
    return DFTGPU_ERR_IO;
  }
  return DFTGPU_OK;
}

// A driver checks the error state of the void entry points it calls: it
// sets a pending error aside on entry and puts it back on exit if the driver
// itself recorded none.
struct ErrorScope {
  int saved;
  ErrorScope() : saved(g_last_error) { g_last_error = 0; }
  ~ErrorScope() { if (!g_last_error) g_last_error = saved; }
};
int pending_error() { return g_last_error; }

}  // namespace

extern "C" {

int dftgpu_grid_file_write(const char *base, int is_complex, INT nx, INT ny, INT nz, const double *meta,
                           const double *values) {
  if (!base || !meta || !values || !dims_ok(nx, ny, nz)) {
    set_error(DFTGPU_ERR_ARG, "dftgpu_grid_file_write: argument");
    return DFTGPU_ERR_ARG;
  }
  const INT n[3] = { nx, ny, nz };
  {
    File out(std::string(base) + ".grd", "wb");
    if (!out.f) { set_error(DFTGPU_ERR_IO, "grid file: cannot open %s.grd", base); return DFTGPU_ERR_IO; }
    bool ok = write_body(out.f, is_complex, nx, ny, nz, meta, values);
    ok = (out.close() == 0) && ok;
    if (!ok) { set_error(DFTGPU_ERR_IO, "grid file: write error on %s.grd", base); return DFTGPU_ERR_IO; }
  }
  return write_cuts(base, is_complex, n, meta, values);
}

int dftgpu_grid_file_read(const char *name, int is_complex, INT nx, INT ny, INT nz, double *meta, double *values) {
  if (!name || !meta || !values || !dims_ok(nx, ny, nz)) {
    set_error(DFTGPU_ERR_ARG, "dftgpu_grid_file_read: argument");
    return DFTGPU_ERR_ARG;
  }
  const std::string path = read_path(name);
  const char *pn = path.c_str();
  File in(path, "rb");
  if (!in.f) { set_error(DFTGPU_ERR_IO, "grid file: cannot open %s", pn); return DFTGPU_ERR_IO; }
  GrdHead h;
  DFT_TRY(read_head(in.f, pn, &h));
  DFT_TRY(check_head(h, pn, is_complex, nx, ny, nz));
  memcpy(meta, h.meta, sizeof(h.meta));
  DFT_TRY(read_vals(in.f, pn, (size_t) nx * ny * nz * (is_complex ? 2 : 1), values));
  return DFTGPU_OK;
}

void rgrid_write_grid(char *base, rgrid *g) {
  if (!g) { set_error(DFTGPU_ERR_ARG, "rgrid_write_grid: NULL grid"); return; }
  std::vector<double> h(gsize(g));
  if (rgrid_copy_to_host(g, h.data()) != DFTGPU_OK) return;
  const double meta[7] = { g->step, g->x0, g->y0, g->z0, 0.0, 0.0, 0.0 };
  dftgpu_grid_file_write(base, 0, g->nx, g->ny, g->nz, meta, h.data());
}

void cgrid_write_grid(char *base, cgrid *g) {
  if (!g) { set_error(DFTGPU_ERR_ARG, "cgrid_write_grid: NULL grid"); return; }
  std::vector<double> h(2 * gsize(g));
  if (cgrid_copy_to_host(g, h.data()) != DFTGPU_OK) return;
  const double meta[7] = { g->step, g->x0, g->y0, g->z0, g->kx0, g->ky0, g->kz0 };
  dftgpu_grid_file_write(base, 1, g->nx, g->ny, g->nz, meta, h.data());
}

void rgrid_read_grid(rgrid *g, char *file) {
  if (!g) { set_error(DFTGPU_ERR_ARG, "rgrid_read_grid: NULL grid"); return; }
  std::vector<double> h(gsize(g));
  double meta[7];
  if (dftgpu_grid_file_read(file, 0, g->nx, g->ny, g->nz, meta, h.data()) != DFTGPU_OK) return;
  if (rgrid_copy_from_host(g, h.data()) != DFTGPU_OK) return;
  rgrid_set_origin(g, meta[1], meta[2], meta[3]);
}

void cgrid_read_grid(cgrid *g, char *file) {
  if (!g) { set_error(DFTGPU_ERR_ARG, "cgrid_read_grid: NULL grid"); return; }
  std::vector<double> h(2 * gsize(g));
  double meta[7];
  if (dftgpu_grid_file_read(file, 1, g->nx, g->ny, g->nz, meta, h.data()) != DFTGPU_OK) return;
  if (cgrid_copy_from_host(g, h.data()) != DFTGPU_OK) return;
  g->x0 = meta[1]; g->y0 = meta[2]; g->z0 = meta[3];
  cgrid_set_momentum(g, meta[4], meta[5], meta[6]);
}

cgrid *cgrid_read(cgrid *g, FILE *in) {
  const char *what = "cgrid_read stream";
  if (!in) { set_error(DFTGPU_ERR_ARG, "cgrid_read: NULL stream"); return nullptr; }
  GrdHead h;
  if (read_head(in, what, &h) != DFTGPU_OK) return nullptr;
  cgrid *made = nullptr;
  if (!g) {
    if (h.kind != 1) { set_error(DFTGPU_ERR_ARG, "grid file: %s holds a real grid", what); return nullptr; }
    made = g = cgrid_alloc((INT) h.nx, (INT) h.ny, (INT) h.nz, h.meta[0], nullptr, nullptr, (char *) "cgrid_read");
    if (!g) return nullptr;
  }
  std::vector<double> v;
  if (check_head(h, what, 1, g->nx, g->ny, g->nz) == DFTGPU_OK) {
    v.resize(2 * gsize(g));
    if (read_vals(in, what, v.size(), v.data()) == DFTGPU_OK && cgrid_copy_from_host(g, v.data()) == DFTGPU_OK) {
      g->x0 = h.meta[1]; g->y0 = h.meta[2]; g->z0 = h.meta[3];
      cgrid_set_momentum(g, h.meta[4], h.meta[5], h.meta[6]);
      return g;
    }
  }
  cgrid_free(made);
  return nullptr;
}

rgrid *rgrid_read(rgrid *g, FILE *in) {
  const char *what = "rgrid_read stream";
  if (!in) { set_error(DFTGPU_ERR_ARG, "rgrid_read: NULL stream"); return nullptr; }
  GrdHead h;
  if (read_head(in, what, &h) != DFTGPU_OK) return nullptr;
  rgrid *made = nullptr;
  if (!g) {
    if (h.kind != 0) { set_error(DFTGPU_ERR_ARG, "grid file: %s holds a complex grid", what); return nullptr; }
    made = g = rgrid_alloc((INT) h.nx, (INT) h.ny, (INT) h.nz, h.meta[0], nullptr, nullptr, (char *) "rgrid_read");
    if (!g) return nullptr;
  }
  std::vector<double> v;
  if (check_head(h, what, 0, g->nx, g->ny, g->nz) == DFTGPU_OK) {
    v.resize(gsize(g));
    if (read_vals(in, what, v.size(), v.data()) == DFTGPU_OK && rgrid_copy_from_host(g, v.data()) == DFTGPU_OK) {
      rgrid_set_origin(g, h.meta[1], h.meta[2], h.meta[3]);
      return g;
    }
  }
  rgrid_free(made);
  return nullptr;
}

void cgrid_write(cgrid *g, FILE *out) {
  if (!g || !out) { set_error(DFTGPU_ERR_ARG, "cgrid_write: NULL argument"); return; }
  std::vector<double> v(2 * gsize(g));
  if (cgrid_copy_to_host(g, v.data()) != DFTGPU_OK) return;
  const double meta[7] = { g->step, g->x0, g->y0, g->z0, g->kx0, g->ky0, g->kz0 };
  if (!write_body(out, 1, g->nx, g->ny, g->nz, meta, v.data())) set_error(DFTGPU_ERR_IO, "cgrid_write: write error");
}

void rgrid_write(rgrid *g, FILE *out) {
  if (!g || !out) { set_error(DFTGPU_ERR_ARG, "rgrid_write: NULL argument"); return; }
  std::vector<double> v(gsize(g));
  if (rgrid_copy_to_host(g, v.data()) != DFTGPU_OK) return;
  const double meta[7] = { g->step, g->x0, g->y0, g->z0, 0.0, 0.0, 0.0 };
  if (!write_body(out, 0, g->nx, g->ny, g->nz, meta, v.data())) set_error(DFTGPU_ERR_IO, "rgrid_write: write error");
}

// ------------------------------------------------------------ potentials from files

// Table of "r value" pairs, equidistant in r (src/common.c:541-576): the
// first two distances fix begin and step; a later distance more than step/10
// off its place is refused.
static int read_pot(const char *file, dft_extpot *pot) {
  if (!file || !pot) { set_error(DFTGPU_ERR_ARG, "dft_common_read_pot: NULL argument"); return DFTGPU_ERR_ARG; }
  File in(file, "r");
  if (!in.f) { set_error(DFTGPU_ERR_IO, "dft_common_read_pot: cannot open %s", file); return DFTGPU_ERR_IO; }
  double begin = 0.0, step = 0.0, r = 0.0, prev;
  INT n;
  int rc = DFTGPU_OK;
  for (n = 0; n < DFT_MAX_POTENTIAL_POINTS; n++) {
    prev = r;
    if (fscanf(in.f, " %le %le", &r, &pot->points[n]) != 2) break;
    if (n == 0) {
      begin = r;
    } else if (n == 1) {
      step = r - begin;
      if (step < 0.0) { rc = DFTGPU_ERR_ARG; set_error(rc, "dft_common_read_pot: %s: distances decrease", file); break; }
    } else if (fabs(r - prev - step) > step / 10.0) {
      rc = DFTGPU_ERR_ARG;
      set_error(rc, "dft_common_read_pot: %s: distances not equidistant at line %ld", file, (long) n + 1);
      break;
    }
  }
  pot->begin = begin;
  pot->length = n;
  pot->step = step;
  return rc;
}

// value of one table at distance r: the entry below r, the first entry
// inside the table's start, 0 beyond its end (src/common.c:606-631)
static double table_at(const dft_extpot *t, double r) {
  const INT i = (INT) ((r - t->begin) / t->step);
  if (i < 0) return t->points[0];
  if (i > t->length - 1) return 0.0;
  return t->points[i];
}

// The three tables combined by direction: sin^2(theta) (cos^2(phi) V_x +
// sin^2(phi) V_y) + cos^2(theta) V_z about the rotated axes, or their
// averages (src/common.c:633-660)
static double extpot(const dft_extpot_set *set, double x, double y, double z) {
  x -= set->x0;
  y -= set->y0;
  z -= set->z0;
  const double r = sqrt(x * x + y * y + z * z);
  double px = table_at(set->x, r), py = table_at(set->y, r), pz = table_at(set->z, r), tmp;
  switch (set->average) {
    case 1: tmp = (px + py) / 2.0; px = py = tmp; break;
    case 2: tmp = (py + pz) / 2.0; py = pz = tmp; break;
    case 3: tmp = (px + pz) / 2.0; px = pz = tmp; break;
    case 4: return (px + py + pz) / 3.0;
    default: break;
  }
  const double theta = acos(z / (r + 1E-3)) - set->theta0, phi = atan(y / (x + 1E-3)) - set->phi0;
  double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
  st *= st; ct *= ct; sp *= sp; cp *= cp;
  return px * st * cp + py * st * sp + pz * ct;
}

void dft_common_read_pot(char *file, dft_extpot *pot) { read_pot(file, pot); }

REAL dft_common_extpot(void *arg, REAL x, REAL y, REAL z) { return extpot((const dft_extpot_set *) arg, x, y, z); }

void dft_common_potential_map(char average, char *filex, char *filey, char *filez, rgrid *potential, REAL theta0,
                              REAL phi0, REAL x0, REAL y0, REAL z0) {
  if (!potential) { set_error(DFTGPU_ERR_ARG, "dft_common_potential_map: NULL grid"); return; }
  std::vector<dft_extpot> t(3);
  dft_extpot_set set = { &t[0], &t[1], &t[2], average, theta0, phi0, x0, y0, z0 };
  fprintf(stderr, "libdft: Mapping potential file with x = %s, y = %s, z = %s. Average = %d - ", filex ? filex : "",
          filey ? filey : "", filez ? filez : "", (int) average);
  if (read_pot(filex, set.x) || read_pot(filey, set.y) || read_pot(filez, set.z)) {
    fprintf(stderr, "not mapped.\n");
    return;
  }
  rgrid_map(potential, dft_common_extpot, &set);
  fprintf(stderr, "done.\n");
}

// ------------------------------------------------------------ drivers

// sqrt(rho) (1 + a cos(k.r)) as a (re, im) map (dft_common_planewave)
static void plane_wave_map(void *arg, REAL x, REAL y, REAL z, REAL *re, REAL *im) {
  const dft_plane_wave *p = (const dft_plane_wave *) arg;
  const REAL amp = sqrt(p->rho);
  *re = amp + p->a * amp * cos(p->kx * x + p->ky * y + p->kz * z);
  *im = 0.0;
}

// Steps until the density at the grid centre has swung through half a period
// of the density wave (src/helium-ot-bulk.c:333-355).  libdft loops without
// limit; this stops after kMaxSteps (1e6) with DFTGPU_ERR_NONFINITE.
REAL dft_ot_dispersion(wf *gwf, dft_ot_functional *otf, REAL ts, REAL *k, REAL amp, char pred, char dir) {
  const long kMaxSteps = 1000000;
  ErrorScope errors;
  if (!gwf || !otf || !k) { set_error(DFTGPU_ERR_ARG, "dft_ot_dispersion: NULL argument"); return NAN; }
  cgrid *g = gwf->grid;
  const INT n[3] = { g->nx, g->ny, g->nz };
  if (dir < 0 || dir > 2 || n[(int) dir] == 1) {
    set_error(DFTGPU_ERR_ARG, "dft_ot_dispersion: direction %d is not 0, 1 or 2 with more than one point", (int) dir);
    return NAN;
  }
  // the wave vector rounded to the grid (src/helium-ot-bulk.c:290-324)
  const REAL dk = 2.0 * M_PI / (((REAL) n[(int) dir]) * g->step);
  dft_plane_wave wave = { 0.0, 0.0, 0.0, amp, otf->rho0 };
  const REAL kk = ((REAL) ((INT) (0.5 + *k / dk))) * dk;
  *k = kk;
  if (kk == 0.0) return 0.0;
  if (dir == 0) wave.kx = kk;
  else if (dir == 1) wave.ky = kk;
  else wave.kz = kk;

  const REAL rho0 = otf->rho0, mu0 = dft_ot_bulk_chempot2(otf);
  wf *gwfp = pred ? grid_wf_clone(gwf, (char *) "gwfp for dft_ot_dispersion") : nullptr;
  cgrid *pot = cgrid_clone(g, (char *) "potential for dft_ot_dispersion");
  REAL omega = NAN;
  if ((pred && !gwfp) || !pot) goto done;
  cgrid_map_re_im(g, plane_wave_map, &wave);
  {
    REAL ival = 0.0;
    long l;
    grid_timer timer;
    for (l = 0; l < kMaxSteps; l++) {
      grid_timer_start(&timer);
      cgrid_zero(pot);
      if (pred) {
        cgrid_copy(gwfp->grid, g);
        dft_ot_potential(otf, pot, gwf);
        cgrid_add_re_im(pot, -mu0, 0.0);
        dftgpu_wf_propagate_predict(gwf, gwfp, pot, ts, 0.0);
        dft_ot_potential(otf, pot, gwfp);
        cgrid_add_re_im(pot, -mu0, 0.0);
        cgrid_multiply_re_im(pot, 0.5, 0.0);
        dftgpu_wf_propagate_correct(gwf, pot, ts, 0.0);
      } else {
        dft_ot_potential(otf, pot, gwf);
        dftgpu_wf_propagate(gwf, pot, ts, 0.0);
      }
      REAL re, im;
      if (cgrid_value_at_index_re_im(g, n[0] / 2, n[1] / 2, n[2] / 2, &re, &im) != DFTGPU_OK || pending_error()) goto done;
      fprintf(stderr, "Iteration %ld - Wall clock time = %le seconds.\n", l, grid_timer_wall_clock_time(&timer));
      ival += pow(hypot(re, im), 2.0) - rho0;
      if (!(ival == ival)) { set_error(DFTGPU_ERR_NONFINITE, "dft_ot_dispersion: density at the centre is not finite"); goto done; }
      if (ival < 0.0) {
        l--;
        break;
      }
    }
    if (l >= kMaxSteps) {
      set_error(DFTGPU_ERR_NONFINITE, "dft_ot_dispersion: no half period within %ld steps", kMaxSteps);
      goto done;
    }
    // src/helium-ot-bulk.c:357-360: 1 / (2 l ts), in K via cm^-1, back to hartree
    const REAL ts_fs = ts * GRID_AUTOFS;
    const REAL w = (1.0 / (2.0 * ((REAL) l) * ts_fs / GRID_AUTOFS));
    omega = (w / GRID_AUTOS) * GRID_HZTOCM1 * 1.439 / GRID_AUTOK;
  }
done:
  if (pot) cgrid_free(pot);
  if (gwfp) grid_wf_free(gwfp);
  return omega;
}

// 1 inside the slab |x| < width / 2, 0 outside (src/helium-ot-bulk.c:471-477)
static void slab_map(void *arg, REAL x, REAL y, REAL z, REAL *re, REAL *im) {
  (void) y; (void) z;
  *re = fabs(x) < *(const REAL *) arg / 2.0 ? 1.0 : 0.0;
  *im = 0.0;
}

// Relax a slab of liquid with time step ts until the energy per surface area
// of its two faces changes by less than 3 % between steps (src/helium-ot-bulk.c:486-518).
// The slab's width is passed to the map; libdft passes NULL there
// (src/helium-ot-bulk.c:499), which would read through a null pointer.
REAL dft_ot_bulk_surface_tension(wf *gwf, dft_ot_functional *otf, REAL ts, REAL width) {
  const long kMaxSteps = 1000000;
  ErrorScope errors;
  if (!gwf || !otf || !otf->density) { set_error(DFTGPU_ERR_ARG, "dft_ot_bulk_surface_tension: NULL argument"); return NAN; }
  cgrid *g = gwf->grid;
  const REAL rho0 = otf->rho0, step = g->step, mu0 = dft_ot_bulk_chempot2(otf);
  cgrid *pot = cgrid_clone(g, (char *) "Surface tension potential");
  rgrid *density = rgrid_clone(otf->density, (char *) "Surface tension density");
  REAL stens = NAN;
  if (pot && density) {
    cgrid_map_re_im(g, slab_map, &width);
    cgrid_multiply_re_im(g, sqrt(rho0), 0.0);
    REAL prev = 1E11;
    long i;
    for (i = 1; i <= kMaxSteps; i++) {
      cgrid_zero(pot);
      dft_ot_potential(otf, pot, gwf);
      cgrid_add_re_im(pot, -mu0, 0.0);
      dftgpu_wf_propagate(gwf, pot, ts, 0.0);
      dft_ot_energy_density(otf, density, gwf);
      const REAL e = grid_wf_energy(gwf, nullptr) + rgrid_integral(density);
      if (pending_error()) { stens = NAN; break; }
      stens = e / (2.0 * ((REAL) g->ny) * ((REAL) g->nz) * step * step);
      if (fabs(stens - prev) / stens < 0.03) break;
      prev = stens;
    }
    if (i > kMaxSteps) {
      set_error(DFTGPU_ERR_NONFINITE, "dft_ot_bulk_surface_tension: not converged within %ld steps", kMaxSteps);
      stens = NAN;
    }
  }
  if (pot) cgrid_free(pot);
  if (density) rgrid_free(density);
  return stens;
}

}  // extern "C"
