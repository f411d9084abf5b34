"""CPU: what libdft's example drivers need around the time step.

* The map callbacks of libdft's src/common.c and src/initial.c exported by
  libdftgpu give the same bits as libdft's own build of those files (the
  reference-built oracle), on a lattice of points and on the core radii.
* The host-only bulk relations added for the drivers (dft_ot_bulk_istatic,
  dft_ot_bulk_chempot3) and the semi-analytic dispersion agree with libdft's
  own build for the three provided models.
* libdft's example drivers compile UNMODIFIED against include/ (their own
  #include <grid/grid.h> ... lines) and link against libdftgpu.so.
* The grid-file layout round-trips and is refused when foreign, truncated or
  of another shape.

The comparisons with libdft's own code need the reference tree and are
skipped where it is absent.  No GPU is used.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import REF_LIB, REF_ROOT, Grids, Oracle, ref_available

LIBDIR = os.path.join(ROOT, "libdft_gb300")
LIB = os.path.join(LIBDIR, "libdftgpu.so")
INCLUDE = os.path.join(ROOT, "include")
REF_EXAMPLES = os.path.join(REF_ROOT, "examples")

needs_ref = pytest.mark.skipif(not ref_available(), reason="reference tree not present")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from libdft_gb300.build import build
        build()
    return C.CDLL(LIB)


@pytest.fixture(scope="module")
def ref():
    return Oracle("ref")


@needs_ref
def test_map_callbacks_bit_identical_to_libdft(lib, ref, tmp_path):
    exe = tmp_path / "callback_parity"
    subprocess.run(["gcc", "-std=gnu11", "-O2", os.path.join(ROOT, "tests", "c", "callback_parity.c"),
                    "-o", str(exe), "-ldl", "-lm"], check=True)
    r = subprocess.run([str(exe), LIB, REF_LIB], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 differ" in r.stdout and int(r.stdout.split()[1]) > 50000


def ot_params(lib, model):
    import libdft_gb300 as G
    p = G.OTParams()
    p.model = model          # dft_ot_alloc sets the model before the parameters (src/ot.c:81,91)
    lib.dft_ot_init_params.argtypes = [C.c_void_p, C.c_long]
    lib.dft_ot_init_params(C.byref(p), model)
    return p


@needs_ref
@pytest.mark.parametrize("model", [0, 1, 8, 9, 16, 32, 32 | 9, 256 | 1, 4096, 262144 | 8])
def test_functional_parameters_bit_identical_to_libdft(lib, ref, model):
    """dft_ot_init_params: every public parameter in atomic units equals the
    value libdft's own conversion gives (src/ot.c:1002-1270)."""
    from oracle import PARAM_NAMES
    p = ot_params(lib, model)
    with Grids(ref, (8, 8, 8), 1.0, 4.002602 / ref.AUTOAMU) as g:
        w = g.wf()
        o = g.ot(model, w)
        out = np.zeros(len(PARAM_NAMES))
        ref.lib.orc_ot_params(C.c_void_p(o), out.ctypes.data_as(C.POINTER(C.c_double)))
    for n, v in zip(PARAM_NAMES, out):
        assert getattr(p, n) == v, (n, getattr(p, n), v)


@needs_ref
@pytest.mark.parametrize("model", [0, 1, 9])
def test_bulk_response_matches_libdft(lib, ref, model):
    p = ot_params(lib, model)
    R = ref.lib
    for name in ("dft_ot_bulk_istatic", "dft_ot_bulk_dispersion"):
        for L in (lib, R):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_double]
    for L in (lib, R):
        L.dft_ot_bulk_chempot3.restype = C.c_double
        L.dft_ot_bulk_chempot3.argtypes = [C.c_void_p, C.c_double]
    with Grids(ref, (8, 8, 8), 1.0, 4.002602 / ref.AUTOAMU) as g:
        w = g.wf()
        o = g.ot(model, w)
        rho0 = p.rho0
        for k in (0.005, 0.05, 0.3, 1.0, 1.9):
            for name in ("dft_ot_bulk_istatic", "dft_ot_bulk_dispersion"):
                ka, kb = C.c_double(k), C.c_double(k)
                a = getattr(lib, name)(C.byref(p), C.byref(ka), rho0)
                b = getattr(R, name)(o, C.byref(kb), rho0)
                assert a == b, (name, model, k, a, b)
        for rho in (0.5 * rho0, rho0, 1.5 * rho0):
            assert lib.dft_ot_bulk_chempot3(C.byref(p), rho) == R.dft_ot_bulk_chempot3(o, rho)


# libdft example drivers that build against this library as they are
# (the others use libgrid internals -- wf->cworkspace, otf->workspace1 -- or
# libgrid functions outside the time step; the design notes list them)
DRIVERS = ["imag_time/imag_time.c", "dynamics/dynamics.c", "dispersion/dispersion.c",
           "dispersion/dispersion2.c", "dispersion/dispersion3.c", "dispersion/static-resp.c",
           "bulk/bulk_properties.c", "piston/piston.c", "shock/shock.c", "1d-bubble/bubble-1d.c",
           "1d-soliton/soliton-1d.c", "soliton/soliton.c", "added_mass_viscosity/analyze4.c"]


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLES), reason="reference tree not present")
@pytest.mark.parametrize("driver", DRIVERS)
def test_libdft_driver_builds_unmodified(lib, tmp_path, driver):
    src = os.path.join(REF_EXAMPLES, driver)
    exe = tmp_path / "driver"
    r = subprocess.run(["gcc", "-std=gnu11", "-O2", "-w", "-I", os.path.dirname(src), "-I", INCLUDE, src,
                        "-o", str(exe), "-L", LIBDIR, "-ldftgpu", "-lm", "-Wl,-rpath," + LIBDIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


class ExtPot(C.Structure):
    """dft_extpot (libdft src/dft.h:32-37; include/dftgpu.h)"""
    _fields_ = [("points", C.c_double * 8192), ("begin", C.c_double), ("length", C.c_long), ("step", C.c_double)]


class ExtPotSet(C.Structure):
    _fields_ = [("x", C.POINTER(ExtPot)), ("y", C.POINTER(ExtPot)), ("z", C.POINTER(ExtPot)), ("average", C.c_char),
                ("theta0", C.c_double), ("phi0", C.c_double), ("x0", C.c_double), ("y0", C.c_double),
                ("z0", C.c_double)]


def pot_file(path, begin, step, n, seed, jitter=0.0):
    rng = np.random.default_rng(seed)
    r = begin + step * np.arange(n) + jitter * rng.standard_normal(n)
    v = 1e-3 * np.exp(-r / 3.0) * (1 + 0.1 * rng.standard_normal(n))
    with open(path, "w") as f:
        for a, b in zip(r, v):
            f.write("%.9g %.9g\n" % (a, b))
    return str(path).encode()


@needs_ref
def test_potential_tables_and_map_callback_bit_identical_to_libdft(lib, ref, tmp_path):
    """dft_common_read_pot and the dft_common_extpot map of
    dft_common_potential_map (src/common.c:541-709) against libdft's build,
    for the five averaging modes, with and without rotation and shift."""
    files = [pot_file(tmp_path / ("p%d.dat" % i), b, s, n, i)
             for i, (b, s, n) in enumerate([(1.0, 0.05, 400), (0.5, 0.1, 150), (2.0, 0.02, 2049)])]
    tabs = {}
    for name, L in (("gpu", lib), ("ref", ref.lib)):
        L.dft_common_read_pot.argtypes = [C.c_char_p, C.POINTER(ExtPot)]
        L.dft_common_extpot.restype = C.c_double
        L.dft_common_extpot.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        tabs[name] = [ExtPot() for _ in files]
        for f, t in zip(files, tabs[name]):
            L.dft_common_read_pot(f, C.byref(t))
    for a, b in zip(tabs["gpu"], tabs["ref"]):
        assert (a.begin, a.length, a.step) == (b.begin, b.length, b.step)
        assert bytes(a.points) == bytes(b.points)
    pts = np.random.default_rng(7).uniform(-30, 30, size=(2000, 3))
    pts[:5] = [[0, 0, 0], [1, 0, 0], [0, 0, 2.5], [-0.001, 0, 0], [0, -3, 0]]
    for avg in range(5):
        for orient in ((0.0, 0.0, 0.0, 0.0, 0.0), (0.4, -1.1, 1.5, -2.0, 0.25)):
            out = []
            for name, L in (("gpu", lib), ("ref", ref.lib)):
                t = tabs[name]
                st = ExtPotSet(C.pointer(t[0]), C.pointer(t[1]), C.pointer(t[2]), bytes([avg]), *orient)
                out.append(np.array([L.dft_common_extpot(C.byref(st), *p) for p in pts]))
            assert out[0].tobytes() == out[1].tobytes(), (avg, orient)


def extpot_on_grid(lib, files, avg, orient, shape, step):
    """dft_common_extpot of this library at the rgrid_map points
    x_i = (i - nx/2) step (origin 0), as a grid"""
    tabs = [ExtPot() for _ in files]
    lib.dft_common_read_pot.argtypes = [C.c_char_p, C.POINTER(ExtPot)]
    lib.dft_common_extpot.restype = C.c_double
    lib.dft_common_extpot.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
    for f, t in zip(files, tabs):
        lib.dft_common_read_pot(f, C.byref(t))
    st = ExtPotSet(C.pointer(tabs[0]), C.pointer(tabs[1]), C.pointer(tabs[2]), bytes([avg]), *orient)
    ax = [(np.arange(n) - n // 2) * step for n in shape]
    out = np.empty(shape)
    for i, x in enumerate(ax[0]):
        for j, y in enumerate(ax[1]):
            for k, z in enumerate(ax[2]):
                out[i, j, k] = lib.dft_common_extpot(C.byref(st), x, y, z)
    return out


@needs_ref
def test_libdft_potential_map_equals_callback_on_grid_points(lib, ref, tmp_path):
    """libdft's own dft_common_potential_map onto its CPU grid gives, point for
    point, this library's callback at the grid coordinates rgrid_map uses --
    the values dft_common_potential_map uploads to a device grid."""
    files = [pot_file(tmp_path / ("q%d.dat" % i), 0.5 + 0.2 * i, 0.05, 600, 10 + i) for i in range(3)]
    shape, step, orient = (10, 8, 12), 0.9, (0.3, 0.7, 0.5, -1.0, 2.0)
    R = ref.lib
    R.dft_common_potential_map.argtypes = [C.c_byte, C.c_char_p, C.c_char_p, C.c_char_p, C.c_void_p] + [C.c_double] * 5
    for avg in (0, 4):
        with Grids(ref, shape, step, 1.0) as g:
            rg = g.rgrid()
            R.dft_common_potential_map(avg, *files, rg, *orient)
            want = g.get_r(rg)
        assert extpot_on_grid(lib, files, avg, orient, shape, step).tobytes() == want.tobytes()


def test_potential_table_refusals(lib, tmp_path):
    lib.dft_common_read_pot.argtypes = [C.c_char_p, C.POINTER(ExtPot)]
    lib.dftgpu_last_error.restype = C.c_int
    t = ExtPot()
    lib.dft_common_read_pot(str(tmp_path / "none.dat").encode(), C.byref(t))
    assert lib.dftgpu_last_error() == 8                                   # DFTGPU_ERR_IO
    lib.dft_common_read_pot(pot_file(tmp_path / "j.dat", 1.0, 0.1, 50, 1, jitter=0.03), C.byref(t))
    assert lib.dftgpu_last_error() == 1                                   # not equidistant
    with open(tmp_path / "d.dat", "w") as f:
        f.write("2.0 1.0\n1.0 2.0\n0.0 3.0\n")
    lib.dft_common_read_pot(str(tmp_path / "d.dat").encode(), C.byref(t))
    assert lib.dftgpu_last_error() == 1                                   # decreasing
    lib.dft_common_read_pot(pot_file(tmp_path / "ok.dat", 1.0, 0.1, 50, 2), C.byref(t))
    assert lib.dftgpu_last_error() == 0 and t.length == 50 and abs(t.step - 0.1) < 1e-8


HOST_DRIVERS = ["dispersion/dispersion3.c", "dispersion/static-resp.c"]


@needs_ref
@pytest.mark.parametrize("driver", HOST_DRIVERS)
def test_host_only_driver_output_identical_to_libdft(lib, ref, tmp_path, driver):
    """Drivers that need no grid (bulk relations of a functional on the stack)
    built twice from the same unmodified source -- against this library and
    against libdft's own build -- print the same bytes.  Both leave
    otf.model to the caller, who does not set it, so the stack is
    zero-initialised in both builds to make that read defined."""
    src = os.path.join(REF_EXAMPLES, driver)
    inc = tmp_path / "inc"
    inc.mkdir()
    os.symlink(os.path.join(os.path.dirname(REF_EXAMPLES), "src"), inc / "dft")
    os.symlink(os.path.join(ROOT, "oracle", "include", "grid"), inc / "grid")
    flags = ["gcc", "-std=gnu11", "-O2", "-w", "-ftrivial-auto-var-init=zero"]
    builds = {
        "gpu": flags + ["-I", INCLUDE, src, "-o", str(tmp_path / "gpu"), "-L", LIBDIR, "-ldftgpu", "-lm",
                        "-Wl,-rpath," + LIBDIR],
        "ref": flags + ["-fgnu89-inline", "-I", str(inc), "-I", os.path.join(os.path.dirname(REF_LIB), "gen"),
                        src, "-o", str(tmp_path / "ref"), REF_LIB, "-lm", "-fopenmp",
                        "-Wl,-rpath," + os.path.dirname(REF_LIB)],
    }
    out = {}
    for name, cmd in builds.items():
        subprocess.run(cmd, check=True)
        r = subprocess.run([str(tmp_path / name)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        out[name] = r.stdout
    assert out["gpu"] == out["ref"]
    assert len(out["gpu"].splitlines()) > 50


def file_api(lib):
    lib.dftgpu_grid_file_write.argtypes = [C.c_char_p, C.c_int, C.c_long, C.c_long, C.c_long,
                                           C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.dftgpu_grid_file_read.argtypes = lib.dftgpu_grid_file_write.argtypes
    return lib.dftgpu_grid_file_write, lib.dftgpu_grid_file_read


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("is_complex", [0, 1])
def test_grid_file_round_trip_and_cuts(lib, tmp_path, is_complex):
    write, read = file_api(lib)
    shape = (6, 4, 10)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(shape + ((2,) if is_complex else ()))
    meta = np.array([0.8, 0.1, -0.2, 0.3, 0.01, 0.02, -0.03])
    base = str(tmp_path / "wf-output-7").encode()
    assert write(base, is_complex, *shape, dp(meta), dp(v)) == 0
    got, gmeta = np.zeros_like(v), np.zeros(7)
    assert read(base, is_complex, *shape, dp(gmeta), dp(got)) == 0
    assert np.array_equal(got, v) and np.array_equal(gmeta, meta)
    # the .x / .y / .z cuts through (nx/2, ny/2, nz/2): coordinate, value(s)
    c = [n // 2 for n in shape]
    for a, ext in enumerate("xyz"):
        rows = np.loadtxt(str(tmp_path / ("wf-output-7." + ext)))
        idx = list(c)
        idx[a] = slice(None)
        want = v[tuple(idx)].reshape(shape[a], -1)
        coord = (np.arange(shape[a]) - shape[a] // 2) * meta[0] - meta[1 + a]
        assert np.allclose(rows[:, 0], coord, rtol=1e-6, atol=1e-12)
        assert np.allclose(rows[:, 1:], want, rtol=1e-6, atol=1e-12)


def test_grid_file_read_takes_the_whole_name(lib, tmp_path):
    """libdft's drivers write with a base name and read with the file's whole
    name: `bubble-100.grd` from the command line (examples/gas-bubble/bubble.c:143)
    or a renamed copy (`restart.chk`, examples/electron/electron.c:163).  A base
    whose .grd exists still reads."""
    import shutil
    write, read = file_api(lib)
    shape = (4, 6, 8)
    v = np.random.default_rng(9).standard_normal(shape + (2,))
    meta = np.array([0.8, 0.0, 0.0, 0.0, 0.0, 0.0, 0.1])
    base = tmp_path / "bubble-100"
    assert write(str(base).encode(), 1, *shape, dp(meta), dp(v)) == 0
    shutil.copy(tmp_path / "bubble-100.grd", tmp_path / "restart.chk")
    for name in ("bubble-100.grd", "restart.chk", "bubble-100"):
        got, gmeta = np.zeros_like(v), np.zeros(7)
        assert read(str(tmp_path / name).encode(), 1, *shape, dp(gmeta), dp(got)) == 0, name
        assert np.array_equal(got, v) and np.array_equal(gmeta, meta), name
    # a directory of that name is not a file: <name>.grd is read instead
    (tmp_path / "bubble-200").mkdir()
    assert read(str(tmp_path / "bubble-200").encode(), 1, *shape, dp(np.zeros(7)), dp(np.zeros_like(v))) == 8


def test_grid_file_refusals(lib, tmp_path):
    write, read = file_api(lib)
    lib.dftgpu_last_error.restype = C.c_int
    shape = (4, 4, 4)
    v, meta = np.ones(shape), np.array([1.0, 0, 0, 0, 0, 0, 0])
    base = str(tmp_path / "g").encode()
    assert write(base, 0, *shape, dp(meta), dp(v)) == 0
    out, m = np.zeros(shape), np.zeros(7)
    assert read(base, 0, 4, 4, 6, dp(m), dp(np.zeros((4, 4, 6)))) == 2     # DFTGPU_ERR_SIZE
    assert read(base, 1, *shape, dp(m), dp(np.zeros(shape + (2,)))) == 1   # DFTGPU_ERR_ARG: real file
    assert read(str(tmp_path / "missing").encode(), 0, *shape, dp(m), dp(out)) == 8   # DFTGPU_ERR_IO
    raw = open(tmp_path / "g.grd", "rb").read()
    open(tmp_path / "t.grd", "wb").write(raw[:-8])
    assert read(str(tmp_path / "t").encode(), 0, *shape, dp(m), dp(out)) == 8         # truncated
    open(tmp_path / "f.grd", "wb").write(b"\0" * len(raw))
    assert read(str(tmp_path / "f").encode(), 0, *shape, dp(m), dp(out)) == 6         # DFTGPU_ERR_UNSUPPORTED
    assert lib.dftgpu_last_error() == 6


@needs_ref
@pytest.mark.parametrize("model", [32, 1024 | 9, 262144])
def test_thermal_bulk_relations_equal_libdft(lib, ref, model):
    """The ideal Bose gas in the bulk relations of the thermal models
    (src/helium-ot-bulk.c:30-31, 54-55 with src/common.c:253-529): the
    library's host restatement against libdft's own code, at the bulk density
    (rho lambda^3 above g_{3/2}(1)) and in the dilute z < 1 branch."""
    p = ot_params(lib, model)
    R = ref.lib
    for L in (lib, R):
        for name in ("dft_ot_bulk_energy", "dft_ot_bulk_dEdRho"):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [C.c_void_p, C.c_double]
    with Grids(ref, (8, 8, 8), 1.0, 4.002602 / ref.AUTOAMU) as g:
        w = g.wf()
        o = g.ot(model, w)
        for f in (1.3, 1.0, 0.2, 0.01, 1e-4, 1e-7):
            rho = f * p.rho0
            for name in ("dft_ot_bulk_energy", "dft_ot_bulk_dEdRho"):
                a, b = getattr(lib, name)(C.byref(p), rho), getattr(R, name)(o, rho)
                assert abs(a - b) <= 1e-15 * abs(b), (name, f, a, b)
