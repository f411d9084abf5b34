"""CPU: the C-ABI library builds, loads and exports every declared entry point.

No compute is issued here (there is no GPU in the build container)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "dftgpu.h")
LIB = os.path.join(ROOT, "libdft_gb300", "libdftgpu.so")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = "\n".join(l for l in src.splitlines() if not l.lstrip().startswith("#"))
    src = re.sub(r"\{[^{}]*\}", ";", src)          # struct bodies
    names = set()
    for stmt in src.split(";"):
        if "typedef" in stmt or "(" not in stmt:
            continue
        m = re.search(r"([A-Za-z_]\w*)\s*\(", stmt)
        if m and m.group(1) not in ("extern",):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def built():
    if not os.path.exists(LIB):
        from libdft_gb300.build import build
        build()
    return LIB


def test_header_declares_the_reference_entry_points():
    names = set(declared_functions())
    for n in ("dft_ot_alloc", "dft_ot_free", "dft_ot_potential", "dft_ot_energy_density", "grid_wf_propagate",
              "grid_wf_propagate_predict", "grid_wf_propagate_correct", "grid_wf_alloc", "grid_wf_density",
              "grid_wf_norm", "grid_wf_normalize", "grid_wf_energy", "grid_wf_velocity", "rgrid_alloc",
              "cgrid_alloc", "grid_real_to_complex_re", "grid_add_real_to_complex_re",
              "dft_ot_bulk_density_pressurized", "dft_ot_bulk_chempot_pressurized", "cuda_enable"):
        assert n in names, n


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_python_binding_signatures_resolve(built):
    import libdft_gb300 as G
    L = G.load(built)
    for name in G.SIGNATURES:
        assert hasattr(L, name), name


def test_init_without_gpu_reports_nodevice(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import libdft_gb300 as G
    L = G.load(built)
    assert L.dftgpu_init(0) == 7
    assert L.dftgpu_last_error() == 7
    # allocation without a device fails cleanly (NULL + error code), no crash
    assert not L.grid_wf_alloc(16, 16, 16, 1.0, 7296.0, 3, 1, b"x")
    assert L.dftgpu_last_error() == 7


@pytest.mark.parametrize("example", ["imag_time", "moving_bubble"])
def test_c_dropin_example_compiles_and_links(built, tmp_path, example):
    """The libdft-style drivers (REAL complex time steps, dft_ot_* calls; the
    moving-background bubble of examples/gas-bubble/bubble.c) compile as C
    against include/dftgpu.h and link against libdftgpu.so."""
    src = os.path.join(ROOT, "libdft_gb300", "examples", example + ".c")
    exe = tmp_path / example
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", str(exe),
                    "-L", os.path.dirname(built), "-ldftgpu", "-lm", "-Wl,-rpath," + os.path.dirname(built)],
                   check=True)
    assert exe.exists()


def test_null_arguments_are_refused_without_a_device(built):
    """The grid and wave-function entry points refuse NULL with DFTGPU_ERR_ARG
    (libdft would dereference it) before any device work."""
    import math
    L = ctypes.CDLL(built)
    L.dftgpu_last_error.restype = ctypes.c_int
    buf = (ctypes.c_double * 8)()
    for name in ("rgrid_copy_to_host", "rgrid_copy_from_host", "cgrid_copy_to_host", "cgrid_copy_from_host",
                 "rgrid_copy_to_host_raw", "cgrid_copy_to_host_raw"):
        f = getattr(L, name)
        f.restype = ctypes.c_int
        assert f(None, buf) == 1, name
    for name in ("dftgpu_wf_propagate", "dftgpu_wf_propagate_correct"):
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        assert f(None, None, 1.0, 0.0) == 1, name
    for name in ("grid_wf_norm", "grid_wf_normalize", "grid_wf_kinetic_energy", "rgrid_integral"):
        f = getattr(L, name)
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_void_p]
        assert math.isnan(f(None)) and L.dftgpu_last_error() == 1, name
    for name in ("rgrid_zero", "cgrid_zero"):
        getattr(L, name)(None)
        assert L.dftgpu_last_error() == 1, name
