"""CPU oracle for the OT-DFT hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this package, and only as the checker.  It loads one of two FP64
CPU libraries built by ``oracle/Makefile``:

* ``port`` -- ``_build/liboracle.so``: this project's C restatement of
  libdft's OT functional (``ot_port.c``) over a restatement of the libgrid
  subset it calls (``grid_shim.c``).  Builds anywhere (x86 and Arm).
* ``ref`` -- ``_ref/libdft_ref.so``: libdft's own ``src/ot.c``,
  ``ot-energy.c``, ``common.c`` and ``helium-ot-bulk.c`` compiled unmodified
  against the same libgrid restatement.  Only buildable where the reference
  tree exists; used to validate ``port`` and to generate golden fixtures.

All arrays crossing the boundary are contiguous float64 / complex128 numpy
arrays in ``[x][y][z]`` order.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libdft_ref.so")
# root of the libdft source tree (read in place; LIBDFT_REFERENCE overrides the default)
REF_ROOT = os.environ.get("LIBDFT_REFERENCE", "/root/reference")
REF_TREE = os.path.join(REF_ROOT, "src")

# model flags (libdft src/ot.h:37-60)
DFT_OT_PLAIN = 0
DFT_OT_KC = 1
DFT_OT_BACKFLOW = 8

PARAM_NAMES = ("b c2 c2_exp c3 c3_exp rho0 h sigma epsilon rho_0s alpha_s l_g mass "
               "g11 g12 g21 g22 a1 a2 div_epsilon max_veloc max_bfpot c_bfpot").split()

_vp = C.c_void_p
_d = C.c_double
_l = C.c_long
_i = C.c_int
_dp = C.POINTER(C.c_double)


def build(kind: str = "port") -> str:
    """Build the requested oracle library with make; returns its path."""
    target = "all" if kind == "port" else "ref"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)
    return PORT_LIB if kind == "port" else REF_LIB


def ref_available() -> bool:
    return os.path.exists(REF_LIB) or os.path.isdir(REF_TREE)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class Oracle:
    """Thin numpy wrapper over one oracle library."""

    def __init__(self, kind: str = "port", build_if_missing: bool = True):
        path = PORT_LIB if kind == "port" else REF_LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise FileNotFoundError(path)
            build(kind)
        self.kind = kind
        L = self.lib = C.CDLL(path)
        sig = {
            "orc_kind": (_i, []),
            "orc_wf_new": (_vp, [_l, _l, _l, _d, _d]),
            "orc_wf_free": (None, [_vp]),
            "orc_wf_grid": (_vp, [_vp]),
            "orc_wf_set_norm": (None, [_vp, _d]),
            "orc_wf_norm": (_d, [_vp]),
            "orc_wf_normalize": (_d, [_vp]),
            "orc_wf_kinetic_energy": (_d, [_vp]),
            "orc_wf_density": (None, [_vp, _vp]),
            "orc_wf_velocity": (None, [_vp, _vp, _vp, _vp, _d]),
            "orc_wf_set_momentum": (None, [_vp, _d, _d, _d]),
            "orc_wf_set_propagator": (None, [_vp, _i]),
            "orc_wf_boundary": (None, [_vp, _vp, _d, _d, _l, _l, _l, _l, _l, _l]),
            "orc_wf_absorb_potential": (None, [_vp, _vp, _d, _d]),
            "orc_cgrid_new": (_vp, [_l, _l, _l, _d]),
            "orc_cgrid_free": (None, [_vp]),
            "orc_cgrid_set": (None, [_vp, _dp]),
            "orc_cgrid_get": (None, [_vp, _dp]),
            "orc_rgrid_new": (_vp, [_l, _l, _l, _d]),
            "orc_rgrid_free": (None, [_vp]),
            "orc_rgrid_set": (None, [_vp, _dp]),
            "orc_rgrid_get": (None, [_vp, _dp]),
            "orc_rgrid_get_spectrum": (None, [_vp, _dp]),
            "orc_rgrid_integral": (_d, [_vp]),
            "orc_rgrid_fft": (None, [_vp]),
            "orc_rgrid_inverse_fft_norm": (None, [_vp]),
            "orc_cgrid_fft": (None, [_vp]),
            "orc_cgrid_inverse_fft_norm": (None, [_vp]),
            "orc_fft1d": (None, [_dp, _l, _i]),
            "orc_ot_new": (_vp, [_l, _vp, _l, _l, _d]),
            "orc_ot_free": (None, [_vp]),
            "orc_ot_params": (_i, [_vp, _dp]),
            "orc_ot_set_limits": (None, [_vp, _d, _d, _d, _d]),
            "orc_ot_kernel": (_i, [_vp, _i, _dp]),
            "orc_ot_potential": (None, [_vp, _vp, _vp]),
            "orc_ot_energy_density": (None, [_vp, _vp, _vp]),
            "orc_propagate": (None, [_vp, _vp, _d, _d]),
            "orc_predict": (None, [_vp, _vp, _vp, _d, _d]),
            "orc_correct": (None, [_vp, _vp, _d, _d]),
            "orc_pc_step": (None, [_vp, _vp, _vp, _vp, _vp, _d, _d, _d]),
            "orc_total_energy": (_d, [_vp, _vp, _vp, _vp]),
            "orc_bulk_density": (_d, [_vp, _d]),
            "orc_bulk_chempot": (_d, [_vp, _d]),
            "orc_bulk_dEdRho": (_d, [_vp, _d]),
            "orc_bulk_energy": (_d, [_vp, _d]),
            "orc_bulk_sound_speed": (_d, [_vp, _d]),
            "orc_bulk_dispersion": (_d, [_vp, _d, _d]),
            "orc_const": (_d, [_i]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if L.orc_kind() == 2:   # libdft's own term-level entry points (reference build only)
            ref_sig = {
                "orc_ref_potential2": (None, [_vp] * 6),
                "orc_ref_add_lj": (None, [_vp] * 3),
                "orc_ref_add_local": (None, [_vp] * 3),
                "orc_ref_backflow": (None, [_vp] * 6),
                "orc_ref_energy_density_kc": (None, [_vp] * 4),
                "orc_ref_energy_density_bf": (None, [_vp] * 4),
            }
            for name, (res, args) in ref_sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args

    # constants
    @property
    def AUTOANG(self): return self.lib.orc_const(0)
    @property
    def AUTOK(self): return self.lib.orc_const(1)
    @property
    def AUTOFS(self): return self.lib.orc_const(2)
    @property
    def AUTOAMU(self): return self.lib.orc_const(3)
    @property
    def AUTOBAR(self): return self.lib.orc_const(4)

    def fft1d(self, x: np.ndarray, sign: int = -1) -> np.ndarray:
        a = np.ascontiguousarray(x, dtype=np.complex128).copy()
        self.lib.orc_fft1d(a.view(np.float64).ctypes.data_as(_dp), a.size, sign)
        return a


class Grids:
    """Owns oracle grid objects for one (nx, ny, nz, step) geometry."""

    def __init__(self, orc: Oracle, shape, step: float, mass: float):
        self.o = orc
        self.shape = tuple(int(s) for s in shape)
        self.step = float(step)
        self.mass = float(mass)
        self._owned = []

    def wf(self, psi: np.ndarray | None = None, propagator: int = 1):
        """propagator: 1 = WF_2ND_ORDER_FFT, 3 = WF_2ND_ORDER_CN"""
        nx, ny, nz = self.shape
        w = self.o.lib.orc_wf_new(nx, ny, nz, self.step, self.mass)
        if not w:
            raise RuntimeError("oracle wf alloc failed")
        self._owned.append(("wf", w))
        if propagator != 1:
            self.o.lib.orc_wf_set_propagator(w, propagator)
        if psi is not None:
            self.set_wf(w, psi)
        return w

    def set_wf(self, w, psi):
        a = np.ascontiguousarray(psi, dtype=np.complex128)
        assert a.shape == self.shape
        self.o.lib.orc_cgrid_set(self.o.lib.orc_wf_grid(w), _ptr(a.view(np.float64)))

    def get_wf(self, w) -> np.ndarray:
        out = np.empty(self.shape, dtype=np.complex128)
        self.o.lib.orc_cgrid_get(self.o.lib.orc_wf_grid(w), _ptr(out.view(np.float64)))
        return out

    def cgrid(self, val: np.ndarray | None = None):
        nx, ny, nz = self.shape
        g = self.o.lib.orc_cgrid_new(nx, ny, nz, self.step)
        self._owned.append(("cgrid", g))
        if val is not None:
            self.set_c(g, val)
        return g

    def set_c(self, g, val):
        a = np.ascontiguousarray(np.broadcast_to(val, self.shape), dtype=np.complex128)
        self.o.lib.orc_cgrid_set(g, _ptr(a.view(np.float64)))

    def get_c(self, g) -> np.ndarray:
        out = np.empty(self.shape, dtype=np.complex128)
        self.o.lib.orc_cgrid_get(g, _ptr(out.view(np.float64)))
        return out

    def rgrid(self, val: np.ndarray | None = None):
        nx, ny, nz = self.shape
        g = self.o.lib.orc_rgrid_new(nx, ny, nz, self.step)
        self._owned.append(("rgrid", g))
        if val is not None:
            self.set_r(g, val)
        return g

    def set_r(self, g, val):
        a = np.ascontiguousarray(np.broadcast_to(val, self.shape), dtype=np.float64)
        self.o.lib.orc_rgrid_set(g, _ptr(a))

    def get_r(self, g) -> np.ndarray:
        out = np.empty(self.shape, dtype=np.float64)
        self.o.lib.orc_rgrid_get(g, _ptr(out))
        return out

    def ot(self, model: int, w, min_ns: int = 4, max_ns: int = 32, lg_bohr: float = 0.0):
        o = self.o.lib.orc_ot_new(model, w, min_ns, max_ns, lg_bohr)
        if not o:
            raise RuntimeError("oracle dft_ot_alloc failed")
        self._owned.append(("ot", o))
        return o

    def params(self, otf) -> dict:
        buf = np.zeros(64)
        n = self.o.lib.orc_ot_params(otf, _ptr(buf))
        return dict(zip(PARAM_NAMES, buf[:n].tolist()))

    def kernel(self, otf, which: int) -> np.ndarray | None:
        nx, ny, nz = self.shape
        out = np.empty((nx, ny, nz // 2 + 1), dtype=np.complex128)
        ok = self.o.lib.orc_ot_kernel(otf, which, _ptr(out.view(np.float64)))
        return out if ok else None

    def potential(self, otf, w, base: np.ndarray | None = None) -> np.ndarray:
        P = self.cgrid(0.0 if base is None else base)
        self.o.lib.orc_ot_potential(otf, P, w)
        return self.get_c(P)

    def energy_density(self, otf, w) -> np.ndarray:
        ed = self.rgrid()
        self.o.lib.orc_ot_energy_density(otf, ed, w)
        return self.get_r(ed)

    def free(self):
        L = self.o.lib
        for kind, h in reversed(self._owned):
            {"wf": L.orc_wf_free, "cgrid": L.orc_cgrid_free, "rgrid": L.orc_rgrid_free,
             "ot": L.orc_ot_free}[kind](h)
        self._owned.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()
