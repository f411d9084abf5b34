"""libdft_gb300 -- GB300 implementation of libdft's OT-DFT time-step hot path.

The product is the C-ABI shared library ``libdftgpu.so`` (sources in
``csrc/``, header ``include/dftgpu.h``).  This module is a thin ctypes
binding over it with numpy conversions, mirroring the reference interface:
``Wf`` (libgrid ``wf``), ``CGrid`` / ``RGrid`` (``cgrid`` / ``rgrid``) and
``OT`` (libdft ``dft_ot_functional``: ``dft_ot_alloc``, ``dft_ot_potential``,
``dft_ot_energy_density``, ``dft_ot_bulk_*``).  Every computation runs in the
CUDA library; there is no CPU fallback -- importing fails loudly if the
library was not built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdftgpu.so")

FP64 = 0
FP32 = 1
DFT_OT_PLAIN = 0
DFT_OT_KC = 1
DFT_OT_BACKFLOW = 8
WF_PERIODIC_BOUNDARY = 3
WF_2ND_ORDER_FFT = 1
WF_2ND_ORDER_CN = 3

AUTOANG = 0.529177210903
AUTOK = 3.1577502480407e5
AUTOFS = 0.024188843265857
AUTOAMU = 1.0 / 1822.888486209
AUTOMPS = 2.18769126364e6
HELIUM_MASS = 4.002602 / AUTOAMU

ERRORS = {0: "ok", 1: "invalid argument", 2: "unsupported size", 3: "out of device memory",
          4: "CUDA error", 5: "non-finite value", 6: "unsupported", 7: "no CUDA device"}

_vp, _d, _l, _i, _c = C.c_void_p, C.c_double, C.c_long, C.c_int, C.c_char
_dp = C.POINTER(C.c_double)

# name: (restype, argtypes)
SIGNATURES = {
    "dftgpu_init": (_i, [_i]),
    "cuda_enable": (None, [_c, _l, C.POINTER(C.c_int)]),
    "dftgpu_set_precision": (_i, [_i]),
    "dftgpu_get_precision": (_i, []),
    "dftgpu_last_error": (_i, []),
    "dftgpu_last_error_message": (C.c_char_p, []),
    "dftgpu_synchronize": (_i, []),
    "dftgpu_set_stream": (_i, [_vp]),
    "dftgpu_get_stream": (_vp, []),
    "rgrid_value_outside_periodic": (_d, [_vp, _l, _l, _l]),
    "rgrid_alloc": (_vp, [_l, _l, _l, _d, _vp, _vp, C.c_char_p]),
    "rgrid_free": (None, [_vp]),
    "rgrid_clone": (_vp, [_vp, C.c_char_p]),
    "rgrid_set_origin": (None, [_vp, _d, _d, _d]),
    "rgrid_zero": (None, [_vp]),
    "rgrid_constant": (None, [_vp, _d]),
    "rgrid_copy": (None, [_vp, _vp]),
    "rgrid_add": (None, [_vp, _d]),
    "rgrid_multiply": (None, [_vp, _d]),
    "rgrid_sum": (None, [_vp, _vp, _vp]),
    "rgrid_product": (None, [_vp, _vp, _vp]),
    "rgrid_add_scaled": (None, [_vp, _d, _vp]),
    "rgrid_add_scaled_product": (None, [_vp, _d, _vp, _vp]),
    "rgrid_integral": (_d, [_vp]),
    "rgrid_map": (None, [_vp, _vp, _vp]),
    "rgrid_value_at_index": (_d, [_vp, _l, _l, _l]),
    "rgrid_copy_to_host": (_i, [_vp, _dp]),
    "rgrid_copy_from_host": (_i, [_vp, _dp]),
    "rgrid_copy_to_host_raw": (_i, [_vp, _vp]),
    "rgrid_copy_from_host_raw": (_i, [_vp, _vp]),
    "cgrid_alloc": (_vp, [_l, _l, _l, _d, _vp, _vp, C.c_char_p]),
    "cgrid_free": (None, [_vp]),
    "cgrid_clone": (_vp, [_vp, C.c_char_p]),
    "cgrid_zero": (None, [_vp]),
    "cgrid_constant_re_im": (None, [_vp, _d, _d]),
    "cgrid_add_re_im": (None, [_vp, _d, _d]),
    "cgrid_multiply_re_im": (None, [_vp, _d, _d]),
    "cgrid_copy": (None, [_vp, _vp]),
    "cgrid_set_momentum": (None, [_vp, _d, _d, _d]),
    "cgrid_map_re_im": (None, [_vp, _vp, _vp]),
    "cgrid_copy_to_host": (_i, [_vp, _dp]),
    "cgrid_copy_from_host": (_i, [_vp, _dp]),
    "cgrid_copy_to_host_raw": (_i, [_vp, _vp]),
    "cgrid_copy_from_host_raw": (_i, [_vp, _vp]),
    "grid_real_to_complex_re": (None, [_vp, _vp]),
    "grid_add_real_to_complex_re": (None, [_vp, _vp]),
    "grid_add_real_to_complex_im": (None, [_vp, _vp]),
    "grid_wf_alloc": (_vp, [_l, _l, _l, _d, _d, _c, _c, C.c_char_p]),
    "grid_wf_clone": (_vp, [_vp, C.c_char_p]),
    "grid_wf_free": (None, [_vp]),
    "grid_wf_constant_re_im": (None, [_vp, _d, _d]),
    "grid_wf_density": (None, [_vp, _vp]),
    "grid_wf_norm": (_d, [_vp]),
    "grid_wf_normalize": (_d, [_vp]),
    "grid_wf_energy": (_d, [_vp, _vp]),
    "grid_wf_kinetic_energy": (_d, [_vp]),
    "grid_wf_velocity": (None, [_vp, _vp, _vp, _vp, _d]),
    "grid_wf_boundary": (None, [_vp, _vp, _d, _d, _l, _l, _l, _l, _l, _l]),
    "grid_wf_absorb_potential": (None, [_vp, _vp, _d, _d]),
    "dftgpu_wf_propagate": (_i, [_vp, _vp, _d, _d]),
    "dftgpu_wf_propagate_predict": (_i, [_vp, _vp, _vp, _d, _d]),
    "dftgpu_wf_propagate_correct": (_i, [_vp, _vp, _d, _d]),
    "grid_wf_propagate": (None, [_vp, _vp, _d, _d]),          # REAL complex dt passed as (re, im)
    "grid_wf_propagate_predict": (None, [_vp, _vp, _vp, _d, _d]),
    "grid_wf_propagate_correct": (None, [_vp, _vp, _d, _d]),
    "grid_wf_constant": (None, [_vp, _d, _d]),
    "cgrid_add": (None, [_vp, _d, _d]),
    "cgrid_multiply": (None, [_vp, _d, _d]),
    "cgrid_constant": (None, [_vp, _d, _d]),
    "cgrid_map": (None, [_vp, _vp, _vp]),
    "grid_wf_map": (None, [_vp, _vp, _vp]),
    "dft_ot_alloc": (_vp, [_l, _vp, _l, _l]),
    "dft_ot_free": (None, [_vp]),
    "dft_ot_potential": (None, [_vp, _vp, _vp]),
    "dft_ot_energy_density": (None, [_vp, _vp, _vp]),
    "dft_ot_init_params": (None, [_vp, _l]),
    "dft_ot_update_kernels": (_i, [_vp, _l, _l]),
    "dft_ot_bulk_energy": (_d, [_vp, _d]),
    "dft_ot_bulk_dEdRho": (_d, [_vp, _d]),
    "dft_ot_bulk_pressure": (_d, [_vp, _d]),
    "dft_ot_bulk_dPdRho": (_d, [_vp, _d]),
    "dft_ot_bulk_density_pressurized": (_d, [_vp, _d]),
    "dft_ot_bulk_chempot_pressurized": (_d, [_vp, _d]),
    "dft_ot_bulk_density": (_d, [_vp]),
    "dft_ot_bulk_chempot": (_d, [_vp]),
    "dft_ot_bulk_chempot2": (_d, [_vp]),
    "dft_ot_bulk_compressibility": (_d, [_vp, _d]),
    "dft_ot_bulk_sound_speed": (_d, [_vp, _d]),
    "dft_ot_bulk_dispersion": (_d, [_vp, _dp, _d]),
    "dftgpu_ot_kernel": (_i, [_vp, _i, _dp]),
    "dftgpu_rgrid_spectrum": (_i, [_vp, _dp]),
    "dftgpu_wf_propagate_noalloc": (_i, [_vp, _vp, _vp, _l, _l, _l, _d, _d, _d, _d, _i, _vp]),
    "dftgpu_pc_step": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _d]),
    "dftgpu_run": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _d, _l, _i]),
    "dftgpu_energy_report": (_i, [_vp, _vp, _vp, _dp, _dp, _dp]),
    "dft_ot_potential2": (None, [_vp] * 6),
    "dft_ot_add_lennard_jones_potential": (None, [_vp] * 5),
    "dft_ot_add_local_correlation_potential": (None, [_vp] * 6),
    "dft_ot_backflow_potential": (None, [_vp] * 12),
    "dft_ot_energy_density_kc": (None, [_vp] * 4),
    "dft_ot_energy_density_bf": (None, [_vp] * 4),
    "dftgpu_ot_potential_vjp": (_i, [_vp, _vp, _vp, _vp]),
    "dftgpu_wf_propagate_vjp": (_i, [_vp, _vp, _d, _d, _vp, _vp, _vp, _vp, _vp]),
    "dftgpu_pc_step_vjp": (_i, [_vp, _vp, _vp, _d, _d, _d, _i, _vp, _vp]),
    "dftgpu_adjoint_run": (_i, [_vp, _vp, _vp, _d, _d, _d, _l, _i, _l, _vp, _dp, _vp, _vp]),
    "dft_ot_bulk_chempot3": (_d, [_vp, _d]),
    "dft_ot_bulk_istatic": (_d, [_vp, _dp, _d]),
    "dft_ot_dispersion": (_d, [_vp, _vp, _d, _dp, _d, C.c_byte, C.c_byte]),
    "dft_ot_bulk_surface_tension": (_d, [_vp, _vp, _d, _d]),
    "cgrid_value_at_index_re_im": (_i, [_vp, _l, _l, _l, _dp, _dp]),
    "rgrid_write_grid": (None, [C.c_char_p, _vp]),
    "cgrid_write_grid": (None, [C.c_char_p, _vp]),
    "rgrid_read_grid": (None, [_vp, C.c_char_p]),
    "cgrid_read_grid": (None, [_vp, C.c_char_p]),
    "dftgpu_grid_file_write": (_i, [C.c_char_p, _i, _l, _l, _l, _dp, _dp]),
    "dftgpu_grid_file_read": (_i, [C.c_char_p, _i, _l, _l, _l, _dp, _dp]),
    "cgrid_read": (_vp, [_vp, _vp]),
    "rgrid_read": (_vp, [_vp, _vp]),
    "cgrid_write": (None, [_vp, _vp]),
    "rgrid_write": (None, [_vp, _vp]),
    "rgrid_power": (None, [_vp, _vp, _d]),
}

OPTIONAL = set()   # entry points allowed to be absent (none)


class DftGpuError(RuntimeError):
    pass


def load(path: str = LIB_PATH) -> C.CDLL:
    if not os.path.exists(path):
        raise DftGpuError("libdftgpu.so not built (run __graft_entry__.build() or python -m libdft_gb300.build)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        try:
            f = getattr(lib, name)
        except AttributeError:
            if name in OPTIONAL:
                continue
            raise
        f.restype = res
        f.argtypes = args
    return lib


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = load()
    return _LIB


def check(rc: int | None = None, what: str = ""):
    """Raise on a non-zero return code or a pending library error."""
    L = lib()
    code = rc if rc else L.dftgpu_last_error()
    if rc and rc != 0:
        L.dftgpu_last_error()
    if code:
        msg = L.dftgpu_last_error_message().decode(errors="replace")
        raise DftGpuError("%s: %s (%d): %s" % (what or "libdftgpu", ERRORS.get(code, "?"), code, msg))


def _dptr(a):
    return a.ctypes.data_as(_dp)


class CGrid:
    def __init__(self, shape, step, ptr=None, own=True):
        L = lib()
        self.shape = tuple(int(s) for s in shape)
        self.step = float(step)
        self.ptr = ptr or L.cgrid_alloc(*self.shape, self.step, None, None, b"cgrid")
        if not self.ptr:
            check(what="cgrid_alloc")
        self.own = own

    def set(self, a):
        a = np.ascontiguousarray(np.broadcast_to(a, self.shape), dtype=np.complex128)
        check(lib().cgrid_copy_from_host(self.ptr, _dptr(a.view(np.float64))), "cgrid_copy_from_host")

    def get(self):
        out = np.empty(self.shape, dtype=np.complex128)
        check(lib().cgrid_copy_to_host(self.ptr, _dptr(out.view(np.float64))), "cgrid_copy_to_host")
        return out

    def zero(self):
        lib().cgrid_zero(self.ptr)

    def free(self):
        if self.ptr and self.own:
            lib().cgrid_free(self.ptr)
        self.ptr = None


class RGrid:
    def __init__(self, shape, step, ptr=None, own=True):
        L = lib()
        self.shape = tuple(int(s) for s in shape)
        self.step = float(step)
        self.ptr = ptr or L.rgrid_alloc(*self.shape, self.step, None, None, b"rgrid")
        if not self.ptr:
            check(what="rgrid_alloc")
        self.own = own

    def set(self, a):
        a = np.ascontiguousarray(np.broadcast_to(a, self.shape), dtype=np.float64)
        check(lib().rgrid_copy_from_host(self.ptr, _dptr(a)), "rgrid_copy_from_host")

    def get(self):
        out = np.empty(self.shape, dtype=np.float64)
        check(lib().rgrid_copy_to_host(self.ptr, _dptr(out)), "rgrid_copy_to_host")
        return out

    def spectrum(self):
        nx, ny, nz = self.shape
        out = np.empty((nx, ny, nz // 2 + 1), dtype=np.complex128)
        check(lib().dftgpu_rgrid_spectrum(self.ptr, _dptr(out.view(np.float64))), "dftgpu_rgrid_spectrum")
        return out

    def integral(self):
        v = lib().rgrid_integral(self.ptr)
        check(what="rgrid_integral")
        return v

    def free(self):
        if self.ptr and self.own:
            lib().rgrid_free(self.ptr)
        self.ptr = None


class Wf:
    """libgrid wave function on the GPU (periodic; 2nd-order FFT propagator, or
    Crank-Nicolson with propagator=WF_2ND_ORDER_CN)."""

    def __init__(self, shape, step, mass=HELIUM_MASS, ptr=None, propagator=WF_2ND_ORDER_FFT):
        L = lib()
        self.shape = tuple(int(s) for s in shape)
        self.step = float(step)
        self.ptr = ptr or L.grid_wf_alloc(*self.shape, self.step, mass, WF_PERIODIC_BOUNDARY, propagator, b"wf")
        if not self.ptr:
            check(what="grid_wf_alloc")

    @property
    def grid_ptr(self):
        return C.cast(self.ptr, C.POINTER(C.c_void_p))[0]

    @property
    def norm_target(self):
        return C.cast(self.ptr, C.POINTER(C.c_double))[2]   # wf.norm after grid ptr and mass

    @norm_target.setter
    def norm_target(self, v):
        C.cast(self.ptr, C.POINTER(C.c_double))[2] = float(v)

    def set(self, psi):
        a = np.ascontiguousarray(psi, dtype=np.complex128)
        check(lib().cgrid_copy_from_host(self.grid_ptr, _dptr(a.view(np.float64))), "wf set")

    def set_momentum(self, kx0, ky0, kz0):
        """Moving background: cgrid_set_momentum on the wave function's grid."""
        lib().cgrid_set_momentum(self.grid_ptr, float(kx0), float(ky0), float(kz0))
        check(what="cgrid_set_momentum")

    def get(self):
        out = np.empty(self.shape, dtype=np.complex128)
        check(lib().cgrid_copy_to_host(self.grid_ptr, _dptr(out.view(np.float64))), "wf get")
        return out

    def norm(self):
        v = lib().grid_wf_norm(self.ptr)
        check(what="grid_wf_norm")
        return v

    def normalize(self):
        v = lib().grid_wf_normalize(self.ptr)
        check(what="grid_wf_normalize")
        return v

    def kinetic_energy(self):
        v = lib().grid_wf_kinetic_energy(self.ptr)
        check(what="grid_wf_kinetic_energy")
        return v

    def propagate(self, pot: CGrid, dt: complex):
        check(lib().dftgpu_wf_propagate(self.ptr, pot.ptr, dt.real, dt.imag), "propagate")

    def predict(self, wfp: "Wf", pot: CGrid, dt: complex):
        check(lib().dftgpu_wf_propagate_predict(self.ptr, wfp.ptr, pot.ptr, dt.real, dt.imag), "predict")

    def propagate_vjp(self, pot: CGrid, dt: complex, psi_in: CGrid, psi_out: CGrid, cot_out: CGrid, cot_in: CGrid,
                      cot_pot: CGrid):
        """cot_in = S(pot,dt)^H cot_out, cot_pot += dJ/dpot (psi_out = S(pot,dt) psi_in)."""
        check(lib().dftgpu_wf_propagate_vjp(self.ptr, pot.ptr, dt.real, dt.imag, psi_in.ptr, psi_out.ptr, cot_out.ptr,
                                            cot_in.ptr, cot_pot.ptr), "dftgpu_wf_propagate_vjp")

    def correct(self, pot: CGrid, dt: complex):
        check(lib().dftgpu_wf_propagate_correct(self.ptr, pot.ptr, dt.real, dt.imag), "correct")

    def free(self):
        if self.ptr:
            lib().grid_wf_free(self.ptr)
        self.ptr = None


class OTParams(C.Structure):
    """Public head of dft_ot_functional (include/dftgpu.h)."""
    _fields_ = [("model", C.c_long)] + [(n, C.c_double) for n in
                ("b", "c2", "c2_exp", "c3", "c3_exp", "c4", "rho_0s", "alpha_s", "l_g", "mass", "rho0", "temp",
                 "h", "sigma", "epsilon", "cval", "g11", "g12", "g21", "g22", "a1", "a2",
                 "beta", "rhom", "C", "mu0", "xi", "rhobf", "div_epsilon", "max_veloc", "max_bfpot", "c_bfpot")] + \
              [("density", C.c_void_p), ("priv", C.c_void_p)]


class OT:
    """libdft dft_ot_functional on the GPU."""

    def __init__(self, model: int, wf: Wf, min_ns: int = 4, max_ns: int = 32, lg_bohr: float | None = None):
        L = lib()
        self.ptr = L.dft_ot_alloc(model, wf.ptr, min_ns, max_ns)
        if not self.ptr:
            check(what="dft_ot_alloc")
        self.shape, self.step = wf.shape, wf.step
        if lg_bohr is not None and (model & DFT_OT_KC):
            self.params.l_g = lg_bohr
            check(L.dft_ot_update_kernels(self.ptr, min_ns, max_ns), "dft_ot_update_kernels")

    @property
    def params(self) -> OTParams:
        return C.cast(self.ptr, C.POINTER(OTParams))[0]

    def potential(self, P: CGrid, wf: Wf):
        lib().dft_ot_potential(self.ptr, P.ptr, wf.ptr)
        check(what="dft_ot_potential")

    def energy_density(self, ed: RGrid, wf: Wf):
        lib().dft_ot_energy_density(self.ptr, ed.ptr, wf.ptr)
        check(what="dft_ot_energy_density")

    def kernel(self, which: int) -> np.ndarray:
        nx, ny, nz = self.shape
        out = np.empty((nz // 2 + 1, nx // 2 + 1, ny // 2 + 1))
        check(lib().dftgpu_ot_kernel(self.ptr, which, _dptr(out)), "dftgpu_ot_kernel")
        return out

    def bulk_density(self, pressure=0.0):
        return lib().dft_ot_bulk_density_pressurized(self.ptr, pressure)

    def bulk_chempot(self, pressure=0.0):
        return lib().dft_ot_bulk_chempot_pressurized(self.ptr, pressure)

    def pc_step(self, wf: Wf, wfp: Wf, P: CGrid, vext: RGrid | None, mu0: float, dt: complex):
        check(lib().dftgpu_pc_step(self.ptr, wf.ptr, wfp.ptr, P.ptr, vext.ptr if vext else None, mu0, dt.real, dt.imag),
              "dftgpu_pc_step")

    def run(self, wf: Wf, wfp: Wf, P: CGrid, vext: RGrid | None, mu0: float, dt: complex, nsteps: int, renorm: bool):
        check(lib().dftgpu_run(self.ptr, wf.ptr, wfp.ptr, P.ptr, vext.ptr if vext else None, mu0, dt.real, dt.imag,
                               nsteps, int(renorm)), "dftgpu_run")

    def energy_report(self, wf: Wf, vext: RGrid | None = None):
        e, n, mu = C.c_double(), C.c_double(), C.c_double()
        check(lib().dftgpu_energy_report(self.ptr, wf.ptr, vext.ptr if vext else None, C.byref(e), C.byref(n),
                                         C.byref(mu)), "dftgpu_energy_report")
        return e.value, n.value, mu.value

    # ---- reverse mode (cotangent of psi: g = 2 dJ/dpsi^*)
    def potential_vjp(self, wf: Wf, cot: CGrid, grad_psi: CGrid):
        """grad_psi += (dV_OT/dpsi)^H cot."""
        check(lib().dftgpu_ot_potential_vjp(self.ptr, wf.ptr, cot.ptr, grad_psi.ptr), "dftgpu_ot_potential_vjp")

    def pc_step_vjp(self, wf: Wf, vext: RGrid | None, mu0: float, dt: complex, renorm: bool, cot: CGrid,
                    grad_vext: RGrid | None = None):
        """cot <- cotangent of the step input; grad_vext += dJ/dVext."""
        check(lib().dftgpu_pc_step_vjp(self.ptr, wf.ptr, vext.ptr if vext else None, mu0, dt.real, dt.imag,
                                       int(renorm), cot.ptr, grad_vext.ptr if grad_vext else None),
              "dftgpu_pc_step_vjp")

    def adjoint_run(self, wf: Wf, vext: RGrid | None, mu0: float, dt: complex, nsteps: int, renorm: bool,
                    rho_target: RGrid, grad_vext: RGrid | None = None, grad_psi0: CGrid | None = None,
                    checkpoint_every: int = 0) -> float:
        """J = int (|psi_T|^2 - rho_target)^2 dV after nsteps steps, with its gradients."""
        J = C.c_double()
        check(lib().dftgpu_adjoint_run(self.ptr, wf.ptr, vext.ptr if vext else None, mu0, dt.real, dt.imag, nsteps,
                                       int(renorm), checkpoint_every, rho_target.ptr, C.byref(J),
                                       grad_vext.ptr if grad_vext else None, grad_psi0.ptr if grad_psi0 else None),
              "dftgpu_adjoint_run")
        return J.value

    def free(self):
        if self.ptr:
            lib().dft_ot_free(self.ptr)
        self.ptr = None


def set_precision(prec: int):
    check(lib().dftgpu_set_precision(prec), "dftgpu_set_precision")


def synchronize():
    check(lib().dftgpu_synchronize(), "dftgpu_synchronize")
