"""GPU: grid checkpoints on a caller's stream and rgrid_power.

libdft's 1-D drivers restart by opening the checkpoint themselves and
reading it with cgrid_read(gwf->grid, fp) (examples/1d-bubble/bubble-1d.c:164-170,
examples/1d-soliton/soliton-1d.c:93-99); the soliton drivers form the
amplitude with rgrid_power(grid, grid, 0.5) (examples/soliton/soliton.c:96).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class CGridHead(C.Structure):
    """The public head of cgrid (include/dftgpu.h)."""
    _fields_ = [("value", C.c_void_p), ("nx", C.c_long), ("ny", C.c_long), ("nz", C.c_long)] + \
               [(n, C.c_double) for n in ("step", "x0", "y0", "z0", "kx0", "ky0", "kz0")] + [("prec", C.c_int)]


class RGridHead(C.Structure):
    _fields_ = [("value", C.c_void_p), ("nx", C.c_long), ("ny", C.c_long), ("nz", C.c_long)] + \
               [(n, C.c_double) for n in ("step", "x0", "y0", "z0")] + [("prec", C.c_int)]


def head(ptr, cls):
    return C.cast(ptr, C.POINTER(cls))[0]


@pytest.mark.parametrize("prec", [0, 1])
def test_stream_grid_io_and_power(gpu, tmp_path, prec):
    """cgrid_write / rgrid_write and cgrid_read / rgrid_read on a stream the
    caller opens, as libdft's 1-D drivers restart (examples/1d-bubble/bubble-1d.c:164-170):
    two bodies in one file, read into a given grid and into a NULL grid (then
    allocated with the file's shape, step and origin); a complex body is
    refused by a real grid.  rgrid_power (examples/soliton/soliton.c:96)
    against numpy, also in place as the drivers call it."""
    L = gpu.lib()
    gpu.set_precision(prec)
    L.dftgpu_last_error()                 # start from a clear error state
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    step = 0.5
    for shape in ((6, 4, 10), (1, 1, 64)):
        rng = np.random.default_rng(5)
        c = gpu.CGrid(shape, step)
        c.set(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
        L.cgrid_set_momentum(c.ptr, 0.1, 0.0, -0.3)
        r = gpu.RGrid(shape, step)
        r.set(rng.uniform(0.5, 2.0, shape))
        L.rgrid_set_origin(r.ptr, 0.5, -1.0, 2.0)
        path = str(tmp_path / ("chk-%d.grd" % shape[0])).encode()
        fp = libc.fopen(path, b"wb")
        assert fp
        L.cgrid_write(c.ptr, fp)
        L.rgrid_write(r.ptr, fp)
        assert libc.fclose(fp) == 0
        assert L.dftgpu_last_error() == 0
        d = gpu.CGrid(shape, step)
        fp = libc.fopen(path, b"rb")
        assert L.cgrid_read(d.ptr, fp) == d.ptr
        p = L.rgrid_read(None, fp)
        libc.fclose(fp)
        assert p and L.dftgpu_last_error() == 0
        s = gpu.RGrid(shape, step, ptr=p)
        assert np.array_equal(d.get(), c.get())
        rv = r.get()
        assert np.array_equal(s.get(), rv)
        hd, hs = head(d.ptr, CGridHead), head(p, RGridHead)
        assert (hd.kx0, hd.ky0, hd.kz0) == (0.1, 0.0, -0.3)
        assert (hs.nx, hs.ny, hs.nz, hs.step, hs.x0, hs.y0, hs.z0) == shape + (step, 0.5, -1.0, 2.0)
        fp = libc.fopen(path, b"rb")
        assert not L.rgrid_read(s.ptr, fp)
        libc.fclose(fp)
        assert L.dftgpu_last_error() == 1                                   # DFTGPU_ERR_ARG
        assert np.array_equal(s.get(), rv)

        tol = 4e-15 if prec == 0 else 1e-6
        q = gpu.RGrid(shape, step)
        L.rgrid_power(q.ptr, r.ptr, 0.5)
        assert L.dftgpu_last_error() == 0
        assert np.abs(q.get() - np.sqrt(rv)).max() <= tol * np.sqrt(rv).max()
        L.rgrid_power(r.ptr, r.ptr, 2.0)
        assert np.abs(r.get() - rv ** 2).max() <= tol * (rv ** 2).max()
        for g in (q, s, r, d, c):
            g.free()
    gpu.set_precision(0)
