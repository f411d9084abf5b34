"""GPU: the allocation-free propagation entry point.

dftgpu_wf_propagate_noalloc exists for callers that cannot call cudaMalloc
(code running inside another component's stream capture, hosts whose own
memory pool owns all device memory, services that may not grow after
start-up).  It takes caller-owned device buffers and uses only the library's
static device scratch.  Here the buffers are owned by torch, i.e. by a
different allocator than the library's, and two steps in a row through the
new entry point must agree with two steps of the allocating entry point
(dftgpu_wf_propagate) within the tolerances the other GPU tests use.

This file is named to be collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-10, 1: 1e-5}


def _psi_and_potential(shape, step, seed):
    rng = np.random.default_rng(seed)
    ax = [(np.arange(n) - n // 2) * step for n in shape]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    rho0 = 0.0218360 * 0.529177210903 ** 3
    psi = np.sqrt(rho0 * (1 + 0.1 * np.cos(2 * np.pi * X / (shape[0] * step)))) \
        * np.exp(0.3j * np.sin(2 * np.pi * Y / (shape[1] * step))) * (1 + 1e-3 * rng.standard_normal(shape))
    V = (rng.standard_normal(shape) + 0.3j * rng.standard_normal(shape)) * 1e-5
    return psi.astype(np.complex128), V.astype(np.complex128)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("shape", [(32, 48, 40), (64, 64, 128), (1, 1, 2048)])
def test_noalloc_propagate_matches_allocating_entry_point(prec, shape):
    """(1, 1, 2048) is a 1-D grid whose z twiddle table is longer than 1024
    entries: the y and x tables must start after it, not inside it."""
    import torch
    import libdft_gb300 as G

    L = G.lib()
    assert L.dftgpu_init(0) == 0
    G.set_precision(prec)
    step, dt = 0.8, 41.3 - 2.0j
    psi, V = _psi_and_potential(shape, step, 21)

    # existing, allocating entry point
    w = G.Wf(shape, step)
    P = G.CGrid(shape, step)
    w.set(psi)
    P.set(V)

    # caller-owned device buffers from another allocator (torch)
    rdt = torch.float64 if prec == 0 else torch.float32
    as_t = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.float64).astype(
        np.float64 if prec == 0 else np.float32)).to("cuda")
    psi_in, pot = as_t(psi), as_t(V)
    psi_out = torch.empty_like(psi_in)
    assert psi_in.dtype == rdt
    nx, ny, nz = shape
    for call in range(2):
        w.propagate(P, dt)
        rc = L.dftgpu_wf_propagate_noalloc(psi_out.data_ptr(), psi_in.data_ptr(), pot.data_ptr(), nx, ny, nz, step,
                                           G.HELIUM_MASS, dt.real, dt.imag, prec, None)
        assert rc == 0, L.dftgpu_last_error_message()
        torch.cuda.synchronize()
        got = psi_out.double().cpu().numpy().view(np.complex128).reshape(shape)
        ref = w.get()
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 3 * TOL[prec], (call, err)
        psi_in.copy_(psi_out)
    w.free()
    P.free()
    G.set_precision(0)


def test_noalloc_rejects_grids_beyond_the_static_scratch():
    import torch
    import libdft_gb300 as G

    L = G.lib()
    assert L.dftgpu_init(0) == 0
    small = torch.zeros(64, device="cuda")   # valid buffers; the size check rejects before any use
    p = small.data_ptr()
    # 256^3 FP32 needs 128 MiB of scratch > 32 MiB
    rc = L.dftgpu_wf_propagate_noalloc(p, p, p, 256, 256, 256, 0.8, G.HELIUM_MASS, 1.0, 0.0, 1, None)
    assert rc == 2
    assert "static scratch" in L.dftgpu_last_error_message().decode()
    L.dftgpu_last_error()


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
def test_noalloc_in_place_allocates_nothing_and_keeps_the_norm(prec):
    """psi_out may be psi_in.  After a first call (which looks up the static
    scratch's address), further calls must not change the device's free
    memory, and in FP32 the norm after many real-time steps must follow the
    allocating entry point (both use unit-circle-rounded twiddles)."""
    import torch
    import libdft_gb300 as G

    L = G.lib()
    assert L.dftgpu_init(0) == 0
    G.set_precision(prec)
    shape, step, dt = (32, 32, 64), 0.8, 41.3 + 0.0j   # real time: the norm is conserved exactly in exact arithmetic
    psi, V = _psi_and_potential(shape, step, 5)
    V = V.real.astype(np.complex128)                   # real potential: unitary step
    w = G.Wf(shape, step)
    P = G.CGrid(shape, step)
    w.set(psi)
    P.set(V)
    as_t = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.float64).astype(
        np.float64 if prec == 0 else np.float32)).to("cuda")
    buf, pot = as_t(psi), as_t(V)
    nx, ny, nz = shape
    call = lambda: L.dftgpu_wf_propagate_noalloc(buf.data_ptr(), buf.data_ptr(), pot.data_ptr(), nx, ny, nz, step,
                                                 G.HELIUM_MASS, dt.real, dt.imag, prec, None)
    assert call() == 0, L.dftgpu_last_error_message()
    w.propagate(P, dt)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    nsteps = 200
    for _ in range(nsteps - 1):
        assert call() == 0, L.dftgpu_last_error_message()
        w.propagate(P, dt)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    got = buf.double().cpu().numpy().view(np.complex128).reshape(shape)
    ref = w.get()
    n0 = np.sum(np.abs(psi) ** 2)
    drift_new = abs(np.sum(np.abs(got) ** 2) / n0 - 1.0)
    drift_ref = abs(np.sum(np.abs(ref) ** 2) / n0 - 1.0)
    # FP32: the drift stays within a small multiple of the allocating path's
    # (a twiddle table with a biased |w|^2 drifts steadily every step);
    # FP64: round-off only
    bound = 2e-12 if prec == 0 else max(3.0 * drift_ref, 2e-6)
    assert drift_new < bound, (drift_new, drift_ref)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < (1e-9 if prec == 0 else 2e-4), err
    w.free()
    P.free()
    G.set_precision(0)
