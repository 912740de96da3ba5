"""The allocation-free grey solve (dnsmc_solve_grey_noalloc) against the
handle API's grey solve, through the C ABI.

That entry point exists for callers that cannot allocate device memory while
they run (a host code whose pool allocator owns all free device memory, or a
run with a fixed footprint after start-up): its intermediate buffers live in
one fixed file-scope device array.  Two calls in a row on different fields
must each equal the handle API's result bit for bit (the tolerance of the
other parity tests), which also shows that the shared scratch is reset
between calls.  The grids cover the three automatic packet shapes (8 x 8, and
16 x 4 / 32 x 2 for short k), j and k sizes that do not divide into packets,
and the largest grid the fixed array holds.  Kept in its own file so it is
collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import _lib

GPU = pytest.mark.gpu


def field(ni, nj, nk, seed):
    rng = np.random.default_rng(seed)
    i = (np.arange(ni) + 0.5) / ni
    base = 350 + 900 * 4 * i * (1 - i)
    f = 1 + 0.05 * rng.uniform(-1, 1, (nk, nj, ni))
    return np.ascontiguousarray(base[None, None, :] * f, dtype=np.float32)


def _torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA (used only to hold the caller's device arrays)")
    return torch


def _noalloc(lib, torch, cfg, xu, T):
    """One allocation-free solve of T; returns (Q, var, status) on the host."""
    ni, nj, nk = cfg.imax, cfg.jmax, cfg.kmax
    dT = torch.from_numpy(T).cuda()
    dQ = torch.full((nk, nj, ni), float("nan"), dtype=torch.float64, device="cuda")
    dV = torch.full((nk, nj, ni), float("nan"), dtype=torch.float64, device="cuda")
    dS = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.dnsmc_solve_grey_noalloc(ctypes.byref(cfg), xu.ctypes.data_as(_lib.c_float_p),
                                      ctypes.c_void_p(dT.data_ptr()), ctypes.c_void_p(dQ.data_ptr()),
                                      ctypes.c_void_p(dV.data_ptr()), ctypes.c_void_p(dS.data_ptr()), None)
    assert rc == 0, lib.dnsmc_last_error()
    torch.cuda.synchronize()
    return dQ.cpu().numpy(), dV.cpu().numpy(), int(dS.cpu().numpy()[0])


@GPU
@pytest.mark.parametrize("ni,nj,nk", [(32, 32, 16),   # 8 x 8 packets
                                      (12, 40, 3),    # kmax < 4: 32 x 2 packets
                                      (10, 36, 6),    # 16 x 4 packets, j and k ragged
                                      (20, 27, 13),   # 8 x 8 packets, j and k ragged
                                      (64, 64, 64)])  # the largest grid the fixed array holds
def test_noalloc_grey_matches_handle_api_twice(ni, nj, nk):
    torch = _torch_cuda()
    rays = (2, 48) if ni * nj * nk < 64 ** 3 else (2, 8)
    cfg = D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853, Lz=3.1415927,
                           stretched_x=1, T_west=300.0, T_east=420.0, kappa=1.3, nvar=rays[0], photmax=rays[1],
                           seed=2024)
    lib = _lib.load()
    for call, seed in enumerate((1, 2)):
        T = field(ni, nj, nk, seed)
        s = D.Solver(cfg)
        s.set_fields(T)
        s.set_rays(cfg.nvar * cfg.photmax)
        Qref, Sref = s.solve(timeout_s=120)
        xu, _, _ = s.geometry()
        s.close()
        Q, V, status = _noalloc(lib, torch, cfg, xu, T)
        assert status == 0, f"call {call}: status {status:#x}"
        np.testing.assert_array_equal(Q, Qref[0], err_msg=f"call {call}")
        np.testing.assert_array_equal(np.sqrt(V), Sref[0], err_msg=f"call {call}")


@GPU
def test_noalloc_reports_bad_temperature_then_recovers():
    """A temperature of 0 sets DNSMC_STATUS_BAD_FIELD in the caller's status
    word; the next call on a good field reports 0 again (the shared status
    word is cleared per call)."""
    torch = _torch_cuda()
    ni, nj, nk = 16, 16, 8
    cfg = D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853, Lz=3.1415927,
                           stretched_x=0, T_west=300.0, T_east=300.0, kappa=1.0, nvar=2, photmax=8, seed=7)
    xu = np.linspace(0, 2.0, ni + 1).astype(np.float32)
    lib = _lib.load()
    T = field(ni, nj, nk, 3)
    T[2, 5, 7] = 0.0
    _, _, status = _noalloc(lib, torch, cfg, xu, T)
    assert status & _lib.STATUS_BAD_FIELD, f"status {status:#x}"
    _, _, status = _noalloc(lib, torch, cfg, xu, field(ni, nj, nk, 4))
    assert status == 0, f"status {status:#x}"


def test_noalloc_rejects_grids_beyond_its_limit():
    cfg = D.default_config(model=D.MODEL_GREY, imax=128, jmax=64, kmax=64)
    xu = np.linspace(0, 1, 129).astype(np.float32)
    lib = _lib.load()
    rc = lib.dnsmc_solve_grey_noalloc(ctypes.byref(cfg), xu.ctypes.data_as(_lib.c_float_p), ctypes.c_void_p(1),
                                      ctypes.c_void_p(1), ctypes.c_void_p(1), None, None)
    assert rc == _lib.ERR_ARG
    assert b"allocation-free limit" in lib.dnsmc_last_error()


@pytest.mark.parametrize("max_steps", [0, (1 << 22) + 1])
def test_noalloc_rejects_step_caps_outside_the_exact_range(max_steps):
    """The march counts crossings in FP32, exact below 2^22: the handle API's
    bound on max_steps holds here too."""
    cfg = D.default_config(model=D.MODEL_GREY, imax=16, jmax=16, kmax=8, max_steps=max_steps)
    xu = np.linspace(0, 1, 17).astype(np.float32)
    lib = _lib.load()
    rc = lib.dnsmc_solve_grey_noalloc(ctypes.byref(cfg), xu.ctypes.data_as(_lib.c_float_p), ctypes.c_void_p(1),
                                      ctypes.c_void_p(1), ctypes.c_void_p(1), None, None)
    assert rc == _lib.ERR_ARG
    assert b"max_steps must be in [1, 4194304]" in lib.dnsmc_last_error()
