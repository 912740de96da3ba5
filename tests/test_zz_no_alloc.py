"""The allocation-free grey solve (dnsmc_solve_grey_noalloc) against the
handle API's grey solve, through the C ABI.

That entry point exists for callers that cannot allocate device memory while
they run (a host code whose pool allocator owns all free device memory, or a
run with a fixed footprint after start-up): its intermediate buffers live in
one fixed file-scope device array.  Two calls in a row on different fields
must each equal the handle API's result bit for bit (the tolerance of the
other parity tests), which also shows that the shared scratch is reset
between calls.  Kept in its own file so it is collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import _lib

pytestmark = pytest.mark.gpu


def field(ni, nj, nk, seed):
    rng = np.random.default_rng(seed)
    i = (np.arange(ni) + 0.5) / ni
    base = 350 + 900 * 4 * i * (1 - i)
    f = 1 + 0.05 * rng.uniform(-1, 1, (nk, nj, ni))
    return np.ascontiguousarray(base[None, None, :] * f, dtype=np.float32)


def test_noalloc_grey_matches_handle_api_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA (used only to hold the caller's device arrays)")
    ni, nj, nk = 32, 32, 16
    cfg = D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853, Lz=3.1415927,
                           stretched_x=1, T_west=300.0, T_east=420.0, kappa=1.3, nvar=2, photmax=48, seed=2024)
    lib = _lib.load()
    for call, seed in enumerate((1, 2)):
        T = field(ni, nj, nk, seed)
        s = D.Solver(cfg)
        s.set_fields(T)
        s.set_rays(cfg.nvar * cfg.photmax)
        Qref, Sref = s.solve(timeout_s=60)
        xu, _, _ = s.geometry()
        s.close()
        dT = torch.from_numpy(T).cuda()
        dQ = torch.full((nk, nj, ni), float("nan"), dtype=torch.float64, device="cuda")
        dV = torch.full((nk, nj, ni), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.dnsmc_solve_grey_noalloc(ctypes.byref(cfg), xu.ctypes.data_as(_lib.c_float_p),
                                          ctypes.c_void_p(dT.data_ptr()), ctypes.c_void_p(dQ.data_ptr()),
                                          ctypes.c_void_p(dV.data_ptr()), None)
        assert rc == 0, lib.dnsmc_last_error()
        torch.cuda.synchronize()
        Q = dQ.cpu().numpy()
        V = dV.cpu().numpy()
        np.testing.assert_array_equal(Q, Qref[0], err_msg=f"call {call}")
        np.testing.assert_array_equal(np.sqrt(V), Sref[0], err_msg=f"call {call}")


def test_noalloc_rejects_grids_beyond_its_limit():
    cfg = D.default_config(model=D.MODEL_GREY, imax=128, jmax=64, kmax=64)
    xu = np.linspace(0, 1, 129).astype(np.float32)
    lib = _lib.load()
    rc = lib.dnsmc_solve_grey_noalloc(ctypes.byref(cfg), xu.ctypes.data_as(_lib.c_float_p), ctypes.c_void_p(1),
                                      ctypes.c_void_p(1), ctypes.c_void_p(1), None)
    assert rc == _lib.ERR_ARG
    assert b"allocation-free limit" in lib.dnsmc_last_error()
