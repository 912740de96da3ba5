"""CPU tests of the packet scheme itself, through the oracle's replay with the
library's own geometry and sampling tables (built on the host, no GPU):

* the isothermal grey slab agrees with the analytic E_2 solution;
* on the reference correlated-k tables the packet estimator (shared
  direction + alias-drawn spectral sample per 32-cell packet, band groups)
  agrees cell by cell with the reference-structured estimator
  (code/mc_gpu.cu:44-438) -- both restated in the oracle;
* FP32 and FP64 replays differ by rounding only.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import dnsmc_gb300 as D
from oracle import oracle as O
from tables_io import write_ck_tables


def smooth_field(ni, nj, nk, lo, hi, seed):
    rng = np.random.default_rng(seed)
    i = (np.arange(ni) + 0.5) / ni
    j = np.arange(nj) / nj
    k = np.arange(nk) / nk
    base = lo + (hi - lo) * 4 * i * (1 - i)
    f = (np.sin(2 * np.pi * j)[None, :, None] * np.cos(2 * np.pi * k)[:, None, None] * 0.04
         + rng.normal(0, 0.01, (nk, nj, ni)))
    return (base[None, None, :] * (1 + f)).astype(np.float32)


def replay(s, T, x, N, use_double, threads=0):
    ni, nj, nk = s.cfg.imax, s.cfg.jmax, s.cfg.kmax
    s._rays, s._nfields = N, 1
    c, keep = O.packet_config(s, T, x, use_double=use_double)
    ng = 1 if s.cfg.model == D.MODEL_GREY else s.sampling()["n_groups"]
    tal, steps = O.packet_mc(c, ng, ni * nj * nk, threads=threads)
    tal = tal.reshape(1, ng, ni, nk, nj, 2).transpose(0, 1, 3, 4, 2, 5)[0]
    m = tal[..., 0] / N
    if s.cfg.sampler == D.SAMPLER_RQMC:
        B = s.cfg.nvar
        v = np.maximum(0, tal[..., 1] / B - m * m) / (B - 1)
    else:
        v = np.maximum(0, tal[..., 1] / N - m * m) / (N - 1)
    return m.sum(0), np.sqrt(v.sum(0)), steps


def test_packet_replay_grey_slab_analytic():
    ni, nj, nk = 32, 32, 8
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853, Lz=3.1415927,
                                  stretched_x=0, T_west=0.0, T_east=300.0, kappa=1.0, seed=3))
    Q, S, _ = replay(s, np.full((nk, nj, ni), 1000.0, np.float32), None, 1024, 1)
    ta, tb = s.packet_shape()  # one cell per packet: the cells of a packet share rays
    npk = (nk // tb) * (nj // ta)
    q = Q[::tb, ::ta, :].mean((0, 1))
    se = np.sqrt((S[::tb, ::ta, :] ** 2).sum((0, 1))) / npk
    ex = O.slab_divq((np.arange(ni) + 0.5) * 2.0 / ni, 2.0, 1.0, 1000.0, 0.0, 300.0)
    z = (q - ex) / se
    assert np.abs(z).max() < 4.0 and math.sqrt((z ** 2).mean()) < 1.5, z
    s.close()


@pytest.mark.parametrize("groups", [1, 4])
def test_packet_scheme_matches_reference_estimator_ck(tmp_path, ck_tables, groups):
    write_ck_tables(str(tmp_path), ck_tables)
    ni, nj, nk = 12, 32, 4
    Lx, Ly, Lz = 0.3, 0.6, 0.15
    s = D.Solver(D.default_config(model=D.MODEL_CK, imax=ni, jmax=nj, kmax=nk, Lx=Lx, Ly=Ly, Lz=Lz, stretched_x=1,
                                  T_west=520, T_east=700, seed=13, n_groups=groups))
    s.load_reference_tables(str(tmp_path), D.MODEL_CK)
    T = smooth_field(ni, nj, nk, 560, 1000, 13)
    s.prepare_sampling(max(float(T.max()), 700.0))
    Q, S, _ = replay(s, T, None, 3000, 1)
    cells = np.array([(i, 0, k) for i in range(ni) for k in range(nk)])
    Tf = np.zeros((nk + 2, nj + 2, ni + 2), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = T
    tables = dict(Tnb=ck_tables["Tnb"], kq=ck_tables["kq"], wvc=ck_tables["wvc"], prob=ck_tables["prob"],
                  probg=ck_tables["probg"], kP=ck_tables["kP"])
    r = O.ref_mc(Tf.ravel(), cells + 1, imax=ni, jmax=nj, kmax=nk, Lx=Lx, Ly=Ly, Lz=Lz, T_west=520, T_east=700,
                 model=0, tables=tables, nvar=3, photmax=1000, grid_num=1, stretched=1, use_double=1, seed=9)
    qg = Q[cells[:, 2], cells[:, 1], cells[:, 0]]
    sg = S[cells[:, 2], cells[:, 1], cells[:, 0]]
    z = (qg - r["Q"]) / np.sqrt(sg ** 2 + r["se"] ** 2)
    assert (np.abs(z) > 3).sum() <= 2, z
    assert 0.5 < math.sqrt((z ** 2).mean()) < 1.5, z
    s.close()


def test_fp32_replay_close_to_fp64():
    ni, nj, nk = 8, 32, 2
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=300, kappa=2.0, seed=8))
    T = smooth_field(ni, nj, nk, 400, 1300, 8)
    a, sa, st_a = replay(s, T, None, 256, 0)
    b, sb, st_b = replay(s, T, None, 256, 1)
    assert abs(st_a - st_b) <= 1e-4 * st_b
    assert np.abs(a - b).max() < 1e-3 * np.abs(b).max()
    s.close()


def test_rqmc_unbiased_and_replicate_variance_is_calibrated():
    """RQMC (shifted Sobol' replicates) on the grey slab: unbiased against the
    analytic solution, and the replicate variance estimate matches the
    seed-to-seed variance of the estimates."""
    ni, nj, nk = 16, 32, 4
    ex = O.slab_divq((np.arange(ni) + 0.5) * 2.0 / ni, 2.0, 1.0, 1000.0, 0.0, 300.0)
    Qs, Vs = [], []
    for seed in range(6):
        s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853,
                                      Lz=3.1415927, stretched_x=0, T_west=0.0, T_east=300.0, kappa=1.0, seed=50 + seed,
                                      sampler=D.SAMPLER_RQMC, nvar=4))
        Q, S, _ = replay(s, np.full((nk, nj, ni), 1000.0, np.float32), None, 256, 1)
        m = S ** 2
        ta, tb = s.packet_shape()  # one cell per packet: the cells of a packet share rays
        Qs.append(Q[::tb, ::ta, :].reshape(-1, ni))
        Vs.append(m[::tb, ::ta, :].reshape(-1, ni))
        s.close()
    Qs, Vs = np.array(Qs), np.array(Vs)
    emp = Qs.var(0, ddof=1).mean()
    est = Vs.mean()
    assert 0.5 < est / emp < 2.0, (est, emp)
    q = Qs.mean((0, 1))
    se = np.sqrt(emp / (Qs.shape[0] * Qs.shape[1]))
    z = (q - ex) / se
    assert np.abs(z).max() < 4.5, z


def test_cv_replay_isothermal_surrogate_cancels():
    """Replay with the control variate on an isothermal grey slab whose
    surrogate equals the medium: X - Y vanishes up to FP32 rounding."""
    import ctypes
    ni, nj, nk = 16, 32, 2
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=0.0, T_east=300.0, kappa=1.0, seed=4))
    T = np.full((nk, nj, ni), 1000.0, np.float32)
    s._rays, s._nfields = 64, 1
    c, keep = O.packet_config(s, T, None, use_double=0)
    sk = np.full((1, 1, ni), 1.0, np.float32)
    sI = np.full((1, 1, ni), np.float32(1000.0) ** 4, np.float32)
    c.cv = 1
    c.sur_k = sk.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    c.sur_I = sI.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    beta = np.zeros((1, 1, nk, nj, ni, 2), np.float32)
    beta[..., 0] = 1.0  # Y_a alone: the surrogate equals the medium
    c.beta = beta.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    tal, _ = O.packet_mc(c, 1, ni * nj * nk)
    c.cv = 0
    tal0, _ = O.packet_mc(c, 1, ni * nj * nk)
    assert np.abs(tal[..., 0]).max() < 1e-4 * np.abs(tal0[..., 0]).max()
    s.close()


def test_march_expm1_within_1p5_ulp():
    """The march's FP32 expm1 (shifter-rounded Cody-Waite reduction, degree-4
    minimax polynomial; the device runs the same operations) against float64
    expm1 over x in [-90, 0], magnitudes from 1e-30 up: within 1.5 ulp of the
    float32 result, and -1 exactly below the clamp at -87."""
    rng = np.random.default_rng(0)
    x = np.concatenate([-np.logspace(-30, np.log10(87.0), 200001), -rng.uniform(0, 90, 200000),
                        [0.0, -0.0, -87.0, -100.0, -1e-45]]).astype(np.float32)
    y = O.expm1n(x).astype(np.float64)
    e = np.expm1(x.astype(np.float64))
    ulp = np.spacing(np.abs(e).astype(np.float32)).astype(np.float64)
    ulp[ulp == 0] = np.spacing(np.float32(0))
    err = np.abs(y - e) / ulp
    assert err.max() <= 1.5, (err.max(), x[np.argmax(err)])
    assert np.all(O.expm1n(np.array([-88.0, -200.0, -1e30], np.float32)) == -1.0)
