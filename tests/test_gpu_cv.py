"""GPU tests of the control variate (CV): Y is the same ray through the
medium of plane-averaged T and x_H2O, its flight read from a table of the
straight flight per (field, spectral sample, plane) and interpolated in
sqrt|mu|; the march tallies X - beta*Y and the exact mean beta*E[Y] of the
tabulated Y is added back.

* bit-exact tallies vs the oracle's FP32 replay (which builds its own table),
  with beta = 1 and with a per-cell beta array;
* the device table equals the oracle's bit for bit, its means (Jhat) the
  oracle's, and they approach the float64 quadrature of the continuous walk;
  E[Y] per cell matches its definition;
* isothermal slab: the surrogate is the medium, so Q equals the analytic
  solution with a variance left only by the interpolation;
* unbiased: CV and plain MC agree cell by cell on the correlated-k channel;
* the variance falls by more than 10x at equal rays.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import synth
from oracle import oracle as O
from test_gpu_parity import group_mean_var, region_tally_to_dense, rays_per_cell, smooth_field

pytestmark = pytest.mark.gpu


def assert_bitexact_cv(s, T, x=None):
    Q, S = s.solve(timeout_s=120)
    Qg, Vg = s.group_results()
    ng = Qg.shape[1]
    c, keep = O.packet_config(s, T, x)
    i0, i1, j0, j1, k0, k1 = s._region
    tal, steps = O.packet_mc(c, ng, (i1 - i0) * (j1 - j0) * (k1 - k0))
    tal = region_tally_to_dense(tal, s, ng)
    muY = s.cv_data()["muY"]
    if getattr(s, "_beta_dev", False):
        beta = s.cv_beta()
    elif s._beta is not None:
        beta = s._beta
    else:
        beta = np.zeros(muY.shape, np.float32)
        beta[..., 0], beta[..., 1] = 1.0, -1.0
    B = s.cfg.nvar
    for g in range(ng):
        N = rays_per_cell(s, g)
        m, v = group_mean_var(tal[:, g], N, B, s.cfg.sampler == D.SAMPLER_RQMC)
        m = m + beta[:, g, ..., 0].astype(np.float64) * muY[:, g, ..., 0]
        m = m + beta[:, g, ..., 1].astype(np.float64) * muY[:, g, ..., 1]
        np.testing.assert_array_equal(Qg[:, g], m)
        np.testing.assert_array_equal(Vg[:, g], v)
    assert s.counters().steps == steps
    return Q, S


def test_cv_bitexact_grey():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=8, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=500, kappa=1.5, seed=11, control_variate=1))
    T = smooth_field(16, 32, 8, 400, 1200, 1)
    s.set_fields(T)
    s.set_rays(64)
    assert_bitexact_cv(s, T)
    s.close()


def test_cv_bitexact_table_x_with_beta():
    tb = synth.ck_table(nbands=12, nq=8, nT=20, nX=4, seed=6)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=8, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=400, T_east=450, seed=31, n_groups=3,
                                  sampler=D.SAMPLER_RQMC, nvar=4, local_sampling=1, control_variate=1))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(8, 32, 4, 450, 1700, 41)
    x = (0.1 + 0.05 * np.random.default_rng(3).uniform(-1, 1, (4, 32, 8))).astype(np.float32)
    s.set_fields(T, x)
    s.set_rays(32)
    assert_bitexact_cv(s, T, x)
    beta = np.random.default_rng(5).uniform(-1.5, 1.5, (1, 3, 4, 32, 8, 2)).astype(np.float32)
    s.set_cv_beta(beta)
    assert_bitexact_cv(s, T, x)
    s.close()


def test_cv_bitexact_table_t_only():
    """A table without an x_H2O axis (k(band, g, T)): the march reads one
    column per row and E[Y] comes from the T-only node sums; tallies stay
    bit-exact and E[Y] matches its per-sample float64 definition."""
    tb = synth.ck_table(nbands=8, nq=4, nT=20, nX=4, seed=13)
    k3 = np.ascontiguousarray(tb["k"][..., 2])                 # x = 0.1 slice
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=12, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=1, T_west=420, T_east=380, seed=17, n_groups=2, control_variate=1))
    s.set_table(k3, tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"])
    assert s.table_info()["nX"] == 1
    T = smooth_field(12, 32, 4, 450, 1700, 23)
    s.set_fields(T)
    s.set_rays(32)
    assert_bitexact_cv(s, T)
    cv = s.cv_data()
    from test_capi import alias_distribution
    smp = s.sampling()
    t = s.table()
    Tg = tb["T0"] + tb["dT"] * np.arange(20)
    nq = 4
    scale = np.abs(cv["muY"]).max()
    for (i, j, k) in ((0, 0, 0), (6, 9, 1), (11, 31, 3)):
        for g in range(2):
            p = alias_distribution(smp, g)
            a, e_ = int(smp["group_start"][g]), int(smp["group_start"][g + 1])
            acc = accB = 0.0
            for e in range(a, e_):
                b, gq = smp["band"][e], smp["gq"][e]
                ki = np.interp(T[k, j, i], Tg, t["k"][b, gq, :, 0])
                ib = np.interp(T[k, j, i], Tg, t["Ib"][b])
                sid = b * nq + gq
                acc += smp["W"][e] * p[e - a] * ki * (ib - cv["Jhat"][0, sid, i, 0])
                accB += smp["W"][e] * p[e - a] * ki * (ib - cv["sur"][0, sid, i, 1]) * cv["Jhat"][0, sid, i, 1]
            mu = cv["muY"][0, g, k, j, i]
            assert abs(mu[0] - acc) <= 1e-4 * abs(acc) + 1e-9 * scale
            assert abs(mu[1] - accB) <= 1e-4 * abs(accB) + 1e-9 * scale
    s.close()


def test_cv_table_and_mean_match_oracle():
    tb = synth.ck_table(nbands=6, nq=4, nT=20, nX=4, seed=9)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=12, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=1, T_west=420, T_east=380, seed=3, n_groups=2, control_variate=1))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(12, 32, 4, 450, 1700, 12)
    x = (0.1 + 0.05 * np.random.default_rng(4).uniform(-1, 1, (4, 32, 12))).astype(np.float32)
    s.set_fields(T, x)
    s.set_rays(8)
    s.solve(timeout_s=60)
    cv = s.cv_data()
    np.testing.assert_allclose(cv["layer"][0, :, 0], T.mean((0, 1)), rtol=1e-6)
    np.testing.assert_allclose(cv["layer"][0, :, 1], x.mean((0, 1)), rtol=1e-5)
    # the oracle's table of the device's layer-mean medium, and its means
    c, keep = O.packet_config(s, T[None], x[None])
    tab_o, JA_o = O.cv_table(c)
    np.testing.assert_array_equal(s.cv_table(), tab_o)
    np.testing.assert_allclose(cv["Jhat"], JA_o, rtol=1e-12, atol=0)
    xu, _, _ = s.geometry()
    smp = s.sampling()
    ibw = smp["ibw"].reshape(2, -1)
    nq = 4
    for sid in (0, 5, 17, 23):  # the continuous flight's means, by quadrature: the tabulated
        # surrogate is a close stand-in (its own means are what E[Y] uses)
        J = O.cv_jhat(cv["sur"][0, sid, :, 0], cv["sur"][0, sid, :, 1], xu, None, ibw[0, sid // nq],
                      ibw[1, sid // nq])
        np.testing.assert_allclose(cv["Jhat"][0, sid, :, 0], J[:, 0], rtol=2e-3)
        np.testing.assert_allclose(cv["Jhat"][0, sid, :, 1], J[:, 1], rtol=5e-3, atol=1e-4)
    # E[Y] per cell from its definition: sum over the group's samples of
    # C_s k_i (Ib_i - Jhat), C_s = W_s * q(s) of the (single-bin) alias table
    from test_capi import alias_distribution
    t = s.table()
    Tg = tb["T0"] + tb["dT"] * np.arange(20)
    Xg = tb["X0"] + tb["dX"] * np.arange(4)
    for (i, j, k) in ((0, 0, 0), (5, 17, 2), (11, 31, 3)):
        for g in range(2):
            p = alias_distribution(smp, g)
            a, e_ = int(smp["group_start"][g]), int(smp["group_start"][g + 1])
            acc = accB = 0.0
            for e in range(a, e_):
                b, gq = smp["band"][e], smp["gq"][e]
                kv = np.array([np.interp(x[k, j, i], Xg, t["k"][b, gq, it]) for it in range(20)])
                ki = np.interp(T[k, j, i], Tg, kv)
                ib = np.interp(T[k, j, i], Tg, t["Ib"][b])
                sid = b * nq + gq
                acc += smp["W"][e] * p[e - a] * ki * (ib - cv["Jhat"][0, sid, i, 0])
                accB += smp["W"][e] * p[e - a] * ki * (ib - cv["sur"][0, sid, i, 1]) * cv["Jhat"][0, sid, i, 1]
            mu = cv["muY"][0, g, k, j, i]
            scale = np.abs(cv["muY"]).max()
            assert abs(mu[0] - acc) <= 1e-4 * abs(acc) + 1e-9 * scale
            assert abs(mu[1] - accB) <= 1e-4 * abs(accB) + 1e-9 * scale
    s.close()


def test_cv_isothermal_slab():
    """The surrogate is the medium itself: what is left of each ray's X - Y
    is the gap between the walk and its tabulated interpolant, so Q is the
    analytic solution within its (tiny) standard error, and that error is
    below 1e-3 of the plain estimate's.  The rays' cut-off is lowered to
    toll = 1e-6: at the default 1e-3 the intensity a ray would still carry
    to the cold walls beyond optical depth ln(1/toll) is absorbed in place,
    which moves Q by about 5e-5 of itself -- many standard errors here."""
    ni, nj, nk = 32, 32, 8
    out = []
    for cv in (1, 0):
        s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853,
                                      Lz=3.1415927, stretched_x=0, T_west=0.0, T_east=300.0, kappa=1.0, seed=3,
                                      toll=1e-6, control_variate=cv))
        s.set_fields(np.full((nk, nj, ni), 1000.0, np.float32))
        s.set_rays(16)
        out.append(s.solve(timeout_s=60))
        s.close()
    (Q, S), (Qp, Sp) = out
    yc = (np.arange(ni) + 0.5) * 2.0 / ni
    exact = O.slab_divq(yc, 2.0, 1.0, 1000.0, 0.0, 300.0)
    err = np.abs(Q[0] - exact[None, None, :])
    # sigma from 16 rays per cell: z follows Student's t with 15 degrees of freedom
    assert (err <= 7.0 * S[0] + 1e-6 * np.abs(exact).max()).all(), (err / S[0]).max()
    assert math.sqrt(float(((Q[0] - exact) ** 2).mean() / (S[0] ** 2).mean())) < 1.5
    assert S.max() < 1e-3 * Sp.max(), (S.max(), Sp.max())


def _channel_pair(seed_plain, seed_cv, rays, n=32, sampler=D.SAMPLER_IID):
    d = synth.ck_channel(n, 0)
    tb = synth.ck_table()
    out = []
    for cv, seed in ((0, seed_plain), (1, seed_cv)):
        s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi,
                                      Lz=math.pi, stretched_x=0, T_west=400, T_east=400, n_groups=8, seed=seed,
                                      sampler=sampler, nvar=4, local_sampling=1, control_variate=cv))
        s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
        s.set_fields(d["T"], d["x"])
        s.set_rays(rays)
        out.append(s.solve(timeout_s=120))
        shape = s.packet_shape()
        s.close()
    return out, shape


def test_cv_unbiased_and_variance_reduction_ck_channel():
    """IID rays (sigma from 128 rays per cell and group), independent seeds."""
    ((Qp, Sp), (Qc, Sc)), (ta, tb) = _channel_pair(101, 202, 128)
    z = (Qc - Qp) / np.sqrt(Sc ** 2 + Sp ** 2)
    z = z[0][::tb, ::ta, :]  # one cell per packet: independent estimates
    assert math.sqrt(float((z ** 2).mean())) < 1.25, z
    assert (np.abs(z) > 3).mean() < 0.01 and np.abs(z).max() < 5.5
    ratio = float((Sp ** 2).mean() / (Sc ** 2).mean())
    assert ratio > 10.0, ratio


def test_cv_moments_bitexact():
    import ctypes
    tb = synth.ck_table(nbands=8, nq=4, nT=20, nX=4, seed=7)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=6, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=400, T_east=450, seed=8, n_groups=2, control_variate=1,
                                  cv_moments=1))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(6, 32, 4, 450, 1700, 2)
    x = (0.1 + 0.05 * np.random.default_rng(6).uniform(-1, 1, (4, 32, 6))).astype(np.float32)
    s.set_fields(T, x)
    s.set_rays(24)
    s.solve(timeout_s=60)
    mom = s.cv_moments()
    c, keep = O.packet_config(s, T, x)
    rm = np.zeros((1, 2, 6 * 32 * 4, 9))
    c.moments = rm.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    O.packet_mc(c, 2, 6 * 32 * 4)
    rm = rm.reshape(1, 2, 6, 4, 32, 9).transpose(0, 1, 3, 4, 2, 5)
    np.testing.assert_array_equal(mom, rm)
    assert np.abs(mom[..., 0]).max() > 0
    s.close()


def test_cv_two_term_default_beats_single_term():
    d = synth.ck_channel(32, 0)
    tb = synth.ck_table()
    var = []
    for beta_b in (0.0, -1.0):
        s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=32, jmax=32, kmax=32, Lx=2.0, Ly=2 * math.pi,
                                      Lz=math.pi, stretched_x=0, T_west=400, T_east=400, n_groups=8, seed=5,
                                      local_sampling=1, control_variate=1))
        s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
        s.set_fields(d["T"], d["x"])
        beta = np.zeros((1, 8, 32, 32, 32, 2), np.float32)
        beta[..., 0], beta[..., 1] = 1.0, beta_b
        s.set_cv_beta(beta)
        s.set_rays(128)
        Q, S = s.solve(timeout_s=120)
        var.append(float((S ** 2).mean()))
        s.close()
    assert var[0] / var[1] > 1.2, var


def test_cv_table_with_many_planes():
    """1500 wall-normal planes: the table's sweep keeps 44 bytes a plane in
    shared memory (66 KB here, past the default 48 KB), its table equals the
    oracle's bit for bit and the march's tallies the replay's on a band of
    planes in the middle."""
    ni, nj, nk = 1500, 16, 8
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=1, T_west=300, T_east=500, kappa=3.0, seed=5, control_variate=1))
    i = (np.arange(ni) + 0.5) / ni
    T = np.ascontiguousarray(np.broadcast_to((400 + 800 * 4 * i * (1 - i))[None, None, :], (nk, nj, ni)),
                             dtype=np.float32)
    s.set_fields(T)
    s.set_region(700, 708, 0, nj, 0, nk)
    s.set_rays(16)
    assert_bitexact_cv(s, T)
    cv = s.cv_data()
    c, keep = O.packet_config(s, T[None], None)
    tab_o, JA_o = O.cv_table(c)
    np.testing.assert_array_equal(s.cv_table(), tab_o)
    np.testing.assert_allclose(cv["Jhat"], JA_o, rtol=1e-12, atol=0)
    s.close()
