"""The oracle's FP64 control-variate solution (oracle.fp64_cv_solution), the
reference against which the bench states the error of a timed field.

* its exact means E[Y] (orc_cv_mean, C, float64) equal the sums of the
  definition built here from the Python quadrature oracle.cv_jhat;
* it agrees with the plain FP64 packet replay (no control variate) within
  their combined statistical error, so the control variate it adds back is
  unbiased, and the layer stride leaves the solved layers unchanged.
Host only (no GPU).
"""
from __future__ import annotations

import math

import numpy as np

import dnsmc_gb300 as D
from dnsmc_gb300 import synth
from oracle import oracle as O


def mirror(tb, n, T, x, Tw, region, groups=2, seed=3):
    cfg = D.default_config(model=D.MODEL_TABLE, imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi, Lz=math.pi,
                           stretched_x=0, T_west=Tw, T_east=Tw, n_groups=groups, seed=seed,
                           sampler=D.SAMPLER_RQMC, local_sampling=1, nvar=2, control_variate=0)
    s = D.Solver(cfg)
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    s.set_region(*region)
    s.prepare_sampling(float(max(T.max(), Tw)), float(x.mean()))
    s.set_rays(8)
    return s


def test_exact_means_follow_their_definition():
    n = 8
    tb = synth.ck_table(nbands=4, nq=2, nT=12, nX=3, seed=2)
    d = synth.ck_channel(n, 1)
    T, x, Tw = d["T"], d["x"], d["T_wall"]
    s = mirror(tb, n, T, x, Tw, (0, n, 0, 8, 0, 8))
    c, keep = O.packet_config(s, T[None], x[None], use_double=1)
    sur_k, sur_I = O.layer_surrogate(s.table(), T[None], x[None])
    c.cv, c.sur_k, c.sur_I = 1, O._fp(sur_k), O._fp(sur_I)
    nb, nq, nG = 4, 2, 2
    sid = np.arange(nb * nq, dtype=np.int32)
    C = np.array([4 * math.pi * 100 * float(np.float32(tb["dnu"][b])) * float(np.float32(tb["wq"][g]))
                  for b in range(nb) for g in range(nq)])
    gs = np.array([0, 4, 8], np.int32)
    mu, w = O.cv_quadrature()
    muY = np.zeros((1, nG, n * 64, 2))
    import ctypes
    assert O.load().orc_cv_mean(ctypes.byref(c), gs.ctypes.data_as(O._i), sid.ctypes.data_as(O._i),
                                C.ctypes.data_as(O._d), mu.ctypes.data_as(O._d), w.ctypes.data_as(O._d), len(mu), 2,
                                muY.ctypes.data_as(O._d)) == 0
    tab = s.table()
    xu, _, _ = s.geometry()
    ibw = np.asarray(s.sampling()["ibw"], np.float64).reshape(2, nb)
    k = np.asarray(tab["k"], np.float64)
    Ib = np.asarray(tab["Ib"], np.float64)
    JA = [O.cv_jhat(sur_k[0, q], sur_I[0, q], xu, c.toll, ibw[0, q // nq], ibw[1, q // nq]) for q in range(nb * nq)]
    rng = np.random.default_rng(0)
    for tc in rng.choice(n * 64, 24, replace=False):
        i, kk, j = tc // 64, (tc // 8) % 8, tc % 8
        Ti, xi_ = float(T[kk, j, i]), float(x[kk, j, i])
        p = min(max((Ti - tb["T0"]) / tb["dT"], 0), tb["k"].shape[2] - 1)
        ti = min(int(p), tb["k"].shape[2] - 2)
        ft = p - ti
        px = min(max((xi_ - tb["X0"]) / tb["dX"], 0), 2)
        xi = min(int(px), 1)
        fx = px - xi
        for G in range(nG):
            ea = eb = 0.0
            for e in range(gs[G], gs[G + 1]):
                q = sid[e]
                b, g = q // nq, q % nq
                kq = k[b, g]
                k0 = kq[ti, xi] + fx * (kq[ti, xi + 1] - kq[ti, xi])
                k1 = kq[ti + 1, xi] + fx * (kq[ti + 1, xi + 1] - kq[ti + 1, xi])
                kc = k0 + ft * (k1 - k0)
                ib = Ib[b, ti] + ft * (Ib[b, ti + 1] - Ib[b, ti])
                J, A = JA[q][i]
                ea += C[e] * kc * (ib - J)
                eb += C[e] * kc * A * (ib - float(sur_I[0, q, i]))
            np.testing.assert_allclose(muY[0, G, tc], [ea, eb], rtol=1e-6)  # cut-off ln(1/toll) in float there
    s.close()


def test_control_variate_solution_agrees_with_plain_fp64():
    n = 16
    tb = synth.ck_table(nbands=8, nq=4, nT=50, nX=4, seed=5)
    d = synth.ck_channel(n, 2)
    T, x, Tw = d["T"], d["x"], d["T_wall"]
    region = (0, n, 0, 8, 0, 8)
    s = mirror(tb, n, T, x, Tw, region)
    Q, V = O.fp64_cv_solution(s, tb["dnu"], tb["wq"], T[None], x[None], rays=256, nbatch=8, seed=11)
    Qs, Vs = O.fp64_cv_solution(s, tb["dnu"], tb["wq"], T[None], x[None], rays=256, nbatch=8, seed=11,
                                layer_step=3)
    np.testing.assert_array_equal(Qs[..., ::3], Q[..., ::3])
    assert np.isnan(Qs[..., 1::3]).all()
    c, keep = O.packet_config(s, T[None], x[None], use_double=1)
    c.cv, c.rays, c.nbatch, c.seed = 0, 4096, 8, 99
    tal, _ = O.packet_mc(c, 2, n * 64)
    m = tal[..., 0] / 4096
    vg = np.maximum(0, tal[..., 1] / 8 - m * m) / 7
    Qp = m.sum(1).reshape(1, n, 8, 8).transpose(0, 2, 3, 1)
    Vp = vg.sum(1).reshape(1, n, 8, 8).transpose(0, 2, 3, 1)
    z = (Q - Qp) / np.sqrt(V + Vp)
    assert np.sqrt((z ** 2).mean()) < 1.5
    # packet means (a packet's cells share their rays): unbiased within 4 sigma
    zp = (Q - Qp).mean(axis=(1, 2)) / np.sqrt((V + Vp).mean(axis=(1, 2)))
    assert np.abs(zp).max() < 4.0
    s.close()
