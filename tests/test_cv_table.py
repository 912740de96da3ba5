"""The control variate's tabulated surrogate in the oracle (orc_cv_table), on
the CPU.

The march does not walk the surrogate ray through the layer-mean medium; it
reads the ray's straight flight from a table per (field, spectral sample,
layer), with nodes uniform in u = sqrt(|mu|) on each hemisphere and linear
interpolation in u.  The table is built by one sweep per node from the far
wall (orc_cv_table; the flight is not cut off at ln(1/toll)).  The estimate
stays unbiased because E[Y] is the exact mean of that interpolant.  Checked
here:

* the table's nodes are the flight itself (float64 restatement, cv_walk
  without cut-off) up to FP32 rounding;
* the means the oracle returns equal the exact integral of the interpolant
  over mu uniform on [-1, 1], by closed form (int sqrt(mu) dmu) and by a fine
  midpoint sum, both written here independently of the oracle's weights;
* those means approach the continuous direction means: the analytic
  isothermal-slab result and the float64 quadrature of a layered medium;
* the interpolant follows the flight between the nodes closely enough for
  the control variate (the mean squared gap is a small fraction of the
  flight's own variance over mu), and the flight is within the ray cut-off
  of the truncated walk the 3-D march performs.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from oracle import oracle as O

NB = O.SUR_BINS


def layered(nw=24, stretched=True, seed=0):
    rng = np.random.default_rng(seed)
    if stretched:
        fw = (1 - np.cos(np.linspace(0, math.pi, nw + 1))).astype(np.float32)
    else:
        fw = np.linspace(0, 2, nw + 1).astype(np.float32)
    k = np.exp(rng.normal(0.0, 1.5, nw)).astype(np.float32)
    I = (rng.uniform(400, 1600, nw) ** 4).astype(np.float32)
    return fw, k, I


def config(fw, k, I, T_west, T_east, toll=1e-4):
    nw = len(k)
    c = O.PacketConfig()
    c.mode, c.nfields, c.nw = 0, 1, nw
    c.fw = O._fp(fw)
    c.T_west, c.T_east, c.toll = T_west, T_east, toll
    sk = np.ascontiguousarray(k.reshape(1, 1, nw), np.float32)
    sI = np.ascontiguousarray(I.reshape(1, 1, nw), np.float32)
    c.cv, c.sur_k, c.sur_I = 1, O._fp(sk), O._fp(sI)
    return c, (fw, sk, sI)


def nodes(tab):
    """Node values J(m), A(m), m = 0 .. NB, per hemisphere from the bins."""
    J = np.concatenate([tab[..., 0], (tab[..., -1, 0] + tab[..., -1, 1])[..., None]], -1)
    A = np.concatenate([tab[..., 2], (tab[..., -1, 2] + tab[..., -1, 3])[..., None]], -1)
    return J, A


def test_table_nodes_are_the_walk():
    fw, k, I = layered()
    Tw, Te = 500.0, 1300.0
    c, keep = config(fw, k, I, Tw, Te)
    tab, _ = O.cv_table(c)
    J, A = nodes(tab[0, 0])  # (nw, 2, NB + 1)
    Iw = (np.float32(Tw) ** 4, np.float32(Te) ** 4)
    for l in (0, 5, 11, 23):
        for h, sgn in ((0, -1.0), (1, 1.0)):
            for m in (0, 1, 7, 32, 63, 64):
                mu = (m / NB) ** 2 if m else 2.0 ** -30
                Je, Ae = O.cv_walk(k, I, fw.astype(np.float64), None, Iw, l, sgn * mu)
                assert abs(J[l, h, m] - Je) <= 2e-5 * Je + 1e-30, (l, h, m, J[l, h, m], Je)
                assert abs(A[l, h, m] - Ae) <= 2e-5, (l, h, m, A[l, h, m], Ae)
    # the grazing node: everything absorbed in the own layer
    np.testing.assert_allclose(J[:, :, 0], np.repeat(I[:, None], 2, 1), rtol=1e-6)
    np.testing.assert_array_equal(A[:, :, 0], 1.0)


def test_table_means_are_the_exact_means_of_the_interpolant():
    fw, k, I = layered(nw=16, seed=3)
    c, keep = config(fw, k, I, 300.0, 900.0)
    tab, JA = O.cv_table(c)
    tab = tab[0, 0].astype(np.float64)  # (nw, 2, NB, 4)
    JA = JA[0, 0]
    m = np.arange(NB, dtype=np.float64)
    a, b = (m / NB) ** 2, ((m + 1) / NB) ** 2
    # int_a^b (J0 + (sqrt(mu) NB - m) dJ) dmu
    Is = (2.0 / 3.0) * (b ** 1.5 - a ** 1.5)
    for q, col in ((0, 0), (1, 2)):
        v0, dv = tab[..., col], tab[..., col + 1]
        per_h = (v0 * (b - a) + dv * (NB * Is - m * (b - a))).sum(-1)  # (nw, 2) over mu in [0, 1]
        np.testing.assert_allclose(JA[:, q], 0.5 * per_h.sum(-1), rtol=1e-12)
    # fine midpoint sum over mu, evaluated the way the march reads the table
    n = 1 << 20
    mu = (np.arange(n) + 0.5) / n
    x = np.sqrt(mu) * NB
    mm = np.minimum(x.astype(np.int64), NB - 1)
    r = x - mm
    for l in (0, 7, 15):
        acc = np.zeros(2)
        for h in (0, 1):
            e = tab[l, h, mm]
            acc += [(e[:, 0] + r * e[:, 1]).mean(), (e[:, 2] + r * e[:, 3]).mean()]
        np.testing.assert_allclose(JA[l], 0.5 * acc, rtol=1e-9)


def test_table_means_approach_the_slab_and_the_quadrature():
    nw = 24
    fw = np.linspace(0, 2, nw + 1).astype(np.float32)
    Ib = np.float32(1000.0) ** 4
    c, keep = config(fw, np.ones(nw, np.float32), np.full(nw, Ib, np.float32), 0.0, 300.0)
    _, JA = O.cv_table(c)
    o = 0.5 * (fw[:-1] + fw[1:]).astype(np.float64)
    ex = Ib - 0.5 * Ib * np.array([O.expn(2, t) for t in o]) \
        - 0.5 * (Ib - 300.0 ** 4) * np.array([O.expn(2, 2 - t) for t in o])
    np.testing.assert_allclose(JA[0, 0, :, 0], ex, rtol=2e-5)
    np.testing.assert_allclose(JA[0, 0, :, 1], 1 - O.expn(2, 1.0 / nw), rtol=1e-3)
    fw, k, I = layered(nw=20, seed=5)
    c, keep = config(fw, k, I, 600.0, 800.0)
    _, JA = O.cv_table(c)
    q = O.cv_jhat(k, I, fw.astype(np.float64), None, np.float32(600.0) ** 4, np.float32(800.0) ** 4)
    np.testing.assert_allclose(JA[0, 0, :, 0], q[:, 0], rtol=2e-4)
    np.testing.assert_allclose(JA[0, 0, :, 1], q[:, 1], rtol=2e-3, atol=1e-4)


def test_interpolant_follows_the_walk_between_the_nodes():
    fw, k, I = layered(nw=24, seed=7)
    c, keep = config(fw, k, I, 700.0, 700.0)
    tab, _ = O.cv_table(c)
    tab = tab[0, 0].astype(np.float64)
    Iw = (np.float32(700.0) ** 4,) * 2
    mus = np.random.default_rng(1).uniform(-1, 1, 400)
    for l in (0, 6, 12, 23):
        Je, Ae, Ji, Ai = [], [], [], []
        for mu in mus:
            J, A = O.cv_walk(k, I, fw.astype(np.float64), None, Iw, l, mu)
            Jt, At = O.cv_walk(k, I, fw.astype(np.float64), c.toll, Iw, l, mu)  # the march's cut-off
            assert abs(Jt - J) <= c.toll * (I.max() + Iw[0]) and abs(At - A) <= c.toll
            x = math.sqrt(abs(mu)) * NB
            m = min(int(x), NB - 1)
            e = tab[l, 1 if mu > 0 else 0, m]
            Je.append(J); Ae.append(A)
            Ji.append(e[0] + (x - m) * e[1]); Ai.append(e[2] + (x - m) * e[3])
        Je, Ae, Ji, Ai = map(np.array, (Je, Ae, Ji, Ai))
        assert ((Ji - Je) ** 2).mean() < 1e-3 * Je.var(), l
        assert ((Ai - Ae) ** 2).mean() < 1e-3 * Ae.var(), l


def test_replay_reads_the_table_like_the_march():
    """The packet replay with a table differs from the replay with the exact
    walk only by the interpolation: on an isothermal grey slab whose
    surrogate is the medium itself the residual X - Y of every ray is the gap
    between the walk and its interpolant, tiny next to the plain estimate."""
    import dnsmc_gb300 as D
    ni, nj, nk = 32, 32, 8
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853,
                                  Lz=3.1415927, stretched_x=0, T_west=0.0, T_east=300.0, kappa=1.0, seed=3))
    T = np.full((nk, nj, ni), 1000.0, np.float32)
    N = 16
    s._rays, s._nfields = N, 1
    c, keep = O.packet_config(s, T, None)
    sk = np.full((1, 1, ni), 1.0, np.float32)
    sI = np.full((1, 1, ni), np.float32(1000.0) ** 4, np.float32)
    c.cv, c.sur_k, c.sur_I = 1, O._fp(sk), O._fp(sI)
    beta = np.zeros((1, 1, nk, nj, ni, 2), np.float32)
    beta[..., 0], beta[..., 1] = 1.0, -1.0
    c.beta = O._fp(beta)
    sig = {}
    for kind in ("walk", "table", "plain"):
        if kind == "table":
            tab, _ = O.cv_table(c)
            c.sur_tab = O._fp(tab)
        if kind == "plain":
            c.cv, c.sur_tab = 0, None
        tal, _ = O.packet_mc(c, 1, ni * nj * nk)
        m1, m2 = tal[0, 0, :, 0] / N, tal[0, 0, :, 1] / N
        sig[kind] = float(np.sqrt(np.maximum(m2 - m1 ** 2, 0.0) / N).max())
    s.close()
    assert sig["walk"] < 1e-6 * sig["plain"], sig
    assert sig["walk"] < sig["table"] < 1e-3 * sig["plain"], sig
