"""Parity at the benchmark's configuration: the 128^3 correlated-k channel
(seed 0), the synthetic table of 64 bands x 16 g x 50 T x 8 x_H2O, 8 band
groups, RQMC rays, spectral sampling at the packet temperature, the control
variate with coefficients and ray counts from the committed network
(dnsmc_gb300/nets/ck128_g8.cvnet), 8 x 8 packets.  The region is one
wall-normal line of packets (i all, j and k < 8): 128 packets, 8192 cells.

* every solved cell and band group equals the host replay of the same rays
  bit for bit (every 4th packet of the line is replayed);
* the field agrees with the oracle's independent FP64 solution (its own
  control variate and exact means) within the combined statistical error,
  per cell and per packet;
* with a uniform x_H2O field (the reference has no x_H2O axis, so its table
  is then exactly the slice at that x) the field agrees per cell within 3
  sigma with the reference's own estimator (one thread per cell, band and
  g-point drawn at Tmax, position-update march) in FP64.  The field is
  scaled so that its maximum is a table temperature: the reference draws
  band and g from the CDFs at the table temperature nearest Tmax but
  weights the ray with kappa_max, k and Ib interpolated at Tmax itself
  (code/mc_gpu.cu:142, :837; code/read_tables.cpp:34-36), which biases its
  estimate unless the two coincide -- by 3-4 % on this table, whose k
  changes steeply between table temperatures.
"""
from __future__ import annotations

import math
import os

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N = 128
GROUPS = 8
NET = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "dnsmc_gb300", "nets",
                   "ck128_g8.cvnet")


@pytest.fixture(scope="module")
def inputs():
    d = synth.ck_channel(N, 0)
    return synth.ck_table(), d["T"], d["x"], d["T_wall"]


def solver(table, Tw, nvar, seed=1000, cv=1):
    cfg = D.default_config(model=D.MODEL_TABLE, imax=N, jmax=N, kmax=N, Lx=2.0, Ly=2 * math.pi, Lz=math.pi,
                           stretched_x=0, T_west=Tw, T_east=Tw, n_groups=GROUPS, seed=seed, block_threads=128,
                           sampler=D.SAMPLER_RQMC, local_sampling=1, nvar=nvar, control_variate=cv)
    s = D.Solver(cfg)
    s.set_table(table["k"], table["wvc"], table["T0"], table["dT"], dnu=table["dnu"], wq=table["wq"],
                X0=table["X0"], dX=table["dX"])
    return s


def network_solve(table, T, x, Tw, nvar, mean_rays, seed=1000):
    s = solver(table, Tw, nvar, seed)
    s.set_fields(T, x)
    s.set_region(0, N, 0, 8, 0, 8)
    s.set_rays(mean_rays)
    s.solve(timeout_s=300)  # control-variate data of the fields, as the bench's pilot
    net = D.CvNet.load(NET)
    net.apply(s, beta=True, rays=True, mean_rays=mean_rays, min_rays=2 * nvar, max_rays=4096)
    Q, S = s.solve(timeout_s=300)
    net.close()
    return s, Q, S


def test_bench_config_bitexact_with_the_replay(inputs):
    table, T, x, Tw = inputs
    s, Q, S = network_solve(table, T, x, Tw, nvar=2, mean_rays=48)
    Qg, _ = s.group_results()
    c, keep = O.packet_config(s, T[None], x[None])
    c.pw_step = 4  # every 4th packet of the line, with its own rays and ray counts
    rc = N * 64
    tal, _ = O.packet_mc(c, GROUPS, rc)
    tal = tal.reshape(1, GROUPS, N, 8, 8, 2).transpose(0, 1, 3, 4, 2, 5)
    rays = s.rays_per_item()
    beta = s.cv_beta()
    muY = s.cv_data()["muY"]
    ii = np.arange(N)[None, None, :]
    pk = ii  # one packet per layer in this line: packet p = i
    for g in range(GROUPS):
        m = tal[:, g, ..., 0] * (1.0 / rays[g][pk])  # the finalize multiplies by the reciprocal
        m = m + beta[:, g, ..., 0].astype(np.float64) * muY[:, g, ..., 0]
        m = m + beta[:, g, ..., 1].astype(np.float64) * muY[:, g, ..., 1]
        np.testing.assert_array_equal(Qg[:, g, ..., ::4], m[..., ::4], err_msg=f"band group {g}")
    assert s.status() == 0
    s.close()


def test_bench_config_agrees_with_the_fp64_oracle(inputs):
    table, T, x, Tw = inputs
    s, Q, S = network_solve(table, T, x, Tw, nvar=8, mean_rays=96)
    s.close()
    m = solver(table, Tw, nvar=8, seed=9001, cv=0)  # host-only mirror for the oracle
    m.set_region(0, N, 0, 8, 0, 8)
    m.prepare_sampling(float(max(T.max(), Tw)), float(x.mean()))
    m.set_rays(8)
    Qo, Vo = O.fp64_cv_solution(m, table["dnu"], table["wq"], T[None], x[None], rays=1024, nbatch=8, seed=9001,
                                layer_step=4)
    m.close()
    Qg, Sg = Q[0][..., ::4], S[0][..., ::4]
    Qo, Vo = Qo[0][..., ::4], Vo[0][..., ::4]
    z = (Qg - Qo) / np.sqrt(Sg ** 2 + Vo)
    assert math.sqrt(float((z ** 2).mean())) < 1.3, z
    assert (np.abs(z) > 4).mean() < 0.01
    # per packet (its cells share their rays): the mean difference
    zp = (Qg - Qo).mean(axis=(0, 1)) / np.sqrt((Sg ** 2 + Vo).mean(axis=(0, 1)))
    assert np.abs(zp).max() < 4.0, zp
    rel = math.sqrt(float(((Qg - Qo) ** 2).mean())) / math.sqrt(float((Qo ** 2).mean()))
    est = math.sqrt(float((Sg ** 2 + Vo).mean())) / math.sqrt(float((Qo ** 2).mean()))
    assert rel < 1.3 * est, (rel, est)


def test_bench_config_uniform_x_agrees_with_the_reference_estimator(inputs):
    table, T, _, Tw = inputs
    # Tmax onto the next table temperature (the reference estimator is
    # unbiased only there)
    Tnb = (table["T0"] + table["dT"] * np.arange(table["k"].shape[2])).astype(np.float32)
    Tg = Tnb[int(np.searchsorted(Tnb, T.max()))]
    top = np.unravel_index(np.argmax(T), T.shape)
    T = (T * np.float32(Tg / T.max())).astype(np.float32)
    T[top] = Tg
    x = np.full(T.shape, 0.1, np.float32)
    s, Q, S = network_solve(table, T, x, Tw, nvar=8, mean_rays=96)
    s.close()
    tables = O.ref_tables_x_slice(table, 0.1)
    Tf = np.zeros((N + 2, N + 2, N + 2), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = T
    i = np.arange(0, N, 4)
    cells = np.stack([i + 1, np.full_like(i, 4), np.full_like(i, 6)], 1)  # 1-based (i, j, k)
    r = O.ref_mc(Tf.ravel(), cells, imax=N, jmax=N, kmax=N, Lx=2.0, Ly=2 * math.pi, Lz=math.pi, T_west=Tw,
                 T_east=Tw, model=0, tables=tables, nvar=8, photmax=6000, grid_num=1, stretched=0, use_double=1,
                 seed=77)
    Qg = Q[0][5, 3, i]  # (k, j, i) = (6-1, 4-1, i)
    Sg = S[0][5, 3, i]
    z = (Qg - r["Q"]) / np.sqrt(Sg ** 2 + r["se"] ** 2)
    assert np.abs(z).max() < 4.5, z
    assert math.sqrt(float((z ** 2).mean())) < 1.5, z
