"""The correlated-k table generator on the GPU (dnsmc_ck_from_lbl) against
the oracle's restatement (orc_ck_from_lbl), which is itself checked against
the reference's compiled correlatedKT (tests/test_ckgen.py).

The bin counts and the g-function are integer and fixed-order work, the bin
values products: the GPU's k at the g-points equals the oracle's but for the
rare interval whose k^0.1 falls within a rounding of a bin edge (the device's
and the host's power functions may round differently); the band means agree
to rounding.  A generated table then drives a solve.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_gpu_generator_matches_the_oracle():
    T = np.linspace(400.0, 2000.0, 9)
    spec = synth.lbl_spectrum(T, (0.05, 0.15, 0.3), nbands=5, band_width=20.0, lines_per_band=30, seed=11)
    gq, wq = synth.gauss_legendre_half(16)
    kq, kavg = D.ck_from_lbl(spec, gq, n_pwrk=10000)
    ko, ao = O.ck_from_lbl(spec, gq, n_pwrk=10000)
    assert (kq == ko).mean() > 0.99
    np.testing.assert_allclose(kq, ko, rtol=1e-5)
    np.testing.assert_allclose(kavg, ao, rtol=1e-9)
    assert (np.diff(kq, axis=1) >= 0).all()


def test_generated_table_drives_a_solve():
    T = np.linspace(300.0, 2100.0, 10)
    X = np.array([0.0, 0.1, 0.2, 0.3])
    spec = synth.lbl_spectrum(T, X, nbands=4, band_width=25.0, lines_per_band=30, seed=5)
    gq, wq = synth.gauss_legendre_half(16)
    kq, _ = D.ck_from_lbl(spec, gq, n_pwrk=10000)
    ni, nj, nk = 16, 32, 8
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=2 * math.pi,
                                  Lz=math.pi, stretched_x=0, T_west=400.0, T_east=400.0, n_groups=2, seed=3,
                                  sampler=D.SAMPLER_RQMC, nvar=2, local_sampling=1))
    s.set_table(kq, spec["wvc"].astype(np.float32), float(T[0]), float(T[1] - T[0]),
                dnu=np.full(4, 25.0, np.float32), wq=wq.astype(np.float32), X0=0.0, dX=0.1)
    d = synth.ck_channel(32, 2)
    Tf = np.ascontiguousarray(d["T"][:nk, :, :ni])
    xf = np.ascontiguousarray(d["x"][:nk, :, :ni])
    s.set_fields(Tf, xf)
    s.set_rays(32)
    Q, S = s.solve(timeout_s=120)
    assert np.isfinite(Q).all() and np.abs(Q).max() > 0 and s.status() == 0
    s.close()
