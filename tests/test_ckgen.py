"""The correlated-k table generator's oracle (orc_ck_from_lbl), on the CPU.

* against the reference's own routine, correlatedKT (distr/correlatedK.cpp:
  145-300), compiled from the reference sources into oracle/_ref with its
  compile-time sizes (52 temperatures, its 16 g-points, 10000 bins): the same
  k at every g-point of every band and temperature, up to rounding (the
  reference sums the bins' spectral fractions point by point, the oracle
  multiplies the interval count; it forms the bin values with pow, the
  oracle with products);
* against the spectra themselves: the k-distribution reproduces the band
  means of the transmissivity exp(-k L) over optical paths from thin to
  thick (what the reference's own error report checks,
  distr/correlatedK.cpp:258-293), and the band mean of k.
"""
from __future__ import annotations

import numpy as np
import pytest

from dnsmc_gb300 import synth
from oracle import oracle as O


def test_oracle_matches_the_reference_correlated_kt(tmp_path):
    if not O.ref_ckgen_available():
        pytest.skip("reference tree absent: its correlatedK.cpp was not built")
    T = 500.0 + 10.0 * np.arange(52)  # the reference's Tinit + DT i
    spec = synth.lbl_spectrum(T, (0.1,), nbands=4, band_width=20.0, lines_per_band=25, seed=3)
    kref, gq, npw = O.ref_correlated_kt(spec, str(tmp_path))
    kq, _ = O.ck_from_lbl(spec, gq, n_pwrk=npw)
    mine = kq[:, :, :, 0].transpose(2, 0, 1).astype(np.float64)  # (nT, nbands, nq)
    np.testing.assert_allclose(mine, kref.astype(np.float32).astype(np.float64), rtol=2e-6, atol=0)
    assert (np.diff(mine, axis=2) >= 0).all()  # k ascends in g


def test_distribution_reproduces_band_transmissivity():
    gq, wq = synth.gauss_legendre_half(16)
    gq01, wq01 = gq, wq  # the reference's 16 points: the positive half of the 32-point rule on (0, 1)
    spec = synth.lbl_spectrum((600.0, 1500.0), (0.05, 0.2), nbands=3, band_width=25.0, lines_per_band=30, seed=7)
    kq, kavg = O.ck_from_lbl(spec, gq01, n_pwrk=10000)
    k = spec["kappa"]
    for b in range(3):
        seg = k[:, :, spec["first"][b]:spec["first"][b] + spec["count"][b]]
        mid = 0.5 * (seg[..., 1:] + seg[..., :-1])  # the intervals the distribution weighs
        for L in (1e-3, 1e-2, 0.1, 1.0):
            lbl = np.exp(-mid * L).mean(-1)
            ck = (np.exp(-kq[b].astype(np.float64) * L) * wq01[:, None, None]).sum(0) / wq01.sum()
            assert np.abs(ck - lbl).max() < 0.01, (b, L, ck, lbl)
        np.testing.assert_allclose(kavg[..., b], mid.mean(-1), rtol=2e-3)


def test_generator_rejects_bad_inputs():
    import dnsmc_gb300 as D
    from dnsmc_gb300 import _lib
    spec = synth.lbl_spectrum((800.0,), (0.1,), nbands=2, band_width=5.0, lines_per_band=5, seed=1)
    gq, _ = synth.gauss_legendre_half(8)
    bad = dict(spec)
    bad["wv_right"] = spec["wv_left"]  # empty bands
    with pytest.raises(D.DnsmcError) as e:
        D.ck_from_lbl(bad, gq)
    assert e.value.code == _lib.ERR_ARG
    with pytest.raises(D.DnsmcError) as e:
        D.ck_from_lbl(spec, gq[::-1])  # g-points must ascend
    assert e.value.code == _lib.ERR_ARG
    neg = dict(spec)
    neg["kappa"] = -spec["kappa"]
    with pytest.raises(D.DnsmcError) as e:
        D.ck_from_lbl(neg, gq)
    assert e.value.code == _lib.ERR_TABLE
