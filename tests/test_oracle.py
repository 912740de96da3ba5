"""CPU tests that pin the oracle to the reference's own data.

The only golden output the reference ships is code/resfortm.txt (plane means
of Q_r, sigma and std_yz(Q) of a rad_main run with particle tables, 64^3,
black x-walls at 500 K, T = 500 + 2000 x(1-x)).  The oracle's restatement of
kernel_fluid/march_ray must reproduce it within the combined statistical
error; the reference's own table reader (compiled from code/read_tables.cpp
into oracle/_ref when the reference tree is present) must read the same
values as the fixtures.
"""
from __future__ import annotations

import math
import os

import numpy as np
import pytest

from conftest import REFERENCE
from oracle import oracle as O


def golden_field(im=64):
    xu = O.ref_faces(im, 1.0, 1)
    x = 0.5 * (xu[1:] + xu[:-1])
    T = np.zeros((im + 2, im + 2, im + 2), np.float32)
    T[1:-1, 1:-1, 1:-1] = (500 - 2000 * x ** 2 + 2000 * x)[None, None, :]
    return x, T


def particle_ref_tables(pt):
    return dict(Tnb=pt["Tnb"], kq=np.repeat(pt["kq"].reshape(-1, 1, 1), pt["Tnb"].size, 1), wvc=pt["wvc"],
                prob=pt["prob"], probg=None, kP=pt["kP"])


def test_philox_uniform_and_distinct():
    key = (0x12345678, 0x9ABCDEF0)
    outs = np.array([O.philox((i, 7, 0, 0), key) for i in range(2000)], dtype=np.uint64)
    assert len({tuple(o) for o in outs}) == 2000
    u = (outs >> 8).astype(np.float64) / 2 ** 24
    assert abs(u.mean() - 0.5) < 0.01
    assert abs(u.var() - 1 / 12) < 0.005


def test_reference_grid_matches_golden_x(resfortm):
    x, _ = golden_field()
    np.testing.assert_allclose(x, resfortm["x"], rtol=0, atol=2e-6)


def test_golden_is_optically_thin(resfortm, particle_tables):
    """code/resfortm.txt equals the optically thin limit in the interior to
    better than 2e-4 (the particle kappa_P is ~6e-11 1/m)."""
    x, _ = golden_field()
    T = 500 - 2000 * x ** 2 + 2000 * x
    thin = O.thin_limit(T, 500.0, particle_tables["Tnb"], particle_tables["kP"])
    rel = resfortm["Q"] / thin - 1
    assert np.abs(rel[16:48]).max() < 2e-4
    assert rel[0] > 0.005  # the near-wall excess from linear Ib interpolation


@pytest.mark.parametrize("grid_num", [5, 1])
def test_oracle_reproduces_resfortm(resfortm, particle_tables, grid_num):
    """Oracle plane means vs the golden plane means, 64 rows, combined 1-sigma
    per row: rms z < 1.6 and max |z| < 4.2."""
    _, T = golden_field()
    rng = np.random.default_rng(0)
    ncper = 4
    cells = np.array([[i, rng.integers(1, 65), rng.integers(1, 65)] for i in range(1, 65) for _ in range(ncper)])
    r = O.ref_mc(T.ravel(), cells, imax=64, jmax=64, kmax=64, Lx=1, Ly=1, Lz=1, T_west=500, T_east=500, model=2,
                 tables=particle_ref_tables(particle_tables), nvar=3, photmax=1000, grid_num=grid_num, hwfilter=1,
                 use_double=1)
    Q = r["Q"].reshape(64, ncper).mean(1)
    se = np.sqrt((r["se"] ** 2).reshape(64, ncper).sum(1)) / ncper
    z = (Q - resfortm["Q"]) / np.sqrt(se ** 2 + (resfortm["plane_std"] / 64) ** 2)
    assert math.sqrt((z ** 2).mean()) < 1.6, z
    assert np.abs(z).max() < 4.2, z


def test_oracle_reference_sigma_normaliser(particle_tables):
    """The reference's sigma (1/((nVar-0.5)(nVar-1)) normaliser over nVar batch
    means) estimates nVar/(nVar-0.5) times the variance of the mean."""
    _, T = golden_field()
    cells = np.array([[32, j, k] for j in range(1, 65, 4) for k in range(1, 65, 8)])
    r = O.ref_mc(T.ravel(), cells, imax=64, jmax=64, kmax=64, Lx=1, Ly=1, Lz=1, T_west=500, T_east=500, model=2,
                 tables=particle_ref_tables(particle_tables), nvar=3, photmax=400, grid_num=5, use_double=1)
    ratio = r["var_ref"].mean() / (r["se"] ** 2).mean()
    assert 0.8 < ratio / (3 / 2.5) < 1.25


def test_oracle_fp32_port_agrees_with_fp64(particle_tables):
    _, T = golden_field()
    cells = np.array([[i, 5, 9] for i in range(1, 65, 3)])
    kw = dict(imax=64, jmax=64, kmax=64, Lx=1, Ly=1, Lz=1, T_west=500, T_east=500, model=2,
              tables=particle_ref_tables(particle_tables), nvar=2, photmax=500, grid_num=5)
    a = O.ref_mc(T.ravel(), cells, use_double=0, **kw)
    b = O.ref_mc(T.ravel(), cells, use_double=1, **kw)
    z = (a["Q"] - b["Q"]) / np.sqrt(a["se"] ** 2 + b["se"] ** 2)
    assert np.abs(z).max() < 1e-2  # same random numbers: only rounding differs


def test_expn_against_series_identities():
    # E_1(1) and E_2(1) published values; recurrence n E_{n+1}(x) = e^-x - x E_n(x)
    assert abs(O.expn(1, 1.0) - 0.21938393439552) < 1e-12
    for x in (0.01, 0.3, 1.0, 2.5, 7.0):
        for n in (1, 2, 3):
            lhs = n * O.expn(n + 1, x)
            rhs = math.exp(-x) - x * O.expn(n, x)
            assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(lhs))
    sp = pytest.importorskip("scipy.special")
    for x in (0.05, 0.5, 1.5, 4.0):
        assert abs(O.expn(2, x) - sp.expn(2, x)) < 1e-13


def test_slab_formula_limits():
    y = np.linspace(0.01, 1.99, 9)
    q = O.slab_divq(y, 2.0, 1.0, 1000.0, 0.0, 0.0)
    np.testing.assert_allclose(q, q[::-1], rtol=1e-12)  # symmetric
    assert q[4] < q[0]  # the centre is more shielded than the wall region
    thin = O.slab_divq(np.array([0.5]), 1.0, 1e-6, 1000.0, 0.0, 0.0)
    assert abs(thin[0] / (4e-6 * O.SIGMA * 1e12) - 1) < 1e-4


def test_spline_coarsening_matches_reference_source():
    """oracle/_ref's interp3D (compiled from code/spline.cpp) against the
    oracle's restatement on a smooth 64^3 field."""
    if not O.ref_tables_available("particle"):
        pytest.skip("reference tree not present: oracle/_ref not built")
    import ctypes
    from oracle import build as ob
    lib = ctypes.CDLL(ob.ref_lib_path("particle"))
    rng = np.random.default_rng(3)
    T = np.zeros((66, 66, 66), np.float32)
    i = np.arange(64)
    T[1:-1, 1:-1, 1:-1] = (800 + 100 * np.sin(i / 9.0)[None, None, :] + 50 * np.cos(i / 7.0)[None, :, None]
                           + 20 * np.sin(i / 5.0)[:, None, None] + rng.normal(0, 1, (64, 64, 64)))
    for level in (1, 3):
        out = np.zeros_like(T).ravel()
        lib.ref_interp3d(T.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), level,
                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        n = 64 >> level
        ref = out[: (n + 2) ** 3].reshape(n + 2, n + 2, n + 2)[1:-1, 1:-1, 1:-1]
        mine = O.coarsen(T.ravel(), 64, 64, 64, 1, 1, 1, 1, 5, level)[1:-1, 1:-1, 1:-1]
        np.testing.assert_allclose(mine, ref, rtol=2e-6, atol=0)


@pytest.mark.parametrize("kind", ["particle", "ck"])
def test_reference_reader_matches_fixtures(kind, particle_tables, ck_tables):
    if not O.ref_tables_available(kind):
        pytest.skip("reference tree not present: oracle/_ref not built")
    r = O.ref_readT(kind, REFERENCE, 1000.0)
    fx = particle_tables if kind == "particle" else ck_tables
    np.testing.assert_allclose(r["Tnb"], fx["Tnb"], rtol=1e-7)
    np.testing.assert_allclose(r["kP"], fx["kP"], rtol=1e-6)
    np.testing.assert_allclose(r["wvc"], fx["wvc"], rtol=1e-6)
    np.testing.assert_allclose(r["prob"], fx["prob"], rtol=1e-6, atol=1e-12)
    if kind == "ck":
        np.testing.assert_allclose(r["kq"], fx["kq"], rtol=1e-6)
        np.testing.assert_allclose(r["probg"], fx["probg"], rtol=1e-6, atol=1e-12)
        kmax_expected = np.interp(1000.0, fx["Tnb"], fx["kP"])
    else:
        np.testing.assert_allclose(r["kq"][:, 0, 0], fx["kq"], rtol=1e-6)
        kmax_expected = np.interp(1000.0, fx["Tnb"], fx["kP"])
    assert abs(r["kappamax"] / kmax_expected - 1) < 1e-5


def test_cv_jhat_quadrature_matches_isothermal_slab():
    """The oracle's layered-slab quadrature of the control-variate mean against
    the analytic isothermal result Ib - 1/2 (Ib - Iw1) E2(t1) - 1/2 (Ib - Iw2) E2(t2)."""
    nw = 24
    fw = np.linspace(0, 2, nw + 1)
    I = np.full(nw, 1000.0 ** 4)
    J = O.cv_jhat(np.full(nw, 1.0), I, fw, 1e-12, 0.0, 300.0 ** 4)
    o = 0.5 * (fw[:-1] + fw[1:])
    ex = I[0] - 0.5 * I[0] * np.array([O.expn(2, t) for t in o]) \
        - 0.5 * (I[0] - 300.0 ** 4) * np.array([O.expn(2, 2 - t) for t in o])
    np.testing.assert_allclose(J[:, 0], ex, rtol=1e-9)
    # own-layer absorptance: 1 - E2(half thickness), same on both sides
    h = 1.0 / nw
    np.testing.assert_allclose(J[:, 1], 1 - O.expn(2, h), rtol=1e-9)


def test_slab_references_reduce_to_the_black_non_scattering_slab():
    """The grey-wall formula at eps = 1 and the scattering Nystrom solution at
    vanishing scattering both equal the black non-scattering E2 solution; the
    Nystrom solution is converged in its sub-cell refinement."""
    faces = np.linspace(0.0, 2.0, 33)
    yc = 0.5 * (faces[1:] + faces[:-1])
    black = O.slab_divq(yc, 2.0, 1.0, 1000.0, 400.0, 400.0)
    np.testing.assert_allclose(O.slab_grey_walls_divq(yc, 2.0, 1.0, 1000.0, 400.0, 1.0), black, rtol=1e-12)
    fine = np.linspace(0.0, 2.0, 32 * 64 + 1)
    cell_avg = O.slab_divq(0.5 * (fine[1:] + fine[:-1]), 2.0, 0.5, 1000.0, 0.0, 0.0).reshape(32, 64).mean(1)
    thin = O.slab_scatter_divq(faces, 0.5, 1e-9, 1000.0, 0.0, 0.0, refine=8)
    np.testing.assert_allclose(thin, cell_avg, rtol=2e-3)
    a = O.slab_scatter_divq(faces, 0.5, 1.0, 1000.0, 0.0, 0.0, refine=8)
    b = O.slab_scatter_divq(faces, 0.5, 1.0, 1000.0, 0.0, 0.0, refine=16)
    np.testing.assert_allclose(a, b, rtol=2e-4)
    # grey walls at T_w: emission from the medium is partly returned
    grey = O.slab_grey_walls_divq(yc, 2.0, 1.0, 1000.0, 400.0, 0.6)
    assert np.all(grey < black) and np.all(grey > 0)
