"""GPU parity tests: the CUDA march (through the C ABI) against the oracle.

* bit-exact: every (cell, band group) tally of a solve equals the oracle's
  FP32 replay of the packet scheme -- same Philox counters, same alias draw,
  same voxel walk, same rounding -- for the grey model, the reference particle
  and correlated-k tables, a synthetic k(T, x_H2O) table with band groups,
  several snapshots, adaptive ray counts and a sub-region;
* trace: the voxel-index walk and the RNG words of single rays;
* Philox pinned to curand's Philox4x32_10;
* statistical: per-cell agreement (combined 3 sigma) with the oracle's
  reference-structured estimator (code/mc_gpu.cu:44-438) on the same field
  and tables;
* analytic: the isothermal grey slab (E_2 solution);
* golden: code/resfortm.txt plane means;
* the drop-in pair mc_gpu_ / get_results_ and the error paths.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import tempfile

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import _lib, synth
from oracle import oracle as O
from tables_io import write_ck_tables, write_particle_tables

pytestmark = pytest.mark.gpu


def smooth_field(ni, nj, nk, lo, hi, seed):
    rng = np.random.default_rng(seed)
    i = (np.arange(ni) + 0.5) / ni
    j = np.arange(nj) / nj
    k = np.arange(nk) / nk
    base = lo + (hi - lo) * 4 * i * (1 - i)
    f = (np.sin(2 * np.pi * j)[None, :, None] * np.cos(2 * np.pi * k)[:, None, None] * 0.04
         + rng.normal(0, 0.01, (nk, nj, ni)))
    return (base[None, None, :] * (1 + f)).astype(np.float32)


def region_tally_to_dense(tal, solver, ng):
    i0, i1, j0, j1, k0, k1 = solver._region
    ni, nj, nk = i1 - i0, j1 - j0, k1 - k0
    nf = tal.shape[0]
    return tal.reshape(nf, ng, ni, nk, nj, 2).transpose(0, 1, 3, 4, 2, 5)


def packet_index(solver):
    """Packet of every region cell, (nk, nj, ni): tile_a x tile_b tiles of
    each wall-normal plane, j fastest."""
    i0, i1, j0, j1, k0, k1 = solver._region
    ni, nj, nk = i1 - i0, j1 - j0, k1 - k0
    ta, tb = solver.packet_shape()
    npa, npb = -(-nj // ta), -(-nk // tb)
    kk, jj, ii = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    return (ii * npb + kk // tb) * npa + jj // ta


def group_mean_var(tal_g, N, B, rqmc):
    """The finalize's mean and variance of the mean of one band group from
    its (sum, sum of squares | sum of squared replicate means) tally, with
    the divisions by the ray counts done as products with the float64
    reciprocals, as the device does."""
    N = np.asarray(N)
    with np.errstate(invalid="ignore", divide="ignore"):
        rN = np.where(N > 0, 1.0 / N, 0.0)
        rN1 = np.where(N > 1, 1.0 / (N - 1), 0.0)
        m = np.where(N > 0, tal_g[..., 0] * rN, 0.0)
        if rqmc:
            v = np.where(N > 0, np.maximum(0.0, tal_g[..., 1] * (1.0 / B) - m * m) * (1.0 / (B - 1)), 0.0)
        else:
            v = np.where(N > 1, np.maximum(0.0, tal_g[..., 1] * rN - m * m) * rN1, 0.0)
    return m, v


def rays_per_cell(solver, g=0):
    i0, i1, j0, j1, k0, k1 = solver._region
    ni, nj, nk = i1 - i0, j1 - j0, k1 - k0
    if not solver._keep:
        return np.full((nk, nj, ni), solver._rays, np.float64)
    rp = solver._keep[0]
    if rp.ndim == 2:  # per (band group, packet)
        rp = rp[g]
    return rp[packet_index(solver)].astype(np.float64)


def assert_bitexact(solver, T, x=None):
    Q, S = solver.solve(timeout_s=120)
    Qg, Vg = solver.group_results()
    ng = Qg.shape[1]
    c, keep = O.packet_config(solver, T, x)
    i0, i1, j0, j1, k0, k1 = solver._region
    tal, steps = O.packet_mc(c, ng, (i1 - i0) * (j1 - j0) * (k1 - k0))
    tal = region_tally_to_dense(tal, solver, ng)
    empty = np.zeros(ng, bool)
    if solver.cfg.model != D.MODEL_GREY:
        gs = solver.sampling()["group_start"]
        empty = gs[1:] == gs[:-1]
    Qexp = np.zeros_like(Q)
    Vexp = np.zeros_like(Q)
    B = solver.cfg.nvar
    for g in range(ng):
        N = rays_per_cell(solver, g)
        m, v = group_mean_var(tal[:, g], N, B, solver.cfg.sampler == D.SAMPLER_RQMC)
        if empty[g]:
            m, v = np.zeros_like(m), np.zeros_like(v)
        np.testing.assert_array_equal(Qg[:, g], m)
        np.testing.assert_array_equal(Vg[:, g], v)
        Qexp = Qexp + m
        Vexp = Vexp + v
    np.testing.assert_array_equal(Q, Qexp)
    np.testing.assert_array_equal(S, np.sqrt(Vexp))
    cnt = solver.counters()
    assert cnt.steps == steps
    assert solver.status() == 0
    assert np.isfinite(Q).all() and np.abs(Q).max() > 0
    return Q, S


def test_bitexact_grey():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=8, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=500, kappa=1.5, seed=11))
    T = smooth_field(16, 32, 8, 400, 1200, 1)
    s.set_fields(T)
    s.set_rays(96)
    assert_bitexact(s, T)
    s.close()


def test_bitexact_particle_tables_stretched(tmp_path, particle_tables):
    write_particle_tables(str(tmp_path), particle_tables)
    s = D.Solver(D.default_config(model=D.MODEL_PARTICLE, imax=16, jmax=16, kmax=8, stretched_x=1, seed=5))
    s.load_reference_tables(str(tmp_path), D.MODEL_PARTICLE)
    T = smooth_field(16, 16, 8, 520, 990, 2)
    s.set_fields(T)
    s.set_rays(48)
    assert_bitexact(s, T)
    s.close()


def test_bitexact_ck_tables(tmp_path, ck_tables):
    write_ck_tables(str(tmp_path), ck_tables)
    s = D.Solver(D.default_config(model=D.MODEL_CK, imax=12, jmax=32, kmax=4, Lx=0.5, Ly=1.0, Lz=0.25,
                                  stretched_x=0, T_west=600, T_east=800, seed=3, n_groups=3))
    s.load_reference_tables(str(tmp_path), D.MODEL_CK)
    T = smooth_field(12, 32, 4, 550, 1000, 3)
    s.set_fields(T)
    s.set_rays(64)
    assert_bitexact(s, T)
    s.close()


def test_bitexact_table_x_groups_fields_region():
    tb = synth.ck_table(nbands=16, nq=8, nT=24, nX=5, seed=4)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=10, jmax=40, kmax=6, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=400, T_east=400, seed=21, n_groups=4, tile_a=16))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = np.stack([smooth_field(10, 40, 6, 450, 1700, 5 + f) for f in range(2)])
    x = np.stack([(0.1 + 0.05 * np.random.default_rng(9 + f).uniform(-1, 1, (6, 40, 10))).astype(np.float32)
                  for f in range(2)])
    s.set_fields(T, x)
    s.set_region(1, 9, 3, 37, 0, 5)
    npk = s.packet_count()
    s.set_rays(0, np.random.default_rng(0).integers(0, 40, npk))
    assert_bitexact(s, T, x)
    s.close()


def test_bitexact_square_packets_ragged_region():
    """The automatic 8 x 8 packets over a region whose j and k extents are
    not multiples of 8 (20 x 11 cells: packets of 8, 8, 4 along j and 8, 3
    along k), with the control variate and RQMC: tallies bit-exact."""
    tb = synth.ck_table(nbands=12, nq=8, nT=20, nX=4, seed=8)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=6, jmax=24, kmax=12, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=1, T_west=420, T_east=400, seed=29, n_groups=3,
                                  sampler=D.SAMPLER_RQMC, nvar=2, local_sampling=1, control_variate=1))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(6, 24, 12, 450, 1700, 33)
    x = (0.1 + 0.05 * np.random.default_rng(12).uniform(-1, 1, (12, 24, 6))).astype(np.float32)
    s.set_fields(T, x)
    s.set_region(0, 6, 2, 22, 1, 12)
    assert s.packet_shape() == (8, 8)
    s.set_rays(16)
    from test_gpu_cv import assert_bitexact_cv
    assert_bitexact_cv(s, T, x)
    s.close()


def test_bitexact_rays_per_item_and_item_steps():
    """Ray counts per (band group, packet), zeros included, under RQMC; the
    per-item step record is positive exactly where rays were cast."""
    tb = synth.ck_table(nbands=16, nq=8, nT=24, nX=5, seed=4)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=12, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=400, T_east=400, seed=23, n_groups=4,
                                  sampler=D.SAMPLER_RQMC, nvar=4))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(12, 32, 4, 450, 1700, 8)[None]
    x = (0.1 + 0.05 * np.random.default_rng(3).uniform(-1, 1, (1, 4, 32, 12))).astype(np.float32)
    s.set_fields(T, x)
    npk = s.packet_count()
    rays = 4 * np.random.default_rng(1).integers(0, 12, (4, npk))
    rays[:, 0] = 0
    s.set_rays_per_item(rays)
    assert_bitexact(s, T, x)
    st = s.item_steps()
    assert st.shape == (1, 4, npk)
    assert ((st[0] > 0) == (rays > 0)).all()
    with pytest.raises(D.DnsmcError):
        s.set_rays_per_item(rays + 1)  # not multiples of nvar
    s.close()


def test_trace_matches_replay(tmp_path, ck_tables):
    write_ck_tables(str(tmp_path), ck_tables)
    s = D.Solver(D.default_config(model=D.MODEL_CK, imax=12, jmax=32, kmax=4, Lx=0.5, Ly=1.0, Lz=0.25,
                                  stretched_x=1, T_west=600, T_east=800, seed=77))
    s.load_reference_tables(str(tmp_path), D.MODEL_CK)
    T = smooth_field(12, 32, 4, 550, 1000, 8)
    s.set_fields(T)
    s.set_rays(8)
    s.solve(timeout_s=60)
    c, keep = O.packet_config(s, T, None)
    npk = s.packet_count()
    for p, r in [(0, 0), (npk - 1, 3), (npk // 2, 7), (5, 1)]:
        rec, n, rng = s.trace(0, 0, p, r)
        rec2, n2, rng2 = O.packet_trace(c, 0, 0, p, r)
        assert n == n2
        np.testing.assert_array_equal(rng, rng2)
        np.testing.assert_array_equal(rec, rec2)
        assert rng[0] == O.philox((r, p, 0, 0), (77, 0))[0]
    s.close()


def test_philox_matches_curand(tmp_path):
    nvcc = "/usr/local/cuda/bin/nvcc"
    so = str(tmp_path / "libpin.so")
    src = os.path.join(os.path.dirname(__file__), "philox_pin.cu")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-Xcompiler", "-fPIC", src,
                    "-o", so], check=True, capture_output=True)
    lib = ctypes.CDLL(so)
    rng = np.random.default_rng(1)
    n = 512
    ctr = rng.integers(0, 2 ** 32, (n, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, (n, 2), dtype=np.uint64).astype(np.uint32)
    out = np.zeros((n, 4), np.uint32)
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    assert lib.curand_philox_batch(p(ctr), p(key), p(out), n) == 0
    mine = np.array([O.philox(ctr[i], key[i]) for i in range(n)], np.uint32)
    np.testing.assert_array_equal(out, mine)


def _zstats(qa, sa, qb, sb):
    z = (qa - qb) / np.sqrt(sa ** 2 + sb ** 2)
    return z, math.sqrt(float((z ** 2).mean())), int((np.abs(z) > 3).sum())


def _parity_vs_reference(s, T, model, tables, Lx, Ly, Lz, Tw, Te, stretched, ncells=64, photmax=1500):
    ni, nj, nk = s.cfg.imax, s.cfg.jmax, s.cfg.kmax
    s.set_fields(T)
    s.set_rays(3 * photmax * 2)
    Q, S = s.solve(timeout_s=300)
    rng = np.random.default_rng(42)
    cells = []
    used = set()
    while len(cells) < ncells:
        i, j, k = int(rng.integers(0, ni)), int(rng.integers(0, nj)), int(rng.integers(0, nk))
        pk = (i, k, j // 32)
        if pk in used:
            continue
        used.add(pk)
        cells.append((i, j, k))
    cells = np.array(cells)
    Tf = np.zeros((nk + 2, nj + 2, ni + 2), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = T
    r = O.ref_mc(Tf.ravel(), cells + 1, imax=ni, jmax=nj, kmax=nk, Lx=Lx, Ly=Ly, Lz=Lz, T_west=Tw, T_east=Te,
                 model=model, tables=tables, kappa=s.cfg.kappa, nvar=3, photmax=photmax, grid_num=1,
                 stretched=stretched, use_double=1, seed=9)
    qg = Q[0][cells[:, 2], cells[:, 1], cells[:, 0]]
    sg = S[0][cells[:, 2], cells[:, 1], cells[:, 0]]
    z, rms, n3 = _zstats(qg, sg, r["Q"], r["se"])
    # 64 independent cells: P(n3 > 3) < 1e-3 under the null
    assert n3 <= 3, (z, rms)
    assert 0.6 < rms < 1.45, (z, rms)


def test_statistical_parity_reference_ck(tmp_path, ck_tables):
    write_ck_tables(str(tmp_path), ck_tables)
    s = D.Solver(D.default_config(model=D.MODEL_CK, imax=16, jmax=32, kmax=8, Lx=0.3, Ly=0.6, Lz=0.3,
                                  stretched_x=1, T_west=520, T_east=700, seed=13))
    s.load_reference_tables(str(tmp_path), D.MODEL_CK)
    T = smooth_field(16, 32, 8, 560, 1000, 13)
    tables = dict(Tnb=ck_tables["Tnb"], kq=ck_tables["kq"], wvc=ck_tables["wvc"], prob=ck_tables["prob"],
                  probg=ck_tables["probg"], kP=ck_tables["kP"])
    _parity_vs_reference(s, T, 0, tables, 0.3, 0.6, 0.3, 520, 700, 1)
    s.close()


def test_statistical_parity_reference_grey_bands():
    s = D.Solver(D.default_config(model=D.MODEL_GREY_BANDS, imax=16, jmax=32, kmax=8, Lx=1.0, Ly=2.0, Lz=1.0,
                                  stretched_x=1, T_west=500, T_east=500, kappa=1.0, seed=17))
    s.use_grey_band_tables()
    T = smooth_field(16, 32, 8, 600, 1100, 17)
    _parity_vs_reference(s, T, 1, None, 1.0, 2.0, 1.0, 500, 500, 1, photmax=800)
    s.close()


def test_grey_slab_matches_analytic_solution():
    """Isothermal slab T = 1000 K, kappa = 1, tau_L = 2, walls 0 K and 300 K."""
    ni, nj, nk = 64, 32, 16
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.2831853,
                                  Lz=3.1415927, stretched_x=0, T_west=0.0, T_east=300.0, kappa=1.0, seed=3))
    s.set_fields(np.full((nk, nj, ni), 1000.0, np.float32))
    s.set_rays(8192)
    Q, S = s.solve(timeout_s=120)
    yc = (np.arange(ni) + 0.5) * 2.0 / ni
    exact = O.slab_divq(yc, 2.0, 1.0, 1000.0, 0.0, 300.0)
    # one cell per packet is independent (the cells of a packet share rays)
    ta, tb = s.packet_shape()
    npk = (nk // tb) * (nj // ta)
    q = Q[0][::tb, ::ta, :].mean((0, 1))
    se = np.sqrt((S[0][::tb, ::ta, :] ** 2).sum((0, 1))) / npk
    z = (q - exact) / se
    assert np.abs(z).max() < 4.0, z
    assert math.sqrt((z ** 2).mean()) < 1.5
    assert np.abs(q / exact - 1).max() < 0.01
    s.close()


def test_golden_resfortm_on_gpu(tmp_path, particle_tables, resfortm):
    """code/resfortm.txt (particle tables, 64^3, black x-walls 500 K,
    T = 500 + 2000 x(1-x), stretched x): plane means over a 32x32 (j,k)
    patch of every x-row agree with the golden rows."""
    write_particle_tables(str(tmp_path), particle_tables)
    s = D.Solver(D.default_config(seed=7))
    s.load_reference_tables(str(tmp_path), D.MODEL_PARTICLE)
    xu, _, _ = s.geometry()
    x = 0.5 * (xu[1:] + xu[:-1])
    T = np.broadcast_to((500 - 2000 * x ** 2 + 2000 * x).astype(np.float32), (64, 64, 64)).copy()
    s.set_fields(T)
    s.set_region(0, 64, 0, 32, 0, 32)
    s.set_rays(3000)
    Q, S = s.solve(timeout_s=300)
    ta, tb = s.packet_shape()
    q = Q[0][::tb, ::ta, :].mean((0, 1))  # one cell per packet: independent packets of each row
    se = np.sqrt((S[0][::tb, ::ta, :] ** 2).sum((0, 1))) / ((32 // tb) * (32 // ta))
    gse = resfortm["plane_std"] / 64
    z = (q - resfortm["Q"]) / np.sqrt(se ** 2 + gse ** 2)
    assert math.sqrt((z ** 2).mean()) < 1.6, z
    assert np.abs(z).max() < 4.2, z
    s.close()


def test_dropin_pair_layouts_and_ghosts():
    ni, nj, nk, prow = 16, 16, 8, 2
    cfg = D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, p_row=prow, Lx=2.0, Ly=6.28, Lz=3.14,
                           stretched_x=1, T_west=300, T_east=300, kappa=1.0, nvar=3, photmax=40, seed=5)
    D.dropin_configure(cfg)
    T = smooth_field(ni, nj, nk, 400, 1200, 21)
    Tf = np.zeros((nk + 2, nj + 2, ni + 2), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = T
    Tf[0] = Tf[-1] = -5.0  # ghost garbage must be ignored
    jl = nj // prow
    Qr = np.full((nk + 2, jl + 2, ni + 2), -7.0, np.float32)
    Vr = np.full_like(Qr, -7.0)
    D.mc_gpu(Tf, 9)
    D.get_results(Qr, Vr)
    D.dropin_release()
    inner = (slice(1, -1), slice(1, -1), slice(1, -1))
    ghost = np.ones(Qr.shape, bool)
    ghost[inner] = False
    assert (Qr[ghost] == -7.0).all() and (Vr[ghost] == -7.0).all()
    s = D.Solver(cfg)
    s.set_fields(T)
    s.set_region(0, ni, 8, 16, 0, nk)
    s.set_rays(120)
    Q, S = s.solve(timeout_s=60)
    np.testing.assert_array_equal(Qr[inner], Q[0].astype(np.float32))
    np.testing.assert_array_equal(Vr[inner], np.sqrt(S[0] ** 2 * 3 / 2.5).astype(np.float32))
    s.close()


def test_float_results_are_the_rounded_double_results():
    """DNSMC_RESULT_F32: the finalize kernel rounds Q and sigma to float on
    the device and only those cross to the host; they equal the double
    results rounded on the host, and the double getter refuses them."""
    ni, nj, nk = 16, 24, 8
    cfg = D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                           stretched_x=1, T_west=300, T_east=500, kappa=0.7, nvar=2, photmax=16, seed=8)
    T = smooth_field(ni, nj, nk, 400, 1200, 22)
    s = D.Solver(cfg)
    s.set_fields(T)
    s.set_rays(32)
    Q, S = s.solve(timeout_s=60)
    s.set_result_type(D.RESULT_F32)
    Qf, Sf = s.solve(timeout_s=60)
    assert Qf.dtype == np.float32 and Sf.dtype == np.float32
    np.testing.assert_array_equal(Qf, Q.astype(np.float32))
    np.testing.assert_array_equal(Sf, S.astype(np.float32))
    with pytest.raises(D.DnsmcError) as e:
        s.results()
    assert e.value.code == _lib.ERR_STATE
    s.set_result_type(D.RESULT_F64)
    Q2, _ = s.solve(timeout_s=60)
    np.testing.assert_array_equal(Q2, Q)
    np.testing.assert_array_equal(s.results_float()[0], Qf)
    s.close()


def test_dropin_reads_reference_tables_by_default(tmp_path, particle_tables, monkeypatch):
    write_particle_tables(str(tmp_path), particle_tables)
    monkeypatch.setenv("DNSMC_IMAX", "16")
    monkeypatch.setenv("DNSMC_JMAX", "32")
    monkeypatch.setenv("DNSMC_KMAX", "8")
    monkeypatch.setenv("DNSMC_PHOTMAX", "20")
    monkeypatch.setenv("DNSMC_TABLES", str(tmp_path))
    D.dropin_configure(None)
    Tf = np.zeros((10, 34, 18), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = smooth_field(16, 32, 8, 520, 990, 4)
    Qr = np.zeros((10, 34, 18), np.float32)
    Vr = np.zeros_like(Qr)
    D.mc_gpu(Tf, 1)
    D.get_results(Qr, Vr)
    D.dropin_release()
    assert np.isfinite(Qr).all() and (Vr[1:-1, 1:-1, 1:-1] > 0).all()


def test_status_and_errors():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=8, max_steps=3, seed=1))
    with pytest.raises(D.DnsmcError) as e:
        s.solve()
    assert e.value.code == _lib.ERR_STATE
    bad = smooth_field(16, 32, 8, 400, 900, 1)
    bad[2, 3, 4] = -1.0
    with pytest.raises(D.DnsmcError) as e:
        s.set_fields(bad)
    assert e.value.code == _lib.ERR_ARG
    s.set_fields(smooth_field(16, 32, 8, 400, 900, 1))
    s.set_rays(16)
    s.solve(timeout_s=60)
    assert s.status() & D.STATUS_STEP_CAP
    s.close()


def test_bounded_wait_times_out_then_completes():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=64, jmax=64, kmax=64, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=300, kappa=0.2, seed=2))
    s.set_fields(synth.grey_channel(64)["T"])
    s.set_rays(2048)
    s.solve_async()
    with pytest.raises(D.DnsmcError) as e:
        s.wait(1e-6)
    assert e.value.code == _lib.ERR_TIMEOUT
    s.wait(120)
    Q, S = s.results()
    assert np.isfinite(Q).all()
    s.close()


def test_device_field_input_matches_host_input():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    T = synth.grey_channel(32)["T"]
    cfg = D.default_config(model=D.MODEL_GREY, imax=32, jmax=32, kmax=32, Lx=2.0, Ly=6.28, Lz=3.14,
                           stretched_x=0, T_west=300, T_east=300, kappa=1.0, seed=4)
    a = D.Solver(cfg)
    a.set_fields(T)
    a.set_rays(64)
    Qa, _ = a.solve(timeout_s=60)
    b = D.Solver(cfg)
    dT = torch.from_numpy(np.ascontiguousarray(T)).cuda()  # the device API takes dense i-fastest memory
    torch.cuda.synchronize()
    _lib.check(b._lib.dnsmc_set_fields_device(b._h, 1, ctypes.c_void_p(dT.data_ptr()), None))
    b._nfields = 1
    b.set_rays(64)
    Qb, _ = b.solve(timeout_s=60)
    np.testing.assert_array_equal(Qa, Qb)
    assert a.tmax() == b.tmax()
    a.close()
    b.close()


def test_bitexact_rqmc_local_bins_and_trace():
    tb = synth.ck_table(nbands=12, nq=8, nT=20, nX=4, seed=6)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=8, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=400, T_east=450, seed=31, n_groups=2,
                                  sampler=D.SAMPLER_RQMC, nvar=4, local_sampling=1))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(8, 32, 4, 450, 1700, 41)
    x = (0.1 + 0.05 * np.random.default_rng(3).uniform(-1, 1, (4, 32, 8))).astype(np.float32)
    s.set_fields(T, x)
    s.set_rays(48)
    assert_bitexact(s, T, x)
    assert s.sampling()["n_tbins"] == 20
    c, keep = O.packet_config(s, T, x)
    npk = s.packet_count()
    for p, r in [(0, 0), (3, 13), (npk - 1, 47)]:
        rec, n, rng = s.trace(0, 1, p, r)
        rec2, n2, rng2 = O.packet_trace(c, 0, 1, p, r)
        assert n == n2
        np.testing.assert_array_equal(rng, rng2)
        np.testing.assert_array_equal(rec, rec2)
    s.close()


def test_fields_checked_on_the_device():
    """Temperatures that are not positive and finite are rejected (host and
    device inputs, checked by the device statistics pass); the solver then
    holds no fields, so a solve fails instead of using them."""
    import torch
    ni, nj, nk = 8, 32, 4
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=300, seed=2))
    T = smooth_field(ni, nj, nk, 400, 1200, 3)
    s.set_fields(T)
    s.set_rays(4)
    s.solve(timeout_s=60)
    assert s.tmax() == float(T.max())
    for bad in (np.nan, -5.0, np.inf, 0.0):
        Tb = T.copy()
        Tb[1, 7, 3] = bad
        with pytest.raises(D.DnsmcError) as e:
            s.set_fields(Tb)
        assert e.value.code == _lib.ERR_ARG
        with pytest.raises(D.DnsmcError):
            s.solve(timeout_s=60)
        dT = torch.from_numpy(Tb).cuda().contiguous()
        with pytest.raises(D.DnsmcError):
            _lib.check(s._lib.dnsmc_set_fields_device(s._h, 1, ctypes.c_void_p(dT.data_ptr()), None))
    s.set_fields(T)
    Q, _ = s.solve(timeout_s=60)
    assert np.isfinite(Q).all()
    s.close()


def test_results_into_caller_arrays():
    ni, nj, nk = 8, 32, 4
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=300, seed=4))
    s.set_fields(smooth_field(ni, nj, nk, 400, 1200, 6))
    s.set_rays(8)
    Q, S = s.solve(timeout_s=60)
    Qo, So = np.full_like(Q, np.nan), np.full_like(S, np.nan)
    Q2, S2 = s.results(out=(Qo, So))
    assert Q2 is Qo and S2 is So
    np.testing.assert_array_equal(Qo, Q)
    np.testing.assert_array_equal(So, S)
    with pytest.raises(ValueError):
        s.results(out=(np.zeros(5), So))
    s.close()


def test_launch_count_counts_every_kernel():
    """dnsmc_get_launch_count: a grey solve launches the march and the
    finalize kernel; a CUDA-graph replay of the same solve adds the graph's
    two kernel nodes (the capture itself launches nothing)."""
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=8, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=300, kappa=1.0, seed=4))
    s.set_fields(smooth_field(16, 32, 8, 400, 900, 2))
    s.set_rays(8)
    for graph in (False, True, True):
        s.set_graph(graph)
        n0 = _lib.launch_count()
        s.solve(timeout_s=60)
        assert _lib.launch_count() - n0 == 2, graph
    s.close()


def test_sampling_tables_follow_fields_tables_and_particles():
    """A solve rebuilds the spectral sampling tables only when what they are
    built from changed (Tmax, mean x_H2O, the tables, the particle optics and
    mean fraction): a solver that solved other fields, another table or
    other particles first gives the same field, bit for bit, as a fresh one."""
    tb = synth.ck_table(nbands=8, nq=4, nT=20, nX=4, seed=21)
    tb2 = synth.ck_table(nbands=8, nq=4, nT=20, nX=4, seed=22)
    ni, nj, nk = 12, 32, 4
    cfg = D.default_config(model=D.MODEL_TABLE, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14, stretched_x=0,
                           T_west=400, T_east=450, seed=13, n_groups=2, local_sampling=1, control_variate=1)
    T1 = smooth_field(ni, nj, nk, 450, 1500, 4)
    T2 = smooth_field(ni, nj, nk, 500, 1700, 5)
    x1 = np.full(T1.shape, 0.1, np.float32)
    x2 = np.full(T1.shape, 0.14, np.float32)

    def fresh(t, T, x, part=None):
        s = D.Solver(cfg)
        s.set_table(t["k"], t["wvc"], t["T0"], t["dT"], dnu=t["dnu"], wq=t["wq"], X0=t["X0"], dX=t["dX"])
        s.set_fields(T, x)
        if part is not None:
            s.set_particles(*part)
            s.set_particle_field(np.full(T.shape, 1e-5, np.float32))
        s.set_rays(16)
        out = s.solve(timeout_s=120)
        s.close()
        return out

    s = D.Solver(cfg)
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    s.set_rays(16)
    s.set_fields(T1, x1)
    Q1, _ = s.solve(timeout_s=120)
    Q1b, _ = s.solve(timeout_s=120)  # the tables are reused
    np.testing.assert_array_equal(Q1b, Q1)
    for T, x in ((T2, x1), (T2, x2)):
        s.set_fields(T, x)
        Q, S = s.solve(timeout_s=120)
        Qf, Sf = fresh(tb, T, x)
        np.testing.assert_array_equal(Q, Qf)
        np.testing.assert_array_equal(S, Sf)
    s.set_table(tb2["k"], tb2["wvc"], tb2["T0"], tb2["dT"], dnu=tb2["dnu"], wq=tb2["wq"], X0=tb2["X0"], dX=tb2["dX"])
    Q, _ = s.solve(timeout_s=120)
    np.testing.assert_array_equal(Q, fresh(tb2, T2, x2)[0])
    part = (np.linspace(2e3, 4e3, 8).astype(np.float32), np.linspace(1e3, 2e3, 8).astype(np.float32), 0.5)
    s.set_particles(*part)
    s.set_particle_field(np.full(T2.shape, 1e-5, np.float32))
    Q, _ = s.solve(timeout_s=120)
    np.testing.assert_array_equal(Q, fresh(tb2, T2, x2, part)[0])
    s.close()
