"""CPU tests of the C ABI: exported symbols, configuration checks, the
reference-format table parsers and the spectral sampling tables -- all host
logic, no kernel launches."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

import dnsmc_gb300 as D
from conftest import REFERENCE, ROOT, has_gpu
from dnsmc_gb300 import _lib
from oracle import oracle as O
from tables_io import write_ck_tables, write_particle_tables


def header_functions():
    src = open(os.path.join(ROOT, "include", "dnsmc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:long\s+long|[a-z_0-9]+)\s*\*?\s*([a-z_][a-z_0-9]*)\s*\(", src, flags=re.M)))


def test_every_declared_function_is_exported():
    names = header_functions()
    assert "mc_gpu_" in names and "get_results_" in names and len(names) > 25
    lib = ctypes.CDLL(D.build.lib_path() if hasattr(D, "build") else _lib._build.lib_path())
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_python_constants_match_the_header():
    """Every DNSMC_STATUS_*, DNSMC_MODEL_*, DNSMC_SAMPLER_* and DNSMC_LAYOUT_*
    value of include/dnsmc.h is the package's constant of the same name."""
    src = open(os.path.join(ROOT, "include", "dnsmc.h")).read()
    defs = dict(re.findall(r"^#define DNSMC_((?:STATUS|MODEL|SAMPLER|LAYOUT)_[A-Z_0-9]+)\s+(0x[0-9a-fA-F]+|\d+)u?",
                           src, flags=re.M))
    assert {"STATUS_STEP_CAP", "STATUS_NONFINITE", "STATUS_BAD_FIELD", "STATUS_COPY_TIMEOUT"} <= set(defs)
    for name, val in defs.items():
        assert hasattr(_lib, name), name
        assert getattr(_lib, name) == int(val, 0), name


def test_default_config_is_reference_param_h():
    c = D.default_config()
    assert (c.imax, c.jmax, c.kmax, c.p_row) == (64, 64, 64, 1)
    assert (c.Lx, c.Ly, c.Lz) == (1.0, 1.0, 1.0)
    assert (c.nvar, c.photmax) == (3, 20000)
    assert (c.T_west, c.T_east) == (500.0, 500.0)
    assert abs(c.toll - 1e-3) < 1e-9 and c.max_steps == 100000
    assert c.model == D.MODEL_PARTICLE and c.stretched_x == 1


@pytest.mark.parametrize("field,value", [("imax", 0), ("p_row", 3), ("toll", 0.0), ("model", 9), ("eps_west", 0.0), ("eps_east", 1.5),
                                         ("grid_num", 7), ("block_threads", 100), ("tile_a", 12), ("nvar", 0)])
def test_bad_config_is_an_error_code(field, value):
    c = D.default_config()
    setattr(c, field, value)
    with pytest.raises(D.DnsmcError) as e:
        D.Solver(c)
    assert e.value.code == _lib.ERR_ARG


def test_control_variate_grid_limit():
    """The surrogate table's sweep keeps per-plane sums in shared memory:
    imax up to 4096 with the control variate."""
    c = D.default_config(control_variate=1, imax=4097)
    with pytest.raises(D.DnsmcError) as e:
        D.Solver(c)
    assert e.value.code == _lib.ERR_ARG
    assert "imax <= 4096" in str(e.value)
    D.Solver(D.default_config(control_variate=1, imax=4096)).close()


def test_config_from_env(monkeypatch):
    lib = _lib.load()
    monkeypatch.setenv("DNSMC_IMAX", "32")
    monkeypatch.setenv("DNSMC_TWEST", "650.5")
    monkeypatch.setenv("DNSMC_SEED", "99")
    c = D.default_config()
    assert lib.dnsmc_config_from_env(ctypes.byref(c)) == 0
    assert c.imax == 32 and c.T_west == 650.5 and c.seed == 99
    monkeypatch.setenv("DNSMC_JMAX", "abc")
    assert lib.dnsmc_config_from_env(ctypes.byref(c)) == _lib.ERR_ARG


def test_missing_table_dir_is_io_error(tmp_path):
    s = D.Solver(D.default_config())
    with pytest.raises(D.DnsmcError) as e:
        s.load_reference_tables(str(tmp_path / "nope"), D.MODEL_PARTICLE)
    assert e.value.code == _lib.ERR_IO
    s.close()


@pytest.mark.skipif(has_gpu(), reason="checks the no-device error path")
def test_device_calls_without_gpu_fail_cleanly():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=8, jmax=8, kmax=8))
    with pytest.raises(D.DnsmcError) as e:
        s.set_fields(np.full((8, 8, 8), 500, np.float32))
    assert e.value.code == _lib.ERR_NODEVICE
    s.close()


def test_particle_parser_roundtrip(tmp_path, particle_tables):
    write_particle_tables(str(tmp_path), particle_tables)
    s = D.Solver(D.default_config())
    s.load_reference_tables(str(tmp_path), D.MODEL_PARTICLE)
    t = s.table()
    assert (t["nbands"], t["nq"], t["nT"], t["nX"]) == (119, 1, 52, 1)
    np.testing.assert_allclose(t["k"][:, 0, 0, 0], particle_tables["kq"], rtol=1e-7)
    np.testing.assert_allclose(t["k"][:, 0, 17, 0], particle_tables["kq"], rtol=1e-7)
    np.testing.assert_allclose(t["prob"], particle_tables["prob"], rtol=1e-7, atol=1e-14)
    np.testing.assert_allclose(t["kP"], particle_tables["kP"], rtol=1e-7)
    assert t["T0"] == 500.0 and t["dT"] == 10.0
    s.close()


def test_ck_parser_roundtrip(tmp_path, ck_tables):
    write_ck_tables(str(tmp_path), ck_tables)
    s = D.Solver(D.default_config(model=D.MODEL_CK))
    s.load_reference_tables(str(tmp_path), D.MODEL_CK)
    t = s.table()
    assert (t["nbands"], t["nq"], t["nT"]) == (119, 16, 52)
    np.testing.assert_allclose(t["k"][..., 0], ck_tables["kq"].transpose(0, 2, 1), rtol=1e-7)
    np.testing.assert_allclose(t["probg"], ck_tables["probg"], rtol=1e-7, atol=1e-14)
    s.close()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "distr", "tables")), reason="reference tree absent")
def test_parsers_read_the_reference_files(particle_tables, ck_tables):
    tab = os.path.join(REFERENCE, "distr", "tables")
    s = D.Solver(D.default_config())
    s.load_reference_tables(tab, D.MODEL_PARTICLE)
    np.testing.assert_allclose(s.table()["prob"], particle_tables["prob"], rtol=1e-6, atol=1e-14)
    s.load_reference_tables(tab, D.MODEL_CK)
    t = s.table()
    np.testing.assert_allclose(t["k"][..., 0], ck_tables["kq"].transpose(0, 2, 1), rtol=1e-6)
    if O.ref_tables_available("ck"):
        r = O.ref_readT("ck", REFERENCE, 1000.0)
        np.testing.assert_array_equal(t["k"][..., 0], r["kq"].transpose(0, 2, 1))
        np.testing.assert_array_equal(t["probg"], r["probg"])
        np.testing.assert_array_equal(t["wvc"], r["wvc"])
    s.close()


# ---- sampling tables ----------------------------------------------------------
def alias_distribution(s, g):
    """Exact probability of every entry of group g as the kernel draws it."""
    gs = s["group_start"]
    a, b = int(gs[g]), int(gs[g + 1])
    K = b - a
    thr = s["prob"][a:b].astype(np.float64)
    al = s["alias"][a:b]
    p = np.zeros(K)
    for j in range(K):
        lo = -(-(j * 2 ** 32) // K)
        hi = -(-((j + 1) * 2 ** 32) // K)
        ps = (hi - lo) / 2 ** 32
        pa = np.ceil(thr[j] * 2 ** 24) / 2 ** 24
        p[j] += ps * pa
        p[al[j]] += ps * (1 - pa)
    return p


def ib_interp(Ib, T0, dT, b, T):
    pos = min(max((T - T0) / dT, 0.0), Ib.shape[1] - 1)
    i = min(int(pos), Ib.shape[1] - 2)
    f = pos - i
    return Ib[b, i] + f * (Ib[b, i + 1] - Ib[b, i])


def test_reference_sampling_reproduces_cdf_and_weights(ck_tables, tmp_path):
    """Reference mode: entries drawn with probability p_band * p_g at the table
    temperature nearest Tmax (code/mc_gpu.cu:830-896), and W * k_m * Ib_m =
    4 kappa_max sigma Tmax^4 (code/mc_gpu.cu:63, :163-169) for every entry."""
    write_ck_tables(str(tmp_path), ck_tables)
    sv = D.Solver(D.default_config(model=D.MODEL_CK, n_groups=1))
    sv.load_reference_tables(str(tmp_path), D.MODEL_CK)
    Tmax = 987.0
    s = sv.prepare_sampling(Tmax)
    t = sv.table()
    ts = 49  # nearest table T to 987 K is 990 K (index 49)
    pb = np.diff(np.concatenate([[0.0], ck_tables["prob"][ts].astype(np.float64)]))
    pg = np.diff(np.concatenate([np.zeros((119, 1)), ck_tables["probg"][ts].astype(np.float64)], axis=1), axis=1)
    target = (pb[:, None] * np.clip(pg, 0, None)).ravel()
    target /= target.sum()
    p = alias_distribution(s, 0)
    ids = s["band"] * 16 + s["gq"]
    np.testing.assert_allclose(p, target[ids], rtol=1e-6, atol=1e-9)
    assert abs(p.sum() - 1) < 1e-12
    kmax = np.interp(Tmax, ck_tables["Tnb"], ck_tables["kP"])
    E = 4 * kmax * O.SIGMA * Tmax ** 4
    pos = (Tmax - 500.0) / 10.0
    ti, f = int(pos), pos - int(pos)
    for e in range(0, len(ids), 37):
        b, g = s["band"][e], s["gq"][e]
        km = t["k"][b, g, ti, 0] + f * (t["k"][b, g, ti + 1, 0] - t["k"][b, g, ti, 0])
        ibm = ib_interp(t["Ib"], 500.0, 10.0, b, Tmax)
        assert abs(s["W"][e] * km * ibm * p[e] / (target[ids[e]] * E) - 1) < 2e-5
    sv.close()


def test_consistent_sampling_emission_identity():
    """Table mode: E_p[W k(T) Ib(T)] = 4 pi sum 100 dnu w_g k Ib for any T,
    per band group and in total, and every sample stays reachable."""
    from dnsmc_gb300 import synth
    tb = synth.ck_table(nbands=16, nq=16, nT=20, nX=4, seed=2)
    for ng in (1, 4):
        sv = D.Solver(D.default_config(model=D.MODEL_TABLE, n_groups=ng))
        sv.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
        s = sv.prepare_sampling(1800.0, 0.1)
        t = sv.table()
        assert s["n_groups"] == ng and len(s["W"]) == 16 * 16
        T, x = 1234.0, 0.12
        tot = 0.0
        for g in range(ng):
            p = alias_distribution(s, g)
            a, b = s["group_start"][g], s["group_start"][g + 1]
            est, exact = 0.0, 0.0
            for e in range(a, b):
                bb, gg = s["band"][e], s["gq"][e]
                kv = np.array([[np.interp(x, tb["X0"] + tb["dX"] * np.arange(4), t["k"][bb, gg, it])
                                for it in range(20)]])[0]
                k = np.interp(T, tb["T0"] + tb["dT"] * np.arange(20), kv)
                ib = ib_interp(t["Ib"], tb["T0"], tb["dT"], bb, T)
                est += p[e - a] * s["W"][e] * k * ib
                exact += 4 * np.pi * 100 * tb["dnu"][bb] * tb["wq"][gg] * k * ib
            assert abs(est / exact - 1) < 1e-5
            tot += est
        sv.close()


def test_local_temperature_bins_emission_identity():
    """Local sampling: one alias table per table temperature; every bin is an
    unbiased sampler of the same emission sum, and bins differ in density."""
    from dnsmc_gb300 import synth
    tb = synth.ck_table(nbands=8, nq=4, nT=12, nX=3, seed=5)
    sv = D.Solver(D.default_config(model=D.MODEL_TABLE, n_groups=2, local_sampling=1))
    sv.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    s = sv.prepare_sampling(2000.0, 0.1)
    t = sv.table()
    assert s["n_tbins"] == 12 and s["group_start"].size == 12 * 2 + 1
    T, x = 900.0, 0.08
    Tg = tb["T0"] + tb["dT"] * np.arange(12)
    Xg = tb["X0"] + tb["dX"] * np.arange(3)
    dens = []
    for b in (0, 5, 11):
        for g in range(2):
            sub = dict(s)
            sub["group_start"] = s["group_start"][b * 2:]
            p = alias_distribution(sub, g)
            a, e_ = int(s["group_start"][b * 2 + g]), int(s["group_start"][b * 2 + g + 1])
            est = exact = 0.0
            for e in range(a, e_):
                bb, gg = s["band"][e], s["gq"][e]
                kv = np.array([np.interp(x, Xg, t["k"][bb, gg, it]) for it in range(12)])
                k = np.interp(T, Tg, kv)
                ib = ib_interp(t["Ib"], tb["T0"], tb["dT"], bb, T)
                est += p[e - a] * s["W"][e] * k * ib
                exact += 4 * np.pi * 100 * tb["dnu"][bb] * tb["wq"][gg] * k * ib
            assert abs(est / exact - 1) < 1e-5
            if g == 0:
                dens.append(p)
    assert np.abs(dens[0] - dens[2]).max() > 1e-3  # cold and hot bins sample differently
    sv.close()


def test_rqmc_requires_replicates_and_divisible_rays():
    with pytest.raises(D.DnsmcError):
        D.Solver(D.default_config(sampler=D.SAMPLER_RQMC, nvar=1))
    s = D.Solver(D.default_config(model=D.MODEL_GREY, sampler=D.SAMPLER_RQMC, nvar=4, imax=8, jmax=8, kmax=8))
    assert s.packet_shape() == (8, 8)  # the grey black-wall march: 64-cell packets, two cells per lane
    assert s.packet_count() == 8        # one packet per wall-normal plane
    with pytest.raises(D.DnsmcError) as e:
        s.set_rays(10)
    assert e.value.code == _lib.ERR_ARG
    s.close()


@pytest.mark.parametrize("jmax,kmax,grid_num,tile_a,shape", [
    (32, 32, 1, 0, (8, 8)), (32, 8, 1, 0, (8, 8)), (32, 6, 1, 0, (16, 4)), (32, 4, 1, 0, (16, 4)),
    (32, 2, 1, 0, (32, 2)), (32, 32, 1, 16, (16, 4)), (32, 32, 1, 32, (32, 2)),
    (64, 64, 5, 0, (32, 1)), (64, 64, 5, 8, (8, 4))])
def test_automatic_packet_shape(jmax, kmax, grid_num, tile_a, shape):
    """64-cell packets of the two-cell march: 8 x 8 unless k is shorter than
    8 (16 x 4) or 4 (32 x 2) cells or tile_a asks otherwise; 32-cell packets
    of the multigrid march: the widest row.  The packet count covers every
    cell of every wall-normal plane."""
    cfg = D.default_config(model=D.MODEL_GREY, imax=16, jmax=jmax, kmax=kmax, grid_num=grid_num, tile_a=tile_a)
    if grid_num > 1:
        cfg.imax = 64
    s = D.Solver(cfg)
    assert s.packet_shape() == shape
    ta, tb = shape
    assert s.packet_count() == cfg.imax * -(-jmax // ta) * -(-kmax // tb)
    s.close()


def test_multigrid_config_checks():
    """grid_num > 1 needs grid sizes divisible by 2^(grid_num - 1) and
    mg_steps >= 1; the reference's shipped 5 levels on 64^3 are valid."""
    D.Solver(D.default_config(grid_num=5)).close()
    for kw in (dict(grid_num=3, mg_steps=0), dict(grid_num=4, imax=36), dict(grid_num=2, kmax=33)):
        with pytest.raises(D.DnsmcError):
            D.Solver(D.default_config(**kw))
