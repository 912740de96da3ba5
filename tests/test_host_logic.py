"""CPU tests of host-side logic added around the march: argument checks of
the newer C entry points (no GPU needed: they validate before touching the
device), the autotuner's sweep and JSON cache with a stand-in solver, and
the training driver's network configuration."""
from __future__ import annotations

import json

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import autotune, cvtrain, synth


def grey_solver(**kw):
    cfg = dict(model=D.MODEL_GREY, imax=8, jmax=32, kmax=4, kappa=1.0)
    cfg.update(kw)
    return D.Solver(D.default_config(**cfg))


def test_rays_per_item_argument_checks():
    s = grey_solver(sampler=D.SAMPLER_RQMC, nvar=4)
    with pytest.raises(ValueError):
        s.set_rays_per_item(np.full((1, 7), 8, np.int32))  # wrong packet count (caught in Python)
    np_ = s.packet_count()
    lib = s._lib
    bad = np.full(np_, 6, np.int32)  # not a multiple of nvar
    assert lib.dnsmc_set_rays_per_item(s._h, 1, bad.ctypes.data_as(D._lib.c_int_p)) == D._lib.ERR_ARG
    neg = np.full(np_, -4, np.int32)
    assert lib.dnsmc_set_rays_per_item(s._h, 1, neg.ctypes.data_as(D._lib.c_int_p)) == D._lib.ERR_ARG
    s.close()


def test_adaptive_rays_argument_checks():
    s = grey_solver(sampler=D.SAMPLER_RQMC, nvar=4)
    with pytest.raises(D.DnsmcError):
        s.set_rays_adaptive(10.0, 6, 64)       # min not a multiple of nvar
    with pytest.raises(D.DnsmcError):
        s.set_rays_adaptive(-1.0, 8, 64)       # rays per tau <= 0
    with pytest.raises(D.DnsmcError):
        s.set_rays_adaptive(10.0, 64, 8)       # max < min
    with pytest.raises(D.DnsmcError):
        s.set_rays_adaptive(10.0, 8, 64)       # no fields yet
    s.close()


def test_particle_argument_checks():
    s = grey_solver()
    one = np.ones(1, np.float32)
    with pytest.raises(D.DnsmcError):
        s.set_particles(one, one, 1.0)         # |g| must be < 1
    with pytest.raises(D.DnsmcError):
        s.set_particles(np.ones(2, np.float32), np.ones(2, np.float32), 0.5)  # grey model: one band
    with pytest.raises(D.DnsmcError):
        s.set_particles(-one, one, 0.5)        # negative coefficient
    with pytest.raises(D.DnsmcError):
        s.set_particle_field(np.ones((4, 32, 8), np.float32))  # no temperature fields yet
    s.close()
    # particles need the grey model or raw tables
    tb = synth.ck_table(nbands=4, nq=2, nT=8, nX=3)
    t = D.Solver(D.default_config(model=D.MODEL_CK, imax=8, jmax=32, kmax=4))
    with pytest.raises(D.DnsmcError):
        t.set_particles(np.ones(4, np.float32), np.ones(4, np.float32), 0.0)
    t.close()
    del tb


def test_grey_walls_are_valid_configuration():
    s = grey_solver(eps_west=0.5, eps_east=0.9)
    s.close()
    for bad in (0.0, -0.1, 1.01):
        with pytest.raises(D.DnsmcError):
            grey_solver(eps_west=bad)


def test_network_needs_a_device_and_valid_config():
    c = D.cvnet_default_config()
    assert (c.n_groups, c.batch, round(c.lr, 6), round(c.ridge, 6)) == (8, 4096, 0.001, 0.01)
    lib = D._lib.load()
    import ctypes
    h = ctypes.c_void_p()
    bad = D.cvnet_default_config(n_groups=17)
    assert lib.dnsmc_cvnet_create(ctypes.byref(bad), ctypes.byref(h)) == D._lib.ERR_ARG
    bad = D.cvnet_default_config(batch=100)
    assert lib.dnsmc_cvnet_create(ctypes.byref(bad), ctypes.byref(h)) == D._lib.ERR_ARG
    rc = lib.dnsmc_cvnet_create(ctypes.byref(c), ctypes.byref(h))
    assert rc in (D._lib.OK, D._lib.ERR_NODEVICE)
    if rc == D._lib.OK:
        lib.dnsmc_cvnet_destroy(h)
    assert lib.dnsmc_cvnet_param_count() == 80 * 128 + 128 + 2 * (128 * 128 + 128) + 64 * 128 + 64


def test_feature_config_spans_the_table():
    tb = synth.ck_table(nbands=4, nq=2, nT=11, nX=5, T_range=(300.0, 2300.0), X_range=(0.0, 0.4))
    c = cvtrain.feature_config(tb, groups=4)
    assert c.n_groups == 4
    assert abs(c.T_center - 1300.0) < 1e-3 and abs(c.T_scale - 1000.0) < 1e-3
    assert abs(c.x_center - 0.2) < 1e-6 and abs(c.x_scale - 0.2) < 1e-6


class FakeSolver:
    """Stand-in with the solver methods the autotuner calls; its solve time
    and variance depend on the knobs in a known way."""

    def __init__(self, bt, ta, ng, log):
        self.k = (bt, ta, ng)
        log.append(self.k)

    def set_rays(self, r):
        self.r = r

    def solve(self, timeout_s=0):
        bt, ta, ng = self.k
        self.ms = 100.0 * ng / 8 * (1.0 if bt == 256 else 1.1) * (1.0 if ta == 16 else 1.05)
        S = np.full(10, 1.0 / ng ** 0.5)
        return np.zeros(10), S

    def timing(self):
        return self.ms, self.ms

    def close(self):
        pass


class FakeStratSolver(FakeSolver):
    """More band groups: time ~ groups, RMS error ~ groups^-0.6 (the
    stratification gains a little)."""

    def solve(self, timeout_s=0):
        bt, ta, ng = self.k
        self.ms = 100.0 * ng / 8
        return np.ones(10), np.full(10, ng ** -0.6)


def test_autotuner_at_target_sees_the_ray_floor(tmp_path):
    space = {"block_threads": (256,), "tile_a": (16,), "group_bands": (4, 8)}  # 8 or 4 groups of 32 bands
    err = lambda Q, S: float(np.sqrt((S ** 2).mean() / (Q ** 2).mean()))
    # plain efficiency: 8 groups (variance x time ~ groups^-0.2)
    r = autotune.autotune(lambda bt, ta, ng: FakeStratSolver(bt, ta, ng, []), lambda s: None, "fake", nbands=32,
                          rays=8, space=space, path=str(tmp_path / "a.json"))
    assert r["config"]["n_groups"] == 8
    # at an error of 0.25 with a floor of 20 rays: 8 groups would need 10.5
    # rays (raised to 20, predicted 250 ms), 4 groups 24.2 (151 ms)
    r = autotune.autotune(lambda bt, ta, ng: FakeStratSolver(bt, ta, ng, []), lambda s: None, "fake", nbands=32,
                          rays=8, space=space, path=str(tmp_path / "b.json"), target_error=0.25, floor=20,
                          error_fn=err)
    assert r["config"]["n_groups"] == 4
    by = {x["n_groups"]: x for x in r["results"]}
    assert by[8]["rays_at_target"] == 20.0 and abs(by[8]["ms_at_target"] - 250.0) < 1e-9
    assert abs(by[4]["rays_at_target"] - 8 * (4 ** -0.6 / 0.25) ** 2) < 1e-9
    # without the floor binding, the same ranking as the plain efficiency
    r = autotune.autotune(lambda bt, ta, ng: FakeStratSolver(bt, ta, ng, []), lambda s: None, "fake", nbands=32,
                          rays=8, space=space, path=str(tmp_path / "c.json"), target_error=0.25, floor=1,
                          error_fn=err)
    assert r["config"]["n_groups"] == 8


def test_autotuner_picks_the_most_efficient_and_caches(tmp_path):
    log = []
    space = {"block_threads": (128, 256), "tile_a": (8, 16), "group_bands": (4, 8)}
    path = str(tmp_path / "t.json")
    r = autotune.autotune(lambda bt, ta, ng: FakeSolver(bt, ta, ng, log), lambda s: None, "fake", nbands=32,
                          rays=8, space=space, path=path)
    assert not r["cached"] and len(r["results"]) == 8 and len(log) == 8
    # time ~ groups, variance ~ 1/groups: efficiency independent of groups, so
    # the launch knobs decide: 256 threads and 16-wide packets
    assert r["config"]["block_threads"] == 256 and r["config"]["tile_a"] == 16
    r2 = autotune.autotune(lambda bt, ta, ng: FakeSolver(bt, ta, ng, log), lambda s: None, "fake", nbands=32,
                           rays=8, space=space, path=path)
    assert r2["cached"] and len(log) == 8
    db = json.load(open(path))
    assert len(db) == 1
    r3 = autotune.autotune(lambda bt, ta, ng: FakeSolver(bt, ta, ng, log), lambda s: None, "fake", nbands=32,
                           rays=8, space=space, path=path, force=True)
    assert not r3["cached"] and len(log) == 16
