"""GPU tests of the batched path: several snapshots in one persistent launch,
ray counts proportional to local optical thickness, CUDA-graph replay of the
solve, and the autotuner with its JSON cache."""
from __future__ import annotations

import json

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import autotune, cvtrain, synth
from test_gpu_cv import assert_bitexact_cv
from test_gpu_parity import assert_bitexact, packet_index, smooth_field

pytestmark = pytest.mark.gpu


def snapshots(n, seeds):
    ds = [synth.ck_channel(n, s) for s in seeds]
    return np.stack([d["T"] for d in ds]), np.stack([d["x"] for d in ds])


def test_adaptive_rays_follow_optical_thickness():
    tb = synth.ck_table(64, 16, 50, 8, seed=0)
    n = 32
    s = cvtrain.ck_solver(tb, n, 400.0, seed=3, cv=False)
    T, x = snapshots(n, (0, 1))
    s.set_fields(T, x)
    s.set_rays_adaptive(40.0, 8, 256)
    rp = s.rays_per_item()
    assert rp.ndim == 1 and rp.shape[0] == s.packet_count()
    assert (rp % 4 == 0).all() and rp.min() >= 8 and rp.max() <= 256
    # expected: Planck-mean kappa on the table grid, bilinear, times (dx dy dz)^(1/3)
    from oracle import oracle as O  # noqa: F401  (tables only)
    Tg = tb["T0"] + tb["dT"] * np.arange(50)
    Xg = tb["X0"] + tb["dX"] * np.arange(8)
    nu = tb["wvc"].astype(np.float64)
    C1, C2 = 3.741771790075259e-16, 0.014387741858429
    Ib = C1 * (nu[:, None] * 100) ** 3 / (np.pi * (np.exp(C2 * nu[:, None] * 100 / Tg[None, :]) - 1))
    kp = np.pi * np.einsum("bgtx,g,bt,b->tx", tb["k"].astype(np.float64), tb["wq"], Ib, tb["dnu"] * 100.0)
    kp /= 5.670373e-08 * Tg[:, None] ** 4
    xu, dy, dz = s.geometry()
    h = np.cbrt(np.diff(xu) * dy * dz)
    from scipy.interpolate import RegularGridInterpolator
    f = RegularGridInterpolator((Tg, Xg), kp)
    tau = f(np.stack([np.clip(T, Tg[0], Tg[-1]), np.clip(x, Xg[0], Xg[-1])], -1).reshape(-1, 2)).reshape(T.shape)
    tau = tau * h[None, None, None, :]
    # per packet: mean over its cells and both snapshots
    pidx = packet_index(s).ravel()                               # (k, j, i) like tau[f]
    npk = s.packet_count()
    tau_p = np.bincount(pidx, tau.mean(axis=0).ravel(), npk) / np.bincount(pidx, minlength=npk)
    expect = np.clip(np.rint(40.0 * tau_p / 4) * 4, 8, 256)
    assert np.abs(rp - expect).max() <= 4
    assert (rp == expect).mean() > 0.95
    s._keep = [rp]
    assert_bitexact(s, T, x)
    s.close()


def test_graph_replay_matches_eager_solves():
    tb = synth.ck_table(16, 8, 24, 5, seed=4)
    n = 24
    T = np.stack([smooth_field(n, 32, 8, 450, 1700, 5 + f) for f in range(2)])
    x = (0.1 + 0.05 * np.random.default_rng(3).uniform(-1, 1, T.shape)).astype(np.float32)
    T2 = np.stack([smooth_field(n, 32, 8, 450, 1650, 15 + f) for f in range(2)])

    def make():
        s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=n, jmax=32, kmax=8, Lx=2.0, Ly=6.28, Lz=3.14,
                                      stretched_x=0, T_west=400, T_east=400, seed=9, n_groups=4,
                                      sampler=D.SAMPLER_RQMC, nvar=4, local_sampling=1, control_variate=1))
        s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
        return s

    eager, graph = make(), make()
    graph.set_graph(True)
    for fields in (T, T2):
        for s in (eager, graph):
            s.set_fields(fields, x)
            s.set_rays_adaptive(60.0, 8, 64)
        for _ in range(2):
            qe, se = eager.solve(timeout_s=60)
            qg, sg = graph.solve(timeout_s=60)
            np.testing.assert_array_equal(qe, qg)
            np.testing.assert_array_equal(se, sg)
    cap, launches = graph.graph_info()
    assert launches == 4 and 1 <= cap <= 2
    assert eager.graph_info() == (0, 0)
    graph._keep = [graph.rays_per_item()]
    assert_bitexact_cv(graph, T2, x)
    eager.close(); graph.close()


def test_batched_snapshots_adaptive_graph_bitexact():
    """Four snapshots of the channel in one persistent march launch, adaptive
    rays, graph replay: tallies bit-exact against the host replay."""
    tb = synth.ck_table(16, 8, 50, 8, seed=1)
    n = 32
    T, x = snapshots(n, (0, 1, 2, 3))
    s = cvtrain.ck_solver(tb, n, 400.0, seed=17, groups=4, cv=False)
    s.set_graph(True)
    s.set_fields(T, x)
    s.set_rays_adaptive(20.0, 8, 64)
    s.solve(timeout_s=120)
    s._keep = [s.rays_per_item()]
    assert_bitexact(s, T, x)
    assert s.graph_info()[1] == 2
    s.close()


def test_autotuner_sweeps_and_caches(tmp_path):
    tb = synth.ck_table(16, 8, 50, 8, seed=1)
    n = 32
    d = synth.ck_channel(n, 0)
    calls = []

    def make(bt, ta, ng):
        calls.append((bt, ta, ng))
        return cvtrain.ck_solver(tb, n, 400.0, seed=5, groups=ng, threads=bt, tile_a=ta, cv=True)

    def inputs(s):
        s.set_fields(d["T"], d["x"])

    space = {"block_threads": (128, 256), "tile_a": (16,), "group_bands": (4, 8)}
    path = str(tmp_path / "tune.json")
    r = autotune.autotune(make, inputs, "ck32 test", nbands=16, rays=8, space=space, path=path)
    assert not r["cached"] and len(r["results"]) == 4 and len(calls) == 4
    assert r["config"]["block_threads"] in (128, 256) and r["config"]["n_groups"] in (4, 2)
    assert all(v["efficiency"] > 0 for v in r["results"])
    r2 = autotune.autotune(make, inputs, "ck32 test", nbands=16, rays=8, space=space, path=path)
    assert r2["cached"] and len(calls) == 4 and r2["config"] == r["config"]
    assert json.load(open(path))
