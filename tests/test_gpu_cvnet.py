"""GPU tests of the learned control variate (dnsmc_cvnet_*, mc_cvnet.cu).

* features: bit-exact against the oracle (oracle/cvnet_oracle.py), with and
  without an x_H2O axis, on a sub-region of a stretched grid;
* forward pass and gradients of the BF16 tensor-core kernels against the
  oracle's bf16-mimicking float64 pass and against the exact float64
  gradient;
* apply: the coefficients and ray counts the network writes into a solver,
  and a bit-exact solve with them against the host replay;
* gain: a network trained on Monte Carlo moments of correlated-k channel
  snapshots lowers variance x cost on an unseen snapshot against the plain
  control variate (beta = (1, -1), uniform rays), and the estimate stays
  unbiased.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import cvtrain, synth
from oracle import cvnet_oracle as NO
from test_gpu_cv import assert_bitexact_cv
from test_gpu_parity import packet_index, smooth_field

pytestmark = pytest.mark.gpu


def small_table():
    return synth.ck_table(nbands=16, nq=8, nT=24, nX=5, seed=4)


def table_solver(tb, ni, nj, nk, **kw):
    cfg = dict(model=D.MODEL_TABLE, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14, stretched_x=0,
               T_west=400, T_east=400, seed=21, n_groups=4)
    cfg.update(kw)
    s = D.Solver(D.default_config(**cfg))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    return s


def random_params(seed):
    rng = np.random.default_rng(seed)
    p = NO.init_params(seed)
    p[NO.OFF_W4:NO.OFF_B4] = rng.normal(0, 0.05, NO.NOUT * NO.HID)
    p[NO.OFF_B1:NO.OFF_W2] = rng.normal(0, 0.1, NO.HID)
    p[NO.OFF_B4:] = rng.normal(0, 0.1, NO.NOUT)
    return p.astype(np.float32)


def test_features_bitexact():
    tb = small_table()
    s = table_solver(tb, 24, 32, 6, stretched_x=1)
    T = np.stack([smooth_field(24, 32, 6, 450, 1700, 5 + f) for f in range(2)])
    x = np.stack([(0.1 + 0.05 * np.random.default_rng(9 + f).uniform(-1, 1, (6, 32, 24))).astype(np.float32)
                  for f in range(2)])
    s.set_fields(T, x)
    s.set_region(2, 21, 3, 30, 1, 5)
    net = D.CvNet(cvtrain.feature_config(tb, groups=4))
    F = net.features(s)
    xu, _, _ = s.geometry()
    net_cfg = cvtrain.feature_config(tb, groups=4)
    ref = NO.features(T, x, xu, s._region, net_cfg.T_center, net_cfg.T_scale, net_cfg.x_center, net_cfg.x_scale)
    np.testing.assert_array_equal(F, ref)
    assert np.abs(F).max() <= 1.0 + 1e-6
    # T-only model: x features are zero
    g = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=4, kappa=1.0, T_west=300,
                                  T_east=300))
    Tg = smooth_field(16, 32, 4, 300, 1000, 3)
    g.set_fields(Tg)
    Fg = net.features(g)
    xg, _, _ = g.geometry()
    refg = NO.features(Tg[None], None, xg, g._region, net_cfg.T_center, net_cfg.T_scale, net_cfg.x_center,
                       net_cfg.x_scale)
    np.testing.assert_array_equal(Fg, refg)
    assert np.all(Fg[:, 1] == 0) and np.all(Fg[:, 35:] == 0)
    s.close(); g.close(); net.close()


def test_forward_matches_oracle():
    net = D.CvNet(D.cvnet_default_config())
    p = random_params(3)
    net.set_params(p, (1.0, 1.0, 1.0))
    rng = np.random.default_rng(0)
    feats = NO.bf16(rng.uniform(-1, 1, (1000, NO.NFEAT)).astype(np.float32))
    out = net.eval(feats)
    ref, _ = NO.forward(p, feats, mimic=True)
    err = np.abs(out - ref)
    assert err.max() <= 5e-3 * np.abs(ref).max(), err.max()
    assert math.sqrt((err ** 2).mean()) <= 5e-4 * math.sqrt((ref ** 2).mean())
    exact, _ = NO.forward(p, feats, mimic=False)
    assert np.abs(out - exact).max() <= 5e-2 * np.abs(exact).max()
    net.close()


def make_labels(rows, G, seed):
    rng = np.random.default_rng(seed)
    lab = np.zeros((rows, G, 8), np.float32)
    A = rng.normal(size=(rows, G, 3, 3))
    C = np.einsum("rgij,rgkj->rgik", A, A)
    lab[..., 0], lab[..., 1], lab[..., 2] = C[..., 0, 0], C[..., 1, 1], C[..., 2, 2]
    lab[..., 3], lab[..., 4], lab[..., 5] = C[..., 0, 1], C[..., 0, 2], C[..., 1, 2]
    lab[..., 6] = rng.uniform(0.2, 3.0, (rows, G))
    lab[..., 7] = rng.uniform(0.2, 3.0, (rows, G))
    return lab


@pytest.mark.parametrize("rows", [512, 300])
def test_gradient_matches_oracle(rows):
    """Gradients of the tensor-core backward pass: per parameter block,
    relative Frobenius error <= 1.5e-2 against the bf16-mimicking oracle and
    <= 6e-2 against the exact float64 gradient; losses to 1e-4."""
    G = 16
    net = D.CvNet(D.cvnet_default_config(ridge=0.05, n_groups=16))
    p = random_params(7)
    scales = np.array([2.0, 1.3, 0.8], np.float32)
    net.set_params(p, scales)
    rng = np.random.default_rng(1)
    feats = NO.bf16(rng.uniform(-1, 1, (rows, NO.NFEAT)).astype(np.float32))
    lab = make_labels(rows, G, 2)
    g, loss = net.gradient(feats, lab)
    gm, lm, _ = NO.gradient(p, feats, lab, scales, 0.05, mimic=True)
    ge, le, _ = NO.gradient(p, feats, lab, scales, 0.05, mimic=False)
    np.testing.assert_allclose(loss[1:], lm, rtol=1e-4)
    blocks = {"W1": (NO.OFF_W1, NO.OFF_B1), "b1": (NO.OFF_B1, NO.OFF_W2), "W2": (NO.OFF_W2, NO.OFF_B2),
              "b2": (NO.OFF_B2, NO.OFF_W3), "W3": (NO.OFF_W3, NO.OFF_B3), "b3": (NO.OFF_B3, NO.OFF_W4),
              "W4": (NO.OFF_W4, NO.OFF_B4), "b4": (NO.OFF_B4, NO.NPARAM)}
    for name, (a, b) in blocks.items():
        rel_m = np.linalg.norm(g[a:b] - gm[a:b]) / np.linalg.norm(gm[a:b])
        rel_e = np.linalg.norm(g[a:b] - ge[a:b]) / np.linalg.norm(ge[a:b])
        assert rel_m <= 1.5e-2, (name, rel_m)
        assert rel_e <= 6e-2, (name, rel_e)
    W1 = g[NO.OFF_W1:NO.OFF_B1].reshape(NO.HID, NO.K0)
    assert np.all(W1[:, NO.NFEAT:] == 0)
    net.close()


def test_params_roundtrip_and_file(tmp_path):
    net = D.CvNet(D.cvnet_default_config(seed=5))
    p = random_params(11)
    net.set_params(p, (1.5, 2.5, 3.5))
    q, sc = net.params()
    np.testing.assert_array_equal(p, q)
    np.testing.assert_array_equal(sc, [1.5, 2.5, 3.5])
    path = str(tmp_path / "n.cvnet")
    net.save(path)
    m = D.CvNet.load(path)
    q2, sc2 = m.params()
    np.testing.assert_array_equal(q2, p)
    feats = NO.bf16(np.random.default_rng(2).uniform(-1, 1, (64, NO.NFEAT)).astype(np.float32))
    np.testing.assert_array_equal(net.eval(feats), m.eval(feats))
    with pytest.raises(D.DnsmcError):
        net.set_params(np.full(net.param_count(), np.nan, np.float32))
    net.close(); m.close()


def tally_to_dense(a, shape):
    """(nf*ni*nk*nj, ...) rows in tally order -> (nf, nk, nj, ni, ...)."""
    nf, nk, nj, ni = shape
    return a.reshape(nf, ni, nk, nj, *a.shape[1:]).transpose(0, 2, 3, 1, *range(4, a.ndim + 3))


def test_apply_sets_coefficients_and_rays_then_solves_bitexact():
    tb = small_table()
    s = table_solver(tb, 12, 32, 4, sampler=D.SAMPLER_RQMC, nvar=4, local_sampling=1, control_variate=1, seed=5)
    T = smooth_field(12, 32, 4, 450, 1700, 8)
    x = (0.1 + 0.05 * np.random.default_rng(3).uniform(-1, 1, (4, 32, 12))).astype(np.float32)
    s.set_fields(T, x)
    s.set_rays(16)
    s.solve(timeout_s=60)  # sampling tables -> group count
    net = D.CvNet(cvtrain.feature_config(tb, groups=4))
    p = random_params(13)
    net.set_params(p, (1.0, 1.0, 30.0))
    net.apply(s, beta=True, rays=True, mean_rays=16, min_rays=4, max_rays=64)
    out = net.eval(net.features(s))                       # tally order
    dense = tally_to_dense(out, (1, 4, 32, 12))           # (1, nk, nj, ni, 32)
    beta = s.cv_beta()                                    # (1, G, nk, nj, ni, 2)
    for g in range(4):
        np.testing.assert_array_equal(beta[:, g, ..., 0], (np.float32(1) + dense[..., 4 * g]))
        np.testing.assert_array_equal(beta[:, g, ..., 1], (np.float32(-1) + dense[..., 4 * g + 1]))
    rays = s.rays_per_item()
    assert rays.shape == (4, s.packet_count())
    assert (rays % 4 == 0).all() and rays.min() >= 4 and rays.max() <= 64
    # the allocation from the outputs, in float64: n ~ sqrt(v_sum / c), expected steps = 16 x uniform
    v = np.exp(np.clip(out[:, 2:16:4], -15, 15)).reshape(12, 4, 32, 4)     # (i, k, j, g)
    cst = 30.0 * np.exp(np.clip(out[:, 3:16:4], -15, 15)).reshape(12, 4, 32, 4)
    # per packet: v summed, c averaged over its cells
    pt = packet_index(s).transpose(2, 0, 1).ravel()                          # (i, k, j) tally order
    npk = s.packet_count()
    cnt = np.bincount(pt, minlength=npk)
    vs = np.stack([np.bincount(pt, v[..., g].ravel(), npk) for g in range(4)])       # (g, packet)
    cs = np.stack([np.bincount(pt, cst[..., g].ravel(), npk) / cnt for g in range(4)])
    w = np.sqrt(vs / np.maximum(cs, 1e-3))
    lam = 16 * cs.sum() / (w * cs).sum()
    expect = np.clip(np.rint(lam * w / 4) * 4, 4, 64)
    assert np.abs(rays - expect).max() <= 4 and (rays == expect).mean() > 0.9
    s._keep = [rays]
    assert_bitexact_cv(s, T[None], x[None])
    s.close(); net.close()


def test_network_gain_and_unbiasedness():
    """Trained on moments of 8 correlated-k channel snapshots (64^3, 8 band
    groups), the network lowers (sum of per-cell variances) x (ray-voxel
    steps) of an unseen snapshot by more than 1.15x against beta = (1, -1)
    with uniform rays, and the two estimates agree within their errors."""
    n = 64
    tb = synth.ck_table(64, 16, 50, 8, seed=0)
    net, info = cvtrain.train(tb, n, range(1, 9), rays=64, epochs=4, j_slab=32)
    d = synth.ck_channel(n, 0)
    res = {}
    for mode in ("plain-cv", "net"):
        acc_v = acc_c = 0.0
        Qs, Vs = [], []
        for seed in (101, 102, 103):
            s = cvtrain.ck_solver(tb, n, d["T_wall"], seed)
            s.set_fields(d["T"], d["x"])
            s.set_rays(32)
            if mode == "net":
                net.apply(s, beta=True, rays=True, mean_rays=32, min_rays=8, max_rays=1024)
            Q, S = s.solve(timeout_s=120)
            acc_v += float((S ** 2).sum())
            acc_c += float(s.item_steps().sum())
            Qs.append(Q)
            Vs.append(S ** 2)
            s.close()
        res[mode] = (acc_v / 3, acc_c / 3, np.mean(Qs, 0), np.mean(Vs, 0) / 3)
    gain = (res["plain-cv"][0] * res["plain-cv"][1]) / (res["net"][0] * res["net"][1])
    print(f"network gain {gain:.3f} (variance {res['plain-cv'][0] / res['net'][0]:.3f}, "
          f"cost {res['plain-cv'][1] / res['net'][1]:.3f}), training {info}")
    assert gain > 1.15, gain
    z = (res["net"][2] - res["plain-cv"][2]) / np.sqrt(res["net"][3] + res["plain-cv"][3])
    assert math.sqrt(float((z ** 2).mean())) < 1.3
    assert (np.abs(z) > 4.5).mean() < 1e-3
    net.close()
