"""GPU tests of the general medium: particles with Henyey-Greenstein
scattering (weighted delta tracking with a warp-shared decision) and grey
diffuse walls.

* bit-exact tallies and voxel walks against the host replay, with and
  without the control variate;
* equilibrium: an isothermal medium between walls at its own temperature has
  Q = 0 exactly, whatever the scattering and wall reflections;
* the isothermal grey slab between grey walls against its analytic solution;
* the isothermal, isotropically scattering slab against a Nystrom solution of
  its integral equation (oracle.slab_scatter_divq);
* unbiasedness of the control variate with particles.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import synth
from oracle import oracle as O
from test_gpu_parity import group_mean_var, region_tally_to_dense, rays_per_cell, smooth_field

pytestmark = pytest.mark.gpu


def replay_group_results(s, T, x=None, fv=None):
    Qg, Vg = s.group_results()
    ng = Qg.shape[1]
    c, keep = O.packet_config(s, T, x, fv=fv)
    i0, i1, j0, j1, k0, k1 = s._region
    tal, steps = O.packet_mc(c, ng, (i1 - i0) * (j1 - j0) * (k1 - k0))
    return Qg, Vg, region_tally_to_dense(tal, s, ng), steps


def check_bitexact(s, T, x=None, fv=None):
    s.solve(timeout_s=120)
    Qg, Vg, tal, steps = replay_group_results(s, T, x, fv)
    ng = Qg.shape[1]
    B = s.cfg.nvar
    cv = s.cfg.control_variate == 1
    muY = s.cv_data()["muY"] if cv else None
    for g in range(ng):
        N = rays_per_cell(s, g)
        m, v = group_mean_var(tal[:, g], N, B, s.cfg.sampler == D.SAMPLER_RQMC)
        if cv:
            m = m + 1.0 * muY[:, g, ..., 0]
            m = m + (-1.0) * muY[:, g, ..., 1]
        np.testing.assert_array_equal(Qg[:, g], m)
        np.testing.assert_array_equal(Vg[:, g], v)
    assert s.counters().steps == steps
    assert s.status() == 0


def particle_table(nb, seed=0):
    rng = np.random.default_rng(seed)
    ext = np.exp(rng.normal(0.0, 0.3, nb)).astype(np.float32) * 1.5e5   # per unit volume fraction [1/m]
    alb = rng.uniform(0.3, 0.9, nb).astype(np.float32)
    return (ext * (1 - alb)).astype(np.float32), (ext * alb).astype(np.float32)


def test_bitexact_grey_walls_grey_model():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=12, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=600, eps_west=0.7, eps_east=0.85, kappa=0.4,
                                  seed=3))
    T = smooth_field(12, 32, 4, 400, 1200, 2)
    s.set_fields(T)
    s.set_rays(24)
    check_bitexact(s, T[None])
    s.close()


@pytest.mark.parametrize("cv", [0, 1])
def test_bitexact_particles_scattering_grey_walls(cv):
    tb = synth.ck_table(nbands=16, nq=8, nT=24, nX=5, seed=4)
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=12, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=1, T_west=420, T_east=380, eps_west=0.8, eps_east=0.8, seed=5,
                                  n_groups=4, sampler=D.SAMPLER_RQMC, nvar=4, local_sampling=1, control_variate=cv))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(12, 32, 4, 450, 1700, 8)
    x = (0.1 + 0.05 * np.random.default_rng(3).uniform(-1, 1, (4, 32, 12))).astype(np.float32)
    fv = (1e-5 * (1 + 0.5 * np.random.default_rng(7).uniform(-1, 1, (4, 32, 12)))).astype(np.float32)
    a, sc = particle_table(16)
    s.set_fields(T, x)
    s.set_particles(a, sc, 0.6)
    s.set_particle_field(fv)
    s.set_rays(16)
    check_bitexact(s, T[None], x[None], fv[None])
    # ray walks against the replay's traces, until some with collisions were seen
    nrec = 4096
    c, keep = O.packet_config(s, T[None], x[None], fv=fv[None])
    collided = 0
    for g in range(4):
        for r in range(16):
            rec, n, rng = s.trace(0, g, 5, r, nrec)
            rec_o, n_o, rng_o = O.packet_trace(c, 0, g, 5, r, nrec)
            assert n == n_o and (rng == rng_o).all()
            np.testing.assert_array_equal(rec, rec_o)
            collided += int((rec[:, 3] == 3).any())
        if collided >= 3:
            break
    assert collided >= 3
    s.close()


def test_equilibrium_is_exactly_zero():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=4, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=900, T_east=900, eps_west=0.5, eps_east=0.3, kappa=0.7,
                                  seed=9))
    s.set_fields(np.full((4, 32, 16), 900.0, np.float32))
    s.set_particles(np.array([0.5e5], np.float32), np.array([2.0e5], np.float32), 0.6)
    s.set_particle_field(np.full((4, 32, 16), 1e-5, np.float32))
    s.set_rays(32)
    Q, S = s.solve(timeout_s=60)
    assert np.all(Q == 0.0) and np.all(S == 0.0)
    assert s.counters().steps > 0
    s.close()


def plane_means(Q, S, packets_per_plane):
    """Plane means and their standard errors.  In a uniform medium the cells
    of a packet share every ray, so their errors are identical: the
    independent samples of a plane are its packets, not its cells."""
    return Q[0].mean(axis=(0, 1)), np.sqrt((S[0] ** 2).mean(axis=(0, 1)) / packets_per_plane)


def test_grey_wall_slab_matches_analytic():
    ni = 32
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=32, kmax=8, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=400, T_east=400, eps_west=0.6, eps_east=0.6, kappa=1.0,
                                  seed=13, sampler=D.SAMPLER_RQMC, nvar=4))
    s.set_fields(np.full((8, 32, ni), 1000.0, np.float32))
    s.set_rays(256)
    Q, S = s.solve(timeout_s=120)
    q, e = plane_means(Q, S, s.packet_count() // ni)
    xu, _, _ = s.geometry()
    yc = 0.5 * (xu[1:] + xu[:-1])
    ex = O.slab_grey_walls_divq(yc, 2.0, 1.0, 1000.0, 400.0, 0.6)
    z = (q - ex) / e
    assert math.sqrt(float((z ** 2).mean())) < 2.0, z
    assert np.abs(z).max() < 5.0, z
    # and differs from the black-wall answer by much more than the error
    black = O.slab_grey_walls_divq(yc, 2.0, 1.0, 1000.0, 400.0, 1.0)
    assert np.abs((q - black) / e).mean() > 10
    s.close()


def test_isotropic_scattering_slab_matches_integral_equation():
    ni = 32
    ka, ss = 0.5, 1.0
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=32, kmax=8, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=0.0, T_east=0.0, kappa=ka, seed=17,
                                  sampler=D.SAMPLER_RQMC, nvar=4))
    s.set_fields(np.full((8, 32, ni), 1000.0, np.float32))
    s.set_particles(np.array([0.0], np.float32), np.array([ss / 1e-5], np.float32), 0.0)
    s.set_particle_field(np.full((8, 32, ni), 1e-5, np.float32))
    s.set_rays(512)  # four independent 64-cell packets per plane
    Q, S = s.solve(timeout_s=120)
    q, e = plane_means(Q, S, s.packet_count() // ni)
    xu, _, _ = s.geometry()
    ref = O.slab_scatter_divq(xu.astype(np.float64), ka, ss, 1000.0, 0.0, 0.0)
    z = (q - ref) / np.sqrt(e ** 2 + (2e-4 * np.abs(ref)) ** 2)
    assert math.sqrt(float((z ** 2).mean())) < 2.0, z
    assert np.abs(z).max() < 5.0, z
    # scattering matters here: the non-scattering answer is far off
    noscat = O.slab_divq(0.5 * (xu[1:] + xu[:-1]).astype(np.float64), 2.0, ka, 1000.0, 0.0, 0.0)
    assert np.abs((q - noscat) / e).mean() > 10
    s.close()


def test_control_variate_with_particles_is_unbiased():
    tb = synth.ck_table(nbands=16, nq=8, nT=24, nX=5, seed=2)
    d = synth.ck_channel(32, 0)
    fv = (1e-5 * (1 + 0.5 * synth.fourier_fluct(32, 32, 32, 5))).astype(np.float32)
    a, sc = particle_table(16, 1)
    out = []
    for cv, seed in ((0, 1), (1, 2)):
        s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=32, jmax=32, kmax=32, Lx=2.0, Ly=2 * math.pi,
                                      Lz=math.pi, stretched_x=0, T_west=400, T_east=400, eps_west=0.8,
                                      eps_east=0.8, n_groups=4, seed=seed, sampler=D.SAMPLER_IID,
                                      local_sampling=1, control_variate=cv))
        s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
        s.set_fields(d["T"], d["x"])
        s.set_particles(a, sc, 0.6)
        s.set_particle_field(fv)
        s.set_rays(128)
        out.append(s.solve(timeout_s=300))
        ppp = s.packet_count() // 32  # packets per wall-normal plane
        s.close()
    (Qp, Sp), (Qc, Sc) = out
    z = (Qc - Qp) / np.sqrt(Sp ** 2 + Sc ** 2)
    assert math.sqrt(float((z ** 2).mean())) < 1.25
    # the scattering weights make sigma from 128 rays heavy-tailed: more
    # |z| > 3 than a Gaussian's 0.27 %
    assert (np.abs(z) > 3).mean() < 0.03
    # no shift between the estimators: wall-normal plane means, the packets
    # of a plane as the independent samples (cells of a packet share rays)
    dq = (Qc - Qp)[0].mean(axis=(0, 1))
    sq = np.sqrt(((Sp ** 2 + Sc ** 2)[0]).mean(axis=(0, 1)) / ppp)
    zp = dq / sq
    assert math.sqrt(float((zp ** 2).mean())) < 1.6, zp
    assert np.abs(zp).max() < 4.5, zp
    assert (Sc ** 2).mean() < (Sp ** 2).mean()  # the surrogate still helps with scattering
