"""GPU tests of the multigrid march (grid_num > 1, the reference's grid
switch, code/mc_gpu.cu:193-207): after mg_steps steps on a grid a ray
continues on the next grid, 2x coarser per axis, whose temperature is the
spline-coarsened field (code/spline.cpp:35-116).

* coarse fields bit-exact against the oracle's restatement of interp3D;
* tallies and traced walks (into the coarse levels) bit-exact against the
  host replay, grey and reference tables, stretched and uniform grids;
* the golden code/resfortm.txt, which the reference produced with its
  shipped grid_num = 5, through the handle API and through the drop-in pair.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import dnsmc_gb300 as D
from oracle import oracle as O
from tables_io import write_ck_tables, write_particle_tables
from test_gpu_parity import assert_bitexact, smooth_field

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("stretched", [1, 0])
def test_coarse_fields_match_the_oracle(stretched):
    ni, nj, nk = 32, 32, 16
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=stretched, grid_num=4, kappa=1.0, T_west=300, T_east=300))
    T = np.stack([smooth_field(ni, nj, nk, 400, 1200, 3 + f) for f in range(2)])
    s.set_fields(T)
    for f in range(2):
        Tf = np.zeros((nk + 2, nj + 2, ni + 2), np.float32)
        Tf[1:-1, 1:-1, 1:-1] = T[f]
        for lv in (1, 2, 3):
            ref = O.coarsen(Tf.ravel(), ni, nj, nk, 2.0, 6.28, 3.14, stretched, 4, lv)[1:-1, 1:-1, 1:-1]
            np.testing.assert_array_equal(s.coarse_field(f, lv), ref)
    s.close()


def test_coarse_fields_from_device_inputs_and_with_x():
    """The coarsening reads the packed device field: fields given as device
    arrays, and fields carrying x_H2O (the T of each (T, x) pair), give the
    same coarse temperatures as host temperatures alone."""
    torch = pytest.importorskip("torch")
    import ctypes
    from dnsmc_gb300 import _lib
    ni, nj, nk = 24, 16, 8
    cfg = D.default_config(model=D.MODEL_GREY, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                           stretched_x=1, grid_num=3, kappa=1.0, T_west=300, T_east=300)
    T = smooth_field(ni, nj, nk, 450, 1300, 9)
    ref = D.Solver(cfg)
    ref.set_fields(T)
    a = D.Solver(cfg)
    dT = torch.from_numpy(T).cuda()
    torch.cuda.synchronize()
    _lib.check(a._lib.dnsmc_set_fields_device(a._h, 1, ctypes.c_void_p(dT.data_ptr()), None))
    b = D.Solver(cfg)
    b.set_fields(T, np.full(T.shape, 0.1, np.float32))
    for lv in (1, 2):
        np.testing.assert_array_equal(a.coarse_field(0, lv), ref.coarse_field(0, lv))
        np.testing.assert_array_equal(b.coarse_field(0, lv), ref.coarse_field(0, lv))
    for s in (ref, a, b):
        s.close()


def traces_reach_coarse_levels(s, T, x=None, n=12):
    c, keep = O.packet_config(s, T, x)
    npk = s.packet_count()
    coarse = 0
    for q in range(n):
        p, r = (q * 7919) % npk, q % 8
        rec, nrec, rng = s.trace(0, 0, p, r)
        rec2, nrec2, rng2 = O.packet_trace(c, 0, 0, p, r)
        assert nrec == nrec2
        np.testing.assert_array_equal(rng, rng2)
        np.testing.assert_array_equal(rec, rec2)
        coarse += int((rec[:, 3] >= 16).any())
    return coarse


def test_bitexact_grey_multigrid():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=8, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=300, T_east=500, kappa=0.3, seed=11, grid_num=3,
                                  mg_steps=3))
    T = smooth_field(16, 32, 8, 400, 1200, 1)
    s.set_fields(T)
    s.set_rays(48)
    assert_bitexact(s, T)
    assert traces_reach_coarse_levels(s, T) > 0
    s.close()


def test_bitexact_ck_tables_multigrid_stretched(tmp_path, ck_tables):
    write_ck_tables(str(tmp_path), ck_tables)
    s = D.Solver(D.default_config(model=D.MODEL_CK, imax=16, jmax=32, kmax=8, Lx=0.5, Ly=1.0, Lz=0.25,
                                  stretched_x=1, T_west=600, T_east=800, seed=77, grid_num=4, mg_steps=2,
                                  n_groups=4, sampler=D.SAMPLER_RQMC, nvar=4, local_sampling=1))
    s.load_reference_tables(str(tmp_path), D.MODEL_CK)
    T = smooth_field(16, 32, 8, 550, 1000, 8)
    s.set_fields(T)
    s.set_rays(16)
    assert_bitexact(s, T)
    assert traces_reach_coarse_levels(s, T) > 0
    s.close()


def test_multigrid_rejects_the_control_variate():
    s = D.Solver(D.default_config(model=D.MODEL_GREY, imax=16, jmax=32, kmax=8, grid_num=2, control_variate=1))
    s.set_fields(smooth_field(16, 32, 8, 400, 1200, 1))
    s.set_rays(8)
    with pytest.raises(D.DnsmcError):
        s.solve(timeout_s=30)
    s.close()


def golden_T(xu):
    x = 0.5 * (xu[1:] + xu[:-1])
    return np.broadcast_to((500 - 2000 * x ** 2 + 2000 * x).astype(np.float32), (64, 64, 64)).copy()


def test_golden_resfortm_with_the_shipped_multigrid(tmp_path, particle_tables, resfortm):
    """code/resfortm.txt came from the reference with grid_num = 5 and
    maxs = 5: plane means over a 32x32 patch of every x-row agree."""
    write_particle_tables(str(tmp_path), particle_tables)
    s = D.Solver(D.default_config(seed=9, grid_num=5, mg_steps=5))
    s.load_reference_tables(str(tmp_path), D.MODEL_PARTICLE)
    xu, _, _ = s.geometry()
    s.set_fields(golden_T(xu))
    s.set_region(0, 64, 0, 32, 0, 32)
    s.set_rays(3000)
    Q, S = s.solve(timeout_s=300)
    q = Q[0][:, 0, :].mean(0)  # one lane per packet: 32 independent packets per row
    se = np.sqrt((S[0][:, 0, :] ** 2).sum(0)) / 32
    z = (q - resfortm["Q"]) / np.sqrt(se ** 2 + (resfortm["plane_std"] / 64) ** 2)
    assert math.sqrt((z ** 2).mean()) < 1.6, z
    assert np.abs(z).max() < 4.2, z
    # optically thin: rays nearly parallel to the walls wrap through the
    # periodic coarse grid until the reference's 100000-step cap, as there
    assert s.status() & ~D.STATUS_STEP_CAP == 0
    s.close()


def test_dropin_pair_with_grid_num_from_the_environment(tmp_path, particle_tables, resfortm, monkeypatch):
    """mc_gpu_ / get_results_ with DNSMC_GRID_NUM=5 (the reference's default
    build): interior cells are written and agree with the golden rows."""
    write_particle_tables(str(tmp_path), particle_tables)
    monkeypatch.setenv("DNSMC_TABLES", str(tmp_path))
    monkeypatch.setenv("DNSMC_GRID_NUM", "5")
    monkeypatch.setenv("DNSMC_PHOTMAX", "400")
    D.dropin_release()
    s = D.Solver(D.default_config())
    xu, _, _ = s.geometry()
    s.close()
    Tf = np.zeros((66, 66, 66), np.float32)
    Tf[1:-1, 1:-1, 1:-1] = golden_T(xu)
    Qr = np.full((66, 66, 66), -1.0, np.float32)
    Vr = np.full((66, 66, 66), -1.0, np.float32)
    D.mc_gpu(Tf, 1)
    D.get_results(Qr, Vr)
    D.dropin_release()
    assert (Qr[0] == -1).all() and (Qr[:, 0] == -1).all() and (Qr[..., 0] == -1).all()
    inner = Qr[1:-1, 1:-1, 1:-1]
    assert np.isfinite(inner).all() and (Vr[1:-1, 1:-1, 1:-1] > 0).all()
    rel = inner.mean(axis=(0, 1)) / resfortm["Q"] - 1
    assert np.abs(rel[8:56]).max() < 0.05
