"""Failure paths of the marches on the GPU, driven without a fault.

The table slab of every ray arrives by a bulk copy whose completion the warp
awaits on a transaction barrier, with a bounded number of polls.  The
environment variable DNSMC_TEST_SLAB_FIRST_POLLS = 0 makes every first wait
run out at once (the copy itself is ordinary and arrives): the warp must set
DNSMC_STATUS_COPY_TIMEOUT, receive the copy in its second wait and carry on,
and the host must report the solve as failed (DNSMC_ERR_TIMEOUT).  The next
solve without the variable must be clean and give the same field as before
(the solves are deterministic), so the barrier phases stayed in step.
Covered for the three marches that copy slabs: the absorbing gas
(march_pair_kernel), the general medium (march_gen_kernel, grey walls) and
the multigrid march (march_mg_kernel, reference tables).
"""
from __future__ import annotations

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import _lib, synth
from tables_io import write_ck_tables
from test_gpu_parity import smooth_field

pytestmark = pytest.mark.gpu


def _table_solver(eps):
    tb = synth.ck_table(nbands=16, nq=8, nT=24, nX=5, seed=4)
    ni, nj, nk = 12, 32, 8
    s = D.Solver(D.default_config(model=D.MODEL_TABLE, imax=ni, jmax=nj, kmax=nk, Lx=2.0, Ly=6.28, Lz=3.14,
                                  stretched_x=0, T_west=400, T_east=400, eps_west=eps, eps_east=eps, seed=5,
                                  n_groups=4, sampler=D.SAMPLER_RQMC, nvar=2, local_sampling=1))
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    T = smooth_field(ni, nj, nk, 450, 1500, 3)
    x = np.full(T.shape, 0.1, np.float32)
    s.set_fields(T, x)
    return s


def _multigrid_solver(tmp_path, ck_tables):
    write_ck_tables(str(tmp_path), ck_tables)
    s = D.Solver(D.default_config(model=D.MODEL_CK, imax=16, jmax=32, kmax=8, Lx=0.5, Ly=1.0, Lz=0.25,
                                  stretched_x=1, T_west=600, T_east=800, seed=77, grid_num=3, mg_steps=2,
                                  n_groups=2, sampler=D.SAMPLER_RQMC, nvar=2, local_sampling=1))
    s.load_reference_tables(str(tmp_path), D.MODEL_CK)
    s.set_fields(smooth_field(16, 32, 8, 550, 1000, 8))
    return s


@pytest.mark.parametrize("kind", ["gas", "general", "multigrid"])
def test_slab_copy_timeout_is_reported_and_the_next_solve_is_clean(kind, monkeypatch, tmp_path, ck_tables):
    if kind == "multigrid":
        s = _multigrid_solver(tmp_path, ck_tables)
    else:
        s = _table_solver(1.0 if kind == "gas" else 0.8)
    s.set_rays(8)
    monkeypatch.delenv("DNSMC_TEST_SLAB_FIRST_POLLS", raising=False)
    Q0, S0 = s.solve(timeout_s=60)
    assert s.status() == 0
    monkeypatch.setenv("DNSMC_TEST_SLAB_FIRST_POLLS", "0")
    with pytest.raises(_lib.DnsmcError) as ei:
        s.solve(timeout_s=60)
    assert ei.value.code == _lib.ERR_TIMEOUT
    assert s.status() & _lib.STATUS_COPY_TIMEOUT
    monkeypatch.delenv("DNSMC_TEST_SLAB_FIRST_POLLS")
    Q1, S1 = s.solve(timeout_s=60)
    assert s.status() == 0
    np.testing.assert_array_equal(Q1, Q0)
    np.testing.assert_array_equal(S1, S0)
    s.close()
