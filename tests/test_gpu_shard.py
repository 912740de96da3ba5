"""The multi-rank split through the real solver on the GPU.

shard.solve_sharded with the solver's own solve (no stand-in): with one rank
it equals the unsharded solve; with two gloo ranks -- two processes sharing
this one GPU, each with the whole field, its own j-slab and its own RNG key,
their kernels independent of each other -- the field gathered on rank 0
equals, slab by slab and bit for bit, the same slabs solved one after the
other in this process with the same keys (the reference's j-slab split,
code/rad_main.f:84-113).
"""
from __future__ import annotations

import math
import os
import socket

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import shard, synth

pytestmark = pytest.mark.gpu

NI, NJ, NK = 16, 64, 8


def _solver(seed):
    tb = synth.ck_table(nbands=16, nq=8, nT=50, nX=5, seed=4)
    cfg = D.default_config(model=D.MODEL_TABLE, imax=NI, jmax=NJ, kmax=NK, Lx=2.0, Ly=2 * math.pi, Lz=math.pi,
                           stretched_x=0, T_west=400, T_east=400, seed=seed, n_groups=4, sampler=D.SAMPLER_RQMC,
                           nvar=2, local_sampling=1, control_variate=1)
    s = D.Solver(cfg)
    s.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    d = synth.ck_channel(NJ, 3)
    T = np.ascontiguousarray(d["T"][:NK, :, :NI])
    x = np.ascontiguousarray(d["x"][:NK, :, :NI])
    s.set_fields(T, x)
    s.set_rays(16)
    return s


def test_one_rank_equals_the_unsharded_solve():
    s = _solver(11)
    Q, S = s.solve(timeout_s=120)
    Qs, Ss = shard.solve_sharded(s, None, 0, 1)
    np.testing.assert_array_equal(Qs, Q)
    np.testing.assert_array_equal(Ss, S)
    s.close()


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s = _solver(shard.rank_seed(7, rank))
    res = shard.solve_sharded(s, dist, rank, world)
    if rank == 0:
        np.savez(out, Q=res[0], S=res[1])
    dist.barrier()
    dist.destroy_process_group()
    s.close()


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def test_two_ranks_gather_the_solver_slabs(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "q.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    Q = np.zeros((1, NK, NJ, NI))
    S = np.zeros_like(Q)
    for r in range(2):
        s = _solver(shard.rank_seed(7, r))
        j0, j1 = shard.slab(NJ, 2, r)
        s.set_region(0, NI, j0, j1, 0, NK)
        q, sg = s.solve(timeout_s=120)
        Q[..., j0:j1, :], S[..., j0:j1, :] = q, sg
        s.close()
    np.testing.assert_array_equal(got["Q"], Q)
    np.testing.assert_array_equal(got["S"], S)
    assert np.isfinite(Q).all() and np.abs(Q).max() > 0
