"""Multi-rank path on CPU (gloo): j-slab partition, per-rank RNG keys and the
host gather of a snapshot split across ranks.  Each rank's slab is computed
by the oracle's packet replay (the GPU march's bit-exact restatement), so
the whole path runs without a GPU."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from dnsmc_gb300 import shard


@pytest.mark.parametrize("jmax,world,align", [(128, 2, 32), (128, 3, 32), (96, 4, 32), (40, 2, 8), (33, 2, 32),
                                              (64, 8, 32)])
def test_slabs_cover_the_grid_in_whole_tiles(jmax, world, align):
    sl = [shard.slab(jmax, world, r, align) for r in range(world)]
    cover = np.zeros(jmax, int)
    for j0, j1 in sl:
        cover[j0:j1] += 1
        assert j0 % align == 0
        assert j1 == jmax or j1 % align == 0
    assert (cover == 1).all()
    sizes = [j1 - j0 for j0, j1 in sl]
    assert max(sizes) - min(sizes) <= align


def test_rank_seeds_distinct():
    s = {shard.rank_seed(12345, r) for r in range(64)}
    assert len(s) == 64 and shard.rank_seed(12345, 0) == 12345


def test_assemble_rejects_gaps_and_overlaps():
    a = np.ones((1, 2, 4, 3))
    with pytest.raises(ValueError):
        shard.assemble([(0, 4, a)], 8)
    with pytest.raises(ValueError):
        shard.assemble([(0, 4, a), (2, 6, a)], 8)


def _problem(seed):
    import dnsmc_gb300 as D
    cfg = D.default_config(model=D.MODEL_GREY, imax=8, jmax=64, kmax=2, Lx=2.0, Ly=6.28, Lz=3.14, stretched_x=0,
                           T_west=300, T_east=300, kappa=1.0, seed=seed)
    s = D.Solver(cfg)
    rng = np.random.default_rng(0)
    T = (600 + 300 * rng.random((2, 64, 8))).astype(np.float32)
    s._nfields = 1  # the fields stay on the host: the replay reads T directly
    s.set_rays(8)
    return s, T


def _replay(solver, T):
    """Oracle replay of the solver's region: (Q, sigma) like solver.solve()."""
    from oracle import oracle as O
    c, keep = O.packet_config(solver, T[None], None)
    i0, i1, j0, j1, k0, k1 = solver._region
    ni, nj, nk = i1 - i0, j1 - j0, k1 - k0
    tal, _ = O.packet_mc(c, 1, ni * nj * nk)
    tal = tal.reshape(1, 1, ni, nk, nj, 2).transpose(0, 1, 3, 4, 2, 5)[:, 0]
    N = solver._rays
    m = tal[..., 0] / N
    v = np.maximum(0.0, tal[..., 1] / N - m * m) / (N - 1)
    return m, np.sqrt(v)


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s, T = _problem(shard.rank_seed(7, rank))
    res = shard.solve_sharded(s, dist, rank, world, compute=lambda sv: _replay(sv, T))
    if rank == 0:
        np.savez(out, Q=res[0], S=res[1])
    dist.barrier()
    dist.destroy_process_group()
    s.close()


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def test_two_gloo_ranks_gather_the_slabs(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "q.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    # the same slabs, solved here one after the other
    Q = np.zeros((1, 2, 64, 8))
    S = np.zeros_like(Q)
    for r in range(2):
        s, T = _problem(shard.rank_seed(7, r))
        j0, j1 = shard.slab(64, 2, r)
        s.set_region(0, 8, j0, j1, 0, 2)
        q, sg = _replay(s, T)
        Q[..., j0:j1, :], S[..., j0:j1, :] = q, sg
        s.close()
    np.testing.assert_array_equal(got["Q"], Q)
    np.testing.assert_array_equal(got["S"], S)
    assert np.isfinite(Q).all() and np.abs(Q).max() > 0
