"""Cells of one snapshot split across ranks (one process per GPU).

Cells are independent given the replicated fields and tables, so a snapshot
shards without any device collective: every rank holds the whole field (the
march needs it), solves the contiguous j-slab of cells it owns, and the
results meet on the host.  This is the reference's own decomposition: the DNS
hands each node the j-slab [xstart(2), xend(2)] of its decomp_2d pencil
(code/rad_main.f:84-102, code/main_comp.f:156-202) and gathers Q_r with MPI
(code/fix_var.f:95-121); here the slab is a solver region and the gather a
torch.distributed collective on host tensors (gloo or NCCL process group).

Slabs are whole packet rows (multiples of the packet width along j, at
most 32 cells), so no packet straddles two ranks, and every rank uses its
own RNG key so the slabs' random streams are independent.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = 0x9E3779B97F4A7C15


def slab(jmax: int, world: int, rank: int, align: int = 32) -> tuple[int, int]:
    """[j0, j1) of `rank`: jmax split into `world` contiguous slabs of whole
    `align`-cell units (the last slabs absorb the remainder)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    units = -(-jmax // align)
    base, extra = divmod(units, world)
    u0 = rank * base + min(rank, extra)
    u1 = u0 + base + (1 if rank < extra else 0)
    return min(jmax, u0 * align), min(jmax, u1 * align)


def rank_seed(seed: int, rank: int) -> int:
    """RNG key of `rank` (distinct per rank, deterministic)."""
    return (int(seed) ^ ((rank * _GOLDEN) & 0xFFFFFFFFFFFFFFFF)) & 0xFFFFFFFFFFFFFFFF


def assemble(parts, jmax: int):
    """Place per-rank slab arrays (..., nk, nj_slab, ni) into full arrays
    (..., nk, jmax, ni); parts = [(j0, j1, array), ...]."""
    shape = list(parts[0][2].shape)
    shape[-2] = jmax
    out = np.zeros(shape, parts[0][2].dtype)
    seen = np.zeros(jmax, bool)
    for j0, j1, a in parts:
        if a.shape[-2] != j1 - j0 or seen[j0:j1].any():
            raise ValueError("slabs overlap or do not match their bounds")
        out[..., j0:j1, :] = a
        seen[j0:j1] = True
    if not seen.all():
        raise ValueError("slabs do not cover the grid")
    return out


def solve_sharded(solver, pg, rank: int, world: int, root: int = 0, compute=None, align: int = 32):
    """Solve this rank's j-slab of the solver's resident snapshots and gather
    (Q, sigma) on `root`.  `solver` holds the whole field; its region is set
    to the slab (all i, all k).  `compute(solver) -> (Q, sigma)` defaults to
    solver.solve().  Returns full-grid (Q, sigma) on root, None elsewhere."""
    cfg = solver.cfg
    j0, j1 = slab(cfg.jmax, world, rank, align)
    parts = None
    if j1 > j0:
        solver.set_region(0, cfg.imax, j0, j1, 0, cfg.kmax)
        Q, S = compute(solver) if compute else solver.solve()
        mine = (j0, j1, np.asarray(Q), np.asarray(S))
    else:
        mine = (j0, j1, None, None)
    if pg is None or world == 1:
        parts = [mine]
    else:
        gathered = [None] * world if rank == root else None
        pg.gather_object(mine, gathered, dst=root)
        parts = gathered
    if rank != root:
        return None
    parts = [p for p in parts if p[2] is not None]
    Q = assemble([(a, b, q) for a, b, q, _ in parts], cfg.jmax)
    S = assemble([(a, b, s) for a, b, _, s in parts], cfg.jmax)
    return Q, S
