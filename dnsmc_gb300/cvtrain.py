"""Training driver of the control-variate network on correlated-k channel
snapshots the Monte Carlo itself produces.

    python -m dnsmc_gb300.cvtrain --n 128 --fields 64 --rays 64 --epochs 3 \\
        --out dnsmc_gb300/nets/ck128_g8.cvnet

Every snapshot (synth.ck_channel with its own seed) is solved with the
control variate and per-ray moments on a sub-region of cells (full wall-normal
lines, a slab of the periodic directions); the network's data are the
region's features and the moment labels.  Training and the data stay on the
device; this module only orchestrates the C ABI (include/dnsmc.h).
"""
from __future__ import annotations

import argparse
import math
import sys
import time

from . import _lib, synth
from .api import CvNet, Solver, cvnet_default_config, default_config

GROUPS = 8
REPLICATES = 4


def ck_solver(table, n: int, T_wall: float, seed: int, *, moments: bool = False, groups: int = GROUPS,
              nvar: int = REPLICATES, cv: bool = True, threads: int = 128, tile_a: int = 0) -> Solver:
    """Solver of the correlated-k channel workload (x, z periodic 2 pi x pi,
    y walls black at T_wall, RQMC rays, sampling at the packet temperature)."""
    cfg = default_config(model=_lib.MODEL_TABLE, imax=n, jmax=n, kmax=n, Lx=2.0, Ly=2 * math.pi, Lz=math.pi,
                         stretched_x=0, T_west=T_wall, T_east=T_wall, n_groups=groups, seed=seed,
                         block_threads=threads, tile_a=tile_a, sampler=_lib.SAMPLER_RQMC, local_sampling=1, nvar=nvar,
                         control_variate=1 if cv else 0, cv_moments=1 if (moments and cv) else 0)
    s = Solver(cfg)
    s.set_table(table["k"], table["wvc"], table["T0"], table["dT"], dnu=table["dnu"], wq=table["wq"],
                X0=table["X0"], dX=table["dX"])
    return s


def feature_config(table, groups: int = GROUPS, **kw):
    """Network configuration whose feature map spans the table's T and x ranges."""
    nT, nX = table["k"].shape[2], table["k"].shape[3]
    T_lo, T_hi = table["T0"], table["T0"] + (nT - 1) * table["dT"]
    x_lo, x_hi = table["X0"], table["X0"] + (nX - 1) * table["dX"]
    return cvnet_default_config(n_groups=groups, T_center=0.5 * (T_lo + T_hi), T_scale=0.5 * (T_hi - T_lo),
                                x_center=0.5 * (x_lo + x_hi), x_scale=max(1e-6, 0.5 * (x_hi - x_lo)), **kw)


def add_snapshots(net: CvNet, table, n: int, seeds, rays: int, j_slab: int | None = None, log=None,
                  groups: int = GROUPS, nvar: int = REPLICATES) -> float:
    """Solve every snapshot (moments on) on cells [0,n) x [j0, j0+j_slab) x
    [0,n) and append them to the network's data; returns the solve seconds."""
    T_wall = synth.ck_channel(8, 0)["T_wall"]
    s = ck_solver(table, n, T_wall, seed=7919, moments=True, groups=groups, nvar=nvar)
    t_solve = 0.0
    try:
        for q, seed in enumerate(seeds):
            d = synth.ck_channel(n, int(seed))
            s.set_fields(d["T"], d["x"])
            if j_slab:
                j0 = (q * j_slab) % n
                s.set_region(0, n, j0, min(n, j0 + j_slab), 0, n)
            s.set_rays(rays)
            t0 = time.time()
            s.solve(timeout_s=600)
            t_solve += time.time() - t0
            net.add_training_data(s)
            if log:
                log(f"snapshot {seed}: {net.training_rows()} rows")
    finally:
        s.close()
    return t_solve


def train(table, n: int, seeds, rays: int = 64, epochs: int = 3, j_slab: int | None = None, net: CvNet | None = None,
          log=None, chunk: int = 0, groups: int = GROUPS, nvar: int = REPLICATES, **cfg) -> tuple[CvNet, dict]:
    """Train on the snapshots `seeds`; with chunk > 0 the data are streamed:
    `chunk` snapshots are solved, trained on for `epochs` passes and dropped
    before the next chunk (device memory stays bounded)."""
    net = net or CvNet(feature_config(table, groups=groups, **cfg))
    seeds = list(seeds)
    step = chunk if chunk > 0 else len(seeds)
    t_data = t_solve = t_train = 0.0
    rows = 0
    losses = None
    for c0 in range(0, len(seeds), step):
        net.clear_training_data()
        t0 = time.time()
        t_solve += add_snapshots(net, table, n, seeds[c0:c0 + step], rays, j_slab, log if chunk == 0 else None,
                                 groups=groups, nvar=nvar)
        t1 = time.time()
        rows += net.training_rows()
        losses = net.train(epochs)
        t2 = time.time()
        t_data += t1 - t0
        t_train += t2 - t1
        if log and chunk:
            log(f"snapshots {c0 + 1}-{min(len(seeds), c0 + step)}: loss {losses}")
    info = dict(fields=len(seeds), rows=rows, rays=rays, epochs=epochs, n=n, chunk=step, groups=groups, nvar=nvar,
                data_s=t_data,
                solve_s=t_solve, train_s=t_train, loss=losses)
    if log:
        log(f"trained: {info}")
    return net, info


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--fields", type=int, default=64)
    ap.add_argument("--first-seed", type=int, default=1)
    ap.add_argument("--rays", type=int, default=64)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--slab", type=int, default=32, help="j cells per snapshot (0: all)")
    ap.add_argument("--chunk", type=int, default=0, help="snapshots per streamed training chunk (0: all at once)")
    ap.add_argument("--groups", type=int, default=GROUPS, help="band groups of the solves (<= 16)")
    ap.add_argument("--nvar", type=int, default=REPLICATES, help="RQMC replicates of the training solves")
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    table = synth.ck_table(64, 16, 50, 8, seed=0)
    seeds = range(a.first_seed, a.first_seed + a.fields)
    net, info = train(table, a.n, seeds, a.rays, a.epochs, a.slab or None, chunk=a.chunk, groups=a.groups, nvar=a.nvar,
                      log=lambda m: print(m, file=sys.stderr, flush=True))
    net.save(a.out)
    print(info)
    return 0


if __name__ == "__main__":
    sys.exit(main())
