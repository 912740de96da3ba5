"""Regenerate the golden fixtures of this directory from the reference tree.

    python tests/golden/make_golden.py [/path/to/reference]

Reads (text, with numpy -- independent of the solver's own C parser):
  code/resfortm.txt                   -> resfortm.npz   (x, <Q>_yz, <sigma>_yz, std_yz(Q))
  distr/tables/particles/*            -> particle_tables.npz
  distr/tables/{planck-mean,NarrBand%d,prob_new2}.txt -> ck_tables.npz
The fixtures let the GPU tests run where the reference tree is absent.
Formats: code/read_tables.cpp:20-92 (ck), :185-241 (particles);
distr/write_tables.cpp:23-107 writes them.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_particles(tab: str, nT: int = 52, nB: int = 119) -> dict:
    pm = np.loadtxt(os.path.join(tab, "particles", "planck-mean.txt"))[:nT]
    hdr = np.array([np.loadtxt(os.path.join(tab, "particles", f"NarrBand{b}.txt"), ndmin=1)[:5] for b in range(nB)])
    pr = np.loadtxt(os.path.join(tab, "particles", "prob.txt"))[: nT * nB]
    return dict(Tnb=pm[:, 0].astype(np.float32), kP=pm[:, 1].astype(np.float32),
                wl=hdr[:, 0].astype(np.float32), wr=hdr[:, 1].astype(np.float32), wvc=hdr[:, 2].astype(np.float32),
                kq=hdr[:, 3].astype(np.float32), prob=pr[:, 2].reshape(nT, nB).astype(np.float32))


def read_ck(tab: str, nT: int = 52, nB: int = 119, nQ: int = 16) -> dict:
    pm = np.loadtxt(os.path.join(tab, "planck-mean.txt"))[:nT]
    wl, wr, wvc = np.zeros(nB), np.zeros(nB), np.zeros(nB)
    kavg = np.zeros((nB, nT))
    kq = np.zeros((nB, nT, nQ))
    for b in range(nB):
        with open(os.path.join(tab, f"NarrBand{b}.txt")) as fh:
            head = fh.readline().split()
            wl[b], wr[b], wvc[b] = map(float, head[:3])
            rows = np.array([list(map(float, ln.split())) for ln in fh if ln.strip()])[:nT]
        kavg[b] = rows[:, 2]
        kq[b] = rows[:, 3:3 + nQ]
    p2 = np.loadtxt(os.path.join(tab, "prob_new2.txt"))[: nT * nB]
    return dict(Tnb=pm[:, 0].astype(np.float32), kP=pm[:, 1].astype(np.float32), wl=wl.astype(np.float32),
                wr=wr.astype(np.float32), wvc=wvc.astype(np.float32), kavg=kavg.astype(np.float32),
                kq=kq.astype(np.float32), prob=p2[:, 2].reshape(nT, nB).astype(np.float32),
                probg=p2[:, 3:3 + nQ].reshape(nT, nB, nQ).astype(np.float32))


def main(ref: str) -> None:
    r = np.loadtxt(os.path.join(ref, "code", "resfortm.txt"))
    np.savez_compressed(os.path.join(HERE, "resfortm.npz"), x=r[:, 0], Q=r[:, 1], sigma=r[:, 2], plane_std=r[:, 3])
    tab = os.path.join(ref, "distr", "tables")
    np.savez_compressed(os.path.join(HERE, "particle_tables.npz"), **read_particles(tab))
    np.savez_compressed(os.path.join(HERE, "ck_tables.npz"), **read_ck(tab))
    for f in ("resfortm.npz", "particle_tables.npz", "ck_tables.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DNSMC_REFERENCE", "/root/reference"))
