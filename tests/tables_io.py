"""Writers of the reference's text table formats (for parser tests that must
run where the reference tree is absent).  Formats as read by
code/read_tables.cpp:20-92 (ck) and :185-241 (particles)."""
from __future__ import annotations

import os

import numpy as np


def write_particle_tables(root: str, t: dict) -> str:
    d = os.path.join(root, "particles")
    os.makedirs(d, exist_ok=True)
    nT, nB = t["prob"].shape
    with open(os.path.join(d, "planck-mean.txt"), "w") as fh:
        for i in range(nT):
            fh.write(f"{t['Tnb'][i]:.6f} {t['kP'][i]:.9e}\n")
    for b in range(nB):
        with open(os.path.join(d, f"NarrBand{b}.txt"), "w") as fh:
            fh.write(f"{t['wl'][b]:.9e}\t{t['wr'][b]:.9e}\t{t['wvc'][b]:.9e}\t{t['kq'][b]:.9e}\t{t['kq'][b]:.9e} \n")
    with open(os.path.join(d, "prob.txt"), "w") as fh:
        for i in range(nT):
            for b in range(nB):
                fh.write(f"{t['Tnb'][i]:.6f} \t {b} \t {t['prob'][i, b]:.12e} \n")
    return root


def write_ck_tables(root: str, t: dict) -> str:
    os.makedirs(root, exist_ok=True)
    nT, nB = t["prob"].shape
    nQ = t["kq"].shape[2]
    with open(os.path.join(root, "planck-mean.txt"), "w") as fh:
        for i in range(nT):
            fh.write(f"{t['Tnb'][i]:.6f} {t['kP'][i]:.9e} {t['kP'][i]:.9e} {t['kP'][i]:.9e}\n")
    for b in range(nB):
        with open(os.path.join(root, f"NarrBand{b}.txt"), "w") as fh:
            fh.write(f"{t['wl'][b]:.9e}\t{t['wr'][b]:.9e}\t{t['wvc'][b]:.9e} \n")
            for i in range(nT):
                row = "\t ".join(f"{v:.9e}" for v in t["kq"][b, i])
                fh.write(f" {t['Tnb'][i]:.6f}\t {0.0:.6e}\t {t['kavg'][b, i]:.9e}\t {row}\t\n")
    with open(os.path.join(root, "prob_new2.txt"), "w") as fh:
        for i in range(nT):
            for b in range(nB):
                row = "\t ".join(f"{v:.12e}" for v in t["probg"][i, b])
                fh.write(f"{t['Tnb'][i]:.6f} \t {b} \t {t['prob'][i, b]:.12e} \t {row}\t\n")
    return root
