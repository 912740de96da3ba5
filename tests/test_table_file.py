"""The binary table file (dnsmc_save_table / dnsmc_load_table): the
x_H2O-extended k(band, g, T, x) table in one checked file, beside the
reference's text formats (code/read_tables.cpp, distr/write_tables.cpp).

Host logic only (no GPU): the file is read back here by an independent numpy
parser of the documented layout, a loaded table equals the saved one array
for array and gives the same sampling tables, and damaged files are refused
with DNSMC_ERR_IO.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import dnsmc_gb300 as D
from dnsmc_gb300 import _lib, synth
from tables_io import write_ck_tables


def parse(path):
    """The file's documented layout, read with numpy."""
    raw = open(path, "rb").read()
    assert raw[:8] == b"DNSMCKT1"
    ver, hdr, nb, nq, nT, nX = np.frombuffer(raw, "<u4", 6, 8)
    T0, dT, X0, dX = np.frombuffer(raw, "<f4", 4, 32)
    flags, zero = np.frombuffer(raw, "<u4", 2, 48)
    nbytes, hsh = np.frombuffer(raw, "<u8", 2, 56)
    assert (ver, hdr, zero) == (1, 72, 0) and nbytes == len(raw) - 72
    h = 0xcbf29ce484222325
    for b in raw[72:]:  # FNV-1a 64
        h = ((h ^ b) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    assert h == hsh
    v = np.frombuffer(raw, "<f4", offset=72)
    out, o = {}, 0

    def take(name, shape):
        nonlocal o
        n = int(np.prod(shape))
        out[name] = v[o:o + n].reshape(shape)
        o += n

    take("k", (nb, nq, nT, nX))
    take("wvc", (nb,))
    take("dnu", (nb,))
    take("wq", (nq,))
    if flags & 1:
        take("Ib", (nb, nT))
    if flags & 2:
        take("prob", (nT, nb))
        take("kP", (nT,))
    if flags & 4:
        take("probg", (nT, nb, nq))
    assert o == v.size
    out.update(T0=T0, dT=dT, X0=X0, dX=dX, flags=int(flags))
    return out


def sampling_equal(a, b):
    sa, sb = a.sampling(), b.sampling()
    assert sa.keys() == sb.keys()
    for key in sa:
        np.testing.assert_array_equal(np.asarray(sa[key]), np.asarray(sb[key]), err_msg=key)


def test_x_table_roundtrip(tmp_path):
    tb = synth.ck_table(nbands=12, nq=8, nT=20, nX=6, seed=3)
    a = D.Solver(D.default_config(model=D.MODEL_TABLE, n_groups=3, local_sampling=1))
    a.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    path = str(tmp_path / "ck.dnsmctab")
    a.save_table(path)
    f = parse(path)
    assert f["flags"] == 0
    np.testing.assert_array_equal(f["k"], np.asarray(tb["k"], np.float32))
    np.testing.assert_array_equal(f["wvc"], np.asarray(tb["wvc"], np.float32))
    np.testing.assert_array_equal(f["dnu"], np.asarray(tb["dnu"], np.float32))
    np.testing.assert_array_equal(f["wq"], np.asarray(tb["wq"], np.float32))
    assert (f["T0"], f["dT"], f["X0"], f["dX"]) == tuple(np.float32(tb[n]) for n in ("T0", "dT", "X0", "dX"))
    b = D.Solver(D.default_config(model=D.MODEL_TABLE, n_groups=3, local_sampling=1))
    b.load_table(path)
    ta, tb2 = a.table(), b.table()
    for key in ta:
        np.testing.assert_array_equal(np.asarray(ta[key]), np.asarray(tb2[key]), err_msg=key)
    a.prepare_sampling(1700.0, 0.12)
    b.prepare_sampling(1700.0, 0.12)
    sampling_equal(a, b)
    a.close()
    b.close()


def test_reference_tables_roundtrip(tmp_path, ck_tables):
    """Reference text tables parsed once, then served from the binary file:
    the reference CDFs and Planck mean travel with it (flags 2 | 4)."""
    write_ck_tables(str(tmp_path / "txt"), ck_tables)
    a = D.Solver(D.default_config(model=D.MODEL_CK, n_groups=2))
    a.load_reference_tables(str(tmp_path / "txt"), D.MODEL_CK)
    path = str(tmp_path / "ref.dnsmctab")
    a.save_table(path)
    f = parse(path)
    assert f["flags"] & 2 and f["flags"] & 4
    b = D.Solver(D.default_config(model=D.MODEL_TABLE, n_groups=2))
    b.load_table(path)
    ta, tb2 = a.table(), b.table()
    for key in ta:
        np.testing.assert_array_equal(np.asarray(ta[key]), np.asarray(tb2[key]), err_msg=key)
    a.prepare_sampling(1000.0)
    b.prepare_sampling(1000.0)
    sampling_equal(a, b)
    a.close()
    b.close()


@pytest.mark.parametrize("damage", ["payload", "truncate", "magic", "append"])
def test_damaged_files_are_refused(tmp_path, damage):
    tb = synth.ck_table(nbands=4, nq=4, nT=8, nX=3, seed=1)
    a = D.Solver(D.default_config(model=D.MODEL_TABLE))
    a.set_table(tb["k"], tb["wvc"], tb["T0"], tb["dT"], dnu=tb["dnu"], wq=tb["wq"], X0=tb["X0"], dX=tb["dX"])
    path = str(tmp_path / "t.dnsmctab")
    a.save_table(path)
    raw = bytearray(open(path, "rb").read())
    if damage == "payload":
        raw[100] ^= 0x10
    elif damage == "truncate":
        raw = raw[:-4]
    elif damage == "magic":
        raw[0] = ord("X")
    else:
        raw += b"\0\0\0\0"
    open(path, "wb").write(bytes(raw))
    b = D.Solver(D.default_config(model=D.MODEL_TABLE))
    with pytest.raises(D.DnsmcError) as e:
        b.load_table(path)
    assert e.value.code == _lib.ERR_IO
    with pytest.raises(D.DnsmcError) as e:
        b.load_table(os.path.join(str(tmp_path), "missing.dnsmctab"))
    assert e.value.code == _lib.ERR_IO
    a.close()
    b.close()
