"""TEST INFRASTRUCTURE ONLY -- Python side of the oracle.

* ctypes wrappers of oracle/liboracle.so (mc_oracle.cpp): the reference-
  structured MC (code/mc_gpu.cu:44-438, 813-896) in FP32 or FP64, the packet
  replay, Philox, the reference grids and the spline coarsening;
* the analytic isothermal grey slab: div q(tau) = 2 kappa sigma
  [(T^4 - Tw1^4) E2(tau) + (T^4 - Tw2^4) E2(tau_L - tau)] (exact solution of
  the radiative transfer equation for a non-scattering isothermal slab between
  black walls; E_n by series / continued fraction, written from their
  definitions);
* the optically thin limit 4 sigma (kappa_P(T) T^4 - kappa_P(T_w) T_w^4) per
  cell for black walls (used to pin the oracle to code/resfortm.txt);
* readers of the reference's own table reader built in oracle/_ref.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import build as _build

SIGMA = 5.670373e-08  # code/param.h:70

_f = ctypes.POINTER(ctypes.c_float)
_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)
_u32 = ctypes.POINTER(ctypes.c_uint32)
_i32 = ctypes.POINTER(ctypes.c_int32)


class RefConfig(ctypes.Structure):
    _fields_ = [
        ("imax", ctypes.c_int), ("jmax", ctypes.c_int), ("kmax", ctypes.c_int),
        ("Lx", ctypes.c_float), ("Ly", ctypes.c_float), ("Lz", ctypes.c_float),
        ("stretched", ctypes.c_int), ("grid_num", ctypes.c_int), ("maxs", ctypes.c_int * 6),
        ("T_west", ctypes.c_float), ("T_east", ctypes.c_float), ("toll", ctypes.c_float),
        ("nvar", ctypes.c_int), ("photmax", ctypes.c_int), ("hwfilter", ctypes.c_int),
        ("use_double", ctypes.c_int), ("seed", ctypes.c_uint64), ("model", ctypes.c_int),
        ("kappa", ctypes.c_float), ("nT", ctypes.c_int), ("nB", ctypes.c_int), ("nQ", ctypes.c_int),
        ("Tnb", _f), ("kq", _f), ("wvc", _f), ("prob", _f), ("probg", _f), ("kP", _f),
    ]


class PacketConfig(ctypes.Structure):
    _fields_ = [
        ("nw", ctypes.c_int), ("na", ctypes.c_int), ("nb", ctypes.c_int),
        ("da", ctypes.c_float), ("db", ctypes.c_float), ("fw", _f),
        ("ew0", ctypes.c_int), ("ew1", ctypes.c_int), ("ea0", ctypes.c_int), ("ea1", ctypes.c_int),
        ("eb0", ctypes.c_int), ("eb1", ctypes.c_int), ("tile_a", ctypes.c_int), ("mode", ctypes.c_int),
        ("nfields", ctypes.c_int), ("fieldT", _f), ("fieldX", _f),
        ("nbands", ctypes.c_int), ("nq", ctypes.c_int), ("nT", ctypes.c_int), ("nX", ctypes.c_int),
        ("T0", ctypes.c_float), ("dT", ctypes.c_float), ("X0", ctypes.c_float), ("dX", ctypes.c_float),
        ("ktab", _f), ("ibtab", _f), ("ibw", _f), ("n_groups", ctypes.c_int), ("group_start", _i),
        ("prob", _f), ("alias", _i), ("band", _i), ("gq", _i), ("W", _f),
        ("kappa", ctypes.c_float), ("T_west", ctypes.c_float), ("T_east", ctypes.c_float),
        ("rays", ctypes.c_int), ("rays_per_packet", _i), ("rays_gstride", ctypes.c_int), ("seed", ctypes.c_uint64),
        ("toll", ctypes.c_float), ("max_steps", ctypes.c_int), ("use_double", ctypes.c_int),
        ("sampler", ctypes.c_int), ("nbatch", ctypes.c_int), ("n_tbins", ctypes.c_int),
        ("cv", ctypes.c_int), ("sur_k", _f), ("sur_I", _f), ("beta", _f), ("moments", _d),
        ("gen", ctypes.c_int), ("fieldV", _f), ("part", _f), ("fv_max", ctypes.c_float), ("hg_g", ctypes.c_float),
        ("eps", ctypes.c_float * 2),
        ("mg_levels", ctypes.c_int), ("mg_steps", ctypes.c_int), ("mgT", _f), ("mgfw", _f),
        ("mg_off", ctypes.c_longlong * 6), ("mg_fwoff", ctypes.c_int * 6), ("mg_da", ctypes.c_float * 6),
        ("mg_db", ctypes.c_float * 6), ("Ly", ctypes.c_float), ("Lz", ctypes.c_float),
        ("cpl", ctypes.c_int), ("pw_step", ctypes.c_int), ("sur_tab", _f),
    ]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.lib_path()):
            _build.build(with_ref=False)
        lib = ctypes.CDLL(_build.lib_path())
        lib.orc_philox.argtypes = [_u32, _u32, _u32]
        lib.orc_ref_faces.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, _f]
        lib.orc_ref_mc.argtypes = [ctypes.POINTER(RefConfig), _f, ctypes.c_int, _i, ctypes.c_int, _d, _d, _d, _d]
        lib.orc_ref_mc.restype = ctypes.c_int
        lib.orc_coarsen.argtypes = [ctypes.c_int] * 3 + [ctypes.c_float] * 3 + [ctypes.c_int, ctypes.c_int, _f,
                                                                                 ctypes.c_int, _f]
        lib.orc_packet_mc.argtypes = [ctypes.POINTER(PacketConfig), ctypes.c_int, _d, _d]
        lib.orc_packet_mc.restype = ctypes.c_int
        lib.orc_packet_trace.argtypes = [ctypes.POINTER(PacketConfig)] + [ctypes.c_int] * 5 + [_i32, _i, _u32]
        lib.orc_expm1n.argtypes = [_f, _f, ctypes.c_longlong]
        lib.orc_cv_mean.argtypes = [ctypes.POINTER(PacketConfig), _i, _i, _d, _d, _d, ctypes.c_int, ctypes.c_int,
                                    _d]
        lib.orc_cv_mean.restype = ctypes.c_int
        lib.orc_cv_table.argtypes = [ctypes.POINTER(PacketConfig), _f, _d]
        lib.orc_cv_table.restype = ctypes.c_int
        _ll = ctypes.POINTER(ctypes.c_longlong)
        lib.orc_ck_from_lbl.argtypes = [_d, ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_int, _ll, _i,
                                        _d, _d, ctypes.c_int, _d, ctypes.c_int, ctypes.c_int, _f, _d]
        lib.orc_ck_from_lbl.restype = ctypes.c_int
        _lib = lib
    return _lib


def _fp(a):
    return None if a is None else a.ctypes.data_as(_f)


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (ctypes.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (ctypes.c_uint32 * 4)()
    load().orc_philox(c, k, o)
    return list(o)


def expm1n(x) -> np.ndarray:
    """The march's FP32 expm1 of x <= 0 (the same operations as the device's
    mc_expm1), element by element."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    load().orc_expm1n(_fp(x), _fp(out), x.size)
    return out


def ref_faces(im: int, L: float, stretched: int = 1, im0: int | None = None) -> np.ndarray:
    xu = np.zeros(im + 1, np.float32)
    load().orc_ref_faces(im, im0 or im, L, stretched, _fp(xu))
    return xu


# ---------------------------------------------------------------------------
# reference-structured MC
# ---------------------------------------------------------------------------
def ref_mc(T_fort: np.ndarray, cells: np.ndarray, *, imax, jmax, kmax, Lx, Ly, Lz, T_west, T_east,
           model: int, tables: dict | None = None, kappa: float = 1.0, nvar: int = 3, photmax: int = 1000,
           grid_num: int = 1, maxs=None, stretched: int = 1, toll: float = 1e-3, hwfilter: int = 0,
           use_double: int = 1, seed: int = 1234, threads: int = 0) -> dict:
    """Run the reference estimator on `cells` ((n, 3) 1-based i, j, k).

    tables (model 0 ck / 2 particle): Tnb [nT], kq [nB][nT][nQ], wvc [nB],
    prob [nT][nB], probg [nT][nB][nQ] or None, kP [nT].  model 1 builds the
    reference grey-band tables from Tmax itself.
    """
    lib = load()
    c = RefConfig()
    c.imax, c.jmax, c.kmax = imax, jmax, kmax
    c.Lx, c.Ly, c.Lz = Lx, Ly, Lz
    c.stretched, c.grid_num = stretched, grid_num
    if maxs is None:
        maxs = [5] * (grid_num - 1) + [100000]
    for i, v in enumerate(maxs):
        c.maxs[i] = v
    c.T_west, c.T_east, c.toll = T_west, T_east, toll
    c.nvar, c.photmax, c.hwfilter, c.use_double, c.seed = nvar, photmax, hwfilter, use_double, seed
    c.model, c.kappa = model, kappa
    keep = []
    if model != 1:
        t = {k: (None if v is None else np.ascontiguousarray(v, np.float32)) for k, v in tables.items()}
        keep.append(t)
        c.nT, c.nB = t["Tnb"].size, t["wvc"].size
        c.nQ = t["kq"].shape[-1] if t["kq"].ndim == 3 else 1
        c.Tnb, c.kq, c.wvc, c.prob, c.kP = (_fp(t["Tnb"]), _fp(t["kq"]), _fp(t["wvc"]), _fp(t["prob"]),
                                            _fp(t["kP"]))
        c.probg = _fp(t.get("probg"))
    T = np.ascontiguousarray(T_fort, np.float32)
    assert T.size == (imax + 2) * (jmax + 2) * (kmax + 2)
    cl = np.ascontiguousarray(cells, np.int32).reshape(-1, 3)
    n = cl.shape[0]
    sol, var, se, steps = (np.zeros(n) for _ in range(4))
    rc = lib.orc_ref_mc(ctypes.byref(c), _fp(T), n, cl.ctypes.data_as(_i), threads,
                        sol.ctypes.data_as(_d), var.ctypes.data_as(_d), se.ctypes.data_as(_d),
                        steps.ctypes.data_as(_d))
    assert rc == 0
    return dict(Q=sol, var_ref=var, se=se, steps=steps)


def coarsen(T_fort, imax, jmax, kmax, Lx, Ly, Lz, stretched, grid_num, level):
    im, jm, km = imax >> level, jmax >> level, kmax >> level
    out = np.zeros((km + 2) * (jm + 2) * (im + 2), np.float32)
    load().orc_coarsen(imax, jmax, kmax, Lx, Ly, Lz, stretched, grid_num,
                       _fp(np.ascontiguousarray(T_fort, np.float32)), level, _fp(out))
    return out.reshape(km + 2, jm + 2, im + 2)


# ---------------------------------------------------------------------------
# packet replay: takes the solver's own geometry, tables and sampling
# ---------------------------------------------------------------------------
def packet_config(solver, T: np.ndarray, x: np.ndarray | None, *, use_double: int = 0, mode: int | None = None,
                  fv: np.ndarray | None = None):
    """Build a PacketConfig mirroring `solver`'s last solve (tables, sampling,
    geometry, region, rays).  T, x: (nfields, kmax, jmax, imax) dense."""
    cfg = solver.cfg
    xu, dy, dz = solver.geometry()
    T = np.ascontiguousarray(T, np.float32).reshape(-1, cfg.kmax, cfg.jmax, cfg.imax)
    keep = dict(T=T, xu=xu)
    c = PacketConfig()
    c.nw, c.na, c.nb, c.da, c.db = cfg.imax, cfg.jmax, cfg.kmax, dy, dz
    c.fw = _fp(xu)
    i0, i1, j0, j1, k0, k1 = solver._region
    c.ew0, c.ew1, c.ea0, c.ea1, c.eb0, c.eb1 = i0, i1, j0, j1, k0, k1
    nj = j1 - j0
    ta, tb = solver.packet_shape()
    c.tile_a, c.cpl = ta, ta * tb // 32
    c.nfields = T.shape[0]
    c.fieldT = _fp(T)
    if x is not None:
        X = np.ascontiguousarray(x, np.float32).reshape(T.shape)
        keep["X"] = X
        c.fieldX = _fp(X)
    c.kappa, c.T_west, c.T_east = cfg.kappa, cfg.T_west, cfg.T_east
    # multigrid: the oracle's own spline coarsening (interp3D restated) and
    # the reference's coarse faces, in the march's layout
    c.mg_levels, c.mg_steps = cfg.grid_num, cfg.mg_steps
    if cfg.grid_num > 1:
        ni_, nj_, nk_ = cfg.imax, cfg.jmax, cfg.kmax
        blocks, faces, off, foff = [], [], 0, 0
        for lv in range(1, cfg.grid_num):
            c.mg_off[lv] = off
            for f in range(T.shape[0]):
                Tf = np.zeros((nk_ + 2, nj_ + 2, ni_ + 2), np.float32)
                Tf[1:-1, 1:-1, 1:-1] = T[f]
                co = coarsen(Tf.ravel(), ni_, nj_, nk_, cfg.Lx, cfg.Ly, cfg.Lz, cfg.stretched_x, cfg.grid_num,
                             lv)[1:-1, 1:-1, 1:-1]
                blocks.append(np.ascontiguousarray(co.transpose(2, 0, 1)).ravel())
                off += co.size
            fw = ref_faces(ni_ >> lv, cfg.Lx, cfg.stretched_x, im0=ni_)
            c.mg_fwoff[lv] = foff
            faces.append(fw)
            foff += fw.size
            c.mg_da[lv] = np.float32(cfg.Ly) / np.float32(nj_ >> lv)
            c.mg_db[lv] = np.float32(cfg.Lz) / np.float32(nk_ >> lv)
        MT = np.concatenate(blocks).astype(np.float32)
        MF = np.concatenate(faces).astype(np.float32)
        keep["mgT"], keep["mgfw"] = MT, MF
        c.mgT, c.mgfw = _fp(MT), _fp(MF)
        c.Ly, c.Lz = cfg.Ly, cfg.Lz
    # general medium: particles (the solver's table, the caller's field) and grey walls
    part = getattr(solver, "_part", None)
    c.gen = 1 if (part is not None or cfg.eps_west < 1 or cfg.eps_east < 1) else 0
    c.eps[0], c.eps[1] = cfg.eps_west, cfg.eps_east
    if part is not None:
        if fv is None:
            raise ValueError("the solver has particles: pass their volume-fraction field")
        P = np.ascontiguousarray(part, np.float32)
        V = np.ascontiguousarray(fv, np.float32).reshape(T.shape)
        keep["part"], keep["fv"] = P, V
        c.part, c.fieldV = _fp(P), _fp(V)
        c.fv_max = float(V.max())
        c.hg_g = solver._hg
    c.seed, c.toll, c.max_steps, c.use_double = cfg.seed, cfg.toll, cfg.max_steps, use_double
    c.sampler, c.nbatch = cfg.sampler, cfg.nvar
    c.rays = solver_rays(solver)
    rp = None
    if getattr(solver, "_rays_dev", False):  # ray table written on the device (network allocation)
        rp = solver.rays_per_item()
    elif getattr(solver, "_keep", None):
        rp = solver._keep[0]
    if rp is not None:
        rp = np.ascontiguousarray(rp, np.int32)
        keep["rp"] = rp
        c.rays_per_packet = rp.ctypes.data_as(_i)
        if rp.ndim == 2:  # per (band group, packet)
            c.rays_gstride = rp.shape[1]
    if cfg.model == 3:
        c.mode = 0
        c.n_groups = 1
    else:
        tb = solver.table()
        s = solver.sampling()
        c.mode = 2 if tb["nX"] > 1 else 1
        c.nbands, c.nq, c.nT, c.nX = tb["nbands"], tb["nq"], tb["nT"], tb["nX"]
        c.T0, c.dT, c.X0, c.dX = tb["T0"], tb["dT"], tb["X0"], tb["dX"]
        k = np.ascontiguousarray(tb["k"], np.float32)
        Ib = np.ascontiguousarray(tb["Ib"], np.float32)
        keep.update(k=k, Ib=Ib, s=s)
        c.ktab, c.ibtab, c.ibw = _fp(k), _fp(Ib), _fp(s["ibw"])
        c.n_groups = s["n_groups"]
        c.n_tbins = s["n_tbins"] if s["n_tbins"] > 1 else 0
        c.group_start = s["group_start"].ctypes.data_as(_i)
        c.prob, c.W = _fp(s["prob"]), _fp(s["W"])
        c.alias = s["alias"].ctypes.data_as(_i)
        c.band = s["band"].ctypes.data_as(_i)
        c.gq = s["gq"].ctypes.data_as(_i)
    if cfg.control_variate:
        cvd = solver.cv_data()
        sk = np.ascontiguousarray(cvd["sur"][..., 0], np.float32)
        sI = np.ascontiguousarray(cvd["sur"][..., 1], np.float32)
        keep.update(sk=sk, sI=sI)
        c.cv = 1
        c.sur_k, c.sur_I = _fp(sk), _fp(sI)
        tab, _ = cv_table(c)
        keep["sur_tab"] = tab
        c.sur_tab = _fp(tab)
        bsrc = solver.cv_beta() if getattr(solver, "_beta_dev", False) else getattr(solver, "_beta", None)
        if bsrc is not None:
            b = np.ascontiguousarray(bsrc, np.float32)
            keep["beta"] = b
            c.beta = _fp(b)
    if mode is not None:
        c.mode = mode
    return c, keep


SUR_BINS = 64  # bins per hemisphere of the surrogate table (nodes uniform in sqrt|mu|)


def cv_table(c):
    """The control variate's surrogate table of the march (orc_cv_table: the
    untruncated straight flight at the nodes) for the layer-mean medium
    c.sur_k / c.sur_I of a PacketConfig: (table
    [f, sample, nw, 2, SUR_BINS, 4] float32 of (J0, dJ, A0, dA) per bin,
    means [f, sample, nw, 2] float64 of (Jhat, Ahat))."""
    ns = 1 if c.mode == 0 else c.nbands * c.nq
    tab = np.zeros((c.nfields, ns, c.nw, 2, SUR_BINS, 4), np.float32)
    JA = np.zeros((c.nfields, ns, c.nw, 2), np.float64)
    assert load().orc_cv_table(ctypes.byref(c), _fp(tab), JA.ctypes.data_as(_d)) == 0
    return tab, JA


def cv_quadrature():
    """Composite 16-point Gauss-Legendre in mu on [0,1e-3],[1e-3,1e-2],
    [1e-2,0.1],[0.1,1] (numpy's nodes, independent of the library's)."""
    x, w = np.polynomial.legendre.leggauss(16)
    mu, wt = [], []
    for a, b in ((0.0, 1e-3), (1e-3, 1e-2), (1e-2, 0.1), (0.1, 1.0)):
        mu.append(0.5 * (b - a) * x + 0.5 * (b + a))
        wt.append(0.5 * (b - a) * w)
    return np.concatenate(mu), np.concatenate(wt)


def cv_walk(sur_k, sur_I, fw, toll, Iw, l, mu):
    """The surrogate walk in float64: from the centre of layer l with
    wall-normal cosine mu (sign: direction, > 0 towards the east wall of
    intensity Iw[1]) through layers of constant (sur_k, sur_I), stopped once
    its optical depth exceeds ln(1/toll) (the rest stays in that layer; toll
    None: never) or at a black wall.  Returns (J, A): collected intensity and
    own-layer absorptance 1 - t0 (t0 = 0 if it stops inside layer l)."""
    nw = len(sur_k)
    dtoll = math.inf if toll is None else -math.log(toll)
    d = 1 if mu > 0 else -1
    m = abs(mu)
    o = 0.5 * (float(fw[l]) + float(fw[l + 1]))
    tau, J, i, t0, dcum = 1.0, 0.0, l, 0.0, 0.0
    seg = (float(fw[l + 1]) - o) if d > 0 else (o - float(fw[l]))
    while True:
        opt = float(sur_k[i]) * seg / m
        if dcum + opt > dtoll:  # optical depth beyond ln(1/toll): the rest stays in layer i
            J += tau * float(sur_I[i])
            break
        a = -math.expm1(-opt)
        J += tau * a * float(sur_I[i])
        tau -= tau * a
        dcum += opt
        if i == l:
            t0 = tau
        i += d
        if i < 0 or i >= nw:
            J += tau * float(Iw[1 if d > 0 else 0])
            break
        seg = float(fw[i + 1]) - float(fw[i])
    return J, 1.0 - t0


def cv_jhat(sur_k, sur_I, fw, toll, Iw_west, Iw_east):
    """For every layer l of a 1-D layered medium (k, Ib per layer; black walls
    with intensities Iw), the direction means of the surrogate walk (cv_walk;
    toll None: the untruncated straight flight) by quadrature
    (cv_quadrature), in float64:
    Jhat[l] = 1/2 int_{-1}^{1} J(mu; l) dmu (absorbed intensity) and
    Ahat[l] = 1/2 int_{-1}^{1} A(mu; l) dmu (own-layer absorptance).
    Returns an (nw, 2) array."""
    nw = len(sur_k)
    mu, wt = cv_quadrature()
    out = np.zeros((nw, 2))
    for l in range(nw):
        acc = accA = 0.0
        for sgn in (-1.0, 1.0):
            for m, wq in zip(mu, wt):
                J, A = cv_walk(sur_k, sur_I, fw, toll, (Iw_west, Iw_east), l, sgn * m)
                acc += wq * J
                accA += wq * A
        out[l] = 0.5 * acc, 0.5 * accA
    return out


def layer_surrogate(tb: dict, T: np.ndarray, x: np.ndarray | None):
    """The oracle's own layer-mean medium: per field and wall-normal layer
    the float64 plane means of T and x_H2O, and at them k of every spectral
    sample (bilinear in T, x) and the band intensity (linear in T), rounded
    to float32.  Returns sur_k, sur_I of shape (nfields, nbands * nq, nw)."""
    T = np.asarray(T, np.float64)
    nf, nw = T.shape[0], T.shape[3]
    Tb = T.mean(axis=(1, 2))                                   # (nf, nw)
    Xb = np.asarray(x, np.float64).mean(axis=(1, 2)) if x is not None else np.zeros_like(Tb)
    k = np.asarray(tb["k"], np.float64)                        # (nb, nq, nT, nX)
    nb, nq, nT, nX = k.shape
    p = np.clip((Tb - tb["T0"]) / tb["dT"], 0, nT - 1)
    ti = np.minimum(p.astype(int), nT - 2)
    ft = p - ti
    if nX > 1:
        px = np.clip((Xb - tb["X0"]) / tb["dX"], 0, nX - 1)
        xi = np.minimum(px.astype(int), nX - 2)
        fx = px - xi
    else:
        xi, fx = np.zeros_like(ti), np.zeros_like(Tb)
    kk = k.reshape(nb * nq, nT, nX)
    xj = np.minimum(xi + 1, nX - 1)
    k00, k01 = kk[:, ti, xi], kk[:, ti, xj]
    k10, k11 = kk[:, ti + 1, xi], kk[:, ti + 1, xj]
    k0 = k00 + fx * (k01 - k00)
    k1 = k10 + fx * (k11 - k10)
    sur_k = (k0 + ft * (k1 - k0)).transpose(1, 0, 2)         # (nf, S, nw)
    Ib = np.asarray(tb["Ib"], np.float64)                      # (nb, nT)
    Ibl = Ib[:, ti] + ft * (Ib[:, ti + 1] - Ib[:, ti])        # (nb, nf, nw)
    sur_I = np.repeat(Ibl, nq, axis=0).transpose(1, 0, 2)
    return np.ascontiguousarray(sur_k, np.float32), np.ascontiguousarray(sur_I, np.float32)


def fp64_cv_solution(mirror, dnu, wq, T: np.ndarray, x: np.ndarray | None, *, rays: int, nbatch: int = 8,
                     seed: int = 7, threads: int = 0, layer_step: int = 1):
    """An FP64 solution of Q over `mirror`'s region, independent of the GPU.

    `mirror` is a host-only Solver carrying the table, geometry, region,
    packet shape and host-built sampling tables (dnsmc_prepare_sampling),
    configured without a control variate (the oracle adds its own);
    dnu, wq: the table's band widths and g weights.
    The estimator is the packet scheme in float64 (Packet<double>) with the
    profile control variate built entirely here: the oracle's own layer-mean
    medium (layer_surrogate), its exact means E[Y] (orc_cv_mean: a float64
    quadrature over the wall-normal cosine with numpy's Gauss-Legendre
    nodes, cv_quadrature), beta = (1, -1); `rays` RQMC rays per cell and
    group in `nbatch` shifted replicates.  Raw tables only (C_s = 4 pi 100
    dnu w_g, the coefficient of dnsmc_set_table without reference CDFs).
    Returns (Q, var) of shape (nfields, nk, nj, ni) over the region, var the
    variance of Q from the replicate means.  layer_step > 1 solves only every
    layer_step-th wall-normal layer of the region (from its first); the other
    layers of the returned arrays are NaN."""
    T = np.ascontiguousarray(T, np.float32)
    c, keep = packet_config(mirror, T, x, use_double=1)
    tb = mirror.table()
    sur_k, sur_I = layer_surrogate(tb, T, x)
    keep.update(sur_k=sur_k, sur_I=sur_I)
    c.cv, c.sur_k, c.sur_I, c.beta = 1, _fp(sur_k), _fp(sur_I), None
    c.sampler, c.nbatch, c.rays, c.seed = 1, nbatch, rays, seed
    c.rays_per_packet, c.rays_gstride = None, 0
    c.pw_step = layer_step
    nG = c.n_groups
    i0, i1, j0, j1, k0, k1 = mirror._region
    ni, nj, nk = i1 - i0, j1 - j0, k1 - k0
    rc = ni * nj * nk
    tal, _ = packet_mc(c, nG, rc, threads)
    # C_s and the band groups of the host's sampling construction
    nb, nq = tb["nbands"], tb["nq"]
    dnu = np.asarray(dnu, np.float32).astype(np.float64)
    wq = np.asarray(wq, np.float32).astype(np.float64)
    sid, C, gs = [], [], [0]
    for G in range(nG):
        for b in range(G * nb // nG, (G + 1) * nb // nG):
            for g in range(nq):
                sid.append(b * nq + g)
                C.append(4.0 * math.pi * 100.0 * dnu[b] * wq[g])
        gs.append(len(sid))
    sid = np.asarray(sid, np.int32)
    C = np.asarray(C, np.float64)
    gs = np.asarray(gs, np.int32)
    mu, w = cv_quadrature()
    muY = np.zeros((T.shape[0], nG, rc, 2), np.float64)
    assert load().orc_cv_mean(ctypes.byref(c), gs.ctypes.data_as(_i), sid.ctypes.data_as(_i),
                              C.ctypes.data_as(_d), mu.ctypes.data_as(_d), w.ctypes.data_as(_d), len(mu), threads,
                              muY.ctypes.data_as(_d)) == 0
    m = tal[..., 0] / rays                                     # (nf, G, rc): mean of X - Y_a + Y_b
    vg = np.maximum(0.0, tal[..., 1] / nbatch - m * m) / (nbatch - 1)
    Qg = m + muY[..., 0] - muY[..., 1]
    shape = (T.shape[0], ni, nk, nj)                           # tally order: i, k, j
    Q = Qg.sum(1).reshape(shape).transpose(0, 2, 3, 1)
    V = vg.sum(1).reshape(shape).transpose(0, 2, 3, 1)
    if layer_step > 1:
        skip = np.ones(ni, bool)
        skip[::layer_step] = False
        Q[..., skip] = np.nan
        V[..., skip] = np.nan
    return np.ascontiguousarray(Q), np.ascontiguousarray(V)


def ref_tables_x_slice(table: dict, xbar: float) -> dict:
    """The reference-format tables (ref_mc, model 0) of a k(band, g, T, x)
    table at one x_H2O: the reference has no x axis.  k(band, T, g) at xbar
    (linear in x), band Planck intensities at the band centres, the band and
    g CDFs of the emission k Ib dnu w_g at every table temperature, and the
    Planck mean kP = pi sum(k Ib dnu w_g) / (sigma T^4), float32."""
    k = np.asarray(table["k"], np.float64)
    X = table["X0"] + table["dX"] * np.arange(k.shape[3])
    kx = np.empty(k.shape[:3], np.float64)
    for b in range(kx.shape[0]):
        for g in range(kx.shape[1]):
            kx[b, g] = [np.interp(xbar, X, k[b, g, t]) for t in range(kx.shape[2])]
    nT = kx.shape[2]
    Tnb = (table["T0"] + table["dT"] * np.arange(nT)).astype(np.float32)
    C1, C2 = 3.741771790075259e-16, 0.014387741858429
    nu = np.asarray(table["wvc"], np.float64)
    Ib = C1 * (nu[None, :] * 100) ** 3 / (np.pi * (np.exp(C2 * nu[None, :] * 100 / Tnb[:, None]) - 1))  # [nT][nB]
    e = kx.transpose(2, 0, 1) * Ib[:, :, None] * np.asarray(table["dnu"])[None, :, None] * 100 \
        * np.asarray(table["wq"])[None, None, :]
    eb = e.sum(2)
    prob = np.cumsum(eb, 1) / eb.sum(1, keepdims=True)
    probg = np.cumsum(e, 2) / np.maximum(e.sum(2, keepdims=True), 1e-300)
    kP = np.pi * eb.sum(1) / (SIGMA * Tnb.astype(np.float64) ** 4)
    return dict(Tnb=Tnb, kq=kx.transpose(0, 2, 1).astype(np.float32), wvc=np.asarray(table["wvc"], np.float32),
                prob=prob.astype(np.float32), probg=probg.astype(np.float32), kP=kP.astype(np.float32))


def ck_from_lbl(spec: dict, gq, n_pwrk: int = 10000, threads: int = 0):
    """The oracle's k-distribution (orc_ck_from_lbl) of a synth.lbl_spectrum
    dict: kq [nbands][nq][nT][nX] float32 and kavg [nT][nX][nbands]."""
    k = np.ascontiguousarray(spec["kappa"], np.float64)
    nT, nX, npts = k.shape
    ns = nT * nX
    nb = len(spec["first"])
    gq = np.ascontiguousarray(gq, np.float64)
    first = np.ascontiguousarray(spec["first"], np.int64)
    count = np.ascontiguousarray(spec["count"], np.int32)
    wl = np.ascontiguousarray(spec["wv_left"], np.float64)
    wr = np.ascontiguousarray(spec["wv_right"], np.float64)
    kq = np.zeros((nb, gq.size, ns), np.float32)
    kavg = np.zeros((ns, nb))
    rc = load().orc_ck_from_lbl(k.ctypes.data_as(_d), ns, npts, float(spec["dwv"]), nb,
                                first.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), count.ctypes.data_as(_i),
                                wl.ctypes.data_as(_d), wr.ctypes.data_as(_d), gq.size, gq.ctypes.data_as(_d),
                                n_pwrk, threads, kq.ctypes.data_as(_f), kavg.ctypes.data_as(_d))
    assert rc == 0
    return kq.reshape(nb, gq.size, nT, nX), kavg.reshape(nT, nX, nb)


def ref_ckgen_available() -> bool:
    return os.path.exists(_build.ref_lib_path("ckgen"))


def ref_correlated_kt(spec: dict, workdir: str):
    """The reference's own correlatedKT (distr/correlatedK.cpp:145-300, built
    from the reference sources into oracle/_ref) on the spectra of the first
    mole fraction: its compile-time sizes (nT spectra, nQuad g-points,
    n_pwrk bins) and gq.  Returns (kq [nT][nbands][nQuad], gq, n_pwrk)."""
    lib = ctypes.CDLL(_build.ref_lib_path("ckgen"))
    nt, nq, npw = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib.ref_ck_sizes(ctypes.byref(nt), ctypes.byref(nq), ctypes.byref(npw))
    gq = np.zeros(nq.value)
    lib.ref_ck_gq(gq.ctypes.data_as(_d))
    k = np.ascontiguousarray(spec["kappa"][:, 0, :], np.float64)
    if k.shape[0] != nt.value:
        raise ValueError(f"the reference routine takes {nt.value} temperatures")
    npts = k.shape[1]
    wvn = spec["wv0"] + spec["dwv"] * np.arange(npts)
    nb = len(spec["first"])
    first = np.ascontiguousarray(spec["first"], np.int64)
    count = np.ascontiguousarray(spec["count"], np.int32)
    wl = np.ascontiguousarray(spec["wv_left"], np.float64)
    wr = np.ascontiguousarray(spec["wv_right"], np.float64)
    kq = np.zeros((nt.value, nb, nq.value))
    _ll = ctypes.POINTER(ctypes.c_longlong)
    lib.ref_ck_correlatedKT.argtypes = [_d, ctypes.c_longlong, _d, ctypes.c_int, _ll, _i, _d, _d, ctypes.c_char_p,
                                        _d]
    rc = lib.ref_ck_correlatedKT(k.ctypes.data_as(_d), npts, wvn.ctypes.data_as(_d), nb, first.ctypes.data_as(_ll),
                                 count.ctypes.data_as(_i), wl.ctypes.data_as(_d), wr.ctypes.data_as(_d),
                                 os.fsencode(workdir), kq.ctypes.data_as(_d))
    assert rc == 0, rc
    return kq, gq, npw.value


def solver_rays(solver) -> int:
    return int(getattr(solver, "_rays", solver.cfg.nvar * solver.cfg.photmax))


def packet_mc(c: PacketConfig, n_groups: int, region_cells: int, threads: int = 0):
    """Tally (nfields, n_groups, region_cells, 2) in the device's order."""
    t = np.zeros((c.nfields, n_groups, region_cells, 2), np.float64)
    steps = ctypes.c_double()
    rc = load().orc_packet_mc(ctypes.byref(c), threads, t.ctypes.data_as(_d), ctypes.byref(steps))
    assert rc == 0
    return t, steps.value


def packet_trace(c: PacketConfig, f: int, g: int, p: int, r: int, max_steps: int = 4096):
    rec = np.zeros((max_steps, 6), np.int32)
    n = ctypes.c_int()
    rng = np.zeros(4, np.uint32)
    load().orc_packet_trace(ctypes.byref(c), f, g, p, r, max_steps, rec.ctypes.data_as(_i32), ctypes.byref(n),
                            rng.ctypes.data_as(_u32))
    return rec[: min(n.value, max_steps)], n.value, rng


# ---------------------------------------------------------------------------
# analytic references
# ---------------------------------------------------------------------------
def expn(n: int, x: float) -> float:
    """Exponential integral E_n(x) = int_1^inf exp(-x t) / t^n dt, x > 0
    (continued fraction for x > 1, power series otherwise)."""
    if x <= 0:
        return math.inf if n <= 1 else 1.0 / (n - 1)
    euler = 0.5772156649015329
    if x > 1.0:
        b = x + n
        c = 1e300
        d = 1.0 / b
        h = d
        for i in range(1, 500):
            a = -i * (n - 1 + i)
            b += 2.0
            d = 1.0 / (a * d + b)
            c = b + a / c
            de = c * d
            h *= de
            if abs(de - 1.0) < 1e-15:
                break
        return h * math.exp(-x)
    ans = (1.0 / (n - 1)) if n != 1 else (-math.log(x) - euler)
    fact = 1.0
    for i in range(1, 500):
        fact *= -x / i
        if i != n - 1:
            de = -fact / (i - n + 1)
        else:
            psi = -euler + sum(1.0 / k for k in range(1, n))
            de = fact * (-math.log(x) + psi)
        ans += de
        if abs(de) < abs(ans) * 1e-16:
            break
    return ans


def slab_divq(y: np.ndarray, L: float, kappa: float, T: float, Tw1: float, Tw2: float) -> np.ndarray:
    """Exact div q [W/m^3] at wall distances y (from wall 1) of an isothermal
    grey slab of thickness L between black walls at Tw1, Tw2."""
    tau = kappa * np.asarray(y, np.float64)
    tl = kappa * L
    e1 = np.array([expn(2, t) for t in tau])
    e2 = np.array([expn(2, tl - t) for t in tau])
    return 2.0 * kappa * SIGMA * ((T ** 4 - Tw1 ** 4) * e1 + (T ** 4 - Tw2 ** 4) * e2)


def thin_limit(T: np.ndarray, Tw: float, Tnb: np.ndarray, kP: np.ndarray) -> np.ndarray:
    """Optically thin limit 4 sigma (kP(T) T^4 - kP(Tw) Tw^4)."""
    k = np.interp(T, Tnb, kP)
    kw = np.interp(Tw, Tnb, kP)
    return 4.0 * SIGMA * (k * T ** 4 - kw * Tw ** 4)


# ---------------------------------------------------------------------------
# the reference's own table reader (oracle/_ref), where it was built
# ---------------------------------------------------------------------------
def ref_tables_available(kind: str) -> bool:
    return os.path.exists(_build.ref_lib_path(kind))


def ref_readT(kind: str, table_root: str, Tmax: float) -> dict:
    """Call the reference's readT (compiled from code/read_tables.cpp); it
    opens ../distr/tables/... relative to the working directory, so this
    switches to <table_root>/code for the call."""
    lib = ctypes.CDLL(_build.ref_lib_path(kind))
    nt, nb, nq = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib.ref_table_sizes(ctypes.byref(nt), ctypes.byref(nb), ctypes.byref(nq))
    nT, nB, nQ = nt.value, nb.value, nq.value
    out = dict(Tnb=np.zeros(nT, np.float32), kP=np.zeros(nT, np.float32), wvc=np.zeros(nB, np.float32),
               kavg=np.zeros(nB, np.float32), kq=np.zeros((nB, nT, nQ), np.float32),
               prob=np.zeros((nT, nB), np.float32), probg=np.zeros((nT, nB, nQ), np.float32))
    km = ctypes.c_float()
    lib.ref_readT.argtypes = [ctypes.c_float] + [_f] * 7 + [_f]
    cwd = os.getcwd()
    os.chdir(os.path.join(table_root, "code"))
    try:
        lib.ref_readT(Tmax, *[_fp(out[k]) for k in ("Tnb", "kP", "wvc", "kavg", "kq", "prob", "probg")],
                      ctypes.byref(km))
    finally:
        os.chdir(cwd)
    out["kappamax"] = km.value
    return out


# ---------------------------------------------------------------------------
# 1-D references of the general medium
# ---------------------------------------------------------------------------
def slab_grey_walls_divq(y, L: float, kappa: float, T: float, T_wall: float, eps: float) -> np.ndarray:
    """div q of an isothermal grey non-scattering slab between two diffuse grey
    walls of emissivity eps at T_wall (both sides), at positions y:
    wall radiosity J = (eps s Tw^4 + (1-eps) pi Ib (1 - 2 E3(tL))) / (1 - 2 (1-eps) E3(tL)),
    Q = 2 pi kappa (Ib - J/pi)(E2(tau) + E2(tL - tau)), Ib = s T^4 / pi."""
    Ib = SIGMA * T ** 4 / math.pi
    tL = kappa * L
    E3 = expn(3, tL)
    J = (eps * SIGMA * T_wall ** 4 + (1 - eps) * math.pi * Ib * (1 - 2 * E3)) / (1 - 2 * (1 - eps) * E3)
    tau = kappa * np.asarray(y, np.float64)
    e2 = np.array([expn(2, t) + expn(2, tL - t) for t in tau])
    return 2 * math.pi * kappa * (Ib - J / math.pi) * e2


def slab_scatter_divq(faces, kappa_a: float, sigma_s: float, T: float, Tw0: float, Tw1: float,
                      refine: int = 8) -> np.ndarray:
    """Cell means of div q = kappa_a (4 pi Ib - G) in an isothermal, isotropically
    scattering slab with black walls (cells between `faces`): the integral
    equation for the source function S = (1 - w) Ib + w G / (4 pi),
    G(t) = 2 pi [Iw0 E2(t) + Iw1 E2(tL - t) + int_0^tL S(t') E1(|t - t'|) dt'],
    solved by Nystrom with piecewise-constant S on `refine` sub-cells per cell
    (exact E1 integrals over each sub-cell via E2)."""
    faces = np.asarray(faces, np.float64)
    beta = kappa_a + sigma_s
    w = sigma_s / beta
    fine = np.concatenate([np.linspace(faces[i], faces[i + 1], refine + 1)[:-1] for i in range(len(faces) - 1)]
                          + [faces[-1:]])
    tf = beta * (fine - fine[0])
    tL = tf[-1]
    tc = 0.5 * (tf[1:] + tf[:-1])
    a, b = tf[:-1], tf[1:]
    E2 = np.vectorize(lambda x: expn(2, x))
    M = len(tc)
    K = np.empty((M, M))
    for i in range(M):
        da = np.abs(tc[i] - a)
        db = np.abs(tc[i] - b)
        K[i] = np.abs(E2(da) - E2(db))
        K[i, i] = 2.0 - expn(2, tc[i] - a[i]) - expn(2, b[i] - tc[i])
    Ib = SIGMA * T ** 4 / math.pi
    Iw0, Iw1 = SIGMA * Tw0 ** 4 / math.pi, SIGMA * Tw1 ** 4 / math.pi
    wall = Iw0 * E2(tc) + Iw1 * E2(tL - tc)
    S = np.linalg.solve(np.eye(M) - 0.5 * w * K, (1 - w) * Ib + 0.5 * w * wall)
    G = 2 * math.pi * (wall + K @ S)
    Q = kappa_a * (4 * math.pi * Ib - G)
    return Q.reshape(-1, refine).mean(1)
