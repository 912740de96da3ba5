"""Python host mirror of the solver's C ABI.

Two surfaces, as in include/dnsmc.h:

* ``mc_gpu(T, ystart)`` / ``get_results(Qr, Vr)`` -- the reference's
  Fortran-facing pair (code/mc_gpu.cu:440, :640) with the same array layouts:
  T is real(4) TMC(0:imax+1,0:jmax+1,0:kmax+1) in Fortran order (numpy
  shape (kmax+2, jmax+2, imax+2), i fastest) and the outputs are
  (kmax+2, jmax/p_row+2, imax+2); only interior cells are written.
* ``Solver`` -- the handle-based API (tables, resident snapshots, band groups,
  adaptive rays, error codes, status, counters).

Arrays are numpy; the C library owns all device memory.  There is no
CPU fallback: every call goes through libdnsmc.so.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import Config, TableDesc, check


def _fp(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(_lib.c_float_p)


def _dp(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(_lib.c_double_p)


def default_config(**overrides) -> Config:
    """The reference's shipped code/param.h values, with keyword overrides."""
    lib = _lib.load()
    c = Config()
    lib.dnsmc_set_default_config(ctypes.byref(c))
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise KeyError(f"unknown config field {k!r}")
        setattr(c, k, v)
    return c


@dataclass
class Counters:
    rays: float
    steps: float
    march_ms: float


class Solver:
    """One solver instance (its own CUDA stream, tables, fields and buffers)."""

    def __init__(self, config: Config | None = None, **overrides):
        self._lib = _lib.load()
        cfg = config if config is not None else default_config()
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        h = ctypes.c_void_p()
        check(self._lib.dnsmc_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._region = (0, cfg.imax, 0, cfg.jmax, 0, cfg.kmax)
        self._nfields = 0
        self._keep = []
        self._rays = cfg.nvar * cfg.photmax
        self._rays_dev = False
        self._beta = None
        self._part = None
        self._hg = 0.0

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dnsmc_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- tables -------------------------------------------------------------
    def load_reference_tables(self, directory: str, model: int, nT: int = 52, nB: int = 119,
                              nQ: int | None = None) -> None:
        if nQ is None:
            nQ = 16 if model == _lib.MODEL_CK else 1
        check(self._lib.dnsmc_load_tables_ref(self._h, directory.encode(), model, nT, nB, nQ))

    def use_grey_band_tables(self, nB: int = 1000, nT: int = 55, wvmax: float = 15000.0,
                             Tmin: float = 500.0) -> None:
        check(self._lib.dnsmc_use_grey_band_tables(self._h, nB, nT, wvmax, Tmin))

    def set_table(self, k, wvc, T0, dT, dnu=None, wq=None, X0=0.0, dX=1.0, Ib=None,
                  prob=None, probg=None, kP=None) -> None:
        """k: array [nbands, nq, nT, nX] (or [nbands, nq, nT]) in 1/m."""
        k = np.ascontiguousarray(k, dtype=np.float32)
        if k.ndim == 3:
            k = k[..., None]
        nb, nq, nT, nX = k.shape
        arrs = dict(k=k, wvc=wvc, dnu=dnu, wq=wq, Ib=Ib, prob=prob, probg=probg, kP=kP)
        conv = {n: (None if a is None else np.ascontiguousarray(a, dtype=np.float32)) for n, a in arrs.items()}
        d = TableDesc()
        d.nbands, d.nq, d.nT, d.nX = nb, nq, nT, nX
        d.T0, d.dT, d.X0, d.dX = T0, dT, X0, dX
        for n, a in conv.items():
            setattr(d, n, _fp(a))
        check(self._lib.dnsmc_set_table(self._h, ctypes.byref(d)))

    def save_table(self, path: str) -> None:
        """Write the current table to a binary table file (dnsmc_save_table)."""
        check(self._lib.dnsmc_save_table(self._h, os.fsencode(path)))

    def load_table(self, path: str) -> None:
        """Set the table from a binary table file (dnsmc_load_table)."""
        check(self._lib.dnsmc_load_table(self._h, os.fsencode(path)))

    def table_info(self) -> dict:
        vals = [ctypes.c_int() for _ in range(4)] + [ctypes.c_float() for _ in range(4)]
        check(self._lib.dnsmc_get_table_info(self._h, *[ctypes.byref(v) for v in vals]))
        keys = ["nbands", "nq", "nT", "nX", "T0", "dT", "X0", "dX"]
        return {k: v.value for k, v in zip(keys, vals)}

    def table(self) -> dict:
        i = self.table_info()
        nb, nq, nT, nX = i["nbands"], i["nq"], i["nT"], i["nX"]
        k = np.zeros((nb, nq, nT, nX), np.float32)
        wvc = np.zeros(nb, np.float32)
        Ib = np.zeros((nb, nT), np.float32)
        prob = np.zeros((nT, nb), np.float32)
        probg = np.zeros((nT, nb, nq), np.float32)
        kP = np.zeros(nT, np.float32)
        check(self._lib.dnsmc_get_table(self._h, _fp(k), _fp(wvc), _fp(Ib), _fp(prob), _fp(probg), _fp(kP)))
        return dict(k=k, wvc=wvc, Ib=Ib, prob=prob, probg=probg, kP=kP, **i)

    # -- fields -------------------------------------------------------------
    def set_fields(self, T, x=None, layout: int = _lib.LAYOUT_DENSE) -> None:
        """T: (nfields, kmax, jmax, imax) or (kmax, jmax, imax) float32, i fastest
        (Fortran order); FORTRAN layout adds the ghost layer on every axis."""
        T = np.ascontiguousarray(T, dtype=np.float32)
        c = self.cfg
        per = (c.kmax, c.jmax, c.imax) if layout == _lib.LAYOUT_DENSE else (c.kmax + 2, c.jmax + 2, c.imax + 2)
        if T.shape == per:
            T = T[None]
        if T.shape[1:] != per:
            raise ValueError(f"field shape {T.shape} does not match {per}")
        X = None
        if x is not None:
            X = np.ascontiguousarray(x, dtype=np.float32).reshape(T.shape)
        check(self._lib.dnsmc_set_fields(self._h, T.shape[0], _fp(T), _fp(X), layout))
        self._nfields = T.shape[0]

    def set_particles(self, absorption, scattering, hg_g: float = 0.0) -> None:
        """Per-band absorption / scattering per unit volume fraction [1/m]
        (None, None removes the particles)."""
        if absorption is None and scattering is None:
            check(self._lib.dnsmc_set_particles(self._h, 0, None, None, 0.0))
            self._part = None
            return
        a = np.ascontiguousarray(absorption, np.float32)
        sc = np.ascontiguousarray(scattering, np.float32)
        check(self._lib.dnsmc_set_particles(self._h, a.size, _fp(a), _fp(sc), float(hg_g)))
        self._part = np.stack([a, sc], 1)
        self._hg = float(hg_g)

    def set_particle_field(self, fv, layout: int = _lib.LAYOUT_DENSE) -> None:
        v = np.ascontiguousarray(fv, dtype=np.float32)
        check(self._lib.dnsmc_set_particle_field(self._h, _fp(v), layout))

    def set_region(self, i0, i1, j0, j1, k0, k1) -> None:
        check(self._lib.dnsmc_set_region(self._h, i0, i1, j0, j1, k0, k1))
        self._region = (i0, i1, j0, j1, k0, k1)
        self._keep = []
        self._rays_dev = False

    def packet_shape(self) -> tuple[int, int]:
        """(tile_a, tile_b): cells of a packet along j and along k (64-cell
        packets on the fine grid, 32 with grid_num > 1)."""
        a, b = ctypes.c_int(), ctypes.c_int()
        check(self._lib.dnsmc_packet_shape(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def packet_count(self) -> int:
        n = ctypes.c_int()
        check(self._lib.dnsmc_packet_count(self._h, ctypes.byref(n)))
        return n.value

    def set_rays(self, rays_per_group: int, rays_per_packet=None) -> None:
        rp = None
        if rays_per_packet is not None:
            rp = np.ascontiguousarray(rays_per_packet, dtype=np.int32)
            if rp.size != self.packet_count():
                raise ValueError("rays_per_packet needs one entry per packet")
            self._keep = [rp]
        else:
            self._keep = []
        check(self._lib.dnsmc_set_rays(self._h, int(rays_per_group),
                                       None if rp is None else rp.ctypes.data_as(_lib.c_int_p)))
        self._rays = int(rays_per_group)
        self._rays_dev = False

    def set_rays_per_item(self, rays) -> None:
        """Ray counts per (band group, packet): int array (n_groups, npackets)."""
        rp = np.ascontiguousarray(rays, dtype=np.int32)
        if rp.ndim != 2 or rp.shape[1] != self.packet_count():
            raise ValueError("rays needs shape (n_groups, npackets)")
        check(self._lib.dnsmc_set_rays_per_item(self._h, rp.shape[0], rp.ctypes.data_as(_lib.c_int_p)))
        self._keep = [rp]
        self._rays_dev = False

    def stream(self) -> int:
        """The solver's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        h = ctypes.c_void_p()
        check(self._lib.dnsmc_get_stream(self._h, ctypes.byref(h)))
        return int(h.value or 0)

    def cv_beta(self):
        """Coefficients in effect: (nfields, n_groups, nk, nj, ni, 2) float32."""
        ng = self.sampling()["n_groups"] if self.cfg.model != _lib.MODEL_GREY else 1
        shp = self._region_shape()
        out = np.zeros((shp[0], ng) + shp[1:] + (2,), np.float32)
        check(self._lib.dnsmc_get_cv_beta(self._h, _fp(out)))
        return out

    def rays_per_item(self):
        """The ray table in effect: (n_groups, npackets) per (group, packet)
        (set here or by a network), (npackets,) per packet (adaptive or
        per-packet rays), or None for uniform rays."""
        ng = ctypes.c_int()
        check(self._lib.dnsmc_get_rays_per_item(self._h, ctypes.byref(ng), None))
        if ng.value == 0:
            return None
        shape = (ng.value, self.packet_count()) if ng.value > 0 else (self.packet_count(),)
        out = np.zeros(shape, np.int32)
        check(self._lib.dnsmc_get_rays_per_item(self._h, ctypes.byref(ng), out.ctypes.data_as(_lib.c_int_p)))
        return out

    def set_rays_adaptive(self, rays_per_tau: float, min_rays: int = 64, max_rays: int = 4096) -> None:
        """Rays per packet ~ local optical thickness (device-computed)."""
        check(self._lib.dnsmc_set_rays_adaptive(self._h, float(rays_per_tau), int(min_rays), int(max_rays)))
        self._keep = []
        self._rays_dev = True

    def coarse_field(self, field: int, level: int):
        """Spline-coarsened T of a multigrid level, (nk, nj, ni) >> level."""
        c = self.cfg
        out = np.zeros((c.kmax >> level, c.jmax >> level, c.imax >> level), np.float32)
        check(self._lib.dnsmc_get_coarse_field(self._h, field, level, _fp(out)))
        return out

    def set_graph(self, enable: bool = True) -> None:
        check(self._lib.dnsmc_set_graph(self._h, 1 if enable else 0))

    def graph_info(self):
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        check(self._lib.dnsmc_get_graph_info(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def item_steps(self):
        """Ray-voxel steps of the last solve per (field, group, packet), summed over rays."""
        ng = self.sampling()["n_groups"]
        out = np.zeros((self._nfields, ng, self.packet_count()), np.float64)
        check(self._lib.dnsmc_get_item_steps(self._h, _dp(out)))
        return out

    # -- solve --------------------------------------------------------------
    def solve_async(self) -> None:
        check(self._lib.dnsmc_solve_async(self._h))

    def wait(self, timeout_s: float = 0.0) -> None:
        check(self._lib.dnsmc_wait(self._h, timeout_s))

    def _region_shape(self):
        i0, i1, j0, j1, k0, k1 = self._region
        return (self._nfields, k1 - k0, j1 - j0, i1 - i0)

    def results(self, out=None):
        """(Q, sigma): float64 arrays (nfields, nk, nj, ni) over the region,
        written into `out` = (Q, sigma) when given (C-contiguous float64 arrays
        of that shape, e.g. the caller's persistent result arrays)."""
        shp = self._region_shape()
        if out is None:
            Q = np.zeros(shp, np.float64)
            S = np.zeros(shp, np.float64)
        else:
            Q, S = out
            for a in (Q, S):
                if a.shape != shp or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"result arrays must be C-contiguous float64 of shape {shp}")
        check(self._lib.dnsmc_get_results(self._h, _dp(Q), _dp(S)))
        return Q, S

    def set_result_type(self, result_type: int) -> None:
        """RESULT_F64 (default) or RESULT_F32: with F32 the device rounds Q and
        sigma to float and only those cross to the host; read them with
        results_float()."""
        check(self._lib.dnsmc_set_result_type(self._h, int(result_type)))
        self._result_type = int(result_type)

    def results_float(self, out=None):
        """(Q, sigma) as float32 arrays (nfields, nk, nj, ni), into `out` when
        given (C-contiguous float32 arrays of that shape)."""
        shp = self._region_shape()
        if out is None:
            Q = np.zeros(shp, np.float32)
            S = np.zeros(shp, np.float32)
        else:
            Q, S = out
            for a in (Q, S):
                if a.shape != shp or a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"result arrays must be C-contiguous float32 of shape {shp}")
        check(self._lib.dnsmc_get_results_float(self._h, Q.ctypes.data_as(_lib.c_float_p),
                                                S.ctypes.data_as(_lib.c_float_p)))
        return Q, S

    def solve(self, timeout_s: float = 0.0):
        self.solve_async()
        self.wait(timeout_s)
        if getattr(self, "_result_type", 0) == _lib.RESULT_F32:
            return self.results_float()
        return self.results()

    def group_results(self):
        """(Qg, varg): (nfields, n_groups, nk, nj, ni) group means and variances."""
        ng = self.sampling()["n_groups"]
        shp = self._region_shape()
        shp = (shp[0], ng) + shp[1:]
        Q = np.zeros(shp, np.float64)
        V = np.zeros(shp, np.float64)
        check(self._lib.dnsmc_get_group_results(self._h, _dp(Q), _dp(V)))
        return Q, V

    def status(self) -> int:
        s = ctypes.c_uint32()
        check(self._lib.dnsmc_status(self._h, ctypes.byref(s)))
        return s.value

    def counters(self) -> Counters:
        r, s, m = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(self._lib.dnsmc_get_counters(self._h, ctypes.byref(r), ctypes.byref(s), ctypes.byref(m)))
        return Counters(r.value, s.value, m.value)

    def timing(self):
        """(solve_ms, march_ms) of the last solve, CUDA events on its stream."""
        a, b = ctypes.c_double(), ctypes.c_double()
        check(self._lib.dnsmc_get_timing(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def tmax(self) -> float:
        t = ctypes.c_float()
        check(self._lib.dnsmc_get_tmax(self._h, ctypes.byref(t)))
        return t.value

    def sampling(self) -> dict:
        ng, nt, ne = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.dnsmc_get_sampling(self._h, ctypes.byref(ng), ctypes.byref(nt), None, ctypes.byref(ne),
                                           None, None, None, None, None, None))
        n, t, e = ng.value, nt.value, ne.value
        gs = np.zeros(n * t + 1, np.int32)
        prob = np.zeros(max(e, 1), np.float32)
        alias = np.zeros(max(e, 1), np.int32)
        band = np.zeros(max(e, 1), np.int32)
        gq = np.zeros(max(e, 1), np.int32)
        W = np.zeros(max(e, 1), np.float32)
        nb = max(self.table_info()["nbands"], 1)
        ibw = np.zeros(2 * nb, np.float32)
        ip = lambda a: a.ctypes.data_as(_lib.c_int_p)
        check(self._lib.dnsmc_get_sampling(self._h, None, None, ip(gs), None, _fp(prob), ip(alias), ip(band), ip(gq),
                                           _fp(W), _fp(ibw)))
        return dict(n_groups=n, n_tbins=t, group_start=gs, prob=prob[:e], alias=alias[:e], band=band[:e], gq=gq[:e],
                    W=W[:e], ibw=ibw)

    def prepare_sampling(self, Tmax: float, xmean: float = 0.0) -> dict:
        """Build the sampling tables on the host for Tmax (no GPU needed)."""
        check(self._lib.dnsmc_prepare_sampling(self._h, float(Tmax), float(xmean)))
        return self.sampling()

    def set_cv_beta(self, beta) -> None:
        """Control-variate coefficient pairs (nfields, n_groups, nk, nj, ni, 2)
        = (beta_a, beta_b), or None for (1, -1)."""
        self._beta_dev = False
        if beta is None:
            check(self._lib.dnsmc_set_cv_beta(self._h, None))
            self._beta = None
            return
        b = np.ascontiguousarray(beta, dtype=np.float32)
        check(self._lib.dnsmc_set_cv_beta(self._h, _fp(b)))
        self._beta = b

    def cv_data(self) -> dict:
        """Layer means, surrogate table, Jhat and E[Y] of the last CV solve."""
        ns = ctypes.c_int()
        check(self._lib.dnsmc_get_cv_data(self._h, ctypes.byref(ns), None, None, None, None))
        c = self.cfg
        S = ns.value
        nf = self._nfields
        ng = self.sampling()["n_groups"] if c.model != _lib.MODEL_GREY else 1
        layer = np.zeros((nf, c.imax, 2), np.float32)
        sur = np.zeros((nf, S, c.imax, 2), np.float32)
        Jhat = np.zeros((nf, S, c.imax, 2), np.float64)
        shp = self._region_shape()
        muY = np.zeros((nf, ng) + shp[1:] + (2,), np.float64)
        check(self._lib.dnsmc_get_cv_data(self._h, None, _fp(layer), _fp(sur), _dp(Jhat), _dp(muY)))
        return dict(layer=layer, sur=sur, Jhat=Jhat, muY=muY, n_samples=S)

    def cv_table(self) -> np.ndarray:
        """The tabulated surrogate of the last CV solve, (nfields, samples,
        imax, 2, CV_BINS, 4) float32: per plane, hemisphere (west, east) and
        bin of sqrt|mu| the (J0, dJ, A0, dA) the march interpolates."""
        ns = ctypes.c_int()
        check(self._lib.dnsmc_get_cv_data(self._h, ctypes.byref(ns), None, None, None, None))
        tab = np.zeros((self._nfields, ns.value, self.cfg.imax, 2, _lib.CV_BINS, 4), np.float32)
        check(self._lib.dnsmc_get_cv_table(self._h, _fp(tab)))
        return tab

    def cv_moments(self):
        """(nfields, n_groups, nk, nj, ni, 9) per-ray moment sums of the last
        solve with cv_moments=1: X, Ya, Yb, X^2, Ya^2, Yb^2, X Ya, X Yb, Ya Yb."""
        ng = self.sampling()["n_groups"] if self.cfg.model != _lib.MODEL_GREY else 1
        shp = self._region_shape()
        m = np.zeros((shp[0], ng) + shp[1:] + (9,), np.float64)
        check(self._lib.dnsmc_get_cv_moments(self._h, _dp(m)))
        return m

    def geometry(self):
        xu = np.zeros(self.cfg.imax + 1, np.float32)
        dy, dz = ctypes.c_float(), ctypes.c_float()
        check(self._lib.dnsmc_get_geometry(self._h, _fp(xu), ctypes.byref(dy), ctypes.byref(dz)))
        return xu, dy.value, dz.value

    def trace(self, f: int, g: int, p: int, r: int, max_steps: int = 4096):
        rec = np.zeros((max_steps, 6), np.int32)
        n = ctypes.c_int()
        rng = np.zeros(4, np.uint32)
        check(self._lib.dnsmc_trace_ray(self._h, f, g, p, r, max_steps, rec.ctypes.data_as(_lib.c_int32_p),
                                        ctypes.byref(n), rng.ctypes.data_as(_lib.c_uint32_p)))
        return rec[: min(n.value, max_steps)], n.value, rng


# -- reference drop-in pair -----------------------------------------------------
def dropin_configure(config: Config | None = None, table_dir: str | None = None) -> None:
    lib = _lib.load()
    check(lib.dnsmc_dropin_configure(None if config is None else ctypes.byref(config),
                                     None if table_dir is None else table_dir.encode()))


def dropin_release() -> None:
    _lib.load().dnsmc_dropin_release()


def mc_gpu(T: np.ndarray, ystart: int) -> None:
    """code/mc_gpu.cu:440 -- enqueue the MC for the slab starting at global j
    = ystart (1-based); returns immediately."""
    lib = _lib.load()
    if T.dtype != np.float32 or not T.flags.c_contiguous:
        raise TypeError("T must be a C-contiguous float32 array in Fortran (i-fastest) order")
    ys = ctypes.c_int(int(ystart))
    lib.mc_gpu_(_fp(T), ctypes.byref(ys))


def get_results(Qr: np.ndarray, Vr: np.ndarray) -> None:
    """code/mc_gpu.cu:640 -- block, then write Q and sigma into interior cells."""
    lib = _lib.load()
    for a in (Qr, Vr):
        if a.dtype != np.float32 or not a.flags.c_contiguous:
            raise TypeError("outputs must be C-contiguous float32 arrays")
    lib.get_results_(_fp(Qr), _fp(Vr))


# ---------------------------------------------------------------------------
# learned control variate
# ---------------------------------------------------------------------------
def cvnet_default_config(**overrides) -> _lib.CvNetConfig:
    lib = _lib.load()
    c = _lib.CvNetConfig()
    lib.dnsmc_cvnet_default_config(ctypes.byref(c))
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise KeyError(f"unknown network config field {k!r}")
        setattr(c, k, v)
    return c


class CvNet:
    """The control-variate network of include/dnsmc.h (dnsmc_cvnet_*): features
    -> per (cell, band group) coefficient pair, log variance and log cost."""

    NFEAT, NOUT, NLABEL = _lib.CVNET_NFEAT, _lib.CVNET_NOUT, _lib.CVNET_NLABEL

    def __init__(self, config: _lib.CvNetConfig | None = None, *, _handle=None, **overrides):
        self._lib = _lib.load()
        if _handle is not None:
            self._h = _handle
            return
        cfg = config if config is not None else cvnet_default_config()
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        h = ctypes.c_void_p()
        check(self._lib.dnsmc_cvnet_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    @classmethod
    def load(cls, path: str) -> "CvNet":
        lib = _lib.load()
        h = ctypes.c_void_p()
        check(lib.dnsmc_cvnet_load(path.encode(), ctypes.byref(h)))
        return cls(_handle=h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dnsmc_cvnet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def param_count() -> int:
        return int(_lib.load().dnsmc_cvnet_param_count())

    def params(self):
        """(params float32 [P], scales float32 [3] = S_beta, S_v, S_c)."""
        p = np.zeros(self.param_count(), np.float32)
        s = np.zeros(3, np.float32)
        check(self._lib.dnsmc_cvnet_get_params(self._h, _fp(p), _fp(s)))
        return p, s

    def set_params(self, params=None, scales=None) -> None:
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        s = None if scales is None else np.ascontiguousarray(scales, np.float32)
        if p is not None and p.size != self.param_count():
            raise ValueError("wrong parameter count")
        check(self._lib.dnsmc_cvnet_set_params(self._h, _fp(p), _fp(s)))

    def save(self, path: str) -> None:
        check(self._lib.dnsmc_cvnet_save(self._h, path.encode()))

    def features(self, solver: "Solver"):
        """[rows][67] features of the solver's region (tally order: field, i, k, j)."""
        i0, i1, j0, j1, k0, k1 = solver._region
        rows = solver._nfields * (i1 - i0) * (j1 - j0) * (k1 - k0)
        out = np.zeros((rows, self.NFEAT), np.float32)
        check(self._lib.dnsmc_cvnet_features(self._h, solver._h, _fp(out)))
        return out

    def add_training_data(self, solver: "Solver") -> None:
        check(self._lib.dnsmc_cvnet_add_training_data(self._h, solver._h))

    def clear_training_data(self) -> None:
        check(self._lib.dnsmc_cvnet_clear_training_data(self._h))

    def training_rows(self) -> int:
        return int(self._lib.dnsmc_cvnet_training_rows(self._h))

    def train(self, epochs: int = 1):
        """Mean losses of the last pass: (total, beta, variance, cost)."""
        l = np.zeros(4, np.float64)
        check(self._lib.dnsmc_cvnet_train(self._h, int(epochs), _dp(l)))
        return tuple(float(v) for v in l)

    def eval(self, features):
        x = np.ascontiguousarray(features, np.float32).reshape(-1, self.NFEAT)
        out = np.zeros((x.shape[0], self.NOUT), np.float32)
        check(self._lib.dnsmc_cvnet_eval(self._h, _fp(x), x.shape[0], _fp(out)))
        return out

    def gradient(self, features, labels):
        """(grad [P], losses (total, beta, variance, cost)) of one forward and
        backward pass on host features [rows][67] and labels [rows][G][8]."""
        x = np.ascontiguousarray(features, np.float32).reshape(-1, self.NFEAT)
        y = np.ascontiguousarray(labels, np.float32)
        G = y.shape[1]
        g = np.zeros(self.param_count(), np.float32)
        l = np.zeros(4, np.float64)
        check(self._lib.dnsmc_cvnet_gradient(self._h, _fp(x), _fp(y), G, x.shape[0], _fp(g), _dp(l)))
        return g, tuple(float(v) for v in l)

    def apply(self, solver: "Solver", beta: bool = True, rays: bool = True, mean_rays: int = 64,
              min_rays: int = 8, max_rays: int = 4096) -> None:
        flags = (_lib.CVNET_BETA if beta else 0) | (_lib.CVNET_RAYS if rays else 0)
        check(self._lib.dnsmc_cvnet_apply(self._h, solver._h, flags, int(mean_rays), int(min_rays),
                                          int(max_rays)))
        if rays:
            solver._keep = []
            solver._rays_dev = True
        if beta:
            solver._beta_dev = True


def ck_from_lbl(spec: dict, gq, n_pwrk: int = 10000):
    """Correlated-k table from line-by-line spectra on the GPU
    (dnsmc_ck_from_lbl): spec holds kappa [nT][nX][npts] (1/m, uniform grid
    wv0 + i dwv in 1/cm) and the bands' first point, point count and edges
    (the keys of synth.lbl_spectrum).  Returns (kq [nbands][nq][nT][nX]
    float32, the layout of Solver.set_table's k, and kavg [nT][nX][nbands])."""
    lib = _lib.load()
    k = np.ascontiguousarray(spec["kappa"], np.float64)
    nT, nX, npts = k.shape
    gq = np.ascontiguousarray(gq, np.float64)
    first = np.ascontiguousarray(spec["first"], np.int64)
    count = np.ascontiguousarray(spec["count"], np.int32)
    wl = np.ascontiguousarray(spec["wv_left"], np.float64)
    wr = np.ascontiguousarray(spec["wv_right"], np.float64)
    d = _lib.LblDesc()
    d.nT, d.nX, d.npts, d.wv0, d.dwv = nT, nX, npts, float(spec["wv0"]), float(spec["dwv"])
    dp = ctypes.POINTER(ctypes.c_double)
    d.kappa = k.ctypes.data_as(dp)
    d.nbands = first.size
    d.first = first.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    d.count = count.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.wv_left, d.wv_right = wl.ctypes.data_as(dp), wr.ctypes.data_as(dp)
    d.nq, d.gq, d.n_pwrk = gq.size, gq.ctypes.data_as(dp), int(n_pwrk)
    kq = np.zeros((first.size, gq.size, nT, nX), np.float32)
    kavg = np.zeros((nT, nX, first.size))
    check(lib.dnsmc_ck_from_lbl(ctypes.byref(d), _fp(kq), _dp(kavg)))
    return kq, kavg


def solver_rays_per_item(solver: "Solver"):
    """The per-(group, packet) ray table in effect, or None."""
    return solver.rays_per_item()
