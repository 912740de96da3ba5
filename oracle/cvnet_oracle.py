"""CPU oracle of the control-variate network (test infrastructure only).

A numpy restatement of the network in dnsmc_gb300/csrc/mc_cvnet.cu: feature
construction (bit-exact, same FP32 operations and bf16 rounding), forward
pass, losses and backward pass.  Two arithmetic modes:

* ``mimic=True``  -- round weights, activations and back-propagated
  pre-activation gradients to bf16 where the CUDA kernels do, accumulate in
  float64 (the kernels accumulate in FP32): the GPU gradient must agree with
  this to bf16 tie-flip noise;
* ``mimic=False`` -- plain float64 end to end: the exact gradient of the
  network as a real function, checked against finite differences on the CPU.

The estimator quantities follow the march (code/mc_gpu.cu:44-438 restated in
oracle/mc_oracle.cpp): per ray X, the surrogate ray Y_a through the layer-mean
medium and its own-layer part Y_b; the tallied residual X - beta_a Y_a -
beta_b Y_b has per-ray variance

    V(beta) = Cxx - 2 beta_a Cxa - 2 beta_b Cxb + beta_a^2 Caa
              + 2 beta_a beta_b Cab + beta_b^2 Cbb.
"""
from __future__ import annotations

import math

import numpy as np

NFEAT, K0, HID, NOUT, NPROF, NLAB = 67, 80, 128, 64, 32, 8

# flat parameter layout (mc_cvnet.cu)
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * K0
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * HID
OFF_W4 = OFF_B3 + HID
OFF_B4 = OFF_W4 + NOUT * HID
NPARAM = OFF_B4 + NOUT


def bf16(a) -> np.ndarray:
    """Round float32 values to bf16 (round to nearest, ties to even); returns
    float32 holding the bf16 values."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isfinite(a), out, a).astype(np.float32)


def unpack(p: np.ndarray):
    p = np.asarray(p)
    W1 = p[OFF_W1:OFF_B1].reshape(HID, K0)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(HID, HID)
    b2 = p[OFF_B2:OFF_W3]
    W3 = p[OFF_W3:OFF_B3].reshape(HID, HID)
    b3 = p[OFF_B3:OFF_W4]
    W4 = p[OFF_W4:OFF_B4].reshape(NOUT, HID)
    b4 = p[OFF_B4:NPARAM]
    return [(W1, b1), (W2, b2), (W3, b3), (W4, b4)]


def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)
    for off, rows, cols, fan in ((OFF_W1, HID, K0, NFEAT), (OFF_W2, HID, HID, HID), (OFF_W3, HID, HID, HID)):
        a = math.sqrt(6.0 / fan)
        p[off:off + rows * cols] = rng.uniform(-a, a, rows * cols)
    p[OFF_W1:OFF_B1].reshape(HID, K0)[:, NFEAT:] = 0.0
    return p


# ---------------------------------------------------------------------------
# features (bit-exact with features_kernel)
# ---------------------------------------------------------------------------
def features(T, X, fw, region, T_center, T_scale, x_center, x_scale) -> np.ndarray:
    """T, X: (nfields, kmax, jmax, imax) float32 (X None without an x axis);
    fw: imax+1 faces; region (i0, i1, j0, j1, k0, k1).  Rows in tally order
    (field, i, k, j fastest), 67 bf16-rounded features as float32."""
    f32 = np.float32
    T = np.asarray(T, f32)
    nf, nk, nj, ni = T.shape
    fw = np.asarray(fw, f32)
    i0, i1, j0, j1, k0, k1 = region
    Tis = f32(1.0) / f32(T_scale)
    Xis = f32(1.0) / f32(x_scale)
    Tc, Xc = f32(T_center), f32(x_center)
    ii = np.arange(i0, i1)
    kk = np.arange(k0, k1)
    jj = np.arange(j0, j1)
    # (nf, niR, nkR, njR) views
    Tr = T[:, k0:k1, j0:j1, :].transpose(0, 3, 1, 2)            # (nf, imax, nkR, njR)
    out = np.zeros((nf, len(ii), len(kk), len(jj), NFEAT), f32)
    out[..., 0] = (Tr[:, ii] - Tc) * Tis
    if X is not None:
        Xr = np.asarray(X, f32)[:, k0:k1, j0:j1, :].transpose(0, 3, 1, 2)
        out[..., 1] = (Xr[:, ii] - Xc) * Xis
    o = f32(0.5) * (fw[ii] + fw[ii + 1])
    eta = (o - fw[0]) / (fw[ni] - fw[0])
    out[..., 2] = (f32(2.0) * eta - f32(1.0))[None, :, None, None]
    for q in range(NPROF):
        l = ((2 * q + 1) * ni) // (2 * NPROF)
        out[..., 3 + q] = ((Tr[:, l] - Tc) * Tis)[:, None]
        if X is not None:
            out[..., 3 + NPROF + q] = ((Xr[:, l] - Xc) * Xis)[:, None]
    return bf16(out.reshape(-1, NFEAT))


# ---------------------------------------------------------------------------
# network
# ---------------------------------------------------------------------------
def gelu(z):
    """GELU in its tanh form (Hendrycks & Gimpel 2016), as the device:
    0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))."""
    return 0.5 * z * (1.0 + np.tanh(math.sqrt(2.0 / math.pi) * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(math.sqrt(2.0 / math.pi) * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * math.sqrt(2.0 / math.pi) * (1.0 + 3 * 0.044715 * z * z)


def forward(p, feats, mimic=True):
    """(out [rows][32], cache) in float64."""
    layers = unpack(np.asarray(p, np.float32 if mimic else np.float64))
    x = np.zeros((feats.shape[0], K0), np.float64)
    x[:, :NFEAT] = bf16(feats) if mimic else feats
    H = [x]
    Z = [None]
    h = x
    for l, (W, b) in enumerate(layers):
        Wm = bf16(W).astype(np.float64) if mimic else W.astype(np.float64)
        z = h @ Wm.T + b.astype(np.float64)
        if l == 3:
            return z, dict(H=H, Z=Z, W=[bf16(L[0]).astype(np.float64) if mimic else L[0].astype(np.float64)
                                        for L in layers])
        h = gelu(z)
        if mimic:
            h = bf16(h.astype(np.float32)).astype(np.float64)
        Z.append(z)
        H.append(h)


def loss_grad(out, labels, scales, ridge):
    """Mean losses (beta, var, cost) over rows and d(total)/d out."""
    Sb, Sv, Sc = (float(s) for s in scales)
    rows, G = labels.shape[0], labels.shape[1]
    d = np.zeros((rows, NOUT))
    lb = lv = lc = 0.0
    for g in range(G):
        y = labels[:, g, :].astype(np.float64)
        Cxx, Caa, Cbb, Cxa, Cxb, Cab, v, c = (y[:, q] for q in range(8))
        da, db = out[:, 4 * g], out[:, 4 * g + 1]
        ba, bb = 1.0 + da, -1.0 + db
        V = Cxx - 2 * ba * Cxa - 2 * bb * Cxb + ba * ba * Caa + 2 * ba * bb * Cab + bb * bb * Cbb
        lb += float(((V + ridge * (Caa * da * da + Cbb * db * db)) / Sb).sum())
        d[:, 4 * g] = (2 * (ba * Caa + bb * Cab - Cxa) + 2 * ridge * Caa * da) / Sb
        d[:, 4 * g + 1] = (2 * (bb * Cbb + ba * Cab - Cxb) + 2 * ridge * Cbb * db) / Sb
        ov = np.clip(out[:, 4 * g + 2], -15, 15)
        e = v / Sv * np.exp(-ov)
        m = v > 0
        lv += float(np.where(m, e + ov, 0.0).sum())
        d[:, 4 * g + 2] = np.where(m, 1.0 - e, 0.0)
        oc = np.clip(out[:, 4 * g + 3], -15, 15)
        e = c / Sc * np.exp(-oc)
        m = c > 0
        lc += float(np.where(m, e + oc, 0.0).sum())
        d[:, 4 * g + 3] = np.where(m, 1.0 - e, 0.0)
    return (lb / rows, lv / rows, lc / rows), d / rows


def backward(cache, dout, mimic=True):
    """Flat gradient (float64) of the parameters."""
    g = np.zeros(NPARAM)
    offs = [(OFF_W1, OFF_B1, K0), (OFF_W2, OFF_B2, HID), (OFF_W3, OFF_B3, HID), (OFF_W4, OFF_B4, HID)]
    dz = bf16(dout.astype(np.float32)).astype(np.float64) if mimic else dout
    for l in (3, 2, 1, 0):
        offW, offB, nin = offs[l]
        h = cache["H"][l]
        nout = dz.shape[1]
        g[offW:offW + nout * nin] = (dz.T @ h).ravel()
        g[offB:offB + nout] = dz.sum(0)
        if l == 0:
            break
        dh = dz @ cache["W"][l]
        dz = dh * gelu_grad(cache["Z"][l])
        if mimic:
            dz = bf16(dz.astype(np.float32)).astype(np.float64)
    return g


def gradient(p, feats, labels, scales, ridge, mimic=True):
    out, cache = forward(p, feats, mimic)
    losses, dout = loss_grad(out, labels, scales, ridge)
    return backward(cache, dout, mimic), losses, out


# ---------------------------------------------------------------------------
# labels and allocation
# ---------------------------------------------------------------------------
def labels_from_moments(mo, rays, varg=None, steps_per_ray=None):
    """mo: (..., 9) per-ray moment sums over `rays` rays -> (..., 8) labels."""
    mo = np.asarray(mo, np.float64)
    n = float(rays)
    m = mo[..., :3] / n
    lab = np.zeros(mo.shape[:-1] + (NLAB,), np.float32)
    lab[..., 0] = np.maximum(0.0, mo[..., 3] / n - m[..., 0] ** 2)
    lab[..., 1] = np.maximum(0.0, mo[..., 4] / n - m[..., 1] ** 2)
    lab[..., 2] = np.maximum(0.0, mo[..., 5] / n - m[..., 2] ** 2)
    lab[..., 3] = mo[..., 6] / n - m[..., 0] * m[..., 1]
    lab[..., 4] = mo[..., 7] / n - m[..., 0] * m[..., 2]
    lab[..., 5] = mo[..., 8] / n - m[..., 1] * m[..., 2]
    if varg is not None:
        lab[..., 6] = varg * n
    if steps_per_ray is not None:
        lab[..., 7] = steps_per_ray
    return lab


def residual_variance(lab, beta_a, beta_b):
    Cxx, Caa, Cbb, Cxa, Cxb, Cab = (lab[..., q].astype(np.float64) for q in range(6))
    return (Cxx - 2 * beta_a * Cxa - 2 * beta_b * Cxb + beta_a ** 2 * Caa + 2 * beta_a * beta_b * Cab
            + beta_b ** 2 * Cbb)
