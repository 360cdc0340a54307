"""CPU restatement of the spectral neural operator (SNO) surrogate network.

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` may import this module, as the
checker of the GPU kernels' forward pass and gradients.  The product package
never calls it.

The surrogate has no pyofss counterpart (parity unpinned against the
reference); this file is its specification.  It follows the Fourier neural
operator of Li et al., "Fourier Neural Operator for Parametric Partial
Differential Equations" (ICLR 2021), with real-valued per-mode mixing:

* lifting      X0 = feat P + bp                               (feat: [B, N, cin])
* layer l      Xh = F X_l                                     (truncated DFT, [2K, W] per sample)
               Yh[:, k] = Xh[:, k] R_l[k]                     (per mode k, [2W] x [2W, 2W])
               Z_l = X_l Wp_l + b_l + G Yh ;  X_{l+1} = GELU(Z_l)
* projection   Zq = X_L Q1 + bq1 ;  out = resid + GELU(Zq) Q2 + bq2

F holds rows cos(2 pi k n / N), -sin(2 pi k n / N) for modes k < K (row 2k, 2k+1);
G is the matching real inverse, G[n, 2k] = c_k cos / N, G[n, 2k+1] = -c_k sin / N
with c_0 = 1, c_k = 2.  GELU is the tanh form.  Like the GPU path, every GEMM
operand is rounded to bfloat16 (round to nearest even) and products are
accumulated in higher precision (here float64).  The loss is the mean over
samples of |out - target|^2 / |target|^2.
"""

import numpy as np


# bfloat16 rounding of GEMM operands (switched off by the finite-difference
# self-check of backward(), which needs a smooth function)
ROUND_BF16 = True


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    if not ROUND_BF16:
        return np.asarray(x, dtype=np.float64)
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def dft_mats(n, modes):
    k = np.arange(modes)[:, None]
    t = np.arange(n)[None, :]
    ang = 2.0 * np.pi * ((k * t) % n) / n
    F = np.empty((2 * modes, n))
    F[0::2] = np.cos(ang)
    F[1::2] = -np.sin(ang)
    c = np.where(np.arange(modes) == 0, 1.0, 2.0)[:, None] / n
    G = np.empty((n, 2 * modes))
    G[:, 0::2] = (c * np.cos(ang)).T
    G[:, 1::2] = (-c * np.sin(ang)).T
    return F, G


def gelu(z):
    c = 0.7978845608028654
    return 0.5 * z * (1.0 + np.tanh(c * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    c = 0.7978845608028654
    u = c * (z + 0.044715 * z ** 3)
    th = np.tanh(u)
    return 0.5 * (1.0 + th) + 0.5 * z * (1.0 - th * th) * c * (1.0 + 3 * 0.044715 * z * z)


def forward(p, feat, resid, F, G):
    """p: dict of float arrays (P, bp, R0.., Wp0.., b0.., Q1, bq1, Q2, bq2); feat [B, N, cin];
    resid [B, N, 2].  Returns (out [B, N, 2], cache)."""
    L = sum(1 for k in p if k.startswith("Wp"))
    B, N, _ = feat.shape
    W = p["P"].shape[1]
    K = F.shape[0] // 2
    Fb, Gb = bf16(F), bf16(G)
    X = bf16(feat) @ bf16(p["P"]) + p["bp"]
    cache = {"feat": feat, "X": [bf16(X)], "Z": [], "Xh": [], "Yh": []}
    Xl = bf16(X)
    for l in range(L):
        Xh = np.einsum("mn,bnw->bmw", Fb, Xl)                  # [B, 2K, W]
        Xh16 = bf16(Xh)
        A = Xh16.reshape(B, K, 2 * W)                           # mode k: [re(W), im(W)]
        Yh = np.einsum("bki,kio->bko", A, bf16(p["R%d" % l]))   # [B, K, 2W]
        Yh16 = bf16(Yh).reshape(B, 2 * K, W)
        Z = Xl @ bf16(p["Wp%d" % l]) + p["b%d" % l] + np.einsum("nm,bmw->bnw", Gb, Yh16)
        cache["Xh"].append(Xh16)
        cache["Yh"].append(Yh16)
        cache["Z"].append(Z)
        Xl = bf16(gelu(Z))
        cache["X"].append(Xl)
    Zq = Xl @ bf16(p["Q1"]) + p["bq1"]
    H = bf16(gelu(Zq))
    out = resid + H @ bf16(p["Q2"]) + p["bq2"]
    cache.update(Zq=Zq, H=H)
    return out, cache


def loss(out, target):
    B = out.shape[0]
    d = (out - target).reshape(B, -1)
    t = target.reshape(B, -1)
    tn = np.sum(t * t, axis=1)
    err = np.sum(d * d, axis=1) / tn
    grad = (2.0 / (tn[:, None] * B) * d).reshape(out.shape)
    return err, grad


def backward(p, cache, dout, F, G):
    """Gradients of every parameter for d loss / d out = dout (GEMM operands in bfloat16)."""
    L = sum(1 for k in p if k.startswith("Wp"))
    B, N, _ = dout.shape
    W = p["P"].shape[1]
    K = F.shape[0] // 2
    Fb, Gb = bf16(F), bf16(G)
    g = {}
    d16 = bf16(dout)
    g["Q2"] = np.einsum("bnh,bno->ho", cache["H"], d16)
    g["bq2"] = dout.sum(axis=(0, 1))
    dH = d16 @ bf16(p["Q2"]).T
    dZq = dH * gelu_grad(cache["Zq"])
    dZq16 = bf16(dZq)
    Xl = cache["X"][L]
    g["Q1"] = np.einsum("bnw,bnh->wh", Xl, dZq16)
    g["bq1"] = dZq.sum(axis=(0, 1))
    dX = dZq16 @ bf16(p["Q1"]).T
    for l in reversed(range(L)):
        dZ = dX * gelu_grad(cache["Z"][l])
        dZ16 = bf16(dZ)
        Xl = cache["X"][l]
        g["Wp%d" % l] = np.einsum("bni,bno->io", Xl, dZ16)
        g["b%d" % l] = dZ.sum(axis=(0, 1))
        dX = dZ16 @ bf16(p["Wp%d" % l]).T
        dYh = np.einsum("nm,bnw->bmw", Gb, dZ16)                # [B, 2K, W]
        dYh16 = bf16(dYh).reshape(B, K, 2 * W)
        A = cache["Xh"][l].reshape(B, K, 2 * W)
        g["R%d" % l] = np.einsum("bki,bko->kio", A, dYh16)
        dXh = np.einsum("bko,kio->bki", dYh16, bf16(p["R%d" % l]))
        dXh16 = bf16(dXh).reshape(B, 2 * K, W)
        dX = dX + np.einsum("mn,bmw->bnw", Fb, dXh16)
    dX16 = bf16(dX)
    g["P"] = np.einsum("bnc,bnw->cw", bf16(cache["feat"]), dX16)
    g["bp"] = dX.sum(axis=(0, 1))
    return g


def init_params(cin, width, modes, layers, hidden, rng):
    """Initial weights (scaled normal) used by the tests; same shapes as the GPU model."""
    p = {"P": rng.standard_normal((cin, width)) / np.sqrt(cin), "bp": np.zeros(width)}
    for l in range(layers):
        p["R%d" % l] = rng.standard_normal((modes, 2 * width, 2 * width)) / (2 * width)
        p["Wp%d" % l] = rng.standard_normal((width, width)) / np.sqrt(width)
        p["b%d" % l] = np.zeros(width)
    p["Q1"] = rng.standard_normal((width, hidden)) / np.sqrt(width)
    p["bq1"] = np.zeros(hidden)
    p["Q2"] = rng.standard_normal((hidden, 2)) / np.sqrt(hidden) * 0.1
    p["bq2"] = np.zeros(2)
    return p
