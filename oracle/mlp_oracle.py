"""CPU restatement of the surrogate MLP (numpy), for tests only.

This is test infrastructure: the oracle for the device MLP in
cac_code_gb300/csrc/mlp.cu and k_gemm.cu, never a product path.  The
reference has no surrogate (it evaluates every element by integration-point
quadrature), so the network has no reference file to cite; this module
restates the device's own definition:

  x0 = bf16((x - in_mean) * (1 / in_std))                       [n][32]
  z_l = h_{l-1} bf16(W_l)^T + b_l,  h_l = bf16(silu(z_l))        l = 1..3
  y = h_3 bf16(W_4)^T + b_4                                      [n][24]
  loss = mean((y - t_norm)^2),  t_norm = (t - out_mean) / out_std
  g_4 = bf16(2 (y - t_norm) / (n 24))
  g_l = bf16((g_{l+1} bf16(W_{l+1})) * silu'(z_l))
  dW_l = g_l^T h_{l-1},  db_l = sum_rows g_l

``exact=True`` drops every bf16 rounding and works in float64, which the
finite-difference test uses to pin the backward formulas themselves.
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 32, 256, 24
SHAPES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)),
          ("W3", (NH, NH)), ("b3", (NH,)), ("W4", (NOUT, NH)), ("b4", (NOUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray) -> dict:
    out, off = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = p[off:off + n].reshape(shp)
        off += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name]).reshape(-1) for name, _ in SHAPES])


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def normalize(x, t, norm):
    in_mean, in_std, out_mean, out_std = norm
    inv = (np.float32(1.0) / in_std.astype(np.float32)).astype(np.float32)
    xn = ((x.astype(np.float32) - in_mean.astype(np.float32)) * inv).astype(np.float32)
    tn = None
    if t is not None:
        tn = ((t.astype(np.float32) - out_mean.astype(np.float32)) / out_std.astype(np.float32)).astype(np.float32)
    return xn, tn


def forward(p: np.ndarray, xn: np.ndarray, exact: bool = False):
    P = unpack(p)
    dt = np.float64
    q = (lambda a: np.asarray(a, dtype=dt)) if exact else (lambda a: bf16(a).astype(dt))
    h = q(xn)
    cache = {"h0": h}
    for l in (1, 2, 3):
        z = h @ q(P[f"W{l}"]).T + P[f"b{l}"].astype(dt)
        if not exact:
            z = z.astype(np.float32).astype(dt)
        h = q(z * _sig(z))
        cache[f"z{l}"], cache[f"h{l}"] = z, h
    y = h @ q(P["W4"]).T + P["b4"].astype(dt)
    return y, cache


def loss_grad(p: np.ndarray, xn: np.ndarray, tn: np.ndarray, exact: bool = False):
    P = unpack(p)
    dt = np.float64
    q = (lambda a: np.asarray(a, dtype=dt)) if exact else (lambda a: bf16(a).astype(dt))
    y, c = forward(p, xn, exact)
    n = xn.shape[0]
    d = y - tn.astype(dt)
    loss = float((d ** 2).mean())
    g = q(2.0 * d / (n * NOUT))
    grads = {"W4": g.T @ c["h3"], "b4": g.sum(axis=0)}
    for l in (3, 2, 1):
        dh = g @ q(P[f"W{l + 1}"])
        z = c[f"z{l}"]
        s = _sig(z)
        g = q(dh * s * (1.0 + z * (1.0 - s)))
        grads[f"W{l}"] = g.T @ c[f"h{l - 1}"]
        grads[f"b{l}"] = g.sum(axis=0)
    return loss, pack(grads)
