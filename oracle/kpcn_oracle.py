"""CPU restatement of the learned denoiser (KPCN U-Net) in float64 NumPy — TEST INFRASTRUCTURE ONLY.

The network described by the learned-denoiser layer table below, layer by layer: 3 x 3 convolutions with zero padding, ReLU,
2 x 2 average pooling, nearest upsampling with skip concatenation, a 32-channel head whose first 25
logits are a softmax 5 x 5 kernel applied to the radiance (borders clamped), the L1 + relative-MSE
loss (relative L1 + relative MSE), and the backward pass of all of these. Activations can be rounded to BF16 after every layer
(as the GPU stores them) so that GPU gradients are compared with the same quantisation; without
rounding it is the exact float64 reference that finite differences pin. Only tests/ use it.
"""

from __future__ import annotations

import numpy as np

# The network of the learned denoiser: a 4-level U-Net of 3 x 3 convolutions with widths 32 / 48 /
# 64 / 96 (two per level on the way down and up, a skip concatenation entering each decoder
# level), and a 32-channel head whose first TAPS logits form a 5 x 5 kernel. Layer names in
# order: encoder e<level>a/b, decoder d<level>a/b, head.
TAPS = 25
LAYERS = ("e0a", "e0b", "e1a", "e1b", "e2a", "e2b", "e3a", "e3b", "d2a", "d2b", "d1a", "d1b", "d0a", "d0b", "head")


def round_bf16(x: np.ndarray) -> np.ndarray:
  """Round-to-nearest-even to BF16 (returned as float64)."""
  f = np.asarray(x, np.float32)
  u = f.view(np.uint32).astype(np.uint64)
  u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
  return u.astype(np.uint32).view(np.float32).astype(np.float64)


def conv(x, w, b):
  n, h, wd, _ = x.shape
  xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
  out = np.zeros((n, h, wd, w.shape[0]))
  for t in range(9):
    dy, dx = divmod(t, 3)
    out += np.einsum("nhwc,oc->nhwo", xp[:, dy : dy + h, dx : dx + wd], w[:, t, :], optimize=True)
  return out + b


def conv_backward(x, w, dy):
  """(dx, dw, db) of conv for output gradient dy."""
  n, h, wd, c = x.shape
  xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
  dxp = np.zeros_like(xp)
  dw = np.zeros_like(w)
  for t in range(9):
    ty, tx = divmod(t, 3)
    dw[:, t, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, ty : ty + h, tx : tx + wd], optimize=True)
    dxp[:, ty : ty + h, tx : tx + wd] += np.einsum("nhwo,oc->nhwc", dy, w[:, t, :], optimize=True)
  return dxp[:, 1:-1, 1:-1], dw, dy.sum(axis=(0, 1, 2))


def pool(x):
  return 0.25 * (x[:, 0::2, 0::2] + x[:, 1::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 1::2])


def up(x):
  return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def apply_kernel(logits, radiance):
  lg = logits[..., :TAPS]
  e = np.exp(lg - lg.max(-1, keepdims=True))
  wts = e / e.sum(-1, keepdims=True)
  n, h, w, _ = radiance.shape
  out = np.zeros((n, h, w, 3))
  taps = []
  for k in range(TAPS):
    dy, dx = k // 5 - 2, k % 5 - 2
    ys = np.clip(np.arange(h) + dy, 0, h - 1)
    xs = np.clip(np.arange(w) + dx, 0, w - 1)
    r = radiance[:, ys][:, :, xs, :3]
    taps.append(r)
    out += wts[..., k : k + 1] * r
  return out, wts, taps


def loss(out, target, w_l1=1.0, w_rel=1.0):
  t = np.maximum(target[..., :3], 0.0)
  d = out - t
  den = t * t + 0.01
  n = d.size
  value = w_l1 * (np.abs(d) / np.sqrt(den)).sum() / n + w_rel * (d * d / den).sum() / n
  grad = (w_l1 * np.sign(d) / np.sqrt(den) + w_rel * 2.0 * d / den) / n
  return value, grad


class Net:
  """Forward / backward of the U-Net for given weights {name: (w (cout, 9, cin), b)}."""

  def __init__(self, params: dict[str, tuple[np.ndarray, np.ndarray]], bf16: bool = True):
    self.p = {k: (np.asarray(w, np.float64), np.asarray(b, np.float64)) for k, (w, b) in params.items()}
    self.q = round_bf16 if bf16 else (lambda x: x)
    # gradients the GPU stores as BF16 (the inputs of its input- and weight-gradient convolutions)
    self.qg = self.q
    if bf16:
      self.p = {k: (round_bf16(w), b) for k, (w, b) in self.p.items()}

  def layer(self, name, x, relu=True):
    w, b = self.p[name]
    y = conv(x, w, b)
    return self.q(np.maximum(y, 0.0) if relu else y)

  def forward(self, x0, radiance):
    q, L = self.q, self.layer
    a = {}
    a["x0"] = x0
    a["a0"] = L("e0a", x0)
    a["s0"] = L("e0b", a["a0"])
    a["p1"] = q(pool(a["s0"]))
    a["a1"] = L("e1a", a["p1"])
    a["s1"] = L("e1b", a["a1"])
    a["p2"] = q(pool(a["s1"]))
    a["a2"] = L("e2a", a["p2"])
    a["s2"] = L("e2b", a["a2"])
    a["p3"] = q(pool(a["s2"]))
    a["a3"] = L("e3a", a["p3"])
    a["b3"] = L("e3b", a["a3"])
    a["u2"] = L("d2a", np.concatenate([a["s2"], up(a["b3"])], -1))
    a["v2"] = L("d2b", a["u2"])
    a["u1"] = L("d1a", np.concatenate([a["s1"], up(a["v2"])], -1))
    a["v1"] = L("d1b", a["u1"])
    a["u0"] = L("d0a", np.concatenate([a["s0"], up(a["v1"])], -1))
    a["v0"] = L("d0b", a["u0"])
    w, b = self.p["head"]
    a["logits"] = conv(a["v0"], w, b)
    out, wts, taps = apply_kernel(a["logits"], radiance)
    a["out"], a["wts"], a["taps"] = out, wts, taps
    self.a = a
    return out

  def backward(self, gout):
    """Parameter gradients {name: (dw, db)} for the output gradient gout (n, h, w, 3)."""
    a, g = self.a, {}
    wts = a["wts"]
    gk = np.stack([np.sum(gout * t, -1) for t in a["taps"]], -1)
    dlog = np.zeros(a["logits"].shape)
    dlog[..., :TAPS] = wts * (gk - np.sum(wts * gk, -1, keepdims=True))

    qg = self.qg
    dlog = qg(dlog)

    def back(name, x, dy, mask=None):
      dx, dw, db = conv_backward(x, self.p[name][0], dy)
      g[name] = (dw, db)
      return qg(dx * (mask > 0)) if mask is not None else dx

    d = back("head", a["v0"], dlog, a["v0"])
    d = back("d0b", a["u0"], d, a["u0"])
    dcat = back("d0a", np.concatenate([a["s0"], up(a["v1"])], -1), d)
    c0 = a["s0"].shape[-1]
    dskip0 = dcat[..., :c0]
    d = qg(pool(dcat[..., c0:]) * 4.0 * (a["v1"] > 0))
    d = back("d1b", a["u1"], d, a["u1"])
    dcat = back("d1a", np.concatenate([a["s1"], up(a["v2"])], -1), d)
    c1 = a["s1"].shape[-1]
    dskip1 = dcat[..., :c1]
    d = qg(pool(dcat[..., c1:]) * 4.0 * (a["v2"] > 0))
    d = back("d2b", a["u2"], d, a["u2"])
    dcat = back("d2a", np.concatenate([a["s2"], up(a["b3"])], -1), d)
    c2 = a["s2"].shape[-1]
    dskip2 = dcat[..., :c2]
    d = qg(pool(dcat[..., c2:]) * 4.0 * (a["b3"] > 0))
    d = back("e3b", a["a3"], d, a["a3"])
    dp = back("e3a", a["p3"], d)
    d = qg((dskip2 + up(dp) * 0.25) * (a["s2"] > 0))
    d = back("e2b", a["a2"], d, a["a2"])
    dp = back("e2a", a["p2"], d)
    d = qg((dskip1 + up(dp) * 0.25) * (a["s1"] > 0))
    d = back("e1b", a["a1"], d, a["a1"])
    dp = back("e1a", a["p1"], d)
    d = qg((dskip0 + up(dp) * 0.25) * (a["s0"] > 0))
    self.ds0 = d
    d = back("e0b", a["a0"], d, a["a0"])
    back("e0a", a["x0"], d)
    return g


def layer_names() -> list[str]:
  return list(LAYERS)
