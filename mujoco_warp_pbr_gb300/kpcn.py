"""Learned kernel-predicting denoiser (KPCN) for the path-traced tier.

A 4-level U-Net (channel widths 32 / 48 / 64 / 96, two 3 x 3 convolutions per level, 2 x 2
average pooling down, nearest upsampling and skip concatenation up) reads 10 feature channels per
pixel (log of the noisy demodulated radiance, first-hit albedo, normal, log depth and the log of
the per-pixel noise estimate; padded to 16) and predicts 25 logits per pixel; their softmax is a 5 x 5 kernel applied to the noisy
demodulated radiance, which the a-trous filter's last pass then remodulates, tone maps and
encodes. Weights and activations are BF16, accumulation FP32; every convolution (forward, input
gradient and weight gradient) runs on the tensor cores through the library (conv.cu), the other
pixel work through kpcn.cu, and the optimiser is Adam on FP32 master weights. The network is
trained on pairs the path tracer itself renders: 1-4 spp noisy features against converged
targets accumulated in FP64 (train_kpcn.py).

The a-trous filter stays the fallback: images whose sizes the convolution tiles do not cover
(width a power of two from 128 or a multiple of 128, height a multiple of 64) are filtered by it.
"""

from __future__ import annotations

import ctypes
import dataclasses
from pathlib import Path
from typing import Any

import numpy as np
import torch

from mujoco_warp_pbr_gb300 import _lib

FEATURES = 16
LOGITS = 32
TAPS = 25
WIDTHS = (32, 48, 64, 96)


@dataclasses.dataclass(frozen=True)
class LayerSpec:
  name: str
  level: int
  c_in: int
  c_in2: int
  c_out: int
  relu: bool


def layer_specs() -> list[LayerSpec]:
  w0, w1, w2, w3 = WIDTHS
  return [
    LayerSpec("e0a", 0, FEATURES, 0, w0, True),
    LayerSpec("e0b", 0, w0, 0, w0, True),
    LayerSpec("e1a", 1, w0, 0, w1, True),
    LayerSpec("e1b", 1, w1, 0, w1, True),
    LayerSpec("e2a", 2, w1, 0, w2, True),
    LayerSpec("e2b", 2, w2, 0, w2, True),
    LayerSpec("e3a", 3, w2, 0, w3, True),
    LayerSpec("e3b", 3, w3, 0, w3, True),
    LayerSpec("d2a", 2, w2, w3, w2, True),
    LayerSpec("d2b", 2, w2, 0, w2, True),
    LayerSpec("d1a", 1, w1, w2, w1, True),
    LayerSpec("d1b", 1, w1, 0, w1, True),
    LayerSpec("d0a", 0, w0, w1, w0, True),
    LayerSpec("d0b", 0, w0, 0, w0, True),
    LayerSpec("head", 0, w0, 0, LOGITS, False),
  ]


def supported(width: int, height: int) -> bool:
  """Image sizes whose four levels the 128-pixel convolution tiles cover."""
  if width % 8 or height % 8:
    return False
  for lv in range(4):
    w, h = width >> lv, height >> lv
    ok = (w % 128 == 0) if w >= 128 else (w >= 16 and 128 % w == 0)
    if not ok or h % (128 // min(w, 128)):
      return False
  return True


def _ptr(t: torch.Tensor | None) -> int | None:
  return t.data_ptr() if t is not None else None


class Layer:
  def __init__(self, spec: LayerSpec, device: torch.device, gen: torch.Generator):
    self.spec = spec
    cin = spec.c_in + spec.c_in2
    std = (2.0 / (9 * cin)) ** 0.5 if spec.name != "head" else 1.0e-3
    w = torch.randn((spec.c_out, 9, cin), generator=gen) * std
    if spec.name == "head":
      w[TAPS:] = 0.0
    self.w = w.to(device)
    self.b = torch.zeros(spec.c_out, device=device)
    self.gw = torch.zeros_like(self.w)
    self.gb = torch.zeros_like(self.b)
    self.mw, self.vw = torch.zeros_like(self.w), torch.zeros_like(self.w)
    self.mb, self.vb = torch.zeros_like(self.b), torch.zeros_like(self.b)
    self.w16 = torch.zeros((spec.c_out, 9, cin), dtype=torch.bfloat16, device=device)
    self.flip16 = torch.zeros((cin, 9, spec.c_out), dtype=torch.bfloat16, device=device)
    self.refresh()

  def refresh(self) -> None:
    """BF16 copies of the FP32 master weights (used after init and load)."""
    self.w16.copy_(self.w.to(torch.bfloat16))
    self.flip16.copy_(self.w.flip(1).permute(2, 1, 0).to(torch.bfloat16))


class KPCN:
  """The network, its optimiser state and per-batch-shape activation workspaces."""

  def __init__(self, device: torch.device | str = "cuda", seed: int = 0):
    self.device = torch.device(device)
    gen = torch.Generator().manual_seed(seed)
    self.layers = {s.name: Layer(s, self.device, gen) for s in layer_specs()}
    self.step_count = 0
    self.error = torch.zeros(1, dtype=torch.int32, device=self.device)
    self._ws: dict[tuple[int, int, int], dict[str, torch.Tensor]] = {}
    self._c_ws: torch.Tensor | None = None  # mjpbr_denoise_learned's workspace
    self._c_weights: _lib.KpcnWeights | None = None

  # ---------------------------------------------------------------- parameters
  def state_dict(self) -> dict[str, np.ndarray]:
    out = {}
    for name, l in self.layers.items():
      out[f"{name}.w"] = l.w.cpu().numpy()
      out[f"{name}.b"] = l.b.cpu().numpy()
    return out

  def load_state_dict(self, state: dict[str, np.ndarray]) -> None:
    for name, l in self.layers.items():
      l.w.copy_(torch.as_tensor(state[f"{name}.w"]))
      l.b.copy_(torch.as_tensor(state[f"{name}.b"]))
      l.refresh()

  def save(self, path: str | Path) -> None:
    np.savez_compressed(path, **self.state_dict())

  @classmethod
  def load(cls, path: str | Path, device: torch.device | str = "cuda") -> KPCN:
    net = cls(device)
    with np.load(path) as f:
      net.load_state_dict({k: f[k] for k in f.files})
    return net

  # ---------------------------------------------------------------- workspace
  def workspace(self, nimg: int, h: int, w: int, backward: bool = False) -> dict[str, torch.Tensor]:
    """Activation buffers of a batch shape (allocated once); the gradient buffers are added the
    first time a backward pass needs them, so inference holds only the forward activations."""
    key = (nimg, h, w)
    ws = self._ws.get(key)
    if ws is None:
      if not supported(w, h):
        raise ValueError(f"the learned denoiser needs images whose 4 levels tile into 128 pixels, got {w}x{h}")
      ws = self._ws[key] = self._alloc(nimg, h, w, self._FORWARD)
    if backward and "dlogits" not in ws:
      ws.update(self._alloc(nimg, h, w, self._BACKWARD))
    return ws

  _FORWARD = {
    # name: (level, channels, fp32)
    "a0": (0, 0, False), "s0": (0, 0, False), "p1": (1, 0, False), "a1": (1, 1, False), "s1": (1, 1, False), "p2": (2, 1, False),
    "a2": (2, 2, False), "s2": (2, 2, False), "p3": (3, 2, False), "a3": (3, 3, False), "b3": (3, 3, False), "u2": (2, 2, False),
    "v2": (2, 2, False), "u1": (1, 1, False), "v1": (1, 1, False), "u0": (0, 0, False), "v0": (0, 0, False),
    "logits": (0, "logits", True), "out": (0, "rgba", True),
    # the decoder's skip inputs upsampled x2 to the level they are concatenated at
    "up2": (2, 3, False), "up1": (1, 2, False), "up0": (0, 1, False),
  }
  _BACKWARD = {
    "kweights": (0, "taps", True), "gout": (0, "rgba", True), "dlogits": (0, "logits", False), "dv0": (0, 0, False), "du0": (0, 0, False), "dcat0": (0, (0, 1), True),
    "dskip0": (0, 0, True), "dv1": (1, 1, False), "du1": (1, 1, False), "dcat1": (1, (1, 2), True), "dskip1": (1, 1, True),
    "dv2": (2, 2, False), "du2": (2, 2, False), "dcat2": (2, (2, 3), True), "dskip2": (2, 2, True), "db3": (3, 3, False),
    "da3": (3, 3, False), "dp3": (3, 2, True), "ds2": (2, 2, False), "da2": (2, 2, False), "dp2": (2, 1, True), "ds1": (1, 1, False),
    "da1": (1, 1, False), "dp1": (1, 0, True), "ds0": (0, 0, False), "da0": (0, 0, False),
  }

  def _alloc(self, nimg: int, h: int, w: int, spec: dict) -> dict[str, torch.Tensor]:
    named = {"logits": LOGITS, "taps": TAPS, "rgba": 4}
    out = {}
    for name, (level, ch, f32) in spec.items():
      if isinstance(ch, tuple):
        c = WIDTHS[ch[0]] + WIDTHS[ch[1]]
      elif isinstance(ch, str):
        c = named[ch]
      else:
        c = WIDTHS[ch]
      dtype = torch.float32 if f32 else torch.bfloat16
      out[name] = torch.zeros((nimg, h >> level, w >> level, c), dtype=dtype, device=self.device)
    if "gout" in out:
      out["sums"] = torch.zeros(2, dtype=torch.float32, device=self.device)
    return out

  # ---------------------------------------------------------------- primitives
  def _stream(self) -> int:
    return torch.cuda.current_stream(self.device).cuda_stream

  def _conv(self, name: str, x: torch.Tensor, out: torch.Tensor | None, x2: torch.Tensor | None = None, out_f32: torch.Tensor | None = None) -> None:
    """x2: the skip input at the resolution of x (already upsampled)."""
    l = self.layers[name]
    s = l.spec
    n, h, w, _ = x.shape
    c = _lib.Conv(
      in_=_ptr(x), in2=_ptr(x2), weight=_ptr(l.w16), bias=_ptr(l.b), out=_ptr(out), out_f32=_ptr(out_f32), mask=None,
      error_word=_ptr(self.error), nimg=n, height=h, width=w, c_in=s.c_in, c_in2=s.c_in2, c_out=s.c_out, relu=int(s.relu),
      in2_full=1,
    )
    _lib.call("mjpbr_conv3x3_bf16", ctypes.byref(c), self._stream())

  def _dgrad(self, name: str, dy: torch.Tensor, out: torch.Tensor | None, mask: torch.Tensor | None = None, out_f32: torch.Tensor | None = None) -> None:
    """Input gradient: the convolution of dy with the flipped, transposed weights."""
    l = self.layers[name]
    s = l.spec
    n, h, w, _ = dy.shape
    c = _lib.Conv(
      in_=_ptr(dy), in2=None, weight=_ptr(l.flip16), bias=None, out=_ptr(out), out_f32=_ptr(out_f32), mask=_ptr(mask),
      error_word=_ptr(self.error), nimg=n, height=h, width=w, c_in=s.c_out, c_in2=0, c_out=s.c_in + s.c_in2, relu=0,
    )
    _lib.call("mjpbr_conv3x3_bf16", ctypes.byref(c), self._stream())

  def _wgrad(self, name: str, x: torch.Tensor, dy: torch.Tensor, x2: torch.Tensor | None = None) -> None:
    """x2: the skip input at the resolution of x (the forward pass's upsampled copy)."""
    l = self.layers[name]
    s = l.spec
    n, h, w, _ = x.shape
    tiles = n * h * w // 128
    per_cta = max(8, (tiles + 2047) // 2048)
    g = _lib.ConvGrad(
      in_=_ptr(x), in2=_ptr(x2), grad_out=_ptr(dy), grad_weight=_ptr(l.gw), grad_bias=_ptr(l.gb), error_word=_ptr(self.error),
      nimg=n, height=h, width=w, c_in=s.c_in, c_in2=s.c_in2, c_out=s.c_out, tiles_per_cta=per_cta, in2_full=1,
    )
    _lib.call("mjpbr_conv3x3_wgrad_bf16", ctypes.byref(g), self._stream())

  def _pool(self, x: torch.Tensor, out: torch.Tensor) -> None:
    n, h, w, c = x.shape
    _lib.call("mjpbr_avgpool2_bf16", _ptr(x), _ptr(out), n, h, w, c, self._stream())

  def _up(self, x: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
    n, h, w, c = x.shape
    _lib.call("mjpbr_upsample2_bf16", _ptr(x), _ptr(out), n, h, w, c, self._stream())
    return out

  # ---------------------------------------------------------------- network
  def forward(self, x0: torch.Tensor, radiance: torch.Tensor, train: bool = False) -> torch.Tensor:
    """x0 (n, h, w, 16) BF16 features, radiance (n, h, w, 4) FP32 noisy demodulated radiance;
    returns the filtered demodulated radiance (n, h, w, 4) (a view of the workspace)."""
    n, h, w, _ = x0.shape
    ws = self.workspace(n, h, w, backward=train)
    c = self._conv
    c("e0a", x0, ws["a0"])
    c("e0b", ws["a0"], ws["s0"])
    self._pool(ws["s0"], ws["p1"])
    c("e1a", ws["p1"], ws["a1"])
    c("e1b", ws["a1"], ws["s1"])
    self._pool(ws["s1"], ws["p2"])
    c("e2a", ws["p2"], ws["a2"])
    c("e2b", ws["a2"], ws["s2"])
    self._pool(ws["s2"], ws["p3"])
    c("e3a", ws["p3"], ws["a3"])
    c("e3b", ws["a3"], ws["b3"])
    c("d2a", ws["s2"], ws["u2"], x2=self._up(ws["b3"], ws["up2"]))
    c("d2b", ws["u2"], ws["v2"])
    c("d1a", ws["s1"], ws["u1"], x2=self._up(ws["v2"], ws["up1"]))
    c("d1b", ws["u1"], ws["v1"])
    c("d0a", ws["s0"], ws["u0"], x2=self._up(ws["v1"], ws["up0"]))
    c("d0b", ws["u0"], ws["v0"])
    c("head", ws["v0"], None, out_f32=ws["logits"])
    _lib.call(
      "mjpbr_kpcn_apply", _ptr(ws["logits"]), _ptr(radiance), _ptr(ws["kweights"]) if train else None, _ptr(ws["out"]), n, h, w,
      self._stream(),
    )
    return ws["out"]

  def backward(self, x0: torch.Tensor, radiance: torch.Tensor) -> None:
    """Accumulates the parameter gradients of the loss whose output gradient is in ws['gout']."""
    n, h, w, _ = x0.shape
    ws = self.workspace(n, h, w, backward=True)
    w0, w1, w2, w3 = WIDTHS
    st = self._stream()
    _lib.call("mjpbr_kpcn_apply_grad", _ptr(ws["gout"]), _ptr(ws["kweights"]), _ptr(radiance), _ptr(ws["dlogits"]), n, h, w, st)
    wg, dg = self._wgrad, self._dgrad
    wg("head", ws["v0"], ws["dlogits"])
    dg("head", ws["dlogits"], ws["dv0"], mask=ws["v0"])
    wg("d0b", ws["u0"], ws["dv0"])
    dg("d0b", ws["dv0"], ws["du0"], mask=ws["u0"])
    wg("d0a", ws["s0"], ws["du0"], x2=ws["up0"])
    dg("d0a", ws["du0"], None, out_f32=ws["dcat0"])
    _lib.call("mjpbr_split_concat_grad", _ptr(ws["dcat0"]), _ptr(ws["v1"]), _ptr(ws["dskip0"]), _ptr(ws["dv1"]), n, h, w, w0, w1, st)
    wg("d1b", ws["u1"], ws["dv1"])
    dg("d1b", ws["dv1"], ws["du1"], mask=ws["u1"])
    wg("d1a", ws["s1"], ws["du1"], x2=ws["up1"])
    dg("d1a", ws["du1"], None, out_f32=ws["dcat1"])
    _lib.call("mjpbr_split_concat_grad", _ptr(ws["dcat1"]), _ptr(ws["v2"]), _ptr(ws["dskip1"]), _ptr(ws["dv2"]), n, h >> 1, w >> 1, w1, w2, st)
    wg("d2b", ws["u2"], ws["dv2"])
    dg("d2b", ws["dv2"], ws["du2"], mask=ws["u2"])
    wg("d2a", ws["s2"], ws["du2"], x2=ws["up2"])
    dg("d2a", ws["du2"], None, out_f32=ws["dcat2"])
    _lib.call("mjpbr_split_concat_grad", _ptr(ws["dcat2"]), _ptr(ws["b3"]), _ptr(ws["dskip2"]), _ptr(ws["db3"]), n, h >> 2, w >> 2, w2, w3, st)
    wg("e3b", ws["a3"], ws["db3"])
    dg("e3b", ws["db3"], ws["da3"], mask=ws["a3"])
    wg("e3a", ws["p3"], ws["da3"])
    dg("e3a", ws["da3"], None, out_f32=ws["dp3"])
    _lib.call("mjpbr_unpool_add_grad", _ptr(ws["dskip2"]), _ptr(ws["dp3"]), _ptr(ws["s2"]), _ptr(ws["ds2"]), n, h >> 2, w >> 2, w2, st)
    wg("e2b", ws["a2"], ws["ds2"])
    dg("e2b", ws["ds2"], ws["da2"], mask=ws["a2"])
    wg("e2a", ws["p2"], ws["da2"])
    dg("e2a", ws["da2"], None, out_f32=ws["dp2"])
    _lib.call("mjpbr_unpool_add_grad", _ptr(ws["dskip1"]), _ptr(ws["dp2"]), _ptr(ws["s1"]), _ptr(ws["ds1"]), n, h >> 1, w >> 1, w1, st)
    wg("e1b", ws["a1"], ws["ds1"])
    dg("e1b", ws["ds1"], ws["da1"], mask=ws["a1"])
    wg("e1a", ws["p1"], ws["da1"])
    dg("e1a", ws["da1"], None, out_f32=ws["dp1"])
    _lib.call("mjpbr_unpool_add_grad", _ptr(ws["dskip0"]), _ptr(ws["dp1"]), _ptr(ws["s0"]), _ptr(ws["ds0"]), n, h, w, w0, st)
    wg("e0b", ws["a0"], ws["ds0"])
    dg("e0b", ws["ds0"], ws["da0"], mask=ws["a0"])
    wg("e0a", x0, ws["da0"])

  def loss_grad(self, target: torch.Tensor, scale: torch.Tensor | None = None, offset: torch.Tensor | None = None, w_l1: float = 1.0, w_rel: float = 1.0) -> torch.Tensor:
    """Loss of ws['out'] against target (n, h, w, 4), in HDR when scale / offset map the
    demodulated radiance there (mjpbr_kpcn_remod): writes ws['gout']; returns the device sums
    (L1, relative MSE) over pixels and channels."""
    n, h, w, _ = target.shape
    ws = self.workspace(n, h, w, backward=True)
    ws["sums"].zero_()
    _lib.call(
      "mjpbr_kpcn_loss", _ptr(ws["out"]), _ptr(target), _ptr(scale), _ptr(offset), _ptr(ws["gout"]), _ptr(ws["sums"]), n * h * w, w_l1, w_rel,
      self._stream(),
    )
    return ws["sums"]

  def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1.0e-8) -> None:
    self.step_count += 1
    st = self._stream()
    for l in self.layers.values():
      s = l.spec
      cin = s.c_in + s.c_in2
      _lib.call("mjpbr_adam", _ptr(l.w), _ptr(l.gw), _ptr(l.mw), _ptr(l.vw), _ptr(l.w16), _ptr(l.flip16), l.w.numel(), s.c_out, cin, lr, beta1, beta2, eps, self.step_count, st)
      _lib.call("mjpbr_adam", _ptr(l.b), _ptr(l.gb), _ptr(l.mb), _ptr(l.vb), None, None, l.b.numel(), 0, 0, lr, beta1, beta2, eps, self.step_count, st)

  def train_step(self, x0: torch.Tensor, radiance: torch.Tensor, target: torch.Tensor, lr: float, scale: torch.Tensor | None = None, offset: torch.Tensor | None = None) -> torch.Tensor:
    self.forward(x0, radiance, train=True)
    sums = self.loss_grad(target, scale, offset)
    self.backward(x0, radiance)
    self.adam(lr)
    return sums

  def zero_grad(self) -> None:
    for l in self.layers.values():
      l.gw.zero_()
      l.gb.zero_()

  # ---------------------------------------------------------------- rendering
  def c_weights(self) -> _lib.KpcnWeights:
    """The network's BF16 weights and FP32 biases as the C ABI's MjpbrKpcnWeights (device pointers,
    valid while the network lives), for mjpbr_denoise_learned."""
    wts = _lib.KpcnWeights()
    for k, spec in enumerate(layer_specs()):
      layer = self.layers[spec.name]
      wts.weight[k] = layer.w16.data_ptr()
      wts.bias[k] = layer.b.data_ptr()
    return wts

  def denoise(self, m: Any, d: Any, rc: Any, chunk: int = 512, driver: str = "c") -> None:
    """Filters a denoising path-traced frame (rendered with render(..., denoise=False)) into the
    context's RGB (and HDR) outputs with the network, every RGB camera in turn, `chunk` worlds at a
    time (the activations of a chunk are the only network memory). Raises ValueError for camera
    sizes the convolution tiles do not cover (the a-trous filter, render(..., denoise=True),
    handles those). Capturable in a CUDA graph after one call outside the capture.

    driver "c" makes the whole pass one library call (mjpbr_denoise_learned); "python" issues the
    same launches from here, one call each (the reference the C driver is tested against)."""
    from mujoco_warp_pbr_gb300.render import scene

    s = scene(m, d, rc)
    for (width, height), on in zip(rc.base.cam_res, rc.base.render_rgb):
      if on and not supported(width, height):
        raise ValueError(f"the learned denoiser needs images whose 4 levels tile into 128 pixels, got {width}x{height}")
    if driver == "c":
      lib = _lib.load()
      nw = min(chunk, rc.nworld)
      need = max(int(lib.mjpbr_kpcn_workspace_bytes(nw, h, w)) for (w, h), on in zip(rc.base.cam_res, rc.base.render_rgb) if on)
      if self._c_ws is None or self._c_ws.numel() < need:
        self._c_ws = torch.empty(need, dtype=torch.uint8, device=self.device)
      if self._c_weights is None:
        self._c_weights = self.c_weights()
      _lib.call("mjpbr_denoise_learned", ctypes.byref(s), ctypes.byref(self._c_weights), self._c_ws.data_ptr(), self._c_ws.numel(), chunk,
                self._stream())
      return
    n = rc.nworld
    st = self._stream()
    src = rc.denoise_buffers[0].view(n, -1, 4)
    dst = rc.denoise_buffers[1].view(n, -1, 4)
    for cam, (width, height) in enumerate(rc.base.cam_res):
      if not rc.base.render_rgb[cam]:
        continue
      adr = rc.base.rgb_adr[cam]
      for w0 in range(0, n, chunk):
        nw = min(chunk, n - w0)
        ws = self.workspace(nw, height, width)
        if "x0" not in ws:
          ws["x0"] = torch.zeros((nw, height, width, FEATURES), dtype=torch.bfloat16, device=self.device)
          ws["radiance"] = torch.zeros((nw, height, width, 4), dtype=torch.float32, device=self.device)
        _lib.call("mjpbr_kpcn_features", ctypes.byref(s), cam, w0, nw, _ptr(ws["x0"]), st)
        ws["radiance"].view(nw, -1, 4).copy_(src[w0 : w0 + nw, adr : adr + width * height])
        out = self.forward(ws["x0"], ws["radiance"])
        dst[w0 : w0 + nw, adr : adr + width * height].copy_(out.view(nw, -1, 4))
    # the a-trous filter's finish pass without filtering remodulates, tone maps and writes the
    # outputs from the network's filtered radiance
    finish = rc._host_cache.get("kpcn_finish")
    if finish is None or finish[0] is not s:
      fs = _lib.Scene.from_buffer_copy(s)
      fs.denoise_buffers[0] = rc.denoise_buffers[1].data_ptr()
      fs.denoise_iterations = 0
      finish = rc._host_cache["kpcn_finish"] = (s, fs)
    _lib.call("mjpbr_denoise_atrous", ctypes.byref(finish[1]), st)


def denoise_launches(rc: Any, chunk: int = 512) -> int:
  """Kernels one KPCN.denoise call launches: per RGB camera and chunk of worlds the features
  kernel and the forward pass (15 convolutions, 3 poolings, 3 upsamplings, the kernel
  application), then one finish pass."""
  per_forward = len(layer_specs()) + 3 + 3 + 1
  chunks = -(-rc.nworld // chunk)
  cams = sum(1 for v in rc.base.render_rgb if v)
  return cams * chunks * (1 + per_forward) + 1


def forward_flops(nimg: int, h: int, w: int) -> int:
  """Multiply-add FLOPs (2 per MAC) of the network's convolutions for a batch."""
  total = 0
  for s in layer_specs():
    px = nimg * (h >> s.level) * (w >> s.level)
    total += 2 * 9 * (s.c_in + s.c_in2) * s.c_out * px
  return total


def _bench() -> None:
  """python -m mujoco_warp_pbr_gb300.kpcn [nimg] [size] [reps]: times the network's forward pass
  (and one training step) on random inputs with CUDA events; prints one JSON line with the
  convolution TFLOP/s."""
  import json
  import sys

  nimg = int(sys.argv[1]) if len(sys.argv) > 1 else 256
  size = int(sys.argv[2]) if len(sys.argv) > 2 else 128
  reps = int(sys.argv[3]) if len(sys.argv) > 3 else 5
  net = KPCN("cuda", seed=0)
  g = torch.Generator(device="cuda").manual_seed(0)
  x0 = torch.rand((nimg, size, size, FEATURES), generator=g, device="cuda").to(torch.bfloat16)
  rad = torch.rand((nimg, size, size, 4), generator=g, device="cuda")
  tgt = torch.rand((nimg, size, size, 4), generator=g, device="cuda")
  for _ in range(2):
    net.forward(x0, rad)
  torch.cuda.synchronize()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record()
  for _ in range(reps):
    net.forward(x0, rad)
  e1.record()
  torch.cuda.synchronize()
  fwd_ms = e0.elapsed_time(e1) / reps
  net.train_step(x0, rad, tgt, 1e-4)
  torch.cuda.synchronize()
  e0.record()
  for _ in range(reps):
    net.train_step(x0, rad, tgt, 1e-4)
  e1.record()
  torch.cuda.synchronize()
  train_ms = e0.elapsed_time(e1) / reps
  flops = forward_flops(nimg, size, size)
  print(json.dumps({
    "nimg": nimg, "size": size, "forward_ms": fwd_ms, "forward_tflops": flops / fwd_ms / 1e9, "mpix_s": nimg * size * size / fwd_ms / 1e3,
    "train_step_ms": train_ms, "train_tflops": 3 * flops / train_ms / 1e9, "error": int(net.error.item()),
  }))


if __name__ == "__main__":
  _bench()
