"""3x3 convolution layers of the learned denoiser (tcgen05 implicit GEMM) against a float64 CPU
convolution of the same BF16 values: every tile geometry (image widths 16 to 256), the skip
concatenation with a half-resolution upsampled input or a full-resolution one, bias, ReLU, the
ReLU-derivative mask and the FP32 output; and the x2 nearest upsampling."""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def conv_ref(x, w, bias=None, x2=None, relu=False, mask=None):
  """x (n, h, w, c1), x2 (n, h/2, w/2, c2), (n, h, w, c2) or None, w (cout, 9, c1 + c2): float64
  NHWC result."""
  if x2 is not None:
    up = x2 if x2.shape[1] == x.shape[1] else np.repeat(np.repeat(x2, 2, axis=1), 2, axis=2)
    x = np.concatenate([x, up], axis=-1)
  n, h, wd, c = x.shape
  xp = np.zeros((n, h + 2, wd + 2, c))
  xp[:, 1:-1, 1:-1] = x
  out = np.zeros((n, h, wd, w.shape[0]))
  for tap in range(9):
    dy, dx = divmod(tap, 3)
    out += np.einsum("nhwc,oc->nhwo", xp[:, dy : dy + h, dx : dx + wd], w[:, tap, :])
  if bias is not None:
    out += bias
  if relu:
    out = np.maximum(out, 0.0)
  if mask is not None:
    out = np.where(mask > 0, out, 0.0)
  return out


def test_conv_argument_errors_without_a_gpu():
  from mujoco_warp_pbr_gb300 import _lib

  lib = _lib.load()
  c = _lib.Conv(in_=16, weight=16, out=16, nimg=1, height=8, width=24, c_in=16, c_out=16)
  assert lib.mjpbr_conv3x3_bf16(ctypes.byref(c), None) == _lib.ERR_ARG
  assert b"width 24" in lib.mjpbr_last_error()
  c = _lib.Conv(in_=16, weight=16, out=16, nimg=1, height=8, width=16, c_in=24, c_out=16)
  assert lib.mjpbr_conv3x3_bf16(ctypes.byref(c), None) == _lib.ERR_ARG
  assert b"multiples of 16" in lib.mjpbr_last_error()
  c = _lib.Conv(in_=16, weight=16, out=16, nimg=1, height=4, width=16, c_in=16, c_out=16)
  assert lib.mjpbr_conv3x3_bf16(ctypes.byref(c), None) == _lib.ERR_ARG
  assert b"height 4" in lib.mjpbr_last_error()


CASES = [
  # nimg, h, w, c1, c2, cout, bias, relu, mask
  (2, 16, 16, 16, 0, 32, False, False, False),
  (1, 8, 128, 32, 0, 48, True, True, False),
  (2, 32, 32, 32, 16, 64, True, True, False),
  (1, 4, 256, 16, 0, 16, False, False, True),
  (3, 16, 64, 48, 96, 160, True, False, True),
  (1, 16, 16, 96, 0, 256, True, True, False),
  # more tiles than one wave of persistent CTAs: weights resident (one staged row with halo) and
  # weights staged per chunk (three shifted copies of two rows)
  (40, 32, 128, 32, 16, 48, True, True, False),
  (24, 64, 64, 48, 0, 96, True, False, True),
]
# the same with a full-resolution skip input
FULL_CASES = [
  (2, 32, 32, 32, 16, 64, True, True, False),
  (3, 16, 64, 48, 96, 160, True, False, True),
  (40, 32, 128, 32, 48, 32, True, True, False),
  (2, 8, 256, 16, 32, 48, False, True, False),
]


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("nimg,h,w,c1,c2,cout,use_bias,relu,use_mask,full", [c + (False,) for c in CASES] + [c + (True,) for c in FULL_CASES])
def test_conv3x3_matches_cpu(nimg, h, w, c1, c2, cout, use_bias, relu, use_mask, full):
  from mujoco_warp_pbr_gb300 import _lib

  g = torch.Generator().manual_seed(nimg * 1000 + h * 10 + w + c1 + c2 + cout)
  x = (torch.rand((nimg, h, w, c1), generator=g) * 2 - 1).to(torch.bfloat16)
  s2 = 1 if full else 2
  x2 = (torch.rand((nimg, h // s2, w // s2, c2), generator=g) * 2 - 1).to(torch.bfloat16) if c2 else None
  wt = ((torch.rand((cout, 9, c1 + c2), generator=g) * 2 - 1) / np.sqrt(9 * (c1 + c2))).to(torch.bfloat16)
  bias = (torch.rand(cout, generator=g) - 0.5) if use_bias else None
  mask = (torch.rand((nimg, h, w, cout), generator=g) - 0.3).to(torch.bfloat16) if use_mask else None
  ref = conv_ref(
    x.float().numpy().astype(np.float64),
    wt.float().numpy().astype(np.float64),
    None if bias is None else bias.numpy().astype(np.float64),
    None if x2 is None else x2.float().numpy().astype(np.float64),
    relu,
    None if mask is None else mask.float().numpy(),
  )
  dev = {k: (v.cuda() if v is not None else None) for k, v in {"x": x, "x2": x2, "w": wt, "b": bias, "m": mask}.items()}
  out = torch.zeros((nimg, h, w, cout), dtype=torch.bfloat16, device="cuda")
  out32 = torch.zeros((nimg, h, w, cout), dtype=torch.float32, device="cuda")
  err = torch.zeros(1, dtype=torch.int32, device="cuda")

  def ptr(t):
    return t.data_ptr() if t is not None else None

  c = _lib.Conv(
    in_=ptr(dev["x"]), in2=ptr(dev["x2"]), weight=ptr(dev["w"]), bias=ptr(dev["b"]), out=ptr(out), out_f32=ptr(out32),
    mask=ptr(dev["m"]), error_word=ptr(err), nimg=nimg, height=h, width=w, c_in=c1, c_in2=c2, c_out=cout, relu=int(relu),
    in2_full=int(full),
  )
  _lib.call("mjpbr_conv3x3_bf16", ctypes.byref(c), torch.cuda.current_stream().cuda_stream)
  torch.cuda.synchronize()
  assert int(err.item()) == 0
  np.testing.assert_allclose(out32.cpu().numpy(), ref, rtol=1e-4, atol=1e-4)
  np.testing.assert_allclose(out.float().cpu().numpy(), ref, rtol=1e-2, atol=1e-2)


def wgrad_ref(x, dy, x2=None):
  if x2 is not None:
    up = x2 if x2.shape[1] == x.shape[1] else np.repeat(np.repeat(x2, 2, axis=1), 2, axis=2)
    x = np.concatenate([x, up], axis=-1)
  n, h, w, c = x.shape
  xp = np.zeros((n, h + 2, w + 2, c))
  xp[:, 1:-1, 1:-1] = x
  gw = np.zeros((dy.shape[-1], 9, c))
  for tap in range(9):
    ty, tx = divmod(tap, 3)
    gw[:, tap, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, ty : ty + h, tx : tx + w])
  return gw, dy.sum(axis=(0, 1, 2))


WGRAD_CASES = [
  # nimg, h, w, c1, c2, cout, tiles_per_cta
  (2, 16, 16, 16, 0, 32, 0),
  (1, 8, 128, 32, 0, 48, 3),
  (2, 32, 32, 32, 16, 64, 5),
  (1, 4, 256, 16, 0, 16, 1),
  (3, 16, 64, 48, 96, 96, 0),
  (40, 32, 128, 32, 0, 32, 0),
]
# the same with a full-resolution skip input
WGRAD_FULL_CASES = [
  (2, 32, 32, 32, 16, 64, 0),
  (3, 16, 64, 48, 96, 96, 0),
  (4, 16, 128, 32, 48, 32, 0),
  (2, 8, 256, 16, 32, 48, 0),
]


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("nimg,h,w,c1,c2,cout,per_cta,full", [c + (False,) for c in WGRAD_CASES] + [c + (True,) for c in WGRAD_FULL_CASES])
def test_conv3x3_wgrad_matches_cpu(nimg, h, w, c1, c2, cout, per_cta, full):
  from mujoco_warp_pbr_gb300 import _lib

  g = torch.Generator().manual_seed(nimg * 100 + h + w * 3 + c1 + c2 + cout)
  x = (torch.rand((nimg, h, w, c1), generator=g) * 2 - 1).to(torch.bfloat16)
  s2 = 1 if full else 2
  x2 = (torch.rand((nimg, h // s2, w // s2, c2), generator=g) * 2 - 1).to(torch.bfloat16) if c2 else None
  dy = (torch.rand((nimg, h, w, cout), generator=g) * 2 - 1).to(torch.bfloat16)
  ref_w, ref_b = wgrad_ref(
    x.float().numpy().astype(np.float64), dy.float().numpy().astype(np.float64), None if x2 is None else x2.float().numpy().astype(np.float64)
  )
  gw = torch.full((cout, 9, c1 + c2), 0.5, dtype=torch.float32, device="cuda")  # accumulates into existing values
  gb = torch.full((cout,), 0.25, dtype=torch.float32, device="cuda")
  err = torch.zeros(1, dtype=torch.int32, device="cuda")
  dx, dx2, ddy = x.cuda(), (x2.cuda() if x2 is not None else None), dy.cuda()
  c = _lib.ConvGrad(
    in_=dx.data_ptr(), in2=dx2.data_ptr() if dx2 is not None else None, grad_out=ddy.data_ptr(), grad_weight=gw.data_ptr(),
    grad_bias=gb.data_ptr(), error_word=err.data_ptr(), nimg=nimg, height=h, width=w, c_in=c1, c_in2=c2, c_out=cout,
    tiles_per_cta=per_cta, in2_full=int(full),
  )
  _lib.call("mjpbr_conv3x3_wgrad_bf16", ctypes.byref(c), torch.cuda.current_stream().cuda_stream)
  torch.cuda.synchronize()
  assert int(err.item()) == 0
  scale = np.sqrt(nimg * h * w)
  np.testing.assert_allclose(gw.cpu().numpy(), ref_w + 0.5, rtol=1e-4, atol=1e-4 * scale)
  np.testing.assert_allclose(gb.cpu().numpy(), ref_b + 0.25, rtol=1e-4, atol=1e-4 * scale)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_upsample2_is_nearest():
  from mujoco_warp_pbr_gb300 import _lib

  g = torch.Generator().manual_seed(5)
  x = torch.randn((3, 5, 7, 24), generator=g).to(torch.bfloat16)
  out = torch.zeros((3, 10, 14, 24), dtype=torch.bfloat16, device="cuda")
  xd = x.cuda()
  _lib.call("mjpbr_upsample2_bf16", xd.data_ptr(), out.data_ptr(), 3, 5, 7, 24, torch.cuda.current_stream().cuda_stream)
  torch.cuda.synchronize()
  ref = x.repeat_interleave(2, dim=1).repeat_interleave(2, dim=2)
  assert torch.equal(out.cpu().view(torch.int16), ref.view(torch.int16))


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("c", [24, 12])
def test_avgpool2_rounds_the_fp32_mean(c):
  """16-byte path (channels a multiple of 8) and the scalar path: bit-exact against the same sums."""
  from mujoco_warp_pbr_gb300 import _lib

  g = torch.Generator().manual_seed(c)
  x = torch.randn((3, 6, 10, c), generator=g).to(torch.bfloat16)
  out = torch.zeros((3, 3, 5, c), dtype=torch.bfloat16, device="cuda")
  xd = x.cuda()
  _lib.call("mjpbr_avgpool2_bf16", xd.data_ptr(), out.data_ptr(), 3, 6, 10, c, torch.cuda.current_stream().cuda_stream)
  torch.cuda.synchronize()
  f = x.float()
  ref = ((f[:, 0::2, 0::2] + f[:, 0::2, 1::2] + f[:, 1::2, 0::2] + f[:, 1::2, 1::2]) * 0.25).to(torch.bfloat16)
  assert torch.equal(out.cpu().view(torch.int16), ref.view(torch.int16))
