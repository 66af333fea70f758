"""Learned denoiser: the NumPy restatement pinned by finite differences, then the GPU network's
forward output and every layer's weight / bias gradients against it (same BF16 weights and
activation rounding), and a short training run whose loss must fall."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mujoco_warp_pbr_gb300 import kpcn  # noqa: E402
from oracle import kpcn_oracle as ko  # noqa: E402

GPU = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]


def _params(seed=0):
  rng = np.random.default_rng(seed)
  params = {}
  for s in kpcn.layer_specs():
    cin = s.c_in + s.c_in2
    w = rng.normal(0, np.sqrt(2 / (9 * cin)), (s.c_out, 9, cin))
    if s.name == "head":
      w *= 0.3
      w[kpcn.TAPS :] = 0.0
    params[s.name] = (w, rng.normal(0, 0.05, s.c_out))
  return params


def _inputs(seed=1, n=1, h=64, w=128):
  rng = np.random.default_rng(seed)
  x0 = rng.uniform(0, 1, (n, h, w, kpcn.FEATURES))
  x0[..., 10:] = 0.0
  rad = np.concatenate([rng.uniform(0, 2, (n, h, w, 3)), np.zeros((n, h, w, 1))], -1)
  tgt = np.concatenate([rng.uniform(0, 2, (n, h, w, 3)), np.zeros((n, h, w, 1))], -1)
  return x0, rad, tgt


def test_supported_sizes():
  assert kpcn.supported(128, 128) and kpcn.supported(256, 256) and kpcn.supported(128, 64)
  assert not kpcn.supported(64, 64) and not kpcn.supported(96, 96) and not kpcn.supported(128, 32)


def test_oracle_gradients_match_finite_differences():
  params = _params()
  x0, rad, tgt = _inputs()
  net = ko.Net(params, bf16=False)
  # the relative-MSE term alone: smooth (the L1 term's kink would break finite differences)
  _, gout = ko.loss(net.forward(x0, rad), tgt, w_l1=0.0)
  g = net.backward(gout)
  for name, idx in [("e0a", (3, 4, 2)), ("e2b", (1, 7, 33)), ("d1a", (5, 0, 60)), ("e3b", (10, 8, 90)), ("head", (7, 4, 11))]:
    w, b = params[name]
    eps = 1e-6  # small: ReLU kinks of the many pre-activations a first-layer weight moves
    vals = []
    for sign in (1, -1):
      wp = w.copy()
      wp[idx] += sign * eps
      p2 = dict(params)
      p2[name] = (wp, b)
      vals.append(ko.loss(ko.Net(p2, bf16=False).forward(x0, rad), tgt, w_l1=0.0)[0])
    np.testing.assert_allclose((vals[0] - vals[1]) / (2 * eps), g[name][0][idx], rtol=1e-3, atol=1e-9)
  # a bias
  w, b = params["d0b"]
  bp, bm = b.copy(), b.copy()
  bp[3] += 1e-5
  bm[3] -= 1e-5
  lp = ko.loss(ko.Net({**params, "d0b": (w, bp)}, bf16=False).forward(x0, rad), tgt, w_l1=0.0)[0]
  lm = ko.loss(ko.Net({**params, "d0b": (w, bm)}, bf16=False).forward(x0, rad), tgt, w_l1=0.0)[0]
  np.testing.assert_allclose((lp - lm) / 2e-5, g["d0b"][1][3], rtol=1e-4, atol=1e-9)


def _gpu_net(params):
  net = kpcn.KPCN("cuda")
  net.load_state_dict({**{f"{k}.w": v[0].astype(np.float32) for k, v in params.items()}, **{f"{k}.b": v[1].astype(np.float32) for k, v in params.items()}})
  return net


# (layer, forward inputs, incoming gradient, outgoing gradient, ReLU mask of the outgoing one)
BACKWARD_CHAIN = [
  ("head", ("v0",), "dlogits", "dv0", "v0"),
  ("d0b", ("u0",), "dv0", "du0", "u0"),
  ("d0a", ("s0", "v1"), "du0", "dcat0", None),
  ("d1b", ("u1",), "dv1", "du1", "u1"),
  ("d1a", ("s1", "v2"), "du1", "dcat1", None),
  ("d2b", ("u2",), "dv2", "du2", "u2"),
  ("d2a", ("s2", "b3"), "du2", "dcat2", None),
  ("e3b", ("a3",), "db3", "da3", "a3"),
  ("e3a", ("p3",), "da3", "dp3", None),
  ("e2b", ("a2",), "ds2", "da2", "a2"),
  ("e2a", ("p2",), "da2", "dp2", None),
  ("e1b", ("a1",), "ds1", "da1", "a1"),
  ("e1a", ("p1",), "da1", "dp1", None),
  ("e0b", ("a0",), "ds0", "da0", "a0"),
  ("e0a", ("x0",), "da0", None, None),
]


def _gpu_step(params, n=2):
  x0, rad, tgt = _inputs(4, n=n)
  net = _gpu_net(params)
  x0_d = torch.as_tensor(x0, dtype=torch.float32).to(torch.bfloat16).cuda()
  rad_d = torch.as_tensor(rad, dtype=torch.float32).cuda()
  tgt_d = torch.as_tensor(tgt, dtype=torch.float32).cuda()
  net.zero_grad()
  out = net.forward(x0_d, rad_d, train=True)
  net.loss_grad(tgt_d)
  net.backward(x0_d, rad_d)
  torch.cuda.synchronize()
  assert int(net.error.item()) == 0
  ws = {k: v.float().cpu().numpy().astype(np.float64) for k, v in net.workspace(n, 64, 128).items()}
  ws["x0"] = x0_d.float().cpu().numpy().astype(np.float64)
  return net, ws, out.cpu().numpy(), (x0, rad, tgt)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_gpu_backward_steps_match_oracle_on_their_own_inputs():
  """Every backward operation of the GPU network, recomputed in float64 from the tensors the GPU
  itself fed it: weight and bias gradients (tensor-core wgrad), input gradients (tensor-core
  dgrad), their ReLU masks and BF16 rounding, the skip / pooling gradient routing and the kernel
  softmax backward."""
  params = _params(3)
  net, ws, _, (_, rad, _) = _gpu_step(params)
  # kernel softmax backward
  lg = ws["logits"][..., : kpcn.TAPS]
  e = np.exp(lg - lg.max(-1, keepdims=True))
  wts = e / e.sum(-1, keepdims=True)
  _, _, taps = ko.apply_kernel(ws["logits"], rad)
  gk = np.stack([np.sum(ws["gout"][..., :3] * t, -1) for t in taps], -1)
  dlog = wts * (gk - np.sum(wts * gk, -1, keepdims=True))
  np.testing.assert_allclose(ws["dlogits"][..., : kpcn.TAPS], ko.round_bf16(dlog), rtol=1e-2, atol=1e-2 * np.abs(dlog).max())
  for name, ins, dy, dx_name, mask in BACKWARD_CHAIN:
    x = ws[ins[0]] if len(ins) == 1 else np.concatenate([ws[ins[0]], ko.up(ws[ins[1]])], -1)
    dx, dw, db = ko.conv_backward(x, ko.round_bf16(params[name][0]), ws[dy])
    layer = net.layers[name]
    for got, ref, what in ((layer.gw.cpu().numpy(), dw, "weight"), (layer.gb.cpu().numpy(), db, "bias")):
      err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-12)
      assert err < 2e-3, f"{name}: {what} gradient relative error {err:.3g} on the GPU's own inputs"
    if dx_name is None:
      continue
    if mask is not None:
      ref = ko.round_bf16(dx * (ws[mask] > 0))
      np.testing.assert_allclose(ws[dx_name], ref, rtol=2e-2, atol=1e-2 * np.abs(ref).max(), err_msg=name)
    else:
      np.testing.assert_allclose(ws[dx_name], dx, rtol=1e-3, atol=1e-4 * np.abs(dx).max(), err_msg=name)
  # gradient routing through the concatenations and poolings
  for dcat, skip, low, dskip, dlow in (("dcat0", "s0", "v1", "dskip0", "dv1"), ("dcat1", "s1", "v2", "dskip1", "dv2"), ("dcat2", "s2", "b3", "dskip2", "db3")):
    c1 = ws[skip].shape[-1]
    np.testing.assert_array_equal(ws[dskip], ws[dcat][..., :c1])
    ref = ko.round_bf16(ko.pool(ws[dcat][..., c1:]) * 4.0 * (ws[low] > 0))
    np.testing.assert_allclose(ws[dlow], ref, rtol=1e-2, atol=1e-3 * np.abs(ref).max())
  for dskip, dp, act, out in (("dskip2", "dp3", "s2", "ds2"), ("dskip1", "dp2", "s1", "ds1"), ("dskip0", "dp1", "s0", "ds0")):
    ref = ko.round_bf16((ws[dskip] + ko.up(ws[dp]) * 0.25) * (ws[act] > 0))
    np.testing.assert_allclose(ws[out], ref, rtol=1e-2, atol=1e-3 * np.abs(ref).max())


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_gpu_forward_and_gradients_match_oracle():
  """End to end against the float64 oracle with the same BF16 weights and storage points: the
  output within BF16 precision, every layer's gradient pointing the same way (cosine similarity;
  BF16 rounding differences compound through the 15 layers, so elementwise equality is not
  expected)."""
  params = _params(3)
  net, ws, out, (x0, rad, tgt) = _gpu_step(params)
  ref = ko.Net(params, bf16=True)
  ref_out = ref.forward(ko.round_bf16(x0), rad)
  np.testing.assert_allclose(out[..., :3], ref_out, rtol=2e-2, atol=2e-2)
  _, gout = ko.loss(out[..., :3].astype(np.float64), tgt)
  g = ref.backward(gout)
  for name, layer in net.layers.items():
    gw = layer.gw.cpu().numpy().ravel()
    rw = g[name][0].ravel()
    cos = float(gw @ rw / (np.linalg.norm(gw) * np.linalg.norm(rw)))
    ratio = float(np.linalg.norm(gw) / np.linalg.norm(rw))
    assert cos > 0.95 and 0.8 < ratio < 1.25, f"{name}: cosine {cos:.4f}, norm ratio {ratio:.3f}"


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_training_reduces_the_loss():
  """Denoising a smooth signal under heavy noise: the loss after 150 Adam steps is well below the
  first."""
  g = torch.Generator().manual_seed(0)
  n, h, w = 4, 64, 128
  yy, xx = torch.meshgrid(torch.linspace(0, 3, h), torch.linspace(0, 6, w), indexing="ij")
  clean = torch.stack([0.6 + 0.4 * torch.sin(xx + k) * torch.cos(yy) for k in range(3)], -1).expand(n, h, w, 3)
  noisy = clean * (torch.rand((n, h, w, 3), generator=g) * 2)
  x0 = torch.zeros((n, h, w, kpcn.FEATURES))
  x0[..., :3] = torch.log1p(noisy)
  x0[..., 3:6] = 1.0
  x0[..., 8] = 1.0
  rad = torch.cat([noisy, torch.zeros((n, h, w, 1))], -1).cuda()
  tgt = torch.cat([clean, torch.zeros((n, h, w, 1))], -1).contiguous().cuda()
  x0 = x0.to(torch.bfloat16).cuda()
  net = kpcn.KPCN("cuda", seed=1)
  losses = []
  for _ in range(150):
    sums = net.train_step(x0, rad, tgt, lr=2e-3)
    losses.append(float(sums.sum().item()))
  assert int(net.error.item()) == 0
  assert np.mean(losses[-10:]) < 0.6 * losses[0], f"loss {losses[0]:.4g} -> {np.mean(losses[-10:]):.4g}"
