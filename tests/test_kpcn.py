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


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_gpu_forward_and_gradients_match_oracle():
  params = _params(3)
  x0, rad, tgt = _inputs(4, n=2)
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

  ref = ko.Net(params, bf16=True)
  ref_out = ref.forward(ko.round_bf16(x0), rad)
  np.testing.assert_allclose(out.cpu().numpy()[..., :3], ref_out, rtol=2e-2, atol=2e-2)
  _, gout = ko.loss(out.cpu().numpy()[..., :3].astype(np.float64), tgt)
  g = ref.backward(gout)
  for name, layer in net.layers.items():
    gw = layer.gw.cpu().numpy()
    gb = layer.gb.cpu().numpy()
    rw, rb = g[name]
    err_w = np.linalg.norm(gw - rw) / max(np.linalg.norm(rw), 1e-12)
    err_b = np.linalg.norm(gb - rb) / max(np.linalg.norm(rb), 1e-12)
    assert err_w < 0.05, f"{name}: weight gradient relative error {err_w:.3g}"
    assert err_b < 0.05 or np.linalg.norm(rb) < 1e-9, f"{name}: bias gradient relative error {err_b:.3g}"


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
