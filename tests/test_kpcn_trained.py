"""What the trained denoiser gains: on a held-out path-traced frame (a scene seed the training
never saw), the committed weights at 2 spp against a converged reference, compared with the
a-trous filter at the same 2 spp (the method without the network), with plain path tracing, and
with the a-trous filter at 16 spp."""

import pytest

torch = pytest.importorskip("torch")

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]


def test_trained_network_beats_the_filter_without_it():
  from pathlib import Path

  from mujoco_warp_pbr_gb300 import kpcn, train_kpcn

  weights = Path(kpcn.__file__).resolve().parent / "weights" / "kpcn_path.npz"
  net = kpcn.KPCN.load(weights)
  ev = train_kpcn.evaluate(net, nworld=32, res=128, ref_spp=2048, seed=9100)
  learned, atrous2, plain2, atrous16 = (ev[k]["rel_mse"] for k in ("learned_2spp", "atrous_2spp", "plain_2spp", "atrous_16spp"))
  assert int(net.error.item()) == 0
  assert learned < 0.5 * atrous2, ev
  assert learned < 0.1 * plain2, ev
  assert learned < 1.1 * atrous16, ev
