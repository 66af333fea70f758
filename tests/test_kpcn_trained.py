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
  # throughput on the path-traced configuration's own batch (1024 worlds x 128x128): at a quarter of
  # it the fixed costs of the network's 25 launches per chunk weigh more than the path tracer's
  ev = train_kpcn.evaluate(net, nworld=32, res=128, ref_spp=2048, seed=9100, time_worlds=1024)
  learned, atrous2, plain2, atrous16 = (ev[k]["rel_mse"] for k in ("learned_2spp", "atrous_2spp", "plain_2spp", "atrous_16spp"))
  speedup = ev["speedup_learned2_vs_atrous16"]
  print(f"relMSE learned 2 spp {learned:.4f}, a-trous 16 spp {atrous16:.4f}, a-trous 2 spp {atrous2:.4f}, plain 2 spp {plain2:.4f}; "
        f"learned 2 spp {ev['learned_2spp']['mpix_s']:.1f} Mpix/s vs a-trous 16 spp {ev['atrous_16spp']['mpix_s']:.1f} ({speedup:.2f}x)")
  assert int(net.error.item()) == 0
  assert learned < 0.5 * atrous2, ev
  assert learned < 0.1 * plain2, ev
  # the target: learned at 2 spp no worse than a-trous at 16 spp, at >= 4x its pixel rate
  # (render + denoise of 1024 worlds x 128x128 each, CUDA events)
  assert learned <= atrous16, ev
  assert speedup >= 4.0, ev


def test_learned_denoiser_in_a_captured_frame_matches_eager():
  """The learned denoiser captured with the frame (capture_frame(..., denoiser=...)) replays to
  the eager images; worlds processed in chunks give the same images as one batch."""
  from pathlib import Path

  import numpy as np

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import kpcn, synthetic

  sc = synthetic.path_scene(seed=77, nworld=6, res=128, spp=2)
  m = mjpbr.put_model(sc.mjm)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, **{**sc.options, "denoise": True})
  synthetic.apply_per_world(sc, m, rc)
  net = kpcn.KPCN.load(Path(kpcn.__file__).resolve().parent / "weights" / "kpcn_path.npz")
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=4, denoise=False)
  net.denoise(m, d, rc)
  torch.cuda.synchronize()
  eager = rc.base.rgb_data.cpu().numpy().copy()
  mjpbr.render(m, d, rc, seed=4, denoise=False)
  net.denoise(m, d, rc, chunk=4)
  torch.cuda.synchronize()
  np.testing.assert_array_equal(rc.base.rgb_data.cpu().numpy(), eager)
  graph = mjpbr.capture_frame(m, d, rc, seed=4, denoiser=lambda: net.denoise(m, d, rc))
  rc.base.rgb_data.zero_()
  graph.replay()
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0 and int(net.error.item()) == 0
  np.testing.assert_array_equal(rc.base.rgb_data.cpu().numpy(), eager)
