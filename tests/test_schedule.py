"""Real-time tier schedules (grid of tiles, persistent warp work queue), the autotuner, CUDA-graph
capture of a frame, and the batched uneven workload (several cameras of different sizes, a
fisheye ray bundle, per-world enable masks) against the oracle."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

GPU = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]


def test_schedule_options_are_validated():
  from mujoco_warp_pbr_gb300 import context, synthetic

  sc = synthetic.primitive_scene(seed=0, nworld=1, res=8)
  with pytest.raises(ValueError, match="schedule must be"):
    context.prepare_context(sc.mjm, 1, schedule="fastest")
  with pytest.raises(ValueError, match="queue_item must be"):
    context.prepare_context(sc.mjm, 1, queue_item=48)
  hc = context.prepare_context(sc.mjm, 1, schedule="queue", queue_item=128)
  assert hc.options["schedule"] == 1 and hc.options["queue_item"] == 128


def test_batched_scene_masks_and_cameras():
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.batched_scene(seed=3, nworld=64, res=(16, 32, 48))
  visible = (sc.per_world["geom_rgba"][:, 1:, 3] > 0).sum(1)
  assert visible.min() >= 2 and visible.max() <= 16 and len(np.unique(visible)) > 8
  assert [tuple(r) for r in sc.options["cam_res"]] == [(16, 16), (32, 32), (48, 48)]
  fisheye = sc.options["camera_rays"][2]
  assert (np.linalg.norm(fisheye[..., 1, :], axis=-1) == 0).any()


def _outputs(rc):
  return (
    rc.base.rgb_data.cpu().numpy().view(np.uint32).copy(),
    rc.base.depth_data.cpu().numpy().copy(),
    rc.base.seg_data.cpu().numpy().copy(),
  )


def _frame(m, d, rc, seed=3):
  import mujoco_warp_pbr_gb300 as mjpbr

  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=seed)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  return _outputs(rc)


def _scenes():
  from mujoco_warp_pbr_gb300 import synthetic

  return {
    "primitives": synthetic.primitive_scene(seed=2, nworld=5, res=40),
    "mesh_ibl": synthetic.mesh_ibl_scene(seed=1, nworld=3, res=40, tex_size=64, env_width=128),
    "batched": synthetic.batched_scene(seed=1, nworld=5, res=(16, 40, 72)),
  }


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("name", ["primitives", "mesh_ibl", "batched"])
def test_queue_schedule_renders_the_grid_images(name):
  from tests import helpers

  sc = _scenes()[name]
  m, d, rc = helpers.gpu_scene(sc, schedule="grid")
  ref = _frame(m, d, rc)
  for item in (32, 64, 128):
    rc.schedule, rc.queue_item = 1, item
    got = _frame(m, d, rc)
    for a, b in zip(got, ref):
      np.testing.assert_array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_batched_scene_matches_oracle():
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.batched_scene(seed=4, nworld=4, res=(16, 40, 72))
  m, d, rc = helpers.gpu_scene(sc, schedule="queue")
  gpu = helpers.render_gpu(m, d, rc, seed=6)
  ref = helpers.oracle_render(sc, seed=6, tables=helpers.gpu_tables(rc))
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  assert diff.max() <= 1, f"max RGB difference {diff.max()}/255"


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_autotune_picks_a_shape_that_renders_the_same_image():
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.batched_scene(seed=2, nworld=16, res=(16, 32, 64))
  m, d, rc = helpers.gpu_scene(sc)
  ref = _frame(m, d, rc)
  result = mjpbr.autotune(m, d, rc, frames=2, use_cache=False)
  assert result["best"] in result["ms"] and len(result["ms"]) >= 3
  got = _frame(m, d, rc)
  for a, b in zip(got, ref):
    np.testing.assert_array_equal(a, b)
  again = mjpbr.autotune(m, d, rc)
  assert again.get("cached") and again["best"] == result["best"]


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize(
  "opts",
  [{"schedule": "queue"}, {"schedule": "wavefront"}, {"tier": 1, "path_samples": 2, "max_depth": 2, "denoise": True}],
  ids=["queue", "wavefront", "path"],
)
def test_captured_frame_replays_the_eager_frame(opts):
  """A graph of step (a copy of the next poses) -> refit -> render (-> denoise) replays to the
  images the eager calls render for those poses."""
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.primitive_scene(seed=5, nworld=4, res=32)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  poses_a = d.geom_xpos.clone()
  poses_b = poses_a.clone()
  poses_b[:, 1:, 2] += 0.05
  d.geom_xpos.copy_(poses_b)
  eager = _frame(m, d, rc, seed=9)
  d.geom_xpos.copy_(poses_a)
  graph = mjpbr.capture_frame(m, d, rc, seed=9, step=lambda: d.geom_xpos.copy_(poses_b))
  for t in (rc.base.rgb_data, rc.base.depth_data, rc.base.seg_data):
    t.zero_()
  d.geom_xpos.copy_(poses_a)
  graph.replay()
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  for a, b in zip(_outputs(rc), eager):
    np.testing.assert_array_equal(a, b)


def test_sample_lane_tiles_cover_each_pixel_once():
  """The real-time grid kernel's 2 x 2 sample-lane mapping (csrc/render_rt.cu, rt_kernel): over a
  CTA's 4 passes, 8 warps x 32 lanes visit every pixel of a ROW (32 x 8) or TILED (16 x 16) tile
  exactly four times, once per sample, and a pixel's four samples sit on four consecutive lanes
  of one warp (the shuffle reduction's assumption)."""
  from collections import defaultdict

  for row in (True, False):
    seen = defaultdict(list)
    for q in range(4):
      for warp in range(8):
        for lane in range(32):
          pix, smp = lane >> 2, lane & 3
          if row:
            px, py = warp * 4 + (pix & 3), q * 2 + (pix >> 2)
          else:
            px, py = (q & 1) * 8 + (warp & 1) * 4 + (pix & 3), (q >> 1) * 8 + (warp >> 1) * 2 + (pix >> 2)
          seen[(px, py)].append((q, warp, lane, smp))
    w, h = (32, 8) if row else (16, 16)
    assert set(seen) == {(x, y) for x in range(w) for y in range(h)}
    for visits in seen.values():
      assert sorted(v[3] for v in visits) == [0, 1, 2, 3]
      q, warp, lane0 = visits[0][0], visits[0][1], min(v[2] for v in visits)
      assert all(v[0] == q and v[1] == warp for v in visits) and lane0 % 4 == 0
      assert sorted(v[2] for v in visits) == [lane0, lane0 + 1, lane0 + 2, lane0 + 3]
