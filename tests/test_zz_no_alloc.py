"""mjpbr_refit_render_static: refit + render for callers that cannot allocate device memory after
start-up (a host that runs inside a fixed device-memory arena, or a plugin whose host owns every
allocation). The call keeps the per-world blocks and the work counter in the library's own static
device memory; the test calls it through the C ABI and compares it with the allocating entry
points on the same scene, twice in a row.

The caller's own world blocks are filled with NaN and both scratch pointers are left out of the
descriptor before the static call, so the images can only match if the static memory is what the
kernels read. The queue schedule of the real-time tier (work counter slot 1) and the path tier
(slot 0) both run through it; a context on the wavefront schedule (whose ray queues live in
caller scratch) renders through it with the grid schedule, to the same images.

Collected last (file name) so it also runs after every other GPU test in one process."""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]


def _outputs(rc):
  return (
    rc.base.rgb_data.cpu().numpy().copy(),
    rc.base.depth_data.cpu().numpy().copy(),
    rc.base.seg_data.cpu().numpy().copy(),
  )


@pytest.mark.parametrize(
  "opts",
  [
    {"schedule": "grid"},
    {"schedule": "queue", "queue_item": 64},
    {"schedule": "wavefront"},
    {"tier": 1, "path_samples": 3, "max_depth": 3},
  ],
  ids=["realtime_grid", "realtime_queue", "realtime_wavefront", "path"],
)
def test_static_scratch_matches_allocating_path(opts):
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib, synthetic
  from tests import helpers

  sc = synthetic.primitive_scene(seed=4, nworld=6, res=40)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=5)
  torch.cuda.synchronize()
  ref = _outputs(rc)
  lib = _lib.load()
  s = _lib.Scene.from_buffer_copy(mjpbr.scene_descriptor(m, d, rc))  # a copy: the cached one stays intact
  s.world_blocks = None
  s.work_counter = None
  stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
  for _ in range(2):
    rc.world_blocks.fill_(float("nan"))
    rc.work_counter.fill_(12345)
    for t in (rc.base.rgb_data, rc.base.depth_data, rc.base.seg_data):
      t.zero_()
    torch.cuda.synchronize()
    assert lib.mjpbr_refit_render_static(ctypes.byref(s), 5, stream) == 0, lib.mjpbr_last_error().decode()
    torch.cuda.synchronize()
    got = _outputs(rc)
    for a, b in zip(got, ref):
      np.testing.assert_array_equal(a, b)
    # the caller's scratch was not touched
    assert bool(torch.isnan(rc.world_blocks).all())
    assert bool((rc.work_counter == 12345).all())
  assert mjpbr.check_errors(rc) == 0


def test_static_scratch_rejects_oversized_scenes():
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib, synthetic
  from tests import helpers

  sc = synthetic.primitive_scene(seed=1, nworld=2, res=8)
  m, d, rc = helpers.gpu_scene(sc)
  s = mjpbr.scene_descriptor(m, d, rc)
  big = _lib.Scene.from_buffer_copy(s)
  big.nworld = (4 << 20) // s.world_block_floats + 1
  lib = _lib.load()
  assert lib.mjpbr_refit_render_static(ctypes.byref(big), 0, None) == _lib.ERR_ARG
  assert b"static scratch holds" in lib.mjpbr_last_error()
