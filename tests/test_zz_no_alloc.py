"""mjpbr_refit_render_static: refit + render with library-owned static scratch (no allocation),
called through the C ABI and compared with the allocating entry points on the same scene.

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


@pytest.mark.parametrize("tier", [0, 1])
def test_static_scratch_matches_allocating_path(tier):
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib, synthetic
  from tests import helpers

  sc = synthetic.primitive_scene(seed=4, nworld=6, res=40)
  opts = {"tier": tier, "path_samples": 3, "max_depth": 3} if tier == 1 else {}
  m, d, rc = helpers.gpu_scene(sc, **opts)
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=5)
  torch.cuda.synchronize()
  ref = _outputs(rc)
  lib = _lib.load()
  s = mjpbr.scene_descriptor(m, d, rc)
  stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
  for _ in range(2):
    for t in (rc.base.rgb_data, rc.base.depth_data, rc.base.seg_data):
      t.zero_()
    assert lib.mjpbr_refit_render_static(ctypes.byref(s), 5, stream) == 0, lib.mjpbr_last_error().decode()
    torch.cuda.synchronize()
    got = _outputs(rc)
    for a, b in zip(got, ref):
      np.testing.assert_array_equal(a, b)
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
