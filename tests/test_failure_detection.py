"""Failure detection without a GPU fault.

* Host side, no GPU: descriptors whose pixel maps (camera images placed past their output rows or
  past the per-world ray range, 32-bit ray-index overflow) or work-queue settings (item sizes the
  queue schedule cannot tile) were corrupted are rejected by the library before any launch, with
  ERR_ARG and a message naming the map.
* GPU: the library's bounded device waits (the mbarrier waits of the tensor-core kernels) give up
  after their poll limit on a barrier that nothing completes, release the other waiting roles
  through the CTA's abort flag, report kErrWaitTimeout in the error word, and leave the context
  usable (mjpbr_wait_probe).
* The autotuner skips launch shapes whose launch fails or whose warm-up frame exceeds its time
  budget on the host, and keeps a shape that renders.
"""

import ctypes

import numpy as np
import pytest

from mujoco_warp_pbr_gb300 import _lib

torch = pytest.importorskip("torch")

FAKE = 0x10000  # a 16-byte aligned stand-in address: validation never dereferences pointers


def _host_scene() -> _lib.Scene:
  """A descriptor that passes validation (two cameras of 8 x 4 and 4 x 4 pixels, three worlds),
  with stand-in addresses instead of device buffers."""
  lib = _lib.load()
  s = _lib.Scene()
  s.abi_version = _lib.ABI_VERSION
  s.nworld, s.ngeom, s.nmat, s.nlight, s.ncam, s.nrender = 3, 2, 1, 0, 2, 2
  s.nbvh_geom, s.nnode = 2, 1
  s.world_block_floats = lib.mjpbr_world_block_floats(2, 1, 0, 2)
  for name in ("geom_type", "geom_xpos", "geom_xmat", "cam_xpos", "cam_xmat", "enabled_geom_ids", "world_blocks", "dfg_lut",
               "rgb_data", "depth_data", "seg_data", "error_word", "work_counter"):
    setattr(s, name, FAKE)
  for name in ("tlas_child", "geom_size", "geom_rgba", "geom_matid", "exposure", "ambient_radiance", "geom_metallic",
               "geom_roughness", "geom_reflectance"):
    b = getattr(s, name)
    b.ptr, b.nbatch = FAKE, 1
  s.dfg_size = 128
  res = [(8, 4), (4, 4)]
  for c, (w, h) in enumerate(res):
    s.cam_res[c][0], s.cam_res[c][1] = w, h
    s.cam_id_map[c] = c
    s.render_rgb[c] = s.render_depth[c] = 1
    s.render_seg[c] = 0
  s.ray_adr[0], s.ray_adr[1] = 0, 32
  s.rgb_adr[0], s.rgb_adr[1] = 0, 32
  s.depth_adr[0], s.depth_adr[1] = 0, 32
  s.seg_adr[0] = s.seg_adr[1] = -1
  s.total_rays = s.rgb_stride = s.depth_stride = 48
  s.seg_stride = 1
  st = s.settings
  st.samples_per_axis = st.shadow_samples = st.max_layers = 1
  st.schedule, st.queue_item = 1, 64
  return s


def _expect_rejected(s, fragment: bytes):
  lib = _lib.load()
  assert lib.mjpbr_render(ctypes.byref(s), 0, None) == _lib.ERR_ARG
  assert fragment in lib.mjpbr_last_error(), lib.mjpbr_last_error()


def test_a_valid_host_descriptor_passes_validation():
  """The uncorrupted descriptor gets past validation: without a GPU the call then fails at its
  first CUDA call (ERR_CUDA), not at the argument checks."""
  if torch.cuda.is_available():
    pytest.skip("with a GPU the stand-in addresses would reach a kernel")
  lib = _lib.load()
  status = lib.mjpbr_render(ctypes.byref(_host_scene()), 0, None)
  assert status != _lib.ERR_ARG, lib.mjpbr_last_error()


@pytest.mark.parametrize(
  "corrupt,fragment",
  [
    (lambda s: setattr(s, "rgb_stride", 40), b"rgb pixels"),  # camera 1's image past the row
    (lambda s: s.depth_adr.__setitem__(1, 40), b"depth pixels"),
    (lambda s: s.ray_adr.__setitem__(1, 40), b"outside total_rays"),
    (lambda s: s.ray_adr.__setitem__(0, -8), b"outside total_rays"),
    (lambda s: setattr(s, "total_rays", 40), b"outside total_rays"),
    (lambda s: (setattr(s, "total_rays", 1 << 20), setattr(s, "nworld", 4096)), b"overflow the 32-bit ray index"),
    (lambda s: setattr(s.settings, "queue_item", 48), b"work queue"),
    (lambda s: setattr(s, "wave_scratch_bytes", -1), b"wave_scratch_bytes"),
    (lambda s: setattr(s.settings, "schedule", 7), b"settings.schedule"),
    (lambda s: setattr(s.settings, "stack_depth", 33), b"settings.stack_depth"),
    (lambda s: setattr(s.settings, "stack_depth", 4), b"settings.stack_depth"),
  ],
)
def test_corrupted_pixel_maps_and_queues_are_rejected_before_launch(corrupt, fragment):
  s = _host_scene()
  corrupt(s)
  _expect_rejected(s, fragment)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("polls", [300, 4096])
def test_bounded_device_waits_give_up_and_report(polls):
  import time

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  words = torch.zeros(2, dtype=torch.int32, device="cuda")
  stream = torch.cuda.current_stream().cuda_stream
  t0 = time.perf_counter()
  _lib.call("mjpbr_wait_probe", polls, words[0:1].data_ptr(), words[1:2].data_ptr(), stream)
  torch.cuda.synchronize()
  elapsed = time.perf_counter() - t0
  error_word, roles_done = (int(v) for v in words.cpu())
  assert error_word & 4, "kErrWaitTimeout not reported"
  assert roles_done == 3, "a waiting role did not return"
  assert elapsed < 5.0
  # the context is still usable: a frame renders and matches the oracle's segmentation
  sc = synthetic.primitive_scene(seed=1, nworld=2, res=16)
  m, d, rc = helpers.gpu_scene(sc)
  gpu = helpers.render_gpu(m, d, rc, seed=2)
  ref = helpers.oracle_render(sc, seed=2, tables=helpers.gpu_tables(rc))
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  assert mjpbr.check_errors(rc) == 0


def test_wait_probe_rejects_bad_arguments_without_a_gpu():
  lib = _lib.load()
  assert lib.mjpbr_wait_probe(0, FAKE, FAKE, None) == _lib.ERR_ARG
  assert lib.mjpbr_wait_probe(1 << 21, FAKE, FAKE, None) == _lib.ERR_ARG
  assert lib.mjpbr_wait_probe(10, None, FAKE, None) == _lib.ERR_ARG


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_autotuner_skips_shapes_that_fail_or_run_too_long(monkeypatch):
  import importlib

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  autotune = importlib.import_module("mujoco_warp_pbr_gb300.autotune")  # the module (the package exports the function)
  sc = synthetic.primitive_scene(seed=2, nworld=4, res=24)
  m, d, rc = helpers.gpu_scene(sc)
  for shape in autotune.CANDIDATES:  # load every kernel once, outside the timed warm-up frames
    if shape.schedule != autotune.QUEUE:
      autotune.apply(rc, shape)
      helpers.render_gpu(m, d, rc)
  real = autotune.render
  calls = {"n": 0}

  def flaky(m_, d_, rc_, seed=0, denoise=True):
    calls["n"] += 1
    if rc_.schedule == autotune.QUEUE:
      raise _lib.MjpbrError("mjpbr_render: injected launch failure (status 2)")
    if rc_.schedule == autotune.GRID and rc_.render_order == autotune.ROW:
      import time

      time.sleep(0.5)  # a slow warm-up frame on the host clock
    return real(m_, d_, rc_, seed=seed, denoise=denoise)

  monkeypatch.setattr(autotune, "render", flaky)
  result = mjpbr.autotune(m, d, rc, frames=1, use_cache=False, timeout_ms=250.0)
  skipped = result["skipped"]
  assert any(k.startswith("queue") and "injected" in v for k, v in skipped.items())
  assert "grid 32x8" in skipped and "warm-up frame took" in skipped["grid 32x8"]
  assert result["best"] in result["ms"] and not result["best"].startswith("queue")
