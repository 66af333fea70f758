"""The counting build of the real-time kernels (libmjpbr_count.so, the instrument behind the bench's
FP32 roofline): it renders the same image as the product library and its counts are consistent
with the frame (one closest-hit query per primary sample at least, shading per hit)."""

import ctypes

import pytest

torch = pytest.importorskip("torch")


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_counting_build_renders_the_same_frame_and_counts_it():
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib
  from mujoco_warp_pbr_gb300 import roofline
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.mesh_ibl_scene(seed=3, nworld=4, res=32)
  m = mjpbr.put_model(sc.mjm)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, **sc.options)
  synthetic.apply_per_world(sc, m, rc)
  stream = torch.cuda.current_stream().cuda_stream
  scene = mjpbr.scene_descriptor(m, d, rc)
  _lib.call("mjpbr_refit_bvh", scene, stream)
  _lib.call("mjpbr_render", scene, 77, stream)
  torch.cuda.synchronize()
  rgb = rc.base.rgb_data.clone()
  seg = rc.base.seg_data.clone()
  counts = roofline.count_frame(scene, 77, stream)
  assert torch.equal(rc.base.rgb_data, rgb) and torch.equal(rc.base.seg_data, seg)
  assert mjpbr.check_errors(rc) == 0
  npix = sc.nworld * 32 * 32
  spp = rc.samples_per_pixel**2  # the option counts supersamples per axis
  assert counts["ray_closest"] >= npix * spp
  assert counts["box"] > 0 and counts["triangle"] > 0
  assert 0 < counts["shade"] <= counts["ray_closest"]
  assert counts["env"] == counts["shade"]  # every shaded hit of this scene takes the IBL terms
  assert roofline.flops(counts) > 0 and roofline.rays(counts) >= counts["ray_closest"]
  # the counts are reproducible
  assert roofline.count_frame(scene, 77, stream) == counts


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_counting_build_counts_the_path_tracer():
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib
  from mujoco_warp_pbr_gb300 import roofline
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.path_scene(seed=2, nworld=4, res=32, spp=2)
  m = mjpbr.put_model(sc.mjm)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, **sc.options)
  synthetic.apply_per_world(sc, m, rc)
  stream = torch.cuda.current_stream().cuda_stream
  scene = mjpbr.scene_descriptor(m, d, rc)
  _lib.call("mjpbr_refit_bvh", scene, stream)
  _lib.call("mjpbr_render", scene, 5, stream)
  torch.cuda.synchronize()
  rgb = rc.base.rgb_data.clone()
  counts = roofline.count_frame(scene, 5, stream)
  assert torch.equal(rc.base.rgb_data, rgb)
  npix = sc.nworld * 32 * 32
  # every sample starts with a camera ray; every vertex is a closest hit
  assert counts["ray_closest"] >= npix * 2
  assert 0 < counts["pt_vertex"] <= counts["ray_closest"]
  assert counts["pt_light"] > 0 and counts["shade"] == 0
