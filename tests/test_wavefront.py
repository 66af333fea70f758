"""The real-time tier's staged wavefront schedule (primary, surface, mirror, shadow and shading
kernels over compacted ray queues): the same images as the megakernel's grid schedule, bit for
bit, on every workload shape (meshes / textures / IBL / mirror floor, soft shadows over two
lights, ragged and depth-only cameras, fisheye ray bundles, enable masks), for every chunking of
the worlds, and against the oracle at the real-time bars."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_wavefront_schedule_option():
  from mujoco_warp_pbr_gb300 import context, synthetic

  sc = synthetic.primitive_scene(seed=0, nworld=1, res=8)
  hc = context.prepare_context(sc.mjm, 1, schedule="wavefront", wave_chunk_worlds=3)
  assert hc.options["schedule"] == 2 and hc.options["wave_chunk_worlds"] == 3
  with pytest.raises(ValueError, match="wave_chunk_worlds must be at least 0"):
    context.prepare_context(sc.mjm, 1, schedule="wavefront", wave_chunk_worlds=-1)


def test_wave_scratch_size_is_exported():
  """mjpbr_wave_scratch_bytes is host-only: it sizes the scratch from a descriptor's counts (no
  device pointers, no GPU), growing with the worlds per chunk."""
  import ctypes

  from mujoco_warp_pbr_gb300 import _lib

  lib = ctypes.CDLL(str(_lib.LIBRARY))
  fn = lib.mjpbr_wave_scratch_bytes
  fn.restype = ctypes.c_int64
  fn.argtypes = [ctypes.POINTER(_lib.Scene), ctypes.c_int32]
  s = _lib.Scene()
  s.abi_version = _lib.ABI_VERSION
  s.nworld, s.nrender, s.nlight = 8, 2, 2
  s.cam_res[0][0], s.cam_res[0][1] = 64, 32
  s.cam_res[1][0], s.cam_res[1][1] = 16, 16
  s.render_rgb[0], s.render_rgb[1] = 1, 0
  s.settings.samples_per_axis = 2
  one, four = fn(ctypes.byref(s), 1), fn(ctypes.byref(s), 4)
  per_sample = 2 * 32 + 2 * 64 + 48 + 2 * (2 * 4 + 2 * 32)
  samples = 64 * 32 * 4  # the depth-only camera takes no records
  assert four - one == 3 * samples * per_sample
  assert one >= samples * per_sample
  assert fn(None, 1) == -1


def _outputs(rc):
  out = {
    "rgb": rc.base.rgb_data.cpu().numpy().view(np.uint32).copy(),
    "depth": rc.base.depth_data.cpu().numpy().copy(),
    "seg": rc.base.seg_data.cpu().numpy().copy(),
  }
  if rc.render_hdr:
    out["hdr"] = rc.hdr_data.cpu().numpy().copy()
  if rc.render_guides:
    out["albedo"] = rc.guide_albedo.cpu().numpy().copy()
    out["normal"] = rc.guide_normal.cpu().numpy().copy()
  return out


def _frame(m, d, rc, seed):
  import mujoco_warp_pbr_gb300 as mjpbr

  for t in (rc.base.rgb_data, rc.base.depth_data, rc.base.seg_data, rc.hdr_data, rc.guide_albedo, rc.guide_normal):
    t.zero_()
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=seed)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  return _outputs(rc)


def _scene(name):
  from mujoco_warp_pbr_gb300 import synthetic

  if name == "primitives":
    return synthetic.primitive_scene(seed=2, nworld=5, res=40, shadow_samples=4), {}
  if name == "primitives_hard":
    return synthetic.primitive_scene(seed=3, nworld=4, res=33, shadow_samples=1), {"samples_per_pixel": 3}
  if name == "mesh_ibl":
    return synthetic.mesh_ibl_scene(seed=1, nworld=3, res=40, tex_size=64, env_width=128), {}
  if name == "batched":
    return synthetic.batched_scene(seed=1, nworld=5, res=(16, 40, 72)), {}
  if name == "hfield":
    return synthetic.hfield_scene(seed=2, nworld=3, res=36), {}
  raise KeyError(name)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("name", ["primitives", "primitives_hard", "mesh_ibl", "batched", "hfield"])
def test_wavefront_renders_the_grid_images(name):
  from tests import helpers

  sc, extra = _scene(name)
  m, d, rc = helpers.gpu_scene(sc, render_hdr=True, render_guides=True, **extra)
  ref = _frame(m, d, rc, seed=9)
  rc.schedule = 2
  for chunk in (0, 1, 2):
    rc.wave_chunk_worlds = chunk
    rc.wave_scratch = None
    got = _frame(m, d, rc, seed=9)
    for key in ref:
      np.testing.assert_array_equal(got[key], ref[key], err_msg=f"{name}: {key} differs (chunk {chunk})")


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_wavefront_ragged_and_depth_only_cameras():
  """Two cameras whose sizes are not multiples of the 16-pixel tile, the second without RGB."""
  from mujoco_warp_pbr_gb300 import synthetic
  from mujoco_warp_pbr_gb300.synthetic import GEOM_BOX, GEOM_PLANE, GEOM_SPHERE, LIGHT_POINT, Builder
  from tests import helpers

  b = Builder()
  b.geom(GEOM_PLANE, (2, 2, 0.1), rgba=(0.7, 0.7, 0.7, 1))
  b.geom(GEOM_SPHERE, (0.3, 0, 0), pos=(0, 0, 0.3), rgba=(0.8, 0.2, 0.2, 1))
  b.geom(GEOM_BOX, (0.2, 0.2, 0.2), pos=(0.5, 0.3, 0.2), rgba=(0.2, 0.8, 0.2, 1))
  b.light(LIGHT_POINT, pos=(0.5, -0.5, 2.0), diffuse=(0.6, 0.6, 0.6), range=10.0, bulbradius=0.05, castshadow=True)
  b.camera(pos=(0.0, -2.5, 1.5), target=(0, 0, 0.3), resolution=(37, 21))
  b.camera(pos=(0.3, -2.0, 1.5), target=(0, 0, 0.3), resolution=(19, 33))
  mjm, mjd = b.build()
  sc = synthetic.SyntheticScene(
    name="ragged", mjm=mjm, mjd=mjd, nworld=3, options={"render_depth": True, "render_seg": True, "render_rgb": [True, False], "samples_per_pixel": 2},
    per_world={}, seed=0,
  )
  m, d, rc = helpers.gpu_scene(sc)
  ref = _frame(m, d, rc, seed=2)
  rc.schedule = 2
  got = _frame(m, d, rc, seed=2)
  for key in ref:
    np.testing.assert_array_equal(got[key], ref[key], err_msg=key)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("seed", [0, 5])
def test_wavefront_mesh_ibl_full_assets_matches_oracle(seed):
  """The mesh / IBL configuration at its own asset sizes on 4 worlds, wavefront schedule, against
  the oracle at the real-time bars."""
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.mesh_ibl_scene(seed=seed, nworld=4, res=128)
  m, d, rc = helpers.gpu_scene(sc, schedule="wavefront")
  gpu = helpers.render_gpu(m, d, rc, seed=seed + 4)
  ref = helpers.oracle_render(sc, seed=seed + 4, tables=helpers.gpu_tables(rc))
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  assert diff.max() <= 1, f"max RGB difference {diff.max()}/255"


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_wavefront_context_with_translucent_layers_renders_with_the_megakernel():
  """Translucent layers are not staged: a wavefront context whose geoms are translucent renders
  through the megakernel, with the grid schedule's images."""
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.primitive_scene(seed=1, nworld=2, res=24)
  rgba = sc.per_world["geom_rgba"].copy()
  rgba[:, 2:5, 3] = 0.5
  sc.per_world["geom_rgba"] = rgba
  m, d, rc = helpers.gpu_scene(sc)
  rc.has_transparency = True  # the per-world colours made geoms translucent after creation
  ref = _frame(m, d, rc, seed=1)
  rc.schedule = 2
  got = _frame(m, d, rc, seed=1)
  assert rc.wave_scratch is None
  for key in ref:
    np.testing.assert_array_equal(got[key], ref[key], err_msg=key)


def test_wavefront_tile_mapping_covers_each_sample_once():
  """The wavefront kernels' sample mapping (csrc/render_wave.cu): index idx of a 16 x 16 tile
  with nn samples per pixel is pixel q = idx / nn in Z order, sample idx % nn. Every (pixel,
  sample) of the tile is visited once, a pixel's samples sit on consecutive indices, and 32
  consecutive pixels form an 8 x 4 block (8 a 4 x 2 block): the rays of a warp stay close."""

  def z_x(q):
    return (q & 1) | ((q >> 1) & 2) | ((q >> 2) & 4) | ((q >> 3) & 8)

  def z_y(q):
    return ((q >> 1) & 1) | ((q >> 2) & 2) | ((q >> 3) & 4) | ((q >> 4) & 8)

  assert sorted((z_x(q), z_y(q)) for q in range(256)) == [(x, y) for x in range(16) for y in range(16)]
  for nn in (1, 4, 9):
    seen = [(z_x(idx // nn), z_y(idx // nn), idx % nn) for idx in range(256 * nn)]
    assert len(set(seen)) == 256 * nn
  for size, (bw, bh) in ((32, (8, 4)), (8, (4, 2))):
    for start in range(0, 256, size):
      xs = {z_x(q) for q in range(start, start + size)}
      ys = {z_y(q) for q in range(start, start + size)}
      assert len(xs) == bw and len(ys) == bh and max(xs) - min(xs) == bw - 1 and max(ys) - min(ys) == bh - 1


def _pt_outputs(rc):
  out = {
    "rgb": rc.base.rgb_data.cpu().numpy().view(np.uint32).copy(),
    "depth": rc.base.depth_data.cpu().numpy().copy(),
    "seg": rc.base.seg_data.cpu().numpy().copy(),
    "hdr": rc.hdr_data.cpu().numpy().copy(),
  }
  if rc.render_guides:
    out["albedo"] = rc.guide_albedo.cpu().numpy().copy()
    out["normal"] = rc.guide_normal.cpu().numpy().copy()
  if rc.denoise:
    out["guide"] = rc.aov_guide.cpu().numpy().copy()
    out["emission"] = rc.aov_emission.cpu().numpy().copy()
    out["demod"] = rc.denoise_buffers[0].cpu().numpy().copy()
  return out


def _pt_frame(m, d, rc, seed):
  import mujoco_warp_pbr_gb300 as mjpbr

  for t in (rc.base.rgb_data, rc.base.depth_data, rc.base.seg_data, rc.hdr_data, rc.guide_albedo, rc.guide_normal, rc.aov_guide,
            rc.aov_emission, rc.denoise_buffers[0]):
    t.zero_()
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=seed, denoise=False)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  return _pt_outputs(rc)


def _pt_scene(name):
  from mujoco_warp_pbr_gb300 import synthetic

  pt = {"tier": 1, "render_hdr": True}
  if name == "path":
    return synthetic.path_scene(seed=3, nworld=5, res=24, spp=3), {**pt, "path_samples": 3, "render_guides": True}
  if name == "path_denoise":
    return synthetic.path_scene(seed=4, nworld=3, res=32, spp=2), {**pt, "path_samples": 2, "denoise": True}
  if name == "mesh_ibl":
    return synthetic.mesh_ibl_scene(seed=1, nworld=3, res=24, tex_size=64, env_width=128), {**pt, "path_samples": 4, "max_depth": 3, "rr_depth": 2}
  if name == "primitives_mirror":
    return synthetic.primitive_scene(seed=2, nworld=3, res=24), {**pt, "path_samples": 2, "max_depth": 4, "rr_depth": 1}
  if name == "large_path_envs":
    return synthetic.large_path_scene(seed=1, nworld=4, res=16, env_width=128), {**pt, "path_samples": 2}
  if name == "hfield":
    return synthetic.hfield_scene(seed=2, nworld=2, res=20), {**pt, "path_samples": 2}
  raise KeyError(name)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("name", ["path", "path_denoise", "mesh_ibl", "primitives_mirror", "large_path_envs", "hfield"])
def test_path_wavefront_renders_the_persistent_kernel_images(name):
  """The staged path tracer (extend / shade / shadow / next-event kernels over path queues) and the
  persistent path kernel give bit-identical images, HDR, guides and denoiser inputs, for one chunk
  of worlds and for chunks of one and two worlds."""
  from tests import helpers

  sc, opts = _pt_scene(name)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  rc.schedule = 0
  ref = _pt_frame(m, d, rc, seed=5)
  rc.schedule = 2
  for chunk in (0, 1, 2):
    rc.wave_chunk_worlds = chunk
    rc.wave_scratch = None
    got = _pt_frame(m, d, rc, seed=5)
    for key in ref:
      np.testing.assert_array_equal(got[key], ref[key], err_msg=f"{name}: {key} differs (chunk {chunk})")


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_path_wavefront_translucent_layers_and_depth_only_camera():
  """Stochastic alpha pass-through (extra bounce iterations) and a second camera without RGB."""
  from mujoco_warp_pbr_gb300 import synthetic
  from mujoco_warp_pbr_gb300.synthetic import GEOM_BOX, GEOM_PLANE, GEOM_SPHERE, LIGHT_POINT, Builder
  from tests import helpers

  b = Builder()
  b.geom(GEOM_PLANE, (2, 2, 0.1), rgba=(0.7, 0.7, 0.7, 1))
  b.geom(GEOM_SPHERE, (0.3, 0, 0), pos=(0, 0, 0.3), rgba=(0.8, 0.2, 0.2, 0.5))
  b.geom(GEOM_BOX, (0.2, 0.2, 0.2), pos=(0.5, 0.3, 0.2), rgba=(0.2, 0.8, 0.2, 1))
  b.light(LIGHT_POINT, pos=(0.5, -0.5, 2.0), diffuse=(0.6, 0.6, 0.6), range=10.0, bulbradius=0.05, castshadow=True)
  b.camera(pos=(0.0, -2.5, 1.5), target=(0, 0, 0.3), resolution=(23, 17))
  b.camera(pos=(0.3, -2.0, 1.5), target=(0, 0, 0.3), resolution=(19, 13))
  mjm, mjd = b.build()
  sc = synthetic.SyntheticScene(
    name="translucent", mjm=mjm, mjd=mjd, nworld=3,
    options={"render_depth": True, "render_seg": True, "render_rgb": [True, False], "tier": 1, "path_samples": 3, "max_layers": 2,
             "render_hdr": True},
    per_world={}, seed=0,
  )
  m, d, rc = helpers.gpu_scene(sc)
  assert rc.has_transparency
  rc.schedule = 0
  ref = _pt_frame(m, d, rc, seed=8)
  rc.schedule = 2
  got = _pt_frame(m, d, rc, seed=8)
  for key in ref:
    np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
