"""GPU parity of the real-time tier against the CPU oracle, through the public API.

Bars: segmentation bit-exact, depth within 1e-5 relative, RGB within 1/255 per channel.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mujoco_warp_pbr_gb300 import synthetic  # noqa: E402
from tests import helpers  # noqa: E402

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("shadow_samples", [1, 4])
def test_primitive_scene_matches_oracle(seed, shadow_samples):
  sc = synthetic.primitive_scene(seed=seed, nworld=4, res=48, shadow_samples=shadow_samples)
  m, d, rc = helpers.gpu_scene(sc, render_hdr=True)
  gpu = helpers.render_gpu(m, d, rc, seed=7)
  ref = helpers.oracle_render(sc, seed=7, tables=helpers.gpu_tables(rc), render_hdr=True)
  _assert_realtime_parity(gpu, ref, f"primitives 4 x 48^2 seed {seed} shadow samples {shadow_samples}")
  np.testing.assert_allclose(gpu["hdr"], ref["hdr"], rtol=2e-3, atol=1e-3 * float(np.abs(ref["hdr"]).max()))


@pytest.mark.parametrize("order", [0, 1, 2])
def test_render_orders_identical(order):
  sc = synthetic.primitive_scene(seed=2, nworld=2, res=37, shadow_samples=4)
  m, d, rc = helpers.gpu_scene(sc, render_order=order)
  a = helpers.render_gpu(m, d, rc, seed=1)
  m2, d2, rc2 = helpers.gpu_scene(sc, render_order=1)
  b = helpers.render_gpu(m2, d2, rc2, seed=1)
  np.testing.assert_array_equal(a["rgb"], b["rgb"])
  np.testing.assert_array_equal(a["seg"], b["seg"])


def test_outputs_unpack():
  import mujoco_warp_pbr_gb300 as mjpbr

  sc = synthetic.primitive_scene(seed=3, nworld=3, res=24)
  m, d, rc = helpers.gpu_scene(sc)
  g = helpers.render_gpu(m, d, rc)
  rgb = torch.zeros((3, 24, 24, 3), device="cuda")
  depth = torch.zeros((2, 24, 24), device="cuda")
  seg = torch.zeros((3, 24, 24, 2), dtype=torch.int32, device="cuda")
  mjpbr.get_rgb(rc, 0, rgb)
  mjpbr.get_depth(rc, 0, 5.0, depth)
  mjpbr.get_segmentation(rc, 0, seg)
  torch.cuda.synchronize()
  from oracle import oracle

  ch = oracle.unpack_rgb(g["rgb"]).reshape(3, 24, 24, 3) / 255.0
  np.testing.assert_allclose(rgb.cpu().numpy(), ch, atol=1e-6)
  np.testing.assert_allclose(depth.cpu().numpy(), np.clip(g["depth"][:2].reshape(2, 24, 24) / 5.0, 0, 1), rtol=1e-6)
  np.testing.assert_array_equal(seg.cpu().numpy(), g["seg"].reshape(3, 24, 24, 2))
  with pytest.raises(ValueError, match="camera_index must be in"):
    mjpbr.get_rgb(rc, 1, rgb)
  with pytest.raises(ValueError, match="rgb_out must have shape"):
    mjpbr.get_rgb(rc, 0, torch.zeros((3, 24, 23, 3), device="cuda"))


def test_dfg_table_matches_oracle():
  import mujoco_warp_pbr_gb300 as mjpbr
  from oracle import oracle

  sc = synthetic.primitive_scene(seed=0, nworld=1, res=8)
  _, _, rc = helpers.gpu_scene(sc)
  gpu = rc.dfg_lut.cpu().numpy()
  ref = oracle.dfg_lut()
  np.testing.assert_allclose(gpu, ref, rtol=1e-4, atol=1e-5)
  assert mjpbr.check_errors(rc) == 0


def _assert_realtime_parity(gpu, ref, what):
  """The real-time bars: segmentation bit-exact, depth within 1e-5 relative, every RGB channel of
  every pixel within 1/255 (the reference's own render tests hold segmentation exact and depth to
  1e-4 / 1e-5: tests/test_render.py:149-188)."""
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  print(f"{what}: max RGB diff {diff.max()}/255, {int((diff > 0).sum())} of {diff.size} pixels differ at all")
  assert diff.max() <= 1, f"{what}: max RGB difference {diff.max()}/255 at {np.argwhere(diff > 1)[:5]}"


@pytest.mark.parametrize("seed", [0, 1])
def test_primitive_config_exact_size_matches_oracle(seed):
  """The plain real-time configuration at its own size: 16 worlds x 64x64, one directional and one
  point light (bulb radius 0.05), soft shadows with 4 samples, flat grey sky."""
  sc = synthetic.primitive_scene(seed=seed, nworld=16, res=64, shadow_samples=4)
  assert sc.mjm.nlight == 2 and sc.options["cam_res"] == (64, 64)
  m, d, rc = helpers.gpu_scene(sc)
  gpu = helpers.render_gpu(m, d, rc, seed=seed + 1)
  ref = helpers.oracle_render(sc, seed=seed + 1, tables=helpers.gpu_tables(rc))
  _assert_realtime_parity(gpu, ref, f"primitives 16 x 64^2 seed {seed}")


@pytest.mark.parametrize("seed", [0, 5])
def test_mesh_ibl_scene_matches_oracle(seed):
  """Meshes, textures with mips, IBL, 2x2 supersampling and the mirror floor (small assets)."""
  sc = synthetic.mesh_ibl_scene(seed=seed, nworld=2, res=48, tex_size=64, env_width=128)
  m, d, rc = helpers.gpu_scene(sc, render_hdr=True)
  gpu = helpers.render_gpu(m, d, rc, seed=3)
  ref = helpers.oracle_render(sc, seed=3, tables=helpers.gpu_tables(rc), render_hdr=True)
  _assert_realtime_parity(gpu, ref, f"mesh/IBL small assets seed {seed}")


@pytest.mark.parametrize("seed", [0, 5])
def test_mesh_ibl_config_full_assets_matches_oracle(seed):
  """The mesh / IBL configuration at its own asset sizes and resolution on 4 worlds: six displaced
  icospheres of 5120 triangles, ten primitives, 512x512 albedo / ORM / normal maps with full mip
  chains, a 1024x512 environment, 128x128 cameras, 2x2 supersampling, mirror floor 0.3."""
  sc = synthetic.mesh_ibl_scene(seed=seed, nworld=4, res=128)
  assert sc.mjm.nmesh == 6 and sc.options["cam_res"] == (128, 128) and sc.options["samples_per_pixel"] == 2
  m, d, rc = helpers.gpu_scene(sc)
  gpu = helpers.render_gpu(m, d, rc, seed=seed + 4)
  ref = helpers.oracle_render(sc, seed=seed + 4, tables=helpers.gpu_tables(rc))
  _assert_realtime_parity(gpu, ref, f"mesh/IBL 4 x 128^2 full assets seed {seed}")


def test_texture_mips_and_prefilter_match_oracle():
  """The context-creation tables of the GPU against the oracle's own host preparation and C / NumPy
  restatements: texture and radiance mip chains bit for bit, the prefiltered stack within float16
  rounding, the SH9 coefficients and importance-sampling tables (double precision on both sides)
  within float32 rounding."""
  from oracle import host_prep, oracle, scene_struct

  sc = synthetic.mesh_ibl_scene(seed=1, nworld=1, res=16, tex_size=128, env_width=256)
  _, _, rc = helpers.gpu_scene(sc)
  torch.cuda.synchronize()
  hc = oracle.OracleScene(sc.mjm, sc.mjd, 1, sc.options, sc.per_world).hc
  desc, data = host_prep.pack_textures(hc.textures, scene_struct.Texture)
  np.testing.assert_array_equal(rc.tex_data.cpu().numpy(), oracle.build_mips(desc, data))
  edesc, edata = oracle.environment_textures(hc.environments)
  env_ref = oracle.build_mips(edesc, edata)
  np.testing.assert_array_equal(rc.env.radiance_data.cpu().numpy(), env_ref)
  stack_gpu = rc.env.prefiltered.cpu().numpy().view(np.float16).astype(np.float32)
  stack_ref = oracle.prefilter(hc.environments, env_ref, edesc).view(np.float16).astype(np.float32)
  np.testing.assert_allclose(stack_gpu, stack_ref, rtol=5e-3, atol=5e-3 * float(stack_ref.max()))
  env = hc.environments
  np.testing.assert_allclose(rc.env.sh.cpu().numpy(), env.sh, rtol=2e-6, atol=1e-6 * float(np.abs(env.sh).max()))
  np.testing.assert_allclose(rc.env.prob.cpu().numpy(), env.prob, rtol=2e-6, atol=1e-12)
  np.testing.assert_allclose(rc.env.marginal.cpu().numpy(), env.marginal, rtol=2e-6, atol=1e-7)
  np.testing.assert_allclose(rc.env.conditional.cpu().numpy(), env.conditional, rtol=2e-6, atol=1e-7)
