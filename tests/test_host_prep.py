"""The oracle's host preparation (oracle/host_prep.py, a restatement of the reference's host-side
rules) against the product's (mujoco_warp_pbr_gb300.context.prepare_context), field by field, on
every synthetic workload and on option variations: both must hand their renderers the same
settings, per-world tables, output layout, enabled geoms, texture texels and environment images.
The two share no code; a difference here would otherwise show up only as an image difference."""

import numpy as np
import pytest

from mujoco_warp_pbr_gb300 import context, synthetic
from oracle import host_prep, oracle, scene_struct


def _scenes():
  return {
    "primitives": (synthetic.primitive_scene(seed=0, nworld=3, res=24), {}),
    "primitives_mujoco_lights": (synthetic.primitive_scene(seed=1, nworld=2, res=16), {"light_model": 1, "ev100": 12.0}),
    "primitives_heuristic": (
      synthetic.primitive_scene(seed=2, nworld=2, res=16),
      {"unset_material": 1, "background_color": (0.2, 0.4, 0.6, 1.0), "render_seg": True, "shadow_light_fraction": 0.25},
    ),
    "primitives_default_material": (synthetic.primitive_scene(seed=3, nworld=2, res=16), {"default_material": {"metallic": 0.3, "roughness": 0.7}}),
    "mesh_ibl": (synthetic.mesh_ibl_scene(seed=1, nworld=2, res=24, tex_size=64, env_width=128), {"envmap_rotation": 30.0}),
    "mesh_ibl_no_textures": (synthetic.mesh_ibl_scene(seed=2, nworld=2, res=24, tex_size=32, env_width=64), {"use_textures": False, "specular_aa": False}),
    "batched": (synthetic.batched_scene(seed=1, nworld=4, res=(16, 24, 32)), {}),
    "batched_cameras": (synthetic.batched_scene(seed=1, nworld=4, res=(16, 24, 32)), {"render_rgb": [True, False, True], "render_depth": False}),
    "path": (synthetic.path_scene(seed=2, nworld=3, res=16), {"denoise": True, "denoise_iterations": 4, "render_hdr": True}),
    "large_path_envs": (synthetic.large_path_scene(seed=1, nworld=4, res=16, env_width=128), {}),
    "hfield": (synthetic.hfield_scene(seed=2, nworld=2, res=16), {}),
  }


@pytest.mark.parametrize("name", sorted(_scenes()))
def test_oracle_host_preparation_matches_the_product(name):
  sc, extra = _scenes()[name]
  options = {**sc.options, **extra}
  hc = context.prepare_context(sc.mjm, sc.nworld, data=sc.mjd, **options)
  ref = host_prep.prepare(sc.mjm, sc.mjd, sc.nworld, options)
  # output layout
  def norm(v):
    if isinstance(v, (list, tuple, np.ndarray)):
      return [norm(x) for x in v]
    return v.item() if isinstance(v, np.generic) else v

  for key, value in ref.outputs.items():
    assert norm(hc.outputs[key]) == norm(value), key
  # settings (every MjpbrSettings field the oracle sets)
  assert set(ref.settings) <= set(scene_struct.Settings._fields_[i][0] for i in range(len(scene_struct.Settings._fields_)))
  for key, value in ref.settings.items():
    if key in ("render_order",):  # launch shape only
      continue
    got = hc.settings[key]
    if isinstance(value, tuple):
      np.testing.assert_allclose(np.asarray(got, np.float64), np.asarray(value, np.float64), rtol=1e-12, atol=0, err_msg=key)
    else:
      assert got == pytest.approx(value, rel=1e-12, abs=0), key
  # per-world tables
  assert set(ref.tables) == set(hc.tables)
  for key, value in ref.tables.items():
    np.testing.assert_array_equal(np.asarray(hc.tables[key]), value, err_msg=key)
  np.testing.assert_array_equal(hc.enabled_geom_ids, ref.enabled_geom_ids)
  np.testing.assert_array_equal(np.asarray(hc.meshes.get("mesh_nface", []), np.int32), ref.mesh_nface[: len(hc.meshes.get("mesh_nface", []))])
  # textures: the same texel bytes at the same offsets
  if hc.textures is None:
    assert not ref.textures
  else:
    desc, data = host_prep.pack_textures(ref.textures, scene_struct.Texture)
    np.testing.assert_array_equal(hc.textures.data, data)
    assert [(d.format, d.width, d.height, d.nlevel) for d in hc.textures.desc] == [(d.format, d.width, d.height, d.nlevel) for d in desc]
  # environments: radiance textures and the shapes of the sampling tables
  env = ref.environments
  if hc.environments is None:
    assert env is None
  else:
    assert hc.environments.nenv == env.nenv
    for a, b in zip(hc.environments.radiance, env.radiance, strict=True):
      np.testing.assert_array_equal(a, b)
    assert (hc.environments.prefilter_levels, hc.environments.prefilter_height, hc.environments.prefilter_width) == (
      env.prefilter_levels, env.prefilter_height, env.prefilter_width)
    assert hc.environments.max_width == env.max_width
    assert hc.environments.cdf_images[0].shape[:2] == env.prob.shape[1:]


def test_environment_images_reduce_like_the_reference():
  """The product's exact 2 x 2 reduction and the reference's mean (the oracle's) agree to float32
  rounding, and both table images have the same shape when maps of different sizes share it."""
  rng = np.random.default_rng(5)
  big = np.exp(rng.normal(0.0, 1.0, (256, 512, 3))).astype(np.float32)
  small = np.exp(rng.normal(0.0, 1.0, (64, 128, 3))).astype(np.float32)
  from mujoco_warp_pbr_gb300 import envmap

  np.testing.assert_allclose(envmap.reduce_width(big, 128), host_prep.downsample(big, 128), rtol=4 * 1.2e-7)  # a few float32 ulp
  he = envmap.prepare_environments([big, small])
  re = host_prep.build_environments([big, small])
  assert he.cdf_images[0].shape[:2] == re.prob.shape[1:] and he.cdf_images[1].shape == he.cdf_images[0].shape


def test_oracle_imports_nothing_of_the_product():
  """The oracle's modules import no mujoco_warp_pbr_gb300 module (so its results are independent
  of the product's host code and it loads no product library)."""
  import ast
  from pathlib import Path

  for path in sorted(Path(oracle.__file__).parent.glob("*.py")):
    tree = ast.parse(path.read_text())
    for node in ast.walk(tree):
      names = []
      if isinstance(node, ast.Import):
        names = [a.name for a in node.names]
      elif isinstance(node, ast.ImportFrom):
        names = [node.module or ""]
      for n in names:
        assert not n.startswith("mujoco_warp_pbr_gb300"), f"{path.name} imports {n}"
