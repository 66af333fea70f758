"""Path-traced tier: the reference's own tests (tests/test_pathtrace.py of mujoco_warp_pbr) restated
on array scenes and run on the CPU oracle and on the GPU, and GPU-vs-oracle parity of the path
tracer on the synthetic scenes.

Parity bars (GPU against the oracle, same seed): segmentation bit-exact, depth within 1e-5
relative, every pixel's RGB within 1/255 per channel, and the mean absolute HDR difference within
1% of the mean HDR value. Paths take the same decisions on both sides: the sampling arithmetic is
plain float with a deterministic sine / cosine. A few surface values that feed a decision (texture
UVs from atan2, spot-cone cosines) use faster functions on the GPU than the oracle's libm; a path
whose decision landed within an ulp of such a threshold would diverge, and the assertion message
lists the pixels that differ. None does on the tested scenes.
"""

import numpy as np
import pytest

from tests import kat
from tests.kat import GEOM_BOX, GEOM_PLANE, GEOM_SPHERE, LIGHT_DIRECTIONAL, LIGHT_POINT, Builder

torch = pytest.importorskip("torch")

GPU = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]
RENDERERS = [pytest.param("oracle", id="oracle"), pytest.param("gpu", id="gpu", marks=GPU)]
PATH = {"tier": 1, "render_hdr": True}


@pytest.fixture(params=RENDERERS)
def render(request):
  return kat.render if request.param == "oracle" else kat.render_gpu


def _sphere(metallic: float, roughness: float) -> Builder:
  b = Builder()
  mat = b.material(rgba=(1, 1, 1, 1), metallic=metallic, roughness=roughness)
  b.geom(GEOM_SPHERE, (0.5, 0, 0), matid=mat)
  b.camera(resolution=(32, 32), fovy=8.0, **kat.FRONT_CAMERA)
  return b


@pytest.mark.parametrize("metallic,roughness", [(0.0, 0.3), (1.0, 0.3), (0.0, 1.0), (1.0, 1.0)])
def test_white_furnace(render, metallic, roughness):
  """A white sphere in a white environment, 512 paths of up to 8 bounces per pixel, shows 1."""
  white = np.ones((32, 64, 3), np.float32)
  out = render(_sphere(metallic, roughness), envmap=white, envmap_intensity=1.0, path_samples=512, max_depth=8, **PATH)
  np.testing.assert_allclose(out["hdr"][0, 8:24, 8:24].mean(axis=(0, 1)), 1.0, rtol=0.03)


def _lambert_plane() -> Builder:
  return kat.plane_scene(
    {"rgba": (0.8, 0.8, 0.8, 1), "roughness": 1.0, "specular": 0.0},
    {"type": LIGHT_POINT, "pos": (0, 0, 1.5), "intensity": 3.0, "range": 1000.0, "bulbradius": 0.0, "castshadow": False},
  )


def test_direct_lambert_matches_realtime(render):
  """With one interaction and a point light, both tiers integrate the same direct lighting."""
  realtime = render(_lambert_plane(), render_hdr=True)["hdr"][0]
  path = render(_lambert_plane(), path_samples=16, max_depth=1, **PATH)["hdr"][0]
  np.testing.assert_allclose(path, realtime, rtol=0.01)


def test_seeded_and_deterministic(render):
  env = np.random.default_rng(0).uniform(0, 2, (32, 64, 3)).astype(np.float32)
  opts = dict(envmap=env, envmap_intensity=1.0, path_samples=4, **PATH)
  a = render(_sphere(0.0, 0.5), seed=0, **opts)["hdr"]
  b = render(_sphere(0.0, 0.5), seed=0, **opts)["hdr"]
  np.testing.assert_array_equal(a, b)
  c = render(_sphere(0.0, 0.5), seed=1, **opts)["hdr"]
  assert not np.array_equal(a, c)


def _three_geoms() -> Builder:
  b = Builder()
  b.light(kat.synthetic.LIGHT_SPOT, pos=(0, 0, 3), dir=(0, 0, -1))
  b.geom(GEOM_PLANE, (3, 3, 0.1))
  b.geom(GEOM_SPHERE, (0.3, 0, 0), pos=(0, 0, 0.4))
  b.geom(GEOM_BOX, (0.2, 0.2, 0.2), pos=(0.6, 0.2, 0.3))
  b.camera(pos=(0, -2.5, 1.2), xyaxes=(1, 0, 0, 0, 0.45, 0.9), resolution=(40, 32))
  return b


def test_depth_and_segmentation_match_realtime(render):
  realtime = render(_three_geoms())
  path = render(_three_geoms(), tier=1, path_samples=2)
  np.testing.assert_array_equal(path["seg"], realtime["seg"])
  np.testing.assert_allclose(path["depth"], realtime["depth"], rtol=1e-5)


def _corner() -> Builder:
  b = Builder()
  b.light(LIGHT_DIRECTIONAL, dir=(0, 0.5, -1), castshadow=True)
  b.geom(GEOM_PLANE, (2, 2, 0.1), rgba=(0.9, 0.9, 0.9, 1))
  b.geom(GEOM_BOX, (2, 0.01, 1), pos=(0, 1, 1), rgba=(0.9, 0.9, 0.9, 1))
  b.camera(pos=(0, -1.5, 0.5), xyaxes=(1, 0, 0, 0, 0.3, 1), fovy=40.0, resolution=(32, 32))
  return b


def test_interreflection_brightens_concave_corner(render):
  """Light bouncing between two walls: more bounces, more light (never less)."""
  one = render(_corner(), path_samples=64, max_depth=1, **PATH)["hdr"][0].mean()
  four = render(_corner(), path_samples=64, max_depth=4, **PATH)["hdr"][0].mean()
  assert four > one * 1.1


# ---------------------------------------------------------------- GPU against the oracle


def _assert_path_parity(gpu, ref):
  from tests import helpers

  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  # every pixel within 1/255: the paths take the same decisions on both sides (no allowance for
  # diverging paths; HDR values may differ in the last bits where shading uses fused arithmetic)
  assert diff.max() <= 1, f"{int((diff > 1).sum())} pixels differ by more than 1/255 (max {diff.max()}) at {np.argwhere(diff > 1)[:5]}"
  mean_err = float(np.abs(gpu["hdr"] - ref["hdr"]).mean())
  assert mean_err <= 0.01 * float(np.abs(ref["hdr"]).mean()) + 1e-6


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("samples,max_depth", [(4, 4), (9, 2)])
def test_primitive_scene_matches_oracle(samples, max_depth):
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.primitive_scene(seed=1, nworld=3, res=40)
  opts = dict(path_samples=samples, max_depth=max_depth, rr_depth=1, **PATH)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=11)
  ref = helpers.oracle_render(sc, seed=11, tables=helpers.gpu_tables(rc), **opts)
  _assert_path_parity(gpu, ref)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("seed", [0, 5])
def test_mesh_ibl_scene_matches_oracle(seed):
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.mesh_ibl_scene(seed=seed, nworld=3, res=40, tex_size=64, env_width=128)
  opts = dict(path_samples=4, max_depth=3, rr_depth=2, **PATH)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=seed + 2)
  ref = helpers.oracle_render(sc, seed=seed + 2, tables=helpers.gpu_tables(rc), **opts)
  _assert_path_parity(gpu, ref)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_large_path_configuration_matches_oracle():
  """The large path-traced configuration's features at a small size: two cameras per world, four
  environments chosen per world (env_id) with per-world rotations, per-world materials and
  emission, 2 spp, depth 4."""
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.large_path_scene(seed=2, nworld=6, res=24, env_width=128)
  assert len(sc.options["envmap"]) == 4 and len(set(sc.per_world["env_id"].tolist())) > 1
  opts = dict(path_samples=2, **PATH)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=6)
  ref = helpers.oracle_render(sc, seed=6, tables=helpers.gpu_tables(rc), **opts)
  _assert_path_parity(gpu, ref)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_tiles_cover_ragged_cameras():
  """Two cameras whose sizes are not multiples of the 32-pixel tile, one without RGB."""
  from tests import helpers

  b = _three_geoms()
  b.camera(pos=(0.3, -2.0, 1.5), target=(0, 0, 0.3), resolution=(33, 17))
  mjm, mjd = b.build()
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.SyntheticScene(
    name="ragged", mjm=mjm, mjd=mjd, nworld=2, options={"render_depth": True, "render_seg": True, "render_rgb": [True, False]}, per_world={}, seed=0
  )
  opts = dict(path_samples=3, max_depth=2, **PATH)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=4)
  ref = helpers.oracle_render(sc, seed=4, tables=helpers.gpu_tables(rc), **opts)
  _assert_path_parity(gpu, ref)


def _rel_mse(x: np.ndarray, ref: np.ndarray) -> float:
  """The reference's relative MSE on linear HDR (benchmarks/validate.py:140)."""
  return float(np.mean((x - ref) ** 2 / (ref**2 + 1.0e-2)))


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_converged_means_at_4096_spp_match_oracle():
  """Path-traced means at 4096 spp on the path workload (emissive quads, NEE, depth 4, Russian
  roulette after bounce 2): the GPU's image against the oracle's with the same seed, and, for
  scale, against an independent 4096-spp oracle estimate (another seed)."""
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.path_scene(seed=3, nworld=2, res=32, spp=4096)
  opts = dict(path_samples=4096, denoise=False, render_hdr=True)
  m, d, rc = helpers.gpu_scene(sc, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=21)["hdr"].astype(np.float64)
  tables = helpers.gpu_tables(rc)
  ref = helpers.oracle_render(sc, seed=21, tables=tables, **opts)["hdr"].astype(np.float64)
  other = helpers.oracle_render(sc, seed=22, tables=tables, **opts)["hdr"].astype(np.float64)
  same_seed, noise = _rel_mse(gpu, ref), _rel_mse(other, ref)
  means = gpu.reshape(2, -1, 3).mean(1), ref.reshape(2, -1, 3).mean(1)
  print(f"4096 spp: relMSE GPU vs oracle (same seed) {same_seed:.3e}, oracle seed 22 vs 21 {noise:.3e}; "
        f"per-world means GPU {means[0].round(5).tolist()} oracle {means[1].round(5).tolist()}")
  np.testing.assert_allclose(means[0], means[1], rtol=1e-3)
  assert same_seed < 0.1 * noise
