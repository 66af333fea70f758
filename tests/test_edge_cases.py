"""Edge cases of the render path, GPU against the oracle (segmentation bit-exact, depth 1e-5, RGB
within 1/255): a 1 x 1 camera, odd image sizes over many worlds, a world whose geoms are all
hidden, a scene without lights, a camera inside a sphere, a scene of one plane, and the same
small cases on the path-traced tier. The oracle side of each case also runs on the CPU."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mujoco_warp_pbr_gb300 import synthetic  # noqa: E402
from mujoco_warp_pbr_gb300.synthetic import GEOM_BOX, GEOM_PLANE, GEOM_SPHERE, LIGHT_DIRECTIONAL, LIGHT_POINT  # noqa: E402
from tests import helpers  # noqa: E402

def _scene(name, build, nworld=1, per_world=None, **options):
  b = synthetic.Builder()
  build(b)
  mjm, mjd = b.build()
  opts = {"render_rgb": True, "render_depth": True, "render_seg": True, **options}
  return synthetic.SyntheticScene(name=name, mjm=mjm, mjd=mjd, nworld=nworld, options=opts, per_world=per_world or {}, seed=0)


def _basic(b, res=(1, 1), lights=True, target=(0, 0, 0.3)):
  b.geom(GEOM_PLANE, (2, 2, 0.1), rgba=(0.6, 0.6, 0.6, 1))
  b.geom(GEOM_SPHERE, (0.3, 0, 0), pos=(0, 0, 0.3), rgba=(0.8, 0.2, 0.2, 1))
  b.geom(GEOM_BOX, (0.15, 0.15, 0.15), pos=(0.5, 0.2, 0.15), rgba=(0.2, 0.3, 0.9, 1))
  if lights:
    b.light(LIGHT_DIRECTIONAL, dir=(0.3, 0.2, -1.0), castshadow=True)
    b.light(LIGHT_POINT, pos=(-0.5, -0.5, 1.5), bulbradius=0.05, castshadow=True)
  b.camera((0.2, -2.0, 1.2), target, resolution=res)


def _hidden_world(nworld):
  rgba = np.broadcast_to(np.array([[0.6, 0.6, 0.6, 1], [0.8, 0.2, 0.2, 1], [0.2, 0.3, 0.9, 1]], np.float32), (nworld, 3, 4)).copy()
  rgba[1, :, 3] = 0.0  # world 1 hides every geom
  return {"geom_rgba": rgba}


def _inside(b):
  b.geom(GEOM_SPHERE, (1.0, 0, 0), rgba=(0.7, 0.7, 0.2, 1))
  b.geom(GEOM_BOX, (0.1, 0.1, 0.1), pos=(0.3, 0.0, 0.0), rgba=(0.2, 0.7, 0.2, 1))
  b.light(LIGHT_POINT, pos=(0, 0, 0.5), castshadow=True)
  b.camera((0, 0, 0), (1, 0, 0), resolution=(24, 16))


def _plane_only(b):
  b.geom(GEOM_PLANE, (0, 0, 0.1), rgba=(0.5, 0.7, 0.5, 1))
  b.light(LIGHT_DIRECTIONAL, dir=(0.0, 0.3, -1.0), castshadow=True)
  b.camera((0, -2.0, 1.0), (0, 0, 0), resolution=(20, 20))


CASES = {
  "pixel_1x1": lambda: _scene("1x1", lambda b: _basic(b, (1, 1)), nworld=3),
  "odd_sizes_many_worlds": lambda: _scene("odd", lambda b: _basic(b, (37, 5)), nworld=67),
  "hidden_world": lambda: _scene("hidden", lambda b: _basic(b, (16, 12)), nworld=3, per_world=_hidden_world(3)),
  "no_lights": lambda: _scene("dark", lambda b: _basic(b, (16, 16), lights=False), nworld=2),
  "camera_inside_sphere": lambda: _scene("inside", _inside, nworld=2),
  "plane_only": lambda: _scene("plane", _plane_only, nworld=2),
}


def _compare(gpu, ref):
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  assert diff.max() <= 1, f"max RGB difference {diff.max()}/255"


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_renders_edge_case(case):
  sc = CASES[case]()
  out = helpers.oracle_render(sc, seed=1)
  seg = out["seg"][..., 0]
  if case == "hidden_world":
    assert np.all(seg[1] == -1) and np.all(out["depth"][1] == 0)
    assert np.any(seg[0] >= 0)
  if case == "camera_inside_sphere":
    # back-face culling (the default) hides the sphere's inner wall: only the box is seen
    assert not np.any(seg == 0) and np.any(seg == 1)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("case", sorted(CASES))
def test_realtime_edge_case_matches_oracle(case):
  sc = CASES[case]()
  m, d, rc = helpers.gpu_scene(sc)
  gpu = helpers.render_gpu(m, d, rc, seed=1)
  ref = helpers.oracle_render(sc, seed=1, tables=helpers.gpu_tables(rc))
  _compare(gpu, ref)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("case", ["pixel_1x1", "odd_sizes_many_worlds", "hidden_world", "camera_inside_sphere"])
def test_path_traced_edge_case_matches_oracle(case):
  sc = CASES[case]()
  opts = {"tier": 1, "path_samples": 3, "max_depth": 3}
  m, d, rc = helpers.gpu_scene(sc, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=4)
  ref = helpers.oracle_render(sc, seed=4, tables=helpers.gpu_tables(rc), **opts)
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  assert float(np.mean(diff <= 1)) >= 0.995


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("schedule", ["grid", "wavefront"])
@pytest.mark.parametrize("tier", [0, 1])
def test_more_worlds_than_one_grid_dimension(schedule, tier):
  """70,000 worlds of 8x8 pixels: more than CUDA's 65,535 blocks in grid y, where the real-time grid
  and wavefront schedules put the worlds (the launches cover them in batches; the path tier's
  launches are one-dimensional). The last worlds match the oracle at the real-time bars."""
  from oracle import oracle

  nworld = 70000
  sc = synthetic.primitive_scene(seed=9, nworld=nworld, res=8, shadow_samples=1)
  opts = {"tier": tier, "path_samples": 2, "max_depth": 2} if tier else {}
  m, d, rc = helpers.gpu_scene(sc, schedule=schedule, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=2)
  o = oracle.OracleScene(sc.mjm, sc.mjd, nworld, {**sc.options, **opts}, sc.per_world, tables=helpers.gpu_tables(rc))
  w0, w1 = nworld - 6, nworld
  ref = o.render(seed=2, worlds=(w0, w1))
  np.testing.assert_array_equal(gpu["seg"][w0:w1], ref["seg"][w0:w1])
  np.testing.assert_allclose(gpu["depth"][w0:w1], ref["depth"][w0:w1], rtol=1e-5, atol=1e-6)
  assert helpers.rgb_diff(gpu["rgb"][w0:w1], ref["rgb"][w0:w1]).max() <= 1
  # every world was rendered (no world left at the cleared value)
  assert np.all(gpu["seg"].reshape(nworld, -1, 2)[:, :, 0].max(axis=1) >= 0)


def _crowded_scene(n: int = 2000, nworld: int = 2, res: int = 32):
  """A ground plane and n small primitives per world: a world block larger than shared memory."""
  rng = np.random.default_rng(5)
  b = synthetic.Builder()
  b.geom(GEOM_PLANE, (8.0, 8.0, 0.1), rgba=(0.6, 0.6, 0.6, 1.0))
  for i in range(n):
    kind = (GEOM_SPHERE, GEOM_BOX)[i % 2]
    pos = (*rng.uniform(-3.0, 3.0, 2), rng.uniform(0.05, 1.5))
    size = (0.06, 0.0, 0.0) if kind == GEOM_SPHERE else (0.05, 0.04, 0.03)
    b.geom(kind, size, pos=pos, rgba=(*rng.uniform(0.1, 1.0, 3), 1.0))
  b.light(LIGHT_DIRECTIONAL, pos=(0, 0, 4), dir=(0.3, 0.2, -1.0), diffuse=(0.7, 0.7, 0.7), castshadow=True)
  b.light(LIGHT_POINT, pos=(0.5, -0.5, 2.0), diffuse=(0.5, 0.5, 0.5), range=10.0, bulbradius=0.05, castshadow=True)
  b.camera((0.0, -5.0, 3.0), (0.0, 0.0, 0.3), fovy=50.0, resolution=(res, res))
  mjm, mjd = b.build()
  return synthetic.SyntheticScene(
    name="crowded", mjm=mjm, mjd=mjd, nworld=nworld,
    options={"cam_res": (res, res), "render_rgb": True, "render_depth": True, "render_seg": True, "shadow_samples": 4},
    per_world={}, seed=5,
  )


def test_crowded_world_block_exceeds_shared_memory():
  from mujoco_warp_pbr_gb300 import _lib, context

  sc = _crowded_scene()
  hc = context.prepare_context(sc.mjm, sc.nworld, data=sc.mjd, **sc.options)
  assert hc.world_block_floats * 4 > 232448  # more than a GB300 CTA's shared memory


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("schedule", ["grid", "wavefront"])
@pytest.mark.parametrize("tier", [0, 1])
def test_crowded_worlds_render_from_global_memory(schedule, tier):
  """2,001 geoms per world: the kernels that stage a world block in shared memory read it in place
  instead, with the same images as the oracle."""
  sc = _crowded_scene()
  opts = {"tier": tier, "path_samples": 2, "max_depth": 2} if tier else {}
  m, d, rc = helpers.gpu_scene(sc, schedule=schedule, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=3)
  ref = helpers.oracle_render(sc, seed=3, tables=helpers.gpu_tables(rc), **opts)
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  assert helpers.rgb_diff(gpu["rgb"], ref["rgb"]).max() <= 1
  assert (gpu["seg"][..., 0] > 0).mean() > 0.2  # many primitives in view


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("tier", [0, 1])
def test_more_geoms_than_the_wavefront_packs(tier):
  """65,601 geoms per world: more than the wavefront's 16-bit slot ids, so a context on the
  wavefront schedule renders with the grid schedule (real-time) or the persistent path kernel, with
  world blocks read in place; the images match the oracle."""
  sc = _crowded_scene(n=65600, nworld=2, res=8)
  opts = {"tier": tier, "path_samples": 2, "max_depth": 2} if tier else {}
  m, d, rc = helpers.gpu_scene(sc, schedule="wavefront", **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=4)
  ref = helpers.oracle_render(sc, seed=4, tables=helpers.gpu_tables(rc), **opts)
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  assert helpers.rgb_diff(gpu["rgb"], ref["rgb"]).max() <= 1
