"""Height fields: traced as closed triangle meshes (the reference queries MuJoCo Warp's height-field
mesh BVH, mujoco_warp_pbr/_src/traverse.py:161-164) and shaded flat with a plane-like texture
mapping (texture.py:147-149).

CPU: the host triangulation (the library's BVH input) is closed, wound outwards and encloses the
height-field solid's volume; the oracle's own triangulation is bit-identical to it; a flat height
field renders like the box of the same solid on the oracle. GPU: the terrain scene matches the
oracle (segmentation bit-exact, depth 1e-5, RGB within 1/255).
"""

from collections import Counter

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mujoco_warp_pbr_gb300 import context  # noqa: E402
from mujoco_warp_pbr_gb300 import synthetic  # noqa: E402
from oracle import oracle  # noqa: E402
from tests import helpers  # noqa: E402


def _model(nrow, ncol, size, seed=0, flat=None):
  b = synthetic.Builder()
  rng = np.random.default_rng(seed)
  elev = np.full((nrow, ncol), flat, np.float32) if flat is not None else rng.uniform(0, 1, (nrow, ncol)).astype(np.float32)
  b.hfield(elev, size)
  return b, elev


@pytest.mark.parametrize("nrow,ncol", [(2, 2), (3, 5), (17, 9)])
def test_triangulation_closed_outward_and_volume(nrow, ncol):
  size = (0.7, 0.4, 0.3, 0.05)
  b, elev = _model(nrow, ncol, size, seed=nrow * ncol)
  b.geom(synthetic.GEOM_HFIELD, (0.7, 0.4, 0.1), dataid=0)
  b.camera((0, 0, 3), (0, 0, 0))
  mjm, _ = b.build()
  vert, face = context.hfield_mesh(mjm, 0)
  assert len(face) == 2 * (nrow - 1) * (ncol - 1) + 3 * (2 * (nrow - 1) + 2 * (ncol - 1))
  # closed and consistently wound: every directed edge appears once, its reverse once
  edges = Counter((int(t[i]), int(t[(i + 1) % 3])) for t in face for i in range(3))
  assert all(n == 1 and edges[(b_, a)] == 1 for (a, b_), n in edges.items())
  # outward: the divergence-theorem volume equals the solid's (top triangles' prisms over the base)
  v = vert.astype(np.float64)
  vol = np.einsum("ij,ij->i", v[face[:, 0]], np.cross(v[face[:, 1]], v[face[:, 2]])).sum() / 6.0
  ntop = 2 * (nrow - 1) * (ncol - 1)
  top = v[face[:ntop]]
  e1, e2 = top[:, 1, :2] - top[:, 0, :2], top[:, 2, :2] - top[:, 0, :2]
  area = 0.5 * np.abs(e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
  expect = float(np.sum(area * (top[:, :, 2].mean(1) + size[3])))
  assert vol == pytest.approx(expect, rel=1e-6)  # float32 vertices
  # the grid: corners at +-size0, +-size1; elevations scaled by size2
  assert vert[:, 0].min() == np.float32(-0.7) and vert[:, 0].max() == np.float32(0.7)
  np.testing.assert_array_equal(vert[: nrow * ncol, 2], (np.float64(np.float32(0.3)) * elev.reshape(-1).astype(np.float64)).astype(np.float32))


@pytest.mark.parametrize("nrow,ncol", [(2, 2), (4, 3), (33, 33)])
def test_oracle_triangulation_is_the_hosts(nrow, ncol):
  b, _ = _model(nrow, ncol, (1.5, 1.1, 0.37, 0.2), seed=3)
  mjm, _ = b.build()
  oracle.set_hfields(oracle.hfield_arrays(mjm))
  v_o, f_o = oracle.hfield_mesh(0)
  v_h, f_h = context.hfield_mesh(mjm, 0)
  np.testing.assert_array_equal(v_o, v_h)
  np.testing.assert_array_equal(f_o, f_h)
  oracle.set_hfields(())


def test_grid_smaller_than_2x2_is_rejected():
  b, _ = _model(1, 4, (1, 1, 1, 0.1))
  b.geom(synthetic.GEOM_HFIELD, (1, 1, 0.5), dataid=0)
  b.camera((0, 0, 3), (0, 0, 0))
  mjm, _ = b.build()
  with pytest.raises(ValueError, match="at least 2"):
    context.hfield_mesh(mjm, 0)
  with pytest.raises(ValueError, match="at least 2"):
    oracle.set_hfields(oracle.hfield_arrays(mjm))


def _solid_scene(use_hfield: bool, res: int = 40):
  """A flat 1.2 x 0.8 m slab, 0.25 m above its base 0.05 m below z = 0: as a height field of
  elevation 0.5 (scale 0.5) or as the box of the same solid."""
  b = synthetic.Builder()
  if use_hfield:
    b.hfield(np.full((5, 7), 0.5, np.float32), (0.6, 0.4, 0.5, 0.05))
    b.geom(synthetic.GEOM_HFIELD, (0.6, 0.4, 0.15), rgba=(0.8, 0.3, 0.2, 1.0), dataid=0)
  else:
    b.geom(synthetic.GEOM_BOX, (0.6, 0.4, 0.15), pos=(0.0, 0.0, 0.1), rgba=(0.8, 0.3, 0.2, 1.0))
  b.light(synthetic.LIGHT_DIRECTIONAL, dir=(0.3, 0.4, -1.0), castshadow=False)
  b.camera((0.3, -1.6, 1.4), (0.0, 0.0, 0.1), resolution=(res, res))
  mjm, mjd = b.build()
  return synthetic.SyntheticScene(name="slab", mjm=mjm, mjd=mjd, nworld=1, options={"cam_res": (res, res), "render_rgb": True, "render_depth": True, "render_seg": True}, per_world={}, seed=0)


def test_flat_height_field_renders_like_its_box_on_the_oracle():
  hf = helpers.oracle_render(_solid_scene(True))
  box = helpers.oracle_render(_solid_scene(False))
  hit = hf["seg"][..., 0] >= 0
  assert 0.2 < hit.mean() < 0.9
  np.testing.assert_array_equal(hit, box["seg"][..., 0] >= 0)
  np.testing.assert_array_equal(hf["seg"][hit], box["seg"][hit])  # (geom id 0, object type geom)
  np.testing.assert_allclose(hf["depth"], box["depth"], rtol=1e-5, atol=1e-6)
  assert helpers.rgb_diff(hf["rgb"], box["rgb"]).max() <= 1


def test_terrain_scene_on_the_oracle():
  sc = synthetic.hfield_scene(seed=0, nworld=2, res=32)
  out = helpers.oracle_render(sc)
  seg = out["seg"][..., 0]
  assert (seg == 0).mean() > 0.3  # the terrain fills a good part of the view
  assert np.all(out["depth"][seg == 0] > 0)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("seed,textured", [(0, True), (1, False)])
def test_terrain_scene_matches_oracle(seed, textured):
  sc = synthetic.hfield_scene(seed=seed, nworld=3, res=48, textured=textured)
  m, d, rc = helpers.gpu_scene(sc, render_hdr=True)
  gpu = helpers.render_gpu(m, d, rc, seed=5)
  ref = helpers.oracle_render(sc, seed=5, tables=helpers.gpu_tables(rc), render_hdr=True)
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  assert diff.max() <= 1, f"max RGB difference {diff.max()}/255 at {np.argwhere(diff > 1)[:5]}"


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_terrain_path_traced_matches_oracle():
  sc = synthetic.hfield_scene(seed=2, nworld=2, res=32, textured=True)
  m, d, rc = helpers.gpu_scene(sc, tier=1, path_samples=2, max_depth=3)
  gpu = helpers.render_gpu(m, d, rc, seed=9)
  ref = helpers.oracle_render(sc, seed=9, tables=helpers.gpu_tables(rc), tier=1, path_samples=2, max_depth=3)
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  assert float(np.mean(diff <= 1)) >= 0.995
