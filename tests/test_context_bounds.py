"""Context creation: the world-batched geom bounds that seed the per-world scene BVHs equal the
per-world computation for every geom type (CPU only)."""

from types import SimpleNamespace

import numpy as np

from mujoco_warp_pbr_gb300 import context


def _rotations(rng, shape):
  q = rng.normal(size=shape + (4,))
  q /= np.linalg.norm(q, axis=-1, keepdims=True)
  w, x, y, z = np.moveaxis(q, -1, 0)
  return np.stack(
    [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w), 2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
     2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    -1,
  )


def test_batched_bounds_match_per_world_bounds():
  rng = np.random.default_rng(11)
  types = np.array([
    context.GEOM_PLANE, context.GEOM_PLANE, context.GEOM_SPHERE, context.GEOM_CAPSULE, context.GEOM_ELLIPSOID, context.GEOM_CYLINDER,
    context.GEOM_BOX, context.GEOM_MESH, context.GEOM_MESH, context.GEOM_SDF, context.GEOM_HFIELD,
  ])
  size = rng.uniform(0.05, 0.5, size=(len(types), 3))
  size[0, :2] = 0.0  # an infinite plane
  dataid = np.array([-1, -1, -1, -1, -1, -1, -1, 0, 1, 0, 0])
  # two meshes and one height field: BVH bounds of the meshes, then of the height field
  mjm = SimpleNamespace(geom_type=types, geom_size=size, geom_dataid=dataid, nmesh=2, hfield_nrow=np.array([3]))
  mesh_bounds = rng.normal(size=(3, 6))
  mesh_bounds[:, 3:] = mesh_bounds[:, :3] + np.abs(mesh_bounds[:, 3:])
  nworld = 5
  xpos = rng.normal(size=(nworld, len(types), 3))
  xmat = _rotations(rng, (nworld, len(types)))
  lo_all, hi_all = context.geom_aabbs_all(mjm, xpos, xmat, mesh_bounds)
  for w in range(nworld):
    lo, hi = context.geom_aabbs(mjm, xpos[w], xmat[w], mesh_bounds)
    np.testing.assert_allclose(lo_all[w], lo, rtol=0, atol=1e-12)
    np.testing.assert_allclose(hi_all[w], hi, rtol=0, atol=1e-12)
  # the height field is bounded by its own BVH box (index nmesh + 0), not by its geom size
  R = xmat[0, -1].reshape(3, 3)
  mb = mesh_bounds[2]
  centre = xpos[0, -1] + R @ (0.5 * (mb[:3] + mb[3:]))
  half = np.abs(R) @ (0.5 * (mb[3:] - mb[:3]))
  np.testing.assert_allclose(lo_all[0, -1], centre - half, atol=1e-12)
  np.testing.assert_allclose(hi_all[0, -1], centre + half, atol=1e-12)
