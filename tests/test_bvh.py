"""Host BVH builders of libmjpbr (scene and mesh trees): structural invariants."""

import numpy as np

from mujoco_warp_pbr_gb300 import context
from mujoco_warp_pbr_gb300 import synthetic


def _walk_scene(child: np.ndarray):
  leaves, order_ok = [], True
  stack = [0]
  while stack:
    i = stack.pop()
    for c in child[i]:
      if c == np.iinfo(np.int32).min:
        continue
      if c < 0:
        leaves.append(~c)
      else:
        order_ok &= c > i
        stack.append(c)
  return leaves, order_ok


def test_scene_bvh_covers_every_slot_once():
  rng = np.random.default_rng(0)
  for n in (1, 2, 3, 9, 17, 64):
    c = rng.uniform(-1, 1, (n, 3))
    e = rng.uniform(0.01, 0.3, (n, 3))
    child = context.build_scene_topology(c - e, c + e)
    assert child.shape == (max(n - 1, 1), 2)
    leaves, order_ok = _walk_scene(child)
    assert sorted(leaves) == list(range(n))
    assert order_ok  # children follow their parent: a reverse sweep refits bottom-up


def test_mesh_bvh_bounds_and_triangles():
  v, f = synthetic.icosphere(3)
  b = synthetic.Builder()
  b.mesh(v, f)
  b.geom(synthetic.GEOM_MESH, (1, 1, 1), dataid=0)
  mjm, _ = b.build()
  m = context.build_mesh_bvhs(mjm)
  nodes, tris = m["blas_nodes"], m["blas_tris"]
  assert tris.shape == (len(f), 12)
  faces = tris[:, 3].view(np.int32)
  assert sorted(faces.tolist()) == list(range(len(f)))
  # triangles are stored with their original vertices
  np.testing.assert_array_equal(tris[:, 0:3], v[f[faces, 0]])
  np.testing.assert_array_equal(tris[:, 4:7], v[f[faces, 1]])
  # every leaf's triangles lie inside the child box that references them
  seen = 0
  for nd in nodes:
    for k in range(2):
      q = nd[k * 8 : k * 8 + 8]
      cnt = q[7:8].view(np.int32)[0]
      ref = q[3:4].view(np.int32)[0]
      if cnt > 0:
        assert cnt <= 4
        pts = np.concatenate([tris[ref : ref + cnt, 0:3], tris[ref : ref + cnt, 4:7], tris[ref : ref + cnt, 8:11]])
        assert np.all(pts >= q[0:3]) and np.all(pts <= q[4:7])
        seen += cnt
  assert seen == len(f)
  np.testing.assert_allclose(m["mesh_bounds"][0], np.concatenate([v.min(0), v.max(0)]), atol=1e-6)
