"""Traversal stack sizing: the host computes how many stack entries a scene's BVHs can need
(settings.stack_depth) and the kernels size their shared-memory stacks to it. The bound is checked
here against a simulated nearest-first traversal that pushes every child (the most a ray can push),
over scene trees from libmjpbr's scene builder with mesh trees from its mesh builder at their leaves
(no GPU needed)."""

import numpy as np
import pytest

from mujoco_warp_pbr_gb300 import _lib, context


def _scene_tree(n: int, rng) -> np.ndarray:
  lo = rng.uniform(-5, 5, (n, 3))
  hi = lo + rng.uniform(0.01, 2.0, (n, 3))
  return context.build_scene_topology(lo, hi)


def _mesh_nodes(nface: int, rng) -> np.ndarray:
  import ctypes

  lib = _lib.load()
  vert = rng.uniform(-1, 1, (nface * 3, 3)).astype(np.float32)
  face = np.arange(nface * 3, dtype=np.int32).reshape(nface, 3)
  nodes = np.zeros((lib.mjpbr_bvh_node_count(nface), 16), np.float32)
  tris = np.zeros((nface, 12), np.float32)
  bnd = np.zeros(6, np.float32)
  nnode = ctypes.c_int32(0)
  assert lib.mjpbr_build_mesh_bvh(vert.ctypes.data, len(vert), face.ctypes.data, nface, 4, nodes.ctypes.data, tris.ctypes.data,
                                  bnd.ctypes.data, ctypes.byref(nnode)) == 0
  return nodes[: nnode.value]


def _levels_recursive(children) -> int:
  def rec(i):
    return 1 + max([rec(c) for c in children(i)] or [0])

  return rec(0)


def _max_stack(scene_children, mesh_children) -> int:
  """Most entries a nearest-first traversal holds when every box is hit: scene entries, then the mesh
  traversal above them at each scene leaf (pop one, push both children)."""
  most = 0
  stack = [0]
  while stack:
    most = max(most, len(stack))
    ref = stack.pop()
    if ref is None:  # a scene leaf: the mesh traversal runs above the remaining entries
      base = len(stack)
      mstack = [0]
      while mstack:
        most = max(most, base + len(mstack))
        mstack.extend(mesh_children(mstack.pop()))
      continue
    stack.extend(scene_children(ref))
  return most


@pytest.mark.parametrize("nprim,nface,seed", [(1, 1, 0), (2, 5, 1), (9, 64, 2), (57, 300, 3), (400, 2000, 4)])
def test_stack_bound_covers_the_deepest_traversal(nprim, nface, seed):
  rng = np.random.default_rng(seed)
  topo = _scene_tree(nprim, rng)
  nodes = _mesh_nodes(nface, rng)
  bits = nodes.view(np.int32)
  empty = np.iinfo(np.int32).min

  def scene_children(i):  # inner children as node ids, leaves (a geom each) as None
    return [int(c) if c >= 0 else None for c in topo[i] if c != empty]

  def mesh_children(i):  # inner children as node ids, leaves (triangles) as -1
    return [int(bits[i, 8 * k + 3]) if bits[i, 8 * k + 7] == 0 else -1 for k in (0, 1) if bits[i, 8 * k + 7] >= 0]

  scene_levels = context.scene_tree_levels(topo[None])
  mesh_levels = context.mesh_tree_levels(nodes)
  assert scene_levels == _levels_recursive(lambda i: [c for c in scene_children(i) if c is not None])
  assert mesh_levels == _levels_recursive(lambda i: [c for c in mesh_children(i) if c >= 0])
  most = _max_stack(scene_children, lambda node: [] if node < 0 else mesh_children(node))
  assert most <= scene_levels + mesh_levels + 1
  depth = context.traversal_stack_depth(scene_levels, mesh_levels)
  assert depth >= min(most, 32) and 8 <= depth <= 32


def test_per_world_topologies_take_the_deepest():
  a = _scene_tree(33, np.random.default_rng(7))
  b = _scene_tree(33, np.random.default_rng(8))
  both = np.stack([a, b])
  assert context.scene_tree_levels(both) == max(context.scene_tree_levels(a[None]), context.scene_tree_levels(b[None]))


def test_stack_depth_reaches_the_settings():
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.hfield_scene(seed=1, nworld=2, res=8, grid=9)
  options = {k: v for k, v in sc.options.items() if k != "device"}
  hc = context.prepare_context(sc.mjm, sc.nworld, data=sc.mjd, **options)
  levels = context.scene_tree_levels(hc.tlas_child)
  want = context.traversal_stack_depth(levels, hc.meshes["mesh_levels"])
  assert hc.settings["stack_depth"] == want
  assert hc.meshes["mesh_levels"] >= 1


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", ["grid", "wavefront"])
def test_a_stack_too_shallow_for_the_scene_is_reported(schedule):
  """Rendering the mesh scene with fewer stack entries than its BVHs need: every push past the
  stack's end is dropped (never written) and reported in the error word; with the computed depth
  the same frame reports nothing."""
  import ctypes

  torch = pytest.importorskip("torch")
  if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU")
  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import synthetic
  from tests import helpers

  sc = synthetic.mesh_ibl_scene(seed=2, nworld=2, res=48, tex_size=64, env_width=128)
  m, d, rc = helpers.gpu_scene(sc, schedule=schedule)
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=1)
  assert mjpbr.check_errors(rc) == 0
  s = _lib.Scene.from_buffer_copy(mjpbr.scene_descriptor(m, d, rc))
  assert s.settings.stack_depth > 8
  s.settings.stack_depth = 8
  stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
  lib = _lib.load()
  assert lib.mjpbr_render(ctypes.byref(s), 1, stream) == 0, lib.mjpbr_last_error().decode()
  assert mjpbr.check_errors(rc) & 1, "no stack overflow reported"
