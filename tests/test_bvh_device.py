"""Device mesh BVH builder (mjpbr_build_mesh_bvh_device, mesh_bvh_constructor="lbvh").

CPU: the oracle restatement (oracle/lbvh_oracle.py) makes valid trees (every triangle in one leaf,
children after parents, boxes around their triangles, leaves of at most 4) and the host side lays
the sources out as the C entry expects. GPU: the device build equals the oracle bit for bit
(nodes, triangles, bounds, node counts) on several sources at once, and a context built with it
renders the mesh / IBL scene at the real-time bars against the oracle renderer and with the same
segmentation and depth as the host SAH build.
"""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mujoco_warp_pbr_gb300 import _lib  # noqa: E402
from mujoco_warp_pbr_gb300 import context  # noqa: E402
from mujoco_warp_pbr_gb300 import synthetic  # noqa: E402
from oracle import lbvh_oracle  # noqa: E402

gpu = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


def _bits(a: np.ndarray) -> np.ndarray:
  return np.ascontiguousarray(a, np.float32).view(np.int32)


def _sources(seed: int = 0) -> list[tuple[np.ndarray, np.ndarray]]:
  """Meshes of 1, 3, 4, 5, 200 and 2562-vertex icosphere triangles, one with repeated centroids."""
  rng = np.random.default_rng(seed)
  out = []
  for n in (1, 3, 4, 5, 200):
    v = rng.uniform(-1, 1, (3 * n, 3)).astype(np.float32)
    out.append((v, np.arange(3 * n, dtype=np.int32).reshape(n, 3)))
  v = rng.uniform(-1, 1, (3, 3)).astype(np.float32)
  out.append((v, np.tile(np.arange(3, dtype=np.int32), (37, 1))))  # 37 identical triangles
  sv, sf = synthetic.icosphere(4)
  sv = (sv * (1.0 + 0.1 * rng.uniform(-1, 1, (len(sv), 1)))).astype(np.float32)
  out.append((sv, sf.astype(np.int32)))
  return out


def _walk(nodes: np.ndarray, tris: np.ndarray, n: int, leaf: int = 4) -> None:
  bits = _bits(nodes)
  seen = np.zeros(n, np.int64)
  for i, nd in enumerate(nodes):
    for k in range(2):
      q = nd[k * 8 : k * 8 + 8]
      ref, cnt = bits[i, k * 8 + 3], bits[i, k * 8 + 7]
      if cnt < 0:
        continue
      if cnt == 0:
        assert ref > i  # pre-order: children follow their parent
        continue
      assert 1 <= cnt <= leaf
      seen[ref : ref + cnt] += 1
      pts = tris[ref : ref + cnt].reshape(cnt, 3, 4)[..., :3].reshape(-1, 3)
      assert np.all(pts >= q[0:3]) and np.all(pts <= q[4:7])
  assert np.all(seen == 1)


def test_oracle_trees_are_valid():
  for v, f in _sources():
    t = lbvh_oracle.build(v, f)
    _walk(t["nodes"], t["tris"], len(f))
    assert len(t["nodes"]) <= max(len(f) - 1, 1)
    assert sorted(t["order"].tolist()) == list(range(len(f)))
    np.testing.assert_array_equal(t["tris"][:, 0:3], v[f[t["order"], 0]])


def test_oracle_inner_boxes_contain_children():
  v, f = _sources()[-1]
  t = lbvh_oracle.build(v, f)
  nodes, bits = t["nodes"], _bits(t["nodes"])
  for i in range(len(nodes)):
    for k in range(2):
      if bits[i, k * 8 + 7] == 0:
        c = bits[i, k * 8 + 3]
        box = nodes[i, k * 8 : k * 8 + 8]
        for kk in range(2):
          if bits[c, kk * 8 + 7] >= 0:
            child = nodes[c, kk * 8 : kk * 8 + 8]
            assert np.all(child[0:3] >= box[0:3] - 1e-4) and np.all(child[4:7] <= box[4:7] + 1e-4)


def test_morton_codes_interleave_axes():
  cen = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float32)
  c = lbvh_oracle.morton_codes(cen)
  assert c[0] == 0
  assert c[1] == 0x24924924 and c[2] == 0x12492492 and c[3] == 0x09249249  # 1023 spread, x on top
  assert c[4] == 0x3FFFFFFF


def test_device_sources_layout():
  sc = synthetic.mesh_ibl_scene(seed=0, nworld=2, res=16, tex_size=16, env_width=32)
  src = context.device_mesh_sources(sc.mjm)
  d = src["device_sources"]
  nface = np.diff(d["face_base"])
  assert len(nface) == sc.mjm.nmesh == 6
  assert d["face_base"][-1] == len(d["face"]) and d["vert_base"][-1] + d["vert_num"][-1] == len(d["vert"])
  assert np.array_equal(d["node_base"], np.concatenate([[0], np.cumsum(np.maximum(nface - 1, 1))[:-1]]))
  host = context.build_mesh_bvhs(sc.mjm)
  np.testing.assert_array_equal(src["mesh_bounds"], host["mesh_bounds"])
  bad = synthetic.Builder()
  bad.mesh(np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.int32), normal=np.zeros((3, 3), np.float32))
  bad.geom(synthetic.GEOM_MESH, (1, 1, 1), dataid=0)
  mjm, _ = bad.build()
  with pytest.raises(ValueError, match="out of range"):
    context.device_mesh_sources(mjm)


def test_scratch_size_entry():
  lib = _lib.load()
  assert lib.mjpbr_mesh_bvh_device_scratch_bytes(0, 10) == -1
  assert lib.mjpbr_mesh_bvh_device_scratch_bytes(3, 2) == -1
  small, big = lib.mjpbr_mesh_bvh_device_scratch_bytes(2, 100), lib.mjpbr_mesh_bvh_device_scratch_bytes(2, 100000)
  assert 0 < small < big and big >= 100000 * (8 + 8 + 4 + 4 + 32)


def _device_build(sources, leaf: int = 4):
  nface = np.array([len(f) for _, f in sources])
  nvert = np.array([len(v) for v, _ in sources])
  arr = {
    "vert": np.concatenate([v for v, _ in sources]).astype(np.float32),
    "face": np.concatenate([f for _, f in sources]).astype(np.int32),
    "vert_base": np.concatenate([[0], np.cumsum(nvert)[:-1]]).astype(np.int32),
    "vert_num": nvert.astype(np.int32),
    "face_base": np.concatenate([[0], np.cumsum(nface)]).astype(np.int32),
    "node_base": np.concatenate([[0], np.cumsum(np.maximum(nface - 1, 1))[:-1]]).astype(np.int32),
    "nodes": int(np.maximum(nface - 1, 1).sum()),
    "names": [f"source {i}" for i in range(len(sources))],
  }
  return arr, context.build_mesh_bvhs_device(arr, torch.device("cuda", 0))


@pytest.mark.gpu
@gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_device_build_matches_oracle(seed):
  sources = _sources(seed)
  arr, built = _device_build(sources)
  nodes = built["blas_nodes"].cpu().numpy()
  tris = built["blas_tris"].cpu().numpy()
  bounds = built["mesh_bounds"].cpu().numpy()
  for s, (v, f) in enumerate(sources):
    ref = lbvh_oracle.build(v, f)
    nb, fb, nn = arr["node_base"][s], arr["face_base"][s], int(built["node_count"][s])
    assert nn == len(ref["nodes"]), f"source {s}: {nn} nodes, oracle {len(ref['nodes'])}"
    np.testing.assert_array_equal(_bits(nodes[nb : nb + nn]), _bits(ref["nodes"]), err_msg=f"source {s} nodes")
    np.testing.assert_array_equal(_bits(tris[fb : fb + len(f)]), _bits(ref["tris"]), err_msg=f"source {s} triangles")
    np.testing.assert_array_equal(bounds[s], ref["bounds"])
    _walk(nodes[nb : nb + nn], tris[fb : fb + len(f)], len(f))


@pytest.mark.gpu
@gpu
def test_device_build_reports_bad_faces():
  """A face naming a vertex out of range is clamped to vertex 0 and reported (error bit 16)."""
  dev = torch.device("cuda", 0)
  vert = torch.rand((3, 3), device=dev)
  face = torch.tensor([[0, 1, 2], [0, 1, 7]], dtype=torch.int32, device=dev)
  z = lambda *a: torch.tensor(a, dtype=torch.int32, device=dev)  # noqa: E731
  vb, vn, fb, nb = z(0), z(3), z(0, 2), z(0)
  nodes = torch.zeros((1, 16), device=dev)
  tris = torch.zeros((2, 12), device=dev)
  bounds = torch.zeros((1, 6), device=dev)
  nnode, err = z(0), z(0)
  nbytes = int(_lib.load().mjpbr_mesh_bvh_device_scratch_bytes(1, 2))
  scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
  _lib.call(
    "mjpbr_build_mesh_bvh_device", vert.data_ptr(), face.data_ptr(), vb.data_ptr(), vn.data_ptr(), fb.data_ptr(), nb.data_ptr(), 1, 2, 4,
    nodes.data_ptr(), tris.data_ptr(), bounds.data_ptr(), nnode.data_ptr(), scratch.data_ptr(), nbytes, err.data_ptr(), torch.cuda.current_stream().cuda_stream,
  )
  torch.cuda.synchronize()
  assert int(err.item()) == 16 and int(nnode.item()) == 1
  with pytest.raises(ValueError, match="scratch"):
    _lib.call(
      "mjpbr_build_mesh_bvh_device", vert.data_ptr(), face.data_ptr(), vb.data_ptr(), vn.data_ptr(), fb.data_ptr(), nb.data_ptr(), 1, 2, 4,
      nodes.data_ptr(), tris.data_ptr(), bounds.data_ptr(), nnode.data_ptr(), scratch.data_ptr(), 16, err.data_ptr(), torch.cuda.current_stream().cuda_stream,
    )


@pytest.mark.gpu
@gpu
def test_lbvh_context_renders_like_the_oracle():
  from tests import helpers

  sc = synthetic.mesh_ibl_scene(seed=1, nworld=2, res=48, tex_size=64, env_width=128)
  m, d, rc = helpers.gpu_scene(sc, mesh_bvh_constructor="lbvh", render_hdr=True)
  gpu_img = helpers.render_gpu(m, d, rc, seed=3)
  ref = helpers.oracle_render(sc, seed=3, tables=helpers.gpu_tables(rc), render_hdr=True)
  np.testing.assert_array_equal(gpu_img["seg"], ref["seg"])
  np.testing.assert_allclose(gpu_img["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu_img["rgb"], ref["rgb"])
  assert diff.max() <= 1
  m2, d2, rc2 = helpers.gpu_scene(sc, render_hdr=True)
  sah = helpers.render_gpu(m2, d2, rc2, seed=3)
  np.testing.assert_array_equal(gpu_img["seg"], sah["seg"])
  np.testing.assert_array_equal(gpu_img["depth"], sah["depth"])
  assert helpers.rgb_diff(gpu_img["rgb"], sah["rgb"]).max() <= 1


def test_default_constructor_builds_large_models_on_the_device():
  for grid in (2, 5, 33):
    sc = synthetic.hfield_scene(seed=0, nworld=1, res=8, grid=grid)
    faces = sum(len(f) for _, _, f in context.mesh_sources(sc.mjm))
    assert context.total_bvh_faces(sc.mjm) == faces
  small = synthetic.mesh_ibl_scene(seed=0, nworld=1, res=8, tex_size=16, env_width=32)
  hc = context.prepare_context(small.mjm, 1, data=small.mjd, **{**small.options, "envmap": None})
  assert "device_sources" not in hc.meshes and hc.meshes["blas_nodes"] is not None
  v, f = synthetic.icosphere(7)
  b = synthetic.Builder()
  b.mesh(v, f, normal=v.astype(np.float32))
  b.geom(synthetic.GEOM_MESH, (1, 1, 1), dataid=0)
  b.light(synthetic.LIGHT_DIRECTIONAL)
  b.camera((0, -3, 1), (0, 0, 0))
  mjm, mjd = b.build()
  assert context.total_bvh_faces(mjm) >= context.DEVICE_BVH_FACES
  hc = context.prepare_context(mjm, 1, data=mjd)
  assert "device_sources" in hc.meshes
  hc = context.prepare_context(mjm, 1, data=mjd, mesh_bvh_constructor="sah")
  assert "device_sources" not in hc.meshes
