"""CPU restatement of the device mesh BVH builder (mjpbr_build_mesh_bvh_device) — TEST
INFRASTRUCTURE ONLY.

The device builder makes linear BVHs in the record layout of the host SAH builder; this module
restates its algorithm in NumPy / Python so tests can compare the GPU's nodes, triangles, bounds
and node counts bit for bit:

  1. per source, centroid bounds of the triangle boxes (centroid = 0.5 * (lo + hi), float32);
  2. 30-bit Morton code of each centroid: per axis u = (c - c0) / (c1 - c0) * 1024 (0 when the
     extent is 0), clamped to [0, 1023], truncated, bits interleaved x, y, z from the top;
  3. a stable sort of (source << 30 | code) keys;
  4. Karras' binary radix tree per source (T. Karras, "Maximizing parallelism in the construction
     of BVHs, octrees, and k-d trees", HPG 2012), equal codes ordered by position;
  5. a subtree of at most leaf_size triangles becomes one leaf (first triangle, count); inner nodes
     are numbered in pre-order, left before right; a source of at most leaf_size triangles is a
     root with one leaf child and one empty child (count -1);
  6. child boxes padded by 1e-5 * (1 + max(|lo|, |hi|)) per axis, as the host builder pads.

The reference gets its mesh BVHs from Warp (wp.Mesh bvh_constructor "lbvh" / "cubql",
mujoco_warp_pbr/_src/io.py:164-179); Warp's builder is third-party code not in the reference tree,
so this is a restatement of the published algorithm, not of Warp's code. Only tests/ use it.
"""

from __future__ import annotations

import numpy as np

f32 = np.float32


def _spread10(x: np.ndarray) -> np.ndarray:
  x = x.astype(np.uint32) & np.uint32(0x3FF)
  x = (x | (x << np.uint32(16))) & np.uint32(0x030000FF)
  x = (x | (x << np.uint32(8))) & np.uint32(0x0300F00F)
  x = (x | (x << np.uint32(4))) & np.uint32(0x030C30C3)
  x = (x | (x << np.uint32(2))) & np.uint32(0x09249249)
  return x


def morton_codes(cen: np.ndarray) -> np.ndarray:
  """30-bit codes of centroids (n, 3) float32 within their own bounds."""
  c0, c1 = cen.min(axis=0), cen.max(axis=0)
  code = np.zeros(len(cen), np.uint32)
  for k in range(3):
    ext = f32(c1[k] - c0[k])
    if ext > 0:
      u = (cen[:, k] - c0[k]) / ext * f32(1024.0)
    else:
      u = np.zeros(len(cen), f32)
    u = np.minimum(np.maximum(u, f32(0.0)), f32(1023.0))
    code |= _spread10(u.astype(np.uint32)) << np.uint32(2 - k)
  return code


def _clz32(x: int) -> int:
  return 32 - int(x).bit_length()


def _radix_tree(codes: np.ndarray) -> list[tuple[int, int, int, int]]:
  """Inner nodes i of Karras' tree over sorted codes: (first, last, left, right), a child >= 0 an
  inner node, < 0 the leaf ~position."""
  n = len(codes)
  c = [int(v) for v in codes]

  def delta(i: int, j: int) -> int:
    if j < 0 or j >= n:
      return -1
    if c[i] == c[j]:
      return 32 + _clz32(i ^ j)
    return _clz32(c[i] ^ c[j])

  nodes = []
  for i in range(n - 1):
    d = 1 if delta(i, i + 1) > delta(i, i - 1) else -1
    dmin = delta(i, i - d)
    lmax = 2
    while delta(i, i + lmax * d) > dmin:
      lmax *= 2
    l, step = 0, lmax // 2
    while step >= 1:
      if delta(i, i + (l + step) * d) > dmin:
        l += step
      step //= 2
    j = i + l * d
    dnode = delta(i, j)
    s, step = 0, l
    while True:
      step = (step + 1) >> 1
      if delta(i, i + (s + step) * d) > dnode:
        s += step
      if step <= 1:
        break
    gamma = i + s * d + min(d, 0)
    first, last = min(i, j), max(i, j)
    left = ~gamma if first == gamma else gamma
    right = ~(gamma + 1) if last == gamma + 1 else gamma + 1
    nodes.append((first, last, left, right))
  return nodes


def _pad_child(lo: np.ndarray, hi: np.ndarray, ref: int, count: int) -> np.ndarray:
  q = np.zeros(8, f32)
  for a in range(3):
    pad = f32(1.0e-5) * (f32(1.0) + max(abs(lo[a]), abs(hi[a])))
    q[a] = f32(lo[a] - pad)
    q[4 + a] = f32(hi[a] + pad)
  q[3:4] = np.array([ref], np.int32).view(f32)
  q[7:8] = np.array([count], np.int32).view(f32)
  return q


def build(vert: np.ndarray, face: np.ndarray, leaf_size: int = 4) -> dict[str, np.ndarray]:
  """One source: nodes (nnode, 16) float32 (int fields as their bits), tris (nface, 12) float32,
  bounds (6,) float32, order (nface,) face index of each leaf position."""
  v = np.asarray(vert, f32).reshape(-1, 3)
  f = np.asarray(face, np.int64).reshape(-1, 3)
  p = v[f]  # (n, 3 corners, 3)
  lo, hi = p.min(axis=1), p.max(axis=1)
  cen = f32(0.5) * (lo + hi)
  codes = morton_codes(cen)
  order = np.argsort(codes, kind="stable")
  sc = codes[order]
  n = len(f)
  bounds = np.concatenate([lo.min(axis=0), hi.max(axis=0)]).astype(f32)
  tris = np.zeros((n, 12), f32)
  tris[:, 0:3], tris[:, 4:7], tris[:, 8:11] = p[order, 0], p[order, 1], p[order, 2]
  tris[:, 3] = order.astype(np.int32).view(f32)
  slo, shi = lo[order], hi[order]

  def range_box(a: int, b: int) -> tuple[np.ndarray, np.ndarray]:
    return slo[a : b + 1].min(axis=0), shi[a : b + 1].max(axis=0)

  if n <= leaf_size:
    node = np.zeros(16, f32)
    node[:8] = _pad_child(bounds[:3], bounds[3:], 0, n)
    node[11:12] = np.array([0], np.int32).view(f32)
    node[15:16] = np.array([-1], np.int32).view(f32)
    return {"nodes": node[None], "tris": tris, "bounds": bounds, "order": order}

  inner = _radix_tree(sc)
  size: dict[int, int] = {}

  def inner_size(g: int) -> int:
    if g not in size:
      first, last, left, right = inner[g]
      if last - first + 1 <= leaf_size:
        size[g] = 0
      else:
        size[g] = 1 + (inner_size(left) if left >= 0 else 0) + (inner_size(right) if right >= 0 else 0)
    return size[g]

  out: list[np.ndarray] = []

  def emit(g: int) -> None:
    pos = len(out)
    out.append(np.zeros(16, f32))
    first, last, left, right = inner[g]
    recs = []
    for k, ch in enumerate((left, right)):
      if ch < 0:
        b = range_box(~ch, ~ch)
        recs.append((b, ~ch, 1, None))
      elif inner_size(ch) == 0:
        cf, cl = inner[ch][0], inner[ch][1]
        recs.append((range_box(cf, cl), cf, cl - cf + 1, None))
      else:
        cf, cl = inner[ch][0], inner[ch][1]
        recs.append((range_box(cf, cl), 0, 0, ch))
    # pre-order: the left inner child right after this node, the right one after the left subtree
    left_size = inner_size(left) if left >= 0 else 0
    node = out[pos]
    for k, (box, ref, count, ch) in enumerate(recs):
      if ch is not None:
        ref = pos + 1 + (left_size if k == 1 else 0)
      node[k * 8 : k * 8 + 8] = _pad_child(box[0], box[1], ref, count)
    for ch in (left, right):
      if ch >= 0 and inner_size(ch) > 0:
        emit(ch)

  import sys

  limit = sys.getrecursionlimit()
  sys.setrecursionlimit(max(limit, 10000))
  try:
    emit(0)
  finally:
    sys.setrecursionlimit(limit)
  return {"nodes": np.stack(out), "tris": tris, "bounds": bounds, "order": order}
