// Host-side BVH builders of libmjpbr: binned-SAH binary trees for the per-world scene BVH (one
// geom per leaf) and for each mesh (up to 4 triangles per leaf). They stand in for the builders
// the reference gets from its dependencies (the scene wp.Bvh of mujoco_warp.create_render_context,
// mujoco_warp_pbr/_src/io.py:511-528, and the per-mesh wp.Mesh BVHs, io.py:164-179,198-203).
// Nodes are emitted in pre-order, so every child follows its parent and a reverse sweep refits
// bottom-up; deep trees fall back to median splits so traversal stacks stay bounded.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "mjpbr.h"

namespace {

constexpr int kBins = 32;
constexpr int kMedianDepth = 22;  // below this depth, always split at the median

struct Box {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void grow(const Box& b) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], b.lo[a]);
      hi[a] = std::max(hi[a], b.hi[a]);
    }
  }
  void grow(const float* p) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], p[a]);
      hi[a] = std::max(hi[a], p[a]);
    }
  }
  float area() const {
    if (lo[0] > hi[0]) return 0.0f;
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.0f * (dx * dy + dy * dz + dz * dx);
  }
};

struct Builder {
  std::vector<Box> prim;
  std::vector<float> cen;  // 3 per prim
  std::vector<int> order;
  int leaf_size = 1;
  // output
  struct Child {
    Box box;
    int ref;    // inner node index or first primitive (in `order`)
    int count;  // 0 inner, > 0 leaf, -1 empty
  };
  struct Node {
    Child c[2];
  };
  std::vector<Node> nodes;

  // Splits order[begin, end) in two non-empty halves; returns the split position.
  int split(int begin, int end, int depth) {
    int n = end - begin;
    Box cb;
    for (int i = begin; i < end; ++i) cb.grow(&cen[order[i] * 3]);
    int axis = 0;
    float ext = -1.0f;
    for (int a = 0; a < 3; ++a) {
      if (cb.hi[a] - cb.lo[a] > ext) {
        ext = cb.hi[a] - cb.lo[a];
        axis = a;
      }
    }
    if (ext > 0.0f && depth < kMedianDepth && n > 2) {
      float best_cost = FLT_MAX;
      int best_axis = -1, best_bin = -1;
      for (int a = 0; a < 3; ++a) {
        float lo = cb.lo[a], w = cb.hi[a] - cb.lo[a];
        if (w <= 0.0f) continue;
        Box bins[kBins];
        int cnt[kBins] = {0};
        for (int i = begin; i < end; ++i) {
          int b = std::min(kBins - 1, (int)((cen[order[i] * 3 + a] - lo) / w * kBins));
          bins[b].grow(prim[order[i]]);
          cnt[b]++;
        }
        Box left[kBins];
        int lc[kBins];
        Box acc;
        int ac = 0;
        for (int b = 0; b < kBins; ++b) {
          acc.grow(bins[b]);
          ac += cnt[b];
          left[b] = acc;
          lc[b] = ac;
        }
        acc = Box();
        ac = 0;
        for (int b = kBins - 1; b > 0; --b) {
          acc.grow(bins[b]);
          ac += cnt[b];
          if (lc[b - 1] == 0 || ac == 0) continue;
          float cost = left[b - 1].area() * lc[b - 1] + acc.area() * ac;
          if (cost < best_cost) {
            best_cost = cost;
            best_axis = a;
            best_bin = b;
          }
        }
      }
      if (best_axis >= 0) {
        float lo = cb.lo[best_axis], w = cb.hi[best_axis] - cb.lo[best_axis];
        int* mid = std::partition(order.data() + begin, order.data() + end, [&](int p) {
          int b = std::min(kBins - 1, (int)((cen[p * 3 + best_axis] - lo) / w * kBins));
          return b < best_bin;
        });
        int m = (int)(mid - order.data());
        if (m > begin && m < end) return m;
      }
    }
    // median split along the widest centroid axis
    int m = begin + n / 2;
    std::nth_element(order.data() + begin, order.data() + m, order.data() + end,
                     [&](int a, int b) { return cen[a * 3 + axis] < cen[b * 3 + axis]; });
    return m;
  }

  Child build(int begin, int end, int depth) {
    Child ch;
    for (int i = begin; i < end; ++i) ch.box.grow(prim[order[i]]);
    if (end - begin <= leaf_size) {
      ch.ref = begin;
      ch.count = end - begin;
      return ch;
    }
    int idx = (int)nodes.size();
    nodes.emplace_back();
    int m = split(begin, end, depth);
    Child a = build(begin, m, depth + 1);
    Child b = build(m, end, depth + 1);
    nodes[idx].c[0] = a;
    nodes[idx].c[1] = b;
    ch.ref = idx;
    ch.count = 0;
    return ch;
  }

  // Builds the tree; a single leaf becomes a root node with one empty child.
  void run() {
    int n = (int)prim.size();
    order.resize(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    cen.resize(n * 3);
    for (int i = 0; i < n; ++i) {
      for (int a = 0; a < 3; ++a) cen[i * 3 + a] = 0.5f * (prim[i].lo[a] + prim[i].hi[a]);
    }
    nodes.clear();
    if (n <= leaf_size) {
      Node root;
      for (int i = 0; i < n; ++i) root.c[0].box.grow(prim[i]);
      root.c[0].ref = 0;
      root.c[0].count = n;
      root.c[1].ref = 0;
      root.c[1].count = -1;
      nodes.push_back(root);
      return;
    }
    build(0, n, 0);
  }
};

}  // namespace

extern "C" {

int32_t mjpbr_bvh_node_count(int32_t nprim) { return nprim > 1 ? nprim - 1 : 1; }

int mjpbr_build_scene_bvh(const float* lower, const float* upper, int32_t nprim, int32_t* child_out) {
  if (!lower || !upper || !child_out || nprim < 1) return MJPBR_ERR_ARG;
  Builder b;
  b.leaf_size = 1;
  b.prim.resize(nprim);
  for (int i = 0; i < nprim; ++i) {
    for (int a = 0; a < 3; ++a) {
      b.prim[i].lo[a] = lower[i * 3 + a];
      b.prim[i].hi[a] = upper[i * 3 + a];
    }
  }
  b.run();
  int32_t nnode = mjpbr_bvh_node_count(nprim);
  if ((int32_t)b.nodes.size() != nnode) return MJPBR_ERR_ARG;
  for (int i = 0; i < nnode; ++i) {
    for (int k = 0; k < 2; ++k) {
      const Builder::Child& c = b.nodes[i].c[k];
      int32_t v;
      if (c.count < 0) {
        v = INT32_MIN;
      } else if (c.count == 0) {
        v = c.ref;
      } else {
        v = ~b.order[c.ref];  // one primitive per leaf: its slot
      }
      child_out[i * 2 + k] = v;
    }
  }
  return MJPBR_OK;
}

int mjpbr_build_mesh_bvh(const float* vert, int32_t nvert, const int32_t* face, int32_t nface, int32_t leaf_size,
                         float* nodes_out, float* tris_out, float* bounds_out, int32_t* nnode_out) {
  if (!vert || !face || !nodes_out || !tris_out || !bounds_out || nface < 1 || nvert < 3 || leaf_size < 1 ||
      leaf_size > 7) {
    return MJPBR_ERR_ARG;
  }
  for (int i = 0; i < nface * 3; ++i) {
    if (face[i] < 0 || face[i] >= nvert) return MJPBR_ERR_ARG;
  }
  Builder b;
  b.leaf_size = leaf_size;
  b.prim.resize(nface);
  Box all;
  for (int f = 0; f < nface; ++f) {
    for (int k = 0; k < 3; ++k) b.prim[f].grow(vert + face[f * 3 + k] * 3);
    all.grow(b.prim[f]);
  }
  b.run();
  // triangles in leaf order: v0 (face id in w), v1, v2
  for (int i = 0; i < nface; ++i) {
    int f = b.order[i];
    float* t = tris_out + i * 12;
    for (int k = 0; k < 3; ++k) {
      const float* p = vert + face[f * 3 + k] * 3;
      t[k * 4] = p[0];
      t[k * 4 + 1] = p[1];
      t[k * 4 + 2] = p[2];
      t[k * 4 + 3] = 0.0f;
    }
    int32_t fid = f;
    std::memcpy(&t[3], &fid, 4);
  }
  int32_t nnode = (int32_t)b.nodes.size();
  for (int i = 0; i < nnode; ++i) {
    float* o = nodes_out + i * 16;
    for (int k = 0; k < 2; ++k) {
      const Builder::Child& c = b.nodes[i].c[k];
      float* q = o + k * 8;
      bool empty = c.count < 0;
      for (int a = 0; a < 3; ++a) {
        // conservative padding: the box test rounds differently from the triangle test
        float pad = 1.0e-5f * (1.0f + std::max(std::fabs(c.box.lo[a]), std::fabs(c.box.hi[a])));
        q[a] = empty ? 0.0f : c.box.lo[a] - pad;
        q[4 + a] = empty ? 0.0f : c.box.hi[a] + pad;
      }
      int32_t ref = c.ref, cnt = c.count;
      std::memcpy(&q[3], &ref, 4);
      std::memcpy(&q[7], &cnt, 4);
    }
  }
  for (int a = 0; a < 3; ++a) {
    bounds_out[a] = all.lo[a];
    bounds_out[3 + a] = all.hi[a];
  }
  *nnode_out = nnode;
  return MJPBR_OK;
}

}  // extern "C"
