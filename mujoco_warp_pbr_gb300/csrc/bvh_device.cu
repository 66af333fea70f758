// Device builder of the triangle BVHs (the BLAS of every mesh and height field of a context) as
// linear BVHs: Morton codes of triangle centroids within each source's centroid bounds, one
// stable radix sort of (source, code) keys over every source at once, Karras' binary radix tree
// per source (one thread per inner node), a bottom-up pass for the boxes, and an emission pass
// that turns every subtree of at most leaf_size triangles into one leaf and writes the nodes in
// pre-order. The records are those of the host builder (mjpbr_build_mesh_bvh), so the render
// kernels read either. It stands in for the GPU mesh BVH builds the reference gets from Warp
// (wp.Mesh with bvh_constructor "lbvh" / "cubql", mujoco_warp_pbr/_src/io.py:164-179).
//
// Launches: bounds (per triangle), Morton keys (per triangle), 2 x passes radix sort (histogram +
// one-CTA scan + scatter per 8-bit digit), hierarchy (per inner node), boxes (per leaf, walking
// up with one atomic per node), emission (per inner node) and triangles (per triangle).
#include "abi_internal.h"
#include "common.cuh"

namespace mjpbr {
namespace {

constexpr int kThreads = 256;
constexpr int kSortThreads = 1024;  // keys per radix-sort tile (one per thread)
constexpr int kDigits = 256;
constexpr int kWarps = kSortThreads / 32;
static_assert(kWarps == 32, "the scan's second level is one warp");

// Order-preserving map of floats to unsigned integers (for atomicMin / atomicMax of bounds).
__device__ __forceinline__ uint32_t ordered(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Source of face f: the last s with face_base[s] <= f.
__device__ __forceinline__ int32_t source_of(const int32_t* __restrict__ face_base, int32_t nsrc, int32_t f) {
  int32_t lo = 0, hi = nsrc - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(face_base + mid) <= f) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct Inputs {
  const float* vert;       // (nvert_total, 3)
  const int32_t* face;     // (nface_total, 3), vertex indices local to the face's source
  const int32_t* vert_base;  // (nsrc,)
  const int32_t* vert_num;   // (nsrc,)
  const int32_t* face_base;  // (nsrc + 1,) face_base[nsrc] = nface_total
  int32_t nsrc, nface;
  int32_t* error_word;
};

// Vertex c of face f (global index) of source s.
__device__ __forceinline__ float3 vertex(const Inputs& in, int32_t s, int32_t f, int c, bool* bad) {
  int32_t v = __ldg(in.face + (int64_t)f * 3 + c);
  if (v < 0 || v >= __ldg(in.vert_num + s)) {
    *bad = true;
    v = 0;
  }
  const float* p = in.vert + ((int64_t)__ldg(in.vert_base + s) + v) * 3;
  return make_float3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

// Triangle boxes (original order) and per-source bounds of centroids and of triangles.
// bmin (nsrc, 6): centroid min, box min as ordered uints; bmax likewise for the maxima.
__global__ void __launch_bounds__(kThreads) tri_bounds_kernel(Inputs in, float4* __restrict__ tri_box,
                                                              uint32_t* __restrict__ bmin, uint32_t* __restrict__ bmax) {
  const int32_t f = blockIdx.x * kThreads + threadIdx.x;
  if (f >= in.nface) return;
  const int32_t s = source_of(in.face_base, in.nsrc, f);
  bool bad = false;
  const float3 a = vertex(in, s, f, 0, &bad);
  const float3 b = vertex(in, s, f, 1, &bad);
  const float3 c = vertex(in, s, f, 2, &bad);
  if (bad) atomicOr(in.error_word, kErrBvhInput);
  const float lo[3] = {fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z))};
  const float hi[3] = {fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z))};
  tri_box[(int64_t)f * 2] = make_float4(lo[0], lo[1], lo[2], 0.0f);
  tri_box[(int64_t)f * 2 + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
  for (int k = 0; k < 3; ++k) {
    const float cen = 0.5f * (lo[k] + hi[k]);
    atomicMin(bmin + s * 6 + k, ordered(cen));
    atomicMax(bmax + s * 6 + k, ordered(cen));
    atomicMin(bmin + s * 6 + 3 + k, ordered(lo[k]));
    atomicMax(bmax + s * 6 + 3 + k, ordered(hi[k]));
  }
}

// 10 bits of x spread to every third bit.
__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3FFu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

// key = source << 30 | 30-bit Morton code of the centroid; value = face index within its source.
__global__ void __launch_bounds__(kThreads) morton_kernel(Inputs in, const float4* __restrict__ tri_box,
                                                          const uint32_t* __restrict__ bmin, const uint32_t* __restrict__ bmax,
                                                          uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int32_t f = blockIdx.x * kThreads + threadIdx.x;
  if (f >= in.nface) return;
  const int32_t s = source_of(in.face_base, in.nsrc, f);
  const float4 lo = tri_box[(int64_t)f * 2], hi = tri_box[(int64_t)f * 2 + 1];
  const float cen[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
  uint32_t code = 0;
  for (int k = 0; k < 3; ++k) {
    const float c0 = unordered(bmin[s * 6 + k]), c1 = unordered(bmax[s * 6 + k]);
    const float ext = c1 - c0;
    float u = ext > 0.0f ? (cen[k] - c0) / ext * 1024.0f : 0.0f;
    u = fminf(fmaxf(u, 0.0f), 1023.0f);
    code |= spread10((uint32_t)u) << (2 - k);
  }
  keys[f] = ((uint64_t)s << 30) | code;
  vals[f] = f - in.face_base[s];
}

// Radix sort, one pass over the 8-bit digit at `shift`: per-tile digit counts, digit-major
// (hist[digit * ntile + tile]).
__global__ void __launch_bounds__(kSortThreads) digit_hist_kernel(const uint64_t* __restrict__ keys, int32_t n, int shift,
                                                                  uint32_t* __restrict__ hist, int32_t ntile) {
  __shared__ uint32_t cnt[kDigits];
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) cnt[d] = 0;
  __syncthreads();
  const int32_t i = blockIdx.x * kSortThreads + threadIdx.x;
  if (i < n) atomicAdd(&cnt[(uint32_t)(keys[i] >> shift) & 0xFFu], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) hist[(int64_t)d * ntile + blockIdx.x] = cnt[d];
}

// Exclusive scan of hist (m entries) in place, one CTA: warp scans, then a scan of the warp sums.
__global__ void __launch_bounds__(kSortThreads) scan_kernel(uint32_t* __restrict__ hist, int64_t m) {
  __shared__ uint32_t warp_sum[kWarps];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < m; base += kSortThreads) {
    const int64_t i = base + threadIdx.x;
    const uint32_t v = i < m ? hist[i] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = warp_sum[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        if (lane >= o) w += y;
      }
      warp_sum[lane] = w;
    }
    __syncthreads();
    if (i < m) hist[i] = carry + (warp > 0 ? warp_sum[warp - 1] : 0u) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_sum[kWarps - 1];
    __syncthreads();
  }
}

// Stable scatter of one tile: rank among equal digits = earlier warps' counts + earlier lanes.
__global__ void __launch_bounds__(kSortThreads) digit_scatter_kernel(const uint64_t* __restrict__ keys_in,
                                                                     const int32_t* __restrict__ vals_in, int32_t n, int shift,
                                                                     const uint32_t* __restrict__ offs, int32_t ntile,
                                                                     uint64_t* __restrict__ keys_out, int32_t* __restrict__ vals_out) {
  __shared__ uint32_t cnt[kWarps][kDigits];
  for (int k = threadIdx.x; k < kWarps * kDigits; k += kSortThreads) (&cnt[0][0])[k] = 0;
  __syncthreads();
  const int32_t i = blockIdx.x * kSortThreads + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool valid = i < n;
  const uint64_t key = valid ? keys_in[i] : 0ull;
  const uint32_t digit = valid ? (uint32_t)(key >> shift) & 0xFFu : (uint32_t)kDigits;
  const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
  const uint32_t below = peers & ((1u << lane) - 1u);
  if (valid && below == 0) cnt[warp][digit] = __popc(peers);
  __syncthreads();
  if (threadIdx.x < kDigits) {
    uint32_t run = 0;
    for (int w = 0; w < kWarps; ++w) {
      const uint32_t c = cnt[w][threadIdx.x];
      cnt[w][threadIdx.x] = run;
      run += c;
    }
  }
  __syncthreads();
  if (valid) {
    const uint32_t dst = offs[(int64_t)digit * ntile + blockIdx.x] + cnt[warp][digit] + __popc(below);
    keys_out[dst] = key;
    vals_out[dst] = vals_in[i];
  }
}

struct Tree {
  const uint64_t* keys;  // sorted
  const int32_t* vals;   // sorted: face index within the source
  const float4* tri_box; // original order, 2 per face
  const int32_t* face_base;
  int32_t nsrc, ninner;  // ninner = nface - nsrc (inner nodes of every source's radix tree)
  int2* range;           // (ninner,) first, last leaf (positions within the source)
  int2* child;           // (ninner,) left, right: inner node g >= 0, leaf ~position
  int32_t* parent;       // (ninner,) global inner index, -1 at a root
  int32_t* leaf_parent;  // (nface,) inner node above each leaf (sorted position), -1 if none
  int32_t* visits;       // (ninner,) arrivals in the bottom-up pass
  int32_t* inner_size;   // (ninner,) output inner nodes in the subtree (0: collapsed into a leaf)
  float4* box;           // (ninner, 2)
  int32_t leaf_size;
};

// Source of global inner node g: inner nodes of source s start at face_base[s] - s.
__device__ __forceinline__ int32_t source_of_inner(const int32_t* __restrict__ face_base, int32_t nsrc, int32_t g) {
  int32_t lo = 0, hi = nsrc - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(face_base + mid) - mid <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Common-prefix length of leaves i and j of one source (n leaves at keys + 0), -1 outside;
// equal codes fall back to the positions.
__device__ __forceinline__ int delta(const uint64_t* __restrict__ keys, int32_t n, int32_t i, int32_t j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = (uint32_t)(keys[i] & 0x3FFFFFFFu), b = (uint32_t)(keys[j] & 0x3FFFFFFFu);
  if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
  return __clz(a ^ b);
}

// Karras (2012), "Maximizing parallelism in the construction of BVHs, octrees, and k-d trees":
// inner node i of a source's radix tree covers leaves [min(i, j), max(i, j)] and splits after gamma.
__global__ void __launch_bounds__(kThreads) hierarchy_kernel(Tree t) {
  const int32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= t.ninner) return;
  const int32_t s = source_of_inner(t.face_base, t.nsrc, g);
  const int32_t fb = t.face_base[s], n = t.face_base[s + 1] - fb, gb = fb - s;
  const uint64_t* keys = t.keys + fb;
  const int32_t i = g - gb;
  const int d = delta(keys, n, i, i + 1) > delta(keys, n, i, i - 1) ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int32_t lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int32_t l = 0;
  for (int32_t step = lmax >> 1; step >= 1; step >>= 1) {
    if (delta(keys, n, i, i + (l + step) * d) > dmin) l += step;
  }
  const int32_t j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int32_t sp = 0, step = l;
  do {
    step = (step + 1) >> 1;
    if (delta(keys, n, i, i + (sp + step) * d) > dnode) sp += step;
  } while (step > 1);
  const int32_t gamma = i + sp * d + min(d, 0);
  const int32_t first = min(i, j), last = max(i, j);
  const int32_t left = first == gamma ? ~gamma : gb + gamma;
  const int32_t right = last == gamma + 1 ? ~(gamma + 1) : gb + gamma + 1;
  t.range[g] = make_int2(first, last);
  t.child[g] = make_int2(left, right);
  if (left >= 0) t.parent[left] = g; else t.leaf_parent[fb + gamma] = g;
  if (right >= 0) t.parent[right] = g; else t.leaf_parent[fb + gamma + 1] = g;
  if (i == 0) t.parent[g] = -1;
}

__device__ __forceinline__ void child_box(const Tree& t, int32_t fb, int32_t c, float4* lo, float4* hi) {
  if (c >= 0) {
    *lo = __ldcg(t.box + (int64_t)c * 2);
    *hi = __ldcg(t.box + (int64_t)c * 2 + 1);
  } else {
    const int32_t f = fb + __ldg(t.vals + fb + ~c);
    *lo = __ldg(t.tri_box + (int64_t)f * 2);
    *hi = __ldg(t.tri_box + (int64_t)f * 2 + 1);
  }
}

__device__ __forceinline__ int32_t child_inner_size(const Tree& t, int32_t c) {
  return c >= 0 ? __ldcg(t.inner_size + c) : 0;
}

// Bottom-up boxes: every leaf walks up; the second arrival at a node computes its box (and its
// output inner-node count) and goes on.
__global__ void __launch_bounds__(kThreads) boxes_kernel(Tree t, int32_t nface) {
  const int32_t k = blockIdx.x * kThreads + threadIdx.x;
  if (k >= nface) return;
  const int32_t s = source_of(t.face_base, t.nsrc, k);
  const int32_t fb = t.face_base[s];
  int32_t g = t.leaf_parent[k];
  while (g >= 0) {
    __threadfence();
    if (atomicAdd(t.visits + g, 1) == 0) return;  // the sibling subtree is not done yet
    __threadfence();
    const int2 c = t.child[g];
    float4 l0, h0, l1, h1;
    child_box(t, fb, c.x, &l0, &h0);
    child_box(t, fb, c.y, &l1, &h1);
    t.box[(int64_t)g * 2] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f);
    t.box[(int64_t)g * 2 + 1] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
    const int2 r = t.range[g];
    t.inner_size[g] = r.y - r.x + 1 > t.leaf_size ? 1 + child_inner_size(t, c.x) + child_inner_size(t, c.y) : 0;
    g = t.parent[g];
  }
}

struct Emit {
  float* nodes;             // (sum of node capacities, 16)
  const int32_t* node_base; // (nsrc,)
  int32_t* nnode;           // (nsrc,)
  float* bounds;            // (nsrc, 6)
  const uint32_t* bmin;
  const uint32_t* bmax;
};

__device__ __forceinline__ void write_child(float* q, float4 lo, float4 hi, int32_t ref, int32_t count) {
  const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
  for (int a = 0; a < 3; ++a) {
    // conservative padding, as the host builder: the box test rounds differently from the triangle test
    const float pad = 1.0e-5f * (1.0f + fmaxf(fabsf(l[a]), fabsf(h[a])));
    q[a] = l[a] - pad;
    q[4 + a] = h[a] + pad;
  }
  q[3] = __int_as_float(ref);
  q[7] = __int_as_float(count);
}

// Pre-order position of output inner node g: one per ancestor edge, plus the left sibling
// subtree for every right turn.
__device__ __forceinline__ int32_t preorder(const Tree& t, int32_t g) {
  int32_t pos = 0;
  for (int32_t c = g, p = t.parent[g]; p >= 0; c = p, p = t.parent[p]) {
    const int2 ch = t.child[p];
    pos += 1 + (ch.y == c ? child_inner_size(t, ch.x) : 0);
  }
  return pos;
}

__global__ void __launch_bounds__(kThreads) emit_kernel(Tree t, Emit e) {
  const int32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= t.ninner) return;
  const int2 r = t.range[g];
  if (r.y - r.x + 1 <= t.leaf_size) return;  // collapsed into a leaf of its parent
  const int32_t s = source_of_inner(t.face_base, t.nsrc, g);
  const int32_t fb = t.face_base[s];
  const int32_t pos = preorder(t, g);
  float* o = e.nodes + ((int64_t)e.node_base[s] + pos) * 16;
  const int2 c = t.child[g];
  const int32_t kids[2] = {c.x, c.y};
  const int32_t left_size = child_inner_size(t, c.x);
  for (int k = 0; k < 2; ++k) {
    float4 lo, hi;
    child_box(t, fb, kids[k], &lo, &hi);
    const int32_t ch = kids[k];
    int32_t ref, count;
    if (ch < 0) {
      ref = ~ch;
      count = 1;
    } else if (t.inner_size[ch] == 0) {
      const int2 cr = t.range[ch];
      ref = cr.x;
      count = cr.y - cr.x + 1;
    } else {
      ref = pos + 1 + (k == 1 ? left_size : 0);
      count = 0;
    }
    write_child(o + k * 8, lo, hi, ref, count);
  }
  if (t.parent[g] < 0) e.nnode[s] = t.inner_size[g];
}

// Sources that are a single leaf (at most leaf_size triangles): a root with one leaf child and
// one empty child; every source: its bounds.
__global__ void __launch_bounds__(kThreads) roots_kernel(Tree t, Emit e) {
  const int32_t s = blockIdx.x * kThreads + threadIdx.x;
  if (s >= t.nsrc) return;
  const int32_t n = t.face_base[s + 1] - t.face_base[s];
  float4 lo = make_float4(unordered(e.bmin[s * 6 + 3]), unordered(e.bmin[s * 6 + 4]), unordered(e.bmin[s * 6 + 5]), 0.0f);
  float4 hi = make_float4(unordered(e.bmax[s * 6 + 3]), unordered(e.bmax[s * 6 + 4]), unordered(e.bmax[s * 6 + 5]), 0.0f);
  float* b = e.bounds + s * 6;
  b[0] = lo.x; b[1] = lo.y; b[2] = lo.z;
  b[3] = hi.x; b[4] = hi.y; b[5] = hi.z;
  if (n > t.leaf_size) return;
  float* o = e.nodes + (int64_t)e.node_base[s] * 16;
  write_child(o, lo, hi, 0, n);
  for (int k = 8; k < 16; ++k) o[k] = 0.0f;
  o[8 + 3] = __int_as_float(0);
  o[8 + 7] = __int_as_float(-1);
  e.nnode[s] = 1;
}

// Triangles in leaf order: v0 (face index within the source in w), v1, v2.
__global__ void __launch_bounds__(kThreads) tris_kernel(Inputs in, const int32_t* __restrict__ vals, float4* __restrict__ tris) {
  const int32_t k = blockIdx.x * kThreads + threadIdx.x;
  if (k >= in.nface) return;
  const int32_t s = source_of(in.face_base, in.nsrc, k);
  const int32_t f = vals[k];
  bool bad = false;
  for (int c = 0; c < 3; ++c) {
    const float3 p = vertex(in, s, in.face_base[s] + f, c, &bad);
    tris[(int64_t)k * 3 + c] = make_float4(p.x, p.y, p.z, c == 0 ? __int_as_float(f) : 0.0f);
  }
}

struct Layout {
  int64_t keys_a, keys_b, vals_a, vals_b, tri_box, bmin, bmax, hist, range, child, parent, leaf_parent, visits, inner_size, box,
      total;
};

Layout layout(int32_t nsrc, int32_t nface) {
  auto up = [](int64_t x) { return (x + 255) & ~(int64_t)255; };
  const int64_t ntile = (nface + kSortThreads - 1) / kSortThreads;
  const int64_t ninner = (int64_t)nface - nsrc > 0 ? (int64_t)nface - nsrc : 1;
  Layout l{};
  int64_t at = 0;
  l.keys_a = at; at = up(at + 8 * (int64_t)nface);
  l.keys_b = at; at = up(at + 8 * (int64_t)nface);
  l.vals_a = at; at = up(at + 4 * (int64_t)nface);
  l.vals_b = at; at = up(at + 4 * (int64_t)nface);
  l.tri_box = at; at = up(at + 32 * (int64_t)nface);
  l.bmin = at; at = up(at + 24 * (int64_t)nsrc);
  l.bmax = at; at = up(at + 24 * (int64_t)nsrc);
  l.hist = at; at = up(at + 4 * (int64_t)kDigits * ntile);
  l.range = at; at = up(at + 8 * ninner);
  l.child = at; at = up(at + 8 * ninner);
  l.parent = at; at = up(at + 4 * ninner);
  l.leaf_parent = at; at = up(at + 4 * (int64_t)nface);
  l.visits = at; at = up(at + 4 * ninner);
  l.inner_size = at; at = up(at + 4 * ninner);
  l.box = at; at = up(at + 32 * ninner);
  l.total = at;
  return l;
}

}  // namespace

int64_t lbvh_scratch_bytes(int32_t nsrc, int32_t nface) {
  if (nsrc < 1 || nface < nsrc) return -1;
  return layout(nsrc, nface).total;
}

int build_mesh_bvh_device_launch(const float* vert, const int32_t* face, const int32_t* vert_base, const int32_t* vert_num,
                                 const int32_t* face_base, const int32_t* node_base, int32_t nsrc, int32_t nface,
                                 int32_t leaf_size, float* nodes, float* tris, float* bounds, int32_t* nnode, void* scratch,
                                 int64_t scratch_bytes, int32_t* error_word, cudaStream_t st) {
  if (nsrc < 1 || nface < nsrc) return set_error(MJPBR_ERR_ARG, "need at least one source and one face per source (%d, %d)", nsrc, nface);
  if (nsrc > (1 << 24)) return set_error(MJPBR_ERR_ARG, "%d sources exceed 2^24", nsrc);
  if (leaf_size < 1 || leaf_size > 7) return set_error(MJPBR_ERR_ARG, "leaf_size must be in [1, 7], got %d", leaf_size);
  if (!vert || !face || !vert_base || !vert_num || !face_base || !node_base || !nodes || !tris || !bounds || !nnode || !scratch ||
      !error_word) {
    return set_error(MJPBR_ERR_ARG, "a BVH build array is NULL");
  }
  const Layout l = layout(nsrc, nface);
  if (scratch_bytes < l.total) return set_error(MJPBR_ERR_ARG, "scratch of %lld bytes, the build needs %lld", (long long)scratch_bytes, (long long)l.total);
  char* base = static_cast<char*>(scratch);
  auto at = [&](int64_t off) { return static_cast<void*>(base + off); };
  uint64_t* keys[2] = {static_cast<uint64_t*>(at(l.keys_a)), static_cast<uint64_t*>(at(l.keys_b))};
  int32_t* vals[2] = {static_cast<int32_t*>(at(l.vals_a)), static_cast<int32_t*>(at(l.vals_b))};
  float4* tri_box = static_cast<float4*>(at(l.tri_box));
  uint32_t* bmin = static_cast<uint32_t*>(at(l.bmin));
  uint32_t* bmax = static_cast<uint32_t*>(at(l.bmax));
  uint32_t* hist = static_cast<uint32_t*>(at(l.hist));
  const int32_t ntile = (nface + kSortThreads - 1) / kSortThreads;
  const int32_t ninner = nface - nsrc;
  Inputs in{vert, face, vert_base, vert_num, face_base, nsrc, nface, error_word};
  const int fgrid = (nface + kThreads - 1) / kThreads;

  cudaMemsetAsync(bmin, 0xFF, 24 * (size_t)nsrc, st);
  cudaMemsetAsync(bmax, 0x00, 24 * (size_t)nsrc, st);
  tri_bounds_kernel<<<fgrid, kThreads, 0, st>>>(in, tri_box, bmin, bmax);
  morton_kernel<<<fgrid, kThreads, 0, st>>>(in, tri_box, bmin, bmax, keys[0], vals[0]);
  int src_bits = 0;
  while ((1 << src_bits) < nsrc) ++src_bits;
  const int key_bits = 30 + src_bits;
  int cur = 0;
  for (int shift = 0; shift < key_bits; shift += 8) {
    digit_hist_kernel<<<ntile, kSortThreads, 0, st>>>(keys[cur], nface, shift, hist, ntile);
    scan_kernel<<<1, kSortThreads, 0, st>>>(hist, (int64_t)kDigits * ntile);
    digit_scatter_kernel<<<ntile, kSortThreads, 0, st>>>(keys[cur], vals[cur], nface, shift, hist, ntile, keys[cur ^ 1], vals[cur ^ 1]);
    cur ^= 1;
  }
  Tree t{keys[cur], vals[cur], tri_box, face_base, nsrc, ninner, static_cast<int2*>(at(l.range)), static_cast<int2*>(at(l.child)),
         static_cast<int32_t*>(at(l.parent)), static_cast<int32_t*>(at(l.leaf_parent)), static_cast<int32_t*>(at(l.visits)),
         static_cast<int32_t*>(at(l.inner_size)), static_cast<float4*>(at(l.box)), leaf_size};
  cudaMemsetAsync(t.leaf_parent, 0xFF, 4 * (size_t)nface, st);
  if (ninner > 0) {
    cudaMemsetAsync(t.visits, 0, 4 * (size_t)ninner, st);
    const int igrid = (ninner + kThreads - 1) / kThreads;
    hierarchy_kernel<<<igrid, kThreads, 0, st>>>(t);
    boxes_kernel<<<fgrid, kThreads, 0, st>>>(t, nface);
  }
  Emit e{nodes, node_base, nnode, bounds, bmin, bmax};
  if (ninner > 0) emit_kernel<<<(ninner + kThreads - 1) / kThreads, kThreads, 0, st>>>(t, e);
  roots_kernel<<<(nsrc + kThreads - 1) / kThreads, kThreads, 0, st>>>(t, e);
  tris_kernel<<<fgrid, kThreads, 0, st>>>(in, t.vals, reinterpret_cast<float4*>(tris));
  return check_launch("build_mesh_bvh_device");
}

}  // namespace mjpbr
