// Layout of one world's block: the per-frame, 16-byte aligned record of everything a render
// thread of that world reads repeatedly (scene BVH nodes, geom frames and materials, lights,
// cameras). mjpbr_refit_bvh writes one block per world from the model/data/context arrays
// (resolving the worldid % nbatch broadcasting once per frame); the render kernels copy their
// world's block into shared memory once per CTA.
//
// floats [0, 4)                      header: nbvh_geom, nnode, nlight, nrender (int bits)
// nodes  nnode x kNodeFloats         child-bounds BVH nodes (see below)
// geoms  nbvh_geom x kGeomFloats     slot order (enabled_geom_ids)
// lights nlight x kLightFloats
// cams   nrender x kCamFloats
//
// A node stores the bounds of both of its children so one fetch tests both:
//   [0..2] child A lower, [3] A ref, [4..6] A upper, [7] A count, [8..15] the same for child B.
// count 0: ref is an inner node; count > 0: a leaf of `count` primitives starting at ref;
// count < 0: no child. Scene BVH leaves hold one geom slot; mesh BVH leaves up to 4 triangles.
#pragma once

#include <cstdint>

namespace mjpbr {

constexpr int32_t kHdrFloats = 4;
constexpr int32_t kNodeFloats = 16;
constexpr int32_t kGeomFloats = 20;
constexpr int32_t kLightFloats = 24;
constexpr int32_t kCamFloats = 24;
constexpr int32_t kTriFloats = 12;

// Geom record: [0..2] pos, [3] type; [4..6] xmat row 0, [7] size.x; [8..10] row 1, [11] size.y;
// [12..14] row 2, [15] size.z; [16] geom id, [17] triangle BVH (mesh id; nmesh + height-field id; -1), [18] material id, [19] flags.
constexpr int32_t kGeomFlagSkip = 1;  // rgba alpha == 0: invisible to every ray

// Light record: [0..2] pos, [3] type; [4..6] dir, [7] flags; [8..10] diffuse, [11] intensity;
// [12..14] specular, [15] range; [16..18] attenuation, [19] bulbradius; [20] cutoff (deg),
// [21] exponent.
constexpr int32_t kLightFlagCastShadow = 1;
constexpr int32_t kLightFlagActive = 2;

// Camera record: [0..2] pos, [3] projection; [4..12] xmat; [13] half height of the image plane at
// z = -1 (perspective: tan(fovy / 2)) or of the frustum (orthographic: fovy / 2); [14] 1 when the
// intrinsics are used; [16..19] intrinsic fx, fy, cx, cy; [20..21] sensor size.

struct BlockLayout {
  int32_t nbvh, nnode, nlight, nrender;
  int32_t node_off, geom_off, light_off, cam_off, total;
};

__host__ __device__ inline BlockLayout block_layout(int32_t nbvh, int32_t nnode, int32_t nlight, int32_t nrender) {
  BlockLayout b;
  b.nbvh = nbvh;
  b.nnode = nnode;
  b.nlight = nlight;
  b.nrender = nrender;
  b.node_off = kHdrFloats;
  b.geom_off = b.node_off + nnode * kNodeFloats;
  b.light_off = b.geom_off + nbvh * kGeomFloats;
  b.cam_off = b.light_off + nlight * kLightFloats;
  b.total = (b.cam_off + nrender * kCamFloats + 3) & ~3;
  return b;
}

}  // namespace mjpbr
