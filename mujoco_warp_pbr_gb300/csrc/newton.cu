// Newton sensor adapter: the two per-frame kernels around a render of a Newton model.
//
//  * newton_sync_poses: geom and camera poses of every render world from Newton's body and shape
//    transforms (newton-pbr/newton_pbr/_render.py:31-77, ScenePoses.sync at :96-131). One thread
//    per (world, geom). Transforms are Newton's (Warp's) transformf: position (3 floats), then a
//    unit quaternion (x, y, z, w). Matrices are written row-major (MuJoCo's xmat).
//  * newton_images: one camera's outputs in Newton's formats (newton-pbr/newton_pbr/sensor.py:45-86):
//    packed colour 0xAABBGGRR (the library's own packing, copied as it is), ray-distance and
//    forward depth with -1 where nothing is hit, shape indices with 0xFFFFFFFF where nothing (or
//    no geom) is hit, linear HDR. One thread per output pixel.
#include "abi_internal.h"
#include "common.cuh"

namespace mjpbr {
namespace {

constexpr int kThreads = 256;
constexpr int32_t kObjGeom = 5;  // mjOBJ_GEOM, the object type of a geom hit in seg_data

struct Xform {
  float3 p;
  float4 q;  // (x, y, z, w)
};

__device__ __forceinline__ Xform load_xform(const float* __restrict__ a, int64_t i) {
  const float* t = a + i * 7;
  return {make_float3(__ldg(t), __ldg(t + 1), __ldg(t + 2)), make_float4(__ldg(t + 3), __ldg(t + 4), __ldg(t + 5), __ldg(t + 6))};
}

// v rotated by the unit quaternion q: v + w t + q.xyz x t with t = 2 q.xyz x v.
__device__ __forceinline__ float3 quat_rotate(float4 q, float3 v) {
  const float tx = 2.0f * (q.y * v.z - q.z * v.y);
  const float ty = 2.0f * (q.z * v.x - q.x * v.z);
  const float tz = 2.0f * (q.x * v.y - q.y * v.x);
  return make_float3(v.x + q.w * tx + (q.y * tz - q.z * ty), v.y + q.w * ty + (q.z * tx - q.x * tz),
                     v.z + q.w * tz + (q.x * ty - q.y * tx));
}

// Hamilton product a * b (apply b, then a).
__device__ __forceinline__ float4 quat_mul(float4 a, float4 b) {
  return make_float4(a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
                     a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z);
}

// a * b: the frame b given in frame a.
__device__ __forceinline__ Xform compose(const Xform& a, const Xform& b) {
  const float3 r = quat_rotate(a.q, b.p);
  return {make_float3(a.p.x + r.x, a.p.y + r.y, a.p.z + r.z), quat_mul(a.q, b.q)};
}

__device__ __forceinline__ void store_pose(const Xform& x, float* __restrict__ pos, float* __restrict__ mat) {
  const float qx = x.q.x, qy = x.q.y, qz = x.q.z, qw = x.q.w;
  pos[0] = x.p.x;
  pos[1] = x.p.y;
  pos[2] = x.p.z;
  mat[0] = 1.0f - 2.0f * (qy * qy + qz * qz);
  mat[1] = 2.0f * (qx * qy - qz * qw);
  mat[2] = 2.0f * (qx * qz + qy * qw);
  mat[3] = 2.0f * (qx * qy + qz * qw);
  mat[4] = 1.0f - 2.0f * (qx * qx + qz * qz);
  mat[5] = 2.0f * (qy * qz - qx * qw);
  mat[6] = 2.0f * (qx * qz - qy * qw);
  mat[7] = 2.0f * (qy * qz + qx * qw);
  mat[8] = 1.0f - 2.0f * (qx * qx + qy * qy);
}

struct SyncArgs {
  const float* body_q;
  int32_t nbody;
  const int32_t* shape_body;
  const float* shape_transform;
  int32_t nshape;
  const int32_t* geom_shape;
  int32_t geom_shape_rows;
  const float* geom_offset;
  const float* camera_transforms;
  int32_t nworld, ngeom, ncam, cam;
  float* geom_xpos;
  float* geom_xmat;
  float* cam_xpos;
  float* cam_xmat;
  int32_t* error_word;
};

// Thread (world, geom) over nworld * max(ngeom, 1); geom 0 also writes the world's camera.
__global__ void __launch_bounds__(kThreads) sync_poses_kernel(SyncArgs a) {
  const int32_t per_world = a.ngeom > 0 ? a.ngeom : 1;
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= (int64_t)a.nworld * per_world) return;
  const int32_t world = (int32_t)(i / per_world);
  const int32_t geom = (int32_t)(i - (int64_t)world * per_world);
  if (geom < a.ngeom) {
    const int32_t row = a.geom_shape_rows == 1 ? 0 : world;
    const int32_t shape = __ldg(a.geom_shape + (int64_t)row * a.ngeom + geom);
    if (shape >= 0 && shape < a.nshape) {
      Xform x = load_xform(a.shape_transform, shape);
      const int32_t body = __ldg(a.shape_body + shape);
      if (body >= a.nbody) {
        atomicOr(a.error_word, kErrPoseIndex);
      } else if (body >= 0) {
        x = compose(load_xform(a.body_q, body), x);
      }
      x = compose(x, load_xform(a.geom_offset, geom));
      const int64_t g = (int64_t)world * a.ngeom + geom;
      store_pose(x, a.geom_xpos + g * 3, a.geom_xmat + g * 9);
    } else {
      atomicOr(a.error_word, kErrPoseIndex);
    }
  }
  if (geom == 0) {
    // Newton and MuJoCo cameras both look along their local -Z axis with +Y up.
    const Xform c = load_xform(a.camera_transforms, world);
    const int64_t k = (int64_t)world * a.ncam + a.cam;
    store_pose(c, a.cam_xpos + k * 3, a.cam_xmat + k * 9);
  }
}

struct ImageArgs {
  const uint32_t* rgb;
  const float* depth_in;
  const int2* seg;
  const float* hdr_in;
  int32_t rgb_stride, rgb_adr, depth_stride, depth_adr, seg_stride, seg_adr;
  const int32_t* geom_shape;
  int32_t geom_shape_rows, ngeom;
  const float* ray_scale;
  int32_t npix;
  int64_t total;
  uint32_t* color;
  float* depth;
  float* forward_depth;
  uint32_t* shape_index;
  float* hdr;
};

__global__ void __launch_bounds__(kThreads) images_kernel(ImageArgs a) {
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= a.total) return;
  const int64_t world = i / a.npix;
  const int32_t pixel = (int32_t)(i - world * a.npix);
  if (a.color) a.color[i] = __ldg(a.rgb + world * a.rgb_stride + a.rgb_adr + pixel);
  if (a.depth || a.forward_depth) {
    float d = __ldg(a.depth_in + world * a.depth_stride + a.depth_adr + pixel);
    if (d <= 0.0f) d = -1.0f;
    if (a.forward_depth) a.forward_depth[i] = d;
    if (a.depth) a.depth[i] = d > 0.0f ? d * __ldg(a.ray_scale + pixel) : d;
  }
  if (a.shape_index) {
    const int2 s = __ldg(a.seg + world * a.seg_stride + a.seg_adr + pixel);
    uint32_t index = 0xFFFFFFFFu;
    if (s.x >= 0 && s.x < a.ngeom && s.y == kObjGeom) {
      const int64_t row = a.geom_shape_rows == 1 ? 0 : world;
      index = (uint32_t)__ldg(a.geom_shape + row * a.ngeom + s.x);
    }
    a.shape_index[i] = index;
  }
  if (a.hdr) {
    const float* src = a.hdr_in + (world * a.rgb_stride + a.rgb_adr + pixel) * 3;
    a.hdr[i * 3] = __ldg(src);
    a.hdr[i * 3 + 1] = __ldg(src + 1);
    a.hdr[i * 3 + 2] = __ldg(src + 2);
  }
}

}  // namespace

int newton_sync_poses_launch(const float* body_q, int32_t nbody, const int32_t* shape_body, const float* shape_transform,
                             int32_t nshape, const int32_t* geom_shape, int32_t geom_shape_rows, const float* geom_offset,
                             const float* camera_transforms, int32_t nworld, int32_t ngeom, int32_t ncam, int32_t cam,
                             float* geom_xpos, float* geom_xmat, float* cam_xpos, float* cam_xmat, int32_t* error_word,
                             cudaStream_t stream) {
  if (nworld < 0 || ngeom < 0 || nbody < 0 || nshape < 0) {
    return set_error(MJPBR_ERR_ARG, "negative count (nworld %d, ngeom %d, nbody %d, nshape %d)", nworld, ngeom, nbody, nshape);
  }
  if (ncam < 1 || cam < 0 || cam >= ncam) return set_error(MJPBR_ERR_ARG, "camera %d of %d cameras", cam, ncam);
  if (geom_shape_rows != 1 && geom_shape_rows != nworld) {
    return set_error(MJPBR_ERR_ARG, "geom_shape has %d rows; 1 or nworld (%d)", geom_shape_rows, nworld);
  }
  if (nworld == 0) return MJPBR_OK;
  if (!camera_transforms || !cam_xpos || !cam_xmat || !error_word) {
    return set_error(MJPBR_ERR_ARG, "camera_transforms, cam_xpos, cam_xmat and error_word must not be NULL");
  }
  if (ngeom > 0 && (!shape_body || !shape_transform || !geom_shape || !geom_offset || !geom_xpos || !geom_xmat)) {
    return set_error(MJPBR_ERR_ARG, "shape and geom arrays must not be NULL when ngeom > 0");
  }
  if (nbody > 0 && !body_q) return set_error(MJPBR_ERR_ARG, "body_q is NULL with %d bodies", nbody);
  SyncArgs a{body_q, nbody, shape_body, shape_transform, nshape, geom_shape, geom_shape_rows, geom_offset, camera_transforms,
             nworld, ngeom, ncam, cam, geom_xpos, geom_xmat, cam_xpos, cam_xmat, error_word};
  const int64_t total = (int64_t)nworld * (ngeom > 0 ? ngeom : 1);
  const int64_t grid = (total + kThreads - 1) / kThreads;
  if (grid > 0x7FFFFFFF) return set_error(MJPBR_ERR_ARG, "%lld poses exceed one launch", (long long)total);
  sync_poses_kernel<<<(unsigned)grid, kThreads, 0, stream>>>(a);
  return check_launch("newton_sync_poses");
}

int newton_images_launch(const MjpbrScene& s, int32_t cam, const int32_t* geom_shape, int32_t geom_shape_rows,
                         const float* ray_scale, uint32_t* color, float* depth, float* forward_depth, uint32_t* shape_index,
                         float* hdr, cudaStream_t stream) {
  if (cam < 0 || cam >= s.nrender) return set_error(MJPBR_ERR_ARG, "camera_index must be in [0, %d), got %d", s.nrender, cam);
  if (color && (s.rgb_adr[cam] < 0 || !s.rgb_data)) return set_error(MJPBR_ERR_ARG, "camera %d renders no RGB", cam);
  if ((depth || forward_depth) && (s.depth_adr[cam] < 0 || !s.depth_data)) {
    return set_error(MJPBR_ERR_ARG, "camera %d renders no depth", cam);
  }
  if (depth && !ray_scale) return set_error(MJPBR_ERR_ARG, "ray_scale is NULL with a depth image");
  if (shape_index) {
    if (s.seg_adr[cam] < 0 || !s.seg_data) return set_error(MJPBR_ERR_ARG, "camera %d renders no segmentation", cam);
    if (!geom_shape) return set_error(MJPBR_ERR_ARG, "geom_shape is NULL with a shape-index image");
    if (geom_shape_rows != 1 && geom_shape_rows != s.nworld) {
      return set_error(MJPBR_ERR_ARG, "geom_shape has %d rows; 1 or nworld (%d)", geom_shape_rows, s.nworld);
    }
  }
  if (hdr && (s.rgb_adr[cam] < 0 || !s.hdr_data)) return set_error(MJPBR_ERR_ARG, "camera %d renders no HDR", cam);
  const int32_t npix = s.cam_res[cam][0] * s.cam_res[cam][1];
  const int64_t total = (int64_t)s.nworld * npix;
  if (total == 0 || !(color || depth || forward_depth || shape_index || hdr)) return MJPBR_OK;
  ImageArgs a{s.rgb_data,      s.depth_data,  reinterpret_cast<const int2*>(s.seg_data), s.hdr_data,  s.rgb_stride,
              s.rgb_adr[cam],  s.depth_stride, s.depth_adr[cam], s.seg_stride, s.seg_adr[cam], geom_shape,
              geom_shape_rows, s.ngeom,       ray_scale,   npix,        total,       color,       depth,
              forward_depth,   shape_index,   hdr};
  const int64_t grid = (total + kThreads - 1) / kThreads;
  if (grid > 0x7FFFFFFF) return set_error(MJPBR_ERR_ARG, "%lld pixels exceed one launch", (long long)total);
  images_kernel<<<(unsigned)grid, kThreads, 0, stream>>>(a);
  return check_launch("newton_images");
}

}  // namespace mjpbr
