// mjpbr_refit_bvh: per-world scene BVH refit and world-block packing.
//
// Replaces mujoco_warp.refit_bvh(m, d, rc.base) (third party; called by the reference at
// tests/conftest.py:44 and benchmarks/bench.py:184-186): per-geom world AABBs from the geom
// poses and sizes, then a bottom-up refit of each world's tree over the enabled geoms. The same
// pass writes the world block (world_block.cuh) the render kernels stage into shared memory, so
// the broadcasting of every batched table (worldid % nbatch) is resolved once per frame instead of
// once per ray. One warp per world: lanes build geom, light and camera records in parallel, lane 0
// sweeps the (small) tree bottom-up.
#include <cfloat>

#include "abi_internal.h"
#include "common.cuh"
#include "world_block.cuh"

namespace mjpbr {
namespace {

constexpr int kWarpsPerCta = 4;
constexpr float kBigExtent = 1.0e6f;  // half extent of infinite planes

// MuJoCo Warp's _geom_rgba: a geom with a material and the default rgba shows the material's.
__device__ float4 effective_rgba(const MjpbrScene& s, int32_t w, int32_t g, int32_t matid) {
  const float* p = s.geom_rgba.ptr + ((int64_t)(w % s.geom_rgba.nbatch) * s.ngeom + g) * 4;
  float4 c = make_float4(p[0], p[1], p[2], p[3]);
  if (matid >= 0 && c.x == 0.5f && c.y == 0.5f && c.z == 0.5f && c.w == 1.0f && s.mat_rgba.ptr) {
    const float* q = s.mat_rgba.ptr + ((int64_t)(w % s.mat_rgba.nbatch) * s.nmat + matid) * 4;
    c = make_float4(q[0], q[1], q[2], q[3]);
  }
  return c;
}

// What a geom's world AABB depends on: its pose, size, type, triangle BVH and flags, as the world
// block's geom record holds them.
struct GeomBoxIn {
  V3 pos;
  float m[9];
  V3 size;
  int32_t type, blas, flags;
};

__device__ __forceinline__ GeomBoxIn geom_box_in(const float* gr) {
  GeomBoxIn in;
  in.pos = V3{gr[0], gr[1], gr[2]};
  in.type = __float_as_int(gr[3]);
  in.m[0] = gr[4], in.m[1] = gr[5], in.m[2] = gr[6];
  in.m[3] = gr[8], in.m[4] = gr[9], in.m[5] = gr[10];
  in.m[6] = gr[12], in.m[7] = gr[13], in.m[8] = gr[14];
  in.size = V3{gr[7], gr[11], gr[15]};
  in.blas = __float_as_int(gr[17]);
  in.flags = __float_as_int(gr[19]);
  return in;
}

// Padded world AABB (lo, hi) of a geom into b[6]; b[0] = FLT_MAX marks a skipped geom.
__device__ __forceinline__ void geom_box(const MjpbrScene& s, const GeomBoxIn& in, float* b) {
  const float* m = in.m;
  const int32_t type = in.type, blas = in.blas;
  const V3 pos = in.pos, size = in.size;
  // world AABB: centre c, half extent e per axis
  V3 c = pos, e;
  float ax[3];
  for (int i = 0; i < 3; ++i) {
    float r0 = fabsf(m[3 * i]), r1 = fabsf(m[3 * i + 1]), r2 = fabsf(m[3 * i + 2]);
    switch (type) {
      case MJPBR_GEOM_SPHERE:
        ax[i] = size.x;
        break;
      case MJPBR_GEOM_CAPSULE:
        ax[i] = r2 * size.y + size.x;
        break;
      case MJPBR_GEOM_ELLIPSOID: {
        float a = m[3 * i] * size.x, bb = m[3 * i + 1] * size.y, cc = m[3 * i + 2] * size.z;
        ax[i] = sqrtf(a * a + bb * bb + cc * cc);
        break;
      }
      case MJPBR_GEOM_CYLINDER:
        ax[i] = r2 * size.y + size.x * sqrtf(fmaxf(0.0f, 1.0f - m[3 * i + 2] * m[3 * i + 2]));
        break;
      case MJPBR_GEOM_BOX:
        ax[i] = r0 * size.x + r1 * size.y + r2 * size.z;
        break;
      case MJPBR_GEOM_PLANE: {
        float sx = size.x > 0.0f ? size.x : kBigExtent;
        float sy = size.y > 0.0f ? size.y : kBigExtent;
        ax[i] = r0 * sx + r1 * sy;
        break;
      }
      default: {  // mesh or height field: transformed local AABB
        if (blas >= 0 && s.mesh_bounds) {
          const float* mb = s.mesh_bounds + blas * 6;
          float hx = 0.5f * (mb[3] - mb[0]), hy = 0.5f * (mb[4] - mb[1]), hz = 0.5f * (mb[5] - mb[2]);
          ax[i] = r0 * hx + r1 * hy + r2 * hz;
        } else {
          ax[i] = 0.0f;
        }
        break;
      }
    }
  }
  if (blas >= 0 && s.mesh_bounds) {
    const float* mb = s.mesh_bounds + blas * 6;
    V3 lc{0.5f * (mb[0] + mb[3]), 0.5f * (mb[1] + mb[4]), 0.5f * (mb[2] + mb[5])};
    c = pos + V3{m[0] * lc.x + m[1] * lc.y + m[2] * lc.z, m[3] * lc.x + m[4] * lc.y + m[5] * lc.z,
                 m[6] * lc.x + m[7] * lc.y + m[8] * lc.z};
  }
  e = V3{ax[0], ax[1], ax[2]};
  // Conservative padding: box tests may round differently from the exact primitive tests.
  float mag = fmaxf(fmaxf(fabsf(c.x), fabsf(c.y)), fabsf(c.z)) + vmax3(e);
  float pad = 1.0e-5f * (1.0f + mag);
  b[0] = c.x - e.x - pad;
  b[1] = c.y - e.y - pad;
  b[2] = c.z - e.z - pad;
  b[3] = c.x + e.x + pad;
  b[4] = c.y + e.y + pad;
  b[5] = c.z + e.z + pad;
  if (in.flags & kGeomFlagSkip) b[0] = FLT_MAX;  // marks an empty leaf
}

// kSmemBoxes: the lanes compute the leaf boxes into shared memory before lane 0's sweep; without
// (worlds whose boxes do not fit), the sweep computes each leaf's box from its geom record.
template <bool kSmemBoxes>
__global__ void __launch_bounds__(kWarpsPerCta * 32) refit_kernel(const __grid_constant__ MjpbrScene s) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int32_t w = blockIdx.x * kWarpsPerCta + warp;
  if (w >= s.nworld) return;
  const int32_t nbvh = s.nbvh_geom;
  float* box = kSmemBoxes ? smem + (int64_t)warp * nbvh * 6 : nullptr;  // leaf AABBs of this world
  BlockLayout L = block_layout(nbvh, s.nnode, s.nlight, s.nrender);
  float* blk = s.world_blocks + (int64_t)w * s.world_block_floats;

  // ---- geom records and leaf boxes
  for (int32_t slot = lane; slot < nbvh; slot += 32) {
    int32_t g = s.enabled_geom_ids[slot];
    int32_t type = s.geom_type[g];
    const float* xp = s.geom_xpos + ((int64_t)w * s.ngeom + g) * 3;
    const float* xm = s.geom_xmat + ((int64_t)w * s.ngeom + g) * 9;
    const float* sz = s.geom_size.ptr + ((int64_t)(w % s.geom_size.nbatch) * s.ngeom + g) * 3;
    int32_t matid = s.geom_matid.ptr[(int64_t)(w % s.geom_matid.nbatch) * s.ngeom + g];
    int32_t dataid = s.geom_dataid.ptr ? s.geom_dataid.ptr[(int64_t)(w % s.geom_dataid.nbatch) * s.ngeom + g] : -1;
    float4 rgba = effective_rgba(s, w, g, matid);
    float m[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) m[k] = xm[k];
    V3 pos{xp[0], xp[1], xp[2]};
    V3 size{sz[0], sz[1], sz[2]};
    int32_t flags = 0;
    // Triangle BVH of a mesh-like geom: the mesh's, or for a height field the one after the meshes.
    int32_t blas = -1;
    if (s.blas_root != nullptr && dataid >= 0) {
      if ((type == MJPBR_GEOM_MESH || type == MJPBR_GEOM_SDF) && dataid < s.nmesh) blas = dataid;
      if (type == MJPBR_GEOM_HFIELD && dataid < s.nhfield) blas = s.nmesh + dataid;
    }
    bool supported = type == MJPBR_GEOM_PLANE || type == MJPBR_GEOM_SPHERE || type == MJPBR_GEOM_CAPSULE ||
                     type == MJPBR_GEOM_ELLIPSOID || type == MJPBR_GEOM_CYLINDER || type == MJPBR_GEOM_BOX || blas >= 0;
    if (rgba.w == 0.0f || !supported) flags |= kGeomFlagSkip;
    float* gr = blk + L.geom_off + slot * kGeomFloats;
    gr[0] = pos.x;
    gr[1] = pos.y;
    gr[2] = pos.z;
    gr[3] = __int_as_float(type);
    gr[4] = m[0];
    gr[5] = m[1];
    gr[6] = m[2];
    gr[7] = size.x;
    gr[8] = m[3];
    gr[9] = m[4];
    gr[10] = m[5];
    gr[11] = size.y;
    gr[12] = m[6];
    gr[13] = m[7];
    gr[14] = m[8];
    gr[15] = size.z;
    gr[16] = __int_as_float(g);
    gr[17] = __int_as_float(blas);
    gr[18] = __int_as_float(matid);
    gr[19] = __int_as_float(flags);

    if constexpr (kSmemBoxes) {
      GeomBoxIn in;
      in.pos = pos;
      for (int k = 0; k < 9; ++k) in.m[k] = m[k];
      in.size = size;
      in.type = type;
      in.blas = blas;
      in.flags = flags;
      geom_box(s, in, box + slot * 6);
    }
  }

  // ---- lights
  for (int32_t li = lane; li < s.nlight; li += 32) {
    float* lr = blk + L.light_off + li * kLightFloats;
    const float* xp = s.light_xpos + ((int64_t)w * s.nlight + li) * 3;
    const float* xd = s.light_xdir + ((int64_t)w * s.nlight + li) * 3;
    int32_t type = s.light_type.ptr[(int64_t)(w % s.light_type.nbatch) * s.nlight + li];
    int32_t cast = s.light_castshadow.ptr[(int64_t)(w % s.light_castshadow.nbatch) * s.nlight + li];
    int32_t act = s.light_active.ptr[(int64_t)(w % s.light_active.nbatch) * s.nlight + li];
    lr[0] = xp[0];
    lr[1] = xp[1];
    lr[2] = xp[2];
    lr[3] = __int_as_float(type);
    lr[4] = xd[0];
    lr[5] = xd[1];
    lr[6] = xd[2];
    lr[7] = __int_as_float((cast ? kLightFlagCastShadow : 0) | (act ? kLightFlagActive : 0));
    const float* dif = s.light_diffuse.ptr + ((int64_t)(w % s.light_diffuse.nbatch) * s.nlight + li) * 3;
    const float* spe = s.light_specular.ptr + ((int64_t)(w % s.light_specular.nbatch) * s.nlight + li) * 3;
    const float* att = s.light_attenuation.ptr + ((int64_t)(w % s.light_attenuation.nbatch) * s.nlight + li) * 3;
    lr[8] = dif[0];
    lr[9] = dif[1];
    lr[10] = dif[2];
    lr[11] = s.light_intensity.ptr[(int64_t)(w % s.light_intensity.nbatch) * s.nlight + li];
    lr[12] = spe[0];
    lr[13] = spe[1];
    lr[14] = spe[2];
    lr[15] = s.light_range.ptr[(int64_t)(w % s.light_range.nbatch) * s.nlight + li];
    lr[16] = att[0];
    lr[17] = att[1];
    lr[18] = att[2];
    lr[19] = s.light_bulbradius.ptr[(int64_t)(w % s.light_bulbradius.nbatch) * s.nlight + li];
    lr[20] = s.light_cutoff.ptr[(int64_t)(w % s.light_cutoff.nbatch) * s.nlight + li];
    lr[21] = s.light_exponent.ptr[(int64_t)(w % s.light_exponent.nbatch) * s.nlight + li];
    lr[22] = 0.0f;
    lr[23] = 0.0f;
  }

  // ---- cameras
  for (int32_t ci = lane; ci < s.nrender; ci += 32) {
    int32_t cam = s.cam_id_map[ci];
    float* cr = blk + L.cam_off + ci * kCamFloats;
    const float* xp = s.cam_xpos + ((int64_t)w * s.ncam + cam) * 3;
    const float* xm = s.cam_xmat + ((int64_t)w * s.ncam + cam) * 9;
    int32_t proj = s.cam_projection[cam];
    float fovy = s.cam_fovy.ptr[(int64_t)(w % s.cam_fovy.nbatch) * s.ncam + cam];
    cr[0] = xp[0];
    cr[1] = xp[1];
    cr[2] = xp[2];
    cr[3] = __int_as_float(proj);
    for (int k = 0; k < 9; ++k) cr[4 + k] = xm[k];
    float half_h;
    if (proj == MJPBR_PROJ_ORTHOGRAPHIC) {
      half_h = fovy * 0.5f;
    } else {
      float sn, cs;
      sincos_turns(fovy / 720.0f, &sn, &cs);
      half_h = sn / cs;
    }
    cr[13] = half_h;
    int32_t use_intr = (s.cam_sensorsize && s.cam_sensorsize[cam * 2] > 0.0f && proj == MJPBR_PROJ_PERSPECTIVE) ? 1 : 0;
    cr[14] = __int_as_float(use_intr);
    cr[15] = 0.0f;
    for (int k = 0; k < 4; ++k) {
      cr[16 + k] = (use_intr && s.cam_intrinsic.ptr)
                       ? s.cam_intrinsic.ptr[((int64_t)(w % s.cam_intrinsic.nbatch) * s.ncam + cam) * 4 + k]
                       : 0.0f;
    }
    cr[20] = s.cam_sensorsize ? s.cam_sensorsize[cam * 2] : 0.0f;
    cr[21] = s.cam_sensorsize ? s.cam_sensorsize[cam * 2 + 1] : 0.0f;
    cr[22] = 0.0f;
    cr[23] = 0.0f;
  }
  __syncwarp();

  // ---- bottom-up refit (children always follow their parent)
  if (lane == 0) {
    blk[0] = __int_as_float(nbvh);
    blk[1] = __int_as_float(s.nnode);
    blk[2] = __int_as_float(s.nlight);
    blk[3] = __int_as_float(s.nrender);
    const int32_t* child = s.tlas_child.ptr + (int64_t)(w % s.tlas_child.nbatch) * s.nnode * 2;
    for (int32_t i = s.nnode - 1; i >= 0; --i) {
      float* nd = blk + L.node_off + i * kNodeFloats;
      for (int k = 0; k < 2; ++k) {
        int32_t c = child[i * 2 + k];
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        int32_t ref = 0, cnt = -1;
        if (c == INT32_MIN) {
          cnt = -1;
        } else if (c < 0) {
          int32_t slot = ~c;
          float tb[6];
          const float* b = tb;
          if constexpr (kSmemBoxes) {
            b = box + slot * 6;
          } else {
            geom_box(s, geom_box_in(blk + L.geom_off + slot * kGeomFloats), tb);
          }
          if (b[0] != FLT_MAX) {
            for (int a = 0; a < 3; ++a) {
              lo[a] = b[a];
              hi[a] = b[3 + a];
            }
            ref = slot;
            cnt = 1;
          }
        } else {
          const float* cn = blk + L.node_off + c * kNodeFloats;
          int32_t ca = __float_as_int(cn[7]), cb = __float_as_int(cn[15]);
          if (ca >= 0 || cb >= 0) {
            for (int a = 0; a < 3; ++a) {
              float l0 = ca >= 0 ? cn[a] : FLT_MAX, l1 = cb >= 0 ? cn[8 + a] : FLT_MAX;
              float h0 = ca >= 0 ? cn[4 + a] : -FLT_MAX, h1 = cb >= 0 ? cn[12 + a] : -FLT_MAX;
              lo[a] = fminf(l0, l1);
              hi[a] = fmaxf(h0, h1);
            }
            ref = c;
            cnt = 0;
          }
        }
        float* o = nd + k * 8;
        o[0] = cnt >= 0 ? lo[0] : 0.0f;
        o[1] = cnt >= 0 ? lo[1] : 0.0f;
        o[2] = cnt >= 0 ? lo[2] : 0.0f;
        o[3] = __int_as_float(ref);
        o[4] = cnt >= 0 ? hi[0] : 0.0f;
        o[5] = cnt >= 0 ? hi[1] : 0.0f;
        o[6] = cnt >= 0 ? hi[2] : 0.0f;
        o[7] = __int_as_float(cnt);
      }
    }
  }
}

}  // namespace

int refit_launch(const MjpbrScene& s, cudaStream_t stream) {
  const size_t smem = (size_t)kWarpsPerCta * s.nbvh_geom * 6 * sizeof(float);
  const int grid = (s.nworld + kWarpsPerCta - 1) / kWarpsPerCta;
  if (smem <= 200 * 1024) {
    if (int rc = ensure_smem(reinterpret_cast<const void*>(refit_kernel<true>), smem, "refit")) return rc;
    refit_kernel<true><<<grid, kWarpsPerCta * 32, smem, stream>>>(s);
  } else {
    refit_kernel<false><<<grid, kWarpsPerCta * 32, 0, stream>>>(s);  // leaf boxes computed in the sweep
  }
  return check_launch("refit_kernel");
}

}  // namespace mjpbr
