"""The Newton sensor adapter (newton-pbr/newton_pbr): scene mapping on the CPU, and on the GPU the
pose and output kernels against oracle/newton_oracle.py plus the rendered images against the
oracle renderer.

Restates newton-pbr/tests/test_sensor.py's scene (a box and a sphere on one body, a capsule on a
turned arm, an off-centre tetrahedron mesh, a ground plane, two worlds with the second shifted)
and its checks (ray depth >= forward depth, the red box stays red, validation errors, shared
meshes), with Newton replaced by tests/newton_fake.py. The reference compares against Newton's
own SensorCamera, which is not installed here; the oracle renderer is the bar instead.

Bars: poses within 2e-6 (float32 transform products against float64); Newton images bit-exact
against the oracle's conversion of the same render buffers; the render itself at the real-time
bars (segmentation exact, depth 1e-5 relative, RGB within 1/255).
"""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mujoco_warp_pbr_gb300 import newton_pbr  # noqa: E402
from oracle import newton_oracle  # noqa: E402
from tests import newton_fake as nf  # noqa: E402

_RES = 48
_FOVY = 50.0
gpu = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


def _tetra() -> nf.Mesh:
  verts = np.array([[0.4, 0.4, 0.0], [0.8, 0.4, 0.0], [0.4, 0.8, 0.0], [0.5, 0.5, 0.5]], dtype=np.float32)
  faces = np.array([0, 2, 1, 0, 1, 3, 1, 2, 3, 2, 0, 3], dtype=np.int32)
  return nf.Mesh(verts, faces)


def _scene(nworld: int = 2, device: str = "cuda"):
  world = nf.ModelBuilder()
  body = world.add_body(xform=nf.xform((0.0, 0.0, 0.5)))
  world.add_shape_box(body, hx=0.3, hy=0.2, hz=0.25, color=(0.9, 0.1, 0.1))
  world.add_shape_sphere(body, xform=nf.xform((0.0, 0.0, 0.45)), radius=0.2)
  arm = world.add_body(xform=nf.xform((0.7, 0.0, 0.4), axis=(1.0, 0.0, 0.0), angle=0.6))
  world.add_shape_capsule(arm, radius=0.1, half_height=0.25)
  # An off-centre tetrahedron, static in its world.
  world.add_shape_mesh(-1, mesh=_tetra(), xform=nf.xform((-1.0, -0.6, 0.0)))
  scene = nf.ModelBuilder()
  scene.add_ground_plane()
  scene.replicate(world, nworld)
  model = scene.finalize(device)
  state = model.state()
  if state.body_q is not None:
    q = state.body_q.clone()
    per_world = len(q) // nworld
    q[per_world:, 1] += 0.3  # world 1 shifted so the views differ
    state.body_q = q
  eye = np.array([0.0, -3.0, 1.2])
  forward = -eye / np.linalg.norm(eye)
  right = np.cross(forward, [0.0, 0.0, 1.0])
  right /= np.linalg.norm(right)
  up = np.cross(right, forward)
  rot = np.stack([right, up, -forward], axis=1)
  cam = (*eye.tolist(), *nf.quat_from_matrix(rot))
  cams = torch.tensor([cam] * nworld, dtype=torch.float32, device=device)
  return model, state, cams


# ---------------------------------------------------------------- CPU: scene mapping and helpers


def test_scene_mapping_of_the_sensor_scene():
  model, _, _ = _scene(device="cpu")
  sc = newton_pbr.build_scene(model, newton_pbr.default_lights(), 45.0, newton=nf.newton)
  mjm = sc.mjm
  # world 0's four shapes then the global ground plane; one row per world
  assert mjm.ngeom == 5 and mjm.nmesh == 1 and mjm.nlight == 2 and mjm.ncam == 1
  assert sc.geom_shape.shape == (2, 5)
  assert sc.geom_shape[0].tolist() == [1, 2, 3, 4, 0] and sc.geom_shape[1].tolist() == [5, 6, 7, 8, 0]
  assert mjm.geom_type.tolist() == [6, 2, 3, 7, 0]
  np.testing.assert_allclose(mjm.geom_size[0], [0.3, 0.2, 0.25], rtol=1e-6)
  # the red box: sRGB (0.9, 0.1, 0.1) made linear, on the geom and its material
  np.testing.assert_allclose(mjm.geom_rgba[0, :3], newton_pbr.srgb_to_linear([0.9, 0.1, 0.1]), rtol=1e-6)
  np.testing.assert_allclose(mjm.mat_rgba[mjm.geom_matid[0]], mjm.geom_rgba[0], rtol=1e-6)
  # meshes keep Newton's vertices: the tetrahedron is not re-centred, offsets are the identity
  np.testing.assert_allclose(mjm.mesh_vert, _tetra().vertices, rtol=1e-6)
  np.testing.assert_array_equal(sc.geom_offset_pos, 0.0)
  np.testing.assert_array_equal(sc.geom_offset_quat, np.tile([1.0, 0.0, 0.0, 0.0], (5, 1)))


def test_initial_poses_follow_the_bodies():
  model, _, _ = _scene(device="cpu")
  sc = newton_pbr.build_scene(model, None, 45.0, newton=nf.newton)
  ref = newton_oracle.sync_poses(model.body_q.numpy(), model.shape_body.numpy(), model.shape_transform.numpy(), sc.geom_shape[:1], np.tile([0, 0, 0, 0, 0, 0, 1.0], (5, 1)), np.tile([0, 0, 0, 0, 0, 0, 1.0], (1, 1)))
  np.testing.assert_allclose(sc.mjd.geom_xpos, ref["geom_xpos"][0], atol=1e-6)
  np.testing.assert_allclose(sc.mjd.geom_xmat, ref["geom_xmat"][0], atol=1e-6)
  # the sphere sits 0.45 above the box's body, at z = 0.95
  np.testing.assert_allclose(sc.mjd.geom_xpos[1], [0.0, 0.0, 0.95], atol=1e-6)


def test_worlds_must_match():
  def world(radius: float) -> nf.ModelBuilder:
    b = nf.ModelBuilder()
    body = b.add_body(xform=nf.xform((0.0, 0.0, 0.5)))
    b.add_shape_sphere(body, radius=radius)
    return b

  scene = nf.ModelBuilder()
  scene.add_world(world(0.2))
  scene.add_world(world(0.3))
  with pytest.raises(ValueError, match="same visible shapes"):
    newton_pbr.build_scene(scene.finalize("cpu"), None, 45.0, newton=nf.newton)
  merged = newton_pbr.build_scene(scene.finalize("cpu"), None, 45.0, merge_worlds=True, newton=nf.newton)
  assert merged.mjm.ngeom == 2 and merged.geom_shape.shape == (1, 2)


def test_shared_meshes_become_one_mesh_per_scale():
  mesh = nf.Mesh([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]], [0, 2, 1, 0, 1, 3, 1, 2, 3, 2, 0, 3])
  b = nf.ModelBuilder()
  for x in (0.0, 1.5):
    b.add_shape_mesh(-1, mesh=mesh, xform=nf.xform((x, 0.0, 0.0)))
  b.add_shape_mesh(-1, mesh=mesh, scale=(2.0, 2.0, 2.0))
  sc = newton_pbr.build_scene(b.finalize("cpu"), None, 45.0, newton=nf.newton)
  assert sc.mjm.ngeom == 3
  assert sc.mjm.nmesh == 2  # one per (mesh, scale)
  np.testing.assert_allclose(sc.mjm.mesh_vert[4:], 2.0 * mesh.vertices, rtol=1e-6)


def test_hidden_sites_and_unsupported_types():
  b = nf.ModelBuilder()
  b.add_shape_sphere(-1, radius=0.2)
  b.add_shape_sphere(-1, radius=0.3, flags=nf.ShapeFlags.VISIBLE | nf.ShapeFlags.SITE)
  b.add_shape_sphere(-1, radius=0.4, flags=nf.ShapeFlags.COLLIDE_SHAPES)
  b._shape(-1, nf.GeoType.SDF, (1.0, 1.0, 1.0), None, None)
  b.add_shape_cone(-1, radius=0.2, half_height=0.3)
  with pytest.warns(UserWarning, match="SDF"):
    sc = newton_pbr.build_scene(b.finalize("cpu"), None, 45.0, newton=nf.newton)
  assert sc.geom_shape.tolist() == [[0, 4]]
  assert sc.mjm.geom_type.tolist() == [2, 7]
  # the meshed cone: 32 ring vertices, apex, base centre; 64 faces
  assert sc.mjm.mesh_vertnum.tolist() == [34] and sc.mjm.mesh_facenum.tolist() == [64]


def test_crease_normals_of_a_tetrahedron_are_face_normals():
  t = _tetra()
  normal, corner = newton_pbr.crease_normals(t.vertices, t.indices.reshape(-1, 3))
  v = t.vertices.astype(np.float64)
  f = t.indices.reshape(-1, 3)
  fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
  fn /= np.linalg.norm(fn, axis=1, keepdims=True)
  # every corner of a tetrahedron is sharper than the crease angle
  np.testing.assert_allclose(normal[corner], np.repeat(fn[:, None], 3, axis=1), atol=1e-6)
  # a finely tessellated sphere keeps smooth vertex normals
  from mujoco_warp_pbr_gb300 import synthetic

  sv, sf = synthetic.icosphere(3)
  _, corner = newton_pbr.crease_normals(sv, sf)
  assert np.array_equal(corner, sf)


def test_textures_and_materials():
  tex = np.random.default_rng(0).random((8, 8, 3)).astype(np.float32)
  verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
  uvs = np.array([[0, 0], [1, 0], [0, 1]], np.float32)
  b = nf.ModelBuilder()
  b.add_shape_mesh(-1, mesh=nf.Mesh(verts, [0, 1, 2], uvs=uvs, texture=tex, roughness=0.3, metallic=1.0), color=(0.2, 0.4, 0.6))
  b.add_shape_box(-1, color=(0.5, 0.5, 0.5))
  sc = newton_pbr.build_scene(b.finalize("cpu"), None, 45.0, checkerboard=newton_pbr.Checkerboard(frozenset({1})), newton=nf.newton)
  mjm = sc.mjm
  assert mjm.ntex == 2
  m0, m1 = mjm.geom_matid
  assert mjm.mat_texid[m0, 1] == 0 and mjm.mat_texid[m1, 1] == 1
  np.testing.assert_allclose(mjm.mat_rgba[m0], [1, 1, 1, 1])  # the texture replaces the colour
  assert mjm.mat_roughness[m0] == pytest.approx(0.3) and mjm.mat_metallic[m0] == 1.0
  np.testing.assert_allclose(mjm.mat_rgba[m1, :3], newton_pbr.srgb_to_linear([0.5] * 3), rtol=1e-6)  # checker multiplies it
  img = mjm.tex_data[: 8 * 8 * 4].reshape(8, 8, 4)
  np.testing.assert_array_equal(img[..., :3], (np.clip(tex, 0, 1) * 255 + 0.5).astype(np.uint8))
  b2 = nf.ModelBuilder()
  b2.add_shape_mesh(-1, mesh=nf.Mesh(verts, [0, 1, 2], uvs=uvs, texture="albedo.png"))
  with pytest.raises(TypeError, match="not decoded"):
    newton_pbr.build_scene(b2.finalize("cpu"), None, 45.0, newton=nf.newton)


def test_lights():
  with pytest.raises(ValueError, match=r"Light\.type"):
    newton_pbr.Light("area")  # type: ignore[arg-type]
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.primitive_scene(seed=0, nworld=1, res=8)
  lights = newton_pbr.lights_from_mujoco(sc.mjm, sc.mjd)
  assert [l.type for l in lights] == ["directional", "point"]
  np.testing.assert_allclose(lights[1].pos, np.asarray(sc.mjd.light_xpos).reshape(-1, 3)[1], rtol=1e-6)
  model, _, _ = _scene(device="cpu")
  mapped = newton_pbr.build_scene(model, lights, 45.0, newton=nf.newton)
  assert mapped.mjm.light_type.tolist() == [1, 2]
  assert mapped.mjm.light_bulbradius[1] == pytest.approx(lights[1].bulb_radius)


def test_ray_scale_matches_oracle():
  # the sensor's table is computed the same way; the oracle's is the restatement
  s = newton_oracle.ray_scale(6, 4, 60.0)
  assert s.shape == (4, 6) and s.dtype == np.float32
  assert np.all(s > 1.0)
  # the corner ray through (x, y) = (tan * aspect, tan) at the outermost pixel centres
  t = np.tan(np.radians(30.0))
  x = (2 * 5.5 / 6 - 1) * t * 1.5
  y = (1 - 2 * 0.5 / 4) * t
  assert s[0, 5] == np.float32(np.sqrt(1 + x * x + y * y))


def test_device_view_rejects_mismatches():
  t = torch.zeros((2, 7))
  with pytest.raises(ValueError, match="CUDA array"):
    newton_pbr.device_view(t, "camera_transforms", (2, 7), ("<f4",), torch.device("cuda", 0))

  class Iface:
    def __init__(self, shape, typestr, strides=None):
      self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (1234, False), "strides": strides, "version": 3}

  dev = torch.device("cuda", 0)
  assert newton_pbr.device_view(Iface((2, 7), "<f4"), "x", (2, 7), ("<f4",), dev) == 1234
  assert newton_pbr.device_view(Iface((3, 4, 5, 3), "<f4"), "x", (3, 4, 5, 3), ("<f4",), dev) == 1234
  with pytest.raises(ValueError, match="x must be"):
    newton_pbr.device_view(Iface((2, 7), "<f8"), "x", (2, 7), ("<f4",), dev)
  with pytest.raises(ValueError, match="x must be"):
    newton_pbr.device_view(Iface((3, 7), "<f4"), "x", (2, 7), ("<f4",), dev)
  with pytest.raises(ValueError, match="x must be"):
    newton_pbr.device_view(Iface((2, 7), "<f4", strides=(56, 8)), "x", (2, 7), ("<f4",), dev)


def test_reserved_render_options_raise():
  model, _, _ = _scene(nworld=1, device="cpu")
  with pytest.raises(TypeError, match="render_rgb"):
    newton_pbr.SensorPbrCamera(model, width=8, height=8, render_rgb=False, newton=nf.newton)


def test_oracle_pose_composition_is_a_group_action():
  """The oracle's transform algebra: (a b) c = a (b c) and matrices of products are products."""
  rng = np.random.default_rng(0)

  def rand(n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return np.concatenate([rng.normal(size=(n, 3)), q], axis=1)

  a, b, c = rand(5), rand(5), rand(5)
  tm = newton_oracle.transform_multiply
  np.testing.assert_allclose(tm(tm(a, b), c), tm(a, tm(b, c)), atol=1e-12)
  ma, mb = newton_oracle.quat_to_matrix(a[:, 3:]).reshape(-1, 3, 3), newton_oracle.quat_to_matrix(b[:, 3:]).reshape(-1, 3, 3)
  np.testing.assert_allclose(newton_oracle.quat_to_matrix(tm(a, b)[:, 3:]).reshape(-1, 3, 3), ma @ mb, atol=1e-12)
  np.testing.assert_allclose(tm(a, b)[:, :3], a[:, :3] + np.einsum("nij,nj->ni", ma, b[:, :3]), atol=1e-12)


# ---------------------------------------------------------------- GPU: kernels and images


@pytest.fixture(scope="module")
def rendered():
  model, state, cams = _scene()
  camera = newton_pbr.SensorPbrCamera(model, width=_RES, height=_RES, fovy=_FOVY, newton=nf.newton)
  out = {
    "color": camera.allocate_image_color(),
    "shape_index": camera.allocate_image_shape_index(),
    "depth": camera.allocate_image_depth(),
    "forward_depth": camera.allocate_image_depth(),
    "hdr": camera.allocate_image_color_hdr(),
  }
  camera.update(state, cams, color_image=out["color"], shape_index_image=out["shape_index"], depth_image=out["depth"], forward_depth_image=out["forward_depth"], hdr_color_image=out["hdr"], seed=3)
  torch.cuda.synchronize()
  from mujoco_warp_pbr_gb300.render import check_errors

  assert check_errors(camera.rc) == 0
  images = {k: v.cpu().numpy() for k, v in out.items()}
  raw = {
    "rgb": camera.rc.base.rgb_data.cpu().numpy().view(np.uint32),
    "depth": camera.rc.base.depth_data.cpu().numpy(),
    "seg": camera.rc.base.seg_data.cpu().numpy(),
    "hdr": camera.rc.hdr_data.cpu().numpy(),
  }
  poses = {k: getattr(camera.d, k).cpu().numpy() for k in ("geom_xpos", "geom_xmat", "cam_xpos", "cam_xmat")}
  return model, state, cams, camera, images, raw, poses


@pytest.mark.gpu
@gpu
def test_pose_kernel_matches_oracle(rendered):
  model, state, cams, camera, _, _, poses = rendered
  ref = newton_oracle.sync_poses(state.body_q.cpu().numpy(), model.shape_body.cpu().numpy(), model.shape_transform.cpu().numpy(), camera.scene.geom_shape, camera.geom_offset.cpu().numpy(), cams.cpu().numpy())
  nw = camera.nworld
  np.testing.assert_allclose(poses["geom_xpos"].reshape(nw, -1, 3), ref["geom_xpos"], atol=2e-6)
  np.testing.assert_allclose(poses["geom_xmat"].reshape(nw, -1, 9), ref["geom_xmat"], atol=2e-6)
  np.testing.assert_allclose(poses["cam_xpos"].reshape(nw, 3), ref["cam_xpos"], atol=2e-6)
  np.testing.assert_allclose(poses["cam_xmat"].reshape(nw, 9), ref["cam_xmat"], atol=2e-6)


@pytest.mark.gpu
@gpu
def test_image_kernel_matches_oracle(rendered):
  _, _, _, camera, images, raw, _ = rendered
  nw, n = camera.nworld, _RES * _RES
  words = raw["rgb"].reshape(nw, -1)[:, :n]
  rgba8 = np.stack([(words >> s) & 0xFF for s in (0, 8, 16, 24)], axis=-1).astype(np.uint8).reshape(nw, _RES, _RES, 4)
  scale = newton_oracle.ray_scale(_RES, _RES, _FOVY)
  np.testing.assert_array_equal(camera.ray_scale.cpu().numpy(), scale)
  ref = newton_oracle.images(
    rgba8,
    raw["depth"].reshape(nw, -1)[:, :n].reshape(nw, _RES, _RES),
    raw["seg"].reshape(nw, -1, 2)[:, :n].reshape(nw, _RES, _RES, 2),
    raw["hdr"].reshape(nw, -1, 3)[:, :n].reshape(nw, _RES, _RES, 3),
    camera.scene.geom_shape,
    scale,
  )
  for k in ("color", "shape_index", "depth", "forward_depth", "hdr"):
    np.testing.assert_array_equal(images[k].view(ref[k].dtype) if images[k].dtype != ref[k].dtype else images[k], ref[k], err_msg=k)


@pytest.mark.gpu
@gpu
def test_render_matches_oracle(rendered):
  """The sensor's render against the oracle renderer on the same host model and synced poses."""
  from tests import helpers
  from oracle import oracle
  from mujoco_warp_pbr_gb300.model import HostData

  _, _, _, camera, _, raw, poses = rendered
  nw, mjm = camera.nworld, camera.mjm
  mjd = HostData(
    geom_xpos=poses["geom_xpos"].reshape(nw, -1, 3),
    geom_xmat=poses["geom_xmat"].reshape(nw, -1, 9),
    cam_xpos=poses["cam_xpos"].reshape(nw, -1, 3),
    cam_xmat=poses["cam_xmat"].reshape(nw, -1, 9),
    light_xpos=np.broadcast_to(camera.scene.mjd.light_xpos, (nw, mjm.nlight, 3)),
    light_xdir=np.broadcast_to(camera.scene.mjd.light_xdir, (nw, mjm.nlight, 3)),
  )
  options = {"cam_res": (_RES, _RES), "render_rgb": True, "render_hdr": True, "render_depth": True, "render_seg": True}
  ref = oracle.OracleScene(mjm, mjd, nw, options, tables=helpers.gpu_tables(camera.rc)).render(seed=3)
  np.testing.assert_array_equal(raw["seg"], ref["seg"])
  np.testing.assert_allclose(raw["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(raw["rgb"], ref["rgb"])
  assert diff.max() <= 1, f"max RGB difference {diff.max()}/255"


@pytest.mark.gpu
@gpu
def test_ray_depth_exceeds_forward_depth(rendered):
  *_, images, _, _ = rendered
  depth, forward = images["depth"], images["forward_depth"]
  hit = forward > 0.0
  assert hit.mean() > 0.3
  assert np.all(depth[hit] >= forward[hit] - 1e-5)
  assert np.all(depth[~hit] < 0.0) and np.all(forward[~hit] == -1.0)


@pytest.mark.gpu
@gpu
def test_shape_colours_and_indices(rendered):
  model, _, _, _, images, _, _ = rendered
  color, index = images["color"], images["shape_index"]
  rgba = np.stack([(color >> s) & 0xFF for s in (0, 8, 16, 24)], axis=-1)
  box = int(np.flatnonzero(model.shape_type.cpu().numpy() == int(nf.GeoType.BOX))[0])
  r, g, b = rgba[index == box][:, :3].mean(axis=0)
  # the red box (sRGB 0.9, 0.1, 0.1) stays red after lighting and tone mapping
  assert r > 2.0 * g and r > 2.0 * b
  # both worlds and every shape type are visible: 2 x (box, sphere, capsule, mesh) + the ground
  assert len(np.unique(index[index != 0xFFFFFFFF])) >= 9
  assert np.all(rgba[..., 3] == 255)


@pytest.mark.gpu
@gpu
def test_output_images_are_validated(rendered):
  model, state, cams, *_ = rendered
  camera = newton_pbr.SensorPbrCamera(model, width=16, height=16, newton=nf.newton)
  wrong = torch.zeros((cams.shape[0], 8, 16), dtype=torch.int32, device="cuda")
  with pytest.raises(ValueError, match="color_image"):
    camera.update(state, cams, color_image=wrong)
  with pytest.raises(ValueError, match="depth_image"):
    camera.update(state, cams, depth_image=camera.allocate_image_shape_index())
  with pytest.raises(ValueError, match="one transform per world"):
    camera.update(state, cams[:1])
  # a static scene (no bodies) and an update with no outputs both run
  camera.update(state, cams)
  torch.cuda.synchronize()


@pytest.mark.gpu
@gpu
def test_static_model_without_bodies():
  b = nf.ModelBuilder()
  b.add_ground_plane(color=(0.5, 0.5, 0.5))
  b.add_shape_box(-1, xform=nf.xform((0.0, 0.0, 0.3)), hx=0.2, hy=0.2, hz=0.2, color=(0.1, 0.8, 0.1))
  model = b.finalize("cuda")
  _, _, cams = _scene(nworld=1)
  camera = newton_pbr.SensorPbrCamera(model, width=24, height=24, fovy=_FOVY, newton=nf.newton)
  index = camera.allocate_image_shape_index()
  state = nf.State()
  state.body_q = None
  camera.update(state, cams, shape_index_image=index)
  torch.cuda.synchronize()
  got = np.unique(index.cpu().numpy())
  assert set(got.tolist()) <= {0, 1, 0xFFFFFFFF} and 1 in got


@pytest.mark.gpu
@gpu
def test_image_step_throughput():
  """The image step is a stream over the render buffers: 28 bytes read and 28 written per pixel.
  Timed alone with CUDA events (L2 flushed before each launch) at 1024 worlds x 128x128 (0.94 GB per
  launch); the floor is loose (1 TB/s), the measured figure is printed."""
  from mujoco_warp_pbr_gb300 import _lib
  from mujoco_warp_pbr_gb300.render import scene as scene_descriptor

  nworld, res = 1024, 128
  model, state, cams = _scene(nworld=nworld)
  camera = newton_pbr.SensorPbrCamera(model, width=res, height=res, fovy=_FOVY, newton=nf.newton)
  out = [camera.allocate_image_color(), camera.allocate_image_depth(), camera.allocate_image_depth(), camera.allocate_image_shape_index(), camera.allocate_image_color_hdr()]
  camera.update(state, cams, color_image=out[0], depth_image=out[1], forward_depth_image=out[2], shape_index_image=out[3], hdr_color_image=out[4])
  sc = scene_descriptor(camera.m, camera.d, camera.rc)
  stream = torch.cuda.current_stream().cuda_stream
  flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
  times = []
  for _ in range(10):
    flush.zero_()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    _lib.call("mjpbr_newton_images", sc, 0, camera.geom_shape.data_ptr(), 1 if camera.geom_shape.shape[0] == 1 else nworld, camera.ray_scale.data_ptr(), *(o.data_ptr() for o in out), stream)
    b.record()
    torch.cuda.synchronize()
    times.append(a.elapsed_time(b))
  ms = float(np.median(times))
  gbs = nworld * res * res * 56 / (ms * 1e-3) / 1e9
  print(f"newton image step: {ms:.3f} ms for {nworld} x {res}^2, {gbs:.0f} GB/s")
  assert gbs > 1000.0
