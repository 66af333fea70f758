"""Per-pixel camera rays (set_camera_rays) and the first-hit guides: the reference's
tests/test_camera_rays.py restated on array scenes, run on the oracle and on the GPU, plus
GPU-vs-oracle parity of a fisheye bundle."""

import numpy as np
import pytest

from tests import kat
from tests.kat import GEOM_BOX, GEOM_PLANE, GEOM_SPHERE, LIGHT_DIRECTIONAL, Builder

torch = pytest.importorskip("torch")

GPU = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]
RENDERERS = [pytest.param("oracle", id="oracle"), pytest.param("gpu", id="gpu", marks=GPU)]
RES = (24, 16)


@pytest.fixture(params=RENDERERS)
def renderer(request):
  return request.param


def _checker(c1, c2, n: int = 64) -> np.ndarray:
  y, x = np.mgrid[0:n, 0:n]
  on = ((x < n // 2) ^ (y < n // 2))[..., None]
  img = np.where(on, np.asarray(c1), np.asarray(c2)) * 255.0 + 0.5
  return np.concatenate([img.astype(np.uint8), np.full((n, n, 1), 255, np.uint8)], -1)


def _scene(two_cameras: bool = True, ortho_top: bool = False) -> Builder:
  b = Builder()
  tex = b.texture(_checker((0.1, 0.2, 0.3), (0.8, 0.8, 0.8)))
  floor = b.material(rgba=(1, 1, 1, 1), texid={1: tex}, texrepeat=(4, 4))
  m = b.material(rgba=(0.8, 0.3, 0.2, 1), metallic=0.5, roughness=0.4)
  b.light(LIGHT_DIRECTIONAL, dir=(0.3, 0.2, -1), castshadow=True)
  b.geom(GEOM_PLANE, (2, 2, 0.1), matid=floor)
  b.geom(GEOM_SPHERE, (0.3, 0, 0), pos=(0, 0, 0.3), matid=m)
  b.geom(GEOM_BOX, (0.15, 0.2, 0.2), pos=(0.6, 0.2, 0.2), rgba=(0.2, 0.8, 0.3, 1))
  if ortho_top:
    b.camera(pos=(0, 0, 3), xyaxes=(1, 0, 0, 0, 1, 0), resolution=RES)
    return b
  b.camera(pos=(0, -2, 1), xyaxes=(1, 0, 0, 0, 0.45, 0.9), fovy=50.0, resolution=RES)
  if two_cameras:
    b.camera(pos=(1.5, -1.5, 1.2), xyaxes=(0.7, 0.7, 0, -0.3, 0.3, 0.9), fovy=70.0, resolution=RES)
  return b


def pinhole_rays(width: int, height: int, fovy_deg: float, offset: float = 0.5) -> np.ndarray:
  """(height, width, 2, 3) camera-frame rays of a pinhole camera through (px, py) + offset."""
  h = np.tan(np.radians(fovy_deg) / 2.0)
  u = (np.arange(width) + offset) / width - 0.5
  v = (np.arange(height) + offset) / height - 0.5
  d = np.stack(np.broadcast_arrays(u[None, :] * 2.0 * h * width / height, -v[:, None] * 2.0 * h, -np.ones((1, 1))), axis=-1)
  d /= np.linalg.norm(d, axis=-1, keepdims=True)
  return np.stack([np.zeros_like(d), d], axis=2).astype(np.float32)


def _pinhole_bundle(fovys=(50.0, 70.0)) -> np.ndarray:
  return np.stack([pinhole_rays(*RES, fovy) for fovy in fovys])


def _ray_scale(offset: float, fovys=(50.0, 70.0)) -> np.ndarray:
  """Distance along the ray per unit of planar depth, both cameras concatenated."""
  return np.concatenate([1.0 / -pinhole_rays(*RES, f, offset)[..., 1, 2].ravel() for f in fovys])


def _render(renderer, b: Builder, nworld: int = 2, **options):
  """(rgb uint32, depth, seg) flat per-world buffers of every camera."""
  options = {"render_rgb": True, "render_depth": True, "render_seg": True, **options}
  mjm, mjd = b.build()
  if renderer == "oracle":
    from oracle import oracle

    out = oracle.OracleScene(mjm, mjd, nworld, options).render(seed=0)
    return out["rgb"].copy(), out["depth"].copy(), out["seg"].copy()
  import mujoco_warp_pbr_gb300 as mjpbr

  m = mjpbr.put_model(mjm)
  d = mjpbr.put_data(mjm, mjd, nworld=nworld)
  rc = mjpbr.create_render_context(mjm, nworld, data=mjd, **options)
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  return rc.base.rgb_data.cpu().numpy().view(np.uint32), rc.base.depth_data.cpu().numpy(), rc.base.seg_data.cpu().numpy()


def _channels(rgb: np.ndarray) -> np.ndarray:
  from oracle import oracle

  return oracle.unpack_rgb(rgb)


@pytest.mark.parametrize(
  "options", [{}, {"samples_per_pixel": 2}, {"tier": 1, "path_samples": 4}], ids=["realtime", "supersampled", "path"]
)
def test_pinhole_rays_match_pinhole_cameras(renderer, options):
  rgb, depth, seg = _render(renderer, _scene(), **options)
  rgb_r, dist_r, seg_r = _render(renderer, _scene(), camera_rays=_pinhole_bundle(), **options)
  diff = np.abs(_channels(rgb) - _channels(rgb_r)).max(axis=-1)
  assert diff.max() <= 2 and np.mean(diff <= 1) > 0.99
  np.testing.assert_array_equal(seg, seg_r)
  # bundle depth is the distance along the ray, pinhole depth is planar, both from sample 0
  offset = 0.25 if options.get("samples_per_pixel") == 2 else 0.5
  np.testing.assert_allclose(dist_r, depth * _ray_scale(offset), rtol=1e-4, atol=1e-6)


def test_rays_without_direction_miss(renderer):
  rays = _pinhole_bundle()
  rays[:, :6, :, 1] = 0.0  # the top 6 rows of both cameras have no ray
  _, _, reference = _render(renderer, _scene(), nworld=1)
  _, depth, seg = _render(renderer, _scene(), nworld=1, camera_rays=rays)
  w, h = RES
  for cam in range(2):
    pixels = slice(cam * w * h, (cam + 1) * w * h)
    image_seg = seg[0, pixels].reshape(h, w, 2)
    assert np.all(image_seg[:6] == -1) and np.all(depth[0, pixels].reshape(h, w)[:6] == 0.0)
    np.testing.assert_array_equal(image_seg[6:], reference[0, pixels].reshape(h, w, 2)[6:])


def test_parallel_rays_measure_distance_from_their_origin(renderer):
  """Orthographic bundle: origins on a grid 0.25 m in front of the camera, all looking along -z."""
  w, h = RES
  x = ((np.arange(w) + 0.5) / w - 0.5) * 1.5
  y = (0.5 - (np.arange(h) + 0.5) / h) * 1.0
  origin = np.stack(np.broadcast_arrays(x[None, :], y[:, None], np.full((1, 1), -0.25)), axis=-1)
  direction = np.broadcast_to([0.0, 0.0, -1.0], origin.shape)
  ortho = np.stack([origin, direction], axis=2).astype(np.float32)
  _, depth, seg = _render(renderer, _scene(ortho_top=True), nworld=1, camera_rays=ortho[None])
  depth = depth[0].reshape(h, w)
  seg = seg[0].reshape(h, w, 2)
  floor = seg[..., 0] == 0
  assert floor.any()
  # camera at z = 3, origins 0.25 m in front of it: the floor (z = 0) is 2.75 m along every ray
  np.testing.assert_allclose(depth[floor], 2.75, atol=1e-4)
  sphere = seg[..., 0] == 1
  np.testing.assert_allclose(depth[sphere].min(), 3.0 - 0.25 - 0.6, atol=0.02)


def test_ray_validation():
  from mujoco_warp_pbr_gb300 import rays

  cam_res = [RES, RES]
  with pytest.raises(ValueError, match="each of the 2 rendering cameras"):
    rays.pack_camera_rays(_pinhole_bundle()[:1], cam_res)
  with pytest.raises(ValueError, match=r"shape \(16, 24, 2\)"):
    rays.pack_camera_rays([pinhole_rays(24, 16, 50.0), pinhole_rays(16, 16, 50.0)], cam_res)
  with pytest.raises(ValueError, match="dtype vec3"):
    rays.pack_camera_rays(torch.zeros((2, 16, 24, 2, 4)), cam_res)
  with pytest.raises(TypeError):
    rays.pack_camera_rays([[1, 2, 3], [4, 5, 6]], cam_res)


def fisheye_rays(width: int, height: int, fov_deg: float = 180.0) -> np.ndarray:
  """Equidistant fisheye: the angle from the optical axis grows linearly with the image radius;
  pixels outside the image circle have no ray (zero direction)."""
  u = (np.arange(width) + 0.5) / width * 2.0 - 1.0
  v = 1.0 - (np.arange(height) + 0.5) / height * 2.0
  x, y = np.meshgrid(u * width / max(width, height), v * height / max(width, height))
  r = np.hypot(x, y)
  theta = r * np.radians(fov_deg) / 2.0
  phi = np.arctan2(y, x)
  d = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), -np.cos(theta)], -1)
  d[r > 1.0] = 0.0
  return np.stack([np.zeros_like(d), d], axis=2).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("options", [{"samples_per_pixel": 2}, {"tier": 1, "path_samples": 3, "max_depth": 2}], ids=["realtime", "path"])
def test_fisheye_bundle_matches_oracle(options):
  """A 180 degree equidistant fisheye (rays off the z = -1 plane, pixels without rays) against the
  oracle: segmentation bit-exact, depth 1e-5, RGB within 1/255 (path: 99.5% of pixels)."""
  from tests import helpers

  b = _scene(two_cameras=False)
  mjm, mjd = b.build()
  opts = {"render_rgb": True, "render_depth": True, "render_seg": True, "camera_rays": fisheye_rays(*RES)[None], **options}
  import mujoco_warp_pbr_gb300 as mjpbr
  from oracle import oracle

  m = mjpbr.put_model(mjm)
  d = mjpbr.put_data(mjm, mjd, nworld=2)
  rc = mjpbr.create_render_context(mjm, 2, data=mjd, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=2)
  ref = oracle.OracleScene(mjm, mjd, 2, opts, tables=helpers.gpu_tables(rc)).render(seed=2)
  np.testing.assert_array_equal(gpu["seg"], ref["seg"])
  np.testing.assert_allclose(gpu["depth"], ref["depth"], rtol=1e-5, atol=1e-6)
  diff = helpers.rgb_diff(gpu["rgb"], ref["rgb"])
  if options.get("tier") == 1:
    assert (diff <= 1).mean() >= 0.995
  else:
    assert diff.max() <= 1


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_rays_are_updated_and_removed():
  import mujoco_warp_pbr_gb300 as mjpbr

  w, h = RES
  mjm, mjd = _scene().build()
  m = mjpbr.put_model(mjm)
  d = mjpbr.put_data(mjm, mjd, nworld=1)
  rc = mjpbr.create_render_context(mjm, 1, data=mjd, render_rgb=True, render_depth=True, render_seg=True)

  def frame():
    mjpbr.refit_bvh(m, d, rc)
    mjpbr.render(m, d, rc)
    torch.cuda.synchronize()
    return rc.base.rgb_data.cpu().numpy().view(np.uint32).copy(), rc.base.depth_data.cpu().numpy().copy(), rc.base.seg_data.cpu().numpy().copy()

  def first_camera(a):
    return a[0, : w * h].reshape(h, w, *a.shape[2:])

  rgb, depth, seg = frame()
  rays = _pinhole_bundle()
  mjpbr.set_camera_rays(rc, rays)
  assert np.abs(_channels(frame()[0]) - _channels(rgb)).max() <= 1
  # mirrored rays (x -> -x) mirror the image
  flipped = rays.copy()
  flipped[..., 0] *= -1.0
  mjpbr.set_camera_rays(rc, [flipped[0], flipped[1]])
  _, depth_f, seg_f = frame()
  np.testing.assert_array_equal(first_camera(seg_f)[:, ::-1], first_camera(seg))
  scale = first_camera(_ray_scale(0.5)[None])
  np.testing.assert_allclose(first_camera(depth_f)[:, ::-1], first_camera(depth) * scale, rtol=1e-4)
  mjpbr.set_camera_rays(rc, None)
  np.testing.assert_array_equal(frame()[0], rgb)
