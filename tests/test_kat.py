"""The reference's analytic known-answer tests (tests/test_render.py, test_ibl.py and
test_effects.py of mujoco_warp_pbr), restated on array scenes. Each runs on the CPU oracle (pinning
the oracle itself) and, on a machine with a GPU, through the public API of the GPU library."""

import numpy as np
import pytest

from tests import kat
from tests.kat import GEOM_BOX, GEOM_PLANE, GEOM_SPHERE, LIGHT_DIRECTIONAL, LIGHT_POINT, Builder, srgb

torch = pytest.importorskip("torch")

RENDERERS = [
  pytest.param("oracle", id="oracle"),
  pytest.param(
    "gpu",
    id="gpu",
    marks=[pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")],
  ),
]


@pytest.fixture(params=RENDERERS)
def render(request):
  return kat.render if request.param == "oracle" else kat.render_gpu


MATTE = {"metallic": 0.0, "roughness": 1.0, "specular": 0.0}


def test_lambertian_plane_point_light(render):
  """Radiance of a white Lambertian plane under a point light: (albedo / pi) * I / d^2."""
  intensity, height, albedo = 3.0, 1.5, 0.8
  b = kat.plane_scene(
    {"rgba": (albedo, albedo, albedo, 1), **MATTE},
    {"type": LIGHT_POINT, "pos": (0, 0, height), "intensity": intensity, "range": 1000.0, "castshadow": False},
  )
  out = render(b, render_hdr=True, tone_mapper=2)
  np.testing.assert_allclose(out["hdr"][0, 16, 16], albedo / np.pi * intensity / height**2, rtol=2e-3)


def test_hdr_holds_physical_radiance(render):
  illuminance = 1.0e6
  b = kat.plane_scene({"rgba": (1, 1, 1, 1), **MATTE}, {"type": LIGHT_DIRECTIONAL, "dir": (0, 0, -1), "intensity": illuminance, "castshadow": False})
  out = render(b, render_hdr=True)
  np.testing.assert_allclose(out["hdr"][0, 16, 16], illuminance / np.pi, rtol=2e-3)


def test_fallback_directional_matches_diffuse_colour(render):
  b = kat.plane_scene({"rgba": (1, 1, 1, 1), **MATTE}, {"type": LIGHT_DIRECTIONAL, "dir": (0, 0, -1), "diffuse": (0.5, 0.25, 0.125), "castshadow": False})
  out = render(b, tone_mapper=2)
  np.testing.assert_allclose(out["rgb"][0, 16, 16], srgb([0.5, 0.25, 0.125]), atol=2.5 / 255)


@pytest.mark.parametrize("light_model", [0, 1])
def test_light_models_agree_for_default_lights(render, light_model):
  b = kat.plane_scene({"rgba": (0.7, 0.7, 0.7, 1), **MATTE}, {"type": LIGHT_DIRECTIONAL, "dir": (0, 0, -1), "diffuse": (0.6, 0.6, 0.6), "castshadow": False})
  out = render(b, light_model=light_model, tone_mapper=2)
  np.testing.assert_allclose(out["rgb"][0, 16, 16], srgb(np.full(3, 0.7 * 0.6)), atol=2.5 / 255)


@pytest.mark.parametrize("roughness,rtol", [(0.0, 0.01), (1.0, 0.02)])
def test_metal_reflects_ambient_energy(render, roughness, rtol):
  """Smooth and rough white metal under constant ambient radiance reflect ~all of it
  (multiscatter compensation)."""
  b = kat.sphere_scene({"rgba": (1, 1, 1, 1), "metallic": 1.0, "roughness": roughness}, headlight_ambient=(0.5, 0.5, 0.5))
  out = render(b, render_hdr=True, tone_mapper=2)
  np.testing.assert_allclose(out["hdr"][0, 16, 16] * out["exposure"], 0.5, rtol=rtol)


def _shadow_scene() -> Builder:
  b = Builder()
  mat = b.material(rgba=(1, 1, 1, 1), roughness=1.0, specular=0.0)
  b.light(LIGHT_DIRECTIONAL, dir=(0, 0, -1), castshadow=True)
  b.geom(GEOM_PLANE, (5, 5, 0.1), matid=mat)
  b.geom(GEOM_BOX, (0.3, 0.3, 0.01), pos=(0, 0, 1), matid=mat)
  b.camera((0, -1, 0.5), xyaxes=(1, 0, 0, 0, 0.447, 0.894), fovy=30.0, resolution=(32, 32))
  return b


def test_shadow_blocks_direct_light(render):
  lit = render(_shadow_scene(), use_shadows=False)["rgb"][0]
  shadowed = render(_shadow_scene(), use_shadows=True)["rgb"][0]
  assert np.all(shadowed <= lit + 1e-6)
  assert (lit - shadowed).max() > 0.5


@pytest.mark.parametrize("nworld", [1, 2])
def test_per_world_metallic(render, nworld):
  def scene():
    b = Builder(headlight_active=True, headlight_ambient=(0.3, 0.3, 0.3), headlight_diffuse=(0.5, 0.5, 0.5))
    mat = b.material(rgba=(0.8, 0.2, 0.2, 1), roughness=0.4)
    b.geom(GEOM_SPHERE, (0.5, 0, 0), matid=mat)
    b.camera(resolution=(32, 32), fovy=25.0, **kat.FRONT_CAMERA)
    return b

  per_world = np.zeros((nworld, 1), np.float32)
  per_world[nworld - 1] = 1.0
  rgb = render(scene(), nworld=nworld, per_world={"geom_metallic": per_world})["rgb"]
  single = render(scene())["rgb"][0]
  np.testing.assert_allclose(rgb[0], single if nworld == 2 else rgb[0])
  if nworld == 2:
    assert not np.allclose(rgb[0], rgb[1])


def test_hdr_is_consistent_with_display_output(render):
  b = kat.plane_scene({"rgba": (0.5, 0.6, 0.7, 1), "roughness": 0.5}, {"type": LIGHT_DIRECTIONAL, "dir": (0.3, 0, -1), "castshadow": False})
  out = render(b, render_hdr=True, tone_mapper=2)
  expected = srgb(np.clip(out["hdr"][0] * out["exposure"], 0.0, 1.0))
  np.testing.assert_allclose(out["rgb"][0], expected, atol=1.5 / 255)


# ---------------------------------------------------------------- image-based lighting


@pytest.mark.parametrize("metallic", [0.0, 1.0])
@pytest.mark.parametrize("roughness", [0.0, 0.5, 1.0])
def test_white_furnace(render, metallic, roughness):
  """A white surface in a uniform white environment reflects (nearly) exactly the environment."""
  white = np.ones((64, 128, 3), np.float32)
  b = kat.sphere_scene({"rgba": (1, 1, 1, 1), "metallic": metallic, "roughness": roughness})
  out = render(b, envmap=white, envmap_intensity=1.0, render_hdr=True)
  np.testing.assert_allclose(out["hdr"][0, 16, 16], 1.0, rtol=0.03)


def test_environment_orientation(render):
  """Row 0 of the map is the zenith: a sky-red / ground-blue map lights an upward plane red."""
  image = np.zeros((64, 128, 3), np.float32)
  image[:32, :, 0] = 1.0
  image[32:, :, 2] = 1.0
  b = kat.plane_scene({"rgba": (1, 1, 1, 1), "roughness": 1.0, "specular": 0.0}, None)
  c = render(b, envmap=image, envmap_intensity=1.0, render_hdr=True)["hdr"][0, 16, 16]
  assert c[0] > 0.9 and c[2] < 0.05


def test_background_shows_environment_and_yaw_rotates_it(render):
  image = np.zeros((64, 128, 3), np.float32)
  image[:, 64:, 1] = 1.0  # +y half of the horizon (phi > 0) is green

  def scene():
    b = Builder()
    b.geom(GEOM_SPHERE, (0.1, 0, 0), pos=(0, -5, 0))
    b.camera((0, 0, 0), xyaxes=(1, 0, 0, 0, 0, 1), fovy=10.0, resolution=(32, 32))
    return b

  green = render(scene(), envmap=image, envmap_intensity=1.0, render_hdr=True)["hdr"][0, 16, 16]
  rotated = render(scene(), envmap=image, envmap_intensity=1.0, envmap_rotation=180.0, render_hdr=True)["hdr"][0, 16, 16]
  assert green[1] > 0.9
  assert rotated[1] < 0.05


@pytest.mark.parametrize("nworld", [1, 2])
def test_per_world_environment(render, nworld):
  maps = [np.full((32, 64, 3), 0.25, np.float32), np.full((32, 64, 3), 1.0, np.float32)]
  b = kat.sphere_scene({"rgba": (1, 1, 1, 1), "metallic": 0.0, "roughness": 1.0})
  hdr = render(b, nworld=nworld, envmap=maps, envmap_intensity=1.0, render_hdr=True, per_world={"env_id": (np.arange(nworld) % 2).astype(np.int32)})["hdr"]
  np.testing.assert_allclose(hdr[0, 16, 16], 0.25, rtol=0.03)
  if nworld == 2:
    np.testing.assert_allclose(hdr[1, 16, 16], 1.0, rtol=0.03)


# ---------------------------------------------------------------- textures and effects


def _normal_map_scene(tilt_deg: float, light_deg: float) -> Builder:
  t = np.radians(tilt_deg)
  rgb = 0.5 * (np.array([np.sin(t), 0.0, np.cos(t)]) + 1.0)
  ld = np.radians(light_deg)
  b = Builder()
  texel = np.concatenate([np.round(rgb * 255.0), [255.0]]).astype(np.uint8)
  tex = b.texture(np.broadcast_to(texel, (8, 8, 4)), colorspace=1)
  mat = b.material(rgba=(1, 1, 1, 1), metallic=0.0, roughness=1.0, specular=0.0, texid={5: tex})
  b.light(LIGHT_DIRECTIONAL, dir=(-np.sin(ld), 0, -np.cos(ld)), castshadow=False)
  b.geom(GEOM_PLANE, (5, 5, 0.1), matid=mat)
  b.camera(resolution=(32, 32), **kat.TOP_CAMERA)
  return b


def test_normal_map_tilts_towards_plus_u(render):
  """MuJoCo maps a plane's +u to +x: a +u-tilted normal map faces a light tilted towards +x."""
  flat = render(_normal_map_scene(0.0, 30.0), render_hdr=True)["hdr"][0, 16, 16]
  toward = render(_normal_map_scene(30.0, 30.0), render_hdr=True)["hdr"][0, 16, 16]
  away = render(_normal_map_scene(-30.0, 30.0), render_hdr=True)["hdr"][0, 16, 16]
  np.testing.assert_allclose(toward / flat, 1.0 / np.cos(np.radians(30.0)), rtol=0.02)
  np.testing.assert_allclose(away / flat, np.cos(np.radians(60.0)) / np.cos(np.radians(30.0)), rtol=0.02)


def test_texture_lod_filters_minified_checker(render):
  """A checker minified far below a pixel averages to the mean of its (linear) texels."""
  checker = np.zeros((256, 256, 4), np.uint8)
  checker[..., 3] = 255
  checker[:128, :128, :3] = 255
  checker[128:, 128:, :3] = 255
  b = Builder(headlight_active=True, headlight_ambient=(1, 1, 1), headlight_diffuse=(0, 0, 0), headlight_specular=(0, 0, 0))
  tex = b.texture(checker)
  mat = b.material(rgba=(1, 1, 1, 1), roughness=1.0, specular=0.0, texid={1: tex}, texrepeat=(4000, 4000))
  b.geom(GEOM_PLANE, (5, 5, 0.1), matid=mat)
  b.camera(resolution=(32, 32), **kat.TOP_CAMERA)
  rgb = render(b, tone_mapper=2, specular_aa=False)["rgb"][0]
  np.testing.assert_allclose(rgb.mean(), srgb(0.5), atol=0.02)
  assert rgb.std() < 0.02


def test_supersampling_resolves_edge_coverage(render):
  def scene():
    b = Builder(headlight_active=True, headlight_ambient=(1, 1, 1), headlight_diffuse=(0, 0, 0), headlight_specular=(0, 0, 0))
    b.geom(GEOM_BOX, (1, 1, 0.1), pos=(-0.987, 0, 0), rgba=(1, 1, 1, 1))
    b.camera((0, 0, 2), xyaxes=(1, 0, 0, 0, 1, 0), fovy=5.0, resolution=(8, 8))
    return b

  hard = render(scene(), samples_per_pixel=1, tone_mapper=2)["rgb"][0]
  soft = render(scene(), samples_per_pixel=4, tone_mapper=2)["rgb"][0]
  assert set(np.unique(hard.round(2))) <= {0.0, 1.0}
  assert np.any((soft > 0.05) & (soft < 0.95))


def test_translucent_layer_blends_over_background(render):
  b = Builder(headlight_active=True, headlight_ambient=(1, 1, 1), headlight_diffuse=(0, 0, 0), headlight_specular=(0, 0, 0))
  b.geom(GEOM_BOX, (1, 1, 0.01), pos=(0, 0, 0), rgba=(1, 0, 0, 1))
  b.geom(GEOM_BOX, (1, 1, 0.01), pos=(0, 0, 0.5), rgba=(0, 0, 1, 0.25))
  b.camera(resolution=(32, 32), **kat.TOP_CAMERA)
  out = render(b, render_hdr=True, tone_mapper=2)
  assert out["settings"]["has_transparency"]
  c = out["hdr"][0, 16, 16] * out["exposure"]
  assert c[0] > 0.6 and c[2] > 0.15 and c[1] < 0.05


def test_mirror_reflects_scene(render):
  b = Builder(headlight_active=True, headlight_ambient=(1, 1, 1), headlight_diffuse=(0, 0, 0), headlight_specular=(0, 0, 0))
  mirror = b.material(rgba=(0, 0, 0, 1), reflectance=1.0, roughness=1.0, specular=0.0)
  b.geom(GEOM_PLANE, (5, 5, 0.1), matid=mirror)
  b.geom(GEOM_BOX, (2, 2, 0.01), pos=(0, 0, 3), rgba=(0, 1, 0, 1))
  b.camera(resolution=(32, 32), **kat.TOP_CAMERA)
  out = render(b, tone_mapper=2)
  assert out["settings"]["has_reflection"]
  c = out["rgb"][0, 16, 16]
  assert c[1] > 0.9 and c[1] - c[0] > 0.5


def test_soft_shadows_have_penumbra(render):
  def row(**kwargs):
    b = Builder()
    b.light(LIGHT_POINT, pos=(0, 0, 2), intensity=50.0, range=100.0, bulbradius=0.4, castshadow=True)
    b.geom(GEOM_PLANE, (5, 5, 0.1), rgba=(1, 1, 1, 1))
    b.geom(GEOM_BOX, (0.25, 0.25, 0.01), pos=(0, 0, 1), rgba=(1, 1, 1, 1))
    b.camera((0, 0.001, 0.6), xyaxes=(1, 0, 0, 0, 1, 0), fovy=120.0, resolution=(64, 64))
    return render(b, render_hdr=True, **kwargs)["hdr"][0, 32, :, 0]

  unshadowed = row(use_shadows=False)
  hard = row(shadow_samples=1) / unshadowed
  soft = row(shadow_samples=32) / unshadowed

  def penumbra(v):
    return int(np.sum((v > 0.05) & (v < 0.95)))

  assert penumbra(hard) == 0
  assert penumbra(soft) > 4
