"""Host-side logic without a GPU: argument validation (exact messages of the reference's
tests/test_context_validation.py), material resolution (tests/test_material.py), .hdr loading,
lighting calibration."""

import numpy as np
import pytest

import mujoco_warp_pbr_gb300 as mjpbr
from mujoco_warp_pbr_gb300 import context
from mujoco_warp_pbr_gb300 import synthetic
from mujoco_warp_pbr_gb300.synthetic import GEOM_PLANE, GEOM_SPHERE, LIGHT_DIRECTIONAL, Builder


@pytest.fixture(scope="module")
def mjm():
  b = Builder()
  b.light(LIGHT_DIRECTIONAL, pos=(0, 0, 3), dir=(0, 0, -1))
  b.camera((0, -3, 1), xyaxes=(1, 0, 0, 0, 0.3, 1), resolution=(8, 8))
  b.geom(GEOM_SPHERE, (0.5, 0, 0), pos=(0, 0, 0.5))
  return b.build()[0]


BAD_ARGS = [
  ({"tier": 5}, "tier must be one of"),
  ({"tone_mapper": -1}, "tone_mapper must be one of"),
  ({"light_model": 3}, "light_model must be one of"),
  ({"render_order": 9}, "render_order must be one of"),
  ({"unset_material": 2}, "unset_material must be one of"),
  ({"samples_per_pixel": 0}, "samples_per_pixel must be at least 1"),
  ({"shadow_samples": 0}, "shadow_samples must be at least 1"),
  ({"path_samples": 0}, "path_samples must be at least 1"),
  ({"max_layers": 0}, "max_layers must be at least 1"),
  ({"max_depth": -1}, "max_depth must be at least 0"),
  ({"tier": 1, "max_depth": 40, "max_layers": 6}, "random number layout"),
  ({"shadow_light_fraction": 1.5}, "shadow_light_fraction must be in"),
  ({"default_material": {"metalic": 0.5}}, "default_material keys"),
  ({"default_material": {"roughness": 2.0}}, r"default_material\['roughness'\] must be in"),
  ({"envmap": np.zeros((8, 16), np.float32)}, r"envmap\[0\] must be a path or a \(height, width, 3\)"),
  ({"envmap": [np.zeros((8, 16, 3), np.float32), np.zeros((8, 16, 5), np.float32)]}, r"envmap\[1\]"),
  ({"denoise": True}, "denoise applies to the path-traced tier"),
  ({"traversal": "hardware"}, "traversal must be"),
  ({"mesh_bvh_frame": "local"}, "mesh_bvh_frame must be"),
  ({"mesh_bvh_constructor": "median"}, "mesh_bvh_constructor must be one of"),
  ({"block_dim": 0}, "block_dim must be at least 1"),
]


@pytest.mark.parametrize("kwargs,match", BAD_ARGS, ids=[m for _, m in BAD_ARGS])
def test_invalid_arguments(mjm, kwargs, match):
  with pytest.raises(ValueError, match=match):
    mjpbr.create_render_context(mjm, cam_res=(8, 8), render_rgb=True, **kwargs)


def test_nothing_to_render(mjm):
  with pytest.raises(ValueError, match="no geoms in the enabled geom groups"):
    context.prepare_context(mjm, 1, enabled_geom_groups=(5,))


def test_enum_arguments_accept_ints(mjm):
  hc = context.prepare_context(mjm, 1, cam_res=(8, 8), tone_mapper=1, render_order=0, tier=0)
  assert hc.settings["tone_mapper"] == mjpbr.ToneMapper.ACES and hc.settings["render_order"] == mjpbr.RenderOrder.ROW


def _material_model():
  b = Builder()
  authored = b.material(metallic=0.3, roughness=0.6, specular=0.7)
  legacy = b.material(shininess=0.8, rgba=(0.5, 0.5, 0.5, 1))
  white = b.material(rgba=(0.9, 0.9, 0.9, 1))
  b.geom(GEOM_SPHERE, (0.1, 0, 0), matid=authored)
  b.geom(GEOM_SPHERE, (0.1, 0, 0), matid=legacy)
  b.geom(GEOM_SPHERE, (0.1, 0, 0), matid=white)
  b.geom(GEOM_SPHERE, (0.1, 0, 0), rgba=(0.1, 0.1, 0.1, 1))
  b.geom(GEOM_PLANE, (1, 1, 0.1), matid=legacy)
  b.camera((0, -1, 0), xyaxes=(1, 0, 0, 0, 0, 1))
  return b.build()[0]


def _resolve(**kwargs):
  m, r, f = mjpbr.resolve_geom_materials(_material_model(), **kwargs)
  names = ["authored", "legacy", "white", "nomat", "floor"]
  return {n: (m[i], r[i], f[i]) for i, n in enumerate(names)}


def test_gltf_policy():
  r = _resolve()
  np.testing.assert_allclose(r["authored"], (0.3, 0.6, 0.7), rtol=1e-6)
  np.testing.assert_allclose(r["legacy"], (0.0, 0.2, 0.5), rtol=1e-6)
  np.testing.assert_allclose(r["nomat"], (0.0, 0.5, 0.5), rtol=1e-6)


def test_default_material_only_fills_unset_fields():
  r = _resolve(default_material={"metallic": 1.0, "roughness": 0.1})
  np.testing.assert_allclose(r["authored"][:2], (0.3, 0.6), rtol=1e-6)
  np.testing.assert_allclose(r["legacy"][:2], (1.0, 0.1), rtol=1e-6)


def test_heuristic_policy():
  r = _resolve(unset_material=mjpbr.UnsetMaterial.HEURISTIC)
  np.testing.assert_allclose(r["authored"], (0.3, 0.6, 0.7), rtol=1e-6)
  np.testing.assert_allclose(r["legacy"], (0.6, 0.40 * (1.3 - 0.8), 0.7), rtol=1e-5)
  np.testing.assert_allclose(r["white"], (0.0, 0.38, 0.65), rtol=1e-6)
  np.testing.assert_allclose(r["nomat"], (0.4, 0.45, 0.35), rtol=1e-6)
  np.testing.assert_allclose(r["floor"], (0.0, 1.0, 0.0), rtol=1e-6)


def _rgbe(image):
  peak = image.max(axis=-1)
  exponent = np.where(peak > 1e-32, np.ceil(np.log2(np.maximum(peak, 1e-32))), -128).astype(np.int32)
  mantissa = np.clip(image / np.ldexp(1.0, exponent)[..., None] * 256.0, 0, 255).astype(np.uint8)
  return np.concatenate([mantissa, (exponent + 128).clip(0, 255).astype(np.uint8)[..., None]], axis=-1)


def _write_flat(path, image):
  header = f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {image.shape[0]} +X {image.shape[1]}\n".encode()
  path.write_bytes(header + _rgbe(image).tobytes())


def _rle_channel(values):
  out = bytearray()
  i, n = 0, len(values)
  while i < n:
    run = 1
    while i + run < n and run < 127 and values[i + run] == values[i]:
      run += 1
    if run >= 3:
      out += bytes([128 + run, int(values[i])])
      i += run
      continue
    j = i
    while j < n and j - i < 128 and not (j + 2 < n and values[j] == values[j + 1] == values[j + 2]):
      j += 1
    out += bytes([j - i]) + bytes(values[i:j])
    i = j
  return bytes(out)


def test_load_hdr_roundtrip(tmp_path):
  image = np.random.default_rng(0).uniform(0.0, 50.0, size=(4, 6, 3)).astype(np.float32)
  _write_flat(tmp_path / "env.hdr", image)
  tolerance = image.max(axis=-1, keepdims=True) / 128.0
  assert np.all(np.abs(mjpbr.load_hdr(tmp_path / "env.hdr") - image) <= tolerance)


def test_load_hdr_run_length(tmp_path):
  rng = np.random.default_rng(0)
  image = rng.uniform(0.0, 4.0, (5, 40, 3)).astype(np.float32)
  image[:, 10:30] = 1.5
  h, w, _ = image.shape
  rgbe = _rgbe(image)
  body = bytearray()
  for y in range(h):
    body += bytes([2, 2, w >> 8, w & 0xFF])
    for c in range(4):
      body += _rle_channel(rgbe[y, :, c])
  (tmp_path / "env.hdr").write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode() + bytes(body))
  scale = np.ldexp(1.0, rgbe[..., 3].astype(np.int32) - 136)
  np.testing.assert_array_equal(mjpbr.load_hdr(tmp_path / "env.hdr"), (rgbe[..., :3] * scale[..., None]).astype(np.float32))


@pytest.mark.parametrize(
  "data,match",
  [
    (b"P6\n", "not a Radiance .hdr file"),
    (b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n", "truncated .hdr header"),
    (b"#?RADIANCE\n\n+Y 2 +X 2\n" + bytes(16), "only '-Y H \\+X W'"),
    (b"#?RADIANCE\n\n-Y 2 +X 2\n" + bytes(10), "truncated pixel data"),
    (b"#?RADIANCE\n\n-Y 1 +X 8\n" + bytes([2, 2, 0, 8, 200, 1]), "bad run-length data"),
    (b"#?RADIANCE\n\n-Y 1 +X 8\n" + bytes([2, 2, 0, 9]), "width does not match"),
    (b"#?RADIANCE\n\n-Y 1 +X 8\n" + bytes([2, 2, 0, 8, 136]), "bad run-length data"),
  ],
)
def test_load_hdr_malformed(tmp_path, data, match):
  (tmp_path / "bad.hdr").write_bytes(data)
  with pytest.raises(ValueError, match=match):
    mjpbr.load_hdr(tmp_path / "bad.hdr")


def test_exposure_from_ev100():
  ev100 = np.log2(16.0**2 / (1 / 125) * 100 / 100)
  assert context.exposure_from_ev100(ev100) == pytest.approx(1.0 / (1.2 * 2**ev100))


def test_fallback_intensity_calibration():
  sc = synthetic.primitive_scene(seed=0, nworld=1, res=8)
  exposure, intensity, ambient = context.resolve_lighting(sc.mjm, sc.mjd.light_xpos[0], 0, context.DEFAULT_EV100)
  assert intensity[0] == pytest.approx(np.pi / exposure, rel=1e-6)  # directional: pi / exposure lux
  d = max(np.linalg.norm(sc.mjd.light_xpos[0][1] - np.asarray(sc.mjm.stat_center)), 0.1 * sc.mjm.stat_extent)
  assert intensity[1] == pytest.approx(np.pi / exposure * d * d, rel=1e-5)


def test_output_layout():
  b = Builder()
  b.geom(GEOM_PLANE, (1, 1, 0.1))
  b.camera((0, 0, 1), xyaxes=(1, 0, 0, 0, 1, 0), resolution=(4, 3))
  b.camera((0, 0, 1), xyaxes=(1, 0, 0, 0, 1, 0), resolution=(5, 2))
  mjm, mjd = b.build()
  hc = context.prepare_context(mjm, 2, data=mjd, render_rgb=[True, False], render_depth=True, render_seg=[False, True])
  o = hc.outputs
  assert o["total_rays"] == 12 + 10 and o["ray_adr"] == [0, 12]
  assert o["rgb_adr"] == [0, -1] and o["rgb_stride"] == 12
  assert o["depth_adr"] == [0, 12] and o["depth_stride"] == 22
  assert o["seg_adr"] == [-1, 0] and o["seg_stride"] == 10


_NESTED = ("headlight_active", "headlight_ambient", "headlight_diffuse", "headlight_specular", "stat_center", "stat_extent", "znear", "zfar")


def _as_mujoco(hm):
  """A stand-in for mujoco.MjModel: HostModel's arrays under their (shared) MuJoCo names, the
  headlight, statistics and clip planes in MuJoCo's nested vis / stat structs."""
  import dataclasses
  from types import SimpleNamespace

  from mujoco_warp_pbr_gb300.model import HostModel

  ns = SimpleNamespace(**{f.name: getattr(hm, f.name) for f in dataclasses.fields(HostModel) if f.name not in _NESTED})
  ns.vis = SimpleNamespace(
    headlight=SimpleNamespace(active=int(hm.headlight_active), ambient=np.array(hm.headlight_ambient, np.float32),
                              diffuse=np.array(hm.headlight_diffuse, np.float32), specular=np.array(hm.headlight_specular, np.float32)),
    map=SimpleNamespace(znear=hm.znear / hm.stat_extent, zfar=hm.zfar / hm.stat_extent),
  )
  ns.stat = SimpleNamespace(center=np.array(hm.stat_center), extent=hm.stat_extent)
  return ns


def test_mujoco_model_is_accepted():
  """A mujoco.MjModel keeps the headlight, statistics and clip planes in nested structs (the
  reference reads mjm.vis.headlight, mjm.stat: io.py:242-243, lights.py:146-147); the context built
  from one equals the context built from the flat HostModel."""
  import dataclasses

  from mujoco_warp_pbr_gb300 import model as model_lib

  sc = synthetic.primitive_scene(seed=4, nworld=2, res=16)
  hm = dataclasses.replace(sc.mjm, headlight_active=True, headlight_ambient=(0.2, 0.1, 0.05), stat_extent=2.5, znear=0.025, zfar=125.0)
  fake = _as_mujoco(hm)
  conv = model_lib.as_host_model(fake)
  for f in dataclasses.fields(type(hm)):
    a, b = getattr(conv, f.name), getattr(hm, f.name)
    if isinstance(b, np.ndarray):
      np.testing.assert_array_equal(a, b, err_msg=f.name)
    else:
      np.testing.assert_allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=1e-6, err_msg=f.name)
  assert model_lib.as_host_model(hm) is hm
  a = context.prepare_context(fake, 2, data=sc.mjd, **sc.options)
  b = context.prepare_context(hm, 2, data=sc.mjd, **sc.options)
  assert a.settings.keys() == b.settings.keys()
  for k in b.settings:
    np.testing.assert_allclose(np.asarray(a.settings[k], np.float64), np.asarray(b.settings[k], np.float64), rtol=1e-6, err_msg=k)
  for k in b.tables:
    np.testing.assert_array_equal(a.tables[k], b.tables[k], err_msg=k)
  np.testing.assert_array_equal(a.tlas_child, b.tlas_child)


def test_mujoco_model_without_required_fields():
  from mujoco_warp_pbr_gb300 import model as model_lib

  fake = _as_mujoco(synthetic.primitive_scene(seed=0, nworld=1, res=8).mjm)
  del fake.light_intensity
  with pytest.raises(ValueError, match="light_intensity .*MuJoCo 3.3"):
    model_lib.as_host_model(fake)
