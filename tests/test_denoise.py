"""A-trous denoiser of the path-traced tier: the reference's tests (tests/test_denoise.py of
mujoco_warp_pbr) restated on array scenes, run on the oracle and on the GPU, and GPU-vs-oracle
parity of the filter itself (the oracle filters the GPU's own demodulated image and guide, so the
comparison isolates the filter from Monte Carlo path divergence)."""

import numpy as np
import pytest

from tests import kat
from tests.kat import GEOM_PLANE, GEOM_SPHERE, Builder

torch = pytest.importorskip("torch")

GPU = [pytest.mark.gpu, pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]
RENDERERS = [pytest.param("oracle", id="oracle"), pytest.param("gpu", id="gpu", marks=GPU)]
# Exposure 1: radiance is display-relative, so the emissive sphere is about as bright as the sky.
PATH = {"tier": 1, "render_hdr": True, "ev100": float(np.log2(1.0 / 1.2))}


@pytest.fixture(params=RENDERERS)
def render(request):
  return kat.render if request.param == "oracle" else kat.render_gpu


def _checker(n: int = 64) -> np.ndarray:
  """MuJoCo's builtin 2 x 2 checker, rgb1 0.9 and rgb2 0.1."""
  y, x = np.mgrid[0:n, 0:n]
  on = ((x < n // 2) ^ (y < n // 2)).astype(bool)
  img = np.where(on[..., None], 0.9, 0.1) * 255.0 + 0.5
  return np.concatenate([img.astype(np.uint8).repeat(3, -1)[..., :3], np.full((n, n, 1), 255, np.uint8)], -1)


def _floor_and_glow(res: int = 64) -> Builder:
  """A checkered rough floor and an emissive sphere (noisy at low sample counts, with texture and
  emission the filter must preserve)."""
  b = Builder()
  tex = b.texture(_checker())
  floor = b.material(rgba=(1, 1, 1, 1), roughness=0.8, texid={1: tex}, texrepeat=(4, 4))
  glow = b.material(rgba=(0.2, 0.2, 0.2, 1), emission=1.0, roughness=0.5)
  b.geom(GEOM_PLANE, (2, 2, 0.1), matid=floor)
  b.geom(GEOM_SPHERE, (0.3, 0, 0), pos=(0, 0, 0.3), matid=glow)
  b.camera(pos=(0, -2.5, 1.5), xyaxes=(1, 0, 0, 0, 0.5, 0.866), fovy=45.0, resolution=(res, res))
  return b


def _env() -> np.ndarray:
  return np.random.default_rng(0).uniform(0, 2, (32, 64, 3)).astype(np.float32)


def test_requires_path_tier():
  import mujoco_warp_pbr_gb300 as mjpbr

  mjm, _ = _floor_and_glow(8).build()
  with pytest.raises(ValueError, match="path-traced"):
    mjpbr.context.prepare_context(mjm, 1, denoise=True)


def test_zero_iterations_is_identity(render):
  opts = dict(envmap=_env(), envmap_intensity=1.0, path_samples=4, **PATH)
  raw = render(_floor_and_glow(), **opts)
  passthrough = render(_floor_and_glow(), denoise=True, denoise_iterations=0, **opts)
  np.testing.assert_allclose(passthrough["hdr"], raw["hdr"], rtol=1e-4, atol=1e-6)
  np.testing.assert_allclose(passthrough["rgb"], raw["rgb"], atol=1.5 / 255)


@pytest.mark.slow
def test_reduces_error(render):
  opts = dict(envmap=_env(), envmap_intensity=1.0, **PATH)
  reference = render(_floor_and_glow(), path_samples=2048, **opts)["hdr"]
  raw = render(_floor_and_glow(), path_samples=4, **opts)["hdr"]
  denoised = render(_floor_and_glow(), path_samples=4, denoise=True, **opts)["hdr"]

  def error(x):
    return np.mean(np.abs(x - reference) / (reference + 0.05))

  assert error(denoised) < 0.6 * error(raw)
  # filtering preserves energy
  np.testing.assert_allclose(denoised.mean(), reference.mean(), rtol=0.03)


def _unpack_guide(g: np.ndarray) -> dict[str, np.ndarray]:
  g = np.ascontiguousarray(g).view(np.uint32)
  halves = g[..., :3].copy().view(np.uint16).view(np.float16).astype(np.float32)
  return {"normal": halves[..., 0:3], "albedo": halves[..., 3:6], "depth": g[..., 3].copy().view(np.float32)}


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("iterations", [1, 3, 5])
def test_filter_matches_oracle(iterations):
  """The GPU filter against the oracle's, on the GPU path tracer's own buffers."""
  import mujoco_warp_pbr_gb300 as mjpbr
  from oracle import oracle
  from tests import helpers

  b = _floor_and_glow(72)
  mjm, mjd = b.build()
  opts = dict(envmap=_env(), envmap_intensity=1.0, path_samples=4, denoise=True, denoise_iterations=iterations, render_rgb=True, **PATH)
  nworld = 2
  m = mjpbr.put_model(mjm)
  d = mjpbr.put_data(mjm, mjd, nworld=nworld)
  rc = mjpbr.create_render_context(mjm, nworld, data=mjd, **opts)
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=3, denoise=False)
  torch.cuda.synchronize()
  guide = rc.aov_guide.cpu().numpy()
  emission = rc.aov_emission.cpu().numpy()
  demod = rc.denoise_buffers[0].cpu().numpy()
  mjpbr.denoise(m, d, rc)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  gpu_rgb = rc.base.rgb_data.cpu().numpy().view(np.uint32)
  gpu_hdr = rc.hdr_data.cpu().numpy()

  o = oracle.OracleScene(mjm, mjd, nworld, opts, {}, tables=helpers.gpu_tables(rc))
  o.aov["guide"][...] = guide.view(np.uint32)
  o.aov["emission"][...] = emission
  o.aov["demod"][...] = demod
  o.denoise()
  diff = helpers.rgb_diff(gpu_rgb, o.rgb)
  assert diff.max() <= 1, f"max RGB difference {diff.max()}/255"
  np.testing.assert_allclose(gpu_hdr, o.hdr, rtol=1e-3, atol=1e-4)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_features_match_oracle():
  """Guide, emission and demodulated radiance of the GPU path tracer against the oracle's."""
  import mujoco_warp_pbr_gb300 as mjpbr
  from tests import helpers

  b = _floor_and_glow(48)
  mjm, mjd = b.build()
  opts = dict(envmap=_env(), envmap_intensity=1.0, path_samples=4, denoise=True, render_rgb=True, **PATH)
  nworld = 2
  m = mjpbr.put_model(mjm)
  d = mjpbr.put_data(mjm, mjd, nworld=nworld)
  rc = mjpbr.create_render_context(mjm, nworld, data=mjd, **opts)
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=9, denoise=False)
  torch.cuda.synchronize()
  from oracle import oracle

  o = oracle.OracleScene(mjm, mjd, nworld, opts, {}, tables=helpers.gpu_tables(rc))
  ref = o.render(seed=9, denoise=False)
  g, r = _unpack_guide(rc.aov_guide.cpu().numpy()), _unpack_guide(ref["aov_guide"])
  np.testing.assert_allclose(g["depth"], r["depth"], rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(g["normal"], r["normal"], atol=2e-3)
  close = np.isclose(g["albedo"], r["albedo"], atol=2e-3).all(-1)
  assert close.mean() >= 0.995
  demod, ref_demod = rc.denoise_buffers[0].cpu().numpy(), ref["aov_demod"]
  err = np.abs(demod[..., :3] - ref_demod[..., :3]).mean()
  assert err <= 0.01 * np.abs(ref_demod[..., :3]).mean()
