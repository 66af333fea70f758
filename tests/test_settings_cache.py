"""Settings and arrays changed after the first render (the reference's tests/test_kernel_cache.py
restated on an array scene): a changed setting renders as a context created with it, the tier can
be switched, replaced arrays take effect, and replaced arrays that need a flag that is off warn.
The warning logic itself runs on the CPU; the renders need a GPU."""

import warnings

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import mujoco_warp_pbr_gb300 as mjpbr  # noqa: E402
from mujoco_warp_pbr_gb300.render import _warn_ignored_overrides  # noqa: E402
from mujoco_warp_pbr_gb300 import synthetic  # noqa: E402
from oracle import oracle  # noqa: E402

RES = (24, 16)  # width, height


def _model():
  """Plane, sphere and box under one shadow-casting light, one camera (as the reference's scene)."""
  b = synthetic.Builder()
  b.geom(synthetic.GEOM_PLANE, (3, 3, 0.1), rgba=(0.7, 0.7, 0.7, 1))
  b.geom(synthetic.GEOM_SPHERE, (0.5, 0, 0), pos=(0, 0, 0.5), rgba=(0.8, 0.3, 0.2, 1))
  b.geom(synthetic.GEOM_BOX, (0.2, 0.2, 0.3), pos=(0.9, 0.3, 0.3), rgba=(0.2, 0.4, 0.9, 1))
  b.light(synthetic.LIGHT_SPOT, pos=(0, 0, 3), dir=(0, 0, -1), castshadow=True, cutoff=45.0)
  b.camera((0, -3, 1.2), xyaxes=(1, 0, 0, 0, 0.35, 1), resolution=RES)
  return b.build()


class Scene:
  def __init__(self, nworld=1, **kwargs):
    self.mjm, self.mjd = _model()
    self.m = mjpbr.put_model(self.mjm)
    self.d = mjpbr.put_data(self.mjm, self.mjd, nworld=nworld)
    self.rc = mjpbr.create_render_context(self.mjm, nworld, data=self.mjd, cam_res=RES, render_seg=True, **kwargs)

  def render(self, seed=0):
    mjpbr.refit_bvh(self.m, self.d, self.rc)
    mjpbr.render(self.m, self.d, self.rc, seed=seed)
    torch.cuda.synchronize()
    assert mjpbr.check_errors(self.rc) == 0
    return self

  def rgb(self):
    return oracle.unpack_rgb(self.rc.base.rgb_data.cpu().numpy().view(np.uint32)).astype(np.float64) / 255.0

  def seg(self):
    return self.rc.base.seg_data.cpu().numpy().copy()


CHANGES = [
  ("render_order", mjpbr.RenderOrder.WORLD),
  ("render_order", mjpbr.RenderOrder.ROW),
  ("tone_mapper", mjpbr.ToneMapper.ACES),
  ("use_shadows", False),
  ("samples_per_pixel", 2),
  ("shadow_light_fraction", 0.5),
]


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("field,value", CHANGES, ids=[f"{f}={v}" for f, v in CHANGES])
def test_change_after_first_render(field, value):
  s = Scene(nworld=2).render()
  setattr(s.rc, field, value)
  s.render()
  expected = Scene(nworld=2, **{field: value}).render()
  np.testing.assert_allclose(s.rgb(), expected.rgb(), atol=1.5 / 255)
  np.testing.assert_array_equal(s.seg(), expected.seg())


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_tier_switch():
  s = Scene(path_samples=2).render()
  s.rc.tier = int(mjpbr.Tier.PATH)
  s.render(seed=3)
  expected = Scene(tier=mjpbr.Tier.PATH, path_samples=2).render(seed=3)
  np.testing.assert_allclose(s.rgb(), expected.rgb(), atol=1.5 / 255)
  np.testing.assert_array_equal(s.seg(), expected.seg())


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_segmentation_background_written_every_frame():
  s = Scene().render()
  seg = s.seg()
  assert np.all(seg[0, 0] == -1)  # the top-left pixel sees the sky
  s.rc.base.seg_data.fill_(7)
  s.render()
  np.testing.assert_array_equal(s.seg(), seg)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_replaced_array_is_used():
  s = Scene().render()
  before = s.rgb()
  np.testing.assert_array_equal(s.render().rgb(), before)
  ngeom = s.mjm.ngeom
  s.rc.geom_roughness = torch.full((1, ngeom), 0.05, device=s.rc.device)
  s.rc.geom_metallic = torch.ones((1, ngeom), device=s.rc.device)
  s.render()
  assert np.abs(s.rgb() - before).max() > 0.05


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_translucent_override_warns_until_enabled():
  s = Scene().render()
  assert not s.rc.has_transparency
  rgba = s.m.geom_rgba.clone()
  rgba[..., 3] = 0.5
  s.m.geom_rgba = rgba
  with pytest.warns(UserWarning, match="has_transparency"):
    s.render()
  opaque = s.rgb()
  s.rc.has_transparency = True
  s.render()
  assert np.abs(s.rgb() - opaque).max() > 0.05


class _Ctx:
  """The two flags and the host cache of a render context, for the CPU check of the warning."""

  def __init__(self):
    self.has_transparency = False
    self.has_reflection = False
    self.mat_reflectance = torch.zeros(1, 2)
    self._host_cache = {}
    self.device = torch.device("cpu")


class _M:
  def __init__(self, rgba):
    self.geom_rgba = rgba


def test_override_warning_rules():
  rc = _Ctx()
  opaque = torch.ones(1, 3, 4)
  with warnings.catch_warnings():
    warnings.simplefilter("error")
    _warn_ignored_overrides(_M(opaque), rc)  # first arrays: not checked
    _warn_ignored_overrides(_M(opaque), rc)  # same array again
    _warn_ignored_overrides(_M(torch.ones(1, 3, 4)), rc)  # replaced, still opaque
    half = torch.ones(1, 3, 4)
    half[..., 3] = 0.0  # alpha 0 hides a geom: needs no flag
    _warn_ignored_overrides(_M(half), rc)
  half = torch.ones(1, 3, 4)
  half[0, 1, 3] = 0.5
  with pytest.warns(UserWarning, match="rc.has_transparency = True"):
    _warn_ignored_overrides(_M(half), rc)
  rc.mat_reflectance = torch.tensor([[0.0, 0.3]])
  with pytest.warns(UserWarning, match="has_reflection"):
    _warn_ignored_overrides(_M(half), rc)
  rc.has_transparency = rc.has_reflection = True
  with warnings.catch_warnings():
    warnings.simplefilter("error")
    _warn_ignored_overrides(_M(half.clone()), rc)
    rc.mat_reflectance = torch.tensor([[0.5, 0.3]])
    _warn_ignored_overrides(_M(half.clone()), rc)
