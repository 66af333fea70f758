"""Shading error at sampled pixels against a float64 CPU re-evaluation (oracle/fp64_shading.py):
the FP32 renderers' linear HDR radiance on the primitive workload (one sample per pixel, hard
shadows, directional + point light, ambient sky) compared pixel by pixel with the same shading
model evaluated in float64 from the scene description. The statistics are printed; the bars are
FP32-level agreement (median relative error below 1e-6, 99th percentile below 1e-4)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mujoco_warp_pbr_gb300 import synthetic  # noqa: E402
from oracle import fp64_shading  # noqa: E402
from oracle import oracle  # noqa: E402
from tests import helpers  # noqa: E402

OPTS = {"render_hdr": True, "specular_aa": False}


def _check(stats):
  print(stats)
  assert stats["pixels"] >= 500
  assert stats["mismatched_hits"] <= 0.02 * (stats["pixels"] + stats["mismatched_hits"])
  assert stats["median"] < 1e-6
  assert stats["p99"] < 1e-4
  assert stats["max"] < 2e-2  # shadow-boundary pixels may flip visibility


@pytest.mark.parametrize("light_model", [0, 1])
def test_oracle_against_float64(light_model):
  sc = synthetic.primitive_scene(seed=1, nworld=3, res=40, shadow_samples=1)
  opts = {**OPTS, "light_model": light_model}
  dfg = oracle.dfg_lut()
  out = helpers.oracle_render(sc, tables={"dfg_lut": dfg}, **opts)
  fp = fp64_shading.Fp64Scene(sc, dfg, **opts)
  _check(fp64_shading.shading_error(fp, out["hdr"], out["seg"], npix=1000))


def test_reevaluation_rejects_unsupported_settings():
  sc = synthetic.primitive_scene(seed=1, nworld=1, res=8, shadow_samples=4)
  with pytest.raises(ValueError, match="hard shadows"):
    fp64_shading.Fp64Scene(sc, oracle.dfg_lut(), **OPTS)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("light_model", [0, 1])
def test_gpu_against_float64(light_model):
  sc = synthetic.primitive_scene(seed=2, nworld=8, res=64, shadow_samples=1)
  opts = {**OPTS, "light_model": light_model}
  m, d, rc = helpers.gpu_scene(sc, **opts)
  gpu = helpers.render_gpu(m, d, rc, seed=0)
  fp = fp64_shading.Fp64Scene(sc, rc.dfg_lut.cpu().numpy(), **opts)
  _check(fp64_shading.shading_error(fp, gpu["hdr"], gpu["seg"], npix=4000))
