"""mjpbr_denoise_learned: the learned denoiser through one C call (what a caller without Python
binds) gives the same images as kpcn.KPCN.denoise, and rejects what it cannot run."""

import ctypes

import numpy as np
import pytest

from mujoco_warp_pbr_gb300 import _lib

torch = pytest.importorskip("torch")


def test_workspace_size_rules():
  lib = _lib.load()
  assert lib.mjpbr_kpcn_workspace_bytes(4, 128, 128) > 0
  assert lib.mjpbr_kpcn_workspace_bytes(4, 120, 128) == -1  # 120 rows: the 16-row level is not tiled
  assert lib.mjpbr_kpcn_workspace_bytes(0, 128, 128) == -1
  assert lib.mjpbr_kpcn_workspace_bytes(8, 128, 128) > lib.mjpbr_kpcn_workspace_bytes(4, 128, 128)


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
def test_c_entry_matches_the_python_denoiser():
  from pathlib import Path

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import kpcn, synthetic
  from tests import helpers

  sc = synthetic.path_scene(seed=4, nworld=6, res=128)
  m, d, rc = helpers.gpu_scene(sc, denoise=True)
  net = kpcn.KPCN.load(Path(kpcn.__file__).resolve().parent / "weights" / "kpcn_path.npz")

  def frame(run):
    for t in (rc.base.rgb_data, rc.hdr_data):
      t.zero_()
    mjpbr.refit_bvh(m, d, rc)
    mjpbr.render(m, d, rc, seed=3, denoise=False)
    run()
    torch.cuda.synchronize()
    assert mjpbr.check_errors(rc) == 0
    return rc.base.rgb_data.cpu().numpy().copy(), rc.hdr_data.cpu().numpy().copy()

  ref = frame(lambda: net.denoise(m, d, rc, chunk=4, driver="python"))
  lib = _lib.load()
  scene = mjpbr.scene_descriptor(m, d, rc)
  nbytes = lib.mjpbr_kpcn_workspace_bytes(4, 128, 128)
  ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
  wts = net.c_weights()
  stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

  def c_call():
    status = lib.mjpbr_denoise_learned(ctypes.byref(scene), ctypes.byref(wts), ctypes.c_void_p(ws.data_ptr()), nbytes, 4, stream)
    assert status == 0, lib.mjpbr_last_error().decode()

  got = frame(c_call)
  for a, b in zip(got, ref):
    np.testing.assert_array_equal(a, b)
  # the default driver of KPCN.denoise is this call
  got2 = frame(lambda: net.denoise(m, d, rc, chunk=4))
  for a, b in zip(got2, ref):
    np.testing.assert_array_equal(a, b)
  # a workspace one byte short and a chunk of zero are rejected before any launch
  assert lib.mjpbr_denoise_learned(ctypes.byref(scene), ctypes.byref(wts), ctypes.c_void_p(ws.data_ptr()), nbytes - 1, 4, stream) == _lib.ERR_ARG
  assert lib.mjpbr_denoise_learned(ctypes.byref(scene), ctypes.byref(wts), ctypes.c_void_p(ws.data_ptr()), nbytes, 0, stream) == _lib.ERR_ARG
