"""BF16 tensor-core GEMM (tcgen05.mma, FP32 accumulation in tensor memory) against a CPU product
of the same BF16 values: pins the shared-memory and instruction descriptor encodings that the
learned denoiser's convolution kernels use."""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_gemm_argument_errors_without_a_gpu():
  from mujoco_warp_pbr_gb300 import _lib

  lib = _lib.load()
  p = ctypes.c_void_p(16)
  assert lib.mjpbr_gemm_bf16(p, p, p, 100, 16, 16, None, None) == _lib.ERR_ARG
  assert b"multiple of 128" in lib.mjpbr_last_error()
  assert lib.mjpbr_gemm_bf16(p, p, p, 128, 20, 16, None, None) == _lib.ERR_ARG
  assert b"N must be" in lib.mjpbr_last_error()
  assert lib.mjpbr_gemm_bf16(p, p, p, 128, 16, 24, None, None) == _lib.ERR_ARG
  assert b"K must be" in lib.mjpbr_last_error()


@pytest.mark.gpu
@pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")
@pytest.mark.parametrize("m,n,k", [(128, 16, 16), (256, 96, 192), (128, 256, 64), (384, 48, 80), (128, 32, 1440)])
def test_gemm_matches_cpu_product(m, n, k):
  from mujoco_warp_pbr_gb300 import _lib

  g = torch.Generator().manual_seed(m * 7 + n * 3 + k)
  a = (torch.rand((m, k), generator=g) * 2 - 1).to(torch.bfloat16)
  b = (torch.rand((n, k), generator=g) * 2 - 1).to(torch.bfloat16)
  ref = a.float().numpy().astype(np.float64) @ b.float().numpy().astype(np.float64).T
  da, db = a.cuda(), b.cuda()
  d = torch.zeros((m, n), dtype=torch.float32, device="cuda")
  err = torch.zeros(1, dtype=torch.int32, device="cuda")
  stream = torch.cuda.current_stream().cuda_stream
  _lib.call("mjpbr_gemm_bf16", da.data_ptr(), db.data_ptr(), d.data_ptr(), m, n, k, err.data_ptr(), stream)
  torch.cuda.synchronize()
  assert int(err.item()) == 0
  np.testing.assert_allclose(d.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.sqrt(k))
