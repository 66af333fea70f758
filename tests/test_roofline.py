"""The FP32 roofline model of the render kernels (mujoco_warp_pbr_gb300/roofline.py) on CPU: the
counter layout matches csrc/opcount.cuh, copies are summed, and the roofline scales counts of a
sample frame to the timed frame."""

import re
from pathlib import Path

import pytest

from mujoco_warp_pbr_gb300 import roofline

ROOT = Path(__file__).resolve().parent.parent


def test_counter_order_matches_the_device_enum():
  src = (ROOT / "mujoco_warp_pbr_gb300" / "csrc" / "opcount.cuh").read_text()
  body = src[src.index("enum OpCount") : src.index("kOpCountN")]
  names = re.findall(r"\bkOp(\w+)", body)
  snake = [re.sub(r"(?<!^)(?=[A-Z])", "_", n).lower() for n in names]
  aliases = {"tri": "triangle"}
  assert [aliases.get(n, n) for n in snake] == list(roofline.OPS)
  assert f"kOpCopies = {roofline.COPIES}" in src
  assert set(roofline.FLOPS_PER_OP) == set(roofline.OPS)


def test_copies_are_summed_and_scaled():
  raw = [0] * (len(roofline.OPS) * roofline.COPIES)
  i_box = roofline.OPS.index("box")
  i_ray = roofline.OPS.index("ray_closest")
  for c in range(roofline.COPIES):
    raw[i_box * roofline.COPIES + c] = 10
    raw[i_ray * roofline.COPIES + c] = 1
  counts = roofline.counts_from_device(raw)
  assert counts["box"] == 10 * roofline.COPIES and counts["ray_closest"] == roofline.COPIES
  assert roofline.rays(counts) == roofline.COPIES
  flops = roofline.flops(counts)
  assert flops == 10 * roofline.COPIES * roofline.FLOPS_PER_OP["box"] + roofline.COPIES * roofline.FLOPS_PER_OP["ray_closest"]
  # a sample of 100 pixels scaled to a 1000-pixel frame rendered in 1 ms
  r = roofline.fp32_roofline(counts, 100, 1000, 1.0)
  assert r["flops_per_px"] == pytest.approx(flops / 100)
  assert r["achieved"] == pytest.approx(flops * 10 / 1e-3 / 1e12)
  assert r["frac"] == pytest.approx(r["achieved"] / roofline.FP32_PEAK_TFLOPS)
  assert roofline.FP32_PEAK_TFLOPS == pytest.approx(80.55, abs=0.01)


def test_bench_reads_committed_traffic():
  """The bench's roofline.traffic comes from the committed ncu figures, per workload."""
  import bench

  assert bench._traffic("mesh_ibl_4096x128") == 138889244928
  assert bench._traffic("path_1024x128_spp2") == 57841523456
  assert bench._traffic("mesh_ibl_1024x128") is None
