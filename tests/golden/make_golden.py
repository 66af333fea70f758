"""Regenerates the golden fixtures of tests/test_golden.py from the CPU oracle.

The reference ships no golden images (its tests are analytic or relative), so these fixtures pin
the oracle itself: geometry (segmentation, depth) must reproduce bit for bit on every machine the
oracle is compiled on (x86-64 or aarch64), colours within 1/255.

  python tests/golden/make_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from mujoco_warp_pbr_gb300 import synthetic  # noqa: E402
from oracle import oracle  # noqa: E402

CASES = {
  "primitives_seed3": lambda: synthetic.primitive_scene(seed=3, nworld=2, res=32, shadow_samples=4),
  "mesh_ibl_seed5": lambda: synthetic.mesh_ibl_scene(seed=5, nworld=1, res=32, tex_size=64, env_width=128),
}
SEED = 11


def render(name: str) -> dict[str, np.ndarray]:
  sc = CASES[name]()
  o = oracle.OracleScene(sc.mjm, sc.mjd, sc.nworld, {**sc.options, "render_hdr": True}, sc.per_world)
  out = o.render(seed=SEED)
  return {"seg": out["seg"].copy(), "depth": out["depth"].copy(), "rgb": out["rgb"].copy(), "hdr": out["hdr"].astype(np.float32)}


def main() -> None:
  for name in CASES:
    np.savez_compressed(HERE / f"{name}.npz", **render(name))
    print("wrote", name)


if __name__ == "__main__":
  main()
