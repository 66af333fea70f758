"""Training and evaluation of the learned denoiser on pairs the path tracer renders itself.

A pair is one world's 128 x 128 image of a seeded path-traced scene (synthetic.path_scene: the
primitive scene with emissive quads, per-world materials and emission): the network input and the
noisy demodulated radiance from a denoising render at 1-4 spp, and the converged target: many
path-traced passes with other seeds, their HDR summed in FP64 on the device
(mjpbr_accumulate_f64) and demodulated with the noisy render's albedo and emission
(mjpbr_kpcn_target).

    python -m mujoco_warp_pbr_gb300.train_kpcn --out weights.npz [--crops 6144 --target-spp 1024 --steps 8000]

The committed weights (weights/kpcn_path.npz) came from --crops 6144 --frame-worlds 256
--target-spp 1024 --steps 8000 --batch 16 --lr 1e-3 --spp 2 --loss-space demod, then fine-tuned on
4096-spp targets: --init <those weights> --crops 2048 --frame-worlds 256 --target-spp 4096
--steps 4000 --batch 16 --lr 3e-4 --spp 2 --loss-space demod (held-out relMSE 0.0143 -> 0.0141).

prints one JSON line: training time and loss curve, and on held-out scenes the relative MSE
(mean((x - ref)^2 / (ref^2 + 0.01)) on linear HDR) against 4096-spp references of the learned
denoiser at 2 spp, the a-trous filter (5 iterations) at 16 spp and plain path tracing at 16 spp,
with the Mpix/s of each pipeline (render + denoise) measured with CUDA events.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import time
from dataclasses import dataclass

import numpy as np
import torch

import mujoco_warp_pbr_gb300 as mjpbr
from mujoco_warp_pbr_gb300 import _lib
from mujoco_warp_pbr_gb300 import kpcn as kpcn_lib
from mujoco_warp_pbr_gb300 import synthetic
from mujoco_warp_pbr_gb300.render import scene as scene_descriptor


@dataclass
class Frame:
  """A seeded batch of worlds on the device, with one context per sample count."""

  sc: synthetic.SyntheticScene
  m: object
  d: object

  def context(self, **opts):
    options = {**self.sc.options, **opts}
    rc = mjpbr.create_render_context(self.sc.mjm, self.sc.nworld, data=self.sc.mjd, **options)
    synthetic.apply_per_world(self.sc, self.m, rc)
    return rc


def make_frame(seed: int, nworld: int, res: int) -> Frame:
  sc = synthetic.path_scene(seed=seed, nworld=nworld, res=res, spp=2)
  m = mjpbr.put_model(sc.mjm)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=nworld)
  return Frame(sc, m, d)


def converged_hdr(fr: Frame, spp: int, per_pass: int = 256, seed0: int = 1_000_003) -> torch.Tensor:
  """FP64 sum over passes of the HDR (nworld, npix, 3) and the pass count (mean = sum / passes)."""
  rc = fr.context(path_samples=min(per_pass, spp), render_hdr=True)
  passes = max(1, spp // per_pass)
  acc = torch.zeros(rc.hdr_data.shape, dtype=torch.float64, device=rc.device)
  mjpbr.refit_bvh(fr.m, fr.d, rc)
  stream = torch.cuda.current_stream().cuda_stream
  for k in range(passes):
    mjpbr.render(fr.m, fr.d, rc, seed=seed0 + 7919 * k)
    _lib.call("mjpbr_accumulate_f64", rc.hdr_data.data_ptr(), acc.data_ptr(), rc.hdr_data.numel(), stream)
  return acc / passes


def noisy_pair(fr: Frame, spp: int, seed: int, gt_hdr: torch.Tensor | None):
  """(x0, radiance, target or None, rc) of a denoising render at spp."""
  rc = fr.context(path_samples=spp, denoise=True, render_hdr=True)
  mjpbr.refit_bvh(fr.m, fr.d, rc)
  mjpbr.render(fr.m, fr.d, rc, seed=seed, denoise=False)
  s = scene_descriptor(fr.m, fr.d, rc)
  n = fr.sc.nworld
  w, h = rc.base.cam_res[0]
  stream = torch.cuda.current_stream().cuda_stream
  x0 = torch.zeros((n, h, w, kpcn_lib.FEATURES), dtype=torch.bfloat16, device=rc.device)
  _lib.call("mjpbr_kpcn_features", ctypes.byref(s), 0, 0, n, x0.data_ptr(), stream)
  radiance = rc.denoise_buffers[0].view(n, h, w, 4).clone()
  target = None
  if gt_hdr is not None:
    hsum = gt_hdr.contiguous()
    target = torch.zeros((n, h, w, 4), dtype=torch.float32, device=rc.device)
    _lib.call("mjpbr_kpcn_target", ctypes.byref(s), 0, hsum.data_ptr(), ctypes.c_double(1.0), target.data_ptr(), stream)
  scale = torch.zeros((n, h, w, 4), dtype=torch.float32, device=rc.device)
  offset = torch.zeros((n, h, w, 4), dtype=torch.float32, device=rc.device)
  _lib.call("mjpbr_kpcn_remod", ctypes.byref(s), 0, scale.data_ptr(), offset.data_ptr(), stream)
  return x0, radiance, target, (scale, offset), rc


def make_dataset(crops: int, frame_worlds: int, res: int, target_spp: int, spp: tuple[int, ...] = (2,), seed0: int = 100):
  """(x0, radiance, target, scale, offset) of `crops` world images, input sample counts cycling
  through spp frame by frame."""
  parts: list[list[torch.Tensor]] = [[], [], [], [], []]
  nframes = (crops + frame_worlds - 1) // frame_worlds
  for f in range(nframes):
    fr = make_frame(seed0 + f, frame_worlds, res)
    gt = converged_hdr(fr, target_spp)
    x0, rad, tgt, (scale, offset), _ = noisy_pair(fr, spp[f % len(spp)], seed=17 + f, gt_hdr=gt)
    for p, t in zip(parts, (x0, rad, tgt, scale, offset)):
      p.append(t)
  return tuple(torch.cat(p)[:crops] for p in parts)


def train(net: kpcn_lib.KPCN, data, steps: int, batch: int, lr: float, seed: int = 0, warmup: int = 100) -> list[float]:
  """Adam with a linear warm-up and cosine decay of the learning rate; the loss is the relative
  error of the remodulated HDR image (of the demodulated radiance when scale is None)."""
  x0, rad, tgt, scale, offset = data
  n = x0.shape[0]
  g = torch.Generator(device="cpu").manual_seed(seed)
  losses = []
  for step in range(steps):
    idx = torch.randint(0, n, (batch,), generator=g).to(x0.device)
    lr_t = lr * min(1.0, (step + 1) / warmup) * 0.5 * (1.0 + np.cos(np.pi * step / steps))
    remod = (scale[idx].contiguous(), offset[idx].contiguous()) if scale is not None else (None, None)
    sums = net.train_step(x0[idx].contiguous(), rad[idx].contiguous(), tgt[idx].contiguous(), lr_t, *remod)
    if step % 50 == 0 or step == steps - 1:
      losses.append(float(sums.sum().item()))
  return losses


def rel_mse(x: torch.Tensor, ref: torch.Tensor) -> float:
  x, ref = x.double(), ref.double()
  return float(((x - ref) ** 2 / (ref * ref + 1.0e-2)).mean().item())


def timed(fn, reps: int = 3) -> float:
  fn()
  torch.cuda.synchronize()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record()
  for _ in range(reps):
    fn()
  e1.record()
  torch.cuda.synchronize()
  return e0.elapsed_time(e1) / reps


def evaluate(net: kpcn_lib.KPCN, nworld: int, res: int, ref_spp: int, seed: int = 9000, time_worlds: int | None = None) -> dict:
  """relMSE against ref_spp references and Mpix/s of the pipelines on a held-out frame of nworld
  worlds; with time_worlds, the Mpix/s are measured on a second frame of that many worlds (the
  same scene seed), so that the quality reference and the throughput batch can differ in size."""
  out = quality_and_speed(net, nworld, res, ref_spp, seed)
  if time_worlds and time_worlds != nworld:
    speed = quality_and_speed(net, time_worlds, res, 0, seed)
    for k, v in speed.items():
      if isinstance(v, dict) and "ms" in v:
        out[k]["ms"], out[k]["mpix_s"] = v["ms"], v["mpix_s"]
    out["time_worlds"] = time_worlds
    out["speedup_learned2_vs_atrous16"] = out["atrous_16spp"]["ms"] / out["learned_2spp"]["ms"]
  return out


def quality_and_speed(net: kpcn_lib.KPCN, nworld: int, res: int, ref_spp: int, seed: int) -> dict:
  """relMSE against ref_spp references (none when ref_spp is 0) and Mpix/s of the pipelines."""
  fr = make_frame(seed, nworld, res)
  ref = converged_hdr(fr, ref_spp).float() if ref_spp > 0 else None
  npix = nworld * res * res
  out = {"ref_spp": ref_spp, "nworld": nworld, "res": res}
  # learned denoiser at 2 spp
  rc2 = fr.context(path_samples=2, denoise=True, render_hdr=True)
  mjpbr.refit_bvh(fr.m, fr.d, rc2)

  def learned():
    mjpbr.render(fr.m, fr.d, rc2, seed=5, denoise=False)
    net.denoise(fr.m, fr.d, rc2)

  ms = timed(learned)
  out["learned_2spp"] = {"rel_mse": rel_mse(rc2.hdr_data, ref) if ref is not None else None, "ms": ms, "mpix_s": npix / ms / 1e3}
  # a-trous at 16 spp, 5 iterations
  rc16 = fr.context(path_samples=16, denoise=True, denoise_iterations=5, render_hdr=True)
  mjpbr.refit_bvh(fr.m, fr.d, rc16)
  ms = timed(lambda: mjpbr.render(fr.m, fr.d, rc16, seed=5))
  out["atrous_16spp"] = {"rel_mse": rel_mse(rc16.hdr_data, ref) if ref is not None else None, "ms": ms, "mpix_s": npix / ms / 1e3}
  # a-trous at 2 spp and plain 16 / 2 spp for context
  rca = fr.context(path_samples=2, denoise=True, denoise_iterations=5, render_hdr=True)
  mjpbr.refit_bvh(fr.m, fr.d, rca)
  ms = timed(lambda: mjpbr.render(fr.m, fr.d, rca, seed=5))
  out["atrous_2spp"] = {"rel_mse": rel_mse(rca.hdr_data, ref) if ref is not None else None, "ms": ms, "mpix_s": npix / ms / 1e3}
  for spp in (2, 16):
    rcp = fr.context(path_samples=spp, render_hdr=True)
    mjpbr.refit_bvh(fr.m, fr.d, rcp)
    ms = timed(lambda rcp=rcp: mjpbr.render(fr.m, fr.d, rcp, seed=5))
    out[f"plain_{spp}spp"] = {"rel_mse": rel_mse(rcp.hdr_data, ref) if ref is not None else None, "ms": ms, "mpix_s": npix / ms / 1e3}
  out["speedup_learned2_vs_atrous16"] = out["atrous_16spp"]["ms"] / out["learned_2spp"]["ms"]
  return out


def main() -> None:
  p = argparse.ArgumentParser()
  p.add_argument("--out", default="kpcn_weights.npz")
  p.add_argument("--crops", type=int, default=6144)
  p.add_argument("--frame-worlds", type=int, default=256)
  p.add_argument("--res", type=int, default=128)
  p.add_argument("--target-spp", type=int, default=1024)
  p.add_argument("--steps", type=int, default=8000)
  p.add_argument("--batch", type=int, default=16)
  p.add_argument("--lr", type=float, default=1e-3)
  p.add_argument("--eval-worlds", type=int, default=64)
  p.add_argument("--eval-ref-spp", type=int, default=4096)
  p.add_argument("--init", default=None, help="weights to start from")
  p.add_argument("--spp", default="2", help="input sample counts, comma separated, cycled per frame")
  p.add_argument("--loss-space", choices=["demod", "hdr"], default="demod", help="relative losses on the demodulated radiance or the remodulated HDR")
  args = p.parse_args()
  t0 = time.time()
  data = make_dataset(args.crops, args.frame_worlds, args.res, args.target_spp, tuple(int(v) for v in args.spp.split(",")))
  torch.cuda.synchronize()
  t_data = time.time() - t0
  net = kpcn_lib.KPCN.load(args.init) if args.init else kpcn_lib.KPCN("cuda", seed=0)
  t1 = time.time()
  if args.loss_space == "demod":
    data = data[:3] + (None, None)
  losses = train(net, data, args.steps, args.batch, args.lr)
  torch.cuda.synchronize()
  t_train = time.time() - t1
  assert int(net.error.item()) == 0
  net.save(args.out)
  del data
  ev = evaluate(net, args.eval_worlds, args.res, args.eval_ref_spp)
  print(json.dumps({"data_s": t_data, "train_s": t_train, "steps": args.steps, "batch": args.batch, "crops": args.crops, "target_spp": args.target_spp, "spp": args.spp, "loss_space": args.loss_space, "losses": losses, "eval": ev}))


if __name__ == "__main__":
  main()
