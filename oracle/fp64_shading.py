"""FP64 re-evaluation of the real-time tier's shading at sampled pixels — TEST INFRASTRUCTURE ONLY.

The renderers compute in FP32. This module re-evaluates a pixel's radiance in float64 NumPy from
the scene description alone: the pixel-centre camera ray, the closest primitive hit, the Filament
BRDF with multiscatter compensation under the scene's lights, hard shadows and the ambient term,
following mujoco_warp_pbr/_src/render.py:67-239 (shadows, shade_surface), _src/brdf.py:32-110,
_src/lights.py:151-198 and _src/ibl.py:117-119 (the DFG table lookup). The result is compared with
an FP32 renderer's linear HDR output to state the shading error at those pixels.

Scope (enough for the primitive workloads): pinhole cameras, one sample per pixel, plane / sphere /
box / capsule geoms, directional / point / spot lights with hard shadows, the ambient term and the
headlight; no environment map, textures, translucency, mirror or specular anti-aliasing (pass
`samples_per_pixel=1, shadow_samples=1, specular_aa=False` to the context). The DFG table is an
input (the renderer's own FP32 table, bilinearly interpolated in float64).

Only tests/ use this module.
"""

from __future__ import annotations

from typing import Any

import numpy as np

from oracle import host_prep

GEOM_PLANE, GEOM_SPHERE, GEOM_CAPSULE, GEOM_BOX = 0, 2, 3, 6
LIGHT_SPOT, LIGHT_DIRECTIONAL = 0, 1
RAY_OFFSET, SHADOW_GAP, UNBOUNDED = 1.0e-4, 1.0e-3, 1.0e8


def _unit(v: np.ndarray) -> np.ndarray:
  return v / np.linalg.norm(v)


def _hit_local(gtype: int, size: np.ndarray, lo: np.ndarray, ld: np.ndarray) -> tuple[float, np.ndarray] | None:
  """(distance, local normal) of the nearest hit in front of the origin, or None."""
  hits: list[tuple[float, np.ndarray]] = []
  if gtype == GEOM_PLANE:  # one-sided, +z up, bounded when a size is positive
    if ld[2] >= 0.0:
      return None
    t = -lo[2] / ld[2]
    p = lo + t * ld
    if t >= 0.0 and (size[0] <= 0 or abs(p[0]) <= size[0]) and (size[1] <= 0 or abs(p[1]) <= size[1]):
      return t, np.array([0.0, 0.0, 1.0])
    return None
  if gtype == GEOM_SPHERE:
    return _sphere(lo, ld, np.zeros(3), size[0])
  if gtype == GEOM_CAPSULE:
    r, h = size[0], size[1]
    a = ld[0] ** 2 + ld[1] ** 2
    if a > 0.0:
      b = lo[0] * ld[0] + lo[1] * ld[1]
      c = lo[0] ** 2 + lo[1] ** 2 - r * r
      disc = b * b - a * c
      if disc >= 0.0:
        for t in ((-b - np.sqrt(disc)) / a, (-b + np.sqrt(disc)) / a):
          p = lo + t * ld
          if t > 0.0 and abs(p[2]) <= h:
            hits.append((t, np.array([p[0], p[1], 0.0]) / r))
    for zc in (h, -h):
      s = _sphere(lo, ld, np.array([0.0, 0.0, zc]), r)
      if s is not None and (lo + s[0] * ld)[2] * np.sign(zc) >= h:
        hits.append(s)
    return min(hits, key=lambda x: x[0]) if hits else None
  if gtype == GEOM_BOX:
    tnear, tfar, axis_n = -np.inf, np.inf, None
    for k in range(3):
      if ld[k] == 0.0:
        if abs(lo[k]) > size[k]:
          return None
        continue
      t1, t2 = (-size[k] - lo[k]) / ld[k], (size[k] - lo[k]) / ld[k]
      if t1 > t2:
        t1, t2 = t2, t1
      if t1 > tnear:
        tnear, axis_n = t1, k
      tfar = min(tfar, t2)
    if tnear > tfar or tnear <= 0.0 or axis_n is None:
      return None
    n = np.zeros(3)
    n[axis_n] = -np.sign(ld[axis_n])
    return tnear, n
  raise NotImplementedError(f"geom type {gtype}")


def _sphere(lo: np.ndarray, ld: np.ndarray, centre: np.ndarray, r: float) -> tuple[float, np.ndarray] | None:
  oc = lo - centre
  b = float(np.dot(oc, ld))
  c = float(np.dot(oc, oc)) - r * r
  disc = b * b - c
  if disc < 0.0:
    return None
  for t in (-b - np.sqrt(disc), -b + np.sqrt(disc)):
    if t > 0.0:
      return t, (oc + t * ld) / r
  return None


def _dfg(lut: np.ndarray, nov: float, pr: float) -> tuple[float, float]:
  n = lut.shape[0]
  fx, fy = nov * n - 0.5, pr * n - 0.5
  x0, y0 = int(np.floor(fx)), int(np.floor(fy))
  tx, ty = fx - x0, fy - y0
  xs = [min(max(x, 0), n - 1) for x in (x0, x0 + 1)]
  ys = [min(max(y, 0), n - 1) for y in (y0, y0 + 1)]
  lut = lut.astype(np.float64)
  a, b = lut[ys[0], xs[0]], lut[ys[0], xs[1]]
  c, d = lut[ys[1], xs[0]], lut[ys[1], xs[1]]
  top, bot = a + (b - a) * tx, c + (d - c) * tx
  r = top + (bot - top) * ty
  return float(r[0]), float(r[1])


class Fp64Scene:
  """A scene prepared for float64 re-evaluation: sc is a synthetic.SyntheticScene (host model,
  per-world data, options and per-world tables); dfg the renderer's DFG table (size, size, 2)."""

  def __init__(self, sc: Any, dfg: np.ndarray, **overrides: Any):
    self.options = {**sc.options, **overrides}
    self.hc = host_prep.prepare(sc.mjm, sc.mjd, sc.nworld, self.options)
    self.mjm, self.mjd, self.nworld = sc.mjm, sc.mjd, sc.nworld
    self.st = self.hc.settings
    if int(self.st["samples_per_axis"]) != 1 or int(self.st["shadow_samples"]) > 1 or self.st["has_env"] or self.st["specular_aa"]:
      raise ValueError("the float64 re-evaluation covers 1 sample per pixel, hard shadows, no environment, no specular AA")
    n = int(round(np.sqrt(np.asarray(dfg).size / 2)))
    self.dfg = np.asarray(dfg, np.float64).reshape(n, n, 2)
    self.t = {k: np.asarray(v) for k, v in self.hc.tables.items()}
    self.rgba = np.asarray(self.mjm.geom_rgba, np.float64)
    for k, v in sc.per_world.items():
      if k == "geom_rgba":
        self.rgba = np.asarray(v, np.float64)
      else:
        self.t[k] = np.asarray(v)

  def _table(self, name: str, w: int) -> np.ndarray:
    a = self.t[name]
    return np.asarray(a[w % a.shape[0]], np.float64)

  def _world(self, name: str, w: int, k: int) -> np.ndarray:
    a = np.asarray(getattr(self.mjd, name), np.float64)
    return a[w].reshape(-1, k) if a.ndim == 3 else a.reshape(-1, k)

  def _geoms(self, w: int) -> list[tuple[int, int, np.ndarray, np.ndarray, np.ndarray]]:
    pos, mat = self._world("geom_xpos", w, 3), self._world("geom_xmat", w, 9)
    rgba = self.rgba[w % self.rgba.shape[0]] if self.rgba.ndim == 3 else self.rgba
    out = []
    for g in np.asarray(self.hc.enabled_geom_ids):
      if rgba[g][3] == 0.0:
        continue
      size = np.asarray(self.mjm.geom_size, np.float64)[g]
      out.append((int(g), int(self.mjm.geom_type[g]), size, pos[g], mat[g].reshape(3, 3)))
    return out

  def _closest(self, geoms, o, d, max_dist=np.inf):
    best = None
    for g, gtype, size, p, R in geoms:
      h = _hit_local(gtype, size, R.T @ (o - p), R.T @ d)
      if h is not None and h[0] < max_dist and (best is None or h[0] < best[1]):
        best = (g, h[0], R @ h[1])
    return best

  def _occluded(self, geoms, o, d, max_dist) -> bool:
    for _, gtype, size, p, R in geoms:
      h = _hit_local(gtype, size, R.T @ (o - p), R.T @ d)
      if h is not None and h[0] < max_dist:
        return True
    return False

  def radiance(self, w: int, cam: int, px: int, py: int) -> tuple[int, np.ndarray] | None:
    """(geom id, linear HDR radiance) of pixel (px, py) of rendering camera cam in world w, or
    None when the pixel-centre ray hits nothing."""
    o = self.hc.outputs
    W, H = o["cam_res"][cam]
    mid = o["cam_id_map"][cam]
    cpos = self._world("cam_xpos", w, 3)[mid]
    cmat = self._world("cam_xmat", w, 9)[mid].reshape(3, 3)
    fovy = float(np.asarray(self.mjm.cam_fovy, np.float64).reshape(-1)[mid])
    half_h = np.tan(np.radians(fovy / 2.0))
    u, v = (px + 0.5) / W, (py + 0.5) / H
    dcam = _unit(np.array([(2.0 * u - 1.0) * half_h * (W / H), (1.0 - 2.0 * v) * half_h, -1.0]))
    d = cmat @ dcam
    geoms = self._geoms(w)
    hit = self._closest(geoms, cpos, d)
    if hit is None:
      return None
    g, dist, n = hit
    point = cpos + dist * d
    n = _unit(n)
    if np.dot(n, d) > 0.0:
      n = -n
    view = -d
    rgba = self.rgba[w % self.rgba.shape[0]] if self.rgba.ndim == 3 else self.rgba
    base = rgba[g][:3]
    metallic = float(self._table("geom_metallic", w)[g])
    rough = float(self._table("geom_roughness", w)[g])
    refl = float(self._table("geom_reflectance", w)[g])
    exposure = float(self._table("exposure", w).reshape(-1)[0])
    ambient = self._table("ambient_radiance", w).reshape(-1)[:3]
    # lobes (brdf.py / ibl.py)
    nov = max(float(np.dot(n, view)), 1.0e-4)
    pr = min(max(rough, 0.045), 1.0)
    alpha = pr * pr
    f0 = base * metallic + 0.16 * refl * refl * (1.0 - metallic)
    dx, dy = _dfg(self.dfg, nov, pr)
    energy = 1.0 + f0 * (1.0 / max(dy, 1.0e-4) - 1.0)
    spec_albedo = (1.0 - f0) * dx + f0 * dy
    diffuse = base * (1.0 - metallic) * (1.0 - spec_albedo)
    spec_ao = min(max((nov + 1.0) ** (2.0 ** (-16.0 * alpha - 1.0)) - 1.0 + 1.0, 0.0), 1.0)
    radiance = ambient * diffuse + ambient * spec_albedo * energy * spec_ao
    lights = self._lights(w)
    if self.st["headlight_active"]:
      lights.append({"type": LIGHT_DIRECTIONAL, "dir": -cmat[:, 2], "diffuse": np.asarray(self.st["headlight_diffuse"], np.float64),
                     "specular": np.asarray(self.st["headlight_specular"], np.float64), "att": np.array([1.0, 0.0, 0.0]),
                     "intensity": float(self.st["headlight_intensity"]) / exposure, "range": 1.0, "castshadow": False, "cutoff": 0.0, "exponent": 0.0})
    for L in lights:
      radiance = radiance + self._shade_light(L, geoms, point, n, view, nov, alpha, f0, energy, diffuse)
    return g, radiance

  def _lights(self, w: int) -> list[dict[str, Any]]:
    m = self.mjm
    xpos, xdir = self._world("light_xpos", w, 3), self._world("light_xdir", w, 3)
    out = []
    for li in range(len(m.light_type)):
      if not int(m.light_active[li]):
        continue
      out.append({
        "type": int(m.light_type[li]), "pos": xpos[li], "dir": xdir[li],
        "diffuse": np.asarray(m.light_diffuse[li], np.float64), "specular": np.asarray(m.light_specular[li], np.float64),
        "att": np.asarray(m.light_attenuation[li], np.float64), "intensity": float(self._table("light_intensity", w)[li]),
        "range": float(self._table("light_range", w)[li]), "castshadow": bool(m.light_castshadow[li]),
        "cutoff": float(m.light_cutoff[li]), "exponent": float(m.light_exponent[li]),
      })
    return out

  def _shade_light(self, L, geoms, point, n, view, nov, alpha, f0, energy, diffuse) -> np.ndarray:
    physical = int(self.st["light_model"]) == host_prep.LIGHT_MODEL_PHYSICAL
    att, dist = 1.0, UNBOUNDED
    if L["type"] == LIGHT_DIRECTIONAL:
      l = -np.asarray(L["dir"], np.float64)
    else:
      to = L["pos"] - point
      dist = float(np.linalg.norm(to))
      l = to / max(dist, 1.0e-9)
      if physical:
        d2, r = dist * dist, max(L["range"], 1.0e-6)
        window = min(max(1.0 - (d2 / (r * r)) ** 2, 0.0), 1.0)
        att = window * window / max(d2, 1.0e-4)
      else:
        a = L["att"]
        att = 1.0 / max(a[0] + a[1] * dist + a[2] * dist * dist, 1.0e-9)
      if L["type"] == LIGHT_SPOT:
        cos_t = float(np.dot(-l, L["dir"]))
        outer = np.radians(L["cutoff"])
        if physical:
          cone = 1.0 / max(np.cos(outer * 0.75) - np.cos(outer), 1.0 / 1024.0)
          sc = min(max((cos_t - np.cos(outer)) * cone, 0.0), 1.0)
          att *= sc * sc
        else:
          att = 0.0 if cos_t < np.cos(outer) else att * max(cos_t, 0.0) ** L["exponent"]
    if physical:
      ds = ss = L["diffuse"] * L["intensity"] * att
    else:
      ds, ss = L["diffuse"] * np.pi * att, L["specular"] * np.pi * att
    nol = float(np.dot(n, l))
    if nol <= 0.0 or (not ds.any() and not ss.any()):
      return np.zeros(3)
    vis = 1.0
    if self.st["use_shadows"] and L["castshadow"]:
      origin = point + n * RAY_OFFSET
      max_dist = UNBOUNDED if L["type"] == LIGHT_DIRECTIONAL else dist - SHADOW_GAP
      if self._occluded(geoms, origin, l, max_dist):
        vis = float(self.st["shadow_light_fraction"])
    h = _unit(l + view)
    noh, loh = max(float(np.dot(n, h)), 0.0), max(float(np.dot(l, h)), 0.0)
    a2 = alpha * alpha
    dggx = a2 / (np.pi * ((noh * a2 - noh) * noh + 1.0) ** 2)
    gv = nol * np.sqrt(nov * nov * (1.0 - a2) + a2)
    gl = nov * np.sqrt(nol * nol * (1.0 - a2) + a2)
    vis_term = 0.5 / (gv + gl)
    fc = (1.0 - loh) ** 5
    fresnel = f0 * (1.0 - fc) + fc
    fr = fresnel * dggx * vis_term * energy
    return (diffuse / np.pi * ds + fr * ss) * nol * vis


def shading_error(fp: Fp64Scene, hdr: np.ndarray, seg: np.ndarray, npix: int = 2000, seed: int = 0) -> dict[str, float]:
  """Relative error of an FP32 renderer's linear HDR (nworld, npixel, 3) against the float64
  re-evaluation at up to npix sampled hit pixels of camera 0: per pixel, the largest channel error
  over the largest reference channel (floored at 1e-3 of the median). Pixels whose float64
  closest hit is another geom than the renderer's (edge and tie pixels) are counted apart."""
  W, H = fp.hc.outputs["cam_res"][0]
  ids = seg[..., 0].reshape(fp.nworld, -1)[:, : W * H]
  cand = np.argwhere(ids >= 0)
  rng = np.random.default_rng(seed)
  pick = cand[rng.permutation(len(cand))[:npix]]
  errs, refs, mismatched = [], [], 0
  rows = []
  for w, p in pick:
    r = fp.radiance(int(w), 0, int(p % W), int(p // W))
    if r is None or r[0] != ids[w, p]:
      mismatched += 1
      continue
    rows.append((np.asarray(hdr[w, p], np.float64), r[1]))
  ref_max = np.array([np.abs(ref).max() for _, ref in rows])
  floor = 1.0e-3 * float(np.median(ref_max)) if len(rows) else 1.0
  for (got, ref), rm in zip(rows, ref_max, strict=True):
    errs.append(float(np.abs(got - ref).max() / max(rm, floor)))
    refs.append(rm)
  e = np.array(errs) if errs else np.zeros(1)
  return {
    "pixels": len(errs),
    "mismatched_hits": mismatched,
    "median": float(np.median(e)),
    "p99": float(np.percentile(e, 99)),
    "p999": float(np.percentile(e, 99.9)),
    "max": float(e.max()),
    "frac_above_1e-3": float(np.mean(e > 1.0e-3)),
  }
