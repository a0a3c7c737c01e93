"""Seeded synthetic frame sequences for the SVGF denoiser (torch, any device).

There is no dataset for this path: the reference's SVGF input is the engine's
ray-traced combined lighting (src/mesh.slang:995-998).  These sequences stand
in for it:

* geometry: 6 random infinite planes, unit normals uniform on the hemisphere
  facing the camera, offsets U[1, 50] m, nearest hit wins; a backdrop plane at
  200 m catches rays that hit nothing; optionally a finite plane that appears
  at a given frame (a forced disocclusion);
* depth: linear view-space depth; normal: the plane's world-space normal;
* ground-truth radiance: albedo U[0.05, 0.9]^3 x (smooth cosine term from a
  point light + two stripe emitters of value U[4, 20] per plane);
* noisy 1-spp radiance: truth x Gamma(k=1, theta=1) (= Exp(1)) iid per pixel
  and channel;
* camera: yaw per frame about world up, plus a per-frame translation; motion
  vectors are the exact reprojection of each pixel's hit point into the
  previous frame's camera, in pixels (previous position minus current centre).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch


@dataclass
class SceneSpec:
    width: int
    height: int
    seed: int = 0
    yaw_deg: float = 0.2                     # camera yaw per frame
    translation: tuple = (0.0, 0.0, 0.0)     # camera translation per frame (metres, world)
    appear_frame: int | None = None          # frame from which an extra finite plane exists
    n_planes: int = 6
    fov_y_deg: float = 60.0
    frames: int = 8
    extra: dict = field(default_factory=dict)  # {"no_emitters": True} drops the stripe emitters


def slow_pan(seed: int = 0) -> SceneSpec:
    """640x360, 8 frames, camera yaw 0.2 deg/frame."""
    return SceneSpec(640, 360, seed=seed, yaw_deg=0.2, frames=8)


def pan_with_disocclusion(width: int = 3840, height: int = 2160, seed: int = 0) -> SceneSpec:
    """60 frames, yaw 0.5 deg/frame + 0.05 m/frame translation, a plane appears at frame 30."""
    s = 0.05 / math.sqrt(2.0)
    return SceneSpec(width, height, seed=seed, yaw_deg=0.5, translation=(s, 0.0, s), appear_frame=30, frames=60)


def stream_specs(n: int, resolutions, weights=None, seed: int = 0, frames: int = 30) -> list[SceneSpec]:
    """n independent camera streams with seeded resolutions and camera paths."""
    rng = np.random.default_rng(seed)
    res = list(resolutions)
    idx = rng.choice(len(res), size=n, p=weights)
    out = []
    for k in range(n):
        w, h = res[int(idx[k])]
        yaw = float(rng.uniform(-0.6, 0.6))
        ang = float(rng.uniform(0, 2 * math.pi))
        sp = float(rng.uniform(0.0, 0.05))
        out.append(SceneSpec(int(w), int(h), seed=int(seed * 100003 + k * 7919 + 1), yaw_deg=yaw,
                             translation=(sp * math.cos(ang), 0.0, sp * math.sin(ang)), frames=frames))
    return out


def _tangents(n):
    up = np.array([0.0, 1.0, 0.0]) if abs(n[1]) < 0.95 else np.array([1.0, 0.0, 0.0])
    a1 = np.cross(n, up)
    a1 /= np.linalg.norm(a1)
    a2 = np.cross(n, a1)
    return a1, a2


class PlaneScene:
    def __init__(self, spec: SceneSpec, device="cpu"):
        self.spec = spec
        self.device = torch.device(device)
        rng = np.random.default_rng(spec.seed)
        planes = []
        for _ in range(spec.n_planes):
            v = rng.normal(size=3)
            v /= np.linalg.norm(v)
            if v[2] > 0:  # face the initial camera, which looks along +z
                v = -v
            planes.append(self._plane(rng, v, float(rng.uniform(1.0, 50.0))))
        planes.append(self._plane(rng, np.array([0.0, 0.0, -1.0]), 200.0))
        self.planes = planes
        self.rect = None
        if spec.appear_frame is not None:
            c, f, r, u = self.camera(spec.appear_frame)
            centre = c + 4.0 * f + 0.4 * r - 0.2 * u
            p = self._plane(rng, -f, float(-np.dot(-f, centre)))
            p["albedo"] = np.array([0.8, 0.35, 0.2])
            p["rect"] = (centre, r, u, 1.2, 0.8)
            self.rect = p
        self.light = np.array([0.0, 4.0, 6.0])

    @staticmethod
    def _plane(rng, n, offset):
        a1, a2 = _tangents(n)
        stripes = []
        for _ in range(2):
            stripes.append(dict(axis=int(rng.integers(0, 2)), period=float(rng.uniform(1.5, 6.0)),
                                phase=float(rng.uniform(0.0, 1.0)), duty=float(rng.uniform(0.04, 0.12)),
                                emission=float(rng.uniform(4.0, 20.0))))
        return dict(n=np.asarray(n, float), offset=offset, albedo=rng.uniform(0.05, 0.9, size=3), a1=a1, a2=a2,
                    stripes=stripes, rect=None)

    def camera(self, t: int):
        th = math.radians(self.spec.yaw_deg * t)
        f = np.array([math.sin(th), 0.0, math.cos(th)])
        r = np.array([math.cos(th), 0.0, -math.sin(th)])
        u = np.array([0.0, 1.0, 0.0])
        c = np.asarray(self.spec.translation, float) * t
        return c, f, r, u

    def _rays(self, t):
        W, H = self.spec.width, self.spec.height
        th = math.tan(math.radians(self.spec.fov_y_deg) / 2)
        asp = W / H
        dev = self.device
        xs = (torch.arange(W, device=dev, dtype=torch.float32) + 0.5) / W * 2 - 1
        ys = 1 - (torch.arange(H, device=dev, dtype=torch.float32) + 0.5) / H * 2
        sx = (xs * th * asp)[None, :, None]
        sy = (ys * th)[:, None, None]
        c, f, r, u = self.camera(t)
        T = lambda v: torch.tensor(v, dtype=torch.float32, device=dev)
        d = T(f)[None, None, :] + sx * T(r)[None, None, :] + sy * T(u)[None, None, :]
        return T(c), d

    def frame(self, t: int, noise: bool = True) -> dict:
        """Inputs of frame t: radiance, truth, depth, normal, motion, plane id."""
        W, H = self.spec.width, self.spec.height
        dev = self.device
        T = lambda v: torch.tensor(np.asarray(v, float), dtype=torch.float32, device=dev)
        c, d = self._rays(t)
        planes = list(self.planes)
        if self.rect is not None and t >= self.spec.appear_frame:
            planes.append(self.rect)
        best = torch.full((H, W), float("inf"), device=dev)
        pid = torch.full((H, W), -1, dtype=torch.int64, device=dev)
        for k, p in enumerate(planes):
            n = T(p["n"])
            nd = (d * n).sum(-1)
            num = -p["offset"] - float(torch.dot(n, c))
            tt = torch.where(nd.abs() > 1e-8, num / torch.where(nd.abs() > 1e-8, nd, torch.ones_like(nd)),
                             torch.full_like(nd, float("inf")))
            ok = tt > 1e-3
            if p["rect"] is not None:
                centre, ra, ua, hw, hh = p["rect"]
                P = c + tt[..., None] * d
                rel = P - T(centre)
                ok = ok & ((rel * T(ra)).sum(-1).abs() <= hw) & ((rel * T(ua)).sum(-1).abs() <= hh)
            tt = torch.where(ok, tt, torch.full_like(tt, float("inf")))
            better = tt < best
            best = torch.where(better, tt, best)
            pid = torch.where(better, torch.full_like(pid, k), pid)
        depth = best
        P = c + depth[..., None] * d
        normal = torch.zeros((H, W, 3), device=dev)
        albedo = torch.zeros((H, W, 3), device=dev)
        emis = torch.zeros((H, W), device=dev)
        for k, p in enumerate(planes):
            m = (pid == k)[..., None]
            normal = torch.where(m, T(p["n"]).expand(H, W, 3), normal)
            albedo = torch.where(m, T(p["albedo"]).expand(H, W, 3), albedo)
            e = torch.zeros((H, W), device=dev)
            for s in ([] if self.spec.extra.get("no_emitters") else p["stripes"]):
                ax = T(p["a1"] if s["axis"] == 0 else p["a2"])
                uu = (P * ax).sum(-1) / s["period"] + s["phase"]
                e = e + s["emission"] * ((uu - torch.floor(uu)) < s["duty"]).float()
            emis = torch.where(m[..., 0], e, emis)
        ldir = T(self.light) - P
        ldir = ldir / ldir.norm(dim=-1, keepdim=True).clamp_min(1e-6)
        shade = 0.1 + 0.9 * (normal * ldir).sum(-1).clamp_min(0.0)
        truth_rgb = albedo * (shade + emis)[..., None]
        truth = torch.cat([truth_rgb, torch.ones((H, W, 1), device=dev)], -1)
        if noise:
            g = torch.Generator(device=dev)
            g.manual_seed(int(self.spec.seed) * 1000003 + int(t) * 7 + 11)
            e = torch.empty((H, W, 3), device=dev).exponential_(1.0, generator=g)
            radiance = torch.cat([truth_rgb * e, torch.ones((H, W, 1), device=dev)], -1)
        else:
            radiance = truth.clone()
        motion = self._motion(t, P)
        return dict(radiance=radiance.contiguous(), truth=truth.contiguous(), depth=depth.contiguous(),
                    normal=normal.contiguous(), motion=motion.contiguous(), plane=pid)

    def _motion(self, t, P):
        W, H = self.spec.width, self.spec.height
        th = math.tan(math.radians(self.spec.fov_y_deg) / 2)
        asp = W / H
        dev = self.device
        T = lambda v: torch.tensor(np.asarray(v, float), dtype=torch.float32, device=dev)
        c, f, r, u = self.camera(t - 1)
        v = P - T(c)
        zp = (v * T(f)).sum(-1)
        safe = torch.where(zp > 1e-3, zp, torch.ones_like(zp))
        sxp = (v * T(r)).sum(-1) / safe
        syp = (v * T(u)).sum(-1) / safe
        xp = (sxp / (th * asp) + 1) * 0.5 * W
        yp = (1 - syp / th) * 0.5 * H
        xc = torch.arange(W, device=dev, dtype=torch.float32)[None, :] + 0.5
        yc = torch.arange(H, device=dev, dtype=torch.float32)[:, None] + 0.5
        mx = torch.where(zp > 1e-3, xp - xc, torch.full_like(xp, -4.0 * W))
        my = torch.where(zp > 1e-3, yp - yc, torch.full_like(yp, -4.0 * H))
        return torch.stack([mx, my], -1)


def to_half(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.float16)


def oct16_encode(n: torch.Tensor) -> torch.Tensor:
    """Octahedral snorm16 encoding (Meyer et al. 2010) of unit normals (..., 3) -> (..., 2) int16."""
    l1 = n.abs().sum(-1, keepdim=True).clamp_min(1e-30)
    p = n[..., :2] / l1
    sgn = torch.where(p >= 0, torch.ones_like(p), -torch.ones_like(p))
    folded = (1 - p.flip(-1).abs()) * sgn
    p = torch.where(n[..., 2:3] < 0, folded, p).clamp(-1, 1)
    return torch.round(p * 32767.0).to(torch.int16)
