"""Seeded synthetic froxel sequences for the volumetric-fog filter (torch, any device).

The reference's filter input is the inject pass's single-frame Monte-Carlo
estimate of in-scattered light per froxel (`src/inject_density.slang`, rgba16f,
320x180x64).  These sequences stand in for it:

* grid and depth range: the reference's froxel constants (320x180x64, near
  0.1 m, far 120 m, logarithmic slices; `src/main.cpp:108-115`), EMA alpha 0.1
  (`src/main.cpp:143`);
* camera: perspective (vertical FOV 60 deg) and look-at view built the way the
  reference's MathLib builds them (`libs/math/include/math/projection.hpp:38-83`:
  right-handed, clip.w = view depth, depth range [0, 1]), yawing and translating
  per frame;
* injected light: a smooth world-space field (height-falloff density, two
  coloured point emitters) at each froxel centre, times Gamma(k=1) noise per
  froxel and channel (the single-frame estimate's noise); alpha carries the
  density.

Matrices are float64 4x4 in mathematical order (clip = M @ [x, y, z, 1]).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch


@dataclass
class FogSpec:
    width: int = 320
    height: int = 180
    depth: int = 64
    near: float = 0.1
    far: float = 120.0
    fov_y_deg: float = 60.0
    yaw_deg: float = 0.5                      # camera yaw per frame
    translation: tuple = (0.0, 0.0, -0.05)    # camera translation per frame (metres, world)
    alpha: float = 0.1
    seed: int = 0
    frames: int = 60


def fog_config(seed: int = 0, **kw) -> FogSpec:
    """The reference's froxel grid (320x180x64, 0.1-120 m, alpha 0.1), 60 frames of camera yaw + translation."""
    return FogSpec(seed=seed, **kw)


def perspective(fov_y: float, aspect: float, near: float, far: float) -> np.ndarray:
    t = math.tan(fov_y * 0.5)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = far / (near - far)
    m[2, 3] = near * far / (near - far)
    m[3, 2] = -1.0
    return m


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = r, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -r @ eye, -u @ eye, f @ eye
    return m


class FogScene:
    def __init__(self, spec: FogSpec, device="cpu"):
        self.spec = spec
        self.device = torch.device(device)
        rng = np.random.default_rng(spec.seed)
        self.eye0 = np.array([0.0, 1.7, 0.0])
        self.emit_pos = [np.array([rng.uniform(-15, 15), rng.uniform(1, 6), -rng.uniform(10, 60)]) for _ in range(2)]
        self.emit_col = [rng.uniform(2.0, 8.0, size=3) for _ in range(2)]
        self.proj = perspective(math.radians(spec.fov_y_deg), spec.width / spec.height, spec.near, spec.far)

    def camera(self, t: int):
        """(view-projection, eye) of frame t."""
        sp = self.spec
        th = math.radians(sp.yaw_deg * t)
        eye = self.eye0 + np.asarray(sp.translation, dtype=np.float64) * t
        fwd = np.array([-math.sin(th), 0.0, -math.cos(th)])
        return self.proj @ look_at(eye, eye + fwd), eye

    def param_args(self, t: int) -> dict:
        """Arguments of the filter's parameter block for frame t (history valid from frame 1)."""
        vp, eye = self.camera(t)
        pvp, _ = self.camera(t - 1) if t > 0 else (vp, eye)
        sp = self.spec
        return dict(inv_view_projection=np.linalg.inv(vp), prev_view_projection=pvp, camera_pos=eye, alpha=sp.alpha,
                    width=sp.width, height=sp.height, depth=sp.depth, history_valid=int(t > 0), near_plane=sp.near,
                    far_plane=sp.far)

    def _centres(self, t: int) -> torch.Tensor:
        """World positions (d, h, w, 3) of the froxel centres of frame t (float32)."""
        sp = self.spec
        vp, eye = self.camera(t)
        inv = np.linalg.inv(vp)
        dev = self.device
        xs = (torch.arange(sp.width, device=dev, dtype=torch.float64) + 0.5) / sp.width * 2 - 1
        ys = 1 - (torch.arange(sp.height, device=dev, dtype=torch.float64) + 0.5) / sp.height * 2
        ndc = torch.stack(torch.broadcast_tensors(xs[None, :], ys[:, None]), -1)
        pts = torch.cat([ndc, torch.zeros_like(ndc[..., :1]), torch.ones_like(ndc[..., :1])], -1)
        w = pts @ torch.tensor(inv.T, device=dev)
        near_w = w[..., :3] / w[..., 3:]
        e = torch.tensor(eye, device=dev)
        ray = near_w - e
        ray = ray / ray.norm(dim=-1, keepdim=True)
        fh = inv @ np.array([0.0, 0.0, 0.0, 1.0])
        fwd = torch.tensor(fh[:3] / fh[3] - eye, device=dev)
        fwd = fwd / fwd.norm()
        rdf = (ray * fwd).sum(-1).clamp_min(1e-4)
        zs = sp.near * (sp.far / sp.near) ** ((torch.arange(sp.depth, device=dev, dtype=torch.float64) + 0.5) / sp.depth)
        tt = zs[:, None, None] / rdf[None]
        return (e + ray[None] * tt[..., None]).to(torch.float32)

    def inject(self, t: int, dtype=torch.float16) -> torch.Tensor:
        """Noisy injected light (d, h, w, 4) of frame t: rgb in-scatter, a density."""
        p = self._centres(t)
        dens = 0.02 * torch.exp(-torch.clamp(p[..., 1], min=0.0) / 8.0)
        light = torch.full_like(p, 0.05)
        for pos, col in zip(self.emit_pos, self.emit_col):
            d2 = ((p - torch.tensor(pos, device=p.device, dtype=p.dtype)) ** 2).sum(-1, keepdim=True)
            light = light + torch.tensor(col, device=p.device, dtype=p.dtype) / (1.0 + d2)
        g = torch.Generator(device="cpu").manual_seed(self.spec.seed * 1000003 + t)
        noise = torch.empty(p.shape, dtype=torch.float32).exponential_(1.0, generator=g).to(p.device)
        rgb = dens[..., None] * light * noise
        return torch.cat([rgb, dens[..., None]], -1).to(dtype).contiguous()
