"""Seeded synthetic workloads.

* ``sphere_rays`` -- rays whose origins are uniform on a sphere of radius 4, aimed at
  the origin with N(0, 0.05^2) jitter on the direction, and uniform [0, 1) targets (the
  CPU-runnable 4096-ray workload).
* ``SphereScene`` -- an analytic scene of constant-density spheres (radius U[0.1, 0.4],
  density 50, colour U[0, 1]) seen by seeded 800x800 pinhole cameras with focal length
  1111 on a sphere of radius 4 around the origin. Target colours come from an FP64
  quadrature (4096 midpoint samples per ray over the aabb segment) on the device. It
  stands in for the Blender lego scene, which is not available here.
* ``unbounded_rays`` -- origins within radius 1, directions uniform on the sphere.
* ``SphereScene.unbounded`` -- spheres at distances 2..12 from the origin in every
  direction, radius proportional to distance, seen from inside by ``unbounded_rays``:
  the unbounded-scene workload (scene contraction to [-2, 2]^3).
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import List, Tuple

import numpy as onp
import torch

from . import _lib, cameras
from ._util import ptr, stream_handle


def sphere_rays(n: int, seed: int, radius: float = 4.0, jitter: float = 0.05):
    rng = onp.random.default_rng(seed)
    o = rng.normal(size=(n, 3))
    o = o / onp.linalg.norm(o, axis=1, keepdims=True) * radius
    d = -o + rng.normal(scale=jitter, size=(n, 3))
    d = d / onp.linalg.norm(d, axis=1, keepdims=True)
    colors = rng.uniform(size=(n, 3))
    return o.astype(onp.float32), d.astype(onp.float32), colors.astype(onp.float32)


def unbounded_rays(n: int, seed: int):
    rng = onp.random.default_rng(seed)
    v = rng.normal(size=(n, 3))
    v /= onp.linalg.norm(v, axis=1, keepdims=True)
    o = v * rng.uniform(size=(n, 1)) ** (1.0 / 3.0)
    d = rng.normal(size=(n, 3))
    d /= onp.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(onp.float32), d.astype(onp.float32)


@dataclasses.dataclass
class SphereScene:
    centers: onp.ndarray  # (S, 3) float64
    radii: onp.ndarray    # (S,)
    colors: onp.ndarray   # (S, 3)
    density: float = 50.0
    aabb: Tuple[Tuple[float, ...], Tuple[float, ...]] = ((-1.5, -1.5, -1.5), (1.5, 1.5, 1.5))

    @staticmethod
    def random(seed: int, count: int = 32, extent: float = 1.0) -> "SphereScene":
        rng = onp.random.default_rng(seed)
        return SphereScene(centers=rng.uniform(-extent, extent, size=(count, 3)),
                           radii=rng.uniform(0.1, 0.4, size=count),
                           colors=rng.uniform(0.0, 1.0, size=(count, 3)))

    @staticmethod
    def unbounded(seed: int, count: int = 128) -> "SphereScene":
        """Spheres around the origin at distances U[2, 12], radius U[0.1, 0.25] times the
        distance, so that rays starting within radius 1 see content in every direction
        and most of it beyond the contraction radius."""
        rng = onp.random.default_rng(seed)
        v = rng.normal(size=(count, 3))
        v /= onp.linalg.norm(v, axis=1, keepdims=True)
        dist = rng.uniform(2.0, 12.0, size=count)
        return SphereScene(centers=v * dist[:, None], radii=rng.uniform(0.1, 0.25, size=count) * dist,
                           colors=rng.uniform(0.0, 1.0, size=(count, 3)),
                           aabb=((-16.0, -16.0, -16.0), (16.0, 16.0, 16.0)))

    def unbounded_training_rays(self, total: int, seed: int, n_samples: int = 8192):
        """``total`` rays from inside radius 1 in uniform directions with their FP64 target
        colours."""
        o, d = unbounded_rays(total, seed)
        rays = cameras.Rays3D(origins=torch.as_tensor(o, device="cuda"), directions=torch.as_tensor(d, device="cuda"))
        return rays, self.render(rays, n_samples)

    def cameras(self, count: int, seed: int, width: int = 800, height: int = 800, focal: float = 1111.0,
                radius: float = 4.0) -> List[cameras.Camera]:
        rng = onp.random.default_rng(seed)
        cams = []
        for _ in range(count):
            v = rng.normal(size=3)
            v /= onp.linalg.norm(v)
            R, eye = cameras.look_at(v * radius)
            cams.append(cameras.Camera.from_focal(R, eye, width, height, focal))
        return cams

    def render(self, rays: cameras.Rays3D, n_samples: int = 4096) -> torch.Tensor:
        """FP64 quadrature of the scene along each ray (tvm_sphere_scene_render)."""
        dev = "cuda"
        c = torch.as_tensor(self.centers, dtype=torch.float64, device=dev).contiguous()
        r = torch.as_tensor(self.radii, dtype=torch.float64, device=dev).contiguous()
        col = torch.as_tensor(self.colors, dtype=torch.float64, device=dev).contiguous()
        aabb = torch.tensor(list(self.aabb[0]) + list(self.aabb[1]), dtype=torch.float32, device=dev)
        o = rays.origins.reshape(-1, 3).contiguous()
        d = rays.directions.reshape(-1, 3).contiguous()
        out = torch.empty((o.shape[0], 3), dtype=torch.float32, device=dev)
        rs = _lib.Rays(count=o.shape[0], origins=ptr(o), directions=ptr(d))
        _lib.call("tvm_sphere_scene_render", ptr(c), ptr(r), ptr(col), len(self.radii), float(self.density),
                  ptr(aabb), ctypes.byref(rs), n_samples, ptr(out), stream_handle())
        return out

    def median_depth(self, origins: onp.ndarray, directions: onp.ndarray) -> onp.ndarray:
        """Exact median depth of each ray in FP64: the distance t at which the optical
        depth from the ray origin reaches ln 2 (transmittance 1/2), from the ray-sphere
        intersections (overlapping spheres add their densities), clipped to the aabb
        segment; +inf where the ray keeps more than half its transmittance. This is
        the analytic counterpart of RenderMode.DIST_MEDIAN, whose rendered value is
        quantised to the sample grid."""
        o = onp.asarray(origins, dtype=onp.float64)
        d = onp.asarray(directions, dtype=onp.float64)
        d = d / onp.linalg.norm(d, axis=1, keepdims=True)
        lo_b, hi_b = onp.asarray(self.aabb[0]), onp.asarray(self.aabb[1])
        with onp.errstate(divide="ignore", invalid="ignore"):
            t1, t2 = (lo_b - o) / d, (hi_b - o) / d
        t_near = onp.maximum(onp.nanmax(onp.minimum(t1, t2), axis=1), 0.0)
        t_far = onp.nanmin(onp.maximum(t1, t2), axis=1)
        oc = o[:, None, :] - self.centers[None, :, :]  # (n, S, 3)
        b = onp.einsum("nsk,nk->ns", oc, d)
        disc = b * b - (onp.einsum("nsk,nsk->ns", oc, oc) - self.radii[None, :] ** 2)
        hit = disc > 0
        root = onp.sqrt(onp.where(hit, disc, 0.0))
        enter = onp.clip(onp.where(hit, -b - root, onp.inf), t_near[:, None], t_far[:, None])
        leave = onp.clip(onp.where(hit, -b + root, onp.inf), t_near[:, None], t_far[:, None])
        S = self.radii.shape[0]
        t_ev = onp.concatenate([enter, leave], axis=1)
        step = onp.concatenate([onp.ones((o.shape[0], S)), -onp.ones((o.shape[0], S))], axis=1)
        step[~onp.isfinite(t_ev)] = 0.0
        t_ev = onp.where(onp.isfinite(t_ev), t_ev, onp.inf)
        order = onp.argsort(t_ev, axis=1, kind="stable")
        t_ev = onp.take_along_axis(t_ev, order, axis=1)
        count = onp.cumsum(onp.take_along_axis(step, order, axis=1), axis=1)  # spheres covering [t_k, t_k+1)
        seg = onp.diff(t_ev, axis=1)
        seg = onp.where(onp.isfinite(seg), seg, 0.0)
        sig = self.density * count[:, :-1]
        tau = onp.concatenate([onp.zeros((o.shape[0], 1)), onp.cumsum(sig * seg, axis=1)], axis=1)
        target = onp.log(2.0)
        reached = tau >= target
        out = onp.full(o.shape[0], onp.inf)
        rows = onp.nonzero(reached.any(axis=1))[0]
        k = onp.argmax(reached[rows], axis=1)  # first event with tau >= ln 2; tau[:, 0] = 0
        out[rows] = t_ev[rows, k - 1] + (target - tau[rows, k - 1]) / sig[rows, k - 1]
        return out

    @staticmethod
    def training_pixels(cams: List[cameras.Camera], total: int, seed: int) -> Tuple[onp.ndarray, onp.ndarray]:
        """The (camera index, flat pixel index) of each of ``total`` training rays, in
        batch order: an equal share of random pixels per camera, then shuffled. Host
        only, so a CPU run can rebuild the same rays."""
        rng = onp.random.default_rng(seed)
        per = [total // len(cams) + (1 if i < total % len(cams) else 0) for i in range(len(cams))]
        cam_idx, pix = [], []
        for i, (cam, n) in enumerate(zip(cams, per)):
            if n == 0:
                continue
            pix.append(rng.integers(0, cam.image_width * cam.image_height, size=n))
            cam_idx.append(onp.full(n, i))
        perm = rng.permutation(total)
        return onp.concatenate(cam_idx)[perm], onp.concatenate(pix)[perm]

    def training_rays(self, cams: List[cameras.Camera], total: int, seed: int,
                      n_samples: int = 4096) -> Tuple[cameras.Rays3D, torch.Tensor]:
        """``total`` random pixels over the cameras with their FP64 target colours."""
        cam_idx, pix = self.training_pixels(cams, total, seed)
        order = onp.argsort(cam_idx, kind="stable")  # batch positions grouped by camera
        bounds = onp.searchsorted(cam_idx[order], onp.arange(len(cams) + 1))
        os_, ds_ = [], []
        for i, cam in enumerate(cams):
            sel = order[bounds[i]:bounds[i + 1]]
            if sel.size:
                rr = cam.pixel_rays_wrt_world(torch.as_tensor(pix[sel], dtype=torch.int64))
                os_.append(rr.origins)
                ds_.append(rr.directions)
        at = torch.as_tensor(order, device="cuda")
        o = torch.empty((total, 3), dtype=torch.float32, device="cuda")
        d = torch.empty((total, 3), dtype=torch.float32, device="cuda")
        o[at] = torch.cat(os_)
        d[at] = torch.cat(ds_)
        rays = cameras.Rays3D(origins=o, directions=d)
        return rays, self.render(rays, n_samples)
