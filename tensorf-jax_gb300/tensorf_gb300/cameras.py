"""GB300 twin of ``tensorf/cameras.py``: ``Rays3D`` and a pinhole ``Camera`` whose
per-pixel rays are generated on the device (the reference builds them on the host CPU,
cameras.py:123-124)."""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Optional

import numpy as onp
import torch

from . import _lib
from ._util import ptr, stream_handle


@dataclasses.dataclass
class Rays3D:
    """cameras.py:10-20. origins / directions (*, 3) float32; camera_indices (*,) int32,
    read by models with FiLM camera embeddings (networks.py:103-111)."""
    origins: torch.Tensor
    directions: torch.Tensor
    camera_indices: Optional[torch.Tensor] = None

    def get_batch_axes(self):
        return tuple(self.origins.shape[:-1])


@dataclasses.dataclass
class Camera:
    """Intrinsics K (3, 3) and the camera-to-world pose (rotation R_wc, position t_wc);
    the reference stores T_camera_world as a jaxlie.SE3 (cameras.py:23-32)."""
    K: onp.ndarray
    R_world_camera: onp.ndarray
    t_world_camera: onp.ndarray
    image_width: int
    image_height: int

    @staticmethod
    def from_fov(R_world_camera, t_world_camera, image_width: int, image_height: int,
                 fov_x_radians: Optional[float] = None, fov_y_radians: Optional[float] = None) -> "Camera":
        """cameras.py:34-76."""
        cx = image_width / 2.0 - 0.5
        cy = image_height / 2.0 - 0.5
        fx = (image_width / 2.0) / math.tan(fov_x_radians / 2.0) if fov_x_radians is not None else None
        fy = (image_height / 2.0) / math.tan(fov_y_radians / 2.0) if fov_y_radians is not None else None
        fx = fy if fx is None else fx
        fy = fx if fy is None else fy
        K = onp.array([[fx, 0.0, cx], [0.0, fy, cy], [0.0, 0.0, 1.0]])
        return Camera(K, onp.asarray(R_world_camera, dtype=onp.float64),
                      onp.asarray(t_world_camera, dtype=onp.float64), image_width, image_height)

    @staticmethod
    def from_focal(R_world_camera, t_world_camera, image_width: int, image_height: int, focal: float) -> "Camera":
        fov_x = 2.0 * math.atan((image_width / 2.0) / focal)
        return Camera.from_fov(R_world_camera, t_world_camera, image_width, image_height, fov_x_radians=fov_x)

    def pixel_rays_wrt_world(self, pixels: Optional[torch.Tensor] = None) -> Rays3D:
        """cameras.py:100-143: rays of every pixel (H*W, row-major) or of the given
        flat pixel indices, built on the device."""
        n = self.image_width * self.image_height if pixels is None else pixels.numel()
        o = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        d = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        K = (ctypes.c_double * 9)(*onp.asarray(self.K, dtype=onp.float64).ravel())
        R = (ctypes.c_double * 9)(*onp.asarray(self.R_world_camera, dtype=onp.float64).ravel())
        t = (ctypes.c_double * 3)(*onp.asarray(self.t_world_camera, dtype=onp.float64).ravel())
        px = None if pixels is None else pixels.to(device="cuda", dtype=torch.int64).contiguous()
        _lib.call("tvm_camera_rays", K, R, t, self.image_width, self.image_height, ptr(px), n, ptr(o), ptr(d),
                  stream_handle())
        return Rays3D(origins=o, directions=d)


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0)):
    """Rotation R_wc (OpenCV convention: +z forward, +y down) of a camera at ``eye``
    looking at ``target``."""
    eye = onp.asarray(eye, dtype=onp.float64)
    fwd = onp.asarray(target, dtype=onp.float64) - eye
    fwd /= onp.linalg.norm(fwd)
    right = onp.cross(fwd, onp.asarray(up, dtype=onp.float64))
    if onp.linalg.norm(right) < 1e-9:
        right = onp.cross(fwd, onp.array([0.0, 1.0, 0.0]))
    right /= onp.linalg.norm(right)
    down = onp.cross(fwd, right)
    return onp.stack([right, down, fwd], axis=1), eye
