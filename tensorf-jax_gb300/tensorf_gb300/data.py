"""GB300 twin of ``tensorf/data.py``: Blender and nerfstudio datasets as flat ray batches.

``make_dataset`` (data.py:32-43) returns a ``BlenderDataset`` (data.py:201-279) or a
``NerfstudioDataset`` (data.py:46-198). ``get_training_rays`` gives a ``RenderedRays``
(data.py:294-303): colors (N, 3) and ``cameras.Rays3D`` with one camera index per ray,
as CUDA tensors, the rays built on the device by ``Camera.pixel_rays_wrt_world`` (Blender)
or from the undistorted pixel directions (nerfstudio).

The reference reads images with PIL and undistorts and resizes with OpenCV. Neither is
a dependency here: images are read through PIL where it is installed, and without it PNG
files are decoded by ``read_png`` (zlib and the five PNG row filters, PNG specification
1.2, section 6); undistortion restates the OpenCV pinhole (Brown-Conrady k1, k2, p1, p2) and
fisheye (Kannala-Brandt k1..k4) models and inverts them iteratively as
``cv2.undistortPoints`` and ``cv2.fisheye.undistortPoints`` do; the resize is bilinear
with half-pixel centres, as ``cv2.resize`` with its default interpolation.
"""
from __future__ import annotations

import dataclasses
import functools
import json
import math
import pathlib
import struct
import zlib
from typing import List, Literal, Tuple, Union

import numpy as onp
import torch

from . import cameras

# Blender camera axes (x right, y up, looking down -z) to the OpenCV convention used by
# cameras.Camera (x right, y down, looking down +z): a half turn about x (data.py:146-150).
_R_BLENDERCAM_CAMERA = onp.diag([1.0, -1.0, -1.0])


# ---------------------------------------------------------------------------------
# Images.
# ---------------------------------------------------------------------------------
_PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"
_PNG_CHANNELS = {0: 1, 2: 3, 4: 2, 6: 4}  # colour type -> samples per pixel


def _unfilter_row(ftype: int, row: bytearray, prev: bytes, bpp: int) -> None:
    """Undo one PNG row filter in place (PNG 1.2 section 6.3). Sub and Up are running sums
    and sums over the row (numpy); Average and Paeth depend on the byte just decoded, one
    byte at a time."""
    n = len(row)
    if ftype == 0:
        return
    if ftype == 1:  # Sub: per channel, a running sum mod 256 along the row
        a = onp.frombuffer(bytes(row), dtype=onp.uint8).reshape(-1, bpp).astype(onp.uint32)
        row[:] = (onp.cumsum(a, axis=0) & 0xFF).astype(onp.uint8).tobytes()
    elif ftype == 2:  # Up
        row[:] = ((onp.frombuffer(bytes(row), dtype=onp.uint8).astype(onp.uint16) +
                   onp.frombuffer(prev, dtype=onp.uint8)) & 0xFF).astype(onp.uint8).tobytes()
    elif ftype == 3:  # Average
        for i in range(n):
            left = row[i - bpp] if i >= bpp else 0
            row[i] = (row[i] + ((left + prev[i]) >> 1)) & 0xFF
    elif ftype == 4:  # Paeth
        for i in range(n):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            row[i] = (row[i] + pred) & 0xFF
    else:
        raise ValueError(f"PNG: unknown row filter {ftype}")


def read_png(path: Union[str, pathlib.Path]) -> onp.ndarray:
    """8-bit, non-interlaced PNG (grey, grey + alpha, RGB or RGBA) -> uint8 (H, W, C)."""
    data = pathlib.Path(path).read_bytes()
    if data[:8] != _PNG_SIGNATURE:
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, header = 8, [], None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if kind == b"IHDR":
            header = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if header is None:
        raise ValueError(f"{path}: PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = header
    if depth != 8 or ctype not in _PNG_CHANNELS or interlace != 0:
        raise ValueError(f"{path}: only 8-bit non-interlaced grey/RGB(A) PNGs are supported "
                         f"(depth {depth}, colour type {ctype}, interlace {interlace})")
    ch = _PNG_CHANNELS[ctype]
    raw = zlib.decompress(b"".join(idat))
    stride = w * ch
    if len(raw) != h * (stride + 1):
        raise ValueError(f"{path}: PNG data size {len(raw)} does not match {h} rows of {stride + 1} bytes")
    out = bytearray(h * stride)
    prev = bytes(stride)
    for y in range(h):
        row = bytearray(raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)])
        _unfilter_row(raw[y * (stride + 1)], row, prev, ch)
        out[y * stride:(y + 1) * stride] = row
        prev = bytes(row)
    return onp.frombuffer(bytes(out), dtype=onp.uint8).reshape(h, w, ch)


def read_image(path: Union[str, pathlib.Path]) -> onp.ndarray:
    """An image file as uint8 (H, W, C), through PIL where it is installed (as the
    reference reads them, data.py:344-354); without PIL, PNG files are decoded here."""
    path = pathlib.Path(path)
    try:
        import PIL.Image
    except ImportError:
        PIL = None
    if PIL is not None:
        return onp.array(PIL.Image.open(path))
    if path.read_bytes()[:8] == _PNG_SIGNATURE:
        return read_png(path)
    raise RuntimeError(f"{path}: only PNG images can be read without PIL")


def resize_bilinear(image: onp.ndarray, width: int, height: int) -> onp.ndarray:
    """Bilinear resize with half-pixel centres and clamped borders (the default
    interpolation of ``cv2.resize``), (H, W, C) -> (height, width, C), same dtype."""
    h, w = image.shape[:2]
    img = image.astype(onp.float64)

    def axis(n_out: int, n_in: int):
        s = (onp.arange(n_out) + 0.5) * (n_in / n_out) - 0.5
        s = onp.clip(s, 0.0, n_in - 1)
        i0 = onp.floor(s).astype(onp.int64)
        i1 = onp.minimum(i0 + 1, n_in - 1)
        return i0, i1, s - i0

    y0, y1, fy = axis(height, h)
    x0, x1, fx = axis(width, w)
    fy, fx = fy[:, None, None], fx[None, :, None]
    top = img[y0][:, x0] * (1 - fx) + img[y0][:, x1] * fx
    bot = img[y1][:, x0] * (1 - fx) + img[y1][:, x1] * fx
    out = top * (1 - fy) + bot * fy
    if onp.issubdtype(image.dtype, onp.integer):
        out = onp.clip(onp.rint(out), onp.iinfo(image.dtype).min, onp.iinfo(image.dtype).max)
    return out.astype(image.dtype)


# ---------------------------------------------------------------------------------
# Undistortion.
# ---------------------------------------------------------------------------------
def undistort_points_opencv(points: onp.ndarray, K: onp.ndarray, dist: onp.ndarray,
                            iterations: int = 5) -> onp.ndarray:
    """Pixel coordinates (n, 2) -> normalised undistorted image coordinates (n, 2) under
    the OpenCV pinhole model with radial k1, k2 and tangential p1, p2: the distorted
    point is x (1 + k1 r^2 + k2 r^4) + [2 p1 x y + p2 (r^2 + 2 x^2), p1 (r^2 + 2 y^2) +
    2 p2 x y]; the fixed-point inversion x <- (x_d - tangential(x)) / radial(x) starts at
    x_d and runs `iterations` times (cv2.undistortPoints' default count)."""
    k1, k2, p1, p2 = (float(v) for v in dist[:4])
    xd = (points[:, 0] - K[0, 2]) / K[0, 0]
    yd = (points[:, 1] - K[1, 2]) / K[1, 1]
    x, y = xd.copy(), yd.copy()
    for _ in range(iterations):
        r2 = x * x + y * y
        radial = 1.0 + k1 * r2 + k2 * r2 * r2
        dx = 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x)
        dy = p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y
        x = (xd - dx) / radial
        y = (yd - dy) / radial
    return onp.stack([x, y], axis=-1)


def undistort_points_fisheye(points: onp.ndarray, K: onp.ndarray, dist: onp.ndarray,
                             iterations: int = 10) -> onp.ndarray:
    """Pixel coordinates (n, 2) -> normalised undistorted coordinates (n, 2) under the
    fisheye (Kannala-Brandt) model theta_d = theta (1 + k1 theta^2 + k2 theta^4 +
    k3 theta^6 + k4 theta^8): theta solved by Newton's method from theta_d (as many
    steps as cv2.fisheye.undistortPoints takes by default), then scaled by
    tan(theta) / theta_d."""
    k1, k2, k3, k4 = (float(v) for v in dist[:4])
    xd = (points[:, 0] - K[0, 2]) / K[0, 0]
    yd = (points[:, 1] - K[1, 2]) / K[1, 1]
    theta_d = onp.minimum(onp.sqrt(xd * xd + yd * yd), math.pi / 2)
    theta = theta_d.copy()
    for _ in range(iterations):
        t2 = theta * theta
        f = theta * (1 + t2 * (k1 + t2 * (k2 + t2 * (k3 + t2 * k4)))) - theta_d
        df = 1 + t2 * (3 * k1 + t2 * (5 * k2 + t2 * (7 * k3 + t2 * 9 * k4)))
        theta = theta - f / df
    scale = onp.where(theta_d > 1e-8, onp.tan(theta) / onp.maximum(theta_d, 1e-30), 1.0)
    return onp.stack([xd * scale, yd * scale], axis=-1)


# ---------------------------------------------------------------------------------
# Datasets.
# ---------------------------------------------------------------------------------
@dataclasses.dataclass
class RenderedRays:
    """data.py:294-303: colors (*, 3) and their rays."""
    colors: torch.Tensor
    rays_wrt_world: cameras.Rays3D

    def get_batch_axes(self) -> Tuple[int, ...]:
        return tuple(self.colors.shape[:-1])


@dataclasses.dataclass
class RegisteredRgbaView:
    """data.py:285-291: an RGBA image (H, W, 4) in [0, 1] and its camera."""
    image_rgba: onp.ndarray
    camera: cameras.Camera


def _pose(transform_matrix: onp.ndarray) -> Tuple[onp.ndarray, onp.ndarray]:
    """Blender camera-to-world matrix -> (R_world_camera, t_world_camera), OpenCV axes."""
    T = onp.asarray(transform_matrix, dtype=onp.float64)
    if T.shape != (4, 4):
        raise ValueError(f"transform_matrix must be 4x4, got {T.shape}")
    return T[:3, :3] @ _R_BLENDERCAM_CAMERA, T[:3, 3].copy()


def rendered_rays_from_views(views: List[RegisteredRgbaView]) -> RenderedRays:
    """data.py:306-350: every pixel's ray (built on the device) and its colour composited
    over a white background, rgb * alpha + (1 - alpha), concatenated over the views."""
    cols, origins, dirs, cams = [], [], [], []
    for i, view in enumerate(views):
        h, w = view.camera.image_height, view.camera.image_width
        rgba = view.image_rgba
        if rgba.shape != (h, w, 4):
            raise ValueError(f"view {i}: image {rgba.shape} does not match its camera ({h}, {w}, 4)")
        rgb = rgba[..., :3] * rgba[..., 3:4] + (1.0 - rgba[..., 3:4])
        rays = view.camera.pixel_rays_wrt_world()
        cols.append(torch.as_tensor(rgb.reshape(-1, 3), dtype=torch.float32).cuda())
        origins.append(rays.origins)
        dirs.append(rays.directions)
        cams.append(torch.full((h * w,), i, dtype=torch.int32, device="cuda"))
    return RenderedRays(torch.cat(cols), cameras.Rays3D(torch.cat(origins), torch.cat(dirs), torch.cat(cams)))


@dataclasses.dataclass(frozen=True)
class BlenderDataset:
    """data.py:201-279: ``transforms_train.json`` with ``camera_angle_x`` and frames of
    ``file_path`` (+ ".png", RGBA) and ``transform_matrix`` (Blender camera-to-world)."""
    dataset_root: pathlib.Path

    def get_training_rays(self) -> RenderedRays:
        return rendered_rays_from_views(self._registered_views)

    def get_cameras(self) -> List[cameras.Camera]:
        return [v.camera for v in self._registered_views]

    @functools.cached_property
    def _registered_views(self) -> List[RegisteredRgbaView]:
        meta = json.loads((pathlib.Path(self.dataset_root) / "transforms_train.json").read_text())
        fov_x = float(meta["camera_angle_x"])
        out = []
        for frame in meta["frames"]:
            if set(frame) != {"file_path", "rotation", "transform_matrix"}:
                raise ValueError(f"unexpected Blender frame keys {sorted(frame)}")
            image = read_image(pathlib.Path(self.dataset_root) / f"{frame['file_path']}.png")
            if image.dtype != onp.uint8 or image.ndim != 3 or image.shape[2] != 4:
                raise ValueError(f"{frame['file_path']}: Blender views are 8-bit RGBA, got {image.shape}")
            h, w = image.shape[:2]
            R, t = _pose(frame["transform_matrix"])
            cam = cameras.Camera.from_fov(R, t, w, h, fov_x_radians=fov_x)
            out.append(RegisteredRgbaView((image / 255.0).astype(onp.float32), cam))
        return out


@dataclasses.dataclass(frozen=True)
class NerfstudioDataset:
    """data.py:46-198: ``transforms.json`` with pinhole intrinsics (fl_x, fl_y, cx, cy, w,
    h), an OPENCV (k1, k2, p1, p2) or OPENCV_FISHEYE (k1..k4) camera model and frames of
    ``file_path`` and ``transform_matrix``. Camera positions are centred on their bounding
    box, scaled to [-1, 1] along its longest side, then by ``scene_scale``."""
    dataset_root: pathlib.Path
    scene_scale: float

    def _metadata(self) -> dict:
        return json.loads((pathlib.Path(self.dataset_root) / "transforms.json").read_text())

    def get_cameras(self) -> List[cameras.Camera]:
        meta = self._metadata()
        mats = []
        for frame in meta["frames"]:
            if set(frame) != {"file_path", "transform_matrix"}:
                raise ValueError(f"unexpected nerfstudio frame keys {sorted(frame)}")
            mats.append(onp.array(frame["transform_matrix"], dtype=onp.float32))
        K = onp.eye(3)
        K[0, 0], K[1, 1], K[0, 2], K[1, 2] = meta["fl_x"], meta["fl_y"], meta["cx"], meta["cy"]
        pos = onp.array(mats)[:, :3, 3]
        lo, hi = pos.min(axis=0), pos.max(axis=0)
        out = []
        for T in mats:
            T = T.copy()
            T[:3, 3] -= lo
            T[:3, 3] -= (hi - lo) / 2.0
            T[:3, 3] /= (hi - lo).max() / 2.0
            T[:3, 3] *= self.scene_scale
            R, t = _pose(T)
            out.append(cameras.Camera(K.copy(), R, t, int(meta["w"]), int(meta["h"])))
        return out

    def get_training_rays(self) -> RenderedRays:
        meta = self._metadata()
        model = meta["camera_model"]
        if model == "OPENCV":
            dist = onp.array([meta.get(k, 0.0) for k in ("k1", "k2", "p1", "p2")])
        elif model == "OPENCV_FISHEYE":
            dist = onp.array([meta[k] for k in ("k1", "k2", "k3", "k4")])
        else:
            raise ValueError(f"unsupported camera model {model}")
        cols, origins, dirs, cams = [], [], [], []
        for i, (frame, cam) in enumerate(zip(meta["frames"], self.get_cameras())):
            image = read_image(pathlib.Path(self.dataset_root) / frame["file_path"])[..., :3]
            h, w = image.shape[:2]
            oh, ow = h, w
            target = 1200 * 1600  # images above this many pixels are scaled down (data.py:81-88)
            if h * w > target:
                s = math.sqrt(target / (h * w))
                h, w = int(h * s), int(w * s)
                image = resize_bilinear(image, w, h)
            # Pixel (u, v) of the resized image at (u, v) * (original / resized) of the
            # original, whose intrinsics K describes (data.py:92-97).
            uv = onp.stack(onp.meshgrid(onp.arange(w), onp.arange(h), indexing="xy"), axis=-1).reshape(-1, 2)
            pts = uv / onp.array([h, w]) * onp.array([oh, ow])
            if model == "OPENCV":
                xy = undistort_points_opencv(pts.astype(onp.float64), cam.K, dist)
            else:
                xy = undistort_points_fisheye(pts.astype(onp.float64), cam.K, dist)
            d = onp.concatenate([xy, onp.ones((h * w, 1))], axis=-1)
            d /= onp.linalg.norm(d, axis=-1, keepdims=True)
            cols.append(torch.as_tensor((image / 255.0).reshape(-1, 3), dtype=torch.float32).cuda())
            dirs.append(torch.as_tensor(d @ cam.R_world_camera.T, dtype=torch.float32).cuda())
            origins.append(torch.as_tensor(onp.tile(cam.t_world_camera[None, :], (h * w, 1)),
                                           dtype=torch.float32).cuda())
            cams.append(torch.full((h * w,), i, dtype=torch.int32, device="cuda"))
        return RenderedRays(torch.cat(cols), cameras.Rays3D(torch.cat(origins), torch.cat(dirs), torch.cat(cams)))


def make_dataset(dataset_type: Literal["blender", "nerfstudio"], dataset_root: Union[str, pathlib.Path],
                 scene_scale: float) -> Union[BlenderDataset, NerfstudioDataset]:
    """data.py:32-43."""
    if dataset_type == "blender":
        if scene_scale != 1.0:
            raise ValueError("Blender scenes take scene_scale 1.0")
        return BlenderDataset(pathlib.Path(dataset_root))
    if dataset_type == "nerfstudio":
        return NerfstudioDataset(pathlib.Path(dataset_root), scene_scale)
    raise ValueError(f"unknown dataset type {dataset_type!r}")
