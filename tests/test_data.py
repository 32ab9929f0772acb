"""Dataset loading (tensorf/data.py): the PNG decoder against images written with every
row filter, the bilinear resize, both undistortion models against their forward models,
and the Blender / nerfstudio metadata and cameras on small synthetic datasets. The rays
themselves are built on the GPU (test_gpu_data.py)."""
import json
import math
import struct
import zlib

import numpy as np
import pytest

from tensorf_gb300 import cameras, data

# ---------------------------------------------------------------------------------
# A minimal PNG writer for the fixtures: each row takes filter (row index mod 5).
# ---------------------------------------------------------------------------------


def _chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _filter_row(ftype, row, prev, bpp):
    out = bytearray(len(row))
    for i in range(len(row)):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        if ftype == 0:
            pred = 0
        elif ftype == 1:
            pred = a
        elif ftype == 2:
            pred = b
        elif ftype == 3:
            pred = (a + b) >> 1
        else:
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
        out[i] = (row[i] - pred) & 0xFF
    return bytes(out)


def write_png(path, img: np.ndarray) -> None:
    h, w, ch = img.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[ch]
    raw = bytearray()
    prev = bytes(w * ch)
    for y in range(h):
        row = img[y].astype(np.uint8).tobytes()
        ftype = y % 5
        raw.append(ftype)
        raw += _filter_row(ftype, row, prev, ch)
        prev = row
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    png += _chunk(b"IDAT", zlib.compress(bytes(raw)))
    png += _chunk(b"IEND", b"")
    path.write_bytes(png)


@pytest.mark.parametrize("ch", [1, 2, 3, 4])
def test_png_decoder_undoes_every_row_filter(tmp_path, ch):
    rng = np.random.default_rng(ch)
    img = rng.integers(0, 256, size=(13, 11, ch), dtype=np.uint8)
    img[3:6] = 200  # flat runs next to noise
    write_png(tmp_path / "a.png", img)
    out = data.read_png(tmp_path / "a.png")
    assert out.dtype == np.uint8 and out.shape == img.shape
    assert np.array_equal(out, img)
    assert np.array_equal(data.read_image(tmp_path / "a.png"), img)


def test_png_decoder_rejects_other_formats(tmp_path):
    (tmp_path / "x.png").write_bytes(b"not a png")
    with pytest.raises(ValueError):
        data.read_png(tmp_path / "x.png")


def test_resize_bilinear_half_pixel_centres():
    img = np.arange(8, dtype=np.float64).reshape(1, 8, 1).repeat(2, axis=0)
    half = data.resize_bilinear(img, 4, 2)
    np.testing.assert_allclose(half[0, :, 0], [0.5, 2.5, 4.5, 6.5])  # pairs averaged
    same = data.resize_bilinear(img, 8, 2)
    np.testing.assert_allclose(same, img)
    up = data.resize_bilinear(np.array([[[0.0], [10.0]]]), 4, 1)
    np.testing.assert_allclose(up[0, :, 0], [0.0, 2.5, 7.5, 10.0])  # borders clamp
    u8 = data.resize_bilinear(np.array([[[0], [255]]], dtype=np.uint8), 4, 1)
    assert u8.dtype == np.uint8 and u8[0, 0, 0] == 0 and u8[0, 3, 0] == 255


K = np.array([[500.0, 0.0, 320.0], [0.0, 480.0, 240.0], [0.0, 0.0, 1.0]])


def test_opencv_undistortion_inverts_the_distortion():
    k1, k2, p1, p2 = 0.04, -0.01, 1e-3, -5e-4
    rng = np.random.default_rng(0)
    xy = rng.uniform(-0.5, 0.5, size=(200, 2))
    x, y = xy[:, 0], xy[:, 1]
    r2 = x * x + y * y
    rad = 1 + k1 * r2 + k2 * r2 * r2
    xd = x * rad + 2 * p1 * x * y + p2 * (r2 + 2 * x * x)
    yd = y * rad + p1 * (r2 + 2 * y * y) + 2 * p2 * x * y
    px = np.stack([xd * K[0, 0] + K[0, 2], yd * K[1, 1] + K[1, 2]], axis=-1)
    got = data.undistort_points_opencv(px, K, np.array([k1, k2, p1, p2]))
    np.testing.assert_allclose(got, xy, atol=2e-6)
    none = data.undistort_points_opencv(px, K, np.zeros(4))  # no distortion: K^-1 only
    np.testing.assert_allclose(none, np.stack([xd, yd], axis=-1), atol=1e-12)


def test_fisheye_undistortion_inverts_the_distortion():
    k = np.array([0.05, -0.01, 0.002, -0.0005])
    rng = np.random.default_rng(1)
    xy = rng.uniform(-1.0, 1.0, size=(200, 2))
    r = np.linalg.norm(xy, axis=-1)
    th = np.arctan(r)
    thd = th * (1 + k[0] * th ** 2 + k[1] * th ** 4 + k[2] * th ** 6 + k[3] * th ** 8)
    xyd = xy * (thd / r)[:, None]
    px = np.stack([xyd[:, 0] * K[0, 0] + K[0, 2], xyd[:, 1] * K[1, 1] + K[1, 2]], axis=-1)
    got = data.undistort_points_fisheye(px, K, k)
    np.testing.assert_allclose(got, xy, atol=1e-8)


def _blender_dataset(root, n_views=2, w=8, h=6, seed=0):
    rng = np.random.default_rng(seed)
    frames, images = [], []
    for i in range(n_views):
        img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
        (root / "train").mkdir(exist_ok=True)
        write_png(root / "train" / f"r_{i}.png", img)
        ang = 0.7 * i
        R_wc, eye = cameras.look_at([4.0 * math.sin(ang), -4.0 * math.cos(ang), 0.5])  # at the origin
        T = np.eye(4)
        T[:3, :3] = R_wc @ np.diag([1.0, -1.0, -1.0])  # OpenCV -> Blender camera axes
        T[:3, 3] = eye
        frames.append({"file_path": f"./train/r_{i}", "rotation": 0.1, "transform_matrix": T.tolist()})
        images.append(img)
    (root / "transforms_train.json").write_text(json.dumps({"camera_angle_x": 0.69, "frames": frames}))
    return frames, images


def test_blender_views_and_cameras(tmp_path):
    frames, images = _blender_dataset(tmp_path)
    ds = data.make_dataset("blender", tmp_path, 1.0)
    views = ds._registered_views
    assert len(views) == 2
    for f, img, v in zip(frames, images, views):
        np.testing.assert_allclose(v.image_rgba, img / 255.0, atol=1e-7)
        T = np.array(f["transform_matrix"])
        np.testing.assert_allclose(v.camera.R_world_camera, T[:3, :3] @ np.diag([1.0, -1.0, -1.0]))
        np.testing.assert_allclose(v.camera.t_world_camera, T[:3, 3])
        fx = (8 / 2.0) / math.tan(0.69 / 2.0)  # cameras.py:34-76
        np.testing.assert_allclose(v.camera.K, [[fx, 0, 3.5], [0, fx, 2.5], [0, 0, 1]])
        assert (v.camera.image_width, v.camera.image_height) == (8, 6)
    with pytest.raises(ValueError):
        data.make_dataset("blender", tmp_path, 2.0)
    with pytest.raises(ValueError):
        data.make_dataset("llff", tmp_path, 1.0)


def _nerfstudio_dataset(root, model="OPENCV", w=10, h=7):
    rng = np.random.default_rng(3)
    frames = []
    for i, pos in enumerate(([1.0, 2.0, 3.0], [3.0, 2.5, 2.0], [2.0, 6.0, 2.5])):
        img = rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
        write_png(root / f"f{i}.png", img)
        T = np.eye(4)
        T[:3, 3] = pos
        frames.append({"file_path": f"f{i}.png", "transform_matrix": T.tolist()})
    meta = {"camera_model": model, "fl_x": 9.0, "fl_y": 8.5, "cx": 4.5, "cy": 3.0, "w": w, "h": h,
            "frames": frames}
    if model == "OPENCV":
        meta.update(k1=0.01, k2=0.0, p1=0.0, p2=0.0)
    else:
        meta.update(k1=0.01, k2=0.0, k3=0.0, k4=0.0)
    (root / "transforms.json").write_text(json.dumps(meta))
    return meta


def test_nerfstudio_cameras_centred_and_scaled(tmp_path):
    _nerfstudio_dataset(tmp_path)
    cams = data.make_dataset("nerfstudio", tmp_path, 0.5).get_cameras()
    pos = np.array([[1.0, 2.0, 3.0], [3.0, 2.5, 2.0], [2.0, 6.0, 2.5]])
    lo, hi = pos.min(0), pos.max(0)
    want = (pos - lo - (hi - lo) / 2) / ((hi - lo).max() / 2) * 0.5  # data.py:176-181
    for c, p in zip(cams, want):
        np.testing.assert_allclose(c.t_world_camera, p, atol=1e-6)
        np.testing.assert_allclose(c.R_world_camera, np.diag([1.0, -1.0, -1.0]))
        np.testing.assert_allclose(c.K, [[9.0, 0, 4.5], [0, 8.5, 3.0], [0, 0, 1]])
