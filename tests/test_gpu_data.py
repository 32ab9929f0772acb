"""Dataset rays on the GPU (tensorf/data.py): Blender views through the device camera
rays against the oracle's pinhole rays, with colours composited over white; nerfstudio
frames through the undistorted pixel directions (without distortion they are the
pinhole rays), and a dataset's rays training a model."""
import math

import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O
from test_data import _blender_dataset, _nerfstudio_dataset

pytestmark = pytest.mark.gpu


def test_blender_training_rays_match_oracle(tmp_path):
    from tensorf_gb300 import data
    _, images = _blender_dataset(tmp_path, n_views=3, w=16, h=12, seed=5)
    ds = data.make_dataset("blender", tmp_path, 1.0)
    rr = ds.get_training_rays()
    n = 16 * 12
    assert rr.get_batch_axes() == (3 * n,)
    assert rr.rays_wrt_world.camera_indices.dtype == torch.int32
    for i, (img, cam) in enumerate(zip(images, ds.get_cameras())):
        sl = slice(i * n, (i + 1) * n)
        rgba = img.reshape(-1, 4) / 255.0
        want = rgba[:, :3] * rgba[:, 3:] + (1 - rgba[:, 3:])  # data.py:328-330
        np.testing.assert_allclose(rr.colors[sl].cpu().numpy(), want, atol=1e-6)
        o, d = O.camera_pixel_rays(cam.K, cam.R_world_camera, cam.t_world_camera, 16, 12)
        np.testing.assert_allclose(rr.rays_wrt_world.origins[sl].cpu().numpy(), o, atol=1e-6)
        np.testing.assert_allclose(rr.rays_wrt_world.directions[sl].cpu().numpy(), d, atol=1e-6)
        assert bool((rr.rays_wrt_world.camera_indices[sl] == i).all())


@pytest.mark.parametrize("model", ["OPENCV", "OPENCV_FISHEYE"])
def test_nerfstudio_rays_without_distortion_coefficients(tmp_path, model):
    """With all coefficients zero the pinhole model gives the pinhole rays; the fisheye
    model is then the equidistant projection (image radius = angle off the axis), so a
    pixel at normalised radius r has the ray at angle r."""
    import json
    from tensorf_gb300 import data
    meta = _nerfstudio_dataset(tmp_path, model)
    for k in ("k1", "k2", "k3", "k4", "p1", "p2"):
        if k in meta:
            meta[k] = 0.0
    (tmp_path / "transforms.json").write_text(json.dumps(meta))
    ds = data.make_dataset("nerfstudio", tmp_path, 1.0)
    rr = ds.get_training_rays()
    n = meta["w"] * meta["h"]
    for i, cam in enumerate(ds.get_cameras()):
        sl = slice(i * n, (i + 1) * n)
        o, d = O.camera_pixel_rays(cam.K, cam.R_world_camera, cam.t_world_camera, meta["w"], meta["h"])
        if model == "OPENCV_FISHEYE":
            v, u = np.mgrid[:meta["h"], :meta["w"]]
            x = (u.ravel() - cam.K[0, 2]) / cam.K[0, 0]
            y = (v.ravel() - cam.K[1, 2]) / cam.K[1, 1]
            r = np.sqrt(x * x + y * y)
            s = np.where(r > 0, np.tan(r) / np.maximum(r, 1e-30), 1.0)
            c = np.stack([x * s, y * s, np.ones_like(x)], axis=-1)
            d = (c / np.linalg.norm(c, axis=-1, keepdims=True)) @ cam.R_world_camera.T
        np.testing.assert_allclose(rr.rays_wrt_world.directions[sl].cpu().numpy(), d, atol=1e-6)
        np.testing.assert_allclose(rr.rays_wrt_world.origins[sl].cpu().numpy(), o, atol=1e-6)
        img = data.read_png(tmp_path / f"f{i}.png")
        np.testing.assert_allclose(rr.colors[sl].cpu().numpy(), img.reshape(-1, 3) / 255.0, atol=1e-6)


def test_nerfstudio_distortion_turns_rays_towards_the_axis(tmp_path):
    """With k1 > 0 a ray's distorted image point lies further from the centre than its
    pinhole projection, so undistortion turns an off-centre pixel's ray towards the
    optical axis."""
    from tensorf_gb300 import data
    meta = _nerfstudio_dataset(tmp_path, "OPENCV")
    ds = data.make_dataset("nerfstudio", tmp_path, 1.0)
    rr = ds.get_training_rays()
    cam = ds.get_cameras()[0]
    n = meta["w"] * meta["h"]
    d = rr.rays_wrt_world.directions[:n].cpu().numpy().astype(np.float64)
    _, d0 = O.camera_pixel_rays(cam.K, cam.R_world_camera, cam.t_world_camera, meta["w"], meta["h"])
    axis = cam.R_world_camera[:, 2]
    corner = 0  # pixel (0, 0)
    assert math.acos(min(1.0, d[corner] @ axis)) < math.acos(min(1.0, d0[corner] @ axis))


def test_blender_dataset_trains(tmp_path):
    """A few training steps on the dataset's rays lower the loss (the loader's rays and
    colours feed TrainState directly)."""
    from tensorf_gb300 import data, render, training
    _blender_dataset(tmp_path, n_views=4, w=32, h=24, seed=9)
    rr = data.make_dataset("blender", tmp_path, 1.0).get_training_rays()
    spec = render.ModelSpec(grid_dim=16)
    cfg = training.TrainConfig(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3, density_samples_per_ray=32,
                               appearance_samples_per_ray=8, density_shift=-1.0, n_iters=40, upsamp_iters=())
    st = training.TrainState.initialize(cfg, spec, seed=2)
    from tensorf_gb300 import cameras
    r = rr.rays_wrt_world
    mses = []
    for i in range(40):
        idx = torch.arange(i * 256, (i + 1) * 256, device="cuda") % r.origins.shape[0]
        _, log = st.training_step(cameras.Rays3D(r.origins[idx], r.directions[idx]), rr.colors[idx])
        mses.append(log["train/mse"])
    assert np.mean(mses[-10:]) < np.mean(mses[:10])
