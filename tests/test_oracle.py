"""CPU tests of the oracle: pins against scipy golden vectors, closed forms, finite
differences, and the reference semantics the CUDA path is checked against."""
import math
import os

import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_map_coordinates.npz")


def test_map_coordinates_matches_scipy_golden():
    z = np.load(GOLDEN)
    for g in (2, 5, 17):
        line = torch.tensor(z[f"line_{g}"])[None]
        plane = torch.tensor(z[f"plane_{g}"])[None]
        y1 = O.map_coordinates_linear_nearest(line, torch.tensor(z[f"c1_{g}"])[None])[0]
        y2 = O.map_coordinates_linear_nearest(plane, torch.tensor(z[f"c2_{g}"]))[0]
        np.testing.assert_allclose(y1.numpy(), z[f"y1_{g}"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(y2.numpy(), z[f"y2_{g}"], rtol=0, atol=1e-12)


def test_map_coordinates_edge_gradient_weight_is_one():
    # A coordinate past the edge sends its whole gradient to the edge texel.
    grid = torch.zeros((1, 5), dtype=torch.float64, requires_grad=True)
    y = O.map_coordinates_linear_nearest(grid, torch.tensor([[-0.7, 4.6, 2.25]], dtype=torch.float64))
    y.sum().backward()
    np.testing.assert_allclose(grid.grad[0].numpy(), [1.0, 0.0, 0.75, 0.25, 1.0])


def test_vm_interpolate_shapes_and_permutation():
    gen = torch.Generator().manual_seed(0)
    vec, mat = O.vm_init(6, 4, gen)
    ijk = torch.rand((3, 7, 5), generator=gen, dtype=torch.float64) * 2 - 1
    f = O.vm_interpolate(vec, mat, ijk)
    assert f.shape == (12, 7, 5)
    # Pair 1 reads its line at coordinate 2 (z) and its plane at (x, y).
    u = (ijk + 1) / 2 * 5
    line = O.map_coordinates_linear_nearest(vec[1], u[2:3])
    plane = O.map_coordinates_linear_nearest(mat[1], u[0:2])
    torch.testing.assert_close(f[4:8], line * plane)


def test_segment_probabilities_closed_form():
    # Constant sigma: p_exit_i = exp(-sigma * t_i), weights sum to 1 - p_exit_last.
    sig = torch.full((2, 50), 3.0, dtype=torch.float64)
    st = torch.full((2, 50), 0.02, dtype=torch.float64)
    pe, pt = O.compute_segment_probabilities(sig, st)
    t = torch.arange(1, 51, dtype=torch.float64) * 0.02
    torch.testing.assert_close(pe[0], torch.exp(-3.0 * t))
    torch.testing.assert_close(pt.sum(-1), 1.0 - pe[:, -1])


def test_topk_tie_break_lower_index_first():
    keys = torch.tensor([[1.0, 3.0, 3.0, -math.inf, 3.0, -math.inf, -math.inf]])
    assert O.topk_desc_lower_index(keys, 5).tolist() == [[1, 2, 4, 0, 3]]


def test_gumbel_topk_matches_sequential_sampling_distribution():
    # Gumbel-top-k over log p draws without replacement with probability ~ p.
    p = torch.tensor([0.5, 0.3, 0.15, 0.05], dtype=torch.float64)
    gen = torch.Generator().manual_seed(1)
    u = torch.rand((200000, 4), generator=gen, dtype=torch.float64)
    g = -torch.log(-torch.log(u))
    first = O.choice_without_replacement(p[None].expand(200000, 4), g, 2)[:, 0]
    freq = torch.bincount(first, minlength=4).double() / 200000
    np.testing.assert_allclose(freq.numpy(), p.numpy(), atol=4e-3)


def test_bbox_sampler_matches_hand_computation():
    o = torch.tensor([[0.0, 0.0, -4.0]], dtype=torch.float64)
    d = torch.tensor([[0.0, 0.0, 1.0]], dtype=torch.float64)
    aabb = torch.tensor([[-1.0, -1.0, -1.0], [1.0, 1.0, 1.0]], dtype=torch.float64)
    t0, t1 = O.ray_segment_from_bounding_box(o, d, aabb)
    # x/y slabs are hit at +-1/1e-8 (direction + 1e-8), z at 3 and 5.
    assert abs(float(t0) - 3.0) < 1e-6 and abs(float(t1) - 5.0) < 1e-6
    pts, ts, steps = O.sample_points_bbox(o, d, aabb, 4, torch.zeros(4, dtype=torch.float64))
    np.testing.assert_allclose(ts[0].numpy(), [3.0, 3.5, 4.0, 4.5], atol=1e-6)
    np.testing.assert_allclose(steps[0].numpy(), [0.5] * 4, atol=1e-7)


def test_bbox_sampler_missing_ray_gets_default_segment():
    o = torch.tensor([[5.0, 5.0, 5.0]], dtype=torch.float64)
    d = torch.tensor([[1.0, 0.0, 0.0]], dtype=torch.float64)
    aabb = torch.tensor([[-1.0] * 3, [1.0] * 3], dtype=torch.float64)
    t0, t1 = O.ray_segment_from_bounding_box(o, d, aabb)
    assert float(t0) == 0.0 and abs(float(t1) - 1e-3) < 1e-12


def test_contraction_maps_into_cube():
    p = torch.tensor([[0.5, 0.2, -0.1], [3.0, -1.0, 0.5], [-100.0, 0.0, 0.0]], dtype=torch.float64)
    c = O.contract_points(p)
    torch.testing.assert_close(c[0], p[0])
    assert torch.all(c.abs().amax(-1) <= 2.0)
    torch.testing.assert_close(c[1], (2 - 1 / 3.0) * p[1] / 3.0)


def test_fourier_encode_layout():
    x = torch.tensor([[0.3, -1.2]], dtype=torch.float64)
    e = O.fourier_encode(x, 2)
    exp = [math.sin(0.3), math.sin(0.6), math.sin(0.3 + math.pi / 2), math.sin(0.6 + math.pi / 2),
           math.sin(-1.2), math.sin(-2.4), math.sin(-1.2 + math.pi / 2), math.sin(-2.4 + math.pi / 2)]
    np.testing.assert_allclose(e[0].numpy(), exp, atol=1e-12)


def _small_problem(dtype=torch.float64, seed=0, R=6, N=24, k=8, G=9, Cd=8, Ca=8):
    gen = torch.Generator().manual_seed(seed)
    params = {"density": O.vm_init(G, Cd, gen, dtype), "appearance": O.vm_init(G, Ca, gen, dtype),
              "mlp": O.mlp_init(3 * Ca, 2, 2, gen, dtype=dtype)}
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(R, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * 4
    d = -o + rng.normal(scale=0.05, size=(R, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3], dtype=dtype)
    jitter = torch.tensor(rng.uniform(size=N), dtype=dtype)
    gumbel = torch.tensor(-np.log(-np.log(rng.uniform(1e-6, 1 - 1e-6, size=N))), dtype=dtype)
    colors = torch.tensor(rng.uniform(size=(R, 3)), dtype=dtype)
    return params, torch.tensor(o, dtype=dtype), torch.tensor(d, dtype=dtype), aabb, jitter, gumbel, colors


def _flat(params):
    leaves = [params["density"][0], params["density"][1], params["appearance"][0], params["appearance"][1]]
    for k in sorted(params["mlp"]):
        leaves += [params["mlp"][k][n] for n in sorted(params["mlp"][k])]
    return leaves


def test_render_rays_gradient_matches_finite_differences():
    params, o, d, aabb, jit, gum, col = _small_problem()
    leaves = _flat(params)
    for t in leaves:
        t.requires_grad_(True)

    def loss():
        out = O.render_rays(params, aabb, o, d, 24, 8, jit, gum, density_shift=-1.0)
        return O.mse(out, col)

    L = loss()
    grads = torch.autograd.grad(L, leaves)
    gen = torch.Generator().manual_seed(5)
    h = 1e-6
    checked = 0
    with torch.no_grad():
        for leaf, g in zip(leaves, grads):
            flat = leaf.view(-1)
            for idx in torch.randint(0, flat.numel(), (4,), generator=gen).tolist():
                old = float(flat[idx])
                flat[idx] = old + h
                lp = float(loss())
                flat[idx] = old - h
                lm = float(loss())
                flat[idx] = old
                fd = (lp - lm) / (2 * h)
                an = float(g.view(-1)[idx])
                assert abs(fd - an) <= 1e-6 + 1e-4 * abs(fd), (fd, an)
                checked += 1
    assert checked == 4 * len(leaves)


def test_dist_median_reference_formula_is_nan_for_terminating_rays():
    params, o, d, aabb, jit, gum, col = _small_problem()
    ref = O.render_rays(params, aabb, o, d, 24, 8, jit, gum, density_shift=10.0, mode="dist_median_reference")
    med = O.render_rays(params, aabb, o, d, 24, 8, jit, gum, density_shift=10.0, mode="dist_median")
    terminated = torch.isfinite(med)
    assert terminated.any()
    assert torch.isnan(ref[terminated]).all()
    assert torch.isinf(ref[~terminated]).all() if (~terminated).any() else True


def test_lr_decay_coeff_schedule():
    assert O.lr_decay_coeff(0, 30000, (2000,)) == 1.0
    np.testing.assert_allclose(O.lr_decay_coeff(15000, 30000, ()), 0.1 ** 0.5, rtol=1e-6)
    # Reset after the upsampling iteration 2000.
    np.testing.assert_allclose(O.lr_decay_coeff(2000 + 3000, 30000, (2000,)), 0.1 ** 0.1, rtol=1e-6)
    assert O.lr_decay_coeff(10 ** 7, 30000, ()) == 0.1


def test_adam_first_step_is_sign_times_lr():
    p = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64)
    g = torch.tensor([0.3, -4.0, 0.0], dtype=torch.float64)
    z = torch.zeros(3, dtype=torch.float64)
    p2, m, v = O.adam_update(p, g, z, z, 1, lr=0.02, lr_decay=1.0)
    # bias-corrected first step: mhat/(sqrt(vhat)+eps) = g/(|g|+eps)
    np.testing.assert_allclose((p2 - p).numpy(), [-0.02, 0.02, 0.0], atol=1e-8)


def test_sphere_scene_quadrature_background_and_opaque():
    o = np.array([[0.0, 0.0, -4.0], [0.0, 3.0, -4.0]])
    d = np.array([[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]])
    out = O.sphere_scene_quadrature(o, d, np.zeros((1, 3)), np.array([0.5]), np.array([[0.2, 0.4, 0.6]]), 50.0,
                                    np.array([2.5, 2.5]), np.array([5.5, 5.5]), 4096)
    np.testing.assert_allclose(out[0], [0.2, 0.4, 0.6], atol=1e-6)  # opaque sphere
    np.testing.assert_allclose(out[1], [1.0, 1.0, 1.0], atol=1e-12)  # background


def test_camera_rays_center_pixel_looks_forward():
    K = O.camera_K_from_fov(800, 800, fov_x=2 * math.atan(400 / 1111.0))
    assert abs(K[0, 0] - 1111.0) < 1e-9 and K[0, 2] == 399.5
    o, d = O.camera_pixel_rays(K, np.eye(3), np.zeros(3), 800, 800)
    mid = 399 * 800 + 399
    assert d[mid][2] > 0.999999


def test_proposal_loss_gradient_matches_finite_differences():
    # Resampling carries no gradient, so the check freezes the resampled intervals and
    # bins and differentiates the bound loss wrt the proposal parameters alone.
    gen = torch.Generator().manual_seed(0)
    G, Gp, R, Np, N, k = 8, 6, 6, 12, 8, 4
    prop = {"vector": torch.randn((3, 4, Gp), generator=gen, dtype=torch.float64) * 0.1,
            "matrix": torch.randn((3, 4, Gp, Gp), generator=gen, dtype=torch.float64) * 0.1,
            "w1": torch.randn((16, 16), generator=gen, dtype=torch.float64) * 0.3,
            "b1": torch.zeros(16, dtype=torch.float64),
            "w2": torch.randn((16, 1), generator=gen, dtype=torch.float64) * 0.3,
            "b2": torch.zeros(1, dtype=torch.float64)}
    params = {"density": O.vm_init(G, 8, gen), "appearance": O.vm_init(G, 8, gen), "mlp": O.mlp_init(24, 2, 2, gen)}
    rng = np.random.default_rng(0)
    o = rng.normal(size=(R, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * 4
    d = -o + rng.normal(scale=0.05, size=(R, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o, d = torch.tensor(o), torch.tensor(d)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3], dtype=torch.float64)
    pj = torch.tensor(rng.uniform(size=(R, Np)))
    jt = torch.tensor(rng.uniform(size=(R, N)))
    gum = torch.tensor(-np.log(-np.log(rng.uniform(size=N))))
    e, wp, _, _ = O.proposal_forward(prop, o, d, aabb, Np, pj, 0.5)
    t, delta, bins = O.resample(e, wp, N, jt)
    assert torch.all(delta >= 0) and torch.all(t[:, 1:] >= t[:, :-1] - 1e-12)
    _, aux = O.render_explicit(params, aabb, o, d, t, delta, k, gum, density_shift=-1.0, return_aux=True)
    wm = aux["p_terminates"].detach()

    def loss():
        _, wp2, _, _ = O.proposal_forward(prop, o, d, aabb, Np, pj, 0.5)
        return O.proposal_loss(wm, wp2, bins, 1.0)

    for tt in prop.values():
        tt.requires_grad_(True)
    grads = torch.autograd.grad(loss(), list(prop.values()))
    h = 1e-6
    with torch.no_grad():
        for tt, gg in zip(prop.values(), grads):
            for idx in range(min(4, tt.numel())):
                old = float(tt.view(-1)[idx])
                tt.view(-1)[idx] = old + h
                lp = float(loss())
                tt.view(-1)[idx] = old - h
                lm = float(loss())
                tt.view(-1)[idx] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - float(gg.view(-1)[idx])) <= 1e-6 * max(1.0, abs(fd)) + 1e-9


def test_resample_quantiles_follow_the_histogram():
    # A proposal with all its mass in one bin puts ~99% of the main edges inside it.
    edges = torch.linspace(0.0, 1.0, 9, dtype=torch.float64)[None]
    w = torch.zeros((1, 8), dtype=torch.float64)
    w[0, 5] = 1.0
    t, delta, bins = O.resample(edges, w, 100, torch.full((1, 100), 0.5, dtype=torch.float64))
    inside = ((t > 0.625) & (t < 0.75)).double().mean()
    assert inside > 0.95
    assert float(delta.sum()) == pytest.approx(1.0)


def test_resize_upsampling_matches_torch_align_corners():
    """resize_with_aligned_corners (tensor_vm.py:202-223) upsampling = bilinear
    interpolation with aligned corners: pinned against torch's own implementation."""
    gen = torch.Generator().manual_seed(4)
    vec = torch.randn((6, 9), generator=gen, dtype=torch.float64)
    mat = torch.randn((6, 9, 9), generator=gen, dtype=torch.float64)
    for n in (9, 17, 23):
        got_v = O.resize_with_aligned_corners(vec, (6, n))
        got_m = O.resize_with_aligned_corners(mat, (6, n, n))
        want_v = torch.nn.functional.interpolate(vec[None], size=n, mode="linear", align_corners=True)[0]
        want_m = torch.nn.functional.interpolate(mat[None], size=(n, n), mode="bilinear", align_corners=True)[0]
        # The sample positions are float32 under jax (x64 off): agreement to float32 rounding.
        assert float((got_v - want_v).abs().max()) < 1e-5
        assert float((got_m - want_m).abs().max()) < 1e-5


def test_resize_downsampling_antialias_properties():
    """Downsampling widens the triangle kernel (antialias): the weights of every output
    sum to one, constants stay constant, and a ramp stays increasing and inside its range
    (the wide, truncated kernels are not exact on a ramp)."""
    import numpy as np
    w = O.scale_translate_weights(40, 12, 11 / 39, -(11 / 39 / 2 - 0.5))
    assert np.allclose(w.sum(axis=0), 1.0, atol=1e-6)
    assert int((w > 0).sum(axis=0).max()) > 2  # wider than linear interpolation
    ramp = torch.linspace(-1.0, 3.0, 40, dtype=torch.float64)[None]
    out = O.resize_with_aligned_corners(ramp, (1, 12))[0]
    want = torch.linspace(-1.0, 3.0, 12, dtype=torch.float64)
    assert bool((out[1:] > out[:-1]).all())
    assert float(out.min()) >= -1.0 and float(out.max()) <= 3.0
    assert float((out[1:-1] - want[1:-1]).abs().max()) < 5e-3
    const = torch.full((2, 40, 40), 0.7, dtype=torch.float64)
    assert float((O.resize_with_aligned_corners(const, (2, 12, 12)) - 0.7).abs().max()) < 1e-6


def test_upsampling_schedule():
    """training.py:358-367: linear from grid_dim_init to grid_dim_final."""
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tensorf-jax_gb300"))
    from tensorf_gb300 import training
    cfg = training.TrainConfig()
    dims = [training.upsampled_grid_dim(cfg, s) for s in cfg.upsamp_iters]
    assert dims == [162, 196, 231, 265, 300]
    assert training.upsampled_grid_dim(cfg, 2001) is None
