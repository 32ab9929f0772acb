"""GPU edge cases against the oracle: the two-samples-per-quad gradient scatter with even
and odd sample counts (pairs that straddle two rays), an empty batch, a single ray with
one sample, rays that miss the box, the minimum grid, and k = N."""
import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def _rel(a, b):
    a = torch.as_tensor(a.detach() if torch.is_tensor(a) else a, dtype=torch.float64).cpu()
    b = torch.as_tensor(b.detach() if torch.is_tensor(b) else b, dtype=torch.float64).cpu()
    assert a.numel() > 0 and a.shape == b.shape
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


def _params(G, seed):
    gen = torch.Generator().manual_seed(seed)
    return {"density": O.vm_init(G, 16, gen, torch.float32), "appearance": O.vm_init(G, 48, gen, torch.float32),
            "mlp": O.mlp_init(144, 2, 2, gen, dtype=torch.float32)}


def _to64(p):
    return {"density": tuple(t.double() for t in p["density"]), "appearance": tuple(t.double() for t in p["appearance"]),
            "mlp": {k: {n: t.double() for n, t in d.items()} for k, d in p["mlp"].items()}}


def _noise(N, seed):
    rng = np.random.default_rng(seed)
    jit = torch.tensor(rng.uniform(size=N), dtype=torch.float32)
    gum = torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32)
    return jit, gum


def _tie_free(ref64, aabb, o, d, N, k, jit, gum, shift):
    _, aux = O.render_rays(ref64, aabb.double(), o.double(), d.double(), N, k, jit.double(), gum.double(),
                           density_shift=shift, return_aux=True)
    keys = torch.log(aux["p_terminates"].detach()) + gum.double()
    if k >= N:
        return torch.ones(keys.shape[0], dtype=torch.bool)
    srt = torch.sort(keys, dim=-1, descending=True).values
    m = srt[:, k - 1] - srt[:, k]
    return (m > 1e-5) | ~torch.isfinite(m)


def _render_parity(G, R, N, k, seed, o, d, shift=-1.0):
    from tensorf_gb300 import cameras, render
    ref = _params(G, seed)
    jit, gum = _noise(N, seed)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    spec = render.ModelSpec(grid_dim=G)
    lp = render.LearnableParams.from_reference(spec, ref)
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    out = render.render_rays(spec.mlp(), lp, aabb, cameras.Rays3D(o.cuda(), d.cuda()),
                             render.RenderNoise(jit.cuda(), gum.cuda()), cfg, density_shift=shift).cpu()
    ref64 = _to64(ref)
    want = O.render_rays(ref64, aabb.double(), o.double(), d.double(), N, k, jit.double(), gum.double(),
                         density_shift=shift)
    ok = _tie_free(ref64, aabb, o, d, N, k, jit, gum, shift)
    assert ok.float().mean() > 0.9
    assert _rel(out[ok], want[ok]) < RTOL


@pytest.mark.parametrize("N,k", [(128, 32), (129, 33), (160, 48)])
def test_pair_scatter_gradients_match_oracle(N, k):
    """N >= 128 and k >= 32 take the merged two-samples-per-quad scatter; odd N and k
    put the second sample of some quads on the next ray."""
    from tensorf_gb300 import cameras, render, scene
    G, R, shift = 24, 160, -1.0
    ref = _params(G, 11 + N)
    o, d, c = (torch.tensor(a) for a in scene.sphere_rays(R, 12 + N))
    jit, gum = _noise(N, 13 + N)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    ref64 = _to64(ref)
    ok = _tie_free(ref64, aabb, o, d, N, k, jit, gum, shift)
    o, d, c = o[ok], d[ok], c[ok]
    spec = render.ModelSpec(grid_dim=G)
    lp = render.LearnableParams.from_reference(spec, ref)
    grads = torch.zeros_like(lp.params)
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    loss = render.loss_and_grad(lp, grads, aabb, cameras.Rays3D(o.cuda(), d.cuda()), c.cuda(),
                                render.RenderNoise(jit.cuda(), gum.cuda()), cfg, density_shift=shift)
    for t in (*ref64["density"], *ref64["appearance"]):
        t.requires_grad_(True)
    for lay in ref64["mlp"].values():
        for t in lay.values():
            t.requires_grad_(True)
    out = O.render_rays(ref64, aabb.double(), o.double(), d.double(), N, k, jit.double(), gum.double(),
                        density_shift=shift)
    L = O.mse(out, c.double())
    L.backward()
    assert abs(float(loss.item()) - float(L.detach())) <= RTOL * float(L.detach())
    g = lp.to_reference(grads)
    for got, want in ((g["density"][0], ref64["density"][0].grad), (g["density"][1], ref64["density"][1].grad),
                      (g["appearance"][0], ref64["appearance"][0].grad),
                      (g["appearance"][1], ref64["appearance"][1].grad)):
        assert _rel(got, want) < 1e-4


def test_empty_batch():
    from tensorf_gb300 import cameras, render
    G, N, k = 8, 32, 8
    spec = render.ModelSpec(grid_dim=G)
    lp = render.LearnableParams.from_reference(spec, _params(G, 1))
    jit, gum = _noise(N, 1)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    empty = cameras.Rays3D(torch.zeros((0, 3), device="cuda"), torch.zeros((0, 3), device="cuda"))
    noise = render.RenderNoise(jit.cuda(), gum.cuda())
    out = render.render_rays(spec.mlp(), lp, aabb, empty, noise, cfg, density_shift=-1.0)
    assert out.shape == (0, 3)
    grads = torch.zeros_like(lp.params)
    loss = render.loss_and_grad(lp, grads, aabb, empty, torch.zeros((0, 3), device="cuda"), noise, cfg,
                                density_shift=-1.0)
    assert float(loss.item()) == 0.0 and float(grads.abs().max()) == 0.0


def test_single_ray_single_sample():
    o, d, _ = (torch.tensor(a) for a in __import__("tensorf_gb300.scene", fromlist=["x"]).sphere_rays(1, 2))
    _render_parity(G=8, R=1, N=1, k=1, seed=2, o=o, d=d)


def test_rays_that_miss_the_box():
    """Rays pointing away from the box get the reference's default segment [0, 1e-3]
    (render.py:426-434) and render as background plus that sliver."""
    rng = np.random.default_rng(3)
    o = torch.tensor(rng.normal(size=(64, 3)), dtype=torch.float32)
    o = o / o.norm(dim=1, keepdim=True) * 4.0
    d = o / o.norm(dim=1, keepdim=True)  # straight away from the origin
    _render_parity(G=8, R=64, N=32, k=8, seed=3, o=o, d=d)


def test_minimum_grid():
    from tensorf_gb300 import scene
    o, d, _ = (torch.tensor(a) for a in scene.sphere_rays(64, 4))
    _render_parity(G=2, R=64, N=32, k=8, seed=4, o=o, d=d)


def test_k_equals_n():
    from tensorf_gb300 import scene
    o, d, _ = (torch.tensor(a) for a in scene.sphere_rays(64, 5))
    _render_parity(G=16, R=64, N=32, k=32, seed=5, o=o, d=d)
