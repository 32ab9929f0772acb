"""GPU tests of the FeatureMlp's FiLM camera embeddings (networks.py:103-111): an
``nn.Embed`` table of one ``units``-wide row per camera, whose first half scales and
second half shifts the upper half of layer 2's output before layer 3.

* tvm_mlp_fwd / tvm_mlp_bwd with camera indices against the float64 oracle: rgb, the
  feature gradient and every weight, bias and embedding gradient, at 1e-4 relative
  (split-tf32 tensor-core GEMMs and plain FP32), rows whose hidden pre-activations lie
  within 1e-4 of a ReLU kink redrawn;
* render_rays and loss_and_grad with per-ray camera indices (each ray's camera repeated
  over its appearance samples, render.py:492-497) against the oracle, every gradient
  segment including the embedding, and render_rays_batched carrying each chunk's cameras;
* a training step moves the embedding rows of the cameras it saw and no others."""
import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-4
KINK = 1e-4
NCAM = 7


def _rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    assert a.shape == b.shape and a.numel() > 0
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


def _ref(G, seed):
    gen = torch.Generator().manual_seed(seed)
    ref = {"density": O.vm_init(G, 16, gen, torch.float32), "appearance": O.vm_init(G, 48, gen, torch.float32),
           "mlp": O.mlp_init(144, 2, 2, gen, dtype=torch.float32, num_cameras=NCAM)}
    for layer in ("Dense_1", "Dense_2", "Dense_3"):
        ref["mlp"][layer]["bias"] = torch.randn(ref["mlp"][layer]["bias"].shape, generator=gen) * 0.1
    return ref


def _mlp_inputs(n, seed, mlp):
    """n rows (features, view directions, cameras, output gradient) whose hidden
    pre-activations all lie at least KINK from zero in the float64 oracle."""
    gen = torch.Generator().manual_seed(seed)
    W = {k: {nm: t.double() for nm, t in d.items()} for k, d in mlp.items()}
    kf, kd = [], []
    while sum(len(t) for t in kf) < n:
        feats = torch.randn((2 * n + 8, 144), generator=gen) * 0.3
        dirs = torch.nn.functional.normalize(torch.randn((2 * n + 8, 3), generator=gen), dim=-1)
        f = feats.double() @ W["Dense_0"]["kernel"]
        x1 = torch.cat([f, dirs.double(), O.fourier_encode(f, 2), O.fourier_encode(dirs.double(), 2)], dim=-1)
        z1 = x1 @ W["Dense_1"]["kernel"] + W["Dense_1"]["bias"]
        z2 = torch.relu(z1) @ W["Dense_2"]["kernel"] + W["Dense_2"]["bias"]
        ok = (z1.abs().min(dim=1).values > KINK) & (z2.abs().min(dim=1).values > KINK)
        kf.append(feats[ok])
        kd.append(dirs[ok])
    feats, dirs = torch.cat(kf)[:n], torch.cat(kd)[:n]
    cams = torch.randint(0, NCAM, (n,), generator=gen, dtype=torch.int32)
    return feats, dirs, cams, torch.randn((n, 3), generator=gen)


@pytest.mark.parametrize("math_", ["tensor", "simt"])
@pytest.mark.parametrize("n", [1, 300, 5000])
def test_film_mlp_matches_oracle(math_, n):
    from tensorf_gb300 import render
    spec = render.ModelSpec(grid_dim=8, num_cameras=NCAM, mlp_math=math_)
    ref = _ref(8, 3)
    lp = render.LearnableParams.from_reference(spec, ref)
    feats, dirs, cams, grad_rgb = _mlp_inputs(n, 40 + n, ref["mlp"])
    f = feats.cuda().requires_grad_(True)
    params = lp.params.requires_grad_(True)  # the flat buffer is the autograd leaf of every MLP weight
    out = spec.mlp().apply(lp, f, dirs.cuda(), cams.cuda())
    (out * grad_rgb.cuda()).sum().backward()
    grads = params.grad
    mlp64 = {k: {nm: t.double().requires_grad_(True) for nm, t in d.items()} for k, d in ref["mlp"].items()}
    f64 = feats.double().requires_grad_(True)
    r64 = O.feature_mlp(mlp64, f64, dirs.double(), 2, 2, camera_indices=cams)
    (r64 * grad_rgb.double()).sum().backward()
    assert _rel(out, r64) < RTOL
    assert _rel(f.grad, f64.grad) < RTOL
    got = lp.mlp_views(grads)
    for layer, v in mlp64.items():
        for name, t in v.items():
            assert _rel(got[layer][name], t.grad) < RTOL, (layer, name, _rel(got[layer][name], t.grad))


def test_film_render_and_gradients_match_oracle():
    import test_gpu_configs as TC
    from tensorf_gb300 import cameras, render, scene
    G, R, N, k, shift = 24, 256, 96, 24, -1.0
    ref = _ref(G, 5)
    o, d, c = (torch.tensor(a) for a in scene.sphere_rays(R, 5))
    cams = torch.randint(0, NCAM, (R,), generator=torch.Generator().manual_seed(6), dtype=torch.int32)
    rng = np.random.default_rng(5)
    jit = torch.tensor(rng.uniform(size=N), dtype=torch.float32)
    gum = torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    # Near-ties depend on the density only and the ReLU kinks lie before the FiLM step,
    # so the filter runs the model without the embedding.
    plain = dict(ref, mlp={n: v for n, v in ref["mlp"].items() if n != "Embed_0"})
    keep, _, _ = TC._keep_rays(TC._to64(plain), aabb.double(), o.double(), d.double(), N, k, jit.double(),
                               gum.double(), shift)
    assert float(keep.float().mean()) > 0.8
    o, d, c, cams = o[keep].contiguous(), d[keep].contiguous(), c[keep].contiguous(), cams[keep].contiguous()

    spec = render.ModelSpec(grid_dim=G, num_cameras=NCAM)
    lp = render.LearnableParams.from_reference(spec, ref)
    rays = cameras.Rays3D(o.cuda(), d.cuda(), cams.cuda())
    noise = render.RenderNoise(jit.cuda(), gum.cuda())
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    img = render.render_rays(spec.mlp(), lp, aabb, rays, noise, cfg, density_shift=shift).cpu()
    grads = torch.zeros_like(lp.params)
    loss = float(render.loss_and_grad(lp, grads, aabb, rays, c.cuda(), noise, cfg, density_shift=shift).item())

    ref64 = TC._to64(ref, grad=True)
    out = O.render_rays(ref64, aabb.double(), o.double(), d.double(), N, k, jit.double(), gum.double(),
                        density_shift=shift, camera_indices=cams)
    L = O.mse(out, c.double())
    L.backward()
    assert _rel(img, out) < RTOL
    assert abs(loss - float(L.detach())) <= RTOL * float(L.detach())
    g = lp.to_reference(grads)
    errs = {f"{grp}.{i}": _rel(g[grp][i], ref64[grp][i].grad) for grp in ("density", "appearance") for i in (0, 1)}
    errs.update({f"{layer}.{nm}": _rel(g["mlp"][layer][nm], ref64["mlp"][layer][nm].grad)
                 for layer in ref64["mlp"] for nm in ref64["mlp"][layer]})
    print({a: f"{b:.1e}" for a, b in errs.items()})
    assert max(errs.values()) < RTOL, errs
    # Chunked rendering hands each chunk its own rays' cameras.
    chunked = render.render_rays_batched(spec.mlp(), lp, aabb, rays, noise, cfg, batch_size=64,
                                         density_shift=shift, to_host=False).cpu()
    assert _rel(chunked, img) < 1e-6


def test_film_training_step_moves_only_seen_cameras():
    from tensorf_gb300 import cameras, render, scene, training
    spec = render.ModelSpec(grid_dim=16, num_cameras=NCAM)
    cfg = training.TrainConfig(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3, density_samples_per_ray=64,
                               appearance_samples_per_ray=16, density_shift=-1.0)
    ts = training.TrainState.initialize(cfg, spec, seed=2)
    o, d, c = scene.sphere_rays(128, 2)
    cams = torch.randint(0, 3, (128,), generator=torch.Generator().manual_seed(2), dtype=torch.int32)  # cameras 0..2
    before = ts.learnable_params.mlp_views()["Embed_0"]["embedding"].clone()
    _, log = ts.training_step(cameras.Rays3D(torch.tensor(o).cuda(), torch.tensor(d).cuda(), cams.cuda()),
                              torch.tensor(c).cuda())
    after = ts.learnable_params.mlp_views()["Embed_0"]["embedding"]
    moved = (after - before).abs().amax(dim=1).cpu()
    assert np.isfinite(log["train/mse"])
    assert bool((moved[:3] > 0).all()) and float(moved[3:].abs().max()) == 0.0
    assert float(ts.grads.abs().max()) == 0.0
