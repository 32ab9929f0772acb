"""GPU parity of the nerfstudio preset (train_nerfstudio.py:23-44), against the float64 oracle.

The preset differs from the bounded defaults in every part of the path at once:
  - scene contraction to [-2, 2]^3 with the reference's contracted sample schedule
    (render.py:122-173) and per-sample jitter;
  - a 32-component density field beside the 48-component appearance field;
  - six Fourier frequencies for features and view directions (a 390-wide encoding,
    which runs the layered split-tf32 FeatureMlp);
  - FiLM camera embeddings (networks.py:103-111), one camera index per ray.

The render, the loss and every gradient segment (both fields, every FeatureMlp kernel
and bias, the embedding table) are compared with the oracle at 1e-4 relative to each
tensor's largest magnitude, on a small grid. Rays with a top-k near-tie or a FeatureMlp
pre-activation within 1e-5 of the layer's RMS of zero are left out, and counted. A short
training run at the preset's own grid and batch checks that the step runs and learns.
"""
import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-4
KINK_REL = 1e-5
TIE_MARGIN = 1e-5
NCAM = 5


def _rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    assert a.shape == b.shape and a.numel() > 0
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


def _reference_params(spec, seed):
    gen = torch.Generator().manual_seed(seed)
    ref = {"density": O.vm_init(spec.grid_dim, spec.density_feat_dim, gen, torch.float32),
           "appearance": O.vm_init(spec.grid_dim, spec.appearance_feat_dim, gen, torch.float32),
           "mlp": O.mlp_init(3 * spec.appearance_feat_dim, spec.feature_n_freqs, spec.viewdir_n_freqs, gen,
                             dtype=torch.float32, num_cameras=spec.num_cameras)}
    for layer in ("Dense_1", "Dense_2", "Dense_3"):
        ref["mlp"][layer]["bias"] = torch.randn(ref["mlp"][layer]["bias"].shape, generator=gen) * 0.05
    return ref


def _to64(p, grad=False):
    t = lambda x: x.double().requires_grad_(grad)  # noqa: E731
    return {"density": tuple(t(x) for x in p["density"]), "appearance": tuple(t(x) for x in p["appearance"]),
            "mlp": {k: {n: t(x) for n, x in d.items()} for k, d in p["mlp"].items()}}


def _keep(ref64, aabb, o, d, N, k, jit, gum, shift, sched, cams, nf, nv):
    """Rays free of top-k near-ties and of ReLU kinks, from an oracle forward pass."""
    with torch.no_grad():
        _, aux = O.render_rays(ref64, aabb, o, d, N, k, jit, gum, nf, nv, density_shift=shift,
                               scene_contraction=True, schedule=sched, return_aux=True, camera_indices=cams)
        keys = O.gumbel_topk_keys(aux["p_terminates"], gum)
        srt = torch.sort(keys, dim=-1, descending=True).values
        margin = srt[:, k - 1] - srt[:, k]
        tie_free = (margin > TIE_MARGIN) | ~torch.isfinite(margin)
        mlp = ref64["mlp"]
        R = o.shape[0]
        f = aux["appearance_features"] @ mlp["Dense_0"]["kernel"]
        vd = d[:, None, :].expand(R, k, 3).reshape(-1, 3)
        x = torch.cat([f, vd, O.fourier_encode(f, nf), O.fourier_encode(vd, nv)], dim=-1)
        z1 = x @ mlp["Dense_1"]["kernel"] + mlp["Dense_1"]["bias"]
        z2 = torch.relu(z1) @ mlp["Dense_2"]["kernel"] + mlp["Dense_2"]["bias"]
    kink = torch.zeros(R * k, dtype=torch.bool)
    for z in (z1, z2):  # FiLM acts after layer 2's ReLU, so these are the only kinks
        kink |= (z.abs() < KINK_REL * float(z.pow(2).mean().sqrt())).any(dim=-1)
    kink_free = ~kink.reshape(R, k).any(dim=-1)
    return tie_free & kink_free, int((~tie_free).sum()), int((~kink_free).sum())


def test_preset_render_and_gradients_match_oracle():
    import dataclasses

    from tensorf_gb300 import cameras, render, scene, training
    _, spec = training.nerfstudio_preset(NCAM)
    spec = dataclasses.replace(spec, grid_dim=20)
    R, N, k, shift = 256, 64, 16, -1.0
    ref = _reference_params(spec, 11)
    o, d = (torch.tensor(a, dtype=torch.float32) for a in scene.unbounded_rays(R, 11))
    c = torch.tensor(np.random.default_rng(11).uniform(size=(R, 3)), dtype=torch.float32)
    cams = torch.randint(0, NCAM, (R,), generator=torch.Generator().manual_seed(12), dtype=torch.int32)
    rng = np.random.default_rng(13)
    jit = torch.tensor(rng.uniform(size=(R, N)), dtype=torch.float32)
    gum = torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32)
    aabb = torch.tensor([[-2.0] * 3, [2.0] * 3])
    sched = torch.tensor(render.contracted_schedule(0.05, 200.0, N))
    nf, nv = spec.feature_n_freqs, spec.viewdir_n_freqs

    keep, n_ties, n_kinks = _keep(_to64(ref), aabb.double(), o.double(), d.double(), N, k, jit.double(),
                                  gum.double(), shift, sched.double(), cams, nf, nv)
    print(f"{R} rays: {n_ties} near-ties, {n_kinks} with a ReLU kink")
    assert float(keep.float().mean()) >= 0.5, (n_ties, n_kinks)
    o, d, c, cams, jit = (t[keep].contiguous() for t in (o, d, c, cams, jit))

    lp = render.LearnableParams.from_reference(spec, ref, scene_contraction=True)
    rays = cameras.Rays3D(o.cuda(), d.cuda(), cams.cuda())
    noise = render.RenderNoise(jit.cuda(), gum.cuda())
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    img = render.render_rays(spec.mlp(), lp, aabb, rays, noise, cfg, density_shift=shift).cpu()
    grads = torch.zeros_like(lp.params)
    loss = float(render.loss_and_grad(lp, grads, aabb, rays, c.cuda(), noise, cfg, density_shift=shift).item())

    ref64 = _to64(ref, grad=True)
    out = O.render_rays(ref64, aabb.double(), o.double(), d.double(), N, k, jit.double(), gum.double(), nf, nv,
                        density_shift=shift, scene_contraction=True, schedule=sched.double(), camera_indices=cams)
    L = O.mse(out, c.double())
    L.backward()
    assert _rel(img, out) < RTOL, _rel(img, out)
    assert abs(loss - float(L.detach())) <= RTOL * float(L.detach()), (loss, float(L.detach()))
    g = lp.to_reference(grads)
    errs = {f"{grp}.{i}": _rel(g[grp][i], ref64[grp][i].grad) for grp in ("density", "appearance") for i in (0, 1)}
    errs.update({f"{layer}.{nm}": _rel(g["mlp"][layer][nm], ref64["mlp"][layer][nm].grad)
                 for layer in ref64["mlp"] for nm in ref64["mlp"][layer]})
    print({a: f"{b:.1e}" for a, b in errs.items()})
    assert "Embed_0.embedding" in errs
    assert max(errs.values()) < RTOL, errs


def test_preset_trains_at_its_own_sizes():
    """The preset's grid (128^3), batch (2048 rays) and sample counts (665 / 99) on the
    unbounded sphere scene, each ray seen by one of NCAM cameras: the loss falls."""
    import dataclasses

    from tensorf_gb300 import cameras, scene, training
    cfg, spec = training.nerfstudio_preset(NCAM)
    cfg = dataclasses.replace(cfg, density_shift=-3.0)  # the shift the unbounded sphere scene trains with
    ts = training.TrainState.initialize(cfg, spec, seed=3)
    sc = scene.SphereScene.unbounded(3)
    rays, colors = sc.unbounded_training_rays(8 * cfg.minibatch_size, 4)
    cams = torch.randint(0, NCAM, (rays.origins.shape[0],), generator=torch.Generator().manual_seed(5),
                         dtype=torch.int32).cuda()
    mses = []
    for step in range(40):
        sl = slice((step % 8) * cfg.minibatch_size, (step % 8 + 1) * cfg.minibatch_size)
        batch = cameras.Rays3D(rays.origins[sl].contiguous(), rays.directions[sl].contiguous(), cams[sl].contiguous())
        _, log = ts.training_step(batch, colors[sl].contiguous())
        mses.append(log["train/mse"])
    assert all(np.isfinite(mses))
    assert np.mean(mses[-8:]) < 0.8 * np.mean(mses[:8]), mses
