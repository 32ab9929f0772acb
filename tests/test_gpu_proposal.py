"""GPU tests of proposal-guided sampling against the oracle's restatement of the same
design, plus a training test of what the learned proposal gains over uniform
sampling with the same number of field samples."""
import math

import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def _rel(a, b):
    a = torch.as_tensor(a.detach() if torch.is_tensor(a) else a, dtype=torch.float64).cpu()
    b = torch.as_tensor(b.detach() if torch.is_tensor(b) else b, dtype=torch.float64).cpu()
    assert a.shape == b.shape and a.numel() > 0
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


def _setup(seed=0, G=24, Gp=16, R=128, Np=32, N=24, k=8, contract=False):
    from tensorf_gb300 import render, scene
    gen = torch.Generator().manual_seed(seed)
    spec = render.ModelSpec(grid_dim=G, proposal_grid=Gp, proposal_units=64)
    ref = {"density": O.vm_init(G, 16, gen, torch.float32), "appearance": O.vm_init(G, 48, gen, torch.float32),
           "mlp": O.mlp_init(144, 2, 2, gen, dtype=torch.float32),
           "proposal": render.init_proposal(Gp, 64, gen)}
    if contract:
        o, d = scene.unbounded_rays(R, seed)
        c = np.random.default_rng(seed).uniform(size=(R, 3)).astype(np.float32)
        aabb = torch.tensor([[-2.0] * 3, [2.0] * 3])
    else:
        o, d, c = scene.sphere_rays(R, seed)
        aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    rng = np.random.default_rng(seed + 1)
    noise = {"jitter": torch.tensor(rng.uniform(size=(R, N)), dtype=torch.float32),
             "pj": torch.tensor(rng.uniform(size=(R, Np)), dtype=torch.float32),
             "gumbel": torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32)}
    return spec, ref, torch.tensor(o), torch.tensor(d), torch.tensor(c), aabb, noise


def _ref64(ref):
    out = {"density": tuple(t.double() for t in ref["density"]), "appearance": tuple(t.double() for t in ref["appearance"]),
           "mlp": {a: {b: t.double() for b, t in v.items()} for a, v in ref["mlp"].items()},
           "proposal": {a: t.double() for a, t in ref["proposal"].items()}}
    return out


def _oracle(ref64, o, d, aabb, noise, Np, N, k, shift_p, shift, contract=False, edges=None):
    e, wp, sp, X = O.proposal_forward(ref64["proposal"], o.double(), d.double(), aabb.double(), Np,
                                      noise["pj"].double(), shift_p, contract, edges)
    t, delta, bins = O.resample(e, wp, N, noise["jitter"].double())
    out, aux = O.render_explicit(ref64, aabb.double(), o.double(), d.double(), t, delta, k, noise["gumbel"].double(),
                                 density_shift=shift, contract=contract, return_aux=True)
    return out, aux, (e, wp, t, delta, bins)


def _near_tie_free(aux, k):
    keys = torch.log(aux["p_terminates"].detach()) + aux["gumbel"]
    srt = torch.sort(keys, dim=-1, descending=True).values
    if k >= keys.shape[1]:
        return torch.ones(keys.shape[0], dtype=torch.bool)
    m = srt[:, k - 1] - srt[:, k]
    return (m > 1e-5) | ~torch.isfinite(m)


@pytest.mark.parametrize("contract", [False, True])
def test_proposal_render_matches_oracle(contract):
    from tensorf_gb300 import cameras, render
    Np, N, k = 32, 24, 8
    spec, ref, o, d, c, aabb, noise = _setup(seed=3, Np=Np, N=N, k=k, contract=contract)
    lp = render.LearnableParams.from_reference(spec, ref, scene_contraction=contract)
    cfg = render.RenderConfig(0.05, 50.0, render.RenderMode.RGB, N, k)
    prop = render.ProposalConfig(samples=Np, shift=0.5, loss_weight=1.0)
    edges = torch.tensor(O.disparity_schedule(0.05, 50.0, Np + 1)) if contract else None
    rn = render.RenderNoise(noise["jitter"].cuda(), noise["gumbel"].cuda(), noise["pj"].cuda())
    out = render.render_rays(spec.mlp(), lp, aabb, cameras.Rays3D(o.cuda(), d.cuda()), rn, cfg, density_shift=-1.0,
                             proposal=prop).cpu()
    r64, aux, _ = _oracle(_ref64(ref), o, d, aabb, noise, Np, N, k, 0.5, -1.0, contract,
                          edges.double() if edges is not None else None)
    ok = _near_tie_free(aux, k)
    assert ok.float().mean() > 0.9
    assert _rel(out[ok], r64[ok]) < RTOL


def test_proposal_gradients_match_oracle():
    from tensorf_gb300 import cameras, render
    Np, N, k = 32, 24, 8
    spec, ref, o, d, c, aabb, noise = _setup(seed=5, Np=Np, N=N, k=k)
    ref64 = _ref64(ref)
    _, aux, _ = _oracle(ref64, o, d, aabb, noise, Np, N, k, 0.5, -1.0)
    ok = _near_tie_free(aux, k)
    o, d, c = o[ok], d[ok], c[ok]
    noise = {"jitter": noise["jitter"][ok], "pj": noise["pj"][ok], "gumbel": noise["gumbel"]}
    lp = render.LearnableParams.from_reference(spec, ref)
    grads = torch.zeros_like(lp.params)
    cfg = render.RenderConfig(0.05, 50.0, render.RenderMode.RGB, N, k)
    prop = render.ProposalConfig(samples=Np, shift=0.5, loss_weight=3.0)
    rn = render.RenderNoise(noise["jitter"].cuda(), noise["gumbel"].cuda(), noise["pj"].cuda())
    loss = render.loss_and_grad(lp, grads, aabb, cameras.Rays3D(o.cuda(), d.cuda()), c.cuda(), rn, cfg,
                                density_shift=-1.0, proposal=prop)
    # Oracle: MSE through the main field; bound loss through the proposal only.
    leaves = {}
    for grp in ("density", "appearance"):
        for t in ref64[grp]:
            t.requires_grad_(True)
    for v in ref64["mlp"].values():
        for t in v.values():
            t.requires_grad_(True)
    for t in ref64["proposal"].values():
        t.requires_grad_(True)
    out, aux, (e, wp, t, delta, bins) = _oracle(ref64, o, d, aabb, noise, Np, N, k, 0.5, -1.0)
    mse = O.mse(out, c.double())
    lprop = O.proposal_loss(aux["p_terminates"], wp, bins, 3.0)
    assert lprop.item() > 0.0  # the untrained proposal does not bound the field yet
    (mse + lprop).backward()
    assert abs(float(loss.item()) - float(mse.detach())) <= RTOL * float(mse.detach())
    g = lp.to_reference(grads)
    pairs = [(g["density"][0], ref64["density"][0].grad), (g["density"][1], ref64["density"][1].grad),
             (g["appearance"][0], ref64["appearance"][0].grad), (g["appearance"][1], ref64["appearance"][1].grad)]
    for layer in ref64["mlp"]:
        for nm in ref64["mlp"][layer]:
            pairs.append((g["mlp"][layer][nm], ref64["mlp"][layer][nm].grad))
    for nm in ("vector", "matrix", "w1", "b1", "w2", "b2"):
        pairs.append((g["proposal"][nm], ref64["proposal"][nm].grad))
    errs = [_rel(got, want) for got, want in pairs]
    assert max(errs) < RTOL, errs


def _psnr(a, b):
    return -10.0 * math.log10(float(((a - b) ** 2).mean()))


def test_trained_proposal_beats_uniform_sampling_at_equal_samples():
    """Train the same field twice on the sphere scene with 32 field samples per ray:
    once with uniform samples, once with samples resampled from a proposal network
    trained alongside. The proposal-guided field reaches a higher held-out PSNR."""
    from tensorf_gb300 import cameras, render, scene, training
    sc = scene.SphereScene.random(7, count=32)
    cams = sc.cameras(24, seed=8, width=200, height=200, focal=1111 / 4)
    rays, colors = sc.training_rays(cams[:20], 20 * 2048, seed=9, n_samples=2048)
    test_rays, test_colors = sc.training_rays(cams[20:], 4096, seed=10, n_samples=2048)
    N, k, R, steps = 32, 16, 2048, 600
    results = {}
    for name, prop in (("uniform", None), ("proposal", render.ProposalConfig(samples=64))):
        spec = render.ModelSpec(grid_dim=64, proposal_grid=32 if prop else 0)
        cfg = training.TrainConfig(initial_aabb_min=sc.aabb[0], initial_aabb_max=sc.aabb[1],
                                   density_samples_per_ray=N, appearance_samples_per_ray=k, n_iters=steps,
                                   upsamp_iters=(), density_shift=-3.0, proposal=prop)
        st = training.TrainState.initialize(cfg, spec, seed=1)
        nb = rays.origins.shape[0] // R
        for i in range(steps):
            j = i % nb
            st.training_step(cameras.Rays3D(rays.origins[j * R:(j + 1) * R], rays.directions[j * R:(j + 1) * R]),
                             colors[j * R:(j + 1) * R], log=False)
        rc = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
        img = render.render_rays(spec.mlp(), st.learnable_params, st.aabb, test_rays, render.NoiseKey(3), rc,
                                 density_shift=-3.0, proposal=prop)
        results[name] = _psnr(img, test_colors)
    print(results)
    assert results["proposal"] > results["uniform"] + 0.5, results


def test_bf16_proposal_gradients_align_with_fp32():
    """The BF16 model's proposal backward (tcgen05, bf16 operands) against the FP32
    model's (FP32 SIMT) on identical parameters: cosine of every proposal segment."""
    from tensorf_gb300 import cameras, render
    Np, N, k = 32, 24, 8
    spec32, ref, o, d, c, aabb, noise = _setup(seed=6, R=4096, Np=Np, N=N, k=k)  # 1024 tiles: several per CTA
    rn = render.RenderNoise(noise["jitter"].cuda(), noise["gumbel"].cuda(), noise["pj"].cuda())
    cfg = render.RenderConfig(0.05, 50.0, render.RenderMode.RGB, N, k)
    prop = render.ProposalConfig(samples=Np, shift=0.5, loss_weight=3.0)
    out = {}
    for prec in ("fp32", "bf16"):
        spec = render.ModelSpec(grid_dim=24, proposal_grid=16, proposal_units=64, precision=prec)
        lp = render.LearnableParams.from_reference(spec, ref)
        g = torch.zeros_like(lp.params)
        render.loss_and_grad(lp, g, aabb, cameras.Rays3D(o.cuda(), d.cuda()), c.cuda(), rn, cfg, density_shift=-1.0,
                             proposal=prop)
        out[prec] = lp.to_reference(g)["proposal"]
    for nm in ("vector", "matrix", "w1", "b1", "w2", "b2"):
        a, b = out["fp32"][nm].double().flatten(), out["bf16"][nm].double().flatten()
        cos = float(torch.dot(a, b) / (a.norm() * b.norm() + 1e-30))
        assert cos > 0.99, (nm, cos)
