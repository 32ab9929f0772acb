"""FP64 central finite differences on the device against the FP32 analytic gradients
(tvm_loss_and_grad) on 64 parameters spread over the density VM, the appearance VM and
every FeatureMlp layer. Every sample reaches the appearance path (k = N), so the loss
is smooth in the parameters. The FP64 loss itself is checked against the oracle's FP64
restatement."""
import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu

G, R, N = 16, 64, 32
H = 1e-6           # finite-difference step: small enough to cross no ReLU kink, FP64 keeps it exact
TOL = 1e-4         # per-parameter |fd - analytic| / max(|analytic|, 1% of the largest)


def _problem(seed=0):
    from tensorf_gb300 import cameras, render, scene
    gen = torch.Generator().manual_seed(seed)
    ref = {"density": O.vm_init(G, 16, gen, torch.float32), "appearance": O.vm_init(G, 48, gen, torch.float32),
           "mlp": O.mlp_init(144, 2, 2, gen, dtype=torch.float32)}
    for lay in ("Dense_1", "Dense_2", "Dense_3"):
        ref["mlp"][lay]["bias"] = torch.randn(ref["mlp"][lay]["bias"].shape, generator=gen) * 0.1
    spec = render.ModelSpec(grid_dim=G)
    lp = render.LearnableParams.from_reference(spec, ref)
    o, d, c = scene.sphere_rays(R, seed)
    rays = cameras.Rays3D(torch.tensor(o).cuda(), torch.tensor(d).cuda())
    rng = np.random.default_rng(seed + 1)
    noise = render.RenderNoise(torch.tensor(rng.uniform(size=N), dtype=torch.float32).cuda(),
                               torch.zeros(N, dtype=torch.float32).cuda())
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    cfg = render.RenderConfig(0.05, 50.0, render.RenderMode.RGB, N, N)
    return ref, lp, rays, torch.tensor(c).cuda(), noise, aabb, cfg


def test_fp64_loss_matches_oracle():
    from tensorf_gb300 import render
    ref, lp, rays, colors, noise, aabb, cfg = _problem(1)
    got = render.loss_f64(lp, aabb, rays, colors, noise, cfg, density_shift=-1.0)
    r64 = {"density": tuple(t.double() for t in ref["density"]), "appearance": tuple(t.double() for t in ref["appearance"]),
           "mlp": {a: {b: t.double() for b, t in v.items()} for a, v in ref["mlp"].items()}}
    out = O.render_rays(r64, aabb.double(), rays.origins.cpu().double(), rays.directions.cpu().double(), N, N,
                        noise.jitter.cpu().double(), torch.zeros(N, dtype=torch.float64), density_shift=-1.0)
    want = float(O.mse(out, colors.cpu().double()))
    assert abs(got - want) <= 1e-9 * want, (got, want)


def test_fp64_finite_differences_match_fp32_gradients():
    from tensorf_gb300 import render
    ref, lp, rays, colors, noise, aabb, cfg = _problem(2)
    grads = torch.zeros_like(lp.params)
    render.loss_and_grad(lp, grads, aabb, rays, colors, noise, cfg, density_shift=-1.0)
    g = grads.cpu().double()
    L = lp.layout
    groups = [(L.density_lines, L.appearance_lines, 16), (L.appearance_lines, L.mlp_begin, 16),
              (L.mlp_w0, L.mlp_w1, 6), (L.mlp_w1, L.mlp_b1, 6), (L.mlp_b1, L.mlp_w2, 4), (L.mlp_w2, L.mlp_b2, 6),
              (L.mlp_b2, L.mlp_w3, 4), (L.mlp_w3, L.mlp_b3, 4), (L.mlp_b3, L.mlp_b3 + 3, 2)]
    rng = np.random.default_rng(3)
    idx = []
    for lo, hi, n in groups:
        seg = g[lo:hi].abs()
        cand = torch.nonzero(seg > seg.max() * 1e-2).flatten().numpy() + lo  # parameters the loss depends on
        idx += list(rng.choice(cand, size=min(n, len(cand)), replace=False))
    assert len(idx) == 64
    fd = []
    for i in idx:
        lp_ = render.loss_f64(lp, aabb, rays, colors, noise, cfg, density_shift=-1.0, perturb_index=int(i),
                              perturb_delta=H)
        lm_ = render.loss_f64(lp, aabb, rays, colors, noise, cfg, density_shift=-1.0, perturb_index=int(i),
                              perturb_delta=-H)
        fd.append((lp_ - lm_) / (2 * H))
    fd = torch.tensor(fd, dtype=torch.float64)
    an = g[torch.tensor(idx)]
    err = (fd - an).abs() / torch.maximum(an.abs(), torch.full_like(an, 1e-2 * float(an.abs().max())))
    print("fd64: median", float(err.median()), "max", float(err.max()))
    assert float(err.max()) < TOL, (float(err.max()), int(err.argmax()))
