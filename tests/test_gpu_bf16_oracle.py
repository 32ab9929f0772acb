"""BF16 mode against the CPU oracle, not against the GPU's own FP32 path.

The oracle here is a bf16-rounding mirror: FP64 arithmetic on the values the BF16
kernels actually use, rounded to bf16 at the points where those kernels round.

* Fields: the gathers read the bf16 shadow, so the mirror's density, appearance and
  proposal fields are the bf16-rounded parameters. Everything around them (sampling,
  compositing, selection, the scatter arithmetic) is FP32 on the device and FP64 here.
* FeatureMlp: the fused tcgen05 kernels round the layer inputs and weights, dZ3 and the
  back-propagated dH2 / dH1 / dH0 to bf16, and accumulate in FP32
  (test_gpu_bf16._mirror_mlp / _mirror_mlp_backward).
* Proposal forward (prop_fwd_tc_kernel): bf16 features X and weights W1 feed the
  product; b1, the ReLU, w2, b2 and the softplus stay FP32.
* Proposal backward (prop_bwd_tc_kernel): bf16 features X, weights W1, hidden units h,
  their gradient dh and the loss gradient dz feed the products; b1, w2 and the scatter
  stay FP32.

Error bound. A mirror value and a device value differ by the device's FP32 (and
tensor-core) accumulation error until one of them is rounded to bf16. Where the two
straddle a bf16 rounding boundary they round to neighbouring bf16 values, one ulp
(2^-8 to 2^-7 relative) apart, and in the FeatureMlp such a flip in an early layer
perturbs every later value of that row by a fraction of an ulp, which flips more of
them. So the device can sit up to about one bf16 ulp from the mirror, and no closer
bound holds for the chained MLP: the tests allow 2^-8 = 3.9e-3 in norm. The proposal
backward has one rounded product per operand and no chain: there the bound is 1e-4.
A missing or extra rounding point shows as an error of the size of the rounding
itself against the mirror, so each main-path tensor must also sit closer to the
mirror than to the unrounded FP64 oracle.

Rays are left out where the oracle's ReLU pre-activations lie within 1e-5 of the
layer's RMS of zero, or the top-k selection has a near-tie (as in the FP32 tests).

Config 3's FP64 finite-difference check runs on an FP32 twin of the BF16 model whose
field tensors and MLP kernels are the BF16 model's rounded values. Its FP64 loss is
the smooth loss at the point the BF16 model evaluates. Central differences of it on 64
parameters give the true gradient there, and the BF16 analytic gradient is compared
against them.
"""
import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O
from test_gpu_bf16 import _mirror_mlp, _mirror_mlp_backward

pytestmark = pytest.mark.gpu

NORM_RTOL = 2.0 ** -8       # main BF16 path: one bf16 ulp, in norm
NORM_RTOL_PROPOSAL = 1e-4    # proposal backward: no chained rounding
KINK_REL = 1e-5


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float64)


def _nrel(a, b):
    a = torch.as_tensor(a.detach() if torch.is_tensor(a) else a, dtype=torch.float64).cpu().flatten()
    b = torch.as_tensor(b.detach() if torch.is_tensor(b) else b, dtype=torch.float64).cpu().flatten()
    assert a.shape == b.shape and a.numel() > 0
    return float((a - b).norm() / (b.norm() + 1e-30))


class _MirrorMlp(torch.autograd.Function):
    """FeatureMlp with the fused BF16 kernels' rounding, forward and backward."""

    @staticmethod
    def forward(ctx, feats, dirs, w0, w1, b1, w2, b2, w3, b3):
        mlp = {"Dense_0": {"kernel": w0}, "Dense_1": {"kernel": w1, "bias": b1},
               "Dense_2": {"kernel": w2, "bias": b2}, "Dense_3": {"kernel": w3, "bias": b3}}
        ctx.save_for_backward(feats, dirs, w0, w1, b1, w2, b2, w3, b3)
        return _mirror_mlp(mlp, feats, dirs)

    @staticmethod
    def backward(ctx, grad_rgb):
        feats, dirs, w0, w1, b1, w2, b2, w3, b3 = ctx.saved_tensors
        mlp = {"Dense_0": {"kernel": w0}, "Dense_1": {"kernel": w1, "bias": b1},
               "Dense_2": {"kernel": w2, "bias": b2}, "Dense_3": {"kernel": w3, "bias": b3}}
        with torch.enable_grad():
            dx0, g = _mirror_mlp_backward(mlp, feats.detach(), dirs.detach(), grad_rgb.detach())
        return (dx0, None, g["Dense_0"]["kernel"], g["Dense_1"]["kernel"], g["Dense_1"]["bias"],
                g["Dense_2"]["kernel"], g["Dense_2"]["bias"], g["Dense_3"]["kernel"], g["Dense_3"]["bias"])


_plain_feature_mlp = O.feature_mlp


def _mirror_feature_mlp(params, features, viewdirs, nf, nv):
    assert nf == 2 and nv == 2
    p = params
    return _MirrorMlp.apply(features, viewdirs, p["Dense_0"]["kernel"], p["Dense_1"]["kernel"], p["Dense_1"]["bias"],
                            p["Dense_2"]["kernel"], p["Dense_2"]["bias"], p["Dense_3"]["kernel"],
                            p["Dense_3"]["bias"])


def _params(G, seed, proposal_grid=0):
    from tensorf_gb300 import render
    gen = torch.Generator().manual_seed(seed)
    ref = {"density": O.vm_init(G, 16, gen, torch.float32), "appearance": O.vm_init(G, 48, gen, torch.float32),
           "mlp": O.mlp_init(144, 2, 2, gen, dtype=torch.float32)}
    for lay in ("Dense_1", "Dense_2", "Dense_3"):
        ref["mlp"][lay]["bias"] = torch.randn(ref["mlp"][lay]["bias"].shape, generator=gen) * 0.1
    if proposal_grid:
        ref["proposal"] = render.init_proposal(proposal_grid, 64, gen)
        ref["proposal"]["b1"] = torch.randn(64, generator=gen) * 0.1
    return ref


def _oracle_bf16(ref, grad=False):
    """FP64 oracle parameters at the values the BF16 model evaluates: bf16 fields, MLP
    weights as given (the mirror rounds them itself)."""
    t = lambda x: x.double().requires_grad_(grad)  # noqa: E731
    out = {"density": tuple(t(_bf(x)) for x in ref["density"]),
           "appearance": tuple(t(_bf(x)) for x in ref["appearance"]),
           "mlp": {k: {n: t(x) for n, x in d.items()} for k, d in ref["mlp"].items()}}
    if "proposal" in ref:
        pr = ref["proposal"]
        out["proposal"] = {"vector": t(_bf(pr["vector"])), "matrix": t(_bf(pr["matrix"])),
                           **{n: t(pr[n]) for n in ("w1", "b1", "w2", "b2")}}
    return out


def _kink_free_rows(mlp, feats, dirs):
    """Rows whose mirror pre-activations (bf16 layer inputs) all lie clear of zero."""
    with torch.no_grad():
        W = {k: {n: x.detach() for n, x in d.items()} for k, d in mlp.items()}
        h0 = _bf(feats) @ _bf(W["Dense_0"]["kernel"])
        x1 = torch.cat([h0, dirs, O.fourier_encode(h0, 2), O.fourier_encode(dirs, 2)], -1)
        z1 = _bf(x1) @ _bf(W["Dense_1"]["kernel"]) + W["Dense_1"]["bias"]
        z2 = _bf(torch.relu(z1)) @ _bf(W["Dense_2"]["kernel"]) + W["Dense_2"]["bias"]
    ok = torch.ones(feats.shape[0], dtype=torch.bool)
    for z in (z1, z2):
        ok &= ~(z.abs() < KINK_REL * float(z.pow(2).mean().sqrt())).any(-1)
    return ok


def test_bf16_render_and_gradients_match_rounding_mirror(monkeypatch):
    """BF16 render, loss and every gradient segment at G=64, N=256, top-64 (the
    pair-merging scatter kernels and the fused tcgen05 MLP) against the mirror."""
    from tensorf_gb300 import cameras, render, scene
    monkeypatch.setattr(O, "feature_mlp", _mirror_feature_mlp)
    G, R, N, k, shift = 64, 256, 256, 64, -1.0
    ref = _params(G, 21)
    o, d, c = (torch.tensor(a) for a in scene.sphere_rays(R, 21))
    rng = np.random.default_rng(21)
    jit = torch.tensor(rng.uniform(size=N), dtype=torch.float32)
    gum = torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    with torch.no_grad():
        _, aux = O.render_rays(_oracle_bf16(ref), aabb.double(), o.double(), d.double(), N, k, jit.double(),
                               gum.double(), density_shift=shift, return_aux=True)
    keys = O.gumbel_topk_keys(aux["p_terminates"], gum.double())
    srt = torch.sort(keys, dim=-1, descending=True).values
    margin = srt[:, k - 1] - srt[:, k]
    keep = (margin > 1e-5) | ~torch.isfinite(margin)
    vd = d.double()[:, None, :].expand(R, k, 3).reshape(-1, 3)
    keep &= _kink_free_rows(_oracle_bf16(ref)["mlp"], aux["appearance_features"], vd).reshape(R, k).all(-1)
    print(f"kept {int(keep.sum())} of {R} rays")
    assert float(keep.float().mean()) > 0.8
    o, d, c = o[keep].contiguous(), d[keep].contiguous(), c[keep].contiguous()

    spec = render.ModelSpec(grid_dim=G, precision="bf16")
    lp = render.LearnableParams.from_reference(spec, ref)
    rays = cameras.Rays3D(o.cuda(), d.cuda())
    noise = render.RenderNoise(jit.cuda(), gum.cuda())
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    img = render.render_rays(spec.mlp(), lp, aabb, rays, noise, cfg, density_shift=shift).cpu()
    grads = torch.zeros_like(lp.params)
    loss = float(render.loss_and_grad(lp, grads, aabb, rays, c.cuda(), noise, cfg, density_shift=shift).item())

    def oracle_grads():
        ref64 = _oracle_bf16(ref, grad=True)
        out = O.render_rays(ref64, aabb.double(), o.double(), d.double(), N, k, jit.double(), gum.double(),
                            density_shift=shift)
        L = O.mse(out, c.double())
        L.backward()
        gr = {f"{grp}.{nm}": ref64[grp][i].grad for grp in ("density", "appearance")
              for i, nm in enumerate(("vector", "matrix"))}
        gr.update({f"{layer}.{nm}": ref64["mlp"][layer][nm].grad for layer in ref64["mlp"] for nm in ref64["mlp"][layer]})
        return out, L, gr

    out, L, want = oracle_grads()
    with monkeypatch.context() as mp:  # the same oracle with an unrounded FP64 FeatureMlp
        mp.setattr(O, "feature_mlp", _plain_feature_mlp)
        _, _, want_plain = oracle_grads()
    g = lp.to_reference(grads)
    got = {f"{grp}.{nm}": g[grp][i] for grp in ("density", "appearance") for i, nm in enumerate(("vector", "matrix"))}
    got.update({f"{layer}.{nm}": g["mlp"][layer][nm] for layer in g["mlp"] for nm in g["mlp"][layer]})
    errs = {"render": _nrel(img, out), "loss": abs(loss - float(L.detach())) / float(L.detach())}
    errs.update({name: _nrel(got[name], want[name]) for name in want})
    plain = {name: _nrel(got[name], want_plain[name]) for name in want}
    print("vs mirror", {k_: f"{v:.1e}" for k_, v in errs.items()})
    print("vs unrounded MLP", {k_: f"{v:.1e}" for k_, v in plain.items()})
    assert max(errs.values()) < NORM_RTOL, errs
    mlp_side = [n for n in want if n.startswith("Dense") or n.startswith("appearance")]
    assert all(errs[n] < plain[n] for n in mlp_side), (errs, plain)


def _proposal_features(prop, o, d, aabb, Np, pj):
    """Bin edges, lengths, and the 16 proposal MLP inputs (FP64) of every bin."""
    e = O.proposal_edges(o, d, aabb, Np)
    length = e[:, 1:] - e[:, :-1]
    t = e[:, :-1] + pj * length
    x = O.normalize_points((o[:, None, :] + d[:, None, :] * t[:, :, None]).permute(2, 0, 1), aabb)
    feats = O.vm_interpolate(prop["vector"].detach(), prop["matrix"].detach(), x).permute(1, 2, 0)
    xp = x.permute(1, 2, 0)
    return e, length, torch.cat([feats, xp, xp.abs().amax(-1, keepdim=True)], -1)


def _proposal_forward_bf16(prop, o, d, aabb, Np, pj, shift_p):
    """prop_fwd_tc_kernel's forward: bin edges and proposal weights from the bf16
    product of X and W1, the rest in FP64."""
    with torch.no_grad():
        e, length, X = _proposal_features(prop, o, d, aabb, Np, pj)
        w1, b1, w2, b2 = (prop[n].detach() for n in ("w1", "b1", "w2", "b2"))
        z = (torch.relu(_bf(X) @ _bf(w1) + b1) @ w2)[..., 0] + b2[0]
        _, wp = O.compute_segment_probabilities(O.softplus(z + shift_p), length)
    return e, wp


def _proposal_mirror_grads(prop, o, d, aabb, Np, pj, shift_p, w_main, bins, loss_w):
    """Gradients of the proposal bound loss with the tensor-core kernels' rounding. prop:
    FP64 proposal parameters with bf16-rounded fields. The forward (and so dz) uses the
    bf16 product of X and W1, as prop_fwd_tc_kernel does."""
    e = O.proposal_edges(o, d, aabb, Np)
    length = e[:, 1:] - e[:, :-1]
    t = e[:, :-1] + pj * length
    pts = o[:, None, :] + d[:, None, :] * t[:, :, None]
    x = O.normalize_points(pts.permute(2, 0, 1), aabb)
    vec = prop["vector"].detach().clone().requires_grad_(True)
    mat = prop["matrix"].detach().clone().requires_grad_(True)
    feats = O.vm_interpolate(vec, mat, x).permute(1, 2, 0)
    xp = x.permute(1, 2, 0)
    X = torch.cat([feats.detach(), xp, xp.abs().amax(-1, keepdim=True)], -1)
    w1, b1, w2, b2 = (prop[n].detach() for n in ("w1", "b1", "w2", "b2"))
    Xb, W1b = _bf(X), _bf(w1)
    pre = Xb @ W1b + b1
    h = torch.relu(pre)
    z = ((h @ w2)[..., 0] + b2[0]).requires_grad_(True)
    _, wp = O.compute_segment_probabilities(O.softplus(z + shift_p), length)
    lprop = O.proposal_loss(w_main, wp, bins, loss_w)
    (dz,) = torch.autograd.grad(lprop, z)
    dh = dz[..., None] * w2[:, 0] * (h > 0)
    Hb, dHb, dzb = _bf(h), _bf(dh), _bf(dz)
    dX = dHb @ W1b.T
    feats.backward(dX[..., :12])
    grads = {"vector": vec.grad, "matrix": mat.grad,
             "w1": Xb.reshape(-1, 16).T @ dHb.reshape(-1, 64),
             "b1": dHb.reshape(-1, 64).sum(0),
             "w2": (Hb * dzb[..., None]).reshape(-1, 64).sum(0)[:, None],
             "b2": dz.sum().reshape(1)}
    kink = (pre.abs() < KINK_REL * float(pre.pow(2).mean().sqrt())).any(-1).any(-1)
    return grads, ~kink


def test_bf16_proposal_backward_matches_rounding_mirror(monkeypatch):
    """prop_bwd_tc_kernel (tcgen05, bf16 operands) on 4096 rays x 32 proposal bins, so
    every CTA accumulates several tiles in TMEM: field and weight gradients of the
    proposal against the mirror."""
    from tensorf_gb300 import cameras, render, scene
    monkeypatch.setattr(O, "feature_mlp", _mirror_feature_mlp)
    G, Gp, R, Np, N, k, shift, shift_p, lw = 24, 16, 4096, 32, 24, 8, -1.0, 0.5, 3.0
    ref = _params(G, 31, proposal_grid=Gp)
    o, d, c = (torch.tensor(a) for a in scene.sphere_rays(R, 31))
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    rng = np.random.default_rng(32)
    jit = torch.tensor(rng.uniform(size=(R, N)), dtype=torch.float32)
    pj = torch.tensor(rng.uniform(size=(R, Np)), dtype=torch.float32)
    gum = torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32)

    def mirror(o_, d_, jit_, pj_):
        r64 = _oracle_bf16(ref)
        with torch.no_grad():
            e, wp = _proposal_forward_bf16(r64["proposal"], o_.double(), d_.double(), aabb.double(), Np,
                                           pj_.double(), shift_p)
            t, delta, bins = O.resample(e, wp, N, jit_.double())
            _, aux = O.render_explicit(r64, aabb.double(), o_.double(), d_.double(), t, delta, k, gum.double(),
                                       density_shift=shift, return_aux=True)
        return _proposal_mirror_grads(r64["proposal"], o_.double(), d_.double(), aabb.double(), Np, pj_.double(),
                                      shift_p, aux["p_terminates"], bins, lw * o_.shape[0] / R)

    _, keep = mirror(o, d, jit, pj)
    print(f"kept {int(keep.sum())} of {R} rays")
    assert float(keep.float().mean()) > 0.8
    o, d, c, jit, pj = (t_[keep].contiguous() for t_ in (o, d, c, jit, pj))
    want, _ = mirror(o, d, jit, pj)

    spec = render.ModelSpec(grid_dim=G, proposal_grid=Gp, proposal_units=64, precision="bf16")
    lp = render.LearnableParams.from_reference(spec, ref)
    grads = torch.zeros_like(lp.params)
    cfg = render.RenderConfig(0.05, 50.0, render.RenderMode.RGB, N, k)
    prop = render.ProposalConfig(samples=Np, shift=shift_p, loss_weight=lw * o.shape[0] / R)
    rn = render.RenderNoise(jit.cuda(), gum.cuda(), pj.cuda())
    render.loss_and_grad(lp, grads, aabb, cameras.Rays3D(o.cuda(), d.cuda()), c.cuda(), rn, cfg, density_shift=shift,
                         proposal=prop)
    got = lp.to_reference(grads)["proposal"]
    errs = {nm: _nrel(got[nm], want[nm]) for nm in ("vector", "matrix", "w1", "b1", "w2", "b2")}
    print({k_: f"{v:.1e}" for k_, v in errs.items()})
    assert max(errs.values()) < NORM_RTOL_PROPOSAL, errs


def test_bf16_gradients_against_fp64_finite_differences():
    """Config 3's check: the BF16 model's analytic gradient on 64 parameters (over both
    VMs and every MLP tensor) against FP64 central differences of the loss at the
    bf16-rounded point, evaluated on the device by tvm_loss_f64."""
    from tensorf_gb300 import cameras, render, scene
    G, R, N = 16, 64, 32
    H = 1e-6
    ref = _params(G, 41)
    rounded = {"density": tuple(_bf(x).float() for x in ref["density"]),
               "appearance": tuple(_bf(x).float() for x in ref["appearance"]),
               "mlp": {k: {n: (_bf(x).float() if n == "kernel" else x.clone()) for n, x in dd.items()}
                       for k, dd in ref["mlp"].items()}}
    lp16 = render.LearnableParams.from_reference(render.ModelSpec(grid_dim=G, precision="bf16"), ref)
    lp32 = render.LearnableParams.from_reference(render.ModelSpec(grid_dim=G), rounded)
    o, d, c = scene.sphere_rays(R, 41)
    rays = cameras.Rays3D(torch.tensor(o).cuda(), torch.tensor(d).cuda())
    colors = torch.tensor(c).cuda()
    rng = np.random.default_rng(42)
    noise = render.RenderNoise(torch.tensor(rng.uniform(size=N), dtype=torch.float32).cuda(),
                               torch.zeros(N, dtype=torch.float32).cuda())
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    cfg = render.RenderConfig(0.05, 50.0, render.RenderMode.RGB, N, N)
    grads = torch.zeros_like(lp16.params)
    render.loss_and_grad(lp16, grads, aabb, rays, colors, noise, cfg, density_shift=-1.0)
    g = grads.cpu().double()
    L = lp16.layout
    groups = [(L.density_lines, L.appearance_lines, 16), (L.appearance_lines, L.mlp_begin, 16),
              (L.mlp_w0, L.mlp_w1, 6), (L.mlp_w1, L.mlp_b1, 6), (L.mlp_b1, L.mlp_w2, 4), (L.mlp_w2, L.mlp_b2, 6),
              (L.mlp_b2, L.mlp_w3, 4), (L.mlp_w3, L.mlp_b3, 4), (L.mlp_b3, L.mlp_b3 + 3, 2)]
    sel = np.random.default_rng(43)
    idx = []
    for lo, hi, n in groups:
        seg = g[lo:hi].abs()
        cand = torch.nonzero(seg > seg.max() * 1e-2).flatten().numpy() + lo
        idx += list(sel.choice(cand, size=min(n, len(cand)), replace=False))
    assert len(idx) == 64
    fd = []
    for i in idx:
        lp_ = render.loss_f64(lp32, aabb, rays, colors, noise, cfg, density_shift=-1.0, perturb_index=int(i),
                              perturb_delta=H)
        lm_ = render.loss_f64(lp32, aabb, rays, colors, noise, cfg, density_shift=-1.0, perturb_index=int(i),
                              perturb_delta=-H)
        fd.append((lp_ - lm_) / (2 * H))
    fd = torch.tensor(fd, dtype=torch.float64)
    an = g[torch.tensor(idx)]
    err = (fd - an).abs() / torch.maximum(an.abs(), torch.full_like(an, 1e-2 * float(an.abs().max())))
    cos = float(torch.dot(fd, an) / (fd.norm() * an.norm()))
    print("bf16 vs fd64: median", float(err.median()), "max", float(err.max()), "cosine", cos)
    # bf16 activations carry 2^-9 relative rounding each; a handful of them on every
    # path keeps the analytic gradient within a few percent of the true one.
    assert float(err.median()) < 1e-2 and float(err.max()) < 5e-2, (float(err.median()), float(err.max()))
    assert cos > 0.999
