"""The proposal network's standalone seams (tvm_proposal_fwd, tvm_proposal_resample,
tvm_proposal_loss, tvm_proposal_bwd) against the oracle's restatement of each stage,
and composed, against the fused training pass that runs the same stages inside
tvm_loss_and_grad.

Tolerances: FP32 results against FP64 at 1e-4 of the largest magnitude (as the other
parity tests); resampled bin indices exactly, but for entries whose quantile target
lies within FP32 rounding of a histogram edge (the sample distance agrees there, as the
two neighbouring bins meet at that edge); the BF16 model's tensor-core backward against
the bf16-rounding mirror at 1e-4 in norm.
"""
import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O
from test_gpu_proposal import _ref64, _rel, _setup

pytestmark = pytest.mark.gpu

RTOL = 1e-4
NP, N, K = 32, 24, 8
SHIFT_P = 0.5


def _case(contract, seed=3, R=128):
    from tensorf_gb300 import cameras, render
    spec, ref, o, d, c, aabb, noise = _setup(seed=seed, R=R, Np=NP, N=N, k=K, contract=contract)
    lp = render.LearnableParams.from_reference(spec, ref, scene_contraction=contract)
    edges = torch.tensor(O.disparity_schedule(0.05, 50.0, NP + 1)) if contract else None
    prop = render.ProposalConfig(samples=NP, shift=SHIFT_P, loss_weight=2.0)
    rays = cameras.Rays3D(o.cuda(), d.cuda())
    return spec, ref, lp, rays, (o, d, c), aabb, noise, edges, prop


@pytest.mark.parametrize("contract", [False, True])
def test_proposal_forward_seam_matches_oracle(contract):
    from tensorf_gb300 import render
    spec, ref, lp, rays, (o, d, c), aabb, noise, edges, prop = _case(contract)
    sig, dl = render.proposal_forward(lp, aabb, rays, noise["pj"].cuda(), prop,
                                      edges.cuda() if edges is not None else None)
    wp = render.compute_segment_probabilities(sig, dl).p_terminates
    e, w64, s64, _ = O.proposal_forward(_ref64(ref)["proposal"], o.double(), d.double(), aabb.double(), NP,
                                        noise["pj"].double(), SHIFT_P, contract,
                                        edges.double() if edges is not None else None)
    assert sig.shape == dl.shape == (o.shape[0], NP)
    assert _rel(sig, s64) < RTOL
    assert _rel(dl, e[:, 1:] - e[:, :-1]) < RTOL
    assert _rel(wp, w64) < RTOL


@pytest.mark.parametrize("contract", [False, True])
def test_proposal_resample_seam_matches_oracle(contract):
    from tensorf_gb300 import render
    spec, ref, lp, rays, (o, d, c), aabb, noise, edges, prop = _case(contract, seed=8, R=512)
    e, w64, _, _ = O.proposal_forward(_ref64(ref)["proposal"], o.double(), d.double(), aabb.double(), NP,
                                      noise["pj"].double(), SHIFT_P, contract,
                                      edges.double() if edges is not None else None)
    w32 = w64.float()  # both sides resample the same FP32 weights
    ts, dl, bins = render.proposal_resample(rays, aabb, w32.cuda(), noise["jitter"].cuda(), N, prop, contract,
                                            edges.cuda() if edges is not None else None)
    t64, d64, b64 = O.resample(e, w32.double(), N, noise["jitter"].double())
    assert ts.shape == dl.shape == (o.shape[0], N) and bins.shape == (o.shape[0], N + 1)
    assert bins.dtype == torch.int32
    same = bins.cpu().long() == b64
    assert float(same.float().mean()) > 0.995, float(same.float().mean())
    assert _rel(ts, t64) < RTOL
    assert _rel(dl, d64) < RTOL
    # Every interval lies inside the ray's bins and the intervals tile them in order.
    assert bool((bins[:, 1:] >= bins[:, :-1]).all()) and int(bins.min()) >= 0 and int(bins.max()) < NP
    assert bool((dl >= 0).all())


def test_proposal_loss_seam_matches_oracle():
    from tensorf_gb300 import render
    R = 300
    rng = np.random.default_rng(5)
    wp = rng.dirichlet(np.full(NP + 1, 0.3), size=R)[:, :NP]       # rows summing to < 1
    wm = rng.dirichlet(np.full(N + 1, 0.3), size=R)[:, :N]
    b = np.sort(rng.integers(0, NP, size=(R, N + 1)), axis=1)
    b[:, 0], b[:, -1] = 0, NP - 1
    wp_t = torch.tensor(wp, dtype=torch.float32)
    wm_t = torch.tensor(wm, dtype=torch.float32)
    b_t = torch.tensor(b, dtype=torch.int32)
    weight = 3.0
    loss, g = render.proposal_loss(wm_t.cuda(), wp_t.cuda(), b_t.cuda(), weight / R)
    wp64 = wp_t.double().requires_grad_(True)
    want = O.proposal_loss(wm_t.double(), wp64, b_t.long(), weight)
    want.backward()
    assert float(want.detach()) > 0.0
    assert abs(float(loss.item()) - float(want.detach())) <= RTOL * float(want.detach())
    assert _rel(g, wp64.grad) < RTOL


def _oracle_backward(ref, o, d, aabb, pj, gs, contract, edges):
    """Gradient of sum(sigma * gs) over the proposal's parameters, in FP64."""
    prop = {k: v.double() for k, v in ref["proposal"].items()}
    for t in prop.values():
        t.requires_grad_(True)
    _, _, sig, _ = O.proposal_forward(prop, o.double(), d.double(), aabb.double(), NP, pj.double(), SHIFT_P,
                                      contract, edges.double() if edges is not None else None)
    (sig * gs.double()).sum().backward()
    return {k: v.grad for k, v in prop.items()}


@pytest.mark.parametrize("contract", [False, True])
def test_proposal_backward_seam_matches_oracle(contract):
    from tensorf_gb300 import render
    spec, ref, lp, rays, (o, d, c), aabb, noise, edges, prop = _case(contract, seed=11)
    ed = edges.cuda() if edges is not None else None
    sig, _ = render.proposal_forward(lp, aabb, rays, noise["pj"].cuda(), prop, ed)
    gs = torch.tensor(np.random.default_rng(12).normal(size=(o.shape[0], NP)), dtype=torch.float32)
    grads = torch.zeros_like(lp.params)
    render.proposal_backward(lp, grads, aabb, rays, noise["pj"].cuda(), prop, sig, gs.cuda(), ed)
    got = lp.to_reference(grads)
    want = _oracle_backward(ref, o, d, aabb, noise["pj"], gs, contract, edges)
    errs = {nm: _rel(got["proposal"][nm], want[nm]) for nm in ("vector", "matrix", "w1", "b1", "w2", "b2")}
    assert max(errs.values()) < RTOL, errs
    # Only the proposal's segments are touched.
    lay = lp.layout
    assert float(grads[:lay.proposal_lines].abs().max()) == 0.0
    # Accumulates: a second call doubles every gradient.
    once = grads.clone()
    render.proposal_backward(lp, grads, aabb, rays, noise["pj"].cuda(), prop, sig, gs.cuda(), ed)
    assert _rel(grads, 2.0 * once) < 1e-5


def _near_bf16_midpoint(v, rel=1e-5):
    """Values within ``rel`` of a bf16 rounding midpoint, where FP32 and FP64 inputs
    may round to neighbouring bf16 values."""
    return (v * (1 + rel)).to(torch.bfloat16) != (v * (1 - rel)).to(torch.bfloat16)


def test_bf16_proposal_backward_seam_matches_rounding_mirror():
    """The BF16 model's seam runs the tcgen05 backward (bf16 X, W1, h, dh and dz
    operands). Mirror: the FP64 gradient with the kernel's roundings, dz = gs *
    sigmoid(z + shift) with z from the bf16 product of X and W1 on the bf16 fields, as
    the tensor-core forward computes it.

    Every sample here has a gradient, so the sums cancel and a single operand that
    rounds to the other bf16 neighbour on the device (an FP32 input within its rounding
    error of a midpoint), or a ReLU mask that flips with it, shows above the tolerance.
    Such samples get a zero gradient: hidden pre-activations within 1e-5 of their RMS
    of zero, and features X or products dh within 1e-5 of a bf16 midpoint."""
    from tensorf_gb300 import cameras, render, scene
    from test_gpu_bf16_oracle import KINK_REL, NORM_RTOL_PROPOSAL, _bf, _nrel, _oracle_bf16, _params
    G, Gp, R = 24, 16, 4096  # 1024 tiles: several per CTA
    ref = _params(G, 41, proposal_grid=Gp)
    o, d, _ = (torch.tensor(a) for a in scene.sphere_rays(R, 41))
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    rng = np.random.default_rng(42)
    pj = torch.tensor(rng.uniform(size=(R, NP)), dtype=torch.float32)
    gs = torch.tensor(rng.normal(size=(R, NP)), dtype=torch.float32)

    p64 = _oracle_bf16(ref)["proposal"]
    o64, d64, a64 = o.double(), d.double(), aabb.double()
    e = O.proposal_edges(o64, d64, a64, NP)
    t = e[:, :-1] + pj.double() * (e[:, 1:] - e[:, :-1])
    x = O.normalize_points((o64[:, None, :] + d64[:, None, :] * t[:, :, None]).permute(2, 0, 1), a64)
    vec = p64["vector"].detach().clone().requires_grad_(True)
    mat = p64["matrix"].detach().clone().requires_grad_(True)
    feats = O.vm_interpolate(vec, mat, x).permute(1, 2, 0)
    xp = x.permute(1, 2, 0)
    X = torch.cat([feats.detach(), xp, xp.abs().amax(-1, keepdim=True)], -1)
    w1, b1, w2, b2 = (p64[n].detach() for n in ("w1", "b1", "w2", "b2"))
    Xb, W1b = _bf(X), _bf(w1)
    pre = Xb @ W1b + b1
    h = torch.relu(pre)
    sgm = torch.sigmoid((h @ w2)[..., 0] + b2[0] + SHIFT_P)
    dh = (gs.double() * sgm)[..., None] * w2[:, 0] * (h > 0)
    drop = _near_bf16_midpoint(X).any(-1) | _near_bf16_midpoint(dh).any(-1)
    drop |= (pre.abs() < KINK_REL * float(pre.pow(2).mean().sqrt())).any(-1)
    print(f"dropped {float(drop.float().mean()):.3f} of the samples")
    assert float(drop.float().mean()) < 0.5
    gs[drop] = 0.0

    spec = render.ModelSpec(grid_dim=G, proposal_grid=Gp, proposal_units=64, precision="bf16")
    lp = render.LearnableParams.from_reference(spec, ref)
    prop = render.ProposalConfig(samples=NP, shift=SHIFT_P)
    rays = cameras.Rays3D(o.cuda(), d.cuda())
    sig, _ = render.proposal_forward(lp, aabb, rays, pj.cuda(), prop)
    grads = torch.zeros_like(lp.params)
    render.proposal_backward(lp, grads, aabb, rays, pj.cuda(), prop, sig, gs.cuda())
    got = lp.to_reference(grads)["proposal"]

    dz = gs.double() * sgm
    dh = dz[..., None] * w2[:, 0] * (h > 0)
    Hb, dHb, dzb = _bf(h), _bf(dh), _bf(dz)
    feats.backward((dHb @ W1b.T)[..., :12])
    want = {"vector": vec.grad, "matrix": mat.grad, "w1": Xb.reshape(-1, 16).T @ dHb.reshape(-1, 64),
            "b1": dHb.reshape(-1, 64).sum(0), "w2": (Hb * dzb[..., None]).reshape(-1, 64).sum(0)[:, None],
            "b2": dz.sum().reshape(1)}
    errs = {nm: _nrel(got[nm], want[nm]) for nm in want}
    print({k_: f"{v:.1e}" for k_, v in errs.items()})
    assert max(errs.values()) < NORM_RTOL_PROPOSAL, errs


@pytest.mark.parametrize("contract", [False, True])
def test_proposal_seams_compose_to_the_fused_pass(contract):
    """fwd -> composite -> resample -> (main weights) -> loss -> composite bwd -> bwd
    gives the proposal gradients tvm_loss_and_grad computes in one pass (the MSE does
    not reach the proposal, so its segments hold the bound loss's gradient alone)."""
    from tensorf_gb300 import render
    spec, ref, lp, rays, (o, d, c), aabb, noise, edges, prop = _case(contract, seed=17, R=256)
    ed = edges.cuda() if edges is not None else None
    pj, jit = noise["pj"].cuda(), noise["jitter"].cuda()
    fused = torch.zeros_like(lp.params)
    cfg = render.RenderConfig(0.05, 50.0, render.RenderMode.RGB, N, K)
    rn = render.RenderNoise(jit, noise["gumbel"].cuda(), pj)
    render.loss_and_grad(lp, fused, aabb, rays, c.cuda(), rn, cfg, density_shift=-1.0, schedule=ed, proposal=prop)

    sig, dl = render.proposal_forward(lp, aabb, rays, pj, prop, ed)
    wp = render.compute_segment_probabilities(sig, dl).p_terminates
    ts, deltas, bins = render.proposal_resample(rays, aabb, wp, jit, N, prop, contract, ed)
    # The main field's weights at the resampled points, from the oracle in FP64.
    _, aux = O.render_explicit(_ref64(ref), aabb.double(), o.double(), d.double(), ts.cpu().double(),
                               deltas.cpu().double(), K, noise["gumbel"].double(), density_shift=-1.0,
                               contract=contract, return_aux=True)
    wm = aux["p_terminates"].detach().float().cuda()
    _, g_wp = render.proposal_loss(wm, wp, bins, prop.loss_weight / o.shape[0])
    g_sig = torch.empty_like(sig)
    from tensorf_gb300 import _lib
    from tensorf_gb300._util import ptr, stream_handle
    _lib.call("tvm_composite_bwd", ptr(sig), ptr(dl), sig.shape[0], NP, ptr(None), ptr(g_wp), ptr(g_sig),
              stream_handle())
    seams = torch.zeros_like(lp.params)
    render.proposal_backward(lp, seams, aabb, rays, pj, prop, sig, g_sig, ed)
    a = lp.to_reference(fused)["proposal"]
    b = lp.to_reference(seams)["proposal"]
    errs = {nm: _rel(b[nm], a[nm]) for nm in ("vector", "matrix", "w1", "b1", "w2", "b2")}
    assert max(errs.values()) < RTOL, errs
