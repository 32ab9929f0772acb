"""GPU tests of the BF16 path: the fused tcgen05 FeatureMlp forward against a CPU
reference that rounds to bf16 at the same points, and the BF16 render / gradients
against the FP32 path on identical parameters."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float64)


def _mirror_mlp(mlp, feats, dirs):
    """FeatureMlp with bf16-rounded layer inputs and weights, fp64 accumulation."""
    h0 = _bf(feats) @ _bf(mlp["Dense_0"]["kernel"])
    x1 = torch.cat([h0, dirs, O.fourier_encode(h0, 2), O.fourier_encode(dirs, 2)], -1)
    h1 = torch.relu(_bf(x1) @ _bf(mlp["Dense_1"]["kernel"]) + mlp["Dense_1"]["bias"])
    h2 = torch.relu(_bf(h1) @ _bf(mlp["Dense_2"]["kernel"]) + mlp["Dense_2"]["bias"])
    return torch.sigmoid(_bf(h2) @ _bf(mlp["Dense_3"]["kernel"]) + mlp["Dense_3"]["bias"])


def _params(G, seed):
    gen = torch.Generator().manual_seed(seed)
    mlp = O.mlp_init(144, 2, 2, gen, dtype=torch.float64)
    for lay in ("Dense_1", "Dense_2", "Dense_3"):
        mlp[lay]["bias"] = torch.randn(mlp[lay]["bias"].shape, generator=gen, dtype=torch.float64) * 0.1
    return {"density": O.vm_init(G, 16, gen, torch.float32), "appearance": O.vm_init(G, 48, gen, torch.float32),
            "mlp": {a: {b: t.float() for b, t in v.items()} for a, v in mlp.items()}}


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 40000])
def test_fused_bf16_mlp_matches_mirror(n):
    from tensorf_gb300 import _lib, render
    spec = render.ModelSpec(grid_dim=8, precision="bf16")
    ref = _params(8, 1)
    lp = render.LearnableParams.from_reference(spec, ref)
    gen = torch.Generator().manual_seed(n)
    feats = torch.randn((n, 144), generator=gen) * 0.3
    dirs = torch.nn.functional.normalize(torch.randn((n, 3), generator=gen), dim=-1)
    out = spec.mlp().apply(lp, feats.cuda(), dirs.cuda()).cpu().double()
    want = _mirror_mlp({a: {b: t.double() for b, t in v.items()} for a, v in ref["mlp"].items()},
                       feats.double(), dirs.double())
    err = float((out - want).abs().max())
    assert err < 4e-3, err
    st = ctypes.c_int32(-1)
    _lib.call("tvm_device_status", ctypes.byref(st), None)
    assert st.value == 0


def _rays(R, seed):
    from tensorf_gb300 import scene
    o, d, c = scene.sphere_rays(R, seed)
    return torch.tensor(o), torch.tensor(d), torch.tensor(c)


def test_bf16_render_tracks_fp32():
    from tensorf_gb300 import cameras, render
    G, R, N, k = 32, 512, 128, 32
    ref = _params(G, 2)
    o, d, c = _rays(R, 2)
    rng = np.random.default_rng(2)
    noise = render.RenderNoise(torch.tensor(rng.uniform(size=N), dtype=torch.float32).cuda(),
                               torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32).cuda())
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    outs = {}
    for prec in ("fp32", "bf16"):
        spec = render.ModelSpec(grid_dim=G, precision=prec)
        lp = render.LearnableParams.from_reference(spec, ref)
        outs[prec] = render.render_rays(spec.mlp(), lp, aabb, cameras.Rays3D(o.cuda(), d.cuda()), noise, cfg,
                                        density_shift=-1.0).cpu()
    diff = (outs["bf16"] - outs["fp32"]).abs()
    assert float(diff.mean()) < 5e-3 and float(torch.quantile(diff.flatten(), 0.99)) < 3e-2


def test_bf16_gradients_align_with_fp32():
    from tensorf_gb300 import cameras, render
    G, R, N, k = 32, 512, 128, 32
    ref = _params(G, 3)
    o, d, c = _rays(R, 3)
    rng = np.random.default_rng(3)
    noise = render.RenderNoise(torch.tensor(rng.uniform(size=N), dtype=torch.float32).cuda(),
                               torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=N))), dtype=torch.float32).cuda())
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, N, k)
    grads = {}
    for prec in ("fp32", "bf16"):
        spec = render.ModelSpec(grid_dim=G, precision=prec)
        lp = render.LearnableParams.from_reference(spec, ref)
        g = torch.zeros_like(lp.params)
        render.loss_and_grad(lp, g, aabb, cameras.Rays3D(o.cuda(), d.cuda()), c.cuda(), noise, cfg, density_shift=-1.0)
        grads[prec] = (lp, g)
    lp32, g32 = grads["fp32"]
    lp16, g16 = grads["bf16"]
    L = lp32.layout
    for lo, hi in ((L.density_lines, L.appearance_lines), (L.appearance_lines, L.mlp_begin), (L.mlp_begin, L.total)):
        a, b = g32[lo:hi].double(), g16[lo:hi].double()
        cos = float(torch.dot(a, b) / (a.norm() * b.norm()))
        assert cos > 0.98, (lo, hi, cos)


def _mirror_mlp_backward(mlp, feats, dirs, grad_rgb):
    """Gradients of FeatureMlp with bf16 rounding at the points where the fused kernel
    rounds (layer inputs, weights, dZ and the back-propagated dH2 / dH1 / dH0), fp64
    elsewhere. Returns (dX0, {layer: {name: grad}})."""
    W = {k: {n: t.double() for n, t in v.items()} for k, v in mlp.items()}
    x0 = _bf(feats)
    h = x0 @ _bf(W["Dense_0"]["kernel"])
    hh = h.clone().requires_grad_(True)
    pe_h = O.fourier_encode(hh, 2)
    x1 = torch.cat([h, dirs, pe_h.detach(), O.fourier_encode(dirs, 2)], -1)
    x1b = _bf(x1)
    h1 = torch.relu(x1b @ _bf(W["Dense_1"]["kernel"]) + W["Dense_1"]["bias"])
    h1b = _bf(h1)
    h2 = torch.relu(h1b @ _bf(W["Dense_2"]["kernel"]) + W["Dense_2"]["bias"])
    h2b = _bf(h2)
    rgb = torch.sigmoid(h2b @ _bf(W["Dense_3"]["kernel"]) + W["Dense_3"]["bias"])
    dz = grad_rgb * rgb * (1 - rgb)
    dzb = _bf(dz)
    dh2 = _bf((dzb @ _bf(W["Dense_3"]["kernel"]).T) * (h2b > 0))
    dh1 = _bf((dh2 @ _bf(W["Dense_2"]["kernel"]).T) * (h1b > 0))
    dx1 = dh1 @ _bf(W["Dense_1"]["kernel"]).T
    (g_pe,) = torch.autograd.grad(pe_h, hh, grad_outputs=dx1[:, 30:138])
    dh0 = _bf(dx1[:, :27] + g_pe)
    grads = {
        "Dense_0": {"kernel": x0.T @ dh0},
        "Dense_1": {"kernel": x1b.T @ dh1, "bias": dh1.sum(0)},
        "Dense_2": {"kernel": h1b.T @ dh2, "bias": dh2.sum(0)},
        "Dense_3": {"kernel": h2b.T @ dzb, "bias": dz.sum(0)},
    }
    return dh0 @ _bf(W["Dense_0"]["kernel"]).T, grads


@pytest.mark.parametrize("n", [1, 200, 5000, 40000])
def test_fused_bf16_mlp_backward_matches_mirror(n):
    """tvm_mlp_bwd on a BF16 model (the fused tcgen05 backward) against the rounding
    mirror: feature gradients and every weight / bias gradient."""
    from tensorf_gb300 import _lib, render
    from tensorf_gb300._util import ptr, stream_handle
    spec = render.ModelSpec(grid_dim=8, precision="bf16")
    ref = _params(8, 4)
    lp = render.LearnableParams.from_reference(spec, ref)
    gen = torch.Generator().manual_seed(100 + n)
    feats = torch.randn((n, 144), generator=gen) * 0.3
    dirs = torch.nn.functional.normalize(torch.randn((n, 3), generator=gen), dim=-1)
    grad_rgb = torch.randn((n, 3), generator=gen)
    md = lp.model_desc()
    ws = torch.empty(_lib.load().tvm_mlp_workspace_size(ctypes.byref(md), n), dtype=torch.uint8, device="cuda")
    f_c, d_c, g_c = feats.cuda().contiguous(), dirs.cuda().contiguous(), grad_rgb.cuda().contiguous()
    gfeat = torch.empty_like(f_c)
    grads = torch.zeros_like(lp.params)
    _lib.call("tvm_mlp_bwd", ctypes.byref(md), ptr(lp.params), ptr(f_c), ptr(d_c), None, n, ptr(g_c), ptr(gfeat),
              ptr(grads), ptr(ws), ws.numel(), stream_handle())
    st = ctypes.c_int32(-1)
    _lib.call("tvm_device_status", ctypes.byref(st), None)
    assert st.value == 0
    dx0, want = _mirror_mlp_backward(ref["mlp"], feats.double(), dirs.double(), grad_rgb.double())

    def rel(a, b):
        a, b = a.double().cpu(), b.double().cpu()
        return float((a - b).norm() / (b.norm() + 1e-30))

    errs = {"dX0": rel(gfeat, dx0)}
    got = lp.mlp_views(grads)
    for layer, v in want.items():
        for name, t in v.items():
            errs[f"{layer}.{name}"] = rel(got[layer][name], t)
    print(n, {k: f"{v:.2e}" for k, v in errs.items()})
    assert max(errs.values()) < 1e-2, errs
