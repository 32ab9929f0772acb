"""GPU tests of the FP32 FeatureMlp entry points (tvm_mlp_fwd / tvm_mlp_bwd) on the
split-tf32 pipelined GEMM path, against the float64 oracle (networks.py:45-121):

- row counts around the 128-row tile and past one tile per SM, and appearance widths
  other than 48 components, for rgb, the feature
  gradient and every weight and bias gradient (the bias and layer-3 gradients come from
  fused epilogues and a one-pass kernel, so each is checked on its own); rows with a
  hidden pre-activation within 1e-4 of a ReLU kink are redrawn;
- feature / view-direction / gradient buffers that are not 16-byte aligned, which take
  the layered first layer and scalar stores: they must agree with the aligned call."""
import ctypes

import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-4       # FP32 forward outputs
GRAD_RTOL = 1e-4  # gradients, as every FP32 parity test
KINK = 1e-4       # smallest |pre-activation| of a compared row


def _rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    assert a.shape == b.shape and a.numel() > 0
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


def _model(seed, ca=48, nf=2, nv=2):
    from tensorf_gb300 import render
    spec = render.ModelSpec(grid_dim=8, appearance_feat_dim=ca, feature_n_freqs=nf, viewdir_n_freqs=nv,
                            precision="fp32")
    gen = torch.Generator().manual_seed(seed)
    ref = {"density": O.vm_init(8, 16, gen, torch.float32), "appearance": O.vm_init(8, ca, gen, torch.float32),
           "mlp": O.mlp_init(3 * ca, nf, nv, gen, dtype=torch.float32)}
    for layer in ("Dense_1", "Dense_2", "Dense_3"):  # non-zero biases, so their gradients matter
        b = ref["mlp"][layer]["bias"]
        b.copy_(torch.randn(b.shape, generator=gen) * 0.1)
    return spec, ref, render.LearnableParams.from_reference(spec, ref)


def _inputs(n, seed, ref, nf=2, nv=2):
    """n rows whose hidden pre-activations all lie at least KINK from zero in the
    float64 oracle: at a ReLU kink an FP32 pre-activation of either sign is correct to
    rounding, but it decides whether that unit's gradient passes, so such rows are
    drawn again rather than compared."""
    gen = torch.Generator().manual_seed(seed)
    W = {k: {nm: t.double() for nm, t in d.items()} for k, d in ref["mlp"].items()}
    feat = W["Dense_0"]["kernel"].shape[0]
    keep_f, keep_d = [], []
    while sum(len(t) for t in keep_f) < n:
        feats = torch.randn((2 * n + 8, feat), generator=gen) * 0.3
        dirs = torch.nn.functional.normalize(torch.randn((2 * n + 8, 3), generator=gen), dim=-1)
        f = feats.double() @ W["Dense_0"]["kernel"]
        x1 = torch.cat([f, dirs.double(), O.fourier_encode(f, nf), O.fourier_encode(dirs.double(), nv)], dim=-1)
        z1 = x1 @ W["Dense_1"]["kernel"] + W["Dense_1"]["bias"]
        z2 = torch.relu(z1) @ W["Dense_2"]["kernel"] + W["Dense_2"]["bias"]
        ok = (z1.abs().min(dim=1).values > KINK) & (z2.abs().min(dim=1).values > KINK)
        keep_f.append(feats[ok])
        keep_d.append(dirs[ok])
    feats, dirs = torch.cat(keep_f)[:n], torch.cat(keep_d)[:n]
    grad_rgb = torch.randn((n, 3), generator=gen)
    return feats, dirs, grad_rgb


def _offset(t):
    """A copy of t on the GPU whose data starts 4 bytes past a 16-byte boundary."""
    flat = torch.zeros(t.numel() + 4, dtype=torch.float32, device="cuda")
    v = flat[1:1 + t.numel()].view(t.shape)
    v.copy_(t)
    return v


def _run(lp, feats, dirs, grad_rgb, out_offset=False):
    from tensorf_gb300 import _lib
    from tensorf_gb300._util import ptr, stream_handle
    lib = _lib.load()
    md = lp.model_desc()
    n = feats.shape[0]
    ws = torch.empty(max(1, lib.tvm_mlp_workspace_size(ctypes.byref(md), n)), dtype=torch.uint8, device="cuda")
    rgb = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    _lib.call("tvm_mlp_fwd", ctypes.byref(md), ptr(lp.params), ptr(feats), ptr(dirs), None, n, ptr(rgb), ptr(ws),
              ws.numel(), stream_handle())
    feat = feats.shape[1]
    gfeat = _offset(torch.zeros((n, feat))) if out_offset else torch.zeros((n, feat), device="cuda")
    grads = torch.zeros_like(lp.params)
    _lib.call("tvm_mlp_bwd", ctypes.byref(md), ptr(lp.params), ptr(feats), ptr(dirs), None, n, ptr(grad_rgb), ptr(gfeat),
              ptr(grads), ptr(ws), ws.numel(), stream_handle())
    st = ctypes.c_int32(-1)
    _lib.call("tvm_device_status", ctypes.byref(st), None)
    assert st.value == 0, "a bounded tensor-core wait gave up"
    torch.cuda.synchronize()
    return rgb, gfeat, lp.mlp_views(grads)


def _check_against_oracle(ref, lp, n, seed, nf=2, nv=2):
    feats, dirs, grad_rgb = _inputs(n, seed, ref, nf, nv)
    rgb, gfeat, got = _run(lp, feats.cuda(), dirs.cuda(), grad_rgb.cuda())

    mlp64 = {k: {nm: t.double().requires_grad_(True) for nm, t in d.items()} for k, d in ref["mlp"].items()}
    f64 = feats.double().requires_grad_(True)
    r64 = O.feature_mlp(mlp64, f64, dirs.double(), nf, nv)
    (r64 * grad_rgb.double()).sum().backward()
    assert _rel(rgb, r64) < RTOL
    assert _rel(gfeat, f64.grad) < GRAD_RTOL
    for layer, v in mlp64.items():
        for name, t in v.items():
            err = _rel(got[layer][name], t.grad)
            assert err < GRAD_RTOL, (layer, name, err)


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 152 * 128 + 77])
def test_fp32_mlp_matches_oracle_at_tile_edges(n):
    _, ref, lp = _model(7)
    _check_against_oracle(ref, lp, n, 1000 + n)


@pytest.mark.parametrize("ca", [8, 16, 24])
def test_fp32_mlp_other_appearance_widths(ca):
    """3 C appearance features other than 144: 24, 48 and the reference's default 72
    (train_config.py:44-45), with a narrower first product and a padded dX0 tile."""
    _, ref, lp = _model(9, ca)
    _check_against_oracle(ref, lp, 1000, 77 + ca)


@pytest.mark.parametrize("n", [1, 129, 5000])
def test_fp32_mlp_six_frequency_encodings(n):
    """feature_n_freqs = viewdir_n_freqs = 6, the nerfstudio preset
    (train_nerfstudio.py:33-34): a 390-wide encoding, which runs the layered split-tf32
    GEMMs with a separate encoding pass rather than the fused pipelined kernel."""
    _, ref, lp = _model(10, nf=6, nv=6)
    _check_against_oracle(ref, lp, n, 500 + n, nf=6, nv=6)


def test_fp32_mlp_unaligned_buffers_match_aligned():
    _, ref, lp = _model(8)
    n = 777
    feats, dirs, grad_rgb = _inputs(n, 8, ref)
    a = _run(lp, feats.cuda(), dirs.cuda(), grad_rgb.cuda())
    b = _run(lp, _offset(feats), _offset(dirs), _offset(grad_rgb), out_offset=True)
    assert _rel(b[0], a[0]) < 1e-5
    assert _rel(b[1], a[1]) < 1e-5
    for layer, v in a[2].items():
        for name, t in v.items():
            assert _rel(b[2][layer][name], t) < 1e-5, (layer, name)
