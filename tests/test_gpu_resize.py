"""GPU tests of grid upsampling: tvm_resize_field against the oracle's restatement of
resize_with_aligned_corners (tensor_vm.py:202-223), and TrainState.resize_grid
(training.py:245-276) carrying parameters and Adam moments over."""
import numpy as np
import pytest
import torch

from oracle import tensorf_oracle as O

pytestmark = pytest.mark.gpu


# Sample positions are float32 on both sides, but the device contracts (o + 0.5) / s -
# t / s into a fused multiply-add: at 300-point grids the positions differ by an ulp
# (~1e-5 voxels), which moves interpolated values by ~1e-5 of the field's range.
RTOL = 1e-4


def _rel(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    assert a.shape == b.shape and a.numel() > 0
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


@pytest.mark.parametrize("m,n", [(8, 19), (19, 8), (16, 16), (128, 300), (300, 128)])
@pytest.mark.parametrize("c", [4, 16, 48])
def test_resize_field_matches_oracle(m, n, c):
    from tensorf_gb300.tensor_vm import TensorVM
    if c == 48 and m * n > 20000:
        pytest.skip("covered by the 16-channel case at this size")
    gen = torch.Generator().manual_seed(m * 1000 + n + c)
    vec, mat = O.vm_init(m, c, gen, torch.float64)
    tv = TensorVM.from_reference(vec.float(), mat.float())
    out = tv.resize(n)
    got_v, got_m = out.to_reference()
    want_v, want_m = O.vm_resize(vec.float().double(), mat.float().double(), n)
    assert _rel(got_v, want_v) < RTOL
    assert _rel(got_m, want_m) < RTOL


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_train_state_resize_grid(precision):
    from tensorf_gb300 import cameras, render, scene, training
    spec = render.ModelSpec(grid_dim=16, precision=precision, proposal_grid=16)
    cfg = training.TrainConfig(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3,
                               density_samples_per_ray=64, appearance_samples_per_ray=16,
                               n_iters=100, upsamp_iters=(2,), grid_dim_init=16, grid_dim_final=24,
                               density_shift=-1.0, proposal=render.ProposalConfig(samples=32))
    st = training.TrainState.initialize(cfg, spec, seed=3)
    o, d, c = scene.sphere_rays(256, 4)
    rays = cameras.Rays3D(torch.tensor(o).cuda(), torch.tensor(d).cuda())
    colors = torch.tensor(c).cuda()
    for _ in range(2):
        st.training_step(rays, colors, log=False)
    torch.cuda.synchronize()
    lp0 = st.learnable_params
    old = {w: [t.clone() for t in lp0.field_views(w)] for w in ("density", "appearance")}
    old_mu = {w: [t.clone() for t in lp0.field_views(w, st.mu)] for w in ("density", "appearance")}
    old_mlp = {k: {n: t.clone() for n, t in v.items()} for k, v in lp0.mlp_views().items()}
    old_prop = {k: t.clone() for k, t in lp0.proposal_views().items()}
    new_g = training.upsampled_grid_dim(cfg, 2)
    assert new_g == 24
    st.resize_grid(new_g)
    lp = st.learnable_params
    assert lp.spec.grid_dim == 24 and lp.params.numel() == render.param_layout(lp.spec).total
    for w in ("density", "appearance"):
        for got, src in ((lp.field_views(w), old[w]), (lp.field_views(w, st.mu), old_mu[w])):
            lines, planes = src
            want_v, want_m = O.vm_resize(lines.permute(0, 2, 1).double().cpu(), planes.permute(0, 3, 1, 2).double().cpu(),
                                         24)
            assert _rel(got[0].permute(0, 2, 1), want_v) < RTOL
            assert _rel(got[1].permute(0, 3, 1, 2), want_m) < RTOL
    for k, v in lp.mlp_views().items():
        for n, t in v.items():
            assert torch.equal(t, old_mlp[k][n])
    for k, t in lp.proposal_views().items():
        assert torch.equal(t, old_prop[k])
    assert float(st.grads.abs().max()) == 0.0
    # Training continues at the new resolution.
    for _ in range(3):
        st.training_step(rays, colors, log=False)
    assert np.isfinite(float(st.loss.item()))


def test_state_dict_round_trip_resumes_identically(tmp_path):
    """state_dict() -> torch.save -> load -> from_state_dict(): the restored buffers are
    bit-identical, and the next training step matches the original's up to the order of
    the floating-point gradient reductions (atomics)."""
    from tensorf_gb300 import cameras, render, scene, training
    spec = render.ModelSpec(grid_dim=16, precision="bf16", proposal_grid=16)
    cfg = training.TrainConfig(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3,
                               density_samples_per_ray=64, appearance_samples_per_ray=16, n_iters=100,
                               upsamp_iters=(), density_shift=-1.0, proposal=render.ProposalConfig(samples=32))
    st = training.TrainState.initialize(cfg, spec, seed=5)
    o, d, c = scene.sphere_rays(256, 6)
    rays = cameras.Rays3D(torch.tensor(o).cuda(), torch.tensor(d).cuda())
    colors = torch.tensor(c).cuda()
    for _ in range(3):
        st.training_step(rays, colors, log=False)
    path = tmp_path / "state.pt"
    torch.save(st.state_dict(), path)
    st2 = training.TrainState.from_state_dict(cfg, torch.load(path))
    assert st2.step == st.step
    for a, b in ((st.learnable_params.params, st2.learnable_params.params), (st.mu, st2.mu), (st.nu, st2.nu)):
        assert torch.equal(a, b)
    st.training_step(rays, colors, log=False)
    st2.training_step(rays, colors, log=False)
    l1, l2 = float(st.loss.item()), float(st2.loss.item())
    assert abs(l1 - l2) <= 1e-6 * abs(l1)
    assert torch.allclose(st.learnable_params.params, st2.learnable_params.params, rtol=1e-4, atol=1e-6)
