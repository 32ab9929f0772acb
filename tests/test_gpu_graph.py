"""TrainState with its step recorded as a CUDA graph (the counterpart of the reference's
jit-compiled step, training.py:101), and with its field updates deferred to the next
step, against the same steps run eagerly and updating at once.

Both states start from the same parameters and key, so they draw the same noise; the
graph path reads the Adam scalars and the noise key from device memory
(tvm_set_step_scalars) and its batches are copied into fixed buffers. After several
steps parameters and both moments agree to the order of the atomic gradient reductions
(FP32: all but a handful of elements to 1e-5; BF16, where last-bit differences flip bf16
roundings: within 3x of a second eager run's distance plus 1e-2 in norm), the logged
learning rates are equal, the replays ran (and counted) their kernels, and a grid resize
records a new graph.
"""
import dataclasses

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _close(x, y, tol=1e-5):
    """Equal but for a handful of elements whose gradient sums to about zero, which may
    take the other Adam direction under another reduction order."""
    x, y = x.double().cpu(), y.double().cpu()
    off = (x - y).abs() > tol * float(x.abs().max())
    return int(off.sum()) <= max(8, x.numel() // 100000), int(off.sum())


def _dist(x, y):
    x, y = x.double().cpu(), y.double().cpu()
    return float((x - y).norm() / x.norm())


def _bf16_close(d, d_eager):
    """BF16 runs drift apart chaotically: a last-bit difference flips a bf16 rounding
    (of a field value, or of a proposal feature, which can move a resampled bin) that
    every later step reads. Runs of the same steps measured 4e-7 to 2e-5 apart (in norm)
    after three steps and 1e-4 to 3e-3 after six, so one second run is a noisy yardstick:
    the run under test may sit 3x further than it, plus 1e-2. A real ordering fault in
    the BF16-only work (a field update whose bf16 shadow is not refreshed before the
    gathers read it) moves every field parameter by a whole Adam step, about 1e-1 of
    their norm; the FP32 cases check the shared scheduling element by element."""
    return d <= 3.0 * d_eager + 1e-2


def _states(cfg, spec, graphs=(False, True)):
    from tensorf_gb300 import render, training
    return [training.TrainState(cfg, render.LearnableParams.initialize(spec, seed=4, scene_contraction=cfg.scene_contraction),
                                seed=7, cuda_graph=g) for g in graphs]


def _batches(R, n, seed, contract=False, cams=0):
    from tensorf_gb300 import cameras, scene
    out = []
    for i in range(n):
        if contract:
            o, d = scene.unbounded_rays(R, seed + i)
            c = np.random.default_rng(seed + i).uniform(size=(R, 3))
        else:
            o, d, c = scene.sphere_rays(R, seed + i)
        ci = (torch.arange(R, dtype=torch.int32) % cams).cuda() if cams else None
        out.append((cameras.Rays3D(torch.tensor(o, dtype=torch.float32).cuda(),
                                   torch.tensor(d, dtype=torch.float32).cuda(), ci),
                    torch.tensor(c, dtype=torch.float32).cuda()))
    return out


@pytest.mark.parametrize("case", ["bounded", "proposal_fp32", "proposal_bf16", "contracted_cameras"])
def test_graph_steps_match_eager_steps(case):
    from tensorf_gb300 import render, training
    kw = dict(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3, density_samples_per_ray=64,
              appearance_samples_per_ray=8, density_shift=-1.0, n_iters=20, upsamp_iters=(3,))
    spec = render.ModelSpec(grid_dim=24)
    contract, cams = False, 0
    if case.startswith("proposal"):
        kw.update(density_samples_per_ray=32, proposal=render.ProposalConfig(samples=32))
        spec = render.ModelSpec(grid_dim=24, precision=case[-4:], proposal_grid=16)
    if case == "contracted_cameras":
        kw.update(initial_aabb_min=(-2.0,) * 3, initial_aabb_max=(2.0,) * 3, scene_contraction=True)
        spec = render.ModelSpec(grid_dim=24, num_cameras=3)
        contract, cams = True, 3
    cfg = training.TrainConfig(**kw)
    bf16 = spec.precision == "bf16"
    # BF16: a last-bit difference in a master weight (another reduction order) can flip the
    # rounding of its bf16 copy, which every later gather reads, so any two runs drift apart
    # element by element; a second eager run measures how far, and the graph run may not
    # drift further from the first.
    states = _states(cfg, spec, (False, True, False) if bf16 else (False, True))
    eager, graph = states[0], states[1]
    batches = _batches(256, 6, 11, contract, cams)
    for rays, colors in batches:
        logs = [st.training_step(rays, colors)[1] for st in states]
        la, lb = logs[0], logs[1]
        assert la["train/lr_tensor"] == lb["train/lr_tensor"] and la["train/lr_mlp"] == lb["train/lr_mlp"]
        assert lb["train/mse"] == pytest.approx(la["train/mse"], rel=1e-3 if bf16 else 1e-4)
    torch.cuda.synchronize()
    assert eager.step == graph.step == 6
    assert graph._graph is not None and graph.graph_kernel_launches >= 5 * graph._graph.launches > 0
    for name in ("params", "mu", "nu"):
        get = (lambda st: st.learnable_params.params) if name == "params" else (lambda st: getattr(st, name))
        if bf16:
            d_graph, d_eager = _dist(get(eager), get(graph)), _dist(get(eager), get(states[2]))
            assert _bf16_close(d_graph, d_eager), (name, d_graph, d_eager)
        else:
            ok, n_off = _close(get(eager), get(graph))
            assert ok, (name, n_off)
    assert float(graph.grads.abs().max()) == 0.0


def test_graph_recorded_again_after_resize():
    from tensorf_gb300 import render, training
    cfg = training.TrainConfig(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3, density_samples_per_ray=64,
                               appearance_samples_per_ray=8, density_shift=-1.0, n_iters=20, upsamp_iters=(2,))
    eager, graph = _states(cfg, render.ModelSpec(grid_dim=16))
    batches = _batches(128, 5, 3)
    for i, (rays, colors) in enumerate(batches):
        if i == 2:
            for st in (eager, graph):
                st.resize_grid(24)
        eager.training_step(rays, colors, log=False)
        graph.training_step(rays, colors, log=False)
    torch.cuda.synchronize()
    assert graph.learnable_params.spec.grid_dim == 24 and graph._graph.key[4] == graph.learnable_params.params.data_ptr()
    ok, n_off = _close(eager.learnable_params.params, graph.learnable_params.params)
    assert ok, n_off


def test_explicit_noise_runs_eagerly():
    from tensorf_gb300 import render, training
    cfg = training.TrainConfig(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3, density_samples_per_ray=32,
                               appearance_samples_per_ray=8, density_shift=-1.0)
    st = training.TrainState.initialize(cfg, render.ModelSpec(grid_dim=16))
    (rays, colors), = _batches(64, 1, 5)
    rng = np.random.default_rng(0)
    noise = render.RenderNoise(torch.tensor(rng.uniform(size=32), dtype=torch.float32).cuda(),
                               torch.tensor(-np.log(-np.log(rng.uniform(1e-7, 1, size=32))),
                                            dtype=torch.float32).cuda())
    st.training_step(rays, colors, noise=noise)
    assert st._graph is None and st.step == 1
    assert dataclasses.is_dataclass(st.config)


@pytest.mark.parametrize("proposal", [False, True])
def test_keyed_noise_equals_key_drawn_noise(proposal):
    """tvm_noise_fill_keyed with the key's stream id in device memory draws bit for bit
    what draw_noise draws from the key on the host, including stream ids past 2^63."""
    from tensorf_gb300 import _lib, render
    from tensorf_gb300._util import stream_handle
    R = 100
    cfg = render.RenderConfig(0.05, 200.0, render.RenderMode.RGB, 24, 4)
    prop = render.ProposalConfig(samples=16) if proposal else None
    scal = torch.zeros(3, dtype=torch.int64, device="cuda")  # tvm_step_scalars
    for stream in (0, 5, 2**63 + 12345):
        key = render.NoiseKey(77, stream)
        want = render.draw_noise(key, R, cfg, False, prop)
        got = render.draw_noise(render.NoiseKey(0), R, cfg, False, prop)
        _lib.call("tvm_set_step_scalars", scal.data_ptr(), 1, 1.0, stream & (2**64 - 1), 0, 0.0, stream_handle())
        render.draw_noise_keyed(77, scal, R, cfg, prop, got)
        for a, b in ((want.jitter, got.jitter), (want.gumbel, got.gumbel), (want.proposal_jitter, got.proposal_jitter)):
            assert (a is None) == (b is None)
            if a is not None:
                assert torch.equal(a, b)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("case", ["bounded", "proposal_fp32", "proposal_bf16"])
def test_deferred_field_updates_match_immediate(case, graph):
    """Steps that leave the fields' Adam update pending (applied by the next step beside
    its start, or when parameters are read) against steps that update at once: equal
    parameters, moments and zero gradients whenever they are read, including mid-run."""
    from tensorf_gb300 import render, training
    kw = dict(initial_aabb_min=(-1.5,) * 3, initial_aabb_max=(1.5,) * 3, density_samples_per_ray=64,
              appearance_samples_per_ray=8, density_shift=-1.0, n_iters=20, upsamp_iters=(3,))
    spec = render.ModelSpec(grid_dim=24)
    if case.startswith("proposal"):
        kw.update(density_samples_per_ray=32, proposal=render.ProposalConfig(samples=32))
        spec = render.ModelSpec(grid_dim=24, precision=case[-4:], proposal_grid=16)
    cfg = training.TrainConfig(**kw)
    bf16 = spec.precision == "bf16"

    def make(defer, cuda_graph):
        lp = render.LearnableParams.initialize(spec, seed=4)
        return training.TrainState(cfg, lp, seed=7, cuda_graph=cuda_graph, defer_field_updates=defer)

    states = [make(False, False), make(True, graph)] + ([make(False, False)] if bf16 else [])
    batches = _batches(256, 6, 21)

    def check():
        ref, dfr = states[0], states[1]
        for name in ("params", "mu", "nu"):
            get = (lambda st: st.learnable_params.params) if name == "params" else (lambda st: getattr(st, name))
            if bf16:
                d_def, d_eager = _dist(get(ref), get(dfr)), _dist(get(ref), get(states[2]))
                assert _bf16_close(d_def, d_eager), (name, d_def, d_eager)
            else:
                ok, n_off = _close(get(ref), get(dfr))
                assert ok, (name, n_off)
        assert float(dfr.grads.abs().max()) == 0.0

    for i, (rays, colors) in enumerate(batches):
        for st in states:
            st.training_step(rays, colors, log=False)
        assert states[1]._pending is not None
        if i == 2:
            check()  # reading applies the pending update; the next step then has none
            assert states[1]._pending is None
    torch.cuda.synchronize()
    check()
    assert states[1].step == 6
