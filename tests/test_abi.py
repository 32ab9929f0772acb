"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, and rejects bad arguments with the documented codes before touching a GPU."""
import ctypes
import os
import re

import pytest

from tensorf_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "tensorf_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"TVM_API\s+[\w\s\*]+?\b(tvm_\w+)\s*\(", text)))


def test_header_declares_what_binding_declares():
    assert set(declared_symbols()) == set(_lib.exported_symbols())


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.tvm_abi_version() == _lib.ABI_VERSION == 3


def _model(**kw):
    d = dict(grid_dim=16, density_channels=16, appearance_channels=48, feature_n_freqs=2, viewdir_n_freqs=2,
             squash_dim=27, units=128, dtype=_lib.TVM_F32)
    d.update(kw)
    return _lib.ModelDesc(**d)


def test_param_layout_sizes():
    lay = _lib.ParamLayout()
    md = _model(grid_dim=300)
    _lib.call("tvm_get_param_layout", ctypes.byref(md), ctypes.byref(lay))
    assert lay.encoded_dim == 150
    assert lay.density_planes - lay.density_lines >= 3 * 300 * 16
    n_field = 3 * 300 * 16 * 301 + 3 * 300 * 48 * 301
    n_mlp = 144 * 27 + 150 * 128 + 128 + 128 * 128 + 128 + 128 * 3 + 3
    assert n_field + n_mlp <= lay.total <= n_field + n_mlp + 64 * 11
    assert lay.mlp_begin >= n_field and lay.mlp_w0 == lay.mlp_begin
    assert lay.shadow_total == 0


def test_bf16_layout_has_shadow():
    lay = _lib.ParamLayout()
    md = _model(dtype=_lib.TVM_BF16)
    _lib.call("tvm_get_param_layout", ctypes.byref(md), ctypes.byref(lay))
    assert lay.shadow_total == lay.mlp_begin


@pytest.mark.parametrize("kw,code", [
    (dict(density_channels=12), -5),
    (dict(grid_dim=1), -2),
    (dict(dtype=7), -3),
    (dict(units=0), -2),
])
def test_bad_model_rejected(kw, code):
    lay = _lib.ParamLayout()
    md = _model(**kw)
    st = _lib.load().tvm_get_param_layout(ctypes.byref(md), ctypes.byref(lay))
    assert st == code
    assert _lib.load().tvm_last_error_message()


def _render(**kw):
    d = _lib.RenderDesc()
    d.density_samples = kw.get("N", 64)
    d.appearance_samples = kw.get("k", 8)
    d.mode = kw.get("mode", _lib.TVM_MODE_RGB)
    d.sampler = kw.get("sampler", _lib.TVM_SAMPLER_BBOX)
    d.density_shift = 10.0
    for i, v in enumerate(kw.get("aabb", [-1, -1, -1, 1, 1, 1])):
        d.aabb[i] = v
    d.gumbel = kw.get("gumbel", 0x1000)
    return d


@pytest.mark.parametrize("kw", [
    dict(k=65),                       # k > N
    dict(k=0),
    dict(N=0),
    dict(aabb=[1, -1, -1, -1, 1, 1]),  # min > max
    dict(gumbel=None),                # RGB without noise
    dict(sampler=1),                  # contraction without schedule / jitter
    dict(mode=9),
])
def test_bad_render_rejected_before_launch(kw):
    md = _model()
    rd = _render(**kw)
    rays = _lib.Rays(count=4, origins=0x1000, directions=0x2000)
    st = _lib.load().tvm_render_fwd(ctypes.byref(md), ctypes.c_void_p(0x1000), None, ctypes.byref(rays),
                                    ctypes.byref(rd), ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000), 1 << 20, None)
    assert st in (-1, -2, -5), st
    assert _lib.load().tvm_render_workspace_size(ctypes.byref(md), ctypes.byref(rd), 4) == 0


def test_null_and_alignment_checks():
    lib = _lib.load()
    md = _model()
    rd = _render()
    rays = _lib.Rays(count=4, origins=0x1000, directions=0x2000)
    st = lib.tvm_render_fwd(ctypes.byref(md), None, None, ctypes.byref(rays), ctypes.byref(rd),
                            ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000), 1 << 20, None)
    assert st == -1
    st = lib.tvm_render_fwd(ctypes.byref(md), ctypes.c_void_p(0x1004), None, ctypes.byref(rays), ctypes.byref(rd),
                            ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000), 1 << 20, None)
    assert st == -4
    bf = _model(dtype=_lib.TVM_BF16)
    st = lib.tvm_render_fwd(ctypes.byref(bf), ctypes.c_void_p(0x1000), None, ctypes.byref(rays), ctypes.byref(rd),
                            ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000), 1 << 20, None)
    assert st == -1  # BF16 needs its shadow buffer


def test_topk_and_composite_argument_checks():
    lib = _lib.load()
    assert lib.tvm_topk_select(ctypes.c_void_p(16), ctypes.c_void_p(16), 0, 4, 8, 9, ctypes.c_void_p(16), None) == -2
    assert lib.tvm_topk_select(None, None, 0, 4, 8, 2, None, None) == -1
    assert lib.tvm_composite_fwd(None, None, 4, 8, None, None, None) == -1
    assert lib.tvm_composite_bwd(ctypes.c_void_p(16), ctypes.c_void_p(16), 4, 0, None, None,
                                 ctypes.c_void_p(16), None) == -2


def test_zero_rays_is_a_no_op():
    lib = _lib.load()
    md = _model()
    rd = _render()
    rays = _lib.Rays(count=0, origins=None, directions=None)
    assert lib.tvm_render_fwd(ctypes.byref(md), ctypes.c_void_p(0x1000), None, ctypes.byref(rays),
                              ctypes.byref(rd), None, None, 0, None) == 0
    assert lib.tvm_topk_select(None, None, 0, 0, 8, 2, None, None) == 0


def test_workspace_sizes_are_monotone_in_rays():
    lib = _lib.load()
    md = _model()
    rd = _render()
    a = lib.tvm_train_workspace_size(ctypes.byref(md), ctypes.byref(rd), 1024)
    b = lib.tvm_train_workspace_size(ctypes.byref(md), ctypes.byref(rd), 4096)
    c = lib.tvm_render_workspace_size(ctypes.byref(md), ctypes.byref(rd), 4096)
    assert 0 < a < b and 0 < c < b


@pytest.mark.parametrize("dtype,ca", [(_lib.TVM_F32, 48), (_lib.TVM_F32, 24), (_lib.TVM_BF16, 48)])
def test_static_scratch_limit_matches_workspace_size(dtype, ca):
    """tvm_mlp_fwd_static_scratch rejects oversized calls on the host, naming the largest
    row count whose forward scratch fits the 32 MiB array: that row count passes the
    size check (and then fails on the NULL pointers), one more row fails it. The
    forward needs less than the forward + backward workspace of tvm_mlp_workspace_size.
    The fused BF16 path needs no per-row scratch, so there the size check passes and
    the NULL pointers are rejected."""
    lib = _lib.load()
    md = _model(dtype=dtype, appearance_channels=ca)
    st = lib.tvm_mlp_fwd_static_scratch(ctypes.byref(md), None, None, None, 1 << 40, None, None)
    if dtype == _lib.TVM_BF16:
        assert st == -1
        return
    assert st == -2
    n = int(re.search(r"at most (\d+) rows", lib.tvm_last_error_message().decode()).group(1))
    assert lib.tvm_mlp_fwd_static_scratch(ctypes.byref(md), None, None, None, n, None, None) == -1
    assert lib.tvm_mlp_fwd_static_scratch(ctypes.byref(md), None, None, None, n + 1, None, None) == -2
    assert lib.tvm_mlp_workspace_size(ctypes.byref(md), n) > (32 << 20)
    assert 0 < n


def test_param_layout_camera_embeddings():
    """FeatureMlp camera embeddings (networks.py:103-111): a (num_cameras, units) segment
    inside the MLP learning-rate group; none without cameras; odd units rejected."""
    lay = _lib.ParamLayout()
    _lib.call("tvm_get_param_layout", ctypes.byref(_model(num_cameras=5)), ctypes.byref(lay))
    assert lay.mlp_embed >= lay.mlp_b3 + 3 and lay.mlp_embed >= lay.mlp_begin and lay.mlp_embed % 64 == 0
    assert lay.total >= lay.mlp_embed + 5 * 128
    plain = _lib.ParamLayout()
    _lib.call("tvm_get_param_layout", ctypes.byref(_model()), ctypes.byref(plain))
    assert plain.mlp_embed == 0 and lay.total == plain.total + 5 * 128
    st = _lib.load().tvm_get_param_layout(ctypes.byref(_model(num_cameras=5, units=127)), ctypes.byref(lay))
    assert st == -2


def test_nerfstudio_preset_matches_reference_defaults():
    """train_nerfstudio.py:23-44: contraction, 32 / 48 components, 6 / 6 frequencies,
    camera embeddings, 128^3 -> 300^3, 2048 rays, three times the sample heuristic; its
    model descriptor lays out."""
    from tensorf_gb300 import render, training
    cfg, spec = training.nerfstudio_preset(5)
    assert (spec.density_feat_dim, spec.appearance_feat_dim) == (32, 48)
    assert (spec.feature_n_freqs, spec.viewdir_n_freqs, spec.num_cameras) == (6, 6, 5)
    assert cfg.scene_contraction and cfg.minibatch_size == 2048 and cfg.train_ray_sample_multiplier == 3.0
    assert (cfg.initial_aabb_min, cfg.initial_aabb_max) == ((-2.0,) * 3, (2.0,) * 3)
    assert (cfg.render_near, cfg.render_far) == (0.05, 200.0)
    assert (cfg.grid_dim_init, cfg.grid_dim_final, cfg.upsamp_iters) == (128, 300, (2500, 5000, 10000))
    assert training.sample_counts(cfg.grid_dim_init, cfg) == (665, 99)
    lay = render.param_layout(spec)
    G = spec.grid_dim
    assert lay.appearance_lines - lay.density_lines >= 3 * 32 * G * (G + 1)



def _proposal_render(**kw):
    rd = _lib.RenderDesc(density_samples=48, appearance_samples=7, mode=_lib.TVM_MODE_RGB,
                         sampler=_lib.TVM_SAMPLER_PROPOSAL, proposal_samples=64)
    for i, v in enumerate((-1.5, -1.5, -1.5, 1.5, 1.5, 1.5)):
        rd.aabb[i] = v
    rd.proposal_jitter = 0x1000
    rd.jitter = 0x2000
    for k, v in kw.items():
        setattr(rd, k, v)
    return rd


def test_proposal_seam_argument_checks():
    """Each proposal seam rejects bad arguments with its code before any launch."""
    lib = _lib.load()
    rays = _lib.Rays(count=4, origins=0x1000, directions=0x2000)
    p16 = ctypes.c_void_p(0x1000)
    no_prop = _model()
    with_prop = _model(proposal_grid=16, proposal_rank=4, proposal_units=64)
    rd = _proposal_render()
    # forward: a model without a proposal network, a wrong sampler, too many bins, no jitter
    assert lib.tvm_proposal_fwd(ctypes.byref(no_prop), p16, None, ctypes.byref(rays), ctypes.byref(rd), p16, p16,
                                None) == -1
    bad = _proposal_render(sampler=_lib.TVM_SAMPLER_BBOX)
    assert lib.tvm_proposal_fwd(ctypes.byref(with_prop), p16, None, ctypes.byref(rays), ctypes.byref(bad), p16, p16,
                                None) == -1
    bad = _proposal_render(proposal_samples=513)
    assert lib.tvm_proposal_fwd(ctypes.byref(with_prop), p16, None, ctypes.byref(rays), ctypes.byref(bad), p16, p16,
                                None) == -2
    bad = _proposal_render(proposal_jitter=None)
    assert lib.tvm_proposal_fwd(ctypes.byref(with_prop), p16, None, ctypes.byref(rays), ctypes.byref(bad), p16, p16,
                                None) == -1
    bad = _proposal_render(contract=1)  # unbounded bins need the caller's edges
    assert lib.tvm_proposal_fwd(ctypes.byref(with_prop), p16, None, ctypes.byref(rays), ctypes.byref(bad), p16, p16,
                                None) == -1
    assert lib.tvm_proposal_fwd(ctypes.byref(with_prop), ctypes.c_void_p(0x1004), None, ctypes.byref(rays),
                                ctypes.byref(rd), p16, p16, None) == -4
    # resample: main samples past 512, missing outputs
    bad = _proposal_render(density_samples=513)
    assert lib.tvm_proposal_resample(ctypes.byref(rays), ctypes.byref(bad), p16, p16, p16, p16, None) == -2
    assert lib.tvm_proposal_resample(ctypes.byref(rays), ctypes.byref(rd), p16, None, p16, p16, None) == -1
    # loss: bin counts, NULL buffers; backward: unaligned gradients
    assert lib.tvm_proposal_loss(p16, p16, p16, 4, 1, 48, ctypes.c_float(1.0), None, p16, None) == -2
    assert lib.tvm_proposal_loss(p16, None, p16, 4, 64, 48, ctypes.c_float(1.0), None, p16, None) == -1
    assert lib.tvm_proposal_bwd(ctypes.byref(with_prop), p16, None, ctypes.c_void_p(0x1008), ctypes.byref(rays),
                                ctypes.byref(rd), p16, p16, None) == -4
    # zero rays: nothing to do
    none = _lib.Rays(count=0, origins=None, directions=None)
    assert lib.tvm_proposal_fwd(ctypes.byref(with_prop), p16, None, ctypes.byref(none), ctypes.byref(rd), None, None,
                                None) == 0
    assert lib.tvm_proposal_loss(None, None, None, 0, 64, 48, ctypes.c_float(1.0), None, None, None) == 0


def test_noise_batch_argument_checks():
    lib = _lib.load()
    jobs = (_lib.NoiseJob * 5)()
    assert lib.tvm_noise_fill_keyed_batch(jobs, 5, 1, ctypes.c_void_p(0x1000), None) == -2
    assert lib.tvm_noise_fill_keyed_batch(jobs, 0, 1, None, None) == 0
    jobs[0].n, jobs[0].kind = 8, 2
    assert lib.tvm_noise_fill_keyed_batch(jobs, 1, 1, ctypes.c_void_p(0x1000), None) == -1
    jobs[0].kind, jobs[0].dst = 0, None
    assert lib.tvm_noise_fill_keyed_batch(jobs, 1, 1, ctypes.c_void_p(0x1000), None) == -1
    jobs[0].dst = 0x1000
    assert lib.tvm_noise_fill_keyed_batch(jobs, 1, 1, ctypes.c_void_p(0x1004), None) == -4


def test_proposal_descriptor_from_python():
    """render._proposal_desc: the seams' descriptor (host logic only)."""
    from tensorf_gb300 import render
    prop = render.ProposalConfig(samples=32, shift=0.25, loss_weight=2.0)
    d = render._proposal_desc(((-1.0, -2.0, -3.0), (1.0, 2.0, 3.0)), prop, 10, False, None, samples=24)
    assert d.sampler == _lib.TVM_SAMPLER_PROPOSAL and d.proposal_samples == 32 and d.density_samples == 24
    assert abs(d.proposal_shift - 0.25) < 1e-7 and abs(d.proposal_loss_weight - 2.0) < 1e-7 and d.contract == 0
    assert list(d.aabb) == [-1.0, -2.0, -3.0, 1.0, 2.0, 3.0]
    assert not d.schedule and not d.proposal_jitter and not d.jitter
    with pytest.raises(ValueError):  # unbounded bins need the caller's edges
        render._proposal_desc(((-2.0,) * 3, (2.0,) * 3), prop, 10, True, None)
