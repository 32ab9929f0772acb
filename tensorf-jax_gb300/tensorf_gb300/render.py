"""GB300 twin of ``tensorf/render.py``.

Same public names as the reference (``RenderMode``, ``RenderConfig``,
``LearnableParams``, ``render_rays``, ``render_rays_batched``,
``compute_segment_probabilities``, ``sample_points_along_ray_within_bbox``), backed by
the C ABI. Differences at the boundary, all deliberate:

* Randomness: the reference threads a JAX PRNG key; here ``prng_key`` is a
  :class:`NoiseKey` (seed, stream) from which the device draws sample jitter and the
  Gumbel noise of the weighted choice, or a :class:`RenderNoise` holding explicit arrays
  (so the reference's own draws can be replayed bit for bit).
* Parameters: ``LearnableParams`` owns one flat FP32 parameter buffer (plus a bf16
  shadow of the field tensors in BF16 mode); ``density_tensor``,
  ``appearance_tensor`` and ``appearance_mlp_params`` are views into it.
* ``density_shift`` (default +10.0, render.py:207) is a keyword.
* ``RenderMode.DIST_MEDIAN`` returns the distance of the first sample where
  1 - p_exit > 0.5 (+inf if none). The reference formula (render.py:248-267) returns
  NaN for every ray that terminates, because it multiplies 0 by inf.
"""
from __future__ import annotations

import ctypes
import dataclasses
import enum
import math
from typing import Dict, Optional, Sequence, Tuple, Union

import numpy as onp
import torch

from . import _lib, cameras, networks
from ._util import ptr, require_cuda, stream_handle, workspace
from .tensor_vm import TensorVM


class RenderMode(enum.Enum):
    RGB = enum.auto()
    DIST_MEDIAN = enum.auto()
    DIST_MEAN = enum.auto()


_MODE_CODE = {RenderMode.RGB: _lib.TVM_MODE_RGB, RenderMode.DIST_MEDIAN: _lib.TVM_MODE_DIST_MEDIAN,
              RenderMode.DIST_MEAN: _lib.TVM_MODE_DIST_MEAN}


@dataclasses.dataclass(frozen=True)
class RenderConfig:
    """render.py:26-36."""
    near: float
    far: float
    mode: RenderMode
    density_samples_per_ray: int
    appearance_samples_per_ray: int


@dataclasses.dataclass(frozen=True)
class ModelSpec:
    """Sizes of the two VM tensors and the FeatureMlp, and the arithmetic mode."""
    grid_dim: int
    density_feat_dim: int = 16
    appearance_feat_dim: int = 48
    feature_n_freqs: int = 2
    viewdir_n_freqs: int = 2
    squash_dim: int = 27
    units: int = 128
    precision: str = "fp32"  # "fp32" or "bf16"
    mlp_math: str = "tensor"  # "tensor" (tcgen05; split-tf32 in fp32 mode) or "simt" (fp32 only)
    proposal_grid: int = 0    # proposal VM grid; 0 = no proposal network
    proposal_units: int = 64
    num_cameras: int = 0      # FeatureMlp camera embeddings (FiLM, networks.py:103-111); 0 = none

    def desc(self) -> _lib.ModelDesc:
        return _lib.ModelDesc(grid_dim=self.grid_dim, density_channels=self.density_feat_dim,
                              appearance_channels=self.appearance_feat_dim,
                              feature_n_freqs=self.feature_n_freqs, viewdir_n_freqs=self.viewdir_n_freqs,
                              squash_dim=self.squash_dim, units=self.units,
                              dtype=_lib.TVM_BF16 if self.precision == "bf16" else _lib.TVM_F32,
                              mlp_math=_lib.TVM_MLP_SIMT_F32 if self.mlp_math == "simt" else _lib.TVM_MLP_DEFAULT,
                              proposal_grid=self.proposal_grid, proposal_rank=4 if self.proposal_grid else 0,
                              proposal_units=self.proposal_units, num_cameras=self.num_cameras)

    def mlp(self) -> networks.FeatureMlp:
        return networks.FeatureMlp(feature_squash_dim=self.squash_dim, units=self.units,
                                   feature_n_freqs=self.feature_n_freqs, viewdir_n_freqs=self.viewdir_n_freqs,
                                   num_cameras=self.num_cameras or None)


def param_layout(spec: ModelSpec) -> _lib.ParamLayout:
    lay = _lib.ParamLayout()
    md = spec.desc()
    _lib.call("tvm_get_param_layout", ctypes.byref(md), ctypes.byref(lay))
    return lay


class LearnableParams:
    """render.py:39-46: appearance MLP params, appearance tensor, density tensor and the
    scene-contraction flag, held in one flat device buffer."""

    def __init__(self, spec: ModelSpec, params: torch.Tensor, shadow: Optional[torch.Tensor] = None,
                 scene_contraction: bool = False):
        self.spec = spec
        self.layout = param_layout(spec)
        if params.numel() != self.layout.total or params.dtype != torch.float32 or not params.is_cuda:
            raise ValueError("params must be a CUDA float32 buffer of layout.total elements")
        self.params = params
        self._md = spec.desc()
        self.scene_contraction = scene_contraction
        self.shadow = shadow
        if spec.precision == "bf16" and shadow is None:
            self.shadow = torch.empty(self.layout.shadow_total, dtype=torch.bfloat16, device=params.device)
            self.refresh_shadow()

    # ---- views -----------------------------------------------------------------
    def model_desc(self) -> _lib.ModelDesc:
        return self._md

    def _seg(self, off: int, shape, buf=None) -> torch.Tensor:
        buf = self.params if buf is None else buf
        n = int(onp.prod(shape))
        return buf[off:off + n].view(*shape)

    def field_views(self, which: str, buf: Optional[torch.Tensor] = None):
        L, s = self.layout, self.spec
        g = s.grid_dim
        c = s.density_feat_dim if which == "density" else s.appearance_feat_dim
        lo = L.density_lines if which == "density" else L.appearance_lines
        po = L.density_planes if which == "density" else L.appearance_planes
        return self._seg(lo, (3, g, c), buf), self._seg(po, (3, g, g, c), buf)

    @property
    def density_tensor(self) -> TensorVM:
        return TensorVM(*self.field_views("density"))

    @property
    def appearance_tensor(self) -> TensorVM:
        return TensorVM(*self.field_views("appearance"))

    def mlp_views(self, buf: Optional[torch.Tensor] = None) -> Dict[str, Dict[str, torch.Tensor]]:
        L, s = self.layout, self.spec
        enc = L.encoded_dim
        f = 3 * s.appearance_feat_dim
        return {
            "Dense_0": {"kernel": self._seg(L.mlp_w0, (f, s.squash_dim), buf)},
            "Dense_1": {"kernel": self._seg(L.mlp_w1, (enc, s.units), buf), "bias": self._seg(L.mlp_b1, (s.units,), buf)},
            "Dense_2": {"kernel": self._seg(L.mlp_w2, (s.units, s.units), buf), "bias": self._seg(L.mlp_b2, (s.units,), buf)},
            "Dense_3": {"kernel": self._seg(L.mlp_w3, (s.units, 3), buf), "bias": self._seg(L.mlp_b3, (3,), buf)},
            **({"Embed_0": {"embedding": self._seg(L.mlp_embed, (s.num_cameras, s.units), buf)}}
               if s.num_cameras else {}),
        }

    @property
    def appearance_mlp_params(self):
        return self.mlp_views()

    def proposal_views(self, buf: Optional[torch.Tensor] = None) -> Dict[str, torch.Tensor]:
        """The proposal network: field lines (3, Gp, 4) / planes (3, Gp, Gp, 4)
        channel-last, MLP w1 (16, U), b1 (U,), w2 (U, 1), b2 (1,)."""
        L, s = self.layout, self.spec
        g, u = s.proposal_grid, s.proposal_units
        return {"lines": self._seg(L.proposal_lines, (3, g, 4), buf),
                "planes": self._seg(L.proposal_planes, (3, g, g, 4), buf),
                "w1": self._seg(L.proposal_w1, (16, u), buf), "b1": self._seg(L.proposal_b1, (u,), buf),
                "w2": self._seg(L.proposal_w2, (u, 1), buf), "b2": self._seg(L.proposal_b2, (1,), buf)}

    # ---- construction ----------------------------------------------------------
    @staticmethod
    def initialize(spec: ModelSpec, seed: int = 94709, scene_contraction: bool = False,
                   device="cuda") -> "LearnableParams":
        """TrainState.initialize's parameter init (training.py:35-99): N(0, 0.1^2)
        field tensors, flax-style MLP init."""
        require_cuda()
        return LearnableParams.from_reference(spec, initial_reference_params(spec, seed), scene_contraction, device)

    @staticmethod
    def from_reference(spec: ModelSpec, ref: dict, scene_contraction: bool = False,
                       device="cuda") -> "LearnableParams":
        """From reference-layout arrays: ref['density'] = (vector (3,C,G), matrix
        (3,C,G,G)), ref['appearance'] likewise, ref['mlp'] = flax tree."""
        require_cuda()
        lay = param_layout(spec)
        params = torch.zeros(lay.total, dtype=torch.float32, device=device)
        lp = LearnableParams.__new__(LearnableParams)
        lp.spec, lp.layout, lp.params, lp.shadow, lp.scene_contraction = spec, lay, params, None, scene_contraction
        lp._md = spec.desc()
        for which in ("density", "appearance"):
            vec, mat = ref[which]
            lines, planes = lp.field_views(which)
            g, c = spec.grid_dim, lines.shape[-1]
            v = vec.to(device=device, dtype=torch.float32).contiguous()
            m = mat.to(device=device, dtype=torch.float32).contiguous()
            _lib.call("tvm_vm_to_channel_last", g, c, ptr(v), ptr(m), _lib.TVM_F32, ptr(lines), ptr(planes),
                      stream_handle())
        views = lp.mlp_views()
        for layer, d in ref["mlp"].items():
            for name, val in d.items():
                views[layer][name].copy_(torch.as_tensor(val, dtype=torch.float32))
        if spec.proposal_grid:
            pv = lp.proposal_views()
            pr = ref["proposal"]
            pv["lines"].copy_(torch.as_tensor(pr["vector"], dtype=torch.float32).permute(0, 2, 1))
            pv["planes"].copy_(torch.as_tensor(pr["matrix"], dtype=torch.float32).permute(0, 2, 3, 1))
            for n in ("w1", "b1", "w2", "b2"):
                pv[n].copy_(torch.as_tensor(pr[n], dtype=torch.float32).reshape(pv[n].shape))
        if spec.precision == "bf16":
            lp.shadow = torch.empty(lay.shadow_total, dtype=torch.bfloat16, device=device)
            lp.refresh_shadow()
        return lp

    def to_reference(self, buf: Optional[torch.Tensor] = None) -> dict:
        """Reference-layout CPU float32 copies of params (or of a same-layout buffer
        such as gradients)."""
        out = {}
        for which in ("density", "appearance"):
            lines, planes = self.field_views(which, buf)
            out[which] = (lines.permute(0, 2, 1).contiguous().cpu(), planes.permute(0, 3, 1, 2).contiguous().cpu())
        out["mlp"] = {k: {n: t.detach().cpu().clone() for n, t in d.items()} for k, d in self.mlp_views(buf).items()}
        if self.spec.proposal_grid:
            pv = self.proposal_views(buf)
            out["proposal"] = {"vector": pv["lines"].permute(0, 2, 1).contiguous().cpu(),
                               "matrix": pv["planes"].permute(0, 3, 1, 2).contiguous().cpu(),
                               **{n: pv[n].detach().cpu().clone() for n in ("w1", "b1", "w2", "b2")}}
        return out

    def refresh_shadow(self) -> None:
        if self.spec.precision == "bf16":
            _lib.call("tvm_refresh_shadow", ctypes.byref(self._md), ptr(self.params), ptr(self.shadow),
                      stream_handle())


# ---------------------------------------------------------------------------------
# Randomness.
# ---------------------------------------------------------------------------------
@dataclasses.dataclass(frozen=True)
class NoiseKey:
    """Stand-in for a JAX PRNG key: a seed and a stream id. ``split`` derives two
    independent keys, like ``jax.random.split``; the device draws the noise."""
    seed: int
    stream: int = 0

    def split(self) -> Tuple["NoiseKey", "NoiseKey"]:
        return NoiseKey(self.seed, self.stream * 2 + 1), NoiseKey(self.seed, self.stream * 2 + 2)

    def uniform(self, n: int, device="cuda", out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """n uniforms in [0, 1); written into ``out`` (n float32 elements) when given."""
        return self._fill(n, 0, device, out)

    def gumbel(self, n: int, device="cuda", out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """n standard Gumbel draws; written into ``out`` when given."""
        return self._fill(n, 1, device, out)

    def _fill(self, n: int, kind: int, device, out: Optional[torch.Tensor]) -> torch.Tensor:
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device=device)
        if out.numel() != n or out.dtype != torch.float32 or not out.is_contiguous():
            raise ValueError(f"noise buffer must be {n} contiguous float32 elements")
        _lib.call("tvm_noise_fill", ptr(out), n, self.seed & (2**64 - 1), self.stream & (2**64 - 1), kind,
                  stream_handle())
        return out


@dataclasses.dataclass
class RenderNoise:
    """Explicit noise: ``jitter`` (N,) shared by all rays (bounded scenes, as the
    reference draws it) or (R, N); ``gumbel`` (N,) shared or (R, N). Proposal-guided
    sampling also needs ``proposal_jitter`` (R, Np) and a per-interval ``jitter`` (R, N)."""
    jitter: Optional[torch.Tensor]
    gumbel: Optional[torch.Tensor]
    proposal_jitter: Optional[torch.Tensor] = None


@dataclasses.dataclass(frozen=True)
class ProposalConfig:
    """Proposal-guided sampling: ``samples`` proposal bins per ray resampled into the
    RenderConfig's density_samples_per_ray main samples. Unbounded scenes take the
    Np+1 bin edges from ``edges`` (default: linear in disparity over [near, far])."""
    samples: int = 64
    shift: float = 0.0
    loss_weight: float = 1.0


def initial_reference_params(spec: ModelSpec, seed: int = 94709) -> dict:
    """The initial parameters of LearnableParams.initialize in the reference's layout,
    on the CPU (float32): N(0, 0.1^2) vector / matrix of both VM tensors
    (training.py:44-56), flax-style FeatureMlp init, and the proposal network when the
    spec has one. Needs no GPU."""
    gen = torch.Generator().manual_seed(seed)
    g = spec.grid_dim
    ref = {
        "density": (torch.randn((3, spec.density_feat_dim, g), generator=gen) * 0.1,
                    torch.randn((3, spec.density_feat_dim, g, g), generator=gen) * 0.1),
        "appearance": (torch.randn((3, spec.appearance_feat_dim, g), generator=gen) * 0.1,
                       torch.randn((3, spec.appearance_feat_dim, g, g), generator=gen) * 0.1),
        "mlp": spec.mlp().init_params(3 * spec.appearance_feat_dim, gen),
    }
    if spec.proposal_grid:
        ref["proposal"] = init_proposal(spec.proposal_grid, spec.proposal_units, gen)
    return ref


def init_proposal(grid: int, units: int, gen: torch.Generator) -> Dict[str, torch.Tensor]:
    """Proposal network init: field N(0, 0.1^2) like the main field, kaiming-normal
    first layer, lecun-normal head, zero biases (CPU float32, reference layout)."""
    return {"vector": torch.randn((3, 4, grid), generator=gen) * 0.1,
            "matrix": torch.randn((3, 4, grid, grid), generator=gen) * 0.1,
            "w1": torch.randn((16, units), generator=gen) * math.sqrt(2.0 / 16),
            "b1": torch.zeros(units), "w2": torch.randn((units, 1), generator=gen) * math.sqrt(1.0 / units),
            "b2": torch.zeros(1)}


def draw_noise(key: NoiseKey, rays: int, config: RenderConfig, scene_contraction: bool,
               proposal: Optional[ProposalConfig] = None, out: Optional[RenderNoise] = None) -> RenderNoise:
    """Draw the noise render_rays needs from a key: the sample key drives the jitter
    ((N,) shared for bounded scenes, (R, N) for contracted ones, render.py:158-160,
    375-379) and the rgb key the Gumbel noise shared by every ray (render.py:461-469).
    Proposal-guided sampling draws per-ray jitter for both proposal bins and main
    intervals. With ``out`` (the result of an earlier call with the same sizes), the draws
    overwrite its buffers, whose addresses then stay fixed."""
    sample_key, rgb_key = key.split()
    n = config.density_samples_per_ray
    o = out if out is not None else RenderNoise(None, None, None)
    flat = lambda t: t.view(-1) if t is not None else None  # noqa: E731
    gumbel = rgb_key.gumbel(n, out=flat(o.gumbel)) if config.mode is RenderMode.RGB else None
    if proposal is not None:
        k1, k2 = sample_key.split()
        return RenderNoise(jitter=k1.uniform(rays * n, out=flat(o.jitter)).view(rays, n), gumbel=gumbel,
                           proposal_jitter=k2.uniform(rays * proposal.samples,
                                                      out=flat(o.proposal_jitter)).view(rays, proposal.samples))
    jitter = sample_key.uniform(rays * n if scene_contraction else n, out=flat(o.jitter))
    if scene_contraction:
        jitter = jitter.view(rays, n)
    return RenderNoise(jitter=jitter, gumbel=gumbel)


def draw_noise_keyed(seed: int, step_scalars: torch.Tensor, rays: int, config: RenderConfig,
                     proposal: Optional[ProposalConfig], out: RenderNoise) -> None:
    """draw_noise(NoiseKey(seed, s), ...) into ``out``'s buffers, with the key's stream id
    s read on the device from ``step_scalars`` (a tvm_step_scalars written by
    tvm_set_step_scalars) when the kernels run. draw_noise's key splits are affine in s
    (split: s -> 2s+1, 2s+2), so each draw is one (mul, add) pair; a recorded training
    step therefore replays each step's own noise."""
    jobs = []

    def fill(buf: torch.Tensor, mul: int, add: int, kind: int) -> None:
        jobs.append(_lib.NoiseJob(dst=ptr(buf).value, n=buf.numel(), mul=mul, add=add, kind=kind))

    if config.mode is RenderMode.RGB:
        fill(out.gumbel, 2, 2, 1)           # rgb key 2s+2
    if proposal is not None:
        fill(out.jitter, 4, 3, 0)           # sample key 2s+1, split: 4s+3
        fill(out.proposal_jitter, 4, 4, 0)  # and 4s+4
    else:
        fill(out.jitter, 2, 1, 0)           # sample key 2s+1
    arr = (_lib.NoiseJob * len(jobs))(*jobs)  # one launch for all of the step's draws
    _lib.call("tvm_noise_fill_keyed_batch", arr, len(jobs), seed & (2**64 - 1), step_scalars.data_ptr(),
              stream_handle())


# ---------------------------------------------------------------------------------
# Descriptors.
# ---------------------------------------------------------------------------------
def contracted_schedule(near: float, far: float, n: int) -> onp.ndarray:
    """render.py:127-151: linear close half, heuristic far half (float64 -> float32)."""
    close_n = n // 2
    far_n = n - close_n
    close_ts = onp.linspace(near, near + 1.0, close_n).astype(onp.float32)
    far_start = near + 1.0 + 1.0 / close_n
    k = 10.0
    far_deltas = (1.0 / (1.0 - onp.linspace(0.0, 1.0 - 1 / ((far - far_start) / k + 1), far_n)) - 1.0) \
        * onp.linspace(1.0, k, far_n)
    return onp.concatenate([close_ts, (far_start + far_deltas).astype(onp.float32)])


def disparity_schedule(near: float, far: float, n: int) -> onp.ndarray:
    """Samples linear in disparity between near and far."""
    s = onp.linspace(0.0, 1.0, n)
    return (1.0 / ((1.0 - s) / near + s / far)).astype(onp.float32)


def _aabb6(aabb) -> Sequence[float]:
    a = torch.as_tensor(aabb, dtype=torch.float32).reshape(2, 3).cpu()
    return [float(v) for v in a[0]] + [float(v) for v in a[1]]


def make_render_desc(config: RenderConfig, aabb, noise: RenderNoise, rays: int, scene_contraction: bool,
                     schedule: Optional[torch.Tensor], density_shift: float, mode: Optional[RenderMode] = None,
                     proposal: Optional[ProposalConfig] = None):
    mode = config.mode if mode is None else mode
    d = _lib.RenderDesc()
    if proposal is not None:
        d.sampler = _lib.TVM_SAMPLER_PROPOSAL
        d.proposal_samples = proposal.samples
        d.proposal_shift = proposal.shift
        d.proposal_loss_weight = proposal.loss_weight
        d.contract = int(scene_contraction)
        d.proposal_jitter = ptr(noise.proposal_jitter).value if noise.proposal_jitter is not None else None
    d.density_samples = config.density_samples_per_ray
    d.appearance_samples = config.appearance_samples_per_ray
    d.mode = _MODE_CODE[mode]
    if proposal is None:
        d.sampler = _lib.TVM_SAMPLER_CONTRACT if scene_contraction else _lib.TVM_SAMPLER_BBOX
    d.density_shift = density_shift
    for i, v in enumerate(_aabb6(aabb)):
        d.aabb[i] = v
    d.schedule = ptr(schedule).value if schedule is not None else None
    d.jitter = ptr(noise.jitter).value if noise.jitter is not None else None
    d.jitter_per_ray = int(noise.jitter is not None and noise.jitter.dim() == 2 and not scene_contraction)
    d.gumbel = ptr(noise.gumbel).value if noise.gumbel is not None else None
    d.gumbel_per_ray = int(noise.gumbel is not None and noise.gumbel.dim() == 2)
    return d


def rays_struct(rays: "cameras.Rays3D") -> _lib.Rays:
    """The C view of a ray batch. Camera indices, when present, must be a contiguous
    int32 CUDA tensor of one index per ray (the struct keeps only its address)."""
    o = rays.origins.reshape(-1, 3)
    dvec = rays.directions.reshape(-1, 3)
    ci = rays.camera_indices
    return _lib.Rays(count=o.shape[0], origins=ptr(o, torch.float32, "origins"),
                     directions=ptr(dvec, torch.float32, "directions"),
                     camera_indices=ptr(ci, torch.int32, "camera_indices") if ci is not None else None)


def _schedule_for(config: RenderConfig, scene_contraction: bool, schedule,
                  proposal: Optional[ProposalConfig] = None) -> Optional[torch.Tensor]:
    if not scene_contraction:
        return None
    if schedule is None:
        if proposal is not None:
            schedule = disparity_schedule(config.near, config.far, proposal.samples + 1)
        else:
            schedule = contracted_schedule(config.near, config.far, config.density_samples_per_ray)
    return torch.as_tensor(schedule, dtype=torch.float32, device="cuda").contiguous()


# ---------------------------------------------------------------------------------
# render_rays.
# ---------------------------------------------------------------------------------
def render_rays(appearance_mlp: networks.FeatureMlp, learnable_params: LearnableParams, aabb,
                rays_wrt_world: "cameras.Rays3D", prng_key: Union[NoiseKey, RenderNoise],
                config: RenderConfig, *, density_shift: float = 10.0, schedule=None,
                proposal: Optional[ProposalConfig] = None) -> torch.Tensor:
    """render.py:105-279. Output (R, 3) for RGB, (R,) for distances. With ``proposal``
    the density samples come from the proposal network (the model must have one)."""
    require_cuda()
    o = rays_wrt_world.origins.reshape(-1, 3)
    r = o.shape[0]
    sc = learnable_params.scene_contraction
    noise = prng_key if isinstance(prng_key, RenderNoise) else draw_noise(prng_key, r, config, sc, proposal)
    sched = _schedule_for(config, sc, schedule, proposal)
    desc = make_render_desc(config, aabb, noise, r, sc, sched, density_shift, proposal=proposal)
    md = learnable_params.model_desc()
    rs = rays_struct(rays_wrt_world)
    nbytes = _lib.load().tvm_render_workspace_size(ctypes.byref(md), ctypes.byref(desc), r)
    if nbytes == 0:
        raise ValueError("invalid render configuration: " + _lib.load().tvm_last_error_message().decode())
    ws = workspace(nbytes, o.device)
    shape = (r, 3) if config.mode is RenderMode.RGB else (r,)
    out = torch.empty(shape, dtype=torch.float32, device=o.device)
    _lib.call("tvm_render_fwd", ctypes.byref(md), ptr(learnable_params.params), ptr(learnable_params.shadow),
              ctypes.byref(rs), ctypes.byref(desc), ptr(out), ptr(ws), ws.numel(), stream_handle())
    return out


def render_rays_batched(appearance_mlp: networks.FeatureMlp, learnable_params: LearnableParams, aabb,
                        rays_wrt_world: "cameras.Rays3D", prng_key, config: RenderConfig, *,
                        batch_size: int = 4096, use_tqdm: bool = False, density_shift: float = 10.0,
                        to_host: bool = True, proposal: Optional[ProposalConfig] = None, schedule=None):
    """render.py:49-102: chunks of ``batch_size`` rays, concatenated. Rays stay on the
    device; ``to_host`` returns a NumPy array like the reference."""
    batch_axes = rays_wrt_world.origins.shape[:-1]
    o = rays_wrt_world.origins.reshape(-1, 3).to("cuda", torch.float32)
    d = rays_wrt_world.directions.reshape(-1, 3).to("cuda", torch.float32)
    ci = rays_wrt_world.camera_indices
    if ci is not None:
        ci = ci.reshape(-1).to("cuda", torch.int32).contiguous()
    total = o.shape[0]
    outs = []
    for start in range(0, total, batch_size):
        chunk = cameras.Rays3D(origins=o[start:start + batch_size], directions=d[start:start + batch_size],
                               camera_indices=ci[start:start + batch_size] if ci is not None else None)
        outs.append(render_rays(appearance_mlp, learnable_params, aabb, chunk, prng_key, config,
                                density_shift=density_shift, schedule=schedule, proposal=proposal))
    out = torch.cat(outs, dim=0)
    out = out.reshape(tuple(batch_axes) + tuple(out.shape[1:]))
    return out.cpu().numpy() if to_host else out


def loss_and_grad(learnable_params: LearnableParams, grads: torch.Tensor, aabb, rays_wrt_world,
                  colors: torch.Tensor, noise: RenderNoise, config: RenderConfig, *, density_shift: float = 10.0,
                  schedule=None, proposal: Optional[ProposalConfig] = None) -> torch.Tensor:
    """MSE of render_rays against colors and its gradient, ACCUMULATED into ``grads``
    (flat layout), plus the proposal bound loss's gradient when ``proposal`` is set.
    Returns the MSE as a device scalar."""
    o = rays_wrt_world.origins.reshape(-1, 3)
    r = o.shape[0]
    sc = learnable_params.scene_contraction
    sched = _schedule_for(config, sc, schedule, proposal)
    desc = make_render_desc(config, aabb, noise, r, sc, sched, density_shift, proposal=proposal)
    md = learnable_params.model_desc()
    rs = rays_struct(rays_wrt_world)
    nbytes = _lib.load().tvm_train_workspace_size(ctypes.byref(md), ctypes.byref(desc), r)
    if nbytes == 0:
        raise ValueError("invalid configuration: " + _lib.load().tvm_last_error_message().decode())
    ws = workspace(nbytes, o.device)
    loss = torch.zeros(1, dtype=torch.float32, device=o.device)
    _lib.call("tvm_loss_and_grad", ctypes.byref(md), ptr(learnable_params.params), ptr(learnable_params.shadow),
              ptr(grads), ctypes.byref(rs), ptr(colors.contiguous()), ctypes.byref(desc), ptr(loss), ptr(ws),
              ws.numel(), stream_handle())
    return loss


def loss_f64(learnable_params: LearnableParams, aabb, rays_wrt_world, colors: torch.Tensor, noise: RenderNoise,
             config: RenderConfig, *, density_shift: float = 10.0, perturb_index: int = -1,
             perturb_delta: float = 0.0) -> float:
    """The training loss evaluated in FP64 on the device, optionally with one flat
    parameter moved by ``perturb_delta``: central finite differences of the FP32
    gradients (bounded sampler, k == N, FP32 models)."""
    o = rays_wrt_world.origins.reshape(-1, 3)
    r = o.shape[0]
    desc = make_render_desc(config, aabb, noise, r, False, None, density_shift)
    md = learnable_params.model_desc()
    rs = rays_struct(rays_wrt_world)
    lib = _lib.load()
    nbytes = lib.tvm_loss_f64_workspace_size(ctypes.byref(md), ctypes.byref(desc), r)
    if nbytes == 0:
        raise ValueError("invalid FP64 loss configuration: " + lib.tvm_last_error_message().decode())
    ws = workspace(nbytes, o.device)
    out = torch.zeros(1, dtype=torch.float64, device=o.device)
    _lib.call("tvm_loss_f64", ctypes.byref(md), ptr(learnable_params.params), ctypes.byref(rs),
              ptr(colors.contiguous()), ctypes.byref(desc), int(perturb_index), float(perturb_delta), ptr(out),
              ptr(ws), ws.numel(), stream_handle())
    return float(out.item())


# ---------------------------------------------------------------------------------
# Seams.
# ---------------------------------------------------------------------------------
@dataclasses.dataclass
class SegmentProbabilities:
    """render.py:282-297."""
    p_exits: torch.Tensor
    p_terminates: torch.Tensor

    def get_batch_axes(self):
        return tuple(self.p_exits.shape)


class _Segment(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sigmas, steps):
        r, n = sigmas.shape
        pe = torch.empty_like(sigmas)
        pt = torch.empty_like(sigmas)
        _lib.call("tvm_composite_fwd", ptr(sigmas), ptr(steps), r, n, ptr(pe), ptr(pt), stream_handle())
        ctx.save_for_backward(sigmas, steps)
        return pe, pt

    @staticmethod
    def backward(ctx, gpe, gpt):
        sigmas, steps = ctx.saved_tensors
        r, n = sigmas.shape
        gs = torch.empty_like(sigmas)
        _lib.call("tvm_composite_bwd", ptr(sigmas), ptr(steps), r, n,
                  ptr(gpe.contiguous()) if gpe is not None else ptr(None),
                  ptr(gpt.contiguous()) if gpt is not None else ptr(None), ptr(gs), stream_handle())
        return gs, None


def compute_segment_probabilities(sigmas: torch.Tensor, step_sizes: torch.Tensor) -> SegmentProbabilities:
    """render.py:300-347 (sigmas and step_sizes of shape (*, N))."""
    batch = sigmas.shape
    s = sigmas.reshape(-1, batch[-1]).to(torch.float32).contiguous()
    st = step_sizes.reshape(-1, batch[-1]).to(torch.float32).contiguous()
    pe, pt = _Segment.apply(s, st)
    return SegmentProbabilities(pe.reshape(batch), pt.reshape(batch))


def sample_points(rays_wrt_world: "cameras.Rays3D", aabb, config: RenderConfig, noise: RenderNoise,
                  scene_contraction: bool = False, schedule=None):
    """The sampler of render_rays (render.py:122-190) plus normalisation
    (render.py:192-196): points (3, R, N) in [-1, 1], ts (R, N), step_sizes (R, N)."""
    r = rays_wrt_world.origins.reshape(-1, 3).shape[0]
    n = config.density_samples_per_ray
    sched = _schedule_for(config, scene_contraction, schedule)
    desc = make_render_desc(config, aabb, noise, r, scene_contraction, sched, 10.0, mode=RenderMode.DIST_MEAN)
    rs = rays_struct(rays_wrt_world)
    pts = torch.empty((3, r, n), dtype=torch.float32, device="cuda")
    ts = torch.empty((r, n), dtype=torch.float32, device="cuda")
    steps = torch.empty((r, n), dtype=torch.float32, device="cuda")
    _lib.call("tvm_sample_points", ctypes.byref(rs), ctypes.byref(desc), ptr(pts), ptr(ts), ptr(steps),
              stream_handle())
    return pts, ts, steps


def sample_points_along_ray_within_bbox(rays_wrt_world, aabb, samples_per_ray: int, jitter: Optional[torch.Tensor]):
    """render.py:350-390 vmapped over rays; un-normalised points (3, R, N), ts (R, N)
    and the per-ray step (R,)."""
    cfg = RenderConfig(near=0.0, far=1.0, mode=RenderMode.DIST_MEAN, density_samples_per_ray=samples_per_ray,
                       appearance_samples_per_ray=1)
    pts, ts, steps = sample_points(rays_wrt_world, aabb, cfg, RenderNoise(jitter=jitter, gumbel=None))
    a = torch.as_tensor(aabb, dtype=torch.float32, device="cuda").reshape(2, 3)
    world = (pts / 2.0 + 0.5) * (a[1] - a[0])[:, None, None] + a[0][:, None, None]
    return world, ts, steps[:, 0]


def weighted_choice(p: torch.Tensor, gumbel: torch.Tensor, k: int) -> torch.Tensor:
    """jax.random.choice(replace=False, p=p) per row with explicit Gumbel noise
    (render.py:459-470): the k largest log(p) + g, largest first, ties -> lower index."""
    r, n = p.shape
    idx = torch.empty((r, k), dtype=torch.int32, device=p.device)
    _lib.call("tvm_topk_select", ptr(p.contiguous()), ptr(gumbel.contiguous()), int(gumbel.dim() == 2), r, n, k,
              ptr(idx), stream_handle())
    return idx


# Proposal network seams: the stages of proposal-guided sampling that render_rays and
# training_step run fused, one call each. ``edges`` (Np + 1,) are the bin edges of
# unbounded scenes (learnable_params.scene_contraction); bounded scenes split each ray's
# aabb segment into Np uniform bins.
def _proposal_desc(aabb, proposal: ProposalConfig, rays: int, contract: bool, edges, proposal_jitter=None,
                   jitter=None, samples: int = 1):
    d = _lib.RenderDesc()
    d.sampler = _lib.TVM_SAMPLER_PROPOSAL
    d.proposal_samples = proposal.samples
    d.proposal_shift = proposal.shift
    d.proposal_loss_weight = proposal.loss_weight
    d.contract = int(contract)
    d.density_samples = samples
    d.appearance_samples = 1
    d.mode = _MODE_CODE[RenderMode.DIST_MEAN]
    for i, v in enumerate(_aabb6(aabb)):
        d.aabb[i] = v
    if contract and edges is None:
        raise ValueError("unbounded proposal sampling needs the Np + 1 bin edges")
    d.schedule = ptr(edges, torch.float32, "edges").value if contract else None
    d.proposal_jitter = ptr(proposal_jitter, torch.float32, "proposal_jitter").value \
        if proposal_jitter is not None else None
    d.jitter = ptr(jitter, torch.float32, "jitter").value if jitter is not None else None
    return d


def proposal_forward(learnable_params: LearnableParams, aabb, rays_wrt_world: "cameras.Rays3D",
                     proposal_jitter: torch.Tensor, proposal: ProposalConfig, edges: Optional[torch.Tensor] = None):
    """tvm_proposal_fwd: proposal densities sigmas (R, Np) at one jittered point per bin
    (proposal_jitter (R, Np)) and the bin lengths deltas (R, Np). The proposal weights
    are compute_segment_probabilities(sigmas, deltas).p_terminates."""
    r = rays_wrt_world.origins.reshape(-1, 3).shape[0]
    desc = _proposal_desc(aabb, proposal, r, learnable_params.scene_contraction, edges, proposal_jitter)
    md = learnable_params.model_desc()
    sig = torch.empty((r, proposal.samples), dtype=torch.float32, device="cuda")
    dl = torch.empty_like(sig)
    _lib.call("tvm_proposal_fwd", ctypes.byref(md), ptr(learnable_params.params), ptr(learnable_params.shadow),
              ctypes.byref(rays_struct(rays_wrt_world)), ctypes.byref(desc), ptr(sig), ptr(dl), stream_handle())
    return sig, dl


def proposal_backward(learnable_params: LearnableParams, grads: torch.Tensor, aabb, rays_wrt_world: "cameras.Rays3D",
                      proposal_jitter: torch.Tensor, proposal: ProposalConfig, sigmas: torch.Tensor,
                      grad_sigmas: torch.Tensor, edges: Optional[torch.Tensor] = None) -> None:
    """tvm_proposal_bwd: the gradient of the proposal sigmas proposal_forward returned,
    ACCUMULATED into the proposal segments of ``grads`` (flat layout)."""
    r = rays_wrt_world.origins.reshape(-1, 3).shape[0]
    desc = _proposal_desc(aabb, proposal, r, learnable_params.scene_contraction, edges, proposal_jitter)
    md = learnable_params.model_desc()
    _lib.call("tvm_proposal_bwd", ctypes.byref(md), ptr(learnable_params.params), ptr(learnable_params.shadow),
              ptr(grads), ctypes.byref(rays_struct(rays_wrt_world)), ctypes.byref(desc),
              ptr(sigmas, torch.float32, "sigmas"), ptr(grad_sigmas.contiguous(), torch.float32, "grad_sigmas"),
              stream_handle())


def proposal_resample(rays_wrt_world: "cameras.Rays3D", aabb, weights: torch.Tensor, jitter: torch.Tensor,
                      samples: int, proposal: ProposalConfig, scene_contraction: bool = False,
                      edges: Optional[torch.Tensor] = None):
    """tvm_proposal_resample: proposal weights (R, Np) -> ``samples`` main intervals at
    the quantiles of the padded histogram, one point each at jitter (R, N): ts, deltas
    (R, N) and the proposal bin of each interval edge, bins (R, N + 1) int32."""
    r = rays_wrt_world.origins.reshape(-1, 3).shape[0]
    desc = _proposal_desc(aabb, proposal, r, scene_contraction, edges, jitter=jitter, samples=samples)
    ts = torch.empty((r, samples), dtype=torch.float32, device="cuda")
    dl = torch.empty_like(ts)
    bins = torch.empty((r, samples + 1), dtype=torch.int32, device="cuda")
    _lib.call("tvm_proposal_resample", ctypes.byref(rays_struct(rays_wrt_world)), ctypes.byref(desc),
              ptr(weights.contiguous(), torch.float32, "weights"), ptr(ts), ptr(dl), ptr(bins), stream_handle())
    return ts, dl, bins


def proposal_loss(main_weights: torch.Tensor, proposal_weights: torch.Tensor, bins: torch.Tensor, scale: float):
    """tvm_proposal_loss: scale * sum of max(0, w - bound)^2 / (w + 1e-7) over the main
    intervals (bound: the proposal mass over each interval's bins) as a device scalar,
    and its gradient with respect to proposal_weights (R, Np)."""
    r, n = main_weights.shape
    npb = proposal_weights.shape[1]
    loss = torch.zeros(1, dtype=torch.float32, device=main_weights.device)
    g = torch.empty_like(proposal_weights)
    _lib.call("tvm_proposal_loss", ptr(main_weights.contiguous(), torch.float32, "main_weights"),
              ptr(proposal_weights.contiguous(), torch.float32, "proposal_weights"),
              ptr(bins.contiguous(), torch.int32, "bins"), r, npb, n, float(scale), ptr(loss), ptr(g),
              stream_handle())
    return loss, g
