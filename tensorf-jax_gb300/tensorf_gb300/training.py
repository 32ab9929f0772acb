"""GB300 twin of the training step of ``tensorf/training.py``.

``TrainState`` owns the flat parameter buffer, its gradient and Adam moments, and
runs one ``training_step`` as a single ``tvm_train_step`` call: sampling, density
VM, compositing and selection, appearance VM, MLP, MSE loss, the full backward and the
fused Adam update (training.py:101-205, 207-243). The learning-rate schedule and its
reset after grid upsampling (training.py:158-181) are host arithmetic.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Optional, Tuple

import numpy as onp
import torch

from . import _lib, cameras, render, utils
from ._util import ptr, stream_handle, workspace


@dataclasses.dataclass(frozen=True)
class OptimizerConfig:
    """train_config.py:6-12."""
    lr_init_tensor: float = 0.02
    lr_init_mlp: float = 1e-3
    lr_decay_iters: Optional[int] = None
    lr_decay_target_ratio: float = 0.1
    lr_upsample_reset: bool = True


@dataclasses.dataclass(frozen=True)
class TrainConfig:
    """The fields of TensorfConfig (train_config.py:15-71) the step uses."""
    minibatch_size: int = 4096
    n_iters: int = 30000
    optimizer: OptimizerConfig = OptimizerConfig()
    initial_aabb_min: Tuple[float, float, float] = (-1.0, -1.0, -1.0)
    initial_aabb_max: Tuple[float, float, float] = (1.0, 1.0, 1.0)
    upsamp_iters: Tuple[int, ...] = (2000, 3000, 4000, 5500, 7000)
    grid_dim_init: int = 128   # train_config.py:54
    grid_dim_final: int = 300  # train_config.py:55
    scene_contraction: bool = False
    # Plain contracted sampler: "reference" keeps render.py's heuristic schedule
    # (render.py:127-151), "disparity" spaces the samples linearly in disparity.
    contracted_spacing: str = "reference"
    render_near: float = 0.05
    render_far: float = 200.0
    train_ray_sample_multiplier: float = 1.0
    density_samples_per_ray: Optional[int] = None  # None: the reference heuristic
    appearance_samples_per_ray: Optional[int] = None
    density_shift: float = 10.0
    proposal: Optional["render.ProposalConfig"] = None  # proposal-guided sampling


def nerfstudio_preset(num_cameras: int) -> Tuple[TrainConfig, "render.ModelSpec"]:
    """The defaults real scenes in the nerfstudio format train with (train_nerfstudio.py:23-44):
    scene contraction, 2048 rays per step for 30000 steps, three times the sample-count
    heuristic, near / far 0.05 / 200, a 32-component density field and a 48-component
    appearance field grown from 128^3 to 300^3 at steps 2500, 5000 and 10000, six Fourier
    frequencies for features and view directions, and camera embeddings (FiLM, one row per
    training camera). Returns the training configuration and the model at its initial
    grid."""
    cfg = TrainConfig(minibatch_size=2048, n_iters=30000, initial_aabb_min=(-2.0, -2.0, -2.0),
                      initial_aabb_max=(2.0, 2.0, 2.0), upsamp_iters=(2_500, 5_000, 10_000), grid_dim_init=128,
                      grid_dim_final=300, scene_contraction=True, render_near=0.05, render_far=200.0,
                      train_ray_sample_multiplier=3.0)
    spec = render.ModelSpec(grid_dim=cfg.grid_dim_init, density_feat_dim=32, appearance_feat_dim=48,
                            feature_n_freqs=6, viewdir_n_freqs=6, num_cameras=int(num_cameras))
    return cfg, spec


def lr_decay_coeff(step: int, cfg: TrainConfig) -> float:
    """training.py:158-181 (optax.exponential_decay with end_value)."""
    o = cfg.optimizer
    if o.lr_upsample_reset:
        deltas = [step - s for s in (0,) + tuple(cfg.upsamp_iters)]
        s = min(d if d >= 0 else 2**31 - 1 for d in deltas)
    else:
        s = step
    di = cfg.n_iters if o.lr_decay_iters is None else o.lr_decay_iters
    if s <= 0:
        return 1.0
    v = float(onp.power(onp.float32(o.lr_decay_target_ratio), onp.float32(s) / onp.float32(di)))
    return max(v, o.lr_decay_target_ratio)


def upsampled_grid_dim(cfg: TrainConfig, train_step: int) -> Optional[int]:
    """The grid dimension training moves to at train_step, or None (training.py:358-367:
    linear from grid_dim_init to grid_dim_final over the upsampling iterations)."""
    if train_step not in cfg.upsamp_iters:
        return None
    index = cfg.upsamp_iters.index(train_step)
    return int(cfg.grid_dim_init + (cfg.grid_dim_final - cfg.grid_dim_init) * ((index + 1) / len(cfg.upsamp_iters)))


def sample_counts(grid_dim: int, cfg: TrainConfig) -> Tuple[int, int]:
    """training.py:115-118 heuristic unless overridden."""
    import math
    n = cfg.density_samples_per_ray or int(math.sqrt(3 * grid_dim**2) * cfg.train_ray_sample_multiplier)
    k = cfg.appearance_samples_per_ray or int(0.15 * n)
    return n, k


@dataclasses.dataclass
class _StepGraph:
    """A training step recorded as a CUDA graph, with the fixed-address buffers it reads:
    rays, colours and camera indices copied in before each replay, the noise buffers the
    recorded draws fill, the contracted sampler's schedule, and the step scalars (Adam
    count and learning-rate decay, the noise key's stream id) of the next step."""
    key: tuple
    origins: torch.Tensor
    directions: torch.Tensor
    colors: torch.Tensor
    camera_indices: Optional[torch.Tensor]
    noise: render.RenderNoise
    schedule: Optional[torch.Tensor]
    step_scalars: torch.Tensor  # tvm_step_scalars: int32 count, float32 lr_decay, uint64 noise stream
    graph: Optional[torch.cuda.CUDAGraph] = None
    launches: int = 0           # kernel launches recorded into the graph


class TrainState:
    """training.py:19-33 with the training step; mutated in place (the reference
    donates its state, training.py:101).

    The reference jit-compiles its step (training.py:101). The GPU counterpart here is a
    CUDA graph: with ``cuda_graph`` set, the first step for a batch size runs eagerly on
    fixed-address input, noise and step-scalar buffers and is then recorded once, noise
    draws included; later steps copy the batch in, write the step's Adam count,
    learning-rate decay and noise key into device memory and replay the graph. Steps
    given explicit ``noise`` run eagerly.

    With ``defer_field_updates`` (and a step that does not log), the step leaves the
    Adam update of the two VM fields pending; the next step applies it on a side stream
    beside its own start, before its gathers read the fields, so Adam's 0.5 GB stream
    overlaps the forward instead of ending the step. Reading ``learnable_params``,
    ``grads``, ``mu`` or ``nu`` applies a pending update first, so every value seen
    outside the step is the one the reference's sequential step would hold."""

    def __init__(self, config: TrainConfig, learnable_params: render.LearnableParams, seed: int = 94709,
                 cuda_graph: bool = True, defer_field_updates: bool = True):
        self.config = config
        self._pending: Optional[Tuple[int, float]] = None  # (count, lr decay) of a pending field update
        self._lp = learnable_params
        self.appearance_mlp = learnable_params.spec.mlp()
        p = learnable_params.params
        self._grads = torch.zeros_like(p)
        self._mu = torch.zeros_like(p)
        self._nu = torch.zeros_like(p)
        self.defer_field_updates = defer_field_updates
        self.aabb = torch.tensor([config.initial_aabb_min, config.initial_aabb_max], dtype=torch.float32)
        self.prng_key = render.NoiseKey(seed)
        self.step = 0
        # The step's MSE and the sum of its squared gradients, written on the device and
        # read back together when the step logs.
        self._stats = torch.zeros(2, dtype=torch.float32, device=p.device)
        self.loss = self._stats[0:1]
        self._ws = None
        self._ws_key = None
        self.cuda_graph = cuda_graph
        self._graphs: dict = {}  # one recorded step per deferral mode
        self._last_graph_mode: Optional[bool] = None
        self.graph_kernel_launches = 0  # kernels run by graph replays (the library counts eager launches)

    # Parameters, gradients and moments as seen from outside the step: a pending field
    # update is applied first.
    @property
    def learnable_params(self) -> render.LearnableParams:
        self.apply_pending()
        return self._lp

    @learnable_params.setter
    def learnable_params(self, value: render.LearnableParams) -> None:
        self.apply_pending()
        self._lp = value
        self._graphs = {}

    @property
    def grads(self) -> torch.Tensor:
        self.apply_pending()
        return self._grads

    @grads.setter
    def grads(self, value: torch.Tensor) -> None:
        self.apply_pending()
        self._grads = value
        self._graphs = {}

    @property
    def mu(self) -> torch.Tensor:
        self.apply_pending()
        return self._mu

    @mu.setter
    def mu(self, value: torch.Tensor) -> None:
        self.apply_pending()
        self._mu = value
        self._graphs = {}

    @property
    def nu(self) -> torch.Tensor:
        self.apply_pending()
        return self._nu

    @nu.setter
    def nu(self, value: torch.Tensor) -> None:
        self.apply_pending()
        self._nu = value
        self._graphs = {}

    @property
    def _graph(self) -> Optional[_StepGraph]:
        """The most recently used recorded step."""
        return self._graphs.get(self._last_graph_mode) if self._graphs else None

    def apply_pending(self) -> None:
        """Apply the field update the last step left pending (tvm_apply_pending_fields)."""
        if self._pending is None:
            return
        count, decay = self._pending
        self._pending = None
        lp = self._lp
        adam = self.adam_desc(count)
        adam.pending_count, adam.pending_lr_decay = count, decay
        _lib.call("tvm_apply_pending_fields", ctypes.byref(lp.model_desc()), ptr(lp.params), ptr(lp.shadow),
                  ptr(self._grads), ptr(self._mu), ptr(self._nu), ctypes.byref(adam), stream_handle())

    def _adam_for_step(self, defer: bool) -> _lib.AdamDesc:
        adam = self.adam_desc(self.step + 1)
        adam.defer_fields = int(defer)
        if self._pending is not None:
            adam.pending_count, adam.pending_lr_decay = self._pending
        return adam

    @staticmethod
    def initialize(config: TrainConfig, spec: render.ModelSpec, seed: int = 94709) -> "TrainState":
        lp = render.LearnableParams.initialize(spec, seed=seed, scene_contraction=config.scene_contraction)
        return TrainState(config, lp, seed=seed)

    def resize_grid(self, new_grid_dim: int) -> "TrainState":
        """TrainState.resize_grid (training.py:245-276): both VM tensors and their Adam
        moments resampled to new_grid_dim (tvm_resize_field), MLP and proposal network
        parameters and moments carried over, gradients zero. The step count is kept; the
        learning-rate decay restarts through upsamp_iters. Mutates and returns self."""
        lp = self.learnable_params
        old_g = lp.spec.grid_dim
        new_spec = dataclasses.replace(lp.spec, grid_dim=int(new_grid_dim))
        dev = lp.params.device
        new_lp = render.LearnableParams(new_spec, torch.zeros(render.param_layout(new_spec).total,
                                                               dtype=torch.float32, device=dev),
                                        scene_contraction=lp.scene_contraction)

        def transfer(src: torch.Tensor) -> torch.Tensor:
            dst = torch.zeros(new_lp.layout.total, dtype=torch.float32, device=dev)
            for which in ("density", "appearance"):
                sl, sp = lp.field_views(which, src)
                dl, dp = new_lp.field_views(which, dst)
                _lib.call("tvm_resize_field", old_g, int(new_grid_dim), sl.shape[-1], ptr(sl), ptr(sp), ptr(dl),
                          ptr(dp), stream_handle())
            new_mlp = new_lp.mlp_views(dst)
            for layer, tensors in lp.mlp_views(src).items():
                for name, t in tensors.items():
                    new_mlp[layer][name].copy_(t)
            if new_spec.proposal_grid:
                new_prop = new_lp.proposal_views(dst)
                for name, t in lp.proposal_views(src).items():
                    new_prop[name].copy_(t)
            return dst

        new_lp.params.copy_(transfer(lp.params))
        new_lp.refresh_shadow()
        self.mu = transfer(self.mu)
        self.nu = transfer(self.nu)
        self.grads = torch.zeros_like(new_lp.params)
        self.learnable_params = new_lp
        self.appearance_mlp = new_spec.mlp()
        self._ws = None
        self._ws_key = None
        self._graphs = {}
        return self

    def state_dict(self) -> dict:
        """The training state in the reference's array layout, on the CPU: params, Adam mu
        and nu as LearnableParams-shaped trees (density / appearance (vector (3,C,G),
        matrix (3,C,G,G)), flax "mlp" tree, "proposal"), the step and the model spec. The
        reference checkpoints the same TrainState fields through its experiment tooling
        (training.py:351-356); torch.save / numpy can store this dict."""
        lp = self.learnable_params
        return {"spec": dataclasses.asdict(lp.spec), "scene_contraction": lp.scene_contraction, "step": self.step,
                "aabb": self.aabb.clone(), "params": lp.to_reference(), "mu": lp.to_reference(self.mu),
                "nu": lp.to_reference(self.nu), "prng_key": dataclasses.asdict(self.prng_key)}

    @staticmethod
    def from_state_dict(config: TrainConfig, state: dict) -> "TrainState":
        """Inverse of state_dict(): device buffers rebuilt in this library's layout."""
        spec = render.ModelSpec(**state["spec"])
        lp = render.LearnableParams.from_reference(spec, state["params"], scene_contraction=state["scene_contraction"])
        ts = TrainState(config, lp)
        ts.mu = render.LearnableParams.from_reference(dataclasses.replace(spec, precision="fp32"), state["mu"]).params
        ts.nu = render.LearnableParams.from_reference(dataclasses.replace(spec, precision="fp32"), state["nu"]).params
        ts.step = int(state["step"])
        ts.aabb = state["aabb"].clone()
        ts.prng_key = render.NoiseKey(**state["prng_key"])
        return ts

    def render_config(self) -> render.RenderConfig:
        n, k = sample_counts(self._lp.spec.grid_dim, self.config)
        return render.RenderConfig(near=self.config.render_near, far=self.config.render_far,
                                   mode=render.RenderMode.RGB, density_samples_per_ray=n,
                                   appearance_samples_per_ray=k)

    def schedule(self) -> Optional[onp.ndarray]:
        """The contracted sampler's fixed schedule when it is not the reference one."""
        if not self._lp.scene_contraction or self.config.proposal is not None:
            return None
        if self.config.contracted_spacing == "disparity":
            cfg = self.render_config()
            return render.disparity_schedule(cfg.near, cfg.far, cfg.density_samples_per_ray)
        if self.config.contracted_spacing != "reference":
            raise ValueError(f"unknown contracted_spacing {self.config.contracted_spacing!r}")
        return None

    def adam_desc(self, count: int) -> _lib.AdamDesc:
        o = self.config.optimizer
        return _lib.AdamDesc(lr_tensor=o.lr_init_tensor, lr_mlp=o.lr_init_mlp, b1=0.9, b2=0.99, eps=1e-8,
                             lr_decay=lr_decay_coeff(self.step, self.config), count=count, defer_fields=0,
                             grad_sq=self._stats[1:].data_ptr())

    def training_step(self, rays: cameras.Rays3D, colors: torch.Tensor,
                      noise: Optional[render.RenderNoise] = None, log: bool = True):
        """One step: returns (self, log_data). ``noise`` replaces the key-drawn noise."""
        defer = self.defer_field_updates and not log  # a logged step reports its whole update
        if noise is None and self.cuda_graph:
            return self._graph_step(rays, colors, log, defer)
        cfg = self.render_config()
        r = rays.origins.reshape(-1, 3).shape[0]
        lp = self._lp
        prop = self.config.proposal
        if noise is None:
            render_key, self.prng_key = self.prng_key.split()
            noise = render.draw_noise(render_key, r, cfg, lp.scene_contraction, prop)
        sched = render._schedule_for(cfg, lp.scene_contraction, self.schedule(), prop)
        desc = render.make_render_desc(cfg, self.aabb, noise, r, lp.scene_contraction, sched,
                                       self.config.density_shift, proposal=prop)
        md = lp.model_desc()
        self._ensure_workspace(md, desc, r, cfg)
        adam = self._adam_for_step(defer)
        rs = render.rays_struct(rays)
        _lib.call("tvm_train_step", ctypes.byref(md), ptr(lp.params), ptr(lp.shadow), ptr(self._grads),
                  ptr(self._mu), ptr(self._nu), ctypes.byref(adam), ctypes.byref(rs), ptr(colors.contiguous()),
                  ctypes.byref(desc), ptr(self.loss), ptr(self._ws), self._ws.numel(), stream_handle())
        self._pending = (adam.count, adam.lr_decay) if defer else None
        self.step += 1
        return self, self._log(log, adam.lr_decay)

    def _log(self, log: bool, decay: float) -> dict:
        if not log:
            return {}
        # training.py:143-196: mse, psnr, both learning rates, the gradient's global norm
        mse, grad_sq = self._stats.tolist()
        return {"train/mse": mse, "train/psnr": utils.psnr_from_mse(mse),
                "train/lr_tensor": decay * self.config.optimizer.lr_init_tensor,
                "train/lr_mlp": decay * self.config.optimizer.lr_init_mlp,
                "train/grad_norm": math.sqrt(max(grad_sq, 0.0))}

    def _ensure_workspace(self, md, desc, r: int, cfg) -> None:
        key = (r, cfg)
        if self._ws_key != key:
            nbytes = _lib.load().tvm_train_workspace_size(ctypes.byref(md), ctypes.byref(desc), r)
            self._ws = workspace(nbytes, self._lp.params.device)
            self._ws_key = key

    def _graph_call(self, g: _StepGraph, cfg, r: int, defer: bool) -> None:
        """tvm_train_step on the graph's fixed buffers; the Adam scalars, the pending
        field update's and the noise key are read on the device."""
        lp = self._lp
        prop = self.config.proposal
        render.draw_noise_keyed(self.prng_key.seed, g.step_scalars, r, cfg, prop, g.noise)
        desc = render.make_render_desc(cfg, self.aabb, g.noise, r, lp.scene_contraction, g.schedule,
                                       self.config.density_shift, proposal=prop)
        md = lp.model_desc()
        self._ensure_workspace(md, desc, r, cfg)
        adam = self.adam_desc(1)
        adam.device_step = g.step_scalars.data_ptr()
        adam.defer_fields = int(defer)
        rs = render.rays_struct(cameras.Rays3D(g.origins, g.directions, g.camera_indices))
        _lib.call("tvm_train_step", ctypes.byref(md), ptr(lp.params), ptr(lp.shadow), ptr(self._grads),
                  ptr(self._mu), ptr(self._nu), ctypes.byref(adam), ctypes.byref(rs), ptr(g.colors),
                  ctypes.byref(desc), ptr(self.loss), ptr(self._ws), self._ws.numel(), stream_handle())

    def _graph_step(self, rays: cameras.Rays3D, colors: torch.Tensor, log: bool, defer: bool):
        cfg = self.render_config()
        lp = self._lp
        prop = self.config.proposal
        o = rays.origins.reshape(-1, 3)
        d = rays.directions.reshape(-1, 3)
        ci = rays.camera_indices
        r = o.shape[0]
        key = (r, cfg, self.config, ci is not None, lp.params.data_ptr(), lp.shadow.data_ptr() if lp.shadow is not None
               else 0, self._grads.data_ptr(), self._mu.data_ptr(), self._nu.data_ptr(), self.loss.data_ptr(),
               self.prng_key.seed, defer)
        g = self._graphs.get(defer)
        fresh = g is None or g.key != key
        if fresh:
            dev = lp.params.device
            sched = render._schedule_for(cfg, lp.scene_contraction, self.schedule(), prop)
            g = _StepGraph(key=key, origins=torch.empty((r, 3), dtype=torch.float32, device=dev),
                           directions=torch.empty((r, 3), dtype=torch.float32, device=dev),
                           colors=torch.empty((r, 3), dtype=torch.float32, device=dev),
                           camera_indices=torch.empty(r, dtype=torch.int32, device=dev) if ci is not None else None,
                           noise=render.draw_noise(render.NoiseKey(0), r, cfg, lp.scene_contraction, prop),
                           schedule=sched, step_scalars=torch.zeros(3, dtype=torch.int64, device=dev))
            self._graphs.pop(defer, None)
        render_key, self.prng_key = self.prng_key.split()
        for dst, src in ((g.origins, o), (g.directions, d), (g.colors, colors.reshape(-1, 3))):
            if dst.data_ptr() != src.data_ptr():
                dst.copy_(src)
        if ci is not None and g.camera_indices.data_ptr() != ci.data_ptr():
            g.camera_indices.copy_(ci.reshape(-1))
        decay = lr_decay_coeff(self.step, self.config)
        pend_count, pend_decay = self._pending if self._pending is not None else (0, 0.0)
        _lib.call("tvm_set_step_scalars", g.step_scalars.data_ptr(), self.step + 1, decay,
                  render_key.stream & (2**64 - 1), pend_count, pend_decay, stream_handle())
        if fresh:
            # This step runs eagerly on the graph's buffers (the library's one-time setup
            # happens here, outside any capture); the next ones replay its recording, the
            # noise draws included.
            self._graph_call(g, cfg, r, defer)
            lib = _lib.load()
            graph = torch.cuda.CUDAGraph()
            before = lib.tvm_kernel_launches()
            with torch.cuda.graph(graph, capture_error_mode="thread_local"):
                self._graph_call(g, cfg, r, defer)
            g.launches = int(lib.tvm_kernel_launches() - before)
            g.graph = graph
            self._graphs[defer] = g
        else:
            g.graph.replay()
            self.graph_kernel_launches += g.launches
        self._last_graph_mode = defer
        self._pending = (self.step + 1, decay) if defer else None
        self.step += 1
        return self, self._log(log, decay)
