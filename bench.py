"""Benchmark of the TensoRF-VM train step and full-frame render on one GB300.

Headline (`value`): the single-GPU training step of a 300^3 VM field with 16 / 48
components per mode, a 4096-ray batch with 512 uniform density samples per ray and
per-ray top-64 weighted selection of appearance samples, the FeatureMlp with
2-frequency encodings, MSE loss, full backward and Adam (lr 0.02 grids / 1e-3 MLP), all
FP32 ("plain FP32"). Beside it, in the same line:

* the same step with planes, lines and MLP in BF16 ("bf16"),
* the proposal-guided BF16 step: a 64^3 rank-4 proposal VM + 16-64-1 MLP, 64 proposal
  samples resampled to 48 field samples ("proposal_bf16"),
* held-out PSNR of each after the same number of training steps, the PSNR gap of the
  proposal path against plain FP32,
* full-frame render: 16 seeded 800x800 views (10.24M rays) in chunks of 65536 rays,
  rays/s for plain FP32 (512 samples) and proposal BF16, their PSNR against each
  other and the median-depth difference.

Targets come from an analytic scene of 32 random spheres (radius U[0.1, 0.4], density
50, RGB U[0, 1]) seen by seeded 800x800 cameras with focal length 1111, rendered by
FP64 quadrature with 4096 samples per ray. ``--impl reference`` times the CPU
restatement of the reference's algorithm (the oracle) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "tensorf-jax_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "train & render rays/s on 1 GB300: proposal+BF16 vs plain FP32 at ≤0.1 dB PSNR gap"
PHASES = ["proposal_fwd", "density_fwd", "composite_select", "appearance_fwd", "mlp_fwd", "color_loss",
          "mlp_bwd", "appearance_bwd", "composite_bwd", "density_bwd", "proposal_bwd", "adam"]


def variant_cfg(name: str, small: bool = False, prop_k: int = 7):
    w = dict(name=name, grid=300, Cd=16, Ca=48, R=4096, N=512, k=64, precision="fp32", proposal=None,
             prop_grid=0)
    if name == "bf16":
        w["precision"] = "bf16"
    if name == "proposal_bf16":
        w.update(precision="bf16", N=48, k=prop_k, proposal=64, prop_grid=64)
    if name.startswith("unbounded_"):
        # Unbounded scene: L-inf contraction to [-2, 2]^3, spacing linear in disparity,
        # 8192 rays per step, BF16; plain 512 samples vs proposal 64 -> 48.
        w.update(precision="bf16", R=8192, contract=True)
        if name == "unbounded_proposal_bf16":
            w.update(N=48, k=prop_k, proposal=64, prop_grid=64)
    if small:  # the same kernels on 1/4 of the rays, for profiler captures
        w["R"] //= 4
    return w


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------------
# Data and models.
# ---------------------------------------------------------------------------------
class Data:
    def __init__(self, R, seed=0, pool_batches=64, test_rays=8192):
        from tensorf_gb300 import scene

        self.sc = scene.SphereScene.random(seed, count=32)
        cams = self.sc.cameras(116, seed=seed + 1)
        self.train_cams, self.test_cams = cams[:100], cams[100:]
        self.R = R
        self.rays, self.colors = self.sc.training_rays(self.train_cams, R * pool_batches, seed=seed + 2,
                                                       n_samples=4096)
        self.test_rays, self.test_colors = self.sc.training_rays(self.test_cams, test_rays, seed=seed + 3,
                                                                 n_samples=4096)

    def batch(self, i):
        from tensorf_gb300 import cameras

        n = self.rays.origins.shape[0] // self.R
        j = i % n
        sl = slice(j * self.R, (j + 1) * self.R)
        return cameras.Rays3D(self.rays.origins[sl], self.rays.directions[sl]), self.colors[sl]


# Training starts directly at 300^3 (no coarse-to-fine upsampling), so the field starts
# half-transparent: softplus(0) = 0.69. With the reference's +10 the 300^3 field starts
# opaque and neither path recovers within the run; with -3 the uniform path starves.
DENSITY_SHIFT = 0.0
# Unbounded scene: step sizes are world distances that grow to hundreds of units at the
# far end, so the field starts more transparent (softplus(-3) = 0.05); 0 and -6 both
# train worse on both paths.
DENSITY_SHIFT_UNBOUNDED = -3.0
UNBOUNDED_NEAR, UNBOUNDED_FAR = 0.5, 1000.0


def shift_of(w):
    return DENSITY_SHIFT_UNBOUNDED if w.get("contract") else DENSITY_SHIFT


class UnboundedData:
    """Rays from inside radius 1 in uniform directions on the unbounded sphere scene."""

    def __init__(self, R, seed=0, pool_batches=32, test_rays=8192):
        from tensorf_gb300 import scene

        self.sc = scene.SphereScene.unbounded(seed + 5)
        self.R = R
        self.rays, self.colors = self.sc.unbounded_training_rays(R * pool_batches, seed=seed + 6)
        self.test_rays, self.test_colors = self.sc.unbounded_training_rays(test_rays, seed=seed + 7)

    def batch(self, i):
        from tensorf_gb300 import cameras

        n = self.rays.origins.shape[0] // self.R
        j = i % n
        sl = slice(j * self.R, (j + 1) * self.R)
        return cameras.Rays3D(self.rays.origins[sl], self.rays.directions[sl]), self.colors[sl]


def make_state(w, data):
    from tensorf_gb300 import render, training

    spec = render.ModelSpec(grid_dim=w["grid"], density_feat_dim=w["Cd"], appearance_feat_dim=w["Ca"],
                            precision=w["precision"], proposal_grid=w["prop_grid"])
    prop = render.ProposalConfig(samples=w["proposal"]) if w["proposal"] else None
    if w.get("contract"):
        cfg = training.TrainConfig(initial_aabb_min=(-2.0,) * 3, initial_aabb_max=(2.0,) * 3, scene_contraction=True,
                                   contracted_spacing="disparity", render_near=UNBOUNDED_NEAR,
                                   render_far=UNBOUNDED_FAR, density_samples_per_ray=w["N"],
                                   appearance_samples_per_ray=w["k"], n_iters=30000, upsamp_iters=(),
                                   density_shift=DENSITY_SHIFT_UNBOUNDED, proposal=prop)
    else:
        cfg = training.TrainConfig(initial_aabb_min=data.sc.aabb[0], initial_aabb_max=data.sc.aabb[1],
                                   density_samples_per_ray=w["N"], appearance_samples_per_ray=w["k"],
                                   n_iters=30000, upsamp_iters=(), density_shift=DENSITY_SHIFT, proposal=prop)
    return training.TrainState.initialize(cfg, spec, seed=94709)


def render_cfg(w, mode=None):
    from tensorf_gb300 import render

    return render.RenderConfig(0.05, 200.0, mode or render.RenderMode.RGB, w["N"], w["k"])


def proposal_of(w):
    from tensorf_gb300 import render

    return render.ProposalConfig(samples=w["proposal"]) if w["proposal"] else None


def max_over_ranks(ms, dist, device):
    """The slowest rank's time (ms); every rank gets it. dist is None on one process."""
    if dist is None:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rays_per_s(rays_per_step, steps, world, ms_max):
    """Whole-job throughput of replicas: every rank processes its own rays_per_step
    each step, the job ends with the slowest rank."""
    return rays_per_step * steps * world / (ms_max / 1e3)


def time_train(state, data, steps, warmup, phases=True, start_step=0):
    """Warm-up, then `steps` timed steps on device-resident batches. Returns (ms total,
    per-phase mean ms, kernel launches: the library's eager launches plus the kernels of
    the replayed CUDA graphs). A phase pass runs the steps eagerly: phase events are
    recorded by the library as it launches, and it applies each step's whole Adam update
    inside that step."""
    import ctypes

    from tensorf_gb300 import _lib

    lib = _lib.load()
    graph_was, defer_was = state.cuda_graph, state.defer_field_updates
    if phases:  # every kernel of a step inside its own phases
        state.cuda_graph = False
        state.defer_field_updates = False
    for i in range(warmup):
        r, c = data.batch(start_step + i)
        state.training_step(r, c, log=False)
    torch.cuda.synchronize()
    n_ev = len(PHASES) + 1
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(n_ev)] for _ in range(steps)] if phases else []
    for row in evs:  # torch creates events lazily: record once so the handles exist
        for e in row:
            e.record()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = lib.tvm_kernel_launches()
    g0 = state.graph_kernel_launches
    start.record()
    for i in range(steps):
        if phases:
            h = (ctypes.c_void_p * n_ev)(*[e.cuda_event for e in evs[i]])
            _lib.call("tvm_set_phase_events", h, n_ev)
        r, c = data.batch(start_step + warmup + i)
        state.training_step(r, c, log=False)
    _lib.call("tvm_set_phase_events", None, 0)
    end.record()
    torch.cuda.synchronize()
    state.cuda_graph, state.defer_field_updates = graph_was, defer_was
    launches = int(lib.tvm_kernel_launches() - l0) + int(state.graph_kernel_launches - g0)
    phase_ms = {}
    if phases:
        phase_ms = {p: statistics.mean(evs[i][j].elapsed_time(evs[i][j + 1]) for i in range(steps))
                    for j, p in enumerate(PHASES)}
    return start.elapsed_time(end), phase_ms, launches


def time_then_phases(state, data, steps, warmup):
    """The timed steps without per-phase events (their records would add to the step),
    then up to 50 more steps with them for the phase breakdown. Returns (ms total of the
    timed steps, per-phase mean ms, kernel launches of the timed steps, steps done)."""
    ms, _, launches = time_train(state, data, steps, warmup, phases=False)
    nph = min(steps, 50)
    _, phase_ms, _ = time_train(state, data, nph, 0, phases=True, start_step=warmup + steps)
    return ms, phase_ms, launches, warmup + steps + nph


def train_more(state, data, steps, start_step):
    """`steps` more training steps; returns their mean ms per step (CUDA events around
    the whole loop, nothing synchronised inside), or None for no steps."""
    if steps <= 0:
        return None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(steps):
        r, c = data.batch(start_step + i)
        state.training_step(r, c, log=False)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def psnr(a, b):
    return -10.0 * math.log10(max(float(((a - b) ** 2).mean()), 1e-10))


def eval_rays(state, w, rays, mode=None, chunk=65536):
    from tensorf_gb300 import render

    rc = render_cfg(w, mode)
    if w.get("contract"):
        rc = render.RenderConfig(UNBOUNDED_NEAR, UNBOUNDED_FAR, rc.mode, w["N"], w["k"])
    return render.render_rays_batched(state.appearance_mlp, state.learnable_params, state.aabb, rays,
                                      render.NoiseKey(12345), rc, batch_size=chunk,
                                      density_shift=shift_of(w), to_host=False, proposal=proposal_of(w),
                                      schedule=state.schedule())


def time_render(state, w, data, views, chunk=65536):
    """Full-frame render of `views` 800x800 views in chunks; device time of ray
    generation + render, rays/s."""
    from tensorf_gb300 import cameras, render

    cams = (data.test_cams * (1 + views // len(data.test_cams)))[:views]
    rc = render_cfg(w)
    prop = proposal_of(w)
    key = render.NoiseKey(777)
    rays = cams[0].pixel_rays_wrt_world()  # warm-up chunk
    render.render_rays(state.appearance_mlp, state.learnable_params, state.aabb,
                       cameras.Rays3D(rays.origins[:chunk], rays.directions[:chunk]), key, rc,
                       density_shift=DENSITY_SHIFT, proposal=prop)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total = 0
    img = None
    e0.record()
    for cam in cams:
        rays = cam.pixel_rays_wrt_world()
        n = rays.origins.shape[0]
        out = torch.empty((n, 3), device="cuda")
        for s in range(0, n, chunk):
            sub = cameras.Rays3D(rays.origins[s:s + chunk], rays.directions[s:s + chunk])
            out[s:s + chunk] = render.render_rays(state.appearance_mlp, state.learnable_params, state.aabb, sub, key,
                                                  rc, density_shift=DENSITY_SHIFT, proposal=prop)
        total += n
        img = out
    e1.record()
    torch.cuda.synchronize()
    return total / (e0.elapsed_time(e1) / 1e3), img


def scene_truth_comparison(states, data, views, per_view=4096, seed=5):
    """Full-frame render scored against the FP64 scene itself, on a seeded subset of
    `per_view` pixels of each of the `views` rendered views: PSNR of each path against
    the FP64 quadrature colours (4096 samples per ray) and the mean absolute error of its
    DIST_MEDIAN depth against the analytic median depth (SphereScene.median_depth), over
    rays where both are finite, plus how often both agree on whether the ray
    terminates."""
    from tensorf_gb300 import cameras, render

    cams = (data.test_cams * (1 + views // len(data.test_cams)))[:views]
    rng = np.random.default_rng(seed)
    os_, ds_ = [], []
    for cam in cams:
        pix = torch.as_tensor(rng.integers(0, cam.image_width * cam.image_height, size=per_view))
        rr = cam.pixel_rays_wrt_world(pix)
        os_.append(rr.origins)
        ds_.append(rr.directions)
    rays = cameras.Rays3D(torch.cat(os_), torch.cat(ds_))
    target = data.sc.render(rays, 4096)
    truth = torch.as_tensor(data.sc.median_depth(rays.origins.cpu().numpy(), rays.directions.cpu().numpy()))
    out = {"pixels": views * per_view, "views": views}
    for name in ("plain_fp32", "proposal_bf16"):
        w, st, _ = states[name]
        img = eval_rays(st, w, rays)
        dep = eval_rays(st, w, rays, render.RenderMode.DIST_MEDIAN).cpu().double()
        both = torch.isfinite(dep) & torch.isfinite(truth)
        out[name] = {"psnr_vs_fp64_db": round(psnr(img, target), 3),
                     "median_depth_abs_err_vs_fp64": round(float((dep[both] - truth[both]).abs().mean()), 5),
                     "termination_agree_vs_fp64": round(float((torch.isfinite(dep) == torch.isfinite(truth))
                                                              .float().mean()), 4)}
    return out


def algorithmic_bytes(w, phase):
    """Algorithmic bytes of one launch of each gather/scatter phase."""
    R, N, k = w["R"], w["N"], w["k"]
    s = 2 if w["precision"] == "bf16" else 4
    dens_el, app_el = 18 * w["Cd"], 18 * w["Ca"]
    G = w["grid"]
    n_field = 3 * G * (G + 1) * (w["Cd"] + w["Ca"])
    if w["prop_grid"]:
        n_field += 3 * w["prop_grid"] * (w["prop_grid"] + 1) * 4
    n_params = n_field + 40115
    return {
        "density_fwd": R * N * dens_el * s + R * N * 4,
        "density_bwd": R * N * dens_el * (s + 4) + R * N * 4,
        "appearance_fwd": R * k * app_el * s + R * k * 3 * w["Ca"] * 4,
        "appearance_bwd": R * k * app_el * (s + 4) + R * k * 3 * w["Ca"] * 4,
        # p, g, m, v read; p, m, v, zeroed g written; plus the bf16 shadow of the field.
        "adam": n_params * 32 + (n_field * 2 if w["precision"] == "bf16" else 0),
    }.get(phase)


def mlp_flops(w, phase):
    """Dense-layer FLOPs of the FeatureMlp per step: forward 2 * rows * 39856 (one
    multiply-add per weight per row at 2-frequency encodings), backward twice that."""
    rows = w["R"] * w["k"]
    per_row = 144 * 27 + 150 * 128 + 128 * 128 + 128 * 3
    return {"mlp_fwd": 2 * rows * per_row, "mlp_bwd": 4 * rows * per_row}.get(phase)


# Phases that are one kernel launch in the single-stream pass, with the kernel the
# headline workload runs (N >= 128 and k >= 32 select the pair-merging scatters).
SINGLE_KERNEL_PHASES = {"density_fwd": "density_fwd_kernel", "appearance_fwd": "appearance_fwd_kernel",
                        "density_bwd": "density_bwd2_kernel", "appearance_bwd": "appearance_bwd2_kernel",
                        "adam": "adam_kernel"}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the headline
# step's kernels, from one ncu capture of the full-size workload; the command and the
# per-kernel figures are in profiles/dram_traffic_train_fp32_300grid_4096rays.md.
NCU_DRAM_BYTES_PER_LAUNCH = {"density_bwd": 46.4e6}


def roofline_for(w, phase_ms, l2):
    """The dominant kernel of the headline step, the longest single-kernel phase.
    The field gathers and scatters work on L2-resident fields, so their bound is L2:
    for a scatter, the algorithmic reduction bytes (one 4-byte reduction per gathered
    element) over the measured L2 float4-reduction bandwidth; its HBM figures are kept
    beside it with the DRAM traffic ncu measured."""
    hbm, bf16, src = measured_peaks()
    dom = max((p for p in SINGLE_KERNEL_PHASES if phase_ms.get(p)), key=lambda p: phase_ms[p])
    ms = phase_ms[dom]
    alg = algorithmic_bytes(w, dom)
    hbm_part = {"achieved": round(alg / (ms / 1e3) / 1e9, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(alg / (ms / 1e3) / 1e9 / hbm, 4), "peak_source": src}
    traffic = NCU_DRAM_BYTES_PER_LAUNCH.get(dom)
    if dom in ("density_bwd", "appearance_bwd") and l2:
        red = gather_scatter_bytes(w, dom)[1]
        gbs = red / (ms / 1e3) / 1e9
        return {"bound": "l2", "kernel": SINGLE_KERNEL_PHASES[dom], "achieved": round(gbs, 1),
                "peak": l2["l2_red_gbs"], "unit": "GB/s", "frac": round(gbs / l2["l2_red_gbs"], 4),
                "traffic": traffic, "algorithmic_bytes": alg, "reduction_bytes": red, "ms": round(ms, 4),
                "hbm": hbm_part, "peak_source": "measured: tvm_l2_probe float4 reductions in this run",
                "note": "L2-resident scatter: reductions over the measured L2 reduction bandwidth; traffic is "
                        "the DRAM bytes ncu measured for one launch at this size"}
    return {"bound": "hbm", "kernel": SINGLE_KERNEL_PHASES[dom], "achieved": hbm_part["achieved"], "peak": hbm,
            "unit": "GB/s", "frac": hbm_part["frac"], "traffic": traffic, "algorithmic_bytes": alg,
            "ms": round(ms, 4), "peak_source": src}


def measure_tf32_peak(n=8192, launches=5):
    """cuBLAS TF32 GEMM throughput on this GPU (fp32 n x n x n with TF32 tensor cores),
    TFLOP/s, best of `launches`: the denominator of the split-tf32 FeatureMlp, which
    issues three TF32 products per FP32 product."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        g = torch.Generator(device="cuda").manual_seed(0)
        a = torch.randn(n, n, device="cuda", generator=g)
        b = torch.randn(n, n, device="cuda", generator=g)
        for _ in range(3):
            a @ b
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(launches):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return {"tflops": round(2 * n ** 3 / (best / 1e3) / 1e12, 1), "n": n,
            "how": "torch fp32 matmul with TF32 tensor cores (cuBLAS), best of 5"}


def measure_l2_peaks(mb=48, passes=20, launches=5):
    """L2 read and float4-reduction bandwidth of this GPU (tvm_l2_probe over an
    L2-resident buffer), GB/s of buffer bytes, best of `launches` timed launches."""
    from tensorf_gb300 import _lib
    from tensorf_gb300._util import ptr, stream_handle

    nbytes = mb << 20
    buf = torch.zeros(nbytes // 4, dtype=torch.float32, device="cuda")
    out = {}
    for kind, name in ((0, "l2_read_gbs"), (1, "l2_red_gbs")):
        _lib.call("tvm_l2_probe", kind, ptr(buf), nbytes, 2, stream_handle())  # warm L2
        best = float("inf")
        for _ in range(launches):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.call("tvm_l2_probe", kind, ptr(buf), nbytes, passes, stream_handle())
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = round(nbytes * passes / (best / 1e3) / 1e9, 1)
    out["buffer_mb"] = mb
    out["how"] = ("tvm_l2_probe: 4 CTAs x 512 threads per SM stream a 48 MiB buffer 20 times per launch with 16-byte "
                  "L1-bypassing loads (read) or float4 reductions to distinct addresses (red); best of 5 launches")
    return out


def gather_scatter_bytes(w, phase):
    """(L2 read bytes, L2 reduction bytes) of one launch of a gather or scatter phase."""
    R, N, k = w["R"], w["N"], w["k"]
    s = 2 if w["precision"] == "bf16" else 4
    dens_el, app_el = 18 * w["Cd"], 18 * w["Ca"]
    return {"density_fwd": (R * N * dens_el * s, 0), "density_bwd": (R * N * dens_el * s, R * N * dens_el * 4),
            "appearance_fwd": (R * k * app_el * s, 0),
            "appearance_bwd": (R * k * app_el * s, R * k * app_el * 4)}.get(phase)


def kernel_rooflines(w, phase_ms, l2, tf32=None):
    """Per phase: achieved algorithmic GB/s (or TFLOP/s for the MLP) and its fraction of
    the peak that bounds it: HBM for Adam, L2 (read + reduction time) for the field
    gathers and scatters, the tensor pipe for the MLP (the measured bf16 peak, or for
    split-tf32 one third of the measured TF32 peak)."""
    hbm, bf16, _ = measured_peaks()
    out = {}
    for ph in ("density_fwd", "appearance_fwd", "density_bwd", "appearance_bwd", "adam", "mlp_fwd", "mlp_bwd"):
        ms = phase_ms.get(ph)
        if not ms:
            continue
        if ph in ("mlp_fwd", "mlp_bwd"):
            tf = mlp_flops(w, ph) / (ms / 1e3) / 1e12
            if w["precision"] == "bf16":
                peak = bf16
            else:
                peak = tf32["tflops"] / 3.0 if tf32 else bf16 / 6.0
            out[ph] = {"ms": round(ms, 4), "tflops": round(tf, 1), "frac_tensor": round(tf / peak, 3)}
            continue
        b = algorithmic_bytes(w, ph)
        e = {"ms": round(ms, 4), "gbs": round(b / (ms / 1e3) / 1e9, 1),
             "frac_hbm": round(b / (ms / 1e3) / 1e9 / hbm, 3)}
        rb = gather_scatter_bytes(w, ph)
        if rb and l2:
            t_l2 = rb[0] / (l2["l2_read_gbs"] * 1e9) + rb[1] / (l2["l2_red_gbs"] * 1e9)
            e["frac_l2"] = round(t_l2 / (ms / 1e3), 3)
        out[ph] = e
    return out


def run_profile_variant(args):
    """Only one variant's warm-up and timed steps (for profiler launch lists)."""
    from tensorf_gb300 import _lib

    _lib.load()
    w = variant_cfg(args.profile_variant, args.small, args.prop_k)
    data = UnboundedData(w["R"], pool_batches=8, test_rays=256) if w.get("contract") else \
        Data(w["R"], pool_batches=8, test_rays=256)
    st = make_state(w, data)
    ms, ph, launches = time_train(st, data, args.steps, args.warmup)
    print(json.dumps({"variant": w["name"], "ms_per_step": round(ms / args.steps, 4), "launches": launches,
                      "phase_ms": {p: round(v, 4) for p, v in ph.items()}}), flush=True)


def run_ours(args):
    from tensorf_gb300 import _lib, cameras, render

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    _lib.load()
    plain = variant_cfg("plain_fp32", args.small)
    data = Data(plain["R"], seed=rank)
    torch.cuda.synchronize()

    # Headline: plain FP32 train step, device-resident batches.
    st_plain = make_state(plain, data)
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        ms, _, launches = time_train(st_plain, data, args.steps, args.warmup, phases=False)
    if dist:
        dist.barrier()
    ms = max_over_ranks(ms, dist, "cuda")
    value = job_rays_per_s(plain["R"], args.steps, world, ms)
    # Phase breakdown in a separate pass: per-phase events add records to the stream.
    nph = min(args.steps, 50)
    _, phase_ms, _ = time_train(st_plain, data, nph, 0, phases=True, start_step=args.warmup + args.steps)
    done_plain = args.warmup + args.steps + nph
    l2 = measure_l2_peaks()
    tf32 = measure_tf32_peak()

    # End to end through the public API: pinned host rays and colours copied in every
    # step, the loss read back every step.
    R = plain["R"]
    host_o = data.rays.origins.cpu().pin_memory()
    host_d = data.rays.directions.cpu().pin_memory()
    host_c = data.colors.cpu().pin_memory()
    dev_o, dev_d, dev_c = (torch.empty((R, 3), device="cuda") for _ in range(3))
    loss_host = torch.empty(1).pin_memory()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    npool = host_o.shape[0] // R
    for i in range(args.steps):
        sl = slice((i % npool) * R, (i % npool + 1) * R)
        dev_o.copy_(host_o[sl], non_blocking=True)
        dev_d.copy_(host_d[sl], non_blocking=True)
        dev_c.copy_(host_c[sl], non_blocking=True)
        st_plain.training_step(cameras.Rays3D(dev_o, dev_d), dev_c, log=False)
        loss_host.copy_(st_plain.loss, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    done_plain += args.steps
    e2e_ms = max_over_ranks(e2e_ms, dist, "cuda")
    e2e_value = job_rays_per_s(R, args.steps, world, e2e_ms)

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": DATA,
        "config": headline_config(plain, world),
        "phase_ms": {p: round(v, 4) for p, v in phase_ms.items()},
        "e2e": {"value": round(e2e_value, 1), "unit": "rays/s", "h2d_bytes_per_step": R * 9 * 4,
                "d2h_bytes_per_step": 4},
        "gpu_launches": launches,
        "roofline": roofline_for(plain, phase_ms, l2),
        "l2_peaks": l2,
        "tf32_peak": tf32,
        "kernels": kernel_rooflines(plain, phase_ms, l2, tf32),
        "clocks": clk.summary(),
    }

    if not args.headline_only and world == 1:
        variants = {"plain_fp32": {"train_rays_per_s": round(value, 1), "ms_per_step": round(ms / args.steps, 4)}}
        states = {"plain_fp32": (plain, st_plain, done_plain)}
        for name in ("bf16", "proposal_bf16"):
            w = variant_cfg(name, args.small, args.prop_k)
            st = make_state(w, data)
            vms, vph, _, vdone = time_then_phases(st, data, args.steps, args.warmup)
            variants[name] = {"train_rays_per_s": round(w["R"] * args.steps / (vms / 1e3), 1),
                              "ms_per_step": round(vms / args.steps, 4),
                              "phase_ms": {p: round(v, 4) for p, v in vph.items()},
                              "kernels": kernel_rooflines(w, vph, l2, tf32),
                              "density_samples": w["N"], "appearance_samples": w["k"],
                              "proposal_samples": w["proposal"]}
            states[name] = (w, st, vdone)
        # The same number of training steps for every variant, then held-out PSNR. The
        # proposal path's step gets cheaper as its network learns where the surfaces are,
        # so the step is also timed over the whole training run and once trained.
        for name, (w, st, done) in states.items():
            n_more = max(0, args.train_steps - done)
            run_ms = train_more(st, data, n_more, done)
            img = eval_rays(st, w, data.test_rays)
            variants[name]["psnr_db"] = round(psnr(img, data.test_colors), 3)
            variants[name]["train_steps"] = max(args.train_steps, done)
            if run_ms is not None:
                variants[name]["training_run"] = {"steps": n_more, "first_step": done,
                                                  "ms_per_step": round(run_ms, 4),
                                                  "rays_per_s": round(w["R"] / (run_ms / 1e3), 1)}
            tms, _, _ = time_train(st, data, args.steps, args.warmup, phases=False, start_step=done + n_more)
            variants[name]["trained"] = {"after_steps": done + n_more + args.warmup,
                                         "ms_per_step": round(tms / args.steps, 4),
                                         "rays_per_s": round(w["R"] * args.steps / (tms / 1e3), 1)}
        # Full-frame render: plain FP32 (512 samples) vs proposal BF16.
        imgs = {}
        for name in ("plain_fp32", "proposal_bf16"):
            w, st, _ = states[name]
            rps, img = time_render(st, w, data, args.render_views)
            variants[name]["render_rays_per_s"] = round(rps, 1)
            imgs[name] = img
        rp, rq = variants["plain_fp32"]["render_rays_per_s"], variants["proposal_bf16"]["render_rays_per_s"]
        # Median depth of the held-out rays under both paths.
        w0, s0, _ = states["plain_fp32"]
        w1, s1, _ = states["proposal_bf16"]
        d0 = eval_rays(s0, w0, data.test_rays, render.RenderMode.DIST_MEDIAN)
        d1 = eval_rays(s1, w1, data.test_rays, render.RenderMode.DIST_MEDIAN)
        both = torch.isfinite(d0) & torch.isfinite(d1)
        line["variants"] = variants
        line["comparison"] = {
            "train_speedup_proposal_bf16_vs_plain_fp32": round(variants["proposal_bf16"]["train_rays_per_s"] / value, 3),
            "train_speedup_trained": round(variants["plain_fp32"]["trained"]["ms_per_step"] /
                                           variants["proposal_bf16"]["trained"]["ms_per_step"], 3),
            "train_speedup_over_training_run": (
                round(variants["plain_fp32"]["training_run"]["ms_per_step"] /
                      variants["proposal_bf16"]["training_run"]["ms_per_step"], 3)
                if "training_run" in variants["plain_fp32"] and "training_run" in variants["proposal_bf16"]
                else None),
            "render_speedup_proposal_bf16_vs_plain_fp32": round(rq / rp, 3),
            "psnr_gap_db_plain_minus_proposal_bf16": round(variants["plain_fp32"]["psnr_db"] -
                                                          variants["proposal_bf16"]["psnr_db"], 3),
            "render_psnr_proposal_vs_plain_db": round(psnr(imgs["proposal_bf16"], imgs["plain_fp32"]), 3),
            "median_depth_abs_diff_mean": round(float((d0[both] - d1[both]).abs().mean()), 5) if both.any() else None,
            "median_depth_terminated_agree": round(float((torch.isfinite(d0) == torch.isfinite(d1)).float().mean()), 4),
            "render_views": args.render_views, "render_chunk": 65536,
            "against_fp64_scene": scene_truth_comparison(states, data, args.render_views),
        }
    if not args.headline_only and world == 1:
        line["unbounded"] = run_unbounded(args)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(plain, args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_unbounded(args):
    """Unbounded scene (contraction to [-2, 2]^3, 8192 rays, BF16): proposal 64 -> 48
    vs plain 512 samples, both spaced linearly in disparity. Train rays/s over the timed
    steps, then held-out PSNR after the same number of steps."""
    out = {}
    data = None
    for name in ("unbounded_plain_bf16", "unbounded_proposal_bf16"):
        w = variant_cfg(name, args.small, args.prop_k)
        if data is None:
            data = UnboundedData(w["R"])
        st = make_state(w, data)
        ms, ph, _, done = time_then_phases(st, data, args.steps, args.warmup)
        train_more(st, data, max(0, args.train_steps - done), done)
        img = eval_rays(st, w, data.test_rays)
        out[name] = {"train_rays_per_s": round(w["R"] * args.steps / (ms / 1e3), 1),
                     "ms_per_step": round(ms / args.steps, 4), "phase_ms": {p: round(v, 4) for p, v in ph.items()},
                     "rays_per_step": w["R"], "density_samples": w["N"], "appearance_samples": w["k"],
                     "proposal_samples": w["proposal"], "psnr_db": round(psnr(img, data.test_colors), 3),
                     "train_steps": max(args.train_steps, done)}
    p, q = out["unbounded_plain_bf16"], out["unbounded_proposal_bf16"]
    out["train_speedup_proposal_vs_plain"] = round(q["train_rays_per_s"] / p["train_rays_per_s"], 3)
    out["psnr_gap_db_plain_minus_proposal"] = round(p["psnr_db"] - q["psnr_db"], 3)
    out["scene"] = ("128 spheres at distances 2..12 around the origin, rays from inside radius 1 in uniform "
                    "directions, FP64 quadrature targets (8192 samples per ray)")
    out["density_shift"] = DENSITY_SHIFT_UNBOUNDED
    return out


# ---------------------------------------------------------------------------------
# CPU: the oracle restatement of the reference algorithm on the host cores.
# ---------------------------------------------------------------------------------
class CpuTrainer:
    """The headline training step run by the float32 oracle on the host cores: the same
    initial parameters, sphere-scene rays and FP64 quadrature targets as the GPU arm
    (rebuilt on the host, without the CUDA library), forward + backward by torch
    autograd, and optax's Adam with its moments kept across steps."""

    def __init__(self, w, rays_per_step, batches=1, seed=0):
        from oracle import tensorf_oracle as O
        from tensorf_gb300 import render, scene

        self.O, self.w, self.R = O, w, rays_per_step
        spec = render.ModelSpec(grid_dim=w["grid"], density_feat_dim=w["Cd"], appearance_feat_dim=w["Ca"])
        ref = render.initial_reference_params(spec, seed=94709)
        self.fields = [*ref["density"], *ref["appearance"]]
        self.mlp = [t for d in ref["mlp"].values() for t in d.values()]
        self.params = ref
        for t in self.fields + self.mlp:
            t.requires_grad_(True)
        self.mu = [torch.zeros_like(t) for t in self.fields + self.mlp]
        self.nu = [torch.zeros_like(t) for t in self.fields + self.mlp]
        self.count = 0
        # Rays of the GPU arm's first batches (Data(): scene seed 0, cameras seed 1,
        # pixels seed 2) and their FP64 quadrature targets.
        sc = scene.SphereScene.random(seed, count=32)
        cams = sc.cameras(116, seed=seed + 1)[:100]
        cam_idx, pix = scene.SphereScene.training_pixels(cams, w["R"] * 64, seed=seed + 2)
        n = rays_per_step * batches
        o = np.empty((n, 3))
        d = np.empty((n, 3))
        for i, cam in enumerate(cams):
            sel = np.nonzero(cam_idx[:n] == i)[0]
            if sel.size:
                o[sel], d[sel] = O.camera_pixel_rays(cam.K, cam.R_world_camera, cam.t_world_camera,
                                                     cam.image_width, cam.image_height, pixels=pix[sel])
        aabb64 = torch.tensor(sc.aabb, dtype=torch.float64)
        t0, t1 = O.ray_segment_from_bounding_box(torch.tensor(o), torch.tensor(d), aabb64)
        c = O.sphere_scene_quadrature(o, d, sc.centers, sc.radii, sc.colors, sc.density, t0.numpy(), t1.numpy(),
                                      4096)
        self.o = torch.tensor(o, dtype=torch.float32)
        self.d = torch.tensor(d, dtype=torch.float32)
        self.c = torch.tensor(c, dtype=torch.float32)
        self.aabb = torch.tensor(sc.aabb, dtype=torch.float32)
        self.gen = torch.Generator().manual_seed(seed + 9)
        self.batches = batches

    def step(self, i):
        O, w, R = self.O, self.w, self.R
        sl = slice((i % self.batches) * R, (i % self.batches + 1) * R)
        jit = torch.rand(w["N"], generator=self.gen)
        gum = -torch.log(-torch.log(torch.rand(w["N"], generator=self.gen).clamp_min(1e-7)))
        out = O.render_rays(self.params, self.aabb, self.o[sl], self.d[sl], w["N"], w["k"], jit, gum,
                            density_shift=DENSITY_SHIFT)
        loss = O.mse(out, self.c[sl])
        leaves = self.fields + self.mlp
        grads = torch.autograd.grad(loss, leaves)
        self.count += 1
        with torch.no_grad():
            for j, (t, g) in enumerate(zip(leaves, grads)):
                lr = 0.02 if j < len(self.fields) else 1e-3
                new, self.mu[j], self.nu[j] = O.adam_update(t, g, self.mu[j], self.nu[j], self.count, lr=lr,
                                                            lr_decay=1.0)
                t.copy_(new)
        return float(loss.detach())


def cpu_rays_per_step(w, budget_s, steps):
    """Rays per CPU step so that `steps` steps take about budget_s: the largest multiple of
    256 up to the full batch, from one measured 256-ray step (its fixed Adam cost makes
    the estimate conservative)."""
    t = time.perf_counter()
    CpuTrainer(w, 256).step(0)
    per_ray = (time.perf_counter() - t) / 256
    fit = int(budget_s / max(steps, 1) / per_ray) // 256 * 256
    return max(256, min(w["R"], fit))


def cpu_train(w, steps, warmup, budget_s):
    """Times `steps` oracle train steps after `warmup` untimed ones. Returns (rays/s, rays
    per step, threads, seconds per step)."""
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    R = cpu_rays_per_step(w, budget_s, steps + warmup)
    tr = CpuTrainer(w, R)
    for i in range(warmup):
        tr.step(i)
    t = time.perf_counter()
    for i in range(steps):
        tr.step(warmup + i)
    dt = time.perf_counter() - t
    return R * steps / dt, R, threads, dt / steps


def cpu_sample_text(w, R, steps, warmup):
    return (f"oracle (torch CPU float32) train steps of {R} of the {w['R']} sphere-scene rays of the GPU arm's "
            f"first batch, forward + backward + Adam over all parameters, {steps} timed after {warmup} warm-up; "
            f"rays/s measured, not scaled")


def cpu_baseline(w, args):
    steps, warmup = 4, 1
    value, R, threads, _ = cpu_train(w, steps, warmup, budget_s=25.0)
    return {"value": round(value, 2), "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": cpu_sample_text(w, R, steps, warmup)}


def headline_config(w, world):
    return {"workload": f"train step fp32: grid {w['grid']}^3, VM {w['Cd']}/{w['Ca']}, "
                        f"{w['R']} rays x {w['N']} uniform samples, top-{w['k']} appearance, Adam",
            "rays_per_step": w["R"], "density_samples": w["N"], "appearance_samples": w["k"],
            "grid": w["grid"], "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": "no flush: each step streams params+grads+Adam moments (277 MB) and >2 GB of per-sample "
                  "work, both larger than the 126 MB L2"}


DATA = "synthetic (32-sphere analytic scene, FP64 quadrature targets, seeded cameras)"


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w = variant_cfg("plain_fp32", args.small)
    value, R, threads, step_s = cpu_train(w, args.steps, args.warmup, budget_s=args.reference_budget_s)
    config = headline_config(w, 1)
    config["rays_per_step"] = R
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "rays/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": config,
        "cpu_baseline": {"value": round(value, 2), "unit": "rays/s", "cores": threads, "kind": "port",
                         "sample": cpu_sample_text(w, R, args.steps, args.warmup)},
        "e2e": {"value": round(value, 2), "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is JAX and JAX is not installed: this is the CPU restatement of its algorithm",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--small", action="store_true", help="1024-ray case for profiler captures")
    ap.add_argument("--headline-only", action="store_true", help="only the plain FP32 train step")
    ap.add_argument("--train-steps", type=int, default=2000, help="training steps before the PSNR comparison")
    ap.add_argument("--render-views", type=int, default=16)
    ap.add_argument("--prop-k", type=int, default=7,
                    help="appearance samples of the proposal path (int(0.15 * 48), the reference's heuristic)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-budget-s", type=float, default=150.0,
                    help="wall time the reference arm's steps aim for; sets its rays per step (at most the batch)")
    ap.add_argument("--profile-variant", choices=["plain_fp32", "bf16", "proposal_bf16", "unbounded_plain_bf16",
                                                  "unbounded_proposal_bf16"], default=None)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    elif args.profile_variant:
        run_profile_variant(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
