"""Benchmark of the TensoRF-VM train step on one GB300 (and N replicas under torchrun).

Default workload (--workload train_fp32): the single-GPU training step of a 300^3 VM
field with 16 / 48 components per mode, a 4096-ray batch with 512 uniform density
samples per ray and per-ray top-64 weighted selection of appearance samples, the
FeatureMlp with 2-frequency encodings, MSE loss, full backward and Adam (lr 0.02 grids
/ 1e-3 MLP), all FP32. Targets: an analytic scene of 32 random spheres (radius
U[0.1, 0.4], density 50, RGB U[0, 1]) seen by seeded 800x800 cameras with focal length
1111, rendered by FP64 quadrature with 4096 samples per ray. Synthetic, seeded.

One JSON line on stdout (rank 0). ``--impl reference`` times the CPU restatement of
the reference's algorithm (the oracle) on the host cores instead.
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
PHASES = ["density_fwd", "composite_select", "appearance_fwd", "mlp_fwd", "color_loss", "mlp_bwd",
          "appearance_bwd", "composite_bwd", "density_bwd", "adam"]


def workload_cfg(name: str, small: bool = False):
    w = dict(grid=300, Cd=16, Ca=48, R=4096, N=512, k=64, precision="fp32", pool_batches=8)
    if name == "train_bf16":
        w["precision"] = "bf16"
    if small:  # a case for ncu captures: same kernels, 1/4 of the rays
        w.update(R=1024, pool_batches=2)
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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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


def build_problem(w, device, seed=0):
    from tensorf_gb300 import render, scene, training

    spec = render.ModelSpec(grid_dim=w["grid"], density_feat_dim=w["Cd"], appearance_feat_dim=w["Ca"],
                            precision=w["precision"])
    sc = scene.SphereScene.random(seed, count=32)
    cams = sc.cameras(100, seed=seed + 1)
    total = w["R"] * w["pool_batches"]
    rays, colors = sc.training_rays(cams, total, seed=seed + 2, n_samples=4096)
    cfg = training.TrainConfig(initial_aabb_min=sc.aabb[0], initial_aabb_max=sc.aabb[1],
                               density_samples_per_ray=w["N"], appearance_samples_per_ray=w["k"],
                               n_iters=30000, upsamp_iters=())
    state = training.TrainState.initialize(cfg, spec, seed=94709)
    return spec, sc, state, rays, colors


def batch(rays, colors, i, R):
    from tensorf_gb300 import cameras

    n = rays.origins.shape[0] // R
    j = i % n
    return (cameras.Rays3D(rays.origins[j * R:(j + 1) * R], rays.directions[j * R:(j + 1) * R]),
            colors[j * R:(j + 1) * R])


def algorithmic_bytes(w, phase):
    """Algorithmic bytes of one launch of each phase (documented in the design doc)."""
    R, N, k = w["R"], w["N"], w["k"]
    s = 2 if w["precision"] == "bf16" else 4
    dens_el, app_el = 18 * w["Cd"], 18 * w["Ca"]
    G = w["grid"]
    n_params = 3 * G * (G + 1) * (w["Cd"] + w["Ca"]) + 40115
    return {
        "density_fwd": R * N * dens_el * s + R * N * 4,
        "density_bwd": R * N * dens_el * (s + 4) + R * N * 4,
        "appearance_fwd": R * k * app_el * s + R * k * 3 * w["Ca"] * 4,
        "appearance_bwd": R * k * app_el * (s + 4) + R * k * 3 * w["Ca"] * 4,
        "adam": n_params * 32,
    }.get(phase)


def run_ours(args):
    import ctypes

    from tensorf_gb300 import _lib, cameras, render, training

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load()
    w = workload_cfg(args.workload, args.small)
    spec, sc, state, rays, colors = build_problem(w, "cuda", seed=rank)
    torch.cuda.synchronize()

    # Warm-up.
    for i in range(args.warmup):
        b_r, b_c = batch(rays, colors, i, w["R"])
        state.training_step(b_r, b_c, log=False)
    torch.cuda.synchronize()

    # Timed region: device-resident inputs, phase events on the launching stream.
    n_ev = len(PHASES) + 1
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(n_ev)] for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for row in evs:  # torch creates events lazily: record once so the handles exist
        for e in row:
            e.record()
    torch.cuda.synchronize()
    launches0 = lib.tvm_kernel_launches()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record()
        for i in range(args.steps):
            handles = (ctypes.c_void_p * n_ev)(*[e.cuda_event for e in evs[i]])
            _lib.call("tvm_set_phase_events", handles, n_ev)
            b_r, b_c = batch(rays, colors, args.warmup + i, w["R"])
            state.training_step(b_r, b_c, log=False)
        _lib.call("tvm_set_phase_events", None, 0)
        end.record()
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = int(lib.tvm_kernel_launches() - launches0)
    ms = start.elapsed_time(end)
    phase_ms = {p: statistics.mean(evs[i][j].elapsed_time(evs[i][j + 1]) for i in range(args.steps))
                for j, p in enumerate(PHASES)}
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = w["R"] * args.steps * world / (ms / 1e3)
    final_loss = float(state.loss.item())

    # End to end through the public API: host (pinned) rays and colours copied in every
    # step, the loss read back every step.
    host_o = rays.origins.cpu().pin_memory()
    host_d = rays.directions.cpu().pin_memory()
    host_c = colors.cpu().pin_memory()
    dev_o = torch.empty((w["R"], 3), device="cuda")
    dev_d = torch.empty((w["R"], 3), device="cuda")
    dev_c = torch.empty((w["R"], 3), device="cuda")
    loss_host = torch.empty(1).pin_memory()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    npool = host_o.shape[0] // w["R"]
    for i in range(args.steps):
        j = i % npool
        sl = slice(j * w["R"], (j + 1) * w["R"])
        dev_o.copy_(host_o[sl], non_blocking=True)
        dev_d.copy_(host_d[sl], non_blocking=True)
        dev_c.copy_(host_c[sl], non_blocking=True)
        state.training_step(cameras.Rays3D(dev_o, dev_d), dev_c, log=False)
        loss_host.copy_(state.loss, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = w["R"] * args.steps * world / (e2e_ms / 1e3)

    # Roofline of the dominant phase.
    hbm, bf16, peak_src = measured_peaks()
    dom = max((p for p in phase_ms if algorithmic_bytes(w, p) is not None), key=lambda p: phase_ms[p])
    achieved = algorithmic_bytes(w, dom) / (phase_ms[dom] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": None, "peak_source": peak_src,
                "note": "gathers/scatters are L2-resident: algorithmic bytes over the measured HBM copy peak"}
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            tr = json.load(f).get(args.workload, {}).get(dom)
        if tr:
            roofline["traffic"] = tr

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if w["precision"] == "fp32" else "bf16",
        "data": "synthetic (32-sphere analytic scene, FP64 quadrature targets, seeded cameras)",
        "config": {"workload": f"train step {w['precision']}: grid {w['grid']}^3, VM {w['Cd']}/{w['Ca']}, "
                               f"{w['R']} rays x {w['N']} samples, top-{w['k']} appearance, Adam",
                   "rays_per_step": w["R"], "density_samples": w["N"], "appearance_samples": w["k"],
                   "grid": w["grid"], "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "no flush: each step streams params+grads+Adam moments (277 MB) and 2.1 GB of "
                         "per-sample work, both larger than the 126 MB L2"},
        "phase_ms": {p: round(v, 4) for p, v in phase_ms.items()},
        "final_loss": final_loss,
        "e2e": {"value": round(e2e_value, 1), "unit": "rays/s", "h2d_bytes_per_step": w["R"] * 9 * 4,
                "d2h_bytes_per_step": 4},
        "gpu_launches": launches,
        "roofline": roofline,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------------
# CPU: the oracle restatement of the reference algorithm on the host cores.
# ---------------------------------------------------------------------------------
def _cpu_step_time(w, rays_sample, seed=0):
    """Seconds for forward+backward of ``rays_sample`` rays of the workload with the
    float32 oracle, plus seconds for one Adam update of the full parameter set."""
    from oracle import tensorf_oracle as O

    gen = torch.Generator().manual_seed(seed)
    G = w["grid"]
    p = {"density": O.vm_init(G, w["Cd"], gen, torch.float32), "appearance": O.vm_init(G, w["Ca"], gen, torch.float32),
         "mlp": O.mlp_init(3 * w["Ca"], 2, 2, gen, dtype=torch.float32)}
    leaves = [*p["density"], *p["appearance"]] + [t for d in p["mlp"].values() for t in d.values()]
    for t in leaves:
        t.requires_grad_(True)
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(rays_sample, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * 4
    d = -o + rng.normal(scale=0.05, size=o.shape)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    aabb = torch.tensor([[-1.5] * 3, [1.5] * 3])
    jit = torch.rand(w["N"], generator=gen)
    gum = -torch.log(-torch.log(torch.rand(w["N"], generator=gen).clamp_min(1e-7)))
    col = torch.rand((rays_sample, 3), generator=gen)
    t0 = time.perf_counter()
    out = O.render_rays(p, aabb, torch.tensor(o, dtype=torch.float32), torch.tensor(d, dtype=torch.float32),
                        w["N"], w["k"], jit, gum)
    loss = O.mse(out, col)
    grads = torch.autograd.grad(loss, leaves)
    t1 = time.perf_counter()
    with torch.no_grad():
        for t, g in zip(leaves, grads):
            z = torch.zeros_like(t)
            O.adam_update(t, g, z, z, 1, lr=0.02, lr_decay=1.0)
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1


def cpu_baseline(w, args):
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    sample = args.cpu_sample_rays
    fb, adam = _cpu_step_time(w, sample)
    step_s = fb * (w["R"] / sample) + adam
    return {"value": round(w["R"] / step_s, 2), "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": f"oracle (torch CPU float32) forward+backward of {sample} of the {w['R']} rays, "
                      f"scaled x{w['R'] // sample}, plus one full Adam update ({fb:.2f} s + {adam:.2f} s)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w = workload_cfg(args.workload, args.small)
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    sample = args.cpu_sample_rays
    for _ in range(max(0, min(args.warmup, 1))):
        _cpu_step_time(w, max(8, sample // 8))
    times = []
    t_start = time.perf_counter()
    for i in range(args.steps):
        fb, adam = _cpu_step_time(w, sample, seed=i)
        times.append(fb * (w["R"] / sample) + adam)
    wall = time.perf_counter() - t_start
    step_s = statistics.mean(times)
    value = w["R"] / step_s
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "rays/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if w["precision"] == "fp32" else "bf16",
        "data": "synthetic (seeded rays, N(0, 0.1^2) parameters)",
        "config": {"workload": f"train step {w['precision']}: grid {w['grid']}^3, VM {w['Cd']}/{w['Ca']}, "
                               f"{w['R']} rays x {w['N']} samples, top-{w['k']} appearance, Adam",
                   "rays_per_step": w["R"]},
        "cpu_baseline": {"value": round(value, 2), "unit": "rays/s", "cores": threads, "kind": "port",
                         "sample": f"each step: oracle forward+backward of {sample} rays scaled to {w['R']}, "
                                   f"plus one full Adam update; wall {wall:.1f} s"},
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
    ap.add_argument("--workload", choices=["train_fp32", "train_bf16"], default="train_fp32")
    ap.add_argument("--small", action="store_true", help="1024-ray case for profiler captures")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-rays", type=int, default=256)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
