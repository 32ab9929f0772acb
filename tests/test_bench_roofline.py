"""bench.py's roofline arithmetic on CPU: the dominant kernel is the longest phase that
is one kernel launch, an L2-resident scatter is measured against the L2 reduction peak
with its HBM figures beside it, and the split-tf32 MLP against a third of the TF32 peak."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

PHASES = {"proposal_fwd": 0.002, "density_fwd": 0.158, "composite_select": 0.038, "appearance_fwd": 0.178,
          "mlp_fwd": 0.296, "color_loss": 0.009, "mlp_bwd": 0.547, "appearance_bwd": 0.303,
          "composite_bwd": 0.028, "density_bwd": 0.426, "proposal_bwd": 0.002, "adam": 0.083}
L2 = {"l2_read_gbs": 16714.8, "l2_red_gbs": 6343.5}


def test_dominant_kernel_is_the_density_scatter_against_l2():
    w = bench.variant_cfg("plain_fp32")
    r = bench.roofline_for(w, PHASES, L2)
    assert r["kernel"] == "density_bwd2_kernel" and r["bound"] == "l2"
    red = 4096 * 512 * 18 * 16 * 4  # one 4-byte reduction per gathered density element
    assert r["reduction_bytes"] == red
    assert r["frac"] == pytest.approx(red / 0.426e-3 / 1e9 / 6343.5, rel=1e-3)
    assert r["algorithmic_bytes"] == 4096 * 512 * (288 * 8 + 4)
    hbm, _, _ = bench.measured_peaks()
    assert r["hbm"]["frac"] == pytest.approx(r["algorithmic_bytes"] / 0.426e-3 / 1e9 / hbm, rel=1e-3)
    assert r["traffic"] == bench.NCU_DRAM_BYTES_PER_LAUNCH["density_bwd"]


def test_adam_dominant_is_hbm_bound():
    w = bench.variant_cfg("plain_fp32")
    r = bench.roofline_for(w, {"adam": 0.09, "density_fwd": 0.01}, L2)
    assert r["bound"] == "hbm" and r["kernel"] == "adam_kernel" and r["unit"] == "GB/s"


def test_split_tf32_mlp_against_a_third_of_tf32():
    w = bench.variant_cfg("plain_fp32")
    k = bench.kernel_rooflines(w, PHASES, L2, {"tflops": 1025.1})
    flops = 4 * 4096 * 64 * (144 * 27 + 150 * 128 + 128 * 128 + 128 * 3)
    assert k["mlp_bwd"]["frac_tensor"] == pytest.approx(flops / 0.547e-3 / 1e12 / (1025.1 / 3), abs=2e-3)
