"""GPU test of tvm_mlp_fwd_static_scratch, the FeatureMlp forward that runs on the
library's static scratch array instead of a caller workspace. Through the C ABI, two
calls in a row (different inputs and row counts, the first at the largest row count
the scratch allows) must give the rgb of tvm_mlp_fwd within the MLP parity
tolerance. Oversized calls must be rejected before any launch; their buffers are
sized for every requested row all the same.

The file name sorts last so that pytest runs it after every other test; it must
also pass alone in a fresh process."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-4  # same relative tolerance as the MLP parity tests


def _max_rows(lp):
    """The row limit the library reports for this model: a call with an impossible row
    count and no pointers fails the size check on the host, before any launch."""
    import re
    from tensorf_gb300 import _lib
    lib = _lib.load()
    md = lp.model_desc()
    status = lib.tvm_mlp_fwd_static_scratch(ctypes.byref(md), None, None, None, 1 << 40, None, None)
    if status != -2:  # no scratch limit for this model (fused BF16 path)
        return None
    return int(re.search(r"at most (\d+) rows", lib.tvm_last_error_message().decode()).group(1))


def _rel_err(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    assert a.shape == b.shape and a.numel() > 0
    return float((a - b).abs().max() / (b.abs().max() + 1e-30))


def _model(precision, seed):
    from tensorf_gb300 import render
    spec = render.ModelSpec(grid_dim=8, precision=precision)
    lp = render.LearnableParams.initialize(spec, seed=seed)
    gen = torch.Generator().manual_seed(seed)
    for layer, v in lp.mlp_views().items():
        if "bias" in v:
            v["bias"].copy_(torch.randn(v["bias"].shape, generator=gen) * 0.1)
    return lp


def _inputs(n, seed):
    gen = torch.Generator().manual_seed(seed)
    feats = (torch.randn((n, 144), generator=gen) * 0.3).cuda()
    dirs = torch.nn.functional.normalize(torch.randn((n, 3), generator=gen), dim=-1).cuda()
    return feats.contiguous(), dirs.contiguous()


def _with_workspace(lp, feats, dirs):
    from tensorf_gb300 import _lib
    from tensorf_gb300._util import ptr, stream_handle
    md = lp.model_desc()
    n = feats.shape[0]
    ws = torch.empty(_lib.load().tvm_mlp_workspace_size(ctypes.byref(md), n), dtype=torch.uint8, device="cuda")
    rgb = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    _lib.call("tvm_mlp_fwd", ctypes.byref(md), ptr(lp.params), ptr(feats), ptr(dirs), None, n, ptr(rgb), ptr(ws),
              ws.numel(), stream_handle())
    return rgb


def _static(lp, feats, dirs, rgb):
    from tensorf_gb300 import _lib
    from tensorf_gb300._util import ptr, stream_handle
    md = lp.model_desc()
    _lib.call("tvm_mlp_fwd_static_scratch", ctypes.byref(md), ptr(lp.params), ptr(feats), ptr(dirs),
              feats.shape[0], ptr(rgb), stream_handle())


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_static_scratch_mlp_matches_workspace_entry_point(precision):
    from tensorf_gb300 import _lib
    lp = _model(precision, seed=11)
    limit = _max_rows(lp)
    assert (limit is None) == (precision == "bf16")
    first_n = limit if limit is not None else 50000
    for call, n in enumerate((first_n, 3001)):
        feats, dirs = _inputs(n, seed=100 + call)
        want = _with_workspace(lp, feats, dirs)
        got = torch.full((n, 3), float("nan"), device="cuda")
        _static(lp, feats, dirs, got)
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        err = _rel_err(got, want)
        assert err < RTOL, (precision, call, err)
    st = ctypes.c_int32(-1)
    _lib.call("tvm_device_status", ctypes.byref(st), None)
    assert st.value == 0


def test_static_scratch_rejects_rows_beyond_maximum():
    from tensorf_gb300 import _lib
    from tensorf_gb300._util import ptr
    lp = _model("fp32", seed=12)
    limit = _max_rows(lp)
    assert limit is not None and 1000 < limit < 40000
    n = limit + 1
    # Buffers hold all n rows, so nothing is out of bounds even if the call ran.
    feats, dirs = _inputs(n, seed=3)
    rgb = torch.zeros((n, 3), device="cuda")
    md = lp.model_desc()
    lib = _lib.load()
    status = lib.tvm_mlp_fwd_static_scratch(ctypes.byref(md), ptr(lp.params), ptr(feats), ptr(dirs), n, ptr(rgb),
                                            None)
    assert status == -2  # TVM_ERR_SHAPE, returned before any launch
    msg = lib.tvm_last_error_message().decode()
    assert f"at most {limit} rows" in msg, msg
    torch.cuda.synchronize()
    assert float(rgb.abs().max()) == 0.0
