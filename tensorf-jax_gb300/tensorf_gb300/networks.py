"""GB300 twin of ``tensorf/networks.py``: the appearance ``FeatureMlp``.

Hyper-parameters and the flax parameter tree (``Dense_0`` .. ``Dense_3``, kernels
``(in, out)``) are the reference's (networks.py:38-121). The weights live in the flat
parameter buffer of ``render.LearnableParams``; ``apply`` runs ``tvm_mlp_fwd`` (and
``tvm_mlp_bwd`` under autograd).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, Optional

import torch

from . import _lib
from ._util import ptr, stream_handle, workspace


@dataclasses.dataclass(frozen=True)
class FeatureMlp:
    feature_squash_dim: int = 27
    units: int = 128
    feature_n_freqs: int = 6
    viewdir_n_freqs: int = 6
    num_cameras: Optional[int] = None  # camera embeddings (FiLM) are not on this path

    def __post_init__(self):
        if self.num_cameras is not None:
            raise NotImplementedError("FiLM camera embeddings (networks.py:103-111) are not implemented")

    def encoded_dim(self) -> int:
        """networks.py:77-82."""
        return (self.feature_squash_dim + 3 + 2 * self.feature_n_freqs * self.feature_squash_dim
                + 2 * self.viewdir_n_freqs * 3)

    def init_params(self, feat_dim: int, generator: Optional[torch.Generator] = None) -> Dict[str, Dict[str, torch.Tensor]]:
        """Flax-layout parameters (CPU float32): lecun_normal for Dense_0 / Dense_3,
        kaiming_normal for Dense_1 / Dense_2 (networks.py:9-10), biases zero. Flax
        samples truncated normals; a plain normal with the same variance is used."""
        def normal(fan_in, fan_out, var):
            return torch.randn((fan_in, fan_out), generator=generator) * math.sqrt(var / fan_in)
        u = self.units
        return {
            "Dense_0": {"kernel": normal(feat_dim, self.feature_squash_dim, 1.0)},
            "Dense_1": {"kernel": normal(self.encoded_dim(), u, 2.0), "bias": torch.zeros(u)},
            "Dense_2": {"kernel": normal(u, u, 2.0), "bias": torch.zeros(u)},
            "Dense_3": {"kernel": normal(u, 3, 1.0), "bias": torch.zeros(3)},
        }

    def apply(self, learnable_params, features: torch.Tensor, viewdirs: torch.Tensor,
              camera_indices: Optional[torch.Tensor] = None) -> torch.Tensor:
        """rgb = FeatureMlp(features (*, 3C), viewdirs (*, 3)) (networks.py:45-121)."""
        batch = features.shape[:-1]
        f = features.reshape(-1, features.shape[-1]).to(torch.float32).contiguous()
        d = viewdirs.reshape(-1, 3).to(torch.float32).contiguous()
        out = _MlpFn.apply(f, d, learnable_params.params, learnable_params)
        return out.reshape(tuple(batch) + (3,))


class _MlpFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, features, viewdirs, params, lp):
        n = features.shape[0]
        md = lp.model_desc()
        ws = workspace(_lib.load().tvm_mlp_workspace_size(ctypes_byref(md), n), features.device)
        rgb = torch.empty((n, 3), dtype=torch.float32, device=features.device)
        _lib.call("tvm_mlp_fwd", ctypes_byref(md), ptr(params), ptr(features), ptr(viewdirs), n, ptr(rgb),
                  ptr(ws), ws.numel(), stream_handle())
        ctx.save_for_backward(features, viewdirs, params)
        ctx.lp = lp
        return rgb

    @staticmethod
    def backward(ctx, grad_rgb):
        features, viewdirs, params = ctx.saved_tensors
        lp = ctx.lp
        n = features.shape[0]
        md = lp.model_desc()
        ws = workspace(_lib.load().tvm_mlp_workspace_size(ctypes_byref(md), n), features.device)
        gfeat = torch.empty_like(features)
        gparams = torch.zeros_like(params)
        _lib.call("tvm_mlp_bwd", ctypes_byref(md), ptr(params), ptr(features), ptr(viewdirs), n,
                  ptr(grad_rgb.contiguous()), ptr(gfeat), ptr(gparams), ptr(ws), ws.numel(), stream_handle())
        return gfeat, None, gparams, None


def ctypes_byref(s):
    import ctypes
    return ctypes.byref(s)
