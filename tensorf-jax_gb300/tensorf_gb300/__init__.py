"""tensorf_gb300: the TensoRF-VM render-and-train path on one GB300 (sm_103a).

Drop-in twins of the reference's tensorf/tensor_vm.py, render.py, networks.py and the
training step of training.py, backed by hand-written CUDA kernels behind the C ABI in
include/tensorf_gb300.h (libtensorf_gb300.so, built in-tree by _build.py).
"""
from . import _lib  # noqa: F401

__all__ = ["cameras", "networks", "render", "scene", "tensor_vm", "training", "utils"]


def load_library():
    """Load libtensorf_gb300.so (raises if it is not built)."""
    return _lib.load()
