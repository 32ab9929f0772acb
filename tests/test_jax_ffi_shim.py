"""CPU checks of the jax.ffi shim (tensorf-jax_gb300/csrc/jax/tvm_jax_ffi.cc and
tensorf_gb300/jax_ops.py) where JAX is not installed:

* the handler source compiles against include/tensorf_gb300.h and a stand-in for the
  XLA FFI binding API (tests/xla_ffi_stub), which fails the build when a handler's
  parameter list differs from its binding's context, argument, result and attribute
  types, in order;
* every handler the source defines is registered by jax_ops.HANDLERS, and the reverse;
* every C entry point the handlers call is declared in the header and exported by the
  built library.

Where jax is importable, a further test builds the shim and runs a wrapper on the GPU."""
import ast
import pathlib
import re
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
SHIM = ROOT / "tensorf-jax_gb300" / "csrc" / "jax" / "tvm_jax_ffi.cc"
OPS = ROOT / "tensorf-jax_gb300" / "tensorf_gb300" / "jax_ops.py"
HEADER = ROOT / "include" / "tensorf_gb300.h"
STUB = ROOT / "tests" / "xla_ffi_stub"


def _handlers_in_source():
    return re.findall(r"XLA_FFI_DEFINE_HANDLER_SYMBOL\(\s*(\w+)\s*,", SHIM.read_text())


def _handlers_registered():
    tree = ast.parse(OPS.read_text())
    for node in tree.body:
        if isinstance(node, ast.Assign) and any(getattr(t, "id", None) == "HANDLERS" for t in node.targets):
            return [elt.value for elt in node.value.elts]
    raise AssertionError("jax_ops.HANDLERS not found")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_shim_compiles_and_every_handler_matches_its_binding():
    cuda_inc = "/usr/local/cuda/include"
    res = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{STUB}", f"-I{ROOT / 'include'}", f"-I{cuda_inc}",
                          str(SHIM)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]


def test_every_handler_is_registered():
    src = _handlers_in_source()
    assert len(src) >= 8 and len(set(src)) == len(src)
    assert sorted(src) == sorted(_handlers_registered())


def test_handlers_call_exported_entry_points():
    from tensorf_gb300 import _lib
    body = SHIM.read_text()
    called = set(re.findall(r"\b(tvm_[a-z0-9_]+)\(", body)) - set(_handlers_in_source())
    declared = set(re.findall(r"TVM_API\s+[\w\s\*]+?\b(tvm_\w+)\s*\(", HEADER.read_text()))
    assert called, "the shim calls no entry point"
    assert called <= declared, called - declared
    assert called <= set(_lib.exported_symbols()), called - set(_lib.exported_symbols())
    so = _lib.LIB_PATH
    if so.exists():
        out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True).stdout
        exported = set(re.findall(r"\bT (tvm_\w+)$", out, re.M))
        assert called <= exported, called - exported


@pytest.mark.gpu
def test_jax_vm_interpolate_matches_torch_path():
    jax = pytest.importorskip("jax")
    import numpy as np
    import torch

    from tensorf_gb300 import jax_ops
    from tensorf_gb300.tensor_vm import TensorVM

    jax_ops.build()
    gen = torch.Generator().manual_seed(0)
    vec, mat = torch.randn((3, 16, 17), generator=gen) * 0.1, torch.randn((3, 16, 17, 17), generator=gen) * 0.1
    coords = torch.rand((3, 500), generator=gen) * 2 - 1
    vm = TensorVM.from_reference(vec, mat)
    want = vm.interpolate(coords.cuda()).cpu().numpy()
    got = jax.jit(jax_ops.vm_interpolate)(jax.numpy.asarray(vm.lines.cpu().numpy()),
                                          jax.numpy.asarray(vm.planes.cpu().numpy()),
                                          jax.numpy.asarray(coords.numpy()))
    np.testing.assert_allclose(np.asarray(got), want, rtol=1e-6, atol=1e-7)
