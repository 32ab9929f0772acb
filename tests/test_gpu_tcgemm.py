"""GPU tests of the dense-layer GEMM behind the MLP (tvm_gemm): tcgen05 bf16, tcgen05
split-tf32 and FP32 SIMT, all orientations, ragged sizes and split-K accumulation,
against float64 products of the same inputs."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu

MATH_BF16, MATH_SPLIT, MATH_SIMT = 0, 1, 2


def _gemm(math, A, B, at, bt, M, N, K, D=None, accumulate=0):
    from tensorf_gb300 import _lib
    from tensorf_gb300._util import ptr, stream_handle
    lda = A.shape[1]
    ldb = B.shape[1]
    if D is None:
        D = torch.full((M, N), float("nan"), device="cuda")
    _lib.call("tvm_gemm", math, int(at), int(bt), M, N, K, ptr(A), lda, ptr(B), ldb, ptr(D), N, accumulate,
              stream_handle())
    st = ctypes.c_int32(-1)
    _lib.call("tvm_device_status", ctypes.byref(st), stream_handle())
    assert st.value == 0, "a bounded tensor-core wait gave up"
    return D


def _ref(A, B, at, bt, math):
    a = A.double().cpu()
    b = B.double().cpu()
    if math == MATH_BF16:
        a = A.bfloat16().double().cpu()
        b = B.bfloat16().double().cpu()
    a = a.t() if at else a
    b = b.t() if bt else b
    return a @ b


CASES = [(128, 16, 16), (128, 128, 64), (256, 160, 160), (300, 144, 32), (77, 27, 144), (1000, 3, 128),
         (129, 150, 128), (64, 256, 200)]


@pytest.mark.parametrize("math", [MATH_BF16, MATH_SPLIT, MATH_SIMT])
@pytest.mark.parametrize("at,bt", [(False, False), (False, True), (True, False), (True, True)])
@pytest.mark.parametrize("M,N,K", CASES)
def test_gemm_matches_float64(math, at, bt, M, N, K):
    g = torch.Generator().manual_seed(M * 1000 + N * 10 + K)
    A = torch.randn((K, M) if at else (M, K), generator=g).cuda()
    B = torch.randn((N, K) if bt else (K, N), generator=g).cuda()
    D = _gemm(math, A, B, at, bt, M, N, K)
    ref = _ref(A, B, at, bt, math)
    err = float((D.double().cpu() - ref).abs().max() / ref.abs().max())
    tol = {MATH_BF16: 1e-5, MATH_SPLIT: 2e-6, MATH_SIMT: 2e-6}[math]
    assert err < tol, err


@pytest.mark.parametrize("math", [MATH_BF16, MATH_SPLIT])
def test_gemm_split_k_accumulate(math):
    # Weight-gradient shape: D (+)= X^T dY over many rows, K split across CTAs.
    g = torch.Generator().manual_seed(5)
    rows, fin, fout = 20000, 150, 128
    X = torch.randn((rows, fin), generator=g).cuda()
    dY = torch.randn((rows, fout), generator=g).cuda()
    D0 = torch.randn((fin, fout), generator=g).cuda()
    D = _gemm(math, X, dY, True, False, fin, fout, rows, D=D0.clone(), accumulate=1)
    ref = D0.double().cpu() + _ref(X, dY, True, False, math)
    err = float((D.double().cpu() - ref).abs().max() / ref.abs().max())
    assert err < 1e-5, err


def test_split_is_fp32_accurate_on_mlp_like_inputs():
    # The FP32-accurate mode must stay well inside the 1e-4 parity budget on the
    # magnitudes the MLP sees.
    g = torch.Generator().manual_seed(9)
    A = (torch.randn((4096, 150), generator=g) * 0.5).cuda()
    B = (torch.randn((150, 128), generator=g) * (2.0 / 150) ** 0.5).cuda()
    D = _gemm(MATH_SPLIT, A, B, False, False, 4096, 128, 150)
    ref = A.double().cpu() @ B.double().cpu()
    err = float((D.double().cpu() - ref).abs().max() / ref.abs().max())
    assert err < 2e-6, err
