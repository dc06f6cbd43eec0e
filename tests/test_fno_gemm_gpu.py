"""tcgen05 BF16 GEMM of the surrogate against a plain PyTorch FP32 product
of the same BF16 operands, through the C-ABI.

Tolerance: 2e-3 of the output's largest magnitude (FP32 accumulation in a
different order; BF16 output rounding adds 2^-8 relative for c_bf16)."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from geoflac_gb300 import capi
    lib = capi.load_library()
    f = lib.gf_gemm_bf16
    f.restype = C.c_int
    f.argtypes = [C.c_void_p] * 3 + [C.c_int] * 4 + [C.c_longlong] * 6 + [C.c_int, C.c_float, C.c_float,
                                                                         C.c_void_p, C.c_void_p]
    lib.gf_gemm_error.restype = C.c_int
    return lib


@pytest.mark.parametrize("batch,M,N,K", [(1, 128, 64, 64), (1, 300, 48, 384), (3, 257, 200, 136),
                                         (2, 1000, 128, 1024), (4, 64, 256, 64), (1, 129, 96, 8)])
@pytest.mark.parametrize("c_bf16", [0, 1])
def test_gemm_matches_torch(batch, M, N, K, c_bf16):
    torch = pytest.importorskip("torch")
    lib = _lib()
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(batch, M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(batch, N, K, generator=g).to(torch.bfloat16).cuda()
    bias = torch.randn(N, generator=g).float().cuda()
    ref = torch.matmul(A.float(), B.float().transpose(1, 2)) * 0.5 + bias
    out = torch.zeros(batch, M, N, dtype=torch.bfloat16 if c_bf16 else torch.float32, device="cuda")
    rc = lib.gf_gemm_bf16(A.data_ptr(), B.data_ptr(), out.data_ptr(), batch, M, N, K, K, M * K, K, N * K, N, M * N,
                          c_bf16, 0.5, 0.0, bias.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert lib.gf_gemm_error() == 0
    err = (out.float() - ref).abs().max().item() / ref.abs().max().item()
    assert err <= (6e-3 if c_bf16 else 2e-3), err


def test_gemm_beta_accumulates():
    torch = pytest.importorskip("torch")
    lib = _lib()
    A = torch.randn(1, 256, 128).to(torch.bfloat16).cuda()
    B = torch.randn(1, 64, 128).to(torch.bfloat16).cuda()
    C0 = torch.randn(1, 256, 64).cuda()
    out = C0.clone()
    assert lib.gf_gemm_bf16(A.data_ptr(), B.data_ptr(), out.data_ptr(), 1, 256, 64, 128, 128, 0, 128, 0, 64, 0, 0,
                            1.0, 1.0, None, None) == 0
    ref = torch.matmul(A.float(), B.float().transpose(1, 2)) + C0
    torch.cuda.synchronize()
    assert (out - ref).abs().max().item() / ref.abs().max().item() <= 2e-3


def test_gemm_rejects_unaligned_strides():
    torch = pytest.importorskip("torch")
    lib = _lib()
    A = torch.zeros(64, 12, dtype=torch.bfloat16, device="cuda")
    out = torch.zeros(64, 64, device="cuda")
    # K = 12 is not a multiple of 8: the TMA row stride would be 24 bytes
    assert lib.gf_gemm_bf16(A.data_ptr(), A.data_ptr(), out.data_ptr(), 1, 64, 64, 12, 12, 0, 12, 0, 64, 0, 0,
                            1.0, 0.0, None, None) == -3


def test_gemm_broadcast_a_and_fused_gelu_copy():
    """sA = -1 shares A among the batches; aux receives BF16 GELU(C)."""
    torch = pytest.importorskip("torch")
    from geoflac_gb300.fno import _lib
    lib = _lib()
    A = torch.randn(1, 384, 48).to(torch.bfloat16).cuda()
    B = torch.randn(37, 64, 48).to(torch.bfloat16).cuda()
    bias = torch.randn(64).cuda()
    C0 = torch.randn(37, 384, 64).cuda()
    out = C0.clone()
    aux = torch.empty(37, 384, 64, dtype=torch.bfloat16, device="cuda")
    assert lib.gf_gemm_bf16_ex(A.data_ptr(), B.data_ptr(), out.data_ptr(), 37, 384, 64, 48, 48, -1, 48, 64 * 48, 64,
                               384 * 64, 0, 1.0, 1.0, bias.data_ptr(), aux.data_ptr(), 1, None) == 0
    torch.cuda.synchronize()
    ref = torch.matmul(A.float().expand(37, -1, -1), B.float().transpose(1, 2)) + C0 + bias
    assert (out - ref).abs().max().item() / ref.abs().max().item() <= 2e-3
    g = torch.nn.functional.gelu(ref)
    assert (aux.float() - g).abs().max().item() / g.abs().max().item() <= 1e-2


def test_gemm_aux_only_output():
    """c_bf16 = 2: C is read for beta (or absent with beta = 0) and left
    unwritten; aux carries the same BF16 GELU(C) as the full call."""
    torch = pytest.importorskip("torch")
    from geoflac_gb300.fno import _lib
    lib = _lib()
    A = torch.randn(1, 1000, 64).to(torch.bfloat16).cuda()
    B = torch.randn(1, 64, 64).to(torch.bfloat16).cuda()
    bias = torch.randn(64).cuda()
    C0 = torch.randn(1, 1000, 64).cuda()
    full, part = C0.clone(), C0.clone()
    aux_full = torch.empty(1, 1000, 64, dtype=torch.bfloat16, device="cuda")
    aux_part = torch.empty_like(aux_full)
    args = (1, 1000, 64, 64, 64, 0, 64, 0, 64, 0)
    assert lib.gf_gemm_bf16_ex(A.data_ptr(), B.data_ptr(), full.data_ptr(), *args, 0, 1.0, 1.0, bias.data_ptr(),
                               aux_full.data_ptr(), 1, None) == 0
    assert lib.gf_gemm_bf16_ex(A.data_ptr(), B.data_ptr(), part.data_ptr(), *args, 2, 1.0, 1.0, bias.data_ptr(),
                               aux_part.data_ptr(), 1, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(part, C0)  # read, not written
    assert torch.equal(aux_part, aux_full)
    # beta = 0 with no C at all
    aux0 = torch.empty_like(aux_full)
    ref0 = torch.empty(1, 1000, 64, device="cuda")
    aux_ref = torch.empty_like(aux_full)
    assert lib.gf_gemm_bf16_ex(A.data_ptr(), B.data_ptr(), None, *args, 2, 1.0, 0.0, bias.data_ptr(),
                               aux0.data_ptr(), 1, None) == 0
    assert lib.gf_gemm_bf16_ex(A.data_ptr(), B.data_ptr(), ref0.data_ptr(), *args, 0, 1.0, 0.0, bias.data_ptr(),
                               aux_ref.data_ptr(), 1, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(aux0, aux_ref)
    # aux-only without aux stores nothing: rejected
    assert lib.gf_gemm_bf16_ex(A.data_ptr(), B.data_ptr(), None, *args, 2, 1.0, 0.0, None, None, 0, None) == -2
