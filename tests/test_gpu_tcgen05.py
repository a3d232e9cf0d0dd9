"""The surrogate network's forward GEMM on the fifth-generation tensor cores (tcgen05.mma with TMEM
accumulators, TMA loads; gdtk_gb300/csrc/mlp_tcgen05.cu) against an FP64 product of the same BF16
values and against the mma.sync kernel it replaces for these shapes.

The cases run smallest first (one K = 16 step into a 16-column accumulator, one tile), then
ragged row counts, the network's shapes (K 16 or 256 into N 256, 256 into the 16-wide output)
and a persistent run of many tiles per CTA."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CASES = [(128, 16, 16, 0), (200, 256, 16, 1), (1000, 256, 256, 1), (333, 16, 256, 0), (4099, 128, 64, 1),
         (300001, 256, 256, 1)]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _gemm(A, Ws, b, act, tc):
    """D = A Ws^T (+ b) (GELU) through gdtk_mlp_gemm with the tcgen05 path on or off."""
    from gdtk_gb300 import lib, check
    M, K = A.shape
    N = Ws.shape[0]
    launches, err = ctypes.c_ulonglong(), ctypes.c_int()
    prev = lib().gdtk_mlp_tcgen05(1 if tc else 0, ctypes.byref(launches), None)
    before = launches.value
    D = torch.empty((M, N), device="cuda")
    Dh = torch.empty((M, N), device="cuda", dtype=torch.bfloat16)
    pre = torch.empty((M, N), device="cuda") if act else None
    try:
        check(lib().gdtk_mlp_gemm(M, N, K, _ptr(A), K, 0, _ptr(Ws), K, 1, _ptr(b), act, _ptr(pre), _ptr(D), _ptr(Dh),
                                  N, 1, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "gdtk_mlp_gemm")
        torch.cuda.synchronize()
        lib().gdtk_mlp_tcgen05(-1, ctypes.byref(launches), ctypes.byref(err))
    finally:
        lib().gdtk_mlp_tcgen05(prev, None, None)
    assert err.value == 0, "a tcgen05 wait gave up (%d)" % err.value
    assert launches.value - before == (1 if tc else 0)
    return D, Dh, pre


@pytest.mark.parametrize("M,N,K,act", CASES)
def test_tcgen05_gemm_matches_fp64_product_and_mma_sync(M, N, K, act):
    g = torch.Generator(device="cuda")
    g.manual_seed(M * 5 + N * 3 + K)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    Ws = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16)   # stored [N][K], as the network's
    b = torch.randn(N, generator=g, device="cuda")
    D, Dh, pre = _gemm(A, Ws, b, act, tc=True)
    ref = A.double() @ Ws.double().t() + b.double()
    scale = (A.double().abs() @ Ws.double().abs().t()).clamp_min(1e-30)
    if act:
        assert ((pre.double() - ref).abs() / scale).max().item() < 1e-6
        z = ref
        ref = 0.5 * z * (1.0 + torch.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))
        assert ((D.double() - ref).abs() / (scale + 1.0)).max().item() < 2e-6
    else:
        assert ((D.double() - ref).abs() / scale).max().item() < 1e-6
    assert ((Dh.double() - D.double()).abs() <= D.double().abs() * 2 ** -8 + 1e-30).all()
    # the mma.sync kernel on the same operands: both are FP32 sums of the same exact BF16 products
    D2, _, _ = _gemm(A, Ws, b, act, tc=False)
    assert ((D.double() - D2.double()).abs() / (scale + 1.0)).max().item() < 2e-6
