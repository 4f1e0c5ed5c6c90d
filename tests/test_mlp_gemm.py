"""The proposal network's tcgen05 BF16 GEMM against a PyTorch fp32 matmul of
the same bf16 operands: every epilogue, each output-tile width (64, 128,
256), ragged M, N and K, the persistent form with many tiles per CTA (both
tensor-memory accumulators cycled, several output-column tiles), the
transposed (weight-gradient) form with split K."""
import pytest
import torch

pytestmark = pytest.mark.gpu

# fp32 accumulation of exact bf16 products, in a different order than the
# reference matmul: relative to the largest |C|
TOL = 2e-5


def _bf(shape, g, scale=1.0):
    return (torch.randn(shape, generator=g) * scale).to(torch.bfloat16).cuda()


def _ref(a, b, bias=None, trans=False):
    a32, b32 = a.float(), b.float()
    c = a32.t() @ b32 if trans else a32 @ b32.t()
    if bias is not None:
        c = c + bias
    return c


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 64, 16), (257, 128, 200), (520, 256, 128), (64, 104, 256)])
def test_gemm_store_and_bias(sgr_lib, M, N, K):
    from partgs_gb300 import proposal_gemm as G
    g = torch.Generator().manual_seed(M + N + K)
    a, b = _bf((M, K), g), _bf((N, K), g)
    bias = torch.randn(N, generator=g).cuda()
    out = torch.full((M, N), float("nan"), device="cuda")
    G.gemm(a, b, out, G.STORE_F32, bias=bias)
    torch.cuda.synchronize()
    ref = _ref(a, b, bias)
    assert int(G.status_word("cuda").item()) == 0
    assert float((out - ref).abs().max()) <= TOL * float(ref.abs().max())


@pytest.mark.parametrize("M,N,K", [(152 * 128 * 3 + 77, 256, 128), (60001, 384, 64), (40000, 64, 16)])
def test_gemm_persistent_many_tiles(sgr_lib, M, N, K):
    """More output tiles than resident CTAs: each CTA loops over tiles,
    alternating its two accumulators, with the last row and column tiles
    ragged."""
    from partgs_gb300 import proposal_gemm as G
    g = torch.Generator().manual_seed(M + N)
    a, b = _bf((M, K), g), _bf((N, K), g)
    bias = torch.randn(N, generator=g).cuda()
    out = torch.full((M, N), float("nan"), device="cuda")
    G.gemm(a, b, out, G.STORE_F32, bias=bias)
    torch.cuda.synchronize()
    ref = _ref(a, b, bias)
    assert int(G.status_word("cuda").item()) == 0
    assert float((out - ref).abs().max()) <= TOL * float(ref.abs().max())
    out16 = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    G.gemm(a, b, out16, G.RELU_BF16, bias=bias)
    ref16 = torch.relu(ref)
    assert float((out16.float() - ref16).abs().max()) <= 1e-2 * float(ref16.abs().max())


def test_gemm_relu_and_mask_epilogues(sgr_lib):
    from partgs_gb300 import proposal_gemm as G
    g = torch.Generator().manual_seed(5)
    M, N, K = 384, 128, 64
    a, b = _bf((M, K), g), _bf((N, K), g)
    bias = torch.randn(N, generator=g).cuda()
    out = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    G.gemm(a, b, out, G.RELU_BF16, bias=bias)
    ref = torch.relu(_ref(a, b, bias))
    assert float((out.float() - ref).abs().max()) <= 1e-2 * float(ref.abs().max())      # bf16 output
    mask = _bf((M, N), g)
    out2 = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    G.gemm(a, b, out2, G.MASK_BF16, mask=mask)
    ref2 = _ref(a, b) * (mask.float() > 0)
    assert float((out2.float() - ref2).abs().max()) <= 1e-2 * float(ref2.abs().max())
    assert bool(((mask.float() <= 0) <= (out2.float() == 0)).all())
    torch.cuda.synchronize()
    assert int(G.status_word("cuda").item()) == 0


@pytest.mark.parametrize("Kin,N,rows", [(64, 128, 4096), (128, 256, 3000), (16, 64, 2048)])
def test_gemm_transposed_split_k(sgr_lib, Kin, N, rows):
    """dW[Kin, N] = X^T dZ over `rows` point rows, split over CTAs."""
    from partgs_gb300 import proposal_gemm as G
    g = torch.Generator().manual_seed(Kin + N)
    x, dz = _bf((rows, Kin), g), _bf((rows, N), g)
    out = torch.zeros((Kin, N), device="cuda")
    G.gemm(x, dz, out, G.ADD_F32, trans=True, split_k=512)
    torch.cuda.synchronize()
    ref = _ref(x, dz, trans=True)
    assert int(G.status_word("cuda").item()) == 0
    assert float((out - ref).abs().max()) <= TOL * float(ref.abs().max()) * 4


def test_timeout_is_reported_and_the_context_stays_usable(sgr_lib):
    """The GEMM's waits are bounded: with the TMA producer told to issue no
    loads (the test switch), the MMA issuer's wait for them runs out after
    about a second with nothing in flight; the call raises SGR_MLP_TIMEOUT in
    the status word, frees its tensor memory and returns, and the next GEMM
    on the same context is correct."""
    import time
    from partgs_gb300 import proposal_gemm as G
    g = torch.Generator().manual_seed(5)
    a = torch.randn(256, 128, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(64, 128, generator=g).to(torch.bfloat16).cuda()
    out = torch.zeros(256, 64, device="cuda")
    G.status_word(out.device).zero_()
    t0 = time.perf_counter()
    G.gemm(a, b, out, G.STORE_F32, skip_loads=True)
    torch.cuda.synchronize()
    waited = time.perf_counter() - t0
    assert int(G.status_word(out.device).item()) == G.TIMEOUT
    assert 0.5 < waited < 30.0
    with pytest.raises(RuntimeError, match="SGR_MLP_TIMEOUT"):
        G.check_status(out.device)
    assert int(G.status_word(out.device).item()) == 0          # cleared by the check
    G.gemm(a, b, out, G.STORE_F32)
    G.check_status(out.device)
    ref = a.float() @ b.float().t()
    assert float((out - ref).abs().max()) <= 1e-2 * float(ref.abs().max())
