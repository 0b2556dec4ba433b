"""The learned preconditioner's layer GEMMs on the tcgen05 tensor cores
(k_row_gemm, k_dw_grad) against a plain PyTorch FP32 reference of the same
operations, over row counts that cut the 128-row tiles in every way (one row,
a partial tile, whole tiles, many CTAs per SM)."""
import pytest
import torch

from arcanefem_gb300 import learned

pytestmark = pytest.mark.gpu

ROWS = [1, 127, 128, 129, 1000, 263169]


def _inputs(M, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    r = lambda *shape: (torch.rand(*shape, generator=g, device="cuda") * 2 - 1)
    X1, X2 = r(M, 64).to(torch.bfloat16), r(M, 64).to(torch.bfloat16)
    W1t, W2t = (r(64, 64) * 0.25).to(torch.bfloat16), (r(64, 64) * 0.25).to(torch.bfloat16)
    return X1, X2, W1t, W2t, r(64)


@pytest.mark.parametrize("M", ROWS)
@pytest.mark.parametrize("two,relu", [(True, True), (False, False), (True, False), (False, True)])
def test_row_gemm_matches_fp32_reference(cuda_ctx, M, two, relu):
    X1, X2, W1t, W2t, bias = _inputs(M, 11 + M)
    ref = X1.float() @ W1t.float().T + bias
    if two:
        ref = ref + X2.float() @ W2t.float().T
    if relu:
        ref = ref.relu()
    Yb, Yf = learned.tc_row_gemm(cuda_ctx, X1, W1t, X2 if two else None, W2t if two else None, bias, relu,
                                 out_bf16=True, out_f32=True)
    scale = ref.abs().max().item()
    # exact BF16 products, FP32 sums in another order: a few FP32 ulps of the magnitude
    assert (Yf - ref).abs().max().item() <= 1e-5 * scale
    # the BF16 output is the FP32 result rounded to BF16
    assert (Yb.float() - ref).abs().max().item() <= 2.0 ** -8 * scale


@pytest.mark.parametrize("M", [1000, 263169])
def test_row_gemm_accumulates_into_fp32(cuda_ctx, M):
    X1, _, W1t, _, _ = _inputs(M, 5)
    base = torch.randn(M, 64, device="cuda")
    _, Yf = learned.tc_row_gemm(cuda_ctx, X1, W1t, out_bf16=False, out_f32=True, Yf=base.clone(), accumulate=True)
    ref = base + X1.float() @ W1t.float().T
    assert (Yf - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()


@pytest.mark.parametrize("M", ROWS)
def test_weight_grad_matches_fp32_reference_and_is_deterministic(cuda_ctx, M):
    X1, X2, _, _, _ = _inputs(M, 7 + M)
    G = (torch.rand(M, 64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(M)) - 0.5)
    G = G.to(torch.bfloat16)
    dW = learned.tc_weight_grad(cuda_ctx, X1, X2, G)
    ref = torch.stack([X1.double().T @ G.double(), X2.double().T @ G.double()]).float()
    err = ((dW - ref).norm() / ref.norm()).item()
    assert err < 1e-5
    assert torch.equal(dW, learned.tc_weight_grad(cuda_ctx, X1, X2, G))
