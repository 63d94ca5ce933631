"""pcg_ozaki_gemm_tc -- the FP64-accurate GEMM with all Ozaki levels in one tcgen05
tensor-core kernel -- against FP64 matmul, on operands whose rows and columns span
8 and 4 decades: ragged M, N, K (tile and chunk tails), row-major and transposed
output strides, accumulation, strided Y, and the kernel's error flag (every bounded
wait ended)."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _operands(M, N, K, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    X = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    X *= torch.pow(10.0, -8 * torch.rand(M, 1, dtype=torch.float64, device="cuda", generator=g))
    Y = torch.randn(K, N, dtype=torch.float64, device="cuda", generator=g)
    Y *= torch.pow(10.0, -4 * torch.rand(1, N, dtype=torch.float64, device="cuda", generator=g))
    return X, Y


def _check(C, ref, X, Y, K):
    scale = X.abs().amax(dim=1, keepdim=True) * Y.abs().amax(dim=0, keepdim=True) * K
    rel = ((C - ref).abs() / scale).max().item()
    assert rel < 1e-12, rel


@pytest.mark.parametrize("M,N,K", [(1000, 80, 208), (300, 128, 37), (129, 208, 298), (5, 16, 1), (256, 64, 64)])
def test_tc_gemm_row_major(M, N, K):
    from pychem_gb300.scf import ozaki_gemm_tc, ozaki_tc_status
    X, Y = _operands(M, N, K, M + N + K)
    C = torch.full((M, N), float("nan"), dtype=torch.float64, device="cuda")
    ozaki_gemm_tc(X, Y, C, M, N, K, K, (N, 1), (N, 1))
    assert ozaki_tc_status("cuda") == 0
    _check(C, X @ Y, X, Y, K)


def test_tc_gemm_transposed_output_accumulate_strided_y():
    from pychem_gb300.scf import ozaki_gemm_tc, ozaki_tc_status
    M, N, K = 777, 80, 208
    X, Y = _operands(M, N, K, 7)
    Yt = Y.t().contiguous()                     # Y[k][n] read as Yt[n][k]: sY = (1, K)
    ref = X @ Y
    C = (0.5 * ref).t().contiguous()          # something of the product's own scale to add to
    ozaki_gemm_tc(X, Yt, C, M, N, K, K, (1, K), (1, M), accumulate=True)   # C[n][m] += (X Y)[m][n]
    assert ozaki_tc_status("cuda") == 0
    _check(C.t(), 1.5 * ref, X, Y, K)
    ozaki_gemm_tc(X, Yt, C, M, N, K, K, (1, K), (1, M), nslice=7)
    assert ozaki_tc_status("cuda") == 0
    _check(C.t(), ref, X, Y, K)


def test_tc_gemm_rejects_bad_sizes():
    from pychem_gb300._lib import PcgError
    from pychem_gb300.scf import ozaki_gemm_tc
    X, Y = _operands(8, 8, 600, 1)
    C = torch.empty(8, 8, dtype=torch.float64, device="cuda")
    with pytest.raises(PcgError, match="K too large"):
        ozaki_gemm_tc(X, Y, C, 8, 8, 600, 600, (8, 1), (8, 1))
