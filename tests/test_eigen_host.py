"""Host-side helpers of the batched spectrum slicing (pychem_gb300.eigen), on CPU
tensors: the split point of an ascending spectrum and the padding of several matrices
to one batched Jacobi launch."""
import pytest

torch = pytest.importorskip("torch")


def test_split_point_largest_gap_within_the_block_limit():
    from pychem_gb300 import eigen
    n = 100
    w = torch.linspace(-10.0, 10.0, n, dtype=torch.float64)
    w[50:] += 5.0                       # the gap between 49 and 50
    s = eigen._split_point(w, n)
    assert s == 50
    # both parts at most EXACT_BLOCK (64) when the window allows it
    assert s <= eigen.EXACT_BLOCK and n - s <= eigen.EXACT_BLOCK


def test_split_point_middle_half_when_the_window_is_narrow():
    from pychem_gb300 import eigen
    n = 200                             # both parts <= 64 is impossible: the middle half
    w = torch.arange(n, dtype=torch.float64)
    w[120:] += 3.0
    assert eigen._split_point(w, n) == 120
    w2 = torch.arange(n, dtype=torch.float64)
    w2[10:] += 3.0                      # a gap outside the middle half is not taken
    s = eigen._split_point(w2, n)
    assert n // 4 <= s <= (3 * n) // 4


def test_padded_blocks_are_decoupled_and_sort_last():
    from pychem_gb300 import eigen
    g = torch.Generator().manual_seed(3)
    mats = []
    for n in (5, 8, 3):
        B = torch.randn(n, n, dtype=torch.float64, generator=g)
        mats.append(0.5 * (B + B.T))
    P = eigen._padded(mats, 8)
    assert P.shape == (3, 8, 8)
    for k, a in enumerate(mats):
        n = a.shape[0]
        assert torch.equal(P[k, :n, :n], a)
        assert torch.count_nonzero(P[k, :n, n:]) == 0 and torch.count_nonzero(P[k, n:, :n]) == 0
        if n < 8:
            pad = torch.diagonal(P[k, n:, n:])
            assert torch.all(pad == pad[0])
            # above every eigenvalue of every matrix of the batch
            assert float(pad[0]) > max(float(torch.linalg.eigvalsh(m).max()) for m in mats)
