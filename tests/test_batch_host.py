"""Host-side helpers of the batched renderer (no GPU needed)."""


def test_chunked_dot_matches_one_dot():
    """The normal loss head's dot product in pieces (cuBLAS takes 32-bit
    lengths; one exhaustive transient of the batched workload holds 2^31
    elements): the same value for chunks that do and do not divide the length,
    and zero for empty vectors."""
    import torch

    from totri_gb300.batch import chunked_dot
    g = torch.Generator().manual_seed(3)
    a = torch.randn(4, 250, dtype=torch.float64, generator=g)
    b = torch.randn(4, 250, dtype=torch.float64, generator=g)
    ref = torch.dot(a.reshape(-1), b.reshape(-1))
    for chunk in (1, 7, 250, 1000, 1 << 30):
        assert torch.allclose(chunked_dot(a, b, chunk=chunk), ref, rtol=1e-12, atol=1e-12)
    assert float(chunked_dot(a[:0], b[:0])) == 0.0
