"""GPU: grns_max_noalloc, the maximum for callers that cannot allocate device
memory when they call (their memory belongs to another allocator, or
cudaMalloc's possible device-wide synchronisation is not acceptable).  It
must return exactly what grns_max returns.  Two calls in a row on different
data check that the shared in-library scratch area is reset between calls.
Collected last so that a run stopping at the first failure has run every
other test; it needs no state from them."""
import ctypes

import numpy as np
import pytest

from oracle.oracle import greedy_moduli

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_max_noalloc_matches_grns_max():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from grns_gb300 import native
    from grns_gb300.workload import S_MAX, S_X
    L = native.lib(build_if_missing=True)
    n = 32
    mods = (ctypes.c_int32 * n)(*greedy_moduli(n))
    ctx = ctypes.c_void_p()
    assert L.grns_ctx_create(mods, n, ctypes.byref(ctx)) == 0
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    try:
        for call, (count, seed, stream_id) in enumerate([(300000, 5, S_MAX), (70001, 6, S_X)]):
            x = torch.empty((n, count), dtype=torch.int32, device="cuda")
            assert L.grns_gen_uniform(ctx, seed, stream_id, count, 0, P(x), stream) == 0
            if call == 1:  # a repeated maximum: the smallest index must win
                x[:, count - 1] = x[:, 17]
            val_ref = torch.zeros(n, dtype=torch.int32, device="cuda")
            idx_ref = torch.zeros(1, dtype=torch.int64, device="cuda")
            assert L.grns_max(ctx, P(x), count, 0, P(val_ref), P(idx_ref), None, 0, stream) == 0
            val = torch.full((n,), -1, dtype=torch.int32, device="cuda")
            idx = torch.full((1,), -2, dtype=torch.int64, device="cuda")
            assert L.grns_max_noalloc(ctx, P(x), count, 0, P(val), P(idx), stream) == 0
            torch.cuda.synchronize()
            assert int(idx.item()) == int(idx_ref.item())
            assert torch.equal(val, val_ref)
            assert 0 <= int(idx.item()) < count
            assert np.array_equal(val.cpu().numpy(), x[:, int(idx.item())].cpu().numpy())
    finally:
        L.grns_ctx_destroy(ctx)
