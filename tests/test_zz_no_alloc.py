"""The allocation-free de-duplication entry point, checked against the
regular one.

pierce_deduplicate_pairs_noalloc exists for callers that cannot allocate
device memory where they need unique pairs (code that must not let
cudaMalloc/cudaFree synchronise the device, plug-ins whose host owns the
memory budget); it takes its scratch from a fixed device array instead.
This file is collected last so that a failure here cannot hide earlier ones,
and it also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _unique_sorted(pairs: np.ndarray) -> np.ndarray:
    return np.unique(pairs.view(np.int64).reshape(-1))


def test_noalloc_matches_merge_and_deduplicate_two_calls():
    torch = pytest.importorskip("torch")
    from pierce_gb300 import capi
    from pierce_gb300 import join as J

    L = capi.lib()
    ctx = J.Context(0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(20261203)
    for call, n in enumerate((300_000, 1_234_567)):
        ids = rng.integers(0, 4000 if call == 0 else 30_000, size=(n, 2)).astype(np.int32)
        d_in = torch.from_numpy(ids).cuda()
        d_out = torch.full((n, 2), -7, dtype=torch.int32, device="cuda")
        d_cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
        st = L.pierce_deduplicate_pairs_noalloc(d_in.data_ptr(), n, d_out.data_ptr(), d_cnt.data_ptr(),
                                                stream.cuda_stream)
        assert st == capi.OK, L.pierce_last_error()
        torch.cuda.synchronize()
        count = int(d_cnt.item())
        got = d_out[:count].cpu().numpy()

        d_ref = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        nu = C.c_int64()
        capi.check(L.pierce_merge_and_deduplicate_pairs(ctx.handle, d_in.data_ptr(), n, None, 0,
                                                        d_ref.data_ptr(), C.byref(nu)), "merge_and_deduplicate")
        want = d_ref[: nu.value].cpu().numpy()

        assert count == nu.value
        assert np.array_equal(_unique_sorted(got), _unique_sorted(want))
        assert np.array_equal(_unique_sorted(want), _unique_sorted(ids))
    ctx.close()


def test_noalloc_keeps_the_pair_minus_one_minus_one():
    """(-1, -1) packs to the empty-slot marker of the hash set; it must come
    out like any other pair, once, on two calls in a row."""
    torch = pytest.importorskip("torch")
    from pierce_gb300 import capi

    L = capi.lib()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    ids = np.array([[-1, -1], [0, 0], [-1, -1], [5, -1], [-1, 5], [0, 0], [7, 9]], np.int32)
    for _ in range(2):
        d_in = torch.from_numpy(ids).cuda()
        d_out = torch.full((len(ids), 2), -7, dtype=torch.int32, device="cuda")
        d_cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
        assert L.pierce_deduplicate_pairs_noalloc(d_in.data_ptr(), len(ids), d_out.data_ptr(), d_cnt.data_ptr(),
                                                  stream.cuda_stream) == capi.OK, L.pierce_last_error()
        torch.cuda.synchronize()
        got = d_out[: int(d_cnt.item())].cpu().numpy()
        assert np.array_equal(_unique_sorted(got), _unique_sorted(ids))
        assert len(got) == len(_unique_sorted(ids))


def test_noalloc_rejects_oversized_input():
    pytest.importorskip("torch")
    from pierce_gb300 import capi

    L = capi.lib()
    d = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = L.pierce_deduplicate_pairs_noalloc(d, capi.NOALLOC_MAX_PAIRS + 1, d, d, None)
    assert st == capi.ERR_INVALID_ARGUMENT
    assert b"exceed the maximum" in L.pierce_last_error()
