"""The allocation-free compaction entry point (lss_compact_u32_noalloc).

It serves callers that cannot allocate device memory when they compact
(device memory reserved once at start-up, or an allocator owned by another
framework), so its scratch is a fixed device array of the library.  This checks it through the C ABI against the allocating entry
point lss_compact_u32 on the same inputs, on two calls in a row (the second
call must not see the first call's scratch), and that sizes above its stated
maximum are refused.  Integer outputs: equality is exact.  The file runs last
so that a stop-at-first-failure run has run every other test first."""
import ctypes as C

import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss

pytestmark = pytest.mark.gpu

MAX_ELEMENTS = 1 << 26


def _run(fn, src, valid):
    import torch
    s = torch.from_numpy(src.view(np.int32)).cuda()
    v = torch.from_numpy(valid.view(np.int32)).cuda()
    d = torch.full((src.size,), -1, dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    rc = fn(C.c_void_p(s.data_ptr()), C.c_void_p(v.data_ptr()), C.c_void_p(d.data_ptr()),
            src.size, C.c_void_p(cnt.data_ptr()),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    n = int(cnt.item())
    return d.cpu().numpy().view(np.uint32)[:n].copy(), n


def test_no_alloc_matches_allocating_entry_point_twice():
    L = lss.load()
    rng = np.random.default_rng(2024)
    for call, (n, p) in enumerate([(3_000_017, 0.3), (1_000_003, 0.05)]):
        src = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
        valid = (rng.random(n) < p).astype(np.uint32)
        a, na = _run(L.lss_compact_u32, src, valid)
        b, nb = _run(L.lss_compact_u32_noalloc, src, valid)
        assert na == nb == int(valid.sum()), call
        assert np.array_equal(a, b), call
        assert np.array_equal(b, src[valid != 0]), call


def test_no_alloc_at_its_maximum_size():
    """The fixed array holds the scratch of the largest accepted n (its tile
    counts fill the array; two scan blocks)."""
    L = lss.load()
    rng = np.random.default_rng(26)
    src = rng.integers(0, 2**32 - 1, size=MAX_ELEMENTS, dtype=np.uint64).astype(np.uint32)
    valid = (rng.random(MAX_ELEMENTS) < 0.5).astype(np.uint32)
    b, nb = _run(L.lss_compact_u32_noalloc, src, valid)
    ref = src[valid != 0]
    assert nb == ref.size
    assert np.array_equal(b, ref)


def test_no_alloc_refuses_sizes_above_its_maximum():
    import torch
    L = lss.load()
    buf = torch.zeros(4, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    rc = L.lss_compact_u32_noalloc(p, p, p, MAX_ELEMENTS + 1, C.c_void_p(cnt.data_ptr()), None)
    assert rc == 9  # LSS_ERR_CAPACITY, buffers untouched
