"""lss_compact_u32 (the kernel-level replacement of the reference's
CudppCompact) against numpy on device buffers: stable order, exact count,
ragged sizes across tile boundaries, empty input, all-valid input."""
import ctypes as C

import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss

pytestmark = pytest.mark.gpu


def compact_gpu(src, valid, offset=0):
    """offset > 0 places src and valid that many elements into their
    allocations (4-byte aligned, not 16-byte: the element-wise reads)."""
    import torch
    L = lss.load()
    pad = max(1, src.size) + offset  # non-null device buffers even for n = 0
    s0 = torch.zeros(pad, dtype=torch.int32, device="cuda")
    v0 = torch.zeros(pad, dtype=torch.int32, device="cuda")
    s, v = s0[offset:], v0[offset:]
    s[: src.size] = torch.from_numpy(src.astype(np.uint32).view(np.int32)).cuda()
    v[: src.size] = torch.from_numpy(valid.astype(np.uint32).view(np.int32)).cuda()
    d = torch.full((max(1, src.size),), -1, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = L.lss_compact_u32(C.c_void_p(s.data_ptr()), C.c_void_p(v.data_ptr()),
                           C.c_void_p(d.data_ptr()), src.size, C.c_void_p(cnt.data_ptr()),
                           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    n = int(cnt.item())
    return d.cpu().numpy().view(np.uint32)[:n], n


@pytest.mark.parametrize("n,p", [(0, 0.5), (1, 1.0), (4095, 0.3), (4096, 0.5), (4097, 0.01),
                                 (100_003, 0.5), (3_000_000, 0.02), (1 << 22, 1.0),
                                 # nothing kept; exactly one full scan block of tile counts;
                                 # more tile counts than one scan block takes (8192 x 4096)
                                 (5_000_001, 0.0), (1 << 25, 0.5), (40_000_003, 0.3)])
def test_compact_matches_numpy(n, p):
    rng = np.random.default_rng(n)
    src = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
    valid = (rng.random(n) < p).astype(np.uint32) * rng.integers(1, 7, size=n).astype(np.uint32)
    out, cnt = compact_gpu(src, valid)
    ref = src[valid != 0]
    assert cnt == ref.size
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("n,offset", [(100_003, 1), (4097, 3)])
def test_compact_unaligned_buffers(n, offset):
    rng = np.random.default_rng(n + offset)
    src = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
    valid = (rng.random(n) < 0.4).astype(np.uint32)
    out, cnt = compact_gpu(src, valid, offset)
    ref = src[valid != 0]
    assert cnt == ref.size
    assert np.array_equal(out, ref)
