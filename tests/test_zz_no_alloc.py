"""gbmm_mpn_toom22_mul_noalloc: the Toom-2.2 product for callers that cannot
allocate device memory.  Operands that fit shared memory run on chip; longer
ones (above about 800 limbs) use the library's fixed device array as scratch.
Checked through the C ABI against gbmm_mpn_toom22_mul with caller scratch, on
calls in a row (a later call reuses the array an earlier one left dirty), and the
long cases against the exact product.  This file is collected last so a failure
here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _noalloc_fn(gbmm):
    fn = gbmm.lib().gbmm_mpn_toom22_mul_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                   ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


# (an, bn, nb, ld): two calls in a row with ld == nb, one with planes wider than
# the batch (ld > nb), and one whose scratch is exactly the array's size
# (itch 512 limbs x ld 8192 x 4 bytes = 16 MiB), which the size check accepts
CASES = [(64, 60, 3000, 3000), (41, 40, 5000, 5000), (64, 60, 3000, 3500), (170, 150, 8000, 8192),
         (850, 800, 64, 64), (851, 700, 40, 41)]


def test_toom22_noalloc_matches_scratch_version(built_lib):
    import torch
    import gbmm
    L = gbmm.lib()
    fn = _noalloc_fn(gbmm)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    assert gbmm.mpn_toom22_mul_itch(170, 150) * 8192 * 4 == 16 * 1024 * 1024
    for call, (an, bn, nb, ld) in enumerate(CASES):
        a = rng.integers(0, 2**32, size=(an, ld), dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 2**32, size=(bn, ld), dtype=np.uint64).astype(np.uint32)
        a[:, :7] = 0xFFFFFFFF  # long carry chains
        da, db = _dev(torch, a), _dev(torch, b)
        ref = torch.full(((an + bn) * ld,), 5, dtype=torch.int32, device="cuda")
        scratch = torch.zeros(gbmm.mpn_toom22_mul_itch(an, bn) * ld, dtype=torch.int32, device="cuda")
        gbmm.check(L.gbmm_mpn_toom22_mul(ref.data_ptr(), da.data_ptr(), an, db.data_ptr(), bn, scratch.data_ptr(),
                                         ld, nb, stream))
        got = torch.full(((an + bn) * ld,), 5, dtype=torch.int32, device="cuda")
        gbmm.check(fn(got.data_ptr(), da.data_ptr(), an, db.data_ptr(), bn, ld, nb, stream))
        torch.cuda.synchronize()
        assert torch.equal(got, ref), f"call {call} differs from the caller-scratch entry point"
        # columns past the batch (ld > nb) are left as they were
        assert bool((got.view(an + bn, ld)[:, nb:] == 5).all())
        if an >= 800:  # the device-array form: also against the exact product
            g = got.cpu().numpy().view(np.uint32).reshape(an + bn, ld)
            for j in (0, nb // 2, nb - 1):
                x = sum(int(a[i, j]) << (32 * i) for i in range(an))
                y = sum(int(b[i, j]) << (32 * i) for i in range(bn))
                assert sum(int(g[i, j]) << (32 * i) for i in range(an + bn)) == x * y, (call, j)


def test_toom22_noalloc_rejects_oversized_batches(built_lib):
    import gbmm
    L = gbmm.lib()
    fn = _noalloc_fn(gbmm)
    an = bn = 128
    nb = (16 * 1024 * 1024) // (4 * gbmm.mpn_toom22_mul_itch(an, bn)) + 1
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check fails first
    assert fn(dummy, dummy, an, dummy, bn, nb, nb, None) == gbmm.ERR_CAPACITY
    assert b"fixed" in L.gbmm_last_error_string()
    # one plane of stride more than the exact fit is rejected too
    assert fn(dummy, dummy, 170, dummy, 150, 8193, 8000, None) == gbmm.ERR_CAPACITY
    # operand lengths whose scratch count would overflow 32 bits are rejected, not wrapped
    big = 2 * 715827883
    assert gbmm.mpn_toom22_mul_itch(big, big) == -1
    assert fn(dummy, dummy, big, dummy, big - 10, 1, 1, None) == gbmm.ERR_CAPACITY
