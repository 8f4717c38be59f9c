"""gbmm_mpn_toom22_mul_noalloc: the Toom-2.2 product for callers that cannot
allocate device memory (scratch is the library's fixed device array).  Checked
through the C ABI against gbmm_mpn_toom22_mul with caller scratch, on two calls
in a row (the second call reuses the array the first one left dirty).  This
file is collected last so a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def test_toom22_noalloc_matches_scratch_version(built_lib):
    import torch
    import gbmm
    L = gbmm.lib()
    fn = L.gbmm_mpn_toom22_mul_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                   ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    for call, (an, bn, nb) in enumerate([(64, 60, 3000), (41, 40, 5000)]):
        a = rng.integers(0, 2**32, size=(an, nb), dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 2**32, size=(bn, nb), dtype=np.uint64).astype(np.uint32)
        a[:, :7] = 0xFFFFFFFF  # long carry chains
        da, db = _dev(torch, a), _dev(torch, b)
        ref = torch.zeros((an + bn) * nb, dtype=torch.int32, device="cuda")
        scratch = torch.zeros(gbmm.mpn_toom22_mul_itch(an, bn) * nb, dtype=torch.int32, device="cuda")
        gbmm.check(L.gbmm_mpn_toom22_mul(ref.data_ptr(), da.data_ptr(), an, db.data_ptr(), bn, scratch.data_ptr(),
                                         nb, nb, stream))
        got = torch.full(((an + bn) * nb,), -1, dtype=torch.int32, device="cuda")
        gbmm.check(fn(got.data_ptr(), da.data_ptr(), an, db.data_ptr(), bn, nb, nb, stream))
        torch.cuda.synchronize()
        assert torch.equal(got, ref), f"call {call} differs from the caller-scratch entry point"


def test_toom22_noalloc_rejects_oversized_batches(built_lib):
    import gbmm
    L = gbmm.lib()
    fn = L.gbmm_mpn_toom22_mul_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                   ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    an = bn = 128
    nb = (16 * 1024 * 1024) // (4 * gbmm.mpn_toom22_mul_itch(an, bn)) + 1
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check fails first
    assert fn(dummy, dummy, an, dummy, bn, nb, nb, None) == gbmm.ERR_CAPACITY
    assert b"fixed" in L.gbmm_last_error_string()
