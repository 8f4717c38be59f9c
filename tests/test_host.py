"""Host-side checks that need no GPU: the C-ABI library loads and exports every
symbol include/gbmm.h declares; text and GMP-limb conversion; error codes."""
import ctypes
import os
import random
import re

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "gbmm.h")).read()
    decl = re.compile(r"^(?:gbmm_status|int32_t|uint64_t|const char \*)\s*(gbmm_[a-z0-9_]+)\(", re.M)
    return sorted(set(decl.findall(text)))


def test_header_symbols_exported(built_lib):
    syms = header_symbols()
    assert len(syms) > 30
    missing = [s for s in syms if not hasattr(built_lib, s)]
    assert not missing, missing


def test_version(built_lib):
    import gbmm
    assert gbmm.lib().gbmm_version().startswith(b"gbmm")


def test_parse_format_roundtrip(built_lib):
    import gbmm
    rng = random.Random(1)
    vals = [0, 1, -1, 2**32 - 1, -(2**32), 2**64 + 5] + [rng.getrandbits(rng.randint(1, 900)) * rng.choice((-1, 1))
                                                         for _ in range(200)]
    rows, cols = 2, len(vals) // 2
    text = gbmm.format_matrix(rows, cols, vals)
    nl = 30
    limbs, sizes, used = gbmm.parse_hex(text, len(vals), nl)
    assert gbmm.planes_to_ints(limbs, sizes) == vals
    assert gbmm.format_hex(limbs, sizes, rows, cols) == text
    # uppercase and leading zeros and extra whitespace are accepted
    l2, s2, _ = gbmm.parse_hex("  00ABc\t-0000f  0  -0 ", 4, 2)
    assert gbmm.planes_to_ints(l2, s2) == [0xabc, -0xf, 0, 0]


def test_parse_errors(built_lib):
    import gbmm
    with pytest.raises(gbmm.GbmmError) as e:
        gbmm.parse_hex("12 zz", 2, 4)
    assert e.value.status == gbmm.ERR_PARSE
    with pytest.raises(gbmm.GbmmError) as e:
        gbmm.parse_hex("12 3", 3, 4)
    assert e.value.status == gbmm.ERR_PARSE
    with pytest.raises(gbmm.GbmmError) as e:
        gbmm.parse_hex("1" + "0" * 40, 1, 4)
    assert e.value.status == gbmm.ERR_CAPACITY


@pytest.mark.parametrize("extra,threads", [(50, 0), (40000, 4)])
def test_gmp_limb_import_export(built_lib, extra, threads):
    import gbmm
    L = gbmm.lib()
    rng = random.Random(2)
    vals = [0, -1, 2**64 - 1, -(2**64), 2**95] + [rng.getrandbits(rng.randint(1, 700)) * rng.choice((-1, 1))
                                                 for _ in range(extra)]
    old = _threads(gbmm, threads)
    limbs64, offsets, sizes64 = [], [], []
    for v in vals:
        m = abs(v)
        n = (m.bit_length() + 63) // 64
        offsets.append(len(limbs64))
        limbs64 += [(m >> (64 * i)) & (2**64 - 1) for i in range(n)]
        sizes64.append(-n if v < 0 else n)
    l64 = np.array(limbs64 + [0], dtype=np.uint64)
    off = np.array(offsets, dtype=np.int64)
    s64 = np.array(sizes64, dtype=np.int32)
    n = len(vals)
    nl = 24
    limbs = np.zeros((nl, n), dtype=np.uint32)
    sizes = np.zeros(n, dtype=np.int32)
    gbmm.check(L.gbmm_import_gmp(n, l64.ctypes.data, off.ctypes.data, s64.ctypes.data, limbs.ctypes.data,
                                 sizes.ctypes.data, nl, n))
    assert gbmm.planes_to_ints(limbs, sizes) == vals
    back = np.zeros_like(l64)
    s_back = np.zeros_like(s64)
    gbmm.check(L.gbmm_export_gmp(n, limbs.ctypes.data, sizes.ctypes.data, nl, n, back.ctypes.data, off.ctypes.data,
                                 s_back.ctypes.data))
    _threads(gbmm, old)
    assert (back == l64).all() and (s_back == s64).all()


def test_limbs_needed(built_lib):
    import gbmm
    assert gbmm.limbs_needed(32, 32, 64, method=gbmm.METHOD_NAIVE) >= 65
    assert gbmm.limbs_needed(64, 64, 256) >= gbmm.limbs_needed(64, 64, 256, method=gbmm.METHOD_NAIVE)


def test_null_arguments_rejected(built_lib):
    import gbmm
    L = gbmm.lib()
    assert L.gbmm_create(None) == gbmm.ERR_INVALID
    assert L.gbmm_mpn_add_n(None, None, None, 4, 4, 1, None, None) == gbmm.ERR_INVALID
    assert b"null" in L.gbmm_last_error_string()


def test_cli_generate_matches_oracle_generator(built_lib, oracle):
    import subprocess
    import build as gbuild
    cli = gbuild.CLI
    ref = oracle.CLI_PATH
    if not os.path.exists(ref):
        oracle.build(with_ref=False)
    for args in (["-n", "3,4,5", "-b", "200", "-s", "9"], ["-n", "1,7,2", "-b", "64", "-s", "1"]):
        a = subprocess.run([cli, "-g"] + args, stdout=subprocess.PIPE, check=True).stdout
        b = subprocess.run([ref, "-g"] + args, stdout=subprocess.PIPE, check=True).stdout
        assert a == b


def _threads(gbmm, n):
    f = gbmm.lib().gbmmx_host_threads
    f.argtypes = [ctypes.c_int32]
    f.restype = ctypes.c_int32
    return f(n)


def test_parallel_text_and_gmp_conversions_match_serial(built_lib):
    """Inputs large enough to split across host threads give the same planes,
    text, errors and consumed offsets as the single-thread path."""
    import gbmm
    rng = random.Random(12)
    vals = [0 if i % 97 == 0 else rng.getrandbits(rng.choice((4, 64, 900, 3000))) * rng.choice((-1, 1))
            for i in range(36000)]
    text = " ".join(format(v, "x") if v >= 0 else "-" + format(-v, "x") for v in vals) + "\n"
    assert len(text) > 7 << 20  # enough for 7 threads of at least 1 MiB each
    old = _threads(gbmm, 1)
    try:
        ref = gbmm.parse_hex(text, len(vals), 100)
        for n in (2, 3, 7):
            _threads(gbmm, n)
            got = gbmm.parse_hex(text, len(vals), 100)
            assert (got[0] == ref[0]).all() and (got[1] == ref[1]).all() and got[2] == ref[2]
            assert gbmm.planes_to_ints(got[0], got[1]) == vals
            assert gbmm.format_hex(got[0], got[1], 360, 100) == gbmm.format_hex(ref[0], ref[1], 360, 100)
        # errors: a bad byte in the middle, a token too long, a short text
        bad = text[:len(text) // 2] + "g" + text[len(text) // 2 + 1:]
        outcomes = []
        for n in (1, 4):
            _threads(gbmm, n)
            res = []
            for t, count, nl in ((bad, len(vals), 100), (text, len(vals), 50), (text, len(vals) + 5, 100)):
                try:
                    gbmm.parse_hex(t, count, nl)
                    res.append(None)
                except gbmm.GbmmError as e:
                    res.append((e.status, str(e)))
            outcomes.append(res)
        assert outcomes[0] == outcomes[1] and all(r is not None for r in outcomes[0])
    finally:
        _threads(gbmm, old)


# FNV-1a checksums of the host-built CRT tables (reconstruction table, Mod's chunk
# values, moduli constants), recorded from the first, one-thread bit-by-bit
# builder; the threaded word-level builder must reproduce them bit for bit.
TABLE_SUMS = {16: 0xf5de9e1fbafc5d3d, 100: 0x29cee628a1c924d9, 516: 0x89360cf85f8369fa,
              1023: 0x583a7024eea96029}


@pytest.mark.parametrize("P", sorted(TABLE_SUMS))
def test_crt_table_build_is_unchanged(built_lib, P):
    f = built_lib.gbmmx_table_build
    f.restype = ctypes.c_uint64
    f.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
    ms = ctypes.c_double()
    assert f(P, ctypes.byref(ms)) == TABLE_SUMS[P]


def test_no_plain_host_to_device_copies():
    """A plain cudaMemcpy from pageable host memory may return before its DMA has
    landed, ordered only against the legacy default stream, so a kernel launched
    next on a non-blocking stream can read stale data (a batch's side-stream
    products read fresh CRT tables this way).  Host-to-device copies and fills
    that are not stream-ordered go through upload_now / fill_now instead."""
    csrc = os.path.join(ROOT, "bachelor-thesis_gb300", "csrc")
    bad = []
    for name in sorted(os.listdir(csrc)):
        if not name.endswith((".cu", ".cpp", ".cuh", ".h")):
            continue
        for no, line in enumerate(open(os.path.join(csrc, name)), 1):
            code = line.split("//")[0]
            if re.search(r"\bcudaMemcpy\([^;]*cudaMemcpyHostToDevice", code) or \
                    re.search(r"\bcudaMemcpyToSymbol\(", code) or re.search(r"\bcudaMemset\(", code):
                bad.append(f"{name}:{no}: {line.strip()}")
    # the device error word is cleared once with a device-wide synchronisation after it
    bad = [b for b in bad if "cudaMemset(p, 0, sizeof(uint32_t))" not in b]
    assert not bad, bad


def _primes_desc_below_2_16():
    sieve = bytearray([1]) * 65536
    sieve[0] = sieve[1] = 0
    for i in range(2, 256):
        if sieve[i]:
            sieve[i * i::i] = bytearray(len(range(i * i, 65536, i)))
    return [p for p in range(65535, 2, -1) if sieve[p]]


def test_modulus_count_covers_the_product_bound(built_lib):
    """The CRT form takes the largest odd primes below 2^16 in descending order,
    as few as make Mod >= 2^(bits_a + bits_b + ceil(log2 k) + 18).  An entry of C
    is a sum of k products below 2^(bits_a + bits_b) in magnitude, so Mod exceeds
    twice its magnitude, with 16 bits to spare for the reconstruction's
    fixed-point sign decision.  Checked with exact integers against the host rule
    (floating-point log2 sums) on the benchmark shapes and random ones."""
    f = built_lib.gbmmx_crt_params
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    assert f(64, 64, 16, None) == 1  # GBMM_ERR_INVALID
    primes = _primes_desc_below_2_16()
    prefix = [1]
    rng = random.Random(11)
    cases = [(4096, 4096, 512), (2048, 2048, 256), (16384, 16384, 512), (16384, 64, 16),
             (64, 64, 16), (1, 1, 1), (32, 32, 2), (8192, 8192, 1024)]
    cases += [(rng.randint(1, 16384), rng.randint(1, 16384), rng.randint(1, 4096)) for _ in range(200)]
    for ba, bb, k in cases:
        out = ctypes.c_int32()
        assert f(ba, bb, k, ctypes.byref(out)) == 0
        P = out.value
        assert 1 <= P <= len(primes)
        while len(prefix) <= P:
            prefix.append(prefix[-1] * primes[len(prefix) - 1])
        need = ba + bb + (k - 1).bit_length() + 18
        assert prefix[P] >= 1 << need, (ba, bb, k, P)
        assert prefix[P - 1] < 1 << need, (ba, bb, k, P)
        assert prefix[P] > 2 * k * (1 << (ba + bb)) << 16


def test_parse_limb_boundaries(built_lib):
    """Tokens of 8j - 1, 8j and 8j + 1 digits (a limb's digits end exactly at a
    limb boundary or one past it), tokens that fill the planes exactly, and tokens
    longer than the planes only through leading zeros; the planes past a token's
    limbs are cleared even when they held data."""
    import gbmm
    nl = 4
    vals = []
    for j in range(1, nl + 1):
        for nd in (8 * j - 1, 8 * j, 8 * j + 1):
            if nd <= 8 * nl:
                vals.append(int("f" + "0" * (nd - 2) + "1", 16) if nd > 1 else 1)
                vals.append(-int("8" + "7" * (nd - 1), 16))
    text = " ".join(format(v, "x") if v >= 0 else "-" + format(-v, "x") for v in vals)
    text += " " + "0" * 40 + "abc" + " -" + "0" * 33 + "f" * 32
    vals += [0xabc, -int("f" * 32, 16)]
    n = len(vals)
    limbs = np.full((nl, n), 0xDEADBEEF, dtype=np.uint32)
    sizes = np.full(n, 77, dtype=np.int32)
    used = ctypes.c_size_t(0)
    b = text.encode()
    gbmm.check(gbmm.lib().gbmm_parse_hex(b, len(b), n, limbs.ctypes.data, sizes.ctypes.data, nl, n,
                                         ctypes.byref(used)))
    assert used.value == len(b)
    assert gbmm.planes_to_ints(limbs, sizes) == vals
    for e, v in enumerate(vals):
        need = (abs(v).bit_length() + 31) // 32
        assert abs(int(sizes[e])) == need
        assert (limbs[need:, e] == 0).all()
    with pytest.raises(gbmm.GbmmError) as err:
        gbmm.parse_hex("1" + "0" * (8 * nl), 1, nl)
    assert err.value.status == gbmm.ERR_CAPACITY
