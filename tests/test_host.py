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


def test_gmp_limb_import_export(built_lib):
    import gbmm
    L = gbmm.lib()
    rng = random.Random(2)
    vals = [0, -1, 2**64 - 1, -(2**64), 2**95] + [rng.getrandbits(rng.randint(1, 700)) * rng.choice((-1, 1))
                                                 for _ in range(50)]
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
