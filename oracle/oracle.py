"""ctypes binding of the CPU oracle (oracle.c).  TEST INFRASTRUCTURE ONLY:
imported by tests/, the smoke check and the benchmark's CPU-baseline leg as the
reference for expected results; never by the product path.

The oracle restates the reference's mat-cpu algorithm (tomsmeding/bachelor-thesis,
mat-cpu/mat.c, matj.c) over a GMP-semantics big-integer restatement; see the
header of oracle.c for the file:line map and how it is pinned.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
CLI_PATH = os.path.join(HERE, "_build", "oracle-cpu")
REF_CLI = os.path.join(HERE, "_ref", "mat-cpu")

_lib = None


def reference_dir():
    """Root of a checkout of the reference (the directory holding mat-cpu/), taken
    from the GBMM_REFERENCE_DIR environment variable; None when unset or absent."""
    d = os.environ.get("GBMM_REFERENCE_DIR", "")
    return d if d and os.path.isdir(os.path.join(d, "mat-cpu")) else None


def build(with_ref=None):
    """Compiles the oracle, and _ref/mat-cpu from the reference's own sources when
    GBMM_REFERENCE_DIR names a checkout of the reference (skipped otherwise)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref = reference_dir()
    if with_ref is None:
        with_ref = ref is not None
    if with_ref and ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.oracle_matmul_text.restype = ctypes.c_void_p
        L.oracle_matmul_text.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.oracle_free.argtypes = [P]
        L.oracle_set_backend.argtypes = [ctypes.c_int]
        L.oracle_matmul_planes.argtypes = [ctypes.c_int] * 3 + [P, P, ctypes.c_int64] * 2 + \
            [P, P, ctypes.c_int32, ctypes.c_int64] + [ctypes.c_int] * 5
        L.oracle_addsub_planes.argtypes = [ctypes.c_int64, P, P, ctypes.c_int64, P, P, ctypes.c_int64,
                                           P, P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int]
        L.oracle_mpz_mulops.argtypes = [ctypes.c_int64, ctypes.c_int, P, P, ctypes.c_int64, P, P, ctypes.c_int64,
                                        P, P, ctypes.c_int32, ctypes.c_int64]
        L.oracle_mpn_add_n.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, P]
        L.oracle_mpn_sub_n.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, P]
        L.oracle_mpn_mul1ops.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P, ctypes.c_int64, ctypes.c_int64, P]
        L.oracle_mpn_mul_basecase.argtypes = [P, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int64, ctypes.c_int64]
        L.oracle_sample_rows.restype = ctypes.c_double
        L.oracle_sample_rows.argtypes = [ctypes.c_int] * 3 + [P, P, ctypes.c_int64] * 2 + \
            [P, P, ctypes.c_int32, ctypes.c_int64] + [ctypes.c_int] * 6
        L.oracle_mpn_addsub.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int64,
                                        ctypes.c_int64, P]
        L.oracle_mpn_addsub_1.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P, ctypes.c_int64, ctypes.c_int64, P]
        L.oracle_mpn_cmp.argtypes = [P, P, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, P]
        L.oracle_mpn_zero_p.argtypes = [P, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, P]
        L.oracle_mpn_neg_com.argtypes = [ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, P]
        _lib = L
    return _lib


def set_backend(gmp):
    """0 = own restatement, 1 = system libgmp.so.10; returns True on success."""
    return lib().oracle_set_backend(int(gmp)) == 0


def gmp_available():
    return bool(lib().oracle_gmp_available())


def matmul_text(text, method=1, basesz=32, jobsz=128, nthreads=1):
    """mat-cpu -i -p equivalent: input text in, mat_write text out, plus seconds."""
    b = text.encode() if isinstance(text, str) else text
    secs = ctypes.c_double(0)
    p = lib().oracle_matmul_text(b, len(b), method, basesz, jobsz, nthreads, ctypes.byref(secs))
    if not p:
        raise ValueError("oracle could not parse the matrix text")
    out = ctypes.string_at(p).decode()
    lib().oracle_free(p)
    return out, secs.value


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def matmul_planes(K, M, N, A, B, cn, method=1, basesz=32, jobsz=128, nthreads=1, C=None):
    """A, B = (limbs [nl, n], sizes [n]) numpy planes; returns C planes with cn limbs.
    With C given, computes C += A*B."""
    Al, As = _c(A[0], np.uint32), _c(A[1], np.int32)
    Bl, Bs = _c(B[0], np.uint32), _c(B[1], np.int32)
    if C is None:
        Cl = np.zeros((cn, K * N), dtype=np.uint32)
        Cs = np.zeros(K * N, dtype=np.int32)
        acc = 0
    else:
        Cl, Cs = _c(C[0], np.uint32).copy(), _c(C[1], np.int32).copy()
        acc = 1
    rc = lib().oracle_matmul_planes(K, M, N, Al.ctypes.data, As.ctypes.data, K * M, Bl.ctypes.data, Bs.ctypes.data,
                                    M * N, Cl.ctypes.data, Cs.ctypes.data, cn, K * N, method, basesz, jobsz, nthreads,
                                    acc)
    if rc != 0:
        raise ValueError("oracle: C capacity too small")
    return Cl, Cs


def sample_rows(K, M, N, A, B, r0, rb, method=1, basesz=32, jobsz=128, nthreads=1, cn=None):
    """Rows [r0, r0 + rb) of C = A*B by mat-cpu's method 1 (naive order) or 31
    (jobsz-blocks with Winograd leaves; rb must equal jobsz), timing only the
    multiplication.  Returns (seconds, (C limbs [cn, rb*N], C sizes [rb*N]))."""
    Al, As = _c(A[0], np.uint32), _c(A[1], np.int32)
    Bl, Bs = _c(B[0], np.uint32), _c(B[1], np.int32)
    cn = cn or (Al.shape[0] + Bl.shape[0] + 2)
    Cl = np.zeros((cn, rb * N), dtype=np.uint32)
    Cs = np.zeros(rb * N, dtype=np.int32)
    secs = lib().oracle_sample_rows(K, M, N, Al.ctypes.data, As.ctypes.data, K * M, Bl.ctypes.data, Bs.ctypes.data,
                                    M * N, Cl.ctypes.data, Cs.ctypes.data, cn, rb * N, r0, rb, method, basesz, jobsz,
                                    nthreads)
    if secs < 0:
        raise ValueError("oracle: bad sample request or C capacity too small")
    return secs, (Cl, Cs)


def addsub_planes(A, B, cn, sub):
    n = A[1].shape[0]
    Al, As, Bl, Bs = _c(A[0], np.uint32), _c(A[1], np.int32), _c(B[0], np.uint32), _c(B[1], np.int32)
    Cl = np.zeros((cn, n), dtype=np.uint32)
    Cs = np.zeros(n, dtype=np.int32)
    rc = lib().oracle_addsub_planes(n, Al.ctypes.data, As.ctypes.data, n, Bl.ctypes.data, Bs.ctypes.data, n,
                                    Cl.ctypes.data, Cs.ctypes.data, cn, n, int(sub))
    if rc:
        raise ValueError("oracle: capacity")
    return Cl, Cs


def mpz_mulops(op, U, V, W, wn):
    """op 0: w = u*v, 1: w += u*v, 2: w -= u*v."""
    n = U[1].shape[0]
    Ul, Us, Vl, Vs = _c(U[0], np.uint32), _c(U[1], np.int32), _c(V[0], np.uint32), _c(V[1], np.int32)
    Wl = np.zeros((wn, n), dtype=np.uint32)
    Ws = np.zeros(n, dtype=np.int32)
    if W is not None:
        Wl[:W[0].shape[0]] = W[0]
        Ws[:] = W[1]
    rc = lib().oracle_mpz_mulops(n, op, Ul.ctypes.data, Us.ctypes.data, n, Vl.ctypes.data, Vs.ctypes.data, n,
                                 Wl.ctypes.data, Ws.ctypes.data, wn, n)
    if rc:
        raise ValueError("oracle: capacity")
    return Wl, Ws


def mpn_add_n(u, v, sub=False):
    """u, v: uint32 [n, nb] -> (r [n, nb], carry [nb])."""
    u, v = _c(u, np.uint32), _c(v, np.uint32)
    n, nb = u.shape
    r = np.zeros_like(u)
    cy = np.zeros(nb, dtype=np.uint32)
    f = lib().oracle_mpn_sub_n if sub else lib().oracle_mpn_add_n
    f(r.ctypes.data, u.ctypes.data, v.ctypes.data, n, nb, nb, cy.ctypes.data)
    return r, cy


def mpn_mul1ops(op, r, u, vl):
    r, u, vl = _c(r, np.uint32).copy(), _c(u, np.uint32), _c(vl, np.uint32)
    n, nb = u.shape
    cy = np.zeros(nb, dtype=np.uint32)
    lib().oracle_mpn_mul1ops(op, r.ctypes.data, u.ctypes.data, n, vl.ctypes.data, nb, nb, cy.ctypes.data)
    return r, cy


def mpn_mul_basecase(u, v):
    u, v = _c(u, np.uint32), _c(v, np.uint32)
    un, nb = u.shape
    vn = v.shape[0]
    r = np.zeros((un + vn, nb), dtype=np.uint32)
    lib().oracle_mpn_mul_basecase(r.ctypes.data, u.ctypes.data, un, v.ctypes.data, vn, nb, nb)
    return r


def mpn_addsub(u, v, sub=False):
    """u [un, nb], v [vn, nb] (un >= vn) -> (r [un, nb], carry / borrow [nb])."""
    u, v = _c(u, np.uint32), _c(v, np.uint32)
    un, nb = u.shape
    vn = v.shape[0]
    r = np.zeros_like(u)
    cy = np.zeros(nb, dtype=np.uint32)
    lib().oracle_mpn_addsub(int(sub), r.ctypes.data, u.ctypes.data, un, v.ctypes.data, vn, nb, nb, cy.ctypes.data)
    return r, cy


def mpn_addsub_1(u, vl, sub=False):
    u, vl = _c(u, np.uint32), _c(vl, np.uint32)
    n, nb = u.shape
    r = np.zeros_like(u)
    cy = np.zeros(nb, dtype=np.uint32)
    lib().oracle_mpn_addsub_1(int(sub), r.ctypes.data, u.ctypes.data, n, vl.ctypes.data, nb, nb, cy.ctypes.data)
    return r, cy


def mpn_cmp(u, v):
    u, v = _c(u, np.uint32), _c(v, np.uint32)
    n, nb = u.shape
    res = np.zeros(nb, dtype=np.int32)
    lib().oracle_mpn_cmp(u.ctypes.data, v.ctypes.data, n, nb, nb, res.ctypes.data)
    return res


def mpn_zero_p(u):
    u = _c(u, np.uint32)
    n, nb = u.shape
    res = np.zeros(nb, dtype=np.int32)
    lib().oracle_mpn_zero_p(u.ctypes.data, n, nb, nb, res.ctypes.data)
    return res


def mpn_neg_com(u, com=False):
    """-u mod B^n with the nonzero flag (neg), or ~u (com)."""
    u = _c(u, np.uint32)
    n, nb = u.shape
    r = np.zeros_like(u)
    cy = np.zeros(nb, dtype=np.uint32)
    lib().oracle_mpn_neg_com(int(com), r.ctypes.data, u.ctypes.data, n, nb, nb, cy.ctypes.data)
    return r, cy


def ref_cli_available():
    return os.path.exists(REF_CLI)


def run_ref_cli(text, method=1, extra=()):
    """Runs the reference's own mat-cpu (built from its sources) on input text."""
    p = subprocess.run([REF_CLI, "-i", "-p", "-m", str(method)] + list(extra), input=text.encode(),
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, check=True)
    return p.stdout.decode()
