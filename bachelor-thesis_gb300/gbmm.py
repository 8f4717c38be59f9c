"""Python binding of gbmm's C ABI (include/gbmm.h) through ctypes.

This module is the host-side mirror of the reference's operator surface
(tomsmeding/bachelor-thesis): the batched ``mpn_*`` / ``mpz_*`` calls of
mat-gpu/gmp-es.h:668-720 and gmp-es-mpz.h:108-126, the matrix operations
``mat_mul`` / ``mat_addmul`` / ``mat_mul_winograd`` / ``mat_mul_strassen`` /
``squarify_mul`` (mat-cpu/mat.h:20-27, mat-gpu/mat-pregpu.h:54-63) and the hex
matrix I/O ``mat_read`` / ``mat_write`` (mat-cpu/mat.c:336-353).  All
arithmetic runs in libgbmm.so; there is no Python or CPU fallback: if the
library is missing or no GPU is present, calls raise.

Device memory is allocated through PyTorch (plumbing only) and handed to the
library as raw pointers; the library enqueues on the current torch stream.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgbmm.so")

OK, ERR_INVALID, ERR_CAPACITY, ERR_CUDA, ERR_PARSE, ERR_NOMEM, ERR_TIMEOUT, ERR_UNSUPPORTED = range(8)
PATH_AUTO, PATH_LIMB, PATH_CRT = 0, 1, 2
METHOD_NAIVE, METHOD_STRASSEN, METHOD_WINOGRAD, METHOD_NAIVE_REC, METHOD_WINOGRAD_CRT = 1, 3, 35, 4, 350
# gbmm_plan: the candidate plans the autotuner times and the cost model predicts
(PLAN_LIMB_NAIVE, PLAN_LIMB_W32, PLAN_LIMB_W64, PLAN_LIMB_W128, PLAN_CRT, PLAN_CRT_SINGLE, PLAN_CRT_PAIR,
 PLAN_CRT_SPLIT) = range(8)
NPLANS = 8


class GbmmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"gbmm status {status}: {msg}")
        self.status = status


class Mat(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int32), ("cols", ctypes.c_int32), ("nlimbs", ctypes.c_int32),
                ("pad_", ctypes.c_int32), ("rs", ctypes.c_int64), ("ld", ctypes.c_int64),
                ("limbs", ctypes.c_void_p), ("sizes", ctypes.c_void_p)]


class Opts(ctypes.Structure):
    _fields_ = [("path", ctypes.c_int32), ("method", ctypes.c_int32), ("cutoff", ctypes.c_int32),
                ("nprimes", ctypes.c_int32), ("accumulate", ctypes.c_int32), ("plan", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 2)]


class Job(ctypes.Structure):
    _fields_ = [("c", Mat), ("a", Mat), ("b", Mat), ("path", ctypes.c_int32), ("cutoff", ctypes.c_int32),
                ("nprimes", ctypes.c_int32), ("chosen_path", ctypes.c_int32), ("chosen_plan", ctypes.c_int32)]


class HostJob(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int32), ("M", ctypes.c_int32), ("N", ctypes.c_int32),
                ("a_nlimbs", ctypes.c_int32), ("b_nlimbs", ctypes.c_int32), ("c_nlimbs", ctypes.c_int32),
                ("a_limbs", ctypes.c_void_p), ("a_sizes", ctypes.c_void_p),
                ("b_limbs", ctypes.c_void_p), ("b_sizes", ctypes.c_void_p),
                ("c_limbs", ctypes.c_void_p), ("c_sizes", ctypes.c_void_p),
                ("path", ctypes.c_int32), ("method", ctypes.c_int32), ("cutoff", ctypes.c_int32),
                ("nprimes", ctypes.c_int32), ("chosen_path", ctypes.c_int32)]


_lib = None

_P = ctypes.c_void_p
_SIGS = {
    "gbmm_create": [ctypes.POINTER(_P)],
    "gbmm_destroy": [_P],
    "gbmm_set_stream": [_P, _P],
    "gbmm_parse_hex": [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int64, _P, _P, ctypes.c_int32, ctypes.c_int64,
                       ctypes.POINTER(ctypes.c_size_t)],
    "gbmm_format_hex": [_P, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
                        _P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
    "gbmm_import_gmp": [ctypes.c_int64, _P, _P, _P, _P, _P, ctypes.c_int32, ctypes.c_int64],
    "gbmm_export_gmp": [ctypes.c_int64, _P, _P, ctypes.c_int32, ctypes.c_int64, _P, _P, _P],
    "gbmm_upload": [Mat, _P, _P, ctypes.c_int32, ctypes.c_int64, _P],
    "gbmm_download": [Mat, _P, _P, ctypes.c_int32, ctypes.c_int64, _P],
    "gbmm_import_hex": [Mat, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), _P],
    "gbmm_export_hex": [Mat, _P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), _P],
    "gbmm_max_bits": [Mat, ctypes.POINTER(ctypes.c_int64), _P],
    "gbmm_mat_add": [Mat, Mat, Mat, _P],
    "gbmm_mat_sub": [Mat, Mat, Mat, _P],
    "gbmm_matmul_limbs_needed": [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Opts),
                                 ctypes.POINTER(ctypes.c_int32)],
    "gbmm_matmul": [_P, Mat, Mat, Mat, ctypes.POINTER(Opts)],
    "gbmm_mat_mul_naive": [Mat, Mat, Mat, ctypes.c_int32, _P],
    "gbmm_matmul_batched": [_P, ctypes.POINTER(Job), ctypes.c_int32, ctypes.POINTER(Opts)],
    "gbmm_set_graphs": [_P, ctypes.c_int32],
    "gbmm_matmul_host": [_P, ctypes.POINTER(HostJob), ctypes.c_int32],
    "gbmm_set_device_budget": [_P, ctypes.c_uint64],
    "gbmm_autotune": [_P, ctypes.POINTER(Job), ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p],
    "gbmm_tune_save": [_P, ctypes.c_char_p],
    "gbmm_tune_load": [_P, ctypes.c_char_p],
    "gbmm_model_features": [ctypes.c_int32] * 5 + [_P],
    "gbmm_model_init": [_P, ctypes.c_uint64],
    "gbmm_model_set_params": [_P, _P],
    "gbmm_model_get_params": [_P, _P, _P],
    "gbmm_model_use": [_P, ctypes.c_int32],
    "gbmm_model_predict": [_P, _P, ctypes.c_int32, _P],
    "gbmm_model_gradient": [_P, _P, _P, ctypes.c_int32, _P, _P],
    "gbmm_model_train": [_P, _P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, _P],
    "gbmm_mpn_add_n": [_P, _P, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_sub_n": [_P, _P, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_add": [_P, _P, ctypes.c_int32, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_sub": [_P, _P, ctypes.c_int32, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_add_1": [_P, _P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_sub_1": [_P, _P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_cmp": [_P, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_zero_p": [_P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_neg": [_P, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_com": [_P, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P],
    "gbmm_mpn_mul_1": [_P, _P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_addmul_1": [_P, _P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_submul_1": [_P, _P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gbmm_mpn_mul_basecase": [_P, _P, ctypes.c_int32, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, _P],
    "gbmm_mpn_toom22_mul": [_P, _P, ctypes.c_int32, _P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int64, _P],
    "gbmm_mpn_mul": [_P, _P, _P, ctypes.c_int32, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64],
    "gbmm_mpz_add": [Mat, Mat, Mat, _P],
    "gbmm_mpz_sub": [Mat, Mat, Mat, _P],
    "gbmm_mpz_mul": [Mat, Mat, Mat, _P],
    "gbmm_mpz_addmul": [Mat, Mat, Mat, _P],
    "gbmm_mpz_submul": [Mat, Mat, Mat, _P],
}


def lib():
    """Loads libgbmm.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libgbmm.so not built ({LIB_PATH}); run __graft_entry__.build()")
    L = ctypes.CDLL(LIB_PATH)
    for name, args in _SIGS.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.gbmm_last_error_string.restype = ctypes.c_char_p
    L.gbmm_version.restype = ctypes.c_char_p
    L.gbmm_kernel_launches.restype = ctypes.c_uint64
    L.gbmm_profile.argtypes = [ctypes.c_int32]
    L.gbmm_profile_read.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.gbmm_model_nparams.restype = ctypes.c_int32
    L.gbmm_mpn_toom22_mul_itch.restype = ctypes.c_int32
    L.gbmm_mpn_toom22_mul_itch.argtypes = [ctypes.c_int32, ctypes.c_int32]
    _lib = L
    return L


def check(status):
    if status != OK:
        msg = lib().gbmm_last_error_string().decode(errors="replace")
        raise GbmmError(status, msg)


def kernel_launches():
    """Kernels launched by the library so far in this process."""
    return int(lib().gbmm_kernel_launches())


def profile(enable):
    check(lib().gbmm_profile(int(bool(enable))))


def profile_read():
    """{kernel name: (launches, total ms)} from CUDA events recorded around launches."""
    import json
    w = ctypes.c_size_t(0)
    check(lib().gbmm_profile_read(None, 0, ctypes.byref(w)))
    buf = ctypes.create_string_buffer(w.value + 1)
    check(lib().gbmm_profile_read(buf, w.value + 1, ctypes.byref(w)))
    return {k: (v[0], v[1]) for k, v in json.loads(buf.value.decode()).items()}


# ----------------------------------------------------------------------------------
# host-side conversions (numpy limb planes <-> Python ints / hex text)
# ----------------------------------------------------------------------------------
def limbs_for_bits(bits):
    return max(0, (int(bits) + 31) // 32)


def ints_to_planes(values, nlimbs=None):
    """Python ints -> (limbs uint32 [nlimbs, n], sizes int32 [n])."""
    vals = [int(v) for v in values]
    n = len(vals)
    if nlimbs is None:
        nlimbs = max([limbs_for_bits(abs(v).bit_length()) for v in vals] + [1])
    limbs = np.zeros((nlimbs, n), dtype=np.uint32)
    sizes = np.zeros(n, dtype=np.int32)
    nbytes = 4 * nlimbs
    for e, v in enumerate(vals):
        m = abs(v)
        if m:
            ln = limbs_for_bits(m.bit_length())
            if ln > nlimbs:
                raise ValueError(f"entry {e} needs {ln} limbs > {nlimbs}")
            limbs[:, e] = np.frombuffer(m.to_bytes(nbytes, "little"), dtype="<u4")
            sizes[e] = -ln if v < 0 else ln
    return limbs, sizes


def planes_to_ints(limbs, sizes):
    limbs = np.ascontiguousarray(np.asarray(limbs, dtype=np.uint32).T)
    out = []
    for e in range(limbs.shape[0]):
        s = int(sizes[e])
        m = int.from_bytes(limbs[e].tobytes(), "little")
        out.append(-m if s < 0 else m)
    return out


def parse_matrix_text(text):
    """Parses mat-cpu's -i format ("K M N", A, B) -> (K, M, N, A ints, B ints)."""
    tok = text.split()
    K, M, N = int(tok[0]), int(tok[1]), int(tok[2])
    vals = [int(t, 16) for t in tok[3:3 + K * M + M * N]]
    return K, M, N, vals[:K * M], vals[K * M:]


def format_matrix(rows, cols, values):
    """mat_write format (mat-cpu/mat.c:344-353): space separated rows, blank line at the end."""
    lines = []
    for r in range(rows):
        lines.append(" ".join(format(v, "x") if v >= 0 else "-" + format(-v, "x")
                              for v in values[r * cols:(r + 1) * cols]))
    return "\n".join(lines) + "\n\n"


def parse_hex(text, count, nlimbs):
    """C parser (gbmm_parse_hex) -> numpy planes."""
    b = text.encode() if isinstance(text, str) else text
    limbs = np.zeros((max(nlimbs, 1), count), dtype=np.uint32)
    sizes = np.zeros(count, dtype=np.int32)
    used = ctypes.c_size_t(0)
    check(lib().gbmm_parse_hex(b, len(b), count, limbs.ctypes.data, sizes.ctypes.data, nlimbs, count,
                               ctypes.byref(used)))
    return limbs[:nlimbs], sizes, used.value


def format_hex(limbs, sizes, rows, cols):
    limbs = np.ascontiguousarray(limbs, dtype=np.uint32)
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    nl = limbs.shape[0]
    ld = limbs.shape[1] if limbs.ndim == 2 else rows * cols
    w = ctypes.c_size_t(0)
    check(lib().gbmm_format_hex(limbs.ctypes.data, sizes.ctypes.data, nl, ld, rows, cols, cols, None, 0,
                                ctypes.byref(w)))
    buf = ctypes.create_string_buffer(w.value + 1)
    check(lib().gbmm_format_hex(limbs.ctypes.data, sizes.ctypes.data, nl, ld, rows, cols, cols, buf, w.value + 1,
                                ctypes.byref(w)))
    return buf.raw[:w.value].decode()


# ----------------------------------------------------------------------------------
# device side
# ----------------------------------------------------------------------------------
def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("gbmm device calls need a CUDA GPU")
    return torch


def stream_ptr():
    return _torch().cuda.current_stream().cuda_stream


class DeviceMatrix:
    """rows x cols signed integers in device limb planes (owns its memory)."""

    def __init__(self, rows, cols, nlimbs):
        torch = _torch()
        self.rows, self.cols, self.nlimbs = int(rows), int(cols), int(nlimbs)
        n = self.rows * self.cols
        self.limbs_t = torch.zeros(max(1, self.nlimbs * n), dtype=torch.int32, device="cuda")
        self.sizes_t = torch.zeros(max(1, n), dtype=torch.int32, device="cuda")

    @property
    def mat(self):
        m = Mat()
        m.rows, m.cols, m.nlimbs = self.rows, self.cols, self.nlimbs
        m.rs = self.cols
        m.ld = self.rows * self.cols
        m.limbs = self.limbs_t.data_ptr()
        m.sizes = self.sizes_t.data_ptr()
        return m

    def view(self, r0, c0, rows, cols):
        m = self.mat
        off = r0 * m.rs + c0
        m.limbs += 4 * off
        m.sizes += 4 * off
        m.rows, m.cols = rows, cols
        return m

    @classmethod
    def from_ints(cls, rows, cols, values, nlimbs=None):
        limbs, sizes = ints_to_planes(values, nlimbs)
        d = cls(rows, cols, limbs.shape[0])
        d.upload(limbs, sizes)
        return d

    def upload(self, limbs, sizes):
        limbs = np.ascontiguousarray(limbs, dtype=np.uint32)
        sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        n = self.rows * self.cols
        check(lib().gbmm_upload(self.mat, limbs.ctypes.data, sizes.ctypes.data, limbs.shape[0], n, stream_ptr()))

    def download(self):
        n = self.rows * self.cols
        limbs = np.zeros((max(self.nlimbs, 1), n), dtype=np.uint32)
        sizes = np.zeros(n, dtype=np.int32)
        check(lib().gbmm_download(self.mat, limbs.ctypes.data, sizes.ctypes.data, self.nlimbs, n, stream_ptr()))
        return limbs[:self.nlimbs], sizes

    def to_ints(self):
        limbs, sizes = self.download()
        return planes_to_ints(limbs, sizes)


class Handle:
    def __init__(self):
        _torch()
        h = ctypes.c_void_p()
        check(lib().gbmm_create(ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().gbmm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind_stream(self):
        check(lib().gbmm_set_stream(self.h, stream_ptr()))

    def matmul(self, C, A, B, path=PATH_AUTO, method=METHOD_WINOGRAD, cutoff=0, nprimes=0, accumulate=False, plan=None):
        """C = A*B (C += A*B with accumulate); `plan` (a PLAN_* id) runs that plan and
        overrides path / method / cutoff."""
        self.bind_stream()
        o = Opts(path, method, cutoff, nprimes, int(bool(accumulate)), 0 if plan is None else 1 + plan)
        check(lib().gbmm_matmul(self.h, _m(C), _m(A), _m(B), ctypes.byref(o)))

    @staticmethod
    def jobs(triples, path=PATH_AUTO):
        """[(C, A, B), ...] -> ctypes array of gbmm_job."""
        arr = (Job * len(triples))()
        for i, (c, a, b) in enumerate(triples):
            arr[i].c, arr[i].a, arr[i].b = _m(c), _m(a), _m(b)
            arr[i].path = path
        return arr

    def matmul_batched(self, jobs, path=PATH_AUTO, plans=False):
        """Runs a ctypes array of gbmm_job; returns the paths the dispatcher chose
        (with plans=True: (path, gbmm_plan) pairs)."""
        self.bind_stream()
        o = Opts(path, METHOD_WINOGRAD, 0, 0, 0, 0)
        check(lib().gbmm_matmul_batched(self.h, jobs, len(jobs), ctypes.byref(o)))
        if plans:
            return [(jobs[i].chosen_path, jobs[i].chosen_plan) for i in range(len(jobs))]
        return [jobs[i].chosen_path for i in range(len(jobs))]

    @staticmethod
    def host_jobs(specs, path=PATH_AUTO, method=0, cutoff=0):
        """[(K, M, N, (Al, As), (Bl, Bs), (Cl, Cs)), ...] with numpy planes (limbs
        [nlimbs, rows*cols] uint32, sizes [rows*cols] int32; C's are filled in) ->
        ctypes array of gbmm_host_job.  The arrays must stay alive during the call."""
        arr = (HostJob * len(specs))()
        for i, (K, M, N, (Al, As), (Bl, Bs), (Cl, Cs)) in enumerate(specs):
            for a in (Al, As, Bl, Bs, Cl, Cs):
                if not a.flags["C_CONTIGUOUS"]:
                    raise ValueError("host planes must be contiguous")
            q = arr[i]
            q.K, q.M, q.N = K, M, N
            q.a_nlimbs, q.b_nlimbs, q.c_nlimbs = Al.shape[0], Bl.shape[0], Cl.shape[0]
            q.a_limbs, q.a_sizes = Al.ctypes.data, As.ctypes.data
            q.b_limbs, q.b_sizes = Bl.ctypes.data, Bs.ctypes.data
            q.c_limbs, q.c_sizes = Cl.ctypes.data, Cs.ctypes.data
            q.path, q.method, q.cutoff = path, method, cutoff
        return arr

    def set_device_budget(self, nbytes):
        """Device bytes a host-buffer product may use before it runs out of core (0: free memory)."""
        check(lib().gbmm_set_device_budget(self.h, int(nbytes)))

    def matmul_host(self, jobs):
        """Runs a ctypes array of gbmm_host_job (pipelined host <-> device copies);
        returns the paths the dispatcher chose."""
        self.bind_stream()
        check(lib().gbmm_matmul_host(self.h, jobs, len(jobs)))
        return [jobs[i].chosen_path for i in range(len(jobs))]

    # ---- learned cost model ----
    def model_init(self, seed=1):
        check(lib().gbmm_model_init(self.h, seed))

    def model_params(self):
        n = lib().gbmm_model_nparams()
        m = np.zeros(n, dtype=np.float32)
        b = np.zeros(n, dtype=np.uint16)
        check(lib().gbmm_model_get_params(self.h, m.ctypes.data, b.ctypes.data))
        return m, b

    def model_set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        check(lib().gbmm_model_set_params(self.h, p.ctypes.data))

    def model_predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], NPLANS), dtype=np.float32)
        self.bind_stream()
        check(lib().gbmm_model_predict(self.h, X.ctypes.data, X.shape[0], Y.ctypes.data))
        return Y

    def model_gradient(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(lib().gbmm_model_nparams(), dtype=np.float32)
        loss = ctypes.c_float(0)
        self.bind_stream()
        check(lib().gbmm_model_gradient(self.h, X.ctypes.data, T.ctypes.data, X.shape[0], g.ctypes.data,
                                        ctypes.byref(loss)))
        return g, loss.value

    def model_train(self, X, T, epochs=300, lr=3e-3):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = ctypes.c_float(0)
        self.bind_stream()
        check(lib().gbmm_model_train(self.h, X.ctypes.data, T.ctypes.data, X.shape[0], epochs, lr,
                                     ctypes.byref(loss)))
        return loss.value

    def model_use(self, enable=True):
        check(lib().gbmm_model_use(self.h, int(bool(enable))))

    def set_graphs(self, enable):
        check(lib().gbmm_set_graphs(self.h, int(bool(enable))))

    def set_breadth_first(self, enable):
        """Winograd products as one breadth-first tree (default) or depth first;
        returns the previous setting (internal switch, for tests and benchmarks)."""
        f = lib().gbmmx_wino_breadth_first
        f.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        f.restype = ctypes.c_int32
        return bool(f(self.h, int(bool(enable))))

    def autotune(self, jobs, repeats=2, log_path=None):
        self.bind_stream()
        check(lib().gbmm_autotune(self.h, jobs, len(jobs), repeats, log_path.encode() if log_path else None))


def _m(x):
    return x.mat if isinstance(x, DeviceMatrix) else x


def model_features(m, k, n, la, lb):
    f = np.zeros(8, dtype=np.float32)
    check(lib().gbmm_model_features(m, k, n, la, lb, f.ctypes.data))
    return f


def limbs_needed(a_nlimbs, b_nlimbs, inner, path=PATH_LIMB, method=METHOD_WINOGRAD, cutoff=0):
    o = Opts(path, method, cutoff, 0, 0, 0)
    out = ctypes.c_int32(0)
    check(lib().gbmm_matmul_limbs_needed(a_nlimbs, b_nlimbs, inner, ctypes.byref(o), ctypes.byref(out)))
    return out.value


# ----------------------------------------------------------------------------------
# reference-shaped operator surface
# ----------------------------------------------------------------------------------
_handle = None


def default_handle():
    global _handle
    if _handle is None:
        _handle = Handle()
    return _handle


def mat_mul(K, M, N, C, A, B, method=METHOD_NAIVE, path=PATH_LIMB, cutoff=0):
    """C = A * B (mat-cpu/mat.c:72-82); C is K x N, A K x M, B M x N (DeviceMatrix)."""
    assert A.rows == K and A.cols == M and B.rows == M and B.cols == N and C.rows == K and C.cols == N
    default_handle().matmul(C, A, B, path=path, method=method, cutoff=cutoff)


def mat_addmul(K, M, N, C, A, B, method=METHOD_NAIVE, path=PATH_LIMB, cutoff=0):
    """C += A * B (mat-cpu/mat.c:84-93)."""
    default_handle().matmul(C, A, B, path=path, method=method, cutoff=cutoff, accumulate=True)


def mat_mul_winograd(N, C, A, B, cutoff=32):
    default_handle().matmul(C, A, B, path=PATH_LIMB, method=METHOD_WINOGRAD, cutoff=cutoff)


def mat_mul_strassen(N, C, A, B, cutoff=32):
    default_handle().matmul(C, A, B, path=PATH_LIMB, method=METHOD_STRASSEN, cutoff=cutoff)


def squarify_mul(K, M, N, C, A, B, method=METHOD_WINOGRAD, cutoff=0, path=PATH_LIMB):
    """squarify_mul_pregpu (mat-gpu/mat-pregpu.cu:548-576) with a square method."""
    default_handle().matmul(C, A, B, path=path, method=method, cutoff=cutoff)


def mat_add(C, A, B):
    check(lib().gbmm_mat_add(_m(C), _m(A), _m(B), stream_ptr()))


def mat_sub(C, A, B):
    check(lib().gbmm_mat_sub(_m(C), _m(A), _m(B), stream_ptr()))


def mpz_add(w, u, v):
    check(lib().gbmm_mpz_add(_m(w), _m(u), _m(v), stream_ptr()))


def mpz_sub(w, u, v):
    check(lib().gbmm_mpz_sub(_m(w), _m(u), _m(v), stream_ptr()))


def mpz_mul(w, u, v):
    check(lib().gbmm_mpz_mul(_m(w), _m(u), _m(v), stream_ptr()))


def mpz_addmul(w, u, v):
    check(lib().gbmm_mpz_addmul(_m(w), _m(u), _m(v), stream_ptr()))


def mpz_submul(w, u, v):
    check(lib().gbmm_mpz_submul(_m(w), _m(u), _m(v), stream_ptr()))


def _dp(t):
    return t.data_ptr()


def mpn_add_n(rp, up, vp, n, ld, nb, cy):
    """Batched mpn_add_n over torch int32 device tensors (planes of stride ld)."""
    check(lib().gbmm_mpn_add_n(_dp(rp), _dp(up), _dp(vp), n, ld, nb, _dp(cy), stream_ptr()))


def mpn_sub_n(rp, up, vp, n, ld, nb, cy):
    check(lib().gbmm_mpn_sub_n(_dp(rp), _dp(up), _dp(vp), n, ld, nb, _dp(cy), stream_ptr()))


def mpn_add(rp, up, un, vp, vn, ld, nb, cy):
    check(lib().gbmm_mpn_add(_dp(rp), _dp(up), un, _dp(vp), vn, ld, nb, _dp(cy), stream_ptr()))


def mpn_sub(rp, up, un, vp, vn, ld, nb, cy):
    check(lib().gbmm_mpn_sub(_dp(rp), _dp(up), un, _dp(vp), vn, ld, nb, _dp(cy), stream_ptr()))


def mpn_add_1(rp, up, n, vl, ld, nb, cy):
    check(lib().gbmm_mpn_add_1(_dp(rp), _dp(up), n, _dp(vl), ld, nb, _dp(cy), stream_ptr()))


def mpn_sub_1(rp, up, n, vl, ld, nb, cy):
    check(lib().gbmm_mpn_sub_1(_dp(rp), _dp(up), n, _dp(vl), ld, nb, _dp(cy), stream_ptr()))


def mpn_cmp(up, vp, n, ld, nb, result):
    check(lib().gbmm_mpn_cmp(_dp(up), _dp(vp), n, ld, nb, _dp(result), stream_ptr()))


def mpn_zero_p(up, n, ld, nb, result):
    check(lib().gbmm_mpn_zero_p(_dp(up), n, ld, nb, _dp(result), stream_ptr()))


def mpn_neg(rp, up, n, ld, nb, cy):
    check(lib().gbmm_mpn_neg(_dp(rp), _dp(up), n, ld, nb, _dp(cy), stream_ptr()))


def mpn_com(rp, up, n, ld, nb):
    check(lib().gbmm_mpn_com(_dp(rp), _dp(up), n, ld, nb, stream_ptr()))


def mpn_mul_1(rp, up, n, vl, ld, nb, cy):
    check(lib().gbmm_mpn_mul_1(_dp(rp), _dp(up), n, _dp(vl), ld, nb, _dp(cy), stream_ptr()))


def mpn_addmul_1(rp, up, n, vl, ld, nb, cy):
    check(lib().gbmm_mpn_addmul_1(_dp(rp), _dp(up), n, _dp(vl), ld, nb, _dp(cy), stream_ptr()))


def mpn_submul_1(rp, up, n, vl, ld, nb, cy):
    check(lib().gbmm_mpn_submul_1(_dp(rp), _dp(up), n, _dp(vl), ld, nb, _dp(cy), stream_ptr()))


def mpn_mul_basecase(rp, up, un, vp, vn, ld, nb):
    check(lib().gbmm_mpn_mul_basecase(_dp(rp), _dp(up), un, _dp(vp), vn, ld, nb, stream_ptr()))


def mpn_toom22_mul_itch(an, bn):
    return lib().gbmm_mpn_toom22_mul_itch(an, bn)


def mpn_toom22_mul(pp, ap, an, bp, bn, scratch, ld, nb):
    check(lib().gbmm_mpn_toom22_mul(_dp(pp), _dp(ap), an, _dp(bp), bn, _dp(scratch), ld, nb, stream_ptr()))


def mpn_mul(rp, up, un, vp, vn, ld, nb):
    h = default_handle()
    h.bind_stream()
    check(lib().gbmm_mpn_mul(h.h, _dp(rp), _dp(up), un, _dp(vp), vn, ld, nb))
