"""Builds gbmm's native library (libgbmm.so) and its command-line front end.

Every CUDA translation unit is compiled for sm_103a only, in parallel, with
nvcc; the objects are linked into ``_build/libgbmm.so`` next to this file.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgbmm.so")
CLI = os.path.join(OUT, "gbmm-cli")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "--expt-relaxed-constexpr", "-I" + os.path.join(HERE, "..", "include")]

LIB_SOURCES = ["host.cpp", "limb.cu", "crt.cu", "batch.cpp", "mlp.cu", "pipeline.cpp"]
CLI_SOURCES = ["cli.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return p.returncode, p.stdout


def build(verbose=False, force=False, extra_flags=()):
    """Compiles the library; returns the path of libgbmm.so.  Raises on failure."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(HERE, "..", "include", "gbmm.h"))
    jobs = []
    objs = []
    for src in LIB_SOURCES + CLI_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [path] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append([nvcc] + NVCC_FLAGS + list(extra_flags) + lang + ["-c", path, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(_run, jobs))
    for cmd, (rc, out) in zip(jobs, results):
        if verbose or rc != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + out)
        if rc != 0:
            raise RuntimeError("nvcc failed for " + cmd[-3])
    lib_objs = [os.path.join(OUT, s + ".o") for s in LIB_SOURCES]
    if force or jobs or not os.path.exists(LIB):
        rc, out = _run([nvcc] + ARCH + ["-shared", "-o", LIB] + lib_objs + ["-lpthread"])
        if rc != 0:
            sys.stderr.write(out)
            raise RuntimeError("link of libgbmm.so failed")
    cli_obj = os.path.join(OUT, "cli.cpp.o")
    if os.path.exists(cli_obj) and (force or jobs or not os.path.exists(CLI)):
        rc, out = _run([nvcc] + ARCH + ["-o", CLI, cli_obj] + lib_objs + ["-lpthread"])
        if rc != 0:
            sys.stderr.write(out)
            raise RuntimeError("link of gbmm-cli failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
