"""Generates the golden fixtures in this folder.

For every case a seeded input in mat-cpu's -i format is drawn with Python's
`random` (distributions follow the benchmark configurations: uniform signed
magnitudes of a given bit length, optional exact zeros and short entries),
the product is computed by the reference's own mat-cpu (built from its sources
by `make -C oracle ref`, method -m 1 = naive GMP triple loop, cross-checked
with -m 35 Winograd), and independently by Python integers; the fixture is
written only if all agree.  Output: <case>.in.gz and <case>.out.gz.

Run with GBMM_REFERENCE_DIR naming a checkout of the reference (make -C oracle
ref reads its mat-cpu sources from there):
    GBMM_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py
"""
import gzip
import os
import random
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
REF = os.path.join(ROOT, "oracle", "_ref", "mat-cpu")

# name: (K, M, N, bits, zero_frac, short_frac, short_bits, special)
CASES = {
    "tiny_1x1x1": (1, 1, 1, 70, 0.0, 0.0, 0, None),
    "vec_1x5x1": (1, 5, 1, 130, 0.0, 0.0, 0, None),
    "rect_3x1x4": (3, 1, 4, 33, 0.0, 0.0, 0, None),
    "rect_7x13x5_zeros": (7, 13, 5, 100, 0.2, 0.0, 0, None),
    "cfg1_like_16x16x16_1024b": (16, 16, 16, 1024, 0.0, 0.0, 0, None),
    "cfg2_like_16x16x16_2048b": (16, 16, 16, 2048, 0.05, 0.05, 64, None),
    "cfg3_like_8x8x8_4096b": (8, 8, 8, 4096, 0.0, 0.0, 0, None),
    "allones_8x8x8_256b": (8, 8, 8, 256, 0.0, 0.0, 0, "allones"),
    "square_64x64x64_64b": (64, 64, 64, 64, 0.1, 0.0, 0, None),
    "rect_40x33x70_300b": (40, 33, 70, 300, 0.05, 0.1, 40, None),
    "zero_matrix_4x4x4": (4, 4, 4, 100, 1.0, 0.0, 0, None),
    "cancel_6x6x6_200b": (6, 6, 6, 200, 0.0, 0.0, 0, "cancel"),
}


def hexs(v):
    return format(v, "x") if v >= 0 else "-" + format(-v, "x")


def draw(rng, n, bits, zf, sf, sbits, special):
    out = []
    for i in range(n):
        if special == "allones":
            m = (1 << bits) - 1
        elif rng.random() < zf:
            m = 0
        elif rng.random() < sf:
            m = rng.getrandbits(sbits)
        else:
            m = rng.getrandbits(bits)
        out.append(-m if rng.random() < 0.5 else m)
    return out


def make(name, spec, seed):
    K, M, N, bits, zf, sf, sbits, special = spec
    rng = random.Random(seed)
    A = draw(rng, K * M, bits, zf, sf, sbits, special)
    B = draw(rng, M * N, bits, zf, sf, sbits, special)
    if special == "cancel":
        # row 0 of A times B cancels: A[0] = [x, -x, ...] against equal rows of B
        for k in range(1, M, 2):
            A[k] = -A[k - 1]
            for x in range(N):
                B[k * N + x] = B[(k - 1) * N + x]
    text = f"{K} {M} {N}\n"
    for r in range(K):
        text += " ".join(hexs(v) for v in A[r * M:(r + 1) * M]) + "\n"
    text += "\n"
    for r in range(M):
        text += " ".join(hexs(v) for v in B[r * N:(r + 1) * N]) + "\n"
    text += "\n"
    C = [sum(A[y * M + k] * B[k * N + x] for k in range(M)) for y in range(K) for x in range(N)]
    expect = "".join(" ".join(hexs(v) for v in C[y * N:(y + 1) * N]) + "\n" for y in range(K)) + "\n"
    for m in ("1", "35", "31"):
        out = subprocess.run([REF, "-i", "-p", "-m", m], input=text.encode(), stdout=subprocess.PIPE,
                             stderr=subprocess.DEVNULL, check=True).stdout.decode()
        if out != expect:
            raise SystemExit(f"{name}: mat-cpu -m {m} disagrees with Python integers")
    with gzip.open(os.path.join(HERE, name + ".in.gz"), "wt") as f:
        f.write(text)
    with gzip.open(os.path.join(HERE, name + ".out.gz"), "wt") as f:
        f.write(expect)


def main():
    if not os.path.exists(REF):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    for i, (name, spec) in enumerate(sorted(CASES.items())):
        make(name, spec, 1000 + i)
        print("wrote", name)


if __name__ == "__main__":
    sys.exit(main())
