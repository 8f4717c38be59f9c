// gbmm-cli: command-line front end with mat-gpu's flags (mat-gpu/main.cu:235-289)
// and matrix text format (mat-cpu/main.c:249-276, mat.c:336-353).
//
//   -h          help
//   -i          read "K M N", A (K x M) and B (M x N) in hex from stdin
//   -g          generate two random matrices and print them (-n, -b, -s)
//   -n K,M,N    sizes for random matrices (KxM * MxN = KxN)
//   -b nbits    bit length of random entries (uniform magnitude, fair sign)
//   -s seed     random seed (default 1)
//   -m method   1/2 naive per-entry kernel, 3 Strassen, 35/357 Winograd,
//               4/47 block recursion, 8 CRT tensor-core path, 0 automatic
//   -B cutoff   recursion cutoff (blocks of at most this size go to the kernel)
//   -P nprimes  CRT: number of moduli (0 = from the bit bound)
//   -p          print the product (mat_write format) to stdout
// Timing goes to stderr as "Time taken: <s> seconds" like mat-gpu.
#include <cuda_runtime.h>
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <string>
#include <vector>

#include "../../include/gbmm.h"

static uint64_t g_rs = 88172645463325252ull;
static uint64_t xr() {
    g_rs ^= g_rs << 13;
    g_rs ^= g_rs >> 7;
    g_rs ^= g_rs << 17;
    return g_rs;
}

// Same stream as the oracle's generator: per entry ceil(nbits/64) words, top
// word masked, then one word whose low bit chooses the sign.
static void gen_entry(int nbits, uint32_t *limbs, int32_t *size, int nl, int64_t ld, int64_t e) {
    int n64 = (nbits + 63) / 64;
    std::vector<uint64_t> d(n64 ? n64 : 1, 0);
    for (int i = 0; i < n64; i++) d[i] = xr();
    if (nbits % 64) d[n64 - 1] &= (1ull << (nbits % 64)) - 1;
    int n = 0;
    for (int i = 0; i < nl; i++) {
        uint32_t v = i / 2 < n64 ? (uint32_t)(d[i / 2] >> (32 * (i % 2))) : 0u;
        limbs[(int64_t)i * ld + e] = v;
        if (v) n = i + 1;
    }
    *size = (xr() & 1) ? -n : n;
}

static void die(const char *what) {
    fprintf(stderr, "%s: %s\n", what, gbmm_last_error_string());
    exit(1);
}

static double now() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char **argv) {
    bool read_input = false, print = false, generate = false;
    int K = -1, M = -1, N = -1, nbits = -1, method = 35, cutoff = 0, nprimes = 0;
    unsigned long seed = 1;
    int opt;
    while ((opt = getopt(argc, argv, "higpn:b:m:s:B:P:")) != -1) {
        switch (opt) {
            case 'h':
                fprintf(stderr,
                        "Usage: %s [-higp] [-n K,M,N] [-b nbits] [-s seed] [-m method] [-B cutoff] [-P nprimes]\n"
                        "  -i  read matrices from stdin    -g  print two random matrices\n"
                        "  -m  1|2 naive, 3 Strassen, 35|357 Winograd, 4|47 block recursion, 8 CRT, 0 auto\n",
                        argv[0]);
                return 0;
            case 'i': read_input = true; break;
            case 'g': generate = true; break;
            case 'p': print = true; break;
            case 'n':
                if (sscanf(optarg, "%d,%d,%d", &K, &M, &N) != 3) { fprintf(stderr, "Invalid -n\n"); return 1; }
                break;
            case 'b': nbits = atoi(optarg); break;
            case 'm': method = atoi(optarg); break;
            case 's': seed = strtoul(optarg, nullptr, 10); break;
            case 'B': cutoff = atoi(optarg); break;
            case 'P': nprimes = atoi(optarg); break;
            default: fprintf(stderr, "Unknown flag, use -h to get info\n"); return 1;
        }
    }
    g_rs ^= seed * 0x9E3779B97F4A7C15ull;
    if (!g_rs) g_rs = 1;

    std::vector<uint32_t> hA, hB;
    std::vector<int32_t> sA, sB;
    int nlA = 1, nlB = 1;
    if (read_input) {
        if (K != -1 || nbits != -1) { fprintf(stderr, "Cannot specify -n or -b with -i\n"); return 1; }
        std::string text;
        char buf[1 << 16];
        size_t r;
        while ((r = fread(buf, 1, sizeof buf, stdin)) > 0) text.append(buf, r);
        size_t pos = 0;
        if (sscanf(text.c_str(), "%d %d %d", &K, &M, &N) != 3) { fprintf(stderr, "bad header\n"); return 1; }
        int lines = 0;
        while (pos < text.size() && lines < 1) if (text[pos++] == '\n') lines++;
        // capacity: longest token decides
        size_t longest = 1, cur = 0;
        for (size_t i = pos; i < text.size(); i++) {
            char c = text[i];
            if (c == ' ' || c == '\n' || c == '\t' || c == '\r') { longest = cur > longest ? cur : longest; cur = 0; }
            else cur++;
        }
        longest = cur > longest ? cur : longest;
        nlA = nlB = (int)((longest + 7) / 8);
        hA.assign((size_t)nlA * K * M, 0); sA.assign((size_t)K * M, 0);
        hB.assign((size_t)nlB * M * N, 0); sB.assign((size_t)M * N, 0);
        size_t used = 0;
        if (gbmm_parse_hex(text.data() + pos, text.size() - pos, (int64_t)K * M, hA.data(), sA.data(), nlA, (int64_t)K * M,
                           &used) != GBMM_OK)
            die("parse A");
        pos += used;
        if (gbmm_parse_hex(text.data() + pos, text.size() - pos, (int64_t)M * N, hB.data(), sB.data(), nlB, (int64_t)M * N,
                           &used) != GBMM_OK)
            die("parse B");
    } else {
        if (K < 0) { fprintf(stderr, "No matrix size specified!\n"); return 1; }
        if (nbits < 0) { fprintf(stderr, "No bit count specified!\n"); return 1; }
        nlA = nlB = (nbits + 31) / 32 > 0 ? (nbits + 31) / 32 : 1;
        hA.assign((size_t)nlA * K * M, 0); sA.assign((size_t)K * M, 0);
        hB.assign((size_t)nlB * M * N, 0); sB.assign((size_t)M * N, 0);
        for (int64_t e = 0; e < (int64_t)K * M; e++) gen_entry(nbits, hA.data(), &sA[e], nlA, (int64_t)K * M, e);
        for (int64_t e = 0; e < (int64_t)M * N; e++) gen_entry(nbits, hB.data(), &sB[e], nlB, (int64_t)M * N, e);
        if (generate) {
            printf("%d %d %d\n", K, M, N);
            size_t w = 0;
            gbmm_format_hex(hA.data(), sA.data(), nlA, (int64_t)K * M, K, M, M, nullptr, 0, &w);
            std::string out(w + 1, '\0');
            gbmm_format_hex(hA.data(), sA.data(), nlA, (int64_t)K * M, K, M, M, &out[0], w + 1, &w);
            fwrite(out.data(), 1, w, stdout);
            gbmm_format_hex(hB.data(), sB.data(), nlB, (int64_t)M * N, M, N, N, nullptr, 0, &w);
            out.assign(w + 1, '\0');
            gbmm_format_hex(hB.data(), sB.data(), nlB, (int64_t)M * N, M, N, N, &out[0], w + 1, &w);
            fwrite(out.data(), 1, w, stdout);
            return 0;
        }
    }
    if (cudaSetDevice(0) != cudaSuccess) { fprintf(stderr, "no CUDA device\n"); return 1; }
    gbmm_handle h;
    if (gbmm_create(&h) != GBMM_OK) die("create");
    gbmm_opts o;
    memset(&o, 0, sizeof o);
    o.cutoff = cutoff;
    o.nprimes = nprimes;
    switch (method) {
        case 0: o.path = GBMM_PATH_AUTO; o.method = GBMM_METHOD_WINOGRAD; break;
        case 1: case 2: o.path = GBMM_PATH_LIMB; o.method = GBMM_METHOD_NAIVE; break;
        case 3: case 37: o.path = GBMM_PATH_LIMB; o.method = GBMM_METHOD_STRASSEN; break;
        case 35: case 357: o.path = GBMM_PATH_LIMB; o.method = GBMM_METHOD_WINOGRAD; break;
        case 4: case 47: o.path = GBMM_PATH_LIMB; o.method = GBMM_METHOD_NAIVE_REC; break;
        case 8: o.path = GBMM_PATH_CRT; break;
        default: fprintf(stderr, "Invalid method %d!\n", method); return 1;
    }
    fprintf(stderr, "Using method %d\n", method);
    int32_t nlC = 0;
    gbmm_matmul_limbs_needed(nlA, nlB, M, &o, &nlC);
    auto dev_mat = [](int rows, int cols, int nl) {
        gbmm_mat m;
        memset(&m, 0, sizeof m);
        m.rows = rows; m.cols = cols; m.nlimbs = nl; m.rs = cols; m.ld = (int64_t)rows * cols;
        size_t n = (size_t)rows * cols;
        if (cudaMalloc(&m.limbs, n * (nl ? nl : 1) * 4 + 16) != cudaSuccess || cudaMalloc(&m.sizes, n * 4 + 16) != cudaSuccess) {
            fprintf(stderr, "cudaMalloc failed\n");
            exit(1);
        }
        return m;
    };
    gbmm_mat dA = dev_mat(K, M, nlA), dB = dev_mat(M, N, nlB), dC = dev_mat(K, N, nlC);
    if (gbmm_upload(dA, hA.data(), sA.data(), nlA, (int64_t)K * M, nullptr) != GBMM_OK) die("upload A");
    if (gbmm_upload(dB, hB.data(), sB.data(), nlB, (int64_t)M * N, nullptr) != GBMM_OK) die("upload B");
    double t0 = now();
    if (gbmm_matmul(h, dC, dA, dB, &o) != GBMM_OK) die("matmul");
    cudaDeviceSynchronize();
    fprintf(stderr, "Time taken: %g seconds\n", now() - t0);
    if (print) {
        std::vector<uint32_t> hC((size_t)nlC * K * N);
        std::vector<int32_t> sC((size_t)K * N);
        if (gbmm_download(dC, hC.data(), sC.data(), nlC, (int64_t)K * N, nullptr) != GBMM_OK) die("download");
        size_t w = 0;
        gbmm_format_hex(hC.data(), sC.data(), nlC, (int64_t)K * N, K, N, N, nullptr, 0, &w);
        std::string out(w + 1, '\0');
        gbmm_format_hex(hC.data(), sC.data(), nlC, (int64_t)K * N, K, N, N, &out[0], w + 1, &w);
        fwrite(out.data(), 1, w, stdout);
    }
    cudaFree(dA.limbs); cudaFree(dA.sizes); cudaFree(dB.limbs); cudaFree(dB.sizes); cudaFree(dC.limbs); cudaFree(dC.sizes);
    gbmm_destroy(h);
    return 0;
}
