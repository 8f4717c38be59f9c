// Batched limb kernels: the plain (non-CRT) form of gbmm.
//
// Numbers are sign-magnitude with 32-bit limbs in limb planes (structure of
// arrays): limb i of operand b lives at p[i*ld + b], so neighbouring threads
// touch neighbouring words.  This is the layout of the reference's interleaved
// mode (mat-gpu/gmp-es-mpz.h:38-42) without the fixed capacity.
//
// Contents
//   - warp carry-lookahead add_n / sub_n        (GMP mpn_add_n / mpn_sub_n)
//   - mul_1 / addmul_1 / submul_1                 (GMP mpn_mul_1 family)
//   - mul_basecase (column / product scanning)   (GMP mpn_mul_basecase)
//   - toom22 (one Karatsuba split)               (GMP mpn_toom22_mul)
//   - mpz add / sub / mul / addmul / submul       (GMP mpz semantics)
//   - elementwise matrix add / sub                (mat-gpu add/sub_matrices_gpu)
//   - the per-entry matrix product kernel         (mat-gpu launcher_mul/addmul)
// All arithmetic algorithms are the textbook ones (Knuth TAOCP vol. 2 §4.3.1,
// §4.3.3); the code is written for GB300, not translated from the reference.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "gbmm_internal.h"

namespace gbmm {

// ---- small device helpers ---------------------------------------------------------
__device__ __forceinline__ int iabs_d(int x) { return x < 0 ? -x : x; }

// 96-bit column accumulator (c0, c1, c2) += a * b.  One 32x32->64 wide multiply
// accumulating into c0, then the high word and the carry.
// The three instructions share the carry flag, so they stay in one asm block.
#define MAC96(c0, c1, c2, a, b)                                                   \
    asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\t"                                      \
        "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"                                     \
        "addc.u32 %2, %2, 0;"                                                     \
        : "+r"(c0), "+r"(c1), "+r"(c2)                                            \
        : "r"(a), "r"(b))

struct MatArgs {
    uint32_t *limbs;
    int32_t *sizes;
    int64_t rs, ld;
    int32_t rows, cols, nlimbs;
};
__host__ __device__ static inline MatArgs margs(const gbmm_mat &m) {
    MatArgs a;
    a.limbs = m.limbs; a.sizes = m.sizes; a.rs = m.rs; a.ld = m.ld;
    a.rows = m.rows; a.cols = m.cols; a.nlimbs = m.nlimbs;
    return a;
}

// ======================================================================================
// mpn add_n / sub_n with warp-level carry-lookahead.
//
// A CTA takes 32 operands.  A chunk of up to 32*Q limbs of those operands is
// staged in shared memory with coalesced loads (limb-major rows, operand
// columns).  Each warp then processes one operand at a time: lane l owns limbs
// [l*Q, l*Q+Q) of the chunk, adds them with carry-in 0, and publishes
// generate (carry out) and propagate (result all ones) bits with __ballot_sync.
// The lane carry-ins are the carries of the 32-bit addition (G|P) + G + cin,
// the classic carry-lookahead identity, so the whole chunk resolves in O(1)
// warp steps instead of a 32*Q-long ripple.
// ======================================================================================
namespace {
constexpr int CLA_Q = 4;                 // limbs per lane per chunk
constexpr int CLA_CHUNK = 32 * CLA_Q;    // limbs per chunk
constexpr int CLA_OPS = 32;              // operands per CTA
}

template <bool SUB>
__global__ void __launch_bounds__(256) k_mpn_addsub_n_cla(uint32_t *rp, const uint32_t *up, const uint32_t *vp,
                                                          int n, int64_t ld, int64_t nb, uint32_t *cy) {
    __shared__ uint32_t su[CLA_CHUNK][CLA_OPS + 1];
    __shared__ uint32_t sv[CLA_CHUNK][CLA_OPS + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t b0 = (int64_t)blockIdx.x * CLA_OPS;
    // carry state per operand handled by this warp (operands warp, warp+8, ...)
    uint32_t carry[CLA_OPS / 8];
#pragma unroll
    for (int j = 0; j < CLA_OPS / 8; j++) carry[j] = 0;

    for (int c0 = 0; c0 < n; c0 += CLA_CHUNK) {
        const int clen = min(CLA_CHUNK, n - c0);
        __syncthreads();
        for (int q = threadIdx.x; q < clen * CLA_OPS; q += blockDim.x) {
            int i = q / CLA_OPS, b = q % CLA_OPS;
            int64_t ob = b0 + b;
            uint32_t x = 0, y = 0;
            if (ob < nb) {
                x = up[(int64_t)(c0 + i) * ld + ob];
                y = vp[(int64_t)(c0 + i) * ld + ob];
            }
            su[i][b] = x;
            sv[i][b] = y;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < CLA_OPS / 8; j++) {
            const int b = warp + 8 * j;
            uint32_t r[CLA_Q];
            uint32_t g = 0, allsat = 1;
            // local add / sub with carry-in 0
            uint32_t c = 0;
#pragma unroll
            for (int t = 0; t < CLA_Q; t++) {
                int i = lane * CLA_Q + t;
                r[t] = 0u;
                if (i < clen) {  // the chain stops at the chunk end
                    uint32_t x = su[i][b], y = sv[i][b];
                    if (!SUB) {
                        uint64_t s = (uint64_t)x + y + c;
                        r[t] = (uint32_t)s; c = (uint32_t)(s >> 32);
                        allsat &= r[t] == 0xFFFFFFFFu;
                    } else {
                        uint64_t d = (uint64_t)x - y - c;
                        r[t] = (uint32_t)d; c = (uint32_t)(d >> 63);
                        allsat &= r[t] == 0u;
                    }
                }
            }
            g = c;
            // lanes entirely past the chunk end neither generate nor propagate
            if (lane * CLA_Q >= clen) { g = 0; allsat = 0; }
            const uint32_t G = __ballot_sync(0xFFFFFFFFu, g);
            const uint32_t P = __ballot_sync(0xFFFFFFFFu, allsat && !g);
            const uint64_t sum = (uint64_t)(G | P) + (uint64_t)G + (uint64_t)carry[j];
            const uint32_t cin_mask = (uint32_t)sum ^ P;  // carry into each lane (bit l)
            // carry out of the chunk: out of the last lane that holds limbs
            const int last_lane = (clen - 1) / CLA_Q;
            uint32_t cin = (cin_mask >> lane) & 1u;
            const uint32_t lane_out = g | (((P >> lane) & 1u) & cin);
            const uint32_t chunk_out = __shfl_sync(0xFFFFFFFFu, lane_out, last_lane);
#pragma unroll
            for (int t = 0; t < CLA_Q; t++) {
                if (!SUB) {
                    uint64_t s = (uint64_t)r[t] + cin;
                    r[t] = (uint32_t)s; cin = (uint32_t)(s >> 32);
                } else {
                    uint64_t d = (uint64_t)r[t] - cin;
                    r[t] = (uint32_t)d; cin = (uint32_t)(d >> 63);
                }
                int i = lane * CLA_Q + t;
                if (i < clen) su[i][b] = r[t];
            }
            carry[j] = chunk_out;
        }
        __syncthreads();
        for (int q = threadIdx.x; q < clen * CLA_OPS; q += blockDim.x) {
            int i = q / CLA_OPS, b = q % CLA_OPS;
            int64_t ob = b0 + b;
            if (ob < nb) rp[(int64_t)(c0 + i) * ld + ob] = su[i][b];
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < CLA_OPS / 8; j++) {
            int64_t ob = b0 + warp + 8 * j;
            if (ob < nb) cy[ob] = carry[j];
        }
    }
}

// ---- add_n / sub_n for large batches: one thread per operand, serial over limbs ------
// Limb i of neighbouring operands is adjacent, so every load and store of a warp is
// one coalesced 128-byte line; with enough operands to fill the GPU this streams at
// HBM speed, where the warp carry-lookahead above leaves lanes idle on short operands.
template <bool SUB>
__global__ void __launch_bounds__(256) k_mpn_addsub_n_serial(uint32_t *rp, const uint32_t *up, const uint32_t *vp,
                                                             int n, int64_t ld, int64_t nb, uint32_t *cy) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    uint32_t c = 0;
#pragma unroll 4
    for (int i = 0; i < n; i++) {
        const uint32_t x = up[(int64_t)i * ld + b], y = vp[(int64_t)i * ld + b];
        if (!SUB) {
            const uint64_t t = (uint64_t)x + y + c;
            rp[(int64_t)i * ld + b] = (uint32_t)t;
            c = (uint32_t)(t >> 32);
        } else {
            const uint64_t t = (uint64_t)x - y - c;
            rp[(int64_t)i * ld + b] = (uint32_t)t;
            c = (uint32_t)(t >> 63);
        }
    }
    cy[b] = c;
}
// batches with at least this many operands take the one-thread-per-operand kernel
constexpr int64_t ADDSUB_SERIAL_MIN_OPS = 16384;

// ---- mul_1 family: one thread per operand, serial over limbs (coalesced) -----------
template <int OP>  // 0 mul_1, 1 addmul_1, 2 submul_1
__global__ void k_mpn_mul1ops(uint32_t *rp, const uint32_t *up, int n, const uint32_t *vl, int64_t ld, int64_t nb,
                              uint32_t *cy) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const uint64_t v = vl[b];
    uint64_t c = 0;
    for (int i = 0; i < n; i++) {
        uint64_t p = (uint64_t)up[(int64_t)i * ld + b] * v + c;
        uint32_t lo = (uint32_t)p;
        c = p >> 32;
        if (OP == 0) {
            rp[(int64_t)i * ld + b] = lo;
        } else if (OP == 1) {
            uint64_t s = (uint64_t)rp[(int64_t)i * ld + b] + lo;
            rp[(int64_t)i * ld + b] = (uint32_t)s;
            c += s >> 32;
        } else {
            uint32_t r = rp[(int64_t)i * ld + b];
            rp[(int64_t)i * ld + b] = r - lo;
            c += (r < lo);
        }
    }
    cy[b] = (uint32_t)c;
}

// ---- the rest of the mpn layer: one thread per operand, serial over coalesced limbs -----
// Neighbouring threads take neighbouring operands, so every limb access of a warp
// is one 128-byte line.  GMP semantics (mat-gpu/addsub.cu:187-326, com.cu:35-42).

// rp = up +/- vp with un >= vn limbs (vp zero-extended to un); carry / borrow out
template <bool SUB>
__global__ void __launch_bounds__(256) k_mpn_addsub(uint32_t *rp, const uint32_t *up, int un, const uint32_t *vp,
                                                    int vn, int64_t ld, int64_t nb, uint32_t *cy) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    uint32_t c = 0;
    int i = 0;
#pragma unroll 4
    for (; i < vn; i++) {
        const uint32_t x = up[(int64_t)i * ld + b], y = vp[(int64_t)i * ld + b];
        const uint64_t t = SUB ? (uint64_t)x - y - c : (uint64_t)x + y + c;
        rp[(int64_t)i * ld + b] = (uint32_t)t;
        c = SUB ? (uint32_t)(t >> 63) : (uint32_t)(t >> 32);
    }
    for (; i < un; i++) {
        const uint32_t x = up[(int64_t)i * ld + b];
        const uint32_t r = SUB ? x - c : x + c;
        rp[(int64_t)i * ld + b] = r;
        c = SUB ? (uint32_t)(x < c) : (uint32_t)(r < c);
    }
    cy[b] = c;
}

// rp = up +/- vl[b] (a single limb per operand), n >= 1; carry / borrow out
template <bool SUB>
__global__ void __launch_bounds__(256) k_mpn_addsub_1(uint32_t *rp, const uint32_t *up, int n, const uint32_t *vl,
                                                      int64_t ld, int64_t nb, uint32_t *cy) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    uint32_t c = vl[b];
#pragma unroll 4
    for (int i = 0; i < n; i++) {
        const uint32_t x = up[(int64_t)i * ld + b];
        const uint32_t r = SUB ? x - c : x + c;
        rp[(int64_t)i * ld + b] = r;
        c = SUB ? (uint32_t)(x < c) : (uint32_t)(r < c);
    }
    cy[b] = c;
}

// res[b] = sign(up - vp) over n limbs, compared from the top
__global__ void __launch_bounds__(256) k_mpn_cmp(const uint32_t *up, const uint32_t *vp, int n, int64_t ld,
                                                 int64_t nb, int32_t *res) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    int r = 0;
    for (int i = n - 1; i >= 0; i--) {
        const uint32_t x = up[(int64_t)i * ld + b], y = vp[(int64_t)i * ld + b];
        if (x != y) {
            r = x > y ? 1 : -1;
            break;
        }
    }
    res[b] = r;
}

// res[b] = 1 when all n limbs of operand b are zero, else 0
__global__ void __launch_bounds__(256) k_mpn_zero_p(const uint32_t *up, int n, int64_t ld, int64_t nb, int32_t *res) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    uint32_t any = 0;
#pragma unroll 4
    for (int i = 0; i < n; i++) any |= up[(int64_t)i * ld + b];
    res[b] = any == 0;
}

// NEG: rp = -up mod B^n (~up + 1), cy[b] = 1 unless up is zero;  COM: rp = ~up
template <bool NEG>
__global__ void __launch_bounds__(256) k_mpn_neg_com(uint32_t *rp, const uint32_t *up, int n, int64_t ld, int64_t nb,
                                                     uint32_t *cy) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    uint32_t c = NEG ? 1u : 0u, any = 0;
#pragma unroll 4
    for (int i = 0; i < n; i++) {
        const uint32_t x = up[(int64_t)i * ld + b];
        const uint32_t r = ~x + c;
        c = NEG ? (uint32_t)(r < c) : 0u;
        any |= x;
        rp[(int64_t)i * ld + b] = r;
    }
    if (NEG) cy[b] = any != 0;
}

// ---- per-thread strided mpn helpers (operand stride `s`) ------------------------------
// r[0..un+vn) = u * v by product scanning: column t is summed in a 96-bit
// accumulator and written once.
__device__ void dev_mul_basecase(uint32_t *r, int64_t rs, const uint32_t *u, int un, int64_t us, const uint32_t *v,
                                 int vn, int64_t vs) {
    uint32_t c0 = 0, c1 = 0, c2 = 0;
    for (int t = 0; t < un + vn - 1; t++) {
        int i0 = t - vn + 1 > 0 ? t - vn + 1 : 0;
        int i1 = t < un - 1 ? t : un - 1;
        for (int i = i0; i <= i1; i++) {
            uint32_t a = u[(int64_t)i * us], b = v[(int64_t)(t - i) * vs];
            MAC96(c0, c1, c2, a, b);
        }
        r[(int64_t)t * rs] = c0;
        c0 = c1; c1 = c2; c2 = 0;
    }
    r[(int64_t)(un + vn - 1) * rs] = c0;
}
__device__ int dev_cmp(const uint32_t *a, int64_t as, const uint32_t *b, int64_t bs, int n) {
    for (int i = n - 1; i >= 0; i--) {
        uint32_t x = a[(int64_t)i * as], y = b[(int64_t)i * bs];
        if (x != y) return x < y ? -1 : 1;
    }
    return 0;
}
// r = a - b over n limbs (a >= b assumed by callers that care); returns borrow
__device__ uint32_t dev_sub_n(uint32_t *r, int64_t rs, const uint32_t *a, int64_t as, const uint32_t *b, int64_t bs,
                              int n) {
    uint32_t br = 0;
    for (int i = 0; i < n; i++) {
        uint64_t d = (uint64_t)a[(int64_t)i * as] - b[(int64_t)i * bs] - br;
        r[(int64_t)i * rs] = (uint32_t)d;
        br = (uint32_t)(d >> 63);
    }
    return br;
}
// r (rn limbs) += a (an <= rn limbs), carry propagated inside rn; returns carry out
__device__ uint32_t dev_add_into(uint32_t *r, int64_t rs, int rn, const uint32_t *a, int64_t as, int an) {
    uint32_t c = 0;
    int i = 0;
    for (; i < an; i++) {
        uint64_t s = (uint64_t)r[(int64_t)i * rs] + a[(int64_t)i * as] + c;
        r[(int64_t)i * rs] = (uint32_t)s;
        c = (uint32_t)(s >> 32);
    }
    for (; c && i < rn; i++) {
        uint32_t x = r[(int64_t)i * rs] + 1;
        r[(int64_t)i * rs] = x;
        c = x == 0;
    }
    return c;
}
__device__ uint32_t dev_sub_from(uint32_t *r, int64_t rs, int rn, const uint32_t *a, int64_t as, int an) {
    uint32_t br = 0;
    int i = 0;
    for (; i < an; i++) {
        uint64_t d = (uint64_t)r[(int64_t)i * rs] - a[(int64_t)i * as] - br;
        r[(int64_t)i * rs] = (uint32_t)d;
        br = (uint32_t)(d >> 63);
    }
    for (; br && i < rn; i++) {
        uint32_t x = r[(int64_t)i * rs];
        r[(int64_t)i * rs] = x - 1;
        br = x == 0;
    }
    return br;
}

__global__ void k_mpn_mul_basecase(uint32_t *rp, const uint32_t *up, int un, const uint32_t *vp, int vn, int64_t ld,
                                   int64_t nb) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    dev_mul_basecase(rp + b, ld, up + b, un, ld, vp + b, vn, ld);
}

// One Karatsuba split (Toom-2.2, Knuth 4.3.3): with a = a1 B^n + a0 and
// b = b1 B^n + b0,  a*b = v0 + (v0 + vinf - vm1) B^n + vinf B^2n  where
// v0 = a0 b0, vinf = a1 b1, vm1 = (a0 - a1)(b0 - b1).  Sub-products use the
// basecase.  Scratch per operand: 6n + 2 limbs (itch).
__global__ void k_mpn_toom22(uint32_t *pp, const uint32_t *ap, int an, const uint32_t *bp, int bn, uint32_t *scratch,
                             int64_t ld, int64_t nb) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int s = an >> 1, n = an - s, t = bn - n;
    const uint32_t *a = ap + b, *bb = bp + b;
    uint32_t *p = pp + b, *w = scratch + b;
    uint32_t *asm1 = w, *bsm1 = w + (int64_t)n * ld, *vm1 = w + (int64_t)2 * n * ld,
             *mid = w + (int64_t)4 * n * ld;
    // asm1 = |a0 - a1| (a1 has s limbs, zero-extended to n)
    int neg = 0;
    {
        int c = 0;
        // compare a0 (n limbs) with a1 (s limbs, top limb 0 if s < n)
        for (int i = n - 1; i >= 0 && c == 0; i--) {
            uint32_t x = a[(int64_t)i * ld], y = i < s ? a[(int64_t)(n + i) * ld] : 0u;
            if (x != y) c = x < y ? -1 : 1;
        }
        uint32_t br = 0;
        for (int i = 0; i < n; i++) {
            uint32_t x = a[(int64_t)i * ld], y = i < s ? a[(int64_t)(n + i) * ld] : 0u;
            if (c < 0) { uint32_t tt = x; x = y; y = tt; }
            uint64_t d = (uint64_t)x - y - br;
            asm1[(int64_t)i * ld] = (uint32_t)d;
            br = (uint32_t)(d >> 63);
        }
        neg ^= c < 0;
    }
    {
        int c = 0;
        for (int i = n - 1; i >= 0 && c == 0; i--) {
            uint32_t x = bb[(int64_t)i * ld], y = i < t ? bb[(int64_t)(n + i) * ld] : 0u;
            if (x != y) c = x < y ? -1 : 1;
        }
        uint32_t br = 0;
        for (int i = 0; i < n; i++) {
            uint32_t x = bb[(int64_t)i * ld], y = i < t ? bb[(int64_t)(n + i) * ld] : 0u;
            if (c < 0) { uint32_t tt = x; x = y; y = tt; }
            uint64_t d = (uint64_t)x - y - br;
            bsm1[(int64_t)i * ld] = (uint32_t)d;
            br = (uint32_t)(d >> 63);
        }
        neg ^= c < 0;
    }
    dev_mul_basecase(vm1, ld, asm1, n, ld, bsm1, n, ld);                 // 2n limbs
    dev_mul_basecase(p, ld, a, n, ld, bb, n, ld);                         // v0 -> p[0..2n)
    if (s >= t) dev_mul_basecase(p + (int64_t)2 * n * ld, ld, a + (int64_t)n * ld, s, ld, bb + (int64_t)n * ld, t, ld);
    else dev_mul_basecase(p + (int64_t)2 * n * ld, ld, bb + (int64_t)n * ld, t, ld, a + (int64_t)n * ld, s, ld);
    // mid = v0 + vinf -/+ vm1   (2n + 1 limbs, nonnegative: equals a0 b1 + a1 b0)
    for (int i = 0; i < 2 * n + 1; i++) mid[(int64_t)i * ld] = i < 2 * n ? p[(int64_t)i * ld] : 0u;
    dev_add_into(mid, ld, 2 * n + 1, p + (int64_t)2 * n * ld, ld, s + t);
    if (neg) dev_add_into(mid, ld, 2 * n + 1, vm1, ld, 2 * n);
    else dev_sub_from(mid, ld, 2 * n + 1, vm1, ld, 2 * n);
    dev_add_into(p + (int64_t)n * ld, ld, an + bn - n, mid, ld, 2 * n + 1 < an + bn - n ? 2 * n + 1 : an + bn - n);
}

// ---- on-chip forms of the batched products --------------------------------------------
// A CTA of NT threads takes NT operands of the batch (one product per thread).
// Their limbs are staged in shared memory once: 128-bit global loads read limb i
// of four neighbouring operands (limb planes are contiguous along the batch),
// a 4 x 4 register transpose turns four such loads into four limbs of each of
// four operands, and 128-bit shared stores put every operand's limbs
// contiguous, zero-padded to a multiple of 4.  Per-thread strings sit SS words
// apart with SS = 4 (mod 8), so the eight threads of a 128-bit access phase hit
// distinct banks.  Each product is then computed from shared memory in 4 x 4
// limb blocks: two 128-bit loads feed 16 MACs.

// per-thread stride (words) of a string of n limbs: a multiple of 4, = 4 (mod 8)
__host__ __device__ __forceinline__ int sm_stride(int n) {
    const int n4 = (n + 3) & ~3;
    return (n4 & 7) == 4 ? n4 : n4 + 4;
}

// Stages limbs [0, n) of operands b0 .. b0 + NT - 1 (limb i of operand b at
// g[i * ld + b]) into dst[t * SS + i], zero-filling limbs n .. roundup4(n) and
// operands past nb.  vec: g and ld allow 16-byte loads (g 16-byte aligned, ld % 4 == 0).
template <int NT>
__device__ __forceinline__ void sm_stage(uint32_t *dst, int SS, const uint32_t *g, int n, int64_t ld, int64_t b0,
                                         int64_t nb, bool vec) {
    const int n4 = (n + 3) >> 2;
    constexpr int NQ = NT / 4;  // groups of four operands
    for (int item = threadIdx.x; item < n4 * NQ; item += NT) {
        const int q = item % NQ, c = item / NQ;  // consecutive threads: neighbouring operand groups
        const int64_t bq = b0 + 4 * q;
        uint32_t L[4][4];  // L[k][j]: limb 4c + k of operand bq + j
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int i = 4 * c + k;
            const uint32_t *row = g + (int64_t)i * ld + bq;
            if (i < n && vec && bq + 3 < nb) {
                const uint4 w = *reinterpret_cast<const uint4 *>(row);
                L[k][0] = w.x; L[k][1] = w.y; L[k][2] = w.z; L[k][3] = w.w;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) L[k][j] = (i < n && bq + j < nb) ? row[j] : 0u;
            }
        }
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
            const int j = (jj + q) & 3;  // rotated: fewer bank conflicts among the stores
            *reinterpret_cast<uint4 *>(dst + (4 * q + j) * SS + 4 * c) = make_uint4(L[0][j], L[1][j], L[2][j], L[3][j]);
        }
    }
}

// The same staging with a map from destination limb d (the first of a chunk of
// four) to its source: planes g, first source limb i, limbs below lim valid, vec
// as above.  Destination limbs d .. d + 3 come from source limbs i .. i + 3.
template <int NT, class Map>
__device__ __forceinline__ void sm_stage_map(uint32_t *dst, int SS, int nchunks, int64_t b0, int64_t nb, int64_t ld,
                                             Map map) {
    constexpr int NQ = NT / 4;
    for (int item = threadIdx.x; item < nchunks * NQ; item += NT) {
        const int q = item % NQ, c = item / NQ;
        const int64_t bq = b0 + 4 * q;
        const uint32_t *g;
        int i0, lim;
        bool vec;
        map(4 * c, g, i0, lim, vec);
        uint32_t L[4][4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int i = i0 + k;
            const uint32_t *row = g + (int64_t)i * ld + bq;
            if (i < lim && vec && bq + 3 < nb) {
                const uint4 w = *reinterpret_cast<const uint4 *>(row);
                L[k][0] = w.x; L[k][1] = w.y; L[k][2] = w.z; L[k][3] = w.w;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) L[k][j] = (i < lim && bq + j < nb) ? row[j] : 0u;
            }
        }
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
            const int j = (jj + q) & 3;
            *reinterpret_cast<uint4 *>(dst + (4 * q + j) * SS + 4 * c) = make_uint4(L[0][j], L[1][j], L[2][j], L[3][j]);
        }
    }
}

// r = u * v for strings of nu4 and nv4 chunks of four limbs (16-byte aligned,
// zero-padded), by block product scanning: column block T gathers the 4 x 4
// blocks (I, T - I); their 7 columns are summed in 96-bit accumulators, the
// block's four columns absorb the carry from below and go out in ascending
// order (out(t, limb) for t < 4 (nu4 + nv4)), the upper three seed the next block.
template <class Out>
__device__ __forceinline__ void sm_mul4(const uint32_t *u, int nu4, const uint32_t *v, int nv4, Out out) {
    uint32_t acc[7][3];
#pragma unroll
    for (int c = 0; c < 7; c++) acc[c][0] = acc[c][1] = acc[c][2] = 0;
    uint32_t k0 = 0, k1 = 0;  // carry into the next column (64 bits)
    const int nT = nu4 + nv4;
    for (int T = 0; T < nT; T++) {
        const int i0 = T - nv4 + 1 > 0 ? T - nv4 + 1 : 0, i1 = T < nu4 - 1 ? T : nu4 - 1;
        for (int I = i0; I <= i1; I++) {
            const uint4 a = *reinterpret_cast<const uint4 *>(u + 4 * I);
            const uint4 b = *reinterpret_cast<const uint4 *>(v + 4 * (T - I));
            const uint32_t x[4] = {a.x, a.y, a.z, a.w}, y[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) MAC96(acc[i + j][0], acc[i + j][1], acc[i + j][2], x[i], y[j]);
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\taddc.u32 %2, %2, 0;"
                : "+r"(acc[c][0]), "+r"(acc[c][1]), "+r"(acc[c][2])
                : "r"(k0), "r"(k1));
            out(4 * T + c, acc[c][0]);
            k0 = acc[c][1];
            k1 = acc[c][2];
        }
#pragma unroll
        for (int c = 0; c < 7; c++) {
#pragma unroll
            for (int w = 0; w < 3; w++) acc[c][w] = c < 3 ? acc[c + 4][w] : 0u;
        }
    }
}

// Batched basecase product on chip: rp = up * vp (un >= vn), NT operands per CTA.
template <int NT>
__global__ void __launch_bounds__(NT) k_mpn_mul_basecase_sm(uint32_t *rp, const uint32_t *up, int un,
                                                            const uint32_t *vp, int vn, int64_t ld, int64_t nb,
                                                            int vec_u, int vec_v) {
    extern __shared__ uint4 sm_raw4[];
    uint32_t *sm = reinterpret_cast<uint32_t *>(sm_raw4);
    const int Su = sm_stride(un), Sv = sm_stride(vn);
    uint32_t *su = sm, *sv = sm + NT * Su;
    const int64_t b0 = (int64_t)blockIdx.x * NT;
    sm_stage<NT>(su, Su, up, un, ld, b0, nb, vec_u);
    sm_stage<NT>(sv, Sv, vp, vn, ld, b0, nb, vec_v);
    __syncthreads();
    const int64_t b = b0 + threadIdx.x;
    if (b >= nb) return;
    uint32_t *r = rp + b;
    const int rn = un + vn;
    sm_mul4(su + threadIdx.x * Su, (un + 3) >> 2, sv + threadIdx.x * Sv, (vn + 3) >> 2, [&](int t, uint32_t x) {
        if (t < rn) r[(int64_t)t * ld] = x;
    });
}

// Shared-memory words per thread of the on-chip Toom-2.2 for an x bn limbs: the
// halves a1 | a0 | b0 | b1, each zero-padded to n4 = roundup4(ceil(an / 2)).
__host__ __device__ __forceinline__ int toom22_sm_words(int an, int bn) {
    (void)bn;
    const int n = an - (an >> 1);
    return sm_stride(4 * ((n + 3) & ~3));
}

// One Karatsuba split (Knuth 4.3.3, as k_mpn_toom22) on chip.  Each thread's
// shared string holds the operand halves X = [a1 | a0 | b0 | b1] (n4 limbs
// each, staged straight from the limb planes).  v0 = a0 b0 and vinf = a1 b1 go
// to the product planes; then |a0 - a1| overwrites a1, |b0 - b1| overwrites b1,
// and vm1 = |a0 - a1| |b0 - b1| fills the dead a0 | b0 middle, which then turns
// into the middle term v0 + vinf -/+ vm1 (= a0 b1 + a1 b0) and is added into
// the product at limb n.  The product planes are read back once for that: the
// lines were just written by the same CTAs, so the reads hit L2 and HBM sees
// the operands once and the product once.
template <int NT>
__global__ void __launch_bounds__(NT) k_mpn_toom22_sm(uint32_t *pp, const uint32_t *ap, int an, const uint32_t *bp,
                                                      int bn, int64_t ld, int64_t nb, int vec_a, int vec_b) {
    extern __shared__ uint4 sm_raw4[];
    uint32_t *sm = reinterpret_cast<uint32_t *>(sm_raw4);
    const int s = an >> 1, n = an - s, t = bn - n;
    const int n4 = (n + 3) & ~3, c4 = n4 >> 2;
    const int SS = sm_stride(4 * n4);
    const int64_t b0 = (int64_t)blockIdx.x * NT;
    // destination chunk c of the four halves -> its source plane (operand, first limb, valid limbs)
    sm_stage_map<NT>(sm, SS, 4 * c4, b0, nb, ld, [&](int d, const uint32_t *&g, int &i, int &lim, bool &vec) {
        const int r = d / n4, off = d - r * n4;
        g = r < 2 ? ap : bp;
        vec = r < 2 ? vec_a : vec_b;
        i = (r == 1 || r == 2) ? off : n + off;
        lim = r == 0 ? n + s : r == 1 ? n : r == 2 ? n : n + t;
    });
    __syncthreads();
    const int64_t bi = b0 + threadIdx.x;
    if (bi >= nb) return;
    uint32_t *X = sm + threadIdx.x * SS;
    uint32_t *A1 = X, *A0 = X + n4, *B0 = X + 2 * n4, *B1 = X + 3 * n4;
    uint32_t *p = pp + bi;
    // v0 -> p[0, 2n), vinf -> p[2n, 2n + s + t)
    sm_mul4(A0, c4, B0, c4, [&](int i, uint32_t x) {
        if (i < 2 * n) p[(int64_t)i * ld] = x;
    });
    sm_mul4(A1, c4, B1, c4, [&](int i, uint32_t x) {
        if (i < s + t) p[(int64_t)(2 * n + i) * ld] = x;
    });
    // |a0 - a1| over a1, |b0 - b1| over b1; neg = the sign of (a0 - a1)(b0 - b1)
    int ca = 0, cb = 0;
    for (int i = n - 1; i >= 0 && ca == 0; i--)
        if (A0[i] != A1[i]) ca = A0[i] < A1[i] ? -1 : 1;
    for (int i = n - 1; i >= 0 && cb == 0; i--)
        if (B0[i] != B1[i]) cb = B0[i] < B1[i] ? -1 : 1;
    {
        uint32_t bra = 0, brb = 0;
        for (int i = 0; i < n4; i++) {
            const uint32_t xa = ca < 0 ? A1[i] : A0[i], ya = ca < 0 ? A0[i] : A1[i];
            const uint32_t xb = cb < 0 ? B1[i] : B0[i], yb = cb < 0 ? B0[i] : B1[i];
            const uint64_t da = (uint64_t)xa - ya - bra, db = (uint64_t)xb - yb - brb;
            A1[i] = (uint32_t)da;
            B1[i] = (uint32_t)db;
            bra = (uint32_t)(da >> 63);
            brb = (uint32_t)(db >> 63);
        }
    }
    const bool neg = (ca < 0) != (cb < 0);
    // vm1 -> V = X[n4, 3 n4): the a0 | b0 middle, no longer read
    uint32_t *V = A0;
    sm_mul4(A1, c4, B1, c4, [&](int i, uint32_t x) { V[i] = x; });
    // V = v0 + vinf -/+ vm1 over 2n + 1 limbs (V[2n] may lie in the dead |b0 - b1|).
    // The product planes are read eight limbs at a time, all eight loads issued
    // before the carry chain uses them (a store in between would order them).
    {
        long long c = 0;
        for (int i0 = 0; i0 < 2 * n + 1; i0 += 8) {
            uint32_t w0[8], wi[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int i = i0 + k;
                w0[k] = i < 2 * n ? p[(int64_t)i * ld] : 0u;
                wi[k] = i < s + t ? p[(int64_t)(2 * n + i) * ld] : 0u;
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int i = i0 + k;
                if (i >= 2 * n + 1) break;
                const long long wm = i < 2 * n ? V[i] : 0;
                const long long x = (long long)w0[k] + wi[k] + (neg ? wm : -wm) + c;
                V[i] = (uint32_t)x;
                c = x >> 32;
            }
        }
    }
    // p[n, an + bn) += V
    {
        uint32_t c = 0;
        const int pn = an + bn - n;
        for (int i0 = 0; i0 < pn; i0 += 8) {
            uint32_t w[8];
#pragma unroll
            for (int k = 0; k < 8; k++) w[k] = i0 + k < pn ? p[(int64_t)(n + i0 + k) * ld] : 0u;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int i = i0 + k;
                if (i >= pn) break;
                const uint64_t x = (uint64_t)w[k] + (i < 2 * n + 1 ? V[i] : 0u) + c;
                p[(int64_t)(n + i) * ld] = (uint32_t)x;
                c = (uint32_t)(x >> 32);
            }
        }
    }
}

// ======================================================================================
// mpz layer (sign-magnitude with GMP size convention) on matrix views.
// ======================================================================================
__device__ __forceinline__ int64_t ent(const MatArgs &m, int64_t e) {
    // elementwise ops treat the view as rows x cols; e is the row-major index
    int64_t r = e / m.cols, c = e - r * m.cols;
    return r * m.rs + c;
}

// w = u + sgn * v for one entry (W's entry at offset iw, U's at iu, V's at iv).
// For opposite signs the magnitudes are compared from the top before the
// subtraction (GMP mpz_add semantics).  W may be U or V (in place).
__device__ void addsub_entry(const MatArgs &W, int64_t iw, const MatArgs &U, int64_t iu, const MatArgs &V, int64_t iv,
                             int sub, uint32_t *err) {
    int su = U.sizes[iu], sv = V.sizes[iv];
    if (sub) sv = -sv;
    const int un = iabs_d(su), vn = iabs_d(sv);
    // a size beyond its operand's planes is malformed input: nothing past the planes is read
    if (un > U.nlimbs || vn > V.nlimbs) { atomicOr(err, DEVERR_BADARG); W.sizes[iw] = 0; return; }
    const uint32_t *up = U.limbs + iu, *vp = V.limbs + iv;
    uint32_t *wp = W.limbs + iw;
    // equal signs (or a zero operand) add magnitudes; opposite signs subtract the
    // smaller magnitude from the larger
    const bool add = (su < 0) == (sv < 0) || un == 0 || vn == 0;
    const int cmp = add ? 1 : (un != vn ? (un < vn ? -1 : 1) : dev_cmp(up, U.ld, vp, V.ld, un));
    const bool swap = cmp < 0;
    const uint32_t *xp = swap ? vp : up, *yp = swap ? up : vp;
    const int xn = swap ? vn : un, yn = swap ? un : vn;
    const int64_t xs = swap ? V.ld : U.ld, ys = swap ? U.ld : V.ld;
    const int neg = add ? (un ? (su < 0) : (sv < 0)) : (swap ? (sv < 0) : (su < 0));
    // operand limbs beyond W's planes: rejected before anything is written, so an
    // in-place call (W aliasing U or V) keeps its operand; only a carry out of W's
    // last plane (found after the pass) leaves W's limbs undefined
    if (xn > W.nlimbs || yn > W.nlimbs) { atomicOr(err, DEVERR_CAPACITY); W.sizes[iw] = 0; return; }
    // every lane runs over all of W's planes, writing the zero tail in the same pass:
    // the warp's stores to a plane go out together as whole sectors
    uint32_t c = 0;  // carry or borrow
    int len = 0;
    for (int i = 0; i < W.nlimbs; i++) {
        const uint32_t x = i < xn ? xp[(int64_t)i * xs] : 0u, y = i < yn ? yp[(int64_t)i * ys] : 0u;
        uint32_t r;
        if (add) {
            const uint64_t t = (uint64_t)x + y + c;
            r = (uint32_t)t;
            c = (uint32_t)(t >> 32);
        } else {
            const uint64_t t = (uint64_t)x - y - c;
            r = (uint32_t)t;
            c = (uint32_t)(t >> 63);
        }
        wp[(int64_t)i * W.ld] = r;
        if (r) len = i + 1;
    }
    // a carry out of W's last plane: W is too small (its size is set to 0 so a
    // later reader of W stays inside its planes)
    if (add && c) { atomicOr(err, DEVERR_CAPACITY); W.sizes[iw] = 0; return; }
    W.sizes[iw] = len == 0 ? 0 : (neg ? -len : len);
}

// w = u + sgn * v, one thread per entry.
__global__ void k_mpz_addsub(MatArgs W, MatArgs U, MatArgs V, int sub, int64_t count, uint32_t *err) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    addsub_entry(W, ent(W, e), U, ent(U, e), V, ent(V, e), sub, err);
}

// w = u * v (op 0), w += u * v (op 1), w -= u * v (op 2); one thread per entry.
// The product is formed column by column (product scanning) and merged with w
// in the same pass.  When w and the product have opposite signs the merge is a
// two's complement subtraction; a final borrow means |uv| > |w| and the
// written limbs are negated in place.
__global__ void k_mpz_mulops(MatArgs W, MatArgs U, MatArgs V, int op, int64_t count, uint32_t *err) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const int64_t iw = ent(W, e), iu = ent(U, e), iv = ent(V, e);
    const int su = U.sizes[iu], sv = V.sizes[iv];
    const int un = iabs_d(su), vn = iabs_d(sv);
    const uint32_t *up = U.limbs + iu, *vp = V.limbs + iv;
    uint32_t *wp = W.limbs + iw;
    const int64_t ws = W.ld;
    int sw = op == 0 ? 0 : W.sizes[iw];
    const int wn = iabs_d(sw);
    int pneg = (su < 0) ^ (sv < 0);
    if (op == 2) pneg ^= 1;
    const int pn = (un && vn) ? un + vn : 0;
    const int subtract = wn && pn && ((sw < 0) != pneg);
    const int rn = (pn > wn ? pn : wn) + (subtract ? 0 : 1);
    const int cap = W.nlimbs;
    // Result limbs [0, rn).  Limbs of w beyond wn are zero by invariant.  Limbs
    // at t >= cap are not stored; hi_nz / hi_ones remember whether any of them
    // is nonzero / all of them are all-ones, which decides overflow below.
    uint32_t c0 = 0, c1 = 0, c2 = 0;  // product column accumulator
    uint32_t carry = 0;              // merge carry / borrow
    int top = 0;
    bool hi_nz = false, hi_ones = true;
    for (int t = 0; t < rn; t++) {
        uint32_t pl = 0;
        if (t < pn - 1) {
            int i0 = t - vn + 1 > 0 ? t - vn + 1 : 0;
            int i1 = t < un - 1 ? t : un - 1;
            for (int i = i0; i <= i1; i++) MAC96(c0, c1, c2, up[(int64_t)i * U.ld], vp[(int64_t)(t - i) * V.ld]);
            pl = c0; c0 = c1; c1 = c2; c2 = 0;
        } else if (t == pn - 1) {
            pl = c0;
        }
        uint32_t wl = (op != 0 && t < wn) ? wp[(int64_t)t * ws] : 0u;
        uint32_t r;
        if (!subtract) {
            uint64_t s = (uint64_t)wl + pl + carry;
            r = (uint32_t)s; carry = (uint32_t)(s >> 32);
        } else {
            uint64_t d = (uint64_t)wl - pl - carry;
            r = (uint32_t)d; carry = (uint32_t)(d >> 63);
        }
        if (t < cap) {
            wp[(int64_t)t * ws] = r;
            if (r) top = t + 1;
        } else {
            hi_nz |= r != 0u;
            hi_ones &= r == 0xFFFFFFFFu;
        }
    }
    int neg = op == 0 ? pneg : (wn ? (sw < 0) : pneg);
    if (subtract && carry) {
        // negative: |result| = 2^(32 rn) - r; it fits in cap limbs iff the
        // dropped high limbs are all ones and the kept low part is nonzero
        if (rn > cap && !(hi_ones && top != 0)) { atomicOr(err, DEVERR_CAPACITY); return; }
        neg = pneg;
        uint32_t c = 1;
        top = 0;
        const int kept = rn < cap ? rn : cap;
        for (int t = 0; t < kept; t++) {
            uint64_t s = (uint64_t)(~wp[(int64_t)t * ws]) + c;
            uint32_t r = (uint32_t)s;
            c = (uint32_t)(s >> 32);
            wp[(int64_t)t * ws] = r;
            if (r) top = t + 1;
        }
    } else if (hi_nz) {
        atomicOr(err, DEVERR_CAPACITY);
        return;
    }
    for (int t = rn < cap ? rn : cap; t < cap; t++) wp[(int64_t)t * ws] = 0u;
    W.sizes[iw] = top == 0 ? 0 : (neg ? -top : top);
}

__global__ void k_mat_zero(MatArgs C, int64_t count) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const int64_t ic = ent(C, e);
    for (int i = 0; i < C.nlimbs; i++) C.limbs[(int64_t)i * C.ld + ic] = 0u;
    C.sizes[ic] = 0;
}

// Sizes of the low (limbs [0,h)) and high (limbs [h, nlimbs)) parts of every
// entry, same sign as the entry; the limb planes themselves are shared views.
__global__ void k_split_sizes(MatArgs X, int h, int32_t *lo, int32_t *hi, int64_t count) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const int64_t ix = ent(X, e);
    const int s = X.sizes[ix], n = iabs_d(s);
    int nlo = n < h ? n : h;
    while (nlo > 0 && X.limbs[(int64_t)(nlo - 1) * X.ld + ix] == 0u) nlo--;
    const int nhi = n > h ? n - h : 0;  // top limb of the entry is nonzero, so no normalisation needed
    lo[ix] = s < 0 ? -nlo : nlo;  // same (row stride) layout as the source sizes
    hi[ix] = s < 0 ? -nhi : nhi;
}

// W = U + V * 2^(32 sh), elementwise and signed; W may be U.
// w = u + v 2^(32 sh) for entry e, one thread (the general form: any signs, results
// past W's planes flagged)
__device__ void add_shifted_serial(const MatArgs &W, const MatArgs &U, const MatArgs &V, int sh, int64_t e,
                                   uint32_t *err) {
    const int64_t iw = ent(W, e), iu = ent(U, e), iv = ent(V, e);
    const int su = U.sizes[iu], sv = V.sizes[iv];
    const int un = iabs_d(su), vn0 = iabs_d(sv), vn = vn0 ? vn0 + sh : 0;
    const uint32_t *up = U.limbs + iu, *vp = V.limbs + iv;
    uint32_t *wp = W.limbs + iw;
    auto ul = [&](int t) -> uint32_t { return t < un ? up[(int64_t)t * U.ld] : 0u; };
    auto vl = [&](int t) -> uint32_t { return (t >= sh && t < vn) ? vp[(int64_t)(t - sh) * V.ld] : 0u; };
    const int mx = un > vn ? un : vn;
    int len = 0, neg;
    if (vn0 == 0 || un == 0 || (su < 0) == (sv < 0)) {
        neg = un ? su < 0 : sv < 0;
        uint32_t c = 0;
        // eight limbs at a time: all sixteen loads go out before the chunk's stores (W may
        // be U itself; a chunk's limbs are read before they are written)
        for (int t0 = 0; t0 < mx; t0 += 8) {
            uint32_t xu[8], xv[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                xu[k] = ul(t0 + k);
                xv[k] = vl(t0 + k);
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int t = t0 + k;
                if (t >= mx) break;
                const uint64_t x = (uint64_t)xu[k] + xv[k] + c;
                if (t >= W.nlimbs) { if ((uint32_t)x) { atomicOr(err, DEVERR_CAPACITY); return; } }
                else wp[(int64_t)t * W.ld] = (uint32_t)x;
                c = (uint32_t)(x >> 32);
                if ((uint32_t)x) len = t + 1;
            }
        }
        if (c) {
            if (mx >= W.nlimbs) { atomicOr(err, DEVERR_CAPACITY); return; }
            wp[(int64_t)mx * W.ld] = c;
            len = mx + 1;
        }
    } else {
        int cmp = 0;
        if (un != vn) cmp = un < vn ? -1 : 1;
        for (int t = mx - 1; t >= 0 && cmp == 0; t--)
            if (ul(t) != vl(t)) cmp = ul(t) < vl(t) ? -1 : 1;
        neg = cmp >= 0 ? su < 0 : sv < 0;
        uint32_t br = 0;
        for (int t0 = 0; t0 < mx; t0 += 8) {
            uint32_t xu[8], xv[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                xu[k] = ul(t0 + k);
                xv[k] = vl(t0 + k);
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int t = t0 + k;
                if (t >= mx) break;
                const uint32_t x = cmp >= 0 ? xu[k] : xv[k], y = cmp >= 0 ? xv[k] : xu[k];
                const uint64_t d = (uint64_t)x - y - br;
                br = (uint32_t)(d >> 63);
                if (t >= W.nlimbs) { if ((uint32_t)d) { atomicOr(err, DEVERR_CAPACITY); return; } }
                else wp[(int64_t)t * W.ld] = (uint32_t)d;
                if ((uint32_t)d) len = t + 1;
            }
        }
    }
    for (int t = mx + 1; t < W.nlimbs; t++) wp[(int64_t)t * W.ld] = 0u;
    if (mx < W.nlimbs && len <= mx) wp[(int64_t)mx * W.ld] = 0u;
    W.sizes[iw] = len == 0 ? 0 : (neg ? -len : len);
}

// The same with the limbs of an addition cut into segments: a CTA takes 32 entries
// (one per lane, loads coalesced across entries) and each of its 8 warps one segment
// of W's planes.  A segment is summed from carry-in 0, noting its carry-out, whether
// it came out all ones and its top nonzero limb; warp 0 then resolves each entry's
// segment carry-ins (carry-select), and a segment that receives a carry adds it from
// its bottom limb (it stops at the first limb that does not wrap).  Subtractions and
// results that would not fit W take the one-thread form.
constexpr int ADDSH_SEGS = 8;
constexpr int64_t ADDSH_SEG_BELOW = 48 * 1024;  // entries below which the segmented form runs

__global__ void k_add_shifted(MatArgs W, MatArgs U, MatArgs V, int sh, int64_t count, uint32_t *err) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    add_shifted_serial(W, U, V, sh, e, err);
}

__global__ void __launch_bounds__(32 * ADDSH_SEGS) k_add_shifted_seg(MatArgs W, MatArgs U, MatArgs V, int sh,
                                                                     int64_t count, uint32_t *err) {
    __shared__ uint32_t s_carry[ADDSH_SEGS][32], s_ones[ADDSH_SEGS][32], s_cin[ADDSH_SEGS][32];
    __shared__ int s_top[ADDSH_SEGS][32];
    const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
    const int64_t e = (int64_t)blockIdx.x * 32 + lane;
    bool seg = false;  // this entry takes the segmented addition
    int64_t iw = 0, iu = 0, iv = 0;
    int su = 0, sv = 0, un = 0, vn0 = 0, vn = 0;
    if (e < count) {
        iw = ent(W, e); iu = ent(U, e); iv = ent(V, e);
        su = U.sizes[iu]; sv = V.sizes[iv];
        un = iabs_d(su); vn0 = iabs_d(sv); vn = vn0 ? vn0 + sh : 0;
        const int mx = un > vn ? un : vn;
        seg = (vn0 == 0 || un == 0 || (su < 0) == (sv < 0)) && mx <= W.nlimbs && un <= U.nlimbs && vn0 <= V.nlimbs;
    }
    const int S = (W.nlimbs + ADDSH_SEGS - 1) / ADDSH_SEGS;
    const int t0 = min(j * S, W.nlimbs), t1 = min(t0 + S, W.nlimbs);
    if (seg) {
        const uint32_t *up = U.limbs + iu, *vp = V.limbs + iv;
        uint32_t *wp = W.limbs + iw;
        uint32_t c = 0, ones = 1;  // an empty segment passes a carry through
        int top = -1;
        for (int tb = t0; tb < t1; tb += 8) {
            uint32_t xu[8], xv[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int t = tb + k;
                xu[k] = t < un ? up[(int64_t)t * U.ld] : 0u;
                xv[k] = (t >= sh && t < vn) ? vp[(int64_t)(t - sh) * V.ld] : 0u;
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int t = tb + k;
                if (t >= t1) break;
                const uint64_t x = (uint64_t)xu[k] + xv[k] + c;
                const uint32_t w = (uint32_t)x;
                wp[(int64_t)t * W.ld] = w;
                c = (uint32_t)(x >> 32);
                ones &= w == 0xFFFFFFFFu;
                if (w) top = t;
            }
        }
        s_carry[j][lane] = c;
        s_ones[j][lane] = ones;
        s_top[j][lane] = top;
    }
    __syncthreads();
    bool cap = false;  // warp 0: a carry out of W's last plane
    if (j == 0 && seg) {
        uint32_t cin = 0;
        for (int q = 0; q < ADDSH_SEGS; q++) {
            s_cin[q][lane] = cin;
            cin = s_carry[q][lane] | (s_ones[q][lane] & cin);
        }
        if (cin) {
            atomicOr(err, DEVERR_CAPACITY);
            cap = true;
        }
    }
    __syncthreads();
    if (seg && s_cin[j][lane] && t1 > t0) {
        uint32_t *wp = W.limbs + iw;
        int t = t0;
        for (; t < t1; t++) {
            const uint32_t w = wp[(int64_t)t * W.ld] + 1u;
            wp[(int64_t)t * W.ld] = w;
            if (w) break;
        }
        s_top[j][lane] = s_ones[j][lane] ? -1 : max(s_top[j][lane], t);
    }
    __syncthreads();
    if (j == 0 && e < count) {
        if (seg) {
            int top = -1;
            for (int q = 0; q < ADDSH_SEGS; q++) top = max(top, s_top[q][lane]);
            const int len = top + 1;
            const int neg = un ? su < 0 : sv < 0;
            // W too small: its size is set to 0 so a later reader stays inside its planes
            W.sizes[iw] = (len == 0 || cap) ? 0 : (neg ? -len : len);
        } else {
            add_shifted_serial(W, U, V, sh, e, err);
        }
    }
}

// dst = src (entries copied with their sizes; planes beyond the value zeroed)
__global__ void k_mat_copy(MatArgs D, MatArgs S, int64_t count, uint32_t *err) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const int64_t id = ent(D, e), is = ent(S, e);
    const int ss = S.sizes[is], n = iabs_d(ss);
    if (n > D.nlimbs) { atomicOr(err, DEVERR_CAPACITY); return; }
    // eight planes at a time: the loads go out together, ahead of the stores
    for (int i0 = 0; i0 < D.nlimbs; i0 += 8) {
        uint32_t v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = i0 + k < n ? S.limbs[(int64_t)(i0 + k) * S.ld + is] : 0u;
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (i0 + k < D.nlimbs) D.limbs[(int64_t)(i0 + k) * D.ld + id] = v[k];
    }
    D.sizes[id] = ss;
}

__global__ void k_max_size(MatArgs A, int64_t count, int32_t *out) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int v = 0;
    if (e < count) v = iabs_d(A.sizes[ent(A, e)]);
    for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    if ((threadIdx.x & 31) == 0 && v) atomicMax(out, v);
}

// ======================================================================================
// Per-entry matrix product  C (K x N) = A (K x M) * B (M x N)   [or C += A*B]
//
// The reference gives one thread a whole C[y][x] and runs mpz_mul followed by
// M-1 serial mpz_addmul calls (mat-gpu/mat-core.h:31-53).  Here a group of G
// threads shares one output entry: the La x Lb limb-product square of every
// term A[y][k]*B[k][x] is tiled into R x R blocks, thread (I, J) of the group
// owns block (I, J) for all k and keeps its 2R-1 partial columns in 96-bit
// two's-complement registers: a term with positive sign is added, a negative
// one subtracted (the sign is the same for the whole group, so the branch is
// warp-uniform when groups span whole warps).  No carry leaves a column inside
// the k loop.  After the loop each thread parks its columns in shared memory,
// the CTA sums the partial columns of every entry (a column gathers the
// blocks on two neighbouring anti-diagonals), and the signed carries are
// propagated (one warp per entry when groups span whole warps, each lane a
// segment of limbs; else one thread per entry), the old C is added for
// C += A*B and the sign-magnitude result is written.  A/B limbs for a chunk of
// KC terms are staged in shared memory by 4-byte cp.async copies coalesced
// along k (A) and along x (B), double-buffered so the next chunk's copies run
// during this chunk's MACs, read back as 128-bit vectors and reused by every
// thread of the CTA's TY x TX entries.  An operand one limb longer than a
// multiple of R (a Winograd sum of full-length entries) does not get a block
// row of its own: the threads on the grid's edge fold its top limb in.
// ======================================================================================
namespace {
constexpr int MM_THREADS = 256;       // CTA size when groups of <= 256 threads share a CTA
constexpr int MM_THREADS_WIDE = 512;  // largest CTA: one group of up to 512 threads
constexpr int MM_KC = 16;  // terms per staged chunk (a power of two: staging index math is shifts and masks)
}

// 4-byte asynchronous global -> shared copy; a copy with valid == false reads
// nothing and writes a zero (src-size 0).  `gsafe` is any valid global address.
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, const void *gsafe, bool valid) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(sa), "l"(valid ? gmem : gsafe),
                 "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

struct MMCfg {
    int R;        // block edge in limbs
    int La, Lb;   // padded limb counts (multiples of R)
    int G, Gp;    // threads per entry (active, padded)
    int NT;       // threads per CTA (entries x Gp, at most MM_THREADS; Gp for one wide group)
    int thinA, thinB;  // the operand has one limb past a multiple of R (and more than R):
                       // the main grid's edge threads fold that top limb in
    int TY, TX;   // entries per CTA
    int TXs;      // log2(TX) (TX is a power of two)
    int M;        // inner dimension
    int accumulate;
};

// (c0, c1, c2) -= a * b on a 96-bit two's-complement accumulator
#define MSC96(c0, c1, c2, a, b)                                                   \
    asm("{\n\t.reg .u32 lo_, hi_;\n\t"                                          \
        "mul.lo.u32 lo_, %3, %4;\n\t"                                            \
        "mul.hi.u32 hi_, %3, %4;\n\t"                                            \
        "sub.cc.u32 %0, %0, lo_;\n\t"                                            \
        "subc.cc.u32 %1, %1, hi_;\n\t"                                           \
        "subc.u32 %2, %2, 0;\n\t}"                                               \
        : "+r"(c0), "+r"(c1), "+r"(c2)                                            \
        : "r"(a), "r"(b))

// Top-limb products of a thin operand (one limb past a multiple of R, a
// Winograd sum of full-length entries): a_top * b_j for every limb j of B
// (b_top included when B is thin too), then a_i * b_top for every limb i of
// A's main grid.  Item it goes to thread it % G, which keeps one extra column
// accumulator per item it holds, so the extra work is spread evenly over the
// group (one or two MACs a term on top of R * R) instead of loading the grid's
// edge threads.  At most MM_XMAX items a thread.
constexpr int MM_XMAX = 3;

// P (+|-)= a-block x b-block (R x R, columns 0 .. 2R - 2).
template <int R, int NC, bool NEG>
__device__ __forceinline__ void block_mac(uint32_t (&P)[NC][3], const uint32_t (&a)[R], const uint32_t (&b)[R]) {
#pragma unroll
    for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < R; j++) {
            if (NEG) MSC96(P[i + j][0], P[i + j][1], P[i + j][2], a[i], b[j]);
            else MAC96(P[i + j][0], P[i + j][1], P[i + j][2], a[i], b[j]);
        }
}
// Signed carry resolution of one entry's column sums by the 32 lanes of a warp
// (all lanes call it).  col[t] = (s0, s1, s2) for t < Lc is column t's value
// s0 + s1 2^32 + s2 2^64 (s2 signed); buf has LB = Lc + 2 words.  Lane l takes
// the limbs [l S, l S + S), S >= 2: it forms them from carry-in 0 and notes its
// carry-out q.  A carry-in c (|c| < 2^53) then changes the carry-out by
// floor((r + c) / 2^(32 len)) in {-1, 0, 1} (r: the segment's limbs), which a
// 31-step shuffle chain resolves from the segment's low 64 bits and whether its
// upper limbs are all ones / all zeros.  Then the sign, the two's-complement
// negation (the +1 reaches a lane when every lower limb is zero: one ballot),
// the normalized size and the store of entry ic of C (plus the old C for C += A*B).
__device__ void resolve_store_warp(const unsigned long long *col, uint32_t *buf, int Lc, int LB, const MatArgs &C,
                                   int64_t ic, int accumulate, uint32_t *err) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    int sc = 0, cn = 0;
    if (accumulate) {
        sc = C.sizes[ic];
        cn = iabs_d(sc);
    }
    if (cn > LB || cn > C.nlimbs) {
        if (lane == 0) atomicOr(err, DEVERR_CAPACITY);
        return;
    }
    const int S = max(2, (LB + 31) / 32);
    const int t0 = min(lane * S, LB), t1 = min(t0 + S, LB);
    const bool empty = t0 >= t1;
    long long q = 0;
    for (int t = t0; t < t1; t++) {
        unsigned long long w0 = 0, w1 = 0;
        long long w2 = 0;
        if (t < Lc) {
            w0 = col[t * 3];
            w1 = col[t * 3 + 1];
            w2 = (long long)col[t * 3 + 2];
        }
        long long extra = 0;
        if (t < cn) {
            const long long v = (long long)C.limbs[(int64_t)t * C.ld + ic];
            extra = sc < 0 ? -v : v;
        }
        const long long lo = (long long)(w0 & 0xFFFFFFFFull) + (q & 0xFFFFFFFFll) + extra;
        buf[t] = (uint32_t)lo;
        q = (lo >> 32) + (q >> 32) + (long long)(w0 >> 32) + (long long)w1 + (w2 << 32);
    }
    bool hi_ones = true, hi_zero = true;
    for (int t = t0 + 2; t < t1; t++) {
        hi_ones &= buf[t] == 0xFFFFFFFFu;
        hi_zero &= buf[t] == 0u;
    }
    const unsigned long long low64 =
        empty ? 0ull : ((unsigned long long)buf[t0] | (t0 + 1 < t1 ? (unsigned long long)buf[t0 + 1] << 32 : 0ull));
    auto carry_out = [&](long long c) -> long long {
        if (empty) return c;
        if (t1 - t0 == 1) return q + (((long long)buf[t0] + c) >> 32);
        if (c >= 0) return q + ((low64 + (unsigned long long)c < low64 && hi_ones) ? 1 : 0);
        return q - ((low64 < (unsigned long long)(-c) && hi_zero) ? 1 : 0);
    };
    long long cin = 0;
    for (int l = 0; l < 31; l++) {
        const long long v = __shfl_sync(FULL, carry_out(cin), l);
        if (lane == l + 1) cin = v;
    }
    const long long fin = __shfl_sync(FULL, carry_out(cin), 31);
    // the exact sum fits LB limbs, so what is left is the sign extension (0 or -1)
    if (fin != 0 && fin != -1) {
        if (lane == 0) atomicOr(err, DEVERR_CAPACITY);
        return;
    }
    long long c = cin;
    for (int t = t0; t < t1; t++) {
        const long long lo = (long long)buf[t] + (c & 0xFFFFFFFFll);
        buf[t] = (uint32_t)lo;
        c = (lo >> 32) + (c >> 32);
    }
    const bool neg = fin < 0;
    if (neg) {
        bool z = true;
        for (int t = t0; t < t1; t++) z &= buf[t] == 0u;
        const unsigned zmask = __ballot_sync(FULL, z);
        const unsigned lower = lane == 0 ? 0u : (FULL >> (32 - lane));
        uint32_t c1 = ((~zmask) & lower) == 0u ? 1u : 0u;
        for (int t = t0; t < t1; t++) {
            const uint32_t v = ~buf[t] + c1;
            c1 = (c1 && v == 0u) ? 1u : 0u;
            buf[t] = v;
        }
    }
    int top = 0;
    for (int t = t0; t < t1; t++)
        if (buf[t]) top = t + 1;
#pragma unroll
    for (int o = 16; o; o >>= 1) top = max(top, __shfl_xor_sync(FULL, top, o));
    if (top > C.nlimbs) {
        if (lane == 0) atomicOr(err, DEVERR_CAPACITY);
        return;
    }
    uint32_t *cl = C.limbs + ic;
    for (int t = t0; t < t1 && t < C.nlimbs; t++) cl[(int64_t)t * C.ld] = t < top ? buf[t] : 0u;
    for (int t = LB + lane; t < C.nlimbs; t += 32) cl[(int64_t)t * C.ld] = 0u;
    if (lane == 0) C.sizes[ic] = neg ? -top : top;
}

// Writes the signed multi-limb value held in buf[0..L) (two's complement,
// `neg` = its sign) into entry ic of C as sign-magnitude.
__device__ void store_signed(uint32_t *buf, int L, bool neg, const MatArgs &C, int64_t ic, uint32_t *err) {
    if (neg) {
        uint32_t c = 1;
        for (int t = 0; t < L; t++) {
            uint64_t v = (uint64_t)(~buf[t]) + c;
            buf[t] = (uint32_t)v;
            c = (uint32_t)(v >> 32);
        }
    }
    int top = 0;
    for (int t = 0; t < L; t++)
        if (buf[t]) top = t + 1;
    if (top > C.nlimbs) { atomicOr(err, DEVERR_CAPACITY); return; }
    uint32_t *cl = C.limbs + ic;
    for (int t = 0; t < C.nlimbs; t++) cl[(int64_t)t * C.ld] = t < top ? buf[t] : 0u;
    C.sizes[ic] = neg ? -top : top;
}

// One CTA tile (TY x TX output entries at tile coordinates by, bx) of the
// per-entry product; shared by the grid kernel and the persistent batched one.
// THIN: an operand has one limb past a multiple of R (cfg.thinA / thinB), which
// the main grid's edge threads fold in.
template <int R, bool THIN>
__device__ __forceinline__ void limb_tile(const MatArgs &C, const MatArgs &A, const MatArgs &B, const MMCfg &cfg,
                                          int by, int bx, unsigned char *smem_raw, uint32_t *err) {
    const int La = cfg.La, Lb = cfg.Lb, TY = cfg.TY, TX = cfg.TX;
    const int sa_stride = La + 4, sb_stride = Lb + 4;  // +4 words: fewer bank conflicts, 16B aligned rows
    // two staging buffers, each [TY][KC][La+4] A limbs, [KC][TX][Lb+4] B limbs,
    // [TY][KC] A sizes, [KC][TX] B sizes; chunk c + 1 is copied in (cp.async)
    // while chunk c is multiplied
    const int stage_words = TY * MM_KC * sa_stride + MM_KC * TX * sb_stride + (TY + TX) * MM_KC;
    uint32_t *stage_base = reinterpret_cast<uint32_t *>(smem_raw);

    const int tid = threadIdx.x, nt = cfg.NT;
    const int g = tid / cfg.Gp, lt = tid % cfg.Gp;
    const int EPC = TY * TX;
    const bool has_entry = g < EPC;
    const int ty = has_entry ? g / TX : 0, tx = has_entry ? g % TX : 0;
    const int y0 = by * TY, x0 = bx * TX;
    const int y = y0 + ty, x = x0 + tx;
    const bool valid = has_entry && y < C.rows && x < C.cols;
    const int nbA = La / R, nbB = Lb / R;
    // the main grid of full R x R blocks: ma x mb (one thread each); a thin operand's
    // top limb sits in limb ma * R (mb * R) and is folded in by the edge threads
    const int tA = THIN ? cfg.thinA : 0, tB = THIN ? cfg.thinB : 0;
    const int ma = nbA - tA, mb = nbB - tB;
    const bool active = valid && lt < cfg.G;
    const int I0 = active ? lt / mb : 0, J0 = active ? lt % mb : 0;
    constexpr int NC = 2 * R - 1;

    uint32_t P[NC][3];
#pragma unroll
    for (int c = 0; c < NC; c++) P[c][0] = P[c][1] = P[c][2] = 0;
    // top-limb items of this thread: limb xi[x] of A times limb xj[x] of B
    constexpr int XM = THIN ? MM_XMAX : 1;
    const int NA = tA * (mb * R + tB), NX = NA + tB * ma * R;
    uint32_t X[XM][3];
    int xi[XM], xj[XM];
#pragma unroll
    for (int x = 0; x < XM; x++) {
        X[x][0] = X[x][1] = X[x][2] = 0;
        const int it = lt + x * cfg.G;
        const bool ok = THIN && active && it < NX;
        xi[x] = !ok ? -1 : it < NA ? ma * R : it - NA;
        xj[x] = !ok ? -1 : it < NA ? it : mb * R;
    }

    const int M = cfg.M, TXs = cfg.TXs;
    const int nchunks = (M + MM_KC - 1) / MM_KC;
    auto stage = [&](int c) {
        uint32_t *sA = stage_base + (c & 1) * stage_words;
        uint32_t *sB = sA + TY * MM_KC * sa_stride;
        uint32_t *ssA = sB + MM_KC * TX * sb_stride;
        uint32_t *ssB = ssA + TY * MM_KC;
        const int k0 = c * MM_KC, kc = min(MM_KC, M - k0);
        // A[y0 + tyy][k0 + kk], limb i: consecutive threads walk kk (contiguous in a plane row)
        for (int tyy = 0; tyy < TY; tyy++) {
            const int yy = y0 + tyy;
            const uint32_t *arow = A.limbs + (int64_t)yy * A.rs + k0;
            for (int q = tid; q < La * MM_KC; q += nt) {
                const int kk = q & (MM_KC - 1), i = q >> 4;
                cp_async4(sA + (tyy * MM_KC + kk) * sa_stride + i, arow + (int64_t)i * A.ld + kk, A.limbs,
                          kk < kc && yy < A.rows && i < A.nlimbs);
            }
        }
        // B[k0 + kk][x0 + txx], limb i: consecutive threads walk txx (contiguous in a plane row)
        for (int q = tid; q < MM_KC * Lb * TX; q += nt) {
            const int txx = q & (TX - 1), r = q >> TXs, kk = r & (MM_KC - 1), i = r >> 4;
            const int xx = x0 + txx;
            cp_async4(sB + (kk * TX + txx) * sb_stride + i,
                      B.limbs + (int64_t)i * B.ld + (int64_t)(k0 + kk) * B.rs + xx, B.limbs,
                      kk < kc && xx < B.cols && i < B.nlimbs);
        }
        for (int q = tid; q < TY * MM_KC; q += nt) {
            const int kk = q & (MM_KC - 1), yy = y0 + (q >> 4);
            cp_async4(ssA + q, A.sizes + (int64_t)yy * A.rs + k0 + kk, A.sizes, kk < kc && yy < A.rows);
        }
        for (int q = tid; q < MM_KC * TX; q += nt) {
            const int txx = q & (TX - 1), kk = q >> TXs, xx = x0 + txx;
            cp_async4(ssB + q, B.sizes + (int64_t)(k0 + kk) * B.rs + xx, B.sizes, kk < kc && xx < B.cols);
        }
    };
    stage(0);
    cp_async_commit();
    for (int c = 0; c < nchunks; c++) {
        if (c + 1 < nchunks) stage(c + 1);
        cp_async_commit();  // an empty group on the last chunk keeps the wait count uniform
        cp_async_wait1();   // this thread's copies of chunk c have landed
        __syncthreads();    // ... and every thread's
        if (active) {
            const uint32_t *sA = stage_base + (c & 1) * stage_words;
            const uint32_t *sB = sA + TY * MM_KC * sa_stride;
            const int32_t *ssA = reinterpret_cast<const int32_t *>(sB + MM_KC * TX * sb_stride);
            const int32_t *ssB = ssA + TY * MM_KC;
            const int kc = min(MM_KC, M - c * MM_KC);
            for (int kk = 0; kk < kc; kk++) {
                const int sa = ssA[ty * MM_KC + kk], sb = ssB[kk * TX + tx];
                if (sa == 0 || sb == 0) continue;
                const bool pos = (sa ^ sb) >= 0;
                const uint32_t *ra = sA + (ty * MM_KC + kk) * sa_stride;
                const uint32_t *rb = sB + (kk * TX + tx) * sb_stride;
                if (THIN) {
#pragma unroll
                    for (int x = 0; x < XM; x++) {
                        if (xi[x] < 0) continue;
                        const uint32_t u = ra[xi[x]], v = rb[xj[x]];
                        if (pos) MAC96(X[x][0], X[x][1], X[x][2], u, v);
                        else MSC96(X[x][0], X[x][1], X[x][2], u, v);
                    }
                }
                if (I0 * R >= iabs_d(sa) || J0 * R >= iabs_d(sb)) continue;
                const uint32_t *pa = ra + I0 * R;
                const uint32_t *pb = rb + J0 * R;
                uint32_t a[R], b[R];
                if (R >= 4) {
#pragma unroll
                    for (int v = 0; v < R; v += 4) {
                        uint4 qa = *reinterpret_cast<const uint4 *>(pa + v);
                        uint4 qb = *reinterpret_cast<const uint4 *>(pb + v);
                        a[v] = qa.x; a[v + 1] = qa.y; a[v + 2] = qa.z; a[v + 3] = qa.w;
                        b[v] = qb.x; b[v + 1] = qb.y; b[v + 2] = qb.z; b[v + 3] = qb.w;
                    }
                } else {
#pragma unroll
                    for (int v = 0; v < R; v++) { a[v] = pa[v]; b[v] = pb[v]; }
                }
                if (pos) block_mac<R, NC, false>(P, a, b);
                else block_mac<R, NC, true>(P, a, b);
            }
        }
        __syncthreads();  // buffer c & 1 is refilled by the copies of chunk c + 2
    }

    // ---- reduction of partial columns ---------------------------------------------------
    const int Lc = La + Lb;       // product columns (padded)
    const int LB = Lc + 2;        // result limbs (two extra for the carry out of the sum over k)
    uint32_t *part = reinterpret_cast<uint32_t *>(smem_raw);  // [EPC][G][NC][3]
    uint32_t *xpart = part + (size_t)EPC * cfg.G * NC * 3;     // [EPC][XM][G][3] (thin operands)
    const size_t part_words = (size_t)EPC * cfg.G * (NC + (THIN ? XM : 0)) * 3;
    unsigned long long *cs = reinterpret_cast<unsigned long long *>(part + ((part_words + 1) & ~(size_t)1));  // [EPC][Lc][3]
    uint32_t *res = reinterpret_cast<uint32_t *>(cs + (size_t)EPC * Lc * 3);                                  // [EPC][LB]
    if (active) {
        uint32_t *dst = part + ((size_t)g * cfg.G + I0 * mb + J0) * NC * 3;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            dst[c * 3 + 0] = P[c][0];
            dst[c * 3 + 1] = P[c][1];
            dst[c * 3 + 2] = P[c][2];
        }
        if (THIN) {
#pragma unroll
            for (int x = 0; x < XM; x++) {
                uint32_t *xd = xpart + (((size_t)g * XM + x) * cfg.G + lt) * 3;
                xd[0] = X[x][0];
                xd[1] = X[x][1];
                xd[2] = X[x][2];
            }
        }
    }
    __syncthreads();
    // column t of entry gg gathers the blocks on diagonal d = t / R - h at offset
    // t % R + h R, for h = 0, 1, and with thin operands the top-limb items that
    // land in it: a_top * b_(t - ma R) and a_(t - mb R) * b_top
    for (int item = tid; item < EPC * Lc; item += nt) {
        const int gg = item / Lc, t = item % Lc;
        unsigned long long s0 = 0, s1 = 0;
        long long s2 = 0;
#pragma unroll
        for (int h = 0; h <= (NC - 1) / R; h++) {
            const int d = t / R - h, off = t % R + h * R;
            if (d < 0 || off >= NC) continue;
            const int i_lo = d - mb + 1 > 0 ? d - mb + 1 : 0, i_hi = d < ma - 1 ? d : ma - 1;
            for (int i = i_lo; i <= i_hi; i++) {
                const uint32_t *w = part + ((size_t)gg * cfg.G + i * mb + (d - i)) * NC * 3 + off * 3;
                s0 += w[0];
                s1 += w[1];
                s2 += (int32_t)w[2];
            }
        }
        if (THIN) {
            const int ia = t - ma * R, ib = t - mb * R;
            const int its[2] = {tA && ia >= 0 && ia < NA ? ia : -1, tB && ib >= 0 && ib < ma * R ? NA + ib : -1};
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (its[q] < 0) continue;
                const uint32_t *w = xpart + (((size_t)gg * XM + its[q] / cfg.G) * cfg.G + its[q] % cfg.G) * 3;
                s0 += w[0];
                s1 += w[1];
                s2 += (int32_t)w[2];
            }
        }
        unsigned long long *o = cs + ((size_t)gg * Lc + t) * 3;
        o[0] = s0;
        o[1] = s1;
        o[2] = (unsigned long long)s2;
    }
    __syncthreads();
    if (cfg.Gp >= 32) {
        // one warp per entry: the group's first 32 threads (a whole warp, as Gp is a multiple of 32)
        if (!(valid && lt < 32)) return;
        resolve_store_warp(cs + (size_t)g * Lc * 3, res + (size_t)g * LB, Lc, LB, C, (int64_t)y * C.rs + x,
                           cfg.accumulate, err);
        return;
    }
    if (!(valid && lt == 0)) return;

    // ---- signed carry propagation, optional C += , write back (one thread per entry) --------
    const int64_t ic = (int64_t)y * C.rs + x;
    const unsigned long long *col = cs + (size_t)g * Lc * 3;
    uint32_t *buf = res + (size_t)g * LB;
    int sc = 0, cn = 0;
    if (cfg.accumulate) {
        sc = C.sizes[ic];
        cn = iabs_d(sc);
        if (cn > LB) { atomicOr(err, DEVERR_CAPACITY); return; }
    }
    long long carry = 0;  // |carry| < 2^52
    for (int t = 0; t < LB; t++) {
        unsigned long long w0 = 0, w1 = 0;
        long long w2 = 0;
        if (t < Lc) {
            w0 = col[t * 3];
            w1 = col[t * 3 + 1];
            w2 = (long long)col[t * 3 + 2];
        }
        long long extra = 0;
        if (t < cn) extra = sc < 0 ? -(long long)C.limbs[(int64_t)t * C.ld + ic] : (long long)C.limbs[(int64_t)t * C.ld + ic];
        const long long lo = (long long)(w0 & 0xFFFFFFFFull) + (carry & 0xFFFFFFFFll) + extra;
        buf[t] = (uint32_t)lo;
        carry = (lo >> 32) + (carry >> 32) + (long long)(w0 >> 32) + (long long)w1 + (w2 << 32);
    }
    // the exact sum fits LB limbs, so what is left is the sign extension (0 or -1)
    if (carry != 0 && carry != -1) { atomicOr(err, DEVERR_CAPACITY); return; }
    store_signed(buf, LB, carry < 0, C, ic, err);
}

// 256-thread CTAs are sized for two per SM (at most 128 registers a thread)
template <int R, int NT, bool THIN>
__global__ void __launch_bounds__(NT, NT <= MM_THREADS ? 2 : 1)
    k_limb_matmul(MatArgs C, MatArgs A, MatArgs B, MMCfg cfg, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    limb_tile<R, THIN>(C, A, B, cfg, blockIdx.y, blockIdx.x, smem_raw, err);
}

// Persistent form for batches of uneven products: every CTA takes (job, tile)
// items from a device work queue (items sorted by cost, largest first, so the
// tail is short) until the queue is empty.  One launch covers all limb-path
// jobs of one block edge R.
struct LimbJob {
    MatArgs C, A, B;
    MMCfg cfg;
};

template <int R, int NT, bool THIN>
__global__ void __launch_bounds__(NT, NT <= MM_THREADS ? 2 : 1)
    k_limb_batched(const LimbJob *jobs, const int *items, int nitems, int *counter, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = atomicAdd(counter, 1);
        __syncthreads();
        const int it = cur;
        if (it >= nitems) break;
        const LimbJob &j = jobs[items[3 * it]];
        const MatArgs C = j.C, A = j.A, B = j.B;
        const MMCfg cfg = j.cfg;
        limb_tile<R, THIN>(C, A, B, cfg, items[3 * it + 1], items[3 * it + 2], smem_raw, err);
        __syncthreads();
    }
}

// ======================================================================================
// Breadth-first Winograd recursion.
//
// The depth-first recursion (host.cpp) issues a level's seven products and
// fifteen additions one after another, each a small launch.  Here the whole
// tree is laid out in workspace arrays and every level is one launch: one for
// all sums of a level, one for all leaf products of the tree (one CTA per leaf
// tile), one for all combinations of a level.  Nodes are numbered from the
// root (level 0); node q at level d has children 7q + j at level d + 1, the
// products of Winograd's scheme in the reference's operation order
// (mat-gpu/mat-defines.h:144-164, mat-cpu/mat.c:193-251):
//   j = 0: M1  = A11 B11        j = 4: M5 = S1 T1
//   j = 1: M2  = A12 B21        j = 5: M6 = S2 T2
//   j = 2: M3  = S4 B22         j = 6: M7 = S3 T3
//   j = 3: M4' = A22 T4'
// with S1 = A21 + A22, S2 = S1 - A11, S3 = A11 - A21, S4 = A12 - S2 and
// T1 = B12 - B11, T2 = B22 - T1, T3 = B22 - B12, T4' = B21 - T2, and
//   C11 = M1 + M2, C12 = M1 + M6 + M5 + M3,
//   C21 = M1 + M6 + M7 + M4', C22 = M1 + M6 + M7 + M5.
// The sums of parent q at level d - 1 are matrices 4q + s (s = 0..3: S1..S4,
// T1..T4') of level d's sum arrays; the products of level d are matrices
// 0..7^d - 1 of its product array; level 0's output is the caller's C.
// Every operand view is computed on the device from the node's index path, so
// a launch takes no job table and the sequence can be captured in a graph.
// ======================================================================================
__device__ __forceinline__ MatArgs wt_quad(MatArgs m, int qr, int qc, int h) {
    const int64_t off = (int64_t)qr * h * m.rs + (int64_t)qc * h;
    m.limbs += off;
    m.sizes += off;
    m.rows = h;
    m.cols = h;
    return m;
}
__device__ __forceinline__ MatArgs wt_dense(uint32_t *limbs, int32_t *sizes, int64_t q, int h, int cap) {
    MatArgs m;
    const int64_t e = (int64_t)h * h;
    m.limbs = limbs + q * e * cap;
    m.sizes = sizes + q * e;
    m.rs = h;
    m.ld = e;
    m.rows = h;
    m.cols = h;
    m.nlimbs = cap;
    return m;
}
// Operand `which` (0: A, 1: B) of node `node` at level d.
__device__ MatArgs wt_operand(const WinoTree &t, int which, int d, int64_t node) {
    MatArgs v = margs(which ? t.B : t.A);
    int h = t.N;
    int64_t pw = 1;
    for (int l = 1; l < d; l++) pw *= 7;
    for (int l = 1; l <= d; l++) {
        const int64_t self = node / pw;  // this node's ancestor at level l
        const int j = (int)(self % 7);
        const int64_t parent = self / 7;
        h >>= 1;
        int s = -1;
        if (which == 0) {
            if (j == 0) v = wt_quad(v, 0, 0, h);
            else if (j == 1) v = wt_quad(v, 0, 1, h);
            else if (j == 3) v = wt_quad(v, 1, 1, h);
            else s = j == 2 ? 3 : j - 4;
        } else {
            if (j == 0) v = wt_quad(v, 0, 0, h);
            else if (j == 1) v = wt_quad(v, 1, 0, h);
            else if (j == 2) v = wt_quad(v, 1, 1, h);
            else s = j == 3 ? 3 : j - 4;
        }
        if (s >= 0)
            v = which ? wt_dense(t.sb_limbs[l], t.sb_sizes[l], 4 * parent + s, h, t.capSB)
                      : wt_dense(t.sa_limbs[l], t.sa_sizes[l], 4 * parent + s, h, t.capSA);
        pw /= 7;
    }
    return v;
}

// Level d's sums: one thread per (operand side, parent, entry of the h x h quadrants).
__global__ void k_wino_sums(WinoTree t, int d, int64_t nparents, int h, uint32_t *err) {
    const int64_t hh = (int64_t)h * h;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 2 * nparents * hh) return;
    const int64_t e = idx % hh, rest = idx / hh;
    const int64_t p = rest % nparents;
    const int which = (int)(rest / nparents);
    const MatArgs par = wt_operand(t, which, d - 1, p);
    const int64_t ip = (e / h) * par.rs + e % h;  // the entry inside each quadrant of the parent
    const MatArgs x11 = wt_quad(par, 0, 0, h), x12 = wt_quad(par, 0, 1, h), x21 = wt_quad(par, 1, 0, h),
                  x22 = wt_quad(par, 1, 1, h);
    uint32_t *L = which ? t.sb_limbs[d] : t.sa_limbs[d];
    int32_t *S = which ? t.sb_sizes[d] : t.sa_sizes[d];
    const int cap = which ? t.capSB : t.capSA;
    const MatArgs o0 = wt_dense(L, S, 4 * p + 0, h, cap), o1 = wt_dense(L, S, 4 * p + 1, h, cap),
                  o2 = wt_dense(L, S, 4 * p + 2, h, cap), o3 = wt_dense(L, S, 4 * p + 3, h, cap);
    if (!which) {
        addsub_entry(o0, e, x21, ip, x22, ip, 0, err);  // S1 = A21 + A22
        addsub_entry(o1, e, o0, e, x11, ip, 1, err);    // S2 = S1 - A11
        addsub_entry(o2, e, x11, ip, x21, ip, 1, err);  // S3 = A11 - A21
        addsub_entry(o3, e, x12, ip, o1, e, 1, err);    // S4 = A12 - S2
    } else {
        addsub_entry(o0, e, x12, ip, x11, ip, 1, err);  // T1 = B12 - B11
        addsub_entry(o1, e, x22, ip, o0, e, 1, err);    // T2 = B22 - T1
        addsub_entry(o2, e, x22, ip, x12, ip, 1, err);  // T3 = B22 - B12
        addsub_entry(o3, e, x21, ip, o1, e, 1, err);    // T4' = B21 - T2
    }
}

// All leaf products of the tree: one CTA per (leaf, TY x TX tile of its output).
template <int R, int NT, bool THIN>
__global__ void __launch_bounds__(NT, NT <= MM_THREADS ? 2 : 1)
    k_wino_leaves(WinoTree t, MMCfg cfg, int ny, int nx, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int64_t tiles = (int64_t)ny * nx;
    const int64_t node = blockIdx.x / tiles;
    const int rem = (int)(blockIdx.x % tiles);
    const int L = t.levels, h = t.N >> L;
    const MatArgs A = wt_operand(t, 0, L, node), B = wt_operand(t, 1, L, node);
    const MatArgs C = wt_dense(t.p_limbs[L], t.p_sizes[L], node, h, t.capP);
    limb_tile<R, THIN>(C, A, B, cfg, rem / nx, rem % nx, smem_raw, err);
}

// Level d's products combined into their parents' outputs (level d - 1): one
// thread per (parent, entry of the h x h quadrants).  Quadrant entries are
// written in place in the order that needs no temporary.
__global__ void k_wino_combine(WinoTree t, int d, int64_t nparents, int h, uint32_t *err) {
    const int64_t hh = (int64_t)h * h;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nparents * hh) return;
    const int64_t e = idx % hh, p = idx / hh;
    const MatArgs Cp = d == 1 ? margs(t.C) : wt_dense(t.p_limbs[d - 1], t.p_sizes[d - 1], p, 2 * h, t.capP);
    const int64_t ic = (e / h) * Cp.rs + e % h;
    const MatArgs c11 = wt_quad(Cp, 0, 0, h), c12 = wt_quad(Cp, 0, 1, h), c21 = wt_quad(Cp, 1, 0, h),
                  c22 = wt_quad(Cp, 1, 1, h);
    MatArgs M[7];
#pragma unroll
    for (int j = 0; j < 7; j++) M[j] = wt_dense(t.p_limbs[d], t.p_sizes[d], 7 * p + j, h, t.capP);
    addsub_entry(c11, ic, M[0], e, M[1], e, 0, err);    // C11 = M1 + M2
    addsub_entry(c12, ic, M[0], e, M[5], e, 0, err);    // U2 = M1 + M6
    addsub_entry(c21, ic, c12, ic, M[6], e, 0, err);    // U3 = U2 + M7
    addsub_entry(c22, ic, c21, ic, M[4], e, 0, err);    // C22 = U3 + M5
    addsub_entry(c21, ic, c21, ic, M[3], e, 0, err);    // C21 = U3 + M4'
    addsub_entry(c12, ic, c12, ic, M[4], e, 0, err);    // U4 = U2 + M5
    addsub_entry(c12, ic, c12, ic, M[2], e, 0, err);    // C12 = U4 + M3
}

// Throughput probe for the per-entry product kernels' roofline: every thread runs
// the 8 x 8 block of 96-bit column multiply-accumulates (MAC96, the inner step of
// limb_tile at R = 8) on register operands, `iters` times, with no memory traffic.
// blocks x 256 x iters x 64 MACs per launch; the rate it reaches is the best the
// product kernels' MAC sequence can do on this GPU.
__global__ void __launch_bounds__(256) k_mac_peak(uint32_t *out, int iters, uint32_t seed) {
    uint32_t a[8], b[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        a[i] = seed * (threadIdx.x + 1) + (uint32_t)i * 0x9E3779B9u;
        b[i] = (seed ^ blockIdx.x) * 0x85EBCA6Bu + (uint32_t)i * 0xC2B2AE35u;
    }
    uint32_t P[15][3];
#pragma unroll
    for (int c = 0; c < 15; c++) P[c][0] = P[c][1] = P[c][2] = 0;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++) MAC96(P[i + j][0], P[i + j][1], P[i + j][2], a[i], b[j]);
        a[0] ^= P[0][0];
    }
    uint32_t acc = 0;
#pragma unroll
    for (int c = 0; c < 15; c++) acc ^= P[c][0] ^ P[c][1] ^ P[c][2];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// ---- host launchers ---------------------------------------------------------------------
static inline int64_t nentries(const gbmm_mat &m) { return (int64_t)m.rows * m.cols; }
static inline unsigned grid1(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }
// CTA size of the on-chip mpn products for `words` shared-memory words per
// operand: the largest of 128, 64, 32 whose staging fits, 0 when none does
constexpr size_t MPN_SM_MAX_BYTES = 200 * 1024;
static int sm_threads(size_t words) {
    for (int nt = 128; nt >= 32; nt >>= 1)
        if ((size_t)nt * words * 4 <= MPN_SM_MAX_BYTES) return nt;
    return 0;
}
bool mpn_basecase_on_chip(int un, int vn) { return sm_threads((size_t)sm_stride(un) + sm_stride(vn)) != 0; }
// whether limb planes at p with stride ld allow 16-byte loads of four operands
static int vec16(const void *p, int64_t ld) { return ((uintptr_t)p % 16 == 0 && ld % 4 == 0) ? 1 : 0; }

gbmm_status launch_mat_addsub(const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int sub, cudaStream_t s) {
    const int64_t n = nentries(c);
    if (n == 0) return GBMM_OK;
    LaunchScope ls_("k_mpz_addsub", s);
    k_mpz_addsub<<<grid1(n, 256), 256, 0, s>>>(margs(c), margs(a), margs(b), sub, n, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_mat_zero(const gbmm_mat &c, cudaStream_t s) {
    const int64_t n = nentries(c);
    if (n == 0) return GBMM_OK;
    LaunchScope ls_("k_mat_zero", s);
    k_mat_zero<<<grid1(n, 256), 256, 0, s>>>(margs(c), n);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_mat_copy(const gbmm_mat &dst, const gbmm_mat &src, cudaStream_t s) {
    const int64_t n = nentries(dst);
    if (n == 0) return GBMM_OK;
    LaunchScope ls_("k_mat_copy", s);
    k_mat_copy<<<grid1(n, 256), 256, 0, s>>>(margs(dst), margs(src), n, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_split_sizes(const gbmm_mat &x, int h, int32_t *lo, int32_t *hi, cudaStream_t s) {
    const int64_t n = nentries(x);
    if (n == 0) return GBMM_OK;
    LaunchScope ls_("k_split_sizes", s);
    k_split_sizes<<<grid1(n, 256), 256, 0, s>>>(margs(x), h, lo, hi, n);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_add_shifted(const gbmm_mat &w, const gbmm_mat &u, const gbmm_mat &v, int sh, cudaStream_t s) {
    const int64_t n = nentries(w);
    if (n == 0) return GBMM_OK;
    // one thread per entry keeps enough loads in flight once there are many entries
    // (75k entries of 660 planes: 0.33 ms, against 0.49 ms segmented); fewer entries
    // take the segmented form (27k entries: 0.22 ms, against 0.29 ms)
    if (n >= ADDSH_SEG_BELOW) {
        LaunchScope ls_("k_add_shifted", s);
        k_add_shifted<<<grid1(n, 256), 256, 0, s>>>(margs(w), margs(u), margs(v), sh, n, device_error_word());
    } else {
        LaunchScope ls_("k_add_shifted_seg", s);
        k_add_shifted_seg<<<grid1(n, 32), 32 * ADDSH_SEGS, 0, s>>>(margs(w), margs(u), margs(v), sh, n,
                                                                    device_error_word());
    }
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_max_size(const gbmm_mat &a, int32_t *d_out, cudaStream_t s) {
    const int64_t n = nentries(a);
    GBMM_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(int32_t), s));
    if (n == 0) return GBMM_OK;
    LaunchScope ls_("k_max_size", s);
    k_max_size<<<grid1(n, 256), 256, 0, s>>>(margs(a), n, d_out);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_mpz_mulops(const gbmm_mat &w, const gbmm_mat &u, const gbmm_mat &v, int op, cudaStream_t s) {
    const int64_t n = nentries(w);
    if (n == 0) return GBMM_OK;
    LaunchScope ls_("k_mpz_mulops", s);
    k_mpz_mulops<<<grid1(n, 128), 128, 0, s>>>(margs(w), margs(u), margs(v), op, n, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

static int roundup(int x, int m) { return (x + m - 1) / m * m; }

// Launches LAUNCH(R, NT, THIN) for a configuration: the block edge, one group
// per CTA of up to 512 threads (R = 8) or CTAs of at most 256, and whether an
// operand is thin (the edge threads fold in a single top limb).
#define LIMB_DISPATCH(cfg_, LAUNCH)                                              \
    do {                                                                         \
        const bool th_ = (cfg_).thinA || (cfg_).thinB;                           \
        if ((cfg_).NT > MM_THREADS) {                                            \
            if (th_) LAUNCH(8, MM_THREADS_WIDE, true);                           \
            else LAUNCH(8, MM_THREADS_WIDE, false);                              \
        } else if (th_) {                                                        \
            switch ((cfg_).R) {                                                  \
                case 2: LAUNCH(2, MM_THREADS, true); break;                      \
                case 4: LAUNCH(4, MM_THREADS, true); break;                      \
                default: LAUNCH(8, MM_THREADS, true); break;                     \
            }                                                                    \
        } else {                                                                 \
            switch ((cfg_).R) {                                                  \
                case 1: LAUNCH(1, MM_THREADS, false); break;                     \
                case 2: LAUNCH(2, MM_THREADS, false); break;                     \
                case 4: LAUNCH(4, MM_THREADS, false); break;                     \
                default: LAUNCH(8, MM_THREADS, false); break;                    \
            }                                                                    \
        }                                                                        \
    } while (0)

// Picks the block edge R and group size for limb counts la x lb.  An operand
// of one limb past a multiple of R (and longer than R) is "thin": its top limb's
// products are spread over the main grid's threads as extra items, so the group
// is the main grid alone (a one-limb-longer Winograd sum of 128-limb entries
// keeps 16 x 16 threads).  Groups of up to 256 threads share 256-thread CTAs; a group of
// 257..512 threads (entries of up to about 176 limbs) gets a CTA of its own.
static bool try_block(int la, int lb, int R, int gmin, int gmax, MMCfg &cfg) {
    int tA = R > 1 && la > R && la % R == 1, tB = R > 1 && lb > R && lb % R == 1;
    const int pa = roundup(la, R), pb = roundup(lb, R);
    int G = (pa / R - tA) * (pb / R - tB);
    // top-limb items of the thin operands: at most MM_XMAX a thread, else whole blocks
    const int nx = tA * ((pb / R - tB) * R + tB) + tB * (pa / R - tA) * R;
    if ((tA || tB) && nx > MM_XMAX * G) {
        tA = tB = 0;
        G = (pa / R) * (pb / R);
    }
    if (G < gmin || G > gmax) return false;
    cfg.R = R; cfg.La = pa; cfg.Lb = pb; cfg.G = G; cfg.Gp = roundup(G, 32);
    cfg.thinA = tA; cfg.thinB = tB;
    cfg.NT = cfg.Gp > MM_THREADS ? cfg.Gp : MM_THREADS;
    return true;
}
static bool choose_mm(int la, int lb, MMCfg &cfg) {
    la = la < 1 ? 1 : la;
    lb = lb < 1 ? 1 : lb;
    const int cand[3] = {8, 4, 2};
    for (int ci = 0; ci < 3; ci++)
        if (try_block(la, lb, cand[ci], 32, MM_THREADS, cfg)) return true;
    const int mx = la > lb ? la : lb;
    if (mx <= 8) {
        const int R = mx <= 1 ? 1 : mx <= 2 ? 2 : mx <= 4 ? 4 : 8;
        cfg.R = R; cfg.La = R; cfg.Lb = R; cfg.G = 1; cfg.Gp = 1; cfg.NT = MM_THREADS;
        cfg.thinA = cfg.thinB = 0;
        return true;
    }
    if (try_block(la, lb, 2, 1, MM_THREADS, cfg)) return true;
    return try_block(la, lb, 8, MM_THREADS + 1, MM_THREADS_WIDE, cfg);
}

// Entries per CTA and their TY x TX arrangement for a chosen group size; the CTA
// has exactly EPC x Gp threads.
static void finish_cfg(MMCfg &cfg, int M, int accumulate) {
    const int EPC = cfg.Gp >= cfg.NT ? 1 : cfg.NT / cfg.Gp;
    if (cfg.Gp < cfg.NT) cfg.NT = EPC * cfg.Gp;
    int TY = 1;
    while (TY * TY * 4 <= EPC) TY *= 2;
    cfg.TY = TY;
    cfg.TX = EPC / TY;
    cfg.TXs = 0;
    while ((1 << cfg.TXs) < cfg.TX) cfg.TXs++;
    cfg.M = M;
    cfg.accumulate = accumulate;
}

bool limb_kernel_fits(int la, int lb) {
    MMCfg cfg;
    return choose_mm(la, lb, cfg);
}

static size_t mm_smem(const MMCfg &c) {
    // two staging buffers (double-buffered chunks), or the reduction's buffers after the loop
    size_t stage = 2 * ((size_t)c.TY * MM_KC * (c.La + 4) * 4 + (size_t)MM_KC * c.TX * (c.Lb + 4) * 4 +
                        (size_t)(c.TY + c.TX) * MM_KC * 4);
    const int EPC = c.TY * c.TX, Lc = c.La + c.Lb, NC = 2 * c.R - 1 + ((c.thinA || c.thinB) ? MM_XMAX : 0);
    size_t red = (size_t)EPC * c.G * NC * 3 * 4 + 8 + (size_t)EPC * Lc * 3 * 8 + (size_t)EPC * (Lc + 2) * 4;
    return stage > red ? stage : red;
}

gbmm_status launch_limb_matmul(const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int accumulate,
                               cudaStream_t s) {
    if (c.rows == 0 || c.cols == 0) return GBMM_OK;
    if (a.cols == 0) {
        if (accumulate) return GBMM_OK;
        return launch_mat_zero(c, s);
    }
    MMCfg cfg;
    if (!choose_mm(a.nlimbs, b.nlimbs, cfg))
        return set_error(GBMM_ERR_UNSUPPORTED, "limb matmul: %d x %d limb entries exceed the per-entry kernel", a.nlimbs,
                         b.nlimbs);
    finish_cfg(cfg, a.cols, accumulate);
    size_t smem = mm_smem(cfg);
    if (smem > 200 * 1024) return set_error(GBMM_ERR_UNSUPPORTED, "limb matmul: shared memory %zu too large", smem);
    dim3 grid((unsigned)((c.cols + cfg.TX - 1) / cfg.TX), (unsigned)((c.rows + cfg.TY - 1) / cfg.TY));
    uint32_t *err = device_error_word();
#define LAUNCH_R(RR, NTT, TH)                                                                          \
    do {                                                                                               \
        if (smem > 48 * 1024)                                                                          \
            GBMM_CUDA_TRY(cudaFuncSetAttribute(k_limb_matmul<RR, NTT, TH>,                             \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
        LaunchScope ls_("k_limb_matmul", s);                                                            \
        k_limb_matmul<RR, NTT, TH><<<grid, cfg.NT, smem, s>>>(margs(c), margs(a), margs(b), cfg, err); \
    } while (0)
    LIMB_DISPATCH(cfg, LAUNCH_R);
#undef LAUNCH_R
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

static int occupancy_ctas(const void *fn, int nt, size_t smem) {
    int n = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, nt, smem) != cudaSuccess || n < 1) n = 1;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return n * (sms > 0 ? sms : 148);
}

gbmm_status plan_limb_batch(const std::vector<gbmm_mat> &C, const std::vector<gbmm_mat> &A,
                            const std::vector<gbmm_mat> &B, LimbBatchPlan &plan) {
    struct Item {
        int job, by, bx;
        double cost;
    };
    // groups (one launch each): block edge 1, 2, 4, 8 on 256-thread CTAs and 8 with
    // one wide group per CTA, each with and without a thin operand
    constexpr int NG = LimbBatchPlan::MAX_GROUPS;
    const int Rs[NG] = {1, 1, 2, 2, 4, 4, 8, 8, 8, 8};
    std::vector<LimbJob> jobs[NG];
    std::vector<Item> items[NG];
    size_t smem[NG] = {};
    int nts[NG];
    for (int g = 0; g < NG; g++) nts[g] = g < 8 ? MM_THREADS : 0;
    for (size_t i = 0; i < C.size(); i++) {
        MMCfg cfg;
        if (!choose_mm(A[i].nlimbs, B[i].nlimbs, cfg))
            return set_error(GBMM_ERR_UNSUPPORTED, "batched limb job %zu: entries too long", i);
        finish_cfg(cfg, A[i].cols, 0);
        const int thin = (cfg.thinA || cfg.thinB) ? 1 : 0;
        int g = 0;
        if (cfg.NT > MM_THREADS) {
            // one launch of the wide group kernel runs with a single CTA size
            g = 8 + thin;
            nts[g] = std::max(nts[g], cfg.NT);
        } else {
            g = (cfg.R == 1 ? 0 : cfg.R == 2 ? 2 : cfg.R == 4 ? 4 : 6) + thin;
        }
        smem[g] = std::max(smem[g], mm_smem(cfg));
        LimbJob lj;
        lj.C = margs(C[i]); lj.A = margs(A[i]); lj.B = margs(B[i]); lj.cfg = cfg;
        const int jid = (int)jobs[g].size();
        jobs[g].push_back(lj);
        const int ny = (C[i].rows + cfg.TY - 1) / cfg.TY, nx = (C[i].cols + cfg.TX - 1) / cfg.TX;
        const double cost = (double)cfg.TY * cfg.TX * cfg.La * cfg.Lb * cfg.M;
        for (int by = 0; by < ny; by++)
            for (int bx = 0; bx < nx; bx++) items[g].push_back(Item{jid, by, bx, cost});
    }
    plan.blob.clear();
    plan.groups.clear();
    for (int g = 0; g < NG; g++) {
        if (jobs[g].empty()) continue;
        if (smem[g] > 200 * 1024) return set_error(GBMM_ERR_UNSUPPORTED, "batched limb: shared memory too large");
        std::stable_sort(items[g].begin(), items[g].end(), [](const Item &x, const Item &y) { return x.cost > y.cost; });
        LimbBatchPlan::Group gr;
        gr.R = Rs[g];
        gr.NT = nts[g];
        gr.thin = g & 1;
        for (auto &j : jobs[g]) j.cfg.NT = nts[g];
        gr.smem = smem[g];
        gr.nitems = (int)items[g].size();
        size_t off = (plan.blob.size() + 255) & ~(size_t)255;
        gr.jobs_off = off;
        plan.blob.resize(off + jobs[g].size() * sizeof(LimbJob));
        memcpy(plan.blob.data() + off, jobs[g].data(), jobs[g].size() * sizeof(LimbJob));
        off = (plan.blob.size() + 255) & ~(size_t)255;
        gr.items_off = off;
        plan.blob.resize(off + items[g].size() * 3 * sizeof(int));
        int *ip = reinterpret_cast<int *>(plan.blob.data() + off);
        for (size_t t = 0; t < items[g].size(); t++) {
            ip[3 * t] = items[g][t].job;
            ip[3 * t + 1] = items[g][t].by;
            ip[3 * t + 2] = items[g][t].bx;
        }
        plan.groups.push_back(gr);
    }
    return GBMM_OK;
}

gbmm_status launch_limb_batch(const LimbBatchPlan &plan, const char *d_blob, int *d_counters, cudaStream_t s) {
    if (plan.groups.empty()) return GBMM_OK;
    GBMM_CUDA_TRY(cudaMemsetAsync(d_counters, 0, sizeof(int) * plan.groups.size(), s));
    uint32_t *err = device_error_word();
    for (size_t g = 0; g < plan.groups.size(); g++) {
        const LimbBatchPlan::Group &gr = plan.groups[g];
        const LimbJob *jobs = reinterpret_cast<const LimbJob *>(d_blob + gr.jobs_off);
        const int *items = reinterpret_cast<const int *>(d_blob + gr.items_off);
#define LAUNCH_B(RR, NTT, TH)                                                                             \
    do {                                                                                                  \
        if (gr.smem > 48 * 1024)                                                                          \
            GBMM_CUDA_TRY(cudaFuncSetAttribute(k_limb_batched<RR, NTT, TH>,                               \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gr.smem)); \
        const int grid =                                                                                  \
            std::min(gr.nitems, occupancy_ctas((const void *)k_limb_batched<RR, NTT, TH>, gr.NT, gr.smem)); \
        LaunchScope ls_("k_limb_batched", s);                                                             \
        k_limb_batched<RR, NTT, TH><<<grid, gr.NT, gr.smem, s>>>(jobs, items, gr.nitems, d_counters + g, err); \
    } while (0)
        MMCfg gc;
        gc.R = gr.R;
        gc.NT = gr.NT;
        gc.thinA = gr.thin;
        gc.thinB = 0;
        LIMB_DISPATCH(gc, LAUNCH_B);
#undef LAUNCH_B
        GBMM_CUDA_TRY(cudaGetLastError());
    }
    return GBMM_OK;
}

static int64_t pow7(int d) {
    int64_t r = 1;
    while (d-- > 0) r *= 7;
    return r;
}

gbmm_status launch_wino_sums(const WinoTree &t, int d, cudaStream_t s) {
    const int64_t np = pow7(d - 1);
    const int h = t.N >> d;
    const int64_t n = 2 * np * h * h;
    LaunchScope ls_("k_wino_sums", s);
    k_wino_sums<<<grid1(n, 128), 128, 0, s>>>(t, d, np, h, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_wino_combine(const WinoTree &t, int d, cudaStream_t s) {
    const int64_t np = pow7(d - 1);
    const int h = t.N >> d;
    const int64_t n = np * h * h;
    LaunchScope ls_("k_wino_combine", s);
    k_wino_combine<<<grid1(n, 128), 128, 0, s>>>(t, d, np, h, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

gbmm_status launch_wino_leaves(const WinoTree &t, cudaStream_t s) {
    const int h = t.N >> t.levels;
    MMCfg cfg;
    if (!choose_mm(t.capSA, t.capSB, cfg))
        return set_error(GBMM_ERR_UNSUPPORTED, "winograd leaves: %d x %d limb operands exceed the per-entry kernel",
                         t.capSA, t.capSB);
    finish_cfg(cfg, h, 0);
    const size_t smem = mm_smem(cfg);
    if (smem > 200 * 1024) return set_error(GBMM_ERR_UNSUPPORTED, "winograd leaves: shared memory %zu too large", smem);
    const int ny = (h + cfg.TY - 1) / cfg.TY, nx = (h + cfg.TX - 1) / cfg.TX;
    const int64_t blocks = pow7(t.levels) * ny * nx;
    if (blocks > 0x7FFFFFFF) return set_error(GBMM_ERR_UNSUPPORTED, "winograd leaves: %lld tiles", (long long)blocks);
    uint32_t *err = device_error_word();
#define LAUNCH_W(RR, NTT, TH)                                                                          \
    do {                                                                                               \
        if (smem > 48 * 1024)                                                                          \
            GBMM_CUDA_TRY(cudaFuncSetAttribute(k_wino_leaves<RR, NTT, TH>,                             \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
        LaunchScope ls_("k_wino_leaves", s);                                                            \
        k_wino_leaves<RR, NTT, TH><<<(unsigned)blocks, cfg.NT, smem, s>>>(t, cfg, ny, nx, err);       \
    } while (0)
    LIMB_DISPATCH(cfg, LAUNCH_W);
#undef LAUNCH_W
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

}  // namespace gbmm

// ======================================================================================
// C ABI: batched mpn / mpz entry points
// ======================================================================================
using namespace gbmm;

static gbmm_status check_batch(const void *a, const void *b, int64_t ld, int64_t nb, int n) {
    if (!a || !b) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (nb < 0 || n < 0 || ld < nb) return set_error(GBMM_ERR_INVALID, "bad batch shape n=%d ld=%lld nb=%lld", n,
                                                     (long long)ld, (long long)nb);
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_mpn_add_n(uint32_t *rp, const uint32_t *up, const uint32_t *vp, int32_t n, int64_t ld,
                                      int64_t nb, uint32_t *cy, void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, n));
    if (!vp || !cy) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (nb == 0) return GBMM_OK;
    if (nb >= ADDSUB_SERIAL_MIN_OPS) {
        LaunchScope ls_("k_mpn_addsub_n_serial", as_stream(stream));
        k_mpn_addsub_n_serial<false><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, vp, n, ld, nb, cy);
    } else {
        LaunchScope ls_("k_mpn_addsub_n_cla", as_stream(stream));
        k_mpn_addsub_n_cla<false><<<grid1(nb, CLA_OPS), 256, 0, as_stream(stream)>>>(rp, up, vp, n, ld, nb, cy);
    }
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_sub_n(uint32_t *rp, const uint32_t *up, const uint32_t *vp, int32_t n, int64_t ld,
                                      int64_t nb, uint32_t *cy, void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, n));
    if (!vp || !cy) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (nb == 0) return GBMM_OK;
    if (nb >= ADDSUB_SERIAL_MIN_OPS) {
        LaunchScope ls_("k_mpn_addsub_n_serial", as_stream(stream));
        k_mpn_addsub_n_serial<true><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, vp, n, ld, nb, cy);
    } else {
        LaunchScope ls_("k_mpn_addsub_n_cla", as_stream(stream));
        k_mpn_addsub_n_cla<true><<<grid1(nb, CLA_OPS), 256, 0, as_stream(stream)>>>(rp, up, vp, n, ld, nb, cy);
    }
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
template <int OP>
static gbmm_status mul1_entry(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld, int64_t nb,
                              uint32_t *cy, void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, n));
    if (!vl || !cy) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_mul1ops", as_stream(stream));
    k_mpn_mul1ops<OP><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, n, vl, ld, nb, cy);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_mul_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                                      int64_t nb, uint32_t *cy, void *stream) {
    return mul1_entry<0>(rp, up, n, vl, ld, nb, cy, stream);
}
extern "C" gbmm_status gbmm_mpn_addmul_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                                         int64_t nb, uint32_t *cy, void *stream) {
    return mul1_entry<1>(rp, up, n, vl, ld, nb, cy, stream);
}
extern "C" gbmm_status gbmm_mpn_submul_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                                         int64_t nb, uint32_t *cy, void *stream) {
    return mul1_entry<2>(rp, up, n, vl, ld, nb, cy, stream);
}
// Internal probe (not part of the public ABI): one launch of k_mac_peak, blocks x 256
// threads, each doing iters x 64 MACs; out holds blocks x 256 words.
extern "C" gbmm_status gbmmx_mac_peak(uint32_t *out, int32_t blocks, int32_t iters, void *stream) {
    if (!out || blocks < 1 || iters < 1) return set_error(GBMM_ERR_INVALID, "mac peak: bad arguments");
    LaunchScope ls_("k_mac_peak", as_stream(stream));
    k_mac_peak<<<blocks, 256, 0, as_stream(stream)>>>(out, iters, 0x2545F491u);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_mpn_add(uint32_t *rp, const uint32_t *up, int32_t un, const uint32_t *vp, int32_t vn,
                                    int64_t ld, int64_t nb, uint32_t *cy, void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, un));
    if ((!vp && vn > 0) || !cy) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (un < vn || vn < 0 || un < 1) return set_error(GBMM_ERR_INVALID, "mpn_add needs un >= vn >= 0, un >= 1");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_addsub", as_stream(stream));
    k_mpn_addsub<false><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, un, vp, vn, ld, nb, cy);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_sub(uint32_t *rp, const uint32_t *up, int32_t un, const uint32_t *vp, int32_t vn,
                                    int64_t ld, int64_t nb, uint32_t *cy, void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, un));
    if ((!vp && vn > 0) || !cy) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (un < vn || vn < 0 || un < 1) return set_error(GBMM_ERR_INVALID, "mpn_sub needs un >= vn >= 0, un >= 1");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_addsub", as_stream(stream));
    k_mpn_addsub<true><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, un, vp, vn, ld, nb, cy);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
template <bool SUB>
static gbmm_status addsub_1_entry(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                                  int64_t nb, uint32_t *cy, void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, n));
    if (!vl || !cy) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (n < 1) return set_error(GBMM_ERR_INVALID, "mpn_add_1 / mpn_sub_1 need n >= 1");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_addsub_1", as_stream(stream));
    k_mpn_addsub_1<SUB><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, n, vl, ld, nb, cy);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_add_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                                      int64_t nb, uint32_t *cy, void *stream) {
    return addsub_1_entry<false>(rp, up, n, vl, ld, nb, cy, stream);
}
extern "C" gbmm_status gbmm_mpn_sub_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                                      int64_t nb, uint32_t *cy, void *stream) {
    return addsub_1_entry<true>(rp, up, n, vl, ld, nb, cy, stream);
}
extern "C" gbmm_status gbmm_mpn_cmp(const uint32_t *up, const uint32_t *vp, int32_t n, int64_t ld, int64_t nb,
                                    int32_t *result, void *stream) {
    GBMM_TRY(check_batch(up, vp, ld, nb, n));
    if (!result) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_cmp", as_stream(stream));
    k_mpn_cmp<<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(up, vp, n, ld, nb, result);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_zero_p(const uint32_t *up, int32_t n, int64_t ld, int64_t nb, int32_t *result,
                                       void *stream) {
    GBMM_TRY(check_batch(up, result, ld, nb, n));
    if (n < 1) return set_error(GBMM_ERR_INVALID, "mpn_zero_p needs n >= 1");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_zero_p", as_stream(stream));
    k_mpn_zero_p<<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(up, n, ld, nb, result);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_neg(uint32_t *rp, const uint32_t *up, int32_t n, int64_t ld, int64_t nb, uint32_t *cy,
                                    void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, n));
    if (!cy) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (n < 1) return set_error(GBMM_ERR_INVALID, "mpn_neg needs n >= 1");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_neg_com", as_stream(stream));
    k_mpn_neg_com<true><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, n, ld, nb, cy);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_com(uint32_t *rp, const uint32_t *up, int32_t n, int64_t ld, int64_t nb,
                                    void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, n));
    if (n < 1) return set_error(GBMM_ERR_INVALID, "mpn_com needs n >= 1");
    if (nb == 0) return GBMM_OK;
    LaunchScope ls_("k_mpn_neg_com", as_stream(stream));
    k_mpn_neg_com<false><<<grid1(nb, 256), 256, 0, as_stream(stream)>>>(rp, up, n, ld, nb, nullptr);
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_mul_basecase(uint32_t *rp, const uint32_t *up, int32_t un, const uint32_t *vp,
                                             int32_t vn, int64_t ld, int64_t nb, void *stream) {
    GBMM_TRY(check_batch(rp, up, ld, nb, un));
    if (!vp) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (un < vn || vn < 1) return set_error(GBMM_ERR_INVALID, "mul_basecase needs un >= vn >= 1 (un=%d vn=%d)", un, vn);
    if (nb == 0) return GBMM_OK;
    const int nt = sm_threads((size_t)sm_stride(un) + sm_stride(vn));
    if (nt == 0) {
        // operands too long to stage: the product reads them from global memory
        LaunchScope ls_("k_mpn_mul_basecase", as_stream(stream));
        k_mpn_mul_basecase<<<grid1(nb, 128), 128, 0, as_stream(stream)>>>(rp, up, un, vp, vn, ld, nb);
        GBMM_CUDA_TRY(cudaGetLastError());
        return GBMM_OK;
    }
    const size_t smem = (size_t)nt * (sm_stride(un) + sm_stride(vn)) * 4;
    const int vu = vec16(up, ld), vv = vec16(vp, ld);
    LaunchScope ls_("k_mpn_mul_basecase_sm", as_stream(stream));
#define BASECASE_SM(NT_)                                                                                      \
    do {                                                                                                      \
        GBMM_CUDA_TRY(cudaFuncSetAttribute(k_mpn_mul_basecase_sm<NT_>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                           (int)smem));                                                       \
        k_mpn_mul_basecase_sm<NT_><<<grid1(nb, NT_), NT_, smem, as_stream(stream)>>>(rp, up, un, vp, vn, ld, nb, vu, \
                                                                                     vv);                      \
    } while (0)
    if (nt == 128) BASECASE_SM(128);
    else if (nt == 64) BASECASE_SM(64);
    else BASECASE_SM(32);
#undef BASECASE_SM
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
// 6n + 2 scratch limbs per operand (n = an - floor(an/2)), or -1 when that count
// does not fit an int32 (an above about 7.1e8 limbs): callers reject those sizes.
static int64_t toom22_itch64(int32_t an) {
    const int64_t n = (int64_t)an - (an >> 1);
    return 6 * n + 2;
}
extern "C" int32_t gbmm_mpn_toom22_mul_itch(int32_t an, int32_t bn) {
    (void)bn;
    const int64_t itch = toom22_itch64(an);
    return itch > INT32_MAX ? -1 : (int32_t)itch;
}
// Toom-2.2 on chip when the per-operand intermediates fit shared memory (the
// scratch planes are then not touched), else through the scratch planes.
static gbmm_status launch_toom22(uint32_t *pp, const uint32_t *ap, int an, const uint32_t *bp, int bn,
                                 uint32_t *scratch, int64_t ld, int64_t nb, cudaStream_t s) {
    const int nt = sm_threads((size_t)toom22_sm_words(an, bn));
    if (nt == 0) {
        LaunchScope ls_("k_mpn_toom22", s);
        k_mpn_toom22<<<grid1(nb, 128), 128, 0, s>>>(pp, ap, an, bp, bn, scratch, ld, nb);
        GBMM_CUDA_TRY(cudaGetLastError());
        return GBMM_OK;
    }
    const size_t smem = (size_t)nt * toom22_sm_words(an, bn) * 4;
    const int va = vec16(ap, ld), vb = vec16(bp, ld);
    LaunchScope ls_("k_mpn_toom22_sm", s);
#define TOOM22_SM(NT_)                                                                                          \
    do {                                                                                                        \
        GBMM_CUDA_TRY(cudaFuncSetAttribute(k_mpn_toom22_sm<NT_>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                           (int)smem));                                                         \
        k_mpn_toom22_sm<NT_><<<grid1(nb, NT_), NT_, smem, s>>>(pp, ap, an, bp, bn, ld, nb, va, vb);             \
    } while (0)
    if (nt == 128) TOOM22_SM(128);
    else if (nt == 64) TOOM22_SM(64);
    else TOOM22_SM(32);
#undef TOOM22_SM
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpn_toom22_mul(uint32_t *pp, const uint32_t *ap, int32_t an, const uint32_t *bp, int32_t bn,
                                           uint32_t *scratch, int64_t ld, int64_t nb, void *stream) {
    GBMM_TRY(check_batch(pp, ap, ld, nb, an));
    if (!bp || !scratch) return set_error(GBMM_ERR_INVALID, "null pointer");
    const int s = an >> 1, n = an - s, t = bn - n;
    if (an < bn || !(0 < s && s <= n && s >= n - 1) || !(0 < t && t <= s))
        return set_error(GBMM_ERR_INVALID, "toom22 preconditions violated (an=%d bn=%d)", an, bn);
    if (toom22_itch64(an) > INT32_MAX) return set_error(GBMM_ERR_INVALID, "toom22: an=%d is too long", an);
    if (nb == 0) return GBMM_OK;
    return launch_toom22(pp, ap, an, bp, bn, scratch, ld, nb, as_stream(stream));
}

// ---- Toom-2.2 without any allocation ---------------------------------------------------
// Scratch for gbmm_mpn_toom22_mul_noalloc lives in this file-scope device array:
// every GPU that loads the library holds it until the process exits, and all
// calls on a device share it.  Host code must not pass `g_toom22_scratch`
// itself to a kernel (on the host that name is only a stand-in for the device
// symbol); its device address is looked up once per device with
// cudaGetSymbolAddress and cached below.
static __device__ __align__(256) uint32_t g_toom22_scratch[GBMM_NOALLOC_SCRATCH_BYTES / 4];

static std::mutex g_noalloc_mu;
static uint32_t *g_noalloc_ptr[64];

// Looks up the device address of the scratch array for the current device
// (first call on each device; no allocation happens).
static gbmm_status noalloc_scratch(uint32_t **out) {
    int dev = 0;
    GBMM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(GBMM_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_toom22_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_toom22_scratch)");
        g_noalloc_ptr[dev] = static_cast<uint32_t *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_mpn_toom22_mul_noalloc(uint32_t *pp, const uint32_t *ap, int32_t an, const uint32_t *bp,
                                                   int32_t bn, int64_t ld, int64_t nb, void *stream) {
    GBMM_TRY(check_batch(pp, ap, ld, nb, an));
    if (!bp) return set_error(GBMM_ERR_INVALID, "null pointer");
    const int s = an >> 1, n = an - s, t = bn - n;
    if (an < bn || !(0 < s && s <= n && s >= n - 1) || !(0 < t && t <= s))
        return set_error(GBMM_ERR_INVALID, "toom22 preconditions violated (an=%d bn=%d)", an, bn);
    const int64_t itch = toom22_itch64(an);  // 64-bit: no wrap for any int32 an
    const double need_d = (double)itch * (double)ld * 4.0;
    const uint64_t need = need_d > 1e18 ? UINT64_MAX : (uint64_t)itch * (uint64_t)ld * 4u;
    if (need > GBMM_NOALLOC_SCRATCH_BYTES)
        return set_error(GBMM_ERR_CAPACITY,
                         "toom22 without allocation: scratch of %llu bytes (itch %lld limbs x plane stride %lld) exceeds "
                         "the fixed %d-byte device array",
                         (unsigned long long)need, (long long)itch, (long long)ld,
                         GBMM_NOALLOC_SCRATCH_BYTES);
    if (nb == 0) return GBMM_OK;
    uint32_t *scratch = nullptr;
    GBMM_TRY(noalloc_scratch(&scratch));
    // every scratch word the kernel reads it has written first in the same call,
    // so nothing is cleared between calls
    return launch_toom22(pp, ap, an, bp, bn, scratch, ld, nb, as_stream(stream));
}

static gbmm_status check_elementwise(const gbmm_mat &w, const gbmm_mat &u, const gbmm_mat &v) {
    GBMM_TRY(validate_mat(w, "w"));
    GBMM_TRY(validate_mat(u, "u"));
    GBMM_TRY(validate_mat(v, "v"));
    if (u.rows != w.rows || v.rows != w.rows || u.cols != w.cols || v.cols != w.cols)
        return set_error(GBMM_ERR_INVALID, "elementwise shapes differ");
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mpz_add(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream) {
    GBMM_TRY(check_elementwise(w, u, v));
    return launch_mat_addsub(w, u, v, 0, as_stream(stream));
}
extern "C" gbmm_status gbmm_mpz_sub(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream) {
    GBMM_TRY(check_elementwise(w, u, v));
    return launch_mat_addsub(w, u, v, 1, as_stream(stream));
}
static gbmm_status mulops_entry(gbmm_mat w, gbmm_mat u, gbmm_mat v, int op, void *stream) {
    GBMM_TRY(check_elementwise(w, u, v));
    if (w.limbs == u.limbs || w.limbs == v.limbs)
        return set_error(GBMM_ERR_INVALID, "mpz mul: w must not alias u or v (as gpu_mpz_mul, mpz-mul.cu:97-101)");
    return launch_mpz_mulops(w, u, v, op, as_stream(stream));
}
extern "C" gbmm_status gbmm_mpz_mul(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream) {
    return mulops_entry(w, u, v, 0, stream);
}
extern "C" gbmm_status gbmm_mpz_addmul(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream) {
    return mulops_entry(w, u, v, 1, stream);
}
extern "C" gbmm_status gbmm_mpz_submul(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream) {
    return mulops_entry(w, u, v, 2, stream);
}
