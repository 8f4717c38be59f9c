// Multi-modular (CRT) form of the exact product C = A * B on the tcgen05
// tensor cores.
//
// Moduli: the P largest primes below 2^16 with prod p_i = Mod > 2^(bitsA +
// bitsB + log2 k + 18).  Every GEMM below multiplies signed 8-bit digits held
// exactly in bf16 and accumulates in FP32; each accumulation is bounded so that
// every partial sum is an integer of magnitude < 2^24, hence exact.
//
//  1. digits    : limb planes -> rows of byte digits (bf16): unsigned bytes, or for
//                 rows longer than 512 digits balanced digits in [-128, 128]; one
//                 row per entry (A in row-major order, B in column-major order).
//  2. residue   : [entries x digits] x [digits x 2P] GEMM with the table
//                 256^j mod p_i (balanced, split in two signed bytes); the
//                 epilogue folds the two halves, reduces mod p_i in FP32,
//                 applies the entry's sign and stores the residue as two
//                 balanced digits in per-modulus planes.  B's table carries the
//                 CRT weight w_i = (Mod/p_i)^-1 mod p_i.
//  3. product   : for each modulus, A's two digit planes against B's two
//                 (pre-weighted) digit planes in four accumulators;
//                 y_i = 65536 a1 u1 + 256 (a1 u0 + a0 u1) + a0 u0 mod p_i, stored
//                 balanced as two digits in per-modulus planes.
//  4. reconstruct: [entries x 2P] x [2P x (32 + Dout)] GEMM against the digits
//                 of Mod/p_i (and 256*Mod/p_i) plus fixed-point digits of
//                 2^96/p_i; the epilogue gets q = round(sum y_i / p_i) and the
//                 sign of C, folds out q*Mod, carries across the digit columns
//                 and writes sign-magnitude limbs.  C = sum y_i Mod/p_i - q*Mod.
// The CRT itself is the textbook one (HAC 14.5, Knuth 4.3.2); the reference's
// crt.cpp (split / merge of one integer through a tree of coprime pairs) is
// unused by the reference and only the idea carries over.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <utility>
#include <cmath>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "gbmm_internal.h"
#include "tc.cuh"

namespace gbmm {

namespace {
constexpr int BM = 128;  // tile rows (TMEM lanes)
constexpr int BK = 64;   // bf16 elements per K step (one 128-byte swizzle row)
constexpr int UK = 16;   // K of one kind::f16 MMA
// residue GEMM: K steps per exact accumulation group: 8 (512 unsigned byte digits,
// 512 * 255 * 128 < 2^24) or, for rows longer than 512 digits, 15 (960 balanced
// digits, 959 * 128 * 128 + 256 * 128 < 2^24)
constexpr int RES_GROUP_STEPS_U = 8, RES_GROUP_STEPS_B = 15;
constexpr int PROD_MAX_K = 512;      // product GEMM: inner dimension of one exact pass
constexpr int SROWS = 32;       // columns before the first output digit in the reconstruction table
constexpr int SUSED = 14;       // of which the fixed-point sum uses the first 14 (98 bits)
constexpr int FIXB = 96;        // fixed-point bits of the 1/p_i weights
constexpr int CTA_THREADS = 192;   // warp 0 TMA, warp 1 MMA, warps 2..5 epilogue
constexpr int CTA_THREADS8 = 320;  // warp 0 TMA, warp 1 MMA, warps 2..9 epilogue (two per lane quadrant)
constexpr int RES_EPI_WARPS = 16;   // residue GEMM: four epilogue warps per lane quadrant
constexpr int RES_THREADS = 32 * (2 + RES_EPI_WARPS);
constexpr int RTAB = 256;          // reconstruction table rows are padded to a multiple of this
}  // namespace

struct ModConst {
    int32_t p;
    float inv_p;
    uint32_t mu;   // floor(2^32 / p)
    uint32_t h16;  // 2^16 mod p
    uint32_t w;    // (Mod / p)^-1 mod p
    uint32_t pad[3];
};

// ---- modular helpers (device) ---------------------------------------------------------
// Every value below is an exact integer held in FP32 with magnitude < 2^24, so
// the reductions run on the FMA pipe with no int<->float conversion.
//
// red(x) = x - rint(x / p) * p for |x| < 2^24 and 2^15 < p < 2^16.  The quotient
// is rounded by adding 1.5 * 2^23 inside one FMA (|x / p| < 2^9 keeps the sum in
// the binade where the ulp is 1); with inv_p = fl(1/p) its error against the
// true x / p is at most 2^9 * 2^-24 = 2^-15, so the result lies in
// [-p/2 - 2, p/2 + 2]: congruent to x, not always the balanced representative.
// The second FMA is exact because the true result is a small integer.
// Downstream bounds use |red(x)| <= 32772.
constexpr float RND_MAGIC = 12582912.0f;  // 1.5 * 2^23

// (p, p', fl(1/p), fl(1/p')) of moduli 2i and 2i+1 for the 1024 largest primes
// below 2^16, in descending order: the moduli of every product are a prefix of
// this list.  Warps read one pair at a time (a constant-cache broadcast, no
// shared-memory traffic); each half is a packed operand of the f32x2 arithmetic.
constexpr int CMOD_PAIRS = 512;
__constant__ float4 c_modpair[CMOD_PAIRS];
__device__ __forceinline__ float red(float x, float p, float inv_p) {
    const float q = __fadd_rn(__fmaf_rn(x, inv_p, RND_MAGIC), -RND_MAGIC);
    return __fmaf_rn(-q, p, x);
}
// r (|r| <= 32772) -> two signed byte digits, r = hi * 256 + lo, |hi|, |lo| <= 128
__device__ __forceinline__ void bal_split(float r, float &hi, float &lo) {
    hi = __fadd_rn(__fmaf_rn(r, 1.0f / 256.0f, RND_MAGIC), -RND_MAGIC);
    lo = __fmaf_rn(-hi, 256.0f, r);
}

// ---- the same steps on two values at once (packed f32x2 arithmetic: one FMA-pipe
// instruction per pair; each lane is rounded exactly as the scalar form) --------
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(f32x2 r, float &a, float &b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r)); }
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// red on both lanes: np = (-p, -p'), ip = (1/p, 1/p')
__device__ __forceinline__ f32x2 red2(f32x2 x, f32x2 np, f32x2 ip) {
    const f32x2 q = add2(fma2(x, ip, pk2(RND_MAGIC, RND_MAGIC)), pk2(-RND_MAGIC, -RND_MAGIC));
    return fma2(q, np, x);
}
__device__ __forceinline__ void bal_split2(f32x2 r, f32x2 &hi, f32x2 &lo) {
    hi = add2(fma2(r, pk2(1.0f / 256.0f, 1.0f / 256.0f), pk2(RND_MAGIC, RND_MAGIC)), pk2(-RND_MAGIC, -RND_MAGIC));
    lo = fma2(hi, pk2(-256.0f, -256.0f), r);
}
// bf16 bit patterns of two small integers (|v| <= 256 has at most 9 significant
// bits, so the low 16 bits of its FP32 encoding are zero and truncation is exact):
// a in the low half, b in the high half
__device__ __forceinline__ uint32_t bf16x2_bits(float a, float b) {
    return __byte_perm(__float_as_uint(a), __float_as_uint(b), 0x7632);
}

struct Barriers {
    uint64_t full[8];
    uint64_t empty[8];
    uint64_t tfull[2];
    uint64_t tempty[2];
    uint32_t tmem_base;
    int abort_flag;
};
constexpr uint32_t SMEM_BARS = 256;  // bytes reserved for Barriers; per-kernel tables follow
static_assert(sizeof(Barriers) <= SMEM_BARS, "barrier block");

__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
    uintptr_t v = reinterpret_cast<uintptr_t>(p);
    return reinterpret_cast<uint8_t *>((v + 1023) & ~(uintptr_t)1023);
}

// Common prologue: barrier init by thread 0, TMEM allocation by warp 1.
__device__ __forceinline__ void cta_setup(Barriers *bars, int stages, uint32_t tmem_cols, uint32_t full_count,
                                          uint32_t tempty_count) {
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; s++) {
            tc::mbar_init(&bars->full[s], full_count);
            tc::mbar_init(&bars->empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&bars->tfull[b], 1);
            tc::mbar_init(&bars->tempty[b], tempty_count);
        }
        bars->abort_flag = 0;
        tc::fence_mbar_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(&bars->tmem_base, tmem_cols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

__device__ __forceinline__ void cta_teardown(Barriers *bars, uint32_t tmem_cols) {
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(bars->tmem_base, tmem_cols);
    }
}

__device__ __forceinline__ void set_abort(Barriers *bars, uint32_t *err) {
    atomicOr(err, DEVERR_TIMEOUT);
    *(volatile int *)&bars->abort_flag = 1;
}
__device__ __forceinline__ bool aborted(Barriers *bars) { return *(volatile int *)&bars->abort_flag != 0; }

// epilogue warps 2..5 cover TMEM lane quadrants (warp % 4)
__device__ __forceinline__ int epi_row() { return ((threadIdx.x >> 5) & 3) * 32 + (threadIdx.x & 31); }
__device__ __forceinline__ uint32_t lane_base(uint32_t tmem) { return tmem + (((threadIdx.x >> 5) & 3) * 32u << 16); }
__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// A grouped launch runs the tiles of several products in one persistent kernel.
// Job j owns the global tiles [tile0[j], tile0[j + 1]); every role of a CTA walks
// the same tile sequence and looks each tile's job up by binary search.  The job
// records (arguments and 64-byte aligned tensor maps) sit in global memory.
template <typename J>
struct Group {
    const J *jobs;
    const int64_t *tile0;  // njobs + 1 entries, tile0[njobs] = all tiles
    int32_t njobs;
};
__device__ __forceinline__ int group_job(const int64_t *tile0, int n, int64_t T) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(tile0 + mid) <= T) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
// A role's walk through the tiles only moves forward: the current job and its tile
// range are kept until the walk leaves that range, so most tiles need no lookup
// (the binary search is a chain of dependent loads).
struct GroupCursor {
    int j = -1;
    int64_t beg = 0, end = 0;
    template <typename J>
    __device__ __forceinline__ void seek(const Group<J> &g, int64_t T) {
        if (j >= 0 && T < end) return;
        j = group_job(g.tile0, g.njobs, T);
        beg = __ldg(g.tile0 + j);
        end = __ldg(g.tile0 + j + 1);
    }
};

// ======================================================================================
// 1. digits
// ======================================================================================
// bf16 bits of bytes k and k+1 of w, byte k in the low half (unsigned digits).
// Each byte b becomes the FP32 value 2^23 + b (bits 0x4B000000 | b, built by one
// byte permute) minus 2^23, which is exact; b has at most 8 significant bits, so
// the top half of its FP32 encoding is its bf16 encoding.
__device__ __forceinline__ uint32_t byte_pair_bf16(uint32_t w, int k) {
    const float lo = __fadd_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + k)), -8388608.0f);
    const float hi = __fadd_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7541u + k)), -8388608.0f);
    return bf16x2_bits(lo, hi);
}

// Balanced byte digits of limb w: byte b_i becomes d_i = b_i + c_i - 256 m_i with
// m_i its top bit and c_i the top bit of the byte below (cin for byte 0), so
// sum d_i 256^i = sum b_i 256^i with every d_i in [-128, 128].  The carry needs no
// propagation: c_i depends on the byte below only.  The last digit of a row
// (last, byte 3) keeps its carry and is not reduced: it lies in [0, 256].
// Computed as e_i = (b_i ^ 128) + c_i = d_i + 128 in [0, 256]: two byte permutes
// and an integer add build the FP32 bits of 2^23 + e_i, and one exact FADD of
// -(2^23 + 128) leaves d_i.  With at most 9 significant bits the top half of the
// FP32 encoding is the bf16 encoding.  No int->float conversion instructions.
__device__ __forceinline__ void limb_digits_bal(uint32_t w, uint32_t cin, bool last, float (&d)[4]) {
    const uint32_t x = w ^ 0x80808080u;                          // b_i ^ 128 per byte
    const uint32_t c = ((w & 0x80808080u) >> 7 << 8) | cin;      // c_i in bit 0 of byte i
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t bits = __byte_perm(x, 0x4B000000u, 0x7650u + i) + __byte_perm(c, 0u, 0x4440u + i);
        d[i] = __fadd_rn(__uint_as_float(bits), -8388736.0f);  // (2^23 + e_i) - (2^23 + 128)
    }
    if (last) {
        // the row's last digit unreduced: b_3 + c_3 (the reduced form subtracted 256 when m_3 = 1)
        d[3] = (w >> 31) ? __fadd_rn(d[3], 256.0f) : d[3];
    }
}

// The digits carry the entry's sign (a negative entry's digits are negated), so
// the residue GEMM yields signed residues directly.
struct DigitArgs {
    const uint32_t *limbs;
    const int32_t *sizes;  // sizes[r * rs + c]: the entry's sign
    int64_t ld, rs;
    int32_t rows, cols, nlimbs;
    int32_t transpose;  // 0: out row r*cols + c ; 1: out row c*rows + r
    int32_t dxp;        // digits per out row (multiple of 64)
    __nv_bfloat16 *out;
};

// BAL: balanced digits.  s[entry][li - LO] holds limb l0 + li for li >= LO; with
// balanced digits LO = -1, so slot 0 holds limb l0 - 1 (its top byte carries into the
// chunk's first digit).  Rows of 65 and 67 words keep the column loads conflict-free.
// One operand of a grouped digits launch: its blocks are (bx, by, bz) in x-fastest
// order, nbx x nby x (chunks of 64 limbs).
struct DigitJob {
    DigitArgs a;
    int32_t nbx, nby;
};

template <bool BAL, bool GRP>
__global__ void __launch_bounds__(256) k_crt_digits(DigitArgs a0, Group<DigitJob> grp) {
    __shared__ uint32_t s[128][BAL ? 67 : 65];
    __shared__ uint32_t sflip[128];  // 0x80008000 for a negative entry: flips both bf16 signs of a word
    DigitArgs a;
    int bx, by, bz;
    tc::grid_dep_wait();    // the operand this launch reads is complete
    tc::grid_dep_launch();  // the residue GEMM's CTAs may set up while the last blocks run
    if (GRP) {
        const int j = group_job(grp.tile0, grp.njobs, blockIdx.x);
        const DigitJob &J = grp.jobs[j];
        a = J.a;
        const int b = (int)(blockIdx.x - __ldg(grp.tile0 + j));
        bx = b % J.nbx;
        by = (b / J.nbx) % J.nby;
        bz = b / J.nbx / J.nby;
    } else {
        a = a0;
        bx = blockIdx.x;
        by = blockIdx.y;
        bz = blockIdx.z;
    }
    const int tr = 4, tcn = 32;
    const int r0 = by * tr, c0 = bx * tcn;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 128) {
        const int r = r0 + (threadIdx.x >> 5), c = c0 + (threadIdx.x & 31);
        sflip[threadIdx.x] = (r < a.rows && c < a.cols && a.sizes[(int64_t)r * a.rs + c] < 0) ? 0x80008000u : 0u;
    }
    {
        // one chunk of 64 limbs per block (blockIdx.z): more, shorter blocks keep the
        // last wave of the grid small
        const int l0 = bz * 64;
        // load limbs [l0 - 1, l0 + 64) of the 4 x 32 entries, coalesced along c: slot
        // 1 + li holds limb l0 + li, slot 0 limb l0 - 1 (its top byte carries into the
        // chunk's first digit)
        constexpr int LO = BAL ? -1 : 0;  // first limb loaded, relative to l0
        for (int q = threadIdx.x; q < (64 - LO) * 128; q += 256) {
            int cc = q & 31, rr = (q >> 5) & 3, li = (q >> 7) + LO;
            int r = r0 + rr, c = c0 + cc, l = l0 + li;
            uint32_t v = 0;
            if (r < a.rows && c < a.cols && l >= 0 && l < a.nlimbs) v = a.limbs[(int64_t)l * a.ld + (int64_t)r * a.rs + c];
            s[rr * 32 + cc][li - LO] = v;
        }
        __syncthreads();
        // each warp writes whole digit rows: lane j -> limbs l0+2j, l0+2j+1 (8 digits, 16 bytes)
        for (int ent = warp; ent < 128; ent += 8) {
            int rr = ent >> 5, cc = ent & 31;
            int r = r0 + rr, c = c0 + cc;
            if (r >= a.rows || c >= a.cols) continue;
            int64_t row = a.transpose ? (int64_t)c * a.rows + r : (int64_t)r * a.cols + c;
            int dg = 4 * (l0 + 2 * lane);
            if (dg >= a.dxp) continue;
            const uint32_t flip = sflip[ent];
            uint4 pk;
            if (BAL) {
                const uint32_t vp = s[ent][2 * lane], v0 = s[ent][2 * lane + 1], v1 = s[ent][2 * lane + 2];
                float d0[4], d1[4];
                limb_digits_bal(v0, vp >> 31, false, d0);
                limb_digits_bal(v1, v0 >> 31, dg + 8 == a.dxp, d1);
                pk.x = bf16x2_bits(d0[0], d0[1]) ^ flip;
                pk.y = bf16x2_bits(d0[2], d0[3]) ^ flip;
                pk.z = bf16x2_bits(d1[0], d1[1]) ^ flip;
                pk.w = bf16x2_bits(d1[2], d1[3]) ^ flip;
            } else {
                const uint32_t v0 = s[ent][2 * lane], v1 = s[ent][2 * lane + 1];
                pk.x = byte_pair_bf16(v0, 0) ^ flip;
                pk.y = byte_pair_bf16(v0, 2) ^ flip;
                pk.z = byte_pair_bf16(v1, 0) ^ flip;
                pk.w = byte_pair_bf16(v1, 2) ^ flip;
            }
            *reinterpret_cast<uint4 *>(a.out + row * a.dxp + dg) = pk;
        }
    }
}

// ======================================================================================
// 2. residue GEMM (persistent; TMEM double-buffered so a tile's epilogue overlaps
//    the next tile's MMAs; 16 epilogue warps, four per TMEM lane quadrant)
// ======================================================================================
struct ResidueArgs {
    int32_t kdim;  // entry e -> (e / kdim, e % kdim) in digit-row order
    int32_t E;     // entries (digit rows)
    int32_t nk;    // K steps of 64 digits
    int32_t BN, G; // table columns per tile, accumulation groups (G * BN <= 256)
    int32_t P;
    int32_t ncols;  // table columns: two per modulus, padded to whole pairs of moduli
    int32_t n_ntiles;
    int32_t ntiles;
    __nv_bfloat16 *R;  // planes [2P][rowsR][kp]
    int64_t plane;     // rowsR * kp
    int32_t kp;
    int32_t tma_out;  // kdim % 32 == 0: each warp's 32 entries share a plane row; TMA stores
};
// One operand of a grouped residue launch.
struct ResidueJob {
    CUtensorMap tmD, tmT, tmR;
    ResidueArgs a;
};

// shared-memory staging of one epilogue warp's chunk: [32 planes][32 entries] bf16
constexpr int RES_STG_BYTES = 32 * 32 * 2;

// One chunk of 32 accumulator columns (16 moduli) of group g folded into res.
// The table orders each pair of moduli (m, m') as four columns: [lo_m, lo_m',
// hi_m, hi_m'] (the byte digits of 256^j mod p times 1 and 256), so the lo sums and
// the hi sums of a pair come as packed operands: res = red(256 red(s1) + red(s0)
// (+ res)) on both lanes at once.  Each term is an integer of magnitude <= 2^24;
// the sum stays below 257 * 32772 + 32772 < 2^24, so every FP32 step is exact.
__device__ __forceinline__ void residue_fold(const uint32_t (&v)[32], int mi0, bool first, f32x2 (&res)[8]) {
#pragma unroll
    for (int g = 0; g < 8; g++) {
        const float4 pc = c_modpair[(mi0 >> 1) + g];  // (p, p', 1/p, 1/p')
        const f32x2 np = pk2(-pc.x, -pc.y), ip = pk2(pc.z, pc.w);
        const f32x2 s0 = pk2(__uint_as_float(v[4 * g]), __uint_as_float(v[4 * g + 1]));
        const f32x2 s1 = pk2(__uint_as_float(v[4 * g + 2]), __uint_as_float(v[4 * g + 3]));
        f32x2 t = fma2(red2(s1, np, ip), pk2(256.f, 256.f), red2(s0, np, ip));
        if (!first) t = add2(t, res[g]);
        res[g] = red2(t, np, ip);
    }
}

// PAIR: a cluster of two CTAs shares one M = 256 tcgen05.mma.cta_group::2 per K
// slice (issued by the even CTA); each CTA stages its own 128 entries and half of
// the tile's table columns, and keeps its own 128 rows of D in its TMEM.
// MC: a cluster of two CTAs with an M = 128 MMA each, on neighbouring 128-entry
// row blocks and the same table columns: each CTA loads half of the table box and
// multicasts it to both, so the table is read from L2 once per pair of row blocks,
// and each CTA's MMA commit frees the stage in both CTAs.
// GRP: a grouped launch (single CTAs only); every stage is sized for GBN table
// columns (the launch's operands have table tiles of at most GBN columns).
template <int STAGES, bool PAIR, bool MC, int GS, bool GRP, int GBN = 256>
__global__ void __launch_bounds__(RES_THREADS, 1)
    k_crt_residue(const __grid_constant__ CUtensorMap tmD, const __grid_constant__ CUtensorMap tmT,
                  const __grid_constant__ CUtensorMap tmR, ResidueArgs a0, Group<ResidueJob> grp, uint32_t *err) {
    static_assert(!GRP || (!PAIR && !MC), "grouped residue launches use single CTAs");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = align1024(smem_raw);
    constexpr bool CL = PAIR || MC;     // launched as clusters of two CTAs
    constexpr int NP = CL ? 2 : 1;      // row blocks per tile (per cluster)
    constexpr int NBUF = PAIR ? 2 : 1;  // staging buffers per epilogue warp
    const uint32_t A_BYTES = BM * 128, B_BYTES = GRP ? (uint32_t)GBN * 128 : (uint32_t)(PAIR ? a0.BN / 2 : a0.BN) * 128,
                   STAGE = A_BYTES + B_BYTES;
    Barriers *bars = reinterpret_cast<Barriers *>(base + STAGES * STAGE);
    uint8_t *stage_out = reinterpret_cast<uint8_t *>(bars) + SMEM_BARS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = CL ? tc::cluster_rank() : 0;
    const int64_t t0 = CL ? (blockIdx.x >> 1) : blockIdx.x, tstep = CL ? (gridDim.x >> 1) : gridDim.x;
    if (MC) {
        // per CTA as below, but every stage is freed by both CTAs' MMA commits
        if (threadIdx.x == 0) {
            for (int s = 0; s < STAGES; s++) {
                tc::mbar_init(&bars->full[s], 1);
                tc::mbar_init(&bars->empty[s], 2);
            }
            for (int b = 0; b < 2; b++) {
                tc::mbar_init(&bars->tfull[b], 1);
                tc::mbar_init(&bars->tempty[b], RES_EPI_WARPS);
            }
            bars->abort_flag = 0;
            tc::fence_mbar_init();
        }
        if (warp == 1) {
            tc::tmem_alloc(&bars->tmem_base, 512);
            tc::tmem_relinquish();
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // both CTAs' barriers exist before any multicast lands
        tc::fence_after_sync();
    } else if (PAIR) {
        if (threadIdx.x == 0) {
            for (int s = 0; s < STAGES; s++) {
                tc::mbar_init(&bars->full[s], 1);
                tc::mbar_init(&bars->empty[s], 1);
            }
            for (int b = 0; b < 2; b++) {
                tc::mbar_init(&bars->tfull[b], 1);
                tc::mbar_init(&bars->tempty[b], 2 * RES_EPI_WARPS);  // the even CTA's: every epilogue warp of both CTAs
            }
            bars->abort_flag = 0;
            tc::fence_mbar_init();
        }
        if (warp == 1) {
            tc::tmem_alloc_pair(&bars->tmem_base, 512);
            tc::tmem_relinquish_pair();
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // both CTAs' barriers exist before any cross-CTA signal
        tc::fence_after_sync();
    } else {
        cta_setup(bars, STAGES, 512, 1, RES_EPI_WARPS);
    }
    tc::grid_dep_wait();  // the digits this launch reads are complete
    const uint32_t tmem = bars->tmem_base;
    // the last table tile may be narrow: its MMA has only the columns it needs
    // (a multiple of 16, of 32 for a pair so that each CTA stages whole 8-row groups)
    const int ngran = CL ? 32 : 16;
    const int64_t total = GRP ? grp.tile0[grp.njobs] : (int64_t)a0.ntiles;
    // global tile T -> its operand's arguments and maps, and the tile within it
    GroupCursor cur;
    auto tile_job = [&](int64_t T, ResidueArgs &a, const CUtensorMap *&mD, const CUtensorMap *&mT,
                        const CUtensorMap *&mR) -> int {
        if (GRP) {
            cur.seek(grp, T);
            const ResidueJob *J = grp.jobs + cur.j;
            a = J->a;
            mD = &J->tmD;
            mT = &J->tmT;
            mR = &J->tmR;
            return (int)(T - cur.beg);
        }
        a = a0;
        mD = &tmD;
        mT = &tmT;
        mR = &tmR;
        return (int)T;
    };

    if (warp == 0) {
        if (lane == 0) {
            if (!GRP) {
                tc::prefetch_tmap(&tmD);
                tc::prefetch_tmap(&tmT);
            }
            int it = 0;
            for (int64_t T = t0; T < total && !aborted(bars); T += tstep) {
                ResidueArgs a;
                const CUtensorMap *mD, *mT, *mR;
                const int t = tile_job(T, a, mD, mT, mR);
                (void)mR;
                const int rb = t / a.n_ntiles;
                const int e0 = rb * (NP * BM) + (int)rank * BM;
                const int n0 = (t - rb * a.n_ntiles) * a.BN;
                const int nn = min(a.BN, (a.ncols - n0 + ngran - 1) / ngran * ngran);
                for (int s = 0; s < a.nk; s++, it++) {
                    const int st = it % STAGES;
                    if (it >= STAGES && !tc::mbar_wait(&bars->empty[st], ((it / STAGES) & 1) ^ 1)) {
                        set_abort(bars, err);
                        break;
                    }
                    uint8_t *sa = base + st * STAGE;
                    if (PAIR) {
                        // this CTA's half of the tile's columns: n0 + rank * nn / 2 onwards
                        const uint32_t full0 = tc::mapa(tc::smem_u32(&bars->full[st]), 0);
                        if (rank == 0) tc::mbar_arrive_expect_tx(&bars->full[st], 2 * STAGE);
                        tc::tma_load_2d_pair(sa, mD, full0, s * BK, (int)e0);
                        tc::tma_load_2d_pair(sa + A_BYTES, mT, full0, s * BK, n0 + (int)rank * (nn / 2));
                    } else if (MC) {
                        // own digit rows; this CTA's half of the table box to both CTAs
                        tc::mbar_arrive_expect_tx(&bars->full[st], STAGE);
                        tc::tma_load_2d(sa, mD, &bars->full[st], s * BK, (int)e0);
                        tc::tma_load_2d_mc(sa + A_BYTES + rank * (B_BYTES / 2), mT, &bars->full[st], s * BK,
                                           n0 + (int)rank * (a.BN / 2), 0x3);
                    } else {
                        // a grouped stage holds this operand's BN table rows of its 256
                        tc::mbar_arrive_expect_tx(&bars->full[st], GRP ? A_BYTES + (uint32_t)a.BN * 128 : STAGE);
                        tc::tma_load_2d(sa, mD, &bars->full[st], s * BK, (int)e0);
                        tc::tma_load_2d(sa + A_BYTES, mT, &bars->full[st], s * BK, n0);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && (rank == 0 || MC)) {
            int it = 0, lt = 0;
            bool ok = true;
            for (int64_t T = t0; T < total && ok; T += tstep, lt++) {
                ResidueArgs a;
                const CUtensorMap *mD, *mT, *mR;
                const int t = tile_job(T, a, mD, mT, mR);
                (void)mD, (void)mT, (void)mR;
                const int b = lt & 1;
                const int n0 = (t % a.n_ntiles) * a.BN;
                const int nn = min(a.BN, (a.ncols - n0 + ngran - 1) / ngran * ngran);
                const uint32_t idesc = tc::idesc_bf16_f32(PAIR ? 2 * BM : BM, nn, 0, 0);
                if (lt >= 2 && !tc::mbar_wait(&bars->tempty[b], ((lt >> 1) & 1) ^ 1)) { set_abort(bars, err); break; }
                tc::fence_after_sync();
                for (int s = 0; s < a.nk; s++, it++) {
                    const int st = it % STAGES;
                    if (!tc::mbar_wait(&bars->full[st], (it / STAGES) & 1)) { set_abort(bars, err); ok = false; break; }
                    tc::fence_after_sync();
                    const uint32_t sa = tc::smem_u32(base + st * STAGE);
                    // accumulation group s / GS (GS K steps each, a compile-time constant: the
                    // issuing thread is on the critical path)
                    const uint32_t d = tmem + (uint32_t)(256 * b + (s / GS) * a.BN);
                    const uint64_t ad = tc::sdesc_kmajor(sa), bd = tc::sdesc_kmajor(sa + A_BYTES);
#pragma unroll
                    for (int kk = 0; kk < BK / UK; kk++) {
                        const uint64_t adesc = tc::sdesc_advance(ad, kk * 32), bdesc = tc::sdesc_advance(bd, kk * 32);
                        const uint32_t acc = (s % GS) != 0 || kk != 0;
                        if (PAIR) tc::mma_bf16_pair(d, adesc, bdesc, idesc, acc);
                        else tc::mma_bf16(d, adesc, bdesc, idesc, acc);
                    }
                    if (PAIR) tc::mma_commit_pair(&bars->empty[st], 0x3);
                    else if (MC) tc::mma_commit_mc(&bars->empty[st], 0x3);
                    else tc::mma_commit(&bars->empty[st]);
                }
                if (ok) {
                    if (PAIR) tc::mma_commit_pair(&bars->tfull[b], 0x3);
                    else tc::mma_commit(&bars->tfull[b]);
                }
            }
        }
    } else {
        // epilogue: warp (2..17) -> lane quadrant warp % 4, column slot (warp - 2) / 4
        // of cpw chunks of 32 columns.  A warp's work on a tile is its live chunks
        // times G groups ("units", one 32-column TMEM load each), chunk-major.  Four
        // warps per scheduler hide the loads' latency.
        const int quad = warp & 3, slot = (warp - 2) >> 2;
        const uint32_t lb = tmem + ((uint32_t)(quad * 32) << 16);
        const uint32_t tempty0 = PAIR ? tc::mapa(tc::smem_u32(&bars->tempty[0]), 0) : 0;
        uint16_t *stg = reinterpret_cast<uint16_t *>(stage_out + (warp - 2) * NBUF * RES_STG_BYTES);
        int lt = 0, sbuf = 0;
        for (int64_t T = t0; T < total; T += tstep, lt++) {
            ResidueArgs a;
            const CUtensorMap *mD, *mT, *mR;
            const int t = tile_job(T, a, mD, mT, mR);
            (void)mD, (void)mT;
            const int cpw = max(1, a.BN / 128);                          // chunks per warp
            const int hcols = slot * cpw * 32;                           // the warp's first column in a tile
            const int nch = max(0, min(cpw, (a.BN - hcols) / 32)), G = a.G;
            const int64_t pstep = 2 * a.plane;  // planes of one modulus
            const uint32_t kdim = (uint32_t)a.kdim, E = (uint32_t)a.E;
            const int b = lt & 1;
            const int rb = t / a.n_ntiles;
            const int n0 = (t - rb * a.n_ntiles) * a.BN;
            const uint32_t ew = (uint32_t)rb * (NP * BM) + rank * BM + quad * 32;  // the warp's first entry
            const uint32_t e = ew + lane;
            if (!tc::mbar_wait(&bars->tfull[b], (lt >> 1) & 1)) { set_abort(bars, err); break; }
            tc::fence_after_sync();
            const uint32_t rw = ew / kdim, cw = ew - rw * kdim;  // plane row and column of the warp's box
            const uint32_t re = e / kdim;
            const int64_t off = e < E ? (int64_t)re * a.kp + (e - re * kdim) : 0;
            const int c00 = n0 + hcols;  // the warp's first table column
            const int nlive = max(0, min(nch, (a.ncols - c00 + 31) / 32));
            const int nunits = nlive * G;
            auto release = [&]() {
                // last TMEM read of this tile by this warp: hand the buffer back
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) {
                    if (PAIR) tc::mbar_arrive_cluster(tempty0 + 8u * b);
                    else tc::mbar_arrive(&bars->tempty[b]);
                }
            };
            if (nunits == 0) {
                release();
                continue;
            }
            f32x2 res[8];  // moduli (mi0 + 2g, mi0 + 2g + 1) of the current chunk
            auto store = [&](int mi0) {
                // bf16 bits of the two balanced byte digits of each residue
                uint16_t hb[16], lbits[16];
#pragma unroll
                for (int g = 0; g < 8; g++) {
                    f32x2 h2, l2;
                    bal_split2(res[g], h2, l2);
                    float h0, h1, l0, l1;
                    upk2(h2, h0, h1);
                    upk2(l2, l0, l1);
                    hb[2 * g] = (uint16_t)(__float_as_uint(h0) >> 16);
                    hb[2 * g + 1] = (uint16_t)(__float_as_uint(h1) >> 16);
                    lbits[2 * g] = (uint16_t)(__float_as_uint(l0) >> 16);
                    lbits[2 * g + 1] = (uint16_t)(__float_as_uint(l1) >> 16);
                }
                if (a.tma_out) {
                    if (ew >= E) return;  // the whole box lies past the last entry
                    if (lane == 0) tc::bulk_wait_read<NBUF - 1>();
                    __syncwarp();
                    uint16_t *buf = stg + sbuf * (RES_STG_BYTES / 2);
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        buf[(2 * j) * 32 + lane] = hb[j];
                        buf[(2 * j + 1) * 32 + lane] = lbits[j];
                    }
                    tc::fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) {
                        // planes past 2P and rows past the last entry are clipped by the map
                        tc::tma_store_3d(mR, buf, (int)cw, (int)rw, 2 * mi0);
                        tc::bulk_commit_group();
                    }
                    if (NBUF > 1) sbuf ^= 1;
                } else if (e < E) {
                    uint16_t *dst = reinterpret_cast<uint16_t *>(a.R + (int64_t)mi0 * pstep + off);
                    const int nj = a.P - mi0;
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        if (j >= nj) break;
                        dst[j * pstep] = hb[j];
                        dst[j * pstep + a.plane] = lbits[j];
                    }
                }
            };
            int lch = 0, lg = 0;  // the next unit to load
            auto load_next = [&](uint32_t(&v)[32]) {
                tc::tmem_ld32(lb + (uint32_t)(256 * b + lg * a.BN + hcols + lch * 32), v);
                if (++lg == G) {
                    lg = 0;
                    lch++;
                }
            };
            int cch = 0, cg = 0;  // the next unit to fold
            auto consume = [&](const uint32_t(&v)[32]) {
                const int mi0 = (c00 + cch * 32) >> 1;
                residue_fold(v, mi0, cg == 0, res);
                if (cg == G - 1) store(mi0);
                if (++cg == G) {
                    cg = 0;
                    cch++;
                }
            };
            uint32_t va[32];
            for (int u = 0; u < nunits; u++) {
                load_next(va);
                tc::tmem_ld_wait(va);
                if (u + 1 == nunits) release();
                consume(va);
            }
        }
        if (lane == 0) tc::bulk_wait_all();  // staging buffers stay live until the stores finish
        __syncwarp();
    }
    tc::grid_dep_launch();
    if (PAIR) {
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // no CTA leaves while its peer may still signal it or write its TMEM
        if (warp == 1) {
            tc::fence_after_sync();
            tc::tmem_dealloc_pair(tmem, 512);
        }
    } else if (MC) {
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // no CTA leaves while its peer may still multicast into it or arrive on it
        if (warp == 1) {
            tc::fence_after_sync();
            tc::tmem_dealloc(tmem, 512);
        }
    } else {
        cta_teardown(bars, 512);
    }
}

// ======================================================================================
// 3. per-modulus product GEMM (persistent over (modulus, 128 x 64 output tiles);
//    TMEM double-buffered; 8 epilogue warps)
//
// With a = 256 a1 + a0 (residues of A as balanced digits) and u = 256 u1 + u0
// (residues of B, already multiplied by the CRT weight w = (Mod/p)^-1 mod p),
// the weighted product is
//     y = a b w = 65536 a1 u1 + 256 (a1 u0 + a0 u1) + a0 u0   (mod p).
// Each K step issues two N = 128 MMAs against the stacked operand [U1; U0]:
// A1 into [a1 u1 | a1 u0] and A0 into [a0 u1 | a0 u0].  Each of the four 64-column
// accumulators sums k products of magnitude <= 2^14: at most 2^23 for k <= 512,
// and the middle pair adds to at most 2^24.
// ======================================================================================
struct ProductArgs {
    int32_t m, n, nk, P;
    int32_t npad;      // entry row pitch of Y: n rounded up to 16 (entry e = y * npad + x)
    int32_t nyt, nxt;
    int64_t ntiles;
    __nv_bfloat16 *Y;  // blocked [Ep/64][2Pp][64]: 64 entries per row, 2Pp rows per block
    int64_t yblk;      // elements per 64-entry block (2Pp * 64)
};
// One product of a grouped product launch.
struct ProductJob {
    CUtensorMap tmA, tmB;
    ProductArgs a;
};
constexpr int PBX = 64;  // output columns per product tile
constexpr int YPAD = 16;  // Y's entry rows are padded to a multiple of this (whole 32-byte runs)

// PAIR: a cluster of two CTAs shares one M = 256 tcgen05.mma.cta_group::2 per K
// slice (issued by the even CTA): each CTA stages its own 128 rows of A1 and A0,
// the even CTA U1's 64 rows and the odd CTA U0's, so per SM a K step moves 40 KB
// instead of 48 KB and the MMAs read 12 KB of shared memory instead of 16 KB.
template <int STAGES, bool PAIR, bool GRP>
__global__ void __launch_bounds__(CTA_THREADS8, 1)
    k_crt_product(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, ProductArgs a0,
                  Group<ProductJob> grp, uint32_t *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = align1024(smem_raw);
    constexpr int NP = PAIR ? 2 : 1;
    // A1, A0 (128 rows each), then U1, U0 (64 rows each; one of them per CTA of a pair):
    // together the 128-row B operand [U1; U0]
    constexpr uint32_t A_BYTES = BM * 128, B_BYTES = PBX * 128, STAGE = 2 * A_BYTES + (3 - NP) * B_BYTES;
    Barriers *bars = reinterpret_cast<Barriers *>(base + STAGES * STAGE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = PAIR ? tc::cluster_rank() : 0;
    const int64_t t0 = PAIR ? (blockIdx.x >> 1) : blockIdx.x, tstep = PAIR ? (gridDim.x >> 1) : gridDim.x;
    if (PAIR) {
        if (threadIdx.x == 0) {
            for (int s = 0; s < STAGES; s++) {
                tc::mbar_init(&bars->full[s], 1);
                tc::mbar_init(&bars->empty[s], 1);
            }
            for (int b = 0; b < 2; b++) {
                tc::mbar_init(&bars->tfull[b], 1);
                tc::mbar_init(&bars->tempty[b], 16);  // the even CTA's: 8 epilogue warps of each CTA
            }
            bars->abort_flag = 0;
            tc::fence_mbar_init();
        }
        if (warp == 1) {
            tc::tmem_alloc_pair(&bars->tmem_base, 512);
            tc::tmem_relinquish_pair();
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // both CTAs' barriers exist before any cross-CTA signal
        tc::fence_after_sync();
    } else {
        cta_setup(bars, STAGES, 512, 1, 8);
    }
    tc::grid_dep_wait();  // the planes this launch reads are complete
    const uint32_t tmem = bars->tmem_base;
    const int64_t total = GRP ? grp.tile0[grp.njobs] : a0.ntiles;
    // global tile T -> its product's arguments and maps, and the tile within it
    GroupCursor cur;
    auto tile_job = [&](int64_t T, ProductArgs &a, const CUtensorMap *&mA, const CUtensorMap *&mB) -> int64_t {
        if (GRP) {
            cur.seek(grp, T);
            const ProductJob *J = grp.jobs + cur.j;
            a = J->a;
            mA = &J->tmA;
            mB = &J->tmB;
            return T - cur.beg;
        }
        a = a0;
        mA = &tmA;
        mB = &tmB;
        return T;
    };

    if (warp == 0) {
        if (lane == 0) {
            if (!GRP) {
                tc::prefetch_tmap(&tmA);
                tc::prefetch_tmap(&tmB);
            }
            int it = 0;
            for (int64_t T = t0; T < total && !aborted(bars); T += tstep) {
                ProductArgs a;
                const CUtensorMap *mA, *mB;
                const int64_t t = tile_job(T, a, mA, mB);
                const int64_t per_mod = (int64_t)a.nyt * a.nxt;
                const int mi = (int)(t / per_mod), r = (int)(t % per_mod);
                const int y0 = (r / a.nxt) * (NP * BM) + (int)rank * BM, x0 = (r % a.nxt) * PBX;
                for (int s = 0; s < a.nk; s++, it++) {
                    const int st = it % STAGES;
                    if (it >= STAGES && !tc::mbar_wait(&bars->empty[st], ((it / STAGES) & 1) ^ 1)) {
                        set_abort(bars, err);
                        break;
                    }
                    uint8_t *sa = base + st * STAGE;
                    if (PAIR) {
                        const uint32_t full0 = tc::mapa(tc::smem_u32(&bars->full[st]), 0);
                        if (rank == 0) tc::mbar_arrive_expect_tx(&bars->full[st], 2 * STAGE);
                        tc::tma_load_2d_pair(sa, mA, full0, s * BK, (2 * mi) * a.m + y0);
                        tc::tma_load_2d_pair(sa + A_BYTES, mA, full0, s * BK, (2 * mi + 1) * a.m + y0);
                        tc::tma_load_2d_pair(sa + 2 * A_BYTES, mB, full0, s * BK, (2 * mi + (int)rank) * a.n + x0);
                    } else {
                        tc::mbar_arrive_expect_tx(&bars->full[st], STAGE);
                        tc::tma_load_2d(sa, mA, &bars->full[st], s * BK, (2 * mi) * a.m + y0);
                        tc::tma_load_2d(sa + A_BYTES, mA, &bars->full[st], s * BK, (2 * mi + 1) * a.m + y0);
                        tc::tma_load_2d(sa + 2 * A_BYTES, mB, &bars->full[st], s * BK, (2 * mi) * a.n + x0);
                        tc::tma_load_2d(sa + 2 * A_BYTES + B_BYTES, mB, &bars->full[st], s * BK,
                                        (2 * mi + 1) * a.n + x0);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {
            const uint32_t idesc = tc::idesc_bf16_f32(NP * BM, 2 * PBX, 0, 0);
            int it = 0, lt = 0;
            bool ok = true;
            for (int64_t T = t0; T < total && ok; T += tstep, lt++) {
                ProductArgs a;
                const CUtensorMap *mA, *mB;
                tile_job(T, a, mA, mB);
                (void)mA, (void)mB;
                const int b = lt & 1;
                if (lt >= 2 && !tc::mbar_wait(&bars->tempty[b], ((lt >> 1) & 1) ^ 1)) { set_abort(bars, err); break; }
                tc::fence_after_sync();
                const uint32_t d = tmem + 256u * b;
                for (int s = 0; s < a.nk; s++, it++) {
                    const int st = it % STAGES;
                    if (!tc::mbar_wait(&bars->full[st], (it / STAGES) & 1)) { set_abort(bars, err); ok = false; break; }
                    tc::fence_after_sync();
                    const uint32_t sa = tc::smem_u32(base + st * STAGE);
                    // three descriptors per K step; the K slices advance them by 32 bytes
                    const uint64_t a1d = tc::sdesc_kmajor(sa), a0d = tc::sdesc_kmajor(sa + A_BYTES),
                                   bd = tc::sdesc_kmajor(sa + 2 * A_BYTES);
#pragma unroll
                    for (int kk = 0; kk < BK / UK; kk++) {
                        const uint64_t bdesc = tc::sdesc_advance(bd, kk * 32);
                        const uint64_t a1 = tc::sdesc_advance(a1d, kk * 32), a0 = tc::sdesc_advance(a0d, kk * 32);
                        const uint32_t acc = s != 0 || kk != 0;
                        if (PAIR) {
                            tc::mma_bf16_pair(d, a1, bdesc, idesc, acc);
                            tc::mma_bf16_pair(d + 2 * PBX, a0, bdesc, idesc, acc);
                        } else {
                            tc::mma_bf16(d, a1, bdesc, idesc, acc);
                            tc::mma_bf16(d + 2 * PBX, a0, bdesc, idesc, acc);
                        }
                    }
                    if (PAIR) tc::mma_commit_pair(&bars->empty[st], 0x3);
                    else tc::mma_commit(&bars->empty[st]);
                }
                if (ok) {
                    if (PAIR) tc::mma_commit_pair(&bars->tfull[b], 0x3);
                    else tc::mma_commit(&bars->tfull[b]);
                }
            }
        }
    } else {
        // warp (2..9) -> lane quadrant warp % 4, output columns 32 * ((warp - 2) / 4) + [0, 32).
        // All four accumulators' 32 columns are read first, so the buffer goes back to the
        // MMA before the arithmetic.
        const int quad = warp & 3, half = (warp - 2) >> 2;
        const uint32_t lb = tmem + ((uint32_t)(quad * 32) << 16);
        const uint32_t tempty0 = PAIR ? tc::mapa(tc::smem_u32(&bars->tempty[0]), 0) : 0;
        int lt = 0;
        for (int64_t T = t0; T < total; T += tstep, lt++) {
            ProductArgs a;
            const CUtensorMap *mA, *mB;
            const int64_t t = tile_job(T, a, mA, mB);
            (void)mA, (void)mB;
            const int64_t per_mod = (int64_t)a.nyt * a.nxt;
            const int b = lt & 1;
            const int mi = (int)(t / per_mod), r = (int)(t % per_mod);
            const int y = (r / a.nxt) * (NP * BM) + (int)rank * BM + quad * 32 + lane;
            const int xh = (r % a.nxt) * PBX + half * 32;  // this warp's 32 output columns
            if (!tc::mbar_wait(&bars->tfull[b], (lt >> 1) & 1)) { set_abort(bars, err); break; }
            tc::fence_after_sync();
            uint32_t D11[32], D10[32], D01[32], D00[32];
            const uint32_t col = 256u * b + half * 32;
            tc::tmem_ld32(lb + col, D11);
            tc::tmem_ld32(lb + col + PBX, D10);
            tc::tmem_ld32(lb + col + 2 * PBX, D01);
            tc::tmem_ld32(lb + col + 3 * PBX, D00);
            tc::tmem_ld_wait();
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) {
                if (PAIR) tc::mbar_arrive_cluster(tempty0 + 8u * b);
                else tc::mbar_arrive(&bars->tempty[b]);
            }
            // p and fl(1/p) of modulus mi from the constant list (a broadcast: the warp's
            // lanes share mi); the same values as the moduli table's
            const float4 cmp = c_modpair[mi >> 1];
            const float pf = (mi & 1) ? cmp.y : cmp.x, ipf = (mi & 1) ? cmp.w : cmp.z;
            const int64_t erow = (int64_t)y * a.npad + xh;  // entry index of this warp's first column
            __nv_bfloat16 *yplane = a.Y + (int64_t)(2 * mi) * 64;  // hi plane; lo plane 64 elements on
#pragma unroll
            for (int c = 0; c < 32; c += 16) {
                const uint32_t *d11 = D11 + c, *d10 = D10 + c, *d01 = D01 + c, *d00 = D00 + c;
                uint32_t phi[8], plo[8];
#pragma unroll
                for (int j = 0; j < 16; j += 2) {
                    float h2[2], l2[2];
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        // |a1 u0 + a0 u1| <= 2^24; each step below stays under 257 * 32772 < 2^24
                        const float r2 = red(__uint_as_float(d11[j + u]), pf, ipf);
                        const float r1 = red(__uint_as_float(d10[j + u]) + __uint_as_float(d01[j + u]), pf, ipf);
                        const float r0 = red(__uint_as_float(d00[j + u]), pf, ipf);
                        const float tt = red(__fmaf_rn(256.f, r2, r1), pf, ipf);
                        bal_split(red(__fmaf_rn(256.f, tt, r0), pf, ipf), h2[u], l2[u]);
                    }
                    phi[j / 2] = bf16x2_bits(h2[0], h2[1]);
                    plo[j / 2] = bf16x2_bits(l2[0], l2[1]);
                }
                if (y >= a.m) continue;
                // rows of Y are padded to whole groups of 16 entries, so every group but a
                // row's last partial one is two aligned 32-byte runs inside one 64-entry block
                const int64_t ec = erow + c;
                if ((ec & 15) == 0 && xh + c < a.n) {
                    __nv_bfloat16 *dst = yplane + (ec >> 6) * a.yblk + (ec & 63);
                    uint4 *dsth = reinterpret_cast<uint4 *>(dst), *dstl = reinterpret_cast<uint4 *>(dst + 64);
                    dsth[0] = make_uint4(phi[0], phi[1], phi[2], phi[3]);
                    dsth[1] = make_uint4(phi[4], phi[5], phi[6], phi[7]);
                    dstl[0] = make_uint4(plo[0], plo[1], plo[2], plo[3]);
                    dstl[1] = make_uint4(plo[4], plo[5], plo[6], plo[7]);
                } else {
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        if (xh + c + j >= a.n) break;
                        const int64_t e = ec + j;
                        uint16_t *dst = reinterpret_cast<uint16_t *>(yplane + (e >> 6) * a.yblk + (e & 63));
                        dst[0] = (uint16_t)(phi[j / 2] >> (16 * (j & 1)));
                        dst[64] = (uint16_t)(plo[j / 2] >> (16 * (j & 1)));
                    }
                }
            }
        }
    }
    tc::grid_dep_launch();
    if (PAIR) {
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // no CTA leaves while its peer may still signal it or write its TMEM
        if (warp == 1) {
            tc::fence_after_sync();
            tc::tmem_dealloc_pair(tmem, 512);
        }
    } else {
        cta_teardown(bars, 512);
    }
}

// ======================================================================================
// 4. reconstruction GEMM (persistent over tiles of 128 entries, or 256 entries
//    for a CTA pair; N tiles of 256 table rows; TMEM double-buffered across N
//    tiles; 8 epilogue warps per CTA, two per entry splitting the columns.  Base-128 table
//    digits keep one FP32 accumulation over all 2P rows exact:
//    2P * 128 * 64 < 2^24.)
//    Y arrives blocked, [E/64][2Pp][64], so each 64-entry x 64-row A box is one
//    contiguous 8 KB run.
//    PAIR: a cluster of two CTAs on two SMs runs one M = 256, N = 256
//    tcgen05.mma.cta_group::2 per K slice.  Each CTA stages its own 128 entries
//    and its own 128 of the 256 table rows, so per SM the K step moves 32 KB
//    through TMA and the MMA reads 8 KB of shared memory per 2^20 FLOP, against
//    48 KB and 12 KB for one CTA with N = 256: shared-memory bandwidth, which
//    bounds the single-SM tile, drops by a third.
// ======================================================================================
struct ReconArgs {
    int64_t mt0;     // first entry tile of this launch (tiles mt0 .. nmt-1)
    int64_t E;       // entries of Y: rows of C x padded row length
    int32_t ncols;   // padded row length of Y's entries (entry e -> row e / ncols, col e % ncols)
    int32_t ccols;   // columns of C: entries with col >= ccols are padding and not stored
    int32_t nk;      // K steps over 2Pp
    int32_t NT;      // N tiles of 256 table rows
    int32_t Dout;    // output base-128 digit positions
    int32_t kpad;    // 2Pp: rows of one 64-entry block of Y
    int64_t nmt;     // entry tiles (128 entries, or 256 for a pair)
    const uint32_t *vtab;  // per 32-digit chunk n: sum_u Mod_(32n+u) 128^u as 7 two's-complement words + sign word
    uint32_t *climbs;
    int32_t *csizes;
    int64_t cld, crs;
    int32_t cnlimbs;
};
// One product of a grouped reconstruction launch (its tiles start at entry tile 0).
struct ReconJob {
    CUtensorMap tmY, tmT;
    ReconArgs a;
};
// Hand-off between the two epilogue warps of a TMEM lane quadrant (per entry slots).
struct ReconXfer {
    uint64_t to1[4], to0[4], qready[4];  // mbarriers per quadrant: half 0 -> 1, half 1 -> 0, q ready
    long long carry1[128], carry0[128];  // carry handed to half 1 / to half 0
    uint32_t ripple1[128], ripple0[128]; // negation ripple handed on
    int32_t q[128], sgn[128], amb[128];  // fixed-point results of an entry's tile 0
    int32_t top0[128];                   // half 0's highest nonzero limb + 1
    uint32_t drop0[128];                 // half 0's dropped-limb flags (bit 0 nonzero, bit 1 all ones)
};

// Y's map is 3-D, [Ep/64 blocks][2P rows][64 entries]: the rows 2P .. 2Pp-1 of a
// block's last K step lie outside it and read as zeros.  GRP: a grouped launch;
// Mod's chunk values are then read from global memory (each product has its own),
// and the epilogue's hand-offs take the form that holds for any sequence of N-tile
// counts (see the half-0 wait at an entry tile's first N tile).
template <int STAGES, bool PAIR, bool GRP>
__global__ void __launch_bounds__(CTA_THREADS8, 1)
    k_crt_recon(const __grid_constant__ CUtensorMap tmY, const __grid_constant__ CUtensorMap tmT, ReconArgs a0,
                Group<ReconJob> grp, uint32_t *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = align1024(smem_raw);
    constexpr int NP = PAIR ? 2 : 1;
    constexpr int RBN = 256;                      // accumulator columns (table rows) per N tile
    constexpr int TROWS = RBN / NP;               // table rows this CTA stages per N tile
    constexpr uint32_t BOX = 64 * 128;            // one 64-entry x 64-row A box
    constexpr uint32_t A_BYTES = BM * 128, B_BYTES = TROWS * 128, STAGE = A_BYTES + B_BYTES;
    Barriers *bars = reinterpret_cast<Barriers *>(base + STAGES * STAGE);
    uint32_t *svtab = reinterpret_cast<uint32_t *>(reinterpret_cast<uint8_t *>(bars) + SMEM_BARS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = PAIR ? tc::cluster_rank() : 0;
    const int64_t t0 = PAIR ? (blockIdx.x >> 1) : blockIdx.x, tstep = PAIR ? (gridDim.x >> 1) : gridDim.x;
    const int vwords = GRP ? 0 : (a0.Dout + 31) / 32 * 8;
    for (int i = threadIdx.x; i < vwords; i += blockDim.x) svtab[i] = a0.vtab[i];
    ReconXfer *xf = reinterpret_cast<ReconXfer *>(svtab + vwords);
    // entry tiles [tbeg, total) in global numbering; tile_job maps one to its
    // product's arguments and maps and to the entry tile within that product
    const int64_t tbeg = GRP ? 0 : a0.mt0, total = GRP ? grp.tile0[grp.njobs] : a0.nmt;
    GroupCursor cur;
    auto tile_job = [&](int64_t T, ReconArgs &a, const CUtensorMap *&mY, const CUtensorMap *&mT) -> int64_t {
        if (GRP) {
            cur.seek(grp, T);
            const ReconJob *J = grp.jobs + cur.j;
            a = J->a;
            mY = &J->tmY;
            mT = &J->tmT;
            return T - cur.beg;
        }
        a = a0;
        mY = &tmY;
        mT = &tmT;
        return T;
    };
    if (threadIdx.x == 0)
        for (int qd = 0; qd < 4; qd++) {
            tc::mbar_init(&xf->to1[qd], 1);
            tc::mbar_init(&xf->to0[qd], 1);
            tc::mbar_init(&xf->qready[qd], 1);
        }
    if (PAIR) {
        if (threadIdx.x == 0) {
            for (int s = 0; s < STAGES; s++) {
                tc::mbar_init(&bars->full[s], 1);
                tc::mbar_init(&bars->empty[s], 1);
            }
            for (int b = 0; b < 2; b++) {
                tc::mbar_init(&bars->tfull[b], 1);
                tc::mbar_init(&bars->tempty[b], 16);  // the even CTA's: 8 epilogue warps of each CTA
            }
            bars->abort_flag = 0;
            tc::fence_mbar_init();
        }
        if (warp == 1) {
            tc::tmem_alloc_pair(&bars->tmem_base, 512);
            tc::tmem_relinquish_pair();
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // both CTAs' barriers exist before any cross-CTA signal
        tc::fence_after_sync();
    } else {
        cta_setup(bars, STAGES, 512, 1, 8);
    }
    tc::grid_dep_wait();  // the planes this launch reads are complete
    const uint32_t tmem = bars->tmem_base;

    if (warp == 0) {
        if (lane == 0) {
            if (!GRP) {
                tc::prefetch_tmap(&tmY);
                tc::prefetch_tmap(&tmT);
            }
            int it = 0;
            for (int64_t T = tbeg + t0; T < total && !aborted(bars); T += tstep) {
                ReconArgs a;
                const CUtensorMap *mY, *mT;
                const int64_t t = tile_job(T, a, mY, mT);
                const int blk0 = (int)(t * (2 * NP) + 2 * rank);  // this CTA's two 64-entry blocks
                for (int j = 0; j < a.NT && !aborted(bars); j++) {
                    for (int s = 0; s < a.nk; s++, it++) {
                        const int st = it % STAGES;
                        if (it >= STAGES && !tc::mbar_wait(&bars->empty[st], ((it / STAGES) & 1) ^ 1)) {
                            set_abort(bars, err);
                            break;
                        }
                        uint8_t *sa = base + st * STAGE;
                        // A (MN-major): two 64-entry blocks x 64 K-rows; blocks past the end of
                        // Y read as zeros and still count their full box bytes
                        if (PAIR) {
                            const uint32_t full0 = tc::mapa(tc::smem_u32(&bars->full[st]), 0);
                            if (rank == 0) tc::mbar_arrive_expect_tx(&bars->full[st], 2 * STAGE);
                            tc::tma_load_3d_pair(sa, mY, full0, 0, s * BK, blk0);
                            tc::tma_load_3d_pair(sa + BOX, mY, full0, 0, s * BK, blk0 + 1);
                            tc::tma_load_2d_pair(sa + A_BYTES, mT, full0, s * BK, j * RBN + (int)rank * TROWS);
                        } else {
                            tc::mbar_arrive_expect_tx(&bars->full[st], STAGE);
                            tc::tma_load_3d(sa, mY, &bars->full[st], 0, s * BK, blk0);
                            tc::tma_load_3d(sa + BOX, mY, &bars->full[st], 0, s * BK, blk0 + 1);
                            tc::tma_load_2d(sa + A_BYTES, mT, &bars->full[st], s * BK, j * RBN);
                        }
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {
            const uint32_t idesc = tc::idesc_bf16_f32(NP * BM, RBN, 1, 0);
            int it = 0, lt = 0;
            bool ok = true;
            for (int64_t T = tbeg + t0; T < total && ok; T += tstep) {
                ReconArgs a;
                const CUtensorMap *mY, *mT;
                tile_job(T, a, mY, mT);
                (void)mY, (void)mT;
                for (int j = 0; j < a.NT && ok; j++, lt++) {
                    const int b = lt & 1;
                    if (lt >= 2 && !tc::mbar_wait(&bars->tempty[b], ((lt >> 1) & 1) ^ 1)) {
                        set_abort(bars, err);
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t d = tmem + 256u * b;
                    for (int s = 0; s < a.nk; s++, it++) {
                        const int st = it % STAGES;
                        if (!tc::mbar_wait(&bars->full[st], (it / STAGES) & 1)) { set_abort(bars, err); ok = false; break; }
                        tc::fence_after_sync();
                        const uint32_t sa = tc::smem_u32(base + st * STAGE);
                        const uint64_t ad = tc::sdesc_mnmajor(sa, BOX), bd = tc::sdesc_kmajor(sa + A_BYTES);
#pragma unroll
                        for (int kk = 0; kk < BK / UK; kk++) {
                            const uint64_t adesc = tc::sdesc_advance(ad, kk * 2048), bdesc = tc::sdesc_advance(bd, kk * 32);
                            const uint32_t acc = s != 0 || kk != 0;
                            if (PAIR) tc::mma_bf16_pair(d, adesc, bdesc, idesc, acc);
                            else tc::mma_bf16(d, adesc, bdesc, idesc, acc);
                        }
                        if (PAIR) tc::mma_commit_pair(&bars->empty[st], 0x3);
                        else tc::mma_commit(&bars->empty[st]);
                    }
                    if (ok) {
                        if (PAIR) tc::mma_commit_pair(&bars->tfull[b], 0x3);
                        else tc::mma_commit(&bars->tfull[b]);
                    }
                }
            }
        }
    } else {
        // 8 epilogue warps.  quad = warp % 4 owns TMEM lanes (entries) quad * 32 .. + 31 and
        // hf = (warp - 2) / 4 owns accumulator columns hf * 128 .. + 127 of every N tile.  An
        // entry's digits run through its carry chain in the order (tile 0, half 0), (tile 0,
        // half 1), (tile 1, half 0), ...  Each half reads its 128 columns at once (so the
        // TMEM buffer goes back to the MMA immediately), turns them into up to 28 limbs
        // starting from carry 0, then takes its predecessor's carry and negation ripple from
        // shared memory, adds them, stores, and hands its own on.  Hand-offs are mbarriers
        // with bounded waits; the exchange slots are per entry.
        const int quad = warp & 3, hf = (warp - 2) >> 2, idx = quad * 32 + lane;
        const uint32_t lb = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(hf * 128);
        const uint32_t tempty0 = PAIR ? tc::mapa(tc::smem_u32(&bars->tempty[0]), 0) : 0;
        int lt = 0, ph1 = 0, ph0 = 0, phq = 0;  // tiles seen; hand-off phases consumed
        bool first = true, ok = true;
        for (int64_t T = tbeg + t0; T < total && ok; T += tstep) {
            ReconArgs a;
            const CUtensorMap *mY, *mT;
            const int64_t t = tile_job(T, a, mY, mT);
            (void)mY, (void)mT;
            // UNI: half 1 hands on at the end of an entry tile only after its finalize,
            // and half 0 takes that hand-off before it writes the next tile's slots (the
            // only order that is safe when N-tile counts vary from tile to tile); else
            // the one-N-tile case alone waits for the finalize
            const bool UNI = GRP || a.NT == 1;
            const int64_t e = t * (NP * BM) + rank * BM + quad * 32 + lane;
            const int64_t er = e / a.ncols, ec = e - er * a.ncols;
            const bool live = e < a.E && ec < a.ccols;
            const int64_t coff = live ? er * a.crs + ec : 0;
            // C = sum_u (acc_u - q Mod_u) 128^u; the limbs written are |C| (negated on the
            // fly when the fixed-point sum says C < 0)
            int32_t q = 0, sgn = 1, amb = 0;
            int top = 0;
            bool drop_nz = false, drop_ones = true;
            long long carry_final = 0;
            uint32_t nc_final = 1;
            const bool last_t = T + tstep >= total;
            for (int j = 0; j < a.NT; j++, lt++) {
                const int b = lt & 1;
                if (!tc::mbar_wait(&bars->tfull[b], (lt >> 1) & 1)) { set_abort(bars, err); ok = false; break; }
                tc::fence_after_sync();
                // columns 0..63 of this half now, 64..127 after two chunks (then the buffer is released)
                uint32_t g[64];
                tc::tmem_ld32(lb + (uint32_t)(256 * b), *reinterpret_cast<uint32_t(*)[32]>(&g[0]));
                tc::tmem_ld32(lb + (uint32_t)(256 * b + 32), *reinterpret_cast<uint32_t(*)[32]>(&g[32]));
                tc::tmem_ld_wait();
                bool took0 = false;  // half 0: the hand-off from half 1 is already taken
                if (j == 0) {
                    if (hf == 0) {
                        // the q, top0 and drop0 slots are free only once half 1 is done with
                        // the previous entry tile (its finalize included).  UNI: take that
                        // hand-off before writing them, so that the slots and qready never run
                        // a tile ahead.  Otherwise (the same N tiles, more than one, for every
                        // entry tile) the hand-off at j = 1 already orders them.
                        if (!first && UNI) {
                            if (!tc::mbar_wait(&xf->to0[quad], ph0 & 1)) { set_abort(bars, err); ok = false; break; }
                            ph0++;
                            took0 = true;
                        }
                        // fixed-point sum S = sum y_i 2^FIXB / p_i from the first SUSED columns
                        // (base 128): S = (q + C / Mod) 2^FIXB + err, |err| <= 128 P < 2^17, and
                        // |C / Mod| < 2^-18, so q = round(S / 2^FIXB) and the sign of
                        // frac = S - q 2^FIXB is the sign of C unless |C| < Mod 2^(20 - FIXB)
                        __int128 S = 0;
#pragma unroll
                        for (int u = SUSED - 1; u >= 0; u--) S = S * 128 + tc::acc_int(g[u]);
                        const __int128 halfw = (__int128)1 << (FIXB - 1);
                        const __int128 qq = (S + halfw) >> FIXB;
                        const __int128 frac = S - (qq << FIXB);
                        const __int128 tol = (__int128)1 << 20;
                        q = (int32_t)qq;
                        sgn = frac < -tol ? -1 : 1;
                        amb = frac <= tol && frac >= -tol;
                        xf->q[idx] = q;
                        xf->sgn[idx] = sgn;
                        xf->amb[idx] = amb;
                        __syncwarp();
                        if (lane == 0) tc::mbar_arrive(&xf->qready[quad]);
                    } else {
                        if (!tc::mbar_wait(&xf->qready[quad], phq & 1)) { set_abort(bars, err); ok = false; break; }
                        phq++;
                        q = xf->q[idx];
                        sgn = xf->sgn[idx];
                        amb = xf->amb[idx];
                    }
                }
                // this half's limbs from carry 0: chunks k = 0..3 are digit columns
                // pos = 256 j + 128 hf + 32 k - SROWS (32 digits = 7 limbs, on limb boundaries)
                uint32_t L[28];
                long long c = 0;
                int nl = 0;
                const int pos0 = 256 * j + 128 * hf - SROWS;
                const int k0 = pos0 < 0 ? 1 : 0;  // the fixed-point columns precede digit 0
                const int li0 = (pos0 + 32 * k0) / 32 * 7;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (k == 2) {
                        tc::tmem_ld32(lb + (uint32_t)(256 * b + 64), *reinterpret_cast<uint32_t(*)[32]>(&g[0]));
                        tc::tmem_ld32(lb + (uint32_t)(256 * b + 96), *reinterpret_cast<uint32_t(*)[32]>(&g[32]));
                        tc::tmem_ld_wait();
                        tc::fence_before_sync();
                        __syncwarp();
                        if (lane == 0) {
                            if (PAIR) tc::mbar_arrive_cluster(tempty0 + 8u * b);
                            else tc::mbar_arrive(&bars->tempty[b]);
                        }
                    }
                    const int pos = pos0 + 32 * k;
                    if (k < k0 || !live || pos >= a.Dout) continue;
                    const uint32_t *W = (GRP ? a.vtab : svtab) + (pos >> 5) * 8;
                    long long A[7];
                    A[0] = c;
#pragma unroll
                    for (int l = 1; l < 7; l++) A[l] = 0;
#pragma unroll
                    for (int u = 0; u < 32; u++)
                        A[(7 * u) >> 5] += (long long)tc::acc_int(g[32 * (k & 1) + u]) * (1LL << ((7 * u) & 31));
#pragma unroll
                    for (int l = 0; l < 7; l++) A[l] -= (long long)q * (long long)W[l];
#pragma unroll
                    for (int l = 0; l < 7; l++) {
                        if (l < 6) A[l + 1] += A[l] >> 32;
                        L[7 * k + l] = (uint32_t)A[l];
                    }
                    // the chunk's Mod value is sum W_l 2^(32 l) - s 2^224 (s = sign word)
                    c = (A[6] >> 32) + (W[7] ? (long long)q : 0LL);
                    nl = 7 * (k + 1);
                }
                // predecessor's carry and negation ripple: half 1 takes half 0's of the same
                // tile; half 0 takes half 1's of the previous tile (none at an entry's tile 0)
                long long cin = 0;
                uint32_t nin = 1;
                if (hf == 1) {
                    if (!tc::mbar_wait(&xf->to1[quad], ph1 & 1)) { set_abort(bars, err); ok = false; break; }
                    ph1++;
                    cin = xf->carry1[idx];
                    nin = xf->ripple1[idx];
                } else if (!first) {
                    if (!took0) {
                        if (!tc::mbar_wait(&xf->to0[quad], ph0 & 1)) { set_abort(bars, err); ok = false; break; }
                        ph0++;
                    }
                    if (j > 0) {
                        cin = xf->carry0[idx];
                        nin = xf->ripple0[idx];
                    }
                }
                first = false;
                // add the carry in, negate when C < 0, store
#pragma unroll
                for (int l = 0; l < 28; l++) {
                    if (l < k0 * 7 || l >= nl || cin == 0) continue;
                    const long long s = (long long)L[l] + cin;
                    L[l] = (uint32_t)s;
                    cin = s >> 32;
                }
                c += cin;
#pragma unroll
                for (int l = 0; l < 28; l++) {
                    if (l < k0 * 7 || l >= nl) continue;
                    uint32_t limb = L[l];
                    if (sgn < 0) {
                        const uint32_t nv = ~limb + nin;
                        nin &= (uint32_t)(limb == 0u);
                        limb = nv;
                    }
                    const int li = li0 + l - k0 * 7;
                    if (li < a.cnlimbs) {
                        a.climbs[(int64_t)li * a.cld + coff] = limb;
                        if (limb) top = li + 1;
                    } else {
                        drop_nz |= limb != 0u;
                        drop_ones &= limb == 0xFFFFFFFFu;
                    }
                }
                // hand on: half 0 -> half 1 of this tile; half 1 -> half 0 of the next tile
                // (also after an entry's last tile, except the CTA's very last one, so that
                // half 0 never runs two hand-offs ahead)
                if (hf == 0) {
                    xf->carry1[idx] = c;
                    xf->ripple1[idx] = nin;
                    if (j == a.NT - 1) {
                        xf->top0[idx] = top;
                        xf->drop0[idx] = (drop_nz ? 1u : 0u) | (drop_ones ? 2u : 0u);
                    }
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&xf->to1[quad]);
                } else {
                    if (j == a.NT - 1) {
                        carry_final = c;
                        nc_final = nin;
                    } else {
                        xf->carry0[idx] = c;
                        xf->ripple0[idx] = nin;
                    }
                    // after an entry's last N tile the hand-off waits for the finalize under
                    // UNI (see half 0's early take at j = 0)
                    if (j < a.NT - 1 || (!UNI && !last_t)) {
                        __syncwarp();
                        if (lane == 0) tc::mbar_arrive(&xf->to0[quad]);
                    }
                }
            }
            if (!ok) break;
            if (hf == 1 && live) {
                // finalize: half 0's top limb and dropped-limb flags arrived with its last hand-off
                top = max(top, xf->top0[idx]);
                const uint32_t d0 = xf->drop0[idx];
                drop_nz |= (d0 & 1u) != 0;
                drop_ones &= (d0 & 2u) != 0;
                const int nl = (a.Dout + 31) / 32 * 7;  // limbs produced
                const int written = nl < a.cnlimbs ? nl : a.cnlimbs;
                int neg = sgn < 0;
                // bits above the produced limbs of the written value: C's own, or -C's
                long long carry = neg ? -carry_final - 1 + (long long)nc_final : carry_final;
                if (carry < 0) {
                    // only reachable on the ambiguous path: two's complement -> magnitude
                    if (!amb || carry != -1 || (nl > a.cnlimbs && !(drop_ones && top != 0)))
                        atomicOr(err, DEVERR_CAPACITY);
                    uint32_t cc = 1;
                    top = 0;
                    for (int l0 = 0; l0 < written; l0 += 8) {
                        uint32_t w[8];
#pragma unroll
                        for (int u = 0; u < 8; u++)
                            w[u] = l0 + u < written ? a.climbs[(int64_t)(l0 + u) * a.cld + coff] : 0u;
#pragma unroll
                        for (int u = 0; u < 8; u++) {
                            if (l0 + u >= written) break;
                            const uint64_t sum = (uint64_t)(~w[u]) + cc;
                            const uint32_t r = (uint32_t)sum;
                            cc = (uint32_t)(sum >> 32);
                            a.climbs[(int64_t)(l0 + u) * a.cld + coff] = r;
                            if (r) top = l0 + u + 1;
                        }
                    }
                    neg = 1;
                } else if (carry != 0 || drop_nz) {
                    atomicOr(err, DEVERR_CAPACITY);
                }
                for (int li = written; li < a.cnlimbs; li++) a.climbs[(int64_t)li * a.cld + coff] = 0u;
                a.csizes[coff] = top == 0 ? 0 : (neg ? -top : top);
            }
            if (hf == 1 && !last_t && UNI) {
                // the finalize is done with half 0's slots: hand on to half 0's next entry tile
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&xf->to0[quad]);
            }
        }
    }
    tc::grid_dep_launch();
    if (PAIR) {
        tc::fence_before_sync();
        __syncthreads();
        tc::cluster_sync_all();  // no CTA leaves while its peer may still signal it or write its TMEM
        if (warp == 1) {
            tc::fence_after_sync();
            tc::tmem_dealloc_pair(tmem, 512);
        }
    } else {
        cta_teardown(bars, 512);
    }
}

// ======================================================================================
// tcgen05 GEMM self-test: D[M x N] (int32) = A * B^T with A K-major [M x K] or
// MN-major [K x M], B K-major [N x K]; used by tests to pin the descriptor
// layouts independently of the CRT arithmetic.
// ======================================================================================
struct TestArgs {
    int32_t M, N, nk, a_mn;
    int32_t *D;
    // failure-path test knobs: the producer leaves K step `skip_step` unloaded and
    // its stage barrier unarmed (-1: none), and every wait gives up after
    // `wait_limit` SM clocks
    int32_t skip_step;
    long long wait_limit;
};

template <int STAGES>
__global__ void __launch_bounds__(CTA_THREADS, 1)
    k_gemm_test(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TestArgs a,
                uint32_t *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = align1024(smem_raw);
    constexpr uint32_t A_BYTES = BM * 128, B_BYTES = BM * 128, STAGE = A_BYTES + B_BYTES;
    Barriers *bars = reinterpret_cast<Barriers *>(base + STAGES * STAGE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BM;
    cta_setup(bars, STAGES, 128, 1, 1);
    const uint32_t tmem = bars->tmem_base;
    const long long lim = a.wait_limit;
    if (warp == 0) {
        if (lane == 0) {
            int issued = 0;  // K steps whose loads were issued: steps [0, issued) except skip_step
            for (int s = 0; s < a.nk; s++) {
                const int st = s % STAGES;
                if (s >= STAGES && !tc::mbar_wait(&bars->empty[st], ((s / STAGES) & 1) ^ 1, lim)) {
                    set_abort(bars, err);
                    break;
                }
                issued = s + 1;
                if (s == a.skip_step) continue;  // nothing arms this stage: its consumer's wait runs out
                uint8_t *sa = base + st * STAGE;
                tc::mbar_arrive_expect_tx(&bars->full[st], STAGE);
                if (a.a_mn) {
                    tc::tma_load_2d(sa, &tmA, &bars->full[st], m0, s * BK);
                    tc::tma_load_2d(sa + A_BYTES / 2, &tmA, &bars->full[st], m0 + 64, s * BK);
                } else {
                    tc::tma_load_2d(sa, &tmA, &bars->full[st], s * BK, m0);
                }
                tc::tma_load_2d(sa + A_BYTES, &tmB, &bars->full[st], s * BK, n0);
            }
            if (aborted(bars)) {
                // before the CTA's shared memory goes away: wait (bounded) until the
                // copies of the last stages issued have landed
                for (int s = issued - 1; s >= 0 && s >= issued - STAGES; s--)
                    if (s != a.skip_step) tc::mbar_wait(&bars->full[s % STAGES], (s / STAGES) & 1, lim);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16_f32(BM, BM, a.a_mn, 0);
            bool ok = true;
            int mma_steps = 0;
            for (int s = 0; s < a.nk; s++) {
                const int st = s % STAGES;
                if (!tc::mbar_wait(&bars->full[st], (s / STAGES) & 1, lim)) { set_abort(bars, err); ok = false; break; }
                mma_steps++;
                tc::fence_after_sync();
                const uint32_t sa = tc::smem_u32(base + st * STAGE), sb = sa + A_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / UK; kk++) {
                    const uint64_t ad =
                        a.a_mn ? tc::sdesc_mnmajor(sa + kk * 2048, A_BYTES / 2) : tc::sdesc_kmajor(sa + kk * 32);
                    tc::mma_bf16(tmem, ad, tc::sdesc_kmajor(sb + kk * 32), idesc, s != 0 || kk != 0);
                }
                tc::mma_commit(&bars->empty[st]);
            }
            if (ok) tc::mma_commit(&bars->tfull[0]);
            else if (mma_steps > 0) {
                // MMAs already issued still write TMEM: wait (bounded) for them before teardown frees it
                tc::mma_commit(&bars->tfull[1]);
                tc::mbar_wait(&bars->tfull[1], 0, lim);
            }
        }
    } else {
        const int row = epi_row();
        bool ok = tc::mbar_wait(&bars->tfull[0], 0, lim);
        if (!ok) set_abort(bars, err);
        tc::fence_after_sync();
        const uint32_t lb = lane_base(tmem);
        for (int c0 = 0; c0 < BM && ok; c0 += 32) {
            uint32_t v[32];
            tc::tmem_ld32(lb + (uint32_t)c0, v);
            tc::tmem_ld_wait();
            const int m = m0 + row;
            if (m < a.M)
                for (int j = 0; j < 32; j++)
                    if (n0 + c0 + j < a.N) a.D[(int64_t)m * a.N + n0 + c0 + j] = tc::acc_int(v[j]);
        }
    }
    cta_teardown(bars, 128);
}

// ======================================================================================
// CTA-pair GEMM self-test: D[M x N] (int32) = A * B^T, A K-major [M x K], B
// K-major [N x K], one 256 x 256 tile per cluster of two CTAs.  The even CTA
// issues tcgen05.mma.cta_group::2 (M = 256, N = 256): each CTA holds its own 128
// rows of A and its own 128 rows of B at the same shared-memory offsets, and
// its TMEM receives its 128 rows of D.  Both CTAs' TMA loads complete on the
// even CTA's stage barrier; the MMA's commit arrives on both CTAs' barriers.
// ======================================================================================
constexpr uint32_t PAIR_TMEM_COLS = 256;
template <int STAGES>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(CTA_THREADS, 1)
    k_gemm_test_pair(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TestArgs a,
                     uint32_t *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = align1024(smem_raw);
    constexpr uint32_t A_BYTES = BM * 128, B_BYTES = BM * 128, STAGE = A_BYTES + B_BYTES;
    Barriers *bars = reinterpret_cast<Barriers *>(base + STAGES * STAGE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = tc::cluster_rank();
    const int tile = blockIdx.x >> 1, tiles_x = (a.N + 255) / 256;
    const int ty = tile / tiles_x, tx = tile % tiles_x;
    const int m0 = ty * 256 + (int)rank * BM, n0 = tx * 256 + (int)rank * BM;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(&bars->full[s], 1);
            tc::mbar_init(&bars->empty[s], 1);
        }
        tc::mbar_init(&bars->tfull[0], 1);
        bars->abort_flag = 0;
        tc::fence_mbar_init();
    }
    if (warp == 1) {
        tc::tmem_alloc_pair(&bars->tmem_base, PAIR_TMEM_COLS);
        tc::tmem_relinquish_pair();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::cluster_sync_all();  // both CTAs' barriers exist before any cross-CTA signal
    tc::fence_after_sync();
    const uint32_t tmem = bars->tmem_base;
    if (threadIdx.x == 0 && rank == 1) {
        // the pair's MMA writes D at the even CTA's TMEM address: both must agree
        uint32_t lead;
        asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(lead) : "r"(tc::mapa(tc::smem_u32(&bars->tmem_base), 0)));
        if (lead != tmem) atomicOr(err, DEVERR_BADARG);
    }

    if (warp == 0) {
        if (lane == 0) {
            for (int s = 0; s < a.nk; s++) {
                const int st = s % STAGES;
                if (s >= STAGES && !tc::mbar_wait(&bars->empty[st], ((s / STAGES) & 1) ^ 1)) {
                    set_abort(bars, err);
                    break;
                }
                uint8_t *sa = base + st * STAGE;
                const uint32_t full_lead = tc::mapa(tc::smem_u32(&bars->full[st]), 0);
                if (rank == 0) tc::mbar_arrive_expect_tx(&bars->full[st], 2 * STAGE);
                tc::tma_load_2d_pair(sa, &tmA, full_lead, s * BK, m0);
                tc::tma_load_2d_pair(sa + A_BYTES, &tmB, full_lead, s * BK, n0);
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {
            const uint32_t idesc = tc::idesc_bf16_f32(2 * BM, 2 * BM, 0, 0);
            bool ok = true;
            for (int s = 0; s < a.nk; s++) {
                const int st = s % STAGES;
                if (!tc::mbar_wait(&bars->full[st], (s / STAGES) & 1)) { set_abort(bars, err); ok = false; break; }
                tc::fence_after_sync();
                const uint32_t sa = tc::smem_u32(base + st * STAGE), sb = sa + A_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / UK; kk++)
                    tc::mma_bf16_pair(tmem, tc::sdesc_kmajor(sa + kk * 32), tc::sdesc_kmajor(sb + kk * 32), idesc,
                                      s != 0 || kk != 0);
                tc::mma_commit_pair(&bars->empty[st], 0x3);
            }
            if (ok) tc::mma_commit_pair(&bars->tfull[0], 0x3);
        }
    } else {
        const int row = (int)rank * BM + epi_row();
        const int m = ty * 256 + row;
        const uint32_t lb = lane_base(tmem);
        if (tc::mbar_wait(&bars->tfull[0], 0)) {
            tc::fence_after_sync();
            for (int c0 = 0; c0 < 256; c0 += 32) {
                uint32_t v[32];
                tc::tmem_ld32(lb + (uint32_t)c0, v);
                tc::tmem_ld_wait();
                if (m < a.M) {
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        if (tx * 256 + c0 + j < a.N) a.D[(int64_t)m * a.N + tx * 256 + c0 + j] = tc::acc_int(v[j]);
                }
            }
        } else {
            set_abort(bars, err);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::cluster_sync_all();  // no CTA leaves while its peer may still signal it or write its TMEM
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc_pair(tmem, PAIR_TMEM_COLS);
    }
}

// ======================================================================================
// host side
// ======================================================================================
typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                     const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static PFN_encodeTiled get_encode() {
    static PFN_encodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_encodeTiled>(p);
    });
    return fn;
}

// 2-D bf16 tensor map: inner dimension `inner` (contiguous), `outer` rows with
// a pitch of `pitch_elems`; box = box_inner x box_outer, 128-byte swizzle.
static gbmm_status make_map(CUtensorMap *m, const void *ptr, uint64_t inner, uint64_t outer, uint64_t pitch_elems,
                            uint32_t box_inner, uint32_t box_outer) {
    PFN_encodeTiled enc = get_encode();
    if (!enc) return set_error(GBMM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (pitch_elems * 2) % 16)
        return set_error(GBMM_ERR_INVALID, "tensor map base or pitch not 16-byte aligned");
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {pitch_elems * 2};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GBMM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return GBMM_OK;
}

// Residue planes [nplanes][rows][pitch] bf16 as a 3-D map for the residue epilogue's
// TMA stores: boxes of 32 entries x 1 row x 32 planes, no swizzle.
static gbmm_status make_map_planes(CUtensorMap *m, const void *ptr, uint64_t cols, uint64_t rows, uint64_t nplanes,
                                   uint64_t pitch_elems, uint64_t plane_elems) {
    PFN_encodeTiled enc = get_encode();
    if (!enc) return set_error(GBMM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (pitch_elems * 2) % 16 || (plane_elems * 2) % 16)
        return set_error(GBMM_ERR_INVALID, "tensor map base or pitch not 16-byte aligned");
    cuuint64_t dims[3] = {cols, rows, nplanes};
    cuuint64_t strides[2] = {pitch_elems * 2, plane_elems * 2};
    cuuint32_t box[3] = {32, 1, 32};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GBMM_ERR_CUDA, "cuTensorMapEncodeTiled (planes) failed (%d)", (int)r);
    return GBMM_OK;
}

// ---- host big integers (tables only) ---------------------------------------------------------
typedef std::vector<uint32_t> big;  // little-endian 32-bit limbs
static void big_mul_small(big &x, uint32_t m) {
    uint64_t c = 0;
    for (auto &l : x) {
        uint64_t t = (uint64_t)l * m + c;
        l = (uint32_t)t;
        c = t >> 32;
    }
    if (c) x.push_back((uint32_t)c);
}
static big big_div_small(const big &x, uint32_t d, uint32_t *rem) {
    big q(x.size());
    uint64_t r = 0;
    for (size_t i = x.size(); i-- > 0;) {
        uint64_t cur = (r << 32) | x[i];
        q[i] = (uint32_t)(cur / d);
        r = cur % d;
    }
    while (!q.empty() && q.back() == 0) q.pop_back();
    if (rem) *rem = (uint32_t)r;
    return q;
}
static uint32_t big_mod_small(const big &x, uint32_t d) {
    uint64_t r = 0;
    for (size_t i = x.size(); i-- > 0;) r = ((r << 32) | x[i]) % d;
    return (uint32_t)r;
}
// balanced base-128 digits (each in [-64, 63]) of a nonnegative integer: digit t
// takes bits [7t, 7t + 7) plus the carry of the digit below.  32 digits span
// exactly 7 words, so each chunk of 32 reads its words once and extracts the
// digits with fixed shifts; the carry is one compare per digit.
static void balanced128(const big &x, int ndig, int *out) {
    const size_t nw = x.size();
    int c = 0;
    for (int t0 = 0; t0 < ndig; t0 += 32) {
        const size_t w0 = (size_t)(t0 / 32) * 7;
        uint64_t w[8];
        for (int k = 0; k < 8; k++) w[k] = w0 + k < nw ? x[w0 + k] : 0;
        const int lim = std::min(32, ndig - t0);
        for (int u = 0; u < 32; u++) {
            if (u >= lim) break;
            const int bit = 7 * u;
            const int b = (int)(((w[bit >> 5] | (w[(bit >> 5) + 1] << 32)) >> (bit & 31)) & 127u);
            const int v = b + c;
            c = v >= 64;
            out[t0 + u] = v - (c << 7);
        }
    }
}
static std::vector<int> balanced128(const big &x, int ndig) {
    std::vector<int> out(ndig, 0);
    balanced128(x, ndig, out.data());
    return out;
}
static uint32_t inv_mod(uint32_t a, uint32_t p) {
    int64_t t = 0, nt = 1, r = p, nr = a % p;
    while (nr) {
        int64_t q = r / nr;
        int64_t tmp = t - q * nt; t = nt; nt = tmp;
        tmp = r - q * nr; r = nr; nr = tmp;
    }
    if (t < 0) t += p;
    return (uint32_t)t;
}
static const std::vector<uint32_t> &primes_desc() {
    static std::vector<uint32_t> pr;
    static std::once_flag once;
    std::call_once(once, [] {
        std::vector<char> sieve(65536, 1);
        sieve[0] = sieve[1] = 0;
        for (int i = 2; i * i < 65536; i++)
            if (sieve[i])
                for (int j = i * i; j < 65536; j += i) sieve[j] = 0;
        for (int i = 65535; i >= 3; i--)
            if (sieve[i]) pr.push_back((uint32_t)i);
    });
    return pr;
}

static uint16_t bf16_bits(float f) {
    __nv_bfloat16 h = __float2bfloat16_rn(f);
    uint16_t b;
    memcpy(&b, &h, 2);
    return b;
}
// bf16 bits of the integers -256 .. 256 (every table digit lies in this range)
static uint16_t bf16_small(int v) {
    static const std::vector<uint16_t> lut = [] {
        std::vector<uint16_t> l(513);
        for (int i = -256; i <= 256; i++) l[i + 256] = bf16_bits((float)i);
        return l;
    }();
    return lut[v + 256];
}

struct crt_cache;
struct crt_tables {
    crt_cache *cache = nullptr;  // the cache that holds these tables (and the shared residue table)
    int P = 0, Pp = 0;   // moduli, padded 2P/2 (2Pp multiple of 64)
    int Dout = 0, NT = 0;
    __nv_bfloat16 *d_recon = nullptr;  // [NT * RTAB][2Pp]
    uint32_t *d_vtab = nullptr;        // [ceil(Dout / 32)][8]: Mod's digits per 32-digit chunk
    std::map<int, __nv_bfloat16 *> residue;  // 2 * dxp + weighted -> [2P rows][dxp]
    std::vector<ModConst> h_mods;
};

struct crt_cache {
    std::mutex mu;
    std::map<int, crt_tables *> by_p;
    // the unweighted residue table of every modulus (256^j mod p_i for all 1024
    // moduli and every digit position an operand can have): each product's
    // unweighted table is a view of it (its first moduli, its first dxp columns)
    __nv_bfloat16 *d_res_all = nullptr;
    ~crt_cache() {
        cudaFree(d_res_all);
        for (auto &kv : by_p) {
            crt_tables *t = kv.second;
            cudaFree(t->d_recon);
            cudaFree(t->d_vtab);
            for (auto &r : t->residue) cudaFree(r.second);
            delete t;
        }
    }
};

crt_cache *crt_cache_create() { return new crt_cache(); }
void crt_cache_destroy(crt_cache *c) { delete c; }

// number of moduli for a product bound of `bits` bits (plus margin)
static int moduli_for_bits(int64_t bits) {
    const auto &pr = primes_desc();
    double acc = 0;
    int n = 0;
    while (acc < (double)bits && n < (int)pr.size()) acc += std::log2((double)pr[n++]);
    return acc >= (double)bits ? n : -1;
}

// Host side of a table set: moduli constants, the reconstruction table, Mod's
// chunk values and the constant (p, 1/p) list.
struct crt_tables_host {
    int P = 0, Pp = 0, Dout = 0, NT = 0;
    std::vector<ModConst> mods;
    std::vector<uint16_t> recon;  // [NT * RTAB][2Pp] bf16 bits
    std::vector<uint32_t> vtab;   // [ceil(Dout / 32)][8]
    std::vector<float> cmod;      // 4 * CMOD_PAIRS
};

static void build_tables_host(int P, crt_tables_host &o) {
    const auto &pr = primes_desc();
    o.P = P;
    o.Pp = (2 * P + 63) / 64 * 32;
    big Mod{1};
    for (int i = 0; i < P; i++) big_mul_small(Mod, pr[i]);
    int modbits = (int)(32 * Mod.size());
    o.Dout = (modbits + 6) / 7 + 2;  // base-128 output digits
    o.NT = (SROWS + o.Dout + RTAB - 1) / RTAB;  // in units of RTAB rows
    const int rows = o.NT * RTAB, cols = 2 * o.Pp;
    o.recon.assign((size_t)rows * cols, bf16_bits(0.f));
    std::vector<uint16_t> &tab = o.recon;
    o.mods.resize(P);
    // the moduli are independent: contiguous ranges of them on up to 16 host threads
    // (each writes its own table columns)
    // The moduli are independent: blocks of MB on up to 16 host threads.  A block's
    // digits go to a small row-major buffer first and then into the table row by
    // row, 2 MB adjacent columns at a time (writing one column at a time would
    // touch a new cache line with every 2-byte store).
    constexpr int MB = 32;
    auto block = [&](int i0, int i1, std::vector<int8_t> &dig, std::vector<int> &tmp) {
        const int nb = i1 - i0;
        for (int q = 0; q < nb; q++) {
            const int i = i0 + q;
            const uint32_t p = pr[i];
            uint32_t rem = 0;
            big Mi = big_div_small(Mod, p, &rem);
            big Mi256 = Mi;
            big_mul_small(Mi256, 256);
            const uint32_t w = inv_mod(big_mod_small(Mi, p), p);
            ModConst mc;
            memset(&mc, 0, sizeof mc);
            mc.p = (int32_t)p;
            mc.inv_p = 1.0f / (float)p;
            mc.mu = (uint32_t)(((uint64_t)1 << 32) / p);
            mc.h16 = (uint32_t)((1u << 16) % p);
            mc.w = w;
            o.mods[i] = mc;
            // column 2i multiplies the high digit (x256), column 2i+1 the low digit
            balanced128(Mi256, o.Dout, tmp.data());
            for (int r = 0; r < o.Dout; r++) dig[(size_t)r * (2 * MB) + 2 * q] = (int8_t)tmp[r];
            balanced128(Mi, o.Dout, tmp.data());
            for (int r = 0; r < o.Dout; r++) dig[(size_t)r * (2 * MB) + 2 * q + 1] = (int8_t)tmp[r];
            // fixed-point weights: round(2^(FIXB+8) / p) for the high digit, round(2^FIXB / p) for the low digit
            const unsigned __int128 one = 1;
            const unsigned __int128 gh = ((one << (FIXB + 8)) + p / 2) / p;
            const unsigned __int128 gl = ((one << FIXB) + p / 2) / p;
            big bh, bl;
            for (int w2 = 0; w2 < 4; w2++) {
                bh.push_back((uint32_t)(gh >> (32 * w2)));
                bl.push_back((uint32_t)(gl >> (32 * w2)));
            }
            std::vector<int> sh = balanced128(bh, SUSED), sl = balanced128(bl, SUSED);
            for (int r = 0; r < SUSED; r++) {
                tab[(size_t)r * cols + 2 * i] = bf16_small(sh[r]);
                tab[(size_t)r * cols + 2 * i + 1] = bf16_small(sl[r]);
            }
        }
        for (int r = 0; r < o.Dout; r++) {
            uint16_t *row = &tab[(size_t)(SROWS + r) * cols + 2 * i0];
            const int8_t *src = &dig[(size_t)r * (2 * MB)];
            for (int c = 0; c < 2 * nb; c++) row[c] = bf16_small(src[c]);
        }
    };
    const int nblocks = (P + MB - 1) / MB;
    const int nthr = std::max(1, std::min<int>({16, (int)std::thread::hardware_concurrency(), nblocks}));
    auto range = [&](int th) {
        std::vector<int8_t> dig((size_t)o.Dout * 2 * MB);
        std::vector<int> tmp(o.Dout);
        for (int bk = th; bk < nblocks; bk += nthr) block(bk * MB, std::min(P, (bk + 1) * MB), dig, tmp);
    };
    if (nthr == 1) {
        range(0);
    } else {
        std::vector<std::thread> pool;
        for (int th = 1; th < nthr; th++) pool.emplace_back(range, th);
        range(0);
        for (auto &th : pool) th.join();
    }
    // Mod's balanced base-128 digits, summed per 32-digit chunk n into the 224-bit
    // value V_n = sum_u Mod_(32n+u) 128^u, kept as 8 words of a 256-bit two's
    // complement number (|V_n| < 2^223, so word 7 is the sign extension)
    std::vector<int> md = balanced128(Mod, o.Dout);
    const int nch = (o.Dout + 31) / 32;
    o.vtab.assign((size_t)nch * 8, 0u);
    for (int n = 0; n < nch; n++) {
        uint32_t *w = &o.vtab[(size_t)n * 8];
        for (int u = 0; u < 32; u++) {
            const int r = 32 * n + u;
            if (r >= o.Dout || md[r] == 0) continue;
            const int bit = 7 * u, k = bit / 32;
            const uint64_t v = (uint64_t)((int64_t)md[r] * ((int64_t)1 << (bit % 32)));  // two's complement
            uint32_t add[8];
            for (int kk = 0; kk < 8; kk++) add[kk] = md[r] < 0 ? 0xFFFFFFFFu : 0u;
            for (int kk = 0; kk < k; kk++) add[kk] = 0u;
            add[k] = (uint32_t)v;
            if (k + 1 < 8) add[k + 1] = (uint32_t)(v >> 32);
            uint64_t c = 0;
            for (int kk = 0; kk < 8; kk++) {
                const uint64_t sum = (uint64_t)w[kk] + add[kk] + c;
                w[kk] = (uint32_t)sum;
                c = sum >> 32;
            }
        }
    }
    // the constant (p, 1/p) list: the same for every table, written with each
    o.cmod.resize(4 * CMOD_PAIRS);
    for (int q = 0; q < CMOD_PAIRS; q++) {
        o.cmod[4 * q] = (float)pr[2 * q];
        o.cmod[4 * q + 1] = (float)pr[2 * q + 1];
        o.cmod[4 * q + 2] = 1.0f / (float)pr[2 * q];
        o.cmod[4 * q + 3] = 1.0f / (float)pr[2 * q + 1];
    }
}

static gbmm_status build_tables(crt_tables *t, int P) {
    crt_tables_host o;
    build_tables_host(P, o);
    t->P = o.P;
    t->Pp = o.Pp;
    t->Dout = o.Dout;
    t->NT = o.NT;
    t->h_mods = o.mods;
    // every upload has landed before the tables are used (kernels that use them may
    // run on any stream)
    {
        cudaStream_t cs = copy_stream();
        if (!cs) return set_error(GBMM_ERR_CUDA, "no copy stream");
        GBMM_CUDA_TRY(cudaMemcpyToSymbolAsync(c_modpair, o.cmod.data(), o.cmod.size() * sizeof(float), 0,
                                              cudaMemcpyHostToDevice, cs));
        GBMM_CUDA_TRY(cudaStreamSynchronize(cs));
    }
    GBMM_CUDA_TRY(cudaMalloc(&t->d_recon, o.recon.size() * 2));
    GBMM_TRY(upload_now(t->d_recon, o.recon.data(), o.recon.size() * 2));
    GBMM_CUDA_TRY(cudaMalloc(&t->d_vtab, o.vtab.size() * 4));
    GBMM_TRY(upload_now(t->d_vtab, o.vtab.data(), o.vtab.size() * 4));
    return GBMM_OK;
}

// Residue table [2P rows][dxp]: rows 2i / 2i+1 hold the low / high balanced
// byte of 256^j mod p_i (weighted = 0) or of w_i 256^j mod p_i (weighted = 1, the
// CRT weight w_i = (Mod/p_i)^-1 mod p_i folded into the B operand).
// GEMM columns of the residue table for P moduli: two per modulus, padded to whole pairs
static int residue_cols(int P) { return (2 * P + 3) / 4 * 4; }
// Digit positions an operand's rows can have: four groups of 15 K steps of 64.
constexpr int RES_DXMAX = 4 * RES_GROUP_STEPS_B * BK;
// Fills rows [2P padded][dxp] of a residue table (pitch `pitch`) for moduli 0..P-1.
static void residue_rows(const crt_tables *t, int P, int dxp, int pitch, int weighted, uint16_t *tab);
// The table of this product and operand: the unweighted one is a view of the
// cache's shared table (pitch RES_DXMAX), the weighted one is built per (P, dxp).
static gbmm_status residue_table(crt_tables *t, int dxp, int weighted, __nv_bfloat16 **out, int *pitch) {
    if (!weighted) {
        crt_cache *c = t->cache;
        if (!c->d_res_all) {
            const int rows = residue_cols(2 * CMOD_PAIRS);
            std::vector<uint16_t> tab((size_t)rows * RES_DXMAX, 0);
            residue_rows(t, 2 * CMOD_PAIRS, RES_DXMAX, RES_DXMAX, 0, tab.data());
            __nv_bfloat16 *d = nullptr;
            GBMM_CUDA_TRY(cudaMalloc(&d, tab.size() * 2));
            GBMM_TRY(upload_now(d, tab.data(), tab.size() * 2));
            c->d_res_all = d;
        }
        *out = c->d_res_all;
        *pitch = RES_DXMAX;
        return GBMM_OK;
    }
    *pitch = dxp;
    const int key = 2 * dxp + weighted;
    auto it = t->residue.find(key);
    if (it != t->residue.end()) { *out = it->second; return GBMM_OK; }
    std::vector<uint16_t> tab((size_t)residue_cols(t->P) * dxp, 0);
    residue_rows(t, t->P, dxp, dxp, 1, tab.data());
    __nv_bfloat16 *d = nullptr;
    GBMM_CUDA_TRY(cudaMalloc(&d, tab.size() * 2));
    GBMM_TRY(upload_now(d, tab.data(), tab.size() * 2));
    t->residue[key] = d;
    *out = d;
    return GBMM_OK;
}

// Rows (table columns of the GEMM) in groups of four per pair of moduli (i, i + 1):
// [lo_i, lo_i+1, hi_i, hi_i+1]; with P odd the last group's second slot stays zero.
// In the shared table every slot holds its modulus; a product with P odd then
// computes one residue past its moduli in the padding column of its last pair,
// bounded like the others and never stored.
static void residue_rows(const crt_tables *t, int P, int dxp, int pitch, int weighted, uint16_t *tab) {
    const auto &pr = primes_desc();
    auto range = [&](int i0, int i1) {
        for (int i = i0; i < i1; i++) {
            const uint32_t p = pr[i];
            const size_t r_lo = (size_t)4 * (i >> 1) + (i & 1), r_hi = r_lo + 2;
            uint32_t v = weighted ? t->h_mods[i].w : 1u;  // (w) 256^j mod p
            for (int j = 0; j < dxp; j++) {
                int32_t b = v > p / 2 ? (int32_t)v - (int32_t)p : (int32_t)v;
                int32_t d0 = ((b + 128) & 255) - 128;
                int32_t d1 = (b - d0) / 256;
                tab[r_lo * pitch + j] = bf16_small(d0);  // x1
                tab[r_hi * pitch + j] = bf16_small(d1);  // x256
                v = (uint32_t)(((uint64_t)v * 256) % p);
            }
        }
    };
    // the moduli's rows are independent: contiguous ranges on up to 16 host threads
    const int nthr = std::max(1, std::min<int>({16, (int)std::thread::hardware_concurrency(), (P * dxp) >> 16}));
    if (nthr == 1) {
        range(0, P);
    } else {
        std::vector<std::thread> pool;
        for (int th = 1; th < nthr; th++) pool.emplace_back(range, (int)((int64_t)P * th / nthr), (int)((int64_t)P * (th + 1) / nthr));
        range(0, P / nthr);
        for (auto &th : pool) th.join();
    }
}

static gbmm_status get_tables(crt_cache *c, int P, crt_tables **out) {
    std::lock_guard<std::mutex> lk(c->mu);
    auto it = c->by_p.find(P);
    if (it != c->by_p.end()) { *out = it->second; return GBMM_OK; }
    crt_tables *t = new crt_tables();
    t->cache = c;
    gbmm_status st = build_tables(t, P);
    if (st != GBMM_OK) { delete t; return st; }
    c->by_p[P] = t;
    *out = t;
    return GBMM_OK;
}

static constexpr int RES_STAGES = 4, PROD_STAGES = 4, REC_STAGES = 4, TEST_STAGES = 4;
static constexpr int REC_STAGES_PAIR = 6;  // a pair CTA stages 32 KB per K step
static constexpr int RES_STAGES_PAIR = 5;  // a pair CTA stages 32 KB per K step
static constexpr int PROD_STAGES_PAIR = 5;  // a pair CTA stages 40 KB per K step
static constexpr int PROD_PAIR_MIN_NK = 8;  // K steps (of 64) from which the product runs on CTA pairs
// residue GEMM form: -1 by the K loop's length, 0 single CTAs, 1 CTA pairs
static int g_residue_mode = -1;  // -1 by size, 0 one CTA, 1 CTA pairs, 2 multicast clusters
static constexpr int RES_PAIR_MIN_NK = 1 << 30;  // the pair form of the residue GEMM measured slower at every size
static bool residue_pair(int nk) { return g_residue_mode < 0 ? nk >= RES_PAIR_MIN_NK : g_residue_mode == 1; }
static bool residue_mc(int nk) { (void)nk; return g_residue_mode == 2; }

static int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 148;
    }
    return n;
}
static size_t smem_bytes(int stages, size_t stage_bytes) { return stages * stage_bytes + SMEM_BARS + 1024 + 64; }

static gbmm_status set_smem(const void *fn, size_t bytes) {
    GBMM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return GBMM_OK;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Programmatic dependent launch: every kernel of the four CRT stages is launched
// with programmatic stream serialization, so its CTAs may be scheduled, set up
// their barriers and allocate TMEM while the kernel before it in the stream
// finishes its last tiles.  Each of them calls tc::grid_dep_wait() before its
// first global-memory access and tc::grid_dep_launch() when its work is issued.
// A kernel's dependences on other streams (events) stay full dependences.
static bool g_pdl = true;

static void set_pdl(cudaLaunchAttribute &at) {
    at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
}

// Launch of one of the four stages' kernels on plain CTAs.
template <typename... KArgs, typename... Args>
static gbmm_status launch_one(void (*kern)(KArgs...), dim3 grid, int threads, size_t smem, cudaStream_t s,
                              Args &&...args) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cudaLaunchAttribute attr[1];
    set_pdl(attr[0]);
    cfg.gridDim = grid;
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = g_pdl ? 1 : 0;
    GBMM_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
    return GBMM_OK;
}

// Launch of a persistent kernel in clusters of two CTAs (one CTA per SM): the
// grid is as many pairs as can be resident at once (GPCs with an odd number of
// free SMs leave one SM without a partner), capped by the work.
template <typename... KArgs, typename... Args>
static gbmm_status launch_pairs(void (*kern)(KArgs...), int threads, int64_t work_pairs, size_t smem, cudaStream_t s,
                                Args &&...args) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3((unsigned)(2 * std::max<int>(1, num_sms() / 2)));
    int resident = 0;
    GBMM_CUDA_TRY(cudaOccupancyMaxActiveClusters(&resident, (const void *)kern, &cfg));
    if (resident < 1) return set_error(GBMM_ERR_UNSUPPORTED, "no CTA pair of this kernel fits on the device");
    cfg.gridDim = dim3((unsigned)(2 * std::min<int64_t>(work_pairs, resident)));
    set_pdl(attr[1]);
    cfg.numAttrs = g_pdl ? 2 : 1;
    GBMM_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
    return GBMM_OK;
}

// ---- launch plans of the four stages (one product, or one record of a grouped launch) ----------

// digit-row length of an operand's entries: 4 digits per limb, padded to 64
static int operand_dxp(const gbmm_mat &X) { return (4 * std::max(X.nlimbs, 1) + 63) / 64 * 64; }
static size_t digits_bytes(const gbmm_mat &X) { return (size_t)X.rows * X.cols * operand_dxp(X) * 2 + 1024; }

// Digits + residues of one operand into planes [2P][rowsR][kp] (A: a1, a0 per
// modulus); B's table is weighted, so B's planes hold u = w b (u1, u0).  Only
// the first kdim columns of each plane row are written.
struct OperandPlan {
    DigitArgs da;
    dim3 dgrid;
    int balanced = 0, gsteps = 0;
    bool pair = false, mc = false;
    CUtensorMap tmD, tmT, tmR;
    ResidueArgs ra;
    size_t smem = 0;
};
static gbmm_status plan_operand(crt_tables *t, const gbmm_mat &X, int transpose, int rowsR, int kdim, int kp, int weighted,
                                __nv_bfloat16 *R, __nv_bfloat16 *D, bool grouped, OperandPlan &op) {
    const int dxp = operand_dxp(X);
    const int64_t E = (int64_t)X.rows * X.cols;
    if (E > (int64_t)INT32_MAX - 4 * BM) return set_error(GBMM_ERR_UNSUPPORTED, "crt: more than 2^31 entries in one operand");
    const int nk = dxp / BK;
    // unsigned byte digits up to 512 per row; longer rows in balanced digits, whose
    // groups are nearly twice as long (fewer groups, wider table tiles)
    op.balanced = nk > RES_GROUP_STEPS_U;
    op.gsteps = op.balanced ? RES_GROUP_STEPS_B : RES_GROUP_STEPS_U;
    DigitArgs &a = op.da;
    memset(&a, 0, sizeof a);
    a.limbs = X.limbs; a.sizes = X.sizes; a.ld = X.ld; a.rs = X.rs; a.rows = X.rows; a.cols = X.cols;
    a.nlimbs = X.nlimbs; a.transpose = transpose; a.dxp = dxp; a.out = D;
    op.dgrid = dim3((unsigned)((X.cols + 31) / 32), (unsigned)((X.rows + 3) / 4), (unsigned)((dxp / 4 + 63) / 64));
    __nv_bfloat16 *T = nullptr;
    int tpitch = dxp;
    GBMM_TRY(residue_table(t, dxp, weighted, &T, &tpitch));
    const int G = (nk + op.gsteps - 1) / op.gsteps;
    int BN = 256;
    while (BN * G > 256) BN /= 2;
    if (BN < 64) return set_error(GBMM_ERR_UNSUPPORTED, "crt: entries longer than 30720 bits");
    op.pair = !grouped && residue_pair(nk);
    op.mc = !grouped && !op.pair && residue_mc(nk);
    const int NP = op.pair || op.mc ? 2 : 1;
    GBMM_TRY(make_map(&op.tmD, D, dxp, E, dxp, BK, BM));
    GBMM_TRY(make_map(&op.tmT, T, dxp, residue_cols(t->P), tpitch, BK, BN / NP));
    ResidueArgs &r = op.ra;
    memset(&r, 0, sizeof r);
    r.kdim = kdim; r.E = (int32_t)E; r.nk = nk;
    r.BN = BN; r.G = G; r.P = t->P; r.R = R; r.plane = (int64_t)rowsR * kp; r.kp = kp;
    r.ncols = residue_cols(t->P);
    r.n_ntiles = (r.ncols + BN - 1) / BN;
    r.ntiles = (int32_t)((int64_t)r.n_ntiles * ((E + NP * BM - 1) / (NP * BM)));
    // 32-entry boxes of one plane row: [32 planes][1 row][32 entries]
    r.tma_out = kdim % 32 == 0;
    if (r.tma_out) GBMM_TRY(make_map_planes(&op.tmR, R, kdim, rowsR, 2 * t->P, kp, r.plane));
    else op.tmR = op.tmD;  // unused
    // a grouped launch sizes every stage for 256 table columns
    const int bcols = grouped ? 256 : (op.pair ? BN / 2 : BN);
    op.smem = smem_bytes(op.pair ? RES_STAGES_PAIR : RES_STAGES, BM * 128 + (size_t)bcols * 128) +
              (size_t)RES_EPI_WARPS * (op.pair ? 2 : 1) * RES_STG_BYTES;
    return GBMM_OK;
}

static gbmm_status launch_operand(const OperandPlan &op, cudaStream_t s) {
    {
        LaunchScope ls_("k_crt_digits", s);
        const Group<DigitJob> none{nullptr, nullptr, 0};
        if (op.balanced) GBMM_TRY(launch_one(k_crt_digits<true, false>, op.dgrid, 256, 0, s, op.da, none));
        else GBMM_TRY(launch_one(k_crt_digits<false, false>, op.dgrid, 256, 0, s, op.da, none));
        GBMM_CUDA_TRY(cudaGetLastError());
    }
    const Group<ResidueJob> none{nullptr, nullptr, 0};
    const size_t sm = op.smem;
    LaunchScope ls_("k_crt_residue", s);
#define RESIDUE_LAUNCH(GS_)                                                                                          \
    do {                                                                                                             \
        if (op.mc) {                                                                                                 \
            GBMM_TRY(set_smem((const void *)k_crt_residue<RES_STAGES, false, true, GS_, false>, sm));                \
            GBMM_TRY(launch_pairs(k_crt_residue<RES_STAGES, false, true, GS_, false>, RES_THREADS, op.ra.ntiles, sm, \
                                  s, op.tmD, op.tmT, op.tmR, op.ra, none, device_error_word()));                     \
        } else if (op.pair) {                                                                                        \
            GBMM_TRY(set_smem((const void *)k_crt_residue<RES_STAGES_PAIR, true, false, GS_, false>, sm));           \
            GBMM_TRY(launch_pairs(k_crt_residue<RES_STAGES_PAIR, true, false, GS_, false>, RES_THREADS,            \
                                  op.ra.ntiles, sm, s, op.tmD, op.tmT, op.tmR, op.ra, none, device_error_word()));   \
        } else {                                                                                                     \
            GBMM_TRY(set_smem((const void *)k_crt_residue<RES_STAGES, false, false, GS_, false>, sm));               \
            dim3 grid((unsigned)std::min<int64_t>(op.ra.ntiles, num_sms()));                                         \
            GBMM_TRY(launch_one(k_crt_residue<RES_STAGES, false, false, GS_, false>, grid, RES_THREADS, sm, s,      \
                                op.tmD, op.tmT, op.tmR, op.ra, none, device_error_word()));                          \
        }                                                                                                            \
    } while (0)
    if (op.gsteps == RES_GROUP_STEPS_B) RESIDUE_LAUNCH(RES_GROUP_STEPS_B);
    else RESIDUE_LAUNCH(RES_GROUP_STEPS_U);
#undef RESIDUE_LAUNCH
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

// Product GEMM over residue planes RA [2P][m][kp] and RB [2P][n][kp].  The maps'
// inner extent is k, not kp: the columns k .. kp-1 of the last K step lie outside
// and read as zeros, so the planes need no cleared padding.
struct ProductPlan {
    CUtensorMap tmA, tmB;
    ProductArgs pa;
    bool pair = false;
    size_t smem = 0;
};
static gbmm_status plan_product(crt_tables *t, __nv_bfloat16 *RA, __nv_bfloat16 *RB, __nv_bfloat16 *Y, int m, int k, int n,
                                int kp, int npad, int tiles, bool grouped, ProductPlan &pp) {
    const int P = t->P;
    GBMM_TRY(make_map(&pp.tmA, RA, k, (uint64_t)2 * P * m, kp, BK, BM));
    GBMM_TRY(make_map(&pp.tmB, RB, k, (uint64_t)2 * P * n, kp, BK, PBX));
    ProductArgs &pa = pp.pa;
    memset(&pa, 0, sizeof pa);
    pa.m = m; pa.n = n; pa.npad = npad; pa.nk = kp / BK; pa.P = P; pa.Y = Y;
    pa.yblk = (int64_t)2 * t->Pp * 64;
    // CTA pairs pay off once the K loop is long enough to hide the pair's per-tile
    // synchronisation (measured: faster at k = 512, slower at k = 256); a plan may
    // fix the form (tiles: 1 one-CTA tiles, 2 CTA pairs); grouped launches use one-CTA tiles
    pp.pair = !grouped && (tiles == 0 ? pa.nk >= PROD_PAIR_MIN_NK : tiles == 2);
    const int NP = pp.pair ? 2 : 1;
    pa.nyt = (m + NP * BM - 1) / (NP * BM);
    pa.nxt = (n + PBX - 1) / PBX;
    pa.ntiles = (int64_t)P * pa.nyt * pa.nxt;
    pp.smem = pp.pair ? smem_bytes(PROD_STAGES_PAIR, 2 * BM * 128 + PBX * 128)
                      : smem_bytes(PROD_STAGES, 2 * BM * 128 + 2 * PBX * 128);
    return GBMM_OK;
}

static gbmm_status launch_product(const ProductPlan &pp, cudaStream_t s) {
    const Group<ProductJob> none{nullptr, nullptr, 0};
    uint32_t *err = device_error_word();
    LaunchScope ls_("k_crt_product", s);
    if (pp.pair) {
        GBMM_TRY(set_smem((const void *)k_crt_product<PROD_STAGES_PAIR, true, false>, pp.smem));
        GBMM_TRY(launch_pairs(k_crt_product<PROD_STAGES_PAIR, true, false>, CTA_THREADS8, pp.pa.ntiles, pp.smem, s,
                              pp.tmA, pp.tmB, pp.pa, none, err));
    } else {
        GBMM_TRY(set_smem((const void *)k_crt_product<PROD_STAGES, false, false>, pp.smem));
        dim3 grid((unsigned)std::min<int64_t>(pp.pa.ntiles, num_sms()));
        GBMM_TRY(launch_one(k_crt_product<PROD_STAGES, false, false>, grid, CTA_THREADS8, pp.smem, s, pp.tmA, pp.tmB,
                            pp.pa, none, err));
    }
    GBMM_CUDA_TRY(cudaGetLastError());
    return GBMM_OK;
}

// Y as a 3-D map [Ep/64 blocks][2P rows][64 entries] with a block pitch of 2Pp
// rows: boxes of 64 entries x 64 rows; rows 2P .. 2Pp-1 read as zeros.
static gbmm_status make_map_yblocks(CUtensorMap *m, const void *ptr, uint64_t rows, uint64_t rows_pitch, uint64_t blocks) {
    PFN_encodeTiled enc = get_encode();
    if (!enc) return set_error(GBMM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    if (reinterpret_cast<uintptr_t>(ptr) & 15) return set_error(GBMM_ERR_INVALID, "tensor map base not 16-byte aligned");
    cuuint64_t dims[3] = {64, rows, blocks};
    cuuint64_t strides[2] = {64 * 2, rows_pitch * 64 * 2};
    cuuint32_t box[3] = {64, (cuuint32_t)BK, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GBMM_ERR_CUDA, "cuTensorMapEncodeTiled (Y blocks) failed (%d)", (int)r);
    return GBMM_OK;
}

// Reconstruction of C (m x n, Y's entries in rows of npad) from Y.
struct ReconPlan {
    CUtensorMap tmY, tmT;
    ReconArgs ra;
    bool pair = false;
    size_t smem = 0;
};
static gbmm_status plan_recon(crt_tables *t, __nv_bfloat16 *Y, int m, int n, int npad, const gbmm_mat &c, int tiles,
                              bool grouped, ReconPlan &rp) {
    const int64_t E = (int64_t)m * npad, Ep = (E + 63) / 64 * 64;
    GBMM_TRY(make_map_yblocks(&rp.tmY, Y, (uint64_t)2 * t->P, (uint64_t)2 * t->Pp, (uint64_t)(Ep / 64)));
    // CTA pairs once the K loop over the 2Pp moduli digits is long enough (see the
    // product), unless the plan fixes the form; grouped launches use CTA pairs
    rp.pair = grouped || (tiles == 0 ? 2 * t->Pp / BK >= PROD_PAIR_MIN_NK : tiles == 2);
    const int NP = rp.pair ? 2 : 1, TROWS = 256 / NP;
    GBMM_TRY(make_map(&rp.tmT, t->d_recon, 2 * t->Pp, (uint64_t)t->NT * RTAB, 2 * t->Pp, BK, TROWS));
    ReconArgs &ra = rp.ra;
    memset(&ra, 0, sizeof ra);
    ra.E = E; ra.ncols = npad; ra.ccols = n; ra.nk = 2 * t->Pp / BK; ra.NT = (SROWS + t->Dout + 255) / 256;
    ra.Dout = t->Dout; ra.vtab = t->d_vtab; ra.climbs = c.limbs; ra.csizes = c.sizes; ra.cld = c.ld; ra.crs = c.rs;
    ra.cnlimbs = c.nlimbs; ra.kpad = 2 * t->Pp;
    ra.mt0 = 0;
    ra.nmt = (E + NP * BM - 1) / (NP * BM);
    // a grouped launch reads Mod's chunk values from global memory
    const size_t extra = (grouped ? 0 : (size_t)(t->Dout + 31) / 32 * 32) + sizeof(ReconXfer) + 64;
    rp.smem = smem_bytes(rp.pair ? REC_STAGES_PAIR : REC_STAGES, BM * 128 + TROWS * 128) + extra;
    return GBMM_OK;
}

int crt_moduli(int64_t bits_a, int64_t bits_b, int k) {
    int lg = 0;
    while ((1LL << lg) < std::max(k, 1)) lg++;
    return moduli_for_bits(bits_a + bits_b + lg + 2 + 16);
}

// device workspace (bytes) of one single-pass product: residue planes, Y, and
// digits (one operand's at a time, or both when `both_digits`)
static size_t crt_workspace(const gbmm_mat &a, const gbmm_mat &b, int64_t bits_a, int64_t bits_b, int nprimes,
                            bool both_digits) {
    const int m = a.rows, k = a.cols, n = b.cols;
    int P = nprimes > 0 ? nprimes : crt_moduli(bits_a, bits_b, k);
    if (P <= 0) return 0;
    const int Pp = (2 * P + 63) / 64 * 32;
    const int kp = (k + 63) / 64 * 64;
    const int64_t Ep = ((int64_t)m * ((n + YPAD - 1) / YPAD * YPAD) + 63) / 64 * 64;
    const size_t da = align256(digits_bytes(a)), db = align256(digits_bytes(b));
    return align256((size_t)2 * P * m * kp * 2) + align256((size_t)2 * P * n * kp * 2) + align256((size_t)2 * Pp * Ep * 2) +
           (both_digits ? da + db : std::max(da, db)) + 8192;
}

bool crt_feasible(int la, int lb, int k) {
    const int P = crt_moduli(32LL * la, 32LL * lb, std::min(k, PROD_MAX_K));
    // at most four residue accumulation groups: digit rows of up to 4 * 15 * 64 digits
    return P > 0 && P <= 1023 && 4 * std::max(la, lb) <= 4 * RES_GROUP_STEPS_B * BK;
}

static gbmm_mat shape_only(int rows, int cols, int nlimbs) {
    gbmm_mat x;
    memset(&x, 0, sizeof x);
    x.rows = rows; x.cols = cols; x.nlimbs = nlimbs;
    return x;
}

size_t crt_workspace_bytes(int la, int lb, int m, int k, int n, int cn) {
    const int kc = std::min(k, PROD_MAX_K);
    size_t ws = crt_workspace(shape_only(m, kc, la), shape_only(kc, n, lb), 32LL * la, 32LL * lb, 0, false);
    // an accumulating chunk adds a product-sized temporary
    if (k > kc) ws += align256((size_t)m * n * (std::max(cn, la + lb + 4) + 1) * 4) + 8192;
    return ws;
}

bool crt_single_pass(int k) { return k <= PROD_MAX_K; }

gbmm_status crt_matmul(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int64_t bits_a,
                       int64_t bits_b, int nprimes, int accumulate, cudaStream_t s) {
    const int m = a.rows, k = a.cols, n = b.cols;
    // stage hooks apply to this product only; any branch but the single-pass one
    // waits for B at once and runs the reconstruction whole
    crt_stage_hooks *hk = h->stage;
    h->stage = nullptr;
    if (hk && (m == 0 || n == 0 || k == 0 || accumulate || k > PROD_MAX_K)) {
        if (hk->b_ready) GBMM_CUDA_TRY(cudaStreamWaitEvent(s, hk->b_ready, 0));
        hk = nullptr;
    }
    if (m == 0 || n == 0) return GBMM_OK;
    if (k == 0) return accumulate ? GBMM_OK : launch_mat_zero(c, s);
    if (accumulate) {
        // C += A*B: product into a workspace matrix, then one elementwise add
        size_t mark = arena_mark(h);
        const int cn = std::max(c.nlimbs, (int)((bits_a + bits_b + 64) / 32) + 2);
        size_t need = align256((size_t)m * n * cn * 4) + align256((size_t)m * n * 4) + 4096;
        GBMM_TRY(arena_reserve(h, need + crt_workspace(a, b, bits_a, bits_b, nprimes, false)));
        gbmm_mat T;
        T.rows = m; T.cols = n; T.nlimbs = cn; T.pad_ = 0; T.rs = n; T.ld = (int64_t)m * n;
        T.limbs = (uint32_t *)arena_alloc(h, (size_t)m * n * cn * 4);
        T.sizes = (int32_t *)arena_alloc(h, (size_t)m * n * 4);
        if (!T.limbs || !T.sizes) return set_error(GBMM_ERR_NOMEM, "crt: accumulate workspace");
        gbmm_status st = crt_matmul(h, T, a, b, bits_a, bits_b, nprimes, 0, s);
        if (st == GBMM_OK) st = launch_mat_addsub(c, c, T, 0, s);
        arena_release(h, mark);
        return st;
    }
    if (k > PROD_MAX_K) {
        // inner dimension in chunks of 512: C = A_0 B_0, then C += A_j B_j
        for (int k0 = 0; k0 < k; k0 += PROD_MAX_K) {
            const int kc = std::min(PROD_MAX_K, k - k0);
            gbmm_mat ac = sub_view(a, 0, k0, m, kc), bc = sub_view(b, k0, 0, kc, n);
            GBMM_TRY(crt_matmul(h, c, ac, bc, bits_a, bits_b, nprimes, k0 > 0, s));
        }
        return GBMM_OK;
    }
    int P = nprimes > 0 ? nprimes : crt_moduli(bits_a, bits_b, k);
    // one exact FP32 accumulation in the reconstruction covers 2P * 2^13 < 2^24
    if (P <= 0 || P > 1023)
        return set_error(GBMM_ERR_UNSUPPORTED, "crt: product bound needs %d moduli (at most 1023)", P);
    crt_tables *t = nullptr;
    GBMM_TRY(get_tables(h->crt, P, &t));
    if (!get_encode()) return set_error(GBMM_ERR_CUDA, "crt: no tensor-map encoder");

    const int kp = (k + 63) / 64 * 64;  // residue-plane row pitch (TMA needs 16-byte pitches)
    // Y's entries: rows of C times n padded to whole groups of 16 (the product
    // GEMM's epilogue then stores only whole 32-byte runs)
    const int npad = (n + YPAD - 1) / YPAD * YPAD;
    const int64_t E = (int64_t)m * npad;
    const int64_t Ep = (E + 63) / 64 * 64;
    GBMM_TRY(arena_reserve(h, crt_workspace(a, b, bits_a, bits_b, P, false)));
    size_t mark = arena_mark(h);
    __nv_bfloat16 *RA = (__nv_bfloat16 *)arena_alloc(h, (size_t)2 * P * m * kp * 2);
    __nv_bfloat16 *RB = (__nv_bfloat16 *)arena_alloc(h, (size_t)2 * P * n * kp * 2);
    __nv_bfloat16 *Y = (__nv_bfloat16 *)arena_alloc(h, (size_t)2 * t->Pp * Ep * 2);
    if (!RA || !RB || !Y) return set_error(GBMM_ERR_NOMEM, "crt: workspace");
    // Nothing is cleared: the product reads RA / RB through maps k columns wide and
    // Y through a map 2P rows deep per 64-entry block, and the padding entries
    // E .. Ep-1 of Y only reach accumulator rows that are never stored.
    {
        size_t mk = arena_mark(h);
        OperandPlan op;
        __nv_bfloat16 *D = (__nv_bfloat16 *)arena_alloc(h, digits_bytes(a));
        if (!D) return set_error(GBMM_ERR_NOMEM, "crt: workspace for digits");
        GBMM_TRY(plan_operand(t, a, 0, m, k, kp, 0, RA, D, false, op));
        GBMM_TRY(launch_operand(op, s));
        arena_release(h, mk);
        if (hk && hk->b_ready) GBMM_CUDA_TRY(cudaStreamWaitEvent(s, hk->b_ready, 0));
        D = (__nv_bfloat16 *)arena_alloc(h, digits_bytes(b));
        if (!D) return set_error(GBMM_ERR_NOMEM, "crt: workspace for digits");
        GBMM_TRY(plan_operand(t, b, 1, n, k, kp, 1, RB, D, false, op));
        GBMM_TRY(launch_operand(op, s));
        arena_release(h, mk);
    }
    {
        ProductPlan pp;
        GBMM_TRY(plan_product(t, RA, RB, Y, m, k, n, kp, npad, h->crt_tiles, false, pp));
        GBMM_TRY(launch_product(pp, s));
    }
    {
        ReconPlan rp;
        GBMM_TRY(plan_recon(t, Y, m, n, npad, c, h->crt_tiles, false, rp));
        ReconArgs ra = rp.ra;
        const int64_t nmt = ra.nmt;
        const Group<ReconJob> none{nullptr, nullptr, 0};
        uint32_t *err = device_error_word();
        if (rp.pair) GBMM_TRY(set_smem((const void *)k_crt_recon<REC_STAGES_PAIR, true, false>, rp.smem));
        else GBMM_TRY(set_smem((const void *)k_crt_recon<REC_STAGES, false, false>, rp.smem));
        const int NP = rp.pair ? 2 : 1;
        // one launch, or (stage hooks) entry ranges each followed by an event
        const int parts = hk ? (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)hk->parts, (int64_t)CRT_MAX_PARTS, nmt})) : 1;
        for (int pi = 0; pi < parts; pi++) {
            ra.mt0 = nmt * pi / parts;
            ra.nmt = nmt * (pi + 1) / parts;
            LaunchScope ls_("k_crt_recon", s);
            if (rp.pair) {
                GBMM_TRY(launch_pairs(k_crt_recon<REC_STAGES_PAIR, true, false>, CTA_THREADS8, ra.nmt - ra.mt0, rp.smem, s,
                                      rp.tmY, rp.tmT, ra, none, err));
            } else {
                dim3 grid((unsigned)std::min<int64_t>(ra.nmt - ra.mt0, num_sms()));
                GBMM_TRY(launch_one(k_crt_recon<REC_STAGES, false, false>, grid, CTA_THREADS8, rp.smem, s, rp.tmY,
                                    rp.tmT, ra, none, err));
            }
            GBMM_CUDA_TRY(cudaGetLastError());
            if (hk && parts > 1) {
                GBMM_CUDA_TRY(cudaEventRecord(hk->part_ev[pi], s));
                // entries of C (dense, row-major) done after this part: Y's entries below
                // ra.nmt * NP * BM, mapped back through the padded row length
                const int64_t ye = std::min<int64_t>(E, ra.nmt * NP * BM);
                hk->part_end[pi] = std::min<int64_t>((int64_t)m * n, (ye / npad) * n + std::min<int64_t>(ye % npad, n));
            }
        }
        if (hk && parts > 1) hk->parts_done = parts;
    }
    arena_release(h, mark);
    return GBMM_OK;
}

// ---- grouped launches -------------------------------------------------------------------------
// The CRT products of a batch, collected without launching: every product's
// workspace is carved at once, its stage records go into per-stage lists, and
// each stage then runs as ONE persistent launch per kernel form over the tiles of
// all products (digits and residues by digit form, products on one-CTA tiles,
// reconstructions on CTA pairs).  Records are ordered by the cost of one tile,
// largest first, so that the long tiles start in the first wave.
struct crt_group {
    struct Rec {
        std::vector<char> bytes;  // one record
        int64_t tiles = 0;
        double cost = 0;  // per tile
    };
    // dig by digit form (unsigned, balanced); res by accumulation groups: unsigned
    // digits (one group), balanced with one group (256-column table tiles), balanced
    // with several (table tiles of 128 or 64 columns, a deeper ring of smaller
    // stages); rec[1]: products with a post step
    std::vector<Rec> dig[2], res[3], prod, rec[2];
    std::vector<std::function<gbmm_status(cudaStream_t)>> post;
    struct Sect {
        size_t jobs_off = 0, tile0_off = 0;
        int n = 0;
        int64_t total = 0;
    };
    Sect sdig[2], sres[3], sprod, srec[2];
    size_t smem_prod = 0, smem_rec = 0;
    std::vector<char> blob;
};

crt_group *crt_group_create() { return new crt_group(); }
void crt_group_destroy(crt_group *g) { delete g; }
bool crt_group_empty(const crt_group *g) { return g->prod.empty() && g->post.empty(); }
void crt_group_post(crt_group *g, std::function<gbmm_status(cudaStream_t)> f) { g->post.push_back(std::move(f)); }

size_t crt_group_ws(int la, int lb, int m, int k, int n) {
    return crt_workspace(shape_only(m, k, la), shape_only(k, n, lb), 32LL * la, 32LL * lb, 0, true) + 2048;
}

template <typename J>
static crt_group::Rec make_rec(const J &j, int64_t tiles, double cost) {
    crt_group::Rec r;
    r.bytes.resize(sizeof(J));
    memcpy(r.bytes.data(), &j, sizeof(J));
    r.tiles = tiles;
    r.cost = cost;
    return r;
}

gbmm_status crt_group_add(gbmm_handle h, crt_group *g, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b,
                          int64_t bits_a, int64_t bits_b, int nprimes, const crt_halves *halves) {
    const int m = a.rows, k = a.cols, n = b.cols;
    if (m == 0 || n == 0 || k == 0 || k > PROD_MAX_K)
        return set_error(GBMM_ERR_UNSUPPORTED, "crt group: needs a nonempty single-pass product");
    const int P = nprimes > 0 ? nprimes : crt_moduli(bits_a, bits_b, k);
    if (P <= 0 || P > 1023)
        return set_error(GBMM_ERR_UNSUPPORTED, "crt: product bound needs %d moduli (at most 1023)", P);
    crt_tables *t = nullptr;
    GBMM_TRY(get_tables(h->crt, P, &t));
    if (!get_encode()) return set_error(GBMM_ERR_CUDA, "crt: no tensor-map encoder");
    const int kp = (k + 63) / 64 * 64;
    const int npad = (n + YPAD - 1) / YPAD * YPAD;
    const int64_t Ep = ((int64_t)m * npad + 63) / 64 * 64;
    __nv_bfloat16 *RA = (__nv_bfloat16 *)arena_alloc(h, (size_t)2 * P * m * kp * 2);
    __nv_bfloat16 *RB = (__nv_bfloat16 *)arena_alloc(h, (size_t)2 * P * n * kp * 2);
    __nv_bfloat16 *Y = (__nv_bfloat16 *)arena_alloc(h, (size_t)2 * t->Pp * Ep * 2);
    __nv_bfloat16 *DA = (__nv_bfloat16 *)arena_alloc(h, digits_bytes(a));
    __nv_bfloat16 *DB = (__nv_bfloat16 *)arena_alloc(h, digits_bytes(b));
    if (!RA || !RB || !Y || !DA || !DB) return set_error(GBMM_ERR_NOMEM, "crt group: workspace");
    for (int side = 0; side < 2; side++) {
        OperandPlan op;
        if (side == 0) GBMM_TRY(plan_operand(t, a, 0, m, k, kp, 0, RA, DA, true, op));
        else GBMM_TRY(plan_operand(t, b, 1, n, k, kp, 1, RB, DB, true, op));
        if (halves && halves->side == side) {
            // the stacked operand's digit rows straight from x's two limb halves: the
            // high half's rows follow the low half's (A: rows m.., B: columns n..); both
            // halves carry x's sign, and digits past a half's limbs read as zeros
            const gbmm_mat &x = halves->x;
            const int64_t xe = (int64_t)x.rows * x.cols;
            for (int hf = 0; hf < 2; hf++) {
                DigitJob dj;
                memset(&dj, 0, sizeof dj);
                dj.a = op.da;
                dj.a.limbs = x.limbs + (hf ? (int64_t)halves->hl * x.ld : 0);
                dj.a.sizes = x.sizes;
                dj.a.ld = x.ld;
                dj.a.rs = x.rs;
                dj.a.rows = x.rows;
                dj.a.cols = x.cols;
                dj.a.nlimbs = hf ? x.nlimbs - halves->hl : halves->hl;
                dj.a.out = op.da.out + (hf ? xe * op.da.dxp : 0);
                dj.nbx = (x.cols + 31) / 32;
                dj.nby = (x.rows + 3) / 4;
                g->dig[op.balanced].push_back(make_rec(dj, (int64_t)dj.nbx * dj.nby * op.dgrid.z, 1.0));
            }
        } else {
            DigitJob dj;
            memset(&dj, 0, sizeof dj);
            dj.a = op.da;
            dj.nbx = (int32_t)op.dgrid.x;
            dj.nby = (int32_t)op.dgrid.y;
            g->dig[op.balanced].push_back(make_rec(dj, (int64_t)op.dgrid.x * op.dgrid.y * op.dgrid.z, 1.0));
        }
        ResidueJob rj;
        memset(&rj, 0, sizeof rj);
        rj.tmD = op.tmD; rj.tmT = op.tmT; rj.tmR = op.tmR; rj.a = op.ra;
        const int rf = op.gsteps == RES_GROUP_STEPS_U ? 0 : (op.ra.BN > 128 ? 1 : 2);
        g->res[rf].push_back(make_rec(rj, op.ra.ntiles, (double)op.ra.nk * op.ra.BN));
    }
    ProductPlan pp;
    GBMM_TRY(plan_product(t, RA, RB, Y, m, k, n, kp, npad, 0, true, pp));
    ProductJob pj;
    memset(&pj, 0, sizeof pj);
    pj.tmA = pp.tmA; pj.tmB = pp.tmB; pj.a = pp.pa;
    g->prod.push_back(make_rec(pj, pp.pa.ntiles, (double)pp.pa.nk));
    g->smem_prod = std::max(g->smem_prod, pp.smem);
    ReconPlan rp;
    GBMM_TRY(plan_recon(t, Y, m, n, npad, c, 0, true, rp));
    ReconJob rj;
    memset(&rj, 0, sizeof rj);
    rj.tmY = rp.tmY; rj.tmT = rp.tmT; rj.a = rp.ra;
    g->rec[halves ? 1 : 0].push_back(make_rec(rj, rp.ra.nmt, (double)rp.ra.NT * rp.ra.nk));
    g->smem_rec = std::max(g->smem_rec, rp.smem);
    return GBMM_OK;
}

// One stage's records, largest tile cost first, then their tile offsets.
static void pack_section(std::vector<char> &blob, std::vector<crt_group::Rec> &recs, crt_group::Sect &sec) {
    std::stable_sort(recs.begin(), recs.end(),
                     [](const crt_group::Rec &x, const crt_group::Rec &y) { return x.cost > y.cost; });
    sec.n = (int)recs.size();
    sec.total = 0;
    if (recs.empty()) return;
    blob.resize((blob.size() + 127) & ~(size_t)127);
    sec.jobs_off = blob.size();
    for (const auto &r : recs) blob.insert(blob.end(), r.bytes.begin(), r.bytes.end());
    blob.resize((blob.size() + 127) & ~(size_t)127);
    sec.tile0_off = blob.size();
    std::vector<int64_t> t0(recs.size() + 1, 0);
    for (size_t i = 0; i < recs.size(); i++) t0[i + 1] = t0[i] + recs[i].tiles;
    sec.total = t0.back();
    const char *p = reinterpret_cast<const char *>(t0.data());
    blob.insert(blob.end(), p, p + t0.size() * sizeof(int64_t));
}

const std::vector<char> &crt_group_blob(crt_group *g) {
    g->blob.clear();
    for (int f = 0; f < 2; f++) pack_section(g->blob, g->dig[f], g->sdig[f]);
    for (int f = 0; f < 3; f++) pack_section(g->blob, g->res[f], g->sres[f]);
    pack_section(g->blob, g->prod, g->sprod);
    for (int f = 0; f < 2; f++) pack_section(g->blob, g->rec[f], g->srec[f]);
    return g->blob;
}

template <typename J>
static Group<J> group_at(const char *d_blob, const crt_group::Sect &sec) {
    return Group<J>{reinterpret_cast<const J *>(d_blob + sec.jobs_off),
                    reinterpret_cast<const int64_t *>(d_blob + sec.tile0_off), sec.n};
}

gbmm_status crt_group_launch(crt_group *g, const char *d_blob, cudaStream_t s, cudaStream_t s2, cudaEvent_t ev) {
    if (reinterpret_cast<uintptr_t>(d_blob) & 127) return set_error(GBMM_ERR_INVALID, "crt group: blob not 128-byte aligned");
    uint32_t *err = device_error_word();
    static const CUtensorMap zmap = {};
    for (int f = 0; f < 2; f++) {
        const crt_group::Sect &sec = g->sdig[f];
        if (!sec.n) continue;
        if (sec.total > INT32_MAX) return set_error(GBMM_ERR_UNSUPPORTED, "crt group: too many digit blocks");
        DigitArgs none;
        memset(&none, 0, sizeof none);
        LaunchScope ls_("k_crt_digits", s);
        const dim3 grid((unsigned)sec.total);
        if (f) GBMM_TRY(launch_one(k_crt_digits<true, true>, grid, 256, 0, s, none, group_at<DigitJob>(d_blob, sec)));
        else GBMM_TRY(launch_one(k_crt_digits<false, true>, grid, 256, 0, s, none, group_at<DigitJob>(d_blob, sec)));
        GBMM_CUDA_TRY(cudaGetLastError());
    }
    // residue GEMMs: 4 stages of 48 KB for 256-column table tiles, 6 of 32 KB for
    // operands whose several accumulation groups narrow the tiles to 128 columns
    static constexpr int RES_STAGES_NARROW = 6;
    for (int f = 0; f < 3; f++) {
        const crt_group::Sect &sec = g->sres[f];
        if (!sec.n) continue;
        ResidueArgs none;
        memset(&none, 0, sizeof none);
        const dim3 grid((unsigned)std::min<int64_t>(sec.total, num_sms()));
        const size_t stg = (size_t)RES_EPI_WARPS * RES_STG_BYTES;
        LaunchScope ls_("k_crt_residue", s);
        if (f == 0) {
            auto kern = k_crt_residue<RES_STAGES, false, false, RES_GROUP_STEPS_U, true, 256>;
            const size_t sm = smem_bytes(RES_STAGES, BM * 128 + 256 * 128) + stg;
            GBMM_TRY(set_smem((const void *)kern, sm));
            GBMM_TRY(launch_one(kern, grid, RES_THREADS, sm, s, zmap, zmap, zmap, none,
                                group_at<ResidueJob>(d_blob, sec), err));
        } else if (f == 1) {
            auto kern = k_crt_residue<RES_STAGES, false, false, RES_GROUP_STEPS_B, true, 256>;
            const size_t sm = smem_bytes(RES_STAGES, BM * 128 + 256 * 128) + stg;
            GBMM_TRY(set_smem((const void *)kern, sm));
            GBMM_TRY(launch_one(kern, grid, RES_THREADS, sm, s, zmap, zmap, zmap, none,
                                group_at<ResidueJob>(d_blob, sec), err));
        } else {
            auto kern = k_crt_residue<RES_STAGES_NARROW, false, false, RES_GROUP_STEPS_B, true, 128>;
            const size_t sm = smem_bytes(RES_STAGES_NARROW, BM * 128 + 128 * 128) + stg;
            GBMM_TRY(set_smem((const void *)kern, sm));
            GBMM_TRY(launch_one(kern, grid, RES_THREADS, sm, s, zmap, zmap, zmap, none,
                                group_at<ResidueJob>(d_blob, sec), err));
        }
        GBMM_CUDA_TRY(cudaGetLastError());
    }
    if (g->sprod.n) {
        ProductArgs none;
        memset(&none, 0, sizeof none);
        auto kern = k_crt_product<PROD_STAGES, false, true>;
        GBMM_TRY(set_smem((const void *)kern, g->smem_prod));
        const dim3 grid((unsigned)std::min<int64_t>(g->sprod.total, num_sms()));
        LaunchScope ls_("k_crt_product", s);
        GBMM_TRY(launch_one(kern, grid, CTA_THREADS8, g->smem_prod, s, zmap, zmap, none,
                            group_at<ProductJob>(d_blob, g->sprod), err));
        GBMM_CUDA_TRY(cudaGetLastError());
    }
    // the products with post steps first: their shifted adds then run on s2 while
    // the other reconstructions do
    for (int f = 1; f >= 0; f--) {
        const crt_group::Sect &sec = g->srec[f];
        if (sec.n) {
            ReconArgs none;
            memset(&none, 0, sizeof none);
            auto kern = k_crt_recon<REC_STAGES_PAIR, true, true>;
            GBMM_TRY(set_smem((const void *)kern, g->smem_rec));
            LaunchScope ls_("k_crt_recon", s);
            GBMM_TRY(launch_pairs(kern, CTA_THREADS8, sec.total, g->smem_rec, s, zmap, zmap, none,
                                  group_at<ReconJob>(d_blob, sec), err));
        }
        if (f == 1 && !g->post.empty()) {
            cudaStream_t sp = s;
            if (s2 && ev) {
                GBMM_CUDA_TRY(cudaEventRecord(ev, s));
                GBMM_CUDA_TRY(cudaStreamWaitEvent(s2, ev, 0));
                sp = s2;
            }
            for (auto &fn : g->post) GBMM_TRY(fn(sp));
        }
    }
    return GBMM_OK;
}

}  // namespace gbmm

using namespace gbmm;

// Internal test hook (not part of the public ABI): D = A * B^T through the
// tcgen05 pipeline.  A: bf16 [M x K] (a_mn = 0) or [K x M] (a_mn = 1), B: bf16
// [N x K]; K a multiple of 64, M and N multiples of 128 ... any (padded by TMA).
extern "C" gbmm_status gbmmx_test_gemm(const void *A, const void *B, int32_t *D, int32_t M, int32_t N, int32_t K,
                                       int32_t a_mn, void *stream) {
    cudaStream_t s = as_stream(stream);
    if (K % 64 || M % 8 || N % 8) return set_error(GBMM_ERR_INVALID, "test gemm: K % 64, M % 8, N % 8 required");
    CUtensorMap tmA, tmB;
    if (a_mn) GBMM_TRY(make_map(&tmA, A, M, K, M, 64, BK));
    else GBMM_TRY(make_map(&tmA, A, K, M, K, BK, BM));
    GBMM_TRY(make_map(&tmB, B, K, N, K, BK, BM));
    TestArgs ta;
    ta.M = M; ta.N = N; ta.nk = K / BK; ta.a_mn = a_mn; ta.D = D;
    ta.skip_step = -1;
    ta.wait_limit = tc::WAIT_LIMIT_CLOCKS;
    const size_t sm = smem_bytes(TEST_STAGES, 2 * BM * 128);
    GBMM_TRY(set_smem((const void *)k_gemm_test<TEST_STAGES>, sm));
    dim3 grid((unsigned)((N + BM - 1) / BM), (unsigned)((M + BM - 1) / BM));
    LaunchScope ls_("k_gemm_test", s);
    k_gemm_test<TEST_STAGES><<<grid, CTA_THREADS, sm, s>>>(tmA, tmB, ta, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return check_device_error(s);
}

// Internal test hook for the failure path: the same single-CTA pipeline (M = N =
// 128, one CTA) with K step `skip_step` never loaded (its stage barrier is never
// armed, so the MMA issuer's wait for it cannot complete) and every wait bounded
// by `wait_limit_clocks`.  Each role gives up when its wait runs out, records
// DEVERR_TIMEOUT, lets its in-flight copies and MMAs finish (bounded waits), and
// the CTA frees its TMEM and exits; the status comes back as GBMM_ERR_TIMEOUT.
extern "C" gbmm_status gbmmx_test_gemm_timeout(const void *A, const void *B, int32_t *D, int32_t K, int32_t skip_step,
                                               int64_t wait_limit_clocks, void *stream) {
    cudaStream_t s = as_stream(stream);
    if (K % 64 || K < 64 || skip_step < 0 || skip_step >= K / BK || wait_limit_clocks < 1000 ||
        wait_limit_clocks > tc::WAIT_LIMIT_CLOCKS)
        return set_error(GBMM_ERR_INVALID, "test gemm timeout: bad arguments");
    CUtensorMap tmA, tmB;
    GBMM_TRY(make_map(&tmA, A, K, BM, K, BK, BM));
    GBMM_TRY(make_map(&tmB, B, K, BM, K, BK, BM));
    TestArgs ta;
    ta.M = BM; ta.N = BM; ta.nk = K / BK; ta.a_mn = 0; ta.D = D;
    ta.skip_step = skip_step;
    ta.wait_limit = wait_limit_clocks;
    const size_t sm = smem_bytes(TEST_STAGES, 2 * BM * 128);
    GBMM_TRY(set_smem((const void *)k_gemm_test<TEST_STAGES>, sm));
    LaunchScope ls_("k_gemm_test", s);
    k_gemm_test<TEST_STAGES><<<dim3(1, 1), CTA_THREADS, sm, s>>>(tmA, tmB, ta, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return check_device_error(s);
}

// Internal test hook: the same product through the CTA-pair kernel (A and B
// K-major only).
extern "C" gbmm_status gbmmx_test_gemm_pair(const void *A, const void *B, int32_t *D, int32_t M, int32_t N, int32_t K,
                                            void *stream) {
    cudaStream_t s = as_stream(stream);
    if (K % 64 || M % 8 || N % 8) return set_error(GBMM_ERR_INVALID, "test gemm: K % 64, M % 8, N % 8 required");
    CUtensorMap tmA, tmB;
    GBMM_TRY(make_map(&tmA, A, K, M, K, BK, BM));
    GBMM_TRY(make_map(&tmB, B, K, N, K, BK, BM));
    TestArgs ta;
    ta.M = M; ta.N = N; ta.nk = K / BK; ta.a_mn = 0; ta.D = D;
    ta.skip_step = -1;
    ta.wait_limit = tc::WAIT_LIMIT_CLOCKS;
    const size_t sm = smem_bytes(TEST_STAGES, 2 * BM * 128);
    GBMM_TRY(set_smem((const void *)k_gemm_test_pair<TEST_STAGES>, sm));
    const unsigned tiles = (unsigned)(((M + 255) / 256) * ((N + 255) / 256));
    LaunchScope ls_("k_gemm_test_pair", s);
    k_gemm_test_pair<TEST_STAGES><<<2 * tiles, CTA_THREADS, sm, s>>>(tmA, tmB, ta, device_error_word());
    GBMM_CUDA_TRY(cudaGetLastError());
    return check_device_error(s);
}

extern "C" gbmm_status gbmmx_crt_params(int64_t bits_a, int64_t bits_b, int32_t k, int32_t *nmoduli) {
    if (!nmoduli) return set_error(GBMM_ERR_INVALID, "null pointer");
    *nmoduli = crt_moduli(bits_a, bits_b, k);
    return GBMM_OK;
}

// Internal hook: builds the host side of the table set for P moduli (no device
// work) and returns an FNV-1a checksum of its contents; *ms gets the build time.
extern "C" uint64_t gbmmx_table_build(int32_t P, double *ms) {
    if (P < 1 || P > 2 * CMOD_PAIRS) return 0;
    const auto t0 = std::chrono::steady_clock::now();
    crt_tables_host o;
    build_tables_host(P, o);
    const auto t1 = std::chrono::steady_clock::now();
    if (ms) *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ull;
    };
    mix(o.recon.data(), o.recon.size() * 2);
    mix(o.vtab.data(), o.vtab.size() * 4);
    mix(o.mods.data(), o.mods.size() * sizeof(ModConst));
    return h;
}

// Test hook: launch the four stages' kernels with programmatic stream
// serialization (1, the default) or as plain stream-ordered launches (0); returns
// the previous setting.
extern "C" int32_t gbmmx_launch_pdl(int32_t enable) {
    const int32_t old = g_pdl ? 1 : 0;
    g_pdl = enable != 0;
    return old;
}

// Test hook: the residue GEMM's form (-1 by the K loop's length, 0 single CTAs,
// 1 CTA pairs); returns the previous setting.
extern "C" int32_t gbmmx_residue_mode(int32_t mode) {
    const int32_t old = g_residue_mode;
    g_residue_mode = mode < 0 ? -1 : (mode > 2 ? 2 : mode);
    return old;
}
