/*
 * oracle.c -- CPU oracle for gbmm.  TEST INFRASTRUCTURE ONLY: the parity
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it to
 * compute expected results.  No product code path calls it.
 *
 * It restates, in plain C, the reference's CPU algorithm for exact signed
 * big-integer matrix multiplication (tomsmeding/bachelor-thesis, mat-cpu/):
 *   - naive triple loop mat_mul / mat_addmul            mat-cpu/mat.c:72-93
 *   - Strassen, 3 temporaries                            mat-cpu/mat.c:103-191
 *   - Winograd, 3 temporaries (mul and addmul forms)     mat-cpu/mat.c:193-334
 *     (operation order of mat-gpu/mat-defines.h:144-187)
 *   - squarify: power-of-two core plus remainders        mat-cpu/matj.c:680-780
 *   - "-m 31": naive 8-product split down to the job size with Winograd
 *     leaves (nlevels = floor(log2(N / basesz)))          mat-cpu/matj.c:571-660
 *   - hex text I/O in mat_read / mat_write format       mat-cpu/mat.c:336-353
 * The arithmetic underneath is the reference's third-party dependency GMP
 * (6.1.2, pinned by mat-cpu/gmp.h:2323-2325; not vendored).  Two backends:
 *   - "own": a restatement of GMP's published mpz semantics (sign-magnitude,
 *     normalized sizes) with schoolbook and Karatsuba products on 64-bit limbs;
 *   - "gmp": the system libgmp.so.10 loaded with dlopen, used only as a second
 *     reference for the tests and as the CPU baseline when present.
 * Batched mpn restatements on 32-bit limbs (add_n, sub_n, mul_1, addmul_1,
 * submul_1, mul_basecase, toom22) mirror the device layer's semantics
 * (GMP's mpn contract) for operation-level tests.
 *
 * Parity pinning: the reference ships no golden vectors; the fixtures under
 * tests/golden/ were produced by the reference's own mat-cpu built from its
 * sources (oracle/Makefile, target "ref") and cross-checked against Python integers,
 * and tests check this file against them.
 */
#define _GNU_SOURCE
#include <ctype.h>
#include <dlfcn.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------------ */
/* Number type.  Same memory shape as GMP's __mpz_struct so the "gmp" backend
 * can run the same matrix code: {int alloc; int size; limb *d}.            */
typedef struct {
    int alloc;
    int size;
    uint64_t *d;
} onum;

typedef struct {
    void (*init)(onum *);
    void (*clear)(onum *);
    void (*add)(onum *, const onum *, const onum *);
    void (*sub)(onum *, const onum *, const onum *);
    void (*mul)(onum *, const onum *, const onum *);
    void (*addmul)(onum *, const onum *, const onum *);
    void (*set)(onum *, const onum *);
} num_ops;

static int iabs_(int x) { return x < 0 ? -x : x; }

static void own_init(onum *z) { z->alloc = 0; z->size = 0; z->d = NULL; }
static void own_clear(onum *z) { free(z->d); z->d = NULL; z->alloc = 0; z->size = 0; }
static void own_reserve(onum *z, int n) {
    if (n > z->alloc) {
        int na = n < 4 ? 4 : n;
        z->d = (uint64_t *)realloc(z->d, (size_t)na * sizeof(uint64_t));
        z->alloc = na;
    }
}
static int mag_norm(const uint64_t *p, int n) { while (n > 0 && p[n - 1] == 0) n--; return n; }
static int mag_cmp(const uint64_t *a, int an, const uint64_t *b, int bn) {
    if (an != bn) return an < bn ? -1 : 1;
    for (int i = an - 1; i >= 0; i--)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}
/* r = a + b (an >= bn), r has room for an+1; returns length */
static int mag_add(uint64_t *r, const uint64_t *a, int an, const uint64_t *b, int bn) {
    uint64_t c = 0;
    int i;
    for (i = 0; i < bn; i++) {
        u128 s = (u128)a[i] + b[i] + c;
        r[i] = (uint64_t)s; c = (uint64_t)(s >> 64);
    }
    for (; i < an; i++) {
        u128 s = (u128)a[i] + c;
        r[i] = (uint64_t)s; c = (uint64_t)(s >> 64);
    }
    r[an] = c;
    return an + (c != 0);
}
/* r = a - b with a >= b; returns normalized length */
static int mag_sub(uint64_t *r, const uint64_t *a, int an, const uint64_t *b, int bn) {
    uint64_t br = 0;
    int i;
    for (i = 0; i < bn; i++) {
        uint64_t x = a[i], y = b[i];
        uint64_t d = x - y - br;
        br = (x < y) || (x - y < br);
        r[i] = d;
    }
    for (; i < an; i++) {
        uint64_t x = a[i];
        r[i] = x - br;
        br = x < br;
    }
    return mag_norm(r, an);
}
/* schoolbook r[0..an+bn) = a * b */
static void mag_mul_school(uint64_t *r, const uint64_t *a, int an, const uint64_t *b, int bn) {
    memset(r, 0, (size_t)(an + bn) * sizeof(uint64_t));
    for (int j = 0; j < bn; j++) {
        uint64_t c = 0, bj = b[j];
        for (int i = 0; i < an; i++) {
            u128 t = (u128)a[i] * bj + r[i + j] + c;
            r[i + j] = (uint64_t)t; c = (uint64_t)(t >> 64);
        }
        r[j + an] = c;
    }
}
/* add b (bn) into r (rn >= bn), propagating the carry within rn */
static void mag_addto(uint64_t *r, int rn, const uint64_t *b, int bn) {
    uint64_t c = 0;
    int i;
    for (i = 0; i < bn; i++) {
        u128 s = (u128)r[i] + b[i] + c;
        r[i] = (uint64_t)s; c = (uint64_t)(s >> 64);
    }
    for (; c && i < rn; i++) { r[i] += c; c = r[i] == 0; }
}
static void mag_subfrom(uint64_t *r, int rn, const uint64_t *b, int bn) {
    uint64_t br = 0;
    int i;
    for (i = 0; i < bn; i++) {
        uint64_t x = r[i], y = b[i];
        r[i] = x - y - br;
        br = (x < y) || (x - y < br);
    }
    for (; br && i < rn; i++) { br = r[i] == 0; r[i] -= 1; }
}
#define KARA_THRESHOLD 24
/* Karatsuba (Knuth TAOCP 4.3.3) on balanced operands, n = an = bn. */
static void mag_mul_kara(uint64_t *r, const uint64_t *a, const uint64_t *b, int n) {
    if (n < KARA_THRESHOLD) { mag_mul_school(r, a, n, b, n); return; }
    int h = n / 2, hi = n - h; /* low h limbs, high hi limbs (hi >= h) */
    uint64_t *sa = (uint64_t *)calloc((size_t)(hi + 1), 8), *sb = (uint64_t *)calloc((size_t)(hi + 1), 8);
    uint64_t *m = (uint64_t *)calloc((size_t)(2 * hi + 2), 8);
    int la = mag_add(sa, a + h, hi, a, h), lb = mag_add(sb, b + h, hi, b, h);
    (void)la; (void)lb;
    /* sa, sb have hi+1 limbs */
    mag_mul_kara(m, sa, sb, hi + 1);
    memset(r, 0, (size_t)(2 * n) * sizeof(uint64_t));
    mag_mul_kara(r, a, b, h);                 /* r[0..2h) = a0 b0 */
    mag_mul_kara(r + 2 * h, a + h, b + h, hi); /* r[2h..2n) = a1 b1 */
    /* m -= a0b0 + a1b1 */
    mag_subfrom(m, 2 * hi + 2, r, 2 * h);
    mag_subfrom(m, 2 * hi + 2, r + 2 * h, 2 * hi);
    mag_addto(r + h, 2 * n - h, m, mag_norm(m, 2 * hi + 2));
    free(sa); free(sb); free(m);
}
static void mag_mul(uint64_t *r, const uint64_t *a, int an, const uint64_t *b, int bn) {
    if (an == bn && an >= KARA_THRESHOLD) { mag_mul_kara(r, a, b, an); return; }
    if (an >= KARA_THRESHOLD && bn >= KARA_THRESHOLD) {
        /* unbalanced: split the longer operand into bn-sized pieces */
        const uint64_t *L = an >= bn ? a : b, *S = an >= bn ? b : a;
        int ln = an >= bn ? an : bn, sn = an >= bn ? bn : an;
        memset(r, 0, (size_t)(an + bn) * 8);
        uint64_t *t = (uint64_t *)malloc((size_t)(2 * sn) * 8);
        int off = 0;
        for (; off + sn <= ln; off += sn) {
            mag_mul_kara(t, L + off, S, sn);
            mag_addto(r + off, an + bn - off, t, 2 * sn);
        }
        if (off < ln) {
            int rem = ln - off;
            mag_mul_school(t, S, sn, L + off, rem);
            mag_addto(r + off, an + bn - off, t, sn + rem);
        }
        free(t);
        return;
    }
    if (an >= bn) mag_mul_school(r, a, an, b, bn); else mag_mul_school(r, b, bn, a, an);
}

static void own_set(onum *w, const onum *u) {
    if (w == u) return;
    int n = iabs_(u->size);
    own_reserve(w, n);
    if (n) memcpy(w->d, u->d, (size_t)n * 8);
    w->size = u->size;
}
/* w = u + sgn*v (sgn = +1 / -1); handles aliasing through a temporary */
static void own_addsub(onum *w, const onum *u, const onum *v, int sgn) {
    int un = iabs_(u->size), vn = iabs_(v->size);
    int us = u->size < 0, vs = (v->size < 0) ^ (sgn < 0);
    int rn = (un > vn ? un : vn) + 1;
    uint64_t *r = (uint64_t *)malloc((size_t)rn * 8);
    int len, neg;
    if (us == vs) {
        len = un >= vn ? mag_add(r, u->d, un, v->d, vn) : mag_add(r, v->d, vn, u->d, un);
        neg = us;
    } else {
        int c = mag_cmp(u->d, un, v->d, vn);
        if (c >= 0) { len = mag_sub(r, u->d, un, v->d, vn); neg = us; }
        else { len = mag_sub(r, v->d, vn, u->d, un); neg = vs; }
    }
    free(w->d);
    w->d = r; w->alloc = rn;
    w->size = len == 0 ? 0 : (neg ? -len : len);
}
static void own_add(onum *w, const onum *u, const onum *v) { own_addsub(w, u, v, +1); }
static void own_sub(onum *w, const onum *u, const onum *v) { own_addsub(w, u, v, -1); }
static void own_mul(onum *w, const onum *u, const onum *v) {
    int un = iabs_(u->size), vn = iabs_(v->size);
    if (un == 0 || vn == 0) { w->size = 0; return; }
    uint64_t *r = (uint64_t *)malloc((size_t)(un + vn) * 8);
    mag_mul(r, u->d, un, v->d, vn);
    int len = mag_norm(r, un + vn);
    int neg = (u->size < 0) ^ (v->size < 0);
    free(w->d);
    w->d = r; w->alloc = un + vn;
    w->size = neg ? -len : len;
}
static void own_addmul(onum *w, const onum *u, const onum *v) {
    onum t; own_init(&t);
    own_mul(&t, u, v);
    own_add(w, w, &t);
    own_clear(&t);
}

static num_ops g_own_ops = {own_init, own_clear, own_add, own_sub, own_mul, own_addmul, own_set};

/* ---- optional GMP backend (system libgmp.so.10 via dlopen) ---------------- */
static num_ops g_gmp_ops;
static int g_gmp_loaded = -1;
static void (*gz_addmul)(onum *, const onum *, const onum *);
static int load_gmp(void) {
    if (g_gmp_loaded >= 0) return g_gmp_loaded;
    g_gmp_loaded = 0;
    void *h = dlopen("libgmp.so.10", RTLD_NOW | RTLD_LOCAL);
    if (!h) return 0;
#define SYM(dst, name) do { *(void **)(&dst) = dlsym(h, name); if (!dst) return 0; } while (0)
    SYM(g_gmp_ops.init, "__gmpz_init");
    SYM(g_gmp_ops.clear, "__gmpz_clear");
    SYM(g_gmp_ops.add, "__gmpz_add");
    SYM(g_gmp_ops.sub, "__gmpz_sub");
    SYM(g_gmp_ops.mul, "__gmpz_mul");
    SYM(gz_addmul, "__gmpz_addmul");
    SYM(g_gmp_ops.set, "__gmpz_set");
#undef SYM
    g_gmp_ops.addmul = gz_addmul;
    g_gmp_loaded = 1;
    return 1;
}

static const num_ops *g_ops = &g_own_ops;

/* Selects the arithmetic backend: 0 = own restatement, 1 = libgmp.so.10.
 * Returns 0 on success, -1 if libgmp.so.10 cannot be loaded. */
int oracle_set_backend(int gmp) {
    if (gmp) {
        if (!load_gmp()) return -1;
        g_ops = &g_gmp_ops;
    } else {
        g_ops = &g_own_ops;
    }
    return 0;
}
int oracle_gmp_available(void) { return load_gmp(); }

/* ------------------------------------------------------------------------ */
/* Matrices: row-major arrays of onum with row strides (mat-cpu/mat.h:7-10). */
typedef onum *mat_t;

static mat_t mat_init(unsigned W, unsigned H) {
    mat_t A = (mat_t)malloc((size_t)W * H * sizeof(onum) + 1);
    for (size_t i = 0; i < (size_t)W * H; i++) g_ops->init(&A[i]);
    return A;
}
static void mat_free(unsigned W, unsigned H, mat_t A) {
    for (size_t i = 0; i < (size_t)W * H; i++) g_ops->clear(&A[i]);
    free(A);
}
static void mat_add(unsigned W, unsigned H, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs) {
    for (unsigned y = 0; y < H; y++)
        for (unsigned x = 0; x < W; x++) g_ops->add(&C[Crs * y + x], &A[Ars * y + x], &B[Brs * y + x]);
}
static void mat_sub(unsigned W, unsigned H, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs) {
    for (unsigned y = 0; y < H; y++)
        for (unsigned x = 0; x < W; x++) g_ops->sub(&C[Crs * y + x], &A[Ars * y + x], &B[Brs * y + x]);
}
/* mat-cpu/mat.c:72-82 */
static void mat_mul(unsigned K, unsigned M, unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs) {
    for (unsigned y = 0; y < K; y++)
        for (unsigned x = 0; x < N; x++) {
            g_ops->mul(&C[Crs * y + x], &A[Ars * y], &B[x]);
            for (unsigned k = 1; k < M; k++) g_ops->addmul(&C[Crs * y + x], &A[Ars * y + k], &B[Brs * k + x]);
        }
}
/* mat-cpu/mat.c:84-93 */
static void mat_addmul(unsigned K, unsigned M, unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs) {
    for (unsigned y = 0; y < K; y++)
        for (unsigned x = 0; x < N; x++)
            for (unsigned k = 0; k < M; k++) g_ops->addmul(&C[Crs * y + x], &A[Ars * y + k], &B[Brs * k + x]);
}

#define SUBM(M_, rs_, ix, iy) ((M_) + (iy) * (N / 2 * (rs_)) + (ix) * (N / 2))

static void mat_mul_winograd(unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs, unsigned nlevels);
static void mat_addmul_winograd(unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs, unsigned nlevels);

/* Strassen, 3 temporaries: mat-cpu/mat.c:103-191 */
static void mat_mul_strassen(unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs, unsigned nlevels) {
    if (nlevels == 0 || N % 2) { mat_mul(N, N, N, C, Crs, A, Ars, B, Brs); return; }
    mat_t T = mat_init(N, N);
    long Trs = N;
    const onum *a11 = SUBM(A, Ars, 0, 0), *a12 = SUBM(A, Ars, 1, 0), *a21 = SUBM(A, Ars, 0, 1), *a22 = SUBM(A, Ars, 1, 1);
    const onum *b11 = SUBM(B, Brs, 0, 0), *b12 = SUBM(B, Brs, 1, 0), *b21 = SUBM(B, Brs, 0, 1), *b22 = SUBM(B, Brs, 1, 1);
    onum *c11 = SUBM(C, Crs, 0, 0), *c12 = SUBM(C, Crs, 1, 0), *c21 = SUBM(C, Crs, 0, 1), *c22 = SUBM(C, Crs, 1, 1);
    onum *p1 = SUBM(T, Trs, 0, 0), *p2 = SUBM(T, Trs, 1, 0), *p3 = SUBM(T, Trs, 0, 1);
    unsigned h = N / 2;
#define ADD(c, cr, a, ar, b, br) mat_add(h, h, c, cr, a, ar, b, br)
#define SUB(c, cr, a, ar, b, br) mat_sub(h, h, c, cr, a, ar, b, br)
#define MUL(c, cr, a, ar, b, br) mat_mul_strassen(h, c, cr, a, ar, b, br, nlevels - 1)
    ADD(p1, Trs, a11, Ars, a22, Ars); ADD(p2, Trs, b11, Brs, b22, Brs); MUL(c11, Crs, p1, Trs, p2, Trs);
    SUB(p1, Trs, b12, Brs, b22, Brs); MUL(c12, Crs, a11, Ars, p1, Trs);
    ADD(c22, Crs, c11, Crs, c12, Crs);
    ADD(p1, Trs, a21, Ars, a22, Ars); MUL(c21, Crs, p1, Trs, b11, Brs);
    SUB(c22, Crs, c22, Crs, c21, Crs);
    SUB(p2, Trs, a12, Ars, a22, Ars); ADD(p3, Trs, b21, Brs, b22, Brs); MUL(p1, Trs, p2, Trs, p3, Trs);
    ADD(c11, Crs, c11, Crs, p1, Trs);
    SUB(p2, Trs, a21, Ars, a11, Ars); ADD(p3, Trs, b11, Brs, b12, Brs); MUL(p1, Trs, p2, Trs, p3, Trs);
    ADD(c22, Crs, c22, Crs, p1, Trs);
    SUB(p2, Trs, b21, Brs, b11, Brs); MUL(p1, Trs, a22, Ars, p2, Trs);
    ADD(c11, Crs, c11, Crs, p1, Trs);
    ADD(c21, Crs, c21, Crs, p1, Trs);
    ADD(p2, Trs, a11, Ars, a12, Ars); MUL(p1, Trs, p2, Trs, b22, Brs);
    SUB(c11, Crs, c11, Crs, p1, Trs);
    ADD(c12, Crs, c12, Crs, p1, Trs);
#undef MUL
    mat_free(N, N, T);
}

/* Winograd, 3 temporaries: mat-cpu/mat.c:193-262, order of WINOGRAD_SEQUENCE
 * (mat-gpu/mat-defines.h:144-164). */
static void mat_mul_winograd(unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs, unsigned nlevels) {
    if (nlevels == 0 || N % 2) { mat_mul(N, N, N, C, Crs, A, Ars, B, Brs); return; }
    mat_t T = mat_init(N, N);
    long Trs = N;
    const onum *a11 = SUBM(A, Ars, 0, 0), *a12 = SUBM(A, Ars, 1, 0), *a21 = SUBM(A, Ars, 0, 1), *a22 = SUBM(A, Ars, 1, 1);
    const onum *b11 = SUBM(B, Brs, 0, 0), *b12 = SUBM(B, Brs, 1, 0), *b21 = SUBM(B, Brs, 0, 1), *b22 = SUBM(B, Brs, 1, 1);
    onum *c11 = SUBM(C, Crs, 0, 0), *c12 = SUBM(C, Crs, 1, 0), *c21 = SUBM(C, Crs, 0, 1), *c22 = SUBM(C, Crs, 1, 1);
    onum *p1 = SUBM(T, Trs, 0, 0), *p2 = SUBM(T, Trs, 1, 0), *p3 = SUBM(T, Trs, 0, 1);
    unsigned h = N / 2;
#define MUL(c, cr, a, ar, b, br) mat_mul_winograd(h, c, cr, a, ar, b, br, nlevels - 1)
#define AML(c, cr, a, ar, b, br) mat_addmul_winograd(h, c, cr, a, ar, b, br, nlevels - 1)
    ADD(p1, Trs, a21, Ars, a22, Ars);
    SUB(p2, Trs, b12, Brs, b11, Brs);
    MUL(c22, Crs, p1, Trs, p2, Trs);
    SUB(p1, Trs, p1, Trs, a11, Ars);
    SUB(p2, Trs, b22, Brs, p2, Trs);
    MUL(p3, Trs, a11, Ars, b11, Brs);
    MUL(c11, Crs, a12, Ars, b21, Brs);
    ADD(c11, Crs, c11, Crs, p3, Trs);
    AML(p3, Trs, p1, Trs, p2, Trs);
    SUB(p1, Trs, a12, Ars, p1, Trs);
    SUB(p2, Trs, b21, Brs, p2, Trs);
    MUL(c12, Crs, p1, Trs, b22, Brs);
    ADD(c12, Crs, c12, Crs, c22, Crs);
    ADD(c12, Crs, c12, Crs, p3, Trs);
    MUL(c21, Crs, a22, Ars, p2, Trs);
    SUB(p1, Trs, a11, Ars, a21, Ars);
    SUB(p2, Trs, b22, Brs, b12, Brs);
    AML(p3, Trs, p1, Trs, p2, Trs);
    ADD(c21, Crs, c21, Crs, p3, Trs);
    ADD(c22, Crs, c22, Crs, p3, Trs);
#undef MUL
#undef AML
    mat_free(N, N, T);
}

/* mat-cpu/mat.c:264-334, order of WINOGRAD_ADDMUL_SEQUENCE (mat-defines.h:166-187) */
static void mat_addmul_winograd(unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs, unsigned nlevels) {
    if (nlevels == 0 || N % 2) { mat_addmul(N, N, N, C, Crs, A, Ars, B, Brs); return; }
    mat_t T = mat_init(N, N);
    long Trs = N;
    const onum *a11 = SUBM(A, Ars, 0, 0), *a12 = SUBM(A, Ars, 1, 0), *a21 = SUBM(A, Ars, 0, 1), *a22 = SUBM(A, Ars, 1, 1);
    const onum *b11 = SUBM(B, Brs, 0, 0), *b12 = SUBM(B, Brs, 1, 0), *b21 = SUBM(B, Brs, 0, 1), *b22 = SUBM(B, Brs, 1, 1);
    onum *c11 = SUBM(C, Crs, 0, 0), *c12 = SUBM(C, Crs, 1, 0), *c21 = SUBM(C, Crs, 0, 1), *c22 = SUBM(C, Crs, 1, 1);
    onum *p1 = SUBM(T, Trs, 0, 0), *p2 = SUBM(T, Trs, 1, 0), *p3 = SUBM(T, Trs, 0, 1);
    unsigned h = N / 2;
#define MUL(c, cr, a, ar, b, br) mat_mul_winograd(h, c, cr, a, ar, b, br, nlevels - 1)
#define AML(c, cr, a, ar, b, br) mat_addmul_winograd(h, c, cr, a, ar, b, br, nlevels - 1)
    ADD(p1, Trs, a21, Ars, a22, Ars);
    SUB(p2, Trs, b12, Brs, b11, Brs);
    MUL(p3, Trs, p1, Trs, p2, Trs);
    ADD(c12, Crs, c12, Crs, p3, Trs);
    ADD(c22, Crs, c22, Crs, p3, Trs);
    SUB(p1, Trs, p1, Trs, a11, Ars);
    SUB(p2, Trs, b22, Brs, p2, Trs);
    MUL(p3, Trs, a11, Ars, b11, Brs);
    ADD(c11, Crs, c11, Crs, p3, Trs);
    AML(p3, Trs, p1, Trs, p2, Trs);
    AML(c11, Crs, a12, Ars, b21, Brs);
    SUB(p1, Trs, a12, Ars, p1, Trs);
    SUB(p2, Trs, b21, Brs, p2, Trs);
    AML(c12, Crs, p1, Trs, b22, Brs);
    ADD(c12, Crs, c12, Crs, p3, Trs);
    AML(c21, Crs, a22, Ars, p2, Trs);
    SUB(p1, Trs, a11, Ars, a21, Ars);
    SUB(p2, Trs, b22, Brs, b12, Brs);
    AML(p3, Trs, p1, Trs, p2, Trs);
    ADD(c21, Crs, c21, Crs, p3, Trs);
    ADD(c22, Crs, c22, Crs, p3, Trs);
#undef MUL
#undef AML
#undef ADD
#undef SUB
    mat_free(N, N, T);
}

/* ---- threaded leaf scheduler (stands in for mat-cpu/job.c's pthread DAG) --- */
/* A square product is cut into output blocks of size <= jobsz; every block
 * C_ij = sum_k A_ik B_kj is one task; each block product runs the Winograd
 * recursion with nlevels = floor(log2(bs / basesz)) (mat-cpu/matj.c:354-357,
 * 583-586).  Tasks are claimed from an atomic counter by nthreads workers. */
typedef struct {
    unsigned nb, bs, M;
    mat_t C; long Crs; const onum *A; long Ars; const onum *B; long Brs;
    unsigned nlevels;
    int method; /* 3 strassen, 35/31 winograd, 1 naive */
    int next;
    pthread_mutex_t mu;
} block_job;

static unsigned ilog2u(unsigned n) { unsigned r = 0; while (n >>= 1) r++; return r; }

static void *block_worker(void *arg) {
    block_job *J = (block_job *)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int t = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (t >= (int)(J->nb * J->nb)) break;
        unsigned bi = (unsigned)t / J->nb, bj = (unsigned)t % J->nb, bs = J->bs;
        onum *Cb = J->C + (long)bi * bs * J->Crs + (long)bj * bs;
        mat_t T = mat_init(bs, bs);
        unsigned nk = J->M / bs;
        for (unsigned k = 0; k < nk; k++) {
            const onum *Ab = J->A + (long)bi * bs * J->Ars + (long)k * bs;
            const onum *Bb = J->B + (long)k * bs * J->Brs + (long)bj * bs;
            onum *dst = k == 0 ? Cb : T;
            long drs = k == 0 ? J->Crs : (long)bs;
            if (J->method == 3) mat_mul_strassen(bs, dst, drs, Ab, J->Ars, Bb, J->Brs, J->nlevels);
            else if (J->method == 1) mat_mul(bs, bs, bs, dst, drs, Ab, J->Ars, Bb, J->Brs);
            else mat_mul_winograd(bs, dst, drs, Ab, J->Ars, Bb, J->Brs, J->nlevels);
            if (k) mat_add(bs, bs, Cb, J->Crs, Cb, J->Crs, T, bs);
        }
        mat_free(bs, bs, T);
    }
    return NULL;
}

static void square_mul(unsigned N, mat_t C, long Crs, const onum *A, long Ars, const onum *B, long Brs,
                       int method, unsigned basesz, unsigned jobsz, int nthreads) {
    if (method == 35 && nthreads <= 1) {
        unsigned nl = N <= basesz ? 0 : ilog2u(N / basesz);
        mat_mul_winograd(N, C, Crs, A, Ars, B, Brs, nl);
        return;
    }
    if (method == 3 && nthreads <= 1) {
        unsigned nl = N <= basesz ? 0 : ilog2u(N / basesz);
        mat_mul_strassen(N, C, Crs, A, Ars, B, Brs, nl);
        return;
    }
    unsigned bs = N;
    while (bs > jobsz && bs % 2 == 0) bs /= 2;
    block_job J;
    J.nb = N / bs; J.bs = bs; J.M = N;
    J.C = C; J.Crs = Crs; J.A = A; J.Ars = Ars; J.B = B; J.Brs = Brs;
    J.nlevels = bs <= basesz ? 0 : ilog2u(bs / basesz);
    J.method = method; J.next = 0;
    pthread_mutex_init(&J.mu, NULL);
    int nt = nthreads < 1 ? 1 : nthreads;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
    for (int i = 0; i < nt; i++) pthread_create(&th[i], NULL, block_worker, &J);
    for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&J.mu);
}

/* naive product threaded over output rows (method 1) */
typedef struct {
    unsigned K, M, N; mat_t C; long Crs; const onum *A; long Ars; const onum *B; long Brs;
    int next; pthread_mutex_t mu; int accumulate;
} row_job;
static void *row_worker(void *arg) {
    row_job *J = (row_job *)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int y = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (y >= (int)J->K) break;
        if (J->accumulate) mat_addmul(1, J->M, J->N, J->C + (long)y * J->Crs, J->Crs, J->A + (long)y * J->Ars, J->Ars, J->B, J->Brs);
        else mat_mul(1, J->M, J->N, J->C + (long)y * J->Crs, J->Crs, J->A + (long)y * J->Ars, J->Ars, J->B, J->Brs);
    }
    return NULL;
}
static void naive_threaded(unsigned K, unsigned M, unsigned N, mat_t C, long Crs, const onum *A, long Ars,
                           const onum *B, long Brs, int nthreads, int accumulate) {
    row_job J = {K, M, N, C, Crs, A, Ars, B, Brs, 0, PTHREAD_MUTEX_INITIALIZER, accumulate};
    int nt = nthreads < 1 ? 1 : nthreads;
    if (nt == 1) { row_worker(&J); return; }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
    for (int i = 0; i < nt; i++) pthread_create(&th[i], NULL, row_worker, &J);
    for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
    free(th);
}

static unsigned remove_factors(unsigned n, unsigned b) { while (n && n % b == 0) n /= b; return n; }

/* squarify: mat-cpu/matj.c:680-780 (sequential restatement of its job DAG) */
static void mul_squarify(unsigned K, unsigned M, unsigned N, mat_t C, long Crs, const onum *A, long Ars,
                         const onum *B, long Brs, int method, unsigned basesz, unsigned jobsz, int nthreads) {
    if (K == 0 || M == 0 || N == 0) return;
    if (method == 1 || K <= basesz || M <= basesz || N <= basesz) {
        naive_threaded(K, M, N, C, Crs, A, Ars, B, Brs, method == 1 ? nthreads : nthreads, 0);
        return;
    }
    if (K == M && M == N && remove_factors(K, 2) <= basesz) {
        square_mul(K, C, Crs, A, Ars, B, Brs, method, basesz, jobsz, nthreads);
        return;
    }
    unsigned mindim = K < M ? K : M; if (N < mindim) mindim = N;
    unsigned ptwo = 1u << ilog2u(mindim);
    mat_t T = mat_init(N, K);
    long Trs = N;
#define BLK(X, rs, ix, iy) ((X) + (long)(iy) * ptwo * (rs) + (long)(ix) * ptwo)
    const onum *a11 = BLK(A, Ars, 0, 0), *a12 = BLK(A, Ars, 1, 0), *a21 = BLK(A, Ars, 0, 1), *a22 = BLK(A, Ars, 1, 1);
    const onum *b11 = BLK(B, Brs, 0, 0), *b12 = BLK(B, Brs, 1, 0), *b21 = BLK(B, Brs, 0, 1), *b22 = BLK(B, Brs, 1, 1);
    onum *c11 = BLK(C, Crs, 0, 0), *c12 = BLK(C, Crs, 1, 0), *c21 = BLK(C, Crs, 0, 1), *c22 = BLK(C, Crs, 1, 1);
    onum *p1 = BLK(T, Trs, 0, 0), *p2 = BLK(T, Trs, 1, 0), *p3 = BLK(T, Trs, 0, 1), *p4 = BLK(T, Trs, 1, 1);
#undef BLK
#define SQ(k, m, n, c, cr, a, ar, b, br) mul_squarify(k, m, n, c, cr, a, ar, b, br, method, basesz, jobsz, nthreads)
    SQ(ptwo, ptwo, ptwo, c11, Crs, a11, Ars, b11, Brs);
    SQ(ptwo, M - ptwo, ptwo, p1, Trs, a12, Ars, b21, Brs);
    if (M > ptwo) mat_add(ptwo, ptwo, c11, Crs, c11, Crs, p1, Trs);
    SQ(ptwo, ptwo, N - ptwo, c12, Crs, a11, Ars, b12, Brs);
    SQ(ptwo, M - ptwo, N - ptwo, p2, Trs, a12, Ars, b22, Brs);
    if (M > ptwo) mat_add(N - ptwo, ptwo, c12, Crs, c12, Crs, p2, Trs);
    SQ(K - ptwo, ptwo, ptwo, c21, Crs, a21, Ars, b11, Brs);
    SQ(K - ptwo, M - ptwo, ptwo, p3, Trs, a22, Ars, b21, Brs);
    if (M > ptwo) mat_add(ptwo, K - ptwo, c21, Crs, c21, Crs, p3, Trs);
    SQ(K - ptwo, ptwo, N - ptwo, c22, Crs, a21, Ars, b12, Brs);
    SQ(K - ptwo, M - ptwo, N - ptwo, p4, Trs, a22, Ars, b22, Brs);
    if (M > ptwo) mat_add(N - ptwo, K - ptwo, c22, Crs, c22, Crs, p4, Trs);
#undef SQ
    mat_free(N, K, T);
}

/* ---- hex text I/O (mat-cpu/mat.c:336-353, GMP base-16 conventions) -------- */
static const char *skip_ws(const char *p, const char *e) { while (p < e && isspace((unsigned char)*p)) p++; return p; }
static int hexval(int c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'f') return c - 'a' + 10;
    if (c >= 'A' && c <= 'F') return c - 'A' + 10;
    return -1;
}
/* parses one signed hex integer into an own-format onum; returns new position or NULL */
static const char *parse_num(const char *p, const char *e, onum *z) {
    p = skip_ws(p, e);
    int neg = 0;
    if (p < e && *p == '-') { neg = 1; p++; }
    const char *s = p;
    while (p < e && hexval((unsigned char)*p) >= 0) p++;
    size_t nd = (size_t)(p - s);
    if (nd == 0) return NULL;
    int nl = (int)((nd + 15) / 16);
    uint64_t *d = (uint64_t *)calloc((size_t)nl, 8);
    for (size_t i = 0; i < nd; i++) {
        size_t pos = nd - 1 - i; /* digit index from least significant */
        d[pos / 16] |= (uint64_t)hexval((unsigned char)s[i]) << (4 * (pos % 16));
    }
    int len = mag_norm(d, nl);
    free(z->d);
    z->d = d; z->alloc = nl; z->size = len == 0 ? 0 : (neg ? -len : len);
    return p;
}
static void put_num(char **buf, size_t *len, size_t *cap, const onum *z) {
    int n = iabs_(z->size);
    size_t need = (size_t)n * 16 + 2;
    if (*len + need + 2 > *cap) {
        *cap = (*len + need + 2) * 2;
        *buf = (char *)realloc(*buf, *cap);
    }
    char *o = *buf + *len;
    if (n == 0) { *o++ = '0'; *len = (size_t)(o - *buf); return; }
    if (z->size < 0) *o++ = '-';
    int started = 0;
    for (int i = n - 1; i >= 0; i--)
        for (int k = 15; k >= 0; k--) {
            int dgt = (int)((z->d[i] >> (4 * k)) & 15);
            if (dgt || started) { *o++ = "0123456789abcdef"[dgt]; started = 1; }
        }
    *len = (size_t)(o - *buf);
}

/* own <-> active backend conversion: parse always produces own layout, which
 * is also valid input to GMP (same struct shape, malloc'd limbs, alloc>=size) */

/* Multiplies the matrices in `in` (mat-cpu -i format: "K M N", A, B) and
 * returns the product in mat_write format (malloc'd, caller frees with
 * oracle_free).  method: 1 naive, 3 Strassen, 35 Winograd, 31 naive split with
 * Winograd leaves.  Returns NULL on a parse error. */
char *oracle_matmul_text(const char *in, size_t inlen, int method, int basesz, int jobsz, int nthreads,
                         double *seconds) {
    const char *p = in, *e = in + inlen;
    unsigned K, M, N;
    {
        char hdr[128];
        size_t hl = 0;
        const char *q = skip_ws(p, e);
        while (q < e && *q != '\n' && hl < sizeof hdr - 1) hdr[hl++] = *q++;
        hdr[hl] = 0;
        if (sscanf(hdr, "%u %u %u", &K, &M, &N) != 3) return NULL;
        p = q;
    }
    int use_gmp = g_ops == &g_gmp_ops;
    g_ops = &g_own_ops; /* parse with own allocator layout */
    mat_t A = mat_init(M, K), B = mat_init(N, M), C = NULL;
    for (size_t i = 0; i < (size_t)K * M; i++) if (!(p = parse_num(p, e, &A[i]))) return NULL;
    for (size_t i = 0; i < (size_t)M * N; i++) if (!(p = parse_num(p, e, &B[i]))) return NULL;
    if (use_gmp) {
        /* move into GMP-managed numbers */
        g_ops = &g_gmp_ops;
        mat_t A2 = mat_init(M, K), B2 = mat_init(N, M);
        for (size_t i = 0; i < (size_t)K * M; i++) g_gmp_ops.set(&A2[i], &A[i]);
        for (size_t i = 0; i < (size_t)M * N; i++) g_gmp_ops.set(&B2[i], &B[i]);
        g_ops = &g_own_ops;
        mat_free(M, K, A); mat_free(N, M, B);
        A = A2; B = B2;
        g_ops = &g_gmp_ops;
    }
    C = mat_init(N, K);
    if (basesz <= 0) basesz = 32;
    if (jobsz <= 0) jobsz = 128;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    mul_squarify(K, M, N, C, N, A, M, B, N, method, (unsigned)basesz, (unsigned)jobsz, nthreads);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (seconds) *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    size_t cap = 1024, len = 0;
    char *buf = (char *)malloc(cap);
    for (unsigned y = 0; y < K; y++) {
        for (unsigned x = 0; x < N; x++) {
            if (x) { if (len + 2 > cap) { cap *= 2; buf = (char *)realloc(buf, cap); } buf[len++] = ' '; }
            put_num(&buf, &len, &cap, &C[(size_t)y * N + x]);
        }
        if (len + 2 > cap) { cap *= 2; buf = (char *)realloc(buf, cap); }
        buf[len++] = '\n';
    }
    if (len + 2 > cap) { cap *= 2; buf = (char *)realloc(buf, cap); }
    buf[len++] = '\n';
    buf[len] = 0;
    mat_free(M, K, A); mat_free(N, M, B); mat_free(N, K, C);
    g_ops = use_gmp ? &g_gmp_ops : &g_own_ops;
    return buf;
}

void oracle_free(void *p) { free(p); }

/* ---- limb-plane interface (gbmm's layout: 32-bit limbs, SoA planes) -------- */
static void planes_to_own(onum *z, const uint32_t *limbs, const int32_t *sizes, int64_t ld, int64_t e) {
    int s = sizes[e], n = iabs_(s);
    int n64 = (n + 1) / 2;
    uint64_t *d = (uint64_t *)calloc((size_t)(n64 ? n64 : 1), 8);
    for (int i = 0; i < n; i++) d[i / 2] |= (uint64_t)limbs[(int64_t)i * ld + e] << (32 * (i % 2));
    free(z->d);
    z->d = d; z->alloc = n64 ? n64 : 1;
    int len = mag_norm(d, n64);
    z->size = s < 0 ? -len : len;
}
/* returns 0 ok, -1 if the value needs more than nlimbs planes */
static int own_to_planes(const onum *z, uint32_t *limbs, int32_t *sizes, int32_t nlimbs, int64_t ld, int64_t e) {
    int n64 = iabs_(z->size);
    int n = 2 * n64;
    if (n64 && (z->d[n64 - 1] >> 32) == 0) n--;
    if (n > nlimbs) return -1;
    for (int i = 0; i < nlimbs; i++)
        limbs[(int64_t)i * ld + e] = i < n ? (uint32_t)(z->d[i / 2] >> (32 * (i % 2))) : 0u;
    sizes[e] = z->size < 0 ? -n : n;
    return 0;
}

/* C (K x N) = A (K x M) * B (M x N) on HOST limb planes (row-major entries,
 * plane strides lda/ldb/ldc).  accumulate != 0 computes C += A*B
 * (mat_addmul, naive order).  Returns 0, or -1 when C lacks capacity. */
int oracle_matmul_planes(int K, int M, int N,
                         const uint32_t *Al, const int32_t *As, int64_t lda,
                         const uint32_t *Bl, const int32_t *Bs, int64_t ldb,
                         uint32_t *Cl, int32_t *Cs, int32_t cn, int64_t ldc,
                         int method, int basesz, int jobsz, int nthreads, int accumulate) {
    const num_ops *saved = g_ops;
    const int use_gmp = g_ops == &g_gmp_ops;
    g_ops = &g_own_ops;
    mat_t A = mat_init((unsigned)M, (unsigned)K), B = mat_init((unsigned)N, (unsigned)M), C = mat_init((unsigned)N, (unsigned)K);
    for (int64_t e = 0; e < (int64_t)K * M; e++) planes_to_own(&A[e], Al, As, lda, e);
    for (int64_t e = 0; e < (int64_t)M * N; e++) planes_to_own(&B[e], Bl, Bs, ldb, e);
    if (accumulate) for (int64_t e = 0; e < (int64_t)K * N; e++) planes_to_own(&C[e], Cl, Cs, ldc, e);
    if (use_gmp) {
        /* move the operands into GMP-managed numbers (same struct shape) */
        g_ops = &g_gmp_ops;
        mat_t A2 = mat_init((unsigned)M, (unsigned)K), B2 = mat_init((unsigned)N, (unsigned)M), C2 = mat_init((unsigned)N, (unsigned)K);
        for (int64_t e = 0; e < (int64_t)K * M; e++) g_gmp_ops.set(&A2[e], &A[e]);
        for (int64_t e = 0; e < (int64_t)M * N; e++) g_gmp_ops.set(&B2[e], &B[e]);
        for (int64_t e = 0; e < (int64_t)K * N; e++) g_gmp_ops.set(&C2[e], &C[e]);
        g_ops = &g_own_ops;
        mat_free((unsigned)M, (unsigned)K, A); mat_free((unsigned)N, (unsigned)M, B); mat_free((unsigned)N, (unsigned)K, C);
        A = A2; B = B2; C = C2;
        g_ops = &g_gmp_ops;
    }
    if (basesz <= 0) basesz = 32;
    if (jobsz <= 0) jobsz = 128;
    if (accumulate) naive_threaded((unsigned)K, (unsigned)M, (unsigned)N, C, N, A, M, B, N, nthreads, 1);
    else mul_squarify((unsigned)K, (unsigned)M, (unsigned)N, C, N, A, M, B, N, method, (unsigned)basesz, (unsigned)jobsz, nthreads);
    int rc = 0;
    for (int64_t e = 0; e < (int64_t)K * N; e++) if (own_to_planes(&C[e], Cl, Cs, cn, ldc, e)) rc = -1;
    mat_free((unsigned)M, (unsigned)K, A); mat_free((unsigned)N, (unsigned)M, B); mat_free((unsigned)N, (unsigned)K, C);
    g_ops = saved;
    return rc;
}

/* ---- bounded CPU samples of the reference's multiplication (benchmark leg) ------
 * Rows [r0, r0 + rb) of C = A*B by one of mat-cpu's methods, with only the
 * multiplication timed (like mat-cpu's "Multiplication took", mat-cpu/main.c).
 *   method 1: the naive order (mat.c:72-82), rows spread over the threads;
 *   method 31: mat-cpu -m 31's decomposition (matj.c:571-660): bs x bs block
 *     products (bs = jobsz) each run mat_mul_winograd with
 *     nlevels = floor(log2(bs / basesz)) (matj.c:583-586, util.c:24-26); the
 *     sample is one block row of C (rb = bs), its N/bs x M/bs block products
 *     spread over the threads, then summed per output block.
 * The sample's share of the full product is rb / K for both methods. */
typedef struct {
    unsigned bs, nbj, nkb, nlevels;
    const onum *A; long Ars; const onum *B; long Brs;
    mat_t *P;   /* nbj * nkb block products */
    int next; pthread_mutex_t mu;
} rowblock_job;
static void *rowblock_worker(void *arg) {
    rowblock_job *J = (rowblock_job *)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int t = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (t >= (int)(J->nbj * J->nkb)) break;
        unsigned bj = (unsigned)t / J->nkb, kb = (unsigned)t % J->nkb, bs = J->bs;
        J->P[t] = mat_init(bs, bs);
        mat_mul_winograd(bs, J->P[t], bs, J->A + (long)kb * bs, J->Ars, J->B + (long)kb * bs * J->Brs + (long)bj * bs,
                         J->Brs, J->nlevels);
    }
    return NULL;
}
double oracle_sample_rows(int K, int M, int N, const uint32_t *Al, const int32_t *As, int64_t lda,
                          const uint32_t *Bl, const int32_t *Bs, int64_t ldb, uint32_t *Cl, int32_t *Cs, int32_t cn,
                          int64_t ldc, int r0, int rb, int method, int basesz, int jobsz, int nthreads) {
    if (r0 < 0 || rb < 1 || r0 + rb > K || M < 1 || N < 1) return -1.0;
    if (basesz <= 0) basesz = 32;
    if (jobsz <= 0) jobsz = 128;
    const int blocked = method == 31 && rb == jobsz && M % jobsz == 0 && N % jobsz == 0;
    if (method != 1 && !blocked) return -1.0;
    const num_ops *saved = g_ops;
    const int use_gmp = g_ops == &g_gmp_ops;
    g_ops = &g_own_ops;
    mat_t A = mat_init((unsigned)M, (unsigned)rb), B = mat_init((unsigned)N, (unsigned)M);
    for (int64_t e = 0; e < (int64_t)rb * M; e++) planes_to_own(&A[e], Al, As, lda, (int64_t)r0 * M + e);
    for (int64_t e = 0; e < (int64_t)M * N; e++) planes_to_own(&B[e], Bl, Bs, ldb, e);
    if (use_gmp) {
        /* move the operands into GMP-managed numbers (same struct shape) */
        g_ops = &g_gmp_ops;
        mat_t A2 = mat_init((unsigned)M, (unsigned)rb), B2 = mat_init((unsigned)N, (unsigned)M);
        for (int64_t e = 0; e < (int64_t)rb * M; e++) g_gmp_ops.set(&A2[e], &A[e]);
        for (int64_t e = 0; e < (int64_t)M * N; e++) g_gmp_ops.set(&B2[e], &B[e]);
        g_ops = &g_own_ops;
        mat_free((unsigned)M, (unsigned)rb, A); mat_free((unsigned)N, (unsigned)M, B);
        A = A2; B = B2;
        g_ops = &g_gmp_ops;
    }
    mat_t C = mat_init((unsigned)N, (unsigned)rb);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (!blocked) {
        naive_threaded((unsigned)rb, (unsigned)M, (unsigned)N, C, N, A, M, B, N, nthreads, 0);
    } else {
        rowblock_job J;
        J.bs = (unsigned)jobsz; J.nbj = (unsigned)(N / jobsz); J.nkb = (unsigned)(M / jobsz);
        J.nlevels = jobsz <= basesz ? 0 : ilog2u((unsigned)(jobsz / basesz));
        J.A = A; J.Ars = M; J.B = B; J.Brs = N;
        J.P = (mat_t *)calloc((size_t)J.nbj * J.nkb, sizeof(mat_t));
        J.next = 0;
        pthread_mutex_init(&J.mu, NULL);
        int nt = nthreads < 1 ? 1 : nthreads;
        pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
        for (int i = 0; i < nt; i++) pthread_create(&th[i], NULL, rowblock_worker, &J);
        for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
        free(th);
        pthread_mutex_destroy(&J.mu);
        for (unsigned bj = 0; bj < J.nbj; bj++) {
            onum *Cb = C + (long)bj * J.bs;
            mat_t *Pb = J.P + (size_t)bj * J.nkb;
            mat_add(J.bs, J.bs, Cb, N, Pb[0], J.bs, Pb[J.nkb > 1 ? 1 : 0], J.bs);
            if (J.nkb == 1) mat_sub(J.bs, J.bs, Cb, N, Cb, N, Pb[0], J.bs);  /* C = P0 + P0 - P0 */
            for (unsigned kb = 2; kb < J.nkb; kb++) mat_add(J.bs, J.bs, Cb, N, Cb, N, Pb[kb], J.bs);
        }
        for (unsigned i = 0; i < J.nbj * J.nkb; i++) mat_free(J.bs, J.bs, J.P[i]);
        free(J.P);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    const double secs = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    int rc = 0;
    if (Cl)
        for (int64_t e = 0; e < (int64_t)rb * N; e++)
            if (own_to_planes(&C[e], Cl, Cs, cn, ldc, e)) rc = -1;
    mat_free((unsigned)M, (unsigned)rb, A); mat_free((unsigned)N, (unsigned)M, B); mat_free((unsigned)N, (unsigned)rb, C);
    g_ops = saved;
    return rc ? -1.0 : secs;
}

/* Elementwise signed add (sub = 0) or subtract (sub = 1) of n entries. */
int oracle_addsub_planes(int64_t n, const uint32_t *Al, const int32_t *As, int64_t lda,
                         const uint32_t *Bl, const int32_t *Bs, int64_t ldb,
                         uint32_t *Cl, int32_t *Cs, int32_t cn, int64_t ldc, int sub) {
    onum a, b, c; own_init(&a); own_init(&b); own_init(&c);
    int rc = 0;
    for (int64_t e = 0; e < n; e++) {
        planes_to_own(&a, Al, As, lda, e);
        planes_to_own(&b, Bl, Bs, ldb, e);
        if (sub) own_sub(&c, &a, &b); else own_add(&c, &a, &b);
        if (own_to_planes(&c, Cl, Cs, cn, ldc, e)) rc = -1;
    }
    own_clear(&a); own_clear(&b); own_clear(&c);
    return rc;
}

/* Elementwise w = u*v (op 0), w += u*v (op 1), w -= u*v (op 2). */
int oracle_mpz_mulops(int64_t n, int op, const uint32_t *Ul, const int32_t *Us, int64_t ldu,
                      const uint32_t *Vl, const int32_t *Vs, int64_t ldv,
                      uint32_t *Wl, int32_t *Ws, int32_t wn, int64_t ldw) {
    onum u, v, w, t; own_init(&u); own_init(&v); own_init(&w); own_init(&t);
    int rc = 0;
    for (int64_t e = 0; e < n; e++) {
        planes_to_own(&u, Ul, Us, ldu, e);
        planes_to_own(&v, Vl, Vs, ldv, e);
        if (op == 0) own_mul(&w, &u, &v);
        else {
            planes_to_own(&w, Wl, Ws, ldw, e);
            own_mul(&t, &u, &v);
            if (op == 1) own_add(&w, &w, &t); else own_sub(&w, &w, &t);
        }
        if (own_to_planes(&w, Wl, Ws, wn, ldw, e)) rc = -1;
    }
    own_clear(&u); own_clear(&v); own_clear(&w); own_clear(&t);
    return rc;
}

/* ---- batched mpn restatements, 32-bit limbs, operand b at p[i*ld + b] ------ */
void oracle_mpn_add_n(uint32_t *rp, const uint32_t *up, const uint32_t *vp, int n, int64_t ld, int64_t nb, uint32_t *cy) {
    for (int64_t b = 0; b < nb; b++) {
        uint64_t c = 0;
        for (int i = 0; i < n; i++) {
            uint64_t s = (uint64_t)up[i * ld + b] + vp[i * ld + b] + c;
            rp[i * ld + b] = (uint32_t)s; c = s >> 32;
        }
        cy[b] = (uint32_t)c;
    }
}
void oracle_mpn_sub_n(uint32_t *rp, const uint32_t *up, const uint32_t *vp, int n, int64_t ld, int64_t nb, uint32_t *cy) {
    for (int64_t b = 0; b < nb; b++) {
        uint64_t br = 0;
        for (int i = 0; i < n; i++) {
            uint64_t d = (uint64_t)up[i * ld + b] - vp[i * ld + b] - br;
            rp[i * ld + b] = (uint32_t)d; br = (d >> 32) & 1;
        }
        cy[b] = (uint32_t)br;
    }
}
/* op 0: rp = up*v, 1: rp += up*v, 2: rp -= up*v; cy = carry / borrow limb */
void oracle_mpn_mul1ops(int op, uint32_t *rp, const uint32_t *up, int n, const uint32_t *vl, int64_t ld, int64_t nb, uint32_t *cy) {
    for (int64_t b = 0; b < nb; b++) {
        uint64_t c = 0, v = vl[b];
        for (int i = 0; i < n; i++) {
            uint64_t p = (uint64_t)up[i * ld + b] * v + c;
            uint32_t lo = (uint32_t)p;
            c = p >> 32;
            if (op == 0) rp[i * ld + b] = lo;
            else if (op == 1) {
                uint64_t s = (uint64_t)rp[i * ld + b] + lo;
                rp[i * ld + b] = (uint32_t)s; c += s >> 32;
            } else {
                uint32_t r = rp[i * ld + b];
                rp[i * ld + b] = r - lo; c += r < lo;
            }
        }
        cy[b] = (uint32_t)c;
    }
}
void oracle_mpn_mul_basecase(uint32_t *rp, const uint32_t *up, int un, const uint32_t *vp, int vn, int64_t ld, int64_t nb) {
    for (int64_t b = 0; b < nb; b++) {
        for (int i = 0; i < un + vn; i++) rp[i * ld + b] = 0;
        for (int j = 0; j < vn; j++) {
            uint64_t c = 0, v = vp[j * ld + b];
            for (int i = 0; i < un; i++) {
                uint64_t t = (uint64_t)up[i * ld + b] * v + rp[(i + j) * ld + b] + c;
                rp[(i + j) * ld + b] = (uint32_t)t; c = t >> 32;
            }
            rp[(j + un) * ld + b] = (uint32_t)c;
        }
    }
}

/* The rest of the mpn layer the reference exposes (mat-gpu/addsub.cu:187-326,
 * mat-gpu/com.cu:35-42), GMP semantics, batched over operands with plane stride
 * ld.  rp = up + vp with un >= vn >= 0 limbs (vp zero-extended), carry out;
 * rp = up - vp, borrow out (addsub.cu:187-192, 284-289). */
void oracle_mpn_addsub(int sub, uint32_t *rp, const uint32_t *up, int un, const uint32_t *vp, int vn, int64_t ld,
                       int64_t nb, uint32_t *cy) {
    for (int64_t b = 0; b < nb; b++) {
        uint64_t c = 0;
        for (int i = 0; i < un; i++) {
            uint64_t y = i < vn ? vp[i * ld + b] : 0;
            if (!sub) {
                uint64_t s = (uint64_t)up[i * ld + b] + y + c;
                rp[i * ld + b] = (uint32_t)s; c = s >> 32;
            } else {
                uint64_t d = (uint64_t)up[i * ld + b] - y - c;
                rp[i * ld + b] = (uint32_t)d; c = (d >> 32) & 1;
            }
        }
        cy[b] = (uint32_t)c;
    }
}
/* rp = up +/- vl[b] (one limb), n >= 1; carry / borrow out (addsub.cu:236-242, 302-308) */
void oracle_mpn_addsub_1(int sub, uint32_t *rp, const uint32_t *up, int n, const uint32_t *vl, int64_t ld, int64_t nb,
                         uint32_t *cy) {
    for (int64_t b = 0; b < nb; b++) {
        uint64_t c = vl[b];
        for (int i = 0; i < n; i++) {
            if (!sub) {
                uint64_t s = (uint64_t)up[i * ld + b] + c;
                rp[i * ld + b] = (uint32_t)s; c = s >> 32;
            } else {
                uint64_t d = (uint64_t)up[i * ld + b] - c;
                rp[i * ld + b] = (uint32_t)d; c = (d >> 32) & 1;
            }
        }
        cy[b] = (uint32_t)c;
    }
}
/* res[b] = sign of up - vp over n limbs: -1, 0, 1 (addsub.cu:244-250) */
void oracle_mpn_cmp(const uint32_t *up, const uint32_t *vp, int n, int64_t ld, int64_t nb, int32_t *res) {
    for (int64_t b = 0; b < nb; b++) {
        int r = 0;
        for (int i = n - 1; i >= 0 && !r; i--) {
            uint32_t x = up[i * ld + b], y = vp[i * ld + b];
            if (x != y) r = x > y ? 1 : -1;
        }
        res[b] = r;
    }
}
/* res[b] = 1 when all n limbs are zero (addsub.cu:260-270) */
void oracle_mpn_zero_p(const uint32_t *up, int n, int64_t ld, int64_t nb, int32_t *res) {
    for (int64_t b = 0; b < nb; b++) {
        int z = 1;
        for (int i = 0; i < n; i++) z &= up[i * ld + b] == 0;
        res[b] = z;
    }
}
/* rp = -up mod B^n, cy = 1 unless up is zero (addsub.cu:310-326); rp = ~up (com.cu:35-42) */
void oracle_mpn_neg_com(int com, uint32_t *rp, const uint32_t *up, int n, int64_t ld, int64_t nb, uint32_t *cy) {
    for (int64_t b = 0; b < nb; b++) {
        uint64_t c = com ? 0 : 1;
        int nz = 0;
        for (int i = 0; i < n; i++) {
            uint32_t u = up[i * ld + b];
            nz |= u != 0;
            uint64_t s = (uint64_t)(uint32_t)~u + c;
            rp[i * ld + b] = (uint32_t)s; c = s >> 32;
        }
        if (cy) cy[b] = (uint32_t)nz;
    }
}

/* ------------------------------------------------------------------------ */
#ifdef ORACLE_MAIN
/* A mat-cpu compatible command line (mat-cpu/main.c:14-34): -g generates
 * matrices from a seeded xorshift stream (not GMP's RNG: inputs are exchanged
 * as text), -i reads them, -p prints, -m method, -B basesz, -J jobsz, -C cores. */
#include <getopt.h>
static uint64_t rs_state = 88172645463325252ull;
static uint64_t xr(void) { rs_state ^= rs_state << 13; rs_state ^= rs_state >> 7; rs_state ^= rs_state << 17; return rs_state; }
static void gen_num(int nbits) {
    int nl = (nbits + 63) / 64;
    uint64_t *d = (uint64_t *)calloc((size_t)(nl ? nl : 1), 8);
    for (int i = 0; i < nl; i++) d[i] = xr();
    if (nbits % 64) d[nl - 1] &= (1ull << (nbits % 64)) - 1;
    onum z = {nl, mag_norm(d, nl), d};
    if (xr() & 1) z.size = -z.size;
    char *buf = NULL; size_t len = 0, cap = 0;
    put_num(&buf, &len, &cap, &z);
    fwrite(buf, 1, len, stdout);
    free(buf); free(d);
}
int main(int argc, char **argv) {
    int mode = 'r', print = 0, method = 31, basesz = 32, jobsz = 128, ncores = 1, gmp = 0;
    unsigned K = 0, M = 0, N = 0; int nbits = 0; unsigned long seed = 1;
    int opt;
    while ((opt = getopt(argc, argv, "hgirpn:b:s:m:B:J:C:G")) != -1) {
        switch (opt) {
        case 'g': case 'i': case 'r': mode = opt; break;
        case 'p': print = 1; break;
        case 'n': if (sscanf(optarg, "%u,%u,%u", &K, &M, &N) != 3) { fprintf(stderr, "Invalid -n\n"); return 1; } break;
        case 'b': nbits = atoi(optarg); break;
        case 's': seed = strtoul(optarg, NULL, 10); break;
        case 'm': method = atoi(optarg); break;
        case 'B': basesz = atoi(optarg); break;
        case 'J': jobsz = atoi(optarg); break;
        case 'C': ncores = atoi(optarg); break;
        case 'G': gmp = 1; break;
        default: fprintf(stderr, "Usage: %s [-hgirpG] [-n K,M,N] [-b bits] [-s seed] [-m method] [-B basesz] [-J jobsz] [-C ncores]\n", argv[0]); return opt == 'h' ? 0 : 1;
        }
    }
    rs_state ^= seed * 0x9E3779B97F4A7C15ull; if (!rs_state) rs_state = 1;
    if (gmp && oracle_set_backend(1)) { fprintf(stderr, "libgmp.so.10 not available\n"); return 1; }
    if (mode == 'g') {
        printf("%u %u %u\n", K, M, N);
        for (unsigned y = 0; y < K; y++) { for (unsigned x = 0; x < M; x++) { if (x) putchar(' '); gen_num(nbits); } putchar('\n'); }
        putchar('\n');
        for (unsigned y = 0; y < M; y++) { for (unsigned x = 0; x < N; x++) { if (x) putchar(' '); gen_num(nbits); } putchar('\n'); }
        putchar('\n');
        return 0;
    }
    size_t cap = 1 << 20, len = 0; char *in = (char *)malloc(cap);
    size_t r;
    while ((r = fread(in + len, 1, cap - len, stdin)) > 0) { len += r; if (len == cap) { cap *= 2; in = (char *)realloc(in, cap); } }
    double secs = 0;
    char *out = oracle_matmul_text(in, len, method, basesz, jobsz, ncores, &secs);
    if (!out) { fprintf(stderr, "parse error\n"); return 1; }
    fprintf(stderr, "Multiplication took %g seconds\n", secs);
    if (print) fputs(out, stdout);
    free(out); free(in);
    return 0;
}
#endif
