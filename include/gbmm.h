/*
 * gbmm.h -- C ABI of gbmm, an exact signed big-integer matrix-multiplication
 * engine for NVIDIA GB300 (sm_103a).
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns a
 * gbmm_status and never aborts.  Device pointers are CUDA global-memory
 * pointers; `stream` is a cudaStream_t passed as void* (NULL = legacy default
 * stream).  Work is enqueued asynchronously on that stream unless a function
 * says otherwise.  The text after "replaces:" names the reference interface
 * (tomsmeding/bachelor-thesis, path:line) that the entry point stands in for.
 *
 * Number format ("limb planes").  A matrix of rows x cols signed integers is
 * stored structure-of-arrays: limb i (32-bit, least significant first) of
 * entry (r, c) lives at limbs[i*ld + r*rs + c] for i < nlimbs, and
 * sizes[r*rs + c] holds the GMP-style signed size: |size| is the normalized
 * limb count (top limb nonzero, zero has size 0) and the sign of size is the
 * sign of the value.  Limbs at positions >= |size| must be zero.  This is the
 * interleaved layout of the reference (mat-gpu/gmp-es-mpz.h:38-42,
 * mat-gpu/main.cu:137-156) with the fixed NUM_SIZE capacity removed.
 *
 * Per-device state.  The library keeps a small amount of state per device
 * ordinal for the life of the process (the device error word kernels report
 * capacity overflow and expired waits in, and the device address of the fixed
 * scratch array of gbmm_mpn_toom22_mul_noalloc).  cudaDeviceReset destroys it
 * behind the library's back: do not call the library on a device after
 * resetting it in the same process.
 */
#ifndef GBMM_H
#define GBMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbmm_status {
    GBMM_OK = 0,
    GBMM_ERR_INVALID = 1,     /* bad argument: null pointer, bad shape, forbidden aliasing */
    GBMM_ERR_CAPACITY = 2,    /* an output has fewer limb planes than the exact result needs */
    GBMM_ERR_CUDA = 3,        /* a CUDA runtime or driver call failed */
    GBMM_ERR_PARSE = 4,       /* malformed hexadecimal matrix text */
    GBMM_ERR_NOMEM = 5,       /* host or device allocation failed */
    GBMM_ERR_TIMEOUT = 6,     /* a bounded device-side wait gave up */
    GBMM_ERR_UNSUPPORTED = 7  /* the request is valid but the library cannot run it */
} gbmm_status;

/* A device matrix view in limb planes (see the file comment). */
typedef struct gbmm_mat {
    int32_t rows;
    int32_t cols;
    int32_t nlimbs;      /* number of limb planes (capacity per entry, 32-bit limbs) */
    int32_t pad_;
    int64_t rs;          /* row stride in entries */
    int64_t ld;          /* plane stride in entries */
    uint32_t *limbs;     /* device pointer */
    int32_t *sizes;      /* device pointer */
} gbmm_mat;

/* Matrix multiplication paths. */
typedef enum gbmm_path {
    GBMM_PATH_AUTO = 0,  /* heuristic (or learned model when loaded) picks */
    GBMM_PATH_LIMB = 1,  /* batched limb kernels (schoolbook column sums) */
    GBMM_PATH_CRT = 2    /* multi-modular: residue GEMMs on tcgen05 tensor cores */
} gbmm_path;

/* Square-recursion methods, numbered like mat-gpu's -m switch (mat-gpu/main.cu:358-502). */
typedef enum gbmm_method {
    GBMM_METHOD_NAIVE = 1,      /* one per-entry kernel over the whole product */
    GBMM_METHOD_STRASSEN = 3,   /* Strassen 7-product recursion, 3 temporaries */
    GBMM_METHOD_WINOGRAD = 35,  /* Winograd 7-product recursion, 3 temporaries */
    GBMM_METHOD_NAIVE_REC = 4,  /* 8-product block recursion */
    /* Winograd's tree down to the cutoff with CRT leaf products (no mat-gpu
     * counterpart): the tree's sums and combinations run as limb kernels, its 7^L
     * leaf products together in the grouped CRT launches.  Square products of
     * single-pass leaves (k <= 512); others take the plain CRT form. */
    GBMM_METHOD_WINOGRAD_CRT = 350
} gbmm_method;

/* Candidate plans for one product: the plans gbmm_autotune times and the
 * learned cost model predicts (one head each), and the unit GBMM_PATH_AUTO
 * chooses among.  No counterpart in the reference (its method is fixed per run
 * by -m, mat-gpu/main.cu:358-502). */
typedef enum gbmm_plan {
    GBMM_PLAN_LIMB_NAIVE = 0,  /* per-entry kernel over the whole product, no recursion */
    GBMM_PLAN_LIMB_W32 = 1,    /* Winograd tree down to blocks of 32 (recursion depth from the size) */
    GBMM_PLAN_LIMB_W64 = 2,    /* ... down to blocks of 64 */
    GBMM_PLAN_LIMB_W128 = 3,   /* ... down to blocks of 128 */
    GBMM_PLAN_CRT = 4,         /* CRT, moduli from the bound, GEMM tile form chosen by size */
    GBMM_PLAN_CRT_SINGLE = 5,  /* CRT with one-CTA tiles of 128 entries in every GEMM */
    GBMM_PLAN_CRT_PAIR = 6,    /* CRT with CTA-pair tiles of 256 entries in the product and reconstruction */
    GBMM_PLAN_CRT_SPLIT = 7,   /* CRT after one limb-half split of the longer operand, its halves stacked
                                  into one product with fewer moduli (the modulus count is the choice) */
    GBMM_NPLANS = 8
} gbmm_plan;

typedef struct gbmm_opts {
    int32_t path;        /* gbmm_path */
    int32_t method;      /* gbmm_method (limb path) */
    int32_t cutoff;      /* recursion stops at blocks <= cutoff (0 = library default) */
    int32_t nprimes;     /* CRT: number of moduli (0 = derived from the bit bound) */
    int32_t accumulate;  /* nonzero: C += A*B (mat_addmul) instead of C = A*B */
    int32_t plan;        /* 0: path / method / cutoff as above; 1 + gbmm_plan: run that plan */
    int32_t reserved[2];
} gbmm_opts;

typedef struct gbmm_handle_s *gbmm_handle;

/* ---- handle / errors -------------------------------------------------- */

/* Creates a handle bound to the current CUDA device.  The handle owns a
 * device workspace arena, a CRT table cache and the tuning tables.
 * replaces: global state of mat-gpu/main.cu:321-326 (cudaSetDevice + pinned buffers). */
gbmm_status gbmm_create(gbmm_handle *out);
gbmm_status gbmm_destroy(gbmm_handle h);
/* Binds the stream that handle-level calls enqueue on (NULL = default stream). */
gbmm_status gbmm_set_stream(gbmm_handle h, void *stream);
/* Thread-local text of the last error reported by any gbmm call in this thread. */
const char *gbmm_last_error_string(void);
/* Library version, "gbmm <major>.<minor>". */
const char *gbmm_version(void);
/* Number of device kernels this process has launched through the library
 * (instrumentation; lets a caller count the kernels inside a timed region).
 * No counterpart in the reference. */
uint64_t gbmm_kernel_launches(void);
/* Per-kernel timing with CUDA events recorded around every library launch on
 * its stream.  gbmm_profile(1) clears and starts recording, gbmm_profile(0)
 * stops; gbmm_profile_read synchronises the recorded events and writes JSON
 * {"kernel": [launches, total_ms], ...}.  Do not enable while capturing a
 * CUDA graph.  replaces: the per-op stderr prints and wall-clock timers of
 * mat-gpu (mat-gpu/mat-gpu.cu:15-29, main.cu:217-218, 401-420). */
gbmm_status gbmm_profile(int32_t enable);
gbmm_status gbmm_profile_read(char *out, size_t cap, size_t *written);

/* ---- host-side text and GMP-limb conversion (no GPU needed) -------------- */

/* Parses `count` whitespace-separated hexadecimal signed integers (optional '-',
 * digits 0-9a-fA-F) from text[0..len) into HOST limb planes with plane stride
 * ld and capacity nlimbs; *consumed receives the number of bytes read.
 * replaces: mat_read (mat-cpu/mat.c:336-342) / gpu_mpz_inp_file (mat-gpu/mpz.cu:148-180). */
gbmm_status gbmm_parse_hex(const char *text, size_t len, int64_t count,
                           uint32_t *limbs, int32_t *sizes, int32_t nlimbs, int64_t ld,
                           size_t *consumed);

/* Formats rows x cols entries from HOST limb planes as mat_write does: entries
 * separated by one space, '\n' after each row, one extra '\n' at the end.
 * Writes at most cap bytes to out (may be NULL to query) and stores the full
 * length (without terminator) in *written.
 * replaces: mat_write (mat-cpu/mat.c:344-353) / gpu_mpz_out_file (mat-gpu/mpz.cu:182-204). */
gbmm_status gbmm_format_hex(const uint32_t *limbs, const int32_t *sizes, int32_t nlimbs,
                            int64_t ld, int32_t rows, int32_t cols, int64_t rs,
                            char *out, size_t cap, size_t *written);

/* Converts `count` numbers given as GMP mpz data (64-bit limbs, numbers laid out
 * back to back: limbs64[offsets[e] .. offsets[e]+|sizes64[e]|), sign in sizes64)
 * into HOST limb planes.  replaces: gpu_crt.cu:19-46 (gpu_from_gmp). */
gbmm_status gbmm_import_gmp(int64_t count, const uint64_t *limbs64, const int64_t *offsets,
                            const int32_t *sizes64, uint32_t *limbs, int32_t *sizes,
                            int32_t nlimbs, int64_t ld);
/* Inverse of gbmm_import_gmp: writes 64-bit limbs at offsets[e], sizes into sizes64.
 * replaces: gpu_crt.cu:19-46 (gmp_from_gpu). */
gbmm_status gbmm_export_gmp(int64_t count, const uint32_t *limbs, const int32_t *sizes,
                            int32_t nlimbs, int64_t ld, uint64_t *limbs64,
                            const int64_t *offsets, int32_t *sizes64);

/* ---- device matrices ------------------------------------------------------ */

/* Copies HOST limb planes (plane stride host_ld, rows x cols row-major) into a
 * device matrix and back.  Synchronous with respect to `stream` completion. */
gbmm_status gbmm_upload(gbmm_mat dst, const uint32_t *host_limbs, const int32_t *host_sizes,
                        int32_t host_nlimbs, int64_t host_ld, void *stream);
gbmm_status gbmm_download(gbmm_mat src, uint32_t *host_limbs, int32_t *host_sizes,
                          int32_t host_nlimbs, int64_t host_ld, void *stream);

/* Text in, device matrix out: parses rows*cols hex entries directly.
 * replaces: mat-gpu/main.cu:342-344 (-i input path). */
gbmm_status gbmm_import_hex(gbmm_mat dst, const char *text, size_t len, size_t *consumed,
                            void *stream);
/* Device matrix to text in mat_write format.  replaces: mat-gpu/main.cu:507-515 (-p). */
gbmm_status gbmm_export_hex(gbmm_mat src, char *out, size_t cap, size_t *written, void *stream);

/* Maximum bit length of the magnitudes in a device matrix (synchronous). */
gbmm_status gbmm_max_bits(gbmm_mat a, int64_t *bits, void *stream);

/* C = A + B and C = A - B, elementwise signed.
 * replaces: add_matrices_gpu / sub_matrices_gpu (mat-gpu/mat-gpu.cu:10-36),
 *           launcher_add / launcher_sub (mat-gpu/mat-gpu-launchers.cu:66-120). */
gbmm_status gbmm_mat_add(gbmm_mat c, gbmm_mat a, gbmm_mat b, void *stream);
gbmm_status gbmm_mat_sub(gbmm_mat c, gbmm_mat a, gbmm_mat b, void *stream);

/* Limb planes each output needs for C = A*B with these inputs and options
 * (includes recursion headroom). */
gbmm_status gbmm_matmul_limbs_needed(int32_t a_nlimbs, int32_t b_nlimbs, int32_t inner,
                                     const gbmm_opts *opts, int32_t *nlimbs);

/* C (K x N) = A (K x M) * B (M x N), or C += A*B when opts->accumulate.
 * replaces: squarify_mul_pregpu (mat-gpu/mat-pregpu.cu:548-576) with
 * winograd_pregpu / strassen_pregpu / naive_recursive_pregpu / naive_smallrect
 * (mat-gpu/mat-pregpu.cu:99-546, mat-gpu/mat-gpu.cu:79-475), and mat_mul /
 * mat_addmul / mat_mul_winograd (mat-cpu/mat.c:72-334). */
gbmm_status gbmm_matmul(gbmm_handle h, gbmm_mat c, gbmm_mat a, gbmm_mat b,
                        const gbmm_opts *opts);

/* The per-entry product kernel alone on one view (no recursion): C = A*B or
 * C += A*B.  replaces: launcher_mul / launcher_addmul and their _strided twins
 * (mat-gpu/mat-gpu-launchers.cu:6-63, mat-gpu/mat-core.h:7-137). */
gbmm_status gbmm_mat_mul_naive(gbmm_mat c, gbmm_mat a, gbmm_mat b, int32_t accumulate,
                               void *stream);

/* One job of a batched call. */
typedef struct gbmm_job {
    gbmm_mat c, a, b;
    int32_t path;        /* gbmm_path, AUTO lets the dispatcher choose per job */
    int32_t cutoff;
    int32_t nprimes;
    int32_t chosen_path; /* out: path the dispatcher used */
    int32_t chosen_plan; /* out: gbmm_plan the dispatcher ran (-1: the options were given field by field) */
} gbmm_job;

/* Runs many independent products of uneven shape and bit length: jobs planned
 * for the limb kernel without recursion go through one persistent kernel over
 * a device work queue; CRT products with inner dimension up to 512 and fewer
 * than 2^15 entries in C (directly or after one limb-half split) run in grouped
 * launches, one persistent launch per CRT stage over the tiles of all of them;
 * the others (Winograd trees, larger CRT products) run side by side on streams
 * forked from the handle's stream.
 * The launch sequence is captured into a CUDA graph and replayed on later calls
 * with the same job signature; capture needs the handle bound to a created stream
 * (gbmm_set_stream): on the legacy default stream every call runs eagerly.  The CRT_SINGLE / CRT_PAIR plans fix the tile
 * form of a product run alone; in the grouped launches every product uses the
 * grouped forms (one-CTA product tiles, CTA-pair reconstruction tiles).
 * replaces: the unused chunked-stream job DAG (mat-gpu/job.cu:32-338). */
gbmm_status gbmm_matmul_batched(gbmm_handle h, gbmm_job *jobs, int32_t njobs, const gbmm_opts *opts);
/* One product on host buffers: dense limb planes (limb i of entry e at
 * [i * rows * cols + e]) and a sizes plane per matrix, C = A * B with C K x N,
 * A K x M, B M x N.  Pinned host memory lets the copies overlap compute. */
typedef struct gbmm_host_job {
    int32_t K, M, N;
    int32_t a_nlimbs, b_nlimbs, c_nlimbs;
    const uint32_t *a_limbs;
    const int32_t *a_sizes;
    const uint32_t *b_limbs;
    const int32_t *b_sizes;
    uint32_t *c_limbs;
    int32_t *c_sizes;
    int32_t path;        /* gbmm_path; AUTO lets the dispatcher choose */
    int32_t method;      /* gbmm_method for the limb path, 0 = Winograd */
    int32_t cutoff;      /* Winograd cutoff, 0 = default */
    int32_t nprimes;     /* CRT moduli, 0 = derived from the bit lengths */
    int32_t chosen_path; /* out: path the dispatcher used */
} gbmm_host_job;

/* Runs a list of products whose operands and results live in host memory and
 * returns when every C is back in host memory.  Two device slots and separate
 * upload / download streams let job j+1's host->device copies and job j-1's
 * device->host copy overlap job j's compute.
 * replaces: the blocking host <-> device transfers around each product
 * (mat-gpu/mat-pregpu.cu:10-96, transfer_recurse; mat-gpu/main.cu:362-381). */
gbmm_status gbmm_matmul_host(gbmm_handle h, gbmm_host_job *jobs, int32_t njobs);

/* Device memory a gbmm_matmul_host product may use (0, the default: 90% of the free
 * memory plus the handle's workspace).  A product that needs more runs out of core:
 * C in row x column blocks, the inner dimension in chunks accumulated on the device,
 * sub-blocks copied straight from and to the host planes.
 * replaces: the host-level recursion above the GPU's memory
 * (mat-gpu/mat-pregpu.cu:273-467). */
gbmm_status gbmm_set_device_budget(gbmm_handle h, uint64_t bytes);

/* Turns CUDA-graph capture and replay of batches on (default) or off.
 * No counterpart in the reference. */
gbmm_status gbmm_set_graphs(gbmm_handle h, int32_t enable);

/* ---- autotuner / dispatch tables -------------------------------------------
 * gbmm_autotune times every candidate plan (gbmm_plan: the limb kernel alone,
 * Winograd at three cutoffs, CRT with three tile forms and with a limb-half
 * split) on each job's own buffers (C is overwritten), keeps the fastest per
 * shape class for GBMM_PATH_AUTO, and appends one JSON line per timing to
 * log_path (may be NULL): the timing record the learned cost model trains on.
 * Limb candidates predicted far slower than any plan needs (m k n la lb > 2e11)
 * and Winograd cutoffs that give no recursion at this size are skipped.
 * replaces: the fixed BASE_SIZE / TRANSFER_SIZE / GPU_BLK_* tuning constants
 * (mat-gpu/mat-params.h:4-14). */
gbmm_status gbmm_autotune(gbmm_handle h, const gbmm_job *jobs, int32_t njobs, int32_t repeats,
                          const char *log_path);
gbmm_status gbmm_tune_save(gbmm_handle h, const char *path);
gbmm_status gbmm_tune_load(gbmm_handle h, const char *path);

/* ---- learned cost model ------------------------------------------------------
 * An 8 -> 64 -> 64 -> GBMM_NPLANS MLP (BF16 weights, FP32 accumulation, ReLU)
 * whose heads predict log2(ms) of each gbmm_plan for one product: the path,
 * the recursion depth (through the Winograd cutoff), the CRT tile form and the
 * modulus count per product (through the split).  When enabled with
 * gbmm_model_use, GBMM_PATH_AUTO runs the plan with the cheapest head; the
 * plain heuristic (and the autotuner's table) stay the fallback.  Training
 * runs on the GPU (forward, backward, Adam kernels) on feature rows from
 * gbmm_model_features and targets from the autotuner's timing log (one column
 * per plan, NaN where a plan was not timed).
 * No counterpart in the reference. */
int32_t gbmm_model_nparams(void);
gbmm_status gbmm_model_features(int32_t m, int32_t k, int32_t n, int32_t la, int32_t lb, float *out8);
gbmm_status gbmm_model_init(gbmm_handle h, uint64_t seed);
gbmm_status gbmm_model_set_params(gbmm_handle h, const float *params);
gbmm_status gbmm_model_get_params(gbmm_handle h, float *master, uint16_t *bf16_params);
gbmm_status gbmm_model_use(gbmm_handle h, int32_t enable);
/* X: nsamp x 8 features, Y: nsamp x GBMM_NPLANS predictions (host arrays). */
gbmm_status gbmm_model_predict(gbmm_handle h, const float *X, int32_t nsamp, float *Y);
/* Mean-squared-error loss and its gradient (gbmm_model_nparams floats) on
 * (X, T); T entries may be NaN for missing heads. */
gbmm_status gbmm_model_gradient(gbmm_handle h, const float *X, const float *T, int32_t nsamp, float *grad,
                                float *loss);
/* Full-batch Adam for `epochs` steps with learning rate lr.  The dispatcher
 * consults a head only once it has trained on at least 8 measured targets, and
 * runs the model's plan instead of the heuristic's only when the model predicts
 * it at least 10% faster. */
gbmm_status gbmm_model_train(gbmm_handle h, const float *X, const float *T, int32_t nsamp, int32_t epochs,
                             float lr, float *final_loss);

/* ---- batched mpn layer ----------------------------------------------------
 * Operand b (0 <= b < nb) of a batched call has limb i at ptr[i*ld + b].
 * Carry / borrow limbs are returned per operand in the device array `cy`.
 * Semantics per operand are GMP's. */

/* rp = up + vp (n limbs), cy[b] = carry.  Warp carry-lookahead.
 * replaces: gpu_mpn_add_n (mat-gpu/add_n.cu:36-59). */
gbmm_status gbmm_mpn_add_n(uint32_t *rp, const uint32_t *up, const uint32_t *vp, int32_t n,
                           int64_t ld, int64_t nb, uint32_t *cy, void *stream);
/* rp = up - vp (n limbs), cy[b] = borrow.  replaces: gpu_mpn_sub_n (mat-gpu/sub_n.cu:36-59). */
gbmm_status gbmm_mpn_sub_n(uint32_t *rp, const uint32_t *up, const uint32_t *vp, int32_t n,
                           int64_t ld, int64_t nb, uint32_t *cy, void *stream);
/* rp (un limbs) = up (un) + vp (vn), un >= vn >= 0, un >= 1; cy[b] = carry.
 * replaces: gpu_mpn_add (mat-gpu/addsub.cu:187-192). */
gbmm_status gbmm_mpn_add(uint32_t *rp, const uint32_t *up, int32_t un, const uint32_t *vp, int32_t vn,
                         int64_t ld, int64_t nb, uint32_t *cy, void *stream);
/* rp (un limbs) = up (un) - vp (vn), un >= vn >= 0, un >= 1; cy[b] = borrow.
 * replaces: gpu_mpn_sub (mat-gpu/addsub.cu:284-289). */
gbmm_status gbmm_mpn_sub(uint32_t *rp, const uint32_t *up, int32_t un, const uint32_t *vp, int32_t vn,
                         int64_t ld, int64_t nb, uint32_t *cy, void *stream);
/* rp = up + vl[b] (one limb per operand), n >= 1; cy[b] = carry.
 * replaces: gpu_mpn_add_1 (mat-gpu/addsub.cu:236-242). */
gbmm_status gbmm_mpn_add_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                           int64_t nb, uint32_t *cy, void *stream);
/* rp = up - vl[b], n >= 1; cy[b] = borrow.  replaces: gpu_mpn_sub_1 (mat-gpu/addsub.cu:302-308). */
gbmm_status gbmm_mpn_sub_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl, int64_t ld,
                           int64_t nb, uint32_t *cy, void *stream);
/* result[b] = -1, 0 or 1: the sign of up - vp over n limbs (device int32 array).
 * replaces: gpu_mpn_cmp (mat-gpu/addsub.cu:244-250). */
gbmm_status gbmm_mpn_cmp(const uint32_t *up, const uint32_t *vp, int32_t n, int64_t ld, int64_t nb,
                         int32_t *result, void *stream);
/* result[b] = 1 when all n >= 1 limbs of operand b are zero, else 0.
 * replaces: gpu_mpn_zero_p (mat-gpu/addsub.cu:260-270). */
gbmm_status gbmm_mpn_zero_p(const uint32_t *up, int32_t n, int64_t ld, int64_t nb, int32_t *result,
                            void *stream);
/* rp = -up mod 2^(32n), n >= 1; cy[b] = 1 unless up is zero (GMP's borrow).
 * replaces: gpu_mpn_neg (mat-gpu/addsub.cu:310-326). */
gbmm_status gbmm_mpn_neg(uint32_t *rp, const uint32_t *up, int32_t n, int64_t ld, int64_t nb, uint32_t *cy,
                         void *stream);
/* rp = ~up (one's complement of every limb), n >= 1.  replaces: gpu_mpn_com (mat-gpu/com.cu:35-42). */
gbmm_status gbmm_mpn_com(uint32_t *rp, const uint32_t *up, int32_t n, int64_t ld, int64_t nb, void *stream);
/* rp = up * vl[b], cy[b] = high limb.  replaces: gpu_mpn_mul_1 (mat-gpu/mul_1.cu:37-58). */
gbmm_status gbmm_mpn_mul_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl,
                           int64_t ld, int64_t nb, uint32_t *cy, void *stream);
/* rp += up * vl[b], cy[b] = carry limb.  replaces: gpu_mpn_addmul_1 (mat-gpu/addmul_1.cu:39-63). */
gbmm_status gbmm_mpn_addmul_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl,
                              int64_t ld, int64_t nb, uint32_t *cy, void *stream);
/* rp -= up * vl[b], cy[b] = borrow limb.  replaces: gpu_mpn_submul_1 (mat-gpu/submul_1.cu:41-65). */
gbmm_status gbmm_mpn_submul_1(uint32_t *rp, const uint32_t *up, int32_t n, const uint32_t *vl,
                              int64_t ld, int64_t nb, uint32_t *cy, void *stream);
/* rp (un+vn limbs) = up (un) * vp (vn), un >= vn >= 1.
 * replaces: gpu_mpn_mul_basecase (mat-gpu/mul_basecase.cu:54-76). */
gbmm_status gbmm_mpn_mul_basecase(uint32_t *rp, const uint32_t *up, int32_t un,
                                  const uint32_t *vp, int32_t vn, int64_t ld, int64_t nb,
                                  void *stream);
/* Scratch limbs per operand that gbmm_mpn_toom22_mul needs (times ld planes):
 * 6n + 2 with n = an - floor(an/2), or -1 when that does not fit an int32
 * (an above about 7.1e8 limbs; the Toom-2.2 entry points reject such an). */
int32_t gbmm_mpn_toom22_mul_itch(int32_t an, int32_t bn);
/* pp (an+bn limbs) = ap * bp by one Karatsuba (Toom-2.2) split; preconditions
 * as GMP: an >= bn, with s = an/2, n = an - s, t = bn - n: 0 < t <= s.
 * scratch holds gbmm_mpn_toom22_mul_itch(an, bn) planes of stride ld.
 * replaces: gpu_mpn_toom22_mul (mat-gpu/toom22_mul.cu:109-240). */
gbmm_status gbmm_mpn_toom22_mul(uint32_t *pp, const uint32_t *ap, int32_t an,
                                const uint32_t *bp, int32_t bn, uint32_t *scratch,
                                int64_t ld, int64_t nb, void *stream);
/* Bytes of the fixed device array that gbmm_mpn_toom22_mul_noalloc uses as
 * scratch (one per GPU that loads the library, held until process exit). */
#define GBMM_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)
/* Same product as gbmm_mpn_toom22_mul, for callers that cannot allocate device
 * memory: code that runs while another component owns every device allocation
 * (an embedding runtime with its own pool or allocation accounting), or a
 * thread that must not enter cudaMalloc / cudaFree because those calls may
 * synchronise the device or take a global lock.  The caller passes inputs and
 * outputs only; the scratch is the library's fixed device array, so
 * gbmm_mpn_toom22_mul_itch(an, bn) * ld * 4 must not exceed
 * GBMM_NOALLOC_SCRATCH_BYTES (GBMM_ERR_CAPACITY otherwise).  The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture.  The address is cached per
 * device ordinal for the life of the process: after cudaDeviceReset (or any
 * teardown of the primary context) it is stale, so do not call this entry
 * point after a reset.  Every call shares the one array, so calls whose
 * kernels may overlap on the GPU (different streams without ordering between
 * them) race on it.  No allocation of any kind.
 * No counterpart in the reference. */
gbmm_status gbmm_mpn_toom22_mul_noalloc(uint32_t *pp, const uint32_t *ap, int32_t an,
                                        const uint32_t *bp, int32_t bn, int64_t ld, int64_t nb,
                                        void *stream);
/* rp (un+vn) = up * vp, un >= vn >= 1, choosing basecase or Toom-2.2 (the
 * Toom-2.2 path uses scratch from the handle).
 * replaces: gpu_mpn_mul (mat-gpu/mul.cu:61-401), gpu_mpn_mul_n (mat-gpu/mul_n.cu:36-111). */
gbmm_status gbmm_mpn_mul(gbmm_handle h, uint32_t *rp, const uint32_t *up, int32_t un,
                         const uint32_t *vp, int32_t vn, int64_t ld, int64_t nb);

/* ---- batched mpz layer ----------------------------------------------------
 * w, u, v are 1 x nb (or any shape, used elementwise) device matrices. */

/* w = u + v, w = u - v.  replaces: gpu_mpz_add / gpu_mpz_sub (mat-gpu/mpz-add.cu:49-122). */
gbmm_status gbmm_mpz_add(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream);
gbmm_status gbmm_mpz_sub(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream);
/* w = u * v.  replaces: gpu_mpz_mul (mat-gpu/mpz-mul.cu:51-107). */
gbmm_status gbmm_mpz_mul(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream);
/* w += u * v and w -= u * v.
 * replaces: gpu_mpz_addmul / gpu_mpz_submul (mat-gpu/mpz-aorsmul.cu:70-290). */
gbmm_status gbmm_mpz_addmul(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream);
gbmm_status gbmm_mpz_submul(gbmm_mat w, gbmm_mat u, gbmm_mat v, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GBMM_H */
