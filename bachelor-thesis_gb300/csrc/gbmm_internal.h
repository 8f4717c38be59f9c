// Internal declarations shared by the gbmm translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/gbmm.h"

namespace gbmm {

// ---- error reporting ---------------------------------------------------------
gbmm_status set_error(gbmm_status st, const char *fmt, ...);
gbmm_status cuda_error(cudaError_t e, const char *what);

#define GBMM_CUDA_TRY(expr)                                                     \
    do {                                                                        \
        cudaError_t e_ = (expr);                                                \
        if (e_ != cudaSuccess) return ::gbmm::cuda_error(e_, #expr);            \
    } while (0)
#define GBMM_TRY(expr)                                                          \
    do {                                                                        \
        gbmm_status s_ = (expr);                                                \
        if (s_ != GBMM_OK) return s_;                                           \
    } while (0)

static inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// ---- device error word ---------------------------------------------------------
// Kernels record failures (capacity overflow, bounded waits that gave up) in a
// per-device word instead of trapping; the host reads and clears it at sync points.
enum device_error_bits : uint32_t {
    DEVERR_CAPACITY = 1u,
    DEVERR_TIMEOUT = 2u,
    DEVERR_BADARG = 4u,
};
uint32_t *device_error_word();  // device pointer, allocated once per device
gbmm_status check_device_error(cudaStream_t s);

// ---- launch accounting -------------------------------------------------------------
// Every kernel launch made by the library bumps this counter (reported through
// gbmm_kernel_launches so a benchmark can state how many of its kernels ran).
void count_launch(uint64_t n = 1);
// Per-kernel CUDA-event timing (enabled with gbmm_profile): a LaunchScope
// placed around a launch counts it and, when profiling is on, records events
// before and after it on the launching stream.
struct LaunchScope {
    LaunchScope(const char *name, cudaStream_t s);
    ~LaunchScope();
    const char *name_;
    cudaStream_t s_;
    int slot_;
};

// ---- view helpers ----------------------------------------------------------------
static inline gbmm_mat sub_view(const gbmm_mat &m, int32_t r0, int32_t c0, int32_t rows, int32_t cols) {
    gbmm_mat v = m;
    int64_t off = (int64_t)r0 * m.rs + c0;
    v.limbs = m.limbs + off;
    v.sizes = m.sizes + off;
    v.rows = rows;
    v.cols = cols;
    return v;
}
gbmm_status validate_mat(const gbmm_mat &m, const char *name);

// ---- limb kernels (limb.cu) -------------------------------------------------------
gbmm_status launch_mat_addsub(const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int sub, cudaStream_t s);
gbmm_status launch_limb_matmul(const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int accumulate,
                               cudaStream_t s);
gbmm_status launch_mat_zero(const gbmm_mat &c, cudaStream_t s);
gbmm_status launch_mat_copy(const gbmm_mat &dst, const gbmm_mat &src, cudaStream_t s);
gbmm_status launch_max_size(const gbmm_mat &a, int32_t *d_out, cudaStream_t s);

// ---- CRT path (crt.cu) --------------------------------------------------------------
struct crt_cache;
crt_cache *crt_cache_create();
void crt_cache_destroy(crt_cache *);
gbmm_status crt_matmul(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b,
                       int64_t bits_a, int64_t bits_b, int nprimes, int accumulate, cudaStream_t s);

// ---- device workspace arena -------------------------------------------------------------
// One growing allocation per handle, carved out stack-wise; freeing happens in
// LIFO order through arena_mark / arena_release.  Nothing is freed while work
// may still use it: growth synchronises the handle's stream first.
struct arena {
    char *base = nullptr;
    size_t cap = 0;
    size_t top = 0;
};

}  // namespace gbmm

struct gbmm_handle_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    gbmm::arena ws;
    gbmm::crt_cache *crt = nullptr;
    // tuning knobs (filled from defaults or the autotuner)
    int limb_cutoff = 32;
    // learned-dispatch model (null when not loaded)
    void *model = nullptr;
};

namespace gbmm {
gbmm_status arena_reserve(gbmm_handle h, size_t bytes);
void *arena_alloc(gbmm_handle h, size_t bytes);  // nullptr when the reservation is too small
static inline size_t arena_mark(gbmm_handle h) { return h->ws.top; }
static inline void arena_release(gbmm_handle h, size_t mark) { h->ws.top = mark; }
}  // namespace gbmm
