// Internal declarations shared by the gbmm translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <functional>
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

// ---- uploads that have landed when they return ---------------------------------
// A plain cudaMemcpy from pageable host memory may return before its DMA has
// completed, ordered only against the legacy default stream: a kernel launched
// right after on a non-blocking stream could read the old contents.  These copy
// (or fill) on a private per-device stream and wait for that stream.
gbmm_status upload_now(void *dst, const void *src, size_t bytes);
gbmm_status fill_now(void *dst, int value, size_t bytes);
cudaStream_t copy_stream();  // the private stream of the current device

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
gbmm_status launch_split_sizes(const gbmm_mat &x, int h, int32_t *lo, int32_t *hi, cudaStream_t s);
gbmm_status launch_add_shifted(const gbmm_mat &w, const gbmm_mat &u, const gbmm_mat &v, int sh, cudaStream_t s);
// whether the per-entry product kernel handles la x lb limb entries
bool limb_kernel_fits(int la, int lb);
// whether the batched basecase product stages un x vn limb operands on chip
bool mpn_basecase_on_chip(int un, int vn);

// Breadth-first Winograd recursion: the whole tree of one square product laid out
// in workspace arrays (see limb.cu).  Level d = 1..levels holds 4 * 7^(d-1) A-side
// and B-side sums and 7^d products, each a dense (N >> d)^2 matrix stored back to
// back (capSA / capSB / capP planes); level 0's output is C.
constexpr int WINO_MAX_LEVELS = 8;
struct WinoTree {
    gbmm_mat A, B, C;
    int N = 0, levels = 0;
    int capSA = 0, capSB = 0, capP = 0;
    uint32_t *sa_limbs[WINO_MAX_LEVELS + 1] = {}, *sb_limbs[WINO_MAX_LEVELS + 1] = {},
             *p_limbs[WINO_MAX_LEVELS + 1] = {};
    int32_t *sa_sizes[WINO_MAX_LEVELS + 1] = {}, *sb_sizes[WINO_MAX_LEVELS + 1] = {},
            *p_sizes[WINO_MAX_LEVELS + 1] = {};
};
// level d's sums from level d - 1's operands; all leaf products; level d's
// products combined into level d - 1's outputs
gbmm_status launch_wino_sums(const WinoTree &t, int d, cudaStream_t s);
gbmm_status launch_wino_leaves(const WinoTree &t, cudaStream_t s);
gbmm_status launch_wino_combine(const WinoTree &t, int d, cudaStream_t s);

// ---- CRT path (crt.cu) --------------------------------------------------------------
struct crt_cache;
crt_cache *crt_cache_create();
void crt_cache_destroy(crt_cache *);
gbmm_status crt_matmul(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b,
                       int64_t bits_a, int64_t bits_b, int nprimes, int accumulate, cudaStream_t s);
// whether the CRT kernels take la x lb limb entries with inner dimension k directly
bool crt_feasible(int la, int lb, int k);
// device workspace one crt_matmul call with these shapes carves from the arena
size_t crt_workspace_bytes(int la, int lb, int m, int k, int n, int cn);
// whether crt_matmul covers inner dimension k in one pass (no chunks of k)
bool crt_single_pass(int k);
// Grouped CRT launches (a batch's CRT products): products are collected without
// launching, each with its whole workspace carved from the arena at once, and
// then run stage by stage, one persistent launch per stage and kernel form over
// the tiles of all of them.  crt_group_add takes single-pass products only (k <=
// 512, no accumulation).
struct crt_group;
crt_group *crt_group_create();
void crt_group_destroy(crt_group *g);
bool crt_group_empty(const crt_group *g);
// An operand of a grouped product given as the two limb halves of x (a limb-half
// split), read in place: side 0, A = [x_lo; x_hi] stacked by rows; side 1, B =
// [x_lo | x_hi] stacked by columns; x_lo holds x's low hl limbs, x_hi the rest.
// The stacked operand passed to crt_group_add then only gives the shape.
struct crt_halves {
    int side;
    gbmm_mat x;
    int hl;
};
gbmm_status crt_group_add(gbmm_handle h, crt_group *g, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b,
                          int64_t bits_a, int64_t bits_b, int nprimes, const crt_halves *halves = nullptr);
// a step run after the reconstructions of the products added with halves (their
// shifted adds): on a second stream while the other reconstructions run
void crt_group_post(crt_group *g, std::function<gbmm_status(cudaStream_t)> f);
// arena bytes crt_group_add takes for one product of these shapes
size_t crt_group_ws(int la, int lb, int m, int k, int n);
// the stage records as one blob (built once every product is added); it goes to
// device memory 128-byte aligned, and crt_group_launch reads it there.  The post
// steps run on s2 (after `ev`, recorded on s) when s2 is given, else on s.
const std::vector<char> &crt_group_blob(crt_group *g);
gbmm_status crt_group_launch(crt_group *g, const char *d_blob, cudaStream_t s, cudaStream_t s2, cudaEvent_t ev);
// Stage hooks the host-buffer pipeline hands to one single-pass CRT product
// (gbmm_handle::stage, consumed and cleared by crt_matmul): B's digits and
// residues wait for b_ready, so A's run while B is still uploading; the
// reconstruction runs in `parts` entry ranges, each followed by part_ev[i], so
// finished ranges of C can go back to the host while the rest is computed.
constexpr int CRT_MAX_PARTS = 4;
struct crt_stage_hooks {
    cudaEvent_t b_ready = nullptr;
    int parts = 1;
    cudaEvent_t part_ev[CRT_MAX_PARTS] = {};
    int64_t part_end[CRT_MAX_PARTS] = {};  // entries of C finished after part i (exclusive end)
    int parts_done = 0;                    // parts recorded (0: none, C finishes with the stream)
};

// ---- persistent batched limb kernel (limb.cu) ---------------------------------------------
// Host-side plan of one batch of limb-path products: a blob holding the job
// descriptors and the (job, tile) work items of every block-edge group.
struct LimbBatchPlan {
    static constexpr int MAX_GROUPS = 10;  // launches per batch at most (block edge x CTA form x thin)
    std::vector<char> blob;
    struct Group {
        int R = 0;
        int NT = 0;    // threads per CTA
        int thin = 0;  // jobs with a one-limb-longer operand (edge threads fold in its top limb)
        size_t jobs_off = 0, items_off = 0;
        int nitems = 0;
        size_t smem = 0;
    };
    std::vector<Group> groups;
};
gbmm_status plan_limb_batch(const std::vector<gbmm_mat> &C, const std::vector<gbmm_mat> &A,
                            const std::vector<gbmm_mat> &B, LimbBatchPlan &plan);
// d_blob holds plan.blob on the device; d_counters has one int per group
gbmm_status launch_limb_batch(const LimbBatchPlan &plan, const char *d_blob, int *d_counters, cudaStream_t s);

// ---- dispatch (host.cpp, batch.cpp) ------------------------------------------------------
struct Plan {
    int path = GBMM_PATH_LIMB;  // GBMM_PATH_LIMB or GBMM_PATH_CRT after resolution
    int method = GBMM_METHOD_NAIVE;  // limb path square method
    int cutoff = 32;   // limb path recursion cutoff
    int nprimes = 0;   // CRT moduli (0 = from the bound)
    int tiles = 0;     // CRT GEMM tiles: 0 by size, 1 one-CTA (128 entries), 2 CTA pairs (256 entries)
    int split = 0;     // limb-half splits forced before the kernels (fewer moduli per CRT product)
    int id = -1;       // the gbmm_plan it stands for, -1 for options given field by field
};
// the gbmm_plan `id` as a Plan
Plan plan_of(int id);
// whether the autotuner times plan `id` for this product (and so whether the
// learned model may pick it): limb plans only below a schoolbook-work bound,
// Winograd cutoffs only when they give recursion, splits only of multi-limb operands
bool plan_admissible(int id, int m, int k, int n, int la, int lb);
int heuristic_plan(int m, int k, int n, int la, int lb);
// AUTO choice: learned model when loaded, tuning table, else the heuristic (a gbmm_plan)
int choose_plan(gbmm_handle h, int m, int k, int n, int la, int lb);
size_t dispatch_ws(const Plan &p, int la, int lb, int m, int k, int n, int cn, int accumulate);
gbmm_status dispatch(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, const Plan &p,
                     int accumulate, cudaStream_t s);
// whether a batch runs this job in the grouped CRT launches (a CRT plan, one pass
// over k, directly or after one limb-half split), the arena bytes it then takes,
// and its collection into the group (workspace carved, nothing launched)
bool crt_groupable(const Plan &p, int la, int lb, int m, int k, int n);
// Winograd's breadth-first tree with CRT leaf products (GBMM_METHOD_WINOGRAD_CRT):
// whether it takes this product, its workspace, and the product itself
bool wino_crt_ok(int la, int lb, int m, int k, int n, int cutoff);
size_t wino_crt_ws(int la, int lb, int N, int cn, int cutoff);
gbmm_status wino_crt(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int cutoff,
                     cudaStream_t s);
size_t crt_group_job_ws(const Plan &p, int la, int lb, int m, int k, int n);
gbmm_status crt_collect(gbmm_handle h, crt_group *g, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b,
                        const Plan &p);
gbmm_status resolve_plan(gbmm_handle h, const gbmm_mat &a, const gbmm_mat &b, const gbmm_opts &o, Plan &p);
void invalidate_graphs(gbmm_handle h);
void batch_state_destroy(gbmm_handle h);
// learned cost model (mlp.cu): the gbmm_plan it picks, or -1 when no model applies
int model_choose(gbmm_handle h, int m, int k, int n, int la, int lb);
void model_destroy(gbmm_handle h);

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
    // Winograd products as one breadth-first tree (1, default) or depth first (0)
    int wino_breadth_first = 1;
    // CRT GEMM tile form for the next product (set around each CRT call by dispatch):
    // 0 by size, 1 one-CTA tiles, 2 CTA-pair tiles for the product and reconstruction
    int crt_tiles = 0;
    // learned-dispatch model (null when not loaded) and whether AUTO consults it
    void *model = nullptr;
    int use_model = 0;
    // batched-execution state: tuning table, graph cache, staging (batch.cpp)
    void *batch = nullptr;
    // host-buffer pipeline: copy streams, two device slots (pipeline.cpp)
    void *pipe = nullptr;
    // device bytes a host-buffer product may use before it runs out of core (0: free memory)
    size_t dev_budget = 0;
    // stage hooks for the next CRT product (pipeline.cpp sets them, crt_matmul clears them)
    gbmm::crt_stage_hooks *stage = nullptr;
};

namespace gbmm {
gbmm_status arena_reserve(gbmm_handle h, size_t bytes);
void pipe_destroy(gbmm_handle h);
void *arena_alloc(gbmm_handle h, size_t bytes);  // nullptr when the reservation is too small
static inline size_t arena_mark(gbmm_handle h) { return h->ws.top; }
static inline void arena_release(gbmm_handle h, size_t mark) { h->ws.top = mark; }
}  // namespace gbmm
