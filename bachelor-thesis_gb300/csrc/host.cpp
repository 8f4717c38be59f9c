// Host side of gbmm: handle, errors, text / GMP-limb conversion, transfers and
// the matrix-recursion drivers (Winograd, Strassen, block recursion, squarify)
// that enqueue the device kernels.  Every entry point returns a status; no
// host synchronisation happens inside the recursion, so a whole product can
// be captured into a CUDA graph.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gbmm_internal.h"

namespace gbmm {

static thread_local std::string g_last_error;

gbmm_status set_error(gbmm_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

gbmm_status cuda_error(cudaError_t e, const char *what) {
    return set_error(e == cudaErrorMemoryAllocation ? GBMM_ERR_NOMEM : GBMM_ERR_CUDA, "%s: %s (%s)", what,
                     cudaGetErrorString(e), cudaGetErrorName(e));
}

// ---- launch accounting ---------------------------------------------------------------
static std::atomic<uint64_t> g_launches{0};
void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

struct ProfRecord {
    std::string name;
    cudaEvent_t start, stop;
};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<ProfRecord> g_prof;

LaunchScope::LaunchScope(const char *name, cudaStream_t s) : name_(name), s_(s), slot_(-1) {
    count_launch();
    if (!g_prof_on) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    ProfRecord r;
    r.name = name;
    if (cudaEventCreate(&r.start) != cudaSuccess) return;
    if (cudaEventCreate(&r.stop) != cudaSuccess) { cudaEventDestroy(r.start); return; }
    cudaEventRecord(r.start, s);
    slot_ = (int)g_prof.size();
    g_prof.push_back(r);
}
LaunchScope::~LaunchScope() {
    if (slot_ < 0) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEventRecord(g_prof[slot_].stop, s_);
}

// ---- per-device error word ----------------------------------------------------------
static std::mutex g_err_mu;
static uint32_t *g_err_words[64];

uint32_t *device_error_word() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (!g_err_words[dev]) {
        uint32_t *p = nullptr;
        if (cudaMalloc(&p, sizeof(uint32_t)) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, sizeof(uint32_t));
        cudaDeviceSynchronize();
        g_err_words[dev] = p;
    }
    return g_err_words[dev];
}

cudaStream_t copy_stream() {
    static std::mutex mu;
    static std::map<int, cudaStream_t> streams;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = streams.find(dev);
    if (it != streams.end()) return it->second;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    streams[dev] = s;
    return s;
}

gbmm_status upload_now(void *dst, const void *src, size_t bytes) {
    cudaStream_t s = copy_stream();
    if (!s) return set_error(GBMM_ERR_CUDA, "no copy stream");
    GBMM_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    GBMM_CUDA_TRY(cudaStreamSynchronize(s));
    return GBMM_OK;
}

gbmm_status fill_now(void *dst, int value, size_t bytes) {
    cudaStream_t s = copy_stream();
    if (!s) return set_error(GBMM_ERR_CUDA, "no copy stream");
    GBMM_CUDA_TRY(cudaMemsetAsync(dst, value, bytes, s));
    GBMM_CUDA_TRY(cudaStreamSynchronize(s));
    return GBMM_OK;
}

gbmm_status check_device_error(cudaStream_t s) {
    uint32_t *w = device_error_word();
    if (!w) return set_error(GBMM_ERR_CUDA, "device error word unavailable");
    uint32_t v = 0;
    GBMM_CUDA_TRY(cudaMemcpyAsync(&v, w, sizeof v, cudaMemcpyDeviceToHost, s));
    GBMM_CUDA_TRY(cudaStreamSynchronize(s));
    if (v) {
        GBMM_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(uint32_t), s));
        GBMM_CUDA_TRY(cudaStreamSynchronize(s));
        if (v & DEVERR_CAPACITY) return set_error(GBMM_ERR_CAPACITY, "a result needed more limb planes than its output has");
        if (v & DEVERR_TIMEOUT) return set_error(GBMM_ERR_TIMEOUT, "a bounded device-side wait expired");
        return set_error(GBMM_ERR_INVALID, "device kernel rejected its arguments (flags 0x%x)", v);
    }
    return GBMM_OK;
}

gbmm_status validate_mat(const gbmm_mat &m, const char *name) {
    if (m.rows < 0 || m.cols < 0) return set_error(GBMM_ERR_INVALID, "%s: negative shape", name);
    if ((int64_t)m.rows * m.cols == 0) return GBMM_OK;
    if (!m.limbs || !m.sizes) return set_error(GBMM_ERR_INVALID, "%s: null pointer", name);
    if (m.nlimbs < 0) return set_error(GBMM_ERR_INVALID, "%s: negative nlimbs", name);
    if (m.rs < m.cols) return set_error(GBMM_ERR_INVALID, "%s: row stride %lld < cols %d", name, (long long)m.rs, m.cols);
    if (m.nlimbs > 1 && m.ld < (int64_t)(m.rows - 1) * m.rs + m.cols)
        return set_error(GBMM_ERR_INVALID, "%s: plane stride %lld too small", name, (long long)m.ld);
    return GBMM_OK;
}

// ---- arena ------------------------------------------------------------------------------
gbmm_status arena_reserve(gbmm_handle h, size_t bytes) {
    if (h->ws.top + bytes <= h->ws.cap) return GBMM_OK;
    if (h->ws.top != 0) return set_error(GBMM_ERR_INVALID, "workspace grow while in use");
    size_t want = std::max(bytes, h->ws.cap * 2);
    want = (want + 0xFFFFF) & ~(size_t)0xFFFFF;
    GBMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
    invalidate_graphs(h);  // captured graphs point into the old block
    if (h->ws.base) GBMM_CUDA_TRY(cudaFree(h->ws.base));
    h->ws.base = nullptr;
    h->ws.cap = 0;
    void *p = nullptr;
    GBMM_CUDA_TRY(cudaMalloc(&p, want));
    h->ws.base = (char *)p;
    h->ws.cap = want;
    return GBMM_OK;
}

void *arena_alloc(gbmm_handle h, size_t bytes) {
    size_t top = (h->ws.top + 255) & ~(size_t)255;
    if (top + bytes > h->ws.cap) return nullptr;
    h->ws.top = top + bytes;
    return h->ws.base + top;
}

// A temporary matrix carved from the arena.
static bool arena_mat(gbmm_handle h, int rows, int cols, int nlimbs, gbmm_mat &m) {
    int64_t n = (int64_t)rows * cols;
    m.rows = rows; m.cols = cols; m.nlimbs = nlimbs; m.pad_ = 0;
    m.rs = cols; m.ld = n;
    m.limbs = (uint32_t *)arena_alloc(h, (size_t)n * nlimbs * 4 + 16);
    m.sizes = (int32_t *)arena_alloc(h, (size_t)n * 4 + 16);
    return m.limbs && m.sizes;
}
static size_t mat_bytes(int64_t n, int nlimbs) { return (size_t)n * nlimbs * 4 + (size_t)n * 4 + 2 * 256 + 32; }
static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace gbmm

using namespace gbmm;

// ======================================================================================
// handle / errors
// ======================================================================================
extern "C" const char *gbmm_last_error_string(void) { return g_last_error.c_str(); }
extern "C" const char *gbmm_version(void) { return "gbmm 0.1"; }
extern "C" uint64_t gbmm_kernel_launches(void) { return g_launches.load(); }

extern "C" gbmm_status gbmm_profile(int32_t enable) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto &r : g_prof) { cudaEventDestroy(r.start); cudaEventDestroy(r.stop); }
    g_prof.clear();
    g_prof_on = enable != 0;
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_profile_read(char *out, size_t cap, size_t *written) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    std::vector<std::pair<std::string, std::pair<int, double>>> agg;
    for (auto &r : g_prof) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.stop) != cudaSuccess) return set_error(GBMM_ERR_CUDA, "profile event sync");
        cudaEventElapsedTime(&ms, r.start, r.stop);
        bool found = false;
        for (auto &a : agg)
            if (a.first == r.name) { a.second.first++; a.second.second += ms; found = true; break; }
        if (!found) agg.push_back({r.name, {1, (double)ms}});
    }
    std::string js = "{";
    for (size_t i = 0; i < agg.size(); i++) {
        char buf[256];
        snprintf(buf, sizeof buf, "%s\"%s\": [%d, %.6f]", i ? ", " : "", agg[i].first.c_str(), agg[i].second.first,
                 agg[i].second.second);
        js += buf;
    }
    js += "}";
    if (written) *written = js.size();
    if (out && cap) {
        size_t n = std::min(cap - 1, js.size());
        memcpy(out, js.data(), n);
        out[n] = 0;
    }
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_create(gbmm_handle *out) {
    if (!out) return set_error(GBMM_ERR_INVALID, "null handle pointer");
    gbmm_handle h = new (std::nothrow) gbmm_handle_s();
    if (!h) return set_error(GBMM_ERR_NOMEM, "handle allocation");
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { delete h; return cuda_error(e, "cudaGetDevice"); }
    if (!device_error_word()) { delete h; return set_error(GBMM_ERR_CUDA, "cannot allocate the device error word"); }
    h->crt = crt_cache_create();
    *out = h;
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_destroy(gbmm_handle h) {
    if (!h) return GBMM_OK;
    cudaStreamSynchronize(h->stream);
    pipe_destroy(h);
    batch_state_destroy(h);
    model_destroy(h);
    if (h->ws.base) cudaFree(h->ws.base);
    crt_cache_destroy(h->crt);
    delete h;
    return GBMM_OK;
}

// Internal switch (not part of the public ABI): Winograd products through the
// breadth-first tree (1, default) or the depth-first recursion (0); returns the
// previous setting, or -1 for a null handle.
extern "C" int32_t gbmmx_wino_breadth_first(gbmm_handle h, int32_t enable) {
    if (!h) return -1;
    const int32_t old = h->wino_breadth_first;
    h->wino_breadth_first = enable != 0;
    return old;
}

extern "C" gbmm_status gbmm_set_stream(gbmm_handle h, void *stream) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    h->stream = as_stream(stream);
    return GBMM_OK;
}

// ======================================================================================
// text <-> limb planes
// ======================================================================================
// value of a hexadecimal digit, -1 for any other byte
struct HexTable {
    int8_t v[256];
    constexpr HexTable() : v() {
        for (int c = 0; c < 256; c++)
            v[c] = (int8_t)(c >= '0' && c <= '9' ? c - '0'
                            : c >= 'a' && c <= 'f' ? c - 'a' + 10
                            : c >= 'A' && c <= 'F' ? c - 'A' + 10
                                                   : -1);
    }
};
static constexpr HexTable HEXV{};
static inline int hexval(unsigned char c) { return HEXV.v[c]; }
static inline bool is_ws(unsigned char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// ---- host-side parallelism for the text and GMP conversions -----------------------------
// Large inputs are cut into chunks that threads handle independently; errors are
// reported for the first offending entry in input order, exactly as the serial path
// does (the serial path is the same code on one chunk).
static std::atomic<int> g_host_threads{0};  // 0: the hardware's thread count
static int host_threads() {
    static const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    const int n = g_host_threads.load(std::memory_order_relaxed);
    return n > 0 ? n : hw;
}
template <typename F>
static void run_chunks(int nchunks, F f) {
    std::vector<std::thread> th;
    th.reserve(nchunks > 0 ? nchunks - 1 : 0);
    for (int c = 1; c < nchunks; c++) th.emplace_back(f, c);
    if (nchunks > 0) f(0);
    for (auto &t : th) t.join();
}
static constexpr size_t PAR_TEXT_BYTES = 1u << 20;   // text per thread before parsing splits
static constexpr int64_t PAR_ENTRIES = 1 << 14;       // entries per thread before loops split

// One token "[-]hexdigits" at text[p] (p on a non-space byte) into entry e.
static gbmm_status parse_one(const char *text, size_t len, size_t &p, int64_t e, uint32_t *limbs, int32_t *sizes,
                             int32_t nlimbs, int64_t ld, char *msg, size_t msgcap) {
    bool neg = false;
    if (p < len && text[p] == '-') { neg = true; p++; }
    size_t s = p;
    while (p < len && hexval((unsigned char)text[p]) >= 0) p++;
    size_t nd = p - s;
    if (nd == 0) {
        snprintf(msg, msgcap, "entry %lld: expected a hexadecimal digit at byte %zu", (long long)e, p);
        return GBMM_ERR_PARSE;
    }
    if (p < len && !is_ws((unsigned char)text[p])) {
        snprintf(msg, msgcap, "entry %lld: invalid character '%c' at byte %zu", (long long)e, text[p], p);
        return GBMM_ERR_PARSE;
    }
    while (nd > 1 && text[s] == '0') { s++; nd--; }  // leading zeros
    int need = (int)((nd + 7) / 8);
    if (nd == 1 && text[s] == '0') need = 0;
    if (need > nlimbs) {
        snprintf(msg, msgcap, "entry %lld needs %d limbs, capacity %d", (long long)e, need, nlimbs);
        return GBMM_ERR_CAPACITY;
    }
    // limb i holds digits [nd - 8(i+1), nd - 8i) of the token, built in a register
    // and stored once; the top limb has the first (nonzero) digit, so it is nonzero
    const unsigned char *d = reinterpret_cast<const unsigned char *>(text + s);
    for (int i = 0; i < need; i++) {
        const size_t hi = nd - 8 * (size_t)i, lo = hi >= 8 ? hi - 8 : 0;
        uint32_t v = 0;
        for (size_t q = lo; q < hi; q++) v = (v << 4) | (uint32_t)HEXV.v[d[q]];
        limbs[(int64_t)i * ld + e] = v;
    }
    for (int i = need; i < nlimbs; i++) limbs[(int64_t)i * ld + e] = 0u;
    sizes[e] = neg ? -need : need;
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_parse_hex(const char *text, size_t len, int64_t count, uint32_t *limbs, int32_t *sizes,
                                      int32_t nlimbs, int64_t ld, size_t *consumed) {
    if ((!text && len) || (count > 0 && (!limbs || !sizes))) return set_error(GBMM_ERR_INVALID, "null pointer");
    if (count > 0 && nlimbs > 0 && ld < count) return set_error(GBMM_ERR_INVALID, "plane stride %lld < count", (long long)ld);
    char msg[256];
    const int T = (int)std::min<size_t>((size_t)host_threads(), len / PAR_TEXT_BYTES);
    if (T < 2 || count < 2 * T) {
        size_t p = 0;
        for (int64_t e = 0; e < count; e++) {
            while (p < len && is_ws((unsigned char)text[p])) p++;
            gbmm_status st = parse_one(text, len, p, e, limbs, sizes, nlimbs, ld, msg, sizeof msg);
            if (st != GBMM_OK) {
                if (consumed) *consumed = p;
                return set_error(st, "%s", msg);
            }
        }
        if (consumed) *consumed = p;
        return GBMM_OK;
    }
    // chunk boundaries on whitespace, so no token straddles two chunks
    std::vector<size_t> bnd(T + 1);
    bnd[0] = 0;
    bnd[T] = len;
    for (int t = 1; t < T; t++) {
        size_t q = std::max(bnd[t - 1], len / T * t);
        while (q < len && !is_ws((unsigned char)text[q])) q++;
        bnd[t] = q;
    }
    std::vector<int64_t> ntok(T, 0), first(T + 1, 0);
    run_chunks(T, [&](int t) {
        int64_t n = 0;
        bool in = false;
        for (size_t q = bnd[t]; q < bnd[t + 1]; q++) {
            const bool w = is_ws((unsigned char)text[q]);
            if (!w && !in) n++;
            in = !w;
        }
        ntok[t] = n;
    });
    for (int t = 0; t < T; t++) first[t + 1] = first[t] + ntok[t];
    struct ChunkResult {
        gbmm_status st = GBMM_OK;
        int64_t e = -1;
        size_t pos = 0, end = 0;
        char msg[256];
    };
    std::vector<ChunkResult> res(T);
    run_chunks(T, [&](int t) {
        ChunkResult &r = res[t];
        size_t p = bnd[t];
        for (int64_t e = first[t]; e < first[t + 1] && e < count; e++) {
            while (p < bnd[t + 1] && is_ws((unsigned char)text[p])) p++;
            gbmm_status st = parse_one(text, len, p, e, limbs, sizes, nlimbs, ld, r.msg, sizeof r.msg);
            if (st != GBMM_OK) {
                r.st = st;
                r.e = e;
                r.pos = p;
                return;
            }
            if (e == count - 1) r.end = p;
        }
    });
    for (int t = 0; t < T; t++)
        if (res[t].st != GBMM_OK) {
            if (consumed) *consumed = res[t].pos;
            return set_error(res[t].st, "%s", res[t].msg);
        }
    if (first[T] < count) {
        if (consumed) *consumed = len;
        return set_error(GBMM_ERR_PARSE, "entry %lld: expected a hexadecimal digit at byte %zu", (long long)first[T], len);
    }
    if (consumed)
        for (int t = 0; t < T; t++)
            if (count - 1 >= first[t] && count - 1 < first[t + 1]) *consumed = res[t].end;
    return GBMM_OK;
}

static const char HEXDIG[] = "0123456789abcdef";

// characters of entry e in the text form ("0", or [-] and hex digits without leading zeros); -1: bad size
static int64_t hex_len(const uint32_t *limbs, const int32_t *sizes, int32_t nlimbs, int64_t ld, int64_t e) {
    int s = sizes[e], n = s < 0 ? -s : s;
    if (n > nlimbs) return -1;
    while (n > 0 && limbs[(int64_t)(n - 1) * ld + e] == 0) n--;
    if (n == 0) return 1;
    uint32_t top = limbs[(int64_t)(n - 1) * ld + e];
    int d = 8;
    while (d > 1 && (top >> (4 * (d - 1))) == 0) d--;
    return (s < 0 ? 1 : 0) + 8 * (int64_t)(n - 1) + d;
}
static char *hex_put(const uint32_t *limbs, const int32_t *sizes, int64_t ld, int64_t e, char *o) {
    int s = sizes[e], n = s < 0 ? -s : s;
    while (n > 0 && limbs[(int64_t)(n - 1) * ld + e] == 0) n--;
    if (n == 0) { *o++ = '0'; return o; }
    if (s < 0) *o++ = '-';
    bool started = false;
    for (int i = n - 1; i >= 0; i--) {
        uint32_t v = limbs[(int64_t)i * ld + e];
        for (int k = 7; k >= 0; k--) {
            int d = (v >> (4 * k)) & 15;
            if (d || started) { *o++ = HEXDIG[d]; started = true; }
        }
    }
    return o;
}

extern "C" gbmm_status gbmm_format_hex(const uint32_t *limbs, const int32_t *sizes, int32_t nlimbs, int64_t ld,
                                       int32_t rows, int32_t cols, int64_t rs, char *out, size_t cap, size_t *written) {
    if (!sizes || (nlimbs > 0 && !limbs)) return set_error(GBMM_ERR_INVALID, "null pointer");
    // row lengths (entries, separators, newline), in parallel over rows
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>(host_threads(), (int64_t)rows * cols / PAR_ENTRIES));
    std::vector<int64_t> rowlen(rows + 1, 0);
    std::vector<int64_t> bad(T, -1);
    run_chunks(T, [&](int t) {
        for (int32_t r = (int32_t)((int64_t)rows * t / T); r < (int32_t)((int64_t)rows * (t + 1) / T); r++) {
            int64_t L = 1 + (cols > 0 ? cols - 1 : 0);
            for (int32_t c = 0; c < cols; c++) {
                int64_t l = hex_len(limbs, sizes, nlimbs, ld, (int64_t)r * rs + c);
                if (l < 0) {
                    if (bad[t] < 0) bad[t] = (int64_t)r * cols + c;
                    l = 0;
                }
                L += l;
            }
            rowlen[r + 1] = L;
        }
    });
    for (int t = 0; t < T; t++)
        if (bad[t] >= 0) {
            const int32_t r = (int32_t)(bad[t] / cols), c = (int32_t)(bad[t] % cols);
            return set_error(GBMM_ERR_INVALID, "entry (%d,%d): size %d exceeds %d planes", r, c, sizes[(int64_t)r * rs + c],
                             nlimbs);
        }
    for (int32_t r = 0; r < rows; r++) rowlen[r + 1] += rowlen[r];  // row offsets
    const size_t w = (size_t)rowlen[rows] + 1;                          // final empty line
    if (written) *written = w;
    if (!out) return GBMM_OK;
    if (w > cap) return set_error(GBMM_ERR_INVALID, "output buffer too small (%zu < %zu)", cap, w);
    run_chunks(T, [&](int t) {
        for (int32_t r = (int32_t)((int64_t)rows * t / T); r < (int32_t)((int64_t)rows * (t + 1) / T); r++) {
            char *o = out + rowlen[r];
            for (int32_t c = 0; c < cols; c++) {
                if (c) *o++ = ' ';
                o = hex_put(limbs, sizes, ld, (int64_t)r * rs + c, o);
            }
            *o++ = '\n';
        }
    });
    out[w - 1] = '\n';
    if (w < cap) out[w] = 0;
    return GBMM_OK;
}

// Internal test hook (not part of the public ABI): threads for the host-side
// conversions, 0 = hardware default; returns the previous setting.
extern "C" int32_t gbmmx_host_threads(int32_t n) { return g_host_threads.exchange(n < 0 ? 0 : n); }

extern "C" gbmm_status gbmm_import_gmp(int64_t count, const uint64_t *limbs64, const int64_t *offsets,
                                       const int32_t *sizes64, uint32_t *limbs, int32_t *sizes, int32_t nlimbs,
                                       int64_t ld) {
    if (count > 0 && (!limbs64 || !offsets || !sizes64 || !limbs || !sizes))
        return set_error(GBMM_ERR_INVALID, "null pointer");
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>(host_threads(), count / PAR_ENTRIES));
    std::vector<int64_t> bad(T, -1);
    std::vector<int> badn(T, 0);
    run_chunks(T, [&](int t) {
        for (int64_t e = count * t / T; e < count * (t + 1) / T; e++) {
            int s = sizes64[e], n64 = s < 0 ? -s : s;
            const uint64_t *d = limbs64 + offsets[e];
            int n = 2 * n64;
            while (n > 0 && (uint32_t)(d[(n - 1) / 2] >> (32 * ((n - 1) % 2))) == 0) n--;
            if (n > nlimbs) {
                bad[t] = e;
                badn[t] = n;
                return;
            }
            for (int i = 0; i < nlimbs; i++) limbs[(int64_t)i * ld + e] = i < n ? (uint32_t)(d[i / 2] >> (32 * (i % 2))) : 0u;
            sizes[e] = s < 0 ? -n : n;
        }
    });
    for (int t = 0; t < T; t++)
        if (bad[t] >= 0)
            return set_error(GBMM_ERR_CAPACITY, "entry %lld needs %d limbs, capacity %d", (long long)bad[t], badn[t], nlimbs);
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_export_gmp(int64_t count, const uint32_t *limbs, const int32_t *sizes, int32_t nlimbs,
                                       int64_t ld, uint64_t *limbs64, const int64_t *offsets, int32_t *sizes64) {
    if (count > 0 && (!limbs64 || !offsets || !sizes64 || !limbs || !sizes))
        return set_error(GBMM_ERR_INVALID, "null pointer");
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>(host_threads(), count / PAR_ENTRIES));
    std::vector<int64_t> bad(T, -1);
    run_chunks(T, [&](int t) {
        for (int64_t e = count * t / T; e < count * (t + 1) / T; e++) {
            int s = sizes[e], n = s < 0 ? -s : s;
            if (n > nlimbs) {
                bad[t] = e;
                return;
            }
            int n64 = (n + 1) / 2;
            uint64_t *d = limbs64 + offsets[e];
            for (int i = 0; i < n64; i++) {
                uint64_t lo = limbs[(int64_t)(2 * i) * ld + e];
                uint64_t hi = 2 * i + 1 < n ? limbs[(int64_t)(2 * i + 1) * ld + e] : 0u;
                d[i] = lo | (hi << 32);
            }
            sizes64[e] = s < 0 ? -n64 : n64;
        }
    });
    for (int t = 0; t < T; t++)
        if (bad[t] >= 0) return set_error(GBMM_ERR_INVALID, "entry %lld: size exceeds planes", (long long)bad[t]);
    return GBMM_OK;
}

// ======================================================================================
// transfers
// ======================================================================================
static gbmm_status copy_planes(gbmm_mat m, uint32_t *hl, int32_t *hs, int32_t hn, int64_t hld, bool up, cudaStream_t s) {
    GBMM_TRY(validate_mat(m, "matrix"));
    if ((int64_t)m.rows * m.cols == 0) return GBMM_OK;
    if (!hl || !hs) return set_error(GBMM_ERR_INVALID, "null host pointer");
    if (hld < (int64_t)m.rows * m.cols) return set_error(GBMM_ERR_INVALID, "host plane stride too small");
    const cudaMemcpyKind kind = up ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    const int64_t E = (int64_t)m.rows * m.cols;
    if (m.rs == m.cols && m.ld == E && hld == E) {
        // dense planes on both sides: one copy for the sizes and one for all shared planes
        const int np = std::min(hn, m.nlimbs);
        GBMM_CUDA_TRY(cudaMemcpyAsync(up ? (void *)m.sizes : (void *)hs, up ? (const void *)hs : (const void *)m.sizes,
                                      (size_t)E * 4, kind, s));
        if (np > 0)
            GBMM_CUDA_TRY(cudaMemcpyAsync(up ? (void *)m.limbs : (void *)hl, up ? (const void *)hl : (const void *)m.limbs,
                                          (size_t)np * E * 4, kind, s));
        if (up && m.nlimbs > np)
            GBMM_CUDA_TRY(cudaMemsetAsync(m.limbs + (int64_t)np * E, 0, (size_t)(m.nlimbs - np) * E * 4, s));
        if (!up && hn > np) memset(hl + (int64_t)np * hld, 0, (size_t)(hn - np) * E * 4);
        GBMM_CUDA_TRY(cudaStreamSynchronize(s));
        return GBMM_OK;
    }
    // sizes: rows with stride rs on the device, contiguous on the host
    GBMM_CUDA_TRY(cudaMemcpy2DAsync(up ? (void *)m.sizes : (void *)hs, (up ? m.rs : m.cols) * 4,
                                    up ? (const void *)hs : (const void *)m.sizes, (up ? m.cols : m.rs) * 4,
                                    (size_t)m.cols * 4, m.rows, kind, s));
    for (int i = 0; i < m.nlimbs; i++) {
        uint32_t *dp = m.limbs + (int64_t)i * m.ld;
        if (i < hn) {
            uint32_t *hp = hl + (int64_t)i * hld;
            GBMM_CUDA_TRY(cudaMemcpy2DAsync(up ? (void *)dp : (void *)hp, (up ? m.rs : m.cols) * 4,
                                            up ? (const void *)hp : (const void *)dp, (up ? m.cols : m.rs) * 4,
                                            (size_t)m.cols * 4, m.rows, kind, s));
        } else if (up) {
            GBMM_CUDA_TRY(cudaMemset2DAsync(dp, m.rs * 4, 0, (size_t)m.cols * 4, m.rows, s));
        }
    }
    if (!up) {
        // host planes beyond the device capacity are zero
        for (int i = m.nlimbs; i < hn; i++) memset(hl + (int64_t)i * hld, 0, (size_t)m.rows * m.cols * 4);
    }
    GBMM_CUDA_TRY(cudaStreamSynchronize(s));
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_upload(gbmm_mat dst, const uint32_t *host_limbs, const int32_t *host_sizes,
                                   int32_t host_nlimbs, int64_t host_ld, void *stream) {
    if (host_nlimbs > dst.nlimbs) {
        // higher host planes must be empty: check sizes
        for (int64_t e = 0; e < (int64_t)dst.rows * dst.cols; e++) {
            int s = host_sizes[e];
            if ((s < 0 ? -s : s) > dst.nlimbs)
                return set_error(GBMM_ERR_CAPACITY, "entry %lld needs %d limbs, device capacity %d", (long long)e, s < 0 ? -s : s,
                                 dst.nlimbs);
        }
    }
    return copy_planes(dst, const_cast<uint32_t *>(host_limbs), const_cast<int32_t *>(host_sizes), host_nlimbs, host_ld,
                       true, as_stream(stream));
}

extern "C" gbmm_status gbmm_download(gbmm_mat src, uint32_t *host_limbs, int32_t *host_sizes, int32_t host_nlimbs,
                                     int64_t host_ld, void *stream) {
    GBMM_TRY(copy_planes(src, host_limbs, host_sizes, host_nlimbs, host_ld, false, as_stream(stream)));
    for (int64_t e = 0; e < (int64_t)src.rows * src.cols; e++) {
        int s = host_sizes[e];
        if ((s < 0 ? -s : s) > host_nlimbs)
            return set_error(GBMM_ERR_CAPACITY, "entry %lld has %d limbs, host capacity %d", (long long)e, s, host_nlimbs);
    }
    return check_device_error(as_stream(stream));
}

extern "C" gbmm_status gbmm_import_hex(gbmm_mat dst, const char *text, size_t len, size_t *consumed, void *stream) {
    GBMM_TRY(validate_mat(dst, "dst"));
    int64_t n = (int64_t)dst.rows * dst.cols;
    std::vector<uint32_t> hl((size_t)n * std::max(dst.nlimbs, 1));
    std::vector<int32_t> hs((size_t)n);
    GBMM_TRY(gbmm_parse_hex(text, len, n, hl.data(), hs.data(), dst.nlimbs, n, consumed));
    return gbmm_upload(dst, hl.data(), hs.data(), dst.nlimbs, n, stream);
}

extern "C" gbmm_status gbmm_export_hex(gbmm_mat src, char *out, size_t cap, size_t *written, void *stream) {
    GBMM_TRY(validate_mat(src, "src"));
    int64_t n = (int64_t)src.rows * src.cols;
    std::vector<uint32_t> hl((size_t)n * std::max(src.nlimbs, 1));
    std::vector<int32_t> hs((size_t)n);
    GBMM_TRY(gbmm_download(src, hl.data(), hs.data(), src.nlimbs, n, stream));
    return gbmm_format_hex(hl.data(), hs.data(), src.nlimbs, n, src.rows, src.cols, src.cols, out, cap, written);
}

extern "C" gbmm_status gbmm_max_bits(gbmm_mat a, int64_t *bits, void *stream) {
    GBMM_TRY(validate_mat(a, "a"));
    if (!bits) return set_error(GBMM_ERR_INVALID, "null pointer");
    cudaStream_t s = as_stream(stream);
    int64_t n = (int64_t)a.rows * a.cols;
    if (n == 0 || a.nlimbs == 0) { *bits = 0; return GBMM_OK; }
    int32_t *d = nullptr;
    GBMM_CUDA_TRY(cudaMallocAsync(&d, sizeof(int32_t), s));
    gbmm_status st = launch_max_size(a, d, s);
    int32_t mx = 0;
    if (st == GBMM_OK) {
        cudaError_t e = cudaMemcpyAsync(&mx, d, sizeof mx, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_error(e, "max_bits readback");
    }
    cudaFreeAsync(d, s);
    *bits = (int64_t)mx * 32;
    return st;
}

// ======================================================================================
// matrix add / sub
// ======================================================================================
static gbmm_status check_same_shape(const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b) {
    GBMM_TRY(validate_mat(c, "C"));
    GBMM_TRY(validate_mat(a, "A"));
    GBMM_TRY(validate_mat(b, "B"));
    if (a.rows != c.rows || b.rows != c.rows || a.cols != c.cols || b.cols != c.cols)
        return set_error(GBMM_ERR_INVALID, "shapes differ");
    return GBMM_OK;
}
extern "C" gbmm_status gbmm_mat_add(gbmm_mat c, gbmm_mat a, gbmm_mat b, void *stream) {
    GBMM_TRY(check_same_shape(c, a, b));
    return launch_mat_addsub(c, a, b, 0, as_stream(stream));
}
extern "C" gbmm_status gbmm_mat_sub(gbmm_mat c, gbmm_mat a, gbmm_mat b, void *stream) {
    GBMM_TRY(check_same_shape(c, a, b));
    return launch_mat_addsub(c, a, b, 1, as_stream(stream));
}

extern "C" gbmm_status gbmm_mat_mul_naive(gbmm_mat c, gbmm_mat a, gbmm_mat b, int32_t accumulate, void *stream) {
    GBMM_TRY(validate_mat(c, "C"));
    GBMM_TRY(validate_mat(a, "A"));
    GBMM_TRY(validate_mat(b, "B"));
    if (a.rows != c.rows || b.cols != c.cols || a.cols != b.rows) return set_error(GBMM_ERR_INVALID, "shape mismatch");
    if (c.limbs == a.limbs || c.limbs == b.limbs) return set_error(GBMM_ERR_INVALID, "C must not alias A or B");
    return launch_limb_matmul(c, a, b, accumulate, as_stream(stream));
}

// ======================================================================================
// recursion drivers (limb path)
// ======================================================================================
namespace {

struct RecCtx {
    gbmm_handle h;
    cudaStream_t s;
    int cutoff;
    int capSA, capSB;  // capacities of A-side and B-side sums
    int capP;          // capacity of products / C quadrants
    bool breadth_first;  // Winograd products through the breadth-first tree when it fits
};

static unsigned ilog2u(unsigned n) { unsigned r = 0; while (n >>= 1) r++; return r; }
static unsigned remove_factors(unsigned n, unsigned b) { while (n && n % b == 0) n /= b; return n; }

static gbmm_mat with_limbs(gbmm_mat m, int nl) { m.nlimbs = nl; return m; }

gbmm_status rec_square(RecCtx &c, int method, gbmm_mat C, gbmm_mat A, gbmm_mat B, int N, int levels, int addmul);

// Winograd's 7-product scheme with 3 temporaries; the operation order is that
// of the reference (WINOGRAD_SEQUENCE / WINOGRAD_ADDMUL_SEQUENCE,
// mat-gpu/mat-defines.h:144-187; mat-cpu/mat.c:193-334).  p1 holds A-side
// sums, p2 B-side sums, p3 products; operand views are narrowed to the
// capacity of what they hold so the leaf kernel does no padded work.
gbmm_status rec_winograd(RecCtx &c, gbmm_mat C, gbmm_mat A, gbmm_mat B, int N, int levels, int addmul) {
    const int h = N / 2;
    size_t mark = arena_mark(c.h);
    const int capT = std::max(std::max(c.capSA, c.capSB), c.capP);
    gbmm_mat T1, T2, T3;
    if (!arena_mat(c.h, h, h, capT, T1) || !arena_mat(c.h, h, h, capT, T2) || !arena_mat(c.h, h, h, capT, T3))
        return set_error(GBMM_ERR_NOMEM, "winograd temporaries exceed the reserved workspace");
    gbmm_mat a11 = sub_view(A, 0, 0, h, h), a12 = sub_view(A, 0, h, h, h), a21 = sub_view(A, h, 0, h, h),
             a22 = sub_view(A, h, h, h, h);
    gbmm_mat b11 = sub_view(B, 0, 0, h, h), b12 = sub_view(B, 0, h, h, h), b21 = sub_view(B, h, 0, h, h),
             b22 = sub_view(B, h, h, h, h);
    gbmm_mat c11 = sub_view(C, 0, 0, h, h), c12 = sub_view(C, 0, h, h, h), c21 = sub_view(C, h, 0, h, h),
             c22 = sub_view(C, h, h, h, h);
    gbmm_mat p1 = with_limbs(T1, c.capSA), p2 = with_limbs(T2, c.capSB), p3 = with_limbs(T3, c.capP);
#define ADD(x, y, z) GBMM_TRY(launch_mat_addsub(x, y, z, 0, c.s))
#define SUB(x, y, z) GBMM_TRY(launch_mat_addsub(x, y, z, 1, c.s))
#define MUL(x, y, z) GBMM_TRY(rec_square(c, GBMM_METHOD_WINOGRAD, x, y, z, h, levels - 1, 0))
#define AML(x, y, z) GBMM_TRY(rec_square(c, GBMM_METHOD_WINOGRAD, x, y, z, h, levels - 1, 1))
    if (!addmul) {
        ADD(p1, a21, a22);
        SUB(p2, b12, b11);
        MUL(c22, p1, p2);
        SUB(p1, p1, a11);
        SUB(p2, b22, p2);
        MUL(p3, a11, b11);
        MUL(c11, a12, b21);
        ADD(c11, c11, p3);
        AML(p3, p1, p2);
        SUB(p1, a12, p1);
        SUB(p2, b21, p2);
        MUL(c12, p1, b22);
        ADD(c12, c12, c22);
        ADD(c12, c12, p3);
        MUL(c21, a22, p2);
        SUB(p1, a11, a21);
        SUB(p2, b22, b12);
        AML(p3, p1, p2);
        ADD(c21, c21, p3);
        ADD(c22, c22, p3);
    } else {
        ADD(p1, a21, a22);
        SUB(p2, b12, b11);
        MUL(p3, p1, p2);
        ADD(c12, c12, p3);
        ADD(c22, c22, p3);
        SUB(p1, p1, a11);
        SUB(p2, b22, p2);
        MUL(p3, a11, b11);
        ADD(c11, c11, p3);
        AML(p3, p1, p2);
        AML(c11, a12, b21);
        SUB(p1, a12, p1);
        SUB(p2, b21, p2);
        AML(c12, p1, b22);
        ADD(c12, c12, p3);
        AML(c21, a22, p2);
        SUB(p1, a11, a21);
        SUB(p2, b22, b12);
        AML(p3, p1, p2);
        ADD(c21, c21, p3);
        ADD(c22, c22, p3);
    }
#undef MUL
#undef AML
    arena_release(c.h, mark);
    return GBMM_OK;
}

// Strassen's scheme with 3 temporaries (mat-gpu/mat-defines.h:78-117,
// mat-cpu/mat.c:103-191).  Here p1 holds A sums, B sums and products in turn,
// so each use gets a view with the matching capacity.
gbmm_status rec_strassen(RecCtx &c, gbmm_mat C, gbmm_mat A, gbmm_mat B, int N, int levels) {
    const int h = N / 2;
    size_t mark = arena_mark(c.h);
    const int capT = std::max(std::max(c.capSA, c.capSB), c.capP);
    gbmm_mat T1, T2, T3;
    if (!arena_mat(c.h, h, h, capT, T1) || !arena_mat(c.h, h, h, capT, T2) || !arena_mat(c.h, h, h, capT, T3))
        return set_error(GBMM_ERR_NOMEM, "strassen temporaries exceed the reserved workspace");
    gbmm_mat a11 = sub_view(A, 0, 0, h, h), a12 = sub_view(A, 0, h, h, h), a21 = sub_view(A, h, 0, h, h),
             a22 = sub_view(A, h, h, h, h);
    gbmm_mat b11 = sub_view(B, 0, 0, h, h), b12 = sub_view(B, 0, h, h, h), b21 = sub_view(B, h, 0, h, h),
             b22 = sub_view(B, h, h, h, h);
    gbmm_mat c11 = sub_view(C, 0, 0, h, h), c12 = sub_view(C, 0, h, h, h), c21 = sub_view(C, h, 0, h, h),
             c22 = sub_view(C, h, h, h, h);
    gbmm_mat p1A = with_limbs(T1, c.capSA), p1B = with_limbs(T1, c.capSB), p1P = with_limbs(T1, c.capP);
    gbmm_mat p2A = with_limbs(T2, c.capSA), p2B = with_limbs(T2, c.capSB);
    gbmm_mat p3B = with_limbs(T3, c.capSB);
#define MUL(x, y, z) GBMM_TRY(rec_square(c, GBMM_METHOD_STRASSEN, x, y, z, h, levels - 1, 0))
    ADD(p1A, a11, a22);
    ADD(p2B, b11, b22);
    MUL(c11, p1A, p2B);
    SUB(p1B, b12, b22);
    MUL(c12, a11, p1B);
    ADD(c22, c11, c12);
    ADD(p1A, a21, a22);
    MUL(c21, p1A, b11);
    SUB(c22, c22, c21);
    SUB(p2A, a12, a22);
    ADD(p3B, b21, b22);
    MUL(p1P, p2A, p3B);
    ADD(c11, c11, p1P);
    SUB(p2A, a21, a11);
    ADD(p3B, b11, b12);
    MUL(p1P, p2A, p3B);
    ADD(c22, c22, p1P);
    SUB(p2B, b21, b11);
    MUL(p1P, a22, p2B);
    ADD(c11, c11, p1P);
    ADD(c21, c21, p1P);
    ADD(p2A, a11, a12);
    MUL(p1P, p2A, b22);
    SUB(c11, c11, p1P);
    ADD(c12, c12, p1P);
#undef MUL
    arena_release(c.h, mark);
    return GBMM_OK;
}

// Plain 8-product block recursion with one temporary (NAIVE_RECURSIVE_SEQUENCE,
// mat-gpu/mat-defines.h:21-36).
gbmm_status rec_naive(RecCtx &c, gbmm_mat C, gbmm_mat A, gbmm_mat B, int N, int levels) {
    const int h = N / 2;
    size_t mark = arena_mark(c.h);
    gbmm_mat T;
    if (!arena_mat(c.h, h, h, c.capP, T)) return set_error(GBMM_ERR_NOMEM, "workspace");
    gbmm_mat a11 = sub_view(A, 0, 0, h, h), a12 = sub_view(A, 0, h, h, h), a21 = sub_view(A, h, 0, h, h),
             a22 = sub_view(A, h, h, h, h);
    gbmm_mat b11 = sub_view(B, 0, 0, h, h), b12 = sub_view(B, 0, h, h, h), b21 = sub_view(B, h, 0, h, h),
             b22 = sub_view(B, h, h, h, h);
    gbmm_mat c11 = sub_view(C, 0, 0, h, h), c12 = sub_view(C, 0, h, h, h), c21 = sub_view(C, h, 0, h, h),
             c22 = sub_view(C, h, h, h, h);
#define MUL(x, y, z) GBMM_TRY(rec_square(c, GBMM_METHOD_NAIVE_REC, x, y, z, h, levels - 1, 0))
    MUL(c11, a11, b11); MUL(T, a12, b21); ADD(c11, c11, T);
    MUL(c12, a11, b12); MUL(T, a12, b22); ADD(c12, c12, T);
    MUL(c21, a21, b11); MUL(T, a22, b21); ADD(c21, c21, T);
    MUL(c22, a21, b12); MUL(T, a22, b22); ADD(c22, c22, T);
#undef MUL
    arena_release(c.h, mark);
    return GBMM_OK;
}

// Workspace of the breadth-first Winograd tree (sums and products of every level).
static size_t wino_bf_ws(int N, int levels, int capSA, int capSB, int capP) {
    size_t total = 0;
    int64_t np = 1;  // parents at level d - 1
    for (int d = 1; d <= levels; d++) {
        const int64_t h = N >> d, e = h * h;
        total += align_up((size_t)(4 * np * e) * capSA * 4, 256) + align_up((size_t)(4 * np * e) * 4, 256);
        total += align_up((size_t)(4 * np * e) * capSB * 4, 256) + align_up((size_t)(4 * np * e) * 4, 256);
        total += align_up((size_t)(7 * np * e) * capP * 4, 256) + align_up((size_t)(7 * np * e) * 4, 256);
        np *= 7;
    }
    return total + 6 * 256 * (size_t)levels;
}

// The breadth-first tree is used for a top-level Winograd product (not C += A*B)
// whose workspace stays below a fixed share of the device: 7^levels leaf products
// need (7/4)^levels times the product's own planes.
static constexpr size_t WINO_BF_MAX_BYTES = (size_t)24 << 30;
static bool wino_bf_ok(int method, int N, int levels, int addmul, int capSA, int capSB, int capP) {
    if (method != GBMM_METHOD_WINOGRAD || addmul || levels < 1 || levels > WINO_MAX_LEVELS) return false;
    if (N % (1 << levels) != 0 || !limb_kernel_fits(capSA, capSB)) return false;
    return wino_bf_ws(N, levels, capSA, capSB, capP) <= WINO_BF_MAX_BYTES;
}

// Breadth-first Winograd: sums of every level, then all leaf products in one
// launch, then the combinations of every level bottom up (kernels in limb.cu).
// Same products and sums as rec_winograd, so the same exact result.
gbmm_status rec_winograd_bf(RecCtx &c, gbmm_mat C, gbmm_mat A, gbmm_mat B, int N, int levels) {
    WinoTree t;
    t.A = A;
    t.B = B;
    t.C = C;
    t.N = N;
    t.levels = levels;
    t.capSA = c.capSA;
    t.capSB = c.capSB;
    t.capP = c.capP;
    const size_t mark = arena_mark(c.h);
    int64_t np = 1;
    for (int d = 1; d <= levels; d++) {
        const int64_t h = N >> d, e = h * h;
        t.sa_limbs[d] = (uint32_t *)arena_alloc(c.h, (size_t)(4 * np * e) * t.capSA * 4);
        t.sa_sizes[d] = (int32_t *)arena_alloc(c.h, (size_t)(4 * np * e) * 4);
        t.sb_limbs[d] = (uint32_t *)arena_alloc(c.h, (size_t)(4 * np * e) * t.capSB * 4);
        t.sb_sizes[d] = (int32_t *)arena_alloc(c.h, (size_t)(4 * np * e) * 4);
        t.p_limbs[d] = (uint32_t *)arena_alloc(c.h, (size_t)(7 * np * e) * t.capP * 4);
        t.p_sizes[d] = (int32_t *)arena_alloc(c.h, (size_t)(7 * np * e) * 4);
        if (!t.sa_limbs[d] || !t.sa_sizes[d] || !t.sb_limbs[d] || !t.sb_sizes[d] || !t.p_limbs[d] || !t.p_sizes[d]) {
            arena_release(c.h, mark);
            return set_error(GBMM_ERR_NOMEM, "winograd tree exceeds the reserved workspace");
        }
        np *= 7;
    }
    gbmm_status st = GBMM_OK;
    for (int d = 1; d <= levels && st == GBMM_OK; d++) st = launch_wino_sums(t, d, c.s);
    if (st == GBMM_OK) st = launch_wino_leaves(t, c.s);
    for (int d = levels; d >= 1 && st == GBMM_OK; d--) st = launch_wino_combine(t, d, c.s);
    arena_release(c.h, mark);
    return st;
}

gbmm_status rec_square(RecCtx &c, int method, gbmm_mat C, gbmm_mat A, gbmm_mat B, int N, int levels, int addmul) {
    // recursion is skipped when the one-limb-longer sums it forms would not fit the per-entry kernel
    if (levels <= 0 || N % 2 != 0 || N / 2 < 1 || !limb_kernel_fits(c.capSA, c.capSB))
        return launch_limb_matmul(C, A, B, addmul, c.s);
    if (c.breadth_first && wino_bf_ok(method, N, levels, addmul, c.capSA, c.capSB, c.capP))
        return rec_winograd_bf(c, C, A, B, N, levels);
    // depth first from here down (the workspace was sized for that)
    RecCtx dc = c;
    dc.breadth_first = false;
    if (method == GBMM_METHOD_WINOGRAD) return rec_winograd(dc, C, A, B, N, levels, addmul);
    if (addmul) return launch_limb_matmul(C, A, B, 1, c.s);
    if (method == GBMM_METHOD_STRASSEN) return rec_strassen(dc, C, A, B, N, levels);
    if (method == GBMM_METHOD_NAIVE_REC) return rec_naive(dc, C, A, B, N, levels);
    return launch_limb_matmul(C, A, B, 0, c.s);
}

static int levels_for(int N, int cutoff) {
    if (N <= cutoff) return 0;
    int l = (int)ilog2u((unsigned)(N / cutoff));
    while (l > 0 && (N % (1 << l)) != 0) l--;
    return l;
}

// Workspace bytes for a square recursion of `levels` levels on N (sums with
// capSA / capSB planes, products with capP); `bf`: the breadth-first tree may be used.
static size_t rec_ws(int method, int N, int levels, int addmul, int capSA, int capSB, int capP, bool bf) {
    if (bf && wino_bf_ok(method, N, levels, addmul, capSA, capSB, capP)) return wino_bf_ws(N, levels, capSA, capSB, capP);
    const int capT = std::max(std::max(capSA, capSB), capP);
    size_t total = 0;
    int n = N;
    for (int l = 0; l < levels; l++) {
        int h = n / 2;
        int ntemps = method == GBMM_METHOD_NAIVE_REC ? 1 : 3;
        total += (size_t)ntemps * mat_bytes((int64_t)h * h, capT);
        n = h;
    }
    return total;
}

// squarify: power-of-two core plus remainders (mat-gpu/mat-pregpu.cu:548-576,
// mat-cpu/matj.c:680-780).  Small or non-square shapes go to the per-entry
// kernel, which handles any shape in one launch.
gbmm_status squarify(RecCtx &c, int method, gbmm_mat C, gbmm_mat A, gbmm_mat B) {
    const int K = A.rows, M = A.cols, N = B.cols;
    if (K == 0 || N == 0) return GBMM_OK;
    if (M == 0) return launch_mat_zero(C, c.s);
    const int base = c.cutoff;
    if (method == GBMM_METHOD_NAIVE || K <= base || M <= base || N <= base) return launch_limb_matmul(C, A, B, 0, c.s);
    if (K == M && M == N && remove_factors((unsigned)K, 2) <= (unsigned)base)
        return rec_square(c, method, C, A, B, K, levels_for(K, base), 0);
    int mindim = std::min(std::min(K, M), N);
    int pt = 1 << ilog2u((unsigned)mindim);
    size_t mark = arena_mark(c.h);
    gbmm_mat T;
    if (!arena_mat(c.h, K, N, c.capP, T)) return set_error(GBMM_ERR_NOMEM, "squarify temporary");
    auto A_ = [&](int r, int cc) { return sub_view(A, r ? pt : 0, cc ? pt : 0, r ? K - pt : pt, cc ? M - pt : pt); };
    auto B_ = [&](int r, int cc) { return sub_view(B, r ? pt : 0, cc ? pt : 0, r ? M - pt : pt, cc ? N - pt : pt); };
    auto C_ = [&](const gbmm_mat &X, int r, int cc) {
        return sub_view(X, r ? pt : 0, cc ? pt : 0, r ? K - pt : pt, cc ? N - pt : pt);
    };
    for (int r = 0; r < 2; r++)
        for (int cc = 0; cc < 2; cc++) {
            gbmm_mat cq = C_(C, r, cc);
            if (cq.rows == 0 || cq.cols == 0) continue;
            GBMM_TRY(squarify(c, method, cq, A_(r, 0), B_(0, cc)));
            if (M > pt) {
                gbmm_mat tq = C_(T, r, cc);
                GBMM_TRY(squarify(c, method, tq, A_(r, 1), B_(1, cc)));
                GBMM_TRY(launch_mat_addsub(cq, cq, tq, 0, c.s));
            }
        }
    arena_release(c.h, mark);
    return GBMM_OK;
}

static size_t squarify_ws(int method, int K, int M, int N, int base, int capSA, int capSB, int capP, bool bf) {
    if (K == 0 || M == 0 || N == 0) return 0;
    if (method == GBMM_METHOD_NAIVE || K <= base || M <= base || N <= base) return 0;
    if (K == M && M == N && remove_factors((unsigned)K, 2) <= (unsigned)base)
        return rec_ws(method, K, levels_for(K, base), 0, capSA, capSB, capP, bf);
    int mindim = std::min(std::min(K, M), N);
    int pt = 1 << ilog2u((unsigned)mindim);
    size_t own = mat_bytes((int64_t)K * N, capP);
    size_t sub = 0;
    int ks[2] = {pt, K - pt}, ms[2] = {pt, M - pt}, ns[2] = {pt, N - pt};
    for (int r = 0; r < 2; r++)
        for (int cc = 0; cc < 2; cc++)
            for (int kk = 0; kk < 2; kk++)
                sub = std::max(sub, squarify_ws(method, ks[r], ms[kk], ns[cc], base, capSA, capSB, capP, bf));
    return own + sub;
}

}  // namespace

// Limbs a C view needs: product bound plus recursion headroom (each recursion
// level can grow intermediate magnitudes by a few bits; 32 bits of headroom per
// 8 levels are provided).
static int limbs_needed(int la, int lb, int inner, int levels) {
    int logm = 0;
    while ((1 << logm) < std::max(inner, 1)) logm++;
    int bits = 32 * (la + lb) + logm + 4 * levels + 2;
    return (bits + 31) / 32;
}

extern "C" gbmm_status gbmm_matmul_limbs_needed(int32_t a_nlimbs, int32_t b_nlimbs, int32_t inner, const gbmm_opts *opts,
                                                int32_t *nlimbs) {
    if (!nlimbs) return set_error(GBMM_ERR_INVALID, "null pointer");
    int levels = 0;
    if (opts && opts->path != GBMM_PATH_CRT && opts->method != GBMM_METHOD_NAIVE) {
        int cutoff = opts->cutoff > 0 ? opts->cutoff : 32;
        levels = levels_for(inner, cutoff);
        if (levels < 0) levels = 0;
        levels += 2;  // squarify splits
    }
    *nlimbs = limbs_needed(a_nlimbs, b_nlimbs, inner, levels);
    return GBMM_OK;
}

namespace gbmm {
gbmm_status matmul_limb(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int method, int cutoff,
                        int accumulate, cudaStream_t s) {
    if (accumulate && (method == GBMM_METHOD_NAIVE || a.rows != a.cols || a.cols != b.cols ||
                       remove_factors((unsigned)a.rows, 2) > (unsigned)cutoff || method != GBMM_METHOD_WINOGRAD))
        return launch_limb_matmul(c, a, b, 1, s);
    RecCtx ctx;
    ctx.h = h;
    ctx.s = s;
    ctx.cutoff = cutoff;
    ctx.capSA = a.nlimbs + 1;
    ctx.capSB = b.nlimbs + 1;
    ctx.capP = c.nlimbs;
    ctx.breadth_first = h->wino_breadth_first != 0;
    size_t ws = accumulate ? rec_ws(method, a.rows, levels_for(a.rows, cutoff), 1, ctx.capSA, ctx.capSB, ctx.capP, false)
                           : squarify_ws(method, a.rows, a.cols, b.cols, cutoff, ctx.capSA, ctx.capSB, ctx.capP,
                                         ctx.breadth_first);
    if (ws) GBMM_TRY(arena_reserve(h, ws + 4096));
    if (accumulate) return rec_square(ctx, method, c, a, b, a.rows, levels_for(a.rows, cutoff), 1);
    return squarify(ctx, method, c, a, b);
}

// ---- Winograd's tree with CRT leaf products ------------------------------------------------
// Host twins of the tree's view arithmetic (wt_quad / wt_dense / wt_operand in limb.cu):
// the operand of node `node` at level d is a quadrant of an ancestor's operand or
// one of the dense sums of its parent.
static gbmm_mat wt_quad_h(gbmm_mat m, int qr, int qc, int h) {
    const int64_t off = (int64_t)qr * h * m.rs + (int64_t)qc * h;
    m.limbs += off;
    m.sizes += off;
    m.rows = h;
    m.cols = h;
    return m;
}
static gbmm_mat wt_dense_h(uint32_t *limbs, int32_t *sizes, int64_t q, int h, int cap) {
    gbmm_mat m;
    memset(&m, 0, sizeof m);
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
static gbmm_mat wt_operand_h(const WinoTree &t, int which, int d, int64_t node) {
    gbmm_mat v = which ? t.B : t.A;
    int h = t.N;
    int64_t pw = 1;
    for (int l = 1; l < d; l++) pw *= 7;
    for (int l = 1; l <= d; l++) {
        const int64_t self = node / pw;  // this node's ancestor at level l
        const int j = (int)(self % 7);
        const int64_t parent = self / 7;
        h >>= 1;
        int sidx = -1;
        if (which == 0) {
            if (j == 0) v = wt_quad_h(v, 0, 0, h);
            else if (j == 1) v = wt_quad_h(v, 0, 1, h);
            else if (j == 3) v = wt_quad_h(v, 1, 1, h);
            else sidx = j == 2 ? 3 : j - 4;
        } else {
            if (j == 0) v = wt_quad_h(v, 0, 0, h);
            else if (j == 1) v = wt_quad_h(v, 1, 0, h);
            else if (j == 2) v = wt_quad_h(v, 1, 1, h);
            else sidx = j == 3 ? 3 : j - 4;
        }
        if (sidx >= 0)
            v = which ? wt_dense_h(t.sb_limbs[l], t.sb_sizes[l], 4 * parent + sidx, h, t.capSB)
                      : wt_dense_h(t.sa_limbs[l], t.sa_sizes[l], 4 * parent + sidx, h, t.capSA);
        pw /= 7;
    }
    return v;
}

static int64_t pow7_h(int l) {
    int64_t r = 1;
    while (l-- > 0) r *= 7;
    return r;
}
static constexpr int WINO_CRT_MAX_LEVELS = 4;  // 2401 leaf products at most

// Whether a product takes Winograd's tree with CRT leaves: square, at least one
// level above the cutoff, and leaves that one CRT pass takes (k <= 512, at most
// 1023 moduli for the one-limb-longer sums).
bool wino_crt_ok(int la, int lb, int m, int k, int n, int cutoff) {
    if (m != k || k != n || cutoff < 1) return false;
    const int L = levels_for(m, cutoff);
    if (L < 1 || L > WINO_CRT_MAX_LEVELS) return false;
    const int hL = m >> L;
    return crt_single_pass(hL) && crt_feasible(la + 1, lb + 1, hL);
}

// Workspace of wino_crt: the tree, a result with headroom when C has too few
// planes, every leaf's CRT workspace and the records' blob.
size_t wino_crt_ws(int la, int lb, int N, int cn, int cutoff) {
    const int L = levels_for(N, cutoff), hL = N >> L;
    const int capSA = la + 1, capSB = lb + 1, need = limbs_needed(la, lb, N, L + 2);
    const int capP = std::max(cn, need);
    const int64_t leaves = pow7_h(L);
    return wino_bf_ws(N, L, capSA, capSB, capP) + (cn < need ? mat_bytes((int64_t)N * N, capP) : 0) +
           (size_t)leaves * (crt_group_ws(capSA, capSB, hL, hL, hL) + 1024) + 4096 * (size_t)leaves + 16384;
}

// C = A B through Winograd's breadth-first tree down to the cutoff: the sums of
// every level and the combinations as limb kernels (k_wino_sums / k_wino_combine),
// the 7^L leaf products as CRT products in the grouped launches, one persistent
// launch per CRT stage over all leaves.  The same tree and operation order as the
// limb form, so the same exact result.  The caller checked wino_crt_ok.
gbmm_status wino_crt(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, int cutoff,
                     cudaStream_t s) {
    const int N = a.rows, L = levels_for(N, cutoff), hL = N >> L;
    const int need = limbs_needed(a.nlimbs, b.nlimbs, N, L + 2);
    WinoTree t;
    t.A = a;
    t.B = b;
    t.N = N;
    t.levels = L;
    t.capSA = a.nlimbs + 1;
    t.capSB = b.nlimbs + 1;
    t.capP = std::max(c.nlimbs, need);
    const size_t mark = arena_mark(h);
    gbmm_status st = GBMM_OK;
    auto fail = [&](gbmm_status e) {
        arena_release(h, mark);
        return e;
    };
    t.C = c;
    if (c.nlimbs < need && !arena_mat(h, N, N, t.capP, t.C)) return fail(set_error(GBMM_ERR_NOMEM, "winograd crt: result"));
    int64_t np = 1;
    for (int d = 1; d <= L; d++) {
        const int64_t hd = N >> d, e = hd * hd;
        t.sa_limbs[d] = (uint32_t *)arena_alloc(h, (size_t)(4 * np * e) * t.capSA * 4);
        t.sa_sizes[d] = (int32_t *)arena_alloc(h, (size_t)(4 * np * e) * 4);
        t.sb_limbs[d] = (uint32_t *)arena_alloc(h, (size_t)(4 * np * e) * t.capSB * 4);
        t.sb_sizes[d] = (int32_t *)arena_alloc(h, (size_t)(4 * np * e) * 4);
        t.p_limbs[d] = (uint32_t *)arena_alloc(h, (size_t)(7 * np * e) * t.capP * 4);
        t.p_sizes[d] = (int32_t *)arena_alloc(h, (size_t)(7 * np * e) * 4);
        if (!t.sa_limbs[d] || !t.sa_sizes[d] || !t.sb_limbs[d] || !t.sb_sizes[d] || !t.p_limbs[d] || !t.p_sizes[d])
            return fail(set_error(GBMM_ERR_NOMEM, "winograd crt: tree exceeds the reserved workspace"));
        np *= 7;
    }
    // every leaf product joins one group: its workspace is carved now, nothing launched
    std::unique_ptr<crt_group, void (*)(crt_group *)> g(crt_group_create(), crt_group_destroy);
    for (int64_t leaf = 0; leaf < np; leaf++) {
        const gbmm_mat la = wt_operand_h(t, 0, L, leaf), lb = wt_operand_h(t, 1, L, leaf);
        const gbmm_mat lp = wt_dense_h(t.p_limbs[L], t.p_sizes[L], leaf, hL, t.capP);
        st = crt_group_add(h, g.get(), lp, la, lb, 32LL * la.nlimbs, 32LL * lb.nlimbs, 0);
        if (st != GBMM_OK) return fail(st);
    }
    const std::vector<char> &blob = crt_group_blob(g.get());
    char *d_blob = (char *)arena_alloc(h, blob.size());
    if (!d_blob) return fail(set_error(GBMM_ERR_NOMEM, "winograd crt: records"));
    // stream-ordered: the region may still serve earlier work on s (pageable source:
    // staged before the call returns)
    cudaError_t ce = cudaMemcpyAsync(d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, s);
    if (ce != cudaSuccess) return fail(cuda_error(ce, "winograd crt: records"));
    for (int d = 1; d <= L && st == GBMM_OK; d++) st = launch_wino_sums(t, d, s);
    if (st == GBMM_OK) st = crt_group_launch(g.get(), d_blob, s, nullptr, nullptr);
    for (int d = L; d >= 1 && st == GBMM_OK; d--) st = launch_wino_combine(t, d, s);
    if (st == GBMM_OK && t.C.limbs != c.limbs) st = launch_mat_copy(c, t.C, s);
    arena_release(h, mark);
    return st;
}
}  // namespace gbmm

namespace gbmm {

Plan plan_of(int id) {
    Plan p;
    p.id = id;
    switch (id) {
        case GBMM_PLAN_LIMB_NAIVE: p.path = GBMM_PATH_LIMB; p.method = GBMM_METHOD_NAIVE; break;
        case GBMM_PLAN_LIMB_W32: p.path = GBMM_PATH_LIMB; p.method = GBMM_METHOD_WINOGRAD; p.cutoff = 32; break;
        case GBMM_PLAN_LIMB_W64: p.path = GBMM_PATH_LIMB; p.method = GBMM_METHOD_WINOGRAD; p.cutoff = 64; break;
        case GBMM_PLAN_LIMB_W128: p.path = GBMM_PATH_LIMB; p.method = GBMM_METHOD_WINOGRAD; p.cutoff = 128; break;
        case GBMM_PLAN_CRT_SINGLE: p.path = GBMM_PATH_CRT; p.tiles = 1; break;
        case GBMM_PLAN_CRT_PAIR: p.path = GBMM_PATH_CRT; p.tiles = 2; break;
        case GBMM_PLAN_CRT_SPLIT: p.path = GBMM_PATH_CRT; p.split = 1; break;
        default: p.path = GBMM_PATH_CRT; p.id = GBMM_PLAN_CRT; break;
    }
    return p;
}

bool plan_admissible(int id, int m, int k, int n, int la, int lb) {
    const Plan p = plan_of(id);
    // about 50 ms of schoolbook work at 4e12 32-bit MAC/s: limb plans beyond it are not timed
    if (p.path == GBMM_PATH_LIMB && (double)m * k * n * la * lb > 2e11) return false;
    if (p.method == GBMM_METHOD_WINOGRAD && std::min(std::min(m, k), n) <= p.cutoff) return false;
    if (p.split && std::max(la, lb) < 2) return false;
    return true;
}

// Plain dispatch rule: the CRT form for products with enough limb work (it pays
// off once the residue and reconstruction passes are amortised), the per-entry
// limb kernel otherwise.  Entries of fewer than 16 limbs together take the CRT
// form from 2^25 schoolbook MACs on (in a batch their CRT stages join the grouped
// launches; measured on a batch of 64 products with m, k, n log-uniform in [16, 512]
// and bit lengths log-uniform in [64, 16384]: 2^25 gave the shortest batch among
// thresholds 2^24 .. 2^30).  Entries too long for one CRT
// product (more than 1023 moduli) still take the CRT path: dispatch() splits them
// into limb halves that fit.
static int64_t g_crt_short_work = (int64_t)1 << 25;  // 0: never for short entries
int heuristic_plan(int m, int k, int n, int la, int lb) {
    const int64_t work = (int64_t)m * k * n * la * lb;
    if (la + lb >= 16 && work >= ((int64_t)1 << 22)) return GBMM_PLAN_CRT;
    if (g_crt_short_work > 0 && work >= g_crt_short_work) return GBMM_PLAN_CRT;
    return GBMM_PLAN_LIMB_NAIVE;
}

static bool direct_ok(const Plan &p, int la, int lb, int k) {
    if (p.split > 0 && std::max(la, lb) >= 2) return false;
    if (p.path == GBMM_PATH_CRT) return crt_feasible(la, lb, k);
    return limb_kernel_fits(la, lb);
}

// Upper bound of the device workspace dispatch() carves from the arena.
size_t dispatch_ws(const Plan &p, int la, int lb, int m, int k, int n, int cn, int accumulate) {
    if (m == 0 || n == 0 || k == 0) return 0;
    if (p.path == GBMM_PATH_CRT && p.method == GBMM_METHOD_WINOGRAD_CRT && !accumulate &&
        wino_crt_ok(la, lb, m, k, n, p.cutoff))
        return wino_crt_ws(la, lb, m, cn, p.cutoff);
    if (direct_ok(p, la, lb, k)) {
        if (p.path == GBMM_PATH_CRT) return crt_workspace_bytes(la, lb, m, k, n, cn);
        if (p.method == GBMM_METHOD_NAIVE) return 0;
        int levels = levels_for(std::max(std::max(m, k), n), p.cutoff) + 2;
        int need = limbs_needed(la, lb, k, levels);
        const int capP = std::max(need, cn);
        // the breadth-first tree's workspace is counted whether or not the handle uses it
        size_t rec = accumulate ? rec_ws(p.method, m, levels_for(m, p.cutoff), 1, la + 1, lb + 1, capP, false)
                                : squarify_ws(p.method, m, k, n, p.cutoff, la + 1, lb + 1, capP, true);
        return (cn < need ? mat_bytes((int64_t)m * n, need) : 0) + rec + 8192;
    }
    const bool sa = la >= lb;
    const int hl = (sa ? la : lb) / 2, hn = (sa ? la : lb) - hl;
    const int64_t xs = sa ? (int64_t)m * k : (int64_t)k * n;
    const int tn = limbs_needed(sa ? hn : la, sa ? lb : hn, k, 0) + 1;
    // half sizes, the stacked halves (2 xs entries of hn limbs) and the stacked product
    size_t own = 2 * (align_up((size_t)xs * 4, 256) + 256) + mat_bytes(2 * xs, hn) + mat_bytes(2 * (int64_t)m * n, tn) +
                 1024;
    Plan q = p;
    q.split = std::max(0, p.split - 1);
    return own + dispatch_ws(q, sa ? hn : la, sa ? lb : hn, sa ? 2 * m : m, k, sa ? n : 2 * n, tn, 0);
}

// C (+)= A*B with the planned path.  An operand too long for the chosen kernels
// is split into low and high limb halves, X = X_hi 2^(32h) + X_lo (the
// Karatsuba-style split of Knuth 4.3.3 without the middle-product trick), and
// the halves are stacked into one operand: A's as rows [A_lo; A_hi], B's as
// columns [B_lo | B_hi].  One product T against the other operand (whose CRT
// residues or staged limbs are then formed once) gives both half products, and
// C (+)= T_0 + T_1 2^(32h).
gbmm_status dispatch(gbmm_handle h, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b, const Plan &p,
                     int accumulate, cudaStream_t s) {
    const int m = a.rows, k = a.cols, n = b.cols;
    if (m == 0 || n == 0) return GBMM_OK;
    if (k == 0) return accumulate ? GBMM_OK : launch_mat_zero(c, s);
    if (p.path == GBMM_PATH_CRT && p.method == GBMM_METHOD_WINOGRAD_CRT && !accumulate &&
        wino_crt_ok(a.nlimbs, b.nlimbs, m, k, n, p.cutoff))
        return wino_crt(h, c, a, b, p.cutoff, s);
    if (direct_ok(p, a.nlimbs, b.nlimbs, k)) {
        if (p.path == GBMM_PATH_CRT) {
            const int saved = h->crt_tiles;
            h->crt_tiles = p.tiles;
            const gbmm_status st = crt_matmul(h, c, a, b, 32LL * a.nlimbs, 32LL * b.nlimbs, p.nprimes, accumulate, s);
            h->crt_tiles = saved;
            return st;
        }
        int levels = p.method == GBMM_METHOD_NAIVE ? 0 : levels_for(std::max(std::max(m, k), n), p.cutoff) + 2;
        int need = limbs_needed(a.nlimbs, b.nlimbs, k, levels);
        if (c.nlimbs < need && p.method != GBMM_METHOD_NAIVE) {
            // the recursion needs headroom for intermediate values: run it into a
            // workspace matrix with enough planes, then copy into C (the copy
            // flags a capacity error if the exact result does not fit C)
            size_t mark = arena_mark(h);
            gbmm_mat T;
            if (!arena_mat(h, m, n, need, T)) return set_error(GBMM_ERR_NOMEM, "workspace");
            if (accumulate) GBMM_TRY(launch_mat_copy(T, c, s));
            gbmm_status st = matmul_limb(h, T, a, b, p.method, p.cutoff, accumulate, s);
            if (st == GBMM_OK) st = launch_mat_copy(c, T, s);
            arena_release(h, mark);
            return st;
        }
        return matmul_limb(h, c, a, b, p.method, p.cutoff, accumulate, s);
    }
    const bool sa = a.nlimbs >= b.nlimbs;
    const gbmm_mat &X = sa ? a : b;
    if (X.nlimbs < 2) return set_error(GBMM_ERR_UNSUPPORTED, "no kernel takes %d x %d limb entries", a.nlimbs, b.nlimbs);
    const int hl = X.nlimbs / 2, hn = X.nlimbs - hl;
    size_t mark = arena_mark(h);
    const size_t xs = (size_t)(X.rows - 1) * X.rs + X.cols;
    int32_t *lo = (int32_t *)arena_alloc(h, xs * 4), *hi = (int32_t *)arena_alloc(h, xs * 4);
    // S: the stacked halves (hn limb planes); T: the stacked product
    gbmm_mat S, T;
    const int tn = limbs_needed(sa ? hn : a.nlimbs, sa ? b.nlimbs : hn, k, 0) + 1;
    if (!lo || !hi || !arena_mat(h, sa ? 2 * m : k, sa ? k : 2 * n, hn, S) ||
        !arena_mat(h, sa ? 2 * m : m, sa ? n : 2 * n, tn, T))
        return set_error(GBMM_ERR_NOMEM, "split workspace");
    GBMM_TRY(launch_split_sizes(X, hl, lo, hi, s));
    gbmm_mat Xlo = X, Xhi = X;
    Xlo.nlimbs = hl;
    Xlo.sizes = lo;
    Xhi.nlimbs = hn;
    Xhi.limbs = X.limbs + (int64_t)hl * X.ld;
    Xhi.sizes = hi;
    const int xr = X.rows, xc = X.cols;
    GBMM_TRY(launch_mat_copy(sa ? sub_view(S, 0, 0, xr, xc) : sub_view(S, 0, 0, xr, xc), Xlo, s));
    GBMM_TRY(launch_mat_copy(sa ? sub_view(S, xr, 0, xr, xc) : sub_view(S, 0, xc, xr, xc), Xhi, s));
    Plan q = p;
    q.split = std::max(0, p.split - 1);
    gbmm_status st = dispatch(h, T, sa ? S : a, sa ? b : S, q, 0, s);
    const gbmm_mat T0 = sub_view(T, 0, 0, m, n), T1 = sa ? sub_view(T, m, 0, m, n) : sub_view(T, 0, n, m, n);
    if (st == GBMM_OK && accumulate) st = launch_add_shifted(c, c, T0, 0, s);
    if (st == GBMM_OK) st = launch_add_shifted(c, accumulate ? c : T0, T1, hl, s);
    arena_release(h, mark);
    return st;
}

// The split above for a batch's grouped CRT launches: the direct form, or one
// limb-half split whose halves go through one single-pass CRT product.
static bool split_halves(const Plan &p, int la, int lb, int k, int &hl, int &hn, Plan &q) {
    const bool sa = la >= lb;
    const int xl = sa ? la : lb;
    if (xl < 2) return false;
    hl = xl / 2;
    hn = xl - hl;
    q = p;
    q.split = std::max(0, p.split - 1);
    return direct_ok(q, sa ? hn : la, sa ? lb : hn, k);
}

// Products of C with at least this many entries fill the GPU alone (their
// reconstruction alone has 128 or more CTA-pair tiles) and keep their own
// tile forms on a side stream.  Measured on a batch of 64 products with m, k, n
// log-uniform in [16, 512] and bit lengths log-uniform in [64, 16384], and on one
// of 72 that adds eight 1024 x 64 x 1024 products: 8.10 / 26.1 ms, against 8.54 /
// 28.5 ms grouping every product and 8.31 / 26.4 ms grouping none (2^17 in between).
constexpr int64_t GROUP_MAX_ENTRIES = (int64_t)1 << 15;

bool crt_groupable(const Plan &p, int la, int lb, int m, int k, int n) {
    if (p.path != GBMM_PATH_CRT || m == 0 || n == 0 || k == 0 || !crt_single_pass(k)) return false;
    if ((int64_t)m * n >= GROUP_MAX_ENTRIES) return false;
    if (direct_ok(p, la, lb, k)) return true;
    int hl, hn;
    Plan q;
    return split_halves(p, la, lb, k, hl, hn, q);
}

size_t crt_group_job_ws(const Plan &p, int la, int lb, int m, int k, int n) {
    if (direct_ok(p, la, lb, k)) return crt_group_ws(la, lb, m, k, n);
    int hl, hn;
    Plan q;
    if (!split_halves(p, la, lb, k, hl, hn, q)) return 0;
    const bool sa = la >= lb;
    const int tn = limbs_needed(sa ? hn : la, sa ? lb : hn, k, 0) + 1;
    return mat_bytes(2 * (int64_t)m * n, tn) + 1024 + crt_group_ws(sa ? hn : la, sa ? lb : hn, sa ? 2 * m : m, k, sa ? n : 2 * n);
}

gbmm_status crt_collect(gbmm_handle h, crt_group *g, const gbmm_mat &c, const gbmm_mat &a, const gbmm_mat &b,
                        const Plan &p) {
    const int m = a.rows, k = a.cols, n = b.cols;
    if (direct_ok(p, a.nlimbs, b.nlimbs, k))
        return crt_group_add(h, g, c, a, b, 32LL * a.nlimbs, 32LL * b.nlimbs, p.nprimes);
    int hl, hn;
    Plan q;
    if (!split_halves(p, a.nlimbs, b.nlimbs, k, hl, hn, q))
        return set_error(GBMM_ERR_UNSUPPORTED, "crt group: no single-pass form for %d x %d limb entries", a.nlimbs,
                         b.nlimbs);
    // as dispatch(): one product T against the halves stacked (read in place by the
    // digits stage), then C = T_0 + T_1 2^(32 hl); T stays carved until the group has run
    const bool sa = a.nlimbs >= b.nlimbs;
    const gbmm_mat &X = sa ? a : b;
    gbmm_mat S, T;
    memset(&S, 0, sizeof S);
    S.rows = sa ? 2 * m : k;
    S.cols = sa ? k : 2 * n;
    S.nlimbs = hn;
    const int tn = limbs_needed(sa ? hn : a.nlimbs, sa ? b.nlimbs : hn, k, 0) + 1;
    if (!arena_mat(h, sa ? 2 * m : m, sa ? n : 2 * n, tn, T)) return set_error(GBMM_ERR_NOMEM, "crt group: split workspace");
    crt_halves hv;
    hv.side = sa ? 0 : 1;
    hv.x = X;
    hv.hl = hl;
    GBMM_TRY(crt_group_add(h, g, T, sa ? S : a, sa ? b : S, 32LL * (sa ? hn : a.nlimbs), 32LL * (sa ? b.nlimbs : hn),
                           q.nprimes, &hv));
    const gbmm_mat T0 = sub_view(T, 0, 0, m, n), T1 = sa ? sub_view(T, m, 0, m, n) : sub_view(T, 0, n, m, n);
    crt_group_post(g, [=](cudaStream_t s) { return launch_add_shifted(c, T0, T1, hl, s); });
    return GBMM_OK;
}

gbmm_status resolve_plan(gbmm_handle h, const gbmm_mat &a, const gbmm_mat &b, const gbmm_opts &o, Plan &p) {
    if (o.plan) {
        if (o.plan < 1 || o.plan > GBMM_NPLANS) return set_error(GBMM_ERR_INVALID, "unknown plan %d", o.plan - 1);
        p = plan_of(o.plan - 1);
        p.nprimes = o.nprimes;
        return GBMM_OK;
    }
    if (o.path == GBMM_PATH_AUTO) {
        p = plan_of(choose_plan(h, a.rows, a.cols, b.cols, a.nlimbs, b.nlimbs));
        if (o.cutoff > 0) p.cutoff = o.cutoff;
        p.nprimes = o.nprimes;
        return GBMM_OK;
    }
    p = Plan();
    p.method = o.method ? o.method : GBMM_METHOD_WINOGRAD;
    p.cutoff = o.cutoff > 0 ? o.cutoff : h->limb_cutoff;
    p.nprimes = o.nprimes;
    // the tree with CRT leaves is a CRT form whatever path was asked for
    p.path = p.method == GBMM_METHOD_WINOGRAD_CRT ? GBMM_PATH_CRT : o.path;
    if (p.path != GBMM_PATH_CRT && p.path != GBMM_PATH_LIMB) return set_error(GBMM_ERR_INVALID, "unknown path %d", o.path);
    return GBMM_OK;
}

}  // namespace gbmm

// Internal hook: schoolbook work (m k n la lb) from which the heuristic takes the CRT
// form for entries of fewer than 16 limbs together (0: never); returns the old value.
extern "C" int64_t gbmmx_crt_short_work(int64_t work) {
    const int64_t old = g_crt_short_work;
    g_crt_short_work = work < 0 ? 0 : work;
    return old;
}

extern "C" gbmm_status gbmm_matmul(gbmm_handle h, gbmm_mat c, gbmm_mat a, gbmm_mat b, const gbmm_opts *opts) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    GBMM_TRY(validate_mat(c, "C"));
    GBMM_TRY(validate_mat(a, "A"));
    GBMM_TRY(validate_mat(b, "B"));
    if (a.rows != c.rows || b.cols != c.cols || a.cols != b.rows)
        return set_error(GBMM_ERR_INVALID, "shape mismatch: C %dx%d, A %dx%d, B %dx%d", c.rows, c.cols, a.rows, a.cols,
                         b.rows, b.cols);
    if (c.limbs == a.limbs || c.limbs == b.limbs) return set_error(GBMM_ERR_INVALID, "C must not alias A or B");
    gbmm_opts o;
    memset(&o, 0, sizeof o);
    if (opts) o = *opts;
    Plan p;
    GBMM_TRY(resolve_plan(h, a, b, o, p));
    GBMM_TRY(arena_reserve(h, dispatch_ws(p, a.nlimbs, b.nlimbs, a.rows, a.cols, b.cols, c.nlimbs, o.accumulate) + 65536));
    return dispatch(h, c, a, b, p, o.accumulate, h->stream);
}

extern "C" gbmm_status gbmm_mpn_mul(gbmm_handle h, uint32_t *rp, const uint32_t *up, int32_t un, const uint32_t *vp,
                                    int32_t vn, int64_t ld, int64_t nb) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    if (un < vn || vn < 1) return set_error(GBMM_ERR_INVALID, "mpn_mul needs un >= vn >= 1");
    const int s = un >> 1, n = un - s, t = vn - n;
    // The on-chip basecase beats the on-chip Toom-2.2 wherever it fits (measured on
    // 2^16 to 2^18 operand pairs: Toom at 0.70x its speed at 64 limbs, 0.80x at 128,
    // 0.86x at 192): the Karatsuba split's additions cost more than the quarter of
    // the MACs it saves.  Longer balanced operands take Toom-2.2.
    const bool toom = !mpn_basecase_on_chip(un, vn) && 4 * un < 5 * vn && 0 < t && t <= s;
    if (!toom) return gbmm_mpn_mul_basecase(rp, up, un, vp, vn, ld, nb, h->stream);
    const int32_t itch = gbmm_mpn_toom22_mul_itch(un, vn);
    if (itch < 0) return set_error(GBMM_ERR_INVALID, "mpn_mul: un=%d is too long", un);
    size_t need = (size_t)itch * (size_t)ld * 4;
    GBMM_TRY(arena_reserve(h, need + 4096));
    size_t mark = arena_mark(h);
    uint32_t *scratch = (uint32_t *)arena_alloc(h, need);
    gbmm_status st = gbmm_mpn_toom22_mul(rp, up, un, vp, vn, scratch, ld, nb, h->stream);
    arena_release(h, mark);
    return st;
}

