// Batched products of uneven shape and bit length, the path dispatcher, the
// autotuner and CUDA-graph replay.
//
// gbmm_matmul_batched splits the jobs by plan.  Limb jobs planned without
// recursion are cut into (job, tile) items, sorted largest first, and run by ONE
// persistent kernel per group (block edge, CTA form, thin operands) that drains a
// device work queue.  CRT jobs with one pass over k (directly or after one
// limb-half split) run in grouped launches: one persistent launch per CRT stage
// and kernel form over the tiles of all of them.  The other jobs (Winograd
// trees, longer CRT products) run through dispatch() on side streams.  The whole launch
// sequence of a batch is captured into a CUDA graph the second time a batch
// with the same signature (shapes, pointers, paths) is seen, and replayed from
// then on.  This replaces the reference's chunked multi-stream job DAG
// (mat-gpu/job.cu:32-338, never called there) with one graph launch.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "gbmm_internal.h"

namespace gbmm {

// ---- tuning table ------------------------------------------------------------------------------
// Key: rounded log2 of m, k, n and of the operand limb counts.
static int lg2r(int x) { return x <= 1 ? 0 : (int)lrint(log2((double)x)); }
static uint64_t tune_key(int m, int k, int n, int la, int lb) {
    return ((uint64_t)lg2r(m) << 32) | ((uint64_t)lg2r(k) << 24) | ((uint64_t)lg2r(n) << 16) |
           ((uint64_t)lg2r(la) << 8) | (uint64_t)lg2r(lb);
}

struct TuneEntry {
    int plan;  // gbmm_plan
    float ms;
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    char *d_blob = nullptr;  // work-queue and grouped-CRT blob owned by this graph
    uint64_t nkern = 0;      // library kernels in the graph (counted as launches per replay)
};

constexpr int NSIDE = 8;  // side streams a batch's dispatched jobs are spread over

struct BatchState {
    std::map<uint64_t, TuneEntry> tune;
    // side streams and the events that fork them from and join them to the handle's stream
    cudaStream_t side[NSIDE] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[NSIDE] = {};
    cudaEvent_t post_ev = nullptr;  // grouped CRT: its post steps' stream waits for it
    // graph cache
    std::map<std::string, GraphEntry> graphs;
    std::map<std::string, int> seen;
    bool use_graphs = true;
    // pinned staging for eager batches, guarded by an event on the last copy
    char *h_stage = nullptr;
    size_t h_cap = 0;
    cudaEvent_t staged = nullptr;
    int *d_counter = nullptr;  // one per work-queue group (LimbBatchPlan::MAX_GROUPS)
};

static BatchState &bstate(gbmm_handle h) {
    if (!h->batch) h->batch = new BatchState();
    return *static_cast<BatchState *>(h->batch);
}

void batch_state_destroy(gbmm_handle h) {
    if (!h->batch) return;
    BatchState *b = static_cast<BatchState *>(h->batch);
    for (auto &kv : b->graphs) {
        cudaGraphExecDestroy(kv.second.exec);
        cudaFree(kv.second.d_blob);
    }
    if (b->staged) cudaEventDestroy(b->staged);
    for (int i = 0; i < NSIDE; i++) {
        if (b->side[i]) cudaStreamDestroy(b->side[i]);
        if (b->join_ev[i]) cudaEventDestroy(b->join_ev[i]);
    }
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->post_ev) cudaEventDestroy(b->post_ev);
    if (b->h_stage) cudaFreeHost(b->h_stage);
    if (b->d_counter) cudaFree(b->d_counter);
    delete b;
    h->batch = nullptr;
}

void invalidate_graphs(gbmm_handle h) {
    if (!h->batch) return;
    BatchState &b = bstate(h);
    for (auto &kv : b.graphs) {
        cudaGraphExecDestroy(kv.second.exec);
        cudaFree(kv.second.d_blob);
    }
    b.graphs.clear();
    b.seen.clear();
}

int choose_plan(gbmm_handle h, int m, int k, int n, int la, int lb) {
    if (h->model && h->use_model) {
        const int p = model_choose(h, m, k, n, la, lb);
        if (p >= 0 && p < GBMM_NPLANS) return p;
    }
    if (h->batch) {
        BatchState &b = bstate(h);
        auto it = b.tune.find(tune_key(m, k, n, la, lb));
        if (it != b.tune.end()) return it->second.plan;
    }
    return heuristic_plan(m, k, n, la, lb);
}

}  // namespace gbmm

using namespace gbmm;

static std::string job_signature(const gbmm_job *jobs, int njobs, const std::vector<Plan> &plans) {
    std::string sig;
    sig.reserve((size_t)njobs * 96);
    char buf[256];
    for (int j = 0; j < njobs; j++) {
        const gbmm_job &q = jobs[j];
        snprintf(buf, sizeof buf, "%p,%p,%p,%p,%p,%p,%d,%d,%d,%d,%d,%d,%lld,%lld,%lld,%lld,%lld,%lld,%d,%d,%d,%d,%d;",
                 (void *)q.c.limbs, (void *)q.c.sizes, (void *)q.a.limbs, (void *)q.a.sizes, (void *)q.b.limbs,
                 (void *)q.b.sizes, q.a.rows, q.a.cols, q.b.cols, q.a.nlimbs, q.b.nlimbs, q.c.nlimbs, (long long)q.a.rs,
                 (long long)q.a.ld, (long long)q.b.rs, (long long)q.b.ld, (long long)q.c.rs, (long long)q.c.ld,
                 plans[j].path, plans[j].cutoff, plans[j].method, plans[j].tiles, plans[j].split);
        sig += buf;
    }
    return sig;
}

// Splits a batch: limb-path jobs planned without recursion that fit the
// per-entry kernel go to the persistent work-queue kernel, everything else
// (Winograd trees, CRT products) through dispatch().
static void split_batch(const gbmm_job *jobs, int njobs, const std::vector<Plan> &plans, std::vector<int> &queue_jobs,
                        std::vector<int> &other) {
    for (int j = 0; j < njobs; j++) {
        const gbmm_job &q = jobs[j];
        if (plans[j].path == GBMM_PATH_LIMB && plans[j].method == GBMM_METHOD_NAIVE &&
            limb_kernel_fits(q.a.nlimbs, q.b.nlimbs) && q.a.rows && q.b.cols && q.a.cols)
            queue_jobs.push_back(j);
        else
            other.push_back(j);
    }
}

// Side streams for batches (created on first use).
static gbmm_status side_streams(BatchState &bs) {
    if (bs.fork_ev) return GBMM_OK;
    for (int i = 0; i < NSIDE; i++) {
        GBMM_CUDA_TRY(cudaStreamCreateWithFlags(&bs.side[i], cudaStreamNonBlocking));
        GBMM_CUDA_TRY(cudaEventCreateWithFlags(&bs.join_ev[i], cudaEventDisableTiming));
    }
    GBMM_CUDA_TRY(cudaEventCreateWithFlags(&bs.post_ev, cudaEventDisableTiming));
    GBMM_CUDA_TRY(cudaEventCreateWithFlags(&bs.fork_ev, cudaEventDisableTiming));
    return GBMM_OK;
}

// Side streams a batch with these dispatched jobs uses.
static int nside_for(size_t njobs) { return (int)std::min<size_t>(NSIDE, njobs); }

// Enqueues one batch on the handle's stream.  d_blob holds the work-queue plan
// on the device (already filled); the persistent limb kernel runs on the
// handle's stream.  The remaining jobs go through dispatch() on side streams
// forked from it (largest estimated work first, each to the least loaded
// stream), so independent products run side by side; every side stream carves
// its workspace from its own slice of the arena (`slice` bytes each, above the
// current top) and the handle's stream waits for all of them at the end.
static gbmm_status enqueue_batch(gbmm_handle h, const gbmm_job *jobs, const std::vector<Plan> &plans,
                                 const LimbBatchPlan &lp, const char *d_blob, const std::vector<int> &other,
                                 size_t slice, size_t base, crt_group *grp, const char *d_crt) {
    BatchState &bs = bstate(h);
    // the grouped CRT launches take side stream 0 (and 1 for their post steps),
    // the dispatched jobs the others
    const int gs = grp && !crt_group_empty(grp) ? 2 : 0;
    const int ns = std::min(NSIDE, gs + nside_for(other.size()));
    if (ns > 0) {
        GBMM_TRY(side_streams(bs));
        GBMM_CUDA_TRY(cudaEventRecord(bs.fork_ev, h->stream));
        for (int i = 0; i < ns; i++) GBMM_CUDA_TRY(cudaStreamWaitEvent(bs.side[i], bs.fork_ev, 0));
    }
    if (!lp.groups.empty()) GBMM_TRY(launch_limb_batch(lp, d_blob, bs.d_counter, h->stream));
    gbmm_status st = GBMM_OK;
    if (gs) st = crt_group_launch(grp, d_crt, bs.side[0], bs.side[1], bs.post_ev);
    std::vector<int> order(other);
    auto work = [&](int j) {
        const gbmm_job &q = jobs[j];
        return (double)q.a.rows * q.a.cols * q.b.cols * std::max(q.a.nlimbs, 1) * std::max(q.b.nlimbs, 1);
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work(x) > work(y); });
    // slice i of the arena (from `base`) serves side stream gs + i.  Slices start
    // above 0, so a reservation inside dispatch() that did not fit its slice fails
    // ("grow while in use") instead of reallocating the arena under work still
    // queued on the other side streams
    const int nd = ns - gs;
    std::vector<double> load(std::max(nd, 1), 0.0);
    for (int j : order) {
        if (st != GBMM_OK) break;
        int i = 0;
        for (int t = 1; t < nd; t++)
            if (load[t] < load[i]) i = t;
        load[i] += work(j);
        const size_t mark = arena_mark(h);
        h->ws.top = base + (size_t)i * slice;
        st = dispatch(h, jobs[j].c, jobs[j].a, jobs[j].b, plans[j], 0, bs.side[gs + i]);
        arena_release(h, mark);
        if (st != GBMM_OK) break;
    }
    for (int i = 0; i < ns; i++) {
        // joined even after an error, so a capture in progress can end cleanly
        GBMM_CUDA_TRY(cudaEventRecord(bs.join_ev[i], bs.side[i]));
        GBMM_CUDA_TRY(cudaStreamWaitEvent(h->stream, bs.join_ev[i], 0));
    }
    return st;
}

extern "C" gbmm_status gbmm_matmul_batched(gbmm_handle h, gbmm_job *jobs, int32_t njobs, const gbmm_opts *opts) {
    if (!h || (njobs > 0 && !jobs)) return set_error(GBMM_ERR_INVALID, "null argument");
    gbmm_opts o;
    memset(&o, 0, sizeof o);
    if (opts) o = *opts;
    if (o.accumulate) return set_error(GBMM_ERR_UNSUPPORTED, "batched products do not accumulate");
    std::vector<Plan> plans(njobs);
    size_t ws = 0;
    for (int j = 0; j < njobs; j++) {
        const gbmm_job &q = jobs[j];
        GBMM_TRY(validate_mat(q.c, "C"));
        GBMM_TRY(validate_mat(q.a, "A"));
        GBMM_TRY(validate_mat(q.b, "B"));
        if (q.a.rows != q.c.rows || q.b.cols != q.c.cols || q.a.cols != q.b.rows)
            return set_error(GBMM_ERR_INVALID, "job %d: shape mismatch", j);
        if (q.c.limbs == q.a.limbs || q.c.limbs == q.b.limbs)
            return set_error(GBMM_ERR_INVALID, "job %d: C must not alias A or B", j);
        gbmm_opts oj = o;
        oj.path = q.path ? q.path : o.path;
        if (q.cutoff) oj.cutoff = q.cutoff;
        if (q.nprimes) oj.nprimes = q.nprimes;
        GBMM_TRY(resolve_plan(h, q.a, q.b, oj, plans[j]));
        jobs[j].chosen_path = plans[j].path;
        jobs[j].chosen_plan = plans[j].id;
    }
    if (njobs == 0) return GBMM_OK;
    std::vector<int> queue_jobs, other, grouped;
    split_batch(jobs, njobs, plans, queue_jobs, other);
    {
        // CRT jobs with one pass over k go to the grouped launches
        std::vector<int> rest;
        for (int j : other) {
            const gbmm_job &q = jobs[j];
            if (crt_groupable(plans[j], q.a.nlimbs, q.b.nlimbs, q.a.rows, q.a.cols, q.b.cols)) grouped.push_back(j);
            else rest.push_back(j);
        }
        other.swap(rest);
    }
    size_t gws = 0;  // the grouped products' workspace, all carved at once
    for (int j : grouped) {
        const gbmm_job &q = jobs[j];
        gws += crt_group_job_ws(plans[j], q.a.nlimbs, q.b.nlimbs, q.a.rows, q.a.cols, q.b.cols) + 4096;
    }
    for (int j : other) {
        const gbmm_job &q = jobs[j];
        ws = std::max(ws, dispatch_ws(plans[j], q.a.nlimbs, q.b.nlimbs, q.a.rows, q.a.cols, q.b.cols, q.c.nlimbs, 0));
    }
    LimbBatchPlan lp;
    {
        std::vector<gbmm_mat> C, A, B;
        for (int j : queue_jobs) {
            C.push_back(jobs[j].c);
            A.push_back(jobs[j].a);
            B.push_back(jobs[j].b);
        }
        GBMM_TRY(plan_limb_batch(C, A, B, lp));
    }
    BatchState &bs = bstate(h);
    if (!bs.d_counter) GBMM_CUDA_TRY(cudaMalloc(&bs.d_counter, LimbBatchPlan::MAX_GROUPS * sizeof(int)));
    if (!bs.staged) GBMM_CUDA_TRY(cudaEventCreateWithFlags(&bs.staged, cudaEventDisableTiming));
    // one arena slice per side stream of the dispatched jobs, each large enough for
    // any of them, then the grouped products' region and the blob; the grouped
    // records take at most 4 KB per product
    const size_t slice = (ws + 65536 + 255) & ~(size_t)255;
    const int ns = nside_for(other.size());
    const size_t crt_blob_max = 4096 * grouped.size() + 4096;
    GBMM_TRY(arena_reserve(h, (size_t)std::max(ns, 1) * slice + gws + lp.blob.size() + crt_blob_max + 65536 + 1024));

    const std::string sig = bs.use_graphs ? job_signature(jobs, njobs, plans) : std::string();
    if (bs.use_graphs) {
        auto g = bs.graphs.find(sig);
        if (g != bs.graphs.end()) {
            count_launch(g->second.nkern);
            GBMM_CUDA_TRY(cudaGraphLaunch(g->second.exec, h->stream));
            return GBMM_OK;
        }
    }
    const bool capture = bs.use_graphs && h->stream != nullptr && bs.seen[sig]++ > 0;
    // Arena layout from the current mark: the dispatched jobs' slices, then the
    // grouped products' workspace (carved now, before any launch or capture: tables
    // and tensor maps are built here), then (eager calls) the blob.  The blob is
    // the work queue followed, 256-byte aligned, by the grouped CRT records.
    const size_t mark = arena_mark(h);
    const size_t base = ((mark + 255) & ~(size_t)255) + 256;
    std::unique_ptr<crt_group, void (*)(crt_group *)> grp(crt_group_create(), crt_group_destroy);
    h->ws.top = base + (size_t)std::max(ns, 1) * slice;
    for (int j : grouped) {
        gbmm_status st = crt_collect(h, grp.get(), jobs[j].c, jobs[j].a, jobs[j].b, plans[j]);
        if (st != GBMM_OK) {
            arena_release(h, mark);
            return st;
        }
    }
    std::vector<char> blob(lp.blob);
    size_t crt_off = 0;
    if (!crt_group_empty(grp.get())) {
        const std::vector<char> &cb = crt_group_blob(grp.get());
        crt_off = (blob.size() + 255) & ~(size_t)255;
        blob.resize(crt_off);
        blob.insert(blob.end(), cb.begin(), cb.end());
    }
    if (!capture) {
        // eager: the blob goes through pinned staging into the arena
        char *d_blob = nullptr;
        if (!blob.empty()) {
            GBMM_CUDA_TRY(cudaEventSynchronize(bs.staged));  // the previous copy out of the staging is done
            if (bs.h_cap < blob.size()) {
                if (bs.h_stage) GBMM_CUDA_TRY(cudaFreeHost(bs.h_stage));
                bs.h_stage = nullptr;
                bs.h_cap = 0;
                GBMM_CUDA_TRY(cudaHostAlloc((void **)&bs.h_stage, blob.size(), cudaHostAllocDefault));
                bs.h_cap = blob.size();
            }
            memcpy(bs.h_stage, blob.data(), blob.size());
            d_blob = (char *)arena_alloc(h, blob.size());
            if (!d_blob) {
                arena_release(h, mark);
                return set_error(GBMM_ERR_NOMEM, "batch work queue");
            }
            GBMM_CUDA_TRY(cudaMemcpyAsync(d_blob, bs.h_stage, blob.size(), cudaMemcpyHostToDevice, h->stream));
            GBMM_CUDA_TRY(cudaEventRecord(bs.staged, h->stream));
        }
        gbmm_status st = enqueue_batch(h, jobs, plans, lp, d_blob, other, slice, base, grp.get(), d_blob + crt_off);
        arena_release(h, mark);
        return st;
    }
    // capture: the blob gets its own device buffer, filled before capture begins
    GraphEntry ge;
    if (!blob.empty()) {
        cudaError_t e = cudaMalloc(&ge.d_blob, blob.size());
        gbmm_status su = e == cudaSuccess ? upload_now(ge.d_blob, blob.data(), blob.size()) : cuda_error(e, "batch blob");
        if (su != GBMM_OK) {
            cudaFree(ge.d_blob);
            arena_release(h, mark);
            return su;
        }
    }
    cudaGraph_t graph = nullptr;
    GBMM_CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    // the kernels captured are counted once here (the graph runs right after)
    const uint64_t k0 = gbmm_kernel_launches();
    gbmm_status st = enqueue_batch(h, jobs, plans, lp, ge.d_blob, other, slice, base, grp.get(), ge.d_blob + crt_off);
    ge.nkern = gbmm_kernel_launches() - k0;
    arena_release(h, mark);
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (st == GBMM_OK && e != cudaSuccess) st = cuda_error(e, "cudaStreamEndCapture");
    if (st == GBMM_OK) {
        e = cudaGraphInstantiate(&ge.exec, graph, 0);
        if (e != cudaSuccess) st = cuda_error(e, "cudaGraphInstantiate");
    }
    if (graph) cudaGraphDestroy(graph);
    if (st != GBMM_OK) {
        cudaFree(ge.d_blob);
        return st;
    }
    bs.graphs[sig] = ge;
    GBMM_CUDA_TRY(cudaGraphLaunch(ge.exec, h->stream));
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_set_graphs(gbmm_handle h, int32_t enable) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    bstate(h).use_graphs = enable != 0;
    if (!enable) invalidate_graphs(h);
    return GBMM_OK;
}

// ---- autotuner -----------------------------------------------------------------------------------
// Times candidate plans on each job's own buffers and keeps the fastest per
// shape class.  Each timing is also appended to `log` (if non-null) as one
// JSON object per line: the engine's record of its own timings, which the
// learned cost model trains on.
extern "C" gbmm_status gbmm_autotune(gbmm_handle h, const gbmm_job *jobs, int32_t njobs, int32_t repeats,
                                     const char *log_path) {
    if (!h || (njobs > 0 && !jobs)) return set_error(GBMM_ERR_INVALID, "null argument");
    BatchState &bs = bstate(h);
    FILE *log = log_path ? fopen(log_path, "a") : nullptr;
    cudaEvent_t e0, e1;
    GBMM_CUDA_TRY(cudaEventCreate(&e0));
    GBMM_CUDA_TRY(cudaEventCreate(&e1));
    gbmm_status st = GBMM_OK;
    for (int j = 0; j < njobs && st == GBMM_OK; j++) {
        const gbmm_job &q = jobs[j];
        const int m = q.a.rows, k = q.a.cols, n = q.b.cols, la = q.a.nlimbs, lb = q.b.nlimbs;
        if (!m || !k || !n) continue;
        float best = 1e30f;
        TuneEntry te{heuristic_plan(m, k, n, la, lb), 0.f};
        for (int id = 0; id < GBMM_NPLANS; id++) {
            const Plan cd = plan_of(id);
            // limb candidates with far more schoolbook work than any plan needs, Winograd
            // cutoffs that give no recursion and splits of one-limb operands are not run;
            // their timing stays unknown
            if (!plan_admissible(id, m, k, n, la, lb)) continue;
            gbmm_opts o;
            memset(&o, 0, sizeof o);
            o.plan = 1 + id;
            float tot = 0.f;
            bool ok = true;
            for (int r = 0; r <= repeats && ok; r++) {
                cudaEventRecord(e0, h->stream);
                gbmm_status s2 = gbmm_matmul(h, q.c, q.a, q.b, &o);
                cudaEventRecord(e1, h->stream);
                if (s2 != GBMM_OK) { ok = false; break; }
                if (cudaEventSynchronize(e1) != cudaSuccess) { ok = false; break; }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (r > 0) tot += ms;  // first run warms tables and workspace
            }
            if (check_device_error(h->stream) != GBMM_OK) ok = false;
            if (!ok) continue;
            const float ms = tot / std::max(1, repeats);
            if (log)
                fprintf(log,
                        "{\"m\": %d, \"k\": %d, \"n\": %d, \"la\": %d, \"lb\": %d, \"plan\": %d, \"path\": %d, "
                        "\"method\": %d, \"cutoff\": %d, \"tiles\": %d, \"split\": %d, \"ms\": %.6f}\n",
                        m, k, n, la, lb, id, cd.path, cd.method, cd.cutoff, cd.tiles, cd.split, ms);
            if (ms < best) {
                best = ms;
                te.plan = id;
                te.ms = ms;
            }
        }
        bs.tune[tune_key(m, k, n, la, lb)] = te;
    }
    if (log) fclose(log);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

extern "C" gbmm_status gbmm_tune_save(gbmm_handle h, const char *path) {
    if (!h || !path) return set_error(GBMM_ERR_INVALID, "null argument");
    FILE *f = fopen(path, "w");
    if (!f) return set_error(GBMM_ERR_INVALID, "cannot write %s", path);
    fprintf(f, "[\n");
    bool first = true;
    for (auto &kv : bstate(h).tune) {
        fprintf(f, "%s  {\"key\": %llu, \"plan\": %d, \"ms\": %.6f}", first ? "" : ",\n",
                (unsigned long long)kv.first, kv.second.plan, kv.second.ms);
        first = false;
    }
    fprintf(f, "\n]\n");
    fclose(f);
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_tune_load(gbmm_handle h, const char *path) {
    if (!h || !path) return set_error(GBMM_ERR_INVALID, "null argument");
    FILE *f = fopen(path, "r");
    if (!f) return set_error(GBMM_ERR_INVALID, "cannot read %s", path);
    char line[512];
    int loaded = 0;
    while (fgets(line, sizeof line, f)) {
        unsigned long long key = 0;
        int p = 0;
        float ms = 0.f;
        const char *q = strstr(line, "\"key\"");
        if (!q) continue;
        if (sscanf(q, "\"key\": %llu, \"plan\": %d, \"ms\": %f", &key, &p, &ms) == 3 && p >= 0 && p < GBMM_NPLANS) {
            bstate(h).tune[key] = TuneEntry{p, ms};
            loaded++;
        }
    }
    fclose(f);
    return loaded >= 0 ? GBMM_OK : set_error(GBMM_ERR_PARSE, "no entries in %s", path);
}
