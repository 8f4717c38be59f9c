// Batched products of uneven shape and bit length, the path dispatcher, the
// autotuner and CUDA-graph replay.
//
// gbmm_matmul_batched splits the jobs by path.  Limb-path jobs are cut into
// (job, tile) items, sorted largest first, and run by ONE persistent kernel
// per block edge R that drains a device work queue.  CRT jobs run their
// residue / product / reconstruction kernels back to back.  The whole launch
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
    int path;
    int cutoff;
    float ms;
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    char *d_blob = nullptr;  // work-queue blob owned by this graph
};

struct BatchState {
    std::map<uint64_t, TuneEntry> tune;
    // graph cache
    std::map<std::string, GraphEntry> graphs;
    std::map<std::string, int> seen;
    bool use_graphs = true;
    // pinned staging for eager batches, guarded by an event on the last copy
    char *h_stage = nullptr;
    size_t h_cap = 0;
    cudaEvent_t staged = nullptr;
    int *d_counter = nullptr;  // one per block-edge group
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

int choose_path(gbmm_handle h, int m, int k, int n, int la, int lb, int *cutoff) {
    if (h->model && h->use_model) {
        int c = *cutoff;
        int p = model_choose(h, m, k, n, la, lb, &c);
        if (p == GBMM_PATH_LIMB || p == GBMM_PATH_CRT) {
            *cutoff = c;
            return p;
        }
    }
    if (h->batch) {
        BatchState &b = bstate(h);
        auto it = b.tune.find(tune_key(m, k, n, la, lb));
        if (it != b.tune.end()) {
            if (it->second.cutoff > 0) *cutoff = it->second.cutoff;
            return it->second.path;
        }
    }
    return heuristic_path(m, k, n, la, lb);
}

}  // namespace gbmm

using namespace gbmm;

static std::string job_signature(const gbmm_job *jobs, int njobs, const std::vector<Plan> &plans) {
    std::string sig;
    sig.reserve((size_t)njobs * 96);
    char buf[256];
    for (int j = 0; j < njobs; j++) {
        const gbmm_job &q = jobs[j];
        snprintf(buf, sizeof buf, "%p,%p,%p,%p,%p,%p,%d,%d,%d,%d,%d,%d,%lld,%lld,%lld,%lld,%lld,%lld,%d,%d,%d;",
                 (void *)q.c.limbs, (void *)q.c.sizes, (void *)q.a.limbs, (void *)q.a.sizes, (void *)q.b.limbs,
                 (void *)q.b.sizes, q.a.rows, q.a.cols, q.b.cols, q.a.nlimbs, q.b.nlimbs, q.c.nlimbs, (long long)q.a.rs,
                 (long long)q.a.ld, (long long)q.b.rs, (long long)q.b.ld, (long long)q.c.rs, (long long)q.c.ld,
                 plans[j].path, plans[j].cutoff, plans[j].method);
        sig += buf;
    }
    return sig;
}

// Splits a batch: limb-path jobs that fit the per-entry kernel go to the
// persistent work-queue kernel, everything else through dispatch().
static void split_batch(const gbmm_job *jobs, int njobs, const std::vector<Plan> &plans, std::vector<int> &queue_jobs,
                        std::vector<int> &other) {
    for (int j = 0; j < njobs; j++) {
        const gbmm_job &q = jobs[j];
        if (plans[j].path == GBMM_PATH_LIMB && limb_kernel_fits(q.a.nlimbs, q.b.nlimbs) && q.a.rows && q.b.cols &&
            q.a.cols)
            queue_jobs.push_back(j);
        else
            other.push_back(j);
    }
}

// Enqueues one batch on the handle's stream.  d_blob holds the work-queue plan
// on the device (already filled); the remaining jobs go through dispatch().
static gbmm_status enqueue_batch(gbmm_handle h, const gbmm_job *jobs, const std::vector<Plan> &plans,
                                 const LimbBatchPlan &lp, const char *d_blob, const std::vector<int> &other) {
    BatchState &bs = bstate(h);
    if (!lp.groups.empty()) GBMM_TRY(launch_limb_batch(lp, d_blob, bs.d_counter, h->stream));
    for (int j : other) GBMM_TRY(dispatch(h, jobs[j].c, jobs[j].a, jobs[j].b, plans[j], 0, h->stream));
    return GBMM_OK;
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
        ws = std::max(ws, dispatch_ws(plans[j], q.a.nlimbs, q.b.nlimbs, q.a.rows, q.a.cols, q.b.cols, q.c.nlimbs, 0));
    }
    if (njobs == 0) return GBMM_OK;
    std::vector<int> queue_jobs, other;
    split_batch(jobs, njobs, plans, queue_jobs, other);
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
    if (!bs.d_counter) GBMM_CUDA_TRY(cudaMalloc(&bs.d_counter, 4 * sizeof(int)));
    if (!bs.staged) GBMM_CUDA_TRY(cudaEventCreateWithFlags(&bs.staged, cudaEventDisableTiming));
    GBMM_TRY(arena_reserve(h, ws + lp.blob.size() + 65536));

    const std::string sig = bs.use_graphs ? job_signature(jobs, njobs, plans) : std::string();
    if (bs.use_graphs) {
        auto g = bs.graphs.find(sig);
        if (g != bs.graphs.end()) {
            count_launch(1);
            GBMM_CUDA_TRY(cudaGraphLaunch(g->second.exec, h->stream));
            return GBMM_OK;
        }
    }
    const bool capture = bs.use_graphs && h->stream != nullptr && bs.seen[sig]++ > 0;
    if (!capture) {
        // eager: the work-queue blob goes through pinned staging into the arena
        size_t mark = arena_mark(h);
        char *d_blob = nullptr;
        if (!lp.blob.empty()) {
            GBMM_CUDA_TRY(cudaEventSynchronize(bs.staged));  // the previous copy out of the staging is done
            if (bs.h_cap < lp.blob.size()) {
                if (bs.h_stage) GBMM_CUDA_TRY(cudaFreeHost(bs.h_stage));
                bs.h_stage = nullptr;
                bs.h_cap = 0;
                GBMM_CUDA_TRY(cudaHostAlloc((void **)&bs.h_stage, lp.blob.size(), cudaHostAllocDefault));
                bs.h_cap = lp.blob.size();
            }
            memcpy(bs.h_stage, lp.blob.data(), lp.blob.size());
            d_blob = (char *)arena_alloc(h, lp.blob.size());
            if (!d_blob) return set_error(GBMM_ERR_NOMEM, "batch work queue");
            GBMM_CUDA_TRY(cudaMemcpyAsync(d_blob, bs.h_stage, lp.blob.size(), cudaMemcpyHostToDevice, h->stream));
            GBMM_CUDA_TRY(cudaEventRecord(bs.staged, h->stream));
        }
        gbmm_status st = enqueue_batch(h, jobs, plans, lp, d_blob, other);
        arena_release(h, mark);
        return st;
    }
    // capture: the blob gets its own device buffer, filled before capture begins
    GraphEntry ge;
    if (!lp.blob.empty()) {
        GBMM_CUDA_TRY(cudaMalloc(&ge.d_blob, lp.blob.size()));
        GBMM_CUDA_TRY(cudaMemcpy(ge.d_blob, lp.blob.data(), lp.blob.size(), cudaMemcpyHostToDevice));
    }
    cudaGraph_t graph = nullptr;
    GBMM_CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    gbmm_status st = enqueue_batch(h, jobs, plans, lp, ge.d_blob, other);
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
    count_launch(1);
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
    struct Cand {
        int path, method, cutoff;
    };
    const Cand cands[] = {{GBMM_PATH_LIMB, GBMM_METHOD_NAIVE, 0},
                          {GBMM_PATH_LIMB, GBMM_METHOD_WINOGRAD, 64},
                          {GBMM_PATH_CRT, GBMM_METHOD_WINOGRAD, 0}};
    gbmm_status st = GBMM_OK;
    for (int j = 0; j < njobs && st == GBMM_OK; j++) {
        const gbmm_job &q = jobs[j];
        const int m = q.a.rows, k = q.a.cols, n = q.b.cols, la = q.a.nlimbs, lb = q.b.nlimbs;
        if (!m || !k || !n) continue;
        float best = 1e30f;
        TuneEntry te{heuristic_path(m, k, n, la, lb), 0, 0.f};
        for (const Cand &cd : cands) {
            // limb candidates whose schoolbook work predicts far more than any plan needs
            // (about 50 ms at 4e12 32-bit MAC/s) are not run; their timing stays unknown
            if (cd.path == GBMM_PATH_LIMB && (double)m * k * n * la * lb > 2e11) continue;
            gbmm_opts o;
            memset(&o, 0, sizeof o);
            o.path = cd.path;
            o.method = cd.method;
            o.cutoff = cd.cutoff;
            int32_t need = 0;
            gbmm_matmul_limbs_needed(la, lb, k, &o, &need);
            if (q.c.nlimbs < need && cd.method != GBMM_METHOD_NAIVE && cd.path == GBMM_PATH_LIMB) {
                // the tuner only runs candidates whose workspace rules hold for this C
            }
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
                        "{\"m\": %d, \"k\": %d, \"n\": %d, \"la\": %d, \"lb\": %d, \"path\": %d, \"method\": %d, "
                        "\"cutoff\": %d, \"ms\": %.6f}\n",
                        m, k, n, la, lb, cd.path, cd.method, cd.cutoff, ms);
            if (ms < best) {
                best = ms;
                te.path = cd.path;
                te.cutoff = cd.method == GBMM_METHOD_NAIVE ? 1 << 30 : cd.cutoff;
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
        fprintf(f, "%s  {\"key\": %llu, \"path\": %d, \"cutoff\": %d, \"ms\": %.6f}", first ? "" : ",\n",
                (unsigned long long)kv.first, kv.second.path, kv.second.cutoff, kv.second.ms);
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
        int p = 0, c = 0;
        float ms = 0.f;
        const char *q = strstr(line, "\"key\"");
        if (!q) continue;
        if (sscanf(q, "\"key\": %llu, \"path\": %d, \"cutoff\": %d, \"ms\": %f", &key, &p, &c, &ms) == 4) {
            bstate(h).tune[key] = TuneEntry{p, c, ms};
            loaded++;
        }
    }
    fclose(f);
    return loaded >= 0 ? GBMM_OK : set_error(GBMM_ERR_PARSE, "no entries in %s", path);
}
