// Products on host buffers, streamed through the GPU.
//
// The host link (NVLink-C2C on Grace, about 200 GB/s each way) moves a 512x512
// 4096-bit product's operands and result in about 2.7 ms, longer than the
// product itself.  gbmm_matmul_host therefore keeps two device slots and three
// streams: job j's host->device copies run on the upload stream while job j-1
// computes on the handle's stream and job j-2's result goes back on the
// download stream.  Each slot is reused only after the compute that read its
// operands and the copy that read its result have finished (events).
//
// The reference moves whole matrices host <-> device around each product with
// blocking copies (mat-gpu/mat-pregpu.cu:10-96, transfer_recurse); this is the
// overlapped replacement for a stream of independent products.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "gbmm_internal.h"

namespace gbmm {

namespace {
struct PipeSlot {
    uint32_t *a = nullptr, *b = nullptr, *c = nullptr;  // device limb planes
    int32_t *as = nullptr, *bs = nullptr, *cs = nullptr;
    size_t acap = 0, bcap = 0, ccap = 0;  // plane bytes allocated
    size_t ecap = 0;                      // entries allocated per sizes plane (max of A, B, C)
    cudaEvent_t uploaded = nullptr, computed = nullptr, downloaded = nullptr;
};
struct PipeState {
    cudaStream_t up = nullptr, down = nullptr;
    PipeSlot slot[2];
};

PipeState *pstate(gbmm_handle h) { return static_cast<PipeState *>(h->pipe); }

gbmm_status ck(cudaError_t e, const char *what) { return e == cudaSuccess ? GBMM_OK : cuda_error(e, what); }

void slot_free(PipeSlot &s) {
    cudaFree(s.a); cudaFree(s.b); cudaFree(s.c);
    cudaFree(s.as); cudaFree(s.bs); cudaFree(s.cs);
    s.a = s.b = s.c = nullptr;
    s.as = s.bs = s.cs = nullptr;
    s.acap = s.bcap = s.ccap = s.ecap = 0;
}

gbmm_status grow(void **p, size_t *cap, size_t need) {
    if (need <= *cap) return GBMM_OK;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    GBMM_CUDA_TRY(cudaMalloc(p, need));
    *cap = need;
    return GBMM_OK;
}

gbmm_status pipe_init(gbmm_handle h) {
    if (h->pipe) return GBMM_OK;
    PipeState *ps = new PipeState();
    h->pipe = ps;
    GBMM_CUDA_TRY(cudaStreamCreateWithFlags(&ps->up, cudaStreamNonBlocking));
    GBMM_CUDA_TRY(cudaStreamCreateWithFlags(&ps->down, cudaStreamNonBlocking));
    for (PipeSlot &s : ps->slot) {
        GBMM_CUDA_TRY(cudaEventCreateWithFlags(&s.uploaded, cudaEventDisableTiming));
        GBMM_CUDA_TRY(cudaEventCreateWithFlags(&s.computed, cudaEventDisableTiming));
        GBMM_CUDA_TRY(cudaEventCreateWithFlags(&s.downloaded, cudaEventDisableTiming));
    }
    return GBMM_OK;
}

gbmm_status check_job(const gbmm_host_job &q, int j) {
    if (q.K < 0 || q.M < 0 || q.N < 0 || q.a_nlimbs < 0 || q.b_nlimbs < 0 || q.c_nlimbs < 0)
        return set_error(GBMM_ERR_INVALID, "host job %d: negative dimension", j);
    if ((!q.a_sizes && (int64_t)q.K * q.M) || (!q.b_sizes && (int64_t)q.M * q.N) || (!q.c_sizes && (int64_t)q.K * q.N))
        return set_error(GBMM_ERR_INVALID, "host job %d: null sizes plane", j);
    if ((!q.a_limbs && q.a_nlimbs && (int64_t)q.K * q.M) || (!q.b_limbs && q.b_nlimbs && (int64_t)q.M * q.N) ||
        (!q.c_limbs && q.c_nlimbs && (int64_t)q.K * q.N))
        return set_error(GBMM_ERR_INVALID, "host job %d: null limb planes", j);
    return GBMM_OK;
}

gbmm_mat view(int32_t rows, int32_t cols, int32_t nl, uint32_t *limbs, int32_t *sizes) {
    gbmm_mat m;
    memset(&m, 0, sizeof m);
    m.rows = rows;
    m.cols = cols;
    m.nlimbs = nl;
    m.rs = cols;
    m.ld = (int64_t)rows * cols;
    m.limbs = limbs;
    m.sizes = sizes;
    return m;
}
}  // namespace

void pipe_destroy(gbmm_handle h) {
    PipeState *ps = pstate(h);
    if (!ps) return;
    if (ps->up) cudaStreamSynchronize(ps->up);
    if (ps->down) cudaStreamSynchronize(ps->down);
    for (PipeSlot &s : ps->slot) {
        slot_free(s);
        if (s.uploaded) cudaEventDestroy(s.uploaded);
        if (s.computed) cudaEventDestroy(s.computed);
        if (s.downloaded) cudaEventDestroy(s.downloaded);
    }
    if (ps->up) cudaStreamDestroy(ps->up);
    if (ps->down) cudaStreamDestroy(ps->down);
    delete ps;
    h->pipe = nullptr;
}

}  // namespace gbmm

using namespace gbmm;

extern "C" gbmm_status gbmm_matmul_host(gbmm_handle h, gbmm_host_job *jobs, int32_t njobs) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    if (njobs < 0 || (njobs > 0 && !jobs)) return set_error(GBMM_ERR_INVALID, "bad job list");
    for (int j = 0; j < njobs; j++) GBMM_TRY(check_job(jobs[j], j));
    GBMM_TRY(pipe_init(h));
    PipeState &ps = *pstate(h);

    // size both slots for the largest job; nothing may be in flight while they grow
    size_t an = 0, bn = 0, cn = 0, en = 1;
    for (int j = 0; j < njobs; j++) {
        const gbmm_host_job &q = jobs[j];
        an = std::max(an, (size_t)q.a_nlimbs * q.K * q.M * 4);
        bn = std::max(bn, (size_t)q.b_nlimbs * q.M * q.N * 4);
        cn = std::max(cn, (size_t)q.c_nlimbs * q.K * q.N * 4);
        en = std::max(en, std::max((size_t)q.K * q.M, std::max((size_t)q.M * q.N, (size_t)q.K * q.N)));
    }
    for (PipeSlot &s : ps.slot) {
        if (an > s.acap || bn > s.bcap || cn > s.ccap || en > s.ecap) {
            GBMM_CUDA_TRY(cudaStreamSynchronize(ps.up));
            GBMM_CUDA_TRY(cudaStreamSynchronize(ps.down));
            GBMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
        }
        GBMM_TRY(grow((void **)&s.a, &s.acap, std::max<size_t>(an, 256)));
        GBMM_TRY(grow((void **)&s.b, &s.bcap, std::max<size_t>(bn, 256)));
        GBMM_TRY(grow((void **)&s.c, &s.ccap, std::max<size_t>(cn, 256)));
        if (en > s.ecap) {
            cudaFree(s.as); cudaFree(s.bs); cudaFree(s.cs);
            s.as = s.bs = s.cs = nullptr;
            s.ecap = 0;
            GBMM_CUDA_TRY(cudaMalloc(&s.as, en * 4));
            GBMM_CUDA_TRY(cudaMalloc(&s.bs, en * 4));
            GBMM_CUDA_TRY(cudaMalloc(&s.cs, en * 4));
            s.ecap = en;
        }
    }

    gbmm_status st = GBMM_OK;
    for (int j = 0; j < njobs && st == GBMM_OK; j++) {
        gbmm_host_job &q = jobs[j];
        PipeSlot &s = ps.slot[j & 1];
        const size_t ea = (size_t)q.K * q.M, eb = (size_t)q.M * q.N, ec = (size_t)q.K * q.N;
        // uploads: the slot's operands are free once the compute two jobs back has run
        st = ck(cudaStreamWaitEvent(ps.up, s.computed, 0), "cudaStreamWaitEvent");
        if (st == GBMM_OK && ea) st = ck(cudaMemcpyAsync(s.as, q.a_sizes, ea * 4, cudaMemcpyHostToDevice, ps.up), "cudaMemcpyAsync");
        if (st == GBMM_OK && ea && q.a_nlimbs)
            st = ck(cudaMemcpyAsync(s.a, q.a_limbs, (size_t)q.a_nlimbs * ea * 4, cudaMemcpyHostToDevice, ps.up),
                            "cudaMemcpyAsync");
        if (st == GBMM_OK && eb) st = ck(cudaMemcpyAsync(s.bs, q.b_sizes, eb * 4, cudaMemcpyHostToDevice, ps.up), "cudaMemcpyAsync");
        if (st == GBMM_OK && eb && q.b_nlimbs)
            st = ck(cudaMemcpyAsync(s.b, q.b_limbs, (size_t)q.b_nlimbs * eb * 4, cudaMemcpyHostToDevice, ps.up),
                            "cudaMemcpyAsync");
        if (st == GBMM_OK) st = ck(cudaEventRecord(s.uploaded, ps.up), "cudaEventRecord");
        // compute: after this job's uploads and after the slot's previous result left
        if (st == GBMM_OK) st = ck(cudaStreamWaitEvent(h->stream, s.uploaded, 0), "cudaStreamWaitEvent");
        if (st == GBMM_OK) st = ck(cudaStreamWaitEvent(h->stream, s.downloaded, 0), "cudaStreamWaitEvent");
        if (st != GBMM_OK) break;
        gbmm_mat A = view(q.K, q.M, q.a_nlimbs, s.a, s.as), B = view(q.M, q.N, q.b_nlimbs, s.b, s.bs),
                 C = view(q.K, q.N, q.c_nlimbs, s.c, s.cs);
        gbmm_opts o;
        memset(&o, 0, sizeof o);
        o.path = q.path;
        o.method = q.method ? q.method : GBMM_METHOD_WINOGRAD;
        o.cutoff = q.cutoff;
        o.nprimes = q.nprimes;
        Plan p;
        st = resolve_plan(h, A, B, o, p);
        if (st != GBMM_OK) break;
        q.chosen_path = p.path;
        st = gbmm_matmul(h, C, A, B, &o);
        if (st == GBMM_OK) st = ck(cudaEventRecord(s.computed, h->stream), "cudaEventRecord");
        // download
        if (st == GBMM_OK) st = ck(cudaStreamWaitEvent(ps.down, s.computed, 0), "cudaStreamWaitEvent");
        if (st == GBMM_OK && ec) st = ck(cudaMemcpyAsync(q.c_sizes, s.cs, ec * 4, cudaMemcpyDeviceToHost, ps.down), "cudaMemcpyAsync");
        if (st == GBMM_OK && ec && q.c_nlimbs)
            st = ck(cudaMemcpyAsync(q.c_limbs, s.c, (size_t)q.c_nlimbs * ec * 4, cudaMemcpyDeviceToHost, ps.down),
                            "cudaMemcpyAsync");
        if (st == GBMM_OK) st = ck(cudaEventRecord(s.downloaded, ps.down), "cudaEventRecord");
    }
    // drain all three streams whatever happened, then report the first error
    const cudaError_t e1 = cudaStreamSynchronize(ps.up), e2 = cudaStreamSynchronize(h->stream),
                      e3 = cudaStreamSynchronize(ps.down);
    if (st != GBMM_OK) return st;
    GBMM_TRY(ck(e1, "upload stream"));
    GBMM_TRY(ck(e2, "compute stream"));
    GBMM_TRY(ck(e3, "download stream"));
    return check_device_error(h->stream);
}
