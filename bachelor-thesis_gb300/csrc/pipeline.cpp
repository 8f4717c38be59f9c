// Products on host buffers, streamed through the GPU.
//
// The host link (NVLink-C2C on Grace, about 200 GB/s each way) moves a 512x512
// 4096-bit product's operands and result in about 2.7 ms, longer than the
// product itself.  gbmm_matmul_host therefore keeps two device slots and three
// streams: job j's host->device copies run on the upload stream while job j-1
// computes on the handle's stream and job j-2's result goes back on the
// download stream.  Each slot is reused only after the compute that read its
// operands and the copy that read its result have finished (events).  A
// single-pass CRT product starts on A while B is still uploading, and the call's
// last product goes back in entry ranges as its reconstruction finishes them
// (crt_stage_hooks).
//
// The reference moves whole matrices host <-> device around each product with
// blocking copies (mat-gpu/mat-pregpu.cu:10-96, transfer_recurse); this is the
// overlapped replacement for a stream of independent products.
//
// A product whose device footprint exceeds the handle's device budget (free
// memory by default) runs out of core: C is cut into row x column blocks and the
// inner dimension into chunks; each block accumulates its chunk products on the
// device (C_blk += A_rows,chunk * B_chunk,cols) and goes back to the host once.
// Sub-blocks move with 2-D copies straight from and to the host planes, two A/B
// slots and two C blocks keep copies and compute overlapped.  The reference
// recurses on the host instead (Winograd above 512, mat-gpu/mat-pregpu.cu:273-467,
// with additions on host memory); here the host only moves blocks and every
// addition happens on the device.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "gbmm_internal.h"

namespace gbmm {

namespace {
struct PipeSlot {
    uint32_t *a = nullptr, *b = nullptr, *c = nullptr;  // device limb planes
    int32_t *as = nullptr, *bs = nullptr, *cs = nullptr;
    size_t acap = 0, bcap = 0, ccap = 0;  // plane bytes allocated
    size_t ecap = 0;                      // entries allocated per sizes plane (max of A, B, C)
    cudaEvent_t a_uploaded = nullptr, uploaded = nullptr, computed = nullptr, downloaded = nullptr;
};
struct PipeState {
    cudaStream_t up = nullptr, down = nullptr;
    PipeSlot slot[2];
    cudaEvent_t part[CRT_MAX_PARTS] = {};  // reconstruction ranges of the call's last product
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
    for (cudaEvent_t &e : ps->part) GBMM_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (PipeSlot &s : ps->slot) {
        GBMM_CUDA_TRY(cudaEventCreateWithFlags(&s.a_uploaded, cudaEventDisableTiming));
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
std::atomic<int64_t> g_last_blocks{0};  // block products of the last out-of-core call (test hook)

// host sub-block (rows r0.., cols c0..) of dense planes with plane stride hld and
// row stride hrs <-> dense device planes (rows x cols per plane)
gbmm_status copy_block(uint32_t *dev, uint32_t *host, int64_t hld, int64_t hrs, int r0, int c0, int rows, int cols,
                       int nl, bool up, cudaStream_t s) {
    if (!rows || !cols) return GBMM_OK;
    for (int i = 0; i < nl; i++) {
        uint32_t *d = dev + (int64_t)i * rows * cols, *hp = host + (int64_t)i * hld + (int64_t)r0 * hrs + c0;
        const cudaError_t e =
            up ? cudaMemcpy2DAsync(d, (size_t)cols * 4, hp, (size_t)hrs * 4, (size_t)cols * 4, rows, cudaMemcpyHostToDevice, s)
               : cudaMemcpy2DAsync(hp, (size_t)hrs * 4, d, (size_t)cols * 4, (size_t)cols * 4, rows, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_error(e, "cudaMemcpy2DAsync");
    }
    return GBMM_OK;
}

gbmm_opts job_opts(const gbmm_host_job &q) {
    gbmm_opts o;
    memset(&o, 0, sizeof o);
    o.path = q.path;
    o.method = q.method ? q.method : GBMM_METHOD_WINOGRAD;
    o.cutoff = q.cutoff;
    o.nprimes = q.nprimes;
    return o;
}

// device bytes of one block step: two A and B slots, two C blocks, the product's workspace
size_t block_footprint(gbmm_handle h, const gbmm_host_job &q, int kb, int mt, int nb) {
    gbmm_mat A = view(kb, mt, q.a_nlimbs, nullptr, nullptr), B = view(mt, nb, q.b_nlimbs, nullptr, nullptr);
    Plan p;
    gbmm_opts o = job_opts(q);
    if (resolve_plan(h, A, B, o, p) != GBMM_OK) return (size_t)-1;
    const size_t ws = dispatch_ws(p, q.a_nlimbs, q.b_nlimbs, kb, mt, nb, q.c_nlimbs, 1);
    return 2 * 4 * ((size_t)kb * mt * (q.a_nlimbs + 1) + (size_t)mt * nb * (q.b_nlimbs + 1) +
                    (size_t)kb * nb * (q.c_nlimbs + 1)) +
           ws + ((size_t)4 << 20);
}

size_t device_budget(gbmm_handle h) {
    if (h->dev_budget) return h->dev_budget;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return (size_t)-1;
    return fr / 10 * 9 + h->ws.cap;  // the arena can be reused
}

// One product too large for the device, in blocks (see the file comment).
gbmm_status run_blocked(gbmm_handle h, PipeState &ps, gbmm_host_job &q, size_t budget) {
    int kb = q.K, mt = q.M, nb = q.N;
    while (block_footprint(h, q, kb, mt, nb) > budget) {
        int *d = &kb;
        if (nb > *d) d = &nb;
        if (mt > *d) d = &mt;
        if (*d <= 16) return set_error(GBMM_ERR_NOMEM, "product does not fit the device budget even in 16x16x16 blocks");
        *d = (*d + 1) / 2;
    }
    const int la = q.a_nlimbs, lb = q.b_nlimbs, lc = q.c_nlimbs;
    {
        gbmm_mat A = view(kb, mt, la, nullptr, nullptr), B = view(mt, nb, lb, nullptr, nullptr);
        Plan p;
        gbmm_opts o = job_opts(q);
        GBMM_TRY(resolve_plan(h, A, B, o, p));
        q.chosen_path = p.path;
    }
    struct Bufs {
        uint32_t *a[2] = {}, *b[2] = {}, *c[2] = {};
        int32_t *as[2] = {}, *bs[2] = {}, *cs[2] = {};
        cudaEvent_t up[2] = {}, comp[2] = {}, down[2] = {}, cdone = nullptr;
    } bf;
    gbmm_status st = GBMM_OK;
    auto alloc = [&](void **p, size_t n) {
        if (st == GBMM_OK && cudaMalloc(p, std::max<size_t>(n, 256)) != cudaSuccess)
            st = set_error(GBMM_ERR_NOMEM, "out-of-core block buffers");
    };
    for (int i = 0; i < 2; i++) {
        alloc((void **)&bf.a[i], (size_t)kb * mt * la * 4);
        alloc((void **)&bf.b[i], (size_t)mt * nb * lb * 4);
        alloc((void **)&bf.c[i], (size_t)kb * nb * lc * 4);
        alloc((void **)&bf.as[i], (size_t)kb * mt * 4);
        alloc((void **)&bf.bs[i], (size_t)mt * nb * 4);
        alloc((void **)&bf.cs[i], (size_t)kb * nb * 4);
        if (st == GBMM_OK) st = ck(cudaEventCreateWithFlags(&bf.up[i], cudaEventDisableTiming), "cudaEventCreate");
        if (st == GBMM_OK) st = ck(cudaEventCreateWithFlags(&bf.comp[i], cudaEventDisableTiming), "cudaEventCreate");
        if (st == GBMM_OK) st = ck(cudaEventCreateWithFlags(&bf.down[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    if (st == GBMM_OK) st = ck(cudaEventCreateWithFlags(&bf.cdone, cudaEventDisableTiming), "cudaEventCreate");
    const gbmm_opts o0 = job_opts(q);
    int64_t blk = 0, cblk = 0;
    for (int r0 = 0; r0 < q.K && st == GBMM_OK; r0 += kb) {
        for (int c0 = 0; c0 < q.N && st == GBMM_OK; c0 += nb, cblk++) {
            const int kr = std::min(kb, q.K - r0), nc = std::min(nb, q.N - c0), cs = (int)(cblk & 1);
            // the C block is free once its previous contents reached the host
            st = ck(cudaStreamWaitEvent(h->stream, bf.down[cs], 0), "cudaStreamWaitEvent");
            for (int t0 = 0; st == GBMM_OK && (t0 < q.M || t0 == 0); t0 += mt, blk++) {
                const int mk = std::min(mt, q.M - t0), s = (int)(blk & 1);
                st = ck(cudaStreamWaitEvent(ps.up, bf.comp[s], 0), "cudaStreamWaitEvent");
                if (st == GBMM_OK)
                    st = copy_block(bf.a[s], const_cast<uint32_t *>(q.a_limbs), (int64_t)q.K * q.M, q.M, r0, t0, kr, mk,
                                    la, true, ps.up);
                if (st == GBMM_OK)
                    st = copy_block((uint32_t *)bf.as[s], (uint32_t *)const_cast<int32_t *>(q.a_sizes), 0, q.M, r0, t0,
                                    kr, mk, 1, true, ps.up);
                if (st == GBMM_OK)
                    st = copy_block(bf.b[s], const_cast<uint32_t *>(q.b_limbs), (int64_t)q.M * q.N, q.N, t0, c0, mk, nc,
                                    lb, true, ps.up);
                if (st == GBMM_OK)
                    st = copy_block((uint32_t *)bf.bs[s], (uint32_t *)const_cast<int32_t *>(q.b_sizes), 0, q.N, t0, c0,
                                    mk, nc, 1, true, ps.up);
                if (st == GBMM_OK) st = ck(cudaEventRecord(bf.up[s], ps.up), "cudaEventRecord");
                if (st == GBMM_OK) st = ck(cudaStreamWaitEvent(h->stream, bf.up[s], 0), "cudaStreamWaitEvent");
                if (st != GBMM_OK) break;
                gbmm_opts o = o0;
                o.accumulate = t0 > 0;
                st = gbmm_matmul(h, view(kr, nc, lc, bf.c[cs], bf.cs[cs]), view(kr, mk, la, bf.a[s], bf.as[s]),
                                 view(mk, nc, lb, bf.b[s], bf.bs[s]), &o);
                if (st == GBMM_OK) st = ck(cudaEventRecord(bf.comp[s], h->stream), "cudaEventRecord");
                if (q.M == 0) break;
            }
            // the finished block goes back to the host on the download stream
            if (st == GBMM_OK) st = ck(cudaEventRecord(bf.cdone, h->stream), "cudaEventRecord");
            if (st == GBMM_OK) st = ck(cudaStreamWaitEvent(ps.down, bf.cdone, 0), "cudaStreamWaitEvent");
            if (st == GBMM_OK) st = copy_block(bf.c[cs], q.c_limbs, (int64_t)q.K * q.N, q.N, r0, c0, kr, nc, lc, false, ps.down);
            if (st == GBMM_OK)
                st = copy_block((uint32_t *)bf.cs[cs], (uint32_t *)q.c_sizes, 0, q.N, r0, c0, kr, nc, 1, false, ps.down);
            if (st == GBMM_OK) st = ck(cudaEventRecord(bf.down[cs], ps.down), "cudaEventRecord");
        }
    }
    cudaStreamSynchronize(ps.up);
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(ps.down);
    for (int i = 0; i < 2; i++) {
        cudaFree(bf.a[i]); cudaFree(bf.b[i]); cudaFree(bf.c[i]);
        cudaFree(bf.as[i]); cudaFree(bf.bs[i]); cudaFree(bf.cs[i]);
        if (bf.up[i]) cudaEventDestroy(bf.up[i]);
        if (bf.comp[i]) cudaEventDestroy(bf.comp[i]);
        if (bf.down[i]) cudaEventDestroy(bf.down[i]);
    }
    if (bf.cdone) cudaEventDestroy(bf.cdone);
    g_last_blocks += blk;
    return st;
}
}  // namespace

void pipe_destroy(gbmm_handle h) {
    PipeState *ps = pstate(h);
    if (!ps) return;
    if (ps->up) cudaStreamSynchronize(ps->up);
    if (ps->down) cudaStreamSynchronize(ps->down);
    for (cudaEvent_t e : ps->part)
        if (e) cudaEventDestroy(e);
    for (PipeSlot &s : ps->slot) {
        slot_free(s);
        if (s.a_uploaded) cudaEventDestroy(s.a_uploaded);
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
    g_last_blocks = 0;

    // products whose two-slot footprint exceeds the device budget run out of core
    const size_t budget = device_budget(h);
    std::vector<char> blocked(njobs, 0);
    for (int j = 0; j < njobs; j++) blocked[j] = block_footprint(h, jobs[j], jobs[j].K, jobs[j].M, jobs[j].N) > budget;

    // size both slots for the largest in-core job; nothing may be in flight while they grow
    size_t an = 0, bn = 0, cn = 0, en = 1;
    for (int j = 0; j < njobs; j++) {
        if (blocked[j]) continue;
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
        if (blocked[j]) {
            // drain the in-core pipeline, then run this product in blocks
            st = ck(cudaStreamSynchronize(ps.up), "upload stream");
            if (st == GBMM_OK) st = ck(cudaStreamSynchronize(h->stream), "compute stream");
            if (st == GBMM_OK) st = ck(cudaStreamSynchronize(ps.down), "download stream");
            if (st == GBMM_OK) st = run_blocked(h, ps, q, budget);
            continue;
        }
        PipeSlot &s = ps.slot[j & 1];
        const size_t ea = (size_t)q.K * q.M, eb = (size_t)q.M * q.N, ec = (size_t)q.K * q.N;
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
        // a single-pass CRT product starts on A while B is still uploading, and the call's
        // last product returns C in entry ranges as its reconstruction finishes them
        const bool staged = p.path == GBMM_PATH_CRT && crt_feasible(q.a_nlimbs, q.b_nlimbs, q.M) &&
                            crt_single_pass(q.M) && ec > 0 && q.M > 0;
        bool last = true;
        for (int j2 = j + 1; j2 < njobs; j2++) last = last && blocked[j2];
        // uploads: the slot's operands are free once the compute two jobs back has run
        st = ck(cudaStreamWaitEvent(ps.up, s.computed, 0), "cudaStreamWaitEvent");
        if (st == GBMM_OK && ea) st = ck(cudaMemcpyAsync(s.as, q.a_sizes, ea * 4, cudaMemcpyHostToDevice, ps.up), "cudaMemcpyAsync");
        if (st == GBMM_OK && ea && q.a_nlimbs)
            st = ck(cudaMemcpyAsync(s.a, q.a_limbs, (size_t)q.a_nlimbs * ea * 4, cudaMemcpyHostToDevice, ps.up),
                            "cudaMemcpyAsync");
        if (st == GBMM_OK) st = ck(cudaEventRecord(s.a_uploaded, ps.up), "cudaEventRecord");
        if (st == GBMM_OK && eb) st = ck(cudaMemcpyAsync(s.bs, q.b_sizes, eb * 4, cudaMemcpyHostToDevice, ps.up), "cudaMemcpyAsync");
        if (st == GBMM_OK && eb && q.b_nlimbs)
            st = ck(cudaMemcpyAsync(s.b, q.b_limbs, (size_t)q.b_nlimbs * eb * 4, cudaMemcpyHostToDevice, ps.up),
                            "cudaMemcpyAsync");
        if (st == GBMM_OK) st = ck(cudaEventRecord(s.uploaded, ps.up), "cudaEventRecord");
        // compute: after this job's uploads (A's only, when staged) and after the slot's
        // previous result left
        if (st == GBMM_OK)
            st = ck(cudaStreamWaitEvent(h->stream, staged ? s.a_uploaded : s.uploaded, 0), "cudaStreamWaitEvent");
        if (st == GBMM_OK) st = ck(cudaStreamWaitEvent(h->stream, s.downloaded, 0), "cudaStreamWaitEvent");
        if (st != GBMM_OK) break;
        crt_stage_hooks hooks;
        if (staged) {
            hooks.b_ready = s.uploaded;
            hooks.parts = last ? CRT_MAX_PARTS : 1;
            for (int i = 0; i < CRT_MAX_PARTS; i++) hooks.part_ev[i] = ps.part[i];
            h->stage = &hooks;
        }
        // the plan resolved above runs as is, so the staging decision and the product agree
        st = arena_reserve(h, dispatch_ws(p, q.a_nlimbs, q.b_nlimbs, q.K, q.M, q.N, q.c_nlimbs, 0) + 65536);
        if (st == GBMM_OK) st = dispatch(h, C, A, B, p, 0, h->stream);
        h->stage = nullptr;
        if (st == GBMM_OK) st = ck(cudaEventRecord(s.computed, h->stream), "cudaEventRecord");
        // download: the whole of C after the compute, or each finished entry range
        const int nparts = hooks.parts_done;
        int64_t e0 = 0;
        for (int pi = 0; pi < std::max(nparts, 1) && st == GBMM_OK; pi++) {
            const int64_t e1 = nparts ? std::min<int64_t>(hooks.part_end[pi], (int64_t)ec) : (int64_t)ec;
            st = ck(cudaStreamWaitEvent(ps.down, nparts ? ps.part[pi] : s.computed, 0), "cudaStreamWaitEvent");
            if (st == GBMM_OK && e1 > e0)
                st = ck(cudaMemcpyAsync(q.c_sizes + e0, s.cs + e0, (size_t)(e1 - e0) * 4, cudaMemcpyDeviceToHost, ps.down),
                        "cudaMemcpyAsync");
            if (st == GBMM_OK && e1 > e0 && q.c_nlimbs)
                st = ck(cudaMemcpy2DAsync(q.c_limbs + e0, ec * 4, s.c + e0, ec * 4, (size_t)(e1 - e0) * 4, q.c_nlimbs,
                                          cudaMemcpyDeviceToHost, ps.down),
                        "cudaMemcpy2DAsync");
            e0 = std::max(e0, e1);
        }
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

extern "C" gbmm_status gbmm_set_device_budget(gbmm_handle h, uint64_t bytes) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    h->dev_budget = (size_t)bytes;
    return GBMM_OK;
}

// Internal test hook (not part of the public ABI): block products run out of core by
// the last gbmm_matmul_host call.
extern "C" int64_t gbmmx_host_blocks(void) { return g_last_blocks.load(); }
