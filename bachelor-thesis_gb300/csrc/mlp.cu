// Learned cost model for the dispatcher: an 8 -> 64 -> 64 -> GBMM_NPLANS MLP
// with BF16 weights and FP32 accumulation.  Its heads predict log2(milliseconds)
// of each candidate plan for one product (gbmm_plan: the limb kernel alone,
// Winograd trees of three cutoffs, i.e. recursion depths, CRT with three GEMM
// tile forms and CRT after a limb-half split, i.e. fewer moduli per product);
// GBMM_PATH_AUTO runs the cheapest trusted one.
//
// Training runs on the GPU with the kernels below (forward, backward with
// FP32 gradient accumulation, Adam on FP32 master weights that are rounded to
// BF16 after every step).  Data: the JSON-lines timings gbmm_autotune records.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gbmm_internal.h"

namespace gbmm {

namespace {
constexpr int NF = 8, NH = 64, NO = GBMM_NPLANS;
constexpr int NW1 = NF * NH, NW2 = NH * NH, NW3 = NH * NO;
constexpr int NPARAM = NW1 + NH + NW2 + NH + NW3 + NO;  // weights then biases per layer
constexpr int OFF_W1 = 0, OFF_B1 = NW1, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NW2, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NW3;
constexpr int MLP_THREADS = 128;
}  // namespace

struct Model {
    std::vector<float> master;            // FP32 master parameters (host copy)
    std::vector<__nv_bfloat16> w16;       // BF16 parameters used by inference (host copy)
    float *d_master = nullptr, *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr;
    __nv_bfloat16 *d_w16 = nullptr;
    int step = 0;
    // measured targets each head has trained on (gbmm_model_train); a head with
    // fewer than MIN_HEAD_SAMPLES is not consulted.  Parameters set from outside
    // count as trained.
    int head_samples[NO] = {};
};
constexpr int MIN_HEAD_SAMPLES = 8;
// the model overrides the plain heuristic's plan only when it predicts at least
// this much gain (log2 of 1.10): switches between plans whose costs differ by
// less than the model's own error would be noise
constexpr float OVERRIDE_MARGIN_LOG2 = 0.1375f;

// Features of one product (all scaled to roughly unit range).
__host__ __device__ inline void job_features(int m, int k, int n, int la, int lb, float *f) {
    const float l2m = log2f((float)(m > 0 ? m : 1)), l2k = log2f((float)(k > 0 ? k : 1)),
                l2n = log2f((float)(n > 0 ? n : 1)), l2a = log2f(32.f * (la > 0 ? la : 1)),
                l2b = log2f(32.f * (lb > 0 ? lb : 1));
    f[0] = l2m / 10.f;
    f[1] = l2k / 10.f;
    f[2] = l2n / 10.f;
    f[3] = l2a / 14.f;
    f[4] = l2b / 14.f;
    f[5] = (l2m + l2k + l2n + l2a + l2b - 10.f) / 50.f;  // log2 of the schoolbook work
    f[6] = fabsf(l2a - l2b) / 8.f;                         // bit-length imbalance
    f[7] = fabsf(l2m - l2n) / 8.f;                         // aspect ratio
}

// ---- kernels ------------------------------------------------------------------------------
// One thread per sample; the BF16 weights are staged in shared memory and every
// dot product accumulates in FP32.  Activations are kept for the backward pass.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_forward(const __nv_bfloat16 *w, const float *X, int nsamp,
                                                             float *H1, float *H2, float *Y) {
    __shared__ float sw[NPARAM];
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sw[i] = __bfloat162float(w[i]);
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsamp) return;
    float x[NF], h1[NH], h2[NH];
#pragma unroll
    for (int i = 0; i < NF; i++) x[i] = X[(int64_t)s * NF + i];
    for (int j = 0; j < NH; j++) {
        float a = sw[OFF_B1 + j];
#pragma unroll
        for (int i = 0; i < NF; i++) a += x[i] * sw[OFF_W1 + i * NH + j];
        h1[j] = a > 0.f ? a : 0.f;
    }
    for (int j = 0; j < NH; j++) {
        float a = sw[OFF_B2 + j];
        for (int i = 0; i < NH; i++) a += h1[i] * sw[OFF_W2 + i * NH + j];
        h2[j] = a > 0.f ? a : 0.f;
    }
    for (int o = 0; o < NO; o++) {
        float a = sw[OFF_B3 + o];
        for (int i = 0; i < NH; i++) a += h2[i] * sw[OFF_W3 + i * NO + o];
        Y[(int64_t)s * NO + o] = a;
    }
    if (H1)
        for (int j = 0; j < NH; j++) H1[(int64_t)s * NH + j] = h1[j];
    if (H2)
        for (int j = 0; j < NH; j++) H2[(int64_t)s * NH + j] = h2[j];
}

// Mean-squared-error gradient of all parameters over nsamp samples; the
// targets T may be NaN for heads without a measurement (masked out).  Each
// CTA sums its samples' contributions in shared memory, then adds them to the
// global FP32 gradient with atomics.  loss receives sum of squared errors / count.
// Backward pass in two kernels, with no atomics on the gradient: k_mlp_delta gives
// every sample's error terms (one thread per sample), k_mlp_wgrad sums them into
// each parameter's gradient (one thread per parameter, a loop over the samples).
// The sums run in sample order, so the gradient is the same on every run.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_delta(const __nv_bfloat16 *w, const float *T, const float *H1,
                                                           const float *H2, const float *Y, int nsamp,
                                                           float inv_count, float *D1, float *D2, float *D3,
                                                           float *loss) {
    __shared__ float sw[NW2 + NW3];  // W2 and W3, the weights the error terms pass back through
    for (int i = threadIdx.x; i < NW2 + NW3; i += blockDim.x)
        sw[i] = __bfloat162float(w[i < NW2 ? OFF_W2 + i : OFF_W3 + (i - NW2)]);
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    float lsum = 0.f;
    if (s < nsamp) {
        float dy[NO], dh2[NH];
        for (int o = 0; o < NO; o++) {
            const float t = T[(int64_t)s * NO + o];
            const float e = isnan(t) ? 0.f : Y[(int64_t)s * NO + o] - t;
            lsum += e * e;
            dy[o] = 2.f * e * inv_count;
            D3[(int64_t)s * NO + o] = dy[o];
        }
        for (int i = 0; i < NH; i++) {
            float a = 0.f;
            for (int o = 0; o < NO; o++) a += dy[o] * sw[NW2 + i * NO + o];
            dh2[i] = H2[(int64_t)s * NH + i] > 0.f ? a : 0.f;
            D2[(int64_t)s * NH + i] = dh2[i];
        }
        for (int i = 0; i < NH; i++) {
            float a = 0.f;
            for (int j = 0; j < NH; j++) a += dh2[j] * sw[i * NH + j];
            D1[(int64_t)s * NH + i] = H1[(int64_t)s * NH + i] > 0.f ? a : 0.f;
        }
    }
    // warp-reduce the loss, one atomic per warp
    for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, lsum * inv_count);
}

// grad[p] for every parameter p: a weight from unit i into unit j of the next layer
// sums (input activation i) x (error term j) over the samples; a bias sums error j.
__global__ void k_mlp_wgrad(const float *X, const float *H1, const float *H2, const float *D1, const float *D2,
                            const float *D3, int nsamp, float *grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const float *in = nullptr, *d;
    int nin = 0, nd, i = 0, j;
    if (p < OFF_B1) {
        in = X; nin = NF; d = D1; nd = NH; i = p / NH; j = p % NH;
    } else if (p < OFF_W2) {
        d = D1; nd = NH; j = p - OFF_B1;
    } else if (p < OFF_B2) {
        in = H1; nin = NH; d = D2; nd = NH; i = (p - OFF_W2) / NH; j = (p - OFF_W2) % NH;
    } else if (p < OFF_W3) {
        d = D2; nd = NH; j = p - OFF_B2;
    } else if (p < OFF_B3) {
        in = H2; nin = NH; d = D3; nd = NO; i = (p - OFF_W3) / NO; j = (p - OFF_W3) % NO;
    } else {
        d = D3; nd = NO; j = p - OFF_B3;
    }
    float g = 0.f;
    if (in) {
        for (int s = 0; s < nsamp; s++) g += in[(int64_t)s * nin + i] * d[(int64_t)s * nd + j];
    } else {
        for (int s = 0; s < nsamp; s++) g += d[(int64_t)s * nd + j];
    }
    grad[p] = g;
}

// Adam step on the FP32 master parameters; the BF16 copy is refreshed.
__global__ void k_mlp_adam(float *master, float *m, float *v, const float *grad, __nv_bfloat16 *w16, float lr,
                           float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float p = master[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    master[i] = p;
    w16[i] = __float2bfloat16_rn(p);
}

// ---- host --------------------------------------------------------------------------------------
static Model *model_of(gbmm_handle h) { return static_cast<Model *>(h->model); }

void model_destroy(gbmm_handle h) {
    Model *md = model_of(h);
    if (!md) return;
    cudaFree(md->d_master);
    cudaFree(md->d_m);
    cudaFree(md->d_v);
    cudaFree(md->d_grad);
    cudaFree(md->d_w16);
    delete md;
    h->model = nullptr;
}

static gbmm_status model_alloc(gbmm_handle h, Model **out) {
    Model *md = model_of(h);
    if (md) { *out = md; return GBMM_OK; }
    md = new Model();
    md->master.assign(NPARAM, 0.f);
    md->w16.assign(NPARAM, __float2bfloat16_rn(0.f));
    if (cudaMalloc(&md->d_master, NPARAM * 4) != cudaSuccess || cudaMalloc(&md->d_m, NPARAM * 4) != cudaSuccess ||
        cudaMalloc(&md->d_v, NPARAM * 4) != cudaSuccess || cudaMalloc(&md->d_grad, NPARAM * 4) != cudaSuccess ||
        cudaMalloc(&md->d_w16, NPARAM * 2) != cudaSuccess) {
        h->model = md;
        model_destroy(h);
        return set_error(GBMM_ERR_NOMEM, "model buffers");
    }
    h->model = md;
    *out = md;
    return GBMM_OK;
}

static gbmm_status model_upload(Model *md) {
    for (int i = 0; i < NPARAM; i++) md->w16[i] = __float2bfloat16_rn(md->master[i]);
    GBMM_TRY(upload_now(md->d_master, md->master.data(), NPARAM * 4));
    GBMM_TRY(upload_now(md->d_w16, md->w16.data(), NPARAM * 2));
    GBMM_TRY(fill_now(md->d_m, 0, NPARAM * 4));
    GBMM_TRY(fill_now(md->d_v, 0, NPARAM * 4));
    md->step = 0;
    return GBMM_OK;
}

// Host forward pass with the same BF16 weights and FP32 accumulation order as
// k_mlp_forward (used for single-product dispatch, which must not synchronise).
static void host_forward(const Model *md, const float *x, float *y) {
    float w[NPARAM];
    for (int i = 0; i < NPARAM; i++) w[i] = __bfloat162float(md->w16[i]);
    float h1[NH], h2[NH];
    for (int j = 0; j < NH; j++) {
        float a = w[OFF_B1 + j];
        for (int i = 0; i < NF; i++) a += x[i] * w[OFF_W1 + i * NH + j];
        h1[j] = a > 0.f ? a : 0.f;
    }
    for (int j = 0; j < NH; j++) {
        float a = w[OFF_B2 + j];
        for (int i = 0; i < NH; i++) a += h1[i] * w[OFF_W2 + i * NH + j];
        h2[j] = a > 0.f ? a : 0.f;
    }
    for (int o = 0; o < NO; o++) {
        float a = w[OFF_B3 + o];
        for (int i = 0; i < NH; i++) a += h2[i] * w[OFF_W3 + i * NO + o];
        y[o] = a;
    }
}

int model_choose(gbmm_handle h, int m, int k, int n, int la, int lb) {
    const Model *md = model_of(h);
    if (!md) return -1;
    float f[NF], y[NO];
    job_features(m, k, n, la, lb, f);
    host_forward(md, f, y);
    // only plans the autotuner would have timed for this product, with heads that
    // trained on enough timings: anything else is an extrapolation, not a prediction
    int best = -1;
    for (int o = 0; o < NO; o++) {
        if (!plan_admissible(o, m, k, n, la, lb) || md->head_samples[o] < MIN_HEAD_SAMPLES) continue;
        if (best < 0 || y[o] < y[best]) best = o;
    }
    const int base = heuristic_plan(m, k, n, la, lb);
    if (best < 0 || best == base) return base;
    if (md->head_samples[base] >= MIN_HEAD_SAMPLES && y[best] > y[base] - OVERRIDE_MARGIN_LOG2) return base;
    return best;
}

}  // namespace gbmm

using namespace gbmm;

// ---- C ABI -------------------------------------------------------------------------------------------
extern "C" int32_t gbmm_model_nparams(void) { return NPARAM; }

extern "C" gbmm_status gbmm_model_features(int32_t m, int32_t k, int32_t n, int32_t la, int32_t lb, float *out8) {
    if (!out8) return set_error(GBMM_ERR_INVALID, "null pointer");
    job_features(m, k, n, la, lb, out8);
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_model_init(gbmm_handle h, uint64_t seed) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    Model *md = nullptr;
    GBMM_TRY(model_alloc(h, &md));
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
    auto rnd = [&]() {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        return (double)(st >> 11) / 9007199254740992.0;
    };
    auto fill = [&](int off, int cnt, int fan_in) {
        const double sc = sqrt(6.0 / fan_in);  // He-uniform for ReLU layers
        for (int i = 0; i < cnt; i++) md->master[off + i] = (float)((2.0 * rnd() - 1.0) * sc);
    };
    fill(OFF_W1, NW1, NF);
    fill(OFF_W2, NW2, NH);
    fill(OFF_W3, NW3, NH);
    for (int i = 0; i < NH; i++) md->master[OFF_B1 + i] = md->master[OFF_B2 + i] = 0.f;
    for (int i = 0; i < NO; i++) md->master[OFF_B3 + i] = 0.f;
    for (int o = 0; o < NO; o++) md->head_samples[o] = 0;  // untrained heads are not consulted
    return model_upload(md);
}

extern "C" gbmm_status gbmm_model_set_params(gbmm_handle h, const float *params) {
    if (!h || !params) return set_error(GBMM_ERR_INVALID, "null argument");
    Model *md = nullptr;
    GBMM_TRY(model_alloc(h, &md));
    memcpy(md->master.data(), params, NPARAM * 4);
    for (int o = 0; o < NO; o++) md->head_samples[o] = MIN_HEAD_SAMPLES;  // parameters given count as trained
    return model_upload(md);
}

extern "C" gbmm_status gbmm_model_get_params(gbmm_handle h, float *master, uint16_t *bf16_params) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    Model *md = model_of(h);
    if (!md) return set_error(GBMM_ERR_INVALID, "no model");
    if (master) memcpy(master, md->master.data(), NPARAM * 4);
    if (bf16_params) memcpy(bf16_params, md->w16.data(), NPARAM * 2);
    return GBMM_OK;
}

extern "C" gbmm_status gbmm_model_use(gbmm_handle h, int32_t enable) {
    if (!h) return set_error(GBMM_ERR_INVALID, "null handle");
    if (enable && !h->model) return set_error(GBMM_ERR_INVALID, "no model loaded");
    h->use_model = enable != 0;
    return GBMM_OK;
}

// Forward pass on the GPU for nsamp feature rows (host arrays in and out).
extern "C" gbmm_status gbmm_model_predict(gbmm_handle h, const float *X, int32_t nsamp, float *Y) {
    if (!h || (nsamp > 0 && (!X || !Y))) return set_error(GBMM_ERR_INVALID, "null argument");
    Model *md = model_of(h);
    if (!md) return set_error(GBMM_ERR_INVALID, "no model");
    if (nsamp == 0) return GBMM_OK;
    float *dX = nullptr, *dY = nullptr;
    GBMM_CUDA_TRY(cudaMalloc(&dX, (size_t)nsamp * NF * 4));
    GBMM_CUDA_TRY(cudaMalloc(&dY, (size_t)nsamp * NO * 4));
    cudaStream_t s = h->stream;
    gbmm_status st = GBMM_OK;
    cudaError_t e = cudaMemcpyAsync(dX, X, (size_t)nsamp * NF * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        LaunchScope ls_("k_mlp_forward", s);
        k_mlp_forward<<<(nsamp + MLP_THREADS - 1) / MLP_THREADS, MLP_THREADS, 0, s>>>(md->d_w16, dX, nsamp, nullptr,
                                                                                       nullptr, dY);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(Y, dY, (size_t)nsamp * NO * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_error(e, "model predict");
    cudaFree(dX);
    cudaFree(dY);
    return st;
}

// Backward pass: per-sample error terms, then every parameter's gradient into d_grad.
static cudaError_t launch_backward(Model *md, const float *dX, const float *dT, const float *dH1, const float *dH2,
                                   const float *dY, float *dD1, float *dD2, float *dD3, int nsamp, int count, float *dL,
                                   cudaStream_t s) {
    const int grid = (nsamp + MLP_THREADS - 1) / MLP_THREADS;
    {
        LaunchScope ls_("k_mlp_delta", s);
        k_mlp_delta<<<grid, MLP_THREADS, 0, s>>>(md->d_w16, dT, dH1, dH2, dY, nsamp, 1.f / (float)std::max(count, 1),
                                                 dD1, dD2, dD3, dL);
    }
    {
        LaunchScope ls_("k_mlp_wgrad", s);
        k_mlp_wgrad<<<(NPARAM + 127) / 128, 128, 0, s>>>(dX, dH1, dH2, dD1, dD2, dD3, nsamp, md->d_grad);
    }
    return cudaGetLastError();
}

// Loss and parameter gradient of the current model on (X, T) (host arrays;
// T rows may hold NaN for missing heads).  grad receives NPARAM floats.
extern "C" gbmm_status gbmm_model_gradient(gbmm_handle h, const float *X, const float *T, int32_t nsamp, float *grad,
                                           float *loss) {
    if (!h || nsamp <= 0 || !X || !T) return set_error(GBMM_ERR_INVALID, "bad argument");
    Model *md = model_of(h);
    if (!md) return set_error(GBMM_ERR_INVALID, "no model");
    cudaStream_t s = h->stream;
    float *buf = nullptr;
    const size_t nX = (size_t)nsamp * NF, nT = (size_t)nsamp * NO, nH = (size_t)nsamp * NH;
    GBMM_CUDA_TRY(cudaMalloc(&buf, (nX + nT + 2 * nH + nT + 1 + 2 * nH + nT) * 4));
    float *dX = buf, *dT = dX + nX, *dH1 = dT + nT, *dH2 = dH1 + nH, *dY = dH2 + nH, *dL = dY + nT;
    float *dD1 = dL + 1, *dD2 = dD1 + nH, *dD3 = dD2 + nH;  // error terms per sample
    int count = 0;
    for (size_t i = 0; i < nT; i++) count += !std::isnan(T[i]);
    gbmm_status st = GBMM_OK;
    cudaError_t e = cudaMemcpyAsync(dX, X, nX * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dT, T, nT * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(md->d_grad, 0, NPARAM * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dL, 0, 4, s);
    const int grid = (nsamp + MLP_THREADS - 1) / MLP_THREADS;
    if (e == cudaSuccess) {
        {
            LaunchScope ls_("k_mlp_forward", s);
            k_mlp_forward<<<grid, MLP_THREADS, 0, s>>>(md->d_w16, dX, nsamp, dH1, dH2, dY);
        }
        e = launch_backward(md, dX, dT, dH1, dH2, dY, dD1, dD2, dD3, nsamp, count, dL, s);
    }
    if (e == cudaSuccess && grad) e = cudaMemcpyAsync(grad, md->d_grad, NPARAM * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, dL, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_error(e, "model gradient");
    cudaFree(buf);
    return st;
}

// Full-batch Adam training for `epochs` steps on (X, T); returns the final loss.
extern "C" gbmm_status gbmm_model_train(gbmm_handle h, const float *X, const float *T, int32_t nsamp, int32_t epochs,
                                        float lr, float *final_loss) {
    if (!h || nsamp <= 0 || !X || !T || epochs < 0) return set_error(GBMM_ERR_INVALID, "bad argument");
    Model *md = model_of(h);
    if (!md) return set_error(GBMM_ERR_INVALID, "no model (gbmm_model_init first)");
    cudaStream_t s = h->stream;
    float *buf = nullptr;
    const size_t nX = (size_t)nsamp * NF, nT = (size_t)nsamp * NO, nH = (size_t)nsamp * NH;
    GBMM_CUDA_TRY(cudaMalloc(&buf, (nX + nT + 2 * nH + nT + 1 + 2 * nH + nT) * 4));
    float *dX = buf, *dT = dX + nX, *dH1 = dT + nT, *dH2 = dH1 + nH, *dY = dH2 + nH, *dL = dY + nT;
    float *dD1 = dL + 1, *dD2 = dD1 + nH, *dD3 = dD2 + nH;  // error terms per sample
    int count = 0;
    for (size_t i = 0; i < nT; i++) count += !std::isnan(T[i]);
    for (int o = 0; o < NO; o++)
        for (int i = 0; i < nsamp; i++) md->head_samples[o] += !std::isnan(T[(size_t)i * NO + o]);
    cudaError_t e = cudaMemcpyAsync(dX, X, nX * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dT, T, nT * 4, cudaMemcpyHostToDevice, s);
    const int grid = (nsamp + MLP_THREADS - 1) / MLP_THREADS;
    const float b1 = 0.9f, b2 = 0.999f;
    for (int ep = 0; ep < epochs && e == cudaSuccess; ep++) {
        e = cudaMemsetAsync(dL, 0, 4, s);
        {
            LaunchScope ls_("k_mlp_forward", s);
            k_mlp_forward<<<grid, MLP_THREADS, 0, s>>>(md->d_w16, dX, nsamp, dH1, dH2, dY);
        }
        if (e == cudaSuccess) e = launch_backward(md, dX, dT, dH1, dH2, dY, dD1, dD2, dD3, nsamp, count, dL, s);
        md->step++;
        const float c1 = 1.f - powf(b1, (float)md->step), c2 = 1.f - powf(b2, (float)md->step);
        {
            LaunchScope ls_("k_mlp_adam", s);
            k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, s>>>(md->d_master, md->d_m, md->d_v, md->d_grad, md->d_w16, lr,
                                                            b1, b2, 1e-8f, c1, c2);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    float lossv = 0.f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&lossv, dL, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(md->master.data(), md->d_master, NPARAM * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(md->w16.data(), md->d_w16, NPARAM * 2, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_error(e, "model train");
    if (final_loss) *final_loss = lossv;
    return GBMM_OK;
}
