// Learned Radau15 predictor: training and inference kernels (see mlp.cuh).
//
// Training runs a minibatch as CTAs of 64 samples.  Each CTA keeps its
// activations in shared memory twice (row-major and transposed, BF16), so
// every GEMM of the forward and backward pass is a plain A * B^T over
// row-major operands fed to mma.sync; weights come from global memory in
// both layouts.  Each CTA writes its parameter gradient; a second kernel
// sums them in CTA order (deterministic), applies Adam to the FP32 master
// weights and refreshes the BF16 copies.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "abi_state.cuh"
#include "ensemble.cuh"
#include "mlp.cuh"

namespace abie {

namespace {

constexpr int TR = 64;  // samples per CTA
constexpr int TT = 128; // threads per CTA
// padded strides (elements) of the shared-memory operands
constexpr int LD_IN = MLP_IN + 8, LD_HID = MLP_HID + 8, LD_OUT = MLP_OUT_PAD + 8, LD_R = TR + 8;

struct MlpState {
    float *master = nullptr, *adam_m = nullptr, *adam_v = nullptr;  // N_PARAMS each
    __nv_bfloat16 *w = nullptr;                                    // W1 W2 W3 W1t W2t W3t
    float *grad_partial = nullptr;
    int grad_cap = 0;  // CTAs
    float *loss_partial = nullptr;
    float *samples = nullptr;  // device sample store
    long long sample_cap = 0, n_samples = 0;
    int *idx = nullptr;
    long long idx_cap = 0;
    long long adam_t = 0;
    float tau[7] = {1, 1, 1, 1, 1, 1, 1};
    bool ready = false, enabled = false;
    LearnedPredictor view = {};
    LearnedPredictor *view_dev = nullptr;
};
MlpState g_mlp;

__nv_bfloat16 *w1(MlpState &s) { return s.w; }
__nv_bfloat16 *w2(MlpState &s) { return s.w + MLP_HID * MLP_IN; }
__nv_bfloat16 *w3(MlpState &s) { return s.w + MLP_HID * MLP_IN + MLP_HID * MLP_HID; }
__nv_bfloat16 *w1t(MlpState &s) { return s.w + MLP_N_PARAMS; }
__nv_bfloat16 *w2t(MlpState &s) { return w1t(s) + MLP_HID * MLP_IN; }
__nv_bfloat16 *w3t(MlpState &s) { return w2t(s) + MLP_HID * MLP_HID; }

struct TrainSmem {
    __nv_bfloat16 X[TR * LD_IN], XT[MLP_IN * LD_R];
    __nv_bfloat16 A1[TR * LD_HID], A1T[MLP_HID * LD_R];
    __nv_bfloat16 A2[TR * LD_HID], A2T[MLP_HID * LD_R];
    __nv_bfloat16 dY[TR * LD_OUT], dYT[MLP_OUT_PAD * LD_R];
    __nv_bfloat16 dZ2[TR * LD_HID], dZ2T[MLP_HID * LD_R];
    __nv_bfloat16 dZ1T[MLP_HID * LD_R];
    float loss[TT];
};

// Forward of one CTA tile of rows into shared memory; returns nothing.
// Y (pre-bias-added outputs) are handed to the epilogue functor.
template <typename YEpi>
__device__ void forward_tile(TrainSmem &S, const LearnedPredictor &P, YEpi yepi)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // layer 1: [TR x 32] x [32 x 128]
    for (int tile = warp; tile < (TR / 16) * (MLP_HID / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_HID / 8)) * 16, n0 = (tile % (MLP_HID / 8)) * 8;
        float c[4];
        mma_tile(S.X, LD_IN, P.W1, MLP_IN, m0, n0, MLP_IN, c);
        for (int e = 0; e < 4; e++) {
            int r = m0 + g + (e >> 1) * 8, n = n0 + 2 * t + (e & 1);
            float h = fmaxf(c[e] + P.b1[n], 0.0f);
            __nv_bfloat16 hb = __float2bfloat16_rn(h);
            S.A1[r * LD_HID + n] = hb;
            S.A1T[n * LD_R + r] = hb;
        }
    }
    __syncthreads();
    // layer 2: [TR x 128] x [128 x 128]
    for (int tile = warp; tile < (TR / 16) * (MLP_HID / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_HID / 8)) * 16, n0 = (tile % (MLP_HID / 8)) * 8;
        float c[4];
        mma_tile(S.A1, LD_HID, P.W2, MLP_HID, m0, n0, MLP_HID, c);
        for (int e = 0; e < 4; e++) {
            int r = m0 + g + (e >> 1) * 8, n = n0 + 2 * t + (e & 1);
            float h = fmaxf(c[e] + P.b2[n], 0.0f);
            __nv_bfloat16 hb = __float2bfloat16_rn(h);
            S.A2[r * LD_HID + n] = hb;
            S.A2T[n * LD_R + r] = hb;
        }
    }
    __syncthreads();
    // layer 3: [TR x 128] x [128 x 32]
    for (int tile = warp; tile < (TR / 16) * (MLP_OUT_PAD / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_OUT_PAD / 8)) * 16, n0 = (tile % (MLP_OUT_PAD / 8)) * 8;
        float c[4];
        mma_tile(S.A2, LD_HID, P.W3, MLP_HID, m0, n0, MLP_HID, c);
        for (int e = 0; e < 4; e++) {
            int r = m0 + g + (e >> 1) * 8, n = n0 + 2 * t + (e & 1);
            yepi(r, n, c[e] + P.b3[n]);
        }
    }
    __syncthreads();
}

__device__ void load_rows(TrainSmem &S, const float *samples, const int *idx, long long row0,
                          long long rows)
{
    for (int e = threadIdx.x; e < TR * MLP_IN; e += TT) {
        int r = e / MLP_IN, k = e % MLP_IN;
        long long gr = row0 + r;
        float v = 0.0f;
        if (gr < rows) {
            long long sid = idx ? idx[gr] : gr;
            v = samples[sid * MLP_SAMPLE + k];
        }
        __nv_bfloat16 b = __float2bfloat16_rn(v);
        S.X[r * LD_IN + k] = b;
        S.XT[k * LD_R + r] = b;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(TT) mlp_forward_kernel(LearnedPredictor P, const float *samples,
                                                          long long rows, float *Y)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
    const long long row0 = (long long)blockIdx.x * TR;
    load_rows(S, samples, nullptr, row0, rows);
    forward_tile(S, P, [&](int r, int n, float y) {
        if (row0 + r < rows) Y[(row0 + r) * MLP_OUT_PAD + n] = y;
    });
}

__global__ void __launch_bounds__(TT) mlp_grad_kernel(LearnedPredictor P, const float *samples,
                                                       const int *idx, long long rows,
                                                       float inv_count, float *grad_partial,
                                                       float *loss_partial)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long row0 = (long long)blockIdx.x * TR;
    float *G = grad_partial + (size_t)blockIdx.x * MLP_N_PARAMS;
    load_rows(S, samples, idx, row0, rows);
    float my_loss = 0.0f;
    forward_tile(S, P, [&](int r, int n, float y) {
        float dy = 0.0f;
        long long gr = row0 + r;
        if (gr < rows && n < MLP_OUT) {
            long long sid = idx ? idx[gr] : gr;
            float d = y - samples[sid * MLP_SAMPLE + MLP_IN + n];
            my_loss += d * d;
            dy = 2.0f * d * inv_count;
        }
        __nv_bfloat16 b = __float2bfloat16_rn(dy);
        S.dY[r * LD_OUT + n] = b;
        S.dYT[n * LD_R + r] = b;
    });
    S.loss[threadIdx.x] = my_loss;
    __syncthreads();
    // dW3 [32 x 128] = dY^T A2
    for (int tile = warp; tile < (MLP_OUT_PAD / 16) * (MLP_HID / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_HID / 8)) * 16, n0 = (tile % (MLP_HID / 8)) * 8;
        float c[4];
        mma_tile(S.dYT, LD_R, S.A2T, LD_R, m0, n0, TR, c);
        for (int e = 0; e < 4; e++) {
            int o = m0 + g + (e >> 1) * 8, h = n0 + 2 * t + (e & 1);
            G[MLP_OFF_W3 + o * MLP_HID + h] = c[e];
        }
    }
    // dA2 [TR x 128] = dY W3, dZ2 = dA2 * relu'
    for (int tile = warp; tile < (TR / 16) * (MLP_HID / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_HID / 8)) * 16, n0 = (tile % (MLP_HID / 8)) * 8;
        float c[4];
        mma_tile(S.dY, LD_OUT, P.W3t, MLP_OUT_PAD, m0, n0, MLP_OUT_PAD, c);
        for (int e = 0; e < 4; e++) {
            int r = m0 + g + (e >> 1) * 8, h = n0 + 2 * t + (e & 1);
            float dz = (__bfloat162float(S.A2[r * LD_HID + h]) > 0.0f) ? c[e] : 0.0f;
            __nv_bfloat16 b = __float2bfloat16_rn(dz);
            S.dZ2[r * LD_HID + h] = b;
            S.dZ2T[h * LD_R + r] = b;
        }
    }
    __syncthreads();
    // dW2 [128 x 128] = dZ2^T A1
    for (int tile = warp; tile < (MLP_HID / 16) * (MLP_HID / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_HID / 8)) * 16, n0 = (tile % (MLP_HID / 8)) * 8;
        float c[4];
        mma_tile(S.dZ2T, LD_R, S.A1T, LD_R, m0, n0, TR, c);
        for (int e = 0; e < 4; e++) {
            int o = m0 + g + (e >> 1) * 8, h = n0 + 2 * t + (e & 1);
            G[MLP_OFF_W2 + o * MLP_HID + h] = c[e];
        }
    }
    // dA1 [TR x 128] = dZ2 W2, dZ1 = dA1 * relu'
    for (int tile = warp; tile < (TR / 16) * (MLP_HID / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_HID / 8)) * 16, n0 = (tile % (MLP_HID / 8)) * 8;
        float c[4];
        mma_tile(S.dZ2, LD_HID, P.W2t, MLP_HID, m0, n0, MLP_HID, c);
        for (int e = 0; e < 4; e++) {
            int r = m0 + g + (e >> 1) * 8, h = n0 + 2 * t + (e & 1);
            float dz = (__bfloat162float(S.A1[r * LD_HID + h]) > 0.0f) ? c[e] : 0.0f;
            S.dZ1T[h * LD_R + r] = __float2bfloat16_rn(dz);
        }
    }
    __syncthreads();
    // dW1 [128 x 32] = dZ1^T X
    for (int tile = warp; tile < (MLP_HID / 16) * (MLP_IN / 8); tile += TT / 32) {
        int m0 = (tile / (MLP_IN / 8)) * 16, n0 = (tile % (MLP_IN / 8)) * 8;
        float c[4];
        mma_tile(S.dZ1T, LD_R, S.XT, LD_R, m0, n0, TR, c);
        for (int e = 0; e < 4; e++) {
            int o = m0 + g + (e >> 1) * 8, i = n0 + 2 * t + (e & 1);
            G[MLP_OFF_W1 + o * MLP_IN + i] = c[e];
        }
    }
    // bias gradients: column sums of the BF16 deltas, in row order
    for (int n = threadIdx.x; n < MLP_HID; n += TT) {
        float s1 = 0.0f, s2 = 0.0f;
        for (int r = 0; r < TR; r++) {
            s1 += __bfloat162float(S.dZ1T[n * LD_R + r]);
            s2 += __bfloat162float(S.dZ2[r * LD_HID + n]);
        }
        G[MLP_OFF_B1 + n] = s1;
        G[MLP_OFF_B2 + n] = s2;
    }
    for (int n = threadIdx.x; n < MLP_OUT_PAD; n += TT) {
        float s3 = 0.0f;
        for (int r = 0; r < TR; r++) s3 += __bfloat162float(S.dY[r * LD_OUT + n]);
        G[MLP_OFF_B3 + n] = s3;
    }
    if (threadIdx.x == 0) {
        float L = 0.0f;
        for (int k = 0; k < TT; k++) L += S.loss[k];
        loss_partial[blockIdx.x] = L;
    }
}

// Sum of the CTA gradients in CTA order; optional Adam step; refresh the
// BF16 copies (row-major and transposed).
__global__ void mlp_update_kernel(float *master, float *am, float *av, __nv_bfloat16 *w,
                                  const float *grad_partial, int ctas, float *grad_out, int adam,
                                  float lr, float b1c, float b2c)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= MLP_N_PARAMS) return;
    float g = 0.0f;
    for (int c = 0; c < ctas; c++) g += grad_partial[(size_t)c * MLP_N_PARAMS + p];
    if (grad_out) grad_out[p] = g;
    float v = master[p];
    if (adam) {
        const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
        float mm = beta1 * am[p] + (1.0f - beta1) * g;
        float vv = beta2 * av[p] + (1.0f - beta2) * g * g;
        am[p] = mm;
        av[p] = vv;
        v -= lr * (mm / b1c) / (sqrtf(vv / b2c) + eps);
        master[p] = v;
    }
    __nv_bfloat16 b = __float2bfloat16_rn(v);
    __nv_bfloat16 *wt = w + MLP_N_PARAMS;
    if (p < MLP_OFF_B1) {
        int o = p / MLP_IN, i = p % MLP_IN;
        w[o * MLP_IN + i] = b;
        wt[i * MLP_HID + o] = b;
    } else if (p >= MLP_OFF_W2 && p < MLP_OFF_B2) {
        int q = p - MLP_OFF_W2, o = q / MLP_HID, i = q % MLP_HID;
        w[MLP_HID * MLP_IN + o * MLP_HID + i] = b;
        wt[MLP_HID * MLP_IN + i * MLP_HID + o] = b;
    } else if (p >= MLP_OFF_W3 && p < MLP_OFF_B3) {
        int q = p - MLP_OFF_W3, o = q / MLP_HID, i = q % MLP_HID;
        w[MLP_HID * MLP_IN + MLP_HID * MLP_HID + o * MLP_HID + i] = b;
        wt[MLP_HID * MLP_IN + MLP_HID * MLP_HID + i * MLP_OUT_PAD + o] = b;
    }
}

int mlp_alloc()
{
    MlpState &s = g_mlp;
    if (s.master) return 0;
    ABIE_CUDA(cudaMalloc(&s.master, MLP_N_PARAMS * sizeof(float)));
    ABIE_CUDA(cudaMalloc(&s.adam_m, MLP_N_PARAMS * sizeof(float)));
    ABIE_CUDA(cudaMalloc(&s.adam_v, MLP_N_PARAMS * sizeof(float)));
    ABIE_CUDA(cudaMalloc(&s.w, 2 * MLP_N_PARAMS * sizeof(__nv_bfloat16)));
    ABIE_CUDA(cudaMalloc(&s.view_dev, sizeof(LearnedPredictor)));
    ABIE_CUDA(cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sizeof(TrainSmem)));
    ABIE_CUDA(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sizeof(TrainSmem)));
    return 0;
}

int mlp_refresh(cudaStream_t st)
{
    MlpState &s = g_mlp;
    // no gradient, no Adam: just rebuild the BF16 copies from the master
    if (s.grad_cap < 1) {
        if (s.grad_partial) cudaFree(s.grad_partial);
        ABIE_CUDA(cudaMalloc(&s.grad_partial, MLP_N_PARAMS * sizeof(float)));
        s.grad_cap = 1;
    }
    ABIE_CUDA(cudaMemsetAsync(s.grad_partial, 0, MLP_N_PARAMS * sizeof(float), st));
    mlp_update_kernel<<<(MLP_N_PARAMS + 255) / 256, 256, 0, st>>>(
        s.master, s.adam_m, s.adam_v, s.w, s.grad_partial, 1, nullptr, 0, 0.f, 1.f, 1.f);
    ABIE_CUDA(cudaGetLastError());
    LearnedPredictor &v = s.view;
    v.W1 = w1(s);
    v.W2 = w2(s);
    v.W3 = w3(s);
    v.W1t = w1t(s);
    v.W2t = w2t(s);
    v.W3t = w3t(s);
    v.b1 = s.master + MLP_OFF_B1;
    v.b2 = s.master + MLP_OFF_B2;
    v.b3 = s.master + MLP_OFF_B3;
    for (int k = 0; k < 7; k++) v.tau[k] = s.tau[k];
    ABIE_CUDA(cudaMemcpyAsync(s.view_dev, &v, sizeof v, cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaStreamSynchronize(st));
    s.ready = true;
    return 0;
}

int ensure_grad_buffers(int ctas)
{
    MlpState &s = g_mlp;
    if (ctas > s.grad_cap) {
        if (s.grad_partial) cudaFree(s.grad_partial);
        if (s.loss_partial) cudaFree(s.loss_partial);
        ABIE_CUDA(cudaMalloc(&s.grad_partial, (size_t)ctas * MLP_N_PARAMS * sizeof(float)));
        ABIE_CUDA(cudaMalloc(&s.loss_partial, (size_t)ctas * sizeof(float)));
        s.grad_cap = ctas;
    }
    if (!s.loss_partial) ABIE_CUDA(cudaMalloc(&s.loss_partial, (size_t)std::max(ctas, 1) * sizeof(float)));
    return 0;
}

// One gradient evaluation over rows (given by idx into the device sample
// store, or the first `rows` samples when idx is null); optional Adam step.
int mlp_step(const int *idx, long long rows, int adam, float lr, float *grad_out_dev,
             double *loss, cudaStream_t st)
{
    MlpState &s = g_mlp;
    int ctas = (int)((rows + TR - 1) / TR);
    int rc = ensure_grad_buffers(ctas);
    if (rc) return rc;
    mlp_grad_kernel<<<ctas, TT, sizeof(TrainSmem), st>>>(s.view, s.samples, idx, rows,
                                                         1.0f / (float)(rows * MLP_OUT),
                                                         s.grad_partial, s.loss_partial);
    ABIE_CUDA(cudaGetLastError());
    float b1c = 1.f, b2c = 1.f;
    if (adam) {
        s.adam_t++;
        b1c = 1.0f - powf(0.9f, (float)s.adam_t);
        b2c = 1.0f - powf(0.999f, (float)s.adam_t);
    }
    mlp_update_kernel<<<(MLP_N_PARAMS + 255) / 256, 256, 0, st>>>(
        s.master, s.adam_m, s.adam_v, s.w, s.grad_partial, ctas, grad_out_dev, adam, lr, b1c, b2c);
    ABIE_CUDA(cudaGetLastError());
    if (loss) {
        std::vector<float> lp(ctas);
        ABIE_CUDA(cudaMemcpyAsync(lp.data(), s.loss_partial, ctas * sizeof(float),
                                  cudaMemcpyDeviceToHost, st));
        ABIE_CUDA(cudaStreamSynchronize(st));
        double L = 0.0;
        for (int c = 0; c < ctas; c++) L += lp[c];
        *loss = L / (double)(rows * MLP_OUT);
    }
    return 0;
}

int ensure_samples(long long n)
{
    MlpState &s = g_mlp;
    if (n <= s.sample_cap) return 0;
    if (s.samples) cudaFree(s.samples);
    s.samples = nullptr;
    ABIE_CUDA(cudaMalloc(&s.samples, (size_t)n * MLP_SAMPLE * sizeof(float)));
    s.sample_cap = n;
    return 0;
}

}  // namespace

const LearnedPredictor *learned_predictor_device()
{
    return (g_mlp.ready && g_mlp.enabled) ? g_mlp.view_dev : nullptr;
}

const LearnedPredictor *learned_predictor_current() { return learned_predictor_device(); }

const float *learned_predictor_tau() { return g_mlp.tau; }

static unsigned long long *g_sample_counter = nullptr;
static long long g_collect_cap = 1 << 20;

// The ensemble appends samples after the ones already stored, up to the
// store's capacity (set by abie_mlp_set_capacity, 2^20 by default).
int mlp_collect_begin(EnsembleLearnIO *io)
{
    MlpState &s = g_mlp;
    if (!s.master) {
        set_error(ABIE_ERR_ARGUMENT, "sample collection needs abie_mlp_init first");
        return ABIE_ERR_ARGUMENT;
    }
    int rc = ensure_samples(g_collect_cap);
    if (rc) return rc;
    if (!g_sample_counter) ABIE_CUDA(cudaMalloc(&g_sample_counter, sizeof(unsigned long long)));
    unsigned long long c = (unsigned long long)s.n_samples;
    ABIE_CUDA(cudaMemcpy(g_sample_counter, &c, sizeof c, cudaMemcpyHostToDevice));
    io->samples = s.samples;
    io->cap = s.sample_cap;
    io->count = g_sample_counter;
    for (int k = 0; k < 7; k++) io->tau[k] = s.tau[k];
    return 0;
}

void mlp_collect_end(EnsembleLearnIO *io)
{
    unsigned long long c = 0;
    if (cudaMemcpy(&c, io->count, sizeof c, cudaMemcpyDeviceToHost) == cudaSuccess)
        g_mlp.n_samples = (long long)std::min<unsigned long long>(c, (unsigned long long)io->cap);
}

}  // namespace abie

using namespace abie;

extern "C" {

int abie_mlp_init(int seed, const double *tau)
{
    int rc = ensure_device(-1);
    if (rc) return rc;
    if ((rc = mlp_alloc())) return rc;
    MlpState &s = g_mlp;
    std::vector<float> p(MLP_N_PARAMS, 0.0f);
    unsigned long long st = 0x9E3779B97F4A7C15ull ^ (unsigned long long)seed;
    auto uni = [&]() {
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        return (double)(st >> 11) / 9007199254740992.0;
    };
    const double a1 = sqrt(6.0 / (MLP_FEAT + MLP_HID)), a2 = sqrt(6.0 / (2.0 * MLP_HID));
    for (int o = 0; o < MLP_HID; o++)
        for (int i = 0; i < MLP_IN; i++)
            p[MLP_OFF_W1 + o * MLP_IN + i] = i < MLP_FEAT ? (float)((2 * uni() - 1) * a1) : 0.0f;
    for (int k = 0; k < MLP_HID * MLP_HID; k++) p[MLP_OFF_W2 + k] = (float)((2 * uni() - 1) * a2);
    // W3, all biases: zero, so the untrained network is the plain predictor
    ABIE_CUDA(cudaMemcpy(s.master, p.data(), MLP_N_PARAMS * sizeof(float), cudaMemcpyHostToDevice));
    ABIE_CUDA(cudaMemset(s.adam_m, 0, MLP_N_PARAMS * sizeof(float)));
    ABIE_CUDA(cudaMemset(s.adam_v, 0, MLP_N_PARAMS * sizeof(float)));
    s.adam_t = 0;
    for (int k = 0; k < 7; k++) s.tau[k] = tau ? (float)tau[k] : 1.0f;
    return mlp_refresh(g_sim.st);
}

int abie_mlp_set_params(const float *params, int n, const double *tau)
{
    if (n != MLP_N_PARAMS) {
        set_error(ABIE_ERR_ARGUMENT, "abie_mlp_set_params: %d values, expected %d", n, MLP_N_PARAMS);
        return ABIE_ERR_ARGUMENT;
    }
    int rc = ensure_device(-1);
    if (rc) return rc;
    if ((rc = mlp_alloc())) return rc;
    ABIE_CUDA(cudaMemcpy(g_mlp.master, params, n * sizeof(float), cudaMemcpyHostToDevice));
    for (int k = 0; k < 7; k++) g_mlp.tau[k] = tau ? (float)tau[k] : 1.0f;
    return mlp_refresh(g_sim.st);
}

int abie_mlp_get_params(float *params, int n)
{
    if (n != MLP_N_PARAMS || !g_mlp.master) return ABIE_ERR_ARGUMENT;
    ABIE_CUDA(cudaMemcpy(params, g_mlp.master, n * sizeof(float), cudaMemcpyDeviceToHost));
    return MLP_N_PARAMS;
}

int abie_mlp_n_params(void) { return MLP_N_PARAMS; }

// rows x 64 floats (32 features, 32 targets) from the host into the sample store
int abie_mlp_load_samples(const float *samples, long long rows)
{
    int rc = ensure_device(-1);
    if (rc) return rc;
    if ((rc = ensure_samples(rows))) return rc;
    ABIE_CUDA(cudaMemcpy(g_mlp.samples, samples, (size_t)rows * MLP_SAMPLE * sizeof(float),
                         cudaMemcpyHostToDevice));
    g_mlp.n_samples = rows;
    return 0;
}

long long abie_mlp_sample_count(void) { return g_mlp.n_samples; }

int abie_mlp_get_samples(float *out, long long rows)
{
    if (rows > g_mlp.n_samples) rows = g_mlp.n_samples;
    if (rows <= 0) return 0;
    ABIE_CUDA(cudaMemcpy(out, g_mlp.samples, (size_t)rows * MLP_SAMPLE * sizeof(float),
                         cudaMemcpyDeviceToHost));
    return (int)rows;
}

void abie_mlp_clear_samples(void) { g_mlp.n_samples = 0; }

// Outputs (rows x 32) of the network on the first `rows` stored samples.
int abie_mlp_forward(long long rows, float *Y)
{
    if (!g_mlp.ready || rows > g_mlp.n_samples) return ABIE_ERR_ARGUMENT;
    float *d = nullptr;
    ABIE_CUDA(cudaMalloc(&d, (size_t)rows * MLP_OUT_PAD * sizeof(float)));
    int ctas = (int)((rows + TR - 1) / TR);
    mlp_forward_kernel<<<ctas, TT, sizeof(TrainSmem), g_sim.st>>>(g_mlp.view, g_mlp.samples, rows, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(Y, d, (size_t)rows * MLP_OUT_PAD * sizeof(float), cudaMemcpyDeviceToHost,
                            g_sim.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g_sim.st);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "abie_mlp_forward");
    return 0;
}

// Loss and summed gradient (N_PARAMS floats) over the first `rows` samples.
int abie_mlp_loss_grad(long long rows, float *grad, double *loss)
{
    if (!g_mlp.ready || rows > g_mlp.n_samples || rows <= 0) return ABIE_ERR_ARGUMENT;
    float *d = nullptr;
    ABIE_CUDA(cudaMalloc(&d, MLP_N_PARAMS * sizeof(float)));
    int rc = mlp_step(nullptr, rows, 0, 0.f, d, loss, g_sim.st);
    if (!rc) {
        cudaError_t e = cudaMemcpy(grad, d, MLP_N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(e, "abie_mlp_loss_grad");
    }
    cudaFree(d);
    return rc;
}

// Adam on random minibatches of the stored samples; loss of the last batch.
int abie_mlp_train(int steps, int batch, double lr, int seed, double *last_loss)
{
    MlpState &s = g_mlp;
    if (!s.ready || s.n_samples <= 0) {
        set_error(ABIE_ERR_ARGUMENT, "abie_mlp_train: no network or no samples");
        return ABIE_ERR_ARGUMENT;
    }
    if (batch > s.n_samples) batch = (int)s.n_samples;
    if (batch > s.idx_cap) {
        if (s.idx) cudaFree(s.idx);
        ABIE_CUDA(cudaMalloc(&s.idx, (size_t)batch * sizeof(int)));
        s.idx_cap = batch;
    }
    std::vector<int> idx(batch);
    unsigned long long r = 0xD1B54A32D192ED03ull ^ (unsigned long long)seed;
    int rc = 0;
    for (int k = 0; k < steps && !rc; k++) {
        for (int i = 0; i < batch; i++) {
            r ^= r << 13;
            r ^= r >> 7;
            r ^= r << 17;
            idx[i] = (int)(r % (unsigned long long)s.n_samples);
        }
        ABIE_CUDA(cudaMemcpyAsync(s.idx, idx.data(), batch * sizeof(int), cudaMemcpyHostToDevice,
                                  g_sim.st));
        rc = mlp_step(s.idx, batch, 1, (float)lr, nullptr, (k == steps - 1) ? last_loss : nullptr,
                      g_sim.st);
    }
    ABIE_CUDA(cudaStreamSynchronize(g_sim.st));
    return rc;
}

// The ensemble uses the network when asked (flag) and when enabled here.
void abie_mlp_enable(int on) { g_mlp.enabled = on != 0; }

void abie_mlp_set_capacity(long long samples) { g_collect_cap = samples > 0 ? samples : 1; }

}  // extern "C"
