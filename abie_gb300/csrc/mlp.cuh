// Learned Radau15 predictor: a BF16 multilayer perceptron that proposes the
// next step's b coefficients of a body.
//
//   in  (32, 30 used): the body's converged b of the step just accepted,
//        b_k[d] / s_k for k < 7, d < 3 (s_k = max_d |b_k[d]|, one scale per
//        order), log2 of the requested and the actual step ratio
//        (dtreq/h, h_next/h) / 4, log10(m / m_star) / 10 and
//        log10(s_k / s_0) / 10 for k = 1..6
//   H1 = relu(in W1^T + b1), H2 = relu(H1 W2^T + b2)      (128, 128)
//   out = H2 W3^T + b3     (32, 21 used): (b_next,k - E_k(q)) / (s_k tau_k)
// where E(q) is the reference's plain predictor (refine_bs) and tau_k fixed
// output scales.  The guess handed to the corrector is E_k + s_k tau_k out,
// so an all-zero output layer is exactly the plain predictor.
//
// Tensor-core operands are BF16, accumulation FP32 (mma.sync m16n8k16).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace abie {

constexpr int MLP_IN = 32, MLP_HID = 128, MLP_OUT = 21, MLP_OUT_PAD = 32, MLP_FEAT = 30;
constexpr int MLP_N_PARAMS = MLP_HID * MLP_IN + MLP_HID + MLP_HID * MLP_HID + MLP_HID +
                             MLP_OUT_PAD * MLP_HID + MLP_OUT_PAD;
// offsets of the tensors in the flat FP32 parameter vector
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_HID * MLP_IN;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_HID;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_HID * MLP_HID;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_HID;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_OUT_PAD * MLP_HID;
constexpr int MLP_SAMPLE = MLP_IN + MLP_OUT_PAD;  // floats per training sample: features, target

struct LearnedPredictor {
    // BF16 weights, row-major [out][in], and their transposes [in][out]
    const __nv_bfloat16 *W1, *W2, *W3;
    const __nv_bfloat16 *W1t, *W2t, *W3t;
    const float *b1, *b2, *b3;
    float tau[7];  // output scale per coefficient order
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// One 16x8 output tile of C = A * B with A row-major [M][K] (lda elements)
// and B given as Bt row-major [N][K] (ldb elements), both BF16; K a
// multiple of 16.  Fragment layouts of mma.m16n8k16: lane = 4 g + t holds
// A rows g and g+8, columns 2t, 2t+1 (+8); B column g, rows 2t, 2t+1 (+8);
// C rows g and g+8, columns 2t, 2t+1.
__device__ __forceinline__ void mma_tile(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *Bt,
                                         int ldb, int m0, int n0, int K, float c[4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    c[0] = c[1] = c[2] = c[3] = 0.0f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4], b[2];
        const __nv_bfloat16 *ar0 = A + (size_t)(m0 + g) * lda + k0 + 2 * t;
        const __nv_bfloat16 *ar1 = A + (size_t)(m0 + g + 8) * lda + k0 + 2 * t;
        a[0] = *reinterpret_cast<const uint32_t *>(ar0);
        a[1] = *reinterpret_cast<const uint32_t *>(ar1);
        a[2] = *reinterpret_cast<const uint32_t *>(ar0 + 8);
        a[3] = *reinterpret_cast<const uint32_t *>(ar1 + 8);
        const __nv_bfloat16 *br = Bt + (size_t)(n0 + g) * ldb + k0 + 2 * t;
        b[0] = *reinterpret_cast<const uint32_t *>(br);
        b[1] = *reinterpret_cast<const uint32_t *>(br + 8);
        mma_bf16_16816(c, a, b);
    }
}

// Learned predictor in use, or null (mlp.cu).
const LearnedPredictor *learned_predictor_device();

}  // namespace abie
