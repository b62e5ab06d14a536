// Warm-start network: a per-node MLP 24 -> 64 -> 64 -> 64 -> 3 (GELU, tanh
// form) evaluated on tensor cores with BF16 operands and FP32 accumulation.
//
// Parameter vector (10,115 FP32 master values): W1 (64x24, row = output), b1,
// W2 (64x64), b2, W3 (64x64), b3, W4 (3x64), b4.  Kernels stage BF16 copies
// of the weights in shared memory:
//   sW1 [64][32]  (inputs padded 24 -> 32 with zeros)
//   sW2 [64][64], sW3 [64][64]
//   sW4 [8][64]   (outputs padded 3 -> 8 with zeros)
// and, for the backward pass, the transposes sW2T, sW3T ([in][out]).
//
// Tensor-core tile: mma.sync m16n8k16 (row-major A = activations, col-major
// B = weights, FP32 C).  A warp owns 16 rows (nodes); a layer's FP32
// accumulators, after bias and GELU, are repacked in registers into the next
// layer's A fragments (accumulator tile n and n+1 form k-block n/2).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pbs {
namespace mlp {

constexpr int IN = 24, KIN = 32, HID = 64, OUT = 3, NOUT = 8;
constexpr int OFF_W1 = 0, OFF_B1 = 1536, OFF_W2 = 1600, OFF_B2 = 5696, OFF_W3 = 5760, OFF_B3 = 9856;
constexpr int OFF_W4 = 9920, OFF_B4 = 10112, NPARAM = 10115;

struct SmemWeights {
    __nv_bfloat16 w1[HID * KIN];
    __nv_bfloat16 w2[HID * HID];
    __nv_bfloat16 w3[HID * HID];
    __nv_bfloat16 w4[NOUT * HID];
    float b1[HID], b2[HID], b3[HID], b4[NOUT];
};

// Stage the BF16 weights (and FP32 biases) of theta into shared memory.
__device__ __forceinline__ void stage_weights(const float *theta, SmemWeights &s) {
    for (int i = threadIdx.x; i < HID * KIN; i += blockDim.x) {
        const int o = i / KIN, k = i % KIN;
        s.w1[i] = __float2bfloat16_rn(k < IN ? theta[OFF_W1 + o * IN + k] : 0.f);
    }
    for (int i = threadIdx.x; i < HID * HID; i += blockDim.x) {
        s.w2[i] = __float2bfloat16_rn(theta[OFF_W2 + i]);
        s.w3[i] = __float2bfloat16_rn(theta[OFF_W3 + i]);
    }
    for (int i = threadIdx.x; i < NOUT * HID; i += blockDim.x) {
        const int o = i / HID;
        s.w4[i] = __float2bfloat16_rn(o < OUT ? theta[OFF_W4 + i] : 0.f);
    }
    for (int i = threadIdx.x; i < HID; i += blockDim.x) {
        s.b1[i] = theta[OFF_B1 + i];
        s.b2[i] = theta[OFF_B2 + i];
        s.b3[i] = theta[OFF_B3 + i];
    }
    for (int i = threadIdx.x; i < NOUT; i += blockDim.x) s.b4[i] = i < OUT ? theta[OFF_B4 + i] : 0.f;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t pack_raw(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// GELU (tanh form) and its derivative.
__device__ __forceinline__ float gelu(float z) {
    const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
    return 0.5f * z * (1.0f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float z) {
    const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
    const float t = tanhf(u);
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * 0.7978845608028654f * (1.0f + 0.134145f * z * z);
}

// acc[j] (output columns 8j..8j+7) = bias + A (16 x 16*KB) * W^T, where W is
// a row-major [64][16*KB] BF16 matrix in shared memory.
template <int KB, int NT>
__device__ __forceinline__ void layer(const uint32_t (&a)[KB][4], const __nv_bfloat16 *W, const float *bias,
                                      float (&acc)[NT][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const float c0 = bias[8 * j + 2 * t], c1 = bias[8 * j + 2 * t + 1];
        acc[j][0] = c0; acc[j][1] = c1; acc[j][2] = c0; acc[j][3] = c1;
        const __nv_bfloat16 *row = W + (8 * j + g) * (16 * KB);
#pragma unroll
        for (int kb = 0; kb < KB; ++kb) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row + 16 * kb + 2 * t);
            const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + 16 * kb + 8 + 2 * t);
            mma16816(acc[j], a[kb], b0, b1);
        }
    }
}

// GELU of 8 accumulator tiles, repacked as 4 k-blocks of A fragments.
__device__ __forceinline__ void gelu_to_frags(const float (&acc)[8][4], uint32_t (&a)[4][4]) {
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
        a[kb][0] = pack_bf16(gelu(acc[2 * kb][0]), gelu(acc[2 * kb][1]));
        a[kb][1] = pack_bf16(gelu(acc[2 * kb][2]), gelu(acc[2 * kb][3]));
        a[kb][2] = pack_bf16(gelu(acc[2 * kb + 1][0]), gelu(acc[2 * kb + 1][1]));
        a[kb][3] = pack_bf16(gelu(acc[2 * kb + 1][2]), gelu(acc[2 * kb + 1][3]));
    }
}

// A fragments of a 16 x 32 input tile from a row-major FP32 [rows][24] array
// (columns 24..31 are zero).  Rows beyond `rows` read as zero.
__device__ __forceinline__ void input_frags(const float *X, int row0, int rows, uint32_t (&a)[2][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r0 = row0 + g, r1 = row0 + g + 8;
#pragma unroll
    for (int kb = 0; kb < 2; ++kb) {
        float v[4][2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int col = 16 * kb + 8 * h + 2 * t;
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                v[2 * h][e] = (r0 < rows && col + e < IN) ? X[(size_t)r0 * IN + col + e] : 0.f;
                v[2 * h + 1][e] = (r1 < rows && col + e < IN) ? X[(size_t)r1 * IN + col + e] : 0.f;
            }
        }
        a[kb][0] = pack_bf16(v[0][0], v[0][1]);
        a[kb][1] = pack_bf16(v[1][0], v[1][1]);
        a[kb][2] = pack_bf16(v[2][0], v[2][1]);
        a[kb][3] = pack_bf16(v[3][0], v[3][1]);
    }
}

// Forward of one 16-row tile; out[0..3] = rows g (c0, c1) and g + 8 (c2, c3)
// of output columns 2t, 2t+1 (t = lane & 3; columns >= 3 are padding).
__device__ __forceinline__ void forward_tile(const SmemWeights &s, const uint32_t (&x)[2][4], float (&out)[4]) {
    float acc[8][4];
    uint32_t a[4][4];
    layer<2, 8>(x, s.w1, s.b1, acc);
    gelu_to_frags(acc, a);
    layer<4, 8>(a, s.w2, s.b2, acc);
    gelu_to_frags(acc, a);
    layer<4, 8>(a, s.w3, s.b3, acc);
    gelu_to_frags(acc, a);
    float o[1][4];
    layer<4, 1>(a, s.w4, s.b4, o);
#pragma unroll
    for (int i = 0; i < 4; ++i) out[i] = o[0][i];
}

}  // namespace mlp
}  // namespace pbs
