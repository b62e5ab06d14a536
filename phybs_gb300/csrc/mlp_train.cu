// Training and batch inference of the warm-start MLP (see mlp.cuh) with
// hand-written BF16 tensor-core kernels (mma.sync m16n8k16, FP32 accumulate).
//
//   k_mlp_forward   rows -> 3 outputs; each warp runs 16-row tiles.
//   k_mlp_grad      forward + backward of a minibatch.  A CTA (4 warps) takes
//                   64-row tiles: warps run the forward and the delta
//                   recursion on their own 16 rows (activations, GELU' and
//                   deltas staged in shared memory), then every warp forms a
//                   16-output-row block of dW1..dW3 as delta^T * h over the
//                   tile's 64 rows on the tensor cores, accumulating in
//                   registers across the CTA's tiles.  Biases and W4's
//                   gradient are small and use SIMT sums.  Each CTA writes
//                   its partial gradient; k_mlp_reduce sums the partials in a
//                   fixed order, so the gradient is deterministic.
//   k_mlp_adam      Adam on the FP32 master parameters.
// Loss: mean over rows of the squared error summed over the 3 outputs.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/phybs.h"
#include "mlp.cuh"

namespace pbs {
namespace mlp {

constexpr int TRAIN_WARPS = 4;
constexpr int TILE = 16 * TRAIN_WARPS;  // rows per CTA tile
constexpr int NPART = NPARAM + 1;       // partial gradient + loss

__global__ void __launch_bounds__(128) k_mlp_forward(const float *theta, const float *X, int rows, float *Y) {
    __shared__ SmemWeights s;
    stage_weights(theta, s);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warps = blockDim.x >> 5, wid = blockIdx.x * warps + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * warps;
    for (int row0 = wid * 16; row0 < rows; row0 += nwarps * 16) {
        uint32_t x[2][4];
        input_frags(X, row0, rows, x);
        float out[4];
        forward_tile(s, x, out);
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int col = 2 * t + e;
            if (col < OUT) {
                if (row0 + g < rows) Y[(size_t)(row0 + g) * OUT + col] = out[e];
                if (row0 + g + 8 < rows) Y[(size_t)(row0 + g + 8) * OUT + col] = out[2 + e];
            }
        }
    }
}

struct TrainSmem {
    SmemWeights w;
    __nv_bfloat16 w2t[HID * HID], w3t[HID * HID];  // [in][out]
    float w4[OUT * HID];
    float zero_bias[HID];
    __nv_bfloat16 xs[TILE * KIN];
    __nv_bfloat16 h1[TILE * HID], h2[TILE * HID], h3[TILE * HID];
    float gd1[TILE * HID], gd2[TILE * HID], gd3[TILE * HID];
    __nv_bfloat16 d1[TILE * HID], d2[TILE * HID], d3[TILE * HID];
    float d4[TILE * 4];
    float acc_b[3 * HID + OUT];  // db1, db2, db3, db4
    float acc_w4[OUT * HID];
    float loss[TRAIN_WARPS];
};

// Store one layer's activations (BF16) and GELU' (FP32) at the C-fragment
// positions of the warp's 16 rows; returns the next layer's A fragments.
__device__ __forceinline__ void store_act(const float (&acc)[8][4], int r0, __nv_bfloat16 *h, float *gd,
                                          uint32_t (&a)[4][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float act[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = r0 + g + (q >= 2 ? 8 : 0), c = 8 * j + 2 * t + (q & 1);
            act[j][q] = gelu(acc[j][q]);
            gd[r * HID + c] = gelu_grad(acc[j][q]);
            h[r * HID + c] = __float2bfloat16_rn(act[j][q]);
        }
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
        a[kb][0] = pack_bf16(act[2 * kb][0], act[2 * kb][1]);
        a[kb][1] = pack_bf16(act[2 * kb][2], act[2 * kb][3]);
        a[kb][2] = pack_bf16(act[2 * kb + 1][0], act[2 * kb + 1][1]);
        a[kb][3] = pack_bf16(act[2 * kb + 1][2], act[2 * kb + 1][3]);
    }
}

// delta = acc (.) GELU'(z), stored BF16 and returned as A fragments.
__device__ __forceinline__ void store_delta(float (&acc)[8][4], int r0, const float *gd, __nv_bfloat16 *d,
                                            uint32_t (&a)[4][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = r0 + g + (q >= 2 ? 8 : 0), c = 8 * j + 2 * t + (q & 1);
            acc[j][q] *= gd[r * HID + c];
            d[r * HID + c] = __float2bfloat16_rn(acc[j][q]);
        }
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
        a[kb][0] = pack_bf16(acc[2 * kb][0], acc[2 * kb][1]);
        a[kb][1] = pack_bf16(acc[2 * kb][2], acc[2 * kb][3]);
        a[kb][2] = pack_bf16(acc[2 * kb + 1][0], acc[2 * kb + 1][1]);
        a[kb][3] = pack_bf16(acc[2 * kb + 1][2], acc[2 * kb + 1][3]);
    }
}

// dW[16w + m][n] += sum_r delta[r][16w + m] * h[r][n] over the tile's rows
// (A = delta^T from shared memory, B = h from shared memory).
template <int NT, int HW>
__device__ __forceinline__ void weight_grad(const __nv_bfloat16 *delta, const __nv_bfloat16 *hin, float (&acc)[NT][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
    const int m0 = 16 * w;
#pragma unroll
    for (int kb = 0; kb < TILE / 16; ++kb) {
        const int r0 = 16 * kb + 2 * t;
        uint32_t a[4];
        a[0] = pack_raw(delta[r0 * HID + m0 + g], delta[(r0 + 1) * HID + m0 + g]);
        a[1] = pack_raw(delta[r0 * HID + m0 + g + 8], delta[(r0 + 1) * HID + m0 + g + 8]);
        a[2] = pack_raw(delta[(r0 + 8) * HID + m0 + g], delta[(r0 + 9) * HID + m0 + g]);
        a[3] = pack_raw(delta[(r0 + 8) * HID + m0 + g + 8], delta[(r0 + 9) * HID + m0 + g + 8]);
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int n = 8 * j + g;
            const uint32_t b0 = pack_raw(hin[r0 * HW + n], hin[(r0 + 1) * HW + n]);
            const uint32_t b1 = pack_raw(hin[(r0 + 8) * HW + n], hin[(r0 + 9) * HW + n]);
            mma16816(acc[j], a, b0, b1);
        }
    }
}

__global__ void __launch_bounds__(128) k_mlp_grad(const float *theta, const float *X, const float *Y, const float *W,
                                                  const int *idx, int batch, float *part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &s = *reinterpret_cast<TrainSmem *>(smem_raw);
    stage_weights(theta, s.w);
    for (int i = threadIdx.x; i < HID * HID; i += blockDim.x) {
        const int o = i / HID, k = i % HID;
        s.w2t[k * HID + o] = __float2bfloat16_rn(theta[OFF_W2 + i]);
        s.w3t[k * HID + o] = __float2bfloat16_rn(theta[OFF_W3 + i]);
    }
    for (int i = threadIdx.x; i < OUT * HID; i += blockDim.x) s.w4[i] = __bfloat162float(__float2bfloat16_rn(theta[OFF_W4 + i]));
    for (int i = threadIdx.x; i < HID; i += blockDim.x) s.zero_bias[i] = 0.f;
    for (int i = threadIdx.x; i < 3 * HID + OUT; i += blockDim.x) s.acc_b[i] = 0.f;
    for (int i = threadIdx.x; i < OUT * HID; i += blockDim.x) s.acc_w4[i] = 0.f;
    if (threadIdx.x < TRAIN_WARPS) s.loss[threadIdx.x] = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
    const int r0 = 16 * w;
    const float inv_b = 1.0f / (float)batch;
    float gw1[4][4] = {}, gw2[8][4] = {}, gw3[8][4] = {};
    float loss = 0.f;
    for (int base = blockIdx.x * TILE; base < batch; base += gridDim.x * TILE) {
        // input tile (BF16, columns 24..31 zero; rows past the batch zero)
        for (int i = threadIdx.x; i < TILE * KIN; i += blockDim.x) {
            const int r = i / KIN, c = i % KIN;
            float v = 0.f;
            if (base + r < batch && c < IN) v = X[(size_t)idx[base + r] * IN + c];
            s.xs[i] = __float2bfloat16_rn(v);
        }
        __syncthreads();
        // ---- forward (own 16 rows)
        uint32_t x[2][4];
#pragma unroll
        for (int kb = 0; kb < 2; ++kb) {
            const __nv_bfloat16 *xr0 = s.xs + (r0 + g) * KIN + 16 * kb + 2 * t;
            const __nv_bfloat16 *xr1 = s.xs + (r0 + g + 8) * KIN + 16 * kb + 2 * t;
            x[kb][0] = *reinterpret_cast<const uint32_t *>(xr0);
            x[kb][1] = *reinterpret_cast<const uint32_t *>(xr1);
            x[kb][2] = *reinterpret_cast<const uint32_t *>(xr0 + 8);
            x[kb][3] = *reinterpret_cast<const uint32_t *>(xr1 + 8);
        }
        float acc[8][4];
        uint32_t a[4][4];
        layer<2, 8>(x, s.w.w1, s.w.b1, acc);
        store_act(acc, r0, s.h1, s.gd1, a);
        layer<4, 8>(a, s.w.w2, s.w.b2, acc);
        store_act(acc, r0, s.h2, s.gd2, a);
        layer<4, 8>(a, s.w.w3, s.w.b3, acc);
        store_act(acc, r0, s.h3, s.gd3, a);
        float o[1][4];
        layer<4, 1>(a, s.w.w4, s.w.b4, o);
        // output deltas 2 w (y - t) / B (w = 1 without sample weights)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int rl = r0 + g + (q >= 2 ? 8 : 0), c = 2 * t + (q & 1);
            float dlt = 0.f;
            if (c < OUT && base + rl < batch) {
                const int row = idx[base + rl];
                const float diff = o[0][q] - Y[(size_t)row * OUT + c];
                const float wd = W ? W[row] * diff : diff;
                loss += wd * diff;
                dlt = 2.0f * wd * inv_b;
            }
            if (c < 4) s.d4[rl * 4 + c] = dlt;
        }
        __syncwarp();
        // ---- backward deltas (own 16 rows)
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int rl = r0 + g + (q >= 2 ? 8 : 0), c = 8 * j + 2 * t + (q & 1);
                acc[j][q] = s.d4[rl * 4] * s.w4[c] + s.d4[rl * 4 + 1] * s.w4[HID + c] + s.d4[rl * 4 + 2] * s.w4[2 * HID + c];
            }
        store_delta(acc, r0, s.gd3, s.d3, a);
        layer<4, 8>(a, s.w3t, s.zero_bias, acc);
        store_delta(acc, r0, s.gd2, s.d2, a);
        layer<4, 8>(a, s.w2t, s.zero_bias, acc);
        store_delta(acc, r0, s.gd1, s.d1, a);
        __syncthreads();
        // ---- weight gradients: warp w owns output rows 16w .. 16w+15
        weight_grad<4, KIN>(s.d1, s.xs, gw1);
        weight_grad<8, HID>(s.d2, s.h1, gw2);
        weight_grad<8, HID>(s.d3, s.h2, gw3);
        // biases and W4 (SIMT; each entry owned by one thread)
        for (int task = threadIdx.x; task < 3 * HID + OUT + OUT * HID; task += blockDim.x) {
            float sum = 0.f;
            if (task < 3 * HID) {
                const __nv_bfloat16 *d = task < HID ? s.d1 : (task < 2 * HID ? s.d2 : s.d3);
                const int c = task % HID;
                for (int r = 0; r < TILE; ++r) sum += __bfloat162float(d[r * HID + c]);
                s.acc_b[task] += sum;
            } else if (task < 3 * HID + OUT) {
                const int c = task - 3 * HID;
                for (int r = 0; r < TILE; ++r) sum += s.d4[r * 4 + c];
                s.acc_b[task] += sum;
            } else {
                const int k = task - 3 * HID - OUT, oo = k / HID, c = k % HID;
                for (int r = 0; r < TILE; ++r) sum += s.d4[r * 4 + oo] * __bfloat162float(s.h3[r * HID + c]);
                s.acc_w4[k] += sum;
            }
        }
        __syncthreads();
    }
    // ---- partial gradient of this CTA
    float *P = part + (size_t)blockIdx.x * NPART;
    const int m0 = 16 * w;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int oo = m0 + g + (q >= 2 ? 8 : 0), c = 8 * j + 2 * t + (q & 1);
            if (c < IN) P[OFF_W1 + oo * IN + c] = gw1[j][q];
        }
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int oo = m0 + g + (q >= 2 ? 8 : 0), c = 8 * j + 2 * t + (q & 1);
            P[OFF_W2 + oo * HID + c] = gw2[j][q];
            P[OFF_W3 + oo * HID + c] = gw3[j][q];
        }
    for (int i = threadIdx.x; i < HID; i += blockDim.x) {
        P[OFF_B1 + i] = s.acc_b[i];
        P[OFF_B2 + i] = s.acc_b[HID + i];
        P[OFF_B3 + i] = s.acc_b[2 * HID + i];
    }
    for (int i = threadIdx.x; i < OUT * HID; i += blockDim.x) P[OFF_W4 + i] = s.acc_w4[i];
    if (threadIdx.x < OUT) P[OFF_B4 + threadIdx.x] = s.acc_b[3 * HID + threadIdx.x];
    // loss: fixed-order warp then CTA sum
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, off);
    if (lane == 0) s.loss[w] = loss;
    __syncthreads();
    if (threadIdx.x == 0) {
        float l = 0.f;
        for (int i = 0; i < TRAIN_WARPS; ++i) l += s.loss[i];
        P[NPARAM] = l * inv_b;
    }
}

__global__ void k_mlp_reduce(const float *part, int nparts, float *grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPART) return;
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += part[(size_t)p * NPART + i];
    grad[i] = s;
}

__global__ void k_mlp_adam(float *theta, float *m, float *v, const float *grad, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    theta[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

int grad_ctas(int batch, int sms) {
    int tiles = (batch + TILE - 1) / TILE;
    return tiles < sms ? (tiles > 0 ? tiles : 1) : sms;
}

}  // namespace mlp
}  // namespace pbs

using namespace pbs::mlp;

struct pbs_mlp {
    cudaStream_t stream = nullptr;
    int sms = 148;
    float *theta = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *part = nullptr;
    float *X = nullptr, *Y = nullptr, *W = nullptr, *io = nullptr;
    int *idx = nullptr;
    int n = 0, cap_part = 0, cap_io = 0, step = 0;
};

#define MCK(x)                                                                               \
    do {                                                                                     \
        cudaError_t e__ = (x);                                                               \
        if (e__ != cudaSuccess) return e__ == cudaErrorMemoryAllocation ? PBS_E_OUT_OF_MEMORY : PBS_E_CUDA; \
    } while (0)

static int ensure_io(pbs_mlp *t, int n) {
    if (n <= t->cap_io) return PBS_OK;
    if (t->io) cudaFree(t->io);
    t->io = nullptr;
    t->cap_io = 0;
    MCK(cudaMalloc(&t->io, sizeof(float) * (size_t)n * (IN + OUT)));
    t->cap_io = n;
    return PBS_OK;
}

static int ensure_part(pbs_mlp *t, int nparts) {
    if (nparts <= t->cap_part) return PBS_OK;
    if (t->part) cudaFree(t->part);
    t->part = nullptr;
    t->cap_part = 0;
    MCK(cudaMalloc(&t->part, sizeof(float) * (size_t)nparts * NPART));
    t->cap_part = nparts;
    return PBS_OK;
}

static int run_grad(pbs_mlp *t, const float *X, const float *Y, const float *W, const int *idx, int batch) {
    const int ctas = grad_ctas(batch, t->sms);
    int rc = ensure_part(t, ctas);
    if (rc != PBS_OK) return rc;
    const size_t smem = sizeof(TrainSmem);
    MCK(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_mlp_grad<<<ctas, 128, smem, t->stream>>>(t->theta, X, Y, W, idx, batch, t->part);
    MCK(cudaGetLastError());
    k_mlp_reduce<<<(NPART + 255) / 256, 256, 0, t->stream>>>(t->part, ctas, t->grad);
    MCK(cudaGetLastError());
    return PBS_OK;
}

extern "C" {

int pbs_mlp_param_count(void) { return NPARAM; }

int pbs_mlp_create(pbs_mlp **out, const float *theta, unsigned long long seed) {
    if (!out) return PBS_E_INVALID_ARG;
    *out = nullptr;
    int dev = 0, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PBS_E_NO_DEVICE;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major != 10 || prop.minor != 3) return PBS_E_NO_DEVICE;
    pbs_mlp *t = new pbs_mlp();
    t->sms = prop.multiProcessorCount;
    std::vector<float> th(NPARAM, 0.f);
    if (theta) {
        std::memcpy(th.data(), theta, sizeof(float) * NPARAM);
    } else {  // He initialisation, zero biases
        std::mt19937_64 rng(seed);
        const int sizes[4][3] = {{OFF_W1, HID, IN}, {OFF_W2, HID, HID}, {OFF_W3, HID, HID}, {OFF_W4, OUT, HID}};
        for (auto &L : sizes) {
            std::normal_distribution<float> nd(0.f, std::sqrt(2.f / L[2]));
            for (int i = 0; i < L[1] * L[2]; ++i) th[L[0] + i] = nd(rng);
        }
    }
    auto fail = [&](int rc) { pbs_mlp_destroy(t); return rc; };
    if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(PBS_E_CUDA);
    if (cudaMalloc(&t->theta, sizeof(float) * NPARAM) != cudaSuccess || cudaMalloc(&t->m, sizeof(float) * NPARAM) != cudaSuccess ||
        cudaMalloc(&t->v, sizeof(float) * NPARAM) != cudaSuccess || cudaMalloc(&t->grad, sizeof(float) * NPART) != cudaSuccess)
        return fail(PBS_E_OUT_OF_MEMORY);
    if (cudaMemcpy(t->theta, th.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(t->m, 0, sizeof(float) * NPARAM) != cudaSuccess || cudaMemset(t->v, 0, sizeof(float) * NPARAM) != cudaSuccess)
        return fail(PBS_E_CUDA);
    *out = t;
    return PBS_OK;
}

void pbs_mlp_destroy(pbs_mlp *t) {
    if (!t) return;
    if (t->stream) cudaStreamSynchronize(t->stream);
    float *bufs[] = {t->theta, t->m, t->v, t->grad, t->part, t->X, t->Y, t->W, t->io};
    for (float *b : bufs)
        if (b) cudaFree(b);
    if (t->idx) cudaFree(t->idx);
    if (t->stream) cudaStreamDestroy(t->stream);
    delete t;
}

int pbs_mlp_get_params(pbs_mlp *t, float *theta) {
    if (!t || !theta) return PBS_E_INVALID_ARG;
    MCK(cudaMemcpy(theta, t->theta, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    return PBS_OK;
}

int pbs_mlp_set_params(pbs_mlp *t, const float *theta) {
    if (!t || !theta) return PBS_E_INVALID_ARG;
    MCK(cudaMemcpy(t->theta, theta, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
    MCK(cudaMemset(t->m, 0, sizeof(float) * NPARAM));
    MCK(cudaMemset(t->v, 0, sizeof(float) * NPARAM));
    t->step = 0;
    return PBS_OK;
}

int pbs_mlp_forward(pbs_mlp *t, const float *X, int n, float *Y) {
    if (!t || !X || !Y || n <= 0) return PBS_E_INVALID_ARG;
    int rc = ensure_io(t, n);
    if (rc != PBS_OK) return rc;
    float *dX = t->io, *dY = t->io + (size_t)n * IN;
    MCK(cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * IN, cudaMemcpyHostToDevice, t->stream));
    const int blocks = std::min((n + 63) / 64, 4 * t->sms);
    k_mlp_forward<<<blocks, 128, 0, t->stream>>>(t->theta, dX, n, dY);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(Y, dY, sizeof(float) * (size_t)n * OUT, cudaMemcpyDeviceToHost, t->stream));
    MCK(cudaStreamSynchronize(t->stream));
    return PBS_OK;
}

int pbs_mlp_gradient(pbs_mlp *t, const float *X, const float *Y, int n, float *grad, float *loss) {
    if (!t || !X || !Y || n <= 0 || !grad) return PBS_E_INVALID_ARG;
    int rc = ensure_io(t, n);
    if (rc != PBS_OK) return rc;
    float *dX = t->io, *dY = t->io + (size_t)n * IN;
    int *didx = nullptr;
    MCK(cudaMalloc(&didx, sizeof(int) * n));
    std::vector<int> iota(n);
    for (int i = 0; i < n; ++i) iota[i] = i;
    cudaError_t e = cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * IN, cudaMemcpyHostToDevice, t->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dY, Y, sizeof(float) * (size_t)n * OUT, cudaMemcpyHostToDevice, t->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(didx, iota.data(), sizeof(int) * n, cudaMemcpyHostToDevice, t->stream);
    if (e != cudaSuccess) { cudaFree(didx); return PBS_E_CUDA; }
    rc = run_grad(t, dX, dY, nullptr, didx, n);
    std::vector<float> g(NPART);
    if (rc == PBS_OK && cudaMemcpyAsync(g.data(), t->grad, sizeof(float) * NPART, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess)
        rc = PBS_E_CUDA;
    if (rc == PBS_OK && cudaStreamSynchronize(t->stream) != cudaSuccess) rc = PBS_E_CUDA;
    cudaFree(didx);
    if (rc != PBS_OK) return rc;
    std::memcpy(grad, g.data(), sizeof(float) * NPARAM);
    if (loss) *loss = g[NPARAM];
    return PBS_OK;
}

int pbs_mlp_set_data(pbs_mlp *t, const float *X, const float *Y, const float *W, int n) {
    if (!t || !X || !Y || n <= 0) return PBS_E_INVALID_ARG;
    if (W)
        for (int i = 0; i < n; ++i)
            if (!(W[i] >= 0.f) || !std::isfinite(W[i])) return PBS_E_INVALID_ARG;
    if (t->X) cudaFree(t->X);
    if (t->Y) cudaFree(t->Y);
    if (t->W) cudaFree(t->W);
    if (t->idx) cudaFree(t->idx);
    t->X = t->Y = t->W = nullptr;
    t->idx = nullptr;
    t->n = 0;
    MCK(cudaMalloc(&t->X, sizeof(float) * (size_t)n * IN));
    MCK(cudaMalloc(&t->Y, sizeof(float) * (size_t)n * OUT));
    if (W) MCK(cudaMalloc(&t->W, sizeof(float) * (size_t)n));
    MCK(cudaMalloc(&t->idx, sizeof(int) * (size_t)n));
    MCK(cudaMemcpyAsync(t->X, X, sizeof(float) * (size_t)n * IN, cudaMemcpyHostToDevice, t->stream));
    MCK(cudaMemcpyAsync(t->Y, Y, sizeof(float) * (size_t)n * OUT, cudaMemcpyHostToDevice, t->stream));
    if (W) MCK(cudaMemcpyAsync(t->W, W, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, t->stream));
    MCK(cudaStreamSynchronize(t->stream));
    t->n = n;
    return PBS_OK;
}

// `steps` Adam steps on minibatches of `batch` rows drawn without replacement
// (a fresh permutation each epoch).  losses (optional, `steps` floats) gets
// each step's minibatch loss.
int pbs_mlp_train(pbs_mlp *t, int steps, int batch, float lr, unsigned long long seed, float *losses) {
    if (!t || steps < 0 || batch <= 0 || !(lr > 0.f) || t->n <= 0) return PBS_E_INVALID_ARG;
    if (batch > t->n) batch = t->n;
    std::mt19937_64 rng(seed);
    std::vector<int> perm(t->n);
    int pos = t->n;
    std::vector<float> lossbuf(steps > 0 ? steps : 1);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int sidx = 0; sidx < steps; ++sidx) {
        if (pos + batch > t->n) {
            for (int i = 0; i < t->n; ++i) perm[i] = i;
            std::shuffle(perm.begin(), perm.end(), rng);
            MCK(cudaMemcpyAsync(t->idx, perm.data(), sizeof(int) * t->n, cudaMemcpyHostToDevice, t->stream));
            pos = 0;
        }
        int rc = run_grad(t, t->X, t->Y, t->W, t->idx + pos, batch);
        if (rc != PBS_OK) return rc;
        pos += batch;
        t->step += 1;
        const float c1 = 1.f - std::pow(b1, (float)t->step), c2 = 1.f - std::pow(b2, (float)t->step);
        k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, t->stream>>>(t->theta, t->m, t->v, t->grad, lr, b1, b2, eps, c1, c2);
        MCK(cudaGetLastError());
        if (losses) MCK(cudaMemcpyAsync(&lossbuf[sidx], t->grad + NPARAM, sizeof(float), cudaMemcpyDeviceToHost, t->stream));
        if (pos + batch > t->n) MCK(cudaStreamSynchronize(t->stream));  // perm is rewritten next step
    }
    MCK(cudaStreamSynchronize(t->stream));
    if (losses) std::memcpy(losses, lossbuf.data(), sizeof(float) * steps);
    return PBS_OK;
}

}  // extern "C"
