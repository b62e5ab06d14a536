// Surface picking and drag forces: the interactive external forces of the
// reference's viewer (a face picked by a ray, then dragged), computed on the
// device from the handle's current positions.
//
//   k_pick_faces + k_pick_final   TetMesh::computeBoundfaceNormals +
//                                 TetMesh::pickFacebyRay (TetMesh.cpp:378-418)
//   k_drag_ring                   TetMesh::dragFaceRing (TetMesh.cpp:443-470)
//
// Every float operation is written with explicit round-to-nearest intrinsics
// in the reference's order (no contraction into FMA), so face ids and forces
// equal the reference's bit for bit.  Eigen 3.2 sums a fixed-size 3-vector dot
// as x0 + (x1 + x2) and a dot of two MatrixXf columns as (x0 + x1) + x2; both
// orders are kept where the reference uses them.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>

#include "../../include/phybs.h"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

namespace {

constexpr int kPickThreads = 256;

// The caller-visible position of padded node i (the value
// pbs_read_positions returns).
__device__ __forceinline__ float3 node_pos(const DevMesh &m, const float4 *uh, const float4 *ul, int i) {
    const float4 X = m.rest[i], h = uh[i], l = ul[i];
    return make_float3(state_position(X.x, h.x, l.x), state_position(X.y, h.y, l.y), state_position(X.z, h.z, l.z));
}

__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}

// a0 b0 + (a1 b1 + a2 b2): a fixed-size Eigen dot
__device__ __forceinline__ float dot_fixed(float3 a, float3 b) {
    return __fadd_rn(__fmul_rn(a.x, b.x), __fadd_rn(__fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)));
}

// (a0 b0 + a1 b1) + a2 b2: a dot of MatrixXf columns
__device__ __forceinline__ float dot_columns(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

// |x[f0.1] - x[f0.0]|: the reference's length scale (first edge of face 0)
__device__ __forceinline__ float first_edge(const DevMesh &m, const float4 *uh, const float4 *ul, int4 f0) {
    const float3 e = sub3(node_pos(m, uh, ul, f0.y), node_pos(m, uh, ul, f0.x));
    return __fsqrt_rn(dot_columns(e, e));
}

// (d2, face) ordered by d2, then by face id: the sequential scan's "first
// strict minimum"
__device__ __forceinline__ bool better(float d2, int id, float bd2, int bid) {
    return d2 < bd2 || (d2 == bd2 && id < bid);
}

__device__ __forceinline__ void block_argmin(float &d2, int &id, float *sd, int *si) {
    sd[threadIdx.x] = d2;
    si[threadIdx.x] = id;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s && better(sd[threadIdx.x + s], si[threadIdx.x + s], sd[threadIdx.x], si[threadIdx.x])) {
            sd[threadIdx.x] = sd[threadIdx.x + s];
            si[threadIdx.x] = si[threadIdx.x + s];
        }
        __syncthreads();
    }
    d2 = sd[0];
    id = si[0];
}

// Per block: the best candidate face among a grid-stride share of the faces.
// A candidate's normal ((x2 - x0) x (x1 - x0), normalised) opposes the ray and
// its centre ((x0 + x1) + x2) / 3 lies within r of the ray (squared distance
// d2 = |o|^2 - (o . dir)^2, o = orig - centre, below r^2 and 1e8).
__global__ void __launch_bounds__(kPickThreads) k_pick_faces(DevMesh m, const float4 *uh, const float4 *ul,
                                                              int n_faces, const int4 *faces, float3 orig,
                                                              float3 dir, float *blk_d2, int *blk_id) {
    __shared__ float sd[kPickThreads];
    __shared__ int si[kPickThreads];
    const float r = first_edge(m, uh, ul, faces[0]);
    const float r2 = __fmul_rn(r, r);
    float best = FLT_MAX;
    int bid = INT_MAX;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n_faces; f += gridDim.x * blockDim.x) {
        const int4 q = faces[f];
        const float3 x0 = node_pos(m, uh, ul, q.x), x1 = node_pos(m, uh, ul, q.y), x2 = node_pos(m, uh, ul, q.z);
        const float3 v1 = sub3(x1, x0), v2 = sub3(x2, x0);
        float3 n = make_float3(__fsub_rn(__fmul_rn(v2.y, v1.z), __fmul_rn(v2.z, v1.y)),
                               __fsub_rn(__fmul_rn(v2.z, v1.x), __fmul_rn(v2.x, v1.z)),
                               __fsub_rn(__fmul_rn(v2.x, v1.y), __fmul_rn(v2.y, v1.x)));
        const float nn = __fsqrt_rn(dot_fixed(n, n));
        n = make_float3(__fdiv_rn(n.x, nn), __fdiv_rn(n.y, nn), __fdiv_rn(n.z, nn));
        if (!(dot_fixed(n, dir) < 0.f)) continue;
        const float3 c = make_float3(__fdiv_rn(__fadd_rn(__fadd_rn(x0.x, x1.x), x2.x), 3.0f),
                                     __fdiv_rn(__fadd_rn(__fadd_rn(x0.y, x1.y), x2.y), 3.0f),
                                     __fdiv_rn(__fadd_rn(__fadd_rn(x0.z, x1.z), x2.z), 3.0f));
        const float3 o = sub3(orig, c);
        const float a = dot_fixed(o, o), b = dot_fixed(o, dir);
        const float d2 = __fsub_rn(a, __fmul_rn(b, b));
        if (d2 < r2 && d2 < 1e8f && better(d2, f, best, bid)) {
            best = d2;
            bid = f;
        }
    }
    block_argmin(best, bid, sd, si);
    if (threadIdx.x == 0) {
        blk_d2[blockIdx.x] = best;
        blk_id[blockIdx.x] = bid;
    }
}

__global__ void __launch_bounds__(kPickThreads) k_pick_final(int n_blk, const float *blk_d2, const int *blk_id,
                                                              int *out) {
    __shared__ float sd[kPickThreads];
    __shared__ int si[kPickThreads];
    float best = FLT_MAX;
    int bid = INT_MAX;
    for (int b = threadIdx.x; b < n_blk; b += blockDim.x)
        if (better(blk_d2[b], blk_id[b], best, bid)) {
            best = blk_d2[b];
            bid = blk_id[b];
        }
    block_argmin(best, bid, sd, si);
    if (threadIdx.x == 0) *out = bid == INT_MAX ? -1 : bid;
}

// One thread per ring entry: factor m dir on the face's own three nodes,
// (0.5 factor m) dir on the rest of the ring, where factor = min(|drag| / r *
// 100, 800) and dir = drag / |drag|.  0.5 * factor * m is formed in FP64 and
// rounded once, as the reference's double literal makes it.  A ring holds
// each node once, so the writes need no atomics; ext is zero elsewhere.
__global__ void k_drag_ring(DevMesh m, const float4 *uh, const float4 *ul, const int4 *faces, const int *ring,
                            int begin, int len, float3 drag, float4 *ext) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= len) return;
    const float r = first_edge(m, uh, ul, faces[0]);
    const float nd = __fsqrt_rn(dot_fixed(drag, drag));
    float factor = __fmul_rn(__fdiv_rn(nd, r), 100.0f);
    if (factor > 800.0f) factor = 800.0f;
    const float3 dir = make_float3(__fdiv_rn(drag.x, nd), __fdiv_rn(drag.y, nd), __fdiv_rn(drag.z, nd));
    const int node = ring[begin + j];
    const float mass = m.info[node].x;  // lumped mass; 1e8 for a pinned node, as the reference sets it
    const float s = j < 3 ? __fmul_rn(factor, mass) : (float)(0.5 * (double)factor * (double)mass);
    ext[node] = make_float4(__fmul_rn(s, dir.x), __fmul_rn(s, dir.y), __fmul_rn(s, dir.z), 0.f);
}

}  // namespace

int pick_blocks(int n_faces, int sms) {
    const int need = (n_faces + kPickThreads - 1) / kPickThreads;
    return need < 2 * sms ? (need > 0 ? need : 1) : 2 * sms;
}

cudaError_t launch_pick_face(cudaStream_t s, const DevMesh &m, const DevState &st, int n_faces, const int4 *faces,
                             float3 orig, float3 dir, int n_blk, float *blk_d2, int *blk_id, int *out) {
    k_pick_faces<<<n_blk, kPickThreads, 0, s>>>(m, st.u0h, st.u0l, n_faces, faces, orig, dir, blk_d2, blk_id);
    k_pick_final<<<1, kPickThreads, 0, s>>>(n_blk, blk_d2, blk_id, out);
    return cudaGetLastError();
}

cudaError_t launch_drag_ring(cudaStream_t s, const DevMesh &m, const DevState &st, const int4 *faces,
                             const int *ring, int begin, int len, float3 drag, float4 *ext) {
    cudaError_t e = cudaMemsetAsync(ext, 0, sizeof(float4) * (size_t)m.Np, s);
    if (e != cudaSuccess || len <= 0) return e;
    k_drag_ring<<<(len + 127) / 128, 128, 0, s>>>(m, st.u0h, st.u0l, faces, ring, begin, len, drag, ext);
    return cudaGetLastError();
}

}  // namespace pbs
