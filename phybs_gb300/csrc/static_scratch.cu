// pbs_eval_nodes_static: elastic node forces with no device allocation in
// the call.
//
// Some callers cannot allocate device memory while they run the solver:
//   * a frame loop that must not stall: cudaMalloc and cudaFree synchronise
//     the whole device, so one allocation inside a frame waits for every
//     stream's work (the renderer's included);
//   * a host application that reserves all device memory up front for its own
//     pool: a cudaMalloc of the library then fails, or evicts the pool.
// This entry point evaluates what pbs_eval_nodes evaluates (the per-tet
// corner forces, then the deterministic per-node gather), but it takes the
// positions and the forces in device memory and keeps its scratch, the 12
// corner-force components of each tet, in one array of fixed size that is
// part of the library's device image.  The array is 24 MiB (524,288 tets
// after per-instance padding; PBS_EVAL_STATIC_MAX_TETS).  Larger handles are
// rejected with PBS_E_CAPACITY.
//
// Set-up: the first call on a device looks up the array's device address
// with that device current (cudaGetSymbolAddress) and keeps it, together with
// the identity of the device's CUDA context, for the later calls on that
// device.  That first call should come before any stream capture.  A later
// call that finds another context current (the caller reset the device with
// cudaDeviceReset, which unloads the library's device image) looks the
// address up again, so no call writes through an address of a context that
// no longer exists; that call too should come before any capture.
//
// Every call on a device shares the one array.  Two calls whose kernels
// overlap on the GPU (on different streams: two handles, or two threads with
// no ordering between them) race on it and corrupt each other's forces; order
// them on one stream or with events.  Nothing in the array has to start at
// zero: the second kernel of a call reads only the slots the first kernel of
// the same call has written.
#include <cuda.h>  // CUcontext / CUresult of the two driver calls looked up below
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/phybs.h"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

using namespace pbs;

namespace {

constexpr int kBlock = 128;
constexpr int kMaxDevices = 64;

// 12 floats per padded tet: corner c's force at [12 t + 3 c, 12 t + 3 c + 2].
static __device__ __align__(256) float g_corner_scratch[12 * (size_t)PBS_EVAL_STATIC_MAX_TETS];

// Per device: the scratch address and the id of the context it belongs to.
struct ScratchSlot {
    float *ptr = nullptr;
    unsigned long long ctx_id = 0;
};
ScratchSlot g_slot[kMaxDevices];
std::mutex g_setup_mutex;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// Unique id (for the process's lifetime) of the current CUDA context, or 0
// when the driver cannot tell.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of g_corner_scratch on `device` (which is current): looked
// up once per device and context.  Without a context id (an old driver) it is
// looked up on every call.
int scratch_for_device(int device, float **out) {
    if (device < 0 || device >= kMaxDevices) return PBS_E_CAPACITY;
    const unsigned long long id = current_context_id();
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ScratchSlot &s = g_slot[device];
    if (!s.ptr || id == 0 || s.ctx_id != id) {
        void *addr = nullptr;
        if (cudaGetSymbolAddress(&addr, g_corner_scratch) != cudaSuccess || !addr) {
            cudaGetLastError();
            s = ScratchSlot();
            return PBS_E_CUDA;
        }
        s.ptr = static_cast<float *>(addr);
        s.ctx_id = id;
    }
    *out = s.ptr;
    return PBS_OK;
}

// Displacement of padded node i from caller-order positions: the rounded
// difference x - X, the same word the position upload keeps as the state's
// high part.
__device__ __forceinline__ float4 node_disp(const DevMesh &m, const float *x, const int *pad2user, int i) {
    const int u = pad2user[i];
    const float4 X = m.rest[i];
    const float *p = x + 3 * (size_t)u;
    return make_float4(__fadd_rn(p[0], -X.x), __fadd_rn(p[1], -X.y), __fadd_rn(p[2], -X.z), 0.f);
}

template <int MATERIAL>
__global__ void __launch_bounds__(kBlock) k_static_corners(DevMesh m, const float *x, const int *pad2user,
                                                           float *scratch) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.Tp) return;
    const int4 q = m.tets[t];
    float f[12] = {0};
    if (q.x >= 0) {
        const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        Kin<float> kin;
        disp_gradient<float>(node_disp(m, x, pad2user, q.x), node_disp(m, x, pad2user, q.y),
                             node_disp(m, x, pad2user, q.z), node_disp(m, x, pad2user, q.w), dinv, kin.G);
        kinematics(kin);
        float P[9];
        if (MATERIAL == PBS_MATERIAL_STRETCH) pk1_stretch(kin, r1.w, r2.w, P);
        else pk1_neohookean<float>(kin, r1.w, r2.w, P);
        corner_forces(P, dinv, r0.w, f);
    }
    float4 *dst = reinterpret_cast<float4 *>(scratch + 12 * (size_t)t);  // 48-byte rows of a 256-aligned array
    dst[0] = make_float4(f[0], f[1], f[2], f[3]);
    dst[1] = make_float4(f[4], f[5], f[6], f[7]);
    dst[2] = make_float4(f[8], f[9], f[10], f[11]);
}

// Node sums in the incidence order (ascending tet, then corner), as the
// gather of pbs_eval_nodes adds them.
__global__ void __launch_bounds__(kBlock) k_static_gather(DevMesh m, const float *scratch, const int *pad2user,
                                                          float *forces) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int u = pad2user[i];
    if (u < 0) return;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
        const int ent = m.inc[j];
        const float *c = scratch + 12 * (size_t)(ent >> 2) + 3 * (ent & 3);
        s0 += c[0];
        s1 += c[1];
        s2 += c[2];
    }
    forces[3 * (size_t)u] = s0;
    forces[3 * (size_t)u + 1] = s1;
    forces[3 * (size_t)u + 2] = s2;
}

// True when p is 4-byte aligned memory of `device` that kernels can read.
bool device_floats(const void *p, int device) {
    if (reinterpret_cast<uintptr_t>(p) % alignof(float)) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == device;
}

}  // namespace

int pbs_eval_nodes_static(pbs_handle *h, const float *positions, float *forces) {
    if (!h || !positions || !forces) return PBS_E_INVALID_ARG;
    HandleView v;
    handle_view(h, &v);
    if (v.mesh.Tp > PBS_EVAL_STATIC_MAX_TETS) return PBS_E_CAPACITY;
    PBS_DEVICE_SCOPE(v.device);
    float *scratch = nullptr;
    int rc = scratch_for_device(v.device, &scratch);
    if (rc != PBS_OK) return rc;
    if (!device_floats(positions, v.device) || !device_floats(forces, v.device)) return PBS_E_INVALID_ARG;
    const int tb = (v.mesh.Tp + kBlock - 1) / kBlock, nb = (v.mesh.Np + kBlock - 1) / kBlock;
    if (v.material == PBS_MATERIAL_STRETCH)
        k_static_corners<PBS_MATERIAL_STRETCH><<<tb, kBlock, 0, v.stream>>>(v.mesh, positions, v.pad2user, scratch);
    else
        k_static_corners<PBS_MATERIAL_NEOHOOKEAN><<<tb, kBlock, 0, v.stream>>>(v.mesh, positions, v.pad2user,
                                                                               scratch);
    k_static_gather<<<nb, kBlock, 0, v.stream>>>(v.mesh, scratch, v.pad2user, forces);
    return cudaGetLastError() == cudaSuccess ? PBS_OK : PBS_E_CUDA;
}
