// Allocation-free absorbing-boundary update.
//
// rtm_k_Hybrid1 + rtm_k_Hybrid2 need a caller-allocated full-grid scratch
// array (DFWb) for the one-way values of the pad cells.  Some callers cannot
// allocate device memory at the point where they advance a wavefield: a host
// application whose device memory is owned by its own pool or allocator, or
// a time loop that must not call cudaMalloc because cudaMalloc can
// synchronise the device.  rtm_k_HybridStatic does the same update with its
// scratch in a fixed device array that this library defines at file scope,
// so it allocates nothing.
//
// Limits and sharing:
//   * the scratch holds RTM_STATIC_PAD_CELLS values, one per pad cell
//     (NZ*NX - (NZ-2*N2)*(NX-2*N2)); larger pads are rejected;
//   * every GPU that loads this library holds the array (4 MiB) until the
//     process exits;
//   * all calls share the array: two calls that overlap on the GPU (different
//     streams, or different host threads) race on it and must be ordered by
//     the caller;
//   * nothing needs to start at zero: each call writes every scratch value
//     it later reads, so the previous call's contents never leak.
//
// Set-up: host code cannot use the array's name as a device address (it is a
// host-side stand-in), so the first call on each device looks the device
// address up with cudaGetSymbolAddress while that device is current and
// caches it together with the unique id of the device's current context.
// A call that finds a different context (the device was reset and its
// context re-created, which can move the array) looks the address up again.
// The first call on a device, and the first after a reset, should therefore
// come before any stream capture.
#include <cudaTypedefs.h>

#include <mutex>

#include "rtm_common.cuh"

#define RTM_STATIC_PAD_CELLS (1 << 20)

static __device__ __align__(256) float g_static_pad_scratch[RTM_STATIC_PAD_CELLS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
float *g_scratch_ptr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};  // context id the address belongs to

// Unique id of the calling thread's current context (cuCtxGetId: unique for
// the life of the process, so a re-created context never matches an old id).
// Returns RTM_OK, 1 when no context is current yet, or an error code.
int current_context_id(unsigned long long *id)
{
    static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    if (!get_cur || !get_id) {
        void *p = nullptr, *q = nullptr;
        cudaDriverEntryPointQueryResult r1, r2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &r1) !=
                cudaSuccess || r1 != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2) !=
                cudaSuccess || r2 != cudaDriverEntryPointSuccess) {
            rtm_set_last_error("rtm_k_HybridStatic: driver context queries unavailable");
            return RTM_ERR_CUDA;
        }
        get_cur = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(q);
    }
    CUcontext ctx = nullptr;
    if (get_cur(&ctx) != CUDA_SUCCESS) {
        rtm_set_last_error("rtm_k_HybridStatic: cuCtxGetCurrent failed");
        return RTM_ERR_CUDA;
    }
    if (!ctx) return 1;
    if (get_id(ctx, id) != CUDA_SUCCESS) {
        rtm_set_last_error("rtm_k_HybridStatic: cuCtxGetId failed");
        return RTM_ERR_CUDA;
    }
    return RTM_OK;
}

int scratch_for_current_device(float **out)
{
    int dev = 0;
    RTM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        rtm_set_last_error("rtm_k_HybridStatic: device ordinal out of range");
        return RTM_ERR_ARG;
    }
    unsigned long long ctx = 0;
    const int have = current_context_id(&ctx);
    if (have < 0) return have;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (have != RTM_OK || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        // (the lookup also makes the device's primary context current)
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_pad_scratch);
        if (e != cudaSuccess) {
            rtm_set_last_error(cudaGetErrorString(e));
            return RTM_ERR_CUDA;
        }
        if (int rc = current_context_id(&ctx)) return rc < 0 ? rc : RTM_ERR_CUDA;
        g_scratch_ptr[dev] = static_cast<float *>(p);
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_ptr[dev];
    return RTM_OK;
}

// One-way value of pad cell t (compact enumeration) into b[t]; same update
// as Hybrid1 / BKHybrid1 (kernel.cu:116-158, 421-463).
__global__ void k_static_oneway(const float *__restrict__ u1, const float *__restrict__ u0,
                                const float *__restrict__ u2, float *__restrict__ b,
                                const float *__restrict__ v, const float *__restrict__ r1, int NZ,
                                int NX, int N2, float taoh, float taoh2)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= abc_count(NZ, NX, N2)) return;
    const AbcCell cc = abc_cell(t, NZ, NX, N2);
    const int z = cc.z, x = cc.x;
    const long c = (long)z * NX + x;
    const int a = min(z, NZ - 1 - z), e = min(x, NX - 1 - x);
    const int dz = (z < NZ - 1 - z) ? 1 : -1, dx = (x < NX - 1 - x) ? 1 : -1;
    float val;
    if (e >= a + 2 || a >= e + 2) {
        long n, s, q;
        if (e >= a + 2) {
            n = c + (long)dz * NX;
            s = 1;
            q = (dz > 0) ? c : (long)(NZ - 1 - z) * NX + x;
        } else {
            n = c + dx;
            s = NX;
            q = (dx > 0) ? (long)x * NX + z : (long)(NX - 1 - x) * NX + z;
        }
        const float vc = v[c], vq = v[q];
        val = 1.0f / (taoh * vc + 1.0f) *
              (taoh * vc * (u2[n] - u0[n] + u0[c]) -
               (-2.0f * u1[c] + u0[c] + u2[n] - 2.0f * u1[n] + u0[n]) +
               taoh2 * vq * vq *
                   (u2[n + s] - 2.0f * u2[n] + u2[n - s] + u0[c + s] - 2.0f * u0[c] + u0[c - s]));
    } else {
        const float rr = r1[c];
        val = 1.0f / (2.0f * rr + 1.0f) * (u1[c] + rr * (u2[c + dx] + u2[c + (long)dz * NX]));
    }
    b[t] = val;
}

// Blend of Hybrid2 / BKHybrid2 (kernel.cu:160-183, 464-487).
__global__ void k_static_blend(float *__restrict__ u2, const float *__restrict__ b,
                               const float *__restrict__ w, int NZ, int NX, int N2)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= abc_count(NZ, NX, N2)) return;
    const AbcCell cc = abc_cell(t, NZ, NX, N2);
    const long c = (long)cc.z * NX + cc.x;
    const float wj = w[blend_index(cc.z, cc.x, NZ, NX, N2)];
    u2[c] = (1.0f - wj) * u2[c] + wj * b[t];
}

}  // namespace

extern "C" int rtm_k_HybridStatic(float *DFW1, float *DFW0, float *DFW2, float *Dv, float *Dr_1,
                                  float *Dw, int NZ, int NX, int N2, float taoh, float taoh2,
                                  rtm_stream_t s)
{
    if (!DFW1 || !DFW0 || !DFW2 || !Dv || !Dr_1 || !Dw || NZ <= 2 * N2 || NX <= 2 * N2 || N2 < 2) {
        rtm_set_last_error("rtm_k_HybridStatic: invalid grid or null buffer");
        return RTM_ERR_ARG;
    }
    const long n = abc_count(NZ, NX, N2);
    if (n > RTM_STATIC_PAD_CELLS) {
        rtm_set_last_error("rtm_k_HybridStatic: the pad has more cells than the fixed scratch "
                           "holds (1048576); use rtm_k_Hybrid1/rtm_k_Hybrid2 with a caller buffer");
        return RTM_ERR_ARG;
    }
    float *scratch = nullptr;
    if (int rc = scratch_for_current_device(&scratch)) return rc;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_static_oneway<<<blocks, 256, 0, s>>>(DFW1, DFW0, DFW2, scratch, Dv, Dr_1, NZ, NX, N2, taoh,
                                           taoh2);
    k_static_blend<<<blocks, 256, 0, s>>>(DFW2, scratch, Dw, NZ, NX, N2);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}
