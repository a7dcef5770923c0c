// noalloc.cu -- a bounding-box entry point that needs no context and allocates
// nothing (nbx_compute_bounding_box_noalloc in include/nbx.h).
//
// nbx_compute_bounding_box works through a context, and nbx_create allocates
// the whole tree pool for max_bodies up front.  Some callers cannot do that:
// a host code that already owns every body array (the way the reference's
// BarnesHut class holds its arrays and only launches kernels on them) and runs
// inside a fixed device-memory budget, or a process whose caching allocator
// has reserved the HBM, where a cudaMalloc between steps fails or stalls the
// device.  This variant takes only the caller's arrays; its scratch (one
// partial box per block and a block ticket) lives in a file-scope __device__
// array that every GPU loading libnbx.so holds until the process exits.
//
// Limits and sharing:
//  * the scratch holds kMaxBoxBlocks = 4096 block partials (128 KiB + 256 B
//    per device); a grid_size above that is rejected with NBX_ERR_SCRATCH;
//  * every call on a device shares the one array, and it keeps the last
//    call's contents: the block ticket is cleared on the stream before each
//    launch, the partials are always written before they are read, and two
//    calls whose kernels overlap on the GPU (different streams, no ordering)
//    race on it and may return wrong boxes;
//  * every call resolves the array's device address on the current device
//    (cudaGetSymbolAddress).  Once the module is loaded on a device that is a
//    host-side lookup; the first call on a device, and the first call after a
//    device reset (cudaDeviceReset ends the context, and the module is loaded
//    again, possibly at another address), may load the module: make those
//    calls before any stream capture.
#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kBoxBlock = 256;           // threads per block (as the context path)
constexpr int kMaxBoxBlocks = 4096;      // partial boxes the scratch can hold
constexpr int kPartStride = 8;           // words per partial (6 used, 32-byte rows)
constexpr int kTicketWord = kMaxBoxBlocks * kPartStride;
constexpr int kScratchWords = kTicketWord + 64;  // ticket in its own 256-byte line

// The scratch.  In host code this name is only a host-side stand-in for the
// symbol; kernels get its device address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned g_box_scratch[kScratchWords];

// Device address of the scratch in the current device's context, resolved on
// every call: no address outlives a context (a cached one would be stale after
// a device reset or in another context on the same device).
int scratch_on_current_device(unsigned **out) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_box_scratch) != cudaSuccess || !p) return NBX_ERR_CUDA;
    *out = static_cast<unsigned *>(p);
    return NBX_OK;
}

// Same per-warp reduction and the same skip of non-finite warp values as the
// context path's kernel (integrate.cu, k_bbox_ref), so that with the same grid
// the boxes are bit-identical; the warps of a block and then the blocks are
// combined on order-preserving integer images, where min/max are exact and do
// not depend on the order.  The last block to finish (block ticket) folds the
// partials into the caller's *minX..*maxZ.
__global__ void __launch_bounds__(kBoxBlock) k_bbox_noalloc(const float *__restrict__ x,
                                                             const float *__restrict__ y,
                                                             const float *__restrict__ z, int n, float *minX,
                                                             float *maxX, float *minY, float *maxY, float *minZ,
                                                             float *maxZ, unsigned *scratch) {
    __shared__ unsigned warp_box[kBoxBlock / 32][6];
    __shared__ int is_last;
    float v[6] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        v[0] = fminf(v[0], x[i]); v[1] = fmaxf(v[1], x[i]);
        v[2] = fminf(v[2], y[i]); v[3] = fmaxf(v[3], y[i]);
        v[4] = fminf(v[4], z[i]); v[5] = fmaxf(v[5], z[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 6; k += 2) {
            v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
            v[k + 1] = fmaxf(v[k + 1], __shfl_xor_sync(0xffffffffu, v[k + 1], o));
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const bool skip = isnan(v[k]) || isinf(v[k]);
            warp_box[warp][k] = skip ? ((k & 1) ? 0u : 0xffffffffu) : f2ord(v[k]);
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        unsigned r = warp_box[0][k];
        for (int w = 1; w < kBoxBlock / 32; w++) r = (k & 1) ? max(r, warp_box[w][k]) : min(r, warp_box[w][k]);
        scratch[blockIdx.x * kPartStride + k] = r;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(&scratch[kTicketWord], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    unsigned r[6] = {0xffffffffu, 0u, 0xffffffffu, 0u, 0xffffffffu, 0u};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const unsigned p = __ldcg(&scratch[b * kPartStride + k]);
            r[k] = (k & 1) ? max(r[k], p) : min(r[k], p);
        }
    }
#pragma unroll
    for (int k = 0; k < 6; k++)
        r[k] = (k & 1) ? __reduce_max_sync(0xffffffffu, r[k]) : __reduce_min_sync(0xffffffffu, r[k]);
    __syncthreads();  // every warp is done with is_last; warp_box is reused below
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 6; k++) warp_box[warp][k] = r[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float *out[6] = {minX, maxX, minY, maxY, minZ, maxZ};
#pragma unroll
        for (int k = 0; k < 6; k++) {
            unsigned a = f2ord(*out[k]);  // merge into the caller's current value
            for (int w = 0; w < kBoxBlock / 32; w++) a = (k & 1) ? max(a, warp_box[w][k]) : min(a, warp_box[w][k]);
            *out[k] = ord2f(a);
        }
    }
}

}  // namespace

}  // namespace nbx

extern "C" int nbx_compute_bounding_box_noalloc(int *mutex, const float *x, const float *y, const float *z,
                                                float *minX, float *maxX, float *minY, float *maxY, float *minZ,
                                                float *maxZ, int n, int grid_size, void *stream) {
    (void)mutex;
    if (n < 1 || !x || !y || !z || !minX || !maxX || !minY || !maxY || !minZ || !maxZ) return NBX_ERR_ARG;
    if (grid_size < 0) return NBX_ERR_ARG;
    if (grid_size > nbx::kMaxBoxBlocks) return NBX_ERR_SCRATCH;
    int grid = grid_size;
    if (grid == 0) {  // the context path's launch shape: at most 8 blocks per multiprocessor
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
            return NBX_ERR_CUDA;
        grid = (n + nbx::kBoxBlock - 1) / nbx::kBoxBlock;
        if (grid > nsm * 8) grid = nsm * 8;
        if (grid > nbx::kMaxBoxBlocks) grid = nbx::kMaxBoxBlocks;
    }
    unsigned *scratch = nullptr;
    int rc = nbx::scratch_on_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(scratch + nbx::kTicketWord, 0, sizeof(unsigned), st) != cudaSuccess) return NBX_ERR_CUDA;
    nbx::k_bbox_noalloc<<<grid, nbx::kBoxBlock, 0, st>>>(x, y, z, n, minX, maxX, minY, maxY, minZ, maxZ, scratch);
    return cudaGetLastError() == cudaSuccess ? NBX_OK : NBX_ERR_CUDA;
}
