// scan.cu -- device-wide exclusive prefix sum (reduce / scan block sums / downsweep;
// arrays of up to 8 x 4096 elements in one block and one launch).
//
// The element count may live on the device (n_dev), so a scan can be launched
// with a capacity-sized grid inside a captured graph: blocks past the count
// contribute zero and write nothing.
#include "nbx_internal.cuh"

namespace nbx {

namespace {

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Exclusive block scan of one value per thread (blockDim = 1024); returns the
// exclusive prefix and writes the block total to *total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T *total) {
    __shared__ T warp_tot[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T inc = warp_incl_scan(v);
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        T t = warp_tot[lane];
        T ti = warp_incl_scan(t);
        warp_tot[lane] = ti - t;
        if (lane == 31) *total = ti;
    }
    __syncthreads();
    T r = warp_tot[w] + inc - v;
    return r;
}

template <typename T>
__device__ __forceinline__ int scan_count(int n_cap, const unsigned *n_dev) {
    if (!n_dev) return n_cap;
    unsigned n = *n_dev;
    return n < (unsigned)n_cap ? (int)n : n_cap;
}

template <typename T>
__global__ void __launch_bounds__(1024) k_scan_reduce(const T *__restrict__ in, int n_cap,
                                                      const unsigned *n_dev, T *__restrict__ blk) {
    const int n = scan_count<T>(n_cap, n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanItems + 4 * threadIdx.x;
    T s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (base + k < n) s += in[base + k];
    __shared__ T tot;
    block_excl_scan<T>(s, &tot);
    __syncthreads();
    if (threadIdx.x == 0) blk[blockIdx.x] = tot;
}

template <typename T>
__global__ void __launch_bounds__(1024) k_scan_blocks(T *blk, int nblk, T *total_out) {
    __shared__ T tot;
    T carry = 0;
    for (int b0 = 0; b0 < nblk; b0 += 1024) {
        int i = b0 + threadIdx.x;
        T v = i < nblk ? blk[i] : T(0);
        T ex = block_excl_scan<T>(v, &tot);
        __syncthreads();
        if (i < nblk) blk[i] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

template <typename T>
__global__ void __launch_bounds__(1024) k_scan_down(const T *in, T *out, int n_cap,
                                                    const unsigned *n_dev, const T *__restrict__ blk) {
    const int n = scan_count<T>(n_cap, n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanItems + 4 * threadIdx.x;
    if ((int64_t)blockIdx.x * kScanItems >= n) return;
    T v[4];
    T s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = base + k < n ? in[base + k] : T(0);
        s += v[k];
    }
    __shared__ T tot;
    T ex = block_excl_scan<T>(s, &tot) + blk[blockIdx.x];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
}

// The whole scan in one block, chunk by chunk with a running carry: for short
// arrays (the radix histograms of small systems) one launch replaces three.
template <typename T>
__global__ void __launch_bounds__(1024) k_scan_single(const T *in, T *out, int n_cap, const unsigned *n_dev,
                                                      T *total_out) {
    const int n = scan_count<T>(n_cap, n_dev);
    __shared__ T tot;
    T carry = 0;
    for (int b0 = 0; b0 < n; b0 += kScanItems) {
        const int base = b0 + 4 * threadIdx.x;
        T v[4];
        T s = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            v[k] = base + k < n ? in[base + k] : T(0);
            s += v[k];
        }
        T ex = block_excl_scan<T>(s, &tot) + carry;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (base + k < n) out[base + k] = ex;
            ex += v[k];
        }
        carry += tot;
        __syncthreads();  // every thread has read tot before the next chunk writes it
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

#ifndef NBX_SCAN_SINGLE_BLOCKS
#define NBX_SCAN_SINGLE_BLOCKS 8
#endif
constexpr int kScanSingleBlocks = NBX_SCAN_SINGLE_BLOCKS;  // chunks of 4096 scanned in one block

template <typename T>
int scan_impl(Ctx *ctx, const T *in, T *out, int n_cap, const unsigned *n_dev, T *total_out,
              cudaStream_t st) {
    if (n_cap <= 0) return NBX_OK;
    int nblk = ceil_div(n_cap, kScanItems);
    if (nblk <= kScanSingleBlocks) {
        k_scan_single<T><<<1, 1024, 0, st>>>(in, out, n_cap, n_dev, total_out);
        ++ctx->launches;
        NBX_CUDA(cudaGetLastError());
        return NBX_OK;
    }
    if (nblk > ctx->cap_scan_blk) {
        ctx->last_error = "scan: block-sum scratch too small";
        return NBX_ERR_CAPACITY;
    }
    T *blk = reinterpret_cast<T *>(ctx->d_scan_blk);
    k_scan_reduce<T><<<nblk, 1024, 0, st>>>(in, n_cap, n_dev, blk);
    ++ctx->launches;
    k_scan_blocks<T><<<1, 1024, 0, st>>>(blk, nblk, total_out);
    ++ctx->launches;
    k_scan_down<T><<<nblk, 1024, 0, st>>>(in, out, n_cap, n_dev, blk);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

}  // namespace

int scan_exclusive_u32(Ctx *ctx, const unsigned *in, unsigned *out, int n_cap,
                       const unsigned *n_dev, unsigned *total_out, cudaStream_t st) {
    return scan_impl<unsigned>(ctx, in, out, n_cap, n_dev, total_out, st);
}

int scan_exclusive_u64(Ctx *ctx, const unsigned long long *in, unsigned long long *out, int n_cap,
                       const unsigned *n_dev, unsigned long long *total_out, cudaStream_t st) {
    return scan_impl<unsigned long long>(ctx, in, out, n_cap, n_dev, total_out, st);
}

}  // namespace nbx
