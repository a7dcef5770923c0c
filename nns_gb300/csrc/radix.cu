// radix.cu -- stable LSD radix sort passes (8-bit digits), warp-per-tile.
//
// A tile is 2048 consecutive keys owned by one warp.  Per pass:
//   k_radix_hist    per-tile digit counts, stored [segment][digit][tile]
//   scan            one exclusive scan over the whole count array: because the
//                   layout is segment-major, digit-major, tile-minor, the scan
//                   value IS the absolute output offset of (segment, digit, tile)
//   k_radix_scatter per-tile stable ranks (warp match + per-warp running
//                   counters) and the scatter.
// Segments are the independent systems of a batch, so one launch sorts every
// system's keys inside its own range; a single system is one segment.
#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kWarpsPerBlock = 8;

struct TileMap {
    // segmented mode
    const int4 *tiles;      // start, len, seg, local tile
    const int2 *seg_tiles;  // tile base, ntiles of the segment
    // uniform mode
    const unsigned *count;  // device-side element count
    int ntiles;             // tiles in the launch
};

template <bool Seg>
__device__ __forceinline__ void tile_info(const TileMap &tm, int t, int &start, int &len,
                                          int64_t &hbase, int &hstride) {
    if (Seg) {
        int4 d = tm.tiles[t];
        int2 s = tm.seg_tiles[d.z];
        start = d.x;
        len = d.y;
        hbase = (int64_t)s.x * kRadixBins + d.w;
        hstride = s.y;
    } else {
        int64_t st = (int64_t)t * kTile;
        int64_t n = (int64_t)*tm.count;
        start = (int)st;
        len = (int)(n > st ? (n - st < kTile ? n - st : kTile) : 0);
        hbase = t;
        hstride = tm.ntiles;
    }
}

template <typename K, bool Seg>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_radix_hist(const K *__restrict__ key, TileMap tm, int shift, unsigned *__restrict__ hist) {
    __shared__ unsigned cnt[kWarpsPerBlock][kRadixBins];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kWarpsPerBlock + w;
    if (t >= tm.ntiles) return;
    for (int d = lane; d < kRadixBins; d += 32) cnt[w][d] = 0;
    __syncwarp();
    int start, len, hstride;
    int64_t hbase;
    tile_info<Seg>(tm, t, start, len, hbase, hstride);
    for (int i = lane; i < len; i += 32) {
        unsigned d = (unsigned)(key[start + i] >> shift) & 0xffu;
        atomicAdd(&cnt[w][d], 1u);
    }
    __syncwarp();
    for (int d = lane; d < kRadixBins; d += 32) hist[hbase + (int64_t)d * hstride] = cnt[w][d];
}

template <typename K, typename V, bool Seg>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_radix_scatter(const K *__restrict__ key_in, K *__restrict__ key_out,
                    const V *__restrict__ val_in, V *__restrict__ val_out, TileMap tm, int shift,
                    const unsigned *__restrict__ offs) {
    __shared__ unsigned cnt[kWarpsPerBlock][kRadixBins];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kWarpsPerBlock + w;
    if (t >= tm.ntiles) return;
    int start, len, hstride;
    int64_t hbase;
    tile_info<Seg>(tm, t, start, len, hbase, hstride);
    if (len <= 0) return;
    for (int d = lane; d < kRadixBins; d += 32) cnt[w][d] = offs[hbase + (int64_t)d * hstride];
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    constexpr int kBatch = 8;  // rounds whose loads are in flight together
    for (int j0 = 0; j0 < len; j0 += 32 * kBatch) {
        K kk[kBatch];
        V vv[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
            const int i = j0 + u * 32 + lane;
            kk[u] = i < len ? key_in[start + i] : K(0);
            if (val_in) vv[u] = i < len ? val_in[start + i] : V(0);
        }
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
            const int j = j0 + u * 32;
            if (j >= len) break;
            const bool valid = j + lane < len;
            const K k = kk[u];
            unsigned d = valid ? ((unsigned)(k >> shift) & 0xffu) : (0x100u + lane);
            unsigned peers = __match_any_sync(0xffffffffu, d);
            unsigned rank = __popc(peers & lt);
            unsigned base = valid ? cnt[w][d] : 0u;
            __syncwarp();
            if (valid && rank == 0) cnt[w][d] = base + __popc(peers);
            __syncwarp();
            if (valid) {
                unsigned dst = base + rank;
                key_out[dst] = k;
                if (val_in) val_out[dst] = vv[u];
            }
        }
    }
}

}  // namespace

// Sorts (d_key, d_val) of every system by the 63-bit key, stably, in place
// (8 passes, result back in d_key / d_val).
int radix_sort_bodies(Ctx *ctx, cudaStream_t st) {
    TileMap tm{ctx->d_tiles, ctx->d_sys_tiles, nullptr, ctx->ntiles_body};
    const int nt = ctx->ntiles_body;
    if (nt == 0) return NBX_OK;
    const int grid = ceil_div(nt, kWarpsPerBlock);
    const int nh = nt * kRadixBins;
    unsigned long long *k0 = ctx->d_key, *k1 = ctx->d_key_alt;
    int *v0 = ctx->d_val, *v1 = ctx->d_val_alt;
    for (int pass = 0; pass < 8; pass++) {
        const int shift = 8 * pass;
        k_radix_hist<unsigned long long, true>
            <<<grid, kWarpsPerBlock * 32, 0, st>>>(k0, tm, shift, ctx->d_hist);
        ++ctx->launches;
        int rc = scan_exclusive_u32(ctx, ctx->d_hist, ctx->d_hist, nh, nullptr, nullptr, st);
        if (rc) return rc;
        k_radix_scatter<unsigned long long, int, true>
            <<<grid, kWarpsPerBlock * 32, 0, st>>>(k0, k1, v0, v1, tm, shift, ctx->d_hist);
        ++ctx->launches;
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

// Stable sort of the node entries (level << 26 | position) by level: one pass
// on bits 24..31, which orders by level and keeps position order within a
// level.  Input d_ent, output d_ent_alt; the element count is on the device.
int radix_sort_entries(Ctx *ctx, cudaStream_t st) {
    const int nt = ctx->cap_tiles_node;
    TileMap tm{nullptr, nullptr, &ctx->d_totals[1], nt};  // clamped node count (0 on overflow)
    const int grid = ceil_div(nt, kWarpsPerBlock);
    const int nh = nt * kRadixBins;
    k_radix_hist<unsigned, false><<<grid, kWarpsPerBlock * 32, 0, st>>>(ctx->d_ent, tm, 24, ctx->d_hist);
    ++ctx->launches;
    int rc = scan_exclusive_u32(ctx, ctx->d_hist, ctx->d_hist, nh, nullptr, nullptr, st);
    if (rc) return rc;
    k_radix_scatter<unsigned, int, false><<<grid, kWarpsPerBlock * 32, 0, st>>>(
        ctx->d_ent, ctx->d_ent_alt, (const int *)nullptr, (int *)nullptr, tm, 24, ctx->d_hist);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

}  // namespace nbx
