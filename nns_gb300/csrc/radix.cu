// radix.cu -- stable LSD radix sort passes, warp-per-tile.
//
// The body keys (63 bits) are sorted in 8 passes of 8-bit digits or 7 passes of
// 9-bit digits (nbx_params.radix_bits).  Any digit width gives the same stable
// order, so the width only trades passes against histogram size.
//
// A tile is up to 2048 consecutive keys (smaller for small systems, so that the
// tiles still fill the GPU).  Per pass:
//   k_radix_hist    per-tile digit counts, stored [segment][digit][tile]
//   scan            one exclusive scan over the whole count array: because the
//                   layout is segment-major, digit-major, tile-minor, the scan
//                   value IS the absolute output offset of (segment, digit, tile)
//   k_radix_scatter one block per tile: its warps rank quarters of the tile
//                   stably (digit peers from bit ballots, per-warp running
//                   counters started from the warps' digit counts) into a
//                   shared-memory copy of the tile in output order, then
//                   coalesced runs per digit.
// Segments are the independent systems of a batch, so one launch sorts every
// system's keys inside its own range; a single system is one segment.
#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kWarpsPerBlock = 8;
#ifndef NBX_RADIX_MATCH
#define NBX_RADIX_MATCH 0  // 1: rank digits with match.any instead of bit ballots
#endif

struct TileMap {
    // segmented mode
    const int4 *tiles;      // start, len, seg, local tile
    const int2 *seg_tiles;  // tile base, ntiles of the segment
    // uniform mode
    const unsigned *count;  // device-side element count
    int ntiles;             // tiles in the launch
    int tile;               // keys per tile (<= kTile)
};

template <bool Seg, int Bins>
__device__ __forceinline__ void tile_info(const TileMap &tm, int t, int &start, int &len,
                                          int64_t &hbase, int &hstride) {
    if (Seg) {
        int4 d = tm.tiles[t];
        int2 s = tm.seg_tiles[d.z];
        start = d.x;
        len = d.y;
        hbase = (int64_t)s.x * Bins + d.w;
        hstride = s.y;
    } else {
        int64_t st = (int64_t)t * tm.tile;
        int64_t n = (int64_t)*tm.count;
        start = (int)st;
        len = (int)(n > st ? (n - st < tm.tile ? n - st : tm.tile) : 0);
        hbase = t;
        hstride = tm.ntiles;
    }
}

template <typename K, bool Seg, int Bits>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_radix_hist(const K *__restrict__ key, TileMap tm, int shift, unsigned *__restrict__ hist) {
    constexpr int kBins = 1 << Bits;
    constexpr unsigned kMask = kBins - 1;
    __shared__ unsigned cnt[kWarpsPerBlock][kBins];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kWarpsPerBlock + w;
    if (t >= tm.ntiles) return;
    for (int d = lane; d < kBins; d += 32) cnt[w][d] = 0;
    __syncwarp();
    int start, len, hstride;
    int64_t hbase;
    tile_info<Seg, kBins>(tm, t, start, len, hbase, hstride);
    constexpr int kBatch = 8;  // loads in flight together (the atomics would serialise them)
    for (int i0 = 0; i0 < len; i0 += 32 * kBatch) {
        unsigned d[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
            const int i = i0 + 32 * u + lane;
            d[u] = i < len ? (unsigned)(key[start + i] >> shift) & kMask : (unsigned)kBins;
        }
#pragma unroll
        for (int u = 0; u < kBatch; u++)
            if (d[u] < (unsigned)kBins) atomicAdd(&cnt[w][d[u]], 1u);
    }
    __syncwarp();
    for (int d = lane; d < kBins; d += 32) hist[hbase + (int64_t)d * hstride] = cnt[w][d];
}

// Scatter with the tile staged in shared memory in output order.  One block of
// kScatterWarps warps per tile; warp w takes the w-th quarter (for 4 warps) of
// the tile's keys, in tile order, into registers:
//   1. each warp counts its quarter's digits (shared-memory atomics);
//   2. per digit, the warps' counts become running positions: the digit's
//      tile-local start plus the counts of the warps before (so the order stays
//      that of the tile: the sort is stable);
//   3. each warp ranks its keys batch by batch (the lanes sharing a digit from
//      bit ballots, rank among them by lane, the leader advances the warp's
//      counter) and writes them to their tile-local sorted positions;
//   4. the block streams the staged tile out so that each digit's run is written
//      by consecutive threads to consecutive addresses (coalesced).
// The tile's count of a digit is the difference of adjacent entries of the
// scanned histogram (the layout is tile-minor and the scan is continuous;
// offs[nh] holds the total).  Shared memory per block: gbase (output offset of
// (digit, tile)), lstart (tile-local start of the digit), the warps' counters,
// then the tile's keys and values.
template <typename K, typename V, int Bits>
__host__ __device__ constexpr size_t stage_bytes(int tile) {
    return ((2 + kScatterWarps) * (size_t(1) << Bits) * sizeof(unsigned) + (size_t)tile * (sizeof(K) + sizeof(V)) +
            15) & ~(size_t)15;
}

template <typename K, typename V, bool Seg, int Bits>
__global__ void __launch_bounds__(kScatterWarps * 32)
    k_radix_scatter(const K *__restrict__ key_in, K *__restrict__ key_out,
                    const V *__restrict__ val_in, V *__restrict__ val_out, TileMap tm, int shift,
                    const unsigned *__restrict__ offs) {
    constexpr int kBins = 1 << Bits;
    constexpr unsigned kMask = kBins - 1;
    constexpr int kW = kScatterWarps;
    constexpr int kPer = kBins / 32;                   // digits owned by one lane of warp 0
    constexpr int kKeys = (kTile + kW * 32 - 1) / (kW * 32);  // keys per lane at the largest tile
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x;
    if (t >= tm.ntiles) return;  // uniform over the block
    int start, len, hstride;
    int64_t hbase;
    tile_info<Seg, kBins>(tm, t, start, len, hbase, hstride);
    if (len <= 0) return;
    unsigned *gbase = reinterpret_cast<unsigned *>(smem_raw);
    unsigned *lstart = gbase + kBins;
    unsigned *wcnt = lstart + kBins;  // [kW][kBins]
    K *skey = reinterpret_cast<K *>(wcnt + kW * kBins);
    V *sval = reinterpret_cast<V *>(skey + tm.tile);
    const unsigned lt = (1u << lane) - 1u;

    // this warp's quarter [q0, q1) of the tile, whole rounds of 32 keys
    const int quarter = (((len + kW - 1) / kW) + 31) & ~31;
    const int q0 = min(len, w * quarter), q1 = min(len, q0 + quarter);
    K kk[kKeys];
    V vv[kKeys];
#pragma unroll
    for (int u = 0; u < kKeys; u++) {
        const int i = q0 + u * 32 + lane;
        kk[u] = i < q1 ? key_in[start + i] : K(0);
        if (val_in) vv[u] = i < q1 ? val_in[start + i] : V(0);
    }
    // the tile's digit counts and starts (warp 0), the warps' counters zeroed
    if (w == 0) {
        unsigned c[kPer], sum = 0;
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const int d = kPer * lane + k;
            const int64_t idx = hbase + (int64_t)d * hstride;
            const unsigned g = offs[idx];
            c[k] = offs[idx + 1] - g;
            gbase[d] = g;
            sum += c[k];
        }
        unsigned incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        unsigned run = incl - sum;
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            lstart[kPer * lane + k] = run;
            run += c[k];
        }
    }
    for (int i = threadIdx.x; i < kW * kBins; i += blockDim.x) wcnt[i] = 0u;
    __syncthreads();
    // 1. this warp's digit counts
#pragma unroll
    for (int u = 0; u < kKeys; u++)
        if (q0 + u * 32 + lane < q1) atomicAdd(&wcnt[w * kBins + ((unsigned)(kk[u] >> shift) & kMask)], 1u);
    __syncthreads();
    // 2. per digit: the warps' starting positions, in tile order
    for (int d = threadIdx.x; d < kBins; d += blockDim.x) {
        unsigned run = lstart[d];
#pragma unroll
        for (int v = 0; v < kW; v++) {
            const unsigned c = wcnt[v * kBins + d];
            wcnt[v * kBins + d] = run;
            run += c;
        }
    }
    __syncthreads();
    // 3. stable ranks within the warp, batch by batch
    unsigned *cnt = wcnt + w * kBins;
#pragma unroll
    for (int u = 0; u < kKeys; u++) {
        if (q0 + u * 32 >= q1) break;  // uniform over the warp
        const bool valid = q0 + u * 32 + lane < q1;
        const K k = kk[u];
        const unsigned d = valid ? ((unsigned)(k >> shift) & kMask) : ((unsigned)kBins + lane);
#if NBX_RADIX_MATCH
        const unsigned peers = __match_any_sync(0xffffffffu, d);
#else
        // the lanes with this lane's digit: the AND over the digit's bits of the
        // ballot of lanes agreeing on that bit (invalid lanes carry digits >= kBins,
        // which no valid digit matches)
        unsigned peers = 0xffffffffu;
#pragma unroll
        for (int b = 0; b <= Bits; b++) {
            const unsigned on = __ballot_sync(0xffffffffu, (d >> b) & 1u);
            peers &= ((d >> b) & 1u) ? on : ~on;
        }
        if (!valid) peers = 1u << lane;
#endif
        const unsigned rnk = __popc(peers & lt);
        const unsigned base = valid ? cnt[d] : 0u;
        __syncwarp();
        if (valid && rnk == 0) cnt[d] = base + __popc(peers);
        __syncwarp();
        if (valid) {
            skey[base + rnk] = k;
            if (val_in) sval[base + rnk] = vv[u];
        }
    }
    __syncthreads();
    // 4. coalesced runs per digit
    for (int j = threadIdx.x; j < len; j += blockDim.x) {
        const K k = skey[j];
        const unsigned d = (unsigned)(k >> shift) & kMask;
        const unsigned dst = gbase[d] + ((unsigned)j - lstart[d]);
        key_out[dst] = k;
        if (val_in) val_out[dst] = sval[j];
    }
}

template <typename K, typename V, bool Seg, int Bits>
int launch_scatter(Ctx *ctx, int nt, const K *kin, K *kout, const V *vin, V *vout, const TileMap &tm, int shift,
                   cudaStream_t st) {
    const size_t smem = stage_bytes<K, V, Bits>(tm.tile);
    k_radix_scatter<K, V, Seg, Bits><<<nt, kScatterWarps * 32, smem, st>>>(kin, kout, vin, vout, tm, shift,
                                                                           ctx->d_hist);
    ++ctx->launches;
    return NBX_OK;
}

template <int Bits>
int sort_bodies(Ctx *ctx, cudaStream_t st) {
    TileMap tm{ctx->d_tiles, ctx->d_sys_tiles, nullptr, ctx->ntiles_body, ctx->tile_body};
    const int nt = ctx->ntiles_body;
    if (nt == 0) return NBX_OK;
    const int grid = ceil_div(nt, kWarpsPerBlock);
    const int nh = nt * (1 << Bits);
    const int passes = radix_passes(Bits);
    // an odd pass count starts from the alternate buffers (where k_keys wrote)
    unsigned long long *k0 = ctx->d_key, *k1 = ctx->d_key_alt;
    int *v0 = ctx->d_val, *v1 = ctx->d_val_alt;
    if (passes & 1) {
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    for (int pass = 0; pass < passes; pass++) {
        const int shift = Bits * pass;
        k_radix_hist<unsigned long long, true, Bits>
            <<<grid, kWarpsPerBlock * 32, 0, st>>>(k0, tm, shift, ctx->d_hist);
        ++ctx->launches;
        int rc = scan_exclusive_u32(ctx, ctx->d_hist, ctx->d_hist, nh, nullptr, ctx->d_hist + nh, st);
        if (rc) return rc;
        launch_scatter<unsigned long long, int, true, Bits>(ctx, nt, k0, k1, v0, v1, tm, shift, st);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

}  // namespace

// Sorts the 63-bit keys of every system stably, with the sort permutation,
// into d_key / d_val.  The keys and identity values are expected in d_key /
// d_val for an even pass count and in d_key_alt / d_val_alt for an odd one
// (keys_in_alt), so that the last pass always writes d_key / d_val.
int radix_sort_bodies(Ctx *ctx, cudaStream_t st) {
    return ctx->radix_bits == 9 ? sort_bodies<9>(ctx, st) : sort_bodies<8>(ctx, st);
}

// Stable sort of the node entries (level << 26 | position) by level: one pass
// on bits 24..31, which orders by level and keeps position order within a
// level.  Input d_ent, output d_ent_alt; the element count is on the device.
int radix_sort_entries(Ctx *ctx, cudaStream_t st) {
    const int nt = ctx->cap_tiles_node;
    TileMap tm{nullptr, nullptr, &ctx->d_totals[1], nt, ctx->tile_node};  // clamped node count (0 on overflow)
    const int grid = ceil_div(nt, kWarpsPerBlock);
    const int nh = nt * 256;
    k_radix_hist<unsigned, false, 8><<<grid, kWarpsPerBlock * 32, 0, st>>>(ctx->d_ent, tm, 24, ctx->d_hist);
    ++ctx->launches;
    int rc = scan_exclusive_u32(ctx, ctx->d_hist, ctx->d_hist, nh, nullptr, ctx->d_hist + nh, st);
    if (rc) return rc;
    launch_scatter<unsigned, int, false, 8>(ctx, nt, ctx->d_ent, ctx->d_ent_alt, (const int *)nullptr, (int *)nullptr,
                                         tm, 24, st);
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

int radix_init(Ctx *ctx) {
    NBX_CUDA(cudaFuncSetAttribute(k_radix_scatter<unsigned long long, int, true, 8>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)stage_bytes<unsigned long long, int, 8>(kTile)));
    NBX_CUDA(cudaFuncSetAttribute(k_radix_scatter<unsigned long long, int, true, 9>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)stage_bytes<unsigned long long, int, 9>(kTile)));
    NBX_CUDA(cudaFuncSetAttribute(k_radix_scatter<unsigned, int, false, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)stage_bytes<unsigned, int, 8>(kTile)));
    return NBX_OK;
}

}  // namespace nbx
