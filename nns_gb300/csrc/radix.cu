// radix.cu -- stable LSD radix sort passes, warp-per-tile.
//
// The body keys (63 bits) are sorted in 8 passes of 8-bit digits or 7 passes of
// 9-bit digits (nbx_params.radix_bits).  Any digit width gives the same stable
// order, so the width only trades passes against histogram size.
//
// A tile is up to 2048 consecutive keys owned by one warp (smaller for small
// systems, so that the tiles still fill the GPU).  Per pass:
//   k_radix_hist    per-tile digit counts, stored [segment][digit][tile]
//   scan            one exclusive scan over the whole count array: because the
//                   layout is segment-major, digit-major, tile-minor, the scan
//                   value IS the absolute output offset of (segment, digit, tile)
//   k_radix_scatter per-tile stable ranks (the lanes sharing a digit from bit
//                   ballots, plus per-warp running counters) into a
//                   shared-memory copy of the tile in output order, then
//                   coalesced runs per digit; the next keys' loads are in
//                   flight while the current ones are ranked.
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

// Scatter with the tile staged in shared memory in output order: every lane
// ranks its key stably (digit peers + running per-digit counters), writes it to
// its tile-local sorted position, and the warp then streams the staged tile
// out so that each digit's run is written by consecutive lanes to consecutive
// addresses (coalesced, instead of one sector per key).  The tile's count of a
// digit is the difference of adjacent entries of the scanned histogram (the
// layout is tile-minor and the scan is continuous; offs[nh] holds the total).
// A warp's stage: gbase (output offset of (digit, tile)), lstart (tile-local
// start of the digit), cnt (running tile-local position), then the tile's keys
// and values; sized for the launch's tile.
template <typename K, typename V, int Bits>
__host__ __device__ constexpr size_t stage_bytes(int tile) {
    return (3 * (size_t(1) << Bits) * sizeof(unsigned) + (size_t)tile * (sizeof(K) + sizeof(V)) + 15) & ~(size_t)15;
}

template <typename K, typename V, int Bits>
struct Stage {
    unsigned *gbase, *lstart, *cnt;
    K *key;
    V *val;
    __device__ Stage(unsigned char *base, int tile) {
        gbase = reinterpret_cast<unsigned *>(base);
        lstart = gbase + (1 << Bits);
        cnt = lstart + (1 << Bits);
        key = reinterpret_cast<K *>(cnt + (1 << Bits));
        val = reinterpret_cast<V *>(key + tile);
    }
};

template <typename K, typename V, bool Seg, int Bits>
__global__ void __launch_bounds__(kScatterWarps * 32)
    k_radix_scatter(const K *__restrict__ key_in, K *__restrict__ key_out,
                    const V *__restrict__ val_in, V *__restrict__ val_out, TileMap tm, int shift,
                    const unsigned *__restrict__ offs) {
    constexpr int kBins = 1 << Bits;
    constexpr unsigned kMask = kBins - 1;
    constexpr int kPer = kBins / 32;  // digits owned by one lane
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kScatterWarps + w;
    if (t >= tm.ntiles) return;
    int start, len, hstride;
    int64_t hbase;
    tile_info<Seg, kBins>(tm, t, start, len, hbase, hstride);
    if (len <= 0) return;
    Stage<K, V, Bits> sg(smem_raw + (size_t)w * stage_bytes<K, V, Bits>(tm.tile), tm.tile);
    // lane owns digits kPer*lane .. kPer*lane+kPer-1: counts, then the tile-local starts
    unsigned c[kPer], sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int d = kPer * lane + k;
        const int64_t idx = hbase + (int64_t)d * hstride;
        const unsigned g = offs[idx];
        c[k] = offs[idx + 1] - g;
        sg.gbase[d] = g;
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
        sg.lstart[kPer * lane + k] = run;
        sg.cnt[kPer * lane + k] = run;
        run += c[k];
    }
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    // Two groups of kBatch rounds of 32 keys: the loads of the next group are in
    // flight while the current group is ranked, so a warp keeps 2 x 8 x 32 keys
    // and values moving (the ranking is a chain of shared-memory round trips and
    // would otherwise leave the loads idle).
    constexpr int kBatch = 8;
    constexpr int kGroup = 32 * kBatch;
    K ka[kBatch], kb[kBatch];
    V va[kBatch], vb[kBatch];
    auto load = [&](K *kk, V *vv, int j0) {
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
            const int i = j0 + u * 32 + lane;
            kk[u] = i < len ? key_in[start + i] : K(0);
            if (val_in) vv[u] = i < len ? val_in[start + i] : V(0);
        }
    };
    auto rank = [&](const K *kk, const V *vv, int j0) {
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
            const int j = j0 + u * 32;
            if (j >= len) break;
            const bool valid = j + lane < len;
            const K k = kk[u];
            const unsigned d = valid ? ((unsigned)(k >> shift) & kMask) : ((unsigned)kBins + lane);
#if NBX_RADIX_MATCH
            const unsigned peers = __match_any_sync(0xffffffffu, d);
#else
            // the lanes with this lane's digit: the AND over the digit's bits of
            // the ballot of lanes agreeing on that bit (invalid lanes carry
            // digits >= kBins, which no valid digit matches)
            unsigned peers = 0xffffffffu;
#pragma unroll
            for (int b = 0; b <= Bits; b++) {
                const unsigned on = __ballot_sync(0xffffffffu, (d >> b) & 1u);
                peers &= ((d >> b) & 1u) ? on : ~on;
            }
            if (!valid) peers = 1u << lane;  // an invalid lane's digit is unique to it
#endif
            const unsigned rnk = __popc(peers & lt);
            const unsigned base = valid ? sg.cnt[d] : 0u;
            __syncwarp();
            if (valid && rnk == 0) sg.cnt[d] = base + __popc(peers);
            __syncwarp();
            if (valid) {
                sg.key[base + rnk] = k;
                if (val_in) sg.val[base + rnk] = vv[u];
            }
        }
    };
    load(ka, va, 0);
    for (int j0 = 0; j0 < len; j0 += 2 * kGroup) {
        if (j0 + kGroup < len) load(kb, vb, j0 + kGroup);
        rank(ka, va, j0);
        if (j0 + kGroup >= len) break;
        if (j0 + 2 * kGroup < len) load(ka, va, j0 + 2 * kGroup);
        rank(kb, vb, j0 + kGroup);
    }
    __syncwarp();
    for (int j = lane; j < len; j += 32) {
        const K k = sg.key[j];
        const unsigned d = (unsigned)(k >> shift) & kMask;
        const unsigned dst = sg.gbase[d] + ((unsigned)j - sg.lstart[d]);
        key_out[dst] = k;
        if (val_in) val_out[dst] = sg.val[j];
    }
}

template <typename K, typename V, bool Seg, int Bits>
int launch_scatter(Ctx *ctx, int nt, const K *kin, K *kout, const V *vin, V *vout, const TileMap &tm, int shift,
                   cudaStream_t st) {
    const size_t smem = stage_bytes<K, V, Bits>(tm.tile) * kScatterWarps;
    k_radix_scatter<K, V, Seg, Bits><<<ceil_div(nt, kScatterWarps), kScatterWarps * 32, smem, st>>>(
        kin, kout, vin, vout, tm, shift, ctx->d_hist);
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
                                  (int)(stage_bytes<unsigned long long, int, 8>(kTile) * kScatterWarps)));
    NBX_CUDA(cudaFuncSetAttribute(k_radix_scatter<unsigned long long, int, true, 9>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(stage_bytes<unsigned long long, int, 9>(kTile) * kScatterWarps)));
    NBX_CUDA(cudaFuncSetAttribute(k_radix_scatter<unsigned, int, false, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(stage_bytes<unsigned, int, 8>(kTile) * kScatterWarps)));
    return NBX_OK;
}

}  // namespace nbx
