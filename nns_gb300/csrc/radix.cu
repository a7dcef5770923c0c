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
//
// Small and mid-size contexts (fewer than 1.5 x 2^20 bodies, 2^17 in a captured
// graph) sort their body keys in one launch per pass instead (k_radix_counts
// once, then the same scatter kernel in its one-sweep form on a tiling of its
// own, whose tiles find their offsets by decoupled look-back); the permutation
// is the same.
#include <cstring>

#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kWarpsPerBlock = 8;
#ifndef NBX_RADIX_MATCH
#define NBX_RADIX_MATCH 0  // 1: rank digits with match.any instead of bit ballots
#endif
#ifndef NBX_RADIX_SWEEP
#define NBX_RADIX_SWEEP 1  // body keys: 1 one-sweep passes below the size switch, 0 always histogram + scan + scatter
#endif
#ifndef NBX_RADIX_SWEEP_MAX
#define NBX_RADIX_SWEEP_MAX (3 << 19)
#endif
#ifndef NBX_RADIX_SWEEP_MAX_GRAPH
#define NBX_RADIX_SWEEP_MAX_GRAPH (1 << 17)
#endif
// One-sweep passes below this many bodies (over all systems).  They save four
// launches per pass, and with their own tiling of at least kTileSweep keys the
// look-back chains stay short.  Eager builds: 4096 bodies 0.20 against 0.24 ms,
// 2^17 0.315 against 0.403, 2^20 0.711 against 0.755; from 2^21 the counts pass
// and the look-back cost more than the launches (1.196 against 1.114 ms, 2^23
// 3.14 against 2.97).  In a captured graph a launch costs less and the switch
// comes earlier: whole graph-replayed steps of 65536 bodies 0.421 against 0.442
// ms, of 2^17 equal.
constexpr int kSweepMaxBodies = NBX_RADIX_SWEEP_MAX;
constexpr int kSweepMaxBodiesGraph = NBX_RADIX_SWEEP_MAX_GRAPH;

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
// then (one-sweep form) the system's start of each digit, then the tile's keys
// and values.
template <typename K, typename V, int Bits, bool Sweep = false>
__host__ __device__ constexpr size_t stage_bytes(int tile) {
    return ((2 + kScatterWarps + (Sweep ? 1 : 0)) * (size_t(1) << Bits) * sizeof(unsigned) +
            (size_t)tile * (sizeof(K) + sizeof(V)) + 15) & ~(size_t)15;
}

// One-sweep body sort (decoupled look-back): per pass one launch ranks and
// scatters every tile, and a tile's output offsets come from the digit counts
// of its system, counted once for all passes before the first (a stable LSD
// sort only permutes keys inside a system, so the counts do not change from
// pass to pass), plus the counts of the system's earlier tiles, which each
// tile publishes per digit in a status word: build counter and pass (32 bits),
// kind (aggregate of the tile alone, or inclusive prefix of the system up to
// it) and count (30 bits).  Tiles are taken in the order blocks start, so a
// block only ever waits for tiles taken before its own, whose blocks are
// already running and publish their aggregates before they look back
// themselves.  Every wait is bounded (NBX_ERR_TIMEOUT).
constexpr unsigned long long kLbAgg = 1ull << 30, kLbPrefix = 1ull << 31;
constexpr unsigned kLbCountMask = (1u << 30) - 1u;
constexpr int kLbSpins = 1 << 20;  // polls of one status word before giving up (an L2 load each: under a second)

struct SweepArgs {
    const int *seg_slot;          // count slot of each system (-1: the system is one tile)
    const unsigned *counts;       // [slot][pass][digit]
    unsigned long long *status;   // [tile][digit] look-back status words
    const unsigned *lb;           // [0] build counter, [1 + pass] next tile of each pass
    unsigned *lb_next;            // the same array, for the tile counters
    DevStatus *st;
    int pass;
    int n;                        // keys over all systems (writes stay below it)
};

__device__ __forceinline__ unsigned long long ld_status(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_status(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// The digit counts of every pass for every system of more than one tile: one
// pass over the keys, blocks taking contiguous tile ranges and adding their
// shared-memory counts to the system's slot when the system changes.  Block 0
// also advances the build counter and rewinds the sweeps' tile counters (the
// sweeps run after this kernel).
template <int Bits>
__global__ void __launch_bounds__(256) k_radix_counts(const unsigned long long *__restrict__ key,
                                                      const int4 *__restrict__ tiles, int ntiles,
                                                      const int *__restrict__ seg_slot, unsigned *__restrict__ counts,
                                                      unsigned *__restrict__ lb) {
    constexpr int kBins = 1 << Bits, kPasses = radix_passes(Bits);
    constexpr unsigned kMask = kBins - 1;
    extern __shared__ unsigned cnt_sh[];  // [kPasses][kBins]
    if (blockIdx.x == 0 && threadIdx.x <= kPasses) {
        if (threadIdx.x == 0) lb[0] += 1u;
        else lb[threadIdx.x] = 0u;
    }
    for (int i = threadIdx.x; i < kPasses * kBins; i += blockDim.x) cnt_sh[i] = 0u;
    __syncthreads();
    const int per = (ntiles + gridDim.x - 1) / gridDim.x;
    const int t0 = blockIdx.x * per, t1 = min(ntiles, t0 + per);
    int cur = -1;
    for (int t = t0; t <= t1; t++) {
        int slot = -1;
        int4 d = make_int4(0, 0, 0, 0);
        if (t < t1) {
            d = tiles[t];
            slot = seg_slot[d.z];
        }
        if ((t == t1 || slot != cur) && cur >= 0) {  // uniform over the block: flush the finished system
            __syncthreads();
            for (int i = threadIdx.x; i < kPasses * kBins; i += blockDim.x) {
                const unsigned v = cnt_sh[i];
                if (v) atomicAdd(&counts[(size_t)cur * kPasses * kBins + i], v);
                cnt_sh[i] = 0u;
            }
            __syncthreads();
        }
        if (t == t1) break;
        cur = slot;
        if (slot < 0) continue;  // a one-tile system ranks from its own tile
        for (int i = threadIdx.x; i < d.y; i += blockDim.x) {
            const unsigned long long k = key[d.x + i];
#pragma unroll
            for (int q = 0; q < kPasses; q++) atomicAdd(&cnt_sh[q * kBins + ((unsigned)(k >> (Bits * q)) & kMask)], 1u);
        }
    }
}

// (six blocks of 4 warps per SM: 80 registers, as the tile's keys and values
// live in registers)
template <typename K, typename V, bool Seg, int Bits, bool Sweep = false>
__global__ void __launch_bounds__(kScatterWarps * 32, 6)
    k_radix_scatter(const K *__restrict__ key_in, K *__restrict__ key_out,
                    const V *__restrict__ val_in, V *__restrict__ val_out, TileMap tm, int shift,
                    const unsigned *__restrict__ offs, SweepArgs sw) {
    static_assert(!Sweep || Seg, "the one-sweep pass runs on the systems' tiles");
    constexpr int kBins = 1 << Bits;
    constexpr unsigned kMask = kBins - 1;
    constexpr int kW = kScatterWarps;
    constexpr int kPer = kBins / 32;                   // digits owned by one lane of warp 0
    constexpr int kKeys = (kTile + kW * 32 - 1) / (kW * 32);  // keys per lane at the largest tile
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int t = blockIdx.x;
    if (Sweep) {  // tiles in the order the blocks start
        __shared__ int s_tile;
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(&sw.lb_next[1 + sw.pass], 1u);
        __syncthreads();
        t = s_tile;
    }
    if (t >= tm.ntiles) return;  // uniform over the block
    int start, len, hstride;
    int64_t hbase;
    tile_info<Seg, kBins>(tm, t, start, len, hbase, hstride);
    if (!Sweep && len <= 0) return;  // (a sweep tile always publishes its counts)
    unsigned *gbase = reinterpret_cast<unsigned *>(smem_raw);
    unsigned *lstart = gbase + kBins;
    unsigned *wcnt = lstart + kBins;  // [kW][kBins]
    unsigned *sbase = wcnt + kW * kBins;  // sweep: the system's start of each digit
    K *skey = reinterpret_cast<K *>(wcnt + kW * kBins + (Sweep ? kBins : 0));
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
    if (!Sweep && w == 0) {
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
    if (Sweep) {
        // the tile's counts, its tile-local starts and the system's digit starts
        const int4 td = tm.tiles[t];  // start, len, system, local tile
        const int slot = sw.seg_slot[td.z];
        const int ltile = td.w;
        const int seg_start = ltile == 0 ? td.x : tm.tiles[t - ltile].x;
        for (int d = threadIdx.x; d < kBins; d += blockDim.x) {
            unsigned c = 0;
#pragma unroll
            for (int v = 0; v < kW; v++) c += wcnt[v * kBins + d];
            gbase[d] = c;
        }
        __syncthreads();
        if (w == 0) {
            // (the counts are read twice, once for the lane sums and once for the
            // starts, so that no per-lane array stays live beside the tile's keys)
            constexpr int kPasses = radix_passes(Bits);
            const unsigned *gc = sw.counts + ((size_t)(slot >= 0 ? slot : 0) * kPasses + sw.pass) * kBins;
            unsigned sum = 0, gsum = 0;
#pragma unroll
            for (int k = 0; k < kPer; k++) {
                const int d = kPer * lane + k;
                const unsigned c = gbase[d];
                sum += c;
                gsum += slot >= 0 ? gc[d] : c;
            }
            unsigned incl = sum, gincl = gsum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
                const unsigned gu = __shfl_up_sync(0xffffffffu, gincl, o);
                if (lane >= o) {
                    incl += u;
                    gincl += gu;
                }
            }
            unsigned run = incl - sum, grun = (unsigned)seg_start + gincl - gsum;
#pragma unroll
            for (int k = 0; k < kPer; k++) {
                const int d = kPer * lane + k;
                const unsigned c = gbase[d];
                lstart[d] = run;
                sbase[d] = grun;
                run += c;
                grun += slot >= 0 ? gc[d] : c;
            }
        }
        __syncthreads();
        // the counts of the system's earlier tiles, per digit (decoupled look-back):
        // first this tile's own counts for every digit (the system's first tile
        // publishes them as its prefix), then the walk back over earlier tiles
        const unsigned ep = sw.lb[0] * 16u + (unsigned)sw.pass + 1u;
        const unsigned long long tag = (unsigned long long)ep << 32;
        if (slot >= 0)
            for (int d = threadIdx.x; d < kBins; d += blockDim.x)
                st_status(sw.status + (size_t)t * kBins + d, tag | (ltile == 0 ? kLbPrefix : kLbAgg) | gbase[d]);
        bool expired = false;
        for (int d = threadIdx.x; d < kBins; d += blockDim.x) {
            const unsigned c = gbase[d];
            unsigned excl = 0;
            if (slot >= 0 && ltile > 0) {
                int j = t - 1;
                for (int it = 0; !expired;) {
                    const unsigned long long v = ld_status(sw.status + (size_t)j * kBins + d);
                    if ((unsigned)(v >> 32) != ep) {
                        if (++it > kLbSpins) {
                            expired = true;
                            set_status(sw.st, NBX_ERR_TIMEOUT, t);
                            break;
                        }
                        __nanosleep(32);
                        continue;
                    }
                    excl += (unsigned)v & kLbCountMask;
                    if (v & kLbPrefix) break;
                    --j;  // an aggregate: go on to the tile before (the system's first tile holds a prefix)
                }
                st_status(sw.status + (size_t)t * kBins + d, tag | kLbPrefix | ((excl + c) & kLbCountMask));
            }
            gbase[d] = sbase[d] + excl;
        }
        __syncthreads();
    }
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
        if (Sweep && dst >= (unsigned)sw.n) continue;  // only after an expired wait (reported)
        key_out[dst] = k;
        if (val_in) val_out[dst] = sval[j];
    }
}

template <typename K, typename V, bool Seg, int Bits>
int launch_scatter(Ctx *ctx, int nt, const K *kin, K *kout, const V *vin, V *vout, const TileMap &tm, int shift,
                   cudaStream_t st) {
    const size_t smem = stage_bytes<K, V, Bits>(tm.tile);
    k_radix_scatter<K, V, Seg, Bits><<<nt, kScatterWarps * 32, smem, st>>>(kin, kout, vin, vout, tm, shift,
                                                                           ctx->d_hist, SweepArgs{});
    ++ctx->launches;
    return NBX_OK;
}

// One-sweep sort of the body keys: the counts of every pass, then one launch
// per pass.
template <int Bits>
int sort_bodies_sweep(Ctx *ctx, cudaStream_t st) {
    TileMap tm{ctx->d_tiles_sw, ctx->d_sys_tiles_sw, nullptr, ctx->ntiles_sw, ctx->tile_sw};
    const int nt = ctx->ntiles_sw;
    if (nt == 0) return NBX_OK;
    constexpr int kBins = 1 << Bits, kPasses = radix_passes(Bits);
    unsigned long long *k0 = ctx->d_key, *k1 = ctx->d_key_alt;
    int *v0 = ctx->d_val, *v1 = ctx->d_val_alt;
    if (kPasses & 1) {
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    if (ctx->nslots > 0)
        NBX_CUDA(cudaMemsetAsync(ctx->d_lb_counts, 0, sizeof(unsigned) * (size_t)ctx->nslots * kPasses * kBins, st));
    const int cgrid = ctx->nslots > 0 ? (nt < 2 * ctx->nsm ? nt : 2 * ctx->nsm) : 1;
    k_radix_counts<Bits><<<cgrid, 256, sizeof(unsigned) * kPasses * kBins, st>>>(k0, ctx->d_tiles_sw, nt,
                                                                                ctx->d_seg_slot, ctx->d_lb_counts,
                                                                                ctx->d_lb);
    ++ctx->launches;
    const size_t smem = stage_bytes<unsigned long long, int, Bits, true>(tm.tile);
    for (int pass = 0; pass < kPasses; pass++) {
        SweepArgs sw{ctx->d_seg_slot, ctx->d_lb_counts, ctx->d_lb_status, ctx->d_lb, ctx->d_lb, ctx->d_status, pass,
                     ctx->nbodies};
        k_radix_scatter<unsigned long long, int, true, Bits, true>
            <<<nt, kScatterWarps * 32, smem, st>>>(k0, k1, v0, v1, tm, Bits * pass, nullptr, sw);
        ++ctx->launches;
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    NBX_CUDA(cudaGetLastError());
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
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    NBX_CUDA(cudaStreamIsCapturing(st, &cs));
    const int lim = cs == cudaStreamCaptureStatusActive ? kSweepMaxBodiesGraph : kSweepMaxBodies;
    if (NBX_RADIX_SWEEP && ctx->nbodies < lim)
        return ctx->radix_bits == 9 ? sort_bodies_sweep<9>(ctx, st) : sort_bodies_sweep<8>(ctx, st);
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

// Self-test of the one-sweep pass's bounded wait (nbx_selftest_sort_wait): a
// system of two 256-key tiles on scratch of its own, whose tile counter starts
// at 1, so the one block takes the second tile, publishes its counts and waits
// for the first tile's, which nothing writes.
int radix_selftest_wait(Ctx *ctx, cudaStream_t st) {
    constexpr int kT = 256, kN = 2 * kT;
    struct Scratch {
        int4 tiles[2];
        int2 seg_tiles[1];
        int seg_slot[1];
        unsigned lb[16];
        unsigned counts[kLbMaxCounts];
        unsigned long long status[2 << kMaxRadixBits];
        unsigned long long key_in[kN], key_out[kN];
        int val_in[kN], val_out[kN];
    };
    Scratch *d = nullptr;
    NBX_CUDA(cudaMalloc(&d, sizeof(Scratch)));
    Scratch h;
    std::memset(&h, 0, sizeof(h));
    h.tiles[0] = make_int4(0, kT, 0, 0);
    h.tiles[1] = make_int4(kT, kT, 0, 1);
    h.seg_tiles[0] = make_int2(0, 2);
    h.seg_slot[0] = 0;
    h.lb[0] = 1;  // build counter: status tags of 1 * 16 + pass + 1, none of them written
    h.lb[1] = 1;  // the pass's next tile: the second
    h.counts[0] = kN;  // every key (0) has digit 0 in every pass
    int rc = NBX_OK;
    if (cudaMemcpyAsync(d, &h, sizeof(Scratch), cudaMemcpyHostToDevice, st) != cudaSuccess) rc = NBX_ERR_CUDA;
    if (rc == NBX_OK) {
        TileMap tm{d->tiles, d->seg_tiles, nullptr, 2, kT};
        SweepArgs sw{d->seg_slot, d->counts, d->status, d->lb, d->lb, ctx->d_status, 0, kN};
        k_radix_scatter<unsigned long long, int, true, 8, true>
            <<<1, kScatterWarps * 32, stage_bytes<unsigned long long, int, 8, true>(kT), st>>>(
                d->key_in, d->key_out, d->val_in, d->val_out, tm, 0, nullptr, sw);
        ++ctx->launches;
        if (cudaGetLastError() != cudaSuccess) rc = NBX_ERR_CUDA;
    }
    // the scratch (and the host copy) outlive the pass
    if (cudaStreamSynchronize(st) != cudaSuccess) rc = NBX_ERR_CUDA;
    cudaFree(d);
    return rc;
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
    NBX_CUDA(cudaFuncSetAttribute(k_radix_scatter<unsigned long long, int, true, 8, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)stage_bytes<unsigned long long, int, 8, true>(kTile)));
    NBX_CUDA(cudaFuncSetAttribute(k_radix_scatter<unsigned long long, int, true, 9, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)stage_bytes<unsigned long long, int, 9, true>(kTile)));
    return NBX_OK;
}

}  // namespace nbx
