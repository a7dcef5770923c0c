// nbx_internal.cuh -- context layout and shared device helpers of libnbx.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/nbx.h"

namespace nbx {

#ifndef NBX_TILE
#define NBX_TILE 2048
#endif
constexpr int kTile = NBX_TILE;   // keys per radix tile (one warp)
#ifndef NBX_TILE_MIN
#define NBX_TILE_MIN 256
#endif
constexpr int kTileMin = NBX_TILE_MIN;  // smallest radix tile (small systems)
#ifndef NBX_TILE_SWEEP
#define NBX_TILE_SWEEP 1024
#endif
constexpr int kTileSweep = NBX_TILE_SWEEP;  // smallest tile of the one-sweep sort (shorter look-back chains)
#ifndef NBX_SCATTER_WARPS
#define NBX_SCATTER_WARPS 4
#endif
constexpr int kScatterWarps = NBX_SCATTER_WARPS;  // warps of a scatter block (one block per tile)

// Radix tile for n keys: the largest power of two <= kTile that still gives
// about 2 x kScatterWarps tiles (scatter blocks) per SM, but not below kTileMin.
inline int tile_for(long long n, int nsm) {
    const long long want = 2ll * nsm * kScatterWarps;
    int t = kTile;
    while (t > kTileMin && n < (long long)t * want) t >>= 1;
    return t;
}
constexpr int kMaxRadixBits = 9;  // body-key digits: 8 or 9 bits (histograms sized for 9)
// LSD passes over the 63-bit body keys for a digit width
constexpr int radix_passes(int bits) { return (63 + bits - 1) / bits; }
// one-sweep body sort: digit counts per system and build, the larger of
// 8 passes x 256 digits and 7 passes x 512
constexpr int kLbMaxCounts = 3584;
constexpr int kMaxLevel = 43;     // 42 key levels + the body level
constexpr int kBodyFlag = int(0x80000000u);
constexpr int kLevelShift = 26;   // build node entry = level << 26 | sorted position
constexpr int kMaxNodes = 1 << 28; // cells + bodies: meta's first-child field has 28 bits
constexpr int kScanItems = 4096;  // elements per scan block (1024 threads x 4)
constexpr int kMaxRun = 4096;     // longest run of equal 21-level keys refined

// Device-side sticky status word layout.
struct DevStatus {
    int code;          // first error code (NBX_*), 0 = ok
    int detail;        // e.g. the offending index
    int refined_runs;
    int max_level;
    unsigned long long interactions;
    unsigned long long opened;
    unsigned long long rounds;      // walk expand/evaluate rounds (production walk)
    unsigned long long candidates;  // candidates evaluated by the production walk
    unsigned walk_next;             // next group of the production walk (cleared per launch)
};

struct Ctx {
    nbx_params p;
    float theta_ref, eps2;
    int compensated;       // 0 plain, 1 split-compensated, 2 Kahan per term
    int walk_variant = 0;  // 0 production walk (walk2.cu), 2 one-cell-at-a-time walk (walk.cu)
    int walk_warps = 8;    // warps per block of the production walk
    int key_order = 0;     // 0 the reference's (Lebesgue) order, 1 Hilbert
    int radix_bits = 8;    // digit width of the body-key sort (8: 8 passes, 9: 7 passes)
    int multipole = 0;     // 0 monopoles (the reference's force), 1 with cell quadrupoles
    int leaf_size = 1;     // bodies per leaf bucket: 1 the reference's tree, 2..8 bucket leaves
    std::string last_error;

    // capacity
    int cap_bodies, cap_sys, cap_nodes, cap_tiles_body, cap_tiles_node;
    int tile_body = kTile, tile_node = kTile;  // radix tile sizes (tile_for)
    int nsm = 152;         // multiprocessors of the device
    int smem_optin = 0;    // shared memory per block (opt-in maximum)
    long long launches = 0;  // kernels launched by this context

    // systems
    int nsys = 0;
    int64_t nbodies = 0;
    int ntiles_body = 0;   // radix tiles over all systems
    int ngroups = 0;       // walk groups over all systems
    int *d_sys_off = nullptr;       // [S+1]
    int *d_body_sys = nullptr;      // [B] system of original index
    int4 *d_tiles = nullptr;        // [tiles] start, len, sys, local tile index
    int2 *d_sys_tiles = nullptr;    // [S] tile base, ntiles
    // one-sweep sort (small contexts): its own tiling of at least kTileSweep keys
    int4 *d_tiles_sw = nullptr;     // [tiles] start, len, sys, local tile index
    int2 *d_sys_tiles_sw = nullptr; // [S] tile base, ntiles
    int *d_seg_slot = nullptr;      // [S] count slot of a system of several tiles, else -1
    int ntiles_sw = 0, tile_sw = 0;
    int nslots = 0;                 // systems of several tiles (count slots in use)
    int *d_groups = nullptr;        // [G] first sorted position of each walk group

    // per-system tree parameters
    unsigned *d_bbox_u = nullptr;   // [6S] ordered-int encodings during the reduction
    float *d_bbox = nullptr;        // [6S]
    double *d_bbox64 = nullptr;     // [6S]
    float *d_depth0 = nullptr;      // [S]
    int *d_root_first = nullptr;    // [S]
    int *d_root_nch = nullptr;      // [S]
    int *d_sys_lvl = nullptr;       // [S] deepest node level of each system's tree (last build)

    // per body
    unsigned long long *d_key = nullptr, *d_key_alt = nullptr;  // [B]
    unsigned long long *d_key_lo = nullptr;                     // [B] levels 22..42 (refined runs)
    int *d_val = nullptr, *d_val_alt = nullptr;                 // [B] permutation
    float4 *d_body4 = nullptr;   // [B] sorted bodies (x,y,z,m)
    unsigned char *d_delta = nullptr;  // [B]
    unsigned char *d_bucket = nullptr; // [B] leaf buckets: level of the bucket cell of each sorted position
    unsigned *d_ecount = nullptr;      // [B] entries per position -> exclusive offsets
    int *d_body_node = nullptr;        // [B] node of sorted position
    int2 *d_gstat = nullptr;           // [G] per walk group: list length, opened cells (last walk)

    // per node (entry / BFS order)
    unsigned *d_ent = nullptr, *d_ent_alt = nullptr;  // [NC] packed level<<26 | position
    unsigned long long *d_flags = nullptr;            // [NC] cell<<32 | first-child
    float4 *d_node4 = nullptr;                        // [NC]
    int *d_meta = nullptr;                            // [NC]
    int *d_parent = nullptr;                          // [NC]
    double4 *d_sums = nullptr;                        // [NC] m, m*x, m*y, m*z (FP64)
    int *d_count = nullptr;                           // [NC]
    int *d_arrive = nullptr;                          // [NC]
    unsigned char *d_lvl8 = nullptr;                  // [NC] tree level of each node (root children: 1)
    double2 *d_m2 = nullptr;       // [3 NC] quadrupole mode: FP64 second moments about the cell's centre of
                                   // mass, (xx, yy) (zz, xy) (xz, yz)
    float4 *d_quad4 = nullptr;     // [NC] quadrupole mode: P = -Q (Q traceless) of cells in FP32, (xx, yy, zz, xy)
    float2 *d_quad2 = nullptr;     // [NC]                                              (xz, yz)
    int *d_fcl = nullptr;                             // [NC+S+1] first-child list
    int *d_cl = nullptr;                              // [NC+S] cell list (BFS index)

    // radix + scan scratch
    unsigned *d_hist = nullptr;        // [2^kMaxRadixBits * max(tiles)]
    unsigned *d_lb_counts = nullptr;   // [slots][passes][digits] one-sweep sort: digit counts of each system
    unsigned long long *d_lb_status = nullptr;  // [tiles][2^kMaxRadixBits] look-back status words
    unsigned *d_lb = nullptr;          // [16] build counter, next tile of each pass
    unsigned long long *d_scan_blk = nullptr;  // block sums
    unsigned *d_totals = nullptr;      // [8] device-side totals: 0 entries, 1 cells+first..., etc
    unsigned long long *d_totals64 = nullptr;
    int cap_scan_blk = 0;

    DevStatus *d_status = nullptr;
    DevStatus *h_status = nullptr;     // pinned mirror

    // reference-array bridge (single system)
    bool built = false;
    int ref_m = 0;         // m of the last successful nbx_build_tree (0 = none)

    // graph
    cudaGraphExec_t graph_exec = nullptr;
    unsigned graph_gen = 0;  // bumped whenever captured launches go stale (systems, constants, walk)
    nbx_state graph_state{};
    int graph_nsys = -1;
    cudaStream_t graph_stream = nullptr;
    cudaEvent_t graph_ev_in = nullptr, graph_ev_out = nullptr;  // order graph_stream against the caller's
};

// ---- host helpers ----
#define NBX_CUDA(call)                                                      \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            ctx->last_error = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return NBX_ERR_CUDA;                                            \
        }                                                                   \
    } while (0)

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// ---- device helpers ----
__device__ __forceinline__ void set_status(DevStatus *st, int code, int detail) {
    if (atomicCAS(&st->code, 0, code) == 0) st->detail = detail;
}

__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// One subdivision step along one axis (Kernels.cu:200-206): returns 1 for the
// lower half.  (double)v < 0.5*(double)(mn+mx)  <=>  v+v < fl(mn+mx), exactly;
// the new bound fl(mn+mx)*0.5 rounds as the reference's double->float store.
__device__ __forceinline__ int split_axis(float v, float &mn, float &mx) {
    float s = __fadd_rn(mn, mx);
    float h = __fmul_rn(s, 0.5f);
    if (__fadd_rn(v, v) < s) { mx = h; return 1; }
    mn = h;
    return 0;
}

// Number of leading equal 3-bit digits of two 63-bit keys (bit 63 unused).
__device__ __forceinline__ int common_digits(unsigned long long a, unsigned long long b) {
    unsigned long long x = a ^ b;
    if (x == 0ull) return 21;
    return (__clzll(x) - 1) / 3;
}

__device__ __forceinline__ int digit_of(unsigned long long hi, unsigned long long lo, int level) {
    return level <= 21 ? (int)((hi >> (3 * (21 - level))) & 7ull)
                       : (int)((lo >> (3 * (42 - level))) & 7ull);
}

// ---- kernels / launchers shared across translation units ----
// scan.cu
int scan_exclusive_u32(Ctx *ctx, const unsigned *in, unsigned *out, int n_cap,
                       const unsigned *n_dev, unsigned *total_out, cudaStream_t st);
int scan_exclusive_u64(Ctx *ctx, const unsigned long long *in, unsigned long long *out, int n_cap,
                       const unsigned *n_dev, unsigned long long *total_out, cudaStream_t st);
// radix.cu
int radix_sort_bodies(Ctx *ctx, cudaStream_t st);
int radix_sort_entries(Ctx *ctx, cudaStream_t st);
int radix_init(Ctx *ctx);
int radix_selftest_wait(Ctx *ctx, cudaStream_t st);
// tree.cu
int build_tree(Ctx *ctx, const nbx_state *s, cudaStream_t st, bool external_bbox,
               const float *const *bbox_ptrs);
// walk.cu
int walk_init(Ctx *ctx);
int walk_forces(Ctx *ctx, const nbx_state *s, cudaStream_t st);
int walk_forces_groups(Ctx *ctx, const nbx_state *s, int first, int count, cudaStream_t st);
int walk_potential(Ctx *ctx, const nbx_state *s, float *pot, cudaStream_t st);
int walk_fp64_lists(Ctx *ctx, const int *group_starts, int ngroups, double *a64, cudaStream_t st);
// integrate.cu
int integrate(Ctx *ctx, const nbx_state *s, float dt, float d, int n, cudaStream_t st);

}  // namespace nbx
