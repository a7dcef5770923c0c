// api.cu -- the C ABI of libnbx: context, reference-compatible phase entry
// points (3D/CUDA/CUDA_NBody/src/KernelsWrapper.cu) and the native pipeline.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "nbx_internal.cuh"
#include "nvtx3/nvToolsExt.h"

namespace {
// NVTX range around an entry point: phases show up by name in a profiler's
// timeline (near-free when no tool is attached)
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};
}  // namespace

namespace nbx {
int build_tree(Ctx *ctx, const nbx_state *s, cudaStream_t st, bool external_bbox, const float *const *bbox_ptrs);
int export_tree_impl(Ctx *ctx, int sys, int *perm, int *root_child, int *cell_child, int *cell_start,
                     int *cell_count, int *cell_level, float *cx, float *cy, float *cz, float *cm, int cap_cells,
                     int64_t *ncells, cudaStream_t st, int sum_mode);
int reset_ref_arrays(Ctx *ctx, int *mutex, float *x, float *y, float *z, float *mass, int *count, int *start,
                     int *sorted, int *child, int *index, float *minX, float *maxX, float *minY, float *maxY,
                     float *minZ, float *maxZ, int n, int m, cudaStream_t st);
int bbox_ref(Ctx *ctx, const float *x, const float *y, const float *z, float *minX, float *maxX, float *minY,
             float *maxY, float *minZ, float *maxZ, int n, cudaStream_t st);
int direct_fp64(Ctx *ctx, const float *x, const float *y, const float *z, const float *m, int n,
                const int *targets, int nt, double eps2, double *acc, cudaStream_t st);
int diagnostics_fp64(Ctx *ctx, const nbx_state *s, int n, double *out, cudaStream_t st);
struct Adj;
int adjoint_create(Ctx *ctx, int T, int C, int lcap, int tape_steps, Adj **out);
void adjoint_destroy(Adj *a);
size_t adjoint_bytes(const Adj *a);
int adjoint_forward(Ctx *ctx, Adj *a, const nbx_state *s, const float *tx, const float *ty, const float *tz,
                    double *loss_host, cudaStream_t st);
int adjoint_backward(Ctx *ctx, Adj *a, const nbx_state *s, float *gx, float *gy, float *gz, float *gvx, float *gvy,
                     float *gvz, float *gm, cudaStream_t st);
int adjoint_record_all(Ctx *ctx, Adj *a, const nbx_state *s, cudaStream_t st);
int adjoint_replay_fp64(Ctx *ctx, Adj *a, const double *state0, double *loss_host, cudaStream_t st);
void adjoint_times(const Adj *a, float *fwd_ms, float *bwd_ms);

namespace {

__global__ void k_body_sys(const int *sys_off, int nsys, int n, int *body_sys) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = nsys - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (sys_off[mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        body_sys[i] = lo;
    }
}

// The walk records one (list length, opened cells) pair per walk group (the
// values are the same for the group's bodies); the export writes them per body
// in original index order.
__global__ void k_expand_gstat(const int2 *gstat, const int *groups, int ngroups, const int *body_sys,
                               const int *sys_off, const int *val, int *nlist, int *nopen) {
    const int g = blockIdx.x;
    if (g >= ngroups) return;
    const int p0 = groups[g];
    const int p = p0 + (int)threadIdx.x;
    if (p >= min(sys_off[body_sys[p0] + 1], p0 + 32)) return;
    const int2 v = gstat[g];
    const int ob = val[p];
    if (nlist) nlist[ob] = v.x;
    if (nopen) nopen[ob] = v.y;
}

__global__ void k_split_gstat(const int2 *gstat, int ngroups, int *list_len, int *opened) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    const int2 v = gstat[g];
    if (list_len) list_len[g] = v.x;
    if (opened) opened[g] = v.y;
}

__global__ void k_depth0_from_ptrs(const float *minX, const float *maxX, float theta_ref, float *depth0) {
    if (threadIdx.x == 0) {
        float r = __fmul_rn(__fsub_rn(*maxX, *minX), 0.5f);
        depth0[0] = __fdiv_rn(__fmul_rn(r, r), theta_ref);
    }
}

template <typename T>
int dmalloc(Ctx *ctx, T **p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        ctx->last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        *p = nullptr;
        return NBX_ERR_NOMEM;
    }
    return NBX_OK;
}

void free_all(Ctx *ctx) {
    void *ptrs[] = {ctx->d_sys_off, ctx->d_body_sys, ctx->d_tiles, ctx->d_sys_tiles, ctx->d_groups,
                    ctx->d_bbox_u, ctx->d_bbox, ctx->d_bbox64, ctx->d_depth0, ctx->d_root_first, ctx->d_sys_lvl,
                    ctx->d_root_nch, ctx->d_key, ctx->d_key_alt, ctx->d_key_lo, ctx->d_val, ctx->d_val_alt,
                    ctx->d_body4, ctx->d_delta, ctx->d_bucket, ctx->d_ecount, ctx->d_body_node, ctx->d_gstat,
                    ctx->d_ent, ctx->d_ent_alt, ctx->d_flags, ctx->d_node4, ctx->d_meta, ctx->d_parent,
                    ctx->d_sums, ctx->d_count, ctx->d_arrive, ctx->d_lvl8, ctx->d_fcl, ctx->d_cl, ctx->d_hist,
                    ctx->d_scan_blk, ctx->d_totals, ctx->d_totals64, ctx->d_status, ctx->d_m2, ctx->d_quad4,
                    ctx->d_quad2, ctx->d_seg_slot, ctx->d_lb_counts, ctx->d_lb_status, ctx->d_lb, ctx->d_tiles_sw,
                    ctx->d_sys_tiles_sw};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph_stream) cudaStreamDestroy(ctx->graph_stream);
    if (ctx->graph_ev_in) cudaEventDestroy(ctx->graph_ev_in);
    if (ctx->graph_ev_out) cudaEventDestroy(ctx->graph_ev_out);
}

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    float *ms;
    cudaStream_t st;
    bool ok = false;  // events created and the start recorded
    Timer(float *ms_, cudaStream_t st_) : ms(ms_), st(st_) {
        if (ms) {
            ok = cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess &&
                 cudaEventRecord(a, st) == cudaSuccess;
        }
    }
    int finish(int rc) {
        if (ms) {
            float t = 0.f;
            if (ok && cudaEventRecord(b, st) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess)
                cudaEventElapsedTime(&t, a, b);
            else if (rc == NBX_OK)
                rc = NBX_ERR_CUDA;
            *ms = t;
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
        return rc;
    }
};

// The quadrupole arrays (second moments and FP32 terms), allocated when the
// multipole mode is first used.
int alloc_quadrupoles(Ctx *ctx) {
    if (ctx->d_m2) return NBX_OK;
    const size_t nc = (size_t)ctx->cap_nodes;
    int rc = dmalloc(ctx, &ctx->d_m2, 3 * nc);
    if (rc == 0) rc = dmalloc(ctx, &ctx->d_quad4, nc);
    if (rc == 0) rc = dmalloc(ctx, &ctx->d_quad2, nc);
    if (rc) {
        cudaFree(ctx->d_m2);
        cudaFree(ctx->d_quad4);
        cudaFree(ctx->d_quad2);
        ctx->d_m2 = nullptr;
        ctx->d_quad4 = nullptr;
        ctx->d_quad2 = nullptr;
    }
    return rc;
}

int ensure_single_system(Ctx *ctx, int n) {
    if (ctx->nsys == 1 && ctx->nbodies == n) return NBX_OK;
    int64_t off[2] = {0, n};
    return nbx_set_systems(reinterpret_cast<nbx_ctx *>(ctx), 1, off);
}

}  // namespace
}  // namespace nbx

using nbx::Ctx;

static Ctx *C(nbx_ctx *c) { return reinterpret_cast<Ctx *>(c); }
static cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" {

void nbx_params_default(nbx_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->max_bodies = 1 << 20;
    p->max_systems = 1;
    p->theta = 0.5f;
    p->theta_ref = 0.f;
    p->eps = 0.05f;
    p->eps2 = 0.f;
    p->dt = 0.001f;
    p->dampening = 1.f;
    p->gravity = 1.f;
    p->group = 32;
    p->stack_depth = 512;
    p->compensated = 0;
    p->leaf_size = 1;
    p->radix_bits = 8;
    p->walk_warps = 0;
    p->walk_variant = 3;  // 96-slot buffers: the fastest at 2^20 and 2^24 bodies
    p->device = 0;
    p->block_size = 256;
    p->grid_size = 1024;
    p->multipole = 0;
}

const char *nbx_status_string(int s) {
    switch (s) {
        case NBX_OK: return "ok";
        case NBX_ERR_ARG: return "invalid argument";
        case NBX_ERR_CUDA: return "CUDA runtime error";
        case NBX_ERR_DEPTH: return "two bodies share a region 42 levels deep (duplicate positions)";
        case NBX_ERR_CAPACITY: return "node pool capacity exceeded";
        case NBX_ERR_STACK: return "walk stack overflow";
        case NBX_ERR_NONFINITE: return "non-finite position";
        case NBX_ERR_CLUSTER: return "more than 4096 bodies share one 21-level key";
        case NBX_ERR_TIMEOUT: return "bounded device wait expired";
        case NBX_ERR_STATE: return "call out of order or inconsistent tree";
        case NBX_ERR_NOMEM: return "device allocation failed";
        case NBX_ERR_SCRATCH: return "request exceeds the static scratch of a no-allocation entry point";
        case NBX_ERR_FORMAT: return "checkpoint header, size or checksum mismatch";
        default: return "unknown status";
    }
}

const char *nbx_last_error(nbx_ctx *c) { return c ? C(c)->last_error.c_str() : "null context"; }

int nbx_create(const nbx_params *p, nbx_ctx **out) {
    if (!p || !out) return NBX_ERR_ARG;
    *out = nullptr;
    if (p->max_bodies < 1 || p->max_bodies > (1 << 26) || p->max_systems < 1 ||
        p->max_systems > p->max_bodies || p->group != 32 || p->leaf_size < 1 || p->leaf_size > 8 || (p->radix_bits != 8 && p->radix_bits != 9) ||
        p->stack_depth < 360 || p->stack_depth > 4096 || p->walk_variant < 0 || p->walk_variant > 3 ||
        p->moments_mode < 0 || p->moments_mode > 2 || p->multipole < 0 || p->multipole > 1 ||
        (p->multipole == 1 && p->walk_variant == 2) ||
        (p->node_capacity != 0 && (p->node_capacity < p->max_bodies + 1 || p->node_capacity > nbx::kMaxNodes)))
        return NBX_ERR_ARG;
    Ctx *ctx = new (std::nothrow) Ctx();
    if (!ctx) return NBX_ERR_NOMEM;
    ctx->p = *p;
    ctx->theta_ref = p->theta_ref > 0.f ? p->theta_ref : p->theta * p->theta;
    ctx->eps2 = p->eps2 > 0.f ? p->eps2 : p->eps * p->eps;
    // a body's own term (d = 0) is 0 * inf without softening; a normal eps2 keeps
    // every softened r^2 >= eps2 out of the subnormal range
    if (!(ctx->theta_ref > 0.f) || !(ctx->eps2 >= FLT_MIN) || !std::isfinite(ctx->theta_ref) || !std::isfinite(ctx->eps2)) {
        delete ctx;
        return NBX_ERR_ARG;
    }
    ctx->compensated = p->compensated;
    ctx->walk_variant = p->walk_variant;
    ctx->key_order = p->key_order;
    ctx->radix_bits = p->radix_bits;
    ctx->multipole = p->multipole;
    ctx->leaf_size = p->leaf_size;
    if (p->key_order < 0 || p->key_order > 1) {
        delete ctx;
        return NBX_ERR_ARG;
    }
    if (p->walk_warps == 4 || p->walk_warps == 8 || p->walk_warps == 16) ctx->walk_warps = p->walk_warps;
    if (!(ctx->theta_ref > 0.f) || p->compensated < 0 || p->compensated > 2) {
        delete ctx;
        return NBX_ERR_ARG;
    }
    if (cudaSetDevice(p->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
        delete ctx;
        return NBX_ERR_CUDA;
    }
    const int B = p->max_bodies, Ss = p->max_systems;
    ctx->cap_bodies = B;
    ctx->cap_sys = Ss;
    const int64_t nc = p->node_capacity ? (int64_t)p->node_capacity : 2ll * B + 65536;
    ctx->cap_nodes = (int)(nc < nbx::kMaxNodes ? nc : nbx::kMaxNodes);
    // a tile below kTile is only chosen while there are fewer than 2 * want tiles
    const int want_tiles = 2 * ctx->nsm * nbx::kScatterWarps;
    ctx->cap_tiles_body = (B / nbx::kTile > 2 * want_tiles ? B / nbx::kTile : 2 * want_tiles) + Ss + 1;
    // no tile is smaller than kTileMin: a small context never needs more tiles than this
    const int64_t most_tiles = (int64_t)B / nbx::kTileMin + Ss + 1;
    if (most_tiles < ctx->cap_tiles_body) ctx->cap_tiles_body = (int)most_tiles;
    ctx->tile_node = nbx::tile_for(ctx->cap_nodes, ctx->nsm);
    ctx->cap_tiles_node = nbx::ceil_div(ctx->cap_nodes, ctx->tile_node);
    const int64_t hist = (1ll << nbx::kMaxRadixBits) * (ctx->cap_tiles_body > ctx->cap_tiles_node ? ctx->cap_tiles_body : ctx->cap_tiles_node);
    int64_t scan_max = hist;
    if (ctx->cap_nodes > scan_max) scan_max = ctx->cap_nodes;
    if (B > scan_max) scan_max = B;
    ctx->cap_scan_blk = nbx::ceil_div(scan_max, nbx::kScanItems) + 1;
    const int NC = ctx->cap_nodes;
    const int G = B / 32 + Ss + 1;
    int rc = 0;
    rc |= nbx::dmalloc(ctx, &ctx->d_sys_off, Ss + 1);
    rc |= nbx::dmalloc(ctx, &ctx->d_body_sys, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_tiles, ctx->cap_tiles_body);
    rc |= nbx::dmalloc(ctx, &ctx->d_sys_tiles, Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_seg_slot, Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_tiles_sw, ctx->cap_tiles_body);
    rc |= nbx::dmalloc(ctx, &ctx->d_sys_tiles_sw, Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_groups, G);
    rc |= nbx::dmalloc(ctx, &ctx->d_bbox_u, 6 * Ss + 6);
    rc |= nbx::dmalloc(ctx, &ctx->d_bbox, 6 * Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_bbox64, 6 * Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_depth0, Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_root_first, Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_root_nch, Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_sys_lvl, Ss);
    rc |= nbx::dmalloc(ctx, &ctx->d_key, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_key_alt, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_key_lo, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_val, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_val_alt, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_body4, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_delta, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_bucket, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_ecount, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_body_node, B);
    rc |= nbx::dmalloc(ctx, &ctx->d_gstat, G);
    rc |= nbx::dmalloc(ctx, &ctx->d_ent, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_ent_alt, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_flags, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_node4, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_meta, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_parent, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_sums, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_count, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_arrive, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_lvl8, NC);
    rc |= nbx::dmalloc(ctx, &ctx->d_fcl, (size_t)NC + Ss + 2);
    rc |= nbx::dmalloc(ctx, &ctx->d_cl, (size_t)NC + Ss + 2);
    rc |= nbx::dmalloc(ctx, &ctx->d_hist, hist + 1);  // + the scanned total
    // one-sweep body sort: a system of several tiles takes at least two, so at most
    // half the tiles (plus one) hold count slots; status words per tile and digit
    rc |= nbx::dmalloc(ctx, &ctx->d_lb_counts, (size_t)(ctx->cap_tiles_body / 2 + 1) * nbx::kLbMaxCounts);
    rc |= nbx::dmalloc(ctx, &ctx->d_lb_status, (size_t)ctx->cap_tiles_body << nbx::kMaxRadixBits);
    rc |= nbx::dmalloc(ctx, &ctx->d_lb, 16);
    rc |= nbx::dmalloc(ctx, &ctx->d_scan_blk, ctx->cap_scan_blk);
    rc |= nbx::dmalloc(ctx, &ctx->d_totals, 8);
    rc |= nbx::dmalloc(ctx, &ctx->d_totals64, 4);
    rc |= nbx::dmalloc(ctx, &ctx->d_status, 1);
    if (rc == 0 && cudaMallocHost((void **)&ctx->h_status, sizeof(nbx::DevStatus)) != cudaSuccess) rc = NBX_ERR_NOMEM;
    if (rc == 0 && cudaMemset(ctx->d_status, 0, sizeof(nbx::DevStatus)) != cudaSuccess) rc = NBX_ERR_CUDA;
    if (rc == 0 && cudaMemset(ctx->d_totals, 0, 8 * sizeof(unsigned)) != cudaSuccess) rc = NBX_ERR_CUDA;
    // status words start at build 0, which no pass ever uses (its tags are >= 1)
    if (rc == 0 && cudaMemset(ctx->d_lb_status, 0, sizeof(unsigned long long) * ((size_t)ctx->cap_tiles_body << nbx::kMaxRadixBits)) != cudaSuccess)
        rc = NBX_ERR_CUDA;
    if (rc == 0 && cudaMemset(ctx->d_lb, 0, 16 * sizeof(unsigned)) != cudaSuccess) rc = NBX_ERR_CUDA;
    if (rc == 0 && ctx->multipole) rc = nbx::alloc_quadrupoles(ctx);
    if (rc == 0) rc = nbx::walk_init(ctx);
    if (rc == 0) rc = nbx::radix_init(ctx);
    if (rc != 0) {
        nbx::free_all(ctx);
        delete ctx;
        return rc == NBX_ERR_NOMEM ? NBX_ERR_NOMEM : (rc ? rc : NBX_ERR_CUDA);
    }
    *out = reinterpret_cast<nbx_ctx *>(ctx);
    return NBX_OK;
}

int nbx_destroy(nbx_ctx *c) {
    if (!c) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    cudaDeviceSynchronize();
    nbx::free_all(ctx);
    delete ctx;
    return NBX_OK;
}

int nbx_get_constants(nbx_ctx *c, float *theta_ref, float *eps2) {
    if (!c) return NBX_ERR_ARG;
    if (theta_ref) *theta_ref = C(c)->theta_ref;
    if (eps2) *eps2 = C(c)->eps2;
    return NBX_OK;
}

int nbx_set_constants(nbx_ctx *c, float theta_ref, float eps2, int compensated) {
    if (!c || !(theta_ref > 0.f) || !(eps2 >= FLT_MIN) || !std::isfinite(theta_ref) || !std::isfinite(eps2))
        return NBX_ERR_ARG;
    if (compensated < 0 || compensated > 2) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    ctx->theta_ref = theta_ref;
    ctx->eps2 = eps2;
    ctx->compensated = compensated;
    ++ctx->graph_gen;
    if (ctx->graph_exec) {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
    }
    return NBX_OK;
}

int nbx_set_multipole(nbx_ctx *c, int multipole) {
    if (!c || multipole < 0 || multipole > 1) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (multipole == 1 && ctx->walk_variant == 2) return NBX_ERR_ARG;
    if (multipole == 1) {
        const int rc = nbx::alloc_quadrupoles(ctx);
        if (rc) return rc;
    }
    if (multipole != ctx->multipole) {
        ctx->multipole = multipole;
        ctx->p.multipole = multipole;
        ctx->built = false;  // the next walk needs moments of this order
        ctx->ref_m = 0;
        ++ctx->graph_gen;
        if (ctx->graph_exec) {
            cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
        }
    }
    return NBX_OK;
}

int nbx_set_leaf_size(nbx_ctx *c, int leaf_size) {
    if (!c || leaf_size < 1 || leaf_size > 8) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (leaf_size != ctx->leaf_size) {
        ctx->leaf_size = leaf_size;
        ctx->p.leaf_size = leaf_size;
        ctx->built = false;  // the next walk needs a tree with these leaves
        ctx->ref_m = 0;
        ++ctx->graph_gen;
        if (ctx->graph_exec) {
            cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
        }
    }
    return NBX_OK;
}

int nbx_set_walk_config(nbx_ctx *c, int warps_per_block, int variant) {
    if (!c || !(warps_per_block == 4 || warps_per_block == 8 || warps_per_block == 16) ||
        !(variant >= 0 && variant <= 3))
        return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (variant == 2 && ctx->multipole) return NBX_ERR_ARG;
    ctx->walk_warps = warps_per_block;
    ctx->walk_variant = variant;
    ++ctx->graph_gen;
    if (ctx->graph_exec) {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
    }
    return NBX_OK;
}

int nbx_set_tuning(nbx_ctx *c, int radix_bits, int stack_depth) {
    if (!c || (radix_bits != 8 && radix_bits != 9) || stack_depth < 360 || stack_depth > 4096) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    ctx->radix_bits = radix_bits;
    ctx->p.radix_bits = radix_bits;
    ctx->p.stack_depth = stack_depth;  // the built tree stays valid: neither changes it
    ++ctx->graph_gen;
    if (ctx->graph_exec) {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
    }
    return NBX_OK;
}

int nbx_set_systems(nbx_ctx *c, int nsys, const int64_t *offsets) {
    if (!c || !offsets || nsys < 1) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (nsys > ctx->cap_sys) return NBX_ERR_ARG;
    if (offsets[0] != 0) return NBX_ERR_ARG;
    for (int s = 0; s < nsys; s++)
        if (offsets[s + 1] <= offsets[s]) return NBX_ERR_ARG;
    if (offsets[nsys] > ctx->cap_bodies) return NBX_ERR_ARG;
    const int n = (int)offsets[nsys];
    const int tile = nbx::tile_for(n, ctx->nsm);
    // the one-sweep sort's tiling: its passes are bound by the look-back chains
    // between a system's tiles, so its tiles are at least kTileSweep keys
    const int tile_sw = tile > nbx::kTileSweep ? tile : (nbx::kTileSweep < nbx::kTile ? nbx::kTileSweep : nbx::kTile);
    std::vector<int> off(nsys + 1);
    std::vector<int4> tiles, tiles_sw;
    std::vector<int2> st(nsys), st_sw(nsys);
    std::vector<int> slot(nsys);
    std::vector<int> groups;
    int nslots = 0;
    for (int s = 0; s <= nsys; s++) off[s] = (int)offsets[s];
    for (int s = 0; s < nsys; s++) {
        const int beg = off[s], end = off[s + 1];
        const int nt = nbx::ceil_div(end - beg, tile);
        st[s] = make_int2((int)tiles.size(), nt);
        for (int t = 0; t < nt; t++) {
            const int a = beg + t * tile;
            const int len = (end - a) < tile ? (end - a) : tile;
            tiles.push_back(make_int4(a, len, s, t));
        }
        const int nts = nbx::ceil_div(end - beg, tile_sw);
        st_sw[s] = make_int2((int)tiles_sw.size(), nts);
        slot[s] = nts > 1 ? nslots++ : -1;
        for (int t = 0; t < nts; t++) {
            const int a = beg + t * tile_sw;
            const int len = (end - a) < tile_sw ? (end - a) : tile_sw;
            tiles_sw.push_back(make_int4(a, len, s, t));
        }
        for (int g = beg; g < end; g += 32) groups.push_back(g);
    }
    if ((int)tiles.size() > ctx->cap_tiles_body || (int)tiles_sw.size() > ctx->cap_tiles_body) return NBX_ERR_ARG;
    NBX_CUDA(cudaMemcpy(ctx->d_sys_off, off.data(), sizeof(int) * (nsys + 1), cudaMemcpyHostToDevice));
    NBX_CUDA(cudaMemcpy(ctx->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice));
    NBX_CUDA(cudaMemcpy(ctx->d_sys_tiles, st.data(), sizeof(int2) * nsys, cudaMemcpyHostToDevice));
    NBX_CUDA(cudaMemcpy(ctx->d_seg_slot, slot.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice));
    NBX_CUDA(cudaMemcpy(ctx->d_tiles_sw, tiles_sw.data(), sizeof(int4) * tiles_sw.size(), cudaMemcpyHostToDevice));
    NBX_CUDA(cudaMemcpy(ctx->d_sys_tiles_sw, st_sw.data(), sizeof(int2) * nsys, cudaMemcpyHostToDevice));
    NBX_CUDA(cudaMemcpy(ctx->d_groups, groups.data(), sizeof(int) * groups.size(), cudaMemcpyHostToDevice));
    nbx::k_body_sys<<<nbx::ceil_div(n, 256) < 4096 ? nbx::ceil_div(n, 256) : 4096, 256>>>(ctx->d_sys_off, nsys, n,
                                                                                          ctx->d_body_sys);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    NBX_CUDA(cudaDeviceSynchronize());
    ctx->nsys = nsys;
    ctx->nbodies = n;
    ctx->ntiles_body = (int)tiles.size();
    ctx->nslots = nslots;
    ctx->ntiles_sw = (int)tiles_sw.size();
    ctx->tile_sw = tile_sw;
    ctx->tile_body = tile;
    ctx->ngroups = (int)groups.size();
    ctx->built = false;
    ctx->ref_m = 0;
    ++ctx->graph_gen;
    if (ctx->graph_exec) {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
    }
    return NBX_OK;
}

/* ---------------- reference-compatible phase entry points ---------------- */

int nbx_reset_arrays(nbx_ctx *c, int *mutex, float *x, float *y, float *z, float *mass, int *count, int *start,
                     int *sorted, int *child, int *index, float *minX, float *maxX, float *minY, float *maxY,
                     float *minZ, float *maxZ, int n, int m, void *stream, float *ms) {
    if (!c || n < 1 || m < n || !mutex || !x || !child || !index) return NBX_ERR_ARG;
    nbx::Timer t(ms, S(stream));
    return t.finish(nbx::reset_ref_arrays(C(c), mutex, x, y, z, mass, count, start, sorted, child, index, minX,
                                          maxX, minY, maxY, minZ, maxZ, n, m, S(stream)));
}

int nbx_compute_bounding_box(nbx_ctx *c, int *mutex, float *x, float *y, float *z, float *minX, float *maxX,
                             float *minY, float *maxY, float *minZ, float *maxZ, int n, void *stream, float *ms) {
    (void)mutex;
    if (!c || n < 1 || !x || !y || !z || !minX) return NBX_ERR_ARG;
    nbx::Timer t(ms, S(stream));
    return t.finish(nbx::bbox_ref(C(c), x, y, z, minX, maxX, minY, maxY, minZ, maxZ, n, S(stream)));
}

int nbx_build_tree(nbx_ctx *c, float *x, float *y, float *z, float *mass, int *count, int *start, int *child,
                   int *index, float *minX, float *maxX, float *minY, float *maxY, float *minZ, float *maxZ, int n,
                   int m, void *stream, float *ms) {
    (void)start;
    if (!c || n < 1 || m < n || !x || !child || !index || !count || !mass) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (n > ctx->cap_bodies) return NBX_ERR_ARG;
    nbx::Timer t(ms, S(stream));
    ctx->ref_m = 0;
    int rc = nbx::ensure_single_system(ctx, n);
    if (rc) return t.finish(rc);
    nbx_state s{};
    s.x = x; s.y = y; s.z = z; s.m = mass;
    const float *bp[6] = {minX, maxX, minY, maxY, minZ, maxZ};
    rc = nbx::build_tree(ctx, &s, S(stream), true, bp);
    if (rc) return t.finish(rc);
    rc = nbx_sync_status(c, stream);
    if (rc) return t.finish(rc);
    int64_t nc = 0;
    rc = nbx::export_tree_impl(ctx, 0, nullptr, child, child + 8ll * n, nullptr, count + n, nullptr, x + n, y + n,
                               z + n, mass + n, m - n, &nc, S(stream), 1);
    if (rc) return t.finish(rc);
    const int idx = n + (int)nc;
    NBX_CUDA(cudaMemcpyAsync(index, &idx, sizeof(int), cudaMemcpyHostToDevice, S(stream)));
    NBX_CUDA(cudaStreamSynchronize(S(stream)));
    ctx->ref_m = m;
    return t.finish(NBX_OK);
}

int nbx_centre_of_mass(nbx_ctx *c, float *x, float *y, float *z, float *mass, int *index, int n, void *stream,
                       float *ms) {
    (void)index;
    if (!c || !x || !mass) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (!ctx->built || ctx->nbodies != n || ctx->ref_m <= n) return NBX_ERR_STATE;
    nbx::Timer t(ms, S(stream));
    int64_t nc = 0;
    int rc = nbx::export_tree_impl(ctx, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, x + n, y + n,
                                   z + n, mass + n, ctx->ref_m - n, &nc, S(stream), 0);
    return t.finish(rc);
}

int nbx_sort(nbx_ctx *c, int *count, int *start, int *sorted, int *child, int *index, int n, void *stream,
             float *ms) {
    (void)count; (void)child; (void)index;
    if (!c || !start || !sorted) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (!ctx->built || ctx->nbodies != n || ctx->ref_m <= n) return NBX_ERR_STATE;
    nbx::Timer t(ms, S(stream));
    int64_t nc = 0;
    int rc = nbx::export_tree_impl(ctx, 0, sorted, nullptr, nullptr, start + n, nullptr, nullptr, nullptr, nullptr,
                                   nullptr, nullptr, ctx->ref_m - n, &nc, S(stream), 0);
    return t.finish(rc);
}

int nbx_compute_forces(nbx_ctx *c, float *x, float *y, float *z, float *vx, float *vy, float *vz, float *ax,
                       float *ay, float *az, float *mass, int *sorted, int *child, float *minX, float *maxX, int n,
                       float g, void *stream, float *ms) {
    (void)x; (void)y; (void)z; (void)vx; (void)vy; (void)vz; (void)mass; (void)sorted; (void)child; (void)g;
    if (!c || !ax || !ay || !az || !minX || !maxX) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (!ctx->built || ctx->nbodies != n) return NBX_ERR_STATE;
    nbx::Timer t(ms, S(stream));
    nbx::k_depth0_from_ptrs<<<1, 32, 0, S(stream)>>>(minX, maxX, ctx->theta_ref, ctx->d_depth0);
    ++ctx->launches;
    nbx_state s{};
    s.ax = ax; s.ay = ay; s.az = az;
    return t.finish(nbx::walk_forces(ctx, &s, S(stream)));
}

int nbx_update(nbx_ctx *c, float *x, float *y, float *z, float *vx, float *vy, float *vz, float *ax, float *ay,
               float *az, int n, float dt, float d, void *stream, float *ms) {
    if (!c || !x || !vx || !ax || n < 0) return NBX_ERR_ARG;
    nbx::Timer t(ms, S(stream));
    nbx_state s{x, y, z, vx, vy, vz, ax, ay, az, nullptr};
    return t.finish(nbx::integrate(C(c), &s, dt, d, n, S(stream)));
}

/* ---------------- native pipeline ---------------- */

static int check_state(Ctx *ctx, const nbx_state *s) {
    if (!s || !s->x || !s->y || !s->z || !s->m) return NBX_ERR_ARG;
    if (ctx->nsys < 1) return NBX_ERR_STATE;
    return NBX_OK;
}

int nbx_build(nbx_ctx *c, const nbx_state *s, void *stream) {
    if (!c) return NBX_ERR_ARG;
    Range r("nbx_build");
    int rc = check_state(C(c), s);
    if (rc) return rc;
    return nbx::build_tree(C(c), s, S(stream), false, nullptr);
}

int nbx_forces(nbx_ctx *c, const nbx_state *s, void *stream) {
    if (!c || !s || !s->ax || !s->ay || !s->az) return NBX_ERR_ARG;
    Range r("nbx_forces");
    return nbx::walk_forces(C(c), s, S(stream));
}

int nbx_group_count(nbx_ctx *c, int *ngroups) {
    if (!c || !ngroups) return NBX_ERR_ARG;
    *ngroups = C(c)->ngroups;
    return NBX_OK;
}

int nbx_forces_groups(nbx_ctx *c, const nbx_state *s, int first_group, int ngroups, void *stream) {
    if (!c || !s || !s->ax || !s->ay || !s->az) return NBX_ERR_ARG;
    Range r("nbx_forces_groups");
    return nbx::walk_forces_groups(C(c), s, first_group, ngroups, S(stream));
}

int nbx_export_group_stats(nbx_ctx *c, int *list_len, int *opened, void *stream) {
    if (!c) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (!ctx->built) return NBX_ERR_STATE;
    if ((list_len || opened) && ctx->ngroups > 0) {
        nbx::k_split_gstat<<<nbx::ceil_div(ctx->ngroups, 256), 256, 0, S(stream)>>>(ctx->d_gstat, ctx->ngroups, list_len,
                                                                                  opened);
        ++ctx->launches;
        NBX_CUDA(cudaGetLastError());
    }
    NBX_CUDA(cudaStreamSynchronize(S(stream)));
    return NBX_OK;
}

int nbx_integrate(nbx_ctx *c, const nbx_state *s, void *stream) {
    if (!c || !s || !s->vx || !s->ax) return NBX_ERR_ARG;
    Range r("nbx_integrate");
    Ctx *ctx = C(c);
    return nbx::integrate(ctx, s, ctx->p.dt, ctx->p.dampening, (int)ctx->nbodies, S(stream));
}

static int one_step(Ctx *ctx, const nbx_state *s, cudaStream_t st) {
    Range r("nbx_step");
    int rc = nbx::build_tree(ctx, s, st, false, nullptr);
    if (rc) return rc;
    rc = nbx::walk_forces(ctx, s, st);
    if (rc) return rc;
    return nbx::integrate(ctx, s, ctx->p.dt, ctx->p.dampening, (int)ctx->nbodies, st);
}

namespace {

// One step captured as a CUDA graph (captured again when the state arrays or
// the systems change; the setters of constants, walk and systems drop it) and
// replayed nsteps times on the context's own stream, ordered after and before
// the caller's stream by events, so the call stays asynchronous.
int replay_steps(Ctx *ctx, const nbx_state *s, int nsteps, cudaStream_t user) {
    if (!ctx->graph_stream) NBX_CUDA(cudaStreamCreateWithFlags(&ctx->graph_stream, cudaStreamNonBlocking));
    if (!ctx->graph_ev_in) NBX_CUDA(cudaEventCreateWithFlags(&ctx->graph_ev_in, cudaEventDisableTiming));
    if (!ctx->graph_ev_out) NBX_CUDA(cudaEventCreateWithFlags(&ctx->graph_ev_out, cudaEventDisableTiming));
    const cudaStream_t st = ctx->graph_stream;
    if (ctx->graph_exec && (std::memcmp(&ctx->graph_state, s, sizeof(nbx_state)) != 0 || ctx->graph_nsys != ctx->nsys)) {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
    }
    NBX_CUDA(cudaEventRecord(ctx->graph_ev_in, user));
    NBX_CUDA(cudaStreamWaitEvent(st, ctx->graph_ev_in, 0));
    if (!ctx->graph_exec) {
        cudaGraph_t g = nullptr;
        NBX_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = one_step(ctx, s, st);
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) {
            ctx->last_error = std::string("graph capture: ") + cudaGetErrorString(e);
            return NBX_ERR_CUDA;
        }
        e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            ctx->graph_exec = nullptr;
            ctx->last_error = std::string("graph instantiate: ") + cudaGetErrorString(e);
            return NBX_ERR_CUDA;
        }
        ctx->graph_state = *s;
        ctx->graph_nsys = ctx->nsys;
    }
    for (int k = 0; k < nsteps; k++) NBX_CUDA(cudaGraphLaunch(ctx->graph_exec, st));
    NBX_CUDA(cudaEventRecord(ctx->graph_ev_out, st));
    NBX_CUDA(cudaStreamWaitEvent(user, ctx->graph_ev_out, 0));
    return NBX_OK;
}

bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

}  // namespace

// Several steps replay one captured step; a single step (or a call made while
// the caller's stream is being captured) launches its kernels directly.
int nbx_step(nbx_ctx *c, const nbx_state *s, int nsteps, void *stream) {
    if (!c || nsteps < 0) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    int rc = check_state(ctx, s);
    if (rc) return rc;
    if (!s->vx || !s->ax) return NBX_ERR_ARG;
    if (nsteps >= 2 && !capturing(S(stream))) return replay_steps(ctx, s, nsteps, S(stream));
    for (int k = 0; k < nsteps; k++) {
        rc = one_step(ctx, s, S(stream));
        if (rc) return rc;
    }
    return NBX_OK;
}

int nbx_graph_step(nbx_ctx *c, const nbx_state *s, int nsteps, void *stream) {
    if (!c || nsteps < 0) return NBX_ERR_ARG;
    Range r("nbx_graph_step");
    Ctx *ctx = C(c);
    int rc = check_state(ctx, s);
    if (rc) return rc;
    if (!s->vx || !s->ax) return NBX_ERR_ARG;
    if (capturing(S(stream))) return NBX_ERR_ARG;  // a captured step cannot be nested in a capture
    return replay_steps(ctx, s, nsteps, S(stream));
}

int nbx_selftest_sort_wait(nbx_ctx *c, void *stream) {
    if (!c) return NBX_ERR_ARG;
    cudaStream_t st = S(stream);
    if (capturing(st)) return NBX_ERR_ARG;
    return nbx::radix_selftest_wait(C(c), st);
}

int nbx_sync_status(nbx_ctx *c, void *stream) {
    if (!c) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    NBX_CUDA(cudaStreamSynchronize(S(stream)));
    NBX_CUDA(cudaMemcpy(ctx->h_status, ctx->d_status, sizeof(nbx::DevStatus), cudaMemcpyDeviceToHost));
    const int code = ctx->h_status->code;
    if (code) {
        char buf[160];
        std::snprintf(buf, sizeof(buf), "device status %d (%s), detail %d", code, nbx_status_string(code),
                      ctx->h_status->detail);
        ctx->last_error = buf;
        int zero[2] = {0, 0};
        NBX_CUDA(cudaMemcpy(ctx->d_status, zero, sizeof(zero), cudaMemcpyHostToDevice));
        // the tree of a step that reported an error may be inconsistent: it is
        // never walked again, the next walk needs a new build
        ctx->built = false;
        ctx->ref_m = 0;
    }
    return code;
}

int nbx_get_tree_info(nbx_ctx *c, void *stream, nbx_tree_info *out) {
    if (!c || !out) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    NBX_CUDA(cudaStreamSynchronize(S(stream)));
    unsigned tot[2];
    unsigned long long t64 = 0;
    NBX_CUDA(cudaMemcpy(tot, ctx->d_totals, sizeof(tot), cudaMemcpyDeviceToHost));
    NBX_CUDA(cudaMemcpy(&t64, ctx->d_totals64, sizeof(t64), cudaMemcpyDeviceToHost));
    NBX_CUDA(cudaMemcpy(ctx->h_status, ctx->d_status, sizeof(nbx::DevStatus), cudaMemcpyDeviceToHost));
    out->nbodies = ctx->nbodies;
    out->ncells = (int64_t)(t64 >> 32);
    out->nnodes = tot[1];
    out->max_level = ctx->h_status->max_level;
    out->nsystems = ctx->nsys;
    out->interactions = (int64_t)ctx->h_status->interactions;
    out->opened = (int64_t)ctx->h_status->opened;
    out->refined_runs = ctx->h_status->refined_runs;
    out->status = ctx->h_status->code;
    out->launches = ctx->launches;
    out->rounds = (int64_t)ctx->h_status->rounds;
    out->candidates = (int64_t)ctx->h_status->candidates;
    return NBX_OK;
}

int nbx_export_tree(nbx_ctx *c, int sys, int *perm, int *root_child, int *cell_child, int *cell_start,
                    int *cell_count, int *cell_level, float *cell_x, float *cell_y, float *cell_z, float *cell_m,
                    int cap_cells, int64_t *ncells, void *stream) {
    if (!c) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    int rc = nbx_sync_status(c, stream);
    if (rc) return rc;
    rc = nbx::export_tree_impl(ctx, sys, perm, root_child, cell_child, cell_start, cell_count, cell_level, cell_x,
                               cell_y, cell_z, cell_m, cap_cells, ncells, S(stream), 0);
    if (rc) return rc;
    NBX_CUDA(cudaStreamSynchronize(S(stream)));
    return NBX_OK;
}

int nbx_export_keys(nbx_ctx *c, uint64_t *keys, int *perm, void *stream) {
    if (!c) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (!ctx->built) return NBX_ERR_STATE;
    if (keys)
        NBX_CUDA(cudaMemcpyAsync(keys, ctx->d_key, sizeof(uint64_t) * ctx->nbodies, cudaMemcpyDeviceToDevice, S(stream)));
    if (perm)
        NBX_CUDA(cudaMemcpyAsync(perm, ctx->d_val, sizeof(int) * ctx->nbodies, cudaMemcpyDeviceToDevice, S(stream)));
    NBX_CUDA(cudaStreamSynchronize(S(stream)));
    return NBX_OK;
}

int nbx_export_walk_stats(nbx_ctx *c, int *nlist, int *nopen, void *stream) {
    if (!c) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (!ctx->built) return NBX_ERR_STATE;
    if ((nlist || nopen) && ctx->ngroups > 0) {
        nbx::k_expand_gstat<<<ctx->ngroups, 32, 0, S(stream)>>>(ctx->d_gstat, ctx->d_groups, ctx->ngroups,
                                                                ctx->d_body_sys, ctx->d_sys_off, ctx->d_val, nlist,
                                                                nopen);
        ++ctx->launches;
        NBX_CUDA(cudaGetLastError());
    }
    NBX_CUDA(cudaStreamSynchronize(S(stream)));
    return NBX_OK;
}

int nbx_direct_fp64(nbx_ctx *c, const float *x, const float *y, const float *z, const float *m, int n,
                    const int *targets, int nt, double eps2, double *acc, void *stream) {
    if (!c || !x || !y || !z || !m || !targets || !acc || n < 0 || nt < 0) return NBX_ERR_ARG;
    return nbx::direct_fp64(C(c), x, y, z, m, n, targets, nt, eps2, acc, S(stream));
}

int nbx_forces_fp64_lists(nbx_ctx *c, const int *group_starts, int ngroups, double *acc, void *stream) {
    if (!c || (ngroups > 0 && (!group_starts || !acc)) || ngroups < 0) return NBX_ERR_ARG;
    return nbx::walk_fp64_lists(C(c), group_starts, ngroups, acc, S(stream));
}

int nbx_potential(nbx_ctx *c, const nbx_state *s, float *phi, void *stream) {
    if (!c || !s || !phi) return NBX_ERR_ARG;
    if (!(C(c)->eps2 > 0.f)) return NBX_ERR_ARG;
    return nbx::walk_potential(C(c), s, phi, S(stream));
}

int nbx_diagnostics_fp64(nbx_ctx *c, const nbx_state *s, int n, double *out, void *stream) {
    if (!c || !s || !out || n < 0) return NBX_ERR_ARG;
    return nbx::diagnostics_fp64(C(c), s, n, out, S(stream));
}

/* ---------------- differentiation ---------------- */

int nbx_adjoint_create(nbx_ctx *c, int nsteps, int checkpoint_every, int list_capacity, int tape_steps,
                       nbx_adjoint **out) {
    if (!c || !out) return NBX_ERR_ARG;
    Ctx *ctx = C(c);
    if (ctx->nsys < 1) return NBX_ERR_STATE;
    if (ctx->multipole || ctx->leaf_size != 1) {
        ctx->last_error = "adjoint: needs monopoles and one body per leaf (multipole 0, leaf_size 1)";
        return NBX_ERR_ARG;
    }
    nbx::Adj *a = nullptr;
    int rc = nbx::adjoint_create(ctx, nsteps, checkpoint_every, list_capacity, tape_steps, &a);
    if (rc) {
        nbx::adjoint_destroy(a);
        *out = nullptr;
        return rc;
    }
    *out = reinterpret_cast<nbx_adjoint *>(a);
    return NBX_OK;
}

int nbx_adjoint_destroy(nbx_adjoint *a) {
    if (!a) return NBX_ERR_ARG;
    cudaDeviceSynchronize();
    nbx::adjoint_destroy(reinterpret_cast<nbx::Adj *>(a));
    return NBX_OK;
}

int nbx_adjoint_forward(nbx_ctx *c, nbx_adjoint *a, const nbx_state *s, const float *tx, const float *ty,
                        const float *tz, double *loss, void *stream) {
    if (!c || !a || !s || !tx || !ty || !tz || !loss) return NBX_ERR_ARG;
    if (C(c)->multipole || C(c)->leaf_size != 1) return NBX_ERR_ARG;  // monopoles, one body per leaf
    int rc = nbx::adjoint_forward(C(c), reinterpret_cast<nbx::Adj *>(a), s, tx, ty, tz, loss, S(stream));
    if (rc) return rc;
    return nbx_sync_status(c, stream);
}

int nbx_adjoint_backward(nbx_ctx *c, nbx_adjoint *a, const nbx_state *s, float *gx, float *gy, float *gz,
                         float *gvx, float *gvy, float *gvz, float *gm, void *stream) {
    if (!c || !a || !s || !gx || !gy || !gz || !gvx || !gvy || !gvz || !gm) return NBX_ERR_ARG;
    int rc = nbx::adjoint_backward(C(c), reinterpret_cast<nbx::Adj *>(a), s, gx, gy, gz, gvx, gvy, gvz, gm,
                                   S(stream));
    if (rc) return rc;
    return nbx_sync_status(c, stream);
}

int nbx_adjoint_record(nbx_ctx *c, nbx_adjoint *a, const nbx_state *s, void *stream) {
    if (!c || !a || !s) return NBX_ERR_ARG;
    if (C(c)->multipole || C(c)->leaf_size != 1) return NBX_ERR_ARG;  // monopoles, one body per leaf
    int rc = nbx::adjoint_record_all(C(c), reinterpret_cast<nbx::Adj *>(a), s, S(stream));
    if (rc) return rc;
    return nbx_sync_status(c, stream);
}

int nbx_adjoint_replay_fp64(nbx_ctx *c, nbx_adjoint *a, const double *state0, double *loss, void *stream) {
    if (!c || !a || !state0 || !loss) return NBX_ERR_ARG;
    int rc = nbx::adjoint_replay_fp64(C(c), reinterpret_cast<nbx::Adj *>(a), state0, loss, S(stream));
    if (rc) return rc;
    return nbx_sync_status(c, stream);
}

int nbx_adjoint_stats(nbx_adjoint *a, int64_t *bytes, float *forward_ms, float *backward_ms) {
    if (!a) return NBX_ERR_ARG;
    const nbx::Adj *p = reinterpret_cast<const nbx::Adj *>(a);
    if (bytes) *bytes = (int64_t)nbx::adjoint_bytes(p);
    nbx::adjoint_times(p, forward_ms, backward_ms);
    return NBX_OK;
}

}  // extern "C"
