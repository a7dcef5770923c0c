// walk.cu -- warp-coherent Barnes-Hut force walk (3D/CUDA/CUDA_NBody/src/Kernels.cu:460-577).
//
// One warp walks the tree for one aligned group of 32 consecutive sorted bodies
// of a system.  Semantics of the reference: the root's children are always
// opened (:505-517), a child body always interacts (:543), a child cell
// interacts only if every body of the group accepts it, dp <= r (:543), with
// dp = depth0 * 0.25^(L-1) for a level-L cell and r = |d|^2 + eps^2, else it is
// pushed (:555-559).  a += m * d * rsqrt(r)^3 (:546-551), G = 1.
// Differences by design: a root child that is a body interacts directly, the
// stack holds int node ids and is bounded with an error flag, and r is
// fma(dz,dz,fma(dy,dy,fma(dx,dx,eps2))) (the oracle uses the same rounding).
//
// Node layout: breadth-first node array, children of a cell contiguous;
// node4 = (x, y, z, m) of the body / centre of mass, meta < 0 marks a body.
// The 8 children of a popped cell are fetched by 8 lanes in one coalesced
// access and broadcast with shuffles.
#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kWalkWarps = 8;

struct Acc {
    float x = 0.f, y = 0.f, z = 0.f;
};

// Mode 0: plain FP32; 1: Kahan per term; 2: the same interaction list
// evaluated in FP64 (MAC decisions still from the FP32 r) -- the reference
// for the FP32 arithmetic error of the walk.
template <int Mode>
struct Accum;

template <>
struct Accum<0> {
    float x = 0.f, y = 0.f, z = 0.f;
    __device__ __forceinline__ void add(float f, float dx, float dy, float dz) {
        x = fmaf(f, dx, x);
        y = fmaf(f, dy, y);
        z = fmaf(f, dz, z);
    }
    __device__ __forceinline__ void get(float &ox, float &oy, float &oz) const { ox = x; oy = y; oz = z; }
};

// Kahan-compensated accumulation per component.
template <>
struct Accum<1> {
    float x = 0.f, y = 0.f, z = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    __device__ __forceinline__ static void kadd(float &s, float &c, float v) {
        const float yv = __fsub_rn(v, c);
        const float t = __fadd_rn(s, yv);
        c = __fsub_rn(__fsub_rn(t, s), yv);
        s = t;
    }
    __device__ __forceinline__ void add(float f, float dx, float dy, float dz) {
        kadd(x, cx, __fmul_rn(f, dx));
        kadd(y, cy, __fmul_rn(f, dy));
        kadd(z, cz, __fmul_rn(f, dz));
    }
    __device__ __forceinline__ void get(float &ox, float &oy, float &oz) const { ox = x; oy = y; oz = z; }
};

template <>
struct Accum<2> {
    double x = 0.0, y = 0.0, z = 0.0;
    __device__ __forceinline__ void add64(float4 c, float4 me, float eps2) {
        const double dx = (double)c.x - me.x, dy = (double)c.y - me.y, dz = (double)c.z - me.z;
        const double r = dx * dx + dy * dy + dz * dz + (double)eps2;
        const double f = (double)c.w / (r * sqrt(r));
        x += f * dx;
        y += f * dy;
        z += f * dz;
    }
};

template <int Mode, typename A>
__device__ __forceinline__ void interact(A &acc, float cx, float cy, float cz, float cw, float dx, float dy,
                                         float dz, float r, float4 me, float eps2) {
    if constexpr (Mode == 2) {
        acc.add64(make_float4(cx, cy, cz, cw), me, eps2);
    } else {
        const float ri = rsqrtf(r);
        acc.add(cw * ri * ri * ri, dx, dy, dz);
    }
}

template <int Mode>
__global__ void __launch_bounds__(kWalkWarps * 32)
    k_walk(const float4 *__restrict__ node4, const int *__restrict__ meta, const unsigned char *__restrict__ lvl8,
           const float4 *__restrict__ body4,
           const int *__restrict__ val, const int *__restrict__ groups, int ngroups,
           const int *__restrict__ body_sys, const int *__restrict__ sys_off, const float *__restrict__ depth0,
           const int *__restrict__ root_first, const int *__restrict__ root_nch, float eps2, int stack_cap,
           float *__restrict__ ax, float *__restrict__ ay, float *__restrict__ az, int2 *__restrict__ gstat,
           DevStatus *st, double *__restrict__ a64, int n64) {
    extern __shared__ int smem_stack[];
    if (st->code != 0) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *stack = smem_stack + w * stack_cap;
    unsigned long long tot_len = 0ull, tot_open = 0ull;
    for (int g = blockIdx.x * kWalkWarps + w; g < ngroups; g += gridDim.x * kWalkWarps) {
        const int p0 = groups[g];
        const int s = body_sys[p0];
        const int end = min(sys_off[s + 1], p0 + 32);
        const int p = p0 + lane;
        const bool valid = p < end;
        const float4 me = body4[valid ? p : p0];
        const float d0 = depth0[s];
        Accum<Mode> acc;
        int top = 0, len = 0, opened = 0;
        bool overflow = false;

        // root children (level 1): bodies interact, cells are opened unconditionally
        {
            const int first = root_first[s], nch = min(root_nch[s], 8);
            float4 c4 = make_float4(0.f, 0.f, 0.f, 0.f);
            int cm = 0;
            if (lane < nch) {
                c4 = node4[first + lane];
                cm = meta[first + lane];
            }
            for (int j = 0; j < nch; j++) {
                const int cmj = __shfl_sync(0xffffffffu, cm, j);
                const float cx = __shfl_sync(0xffffffffu, c4.x, j);
                const float cy = __shfl_sync(0xffffffffu, c4.y, j);
                const float cz = __shfl_sync(0xffffffffu, c4.z, j);
                const float cw = __shfl_sync(0xffffffffu, c4.w, j);
                if (cmj < 0) {
                    const float dx = cx - me.x, dy = cy - me.y, dz = cz - me.z;
                    const float r = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                    interact<Mode>(acc, cx, cy, cz, cw, dx, dy, dz, r, me, eps2);
                    len++;
                } else {
                    if (lane == 0) stack[top] = first + j;
                    top++;
                    opened++;
                }
            }
            __syncwarp();
        }

        while (top > 0) {
            const int b = stack[top - 1];  // stack entries are node indices
            __syncwarp();
            top--;
            const int lvl = lvl8[b];
            const int mb = meta[b];
            const int first = mb & 0x0fffffff;
            const int nch = ((mb >> 28) & 7) + 1;
            const float dp = ldexpf(d0, -2 * lvl);
            float4 c4 = make_float4(0.f, 0.f, 0.f, 0.f);
            int cm = 0;
            if (lane < nch) {
                c4 = node4[first + lane];
                cm = meta[first + lane];
            }
            for (int j = 0; j < nch; j++) {
                const int cmj = __shfl_sync(0xffffffffu, cm, j);
                const float cx = __shfl_sync(0xffffffffu, c4.x, j);
                const float cy = __shfl_sync(0xffffffffu, c4.y, j);
                const float cz = __shfl_sync(0xffffffffu, c4.z, j);
                const float cw = __shfl_sync(0xffffffffu, c4.w, j);
                const float dx = cx - me.x, dy = cy - me.y, dz = cz - me.z;
                const float r = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                const bool accept = (cmj < 0) || __all_sync(0xffffffffu, !valid || dp <= r);
                if (accept) {
                    interact<Mode>(acc, cx, cy, cz, cw, dx, dy, dz, r, me, eps2);
                    len++;
                } else {
                    if (top >= stack_cap) {
                        overflow = true;
                        break;
                    }
                    if (lane == 0) stack[top] = first + j;
                    top++;
                    opened++;
                }
            }
            __syncwarp();
            if (overflow) break;
        }
        if (overflow) {
            if (lane == 0) set_status(st, NBX_ERR_STACK, g);
            continue;
        }
        if (valid) {
            const int ob = val[p];
            if constexpr (Mode == 2) {
                a64[ob] = acc.x;
                a64[(size_t)n64 + ob] = acc.y;
                a64[2 * (size_t)n64 + ob] = acc.z;
            } else {
                float fx, fy, fz;
                acc.get(fx, fy, fz);
                ax[ob] = fx;
                ay[ob] = fy;
                az[ob] = fz;
            }
        }
        if (gstat && lane == 0) gstat[g] = make_int2(len, opened);
        tot_len += (unsigned long long)len * (unsigned long long)(end - p0);
        tot_open += (unsigned long long)opened;
    }
    if (Mode != 2 && lane == 0 && (tot_len | tot_open)) {
        atomicAdd(&st->interactions, tot_len);
        atomicAdd(&st->opened, tot_open);
    }
}

}  // namespace

int walk2_init(Ctx *ctx);
int walk2_forces(Ctx *ctx, const nbx_state *s, float *pot, int warps, cudaStream_t st, int g0 = 0, int gn = -1);

int walk_init(Ctx *ctx) {
    // the attribute is per kernel, not per context: allow the device maximum
    // (8 warps x 4096 entries x 4 bytes = 128 KB at most)
    NBX_CUDA(cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->p.device));
    NBX_CUDA(cudaDeviceGetAttribute(&ctx->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->p.device));
    NBX_CUDA(cudaFuncSetAttribute(k_walk<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin));
    NBX_CUDA(cudaFuncSetAttribute(k_walk<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin));
    NBX_CUDA(cudaFuncSetAttribute(k_walk<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin));
    return walk2_init(ctx);
}

int walk_potential(Ctx *ctx, const nbx_state *s, float *pot, cudaStream_t st) {
    if (!ctx->built) return NBX_ERR_STATE;
    return walk2_forces(ctx, s, pot, ctx->walk_warps, st);
}

// A rank's share of a system split over several GPUs: the walk of groups
// [first, first + count) only (production walk variants).
int walk_forces_groups(Ctx *ctx, const nbx_state *s, int first, int count, cudaStream_t st) {
    if (!ctx->built) return NBX_ERR_STATE;
    if (first < 0 || count < 0 || first > ctx->ngroups || count > ctx->ngroups - first) return NBX_ERR_ARG;
    if (ctx->walk_variant == 2) {
        ctx->last_error = "walk of a group range: the one-cell walk (variant 2) walks all groups";
        return NBX_ERR_ARG;
    }
    if (count == 0) return NBX_OK;
    return walk2_forces(ctx, s, nullptr, ctx->walk_warps, st, first, count);
}

int walk_forces(Ctx *ctx, const nbx_state *s, cudaStream_t st) {
    if (!ctx->built) return NBX_ERR_STATE;
    if (ctx->walk_variant != 2) return walk2_forces(ctx, s, nullptr, ctx->walk_warps, st);
    const int cap = ctx->p.stack_depth;
    const size_t smem = (size_t)kWalkWarps * cap * sizeof(int);
    const int blocks_needed = ceil_div(ctx->ngroups, kWalkWarps);
    const int grid = blocks_needed < ctx->nsm * 8 ? blocks_needed : ctx->nsm * 8;
    if (grid <= 0) return NBX_OK;
    if (ctx->compensated) {
        k_walk<1><<<grid, kWalkWarps * 32, smem, st>>>(
            ctx->d_node4, ctx->d_meta, ctx->d_lvl8, ctx->d_body4, ctx->d_val, ctx->d_groups, ctx->ngroups, ctx->d_body_sys,
            ctx->d_sys_off, ctx->d_depth0, ctx->d_root_first, ctx->d_root_nch, ctx->eps2, cap, s->ax, s->ay,
            s->az, ctx->d_gstat, ctx->d_status, nullptr, 0);
        ++ctx->launches;
    } else {
        k_walk<0><<<grid, kWalkWarps * 32, smem, st>>>(
            ctx->d_node4, ctx->d_meta, ctx->d_lvl8, ctx->d_body4, ctx->d_val, ctx->d_groups, ctx->ngroups, ctx->d_body_sys,
            ctx->d_sys_off, ctx->d_depth0, ctx->d_root_first, ctx->d_root_nch, ctx->eps2, cap, s->ax, s->ay,
            s->az, ctx->d_gstat, ctx->d_status, nullptr, 0);
        ++ctx->launches;
    }
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

// The last build's interaction lists of the given walk groups (first sorted
// positions, device array) evaluated in FP64 into a64 [3][nbodies] (original
// order; rows of bodies outside those groups are untouched).
int walk_fp64_lists(Ctx *ctx, const int *group_starts, int ngroups, double *a64, cudaStream_t st) {
    if (!ctx->built) return NBX_ERR_STATE;
    if (ngroups <= 0) return NBX_OK;
    const int cap = ctx->p.stack_depth;
    const size_t smem = (size_t)kWalkWarps * cap * sizeof(int);
    const int blocks_needed = ceil_div(ngroups, kWalkWarps);
    const int grid = blocks_needed < ctx->nsm * 8 ? blocks_needed : ctx->nsm * 8;
    k_walk<2><<<grid, kWalkWarps * 32, smem, st>>>(
        ctx->d_node4, ctx->d_meta, ctx->d_lvl8, ctx->d_body4, ctx->d_val, group_starts, ngroups, ctx->d_body_sys, ctx->d_sys_off,
        ctx->d_depth0, ctx->d_root_first, ctx->d_root_nch, ctx->eps2, cap, nullptr, nullptr, nullptr, nullptr,
        ctx->d_status, a64, (int)ctx->nbodies);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

}  // namespace nbx
