// walk2.cu -- the production force walk: same interaction lists as walk.cu
// (the reference's warp-coherent MAC, 3D/CUDA/CUDA_NBody/src/Kernels.cu:460-577),
// organised for throughput on sm_103a.
//
// Per warp (one aligned group of 32 sorted bodies), rounds of
//   expand   up to P stack cells are popped at once, one per lane; their child
//            blocks (contiguous in the BFS node array) are copied into a
//            per-warp candidate buffer in shared memory, each candidate with its
//            acceptance threshold dp (-inf for a body: bodies always interact;
//            dp = depth0 * 0.25^(L-1) for a level-L cell);
//   evaluate every lane streams the buffer with broadcast shared-memory loads;
//            two candidates per instruction with the packed FP32 pair
//            instructions (add/fma/mul .rn.f32x2, each lane an IEEE FP32 op, so r
//            and the MAC decisions are bit-identical to the scalar form); one warp
//            vote per candidate decides accept (interact) or reject (push to the
//            stack); rejected cells are pushed 32 at a time with a ballot prefix.
// P is bounded by the buffer (8 children per cell) and by the stack headroom
// (a round grows the stack by at most 7 per popped cell), so the stack cannot
// overflow unless a single depth-first path needs more than stack_cap entries,
// which is reported as NBX_ERR_STACK.
//
// Accumulation modes: 0 plain FP32 (two packed partial sums), 1 split
// compensation (plain FP32 within a round, Kahan across rounds), 2 Kahan on
// every term.  Optional per-body potential for the energy diagnostics.
#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kCB = 128;          // candidate slots per warp (even)
constexpr int kPairs = kCB / 2;

typedef unsigned long long u64;

__device__ __forceinline__ u64 pk(float a, float b) {
    u64 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(u64 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ u64 sub2(u64 a, u64 b) {
    u64 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ u64 add2(u64 a, u64 b) {
    u64 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ u64 mul2(u64 a, u64 b) {
    u64 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ u64 fma2(u64 a, u64 b, u64 c) {
    u64 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Kahan step s += v with compensation c (scalar, explicit rounding).
__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = __fsub_rn(v, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

struct WarpBuf {
    ulonglong2 a[kPairs];  // (x0,x1) (y0,y1)
    ulonglong2 b[kPairs];  // (z0,z1) (m0,m1)
    u64 d[kPairs];         // (dp0,dp1)
    int id[kCB];           // node | level << 26 (only read for rejected cells)
};

__device__ __forceinline__ void put_cand(WarpBuf &w, int slot, float4 q, float dp, int id) {
    float *a = reinterpret_cast<float *>(&w.a[slot >> 1]);
    float *b = reinterpret_cast<float *>(&w.b[slot >> 1]);
    float *d = reinterpret_cast<float *>(&w.d[slot >> 1]);
    const int h = slot & 1;
    a[h] = q.x;
    a[2 + h] = q.y;
    b[h] = q.z;
    b[2 + h] = q.w;
    d[h] = dp;
    w.id[slot] = id;
}

template <int Mode, bool Pot>
__global__ void __launch_bounds__(512, 1)
    k_walk2(const float4 *__restrict__ node4, const int *__restrict__ meta, const float4 *__restrict__ body4,
            const int *__restrict__ val, const int *__restrict__ groups, int ngroups,
            const int *__restrict__ body_sys, const int *__restrict__ sys_off, const float *__restrict__ depth0,
            const int *__restrict__ root_first, const int *__restrict__ root_nch, float eps2, int stack_cap,
            float *__restrict__ ax, float *__restrict__ ay, float *__restrict__ az, float *__restrict__ pot,
            int *__restrict__ nlist, int *__restrict__ nopen, DevStatus *st) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (st->code != 0) return;
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpBuf &buf = reinterpret_cast<WarpBuf *>(smem_raw)[w];
    int *stack = reinterpret_cast<int *>(smem_raw + sizeof(WarpBuf) * warps) + w * stack_cap;
    const unsigned lt = (1u << lane) - 1u;
    const u64 eps2x2 = pk(eps2, eps2);
    unsigned long long tot_len = 0ull, tot_open = 0ull;

    for (int g = blockIdx.x * warps + w; g < ngroups; g += gridDim.x * warps) {
        const int p0 = groups[g];
        const int s = body_sys[p0];
        const int end = min(sys_off[s + 1], p0 + 32);
        const int p = p0 + lane;
        const bool valid = p < end;
        // lanes past the end of the system take lane 0's body: their MAC votes
        // repeat lane 0's and their results are discarded
        const float4 me = body4[valid ? p : p0];
        const u64 px = pk(me.x, me.x), py = pk(me.y, me.y), pz = pk(me.z, me.z);
        const float d0 = depth0[s];
        u64 sx = 0ull, sy = 0ull, sz = 0ull, sp = 0ull;  // packed partial sums (+0.0f, +0.0f)
        float kx = 0.f, ky = 0.f, kz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;  // Kahan totals
        int top = 0, ncand = 0, len = 0, opened = 0;
        bool overflow = false;

        // root children: cells are opened unconditionally, bodies interact
        {
            const int rf = root_first[s], rn = min(root_nch[s], 8);
            int cm = 0;
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < rn) {
                cm = meta[rf + lane];
                q = node4[rf + lane];
            }
            const unsigned bodies = __ballot_sync(0xffffffffu, lane < rn && cm < 0);
            const unsigned cells = __ballot_sync(0xffffffffu, lane < rn && cm >= 0);
            if (lane < rn && cm < 0) put_cand(buf, __popc(bodies & lt), q, -INFINITY, rf + lane);
            if (lane < rn && cm >= 0) stack[__popc(cells & lt)] = (rf + lane) | (1 << kLevelShift);
            ncand = __popc(bodies);
            top = __popc(cells);
            opened += top;
            __syncwarp();
        }

        while (top > 0 || ncand > 0) {
            // ---- expand
            int P = min(min(top, 32), min((kCB - ncand) >> 3, (stack_cap - top) / 7));
            if (P <= 0 && ncand == 0) {
                overflow = true;
                break;
            }
            if (P < 0) P = 0;
            int first = 0, nch = 0, lvl = 0;
            if (lane < P) {
                const int e = stack[top - 1 - lane];
                const int b = e & ((1 << kLevelShift) - 1);
                lvl = e >> kLevelShift;
                const int mb = meta[b];
                first = mb & 0x0fffffff;
                nch = ((mb >> 28) & 7) + 1;
            }
            int incl = nch;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += u;
            }
            const int T = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            top -= P;
            if (nch > 0) {
                const float dpc = ldexpf(d0, -2 * lvl);  // children are at level lvl+1
                const int base = ncand + incl - nch;
                for (int k = 0; k < nch; k++) {
                    const int c = first + k;
                    const int cm = meta[c];
                    put_cand(buf, base + k, node4[c], cm < 0 ? -INFINITY : dpc, c | ((lvl + 1) << kLevelShift));
                }
            }
            const int nreal = ncand + T;
            int npad = nreal;
            if (nreal & 1) {
                if (lane == 0) put_cand(buf, nreal, make_float4(1e18f, 1e18f, 1e18f, 0.f), -INFINITY, 0);
                npad = nreal + 1;
            }
            __syncwarp();

            // ---- evaluate
            const int npairs = npad >> 1;
            int nrej = 0;
            for (int c0 = 0; c0 < npairs; c0 += 16) {
                const int cnt = min(16, npairs - c0);
                unsigned rej = 0u;
#pragma unroll 2
                for (int q = 0; q < cnt; q++) {
                    const ulonglong2 A = buf.a[c0 + q];
                    const ulonglong2 B = buf.b[c0 + q];
                    float dpa, dpb;
                    upk(buf.d[c0 + q], dpa, dpb);
                    const u64 dx = sub2(A.x, px);
                    const u64 dy = sub2(A.y, py);
                    const u64 dz = sub2(B.x, pz);
                    u64 r = fma2(dx, dx, eps2x2);
                    r = fma2(dy, dy, r);
                    r = fma2(dz, dz, r);
                    float ra, rb;
                    upk(r, ra, rb);
                    const bool oka = __all_sync(0xffffffffu, dpa <= ra);
                    const bool okb = __all_sync(0xffffffffu, dpb <= rb);
                    float ma, mb;
                    upk(B.y, ma, mb);
                    const u64 ri = pk(rsqrtf(ra), rsqrtf(rb));
                    const u64 mm = pk(oka ? ma : 0.f, okb ? mb : 0.f);
                    const u64 f = mul2(mul2(mul2(mm, ri), ri), ri);
                    if (Mode == 2) {
                        float xa, xb, ya, yb, za, zb;
                        upk(mul2(f, dx), xa, xb);
                        upk(mul2(f, dy), ya, yb);
                        upk(mul2(f, dz), za, zb);
                        kahan(kx, cx, xa); kahan(kx, cx, xb);
                        kahan(ky, cy, ya); kahan(ky, cy, yb);
                        kahan(kz, cz, za); kahan(kz, cz, zb);
                    } else {
                        sx = fma2(f, dx, sx);
                        sy = fma2(f, dy, sy);
                        sz = fma2(f, dz, sz);
                    }
                    if (Pot) sp = fma2(mm, ri, sp);
                    rej |= (oka ? 0u : 1u) << (2 * q);
                    rej |= (okb ? 0u : 1u) << (2 * q + 1);
                }
                if (rej) {
                    const int nr = __popc(rej);
                    if ((rej >> lane) & 1u) {
                        const int pos = top + __popc(rej & lt);
                        stack[pos] = buf.id[2 * c0 + lane];
                    }
                    top += nr;
                    nrej += nr;
                }
            }
            len += nreal - nrej;
            opened += nrej;
            ncand = 0;
            if (Mode == 1) {  // fold this round's partial sums into the compensated totals
                float a0, a1;
                upk(sx, a0, a1); kahan(kx, cx, a0); kahan(kx, cx, a1);
                upk(sy, a0, a1); kahan(ky, cy, a0); kahan(ky, cy, a1);
                upk(sz, a0, a1); kahan(kz, cz, a0); kahan(kz, cz, a1);
                sx = sy = sz = 0ull;
            }
            __syncwarp();
        }
        if (overflow) {
            if (lane == 0) set_status(st, NBX_ERR_STACK, g);
            continue;
        }
        if (valid) {
            float fx, fy, fz;
            if (Mode == 0) {
                float a0, a1;
                upk(sx, a0, a1); fx = a0 + a1;
                upk(sy, a0, a1); fy = a0 + a1;
                upk(sz, a0, a1); fz = a0 + a1;
            } else {
                fx = kx - cx;
                fy = ky - cy;
                fz = kz - cz;
            }
            const int ob = val[p];
            ax[ob] = fx;
            ay[ob] = fy;
            az[ob] = fz;
            if (Pot) {
                float a0, a1;
                upk(sp, a0, a1);
                // remove the body's own term m * rsqrt(eps2), then phi = -sum
                pot[ob] = -((a0 + a1) - me.w * rsqrtf(eps2));
            }
            if (nlist) nlist[ob] = len;
            if (nopen) nopen[ob] = opened;
        }
        tot_len += (unsigned long long)len * (unsigned long long)(end - p0);
        tot_open += (unsigned long long)opened;
    }
    if (lane == 0 && (tot_len | tot_open)) {
        atomicAdd(&st->interactions, tot_len);
        atomicAdd(&st->opened, tot_open);
    }
}

template <int Mode, bool Pot>
int launch(Ctx *ctx, const nbx_state *s, float *pot, int warps, cudaStream_t st) {
    const int cap = ctx->p.stack_depth;
    const size_t smem = (size_t)warps * (sizeof(WarpBuf) + (size_t)cap * sizeof(int));
    const int blocks_needed = ceil_div(ctx->ngroups, warps);
    int per_sm = 1;
    NBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk2<Mode, Pot>, warps * 32, smem));
    if (per_sm < 1) per_sm = 1;
    const int grid = blocks_needed < ctx->nsm * per_sm ? blocks_needed : ctx->nsm * per_sm;
    if (grid <= 0) return NBX_OK;
    k_walk2<Mode, Pot><<<grid, warps * 32, smem, st>>>(
        ctx->d_node4, ctx->d_meta, ctx->d_body4, ctx->d_val, ctx->d_groups, ctx->ngroups, ctx->d_body_sys,
        ctx->d_sys_off, ctx->d_depth0, ctx->d_root_first, ctx->d_root_nch, ctx->eps2, cap, s->ax, s->ay, s->az,
        pot, ctx->d_nlist, ctx->d_nopen, ctx->d_status);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

template <int Mode, bool Pot>
int set_attr(Ctx *ctx, int smem_max) {
    NBX_CUDA(cudaFuncSetAttribute(k_walk2<Mode, Pot>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
    return NBX_OK;
}

}  // namespace

size_t walk2_smem_per_warp(int stack_cap) { return sizeof(WarpBuf) + (size_t)stack_cap * sizeof(int); }

int walk2_init(Ctx *ctx) {
    int smem_optin = 0;
    NBX_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->p.device));
    const int smem_max = smem_optin;
    int rc = 0;
    rc |= set_attr<0, false>(ctx, smem_max);
    rc |= set_attr<1, false>(ctx, smem_max);
    rc |= set_attr<2, false>(ctx, smem_max);
    rc |= set_attr<0, true>(ctx, smem_max);
    return rc;
}

int walk2_forces(Ctx *ctx, const nbx_state *s, float *pot, int warps, cudaStream_t st) {
    if (pot) return launch<0, true>(ctx, s, pot, warps, st);
    switch (ctx->compensated) {
        case 1: return launch<1, false>(ctx, s, nullptr, warps, st);
        case 2: return launch<2, false>(ctx, s, nullptr, warps, st);
        default: return launch<0, false>(ctx, s, nullptr, warps, st);
    }
}

}  // namespace nbx
