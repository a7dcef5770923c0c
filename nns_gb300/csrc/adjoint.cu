// adjoint.cu -- gradients of a trajectory loss through the Barnes-Hut pipeline.
//
// Forward (kick-drift, Kernels.cu:581-600):  v' = v + dt a(x, m);  x' = x + d dt v'
// with a_i = sum_{c in L(i)} M_c d (|d|^2+eps2)^-3/2, d = X_c - x_i, over the
// interaction list L(i) of i's walk group, X_c, M_c the cell's centre of mass and
// mass (a body: its position and mass).  The lists (MAC decisions) are piecewise
// constant in the state and are frozen to the ones the forward recorded.
//
// Reverse step (lx, lv: gradients w.r.t. the step's outputs x', v'):
//   lv_tot = lv + d dt lx;  g = dt lv_tot                       (k_adj_prep)
//   force VJP with cotangent g, J(d) = I s^-3 - 3 d d^T s^-5:     (k_adj_force)
//     target term  lx_i -= sum_c M_c J(d_ic) g_i
//     source terms Gx_c += sum_i M_c J(d_ic) g_i, Gm_c += sum_i g_i . d_ic s^-3
//   through X_c = sum m_j x_j / M_c, M_c = sum m_j to every member body j:   (k_adj_bodies)
//     lx_j += m_j sum_{c ∋ j} Gx_c / M_c + Gx_body(j)
//     lm_j += x_j . sum_{c ∋ j} Gx_c / M_c + sum_{c ∋ j} (Gm_c - Gx_c . X_c / M_c) + Gm_body(j)
//   lx = lx + (terms above);  lv = lv_tot.
// Loss L = sum_i |x_i(T) - x*_i|^2, so lx(T) = 2 (x(T) - x*), lv(T) = 0.
//
// Memory: checkpoints of (x, v) every C steps; a segment of C steps is
// recomputed with each step's tree and interaction lists recorded on a tape,
// then reversed.  The forward steps with the recording walk's kernel (96-slot
// buffers, plain FP32) without the recording, so the recompute is bit-identical
// (every kernel is deterministic).  The forward records the last segment as it
// goes, so the reverse pass starts without recomputing it.
//
// An FP64 replay of the recorded trajectory (same lists and tree structure,
// centres of mass recomputed from the perturbed state) gives the FP64 loss
// used for finite-difference checks of the gradients.
#include <cstring>
#include <vector>

#include "f32x2.cuh"
#include "nbx_internal.cuh"

namespace nbx {

int build_tree(Ctx *ctx, const nbx_state *s, cudaStream_t st, bool external_bbox, const float *const *bbox_ptrs);
int walk2_record(Ctx *ctx, const nbx_state *s, int *rec_list, int *rec_len, int rec_cap, cudaStream_t st);
int walk2_unrecorded(Ctx *ctx, const nbx_state *s, cudaStream_t st);

struct TapeStep {
    float4 *node4 = nullptr;
    int *meta = nullptr, *parent = nullptr, *val = nullptr, *body_node = nullptr;
    float4 *body4 = nullptr;
    int *lists = nullptr, *list_len = nullptr;
    unsigned *lvl = nullptr;  // BFS level starts (kMaxLevel + 2 entries)
};

struct Adj {
    int T = 0, C = 0, lcap = 0, nseg = 0, n = 0, ngroups = 0, tape_steps = 0;
    float *ckpt = nullptr;   // [nseg][6][n]: x,y,z,vx,vy,vz at the start of each segment
    float *work = nullptr;   // [9][n]: working state
    float *target = nullptr; // [3][n]
    double *lam = nullptr;   // [7][n]: lx,ly,lz,lvx,lvy,lvz,lm
    float *gcot = nullptr;   // [3][n]
    float *tdx = nullptr;    // [3][n] target terms
    double *G = nullptr;     // [4][NC]: Gx,Gy,Gz,Gm
    double *loss = nullptr;  // [1]
    double *r64 = nullptr;   // FP64 replay: [10][n] state + [4][NC] moments
    std::vector<TapeStep> tape;
    size_t bytes = 0;
    // saved context pointers (the tape steps are swapped in for recording)
    float4 *ctx_node4 = nullptr, *ctx_body4 = nullptr;
    int *ctx_meta = nullptr, *ctx_parent = nullptr, *ctx_val = nullptr, *ctx_body_node = nullptr;
    float fwd_ms = 0.f, bwd_ms = 0.f;
    bool tail_taped = false;  // the forward recorded the last segment into the tape
    float *mass = nullptr;    // [n] the caller's masses, copied by the forward
    // The steps run as CUDA graphs, captured on first use and replayed: one plain
    // forward step, one recorded step and one reverse step per tape slot.  They
    // read only the adjoint's own buffers, so they stay valid from call to call
    // until the context's systems, constants or walk change (graph_gen).
    cudaStream_t gs = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t g_plain = nullptr;
    std::vector<cudaGraphExec_t> g_rec, g_rev;
    unsigned gen = 0;
};

namespace {

constexpr int kB = 256;

// start/stop events of a timed call, destroyed on every return path
struct EventPair {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = false;
    EventPair() { ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess; }
    ~EventPair() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
    EventPair(const EventPair &) = delete;
    EventPair &operator=(const EventPair &) = delete;
};

__global__ void k_copy_state(const float *x, const float *y, const float *z, const float *vx, const float *vy,
                             const float *vz, float *dst, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dst[i] = x[i];
        dst[n + i] = y[i];
        dst[2 * n + i] = z[i];
        dst[3 * n + i] = vx[i];
        dst[4 * n + i] = vy[i];
        dst[5 * n + i] = vz[i];
    }
}

__global__ void k_loss_init(const float *x, const float *y, const float *z, const float *target, int n,
                            double *lam, double *loss) {
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double dx = (double)x[i] - target[i], dy = (double)y[i] - target[n + i],
                     dz = (double)z[i] - target[2 * n + i];
        acc += dx * dx + dy * dy + dz * dz;
        lam[i] = 2.0 * dx;
        lam[n + i] = 2.0 * dy;
        lam[2 * n + i] = 2.0 * dz;
        lam[3 * n + i] = 0.0;
        lam[4 * n + i] = 0.0;
        lam[5 * n + i] = 0.0;
        lam[6 * n + i] = 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// lv_tot = lv + d dt lx; g = dt lv_tot
__global__ void k_adj_prep(double *lam, float *gcot, int n, double dt, double ddt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double lv = lam[(3 + k) * n + i] + ddt * lam[k * n + i];
            lam[(3 + k) * n + i] = lv;
            gcot[k * n + i] = (float)(dt * lv);
        }
    }
}

// Force VJP over the recorded lists, one block per walk group: its warps take
// interleaved chunks of 8 list entries (more warps in flight hide the list and
// node gathers), and their per-lane target terms are summed in shared memory in
// a fixed warp order.  Each lane evaluates two entries per packed f32x2
// instruction.  Per-lane contributions to each list entry are reduced through
// shared memory (lane l sums row l with 16-byte loads; the row stride of 36
// floats keeps every quarter-warp on distinct banks) and added to the FP64
// source gradients with atomics.
#ifndef NBX_ADJ_WARPS
#define NBX_ADJ_WARPS 8
#endif
constexpr int kAdjWarps = NBX_ADJ_WARPS;  // warps sharing one group's list

// Asynchronous 16-byte global-to-shared copies (cp.async, sm_80+): the copy
// proceeds while the warp computes; wait_group orders it before the reads.
__device__ __forceinline__ void cp_async16(float4 *dst, const float4 *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
constexpr int kChunk = 8;
constexpr int kRedStride = 36;

__global__ void __launch_bounds__(kAdjWarps * 32)
    k_adj_force(const float4 *__restrict__ node4, const float4 *__restrict__ body4, const int *__restrict__ val,
                const int *__restrict__ body_node, const int *__restrict__ groups, int ngroups,
                const int *__restrict__ body_sys, const int *__restrict__ sys_off, const int *__restrict__ lists,
                const int *__restrict__ list_len, int lcap, const float *__restrict__ gcot, int n, float eps2,
                double *__restrict__ G, int nc_cap, float *__restrict__ tdx) {
    __shared__ __align__(16) float red[kAdjWarps][kChunk * 4][kRedStride];
    __shared__ __align__(16) float4 stage[kAdjWarps][2][kChunk];  // node records of two chunks
    __shared__ float part[kAdjWarps][3][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const u64 eps2x2 = pk(eps2, eps2), mthree2 = pk(-3.f, -3.f);
    for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int p0 = groups[g];
        const int s = body_sys[p0];
        const int end = min(sys_off[s + 1], p0 + 32);
        const int p = p0 + lane;
        const bool valid = p < end;
        const float4 me = body4[valid ? p : p0];
        const int mynode = valid ? body_node[p] : -1;
        float gx = 0.f, gy = 0.f, gz = 0.f;
        int ob = 0;
        if (valid) {
            ob = val[p];
            gx = gcot[ob];
            gy = gcot[n + ob];
            gz = gcot[2 * n + ob];
        }
        const u64 px = pk(me.x, me.x), py = pk(me.y, me.y), pz = pk(me.z, me.z);
        const u64 gx2 = pk(gx, gx), gy2 = pk(gy, gy), gz2 = pk(gz, gz);
        u64 ox = 0ull, oy = 0ull, oz = 0ull;  // packed (+0, +0)
        const int len = list_len[g];
        const int *L = lists + (size_t)g * lcap;
        // A three-stage pipeline per warp: the records of the next chunk are in
        // flight (cp.async into this warp's staging slot) and the list entries of
        // the chunk after it are loading while this chunk computes.  Lanes past a
        // chunk's end fetch node 0, so every staged record is a valid float4.
        constexpr int kStride = kAdjWarps * kChunk;
        const int base0 = w * kChunk;
        int cmine = (lane < kChunk && base0 + lane < len) ? L[base0 + lane] : 0;
        if (lane < kChunk) cp_async16(&stage[w][0][lane], &node4[cmine]);
        cp_async_commit();
        int cnext = (lane < kChunk && base0 + kStride + lane < len) ? L[base0 + kStride + lane] : 0;
        int sb = 0;
        for (int base = base0; base < len; base += kStride) {
            const int cnt = min(kChunk, len - base);
            if (lane < kChunk) cp_async16(&stage[w][sb ^ 1][lane], &node4[cnext]);
            cp_async_commit();
            const int c2 = base + 2 * kStride + lane;
            const int cafter = (lane < kChunk && c2 < len) ? L[c2] : 0;
            cp_async_wait_one();  // this chunk's records have landed
            __syncwarp();
#pragma unroll
            for (int e = 0; e < kChunk; e += 2) {
                const int ca = __shfl_sync(0xffffffffu, cmine, e);
                const int cb = __shfl_sync(0xffffffffu, cmine, e + 1);
                const float4 qa = stage[w][sb][e], qb = stage[w][sb][e + 1];
                const u64 dx = sub2(pk(qa.x, qb.x), px);
                const u64 dy = sub2(pk(qa.y, qb.y), py);
                const u64 dz = sub2(pk(qa.z, qb.z), pz);
                u64 s2 = fma2(dx, dx, eps2x2);
                s2 = fma2(dy, dy, s2);
                s2 = fma2(dz, dz, s2);
                float sa, sb;
                upk(s2, sa, sb);
                // m (g s^-3/2 - 3 (d.g) d s^-5/2) = (m r^-3) (g - 3 (e.g) e), e = d / r:
                // in the unit vector e no intermediate leaves the FP32 range (s^-5/2
                // alone overflows once r is below about 2e-8, and a body's own entry,
                // d = 0, then gave 0 * inf)
                const u64 inv = pk(rsq(sa), rsq(sb));
                const u64 inv2 = mul2(inv, inv);
                const u64 ex = mul2(dx, inv), ey = mul2(dy, inv), ez = mul2(dz, inv);
                u64 eg = mul2(ex, gx2);
                eg = fma2(ey, gy2, eg);
                eg = fma2(ez, gz2, eg);
                const u64 m3eg = mul2(eg, mthree2);  // -3 (e.g)
                // a body's own entry has d = 0 and contributes nothing net; entries
                // past the chunk's end contribute nothing
                const bool la = e < cnt, lb = e + 1 < cnt;
                const u64 mm = pk(la && ca != mynode ? qa.w : 0.f, lb && cb != mynode ? qb.w : 0.f);
                const u64 mi3 = mul2(mul2(mm, inv), inv2);  // m r^-3, grouped as in the forward walk
                const u64 vx = mul2(mi3, fma2(ex, m3eg, gx2));
                const u64 vy = mul2(mi3, fma2(ey, m3eg, gy2));
                const u64 vz = mul2(mi3, fma2(ez, m3eg, gz2));
                ox = add2(ox, vx);
                oy = add2(oy, vy);
                oz = add2(oz, vz);
                float xa, xb, ya, yb, za, zb, ma, mb;
                upk(vx, xa, xb);
                upk(vy, ya, yb);
                upk(vz, za, zb);
                upk(mul2(eg, inv2), ma, mb);  // (d.g) r^-3
                red[w][4 * e + 0][lane] = xa;
                red[w][4 * e + 1][lane] = ya;
                red[w][4 * e + 2][lane] = za;
                red[w][4 * e + 3][lane] = la ? ma : 0.f;
                red[w][4 * e + 4][lane] = xb;
                red[w][4 * e + 5][lane] = yb;
                red[w][4 * e + 6][lane] = zb;
                red[w][4 * e + 7][lane] = lb ? mb : 0.f;
            }
            __syncwarp();
            // lane l reduces row l: entry l/4, component l%4
            const int crow = __shfl_sync(0xffffffffu, cmine, (lane >> 2) & 7);
            if (lane < 4 * cnt) {
                const float4 *row = reinterpret_cast<const float4 *>(&red[w][lane][0]);
                u64 s01 = 0ull, s23 = 0ull;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const float4 v = row[k];
                    s01 = add2(s01, pk(v.x, v.y));
                    s23 = add2(s23, pk(v.z, v.w));
                }
                float a0, a1, a2, a3;
                upk(s01, a0, a1);
                upk(s23, a2, a3);
                if (crow < nc_cap) atomicAdd(&G[(size_t)(lane & 3) * nc_cap + crow], (double)((a0 + a1) + (a2 + a3)));
            }
            __syncwarp();  // the staging slot and the reduction rows are free again
            cmine = cnext;
            cnext = cafter;
            sb ^= 1;
        }
        cp_async_wait_all();  // nothing of this group stays in flight
        __syncwarp();
        float xa, xb;
        upk(ox, xa, xb);
        part[w][0][lane] = xa + xb;
        upk(oy, xa, xb);
        part[w][1][lane] = xa + xb;
        upk(oz, xa, xb);
        part[w][2][lane] = xa + xb;
        __syncthreads();
        if (w == 0 && valid) {
            float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
            for (int k = 0; k < kAdjWarps; k++) {
                sx += part[k][0][lane];
                sy += part[k][1][lane];
                sz += part[k][2][lane];
            }
            tdx[ob] = -sx;
            tdx[n + ob] = -sy;
            tdx[2 * n + ob] = -sz;
        }
        __syncthreads();  // part is reused by the next group
    }
}

// Per cell, once: the terms every member body adds, (Gx_c / M_c, Gm_c - Gx_c . X_c / M_c),
// written over the cell's G entries (FP64 divisions are slow on this part: one
// per cell instead of one per body and ancestor).  Body entries stay as they are.
__global__ void k_adj_cells(const float4 *__restrict__ node4, const int *__restrict__ meta,
                            const unsigned *__restrict__ lvl, double *__restrict__ G, int nc_cap) {
    const int T = (int)lvl[kMaxLevel + 1];  // node count
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < T; c += gridDim.x * blockDim.x) {
        if (meta[c] < 0) continue;
        const float4 q = node4[c];
        const double M = q.w;
        const double gxc = G[c], gyc = G[(size_t)nc_cap + c], gzc = G[2 * (size_t)nc_cap + c],
                     gmc = G[3 * (size_t)nc_cap + c];
        G[c] = gxc / M;
        G[(size_t)nc_cap + c] = gyc / M;
        G[2 * (size_t)nc_cap + c] = gzc / M;
        G[3 * (size_t)nc_cap + c] = gmc - (gxc * q.x + gyc * q.y + gzc * q.z) / M;
    }
}

// Gradients through the centres of mass to every body, and the state update.
__global__ void k_adj_bodies(const float4 *__restrict__ body4, const int *__restrict__ val,
                             const int *__restrict__ body_node, const int *__restrict__ parent,
                             const double *__restrict__ G, int nc_cap, const float *__restrict__ tdx, double *lam,
                             int n) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int i = val[p];
        const int b = body_node[p];
        const float4 me = body4[p];
        double sax = 0.0, say = 0.0, saz = 0.0, sb = 0.0;
        int cur = parent[b];
        for (int guard = 0; guard < 64 && cur >= 0; guard++) {
            sax += G[cur];
            say += G[(size_t)nc_cap + cur];
            saz += G[2 * (size_t)nc_cap + cur];
            sb += G[3 * (size_t)nc_cap + cur];
            cur = parent[cur];
        }
        const double m = me.w;
        lam[i] += tdx[i] + m * sax + G[b];
        lam[n + i] += tdx[n + i] + m * say + G[(size_t)nc_cap + b];
        lam[2 * n + i] += tdx[2 * n + i] + m * saz + G[2 * (size_t)nc_cap + b];
        lam[6 * n + i] += (double)me.x * sax + (double)me.y * say + (double)me.z * saz + sb +
                          G[3 * (size_t)nc_cap + b];
    }
}

__global__ void k_lam_out(const double *lam, int n, float *gx, float *gy, float *gz, float *gvx, float *gvy,
                          float *gvz, float *gm) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        gx[i] = (float)lam[i];
        gy[i] = (float)lam[n + i];
        gz[i] = (float)lam[2 * n + i];
        gvx[i] = (float)lam[3 * n + i];
        gvy[i] = (float)lam[4 * n + i];
        gvz[i] = (float)lam[5 * n + i];
        gm[i] = (float)lam[6 * n + i];
    }
}

// ---- FP64 replay of a recorded trajectory ------------------------------
// r64 layout: [0..2] x,y,z  [3..5] vx,vy,vz  [6] m  [7..9] a  (original order, n each)
__global__ void k_r64_moments_level(int level, const unsigned *lvl, const int *__restrict__ meta,
                                    const int *__restrict__ val, const double *__restrict__ r64, int n,
                                    double *__restrict__ M64, int nc_cap) {
    const unsigned beg = lvl[level], end = lvl[level + 1];
    for (unsigned b = beg + blockIdx.x * blockDim.x + threadIdx.x; b < end; b += gridDim.x * blockDim.x) {
        const int pm = meta[b];
        if (pm < 0) continue;
        const int first = pm & 0x0fffffff, nch = ((pm >> 28) & 7) + 1;
        double sm = 0, sx = 0, sy = 0, sz = 0;
        for (int c = first; c < first + nch; c++) {
            const int cm = meta[c];
            if (cm < 0) {
                const int i = val[cm & 0x03ffffff];
                const double mb = r64[6 * (size_t)n + i];
                sm += mb;
                sx += mb * r64[i];
                sy += mb * r64[(size_t)n + i];
                sz += mb * r64[2 * (size_t)n + i];
            } else {
                sm += M64[c];
                sx += M64[c] * M64[(size_t)nc_cap + c];
                sy += M64[c] * M64[2 * (size_t)nc_cap + c];
                sz += M64[c] * M64[3 * (size_t)nc_cap + c];
            }
        }
        M64[b] = sm;
        M64[(size_t)nc_cap + b] = sx / sm;
        M64[2 * (size_t)nc_cap + b] = sy / sm;
        M64[3 * (size_t)nc_cap + b] = sz / sm;
    }
}

__global__ void __launch_bounds__(128) k_r64_force(const int *__restrict__ meta, const int *__restrict__ val,
                                                  const int *__restrict__ groups, int ngroups,
                                                  const int *__restrict__ body_sys, const int *__restrict__ sys_off,
                                                  const int *__restrict__ lists, const int *__restrict__ list_len,
                                                  int lcap, double *r64, int n, const double *__restrict__ M64,
                                                  int nc_cap, double eps2) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int g = blockIdx.x * warps + w; g < ngroups; g += gridDim.x * warps) {
        const int p0 = groups[g];
        const int end = min(sys_off[body_sys[p0] + 1], p0 + 32);
        const int p = p0 + lane;
        const bool valid = p < end;
        const int i = val[valid ? p : p0];
        const double xi = r64[i], yi = r64[(size_t)n + i], zi = r64[2 * (size_t)n + i];
        double ax = 0, ay = 0, az = 0;
        const int len = list_len[g];
        const int *L = lists + (size_t)g * lcap;
        for (int e = 0; e < len; e++) {
            const int c = L[e];
            const int cm = meta[c];
            double X, Y, Z, Mc;
            if (cm < 0) {
                const int j = val[cm & 0x03ffffff];
                X = r64[j];
                Y = r64[(size_t)n + j];
                Z = r64[2 * (size_t)n + j];
                Mc = r64[6 * (size_t)n + j];
            } else {
                Mc = M64[c];
                X = M64[(size_t)nc_cap + c];
                Y = M64[2 * (size_t)nc_cap + c];
                Z = M64[3 * (size_t)nc_cap + c];
            }
            const double dx = X - xi, dy = Y - yi, dz = Z - zi;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double f = Mc / (r2 * sqrt(r2));
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
        if (valid) {
            r64[7 * (size_t)n + i] = ax;
            r64[8 * (size_t)n + i] = ay;
            r64[9 * (size_t)n + i] = az;
        }
    }
}

__global__ void k_r64_update(double *r64, int n, double dt, double ddt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; k++) {
            const double v = r64[(3 + k) * (size_t)n + i] + dt * r64[(7 + k) * (size_t)n + i];
            r64[(3 + k) * (size_t)n + i] = v;
            r64[k * (size_t)n + i] += ddt * v;
        }
    }
}

__global__ void k_r64_loss(const double *r64, const float *target, int n, double *loss) {
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double dx = r64[i] - target[i], dy = r64[(size_t)n + i] - target[n + i],
                     dz = r64[2 * (size_t)n + i] - target[2 * n + i];
        acc += dx * dx + dy * dy + dz * dz;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

__global__ void k_copy_lvl(const unsigned *hist, int ntiles, const unsigned *totals, unsigned *lvl) {
    const int l = threadIdx.x;
    if (l <= kMaxLevel + 1) {
        const unsigned T = totals[1];
        unsigned v = l >= 64 ? T : hist[(size_t)(l << 2) * ntiles];
        lvl[l] = v < T ? v : T;
    }
}

int grid_for(int n) {
    int g = ceil_div(n, kB);
    return g < 1 ? 1 : (g > 2048 ? 2048 : g);
}

void swap_in(Ctx *ctx, Adj *a, int j) {
    TapeStep &t = a->tape[j];
    ctx->d_node4 = t.node4;
    ctx->d_meta = t.meta;
    ctx->d_parent = t.parent;
    ctx->d_val = t.val;
    ctx->d_body_node = t.body_node;
    ctx->d_body4 = t.body4;
}

// Back to the context's own node arrays.  Its per-build arrays (roots, cell
// list, status) now describe the tape's tree: a walk needs a new build first.
void swap_out(Ctx *ctx, Adj *a) {
    ctx->built = false;
    ctx->d_node4 = a->ctx_node4;
    ctx->d_meta = a->ctx_meta;
    ctx->d_parent = a->ctx_parent;
    ctx->d_val = a->ctx_val;
    ctx->d_body_node = a->ctx_body_node;
    ctx->d_body4 = a->ctx_body4;
}

template <typename T>
int amalloc(Ctx *ctx, Adj *a, T **p, size_t count) {
    if (count == 0) count = 1;
    if (cudaMalloc((void **)p, count * sizeof(T)) != cudaSuccess) {
        ctx->last_error = "adjoint: device allocation failed";
        *p = nullptr;
        return NBX_ERR_NOMEM;
    }
    a->bytes += count * sizeof(T);
    return NBX_OK;
}

// One recorded step j of the working state: build into tape slot j, walk with
// list recording, integrate.
int recorded_step(Ctx *ctx, Adj *a, const nbx_state *s, int j, cudaStream_t st) {
    swap_in(ctx, a, j);
    int rc = build_tree(ctx, s, st, false, nullptr);
    if (!rc) {
        k_copy_lvl<<<1, 64, 0, st>>>(ctx->d_hist, ctx->cap_tiles_node, ctx->d_totals, a->tape[j].lvl);
        ++ctx->launches;
        rc = walk2_record(ctx, s, a->tape[j].lists, a->tape[j].list_len, a->lcap, st);
    }
    if (!rc) rc = integrate(ctx, s, ctx->p.dt, ctx->p.dampening, a->n, st);
    swap_out(ctx, a);
    return rc;
}

nbx_state work_state(Adj *a) {
    const int n = a->n;
    nbx_state w{};
    w.x = a->work;
    w.y = a->work + n;
    w.z = a->work + 2 * n;
    w.vx = a->work + 3 * n;
    w.vy = a->work + 4 * n;
    w.vz = a->work + 5 * n;
    w.ax = a->work + 6 * n;
    w.ay = a->work + 7 * n;
    w.az = a->work + 8 * n;
    w.m = a->mass;
    return w;
}

void destroy_graphs(Adj *a) {
    if (a->g_plain) cudaGraphExecDestroy(a->g_plain);
    a->g_plain = nullptr;
    for (auto *v : {&a->g_rec, &a->g_rev})
        for (cudaGraphExec_t &g : *v) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

// Replays *g on st, capturing body() into it first if it is empty.
template <typename F>
int replay(Ctx *ctx, cudaStream_t st, cudaGraphExec_t *g, F &&body) {
    if (!*g) {
        cudaGraph_t graph = nullptr;
        NBX_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = body();
        const cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (rc || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            if (rc) return rc;
            ctx->last_error = std::string("adjoint graph capture: ") + cudaGetErrorString(e);
            return NBX_ERR_CUDA;
        }
        const cudaError_t ei = cudaGraphInstantiate(g, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            *g = nullptr;
            ctx->last_error = std::string("adjoint graph instantiate: ") + cudaGetErrorString(ei);
            return NBX_ERR_CUDA;
        }
    }
    NBX_CUDA(cudaGraphLaunch(*g, st));
    return NBX_OK;
}

// The caller's stream and the adjoint's stream, ordered both ways by events.
int enter(Ctx *ctx, Adj *a, cudaStream_t user) {
    if (a->gen != ctx->graph_gen) {
        destroy_graphs(a);
        a->gen = ctx->graph_gen;
    }
    NBX_CUDA(cudaEventRecord(a->ev_in, user));
    NBX_CUDA(cudaStreamWaitEvent(a->gs, a->ev_in, 0));
    return NBX_OK;
}

int leave(Ctx *ctx, Adj *a, cudaStream_t user) {
    ctx->built = false;  // the context's per-build arrays describe a tape's tree
    NBX_CUDA(cudaEventRecord(a->ev_out, a->gs));
    NBX_CUDA(cudaStreamWaitEvent(user, a->ev_out, 0));
    return NBX_OK;
}

// One reverse step through tape slot j.
int reverse_step(Ctx *ctx, Adj *a, int j, cudaStream_t st) {
    const int n = a->n, NC = ctx->cap_nodes;
    const double dt = ctx->p.dt, ddt = (double)ctx->p.dampening * ctx->p.dt;
    TapeStep &t = a->tape[j];
    k_adj_prep<<<grid_for(n), kB, 0, st>>>(a->lam, a->gcot, n, dt, ddt);
    NBX_CUDA(cudaMemsetAsync(a->G, 0, sizeof(double) * 4 * (size_t)NC, st));
    const int blocks = a->ngroups;
    k_adj_force<<<blocks < ctx->nsm * 16 ? blocks : ctx->nsm * 16, kAdjWarps * 32, 0, st>>>(
        t.node4, t.body4, t.val, t.body_node, ctx->d_groups, a->ngroups, ctx->d_body_sys, ctx->d_sys_off, t.lists,
        t.list_len, a->lcap, a->gcot, n, ctx->eps2, a->G, NC, a->tdx);
    k_adj_cells<<<grid_for(NC), kB, 0, st>>>(t.node4, t.meta, t.lvl, a->G, NC);
    k_adj_bodies<<<grid_for(n), kB, 0, st>>>(t.body4, t.val, t.body_node, t.parent, a->G, NC, a->tdx, a->lam, n);
    ctx->launches += 4;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

}  // namespace

int adjoint_create(Ctx *ctx, int T, int C, int lcap, int tape_steps, Adj **out) {
    *out = nullptr;
    if (ctx->nsys < 1 || T < 1 || C < 1 || lcap < 64 || tape_steps < C) return NBX_ERR_ARG;
    Adj *a = new Adj();
    a->T = T;
    a->C = C;
    a->lcap = lcap;
    a->n = (int)ctx->nbodies;
    a->ngroups = ctx->ngroups;
    a->nseg = ceil_div(T, C);
    a->tape_steps = tape_steps;
    const int n = a->n, NC = ctx->cap_nodes;
    int rc = 0;
    rc |= amalloc(ctx, a, &a->ckpt, (size_t)a->nseg * 6 * n);
    rc |= amalloc(ctx, a, &a->work, (size_t)9 * n);
    rc |= amalloc(ctx, a, &a->target, (size_t)3 * n);
    rc |= amalloc(ctx, a, &a->lam, (size_t)7 * n);
    rc |= amalloc(ctx, a, &a->gcot, (size_t)3 * n);
    rc |= amalloc(ctx, a, &a->tdx, (size_t)3 * n);
    rc |= amalloc(ctx, a, &a->G, (size_t)4 * NC);
    rc |= amalloc(ctx, a, &a->loss, 2);
    rc |= amalloc(ctx, a, &a->r64, (size_t)10 * n + (size_t)4 * NC);
    rc |= amalloc(ctx, a, &a->mass, (size_t)n);
    if (cudaStreamCreateWithFlags(&a->gs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&a->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&a->ev_out, cudaEventDisableTiming) != cudaSuccess) {
        ctx->last_error = "adjoint: stream or event creation failed";
        rc |= NBX_ERR_CUDA;
    }
    a->g_rec.assign(tape_steps, nullptr);
    a->g_rev.assign(tape_steps, nullptr);
    a->gen = ctx->graph_gen;
    a->tape.resize(tape_steps);
    for (int j = 0; j < tape_steps && rc == 0; j++) {
        TapeStep &t = a->tape[j];
        rc |= amalloc(ctx, a, &t.node4, NC);
        rc |= amalloc(ctx, a, &t.meta, NC);
        rc |= amalloc(ctx, a, &t.parent, NC);
        rc |= amalloc(ctx, a, &t.val, ctx->cap_bodies);
        rc |= amalloc(ctx, a, &t.body_node, ctx->cap_bodies);
        rc |= amalloc(ctx, a, &t.body4, ctx->cap_bodies);
        rc |= amalloc(ctx, a, &t.lists, (size_t)a->ngroups * lcap);
        rc |= amalloc(ctx, a, &t.list_len, a->ngroups);
        rc |= amalloc(ctx, a, &t.lvl, kMaxLevel + 2);
    }
    a->ctx_node4 = ctx->d_node4;
    a->ctx_meta = ctx->d_meta;
    a->ctx_parent = ctx->d_parent;
    a->ctx_val = ctx->d_val;
    a->ctx_body_node = ctx->d_body_node;
    a->ctx_body4 = ctx->d_body4;
    *out = a;
    return rc;
}

void adjoint_destroy(Adj *a) {
    if (!a) return;
    destroy_graphs(a);
    if (a->ev_in) cudaEventDestroy(a->ev_in);
    if (a->ev_out) cudaEventDestroy(a->ev_out);
    if (a->gs) cudaStreamDestroy(a->gs);
    void *p[] = {a->ckpt, a->work, a->target, a->lam, a->gcot, a->tdx, a->G, a->loss, a->r64, a->mass};
    for (void *q : p)
        if (q) cudaFree(q);
    for (TapeStep &t : a->tape) {
        void *r[] = {t.node4, t.meta, t.parent, t.val, t.body_node, t.body4, t.lists, t.list_len, t.lvl};
        for (void *q : r)
            if (q) cudaFree(q);
    }
    delete a;
}

size_t adjoint_bytes(const Adj *a) { return a->bytes; }

// Forward T steps from s (x, v, m), checkpoints every C steps; s ends at x(T), v(T)
// (and its accelerations are those of the last step).  The steps run on the
// adjoint's own copy of the state.
int adjoint_forward(Ctx *ctx, Adj *a, const nbx_state *s, const float *tx, const float *ty, const float *tz,
                    double *loss_host, cudaStream_t user) {
    const int n = a->n;
    if (n != ctx->nbodies) return NBX_ERR_STATE;
    int rc = enter(ctx, a, user);
    if (rc) return rc;
    const cudaStream_t st = a->gs;
    EventPair ev;
    if (!ev.ok) return NBX_ERR_CUDA;
    NBX_CUDA(cudaEventRecord(ev.e0, st));
    const float *tgt[3] = {tx, ty, tz};
    for (int k = 0; k < 3; k++)
        NBX_CUDA(cudaMemcpyAsync(a->target + (size_t)k * n, tgt[k], sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    float *const caller[9] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->ax, s->ay, s->az};
    for (int k = 0; k < 6; k++)
        NBX_CUDA(cudaMemcpyAsync(a->work + (size_t)k * n, caller[k], sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    NBX_CUDA(cudaMemcpyAsync(a->mass, s->m, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    const nbx_state w = work_state(a);
    a->tail_taped = false;
    const int k_tail = (a->nseg - 1) * a->C;  // first step of the last segment
    for (int k = 0; k < a->T && !rc; k++) {
        if (k % a->C == 0) {
            k_copy_state<<<grid_for(n), kB, 0, st>>>(w.x, w.y, w.z, w.vx, w.vy, w.vz,
                                                     a->ckpt + (size_t)(k / a->C) * 6 * n, n);
            ++ctx->launches;
        }
        if (k >= k_tail) {
            const int j = k - k_tail;
            rc = replay(ctx, st, &a->g_rec[j], [&] { return recorded_step(ctx, a, &w, j, st); });
        } else {
            rc = replay(ctx, st, &a->g_plain, [&] {
                int r = build_tree(ctx, &w, st, false, nullptr);
                if (!r) r = walk2_unrecorded(ctx, &w, st);
                if (!r) r = integrate(ctx, &w, ctx->p.dt, ctx->p.dampening, n, st);
                return r;
            });
        }
    }
    if (rc) {
        leave(ctx, a, user);
        return rc;
    }
    a->tail_taped = true;
    for (int k = 0; k < 9; k++)
        NBX_CUDA(cudaMemcpyAsync(caller[k], a->work + (size_t)k * n, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    NBX_CUDA(cudaMemsetAsync(a->loss, 0, sizeof(double), st));
    k_loss_init<<<grid_for(n), kB, 0, st>>>(w.x, w.y, w.z, a->target, n, a->lam, a->loss);
    ++ctx->launches;
    NBX_CUDA(cudaEventRecord(ev.e1, st));
    NBX_CUDA(cudaMemcpyAsync(loss_host, a->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    NBX_CUDA(cudaStreamSynchronize(st));
    cudaEventElapsedTime(&a->fwd_ms, ev.e0, ev.e1);
    return leave(ctx, a, user);
}

// Reverse through all segments; writes dL/dx0, dL/dv0, dL/dm (original order).
int adjoint_backward(Ctx *ctx, Adj *a, const nbx_state *s, float *gx, float *gy, float *gz, float *gvx, float *gvy,
                     float *gvz, float *gm, cudaStream_t user) {
    (void)s;  // the reverse pass works on the forward's copy of the state
    const int n = a->n;
    int rc = enter(ctx, a, user);
    if (rc) return rc;
    const cudaStream_t st = a->gs;
    const nbx_state w = work_state(a);
    EventPair ev;
    if (!ev.ok) return NBX_ERR_CUDA;
    NBX_CUDA(cudaEventRecord(ev.e0, st));
    for (int seg = a->nseg - 1; seg >= 0 && !rc; seg--) {
        const int k0 = seg * a->C;
        const int steps = (k0 + a->C <= a->T) ? a->C : a->T - k0;
        if (!(seg == a->nseg - 1 && a->tail_taped)) {
            NBX_CUDA(cudaMemcpyAsync(a->work, a->ckpt + (size_t)seg * 6 * n, sizeof(float) * 6 * n,
                                     cudaMemcpyDeviceToDevice, st));
            for (int j = 0; j < steps && !rc; j++)
                rc = replay(ctx, st, &a->g_rec[j], [&] { return recorded_step(ctx, a, &w, j, st); });
        }
        a->tail_taped = false;  // the tape now holds this segment
        for (int j = steps - 1; j >= 0 && !rc; j--)
            rc = replay(ctx, st, &a->g_rev[j], [&] { return reverse_step(ctx, a, j, st); });
    }
    if (rc) {
        leave(ctx, a, user);
        return rc;
    }
    k_lam_out<<<grid_for(n), kB, 0, st>>>(a->lam, n, gx, gy, gz, gvx, gvy, gvz, gm);
    ++ctx->launches;
    NBX_CUDA(cudaEventRecord(ev.e1, st));
    NBX_CUDA(cudaStreamSynchronize(st));
    cudaEventElapsedTime(&a->bwd_ms, ev.e0, ev.e1);
    NBX_CUDA(cudaGetLastError());
    return leave(ctx, a, user);
}

// Records the whole T-step trajectory from s (needs tape_steps >= T).
int adjoint_record_all(Ctx *ctx, Adj *a, const nbx_state *s, cudaStream_t st) {
    if (a->tape_steps < a->T) return NBX_ERR_ARG;
    a->tail_taped = false;
    const int n = a->n;
    const nbx_state w = work_state(a);
    k_copy_state<<<grid_for(n), kB, 0, st>>>(s->x, s->y, s->z, s->vx, s->vy, s->vz, a->work, n);
    ++ctx->launches;
    NBX_CUDA(cudaMemcpyAsync(a->mass, s->m, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    for (int k = 0; k < a->T; k++) {
        int rc = recorded_step(ctx, a, &w, k, st);
        if (rc) return rc;
    }
    ctx->built = false;
    NBX_CUDA(cudaStreamSynchronize(st));
    return NBX_OK;
}

// FP64 loss of the recorded trajectory from an FP64 initial state (x0,v0,m as
// double arrays [7][n] on the device), lists and tree structure frozen.
int adjoint_replay_fp64(Ctx *ctx, Adj *a, const double *state0, double *loss_host, cudaStream_t st) {
    if (a->tape_steps < a->T) return NBX_ERR_ARG;
    const int n = a->n, NC = ctx->cap_nodes;
    double *M64 = a->r64 + (size_t)10 * n;
    NBX_CUDA(cudaMemcpyAsync(a->r64, state0, sizeof(double) * 7 * n, cudaMemcpyDeviceToDevice, st));
    const double dt = ctx->p.dt, ddt = (double)ctx->p.dampening * ctx->p.dt;
    for (int k = 0; k < a->T; k++) {
        TapeStep &t = a->tape[k];
        for (int level = kMaxLevel - 2; level >= 1; level--)
            k_r64_moments_level<<<ctx->nsm * 2, kB, 0, st>>>(level, t.lvl, t.meta, t.val, a->r64, n, M64, NC);
        const int blocks = ceil_div(a->ngroups, 4);
        k_r64_force<<<blocks < ctx->nsm * 16 ? blocks : ctx->nsm * 16, 128, 0, st>>>(
            t.meta, t.val, ctx->d_groups, a->ngroups, ctx->d_body_sys, ctx->d_sys_off, t.lists, t.list_len, a->lcap,
            a->r64, n, M64, NC, (double)ctx->eps2);
        k_r64_update<<<grid_for(n), kB, 0, st>>>(a->r64, n, dt, ddt);
        ctx->launches += kMaxLevel - 2 + 2;
    }
    NBX_CUDA(cudaMemsetAsync(a->loss + 1, 0, sizeof(double), st));
    k_r64_loss<<<grid_for(n), kB, 0, st>>>(a->r64, a->target, n, a->loss + 1);
    ++ctx->launches;
    NBX_CUDA(cudaMemcpyAsync(loss_host, a->loss + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
    NBX_CUDA(cudaStreamSynchronize(st));
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

void adjoint_times(const Adj *a, float *fwd_ms, float *bwd_ms) {
    if (fwd_ms) *fwd_ms = a->fwd_ms;
    if (bwd_ms) *bwd_ms = a->bwd_ms;
}

}  // namespace nbx
