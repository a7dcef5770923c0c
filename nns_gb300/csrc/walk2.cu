// walk2.cu -- the production force walk: same interaction lists as walk.cu
// (the reference's warp-coherent MAC, 3D/CUDA/CUDA_NBody/src/Kernels.cu:460-577),
// organised for throughput on sm_103a.
//
// Per warp (one aligned group of 32 sorted bodies), rounds of
//   expand   the P top-of-stack cells whose children fit the buffers are popped
//            at once, one per lane; their child blocks (contiguous in the BFS
//            node array) are spread over the lanes, one child per lane.  Each
//            lane classifies its child cell against the group's box and the
//            representative pair of the child's octant (exactly, see below): surely accepted cells
//            join the bodies in the body buffer, surely rejected cells are
//            pushed at once, the rest go to the cell buffer with their
//            threshold dp = depth0 * 0.25^(L-1) and id;
//   evaluate every lane streams the buffers with broadcast shared-memory loads,
//            two candidates per instruction with the packed FP32 pair
//            instructions (add/fma/mul .rn.f32x2: each lane an IEEE FP32 op, so r
//            and the MAC decisions are bit-identical to the scalar form).  Body
//            buffer pairs go straight to the accumulation; each cell of the cell
//            buffer takes one warp vote (dp <= r on every lane) and is
//            accumulated or pushed.
// Wide rounds run while the stack keeps a depth-first reserve free (7 entries
// per level of the group's system's deepest level); beyond that the walk pops
// one cell per round, which can never outgrow the reserve, so a stack of at
// least kDfsReserve + 7*8 entries cannot overflow (NBX_ERR_STACK otherwise).
//
// Accumulation modes: 0 plain FP32 (two packed partial sums), 1 split
// compensation (plain FP32 within a round, Kahan across rounds), 2 Kahan on
// every term.  Optional per-body potential for the energy diagnostics.
#include "f32x2.cuh"
#include "nbx_internal.cuh"

namespace nbx {

namespace {

// Stack entries kept free for depth-first descent: from any stack content a
// depth-first walk (one cell per round) grows the stack by at most 7 entries per
// level below the popped cell, i.e. by less than 7 * (deepest level) <= 7 * 42.
// The walk uses the bound of the tree at hand (its deepest level, recorded by
// the build); kDfsReserve is the bound for any tree.
constexpr int kDfsReserve = 7 * 42 + 8;

// Build-time tuning knobs of the evaluation loops (defaults are the measured best).
#ifndef NBX_BODY_UNROLL
#define NBX_BODY_UNROLL 16
#endif
#ifndef NBX_CELL_UNROLL
#define NBX_CELL_UNROLL 4
#endif
#ifndef NBX_WALK64_THREADS
#define NBX_WALK64_THREADS 512
#endif
#ifndef NBX_WALK64_MINB
#define NBX_WALK64_MINB 2
#endif
#ifndef NBX_WALK128_THREADS
#define NBX_WALK128_THREADS 256
#endif
#ifndef NBX_WALK128_MINB
#define NBX_WALK128_MINB 3
#endif
// (#pragma arguments are not macro-expanded: the unroll factors go through constants)
constexpr int kBodyUnroll = NBX_BODY_UNROLL;
constexpr int kCellUnroll = NBX_CELL_UNROLL;

// depth0 * 4^-k exactly (a power-of-two product is exact unless it underflows)
__device__ __forceinline__ float scale4(float d0, int k) {
    return d0 * __int_as_float((127 - 2 * k) << 23);
}

// Kahan step s += v with compensation c (scalar, explicit rounding).
__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = __fsub_rn(v, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// Per-warp candidate buffers of CB slots each.
template <int CB>
struct WarpBuf {
    static constexpr int kPairs = CB / 2;
    ulonglong2 ba[kPairs];  // bodies: (x0,x1) (y0,y1)
    ulonglong2 bb[kPairs];  //         (z0,z1) (m0,m1)
    ulonglong2 ca[kPairs];  // cells:  (x0,x1) (y0,y1)
    ulonglong2 cb[kPairs];  //         (z0,z1) (m0,m1)
    u64 cd[kPairs];         //         (dp0,dp1)
    int cid[CB];            //         node index
    int bid[CB];            // body node ids (interaction-list recording only)
    float4 cls[3];          // group box lo, hi, centre
    ulonglong2 rxy[8];      // representative bodies, in pairs: (x0,x1) (y0,y1)
    u64 rz[8];              //                                  (z0,z1)
};

__device__ __forceinline__ void put4(ulonglong2 *a, ulonglong2 *b, int slot, float4 q) {
    float *pa = reinterpret_cast<float *>(&a[slot >> 1]);
    float *pb = reinterpret_cast<float *>(&b[slot >> 1]);
    const int h = slot & 1;
    pa[h] = q.x;
    pa[2 + h] = q.y;
    pb[h] = q.z;
    pb[2 + h] = q.w;
}

// Quadrupole mode: the traceless quadrupoles of the cell buffer's slots, in
// pairs: (xx, yy), (zz, xy), (xz, yz).
template <int CB>
struct QuadBuf {
    static constexpr int kPairs = CB / 2;
    ulonglong2 qa[kPairs];
    ulonglong2 qb[kPairs];
    ulonglong2 qc[kPairs];
};

__device__ __forceinline__ void putq(ulonglong2 *qa, ulonglong2 *qb, ulonglong2 *qc, int slot, float4 q4, float2 q2) {
    float *pa = reinterpret_cast<float *>(&qa[slot >> 1]);
    float *pb = reinterpret_cast<float *>(&qb[slot >> 1]);
    float *pc = reinterpret_cast<float *>(&qc[slot >> 1]);
    const int h = slot & 1;
    pa[h] = q4.x;
    pa[2 + h] = q4.y;
    pb[h] = q4.z;
    pb[2 + h] = q4.w;
    pc[h] = q2.x;
    pc[2 + h] = q2.y;
}

struct Sums {
    u64 x = 0ull, y = 0ull, z = 0ull, p = 0ull;  // packed partial sums (+0.0f, +0.0f)
    float kx = 0.f, ky = 0.f, kz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;  // Kahan totals
};

// Accumulate the packed force factor f = m*rsqrt(r)^3 of two candidates.
template <int Mode, bool Pot>
__device__ __forceinline__ void accumulate(Sums &a, u64 f, u64 mm, u64 ri, u64 dx, u64 dy, u64 dz) {
    if (Mode == 2) {
        float xa, xb, ya, yb, za, zb;
        upk(mul2(f, dx), xa, xb);
        upk(mul2(f, dy), ya, yb);
        upk(mul2(f, dz), za, zb);
        kahan(a.kx, a.cx, xa);
        kahan(a.kx, a.cx, xb);
        kahan(a.ky, a.cy, ya);
        kahan(a.ky, a.cy, yb);
        kahan(a.kz, a.cz, za);
        kahan(a.kz, a.cz, zb);
    } else {
        a.x = fma2(f, dx, a.x);
        a.y = fma2(f, dy, a.y);
        a.z = fma2(f, dz, a.z);
    }
    if (Pot) a.p = fma2(mm, ri, a.p);
}

// Accumulate r^-2 v for two candidates: the quadrupole mode's contribution.
template <int Mode>
__device__ __forceinline__ void accumulate_quad(Sums &a, u64 ri2, u64 vx, u64 vy, u64 vz) {
    if (Mode == 2) {
        float xa, xb, ya, yb, za, zb;
        upk(mul2(ri2, vx), xa, xb);
        upk(mul2(ri2, vy), ya, yb);
        upk(mul2(ri2, vz), za, zb);
        kahan(a.kx, a.cx, xa);
        kahan(a.kx, a.cx, xb);
        kahan(a.ky, a.cy, ya);
        kahan(a.ky, a.cy, yb);
        kahan(a.kz, a.cz, za);
        kahan(a.kz, a.cz, zb);
    } else {
        a.x = fma2(ri2, vx, a.x);
        a.y = fma2(ri2, vy, a.y);
        a.z = fma2(ri2, vz, a.z);
    }
}

// One pair of cells of the quadrupole mode, with the cells' negated traceless
// quadrupoles P = -Q from slot pair q of the buffer (d = cell - body,
// r^2 = |d|^2 + eps^2, e = d / r):
//   a += m d r^-3 - Q d r^-5 + 5/2 (d.Q.d) d r^-7
//      = r^-2 [ (m - 5/2 (e.P.e) r^-2) e + (P e) r^-2 ].
// In the unit-vector form every intermediate is bounded by |Q| or by the
// mass and force scales, and the only power of r^-1 is r^-2 <= 1 / eps^2.
// With d itself, r^-5 and r^-7 overflow FP32 once r is below about 1e-8, and
// d.Q.d (~ |Q| d^2) underflows for cells of about 1e-12 and less, dropping a
// term that is 1e-2 of such a pair's force.  A rejected half of a voted pair
// comes with ri = 0, so its e and r^-2, and its whole term, are 0.
template <int Mode, int CB>
__device__ __forceinline__ void quad_term(Sums &acc, const QuadBuf<CB> &qbuf, int q, u64 mm, u64 ri, u64 dx, u64 dy,
                                          u64 dz) {
    const ulonglong2 QA = qbuf.qa[q], QB = qbuf.qb[q], QC = qbuf.qc[q];
    const u64 ri2 = mul2(ri, ri);
    const u64 ex = mul2(dx, ri), ey = mul2(dy, ri), ez = mul2(dz, ri);
    // P e: P = (xx, yy, zz, xy | xz, yz) in QA = (xx, yy), QB = (zz, xy), QC = (xz, yz)
    const u64 px = fma2(QC.x, ez, fma2(QB.y, ey, mul2(QA.x, ex)));
    const u64 py = fma2(QC.y, ez, fma2(QA.y, ey, mul2(QB.y, ex)));
    const u64 pz = fma2(QB.x, ez, fma2(QC.y, ey, mul2(QC.x, ex)));
    const u64 epe = fma2(ez, pz, fma2(ey, py, mul2(ex, px)));
    const u64 mq = fma2(mul2(epe, ri2), pk(-2.5f, -2.5f), mm);
    accumulate_quad<Mode>(acc, ri2, fma2(mq, ex, mul2(px, ri2)), fma2(mq, ey, mul2(py, ri2)),
                          fma2(mq, ez, mul2(pz, ri2)));
}

// CB = 64 and 96: 64-register budget (two 16-warp or four 8-warp blocks per SM);
// CB = 128: up to 85 registers for more loads in flight (three 8-warp blocks).
template <int CB>
struct WalkBounds {
    static constexpr int kThreads = CB <= 96 ? NBX_WALK64_THREADS : NBX_WALK128_THREADS;
    static constexpr int kMinBlocks = CB <= 96 ? NBX_WALK64_MINB : NBX_WALK128_MINB;
};

template <int CB, int Mode, bool Pot, bool Rec, bool Quad = false>
__global__ void __launch_bounds__(WalkBounds<CB>::kThreads, WalkBounds<CB>::kMinBlocks)
    k_walk2(const float4 *__restrict__ node4, const int *__restrict__ meta, const unsigned char *__restrict__ lvl8,
            const float4 *__restrict__ quad4, const float2 *__restrict__ quad2, const float4 *__restrict__ body4,
            const int *__restrict__ val, const int *__restrict__ groups, int ngroups,
            const int *__restrict__ body_sys, const int *__restrict__ sys_off, const float *__restrict__ depth0,
            const int *__restrict__ root_first, const int *__restrict__ root_nch, const int *__restrict__ sys_lvl,
            float eps2, int stack_cap,
            float *__restrict__ ax, float *__restrict__ ay, float *__restrict__ az, float *__restrict__ pot,
            int2 *__restrict__ gstat, DevStatus *st, int *__restrict__ rec_list,
            int *__restrict__ rec_len, int rec_cap) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (st->code != 0) return;
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kCB = CB;
    WarpBuf<CB> &buf = reinterpret_cast<WarpBuf<CB> *>(smem_raw)[w];
    constexpr size_t kQuadBytes = Quad ? sizeof(QuadBuf<CB>) : 0;
    QuadBuf<CB> &qbuf = reinterpret_cast<QuadBuf<CB> *>(smem_raw + sizeof(WarpBuf<CB>) * warps)[w];
    int *stack = reinterpret_cast<int *>(smem_raw + (sizeof(WarpBuf<CB>) + kQuadBytes) * warps) + w * stack_cap;
    const unsigned lt = (1u << lane) - 1u;
    const u64 eps2x2 = pk(eps2, eps2);
    unsigned long long tot_len = 0ull, tot_open = 0ull, tot_rounds = 0ull, tot_cand = 0ull;

    // groups are handed out dynamically (costs vary widely between groups)
    for (;;) {
        int g = 0;
        if (lane == 0) g = (int)atomicAdd(&st->walk_next, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= ngroups) break;
        const int p0 = groups[g];
        const int s = body_sys[p0];
        const int end = min(sys_off[s + 1], p0 + 32);
        // the depth-first reserve from this system's own tree, so that a system's
        // rounds (and force sums) do not depend on the other systems of a batch
        const int reserve = 7 * min(max(sys_lvl[s], 1), 42) + 8;
        const int p = p0 + lane;
        const bool valid = p < end;
        // lanes past the end of the system take lane 0's body: their MAC votes
        // repeat lane 0's and their results are discarded
        const float4 me = body4[valid ? p : p0];
        const u64 px = pk(me.x, me.x), py = pk(me.y, me.y), pz = pk(me.z, me.z);
        const float d0 = depth0[s];
        {
            // the group's box and representative bodies, for classifying children
            float b[6] = {me.x, me.x, me.y, me.y, me.z, me.z};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                for (int k = 0; k < 6; k += 2) {
                    b[k] = fminf(b[k], __shfl_xor_sync(0xffffffffu, b[k], o));
                    b[k + 1] = fmaxf(b[k + 1], __shfl_xor_sync(0xffffffffu, b[k + 1], o));
                }
            }
            // the body nearest the box centre (lane lc)
            const float ex = me.x - 0.5f * (b[0] + b[1]), ey = me.y - 0.5f * (b[2] + b[3]);
            const float ez = me.z - 0.5f * (b[4] + b[5]);
            const unsigned key = __float_as_uint(ex * ex + ey * ey + ez * ez);
            const unsigned kmin = __reduce_min_sync(0xffffffffu, key);
            const int lc = __ffs(__ballot_sync(0xffffffffu, key == kmin)) - 1;
            if (lane == 0) {
                buf.cls[0] = make_float4(b[0], b[2], b[4], 0.f);
                buf.cls[1] = make_float4(b[1], b[3], b[5], 0.f);
                buf.cls[2] = make_float4(0.5f * (b[0] + b[1]), 0.5f * (b[2] + b[3]), 0.5f * (b[4] + b[5]), 0.f);
            }
            // representative pairs for the sure-reject test, one per octant k (bit
            // a set: the cell lies on the + side of axis a, seen from the box
            // centre): the body furthest along that diagonal and the body nearest
            // the centre.  Any valid body is a correct representative; these two
            // catch 86 % of the rejected cells before the vote (the first and last
            // body of the group caught 58 %).
            {
                const float nx = __shfl_sync(0xffffffffu, me.x, lc), ny = __shfl_sync(0xffffffffu, me.y, lc);
                const float nz = __shfl_sync(0xffffffffu, me.z, lc);
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const float pj = (k & 1 ? ex : -ex) + (k & 2 ? ey : -ey) + (k & 4 ? ez : -ez);
                    const unsigned key_k = valid ? f2ord(pj) : 0u;
                    const unsigned kmax = __reduce_max_sync(0xffffffffu, key_k);
                    const int le = __ffs(__ballot_sync(0xffffffffu, key_k == kmax)) - 1;
                    const float xk = __shfl_sync(0xffffffffu, me.x, le), yk = __shfl_sync(0xffffffffu, me.y, le);
                    const float zk = __shfl_sync(0xffffffffu, me.z, le);
                    if (lane == k) {
                        buf.rxy[k] = make_ulonglong2(pk(xk, nx), pk(yk, ny));
                        buf.rz[k] = pk(zk, nz);
                    }
                }
            }
            __syncwarp();
        }
        Sums acc;
        int top = 0, nb = 0, len = 0, opened = 0, nrec = 0;
        bool overflow = false;
        int *rec = Rec ? rec_list + (size_t)g * rec_cap : nullptr;

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
            if (lane < rn && cm < 0) {
                put4(buf.ba, buf.bb, __popc(bodies & lt), q);
                if (Rec) buf.bid[__popc(bodies & lt)] = rf + lane;
            }
            if (lane < rn && cm >= 0) stack[__popc(cells & lt)] = rf + lane;
            nb = __popc(bodies);
            top = __popc(cells);
            opened += top;
            __syncwarp();
        }

        while (top > 0 || nb > 0) {
            // ---- expand: lane j pops stack[top-1-j] and copies its children
            // wide rounds while the stack keeps the depth-first reserve free,
            // else one cell per round (depth-first), which cannot outgrow it
            // P = the most top-of-stack cells whose children fit the buffers
            const int avail = min(top, 32);
            int first = 0, nch = 0;
            float dpp = 0.f;  // the children's opening threshold, depth0 * 4^-level(popped cell)
            if (lane < avail) {
                const int b = stack[top - 1 - lane];  // stack entries are node indices
                const int mb = meta[b];
                first = mb & 0x0fffffff;
                nch = ((mb >> 28) & 7) + 1;
                dpp = scale4(d0, lvl8[b]);
            }
            int incl = nch;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += u;
            }
            const int excl = incl - nch;
            const int cbase = first - excl;  // child t of this lane's cell is node cbase + t
            // (the quadrupole mode keeps one slot free: its two cell regions are
            // padded to whole pairs independently)
            int P = __popc(__ballot_sync(0xffffffffu, lane < avail && incl <= kCB - nb - (Quad ? 1 : 0)));
            int T = __shfl_sync(0xffffffffu, incl, (P + 31) & 31);
            // the stack grows by at most T - P: wide rounds only while that keeps
            // the depth-first reserve free, else one cell
            if (P > 1 && top - P + T > stack_cap - reserve) {
                P = 1;
                T = __shfl_sync(0xffffffffu, incl, 0);
            }
            if (P > 0 && top - P + T > stack_cap) P = 0;
            if (P == 0) T = 0;
            if (P == 0 && nb == 0) {
                overflow = true;
                break;
            }
            __syncwarp();
            top -= P;
            // the T children are spread over the lanes, 32 at a time: lane t
            // finds its popped cell j (largest j < P with excl_j <= t) by counting
            // the segment starts at or below t in a bit mask of the starts
            unsigned seg[kCB / 32];
#pragma unroll
            for (int k = 0; k < kCB / 32; k++)
                seg[k] = __reduce_or_sync(0xffffffffu, (lane < P && (excl >> 5) == k) ? 1u << (excl & 31) : 0u);
            // Each child cell is classified by its lane before any warp-wide work:
            //   sure accept: a lower bound of every lane's r (the gaps between the
            //     cell and the group box, in the walk's own FP32 operation order;
            //     rounding is monotone) is >= dp, so the vote would pass: the cell
            //     goes to the body buffer (no vote);
            //   sure reject: a representative body's r (computed exactly as its
            //     lane does) is < dp, so the vote would fail: pushed at once;
            //   otherwise it is voted on in the cell buffer.
            // The interaction lists are unchanged; only their order differs.
            int nbody = nb, ncell = 0, nsrej = 0, nacc = 0;
            int jbase = -1;
#pragma unroll
            for (int k = 0; k < kCB / 32; k++) {
                const int t0 = 32 * k;
                if (t0 >= T) break;
                const int t = t0 + lane;
                const unsigned le = lane == 31 ? 0xffffffffu : (2u << lane) - 1u;
                const int j = jbase + __popc(seg[k] & le);
                jbase += __popc(seg[k]);
                const int bj = __shfl_sync(0xffffffffu, cbase, j);
                const float dpc = __shfl_sync(0xffffffffu, dpp, j);
                const bool ok = t < T;
                const int c = bj + t;
                const int cm = ok ? meta[c] : 0;
                const float4 q = ok ? node4[c] : make_float4(0.f, 0.f, 0.f, 0.f);
                const bool isc = ok && cm >= 0;
                float4 qq4 = make_float4(0.f, 0.f, 0.f, 0.f);
                float2 qq2 = make_float2(0.f, 0.f);
                if (Quad && isc) {
                    qq4 = quad4[c];
                    qq2 = quad2[c];
                }
                bool sacc = false, srej = false;
                {  // on every lane, without a branch; the results are masked by isc below
                    const float4 lo = buf.cls[0], hi = buf.cls[1];
                    const float gx = fmaxf(0.f, fmaxf(__fsub_rn(lo.x, q.x), __fsub_rn(q.x, hi.x)));
                    const float gy = fmaxf(0.f, fmaxf(__fsub_rn(lo.y, q.y), __fsub_rn(q.y, hi.y)));
                    const float gz = fmaxf(0.f, fmaxf(__fsub_rn(lo.z, q.z), __fsub_rn(q.z, hi.z)));
                    sacc = dpc <= __fmaf_rn(gz, gz, __fmaf_rn(gy, gy, __fmaf_rn(gx, gx, eps2)));
                    // the representative pair of the cell's octant, in one packed
                    // instruction with the operations and order of the evaluation
                    // (so r is their lanes' r exactly)
                    const u64 qx = pk(q.x, q.x), qy = pk(q.y, q.y), qz = pk(q.z, q.z);
                    {
                        const float4 cen = buf.cls[2];
                        const int oct = (q.x > cen.x ? 1 : 0) | (q.y > cen.y ? 2 : 0) | (q.z > cen.z ? 4 : 0);
                        const ulonglong2 R = buf.rxy[oct];
                        const u64 dx = sub2(qx, R.x), dy = sub2(qy, R.y), dz = sub2(qz, buf.rz[oct]);
                        float ra, rb;
                        upk(fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, eps2x2))), ra, rb);
                        srej = ra < dpc || rb < dpc;
                    }
                }
                // quadrupole mode: accepted cells need their quadrupoles, so a surely
                // accepted cell goes to the top of the cell buffer (filled downwards),
                // evaluated without a vote; the cells to vote on fill it upwards
                const bool tob = ok && (cm < 0 || (!Quad && isc && sacc));
                const bool toc = isc && !sacc && !srej;
                const bool tos = isc && !sacc && srej;
                const bool toa = Quad && isc && sacc;
                const unsigned bm = __ballot_sync(0xffffffffu, tob);
                const unsigned cmk = __ballot_sync(0xffffffffu, toc);
                const unsigned smk = __ballot_sync(0xffffffffu, tos);
                if (Quad) {
                    const unsigned amk = __ballot_sync(0xffffffffu, toa);
                    if (toa) {
                        const int slot = kCB - 1 - (nacc + __popc(amk & lt));
                        put4(buf.ca, buf.cb, slot, q);
                        putq(qbuf.qa, qbuf.qb, qbuf.qc, slot, qq4, qq2);
                    }
                    nacc += __popc(amk);
                }
                if (tob) {
                    put4(buf.ba, buf.bb, nbody + __popc(bm & lt), q);
                    if (Rec) buf.bid[nbody + __popc(bm & lt)] = c;
                }
                if (toc) {
                    const int slot = ncell + __popc(cmk & lt);
                    put4(buf.ca, buf.cb, slot, q);
                    reinterpret_cast<float *>(&buf.cd[slot >> 1])[slot & 1] = dpc;
                    buf.cid[slot] = c;
                    if (Quad) putq(qbuf.qa, qbuf.qb, qbuf.qc, slot, qq4, qq2);
                }
                if (tos) stack[top + nsrej + __popc(smk & lt)] = c;
                nbody += __popc(bm);
                ncell += __popc(cmk);
                nsrej += __popc(smk);
            }
            top += nsrej;
            // pad odd buffers with a massless far-away candidate that is accepted
            if (lane == 0 && (nbody & 1)) put4(buf.ba, buf.bb, nbody, make_float4(1e18f, 1e18f, 1e18f, 0.f));
            if (lane == 1 && (ncell & 1)) {
                put4(buf.ca, buf.cb, ncell, make_float4(1e18f, 1e18f, 1e18f, 0.f));
                reinterpret_cast<float *>(&buf.cd[ncell >> 1])[1] = -INFINITY;
                if (Quad)
                    putq(qbuf.qa, qbuf.qb, qbuf.qc, ncell, make_float4(0.f, 0.f, 0.f, 0.f), make_float2(0.f, 0.f));
            }
            // the accepted region [kCB - nacc, kCB) starts on a whole pair: a
            // massless, quadrupole-free far candidate fills its odd first slot
            // (ncell + nacc < kCB keeps it clear of the voted region's pad)
            const int abeg = (kCB - nacc) & ~1;
            if (Quad && lane == 2 && ((kCB - nacc) & 1)) {
                put4(buf.ca, buf.cb, abeg, make_float4(1e18f, 1e18f, 1e18f, 0.f));
                putq(qbuf.qa, qbuf.qb, qbuf.qc, abeg, make_float4(0.f, 0.f, 0.f, 0.f), make_float2(0.f, 0.f));
            }
            __syncwarp();

            // ---- evaluate bodies: no MAC
            const int nbp = (nbody + 1) >> 1;
#pragma unroll (kBodyUnroll)
            for (int q = 0; q < nbp; q++) {
                const ulonglong2 A = buf.ba[q];
                const ulonglong2 B = buf.bb[q];
                const u64 dx = sub2(A.x, px);
                const u64 dy = sub2(A.y, py);
                const u64 dz = sub2(B.x, pz);
                u64 r = fma2(dx, dx, eps2x2);
                r = fma2(dy, dy, r);
                r = fma2(dz, dz, r);
                float ra, rb;
                upk(r, ra, rb);
                const u64 ri = pk(rsq(ra), rsq(rb));
                // no MAC depends on this product: (m ri)(ri ri) shortens its dependency chain
                const u64 f = mul2(mul2(B.y, ri), mul2(ri, ri));
                accumulate<Mode, Pot>(acc, f, B.y, ri, dx, dy, dz);
            }
            if (Rec) {  // every body candidate is an interaction
                for (int t = lane; t < nbody; t += 32)
                    if (nrec + t < rec_cap) rec[nrec + t] = buf.bid[t];
                nrec += nbody;
            }
            // ---- quadrupole mode: surely accepted cells, no vote
            if (Quad) {
#pragma unroll (kCellUnroll)
                for (int q = abeg >> 1; q < kCB / 2; q++) {
                    const ulonglong2 A = buf.ca[q];
                    const ulonglong2 B = buf.cb[q];
                    const u64 dx = sub2(A.x, px);
                    const u64 dy = sub2(A.y, py);
                    const u64 dz = sub2(B.x, pz);
                    u64 r = fma2(dx, dx, eps2x2);
                    r = fma2(dy, dy, r);
                    r = fma2(dz, dz, r);
                    float ra, rb;
                    upk(r, ra, rb);
                    const u64 ri = pk(rsq(ra), rsq(rb));
                    quad_term<Mode>(acc, qbuf, q, B.y, ri, dx, dy, dz);
                }
            }
            // ---- evaluate cells: one vote per cell, accept or push
            const int ncp = (ncell + 1) >> 1;
            int nrej = 0;
#pragma unroll (kCellUnroll)
            for (int q = 0; q < ncp; q++) {
                const ulonglong2 A = buf.ca[q];
                const ulonglong2 B = buf.cb[q];
                float dpa, dpb;
                upk(buf.cd[q], dpa, dpb);
                const u64 dx = sub2(A.x, px);
                const u64 dy = sub2(A.y, py);
                const u64 dz = sub2(B.x, pz);
                u64 r = fma2(dx, dx, eps2x2);
                r = fma2(dy, dy, r);
                r = fma2(dz, dz, r);
                float ra, rb;
                upk(r, ra, rb);
#ifdef NBX_REDUX_VOTE
                const unsigned vab = __reduce_and_sync(0xffffffffu, (dpa <= ra ? 1u : 0u) | (dpb <= rb ? 2u : 0u));
                const bool oka = vab & 1u, okb = (vab >> 1) & 1u;
#else
                const bool oka = __all_sync(0xffffffffu, dpa <= ra);
                const bool okb = __all_sync(0xffffffffu, dpb <= rb);
#endif
                if (oka || okb) {  // warp-uniform: a pair of rejected cells adds nothing
                    if (!Quad) {
                        float ma, mb;
                        upk(B.y, ma, mb);
                        const u64 ri = pk(rsq(ra), rsq(rb));
                        const u64 mm = pk(oka ? ma : 0.f, okb ? mb : 0.f);
                        const u64 f = mul2(mul2(mul2(mm, ri), ri), ri);
                        accumulate<Mode, Pot>(acc, f, mm, ri, dx, dy, dz);
                    } else {
                        // the rejected half of the pair masked through r^-1 (its term is 0)
                        const u64 ri = pk(oka ? rsq(ra) : 0.f, okb ? rsq(rb) : 0.f);
                        quad_term<Mode>(acc, qbuf, q, B.y, ri, dx, dy, dz);
                    }
                }
                if (!oka) {
                    if (lane == 0) stack[top + nrej] = buf.cid[2 * q];
                    nrej++;
                } else if (Rec && 2 * q < ncell) {
                    if (lane == 0 && nrec < rec_cap) rec[nrec] = buf.cid[2 * q];
                    nrec++;
                }
                if (!okb) {
                    if (lane == 0) stack[top + nrej] = buf.cid[2 * q + 1];
                    nrej++;
                } else if (Rec && 2 * q + 1 < ncell) {
                    if (lane == 0 && nrec < rec_cap) rec[nrec] = buf.cid[2 * q + 1];
                    nrec++;
                }
            }
            top += nrej;
            tot_rounds += 1ull;
            tot_cand += (unsigned long long)(nbody + ncell + nsrej + nacc);
            len += nbody + ncell - nrej + nacc;
            opened += nrej + nsrej;
            nb = 0;
            if (Mode == 1) {  // fold this round's partial sums into the compensated totals
                float a0, a1;
                upk(acc.x, a0, a1);
                kahan(acc.kx, acc.cx, a0);
                kahan(acc.kx, acc.cx, a1);
                upk(acc.y, a0, a1);
                kahan(acc.ky, acc.cy, a0);
                kahan(acc.ky, acc.cy, a1);
                upk(acc.z, a0, a1);
                kahan(acc.kz, acc.cz, a0);
                kahan(acc.kz, acc.cz, a1);
                acc.x = acc.y = acc.z = 0ull;
            }
            __syncwarp();
        }
        if (overflow) {
            if (lane == 0) set_status(st, NBX_ERR_STACK, g);
            continue;
        }
        if (Rec && lane == 0) {
            rec_len[g] = nrec < rec_cap ? nrec : rec_cap;
            if (nrec > rec_cap) set_status(st, NBX_ERR_CAPACITY, g);
        }
        if (valid) {
            float fx, fy, fz;
            if (Mode == 0) {
                float a0, a1;
                upk(acc.x, a0, a1);
                fx = a0 + a1;
                upk(acc.y, a0, a1);
                fy = a0 + a1;
                upk(acc.z, a0, a1);
                fz = a0 + a1;
            } else {
                fx = acc.kx - acc.cx;
                fy = acc.ky - acc.cy;
                fz = acc.kz - acc.cz;
            }
            const int ob = val[p];
            ax[ob] = fx;
            ay[ob] = fy;
            az[ob] = fz;
            if (Pot) {
                float a0, a1;
                upk(acc.p, a0, a1);
                // remove the body's own term m * rsqrt(eps2), then phi = -sum
                pot[ob] = -((a0 + a1) - me.w * rsq(eps2));
            }
        }
        if (lane == 0) gstat[g] = make_int2(len, opened);
        tot_len += (unsigned long long)len * (unsigned long long)(end - p0);
        tot_open += (unsigned long long)opened;
    }
    if (lane == 0 && (tot_len | tot_open)) {
        atomicAdd(&st->interactions, tot_len);
        atomicAdd(&st->opened, tot_open);
        atomicAdd(&st->rounds, tot_rounds);
        atomicAdd(&st->candidates, tot_cand);
    }
}

template <int CB, int Mode, bool Pot, bool Rec = false, bool Quad = false>
int launch(Ctx *ctx, const nbx_state *s, float *pot, int warps, cudaStream_t st, int *rec_list = nullptr,
           int *rec_len = nullptr, int rec_cap = 0, int g_first = 0, int g_count = -1) {
    if (g_count < 0) g_count = ctx->ngroups - g_first;
    const int cap = ctx->p.stack_depth;
    const size_t smem = (size_t)warps * (sizeof(WarpBuf<CB>) + (Quad ? sizeof(QuadBuf<CB>) : 0) +
                                         (size_t)cap * sizeof(int));
    if (smem > (size_t)ctx->smem_optin) {
        ctx->last_error = "walk: stack_depth too large for the launch shape's shared memory";
        return NBX_ERR_ARG;
    }
    const int blocks_needed = ceil_div(g_count, warps);
    int per_sm = 1;
    NBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk2<CB, Mode, Pot, Rec, Quad>, warps * 32,
                                                           smem));
    if (per_sm < 1) per_sm = 1;
    const int grid = blocks_needed < ctx->nsm * per_sm ? blocks_needed : ctx->nsm * per_sm;
    if (grid <= 0) return NBX_OK;
    NBX_CUDA(cudaMemsetAsync(&ctx->d_status->walk_next, 0, sizeof(unsigned), st));
    k_walk2<CB, Mode, Pot, Rec, Quad><<<grid, warps * 32, smem, st>>>(
        ctx->d_node4, ctx->d_meta, ctx->d_lvl8, ctx->d_quad4, ctx->d_quad2, ctx->d_body4, ctx->d_val,
        ctx->d_groups + g_first, g_count, ctx->d_body_sys, ctx->d_sys_off, ctx->d_depth0, ctx->d_root_first,
        ctx->d_root_nch, ctx->d_sys_lvl, ctx->eps2, cap, s->ax, s->ay, s->az, pot, ctx->d_gstat + g_first, ctx->d_status, rec_list,
        rec_len, rec_cap);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

template <int CB, int Mode, bool Pot, bool Rec = false, bool Quad = false>
int set_attr(Ctx *ctx, int smem_max) {
    NBX_CUDA(cudaFuncSetAttribute(k_walk2<CB, Mode, Pot, Rec, Quad>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_max));
    return NBX_OK;
}

template <int CB>
int forces_cb(Ctx *ctx, const nbx_state *s, float *pot, int warps, cudaStream_t st, int g0, int gn) {
    if (pot) return launch<CB, 0, true>(ctx, s, pot, warps, st, nullptr, nullptr, 0, g0, gn);
    if (ctx->multipole) {
        if (!ctx->d_quad4) return NBX_ERR_STATE;
        switch (ctx->compensated) {
            case 1: return launch<CB, 1, false, false, true>(ctx, s, nullptr, warps, st, nullptr, nullptr, 0, g0, gn);
            case 2: return launch<CB, 2, false, false, true>(ctx, s, nullptr, warps, st, nullptr, nullptr, 0, g0, gn);
            default: return launch<CB, 0, false, false, true>(ctx, s, nullptr, warps, st, nullptr, nullptr, 0, g0, gn);
        }
    }
    switch (ctx->compensated) {
        case 1: return launch<CB, 1, false>(ctx, s, nullptr, warps, st, nullptr, nullptr, 0, g0, gn);
        case 2: return launch<CB, 2, false>(ctx, s, nullptr, warps, st, nullptr, nullptr, 0, g0, gn);
        default: return launch<CB, 0, false>(ctx, s, nullptr, warps, st, nullptr, nullptr, 0, g0, gn);
    }
}

}  // namespace

int walk2_init(Ctx *ctx) {
    const int smem_optin = ctx->smem_optin;
    int rc = 0;
    rc |= set_attr<64, 0, false>(ctx, smem_optin);
    rc |= set_attr<64, 1, false>(ctx, smem_optin);
    rc |= set_attr<64, 2, false>(ctx, smem_optin);
    rc |= set_attr<64, 0, true>(ctx, smem_optin);
    rc |= set_attr<128, 0, false>(ctx, smem_optin);
    rc |= set_attr<128, 1, false>(ctx, smem_optin);
    rc |= set_attr<128, 2, false>(ctx, smem_optin);
    rc |= set_attr<128, 0, true>(ctx, smem_optin);
    rc |= set_attr<96, 0, false>(ctx, smem_optin);
    rc |= set_attr<96, 1, false>(ctx, smem_optin);
    rc |= set_attr<96, 2, false>(ctx, smem_optin);
    rc |= set_attr<96, 0, true>(ctx, smem_optin);
    rc |= set_attr<96, 0, false, true>(ctx, smem_optin);
    rc |= set_attr<64, 0, false, false, true>(ctx, smem_optin);
    rc |= set_attr<64, 1, false, false, true>(ctx, smem_optin);
    rc |= set_attr<64, 2, false, false, true>(ctx, smem_optin);
    rc |= set_attr<128, 0, false, false, true>(ctx, smem_optin);
    rc |= set_attr<128, 1, false, false, true>(ctx, smem_optin);
    rc |= set_attr<128, 2, false, false, true>(ctx, smem_optin);
    rc |= set_attr<96, 0, false, false, true>(ctx, smem_optin);
    rc |= set_attr<96, 1, false, false, true>(ctx, smem_optin);
    rc |= set_attr<96, 2, false, false, true>(ctx, smem_optin);
    return rc;
}

// Plain walk that also records every group's interaction list (node ids, in
// evaluation order) into rec_list[g * rec_cap ...], its length into rec_len[g].
int walk2_record(Ctx *ctx, const nbx_state *s, int *rec_list, int *rec_len, int rec_cap, cudaStream_t st) {
    return launch<96, 0, false, true>(ctx, s, nullptr, ctx->walk_warps, st, rec_list, rec_len, rec_cap);
}

// The same walk without recording: the recording adds stores only, so both
// give the same forces bit for bit (the adjoint's forward and recompute).
int walk2_unrecorded(Ctx *ctx, const nbx_state *s, cudaStream_t st) {
    return launch<96, 0, false, false>(ctx, s, nullptr, ctx->walk_warps, st, nullptr, nullptr, 0);
}

// variant 0: 64-slot candidate buffers; 1: 128-slot buffers (<= 8 warps); 3: 96-slot buffers.
// Walk groups [g0, g0 + gn) of the last build (gn < 0: all groups from g0).
int walk2_forces(Ctx *ctx, const nbx_state *s, float *pot, int warps, cudaStream_t st, int g0, int gn) {
    if (ctx->walk_variant == 1) return forces_cb<128>(ctx, s, pot, warps > 8 ? 8 : warps, st, g0, gn);
    if (ctx->walk_variant == 3) return forces_cb<96>(ctx, s, pot, warps, st, g0, gn);
    return forces_cb<64>(ctx, s, pot, warps, st, g0, gn);
}

}  // namespace nbx
