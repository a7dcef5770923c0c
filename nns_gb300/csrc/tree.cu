// tree.cu -- bounding box, keys, key sort, key-built octree and FP64 moments.
//
// Replaces the reference's insertion build (3D/CUDA/CUDA_NBody/src/Kernels.cu:157-377),
// its bounding box (:67-154), centre of mass (:381-399) and sort (:403-456) with a
// sort-based construction that produces the same tree:
//
//  keys     each body replays the reference's float subdivision (:200-258) for 21
//           levels; the child codes c = [x<mid] + 2[y<mid] + 4[z<mid] packed most
//           significant first give a 63-bit key whose ascending order is the
//           reference's in-order body order.  Bodies sharing all 21 levels are
//           refined to 42 levels (k_refine).
//  delta    delta(i) = number of leading levels sorted neighbours i, i+1 share.
//           A cell (a region holding >= 2 bodies) at level L starts at sorted
//           position a iff delta(a-1) < L <= delta(a); the body at position i sits
//           at level max(delta(i-1), delta(i)) + 1.  Position i therefore owns the
//           node levels lo..hi = delta(i-1)+1 .. max(delta(i-1),delta(i))+1.
//  nodes    entries (level, position) generated in position order are the
//           depth-first pre-order; a stable sort by level gives breadth-first
//           order, in which the children of every cell are contiguous.
//  links    a node is the first child of its parent iff the parent starts at the
//           same position.  The k-th first child in BFS order belongs to the k-th
//           cell in BFS order (roots first), so two prefix counts give every cell's
//           child block and every node's parent -- no search, no locks.
//  moments  bottom-up FP64 sums in child order, deterministic: one BFS level
//           per launch, deepest first, or for small systems one launch in
//           which the last child to finish sums its parent.
#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kBlock = 256;
#ifndef NBX_MOMENTS_UP_MAX
#define NBX_MOMENTS_UP_MAX (1 << 21)
#endif
constexpr int kMomentsUpMaxBodies = NBX_MOMENTS_UP_MAX;  // one-launch moments up to this many bodies

__device__ __forceinline__ int grid_stride_start() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int grid_stride() { return gridDim.x * blockDim.x; }

__global__ void k_step_reset(unsigned *bbox_u, int nsys, DevStatus *st, int *sys_lvl) {
    int i = grid_stride_start();
    if (i < 6 * nsys) bbox_u[i] = f2ord(0.0f);  // Kernels.cu:56-62: the box contains the origin
    if (i < nsys) sys_lvl[i] = 0;
    if (i == 0) {
        st->refined_runs = 0;
        st->max_level = 0;
        st->interactions = 0ull;
        st->opened = 0ull;
        st->rounds = 0ull;
        st->candidates = 0ull;
    }
}

// Per-tile min/max of the bodies of one system, merged with ordered-int atomics.
__global__ void __launch_bounds__(kBlock) k_bbox(const float *__restrict__ x, const float *__restrict__ y,
                                                  const float *__restrict__ z, const int4 *__restrict__ tiles,
                                                  int ntiles, unsigned *bbox_u) {
    const int t = blockIdx.x;
    if (t >= ntiles) return;
    const int4 tl = tiles[t];
    float v[6] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY};
    for (int i = threadIdx.x; i < tl.y; i += kBlock) {
        float a = x[tl.x + i], b = y[tl.x + i], c = z[tl.x + i];
        v[0] = fminf(v[0], a); v[1] = fmaxf(v[1], a);
        v[2] = fminf(v[2], b); v[3] = fmaxf(v[3], b);
        v[4] = fminf(v[4], c); v[5] = fmaxf(v[5], c);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 6; k += 2) {
            v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
            v[k + 1] = fmaxf(v[k + 1], __shfl_xor_sync(0xffffffffu, v[k + 1], o));
        }
    }
    __shared__ float part[kBlock / 32][6];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 6; k++) part[w][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        float r = part[0][k];
        for (int q = 1; q < kBlock / 32; q++) r = (k & 1) ? fmaxf(r, part[q][k]) : fminf(r, part[q][k]);
        if (!isnan(r) && !isinf(r)) {
            unsigned *dst = &bbox_u[6 * tl.z + k];
            if (k & 1) atomicMax(dst, f2ord(r));
            else atomicMin(dst, f2ord(r));
        }
    }
}

__device__ __forceinline__ float depth0_of(float mnx, float mxx, float theta_ref) {
    float r = __fmul_rn(__fsub_rn(mxx, mnx), 0.5f);  // Kernels.cu:477
    return __fdiv_rn(__fmul_rn(r, r), theta_ref);    // Kernels.cu:513
}

__global__ void k_bbox_finalize(const unsigned *bbox_u, int nsys, float theta_ref, float *bbox,
                                double *bbox64, float *depth0) {
    int s = grid_stride_start();
    if (s >= nsys) return;
    float b[6];
    for (int k = 0; k < 6; k++) {
        b[k] = __fadd_rn(ord2f(bbox_u[6 * s + k]), 0.0f);  // -0 -> +0
        bbox[6 * s + k] = b[k];
        bbox64[6 * s + k] = (double)b[k];
    }
    depth0[s] = depth0_of(b[0], b[1], theta_ref);
}

// Single-system box supplied by the caller (reference-compatible entry points).
__global__ void k_bbox_from_ptrs(const float *mnx, const float *mxx, const float *mny,
                                 const float *mxy, const float *mnz, const float *mxz,
                                 float theta_ref, float *bbox, double *bbox64, float *depth0,
                                 DevStatus *st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float b[6] = {*mnx, *mxx, *mny, *mxy, *mnz, *mxz};
    for (int k = 0; k < 6; k++) { bbox[k] = b[k]; bbox64[k] = (double)b[k]; }
    depth0[0] = depth0_of(b[0], b[1], theta_ref);
    st->refined_runs = 0;
    st->max_level = 0;
}

// Optional Hilbert order (key_order = 1).  The 12-state Lebesgue-to-Hilbert
// tables of the reference's domain-decomposition code
// (MolecularDynamics/BarnesHutParallel/SpaceFillingCurves/src/Tree.cpp:70-104),
// indexed by the Lebesgue child number b = [x>=mid] + 2[y>=mid] + 4[z>=mid]
// = 7 - c.  Digits map one-to-one per level, so two keys share a Hilbert prefix
// exactly when they share the Lebesgue one: the same cells, siblings reordered.
__constant__ unsigned char kHilbertDigit[12][8] = {
    {0, 7, 3, 4, 1, 6, 2, 5}, {4, 3, 7, 0, 5, 2, 6, 1}, {6, 1, 5, 2, 7, 0, 4, 3}, {2, 5, 1, 6, 3, 4, 0, 7},
    {0, 1, 7, 6, 3, 2, 4, 5}, {6, 7, 1, 0, 5, 4, 2, 3}, {2, 3, 5, 4, 1, 0, 6, 7}, {4, 5, 3, 2, 7, 6, 0, 1},
    {0, 3, 1, 2, 7, 4, 6, 5}, {2, 1, 3, 0, 5, 6, 4, 7}, {4, 7, 5, 6, 3, 0, 2, 1}, {6, 5, 7, 4, 1, 2, 0, 3}};
__constant__ unsigned char kHilbertState[12][8] = {
    {8, 10, 3, 3, 4, 5, 4, 5}, {2, 2, 11, 9, 4, 5, 4, 5}, {7, 6, 7, 6, 8, 10, 1, 1}, {7, 6, 7, 6, 0, 0, 11, 9},
    {0, 8, 1, 11, 6, 8, 6, 11}, {10, 0, 9, 1, 10, 7, 9, 7}, {10, 4, 9, 4, 10, 2, 9, 3}, {5, 8, 5, 11, 2, 8, 3, 11},
    {4, 9, 0, 0, 7, 9, 2, 2}, {1, 1, 8, 5, 3, 3, 8, 6}, {11, 5, 0, 0, 11, 6, 2, 2}, {1, 1, 4, 10, 3, 3, 7, 10}};

// The lanes of a warp index the tables by their own states, which the constant
// cache would serialise: each block copies them to shared memory, one byte per
// (state, child) holding digit | next state << 3.
__device__ __forceinline__ void load_hilbert(unsigned char *t, int order) {
    if (order == 0) return;  // uniform over the launch
    for (int i = threadIdx.x; i < 96; i += blockDim.x)
        t[i] = (unsigned char)(kHilbertDigit[i >> 3][i & 7] | (kHilbertState[i >> 3][i & 7] << 3));
    __syncthreads();
}

__device__ __forceinline__ int to_digit(int c, int &state, int order, const unsigned char *t) {
    if (order == 0) return c;
    const int e = t[(state << 3) + 7 - c];
    state = e >> 3;
    return e & 7;
}

__device__ __forceinline__ unsigned long long make_key(float px, float py, float pz, const float *bb, int order,
                                                       const unsigned char *t) {
    float mnx = bb[0], mxx = bb[1], mny = bb[2], mxy = bb[3], mnz = bb[4], mxz = bb[5];
    unsigned long long key = 0ull;
    int state = 0;
#pragma unroll 3
    for (int l = 1; l <= 21; l++) {
        int c = split_axis(px, mnx, mxx) + 2 * split_axis(py, mny, mxy) + 4 * split_axis(pz, mnz, mxz);
        key = (key << 3) | (unsigned long long)to_digit(c, state, order, t);
    }
    return key;
}

// Also packs the bodies as float4 (x, y, z, m) in their original order, so that
// the gather into sorted order reads one 16-byte record per body.
__global__ void __launch_bounds__(kBlock) k_keys(const float *__restrict__ x, const float *__restrict__ y,
                                                  const float *__restrict__ z, const float *__restrict__ m,
                                                  const int *__restrict__ body_sys,
                                                  const float *__restrict__ bbox, int n,
                                                  unsigned long long *__restrict__ key, int *__restrict__ val,
                                                  float4 *__restrict__ pos4, DevStatus *st, int order) {
    __shared__ unsigned char ht[96];
    load_hilbert(ht, order);
    for (int i = grid_stride_start(); i < n; i += grid_stride()) {
        const float px = x[i], py = y[i], pz = z[i];
        pos4[i] = make_float4(px, py, pz, m[i]);
        if (!isfinite(px) || !isfinite(py) || !isfinite(pz)) set_status(st, NBX_ERR_NONFINITE, i);
        const int s = body_sys[i];
        float bb[6];
#pragma unroll
        for (int k = 0; k < 6; k++) bb[k] = bbox[6 * s + k];
        key[i] = make_key(px, py, pz, bb, order, ht);
        val[i] = i;
    }
}

// Runs of equal 21-level keys: compute levels 22..42 and order the run by them.
__global__ void k_refine(const float *__restrict__ x, const float *__restrict__ y,
                         const float *__restrict__ z, const int *__restrict__ body_sys,
                         const int *__restrict__ sys_off, const float *__restrict__ bbox, int n,
                         const unsigned long long *__restrict__ key,
                         unsigned long long *__restrict__ key_lo, int *__restrict__ val,
                         DevStatus *st, int order) {
    __shared__ unsigned char ht[96];
    load_hilbert(ht, order);
    for (int p = grid_stride_start(); p < n; p += grid_stride()) {
        const int s = body_sys[p];
        const int beg = sys_off[s], end = sys_off[s + 1];
        const unsigned long long k = key[p];
        if (p + 1 >= end || key[p + 1] != k) continue;
        if (p > beg && key[p - 1] == k) continue;
        int e = p + 1;
        while (e + 1 < end && key[e + 1] == k) e++;
        if (e - p + 1 > kMaxRun) {
            set_status(st, NBX_ERR_CLUSTER, p);
            continue;
        }
        atomicAdd(&st->refined_runs, 1);
        float bb[6];
        for (int q = 0; q < 6; q++) bb[q] = bbox[6 * s + q];
        for (int q = p; q <= e; q++) {
            const int b = val[q];
            float mnx = bb[0], mxx = bb[1], mny = bb[2], mxy = bb[3], mnz = bb[4], mxz = bb[5];
            unsigned long long lo = 0ull;
            const float px = x[b], py = y[b], pz = z[b];
            int state = 0;
            for (int l = 1; l <= 42; l++) {
                int c = split_axis(px, mnx, mxx) + 2 * split_axis(py, mny, mxy) + 4 * split_axis(pz, mnz, mxz);
                const int d = to_digit(c, state, order, ht);
                if (l > 21) lo = (lo << 3) | (unsigned long long)d;
            }
            key_lo[q] = lo;
        }
        // stable insertion sort of the run by key_lo (runs are short)
        for (int q = p + 1; q <= e; q++) {
            unsigned long long kl = key_lo[q];
            int v = val[q];
            int r = q - 1;
            while (r >= p && key_lo[r] > kl) {
                key_lo[r + 1] = key_lo[r];
                val[r + 1] = val[r];
                r--;
            }
            key_lo[r + 1] = kl;
            val[r + 1] = v;
        }
        for (int q = p; q < e; q++)
            if (key_lo[q] == key_lo[q + 1]) set_status(st, NBX_ERR_DEPTH, val[q]);
    }
}

__device__ __forceinline__ int delta_of(const unsigned long long *key, const unsigned long long *key_lo,
                                        int a) {
    const unsigned long long ka = key[a], kb = key[a + 1];
    if (ka != kb) return common_digits(ka, kb);
    int d = 21 + common_digits(key_lo[a], key_lo[a + 1]);
    return d > 41 ? 41 : d;  // equal 42-level keys were reported as NBX_ERR_DEPTH
}

// Sorted bodies as float4 plus delta and the number of node entries per position.
__global__ void __launch_bounds__(kBlock) k_delta(const float4 *__restrict__ pos4,
                                                   const int *__restrict__ body_sys, const int *__restrict__ sys_off,
                                                   int n, const unsigned long long *__restrict__ key,
                                                   const unsigned long long *__restrict__ key_lo,
                                                   const int *__restrict__ val, float4 *__restrict__ body4,
                                                   unsigned char *__restrict__ delta,
                                                   unsigned *__restrict__ ecount, DevStatus *st,
                                                   int *__restrict__ sys_lvl) {
    int lvl_max = 0;
    for (int p = grid_stride_start(); p < n; p += grid_stride()) {
        const int s = body_sys[p];
        const int beg = sys_off[s], end = sys_off[s + 1];
        const int di = p + 1 < end ? delta_of(key, key_lo, p) : 0;
        const int dp = p > beg ? delta_of(key, key_lo, p - 1) : 0;
        delta[p] = (unsigned char)di;
        ecount[p] = (unsigned)((di > dp ? di - dp : 0) + 1);
        body4[p] = pos4[val[p]];
        const int lv = max(di, dp) + 1;
        lvl_max = max(lvl_max, lv);
        // each system's deepest level (the walk's depth-first reserve of its
        // groups); the L2 read skips the atomic for all but the few new maxima
        if (lv > __ldcg(&sys_lvl[s])) atomicMax(&sys_lvl[s], lv);
    }
    lvl_max = __reduce_max_sync(0xffffffffu, lvl_max);
    if ((threadIdx.x & 31) == 0 && lvl_max > 0) atomicMax(&st->max_level, lvl_max);
}

// Node levels owned by sorted position p: the cells starting at p (levels
// lo..hi-1) and the body (level hi).  With leaf buckets (bucket != nullptr) the
// body hangs directly below its bucket cell (level bucket[p]): deeper cells
// are dropped and the body's level is at most bucket[p] + 1.
__device__ __forceinline__ void levels_of(const unsigned char *delta, const unsigned char *bucket, int p, int beg,
                                          int &lo, int &hi, int &dp) {
    dp = p > beg ? (int)delta[p - 1] : 0;
    const int di = delta[p];
    lo = dp + 1;
    hi = max(dp, di) + 1;
    if (bucket) {
        hi = min(hi, (int)bucket[p] + 1);
        lo = min(lo, hi);
    }
}

// Leaf buckets (nbx_params.leaf_size k > 1; not the reference's tree, which has
// one body per leaf): the bucket of a body is the shallowest cell around it
// holding at most k bodies.  The cell at level L around p holds more than k
// bodies exactly when some window of k+1 consecutive positions of the system
// containing p shares at least L levels, i.e. all k deltas inside the window
// are >= L; so the bucket level is 1 + the largest inner-delta minimum over
// those windows.  Rewrites the node entries per position accordingly.
__global__ void __launch_bounds__(kBlock) k_bucket(const int *__restrict__ body_sys, const int *__restrict__ sys_off,
                                                    int n, int k, const unsigned char *__restrict__ delta,
                                                    unsigned char *__restrict__ bucket, unsigned *__restrict__ ecount) {
    for (int p = grid_stride_start(); p < n; p += grid_stride()) {
        const int s = body_sys[p];
        const int beg = sys_off[s], end = sys_off[s + 1];
        int best = 0;
        for (int a = max(p - k, beg); a <= p && a + k <= end - 1; a++) {
            int mn = 255;
            for (int j = a; j < a + k; j++) mn = min(mn, (int)delta[j]);
            best = max(best, mn);
        }
        bucket[p] = (unsigned char)(best + 1);
        int lo, hi, dp;
        levels_of(delta, bucket, p, beg, lo, hi, dp);
        ecount[p] = (unsigned)(hi - lo + 1);
    }
}

// Node entries (level << 26 | position) in position order = depth-first pre-order.
__global__ void __launch_bounds__(kBlock) k_entries(const int *__restrict__ body_sys,
                                                     const int *__restrict__ sys_off, int n,
                                                     const unsigned char *__restrict__ delta,
                                                     const unsigned char *__restrict__ bucket,
                                                     const unsigned *__restrict__ eoff, unsigned *totals,
                                                     int cap_nodes, unsigned *__restrict__ ent,
                                                     DevStatus *st) {
    if (grid_stride_start() == 0) {
        unsigned T = totals[0];
        if (T > (unsigned)cap_nodes) {
            set_status(st, NBX_ERR_CAPACITY, (int)min(T, 0x7fffffffu));
            T = 0u;  // nothing downstream reads a partial entry list
        }
        totals[1] = T;  // node count used downstream
    }
    for (int p = grid_stride_start(); p < n; p += grid_stride()) {
        const int beg = sys_off[body_sys[p]];
        int lo, hi, dp;
        levels_of(delta, bucket, p, beg, lo, hi, dp);
        const unsigned e = eoff[p];
        if (e + (unsigned)(hi - lo + 1) > (unsigned)cap_nodes) continue;
        for (int l = lo; l <= hi; l++) ent[e + (l - lo)] = ((unsigned)l << kLevelShift) | (unsigned)p;
    }
}

__device__ __forceinline__ void node_kind(unsigned u, const int *body_sys, const int *sys_off,
                                          const unsigned char *delta, const unsigned char *bucket, int &p, int &l,
                                          bool &is_cell, bool &first) {
    l = (int)(u >> kLevelShift);
    p = (int)(u & ((1u << kLevelShift) - 1u));
    const int beg = sys_off[body_sys[p]];
    int lo, hi, dp;
    levels_of(delta, bucket, p, beg, lo, hi, dp);
    is_cell = l < hi;
    first = (l == 1) ? (p == beg) : (dp < l - 1);
}

__global__ void __launch_bounds__(kBlock) k_node_flags(const unsigned *__restrict__ ent_bfs,
                                                        const unsigned *__restrict__ totals,
                                                        const int *__restrict__ body_sys,
                                                        const int *__restrict__ sys_off,
                                                        const unsigned char *__restrict__ delta,
                                                     const unsigned char *__restrict__ bucket,
                                                        unsigned long long *__restrict__ flags) {
    const int T = (int)totals[1];
    for (int b = grid_stride_start(); b < T; b += grid_stride()) {
        int p, l;
        bool c, f;
        node_kind(ent_bfs[b], body_sys, sys_off, delta, bucket, p, l, c, f);
        flags[b] = ((unsigned long long)c << 32) | (unsigned long long)f;
    }
}

__global__ void __launch_bounds__(kBlock) k_nodes_a(const unsigned *__restrict__ ent_bfs,
                                                     const unsigned *__restrict__ totals,
                                                     const unsigned long long *__restrict__ totals64,
                                                     const int *__restrict__ body_sys,
                                                     const int *__restrict__ sys_off,
                                                     const unsigned char *__restrict__ delta,
                                                     const unsigned char *__restrict__ bucket,
                                                     const unsigned long long *__restrict__ flags_ex,
                                                     const float4 *__restrict__ body4, int nsys,
                                                     int *__restrict__ fcl, int *__restrict__ cl,
                                                     float4 *__restrict__ node4, int *__restrict__ meta,
                                                     int *__restrict__ body_node, int *__restrict__ count,
                                                     int *__restrict__ arrive, unsigned char *__restrict__ lvl8,
                                                     DevStatus *st) {
    const int T = (int)totals[1];
    if (grid_stride_start() == 0) {
        const unsigned long long tot = totals64[0];
        const int ncell = (int)(tot >> 32), nfirst = (int)(tot & 0xffffffffull);
        if (nfirst != nsys + ncell && st->code == 0) set_status(st, NBX_ERR_STATE, nfirst);
        fcl[nsys + ncell] = T;
    }
    for (int b = grid_stride_start(); b < T; b += grid_stride()) {
        int p, l;
        bool c, f;
        node_kind(ent_bfs[b], body_sys, sys_off, delta, bucket, p, l, c, f);
        const unsigned long long ex = flags_ex[b];
        if (f) fcl[(int)(ex & 0xffffffffull)] = b;
        arrive[b] = 0;
        lvl8[b] = (unsigned char)l;
        if (c) {
            cl[nsys + (int)(ex >> 32)] = b;
        } else {
            node4[b] = body4[p];
            meta[b] = kBodyFlag | p;
            body_node[p] = b;
            count[b] = 1;
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_nodes_b(const unsigned *__restrict__ ent_bfs,
                                                     const unsigned *__restrict__ totals,
                                                     const int *__restrict__ body_sys,
                                                     const int *__restrict__ sys_off,
                                                     const unsigned char *__restrict__ delta,
                                                     const unsigned char *__restrict__ bucket,
                                                     const unsigned long long *__restrict__ flags_ex,
                                                     int nsys, const int *__restrict__ fcl,
                                                     const int *__restrict__ cl, int *__restrict__ meta,
                                                     int *__restrict__ parent, int *__restrict__ root_first,
                                                     int *__restrict__ root_nch, DevStatus *st) {
    const int T = (int)totals[1];
    for (int s = grid_stride_start(); s < nsys; s += grid_stride()) {
        const bool ok = st->code == 0;  // a failed build leaves empty roots
        root_first[s] = ok ? fcl[s] : 0;
        root_nch[s] = ok ? fcl[s + 1] - fcl[s] : 0;
    }
    for (int b = grid_stride_start(); b < T; b += grid_stride()) {
        int p, l;
        bool c, f;
        node_kind(ent_bfs[b], body_sys, sys_off, delta, bucket, p, l, c, f);
        const unsigned long long ex = flags_ex[b];
        const int fcx = (int)(ex & 0xffffffffull);
        if (c) {
            const int k = nsys + (int)(ex >> 32);
            const int first = fcl[k];
            const int nch = fcl[k + 1] - first;
            if (nch < 1 || nch > 8) {
                set_status(st, NBX_ERR_STATE, b);
                meta[b] = first;  // keeps the walk in bounds
            } else {
                meta[b] = first | ((nch - 1) << 28);
            }
        }
        const int j = fcx + (f ? 1 : 0) - 1;
        parent[b] = j < nsys ? (-1 - j) : cl[j];
    }
}

// Quadrupole mode: the FP64 second moments of a cell about its centre of mass c,
// composed from its children in child order -- M2 = sum over children of
// [M2_child + m_child d d^T], d = c_child - c (a body child: M2 = 0, c_child =
// its position) -- and the cell's traceless quadrupole Q = 3 M2 - tr(M2) I,
// stored negated in FP32 as P = -Q = tr(M2) I - 3 M2 (the walk's form of the
// term; the FP64 differences are negated before rounding, so P is exactly -Q).
// Every FP64 operation is rounded explicitly (no contraction), in the order of
// the oracle's restatement, so both give the same bits.
__device__ __forceinline__ void m2_add_point(double *a, double mc, double dx, double dy, double dz) {
    a[0] = __dadd_rn(a[0], __dmul_rn(__dmul_rn(mc, dx), dx));
    a[1] = __dadd_rn(a[1], __dmul_rn(__dmul_rn(mc, dy), dy));
    a[2] = __dadd_rn(a[2], __dmul_rn(__dmul_rn(mc, dz), dz));
    a[3] = __dadd_rn(a[3], __dmul_rn(__dmul_rn(mc, dx), dy));
    a[4] = __dadd_rn(a[4], __dmul_rn(__dmul_rn(mc, dx), dz));
    a[5] = __dadd_rn(a[5], __dmul_rn(__dmul_rn(mc, dy), dz));
}

// b: the cell; its children [first, first + nch); (cx, cy, cz) its FP64 centre of mass
__device__ __forceinline__ void quad_cell(int b, int first, int nch, double cx, double cy, double cz,
                                          const int *__restrict__ meta, const float4 *node4, const double4 *sums,
                                          double2 *m2, float4 *quad4, float2 *quad2) {
    double a[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int c = first; c < first + nch; c++) {
        double mc, dx, dy, dz;
        if (meta[c] < 0) {
            const float4 q = node4[c];
            mc = (double)q.w;
            dx = __dsub_rn((double)q.x, cx);
            dy = __dsub_rn((double)q.y, cy);
            dz = __dsub_rn((double)q.z, cz);
        } else {
            const double2 *vp = reinterpret_cast<const double2 *>(&sums[c]);
            const double2 v0 = __ldcg(vp), v1 = __ldcg(vp + 1);
            mc = v0.x;
            dx = __dsub_rn(__ddiv_rn(v0.y, mc), cx);
            dy = __dsub_rn(__ddiv_rn(v1.x, mc), cy);
            dz = __dsub_rn(__ddiv_rn(v1.y, mc), cz);
            const double2 w0 = __ldcg(&m2[3 * (size_t)c]), w1 = __ldcg(&m2[3 * (size_t)c + 1]),
                          w2 = __ldcg(&m2[3 * (size_t)c + 2]);
            a[0] = __dadd_rn(a[0], w0.x);
            a[1] = __dadd_rn(a[1], w0.y);
            a[2] = __dadd_rn(a[2], w1.x);
            a[3] = __dadd_rn(a[3], w1.y);
            a[4] = __dadd_rn(a[4], w2.x);
            a[5] = __dadd_rn(a[5], w2.y);
        }
        m2_add_point(a, mc, dx, dy, dz);
    }
    m2[3 * (size_t)b] = make_double2(a[0], a[1]);
    m2[3 * (size_t)b + 1] = make_double2(a[2], a[3]);
    m2[3 * (size_t)b + 2] = make_double2(a[4], a[5]);
    const double tr = __dadd_rn(__dadd_rn(a[0], a[1]), a[2]);
    quad4[b] = make_float4((float)__dsub_rn(tr, __dmul_rn(3.0, a[0])), (float)__dsub_rn(tr, __dmul_rn(3.0, a[1])),
                           (float)__dsub_rn(tr, __dmul_rn(3.0, a[2])), (float)__dmul_rn(-3.0, a[3]));
    quad2[b] = make_float2((float)__dmul_rn(-3.0, a[4]), (float)__dmul_rn(-3.0, a[5]));
}

// Bottom-up FP64 moments, one BFS level per launch (deepest first): a cell sums
// its children -- contiguous, one level below, already final -- in child order,
// so the result is deterministic.  Level L occupies BFS indices
// [start(L), start(L+1)); start(L) is the scanned count of level-sort digit 4L.
template <bool Quad>
__global__ void __launch_bounds__(kBlock) k_moments_level(int level, const unsigned *__restrict__ lvl_off,
                                                           int ntiles, const unsigned *__restrict__ totals,
                                                           const unsigned long long *__restrict__ totals64,
                                                           const unsigned long long *__restrict__ flags_ex,
                                                           const int *__restrict__ cl, int nsys,
                                                           const int *__restrict__ meta, float4 *node4,
                                                           double4 *sums, int *count, double2 *m2, float4 *quad4,
                                                           float2 *quad2, const DevStatus *st) {
    if (st->code != 0) return;  // an inconsistent tree is never summed
    const unsigned T = totals[1];
    unsigned beg = lvl_off[(size_t)(level << 2) * ntiles];
    unsigned end = lvl_off[(size_t)((level + 1) << 2) * ntiles];
    if (end > T) end = T;
    if (beg > end) beg = end;
    // the level's cells are a contiguous range of the BFS-ordered cell list:
    // their ranks are the scanned cell flags at the level's first and end nodes
    const unsigned ncell = (unsigned)(totals64[0] >> 32);
    const unsigned cbeg = beg < T ? (unsigned)(flags_ex[beg] >> 32) : ncell;
    const unsigned cend = end < T ? (unsigned)(flags_ex[end] >> 32) : ncell;
    for (unsigned k = cbeg + grid_stride_start(); k < cend; k += grid_stride()) {
        const int b = cl[nsys + k];
        const int pm = meta[b];
        if (pm < 0) continue;  // never: the list holds cells only
        const int first = pm & 0x0fffffff;
        const int nch = ((pm >> 28) & 7) + 1;
        double sm = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
        int cnt = 0;
        for (int c = first; c < first + nch; c++) {
            if (meta[c] < 0) {
                const float4 q = node4[c];
                const double mb = (double)q.w;
                sm += mb;
                sx += mb * (double)q.x;
                sy += mb * (double)q.y;
                sz += mb * (double)q.z;
                cnt += 1;
            } else {
                const double4 v = sums[c];
                sm += v.x;
                sx += v.y;
                sy += v.z;
                sz += v.w;
                cnt += count[c];
            }
        }
        sums[b] = make_double4(sm, sx, sy, sz);
        count[b] = cnt;
        node4[b] = make_float4((float)(sx / sm), (float)(sy / sm), (float)(sz / sm), (float)sm);
        if (Quad) quad_cell(b, first, nch, sx / sm, sy / sm, sz / sm, meta, node4, sums, m2, quad4, quad2);
    }
}

// Bottom-up FP64 moments in one launch, one thread per cell in BFS order.
// Every child arrives once at its cell's counter: the cell's own thread adds
// the number of its body children in one step, and each child cell arrives
// when it is complete.  The arrival that brings the count to the cell's number
// of children sums the cell (children in child order: the same additions as
// k_moments_level) and climbs on to the parent.  Nothing waits: a thread whose
// arrival is not the last stops.  A cell's arrival is acquire-release: it
// publishes the thread's sums and, when last, orders the reads of the
// siblings' sums (through L2) after their arrivals.  Counters are zeroed by
// k_nodes_a.
__device__ __forceinline__ int arrive_acq_rel(int *p) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// A cell's sums from its children in child order.  Every child's body record
// and cell sums are loaded at once and the child's kind picks one (a body's
// sums entry is never read for its value), so the loads take one round trip.
template <bool Quad>
__device__ __forceinline__ void sum_cell(int b, int first, int nch, const int *__restrict__ meta, float4 *node4,
                                         double4 *sums, int *count, double2 *m2, float4 *quad4, float2 *quad2) {
    int mk[8], ck[8];
    float4 q[8];
    double2 v0[8], v1[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        if (j < nch) {
            const int c = first + j;
            mk[j] = meta[c];
            q[j] = node4[c];
            const double2 *v = reinterpret_cast<const double2 *>(&sums[c]);
            v0[j] = __ldcg(v);
            v1[j] = __ldcg(v + 1);
            ck[j] = __ldcg(&count[c]);
        }
    }
    double sm = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        if (j < nch) {
            if (mk[j] < 0) {
                const double mb = (double)q[j].w;
                sm += mb;
                sx += mb * (double)q[j].x;
                sy += mb * (double)q[j].y;
                sz += mb * (double)q[j].z;
                cnt += 1;
            } else {
                sm += v0[j].x;
                sx += v0[j].y;
                sy += v1[j].x;
                sz += v1[j].y;
                cnt += ck[j];
            }
        }
    }
    sums[b] = make_double4(sm, sx, sy, sz);
    count[b] = cnt;
    node4[b] = make_float4((float)(sx / sm), (float)(sy / sm), (float)(sz / sm), (float)sm);
    if (Quad) quad_cell(b, first, nch, sx / sm, sy / sm, sz / sm, meta, node4, sums, m2, quad4, quad2);
}

template <bool Quad>
__global__ void __launch_bounds__(kBlock) k_moments_up(const unsigned long long *__restrict__ totals64,
                                                       const int *__restrict__ cl, int nsys,
                                                       const int *__restrict__ parent,
                                                       const int *__restrict__ meta, float4 *node4,
                                                       double4 *sums, int *count, int *counter, double2 *m2,
                                                       float4 *quad4, float2 *quad2, const DevStatus *st) {
    if (st->code != 0) return;  // an inconsistent tree is never summed
    const int ncell = (int)(totals64[0] >> 32);
    for (int k = grid_stride_start(); k < ncell; k += grid_stride()) {
        int b = cl[nsys + k];
        int pm = meta[b];
        int first = pm & 0x0fffffff, nch = ((pm >> 28) & 7) + 1;
        int nbody = 0;
        for (int c = first; c < first + nch; c++) nbody += meta[c] < 0;
        if (nbody == 0) continue;  // completed by the arrival of its last child cell
        if (nbody < nch) {  // cell children too: the bodies arrive together (relaxed: nothing to publish)
            if (atomicAdd(&counter[b], nbody) + nbody != nch) continue;
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
        }
        for (;;) {
            // the parent and its meta load while the sums do
            const int up = parent[b];
            sum_cell<Quad>(b, first, nch, meta, node4, sums, count, m2, quad4, quad2);
            if (up < 0) break;
            pm = meta[up];
            if (arrive_acq_rel(&counter[up]) != ((pm >> 28) & 7)) break;  // last of its children?
            b = up;
            first = pm & 0x0fffffff;
            nch = ((pm >> 28) & 7) + 1;
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
int build_tree(Ctx *ctx, const nbx_state *s, cudaStream_t st, bool external_bbox,
               const float *const *bbox_ptrs) {
    const int n = (int)ctx->nbodies;
    const int S = ctx->nsys;
    if (n <= 0 || S <= 0) return NBX_ERR_STATE;
    const int gb = ceil_div(n, kBlock) < ctx->nsm * 8 ? ceil_div(n, kBlock) : ctx->nsm * 8;
    k_step_reset<<<ceil_div(6 * S + 1, kBlock), kBlock, 0, st>>>(ctx->d_bbox_u, S, ctx->d_status, ctx->d_sys_lvl);
    ++ctx->launches;
    if (!external_bbox) {
        k_bbox<<<ctx->ntiles_body, kBlock, 0, st>>>(s->x, s->y, s->z, ctx->d_tiles, ctx->ntiles_body,
                                                    ctx->d_bbox_u);
        ++ctx->launches;
        k_bbox_finalize<<<ceil_div(S, kBlock), kBlock, 0, st>>>(ctx->d_bbox_u, S, ctx->theta_ref,
                                                                ctx->d_bbox, ctx->d_bbox64, ctx->d_depth0);
        ++ctx->launches;
    } else {
        k_bbox_from_ptrs<<<1, 32, 0, st>>>(bbox_ptrs[0], bbox_ptrs[1], bbox_ptrs[2], bbox_ptrs[3],
                                           bbox_ptrs[4], bbox_ptrs[5], ctx->theta_ref, ctx->d_bbox,
                                           ctx->d_bbox64, ctx->d_depth0, ctx->d_status);
        ++ctx->launches;
    }
    // the node array is free until the nodes are written: it holds the packed bodies
    float4 *pos4 = ctx->d_node4;
    // the sort's last pass writes d_key / d_val: an odd pass count starts from the alternates
    const bool alt = radix_passes(ctx->radix_bits) & 1;
    k_keys<<<gb, kBlock, 0, st>>>(s->x, s->y, s->z, s->m, ctx->d_body_sys, ctx->d_bbox, n,
                                  alt ? ctx->d_key_alt : ctx->d_key, alt ? ctx->d_val_alt : ctx->d_val, pos4,
                                  ctx->d_status, ctx->key_order);
    ++ctx->launches;
    int rc = radix_sort_bodies(ctx, st);
    if (rc) return rc;
    k_refine<<<gb, kBlock, 0, st>>>(s->x, s->y, s->z, ctx->d_body_sys, ctx->d_sys_off, ctx->d_bbox, n,
                                    ctx->d_key, ctx->d_key_lo, ctx->d_val, ctx->d_status, ctx->key_order);
    ++ctx->launches;
    k_delta<<<gb, kBlock, 0, st>>>(pos4, ctx->d_body_sys, ctx->d_sys_off, n, ctx->d_key,
                                   ctx->d_key_lo, ctx->d_val, ctx->d_body4, ctx->d_delta, ctx->d_ecount,
                                   ctx->d_status, ctx->d_sys_lvl);
    ++ctx->launches;
    const unsigned char *bucket = ctx->leaf_size > 1 ? ctx->d_bucket : nullptr;
    if (bucket) {
        k_bucket<<<gb, kBlock, 0, st>>>(ctx->d_body_sys, ctx->d_sys_off, n, ctx->leaf_size, ctx->d_delta,
                                        ctx->d_bucket, ctx->d_ecount);
        ++ctx->launches;
    }
    rc = scan_exclusive_u32(ctx, ctx->d_ecount, ctx->d_ecount, n, nullptr, &ctx->d_totals[0], st);
    if (rc) return rc;
    k_entries<<<gb, kBlock, 0, st>>>(ctx->d_body_sys, ctx->d_sys_off, n, ctx->d_delta, bucket, ctx->d_ecount,
                                     ctx->d_totals, ctx->cap_nodes, ctx->d_ent, ctx->d_status);
    ++ctx->launches;
    rc = radix_sort_entries(ctx, st);  // d_ent -> d_ent_alt (BFS order)
    if (rc) return rc;
    const int gn = ceil_div(ctx->cap_nodes, kBlock) < ctx->nsm * 8 ? ceil_div(ctx->cap_nodes, kBlock) : ctx->nsm * 8;
    k_node_flags<<<gn, kBlock, 0, st>>>(ctx->d_ent_alt, ctx->d_totals, ctx->d_body_sys, ctx->d_sys_off,
                                        ctx->d_delta, bucket, ctx->d_flags);
    ++ctx->launches;
    rc = scan_exclusive_u64(ctx, ctx->d_flags, ctx->d_flags, ctx->cap_nodes, &ctx->d_totals[1],
                            &ctx->d_totals64[0], st);
    if (rc) return rc;
    k_nodes_a<<<gn, kBlock, 0, st>>>(ctx->d_ent_alt, ctx->d_totals, ctx->d_totals64, ctx->d_body_sys,
                                     ctx->d_sys_off, ctx->d_delta, bucket, ctx->d_flags, ctx->d_body4, S, ctx->d_fcl,
                                     ctx->d_cl, ctx->d_node4, ctx->d_meta, ctx->d_body_node, ctx->d_count,
                                     ctx->d_arrive, ctx->d_lvl8, ctx->d_status);
    ++ctx->launches;
    k_nodes_b<<<gn, kBlock, 0, st>>>(ctx->d_ent_alt, ctx->d_totals, ctx->d_body_sys, ctx->d_sys_off,
                                     ctx->d_delta, bucket, ctx->d_flags, S, ctx->d_fcl, ctx->d_cl, ctx->d_meta,
                                     ctx->d_parent, ctx->d_root_first, ctx->d_root_nch, ctx->d_status);
    ++ctx->launches;
    // up to 2^21 bodies the 41 per-level launches cost more than the sums: one
    // bottom-up launch (2^16: 0.37 against 0.55 ms per build); above, the
    // per-level launches stream the levels and are faster
    const int mode = ctx->p.moments_mode;
    const bool quad = ctx->multipole != 0;
    if (quad && !ctx->d_m2) return NBX_ERR_STATE;
    if (mode == 2 || (mode == 0 && n <= kMomentsUpMaxBodies)) {
        auto kern = quad ? k_moments_up<true> : k_moments_up<false>;
        kern<<<gn, kBlock, 0, st>>>(ctx->d_totals64, ctx->d_cl, S, ctx->d_parent, ctx->d_meta, ctx->d_node4,
                                    ctx->d_sums, ctx->d_count, ctx->d_arrive, ctx->d_m2, ctx->d_quad4, ctx->d_quad2,
                                    ctx->d_status);
        ++ctx->launches;
    } else {
        // cells exist at levels 1..41 (two bodies share at most 41 levels without error)
        auto kern = quad ? k_moments_level<true> : k_moments_level<false>;
        for (int level = kMaxLevel - 2; level >= 1; level--) {
            kern<<<ctx->nsm * 4, kBlock, 0, st>>>(level, ctx->d_hist, ctx->cap_tiles_node, ctx->d_totals,
                                                  ctx->d_totals64, ctx->d_flags, ctx->d_cl, S, ctx->d_meta,
                                                  ctx->d_node4, ctx->d_sums, ctx->d_count, ctx->d_m2, ctx->d_quad4,
                                                  ctx->d_quad2, ctx->d_status);
            ++ctx->launches;
        }
    }
    NBX_CUDA(cudaGetLastError());
    ctx->built = true;
    return NBX_OK;
}

// ---------------------------------------------------------------------------
// Export of one system's tree in the reference's array format.
namespace {

__global__ void __launch_bounds__(kBlock) k_export(const unsigned *__restrict__ ent_bfs,
                                                    const unsigned *__restrict__ totals,
                                                    const int *__restrict__ body_sys,
                                                    const int *__restrict__ sys_off,
                                                    const unsigned char *__restrict__ delta,
                                                    const unsigned *__restrict__ eoff,
                                                    const unsigned long long *__restrict__ key,
                                                    const unsigned long long *__restrict__ key_lo,
                                                    const int *__restrict__ val, const int *__restrict__ parent,
                                                    const float4 *__restrict__ node4,
                                                    const double4 *__restrict__ sums,
                                                    const int *__restrict__ count, int sys, int cells_before,
                                                    int cap_cells, int *root_child, int *cell_child,
                                                    int *cell_start, int *cell_count, int *cell_level,
                                                    float *cx, float *cy, float *cz, float *cm, int sum_mode) {
    const int T = (int)totals[1];
    const int beg = sys_off[sys];
    const int nsys_bodies = sys_off[sys + 1] - beg;
    for (int b = grid_stride_start(); b < T; b += grid_stride()) {
        const unsigned u = ent_bfs[b];
        const int l = (int)(u >> kLevelShift);
        const int p = (int)(u & ((1u << kLevelShift) - 1u));
        if (body_sys[p] != sys) continue;
        int lo, hi, dp;
        levels_of(delta, nullptr, p, beg, lo, hi, dp);
        const bool is_cell = l < hi;
        const int pre = (int)(eoff[p] - (unsigned)p) - cells_before + (l - lo);
        int value;
        if (is_cell) {
            value = nsys_bodies + pre;
            if (pre < cap_cells) {
                if (cell_start) cell_start[pre] = p - beg;
                if (cell_count) cell_count[pre] = count[b];
                if (cell_level) cell_level[pre] = l;
                if (sum_mode) {
                    const double4 q = sums[b];
                    if (cx) cx[pre] = (float)q.y;
                    if (cy) cy[pre] = (float)q.z;
                    if (cz) cz[pre] = (float)q.w;
                    if (cm) cm[pre] = (float)q.x;
                } else {
                    const float4 q = node4[b];
                    if (cx) cx[pre] = q.x;
                    if (cy) cy[pre] = q.y;
                    if (cz) cz[pre] = q.z;
                    if (cm) cm[pre] = q.w;
                }
            }
        } else {
            value = val[p] - beg;
        }
        const int slot = digit_of(key[p], key_lo[p], l);
        const int par = parent[b];
        if (par < 0) {
            if (root_child) root_child[slot] = value;
        } else if (cell_child) {
            const unsigned pu = ent_bfs[par];
            const int pl = (int)(pu >> kLevelShift);
            const int pp = (int)(pu & ((1u << kLevelShift) - 1u));
            int plo, phi, pdp;
            levels_of(delta, nullptr, pp, beg, plo, phi, pdp);
            const int ppre = (int)(eoff[pp] - (unsigned)pp) - cells_before + (pl - plo);
            if (ppre < cap_cells) cell_child[8 * ppre + slot] = value;
        }
    }
}

__global__ void k_perm_export(const int *val, int beg, int n, int *perm) {
    for (int i = grid_stride_start(); i < n; i += grid_stride()) perm[i] = val[beg + i] - beg;
}

}  // namespace

int export_tree_impl(Ctx *ctx, int sys, int *perm, int *root_child, int *cell_child, int *cell_start,
                     int *cell_count, int *cell_level, float *cx, float *cy, float *cz, float *cm,
                     int cap_cells, int64_t *ncells, cudaStream_t st, int sum_mode) {
    // the reference's array format holds the reference's tree: Lebesgue order, one body per leaf
    if (!ctx->built || ctx->key_order != 0 || ctx->leaf_size != 1) return NBX_ERR_STATE;
    if (sys < 0 || sys >= ctx->nsys) return NBX_ERR_ARG;
    int off[2];
    NBX_CUDA(cudaMemcpyAsync(off, ctx->d_sys_off + sys, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    unsigned e_beg = 0, e_end = 0, T = 0;
    NBX_CUDA(cudaMemcpyAsync(&e_beg, ctx->d_ecount + off[0], sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    NBX_CUDA(cudaMemcpyAsync(&T, ctx->d_totals + 0, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    if (off[1] < ctx->nbodies)
        NBX_CUDA(cudaMemcpyAsync(&e_end, ctx->d_ecount + off[1], sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    NBX_CUDA(cudaStreamSynchronize(st));
    if (off[1] >= ctx->nbodies) e_end = T;
    const int cells_before = (int)e_beg - off[0];
    const int nc = (int)e_end - off[1] - cells_before;
    if (ncells) *ncells = nc;
    if (nc > cap_cells) {
        ctx->last_error = "export: cell capacity too small";
        return NBX_ERR_CAPACITY;
    }
    const int nb = off[1] - off[0];
    if (perm) {
        k_perm_export<<<ceil_div(nb, kBlock), kBlock, 0, st>>>(ctx->d_val, off[0], nb, perm);
        ++ctx->launches;
    }
    if (root_child) NBX_CUDA(cudaMemsetAsync(root_child, 0xff, 8 * sizeof(int), st));
    if (cell_child && nc > 0) NBX_CUDA(cudaMemsetAsync(cell_child, 0xff, 8 * sizeof(int) * (size_t)nc, st));
    const int gn = ceil_div(ctx->cap_nodes, kBlock) < ctx->nsm * 8 ? ceil_div(ctx->cap_nodes, kBlock) : ctx->nsm * 8;
    k_export<<<gn, kBlock, 0, st>>>(ctx->d_ent_alt, ctx->d_totals, ctx->d_body_sys, ctx->d_sys_off,
                                    ctx->d_delta, ctx->d_ecount, ctx->d_key, ctx->d_key_lo, ctx->d_val,
                                    ctx->d_parent, ctx->d_node4, ctx->d_sums, ctx->d_count, sys, cells_before,
                                    cap_cells, root_child, cell_child, cell_start, cell_count, cell_level, cx,
                                    cy, cz, cm, sum_mode);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

}  // namespace nbx
