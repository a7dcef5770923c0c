/*
 * refemu.c -- CPU restatement of the Barnes-Hut kernel chain of
 * 3D/CUDA/CUDA_NBody/src/Kernels.cu (MichaelSt98/NNS).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it to check the CUDA
 * path.  The product path (nns_gb300/libnbx.so) never links or calls it.
 *
 * Semantics restated here (the "intended" behaviour of the reference kernels):
 *   bbox   Kernels.cu:21-64 resets min/max to 0, so the root box is the
 *          bounding box of the bodies AND the origin; :67-154 reduce it.
 *   build  Kernels.cu:157-377 Burtscher insertion.  At every level the
 *          midpoint is 0.5*(min+max) with min+max rounded to float, the
 *          comparison made against the exact half and the new bound stored
 *          as float (:200-258, :297-345).  Child code
 *          c = [x<mid] + 2[y<mid] + 4[z<mid]; a slot holding a body is split
 *          until the two bodies separate (:285-362).
 *          The final tree is independent of insertion order: a cell exists
 *          for every subdivision region holding >= 2 bodies.  Cells are
 *          numbered canonically in depth-first pre-order (children 0..7),
 *          as ids n .. n+ncells-1 (the reference allocates ids from n
 *          upwards, :288).
 *   COM    Kernels.cu:260-266 + :381-399 (sum of m*x over the cell, divided
 *          by the summed mass).  Restated deterministically: sums in FP64 in
 *          child-slot order, rounded to FP32 once.
 *   sort   Kernels.cu:403-456: in-order listing of bodies, children 0..7.
 *   force  Kernels.cu:460-577: warp-coherent walk.  The bodies of one aligned
 *          group of `group` consecutive sorted positions share one traversal:
 *          root children are always opened (:505-517); a child body always
 *          interacts (:543); a child cell interacts only if every body of
 *          the group accepts it, dp <= r (:543) with dp = depth0 * 0.25^(L-1)
 *          for a level-L cell (:513,:525,:557), depth0 = radius^2/theta_ref
 *          (:477,:513), radius = 0.5*(maxX-minX).  Interaction
 *          a += m * d * rsqrt(r)^3, r = |d|^2 + eps^2 (:538,:546-551).
 *          Intended semantics where the reference is defective: a body that
 *          is a direct child of the root interacts directly (the reference
 *          pushes it as a node, :505-516); the stack is unbounded (the
 *          reference has 64 float-typed entries per warp).
 *          r is evaluated as fma(dz,dz,fma(dy,dy,fma(dx,dx,eps2))), the
 *          rounding the CUDA path uses, so MAC decisions agree bit for bit.
 *   update Kernels.cu:581-600: v += dt*a; x += d*dt*v (as fused multiply-adds).
 *
 * Also: FP64 direct summation (the ground truth for force errors) and the
 * FP64 evaluation of the same interaction lists.
 *
 * Compile with -ffp-contract=off so that x86-64 and aarch64 round alike.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ERR_DEPTH 3
#define ORC_ERR_CAPACITY 4
#define ORC_ERR_ARG 5

/* ------------------------------------------------------------------ bbox */
int orc_bbox(int n, const float *x, const float *y, const float *z, float *out)
{
    float mnx = 0.f, mxx = 0.f, mny = 0.f, mxy = 0.f, mnz = 0.f, mxz = 0.f;
    for (int i = 0; i < n; i++) {
        mnx = fminf(mnx, x[i]); mxx = fmaxf(mxx, x[i]);
        mny = fminf(mny, y[i]); mxy = fmaxf(mxy, y[i]);
        mnz = fminf(mnz, z[i]); mxz = fmaxf(mxz, z[i]);
    }
    /* + 0.0f turns a -0 bound into +0, so the box does not depend on how
     * fminf orders signed zeros */
    out[0] = mnx + 0.0f; out[1] = mxx + 0.0f; out[2] = mny + 0.0f;
    out[3] = mxy + 0.0f; out[4] = mnz + 0.0f; out[5] = mxz + 0.0f;
    return ORC_OK;
}

/* One subdivision step along one axis (Kernels.cu:200-206): returns 1 for the
 * lower half.  The midpoint is the exact half of the float sum min+max. */
static inline int split_axis(float v, float *mn, float *mx)
{
    float s = *mn + *mx;
    double mid = 0.5 * (double)s;
    if ((double)v < mid) { *mx = (float)mid; return 1; }
    *mn = (float)mid;
    return 0;
}

static inline int probe_axis(float v, float mn, float mx)
{
    float s = mn + mx;
    return (double)v < 0.5 * (double)s;
}

/* ------------------------------------------------------------------ keys
 * Replays the subdivision for `levels` levels (<= 42) and packs the child
 * codes 3 bits per level, most significant first: key_hi holds levels 1..21,
 * key_lo levels 22..42 (when levels > 21).  Ascending (key_hi, key_lo) is the
 * reference's in-order body order. */
int orc_keys(int n, const float *x, const float *y, const float *z, const float *bb,
             int levels, uint64_t *key_hi, uint64_t *key_lo)
{
    if (levels < 1 || levels > 42) return ORC_ERR_ARG;
    for (int i = 0; i < n; i++) {
        float mnx = bb[0], mxx = bb[1], mny = bb[2], mxy = bb[3], mnz = bb[4], mxz = bb[5];
        uint64_t hi = 0, lo = 0;
        for (int l = 1; l <= levels; l++) {
            int c = split_axis(x[i], &mnx, &mxx) + 2 * split_axis(y[i], &mny, &mxy) +
                    4 * split_axis(z[i], &mnz, &mxz);
            if (l <= 21) hi |= (uint64_t)c << (3 * (21 - l));
            else lo |= (uint64_t)c << (3 * (42 - l));
        }
        key_hi[i] = hi;
        if (key_lo) key_lo[i] = lo;
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------ build */
typedef struct {
    int child[8]; /* -1 null; >= 0 body id; <= -2 cell (-2 - raw cell id) */
} raw_cell;

#define RAW_CELL(k) (-2 - (k))
#define IS_RAW_CELL(v) ((v) <= -2)
#define RAW_CELL_ID(v) (-2 - (v))

typedef struct {
    raw_cell *cells;
    int ncells, cap;
} raw_tree;

static int raw_new_cell(raw_tree *t)
{
    if (t->ncells == t->cap) {
        int ncap = t->cap ? 2 * t->cap : 1024;
        raw_cell *nc = (raw_cell *)realloc(t->cells, (size_t)ncap * sizeof(raw_cell));
        if (!nc) return -1;
        t->cells = nc;
        t->cap = ncap;
    }
    int k = t->ncells++;
    for (int s = 0; s < 8; s++) t->cells[k].child[s] = -1;
    return k;
}

/* Serial insertion (Kernels.cu:182-374 with a single thread). Raw cell 0 is
 * the root. Returns ORC_ERR_DEPTH when two bodies share a region deeper than
 * max_depth levels (the reference would loop forever on duplicates). */
static int raw_insert_all(raw_tree *t, int n, const float *x, const float *y, const float *z,
                          const float *bb, int max_depth)
{
    if (raw_new_cell(t) != 0) return ORC_ERR_CAPACITY;
    for (int b = 0; b < n; b++) {
        float mnx = bb[0], mxx = bb[1], mny = bb[2], mxy = bb[3], mnz = bb[4], mxz = bb[5];
        int cell = 0, depth = 1;
        int c = split_axis(x[b], &mnx, &mxx) + 2 * split_axis(y[b], &mny, &mxy) +
                4 * split_axis(z[b], &mnz, &mxz);
        for (;;) {
            int ch = t->cells[cell].child[c];
            if (ch == -1) { t->cells[cell].child[c] = b; break; }
            if (IS_RAW_CELL(ch)) {
                cell = RAW_CELL_ID(ch);
                c = split_axis(x[b], &mnx, &mxx) + 2 * split_axis(y[b], &mny, &mxy) +
                    4 * split_axis(z[b], &mnz, &mxz);
                depth++;
                continue;
            }
            /* slot holds body `ch`: split until separated (Kernels.cu:285-362) */
            int o = ch;
            for (;;) {
                if (depth >= max_depth) return ORC_ERR_DEPTH;
                int k = raw_new_cell(t);
                if (k < 0) return ORC_ERR_CAPACITY;
                t->cells[cell].child[c] = RAW_CELL(k);
                int co = probe_axis(x[o], mnx, mxx) + 2 * probe_axis(y[o], mny, mxy) +
                         4 * probe_axis(z[o], mnz, mxz);
                int cb = split_axis(x[b], &mnx, &mxx) + 2 * split_axis(y[b], &mny, &mxy) +
                         4 * split_axis(z[b], &mnz, &mxz);
                depth++;
                t->cells[k].child[co] = o;
                cell = k;
                c = cb;
                if (co != cb) { t->cells[k].child[cb] = b; break; }
            }
            break;
        }
    }
    return ORC_OK;
}

typedef struct {
    double m, sx, sy, sz;
    int count;
} moments;

/* Canonicalisation: pre-order renumbering, in-order body list, FP64 moments
 * summed in slot order.  Iterative to keep the C stack small. */
typedef struct {
    int raw;   /* raw cell id */
    int canon; /* canonical cell index (0-based) or -1 for the root */
    int slot;  /* next slot to visit */
    int level;
    moments mom;
} frame;

int orc_build(int n, const float *x, const float *y, const float *z, const float *m,
              const float *bb, int max_depth, int cap_cells,
              int *perm, int *ncells_out, int *root_child,
              int *cell_child, int *cell_start, int *cell_count, int *cell_level,
              float *cell_x, float *cell_y, float *cell_z, float *cell_m,
              double *cell_m64, double *cell_com64)
{
    raw_tree t = {0};
    *ncells_out = 0;
    int rc = raw_insert_all(&t, n, x, y, z, bb, max_depth);
    if (rc != ORC_OK) { free(t.cells); return rc; }
    int ncells = t.ncells - 1;
    if (ncells > cap_cells) { free(t.cells); return ORC_ERR_CAPACITY; }

    frame *st = (frame *)malloc(sizeof(frame) * (size_t)(max_depth + 4));
    if (!st) { free(t.cells); return ORC_ERR_CAPACITY; }
    int sp = 0, next_canon = 0, pos = 0;
    st[0].raw = 0; st[0].canon = -1; st[0].slot = 0; st[0].level = 0;
    memset(&st[0].mom, 0, sizeof(moments));
    while (sp >= 0) {
        frame *f = &st[sp];
        if (f->slot == 8) {
            /* finalise this cell and fold its moments into the parent */
            if (f->canon >= 0) {
                int k = f->canon;
                cell_count[k] = f->mom.count;
                cell_m[k] = (float)f->mom.m;
                cell_x[k] = (float)(f->mom.sx / f->mom.m);
                cell_y[k] = (float)(f->mom.sy / f->mom.m);
                cell_z[k] = (float)(f->mom.sz / f->mom.m);
                if (cell_m64) cell_m64[k] = f->mom.m;
                if (cell_com64) {
                    cell_com64[3 * k + 0] = f->mom.sx / f->mom.m;
                    cell_com64[3 * k + 1] = f->mom.sy / f->mom.m;
                    cell_com64[3 * k + 2] = f->mom.sz / f->mom.m;
                }
                frame *p = &st[sp - 1];
                p->mom.m += f->mom.m;
                p->mom.sx += f->mom.sx;
                p->mom.sy += f->mom.sy;
                p->mom.sz += f->mom.sz;
                p->mom.count += f->mom.count;
            }
            sp--;
            continue;
        }
        int s = f->slot++;
        int ch = t.cells[f->raw].child[s];
        int *dst = f->canon < 0 ? &root_child[s] : &cell_child[8 * f->canon + s];
        if (ch == -1) { *dst = -1; continue; }
        if (!IS_RAW_CELL(ch)) {
            *dst = ch;
            perm[pos++] = ch;
            double mb = (double)m[ch];
            f->mom.m += mb;
            f->mom.sx += mb * (double)x[ch];
            f->mom.sy += mb * (double)y[ch];
            f->mom.sz += mb * (double)z[ch];
            f->mom.count += 1;
            continue;
        }
        int k = next_canon++;
        *dst = n + k;
        cell_start[k] = pos;
        cell_level[k] = f->level + 1;
        frame *g = &st[++sp];
        g->raw = RAW_CELL_ID(ch);
        g->canon = k;
        g->slot = 0;
        g->level = f->level + 1;
        memset(&g->mom, 0, sizeof(moments));
    }
    free(st);
    free(t.cells);
    *ncells_out = ncells;
    return ORC_OK;
}

/* depth0 = radius^2 / theta_ref with radius = 0.5*(maxX-minX) (Kernels.cu:477,513) */
float orc_depth0(const float *bb, float theta_ref)
{
    float radius = (float)(0.5 * (double)(bb[1] - bb[0]));
    return (radius * radius) / theta_ref;
}

/* Traceless quadrupole moments of the canonical cells (an extension: the
 * reference's kernels carry monopoles only).  Per cell, about its FP64 centre
 * of mass c: M2 = sum over children in child order of [M2_child +
 * m_child (c_child - c)(c_child - c)^T] (a body child has M2 = 0 and c_child
 * = its position), all in FP64; Q = 3 M2 - tr(M2) I, stored per cell as
 * (xx, yy, zz, xy, xz, yz).  Cells are in depth-first pre-order, so every
 * child cell has a larger index than its parent and a reverse sweep composes
 * each cell from finished children. */
int orc_quad(int n, const float *x, const float *y, const float *z, const float *m, int ncells,
             const int *cell_child, const double *cell_m64, const double *cell_com64, double *q)
{
    double *m2 = (double *)malloc(sizeof(double) * 6 * (size_t)(ncells > 0 ? ncells : 1));
    if (!m2) return ORC_ERR_CAPACITY;
    for (int k = ncells - 1; k >= 0; k--) {
        const double cx = cell_com64[3 * k], cy = cell_com64[3 * k + 1], cz = cell_com64[3 * k + 2];
        double a[6] = {0, 0, 0, 0, 0, 0};
        for (int s = 0; s < 8; s++) {
            int ch = cell_child[8 * k + s];
            if (ch < 0) continue;
            double mc, dx, dy, dz;
            if (ch < n) {
                mc = (double)m[ch];
                dx = (double)x[ch] - cx; dy = (double)y[ch] - cy; dz = (double)z[ch] - cz;
            } else {
                int j = ch - n;
                mc = cell_m64[j];
                dx = cell_com64[3 * j] - cx; dy = cell_com64[3 * j + 1] - cy; dz = cell_com64[3 * j + 2] - cz;
                for (int t = 0; t < 6; t++) a[t] += m2[6 * j + t];
            }
            a[0] += mc * dx * dx; a[1] += mc * dy * dy; a[2] += mc * dz * dz;
            a[3] += mc * dx * dy; a[4] += mc * dx * dz; a[5] += mc * dy * dz;
        }
        for (int t = 0; t < 6; t++) m2[6 * k + t] = a[t];
        const double tr = a[0] + a[1] + a[2];
        q[6 * k + 0] = 3.0 * a[0] - tr;
        q[6 * k + 1] = 3.0 * a[1] - tr;
        q[6 * k + 2] = 3.0 * a[2] - tr;
        q[6 * k + 3] = 3.0 * a[3];
        q[6 * k + 4] = 3.0 * a[4];
        q[6 * k + 5] = 3.0 * a[5];
    }
    free(m2);
    return ORC_OK;
}

/* ------------------------------------------------------------------ force */
static inline float mac_r(float dx, float dy, float dz, float eps2)
{
    return fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
}

typedef struct { int node; float dp; } sentry;

/* Warp-coherent walk over aligned groups of `group` sorted positions.
 * groups: list of group indices to evaluate (NULL = all).
 * Outputs are indexed by ORIGINAL body id.  Returns the total list length. */
long long orc_forces(int n, const float *x, const float *y, const float *z, const float *m,
                     const int *perm, int ncells, const int *root_child, const int *cell_child,
                     const float *cell_x, const float *cell_y, const float *cell_z,
                     const float *cell_m, float depth0, float eps2, int group,
                     const int *groups, int ngroups,
                     float *ax, float *ay, float *az,
                     double *ax64, double *ay64, double *az64, int *nlist, int *nopen,
                     const double *cell_q)
{
    (void)ncells;
    if (group < 1 || group > 1024) return -1;
    int ngroups_all = (n + group - 1) / group;
    if (!groups) ngroups = ngroups_all;
    int cap = 1024;
    sentry *stack = (sentry *)malloc(sizeof(sentry) * (size_t)cap);
    float px[1024], py[1024], pz[1024], fx[1024], fy[1024], fz[1024];
    double gx[1024], gy[1024], gz[1024];
    long long total = 0;
    for (int gi = 0; gi < ngroups; gi++) {
        int g = groups ? groups[gi] : gi;
        if (g < 0 || g >= ngroups_all) continue;
        int p0 = g * group, p1 = p0 + group;
        if (p1 > n) p1 = n;
        int L = p1 - p0;
        for (int l = 0; l < L; l++) {
            int b = perm[p0 + l];
            px[l] = x[b]; py[l] = y[b]; pz[l] = z[b];
            fx[l] = fy[l] = fz[l] = 0.f;
            gx[l] = gy[l] = gz[l] = 0.0;
        }
        int len = 0, opened = 0, top = 0;
#define NODE_POS(ch, cx, cy, cz, cm)                                                  \
    do {                                                                              \
        if ((ch) < n) { cx = x[ch]; cy = y[ch]; cz = z[ch]; cm = m[ch]; }             \
        else { int k_ = (ch) - n; cx = cell_x[k_]; cy = cell_y[k_]; cz = cell_z[k_];  \
               cm = cell_m[k_]; }                                                     \
    } while (0)
#define INTERACT(cx, cy, cz, cm, ch)                                                  \
    do {                                                                              \
        const double *q_ = (cell_q && (ch) >= n) ? cell_q + 6 * (size_t)((ch) - n) : 0; \
        for (int l = 0; l < L; l++) {                                                 \
            float dx = cx - px[l], dy = cy - py[l], dz = cz - pz[l];                  \
            float r = mac_r(dx, dy, dz, eps2);                                        \
            float ri = 1.0f / sqrtf(r);                                               \
            float f = cm * ri * ri * ri;                                              \
            fx[l] = fmaf(f, dx, fx[l]); fy[l] = fmaf(f, dy, fy[l]);                   \
            fz[l] = fmaf(f, dz, fz[l]);                                               \
            double ddx = (double)cx - (double)px[l], ddy = (double)cy - (double)py[l], \
                   ddz = (double)cz - (double)pz[l];                                  \
            double rr = ddx * ddx + ddy * ddy + ddz * ddz + (double)eps2;             \
            double f64 = (double)cm / (rr * sqrt(rr));                                \
            if (q_) {                                                                 \
                /* a += -Q d / r^5 + 5/2 (d.Q.d) d / r^7, d = cell - body */          \
                double qx = q_[0] * ddx + q_[3] * ddy + q_[4] * ddz;                  \
                double qy = q_[3] * ddx + q_[1] * ddy + q_[5] * ddz;                  \
                double qz = q_[4] * ddx + q_[5] * ddy + q_[2] * ddz;                  \
                double r5 = 1.0 / (rr * rr * sqrt(rr));                               \
                double c = 2.5 * (ddx * qx + ddy * qy + ddz * qz) * r5 / rr;          \
                gx[l] += (f64 + c) * ddx - r5 * qx;                                   \
                gy[l] += (f64 + c) * ddy - r5 * qy;                                   \
                gz[l] += (f64 + c) * ddz - r5 * qz;                                   \
            } else {                                                                  \
                gx[l] += f64 * ddx; gy[l] += f64 * ddy; gz[l] += f64 * ddz;           \
            }                                                                         \
        }                                                                             \
        len++;                                                                        \
    } while (0)
        for (int s = 0; s < 8; s++) {
            int ch = root_child[s];
            if (ch < 0) continue;
            if (ch < n) {
                float cx, cy, cz, cm;
                NODE_POS(ch, cx, cy, cz, cm);
                INTERACT(cx, cy, cz, cm, ch);
            } else {
                stack[top].node = ch; stack[top].dp = depth0; top++;
                opened++;
            }
        }
        while (top > 0) {
            top--;
            int node = stack[top].node;
            float dp = 0.25f * stack[top].dp;
            for (int s = 0; s < 8; s++) {
                int ch = cell_child[8 * (node - n) + s];
                if (ch < 0) continue;
                float cx, cy, cz, cm;
                NODE_POS(ch, cx, cy, cz, cm);
                int accept = 1;
                if (ch >= n) {
                    for (int l = 0; l < L; l++) {
                        float dx = cx - px[l], dy = cy - py[l], dz = cz - pz[l];
                        if (!(dp <= mac_r(dx, dy, dz, eps2))) { accept = 0; break; }
                    }
                }
                if (accept) {
                    INTERACT(cx, cy, cz, cm, ch);
                } else {
                    if (top == cap) {
                        cap *= 2;
                        stack = (sentry *)realloc(stack, sizeof(sentry) * (size_t)cap);
                    }
                    stack[top].node = ch; stack[top].dp = dp; top++;
                    opened++;
                }
            }
        }
#undef NODE_POS
#undef INTERACT
        for (int l = 0; l < L; l++) {
            int b = perm[p0 + l];
            if (ax) { ax[b] = fx[l]; ay[b] = fy[l]; az[b] = fz[l]; }
            if (ax64) { ax64[b] = gx[l]; ay64[b] = gy[l]; az64[b] = gz[l]; }
            if (nlist) nlist[b] = len;
            if (nopen) nopen[b] = opened;
        }
        total += (long long)len * L;
    }
    free(stack);
    return total;
}

/* ------------------------------------------------------------------ update */
void orc_update(int n, float *x, float *y, float *z, float *vx, float *vy, float *vz,
                const float *ax, const float *ay, const float *az, float dt, float d)
{
    float ddt = d * dt;
    for (int i = 0; i < n; i++) {
        vx[i] = fmaf(dt, ax[i], vx[i]);
        vy[i] = fmaf(dt, ay[i], vy[i]);
        vz[i] = fmaf(dt, az[i], vz[i]);
        x[i] = fmaf(ddt, vx[i], x[i]);
        y[i] = fmaf(ddt, vy[i], y[i]);
        z[i] = fmaf(ddt, vz[i], z[i]);
    }
}

/* ------------------------------------------------------------------ FP64 direct sum */
void orc_direct_fp64(int n, const float *x, const float *y, const float *z, const float *m,
                     double eps2, int nt, const int *targets, double *ax, double *ay, double *az)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int t = 0; t < nt; t++) {
        int i = targets[t];
        double xi = x[i], yi = y[i], zi = z[i];
        double sx = 0, sy = 0, sz = 0;
        for (int j = 0; j < n; j++) {
            double dx = (double)x[j] - xi, dy = (double)y[j] - yi, dz = (double)z[j] - zi;
            double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double f = (double)m[j] / (r2 * sqrt(r2));
            sx += f * dx; sy += f * dy; sz += f * dz;
        }
        ax[t] = sx; ay[t] = sy; az[t] = sz;
    }
}

/* FP64 direct-sum potential phi_i = -sum_{j != i} m_j / sqrt(|d|^2 + eps2) */
void orc_direct_pot_fp64(int n, const float *x, const float *y, const float *z, const float *m,
                         double eps2, int nt, const int *targets, double *phi)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int t = 0; t < nt; t++) {
        int i = targets[t];
        double xi = x[i], yi = y[i], zi = z[i], s = 0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double dx = (double)x[j] - xi, dy = (double)y[j] - yi, dz = (double)z[j] - zi;
            s -= (double)m[j] / sqrt(dx * dx + dy * dy + dz * dz + eps2);
        }
        phi[t] = s;
    }
}

/* ------------------------------------------------------------------ FP64 direct-sum adjoint
 * Kick-drift with direct-sum forces (G = 1, Plummer softening) in FP64 and the
 * exact gradient of L = sum_i |x_i(T) - x*_i|^2 w.r.t. x0, v0, m.  Arrays are
 * [3][n] (x0, v0, target, gx, gv) and [n] (m, gm).  Used to check the GPU
 * adjoint (which differs by the Barnes-Hut approximation). */
static void direct_acc64(int n, const double *x, const double *m, double eps2, double *a)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; i++) {
        double sx = 0, sy = 0, sz = 0;
        for (int j = 0; j < n; j++) {
            double dx = x[j] - x[i], dy = x[n + j] - x[n + i], dz = x[2 * n + j] - x[2 * n + i];
            double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double f = m[j] / (r2 * sqrt(r2));
            sx += f * dx; sy += f * dy; sz += f * dz;
        }
        a[i] = sx; a[n + i] = sy; a[2 * n + i] = sz;
    }
}

int orc_direct_adjoint(int n, const double *x0, const double *v0, const double *m,
                       const double *target, double eps2, double dt, double d, int T,
                       double *loss, double *gx, double *gv, double *gm)
{
    size_t sz = (size_t)3 * n;
    double *X = (double *)malloc(sizeof(double) * sz * (size_t)(T + 1));
    double *v = (double *)malloc(sizeof(double) * sz);
    double *a = (double *)malloc(sizeof(double) * sz);
    double *lx = gx, *lv = gv;
    double *g = (double *)malloc(sizeof(double) * sz);
    double *tx = (double *)malloc(sizeof(double) * sz);
    if (!X || !v || !a || !g || !tx) return ORC_ERR_CAPACITY;
    memcpy(X, x0, sizeof(double) * sz);
    memcpy(v, v0, sizeof(double) * sz);
    for (int k = 0; k < T; k++) {
        double *xk = X + sz * k, *xn = X + sz * (k + 1);
        direct_acc64(n, xk, m, eps2, a);
        for (size_t q = 0; q < sz; q++) {
            v[q] += dt * a[q];
            xn[q] = xk[q] + d * dt * v[q];
        }
    }
    double L = 0;
    double *xT = X + sz * T;
    for (size_t q = 0; q < sz; q++) {
        double e = xT[q] - target[q];
        L += e * e;
        lx[q] = 2 * e;
        lv[q] = 0;
    }
    for (int i = 0; i < n; i++) gm[i] = 0;
    *loss = L;
    for (int k = T - 1; k >= 0; k--) {
        double *x = X + sz * k;
        for (size_t q = 0; q < sz; q++) {
            lv[q] += d * dt * lx[q];
            g[q] = dt * lv[q];
        }
        /* target terms: lx_i -= sum_j m_j J(d_ij) g_i */
#pragma omp parallel for schedule(dynamic, 16)
        for (int i = 0; i < n; i++) {
            double ox = 0, oy = 0, oz = 0;
            double gxi = g[i], gyi = g[n + i], gzi = g[2 * n + i];
            for (int j = 0; j < n; j++) {
                if (j == i) continue;
                double dx = x[j] - x[i], dy = x[n + j] - x[n + i], dz = x[2 * n + j] - x[2 * n + i];
                double r2 = dx * dx + dy * dy + dz * dz + eps2, s = sqrt(r2);
                double i3 = 1.0 / (r2 * s), i5 = i3 / r2;
                double dg = dx * gxi + dy * gyi + dz * gzi;
                ox += m[j] * (gxi * i3 - 3 * dx * dg * i5);
                oy += m[j] * (gyi * i3 - 3 * dy * dg * i5);
                oz += m[j] * (gzi * i3 - 3 * dz * dg * i5);
            }
            tx[i] = -ox; tx[n + i] = -oy; tx[2 * n + i] = -oz;
        }
        /* source terms: lx_j += sum_i m_j J(d_ij) g_i, lm_j += sum_i g_i . d_ij |d_ij|^-3 */
#pragma omp parallel for schedule(dynamic, 16)
        for (int j = 0; j < n; j++) {
            double sx = 0, sy = 0, sz2 = 0, sm = 0;
            for (int i = 0; i < n; i++) {
                if (j == i) continue;
                double dx = x[j] - x[i], dy = x[n + j] - x[n + i], dz = x[2 * n + j] - x[2 * n + i];
                double r2 = dx * dx + dy * dy + dz * dz + eps2, s = sqrt(r2);
                double i3 = 1.0 / (r2 * s), i5 = i3 / r2;
                double gxi = g[i], gyi = g[n + i], gzi = g[2 * n + i];
                double dg = dx * gxi + dy * gyi + dz * gzi;
                sx += gxi * i3 - 3 * dx * dg * i5;
                sy += gyi * i3 - 3 * dy * dg * i5;
                sz2 += gzi * i3 - 3 * dz * dg * i5;
                sm += dg * i3;
            }
            lx[j] += tx[j] + m[j] * sx;
            lx[n + j] += tx[n + j] + m[j] * sy;
            lx[2 * n + j] += tx[2 * n + j] + m[j] * sz2;
            gm[j] += sm;
        }
    }
    free(X); free(v); free(a); free(g); free(tx);
    return ORC_OK;
}

/* ---------------------------------------------------------------------------
 * Headless frame: restatement of the reference renderer's splat
 * (3D/CUDA/CUDA_NBody/src/Renderer.cpp:54-147), bodies in input order, double
 * precision throughout, as the reference.
 *   px = (W/2) (1 + x / (systemSize renderScale))               (:86-89)
 *   a body is drawn when dot < int(px) < W - dot (same for y)   (:66-71)
 *   vPortion = sqrt((|v| - vmin) / vmax); colour ramp clamped   (:96-104)
 *   dot: i, j in [-dot/2, dot/2), pixel (floor(px)+i, floor(py)+j) gains
 *   colour * brightness / (pow(exp((s (floor(px)+i-px))^2)
 *                             + exp((s (floor(py)+j-py))^2), 0.75) + 1)  (:106-128)
 *   byte = int(255 clamp(sum))                                   (:144-147)
 * hd (3 W H doubles) is scratch; rgb receives W*H*3 bytes.
 * ------------------------------------------------------------------------- */
static double clamp01(double v) { return fmax(fmin(v, 1.0), 0.0); }

static double to_pixel(double p, int size, double system_size, double scale)
{
    return (size / 2.0) * (1.0 + p / (system_size * scale));
}

int orc_render(int n, const float *x, const float *y, const float *z, const float *vx,
               const float *vy, const float *vz, int width, int height, double render_scale,
               double vmax, double vmin, double brightness, double sharpness, int dot,
               double system_size, double *hd, unsigned char *rgb)
{
    (void)z;
    if (width < 1 || height < 1 || dot < 0) return ORC_ERR_ARG;
    memset(hd, 0, sizeof(double) * 3 * (size_t)width * (size_t)height);
    for (int b = 0; b < n; b++) {
        const double bx = x[b], by = y[b];
        const double pxs = to_pixel(bx, width, system_size, render_scale);
        const double pys = to_pixel(by, height, system_size, render_scale);
        const int xi = (int)pxs, yi = (int)pys;
        if (!(xi > dot && xi < width - dot && yi > dot && yi < height - dot)) continue;
        const double vxd = vx[b], vyd = vy[b], vzd = vz[b];
        const double vmag = sqrt(vxd * vxd + vyd * vyd + vzd * vzd);
        if (vmag < vmin) continue;
        const double vp = sqrt((vmag - vmin) / vmax);
        const double cr = clamp01(4 * (vp - 0.333));
        const double cg = clamp01(fmin(4 * vp, 4.0 * (1.0 - vp)));
        const double cb = clamp01(4 * (0.5 - vp));
        for (int i = -dot / 2; i < dot / 2; i++) {
            for (int j = -dot / 2; j < dot / 2; j++) {
                const double xp = floor(pxs), yp = floor(pys);
                const double f = brightness /
                                 (pow(exp(pow(sharpness * (xp + i - pxs), 2.0)) +
                                          exp(pow(sharpness * (yp + j - pys), 2.0)), 0.75) + 1.0);
                const size_t pix = 3 * ((size_t)(int)(xp + i) + (size_t)width * (size_t)(int)(yp + j));
                hd[pix + 0] += cr * f;
                hd[pix + 1] += cg * f;
                hd[pix + 2] += cb * f;
            }
        }
    }
    for (size_t k = 0; k < 3 * (size_t)width * (size_t)height; k++)
        rgb[k] = (unsigned char)(int)(255.0 * clamp01(hd[k]));
    return ORC_OK;
}
