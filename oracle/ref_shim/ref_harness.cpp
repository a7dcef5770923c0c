/*
 * ref_harness.cpp -- drives the reference's own kernels
 * (3D/CUDA/CUDA_NBody/src/Kernels.cu, compiled unmodified with g++ against
 * the CPU stand-in cuda.h) through one Barnes-Hut step, in the order of
 * BarnesHut::update (3D/CUDA/CUDA_NBody/src/BarnesHut.cu:195-258), and
 * canonicalises the resulting tree for comparison.
 *
 * TEST INFRASTRUCTURE ONLY (oracle recipe): used to generate the golden
 * fixtures under tests/golden/ and to pin the C restatement (refemu.c).
 *
 * Launch shapes: every kernel runs as <<<1,1>>> except the force kernel,
 * which runs as <<<1,32>>> with warp=32 so that one emulated warp walks each
 * aligned group of 32 sorted bodies, exactly as on the GPU.  The per-warp
 * stack is given `stack_size` entries (the reference's 64 can overflow).
 */
#include "cuda.h"
#include "Kernels.cuh"

#include <functional>
#include <math.h>
#include <string.h>
#include <vector>

int nbx_launch(int grid, int block, std::function<void()> body);

/* Shared memory of the emulated block (Kernels.cu:89, :472). */
float buffer[1 << 20];

extern "C" int ref_run_step(int n, float *x, float *y, float *z, float *vx, float *vy, float *vz,
                            const float *mass_in, float dt, float force_min_x, float force_max_x,
                            int stack_size, float *bbox_out, int *perm, int *ncells_out,
                            int cap_cells, int *root_child, int *cell_child, int *cell_start,
                            int *cell_count, int *cell_level, float *cell_x, float *cell_y,
                            float *cell_z, float *cell_m, float *ax_out, float *ay_out,
                            float *az_out)
{
    const int m = 2 * n + 12000; /* BarnesHut.cu:18 */
    if (2 * stack_size > (int)(sizeof(buffer) / sizeof(float))) return -2;
    std::vector<float> X(m), Y(m), Z(m), VX(m), VY(m), VZ(m), AX(m), AY(m), AZ(m), M(m);
    std::vector<int> child(8 * (size_t)m), start(m), sorted(m), count(m);
    int mutex = 0, index = 0;
    float bb[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; i++) {
        X[i] = x[i]; Y[i] = y[i]; Z[i] = z[i];
        VX[i] = vx[i]; VY[i] = vy[i]; VZ[i] = vz[i];
        M[i] = mass_in[i];
    }
    float *d = X.data();
    (void)d;
    int rc = 0;
    rc |= nbx_launch(1, 1, [&] {
        resetArraysKernel(&mutex, X.data(), Y.data(), Z.data(), M.data(), count.data(),
                          start.data(), sorted.data(), child.data(), &index, &bb[0], &bb[1],
                          &bb[2], &bb[3], &bb[4], &bb[5], n, m);
    });
    rc |= nbx_launch(1, 1, [&] {
        computeBoundingBoxKernel(&mutex, X.data(), Y.data(), Z.data(), &bb[0], &bb[1], &bb[2],
                                 &bb[3], &bb[4], &bb[5], n, 1);
    });
    rc |= nbx_launch(1, 1, [&] {
        buildTreeKernel(X.data(), Y.data(), Z.data(), M.data(), count.data(), start.data(),
                        child.data(), &index, &bb[0], &bb[1], &bb[2], &bb[3], &bb[4], &bb[5], n,
                        m);
    });
    rc |= nbx_launch(1, 1, [&] { centreOfMassKernel(X.data(), Y.data(), Z.data(), M.data(), &index, n); });
    rc |= nbx_launch(1, 1, [&] {
        sortKernel(count.data(), start.data(), sorted.data(), child.data(), &index, n);
    });
    float fmin = isnan(force_min_x) ? bb[0] : force_min_x;
    float fmax = isnan(force_max_x) ? bb[1] : force_max_x;
    rc |= nbx_launch(1, 32, [&] {
        computeForcesKernel(X.data(), Y.data(), Z.data(), VX.data(), VY.data(), VZ.data(),
                            AX.data(), AY.data(), AZ.data(), M.data(), sorted.data(),
                            child.data(), &fmin, &fmax, n, 1.0f, 32, 32, stack_size);
    });
    if (rc) return -1;
    for (int i = 0; i < n; i++) { ax_out[i] = AX[i]; ay_out[i] = AY[i]; az_out[i] = AZ[i]; }
    rc |= nbx_launch(1, 1, [&] {
        updateKernel(X.data(), Y.data(), Z.data(), VX.data(), VY.data(), VZ.data(), AX.data(),
                     AY.data(), AZ.data(), n, dt, 1.0f);
    });
    if (rc) return -1;
    for (int i = 0; i < 6; i++) bbox_out[i] = bb[i];
    for (int i = 0; i < n; i++) {
        perm[i] = sorted[i];
        x[i] = X[i]; y[i] = Y[i]; z[i] = Z[i];
        vx[i] = VX[i]; vy[i] = VY[i]; vz[i] = VZ[i];
    }

    /* canonicalise: pre-order renumbering of the cells reachable from the
     * root slots child[0..7] (Kernels.cu:225, the root's slots alias node 0) */
    int ncells = index - n;
    if (ncells > cap_cells) return -3;
    std::vector<int> canon(m, -1);
    struct fr { int cell, slot, level; };
    std::vector<fr> st;
    int next = 0;
    st.push_back({-1, 0, 0});
    while (!st.empty()) {
        fr &f = st.back();
        if (f.slot == 8) { st.pop_back(); continue; }
        int s = f.slot++;
        int raw = f.cell < 0 ? child[s] : child[8 * f.cell + s];
        int *dst = f.cell < 0 ? &root_child[s] : &cell_child[8 * canon[f.cell] + s];
        if (raw < 0) { *dst = -1; continue; }
        if (raw < n) { *dst = raw; continue; }
        int k = next++;
        if (k >= cap_cells) return -3;
        canon[raw] = k;
        *dst = n + k;
        cell_start[k] = start[raw];
        cell_count[k] = count[raw];
        cell_level[k] = f.level + 1;
        cell_x[k] = X[raw]; cell_y[k] = Y[raw]; cell_z[k] = Z[raw]; cell_m[k] = M[raw];
        int lvl = f.level + 1;
        st.push_back({raw, 0, lvl});
    }
    *ncells_out = next;
    if (next != ncells) return -4; /* unreachable cells would mean a broken build */
    return 0;
}
