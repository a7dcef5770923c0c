/*
 * serial_harness.cpp -- drives the reference's 3D/Serial tree code
 * (3D/Serial/NBody/src/{Interaction,Tree,Octant,Body,...}.cpp, staged from the
 * checkout by oracle/ref_cpu.py) on our synthetic bodies, on one thread, for
 * the timed CPU baseline.  TEST/BASELINE INFRASTRUCTURE ONLY.
 *
 * Units as omp_harness.cpp: the staged Constants.h sets TO_METERS = 1,
 * G = dt^2, TIME_STEP = 1 and the velocities handed in are dt*v, so one
 * reference step is one kick-drift step of length dt with G = 1.  The Serial
 * code's root is the fixed cube 60 * SYSTEM_SIZE (Interaction.cpp:122-125);
 * SYSTEM_SIZE is set so that this cube is the bodies' extent.
 *
 *   forces <in> <out>  the reference's tree build and force loop over all bodies
 *          with G = 1; writes the accelerations (n x 3 float64) to <out>.
 *   sample <in> <steps> <warmup> <k> <seed>  the reference's serial tree build
 *          over ALL bodies (Interaction.cpp:122-134), timed once; then per step
 *          the reference's force loop (:153-160) over k sampled bodies and its
 *          update (:166-200); the estimated step is build + force * n/k + update.
 * Input file: int32 n, float32 theta, eps, then float32 x,y,z,vx,vy,vz,m.
 */
#define private public
#include "Interaction.h"
#undef private

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#ifndef NBX_DT
#define NBX_DT 5e-4
#endif
double G = (NBX_DT) * (NBX_DT);
int NUM_BODIES = 0;
int NUM_SUNS = 0;
double SYSTEM_SIZE = 1.0;
double SOFTENING = 0.0;
double MAX_DISTANCE = 0.5;
structlog LOGCFG = {};

static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char **argv) {
    const bool forces = argc == 4 && std::strcmp(argv[1], "forces") == 0;
    if (!forces && (argc < 7 || std::strcmp(argv[1], "sample") != 0)) {
        std::fprintf(stderr, "usage: %s sample <in> <steps> <warmup> <k> <seed> | forces <in> <out>\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    int n = 0;
    float hdr[2];
    if (std::fread(&n, sizeof(int), 1, f) != 1) return 3;
    if (std::fread(hdr, sizeof(float), 2, f) != 2) return 3;
    std::vector<float> a(7 * (size_t)n);
    if (std::fread(a.data(), sizeof(float), a.size(), f) != a.size()) return 3;
    std::fclose(f);
    const int steps = forces ? 0 : std::atoi(argv[3]), warmup = forces ? 0 : std::atoi(argv[4]);
    const int k = forces ? 0 : std::atoi(argv[5]);
    const unsigned seed = forces ? 1u : (unsigned)std::atoi(argv[6]);
    NUM_BODIES = n;
    MAX_DISTANCE = hdr[0];
    SOFTENING = hdr[1];
    Body *suns = new Body[1];
    Body *bods = new Body[n];
    double ext = 0.0;
    for (int i = 0; i < n; i++) {
        bods[i].position.x = a[i];
        bods[i].position.y = a[(size_t)n + i];
        bods[i].position.z = a[2 * (size_t)n + i];
        bods[i].velocity.x = a[3 * (size_t)n + i];
        bods[i].velocity.y = a[4 * (size_t)n + i];
        bods[i].velocity.z = a[5 * (size_t)n + i];
        bods[i].mass = a[6 * (size_t)n + i];
        bods[i].acceleration.x = bods[i].acceleration.y = bods[i].acceleration.z = 0.0;
        ext = std::fmax(ext, std::fmax(std::fabs(a[i]), std::fmax(std::fabs(a[(size_t)n + i]),
                                                                     std::fabs(a[2 * (size_t)n + i]))));
    }
    SYSTEM_SIZE = 2.0 * ext * 1.0001 / 60.0;
    Interaction handler(false);
    LOGCFG.level = ERROR;
    LOGCFG.headers = false;
    if (forces) {
        /* Interaction.cpp:122-160 without the update: G = 1, accelerations of all
         * bodies read before updateBodies would zero them */
        G = 1.0;
        Tree *tree = new Tree(Octant(0.0, 0.0, 0.0, 60.0 * SYSTEM_SIZE));
        for (int i = 0; i < n; i++)
            if (tree->getOctant().contains(bods[i].position)) tree->insert(&bods[i]);
        for (int i = 0; i < n; i++)
            if (tree->getOctant().contains(bods[i].position)) handler.treeInteraction(tree, &bods[i]);
        delete tree;
        FILE *o = std::fopen(argv[3], "wb");
        if (!o) return 3;
        for (int i = 0; i < n; i++) {
            const double acc[3] = {bods[i].acceleration.x, bods[i].acceleration.y, bods[i].acceleration.z};
            std::fwrite(acc, sizeof(double), 3, o);
        }
        std::fclose(o);
        return 0;
    }
    std::printf("{\"threads\": 1, \"n\": %d, \"mode\": \"sample\", \"steps\": [", n);
    std::mt19937 rng(seed);
    /* Interaction.cpp:122-134: fixed root cube, serial inserts; built once */
    double t0 = now();
    Tree *tree = new Tree(Octant(0.0, 0.0, 0.0, 60.0 * SYSTEM_SIZE));
    for (int i = 0; i < n; i++)
        if (tree->getOctant().contains(bods[i].position)) tree->insert(&bods[i]);
    const double t_build = now() - t0;
    for (int s = 0; s < warmup + steps; s++) {
        std::vector<int> idx(k);
        for (int j = 0; j < k; j++) idx[j] = (int)(rng() % (unsigned)n);
        double t1 = now();
        for (int j = 0; j < k; j++) {  // Interaction.cpp:153-160 on the sampled bodies
            Body *b = &bods[idx[j]];
            if (tree->getOctant().contains(b->position)) handler.treeInteraction(tree, b);
        }
        const double tf = now() - t1;
        double t2 = now();
        handler.updateBodies(suns, bods);
        const double tu = now() - t2;
        if (s >= warmup)
            std::printf("%s[%.6f, %.6f, %.6f]", s > warmup ? ", " : "", t_build, tf * ((double)n / k), tu);
        std::fflush(stdout);
    }
    delete tree;
    std::printf("]}\n");
    return 0;
}
