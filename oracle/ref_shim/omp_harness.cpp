/*
 * omp_harness.cpp -- drives the reference's 3D/OpenMP tree code
 * (3D/OpenMP/OpenMP_NBody/src/{Interaction,Tree,Octant,Body,...}.cpp, staged
 * from the checkout by oracle/ref_cpu.py) on our synthetic bodies, for the
 * timed CPU baseline.  TEST/BASELINE INFRASTRUCTURE ONLY.
 *
 * Units: the reference's kick is v += TIME_STEP*G*m*d/((d^2+s^2)*d) and its
 * drift x += TIME_STEP*v/TO_METERS (Interaction.cpp:144-182, 346-381).  The
 * staged Constants.h sets TO_METERS = 1 and TIME_STEP = 1, this file sets
 * G = dt^2 (dt from the environment variable NBX_REF_DT, else NBX_DT), and the
 * velocities handed in are dt*v, which makes one reference step one kick-drift
 * step of length dt with G = 1.
 *
 * Modes (argv[1]):
 *   full   <in> <steps> <warmup>             Interaction::interactBodies per step
 *   sample <in> <steps> <warmup> <k> <seed>  the reference's serial tree build
 *          over ALL bodies (Interaction.cpp:306-313), timed once; then per step
 *          the reference's parallel force loop (:330-336) over k sampled bodies
 *          and its update; the estimated step is build + force * n/k + update.
 * Input file: int32 n, then float32 x,y,z,vx,vy,vz,m arrays; theta, eps from
 * the staged Constants via the extern globals below.
 */
#define private public
#include "Interaction.h"
#undef private

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

double G = (NBX_DT) * (NBX_DT);
int NUM_BODIES = 0;
int NUM_SUNS = 0;
double SYSTEM_SIZE = 1.0;
double SYSTEM_THICKNESS = 0.0;
double INNER_BOUND = 0.0;
double SOFTENING = 0.0;
double SOLAR_MASS = 1.0;
double EXTRA_MASS = 0.0;
double MAX_DISTANCE = 0.5;
int TIME_STEP = 1;
int STEP_COUNT = 1;
bool BINARY = false;
double BINARY_SEPARATION = 0.0;
structlog LOGCFG = {};

static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s full|sample <in> <steps> <warmup> [k seed]\n", argv[0]);
        return 2;
    }
    const bool sample = std::strcmp(argv[1], "sample") == 0;
    if (const char *e = std::getenv("NBX_REF_DT")) {
        const double dt = std::atof(e);
        if (dt > 0.0) G = dt * dt;
    }
    FILE *f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    int n = 0;
    float hdr[2];
    if (std::fread(&n, sizeof(int), 1, f) != 1) return 3;
    if (std::fread(hdr, sizeof(float), 2, f) != 2) return 3;  // theta, eps
    std::vector<float> a(7 * (size_t)n);
    if (std::fread(a.data(), sizeof(float), a.size(), f) != a.size()) return 3;
    std::fclose(f);
    const int steps = std::atoi(argv[3]), warmup = std::atoi(argv[4]);
    const int k = sample && argc > 5 ? std::atoi(argv[5]) : n;
    const unsigned seed = sample && argc > 6 ? (unsigned)std::atoi(argv[6]) : 1u;
    NUM_BODIES = n;
    MAX_DISTANCE = hdr[0];
    SOFTENING = hdr[1];
    Body *suns = new Body[1];
    Body *bods = new Body[n];
    for (int i = 0; i < n; i++) {
        bods[i].position.x = a[i];
        bods[i].position.y = a[(size_t)n + i];
        bods[i].position.z = a[2 * (size_t)n + i];
        bods[i].velocity.x = a[3 * (size_t)n + i];
        bods[i].velocity.y = a[4 * (size_t)n + i];
        bods[i].velocity.z = a[5 * (size_t)n + i];
        bods[i].mass = a[6 * (size_t)n + i];
        bods[i].acceleration.x = bods[i].acceleration.y = bods[i].acceleration.z = 0.0;
    }
    Interaction handler(false);
    LOGCFG.level = ERROR;
    LOGCFG.headers = false;
    std::printf("{\"threads\": %d, \"n\": %d, \"mode\": \"%s\", \"steps\": [", omp_get_max_threads(), n,
                sample ? "sample" : "full");
    std::mt19937 rng(seed);
    Tree *tree = nullptr;
    double t_build = 0.0;
    if (sample) {
        /* Interaction.cpp:256-313: bbox-sized root, serial inserts; built once,
         * its time is charged to every step */
        double t0 = now();
        double xMin = 0, xMax = 0, yMin = 0, yMax = 0, zMin = 0, zMax = 0;
        for (int i = 0; i < n; i++) {
            const Body *b = &bods[i];
            xMin = b->position.x < xMin ? b->position.x : xMin;
            yMin = b->position.y < yMin ? b->position.y : yMin;
            zMin = b->position.z < zMin ? b->position.z : zMin;
            xMax = b->position.x > xMax ? b->position.x : xMax;
            yMax = b->position.y > yMax ? b->position.y : yMax;
            zMax = b->position.z > zMax ? b->position.z : zMax;
        }
        double span = std::fabs(xMax - xMin);
        span = std::fabs(yMax - yMin) > span ? std::fabs(yMax - yMin) : span;
        span = std::fabs(zMax - zMin) > span ? std::fabs(zMax - zMin) : span;
        tree = new Tree(Octant(0., 0., 0., span));
        for (int i = 0; i < n; i++)
            if (tree->getOctant().contains(bods[i].position)) tree->insert(&bods[i]);
        t_build = now() - t0;
    }
    for (int s = 0; s < warmup + steps; s++) {
        double t0 = now(), tb = 0, tf = 0, tu = 0;
        if (!sample) {
            handler.interactBodies(suns, bods, false);
            tb = now() - t0;
        } else {
            tb = t_build;
            std::vector<int> idx(k);
            for (int j = 0; j < k; j++) idx[j] = (int)(rng() % (unsigned)n);
            double t1 = now();
            /* Interaction.cpp:330-336 on the sampled bodies */
#pragma omp parallel for
            for (int j = 0; j < k; j++) {
                Body *b = &bods[idx[j]];
                if (tree->getOctant().contains(b->position)) handler.treeInteraction(tree, b);
            }
            tf = now() - t1;
            double t2 = now();
            handler.updateBodies(suns, bods);
            tu = now() - t2;
        }
        if (s >= warmup)
            std::printf("%s[%.6f, %.6f, %.6f]", s > warmup ? ", " : "", tb, tf * ((double)n / k), tu);
        std::fflush(stdout);
    }
    delete tree;
    std::printf("]}\n");
    return 0;
}
