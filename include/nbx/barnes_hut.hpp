// barnes_hut.hpp -- header-only C++ host classes over the C ABI (include/nbx.h)
// with the interface of the reference's host side, so that code written
// against 3D/CUDA/CUDA_NBody/include/KernelsWrapper.cuh and BarnesHut.cuh can
// switch to libnbx by swapping includes:
//
//   nbx::KernelsWrapper  -- same seven methods, argument order and array
//                           semantics as KernelsWrapper (KernelsWrapper.cuh:28-48),
//                           each returning elapsed ms (0 when timing == false).
//   nbx::BarnesHut       -- owns the SoA device arrays of numNodes = 2N+12000
//                           entries (BarnesHut.cu:18) and runs one step per
//                           update(step) (BarnesHut.cu:195-301).
//
// Unlike the reference, every call is checked: a failing status throws
// nbx::Error with the library's message (the reference printed and waited on
// getchar(), BarnesHut.cu:3-10).
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../nbx.h"

namespace nbx {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc, const char *where, nbx_ctx *ctx = nullptr) {
    if (rc != NBX_OK) {
        std::string msg = std::string(where) + ": " + nbx_status_string(rc);
        if (ctx) msg += std::string(" (") + nbx_last_error(ctx) + ")";
        throw Error(rc, msg);
    }
}

// Mirrors SimulationParameters (3D/CUDA/CUDA_NBody/include/Constants.h:4-22)
// plus the MAC and softening constants that the reference hard-codes
// (Kernels.cu:17-18).
struct SimulationParameters {
    bool timeKernels = true;
    int iterations = 100;
    int numberOfParticles = 524288;
    float timestep = 0.001f;
    float gravity = 1.0f;
    float dampening = 1.0f;
    int gridSize = 1024;
    int blockSize = 256;
    int warp = 32;
    int stackSize = 64;
    int renderInterval = 10;
    float theta_ref = 1.5f;     // Kernels.cu:18
    float eps_squared = 0.0025f;  // Kernels.cu:17
};

class KernelsWrapper {
  public:
    nbx_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;
    int gridSize = 0, blockSize = 0, warp = 32, stackSize = 64;

    KernelsWrapper() = default;
    KernelsWrapper(nbx_ctx *c, const SimulationParameters &p, cudaStream_t s = nullptr)
        : ctx(c), stream(s), gridSize(p.gridSize), blockSize(p.blockSize), warp(p.warp), stackSize(p.stackSize) {}

    float resetArrays(int *mutex, float *x, float *y, float *z, float *mass, int *count, int *start, int *sorted,
                      int *child, int *index, float *minX, float *maxX, float *minY, float *maxY, float *minZ,
                      float *maxZ, int n, int m, bool timing = false) {
        float ms = 0.f;
        check(nbx_reset_arrays(ctx, mutex, x, y, z, mass, count, start, sorted, child, index, minX, maxX, minY, maxY,
                               minZ, maxZ, n, m, stream, timing ? &ms : nullptr),
              "resetArrays", ctx);
        return ms;
    }
    float computeBoundingBox(int *mutex, float *x, float *y, float *z, float *minX, float *maxX, float *minY,
                             float *maxY, float *minZ, float *maxZ, int n, bool timing = false) {
        float ms = 0.f;
        check(nbx_compute_bounding_box(ctx, mutex, x, y, z, minX, maxX, minY, maxY, minZ, maxZ, n, stream,
                                       timing ? &ms : nullptr),
              "computeBoundingBox", ctx);
        return ms;
    }
    float buildTree(float *x, float *y, float *z, float *mass, int *count, int *start, int *child, int *index,
                    float *minX, float *maxX, float *minY, float *maxY, float *minZ, float *maxZ, int n, int m,
                    bool timing = false) {
        float ms = 0.f;
        check(nbx_build_tree(ctx, x, y, z, mass, count, start, child, index, minX, maxX, minY, maxY, minZ, maxZ, n,
                             m, stream, timing ? &ms : nullptr),
              "buildTree", ctx);
        return ms;
    }
    float centreOfMass(float *x, float *y, float *z, float *mass, int *index, int n, bool timing = false) {
        float ms = 0.f;
        check(nbx_centre_of_mass(ctx, x, y, z, mass, index, n, stream, timing ? &ms : nullptr), "centreOfMass",
              ctx);
        return ms;
    }
    float sort(int *count, int *start, int *sorted, int *child, int *index, int n, bool timing = false) {
        float ms = 0.f;
        check(nbx_sort(ctx, count, start, sorted, child, index, n, stream, timing ? &ms : nullptr), "sort", ctx);
        return ms;
    }
    float computeForces(float *x, float *y, float *z, float *vx, float *vy, float *vz, float *ax, float *ay,
                        float *az, float *mass, int *sorted, int *child, float *minX, float *maxX, int n, float g,
                        bool timing = false) {
        float ms = 0.f;
        check(nbx_compute_forces(ctx, x, y, z, vx, vy, vz, ax, ay, az, mass, sorted, child, minX, maxX, n, g,
                                 stream, timing ? &ms : nullptr),
              "computeForces", ctx);
        return ms;
    }
    float update(float *x, float *y, float *z, float *vx, float *vy, float *vz, float *ax, float *ay, float *az,
                 int n, float dt, float d, bool timing = false) {
        float ms = 0.f;
        check(nbx_update(ctx, x, y, z, vx, vy, vz, ax, ay, az, n, dt, d, stream, timing ? &ms : nullptr), "update",
              ctx);
        return ms;
    }
};

class BarnesHut {
  public:
    SimulationParameters parameters;
    KernelsWrapper KernelHandler;
    nbx_ctx *ctx = nullptr;
    int step = 0, numParticles = 0, numNodes = 0;
    bool timeKernels = true;
    std::vector<float> h_x, h_y, h_z, h_vx, h_vy, h_vz, h_mass;
    float *d_x = nullptr, *d_y = nullptr, *d_z = nullptr, *d_vx = nullptr, *d_vy = nullptr, *d_vz = nullptr;
    float *d_ax = nullptr, *d_ay = nullptr, *d_az = nullptr, *d_mass = nullptr;
    float *d_min_x = nullptr, *d_max_x = nullptr, *d_min_y = nullptr, *d_max_y = nullptr, *d_min_z = nullptr,
          *d_max_z = nullptr;
    int *d_index = nullptr, *d_child = nullptr, *d_start = nullptr, *d_sorted = nullptr, *d_count = nullptr,
        *d_mutex = nullptr;
    // per-step kernel times (BarnesHut.cuh:100-125)
    std::vector<float> time_resetArrays, time_computeBoundingBox, time_buildTree, time_centreOfMass, time_sort,
        time_computeForces, time_update, time_copyDeviceToHost, time_all;

    // Bodies come from the caller (the reference hard-wires diskModel, BarnesHut.cu:105).
    BarnesHut(const SimulationParameters &p, const float *x, const float *y, const float *z, const float *vx,
              const float *vy, const float *vz, const float *mass)
        : parameters(p), numParticles(p.numberOfParticles), numNodes(2 * p.numberOfParticles + 12000),
          timeKernels(p.timeKernels) {
        nbx_params np;
        nbx_params_default(&np);
        np.max_bodies = numParticles;
        np.theta_ref = p.theta_ref;
        np.eps2 = p.eps_squared;
        np.dt = p.timestep;
        np.dampening = p.dampening;
        np.gravity = p.gravity;
        np.block_size = p.blockSize;
        np.grid_size = p.gridSize;
        check(nbx_create(&np, &ctx), "nbx_create");
        KernelHandler = KernelsWrapper(ctx, p);
        const size_t m = (size_t)numNodes;
        float **fa[] = {&d_x, &d_y, &d_z, &d_vx, &d_vy, &d_vz, &d_ax, &d_ay, &d_az, &d_mass};
        for (float **a : fa) alloc(a, m);
        float **bb[] = {&d_min_x, &d_max_x, &d_min_y, &d_max_y, &d_min_z, &d_max_z};
        for (float **a : bb) alloc(a, 1);
        alloc(&d_index, 1);
        alloc(&d_mutex, 1);
        alloc(&d_child, 8 * m);
        alloc(&d_start, m);
        alloc(&d_sorted, m);
        alloc(&d_count, m);
        const size_t nb = (size_t)numParticles * sizeof(float);
        const float *src[] = {x, y, z, vx, vy, vz, mass};
        float *dst[] = {d_x, d_y, d_z, d_vx, d_vy, d_vz, d_mass};
        for (int k = 0; k < 7; k++) cudaMemcpy(dst[k], src[k], nb, cudaMemcpyHostToDevice);
        h_x.resize(numParticles);
        h_y.resize(numParticles);
        h_z.resize(numParticles);
        h_vx.resize(numParticles);
        h_vy.resize(numParticles);
        h_vz.resize(numParticles);
    }

    ~BarnesHut() {
        void *ptrs[] = {d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, d_mass, d_min_x, d_max_x, d_min_y,
                        d_max_y, d_min_z, d_max_z, d_index, d_mutex, d_child, d_start, d_sorted, d_count};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        if (ctx) nbx_destroy(ctx);
    }

    BarnesHut(const BarnesHut &) = delete;
    BarnesHut &operator=(const BarnesHut &) = delete;

    // One step, in the order of BarnesHut::update (BarnesHut.cu:195-301).
    void update(int s) {
        (void)s;
        auto &K = KernelHandler;
        const int n = numParticles, m = numNodes;
        const bool t = timeKernels;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, K.stream);
        time_resetArrays.push_back(K.resetArrays(d_mutex, d_x, d_y, d_z, d_mass, d_count, d_start, d_sorted, d_child,
                                                 d_index, d_min_x, d_max_x, d_min_y, d_max_y, d_min_z, d_max_z, n,
                                                 m, t));
        time_computeBoundingBox.push_back(K.computeBoundingBox(d_mutex, d_x, d_y, d_z, d_min_x, d_max_x, d_min_y,
                                                               d_max_y, d_min_z, d_max_z, n, t));
        time_buildTree.push_back(K.buildTree(d_x, d_y, d_z, d_mass, d_count, d_start, d_child, d_index, d_min_x,
                                             d_max_x, d_min_y, d_max_y, d_min_z, d_max_z, n, m, t));
        time_centreOfMass.push_back(K.centreOfMass(d_x, d_y, d_z, d_mass, d_index, n, t));
        time_sort.push_back(K.sort(d_count, d_start, d_sorted, d_child, d_index, n, t));
        time_computeForces.push_back(K.computeForces(d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, d_mass,
                                                     d_sorted, d_child, d_min_x, d_max_x, n, parameters.gravity, t));
        time_update.push_back(K.update(d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, n, parameters.timestep,
                                       parameters.dampening, t));
        cudaEvent_t c0, c1;
        cudaEventCreate(&c0);
        cudaEventCreate(&c1);
        cudaEventRecord(c0, K.stream);
        const size_t nb = (size_t)n * sizeof(float);
        cudaMemcpyAsync(h_x.data(), d_x, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_y.data(), d_y, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_z.data(), d_z, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_vx.data(), d_vx, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_vy.data(), d_vy, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_vz.data(), d_vz, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaEventRecord(c1, K.stream);
        cudaEventRecord(b, K.stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c0, c1);
        time_copyDeviceToHost.push_back(ms);
        cudaEventElapsedTime(&ms, a, b);
        time_all.push_back(ms);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaEventDestroy(c0);
        cudaEventDestroy(c1);
        step++;
    }

    float getSystemSize() const {  // BarnesHut.cu:417-449
        float s = 0.f;
        for (int i = 0; i < numParticles; i++) {
            const float v[3] = {h_x.empty() ? 0.f : h_x[i], h_y.empty() ? 0.f : h_y[i], h_z.empty() ? 0.f : h_z[i]};
            for (float a : v) s = a < 0 ? (-a > s ? -a : s) : (a > s ? a : s);
        }
        return s;
    }

  private:
    template <typename T>
    void alloc(T **p, size_t n) {
        if (cudaMalloc((void **)p, n * sizeof(T)) != cudaSuccess) throw Error(NBX_ERR_NOMEM, "cudaMalloc");
        cudaMemset(*p, 0, n * sizeof(T));
    }
};

}  // namespace nbx
