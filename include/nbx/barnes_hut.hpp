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
//                           update(step) (BarnesHut.cu:195-301).  Its
//                           BarnesHut(parameters) constructor builds the
//                           reference's disk model, and its h_x.. / time_*
//                           members are raw arrays as in BarnesHut.cuh:100-125.
//
// include/nbx/BarnesHut.cuh and include/nbx/KernelsWrapper.cuh bring the two
// classes into the global namespace under the reference's header names, so a
// driver written against the reference (3D/CUDA/CUDA_NBody/src/main.cu) builds
// by pointing its two includes there and linking libnbx.
//
// Unlike the reference, every call is checked: a failing status throws
// nbx::Error with the library's message (the reference printed and waited on
// getchar(), BarnesHut.cu:3-10).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
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
    // P: the reference's SimulationParameters or nbx::SimulationParameters
    template <class P>
    KernelsWrapper(nbx_ctx *c, const P &p, cudaStream_t s = nullptr)
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

namespace detail {

// Counter-based SplitMix64 stream: draw `draw` of body i under `seed` (the
// generator of nns_gb300/ic.py, so host codes and the Python side agree).
inline uint64_t mix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double uniform01(uint64_t seed, uint64_t i, uint64_t draw) {
    const uint64_t base = mix64(seed * 0x9E3779B97F4A7C15ull + draw * 0xD1B54A32D192ED03ull);
    return (double)(mix64(base + (i + 1) * 0x9E3779B97F4A7C15ull) >> 11) * (1.0 / 9007199254740992.0);
}

// The reference's SimulationParameters (Constants.h:4-22) carries no MAC or
// softening: its kernels hard-code theta = 1.5 and eps^2 = 0.0025
// (Kernels.cu:17-18).  A parameter struct that has theta_ref / eps_squared
// (nbx::SimulationParameters) sets them.
template <class P, class = void>
struct has_mac : std::false_type {};
template <class P>
struct has_mac<P, std::void_t<decltype(std::declval<const P &>().theta_ref),
                              decltype(std::declval<const P &>().eps_squared)>> : std::true_type {};
template <class P>
float theta_ref_of(const P &p) {
    if constexpr (has_mac<P>::value) return (float)p.theta_ref;
    else return 1.5f;
}
template <class P>
float eps_squared_of(const P &p) {
    if constexpr (has_mac<P>::value) return (float)p.eps_squared;
    else return 0.0025f;
}

}  // namespace detail

// Initial conditions of the reference's host class, restated with the seeded
// generator above (the reference draws from an unseeded std::default_random_engine):
//
// disk_model -- BarnesHut::diskModel (BarnesHut.cu:356-415), the reference
//   constructor's choice: a 1e5 central mass at the origin; n-1 bodies of mass
//   2e5/n, radius in [1.5, 12), azimuth in [0, 2 pi), z = +-i*1e-7, clockwise
//   circular speed sqrt(1e5/r) (vx = v sin(phi), vy = -v cos(phi)).
inline void disk_model(int n, uint64_t seed, float *x, float *y, float *z, float *vx, float *vy, float *vz,
                       float *m) {
    const double pi = 3.14159265358979323846, sun = 100000.0;
    for (int i = 0; i < n; i++) {
        x[i] = y[i] = z[i] = vx[i] = vy[i] = vz[i] = 0.f;
        if (i == 0) {
            m[i] = (float)sun;
            continue;
        }
        const double th = 2 * pi * detail::uniform01(seed, i, 0), r = 1.5 + 10.5 * detail::uniform01(seed, i, 1);
        m[i] = (float)(2 * sun / n);
        x[i] = (float)(r * std::cos(th));
        y[i] = (float)(r * std::sin(th));
        z[i] = (float)((i % 2 == 0 ? 1e-7 : -1e-7) * i);
        const double v = std::sqrt(sun / r);
        vx[i] = (float)(v * std::sin(th));
        vy[i] = (float)(-v * std::cos(th));
    }
}

// plummer_model -- BarnesHut::plummerModel (BarnesHut.cu:304-354; present in the
//   reference but not called): unit masses, r = a / sqrt(u^-2/3 - 1) in the x-y
//   plane, z = +-i*1e-3, in-plane speed 100 q sqrt(2) (1 + r^2)^-1/4 with q by
//   rejection on q^2 (1 - q^2)^3.5 (bound 0.1).
inline void plummer_model(int n, uint64_t seed, float *x, float *y, float *z, float *vx, float *vy, float *vz,
                          float *m) {
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < n; i++) {
        const double phi = 2 * pi * detail::uniform01(seed, i, 0);
        const double u = std::max(detail::uniform01(seed, i, 1), 1e-12);
        const double r = 1.0 / std::sqrt(std::pow(u, -0.666666) - 1.0);
        m[i] = 1.f;
        x[i] = (float)(r * std::cos(phi));
        y[i] = (float)(r * std::sin(phi));
        z[i] = (float)((i % 2 == 0 ? 1e-3 : -1e-3) * i);
        double q = 0.0;
        for (int d = 2; d < 4000; d += 2) {
            const double qq = detail::uniform01(seed, i, d), tt = 0.1 * detail::uniform01(seed, i, d + 1);
            if (tt <= qq * qq * std::pow(1 - qq * qq, 3.5)) {
                q = qq;
                break;
            }
        }
        const double v = 100 * q * std::sqrt(2.0) * std::pow(1 + r * r, -0.25);
        const double ph2 = 2 * pi * detail::uniform01(seed, i, 4001);
        vx[i] = (float)(v * std::cos(ph2));
        vy[i] = (float)(v * std::sin(ph2));
        vz[i] = 0.f;
    }
}

// The reference's host class (BarnesHut.cuh:18-127) over libnbx.  Its public
// members keep the reference's types: h_x .. h_vz are host arrays of numNodes
// floats refreshed after every step, time_* are arrays of `iterations` floats
// indexed by the step number (BarnesHut.cu:195-301), so code written against
// the reference (its main.cu) compiles and runs unchanged.
class BarnesHut {
  public:
    SimulationParameters parameters;
    KernelsWrapper KernelHandler;
    nbx_ctx *ctx = nullptr;
    int step = 0, numParticles = 0, numNodes = 0, iterations = 0;
    bool timeKernels = true;
    float *h_x = nullptr, *h_y = nullptr, *h_z = nullptr, *h_vx = nullptr, *h_vy = nullptr, *h_vz = nullptr;
    float *h_mass = nullptr;
    float *d_x = nullptr, *d_y = nullptr, *d_z = nullptr, *d_vx = nullptr, *d_vy = nullptr, *d_vz = nullptr;
    float *d_ax = nullptr, *d_ay = nullptr, *d_az = nullptr, *d_mass = nullptr;
    float *d_min_x = nullptr, *d_max_x = nullptr, *d_min_y = nullptr, *d_max_y = nullptr, *d_min_z = nullptr,
          *d_max_z = nullptr;
    int *d_index = nullptr, *d_child = nullptr, *d_start = nullptr, *d_sorted = nullptr, *d_count = nullptr,
        *d_mutex = nullptr;
    // per-step kernel times in ms (BarnesHut.cuh:100-125), `iterations` entries
    float *time_resetArrays = nullptr, *time_computeBoundingBox = nullptr, *time_buildTree = nullptr,
          *time_centreOfMass = nullptr, *time_sort = nullptr, *time_computeForces = nullptr, *time_update = nullptr,
          *time_copyDeviceToHost = nullptr, *time_all = nullptr;

    // BarnesHut(parameters) as in the reference (BarnesHut.cu:12-119): the bodies
    // are the reference's disk model (disk_model above, seed 20261203).  P is the
    // reference's SimulationParameters or nbx::SimulationParameters.
    template <class P>
    explicit BarnesHut(const P &p, uint64_t seed = 20261203ull) {
        const int n = p.numberOfParticles;
        if (n < 1) throw Error(NBX_ERR_ARG, "BarnesHut: numberOfParticles < 1");
        std::vector<float> b(7 * (size_t)n);
        float *a = b.data();
        disk_model(n, seed, a, a + n, a + 2 * (size_t)n, a + 3 * (size_t)n, a + 4 * (size_t)n, a + 5 * (size_t)n,
                   a + 6 * (size_t)n);
        init(p, a, a + n, a + 2 * (size_t)n, a + 3 * (size_t)n, a + 4 * (size_t)n, a + 5 * (size_t)n,
             a + 6 * (size_t)n);
    }

    // Bodies from the caller (host arrays of numberOfParticles floats).
    template <class P>
    BarnesHut(const P &p, const float *x, const float *y, const float *z, const float *vx, const float *vy,
              const float *vz, const float *mass) {
        init(p, x, y, z, vx, vy, vz, mass);
    }

    ~BarnesHut() { release(); }

    BarnesHut(const BarnesHut &) = delete;
    BarnesHut &operator=(const BarnesHut &) = delete;

    // One step, in the order of BarnesHut::update (BarnesHut.cu:195-301); the
    // times are recorded at index `s` (steps beyond `iterations` are not recorded).
    void update(int s) {
        auto &K = KernelHandler;
        const int n = numParticles, m = numNodes;
        const bool t = timeKernels;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, K.stream);
        const float t_reset = K.resetArrays(d_mutex, d_x, d_y, d_z, d_mass, d_count, d_start, d_sorted, d_child,
                                            d_index, d_min_x, d_max_x, d_min_y, d_max_y, d_min_z, d_max_z, n, m, t);
        const float t_bbox = K.computeBoundingBox(d_mutex, d_x, d_y, d_z, d_min_x, d_max_x, d_min_y, d_max_y,
                                                  d_min_z, d_max_z, n, t);
        const float t_build = K.buildTree(d_x, d_y, d_z, d_mass, d_count, d_start, d_child, d_index, d_min_x,
                                          d_max_x, d_min_y, d_max_y, d_min_z, d_max_z, n, m, t);
        const float t_com = K.centreOfMass(d_x, d_y, d_z, d_mass, d_index, n, t);
        const float t_sort = K.sort(d_count, d_start, d_sorted, d_child, d_index, n, t);
        const float t_forces = K.computeForces(d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, d_mass, d_sorted,
                                               d_child, d_min_x, d_max_x, n, parameters.gravity, t);
        const float t_update = K.update(d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, n, parameters.timestep,
                                        parameters.dampening, t);
        cudaEvent_t c0, c1;
        cudaEventCreate(&c0);
        cudaEventCreate(&c1);
        cudaEventRecord(c0, K.stream);
        const size_t nb = (size_t)n * sizeof(float);
        cudaMemcpyAsync(h_x, d_x, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_y, d_y, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_z, d_z, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_vx, d_vx, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_vy, d_vy, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaMemcpyAsync(h_vz, d_vz, nb, cudaMemcpyDeviceToHost, K.stream);
        cudaEventRecord(c1, K.stream);
        cudaEventRecord(b, K.stream);
        const cudaError_t e = cudaEventSynchronize(b);
        float t_copy = 0.f, t_all = 0.f;
        cudaEventElapsedTime(&t_copy, c0, c1);
        cudaEventElapsedTime(&t_all, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaEventDestroy(c0);
        cudaEventDestroy(c1);
        if (e != cudaSuccess) throw Error(NBX_ERR_CUDA, std::string("BarnesHut::update: ") + cudaGetErrorString(e));
        if (s >= 0 && s < iterations) {
            time_resetArrays[s] = t_reset;
            time_computeBoundingBox[s] = t_bbox;
            time_buildTree[s] = t_build;
            time_centreOfMass[s] = t_com;
            time_sort[s] = t_sort;
            time_computeForces[s] = t_forces;
            time_update[s] = t_update;
            time_copyDeviceToHost[s] = t_copy;
            time_all[s] = t_all;
        }
        step++;
    }

    // Largest |coordinate| of the current host copy (BarnesHut.cu:417-449).
    float getSystemSize() const {
        float s = 0.f;
        for (int i = 0; i < numParticles; i++) {
            const float v[3] = {std::fabs(h_x[i]), std::fabs(h_y[i]), std::fabs(h_z[i])};
            for (float a : v) s = a > s ? a : s;
        }
        return s;
    }

  private:
    template <class P>
    void init(const P &p, const float *x, const float *y, const float *z, const float *vx, const float *vy,
              const float *vz, const float *mass) {
        parameters.timeKernels = p.timeKernels;
        parameters.iterations = p.iterations;
        parameters.numberOfParticles = p.numberOfParticles;
        parameters.timestep = p.timestep;
        parameters.gravity = p.gravity;
        parameters.dampening = p.dampening;
        parameters.gridSize = p.gridSize;
        parameters.blockSize = p.blockSize;
        parameters.warp = p.warp;
        parameters.stackSize = p.stackSize;
        parameters.renderInterval = p.renderInterval;
        parameters.theta_ref = detail::theta_ref_of(p);
        parameters.eps_squared = detail::eps_squared_of(p);
        numParticles = p.numberOfParticles;
        numNodes = 2 * p.numberOfParticles + 12000;  // BarnesHut.cu:18
        iterations = p.iterations > 0 ? p.iterations : 0;
        timeKernels = p.timeKernels;
        if (numParticles < 1) throw Error(NBX_ERR_ARG, "BarnesHut: numberOfParticles < 1");
        try {
            nbx_params np;
            nbx_params_default(&np);
            np.max_bodies = numParticles;
            np.theta_ref = parameters.theta_ref;
            np.eps2 = parameters.eps_squared;
            np.dt = parameters.timestep;
            np.dampening = parameters.dampening;
            np.gravity = parameters.gravity;
            np.block_size = parameters.blockSize;
            np.grid_size = parameters.gridSize;
            check(nbx_create(&np, &ctx), "nbx_create");
            KernelHandler = KernelsWrapper(ctx, parameters);
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
            for (int k = 0; k < 7; k++)
                if (cudaMemcpy(dst[k], src[k], nb, cudaMemcpyHostToDevice) != cudaSuccess)
                    throw Error(NBX_ERR_CUDA, "BarnesHut: cudaMemcpy");
            float **ha[] = {&h_x, &h_y, &h_z, &h_vx, &h_vy, &h_vz, &h_mass};
            for (float **h : ha) *h = new float[m]();
            const float *hs[] = {x, y, z, vx, vy, vz, mass};
            for (int k = 0; k < 7; k++) std::copy(hs[k], hs[k] + numParticles, *ha[k]);
            float **ta[] = {&time_resetArrays, &time_computeBoundingBox, &time_buildTree, &time_centreOfMass,
                            &time_sort, &time_computeForces, &time_update, &time_copyDeviceToHost, &time_all};
            for (float **t : ta) *t = new float[iterations > 0 ? iterations : 1]();
        } catch (...) {
            release();
            throw;
        }
    }

    void release() {
        void *ptrs[] = {d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, d_mass, d_min_x, d_max_x, d_min_y,
                        d_max_y, d_min_z, d_max_z, d_index, d_mutex, d_child, d_start, d_sorted, d_count};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        float *hs[] = {h_x, h_y, h_z, h_vx, h_vy, h_vz, h_mass, time_resetArrays, time_computeBoundingBox,
                       time_buildTree, time_centreOfMass, time_sort, time_computeForces, time_update,
                       time_copyDeviceToHost, time_all};
        for (float *h : hs) delete[] h;
        if (ctx) nbx_destroy(ctx);
        ctx = nullptr;
    }

    template <typename T>
    void alloc(T **p, size_t n) {
        if (cudaMalloc((void **)p, n * sizeof(T)) != cudaSuccess) throw Error(NBX_ERR_NOMEM, "cudaMalloc");
        cudaMemset(*p, 0, n * sizeof(T));
    }
};

}  // namespace nbx
