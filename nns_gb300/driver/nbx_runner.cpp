// nbx_runner -- command-line driver with the reference driver's flags and
// report (3D/CUDA/CUDA_NBody/src/main.cu:19-190), running the reference's
// BarnesHut::update flow through libnbx (include/nbx/barnes_hut.hpp).
//
//   -i, --iterations N      number of iterations (100)
//   -n, --particles N       number of particles (524288)
//   -b, --blocksize N       block size hint (256)
//   -g, --gridsize N        grid size hint (1024)
//   -R, --renderinterval N  render interval (10)
//   -r, --render            write a frame every renderinterval steps to images/StepNNNNN.ppm
//                           (Renderer::createFrame, Renderer.cpp:37-161, through nbx_render_frame)
//   -v                      verbosity (repeat)
//   --model ref-disk|ref-plummer|disk|plummer   initial conditions (ref-disk and
//                           ref-plummer: the recipes of BarnesHut::diskModel and
//                           BarnesHut::plummerModel, BarnesHut.cu:304-415)
//   --theta-ref X --eps2 X  MAC constant and squared softening (Kernels.cu:17-18 defaults)
//   --seed N
#include <sys/stat.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nbx/barnes_hut.hpp"

namespace {

// Draw `draw` of body i under `seed` (the generator of nns_gb300/ic.py).
double uniform(uint64_t seed, uint64_t i, uint64_t draw) { return nbx::detail::uniform01(seed, i, draw); }

struct Bodies {
    std::vector<float> x, y, z, vx, vy, vz, m;
    explicit Bodies(int n) : x(n), y(n), z(n), vx(n), vy(n), vz(n), m(n) {}
};

// The reference constructor's disk and its Plummer recipe (nbx::disk_model,
// nbx::plummer_model in include/nbx/barnes_hut.hpp).
Bodies ref_disk(int n, uint64_t seed) {
    Bodies b(n);
    nbx::disk_model(n, seed, b.x.data(), b.y.data(), b.z.data(), b.vx.data(), b.vy.data(), b.vz.data(), b.m.data());
    return b;
}

Bodies ref_plummer(int n, uint64_t seed) {
    Bodies b(n);
    nbx::plummer_model(n, seed, b.x.data(), b.y.data(), b.z.data(), b.vx.data(), b.vy.data(), b.vz.data(),
                       b.m.data());
    return b;
}

// The star + disk workload (mass-1 star, disk bodies of mass 1e-6, r in [0.1, 1]).
Bodies star_disk(int n, uint64_t seed) {
    Bodies b(n);
    const double pi = 3.14159265358979323846;
    b.m[0] = 1.f;
    for (int i = 1; i < n; i++) {
        const uint64_t k = (uint64_t)(i - 1);
        const double r = 0.1 + 0.9 * uniform(seed, k, 0), ph = 2 * pi * uniform(seed, k, 1);
        const double u1 = uniform(seed, k, 2), u2 = uniform(seed, k, 3);
        const double g = std::sqrt(-2.0 * std::log1p(-u1)) * std::cos(2 * pi * u2);
        const double v = std::sqrt(1.0 / r);
        b.x[i] = (float)(r * std::cos(ph));
        b.y[i] = (float)(r * std::sin(ph));
        b.z[i] = (float)(0.01 * r * g);
        b.vx[i] = (float)(v * std::sin(ph));
        b.vy[i] = (float)(-v * std::cos(ph));
        b.m[i] = 1e-6f;
    }
    return b;
}

Bodies plummer(int n, uint64_t seed) {
    Bodies b(n);
    const double pi = 3.14159265358979323846, umax = std::pow(1.0 + 1.0 / 400.0, -1.5);
    for (int i = 0; i < n; i++) {
        const double u = std::max(uniform(seed, i, 0) * umax, 1e-300);
        const double r = 1.0 / std::sqrt(std::pow(u, -2.0 / 3.0) - 1.0);
        const double ct = 2 * uniform(seed, i, 1) - 1, st = std::sqrt(std::max(0.0, 1 - ct * ct));
        const double ph = 2 * pi * uniform(seed, i, 2);
        b.x[i] = (float)(r * st * std::cos(ph));
        b.y[i] = (float)(r * st * std::sin(ph));
        b.z[i] = (float)(r * ct);
        double q = 0;
        for (int d = 3; d < 4000; d += 2) {
            const double qq = uniform(seed, i, d), tt = 0.1 * uniform(seed, i, d + 1);
            if (tt < qq * qq * std::pow(1 - qq * qq, 3.5)) {
                q = qq;
                break;
            }
        }
        const double v = q * std::sqrt(2.0) * std::pow(1 + r * r, -0.25);
        const double ct2 = 2 * uniform(seed, i, 1001) - 1, st2 = std::sqrt(std::max(0.0, 1 - ct2 * ct2));
        const double ph2 = 2 * pi * uniform(seed, i, 1002);
        b.vx[i] = (float)(v * st2 * std::cos(ph2));
        b.vy[i] = (float)(v * st2 * std::sin(ph2));
        b.vz[i] = (float)(v * ct2);
        b.m[i] = (float)(1.0 / n);
    }
    return b;
}

void usage() {
    std::printf("./nbx_runner [-i iterations] [-n particles] [-b blocksize] [-g gridsize] [-R renderinterval]\n"
                "             [-r] [-v...] [--model ref-disk|ref-plummer|disk|plummer] [--theta-ref X] [--eps2 X] [--seed N]\n");
}

}  // namespace

int main(int argc, char **argv) {
    nbx::SimulationParameters p;
    std::string model = "ref-disk";
    uint64_t seed = 20261203;
    int verbosity = 0;
    bool render = false;
    for (int a = 1; a < argc; a++) {
        const std::string s = argv[a];
        auto next = [&](const char *what) -> const char * {
            if (a + 1 >= argc) {
                std::fprintf(stderr, "missing value for %s\n", what);
                std::exit(2);
            }
            return argv[++a];
        };
        if (s == "-h" || s == "--help") {
            usage();
            return 0;
        } else if (s == "-i" || s == "--iterations") p.iterations = std::atoi(next("-i"));
        else if (s == "-n" || s == "--particles") p.numberOfParticles = std::atoi(next("-n"));
        else if (s == "-b" || s == "--blocksize") p.blockSize = std::atoi(next("-b"));
        else if (s == "-g" || s == "--gridsize") p.gridSize = std::atoi(next("-g"));
        else if (s == "-R" || s == "--renderinterval") p.renderInterval = std::atoi(next("-R"));
        else if (s == "-r" || s == "--render") render = true;
        else if (s.size() >= 2 && s[0] == '-' && s[1] == 'v' && s.find_first_not_of('v', 1) == std::string::npos)
            verbosity += (int)s.size() - 1;
        else if (s == "--model") model = next("--model");
        else if (s == "--theta-ref") p.theta_ref = (float)std::atof(next("--theta-ref"));
        else if (s == "--eps2") p.eps_squared = (float)std::atof(next("--eps2"));
        else if (s == "--seed") seed = std::strtoull(next("--seed"), nullptr, 10);
        else {
            std::fprintf(stderr, "unknown option %s\n", s.c_str());
            usage();
            return 2;
        }
    }
    const int n = p.numberOfParticles;
    if (n < 1 || p.iterations < 1) {
        usage();
        return 2;
    }
    if (model != "ref-disk" && model != "ref-plummer" && model != "disk" && model != "plummer") {
        std::fprintf(stderr, "unknown model %s\n", model.c_str());
        return 2;
    }
    Bodies b = model == "disk"          ? star_disk(n, seed)
               : model == "plummer"     ? plummer(n, seed)
               : model == "ref-plummer" ? ref_plummer(n, seed)
                                        : ref_disk(n, seed);
    try {
        nbx::BarnesHut bh(p, b.x.data(), b.y.data(), b.z.data(), b.vx.data(), b.vy.data(), b.vz.data(),
                          b.m.data());
        // main.cu:93-95: the renderer's system size is twice BarnesHut::getSystemSize()
        // of the initial state (BarnesHut.cu:417-445)
        float half = 0.f;
        for (int i = 0; i < n; i++)
            half = std::max(half, std::max(std::fabs(b.x[i]), std::max(std::fabs(b.y[i]), std::fabs(b.z[i]))));
        nbx_render_params rp;
        nbx_render_params_default(&rp);
        rp.system_size = 2.0 * (double)half;
        const size_t npix = 3 * (size_t)rp.width * (size_t)rp.height;
        float *d_accum = nullptr;
        unsigned char *d_rgb = nullptr;
        std::vector<unsigned char> h_rgb;
        if (render) {
            nbx::check(cudaMalloc(&d_accum, npix * sizeof(float)) == cudaSuccess ? NBX_OK : NBX_ERR_NOMEM,
                       "cudaMalloc");
            nbx::check(cudaMalloc(&d_rgb, npix) == cudaSuccess ? NBX_OK : NBX_ERR_NOMEM, "cudaMalloc");
            h_rgb.resize(npix);
            mkdir("images", 0755);
        }
        for (int i = 0; i < p.iterations; i++) {
            bh.update(i);
            if (verbosity > 0) std::printf("Elapsed time for step %d : %g ms\n", i, bh.time_all[i]);
            if (render && i % p.renderInterval == 0) {
                nbx_state st{};
                st.x = bh.d_x; st.y = bh.d_y; st.z = bh.d_z;
                st.vx = bh.d_vx; st.vy = bh.d_vy; st.vz = bh.d_vz;
                nbx::check(nbx_render_frame(bh.ctx, &st, n, &rp, d_accum, d_rgb, nullptr), "nbx_render_frame");
                nbx::check(cudaMemcpy(h_rgb.data(), d_rgb, npix, cudaMemcpyDeviceToHost) == cudaSuccess
                               ? NBX_OK : NBX_ERR_CUDA, "cudaMemcpy");
                char name[64];
                std::snprintf(name, sizeof(name), "images/Step%05d.ppm", i / p.renderInterval + 1);
                if (FILE *f = std::fopen(name, "wb")) {
                    std::fprintf(f, "P6\n%d %d\n255\n", rp.width, rp.height);
                    std::fwrite(h_rgb.data(), 1, npix, f);
                    std::fclose(f);
                }
                if (verbosity > 0) std::printf("Writing frame %d\n", i);
            }
        }
        if (render) {
            cudaFree(d_accum);
            cudaFree(d_rgb);
        }
        auto total = [&](const float *v) {
            double t = 0;
            for (int i = 0; i < p.iterations; i++) t += v[i];
            return t;
        };
        const double it = p.iterations;
        struct Row {
            const char *name;
            double t;
        } rows[] = {{"reset arrays", total(bh.time_resetArrays)},
                    {"compute bounding boxes", total(bh.time_computeBoundingBox)},
                    {"build tree", total(bh.time_buildTree)},
                    {"compute COM", total(bh.time_centreOfMass)},
                    {"sort", total(bh.time_sort)},
                    {"compute forces", total(bh.time_computeForces)},
                    {"update bodies", total(bh.time_update)},
                    {"copy from device to host", total(bh.time_copyDeviceToHost)}};
        std::printf("----------------------FINISHED----------------------\n");
        for (const Row &r : rows) std::printf("Time to %s: %gms\n\tper step: %gms\n", r.name, r.t, r.t / it);
        const double all = total(bh.time_all), copy = total(bh.time_copyDeviceToHost);
        std::printf("----------------------------------------------\n");
        std::printf("TOTAL TIME: %gms\n\tper step: %gms\n", all, all / it);
        std::printf("TOTAL TIME (without copying): %gms\n\tper step: %gms\n", all - copy, (all - copy) / it);
        std::printf("----------------------------------------------\n");
        std::printf("Number of particles: %d\nNumber of iterations: %d\n", n, p.iterations);
        std::printf("final position of body 1: %.9g %.9g %.9g\n", bh.h_x[n > 1 ? 1 : 0], bh.h_y[n > 1 ? 1 : 0],
                    bh.h_z[n > 1 ? 1 : 0]);
    } catch (const nbx::Error &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
