// C entry point around the reference's own renderer (3D/CUDA/CUDA_NBody/src/
// Renderer.cpp, Body.cpp, Logger.cpp compiled unmodified from the checkout) for
// the parity tests of the headless frame.  Test infrastructure only.
//
// renderClear and renderBodies (Renderer.cpp:54-129) are the reference's; the
// byte conversion of writeRender (:144-147) is applied here without its file
// output.  The constructor's log lines are silenced.
#include <iostream>
#include <vector>

#define private public
#include "Renderer.h"
#undef private

structlog LOGCFG = {};

extern "C" int ref_render(int n, const float *x, const float *y, const float *z, const float *vx, const float *vy,
                          const float *vz, int width, int height, double render_scale, double vmax, double vmin,
                          double brightness, double sharpness, int dot, double system_size, unsigned char *rgb) {
    std::cout.setstate(std::ios::failbit);
    Renderer r(n, width, height, render_scale, vmax, vmin, brightness, sharpness, dot, system_size, 1);
    std::vector<Body> b(n);
    for (int i = 0; i < n; i++) {
        b[i].position = Vector3D(x[i], y[i], z[i]);
        b[i].velocity = Vector3D(vx[i], vy[i], vz[i]);
    }
    const size_t np = 3 * (size_t)width * (size_t)height;
    std::vector<char> image(np);
    std::vector<double> hd(np);
    r.renderClear(image.data(), hd.data());
    r.renderBodies(b.data(), hd.data());
    for (size_t i = 0; i < np; i++) rgb[i] = (unsigned char)(int)(255.0 * r.clamp(hd[i]));
    std::cout.clear();
    return 0;
}
