// render.cu -- headless frame: the reference renderer's velocity-coloured dot
// splat (3D/CUDA/CUDA_NBody/src/Renderer.cpp:54-147) into a device RGB buffer.
//
// Per drawn body (same selection, colour ramp and pixel mapping as the
// reference): the dot covers (floor(px)+i, floor(py)+j), i, j in
// [-dot/2, dot/2), with weight
//   brightness / ((exp((s a_i)^2) + exp((s b_j)^2))^0.75 + 1),
//   a_i = floor(px)+i-px, b_j = floor(py)+j-py.
// The pixel position px, py and its floor are FP64 like the reference, so
// every dot lands where the reference puts it.  The colour ramp, the offsets
// a_i, b_j (from the FP64 fraction px - floor(px)) and the weights are FP32:
// an 8-bit output needs far less, and FP64 runs at a small fraction of the
// FP32 rate on this part.  The power is exp2(0.75 log2(.)).
// Bodies are visited in the tree's sorted order when the context holds a tree
// for them, so a block's 256 consecutive bodies cover a small pixel window:
// that window is accumulated with shared-memory integer atomics in fixed point
// and flushed once as FP32; a block whose window is too large adds to global
// memory directly.  A final pass converts to bytes as int(255 clamp(v)).
#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kSplatBlock = 256;
constexpr int kWinPix = 4096;  // pixels of the shared-memory window (48 KB of FP32 RGB)
constexpr int kMaxDot = 16;

struct RenderConst {
    int w, h, dot;
    double half_w, half_h, inv_extent;  // size/2, 1/(system_size * render_scale)
    float vmin, vmax;  // velocity colour range
    float bright, sharp;
    float fix;         // fixed-point units per 1.0 in the shared-memory window
};

__device__ __forceinline__ double clamp01(double v) { return fmax(fmin(v, 1.0), 0.0); }
__device__ __forceinline__ float clamp01f(float v) { return fmaxf(fminf(v, 1.f), 0.f); }

__global__ void __launch_bounds__(kSplatBlock) k_splat(const float *__restrict__ x, const float *__restrict__ y,
                                                        const float *__restrict__ vx, const float *__restrict__ vy,
                                                        const float *__restrict__ vz, const int *__restrict__ order,
                                                        int n, RenderConst rc, float *__restrict__ accum) {
    __shared__ unsigned win[3 * kWinPix];  // fixed point, rc.fix units per 1.0
    __shared__ int wbox[4];
    const int half = rc.dot / 2, nd = 2 * half;
    for (int base = blockIdx.x * kSplatBlock; base < n; base += gridDim.x * kSplatBlock) {
        __syncthreads();  // the previous chunk's window box was read and its window flushed
        if (threadIdx.x == 0) {
            wbox[0] = wbox[2] = 0x7fffffff;
            wbox[1] = wbox[3] = -0x7fffffff;
        }
        const int p = base + threadIdx.x;
        bool draw = false;
        int xp = 0, yp = 0;
        float fx = 0.f, fy = 0.f;  // px - floor(px), py - floor(py)
        float cr = 0.f, cg = 0.f, cb = 0.f;
        if (p < n) {
            const int b = order ? order[p] : p;
            const double pxs = rc.half_w * (1.0 + (double)x[b] * rc.inv_extent);  // Renderer.cpp:86-89
            const double pys = rc.half_h * (1.0 + (double)y[b] * rc.inv_extent);
            const int xi = (int)pxs, yi = (int)pys;  // :66-71
            draw = xi > rc.dot && xi < rc.w - rc.dot && yi > rc.dot && yi < rc.h - rc.dot;
            if (draw) {
                const float ux = vx[b], uy = vy[b], uz = vz[b];
                const float vmag = sqrtf(ux * ux + uy * uy + uz * uz);  // Body.cpp:11-13
                if (vmag < rc.vmin) {
                    draw = false;
                } else {  // :99-104
                    const float vp = sqrtf((vmag - rc.vmin) / rc.vmax);
                    cr = clamp01f(4.f * (vp - 0.333f));
                    cg = clamp01f(fminf(4.f * vp, 4.f * (1.f - vp)));
                    cb = clamp01f(4.f * (0.5f - vp));
                    const double flx = floor(pxs), fly = floor(pys);
                    xp = (int)flx;
                    yp = (int)fly;
                    fx = (float)(pxs - flx);
                    fy = (float)(pys - fly);
                }
            }
        }
        __syncthreads();  // wbox initialised
        if (draw) {
            atomicMin(&wbox[0], xp - half);
            atomicMax(&wbox[1], xp + half - 1);
            atomicMin(&wbox[2], yp - half);
            atomicMax(&wbox[3], yp + half - 1);
        }
        __syncthreads();
        const int wx0 = wbox[0], wy0 = wbox[2];
        const int ww = wbox[1] - wx0 + 1, wh = wbox[3] - wy0 + 1;
        if (ww <= 0) continue;  // nothing drawn in this chunk (uniform)
        const bool local = (long long)ww * wh <= kWinPix;
        if (local)
            for (int k = threadIdx.x; k < 3 * ww * wh; k += kSplatBlock) win[k] = 0u;
        __syncthreads();
        if (draw) {
            // lanes start their rows at different offsets, so lanes drawing the
            // same dot centre (dense regions) add to different pixels at a time
            const int rot = nd > 0 ? (threadIdx.x & 31) % nd : 0;
            for (int i = 0; i < nd; i++) {
                const float tx = rc.sharp * ((float)(i - half) - fx);
                const float ex = expf(tx * tx);
                const int gx = xp - half + i;
                int j = rot;
                for (int jj = 0; jj < nd; jj++) {
                    const float ty = rc.sharp * ((float)(j - half) - fy);
                    const float f = rc.bright / (exp2f(0.75f * __log2f(ex + expf(ty * ty))) + 1.0f);
                    const int gy = yp - half + j;
                    if (local) {  // integer shared atomics: one pass; float ones serialise per lane
                        unsigned *q = &win[3 * ((gy - wy0) * ww + (gx - wx0))];
                        atomicAdd(q + 0, __float2uint_rn(cr * f * rc.fix));
                        atomicAdd(q + 1, __float2uint_rn(cg * f * rc.fix));
                        atomicAdd(q + 2, __float2uint_rn(cb * f * rc.fix));
                    } else {
                        float *q = &accum[3 * ((size_t)gy * rc.w + gx)];
                        atomicAdd(q + 0, cr * f);
                        atomicAdd(q + 1, cg * f);
                        atomicAdd(q + 2, cb * f);
                    }
                    j = j + 1 == nd ? 0 : j + 1;
                }
            }
        }
        if (local) {
            __syncthreads();
            for (int k = threadIdx.x; k < 3 * ww * wh; k += kSplatBlock) {
                const unsigned v = win[k];
                if (v != 0u) {
                    const int pix = k / 3, c = k - 3 * pix;
                    const int gy = wy0 + pix / ww, gx = wx0 + pix % ww;
                    atomicAdd(&accum[3 * ((size_t)gy * rc.w + gx) + c], (float)v / rc.fix);
                }
            }
        }
    }
}

// Renderer.cpp:144-147: byte = int(255 * clamp(v))
__global__ void k_tonemap(const float *__restrict__ accum, unsigned char *__restrict__ rgb, size_t count) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x)
        rgb[k] = (unsigned char)(int)(255.0 * clamp01((double)accum[k]));
}

}  // namespace

}  // namespace nbx

using nbx::Ctx;

extern "C" void nbx_render_params_default(nbx_render_params *p) {
    if (!p) return;
    // Constants.h:31-38
    p->width = 1024;
    p->height = 1024;
    p->render_scale = 2.5;
    p->max_velocity_color = 1500.0;
    p->min_velocity_color = 0.0;
    p->particle_brightness = 0.35;
    p->particle_sharpness = 1.0;
    p->dot_size = 8;
    p->system_size = 0.0;  // must be set: main.cu:95 passes 2 * BarnesHut::getSystemSize()
}

extern "C" int nbx_render_frame(nbx_ctx *c, const nbx_state *s, int n, const nbx_render_params *p, float *accum,
                                unsigned char *rgb, void *stream) {
    if (!c || !s || !p || !accum || !rgb || n < 1 || !s->x || !s->y || !s->vx || !s->vy || !s->vz)
        return NBX_ERR_ARG;
    if (p->width < 1 || p->height < 1 || p->dot_size < 0 || p->dot_size > nbx::kMaxDot ||
        !(p->system_size > 0.0) || !(p->render_scale > 0.0) || !(p->max_velocity_color > 0.0) ||
        !(p->particle_brightness >= 0.0) ||
        (long long)p->width * p->height > (1ll << 28))
        return NBX_ERR_ARG;
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    nbx::RenderConst rc;
    rc.w = p->width;
    rc.h = p->height;
    rc.dot = p->dot_size;
    rc.half_w = p->width / 2.0;
    rc.half_h = p->height / 2.0;
    rc.inv_extent = 1.0 / (p->system_size * p->render_scale);
    rc.vmin = (float)p->min_velocity_color;
    rc.vmax = (float)p->max_velocity_color;
    rc.bright = (float)p->particle_brightness;
    // a window pixel sums at most kSplatBlock dots of weight <= brightness per
    // channel: keep that below 2^31 units; 2^20 units per 1.0 at most (an 8-bit
    // output needs ~2^8, so the rounding of each term, 2^-21, is invisible)
    {
        const double cap = 2147483648.0 / ((double)nbx::kSplatBlock * (p->particle_brightness > 1e-30 ? p->particle_brightness : 1e-30));
        rc.fix = (float)(cap < 1048576.0 ? cap : 1048576.0);
    }
    rc.sharp = (float)p->particle_sharpness;
    const size_t count = 3 * (size_t)p->width * (size_t)p->height;
    NBX_CUDA(cudaMemsetAsync(accum, 0, count * sizeof(float), st));
    // the sorted order of the context's tree, when it was built over these n bodies
    const int *order = (ctx->built && ctx->nbodies == n) ? ctx->d_val : nullptr;
    int grid = (n + nbx::kSplatBlock - 1) / nbx::kSplatBlock;
    if (grid > ctx->nsm * 8) grid = ctx->nsm * 8;
    nbx::k_splat<<<grid, nbx::kSplatBlock, 0, st>>>(s->x, s->y, s->vx, s->vy, s->vz, order, n, rc, accum);
    ++ctx->launches;
    int tg = (int)((count + 255) / 256);
    if (tg > ctx->nsm * 8) tg = ctx->nsm * 8;
    nbx::k_tonemap<<<tg, 256, 0, st>>>(accum, rgb, count);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}
