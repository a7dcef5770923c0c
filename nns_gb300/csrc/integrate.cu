// integrate.cu -- kick-drift update, reference-array resets, FP64 checks.
#include <cstdint>

#include "nbx_internal.cuh"

namespace nbx {

namespace {

constexpr int kBlock = 256;

// Kernels.cu:581-600: v += dt*a; x += d*dt*v, as fused multiply-adds.
__global__ void __launch_bounds__(kBlock) k_update(float *__restrict__ x, float *__restrict__ y,
                                                    float *__restrict__ z, float *__restrict__ vx,
                                                    float *__restrict__ vy, float *__restrict__ vz,
                                                    const float *__restrict__ ax, const float *__restrict__ ay,
                                                    const float *__restrict__ az, int n, float dt, float ddt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float nvx = __fmaf_rn(dt, ax[i], vx[i]);
        const float nvy = __fmaf_rn(dt, ay[i], vy[i]);
        const float nvz = __fmaf_rn(dt, az[i], vz[i]);
        vx[i] = nvx;
        vy[i] = nvy;
        vz[i] = nvz;
        x[i] = __fmaf_rn(ddt, nvx, x[i]);
        y[i] = __fmaf_rn(ddt, nvy, y[i]);
        z[i] = __fmaf_rn(ddt, nvz, z[i]);
    }
}

// The same update, four bodies per thread with 16-byte loads and stores of
// each array (every array 16-byte aligned; bodies [0, 4*n4)).  Per element the
// operations are those of k_update, so the results are identical.
__global__ void __launch_bounds__(kBlock) k_update4(float4 *__restrict__ x, float4 *__restrict__ y,
                                                     float4 *__restrict__ z, float4 *__restrict__ vx,
                                                     float4 *__restrict__ vy, float4 *__restrict__ vz,
                                                     const float4 *__restrict__ ax, const float4 *__restrict__ ay,
                                                     const float4 *__restrict__ az, int n4, float dt, float ddt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        float4 v[3] = {vx[i], vy[i], vz[i]};
        const float4 a[3] = {ax[i], ay[i], az[i]};
        float4 p[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            v[k].x = __fmaf_rn(dt, a[k].x, v[k].x);
            v[k].y = __fmaf_rn(dt, a[k].y, v[k].y);
            v[k].z = __fmaf_rn(dt, a[k].z, v[k].z);
            v[k].w = __fmaf_rn(dt, a[k].w, v[k].w);
            p[k].x = __fmaf_rn(ddt, v[k].x, p[k].x);
            p[k].y = __fmaf_rn(ddt, v[k].y, p[k].y);
            p[k].z = __fmaf_rn(ddt, v[k].z, p[k].z);
            p[k].w = __fmaf_rn(ddt, v[k].w, p[k].w);
        }
        vx[i] = v[0];
        vy[i] = v[1];
        vz[i] = v[2];
        x[i] = p[0];
        y[i] = p[1];
        z[i] = p[2];
    }
}

// Kernels.cu:21-64
__global__ void __launch_bounds__(kBlock) k_reset_ref(int *mutex, float *x, float *y, float *z, float *mass,
                                                       int *count, int *start, int *sorted, int *child,
                                                       int *index, float *minX, float *maxX, float *minY,
                                                       float *maxY, float *minZ, float *maxZ, int n, int m) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < 8; k++) child[8 * (size_t)i + k] = -1;
        if (i < n) {
            count[i] = 1;
        } else {
            x[i] = 0.f;
            y[i] = 0.f;
            z[i] = 0.f;
            mass[i] = 0.f;
            count[i] = 0;
        }
        start[i] = -1;
        sorted[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *mutex = 0;
        *index = n;
        *minX = 0.f;
        *maxX = 0.f;
        *minY = 0.f;
        *maxY = 0.f;
        *minZ = 0.f;
        *maxZ = 0.f;
    }
}

// Kernels.cu:67-154 without the spin mutex: ordered-int atomics into a scratch
// box seeded with the caller's current values, then written back.
__global__ void k_bbox_ref_seed(unsigned *bu, const float *minX, const float *maxX, const float *minY,
                                const float *maxY, const float *minZ, const float *maxZ) {
    if (threadIdx.x == 0) {
        bu[0] = f2ord(*minX); bu[1] = f2ord(*maxX);
        bu[2] = f2ord(*minY); bu[3] = f2ord(*maxY);
        bu[4] = f2ord(*minZ); bu[5] = f2ord(*maxZ);
    }
}

__global__ void __launch_bounds__(kBlock) k_bbox_ref(const float *__restrict__ x, const float *__restrict__ y,
                                                      const float *__restrict__ z, int n, unsigned *bu) {
    float v[6] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        v[0] = fminf(v[0], x[i]); v[1] = fmaxf(v[1], x[i]);
        v[2] = fminf(v[2], y[i]); v[3] = fmaxf(v[3], y[i]);
        v[4] = fminf(v[4], z[i]); v[5] = fmaxf(v[5], z[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 6; k += 2) {
            v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
            v[k + 1] = fmaxf(v[k + 1], __shfl_xor_sync(0xffffffffu, v[k + 1], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 6; k++) {
            if (isnan(v[k]) || isinf(v[k])) continue;
            if (k & 1) atomicMax(&bu[k], f2ord(v[k]));
            else atomicMin(&bu[k], f2ord(v[k]));
        }
    }
}

__global__ void k_bbox_ref_store(const unsigned *bu, float *minX, float *maxX, float *minY, float *maxY,
                                 float *minZ, float *maxZ) {
    if (threadIdx.x == 0) {
        *minX = ord2f(bu[0]); *maxX = ord2f(bu[1]);
        *minY = ord2f(bu[2]); *maxY = ord2f(bu[3]);
        *minZ = ord2f(bu[4]); *maxZ = ord2f(bu[5]);
    }
}

// FP64 direct summation over bodies [0,n) for the given targets; the body
// range is split over blockIdx.y and accumulated with FP64 atomics.
__global__ void __launch_bounds__(kBlock) k_direct_fp64(const float *__restrict__ x, const float *__restrict__ y,
                                                         const float *__restrict__ z, const float *__restrict__ m,
                                                         int n, const int *__restrict__ targets, int nt,
                                                         double eps2, double *acc) {
    __shared__ double4 tile[kBlock];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int chunk = (n + gridDim.y - 1) / gridDim.y;
    const int j0 = blockIdx.y * chunk;
    const int j1 = min(n, j0 + chunk);
    double xi = 0.0, yi = 0.0, zi = 0.0;
    if (t < nt) {
        const int i = targets[t];
        xi = x[i];
        yi = y[i];
        zi = z[i];
    }
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int jb = j0; jb < j1; jb += kBlock) {
        const int j = jb + threadIdx.x;
        __syncthreads();
        tile[threadIdx.x] = j < j1 ? make_double4(x[j], y[j], z[j], m[j]) : make_double4(0.0, 0.0, 0.0, 0.0);
        __syncthreads();
        const int cnt = min(kBlock, j1 - jb);
        for (int k = 0; k < cnt; k++) {
            const double4 q = tile[k];
            const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double f = q.w / (r2 * sqrt(r2));
            sx += f * dx;
            sy += f * dy;
            sz += f * dz;
        }
    }
    if (t < nt) {
        atomicAdd(&acc[3 * t + 0], sx);
        atomicAdd(&acc[3 * t + 1], sy);
        atomicAdd(&acc[3 * t + 2], sz);
    }
}

__global__ void __launch_bounds__(kBlock) k_diag_fp64(const float *__restrict__ x, const float *__restrict__ y,
                                                       const float *__restrict__ z, const float *__restrict__ vx,
                                                       const float *__restrict__ vy, const float *__restrict__ vz,
                                                       const float *__restrict__ m, int n, double *out) {
    double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double mi = m[i], px = x[i], py = y[i], pz = z[i], ux = vx[i], uy = vy[i], uz = vz[i];
        a[0] += mi * ux;
        a[1] += mi * uy;
        a[2] += mi * uz;
        a[3] += 0.5 * mi * (ux * ux + uy * uy + uz * uz);
        a[4] += mi * (py * uz - pz * uy);
        a[5] += mi * (pz * ux - px * uz);
        a[6] += mi * (px * uy - py * ux);
        a[7] += mi;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        double v = a[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&out[k], v);
    }
}

}  // namespace

int integrate(Ctx *ctx, const nbx_state *s, float dt, float d, int n, cudaStream_t st) {
    if (n <= 0) return NBX_OK;
    const float ddt = d * dt;
    const float *arr[9] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->ax, s->ay, s->az};
    bool aligned = true;
    for (const float *a : arr) aligned &= (reinterpret_cast<uintptr_t>(a) & 15u) == 0;
    int done = 0;  // bodies [0, done) updated four at a time
    if (aligned && n >= 4) {
        const int n4 = n >> 2;
        int grid = ceil_div(n4, kBlock);
        if (grid > ctx->nsm * 16) grid = ctx->nsm * 16;
        k_update4<<<grid, kBlock, 0, st>>>(
            reinterpret_cast<float4 *>(s->x), reinterpret_cast<float4 *>(s->y), reinterpret_cast<float4 *>(s->z),
            reinterpret_cast<float4 *>(s->vx), reinterpret_cast<float4 *>(s->vy), reinterpret_cast<float4 *>(s->vz),
            reinterpret_cast<const float4 *>(s->ax), reinterpret_cast<const float4 *>(s->ay),
            reinterpret_cast<const float4 *>(s->az), n4, dt, ddt);
        ++ctx->launches;
        done = n4 << 2;
    }
    if (done < n) {
        const int m = n - done;
        int grid = ceil_div(m, kBlock);
        if (grid > ctx->nsm * 16) grid = ctx->nsm * 16;
        k_update<<<grid, kBlock, 0, st>>>(s->x + done, s->y + done, s->z + done, s->vx + done, s->vy + done,
                                          s->vz + done, s->ax + done, s->ay + done, s->az + done, m, dt, ddt);
        ++ctx->launches;
    }
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

int reset_ref_arrays(Ctx *ctx, int *mutex, float *x, float *y, float *z, float *mass, int *count, int *start,
                     int *sorted, int *child, int *index, float *minX, float *maxX, float *minY, float *maxY,
                     float *minZ, float *maxZ, int n, int m, cudaStream_t st) {
    int grid = ceil_div(m, kBlock);
    if (grid > ctx->nsm * 16) grid = ctx->nsm * 16;
    k_reset_ref<<<grid, kBlock, 0, st>>>(mutex, x, y, z, mass, count, start, sorted, child, index, minX, maxX,
                                         minY, maxY, minZ, maxZ, n, m);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

int bbox_ref(Ctx *ctx, const float *x, const float *y, const float *z, float *minX, float *maxX, float *minY,
             float *maxY, float *minZ, float *maxZ, int n, cudaStream_t st) {
    k_bbox_ref_seed<<<1, 32, 0, st>>>(ctx->d_bbox_u, minX, maxX, minY, maxY, minZ, maxZ);
    ++ctx->launches;
    int grid = ceil_div(n, kBlock);
    if (grid > ctx->nsm * 8) grid = ctx->nsm * 8;
    if (grid > 0) {
        k_bbox_ref<<<grid, kBlock, 0, st>>>(x, y, z, n, ctx->d_bbox_u);
        ++ctx->launches;
    }
    k_bbox_ref_store<<<1, 32, 0, st>>>(ctx->d_bbox_u, minX, maxX, minY, maxY, minZ, maxZ);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

int direct_fp64(Ctx *ctx, const float *x, const float *y, const float *z, const float *m, int n,
                const int *targets, int nt, double eps2, double *acc, cudaStream_t st) {
    if (nt <= 0 || n <= 0) return NBX_OK;
    const int gx = ceil_div(nt, kBlock);
    int gy = ceil_div(ctx->nsm * 4, gx);
    if (gy > ceil_div(n, kBlock)) gy = ceil_div(n, kBlock);
    if (gy < 1) gy = 1;
    k_direct_fp64<<<dim3(gx, gy), kBlock, 0, st>>>(x, y, z, m, n, targets, nt, eps2, acc);
    ++ctx->launches;
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

int diagnostics_fp64(Ctx *ctx, const nbx_state *s, int n, double *out, cudaStream_t st) {
    NBX_CUDA(cudaMemsetAsync(out, 0, 8 * sizeof(double), st));
    int grid = ceil_div(n, kBlock);
    if (grid > ctx->nsm * 4) grid = ctx->nsm * 4;
    if (grid > 0) {
        k_diag_fp64<<<grid, kBlock, 0, st>>>(s->x, s->y, s->z, s->vx, s->vy, s->vz, s->m, n, out);
        ++ctx->launches;
    }
    NBX_CUDA(cudaGetLastError());
    return NBX_OK;
}

}  // namespace nbx
