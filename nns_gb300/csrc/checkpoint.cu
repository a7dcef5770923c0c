// checkpoint.cu -- raw SoA checkpoint / resume of a context's systems
// (nbx_checkpoint_bytes / _save / _restore in include/nbx.h).
//
// Layout (little-endian, 8-byte aligned sections):
//   Header   magic "NBXCKPT1", version, nsys, nbodies, the step constants,
//            the walk's launch shape, buffer variant and stack depth (the
//            buffer width and the stack depth set how the walk's rounds group
//            the candidates, i.e. the order of the force sums, so a bit-exact
//            resume needs them), the multipole order and the leaf bucket size,
//            FNV-1a 64 of the header bytes before it and of the offsets
//   int64    offsets[nsys + 1]
//   float    x, y, z, vx, vy, vz, m   [nbodies] each
//   uint64   weighted checksum of the float payload (as 32-bit words)
// A restore checks the magic, version, sizes and both checksums before it
// changes anything, then sets the systems and constants and copies the bodies.
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#include "nbx_internal.cuh"

namespace nbx {

namespace {

struct CkptHeader {
    char magic[8];
    uint32_t version;
    int32_t nsys;
    int64_t nbodies;
    float theta_ref, eps2, dt, dampening;
    int32_t compensated, key_order;
    int32_t walk_warps, walk_variant;
    int32_t multipole, leaf_size;
    int32_t stack_depth, reserved;
    uint64_t header_hash;  // of the bytes above and of the offsets
};
static_assert(sizeof(CkptHeader) == 80, "checkpoint header layout");

constexpr char kMagic[8] = {'N', 'B', 'X', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t kVersion = 4;
constexpr int kArrays = 7;

uint64_t fnv1a(const void *p, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

// sum of the 32-bit words times odd weights: any single changed word changes it
uint64_t payload_sum(const float *a, size_t count) {
    uint64_t s = 0;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a);
    for (size_t i = 0; i < count; i++) s += (uint64_t)w[i] * (uint64_t)(2 * (i & 0xffff) + 1);
    return s;
}

size_t offsets_at() { return sizeof(CkptHeader); }
size_t arrays_at(int nsys) { return offsets_at() + sizeof(int64_t) * (size_t)(nsys + 1); }

int64_t total_bytes(int64_t n, int nsys) {
    return (int64_t)arrays_at(nsys) + (int64_t)kArrays * n * (int64_t)sizeof(float) + (int64_t)sizeof(uint64_t);
}

uint64_t header_hash(const CkptHeader &h, const int64_t *offs, int nsys) {
    return fnv1a(offs, sizeof(int64_t) * (size_t)(nsys + 1), fnv1a(&h, offsetof(CkptHeader, header_hash)));
}

}  // namespace

}  // namespace nbx

using nbx::Ctx;

extern "C" int64_t nbx_checkpoint_bytes(int64_t nbodies, int nsystems) {
    if (nbodies < 1 || nsystems < 1) return 0;
    return nbx::total_bytes(nbodies, nsystems);
}

extern "C" int nbx_checkpoint_save(nbx_ctx *c, const nbx_state *s, void *host, int64_t capacity, int64_t *written,
                                   void *stream) {
    if (!c || !s || !host) return NBX_ERR_ARG;
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    const int nsys = ctx->nsys;
    const int64_t n = ctx->nbodies;
    if (nsys < 1 || n < 1) return NBX_ERR_STATE;
    const float *arr[nbx::kArrays] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->m};
    for (const float *a : arr)
        if (!a) return NBX_ERR_ARG;
    const int64_t need = nbx::total_bytes(n, nsys);
    if (capacity < need) return NBX_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *out = static_cast<unsigned char *>(host);
    std::vector<int> off32(nsys + 1);
    NBX_CUDA(cudaMemcpyAsync(off32.data(), ctx->d_sys_off, sizeof(int) * (nsys + 1), cudaMemcpyDeviceToHost, st));
    float *payload = reinterpret_cast<float *>(out + nbx::arrays_at(nsys));
    for (int k = 0; k < nbx::kArrays; k++)
        NBX_CUDA(cudaMemcpyAsync(payload + (size_t)k * n, arr[k], sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    NBX_CUDA(cudaStreamSynchronize(st));
    int64_t *offs = reinterpret_cast<int64_t *>(out + nbx::offsets_at());
    for (int i = 0; i <= nsys; i++) offs[i] = off32[i];
    nbx::CkptHeader h{};
    std::memcpy(h.magic, nbx::kMagic, 8);
    h.version = nbx::kVersion;
    h.nsys = nsys;
    h.nbodies = n;
    h.theta_ref = ctx->theta_ref;
    h.eps2 = ctx->eps2;
    h.dt = ctx->p.dt;
    h.dampening = ctx->p.dampening;
    h.compensated = ctx->compensated;
    h.key_order = ctx->key_order;
    h.walk_warps = ctx->walk_warps;
    h.walk_variant = ctx->walk_variant;
    h.multipole = ctx->multipole;
    h.leaf_size = ctx->leaf_size;
    h.stack_depth = ctx->p.stack_depth;
    h.header_hash = nbx::header_hash(h, offs, nsys);
    std::memcpy(out, &h, sizeof(h));
    const uint64_t sum = nbx::payload_sum(payload, (size_t)nbx::kArrays * n);
    std::memcpy(out + need - sizeof(uint64_t), &sum, sizeof(sum));
    if (written) *written = need;
    return NBX_OK;
}

extern "C" int nbx_checkpoint_restore(nbx_ctx *c, nbx_state *s, const void *host, int64_t bytes, void *stream) {
    if (!c || !s || !host) return NBX_ERR_ARG;
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    float *arr[nbx::kArrays] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->m};
    for (float *a : arr)
        if (!a) return NBX_ERR_ARG;
    const unsigned char *in = static_cast<const unsigned char *>(host);
    if (bytes < (int64_t)sizeof(nbx::CkptHeader)) return NBX_ERR_FORMAT;
    nbx::CkptHeader h;
    std::memcpy(&h, in, sizeof(h));
    if (std::memcmp(h.magic, nbx::kMagic, 8) != 0 || h.version != nbx::kVersion || h.nsys < 1 || h.nbodies < 1 ||
        h.nbodies > ((int64_t)1 << 31))
        return NBX_ERR_FORMAT;
    const int nsys = h.nsys;
    const int64_t n = h.nbodies;
    const int64_t need = nbx::total_bytes(n, nsys);
    if (bytes != need) return NBX_ERR_FORMAT;
    std::vector<int64_t> off(nsys + 1);
    std::memcpy(off.data(), in + nbx::offsets_at(), sizeof(int64_t) * (nsys + 1));
    if (nbx::header_hash(h, off.data(), nsys) != h.header_hash || off[nsys] != n) return NBX_ERR_FORMAT;
    const float *payload = reinterpret_cast<const float *>(in + nbx::arrays_at(nsys));
    uint64_t sum;
    std::memcpy(&sum, in + need - sizeof(uint64_t), sizeof(sum));
    if (nbx::payload_sum(payload, (size_t)nbx::kArrays * n) != sum) return NBX_ERR_FORMAT;
    // settings outside their ranges are a malformed checkpoint: refused before anything changes
    if (h.multipole < 0 || h.multipole > 1 || h.leaf_size < 1 || h.leaf_size > 8 || h.walk_variant < 0 ||
        h.walk_variant > 3 || !(h.walk_warps == 4 || h.walk_warps == 8 || h.walk_warps == 16) || h.stack_depth < 360 ||
        h.stack_depth > 4096 || (h.multipole == 1 && h.walk_variant == 2) || h.compensated < 0 || h.compensated > 2 ||
        !(h.theta_ref > 0.f) || !(h.eps2 >= FLT_MIN) || !std::isfinite(h.theta_ref) || !std::isfinite(h.eps2))
        return NBX_ERR_FORMAT;
    if (n > ctx->cap_bodies || nsys > ctx->cap_sys || h.key_order != ctx->key_order) return NBX_ERR_ARG;
    int rc = nbx_set_systems(c, nsys, off.data());
    if (rc) return rc;
    rc = nbx_set_constants(c, h.theta_ref, h.eps2, h.compensated);
    if (rc) return rc;
    // the one-cell walk (variant 2) has no quadrupole form: leave quadrupoles
    // before choosing it, choose the walk before entering them
    if (h.multipole == 0) {
        rc = nbx_set_multipole(c, 0);
        if (rc) return rc;
    }
    rc = nbx_set_walk_config(c, h.walk_warps, h.walk_variant);
    if (rc) return rc;
    if (h.multipole != 0) {
        rc = nbx_set_multipole(c, h.multipole);
        if (rc) return rc;
    }
    rc = nbx_set_leaf_size(c, h.leaf_size);
    if (rc) return rc;
    rc = nbx_set_tuning(c, ctx->radix_bits, h.stack_depth);
    if (rc) return rc;
    ctx->p.dt = h.dt;
    ctx->p.dampening = h.dampening;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int k = 0; k < nbx::kArrays; k++)
        NBX_CUDA(cudaMemcpyAsync(arr[k], payload + (size_t)k * n, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    NBX_CUDA(cudaStreamSynchronize(st));
    return NBX_OK;
}
