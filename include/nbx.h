/*
 * nbx.h -- C ABI of the GB300-native Barnes-Hut pipeline (libnbx.so).
 *
 * Plain pointers and sizes only.  Device pointers are CUDA device memory of
 * the current device; `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Every entry point returns an nbx status code; no
 * entry point synchronises the host except where stated (timing out-params and
 * nbx_sync_status).
 *
 * Two layers:
 *  1. Phase entry points with the argument lists and array semantics of the
 *     reference's KernelsWrapper (3D/CUDA/CUDA_NBody/include/KernelsWrapper.cuh:28-48,
 *     src/KernelsWrapper.cu:28-208), so that the reference's BarnesHut host class
 *     (src/BarnesHut.cu:195-258) can be relinked against them:
 *       SoA float arrays of length m, child[8m], -1 = null, bodies [0,n),
 *       cells [n, m) (canonical depth-first numbering), *index = n + ncells.
 *     Each takes a context (holding the tree scratch), the stream, and an
 *     optional `ms` out-param: when non-NULL the call is timed with CUDA events
 *     and synchronises, like the reference's `timing=true` path.
 *  2. The native pipeline over device-resident SoA state with any number of
 *     independent systems (nbx_set_systems / nbx_step / nbx_graph_step ...).
 */
#ifndef NBX_H
#define NBX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define NBX_OK 0
#define NBX_ERR_ARG 1       /* invalid argument */
#define NBX_ERR_CUDA 2      /* a CUDA runtime call failed */
#define NBX_ERR_DEPTH 3     /* two bodies share a subdivision region 42 levels deep (duplicates) */
#define NBX_ERR_CAPACITY 4  /* the node pool of the context is too small for this tree */
#define NBX_ERR_STACK 5     /* a walk stack overflowed (raise nbx_params.stack_depth) */
#define NBX_ERR_NONFINITE 6 /* a position is NaN or infinite */
#define NBX_ERR_CLUSTER 7   /* more than 4096 bodies share one 21-level key */
#define NBX_ERR_TIMEOUT 8   /* a bounded device-side wait expired */
#define NBX_ERR_STATE 9     /* call out of order (e.g. forces before a build) */
#define NBX_ERR_NOMEM 10    /* device allocation failed */
#define NBX_ERR_SCRATCH 11  /* request larger than the static scratch of a no-allocation entry point */
#define NBX_ERR_FORMAT 12   /* checkpoint header, size or checksum mismatch */

typedef struct nbx_ctx nbx_ctx;

typedef struct nbx_params {
    int max_bodies;    /* capacity: total bodies over all systems (<= 2^26) */
    int max_systems;   /* capacity: independent systems */
    float theta;       /* opening angle: a cell of x-side s at squared distance r
                          (softened) is accepted when s^2 / theta^2 <= r, i.e. the
                          reference's raw constant is theta^2 */
    float theta_ref;   /* > 0: use this raw MAC constant (Kernels.cu:18 `theta`) */
    float eps;         /* Plummer softening length (the squared softening in use
                          must be > 0: a body's own term, d = 0, is 0 * inf otherwise) */
    float eps2;        /* > 0: use this squared softening (Kernels.cu:17) */
    float dt;          /* time step (main.cu:52) */
    float dampening;   /* velocity factor of the drift (main.cu:54) */
    float gravity;     /* accepted for interface parity; the force uses G = 1 (Kernels.cu:462) */
    int group;         /* bodies sharing one walk (warp-coherent MAC vote): 32 */
    int stack_depth;   /* walk stack entries per warp, 360..4096 (512); the stacks and buffers of
                          one walk block must fit its shared memory (NBX_ERR_ARG otherwise) */
    int compensated;   /* 0 plain FP32; 1 split compensation (FP32 partial sums per
                          walk round, Kahan across rounds); 2 Kahan on every term */
    int leaf_size;     /* bodies per leaf: 1, the reference's tree (Kernels.cu:284-362; the parity
                          mode); 2..8: every cell holding at most leaf_size bodies whose parent
                          holds more is a leaf with its bodies as children (fewer cells, longer
                          lists; trees and lists differ from the reference's, nbx_export_tree
                          refuses them).  Not available with the adjoint */
    int radix_bits;    /* radix digit width of the key sort: 8 (8 passes) or 9 (7 passes) */
    int walk_warps;    /* warps per block of the walk kernel (0 = autotuned default) */
    int device;        /* CUDA device ordinal */
    int block_size;    /* reference launch-shape hints (main.cu:30-31); informational */
    int grid_size;
    int walk_variant;  /* 0 production walk, 64-slot candidate buffers; 1 the same with
                          128-slot buffers; 2 one-cell-at-a-time walk (comparison);
                          3 production walk, 96-slot buffers */
    int key_order;     /* 0: the reference's body order (Lebesgue keys; bit-exact parity);
                          1: Hilbert keys -- same cells, siblings reordered, so walk groups
                          are compact but the interaction lists differ from the reference */
    int node_capacity; /* node pool (cells + bodies); 0: 2*max_bodies + 65536.  A tree that
                          needs more nodes reports NBX_ERR_CAPACITY */
    int moments_mode;  /* centre-of-mass pass: 0 by size (one launch up to 2^21 bodies,
                          per level above); 1 one launch per tree level; 2 one launch in
                          which the last child to finish sums its parent.  The sums are
                          the same FP64 additions in the same order in every mode */
    int multipole;     /* 0: monopoles, the reference's force (Kernels.cu:538-551; the parity
                          mode); 1: monopoles plus the traceless quadrupole of every accepted
                          cell (FP64 second moments, FP32 terms).  The interaction lists are
                          the same in both; quadrupoles only change what an accepted cell adds.
                          Not available with walk_variant 2 or the adjoint */
} nbx_params;

/* SoA device state of all systems; systems are contiguous ranges. */
typedef struct nbx_state {
    float *x, *y, *z;
    float *vx, *vy, *vz;
    float *ax, *ay, *az;
    float *m;
} nbx_state;

typedef struct nbx_tree_info {
    int64_t nbodies;       /* bodies in the last build */
    int64_t ncells;        /* cells (internal nodes, roots excluded) */
    int64_t nnodes;        /* cells + bodies */
    int32_t max_level;     /* deepest node level (root children = 1) */
    int32_t nsystems;
    int64_t interactions;  /* sum over bodies of interaction-list length, last walk */
    int64_t opened;        /* sum over groups of cells opened, last walk */
    int32_t refined_runs;  /* runs of equal 21-level keys refined past level 21 */
    int32_t status;        /* sticky device error status */
    int64_t launches;      /* kernels launched by this context so far */
    int64_t rounds;        /* walk rounds (expand + evaluate) over all groups, last walk */
    int64_t candidates;    /* candidates evaluated by those rounds */
} nbx_tree_info;

/* ---- context -------------------------------------------------------- */
void nbx_params_default(nbx_params *p);
int nbx_create(const nbx_params *p, nbx_ctx **out);
int nbx_destroy(nbx_ctx *ctx);
const char *nbx_status_string(int status);
const char *nbx_last_error(nbx_ctx *ctx);
/* Current effective MAC constant and softening of the context.  nbx_create
 * and nbx_set_constants take a finite theta_ref > 0 and a finite, normal
 * eps2 >= FLT_MIN (NBX_ERR_ARG otherwise). */
int nbx_get_constants(nbx_ctx *ctx, float *theta_ref, float *eps2);
int nbx_set_constants(nbx_ctx *ctx, float theta_ref, float eps2, int compensated);
/* Launch shape of the walk: warps per block (4, 8 or 16) and variant; used by
 * the autotuner (nns_gb300/autotune.py). */
int nbx_set_walk_config(nbx_ctx *ctx, int warps_per_block, int variant);
/* Sort digit width (8: 8 passes, 9: 7 passes over the 63-bit keys; both give the
 * same stable order) and walk stack entries per warp (360..4096; a launch whose
 * stacks and buffers exceed the device's shared memory per block fails with
 * NBX_ERR_ARG).  The stack depth never changes the interaction lists, but it
 * sets how the walk groups candidates into rounds near the depth-first reserve,
 * so forces can differ in their last bits between depths.  A built tree stays
 * valid.  Used by the autotuner. */
int nbx_set_tuning(nbx_ctx *ctx, int radix_bits, int stack_depth);
/* Multipole order of the force (nbx_params.multipole: 0 monopoles, 1 with
 * quadrupoles).  The context needs a new build before its next walk
 * (NBX_ERR_STATE otherwise); switching to 1 allocates the quadrupole arrays
 * on first use (NBX_ERR_NOMEM if that fails).  No counterpart in the
 * reference, whose kernels carry monopoles only. */
int nbx_set_multipole(nbx_ctx *ctx, int multipole);
/* Bodies per leaf bucket (nbx_params.leaf_size, 1..8); the context needs a new
 * build before its next walk.  Used by the autotuner outside the parity mode. */
int nbx_set_leaf_size(nbx_ctx *ctx, int leaf_size);

/* ---- reference-compatible phase entry points (KernelsWrapper.cu) ---- */
/* KernelsWrapper::resetArrays (KernelsWrapper.cu:28; Kernels.cu:21-64) */
int nbx_reset_arrays(nbx_ctx *ctx, int *mutex, float *x, float *y, float *z, float *mass,
                     int *count, int *start, int *sorted, int *child, int *index, float *minX,
                     float *maxX, float *minY, float *maxY, float *minZ, float *maxZ, int n, int m,
                     void *stream, float *ms);
/* KernelsWrapper::computeBoundingBox (KernelsWrapper.cu:56; Kernels.cu:67-154):
 * merges the bounding box of bodies [0,n) into *minX..*maxZ. */
int nbx_compute_bounding_box(nbx_ctx *ctx, int *mutex, float *x, float *y, float *z, float *minX,
                             float *maxX, float *minY, float *maxY, float *minZ, float *maxZ,
                             int n, void *stream, float *ms);
/* Context-free variant of nbx_compute_bounding_box that allocates nothing; it has
 * no counterpart in the reference.  For callers that own their body arrays but
 * cannot allocate device memory (a fixed memory budget, or an allocator that
 * has already reserved the HBM) and so cannot create a context.  Same merge
 * into *minX..*maxZ and, with grid_size 0 (the context path's grid), the same
 * bits.  Its scratch is a static per-device array of 4096 block partials
 * (128 KiB + 256 B) held by every GPU that loads the library: grid_size above
 * 4096 returns NBX_ERR_SCRATCH.  All calls on a device share that array, so
 * calls that overlap on the GPU race.  Every call resolves the array's address
 * in the current context (cudaGetSymbolAddress); the first call on a device,
 * and the first after a device reset (which invalidates the old address), may
 * load the module: make those calls before any stream capture.
 * `mutex` is accepted for the reference signature and unused. */
int nbx_compute_bounding_box_noalloc(int *mutex, const float *x, const float *y, const float *z,
                                     float *minX, float *maxX, float *minY, float *maxY, float *minZ,
                                     float *maxZ, int n, int grid_size, void *stream);
/* KernelsWrapper::buildTree (KernelsWrapper.cu:81; Kernels.cu:157-377): keys, sort
 * and key-built octree; writes child[], count[] and mass[], x/y/z (= sum m*x) of
 * the cells, *index. */
int nbx_build_tree(nbx_ctx *ctx, float *x, float *y, float *z, float *mass, int *count,
                   int *start, int *child, int *index, float *minX, float *maxX, float *minY,
                   float *maxY, float *minZ, float *maxZ, int n, int m, void *stream, float *ms);
/* KernelsWrapper::centreOfMass (KernelsWrapper.cu:109; Kernels.cu:381-399) */
int nbx_centre_of_mass(nbx_ctx *ctx, float *x, float *y, float *z, float *mass, int *index, int n,
                       void *stream, float *ms);
/* KernelsWrapper::sort (KernelsWrapper.cu:133; Kernels.cu:403-456) */
int nbx_sort(nbx_ctx *ctx, int *count, int *start, int *sorted, int *child, int *index, int n,
             void *stream, float *ms);
/* KernelsWrapper::computeForces (KernelsWrapper.cu:157; Kernels.cu:460-577) */
int nbx_compute_forces(nbx_ctx *ctx, float *x, float *y, float *z, float *vx, float *vy,
                       float *vz, float *ax, float *ay, float *az, float *mass, int *sorted,
                       int *child, float *minX, float *maxX, int n, float g, void *stream,
                       float *ms);
/* KernelsWrapper::update (KernelsWrapper.cu:185; Kernels.cu:581-600) */
int nbx_update(nbx_ctx *ctx, float *x, float *y, float *z, float *vx, float *vy, float *vz,
               float *ax, float *ay, float *az, int n, float dt, float d, void *stream,
               float *ms);

/* ---- native pipeline (no counterpart in the reference's API) --------- */
/* Systems are the ranges [offsets[s], offsets[s+1]) of the state arrays;
 * offsets is a HOST array of nsys+1 entries, offsets[0] = 0, each system >= 1 body. */
int nbx_set_systems(nbx_ctx *ctx, int nsys, const int64_t *offsets);
/* bbox, keys, sort and tree + moments of every system */
int nbx_build(nbx_ctx *ctx, const nbx_state *s, void *stream);
/* tree walk of the last build -> s->ax, s->ay, s->az */
int nbx_forces(nbx_ctx *ctx, const nbx_state *s, void *stream);
/* Walk groups: runs of up to 32 consecutive sorted bodies of one system (the
 * warp-coherent MAC's group), numbered system by system in sorted order, so a
 * range of groups is a range of keys.  nbx_group_count gives their number. */
int nbx_group_count(nbx_ctx *ctx, int *ngroups);
/* The walk of groups [first_group, first_group + ngroups) of the last build
 * only: the forces of those groups' bodies are written, every other body's
 * acceleration is left as it was.  One rank's share when one system is split
 * over several GPUs by key ranges (the reference's SFC decomposition,
 * MolecularDynamics/BarnesHutParallel/SpaceFillingCurves/src/Tree.cpp:165-317,
 * here over a replicated tree): each rank zeroes the accelerations, walks its
 * groups and the ranks sum the accelerations (nns_gb300/dist.py).  Not for
 * walk_variant 2. */
int nbx_forces_groups(nbx_ctx *ctx, const nbx_state *s, int first_group, int ngroups, void *stream);
/* Per-group interaction-list length and opened cells of the last walk (device
 * int arrays of nbx_group_count entries; either may be NULL): the work
 * measure for balancing key ranges.  Synchronises `stream`. */
int nbx_export_group_stats(nbx_ctx *ctx, int *list_len, int *opened, void *stream);
/* kick-drift with the context's dt and dampening */
int nbx_integrate(nbx_ctx *ctx, const nbx_state *s, void *stream);
/* nsteps x (build, forces, integrate).  One step is launched kernel by kernel;
   several replay nbx_graph_step's captured step (not while `stream` is being
   captured: then every step is launched kernel by kernel). */
int nbx_step(nbx_ctx *ctx, const nbx_state *s, int nsteps, void *stream);
/* the same steps replayed from a CUDA graph captured once per state, on the
   context's own stream, ordered after and before `stream` by events
   (asynchronous; NBX_ERR_ARG while `stream` is being captured) */
int nbx_graph_step(nbx_ctx *ctx, const nbx_state *s, int nsteps, void *stream);
/* synchronises `stream` and returns (and clears) the sticky device status */
int nbx_sync_status(nbx_ctx *ctx, void *stream);
/* Self-test of the bounded wait in the one-sweep body sort (contexts below
 * 1.5 x 2^20 bodies; its tiles wait for the counts of their system's earlier
 * tiles): one pass
 * over the second tile of a two-tile system whose first tile never runs, on
 * scratch of its own.  Its wait gives up within a second and records
 * NBX_ERR_TIMEOUT in the context's device status (which keeps the first error
 * recorded: call it with no error pending), which the next nbx_sync_status
 * returns and clears; the context stays usable.  Writes nothing outside its
 * scratch. */
int nbx_selftest_sort_wait(nbx_ctx *ctx, void *stream);
/* synchronises and reports the last build/walk */
int nbx_get_tree_info(nbx_ctx *ctx, void *stream, nbx_tree_info *out);

/* Export of the last build of system `sys` in the reference's array format
 * (device pointers; cells numbered n_sys + depth-first index): sorted body
 * order (system-local original indices), root_child[8], cell_child[8*ncells],
 * cell start/count/level, cell centre of mass and mass.  Any pointer may be
 * NULL.  cap_cells bounds the cell arrays; *ncells receives the count. */
int nbx_export_tree(nbx_ctx *ctx, int sys, int *perm, int *root_child, int *cell_child,
                    int *cell_start, int *cell_count, int *cell_level, float *cell_x,
                    float *cell_y, float *cell_z, float *cell_m, int cap_cells, int64_t *ncells,
                    void *stream);
/* Sorted 21-level keys (ascending = the reference's in-order body order) and
 * the sort permutation (global original indices), both of length nbodies. */
int nbx_export_keys(nbx_ctx *ctx, uint64_t *keys, int *perm, void *stream);
/* Per-body interaction-list length and opened-cell count of the last walk
 * (global original index order). */
int nbx_export_walk_stats(nbx_ctx *ctx, int *nlist, int *nopen, void *stream);

/* FP64 direct summation (ground truth) for `nt` target indices over bodies
 * [0,n): acc[3*t+k] += sum_j m_j d (|d|^2+eps2)^-3/2 in FP64. */
int nbx_direct_fp64(nbx_ctx *ctx, const float *x, const float *y, const float *z, const float *m,
                    int n, const int *targets, int nt, double eps2, double *acc, void *stream);
/* The last walk's interaction lists of the given walk groups (device array of
 * the groups' first sorted positions, multiples of 32 from each system's start)
 * re-evaluated in FP64: acc is a device double[3*nbodies] ([3][n], original
 * order; rows outside the groups are untouched).  Against the FP32 walk this
 * isolates the FP32 arithmetic error from the tree approximation. */
int nbx_forces_fp64_lists(nbx_ctx *ctx, const int *group_starts, int ngroups, double *acc,
                          void *stream);
/* Per-body potential phi_i = -sum_j m_j / sqrt(|d|^2+eps2) over the walk's
 * interaction lists (self term removed), original index order; needs eps2 > 0. */
int nbx_potential(nbx_ctx *ctx, const nbx_state *s, float *phi, void *stream);
/* ---- differentiation (no counterpart in the reference) -------------------
 * Gradients of L = sum_i |x_i(T) - x*_i|^2 after T kick-drift steps with
 * respect to the initial positions, velocities and masses, through the
 * Barnes-Hut forces with the interaction lists frozen to the recorded ones.
 * Checkpoints every `checkpoint_every` steps; each segment is recomputed with
 * its trees and interaction lists recorded (list_capacity entries per walk
 * group) and reversed.  tape_steps >= checkpoint_every slots are allocated
 * (tape_steps >= nsteps also enables nbx_adjoint_record / _replay_fp64). */
typedef struct nbx_adjoint nbx_adjoint;
int nbx_adjoint_create(nbx_ctx *ctx, int nsteps, int checkpoint_every, int list_capacity,
                       int tape_steps, nbx_adjoint **out);
int nbx_adjoint_destroy(nbx_adjoint *adj);
/* Runs the T forward steps from s (advancing it) and returns the loss against
 * the target positions (device arrays of n floats). */
int nbx_adjoint_forward(nbx_ctx *ctx, nbx_adjoint *adj, const nbx_state *s, const float *tx,
                        const float *ty, const float *tz, double *loss, void *stream);
/* Reverse pass after nbx_adjoint_forward: dL/dx0, dL/dv0, dL/dm (device, n each). */
int nbx_adjoint_backward(nbx_ctx *ctx, nbx_adjoint *adj, const nbx_state *s, float *gx, float *gy,
                         float *gz, float *gvx, float *gvy, float *gvz, float *gm, void *stream);
/* Records all T steps from s (trees and lists) for nbx_adjoint_replay_fp64. */
int nbx_adjoint_record(nbx_ctx *ctx, nbx_adjoint *adj, const nbx_state *s, void *stream);
/* FP64 loss of the recorded trajectory from an FP64 initial state
 * (device double[7*n]: x,y,z,vx,vy,vz,m), structure and lists frozen. */
int nbx_adjoint_replay_fp64(nbx_ctx *ctx, nbx_adjoint *adj, const double *state0, double *loss,
                            void *stream);
/* Device bytes held by the adjoint, and the last forward / backward times. */
int nbx_adjoint_stats(nbx_adjoint *adj, int64_t *bytes, float *forward_ms, float *backward_ms);

/* FP64 diagnostics of bodies [0,n): out[0..2] momentum, out[3] kinetic energy,
 * out[4..6] angular momentum, out[7] total mass (device double[8]). */
int nbx_diagnostics_fp64(nbx_ctx *ctx, const nbx_state *s, int n, double *out, void *stream);

/* ---- checkpoint / resume -------------------------------------------------
 * The reference has none (it only writes frames).  A checkpoint is a raw dump
 * of every system's bodies (x, y, z, vx, vy, vz, m: the state a kick-drift step
 * needs) plus the system offsets, the step's constants (MAC constant,
 * softening, dt, dampening, compensation, key order), the walk's launch
 * shape, buffer variant and stack depth (which fix the order of the force
 * sums), the multipole order and the leaf bucket size, into a caller-owned host
 * buffer: a versioned header (80 bytes), the offsets, the
 * seven float arrays, and 64-bit checksums of header and payload.  Restoring
 * it into a context (capacity permitting) sets the systems, constants, walk
 * configuration, multipole order and leaf size and copies the bodies into the
 * caller's device state, so that the run continues bit for bit.  The sort's
 * digit width changes no result and is not recorded. */
int64_t nbx_checkpoint_bytes(int64_t nbodies, int nsystems);
/* Synchronises `stream`; *written receives the bytes used. */
int nbx_checkpoint_save(nbx_ctx *ctx, const nbx_state *s, void *host, int64_t capacity, int64_t *written,
                        void *stream);
/* NBX_ERR_FORMAT on a bad header, size or checksum (nothing is changed then);
 * NBX_ERR_ARG when the context is too small for it or uses another key order.
 * Synchronises `stream`. */
int nbx_checkpoint_restore(nbx_ctx *ctx, nbx_state *s, const void *host, int64_t bytes, void *stream);

/* ---- headless frame ------------------------------------------------------
 * The reference renderer's velocity-coloured dot splat
 * (3D/CUDA/CUDA_NBody/src/Renderer.cpp:54-147; constants Constants.h:31-38) into
 * a device RGB buffer instead of a window or file: rgb[3*(x + width*y) + c],
 * the payload of the reference's P6 frame.  Selection, colour ramp and pixel
 * mapping are FP64 like the reference; the dot weights are FP32.  */
typedef struct nbx_render_params {
    int width, height;          /* WIDTH, HEIGHT */
    double render_scale;        /* RENDER_SCALE */
    double max_velocity_color;  /* MAX_VEL_COLOR */
    double min_velocity_color;  /* MIN_VEL_COLOR */
    double particle_brightness; /* PARTICLE_BRIGHTNESS (>= 0) */
    double particle_sharpness;  /* PARTICLE_SHARPNESS */
    int dot_size;               /* DOT_SIZE (<= 16) */
    double system_size;         /* > 0; main.cu:95 passes 2 * BarnesHut::getSystemSize() */
} nbx_render_params;
void nbx_render_params_default(nbx_render_params *p);
/* Renderer::createFrame without the file (Renderer.cpp:37-52): accum is device
 * scratch of 3*width*height floats, rgb receives 3*width*height bytes.  Bodies
 * [0,n) of s (x, y, vx, vy, vz) are drawn; the context's sorted order is used
 * when its tree covers n bodies. */
int nbx_render_frame(nbx_ctx *ctx, const nbx_state *s, int n, const nbx_render_params *p, float *accum,
                     unsigned char *rgb, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NBX_H */
