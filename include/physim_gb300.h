/*
 * physim_gb300.h -- C ABI of libphysim_gb300.so, a GB300 (sm_103a) build of
 * physim's gravity + integration hot path.
 *
 * Two front doors:
 *
 *  1. A drop-in physim *transform plugin*.  The library exports exactly the
 *     symbols that physim's plugin loader binds for a C plugin
 *     (physim-core/src/plugin/discover.rs:327-373, plugin/transform.rs:32-104,
 *     c_plugin/plugin.c:133-284), for the three gravity elements of the astro
 *     crate: `astro` (quadtree Barnes-Hut), `astro2` (octree Barnes-Hut) and
 *     `simple_astro` (direct sum), astro/src/transformers.rs:16-271.  Element
 *     names, properties (`theta`, `e`) and the Entity layout are unchanged, so
 *     pipeline TOML files and CLI strings load it unchanged.
 *
 *  2. A device-resident C API (physim_gpu_*): the verlet, euler and rk4
 *     integrators (integrators/src/) over host arrays, and simulations whose
 *     state stays in HBM between steps.
 *
 * Types below have the layout of c_plugin/physim.h:6-94 (same type names;
 * enum constants carry a PHYSIM_ prefix).  All functions are thread-compatible:
 * one call at a time per object, as physim's pipeline does.
 */
#ifndef PHYSIM_GB300_H
#define PHYSIM_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------- */
/* Types shared with physim (c_plugin/physim.h)                             */
/* ----------------------------------------------------------------------- */

/* physim-core/src/plugin/meta.rs ElementKind (c_plugin/physim.h:6-13) */
typedef enum ElementKind {
    PHYSIM_KIND_INITIALISER = 0,
    PHYSIM_KIND_TRANSFORM = 1,
    PHYSIM_KIND_RENDER = 2,
    PHYSIM_KIND_SYNTH = 3,
    PHYSIM_KIND_TRANSMUTE = 4,
    PHYSIM_KIND_INTEGRATOR = 5
} ElementKind;

/* physim-core/src/messages.rs:29-36 -- messages posted from C must say C. */
typedef enum MessageOrigin { PHYSIM_ORIGIN_RUST = 0, PHYSIM_ORIGIN_C = 1 } MessageOrigin;

/* physim-core/src/messages.rs:11-19 */
typedef enum MessagePriority {
    PHYSIM_PRIORITY_BACKGROUND = 0,
    PHYSIM_PRIORITY_LOW = 1,
    PHYSIM_PRIORITY_NORMAL = 2,
    PHYSIM_PRIORITY_HIGH = 3,
    PHYSIM_PRIORITY_REALTIME = 4,
    PHYSIM_PRIORITY_CRITICAL = 5
} MessagePriority;

/* physim-core/src/messages.rs:38-46 */
typedef struct CMessage {
    MessagePriority priority;
    const char *topic;
    const char *message;
    uintptr_t sender_id;
    MessageOrigin origin;
} CMessage;

/* physim-core/src/lib.rs:16-29: 80 bytes, id at 64, fixed at 72. */
typedef struct Entity {
    double x;
    double y;
    double z;
    double vx;
    double vy;
    double vz;
    double radius;
    double mass;
    uintptr_t id;
    bool fixed;
} Entity;

/* physim-core/src/lib.rs:31-37 */
typedef struct Acceleration {
    double x;
    double y;
    double z;
} Acceleration;

/* physim-core/src/plugin/mod.rs RustStringAllocFn (host_alloc_string) */
typedef char *(*RustStringAllocFn)(const char *);

/* physim-core/src/plugin/transform.rs:32-50 (48 bytes of function pointers) */
typedef struct TransformElementAPI {
    void *(*init)(const uint8_t *, uintptr_t);
    void (*transform)(const void *, const Entity *, uintptr_t, Acceleration *, uintptr_t);
    void (*destroy)(void *);
    char *(*get_property_descriptions)(void *, RustStringAllocFn);
    void (*recv_message)(void *obj, const CMessage *msg);
    void (*post_configuration_messages)(void *obj);
} TransformElementAPI;

/* physim-core/src/plugin/meta.rs:94-106 */
typedef struct ElementMetaFFI {
    ElementKind kind;
    char *name;
    char *plugin;
    char *version;
    char *license;
    char *author;
    char *blurb;
    char *repo;
} ElementMetaFFI;

/* ----------------------------------------------------------------------- */
/* 1. Plugin discovery (physim-core/src/plugin/discover.rs:327-373,         */
/*    physim-core/src/plugin/mod.rs:118-160, c_plugin/plugin.c:133-147)     */
/* ----------------------------------------------------------------------- */

/* Returns "C": physim then skips its rustc-version check (discover.rs:345). */
const char *get_plugin_abi_info(void);
/* Returns "astro,astro2,simple_astro" (discover.rs:362-371). */
const char *register_plugin(void);
/* Stores physim's message-bus pointer (plugin/mod.rs:234-244).  The library
 * resolves physim's `post_bus_callback` (messages.rs:201-226) at run time. */
void set_callback_target(void *target);
/* Routes the configuration messages to `fn` instead of physim's
 * `post_bus_callback` (NULL restores the lookup), for hosts other than
 * physim's binary that mirror its message bus (messages.rs:201-226); the
 * message and its strings are valid during the call only.  physim itself
 * never calls this. */
typedef void (*PhysimBusFn)(void *target, const CMessage *message);
int physim_gpu_set_bus_callback(PhysimBusFn fn);

/* ----------------------------------------------------------------------- */
/* 1a. Transform elements.  Each set replaces the symbols that             */
/*     physim-attribute/src/lib.rs:39-202 generates for the element:        */
/*       astro2       -> AstroOctreeElement  astro/src/transformers.rs:114-203
 *       astro        -> AstroElement        astro/src/transformers.rs:16-112
 *       simple_astro -> SimpleAstroElement  astro/src/transformers.rs:205-271
 *
 *  init(json, len): a JSON object (not NUL-terminated).  Keys read:
 *    theta  (astro, astro2; default 1.0), e (all; absolute value; default 1.0)
 *  and, for this library only (ignored by the reference, so TOML stays valid):
 *    leaf_size  (astro, astro2; bodies per tree leaf, 1..64; default 1 = the
 *                reference's tree)
 *    traversal  ("exact": each body uses its own reference interaction list,
 *                the default; "warp": a cell is accepted only when every body
 *                of a 32-body warp accepts it)
 *    quadrupole (astro, astro2; true adds the cells' quadrupole moments;
 *                default false = the reference's monopole pseudo-particles)
 *    com_theta  (astro, astro2; > 0 also requires b_max < com_theta |x - c|
 *                to accept a cell, see PhysimSimConfig; default 0 = off)
 *    device     (CUDA device ordinal, default 0)
 *  Returns NULL for text that is not a JSON object (transform.rs:72-76).  It
 *  does not touch the GPU; the CUDA context is created by the first transform.
 *
 *  transform(obj, state, n, acc, n_acc): acc[i] += a_i for every non-fixed
 *  body i, as the reference does.  On a CUDA error or n_acc < n the library
 *  prints the reason to stderr and aborts, which is what the reference's
 *  catch_unwind wrapper does on a panic (physim-attribute/src/lib.rs:94-97).
 * ----------------------------------------------------------------------- */
const TransformElementAPI *astro2_get_api(void);
ElementMetaFFI astro2_register(RustStringAllocFn alloc);
void *astro2_init(const uint8_t *config, uintptr_t len);
void astro2_transform(const void *obj, const Entity *state, uintptr_t state_len,
                      Acceleration *acceleration, uintptr_t acceleration_len);
void astro2_destroy(void *obj);
char *astro2_get_property_descriptions(void *obj, RustStringAllocFn alloc);
void astro2_recv_message(void *obj, const CMessage *msg);
void astro2_post_configuration_messages(void *obj);

const TransformElementAPI *astro_get_api(void);
ElementMetaFFI astro_register(RustStringAllocFn alloc);
void *astro_init(const uint8_t *config, uintptr_t len);
void astro_transform(const void *obj, const Entity *state, uintptr_t state_len,
                     Acceleration *acceleration, uintptr_t acceleration_len);
void astro_destroy(void *obj);
char *astro_get_property_descriptions(void *obj, RustStringAllocFn alloc);
void astro_recv_message(void *obj, const CMessage *msg);
void astro_post_configuration_messages(void *obj);

const TransformElementAPI *simple_astro_get_api(void);
ElementMetaFFI simple_astro_register(RustStringAllocFn alloc);
void *simple_astro_init(const uint8_t *config, uintptr_t len);
void simple_astro_transform(const void *obj, const Entity *state, uintptr_t state_len,
                            Acceleration *acceleration, uintptr_t acceleration_len);
void simple_astro_destroy(void *obj);
char *simple_astro_get_property_descriptions(void *obj, RustStringAllocFn alloc);
void simple_astro_recv_message(void *obj, const CMessage *msg);
void simple_astro_post_configuration_messages(void *obj);

/* ----------------------------------------------------------------------- */
/* 2. Device-resident C API                                                 */
/* ----------------------------------------------------------------------- */

/* Status codes returned by every physim_gpu_* function. */
enum {
    PHYSIM_OK = 0,
    PHYSIM_ERR_ARGUMENT = 1, /* invalid argument (message in physim_gpu_last_error) */
    PHYSIM_ERR_CUDA = 2,     /* a CUDA runtime call failed */
    PHYSIM_ERR_MEMORY = 3,   /* host or device allocation failed / over budget */
    PHYSIM_ERR_TREE = 4,     /* tree build or traversal overflowed its bounds */
    PHYSIM_ERR_TIMEOUT = 5   /* a bounded device-side wait gave up */
};

/* Message for the last failing call on this thread ("" if none). */
const char *physim_gpu_last_error(void);

/* How the calls that take the caller's host arrays (the elements' transform
 * calls, physim_gpu_verlet_integrate) move them to and from the GPU.
 *   COPY:   cudaMemcpyAsync into device buffers and back.
 *   DIRECT: the kernels read and write the caller's arrays where they are,
 *           in contiguous block-wide runs.  Needs a device that reaches
 *           pageable host memory through the host's page tables
 *           (cudaDevAttrPageableMemoryAccessUsesHostPageTables: a Grace-
 *           Blackwell GPU over NVLink-C2C); a call on another device then
 *           fails with PHYSIM_ERR_ARGUMENT.
 *   AUTO:   DIRECT where the device supports it, else COPY (the default).
 * Results are bit-identical in every mode.  The setting is process-wide and
 * read at the start of each call. */
typedef enum PhysimHostAccess {
    PHYSIM_HOST_ACCESS_AUTO = 0,
    PHYSIM_HOST_ACCESS_COPY = 1,
    PHYSIM_HOST_ACCESS_DIRECT = 2
} PhysimHostAccess;
int physim_gpu_set_host_access(uint32_t mode);
/* The mode that calls on `device` use now: COPY or DIRECT. */
int physim_gpu_host_access(int32_t device, uint32_t *mode);

/* Gravity elements, by the reference's element names. */
typedef enum PhysimGravity {
    PHYSIM_GRAVITY_SIMPLE_ASTRO = 0, /* direct sum, transformers.rs:205-271 */
    PHYSIM_GRAVITY_ASTRO2 = 1,       /* octree Barnes-Hut, transformers.rs:114-203 */
    PHYSIM_GRAVITY_ASTRO = 2         /* quadtree Barnes-Hut, transformers.rs:16-112 */
} PhysimGravity;

typedef enum PhysimTraversal {
    PHYSIM_TRAVERSAL_EXACT = 0, /* per-body reference interaction lists */
    PHYSIM_TRAVERSAL_WARP = 1   /* a cell is accepted only if the whole warp accepts it */
} PhysimTraversal;

/* Cell expansion order of the Barnes-Hut force. */
typedef enum PhysimMultipole {
    PHYSIM_MULTIPOLE_MONOPOLE = 0,  /* the reference's pseudo-particle (astro/src/lib.rs:64-76) */
    PHYSIM_MULTIPOLE_QUADRUPOLE = 1 /* + second moments about the centre of mass */
} PhysimMultipole;

/* Integrator elements, by the reference's element names. */
typedef enum PhysimIntegratorKind {
    PHYSIM_INTEGRATOR_VERLET = 0, /* integrators/src/verlet.rs:19-121 (position Verlet) */
    PHYSIM_INTEGRATOR_EULER = 1,  /* integrators/src/euler.rs:11-49 (Taylor step) */
    PHYSIM_INTEGRATOR_RK4 = 2     /* integrators/src/rk4.rs:11-178 (4 force evaluations) */
} PhysimIntegratorKind;

/* Settings of one device-resident simulation. */
typedef struct PhysimSimConfig {
    uint32_t gravity;     /* PhysimGravity */
    uint32_t leaf_size;   /* Barnes-Hut bodies per leaf, 1..64 (1 = reference tree) */
    uint32_t traversal;   /* PhysimTraversal */
    uint32_t compensated; /* 1: FP32 pairs, compensated per-body sums; 0: plain FP32 sums */
    double theta;         /* opening parameter: extent/r < theta accepts a cell */
    double e;             /* easing factor added to r^2 (astro/src/lib.rs:95-98) */
    double dt;            /* integrator time step */
    void *stream;         /* cudaStream_t to run on; NULL: the simulation makes its own */
    int32_t device;       /* CUDA device ordinal */
    uint32_t integrator;  /* PhysimIntegratorKind */
    /* Accuracy options of astro/astro2 beyond the reference (0 = off, the
     * reference's monopole cells and opening rule): */
    uint32_t multipole;   /* PhysimMultipole */
    float com_theta;      /* also require b_max < com_theta * |x - c| to accept a
                           * cell (c its centre of mass, b_max = sqrt(3) extent +
                           * |c - centre| bounds its bodies' distance from c) */
} PhysimSimConfig;

/* Fills *cfg with the reference's defaults: simple_astro, theta 1.0, e 1.0,
 * dt 1e-6 (pipeline.rs:334), leaf 1, exact traversal, compensated sums,
 * verlet, monopole cells, no centre-of-mass guard. */
void physim_gpu_sim_config_default(PhysimSimConfig *cfg);

typedef struct PhysimSim PhysimSim;

/* Allocates device state for n bodies.  Nothing is uploaded yet. */
int physim_gpu_sim_create(const PhysimSimConfig *cfg, size_t n, PhysimSim **out);
/* Copies the host state in and clears the verlet history, so the next step
 * is the reference's Taylor first step (verlet.rs:24-50). */
int physim_gpu_sim_upload(PhysimSim *sim, const Entity *state, size_t n);
/* Enqueues `steps` pipeline steps, asynchronously on the simulation's stream:
 * gravity then the integrator's update; rk4 evaluates gravity four times per
 * step, at the stage states (rk4.rs:33-112).  Updates are f64 in the
 * reference's operation order, so given the same accelerations the new state
 * is bit-identical to the reference integrator's. */
int physim_gpu_sim_step(PhysimSim *sim, uint32_t steps);
/* The `cube` and `plummer` initialiser elements (astro/src/initialisers.rs:15-133,
 * :212-358) with the reference's properties, generated on the device.  The
 * reference's uniform variates come from a ChaCha8 stream that cannot be
 * reproduced; here variate k (0..2) of body i is the SplitMix64 finaliser of
 * seed + (3i + k + 1) * 0x9E3779B97F4A7C15, scaled to [0, 1) with 53 bits.  Given
 * the variates, positions, velocities, masses and radii follow the reference's
 * formulas in f64. */
typedef struct PhysimCubeParams {
    uint64_t seed;     /* default 0 */
    double spin;       /* v = (y, -x, 0) * spin, default 0 */
    double size;       /* x, y in [-size, size), z in [0, size), default 1 */
    double mass;       /* total mass, default 1 */
    double centre[3];  /* default (0, 0, 0) */
    uint64_t id;       /* default 0 */
} PhysimCubeParams;

typedef struct PhysimPlummerParams {
    uint64_t seed;     /* default 0 */
    double mass;       /* total mass, default 1 */
    double a;          /* Plummer radius, default 1 */
    double spin;       /* tangential speed factor, default 0 */
    double centre[3];  /* default (0, 0, 0) */
    double v[3];       /* bulk velocity, default (0, 0, 0) */
    uint64_t id;       /* default 0 */
} PhysimPlummerParams;

/* Fill the simulation's state with n = its body count generated bodies (like
 * physim_gpu_sim_upload: the next step is the Taylor first step). */
int physim_gpu_sim_init_cube(PhysimSim *sim, const PhysimCubeParams *p);
int physim_gpu_sim_init_plummer(PhysimSim *sim, const PhysimPlummerParams *p);
/* The same bodies written to a host Entity array (generated on `device`). */
int physim_gpu_generate_cube(const PhysimCubeParams *p, Entity *out, size_t n, int32_t device);
int physim_gpu_generate_plummer(const PhysimPlummerParams *p, Entity *out, size_t n,
                                int32_t device);

/* Waits for the stream, then copies the current state out.  This call, sim_accelerations
 * and sim_synchronize report a Barnes-Hut traversal stack overflow
 * (PHYSIM_ERR_TREE) or a radix-sort wait that gave up (PHYSIM_ERR_TIMEOUT) raised by
 * the kernels since the last check. */
int physim_gpu_sim_download(PhysimSim *sim, Entity *state, size_t n);
/* Waits, then writes the accelerations of the current state (not +=). */
int physim_gpu_sim_accelerations(PhysimSim *sim, Acceleration *acc, size_t n);
/* Waits, then writes the reference's direct-sum accelerations in f64 of the
 * bodies idx[0..count) of the current state to out[0..count): the pair law of
 * astro/src/lib.rs:84-113 with every f64 operation in the reference's order,
 * bodies at equal positions skipped, F/m_i (NaN for m_i = 0, 0 for fixed
 * bodies), summed over all bodies in a fixed tree order.  An accuracy
 * reference for every gravity element; f64 is slow on GB300, so sample
 * (16,384 bodies of 1,048,580 take about 2 s).  Indices must be < n. */
int physim_gpu_sim_accelerations_f64(PhysimSim *sim, const int64_t *idx, size_t count,
                                     Acceleration *out);
/* Waits for all work enqueued on the simulation's stream. */
int physim_gpu_sim_synchronize(PhysimSim *sim);
/* The cudaStream_t the simulation runs on. */
void *physim_gpu_sim_stream(PhysimSim *sim);
/* Pair-kernel plan of a simple_astro simulation: threads per block, bodies
 * per thread, j-range splits, candidates timed, whether every unordered pair
 * is evaluated once (and in how many body tiles of 1,024), time of one force
 * pass. */
typedef struct PhysimDirectTuning {
    uint32_t block;
    uint32_t ipt;
    uint32_t splits;
    uint32_t candidates;
    uint32_t symmetric;
    uint32_t tiles;
    double force_ms;
} PhysimDirectTuning;

/* Times every candidate pair-kernel plan on the simulation's bodies (force
 * passes only; the state is not advanced) and keeps the fastest.  The
 * simulation starts with a heuristic plan; this makes the choice by
 * measurement.  No-op for astro/astro2.  out may be NULL. */
int physim_gpu_sim_autotune(PhysimSim *sim, PhysimDirectTuning *out);
/* Sets the pair-kernel plan of a simple_astro simulation: the symmetric plan
 * (plan->symmetric != 0; compensated simulations only) or a one-pair kernel
 * of plan->block threads, plan->ipt bodies per thread and plan->splits
 * j-range splits.  Other fields are ignored. */
int physim_gpu_sim_set_plan(PhysimSim *sim, const PhysimDirectTuning *plan);
/* Largest slot buffer (bytes) the heuristic direct-sum plan of a simulation or
 * a simple_astro element may give the each-pair-once (symmetric) plan; 0
 * restores the default, a quarter of the device's memory.  The symmetric plan
 * is also skipped when its buffer plus 1 GiB exceeds the device's free memory
 * when the plan is made, and a symmetric plan whose allocation fails falls
 * back to a one-pair plan.  Process-wide, read when a plan is made.  This
 * builds on simple_astro (transformers.rs:219-244), which has no plans. */
int physim_gpu_set_symmetric_cap(uint64_t bytes);
/* The each-pair-once plan runs one block per pair of 1,024-body tiles while
 * that schedule's slot buffer (12 bytes per body per tile) is at most `bytes`
 * (0 restores the default, 4 GiB: up to about 600,000 bodies), and in
 * thread-block clusters over runs of tiles above that (slot sums 3T^2/32 x
 * 12 KB for T tiles: 1.2 GB instead of 12.9 GB at 1,048,580 bodies).  Both
 * give the same results within FP32 rounding.  Process-wide, read when a plan
 * is made.  No reference counterpart (simple_astro, transformers.rs:219-244,
 * has no plans). */
int physim_gpu_set_symmetric_pairs_limit(uint64_t bytes);
/* Barnes-Hut builds wait on other thread blocks only in the radix sort: its
 * decoupled look-back and, when its passes run as one launch, the barrier
 * between passes.  Every such wait gives up after `polls` polls that saw no
 * progress (0 restores the default, 2^20), raising an error flag: later
 * kernels of the build and the traversal then return at once and the next
 * synchronising call (physim_gpu_sim_synchronize / _download, the transform)
 * reports PHYSIM_ERR_TIMEOUT.  Process-wide, read when a build is enqueued or
 * captured.  No reference counterpart (the reference builds its tree on one
 * CPU thread, octree.rs:27-128). */
int physim_gpu_set_wait_limit(uint32_t polls);
/* How the Barnes-Hut build runs its 7-pass radix sort: `on` != 0 (default)
 * runs every pass in one cooperative launch where the device supports
 * cooperative launches (a grid barrier between passes, bounded by the wait
 * limit above), 0 runs one launch per pass.  The sorted order, and so every
 * result, is the same either way.  Process-wide, read when a build is enqueued
 * or captured.  No reference counterpart (octree.rs:27-128 sorts on one CPU
 * thread). */
int physim_gpu_set_sort_single_launch(int32_t on);
/* Test hook for the path above: tile `tile` (>= 0; -1 turns it off) of each
 * radix pass sees no predecessor word, so its wait always runs out.
 * Process-wide, read when a build is enqueued or captured. */
int physim_gpu_test_stall_sort(int32_t tile);
/* The current pair-kernel plan of a simple_astro simulation (block, ipt,
 * splits, symmetric, tiles; the other fields 0); all zero for astro/astro2. */
int physim_gpu_sim_plan(PhysimSim *sim, PhysimDirectTuning *out);
/* Number of kernel launches one step enqueues (for launch accounting). */
int physim_gpu_sim_launches_per_step(PhysimSim *sim);
/* Records CUDA events around the gravity kernels and the integrator of each
 * step (enable != 0); physim_gpu_sim_last_step_ms waits for the last step and
 * returns the two device times in milliseconds. */
int physim_gpu_sim_set_profiling(PhysimSim *sim, int enable);
int physim_gpu_sim_last_step_ms(PhysimSim *sim, double *gravity_ms, double *integrate_ms);
/* simple_astro with profiling on: device milliseconds of the last step's pair
 * kernel alone (the gravity time less the reduction of the symmetric plan's
 * slot sums). */
int physim_gpu_sim_last_pair_ms(PhysimSim *sim, double *pair_ms);
void physim_gpu_sim_destroy(PhysimSim *sim);

/* The Barnes-Hut tree of a simulation's current state, copied to host arrays
 * supplied by the caller (any pointer may be NULL).  Nodes are stored level by
 * level; the children of a node are contiguous and in octant order. */
typedef struct PhysimTreeSnapshot {
    size_t cap_nodes;      /* in: capacity of the node_* arrays */
    uint64_t *keys;        /* [n] Morton key of each sorted position */
    uint32_t *order;       /* [n] body index at each sorted position */
    int32_t *node_begin;   /* [cap] first sorted body of the node */
    int32_t *node_count;   /* [cap] bodies in the node */
    int32_t *node_child;   /* [cap] index of the first child, -1 for a leaf */
    uint8_t *node_nchild;  /* [cap] number of children */
    uint8_t *node_level;   /* [cap] depth below the root */
    double *node_centre;   /* [4*m] planes cx, cy, cz, half-width; m = min(n_nodes, cap);
                              f64 centres are kept with the exact traversal only (the warp
                              traversal keeps f32 geometry: the planes are then not written) */
    float *node_com;       /* [4*cap] centre of mass x, y, z and mass, per node */
    float *node_quad;      /* [8*m] second moments about the centre of mass (quadrupole
                            * builds): m x (Sxx, Syy, Szz, trace), then m x (Sxy, Sxz, Syz, 0) */
    size_t n_bodies;       /* out */
    size_t n_nodes;        /* out: nodes in the tree */
    double extent;         /* out: root half-width X (transformers.rs:126-132) */
    uint32_t flags;        /* out: bit 0 node arrays full (tree truncated), bit 1 stack
                            * overflow, bit 2 radix-sort look-back wait gave up */
} PhysimTreeSnapshot;

/* Builds the tree of the current state of an astro/astro2 simulation and
 * copies it out. */
int physim_gpu_sim_tree_snapshot(PhysimSim *sim, PhysimTreeSnapshot *out);
/* Whole-system diagnostics, summed in f64 on the device.  The potential is the
 * one whose gradient is the reference's pair force G m_a m_b / (r^2 + e)
 * (astro/src/lib.rs:84-113): V = -G m_a m_b atan(sqrt(e)/r)/sqrt(e), or
 * -G m_a m_b / r for e = 0, over pairs at distinct positions (physim's debug
 * energysink, debug/src/energysink.rs:35-99, reports K, V and dE with a
 * 1/r potential). */
typedef struct PhysimDiagnostics {
    double mass;
    double centre_of_mass[3];
    double momentum[3];
    double kinetic;
    double potential; /* 0 unless requested (it is an O(N^2) pass) */
    double energy;    /* kinetic + potential */
} PhysimDiagnostics;

/* Waits for the stream; with_potential != 0 also evaluates the potential. */
int physim_gpu_sim_diagnostics(PhysimSim *sim, PhysimDiagnostics *out, int with_potential);

/* The same diagnostics of a host Entity array, for a sink that receives the
 * pipeline's states: the computation behind physim's `energysink` element
 * (debug/src/energysink.rs:35-99), which prints K, V and the change of E and
 * turns its potential on when a gravity element posts ("energysink",
 * "gravity") (energysink.rs:112-117, transformers.rs:107-111).  All sums are
 * f64 (pair terms FP32, see physim_gpu_sim_diagnostics): V is the total over
 * every pair (energysink.rs:86 keeps only the last pair, `=` for `+=`), with
 * e = 0 the reference sink's -m_a m_b / r, with e > 0 the potential whose
 * gradient is the reference's softened force.  The state is copied to the
 * device; one call at a time per object. */
typedef struct PhysimEnergy PhysimEnergy;
int physim_gpu_energy_create(int32_t device, PhysimEnergy **out);
int physim_gpu_energy_compute(PhysimEnergy *energy, const Entity *state, size_t n, double e,
                              int with_potential, PhysimDiagnostics *out);
void physim_gpu_energy_destroy(PhysimEnergy *energy);

/* Waits for the stream, then reports the most recent Barnes-Hut traversal:
 * node visits (one per warp and node), pair interactions (per body) and,
 * with profiling on, the traversal kernel's device time (else -1). */
int physim_gpu_sim_bh_stats(PhysimSim *sim, uint64_t *node_visits, uint64_t *interactions,
                            double *traversal_ms);

/* ----------------------------------------------------------------------- */
/* Batched ensembles: many independent simple_astro + verlet simulations of  */
/* uneven size, advanced together by one persistent pair kernel per step    */
/* (a work queue of (member, i tile, j chunk) units), captured in a graph.   */
/* ----------------------------------------------------------------------- */
typedef struct PhysimEnsemble PhysimEnsemble;

typedef struct PhysimEnsembleTuning {
    uint32_t block;        /* threads per block of the pair kernel */
    uint32_t ipt;          /* bodies per thread */
    uint32_t chunk_bodies; /* j bodies per work unit */
    uint32_t candidates;   /* plans timed */
    uint32_t symmetric_from; /* members from this many bodies evaluate each
                              * unordered pair once (0: none) */
    uint32_t reserved;
    double force_ms;       /* time of one pair-kernel pass with the chosen plan */
} PhysimEnsembleTuning;

/* Members 0..count-1 hold sizes[k] bodies each.  cfg supplies the device,
 * stream, compensated flag and the default e and dt (gravity must be
 * simple_astro).  Members take no steps until they are uploaded. */
int physim_gpu_ensemble_create(const PhysimSimConfig *cfg, const size_t *sizes, size_t count,
                               PhysimEnsemble **out);
/* Copies a member's state in; its next step is the Taylor first step and it
 * steps without limit until set_member says otherwise. */
int physim_gpu_ensemble_upload(PhysimEnsemble *ens, size_t index, const Entity *state, size_t n);
/* Per-member easing factor, time step and number of steps still to take
 * (UINT64_MAX: unlimited; 0: the member is skipped by the kernels). */
int physim_gpu_ensemble_set_member(PhysimEnsemble *ens, size_t index, double e, double dt,
                                   uint64_t steps_remaining);
/* Times every candidate kernel shape and j-chunk length on the members' data
 * (force passes only; the state is not advanced) and keeps the fastest. */
int physim_gpu_ensemble_autotune(PhysimEnsemble *ens, PhysimEnsembleTuning *out);
/* Re-sizes member `index` to n bodies, 0 <= n <= the count it was created
 * with, reusing its slot (continuous batching: a finished member's slot takes
 * the next job).  Waits for the stream; the member takes no steps until it is
 * uploaded (n bodies) and given a step budget by set_member. */
int physim_gpu_ensemble_resize_member(PhysimEnsemble *ens, size_t index, size_t n);
/* Enqueues `steps` steps of every member with steps left (asynchronous). */
int physim_gpu_ensemble_step(PhysimEnsemble *ens, uint32_t steps);
int physim_gpu_ensemble_download(PhysimEnsemble *ens, size_t index, Entity *state, size_t n);
/* Waits, then copies per-member steps taken / steps remaining (either may be NULL). */
int physim_gpu_ensemble_progress(PhysimEnsemble *ens, uint64_t *steps_done, uint64_t *remaining);
int physim_gpu_ensemble_synchronize(PhysimEnsemble *ens);
void *physim_gpu_ensemble_stream(PhysimEnsemble *ens);
int physim_gpu_ensemble_launches_per_step(PhysimEnsemble *ens);
void physim_gpu_ensemble_destroy(PhysimEnsemble *ens);

/* simple_astro accelerations for callers that cannot allocate device memory.
 * This entry point has no counterpart in the reference.  It serves code that
 * must not call cudaMalloc (a framework's memory pool or arena, a real-time
 * loop, a process whose device memory is handed out up front): the caller
 * passes device-accessible arrays, state[n] (read) and acc[n] (acc[i] += a_i
 * for every non-fixed body, as simple_astro_transform does), and the work is
 * enqueued on `stream` (a cudaStream_t; NULL: the legacy default stream).
 * Pageable host arrays are rejected with PHYSIM_ERR_ARGUMENT on a device
 * without pageable memory access, and device arrays of another device.
 * Scratch lives in one static device array of about 7.9 MiB that every GPU
 * loading the library holds until exit; at most 65,536 bodies (larger n is
 * rejected with PHYSIM_ERR_ARGUMENT).  The first call on a device looks up
 * that array's device address and keeps it for the life of the process, so
 * make it before any stream capture, and do not call this entry point after
 * a cudaDeviceReset of a device it was used on.  All calls share the array:
 * calls that overlap on the GPU race. */
int physim_gpu_simple_astro_accumulate_static(const Entity *state, size_t n, double e,
                                              Acceleration *acc, void *stream);

/* Verlet integrator over host arrays (integrators/src/verlet.rs:19-121).
 * A Rust IntegratorElement shim evaluates acc_fn itself and hands the
 * accelerations over; the step runs on the GPU in f64 in the reference's
 * operation order, so new_state is bit-identical to the reference's. */
typedef struct PhysimVerlet PhysimVerlet;
int physim_gpu_verlet_create(int32_t device, PhysimVerlet **out);
int physim_gpu_verlet_integrate(PhysimVerlet *v, const Entity *entities, Entity *new_state,
                                size_t n, const Acceleration *acc, double dt);
void physim_gpu_verlet_destroy(PhysimVerlet *v);

/* Any of the three integrators over host arrays, in the shape of physim's
 * IntegratorElement::integrate(entities, new_state, acc_fn, dt)
 * (physim-core/src/plugin/integrator.rs:5-13): the library calls acc_fn once
 * (verlet, euler) or four times (rk4) with a host state and zeroed host
 * accelerations that acc_fn adds into (physim's transform_fn,
 * pipeline.rs:137-141), and computes the stage states and the update on the
 * GPU in f64 in the reference's operation order.  This is what a Rust
 * IntegratorElement shim for `verlet`, `euler` or `rk4` binds
 * (verlet_create_element etc., physim-attribute/src/lib.rs:384-427).
 * verlet keeps previous_state on the device between calls (verlet.rs:102). */
typedef void (*PhysimAccFn)(void *user, const Entity *state, size_t n, Acceleration *acc);
typedef struct PhysimIntegrator PhysimIntegrator;
int physim_gpu_integrator_create(uint32_t kind, int32_t device, PhysimIntegrator **out);
int physim_gpu_integrator_integrate(PhysimIntegrator *it, const Entity *entities,
                                    Entity *new_state, size_t n, PhysimAccFn acc_fn, void *user,
                                    double dt);
void physim_gpu_integrator_destroy(PhysimIntegrator *it);

#ifdef __cplusplus
}
#endif

#endif /* PHYSIM_GB300_H */
