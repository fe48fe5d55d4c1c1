/*
 * ag2.h -- C-ABI of the GB300 (sm_103a) implementation of AstroGen2's force hot
 * path: octree build, SPH density, Barnes-Hut walk with in-walk SPH force, and
 * the leapfrog kick/drift.
 *
 * Every entry point returns an int status (AG2_OK = 0, negative = AG2_E_*).
 * Work is ordered on the context's CUDA stream; calls that hand results back
 * to host memory synchronise that stream.  One context per host thread.  Host
 * buffers are only borrowed for the duration of a call.  Quantities are FP64
 * in the caller's units with gravitational constant params.G (1 for code
 * units).
 *
 * Mapping to the reference (simulation/src/...):
 *   ag2_build_tree      Tree::buildTree            Physics/Tree/Tree.cpp:24-55
 *                       (+ Node::insert            Physics/Tree/Node.cpp:405-534, 597-719)
 *   ag2_root_radius     Tree::calcTreeWidth        Physics/Tree/Tree.cpp:86-117
 *   ag2_visual_density  Tree::calcVisualDensity    Physics/Tree/Tree.cpp:152-175, Node.cpp:832-877
 *   ag2_sph_density     Tree::calcGasDensity       Physics/Tree/Tree.cpp:119-150, Node.cpp:722-796
 *   ag2_forces          Tree::calculateForces      Physics/Tree/Tree.cpp:57-83, Node.cpp:88-172, 247-399
 *   ag2_kick            TimeIntegration::Kick      Physics/TimeIntegration.cpp:10-19
 *   ag2_drift           TimeIntegration::Drift     Physics/TimeIntegration.cpp:21-25
 *   ag2_ueuler          TimeIntegration::Ueuler    Physics/TimeIntegration.cpp:28-40
 *   ag2_step            one pass of the step loop  Physics/Simulation.cpp:256-341
 *   ag2_upload/download Simulation::particles       Physics/Simulation.h:70, Physics/Particle.h:9-57
 */
#ifndef AG2_C_ABI_H_
#define AG2_C_ABI_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AG2_ABI_VERSION 1

enum ag2_status {
    AG2_OK = 0,
    AG2_E_INVALID = -1,     /* bad argument or state (e.g. forces before a tree) */
    AG2_E_CUDA = -2,        /* a CUDA runtime call failed */
    AG2_E_NOMEM = -3,       /* device allocation failed */
    AG2_E_COINCIDENT = -4,  /* particles too close to separate: the reference recurses without end */
    AG2_E_DEPTH = -5,       /* octree deeper than AG2_MAX_DEPTH levels */
    AG2_E_STACK = -6,       /* walk stack overflow (reported by the kernel, no fault) */
    AG2_E_NAN = -7,         /* non-finite particle position */
    AG2_E_CAPACITY = -8,    /* more particles than the context was created for */
    AG2_E_FORMAT = -9,      /* unknown format, or a file the reference's reader rejects or reads past its end */
    AG2_E_IO = -10          /* a file could not be opened, read or written */
};

#define AG2_MAX_DEPTH 96

enum ag2_precision {
    AG2_PREC_FP64 = 0,      /* plain walk: all arithmetic in FP64 */
    AG2_PREC_FP32 = 1       /* FP32 offsets from the walk group's centre + compensated sums */
};

enum ag2_field {
    AG2_POS = 0,   /* 3n doubles, xyz interleaved */
    AG2_VEL = 1,   /* 3n */
    AG2_ACC = 2,   /* 3n */
    AG2_MASS = 3,  /* n  */
    AG2_H = 4,     /* n  smoothing length */
    AG2_RHO = 5,   /* n  */
    AG2_P = 6,     /* n  */
    AG2_T = 7,     /* n  */
    AG2_U = 8,     /* n  internal energy */
    AG2_DUDT = 9,  /* n  */
    AG2_VDENS = 10, /* n  visualDensity */
    AG2_TSTEP = 11, /* n  block time step of the particle (ag2_block_init) */
    AG2_TNEXT = 12  /* n  its next integration time */
};

typedef struct ag2_params {
    double G;             /* gravitational constant */
    double e0;            /* softening length, Simulation::e0 */
    double theta;         /* opening angle, Simulation::theta */
    double massInH;       /* SPH neighbour mass, Simulation::massInH */
    int32_t split_threshold; /* Node::insert switches to serial insertion below this
                                many particles; the reference uses
                                omp_get_max_threads()*100 (Node.cpp:420) */
    int32_t precision;    /* enum ag2_precision */
    int32_t group_size;   /* particles per FP32/FP64 walk group, 1..32 (0 = 32); ag2_autotune_walk
                             may change it */
    int32_t reserved;
} ag2_params;

typedef struct ag2_ctx ag2_ctx;

/* Defaults: G = 1, e0 = 0.01, theta = 0.5, massInH = 0, split_threshold = 100,
 * FP32 walk, group_size 32. */
void ag2_default_params(ag2_params *p);

/* Create a context on the current CUDA device for up to `capacity` particles.
 * All device memory is allocated here (and grown by ag2_build_tree when the
 * octree outgrows its node pool). */
int ag2_create(ag2_ctx **ctx, const ag2_params *params, size_t capacity);
int ag2_destroy(ag2_ctx *ctx);
int ag2_set_params(ag2_ctx *ctx, const ag2_params *params);
int ag2_get_params(const ag2_ctx *ctx, ag2_params *params);
/* Order all work on `stream` (a cudaStream_t; NULL = the context's own stream). */
int ag2_set_stream(ag2_ctx *ctx, void *stream);
const char *ag2_last_error_string(const ag2_ctx *ctx);

/* Copy n particles in: FP64 xyz position/velocity, mass, internal energy U and
 * type (1 star, 2 gas, 3 dark matter).  vel/U may be NULL (zero).  Clears
 * acc, dUdt, h, rho, P, T and visualDensity, drops any tree.  The _device
 * variant takes device pointers. */
int ag2_upload(ag2_ctx *ctx, size_t n, const double *pos, const double *vel, const double *mass,
               const double *U, const uint8_t *type);
int ag2_upload_device(ag2_ctx *ctx, size_t n, const double *pos, const double *vel, const double *mass,
                      const double *U, const uint8_t *type);
/* Overwrite one field (host or device buffer) in the original particle order. */
int ag2_set_field(ag2_ctx *ctx, int field, const double *src, int src_is_device);
/* Read one field back in the original particle order (host or device buffer). */
int ag2_download(ag2_ctx *ctx, int field, double *dst, int dst_is_device);
/* One step of the reference's loop with the caller's particle arrays as its
 * source and destination (upload order, host memory): ag2_upload(pos, vel,
 * mass, U, type) and ag2_set_field(ACC, acc), ag2_step(dt, hubble_factor,
 * with_visual_density, visualDensityRadius), then pos/vel/acc/U read back into
 * the *_out arrays (a NULL input is not uploaded, a NULL output not read).
 * The positions' read-back overlaps the walk (they are final after the
 * drift).  The out arrays may be the input arrays.  With first != NULL the
 * particles are n_inst simulations, as ag2_set_instances(n_inst, first,
 * massInH) after the upload.
 * Host memory: the read-backs are asynchronous copies into the *_out arrays
 * while later stages run.  They overlap the device work only when the arrays
 * are page-locked (cudaHostAlloc / cudaHostRegister); with pageable memory each
 * copy blocks until it has landed and the stages after it queue behind it.
 * The arrays are written until the call returns, on success and on failure
 * alike (a failing call waits for the copies it started before returning).
 * The first call with acc != NULL allocates a staging buffer of 3 doubles per
 * particle of capacity for the accelerations (kept until ag2_destroy), whose
 * copy then runs beside the gather of the other fields. */
typedef struct ag2_host_io {
    const double *pos, *vel, *mass, *U, *acc;
    const uint8_t *type;
    double *pos_out, *vel_out, *acc_out, *U_out;
    int32_t n_inst;
    const int64_t *first;
    const double *massInH;
} ag2_host_io;
int ag2_step_host(ag2_ctx *ctx, size_t n, double dt, double hubble_factor, int with_visual_density,
                  double visualDensityRadius, const ag2_host_io *io);
/* Several fields to host buffers in one call, as ag2_download each: the
 * gather of one field into upload order runs while the previous one crosses
 * to the host, and the call returns once every copy has landed (also when it
 * fails).  The overlap needs page-locked destination buffers; pageable ones
 * are filled one copy after another. */
int ag2_download_fields(ag2_ctx *ctx, int nfields, const int *fields, double *const *dst);
/* Host-side fault injection for tests of the error paths: with site 1 the
 * next ag2_step_host fails with `code` (an AG2_E_* value) right after the walk
 * and its check, as it would when the walk reports AG2_E_STACK, with the
 * position and acceleration read-backs already queued.  Site 0 clears it.
 * Nothing on the device is made to fail.  No counterpart in the reference. */
int ag2_inject_fault(ag2_ctx *ctx, int site, int code);
size_t ag2_count(const ag2_ctx *ctx);

/* Independent simulations in one context (the batched ensemble and the
 * serving loop): after ag2_upload, instance k is the particles with upload
 * indices [first[k], first[k+1]) (first[0] = 0, first[n_inst] = n).  Each
 * instance gets its own octree (root half-width, modes, moments), its own SPH
 * neighbour mass (massInH[k]; NULL = params.massInH) and its own walk groups, so
 * its results do not depend on what else shares the context; every hot-path
 * call below then processes all instances at once.  ag2_upload resets the
 * layout to one instance that follows params.massInH; a layout set here (even
 * of one instance) keeps its own massInH until the next upload. */
int ag2_set_instances(ag2_ctx *ctx, int32_t n_inst, const int64_t *first, const double *massInH);
int ag2_instance_radius(ag2_ctx *ctx, int32_t instance, double *radius);

/* Hot path.  The tree is device resident until the next build or upload. */
int ag2_build_tree(ag2_ctx *ctx);
int ag2_visual_density(ag2_ctx *ctx, double visualDensityRadius);
int ag2_sph_density(ag2_ctx *ctx);
int ag2_forces(ag2_ctx *ctx);
int ag2_kick(ag2_ctx *ctx, double dt);
int ag2_drift(ag2_ctx *ctx, double dt);
int ag2_kick_drift(ag2_ctx *ctx, double dt);
int ag2_ueuler(ag2_ctx *ctx, double dt);
int ag2_scale_positions(ag2_ctx *ctx, double factor);
/* One step of Simulation::run with every particle active at the same dt:
 * kick+drift, build, [visual density], SPH density, forces, Ueuler (gas),
 * Hubble factor, kick. */
int ag2_step(ag2_ctx *ctx, double dt, double hubble_factor, int with_visual_density,
             double visualDensityRadius);
/* Run every later ag2_step as a replay of a CUDA graph captured from it (enable
 * = 1) or as separate launches (0, the default).  The graph holds the whole
 * step; the build's data-dependent parts (the level loop, the moments levels)
 * are conditional WHILE nodes whose conditions the device sets, so a step
 * needs no host round trip.  Graphs are captured again when the particle set,
 * the instance layout, the parameters, the stream, dt, the Hubble factor or a
 * pool size change.  The node pool is sized for twice the last tree; a tree
 * that outgrows it fails the step with AG2_E_NOMEM (redo it after a plain
 * ag2_build_tree, which grows the pool). */
int ag2_step_graphs(ag2_ctx *ctx, int enable);
/* Block time steps (Simulation.cpp:188-341 with minTimeStep < maxTimeStep).
 * ag2_block_init gives every particle the step eta*sqrt(e0/|a|) clamped to
 * [min_dt, max_dt] and floored to a power of two (min_dt when a = 0), from the
 * current acc (after the initial ag2_forces), and its next integration time
 * global_time + step.  Each ag2_block_step then: renews the steps of particles
 * whose time has come; advances the global time to the earliest next
 * integration time; kicks and drifts the particles due then; builds the tree,
 * visual density (with_visual) and gas density over all particles; walks the
 * due particles only; closes them (Ueuler for gas, position *= exp(H0*step),
 * kick) and schedules their next time.  *global_time and *active return the new
 * time and the number of due particles.  AG2_TSTEP / AG2_TNEXT read the state. */
int ag2_block_init(ag2_ctx *ctx, double eta, double min_dt, double max_dt, double global_time);
int ag2_block_step(ag2_ctx *ctx, double H0, int with_visual, double Rv, double *global_time, int64_t *active);

/* Walk autotuner.  Times each FP32-walk candidate on the current tree and
 * keeps the fastest for later ag2_forces calls of this context.  A candidate
 * is a compiled variant (register budget per thread and first-pass stack
 * depth, which together set the warps resident per SM, and whether the child
 * records of nodes to open are prefetched into L1) with a walk group size
 * (particles per warp group: 32 or 16).  The chosen group size is written to
 * the context's params.group_size.  Variant and stack depth do not change the
 * results; the group size changes the FP32 sums in their last bits, within
 * the walk's accuracy contract.  ag2_autotune returns the chosen variant;
 * ag2_autotune_walk also reports every candidate with its time (up to max
 * entries; *count = candidates timed, *chosen = index of the choice). */
typedef struct ag2_walk_config {
    int32_t variant;        /* compiled variant of the FP32 walk */
    int32_t regs;           /* register budget per thread (0 = the compiler's choice) */
    int32_t blocks_per_sm;  /* resident 4-warp blocks per SM the budget is built for (0 = compiler) */
    int32_t stack;          /* first-pass stack entries per warp (deeper groups go to a retry pass) */
    int32_t prefetch;       /* 1: child records of nodes pushed for opening are prefetched into L1 */
    int32_t group_size;     /* particles per walk group */
    float ms;               /* measured walk time on the context's tree */
} ag2_walk_config;
int ag2_autotune(ag2_ctx *ctx, int *variant);
int ag2_autotune_walk(ag2_ctx *ctx, int max, ag2_walk_config *out, int *count, int *chosen);
/* Use FP32-walk variant `variant` (an ag2_walk_config.variant, 0..5) without
 * timing anything, e.g. a choice kept from an earlier ag2_autotune_walk;
 * the group size is params.group_size. */
int ag2_set_walk_variant(ag2_ctx *ctx, int variant);

/* Phase timers (CUDA events on the context's stream).  When enabled,
 * ag2_build_tree records its sub-phases and ag2_step records the phases the
 * reference logs with Log::startProcess (Simulation.cpp:256-351: "first kick",
 * "build tree", "Visual Density", "SPH density and update", "Force
 * Calculation", "second kick").  ag2_phase_times copies up to max phase names
 * and durations (ms) of the last measured call and returns how many there are. */
int ag2_phase_timing(ag2_ctx *ctx, int enable);
int ag2_phase_times(const ag2_ctx *ctx, int max, const char **names, float *ms);

/* Tree introspection (synchronises). */
int ag2_root_radius(ag2_ctx *ctx, double *radius);
int ag2_node_count(ag2_ctx *ctx, int64_t *nodes, int64_t *internal, int32_t *max_depth);
/* Depth-first preorder export, children in octant order 0..7, same layout as the
 * checker's orc_topology.  Arrays hold `nodes` entries (any may be NULL); the
 * particle index is the original upload index. */
int ag2_topology(ag2_ctx *ctx, int32_t *depth, int32_t *is_leaf, int32_t *particle, int64_t *cp_count,
                 uint64_t *cp_hash, double *mass, double *com3, double *gas_mass, double *mvel3,
                 double *center3, double *radius);
/* The FP32 walk's node records in ag2_topology's numbering, 16 floats per node
 * (zeros for an empty node): centre of mass as hi floats and mass * ls^2; the
 * lo floats of the centre of mass and (radius * ls / theta)^2 (-1 for a leaf);
 * first child, leaf particle slot, child mask and 0 as int32 bits; gas velocity
 * and gasMass * ls^2 (zeros for a node that holds no gas mass).  ls = 2^k with k = 1022 - (the biased exponent of the
 * instance's root half-width), so scaled lengths are below 1.  A diagnostic of
 * the records the reference's calculateGravityForce reads as doubles
 * (Node.cpp:285-305); the reference has no such view. */
int ag2_walk_records(ag2_ctx *ctx, float *out16);
/* For each particle (original upload order): the preorder index, in the
 * ag2_topology numbering, of the node the reference's Particle::node points at
 * after the build (its leaf; see Node.cpp:412-413, 621-625), or -1 for null. */
int ag2_particle_node(ag2_ctx *ctx, int64_t *out);
/* Interactions counted by the last ag2_forces: gravity (P2P + accepted nodes)
 * and SPH pairs. */
int ag2_interactions(ag2_ctx *ctx, int64_t *gravity, int64_t *sph);
/* Diagnostics.  FP64 direct summation with the reference's softened pair law
 * (Node.cpp:285-305) for `ns` particles given by upload index: out[3k..3k+2] =
 * acceleration of particle ids[k] due to all others (host buffers).  No
 * counterpart in the reference beyond its unused, unsoftened
 * Simulation::calculateForcesWithoutOctree (Simulation.cpp:367-382). */
int ag2_direct_sum(ag2_ctx *ctx, size_t ns, const int64_t *ids, double *out);
/* out[0..7] = total mass, kinetic energy, momentum xyz, angular momentum xyz. */
int ag2_diagnostics(ag2_ctx *ctx, double *out8);
/* Energy of the current state: out[0] kinetic sum m v^2 / 2, out[1] potential
 * sum m phi / 2, out[2] thermal sum over gas of m U, out[3] their total.  phi
 * is the potential of the walk's own pair force G m / (r^2 + e0^2) along d/r
 * (Node.cpp:285-305 with e0 < 0.6), -(G m / e0) atan(e0 / r), summed over the
 * nodes and particles the FP64 walk accepts (the same opening rule, FP64).
 * Needs a tree built from the current positions (after ag2_build_tree or
 * ag2_step); AG2_E_INVALID for e0 outside (0, 0.6).  No counterpart in the
 * reference, which computes no potential; this is the energy-drift check. */
int ag2_energy(ag2_ctx *ctx, double *out4);
/* FP32 FMA throughput of this GPU in GFLOP/s (roofline denominator of the walk). */
int ag2_fp32_peak_probe(ag2_ctx *ctx, double *gflops);
/* Allocation-free root half-width.  No counterpart in the reference: it computes
 * the same quantity as ag2_root_radius (Tree::calcTreeWidth) for callers that
 * cannot allocate device memory, such as a host code that has reserved the
 * GPU's memory for its own pools or code in the middle of capturing a CUDA
 * stream into a graph.  The caller passes device buffers: pos holds n
 * xyz-interleaved doubles, radius receives one double; the work is enqueued on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) and nothing is
 * allocated.  Scratch space is a fixed 32 KiB array inside this library on each
 * device that uses it, kept until the process exits.  The first call on a
 * device looks up that array's address (make it before any stream capture).
 * Calls that overlap on the GPU share the array and race.  n must lie in
 * 1..AG2_NOALLOC_MAX_PARTICLES; larger n returns AG2_E_CAPACITY and launches
 * nothing. */
#define AG2_NOALLOC_MAX_PARTICLES 8355840
int ag2_root_radius_noalloc(const double *pos, int64_t n, double *radius, void *stream);

/* Snapshot and initial-condition files of the reference's DataManager
 * (File/DataManager.h:13-91, DataManager.cpp:86-1337).  The formats are the
 * values of its outputDataFormat / inputDataFormat keys: */
enum ag2_format {
    AG2_FMT_AG = 0,      /* "ag": FP64 records (position, mass, T, visualDensity, sfr, type, galaxyPart, id) */
    AG2_FMT_AGC = 1,     /* "agc": FP32 records (position, visualDensity, sfr, T, type, galaxyPart) */
    AG2_FMT_AGE = 2,     /* "age": FP64 records (position, velocity, mass, T, P, visualDensity, U, type, galaxyPart, id) */
    AG2_FMT_GADGET = 3,  /* "gadget": Gadget-2 format 1 (kpc, km/s, 1e10 Msun, U / 1e6) */
    AG2_FMT_MAKEGAL = 4  /* "makeGal": Gadget-2 format 2 with block labels (input only) */
};

/* Per-particle values that the hot path carries along unchanged, in upload
 * order: Particle::id, Particle::galaxyPart (1 disk, 2 bulge, 3 halo) and
 * Particle::sfr.  ag2_upload sets id = upload index, galaxyPart = 1, sfr = 0;
 * ag2_load_ics sets what the file holds.  NULL arguments are left alone. */
int ag2_set_tags(ag2_ctx *ctx, const uint32_t *id, const uint8_t *galaxy_part, const double *sfr, int src_is_device);
int ag2_get_tags(ag2_ctx *ctx, uint32_t *id, uint8_t *galaxy_part, double *sfr, int dst_is_device);

/* DataManager::saveData (DataManager.cpp:86-424) of the first `count`
 * particles in upload order (numParticlesOutput; count <= ag2_count).  The
 * file image is encoded on the device from the resident state, byte for byte
 * the reference's layout; the 4 padding bytes of the ag/agc/age header, which
 * the reference leaves uninitialised, are zero.  Gadget ignores delta_time and
 * end_time and stores current_time as the header's time.
 * ag2_snapshot_size: bytes of the image (exact for ag/agc/age, an upper bound
 * for gadget, whose particle lists depend on type and galaxyPart).
 * ag2_snapshot_encode: the image into host memory dst (dst_cap bytes), *len =
 * its length; synchronous.
 * ag2_snapshot_write: the image into the file `path`.  With async = 1 the call
 * returns once the encode and the device-to-host copy are queued; a background
 * thread waits for the copy and writes the file while later calls run on the
 * device.  With ag2_phase_timing on, ag2_snapshot_encode records the phases
 * "snapshot encode" and "snapshot copy", ag2_load_ics "ic copy" and "ic decode".  ag2_snapshot_wait joins it and returns the write's status; the next
 * snapshot, ag2_load_ics and ag2_destroy join it first. */
int ag2_snapshot_size(ag2_ctx *ctx, int format, int64_t count, size_t *bytes);
int ag2_snapshot_encode(ag2_ctx *ctx, int format, int64_t count, double delta_time, double end_time,
                        double current_time, void *dst, size_t dst_cap, size_t *len);
int ag2_snapshot_write(ag2_ctx *ctx, int format, int64_t count, double delta_time, double end_time,
                       double current_time, const char *path, int async);
int ag2_snapshot_wait(ag2_ctx *ctx);

/* DataManager::loadICs (DataManager.cpp:434-1332) into the context: the file
 * is read once into pinned memory, copied to the device as it is, and decoded
 * there into the particle arrays (as ag2_upload does, plus T, P,
 * visualDensity and the tags where the format holds them), in file order.
 * The reference's own units conversions apply (gadget and makeGal: kpc, km/s,
 * 1e10 Msun, U * 1e6).  The reference's makeGal reader shuffles the particles
 * with an unseeded generator and Simulation::init shuffles again; neither
 * shuffle is done here.  times3 (may be NULL) receives the header's
 * deltaTime, endTime and currentTime (ag/agc/age) or 0, 0, time (gadget,
 * makeGal).  ag2_ic_count reads the particle count of a file's header. */
int ag2_ic_count(const char *path, int format, int64_t *n);
int ag2_load_ics(ag2_ctx *ctx, const char *path, int format, double *times3);

/* Number of kernels this library launched since the context was created. */
int64_t ag2_launch_count(const ag2_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
