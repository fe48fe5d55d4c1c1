// ag2_internal.cuh -- device-side layout of the AstroGen2 GB300 hot path.
//
// Particle state lives in HBM as structure-of-arrays in *tree order*: every
// ag2_build_tree re-sorts it so that each octree node owns a contiguous range
// of particles and each walk group (32 consecutive particles) is spatially
// compact.  `id` maps a tree-order slot back to the caller's upload index.
//
// The octree is a pool of nodes in structure-of-arrays form.  Every split node
// owns 8 consecutive children (empty ones included, exactly as the reference's
// Node::insert creates all 8, Node.cpp:433-443 / 630-642), so the node count
// equals the reference's.  Nodes of one level are contiguous in the pool.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "ag2.h"

namespace ag2 {

// Node modes: how Node::insert(vector, cores) treats the node (Node.cpp:405-428).
enum NodeMode : uint8_t {
    MODE_EMPTY = 0,      // nothing routed here
    MODE_PAR = 1,        // list of >= split_threshold particles: parallel partition
    MODE_VEC1 = 2,       // list of exactly one particle: leaf without bounds test
    MODE_SER_ENTRY = 3,  // list of 2..threshold-1: serial insertion, list kept in childParticles
    MODE_SER = 4         // below a serial node: one-by-one insertion
};

struct Particles {
    double *px, *py, *pz;
    double *vx, *vy, *vz;
    double *ax, *ay, *az;
    double *m, *U, *dUdt, *h, *rho, *P, *T, *vdens;
    double *tstep, *tnext;  // block time steps: the particle's step and its next integration time
    uint8_t *type;
    int32_t *id;
};

// A node's moments as the reference keeps them (Node.h): mass, centre of mass,
// gasMass and the gas velocity mVel.  One 64-byte record per node.
struct alignas(64) NodeMom {
    double mass, cx, cy, cz, gas, mvx, mvy, mvz;
};

// A node's FP32 walk record, in the instance's scaled units: A = centre of mass
// (hi floats) and mass * ls^2; B = centre of mass (lo floats) and the opening
// threshold (radius * ls / theta)^2 (-1 for a leaf); C = first child (-1 leaf),
// leaf particle slot (-1 none), child mask, 0; D = gas velocity (mVel, or the
// leaf particle's velocity) and gasMass * ls^2, zeros for a node without gas.
// One 64-byte record, so a staged child is two sectors of one cache line.
struct alignas(64) WalkRec {
    float4 A, B;
    int4 C;
    float4 D;
};

// Sums of a node's whole routed range: mass, mass-weighted position, gas mass
// and gas momentum, the mass of its lowest upload index, gas count and that
// index.  80 bytes of data padded to three whole 32-byte sectors and written
// whole (pad included): a record written at a scattered node index then
// leaves no sector partly written for the memory system to merge.
struct alignas(32) NodeSum {
    double m, mx, my, mz, g, gvx, gvy, gvz;
    double first_m;
    int32_t ng, first_id;
    double pad[2];
};

// The first node index after the roots (instance k's root is node k): the pool
// starts on a multiple of 8, so that every node's 8-child block is 8-aligned
// and the children's 4- and 8-byte fields fill whole 32-byte sectors.  The
// indices in between are never reached (every traversal starts at a root).
__host__ __device__ inline int64_t first_pool_node(int64_t n_inst) { return (n_inst + 7) & ~(int64_t)7; }

struct Nodes {
    // topology (written by the level-wise build)
    int32_t *start, *count, *ndrop, *first, *parent, *leafpos;
    int8_t *level;
    uint8_t *mode;
    uint8_t *needs;      // node gets a digit pass at its level (level loop's nodes only)
    double *cx, *cy, *cz;
    double *radius;      // half-width (the root's R halved per level, exactly as Node.cpp:440)
    int32_t *inst;       // simulation instance the node belongs to
    int64_t *bkey;       // 9 ordered-integer keys per level-loop node: lo xyz, hi xyz, centre xyz
    // moments (reference semantics, FP64), one record per node
    NodeMom *mom;
    // sums over the whole routed range (bottom-up helper), one record per node
    // so a node's eight children are one contiguous read
    NodeSum *tsum;
    // walk records (FP32 view)
    WalkRec *wrec;  // FP32 walk record per node (64 B, one cache-line half)
    // SPH / visual density scratch
    uint8_t *flag;
    double *rho;
    // build scratch sized by the node pool
    int32_t *nlx;    // index of a node in its level's split list
    int2 *lint;      // internal nodes with their level (padding: node -1)
    int32_t *lil;    // the same, one segment per level, deepest last
};

struct Ctx {
    ag2_params prm;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t side_stream = nullptr;  // captures the bodies of a step graph's loops
    bool capturing = false;              // a step graph is being captured on `stream`
    // step graphs (ag2_step_graphs): one per state buffer the step starts from
    bool use_graphs = false;
    cudaGraphExec_t step_exec[2] = {};
    unsigned long long step_key = 0;     // parameters the graphs were captured for
    int64_t graph_launches[2] = {};      // kernels captured outside the loops
    double *inst_R_pin = nullptr;        // pinned copy of the root half-widths (step graphs)
    double *inst_R_rb = nullptr;         // pinned read-back of the root half-widths (launched builds)
    size_t inst_R_rb_cap = 0;
    // block time steps (ag2_block_init / ag2_block_step)
    bool blk_ready = false;
    double blk_eta = 0, blk_dmin = 0, blk_dmax = 0, blk_t = 0;
    long long *blk_key = nullptr;  // device: earliest next integration time (ordered key)
    int32_t *blk_count = nullptr;  // device: due particles

    // Per-particle values that ride along unchanged, in upload order:
    // Particle::id, galaxyPart (1 disk, 2 bulge, 3 halo) and sfr
    uint32_t *tag_id = nullptr;
    uint8_t *tag_gp = nullptr;
    double *tag_sfr = nullptr;
    // snapshot / initial-condition files: the file image on the device (with
    // slack after its end), its pinned host copy, scratch (inverse permutation,
    // per-block counts) and the background writer of the last snapshot
    uint8_t *io_dev = nullptr;
    size_t io_dev_cap = 0;
    uint8_t *io_host = nullptr;
    size_t io_host_cap = 0;
    int32_t *io_scratch = nullptr;
    size_t io_scratch_cap = 0;
    int64_t *io_len_dev = nullptr;   // image length computed on the device
    int64_t *io_len_host = nullptr;  // pinned
    cudaStream_t io_stream = nullptr;
    cudaEvent_t io_event = nullptr;
    std::thread io_thread;
    int io_status = 0;
    std::string io_err;
    const uint8_t *walk_active = nullptr;  // per slot: walk it (null = every particle)
    size_t inst_R_pin_cap = 0;
    int64_t graph_epoch = 0;             // bumped when the particle set, layout or parameters change
    int device = 0;
    int sms = 152;       // multiprocessors of the device
    // k_local's launch for captured builds (set before the capture)
    int loc_lcap = 0, loc_wpb = 0, loc_blocks = 0;
    size_t loc_smem = 0;
    size_t cap = 0;      // particle capacity
    size_t n = 0;        // particles uploaded
    size_t node_cap = 0; // node pool capacity
    int64_t nnodes = 0;  // nodes in the current tree
    int64_t ninternal = 0;
    int max_level = 0;
    std::vector<int64_t> level_base;  // node index of the first node of each level
    bool have_tree = false;
    double root_radius = 0.0;
    int64_t launches = 0;
    bool debug_sync = false;  // AG2_DEBUG_SYNC=1: synchronise and check after every launch
    int64_t inter_grav = 0, inter_sph = 0;
    int32_t inject_site = 0, inject_code = 0;  // ag2_inject_fault: one host-side failure, then cleared
    std::string err;

    Particles st[2] = {};
    int cur = 0;

    // build scratch.  During the level loop a slot (position in the partition)
    // is active while its node is still split; perm/posnode/pkey hold the
    // active slots' particle, split-list index and coordinate keys (two
    // buffers, level after level), perm_final the particle a slot ends with.
    int32_t *perm = nullptr, *perm2 = nullptr, *posnode = nullptr, *posnode2 = nullptr;
    int32_t *perm_final = nullptr;
    int32_t *ap[2] = {};          // active slots of a level (compact list)
    int32_t *nl[2] = {};          // split list of a level (node ids)
    int32_t *lroots = nullptr;    // roots of serial subtrees built by one warp each
    int64_t *pkey = nullptr;      // 2 buffers x 3 coordinates x cap ordered keys
    int64_t nnodes_true = 0;      // nodes of the tree (nnodes also counts unused pool tails)
    std::vector<int32_t> lvl_cnt_h, lvl_start_h;  // internal nodes per level and their list segments
    int32_t *pnode = nullptr;     // deepest node whose range holds a tree-order slot
    int32_t *refnode = nullptr;   // the reference's Particle::node per slot (-1 = null)
    int32_t *slot_of = nullptr;   // tree-order slot of each upload index
    double2 *rdist = nullptr;     // |x| of each particle and its square (tree order) for the root half-width
    int32_t *finalnode = nullptr; // SPH / visual density result node per slot
    int32_t *nodelist = nullptr;  // compacted node list (SPH density nodes)
    int32_t *gas_slots = nullptr; // SPH density: the gas particles' tree-order slots
    int32_t *drop_list = nullptr; // nodes with out-of-bounds tails (65536 entries)
    uint8_t *digit = nullptr;
    int32_t *hist = nullptr;      // 9 per node of a level
    int32_t *cursor = nullptr;
    size_t hist_cap = 0;
    bool hist_dirty = false;      // a failed build may have left histogram entries set
    double *gas_prefix = nullptr; // sequential sums k*m_gas (uniform gas mass)
    size_t gas_prefix_cap = 0;
    void *gas_pin = nullptr;     // pinned read-back of the gas statistics (kmin, kmax, count per instance)
    size_t gas_pin_cap = 0;      // instances it holds
    bool gas_pending = false;    // statistics queued for read-back, not yet compared
    double *staging = nullptr;    // 6n doubles for upload/download
    uint8_t *staging_u8 = nullptr;
    double *width_part = nullptr; // partial sums of the root width (pairs), laid out by the task table
    int4 *wsum_task = nullptr;    // root-width summation tasks, level after level
    int32_t *wsum_final = nullptr; // per instance: position of its final pair
    std::vector<int32_t> wsum_level;  // task offsets of each level
    int32_t *wsum_long = nullptr;     // level-0 tasks of more than kWsumRun terms
    int32_t nwsum_long = 0;
    double *width_thr = nullptr;  // mean + 10 sigma per instance
    double gas_table_mass = -1.0; // gas particle mass the gasMass table was built for
    int32_t gas_table_n = -1;
    bool gas_uniform = false;
    bool gas_stats_dirty = true;  // masses or types changed since the last statistics
    // what the gasMass tables in gas_prefix were built for (gas count and mass key
    // per instance): a table is a sequential sum, rebuilt only when these change
    std::vector<int32_t> gas_tab_cnt;
    std::vector<long long> gas_tab_lo, gas_tab_hi;
    int32_t ngas = 0;
    double gas_mass_min = 0.0, gas_mass_max = 0.0;
    double tree_theta = 0.0;      // opening angle baked into the walk records
    int walk_variant = 1;         // FP32 walk register-budget variant (ag2_autotune)

    // Independent simulations ("instances") sharing this context: instance k
    // owns upload indices [inst_first[k], inst_first[k+1]); in tree order it
    // owns the same slot range (every build only permutes inside each root's
    // range), its tree's root is node k, and its walk groups never mix with
    // another instance's.
    int32_t n_inst = 1;
    std::vector<int64_t> inst_first_h{0, 0};
    std::vector<double> inst_massInH_h{0.0};
    size_t inst_cap = 0;
    int64_t *inst_first = nullptr;  // device, n_inst + 1
    double *inst_R = nullptr;       // device, root half-width per instance
    double *inst_massInH = nullptr; // device
    int32_t *pinst = nullptr;       // device, instance of each slot
    int4 *groups = nullptr;         // device walk groups: (first slot, lanes, instance, 0)
    int32_t *retry_groups = nullptr; // device, groups_cap: groups for the FP32 walk's retry pass
    int32_t ngroups = 0;
    int32_t groups_gs = 0;           // group size the table was built for
    size_t groups_cap = 0;
    bool inst_dirty = true;         // instance tables need uploading
    bool inst_explicit = false;     // layout from ag2_set_instances (keeps its massInH)
    std::vector<int64_t> inst_tab_first;  // layout the device instance tables and walk groups describe
    // Slot order of the state: upload order (slot i holds upload index i), or
    // the permutation of the last build, which keeps every instance of layout
    // perm_first inside its own slot range
    bool upload_order = true;
    std::vector<int64_t> perm_first;
    // ag2_download_fields: device-to-host copies on their own stream, behind
    // the gathers of the context's stream (two staging halves)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t dl_gathered[2] = {}, dl_copied[2] = {};
    // ag2_step_host's accelerations: their own staging (3 doubles per particle
    // of capacity, made on first use) and the events that order their copy
    double *acc_stage = nullptr;
    cudaEvent_t up_ev[2] = {};
    // gasMass tables: instance k's sequential partial sums start at gas_off[k]
    int32_t *gas_off = nullptr;     // device
    uint8_t *gas_uni = nullptr;     // device: instance's gas particles share one mass
    int32_t *gas_cnt = nullptr;     // device scratch: gas count per instance
    long long *gas_kmin = nullptr, *gas_kmax = nullptr;  // device scratch
    std::vector<double> inst_R_h;   // host copy after a build

    // small device control block
    struct Ctl {
        double sum_d, sum_d2, thr, R;
        int64_t node_count;
        int32_t err_code;
        int32_t err_info;
        int32_t next_needs;     // nodes needing a digit pass at the next level
        int32_t any_drop;
        int32_t gas_uniform;
        int32_t ngas_total;
        long long gas_key_min, gas_key_max;
        unsigned long long inter_grav, inter_sph;
        int32_t list_count;
        int32_t retry_count;    // FP32 walk: groups sent to the retry pass
        int32_t retry_claim;    // ... and claimed by it
        int32_t ndrop_nodes;
        int32_t next_active;    // active slots at the next level
        int32_t nlocal;         // serial subtree roots for k_local
        int32_t nlint;          // entries of the internal-node list
        int32_t level;          // level loop: the level being split
        int32_t cur_nnl;        // ... its split list
        int32_t cur_nap;        // ... its active slots
        int32_t mlev;           // moments: the level being finished (-1 when done)
        int64_t loop_nodes;     // node count at the end of the level loop
        int32_t lvl_start[AG2_MAX_DEPTH];  // internal-node list segments per level
        int32_t lvl_cnt[AG2_MAX_DEPTH];  // internal nodes per level
        int32_t lvl_off[AG2_MAX_DEPTH];  // bucketing cursors
        int32_t maxlev;         // deepest level of the serial subtrees
        int32_t nlocal_part;    // particles in serial subtrees
        int32_t mlev_last;      // moments: the shallowest level the last launch finished
        int32_t ngas_slots;     // SPH density: gas slots listed by k_climb
        uint32_t scatter_done;  // blocks of the running k_scatter that have finished (launched level loop)
        unsigned long long local_splits;  // split nodes of the serial subtrees
    };
    Ctl *ctl = nullptr;      // device
    Ctl *ctl_host = nullptr; // pinned mirror
    // the launched level loop's control-block snapshots (pinned, two levels in
    // flight) and the events that mark them copied
    Ctl *ctl_snap = nullptr;
    cudaEvent_t snap_ev[2] = {};

    Nodes nd = {};

    // phase timers (CUDA events), enabled by ag2_phase_timing
    static constexpr int kMaxPhases = 16;
    bool timing = false;
    cudaEvent_t ev[kMaxPhases + 1] = {};
    const char *phase_name[kMaxPhases] = {};
    int nphase = 0;          // phases recorded since the last reset
    float phase_ms[kMaxPhases] = {};
    int phase_count = 0;     // phases of the last completed measurement

    Particles &S() { return st[cur]; }
};

// Phase timing helpers: reset at the start of a measured call, mark after each
// phase, finish (synchronises) at the end.
void phase_reset(Ctx *c);
void phase_mark(Ctx *c, const char *name);
void phase_finish(Ctx *c);

// ordered 64-bit integer key of a double: a < b (as doubles, -0 == +0 mapped
// to +0) iff key(a) < key(b)
__host__ __device__ inline int64_t okey(double x)
{
    long long b;
#ifdef __CUDA_ARCH__
    b = __double_as_longlong(x);
#else
    __builtin_memcpy(&b, &x, 8);
#endif
    // -0.0 -> +0.0 on the bit pattern (x + 0.0 would spend an FP64 add, which
    // this part issues at 1/64 of the FP32 rate)
    if (b == (long long)0x8000000000000000ULL) b = 0;
    return b >= 0 ? (int64_t)b : (int64_t)(b ^ 0x7FFFFFFFFFFFFFFFLL);
}

// Power-of-two length scale of an instance's FP32 walk: 2^-e for the root
// half-width R = f * 2^e, f in [0.5, 1) (1 when R is 0 or not finite).  The
// walk records and the walk's offsets are in units of 2^e: scaling by a power
// of two is exact, and it keeps r^2, (radius/theta)^2 and h^4 inside FP32's
// range in any unit system (the reference works in SI, positions ~1e20 m).
__host__ __device__ inline int64_t dbits(double x)
{
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    int64_t b;
    __builtin_memcpy(&b, &x, 8);
    return b;
#endif
}
__host__ __device__ inline double bits_d(int64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    __builtin_memcpy(&x, &b, 8);
    return x;
#endif
}
// the exponent k of the scale 2^k (integer operations only: this part issues
// FP64 at 1/64 of the FP32 rate)
__host__ __device__ inline int walk_scale_exp(double R)
{
    const int64_t b = dbits(R);
    const int ef = (int)((b >> 52) & 0x7ff);
    if (b <= 0 || ef == 0 || ef == 0x7ff) return 0;  // R <= 0, subnormal, inf or NaN: scale 1
    return 1022 - ef;  // R = f 2^e, f in [0.5, 1), e = ef - 1022
}
__host__ __device__ inline double walk_scale(double R) { return bits_d((int64_t)(1023 + walk_scale_exp(R)) << 52); }
// x * 2^k exactly; on the exponent bits when x and the result are normal
__host__ __device__ inline double scale2(double x, int k)
{
    const int64_t b = dbits(x);
    const int ef = (int)((b >> 52) & 0x7ff);
    if (ef > 0 && ef < 0x7ff && ef + k > 0 && ef + k < 0x7ff) return bits_d(b + ((int64_t)k << 52));
    return x * ldexp(1.0, k);  // zero, subnormal, inf, NaN, or a result outside the normal range
}


// the root half-width's sums are sequential (the reference's, bit for bit) up to
// this many particles per instance, a 64-ary tree of sequential runs above
constexpr int kSeqWidthMax = 4096;
// root-width tasks of more terms than this (the one sequential sum of an
// instance of 65..4096 particles) run on warps of their own (k_wsum_long)
constexpr int kWsumRun = 64;

// status helpers
int set_err(Ctx *c, int code, const std::string &msg);
int cuda_check(Ctx *c, cudaError_t e, const char *what);
#define AG2_CUDA(c, call)                                   \
    do {                                                    \
        cudaError_t _e = (call);                            \
        if (_e != cudaSuccess) return cuda_check(c, _e, #call); \
    } while (0)

inline unsigned grid_for(size_t n, int block) { return (unsigned)((n + block - 1) / block); }
inline bool launch_ok(unsigned long long g) { return g > 0; }
inline bool launch_ok(const dim3 &g) { return g.x > 0 && g.y > 0 && g.z > 0; }

// launch accounting: every kernel launch goes through this
#define AG2_LAUNCH(c, kern, grid, block, smem, ...)                          \
    do {                                                                     \
        if (launch_ok(grid)) {                                               \
            kern<<<(grid), (block), (smem), (c)->stream>>>(__VA_ARGS__);     \
            (c)->launches++;                                                 \
            cudaError_t _le = cudaGetLastError();                            \
            if (_le == cudaSuccess && (c)->debug_sync && !(c)->capturing)    \
                _le = cudaStreamSynchronize((c)->stream);                    \
            if (_le != cudaSuccess) return cuda_check(c, _le, #kern);        \
        }                                                                    \
    } while (0)

// entry points implemented per translation unit
int build_tree(Ctx *c);
int ensure_instance_tables(Ctx *c);
int build_groups(Ctx *c);
int group_size_of(const ag2_params &p);
int build_tree_captured(Ctx *c);
int moments_launches(const int32_t *lvl_cnt);  // launches of a captured build's internal-moments loop
void build_tree_finish_captured(Ctx *c);
int prepare_captured_build(Ctx *c);
int ensure_node_capacity(Ctx *c, size_t need);
int run_forces(Ctx *c);
int run_sph_density(Ctx *c);
int run_visual_density(Ctx *c, double R);
int run_kick(Ctx *c, double dt);
int run_drift(Ctx *c, double dt);
int run_kick_drift(Ctx *c, double dt);
int run_ueuler(Ctx *c, double dt);
int run_scale(Ctx *c, double f);
int sync_ctl(Ctx *c);  // copy ctl to host (synchronises the stream)
int run_direct_sum(Ctx *c, size_t ns, const int64_t *ids_host, double *out_host);
int run_diagnostics(Ctx *c, double *out8);
int run_energy(Ctx *c, double *out4);
int run_block_init(Ctx *c, double eta, double dmin, double dmax, double t);
int run_block_step(Ctx *c, double H0, int with_visual, double Rv, double *t_out, int64_t *active_out);
int run_fma_probe(Ctx *c, double *gflops);
int io_reset_tags(Ctx *c, size_t n);
void io_release(Ctx *c);
constexpr int kWalkVariantCount = 6;  // FP32 walk variants (ag2_walk.cu kVariants)
int run_autotune(Ctx *c, int *chosen, ag2_walk_config *out = nullptr, int max_out = 0, int *count = nullptr);

// physical constants of the reference (Constants.h:14-15, Particle.h:40)
constexpr double kGamma = 5.0 / 3.0;
constexpr double kBoltzmann = 1.38064852e-23;
constexpr double kProton = 1.6726219e-27;
constexpr double kPi = 3.14159265358979323846;

}  // namespace ag2

// the opaque handle of the C interface
struct ag2_ctx : public ag2::Ctx {};

