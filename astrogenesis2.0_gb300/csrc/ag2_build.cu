// ag2_build.cu -- device octree build with the reference's subdivision rule.
//
// Reference: simulation/src/Physics/Tree/Tree.cpp:24-55 (buildTree), :86-117
// (calcTreeWidth); simulation/src/Physics/Tree/Node.cpp:405-534 (vector
// insertion), :597-699 (serial insertion), :702-719 (getOctant).
//
// The reference decides octants by FP64 comparisons against node centres that
// are accumulated as c + r*(+-0.5) from the root, with inclusive bounds tests
// at every node.  The tree is built as a most-significant-digit radix sort of
// the particles by those decisions, one tree level per pass: each node that is
// split at level L gets one pass in which every particle of its range computes
// its 4-bit digit (octant 0..7, or 8 = outside this node's bounds) against the
// node's precomputed bounds, and the range is partitioned by digit.  The digit
// sequence of a particle is its Morton key under the reference's own rounding.
// Node centres are computed once per node in FP64 exactly as the reference
// does; particles only compare (as order-preserving 64-bit integers), so the
// topology is bit-exact.
//
// Node modes reproduce Node::insert's switch at threads*100 particles: lists of
// at least split_threshold particles take the parallel path (always split,
// mass over the whole list), single-particle lists become leaves, and shorter
// lists are inserted one by one (split when two particles land in-bounds).
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>

#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kBlock = 256;
constexpr int kMaxDropNodes = 1 << 16;  // nodes with out-of-bounds tails tracked for the ordering pass

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// warp-aggregated atomicAdd(&arr[slot], 1); returns the value before this
// lane's increment
__device__ __forceinline__ int agg_inc(int32_t *arr, int slot)
{
    unsigned act = __activemask();
    unsigned peers = __match_any_sync(act, slot);
    int leader = __ffs(peers) - 1;
    int lane = lane_id();
    int rank = __popc(peers & ((1u << lane) - 1u));
    int v = 0;
    if (lane == leader) v = atomicAdd(&arr[slot], __popc(peers));
    v = __shfl_sync(peers, v, leader);
    return v + rank;
}

// Reduce v over the lanes of `peers` (this lane's group from __match_any_sync,
// any bit pattern); every lane of the group gets the result.  The lanes of one
// group run the loop together (same mask, same trip count), 32 shuffles per
// warp in total whatever the grouping.
template <class T, class Op>
__device__ __forceinline__ T group_reduce(unsigned peers, T v, Op op)
{
    unsigned rest = peers;
    T r = __shfl_sync(peers, v, __ffs(rest) - 1);
    rest &= rest - 1u;
    while (rest) {
        const int l = __ffs(rest) - 1;
        rest &= rest - 1u;
        r = op(r, __shfl_sync(peers, v, l));
    }
    return r;
}

__device__ __forceinline__ double dist0(double x, double y, double z)
{
    // vec3::length(): sqrt(x*x + y*y + z*z), evaluated left to right, no FMA
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
}

// ---- Tree::calcTreeWidth, per instance -------------------------------------
//
// Sums of |x| and |x|^2 in the caller's particle order (Tree.cpp:99-103).  Up to
// kSeqWidthMax particles they are the reference's sequential sums, bit for bit.
// Above that the sums follow a fixed 64-ary tree over the instance's particles:
// runs of 64 consecutive values are added sequentially, then runs of 64 of
// those sums, and so on.  The rule depends only on the instance's own particles,
// so an instance gets the same half-width alone or sharing the context.

// slot of each particle in the caller's (upload) order: the state is kept in
// tree order, but the reference sums distances in its particle array order
__global__ void k_slot_of(int n, const int32_t *__restrict__ id, int32_t *__restrict__ slot_of)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) slot_of[id[i]] = i;
}

// |x| of every particle once, in tree order, with its square: (d, d*d) pairs.
// Both are the products the reference's sums take (Tree.cpp:99-103); the
// sequential sums below then chain only their additions.  On this part one
// FP64 instruction holds a warp's FP64 pipe for about 64 cycles whatever its
// active lanes, so a 4096-term sequential sum is bound by its FP64
// instructions, and taking the squares out of it removes a third of them.
__global__ void k_dist(int n, const double *__restrict__ px, const double *__restrict__ py,
                       const double *__restrict__ pz, double2 *__restrict__ dist)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double d = dist0(px[i], py[i], pz[i]);
        dist[i] = make_double2(d, __dmul_rn(d, d));
    }
}

// first level: task (first caller index, count, destination) over particles
__global__ void k_wsum_particles(int ntask, const int4 *__restrict__ task, const double2 *__restrict__ dist,
                                 const int32_t *slot_of, double *buf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntask) return;
    const int4 q = task[t];
    if (q.y > kWsumRun) return;  // a long sequential sum: k_wsum_long
    double s = 0.0, s2 = 0.0;
    for (int j = 0; j < q.y; j++) {
        const double2 d = dist[slot_of[q.x + j]];
        s = __dadd_rn(s, d.x);
        s2 = __dadd_rn(s2, d.y);
    }
    buf[2 * (int64_t)q.z] = s;
    buf[2 * (int64_t)q.z + 1] = s2;
}

// The long first-level tasks: one sequential sum per instance of 65..4096
// particles (Tree.cpp:99-103), up to 4096 dependent FP64 additions.  Two warps
// per task, one per chain (sum of |x|, sum of |x|^2), so that each chain has
// an SM partition's FP64 pipe to itself; the lanes load 32 terms at a time in
// parallel and every lane adds them in order, taking them by shuffle (the
// same sums on every lane, bit for bit those of one thread).
__global__ void k_wsum_long(int nlong, const int32_t *__restrict__ longt, const int4 *__restrict__ task,
                            const double2 *__restrict__ dist, const int32_t *__restrict__ slot_of, double *buf)
{
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= 2 * nlong) return;
    const int chain = w & 1;
    const int4 q = task[longt[w >> 1]];
    double s = 0.0;
    for (int j0 = 0; j0 < q.y; j0 += 32) {
        const int j = j0 + lane;
        double v = 0.0;
        if (j < q.y) {
            const double2 d = dist[slot_of[q.x + j]];
            v = chain ? d.y : d.x;
        }
        if (q.y - j0 >= 32) {
            // a full block: every shuffle can issue ahead of the chain of additions
#pragma unroll
            for (int u = 0; u < 32; u++) s = __dadd_rn(s, __shfl_sync(0xffffffffu, v, u));
        } else {
            for (int u = 0; u < q.y - j0; u++) s = __dadd_rn(s, __shfl_sync(0xffffffffu, v, u));
        }
    }
    if (lane == 0) buf[2 * (int64_t)q.z + chain] = s;
}

// higher levels: task (first source sum, count, destination)
__global__ void k_wsum_sums(int ntask, const int4 *__restrict__ task, double *buf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntask) return;
    const int4 q = task[t];
    double s = 0.0, s2 = 0.0;
    for (int j = 0; j < q.y; j++) {
        s = __dadd_rn(s, buf[2 * ((int64_t)q.x + j)]);
        s2 = __dadd_rn(s2, buf[2 * ((int64_t)q.x + j) + 1]);
    }
    buf[2 * (int64_t)q.z] = s;
    buf[2 * (int64_t)q.z + 1] = s2;
}

// one thread per instance: threshold mean + 10 sigma from the instance's sums
__global__ void k_width_thr(int n_inst, const int64_t *first, const int32_t *final_pos, const double *buf,
                            double *thr, double *R)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_inst) return;
    const int64_t n = first[k + 1] - first[k];
    R[k] = 0.0;
    if (n == 0) {
        thr[k] = 0.0;
        return;
    }
    const double s = buf[2 * (int64_t)final_pos[k]], s2 = buf[2 * (int64_t)final_pos[k] + 1];
    const double mean = s / (double)n;
    const double sd = sqrt(__dsub_rn(s2 / (double)n, __dmul_rn(mean, mean)));
    thr[k] = __dadd_rn(mean, __dmul_rn(10.0, sd));  // mean + acceptanceRatio*stdev (Tree.cpp:89,105)
}

// R = max |x| over |x| <= thr (Tree.cpp:107-116); a NaN threshold keeps R = 0
__global__ void k_width_max(int n, const double2 *__restrict__ dist, const int32_t *pinst, const double *thr,
                            double *R)
{
    __shared__ int32_t kmin, kmax;
    __shared__ unsigned long long bbest;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = i < n ? pinst[i] : -1;
    unsigned long long best = 0ull;
    if (i < n) {
        const double d = dist[i].x;
        if (d <= thr[k] && d > 0.0) best = (unsigned long long)__double_as_longlong(d);
    }
    if (threadIdx.x == 0) {
        kmin = INT32_MAX;
        kmax = -1;
        bbest = 0ull;
    }
    __syncthreads();
    if (k >= 0) {
        atomicMin_block(&kmin, k);
        atomicMax_block(&kmax, k);
    }
    __syncthreads();
    if (kmin == kmax) {  // one instance in the block (the usual case): one global atomic per block
        if (best) atomicMax_block(&bbest, best);
        __syncthreads();
        if (threadIdx.x == 0 && bbest) atomicMax((unsigned long long *)&R[kmin], bbest);
        return;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    best = group_reduce(peers, best, [](unsigned long long a, unsigned long long b) { return a > b ? a : b; });
    if (k >= 0 && best != 0ull && (threadIdx.x & 31) == __ffs(peers) - 1)
        atomicMax((unsigned long long *)&R[k], best);
}

// ---- level-wise partition --------------------------------------------------

__device__ __forceinline__ void set_bounds_v(Nodes nd, int64_t c, double cx, double cy, double cz, double r)
{
    int64_t *k = nd.bkey + 9 * c;
    k[0] = okey(__dsub_rn(cx, r));
    k[1] = okey(__dsub_rn(cy, r));
    k[2] = okey(__dsub_rn(cz, r));
    k[3] = okey(__dadd_rn(cx, r));
    k[4] = okey(__dadd_rn(cy, r));
    k[5] = okey(__dadd_rn(cz, r));
    k[6] = okey(cx);
    k[7] = okey(cy);
    k[8] = okey(cz);
}
__device__ __forceinline__ void set_bounds(Nodes nd, int64_t c, double r)
{
    set_bounds_v(nd, c, nd.cx[c], nd.cy[c], nd.cz[c], r);
}
// The same nine keys of node v, formed from its centre and half-width where
// they are used: the serial subtrees (k_local) keep none in memory.
__device__ __forceinline__ void local_keys(const Nodes &nd, int64_t v, int64_t *k)
{
    const double x = nd.cx[v], y = nd.cy[v], z = nd.cz[v], r = nd.radius[v];
    k[0] = okey(__dsub_rn(x, r));
    k[1] = okey(__dsub_rn(y, r));
    k[2] = okey(__dsub_rn(z, r));
    k[3] = okey(__dadd_rn(x, r));
    k[4] = okey(__dadd_rn(y, r));
    k[5] = okey(__dadd_rn(z, r));
    k[6] = okey(x);
    k[7] = okey(y);
    k[8] = okey(z);
}

// root of instance k is node k (Tree.cpp:28-33: centre at the origin, half-width
// from calcTreeWidth, depth 0)
__global__ void k_root_init(int n_inst, Nodes nd, Ctx::Ctl *ctl, const int64_t *first, const double *R, int thresh,
                            int32_t *nl0, bool local_ok, int32_t *lroots)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_inst) return;
    // the pool starts after the roots (the rest of the control block is zero
    // from the memset at the start of the build)
    if (k == 0) ctl->node_count = first_pool_node(n_inst);
    const int32_t start = (int32_t)first[k];
    const int32_t n = (int32_t)(first[k + 1] - first[k]);
    nd.start[k] = start;
    nd.count[k] = n;
    nd.ndrop[k] = 0;
    nd.first[k] = -1;
    nd.parent[k] = -1;
    nd.level[k] = 0;
    nd.cx[k] = 0.0;
    nd.cy[k] = 0.0;
    nd.cz[k] = 0.0;
    nd.radius[k] = R[k];
    nd.inst[k] = k;
    const uint8_t mode = n == 0 ? MODE_EMPTY : n == 1 ? MODE_VEC1 : n < thresh ? MODE_SER_ENTRY : MODE_PAR;
    nd.mode[k] = mode;
    // 1: split by the level loop; 2: a serial subtree built by one warp (k_local)
    const uint8_t needs = mode == MODE_PAR ? 1 : mode == MODE_SER_ENTRY ? (local_ok ? 2 : 1) : 0;
    nd.needs[k] = needs;
    nd.leafpos[k] = (mode == MODE_VEC1) ? start : -1;
    if (needs == 2) atomicAdd(&ctl->nlocal_part, n);
    if (needs) set_bounds(nd, k, R[k]);
    if (needs == 1) {
        const int q = atomicAdd(&ctl->next_needs, 1);
        nl0[q] = k;
        nd.nlx[k] = q;
    } else if (needs == 2) {
        lroots[atomicAdd(&ctl->nlocal, 1)] = k;
    }
}

// Block-wide reservation in a compact list: every thread of the block calls
// this (no early return before it).  A flagged thread gets the position of its
// `stride` entries in the list whose length is *counter; one atomicAdd per block.
template <class T>
__device__ __forceinline__ T block_reserve(bool flag, T *counter, T stride, int32_t *sh, T *sbase)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned b = __ballot_sync(0xffffffffu, flag);
    if (lane == 0) sh[w] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < nw; k++) {
            const int v = sh[k];
            sh[k] = acc;
            acc += v;
        }
        *sbase = acc ? atomicAdd(counter, (T)acc * stride) : (T)0;
    }
    __syncthreads();
    const T r = flag ? *sbase + (T)(sh[w] + __popc(b & ((1u << lane) - 1u))) * stride : (T)0;
    __syncthreads();
    return r;
}

// block_reserve for a loop that calls it once per round: the two rounds in
// flight use the two halves of sh (kBlock / 32 entries each) and of sbase
// alternately, so a round needs no barrier after reading its offsets.  A
// thread writes a half again two rounds later, after the next round's first
// barrier, which every thread reaches only after reading its offsets here.
__device__ __forceinline__ int32_t block_reserve_rounds(bool flag, int32_t *counter, int32_t *sh, int32_t *sbase,
                                                        int round)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int32_t *const shr = sh + (round & 1) * nw;
    int32_t *const sb = sbase + (round & 1);
    const unsigned b = __ballot_sync(0xffffffffu, flag);
    if (lane == 0) shr[w] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < nw; k++) {
            const int v = shr[k];
            shr[k] = acc;
            acc += v;
        }
        *sb = acc ? atomicAdd(counter, acc) : 0;
    }
    __syncthreads();
    return flag ? *sb + shr[w] + __popc(b & ((1u << lane) - 1u)) : 0;
}

// Buffers of one level of the partition.  A slot is a position in the
// partition; it is active while the node whose range holds it is still split.
struct LevelBufs {
    const int32_t *ap;       // active slots of this level
    int32_t *ap_next;        // ... of the next level
    const int32_t *posnode;  // per active slot: index of its node in this level's split list
    int32_t *posnode_next;
    const int32_t *perm;     // per active slot: index of the particle there in the state arrays
    int32_t *perm_next;
    const int64_t *kx, *ky, *kz;  // per active slot: ordered keys of the particle's coordinates
    int64_t *kx_next, *ky_next, *kz_next;
    int32_t *perm_final;     // per slot, written when the particle there settles
    int32_t *pnode;          // per slot: node the settled particle ends in
    const uint8_t *digit;    // per slot: octant digit of the particle there in its node of this level
    uint8_t *digit_next;     // ... of the next level (written as particles move there)
    int32_t *hist, *cursor;  // 9 per split-list entry
    const int32_t *nl;       // this level's split list (node ids)
    int32_t *nl_next;
    int32_t *drop_list;      // nodes with out-of-bounds tails of two or more
    int32_t *lroots;         // roots of serial subtrees for k_local
    bool local_ok;           // serial subtrees go to k_local (else they stay in the level loop)
};

// The buffers of both level parities: a level reads b[level & 1], the level it
// runs at coming from the control block, so the same launches serve every level.
struct LevelPair {
    LevelBufs b[2];
};

// Octant digit of ordered keys against a node's 9 bound keys: 0..7, or 8 when
// outside the node's inclusive bounds (Node.cpp:606-608, 706-716).  The level
// loop computes a particle's digit for the next level where it moves the
// particle into its child (k_scatter), and level 0's in k_level0.
__device__ __forceinline__ int octant_digit(const int64_t *k, int64_t kx, int64_t ky, int64_t kz)
{
    if (kx < k[0] || kx > k[3] || ky < k[1] || ky > k[4] || kz < k[2] || kz > k[5]) return 8;
    return (kx > k[6] ? 1 : 0) | (ky > k[7] ? 2 : 0) | (kz > k[8] ? 4 : 0);
}

// Level 0: the slots of an instance whose root is split are active (the
// coordinates become ordered keys, in slot order); the slot of a one-particle
// root is final at once.
__global__ void __launch_bounds__(kBlock) k_level0(int n, const int32_t *__restrict__ pinst, Nodes nd,
                                                   const double *__restrict__ px, const double *__restrict__ py,
                                                   const double *__restrict__ pz, LevelBufs b, Ctx::Ctl *ctl)
{
    __shared__ int32_t sh[kBlock / 32 + 1];
    __shared__ int32_t sbase;
    __shared__ int32_t jmin, jmax, bh[9];
    if (threadIdx.x == 0) {
        jmin = INT32_MAX;
        jmax = -1;
    }
    if (threadIdx.x < 9) bh[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int hj = -1, hd = 0;  // this particle's histogram entry
    bool act = false;
    int32_t *perm = const_cast<int32_t *>(b.perm);
    int32_t *posnode = const_cast<int32_t *>(b.posnode);
    if (i < n) {
        const int k = pinst[i];
        const uint8_t nk = nd.needs[k];
        if (nk == 1) {
            act = true;
            perm[i] = i;
            const int j = nd.nlx[k];
            posnode[i] = j;
            const int64_t kx = okey(px[i]), ky = okey(py[i]), kz = okey(pz[i]);
            const_cast<int64_t *>(b.kx)[i] = kx;
            const_cast<int64_t *>(b.ky)[i] = ky;
            const_cast<int64_t *>(b.kz)[i] = kz;
            const int d = octant_digit(nd.bkey + 9 * (int64_t)k, kx, ky, kz);
            const_cast<uint8_t *>(b.digit)[i] = (uint8_t)d;
            hj = j;
            hd = d;
            atomicMin_block(&jmin, j);
            atomicMax_block(&jmax, j);
        } else {
            b.perm_final[i] = i;
            b.pnode[i] = k;  // one-particle root, or a serial root for k_local
            if (nk == 2) {
                const_cast<int64_t *>(b.kx)[i] = okey(px[i]);
                const_cast<int64_t *>(b.ky)[i] = okey(py[i]);
                const_cast<int64_t *>(b.kz)[i] = okey(pz[i]);
            }
        }
    }
    __syncthreads();
    if (jmin == jmax) {  // one root in the block (the usual case): block counts, one atomic per digit
        if (hj >= 0) atomicAdd_block(&bh[hd], 1);
        __syncthreads();
        if (threadIdx.x < 9 && bh[threadIdx.x]) atomicAdd(&b.hist[9 * jmin + threadIdx.x], bh[threadIdx.x]);
    } else if (hj >= 0) {
        agg_inc(b.hist, 9 * hj + hd);
    }
    const int32_t q = block_reserve<int32_t>(act, &ctl->next_active, 1, sh, &sbase);
    if (act) const_cast<int32_t *>(b.ap)[q] = i;
}

// Split decisions and children of the nodes of this level's split list.  Eight
// threads per node (one per child octant) so that the children's fields are
// written with coalesced stores; the first thread of each group of eight
// decides the split and writes the parent.  Child blocks, the next split list,
// the leaf list and the internal-node list are reserved once per thread block.
__global__ void __launch_bounds__(kBlock) k_nodes(LevelPair lpair, int thresh, int64_t node_cap, Nodes nd,
                                                  Ctx::Ctl *ctl, int max_depth)
{
    __shared__ int32_t sh[kBlock / 32 + 1];
    __shared__ unsigned long long sbase64;
    __shared__ int32_t sbase;
    const int nnl = ctl->cur_nnl, level = ctl->level;
    const LevelBufs &b = lpair.b[level & 1];
    // block-uniform trip count: the block-wide reservations need every thread
    for (int64_t t0 = blockIdx.x * (int64_t)blockDim.x; t0 < 8 * (int64_t)nnl; t0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = t0 + threadIdx.x;
    const int lane = lane_id();
    const int o = lane & 7;
    const int64_t j = t >> 3;
    const bool exists = j < nnl;
    const int64_t nid = exists ? b.nl[j] : 0;
    int32_t cnt = 0, start = 0, ndrop = 0, reached = 0;
    uint8_t mode = 0;
    bool internal = false;
    const int32_t *h = b.hist + 9 * (exists ? j : 0);
    if (exists) {
        cnt = nd.count[nid];
        start = nd.start[nid];
        ndrop = h[8];
        reached = cnt - ndrop;
        mode = nd.mode[nid];
        internal = (mode == MODE_PAR) || (reached >= 2);
    }
    if (exists && o == 0) {
        nd.ndrop[nid] = ndrop;
        if (ndrop) ctl->any_drop = 1;
        if (ndrop >= 2) {  // tails to put in upload order after the partition
            int k = atomicAdd(&ctl->ndrop_nodes, 1);
            if (k < kMaxDropNodes) b.drop_list[k] = (int32_t)nid;
        }
        int32_t acc = start;
        for (int d = 0; d < 9; d++) {
            b.cursor[9 * j + d] = acc;
            acc += h[d];
        }
        if (!internal) {
            nd.first[nid] = -1;
            nd.leafpos[nid] = (reached == 1) ? start : -1;
        }
    }
    bool split = exists && internal;
    if (split && level + 1 >= max_depth) {
        if (o == 0) {
            atomicExch(&ctl->err_code, (int)AG2_E_COINCIDENT);
            atomicExch(&ctl->err_info, (int)nid);
            nd.first[nid] = -1;
            nd.leafpos[nid] = -1;
        }
        split = false;
    }
    const unsigned long long cb0 =
        block_reserve<unsigned long long>(split && o == 0, (unsigned long long *)&ctl->node_count, 8ull, sh, &sbase64);
    const unsigned long long cb = __shfl_sync(0xffffffffu, cb0, lane & ~7);
    if (split && (int64_t)cb + 8 > node_cap) {
        if (o == 0) {
            atomicExch(&ctl->err_code, (int)AG2_E_NOMEM);
            nd.first[nid] = -1;
        }
        split = false;
    }
    int64_t c = 0;
    uint8_t cm = MODE_EMPTY;
    if (split) {
        const int64_t c0 = (int64_t)cb;
        if (o == 0) {
            nd.first[nid] = (int32_t)c0;
            nd.leafpos[nid] = -1;
        }
        // child o: centre c + r*(+-0.5), radius r/2 (Node.cpp:433-443, 630-642)
        const double r = nd.radius[nid];
        const double rc = r / 2;  // Node.cpp:440; also r*0.5 of the centre offset, exactly
        c = c0 + o;
        int32_t s = start;
        for (int d = 0; d < o; d++) s += h[d];
        const int32_t cc = h[o];
        nd.start[c] = s;
        nd.count[c] = cc;
        nd.ndrop[c] = 0;
        nd.first[c] = -1;
        nd.parent[c] = (int32_t)nid;
        nd.level[c] = (int8_t)(level + 1);
        nd.radius[c] = rc;
        nd.inst[c] = nd.inst[nid];
        if (cc == 0)
            cm = MODE_EMPTY;
        else if (mode != MODE_PAR)
            cm = MODE_SER;
        else if (cc == 1)
            cm = MODE_VEC1;
        else if (cc < thresh)
            cm = MODE_SER_ENTRY;
        else
            cm = MODE_PAR;
        nd.mode[c] = cm;
        const bool clocal = b.local_ok && cm == MODE_SER_ENTRY;
        const bool cneeds = (cm == MODE_PAR || cm == MODE_SER_ENTRY || cm == MODE_SER) && !clocal;
        nd.needs[c] = cneeds ? 1 : clocal ? 2 : 0;
        nd.leafpos[c] = (cm == MODE_VEC1) ? s : -1;
        if (cc > 0) {  // empty children's centres are never read on the device
            const double x = __dadd_rn(nd.cx[nid], (o & 1) ? rc : -rc);
            const double y = __dadd_rn(nd.cy[nid], (o & 2) ? rc : -rc);
            const double z = __dadd_rn(nd.cz[nid], (o & 4) ? rc : -rc);
            nd.cx[c] = x;
            nd.cy[c] = y;
            nd.cz[c] = z;
            // a serial root's keys are formed by k_local from this centre and half-width
            if (cm != MODE_VEC1 && !clocal) set_bounds_v(nd, c, x, y, z, rc);
        }
    }
    const bool clocal = split && b.local_ok && cm == MODE_SER_ENTRY;
    const int32_t qr = block_reserve<int32_t>(clocal, &ctl->nlocal, 1, sh, &sbase);
    if (clocal) b.lroots[qr] = (int32_t)c;
    {
        const unsigned lp = __reduce_add_sync(0xffffffffu, clocal ? (unsigned)h[o] : 0u);
        if (lane == 0 && lp) atomicAdd(&ctl->nlocal_part, (int)lp);
    }
    const bool cneeds = split && !clocal && (cm == MODE_PAR || cm == MODE_SER_ENTRY || cm == MODE_SER);
    const int32_t q = block_reserve<int32_t>(cneeds, &ctl->next_needs, 1, sh, &sbase);
    if (cneeds) {
        b.nl_next[q] = (int32_t)c;
        nd.nlx[c] = q;
    }
    // internal nodes with their level
    const bool iflag = split && o == 0;
    const int32_t qi = block_reserve<int32_t>(iflag, &ctl->nlint, 1, sh, &sbase);
    if (iflag) nd.lint[qi] = make_int2((int)nid, level);
    // the histogram entries of this node are consumed: leave them zero for the next level
    __syncwarp();
    if (exists) {
        int32_t *hw = b.hist + 9 * j;
        hw[o] = 0;
        if (o == 0) hw[8] = 0;
    }
    }
}

// Partition of every active slot's particle by digit; settled particles go to
// their final slot, the others (and their keys) to the next level's buffers.
// The next level's active slots are the slots that land in a child that is
// split again; the thread that moves a particle there lists its new slot.  The
// list's order (like the order of the particles within a child, which the
// cursor atomics set) changes no result: a node's final range is its children
// in octant order followed by its out-of-bounds tail in upload order.
__global__ void __launch_bounds__(kBlock) k_scatter(LevelPair lpair, Nodes nd, Ctx::Ctl *ctl, int advance)
{
    __shared__ int32_t sh[2 * (kBlock / 32)];
    __shared__ int32_t sbase[2];
    const int nap = ctl->cur_nap;
    const LevelBufs &b = lpair.b[ctl->level & 1];
    int round = 0;
    for (int t0 = blockIdx.x * blockDim.x; t0 < nap; t0 += gridDim.x * blockDim.x, round++) {  // block-uniform trip count
    const int t = t0 + threadIdx.x;
    bool act = false;
    int i = 0, nj = 0;
    if (t < nap) {
        i = b.ap[t];
        const int j = b.posnode[i];
        const int32_t p = b.perm[i];
        const int d = b.digit[i];
        // the keys are loaded with the slot's other fields, off the chain
        // through the node, the cursor atomic and the child
        const int64_t kx = b.kx[i], ky = b.ky[i], kz = b.kz[i];
        const int32_t nid = b.nl[j];
        const int np = agg_inc(b.cursor, 9 * j + d);
        const int32_t first = nd.first[nid];
        if (first >= 0 && d < 8) {
            const int32_t child = first + d;
            const uint8_t cn = nd.needs[child];
            if (cn) {  // split again: by the next level (1) or by k_local (2), which reads the keys there
                b.kx_next[np] = kx;
                b.ky_next[np] = ky;
                b.kz_next[np] = kz;
            }
            if (cn == 1) {
                // its digit in the child for the next level, and the child's histogram
                // (k_nodes of this level has left the histogram zero); its new
                // slot np is active at the next level, under the child's entry
                // in the next split list
                const int32_t cj = nd.nlx[child];
                const int d2 = octant_digit(nd.bkey + 9 * (int64_t)child, kx, ky, kz);
                b.digit_next[np] = (uint8_t)d2;
                agg_inc(b.hist, 9 * cj + d2);
                b.perm_next[np] = p;
                act = true;
                i = np;
                nj = cj;
            } else {
                b.perm_final[np] = p;
                b.pnode[np] = child;  // single-particle leaf, or a serial root for k_local
            }
        } else {
            b.perm_final[np] = p;
            b.pnode[np] = nid;  // leaf of a serial node, or the node's out-of-bounds tail
        }
    }
    const int32_t q = block_reserve_rounds(act, &ctl->next_active, sh, sbase, round);
    if (act) {
        b.ap_next[q] = i;
        b.posnode_next[i] = nj;
    }
    }
    if (!advance) return;
    // launched level loop: the last block to finish also advances the level
    // (k_level_next's bookkeeping, without a launch of its own); a captured
    // loop keeps k_level_next, which sets the loop's condition
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();  // this block's counts before its arrival
        last = atomicAdd(&ctl->scatter_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();  // every block's counts before they are read
        volatile Ctx::Ctl *v = ctl;
        if (v->cur_nnl != 0) {  // a level queued past the last one leaves the block as it was
            v->level += 1;
            v->cur_nnl = v->next_needs;
            v->cur_nap = v->next_active;
            v->next_needs = 0;
            v->next_active = 0;
        }
        v->scatter_done = 0u;
    }
}

// Between levels: the counts the last level produced become the next level's,
// the accumulators restart.  `inc` advances the level (0 before the first).
// In a captured step the loop is a conditional node whose condition this sets.
__global__ void k_level_next(Ctx::Ctl *ctl, int inc, int max_depth, cudaGraphConditionalHandle h, int use_h)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    // a level queued past the last one (the launched loop runs one level ahead
    // of the host) had no split nodes: it leaves the control block as it was
    if (inc && ctl->cur_nnl == 0) return;
    ctl->level += inc;
    ctl->cur_nnl = ctl->next_needs;
    ctl->cur_nap = ctl->next_active;
    ctl->next_needs = 0;
    ctl->next_active = 0;
    // a captured loop runs on after an error until no node splits: a node that
    // could not split (pool exhausted, maximum depth) is a leaf holding its
    // particles, so every slot settles and the kernels after the build read a
    // whole tree; the host then reports the error
    if (use_h) cudaGraphSetConditional(h, (ctl->cur_nnl > 0 && ctl->level < max_depth) ? 1u : 0u);
}

// Out-of-bounds tails are the only ranges whose order the partition leaves
// open; put them in upload order so the build is deterministic.  One block per
// node with a tail of two or more: bitonic sort of (upload index, slot) pairs in
// shared memory (tails up to kDropSort), or a block-strided rank sort for longer
// tails.
constexpr int kDropSort = 4096;

__global__ void k_sort_drops(Ctx::Ctl *ctl, const int32_t *drop_list, Nodes nd, int32_t *perm, const int32_t *id,
                             int32_t *scratch)
{
    __shared__ long long key[kDropSort];
    const int ndn = min(ctl->ndrop_nodes, kMaxDropNodes);
    if (ctl->ndrop_nodes > kMaxDropNodes && blockIdx.x == 0 && threadIdx.x == 0)
        atomicExch(&ctl->err_code, (int)AG2_E_CAPACITY);
    for (int q = blockIdx.x; q < ndn; q += gridDim.x) {
        const int64_t nid = drop_list[q];
        const int32_t nd8 = nd.ndrop[nid];
        if (nd8 < 2) continue;
        const int32_t e = nd.start[nid] + nd.count[nid];
        const int32_t b = e - nd8;
        if (nd8 <= kDropSort) {
            int m = 1;
            while (m < nd8) m <<= 1;
            for (int t = threadIdx.x; t < m; t += blockDim.x)
                key[t] = t < nd8 ? (((long long)id[perm[b + t]]) << 32) | (unsigned)perm[b + t] : LLONG_MAX;
            __syncthreads();
            for (int k = 2; k <= m; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int t = threadIdx.x; t < m; t += blockDim.x) {
                        int u = t ^ j;
                        if (u > t) {
                            bool up = (t & k) == 0;
                            long long x = key[t], y = key[u];
                            if ((x > y) == up) {
                                key[t] = y;
                                key[u] = x;
                            }
                        }
                    }
                    __syncthreads();
                }
            for (int t = threadIdx.x; t < nd8; t += blockDim.x) perm[b + t] = (int32_t)(key[t] & 0xffffffffLL);
            __syncthreads();
        } else {
            // rank of each element by its upload index (all distinct), O(k^2 / threads)
            for (int t = threadIdx.x; t < nd8; t += blockDim.x) {
                int32_t v = perm[b + t], kv = id[v], r = 0;
                for (int u = 0; u < nd8; u++) r += id[perm[b + u]] < kv ? 1 : 0;
                scratch[b + r] = v;
            }
            __syncthreads();
            for (int t = threadIdx.x; t < nd8; t += blockDim.x) perm[b + t] = scratch[b + t];
            __syncthreads();
        }
    }
}

__global__ void k_reorder(int n, const int32_t *__restrict__ perm, Particles s, Particles d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = perm[i];
    d.px[i] = s.px[p];
    d.py[i] = s.py[p];
    d.pz[i] = s.pz[p];
    d.vx[i] = s.vx[p];
    d.vy[i] = s.vy[p];
    d.vz[i] = s.vz[p];
    d.ax[i] = s.ax[p];
    d.ay[i] = s.ay[p];
    d.az[i] = s.az[p];
    d.m[i] = s.m[p];
    d.U[i] = s.U[p];
    d.dUdt[i] = s.dUdt[p];
    d.h[i] = s.h[p];
    d.rho[i] = s.rho[p];
    d.P[i] = s.P[p];
    d.T[i] = s.T[p];
    d.vdens[i] = s.vdens[p];
    d.tstep[i] = s.tstep[p];
    d.tnext[i] = s.tnext[p];
    d.type[i] = s.type[p];
    d.id[i] = s.id[p];
}

// Particle::node as the reference leaves it.  A particle lands on a node when
// it is the first to reach it during serial insertion and keeps the pointer as
// the node splits and the particle moves down (Node.cpp:621-625, 645-651).  So a
// leaf particle points at its leaf; a particle that fails the bounds of a
// serial child keeps pointing at the parent if it was the first (lowest upload
// index) to reach that parent, and is null otherwise (the parallel root resets
// every pointer, Node.cpp:472).
__global__ void k_refnode(int n, Nodes nd, const int32_t *__restrict__ pnode, const int32_t *__restrict__ id,
                          int32_t *__restrict__ refnode)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t pn = pnode[i];
    int32_t ref = -1;
    if (nd.leafpos[pn] == i) {
        ref = pn;
    } else if (nd.mode[pn] == MODE_SER && i >= nd.start[pn] + nd.count[pn] - nd.ndrop[pn]) {
        int32_t X = nd.parent[pn];
        int32_t b = nd.start[X], e = b + nd.count[X] - nd.ndrop[X];
        int32_t lo = INT32_MAX;
        for (int32_t j = b; j < e; j++) lo = min(lo, id[j]);
        if (id[i] == lo) ref = X;
    }
    refnode[i] = ref;
}

// ---- moments, bottom-up ----------------------------------------------------

struct Sums {
    double m, mx, my, mz, g, gvx, gvy, gvz;
    int32_t ng;
    int32_t first_id;     // lowest upload index in the set (the first one serial insertion sees)
    double first_m;       // its mass
    __device__ void zero()
    {
        m = mx = my = mz = g = gvx = gvy = gvz = 0.0;
        ng = 0;
        first_id = INT32_MAX;
        first_m = 1.0;
    }
    __device__ void add_particle(const Particles &P, int i)
    {
        double mi = P.m[i];
        if (P.id[i] < first_id) {
            first_id = P.id[i];
            first_m = mi;
        }
        m += mi;
        mx += P.px[i] * mi;
        my += P.py[i] * mi;
        mz += P.pz[i] * mi;
        if (P.type[i] == 2) {
            g += mi;
            gvx += P.vx[i] * mi;
            gvy += P.vy[i] * mi;
            gvz += P.vz[i] * mi;
            ng += 1;
        }
    }
    __device__ void add_sum(const NodeSum &t)
    {
        if (t.first_id < first_id) {
            first_id = t.first_id;
            first_m = t.first_m;
        }
        m += t.m;
        mx += t.mx;
        my += t.my;
        mz += t.mz;
        if (t.ng) {  // without gas the four sums are exact zeros: adding them changes nothing
            g += t.g;
            gvx += t.gvx;
            gvy += t.gvy;
            gvz += t.gvz;
            ng += t.ng;
        }
    }
};

// RN(q/m) for q = RN(x*m) and m > 0, without a division.  With q = x*m*(1+e),
// |e| <= 2^-53, the quotient q/m lies strictly within one unit in the last
// place of x, so it rounds to x or to x's neighbour on the quotient's side.
// The residual r = q - x*m is exact (one fma) and q/m - x = r/m.  Half the gap
// to that neighbour is a power of two, so comparing |r| with it times m is a
// comparison of bit patterns after an exponent shift; ties go to the even
// significand.  Outside magnitudes 2^-400 .. 2^400 (where none of this can
// underflow or overflow), divide.
__device__ __forceinline__ double div_back(double x, double m, double q)
{
    const long long bx = __double_as_longlong(x), bm = __double_as_longlong(m);
    const int ex = (int)((bx >> 52) & 0x7ff), em = (int)((bm >> 52) & 0x7ff);
    const bool xzero = (bx << 1) == 0;
    if (bm < 0 || em < 1023 - 400 || em >= 1023 + 400 || (!xzero && (ex < 1023 - 400 || ex >= 1023 + 400)))
        return __ddiv_rn(q, m);
    if (xzero) return x;
    const double r = __fma_rn(-x, m, q);  // exact: q - x*m
    const long long br = __double_as_longlong(r);
    if ((br << 1) == 0) return x;
    const bool away = (br < 0) == (bx < 0);  // |q/m| > |x|
    // half the gap on that side: 2^(e-53) for the ulp 2^(e-52) of x's binade,
    // 2^(e-54) toward zero from a power of two (the binade below is twice as fine)
    const bool pow2 = (bx & 0x000fffffffffffffLL) == 0;
    const int k = (ex - 1023) - 53 - ((!away && pow2) ? 1 : 0);
    const long long blim = bm + ((long long)k << 52);  // m * 2^k, still normal in the guarded range
    const long long bar = br & 0x7fffffffffffffffLL;   // |r|
    const long long by = away ? bx + 1 : bx - 1;       // the neighbour
    if (bar < blim) return x;
    if (bar > blim) return __longlong_as_double(by);
    return (bx & 1) ? __longlong_as_double(by) : x;
}

// node record shared by leaves and internal nodes: moments, FP32 walk records
// what the FP32 walk records need beyond a node's moments
struct RecArgs {
    float theta;           // (float)theta, rounded once on the host
    const double *inst_R;  // root half-width per instance (walk_scale)
};

// first_child and leafslot are the node's nd.first and nd.leafpos, which the
// callers already hold (a leaf's first is -1; an internal node's leafpos is -1)
__device__ __forceinline__ void store_node(Nodes &nd, int64_t nid, const Particles &P, const Sums &tot, double mass,
                                           double cx, double cy, double cz, double gas, double mvx, double mvy,
                                           double mvz, int32_t ng, uint8_t cmask, bool leaf, int32_t lp,
                                           int32_t first_child, int32_t leafslot, RecArgs ra)
{
    NodeSum ts;
    ts.m = tot.m;
    ts.mx = tot.mx;
    ts.my = tot.my;
    ts.mz = tot.mz;
    ts.g = tot.g;
    ts.gvx = tot.gvx;
    ts.gvy = tot.gvy;
    ts.gvz = tot.gvz;
    ts.first_m = tot.first_m;
    ts.ng = tot.ng;
    ts.first_id = tot.first_id;
    ts.pad[0] = ts.pad[1] = 0.0;
    nd.tsum[nid] = ts;
    NodeMom mm;
    mm.mass = mass;
    mm.cx = cx;
    mm.cy = cy;
    mm.cz = cz;
    mm.gas = gas;
    mm.mvx = mvx;
    mm.mvy = mvy;
    mm.mvz = mvz;
    nd.mom[nid] = mm;
    // FP32 walk record, lengths in the instance's scaled units (walk_scale):
    // COM split into hi + lo floats, mass * ls^2 (the walk's accelerations come
    // out in the caller's units), (radius/theta)^2, gasMass * ls^2 (the FP32
    // SPH pair's scaled mass); velocities as they are
    const int k = walk_scale_exp(ra.inst_R[nd.inst[nid]]);
    const double sx = scale2(cx, k), sy = scale2(cy, k), sz = scale2(cz, k);
    const float hx = (float)sx, hy = (float)sy, hz = (float)sz;
    const float lx = (float)(sx - (double)hx), ly = (float)(sy - (double)hy), lz = (float)(sz - (double)hz);
    WalkRec w;
    w.A = make_float4(hx, hy, hz, (float)scale2(mass, 2 * k));
    float mac = -1.0f;
    if (!leaf) {
        // accept when radius/r < theta  <=>  r^2 > (radius/theta)^2; FP32 is
        // enough for the threshold the FP32 walk tests with its guard band
        const float q = (float)scale2(nd.radius[nid], k) / ra.theta;
        mac = q * q;
    }
    w.B = make_float4(lx, ly, lz, mac);
    w.C = make_int4(first_child, leafslot, (int)cmask, 0);
    if ((dbits(gas) << 1) == 0)
        w.D = make_float4(0.f, 0.f, 0.f, 0.f);  // no gas: the walk reads none of it (its SPH needs D.w > 0)
    else if (leaf && lp >= 0)
        w.D = make_float4((float)P.vx[lp], (float)P.vy[lp], (float)P.vz[lp], (float)scale2(gas, 2 * k));
    else
        w.D = make_float4((float)mvx, (float)mvy, (float)mvz, (float)scale2(gas, 2 * k));
    nd.wrec[nid] = w;
}

// Moments from the node's own mass set: the centre of mass and gas velocity as
// ratios of sums, the NaN rule of serial nodes whose first particle is
// massless, and the uniform-gas gasMass table.
__device__ __forceinline__ void finish_sums(Nodes &nd, int64_t nid, uint8_t mode, const Sums &own,
                                            const double *gas_prefix, const int32_t *gas_off, const uint8_t *gas_uni,
                                            double &mass, double &cx, double &cy, double &cz, double &gas,
                                            double &mvx, double &mvy, double &mvz)
{
    mass = own.m;
    gas = own.g;
    cx = cy = cz = mvx = mvy = mvz = 0.0;
    const bool serial = (mode == MODE_SER || mode == MODE_SER_ENTRY);
    if (serial && own.first_m == 0.0 && own.first_id != INT32_MAX) {
        // serial insertion's running mean starts with (0*0 + x*0)/0 when the
        // first particle to arrive is massless (Node.cpp:698): the centre of
        // mass is NaN from then on, so the node is always opened
        cx = cy = cz = __longlong_as_double(0x7ff8000000000000LL);
    } else if (mass > 0.0) {
        const double im = 1.0 / mass;  // one FP64 division per node
        cx = own.mx * im;
        cy = own.my * im;
        cz = own.mz * im;
    }
    const int k = nd.inst[nid];
    if (gas_uni[k]) gas = gas_prefix[gas_off[k] + own.ng];
    if (own.g > 0) {
        const double ig = 1.0 / own.g;
        mvx = own.gvx * ig;
        mvy = own.gvy * ig;
        mvz = own.gvz * ig;
    }
}

// Leaf moments.  idx(k) is the state index of the k-th particle of the node's
// range (the leaf particle, when there is one, is the first).
template <class Idx>
__device__ __forceinline__ void moments_leaf(Nodes &nd, int64_t nid, const Particles &P, Idx idx,
                                             const double *gas_prefix, const int32_t *gas_off,
                                             const uint8_t *gas_uni, RecArgs ra)
{
    const int32_t cnt = nd.count[nid], ndrop = nd.ndrop[nid];
    const uint8_t mode = nd.mode[nid];
    if (cnt == 1 && ndrop == 0) {
        // the common leaf: one particle inside its bounds.  Its sums are the
        // particle's own values (0 + a = a and 0 + x*m = RN(x*m) exactly).
        const int32_t i = idx(0);
        const double mp = P.m[i], px = P.px[i], py = P.py[i], pz = P.pz[i];
        const bool isgas = P.type[i] == 2;
        Sums t;
        t.m = mp;
        t.mx = __dmul_rn(px, mp);
        t.my = __dmul_rn(py, mp);
        t.mz = __dmul_rn(pz, mp);
        t.g = isgas ? mp : 0.0;
        t.gvx = t.gvy = t.gvz = 0.0;
        double mvx = 0.0, mvy = 0.0, mvz = 0.0;
        if (isgas) {
            const double vx = P.vx[i], vy = P.vy[i], vz = P.vz[i];
            t.gvx = __dmul_rn(vx, mp);
            t.gvy = __dmul_rn(vy, mp);
            t.gvz = __dmul_rn(vz, mp);
            if (mode != MODE_VEC1 && __double_as_longlong(mp) > 0) {  // Node.cpp:679-696
                mvx = vx;
                mvy = vy;
                mvz = vz;
            }
        }
        t.ng = isgas ? 1 : 0;
        t.first_id = P.id[i];
        t.first_m = mp;
        double cx = px, cy = py, cz = pz;  // VEC1: the position itself (Node.cpp:409-418)
        if (mode != MODE_VEC1) {
            // one serial insertion into an empty leaf (Node.cpp:678-698): the
            // running mean (0*(m-m) + x*m)/m, rounded as the reference rounds it
            const long long bm = __double_as_longlong(mp);
            if (bm > 0) {
                cx = div_back(px, mp, t.mx);
                cy = div_back(py, mp, t.my);
                cz = div_back(pz, mp, t.mz);
            } else if ((bm << 1) != 0) {
                cx = __ddiv_rn(t.mx, mp);
                cy = __ddiv_rn(t.my, mp);
                cz = __ddiv_rn(t.mz, mp);
            } else {
                cx = cy = cz = 0.0;
            }
        }
        // one particle inside its bounds: it sits at the leaf's first slot (leafpos)
        store_node(nd, nid, P, t, mp, cx, cy, cz, t.g, mvx, mvy, mvz, t.ng, 0, true, i, -1, i, ra);
        return;
    }
    Sums tot, own;  // tot: whole routed range; own: the reference's mass set
    tot.zero();
    for (int32_t k = 0; k < cnt; k++) tot.add_particle(P, idx(k));
    if (mode == MODE_VEC1) {
        own = tot;
    } else {
        own.zero();
        for (int32_t k = 0; k < cnt - ndrop; k++) own.add_particle(P, idx(k));
    }
    double mass, cx, cy, cz, gas, mvx, mvy, mvz;
    const int32_t lslot = nd.leafpos[nid];
    const bool has = lslot >= 0;
    const int32_t lp = has ? idx(0) : -1;
    if (has) {
        const double mp = P.m[lp];
        const bool isgas = P.type[lp] == 2;
        mass = mp;
        gas = isgas ? mp : 0.0;
        mvx = mvy = mvz = 0.0;
        if (mode == MODE_VEC1) {
            // Node.cpp:409-418: COM is the position itself, mVel stays zero
            cx = P.px[lp];
            cy = P.py[lp];
            cz = P.pz[lp];
        } else {
            // one serial insertion into an empty leaf (Node.cpp:678-698): the
            // running mean (0*(m-m) + x*m)/m, rounded as the reference rounds it
            cx = cy = cz = 0.0;
            if (mass > 0.0) {
                cx = div_back(P.px[lp], mp, __dmul_rn(P.px[lp], mp));
                cy = div_back(P.py[lp], mp, __dmul_rn(P.py[lp], mp));
                cz = div_back(P.pz[lp], mp, __dmul_rn(P.pz[lp], mp));
            } else if (mass != 0.0) {
                cx = __ddiv_rn(__dmul_rn(P.px[lp], mp), mass);
                cy = __ddiv_rn(__dmul_rn(P.py[lp], mp), mass);
                cz = __ddiv_rn(__dmul_rn(P.pz[lp], mp), mass);
            }
            if (isgas && gas > 0) {
                // gas velocity of a leaf is only ever read for export (the walk
                // uses the leaf particle's own velocity, Node.cpp:111-113)
                mvx = P.vx[lp];
                mvy = P.vy[lp];
                mvz = P.vz[lp];
            }
        }
    } else {
        finish_sums(nd, nid, mode, own, gas_prefix, gas_off, gas_uni, mass, cx, cy, cz, gas, mvx, mvy, mvz);
    }
    store_node(nd, nid, P, tot, mass, cx, cy, cz, gas, mvx, mvy, mvz, own.ng, 0, true, lp, -1, lslot, ra);
}

// Internal-node moments after its children's: sums over the children in octant
// order, plus the node's out-of-bounds tail (idx(k), k in [count - ndrop, count))
// for the routed range.
template <class Idx>
__device__ __forceinline__ void moments_internal(Nodes &nd, int64_t nid, const Particles &P, Idx idx,
                                                 const double *gas_prefix, const int32_t *gas_off,
                                                 const uint8_t *gas_uni, RecArgs ra)
{
    const int32_t ndrop = nd.ndrop[nid], first = nd.first[nid];
    const uint8_t mode = nd.mode[nid];
    Sums tot, own;
    own.zero();
    uint8_t cmask = 0;
    unsigned live = 0;
#pragma unroll
    for (int o = 0; o < 8; o++) live |= (nd.count[first + o] != 0 ? 1u : 0u) << o;
    while (live) {
        const int o = __ffs(live) - 1;
        live &= live - 1;
        const int64_t c = first + o;
        const NodeSum t = nd.tsum[c];
        own.add_sum(t);
        // bit o: the child's own mass != 0 (on the bits).  Without an
        // out-of-bounds tail that mass is its routed sum t.m, bit for bit (the
        // same terms in the same order; a one-particle leaf's is the particle's
        // mass); with one, it is the mass the child stored.
        const double cm = nd.ndrop[c] ? nd.mom[c].mass : t.m;
        if ((dbits(cm) << 1) != 0) cmask |= (uint8_t)(1u << o);
    }
    tot = own;
    if (ndrop) {  // the node's own out-of-bounds tail ends its range
        const int32_t cnt = nd.count[nid];
        for (int32_t k = cnt - ndrop; k < cnt; k++) tot.add_particle(P, idx(k));
    }
    if (mode == MODE_PAR) own = tot;  // the parallel path sums escapers too (Node.cpp:477-499)
    double mass, cx, cy, cz, gas, mvx, mvy, mvz;
    finish_sums(nd, nid, mode, own, gas_prefix, gas_off, gas_uni, mass, cx, cy, cz, gas, mvx, mvy, mvz);
    store_node(nd, nid, P, tot, mass, cx, cy, cz, gas, mvx, mvy, mvz, own.ng, cmask, false, -1, first, -1, ra);
}

// Leaves (every level at once), on the state in tree order, one thread per
// slot: the thread of a leaf's first slot computes it.  pnode[s] is the node a
// slot settled in (its leaf, or the node whose out-of-bounds tail holds it),
// and a leaf's in-bounds particle sits at its first slot, so these are exactly
// the non-empty leaves, met in tree order: neighbouring threads read
// neighbouring particles.
__global__ void __launch_bounds__(kBlock) k_moments_leaf(int n, const int32_t *__restrict__ pnode, Nodes nd,
                                                         Particles P, const double *gas_prefix,
                                                         const int32_t *gas_off, const uint8_t *gas_uni, RecArgs ra)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int32_t v = pnode[s];
        // a leaf's slots all settled in it, so its first slot is the one whose
        // left neighbour settled elsewhere (a coalesced read, not nd.start[v])
        if (v < 0 || (s > 0 && pnode[s - 1] == v) || nd.first[v] >= 0) continue;
        moments_leaf(nd, v, P, [=](int32_t k) { return s + k; }, gas_prefix, gas_off, gas_uni, ra);
    }
}

// Internal nodes of one level, after the level below: the level's list
// segment given explicitly, or (kDev) the level ctl->mlev of the control block.
//
// Levels of at most kFewNodes internal nodes are finished by one thread block,
// a run of them in one launch with a block barrier between levels: a level
// that small would otherwise pay a whole dependent launch for one pass of its
// nodes' load chains (the top levels of the level loop, the deepest levels of
// the serial subtrees).
constexpr int kFewNodes = 2 * kBlock;

// levels hi down to lo (deepest first) by the calling block alone
__device__ __forceinline__ void moments_levels(int hi, int lo, const int32_t *__restrict__ lil, const Ctx::Ctl *ctl,
                                               Nodes &nd, const Particles &P, const double *gas_prefix,
                                               const int32_t *gas_off, const uint8_t *gas_uni, RecArgs ra)
{
    for (int L = hi; L >= lo; L--) {
        const int32_t cnt = ctl->lvl_cnt[L];
        const int32_t *list = lil + ctl->lvl_start[L];
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int64_t nid = list[t];
            moments_internal(nd, nid, P, [=](int32_t k) { return nd.start[nid] + k; }, gas_prefix, gas_off, gas_uni,
                             ra);
        }
        __syncthreads();  // this level's records before the next level reads them
    }
}

// the shallowest level of the run of small levels that starts at level hi
__device__ __forceinline__ int few_run_end(const Ctx::Ctl *ctl, int hi)
{
    int lo = hi;
    while (lo > 0 && ctl->lvl_cnt[lo - 1] <= kFewNodes) lo--;
    return lo;
}

template <bool kDev>
__global__ void __launch_bounds__(kBlock) k_moments_int(int cnt_lvl, const int32_t *__restrict__ list,
                                                        Ctx::Ctl *ctl, Nodes nd, Particles P,
                                                        const double *gas_prefix, const int32_t *gas_off,
                                                        const uint8_t *gas_uni, RecArgs ra)
{
    if (kDev) {
        const int L = ctl->mlev;
        if (L < 0) return;
        cnt_lvl = ctl->lvl_cnt[L];
        if (cnt_lvl <= kFewNodes) {  // a run of small levels: block 0 alone
            if (blockIdx.x != 0) return;
            const int lo = few_run_end(ctl, L);
            moments_levels(L, lo, list, ctl, nd, P, gas_prefix, gas_off, gas_uni, ra);
            if (threadIdx.x == 0) ctl->mlev_last = lo;
            return;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mlev_last = L;
        list += ctl->lvl_start[L];
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt_lvl; t += gridDim.x * blockDim.x) {
        const int64_t nid = list[t];
        // the node's start is read only for an out-of-bounds tail
        moments_internal(nd, nid, P, [=](int32_t k) { return nd.start[nid] + k; }, gas_prefix, gas_off, gas_uni, ra);
    }
}

// levels hi down to lo, each of at most kFewNodes internal nodes, in one block
__global__ void __launch_bounds__(kBlock) k_moments_few(int hi, int lo, const int32_t *__restrict__ lil,
                                                        const Ctx::Ctl *ctl, Nodes nd, Particles P,
                                                        const double *gas_prefix, const int32_t *gas_off,
                                                        const uint8_t *gas_uni, RecArgs ra)
{
    moments_levels(hi, lo, lil, ctl, nd, P, gas_prefix, gas_off, gas_uni, ra);
}

// internal nodes per level (one shared-memory histogram per block)
__global__ void __launch_bounds__(kBlock) k_lvl_hist(Ctx::Ctl *ctl, const int2 *__restrict__ lint, int64_t cap)
{
    __shared__ int32_t hs[AG2_MAX_DEPTH];
    for (int k = threadIdx.x; k < AG2_MAX_DEPTH; k += blockDim.x) hs[k] = 0;
    __syncthreads();
    const int n = (int)min((int64_t)ctl->nlint, cap);  // entries a failed reservation counted are not there
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int2 e = lint[t];
        if (e.x >= 0 && e.y >= 0 && e.y < AG2_MAX_DEPTH) atomicAdd(&hs[e.y], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < AG2_MAX_DEPTH; k += blockDim.x)
        if (hs[k]) atomicAdd(&ctl->lvl_cnt[k], hs[k]);
}

// node count at the end of the level loop (the serial subtrees allocate from a pool after it)
__global__ void k_mark_loop_nodes(Ctx::Ctl *ctl)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) ctl->loop_nodes = ctl->node_count;
}

// list segments per level (and the bucketing cursors); the deepest level with
// internal nodes starts the moments pass
__global__ void k_lvl_prefix(Ctx::Ctl *ctl, cudaGraphConditionalHandle h, int use_h)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int32_t acc = 0, deepest = -1;
    for (int L = 0; L < AG2_MAX_DEPTH; L++) {
        ctl->lvl_start[L] = acc;
        ctl->lvl_off[L] = acc;
        acc += ctl->lvl_cnt[L];
        if (ctl->lvl_cnt[L]) deepest = L;
    }
    ctl->mlev = deepest;
    if (use_h) cudaGraphSetConditional(h, deepest >= 0 ? 1u : 0u);
}

// the next shallower level with internal nodes (-1 when done)
__global__ void k_mlev_next(Ctx::Ctl *ctl, cudaGraphConditionalHandle h, int use_h)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int L = ctl->mlev_last - 1;
    while (L >= 0 && ctl->lvl_cnt[L] == 0) L--;
    ctl->mlev = L;
    if (use_h) cudaGraphSetConditional(h, L >= 0 ? 1u : 0u);
}

// internal nodes into one list segment per level (cursors start at the
// segments).  A block ranks its entries per level in shared memory and takes
// one range per level from the global cursor: the ~20 cursors are the same
// words for every block, and per-warp atomics on them serialise.  The order
// within a segment changes no result (each node's moments are its own).
__global__ void __launch_bounds__(kBlock) k_bucket(Ctx::Ctl *ctl, const int2 *__restrict__ lint, int32_t *lil,
                                                   int64_t cap)
{
    __shared__ int32_t cnt[AG2_MAX_DEPTH], base[AG2_MAX_DEPTH];
    const int n = (int)min((int64_t)ctl->nlint, cap);
    for (int t0 = blockIdx.x * blockDim.x; t0 < n; t0 += gridDim.x * blockDim.x) {  // block-uniform trip count
        for (int k = threadIdx.x; k < AG2_MAX_DEPTH; k += blockDim.x) cnt[k] = 0;
        __syncthreads();
        const int t = t0 + threadIdx.x;
        int2 e = make_int2(-1, 0);
        int r = 0;
        if (t < n) {
            e = lint[t];
            if (e.y < 0 || e.y >= AG2_MAX_DEPTH) e.x = -1;
            if (e.x >= 0) r = atomicAdd_block(&cnt[e.y], 1);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < AG2_MAX_DEPTH; k += blockDim.x)
            if (cnt[k]) base[k] = atomicAdd(&ctl->lvl_off[k], cnt[k]);
        __syncthreads();
        if (e.x >= 0) lil[base[e.y] + r] = e.x;
        __syncthreads();  // cnt and base are reset for the next stride
    }
}

// ---- serial subtrees, one warp each ---------------------------------------
//
// A node with fewer than split_threshold particles under a parallel node is the
// root of a serial subtree (Node.cpp:420-428, 597-699): every node below it
// splits when two of its particles land inside its bounds.  Such a subtree
// never holds more than split_threshold - 1 particles, so one warp builds it in
// shared memory, level by level, with the level loop's rules: the same rounded
// bounds, digits, modes, drop tails in upload order, child centres and
// half-widths.  Its internal nodes join the list the internal moments read.
//
// Nodes come from a warp-private pool of kPoolChunk nodes (one global atomic
// per chunk); a chunk's unused tail stays a hole in the pool, which no kernel
// reaches (every traversal starts at a root, and the per-node passes only
// touch a node's own fields).

constexpr int kLocalCapMax = 1024;  // largest serial subtree (particles) built by one warp
constexpr int kLocalWarps = 7;      // warps per thread block of k_local (fewer for large subtrees)
constexpr int kLocalBlocks = 4;     // resident blocks per SM the registers are budgeted for
constexpr int kPoolChunk = 512;     // nodes per warp-private pool chunk
constexpr int kIntChunk = 128;      // internal-node-list entries per warp-private stretch
constexpr int kCoop = 16;           // frontier nodes of more particles are done by the whole warp

// Shared memory of one warp for subtrees of up to `cap` particles (cap a
// multiple of 8).  Per particle: keys 3 x 8 B and particle index 4 B (fixed
// slots), position -> slot 2 x 2 B, digit 1 B.  Per frontier node (at most one
// per particle): node 2 x 4 B, start and count 2 x 2 x 2 B, first child 4 B,
// digit starts 9 x 2 B, parent of a next-frontier node 4 B.
__host__ __device__ constexpr size_t local_smem_bytes(int cap) { return (size_t)cap * 76; }

__global__ void __launch_bounds__(kLocalWarps * 32, kLocalBlocks) k_local(const int32_t *__restrict__ roots, int cap,
                                                            Nodes nd, Ctx::Ctl *ctl, const int64_t *__restrict__ pkey,
                                                            int64_t keycap, int32_t *perm_final, int32_t *pnode,
                                                            const int32_t *__restrict__ sid, int max_depth,
                                                            int64_t node_cap)
{
    extern __shared__ __align__(16) unsigned char lsm[];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    const unsigned lt = (1u << lane) - 1u;
    unsigned char *base = lsm + (size_t)wib * local_smem_bytes(cap);
    int64_t *KX = reinterpret_cast<int64_t *>(base);
    int64_t *KY = KX + cap, *KZ = KY + cap;
    int32_t *PID = reinterpret_cast<int32_t *>(KZ + cap);
    int32_t *const FN0 = PID + cap, *const FN1 = PID + 2 * cap;
    int32_t *FF = PID + 3 * cap;  // per frontier node: first child, -1 leaf, -2 cannot split
    int16_t *const L0 = reinterpret_cast<int16_t *>(FF + cap);
    int16_t *const L1 = L0 + cap;
    int16_t *const FS0 = L1 + cap, *const FS1 = L1 + 2 * cap;
    int16_t *const FC0 = L1 + 3 * cap, *const FC1 = L1 + 4 * cap;
    int16_t *const FH = L1 + 5 * cap;  // 9 per frontier node
    uint8_t *DIG = reinterpret_cast<uint8_t *>(FH + 9 * cap);
    int32_t *FPAR = reinterpret_cast<int32_t *>(DIG + cap);  // parent of each next-frontier node

    const int nroots = ctl->nlocal;
    unsigned long long pool = 0, pool_end = 0;  // warp-private node pool [pool, pool_end)
    int ipool = 0, ipool_end = 0;                // warp-private stretch of the internal-node list
    long long splits = 0;
    int deepest = 0;
    for (int r = blockIdx.x * (blockDim.x >> 5) + wib; r < nroots; r += nwarps) {
        const int32_t v0 = roots[r];
        const int32_t s0 = nd.start[v0], n = nd.count[v0];
        int level = nd.level[v0];
        {
            const int bsel = level & 1;  // the level loop left the keys in the buffer of this node's level
            const int64_t *gx = pkey + (3 * bsel + 0) * keycap, *gy = pkey + (3 * bsel + 1) * keycap,
                          *gz = pkey + (3 * bsel + 2) * keycap;
            for (int j = lane; j < n; j += 32) {
                PID[j] = perm_final[s0 + j];
                KX[j] = gx[s0 + j];
                KY[j] = gy[s0 + j];
                KZ[j] = gz[s0 + j];
                L0[j] = (int16_t)j;
            }
        }
        if (lane == 0) {
            FN0[0] = v0;
            FS0[0] = 0;
            FC0[0] = (int16_t)n;
        }
        int nf = 1, cur = 0;
        __syncwarp();
        while (nf > 0) {
            const int nxt = cur ^ 1;
            // this level's (c) and the next level's (n) halves of the double buffers
            int32_t *const fnc = cur ? FN1 : FN0, *const fnn = cur ? FN0 : FN1;
            int16_t *const fsc = cur ? FS1 : FS0, *const fsn = cur ? FS0 : FS1;
            int16_t *const fcc = cur ? FC1 : FC0, *const fcn = cur ? FC0 : FC1;
            int16_t *const lc = cur ? L1 : L0, *const ln = cur ? L0 : L1;
            // (a) digits and split decision.  A frontier node of more than kCoop
            // particles is done by the whole warp, 32 particles at a time with
            // the digit counts from ballots; the others take one lane each.
            auto digit_of = [&](int q, const int64_t *b) -> int {
                const int64_t x = KX[q], y = KY[q], z = KZ[q];
                // inclusive bounds and octant of Node.cpp:606-608, 706-716, as in k_digit
                if (x < b[0] || x > b[3] || y < b[1] || y > b[4] || z < b[2] || z > b[5]) return 8;
                return (x > b[6] ? 1 : 0) | (y > b[7] ? 2 : 0) | (z > b[8] ? 4 : 0);
            };
            auto decide = [&](int f, int32_t v, int32_t ls, int32_t cnt, int16_t *hh) {
                // hh holds the digit counts: counts -> starts, drops, split decision
                const int32_t ndrop = hh[8], reached = cnt - ndrop;
                int32_t acc = ls;
#pragma unroll
                for (int d = 0; d < 9; d++) {
                    const int32_t cd = hh[d];
                    hh[d] = (int16_t)acc;
                    acc += cd;
                }
                nd.ndrop[v] = ndrop;
                if (ndrop) ctl->any_drop = 1;
                int32_t flag = 1;
                if (reached < 2) {  // a leaf: serial insertion splits only for a second in-bounds particle
                    nd.first[v] = -1;
                    nd.leafpos[v] = reached == 1 ? s0 + ls : -1;
                    flag = -1;
                } else if (level + 1 >= max_depth) {
                    atomicExch(&ctl->err_code, (int)AG2_E_COINCIDENT);
                    atomicExch(&ctl->err_info, (int)v);
                    nd.first[v] = -1;
                    nd.leafpos[v] = -1;
                    flag = -2;
                }
                FF[f] = flag;
            };
            for (int f0 = 0; f0 < nf; f0 += 32) {
                unsigned bigm = __ballot_sync(full, f0 + lane < nf && fcc[f0 + lane] > kCoop);
                while (bigm) {
                    const int f = f0 + __ffs(bigm) - 1;
                    bigm &= bigm - 1;
                    const int32_t v = fnc[f], ls = fsc[f], cnt = fcc[f];
                    int64_t b[9];
                    {
                        // lane k < 9 forms key k (one FP64 addition for the warp), every lane takes all nine
                        const int ax = lane % 3;
                        const double x = ax == 0 ? nd.cx[v] : ax == 1 ? nd.cy[v] : nd.cz[v];
                        const double r = nd.radius[v];
                        const double t = lane < 6 ? __dadd_rn(x, lane < 3 ? -r : r) : x;
                        const int64_t key = okey(t);
#pragma unroll
                        for (int k = 0; k < 9; k++) b[k] = __shfl_sync(full, key, k);
                    }
                    int cn[9];
#pragma unroll
                    for (int d = 0; d < 9; d++) cn[d] = 0;
                    for (int j0 = ls; j0 < ls + cnt; j0 += 32) {
                        const int j = j0 + lane;
                        int d = 15;
                        if (j < ls + cnt) {
                            d = digit_of(lc[j], b);
                            DIG[j] = (uint8_t)d;
                        }
#pragma unroll
                        for (int e = 0; e < 9; e++) cn[e] += __popc(__ballot_sync(full, d == e));
                    }
                    if (lane == 0) {
                        int16_t *hh = FH + 9 * f;
#pragma unroll
                        for (int d = 0; d < 9; d++) hh[d] = (int16_t)cn[d];
                        decide(f, v, ls, cnt, hh);
                    }
                }
            }
            for (int f = lane; f < nf; f += 32) {
                const int32_t v = fnc[f], ls = fsc[f], cnt = fcc[f];
                if (cnt > kCoop) continue;
                int64_t b[9];
                local_keys(nd, v, b);
                int16_t *hh = FH + 9 * f;
#pragma unroll
                for (int d = 0; d < 9; d++) hh[d] = 0;
                for (int j = ls; j < ls + cnt; j++) {
                    const int d = digit_of(lc[j], b);
                    DIG[j] = (uint8_t)d;
                    hh[d]++;
                }
                decide(f, v, ls, cnt, hh);
            }
            __syncwarp();
            // (b) 8-child blocks of this level's splits, from the warp's pool
            int ns = 0;
            for (int f = lane; f < nf; f += 32) ns += FF[f] == 1 ? 1 : 0;
            ns = (int)__reduce_add_sync(full, (unsigned)ns);
            unsigned long long cbase = 0;
            if (ns) {
                const unsigned long long need = 8ull * (unsigned long long)ns;
                bool room = true;
                if (pool + need > pool_end) {
                    const unsigned long long grab = need > (unsigned long long)kPoolChunk ? need : kPoolChunk;
                    unsigned long long b = 0;
                    if (lane == 0) b = atomicAdd((unsigned long long *)&ctl->node_count, grab);
                    b = __shfl_sync(full, b, 0);
                    room = (int64_t)(b + grab) <= node_cap;
                    if (room) {
                        pool = b;
                        pool_end = b + grab;
                    }
                }
                if (room) {
                    cbase = pool;
                    pool += need;
                    splits += ns;
                } else {
                    // pool exhausted: this level's split nodes stay leaves
                    // holding their particles (as at the maximum depth), so
                    // every slot still settles; the host reports the error
                    if (lane == 0) atomicExch(&ctl->err_code, (int)AG2_E_NOMEM);
                    for (int f = lane; f < nf; f += 32)
                        if (FF[f] == 1) {
                            FF[f] = -2;
                            nd.first[fnc[f]] = -1;
                            nd.leafpos[fnc[f]] = -1;
                        }
                    __syncwarp();
                }
            }
            {
                int run = 0;
                for (int f0 = 0; f0 < nf; f0 += 32) {
                    const int f = f0 + lane;
                    const bool s = f < nf && FF[f] == 1;
                    const unsigned bb = __ballot_sync(full, s);
                    if (s) {
                        const int32_t fc = (int32_t)(cbase + 8ull * (unsigned long long)(run + __popc(bb & lt)));
                        FF[f] = fc;
                        nd.first[fnc[f]] = fc;
                        nd.leafpos[fnc[f]] = -1;
                    }
                    run += __popc(bb);
                }
            }
            // this level's internal nodes join the internal-node list with their level
            {
                int ni = 0;
                for (int f = lane; f < nf; f += 32) ni += FF[f] >= 0 ? 1 : 0;
                ni = (int)__reduce_add_sync(full, (unsigned)ni);
                if (ni) {
                    const int rem = ipool_end - ipool;
                    int nb = 0, grab = 0;
                    if (ni > rem) {
                        grab = max(ni - rem, kIntChunk);
                        if (lane == 0) nb = atomicAdd(&ctl->nlint, grab);
                        nb = __shfl_sync(full, nb, 0);
                        if ((int64_t)nb + grab > node_cap) {
                            if (lane == 0) atomicExch(&ctl->err_code, (int)AG2_E_NOMEM);
                            return;
                        }
                    }
                    int run = 0;
                    for (int f0 = 0; f0 < nf; f0 += 32) {
                        const int f = f0 + lane;
                        const bool isi = f < nf && FF[f] >= 0;
                        const unsigned bi = __ballot_sync(full, isi);
                        if (isi) {
                            const int k = run + __popc(bi & lt);
                            nd.lint[k < rem ? ipool + k : nb + (k - rem)] = make_int2(fnc[f], level);
                        }
                        run += __popc(bi);
                    }
                    if (ni > rem) {
                        ipool = nb + (ni - rem);
                        ipool_end = nb + grab;
                    } else {
                        ipool += ni;
                    }
                }
            }
            __syncwarp();
            // (c) partition by digit into the other order; leaves and drop tails settle
            // (the digit starts serve as cursors: afterwards hh[d] is the end of digit d).
            // Nodes of more than kCoop particles: the whole warp, a stable
            // partition of 32 at a time (ranks among the lanes of equal digit).
            auto settle = [&](int f, int32_t v, int32_t ls, int32_t cnt, const int16_t *hh) {
                // the out-of-bounds tail in upload order (the level loop's k_sort_drops rule)
                const int32_t tb = hh[7], te = ls + cnt;
                for (int a = tb + 1; a < te; a++) {
                    const int16_t la = ln[a];
                    const int32_t ka = sid[PID[la]];
                    int bpos = a - 1;
                    while (bpos >= tb && sid[PID[ln[bpos]]] > ka) {
                        ln[bpos + 1] = ln[bpos];
                        bpos--;
                    }
                    ln[bpos + 1] = la;
                }
                const int32_t sb = FF[f] >= 0 ? tb : ls;  // a split node settles its tail; a leaf everything
                for (int p = sb; p < te; p++) {
                    perm_final[s0 + p] = PID[ln[p]];
                    pnode[s0 + p] = v;
                }
            };
            for (int f0 = 0; f0 < nf; f0 += 32) {
                unsigned bigm = __ballot_sync(full, f0 + lane < nf && fcc[f0 + lane] > kCoop);
                while (bigm) {
                    const int f = f0 + __ffs(bigm) - 1;
                    bigm &= bigm - 1;
                    const int32_t v = fnc[f], ls = fsc[f], cnt = fcc[f];
                    int16_t *hh = FH + 9 * f;
                    for (int j0 = ls; j0 < ls + cnt; j0 += 32) {
                        const int j = j0 + lane;
                        const bool valid = j < ls + cnt;
                        const int d = valid ? (int)DIG[j] : 15;
                        const unsigned peers = __match_any_sync(full, d);
                        const int rank = __popc(peers & lt);
                        const int dst = valid ? hh[d] + rank : 0;
                        __syncwarp();
                        if (valid) {
                            ln[dst] = lc[j];
                            if (rank == 0) hh[d] = (int16_t)(dst + __popc(peers));
                        }
                        __syncwarp();
                    }
                    if (lane == 0) settle(f, v, ls, cnt, hh);
                }
            }
            for (int f = lane; f < nf; f += 32) {
                const int32_t v = fnc[f], ls = fsc[f], cnt = fcc[f];
                if (cnt > kCoop) continue;
                int16_t *hh = FH + 9 * f;
                for (int j = ls; j < ls + cnt; j++) {
                    const int d = DIG[j];
                    ln[hh[d]] = lc[j];
                    hh[d]++;
                }
                settle(f, v, ls, cnt, hh);
            }
            __syncwarp();
            // (d) children: 8 lanes per split node, coalesced; non-empty ones form the
            // next frontier.  Their FP64 centres and bounds come after, 32 at a
            // time over that compact list, so no FP64 instruction runs for an
            // empty child (this part issues FP64 at 1/64 of the FP32 rate).
            int nn = 0;
            for (int f0 = 0; f0 < nf; f0 += 4) {
                const int f = f0 + (lane >> 3), o = lane & 7;
                const int32_t ff = f < nf ? FF[f] : -1;
                bool join = false;
                int32_t c = 0, cs = 0, cc = 0, v = 0;
                if (ff >= 0) {
                    v = fnc[f];
                    const int16_t *hh = FH + 9 * f;
                    c = ff + o;
                    cs = o ? hh[o - 1] : fsc[f];
                    cc = hh[o] - cs;
                    const double rc = scale2(nd.radius[v], -1);  // radius / 2 (Node.cpp:640), on the exponent
                    nd.start[c] = s0 + cs;
                    nd.count[c] = cc;
                    nd.ndrop[c] = 0;
                    nd.first[c] = -1;
                    nd.parent[c] = v;
                    nd.level[c] = (int8_t)(level + 1);
                    nd.radius[c] = rc;
                    nd.inst[c] = nd.inst[v];
                    nd.mode[c] = cc ? MODE_SER : MODE_EMPTY;
                    nd.leafpos[c] = -1;
                    join = cc > 0;
                }
                const unsigned bj = __ballot_sync(full, join);
                if (join) {
                    const int q = nn + __popc(bj & lt);
                    fnn[q] = c;
                    fsn[q] = (int16_t)cs;
                    fcn[q] = (int16_t)cc;
                    FPAR[q] = v;
                    DIG[q] = (uint8_t)o;  // the digits of this level are consumed
                }
                nn += __popc(bj);
            }
            __syncwarp();
            for (int q = lane; q < nn; q += 32) {  // child o: centre c + r*(+-0.5) (Node.cpp:630-642)
                const int32_t c = fnn[q], v = FPAR[q];
                const int o = DIG[q];
                const double rc = scale2(nd.radius[v], -1);
                const double x = __dadd_rn(nd.cx[v], (o & 1) ? rc : -rc);
                const double y = __dadd_rn(nd.cy[v], (o & 2) ? rc : -rc);
                const double z = __dadd_rn(nd.cz[v], (o & 4) ? rc : -rc);
                nd.cx[c] = x;
                nd.cy[c] = y;
                nd.cz[c] = z;
            }
            __syncwarp();
            if (nn) deepest = max(deepest, level + 1);
            cur = nxt;
            nf = nn;
            level++;
        }
    }
    for (int k = ipool + lane; k < ipool_end; k += 32) nd.lint[k] = make_int2(-1, 0);
    if (lane == 0) {
        if (splits) atomicAdd((unsigned long long *)&ctl->local_splits, (unsigned long long)splits);
        if (deepest) atomicMax(&ctl->maxlev, deepest);
    }
}

// count, min and max mass of each instance's gas particles (order-preserving
// integer atomics)
constexpr int kGasPer = 16;  // particles per thread of k_gas_stats

__global__ void __launch_bounds__(kBlock) k_gas_stats(int n, const double *m, const uint8_t *type,
                                                      const int32_t *pinst, int32_t *cnt, long long *kmin,
                                                      long long *kmax)
{
    // a block takes kBlock * kGasPer consecutive slots, which an instance's
    // contiguous slot range nearly always covers alone: then the block sends
    // one update per statistic, not one per warp to the same three words
    __shared__ int32_t s_kmin, s_kmax, s_c;
    __shared__ long long s_lo, s_hi;
    if (threadIdx.x == 0) {
        s_kmin = INT32_MAX;
        s_kmax = -1;
        s_c = 0;
        s_lo = LLONG_MAX;
        s_hi = LLONG_MIN;
    }
    __syncthreads();
    int k0 = -1, c = 0;
    long long lo = LLONG_MAX, hi = LLONG_MIN;
    const int64_t base = (int64_t)blockIdx.x * blockDim.x * kGasPer;
    for (int r = 0; r < kGasPer; r++) {
        const int64_t i = base + (int64_t)r * blockDim.x + threadIdx.x;
        if (i >= n || type[i] != 2) continue;
        const int k = pinst[i];
        if (k != k0) {  // the thread's slots enter another instance: send the last one's now
            if (k0 >= 0) {
                atomicMin(&kmin[k0], lo);
                atomicMax(&kmax[k0], hi);
                atomicAdd(&cnt[k0], c);
            }
            k0 = k;
            lo = LLONG_MAX;
            hi = LLONG_MIN;
            c = 0;
        }
        const long long key = okey(m[i]);
        lo = key < lo ? key : lo;
        hi = key > hi ? key : hi;
        c++;
    }
    if (k0 >= 0) {
        atomicMin_block(&s_kmin, k0);
        atomicMax_block(&s_kmax, k0);
    }
    __syncthreads();
    if (s_kmin == s_kmax) {  // one instance left in the whole block
        if (k0 >= 0) {
            atomicMin_block(&s_lo, lo);
            atomicMax_block(&s_hi, hi);
            atomicAdd_block(&s_c, c);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicMin(&kmin[s_kmin], s_lo);
            atomicMax(&kmax[s_kmin], s_hi);
            atomicAdd(&cnt[s_kmin], s_c);
        }
    } else if (k0 >= 0) {
        atomicMin(&kmin[k0], lo);
        atomicMax(&kmax[k0], hi);
        atomicAdd(&cnt[k0], c);
    }
}

__global__ void k_gas_stats_init(int n_inst, int32_t *cnt, long long *kmin, long long *kmax)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_inst) return;
    cnt[k] = 0;
    kmin[k] = LLONG_MAX;
    kmax[k] = LLONG_MIN;
}

// gasMass of a node whose gas particles all weigh mg: the reference adds them
// one at a time (Node.cpp:479-480, 681), so its value is the k-th partial sum.
// One thread per instance with a uniform gas mass.
__global__ void k_gas_prefix(int n_inst, const int32_t *cnt, const long long *kmin, const uint8_t *uni,
                             const int32_t *off, double *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_inst || !uni[k]) return;
    const long long key = kmin[k];
    const double mg = __longlong_as_double(key >= 0 ? key : (key ^ 0x7FFFFFFFFFFFFFFFLL));
    double s = 0.0;
    double *t = out + off[k];
    t[0] = 0.0;
    for (int j = 1; j <= cnt[k]; j++) {
        s = __dadd_rn(s, mg);
        t[j] = s;
    }
}

template <class T>
int grow(Ctx *c, T *&p, size_t old_n, size_t new_n)
{
    T *np = nullptr;
    cudaError_t e = cudaMalloc((void **)&np, new_n * sizeof(T));
    if (e != cudaSuccess) return set_err(c, AG2_E_NOMEM, "node pool allocation failed");
    if (p && old_n) {
        AG2_CUDA(c, cudaMemcpyAsync(np, p, old_n * sizeof(T), cudaMemcpyDeviceToDevice, c->stream));
        AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    if (p) cudaFree(p);
    p = np;
    return AG2_OK;
}

}  // namespace

// launches of the internal-moments passes for these per-level counts: one per
// level of more than kFewNodes nodes, one per run of smaller levels
int moments_launches(const int32_t *lvl_cnt)
{
    int k = 0;
    for (int L = AG2_MAX_DEPTH - 1; L >= 0; L--) {
        if (!lvl_cnt[L]) continue;
        k++;
        if (lvl_cnt[L] <= kFewNodes)
            while (L > 0 && lvl_cnt[L - 1] <= kFewNodes) L--;
    }
    return k;
}

int ensure_node_capacity(Ctx *c, size_t need)
{
    if (need <= c->node_cap) return AG2_OK;
    size_t old = c->node_cap;
    size_t nc = std::max(need + need / 4 + 1024, (size_t)1024);
    nc = (nc + 3) & ~(size_t)3;  // byte flags are updated as 32-bit words
    Nodes &d = c->nd;
    int rc = AG2_OK;
#define G(x) \
    if ((rc = grow(c, d.x, old, nc)) != AG2_OK) return rc;
    G(start) G(count) G(ndrop) G(first) G(parent) G(leafpos) G(level) G(mode) G(needs)
    G(cx) G(cy) G(cz) G(radius) G(inst) G(mom)
    G(tsum) G(wrec) G(flag)
    G(rho) G(nlx) G(lint) G(lil)
#undef G
    if ((rc = grow(c, d.bkey, 9 * old, 9 * nc)) != AG2_OK) return rc;
    c->node_cap = nc;
    return AG2_OK;
}

static int ensure_hist(Ctx *c, size_t nodes_in_level)
{
    size_t need = 9 * nodes_in_level;
    if (need <= c->hist_cap) return AG2_OK;
    size_t nc = std::max(need * 2, (size_t)4096);
    if (c->hist) cudaFree(c->hist);
    if (c->cursor) cudaFree(c->cursor);
    c->hist = c->cursor = nullptr;
    if (cudaMalloc(&c->hist, nc * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&c->cursor, nc * sizeof(int32_t)) != cudaSuccess)
        return set_err(c, AG2_E_NOMEM, "histogram allocation failed");
    c->hist_cap = nc;
    // k_nodes leaves every entry it used zero again, so the histogram is zeroed only here
    AG2_CUDA(c, cudaMemsetAsync(c->hist, 0, nc * sizeof(int32_t), c->stream));
    return AG2_OK;
}

// Gas statistics depend only on masses, types and instances, so they are
// refreshed when those change (upload, ag2_set_field of the mass,
// ag2_set_instances), not every build.  gas_stats_begin computes them on the
// device and queues their copy into pinned memory without waiting;
// gas_stats_finish reads them after a later synchronisation of the stream and
// rebuilds the gasMass tables only when they changed.  So an upload of the
// same particles costs the build no extra round trip to the host.
static int gas_stats_begin(Ctx *c, int n)
{
    if (!c->gas_stats_dirty) return AG2_OK;
    const int K = c->n_inst;
    if ((size_t)K > c->gas_pin_cap) {
        if (c->gas_pin) cudaFreeHost(c->gas_pin);
        c->gas_pin = nullptr;
        c->gas_pin_cap = 0;
        AG2_CUDA(c, cudaMallocHost(&c->gas_pin, (size_t)K * 20));
        c->gas_pin_cap = K;
    }
    Particles &S = c->S();
    AG2_LAUNCH(c, k_gas_stats_init, grid_for(K, kBlock), kBlock, 0, K, c->gas_cnt, c->gas_kmin, c->gas_kmax);
    AG2_LAUNCH(c, k_gas_stats, grid_for(n, kBlock * kGasPer), kBlock, 0, n, S.m, S.type, c->pinst, c->gas_cnt,
               c->gas_kmin, c->gas_kmax);
    // pinned layout: kmin (K x 8 B), kmax (K x 8 B), count (K x 4 B)
    unsigned char *pin = static_cast<unsigned char *>(c->gas_pin);
    AG2_CUDA(c, cudaMemcpyAsync(pin, c->gas_kmin, K * 8, cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(pin + 8 * (size_t)K, c->gas_kmax, K * 8, cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(pin + 16 * (size_t)K, c->gas_cnt, K * 4, cudaMemcpyDeviceToHost, c->stream));
    c->gas_pending = true;
    return AG2_OK;
}

// after a synchronisation of the stream that followed gas_stats_begin
static int gas_stats_finish(Ctx *c)
{
    if (!c->gas_pending) return AG2_OK;
    c->gas_pending = false;
    const int K = c->n_inst;
    const unsigned char *pin = static_cast<const unsigned char *>(c->gas_pin);
    std::vector<long long> lo(K), hi(K);
    std::vector<int32_t> cnt(K);
    std::memcpy(lo.data(), pin, K * 8);
    std::memcpy(hi.data(), pin + 8 * (size_t)K, K * 8);
    std::memcpy(cnt.data(), pin + 16 * (size_t)K, K * 4);
    std::vector<int32_t> off(K);
    std::vector<uint8_t> uni(K);
    size_t total = 0;
    c->ngas = 0;
    for (int k = 0; k < K; k++) {
        off[k] = (int32_t)total;
        uni[k] = cnt[k] > 0 && lo[k] == hi[k];
        total += (size_t)cnt[k] + 1;
        c->ngas += cnt[k];
    }
    // the tables are sequential partial sums k * m_gas (one thread per instance):
    // an upload that keeps every instance's gas count and mass keeps them
    if (cnt == c->gas_tab_cnt && lo == c->gas_tab_lo && hi == c->gas_tab_hi && total <= c->gas_prefix_cap) {
        c->gas_stats_dirty = false;
        return AG2_OK;
    }
    if (total > c->gas_prefix_cap) {
        if (c->gas_prefix) cudaFree(c->gas_prefix);
        c->gas_prefix = nullptr;
        if (cudaMalloc(&c->gas_prefix, total * sizeof(double)) != cudaSuccess)
            return set_err(c, AG2_E_NOMEM, "gas table allocation failed");
        c->gas_prefix_cap = total;
    }
    AG2_CUDA(c, cudaMemcpyAsync(c->gas_off, off.data(), K * 4, cudaMemcpyHostToDevice, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(c->gas_uni, uni.data(), K, cudaMemcpyHostToDevice, c->stream));
    AG2_LAUNCH(c, k_gas_prefix, grid_for(K, kBlock), kBlock, 0, K, c->gas_cnt, c->gas_kmin, c->gas_uni, c->gas_off,
               c->gas_prefix);
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));  // host vectors above go out of scope
    c->gas_tab_cnt = cnt;
    c->gas_tab_lo = lo;
    c->gas_tab_hi = hi;
    c->gas_stats_dirty = false;
    return AG2_OK;
}

// both at once (before a captured build, which reads the tables inside the graph)
static int prepare_gas_tables(Ctx *c, int n)
{
    int rc = gas_stats_begin(c, n);
    if (rc || !c->gas_pending) return rc;
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    return gas_stats_finish(c);
}

// buffers of a level: w = level & 1 selects the current half of each pair
static LevelBufs level_bufs(Ctx *c, int w)
{
    int32_t *perm[2] = {c->perm, c->perm2};
    int32_t *pos[2] = {c->posnode, c->posnode2};
    const size_t cap = c->cap;
    int64_t *key = c->pkey;  // [buffer][coordinate][cap]
    LevelBufs b;
    b.ap = c->ap[w];
    b.ap_next = c->ap[w ^ 1];
    b.posnode = pos[w];
    b.posnode_next = pos[w ^ 1];
    b.perm = perm[w];
    b.perm_next = perm[w ^ 1];
    b.kx = key + (3 * w + 0) * cap;
    b.ky = key + (3 * w + 1) * cap;
    b.kz = key + (3 * w + 2) * cap;
    b.kx_next = key + (3 * (w ^ 1) + 0) * cap;
    b.ky_next = key + (3 * (w ^ 1) + 1) * cap;
    b.kz_next = key + (3 * (w ^ 1) + 2) * cap;
    b.perm_final = c->perm_final;
    b.pnode = c->pnode;
    b.digit = c->digit + (size_t)w * cap;
    b.digit_next = c->digit + (size_t)(w ^ 1) * cap;
    b.hist = c->hist;
    b.cursor = c->cursor;
    b.nl = c->nl[w];
    b.nl_next = c->nl[w ^ 1];
    b.drop_list = c->drop_list;
    b.lroots = c->lroots;
    b.local_ok = false;
    return b;
}

// Launch configuration of k_local for split threshold `thresh` (persistent
// grid: every resident block, each warp looping over subtree roots).
struct LocalConfig {
    int lcap = 0, wpb = 0, blocks = 0;
    size_t smem = 0;
};
static int local_config(Ctx *c, int thresh, LocalConfig &lc)
{
    lc.lcap = std::max(8, ((thresh - 1) + 7) & ~7);
    // kLocalBlocks blocks per SM when the subtrees are small enough (224 KB of
    // shared memory per SM), else fewer, larger ones
    lc.wpb = (int)std::max<size_t>(1, std::min<size_t>(kLocalWarps, (56u << 10) / local_smem_bytes(lc.lcap)));
    lc.smem = (size_t)lc.wpb * local_smem_bytes(lc.lcap);
    AG2_CUDA(c, cudaFuncSetAttribute(k_local, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lc.smem));
    int per_sm = 0;
    AG2_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_local, lc.wpb * 32, lc.smem));
    lc.blocks = std::max(per_sm, 1) * c->sms;
    return AG2_OK;
}

static int build_error(Ctx *c, int code)
{
    c->hist_dirty = true;
    if (code == AG2_E_COINCIDENT)
        return set_err(c, AG2_E_COINCIDENT,
                       "particles too close to separate within AG2_MAX_DEPTH levels "
                       "(the reference recurses without end on coincident particles)");
    if (code == AG2_E_CAPACITY) return set_err(c, AG2_E_CAPACITY, "more than 65536 nodes with out-of-bounds particles");
    return set_err(c, code, "octree build failed");
}

// Run `body` (launches on c->stream) as the body of a WHILE node of the graph
// being captured on c->stream; `h` is the node's condition.
template <class F>
static int capture_while(Ctx *c, cudaGraphConditionalHandle h, F body)
{
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edata = nullptr;
    size_t nd = 0;
    AG2_CUDA(c, cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, &edata, &nd));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    AG2_CUDA(c, cudaGraphAddNode(&node, g, deps, edata, nd, &p));
    AG2_CUDA(c, cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t bodyg = p.conditional.phGraph_out[0];
    cudaStream_t outer = c->stream;
    c->stream = c->side_stream;
    cudaError_t e = cudaStreamBeginCaptureToGraph(c->stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    int rc = e == cudaSuccess ? body() : cuda_check(c, e, "cudaStreamBeginCaptureToGraph");
    cudaGraph_t out = nullptr;
    e = cudaStreamEndCapture(c->stream, &out);
    c->stream = outer;
    if (rc) return rc;
    return e == cudaSuccess ? AG2_OK : cuda_check(c, e, "cudaStreamEndCapture");
}

static int build_tree_once(Ctx *c, bool &local_nomem, bool capture);

// The pool is sized before each level of the loop; serial subtrees may still
// need more nodes than estimated, in which case the build is redone with a
// larger pool (the particle state is untouched until the reorder).
int build_tree(Ctx *c)
{
    for (int attempt = 0;; attempt++) {
        bool local_nomem = false;
        const int rc = build_tree_once(c, local_nomem, false);
        if (rc == AG2_E_NOMEM && local_nomem && attempt < 4) {
            c->err.clear();
            const int g = ensure_node_capacity(c, 2 * c->node_cap);
            if (g != AG2_OK) return g;
            continue;
        }
        return rc;
    }
}

// The build inside a captured step: every count stays on the device (fixed
// grids, the level loop and the moments levels as WHILE nodes).  The caller
// has prepared the tables and sized the pools.
int build_tree_captured(Ctx *c)
{
    bool unused = false;
    return build_tree_once(c, unused, true);
}

// Host-side view of the tree after a captured step (from the control block).
void build_tree_finish_captured(Ctx *c)
{
    const Ctx::Ctl &h = *c->ctl_host;
    c->max_level = std::max((int)h.level, (int)h.maxlev);
    c->nnodes = h.node_count;
    c->nnodes_true = h.loop_nodes - (first_pool_node(c->n_inst) - c->n_inst) + 8 * (int64_t)h.local_splits;
    c->ninternal = (c->nnodes_true - c->n_inst) / 8;
    c->root_radius = c->inst_R_pin ? c->inst_R_pin[0] : 0.0;
    c->inst_R_h.assign(c->inst_R_pin, c->inst_R_pin + c->n_inst);
    c->have_tree = true;
    c->tree_theta = c->prm.theta;
}

// Sizes a captured build needs fixed in advance: histogram of a split list as
// long as the particle count, and a node pool with room to grow.
int prepare_captured_build(Ctx *c)
{
    int rc;
    if ((rc = ensure_instance_tables(c)) != AG2_OK) return rc;
    if ((rc = prepare_gas_tables(c, (int)c->n)) != AG2_OK) return rc;
    if ((rc = ensure_hist(c, std::max<size_t>(c->n, 1))) != AG2_OK) return rc;
    LocalConfig lc;
    if ((rc = local_config(c, c->prm.split_threshold, lc)) != AG2_OK) return rc;
    c->loc_lcap = lc.lcap;
    c->loc_wpb = lc.wpb;
    c->loc_blocks = lc.blocks;
    c->loc_smem = lc.smem;
    const size_t want = (size_t)(2 * std::max<int64_t>(c->nnodes, 4 * (int64_t)c->n)) +
                        (size_t)lc.blocks * lc.wpb * kPoolChunk + 1024;
    if ((rc = ensure_node_capacity(c, want)) != AG2_OK) return rc;
    if (c->hist_dirty) {
        AG2_CUDA(c, cudaMemsetAsync(c->hist, 0, c->hist_cap * sizeof(int32_t), c->stream));
        c->hist_dirty = false;
    }
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    return AG2_OK;
}

static int build_tree_once(Ctx *c, bool &local_nomem, bool capture)
{
    const int n = (int)c->n;
    c->have_tree = false;
    int rc;
    if (!capture) {
        if ((rc = ensure_instance_tables(c)) != AG2_OK) return rc;
        if ((rc = gas_stats_begin(c, n)) != AG2_OK) return rc;  // read at the first synchronisation below
        // the histogram holds a level's split list (at most n/2 nodes plus the roots);
        // it is sized before the level loop, which fills the next level's while it
        // consumes this one's
        if ((rc = ensure_hist(c, std::max<size_t>(c->n, 1))) != AG2_OK) return rc;
        if (c->hist_dirty) {
            AG2_CUDA(c, cudaMemsetAsync(c->hist, 0, c->hist_cap * sizeof(int32_t), c->stream));
            c->hist_dirty = false;
        }
    }
    const int K = c->n_inst;
    Particles &S = c->S();
    const unsigned fixed_grid = (unsigned)c->sms * 8;  // grid-stride launches of a captured build

    // root half-width of every instance
    AG2_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(Ctx::Ctl), c->stream));
    if (n > 0) {
        AG2_LAUNCH(c, k_slot_of, grid_for(n, kBlock), kBlock, 0, n, S.id, c->slot_of);
        AG2_LAUNCH(c, k_dist, grid_for(n, kBlock), kBlock, 0, n, S.px, S.py, S.pz, c->rdist);
        for (size_t l = 0; l + 1 < c->wsum_level.size(); l++) {
            const int nt = c->wsum_level[l + 1] - c->wsum_level[l];
            const int4 *tk = c->wsum_task + c->wsum_level[l];
            if (l == 0) {
                AG2_LAUNCH(c, k_wsum_particles, grid_for(nt, kBlock), kBlock, 0, nt, tk, c->rdist, c->slot_of,
                           c->width_part);
                // one task (its two warps) per block, so that the tasks spread
                // over the SMs and no two chains share a partition's FP64 pipe
                if (c->nwsum_long > 0)
                    AG2_LAUNCH(c, k_wsum_long, (unsigned)c->nwsum_long, 64, 0, c->nwsum_long, c->wsum_long, tk,
                               c->rdist, c->slot_of, c->width_part);
            } else
                AG2_LAUNCH(c, k_wsum_sums, grid_for(nt, kBlock), kBlock, 0, nt, tk, c->width_part);
        }
    }
    AG2_LAUNCH(c, k_width_thr, grid_for(K, kBlock), kBlock, 0, K, c->inst_first, c->wsum_final, c->width_part,
               c->width_thr, c->inst_R);
    if (n > 0)
        AG2_LAUNCH(c, k_width_max, grid_for(n, kBlock), kBlock, 0, n, c->rdist, c->pinst, c->width_thr, c->inst_R);
    phase_mark(c, "build: root width");
    if (!capture && (rc = ensure_node_capacity(c, (size_t)K + 1024)) != AG2_OK) return rc;
    const int thresh = c->prm.split_threshold;
    // serial subtrees (fewer than split_threshold particles) are built one warp each when they fit
    const bool local_ok = thresh - 1 <= kLocalCapMax;
    AG2_LAUNCH(c, k_root_init, grid_for(K, kBlock), kBlock, 0, K, c->nd, c->ctl, c->inst_first, c->inst_R, thresh,
               c->nl[0], local_ok, c->lroots);
    AG2_LAUNCH(c, k_level0, grid_for(n, kBlock), kBlock, 0, n, c->pinst, c->nd, S.px, S.py, S.pz, level_bufs(c, 0),
               c->ctl);
    LevelPair lpair;
    lpair.b[0] = level_bufs(c, 0);
    lpair.b[1] = level_bufs(c, 1);
    lpair.b[0].local_ok = lpair.b[1].local_ok = local_ok;

    // the level loop
    c->level_base.assign({0, (int64_t)K});
    if (capture) {
        cudaStreamCaptureStatus st;
        cudaGraph_t g = nullptr;
        AG2_CUDA(c, cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g));
        cudaGraphConditionalHandle h;
        AG2_CUDA(c, cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
        AG2_LAUNCH(c, k_level_next, 1, 32, 0, c->ctl, 0, (int)AG2_MAX_DEPTH, h, 1);
        rc = capture_while(c, h, [&]() -> int {
            AG2_LAUNCH(c, k_nodes, fixed_grid, kBlock, 0, lpair, thresh, (int64_t)c->node_cap, c->nd, c->ctl,
                       (int)AG2_MAX_DEPTH);
            AG2_LAUNCH(c, k_scatter, fixed_grid, kBlock, 0, lpair, c->nd, c->ctl, 0);
            AG2_LAUNCH(c, k_level_next, 1, 32, 0, c->ctl, 1, (int)AG2_MAX_DEPTH, h, 1);
            return AG2_OK;
        });
        if (rc) return rc;
        AG2_LAUNCH(c, k_mark_loop_nodes, 1, 32, 0, c->ctl);
    } else {
        cudaGraphConditionalHandle none = 0;
        AG2_LAUNCH(c, k_level_next, 1, 32, 0, c->ctl, 0, (int)AG2_MAX_DEPTH, none, 0);
        // The levels run one ahead of the host: level k + 1 is queued before
        // the host waits for level k's counts (a snapshot of the control block
        // copied behind it), so the device does not idle between levels.  A
        // level queued past the last one finds no split node and changes
        // nothing.  Kernels take their counts from the control block (grid-
        // stride launches of a fixed grid, as in a captured build).  The first
        // levels are queued on bounds (at most one split per root, at most n
        // active slots), so the host does not wait for the root half-widths.
        if (!c->ctl_snap) {
            AG2_CUDA(c, cudaMallocHost(&c->ctl_snap, 2 * sizeof(Ctx::Ctl)));
            for (auto &e : c->snap_ev) AG2_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        // the root half-widths come back with the first snapshot
        if (c->inst_R_rb_cap < (size_t)K) {
            if (c->inst_R_rb) cudaFreeHost(c->inst_R_rb);
            c->inst_R_rb = nullptr;
            c->inst_R_rb_cap = 0;
            AG2_CUDA(c, cudaMallocHost(&c->inst_R_rb, K * sizeof(double)));
            c->inst_R_rb_cap = K;
        }
        AG2_CUDA(c, cudaMemcpyAsync(c->inst_R_rb, c->inst_R, K * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        int64_t known_nodes = first_pool_node(K);  // nodes after the last level read back
        int64_t nnl = K;          // split nodes of the level after it (a bound until the first read)
        int64_t nap = n;          // and its active slots (likewise)
        int queued = 0, seen = 0;
        bool more = n > 0;
        while (more) {
            // pool room for the levels in flight: the one read back next
            // allocates 8 * nnl children; of those, the ones the level queued
            // now splits are at most 8 * nnl, and each holds two or more of
            // the nap active particles
            const int64_t next_split = std::min<int64_t>(8 * nnl, nap / 2);
            if ((rc = ensure_node_capacity(c, (size_t)(known_nodes + 8 * nnl + 8 * next_split + 8))) != AG2_OK)
                return rc;
            lpair.b[0] = level_bufs(c, 0);
            lpair.b[1] = level_bufs(c, 1);
            lpair.b[0].local_ok = lpair.b[1].local_ok = local_ok;
            AG2_LAUNCH(c, k_nodes, fixed_grid, kBlock, 0, lpair, thresh, (int64_t)c->node_cap, c->nd, c->ctl,
                       (int)AG2_MAX_DEPTH);
            AG2_LAUNCH(c, k_scatter, fixed_grid, kBlock, 0, lpair, c->nd, c->ctl, 1);  // and advances the level
            const int slot = queued & 1;
            AG2_CUDA(c, cudaMemcpyAsync(c->ctl_snap + slot, c->ctl, sizeof(Ctx::Ctl), cudaMemcpyDeviceToHost,
                                        c->stream));
            AG2_CUDA(c, cudaEventRecord(c->snap_ev[slot], c->stream));
            queued++;
            if (queued - seen < 2) continue;  // keep one level queued ahead
            AG2_CUDA(c, cudaEventSynchronize(c->snap_ev[seen & 1]));
            const Ctx::Ctl &h = c->ctl_snap[seen & 1];
            seen++;
            if (h.err_code) {
                if ((rc = sync_ctl(c)) != AG2_OK) return rc;
                if (c->ctl_host->err_code == AG2_E_NOMEM) local_nomem = true;  // grow the pool and build again
                return build_error(c, c->ctl_host->err_code);
            }
            if (h.level + 2 > (int)c->level_base.size()) c->level_base.push_back(h.node_count);  // a new level
            known_nodes = h.node_count;
            nnl = h.cur_nnl;
            nap = h.cur_nap;
            more = nnl > 0;
        }
        // the host mirror after the loop (the serial subtrees' launch reads its
        // counts) is the last snapshot read: the level queued past the last
        // one leaves the block unchanged.  Waiting on a snapshot also waited
        // for the root half-widths' and the gas statistics' read-backs queued
        // before the loop.
        if (seen > 0) {
            std::memcpy(c->ctl_host, c->ctl_snap + ((seen - 1) & 1), sizeof(Ctx::Ctl));
        } else if ((rc = sync_ctl(c)) != AG2_OK) {
            return rc;
        }
        if (c->ctl_host->err_code) return build_error(c, c->ctl_host->err_code);
        c->inst_R_h.assign(c->inst_R_rb, c->inst_R_rb + K);
        c->root_radius = c->inst_R_h[0];
        if ((rc = gas_stats_finish(c)) != AG2_OK) return rc;
    }
    phase_mark(c, "build: levels");

    // serial subtrees: one warp each
    LocalConfig lc;
    if (capture) {
        lc.lcap = c->loc_lcap;  // set up before the capture (no runtime calls inside it)
        lc.wpb = c->loc_wpb;
        lc.blocks = c->loc_blocks;
        lc.smem = c->loc_smem;
        AG2_LAUNCH(c, k_local, lc.blocks, lc.wpb * 32, lc.smem, c->lroots, lc.lcap, c->nd, c->ctl, c->pkey,
                   (int64_t)c->cap, c->perm_final, c->pnode, S.id,
                   (int)AG2_MAX_DEPTH, (int64_t)c->node_cap);
        AG2_LAUNCH(c, k_sort_drops, fixed_grid, kBlock, 0, c->ctl, c->drop_list, c->nd, c->perm_final, S.id, c->perm2);
    } else {
        const int nloc = c->ctl_host->nlocal;
        const int64_t loop_nodes = c->ctl_host->node_count;
        if (nloc > 0) {
            if ((rc = local_config(c, thresh, lc)) != AG2_OK) return rc;
            const int blocks = std::max(1, std::min((nloc + lc.wpb - 1) / lc.wpb, lc.blocks));
            const size_t need = (size_t)loop_nodes + 12 * (size_t)c->ctl_host->nlocal_part +
                                (size_t)blocks * lc.wpb * kPoolChunk + 1024;
            if ((rc = ensure_node_capacity(c, need)) != AG2_OK) return rc;
            AG2_LAUNCH(c, k_local, blocks, lc.wpb * 32, lc.smem, c->lroots, lc.lcap, c->nd, c->ctl, c->pkey,
                       (int64_t)c->cap, c->perm_final, c->pnode, S.id,
                       (int)AG2_MAX_DEPTH, (int64_t)c->node_cap);
        }
        // the internal-node list by level (these read the list within its
        // capacity, so they are safe after a failed k_local), then one
        // synchronisation for the serial subtrees' counts and errors and the
        // levels' sizes
        {
            cudaGraphConditionalHandle none = 0;
            AG2_LAUNCH(c, k_lvl_hist, fixed_grid, kBlock, 0, c->ctl, c->nd.lint, (int64_t)c->node_cap);
            AG2_LAUNCH(c, k_lvl_prefix, 1, 32, 0, c->ctl, none, 0);
            AG2_LAUNCH(c, k_bucket, fixed_grid, kBlock, 0, c->ctl, c->nd.lint, c->nd.lil, (int64_t)c->node_cap);
        }
        if ((rc = sync_ctl(c)) != AG2_OK) return rc;
        if (c->ctl_host->err_code) {
            if (c->ctl_host->err_code == AG2_E_NOMEM) local_nomem = true;
            return build_error(c, c->ctl_host->err_code);
        }
        if (nloc > 0) phase_mark(c, "build: serial subtrees");
        c->max_level = std::max((int)c->level_base.size() - 2, (int)c->ctl_host->maxlev);
        c->nnodes = c->ctl_host->node_count;
        c->nnodes_true = loop_nodes - (first_pool_node(K) - K) + 8 * (int64_t)c->ctl_host->local_splits;
        c->ninternal = (c->nnodes_true - K) / 8;
        if (c->ctl_host->ndrop_nodes > kMaxDropNodes) return build_error(c, AG2_E_CAPACITY);
        if (c->ctl_host->ndrop_nodes > 0)
            AG2_LAUNCH(c, k_sort_drops, (unsigned)c->ctl_host->ndrop_nodes, kBlock, 0, c->ctl, c->drop_list, c->nd,
                       c->perm_final, S.id, c->perm2);
    }

    // particle state into tree order
    Particles &src = c->st[c->cur];
    Particles &dst = c->st[c->cur ^ 1];
    AG2_LAUNCH(c, k_reorder, grid_for(n, kBlock), kBlock, 0, n, c->perm_final, src, dst);
    c->cur ^= 1;
    c->upload_order = false;  // tree order, within each instance's slot range
    c->perm_first = c->inst_first_h;
    AG2_LAUNCH(c, k_refnode, grid_for(n, kBlock), kBlock, 0, n, c->nd, c->pnode, c->S().id, c->refnode);
    phase_mark(c, "build: reorder");

    // moments: every leaf at once, then the internal nodes level by level,
    // deepest first (the internal-node list bucketed by level)
    const unsigned gl = capture ? fixed_grid : std::max(1u, grid_for(n, kBlock));
    AG2_LAUNCH(c, k_moments_leaf, gl, kBlock, 0, n, c->pnode, c->nd, c->S(), c->gas_prefix, c->gas_off,
               c->gas_uni, RecArgs{(float)c->prm.theta, c->inst_R});
    phase_mark(c, "build: leaf moments");
    if (capture) {
        AG2_LAUNCH(c, k_lvl_hist, fixed_grid, kBlock, 0, c->ctl, c->nd.lint, (int64_t)c->node_cap);
        cudaStreamCaptureStatus st;
        cudaGraph_t g = nullptr;
        AG2_CUDA(c, cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g));
        cudaGraphConditionalHandle h;
        AG2_CUDA(c, cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
        AG2_LAUNCH(c, k_lvl_prefix, 1, 32, 0, c->ctl, h, 1);
        AG2_LAUNCH(c, k_bucket, fixed_grid, kBlock, 0, c->ctl, c->nd.lint, c->nd.lil, (int64_t)c->node_cap);
        rc = capture_while(c, h, [&]() -> int {
            AG2_LAUNCH(c, k_moments_int<true>, fixed_grid, kBlock, 0, 0, c->nd.lil, c->ctl, c->nd, c->S(),
                       c->gas_prefix, c->gas_off, c->gas_uni, RecArgs{(float)c->prm.theta, c->inst_R});
            AG2_LAUNCH(c, k_mlev_next, 1, 32, 0, c->ctl, h, 1);
            return AG2_OK;
        });
        if (rc) return rc;
    } else {
        // the levels' sizes came back with the serial subtrees' synchronisation
        c->lvl_cnt_h.assign(c->ctl_host->lvl_cnt, c->ctl_host->lvl_cnt + AG2_MAX_DEPTH);
        c->lvl_start_h.assign(c->ctl_host->lvl_start, c->ctl_host->lvl_start + AG2_MAX_DEPTH);
        for (int L = AG2_MAX_DEPTH - 1; L >= 0; L--) {
            const int32_t cnt = c->lvl_cnt_h[L];
            if (!cnt) continue;
            const RecArgs ra{(float)c->prm.theta, c->inst_R};
            if (cnt <= kFewNodes) {  // this level and the small ones above it: one block
                int lo = L;
                while (lo > 0 && c->lvl_cnt_h[lo - 1] <= kFewNodes) lo--;
                AG2_LAUNCH(c, k_moments_few, 1, kBlock, 0, L, lo, c->nd.lil, c->ctl, c->nd, c->S(), c->gas_prefix,
                           c->gas_off, c->gas_uni, ra);
                L = lo;
                continue;
            }
            AG2_LAUNCH(c, k_moments_int<false>, grid_for(cnt, kBlock), kBlock, 0, cnt, c->nd.lil + c->lvl_start_h[L],
                       c->ctl, c->nd, c->S(), c->gas_prefix, c->gas_off, c->gas_uni, ra);
        }
    }
    phase_mark(c, "build: internal moments");
    c->have_tree = true;  // (inside a capture: for the launches that follow it)
    c->tree_theta = c->prm.theta;
    return AG2_OK;
}

}  // namespace ag2
