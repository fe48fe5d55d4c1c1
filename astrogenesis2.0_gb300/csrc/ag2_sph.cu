// ag2_sph.cu -- SPH density and visual density on the device octree.
//
// Reference: simulation/src/Physics/Tree/Tree.cpp:119-150 (calcGasDensity),
// :152-175 (calcVisualDensity); Node.cpp:722-796 (Node::calcGasDensity),
// :832-877 (Node::calcVisualDensity); kernel.cpp:4-16 (cubic spline).
//
// The reference runs a serial loop in particle order: a gas particle whose h is
// still 0 climbs from its leaf while its node holds less than massInH of gas
// and the parent's gas mass is strictly closer to massInH, then (if the stop
// node is strictly closer than its own parent) sets h = 2*radius and one
// node-level density for every gas particle in that node's childParticles.
// Later firings overwrite earlier ones.  Because the stop rule depends only on
// the node, and a node that fired covers every particle inside it, the nodes
// that fire inside a given node always fire before it; so the value a particle
// ends with comes from the outermost valid stop node that contains it.  The
// kernels below compute exactly that without the serial loop:
//   k_climb   every gas leaf particle climbs in parallel and flags its stop node
//   k_final   every gas particle walks up its path and keeps the outermost
//             flagged node whose childParticles hold it
//   k_rho     one warp per selected node sums m W(|x - COM|, 2 r) over the
//             node's childParticles (with the reference's duplicates)
//   k_assign  h, rho, P, T per particle
#include <algorithm>

#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kBlock = 256;

struct TreeView {
    const int32_t *start, *count, *ndrop, *parent, *leafpos, *pnode, *refnode;
    const int8_t *level;
    const uint8_t *mode;
    const NodeMom *mom;
    const double *radius;
    const int32_t *pinst;
};

TreeView view(Ctx *c)
{
    TreeView t;
    t.start = c->nd.start;
    t.count = c->nd.count;
    t.ndrop = c->nd.ndrop;
    t.parent = c->nd.parent;
    t.leafpos = c->nd.leafpos;
    t.pnode = c->pnode;
    t.refnode = c->refnode;
    t.level = c->nd.level;
    t.mode = c->nd.mode;
    t.mom = c->nd.mom;
    t.radius = c->nd.radius;
    t.pinst = c->pinst;
    return t;
}

// Is tree-order slot i in node n's childParticles?  (Node.cpp:515-522 gives a
// non-root list to every node the parallel path creates; serial insertion
// pushes only particles inside the node's bounds, Node.cpp:606-615; the root
// receives no list.)
__device__ __forceinline__ bool cp_member(const TreeView &t, int64_t n, int i)
{
    uint8_t md = t.mode[n];
    int32_t reached_end = t.start[n] + t.count[n] - t.ndrop[n];
    if (t.parent[n] < 0) return md == MODE_SER_ENTRY && i < reached_end;
    if (md == MODE_SER) return i < reached_end;
    return md != MODE_EMPTY;
}

// Every slot: a gas slot is listed for k_final and k_assign, which then run
// over the gas alone (one reservation per block: warps of every block taking
// places on one counter serialise there), and climbs to its density node.
__global__ void __launch_bounds__(kBlock) k_climb(int n, TreeView t, const uint8_t *type,
                                                  const double *inst_massInH, uint8_t *flag, int32_t *gas_slots,
                                                  Ctx::Ctl *ctl)
{
    __shared__ int32_t wcnt[kBlock / 32], bbase;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const bool gas = i < n && type[i] == 2;
    const unsigned gm = __ballot_sync(0xffffffffu, gas);
    if (lane == 0) wcnt[w] = __popc(gm);
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t tot = 0;
        for (int k = 0; k < kBlock / 32; k++) {
            const int32_t c = wcnt[k];
            wcnt[k] = tot;
            tot += c;
        }
        bbase = tot ? atomicAdd(&ctl->ngas_slots, tot) : 0;
    }
    __syncthreads();
    if (!gas) return;
    gas_slots[bbase + wcnt[w] + __popc(gm & ((1u << lane) - 1u))] = i;
    const double M = inst_massInH[t.pinst[i]];
    int pn = t.refnode[i];
    if (pn < 0) return;  // Particle::node is null
    int64_t nd = pn;
    for (;;) {
        double g = t.mom[nd].gas;
        if (g == 0) return;
        int32_t par = t.parent[nd];
        if (par < 0) return;
        double md = M - g, pmd = M - t.mom[par].gas;
        if (g < M && fabs(md) > fabs(pmd)) {
            nd = par;
            continue;
        }
        if (fabs(md) < fabs(pmd) && g != 0) flag[nd] = 1;
        return;
    }
}

// the gas slots k_climb listed
__global__ void k_final(const int32_t *gas_slots, TreeView t, uint8_t *flag, int32_t *finalnode, int32_t *list,
                        Ctx::Ctl *ctl)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ctl->ngas_slots) return;
    const int i = gas_slots[k];
    int64_t nd = t.pnode[i];
    int32_t fin = -1;
    while (nd >= 0) {
        if ((flag[nd] & 1) && cp_member(t, nd, i)) fin = (int32_t)nd;
        nd = t.parent[nd];
    }
    finalnode[i] = fin;
    if (fin >= 0) {
        unsigned int *w = (unsigned int *)(flag + (fin & ~3));
        unsigned int bit = 2u << (8 * (fin & 3));
        unsigned int old = atomicOr(w, bit);
        if (!(old & bit)) list[atomicAdd(&ctl->list_count, 1)] = fin;
    }
}

// kRhoWarps warps per selected node, one block, each warp taking every
// kRhoWarps-th stretch of 32 slots of the node's range: a few thousand nodes
// with ~1000 slots each give a warp per node too little to wait on its loads
// with.  The warps' sums are added in warp order, so the result is the same
// on every run.  Each warp gathers its gas particles 32 at a time into a
// queue (ballot over its stretch), so every FP64 square root and division runs
// on 32 gas lanes rather than on the one or two gas lanes of a mixed stretch
// (FP64 issues at 1/64 of the FP32 rate, whatever the active lanes).  alpha =
// 1 / (pi h^3) is the same for every particle of the node (kernel.cpp:4-16
// computes it per call from the same h).
constexpr int kRhoWarps = 4;

__global__ void __launch_bounds__(32 * kRhoWarps) k_rho(TreeView t, const double *px, const double *py,
                                                        const double *pz, const double *m, const uint8_t *type,
                                                        const int32_t *list, const Ctx::Ctl *ctl, double *rho_node)
{
    __shared__ int32_t queue[kRhoWarps][64];
    __shared__ double part[kRhoWarps];
    const int wi = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int nlist = ctl->list_count;
    int32_t *q = queue[wi];
    const unsigned lt = (1u << lane) - 1u;
    for (int b = blockIdx.x; b < nlist; b += gridDim.x) {  // block-uniform
        const int64_t nd = list[b];
        const double h = t.radius[nd] * 2;  // h = radius * 2 (Node.cpp:765)
        const double alpha = 1.0 / (kPi * h * h * h);
        const double cx = t.mom[nd].cx, cy = t.mom[nd].cy, cz = t.mom[nd].cz;
        const int32_t s = t.start[nd], e = s + t.count[nd], reached_end = e - t.ndrop[nd];
        const uint8_t md = t.mode[nd];
        // the childParticles multiplicity of slot j: the parent's list plus serial
        // insertion for a serial entry node (Node.cpp:518, 615), in-bounds only below it
        auto mult = [&](int32_t j) -> int {
            if (md == MODE_SER_ENTRY) return j < reached_end ? 2 : 1;
            if (md == MODE_SER) return j < reached_end ? 1 : 0;
            return 1;
        };
        double acc = 0.0;
        auto add = [&](int32_t j) {
            const double dx = px[j] - cx, dy = py[j] - cy, dz = pz[j] - cz;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            const double qh = r / h;  // kernel::cubicSplineKernel (kernel.cpp:4-16)
            double W = 0.0;
            if (qh < 1.0) {
                W = alpha * (1 - 1.5 * qh * qh + 0.75 * qh * qh * qh);
            } else if (qh < 2.0) {
                const double u = 2 - qh;
                W = alpha * 0.25 * (u * u * u);
            }
            acc += mult(j) * (m[j] * W);
        };
        int qn = 0;
        for (int32_t j0 = s + 32 * wi; j0 < e; j0 += 32 * kRhoWarps) {
            const int32_t j = j0 + lane;
            const bool g = j < e && type[j] == 2 && mult(j) != 0;
            const unsigned bm = __ballot_sync(0xffffffffu, g);
            if (g) q[qn + __popc(bm & lt)] = j;
            qn += __popc(bm);
            __syncwarp();
            if (qn >= 32) {
                const int32_t jj = q[lane];
                __syncwarp();
                if (lane < qn - 32) q[lane] = q[32 + lane];
                qn -= 32;
                __syncwarp();
                add(jj);
            }
        }
        if (lane < qn) add(q[lane]);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) part[wi] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double r = part[0];
            for (int k = 1; k < kRhoWarps; k++) r += part[k];
            rho_node[nd] = r;
        }
        __syncthreads();  // part and the queues are free for the next node
    }
}

// the gas slots k_climb listed
__global__ void k_assign(const int32_t *gas_slots, const Ctx::Ctl *ctl, TreeView t, const int32_t *finalnode,
                         const double *U, const double *rho_node, double *h, double *rho, double *P, double *T)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ctl->ngas_slots) return;
    const int i = gas_slots[k];
    int32_t f = finalnode[i];
    if (f < 0) {
        h[i] = 0.0;  // Tree.cpp:123-133 resets h; rho, P, T keep their old values
        return;
    }
    h[i] = t.radius[f] * 2;
    double r = rho_node[f];
    rho[i] = r;
    P[i] = (kGamma - 1.0) * U[i] * r;                           // Node.cpp:789
    T[i] = (kGamma - 1.0) * U[i] * kProton * 0.58 / kBoltzmann;  // Node.cpp:791, mu = 0.58
}

// ---- visual density --------------------------------------------------------

__global__ void k_vclimb(int n, TreeView t, double Rv, uint8_t *flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int pn = t.refnode[i];
    if (pn < 0) return;
    int64_t nd = pn;
    for (;;) {
        int32_t par = t.parent[nd];
        if (par < 0) return;
        double r = t.radius[nd];
        double rp = t.radius[par];
        if (fabs(Rv - r) > fabs(Rv - rp)) {
            nd = par;
            continue;
        }
        double vol = r * r * r;
        double mass = t.mom[nd].mass;
        if (vol == 0 || mass == 0) return;
        double dens = mass / vol;
        if (dens == 0 || isinf(dens)) return;
        flag[nd] = 1;
        return;
    }
}

__global__ void k_vfinal(int n, TreeView t, const uint8_t *flag, double *vdens)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t nd = t.pnode[i];
    double v = 0.0;
    while (nd >= 0) {
        if (flag[nd] && cp_member(t, nd, i)) {
            double r = t.radius[nd];
            v = t.mom[nd].mass / (r * r * r);
        }
        nd = t.parent[nd];
    }
    vdens[i] = v;
}

}  // namespace

int run_sph_density(Ctx *c)
{
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "ag2_sph_density needs a tree (call ag2_build_tree)");
    const int n = (int)c->n;
    if (n == 0 || c->ngas == 0) return AG2_OK;
    Particles &S = c->S();
    TreeView t = view(c);
    AG2_CUDA(c, cudaMemsetAsync(c->nd.flag, 0, std::min(((size_t)c->nnodes + 3) & ~(size_t)3, c->node_cap), c->stream));
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->list_count, 0, sizeof(int32_t), c->stream));
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->ngas_slots, 0, sizeof(int32_t), c->stream));
    if (c->n_inst == 1 && !c->inst_explicit && !c->capturing)  // a single simulation follows ag2_set_params
        AG2_CUDA(c, cudaMemcpyAsync(c->inst_massInH, &c->prm.massInH, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    const int ngas = c->ngas;  // the gas slots k_climb lists
    AG2_LAUNCH(c, k_climb, grid_for(n, kBlock), kBlock, 0, n, t, S.type, c->inst_massInH, c->nd.flag, c->gas_slots,
               c->ctl);
    AG2_LAUNCH(c, k_final, grid_for(ngas, kBlock), kBlock, 0, c->gas_slots, t, c->nd.flag, c->finalnode, c->nodelist,
               c->ctl);
    // one block per selected node (at most one per gas particle), striding over the list
    const unsigned rho_blocks = (unsigned)std::max<size_t>(1, std::min<size_t>((size_t)ngas, (size_t)c->sms * 16));
    AG2_LAUNCH(c, k_rho, rho_blocks, 32 * kRhoWarps, 0, t, S.px, S.py, S.pz, S.m, S.type, c->nodelist, c->ctl,
               c->nd.rho);
    AG2_LAUNCH(c, k_assign, grid_for(ngas, kBlock), kBlock, 0, c->gas_slots, c->ctl, t, c->finalnode, S.U,
               c->nd.rho, S.h, S.rho, S.P, S.T);
    return AG2_OK;
}

int run_visual_density(Ctx *c, double Rv)
{
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "ag2_visual_density needs a tree (call ag2_build_tree)");
    const int n = (int)c->n;
    if (n == 0) return AG2_OK;
    Particles &S = c->S();
    TreeView t = view(c);
    AG2_CUDA(c, cudaMemsetAsync(c->nd.flag, 0, std::min(((size_t)c->nnodes + 3) & ~(size_t)3, c->node_cap), c->stream));
    AG2_LAUNCH(c, k_vclimb, grid_for(n, kBlock), kBlock, 0, n, t, Rv, c->nd.flag);
    AG2_LAUNCH(c, k_vfinal, grid_for(n, kBlock), kBlock, 0, n, t, c->nd.flag, S.vdens);
    return AG2_OK;
}

}  // namespace ag2
