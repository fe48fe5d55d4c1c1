// ag2_walk.cu -- Barnes-Hut walk with softened gravity and in-walk SPH force.
//
// Reference: simulation/src/Physics/Tree/Tree.cpp:57-83 (calculateForces),
// Node.cpp:247-399 (calculateGravityForce), :285-305 (softened pair law),
// :88-172 (calcSPHForce), simulation/src/Math/kernel.cpp (kernels).
//
// One warp walks the tree for a group of 32 consecutive tree-order particles
// (one per lane).  The reference decides per particle: open a node unless
// radius/r < theta, with r the distance to the node's centre of mass.  To keep
// those decisions per particle, every stack entry carries a 32-bit lane mask:
// a node is opened for exactly the lanes whose own test failed, and a lane
// that accepted a node never sees its descendants.  The stack lives in shared
// memory (one slice per warp); node records are broadcast loads (every lane
// reads the same address).  Groups are handed out by an atomic counter so
// dense regions do not stall a fixed partition.
//
// Two arithmetic forms:
//   FP64  -- "plain": everything in double, opening test exactly as the
//            reference writes it (radius / r < theta).
//   FP32  -- positions become float offsets from the group's centre; node
//            centres of mass are stored as hi+lo float pairs, so a nearby node's
//            offset keeps ~48 bits.  Opening tests and forces run in FP32; a
//            test within 1e-5 of the threshold (or a distance that rounds to
//            ~0) is re-decided in FP64 so the accepted node set matches the
//            FP64 walk.  Accelerations are summed per child batch and added to a
//            compensated (Kahan) accumulator.
#include <algorithm>
#include <cstdio>

#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kWalkBlock = 128;  // 4 warps
constexpr int kStack = 512;      // stack entries per warp (FP64 walk, potential, FP32 retry pass)
// The FP32 walk's first pass uses a shallower stack (a variant parameter):
// more blocks fit an SM.  The deepest stack measured on the bench workloads is
// under 50 entries; a group that would overflow leaves its sums, goes to a
// retry list and is walked again by a second launch with the full stack.
constexpr float kGuard = 1e-5f;
// FP32 walk variants the autotuner chooses among: the register budget (through
// the resident 4-warp blocks per SM it is built for; 1 = the compiler's
// choice) and the first pass's stack depth, which sets the shared memory per
// block.  Together they set how many warps an SM holds: 16 (compiler, ~120
// registers), 24 (80 registers, 256 entries), 28 (72 registers, 128 entries),
// 32 (64 registers, 64 entries; 8 blocks of ~27 KB).  A shallower stack sends
// more groups to the retry pass; the deepest stack on the bench workloads is
// under 50 entries.  The prefetch variants also ask for the child records of
// every node they push for opening (512 bytes from its first child) to be
// brought into L1, so that the next batch's staging, which takes exactly those
// children, finds them there.  Results do not depend on the variant.
struct WalkVariant {
    int min_blocks, stack, regs;
    bool prefetch;
};
constexpr WalkVariant kVariants[] = {{1, 256, 0, false}, {6, 256, 80, false}, {7, 128, 72, false},
                                     {8, 64, 64, false},  {6, 256, 80, true},  {7, 128, 72, true}};
constexpr int kWalkVariants = kWalkVariantCount;
static_assert(sizeof(kVariants) / sizeof(kVariants[0]) == kWalkVariants, "variant table");

struct WalkArgs {
    int n;
    const double *px, *py, *pz, *vx, *vy, *vz, *m, *h, *rho, *P;
    const uint8_t *type;
    const int32_t *pnode;
    double *ax, *ay, *az, *dUdt;
    const WalkRec *wrec;
    const int32_t *first, *leafpos;
    const int8_t *level;
    const NodeMom *mom;
    const double *radius;
    const int4 *groups;  // (first slot, lanes, instance = root node, 0)
    int ngroups;
    const uint8_t *active;  // per slot: walk it (block time steps); null = every particle
    int32_t *retry_groups;  // groups the FP32 walk's first pass sends to the retry pass
    const double *inst_R;   // root half-width per instance: the FP32 walk's length scale (walk_scale)
    double theta, e0, G;
    Ctx::Ctl *ctl;
};

// ---- reference kernels (FP64) ------------------------------------------------

__device__ double softening_kernel(double u)
{
    // kernel::softeningKernel (kernel.cpp:41-56), same polynomial
    if (u >= 0 && u < 0.5)
        return (16.0 / 3.0) * (u * u) - (48.0 / 5.0) * pow(u, 4.0) + (32.0 / 5.0) * pow(u, 5.0) - (14.0 / 5.0);
    if (u >= 0.5 && u < 1.0)
        return (1.0 / (15.0 * u)) + (32.0 / 3.0) * (u * u) - 16.0 * pow(u, 3.0) - (48.0 / 5.0) * pow(u, 4.0) -
               (32.0 / 15.0) * pow(u, 5.0) - (16.0 / 5.0);
    if (u >= 1.0) return -1.0 / u;
    return 0.0;
}

// Softening length actually used by Node.cpp:285-305.  The reference writes
// abs(e) unqualified; in its translation unit that is int abs(int), so the test
// e0*1e-4 < |e| < 1e30 sees |e| truncated to an integer (x86-64 conversion
// semantics out of range).  Returns false where the reference returns early.
__device__ bool general_eps2(double r, double e0, double *eps2)
{
    double u = r / (2.8 * e0);
    double K = softening_kernel(u);
    if ((K - r) == 0) return false;
    double e = -(2.8 * e0) / (K - r);
    if (isnan(e)) return false;
    double ae;
    if (!(e > -2147483649.0 && e < 2147483648.0))
        ae = -2147483648.0;
    else
        ae = fabs(trunc(e));
    double eps = (ae > e0 * 0.0001 && ae < 1e30) ? e : e0;
    *eps2 = eps * eps;
    return true;
}

template <class F>
struct Vec3 {
    F x, y, z;
};

// kernel::gradientCubicSplineKernel (kernel.cpp:18-39): returns the scalar s
// with gradW = d * s
template <class F>
__device__ __forceinline__ F grad_w_scale(F r, F h)
{
    if (r == F(0)) return F(0);
    F alpha = F(1) / (F(kPi) * h * h * h);
    F q = r / h;
    F g;
    if (q < F(1))
        g = alpha * (F(-3) * q + F(2.25) * q * q);
    else if (q < F(2))
        g = alpha * (F(-0.75) * (F(2) - q) * (F(2) - q));
    else
        return F(0);
    g = g / h;
    return g / r;
}

// Node::calcSPHForce with j = i substitutions (Node.cpp:88-172).
// dd = x_i - COM, vij = v_i - v_j.  Adds to f (unless NaN) and du.
template <class F>
__device__ __forceinline__ void sph_pair(F gm, F dx, F dy, F dz, F r, F vx, F vy, F vz, F h, F pr, F c,
                                         Vec3<F> &f, F &du)
{
    F s = grad_w_scale<F>(r, h);
    F gx = dx * s, gy = dy * s, gz = dz * s;
    F fx = -gm * pr * gx, fy = -gm * pr * gy, fz = -gm * pr * gz;
    F vd = vx * dx + vy * dy + vz * dz;
    F mu = h * vd / (r * r + F(0.01) * (h * h));
    F MU = F(0);
    if (vd < F(0)) MU = F(-0.5) * c * mu + F(1) * (mu * mu);
    fx += -gm * MU * gx;
    fy += -gm * MU * gy;
    fz += -gm * MU * gz;
    du += F(0.5) * gm * (pr + MU) * (vx * gx + vy * gy + vz * gz);
    if (isnan(fx) || isnan(fy) || isnan(fz)) return;
    f.x += fx;
    f.y += fy;
    f.z += fz;
}

// The FP32 walk's form of sph_pair: the same terms regrouped around q = r/h
// so that no intermediate leaves FP32's range in SI units.  Lengths (d, r, h)
// are in the instance's scaled units, gm2 = gasMass * ls^2 and pr2 = pr *
// ls^2; velocities and c as they are.  With s = g(q) / (pi h^4 r) the
// reference's force -gm pr d s - gm MU d s is -(d/r) g(q)/pi K and its du term
// 0.5 gm (pr + MU) (v . d) s is 0.5 (v . d/r) g(q)/pi K, where
// K = gm (pr + MU) / h^4 = gm2 (pr2 + MU ls^2) / h'^4 (the scales cancel), and
// mu = h (v . d) / (r^2 + 0.01 h^2) = (v . d/h) / (q^2 + 0.01).
__device__ __forceinline__ void sph_pair32(float gm2, float dx, float dy, float dz, float r2, float vx, float vy,
                                           float vz, float ih, float pr2, float c, float ls2, Vec3<float> &f, float &du)
{
    if (r2 == 0.0f) return;
    const float ir = rsqrtf(r2);
    const float q = r2 * ir * ih;
    float g;
    if (q < 1.0f)
        g = -3.0f * q + 2.25f * q * q;
    else if (q < 2.0f)
        g = -0.75f * (2.0f - q) * (2.0f - q);
    else
        return;
    const float vd = vx * dx + vy * dy + vz * dz;
    const float mu = __fdividef(vd * ih, q * q + 0.01f);
    float MU = 0.0f;
    if (vd < 0.0f) MU = -0.5f * c * mu + mu * mu;
    const float ih2 = ih * ih;
    const float K = gm2 * (pr2 + MU * ls2) * (ih2 * ih2);
    const float t = g * (1.0f / (float)kPi) * K * ir;
    du += 0.5f * vd * t;
    const float fx = -dx * t, fy = -dy * t, fz = -dz * t;
    if (isnan(fx) || isnan(fy) || isnan(fz)) return;
    f.x += fx;
    f.y += fy;
    f.z += fz;
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float v)
{
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// ---- FP64 plain walk ---------------------------------------------------------

template <bool kGeneral, bool kGas>
__global__ void __launch_bounds__(kWalkBlock) k_walk64(WalkArgs a)
{
    __shared__ int2 stk_all[(kWalkBlock / 32) * kStack];
    const int lane = threadIdx.x & 31;
    int2 *stk = stk_all + (threadIdx.x >> 5) * kStack;
    const int ngroups = a.ngroups;
    const double eps02 = a.e0 * a.e0;
    unsigned long long cnt_g = 0, cnt_s = 0;
    for (;;) {
        int grp = 0;
        if (lane == 0) grp = atomicAdd(&a.ctl->list_count, 1);
        grp = __shfl_sync(0xffffffffu, grp, 0);
        if (grp >= ngroups) break;
        const int4 gd = a.groups[grp];
        const int i = gd.x + lane;
        const bool live = lane < gd.y;
        const int root = gd.z;
        const bool act = live && (!a.active || a.active[i]);  // block steps walk the due particles only
        const bool valid = act && a.m[i] != 0.0;
        double xi = 0, yi = 0, zi = 0, hi_ = 0, pr = 0, cs = 0, vxi = 0, vyi = 0, vzi = 0;
        bool gas_i = false;
        int myleaf = -1;
        if (live) {
            xi = a.px[i];
            yi = a.py[i];
            zi = a.pz[i];
            int pn = a.pnode[i];
            myleaf = (pn >= 0 && a.leafpos[pn] == i) ? pn : -1;
            if (kGas && a.type[i] == 2) {
                gas_i = true;
                hi_ = a.h[i];
                double rho = a.rho[i], P = a.P[i];
                pr = P / (rho * rho) + P / (rho * rho);
                cs = sqrt(kGamma * P / rho);
                vxi = a.vx[i];
                vyi = a.vy[i];
                vzi = a.vz[i];
            }
        }
        Vec3<double> acc = {0, 0, 0};
        double du = 0;
        const unsigned all = __ballot_sync(0xffffffffu, valid);
        int sp = 0;
        bool overflow = false;
        if (all && a.mom[root].mass != 0.0) {
            stk[0] = make_int2(root, (int)all);  // evaluate the root itself
            sp = 1;
        }
        __syncwarp();
        // stack entries: (node, lanes) -- evaluate `node` for these lanes
        while (sp > 0) {
            sp--;
            const int2 e = stk[sp];
            __syncwarp();
            const int c = e.x;
            const unsigned msk = (unsigned)e.y;
            const bool in = (msk >> lane) & 1u;
            bool open = false;
            const int32_t fc = a.first[c];
            const bool leaf = fc < 0;
            if (in && !(leaf && c == myleaf)) {
                double dx = a.mom[c].cx - xi, dy = a.mom[c].cy - yi, dz = a.mom[c].cz - zi;
                double r = sqrt(dx * dx + dy * dy + dz * dz);
                if (r != 0.0) {
                    bool interact = leaf;
                    if (!leaf) {
                        double rad = a.radius[c];
                        if (rad / r < a.theta)
                            interact = true;
                        else
                            open = true;
                    }
                    if (interact) {
                        double e2 = eps02;
                        bool ok = true;
                        if (kGeneral) ok = general_eps2(r, a.e0, &e2);
                        if (ok) {
                            double s = a.G * a.mom[c].mass / (r * r + e2);
                            double gx = (dx / r) * s, gy = (dy / r) * s, gz = (dz / r) * s;
                            if (!(isnan(gx) || isnan(gy) || isnan(gz))) {
                                acc.x += gx;
                                acc.y += gy;
                                acc.z += gz;
                                cnt_g++;
                                if (kGas && gas_i && r < hi_ * 2) {
                                    double gm = a.mom[c].gas;
                                    if (gm > 0) {
                                        double vjx, vjy, vjz;
                                        if (leaf) {
                                            int lp = a.leafpos[c];
                                            vjx = a.vx[lp];
                                            vjy = a.vy[lp];
                                            vjz = a.vz[lp];
                                        } else {
                                            vjx = a.mom[c].mvx;
                                            vjy = a.mom[c].mvy;
                                            vjz = a.mom[c].mvz;
                                        }
                                        sph_pair<double>(gm, -dx, -dy, -dz, r, vxi - vjx, vyi - vjy, vzi - vjz, hi_,
                                                         pr, cs, acc, du);
                                        cnt_s++;
                                    }
                                }
                            }
                        }
                    }
                }
            }
            const unsigned om = __ballot_sync(0xffffffffu, open);
            if (om) {
                const unsigned cm = (unsigned)a.wrec[c].C.z;  // bit o: child o has mass
                const int nch = __popc(cm);
                if (sp + nch > kStack) {
                    overflow = true;
                    break;
                }
                // push children 7..0 so that child 0 is evaluated first (DFS order)
                for (int o = 7; o >= 0; o--)
                    if ((cm >> o) & 1u) {
                        if (lane == 0) stk[sp] = make_int2(fc + o, (int)om);
                        sp++;
                    }
            }
            __syncwarp();
        }
        if (overflow && lane == 0) {
            atomicExch(&a.ctl->err_code, (int)AG2_E_STACK);
            atomicExch(&a.ctl->err_info, grp);
        }
        if (act) {
            a.ax[i] = valid ? acc.x : 0.0;
            a.ay[i] = valid ? acc.y : 0.0;
            a.az[i] = valid ? acc.z : 0.0;
            if (kGas && gas_i && valid) a.dUdt[i] += du;
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt_g += __shfl_down_sync(0xffffffffu, cnt_g, o);
        cnt_s += __shfl_down_sync(0xffffffffu, cnt_s, o);
    }
    if (lane == 0) {
        atomicAdd(&a.ctl->inter_grav, cnt_g);
        atomicAdd(&a.ctl->inter_sph, cnt_s);
    }
}

// ---- FP32-offset walk --------------------------------------------------------

// warp min / max of ordered integer keys (okey), on the integer pipe
__device__ __forceinline__ long long warp_kmin(long long v)
{
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_kmax(long long v)
{
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// the double of an ordered key (okey's inverse; -0 comes back as +0)
__device__ __forceinline__ double unkey(long long k)
{
    return __longlong_as_double(k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFLL));
}

// Shared-memory layout per warp: the stack, the batch of up to 32 children
// being decided (staged one per lane), and the interaction list (accepted node
// + the lanes that accepted it) that the force loop consumes.
constexpr int kBatch = 32;
constexpr int kList = 96;
template <int kStk>
struct alignas(16) WarpSmemT {
    float4 cpos[kBatch];     // com - group centre (lane-invariant part), mass
    float4 cgas[kBatch];     // gas velocity, gasMass
    float cmac[kBatch];      // (radius/theta)^2, or -1 for a leaf
    float4 cthr[kBatch];     // per-lane test thresholds on r^2: open above .y and below .z, accept above .w
    int cfirst[kBatch];      // first child of the child (-1 leaf)
    int bchild[kBatch];      // node index of batch slot j
    unsigned bmask[kBatch];  // lanes that evaluate batch slot j
    unsigned char ccm[kBatch];  // child mask of the child
    unsigned char ccls[kBatch]; // group-level class: 0 per-lane, 1 every lane opens, 2 every lane accepts
    unsigned cself[kBatch];     // lane whose own leaf this child is (bit), else 0
    unsigned bkeep[kBatch];     // lanes that evaluate batch slot j, less the one whose own leaf it is
    unsigned char mq[kBatch];   // batch slot of the q-th child the lanes decide one by one
    // ... its centre and thresholds, two children per three float4 so that the
    // decision loop reads packed pairs: (x0 x1 y0 y1) (z0 z1 acc0 acc1)
    // (open-above0 open-above1 open-below0 open-below1), children 2p and 2p+1
    float4 mpair[3 * kBatch / 2];
    unsigned mkeep[kBatch];     // ... and the lanes that decide it
    // accepted nodes, two entries per two float4: (x0 x1 y0 y1) (z0 z1 w0 w1)
    // for entries 2p and 2p+1 (relative com, G m ls^2)
    float4 lpair[kList];
    unsigned lmask[kList];   // lanes that accepted them
    double xd[3][32];        // FP64 positions of the group (read only by the exact re-check)
    int2 stk[kStk];          // (first child of a node to open, lane mask)
    unsigned char stkcm[kStk];
};

// 32 x 32 bit transpose across the warp: lane i holds row i (bit j = column
// j); afterwards lane j holds column j (bit i = row i).  Five butterfly stages
// swap the off-diagonal blocks of halving size.
__device__ __forceinline__ unsigned transpose32(unsigned x, int lane)
{
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        const unsigned m = s == 16 ? 0x0000ffffu : s == 8 ? 0x00ff00ffu : s == 4 ? 0x0f0f0f0fu : s == 2 ? 0x33333333u
                                                                                                  : 0x55555555u;
        const unsigned y = __shfl_xor_sync(0xffffffffu, x, s);
        x = (lane & s) ? ((x & ~m) | ((y & ~m) >> s)) : ((x & m) | ((y & m) << s));
    }
    return x;
}

// Interaction-list entry q: its node's relative centre of mass and G m ls^2
// into the pair layout, and the lanes that take it.
template <class WS>
__device__ __forceinline__ void put_entry(WS &W, int q, float4 P, unsigned lanes)
{
    float *L = reinterpret_cast<float *>(W.lpair) + 8 * (q >> 1) + (q & 1);
    L[0] = P.x;
    L[2] = P.y;
    L[4] = P.z;
    L[6] = P.w;
    W.lmask[q] = lanes;
}
template <class WS>
__device__ __forceinline__ float4 get_entry(const WS &W, int q)
{
    const float *L = reinterpret_cast<const float *>(W.lpair) + 8 * (q >> 1) + (q & 1);
    return make_float4(L[0], L[2], L[4], L[6]);
}

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Force loop over the interaction list: every lane evaluates every entry and
// keeps it when its bit is set, summing into a batch that is added to the
// compensated accumulator once per flush.  Entries go two at a time through
// packed FP32 instructions (fma/add/mul.rn.f32x2, IEEE rounding per element):
// entry 2p in the low and 2p+1 in the high half of every pair, so the low and
// high halves of the batch sums hold the even and the odd entries, added
// together at the end of the flush.  An entry a lane does not take gets the
// factor 0 (a select), which leaves the sums unchanged.  With kOneRsq the
// factor 1 / (r (r^2 + e^2)) is one reciprocal square root of
// r^2 (r^2 + e^2)^2 instead of a reciprocal square root and a reciprocal; the
// caller takes it when e0^2 (scaled) exceeds 3e-9, where every distance the
// list holds (r^2 above 1e-12 e0^2, smaller ones go to the FP64 path) keeps
// that product above 1e-12 e0^6 > 2.7e-37, inside FP32's normal range.  The
// general softening law decides per lane in FP64 and keeps the scalar loop.
template <bool kGeneral, bool kOneRsq = false, class WS>
__device__ __forceinline__ void flush_list(WS &W, int cnt, int lane, float ox, float oy, float oz,
                                           float eps02, double e0, double ls, float &sx, float &sy, float &sz,
                                           float &kx, float &ky, float &kz, unsigned long long &cnt_g)
{
    float bx = 0.f, by = 0.f, bz = 0.f;
    if (kGeneral) {
        int mine = 0;
#pragma unroll 1
        for (int j = 0; j < cnt; j++) {
            const float4 P = get_entry(W, j);
            bool take = (W.lmask[j] >> lane) & 1u;
            const float dx = P.x - ox, dy = P.y - oy, dz = P.z - oz;
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float ir = rsqrtf(r2);
            float e2 = eps02;
            // the general law decides on the distance in the caller's units
            double de2 = 0.0;
            if (take) {
                if (general_eps2((double)(r2 * ir) / ls, e0, &de2))
                    e2 = (float)(de2 * ls * ls);
                else
                    take = false;  // the reference returns without a force (Node.cpp:285-305)
            }
            mine += take ? 1 : 0;
            const float sc = __fdividef(P.w * ir, r2 + e2);
            if (take) {
                bx = fmaf(dx, sc, bx);
                by = fmaf(dy, sc, by);
                bz = fmaf(dz, sc, bz);
            }
        }
        cnt_g += (unsigned long long)mine;
    } else {
        if (cnt & 1) {  // an odd list ends with a pair whose high entry no lane takes
            if (lane == 0) put_entry(W, cnt, make_float4(0.f, 0.f, 0.f, 0.f), 0u);
            __syncwarp();
        }
        const float2 nox = f2(-ox, -ox), noy = f2(-oy, -oy), noz = f2(-oz, -oz), e2 = f2(eps02, eps02);
        float2 px = f2(0.f, 0.f), py = f2(0.f, 0.f), pz = f2(0.f, 0.f);
        const int np = (cnt + 1) >> 1;
#pragma unroll 2
        for (int p = 0; p < np; p++) {
            const float4 A = W.lpair[2 * p], B = W.lpair[2 * p + 1];
            const uint2 M = reinterpret_cast<const uint2 *>(W.lmask)[p];
            const float2 dx = __fadd2_rn(f2(A.x, A.y), nox), dy = __fadd2_rn(f2(A.z, A.w), noy),
                         dz = __fadd2_rn(f2(B.x, B.y), noz);
            const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
            const float2 t = __fadd2_rn(r2, e2);
            float2 sc;
            if (kOneRsq) {
                const float2 q = __fmul2_rn(__fmul2_rn(r2, t), t);
                sc = __fmul2_rn(f2(B.z, B.w), f2(rsqrtf(q.x), rsqrtf(q.y)));
            } else {
                const float2 num = __fmul2_rn(f2(B.z, B.w), f2(rsqrtf(r2.x), rsqrtf(r2.y)));
                sc = f2(__fdividef(num.x, t.x), __fdividef(num.y, t.y));
            }
            sc.x = ((M.x >> lane) & 1u) ? sc.x : 0.f;
            sc.y = ((M.y >> lane) & 1u) ? sc.y : 0.f;
            px = __ffma2_rn(dx, sc, px);
            py = __ffma2_rn(dy, sc, py);
            pz = __ffma2_rn(dz, sc, pz);
        }
        bx = px.x + px.y;
        by = py.x + py.y;
        bz = pz.x + pz.y;
        // every set mask bit is one interaction: count them lane-parallel
        for (int j = lane; j < cnt; j += 32) cnt_g += (unsigned long long)__popc(W.lmask[j]);
    }
    kahan_add(sx, kx, bx);
    kahan_add(sy, ky, by);
    kahan_add(sz, kz, bz);
}

// Rare path of the FP32 walk: an opening test within the guard band of the
// threshold, or a distance too small for the float offsets, is decided again
// exactly as the FP64 walk decides it (and such a tiny-distance interaction is
// evaluated in FP64).  Returns 0 skip, 1 interact in FP32, 2 open, 3 done.
template <bool kGeneral>
__device__ __noinline__ int recheck_fp64(const WalkArgs &a, int c, bool leaf, const double (*xd)[32], int lane,
                                         bool tiny, Vec3<float> &bs, unsigned long long &cnt_g)
{
    const double xi = xd[0][lane], yi = xd[1][lane], zi = xd[2][lane];
    double ddx = a.mom[c].cx - xi, ddy = a.mom[c].cy - yi, ddz = a.mom[c].cz - zi;
    double r = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    if (r == 0.0) return 0;
    int decision = (leaf || a.radius[c] / r < a.theta) ? 1 : 2;
    if (decision == 1 && tiny) {
        double e2 = a.e0 * a.e0;
        if (!kGeneral || general_eps2(r, a.e0, &e2)) {
            double sc = a.G * a.mom[c].mass / (r * r + e2);
            bs.x += (float)((ddx / r) * sc);
            bs.y += (float)((ddy / r) * sc);
            bs.z += (float)((ddz / r) * sc);
            cnt_g++;
        }
        return 3;
    }
    return decision;
}

// The child block of a node pushed for opening, its 8 walk records (512 bytes
// from the first child, 4 or 5 cache lines), into L1 ahead of the batch that
// stages them.  A hint: nothing waits for it.
__device__ __forceinline__ void prefetch_children(const WalkRec *r)
{
    const char *p = reinterpret_cast<const char *>(r);
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 128));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 256));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 384));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 511));
}

// kStk = kStack: the second pass over the groups the first one could not hold
// in its stack (a.retry_groups, ctl->retry_count of them), with the full stack.
template <bool kGeneral, bool kGas, int kMinBlocks, int kStk, bool kPrefetch = false>
__global__ void __launch_bounds__(kWalkBlock, kMinBlocks) k_walk32(WalkArgs a)
{
    constexpr bool kRetry = kStk == kStack;
    using WS = WarpSmemT<kStk>;
    __shared__ WS sm_all[kWalkBlock / 32];
    const int lane = threadIdx.x & 31;
    WS &W = sm_all[threadIdx.x >> 5];
    const int ngroups = kRetry ? a.ctl->retry_count : a.ngroups;
    const float G = (float)a.G;
    unsigned long long cnt_g = 0, cnt_s = 0;
    for (;;) {
        int grp = 0;
        if (lane == 0) grp = atomicAdd(kRetry ? &a.ctl->retry_claim : &a.ctl->list_count, 1);
        grp = __shfl_sync(0xffffffffu, grp, 0);
        if (grp >= ngroups) break;
        if (kRetry) grp = a.retry_groups[grp];
        const unsigned long long cg0 = cnt_g, cs0 = cnt_s;  // a group sent to the retry pass counts there
        const int4 gd = a.groups[grp];
        const int i = gd.x + lane;
        const bool live = lane < gd.y;
        const int root = gd.z;
        const bool act = live && (!a.active || a.active[i]);  // block steps walk the due particles only
        const bool valid = act && a.m[i] != 0.0;
        // the instance's length scale: offsets, r^2, e0^2, h are in its units
        const int lsk = walk_scale_exp(a.inst_R[root]);
        const double ls = walk_scale(a.inst_R[root]);
        const float eps02 = (float)(a.e0 * a.e0 * ls * ls);
        const float ls2f = (float)(ls * ls);
        // Group set-up in FP64 (positions, group centre, float offsets).  No FP64
        // value stays live past this block: on this part FP64 instructions issue
        // at 1/64 of the FP32 rate, so the compiler must not be able to
        // re-derive the float offsets from doubles inside the walk.
        float ghx, ghy, ghz, glx, gly, glz, ox, oy, oz;
        {
            double xi = 0, yi = 0, zi = 0;
            if (live) {
                xi = a.px[i];
                yi = a.py[i];
                zi = a.pz[i];
            }
            W.xd[0][lane] = xi;
            W.xd[1][lane] = yi;
            W.xd[2][lane] = zi;
            // the group's box: min and max of ordered integer keys (no FP64
            // compare; this part issues FP64 at 1/64 of the FP32 rate)
            double gx = 0, gy = 0, gz = 0;
            const long long kx = okey(xi), ky = okey(yi), kz = okey(zi);
            const long long klx = warp_kmin(valid ? kx : LLONG_MAX), kly = warp_kmin(valid ? ky : LLONG_MAX),
                            klz = warp_kmin(valid ? kz : LLONG_MAX);
            const long long kux = warp_kmax(valid ? kx : LLONG_MIN), kuy = warp_kmax(valid ? ky : LLONG_MIN),
                            kuz = warp_kmax(valid ? kz : LLONG_MIN);
            if (klx <= kux) {
                gx = scale2(unkey(klx) + unkey(kux), -1);
                gy = scale2(unkey(kly) + unkey(kuy), -1);
                gz = scale2(unkey(klz) + unkey(kuz), -1);
            }
            const double sgx = scale2(gx, lsk), sgy = scale2(gy, lsk), sgz = scale2(gz, lsk);
            ghx = (float)sgx;
            ghy = (float)sgy;
            ghz = (float)sgz;
            glx = (float)(sgx - (double)ghx);
            gly = (float)(sgy - (double)ghy);
            glz = (float)(sgz - (double)ghz);
            ox = (float)scale2(xi - gx, lsk);
            oy = (float)scale2(yi - gy, lsk);
            oz = (float)scale2(zi - gz, lsk);
            // opaque copies: the walk below sees plain floats
            asm volatile("" : "+f"(ghx), "+f"(ghy), "+f"(ghz), "+f"(glx), "+f"(gly), "+f"(glz));
            asm volatile("" : "+f"(ox), "+f"(oy), "+f"(oz));
        }
        int myleaf = -1;
        float hi_ = 0, ih_ = 0, pr = 0, cs = 0, vxi = 0, vyi = 0, vzi = 0;
        bool gas_i = false;
        if (live) {
            int pn = a.pnode[i];
            myleaf = (pn >= 0 && a.leafpos[pn] == i) ? pn : -1;
            if (kGas && a.type[i] == 2) {
                gas_i = true;
                hi_ = (float)scale2(a.h[i], lsk);
                ih_ = 1.0f / hi_;
                double rho = a.rho[i], P = a.P[i];
                const double q = P / (rho * rho);
                pr = (float)scale2(q + q, 2 * lsk);  // P/rho^2 + P/rho^2 (Node.cpp:97), in scaled units
                cs = (float)sqrt(kGamma * P / rho);
                vxi = (float)a.vx[i];
                vyi = (float)a.vy[i];
                vzi = (float)a.vz[i];
            }
        }
        asm volatile("" : "+f"(hi_), "+f"(ih_), "+f"(pr), "+f"(cs), "+f"(vxi), "+f"(vyi), "+f"(vzi));
        const float h2x4 = 4.0f * hi_ * hi_;
        // group bounding box (half-extents about the group centre, with slack for
        // rounding) and the largest SPH reach of its gas lanes
        float hbx = valid ? fabsf(ox) : 0.f, hby = valid ? fabsf(oy) : 0.f, hbz = valid ? fabsf(oz) : 0.f;
        float gas_reach2 = (kGas && gas_i && valid) ? h2x4 : 0.f;
        for (int o = 16; o > 0; o >>= 1) {
            hbx = fmaxf(hbx, __shfl_xor_sync(0xffffffffu, hbx, o));
            hby = fmaxf(hby, __shfl_xor_sync(0xffffffffu, hby, o));
            hbz = fmaxf(hbz, __shfl_xor_sync(0xffffffffu, hbz, o));
            gas_reach2 = fmaxf(gas_reach2, __shfl_xor_sync(0xffffffffu, gas_reach2, o));
        }
        hbx = hbx * (1.0f + 1e-6f) + 1e-30f;
        hby = hby * (1.0f + 1e-6f) + 1e-30f;
        hbz = hbz * (1.0f + 1e-6f) + 1e-30f;
        float sx = 0, sy = 0, sz = 0, kx = 0, ky = 0, kz = 0;  // Kahan sums
        Vec3<float> side = {0, 0, 0};  // SPH and FP64-path contributions
        float du = 0;
        const unsigned all = __ballot_sync(0xffffffffu, valid);
        int sp = 0, nl = 0;
        bool overflow = false;
        // the root is the only child of a virtual parent (decided like any child)
        if (all && a.mom[root].mass != 0.0) {
            if (lane == 0) {
                W.stk[0] = make_int2(root, (int)all);
                W.stkcm[0] = 1;
            }
            sp = 1;
        }
        __syncwarp();
        while (sp > 0) {
            // gather up to 32 children from the top stack entries: lane k looks at
            // entry sp-1-k; an inclusive scan of their child counts decides how
            // many entries fit, and each taking lane expands its own entry
            int nc = 0;
            {
                const int idx = sp - 1 - lane;
                unsigned cmk = 0;
                int2 ek = make_int2(0, 0);
                if (idx >= 0) {
                    cmk = W.stkcm[idx];
                    ek = W.stk[idx];
                }
                const int k = __popc(cmk);
                int incl = k;
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                const bool take = idx >= 0 && incl <= kBatch;
                const unsigned tm = __ballot_sync(0xffffffffu, take);
                const int t = __popc(tm);
                nc = t ? __shfl_sync(0xffffffffu, incl, t - 1) : 0;
                if (take) {
                    int q = incl - k;
#pragma unroll
                    for (int o = 0; o < 8; o++)
                        if ((cmk >> o) & 1u) {
                            W.bchild[q] = ek.x + o;
                            W.bmask[q] = (unsigned)ek.y;
                            q++;
                        }
                }
                sp -= t;
            }
            __syncwarp();
            // stage: lane j loads batch slot j (one round trip for the batch)
            if (lane < nc) {
                const int c = W.bchild[lane];
                const WalkRec *R = a.wrec + c;
                const float4 A = R->A;
                const float4 B = R->B;
                const int4 C4 = R->C;
                const int f = C4.x;
                const unsigned char ccm = (unsigned char)C4.z;
                float4 D;
                if (kGas) D = R->D;
                const float cx = (A.x - ghx) + (B.x - glx), cy = (A.y - ghy) + (B.y - gly),
                            cz = (A.z - ghz) + (B.z - glz);
                W.cpos[lane] = make_float4(cx, cy, cz, G * A.w);
                W.cmac[lane] = B.w;
                {
                    // r^2 at or below `tiny`, or within the guard band around the
                    // opening threshold, is decided exactly in FP64 (recheck_fp64)
                    const float m = B.w;
                    const float tiny = m < 0.0f ? 1e-12f * eps02 : 1e-10f * m;
                    W.cthr[lane] = m < 0.0f ? make_float4(m, tiny, -1.0f, tiny)
                                            : make_float4(m, tiny, m - kGuard * m, m + kGuard * m);
                }
                W.cfirst[lane] = f;
                W.ccm[lane] = ccm;
                if (kGas) W.cgas[lane] = D;
                // Every lane's squared distance lies in [lo2, hi2], the nearest and
                // farthest points of the group's box.  When the whole interval is
                // clear of the opening threshold (outside the guard band) and of
                // the near-zero and SPH cases, all lanes decide alike and no
                // per-lane test is needed.  NaN centres fall through.
                unsigned selfm = 0u;
                if (B.w < 0.0f) {
                    const int lp = C4.y - gd.x;
                    if (lp >= 0 && lp < 32) selfm = 1u << lp;
                }
                W.cself[lane] = selfm;
                W.bkeep[lane] = W.bmask[lane] & ~selfm;
                const float ax_ = fabsf(cx), ay_ = fabsf(cy), az_ = fabsf(cz);
                const float nx = fmaxf(ax_ - hbx, 0.f), ny = fmaxf(ay_ - hby, 0.f), nz = fmaxf(az_ - hbz, 0.f);
                const float fx = ax_ + hbx, fy = ay_ + hby, fz = az_ + hbz;
                const float lo2 = fmaf(nx, nx, fmaf(ny, ny, nz * nz)), hi2 = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
                const float mac = B.w;
                unsigned char cls = 0;
                const bool no_sph = !kGas || !(D.w > 0.0f) || lo2 > gas_reach2;
                if (mac >= 0.0f) {
                    if (lo2 > 0.0f && hi2 < mac * (1.0f - 4.0f * kGuard))
                        cls = 1;
                    else if (lo2 > mac * (1.0f + 4.0f * kGuard) && no_sph)
                        cls = 2;
                } else if (lo2 > 4e-12f * eps02 && no_sph) {
                    cls = 2;
                }
                W.ccls[lane] = cls;
            }
            __syncwarp();
            // children every lane decides alike: lane j places child j at once
            unsigned mixed;
            {
                const int j = lane;
                const unsigned char cls = j < nc ? W.ccls[j] : (unsigned char)255;
                const unsigned bm = j < nc ? W.bmask[j] : 0u;
                const unsigned keep = j < nc ? W.bkeep[j] : 0u;
                const bool opn = cls == 1;
                const bool acc = cls == 2 && keep != 0u;
                const unsigned om = __ballot_sync(0xffffffffu, opn);
                const unsigned am = __ballot_sync(0xffffffffu, acc);
                mixed = __ballot_sync(0xffffffffu, cls == 0);
                const unsigned below = (1u << lane) - 1u;
                if (sp + __popc(om) > kStk) {
                    overflow = true;
                } else {
                    if (opn) {
                        const int q = sp + __popc(om & below);
                        W.stk[q] = make_int2(W.cfirst[j], (int)bm);
                        W.stkcm[q] = W.ccm[j];
                        if (kPrefetch) prefetch_children(a.wrec + W.cfirst[j]);
                    }
                    sp += __popc(om);
                }
                if (acc) put_entry(W, nl + __popc(am & below), W.cpos[j], keep);
                nl += __popc(am);
            }
            __syncwarp();
            // children the lanes decide one by one: every lane decides all of them
            // (bit q of its masks for the q-th), then a transpose gives lane q the
            // lanes that accept / open that child, and the entries are placed at once
            if (mixed) {
                const unsigned below = (1u << lane) - 1u;
                const int nm = __popc(mixed);
                if ((mixed >> lane) & 1u) {
                    const int q = __popc(mixed & below);
                    W.mq[q] = (unsigned char)lane;
                    const float4 P = W.cpos[lane], T = W.cthr[lane];
                    float *M = reinterpret_cast<float *>(W.mpair) + 12 * (q >> 1) + (q & 1);
                    M[0] = P.x;
                    M[2] = P.y;
                    M[4] = P.z;
                    M[6] = T.w;
                    M[8] = T.y;
                    M[10] = T.z;
                    W.mkeep[q] = W.bkeep[lane];
                }
                if (lane == 0 && (nm & 1)) W.mkeep[nm] = 0u;  // the high half of the last pair: no lane
                __syncwarp();
                unsigned accb = 0u, opnb = 0u, sphb = 0u, rqb = 0u;
                {
                    // two children per iteration: r^2 of both in packed FP32 (the
                    // same roundings per element as fmaf(dx, dx, fmaf(dy, dy, dz*dz))),
                    // then each child's tests for the lanes that decide it (all
                    // but the one whose own leaf it is)
                    const float2 nox = f2(-ox, -ox), noy = f2(-oy, -oy), noz = f2(-oz, -oz);
                    const int npair = (nm + 1) >> 1;
#pragma unroll 2
                    for (int p = 0; p < npair; p++) {
                        const float4 A = W.mpair[3 * p], B = W.mpair[3 * p + 1], T = W.mpair[3 * p + 2];
                        const uint2 K = reinterpret_cast<const uint2 *>(W.mkeep)[p];
                        const float2 dx = __fadd2_rn(f2(A.x, A.y), nox), dy = __fadd2_rn(f2(A.z, A.w), noy),
                                     dz = __fadd2_rn(f2(B.x, B.y), noz);
                        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                        const bool k0 = (K.x >> lane) & 1u, k1 = (K.y >> lane) & 1u;
                        const bool a0 = k0 && r2.x > B.z, a1 = k1 && r2.y > B.w;
                        const bool o0 = k0 && r2.x > T.x && r2.x < T.z, o1 = k1 && r2.y > T.y && r2.y < T.w;
                        const unsigned b0 = 1u << (2 * p), b1 = b0 << 1;
                        accb |= (a0 ? b0 : 0u) | (a1 ? b1 : 0u);
                        opnb |= (o0 ? b0 : 0u) | (o1 ? b1 : 0u);
                        rqb |= (k0 && !(a0 || o0) ? b0 : 0u) | (k1 && !(a1 || o1) ? b1 : 0u);
                        if (kGas && gas_i)
                            sphb |= (a0 && r2.x < h2x4 ? b0 : 0u) | (a1 && r2.y < h2x4 ? b1 : 0u);
                    }
                }
                // the rare tests decided in FP64 (near zero distance, or the guard band)
                if (__any_sync(0xffffffffu, rqb != 0u)) {
#pragma unroll 1
                    for (unsigned bq = rqb; bq; bq &= bq - 1u) {
                        const int q = __ffs(bq) - 1, j = W.mq[q];
                        const float4 Pc = W.cpos[j];
                        const float mac = W.cmac[j];
                        const bool leaf = mac < 0.0f;
                        const float dx = Pc.x - ox, dy = Pc.y - oy, dz = Pc.z - oz;
                        const float r2 = dx * dx + dy * dy + dz * dz;
                        const float tiny = leaf ? 1e-12f * eps02 : 1e-10f * mac;
                        const int decision = recheck_fp64<kGeneral>(a, W.bchild[j], leaf, W.xd, lane, r2 <= tiny, side,
                                                                    cnt_g);  // 0 skip, 1 accept, 2 open, 3 done
                        accb |= (decision == 1 ? 1u : 0u) << q;
                        opnb |= (decision == 2 ? 1u : 0u) << q;
                        if (kGas && gas_i && (decision == 1 || decision == 3) && r2 < h2x4) sphb |= 1u << q;
                    }
                }
                // SPH pairs (gas lane p, mixed child q): a separate pass keeps the loop
                // above small.  The pairs are spread over all lanes, 32 at a time (gas
                // lanes are few, so a loop per lane would leave most lanes idle); each
                // lane then adds its own pairs' contributions in its bit order, as that
                // loop would, so the sums are the same bits.
                if (kGas && __any_sync(0xffffffffu, sphb != 0u)) {
                    const int cp = __popc(sphb);
                    int incl = cp;
                    for (int o = 1; o < 32; o <<= 1) {
                        const int v = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= o) incl += v;
                    }
                    const int ex = incl - cp;  // this lane's first pair
                    const int total = __shfl_sync(0xffffffffu, incl, 31);
#pragma unroll 1
                    for (int k0 = 0; k0 < total; k0 += 32) {
                        const int k = k0 + lane;
                        int p = 0;  // owner: the last lane whose first pair is at or before k
#pragma unroll
                        for (int st = 16; st > 0; st >>= 1) {
                            const int e = __shfl_sync(0xffffffffu, ex, p + st);
                            if (e <= k) p += st;
                        }
                        const unsigned pb = __shfl_sync(0xffffffffu, sphb, p);
                        const int pe = __shfl_sync(0xffffffffu, ex, p);
                        const float pox = __shfl_sync(0xffffffffu, ox, p), poy = __shfl_sync(0xffffffffu, oy, p),
                                    poz = __shfl_sync(0xffffffffu, oz, p), pih = __shfl_sync(0xffffffffu, ih_, p),
                                    ppr = __shfl_sync(0xffffffffu, pr, p), pcs = __shfl_sync(0xffffffffu, cs, p),
                                    pvx = __shfl_sync(0xffffffffu, vxi, p), pvy = __shfl_sync(0xffffffffu, vyi, p),
                                    pvz = __shfl_sync(0xffffffffu, vzi, p);
                        Vec3<float> f = {0.f, 0.f, 0.f};
                        float dd = 0.f;
                        if (k < total) {
                            // the (k - pe)-th set bit of the owner's mask
                            int rem = k - pe, q = 0;
                            unsigned m = pb;
#pragma unroll
                            for (int w = 16; w > 0; w >>= 1) {
                                const int c = __popc(m & ((1u << w) - 1u));
                                if (rem >= c) {
                                    rem -= c;
                                    m >>= w;
                                    q += w;
                                }
                            }
                            const int j = W.mq[q];
                            const float4 D = W.cgas[j];
                            if (D.w > 0.0f) {
                                const float4 Pc = W.cpos[j];
                                const float dx = Pc.x - pox, dy = Pc.y - poy, dz = Pc.z - poz;
                                sph_pair32(D.w, -dx, -dy, -dz, dx * dx + dy * dy + dz * dz, pvx - D.x, pvy - D.y,
                                           pvz - D.z, pih, ppr, pcs, ls2f, f, dd);
                                cnt_s++;
                            }
                        }
                        // this lane's pairs in the chunk sit in lanes [wb, we)
                        const int wb = max(ex - k0, 0), we = min(ex + cp - k0, 32);
                        const int mine = max(we - wb, 0);
                        const int most = (int)__reduce_max_sync(0xffffffffu, (unsigned)mine);
                        for (int s = 0; s < most; s++) {
                            const int w = (wb + s) & 31;
                            const float rx = __shfl_sync(0xffffffffu, f.x, w), ry = __shfl_sync(0xffffffffu, f.y, w),
                                        rz = __shfl_sync(0xffffffffu, f.z, w), rd = __shfl_sync(0xffffffffu, dd, w);
                            if (s < mine) {
                                side.x += rx;
                                side.y += ry;
                                side.z += rz;
                                du += rd;
                            }
                        }
                    }
                }
                accb = transpose32(accb, lane);
                opnb = transpose32(opnb, lane);
                const int jq = lane < nm ? (int)W.mq[lane] : 0;
                const bool ha = lane < nm && accb != 0u, ho = lane < nm && opnb != 0u;
                const unsigned hab = __ballot_sync(0xffffffffu, ha), hob = __ballot_sync(0xffffffffu, ho);
                if (ha) put_entry(W, nl + __popc(hab & below), W.cpos[jq], accb);
                nl += __popc(hab);
                const int nop = __popc(hob);
                if (sp + nop > kStk) {
                    overflow = true;
                } else {
                    if (ho) {
                        const int p = sp + __popc(hob & below);
                        W.stk[p] = make_int2(W.cfirst[jq], (int)opnb);
                        W.stkcm[p] = W.ccm[jq];
                        if (kPrefetch) prefetch_children(a.wrec + W.cfirst[jq]);
                    }
                    sp += nop;
                }
            }
            __syncwarp();
            if (overflow) break;
            if (nl > kList - kBatch) {
                if (eps02 > 3e-9f)
                    flush_list<kGeneral, true>(W, nl, lane, ox, oy, oz, eps02, a.e0, ls, sx, sy, sz, kx, ky, kz, cnt_g);
                else
                    flush_list<kGeneral>(W, nl, lane, ox, oy, oz, eps02, a.e0, ls, sx, sy, sz, kx, ky, kz, cnt_g);
                nl = 0;
                __syncwarp();
            }
        }
        if (nl > 0) {
            if (eps02 > 3e-9f)
                flush_list<kGeneral, true>(W, nl, lane, ox, oy, oz, eps02, a.e0, ls, sx, sy, sz, kx, ky, kz, cnt_g);
            else
                flush_list<kGeneral>(W, nl, lane, ox, oy, oz, eps02, a.e0, ls, sx, sy, sz, kx, ky, kz, cnt_g);
        }
        kahan_add(sx, kx, side.x);
        kahan_add(sy, ky, side.y);
        kahan_add(sz, kz, side.z);
        if (overflow) {
            if (!kRetry) {  // the retry pass walks this group again with the full stack
                if (lane == 0) a.retry_groups[atomicAdd(&a.ctl->retry_count, 1)] = grp;
                cnt_g = cg0;
                cnt_s = cs0;
                __syncwarp();
                continue;
            }
            if (lane == 0) {
                atomicExch(&a.ctl->err_code, (int)AG2_E_STACK);
                atomicExch(&a.ctl->err_info, grp);
            }
        }
        if (act) {
            a.ax[i] = valid ? (double)sx - (double)kx : 0.0;
            a.ay[i] = valid ? (double)sy - (double)ky : 0.0;
            a.az[i] = valid ? (double)sz - (double)kz : 0.0;
            if (kGas && gas_i && valid) a.dUdt[i] += (double)du;
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt_g += __shfl_down_sync(0xffffffffu, cnt_g, o);
        cnt_s += __shfl_down_sync(0xffffffffu, cnt_s, o);
    }
    if (lane == 0) {
        atomicAdd(&a.ctl->inter_grav, cnt_g);
        atomicAdd(&a.ctl->inter_sph, cnt_s);
    }
}

// Potential of every particle for the energy check, FP64, with the FP64
// walk's traversal and opening rule: phi_i = sum over accepted nodes and
// particles of -(G m / e0) atan(e0 / r), the potential of the pair force
// G m / (r^2 + e0^2) along d/r (Node.cpp:285-305 for e0 < 0.6).
__global__ void __launch_bounds__(kWalkBlock) k_potential(WalkArgs a, double *phi)
{
    __shared__ int2 stk_all[(kWalkBlock / 32) * kStack];
    const int lane = threadIdx.x & 31;
    int2 *stk = stk_all + (threadIdx.x >> 5) * kStack;
    const double e0 = a.e0;
    for (;;) {
        int grp = 0;
        if (lane == 0) grp = atomicAdd(&a.ctl->list_count, 1);
        grp = __shfl_sync(0xffffffffu, grp, 0);
        if (grp >= a.ngroups) break;
        const int4 gd = a.groups[grp];
        const int i = gd.x + lane;
        const bool live = lane < gd.y;
        const bool valid = live && a.m[i] != 0.0;
        double xi = 0, yi = 0, zi = 0;
        int myleaf = -1;
        if (live) {
            xi = a.px[i];
            yi = a.py[i];
            zi = a.pz[i];
            const int pn = a.pnode[i];
            myleaf = (pn >= 0 && a.leafpos[pn] == i) ? pn : -1;
        }
        double p = 0.0;
        const unsigned all = __ballot_sync(0xffffffffu, valid);
        int sp = 0;
        bool overflow = false;
        if (all && a.mom[gd.z].mass != 0.0) {
            stk[0] = make_int2(gd.z, (int)all);
            sp = 1;
        }
        __syncwarp();
        while (sp > 0) {
            sp--;
            const int2 e = stk[sp];
            __syncwarp();
            const int c = e.x;
            const bool in = ((unsigned)e.y >> lane) & 1u;
            bool open = false;
            const int32_t fc = a.first[c];
            const bool leaf = fc < 0;
            if (in && !(leaf && c == myleaf)) {
                const double dx = a.mom[c].cx - xi, dy = a.mom[c].cy - yi, dz = a.mom[c].cz - zi;
                const double r = sqrt(dx * dx + dy * dy + dz * dz);
                if (r != 0.0) {
                    if (leaf || a.radius[c] / r < a.theta) {
                        const double t = -(a.G * a.mom[c].mass / e0) * atan(e0 / r);
                        if (!isnan(t)) p += t;
                    } else {
                        open = true;
                    }
                }
            }
            const unsigned om = __ballot_sync(0xffffffffu, open);
            if (om) {
                const unsigned cm = (unsigned)a.wrec[c].C.z;  // bit o: child o has mass
                if (sp + __popc(cm) > kStack) {
                    overflow = true;
                    break;
                }
                for (int o = 7; o >= 0; o--)
                    if ((cm >> o) & 1u) {
                        if (lane == 0) stk[sp] = make_int2(fc + o, (int)om);
                        sp++;
                    }
            }
            __syncwarp();
        }
        if (overflow && lane == 0) {
            atomicExch(&a.ctl->err_code, (int)AG2_E_STACK);
            atomicExch(&a.ctl->err_info, grp);
        }
        if (live) phi[i] = valid ? p : 0.0;
        __syncwarp();
    }
}

// per-block sums of m v^2 / 2, m phi / 2 and (gas) m U, in a fixed order
__global__ void __launch_bounds__(256) k_energy_sums(int n, const double *m, const double *vx, const double *vy,
                                                    const double *vz, const double *phi, const double *U,
                                                    const uint8_t *type, double *part)
{
    __shared__ double sh[3][256];
    double k = 0, w = 0, u = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double mi = m[i];
        k += 0.5 * mi * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        w += 0.5 * mi * phi[i];
        if (type[i] == 2) u += mi * U[i];
    }
    sh[0][threadIdx.x] = k;
    sh[1][threadIdx.x] = w;
    sh[2][threadIdx.x] = u;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 3; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) part[3 * blockIdx.x + q] = sh[q][0];
}

// Every index of the pool up to its high-water mark, the holes that no
// traversal reaches included (their fields were never written): the instance
// index is checked before it indexes the table.
__global__ void k_update_mac(int64_t nnodes, const int32_t *first, const double *radius, const int32_t *inst,
                             int n_inst, const double *inst_R, WalkRec *wrec, double theta)
{
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    if (first[j] < 0) return;
    const int k = inst[j];
    if (k < 0 || k >= n_inst) return;
    const float q = (float)scale2(radius[j], walk_scale_exp(inst_R[k])) / (float)theta;
    wrec[j].B.w = q * q;
}

}  // namespace

static WalkArgs walk_args(Ctx *c)
{
    Particles &S = c->S();
    WalkArgs a;
    a.n = (int)c->n;
    a.px = S.px; a.py = S.py; a.pz = S.pz;
    a.vx = S.vx; a.vy = S.vy; a.vz = S.vz;
    a.m = S.m; a.h = S.h; a.rho = S.rho; a.P = S.P;
    a.type = S.type;
    a.pnode = c->pnode;
    a.ax = S.ax; a.ay = S.ay; a.az = S.az; a.dUdt = S.dUdt;
    a.wrec = c->nd.wrec;
    a.first = c->nd.first; a.leafpos = c->nd.leafpos; a.level = c->nd.level;
    a.mom = c->nd.mom;
    a.radius = c->nd.radius;
    a.groups = c->groups;
    a.active = c->walk_active;
    a.retry_groups = c->retry_groups;
    a.inst_R = c->inst_R;
    a.ngroups = c->ngroups;
    a.theta = c->prm.theta;
    a.e0 = c->prm.e0;
    a.G = c->prm.G;
    a.ctl = c->ctl;
    return a;
}

int run_energy(Ctx *c, double *out4)
{
    for (int k = 0; k < 4; k++) out4[k] = 0.0;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "ag2_energy needs a tree of the current positions");
    if (!(c->prm.e0 > 0.0 && c->prm.e0 < 0.6))
        return set_err(c, AG2_E_INVALID, "ag2_energy needs 0 < e0 < 0.6 (the softening law's Plummer form)");
    const int n = (int)c->n;
    if (n == 0) return AG2_OK;
    Particles &S = c->S();
    WalkArgs a = walk_args(c);
    double *phi = c->staging;        // n doubles
    double *part = c->staging + n;   // 3 per block (the staging area holds 6 doubles per particle)
    const int eb = (int)std::max<int64_t>(1, std::min<int64_t>(256, (6 * (int64_t)c->cap - n) / 3));
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->list_count, 0, sizeof(int32_t), c->stream));
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    const int blocks = std::min((c->ngroups + 3) / 4, c->sms * 16);
    AG2_LAUNCH(c, k_potential, std::max(blocks, 1), kWalkBlock, 0, a, phi);
    AG2_LAUNCH(c, k_energy_sums, eb, 256, 0, n, S.m, S.vx, S.vy, S.vz, phi, S.U, S.type, part);
    std::vector<double> h(3 * eb);
    AG2_CUDA(c, cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int rc = sync_ctl(c);
    if (rc) return rc;
    if (c->ctl_host->err_code) return set_err(c, c->ctl_host->err_code, "potential walk failed");
    for (int b = 0; b < eb; b++)
        for (int q = 0; q < 3; q++) out4[q] += h[3 * b + q];
    out4[3] = out4[0] + out4[1] + out4[2];
    return AG2_OK;
}

int run_forces(Ctx *c)
{
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "ag2_forces needs a tree (call ag2_build_tree)");
    if (c->n == 0) return AG2_OK;
    if (c->prm.theta != c->tree_theta) {
        AG2_LAUNCH(c, k_update_mac, grid_for((size_t)c->nnodes, 256), 256, 0, c->nnodes, c->nd.first, c->nd.radius,
                   c->nd.inst, c->n_inst, c->inst_R, c->nd.wrec, c->prm.theta);
        c->tree_theta = c->prm.theta;
    }
    WalkArgs a = walk_args(c);
    // The softening law reduces to Plummer softening with e0 whenever the
    // truncated |e| of Node.cpp:302 is 0 for every distance, i.e. e0 < 0.66.
    const bool general = !(c->prm.e0 > 0.0 && c->prm.e0 < 0.6);
    const bool gas = c->ngas > 0;
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->list_count, 0, sizeof(int32_t), c->stream));
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->retry_count, 0, 2 * sizeof(int32_t), c->stream));
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->inter_grav, 0, 2 * sizeof(unsigned long long), c->stream));
    const int dev_sms = c->sms;
    const int ngroups = c->ngroups;
    int blocks = std::min((ngroups + 3) / 4, dev_sms * 16);
    if (blocks < 1) blocks = 1;
#define WALK(K) AG2_LAUNCH(c, K, blocks, kWalkBlock, 0, a)
    if (c->prm.precision == AG2_PREC_FP64) {
        if (general) {
            if (gas) WALK((k_walk64<true, true>)); else WALK((k_walk64<true, false>));
        } else {
            if (gas) WALK((k_walk64<false, true>)); else WALK((k_walk64<false, false>));
        }
    } else {
        // the autotuned variant (kVariants: register budget and first-pass stack)
        const int v = c->walk_variant;
#define W32(G, S)                                                                 \
    do {                                                                          \
        if (v == 1) WALK((k_walk32<G, S, 6, 256>));                               \
        else if (v == 2) WALK((k_walk32<G, S, 7, 128>));                          \
        else if (v == 3) WALK((k_walk32<G, S, 8, 64>));                           \
        else if (v == 4) WALK((k_walk32<G, S, 6, 256, true>));                    \
        else if (v == 5) WALK((k_walk32<G, S, 7, 128, true>));                    \
        else WALK((k_walk32<G, S, 1, 256>));                                      \
        /* groups whose stack outgrew the first pass (none in the usual case) */  \
        AG2_LAUNCH(c, (k_walk32<G, S, 1, kStack>), dev_sms, kWalkBlock, 0, a);    \
    } while (0)
        if (general) {
            if (gas) W32(true, true); else W32(true, false);
        } else {
            if (gas) W32(false, true); else W32(false, false);
        }
#undef W32
    }
#undef WALK
    return AG2_OK;
}

// Walk time of each candidate (variant x group size) on the current tree,
// keeping the fastest.  The group size changes the groups' centres and hence
// the FP32 sums in their last bits (within the accuracy contract); the variant
// changes nothing in the results.
int run_autotune(Ctx *c, int *chosen, ag2_walk_config *out, int max_out, int *count)
{
    if (count) *count = 0;
    if (!c->have_tree) return set_err(c, AG2_E_INVALID, "ag2_autotune needs a tree (call ag2_build_tree)");
    if (c->prm.precision != AG2_PREC_FP32 || c->n == 0) {
        *chosen = c->walk_variant;
        return AG2_OK;
    }
    static const int kGroupSizes[] = {32, 16};
    cudaEvent_t e0, e1;
    AG2_CUDA(c, cudaEventCreate(&e0));
    AG2_CUDA(c, cudaEventCreate(&e1));
    const int gs0 = c->prm.group_size;
    float best = 1e30f;
    int best_v = 0, best_gs = 32, k = 0;
    int rc = AG2_OK;
    for (int gs : kGroupSizes) {
        c->prm.group_size = gs;
        if ((rc = build_groups(c))) break;
        for (int v = 0; v < kWalkVariants && !rc; v++) {
            c->walk_variant = v;
            float ms = 0;
            for (int rep = 0; rep < 2 && !rc; rep++) {  // the first run warms caches
                cudaEventRecord(e0, c->stream);
                if ((rc = run_forces(c))) break;
                cudaEventRecord(e1, c->stream);
                if (cudaEventSynchronize(e1) != cudaSuccess) rc = set_err(c, AG2_E_CUDA, "autotune timing failed");
                cudaEventElapsedTime(&ms, e0, e1);
            }
            if (rc) break;
            if (out && k < max_out)
                out[k] = ag2_walk_config{v, kVariants[v].regs, kVariants[v].min_blocks > 1 ? kVariants[v].min_blocks : 0,
                                         kVariants[v].stack, kVariants[v].prefetch ? 1 : 0, gs, ms};
            k++;
            if (ms < best) {
                best = ms;
                best_v = v;
                best_gs = gs;
            }
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        c->prm.group_size = gs0;
        build_groups(c);
        return rc;
    }
    c->walk_variant = best_v;
    c->prm.group_size = best_gs;
    if ((rc = build_groups(c))) return rc;
    c->graph_epoch++;
    *chosen = best_v;
    if (count) *count = k;
    return AG2_OK;
}

}  // namespace ag2
