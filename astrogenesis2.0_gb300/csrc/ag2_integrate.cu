// ag2_integrate.cu -- leapfrog kick/drift and internal-energy update.
//
// Reference: simulation/src/Physics/TimeIntegration.cpp:10-40 (Kick, Drift,
// Ueuler) and the step loop in simulation/src/Physics/Simulation.cpp:256-341
// (Hubble factor at :330-332).  The arithmetic is written in the reference's
// operation order with explicitly rounded FP64 operations, so the results are
// bit-identical to the reference's for the same inputs.
#include <climits>
#include <cstring>

#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ bool acc_nan(const Particles &s, int i)
{
    return isnan(s.ax[i]) || isnan(s.ay[i]) || isnan(s.az[i]);
}

// x / 2, exactly: the exponent field less one where x and the result are
// normal, else the multiply by 0.5 (zero, subnormal, infinity, NaN).  Both are
// the correctly rounded value of the same real number; the integer path keeps
// the FP64 pipe (1/64 of the FP32 rate on this part) for the other arithmetic.
__device__ __forceinline__ double half_of(double x)
{
    const long long b = __double_as_longlong(x);
    const int ef = (int)((b >> 52) & 0x7ff);
    return (ef > 1 && ef < 0x7ff) ? __longlong_as_double(b - (1LL << 52)) : __dmul_rn(x, 0.5);
}

// v = v + a*dt/2, skipped when acc has a NaN (TimeIntegration.cpp:12-18)
__device__ __forceinline__ void kick1(Particles &s, int i, double dt)
{
    if (acc_nan(s, i)) return;
    s.vx[i] = __dadd_rn(s.vx[i], half_of(__dmul_rn(s.ax[i], dt)));
    s.vy[i] = __dadd_rn(s.vy[i], half_of(__dmul_rn(s.ay[i], dt)));
    s.vz[i] = __dadd_rn(s.vz[i], half_of(__dmul_rn(s.az[i], dt)));
}

// x = x + v*dt (TimeIntegration.cpp:21-25)
__device__ __forceinline__ void drift1(Particles &s, int i, double dt)
{
    s.px[i] = __dadd_rn(s.px[i], __dmul_rn(s.vx[i], dt));
    s.py[i] = __dadd_rn(s.py[i], __dmul_rn(s.vy[i], dt));
    s.pz[i] = __dadd_rn(s.pz[i], __dmul_rn(s.vz[i], dt));
}

__global__ void k_kick(int n, Particles s, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) kick1(s, i, dt);
}

__global__ void k_drift(int n, Particles s, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) drift1(s, i, dt);
}

__global__ void k_kick_drift(int n, Particles s, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    kick1(s, i, dt);
    drift1(s, i, dt);
}

// U += dUdt*dt unless NaN, then dUdt = 0, for gas (TimeIntegration.cpp:28-40,
// called for type 2 only, Simulation.cpp:322-326)
__global__ void k_ueuler(int n, Particles s, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || s.type[i] != 2) return;
    double du = s.dUdt[i];
    if (!isnan(du)) s.U[i] = __dadd_rn(s.U[i], __dmul_rn(du, dt));
    s.dUdt[i] = 0.0;
}

__global__ void k_scale(int n, Particles s, double f)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    s.px[i] = __dmul_rn(s.px[i], f);
    s.py[i] = __dmul_rn(s.py[i], f);
    s.pz[i] = __dmul_rn(s.pz[i], f);
}

// second half of a step for every particle (Simulation.cpp:305-337):
// Ueuler for gas, position *= Hubble factor, kick
__global__ void k_close_step(int n, Particles s, double dt, double f)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (s.type[i] == 2) {
        double du = s.dUdt[i];
        if (!isnan(du)) s.U[i] = __dadd_rn(s.U[i], __dmul_rn(du, dt));
        s.dUdt[i] = 0.0;
    }
    if (f != 1.0) {  // x * 1 is x: without expansion the positions are not touched
        s.px[i] = __dmul_rn(s.px[i], f);
        s.py[i] = __dmul_rn(s.py[i], f);
        s.pz[i] = __dmul_rn(s.pz[i], f);
    }
    kick1(s, i, dt);
}

// ---- block time steps (Simulation.cpp:188-341 with min < max time step) -----
//
// Every particle carries its own power-of-two step and its next integration
// time.  A step advances the global time to the earliest next integration
// time; only the particles due then are kicked, drifted, walked and closed,
// while the tree, the visual density and the gas density cover every particle,
// as in the reference.

// eta*sqrt(e0/|a|) clamped to [min, max], then the power of two at or below it,
// not below min; min when |a| is zero (Simulation.cpp:196-206, 221-232)
__device__ __forceinline__ double block_dt(const Particles &s, int i, double eta, double e0, double dmin, double dmax)
{
    const double ax = s.ax[i], ay = s.ay[i], az = s.az[i];
    const double a = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)), __dmul_rn(az, az)));
    if (!(a > 0.0)) return dmin;
    double ts = __dmul_rn(eta, sqrt(__ddiv_rn(e0, a)));
    ts = ts < dmin ? dmin : (dmax < ts ? dmax : ts);  // std::clamp
    // std::pow(2, std::floor(std::log2(ts))): the exponent of ts with a unit significand
    const long long b = __double_as_longlong(ts);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ts > 0.0 && ex != 0 && ex != 0x7ff) ts = __longlong_as_double(b & 0x7ff0000000000000LL);
    return ts < dmin ? dmin : ts;  // std::max
}

__global__ void k_block_init(int n, Particles s, double eta, double e0, double dmin, double dmax, double t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ts = block_dt(s, i, eta, e0, dmin, dmax);
    s.tstep[i] = ts;
    s.tnext[i] = __dadd_rn(t, ts);
}

// new steps for particles whose time has come (Simulation.cpp:214-232), then the
// earliest next integration time (as an ordered integer key, atomicMin)
__global__ void k_block_sched(int n, Particles s, double eta, double e0, double dmin, double dmax, double t,
                              long long *tkey)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    long long k = LLONG_MAX;
    if (i < n) {
        double tn = s.tnext[i];
        if (t >= tn) {
            const double ts = block_dt(s, i, eta, e0, dmin, dmax);
            s.tstep[i] = ts;
            tn = __dadd_rn(t, ts);
            s.tnext[i] = tn;
        }
        k = okey(tn);
    }
    for (int o = 16; o > 0; o >>= 1) k = min(k, __shfl_xor_sync(0xffffffffu, k, o));
    // one update per block: warps of every block updating the one word serialise there
    __shared__ long long wmin[32];
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long b = LLONG_MAX;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) b = min(b, wmin[w]);
        if (b != LLONG_MAX) atomicMin(tkey, b);
    }
}

__device__ __forceinline__ double key_to_double(long long k)
{
    return __longlong_as_double(k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFLL));
}

// first kick and drift of the due particles (Simulation.cpp:258-271)
__global__ void k_block_kick_drift(int n, Particles s, const long long *tkey)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || s.tnext[i] != key_to_double(*tkey)) return;
    const double ts = s.tstep[i];
    kick1(s, i, ts);
    drift1(s, i, ts);
}

// the due particles in tree order (after the build), and how many
__global__ void k_block_flags(int n, const Particles s, const long long *tkey, uint8_t *active, int32_t *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool a = i < n && s.tnext[i] == key_to_double(*tkey);
    if (i < n) active[i] = a ? 1 : 0;
    const unsigned b = __ballot_sync(0xffffffffu, a);
    __shared__ int32_t wcnt[32];  // one update per block, as in k_block_sched
    if ((threadIdx.x & 31) == 0) wcnt[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t t = 0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) t += wcnt[w];
        if (t) atomicAdd(count, t);
    }
}

// second half for the due particles (Simulation.cpp:294-337): Ueuler for gas,
// position *= exp(H0*dt), kick, next integration time += dt
__global__ void k_block_close(int n, Particles s, const long long *tkey, double H0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || s.tnext[i] != key_to_double(*tkey)) return;
    const double ts = s.tstep[i];
    if (s.type[i] == 2) {
        const double du = s.dUdt[i];
        if (!isnan(du)) s.U[i] = __dadd_rn(s.U[i], __dmul_rn(du, ts));
        s.dUdt[i] = 0.0;
    }
    const double f = exp(__dmul_rn(H0, ts));
    s.px[i] = __dmul_rn(s.px[i], f);
    s.py[i] = __dmul_rn(s.py[i], f);
    s.pz[i] = __dmul_rn(s.pz[i], f);
    kick1(s, i, ts);
    s.tnext[i] = __dadd_rn(s.tnext[i], ts);
}

}  // namespace

int run_block_init(Ctx *c, double eta, double dmin, double dmax, double t)
{
    if (!(eta > 0.0) || !(dmin > 0.0) || !(dmax >= dmin)) return set_err(c, AG2_E_INVALID, "block steps: bad eta or limits");
    if (!c->blk_key) {
        AG2_CUDA(c, cudaMalloc(&c->blk_key, sizeof(long long) + sizeof(int32_t) * 2));
        c->blk_count = reinterpret_cast<int32_t *>(c->blk_key + 1);
    }
    c->blk_eta = eta;
    c->blk_dmin = dmin;
    c->blk_dmax = dmax;
    c->blk_t = t;
    c->blk_ready = true;
    AG2_LAUNCH(c, k_block_init, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), eta, c->prm.e0, dmin, dmax, t);
    AG2_CUDA(c, cudaStreamSynchronize(c->stream));
    return AG2_OK;
}

int run_block_step(Ctx *c, double H0, int with_visual, double Rv, double *t_out, int64_t *active_out)
{
    if (!c->blk_ready) return set_err(c, AG2_E_INVALID, "ag2_block_step needs ag2_block_init");
    const int n = (int)c->n;
    int rc;
    AG2_CUDA(c, cudaMemsetAsync(c->blk_key, 0x7f, sizeof(long long) + sizeof(int32_t), c->stream));
    AG2_LAUNCH(c, k_block_sched, grid_for(n, kBlock), kBlock, 0, n, c->S(), c->blk_eta, c->prm.e0, c->blk_dmin,
               c->blk_dmax, c->blk_t, c->blk_key);
    AG2_LAUNCH(c, k_block_kick_drift, grid_for(n, kBlock), kBlock, 0, n, c->S(), c->blk_key);
    if ((rc = build_tree(c)) != AG2_OK) return rc;
    if (with_visual && (rc = run_visual_density(c, Rv)) != AG2_OK) return rc;
    if ((rc = run_sph_density(c)) != AG2_OK) return rc;
    AG2_CUDA(c, cudaMemsetAsync(c->blk_count, 0, sizeof(int32_t), c->stream));
    AG2_LAUNCH(c, k_block_flags, grid_for(n, kBlock), kBlock, 0, n, c->S(), c->blk_key, c->staging_u8, c->blk_count);
    AG2_CUDA(c, cudaMemsetAsync(&c->ctl->err_code, 0, sizeof(int32_t), c->stream));
    c->walk_active = c->staging_u8;
    rc = run_forces(c);
    c->walk_active = nullptr;
    if (rc) return rc;
    AG2_LAUNCH(c, k_block_close, grid_for(n, kBlock), kBlock, 0, n, c->S(), c->blk_key, H0);
    if (H0 != 0.0) c->have_tree = false;
    long long key = 0;
    int32_t cnt = 0;
    AG2_CUDA(c, cudaMemcpyAsync(&key, c->blk_key, sizeof(key), cudaMemcpyDeviceToHost, c->stream));
    AG2_CUDA(c, cudaMemcpyAsync(&cnt, c->blk_count, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
    if ((rc = sync_ctl(c)) != AG2_OK) return rc;
    const long long kb = key >= 0 ? key : (key ^ 0x7FFFFFFFFFFFFFFFLL);
    std::memcpy(&c->blk_t, &kb, sizeof(double));
    c->inter_grav = (int64_t)c->ctl_host->inter_grav;
    c->inter_sph = (int64_t)c->ctl_host->inter_sph;
    if (c->ctl_host->err_code == AG2_E_STACK)
        return set_err(c, AG2_E_STACK, "walk stack overflow (tree deeper than the walk stack supports)");
    if (t_out) *t_out = c->blk_t;
    if (active_out) *active_out = cnt;
    return AG2_OK;
}

int run_kick(Ctx *c, double dt)
{
    AG2_LAUNCH(c, k_kick, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), dt);
    return AG2_OK;
}

int run_drift(Ctx *c, double dt)
{
    AG2_LAUNCH(c, k_drift, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), dt);
    c->have_tree = false;  // positions moved: the tree no longer describes them
    return AG2_OK;
}

int run_kick_drift(Ctx *c, double dt)
{
    AG2_LAUNCH(c, k_kick_drift, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), dt);
    c->have_tree = false;
    return AG2_OK;
}

int run_ueuler(Ctx *c, double dt)
{
    AG2_LAUNCH(c, k_ueuler, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), dt);
    return AG2_OK;
}

int run_scale(Ctx *c, double f)
{
    AG2_LAUNCH(c, k_scale, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), f);
    if (f != 1.0) c->have_tree = false;
    return AG2_OK;
}

int run_close_step(Ctx *c, double dt, double f)
{
    AG2_LAUNCH(c, k_close_step, grid_for(c->n, kBlock), kBlock, 0, (int)c->n, c->S(), dt, f);
    if (f != 1.0) c->have_tree = false;
    return AG2_OK;
}

}  // namespace ag2
