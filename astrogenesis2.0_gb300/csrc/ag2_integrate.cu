// ag2_integrate.cu -- leapfrog kick/drift and internal-energy update.
//
// Reference: simulation/src/Physics/TimeIntegration.cpp:10-40 (Kick, Drift,
// Ueuler) and the step loop in simulation/src/Physics/Simulation.cpp:256-341
// (Hubble factor at :330-332).  The arithmetic is written in the reference's
// operation order with explicitly rounded FP64 operations, so the results are
// bit-identical to the reference's for the same inputs.
#include "ag2_internal.cuh"

namespace ag2 {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ bool acc_nan(const Particles &s, int i)
{
    return isnan(s.ax[i]) || isnan(s.ay[i]) || isnan(s.az[i]);
}

// v = v + a*dt/2, skipped when acc has a NaN (TimeIntegration.cpp:12-18)
__device__ __forceinline__ void kick1(Particles &s, int i, double dt)
{
    if (acc_nan(s, i)) return;
    s.vx[i] = __dadd_rn(s.vx[i], __ddiv_rn(__dmul_rn(s.ax[i], dt), 2.0));
    s.vy[i] = __dadd_rn(s.vy[i], __ddiv_rn(__dmul_rn(s.ay[i], dt), 2.0));
    s.vz[i] = __dadd_rn(s.vz[i], __ddiv_rn(__dmul_rn(s.az[i], dt), 2.0));
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
    s.px[i] = __dmul_rn(s.px[i], f);
    s.py[i] = __dmul_rn(s.py[i], f);
    s.pz[i] = __dmul_rn(s.pz[i], f);
    kick1(s, i, dt);
}

}  // namespace

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
