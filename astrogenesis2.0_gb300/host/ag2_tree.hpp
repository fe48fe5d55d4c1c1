// ag2_tree.hpp -- C++ drop-in for the reference's Tree and TimeIntegration
// classes (simulation/src/Physics/Tree/Tree.h:13-27,
// simulation/src/Physics/TimeIntegration.h:6-22), built on the C-ABI of
// include/ag2.h.
//
// The reference's integrator keeps its particles on the host as a
// std::vector<Particle*> and calls, every step (Simulation.cpp:267-336):
//
//   timeIntegration->Kick(p, dt); timeIntegration->Drift(p, dt);   // per particle
//   Tree* tree = new Tree(this);
//   tree->buildTree(); tree->calcVisualDensity(); tree->calcGasDensity();
//   tree->calculateForces();
//   timeIntegration->Ueuler(p, dt); ...; timeIntegration->Kick(p, dt);
//   delete tree;
//
// ag2host::Tree<Simulation> has the same constructor and methods.  buildTree()
// uploads the particles' position, velocity, mass, U and type to the GPU and
// builds the octree there; calcVisualDensity / calcGasDensity / calculateForces
// run on the device and write visualDensity / h, rho, P, T / acc, dUdt back
// into the Particle records, which is all the reference's loop reads.  The
// device context is shared by all Tree objects of one Simulation (a new Tree per
// step does not reallocate).  TimeIntegration keeps the reference's per-particle
// host arithmetic (a handful of FP64 operations per particle), bit for bit.
//
// Errors: the reference's methods return void and print to std::cerr; these do
// the same and additionally remember the last status (ag2host::last_status()).
//
// Requirements on the templates' arguments (the reference's own types satisfy
// them): Sim has `std::vector<P*> particles`, `int numberOfParticles`,
// `double e0, theta, massInH, visualDensityRadius`; P has `vec3 position,
// velocity, acc` (members x, y, z), `double mass, h, rho, P, T, U, dUdt,
// visualDensity` and `uint8_t type`.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <filesystem>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "ag2.h"

namespace ag2host {

inline int &last_status_ref()
{
    static thread_local int s = AG2_OK;
    return s;
}
inline int last_status() { return last_status_ref(); }

// One device context per simulation object, grown when the particle count grows.
struct DeviceState {
    ag2_ctx *ctx = nullptr;
    size_t cap = 0;
    ~DeviceState()
    {
        if (ctx) ag2_destroy(ctx);
    }
};

template <class Sim>
DeviceState &device_state(const Sim *sim)
{
    // keyed by the simulation's address; the reference creates one Simulation
    static thread_local const void *owner = nullptr;
    static thread_local std::unique_ptr<DeviceState> st;
    if (owner != static_cast<const void *>(sim) || !st) {
        st.reset(new DeviceState());
        owner = sim;
    }
    return *st;
}

// What the integrator reads of the root node (Simulation.cpp:123-126:
// tree->root->radius for the initial size and visualDensityRadius).
struct RootInfo {
    double radius = 0.0;
};

template <class Sim>
class Tree {
public:
    explicit Tree(Sim *sim) : simulation(sim) {}
    ~Tree() = default;
    Tree(const Tree &) = delete;
    Tree &operator=(const Tree &) = delete;

    Sim *simulation;
    RootInfo *root = &root_info_;  // valid after buildTree

    // Tree::buildTree (Tree.cpp:24-55)
    void buildTree()
    {
        if (!ensure()) return;
        auto &ps = simulation->particles;
        const size_t n = ps.size();
        pos_.resize(3 * n);
        vel_.resize(3 * n);
        mass_.resize(n);
        U_.resize(n);
        type_.resize(n);
        for (size_t i = 0; i < n; i++) {
            const auto *p = ps[i];
            pos_[3 * i] = p->position.x;
            pos_[3 * i + 1] = p->position.y;
            pos_[3 * i + 2] = p->position.z;
            vel_[3 * i] = p->velocity.x;
            vel_[3 * i + 1] = p->velocity.y;
            vel_[3 * i + 2] = p->velocity.z;
            mass_[i] = p->mass;
            U_[i] = p->U;
            type_[i] = p->type;
        }
        if (!check(ag2_upload(ctx(), n, pos_.data(), vel_.data(), mass_.data(), U_.data(), type_.data()),
                   "buildTree"))
            return;
        // dUdt accumulates across calculateForces calls until Ueuler consumes it
        dudt_.resize(n);
        for (size_t i = 0; i < n; i++) dudt_[i] = ps[i]->dUdt;
        if (!check(ag2_set_field(ctx(), AG2_DUDT, dudt_.data(), 0), "buildTree")) return;
        if (!check(ag2_build_tree(ctx()), "buildTree")) return;
        check(ag2_root_radius(ctx(), &root_info_.radius), "buildTree");
    }

    // Tree::calculateForces (Tree.cpp:57-83): acc and dUdt of every particle
    void calculateForces()
    {
        if (!sync_params()) return;
        if (!check(ag2_forces(ctx()), "calculateForces")) return;
        auto &ps = simulation->particles;
        const size_t n = ps.size();
        acc_.resize(3 * n);
        dudt_.resize(n);
        if (!check(ag2_download(ctx(), AG2_ACC, acc_.data(), 0), "calculateForces")) return;
        if (!check(ag2_download(ctx(), AG2_DUDT, dudt_.data(), 0), "calculateForces")) return;
        for (size_t i = 0; i < n; i++) {
            auto *p = ps[i];
            p->acc.x = acc_[3 * i];
            p->acc.y = acc_[3 * i + 1];
            p->acc.z = acc_[3 * i + 2];
            p->dUdt = dudt_[i];
        }
    }

    // Tree::calcTreeWidth (Tree.cpp:86-117); valid after buildTree
    double calcTreeWidth()
    {
        double r = 0.0;
        check(ag2_root_radius(ctx(), &r), "calcTreeWidth");
        return r;
    }

    // Tree::calcVisualDensity (Tree.cpp:152-175)
    void calcVisualDensity()
    {
        if (!check(ag2_visual_density(ctx(), simulation->visualDensityRadius), "calcVisualDensity")) return;
        pull(AG2_VDENS, [](auto *p, double v) { p->visualDensity = v; });
    }

    // Tree::calcGasDensity (Tree.cpp:119-150)
    void calcGasDensity()
    {
        if (!sync_params()) return;
        if (!check(ag2_sph_density(ctx()), "calcGasDensity")) return;
        pull(AG2_H, [](auto *p, double v) { p->h = v; });
        pull(AG2_RHO, [](auto *p, double v) { p->rho = v; });
        pull(AG2_P, [](auto *p, double v) { p->P = v; });
        pull(AG2_T, [](auto *p, double v) { p->T = v; });
    }

private:
    RootInfo root_info_;
    std::vector<double> pos_, vel_, mass_, U_, acc_, dudt_, tmp_;
    std::vector<uint8_t> type_;

    ag2_ctx *ctx() { return device_state(simulation).ctx; }

    bool check(int rc, const char *what)
    {
        last_status_ref() = rc;
        if (rc != AG2_OK) {
            std::cerr << "Error (" << what << "): " << ag2_last_error_string(ctx()) << " (status " << rc << ")"
                      << std::endl;
            return false;
        }
        return true;
    }

    bool ensure()
    {
        DeviceState &d = device_state(simulation);
        const size_t n = simulation->particles.size();
        if (d.ctx && d.cap >= n) return sync_params();
        if (d.ctx) ag2_destroy(d.ctx);
        d.ctx = nullptr;
        ag2_params p;
        ag2_default_params(&p);
        fill(p);
        int rc = ag2_create(&d.ctx, &p, n ? n : 1);
        last_status_ref() = rc;
        if (rc != AG2_OK) {
            std::cerr << "Error (buildTree): cannot create the device context (status " << rc << ")" << std::endl;
            d.ctx = nullptr;
            return false;
        }
        d.cap = n ? n : 1;
        return true;
    }

    void fill(ag2_params &p)
    {
        p.e0 = simulation->e0;
        p.theta = simulation->theta;
        p.massInH = simulation->massInH;
    }

    bool sync_params()
    {
        ag2_params p;
        if (ag2_get_params(ctx(), &p) != AG2_OK) return false;
        fill(p);
        return check(ag2_set_params(ctx(), &p), "parameters");
    }

    template <class F>
    void pull(int field, F set)
    {
        auto &ps = simulation->particles;
        tmp_.resize(ps.size());
        if (!check(ag2_download(ctx(), field, tmp_.data(), 0), "download")) return;
        for (size_t i = 0; i < ps.size(); i++) set(ps[i], tmp_[i]);
    }
};

// TimeIntegration (TimeIntegration.cpp:10-40), same per-particle arithmetic.
class TimeIntegration {
public:
    template <class P>
    void Kick(P *particle, double deltaTime)
    {
        if (std::isnan(particle->acc.x) || std::isnan(particle->acc.y) || std::isnan(particle->acc.z)) return;
        particle->velocity.x = particle->velocity.x + particle->acc.x * deltaTime / 2;
        particle->velocity.y = particle->velocity.y + particle->acc.y * deltaTime / 2;
        particle->velocity.z = particle->velocity.z + particle->acc.z * deltaTime / 2;
    }
    template <class P>
    void Drift(P *particle, double deltaTime)
    {
        particle->position.x = particle->position.x + particle->velocity.x * deltaTime;
        particle->position.y = particle->position.y + particle->velocity.y * deltaTime;
        particle->position.z = particle->position.z + particle->velocity.z * deltaTime;
    }
    template <class P>
    void Ueuler(P *particle, double deltaTime)
    {
        if (!particle) return;
        if (!std::isnan(particle->dUdt)) particle->U += particle->dUdt * deltaTime;
        particle->dUdt = 0;
    }
};

// DataManager's formats by the names of its outputDataFormat / inputDataFormat
// keys (DataManager.cpp:100-110, 446-580); -1 for anything else ("hdf5" is not
// implemented by the reference either).
inline int format_code(const std::string &name)
{
    if (name == "ag") return AG2_FMT_AG;
    if (name == "agc") return AG2_FMT_AGC;
    if (name == "age") return AG2_FMT_AGE;
    if (name == "gadget") return AG2_FMT_GADGET;
    if (name == "makeGal") return AG2_FMT_MAKEGAL;
    return -1;
}

// DataManager::saveData (DataManager.cpp:86-118) for an engine whose particles
// are resident in a context: creates outputPath if needed and writes
// outputPath + std::to_string(timeStep) + "." + outputFormat holding the first
// numberOfParticles particles; with async the file is written in the
// background (ag2_snapshot_wait collects the status).
inline int save_snapshot(ag2_ctx *ctx, const std::string &outputPath, const std::string &outputFormat, int timeStep,
                         int numberOfParticles, double deltaTime, double endTime, double currentTime,
                         bool async = true)
{
    const int fmt = format_code(outputFormat);
    if (fmt < 0 || fmt == AG2_FMT_MAKEGAL) {
        std::cerr << "Unknown output data format: " << outputFormat << std::endl;
        return last_status_ref() = AG2_E_FORMAT;
    }
    std::error_code ec;
    std::filesystem::create_directories(outputPath, ec);
    const std::string file = outputPath + std::to_string(timeStep) + "." + outputFormat;
    const int64_t count = std::min<int64_t>(numberOfParticles, (int64_t)ag2_count(ctx));
    const int rc = ag2_snapshot_write(ctx, fmt, count, deltaTime, endTime, currentTime, file.c_str(), async ? 1 : 0);
    if (rc != AG2_OK) std::cerr << "Error opening datafile: " << file << " (" << ag2_last_error_string(ctx) << ")" << std::endl;
    return last_status_ref() = rc;
}

// DataManager::loadICs (DataManager.cpp:434-1332) into a context.  The
// reference opens "../../input_data/" + inputPath; pass the resolved path.
inline int load_ics(ag2_ctx *ctx, const std::string &path, const std::string &inputFormat)
{
    const int fmt = format_code(inputFormat);
    if (fmt < 0) {
        std::cout << "invalid input data format: " << inputFormat << std::endl;
        return last_status_ref() = AG2_E_FORMAT;
    }
    const int rc = ag2_load_ics(ctx, path.c_str(), fmt, nullptr);
    if (rc != AG2_OK) std::cerr << "Error reading initial conditions " << path << ": " << ag2_last_error_string(ctx) << std::endl;
    return last_status_ref() = rc;
}

}  // namespace ag2host
