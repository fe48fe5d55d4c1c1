// A miniature of the reference's step loop (Simulation.cpp:256-341) driving
// ag2host::Tree / ag2host::TimeIntegration, the drop-in for the reference's
// Tree and TimeIntegration classes.  The Particle / Simulation structs carry the
// fields the reference's loop uses on this path.
//
// usage: shim_demo <in.bin> <out.bin> <steps>
//   in.bin : int64 n, then n*(pos3, vel3, mass, U) doubles and n uint8 types,
//            then e0, theta, massInH, dt
//   out.bin: n*(pos3, vel3, acc3, h, rho, U) doubles after the steps
#include <cstdint>
#include <cstdio>
#include <vector>

#include "ag2_tree.hpp"

struct vec3 {
    double x = 0, y = 0, z = 0;
};

struct Particle {
    vec3 position, velocity, acc;
    double mass = 0, h = 0, rho = 0, P = 0, T = 0, U = 0, dUdt = 0, visualDensity = 0;
    uint8_t type = 1;
};

struct Simulation {
    std::vector<Particle *> particles;
    int numberOfParticles = 0;
    double e0 = 0.01, theta = 0.5, massInH = 0, visualDensityRadius = 0;
};

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int64_t n = 0;
    if (std::fread(&n, 8, 1, f) != 1) return 3;
    std::vector<double> rec(8 * n);
    std::vector<uint8_t> type(n);
    double prm[4];
    if (std::fread(rec.data(), 8, rec.size(), f) != rec.size() || std::fread(type.data(), 1, n, f) != (size_t)n ||
        std::fread(prm, 8, 4, f) != 4)
        return 3;
    std::fclose(f);
    Simulation sim;
    std::vector<Particle> store(n);
    for (int64_t i = 0; i < n; i++) {
        Particle &p = store[i];
        p.position = {rec[8 * i], rec[8 * i + 1], rec[8 * i + 2]};
        p.velocity = {rec[8 * i + 3], rec[8 * i + 4], rec[8 * i + 5]};
        p.mass = rec[8 * i + 6];
        p.U = rec[8 * i + 7];
        p.type = type[i];
        sim.particles.push_back(&p);
    }
    sim.numberOfParticles = (int)n;
    sim.e0 = prm[0];
    sim.theta = prm[1];
    sim.massInH = prm[2];
    const double dt = prm[3];
    const int steps = std::atoi(argv[3]);
    ag2host::TimeIntegration ti;
    {
        // initial forces (Simulation.cpp:120-139)
        ag2host::Tree<Simulation> tree(&sim);
        tree.buildTree();
        sim.visualDensityRadius = tree.root->radius / 100000;  // Simulation.cpp:126
        tree.calcVisualDensity();
        tree.calcGasDensity();
        tree.calculateForces();
    }
    for (int s = 0; s < steps; s++) {
        for (Particle *p : sim.particles) {
            ti.Kick(p, dt);
            ti.Drift(p, dt);
        }
        auto *tree = new ag2host::Tree<Simulation>(&sim);
        tree->buildTree();
        tree->calcGasDensity();
        tree->calculateForces();
        for (Particle *p : sim.particles) {
            if (p->type == 2) ti.Ueuler(p, dt);
            ti.Kick(p, dt);
        }
        delete tree;
    }
    if (ag2host::last_status() != AG2_OK) return 4;
    FILE *g = std::fopen(argv[2], "wb");
    for (Particle *p : sim.particles) {
        double o[12] = {p->position.x, p->position.y, p->position.z, p->velocity.x, p->velocity.y, p->velocity.z,
                        p->acc.x,      p->acc.y,      p->acc.z,      p->h,          p->rho,        p->U};
        std::fwrite(o, 8, 12, g);
    }
    std::fclose(g);
    return 0;
}
