// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Implements the checker interface of ag2_oracle.h on top of the reference's
// own, unmodified C++ sources (Tree, Node, kernel, vec3, TimeIntegration,
// Simulation), compiled by oracle/Makefile into oracle/_ref/libag2ref.so with
// the G = 1 shadow Constants.h.  It exists to pin the plain-C restatement in
// ag2_oracle.c against the reference itself and to generate the golden
// fixtures under tests/golden/; nothing in the product links it.
//
// Determinism settings (the reference's build and SPH density race above one
// thread): the caller chooses the OpenMP thread count of buildTree (its
// parallel/serial switch is threads*100, Node.cpp:420) and calcGasDensity runs
// with one thread.  Particles keep their array order (no init() shuffle).
#include "ag2_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "Simulation.h"
#include "Tree.h"
#include "TimeIntegration.h"
#include "DataManager.h"
#include "Log.h"

#include <unistd.h>

struct orc_world {
    Simulation *sim = nullptr;
    Tree *tree = nullptr;
    TimeIntegration ti;
    std::vector<Particle *> owned;
};

extern "C" {

double orc_get_G(void) { return Constants::G; }
void orc_set_G(double) {}

orc_world *orc_create(int n, const double *pos, const double *vel, const double *mass, const double *U,
                      const uint8_t *type)
{
    orc_world *w = new orc_world();
    w->sim = new Simulation();
    w->sim->numberOfParticles = n;
    w->sim->globalTime = 0.0;
    w->sim->e0 = 0.0;
    w->sim->theta = 0.5;
    w->sim->massInH = 0.0;
    w->sim->visualDensityRadius = 0.0;
    w->sim->H0 = 0.0;
    w->sim->particles.resize(n);
    for (int i = 0; i < n; i++) {
        Particle *p = new Particle();
        p->position = vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        if (vel) p->velocity = vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        p->mass = mass[i];
        p->type = type[i];
        if (U) p->U = U[i];
        p->id = (unsigned)i;
        p->node = nullptr;
        p->nextIntegrationTime = 0.0;
        w->sim->particles[i] = p;
        w->owned.push_back(p);
    }
    return w;
}

void orc_destroy(orc_world *w)
{
    if (!w) return;
    delete w->tree;
    for (Particle *p : w->owned) delete p;
    // The Simulation object is intentionally leaked: its destructor would not
    // free the particles either, and leaking keeps this harness independent of
    // the reference's shutdown path.
    delete w;
}

int orc_build(orc_world *w, int threads)
{
    delete w->tree;
    w->tree = nullptr;
    omp_set_num_threads(threads < 1 ? 1 : threads);
    w->tree = new Tree(w->sim);
    w->tree->buildTree();
    return 0;
}

int orc_visual_density(orc_world *w, double R)
{
    if (!w->tree) return -1;
    w->sim->visualDensityRadius = R;
    omp_set_num_threads(1);
    w->tree->calcVisualDensity();
    return 0;
}

int orc_gas_density(orc_world *w, double massInH)
{
    if (!w->tree) return -1;
    w->sim->massInH = massInH;
    omp_set_num_threads(1);
    w->tree->calcGasDensity();
    return 0;
}

int orc_forces(orc_world *w, double e0, double theta, int)
{
    if (!w->tree) return -1;
    w->sim->e0 = e0;
    w->sim->theta = theta;
    w->sim->globalTime = 0.0;
    for (Particle *p : w->sim->particles) p->nextIntegrationTime = 0.0;
    w->tree->calculateForces();
    return 0;
}

int orc_forces_subset(orc_world *w, double e0, double theta, int threads, int ns, const int32_t *idx)
{
    if (!w->tree) return -1;
    omp_set_num_threads(threads < 1 ? 1 : threads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int k = 0; k < ns; k++) {
        Particle *p = w->sim->particles[idx[k]];
        p->acc = vec3(0.0, 0.0, 0.0);
        w->tree->root->calculateGravityForce(p, e0, theta);
    }
    return 0;
}

void orc_kick(orc_world *w, double dt)
{
    for (Particle *p : w->sim->particles) w->ti.Kick(p, dt);
}

void orc_drift(orc_world *w, double dt)
{
    for (Particle *p : w->sim->particles) w->ti.Drift(p, dt);
}

void orc_ueuler(orc_world *w, double dt)
{
    for (Particle *p : w->sim->particles) w->ti.Ueuler(p, dt);
}

void orc_scale_positions(orc_world *w, double f)
{
    for (Particle *p : w->sim->particles) p->position *= f;
}

void orc_get(orc_world *w, int f, double *out)
{
    auto &ps = w->sim->particles;
    for (size_t i = 0; i < ps.size(); i++) {
        Particle *p = ps[i];
        switch (f) {
        case ORC_POS: out[3 * i] = p->position.x; out[3 * i + 1] = p->position.y; out[3 * i + 2] = p->position.z; break;
        case ORC_VEL: out[3 * i] = p->velocity.x; out[3 * i + 1] = p->velocity.y; out[3 * i + 2] = p->velocity.z; break;
        case ORC_ACC: out[3 * i] = p->acc.x; out[3 * i + 1] = p->acc.y; out[3 * i + 2] = p->acc.z; break;
        case ORC_MASS: out[i] = p->mass; break;
        case ORC_H: out[i] = p->h; break;
        case ORC_RHO: out[i] = p->rho; break;
        case ORC_P: out[i] = p->P; break;
        case ORC_T: out[i] = p->T; break;
        case ORC_U: out[i] = p->U; break;
        case ORC_DUDT: out[i] = p->dUdt; break;
        case ORC_VDENS: out[i] = p->visualDensity; break;
        }
    }
}

void orc_set(orc_world *w, int f, const double *in)
{
    auto &ps = w->sim->particles;
    for (size_t i = 0; i < ps.size(); i++) {
        Particle *p = ps[i];
        switch (f) {
        case ORC_POS: p->position = vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
        case ORC_VEL: p->velocity = vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
        case ORC_ACC: p->acc = vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
        case ORC_MASS: p->mass = in[i]; break;
        case ORC_H: p->h = in[i]; break;
        case ORC_RHO: p->rho = in[i]; break;
        case ORC_P: p->P = in[i]; break;
        case ORC_T: p->T = in[i]; break;
        case ORC_U: p->U = in[i]; break;
        case ORC_DUDT: p->dUdt = in[i]; break;
        case ORC_VDENS: p->visualDensity = in[i]; break;
        }
    }
}

double orc_root_radius(orc_world *w) { return (w->tree && w->tree->root) ? w->tree->root->radius : 0.0; }

// The reference's own step loop with block time steps: Simulation::run
// (Simulation.cpp:166-364) on the world's particles, which must carry their
// initial accelerations (orc_build + orc_forces, as Simulation::init computes
// them before run).  run() starts at globalTime 0, gives every particle its
// power-of-two step from |acc| (eta, min_dt, max_dt) and loops while
// globalTime < end_time: renew due steps, advance to the earliest next time,
// kick+drift, build, visual and gas density, walk, close (Ueuler, Hubble
// factor, kick).  Snapshots are switched off (fixedStep beyond end_time) and
// the phase log goes to logdir.  Inside run(), Tree::calculateForces sets the
// OpenMP thread count to std::thread::hardware_concurrency() (Tree.cpp:59-60),
// so every build after the first walk splits at 100 * that count; *cores
// returns it.  Outputs: the final globalTime, and per particle its time step
// and next integration time.
int orc_ref_run(orc_world *w, const char *logdir, double eta, double min_dt, double max_dt, double end_time,
                double e0, double theta, double massInH, double H0, double *global_time, double *tstep,
                double *tnext, int *cores)
{
    Simulation *s = w->sim;
    Log::setOutputDir(logdir);
    s->eta = eta;
    s->minTimeStep = min_dt;
    s->maxTimeStep = max_dt;
    s->endTime = end_time;
    s->fixedStep = 1e300;
    s->fixedTimeSteps = 1;
    s->numParticlesOutput = 0;
    s->e0 = e0;
    s->theta = theta;
    s->massInH = massInH;
    s->H0 = H0;
    s->starFormation = false;
    s->coolingEnabled = false;
    s->run();
    delete w->tree;  // run() built and deleted its own trees; the world's old one is stale
    w->tree = nullptr;
    *global_time = s->globalTime;
    for (size_t i = 0; i < s->particles.size(); i++) {
        tstep[i] = s->particles[i]->timeStep;
        tnext[i] = s->particles[i]->nextIntegrationTime;
    }
    *cores = (int)std::thread::hardware_concurrency();
    return 0;
}

static int64_t count_nodes(const Node *n)
{
    if (!n) return 0;
    int64_t c = 1;
    for (int i = 0; i < 8; i++) c += count_nodes(n->children[i]);
    return c;
}

int64_t orc_node_count(orc_world *w) { return (w->tree) ? count_nodes(w->tree->root) : 0; }

uint64_t orc_id_hash(uint64_t id)
{
    uint64_t z = id + 1 + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

namespace {
struct Export {
    int32_t *depth, *is_leaf, *particle;
    int64_t *cp_count;
    uint64_t *cp_hash;
    double *mass, *com3, *gas_mass, *mvel3, *center3, *radius;
    int64_t k = 0;
};

void export_rec(const Node *n, Export &e)
{
    int64_t k = e.k++;
    if (e.depth) e.depth[k] = n->depth;
    if (e.is_leaf) e.is_leaf[k] = n->isLeaf ? 1 : 0;
    if (e.particle) e.particle[k] = n->particle ? (int32_t)n->particle->id : -1;
    if (e.cp_count) e.cp_count[k] = (int64_t)n->childParticles.size();
    if (e.cp_hash) {
        uint64_t h = 0;
        for (const Particle *p : n->childParticles) h += orc_id_hash(p->id);
        e.cp_hash[k] = h;
    }
    if (e.mass) e.mass[k] = n->mass;
    if (e.com3) { e.com3[3 * k] = n->centerOfMass.x; e.com3[3 * k + 1] = n->centerOfMass.y; e.com3[3 * k + 2] = n->centerOfMass.z; }
    if (e.gas_mass) e.gas_mass[k] = n->gasMass;
    if (e.mvel3) { e.mvel3[3 * k] = n->mVel.x; e.mvel3[3 * k + 1] = n->mVel.y; e.mvel3[3 * k + 2] = n->mVel.z; }
    if (e.center3) { e.center3[3 * k] = n->position.x; e.center3[3 * k + 1] = n->position.y; e.center3[3 * k + 2] = n->position.z; }
    if (e.radius) e.radius[k] = n->radius;
    for (int i = 0; i < 8; i++)
        if (n->children[i]) export_rec(n->children[i], e);
}

void index_rec(const Node *n, int64_t &k, std::vector<std::pair<const Node *, int64_t>> &out)
{
    out.push_back({n, k++});
    for (int i = 0; i < 8; i++)
        if (n->children[i]) index_rec(n->children[i], k, out);
}
} // namespace

void orc_topology(orc_world *w, int32_t *depth, int32_t *is_leaf, int32_t *particle, int64_t *cp_count,
                  uint64_t *cp_hash, double *mass, double *com3, double *gas_mass, double *mvel3, double *center3,
                  double *radius)
{
    if (!w->tree || !w->tree->root) return;
    Export e{depth, is_leaf, particle, cp_count, cp_hash, mass, com3, gas_mass, mvel3, center3, radius};
    export_rec(w->tree->root, e);
}

void orc_leaf_index(orc_world *w, int64_t *out)
{
    auto &ps = w->sim->particles;
    for (size_t i = 0; i < ps.size(); i++) out[i] = -1;
    if (!w->tree || !w->tree->root) return;
    std::vector<std::pair<const Node *, int64_t>> idx;
    int64_t k = 0;
    index_rec(w->tree->root, k, idx);
    std::vector<std::pair<const Node *, int64_t>> sorted(idx);
    std::sort(sorted.begin(), sorted.end());
    for (size_t i = 0; i < ps.size(); i++) {
        const Node *n = ps[i]->node;
        if (!n) continue;
        auto it = std::lower_bound(sorted.begin(), sorted.end(), std::make_pair(n, (int64_t)-1));
        if (it != sorted.end() && it->first == n) out[i] = it->second;
    }
}

void orc_direct_sum(int n, const double *pos, const double *mass, double e0, double, int ns, const int32_t *sample,
                    double *out, int threads)
{
    // Pair force through the reference's own leaf branch of
    // Node::calculateGravityForce (Node.cpp:279-313): one temporary leaf per
    // source particle.
    std::vector<Particle> parts(n);
    for (int j = 0; j < n; j++) {
        parts[j].position = vec3(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]);
        parts[j].mass = mass[j];
        parts[j].type = 1;
        parts[j].h = 0;
        parts[j].node = nullptr;
    }
    omp_set_num_threads(threads < 1 ? 1 : threads);
#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < ns; k++) {
        Particle probe = parts[sample[k]];
        probe.acc = vec3(0, 0, 0);
        Node leaf;
        for (int j = 0; j < n; j++) {
            if (j == sample[k] || mass[j] == 0) continue;
            leaf.isLeaf = true;
            leaf.particle = &parts[j];
            leaf.centerOfMass = parts[j].position;
            leaf.mass = parts[j].mass;
            leaf.calculateGravityForce(&probe, e0, 0.0);
        }
        leaf.particle = nullptr;
        out[3 * k] = probe.acc.x;
        out[3 * k + 1] = probe.acc.y;
        out[3 * k + 2] = probe.acc.z;
    }
}

// DataManager::saveData on particles given as arrays (upload order): writes
// <dir><timeStep>.<format> exactly as the reference does.
int orc_ref_save(const char *dir, const char *format, int n, int count, const double *pos, const double *vel,
                 const double *mass, const double *T, const double *P, const double *vdens, const double *U,
                 const double *sfr, const uint8_t *type, const uint8_t *gp, const uint32_t *id, int timeStep,
                 double dt, double endTime, double t)
{
    DataManager dm(dir);
    dm.outputFormat = format;
    std::vector<Particle *> ps(n);
    for (int i = 0; i < n; i++) {
        Particle *q = new Particle();
        q->position = vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        q->velocity = vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        q->mass = mass[i];
        q->T = T[i];
        q->P = P[i];
        q->visualDensity = vdens[i];
        q->U = U[i];
        q->sfr = sfr[i];
        q->type = type[i];
        q->galaxyPart = gp[i];
        q->id = id[i];
        ps[i] = q;
    }
    dm.saveData(ps, timeStep, 0, count, dt, endTime, t);
    for (Particle *q : ps) delete q;
    return 0;
}

// DataManager::loadICs of <workdir>/../../input_data/<name>: the reader opens
// "../../input_data/" + inputPath relative to the working directory, which is
// switched to workdir for the call.  Copies up to cap particles out, returns
// their number and sets *ok to the reader's return value (its makeGal branch
// fills the particles and then returns false, DataManager.cpp:580-809, 1331).
int orc_ref_load(const char *workdir, const char *name, const char *format, int cap, double *pos, double *vel,
                 double *mass, double *T, double *P, double *vdens, double *U, double *sfr, uint8_t *type,
                 uint8_t *gp, uint32_t *id, int *ok_out)
{
    char old[4096];
    if (!getcwd(old, sizeof old) || chdir(workdir) != 0) return -2;
    DataManager dm("");
    dm.inputPath = name;
    dm.inputFormat = format;
    Simulation *sim = new Simulation();
    std::vector<Particle *> ps;
    const bool ok = dm.loadICs(ps, sim);
    if (chdir(old) != 0) return -2;
    *ok_out = ok ? 1 : 0;
    const int n = (int)ps.size();
    for (int i = 0; i < n && i < cap; i++) {
        const Particle *q = ps[i];
        pos[3 * i] = q->position.x;
        pos[3 * i + 1] = q->position.y;
        pos[3 * i + 2] = q->position.z;
        vel[3 * i] = q->velocity.x;
        vel[3 * i + 1] = q->velocity.y;
        vel[3 * i + 2] = q->velocity.z;
        mass[i] = q->mass;
        T[i] = q->T;
        P[i] = q->P;
        vdens[i] = q->visualDensity;
        U[i] = q->U;
        sfr[i] = q->sfr;
        type[i] = q->type;
        gp[i] = q->galaxyPart;
        id[i] = q->id;
    }
    for (Particle *q : ps) delete q;
    return n;
}

} // extern "C"
