/*
 * ag2_oracle.h -- test-infrastructure API shared by the two CPU checkers of the
 * AstroGen2 force hot path:
 *
 *   liboracle.so       the plain-C restatement in ag2_oracle.c (builds anywhere);
 *   _ref/libag2ref.so  a harness that links the reference's own Tree/Node/kernel
 *                      sources (ref_harness.cpp, built only where those sources
 *                      exist).
 *
 * Both implement exactly this interface so that tests can run one against the
 * other.  Nothing in the product links either library: they are checkers only,
 * called from tests/, __graft_entry__.smoke() and bench.py's CPU legs.
 *
 * A "world" owns a copy of the particle state (the reference's Particle fields
 * that the hot path reads or writes, simulation/src/Physics/Particle.h:9-57) and
 * the tree built over it.  All quantities are FP64 in G = 1 code units.
 */
#ifndef AG2_ORACLE_H
#define AG2_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_world orc_world;

enum orc_field {
    ORC_POS = 0,   /* 3n: position             */
    ORC_VEL = 1,   /* 3n: velocity             */
    ORC_ACC = 2,   /* 3n: acc                  */
    ORC_MASS = 3,  /* n                        */
    ORC_H = 4,     /* n: smoothing length h    */
    ORC_RHO = 5,   /* n: rho                   */
    ORC_P = 6,     /* n: pressure              */
    ORC_T = 7,     /* n: temperature           */
    ORC_U = 8,     /* n: internal energy       */
    ORC_DUDT = 9,  /* n: dU/dt accumulator     */
    ORC_VDENS = 10 /* n: visualDensity         */
};

/* Create a world over n particles (copies the arrays; type: 1 star, 2 gas, 3 DM). */
orc_world *orc_create(int n, const double *pos, const double *vel, const double *mass,
                      const double *U, const uint8_t *type);
void orc_destroy(orc_world *w);

/* Gravitational constant the checker was built with (the reference harness is
 * built with G = 1; the restatement takes it from orc_set_G). */
double orc_get_G(void);
void orc_set_G(double G);

/* Tree::buildTree (Tree.cpp:24-55) with `threads` OpenMP threads; the
 * parallel/serial switch of Node::insert uses threads*100 (Node.cpp:420). */
int orc_build(orc_world *w, int threads);
/* Tree::calcVisualDensity (Tree.cpp:152-175). */
int orc_visual_density(orc_world *w, double visualDensityRadius);
/* Tree::calcGasDensity (Tree.cpp:119-150), single-threaded order. */
int orc_gas_density(orc_world *w, double massInH);
/* Tree::calculateForces (Tree.cpp:57-83) for every particle (all active). */
int orc_forces(orc_world *w, double e0, double theta, int threads);

/* The same walk for `ns` particles only (timing samples of the CPU baseline). */
int orc_forces_subset(orc_world *w, double e0, double theta, int threads, int ns, const int32_t *idx);

/* TimeIntegration (TimeIntegration.cpp:10-40) over all particles. */
void orc_kick(orc_world *w, double dt);
void orc_drift(orc_world *w, double dt);
void orc_ueuler(orc_world *w, double dt);
/* Hubble factor applied in Simulation::run (Simulation.cpp:330-332). */
void orc_scale_positions(orc_world *w, double factor);

void orc_get(orc_world *w, int field, double *out);
void orc_set(orc_world *w, int field, const double *in);

double orc_root_radius(orc_world *w);
/* Number of nodes of the current tree (all 8 children of every split node). */
int64_t orc_node_count(orc_world *w);
/* Export the tree in depth-first preorder, children 0..7.  Any pointer may be
 * NULL.  cp_count/cp_hash describe the node's childParticles multiset (count and
 * sum of orc_id_hash over the members, mod 2^64). */
void orc_topology(orc_world *w, int32_t *depth, int32_t *is_leaf, int32_t *particle,
                  int64_t *cp_count, uint64_t *cp_hash, double *mass, double *com3,
                  double *gas_mass, double *mvel3, double *center3, double *radius);
/* Preorder index of each particle's leaf node (Particle::node), -1 if none. */
void orc_leaf_index(orc_world *w, int64_t *out);

/* Hash used for membership digests (splitmix64 of id+1). */
uint64_t orc_id_hash(uint64_t id);

/* FP64 direct summation with the reference's softened pair law (Node.cpp:285-305)
 * for `ns` sample particles: out[3*k..] = acceleration of particle sample[k] due
 * to every other particle. */
void orc_direct_sum(int n, const double *pos, const double *mass, double e0, double G,
                    int ns, const int32_t *sample, double *out, int threads);

#ifdef __cplusplus
}
#endif
#endif
