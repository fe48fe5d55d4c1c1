/*
 * ag2_oracle.c -- CPU restatement of the AstroGen2 force hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against, and the timed CPU baseline of bench.py.  It is never linked
 * into, or called by, the product library.
 *
 * It restates, function by function, the reference's pointer octree
 * (simulation/src/Physics/Tree/Node.cpp, Tree.cpp), its kernels
 * (simulation/src/Math/kernel.cpp) and its leapfrog
 * (simulation/src/Physics/TimeIntegration.cpp).  Each routine cites the lines
 * it follows.  Floating-point operations are written in the reference's order
 * and the file is compiled with -ffp-contract=off, so that on the same inputs it
 * reproduces the reference harness (ref_harness.cpp) to the last bit on x86-64;
 * the parity pin lives in tests/test_oracle_golden.py.
 *
 * Deliberate differences from the reference, all of them fixes of data races
 * that make the reference nondeterministic above one thread:
 *   - the SPH density sum (Node.cpp:771-779) is a plain sequential sum;
 *   - the parallel partition (Node.cpp:465-506) uses contiguous static chunks so
 *     that every child receives its particles in array order, and the gas
 *     velocity mean of that partition is taken as a mass-weighted sum.
 * At threads = 1 neither difference is visible.
 */
#include "ag2_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* SI constants as in simulation/src/Math/Constants.h:7-15 (G is a parameter here). */
#define ORC_PI 3.14159265358979323846
#define ORC_GAMMA (5.0 / 3.0)
#define ORC_KB 1.38064852e-23
#define ORC_PRTN 1.6726219e-27

static double g_G = 1.0;
double orc_get_G(void) { return g_G; }
void orc_set_G(double G) { g_G = G; }

/* ------------------------------------------------------------------------- */
/* Node (simulation/src/Physics/Tree/Node.h:10-57)                            */
/* ------------------------------------------------------------------------- */
typedef struct onode {
    double pos[3]; /* geometric centre ("position") */
    double radius; /* half width */
    double com[3];
    double mass;
    double gasMass;
    double mVel[3];
    int depth;
    int isLeaf;
    int particle; /* index, -1 = none */
    struct onode *children[8];
    struct onode *parent;
    int *cp; /* childParticles */
    int ncp, capcp;
} onode;

struct orc_world {
    int n;
    double *x, *v, *a, *m, *h, *rho, *P, *T, *U, *dUdt, *mu, *vdens;
    uint8_t *type;
    onode **node; /* Particle::node */
    onode *root;
};

static onode *node_new(void)
{
    /* Node::Node (Node.cpp:13-29): leaf, no particle, zero mass and radius. */
    onode *n = (onode *)calloc(1, sizeof(onode));
    n->isLeaf = 1;
    n->particle = -1;
    return n;
}

static void node_free(onode *n)
{
    if (!n) return;
    for (int i = 0; i < 8; i++) node_free(n->children[i]);
    free(n->cp);
    free(n);
}

static void cp_push(onode *n, int p)
{
    if (n->ncp == n->capcp) {
        n->capcp = n->capcp ? 2 * n->capcp : 4;
        n->cp = (int *)realloc(n->cp, sizeof(int) * (size_t)n->capcp);
    }
    n->cp[n->ncp++] = p;
}

static void make_children(onode *n)
{
    /* Child centres c + r*(+-0.5), radius r/2 (Node.cpp:433-443, 630-642). */
    for (int i = 0; i < 8; i++) {
        onode *c = node_new();
        c->pos[0] = n->pos[0] + n->radius * ((i & 1) ? 0.5 : -0.5);
        c->pos[1] = n->pos[1] + n->radius * ((i & 2) ? 0.5 : -0.5);
        c->pos[2] = n->pos[2] + n->radius * ((i & 4) ? 0.5 : -0.5);
        c->radius = n->radius / 2;
        c->depth = n->depth + 1;
        c->parent = n;
        n->children[i] = c;
    }
}

static int out_of_bounds(const onode *n, const double *x)
{
    /* Inclusive bounds test of Node::insert(Particle*) / getOctant (Node.cpp:606-608, 706-708). */
    return x[0] < n->pos[0] - n->radius || x[0] > n->pos[0] + n->radius ||
           x[1] < n->pos[1] - n->radius || x[1] > n->pos[1] + n->radius ||
           x[2] < n->pos[2] - n->radius || x[2] > n->pos[2] + n->radius;
}

static int get_octant(const onode *n, const double *x)
{
    /* Node::getOctant (Node.cpp:702-719). */
    if (out_of_bounds(n, x)) return -1;
    int o = 0;
    if (x[0] > n->pos[0]) o |= 1;
    if (x[1] > n->pos[1]) o |= 2;
    if (x[2] > n->pos[2]) o |= 4;
    return o;
}

/* Node::insert(Particle*) (Node.cpp:597-699): serial one-particle insertion. */
static void insert_one(orc_world *w, onode *n, int p)
{
    const double *x = w->x + 3 * (size_t)p;
    if (out_of_bounds(n, x)) return; /* dropped (Node.cpp:606-612) */
    cp_push(n, p);                   /* Node.cpp:615 */
    if (n->isLeaf) {
        if (n->particle < 0) {
            n->particle = p;
            w->node[p] = n;
        } else {
            make_children(n);
            int q = n->particle;
            int o = get_octant(n, w->x + 3 * (size_t)q);
            if (o != -1) insert_one(w, n->children[o], q);
            o = get_octant(n, x);
            if (o != -1) insert_one(w, n->children[o], p);
            n->isLeaf = 0;
            n->particle = -1;
        }
    } else {
        int o = get_octant(n, x);
        if (o != -1) insert_one(w, n->children[o], p);
    }
    double mp = w->m[p];
    n->mass += mp;
    if (w->type[p] == 2) {
        n->gasMass += mp;
        if (n->gasMass > 0) {
            const double *v = w->v + 3 * (size_t)p;
            double f = n->gasMass - mp;
            for (int k = 0; k < 3; k++) n->mVel[k] = (n->mVel[k] * f + v[k] * mp) / n->gasMass;
        }
    }
    double f = n->mass - mp;
    for (int k = 0; k < 3; k++) n->com[k] = (n->com[k] * f + x[k] * mp) / n->mass;
}

/* Node::insert(const std::vector<Particle*>, int cores) (Node.cpp:405-534). */
static void insert_vec(orc_world *w, onode *n, const int *list, int cnt, int cores)
{
    if (cnt == 0) return;
    if (cnt == 1) { /* Node.cpp:409-418 */
        int p = list[0];
        n->isLeaf = 1;
        n->particle = p;
        w->node[p] = n;
        memcpy(n->com, w->x + 3 * (size_t)p, 3 * sizeof(double));
        n->mass = w->m[p];
        n->gasMass = (w->type[p] == 2) ? w->m[p] : 0.0;
        return;
    }
    if (cnt < cores * 100) { /* Node.cpp:420-428 */
        for (int i = 0; i < cnt; i++) insert_one(w, n, list[i]);
        return;
    }
    n->isLeaf = 0;
    make_children(n);

    /* Sums over every particle of the list, including those that fall outside
     * this node (Node.cpp:465-506), then the octant partition. */
    int nt = cores > 0 ? cores : 1;
    if (nt > cnt) nt = cnt;
    double *part = (double *)calloc((size_t)nt * 8, sizeof(double));
    int *counts = (int *)calloc((size_t)nt * 8, sizeof(int));
    int *oct = (int *)malloc(sizeof(int) * (size_t)cnt);
    if (n->depth == 0)
        for (int i = 0; i < cnt; i++) w->node[list[i]] = NULL; /* Node.cpp:472 */

    if (nt == 1) {
        /* One thread: the reference's running gas-velocity mean, in list order. */
        double tm = 0, tg = 0, sx = 0, sy = 0, sz = 0;
        for (int i = 0; i < cnt; i++) {
            int p = list[i];
            double mp = w->m[p];
            const double *x = w->x + 3 * (size_t)p;
            tm += mp;
            if (w->type[p] == 2) {
                tg += mp;
                n->gasMass += mp;
                if (n->gasMass > 0) {
                    const double *v = w->v + 3 * (size_t)p;
                    double f = n->gasMass - mp;
                    for (int k = 0; k < 3; k++) n->mVel[k] = (n->mVel[k] * f + v[k] * mp) / n->gasMass;
                }
            }
            sx += x[0] * mp;
            sy += x[1] * mp;
            sz += x[2] * mp;
            oct[i] = get_octant(n, x);
        }
        part[0] = tm; part[1] = tg; part[2] = sx; part[3] = sy; part[4] = sz;
    } else {
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
        {
#ifdef _OPENMP
            int t = omp_get_thread_num();
#else
            int t = 0;
#endif
            int lo = (int)((int64_t)cnt * t / nt), hi = (int)((int64_t)cnt * (t + 1) / nt);
            double tm = 0, tg = 0, sx = 0, sy = 0, sz = 0, gv[3] = {0, 0, 0};
            for (int i = lo; i < hi; i++) {
                int p = list[i];
                double mp = w->m[p];
                const double *x = w->x + 3 * (size_t)p;
                tm += mp;
                if (w->type[p] == 2) {
                    tg += mp;
                    for (int k = 0; k < 3; k++) gv[k] += w->v[3 * (size_t)p + k] * mp;
                }
                sx += x[0] * mp;
                sy += x[1] * mp;
                sz += x[2] * mp;
                oct[i] = get_octant(n, x);
            }
            double *q = part + 8 * t;
            q[0] = tm; q[1] = tg; q[2] = sx; q[3] = sy; q[4] = sz;
            q[5] = gv[0]; q[6] = gv[1]; q[7] = gv[2];
        }
        double gv[3] = {0, 0, 0};
        for (int t = 1; t < nt; t++)
            for (int k = 0; k < 8; k++) part[k] += part[8 * t + k];
        gv[0] = part[5]; gv[1] = part[6]; gv[2] = part[7];
        if (part[1] > 0)
            for (int k = 0; k < 3; k++) n->mVel[k] = gv[k] / part[1];
    }
    n->mass = 0.0 + part[0];
    n->gasMass = 0.0 + part[1];
    if (n->mass > 0.0) {
        n->com[0] = (0.0 + part[2]) / n->mass;
        n->com[1] = (0.0 + part[3]) / n->mass;
        n->com[2] = (0.0 + part[4]) / n->mass;
    }
    /* Partition in list order (Node.cpp:515-522 with contiguous chunks). */
    for (int i = 0; i < cnt; i++)
        if (oct[i] >= 0) cp_push(n->children[oct[i]], list[i]);
    free(oct);
    free(counts);
    free(part);

    for (int i = 0; i < 8; i++) { /* Node.cpp:526-532: the child gets a copy of its list */
        onode *c = n->children[i];
        if (c->ncp > 0) {
            int cc = c->ncp;
            int *copy = (int *)malloc(sizeof(int) * (size_t)cc);
            memcpy(copy, c->cp, sizeof(int) * (size_t)cc);
            insert_vec(w, c, copy, cc, cores);
            free(copy);
        }
    }
}

/* Tree::calcTreeWidth (Tree.cpp:86-117). */
static double tree_width(const orc_world *w)
{
    int n = w->n;
    if (n == 0) return 0;
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) {
        const double *x = w->x + 3 * (size_t)i;
        d[i] = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    }
    double sum = 0.0;
    for (int i = 0; i < n; i++) sum = sum + d[i];
    double mean = sum / n;
    double sq = 0.0;
    for (int i = 0; i < n; i++) sq = sq + d[i] * d[i];
    double stdev = sqrt(sq / n - mean * mean);
    double maxd = mean + 10 * stdev;
    double mx = 0;
    for (int i = 0; i < n; i++)
        if (d[i] <= maxd && d[i] > mx) mx = d[i];
    free(d);
    return mx;
}

int orc_build(orc_world *w, int threads)
{
    /* Tree::buildTree (Tree.cpp:24-55). */
    if (w->root) node_free(w->root);
    w->root = node_new();
    w->root->radius = tree_width(w);
    w->root->depth = 0;
    if (threads < 1) threads = 1;
    int *all = (int *)malloc(sizeof(int) * (size_t)(w->n > 0 ? w->n : 1));
    for (int i = 0; i < w->n; i++) all[i] = i;
    insert_vec(w, w->root, all, w->n, threads);
    free(all);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Kernels (simulation/src/Math/kernel.cpp)                                   */
/* ------------------------------------------------------------------------- */
static double cubic_spline(double r, double h)
{
    /* kernel::cubicSplineKernel (kernel.cpp:4-16). */
    double alpha = 1.0 / (ORC_PI * h * h * h);
    double q = r / h;
    if (q < 1.0) return alpha * (1 - 1.5 * q * q + 0.75 * q * q * q);
    if (q < 2.0) return alpha * 0.25 * pow(2 - q, 3);
    return 0.0;
}

static void grad_cubic_spline(const double *d, double h, double *out)
{
    /* kernel::gradientCubicSplineKernel (kernel.cpp:18-39). */
    double rn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    out[0] = out[1] = out[2] = 0.0;
    if (rn == 0.0) return;
    double alpha = 1.0 / (ORC_PI * h * h * h);
    double q = rn / h;
    double g;
    if (q < 1.0)
        g = alpha * (-3.0 * q + 2.25 * q * q);
    else if (q < 2.0)
        g = alpha * (-0.75 * pow(2 - q, 2));
    else
        return;
    g /= h;
    double s = g / rn;
    out[0] = d[0] * s;
    out[1] = d[1] * s;
    out[2] = d[2] * s;
}

static double softening_kernel(double u)
{
    /* kernel::softeningKernel (kernel.cpp:41-56). */
    if (u >= 0 && u < 1.0 / 2.0)
        return (16.0 / 3.0) * pow(u, 2) - (48.0 / 5.0) * pow(u, 4) + (32.0 / 5.0) * pow(u, 5) - (14.0 / 5.0);
    if (u >= 1.0 / 2.0 && u < 1.0)
        return (1.0 / (15.0 * u)) + (32.0 / 3.0) * pow(u, 2) - (16.0) * pow(u, 3) - (48.0 / 5.0) * pow(u, 4) -
               (32.0 / 15.0) * pow(u, 5) - (16.0 / 5.0);
    if (u >= 1.0) return -1.0 / u;
    return 0.0;
}

/* The reference writes `abs(e)` unqualified (Node.cpp:302, 354); in that
 * translation unit this resolves to the C library's int abs(int), so |e| is the
 * truncated integer.  Out-of-range conversions behave as on x86-64 (INT_MIN,
 * whose abs stays INT_MIN). */
static double ref_int_abs(double e)
{
    if (!(e > -2147483649.0 && e < 2147483648.0)) return -2147483648.0;
    double t = trunc(e);
    return t < 0 ? -t : t;
}

/* Softened pair acceleration of Node.cpp:285-313 / 337-365.  Returns 0 when the
 * reference returns early (K-r == 0, e NaN, acceleration NaN). */
static int soft_gravity(double mass, const double *d, double r, double e0, double *acc)
{
    double u = r / (2.8 * e0);
    double K = softening_kernel(u);
    if ((K - r) == 0) return 0;
    double e = -(2.8 * e0) / (K - r);
    if (isnan(e)) return 0;
    double ae = ref_int_abs(e);
    double eps = e0;
    if (ae > (e0 * 0.0001) && ae < 1e30) eps = e;
    double s = g_G * mass / (r * r + eps * eps);
    double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double g[3] = {0, 0, 0};
    if (len > 0) {
        g[0] = (d[0] / len) * s;
        g[1] = (d[1] / len) * s;
        g[2] = (d[2] / len) * s;
    }
    if (isnan(g[0]) || isnan(g[1]) || isnan(g[2])) return 0;
    acc[0] += g[0];
    acc[1] += g[1];
    acc[2] += g[2];
    return 1;
}

/* Node::calcSPHForce (Node.cpp:88-172); j quantities are replaced by i's. */
static void sph_force(orc_world *w, const onode *n, int i, double *acc)
{
    double h_i = w->h[i];
    double h_ij = (h_i + h_i) / 2.0;
    double rho_i = w->rho[i];
    double P_i = w->P[i];
    const double *vi = w->v + 3 * (size_t)i;
    const double *vj = n->isLeaf ? w->v + 3 * (size_t)n->particle : n->mVel;
    double vij[3] = {vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2]};
    const double *xi = w->x + 3 * (size_t)i;
    double d[3] = {xi[0] - n->com[0], xi[1] - n->com[1], xi[2] - n->com[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double c_i = sqrt(ORC_GAMMA * P_i / rho_i);
    double c_ij = (c_i + c_i) / 2.0;
    double gm = n->gasMass;
    double f[3] = {0, 0, 0};
    double gi[3], gij[3];
    grad_cubic_spline(d, h_i, gi);
    double pr = (P_i / (rho_i * rho_i) + P_i / (rho_i * rho_i));
    for (int k = 0; k < 3; k++) f[k] += (-gm * pr) * gi[k];
    double MU = 0.0;
    {
        double alpha = 0.5, beta = 1.0, eta = 0.01;
        double vd = vij[0] * d[0] + vij[1] * d[1] + vij[2] * d[2];
        double mu = h_ij * vd / (r * r + eta * (h_ij * h_ij));
        if (vd < 0) MU = -alpha * c_ij * mu + beta * (mu * mu);
        grad_cubic_spline(d, h_ij, gij);
        for (int k = 0; k < 3; k++) f[k] += (-gm * MU) * gij[k];
    }
    grad_cubic_spline(d, h_i, gi);
    double vg = vij[0] * gi[0] + vij[1] * gi[1] + vij[2] * gi[2];
    w->dUdt[i] += 1.0 / 2.0 * gm * (pr + MU) * vg;
    if (isnan(f[0]) || isnan(f[1]) || isnan(f[2])) return;
    acc[0] += f[0];
    acc[1] += f[1];
    acc[2] += f[2];
}

/* Node::calculateGravityForce (Node.cpp:247-399). */
static void walk(orc_world *w, const onode *n, int i, double e0, double theta, double *acc)
{
    if (n->mass == 0) return;
    if (i == n->particle) return;
    if (w->m[i] == 0) return;
    const double *xi = w->x + 3 * (size_t)i;
    double d[3] = {n->com[0] - xi[0], n->com[1] - xi[1], n->com[2] - xi[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (r == 0) return;
    if (n->isLeaf) {
        if (n->particle >= 0 && i != n->particle) {
            if (!soft_gravity(n->mass, d, r, e0, acc)) return;
            if (r < w->h[i] * 2)
                if (w->type[n->particle] == 2 && w->type[i] == 2) sph_force(w, n, i, acc);
        }
    } else {
        double s = n->radius / r;
        if (s < theta) {
            if (!soft_gravity(n->mass, d, r, e0, acc)) return;
            if (r < w->h[i] * 2)
                if (w->type[i] == 2 && n->gasMass > 0) sph_force(w, n, i, acc);
        } else {
            for (int k = 0; k < 8; k++) {
                const onode *c = n->children[k];
                if (!c || c->mass == 0) continue;
                walk(w, c, i, e0, theta, acc);
            }
        }
    }
}

int orc_forces(orc_world *w, double e0, double theta, int threads)
{
    /* Tree::calculateForces (Tree.cpp:57-83); every particle is active. */
    if (!w->root) return -1;
    if (threads < 1) threads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int i = 0; i < w->n; i++) {
        double *a = w->a + 3 * (size_t)i;
        a[0] = a[1] = a[2] = 0.0;
        walk(w, w->root, i, e0, theta, a);
    }
    return 0;
}

int orc_forces_subset(orc_world *w, double e0, double theta, int threads, int ns, const int32_t *idx)
{
    if (!w->root) return -1;
    if (threads < 1) threads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int k = 0; k < ns; k++) {
        int i = idx[k];
        double *a = w->a + 3 * (size_t)i;
        a[0] = a[1] = a[2] = 0.0;
        walk(w, w->root, i, e0, theta, a);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* SPH density (Tree.cpp:119-150, Node.cpp:722-796)                           */
/* ------------------------------------------------------------------------- */
static void gas_density_node(orc_world *w, onode *n, double massInH)
{
    if (n->gasMass == 0) return;
    onode *par = n->parent;
    if (!par) return;
    if (n->gasMass < massInH) {
        double md = massInH - n->gasMass;
        double pmd = massInH - par->gasMass;
        if (fabs(md) > fabs(pmd)) gas_density_node(w, par, massInH);
    }
    double md = massInH - n->gasMass;
    double pmd = massInH - par->gasMass;
    if (fabs(md) < fabs(pmd) && n->gasMass != 0) {
        for (int k = 0; k < n->ncp; k++) {
            int p = n->cp[k];
            if (w->type[p] == 2) w->h[p] = n->radius * 2;
        }
        double rho = 0;
        for (int k = 0; k < n->ncp; k++) {
            int p = n->cp[k];
            if (w->type[p] == 2) {
                const double *x = w->x + 3 * (size_t)p;
                double dd[3] = {x[0] - n->com[0], x[1] - n->com[1], x[2] - n->com[2]};
                double len = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
                rho += w->m[p] * cubic_spline(len, w->h[p]);
            }
        }
        for (int k = 0; k < n->ncp; k++) {
            int p = n->cp[k];
            if (w->type[p] == 2) {
                w->rho[p] = rho;
                w->P[p] = (ORC_GAMMA - 1.0) * w->U[p] * w->rho[p];
                w->T[p] = (ORC_GAMMA - 1.0) * w->U[p] * ORC_PRTN * w->mu[p] / (ORC_KB);
            }
        }
    }
}

int orc_gas_density(orc_world *w, double massInH)
{
    for (int i = 0; i < w->n; i++)
        if (w->type[i] == 2) w->h[i] = 0;
    for (int i = 0; i < w->n; i++)
        if (w->type[i] == 2 && w->node[i] && w->h[i] == 0) gas_density_node(w, w->node[i], massInH);
    return 0;
}

/* Node::calcVisualDensity (Node.cpp:832-877) and Tree::calcVisualDensity (Tree.cpp:152-175). */
static void visual_density_node(orc_world *w, onode *n, double R)
{
    onode *par = n->parent;
    if (!par) return;
    double rd = R - n->radius;
    double prd = R - par->radius;
    if (fabs(rd) > fabs(prd)) {
        visual_density_node(w, par, R);
    } else {
        double vol = n->radius * n->radius * n->radius;
        if (vol == 0 || n->mass == 0) return;
        double dens = n->mass / vol;
        if (dens == 0 || isinf(dens)) return;
        for (int k = 0; k < n->ncp; k++) w->vdens[n->cp[k]] = dens;
    }
}

int orc_visual_density(orc_world *w, double R)
{
    for (int i = 0; i < w->n; i++) w->vdens[i] = 0;
    for (int i = 0; i < w->n; i++) {
        if (w->vdens[i] != 0) continue;
        if (w->node[i]) visual_density_node(w, w->node[i], R);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Leapfrog (TimeIntegration.cpp:10-40)                                       */
/* ------------------------------------------------------------------------- */
void orc_kick(orc_world *w, double dt)
{
    for (int i = 0; i < w->n; i++) {
        double *a = w->a + 3 * (size_t)i, *v = w->v + 3 * (size_t)i;
        if (isnan(a[0]) || isnan(a[1]) || isnan(a[2])) continue;
        for (int k = 0; k < 3; k++) v[k] = v[k] + a[k] * dt / 2;
    }
}

void orc_drift(orc_world *w, double dt)
{
    for (int i = 0; i < w->n; i++)
        for (int k = 0; k < 3; k++) w->x[3 * (size_t)i + k] = w->x[3 * (size_t)i + k] + w->v[3 * (size_t)i + k] * dt;
}

void orc_ueuler(orc_world *w, double dt)
{
    for (int i = 0; i < w->n; i++) {
        if (!isnan(w->dUdt[i])) w->U[i] += w->dUdt[i] * dt;
        w->dUdt[i] = 0;
    }
}

void orc_scale_positions(orc_world *w, double f)
{
    for (size_t i = 0; i < 3 * (size_t)w->n; i++) w->x[i] *= f;
}

/* ------------------------------------------------------------------------- */
/* World management and export                                               */
/* ------------------------------------------------------------------------- */
orc_world *orc_create(int n, const double *pos, const double *vel, const double *mass, const double *U,
                      const uint8_t *type)
{
    orc_world *w = (orc_world *)calloc(1, sizeof(orc_world));
    size_t N = n > 0 ? (size_t)n : 1;
    w->n = n;
    w->x = (double *)calloc(3 * N, sizeof(double));
    w->v = (double *)calloc(3 * N, sizeof(double));
    w->a = (double *)calloc(3 * N, sizeof(double));
    w->m = (double *)calloc(N, sizeof(double));
    w->h = (double *)calloc(N, sizeof(double));
    w->rho = (double *)calloc(N, sizeof(double));
    w->P = (double *)calloc(N, sizeof(double));
    w->T = (double *)calloc(N, sizeof(double));
    w->U = (double *)calloc(N, sizeof(double));
    w->dUdt = (double *)calloc(N, sizeof(double));
    w->mu = (double *)calloc(N, sizeof(double));
    w->vdens = (double *)calloc(N, sizeof(double));
    w->type = (uint8_t *)calloc(N, 1);
    w->node = (onode **)calloc(N, sizeof(onode *));
    if (n > 0) {
        memcpy(w->x, pos, 3 * N * sizeof(double));
        if (vel) memcpy(w->v, vel, 3 * N * sizeof(double));
        memcpy(w->m, mass, N * sizeof(double));
        if (U) memcpy(w->U, U, N * sizeof(double));
        memcpy(w->type, type, N);
    }
    for (size_t i = 0; i < N; i++) w->mu[i] = 0.58; /* Particle.h:40 */
    return w;
}

void orc_destroy(orc_world *w)
{
    if (!w) return;
    node_free(w->root);
    free(w->x); free(w->v); free(w->a); free(w->m); free(w->h); free(w->rho); free(w->P);
    free(w->T); free(w->U); free(w->dUdt); free(w->mu); free(w->vdens); free(w->type); free(w->node);
    free(w);
}

static double *field_ptr(orc_world *w, int f, size_t *cnt)
{
    size_t n = (size_t)w->n;
    *cnt = n;
    switch (f) {
    case ORC_POS: *cnt = 3 * n; return w->x;
    case ORC_VEL: *cnt = 3 * n; return w->v;
    case ORC_ACC: *cnt = 3 * n; return w->a;
    case ORC_MASS: return w->m;
    case ORC_H: return w->h;
    case ORC_RHO: return w->rho;
    case ORC_P: return w->P;
    case ORC_T: return w->T;
    case ORC_U: return w->U;
    case ORC_DUDT: return w->dUdt;
    case ORC_VDENS: return w->vdens;
    }
    *cnt = 0;
    return NULL;
}

void orc_get(orc_world *w, int f, double *out)
{
    size_t c;
    double *p = field_ptr(w, f, &c);
    if (p && c) memcpy(out, p, c * sizeof(double));
}

void orc_set(orc_world *w, int f, const double *in)
{
    size_t c;
    double *p = field_ptr(w, f, &c);
    if (p && c) memcpy(p, in, c * sizeof(double));
}

double orc_root_radius(orc_world *w) { return w->root ? w->root->radius : 0.0; }

static int64_t count_nodes(const onode *n)
{
    if (!n) return 0;
    int64_t c = 1;
    for (int i = 0; i < 8; i++) c += count_nodes(n->children[i]);
    return c;
}

int64_t orc_node_count(orc_world *w) { return count_nodes(w->root); }

uint64_t orc_id_hash(uint64_t id)
{
    uint64_t z = id + 1 + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    int32_t *depth, *is_leaf, *particle;
    int64_t *cp_count;
    uint64_t *cp_hash;
    double *mass, *com3, *gas_mass, *mvel3, *center3, *radius;
    int64_t k;
    int64_t *leaf_of;
} export_ctx;

static void export_rec(const onode *n, export_ctx *e)
{
    int64_t k = e->k++;
    if (e->depth) e->depth[k] = n->depth;
    if (e->is_leaf) e->is_leaf[k] = n->isLeaf;
    if (e->particle) e->particle[k] = n->particle;
    if (e->cp_count) e->cp_count[k] = n->ncp;
    if (e->cp_hash) {
        uint64_t h = 0;
        for (int i = 0; i < n->ncp; i++) h += orc_id_hash((uint64_t)n->cp[i]);
        e->cp_hash[k] = h;
    }
    if (e->mass) e->mass[k] = n->mass;
    if (e->com3) memcpy(e->com3 + 3 * k, n->com, 3 * sizeof(double));
    if (e->gas_mass) e->gas_mass[k] = n->gasMass;
    if (e->mvel3) memcpy(e->mvel3 + 3 * k, n->mVel, 3 * sizeof(double));
    if (e->center3) memcpy(e->center3 + 3 * k, n->pos, 3 * sizeof(double));
    if (e->radius) e->radius[k] = n->radius;
    if (e->leaf_of && n->isLeaf && n->particle >= 0) e->leaf_of[n->particle] = k;
    for (int i = 0; i < 8; i++)
        if (n->children[i]) export_rec(n->children[i], e);
}

void orc_topology(orc_world *w, int32_t *depth, int32_t *is_leaf, int32_t *particle, int64_t *cp_count,
                  uint64_t *cp_hash, double *mass, double *com3, double *gas_mass, double *mvel3, double *center3,
                  double *radius)
{
    export_ctx e = {depth, is_leaf, particle, cp_count, cp_hash, mass, com3, gas_mass, mvel3, center3, radius, 0, NULL};
    if (w->root) export_rec(w->root, &e);
}

typedef struct {
    const onode *target;
    int64_t k, found;
} find_ctx;

static void find_rec(const onode *n, find_ctx *f)
{
    if (f->found >= 0) return;
    if (n == f->target) {
        f->found = f->k;
        return;
    }
    f->k++;
    for (int i = 0; i < 8 && f->found < 0; i++)
        if (n->children[i]) find_rec(n->children[i], f);
}

void orc_leaf_index(orc_world *w, int64_t *out)
{
    /* Preorder numbering: export leaves once, then resolve nodes that are not
     * leaves holding that particle (rare: a particle whose leaf was split and
     * whose reinsertion was dropped) by search. */
    for (int i = 0; i < w->n; i++) out[i] = -1;
    if (!w->root) return;
    export_ctx e = {0};
    e.leaf_of = out;
    export_rec(w->root, &e);
    for (int i = 0; i < w->n; i++) {
        if (!w->node[i]) { out[i] = -1; continue; }
        if (w->node[i]->isLeaf && w->node[i]->particle == i) continue;
        find_ctx f = {w->node[i], 0, -1};
        find_rec(w->root, &f);
        out[i] = f.found;
    }
}

void orc_direct_sum(int n, const double *pos, const double *mass, double e0, double G, int ns, const int32_t *sample,
                    double *out, int threads)
{
    double saveG = g_G;
    g_G = G;
    if (threads < 1) threads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (int k = 0; k < ns; k++) {
        int i = sample[k];
        double acc[3] = {0, 0, 0};
        const double *xi = pos + 3 * (size_t)i;
        for (int j = 0; j < n; j++) {
            if (j == i || mass[j] == 0) continue;
            const double *xj = pos + 3 * (size_t)j;
            double d[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (r == 0) continue;
            soft_gravity(mass[j], d, r, e0, acc);
        }
        out[3 * k] = acc[0];
        out[3 * k + 1] = acc[1];
        out[3 * k + 2] = acc[2];
    }
    g_G = saveG;
}
