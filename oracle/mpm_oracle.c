/*
 * CPU restatement of the reference's explicit-MPM double-pass step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA engine is
 * checked against, and the CPU baseline that bench.py times beside it.  The
 * product path never links, loads or calls it.
 *
 * It restates, operation for operation (same association order, no FMA
 * contraction: build with -ffp-contract=off), the reference solver:
 *   non-contact step  PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp
 *                     :4-22 ResetGrid, :23-47 FindAGPs, :48-89 M2G,
 *                     :90-142 IntegrateGrid, :143-174 DisplacementControl,
 *                     :175-280 G2P_P2_SmallStrain, :439-815 driver loop
 *   contact step      PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks_Contact.cpp:4-566
 *   cell lookup       GridPoint_Mediator.cpp:4-54, bases :95-144
 *   node positions    GridPoint_Factory.h:33-68
 *   constitutive      ConstitutiveRelation_calculateIncrement_Elastic.cpp:4-18,
 *                     …_PerfectlyPlastic.cpp:4-76, …_VonMisesHardening.cpp:4-92
 *   platen timeline   TimeLine.h:33-46
 * with glm's arithmetic as written in oracle/glmshim/glm/glm.hpp.
 *
 * Without OpenMP every loop runs in particle / node index order, which fixes
 * the order of every scatter-add and of every overwrite (displacement
 * control, contact normals) to that of a one-thread reference run; that is
 * the order the golden states were produced in.  Built with -fopenmp the
 * loops are shared by a team and the scatter-adds take one lock per node,
 * like the reference (…MPLocks.cpp:66,86,556,562); that build is only timed.
 *
 * One extension beyond the reference, off unless requested: floor friction
 * on the contact path (opts.floor_friction), Coulomb friction on the x and y
 * tangents of z-fixed nodes, in the same per-component form as the
 * reference's x-wall friction (…MPLocks.cpp:106-124).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mpm_snapshot.h"

#define ELASTIC 0
#define PLASTIC 3
#define VONMISESHARDENING 4

typedef struct oracle_opts {
    int contact;
    int floor_friction;
    int threads; /* OpenMP team size (ignored without OpenMP) */
} oracle_opts;

typedef struct agp {
    uint32_t idx;
    double N;
    double G[3];
} agp;

typedef struct work {
    agp* agps;     /* [n][8] */
    uint8_t* nagp; /* [n] */
    double h[3];
    int nn[3];
    double* xnode; /* [nn][3] */
    /* boundary work (an extension; NULL bw: off): the step's sums and the
     * scratch of the displacement-control term */
    double* bw;       /* [2] accumulated work: displacement control, friction */
    double bw_dc, bw_fr;
    double* fsave;    /* [nn][3] force of a controlled node before the control zeroes it */
    uint8_t* dcax;    /* [nn] axes the list controls on the node */
#ifdef _OPENMP
    omp_lock_t* locks;
#endif
} work;

/* ---- glm scalar helpers (glmshim semantics) ----------------------------- */
static inline double gabs(double x) { return x >= 0.0 ? x : -x; }
static inline double gsign(double x) { return (double)((0.0 < x) - (x < 0.0)); }
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double len3(const double* a) { return sqrt(dot3(a, a)); }

/* ---- TimeLine::getVelocity (TimeLine.h:33-46) --------------------------- */
static void timeline_velocity(const mpmsnap* s, double t, double out[3]) {
    out[0] = out[1] = out[2] = 0.0;
    for (int k = 0; k + 1 < (int)s->h.n_timeline; ++k) {
        if (s->tl_time[k] <= t && t < s->tl_time[k + 1]) {
            double sc = (t - s->tl_time[k]) / (s->tl_time[k + 1] - s->tl_time[k]);
            for (int c = 0; c < 3; ++c) out[c] = (1.0 - sc) * s->tl_vel[3 * k + c] + sc * s->tl_vel[3 * (k + 1) + c];
        }
    }
}

/* ---- ConstitutiveRelation increments ------------------------------------ */
typedef struct cr_out {
    double dsig[6];
    double deps_p[6];
    double dR;
} cr_out;

/* …_Elastic.cpp:4-18 */
static void cr_elastic(const mpmsnap_material* m, const double e[6], cr_out* o) {
    double E = m->E, nu = m->nu;
    double C = E / (1.0 + nu) / (1.0 - 2.0 * nu);
    o->dsig[0] = C * ((1.0 - nu) * e[0] + nu * e[1] + nu * e[2]);
    o->dsig[1] = C * ((1.0 - nu) * e[1] + nu * e[0] + nu * e[2]);
    o->dsig[2] = C * ((1.0 - nu) * e[2] + nu * e[0] + nu * e[1]);
    o->dsig[3] = C * ((0.5 - nu) * e[3]);
    o->dsig[4] = C * ((0.5 - nu) * e[4]);
    o->dsig[5] = C * ((0.5 - nu) * e[5]);
}

/* Shared J2 radial return of …_PerfectlyPlastic.cpp:4-76 and
 * …_VonMisesHardening.cpp:4-92.  hardening = 0: radius k0 (PerfectlyPlastic);
 * hardening = 1: radius k0 + R/sqrt(2) and the explicit back-stress update. */
static void cr_j2(const mpmsnap_material* m, double R, const double sig[6], const double e[6], int hardening,
                  cr_out* o) {
    double E = m->E, nu = m->nu, Y = m->yield;
    double dtr[6], tr[6], dev[6];
    double C = E / (1.0 + nu) / (1.0 - 2.0 * nu);
    dtr[0] = C * ((1.0 - nu) * e[0] + nu * e[1] + nu * e[2]);
    dtr[1] = C * ((1.0 - nu) * e[1] + nu * e[0] + nu * e[2]);
    dtr[2] = C * ((1.0 - nu) * e[2] + nu * e[0] + nu * e[1]);
    dtr[3] = C * ((0.5 - nu) * e[3]);
    dtr[4] = C * ((0.5 - nu) * e[4]);
    dtr[5] = C * ((0.5 - nu) * e[5]);
    for (int i = 0; i < 6; ++i) tr[i] = sig[i] + dtr[i];
    double hyd = 1.0 / 3.0 * (tr[0] + tr[1] + tr[2]);
    for (int i = 0; i < 6; ++i) dev[i] = tr[i];
    dev[0] -= hyd;
    dev[1] -= hyd;
    dev[2] -= hyd;
    double J2 = 0.0;
    J2 += 1.0 / 6.0 * (tr[0] - tr[1]) * (tr[0] - tr[1]);
    J2 += 1.0 / 6.0 * (tr[1] - tr[2]) * (tr[1] - tr[2]);
    J2 += 1.0 / 6.0 * (tr[2] - tr[0]) * (tr[2] - tr[0]);
    J2 += tr[3] * tr[3];
    J2 += tr[4] * tr[4];
    J2 += tr[5] * tr[5];
    double k0 = Y / sqrt(3.0);
    double rad = k0;
    if (hardening) {
        double Rs = R / sqrt(2.0);
        rad = k0 + Rs;
    }
    if (J2 <= rad * rad) {
        for (int i = 0; i < 6; ++i) o->dsig[i] = dtr[i];
        for (int i = 0; i < 6; ++i) o->deps_p[i] = 0.0;
        if (hardening) o->dR = 0.0;
        return;
    }
    for (int i = 0; i < 6; ++i) dev[i] *= rad / sqrt(J2);
    for (int i = 0; i < 6; ++i) o->dsig[i] = dev[i] - sig[i];
    o->dsig[0] += hyd;
    o->dsig[1] += hyd;
    o->dsig[2] += hyd;
    double G = 0.5 * E / (1.0 + nu);
    double ee[6];
    ee[0] = o->dsig[0] / E - o->dsig[1] * nu / E - o->dsig[2] * nu / E;
    ee[1] = o->dsig[1] / E - o->dsig[0] * nu / E - o->dsig[2] * nu / E;
    ee[2] = o->dsig[2] / E - o->dsig[0] * nu / E - o->dsig[1] * nu / E;
    ee[3] = o->dsig[3] / G;
    ee[4] = o->dsig[4] / G;
    ee[5] = o->dsig[5] / G;
    for (int i = 0; i < 6; ++i) o->deps_p[i] = e[i] - ee[i];
    if (!hardening) return;
    double ep = 0.0;
    for (int i = 0; i < 6; ++i) ep += o->deps_p[i] * o->deps_p[i];
    ep *= 2.0 / 3.0;
    ep = sqrt(ep);
    if ((sqrt(2.0 / 3.0) * m->C1 - R) > 0.0)
        o->dR = m->C0 * (sqrt(2.0 / 3.0) * m->C1 - R) * ep;
    else
        o->dR = 0.0;
}

/* Dispatch of …MPLocks.cpp:232-239 (unknown type -> PerfectlyPlastic). */
static void cr_increment(const mpmsnap_material* m, double R, const double sig[6], const double e[6], cr_out* o) {
    memset(o, 0, sizeof(*o));
    if (m->type == ELASTIC)
        cr_elastic(m, e, o);
    else if (m->type == VONMISESHARDENING)
        cr_j2(m, R, sig, e, 1, o);
    else
        cr_j2(m, R, sig, e, 0, o);
}

/* ---- grid geometry ------------------------------------------------------ */
static int work_init(work* w, const mpmsnap* s) {
    memset(w, 0, sizeof(*w));
    for (int a = 0; a < 3; ++a) {
        w->h[a] = s->h.length[a] / (double)s->h.cells[a];
        w->nn[a] = s->h.cells[a] + 1;
    }
    size_t n = (size_t)s->h.n_particles, nn = (size_t)s->h.n_nodes;
    w->agps = (agp*)malloc(sizeof(agp) * 8 * (n ? n : 1));
    w->nagp = (uint8_t*)calloc(n ? n : 1, 1);
    w->xnode = (double*)malloc(sizeof(double) * 3 * nn);
    if (!w->agps || !w->nagp || !w->xnode) return -1;
    /* GridPoint_Factory.h:43-63: dx = i_x * L / cells */
    for (int iz = 0; iz < w->nn[2]; ++iz)
        for (int iy = 0; iy < w->nn[1]; ++iy)
            for (int ix = 0; ix < w->nn[0]; ++ix) {
                size_t id = (size_t)ix + (size_t)iy * w->nn[0] + (size_t)iz * w->nn[0] * w->nn[1];
                w->xnode[3 * id + 0] = ix * s->h.length[0] / s->h.cells[0];
                w->xnode[3 * id + 1] = iy * s->h.length[1] / s->h.cells[1];
                w->xnode[3 * id + 2] = iz * s->h.length[2] / s->h.cells[2];
            }
#ifdef _OPENMP
    w->locks = (omp_lock_t*)malloc(sizeof(omp_lock_t) * (nn ? nn : 1));
    for (size_t i = 0; i < nn; ++i) omp_init_lock(&w->locks[i]);
#endif
    return 0;
}

static void work_free(work* w, const mpmsnap* s) {
#ifdef _OPENMP
    for (size_t i = 0; i < (size_t)s->h.n_nodes; ++i) omp_destroy_lock(&w->locks[i]);
    free(w->locks);
#else
    (void)s;
#endif
    free(w->agps);
    free(w->nagp);
    free(w->xnode);
    free(w->fsave);
    free(w->dcax);
}

/* ---- boundary work (an extension, off unless requested) ----------------------
 * Not in the reference, whose energy report has no external-work term
 * (PhysicsEngine.cpp:140-156).  A displacement-controlled node axis takes the
 * platen particle's velocity v and its force f is zeroed, so the platen
 * supplies -f there and works -f v dt; a friction law that adds df to a
 * tangent force works df (p/m) dt at the node's updated momentum p.  The
 * displacement-control term is counted at the first control pass of a step
 * (the one before G2P pass 1), with the force each controlled node had just
 * before that pass and the velocity the list's last writer imposed. */
static void dc_work_begin(mpmsnap* s, work* w, int contact) {
    if (!w->bw) return;
    for (long k = 0; k < (long)s->h.n_dc; ++k) {
        size_t p = s->dc_list[k];
        uint8_t axes = contact ? 7u : (uint8_t)(s->pflags[p] & 7u);
        for (int j = 0; j < w->nagp[p]; ++j) {
            uint32_t i = w->agps[8 * p + j].idx;
            for (int c = 0; c < 3; ++c) w->fsave[3 * (size_t)i + c] = s->g_force[3 * (size_t)i + c];
            w->dcax[i] |= axes;
        }
    }
}

static void dc_work_end(mpmsnap* s, work* w) {
    if (!w->bw) return;
    for (long k = 0; k < (long)s->h.n_dc; ++k) {
        size_t p = s->dc_list[k];
        for (int j = 0; j < w->nagp[p]; ++j) {
            size_t i = w->agps[8 * p + j].idx;
            if (!w->dcax[i]) continue;
            double sum = 0.0;
            for (int c = 0; c < 3; ++c)
                if (w->dcax[i] & (1u << c)) sum -= w->fsave[3 * i + c] * s->g_vel[3 * i + c];
            w->bw_dc += sum;
            w->dcax[i] = 0;
        }
    }
}

/* friction work of node i after its update; dfr: the force the friction law added per axis */
static void friction_work(mpmsnap* s, work* w, size_t i, const double dfr[3]) {
    if (!w->bw || (dfr[0] == 0.0 && dfr[1] == 0.0) || !(s->g_mass[i] > s->h.mass_min)) return;
    w->bw_fr += (dfr[0] * s->g_mom[3 * i] + dfr[1] * s->g_mom[3 * i + 1]) / s->g_mass[i];
}

#ifdef _OPENMP
#define LOCK(w, i) omp_set_lock(&(w)->locks[i])
#define UNLOCK(w, i) omp_unset_lock(&(w)->locks[i])
#else
#define LOCK(w, i) ((void)0)
#define UNLOCK(w, i) ((void)0)
#endif

/* findAdjacentGridPoints (GridPoint_Mediator.cpp:4-54) + calculateBases_Classic (:95-144) */
static void find_agps(const mpmsnap* s, work* w, size_t p) {
    const double* x = &s->pos[3 * p];
    double q[3];
    int b[3], ls[3] = {0, 0, 0}, le[3] = {2, 2, 2};
    for (int a = 0; a < 3; ++a) {
        q[a] = floor(x[a] / w->h[a]);
        b[a] = (int)q[a];
    }
    for (int a = 0; a < 3; ++a) {
        if ((((double)b[a] + 1.0 - x[a] / w->h[a])) < 0.0) ls[a] = 1;
        if (((x[a] / w->h[a]) - (double)b[a]) < 0.0) le[a] = 1;
    }
    int cnt = 0;
    agp* out = &w->agps[8 * p];
    for (int ix = ls[0]; ix < le[0]; ++ix)
        for (int iy = ls[1]; iy < le[1]; ++iy)
            for (int iz = ls[2]; iz < le[2]; ++iz) {
                int nx = b[0] + ix, ny = b[1] + iy, nz = b[2] + iz;
                if (nx < 0 || ny < 0 || nz < 0) continue;
                if (nx > w->nn[0] - 1 || ny > w->nn[1] - 1 || nz > w->nn[2] - 1) continue;
                uint32_t id = (uint32_t)(nx + ny * w->nn[0] + nz * (w->nn[0] * w->nn[1]));
                const double* xn = &w->xnode[3 * (size_t)id];
                double d[3], Nv[3], r[3];
                for (int a = 0; a < 3; ++a) {
                    d[a] = x[a] - xn[a];
                    r[a] = d[a] / w->h[a];
                    Nv[a] = 1.0 - gabs(r[a]);
                    if (Nv[a] < 0.0 || Nv[a] > 1.0) Nv[a] = 0.0;
                }
                agp* g = &out[cnt++];
                g->idx = id;
                g->N = Nv[0] * Nv[1] * Nv[2];
                g->G[0] = g->G[1] = g->G[2] = 0.0;
                if (gabs(d[0] / w->h[0]) > 1.0e-12 && gabs(d[0] / w->h[0]) < 1.0 - 1.0e-12)
                    g->G[0] = -Nv[1] * Nv[2] * gsign(d[0]) / w->h[0];
                if (gabs(d[1] / w->h[1]) > 1.0e-12 && gabs(d[1] / w->h[1]) < 1.0 - 1.0e-12)
                    g->G[1] = -Nv[0] * Nv[2] * gsign(d[1]) / w->h[1];
                if (gabs(d[2] / w->h[2]) > 1.0e-12 && gabs(d[2] / w->h[2]) < 1.0 - 1.0e-12)
                    g->G[2] = -Nv[0] * Nv[1] * gsign(d[2]) / w->h[2];
                s->g_state[id] |= MPM_NS_ACTIVE; /* thisAGP->b_Active = true */
            }
    w->nagp[p] = (uint8_t)cnt;
}

/* Displacement control, non-contact form (…MPLocks.cpp:143-174): flagged axes only. */
static void displacement_control(mpmsnap* s, work* w) {
#pragma omp for
    for (long k = 0; k < (long)s->h.n_dc; ++k) {
        size_t p = s->dc_list[k];
        uint8_t fl = s->pflags[p];
        for (int j = 0; j < w->nagp[p]; ++j) {
            uint32_t i = w->agps[8 * p + j].idx;
            for (int c = 0; c < 3; ++c) {
                if (fl & (1u << c)) {
                    s->g_vel[3 * i + c] = s->vel[3 * p + c];
                    s->g_mom[3 * i + c] = s->g_mass[i] * s->vel[3 * p + c];
                    s->g_force[3 * i + c] = 0.0;
                }
            }
        }
    }
}

static void zero_fixed(mpmsnap* s, size_t i, int c) {
    s->g_vel[3 * i + c] = 0.0;
    s->g_mom[3 * i + c] = 0.0;
    s->g_force[3 * i + c] = 0.0;
}

/* Coulomb friction of one tangent component t against normal force fn
 * (…MPLocks.cpp:108-119, written for normal x / tangent y). */
static void coulomb(mpmsnap* s, size_t i, int t, double fn, double dt) {
    double* p = &s->g_mom[3 * i];
    double* f = &s->g_force[3 * i];
    double trial_t = p[t] + f[t] * dt;
    double mu = s->friction[i];
    double ff = mu * gsign(-trial_t) * gabs(fn);
    if (gabs(ff * dt) > gabs(trial_t)) ff *= gabs(trial_t / dt) / gabs(ff);
    f[t] += ff;
}

static void damping(mpmsnap* s, size_t i) {
    double* p = &s->g_mom[3 * i];
    double* f = &s->g_force[3 * i];
    if (len3(p) > 1.0e-24) {
        double inv = 1.0 / sqrt(dot3(p, p));
        double nrm[3] = {p[0] * inv, p[1] * inv, p[2] * inv};
        double dd = gabs(dot3(f, nrm));
        double sc = s->h.damping * dd;
        for (int c = 0; c < 3; ++c) f[c] = f[c] - sc * nrm[c];
    }
}

/* IntegrateGrid, non-contact (…MPLocks.cpp:90-142) */
static void integrate_grid(mpmsnap* s, work* w, double dt) {
#pragma omp for
    for (long li = 0; li < (long)s->h.n_nodes; ++li) {
        size_t i = (size_t)li;
        if (!(s->g_state[i] & MPM_NS_ACTIVE)) continue;
        double* p = &s->g_mom[3 * i];
        double* f = &s->g_force[3 * i];
        damping(s, i);
        double dfr[3] = {0.0, 0.0, 0.0};
        if (s->fixed[i] & MPM_NF_FIX_X) {
            double trial_y = p[1] + f[1] * dt;
            if (gabs(trial_y * dt) > 1.0e-24 && f[0] > 0.0) {
                double f0 = f[1];
                coulomb(s, i, 1, f[0], dt);
                dfr[1] = f[1] - f0;
            }
            zero_fixed(s, i, 0);
        }
        if (s->fixed[i] & MPM_NF_FIX_Y) {
            s->g_vel[3 * i + 1] = 0.0;
            p[1] = 0.0;
            s->g_force_temp[3 * i + 1] += f[1];
            f[1] = 0.0;
        }
        if (s->fixed[i] & MPM_NF_FIX_Z) zero_fixed(s, i, 2);
        for (int c = 0; c < 3; ++c) p[c] = p[c] + f[c] * dt;
        friction_work(s, w, i, dfr);
    }
}

/* IntegrateGrid, contact form (…_Contact.cpp:242-277), with the optional floor friction. */
static void integrate_grid_contact(mpmsnap* s, work* w, double dt, int floor_friction) {
#pragma omp for
    for (long li = 0; li < (long)s->h.n_nodes; ++li) {
        size_t i = (size_t)li;
        if (!(s->g_state[i] & MPM_NS_ACTIVE)) continue;
        double* p = &s->g_mom[3 * i];
        double* f = &s->g_force[3 * i];
        damping(s, i);
        double dfr[3] = {0.0, 0.0, 0.0};
        if (floor_friction && (s->fixed[i] & MPM_NF_FIX_Z) && s->friction[i] > 0.0 && f[2] < 0.0) {
            double fz = f[2];
            for (int t = 0; t < 2; ++t) {
                double trial_t = p[t] + f[t] * dt;
                if (gabs(trial_t * dt) > 1.0e-24) {
                    double f0 = f[t];
                    coulomb(s, i, t, fz, dt);
                    dfr[t] = f[t] - f0;
                }
            }
        }
        for (int c = 0; c < 3; ++c) p[c] = p[c] + f[c] * dt;
        if (s->fixed[i] & MPM_NF_FIX_X) zero_fixed(s, i, 0);
        if (s->fixed[i] & MPM_NF_FIX_Y) {
            s->g_vel[3 * i + 1] = 0.0;
            p[1] = 0.0;
            s->g_force_temp[3 * i + 1] += f[1];
            f[1] = 0.0;
        }
        if (s->fixed[i] & MPM_NF_FIX_Z) zero_fixed(s, i, 2);
        friction_work(s, w, i, dfr);
    }
}

/* BC reapply (…MPLocks.cpp:573-599; contact :383-410) */
static void reapply_bc(mpmsnap* s) {
#pragma omp for
    for (long li = 0; li < (long)s->h.n_nodes; ++li) {
        size_t i = (size_t)li;
        if (!(s->g_state[i] & MPM_NS_ACTIVE)) continue;
        for (int c = 0; c < 3; ++c)
            if (s->fixed[i] & (1u << c)) zero_fixed(s, i, c);
    }
}

static void reset_grid(mpmsnap* s, int contact) {
#pragma omp for
    for (long li = 0; li < (long)s->h.n_nodes; ++li) {
        size_t i = (size_t)li;
        if (!(s->g_state[i] & MPM_NS_ACTIVE)) continue;
        s->g_state[i] = contact ? 0 : (uint8_t)(s->g_state[i] & ~MPM_NS_ACTIVE);
        s->g_mass[i] = 0.0;
        for (int c = 0; c < 3; ++c) {
            if (contact) s->g_mass_gradient[3 * i + c] = 0.0;
            s->g_vel[3 * i + c] = 0.0;
            s->g_mom[3 * i + c] = 0.0;
            s->g_force[3 * i + c] = 0.0;
            s->g_force_temp[3 * i + c] = 0.0;
        }
    }
}

/* M2G (…MPLocks.cpp:48-89; contact :110-150 adds the mass gradient) */
static void p2g(mpmsnap* s, work* w, int contact) {
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        const double m = s->mass[p];
        const double* v = &s->vel[3 * p];
        const double* sg = &s->stress[6 * p];
        const double* fe = &s->fext[3 * p];
        for (int j = 0; j < w->nagp[p]; ++j) {
            const agp* g = &w->agps[8 * p + j];
            size_t i = g->idx;
            double N = g->N;
            const double* G = g->G;
            LOCK(w, i);
            s->g_mass[i] += N * m;
            if (contact)
                for (int c = 0; c < 3; ++c) s->g_mass_gradient[3 * i + c] += G[c] * m;
            for (int c = 0; c < 3; ++c) s->g_mom[3 * i + c] += N * (m * v[c]);
            double V = s->vol[p];
            s->g_force[3 * i + 0] += -V * (G[0] * sg[0] + G[1] * sg[3] + G[2] * sg[5]);
            s->g_force[3 * i + 1] += -V * (G[1] * sg[1] + G[0] * sg[3] + G[2] * sg[4]);
            s->g_force[3 * i + 2] += -V * (G[2] * sg[2] + G[0] * sg[5] + G[1] * sg[4]);
            for (int c = 0; c < 3; ++c) s->g_force[3 * i + c] += N * fe[c];
            UNLOCK(w, i);
        }
    }
}

/* Contact detection phases (…_Contact.cpp:152-237) */
static void contact_phases(mpmsnap* s, work* w) {
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        if (!(s->pflags[p] & MPM_PF_SURFACE)) continue;
        double* gp = &s->mp_mass_gradient[3 * p];
        gp[0] = gp[1] = gp[2] = 0.0;
        for (int j = 0; j < w->nagp[p]; ++j) {
            const double* gi = &s->g_mass_gradient[3 * (size_t)w->agps[8 * p + j].idx];
            if (len3(gi) > len3(gp)) memcpy(gp, gi, 3 * sizeof(double));
        }
    }
#pragma omp for
    for (long li = 0; li < (long)s->h.n_nodes; ++li) {
        size_t i = (size_t)li;
        if (!(s->g_state[i] & MPM_NS_ACTIVE)) continue;
        s->g_mass_gradient[3 * i + 0] = s->g_mass_gradient[3 * i + 1] = s->g_mass_gradient[3 * i + 2] = 0.0;
    }
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        if (!(s->pflags[p] & MPM_PF_SURFACE)) continue;
        const double* gp = &s->mp_mass_gradient[3 * p];
        for (int j = 0; j < w->nagp[p]; ++j) {
            size_t i = w->agps[8 * p + j].idx;
            double d[3];
            for (int c = 0; c < 3; ++c) d[c] = w->xnode[3 * i + c] - s->pos[3 * p + c];
            if (dot3(d, gp) > 0.0) memcpy(&s->g_mass_gradient[3 * i], gp, 3 * sizeof(double));
        }
    }
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        if (!(s->pflags[p] & MPM_PF_SURFACE)) continue;
        const double* gp = &s->mp_mass_gradient[3 * p];
        for (int j = 0; j < w->nagp[p]; ++j) {
            size_t i = w->agps[8 * p + j].idx;
            const double* gi = &s->g_mass_gradient[3 * i];
            double tol = 0.001 * len3(gi) * len3(gp);
            double dd = dot3(gi, gp);
            if (dd >= tol)
                s->g_state[i] |= MPM_NS_POSITIVE;
            else if (dd <= -tol)
                s->g_state[i] |= MPM_NS_NEGATIVE;
        }
    }
}

/* G2P pass 1 (…MPLocks.cpp:489-510) and velocity remap (:539-564) */
static void g2p_pass1(mpmsnap* s, work* w, double dt, int skip_dc) {
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        if (skip_dc && (s->pflags[p] & MPM_PF_DC_SKIP)) continue;
        double* v = &s->vel[3 * p];
        for (int j = 0; j < w->nagp[p]; ++j) {
            const agp* g = &w->agps[8 * p + j];
            size_t i = g->idx;
            double mi = s->g_mass[i];
            if (mi > s->h.mass_min)
                for (int c = 0; c < 3; ++c) v[c] = v[c] + g->N * (s->g_force[3 * i + c] / mi) * dt;
        }
    }
}

static void remap(mpmsnap* s, work* w, int skip_dc) {
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        if (skip_dc && (s->pflags[p] & MPM_PF_DC_SKIP)) continue;
        const double m = s->mass[p];
        const double* v = &s->vel[3 * p];
        for (int j = 0; j < w->nagp[p]; ++j) {
            const agp* g = &w->agps[8 * p + j];
            size_t i = g->idx;
            LOCK(w, i);
            double mi = s->g_mass[i];
            if (mi > s->h.mass_min)
                for (int c = 0; c < 3; ++c) s->g_vel[3 * i + c] += g->N * (m * v[c]) / mi;
            UNLOCK(w, i);
        }
    }
}

/* glm dmat3 helpers, column-major F[c][r] at 3*c + r */
static void mat_mul(const double* A, const double* B, double* R) {
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) R[3 * c + r] = A[0 + r] * B[3 * c + 0] + A[3 + r] * B[3 * c + 1] + A[6 + r] * B[3 * c + 2];
}
static double mat_det(const double* m) {
    return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) + m[6] * (m[1] * m[5] - m[4] * m[2]);
}

/* Position update and velocity gradient shared by both pass-2 forms. */
static void gather_pass2(mpmsnap* s, work* w, size_t p, double dt, double L[9]) {
    double* x = &s->pos[3 * p];
    for (int k = 0; k < 9; ++k) L[k] = 0.0;
    for (int j = 0; j < w->nagp[p]; ++j) {
        const agp* g = &w->agps[8 * p + j];
        size_t i = g->idx;
        double mi = s->g_mass[i];
        if (mi > s->h.mass_min)
            for (int c = 0; c < 3; ++c) x[c] = x[c] + g->N * (s->g_mom[3 * i + c] / mi) * dt;
        /* outerProduct(v_i, G): column c, row r = v_i[r] * G[c] */
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) L[3 * c + r] = L[3 * c + r] + s->g_vel[3 * i + r] * g->G[c];
    }
}

static const mpmsnap_material* material_of(const mpmsnap* s, size_t p) {
    int32_t m = s->material[p];
    if (m < 0 || (uint32_t)m >= s->h.n_materials) return NULL;
    return &s->materials[m];
}

/* G2P_P2_SmallStrain (…MPLocks.cpp:175-280) */
static void g2p_pass2(mpmsnap* s, work* w, double dt) {
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        double L[9], dF[9], S[9], e[6];
        gather_pass2(s, w, p, dt, L);
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) dF[3 * c + r] = (c == r ? 1.0 : 0.0) + L[3 * c + r] * dt;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) S[3 * c + r] = 0.5 * (dF[3 * r + c] + dF[3 * c + r]) - (c == r ? 1.0 : 0.0);
        e[0] = S[0];
        e[1] = S[4];
        e[2] = S[8];
        e[3] = S[1] + S[3];
        e[4] = S[5] + S[7];
        e[5] = S[6] + S[2];
        const mpmsnap_material* mat = material_of(s, p);
        if (!mat) continue;
        cr_out o;
        cr_increment(mat, s->backstress[p], &s->stress[6 * p], e, &o);
        double Fn[9];
        mat_mul(&s->F[9 * p], dF, Fn);
        memcpy(&s->F[9 * p], Fn, sizeof(Fn));
        double det = mat_det(&s->F[9 * p]);
        s->vol[p] = det * s->vol0[p];
        for (int k = 0; k < 6; ++k) s->strain[6 * p + k] += e[k];
        for (int k = 0; k < 6; ++k) s->stress[6 * p + k] += o.dsig[k];
        for (int k = 0; k < 6; ++k) s->eps_p[6 * p + k] += o.deps_p[k];
        double dEs = 0.0;
        for (int k = 0; k < 6; ++k) dEs += (s->stress[6 * p + k] - 0.5 * o.dsig[k]) * e[k] * s->vol[p];
        s->e_strain[p] += dEs;
        s->e_strain_ti[p] += s->e_strain[p] * dt;
        if (s->e_strain[p] > s->e_strain_max[p]) s->e_strain_max[p] = s->e_strain[p];
        double dEp = 0.0;
        for (int k = 0; k < 6; ++k) dEp += (s->stress[6 * p + k] - 0.5 * o.dsig[k]) * o.deps_p[k] * s->vol[p];
        s->e_plastic[p] += dEp;
        s->backstress[p] += o.dR;
    }
}

/* The matrix series of the large-strain pass
 * (ConstitutiveRelation_MatrixAlgebra.cpp:25-53): log A = sum over n = 1..8 of
 * (-1)^(n+1) (A - I)^n / n, exp A = sum over n = 0..8 of A^n / n!.  Each power
 * is the previous one times the base (getPower multiplies I by the base n
 * times), so every term is the reference's. */
static void mat_log8(const double* A, double* R) {
    double B[9], P[9], T[9];
    for (int k = 0; k < 9; ++k) {
        const double I = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
        B[k] = A[k] - I;
        P[k] = I;
        R[k] = 0.0;
    }
    for (int n = 1; n <= 8; ++n) {
        mat_mul(P, B, T);
        memcpy(P, T, sizeof(P));
        const double inv = 1.0 / n, sign = (n & 1) ? 1.0 : -1.0;
        for (int k = 0; k < 9; ++k) R[k] = R[k] + (P[k] * inv) * sign;
    }
}
static void mat_exp8(const double* A, double* R) {
    double P[9], T[9], fact = 1.0;
    for (int k = 0; k < 9; ++k) {
        P[k] = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
        R[k] = 0.0 + P[k] / 1.0;
    }
    for (int n = 1; n <= 8; ++n) {
        mat_mul(P, A, T);
        memcpy(P, T, sizeof(P));
        fact *= n;
        for (int k = 0; k < 9; ++k) R[k] = R[k] + P[k] / fact;
    }
}
/* 0.5 log(M M^T) in Voigt order with engineering shear */
static void half_log_voigt(const double* M, double v[6]) {
    double Mt[9], MMt[9], lg[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Mt[3 * c + r] = M[3 * r + c];
    mat_mul(M, Mt, MMt);
    mat_log8(MMt, lg);
    for (int k = 0; k < 9; ++k) lg[k] = 0.5 * lg[k];
    v[0] = lg[0];
    v[1] = lg[4];
    v[2] = lg[8];
    v[3] = lg[1] + lg[3];
    v[4] = lg[5] + lg[7];
    v[5] = lg[6] + lg[2];
}

/* G2P_P2_LargeStrain (…MPLocks.cpp:281-437), disabled in the reference's loop
 * (:605): logarithmic strains of F F^T, of the trial elastic gradient and of
 * the increment; the constitutive map takes zero stress and the trial elastic
 * strain and returns the Kirchhoff stress; F_e = exp of the elastic strain. */
static void g2p_pass2_large_strain(mpmsnap* s, work* w, double dt) {
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        double L[9], dF[9], et[6], ee[6], einc[6];
        gather_pass2(s, w, p, dt, L);
        for (int k = 0; k < 6; ++k) s->stress[6 * p + k] = 0.0;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) dF[3 * c + r] = (c == r ? 1.0 : 0.0) + L[3 * c + r] * dt;
        double* F = &s->F[9 * p];
        double* Fe = &s->F_elastic[9 * p];
        half_log_voigt(F, et);
        double Fet[9];
        mat_mul(dF, Fe, Fet);
        half_log_voigt(Fet, ee);
        half_log_voigt(dF, einc);
        const mpmsnap_material* mat = material_of(s, p);
        if (!mat) continue;
        cr_out o;
        cr_increment(mat, s->backstress[p], &s->stress[6 * p], ee, &o);
        double el[6], E[9];
        for (int k = 0; k < 6; ++k) el[k] = ee[k] - o.deps_p[k];
        E[0] = el[0];
        E[4] = el[1];
        E[8] = el[2];
        E[3] = E[1] = 0.5 * el[3]; /* [1][0] and [0][1] */
        E[7] = E[5] = 0.5 * el[4]; /* [2][1] and [1][2] */
        E[2] = E[6] = 0.5 * el[5]; /* [0][2] and [2][0] */
        mat_exp8(E, Fe);
        double Fn[9];
        mat_mul(F, dF, Fn);
        memcpy(F, Fn, sizeof(Fn));
        const double det = mat_det(F);
        s->vol[p] = det * s->vol0[p];
        for (int k = 0; k < 6; ++k) s->strain[6 * p + k] = et[k];
        for (int k = 0; k < 6; ++k) s->stress[6 * p + k] = (1.0 / det) * o.dsig[k];
        for (int k = 0; k < 6; ++k) s->eps_p[6 * p + k] += o.deps_p[k];
        for (int k = 0; k < 6; ++k) s->e_strain[p] += s->stress[6 * p + k] * einc[k] * s->vol[p];
        for (int k = 0; k < 6; ++k) s->e_plastic[p] += s->stress[6 * p + k] * o.deps_p[k] * s->vol[p];
        s->backstress[p] += o.dR;
    }
}

/* Contact pass 2 (…_Contact.cpp:438-525) */
static void g2p_pass2_contact(mpmsnap* s, work* w, double dt) {
#pragma omp for
    for (long lp = 0; lp < (long)s->h.n_particles; ++lp) {
        size_t p = (size_t)lp;
        if (s->pflags[p] & MPM_PF_DC_SKIP) continue;
        double L[9], M[9], dF[9], e[6];
        gather_pass2(s, w, p, dt, L);
        double* F = &s->F[9 * p];
        mat_mul(L, F, M);
        for (int k = 0; k < 9; ++k) F[k] += M[k] * dt;
        double det = mat_det(F);
        s->vol[p] = det * s->vol0[p];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) dF[3 * c + r] = (c == r ? 1.0 : 0.0) + L[3 * c + r] * dt;
        e[0] = dF[0] - 1.0;
        e[1] = dF[4] - 1.0;
        e[2] = dF[8] - 1.0;
        e[3] = dF[1] + dF[3];
        e[4] = dF[5] + dF[7];
        e[5] = dF[6] + dF[2];
        for (int k = 0; k < 6; ++k) s->strain[6 * p + k] += e[k];
        const mpmsnap_material* mat = material_of(s, p);
        if (!mat) continue;
        cr_out o;
        cr_increment(mat, s->backstress[p], &s->stress[6 * p], e, &o);
        for (int k = 0; k < 6; ++k) s->strain_rate[6 * p + k] = e[k] / dt;
        for (int k = 0; k < 6; ++k) s->stress[6 * p + k] += o.dsig[k];
        for (int k = 0; k < 6; ++k) s->eps_p[6 * p + k] += o.deps_p[k];
        for (int k = 0; k < 6; ++k) s->e_strain[p] += s->stress[6 * p + k] * e[k] * s->vol[p];
        for (int k = 0; k < 6; ++k) s->e_plastic[p] += s->stress[6 * p + k] * o.deps_p[k] * s->vol[p];
        s->backstress[p] += o.dR;
    }
}

/* Contact displacement control (…_Contact.cpp:283-297, :416-432): all axes. */
static void displacement_control_contact(mpmsnap* s, work* w) {
#pragma omp for
    for (long k = 0; k < (long)s->h.n_dc; ++k) {
        size_t p = s->dc_list[k];
        for (int j = 0; j < w->nagp[p]; ++j) {
            size_t i = w->agps[8 * p + j].idx;
            for (int c = 0; c < 3; ++c) {
                s->g_vel[3 * i + c] = s->vel[3 * p + c];
                s->g_mom[3 * i + c] = s->g_mass[i] * s->vel[3 * p + c];
                s->g_force[3 * i + c] = 0.0;
            }
        }
    }
}

/* One time step at time t with increment dt. */
static void step(mpmsnap* s, work* w, double dt, const oracle_opts* o) {
    double tv[3];
    timeline_velocity(s, s->h.time, tv);
    /* contact 2: the non-contact loop with the large-strain pass 2 */
    const int large = o->contact == 2;
    const int contact = o->contact == 1;
#pragma omp parallel
    {
        reset_grid(s, contact);
#pragma omp barrier
#pragma omp for
        for (long lp = 0; lp < (long)s->h.n_particles; ++lp) find_agps(s, w, (size_t)lp);
        p2g(s, w, contact);
        if (!contact) {
            dc_work_begin(s, w, 0);
            displacement_control(s, w);
            dc_work_end(s, w);
            integrate_grid(s, w, dt);
            g2p_pass1(s, w, dt, 0);
            remap(s, w, 0);
            displacement_control(s, w);
            reapply_bc(s);
            if (large)
                g2p_pass2_large_strain(s, w, dt);
            else
                g2p_pass2(s, w, dt);
#pragma omp for
            for (long k = 0; k < (long)s->h.n_dc; ++k) {
                size_t p = s->dc_list[k];
                if (s->h.n_timeline != 0)
                    for (int c = 0; c < 3; ++c)
                        if (s->pflags[p] & (1u << c)) s->vel[3 * p + c] = (double)s->dc_mult[p] * tv[c];
            }
        } else {
            contact_phases(s, w);
            integrate_grid_contact(s, w, dt, o->floor_friction);
            dc_work_begin(s, w, 1);
            displacement_control_contact(s, w);
            dc_work_end(s, w);
            g2p_pass1(s, w, dt, 1);
            remap(s, w, 1);
            reapply_bc(s);
            displacement_control_contact(s, w);
            g2p_pass2_contact(s, w, dt);
#pragma omp for
            for (long k = 0; k < (long)s->h.n_dc; ++k) {
                size_t p = s->dc_list[k];
                if (s->h.n_timeline != 0)
                    for (int c = 0; c < 3; ++c) s->vel[3 * p + c] = (double)s->dc_mult[p] * tv[c];
                for (int c = 0; c < 3; ++c) s->pos[3 * p + c] += s->vel[3 * p + c] * dt;
            }
        }
    }
    if (w->bw) {
        w->bw[0] += w->bw_dc * dt;
        w->bw[1] += w->bw_fr * dt;
        w->bw_dc = w->bw_fr = 0.0;
    }
    s->h.time += dt;
    s->h.step += 1;
}

/* ---- public entry points ------------------------------------------------ */
int oracle_threads_available(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Advance the state in place by `steps` steps of s->h.dt_max.  Returns 0 on
 * success; *seconds (if given) receives the wall time of the step loop. */
int oracle_advance(mpmsnap* s, int steps, int contact, int floor_friction, int threads, double* seconds) {
    oracle_opts o = {contact, floor_friction, threads};
    work w;
    if (work_init(&w, s) != 0) return -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
    double t0 = omp_get_wtime();
#else
    (void)threads;
#endif
    for (int k = 0; k < steps; ++k) step(s, &w, s->h.dt_max, &o);
#ifdef _OPENMP
    if (seconds) *seconds = omp_get_wtime() - t0;
#else
    if (seconds) *seconds = 0.0;
#endif
    s->h.contact = (uint32_t)contact;
    work_free(&w, s);
    return 0;
}

/* As oracle_advance in the one-thread build, also adding the steps' boundary
 * work to bwork[0] (displacement control) and bwork[1] (friction). */
int oracle_advance_work(mpmsnap* s, int steps, int contact, int floor_friction, double* bwork) {
#ifdef _OPENMP
    (void)s, (void)steps, (void)contact, (void)floor_friction, (void)bwork;
    return -2; /* the work sums are restated in index order: one-thread build only */
#else
    oracle_opts o = {contact, floor_friction, 0};
    work w;
    if (work_init(&w, s) != 0) return -1;
    size_t nn = (size_t)s->h.n_nodes;
    w.bw = bwork;
    w.fsave = (double*)malloc(sizeof(double) * 3 * (nn ? nn : 1));
    w.dcax = (uint8_t*)calloc(nn ? nn : 1, 1);
    if (!w.fsave || !w.dcax) {
        work_free(&w, s);
        return -1;
    }
    for (int k = 0; k < steps; ++k) step(s, &w, s->h.dt_max, &o);
    s->h.contact = (uint32_t)contact;
    work_free(&w, s);
    return 0;
#endif
}

/* File form: read in_path, advance, write out_path. */
int oracle_run_file(const char* in_path, const char* out_path, int steps, int contact, int floor_friction) {
    mpmsnap s;
    int rc = mpmsnap_read(in_path, &s);
    if (rc != 0) return rc;
    rc = oracle_advance(&s, steps, contact, floor_friction, 0, NULL);
    if (rc == 0) rc = mpmsnap_write(out_path, &s);
    mpmsnap_free(&s);
    return rc;
}

#ifdef MPM_ORACLE_MAIN
int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s in.snap out.snap steps contact [floor_friction]\n", argv[0]);
        return 2;
    }
    return oracle_run_file(argv[1], argv[2], atoi(argv[3]), atoi(argv[4]), argc > 5 ? atoi(argv[5]) : 0) == 0 ? 0 : 1;
}
#endif
