/*
 * oxdna_oracle.c - FP64 CPU oracle (test infrastructure; see oxdna_oracle.h).
 *
 * Every routine restates the reference plugin's arithmetic in double precision and
 * cites the reference file:line it follows (paths relative to the hoomd-oxDNA tree).
 * The HOOMD semantics the reference relies on (driver loop, minimum image, bond
 * exclusions, 0.5*E split, Langevin) are restated from HOOMD-blue's documented
 * behaviour and the reference's call sites.
 */
#include "oxdna_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------- vector algebra */
typedef struct { double x, y, z; } v3;
typedef struct { double s; v3 v; } qt;

static inline v3 V(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, double s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b)
{
    return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 vld(const double* p) { return V(p[0], p[1], p[2]); }
static inline void vst(double* p, v3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }
static inline void vacc(double* p, v3 a) { p[0] += a.x; p[1] += a.y; p[2] += a.z; }

static inline qt qld(const double* p) { qt q; q.s = p[0]; q.v = V(p[1], p[2], p[3]); return q; }
/* HOOMD's rotate(q, v) = (s^2 - u.u) v + 2 s (u x v) + 2 (u.v) u. The reference
 * relies on rotate(q, e_x) == a1 (oxdna/io.py:127-150). */
static inline v3 qrot(qt q, v3 a)
{
    double ss = q.s * q.s - vdot(q.v, q.v);
    v3 r = vmul(a, ss);
    r = vadd(r, vmul(vcross(q.v, a), 2.0 * q.s));
    r = vadd(r, vmul(q.v, 2.0 * vdot(q.v, a)));
    return r;
}

/* ------------------------------------------------------------ numerics (L1) --- */
/* src/OxDNANumerics.h:50-54 */
static double fene_energy(double dr, double eps, double delta2)
{
    return -0.5 * eps * log(1.0 - dr * dr / delta2);
}
/* src/OxDNANumerics.h:58-62 */
static double fene_force_prefactor(double dr, double rmod, double eps, double delta2)
{
    return -(eps * dr / (delta2 - dr * dr)) / rmod;
}
/* src/OxDNANumerics.h:76-107: smoothed LJ core; *fq = force on the q (second) site,
 * r = site_q - site_p. */
static double repulsive_lj(v3 r, double eps, double sigma, double rstar, double b, double rc,
                           v3* fq)
{
    double rsq = vdot(r, r);
    *fq = V(0, 0, 0);
    if (!(rsq < rc * rc))
        return 0.0;
    if (rsq > rstar * rstar) {
        double rmod = sqrt(rsq);
        double d = rmod - rc;
        *fq = vmul(r, -2.0 * eps * b * d / rmod);
        return eps * b * d * d;
    }
    double s2 = sigma * sigma / rsq;
    double lj = s2 * s2 * s2;
    *fq = vmul(r, -24.0 * eps * (lj - 2.0 * lj * lj) / rsq);
    return 4.0 * eps * (lj * lj - lj);
}
/* f1 = (a, r0, rlow, rhigh, rclow, rchigh, blow, bhigh); src/OxDNANumerics.h:114-133 */
static double f1_val(double r, const double* f1, double eps, double shift)
{
    double a = f1[0], r0 = f1[1], rlow = f1[2], rhigh = f1[3], rclow = f1[4],
           rchigh = f1[5], blow = f1[6], bhigh = f1[7];
    if (!(r < rchigh))
        return 0.0;
    if (r > rhigh)
        return eps * bhigh * (r - rchigh) * (r - rchigh);
    if (r > rlow) {
        double t = 1.0 - exp(-(r - r0) * a);
        return eps * t * t - shift;
    }
    if (r > rclow)
        return eps * blow * (r - rclow) * (r - rclow);
    return 0.0;
}
/* src/OxDNANumerics.h:136-155 */
static double f1_deriv(double r, const double* f1, double eps)
{
    double a = f1[0], r0 = f1[1], rlow = f1[2], rhigh = f1[3], rclow = f1[4],
           rchigh = f1[5], blow = f1[6], bhigh = f1[7];
    double v = 0.0;
    if (r < rchigh) {
        if (r > rhigh)
            v = 2.0 * bhigh * (r - rchigh);
        else if (r > rlow) {
            double t = exp(-(r - r0) * a);
            v = 2.0 * (1.0 - t) * t * a;
        } else if (r > rclow)
            v = 2.0 * blow * (r - rclow);
    }
    return eps * v;
}
/* f2 = (k, r0, rc, rlow, rhigh, rclow, rchigh, blow, bhigh); src/OxDNANumerics.h:158-174 */
static double f2_val(double r, const double* f2)
{
    double k = f2[0], r0 = f2[1], rc = f2[2], rlow = f2[3], rhigh = f2[4], rclow = f2[5],
           rchigh = f2[6], blow = f2[7], bhigh = f2[8];
    if (!(r < rchigh))
        return 0.0;
    if (r > rhigh)
        return k * bhigh * (r - rchigh) * (r - rchigh);
    if (r > rlow)
        return 0.5 * k * ((r - r0) * (r - r0) - (rc - r0) * (rc - r0));
    if (r > rclow)
        return k * blow * (r - rclow) * (r - rclow);
    return 0.0;
}
/* src/OxDNANumerics.h:177-192 */
static double f2_deriv(double r, const double* f2)
{
    double k = f2[0], r0 = f2[1], rlow = f2[3], rhigh = f2[4], rclow = f2[5],
           rchigh = f2[6], blow = f2[7], bhigh = f2[8];
    if (!(r < rchigh))
        return 0.0;
    if (r > rhigh)
        return 2.0 * k * bhigh * (r - rchigh);
    if (r > rlow)
        return k * (r - r0);
    if (r > rclow)
        return 2.0 * k * blow * (r - rclow);
    return 0.0;
}
/* src/OxDNANumerics.h:194-198 */
static double clamp_cos(double c) { return c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c); }
/* f4 = (A, B, T0, TS, TC); src/OxDNANumerics.h:201-215 */
static double f4_angle(double t, const double* f4)
{
    double d = fabs(t - f4[2]);
    if (!(d < f4[4]))
        return 0.0;
    if (d > f4[3])
        return f4[1] * (f4[4] - d) * (f4[4] - d);
    return 1.0 - f4[0] * d * d;
}
/* (d f4 / d theta) / sin(theta); src/OxDNANumerics.h:218-244 */
static double f4_dsin_angle(double t, const double* f4)
{
    double d = t - f4[2];
    double m = 1.0;
    if (d < 0.0) {
        d = -d;
        m = -1.0;
    }
    if (!(d < f4[4]))
        return 0.0;
    double st = sin(t);
    if (d > f4[3])
        return m * 2.0 * f4[1] * (d - f4[4]) / st;
    if (st * st > 1e-8)
        return -m * 2.0 * f4[0] * d / st;
    return -m * 2.0 * f4[0];
}
/* f5 = (A, B, XC, XS); src/OxDNANumerics.h:261-274 */
static double f5_val(double f, const double* f5)
{
    if (!(f > f5[2]))
        return 0.0;
    if (f < f5[3])
        return f5[1] * (f5[2] - f) * (f5[2] - f);
    if (f < 0.0)
        return 1.0 - f5[0] * f * f;
    return 1.0;
}
/* src/OxDNANumerics.h:277-290 */
static double f5_deriv(double f, const double* f5)
{
    if (!(f > f5[2]))
        return 0.0;
    if (f < f5[3])
        return 2.0 * f5[1] * (f - f5[2]);
    if (f < 0.0)
        return -2.0 * f5[0] * f;
    return 0.0;
}

/* -------------------------------------------------- BASE-BASE machinery (L2) --- */
typedef struct { double val, dsin; } angf;

/* One acos per angle; the reflected branch uses pi - theta (src/OxDNABaseBase.h:52-67). */
static angf angular(double cost, const double* t, int symmetrize, double sign)
{
    double th = acos(clamp_cos(cost));
    angf a;
    a.val = f4_angle(th, t);
    double d = f4_dsin_angle(th, t);
    if (symmetrize) {
        double thn = M_PI - th;
        a.val += f4_angle(thn, t);
        d -= f4_dsin_angle(thn, t);
    }
    a.dsin = sign * d;
    return a;
}

typedef struct {
    int valid;
    v3 a1, a3, b1, b3, base_i, base_j, rdir;
    double rmod, c1, c2, c3, c4, c7, c8;
} bbgeom;

/* src/OxDNABaseBase.h:84-121 (rsq already tested by the caller). */
static bbgeom bb_geometry(v3 dr, qt qi, qt qj, const double* base_site)
{
    bbgeom g;
    memset(&g, 0, sizeof(g));
    g.a1 = qrot(qi, V(1, 0, 0));
    g.a3 = qrot(qi, V(0, 0, 1));
    g.b1 = qrot(qj, V(1, 0, 0));
    g.b3 = qrot(qj, V(0, 0, 1));
    v3 site = vld(base_site);
    g.base_i = qrot(qi, site);
    g.base_j = qrot(qj, site);
    v3 r = vadd(vsub(vneg(dr), g.base_i), g.base_j); /* r_j - r_i + base_j - base_i */
    g.rmod = sqrt(vdot(r, r));
    if (!(g.rmod > 0.0))
        return g;
    g.rdir = vmul(r, 1.0 / g.rmod);
    g.c1 = -vdot(g.a1, g.b1);
    g.c2 = -vdot(g.b1, g.rdir);
    g.c3 = vdot(g.a1, g.rdir);
    g.c4 = vdot(g.a3, g.b3);
    g.c7 = -vdot(g.b3, g.rdir);
    g.c8 = vdot(g.a3, g.rdir);
    g.valid = 1;
    return g;
}

/* radial factor: f1 Morse (kind 1, with eps and shift) or f2 harmonic (kind 2) */
typedef struct { int kind; const double* prm; double eps, shift; } radial;

static void radial_eval(const radial* R, double r, double* val, double* der)
{
    if (R->kind == 1) {
        *val = f1_val(r, R->prm, R->eps, R->shift);
        *der = f1_deriv(r, R->prm, R->eps);
    } else {
        *val = f2_val(r, R->prm);
        *der = f2_deriv(r, R->prm);
    }
}

/* One BASE-BASE term ADDED to the accumulators (force on i, torques lab frame).
 * src/OxDNABaseBase.h:128-219. */
static void bb_term(const bbgeom* g, const double* t1, const double* t23, const double* t4,
                    const double* t78, int sym, const radial* R, int include_t4, v3* facc,
                    double* eacc, v3* tiacc, v3* tjacc)
{
    angf A1 = angular(g->c1, t1, 0, -1.0);
    angf A2 = angular(g->c2, t23, 0, -1.0);
    angf A3 = angular(g->c3, t23, 0, 1.0);
    angf A4;
    if (include_t4)
        A4 = angular(g->c4, t4, sym, 1.0);
    else {
        A4.val = 1.0;
        A4.dsin = 0.0;
    }
    angf A7 = angular(g->c7, t78, sym, -1.0);
    angf A8 = angular(g->c8, t78, sym, 1.0);
    double prod = A1.val * A2.val * A3.val * A4.val * A7.val * A8.val;
    double rv, rd;
    radial_eval(R, g->rmod, &rv, &rd);
    double energy = rv * prod;
    *eacc += energy;
    if (energy == 0.0)
        return;

    v3 a1 = g->a1, a3 = g->a3, b1 = g->b1, b3 = g->b3, rdir = g->rdir;
    double rmod = g->rmod;
    v3 fq = vmul(rdir, -(rd * prod)); /* force on q = j */
    v3 tp = V(0, 0, 0), tq = V(0, 0, 0);

    /* theta4 */
    v3 dir = vcross(a3, b3);
    double tm = -rv * A1.val * A2.val * A3.val * A4.dsin * A7.val * A8.val;
    tp = vsub(tp, vmul(dir, tm));
    tq = vadd(tq, vmul(dir, tm));
    /* theta1 */
    dir = vcross(a1, b1);
    tm = -rv * A1.dsin * A2.val * A3.val * A4.val * A7.val * A8.val;
    tp = vsub(tp, vmul(dir, tm));
    tq = vadd(tq, vmul(dir, tm));
    /* theta2 */
    double fact = rv * A1.val * A2.dsin * A3.val * A4.val * A7.val * A8.val;
    fq = vadd(fq, vmul(vadd(b1, vmul(rdir, g->c2)), fact / rmod));
    tq = vsub(tq, vmul(vcross(rdir, b1), fact));
    /* theta3 */
    fact = rv * A1.val * A2.val * A3.dsin * A4.val * A7.val * A8.val;
    fq = vadd(fq, vmul(vsub(a1, vmul(rdir, g->c3)), fact / rmod));
    tp = vsub(tp, vmul(vcross(rdir, a1), fact));
    /* theta7 */
    fact = rv * A1.val * A2.val * A3.val * A4.val * A7.dsin * A8.val;
    fq = vadd(fq, vmul(vadd(b3, vmul(rdir, g->c7)), fact / rmod));
    tq = vsub(tq, vmul(vcross(rdir, b3), fact));
    /* theta8 */
    fact = rv * A1.val * A2.val * A3.val * A4.val * A7.val * A8.dsin;
    fq = vadd(fq, vmul(vsub(a3, vmul(rdir, g->c8)), fact / rmod));
    tp = vsub(tp, vmul(vcross(rdir, a3), fact));
    /* site offsets */
    tp = vsub(tp, vcross(g->base_i, fq));
    tq = vadd(tq, vcross(g->base_j, fq));

    *facc = vsub(*facc, fq);
    *tiacc = vadd(*tiacc, tp);
    *tjacc = vadd(*tjacc, tq);
}

static void zero_out(double f[3], double* e, double ti[3], double tj[3])
{
    f[0] = f[1] = f[2] = 0.0;
    ti[0] = ti[1] = ti[2] = 0.0;
    tj[0] = tj[1] = tj[2] = 0.0;
    *e = 0.0;
}

/* ---------------------------------------------------------- pair evaluators --- */
/* src/EvaluatorPairOxDNAExcVol.h:107-149 */
int oxo_excvol(const oxg_excvol_params* p, const double dr_[3], const double qi_[4],
               const double qj_[4], double rcutsq, double f[3], double* e, double ti[3],
               double tj[3])
{
    zero_out(f, e, ti, tj);
    v3 dr = vld(dr_);
    if (!(vdot(dr, dr) < rcutsq))
        return 0;
    qt qi = qld(qi_), qj = qld(qj_);
    v3 base_i = qrot(qi, vld(p->base_site)), back_i = qrot(qi, vld(p->back_site));
    v3 base_j = qrot(qj, vld(p->base_site)), back_j = qrot(qj, vld(p->back_site));
    v3 rc = vneg(dr);
    const v3* si[4] = {&back_i, &base_i, &base_i, &back_i};
    const v3* sj[4] = {&back_j, &base_j, &back_j, &base_j};
    v3 F = V(0, 0, 0), Ti = V(0, 0, 0), Tj = V(0, 0, 0);
    double E = 0.0;
    for (int k = 0; k < 4; ++k) {
        v3 r = vsub(vadd(rc, *sj[k]), *si[k]);
        v3 fq;
        E += repulsive_lj(r, p->eps, p->sigma[k], p->rstar[k], p->b[k], p->rc[k], &fq);
        F = vsub(F, fq);
        Ti = vadd(Ti, vcross(*si[k], vneg(fq)));
        Tj = vadd(Tj, vcross(*sj[k], fq));
    }
    vst(f, F);
    vst(ti, Ti);
    vst(tj, Tj);
    *e = E;
    return 1;
}

static int bb_single(const double dr_[3], const double qi_[4], const double qj_[4],
                     double rcutsq, const double* base_site, const double* t1,
                     const double* t23, const double* t4, const double* t78, int sym,
                     const radial* R, int include_t4, double f[3], double* e, double ti[3],
                     double tj[3])
{
    /* src/OxDNABaseBase.h:223-261 */
    zero_out(f, e, ti, tj);
    v3 dr = vld(dr_);
    if (!(vdot(dr, dr) < rcutsq))
        return 0;
    bbgeom g = bb_geometry(dr, qld(qi_), qld(qj_), base_site);
    if (!g.valid)
        return 1;
    v3 F = V(0, 0, 0), Ti = V(0, 0, 0), Tj = V(0, 0, 0);
    double E = 0.0;
    bb_term(&g, t1, t23, t4, t78, sym, R, include_t4, &F, &E, &Ti, &Tj);
    vst(f, F);
    vst(ti, Ti);
    vst(tj, Tj);
    *e = E;
    return 1;
}

/* src/EvaluatorPairOxDNAHBond.h:104-116 (f1 radial, not symmetrised) */
int oxo_hbond(const oxg_hbond_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
              double tj[3])
{
    radial R = {1, p->f1, p->eps, p->eps * p->shift_factor};
    return bb_single(dr, qi, qj, rcutsq, p->base_site, p->t1, p->t23, p->t4, p->t78, 0, &R,
                     1, f, e, ti, tj);
}

/* src/EvaluatorPairOxDNACrossStacking.h:101-113 (f2 radial, symmetrised t4/t7/t8) */
int oxo_cross(const oxg_cross_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
              double tj[3])
{
    radial R = {2, p->f2, 0.0, 0.0};
    return bb_single(dr, qi, qj, rcutsq, p->base_site, p->t1, p->t23, p->t4, p->t78, 1, &R,
                     p->t4_enabled != 0, f, e, ti, tj);
}

/* src/EvaluatorPairOxDNAHBondCross.h:138-178 (one geometry, both terms) */
int oxo_hbondcross(const oxg_hbondcross_params* p, const double dr_[3], const double qi_[4],
                   const double qj_[4], double rcutsq, double f[3], double* e, double ti[3],
                   double tj[3])
{
    zero_out(f, e, ti, tj);
    v3 dr = vld(dr_);
    if (!(vdot(dr, dr) < rcutsq))
        return 0;
    bbgeom g = bb_geometry(dr, qld(qi_), qld(qj_), p->base_site);
    if (!g.valid)
        return 1;
    v3 F = V(0, 0, 0), Ti = V(0, 0, 0), Tj = V(0, 0, 0);
    double E = 0.0;
    radial hb = {1, p->f1, p->eps, p->eps * p->shift_factor};
    bb_term(&g, p->hb_t1, p->hb_t23, p->hb_t4, p->hb_t78, 0, &hb, 1, &F, &E, &Ti, &Tj);
    radial cs = {2, p->f2, 0.0, 0.0};
    bb_term(&g, p->cs_t1, p->cs_t23, p->cs_t4, p->cs_t78, 1, &cs, 1, &F, &E, &Ti, &Tj);
    vst(f, F);
    vst(ti, Ti);
    vst(tj, Tj);
    *e = E;
    return 1;
}

/* src/EvaluatorPairOxDNACoaxStacking.h:134-372 */
int oxo_coax(const oxg_coax_params* p, const double dr_[3], const double qi_[4],
             const double qj_[4], double rcutsq, double f[3], double* e, double ti[3],
             double tj[3])
{
    zero_out(f, e, ti, tj);
    v3 dr = vld(dr_);
    if (!(vdot(dr, dr) < rcutsq))
        return 0;
    qt qi = qld(qi_), qj = qld(qj_);
    v3 a1 = qrot(qi, V(1, 0, 0)), a2 = qrot(qi, V(0, 1, 0)), a3 = qrot(qi, V(0, 0, 1));
    v3 b1 = qrot(qj, V(1, 0, 0)), b3 = qrot(qj, V(0, 0, 1));
    v3 stack_i = qrot(qi, vld(p->stack_site)), stack_j = qrot(qj, vld(p->stack_site));
    v3 bref_i = qrot(qi, vld(p->stack_back_ref)), bref_j = qrot(qj, vld(p->stack_back_ref));
    v3 rc = vneg(dr);
    v3 rstack = vsub(vadd(rc, stack_j), stack_i);
    double rsm = sqrt(vdot(rstack, rstack));
    if (!(rsm > 0.0))
        return 1;
    v3 rsd = vmul(rstack, 1.0 / rsm);
    double c1 = -vdot(a1, b1), c4 = vdot(a3, b3), c5 = vdot(a3, rsd), c6 = -vdot(b3, rsd);
    v3 rbr = vsub(vadd(rc, bref_j), bref_i);
    double rbm = sqrt(vdot(rbr, rbr));
    v3 rbd = vmul(rbr, 1.0 / rbm);
    double cphi3 = vdot(rsd, vcross(rbd, a1));

    double f2 = f2_val(rsm, p->f2);
    double th1 = acos(clamp_cos(c1));
    double th4 = acos(clamp_cos(c4));
    double th5 = acos(clamp_cos(c5)), th6 = acos(clamp_cos(c6));
    double th5n = M_PI - th5, th6n = M_PI - th6;

    double f4t1 = f4_angle(th1, p->t1);
    if (p->t1_mode == 0)
        f4t1 += f4_angle(2.0 * M_PI - th1, p->t1);
    else if (th1 > p->t1_sb)
        f4t1 += p->t1_sa * (th1 - p->t1_sb) * (th1 - p->t1_sb);
    double f4t4 = f4_angle(th4, p->t4);
    double f4t5 = f4_angle(th5, p->t56) + f4_angle(th5n, p->t56);
    double f4t6 = f4_angle(th6, p->t56) + f4_angle(th6n, p->t56);

    double f5p3 = 0.0, f5p4 = 0.0, cphi4 = 0.0, phif = 1.0;
    if (p->rna_coax) {
        cphi4 = vdot(rsd, vcross(rbd, b1));
        f5p3 = f5_val(cphi3, p->phi3);
        f5p4 = f5_val(cphi4, p->phi4);
        phif = f5p3 * f5p4;
    } else if (p->phi3_enabled) {
        f5p3 = f5_val(cphi3, p->phi3);
        phif = f5p3 * f5p3;
    }
    double energy = f2 * f4t1 * f4t4 * f4t5 * f4t6 * phif;
    *e = energy;
    if (energy == 0.0)
        return 1;

    double f2D = f2_deriv(rsm, p->f2);
    double f4t1D = -f4_dsin_angle(th1, p->t1);
    if (p->t1_mode == 0)
        f4t1D += -f4_dsin_angle(2.0 * M_PI - th1, p->t1);
    else if (th1 > p->t1_sb) {
        double s1 = sin(th1);
        double hd = (s1 * s1 > 1e-8) ? 2.0 * p->t1_sa * (th1 - p->t1_sb) / s1 : 2.0 * p->t1_sa;
        f4t1D += -hd;
    }
    double f4t4D = f4_dsin_angle(th4, p->t4);
    double f4t5D = f4_dsin_angle(th5, p->t56) - f4_dsin_angle(th5n, p->t56);
    double f4t6D = -f4_dsin_angle(th6, p->t56) + f4_dsin_angle(th6n, p->t56);

    v3 fq = vmul(rsd, -(f2D * f4t1 * f4t4 * f4t5 * f4t6 * phif));
    v3 tp = V(0, 0, 0), tq = V(0, 0, 0);
    /* theta1 */
    v3 dir = vcross(a1, b1);
    double tm = -f2 * f4t1D * f4t4 * f4t5 * f4t6 * phif;
    tp = vsub(tp, vmul(dir, tm));
    tq = vadd(tq, vmul(dir, tm));
    /* theta4 */
    dir = vcross(a3, b3);
    tm = -f2 * f4t1 * f4t4D * f4t5 * f4t6 * phif;
    tp = vsub(tp, vmul(dir, tm));
    tq = vadd(tq, vmul(dir, tm));
    /* theta5 */
    double fact = f2 * f4t1 * f4t4 * f4t5D * f4t6 * phif;
    fq = vadd(fq, vmul(vsub(a3, vmul(rsd, c5)), fact / rsm));
    tp = vsub(tp, vmul(vcross(rsd, a3), fact));
    /* theta6 */
    fact = f2 * f4t1 * f4t4 * f4t5 * f4t6D * phif;
    fq = vadd(fq, vmul(vadd(b3, vmul(rsd, c6)), fact / rsm));
    tq = vsub(tq, vmul(vcross(rsd, b3), fact));

    if (p->rna_coax) {
        /* oxRNA two dihedrals from the real BACK-BACK vector (:282-317) */
        tp = vsub(tp, vcross(stack_i, fq));
        tq = vadd(tq, vcross(stack_j, fq));
        double base = f2 * f4t1 * f4t4 * f4t5 * f4t6;
        double f5D3 = f5_deriv(cphi3, p->phi3), f5D4 = f5_deriv(cphi4, p->phi4);
        for (int w = 0; w < 2; ++w) {
            v3 v = (w == 0) ? a1 : b1;
            double fc = (w == 0) ? base * f5p4 * f5D3 : base * f5p3 * f5D4;
            v3 rbv = vcross(rbd, v);
            v3 vrs = vcross(v, rsd);
            v3 fs = vmul(vsub(rbv, vmul(rsd, vdot(rsd, rbv))), -fc / rsm);
            v3 fb = vmul(vsub(vrs, vmul(rbd, vdot(rbd, vrs))), -fc / rbm);
            fq = vadd(fq, vadd(fs, fb));
            tp = vsub(tp, vadd(vcross(stack_i, fs), vcross(bref_i, fb)));
            tq = vadd(tq, vadd(vcross(stack_j, fs), vcross(bref_j, fb)));
            v3 pure = vmul(vcross(v, vcross(rsd, rbd)), fc);
            if (w == 0)
                tp = vsub(tp, pure);
            else
                tq = vsub(tq, pure);
        }
        vst(f, vneg(fq));
        vst(ti, tp);
        vst(tj, tq);
        return 1;
    }

    if (p->phi3_enabled) {
        /* oxDNA1 phi3 dihedral (:320-361) */
        double f5D3 = f5_deriv(cphi3, p->phi3);
        double g = p->gamma, g3 = g * g * g;
        double rbm3 = rbm * rbm * rbm;
        double a2b1 = vdot(a2, b1), a3b1 = vdot(a3, b1);
        double ra1 = vdot(rsd, a1), ra2 = vdot(rsd, a2), ra3 = vdot(rsd, a3), rb1 = vdot(rsd, b1);
        double par = ra3 * a2b1 - ra2 * a3b1;
        double dcdr = -g * par * (g * (ra1 - rb1) + rsm) / rbm3;
        double dcda1b1 = g3 * par / rbm3;
        double dcda2b1 = g * ra3 / rbm;
        double dcda3b1 = -g * ra2 / rbm;
        double dcdra1 = -g * g * par * rsm / rbm3;
        double dcdra2 = -g * a3b1 / rbm;
        double dcdra3 = g * a2b1 / rbm;
        double dcdrb1 = g * g * par * rsm / rbm3;
        double fc = f2 * f4t1 * f4t4 * f4t5 * f4t6 * 2.0 * f5p3 * f5D3;
        v3 s = vmul(rsd, dcdr);
        v3 inner = vadd(vadd(vmul(vsub(a1, vmul(rsd, ra1)), dcdra1),
                             vmul(vsub(a2, vmul(rsd, ra2)), dcdra2)),
                        vadd(vmul(vsub(a3, vmul(rsd, ra3)), dcdra3),
                             vmul(vsub(b1, vmul(rsd, rb1)), dcdrb1)));
        s = vadd(s, vmul(inner, 1.0 / rsm));
        fq = vadd(fq, vmul(s, -fc));
        v3 tpa = vadd(vadd(vmul(vcross(rsd, a1), dcdra1), vmul(vcross(rsd, a2), dcdra2)),
                      vmul(vcross(rsd, a3), dcdra3));
        tp = vadd(tp, vmul(tpa, fc));
        tq = vadd(tq, vmul(vcross(rsd, b1), fc * dcdrb1));
        v3 pure = vmul(vadd(vadd(vmul(vcross(a1, b1), dcda1b1), vmul(vcross(a2, b1), dcda2b1)),
                            vmul(vcross(a3, b1), dcda3b1)),
                       fc);
        tp = vsub(tp, pure);
        tq = vadd(tq, pure);
    }
    tp = vsub(tp, vcross(stack_i, fq));
    tq = vadd(tq, vcross(stack_j, fq));
    vst(f, vneg(fq));
    vst(ti, tp);
    vst(tj, tq);
    return 1;
}

/* src/EvaluatorPairOxDNADebye.h:244-303 */
int oxo_debye(const oxg_debye_params* p, const double dr_[3], const double qi_[4],
              const double qj_[4], double rcutsq, double charge_i, double charge_j,
              double f[3], double* e, double ti[3], double tj[3])
{
    zero_out(f, e, ti, tj);
    v3 dr = vld(dr_);
    if (!(vdot(dr, dr) < rcutsq))
        return 0;
    qt qi = qld(qi_), qj = qld(qj_);
    v3 back_i = qrot(qi, vld(p->back_site)), back_j = qrot(qj, vld(p->back_site));
    v3 rb = vsub(vadd(vneg(dr), back_j), back_i);
    double rbm = sqrt(vdot(rb, rb));
    if (!(rbm > 0.0) || !(rbm < p->rc))
        return 1;
    double cut = charge_i * charge_j;
    v3 rbd = vmul(rb, 1.0 / rbm);
    double energy;
    v3 fq;
    if (rbm < p->rhigh) {
        double ex = exp(rbm * p->minus_kappa);
        energy = ex * (p->prefactor / rbm);
        fq = vmul(rbd, -(p->prefactor * ex) * (p->minus_kappa / rbm - 1.0 / (rbm * rbm)));
    } else {
        double d = rbm - p->rc;
        energy = p->b_smooth * d * d;
        fq = vmul(rbd, -2.0 * p->b_smooth * d);
    }
    energy *= cut;
    fq = vmul(fq, cut);
    *e = energy;
    vst(ti, vneg(vcross(back_i, fq)));
    vst(tj, vcross(back_j, fq));
    vst(f, vneg(fq));
    return 1;
}

/* ------------------------------------------------------------- bonded (L2) --- */
static void vir_acc(double vir[6], v3 r, v3 f)
{
    /* src/OxDNABondedKernel.h:48-58 */
    vir[0] += 0.5 * r.x * f.x;
    vir[1] += 0.5 * r.x * f.y;
    vir[2] += 0.5 * r.x * f.z;
    vir[3] += 0.5 * r.y * f.y;
    vir[4] += 0.5 * r.y * f.z;
    vir[5] += 0.5 * r.z * f.z;
}

/* DNA stacking, oxDNA p = B, q = A. src/OxDNABondedKernel.h:69-231 */
static double stacking_dna(const oxg_bonded_params* p, v3 Rc, qt qA, qt qB, int tA, int tB,
                           v3* FB, v3* tauA, v3* tauB, double vir[6])
{
    v3 a1 = qrot(qB, V(1, 0, 0)), a2 = qrot(qB, V(0, 1, 0)), a3 = qrot(qB, V(0, 0, 1));
    v3 b1 = qrot(qA, V(1, 0, 0)), b2 = qrot(qA, V(0, 1, 0)), b3 = qrot(qA, V(0, 0, 1));
    v3 stP = qrot(qB, vld(p->stack_site)), stQ = qrot(qA, vld(p->stack_site));
    v3 brP = qrot(qB, vld(p->stack_back_ref)), brQ = qrot(qA, vld(p->stack_back_ref));
    v3 Rpq = vneg(Rc);
    v3 rbr = vsub(vadd(Rpq, brQ), brP);
    double rbm = sqrt(vdot(rbr, rbr));
    v3 rs = vsub(vadd(Rpq, stQ), stP);
    double rsm = sqrt(vdot(rs, rs));
    v3 rsd = vmul(rs, 1.0 / rsm);
    double c4 = vdot(a3, b3), c5 = vdot(a3, rsd), c6 = -vdot(b3, rsd);
    double cp1 = vdot(a2, rbr) / rbm, cp2 = vdot(b2, rbr) / rbm;
    double eps = p->st_eps[tA][tB];
    double shift = eps * p->st_f1[8];
    double th4 = acos(clamp_cos(c4)), th5 = acos(clamp_cos(-c5)), th6 = acos(clamp_cos(c6));
    double f1 = f1_val(rsm, p->st_f1, eps, shift);
    double f4t4 = f4_angle(th4, p->t4), f4t5 = f4_angle(th5, p->t5), f4t6 = f4_angle(th6, p->t5);
    double f5p1 = f5_val(cp1, p->p1), f5p2 = f5_val(cp2, p->p1);
    double es = f1 * f4t4 * f4t5 * f4t6 * f5p1 * f5p2;
    if (es == 0.0)
        return es;
    double f1D = f1_deriv(rsm, p->st_f1, eps);
    double f4t4D = f4_dsin_angle(th4, p->t4), f4t5D = f4_dsin_angle(th5, p->t5),
           f4t6D = f4_dsin_angle(th6, p->t5);
    double f5p1D = f5_deriv(cp1, p->p1), f5p2D = f5_deriv(cp2, p->p1);

    v3 force = vmul(rsd, -(f1D * f4t4 * f4t5 * f4t6 * f5p1 * f5p2));
    force = vsub(force, vmul(vsub(a3, vmul(rsd, c5)), f1 * f4t4 * f4t5D * f4t6 * f5p1 * f5p2 / rsm));
    force = vsub(force, vmul(vadd(b3, vmul(rsd, c6)), f1 * f4t4 * f4t5 * f4t6D * f5p1 * f5p2 / rsm));

    double g = p->st_gamma, rbm3 = rbm * rbm * rbm;
    double ra2 = vdot(rsd, a2), ra1 = vdot(rsd, a1), rb1 = vdot(rsd, b1), a2b1 = vdot(a2, b1);
    double par = rsm * ra2 - a2b1 * g;
    double d1dr = (rsm * rsm * ra2 - ra2 * rbm * rbm - rsm * (a2b1 + ra2 * (-ra1 + rb1)) * g
                   + a2b1 * (-ra1 + rb1) * g * g) / rbm3;
    double d1dra1 = rsm * g * par / rbm3;
    double d1dra2 = -rsm / rbm;
    double d1drb1 = -rsm * g * par / rbm3;
    double d1da1b1 = -g * g * par / rbm3;
    double d1da2b1 = g / rbm;
    double fpp1 = -f1 * f4t4 * f4t5 * f4t6 * f5p1D * f5p2;
    v3 in1 = vadd(vadd(vmul(vsub(a2, vmul(rsd, ra2)), d1dra2), vmul(vsub(a1, vmul(rsd, ra1)), d1dra1)),
                  vmul(vsub(b1, vmul(rsd, rb1)), d1drb1));
    force = vsub(force, vmul(vadd(vmul(rsd, d1dr), vmul(in1, 1.0 / rsm)), fpp1));

    double r2a2 = vdot(rsd, b2), r2a1 = vdot(rsd, b1), r2b1 = vdot(rsd, a1), a2b1_2 = vdot(b2, a1);
    double par2 = rsm * r2a2 + a2b1_2 * g;
    double d2dr = (par2 * (rsm + (r2b1 - r2a1) * g) - r2a2 * rbm * rbm) / rbm3;
    double d2dra1 = -rsm * g * (rsm * r2a2 + a2b1_2 * g) / rbm3;
    double d2dra2 = -rsm / rbm;
    double d2drb1 = rsm * g * par2 / rbm3;
    double d2da1b1 = -g * g * par2 / rbm3;
    double d2da2b1 = -g / rbm;
    double fpp2 = -f1 * f4t4 * f4t5 * f4t6 * f5p1 * f5p2D;
    v3 in2 = vadd(vadd(vmul(vsub(b2, vmul(rsd, r2a2)), d2dra2), vmul(vsub(b1, vmul(rsd, r2a1)), d2dra1)),
                  vmul(vsub(a1, vmul(rsd, r2b1)), d2drb1));
    force = vsub(force, vmul(vadd(vmul(rsd, d2dr), vmul(in2, 1.0 / rsm)), fpp2));

    /* force is on q = A; B gets -force */
    *FB = vsub(*FB, force);
    vir_acc(vir, rs, force);

    v3 tp = V(0, 0, 0), tq = V(0, 0, 0);
    tp = vsub(tp, vcross(stP, force));
    tq = vadd(tq, vcross(stQ, force));
    v3 t4d = vcross(b3, a3);
    double tmod = f1 * f4t4D * f4t5 * f4t6 * f5p1 * f5p2;
    tp = vsub(tp, vmul(t4d, tmod));
    tq = vadd(tq, vmul(t4d, tmod));
    v3 t5d = vcross(rsd, a3);
    tmod = -f1 * f4t4 * f4t5D * f4t6 * f5p1 * f5p2;
    tp = vsub(tp, vmul(t5d, tmod));
    v3 t6d = vcross(rsd, b3);
    tmod = f1 * f4t4 * f4t5 * f4t6D * f5p1 * f5p2;
    tq = vadd(tq, vmul(t6d, tmod));

    tp = vadd(tp, vadd(vmul(vcross(rsd, a2), fpp1 * d1dra2), vmul(vcross(rsd, a1), fpp1 * d1dra1)));
    tq = vadd(tq, vmul(vcross(rsd, b1), fpp1 * d1drb1));
    v3 pure = vadd(vmul(vcross(a2, b1), fpp1 * d1da2b1), vmul(vcross(a1, b1), fpp1 * d1da1b1));
    tp = vsub(tp, pure);
    tq = vadd(tq, pure);

    tp = vadd(tp, vmul(vcross(rsd, a1), fpp2 * d2drb1));
    tq = vadd(tq, vadd(vmul(vcross(rsd, b2), fpp2 * d2dra2), vmul(vcross(rsd, b1), fpp2 * d2dra1)));
    pure = vadd(vmul(vcross(a1, b2), fpp2 * d2da2b1), vmul(vcross(a1, b1), fpp2 * d2da1b1));
    tp = vsub(tp, pure);
    tq = vadd(tq, pure);

    *tauB = vadd(*tauB, tp);
    *tauA = vadd(*tauA, tq);
    return es;
}

/* RNA stacking, p = B, q = A. src/OxDNABondedKernel.h:238-353 */
static double stacking_rna(const oxg_bonded_params* p, v3 Rc, qt qA, qt qB, int tA, int tB,
                           v3* FB, v3* tauA, v3* tauB, double vir[6])
{
    v3 a2 = qrot(qB, V(0, 1, 0)), a3 = qrot(qB, V(0, 0, 1));
    v3 b2 = qrot(qA, V(0, 1, 0)), b3 = qrot(qA, V(0, 0, 1));
    v3 stP = qrot(qB, vld(p->stack_3_site)), stQ = qrot(qA, vld(p->stack_5_site));
    v3 bkP = qrot(qB, vld(p->back_site)), bkQ = qrot(qA, vld(p->back_site));
    v3 bvP = qrot(qB, vld(p->bbvector_3)), bvQ = qrot(qA, vld(p->bbvector_5));
    v3 Rpq = vneg(Rc);
    v3 rs = vsub(vadd(Rpq, stQ), stP);
    double rsm = sqrt(vdot(rs, rs));
    v3 rsd = vmul(rs, 1.0 / rsm);
    v3 rb = vsub(vadd(Rpq, bkQ), bkP);
    double rbm = sqrt(vdot(rb, rb));
    v3 rbd = vmul(rb, 1.0 / rbm);
    double c5 = vdot(a3, rsd), c6 = -vdot(b3, rsd);
    double cB1 = -vdot(rbd, bvP), cB2 = -vdot(rbd, bvQ);
    double cp1 = vdot(a2, rb) / rbm, cp2 = vdot(b2, rb) / rbm;
    double eps = p->st_eps[tA][tB];
    double shift = eps * p->st_f1[8];
    double th5 = acos(clamp_cos(-c5)), th6 = acos(clamp_cos(c6));
    double thB1 = acos(clamp_cos(cB1)), thB2 = acos(clamp_cos(cB2));
    double f1 = f1_val(rsm, p->st_f1, eps, shift);
    double f4t5 = f4_angle(th5, p->t5), f4t6 = f4_angle(th6, p->t5);
    double f4B1 = f4_angle(thB1, p->tB1), f4B2 = f4_angle(thB2, p->tB2);
    double f5p1 = f5_val(cp1, p->p1), f5p2 = f5_val(cp2, p->p1);
    double es = f1 * f4t5 * f4t6 * f4B1 * f4B2 * f5p1 * f5p2;
    if (es == 0.0)
        return es;
    double f1D = f1_deriv(rsm, p->st_f1, eps);
    double f4t5D = f4_dsin_angle(th5, p->t5), f4t6D = f4_dsin_angle(th6, p->t5);
    double f4B1D = f4_dsin_angle(thB1, p->tB1), f4B2D = f4_dsin_angle(thB2, p->tB2);
    double f5p1D = f5_deriv(cp1, p->p1), f5p2D = f5_deriv(cp2, p->p1);

    v3 force = vmul(rsd, -(f1D * f4t5 * f4t6 * f4B1 * f4B2 * f5p1 * f5p2));
    force = vsub(force, vmul(vsub(a3, vmul(rsd, c5)), f1 * f4t5D * f4t6 * f4B1 * f4B2 * f5p1 * f5p2 / rsm));
    force = vsub(force, vmul(vadd(b3, vmul(rsd, c6)), f1 * f4t5 * f4t6D * f4B1 * f4B2 * f5p1 * f5p2 / rsm));

    v3 pb = V(0, 0, 0);
    pb = vsub(pb, vmul(vadd(bvP, vmul(rbd, cB1)), f1 * f4t5 * f4t6 * f4B1D * f4B2 * f5p1 * f5p2 / rbm));
    pb = vsub(pb, vmul(vadd(bvQ, vmul(rbd, cB2)), f1 * f4t5 * f4t6 * f4B1 * f4B2D * f5p1 * f5p2 / rbm));
    double fpp1 = -f1 * f4t5 * f4t6 * f4B1 * f4B2 * f5p1D * f5p2;
    pb = vadd(pb, vmul(vsub(a2, vmul(rb, cp1 / rbm)), fpp1 / rbm));
    double fpp2 = -f1 * f4t5 * f4t6 * f4B1 * f4B2 * f5p1 * f5p2D;
    pb = vadd(pb, vmul(vsub(b2, vmul(rb, cp2 / rbm)), fpp2 / rbm));

    *FB = vsub(*FB, vadd(force, pb));
    vir_acc(vir, rs, force);
    vir_acc(vir, rb, pb);

    v3 tp = V(0, 0, 0), tq = V(0, 0, 0);
    tp = vsub(tp, vcross(stP, force));
    tq = vadd(tq, vcross(stQ, force));
    tp = vsub(tp, vcross(bkP, pb));
    tq = vadd(tq, vcross(bkQ, pb));
    tp = vsub(tp, vmul(vcross(rsd, a3), -f1 * f4t5D * f4t6 * f4B1 * f4B2 * f5p1 * f5p2));
    tq = vadd(tq, vmul(vcross(rsd, b3), f1 * f4t5 * f4t6D * f4B1 * f4B2 * f5p1 * f5p2));
    tp = vadd(tp, vmul(vcross(rbd, bvP), f1 * f4t5 * f4t6 * f4B1D * f4B2 * f5p1 * f5p2));
    tq = vadd(tq, vmul(vcross(rbd, bvQ), f1 * f4t5 * f4t6 * f4B1 * f4B2D * f5p1 * f5p2));
    tp = vadd(tp, vmul(vcross(a2, rbd), fpp1));
    tq = vadd(tq, vmul(vcross(b2, rbd), fpp2));
    *tauB = vadd(*tauB, tp);
    *tauA = vadd(*tauA, tq);
    return es;
}

/* src/OxDNABondedKernel.h:357-431 */
void oxo_bonded(const oxg_bonded_params* p, const double Rc_[3], const double qA_[4],
                const double qB_[4], int typeA, int typeB, double FB_[3], double tauA_[3],
                double tauB_[3], double e[3], double vir[6])
{
    v3 Rc = vld(Rc_);
    qt qA = qld(qA_), qB = qld(qB_);
    v3 FB = V(0, 0, 0), tA = V(0, 0, 0), tB = V(0, 0, 0);
    e[0] = e[1] = e[2] = 0.0;
    for (int k = 0; k < 6; ++k)
        vir[k] = 0.0;

    /* FENE between BACK sites (always double; broken bond -> 1e12, no force) */
    v3 backA = qrot(qA, vld(p->back_site)), backB = qrot(qB, vld(p->back_site));
    v3 rback = vsub(vadd(Rc, backB), backA);
    double rmod = sqrt(vdot(rback, rback));
    double dr = rmod - p->r0_backbone;
    if (fabs(dr) >= p->delta_backbone) {
        e[0] = 1.0e12;
    } else {
        e[0] = fene_energy(dr, p->eps_backbone, p->delta2);
        v3 f = vmul(rback, fene_force_prefactor(dr, rmod, p->eps_backbone, p->delta2));
        FB = vadd(FB, f);
        tA = vadd(tA, vcross(backA, vneg(f)));
        tB = vadd(tB, vcross(backB, f));
        vir_acc(vir, rback, f);
    }
    /* bonded excluded volume: base-base, base(A)-back(B), back(A)-base(B) */
    v3 baseA = qrot(qA, vld(p->base_site)), baseB = qrot(qB, vld(p->base_site));
    const v3* si[3] = {&baseA, &baseA, &backA};
    const v3* sj[3] = {&baseB, &backB, &baseB};
    for (int k = 0; k < 3; ++k) {
        v3 r = vsub(vadd(Rc, *sj[k]), *si[k]);
        v3 f;
        e[1] += repulsive_lj(r, p->excl_eps, p->bx_sigma[k], p->bx_rstar[k], p->bx_b[k],
                             p->bx_rc[k], &f);
        FB = vadd(FB, f);
        tA = vadd(tA, vcross(*si[k], vneg(f)));
        tB = vadd(tB, vcross(*sj[k], f));
        vir_acc(vir, r, f);
    }
    if (p->stacking_enabled) {
        if (p->rna_stacking)
            e[2] = stacking_rna(p, Rc, qA, qB, typeA, typeB, &FB, &tA, &tB, vir);
        else
            e[2] = stacking_dna(p, Rc, qA, qB, typeA, typeB, &FB, &tA, &tB, vir);
    }
    vst(FB_, FB);
    vst(tauA_, tA);
    vst(tauB_, tB);
}

/* ------------------------------------------------------------ system driver --- */
static inline double min_image1(double d, double L) { return d - L * rint(d / L); }

static void min_image(const double* box, const double* a, const double* b, double out[3])
{
    for (int k = 0; k < 3; ++k)
        out[k] = min_image1(a[k] - b[k], box[k]);
}

/* Evaluate term t for the ordered pair (i, j); dr = r_i - r_j. Returns evaluated flag. */
static int eval_term(const oxo_model* m, const oxo_system* s, int t, int i, int j,
                     const double dr[3], double f[3], double* e, double ti[3], double tj[3])
{
    int a = s->type[i], b = s->type[j];
    int idx = a * m->n_types + b;
    double rc = m->r_cut[t][idx];
    double rcsq = rc * rc;
    const double* qi = s->quat + 4 * (size_t)i;
    const double* qj = s->quat + 4 * (size_t)j;
    switch (t) {
    case OXG_EXCVOL: return oxo_excvol(&m->excvol[idx], dr, qi, qj, rcsq, f, e, ti, tj);
    case OXG_HBOND: return oxo_hbond(&m->hbond[idx], dr, qi, qj, rcsq, f, e, ti, tj);
    case OXG_CROSS: return oxo_cross(&m->cross[idx], dr, qi, qj, rcsq, f, e, ti, tj);
    case OXG_HBONDCROSS: return oxo_hbondcross(&m->hbondcross[idx], dr, qi, qj, rcsq, f, e, ti, tj);
    case OXG_COAX: return oxo_coax(&m->coax[idx], dr, qi, qj, rcsq, f, e, ti, tj);
    case OXG_DEBYE: {
        double ci = s->charge ? s->charge[i] : 1.0, cj = s->charge ? s->charge[j] : 1.0;
        return oxo_debye(&m->debye[idx], dr, qi, qj, rcsq, ci, cj, f, e, ti, tj);
    }
    }
    return 0;
}

static int term_present(const oxo_model* m, int t)
{
    switch (t) {
    case OXG_EXCVOL: return m->excvol != NULL;
    case OXG_HBOND: return m->hbond != NULL;
    case OXG_CROSS: return m->cross != NULL;
    case OXG_HBONDCROSS: return m->hbondcross != NULL;
    case OXG_COAX: return m->coax != NULL;
    case OXG_DEBYE: return m->debye != NULL;
    }
    return 0;
}

static double max_rcut(const oxo_model* m, uint32_t mask)
{
    double r = 0.0;
    for (int t = 0; t < OXG_N_PAIR_TERMS; ++t) {
        if (!(mask & (1u << t)) || !term_present(m, t))
            continue;
        for (int k = 0; k < m->n_types * m->n_types; ++k)
            if (m->r_cut[t][k] > r)
                r = m->r_cut[t][k];
    }
    return r;
}

/* bond exclusion table: up to 4 bonded partners per particle */
#define OXO_MAX_EXCL 4
static int build_exclusions(const oxo_system* s, int* excl)
{
    for (int i = 0; i < s->N * OXO_MAX_EXCL; ++i)
        excl[i] = -1;
    for (int b = 0; b < s->n_bonds; ++b) {
        int A = s->bonds[3 * b], B = s->bonds[3 * b + 1];
        if (A < 0 || B < 0 || A >= s->N || B >= s->N)
            return -1;
        int ok = 0;
        for (int k = 0; k < OXO_MAX_EXCL; ++k)
            if (excl[A * OXO_MAX_EXCL + k] < 0) {
                excl[A * OXO_MAX_EXCL + k] = B;
                ok = 1;
                break;
            }
        for (int k = 0; k < OXO_MAX_EXCL && ok; ++k)
            if (excl[B * OXO_MAX_EXCL + k] < 0) {
                excl[B * OXO_MAX_EXCL + k] = A;
                ok = 2;
                break;
            }
        if (ok != 2)
            return -1;
    }
    return 0;
}

static inline int excluded(const int* excl, int i, int j)
{
    for (int k = 0; k < OXO_MAX_EXCL; ++k)
        if (excl[i * OXO_MAX_EXCL + k] == j)
            return 1;
    return 0;
}

/* Half neighbour list (j > i, bond-excluded) of radius rl: CSR arrays. */
typedef struct {
    int* start; /* N+1 */
    int* nbr;
    int cap;
} halflist;

static void halflist_free(halflist* h)
{
    free(h->start);
    free(h->nbr);
    h->start = NULL;
    h->nbr = NULL;
    h->cap = 0;
}

static int build_halflist(const oxo_system* s, const double* pos, const int* excl, double rl,
                          int brute_force, halflist* h)
{
    int N = s->N;
    double rl2 = rl * rl;
    int nc[3];
    int use_cells = !brute_force;
    for (int k = 0; k < 3; ++k) {
        nc[k] = (int)floor(s->box[k] / rl);
        if (nc[k] < 3)
            use_cells = 0;
    }
    if (!h->start)
        h->start = (int*)malloc(sizeof(int) * (N + 1));
    int* cell_of = NULL;
    int* cstart = NULL;
    int* cidx = NULL;
    int ncell = 1;
    if (use_cells) {
        ncell = nc[0] * nc[1] * nc[2];
        cell_of = (int*)malloc(sizeof(int) * N);
        cstart = (int*)calloc(ncell + 1, sizeof(int));
        cidx = (int*)malloc(sizeof(int) * N);
        for (int i = 0; i < N; ++i) {
            int c[3];
            for (int k = 0; k < 3; ++k) {
                double x = pos[3 * i + k] / s->box[k] + 0.5;
                x -= floor(x);
                c[k] = (int)(x * nc[k]);
                if (c[k] >= nc[k])
                    c[k] = nc[k] - 1;
            }
            cell_of[i] = (c[2] * nc[1] + c[1]) * nc[0] + c[0];
            cstart[cell_of[i] + 1]++;
        }
        for (int c = 0; c < ncell; ++c)
            cstart[c + 1] += cstart[c];
        int* fill = (int*)malloc(sizeof(int) * ncell);
        memcpy(fill, cstart, sizeof(int) * ncell);
        for (int i = 0; i < N; ++i)
            cidx[fill[cell_of[i]]++] = i;
        free(fill);
    }
    int cnt = 0;
    for (int pass = 0; pass < 2; ++pass) {
        cnt = 0;
        for (int i = 0; i < N; ++i) {
            if (pass == 1)
                h->start[i] = cnt;
            if (use_cells) {
                int ci = cell_of[i];
                int cx = ci % nc[0], cy = (ci / nc[0]) % nc[1], cz = ci / (nc[0] * nc[1]);
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            int x = (cx + dx + nc[0]) % nc[0], y = (cy + dy + nc[1]) % nc[1],
                                z = (cz + dz + nc[2]) % nc[2];
                            int c = (z * nc[1] + y) * nc[0] + x;
                            for (int q = cstart[c]; q < cstart[c + 1]; ++q) {
                                int j = cidx[q];
                                if (j <= i || excluded(excl, i, j))
                                    continue;
                                double d[3];
                                min_image(s->box, pos + 3 * i, pos + 3 * j, d);
                                if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] < rl2) {
                                    if (pass == 1)
                                        h->nbr[cnt] = j;
                                    cnt++;
                                }
                            }
                        }
            } else {
                for (int j = i + 1; j < N; ++j) {
                    if (excluded(excl, i, j))
                        continue;
                    double d[3];
                    min_image(s->box, pos + 3 * i, pos + 3 * j, d);
                    if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] < rl2) {
                        if (pass == 1)
                            h->nbr[cnt] = j;
                        cnt++;
                    }
                }
            }
        }
        if (pass == 0 && cnt > h->cap) {
            free(h->nbr);
            h->cap = cnt + cnt / 4 + 16;
            h->nbr = (int*)malloc(sizeof(int) * h->cap);
        }
    }
    h->start[N] = cnt;
    free(cell_of);
    free(cstart);
    free(cidx);
    return cnt;
}

/* Accumulate all selected forces. acc layout per particle: f(3) e(1) t(3) = 7 doubles. */
static void accumulate_forces(const oxo_model* m, const oxo_system* s, const halflist* h,
                              uint32_t mask, int bonded, double* acc, double* pair_energy,
                              double* bonded_energy, int64_t* pair_count, int n_threads)
{
    int N = s->N;
    int nt = n_threads > 0 ? n_threads : 1;
    double* priv = NULL;
    if (nt > 1)
        priv = (double*)calloc((size_t)nt * 7 * N, sizeof(double));
    double pe[OXG_N_PAIR_TERMS] = {0};
    int64_t pc[OXG_N_PAIR_TERMS] = {0};
    int terms[OXG_N_PAIR_TERMS];
    int n_terms = 0;
    for (int t = 0; t < OXG_N_PAIR_TERMS; ++t)
        if ((mask & (1u << t)) && term_present(m, t))
            terms[n_terms++] = t;

#ifdef _OPENMP
#pragma omp parallel num_threads(nt) if (nt > 1)
#endif
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* a = (nt > 1) ? priv + (size_t)tid * 7 * N : acc;
        double lpe[OXG_N_PAIR_TERMS] = {0};
        int64_t lpc[OXG_N_PAIR_TERMS] = {0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (int i = 0; i < N; ++i) {
            for (int q = h->start[i]; q < h->start[i + 1]; ++q) {
                int j = h->nbr[q];
                double dr[3];
                min_image(s->box, s->pos + 3 * i, s->pos + 3 * j, dr);
                for (int k = 0; k < n_terms; ++k) {
                    int t = terms[k];
                    double f[3], e, ti[3], tj[3];
                    if (!eval_term(m, s, t, i, j, dr, f, &e, ti, tj))
                        continue;
                    lpc[t]++;
                    lpe[t] += e;
                    a[7 * i + 0] += f[0];
                    a[7 * i + 1] += f[1];
                    a[7 * i + 2] += f[2];
                    a[7 * i + 3] += 0.5 * e;
                    a[7 * i + 4] += ti[0];
                    a[7 * i + 5] += ti[1];
                    a[7 * i + 6] += ti[2];
                    a[7 * j + 0] -= f[0];
                    a[7 * j + 1] -= f[1];
                    a[7 * j + 2] -= f[2];
                    a[7 * j + 3] += 0.5 * e;
                    a[7 * j + 4] += tj[0];
                    a[7 * j + 5] += tj[1];
                    a[7 * j + 6] += tj[2];
                }
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            for (int t = 0; t < OXG_N_PAIR_TERMS; ++t) {
                pe[t] += lpe[t];
                pc[t] += lpc[t];
            }
        }
    }
    if (nt > 1) {
        for (int t = 0; t < nt; ++t)
            for (size_t k = 0; k < (size_t)7 * N; ++k)
                acc[k] += priv[(size_t)t * 7 * N + k];
        free(priv);
    }
    if (pair_energy)
        for (int t = 0; t < OXG_N_PAIR_TERMS; ++t)
            pair_energy[t] += pe[t];
    if (pair_count)
        for (int t = 0; t < OXG_N_PAIR_TERMS; ++t)
            pair_count[t] += pc[t];

    if (bonded && m->bonded) {
        /* src/OxDNABondedForceCompute.cc:76-133 */
        for (int b = 0; b < s->n_bonds; ++b) {
            int A = s->bonds[3 * b], B = s->bonds[3 * b + 1], bt = s->bonds[3 * b + 2];
            double Rc[3], FB[3], tA[3], tB[3], e[3], vir[6];
            min_image(s->box, s->pos + 3 * B, s->pos + 3 * A, Rc);
            oxo_bonded(&m->bonded[bt], Rc, s->quat + 4 * (size_t)A, s->quat + 4 * (size_t)B,
                       s->type[A], s->type[B], FB, tA, tB, e, vir);
            double eh = 0.5 * (e[0] + e[1] + e[2]);
            acc[7 * A + 0] -= FB[0];
            acc[7 * A + 1] -= FB[1];
            acc[7 * A + 2] -= FB[2];
            acc[7 * A + 3] += eh;
            acc[7 * A + 4] += tA[0];
            acc[7 * A + 5] += tA[1];
            acc[7 * A + 6] += tA[2];
            acc[7 * B + 0] += FB[0];
            acc[7 * B + 1] += FB[1];
            acc[7 * B + 2] += FB[2];
            acc[7 * B + 3] += eh;
            acc[7 * B + 4] += tB[0];
            acc[7 * B + 5] += tB[1];
            acc[7 * B + 6] += tB[2];
            if (bonded_energy) {
                bonded_energy[0] += e[0];
                bonded_energy[1] += e[1];
                bonded_energy[2] += e[2];
            }
        }
    }
}

int oxo_forces(const oxo_model* m, const oxo_system* s, uint32_t term_mask, int bonded,
               int use_cells, double* force, double* torque, double* pair_energy,
               double* bonded_energy, int64_t* pair_count)
{
    int N = s->N;
    if (pair_energy)
        for (int t = 0; t < OXG_N_PAIR_TERMS; ++t)
            pair_energy[t] = 0.0;
    if (pair_count)
        for (int t = 0; t < OXG_N_PAIR_TERMS; ++t)
            pair_count[t] = 0;
    if (bonded_energy)
        bonded_energy[0] = bonded_energy[1] = bonded_energy[2] = 0.0;
    int* excl = (int*)malloc(sizeof(int) * OXO_MAX_EXCL * (N > 0 ? N : 1));
    if (build_exclusions(s, excl) != 0) {
        free(excl);
        return -1;
    }
    double rl = max_rcut(m, term_mask);
    halflist h = {0};
    double* acc = (double*)calloc((size_t)7 * (N > 0 ? N : 1), sizeof(double));
    if (rl > 0.0)
        build_halflist(s, s->pos, excl, rl * (1.0 + 1e-12), !use_cells, &h);
    else
        h.start = (int*)calloc(N + 1, sizeof(int));
    accumulate_forces(m, s, &h, term_mask, bonded, acc, pair_energy, bonded_energy, pair_count,
                      1);
    for (int i = 0; i < N; ++i) {
        if (force) {
            force[4 * i + 0] = acc[7 * i + 0];
            force[4 * i + 1] = acc[7 * i + 1];
            force[4 * i + 2] = acc[7 * i + 2];
            force[4 * i + 3] = acc[7 * i + 3];
        }
        if (torque) {
            torque[3 * i + 0] = acc[7 * i + 4];
            torque[3 * i + 1] = acc[7 * i + 5];
            torque[3 * i + 2] = acc[7 * i + 6];
        }
    }
    halflist_free(&h);
    free(acc);
    free(excl);
    return 0;
}

/* --------------------------------------------------------------- Langevin ---- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper. */
void oxo_philox4x32(uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static void rng4(uint64_t seed, uint64_t step, uint32_t tag, uint32_t stream, uint32_t out[4])
{
    uint32_t ctr[4] = {tag, (uint32_t)step, (uint32_t)(step >> 32), stream};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    oxo_philox4x32(ctr, key, out);
}

/* uniform in [-1, 1) from the top bits; normal via Box-Muller from two words */
static double u_sym(uint32_t u) { return (double)(int32_t)u * (1.0 / 2147483648.0); }
static void normal2(uint32_t a, uint32_t b, double* n0, double* n1)
{
    double u1 = ((double)a + 1.0) * (1.0 / 4294967296.0); /* (0, 1] */
    double u2 = (double)b * (1.0 / 4294967296.0);         /* [0, 1) */
    double r = sqrt(-2.0 * log(u1));
    *n0 = r * cos(2.0 * M_PI * u2);
    *n1 = r * sin(2.0 * M_PI * u2);
}

/* quaternion helpers on (s, x, y, z) arrays */
static void qmul_vec(const double q[4], const double t[3], double out[4])
{
    /* q * (0, t) */
    out[0] = -(q[1] * t[0] + q[2] * t[1] + q[3] * t[2]);
    out[1] = q[0] * t[0] + q[2] * t[2] - q[3] * t[1];
    out[2] = q[0] * t[1] + q[3] * t[0] - q[1] * t[2];
    out[3] = q[0] * t[2] + q[1] * t[1] - q[2] * t[0];
}
static void rot_conj(const double q[4], const double v[3], double out[3])
{
    qt c;
    c.s = q[0];
    c.v = V(-q[1], -q[2], -q[3]);
    vst(out, qrot(c, vld(v)));
}
static void rot_q(const double q[4], const double v[3], double out[3])
{
    vst(out, qrot(qld(q), vld(v)));
}
/* permutations P1, P2, P3 of Miller et al., J. Chem. Phys. 116, 8649 (2002) */
static void perm(int k, const double a[4], double o[4])
{
    if (k == 1) { o[0] = -a[1]; o[1] = a[0]; o[2] = a[3]; o[3] = -a[2]; }
    else if (k == 2) { o[0] = -a[2]; o[1] = -a[3]; o[2] = a[0]; o[3] = a[1]; }
    else { o[0] = -a[3]; o[1] = a[2]; o[2] = -a[1]; o[3] = a[0]; }
}
static void free_rotor(int k, double h, double I, double p[4], double q[4])
{
    double pp[4], pq[4];
    perm(k, q, pq);
    double phi = (p[0] * pq[0] + p[1] * pq[1] + p[2] * pq[2] + p[3] * pq[3]) / (4.0 * I);
    double c = cos(h * phi), s = sin(h * phi);
    perm(k, p, pp);
    for (int m = 0; m < 4; ++m) {
        p[m] = c * p[m] + s * pp[m];
        q[m] = c * q[m] + s * pq[m];
    }
}

long oxo_langevin_run(const oxo_model* m, oxo_system* s, double* pos, double* quat,
                      double* vel, double* angmom, uint32_t term_mask, int bonded,
                      double dt, double kT, double gamma, double gamma_r, uint64_t seed,
                      long step0, long nsteps, double buffer, int n_threads)
{
    int N = s->N;
    int* excl = (int*)malloc(sizeof(int) * OXO_MAX_EXCL * (N > 0 ? N : 1));
    if (build_exclusions(s, excl) != 0) {
        free(excl);
        return -1;
    }
    s->pos = pos;
    s->quat = quat;
    double rl = max_rcut(m, term_mask) + buffer;
    double* ref = (double*)malloc(sizeof(double) * 3 * N);
    double* acc = (double*)malloc(sizeof(double) * 7 * N);
    double* accel = (double*)malloc(sizeof(double) * 3 * N);
    double* tnet = (double*)malloc(sizeof(double) * 3 * N);
    halflist h = {0};
    long builds = 0;
    const double I = 1.0, mass = 1.0;

    /* wrap into the box and build */
    for (int i = 0; i < 3 * N; ++i)
        pos[i] = min_image1(pos[i], s->box[i % 3]);
    build_halflist(s, pos, excl, rl, 0, &h);
    memcpy(ref, pos, sizeof(double) * 3 * N);
    builds++;
    /* prepRun: forces at the start state, a = F/m, no bath forces */
    memset(acc, 0, sizeof(double) * 7 * N);
    accumulate_forces(m, s, &h, term_mask, bonded, acc, NULL, NULL, NULL, n_threads);
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            accel[3 * i + k] = acc[7 * i + k] / mass;
            tnet[3 * i + k] = acc[7 * i + 4 + k];
        }
    double half_buf2 = 0.25 * buffer * buffer;
    for (long st = step0; st < step0 + nsteps; ++st) {
        /* step one: v += dt/2 a, x += dt v, p kick + NO_SQUISH free rotor */
        int rebuild = 0;
        for (int i = 0; i < N; ++i) {
            for (int k = 0; k < 3; ++k) {
                vel[3 * i + k] += 0.5 * dt * accel[3 * i + k];
                pos[3 * i + k] += dt * vel[3 * i + k];
                pos[3 * i + k] = min_image1(pos[3 * i + k], s->box[k]);
            }
            double d[3];
            min_image(s->box, pos + 3 * i, ref + 3 * i, d);
            if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] > half_buf2)
                rebuild = 1;
            double* q = quat + 4 * (size_t)i;
            double* p = angmom + 4 * (size_t)i;
            double tb[3], dq[4];
            rot_conj(q, tnet + 3 * i, tb);
            qmul_vec(q, tb, dq);
            for (int c = 0; c < 4; ++c)
                p[c] += dt * dq[c];
            free_rotor(3, 0.5 * dt, I, p, q);
            free_rotor(2, 0.5 * dt, I, p, q);
            free_rotor(1, dt, I, p, q);
            free_rotor(2, 0.5 * dt, I, p, q);
            free_rotor(3, 0.5 * dt, I, p, q);
            double nq = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
            for (int c = 0; c < 4; ++c)
                q[c] *= nq;
        }
        if (rebuild) {
            build_halflist(s, pos, excl, rl, 0, &h);
            memcpy(ref, pos, sizeof(double) * 3 * N);
            builds++;
        }
        memset(acc, 0, sizeof(double) * 7 * N);
        accumulate_forces(m, s, &h, term_mask, bonded, acc, NULL, NULL, NULL, n_threads);
        /* step two: bath forces/torques (timestep index st + 1), then kick */
        uint64_t ts = (uint64_t)(st + 1);
        double ct = sqrt(6.0 * gamma * kT / dt);
        double cr = sqrt(2.0 * gamma_r * kT / dt);
        for (int i = 0; i < N; ++i) {
            uint32_t r0[4], r1[4];
            rng4(seed, ts, (uint32_t)i, 0u, r0);
            rng4(seed, ts, (uint32_t)i, 1u, r1);
            double* q = quat + 4 * (size_t)i;
            double* p = angmom + 4 * (size_t)i;
            for (int k = 0; k < 3; ++k) {
                double bd = u_sym(r0[k]) * ct - gamma * vel[3 * i + k];
                accel[3 * i + k] = (acc[7 * i + k] + bd) / mass;
            }
            /* s = (1/2 conj(q) p).v : body-frame angular momentum */
            double sv[3];
            sv[0] = 0.5 * (q[0] * p[1] - p[0] * q[1] - (q[2] * p[3] - q[3] * p[2]));
            sv[1] = 0.5 * (q[0] * p[2] - p[0] * q[2] - (q[3] * p[1] - q[1] * p[3]));
            sv[2] = 0.5 * (q[0] * p[3] - p[0] * q[3] - (q[1] * p[2] - q[2] * p[1]));
            double n[4];
            normal2(r1[0], r1[1], &n[0], &n[1]);
            normal2(r1[2], r1[3], &n[2], &n[3]);
            double bt[3], btl[3];
            for (int k = 0; k < 3; ++k)
                bt[k] = n[k] * cr - gamma_r * sv[k] / I;
            rot_q(q, bt, btl);
            for (int k = 0; k < 3; ++k) {
                tnet[3 * i + k] = acc[7 * i + 4 + k] + btl[k];
                vel[3 * i + k] += 0.5 * dt * accel[3 * i + k];
            }
            double tb[3], dq[4];
            rot_conj(q, tnet + 3 * i, tb);
            qmul_vec(q, tb, dq);
            for (int c = 0; c < 4; ++c)
                p[c] += dt * dq[c];
        }
    }
    halflist_free(&h);
    free(ref);
    free(acc);
    free(accel);
    free(tnet);
    free(excl);
    return builds;
}
