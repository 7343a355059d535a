/*
 * ref_wrap.cpp - C wrapper around the reference plugin's OWN evaluator and bonded
 * headers, compiled unchanged from the reference tree by oracle/build_ref.sh into
 * oracle/_ref/ (never committed). TEST INFRASTRUCTURE ONLY: it pins the C oracle
 * (oracle/oxdna_oracle.c) and generates the golden fixtures in tests/golden/.
 *
 * Built three times: FP64 (HOOMD_HAS_FORCEREAL undefined, ForceReal == Scalar == double:
 * the reference's upstream-HOOMD arithmetic), FP32 (HOOMD_HAS_FORCEREAL defined,
 * ForceReal == float: the reference's mixed-precision GPU arithmetic emulated on the
 * host, src/MixedPrecisionCompat.h:20-35) and the flop census (OXREF_COUNTING:
 * ForceReal counts its operations, ref_shim/oxref_count.h).
 *
 * Each ref_* function converts this project's POD parameter structs into the
 * reference param_type (same fields) and calls evaluate() / oxdna_bonded_pair().
 */
#include <pybind11/pybind11.h>

#include "EvaluatorPairOxDNACoaxStacking.h"
#include "EvaluatorPairOxDNACrossStacking.h"
#include "EvaluatorPairOxDNADebye.h"
#include "EvaluatorPairOxDNAExcVol.h"
#include "EvaluatorPairOxDNAHBond.h"
#include "EvaluatorPairOxDNAHBondCross.h"
#include "OxDNABondedKernel.h"

#include "../include/oxdna_gb300.h"
#include "oxdna_oracle.h"

#include <cmath>
#include <vector>

using namespace hoomd;
using namespace hoomd::md;

namespace
{
vec3<Scalar> v3(const double* a) { return vec3<Scalar>(a[0], a[1], a[2]); }
void cp(Scalar* dst, const double* src, int n)
{
    for (int k = 0; k < n; ++k)
        dst[k] = src[k];
}

OxDNAExcVolParams cvt(const oxg_excvol_params* s)
{
    OxDNAExcVolParams p;
    p.eps = s->eps;
    p.base_site = v3(s->base_site);
    p.back_site = v3(s->back_site);
    cp(p.sigma, s->sigma, 4);
    cp(p.rstar, s->rstar, 4);
    cp(p.b, s->b, 4);
    cp(p.rc, s->rc, 4);
    return p;
}
OxDNAHBondParams cvt(const oxg_hbond_params* s)
{
    OxDNAHBondParams p;
    p.eps = s->eps;
    p.shift_factor = s->shift_factor;
    p.base_site = v3(s->base_site);
    p.f1_a = s->f1[0];
    p.f1_r0 = s->f1[1];
    p.f1_rlow = s->f1[2];
    p.f1_rhigh = s->f1[3];
    p.f1_rclow = s->f1[4];
    p.f1_rchigh = s->f1[5];
    p.f1_blow = s->f1[6];
    p.f1_bhigh = s->f1[7];
    cp(p.t1, s->t1, 5);
    cp(p.t23, s->t23, 5);
    cp(p.t4, s->t4, 5);
    cp(p.t78, s->t78, 5);
    return p;
}
OxDNACrossStackingParams cvt(const oxg_cross_params* s)
{
    OxDNACrossStackingParams p;
    p.base_site = v3(s->base_site);
    p.f2_k = s->f2[0];
    p.f2_r0 = s->f2[1];
    p.f2_rc = s->f2[2];
    p.f2_rlow = s->f2[3];
    p.f2_rhigh = s->f2[4];
    p.f2_rclow = s->f2[5];
    p.f2_rchigh = s->f2[6];
    p.f2_blow = s->f2[7];
    p.f2_bhigh = s->f2[8];
    cp(p.t1, s->t1, 5);
    cp(p.t23, s->t23, 5);
    cp(p.t4, s->t4, 5);
    cp(p.t78, s->t78, 5);
    p.t4_enabled = s->t4_enabled != 0;
    return p;
}
OxDNAHBondCrossParams cvt(const oxg_hbondcross_params* s)
{
    OxDNAHBondCrossParams p;
    p.base_site = v3(s->base_site);
    p.eps = s->eps;
    p.shift_factor = s->shift_factor;
    p.f1_a = s->f1[0];
    p.f1_r0 = s->f1[1];
    p.f1_rlow = s->f1[2];
    p.f1_rhigh = s->f1[3];
    p.f1_rclow = s->f1[4];
    p.f1_rchigh = s->f1[5];
    p.f1_blow = s->f1[6];
    p.f1_bhigh = s->f1[7];
    cp(p.hb_t1, s->hb_t1, 5);
    cp(p.hb_t23, s->hb_t23, 5);
    cp(p.hb_t4, s->hb_t4, 5);
    cp(p.hb_t78, s->hb_t78, 5);
    p.f2_k = s->f2[0];
    p.f2_r0 = s->f2[1];
    p.f2_rc = s->f2[2];
    p.f2_rlow = s->f2[3];
    p.f2_rhigh = s->f2[4];
    p.f2_rclow = s->f2[5];
    p.f2_rchigh = s->f2[6];
    p.f2_blow = s->f2[7];
    p.f2_bhigh = s->f2[8];
    cp(p.cs_t1, s->cs_t1, 5);
    cp(p.cs_t23, s->cs_t23, 5);
    cp(p.cs_t4, s->cs_t4, 5);
    cp(p.cs_t78, s->cs_t78, 5);
    return p;
}
OxDNACoaxStackingParams cvt(const oxg_coax_params* s)
{
    OxDNACoaxStackingParams p;
    p.stack_site = v3(s->stack_site);
    p.stack_back_ref = v3(s->stack_back_ref);
    p.gamma = s->gamma;
    p.f2_k = s->f2[0];
    p.f2_r0 = s->f2[1];
    p.f2_rc = s->f2[2];
    p.f2_rlow = s->f2[3];
    p.f2_rhigh = s->f2[4];
    p.f2_rclow = s->f2[5];
    p.f2_rchigh = s->f2[6];
    p.f2_blow = s->f2[7];
    p.f2_bhigh = s->f2[8];
    cp(p.t1, s->t1, 5);
    cp(p.t4, s->t4, 5);
    cp(p.t56, s->t56, 5);
    cp(p.phi3, s->phi3, 4);
    cp(p.phi4, s->phi4, 4);
    p.t1_mode = s->t1_mode;
    p.t1_sa = s->t1_sa;
    p.t1_sb = s->t1_sb;
    p.phi3_enabled = s->phi3_enabled != 0;
    p.rna_coax = s->rna_coax != 0;
    return p;
}
OxDNADebyeParams cvt(const oxg_debye_params* s)
{
    OxDNADebyeParams p;
    p.back_site = v3(s->back_site);
    p.minus_kappa = s->minus_kappa;
    p.prefactor = s->prefactor;
    p.b_smooth = s->b_smooth;
    p.rc = s->rc;
    p.rhigh = s->rhigh;
    return p;
}
oxdna_bonded_params cvt(const oxg_bonded_params* s)
{
    oxdna_bonded_params p;
    p.eps_backbone = s->eps_backbone;
    p.r0_backbone = s->r0_backbone;
    p.delta_backbone = s->delta_backbone;
    p.delta2 = s->delta2;
    p.back_site = v3(s->back_site);
    p.base_site = v3(s->base_site);
    p.excl_eps = s->excl_eps;
    cp(p.bx_sigma, s->bx_sigma, 3);
    cp(p.bx_rstar, s->bx_rstar, 3);
    cp(p.bx_b, s->bx_b, 3);
    cp(p.bx_rc, s->bx_rc, 3);
    p.stacking_enabled = s->stacking_enabled != 0;
    p.stack_site = v3(s->stack_site);
    p.stack_back_ref = v3(s->stack_back_ref);
    p.st_gamma = s->st_gamma;
    p.st_a = s->st_f1[0];
    p.st_r0 = s->st_f1[1];
    p.st_rlow = s->st_f1[2];
    p.st_rhigh = s->st_f1[3];
    p.st_rclow = s->st_f1[4];
    p.st_rchigh = s->st_f1[5];
    p.st_blow = s->st_f1[6];
    p.st_bhigh = s->st_f1[7];
    p.st_shift_factor = s->st_f1[8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            p.st_eps[i][j] = s->st_eps[i][j];
    p.t4_a = s->t4[0];
    p.t4_b = s->t4[1];
    p.t4_t0 = s->t4[2];
    p.t4_ts = s->t4[3];
    p.t4_tc = s->t4[4];
    p.t5_a = s->t5[0];
    p.t5_b = s->t5[1];
    p.t5_t0 = s->t5[2];
    p.t5_ts = s->t5[3];
    p.t5_tc = s->t5[4];
    p.p1_a = s->p1[0];
    p.p1_b = s->p1[1];
    p.p1_xc = s->p1[2];
    p.p1_xs = s->p1[3];
    p.rna_stacking = s->rna_stacking != 0;
    p.stack_3_site = v3(s->stack_3_site);
    p.stack_5_site = v3(s->stack_5_site);
    p.bbvector_3 = v3(s->bbvector_3);
    p.bbvector_5 = v3(s->bbvector_5);
    p.tB1_a = s->tB1[0];
    p.tB1_b = s->tB1[1];
    p.tB1_t0 = s->tB1[2];
    p.tB1_ts = s->tB1[3];
    p.tB1_tc = s->tB1[4];
    p.tB2_a = s->tB2[0];
    p.tB2_b = s->tB2[1];
    p.tB2_t0 = s->tB2[2];
    p.tB2_ts = s->tB2[3];
    p.tB2_tc = s->tB2[4];
    return p;
}

template<class Eval, class P>
int run_eval(const P& p, const double dr[3], const double qi[4], const double qj[4],
             double rcutsq, double ci, double cj, double f[3], double* e, double ti[3],
             double tj[3])
{
    ForceReal3 d;
    d.x = ForceReal(dr[0]);
    d.y = ForceReal(dr[1]);
    d.z = ForceReal(dr[2]);
    Scalar4 a = make_scalar4(qi[0], qi[1], qi[2], qi[3]);
    Scalar4 b = make_scalar4(qj[0], qj[1], qj[2], qj[3]);
    Eval ev(d, a, b, ForceReal(rcutsq), p);
    ev.setCharge(ci, cj);
    ForceReal3 F, Ti, Tj;
    ForceReal E = 0;
    bool r = ev.evaluate(F, E, false, Ti, Tj);
    if (!r) {
        f[0] = f[1] = f[2] = ti[0] = ti[1] = ti[2] = tj[0] = tj[1] = tj[2] = 0.0;
        *e = 0.0;
        return 0;
    }
    f[0] = F.x;
    f[1] = F.y;
    f[2] = F.z;
    ti[0] = Ti.x;
    ti[1] = Ti.y;
    ti[2] = Ti.z;
    tj[0] = Tj.x;
    tj[1] = Tj.y;
    tj[2] = Tj.z;
    *e = E;
    return 1;
}
// The reference's own dict -> param_type constructor beside this project's route
// (dict -> POD struct -> cvt), both serialised by the reference's own toPython() /
// asDict(): the caller compares the two dicts. Called through ctypes.PyDLL (GIL held).
template <class T, class POD> PyObject* pair_dicts(PyObject* d, const void* pod)
{
    pybind11::dict v = pybind11::reinterpret_borrow<pybind11::dict>(pybind11::handle(d));
    T a(v, false);
    T b = cvt(static_cast<const POD*>(pod));
    return pybind11::make_tuple(a.toPython(), b.toPython()).release().ptr();
}
} // namespace

extern "C" PyObject* ref_param_dicts(int term, PyObject* d, const void* pod)
{
    try
        {
        switch (term)
            {
        case 0: return pair_dicts<OxDNAExcVolParams, oxg_excvol_params>(d, pod);
        case 1: return pair_dicts<OxDNAHBondParams, oxg_hbond_params>(d, pod);
        case 2: return pair_dicts<OxDNACrossStackingParams, oxg_cross_params>(d, pod);
        case 3: return pair_dicts<OxDNAHBondCrossParams, oxg_hbondcross_params>(d, pod);
        case 4: return pair_dicts<OxDNACoaxStackingParams, oxg_coax_params>(d, pod);
        case 5: return pair_dicts<OxDNADebyeParams, oxg_debye_params>(d, pod);
        case 6:
            {
            pybind11::dict v = pybind11::reinterpret_borrow<pybind11::dict>(pybind11::handle(d));
            oxdna_bonded_params a(v);
            oxdna_bonded_params b = cvt(static_cast<const oxg_bonded_params*>(pod));
            return pybind11::make_tuple(a.asDict(), b.asDict()).release().ptr();
            }
            }
        PyErr_SetString(PyExc_ValueError, "term must be 0..6");
        }
    catch (pybind11::error_already_set& e)
        {
        e.restore();
        }
    catch (const std::exception& e)
        {
        PyErr_SetString(PyExc_RuntimeError, e.what());
        }
    return nullptr;
}

extern "C" {

int ref_is_fp32(void) { return sizeof(ForceReal) == 4; }

#ifdef OXREF_COUNTING
// flop census: the operation tallies since the last reset, in the order of oxref_count.h
// (add, mul, div, sqrt, exp, log, acos, sin, cos)
int ref_count_n(void) { return oxref::kNCount; }
void ref_count_get(unsigned long long* out)
{
    for (int k = 0; k < oxref::kNCount; ++k)
        out[k] = oxref::op_counts()[k];
}
void ref_count_reset(void)
{
    for (int k = 0; k < oxref::kNCount; ++k)
        oxref::op_counts()[k] = 0;
}
#endif

int ref_excvol(const oxg_excvol_params* p, const double dr[3], const double qi[4],
               const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
               double tj[3])
{
    return run_eval<EvaluatorPairOxDNAExcVol>(cvt(p), dr, qi, qj, rcutsq, 1, 1, f, e, ti, tj);
}
int ref_hbond(const oxg_hbond_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
              double tj[3])
{
    return run_eval<EvaluatorPairOxDNAHBond>(cvt(p), dr, qi, qj, rcutsq, 1, 1, f, e, ti, tj);
}
int ref_cross(const oxg_cross_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
              double tj[3])
{
    return run_eval<EvaluatorPairOxDNACrossStacking>(cvt(p), dr, qi, qj, rcutsq, 1, 1, f, e,
                                                     ti, tj);
}
int ref_hbondcross(const oxg_hbondcross_params* p, const double dr[3], const double qi[4],
                   const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
                   double tj[3])
{
    return run_eval<EvaluatorPairOxDNAHBondCross>(cvt(p), dr, qi, qj, rcutsq, 1, 1, f, e, ti,
                                                  tj);
}
int ref_coax(const oxg_coax_params* p, const double dr[3], const double qi[4],
             const double qj[4], double rcutsq, double f[3], double* e, double ti[3],
             double tj[3])
{
    return run_eval<EvaluatorPairOxDNACoaxStacking>(cvt(p), dr, qi, qj, rcutsq, 1, 1, f, e,
                                                    ti, tj);
}
int ref_debye(const oxg_debye_params* p, const double dr[3], const double qi[4],
              const double qj[4], double rcutsq, double ci, double cj, double f[3],
              double* e, double ti[3], double tj[3])
{
    return run_eval<EvaluatorPairOxDNADebye>(cvt(p), dr, qi, qj, rcutsq, ci, cj, f, e, ti, tj);
}
void ref_bonded(const oxg_bonded_params* pp, const double Rc[3], const double qA[4],
                const double qB[4], int typeA, int typeB, double FB[3], double tauA[3],
                double tauB[3], double e[3], double vir[6])
{
    oxdna_bonded_params p = cvt(pp);
    quat<Scalar> a(make_scalar4(qA[0], qA[1], qA[2], qA[3]));
    quat<Scalar> b(make_scalar4(qB[0], qB[1], qB[2], qB[3]));
    oxdna::BondedResult r;
    oxdna::oxdna_bonded_pair(p, vec3<Scalar>(Rc[0], Rc[1], Rc[2]), a, b, (unsigned)typeA,
                             (unsigned)typeB, r);
    FB[0] = r.FB.x;
    FB[1] = r.FB.y;
    FB[2] = r.FB.z;
    tauA[0] = r.tauA.x;
    tauA[1] = r.tauA.y;
    tauA[2] = r.tauA.z;
    tauB[0] = r.tauB.x;
    tauB[1] = r.tauB.y;
    tauB[2] = r.tauB.z;
    e[0] = r.e_fene;
    e[1] = r.e_bexc;
    e[2] = r.e_stack;
    for (int k = 0; k < 6; ++k)
        vir[k] = r.vir[k];
}

// A whole system's forces through the reference's own evaluators, with HOOMD's CPU
// driver semantics (hoomd/md/AnisoPotentialPair.h: half neighbour list and the third
// law; src/OxDNABondedForceCompute.cc:55-134 for the bonds): for each listed pair (i, j)
// dr = r_i - r_j (minimum image), every selected term within its cutoff adds F to i and
// -F to j, its torques to each end and half its energy to each; each bond (A, B) takes
// Rc = r_B - r_A. Parameters are converted to the reference param_type once per call.
// It times the reference's arithmetic on the host beside the C restatement.
// pairs: 2 * n_pairs particle indices (the caller's half list); outputs as oxo_forces
// (force[4N] with the per-particle energy, torque[3N], pair_energy[6], bonded_energy[3]).
int ref_system_forces(const oxo_model* m, const oxo_system* s, uint32_t mask, int bonded,
                      int n_pairs, const int32_t* pairs, double* force, double* torque,
                      double* pair_energy, double* bonded_energy)
{
    const int nt = m->n_types, np = nt * nt, N = s->N;
    std::vector<OxDNAExcVolParams> pe(np);
    std::vector<OxDNAHBondParams> ph(np);
    std::vector<OxDNACrossStackingParams> pc(np);
    std::vector<OxDNAHBondCrossParams> px(np);
    std::vector<OxDNACoaxStackingParams> pk(np);
    std::vector<OxDNADebyeParams> pd(np);
    std::vector<double> rc2(6 * np, -1.0);
    for (int k = 0; k < np; ++k) {
        if (m->excvol) pe[k] = cvt(&m->excvol[k]);
        if (m->hbond) ph[k] = cvt(&m->hbond[k]);
        if (m->cross) pc[k] = cvt(&m->cross[k]);
        if (m->hbondcross) px[k] = cvt(&m->hbondcross[k]);
        if (m->coax) pk[k] = cvt(&m->coax[k]);
        if (m->debye) pd[k] = cvt(&m->debye[k]);
        for (int t = 0; t < 6; ++t)
            if (((mask >> t) & 1u) && m->r_cut[t]) rc2[t * np + k] = m->r_cut[t][k] * m->r_cut[t][k];
    }
    for (int k = 0; k < 4 * N; ++k) force[k] = 0.0;
    for (int k = 0; k < 3 * N; ++k) torque[k] = 0.0;
    for (int t = 0; t < 6; ++t) pair_energy[t] = 0.0;
    for (int t = 0; t < 3; ++t) bonded_energy[t] = 0.0;
    auto wrap = [&](double d, int k) { return d - s->box[k] * std::rint(d / s->box[k]); };
    for (int n = 0; n < n_pairs; ++n) {
        const int i = pairs[2 * n], j = pairs[2 * n + 1];
        ForceReal3 d;
        d.x = ForceReal(wrap(s->pos[3 * i] - s->pos[3 * j], 0));
        d.y = ForceReal(wrap(s->pos[3 * i + 1] - s->pos[3 * j + 1], 1));
        d.z = ForceReal(wrap(s->pos[3 * i + 2] - s->pos[3 * j + 2], 2));
        const double rsq = double(d.x) * d.x + double(d.y) * d.y + double(d.z) * d.z;
        const int k = s->type[i] * nt + s->type[j];
        const double* qa = s->quat + 4 * i;
        const double* qb = s->quat + 4 * j;
        const Scalar4 a = make_scalar4(qa[0], qa[1], qa[2], qa[3]);
        const Scalar4 b = make_scalar4(qb[0], qb[1], qb[2], qb[3]);
        const double ci = s->charge ? s->charge[i] : 1.0, cj = s->charge ? s->charge[j] : 1.0;
        for (int t = 0; t < 6; ++t) {
            const double r2 = rc2[t * np + k];
            if (!(rsq < r2)) continue;
            ForceReal3 F, Ti, Tj;
            ForceReal E = 0;
            bool ok = false;
            switch (t) {
            case OXG_EXCVOL: {
                EvaluatorPairOxDNAExcVol ev(d, a, b, ForceReal(r2), pe[k]);
                ok = ev.evaluate(F, E, false, Ti, Tj);
                break;
            }
            case OXG_HBOND: {
                EvaluatorPairOxDNAHBond ev(d, a, b, ForceReal(r2), ph[k]);
                ok = ev.evaluate(F, E, false, Ti, Tj);
                break;
            }
            case OXG_CROSS: {
                EvaluatorPairOxDNACrossStacking ev(d, a, b, ForceReal(r2), pc[k]);
                ok = ev.evaluate(F, E, false, Ti, Tj);
                break;
            }
            case OXG_HBONDCROSS: {
                EvaluatorPairOxDNAHBondCross ev(d, a, b, ForceReal(r2), px[k]);
                ok = ev.evaluate(F, E, false, Ti, Tj);
                break;
            }
            case OXG_COAX: {
                EvaluatorPairOxDNACoaxStacking ev(d, a, b, ForceReal(r2), pk[k]);
                ok = ev.evaluate(F, E, false, Ti, Tj);
                break;
            }
            default: {
                EvaluatorPairOxDNADebye ev(d, a, b, ForceReal(r2), pd[k]);
                ev.setCharge(ci, cj);
                ok = ev.evaluate(F, E, false, Ti, Tj);
                break;
            }
            }
            if (!ok) continue;
            const double f[3] = {double(F.x), double(F.y), double(F.z)};
            for (int c = 0; c < 3; ++c) {
                force[4 * i + c] += f[c];
                force[4 * j + c] -= f[c];
            }
            force[4 * i + 3] += 0.5 * double(E);
            force[4 * j + 3] += 0.5 * double(E);
            torque[3 * i] += Ti.x;
            torque[3 * i + 1] += Ti.y;
            torque[3 * i + 2] += Ti.z;
            torque[3 * j] += Tj.x;
            torque[3 * j + 1] += Tj.y;
            torque[3 * j + 2] += Tj.z;
            pair_energy[t] += E;
        }
    }
    if (bonded && m->bonded) {
        std::vector<oxdna_bonded_params> pb(m->n_bond_types);
        for (int k = 0; k < m->n_bond_types; ++k) pb[k] = cvt(&m->bonded[k]);
        for (int n = 0; n < s->n_bonds; ++n) {
            const int A = s->bonds[3 * n], B = s->bonds[3 * n + 1], bt = s->bonds[3 * n + 2];
            const vec3<Scalar> Rc(wrap(s->pos[3 * B] - s->pos[3 * A], 0),
                                  wrap(s->pos[3 * B + 1] - s->pos[3 * A + 1], 1),
                                  wrap(s->pos[3 * B + 2] - s->pos[3 * A + 2], 2));
            const double* qa = s->quat + 4 * A;
            const double* qb = s->quat + 4 * B;
            quat<Scalar> a(make_scalar4(qa[0], qa[1], qa[2], qa[3]));
            quat<Scalar> b(make_scalar4(qb[0], qb[1], qb[2], qb[3]));
            oxdna::BondedResult r;
            oxdna::oxdna_bonded_pair(pb[bt], Rc, a, b, (unsigned)s->type[A], (unsigned)s->type[B], r);
            const double e = r.e_fene + r.e_bexc + r.e_stack;
            force[4 * B] += r.FB.x;
            force[4 * B + 1] += r.FB.y;
            force[4 * B + 2] += r.FB.z;
            force[4 * A] -= r.FB.x;
            force[4 * A + 1] -= r.FB.y;
            force[4 * A + 2] -= r.FB.z;
            force[4 * A + 3] += 0.5 * e;
            force[4 * B + 3] += 0.5 * e;
            torque[3 * A] += r.tauA.x;
            torque[3 * A + 1] += r.tauA.y;
            torque[3 * A + 2] += r.tauA.z;
            torque[3 * B] += r.tauB.x;
            torque[3 * B + 1] += r.tauB.y;
            torque[3 * B + 2] += r.tauB.z;
            bonded_energy[0] += r.e_fene;
            bonded_energy[1] += r.e_bexc;
            bonded_energy[2] += r.e_stack;
        }
    }
    return 0;
}
} // extern "C"
