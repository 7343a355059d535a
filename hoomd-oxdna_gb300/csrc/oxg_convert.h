// oxg_convert.h - host conversion of the C-ABI parameter PODs (double, the
// reference param_type fields) into the FP32 device structs of oxg_params.h.
#pragma once
#include <cmath>
#include <cstring>

#include "../../include/oxdna_gb300.h"
#include "oxg_params.h"

namespace oxg {

// f4 set (A, B, T0, TS, TC) -> device form with the cosine support interval, widened
// by 1e-5 so the zero-factor test stays conservative under FP32 rounding.
inline F4 mk_f4(const double* t)
{
    F4 f;
    f.a = (float)t[0];
    f.b = (float)t[1];
    f.t0 = (float)t[2];
    f.ts = (float)t[3];
    f.tc = (float)t[4];
    const double lo = t[2] - t[4], hi = t[2] + t[4];
    f.cmax = lo > 0.0 ? (float)(std::cos(lo) + 1e-5) : 2.f;
    f.cmin = hi < M_PI ? (float)(std::cos(hi) - 1e-5) : -2.f;
    const double near = 0.05;
    f.precise = ((lo < near && t[2] > 1e-6) || (hi > M_PI - near && t[2] < M_PI - 1e-6)) ? 1.f : 0.f;
    return f;
}
inline void cp3(float* d, const double* s) { d[0] = (float)s[0]; d[1] = (float)s[1]; d[2] = (float)s[2]; }
inline void cpn(float* d, const double* s, int n) { for (int k = 0; k < n; ++k) d[k] = (float)s[k]; }
inline float sq(double r) { return (float)(r * r); }

inline DExcVol to_dev(const oxg_excvol_params& s, double rcut)
{
    DExcVol d;
    std::memset(&d, 0, sizeof(d));
    d.eps = (float)s.eps;
    cp3(d.base, s.base_site);
    cp3(d.back, s.back_site);
    for (int k = 0; k < 4; ++k) {
        d.sigma2[k] = sq(s.sigma[k]);
        d.rstar2[k] = sq(s.rstar[k]);
        d.b[k] = (float)s.b[k];
        d.rc[k] = (float)s.rc[k];
        d.rc2[k] = sq(s.rc[k]);
    }
    d.rcutsq = sq(rcut);
    return d;
}
inline DHBond to_dev(const oxg_hbond_params& s, double rcut)
{
    DHBond d;
    std::memset(&d, 0, sizeof(d));
    d.shift_factor = (float)s.shift_factor;
    cp3(d.base, s.base_site);
    cpn(d.f1, s.f1, 8);
    d.t1 = mk_f4(s.t1);
    d.t23 = mk_f4(s.t23);
    d.t4 = mk_f4(s.t4);
    d.t78 = mk_f4(s.t78);
    d.rcutsq = sq(rcut);
    return d;
}
inline DCross to_dev(const oxg_cross_params& s, double rcut)
{
    DCross d;
    std::memset(&d, 0, sizeof(d));
    cp3(d.base, s.base_site);
    cpn(d.f2, s.f2, 9);
    d.t1 = mk_f4(s.t1);
    d.t23 = mk_f4(s.t23);
    d.t4 = mk_f4(s.t4);
    d.t78 = mk_f4(s.t78);
    d.rcutsq = sq(rcut);
    d.t4_enabled = s.t4_enabled;
    return d;
}
inline DHBCross to_dev(const oxg_hbondcross_params& s, double rcut)
{
    DHBCross d;
    std::memset(&d, 0, sizeof(d));
    cp3(d.base, s.base_site);
    d.shift_factor = (float)s.shift_factor;
    cpn(d.f1, s.f1, 8);
    d.hb_t1 = mk_f4(s.hb_t1);
    d.hb_t23 = mk_f4(s.hb_t23);
    d.hb_t4 = mk_f4(s.hb_t4);
    d.hb_t78 = mk_f4(s.hb_t78);
    cpn(d.f2, s.f2, 9);
    d.cs_t1 = mk_f4(s.cs_t1);
    d.cs_t23 = mk_f4(s.cs_t23);
    d.cs_t4 = mk_f4(s.cs_t4);
    d.cs_t78 = mk_f4(s.cs_t78);
    d.rcutsq = sq(rcut);
    return d;
}
inline DCoax to_dev(const oxg_coax_params& s, double rcut)
{
    DCoax d;
    std::memset(&d, 0, sizeof(d));
    cp3(d.stack, s.stack_site);
    cp3(d.bref, s.stack_back_ref);
    d.gamma = (float)s.gamma;
    cpn(d.f2, s.f2, 9);
    d.t1 = mk_f4(s.t1);
    d.t4 = mk_f4(s.t4);
    d.t56 = mk_f4(s.t56);
    cpn(d.phi3, s.phi3, 4);
    cpn(d.phi4, s.phi4, 4);
    d.t1_mode = s.t1_mode;
    d.phi3_enabled = s.phi3_enabled;
    d.rna_coax = s.rna_coax;
    d.t1_sa = (float)s.t1_sa;
    d.t1_sb = (float)s.t1_sb;
    d.rcutsq = sq(rcut);
    return d;
}
inline DDebye to_dev(const oxg_debye_params& s, double rcut)
{
    DDebye d;
    std::memset(&d, 0, sizeof(d));
    cp3(d.back, s.back_site);
    d.minus_kappa = (float)s.minus_kappa;
    d.prefactor = (float)s.prefactor;
    d.b_smooth = (float)s.b_smooth;
    d.rc = (float)s.rc;
    d.rhigh = (float)s.rhigh;
    d.rcutsq = sq(rcut);
    return d;
}
inline DBonded to_dev(const oxg_bonded_params& s)
{
    DBonded d;
    std::memset(&d, 0, sizeof(d));
    d.eps_backbone = s.eps_backbone;
    d.r0_backbone = s.r0_backbone;
    d.delta_backbone = s.delta_backbone;
    d.delta2 = s.delta2;
    for (int k = 0; k < 3; ++k) d.back_site[k] = s.back_site[k];
    cp3(d.back, s.back_site);
    cp3(d.base, s.base_site);
    d.excl_eps = (float)s.excl_eps;
    for (int k = 0; k < 3; ++k) {
        d.bx_sigma2[k] = sq(s.bx_sigma[k]);
        d.bx_rstar2[k] = sq(s.bx_rstar[k]);
        d.bx_b[k] = (float)s.bx_b[k];
        d.bx_rc[k] = (float)s.bx_rc[k];
    }
    d.stacking_enabled = s.stacking_enabled;
    d.rna_stacking = s.rna_stacking;
    cp3(d.stack, s.stack_site);
    cp3(d.bref, s.stack_back_ref);
    d.gamma = (float)s.st_gamma;
    cpn(d.f1, s.st_f1, 8);
    d.shift_factor = (float)s.st_f1[8];
    for (int i = 0; i < kMaxTypes; ++i)
        for (int j = 0; j < kMaxTypes; ++j) d.st_eps[i][j] = (float)s.st_eps[i][j];
    d.t4 = mk_f4(s.t4);
    d.t5 = mk_f4(s.t5);
    d.tB1 = mk_f4(s.tB1);
    d.tB2 = mk_f4(s.tB2);
    cpn(d.p1, s.p1, 4);
    cp3(d.stack3, s.stack_3_site);
    cp3(d.stack5, s.stack_5_site);
    cp3(d.bbv3, s.bbvector_3);
    cp3(d.bbv5, s.bbvector_5);
    return d;
}

}  // namespace oxg
