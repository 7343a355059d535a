// devmath.cu - test-only host harness: runs the engine's FP32 device physics
// (hoomd-oxdna_gb300/csrc/oxg_device.cuh, host+device functions) on the CPU so that
// the numerics tests can check the kernels' arithmetic against the golden fixtures
// without a GPU. Not part of the library; built by tests/test_fp32_math.py.
#include <cmath>

#include "../../hoomd-oxdna_gb300/csrc/oxg_convert.h"
#include "../../hoomd-oxdna_gb300/csrc/oxg_device.cuh"

using namespace oxg;

extern "C" int devmath_pair(int term, const void* pod, double rcut, const double* dr,
                            const double* qi, const double* qj, double ci, double cj,
                            double* f, double* e, double* ti, double* tj)
{
    const float3 d = make_float3((float)dr[0], (float)dr[1], (float)dr[2]);
    const float rsq = d.x * d.x + d.y * d.y + d.z * d.z;
    const Frame fi = quat_frame(make_float4((float)qi[0], (float)qi[1], (float)qi[2], (float)qi[3]));
    const Frame fj = quat_frame(make_float4((float)qj[0], (float)qj[1], (float)qj[2], (float)qj[3]));
    const float3 rc = make_float3(-d.x, -d.y, -d.z);
    PairAcc acc;
    acc.fi = acc.ti = acc.tj = make_float3(0.f, 0.f, 0.f);
    float E = 0.f;
    const float rcsq = sq(rcut);
    bool in = rsq < rcsq;
    if (in) {
        switch (term) {
        case kExcVol: E = excvol_term(to_dev(*(const oxg_excvol_params*)pod, rcut), rc, fi, fj, acc); break;
        case kHBond: {
            const oxg_hbond_params& p = *(const oxg_hbond_params*)pod;
            const DHBond D = to_dev(p, rcut);
            BBGeom g;
            if (bb_geometry(rc, fi, fj, D.base, g)) {
                RadialF1 R{D.f1, (float)p.eps, (float)(p.eps * p.shift_factor)};
                E = bb_term<false>(g, fi, fj, D.t1, D.t23, D.t4, D.t78, true, R, acc);
            }
            break;
        }
        case kCross: {
            const DCross D = to_dev(*(const oxg_cross_params*)pod, rcut);
            BBGeom g;
            if (bb_geometry(rc, fi, fj, D.base, g)) {
                RadialF2 R{D.f2};
                E = bb_term<true>(g, fi, fj, D.t1, D.t23, D.t4, D.t78, D.t4_enabled != 0, R, acc);
            }
            break;
        }
        case kHBCross: {
            const oxg_hbondcross_params& p = *(const oxg_hbondcross_params*)pod;
            const DHBCross D = to_dev(p, rcut);
            BBGeom g;
            if (bb_geometry(rc, fi, fj, D.base, g)) {
                RadialF1 R1{D.f1, (float)p.eps, (float)(p.eps * p.shift_factor)};
                E = bb_term<false>(g, fi, fj, D.hb_t1, D.hb_t23, D.hb_t4, D.hb_t78, true, R1, acc);
                RadialF2 R2{D.f2};
                E += bb_term<true>(g, fi, fj, D.cs_t1, D.cs_t23, D.cs_t4, D.cs_t78, true, R2, acc);
            }
            break;
        }
        case kCoax: E = coax_term(to_dev(*(const oxg_coax_params*)pod, rcut), rc, fi, fj, acc); break;
        case kDebye:
            E = debye_term(to_dev(*(const oxg_debye_params*)pod, rcut), rc, fi, fj, (float)ci, (float)cj, acc);
            break;
        }
    }
    f[0] = acc.fi.x; f[1] = acc.fi.y; f[2] = acc.fi.z;
    ti[0] = acc.ti.x; ti[1] = acc.ti.y; ti[2] = acc.ti.z;
    tj[0] = acc.tj.x; tj[1] = acc.tj.y; tj[2] = acc.tj.z;
    *e = E;
    return in ? 1 : 0;
}

// full64 = 1: the drop-in's all-FP64 FENE; 0: the engine's (FP32 BACK-site rotations).
extern "C" void devmath_bonded(const oxg_bonded_params* p, const double* Rc, const double* qA,
                               const double* qB, int tA, int tB, double* FB, double* tauA,
                               double* tauB, double* e, double* vir, int full64)
{
    const DBonded D = to_dev(*p);
    BondAcc acc;
    const double3 R = make_double3(Rc[0], Rc[1], Rc[2]);
    const double4_32a a4 = make_double4_32a(qA[0], qA[1], qA[2], qA[3]);
    const double4_32a b4 = make_double4_32a(qB[0], qB[1], qB[2], qB[3]);
    // full64: bit 0 the FP64 BACK-site rotations; bits 1-2 the part (0 whole bond,
    // 1 FENE + bonded excluded volume, 2 stacking)
    const int part = full64 >> 1;
    if (part == 1) bonded_pair<false, 1>(D, R, a4, b4, tA, tB, acc);
    else if (part == 2) bonded_pair<false, 2>(D, R, a4, b4, tA, tB, acc);
    else if (full64 & 1) bonded_pair<true>(D, R, a4, b4, tA, tB, acc);
    else bonded_pair<false>(D, R, a4, b4, tA, tB, acc);
    FB[0] = acc.fB.x; FB[1] = acc.fB.y; FB[2] = acc.fB.z;
    tauA[0] = acc.tA.x; tauA[1] = acc.tA.y; tauA[2] = acc.tA.z;
    tauB[0] = acc.tB.x; tauB[1] = acc.tB.y; tauB[2] = acc.tB.z;
    for (int k = 0; k < 3; ++k) e[k] = acc.e[k];
    for (int k = 0; k < 6; ++k) vir[k] = acc.vir[k];
}

// The surrogate's map from an energy's feature gradient to forces and torques
// (mlp_grad_to_forces), on a smooth test energy of the base-base features,
// E = sum_k a_k x_k + b_k x_k^2 with x = (r, c1, c2, c3, c4, c7, c8); the caller checks
// it against finite differences of E over positions and rotations.
#include "../../hoomd-oxdna_gb300/csrc/oxg_mlp.cuh"

extern "C" int devmath_mlp_map(const double* base_site, const double* dr, const double* qi,
                               const double* qj, const double* coef, double* e, double* f,
                               double* ti, double* tj)
{
    const float base[3] = {(float)base_site[0], (float)base_site[1], (float)base_site[2]};
    const Frame fi = quat_frame(make_float4((float)qi[0], (float)qi[1], (float)qi[2], (float)qi[3]));
    const Frame fj = quat_frame(make_float4((float)qj[0], (float)qj[1], (float)qj[2], (float)qj[3]));
    const float3 rc = make_float3((float)-dr[0], (float)-dr[1], (float)-dr[2]);
    BBGeom g;
    if (!bb_geometry(rc, fi, fj, base, g)) return 0;
    float x[kMlpIn], dE[kMlpIn];
    mlp_features(g, x);
    double E = 0.0;
    for (int k = 0; k < kMlpIn; ++k) {
        E += coef[k] * x[k] + coef[kMlpIn + k] * x[k] * x[k];
        dE[k] = (float)(coef[k] + 2.0 * coef[kMlpIn + k] * x[k]);
    }
    PairAcc acc;
    acc.fi = acc.ti = acc.tj = make_float3(0.f, 0.f, 0.f);
    mlp_grad_to_forces(g, fi, fj, dE, acc);
    *e = E;
    f[0] = acc.fi.x; f[1] = acc.fi.y; f[2] = acc.fi.z;
    ti[0] = acc.ti.x; ti[1] = acc.ti.y; ti[2] = acc.ti.z;
    tj[0] = acc.tj.x; tj[1] = acc.tj.y; tj[2] = acc.tj.z;
    return 1;
}
