// oxg_params.h - device-side (FP32) parameter layout of the oxDNA force engine.
//
// The host converts each term's double-precision POD (include/oxdna_gb300.h) into
// these FP32 structs once per upload and precomputes what the kernels need
// (squared cutoffs, shift = eps * shift_factor, the cosine interval on which each
// f4 factor is non-zero). A term whose parameters are identical for every type pair
// except its epsilon ("uniform") is stored once; otherwise one struct per ordered
// type pair is stored. Kernels copy the whole block into shared memory.
#pragma once
#include <stdint.h>

namespace oxg {

constexpr int kMaxTypes = 4;  // oxDNA/oxRNA use 4 base types (A, G, C, T/U)
constexpr int kMaxPairs = kMaxTypes * kMaxTypes;
constexpr int kMaxBondTypes = 4;

// f4 angular modulation (A, B, T0, TS, TC) plus the open interval (cmin, cmax) of
// cos(theta) on which f4(theta) != 0, i.e. |theta - T0| < TC
// (src/OxDNANumerics.h:201-215). Used to skip acos for pairs whose energy is 0.
// `precise` is 1 when the support reaches theta = 0 or pi while T0 is away from them:
// there f4 has a non-zero slope where acos of an FP32 cosine cannot resolve the angle,
// so the kernels take the angle from atan2(|u x v|, u . v) instead.
struct F4 {
    float a, b, t0, ts, tc, cmin, cmax, precise;
};

struct DExcVol {  // src/EvaluatorPairOxDNAExcVol.h:30-39
    float eps;
    float base[3], back[3];
    float sigma2[4], rstar2[4], b[4], rc[4], rc2[4];
    float rcutsq;
    float pad;
};

struct DHBond {  // src/EvaluatorPairOxDNAHBond.h:30-36 (eps comes from the eps table)
    float shift_factor;
    float base[3];
    float f1[8];  // a, r0, rlow, rhigh, rclow, rchigh, blow, bhigh
    F4 t1, t23, t4, t78;
    float rcutsq;
    float pad[3];
};

struct DCross {  // src/EvaluatorPairOxDNACrossStacking.h:30-37
    float base[3];
    float f2[9];  // k, r0, rc, rlow, rhigh, rclow, rchigh, blow, bhigh
    F4 t1, t23, t4, t78;
    float rcutsq;
    int t4_enabled;
    float pad[2];
};

struct DHBCross {  // src/EvaluatorPairOxDNAHBondCross.h:37-47
    float base[3];
    float shift_factor;
    float f1[8];
    F4 hb_t1, hb_t23, hb_t4, hb_t78;
    float f2[9];
    float rcutsq;
    float pad[2];
    F4 cs_t1, cs_t23, cs_t4, cs_t78;
};

struct DCoax {  // src/EvaluatorPairOxDNACoaxStacking.h:32-47
    float stack[3], bref[3];
    float gamma;
    float f2[9];
    F4 t1, t4, t56;
    float phi3[4], phi4[4];
    int t1_mode, phi3_enabled, rna_coax;
    float t1_sa, t1_sb;
    float rcutsq;
    float pad[2];
};

struct DDebye {  // src/EvaluatorPairOxDNADebye.h:28-31
    float back[3];
    float minus_kappa, prefactor, b_smooth, rc, rhigh;
    float rcutsq;
    float pad[3];
};

struct DBonded {  // src/OxDNABondedParams.h:35-73
    double eps_backbone, r0_backbone, delta_backbone, delta2;  // FENE stays FP64
    double back_site[3];
    float back[3], base[3];
    float excl_eps;
    float bx_sigma2[3], bx_rstar2[3], bx_b[3], bx_rc[3];
    int stacking_enabled, rna_stacking;
    float stack[3], bref[3];
    float gamma;
    float f1[8];
    float shift_factor;
    float st_eps[kMaxTypes][kMaxTypes];
    F4 t4, t5, tB1, tB2;
    float p1[4];
    float stack3[3], stack5[3], bbv3[3], bbv5[3];
    float pad;
};

// Term ids (match include/oxdna_gb300.h).
enum { kExcVol = 0, kHBond = 1, kCross = 2, kHBCross = 3, kCoax = 4, kDebye = 5, kNTerms = 6 };

// Header of the parameter block (16-byte aligned). Offsets are in bytes from the block
// start; stride[t] is 0 for a uniform term, else sizeof(struct) per ordered type pair.
struct ParamHeader {
    int n_types;
    uint32_t present;     // bit t set when term t has parameters
    int n_bond_types;
    int hb_cs_same_site;  // HB and cross-stacking share the BASE site (geometry reuse)
    int off[kNTerms];
    int stride[kNTerms];
    int off_bonded;
    int total_bytes;
    float hb_eps[kMaxPairs];    // HBond epsilon per ordered type pair
    float hb_shift[kMaxPairs];  // HBond f1 shift = eps * shift_factor (rounded once)
    float hbx_eps[kMaxPairs];   // HBondCross epsilon per ordered type pair
    float hbx_shift[kMaxPairs];
    float rcutsq_short;         // max squared COM cutoff over the short-range terms
    float rcutsq_max;           // max squared COM cutoff over all present terms
    float pad[2];
};

constexpr int kParamBlockMax = 16384 + 4096;

}  // namespace oxg
