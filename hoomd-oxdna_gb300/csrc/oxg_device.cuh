// oxg_device.cuh - FP32 device physics of the oxDNA / oxRNA force hot path.
//
// Each function restates one reference routine (cited file:line, paths relative to
// the hoomd-oxDNA tree) in single precision. The arithmetic per non-zero term is the
// reference's; what differs is the order of work: every term first tests, on cheap
// quantities (site distances and angle cosines), whether any of its multiplicative
// factors is exactly zero, and skips the acos / sin / exp work when it is. Those
// pairs contribute exactly zero energy, force and torque in the reference too
// (src/OxDNABaseBase.h:159-160, src/EvaluatorPairOxDNACoaxStacking.h:222-225,
// src/OxDNABondedKernel.h:126-128), so the results are unchanged.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "oxg_params.h"

// Physics functions are host+device so that the exact FP32 arithmetic of the kernels
// can also be exercised by the host-side numerics tests (tests/native/).
#define OXG_HD __host__ __device__ __forceinline__
// Shared (out-of-line) device code for the long per-pair evaluations: one copy of the
// angle and BASE-BASE term code for every caller keeps the hot code small enough to
// stay in the instruction caches when few warps run it once per step.
#ifndef OXG_SHARED_ANGLES
#define OXG_SHARED_ANGLES 1
#endif
#ifndef OXG_SHARED_STACKING
#define OXG_SHARED_STACKING 0
#endif
#ifndef OXG_SHARED_TERMS
#define OXG_SHARED_TERMS 0
#endif
#if OXG_SHARED_ANGLES
#define OXG_HD_ANG static __host__ __device__ __noinline__
#else
#define OXG_HD_ANG OXG_HD
#endif
#if OXG_SHARED_STACKING
#define OXG_HD_STACK static __host__ __device__ __noinline__
#else
#define OXG_HD_STACK OXG_HD
#endif
#if OXG_SHARED_TERMS
#define OXG_HD_TERM static __host__ __device__ __noinline__
#else
#define OXG_HD_TERM OXG_HD
#endif

namespace oxg {

constexpr float kPi = 3.14159265358979323846f;

// ------------------------------------------------------------------ float3 algebra
OXG_HD float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
OXG_HD float3 operator+(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
OXG_HD float3 operator-(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
OXG_HD float3 operator-(float3 a) { return mk3(-a.x, -a.y, -a.z); }
OXG_HD float3 operator*(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
OXG_HD float3 operator*(float s, float3 a) { return mk3(a.x * s, a.y * s, a.z * s); }
OXG_HD void operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
OXG_HD void operator-=(float3& a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
OXG_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
OXG_HD float3 cross(float3 a, float3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Body frame of a quaternion q = (w, x, y, z) stored in (.x, .y, .z, .w): the columns
// of HOOMD's rotate(q, .) = (s^2 - u.u) v + 2 s (u x v) + 2 (u.v) u, written out as a
// matrix (exact for any |q|, like the reference's rotate).
struct Frame {
    float3 a1, a2, a3;
};
OXG_HD Frame quat_frame(float4 q)
{
    const float s = q.x, x = q.y, y = q.z, z = q.w;
    const float ss = s * s, xx = x * x, yy = y * y, zz = z * z;
    const float xy = x * y, xz = x * z, yz = y * z, sx = s * x, sy = s * y, sz = s * z;
    Frame f;
    f.a1 = mk3(ss + xx - yy - zz, 2.f * (xy + sz), 2.f * (xz - sy));
    f.a2 = mk3(2.f * (xy - sz), ss - xx + yy - zz, 2.f * (yz + sx));
    f.a3 = mk3(2.f * (xz + sy), 2.f * (yz - sx), ss - xx - yy + zz);
    return f;
}
OXG_HD float3 body_to_lab(const Frame& f, const float* s)
{
    return f.a1 * s[0] + f.a2 * s[1] + f.a3 * s[2];
}

// ---------------------------------------------------------------- numerics (L1)
// src/OxDNANumerics.h:194-198
OXG_HD float clamp_cos(float c) { return c > 1.f ? 1.f : (c < -1.f ? -1.f : c); }
// sin(acos(c)) = sqrt((1 - c)(1 + c)): 1 - c (or 1 + c) is exact in FP32 for |c| >= 1/2,
// so this is as accurate as sinf(acosf(c)) and does not wait for the acos.
OXG_HD float sin_of_acos(float c)
{
    const float cc = clamp_cos(c);
    return sqrtf(fmaxf(0.f, (1.f - cc) * (1.f + cc)));
}

// src/OxDNANumerics.h:201-215
OXG_HD float f4_angle(float t, const F4& p)
{
    // both non-zero branches computed and selected (no divergence; NaN d gives 0)
    const float d = fabsf(t - p.t0);
    const float e = p.tc - d;
    const float smooth = p.b * e * e, core = 1.f - p.a * d * d;
    return d < p.tc ? (d > p.ts ? smooth : core) : 0.f;
}
// (d f4 / d theta) / sin(theta); src/OxDNANumerics.h:218-244, with sin(theta) passed in.
// Callers compute sin(theta) once per angle and pass sin(pi - theta) = sin(theta) and
// sin(2 pi - theta) = -sin(theta) for the reflected branches: the same quantities as
// the reference, without the FP32 rounding of pi and 2 pi that otherwise dominates
// near theta = 0 or pi, where the two reflected 1/sin terms cancel.
OXG_HD float f4_dsin(float t, float st, const F4& p)
{
    float d = t - p.t0;
    float m = 1.f;
    if (d < 0.f) {
        d = -d;
        m = -1.f;
    }
    if (!(d < p.tc)) return 0.f;
    if (d > p.ts) return m * 2.f * p.b * (d - p.tc) / st;
    if (st * st > 1e-8f) return -m * 2.f * p.a * d / st;
    return -m * 2.f * p.a;
}
// The same with 1 / sin(theta) supplied (one reciprocal shared by an angle's branches).
OXG_HD float f4_dsin_inv(float t, float st, float inv_st, const F4& p)
{
    // branch-free form of f4_dsin (same selections, same guard)
    const float x = t - p.t0;
    const float m = x < 0.f ? -1.f : 1.f;
    const float d = fabsf(x);
    const float smooth = m * 2.f * p.b * (d - p.tc) * inv_st;
    const float core = st * st > 1e-8f ? -m * 2.f * p.a * d * inv_st : -m * 2.f * p.a;
    return d < p.tc ? (d > p.ts ? smooth : core) : 0.f;
}
// cos(theta) in the open support interval of f4 (or, symmetrised, of f4(pi - theta))
template <bool SYM>
OXG_HD bool f4_support(float c, const F4& p)
{
    bool in = (c > p.cmin) & (c < p.cmax);
    if (SYM) in |= (-c > p.cmin) & (-c < p.cmax);
    return in;
}
// src/OxDNANumerics.h:261-290 (f = (A, B, XC, XS))
OXG_HD float f5_val(float f, const float* p)
{
    if (!(f > p[2])) return 0.f;
    if (f < p[3]) return p[1] * (p[2] - f) * (p[2] - f);
    if (f < 0.f) return 1.f - p[0] * f * f;
    return 1.f;
}
OXG_HD float f5_deriv(float f, const float* p)
{
    if (!(f > p[2])) return 0.f;
    if (f < p[3]) return 2.f * p[1] * (f - p[2]);
    if (f < 0.f) return -2.f * p[0] * f;
    return 0.f;
}
// f1 Morse radial value and derivative, one exp (src/OxDNANumerics.h:114-155)
OXG_HD void f1_eval(float r, const float* f1, float eps, float shift,
                                        float& val, float& der)
{
    const float a = f1[0], r0 = f1[1], rlow = f1[2], rhigh = f1[3], rclow = f1[4],
                rchigh = f1[5], blow = f1[6], bhigh = f1[7];
    val = 0.f;
    der = 0.f;
    if (r < rchigh) {
        if (r > rhigh) {
            val = eps * bhigh * (r - rchigh) * (r - rchigh);
            der = eps * (2.f * bhigh * (r - rchigh));
        } else if (r > rlow) {
            const float t = expf(-(r - r0) * a);
            const float om = 1.f - t;
            val = eps * om * om - shift;
            der = eps * (2.f * om * t * a);
        } else if (r > rclow) {
            val = eps * blow * (r - rclow) * (r - rclow);
            der = eps * (2.f * blow * (r - rclow));
        }
    }
}
// f2 harmonic radial value and derivative (src/OxDNANumerics.h:158-192)
OXG_HD void f2_eval(float r, const float* f2, float& val, float& der)
{
    const float k = f2[0], r0 = f2[1], rc = f2[2], rlow = f2[3], rhigh = f2[4], rclow = f2[5],
                rchigh = f2[6], blow = f2[7], bhigh = f2[8];
    val = 0.f;
    der = 0.f;
    if (r < rchigh) {
        if (r > rhigh) {
            val = k * bhigh * (r - rchigh) * (r - rchigh);
            der = 2.f * k * bhigh * (r - rchigh);
        } else if (r > rlow) {
            val = (k / 2.f) * ((r - r0) * (r - r0) - (rc - r0) * (rc - r0));
            der = k * (r - r0);
        } else if (r > rclow) {
            val = k * blow * (r - rclow) * (r - rclow);
            der = 2.f * k * blow * (r - rclow);
        }
    }
}
// Smoothed LJ core; returns E and the force on the second site (r = site_q - site_p).
// src/OxDNANumerics.h:76-107 (sigma2 = sigma^2, rstar2 = r*^2, rc2 = rc^2).
OXG_HD float repulsive_lj(float3 r, float eps, float sigma2, float rstar2,
                                              float b, float rc, float rc2, float3& fq)
{
    const float rsq = dot(r, r);
    fq = mk3(0.f, 0.f, 0.f);
    if (!(rsq < rc2)) return 0.f;
    if (rsq > rstar2) {
        const float rmod = sqrtf(rsq);
        const float d = rmod - rc;
        fq = r * (-2.f * eps * b * d / rmod);
        return eps * b * d * d;
    }
    const float s2 = sigma2 / rsq;
    const float lj = s2 * s2 * s2;
    fq = r * (-24.f * eps * (lj - 2.f * lj * lj) / rsq);
    return 4.f * eps * (lj * lj - lj);
}

// ------------------------------------------------------- pair accumulator (L2)
struct PairAcc {
    float3 fi;  // force on i
    float3 ti;  // torque on i
    float3 tj;  // torque on j
};

// ------------------------------------------------------------- excluded volume
// src/EvaluatorPairOxDNAExcVol.h:107-149. rc = r_j - r_i (= -dr).
OXG_HD float excvol_term(const DExcVol& p, float3 rc, const Frame& fi,
                                             const Frame& fj, PairAcc& acc)
{
    const float3 back_i = body_to_lab(fi, p.back), base_i = body_to_lab(fi, p.base);
    const float3 back_j = body_to_lab(fj, p.back), base_j = body_to_lab(fj, p.base);
    float e = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float3 si = (k == 0 || k == 3) ? back_i : base_i;
        const float3 sj = (k == 0 || k == 2) ? back_j : base_j;
        const float3 r = rc + sj - si;
        if (!(dot(r, r) < p.rc2[k])) continue;
        float3 fq;
        e += repulsive_lj(r, p.eps, p.sigma2[k], p.rstar2[k], p.b[k], p.rc[k], p.rc2[k], fq);
        acc.fi -= fq;
        acc.ti += cross(si, -fq);
        acc.tj += cross(sj, fq);
    }
    return e;
}

// --------------------------------------------------------- BASE-BASE machinery
struct Ang {
    float val, dsin;
};
// one acos per angle; the reflected branch reuses pi - theta (src/OxDNABaseBase.h:52-67)
// theta and sin(theta) of the angle whose cosine is c = u . v (u, v unit vectors).
// acos(c) as in the reference; for parameter sets flagged `precise` and |c| > 0.9 the
// same angle from atan2(|u x v|, c), which keeps full FP32 accuracy near 0 and pi.
OXG_HD void angle_of(float c, float3 u, float3 v, const F4& t, float& th, float& st)
{
    if (t.precise != 0.f && fabsf(c) > 0.9f) {
        const float3 w = cross(u, v);
        st = sqrtf(dot(w, w));
        th = atan2f(st, c);
    } else {
        th = acosf(clamp_cos(c));
        st = sin_of_acos(c);
    }
}

// f4 value and torque coefficient of one angle; the reflected branch (SYM) reuses
// pi - theta and sin(pi - theta) = sin(theta) (src/OxDNABaseBase.h:52-67).
template <bool SYM>
OXG_HD_ANG Ang angular(float cost, float3 u, float3 v, const F4& t, float sign)
{
    float th, st;
    angle_of(cost, u, v, t, th, st);
    Ang a;
    a.val = f4_angle(th, t);
    const float inv_st = 1.f / st;
    float d = f4_dsin_inv(th, st, inv_st, t);
    if (SYM) {
        const float thn = kPi - th;
        a.val += f4_angle(thn, t);
        d -= f4_dsin_inv(thn, st, inv_st, t);
    }
    a.dsin = sign * d;
    return a;
}

// Shared six-angle BASE-BASE geometry (src/OxDNABaseBase.h:84-121).
struct BBGeom {
    float3 rdir, base_i, base_j;
    float rmod, c1, c2, c3, c4, c7, c8;
};
OXG_HD bool bb_geometry(float3 rc, const Frame& fi, const Frame& fj,
                                            const float* base, BBGeom& g)
{
    g.base_i = body_to_lab(fi, base);
    g.base_j = body_to_lab(fj, base);
    const float3 r = rc + g.base_j - g.base_i;
    g.rmod = sqrtf(dot(r, r));
    if (!(g.rmod > 0.f)) return false;
    const float inv = 1.f / g.rmod;
    g.rdir = r * inv;
    g.c1 = -dot(fi.a1, fj.a1);
    g.c2 = -dot(fj.a1, g.rdir);
    g.c3 = dot(fi.a1, g.rdir);
    g.c4 = dot(fi.a3, fj.a3);
    g.c7 = -dot(fj.a3, g.rdir);
    g.c8 = dot(fi.a3, g.rdir);
    return true;
}

// Radial factors of the two BASE-BASE terms.
struct RadialF1 {  // hydrogen bonding: Morse with per-pair eps
    const float* f1;
    float eps, shift;
    OXG_HD bool support(float r) const { return eps != 0.f && r > f1[4] && r < f1[5]; }
    OXG_HD void eval(float r, float& v, float& d) const { f1_eval(r, f1, eps, shift, v, d); }
};
struct RadialF2 {  // cross-stacking: harmonic
    const float* f2;
    OXG_HD bool support(float r) const { return f2[0] != 0.f && r > f2[5] && r < f2[6]; }
    OXG_HD void eval(float r, float& v, float& d) const { f2_eval(r, f2, v, d); }
};

// One BASE-BASE term; adds force on i and both torques. src/OxDNABaseBase.h:128-219.
// True when no factor of the BASE-BASE term is exactly zero: the tests bb_term starts
// with, used to decide which pairs go on to the full (acos-heavy) evaluation.
template <bool SYM, class Radial>
OXG_HD bool bb_support(const BBGeom& g, const F4& t1, const F4& t23, const F4& t4, const F4& t78,
                       bool inc_t4, const Radial& R)
{
    return R.support(g.rmod) && f4_support<false>(g.c1, t1) && f4_support<false>(g.c2, t23) &&
           f4_support<false>(g.c3, t23) && (!inc_t4 || f4_support<SYM>(g.c4, t4)) &&
           f4_support<SYM>(g.c7, t78) && f4_support<SYM>(g.c8, t78);
}

template <bool SYM, class Radial>
OXG_HD_TERM float bb_term(const BBGeom& g, const Frame& fi, const Frame& fj,
                                         const F4& t1, const F4& t23, const F4& t4,
                                         const F4& t78, bool inc_t4, const Radial& R,
                                         PairAcc& acc)
{
    if (!R.support(g.rmod)) return 0.f;
    if (!(f4_support<false>(g.c1, t1) && f4_support<false>(g.c2, t23) &&
          f4_support<false>(g.c3, t23) && (!inc_t4 || f4_support<SYM>(g.c4, t4)) &&
          f4_support<SYM>(g.c7, t78) && f4_support<SYM>(g.c8, t78)))
        return 0.f;
    // cosines with the vector pairs they are dot products of (src/OxDNABaseBase.h:113-118)
    const Ang A1 = angular<false>(g.c1, -fi.a1, fj.a1, t1, -1.f);
    const Ang A2 = angular<false>(g.c2, -fj.a1, g.rdir, t23, -1.f);
    const Ang A3 = angular<false>(g.c3, fi.a1, g.rdir, t23, 1.f);
    Ang A4;
    if (inc_t4) A4 = angular<SYM>(g.c4, fi.a3, fj.a3, t4, 1.f);
    else { A4.val = 1.f; A4.dsin = 0.f; }
    const Ang A7 = angular<SYM>(g.c7, -fj.a3, g.rdir, t78, -1.f);
    const Ang A8 = angular<SYM>(g.c8, fi.a3, g.rdir, t78, 1.f);
    float rv, rd;
    R.eval(g.rmod, rv, rd);
    const float prod = A1.val * A2.val * A3.val * A4.val * A7.val * A8.val;
    const float energy = rv * prod;
    if (energy == 0.f) return 0.f;

    const float3 a1 = fi.a1, a3 = fi.a3, b1 = fj.a1, b3 = fj.a3, rdir = g.rdir;
    const float rmod = g.rmod;
    float3 fq = rdir * (-(rd * prod));  // force on j
    float3 tp = mk3(0.f, 0.f, 0.f), tq = mk3(0.f, 0.f, 0.f);

    float3 dir = cross(a3, b3);  // theta4
    float tm = -rv * A1.val * A2.val * A3.val * A4.dsin * A7.val * A8.val;
    tp -= dir * tm;
    tq += dir * tm;
    dir = cross(a1, b1);  // theta1
    tm = -rv * A1.dsin * A2.val * A3.val * A4.val * A7.val * A8.val;
    tp -= dir * tm;
    tq += dir * tm;
    float fact = rv * A1.val * A2.dsin * A3.val * A4.val * A7.val * A8.val;  // theta2
    fq += (b1 + rdir * g.c2) * (fact / rmod);
    tq -= cross(rdir, b1) * fact;
    fact = rv * A1.val * A2.val * A3.dsin * A4.val * A7.val * A8.val;  // theta3
    fq += (a1 - rdir * g.c3) * (fact / rmod);
    tp -= cross(rdir, a1) * fact;
    fact = rv * A1.val * A2.val * A3.val * A4.val * A7.dsin * A8.val;  // theta7
    fq += (b3 + rdir * g.c7) * (fact / rmod);
    tq -= cross(rdir, b3) * fact;
    fact = rv * A1.val * A2.val * A3.val * A4.val * A7.val * A8.dsin;  // theta8
    fq += (a3 - rdir * g.c8) * (fact / rmod);
    tp -= cross(rdir, a3) * fact;
    tp -= cross(g.base_i, fq);  // site-offset torques
    tq += cross(g.base_j, fq);

    acc.fi -= fq;
    acc.ti += tp;
    acc.tj += tq;
    return energy;
}

// ------------------------------------------------------------ coaxial stacking
// src/EvaluatorPairOxDNACoaxStacking.h:134-372. rc = r_j - r_i.
// The zero-factor tests coax_term starts with (radial f2 and the theta4/5/6 supports).
OXG_HD bool coax_support(const DCoax& p, float3 rc, const Frame& fi, const Frame& fj)
{
    const float3 rstack = rc + body_to_lab(fj, p.stack) - body_to_lab(fi, p.stack);
    const float rsm = sqrtf(dot(rstack, rstack));
    if (!(rsm > 0.f && p.f2[0] != 0.f && rsm > p.f2[5] && rsm < p.f2[6])) return false;
    const float3 rsd = rstack * (1.f / rsm);
    return f4_support<false>(dot(fi.a3, fj.a3), p.t4) && f4_support<true>(dot(fi.a3, rsd), p.t56) &&
           f4_support<true>(-dot(fj.a3, rsd), p.t56);
}

OXG_HD_TERM float coax_term(const DCoax& p, float3 rc, const Frame& fi,
                                           const Frame& fj, PairAcc& acc)
{
    const float3 stack_i = body_to_lab(fi, p.stack), stack_j = body_to_lab(fj, p.stack);
    const float3 rstack = rc + stack_j - stack_i;
    const float rsm = sqrtf(dot(rstack, rstack));
    if (!(rsm > 0.f)) return 0.f;
    if (!(p.f2[0] != 0.f && rsm > p.f2[5] && rsm < p.f2[6])) return 0.f;  // f2 == 0
    const float3 a1 = fi.a1, a2 = fi.a2, a3 = fi.a3, b1 = fj.a1, b3 = fj.a3;
    const float3 rsd = rstack * (1.f / rsm);
    const float c4 = dot(a3, b3), c5 = dot(a3, rsd), c6 = -dot(b3, rsd);
    if (!(f4_support<false>(c4, p.t4) && f4_support<true>(c5, p.t56) &&
          f4_support<true>(c6, p.t56)))
        return 0.f;
    const float c1 = -dot(a1, b1);
    const float3 bref_i = body_to_lab(fi, p.bref), bref_j = body_to_lab(fj, p.bref);
    const float3 rbr = rc + bref_j - bref_i;
    const float rbm = sqrtf(dot(rbr, rbr));
    const float3 rbd = rbr * (1.f / rbm);
    const float cphi3 = dot(rsd, cross(rbd, a1));

    float f2v, f2D;
    f2_eval(rsm, p.f2, f2v, f2D);
    float th1, th4, th5, th6, s1, s4, s5, s6;
    angle_of(c1, -a1, b1, p.t1, th1, s1);
    angle_of(c4, a3, b3, p.t4, th4, s4);
    angle_of(c5, a3, rsd, p.t56, th5, s5);
    angle_of(c6, -b3, rsd, p.t56, th6, s6);
    const float th5n = kPi - th5, th6n = kPi - th6;
    float f4t1 = f4_angle(th1, p.t1);
    if (p.t1_mode == 0) f4t1 += f4_angle(2.f * kPi - th1, p.t1);
    else if (th1 > p.t1_sb) f4t1 += p.t1_sa * (th1 - p.t1_sb) * (th1 - p.t1_sb);
    const float f4t4 = f4_angle(th4, p.t4);
    const float f4t5 = f4_angle(th5, p.t56) + f4_angle(th5n, p.t56);
    const float f4t6 = f4_angle(th6, p.t56) + f4_angle(th6n, p.t56);
    float f5p3 = 0.f, f5p4 = 0.f, cphi4 = 0.f, phif = 1.f;
    if (p.rna_coax) {
        cphi4 = dot(rsd, cross(rbd, b1));
        f5p3 = f5_val(cphi3, p.phi3);
        f5p4 = f5_val(cphi4, p.phi4);
        phif = f5p3 * f5p4;
    } else if (p.phi3_enabled) {
        f5p3 = f5_val(cphi3, p.phi3);
        phif = f5p3 * f5p3;
    }
    const float energy = f2v * f4t1 * f4t4 * f4t5 * f4t6 * phif;
    if (energy == 0.f) return 0.f;

    float f4t1D = -f4_dsin(th1, s1, p.t1);
    if (p.t1_mode == 0) f4t1D += -f4_dsin(2.f * kPi - th1, -s1, p.t1);  // sin(2pi - t) = -sin t
    else if (th1 > p.t1_sb) {
        const float hd = (s1 * s1 > 1e-8f) ? 2.f * p.t1_sa * (th1 - p.t1_sb) / s1 : 2.f * p.t1_sa;
        f4t1D += -hd;
    }
    const float f4t4D = f4_dsin(th4, s4, p.t4);
    const float f4t5D = f4_dsin(th5, s5, p.t56) - f4_dsin(th5n, s5, p.t56);
    const float f4t6D = -f4_dsin(th6, s6, p.t56) + f4_dsin(th6n, s6, p.t56);

    float3 fq = rsd * (-(f2D * f4t1 * f4t4 * f4t5 * f4t6 * phif));
    float3 tp = mk3(0.f, 0.f, 0.f), tq = mk3(0.f, 0.f, 0.f);
    float3 dir = cross(a1, b1);  // theta1
    float tm = -f2v * f4t1D * f4t4 * f4t5 * f4t6 * phif;
    tp -= dir * tm;
    tq += dir * tm;
    dir = cross(a3, b3);  // theta4
    tm = -f2v * f4t1 * f4t4D * f4t5 * f4t6 * phif;
    tp -= dir * tm;
    tq += dir * tm;
    float fact = f2v * f4t1 * f4t4 * f4t5D * f4t6 * phif;  // theta5
    fq += (a3 - rsd * c5) * (fact / rsm);
    tp -= cross(rsd, a3) * fact;
    fact = f2v * f4t1 * f4t4 * f4t5 * f4t6D * phif;  // theta6
    fq += (b3 + rsd * c6) * (fact / rsm);
    tq -= cross(rsd, b3) * fact;

    if (p.rna_coax) {  // oxRNA: two dihedrals from the real BACK-BACK vector (:282-317)
        tp -= cross(stack_i, fq);
        tq += cross(stack_j, fq);
        const float base = f2v * f4t1 * f4t4 * f4t5 * f4t6;
        const float f5D3 = f5_deriv(cphi3, p.phi3), f5D4 = f5_deriv(cphi4, p.phi4);
#pragma unroll
        for (int w = 0; w < 2; ++w) {
            const float3 v = (w == 0) ? a1 : b1;
            const float fc = (w == 0) ? base * f5p4 * f5D3 : base * f5p3 * f5D4;
            const float3 rbv = cross(rbd, v);
            const float3 vrs = cross(v, rsd);
            const float3 fs = (rbv - rsd * dot(rsd, rbv)) * (-fc / rsm);
            const float3 fb = (vrs - rbd * dot(rbd, vrs)) * (-fc / rbm);
            fq += fs + fb;
            tp -= cross(stack_i, fs) + cross(bref_i, fb);
            tq += cross(stack_j, fs) + cross(bref_j, fb);
            const float3 pure = cross(v, cross(rsd, rbd)) * fc;
            if (w == 0) tp -= pure;
            else tq -= pure;
        }
        acc.fi -= fq;
        acc.ti += tp;
        acc.tj += tq;
        return energy;
    }
    if (p.phi3_enabled) {  // oxDNA1 phi3 dihedral (:320-361)
        const float f5D3 = f5_deriv(cphi3, p.phi3);
        const float gm = p.gamma, g3 = gm * gm * gm;
        const float rbm3 = rbm * rbm * rbm;
        const float a2b1 = dot(a2, b1), a3b1 = dot(a3, b1);
        const float ra1 = dot(rsd, a1), ra2 = dot(rsd, a2), ra3 = dot(rsd, a3), rb1 = dot(rsd, b1);
        const float par = ra3 * a2b1 - ra2 * a3b1;
        const float dcdr = -gm * par * (gm * (ra1 - rb1) + rsm) / rbm3;
        const float dcda1b1 = g3 * par / rbm3;
        const float dcda2b1 = gm * ra3 / rbm;
        const float dcda3b1 = -gm * ra2 / rbm;
        const float dcdra1 = -gm * gm * par * rsm / rbm3;
        const float dcdra2 = -gm * a3b1 / rbm;
        const float dcdra3 = gm * a2b1 / rbm;
        const float dcdrb1 = gm * gm * par * rsm / rbm3;
        const float fc = f2v * f4t1 * f4t4 * f4t5 * f4t6 * 2.f * f5p3 * f5D3;
        fq -= (rsd * dcdr + ((a1 - rsd * ra1) * dcdra1 + (a2 - rsd * ra2) * dcdra2 +
                             (a3 - rsd * ra3) * dcdra3 + (b1 - rsd * rb1) * dcdrb1) *
                                (1.f / rsm)) *
              fc;
        tp += (cross(rsd, a1) * dcdra1 + cross(rsd, a2) * dcdra2 + cross(rsd, a3) * dcdra3) * fc;
        tq += cross(rsd, b1) * (dcdrb1 * fc);
        const float3 pure =
            (cross(a1, b1) * dcda1b1 + cross(a2, b1) * dcda2b1 + cross(a3, b1) * dcda3b1) * fc;
        tp -= pure;
        tq += pure;
    }
    tp -= cross(stack_i, fq);
    tq += cross(stack_j, fq);
    acc.fi -= fq;
    acc.ti += tp;
    acc.tj += tq;
    return energy;
}

// ------------------------------------------------------------------ Debye-Hueckel
// src/EvaluatorPairOxDNADebye.h:244-303. rc = r_j - r_i.
OXG_HD float debye_term(const DDebye& p, float3 rc, const Frame& fi,
                                            const Frame& fj, float ci, float cj, PairAcc& acc)
{
    const float3 back_i = body_to_lab(fi, p.back), back_j = body_to_lab(fj, p.back);
    const float3 rb = rc + back_j - back_i;
    const float rbm = sqrtf(dot(rb, rb));
    if (!(rbm > 0.f) || !(rbm < p.rc)) return 0.f;
    const float cut = ci * cj;
    const float3 rbd = rb * (1.f / rbm);
    float energy;
    float3 fq;
    if (rbm < p.rhigh) {
        const float ex = expf(rbm * p.minus_kappa);
        energy = ex * (p.prefactor / rbm);
        fq = rbd * (-(p.prefactor * ex) * (p.minus_kappa / rbm - 1.f / (rbm * rbm)));
    } else {
        const float d = rbm - p.rc;
        energy = p.b_smooth * d * d;
        fq = rbd * (-(2.f * p.b_smooth * d));
    }
    energy *= cut;
    fq = fq * cut;
    acc.ti -= cross(back_i, fq);
    acc.tj += cross(back_j, fq);
    acc.fi -= fq;
    return energy;
}

// ------------------------------------------------------------------------ bonded
struct BondAcc {
    float3 fB;    // force on B (A receives -fB)
    float3 tA, tB;
    double e[3];  // fene, bexc, stack
    float vir[6];
};
OXG_HD void vir_acc(float* v, float3 r, float3 f)
{
    // src/OxDNABondedKernel.h:48-58
    v[0] += 0.5f * r.x * f.x;
    v[1] += 0.5f * r.x * f.y;
    v[2] += 0.5f * r.x * f.z;
    v[3] += 0.5f * r.y * f.y;
    v[4] += 0.5f * r.y * f.z;
    v[5] += 0.5f * r.z * f.z;
}

// DNA stacking, oxDNA p = B, q = A (src/OxDNABondedKernel.h:69-231). Rc = r_B - r_A.
OXG_HD_STACK float stacking_dna(const DBonded& p, float3 Rc, const Frame& fA,
                                              const Frame& fB, int tA, int tB, BondAcc& acc)
{
    const float3 a1 = fB.a1, a2 = fB.a2, a3 = fB.a3;
    const float3 b1 = fA.a1, b2 = fA.a2, b3 = fA.a3;
    const float3 stP = body_to_lab(fB, p.stack), stQ = body_to_lab(fA, p.stack);
    const float3 Rpq = -Rc;
    const float3 rs = Rpq + stQ - stP;
    const float rsm = sqrtf(dot(rs, rs));
    const float eps = p.st_eps[tA][tB];
    // f1 support (eps != 0, rclow < r < rchigh)
    if (!(eps != 0.f && rsm > p.f1[4] && rsm < p.f1[5])) return 0.f;
    const float3 rsd = rs * (1.f / rsm);
    const float c4 = dot(a3, b3), c5 = dot(a3, rsd), c6 = -dot(b3, rsd);
    if (!(f4_support<false>(c4, p.t4) && f4_support<false>(-c5, p.t5) &&
          f4_support<false>(c6, p.t5)))
        return 0.f;
    const float3 brP = body_to_lab(fB, p.bref), brQ = body_to_lab(fA, p.bref);
    const float3 rbr = Rpq + brQ - brP;
    const float rbm = sqrtf(dot(rbr, rbr));
    const float cp1 = dot(a2, rbr) / rbm, cp2 = dot(b2, rbr) / rbm;
    if (!(cp1 > p.p1[2] && cp2 > p.p1[2])) return 0.f;  // f5 == 0
    const float shift = eps * p.shift_factor;
    const float th4 = acosf(clamp_cos(c4)), th5 = acosf(clamp_cos(-c5)), th6 = acosf(clamp_cos(c6));
    float f1, f1D;
    f1_eval(rsm, p.f1, eps, shift, f1, f1D);
    const float f4t4 = f4_angle(th4, p.t4), f4t5 = f4_angle(th5, p.t5), f4t6 = f4_angle(th6, p.t5);
    const float f5p1 = f5_val(cp1, p.p1), f5p2 = f5_val(cp2, p.p1);
    const float es = f1 * f4t4 * f4t5 * f4t6 * f5p1 * f5p2;
    if (es == 0.f) return 0.f;
    const float f4t4D = f4_dsin(th4, sin_of_acos(c4), p.t4), f4t5D = f4_dsin(th5, sin_of_acos(-c5), p.t5),
                f4t6D = f4_dsin(th6, sin_of_acos(c6), p.t5);
    const float f5p1D = f5_deriv(cp1, p.p1), f5p2D = f5_deriv(cp2, p.p1);

    float3 force = rsd * (-(f1D * f4t4 * f4t5 * f4t6 * f5p1 * f5p2));
    force -= (a3 - rsd * c5) * (f1 * f4t4 * f4t5D * f4t6 * f5p1 * f5p2 / rsm);
    force -= (b3 + rsd * c6) * (f1 * f4t4 * f4t5 * f4t6D * f5p1 * f5p2 / rsm);

    const float g = p.gamma, rbm3 = rbm * rbm * rbm;
    float ra2 = dot(rsd, a2), ra1 = dot(rsd, a1), rb1 = dot(rsd, b1), a2b1 = dot(a2, b1);
    float par = rsm * ra2 - a2b1 * g;
    const float d1dr = (rsm * rsm * ra2 - ra2 * rbm * rbm - rsm * (a2b1 + ra2 * (-ra1 + rb1)) * g +
                        a2b1 * (-ra1 + rb1) * g * g) / rbm3;
    const float d1dra1 = rsm * g * par / rbm3;
    const float d1dra2 = -rsm / rbm;
    const float d1drb1 = -rsm * g * par / rbm3;
    const float d1da1b1 = -g * g * par / rbm3;
    const float d1da2b1 = g / rbm;
    const float fpp1 = -f1 * f4t4 * f4t5 * f4t6 * f5p1D * f5p2;
    force -= (rsd * d1dr + ((a2 - rsd * ra2) * d1dra2 + (a1 - rsd * ra1) * d1dra1 +
                            (b1 - rsd * rb1) * d1drb1) * (1.f / rsm)) * fpp1;

    ra2 = dot(rsd, b2);
    ra1 = dot(rsd, b1);
    rb1 = dot(rsd, a1);
    a2b1 = dot(b2, a1);
    par = rsm * ra2 + a2b1 * g;
    const float d2dr = (par * (rsm + (rb1 - ra1) * g) - ra2 * rbm * rbm) / rbm3;
    const float d2dra1 = -rsm * g * (rsm * ra2 + a2b1 * g) / rbm3;
    const float d2dra2 = -rsm / rbm;
    const float d2drb1 = rsm * g * par / rbm3;
    const float d2da1b1 = -g * g * par / rbm3;
    const float d2da2b1 = -g / rbm;
    const float fpp2 = -f1 * f4t4 * f4t5 * f4t6 * f5p1 * f5p2D;
    force -= (rsd * d2dr + ((b2 - rsd * ra2) * d2dra2 + (b1 - rsd * ra1) * d2dra1 +
                            (a1 - rsd * rb1) * d2drb1) * (1.f / rsm)) * fpp2;

    acc.fB -= force;  // force is on q = A
    vir_acc(acc.vir, rs, force);

    float3 tp = -cross(stP, force), tq = cross(stQ, force);
    const float3 t4d = cross(b3, a3);
    float tmod = f1 * f4t4D * f4t5 * f4t6 * f5p1 * f5p2;
    tp -= t4d * tmod;
    tq += t4d * tmod;
    tmod = -f1 * f4t4 * f4t5D * f4t6 * f5p1 * f5p2;
    tp -= cross(rsd, a3) * tmod;
    tmod = f1 * f4t4 * f4t5 * f4t6D * f5p1 * f5p2;
    tq += cross(rsd, b3) * tmod;
    tp += cross(rsd, a2) * (fpp1 * d1dra2) + cross(rsd, a1) * (fpp1 * d1dra1);
    tq += cross(rsd, b1) * (fpp1 * d1drb1);
    float3 pure = cross(a2, b1) * (fpp1 * d1da2b1) + cross(a1, b1) * (fpp1 * d1da1b1);
    tp -= pure;
    tq += pure;
    tp += cross(rsd, a1) * (fpp2 * d2drb1);
    tq += cross(rsd, b2) * (fpp2 * d2dra2) + cross(rsd, b1) * (fpp2 * d2dra1);
    pure = cross(a1, b2) * (fpp2 * d2da2b1) + cross(a1, b1) * (fpp2 * d2da1b1);
    tp -= pure;
    tq += pure;
    acc.tB += tp;
    acc.tA += tq;
    return es;
}

// RNA stacking, p = B, q = A (src/OxDNABondedKernel.h:238-353).
OXG_HD_STACK float stacking_rna(const DBonded& p, float3 Rc, const Frame& fA,
                                              const Frame& fB, int tA, int tB, BondAcc& acc)
{
    const float3 a2 = fB.a2, a3 = fB.a3, b2 = fA.a2, b3 = fA.a3;
    const float3 stP = body_to_lab(fB, p.stack3), stQ = body_to_lab(fA, p.stack5);
    const float3 Rpq = -Rc;
    const float3 rs = Rpq + stQ - stP;
    const float rsm = sqrtf(dot(rs, rs));
    const float eps = p.st_eps[tA][tB];
    if (!(eps != 0.f && rsm > p.f1[4] && rsm < p.f1[5])) return 0.f;
    const float3 rsd = rs * (1.f / rsm);
    const float c5 = dot(a3, rsd), c6 = -dot(b3, rsd);
    if (!(f4_support<false>(-c5, p.t5) && f4_support<false>(c6, p.t5))) return 0.f;
    const float3 bkP = body_to_lab(fB, p.back), bkQ = body_to_lab(fA, p.back);
    const float3 bvP = body_to_lab(fB, p.bbv3), bvQ = body_to_lab(fA, p.bbv5);
    const float3 rb = Rpq + bkQ - bkP;
    const float rbm = sqrtf(dot(rb, rb));
    const float3 rbd = rb * (1.f / rbm);
    const float cB1 = -dot(rbd, bvP), cB2 = -dot(rbd, bvQ);
    const float cp1 = dot(a2, rb) / rbm, cp2 = dot(b2, rb) / rbm;
    if (!(f4_support<false>(cB1, p.tB1) && f4_support<false>(cB2, p.tB2) && cp1 > p.p1[2] &&
          cp2 > p.p1[2]))
        return 0.f;
    const float shift = eps * p.shift_factor;
    const float th5 = acosf(clamp_cos(-c5)), th6 = acosf(clamp_cos(c6));
    const float thB1 = acosf(clamp_cos(cB1)), thB2 = acosf(clamp_cos(cB2));
    float f1, f1D;
    f1_eval(rsm, p.f1, eps, shift, f1, f1D);
    const float f4t5 = f4_angle(th5, p.t5), f4t6 = f4_angle(th6, p.t5);
    const float f4B1 = f4_angle(thB1, p.tB1), f4B2 = f4_angle(thB2, p.tB2);
    const float f5p1 = f5_val(cp1, p.p1), f5p2 = f5_val(cp2, p.p1);
    const float es = f1 * f4t5 * f4t6 * f4B1 * f4B2 * f5p1 * f5p2;
    if (es == 0.f) return 0.f;
    const float f4t5D = f4_dsin(th5, sin_of_acos(-c5), p.t5), f4t6D = f4_dsin(th6, sin_of_acos(c6), p.t5);
    const float f4B1D = f4_dsin(thB1, sin_of_acos(cB1), p.tB1), f4B2D = f4_dsin(thB2, sin_of_acos(cB2), p.tB2);
    const float f5p1D = f5_deriv(cp1, p.p1), f5p2D = f5_deriv(cp2, p.p1);

    float3 force = rsd * (-(f1D * f4t5 * f4t6 * f4B1 * f4B2 * f5p1 * f5p2));
    force -= (a3 - rsd * c5) * (f1 * f4t5D * f4t6 * f4B1 * f4B2 * f5p1 * f5p2 / rsm);
    force -= (b3 + rsd * c6) * (f1 * f4t5 * f4t6D * f4B1 * f4B2 * f5p1 * f5p2 / rsm);
    float3 pb = mk3(0.f, 0.f, 0.f);
    pb -= (bvP + rbd * cB1) * (f1 * f4t5 * f4t6 * f4B1D * f4B2 * f5p1 * f5p2 / rbm);
    pb -= (bvQ + rbd * cB2) * (f1 * f4t5 * f4t6 * f4B1 * f4B2D * f5p1 * f5p2 / rbm);
    const float fpp1 = -f1 * f4t5 * f4t6 * f4B1 * f4B2 * f5p1D * f5p2;
    pb += (a2 - rb * (cp1 / rbm)) * (fpp1 / rbm);
    const float fpp2 = -f1 * f4t5 * f4t6 * f4B1 * f4B2 * f5p1 * f5p2D;
    pb += (b2 - rb * (cp2 / rbm)) * (fpp2 / rbm);

    acc.fB -= force + pb;
    vir_acc(acc.vir, rs, force);
    vir_acc(acc.vir, rb, pb);

    float3 tp = -cross(stP, force) - cross(bkP, pb);
    float3 tq = cross(stQ, force) + cross(bkQ, pb);
    tp -= cross(rsd, a3) * (-f1 * f4t5D * f4t6 * f4B1 * f4B2 * f5p1 * f5p2);
    tq += cross(rsd, b3) * (f1 * f4t5 * f4t6D * f4B1 * f4B2 * f5p1 * f5p2);
    tp += cross(rbd, bvP) * (f1 * f4t5 * f4t6 * f4B1D * f4B2 * f5p1 * f5p2);
    tq += cross(rbd, bvQ) * (f1 * f4t5 * f4t6 * f4B1 * f4B2D * f5p1 * f5p2);
    tp += cross(a2, rbd) * fpp1;
    tq += cross(b2, rbd) * fpp2;
    acc.tB += tp;
    acc.tA += tq;
    return es;
}

// One bond (A, B = A's 5' neighbour): FENE in FP64, bonded excluded volume and
// stacking in FP32. src/OxDNABondedKernel.h:357-431. Rc = r_B - r_A in double;
// qA, qB the quaternions (promoted to double for FENE).
// FULL64: the BACK sites of FENE are rotated in FP64 too (the evaluator-level drop-in,
// whose Rc is exact in double). The engine's Rc comes from FP32 double-float position
// differences (~1e-7 absolute), which FP32 rotations of the BACK sites match, so there
// FULL64 = false rotates in FP32 and keeps FP64 for the FENE scalar arithmetic itself
// (|r|, r - r0, log(1 - dr^2 / delta^2), the restoring force): a third of the FP64 work.
// PART: 0 the whole bond; 1 FENE + bonded excluded volume; 2 stacking alone (two lanes
// evaluating parts 1 and 2 of a bond sum to part 0).
template <bool FULL64 = true, int PART = 0>
OXG_HD void bonded_pair(const DBonded& p, double3 Rc, double4_32a qA,
                                            double4_32a qB, int tA, int tB, BondAcc& acc)
{
    acc.fB = mk3(0.f, 0.f, 0.f);
    acc.tA = mk3(0.f, 0.f, 0.f);
    acc.tB = mk3(0.f, 0.f, 0.f);
    acc.e[0] = acc.e[1] = acc.e[2] = 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) acc.vir[k] = 0.f;

    // --- FENE between the BACK sites, FP64 (catastrophic cancellation in FP32) ---
    auto rot_d = [](double4_32a q, const double* v) {
        const double s = q.x, x = q.y, y = q.z, z = q.w;
        const double ss = s * s - (x * x + y * y + z * z);
        const double ud = x * v[0] + y * v[1] + z * v[2];
        double3 r;
        r.x = ss * v[0] + 2.0 * s * (y * v[2] - z * v[1]) + 2.0 * ud * x;
        r.y = ss * v[1] + 2.0 * s * (z * v[0] - x * v[2]) + 2.0 * ud * y;
        r.z = ss * v[2] + 2.0 * s * (x * v[1] - y * v[0]) + 2.0 * ud * z;
        return r;
    };
    const Frame fA = quat_frame(make_float4((float)qA.x, (float)qA.y, (float)qA.z, (float)qA.w));
    const Frame fB = quat_frame(make_float4((float)qB.x, (float)qB.y, (float)qB.z, (float)qB.w));
    const float3 Rcf = mk3((float)Rc.x, (float)Rc.y, (float)Rc.z);
    if (PART == 2) {
        if (p.stacking_enabled)
            acc.e[2] = p.rna_stacking ? stacking_rna(p, Rcf, fA, fB, tA, tB, acc)
                                      : stacking_dna(p, Rcf, fA, fB, tA, tB, acc);
        return;
    }
    const float3 backA = body_to_lab(fA, p.back), backB = body_to_lab(fB, p.back);
    double3 bA, bB;
    double rbx, rby, rbz;
    if (FULL64) {
        bA = rot_d(qA, p.back_site);
        bB = rot_d(qB, p.back_site);
        rbx = Rc.x + bB.x - bA.x;
        rby = Rc.y + bB.y - bA.y;
        rbz = Rc.z + bB.z - bA.z;
    } else {
        const float3 rb = Rcf + backB - backA;
        rbx = rb.x;
        rby = rb.y;
        rbz = rb.z;
    }
    const double rmod = sqrt(rbx * rbx + rby * rby + rbz * rbz);
    const double dr = rmod - p.r0_backbone;
    if (fabs(dr) >= p.delta_backbone) {
        acc.e[0] = 1.0e12;  // broken bond: energy clamp, no force
    } else {
        acc.e[0] = -0.5 * p.eps_backbone * log(1.0 - dr * dr / p.delta2);
        const double pref = -(p.eps_backbone * dr / (p.delta2 - dr * dr)) / rmod;
        const double fx = pref * rbx, fy = pref * rby, fz = pref * rbz;
        acc.fB = mk3((float)fx, (float)fy, (float)fz);
        if (FULL64) {
            // torques: backA x (-f), backB x f
            const double tAx = -(bA.y * fz - bA.z * fy), tAy = -(bA.z * fx - bA.x * fz),
                         tAz = -(bA.x * fy - bA.y * fx);
            const double tBx = bB.y * fz - bB.z * fy, tBy = bB.z * fx - bB.x * fz,
                         tBz = bB.x * fy - bB.y * fx;
            acc.tA = mk3((float)tAx, (float)tAy, (float)tAz);
            acc.tB = mk3((float)tBx, (float)tBy, (float)tBz);
        } else {
            acc.tA = cross(backA, -acc.fB);
            acc.tB = cross(backB, acc.fB);
        }
        vir_acc(acc.vir, mk3((float)rbx, (float)rby, (float)rbz), acc.fB);
    }

    // --- bonded excluded volume + stacking, FP32 ---
    const float3 baseA = body_to_lab(fA, p.base), baseB = body_to_lab(fB, p.base);
    float eb = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float3 si = (k == 2) ? backA : baseA;
        const float3 sj = (k == 1) ? backB : baseB;
        const float3 r = Rcf + sj - si;
        float3 f;
        eb += repulsive_lj(r, p.excl_eps, p.bx_sigma2[k], p.bx_rstar2[k], p.bx_b[k], p.bx_rc[k],
                           p.bx_rc[k] * p.bx_rc[k], f);
        acc.fB += f;
        acc.tA += cross(si, -f);
        acc.tB += cross(sj, f);
        vir_acc(acc.vir, r, f);
    }
    acc.e[1] = eb;
    if (PART == 0 && p.stacking_enabled) {
        acc.e[2] = p.rna_stacking ? stacking_rna(p, Rcf, fA, fB, tA, tB, acc)
                                  : stacking_dna(p, Rcf, fA, fB, tA, tB, acc);
    }
}

}  // namespace oxg
