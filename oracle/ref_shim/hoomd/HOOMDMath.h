/*
 * Minimal stand-in for HOOMD-blue's hoomd/HOOMDMath.h, written for this project so
 * the reference plugin's evaluator headers compile unchanged on the host for the
 * oracle pin (HOOMD-blue itself is not available). Only what those headers use:
 * Scalar (double), Scalar2/3/4, make_scalar3/4, __scalar_as_int / __int_as_scalar.
 * With HOOMD_HAS_FORCEREAL defined, ForceReal is float (the mixed-precision build
 * the reference ships its GPU numbers with), or with OXREF_COUNTING also defined the
 * operation-counting real of oxref_count.h; otherwise MixedPrecisionCompat.h aliases
 * ForceReal to Scalar.
 */
#ifndef OXREF_SHIM_HOOMDMATH_H
#define OXREF_SHIM_HOOMDMATH_H
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef OXREF_COUNTING
#include "../oxref_count.h"
#endif

namespace hoomd
{
typedef double Scalar;
struct Scalar2 { Scalar x, y; };
struct Scalar3 { Scalar x, y, z; };
struct Scalar4 { Scalar x, y, z, w; };
inline Scalar3 make_scalar3(Scalar x, Scalar y, Scalar z)
{
    Scalar3 r;
    r.x = x; r.y = y; r.z = z;
    return r;
}
inline Scalar4 make_scalar4(Scalar x, Scalar y, Scalar z, Scalar w)
{
    Scalar4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}
/* type id stored in the low 32 bits of a double's bit pattern */
inline int __scalar_as_int(Scalar a)
{
    int64_t b;
    memcpy(&b, &a, sizeof(b));
    return (int)(b & 0xffffffff);
}
inline Scalar __int_as_scalar(int a)
{
    int64_t b = (int64_t)(uint32_t)a;
    Scalar r;
    memcpy(&r, &b, sizeof(r));
    return r;
}
#ifdef HOOMD_HAS_FORCEREAL
#ifdef OXREF_COUNTING
typedef oxref::Counted ForceReal;  /* the flop census: every ForceReal operation counted */
#else
typedef float ForceReal;
#endif
struct ForceReal2 { ForceReal x, y; };
struct ForceReal3 { ForceReal x, y, z; };
struct ForceReal4 { ForceReal x, y, z, w; };
inline ForceReal3 make_forcereal3(ForceReal x, ForceReal y, ForceReal z)
{
    ForceReal3 r;
    r.x = x; r.y = y; r.z = z;
    return r;
}
inline ForceReal4 make_forcereal4(ForceReal x, ForceReal y, ForceReal z, ForceReal w)
{
    ForceReal4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}
#endif
} // namespace hoomd
#endif
