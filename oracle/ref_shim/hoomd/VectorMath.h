/*
 * Minimal stand-in for HOOMD-blue's hoomd/VectorMath.h (vec3, quat, rotate), written
 * for this project so the reference plugin's headers compile unchanged for the oracle
 * pin. The quaternion convention is HOOMD's: quat(Scalar4 a) has s = a.x and
 * v = (a.y, a.z, a.w); rotate(q, v) = (s^2 - u.u) v + 2 s (u x v) + 2 (u.v) u, which
 * the reference pins with rotate(q, e_x) == a1 (oxdna/io.py:127-150).
 */
#ifndef OXREF_SHIM_VECTORMATH_H
#define OXREF_SHIM_VECTORMATH_H
#include "HOOMDMath.h"

namespace hoomd
{
template<class Real> struct vec3
{
    Real x, y, z;
    vec3() : x(0), y(0), z(0) { }
    vec3(Real a, Real b, Real c) : x(a), y(b), z(c) { }
    template<class U> explicit vec3(const vec3<U>& o) : x(Real(o.x)), y(Real(o.y)), z(Real(o.z)) { }
    explicit vec3(const Scalar3& o) : x(Real(o.x)), y(Real(o.y)), z(Real(o.z)) { }
#ifdef HOOMD_HAS_FORCEREAL
    explicit vec3(const ForceReal3& o) : x(Real(o.x)), y(Real(o.y)), z(Real(o.z)) { }
#endif
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(Real s) { x *= s; y *= s; z *= s; return *this; }
};
template<class Real> inline vec3<Real> operator+(const vec3<Real>& a, const vec3<Real>& b)
{ return vec3<Real>(a.x + b.x, a.y + b.y, a.z + b.z); }
template<class Real> inline vec3<Real> operator-(const vec3<Real>& a, const vec3<Real>& b)
{ return vec3<Real>(a.x - b.x, a.y - b.y, a.z - b.z); }
template<class Real> inline vec3<Real> operator-(const vec3<Real>& a)
{ return vec3<Real>(-a.x, -a.y, -a.z); }
template<class Real> inline vec3<Real> operator*(const vec3<Real>& a, Real s)
{ return vec3<Real>(a.x * s, a.y * s, a.z * s); }
template<class Real> inline vec3<Real> operator*(Real s, const vec3<Real>& a)
{ return vec3<Real>(a.x * s, a.y * s, a.z * s); }
template<class Real> inline vec3<Real> operator/(const vec3<Real>& a, Real s)
{ return vec3<Real>(a.x / s, a.y / s, a.z / s); }
template<class Real> inline Real dot(const vec3<Real>& a, const vec3<Real>& b)
{ return a.x * b.x + a.y * b.y + a.z * b.z; }
template<class Real> inline vec3<Real> cross(const vec3<Real>& a, const vec3<Real>& b)
{ return vec3<Real>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
template<class Real> inline Scalar3 vec_to_scalar3(const vec3<Real>& a)
{ return make_scalar3(Scalar(a.x), Scalar(a.y), Scalar(a.z)); }

template<class Real> struct quat
{
    Real s;
    vec3<Real> v;
    quat() : s(1), v(0, 0, 0) { }
    quat(Real a, const vec3<Real>& b) : s(a), v(b) { }
    explicit quat(const Scalar4& a) : s(Real(a.x)), v(Real(a.y), Real(a.z), Real(a.w)) { }
    template<class U> explicit quat(const quat<U>& o) : s(Real(o.s)), v(vec3<Real>(o.v)) { }
};
template<class Real> inline vec3<Real> rotate(const quat<Real>& q, const vec3<Real>& a)
{
    return (q.s * q.s - dot(q.v, q.v)) * a + Real(2) * q.s * cross(q.v, a)
           + Real(2) * dot(q.v, a) * q.v;
}
} // namespace hoomd
#endif
