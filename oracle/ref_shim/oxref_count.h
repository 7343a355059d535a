/*
 * Operation-counting real number for the flop census of the reference evaluators
 * (test and measurement infrastructure only; never part of the product).
 *
 * With OXREF_COUNTING defined, the HOOMDMath.h stand-in makes ForceReal this type, so
 * the reference's own evaluator and bonded headers compile unchanged and every
 * arithmetic operation they perform in ForceReal is tallied: additions and
 * subtractions, multiplications (an FMA is one of each, i.e. two flops), divisions,
 * and the calls sqrt, exp, log, acos, sin, cos. The value is carried in double, so
 * branch decisions follow the FP64 reference. Sign flips, comparisons, fabs and
 * conversions are free. Scalar (double) arithmetic, the FP64 FENE bond, is not counted.
 */
#ifndef OXREF_COUNT_H
#define OXREF_COUNT_H
#include <math.h>
#include <type_traits>

namespace oxref
{
enum
{
    kAdd,
    kMul,
    kDiv,
    kSqrt,
    kExp,
    kLog,
    kAcos,
    kSin,
    kCos,
    kNCount
};

inline unsigned long long* op_counts()
{
    static unsigned long long c[kNCount];
    return c;
}

struct Counted
{
    double v;
    Counted() : v(0.0) { }
    template<class T, class = typename std::enable_if<std::is_arithmetic<T>::value>::type>
    Counted(T x) : v((double)x)
    {
    }
    operator double() const { return v; }
    Counted operator-() const { return Counted(-v); }
    Counted operator+() const { return *this; }
    Counted& operator+=(const Counted& o)
    {
        ++op_counts()[kAdd];
        v += o.v;
        return *this;
    }
    Counted& operator-=(const Counted& o)
    {
        ++op_counts()[kAdd];
        v -= o.v;
        return *this;
    }
    Counted& operator*=(const Counted& o)
    {
        ++op_counts()[kMul];
        v *= o.v;
        return *this;
    }
    Counted& operator/=(const Counted& o)
    {
        ++op_counts()[kDiv];
        v /= o.v;
        return *this;
    }
};

template<class T>
using if_arith = typename std::enable_if<std::is_arithmetic<T>::value, int>::type;

#define OXREF_BINOP(OP, KIND)                                                                 \
    inline Counted operator OP(const Counted& a, const Counted& b)                            \
    {                                                                                         \
        ++op_counts()[KIND];                                                                  \
        return Counted(a.v OP b.v);                                                           \
    }                                                                                         \
    template<class T, if_arith<T> = 0> inline Counted operator OP(const Counted& a, T b)     \
    {                                                                                         \
        ++op_counts()[KIND];                                                                  \
        return Counted(a.v OP(double) b);                                                     \
    }                                                                                         \
    template<class T, if_arith<T> = 0> inline Counted operator OP(T a, const Counted& b)     \
    {                                                                                         \
        ++op_counts()[KIND];                                                                  \
        return Counted((double)a OP b.v);                                                     \
    }
OXREF_BINOP(+, kAdd)
OXREF_BINOP(-, kAdd)
OXREF_BINOP(*, kMul)
OXREF_BINOP(/, kDiv)
#undef OXREF_BINOP

#define OXREF_CMP(OP)                                                                         \
    inline bool operator OP(const Counted& a, const Counted& b) { return a.v OP b.v; }        \
    template<class T, if_arith<T> = 0> inline bool operator OP(const Counted& a, T b)        \
    {                                                                                         \
        return a.v OP(double) b;                                                              \
    }                                                                                         \
    template<class T, if_arith<T> = 0> inline bool operator OP(T a, const Counted& b)        \
    {                                                                                         \
        return (double)a OP b.v;                                                              \
    }
OXREF_CMP(<)
OXREF_CMP(>)
OXREF_CMP(<=)
OXREF_CMP(>=)
OXREF_CMP(==)
OXREF_CMP(!=)
#undef OXREF_CMP

#define OXREF_FN(NAME, KIND)                                                                  \
    inline Counted NAME(const Counted& a)                                                     \
    {                                                                                         \
        ++op_counts()[KIND];                                                                  \
        return Counted(::NAME(a.v));                                                          \
    }
OXREF_FN(sqrt, kSqrt)
OXREF_FN(exp, kExp)
OXREF_FN(log, kLog)
OXREF_FN(acos, kAcos)
OXREF_FN(sin, kSin)
OXREF_FN(cos, kCos)
#undef OXREF_FN
inline Counted fabs(const Counted& a) { return Counted(::fabs(a.v)); }

} // namespace oxref
#endif
