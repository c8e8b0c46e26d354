// A counting stand-in for amrex::Real (test infrastructure): a double that tallies
// every floating-point operation applied to it, so that the reference's own
// kernel headers, compiled against it (oracle/ref/flop_count.cpp, make -C oracle
// flops), give the exact operation count of each point function.  Selected in
// amrex_shim.H by -DOCFD_COUNT_FLOPS.
#ifndef OCFD_FLOP_REAL_H
#define OCFD_FLOP_REAL_H

#include <cmath>

struct FlopTally {
    long long add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0, other = 0;
};
inline FlopTally& flop_tally() {
    static FlopTally t;
    return t;
}

struct CountedReal {
    double v;
    constexpr CountedReal() : v(0.0) {}
    constexpr CountedReal(double x) : v(x) {}
    CountedReal& operator+=(CountedReal o) { ++flop_tally().add; v += o.v; return *this; }
    CountedReal& operator-=(CountedReal o) { ++flop_tally().add; v -= o.v; return *this; }
    CountedReal& operator*=(CountedReal o) { ++flop_tally().mul; v *= o.v; return *this; }
    CountedReal& operator/=(CountedReal o) { ++flop_tally().div; v /= o.v; return *this; }
    CountedReal operator-() const { return CountedReal(-v); }  // a sign flip, not counted
    // the reference keeps some intermediates in plain double (LiDryer.H)
    operator double() const { return v; }
};

inline double& operator+=(double& a, CountedReal b) { ++flop_tally().add; a += b.v; return a; }
inline double& operator-=(double& a, CountedReal b) { ++flop_tally().add; a -= b.v; return a; }
inline double& operator*=(double& a, CountedReal b) { ++flop_tally().mul; a *= b.v; return a; }
inline double& operator/=(double& a, CountedReal b) { ++flop_tally().div; a /= b.v; return a; }

#define OCFD_FLOP_BINOP(OP, FIELD)                                                                         \
    inline CountedReal operator OP(CountedReal a, CountedReal b) { ++flop_tally().FIELD; return CountedReal(a.v OP b.v); } \
    inline CountedReal operator OP(double a, CountedReal b) { ++flop_tally().FIELD; return CountedReal(a OP b.v); }      \
    inline CountedReal operator OP(CountedReal a, double b) { ++flop_tally().FIELD; return CountedReal(a.v OP b); }
OCFD_FLOP_BINOP(+, add)
OCFD_FLOP_BINOP(-, add)
OCFD_FLOP_BINOP(*, mul)
OCFD_FLOP_BINOP(/, div)
#undef OCFD_FLOP_BINOP

#define OCFD_FLOP_CMP(OP)                                                                          \
    inline bool operator OP(CountedReal a, CountedReal b) { ++flop_tally().cmp; return a.v OP b.v; } \
    inline bool operator OP(double a, CountedReal b) { ++flop_tally().cmp; return a OP b.v; }        \
    inline bool operator OP(CountedReal a, double b) { ++flop_tally().cmp; return a.v OP b; }
OCFD_FLOP_CMP(<)
OCFD_FLOP_CMP(>)
OCFD_FLOP_CMP(<=)
OCFD_FLOP_CMP(>=)
OCFD_FLOP_CMP(==)
OCFD_FLOP_CMP(!=)
#undef OCFD_FLOP_CMP

inline CountedReal sqrt(CountedReal a) { ++flop_tally().sqrt; return CountedReal(std::sqrt(a.v)); }
inline CountedReal abs(CountedReal a) { return CountedReal(std::fabs(a.v)); }  // a sign clear, not counted
inline CountedReal fabs(CountedReal a) { return CountedReal(std::fabs(a.v)); }
inline CountedReal exp(CountedReal a) { ++flop_tally().other; return CountedReal(std::exp(a.v)); }
inline CountedReal log(CountedReal a) { ++flop_tally().other; return CountedReal(std::log(a.v)); }
inline CountedReal log10(CountedReal a) { ++flop_tally().other; return CountedReal(std::log10(a.v)); }
inline CountedReal pow(CountedReal a, CountedReal b) { ++flop_tally().other; return CountedReal(std::pow(a.v, b.v)); }
inline CountedReal pow(double a, CountedReal b) { ++flop_tally().other; return CountedReal(std::pow(a, b.v)); }
inline CountedReal pow(CountedReal a, double b) { ++flop_tally().other; return CountedReal(std::pow(a.v, b)); }
inline CountedReal cos(CountedReal a) { ++flop_tally().other; return CountedReal(std::cos(a.v)); }
inline CountedReal sin(CountedReal a) { ++flop_tally().other; return CountedReal(std::sin(a.v)); }

// the reference calls std::sqrt / std::abs explicitly
namespace std {
inline CountedReal sqrt(CountedReal a) { return ::sqrt(a); }
inline CountedReal abs(CountedReal a) { return ::abs(a); }
inline CountedReal exp(CountedReal a) { return ::exp(a); }
inline CountedReal log(CountedReal a) { return ::log(a); }
inline CountedReal log10(CountedReal a) { return ::log10(a); }
inline CountedReal pow(CountedReal a, CountedReal b) { return ::pow(a, b); }
inline CountedReal pow(double a, CountedReal b) { return ::pow(a, b); }
inline CountedReal pow(CountedReal a, double b) { return ::pow(a, b); }
inline CountedReal cos(CountedReal a) { return ::cos(a); }
inline CountedReal sin(CountedReal a) { return ::sin(a); }
}  // namespace std

#endif
