// TEST INFRASTRUCTURE (oracle).  Not part of the product.
//
// A double that counts the floating-point operations done on it.  The oracle
// compiled with -DORC_COUNT_FLOPS computes in this type instead of double
// (every value is still the same IEEE double, computed by the same
// operations in the same order, so the results are bit-identical), and the
// counts give the algorithmic operation count of each stage of the
// reference's step.
//
// Counted: additions and subtractions (add), multiplications (mul),
// divisions (div), square roots (sqrt), pow calls (pow), explicit fused
// multiply-adds (fma, two operations).  Not counted: comparisons,
// negation, fabs, floor and conversions, and arithmetic on plain double
// constants (the configuration's gamma, dt/2 and the like), which a
// compiler hoists out of the loops.
#pragma once
#include <cmath>

namespace orc {

struct FlopCounts {
    unsigned long long add, mul, div, sqrt, pow, fma;
};

inline FlopCounts &flop_counts() {
    static FlopCounts c{};
    return c;
}

struct Counted {
    double v;
    Counted() = default;
    constexpr Counted(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
    Counted operator-() const { return Counted(-v); }
    Counted &operator+=(Counted o) { ++flop_counts().add; v += o.v; return *this; }
    Counted &operator-=(Counted o) { ++flop_counts().add; v -= o.v; return *this; }
    Counted &operator*=(Counted o) { ++flop_counts().mul; v *= o.v; return *this; }
    Counted &operator/=(Counted o) { ++flop_counts().div; v /= o.v; return *this; }
};

inline Counted operator+(Counted a, Counted b) { ++flop_counts().add; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { ++flop_counts().add; return Counted(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { ++flop_counts().mul; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { ++flop_counts().div; return Counted(a.v / b.v); }
inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { return a.v >= b.v; }
inline bool operator==(Counted a, Counted b) { return a.v == b.v; }
inline bool operator!=(Counted a, Counted b) { return a.v != b.v; }

inline Counted sqrt(Counted a) { ++flop_counts().sqrt; return Counted(std::sqrt(a.v)); }
inline Counted pow(Counted a, Counted b) { ++flop_counts().pow; return Counted(std::pow(a.v, b.v)); }
inline Counted fma(Counted a, Counted b, Counted c) { ++flop_counts().fma; return Counted(std::fma(a.v, b.v, c.v)); }
inline Counted fabs(Counted a) { return Counted(std::fabs(a.v)); }
inline Counted floor(Counted a) { return Counted(std::floor(a.v)); }

static_assert(sizeof(Counted) == sizeof(double), "Counted must have the layout of a double");

}  // namespace orc
