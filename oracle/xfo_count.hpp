// xfo_count.hpp - counting scalar for the algorithmic flop count of the oracle (test infrastructure).
//
// Cnt behaves like double and counts each +, -, *, /, sqrt, log, exp as one flop. Comparisons,
// negation, fabs, fmin and fmax are not counted. Arithmetic on two compile-time constants is
// folded by the compiler and never reaches Cnt. The count is what the restated algorithm needs;
// it is the numerator of the roofline fraction reported for the compute-bound kernels.
#pragma once

#include <cmath>
#include <cstdint>

namespace xfo {

struct Cnt {
    double v;
    static thread_local uint64_t flops;
    Cnt() : v(0.0) {}
    Cnt(double x) : v(x) {}  // NOLINT: implicit like a double
    explicit operator double() const { return v; }
    Cnt operator-() const { return Cnt(-v); }
    Cnt &operator+=(const Cnt &o) { ++flops; v += o.v; return *this; }
    Cnt &operator-=(const Cnt &o) { ++flops; v -= o.v; return *this; }
    Cnt &operator*=(const Cnt &o) { ++flops; v *= o.v; return *this; }
    Cnt &operator/=(const Cnt &o) { ++flops; v /= o.v; return *this; }
    friend Cnt operator+(Cnt a, Cnt b) { ++flops; return Cnt(a.v + b.v); }
    friend Cnt operator-(Cnt a, Cnt b) { ++flops; return Cnt(a.v - b.v); }
    friend Cnt operator*(Cnt a, Cnt b) { ++flops; return Cnt(a.v * b.v); }
    friend Cnt operator/(Cnt a, Cnt b) { ++flops; return Cnt(a.v / b.v); }
    friend bool operator<(Cnt a, Cnt b) { return a.v < b.v; }
    friend bool operator>(Cnt a, Cnt b) { return a.v > b.v; }
    friend bool operator<=(Cnt a, Cnt b) { return a.v <= b.v; }
    friend bool operator>=(Cnt a, Cnt b) { return a.v >= b.v; }
    friend bool operator==(Cnt a, Cnt b) { return a.v == b.v; }
    friend Cnt sqrt(Cnt a) { ++flops; return Cnt(std::sqrt(a.v)); }
    friend Cnt log(Cnt a) { ++flops; return Cnt(std::log(a.v)); }
    friend Cnt exp(Cnt a) { ++flops; return Cnt(std::exp(a.v)); }
    friend Cnt fabs(Cnt a) { return Cnt(std::fabs(a.v)); }
    friend Cnt fmax(Cnt a, Cnt b) { return Cnt(std::fmax(a.v, b.v)); }
    friend Cnt fmin(Cnt a, Cnt b) { return Cnt(std::fmin(a.v, b.v)); }
};

inline double dval(Cnt x) { return x.v; }

}  // namespace xfo
