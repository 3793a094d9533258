// armando_oracle_flops.hpp -- floating-point operation count of the reference
// algorithm. Test and measurement infrastructure only.
//
// Flop is an FP64 value whose every arithmetic operation increments one
// counter: +, -, *, / and sqrt, exp count 1 each; negation, fabs and
// comparisons count 0; there are no fused multiply-adds in the restatement.
// Running the templated pair-loop oracle (armando_oracle.hpp, the restatement
// of CERNsource time_integration.f / single_step.f / link_list.f) on Flop
// values counts the operations one iteration of the reference's algorithm
// takes on a given state: link_list's cell ids and pair tests (each pair j > i
// tested once), density, EOS, forces, artificial viscosity and heat, external
// heat, predictor and corrector. That count per particle is the algorithmic
// FLOP figure the measured step time is set against.
#pragma once
#include <cmath>

#include "armando_oracle.hpp"

namespace ao {

struct Flop {
    double v = 0.0;
    static inline unsigned long long count = 0;
    Flop() = default;
    Flop(double a) : v(a) {}  // NOLINT: implicit constants
    explicit operator double() const { return v; }
    explicit operator float() const { return (float)v; }
    explicit operator int() const { return (int)v; }
};
inline Flop operator+(Flop a, Flop b) { ++Flop::count; return Flop(a.v + b.v); }
inline Flop operator-(Flop a, Flop b) { ++Flop::count; return Flop(a.v - b.v); }
inline Flop operator*(Flop a, Flop b) { ++Flop::count; return Flop(a.v * b.v); }
inline Flop operator/(Flop a, Flop b) { ++Flop::count; return Flop(a.v / b.v); }
inline Flop operator-(Flop a) { return Flop(-a.v); }
inline bool operator<(Flop a, Flop b) { return a.v < b.v; }
inline bool operator>(Flop a, Flop b) { return a.v > b.v; }
inline bool operator<=(Flop a, Flop b) { return a.v <= b.v; }
inline bool operator>=(Flop a, Flop b) { return a.v >= b.v; }
inline bool operator==(Flop a, Flop b) { return a.v == b.v; }
inline bool operator!=(Flop a, Flop b) { return a.v != b.v; }
inline Flop sqrt(Flop a) { ++Flop::count; return Flop(std::sqrt(a.v)); }
inline Flop exp(Flop a) { ++Flop::count; return Flop(std::exp(a.v)); }
inline Flop pow(Flop a, double e) { ++Flop::count; return Flop(std::pow(a.v, e)); }
inline Flop fabs(Flop a) { return Flop(std::fabs(a.v)); }

}  // namespace ao
