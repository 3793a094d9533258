// armando_oracle_tangent.hpp -- FP64 tangent-linear of the oracle step and the
// losses the GPU adjoint is checked on. Test infrastructure only.
//
// Forward-mode dual numbers (value + one directional derivative) run through
// the templated pair-loop oracle (armando_oracle.hpp, a restatement of
// CERNsource time_integration.f / single_step.f), so the derivative of a loss
// along any seed (parameters alpha, beta, c0, q0 and initial x, v, u) comes out
// exactly as the FP64 tangent-linear model. Non-smooth branches follow the
// value part: art_visc acts only while v_ij . r_ij < 0, the Tait clamp sets a
// constant, u = max(0, .) is flat below zero.
#pragma once
#include "armando_oracle.hpp"

namespace ao {

struct Dual {
    double v = 0.0, d = 0.0;
    Dual() = default;
    Dual(double a) : v(a), d(0.0) {}  // NOLINT: implicit constants
    Dual(double a, double b) : v(a), d(b) {}
    explicit operator double() const { return v; }
    explicit operator float() const { return (float)v; }
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
inline bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
inline Dual sqrt(Dual a) {
    double s = std::sqrt(a.v);
    return {s, s > 0 ? a.d / (2.0 * s) : 0.0};
}
inline Dual exp(Dual a) {
    double e = std::exp(a.v);
    return {e, e * a.d};
}
inline Dual fabs(Dual a) { return a.v < 0 ? -a : a; }
inline Dual pow(Dual a, double e) {
    const double pv = std::pow(a.v, e);
    return {pv, a.v != 0.0 ? e * pv / a.v * a.d : 0.0};
}

// Loss on the final state of a run of `steps` iterations:
//   L = w_ke * sum_fluid m |v|^2 / 2
//     + w_p  * sum_fluid w(x) p / w_ref    (p: pressure output of the last
//                                           iteration, its summation density)
//     + w_u  * sum_fluid w(x) u / w_ref
// with the smooth probe w(x) = (1 - |x - c|^2 / R^2)^3 inside radius R.
struct LossSpec {
    double w_ke = 1.0, w_p = 0.0, w_u = 0.0;
    double c[3] = {0, 0, 0};
    double radius = 1.0;
    double w_ref = 1.0;
};

template <class R>
inline R probe_weight(const R* x, int dim, const LossSpec& L) {
    R r2 = R(0);
    for (int d = 0; d < dim; ++d) {
        R e = x[d] - R(L.c[d]);
        r2 = r2 + e * e;
    }
    R t = R(1) - r2 / R(L.radius * L.radius);
    if (!(t > R(0))) return R(0);
    return t * t * t;
}

template <class R>
R run_loss(State<R>& s, const Params<R>& P, int its0, int steps, double dt, const LossSpec& L) {
    for (int k = 0; k < steps; ++k) leapfrog_step<R, double>(s, P, its0 + k, dt);
    R ke = R(0), lp = R(0), lu = R(0);
    for (int64_t i = 0; i < s.n; ++i) {
        if (!s.fluid(i)) continue;
        R v2 = R(0);
        for (int d = 0; d < s.dim; ++d) v2 = v2 + s.v[i * s.dim + d] * s.v[i * s.dim + d];
        ke = ke + R(0.5) * s.m[i] * v2;
        if (L.w_p != 0.0 && steps > 0) lp = lp + probe_weight(&s.x[i * s.dim], s.dim, L) * s.p[i];
        if (L.w_u != 0.0) lu = lu + probe_weight(&s.x[i * s.dim], s.dim, L) * s.u[i];
    }
    return R(L.w_ke) * ke + R(L.w_p / L.w_ref) * lp + R(L.w_u / L.w_ref) * lu;
}

}  // namespace ao
