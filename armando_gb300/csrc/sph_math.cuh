// sph_math.cuh -- per-pair arithmetic of the fused SPH passes.
//
// Compiles as CUDA device code and as plain C++ (host shims below), so the
// exact FP32 operation sequence of the kernels can be replayed on a CPU.
//
// Formulas:
//   Wendland C2 (ArmandoThrust/armando.cu:137-191; 2D constant acpu.c:162):
//     W      = K_dim / h^dim * (1 - q/2)^4 (1 + 2q),          q = r / h
//     dW/dx  = K_dim * 5/8 / h^(dim+2) * (q - 2)^3 * (x_i - x_j)
//     K_2 = 7/(4 pi), K_3 = 21/(16 pi) (15/(16 pi) with the legacy switch)
//   Pair test (CERNsource/link_list.f:154-159): dr^2 < (h_i + h_j)^2 with dr^2
//     summed over axes in order, no fused multiply-add, so neighbour sets are
//     bit-identical to the FP32 link_list of the oracle.
//   Tait (FORTRANsource/eos.f90:255-283): p = rho0 c0^2/7 ((1+d)^7 - 1),
//     d = (rho - rho0)/rho0, evaluated as the exact binomial polynomial in d.
#pragma once

#if defined(__CUDACC__)
#define SPH_HD __device__ __forceinline__
#else
#include <cmath>
#define SPH_HD inline
// Host stand-ins for the round-to-nearest intrinsics (build with -ffp-contract=off).
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __fsqrt_rn(float a) { return std::sqrt(a); }
inline float rsqrtf(float a) { return 1.0f / std::sqrt(a); }
#endif

namespace sph {

// ---- float-float (unevaluated sum hi + lo) helpers: error-free transforms ----
struct ff {
    float hi, lo;
};

// Knuth TwoSum: s + e == a + b exactly.
SPH_HD ff two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// a - b == s + e exactly (TwoSum of a and -b).
SPH_HD ff two_diff(float a, float b) {
    float s = __fsub_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fsub_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fadd_rn(b, bb));
    return {s, e};
}
// Dekker Fast2Sum, requires |a| >= |b|.
SPH_HD ff fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}
// a * b == p + e exactly (fused multiply-add residual).
SPH_HD ff two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float e = fmaf(a, b, -p);
    return {p, e};
}
// (a.hi + a.lo) * (b.hi + b.lo), relative error ~2^-44.
SPH_HD ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return p;
}
SPH_HD ff ff_mul_f(ff a, float b) {
    ff p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return p;
}
SPH_HD ff ff_sqr(ff a) {
    ff p = two_prod(a.hi, a.hi);
    p.lo = fmaf(__fmul_rn(2.0f, a.hi), a.lo, p.lo);
    return p;
}
// Accumulate x into acc (acc.lo collects every rounding error).
SPH_HD void ff_acc(ff& acc, ff x) {
    ff s = two_sum(acc.hi, x.hi);
    acc.hi = s.hi;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, x.lo));
}
SPH_HD ff ff_from_double_parts(float hi, float lo) { return {hi, lo}; }

// 1/h as float-float: Newton residual of the correctly rounded reciprocal.
SPH_HD ff ff_recip(float h) {
    float r = __frcp_rn(h);
    float e = fmaf(-r, h, 1.0f);  // exact: 1 - r*h
    return {r, __fmul_rn(e, r)};
}

// ---- Pair test (bit-exact mirror of the oracle's FP32 link_list) ----
template <int DIM>
SPH_HD float dist2_exact(const float* d) {
    float s = __fmul_rn(d[0], d[0]);
    s = __fadd_rn(s, __fmul_rn(d[1], d[1]));
    if (DIM == 3) s = __fadd_rn(s, __fmul_rn(d[2], d[2]));
    return s;
}
SPH_HD bool within_support(float dr2, float hi, float hj) {
    float s = __fadd_rn(hi, hj);
    return dr2 < __fmul_rn(s, s);
}
// Minimum image on a periodic axis, same branch order as the oracle.
SPH_HD float min_image(float dx, float L, float half) {
    if (dx > half) return __fsub_rn(dx, L);
    if (dx < -half) return __fadd_rn(dx, L);
    return dx;
}

// ---- Wendland weight in float-float (density pass) ----
// Returns m_j * W(r, h) with relative error ~1e-12 for the exact pair
// difference x_i - x_j = dh + dl per axis (a float difference is not exact
// when the coordinates differ by more than a factor 2, e.g. near the origin),
// h = (h_i + h_j)/2 passed as its reciprocal ih and the prefactor
// alpha = K_dim * ih^dim (both float-float).
// CLAMP: zero beyond the support (q >= 2), so pairs need no separate test.
template <int DIM, bool CLAMP = false>
SPH_HD ff wendland_mw_ff(const float* dh, const float* dl, ff ih, ff alpha, float mj) {
    // dr^2 = sum (dh + dl)^2 as hi + lo (dl^2 is below the float-float unit).
    ff s0 = two_prod(dh[0], dh[0]);
    float hi = s0.hi;
    float lo = fmaf(__fmul_rn(2.0f, dh[0]), dl[0], s0.lo);
#pragma unroll
    for (int a = 1; a < DIM; ++a) {
        ff sa = two_prod(dh[a], dh[a]);
        float la = fmaf(__fmul_rn(2.0f, dh[a]), dl[a], sa.lo);
        ff t = two_sum(hi, sa.hi);
        hi = t.hi;
        lo = __fadd_rn(lo, __fadd_rn(t.lo, la));
    }
    ff dr2 = fast_two_sum(hi, lo);
    // r = sqrt(dr2): hardware reciprocal square root (a few ulp) and one exact
    // Newton correction from the FMA residual dr2 - r0^2.
    ff r = {0.0f, 0.0f};
    if (dr2.hi > 0.0f) {
        const float rs = rsqrtf(dr2.hi);
        r.hi = __fmul_rn(dr2.hi, rs);
        const float res = fmaf(-r.hi, r.hi, dr2.hi);
        r.lo = __fmul_rn(__fadd_rn(res, dr2.lo), __fmul_rn(0.5f, rs));
    }
    ff q = ff_mul(r, ih);
    // t = 1 - q/2 (q < 2 so |1| >= |q/2|).
    ff t = fast_two_sum(1.0f, __fmul_rn(-0.5f, q.hi));
    t.lo = fmaf(-0.5f, q.lo, t.lo);
    if (CLAMP && !(t.hi + t.lo > 0.0f)) t = ff{0.0f, 0.0f};
    ff t2 = ff_sqr(t);
    ff t4 = ff_sqr(t2);
    // g = 1 + 2q.
    ff g = two_sum(1.0f, __fmul_rn(2.0f, q.hi));
    g.lo = fmaf(2.0f, q.lo, g.lo);
    ff f = ff_mul(t4, g);
    return ff_mul(f, ff_mul_f(alpha, mj));
}

// ---- Wendland gradient factor, plain FP32 (force passes) ----
// dW/dx_i = gw * (x_i - x_j), gw = K_dim * 5/8 * ih^(dim+2) * (q - 2)^3.
template <int DIM>
SPH_HD float wendland_grad_factor(float r, float ih, float kg_ih) {
    float q = __fmul_rn(r, ih);
    float t = __fsub_rn(q, 2.0f);
    return __fmul_rn(kg_ih, __fmul_rn(__fmul_rn(t, t), t));
}

// Tait pressure from d = rho/rho0 - 1: B * ((1+d)^7 - 1), B = rho0 c0^2 / 7.
SPH_HD float tait_poly(float d, float B) {
    float y = __fadd_rn(7.0f, d);
    y = fmaf(y, d, 21.0f);
    y = fmaf(y, d, 35.0f);
    y = fmaf(y, d, 35.0f);
    y = fmaf(y, d, 21.0f);
    y = fmaf(y, d, 7.0f);
    return __fmul_rn(B, __fmul_rn(y, d));
}

}  // namespace sph
