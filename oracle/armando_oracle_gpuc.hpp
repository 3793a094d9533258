// armando_oracle_gpuc.hpp -- CPU restatement of the GPU-C step variant, used
// ONLY as the checker of the library (tests, smoke check, CPU baseline leg).
//
// The GPU-C codes integrate with the third-order TVD Runge-Kutta scheme and
// the continuity equation, with one neighbour list per step:
//   RKintegrateHost    ArmandoThrust/acpu.c:2338-2379 (list, backup, 3 stages)
//   RKstepHost         acpu.c:2293-2336 (loads, pair rates, energy, update)
//   updateListHost     acpu.c:2201-2240 (j with |x_i - x_j| < 2 h_i)
//   pair rates, variant 1 (host path)    acpu.c:346-437  balanceMassMomentumHost
//   pair rates, variant 2 (device path)  ArmandoThrust/armando.cu:429-513
//   energy rate        acpu.c:510-534    de/dt = p drho/dt / rho^2
//   loads              acpu.c:1047-1076  (gravity, then load zones, on itype > 0)
//   fix zones          acpu.c:916-926, armando.cu:1026-1036 (after the update)
//   update + EOS       acpu.c:873-966 (variant 1), armando.cu:987-1074 (variant 2)
//   EOS functions      acpu.c:560-870; ESS from Code/armando.cu:572-598, 703-723
//   Wendland W, dW/dr  acpu.c:146-201 with h_i (2D alpha 7/(4 pi h^2); 3D as
//                      the CERN path: 21/(16 pi h^3), 15/16 pi behind the switch)
// Restated without the reference's capacity limits: no cap on the neighbour
// list (the reference keeps the first MAXN = 21 in 2D, self included).
// Departures, each noted where it is made: the device variant indexes the
// material table with |itype| (armando.cu:1030 indexes it with the signed
// Material); ESS is restated on absolute density (Code/armando.cu stores the
// density perturbation there).
#pragma once
#include <array>
#include <cmath>
#include <vector>

#include "armando_oracle.hpp"

namespace ao {

// EOS types (hMatType, acpu.c:1795-1798; Code/armando.cu:884-887).
enum GpucEos { EOS_BOUNDARY = 0, EOS_GAS = 1, EOS_POLY = 2, EOS_SHOCK = 3, EOS_TAIT = 4, EOS_ESS = 5 };

struct GpucMaterial {
    int type = EOS_TAIT;
    double prop[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
};

// Load and fix zones (acpu.c:33-48): the open box lo < x < hi, x and y only
// in 2D (armando2D.cu:756-762).
struct GpucLoad {
    float lo[3], hi[3], g[3], w;
};
struct GpucFix {
    float lo[3], hi[3], v[3];
    float tau = 0.f;  // > 0: a pump zone, Code/armando.cu:1046-1055 (a rate, not a set velocity)
};

template <class R>
inline bool gpuc_in_zone(const float* lo, const float* hi, const R* x, int dim) {
    for (int d = 0; d < dim; ++d)
        if (!(x[d] > R(lo[d]) && x[d] < R(hi[d]))) return false;
    return true;
}

template <class R>
struct GpucSetup {
    int variant = 1;  // 1: host path (acpu.c), 2: device kernels (armando.cu)
    int legacy3d = 0;
    R gravity[3] = {R(0), R(0), R(0)};
    std::vector<GpucMaterial> mat;  // by |itype|
    std::vector<GpucLoad> loads;
    std::vector<GpucFix> fixes;
};

// Density clamp rho >= 0.9 rho0 (densityTait/Poly/Shock, acpu.c:843-870).
template <class R>
inline R gpuc_clamp(R rho, R rho0) {
    return (rho < R(0.9) * rho0) ? R(0.9) * rho0 : rho;
}

// The EOS of one particle after its update (acpu.c:932-962): rho (clamped
// where the type clamps), p and c from rho and u.
template <class R>
inline void gpuc_eos(const GpucMaterial& M, R& rho, const R& u, R& p, R& c) {
    using std::pow;
    using std::sqrt;
    const R p0 = R(M.prop[0]), p1 = R(M.prop[1]), p2 = R(M.prop[2]), p3 = R(M.prop[3]),
            p4 = R(M.prop[4]), p5 = R(M.prop[5]), p6 = R(M.prop[6]), p7 = R(M.prop[7]);
    switch (M.type) {
    case EOS_BOUNDARY:  // acpu.c:934-937: clamp, p = 0 * pressureTait, c = c0
        rho = gpuc_clamp(rho, p0);
        p = R(0);
        c = p1;
        break;
    case EOS_GAS: {  // acpu.c:560-580, 712-725
        p = (p1 - R(1)) * rho * u + p2;
        c = sqrt(p1 * (p1 - R(1)) * u);
        break;
    }
    case EOS_POLY: {  // acpu.c:582-620, 727-740
        rho = gpuc_clamp(rho, p0);
        const R mu = (rho - p0) / p0;
        if (mu < R(0)) p = (p6 * mu + p7 * mu * mu) + (p4 * p0 * u);
        else p = (p1 * mu + p2 * mu * mu + p3 * mu * mu * mu) + ((p4 + p5 * mu) * p0 * u);
        c = sqrt(p1 / rho);
        break;
    }
    case EOS_SHOCK: {  // acpu.c:622-651, 742-754
        rho = gpuc_clamp(rho, p0);
        const R mu = (rho - p0) / p0;
        const R den = R(1) - (p3 - R(1)) * mu;
        const R ph = (p0 * p1 * p1 * mu * (R(1) + mu)) / (den * den);
        p = ph + p2 * p0 * (u - (R(0.5) * ph / p0 * (mu / (R(1) + mu))));
        c = p1;
        break;
    }
    case EOS_TAIT: {  // acpu.c:663-680, 768-780 (no pmin clamp there)
        rho = gpuc_clamp(rho, p0);
        const R r = rho / p0, r2 = r * r, r7 = r2 * r2 * r2 * r;
        p = p0 * p1 * p1 / R(7) * (r7 - R(1));
        c = p1;
        break;
    }
    case EOS_ESS: {  // Code/armando.cu:572-598, 703-723, on absolute density
        const R mu = rho / p0 - R(1);
        p = mu * p0 * p1 * p1 + u * p0 * p2;
        if (p < p3) p = p3;
        c = p1;
        break;
    }
    default:  // acpu.c:963-964
        p = R(0);
        break;
    }
}

// Sound speed of a particle from its state (the value the previous update
// left in Sound, for the first stage of a step).
template <class R>
inline R gpuc_sound(const GpucMaterial& M, R rho, const R& u) {
    R p = R(0), c = R(0);
    gpuc_eos(M, rho, u, p, c);
    return c;
}

inline const GpucMaterial& gpuc_material(const std::vector<GpucMaterial>& mat, int itype) {
    const int k = itype < 0 ? -itype : itype;
    if (k >= (int)mat.size()) throw std::runtime_error("itype outside the material table");
    return mat[k];
}

// updateListHost (acpu.c:2201-2240): for every i the particles j != i with
// sqrtf(dx^2 + dy^2 + dz^2) < 2 h_i, distances in coordinate precision Rc,
// axes summed in order; cells of 2 max(h), 3^dim stencil.
template <class Rc>
std::vector<std::vector<int>> gpuc_list(int64_t n, int dim, const Rc* x, const Rc* h) {
    Rc lo[3] = {Rc(0), Rc(0), Rc(0)}, hi[3] = {Rc(0), Rc(0), Rc(0)}, mh = Rc(0);
    for (int d = 0; d < dim; ++d) {
        lo[d] = Rc(1e30);
        hi[d] = Rc(-1e30);
    }
    for (int64_t i = 0; i < n; ++i) {
        for (int d = 0; d < dim; ++d) {
            lo[d] = std::min(lo[d], x[i * dim + d]);
            hi[d] = std::max(hi[d], x[i * dim + d]);
        }
        mh = std::max(mh, h[i]);
    }
    const double cell = 2.0 * (double)mh;
    int nc[3] = {1, 1, 1};
    for (int d = 0; d < dim; ++d) nc[d] = (int)(((double)hi[d] - (double)lo[d]) / cell) + 1;
    auto coord = [&](int64_t i, int d) {
        int c = (int)(((double)x[i * dim + d] - (double)lo[d]) / cell);
        return std::min(std::max(c, 0), nc[d] - 1);
    };
    std::vector<std::vector<int>> cells((size_t)nc[0] * nc[1] * nc[2]);
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        for (int d = dim - 1; d >= 0; --d) c = c * nc[d] + coord(i, d);
        cells[c].push_back((int)i);
    }
    std::vector<std::vector<int>> list(n);
    for (int64_t i = 0; i < n; ++i) {
        int cc[3] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) cc[d] = coord(i, d);
        const Rc lim = Rc(Rc(2) * h[i]);
        for (int kz = (dim == 3 ? -1 : 0); kz <= (dim == 3 ? 1 : 0); ++kz)
            for (int ky = -1; ky <= 1; ++ky)
                for (int kx = -1; kx <= 1; ++kx) {
                    const int q[3] = {cc[0] + kx, cc[1] + ky, cc[2] + kz};
                    bool in = true;
                    for (int d = 0; d < dim; ++d) in = in && q[d] >= 0 && q[d] < nc[d];
                    if (!in) continue;
                    int64_t c = 0;
                    for (int d = dim - 1; d >= 0; --d) c = c * nc[d] + q[d];
                    for (int j : cells[c]) {
                        if (j == i) continue;
                        Rc r2 = Rc(0);
                        for (int d = 0; d < dim; ++d) {
                            const Rc e = Rc(x[i * dim + d] - x[(int64_t)j * dim + d]);
                            const Rc sq = Rc(e * e);
                            r2 = (d == 0) ? sq : Rc(r2 + sq);
                        }
                        using std::sqrt;
                        if (Rc(sqrt(r2)) < lim) list[i].push_back(j);
                    }
                }
        std::sort(list[i].begin(), list[i].end());
    }
    return list;
}

// Pair rates of one stage: drho/dt, dv/dt (+ loads), de/dt.
template <class R>
void gpuc_rates(const State<R>& s, const std::vector<std::vector<int>>& list,
                const GpucSetup<R>& G, std::vector<R>& dv, std::vector<R>& drho,
                std::vector<R>& du) {
    using std::sqrt;
    const int dim = s.dim;
    const int64_t n = s.n;
    dv.assign(n * dim, R(0));
    drho.assign(n, R(0));
    du.assign(n, R(0));
    for (int64_t i = 0; i < n; ++i) {
        R wz = R(0);
        if (s.itype[i] > 0) {  // updateLoadsHost: gravity over every fluid particle, then the zones
            for (int d = 0; d < dim; ++d) dv[i * dim + d] = G.gravity[d];
            for (const GpucLoad& Z : G.loads) {
                if (!gpuc_in_zone(Z.lo, Z.hi, &s.x[i * dim], dim)) continue;
                for (int d = 0; d < dim; ++d) dv[i * dim + d] = dv[i * dim + d] + R(Z.g[d]);
                wz = wz + R(Z.w);
            }
            // pump zones (Code/armando.cu:1046-1055): dv/dt += (vel - v) / tau
            for (const GpucFix& Z : G.fixes) {
                if (!(Z.tau > 0.f) || !gpuc_in_zone(Z.lo, Z.hi, &s.x[i * dim], dim)) continue;
                for (int d = 0; d < dim; ++d)
                    dv[i * dim + d] = dv[i * dim + d] + (R(Z.v[d]) - s.v[i * dim + d]) / R(Z.tau);
            }
        }
        const R hi = s.h[i];
        const R w0 = kernel_w(R(0), hi, dim, G.legacy3d);
        R rd = R(0), a[3] = {R(0), R(0), R(0)};
        for (int j : list[i]) {
            R dx[3] = {R(0), R(0), R(0)}, r2 = R(0), dvr = R(0);
            for (int d = 0; d < dim; ++d) {
                dx[d] = s.x[i * dim + d] - s.x[(int64_t)j * dim + d];
                r2 = r2 + dx[d] * dx[d];
                dvr = dvr + dx[d] * (s.v[i * dim + d] - s.v[(int64_t)j * dim + d]);
            }
            R dr = sqrt(r2);
            if (dr < R(0.01) * hi) continue;  // dr := 100 h: W = dW/dr = 0 (acpu.c:379)
            const R w = kernel_w(dr, hi, dim, G.legacy3d);
            const R dwdr = kernel_dwdr(dr, hi, dim, G.legacy3d);
            const R mj = s.m[j];
            const R rhoi = s.rho[i], rhoj = s.rho[(size_t)j];
            const R ci = s.c[i], cj = s.c[(size_t)j];
            const bool same = s.itype[i] == s.itype[(size_t)j];
            R fpair = R(0);  // along (x_i - x_j)/dr, times dW/dr
            if (G.variant == 1 || same) {
                rd = rd + mj * dvr * dwdr / dr;  // continuity
                if (G.variant == 1)              // acpu.c:398-400
                    fpair = fpair + mj * (-(s.p[i] + s.p[(size_t)j]) / (rhoi * rhoj));
                else  // armando.cu:483-485
                    fpair = fpair + mj * (-(s.p[i] / (rhoi * rhoi) + s.p[(size_t)j] / (rhoj * rhoj)));
                // shock correction for mass (acpu.c:407-411)
                rd = rd + mj * ((rhoi - rhoj) * (R(2) * ci / (rhoi + rhoj))) * dwdr;
                // shock correction for momentum (acpu.c:413-422)
                const R vneg = dvr < R(0) ? dvr : R(0);
                const R f = vneg * hi / (dr * dr + R(0.01) * hi * hi) * (R(2) * ci / (rhoi + rhoj)) * R(0.03);
                fpair = fpair + mj * f;
            }
            for (int d = 0; d < dim; ++d) a[d] = a[d] + fpair * dwdr * dx[d] / dr;
            if (!same) {  // boundary repulsion along (x_i - x_j)/dr
                R f;
                if (G.variant == 1)  // acpu.c:424-429
                    f = mj / (s.m[i] + mj) * (R(0.02) * w / w0 * ci * cj / dr);
                else  // armando.cu:507-512
                    f = R(0.5) * w * mj / rhoj / s.h[(size_t)j] * cj * cj;
                for (int d = 0; d < dim; ++d) a[d] = a[d] + f * dx[d] / dr;
            }
        }
        drho[i] = rd;
        for (int d = 0; d < dim; ++d) dv[i * dim + d] = dv[i * dim + d] + a[d];
        du[i] = wz + s.p[i] * rd / (s.rho[i] * s.rho[i]);  // balanceEnergyHost on the loads' w
    }
}

// Open boundaries (ArmandoThrust/armando.cu:2640-2856), applied at a step's
// start, inlets before outlets as RKintegrateDevice calls them (armando.cu:
// 3314-3318). Geometry in FP32 with the reference's operation order, so the
// emitted positions are the library's bit for bit.
struct GpucInlet {
    float o[3], n[3], R;
    int itype;
    float mass, h, speed, rho, u;
    float dist = 0.f;
};
struct GpucOutlet {
    float o[3], n[3], R;
};
struct GpucOpen {
    std::vector<GpucInlet> in;
    std::vector<GpucOutlet> out;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

// inletDevice (armando.cu:2792-2845): the lattice of one emission. 3D: the
// inlet's unit normal w, u the coordinate axis of w's smallest |component|
// (the last of x, y, z on ties), v = w x u, points (iu u + iv v) h/1.2 with
// |r| < R, iu, iv in [-n, n], n = roundf(1.2 R/h). 2D: the same rows along
// u = (-w_y, w_x) only (the 2D form of the disk: a segment across the inflow).
inline void gpuc_inlet_lattice(const GpucInlet& I, int dim, std::vector<float>& pos, float w[3]) {
    const float len = std::sqrt(I.n[0] * I.n[0] + I.n[1] * I.n[1] + I.n[2] * I.n[2]);
    for (int d = 0; d < 3; ++d) w[d] = I.n[d] / len;
    const float sp = I.h / 1.2f;
    const int nn = (int)std::lround(1.2f * I.R / I.h);
    pos.clear();
    if (dim == 2) {
        const float u[2] = {-w[1], w[0]};
        for (int iu = -nn; iu <= nn; ++iu) {
            const float r0 = ((float)iu * u[0]) * sp, r1 = ((float)iu * u[1]) * sp;
            if (std::sqrt(r0 * r0 + r1 * r1) < I.R) {
                pos.push_back(I.o[0] + r0);
                pos.push_back(I.o[1] + r1);
            }
        }
        return;
    }
    float u[3] = {0, 0, 0};
    const float a[3] = {std::fabs(w[0]), std::fabs(w[1]), std::fabs(w[2])};
    if (a[0] <= a[1] && a[0] <= a[2]) u[0] = 1.f, u[1] = 0.f, u[2] = 0.f;
    if (a[1] <= a[0] && a[1] <= a[2]) u[0] = 0.f, u[1] = 1.f, u[2] = 0.f;
    if (a[2] <= a[0] && a[2] <= a[1]) u[0] = 0.f, u[1] = 0.f, u[2] = 1.f;
    const float v[3] = {w[1] * u[2] - w[2] * u[1], w[2] * u[0] - w[0] * u[2], w[0] * u[1] - w[1] * u[0]};
    for (int iv = -nn; iv <= nn; ++iv)
        for (int iu = -nn; iu <= nn; ++iu) {
            float r[3];
            for (int d = 0; d < 3; ++d) r[d] = ((float)iu * u[d] + (float)iv * v[d]) * sp;
            if (std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) < I.R)
                for (int d = 0; d < 3; ++d) pos.push_back(I.o[d] + r[d]);
        }
}

// checkOutDevice (armando.cu:2682-2722): behind an outlet within its radius,
// or outside the box.
inline bool gpuc_leaves(const float* x, int dim, const GpucOpen& O) {
    for (const GpucOutlet& Q : O.out) {
        float dn = 0.f;
        for (int d = 0; d < dim; ++d) dn = dn + (x[d] - Q.o[d]) * Q.n[d];
        float dr = 0.f;
        for (int d = 0; d < dim; ++d) {
            const float e = (x[d] - Q.o[d]) - dn * Q.n[d];
            dr = dr + e * e;
        }
        if (dn < 0.f && std::sqrt(dr) < Q.R) return true;
    }
    for (int d = 0; d < dim; ++d)
        if (x[d] > O.hi[d] || x[d] < O.lo[d]) return true;
    return false;
}

// Emission then removal on the state (order kept: survivors, then the new
// particles in emission order).
template <class R>
void gpuc_open(State<R>& s, GpucOpen& O, double dt) {
    const int dim = s.dim;
    std::vector<float> pos;
    float w[3];
    for (GpucInlet& I : O.in) {
        if (I.itype == 0) continue;
        I.dist = I.dist + I.speed * (float)dt;
        if (!(I.dist > I.h / 1.2f)) continue;
        I.dist = I.dist - I.h / 1.2f;
        gpuc_inlet_lattice(I, dim, pos, w);
        const int64_t k = (int64_t)pos.size() / dim;
        for (int64_t q = 0; q < k; ++q) {
            for (int d = 0; d < dim; ++d) {
                s.x.push_back(R(pos[q * dim + d]));
                s.v.push_back(R(I.speed * w[d]));
                s.dvdt.push_back(R(0));
            }
            s.m.push_back(R(I.mass));
            s.h.push_back(R(I.h));
            s.rho.push_back(R(I.rho));
            s.p.push_back(R(0));
            s.u.push_back(R(I.u));
            s.c.push_back(R(0));
            s.itype.push_back(I.itype);
            s.dudt.push_back(R(0));
        }
        s.n += k;
    }
    int64_t keep = 0;
    for (int64_t i = 0; i < s.n; ++i) {
        float xf[3];
        for (int d = 0; d < dim; ++d) xf[d] = (float)s.x[i * dim + d];
        if (gpuc_leaves(xf, dim, O)) continue;
        for (int d = 0; d < dim; ++d) {
            s.x[keep * dim + d] = s.x[i * dim + d];
            s.v[keep * dim + d] = s.v[i * dim + d];
            s.dvdt[keep * dim + d] = s.dvdt[i * dim + d];
        }
        s.m[keep] = s.m[i];
        s.h[keep] = s.h[i];
        s.rho[keep] = s.rho[i];
        s.p[keep] = s.p[i];
        s.u[keep] = s.u[i];
        s.c[keep] = s.c[i];
        s.itype[keep] = s.itype[i];
        s.dudt[keep] = s.dudt[i];
        ++keep;
    }
    s.n = keep;
    s.x.resize(keep * dim);
    s.v.resize(keep * dim);
    s.dvdt.resize(keep * dim);
    for (auto* a : {&s.m, &s.h, &s.rho, &s.p, &s.u, &s.c, &s.dudt}) a->resize(keep);
    s.itype.resize(keep);
}

// One TVD-RK3 step (acpu.c:2360-2373): the list at the step's start, then
// X = X0 + alpha (X + dt dX/dt - X0) for alpha = 1, 1/4, 2/3. s.p holds the
// pressures of the previous update on entry; s.c is recomputed from rho, u.
// rates_out: dv/dt [n*dim] and de/dt [n] of the last stage.
template <class R, class Rc = R>
void gpuc_rk3_step(State<R>& s, const GpucSetup<R>& G, double dt, std::vector<R>* dv_out = nullptr,
                   std::vector<R>* du_out = nullptr, GpucOpen* open = nullptr) {
    if (open) gpuc_open(s, *open, dt);
    const int dim = s.dim;
    const int64_t n = s.n;
    if (n == 0) {  // every particle left: nothing to step until an inlet emits
        if (dv_out) dv_out->clear();
        if (du_out) du_out->clear();
        return;
    }
    std::vector<Rc> xc(n * dim), hc(n);
    for (int64_t i = 0; i < n * dim; ++i) xc[i] = Rc(s.x[i]);
    for (int64_t i = 0; i < n; ++i) hc[i] = Rc(s.h[i]);
    const std::vector<std::vector<int>> list = gpuc_list<Rc>(n, dim, xc.data(), hc.data());
    for (int64_t i = 0; i < n; ++i) s.c[i] = gpuc_sound(gpuc_material(G.mat, s.itype[i]), s.rho[i], s.u[i]);
    const std::vector<R> x0 = s.x, v0 = s.v, rho0 = s.rho, u0 = s.u;
    const R Rdt = R(dt);
    std::vector<R> dv, drho, du;
    for (int stage = 0; stage < 3; ++stage) {
        const R alpha = stage == 0 ? R(1) : stage == 1 ? R(0.25) : R(2) / R(3);
        gpuc_rates(s, list, G, dv, drho, du);
        for (int64_t i = 0; i < n; ++i) {
            const int it = s.itype[i];
            if (G.variant == 1 && it == 0) continue;  // acpu.c:894
            for (int d = 0; d < dim; ++d) {
                const int64_t k = i * dim + d;
                s.x[k] = x0[k] + alpha * (s.x[k] + Rdt * s.v[k] - x0[k]);
            }
            for (int d = 0; d < dim; ++d) {
                const int64_t k = i * dim + d;
                s.v[k] = v0[k] + alpha * (s.v[k] + Rdt * dv[k] - v0[k]);
            }
            s.rho[i] = rho0[i] + alpha * (s.rho[i] + Rdt * drho[i] - rho0[i]);
            s.u[i] = u0[i] + alpha * (s.u[i] + Rdt * du[i] - u0[i]);
            const GpucMaterial& M = gpuc_material(G.mat, it);
            if (G.variant == 1 && it <= 0)  // acpu.c:910-914
                for (int d = 0; d < dim; ++d) s.v[i * dim + d] = v0[i * dim + d];
            for (const GpucFix& Z : G.fixes)  // acpu.c:916-926 at the new position
                if (Z.tau == 0.f && gpuc_in_zone(Z.lo, Z.hi, &s.x[i * dim], dim))
                    for (int d = 0; d < dim; ++d) s.v[i * dim + d] = R(Z.v[d]);
            if (M.type == EOS_BOUNDARY)
                for (int d = 0; d < dim; ++d) s.v[i * dim + d] = v0[i * dim + d];
            gpuc_eos(M, s.rho[i], s.u[i], s.p[i], s.c[i]);
        }
    }
    if (dv_out) *dv_out = dv;
    if (du_out) *du_out = du;
}

}  // namespace ao
