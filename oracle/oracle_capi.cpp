// oracle_capi.cpp -- extern "C" entry points of the CPU oracle, for the test
// suite, the smoke check and the CPU-baseline leg of the benchmark only.
// The product library never links this file.
#include <cstdio>
#include <cstring>

#include "../include/armando.h"
#include "armando_oracle.hpp"
#include "armando_oracle_gather.hpp"
#include "armando_oracle_flops.hpp"
#include "armando_oracle_gpuc.hpp"
#include "armando_oracle_tangent.hpp"

namespace {

template <class R>
ao::Params<R> to_params(const armando_params* p) {
    ao::Params<R> P;
    P.dim = p->dim;
    P.pa_sph = p->pa_sph;
    P.visc = p->visc;
    P.visc_artificial = p->visc_artificial;
    P.heat_artificial = p->heat_artificial;
    P.heat_external = p->heat_external;
    P.kernel_3d_legacy = p->kernel_3d_legacy;
    for (int d = 0; d < 3; ++d) {
        P.periodic[d] = p->periodic[d];
        P.gravity[d] = R(p->gravity[d]);
        P.heat_center[d] = R(p->heat_center[d]);
        P.period_lo[d] = p->period_lo[d];
        P.period_hi[d] = p->period_hi[d];
    }
    P.rho0 = R(p->rho0);
    P.c0 = R(p->c0);
    P.pmin = R(p->pmin);
    P.eta = R(p->eta);
    P.av_alpha = R(p->av_alpha);
    P.av_beta = R(p->av_beta);
    P.av_eta = R(p->av_eta);
    P.ah_g1 = R(p->ah_g1);
    P.ah_g2 = R(p->ah_g2);
    P.ah_eta = R(p->ah_eta);
    P.heat_q0 = R(p->heat_q0);
    P.heat_sigma = R(p->heat_sigma);
    P.heat_t_end = p->heat_t_end;
    P.wall_model = p->wall_model;
    P.density_form = p->density_form;
    P.average_velocity = p->average_velocity;
    P.sle = p->sle;
    return P;
}

template <class R>
ao::State<R> load_state(int dim, int64_t n, const R* x, const R* v, const R* m, const R* rho,
                        const R* p, const R* u, const R* h, const int* itype, const R* dvdt,
                        const R* dudt) {
    ao::State<R> s;
    s.n = n;
    s.dim = dim;
    s.x.assign(x, x + n * dim);
    s.v.assign(v, v + n * dim);
    s.m.assign(m, m + n);
    s.rho.assign(rho, rho + n);
    s.p.assign(p, p + n);
    s.u.assign(u, u + n);
    s.h.assign(h, h + n);
    s.c.assign(n, R(0));
    s.itype.assign(itype, itype + n);
    if (dvdt) s.dvdt.assign(dvdt, dvdt + n * dim);
    else s.dvdt.assign(n * dim, R(0));
    if (dudt) s.dudt.assign(dudt, dudt + n);
    else s.dudt.assign(n, R(0));
    return s;
}

template <class R>
void store_state(const ao::State<R>& s, R* x, R* v, R* rho, R* p, R* u, R* dvdt, R* dudt) {
    std::memcpy(x, s.x.data(), sizeof(R) * s.n * s.dim);
    std::memcpy(v, s.v.data(), sizeof(R) * s.n * s.dim);
    std::memcpy(rho, s.rho.data(), sizeof(R) * s.n);
    std::memcpy(p, s.p.data(), sizeof(R) * s.n);
    std::memcpy(u, s.u.data(), sizeof(R) * s.n);
    if (dvdt) std::memcpy(dvdt, s.dvdt.data(), sizeof(R) * s.n * s.dim);
    if (dudt) std::memcpy(dudt, s.dudt.data(), sizeof(R) * s.n);
}

template <class Rc>
int64_t link_list_impl(int64_t n, int dim, const Rc* x, const Rc* h, const int* periodic,
                       const double* lo, const double* hi, int32_t* pi, int32_t* pj, int64_t cap,
                       int64_t* cell_ids, double* grid_out, int use_direct) {
    int per0[3] = {0, 0, 0};
    const int* per = periodic ? periodic : per0;
    double lo0[3] = {0, 0, 0}, hi0[3] = {0, 0, 0};
    ao::PairList pl;
    std::vector<int64_t> cid;
    ao::Grid<Rc> g;
    try {
        g = ao::link_list<Rc>(n, dim, x, h, per, lo ? lo : lo0, hi ? hi : hi0, pl, &cid);
        if (use_direct) ao::direct_find<Rc>(n, dim, x, h, per, g, pl);
    } catch (const std::exception&) {
        return -1;
    }
    if (cell_ids) std::memcpy(cell_ids, cid.data(), sizeof(int64_t) * n);
    if (grid_out) {  // o[3], size[3], n[3], ncells
        for (int d = 0; d < 3; ++d) {
            grid_out[d] = (double)g.o[d];
            grid_out[3 + d] = (double)g.size[d];
            grid_out[6 + d] = (double)g.n[d];
        }
        grid_out[9] = (double)g.ncells;
    }
    int64_t np = (int64_t)pl.pi.size();
    if (pi && pj && np <= cap) {
        std::memcpy(pi, pl.pi.data(), sizeof(int32_t) * np);
        std::memcpy(pj, pl.pj.data(), sizeof(int32_t) * np);
    }
    return np;
}

}  // namespace

extern "C" {

// Neighbour pairs (i < j) by link_list (use_direct = 0) or direct_find (1), in
// FP64 or FP32 coordinates. Returns the pair count (pairs copied only when it
// fits in cap), -1 on error. grid_out: o[3], size[3], n[3], ncells.
int64_t ao_link_list_f64(int64_t n, int dim, const double* x, const double* h, const int* periodic,
                         const double* lo, const double* hi, int32_t* pi, int32_t* pj, int64_t cap,
                         int64_t* cell_ids, double* grid_out, int use_direct) {
    return link_list_impl<double>(n, dim, x, h, periodic, lo, hi, pi, pj, cap, cell_ids, grid_out,
                                  use_direct);
}
int64_t ao_link_list_f32(int64_t n, int dim, const float* x, const float* h, const int* periodic,
                         const double* lo, const double* hi, int32_t* pi, int32_t* pj, int64_t cap,
                         int64_t* cell_ids, double* grid_out, int use_direct) {
    return link_list_impl<float>(n, dim, x, h, periodic, lo, hi, pi, pj, cap, cell_ids, grid_out,
                                 use_direct);
}

// Wendland W and dW/dr at (r, h) (armando.cu:137-191).
void ao_kernel_f64(int dim, int legacy3d, int64_t n, const double* r, const double* h, double* w,
                   double* dwdr) {
    for (int64_t i = 0; i < n; ++i) {
        w[i] = ao::kernel_w(r[i], h[i], dim, legacy3d);
        dwdr[i] = ao::kernel_dwdr(r[i], h[i], dim, legacy3d);
    }
}

// Tait pressure (eos.f90:255-283) of every rho, without the pmin clamp when
// clamp == 0.
void ao_tait_f64(int64_t n, const double* rho, double rho0, double c0, double pmin, int clamp,
                 double* p) {
    ao::Params<double> P;
    P.rho0 = rho0;
    P.c0 = c0;
    P.pmin = clamp ? pmin : -INFINITY;
    for (int64_t i = 0; i < n; ++i) {
        double r = rho[i];
        ao::eos_tait(r, p[i], P);
    }
}

// int_force (+ art_visc when enabled) rates with the given rho and p (no
// density summation, no EOS): dvdt[n*dim], dudt[n]. Pairs from link_list.
int ao_forces_f64(const armando_params* prm, int64_t n, const double* x, const double* v,
                  const double* m, const double* rho, const double* p, const double* u,
                  const double* h, const int* itype, double* dvdt, double* dudt) {
    ao::Params<double> P = to_params<double>(prm);
    ao::State<double> s = load_state<double>(P.dim, n, x, v, m, rho, p, u, h, itype, nullptr, nullptr);
    for (int64_t i = 0; i < n; ++i) s.c[i] = P.c0;
    ao::PairList pl;
    ao::Grid<double> g;
    try {
        g = ao::neighbour_search<double, double>(s, P, pl);
    } catch (const std::exception&) {
        return 1;
    }
    std::vector<double> dv, du, tds, avdv, avdu, rpdv;
    ao::PairList same, other;
    const ao::PairList& body = ao::split_by_itype(s, P, pl, same, other);
    ao::int_force(s, g, P, body, dv, du, tds);
    if (P.visc_artificial) {
        ao::art_visc(s, g, P, body, avdv, avdu);
        for (size_t k = 0; k < dv.size(); ++k) dv[k] += avdv[k];
        for (size_t k = 0; k < du.size(); ++k) du[k] += avdu[k];
    }
    if (ao::repulsive_walls(P)) {
        ao::wall_repulsion(s, g, P, other, rpdv);
        for (size_t k = 0; k < dv.size(); ++k) dv[k] += rpdv[k];
    }
    std::memcpy(dvdt, dv.data(), sizeof(double) * n * P.dim);
    std::memcpy(dudt, du.data(), sizeof(double) * n);
    return 0;
}

// con_density (density.f:161-218): drho/dt[n] of the fluid particles for the
// given velocities. Pairs from link_list.
int ao_con_density_f64(const armando_params* prm, int64_t n, const double* x, const double* v,
                       const double* m, const double* rho, const double* h, const int* itype,
                       double* drho) {
    ao::Params<double> P = to_params<double>(prm);
    std::vector<double> zero(n, 0.0);
    ao::State<double> s = load_state<double>(P.dim, n, x, v, m, rho, zero.data(), zero.data(), h,
                                             itype, nullptr, nullptr);
    ao::PairList pl;
    ao::Grid<double> g;
    try {
        g = ao::neighbour_search<double, double>(s, P, pl);
    } catch (const std::exception&) {
        return 1;
    }
    std::vector<double> dr;
    ao::con_density(s, g, P, pl, dr);
    std::memcpy(drho, dr.data(), sizeof(double) * n);
    return 0;
}

// One leapfrog iteration `its` (time_integration.f:131-218), pair-loop form.
// nbr_fp32 = 1 runs the neighbour search in FP32 coordinates (GPU mirror).
// extra (optional, n*2): per particle tdsdt, divv of the step.
int ao_step_f64(const armando_params* prm, int64_t n, int its, double dt, double* x, double* v,
                const double* m, double* rho, double* p, double* u, double* h,
                const int* itype, double* dvdt, double* dudt, double* drho, int nbr_fp32,
                double* extra) {
    ao::Params<double> P = to_params<double>(prm);
    ao::State<double> s = load_state<double>(P.dim, n, x, v, m, rho, p, u, h, itype, dvdt, dudt);
    if (drho) s.drho.assign(drho, drho + n);
    ao::Rates<double> r;
    try {
        if (nbr_fp32) ao::leapfrog_step<double, float>(s, P, its, dt, &r);
        else ao::leapfrog_step<double, double>(s, P, its, dt, &r);
    } catch (const std::exception&) {
        return 1;
    }
    store_state(s, x, v, rho, p, u, dvdt, dudt);
    std::memcpy(h, s.h.data(), sizeof(double) * n);  // evolved with params->sle
    if (drho && !s.drho.empty()) std::memcpy(drho, s.drho.data(), sizeof(double) * n);
    if (extra) {
        for (int64_t i = 0; i < n; ++i) {
            extra[2 * i] = r.tdsdt.empty() ? 0.0 : r.tdsdt[i];
            extra[2 * i + 1] = r.divv.empty() ? 0.0 : r.divv[i];
        }
    }
    return 0;
}

// Same iteration evaluated entirely in FP32 (the error floor of plain FP32
// arithmetic on this algorithm).
int ao_step_f32(const armando_params* prm, int64_t n, int its, double dt, float* x, float* v,
                const float* m, float* rho, float* p, float* u, const float* h, const int* itype,
                float* dvdt, float* dudt) {
    ao::Params<float> P = to_params<float>(prm);
    ao::State<float> s = load_state<float>(P.dim, n, x, v, m, rho, p, u, h, itype, dvdt, dudt);
    try {
        ao::leapfrog_step<float, float>(s, P, its, dt);
    } catch (const std::exception&) {
        return 1;
    }
    store_state(s, x, v, rho, p, u, dvdt, dudt);
    return 0;
}

// `steps` iterations its0.. of the threaded gather form (FP64) on nthreads
// host threads. The CPU baseline.
int ao_integrate_gather_f64(const armando_params* prm, int64_t n, int its0, int steps, double dt,
                            double* x, double* v, const double* m, double* rho, double* p,
                            double* u, const double* h, const int* itype, double* dvdt,
                            double* dudt, int nthreads) {
    ao::Params<double> P = to_params<double>(prm);
    // the gather form restates wall_model 0 and summation density only
    if (P.wall_model != 0 || P.density_form != 0 || P.average_velocity || P.sle) return 2;
    ao::State<double> s = load_state<double>(P.dim, n, x, v, m, rho, p, u, h, itype, dvdt, dudt);
    try {
        for (int k = 0; k < steps; ++k) ao::leapfrog_step_gather(s, P, its0 + k, dt, nthreads);
    } catch (const std::exception&) {
        return 1;
    }
    store_state(s, x, v, rho, p, u, dvdt, dudt);
    return 0;
}

// Loss specification shared with the Python wrapper (see armando_oracle_tangent.hpp).
struct ao_loss_c {
    double w_ke, w_p, w_u, c[3], radius, w_ref;
};

static ao::LossSpec to_loss(const ao_loss_c* l) {
    ao::LossSpec L;
    L.w_ke = l->w_ke;
    L.w_p = l->w_p;
    L.w_u = l->w_u;
    for (int d = 0; d < 3; ++d) L.c[d] = l->c[d];
    L.radius = l->radius;
    L.w_ref = l->w_ref;
    return L;
}

// FP64 loss after `steps` iterations its0.. (pair-loop oracle). NaN on error.
double ao_loss_f64(const armando_params* prm, int64_t n, int its0, int steps, double dt,
                   const double* x, const double* v, const double* m, const double* rho,
                   const double* p, const double* u, const double* h, const int* itype,
                   const double* dvdt, const double* dudt, const ao_loss_c* l) {
    ao::Params<double> P = to_params<double>(prm);
    ao::State<double> s = load_state<double>(P.dim, n, x, v, m, rho, p, u, h, itype, dvdt, dudt);
    try {
        return ao::run_loss<double>(s, P, its0, steps, dt, to_loss(l));
    } catch (const std::exception&) {
        return NAN;
    }
}

// FP64 tangent-linear: out[0] = L, out[1] = dL along the seed (dparam[4] =
// d alpha, d beta, d c0, d q0; dx0, dv0 [n*dim] and du0 [n], each nullable).
int ao_tangent_f64(const armando_params* prm, int64_t n, int its0, int steps, double dt,
                   const double* x, const double* v, const double* m, const double* rho,
                   const double* p, const double* u, const double* h, const int* itype,
                   const double* dvdt, const double* dudt, const ao_loss_c* l,
                   const double* dparam, const double* dx0, const double* dv0,
                   const double* du0, double* out) {
    using ao::Dual;
    ao::Params<Dual> P = to_params<Dual>(prm);
    if (dparam) {
        P.av_alpha.d = dparam[0];
        P.av_beta.d = dparam[1];
        P.c0.d = dparam[2];
        P.heat_q0.d = dparam[3];
    }
    const int dim = P.dim;
    ao::State<Dual> s;
    s.n = n;
    s.dim = dim;
    auto lift = [](const double* a, int64_t k, const double* da) {
        std::vector<Dual> r(k);
        for (int64_t i = 0; i < k; ++i) r[i] = Dual(a[i], da ? da[i] : 0.0);
        return r;
    };
    s.x = lift(x, n * dim, dx0);
    s.v = lift(v, n * dim, dv0);
    s.m = lift(m, n, nullptr);
    s.rho = lift(rho, n, nullptr);
    s.p = lift(p, n, nullptr);
    s.u = lift(u, n, du0);
    s.h = lift(h, n, nullptr);
    s.c.assign(n, Dual(0.0));
    s.itype.assign(itype, itype + n);
    s.dvdt = dvdt ? lift(dvdt, n * dim, nullptr) : std::vector<Dual>(n * dim, Dual(0.0));
    s.dudt = dudt ? lift(dudt, n, nullptr) : std::vector<Dual>(n, Dual(0.0));
    try {
        Dual L = ao::run_loss<Dual>(s, P, its0, steps, dt, to_loss(l));
        out[0] = L.v;
        out[1] = L.d;
    } catch (const std::exception&) {
        return 1;
    }
    return 0;
}

// Operation count of iteration `its` of the reference algorithm on this state
// (armando_oracle_flops.hpp): out[0] = the whole iteration, out[1] = its
// neighbour search (link_list) alone. The state is not modified.
int ao_flops_f64(const armando_params* prm, int64_t n, int its, double dt, const double* x,
                 const double* v, const double* m, const double* rho, const double* p,
                 const double* u, const double* h, const int* itype, const double* dvdt,
                 const double* dudt, double* out) {
    using ao::Flop;
    ao::Params<Flop> P = to_params<Flop>(prm);
    const int dim = P.dim;
    ao::State<Flop> s;
    s.n = n;
    s.dim = dim;
    auto lift = [](const double* a, int64_t k) {
        std::vector<Flop> r(k);
        for (int64_t i = 0; i < k; ++i) r[i] = Flop(a[i]);
        return r;
    };
    s.x = lift(x, n * dim);
    s.v = lift(v, n * dim);
    s.m = lift(m, n);
    s.rho = lift(rho, n);
    s.p = lift(p, n);
    s.u = lift(u, n);
    s.h = lift(h, n);
    s.c.assign(n, Flop(0.0));
    s.itype.assign(itype, itype + n);
    s.dvdt = dvdt ? lift(dvdt, n * dim) : std::vector<Flop>(n * dim, Flop(0.0));
    s.dudt = dudt ? lift(dudt, n) : std::vector<Flop>(n, Flop(0.0));
    try {
        ao::PairList pl;
        Flop::count = 0;
        ao::neighbour_search<Flop, Flop>(s, P, pl);
        const double search = (double)Flop::count;
        Flop::count = 0;
        ao::leapfrog_step<Flop, Flop>(s, P, its, dt);
        out[0] = (double)Flop::count;
        out[1] = search;
    } catch (const std::exception&) {
        return 1;
    }
    return 0;
}

// Mirror ghosts (wall_model 3, ghost.f) of a state at its current positions,
// velocities as given (no predictor): returns the ghost count (-1 on error)
// and fills owner[ng], wall[ng], xg[ng*dim], vg[ng*dim] (capacity n each).
// fp32 = 1: candidates and the nearest wall in FP32 coordinates.
int64_t ao_ghosts_f64(const armando_params* prm, int64_t n, const double* x, const double* v,
                      const double* h, const int* itype, int fp32, int64_t* owner, int64_t* wall,
                      double* xg, double* vg) {
    ao::Params<double> P = to_params<double>(prm);
    const int dim = P.dim;
    std::vector<double> zero(n, 0.0);
    ao::State<double> s = load_state<double>(dim, n, x, v, zero.data(), zero.data(), zero.data(),
                                             zero.data(), h, itype, nullptr, nullptr);
    auto emit = [&](const auto& G) {
        const int64_t ng = (int64_t)G.owner.size();
        for (int64_t k = 0; k < ng; ++k) {
            owner[k] = G.owner[k];
            wall[k] = G.wall[k];
            for (int d = 0; d < dim; ++d) {
                xg[k * dim + d] = s.x[(n + k) * dim + d];
                vg[k * dim + d] = s.v[(n + k) * dim + d];
            }
        }
        return ng;
    };
    try {
        if (fp32) {
            ao::Ghosts<double, float> G;
            ao::ghost_particles(s, P, G);
            return emit(G);
        }
        ao::Ghosts<double, double> G;
        ao::ghost_particles(s, P, G);
        return emit(G);
    } catch (const std::exception&) {
        return -1;
    }
}

// Setup of the GPU-C schemes: variant, kernel switch, gravity, the material
// table (nmat entries; NULL: Tait with rho0, c0 for every |itype|) and the
// load and fix zones.
static ao::GpucSetup<double> gpuc_setup(const armando_params* prm, int32_t nmat, const armando_material* table,
                                        int32_t n_load, const armando_load_zone* loads, int32_t n_fix,
                                        const armando_fix_zone* fixes) {
    ao::GpucSetup<double> G;
    G.variant = prm->scheme;
    G.legacy3d = prm->kernel_3d_legacy;
    for (int d = 0; d < 3; ++d) G.gravity[d] = prm->gravity[d];
    G.mat.resize(table ? nmat : ARMANDO_MAX_MATERIALS);
    for (size_t k = 0; k < G.mat.size(); ++k) {
        if (table) {
            G.mat[k].type = table[k].eos;
            for (int q = 0; q < 10; ++q) G.mat[k].prop[q] = table[k].prop[q];
        } else {
            G.mat[k].type = ao::EOS_TAIT;
            G.mat[k].prop[0] = prm->rho0;
            G.mat[k].prop[1] = prm->c0;
        }
    }
    for (int k = 0; k < n_load; ++k) {
        ao::GpucLoad Z;
        for (int d = 0; d < 3; ++d) {
            Z.lo[d] = loads[k].lo[d];
            Z.hi[d] = loads[k].hi[d];
            Z.g[d] = loads[k].accel[d];
        }
        Z.w = loads[k].w;
        G.loads.push_back(Z);
    }
    for (int k = 0; k < n_fix; ++k) {
        ao::GpucFix Z;
        for (int d = 0; d < 3; ++d) {
            Z.lo[d] = fixes[k].lo[d];
            Z.hi[d] = fixes[k].hi[d];
            Z.v[d] = fixes[k].vel[d];
        }
        Z.tau = fixes[k].tau;
        G.fixes.push_back(Z);
    }
    return G;
}

// GPU-C scheme (params->scheme 1 or 2): `steps` TVD-RK3 steps in place, with
// the setup of gpuc_setup. fp32 = 1: neighbour lists in FP32 coordinates (the
// library's). dvdt, dudt (nullable): rates of the last stage.
int ao_gpuc_step_f64(const armando_params* prm, int32_t nmat, const armando_material* table,
                     int32_t n_load, const armando_load_zone* loads, int32_t n_fix,
                     const armando_fix_zone* fixes, int64_t n, int steps, double dt, double* x,
                     double* v, const double* m, double* rho, double* p, double* u, const double* h,
                     const int* itype, double* dvdt, double* dudt, int fp32) {
    if (prm->scheme != 1 && prm->scheme != 2) return 2;
    ao::Params<double> P = to_params<double>(prm);
    const ao::GpucSetup<double> G = gpuc_setup(prm, nmat, table, n_load, loads, n_fix, fixes);
    ao::State<double> s = load_state<double>(P.dim, n, x, v, m, rho, p, u, h, itype, nullptr, nullptr);
    std::vector<double> dv, du;
    try {
        for (int k = 0; k < steps; ++k) {
            if (fp32) ao::gpuc_rk3_step<double, float>(s, G, dt, &dv, &du);
            else ao::gpuc_rk3_step<double, double>(s, G, dt, &dv, &du);
        }
    } catch (const std::exception&) {
        return 1;
    }
    store_state<double>(s, x, v, rho, p, u, nullptr, nullptr);
    if (dvdt && !dv.empty()) std::memcpy(dvdt, dv.data(), sizeof(double) * n * P.dim);
    if (dudt && !du.empty()) std::memcpy(dudt, du.data(), sizeof(double) * n);
    return 0;
}

// Pair rates of the GPU-C scheme at one state, as the first stage of a step
// evaluates them (the list of gpuc_list, gpuc_rates): drho/dt, dv/dt (loads
// included) and de/dt, with p as given (not from the EOS) and c from the
// material's EOS. fp32 = 1: the list in FP32 coordinates.
int ao_gpuc_rates_f64(const armando_params* prm, int32_t nmat, const armando_material* table,
                      int64_t n, const double* x, const double* v, const double* m,
                      const double* rho, const double* p, const double* u, const double* h,
                      const int* itype, double* drho, double* dvdt, double* dudt, int fp32) {
    if (prm->scheme != 1 && prm->scheme != 2) return 2;
    ao::Params<double> P = to_params<double>(prm);
    const ao::GpucSetup<double> G = gpuc_setup(prm, nmat, table, 0, nullptr, 0, nullptr);
    ao::State<double> s = load_state<double>(P.dim, n, x, v, m, rho, p, u, h, itype, nullptr, nullptr);
    const int dim = P.dim;
    std::vector<float> xf(n * dim), hf(n);
    for (int64_t i = 0; i < n * dim; ++i) xf[i] = (float)x[i];
    for (int64_t i = 0; i < n; ++i) hf[i] = (float)h[i];
    const std::vector<std::vector<int>> list =
        fp32 ? ao::gpuc_list<float>(n, dim, xf.data(), hf.data()) : ao::gpuc_list<double>(n, dim, x, h);
    for (int64_t i = 0; i < n; ++i)
        s.c[i] = ao::gpuc_sound(ao::gpuc_material(G.mat, s.itype[i]), s.rho[i], s.u[i]);
    std::vector<double> dv, dr, du;
    ao::gpuc_rates(s, list, G, dv, dr, du);
    std::memcpy(drho, dr.data(), sizeof(double) * n);
    std::memcpy(dvdt, dv.data(), sizeof(double) * n * dim);
    std::memcpy(dudt, du.data(), sizeof(double) * n);
    return 0;
}

// GPU-C scheme with open boundaries: `steps` steps on *n particles (in/out);
// arrays hold `capacity` entries (x, v, dvdt: capacity*dim). Returns 0, 1 on a
// failed step, 3 when the particles outgrow the capacity.
int ao_gpuc_open_f64(const armando_params* prm, int32_t nmat, const armando_material* table,
                     int32_t n_load, const armando_load_zone* loads, int32_t n_fix,
                     const armando_fix_zone* fixes, int32_t n_in, const armando_inlet* inlets,
                     int32_t n_out, const armando_outlet* outlets, const float* lo, const float* hi,
                     int64_t capacity, int64_t* n, int steps, double dt, double* x, double* v,
                     double* m, double* rho, double* p, double* u, double* h, int* itype,
                     double* dvdt, double* dudt, int fp32) {
    if (prm->scheme != 1 && prm->scheme != 2) return 2;
    const ao::GpucSetup<double> G = gpuc_setup(prm, nmat, table, n_load, loads, n_fix, fixes);
    ao::GpucOpen O;
    for (int k = 0; k < n_in; ++k) {
        ao::GpucInlet I;
        for (int d = 0; d < 3; ++d) {
            I.o[d] = inlets[k].origin[d];
            I.n[d] = inlets[k].normal[d];
        }
        I.R = inlets[k].radius;
        I.itype = inlets[k].itype;
        I.mass = inlets[k].mass;
        I.h = inlets[k].hsml;
        I.speed = inlets[k].speed;
        I.rho = inlets[k].rho;
        I.u = inlets[k].u;
        O.in.push_back(I);
    }
    for (int k = 0; k < n_out; ++k) {
        ao::GpucOutlet Q;
        for (int d = 0; d < 3; ++d) {
            Q.o[d] = outlets[k].origin[d];
            Q.n[d] = outlets[k].normal[d];
        }
        Q.R = outlets[k].radius;
        O.out.push_back(Q);
    }
    for (int d = 0; d < 3; ++d) {
        O.lo[d] = lo[d];
        O.hi[d] = hi[d];
    }
    const int dim = prm->dim;
    ao::State<double> s = load_state<double>(dim, *n, x, v, m, rho, p, u, h, itype, nullptr, nullptr);
    std::vector<double> dv, du;
    try {
        for (int k = 0; k < steps; ++k) {
            if (fp32) ao::gpuc_rk3_step<double, float>(s, G, dt, &dv, &du, &O);
            else ao::gpuc_rk3_step<double, double>(s, G, dt, &dv, &du, &O);
            if (s.n > capacity) return 3;
        }
    } catch (const std::exception&) {
        return 1;
    }
    *n = s.n;
    store_state<double>(s, x, v, rho, p, u, nullptr, nullptr);
    std::memcpy(m, s.m.data(), sizeof(double) * s.n);
    std::memcpy(h, s.h.data(), sizeof(double) * s.n);
    std::memcpy(itype, s.itype.data(), sizeof(int) * s.n);
    if (!dv.empty()) std::memcpy(dvdt, dv.data(), sizeof(double) * s.n * dim);
    if (!du.empty()) std::memcpy(dudt, du.data(), sizeof(double) * s.n);
    return 0;
}

// EOS of the GPU-C schemes for one material: rho (clamped where the type
// clamps), p and c for n states (rho_in, u).
void ao_gpuc_eos_f64(const armando_material* mat, int64_t n, const double* rho_in, const double* u,
                     double* rho, double* p, double* c) {
    ao::GpucMaterial M;
    M.type = mat->eos;
    for (int q = 0; q < 10; ++q) M.prop[q] = mat->prop[q];
    for (int64_t i = 0; i < n; ++i) {
        double r = rho_in[i], pp = 0.0, cc = 0.0;
        ao::gpuc_eos(M, r, u[i], pp, cc);
        rho[i] = r;
        p[i] = pp;
        c[i] = cc;
    }
}

int ao_hardware_threads(void) {
    unsigned t = std::thread::hardware_concurrency();
    return t ? (int)t : 1;
}

}  // extern "C"
