// armando_oracle_gather.hpp -- multithreaded FP64 form of the oracle step, used
// ONLY as the timed CPU baseline and as a cross-check; it is test
// infrastructure, not part of the product.
//
// Same mathematics as armando_oracle.hpp (CERNsource time_integration.f +
// single_step.f and the routines they call), rearranged from the reference's
// i<j pair loops with scatter to both partners into per-particle gathers over
// the 3^dim link_list cells, so host threads never write the same particle.
// Results agree with the pair-loop form to FP64 rounding (summation order only).
#pragma once
#include "armando_oracle.hpp"

namespace ao {

template <class F>
void parallel_for(int64_t n, int nthreads, F&& f) {
    if (nthreads <= 1 || n < 4096) {
        f(int64_t(0), n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

struct CellIndex {
    Grid<double> g;
    std::vector<int64_t> start;  // ncells + 1
    std::vector<int> part;       // particles sorted by cell (stable)
    std::vector<int64_t> cid;
};

inline void build_cells(int64_t n, int dim, const double* x, const double* h, const int* periodic,
                        const double* lo, const double* hi, CellIndex& ci) {
    ci.g = make_grid<double>(n, dim, x, h, periodic, lo, hi);
    ci.cid.resize(n);
    ci.start.assign(ci.g.ncells + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        ci.cid[i] = cell_id(x + i * dim, ci.g, dim);
        ci.start[ci.cid[i] + 1]++;
    }
    for (int64_t c = 0; c < ci.g.ncells; ++c) ci.start[c + 1] += ci.start[c];
    std::vector<int64_t> fill(ci.start.begin(), ci.start.end() - 1);
    ci.part.resize(n);
    for (int64_t i = 0; i < n; ++i) ci.part[fill[ci.cid[i]]++] = (int)i;
}

// Calls f(j) for every neighbour j != i of particle i (link_list pair test).
template <class F>
inline void for_neighbours(const CellIndex& ci, int dim, const double* x, const double* h,
                           const int* periodic, int64_t i, F&& f) {
    const Grid<double>& g = ci.g;
    int ijk[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) ijk[d] = cell_coord(x[i * dim + d], g, d);
    int lo3[3] = {0, 0, 0}, hi3[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
        if (periodic[d]) {
            lo3[d] = ijk[d] - 1;
            hi3[d] = ijk[d] + 1;
        } else {
            lo3[d] = std::max(ijk[d] - 1, 0);
            hi3[d] = std::min(ijk[d] + 1, g.n[d] - 1);
        }
    }
    for (int kg = lo3[2]; kg <= hi3[2]; ++kg)
        for (int jg = lo3[1]; jg <= hi3[1]; ++jg)
            for (int ig = lo3[0]; ig <= hi3[0]; ++ig) {
                int cc[3] = {ig, jg, kg};
                int64_t c = 0;
                for (int d = dim - 1; d >= 0; --d) {
                    int v = cc[d];
                    if (periodic[d]) v = (v + g.n[d]) % g.n[d];
                    c = c * g.n[d] + v;
                }
                for (int64_t k = ci.start[c]; k < ci.start[c + 1]; ++k) {
                    int j = ci.part[k];
                    if (j == i) continue;
                    if (pair_test(x + i * dim, x + (int64_t)j * dim, h[i], h[j], dim, g, periodic))
                        f(j);
                }
            }
}

// One leapfrog iteration, gather form, nthreads host threads.
inline void leapfrog_step_gather(State<double>& s, const Params<double>& P, int its, double dt,
                                 int nthreads) {
    const int dim = s.dim;
    const int64_t n = s.n;
    const double hdt = dt / 2.0;
    std::vector<double> u_min = s.u, v_min = s.v;
    if (its != 1) {
        parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; ++i) {
                if (!s.fluid(i)) continue;
                s.u[i] = s.u[i] + hdt * s.dudt[i];
                if (s.u[i] < 0) s.u[i] = 0;
                for (int d = 0; d < dim; ++d) s.v[i * dim + d] += hdt * s.dvdt[i * dim + d];
            }
        });
    }
    CellIndex ci;
    build_cells(n, dim, s.x.data(), s.h.data(), P.periodic, P.period_lo, P.period_hi, ci);
    const double* x = s.x.data();
    const double* h = s.h.data();
    auto geom = [&](int64_t i, int j, PairGeom<double, double>& pg) {
        pair_geom(s, ci.g, P, (int)i, j, pg);
    };
    // Density + EOS (density.f, eos.f90).
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        PairGeom<double, double> pg;
        for (int64_t i = b; i < e; ++i) {
            s.c[i] = P.c0;
            if (!s.fluid(i)) continue;
            double rho = kernel_w(0.0, s.h[i], dim, P.kernel_3d_legacy) * s.m[i];
            for_neighbours(ci, dim, x, h, P.periodic, i, [&](int j) {
                geom(i, j, pg);
                rho += s.m[j] * pg.w;
            });
            s.rho[i] = rho;
            eos_tait(s.rho[i], s.p[i], P);
        }
    });
    // Shear tensor (visc) and div v (art_heat), every particle.
    std::vector<double> T, divv;
    if (P.visc) T.assign(n * 6, 0.0);
    if (P.heat_artificial) divv.assign(n, 0.0);
    if (P.visc || P.heat_artificial) {
        parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
            PairGeom<double, double> pg;
            for (int64_t i = b; i < e; ++i) {
                double t[6] = {0, 0, 0, 0, 0, 0}, dvs = 0;
                for_neighbours(ci, dim, x, h, P.periodic, i, [&](int j) {
                    geom(i, j, pg);
                    double dv[3] = {0, 0, 0};
                    for (int d = 0; d < dim; ++d) dv[d] = s.v[(int64_t)j * dim + d] - s.v[i * dim + d];
                    const double* w = pg.dwdx;
                    if (P.visc) {
                        double hh[6] = {0, 0, 0, 0, 0, 0};
                        if (dim == 2) {
                            hh[0] = 2 * dv[0] * w[0] - dv[1] * w[1];
                            hh[1] = 2 * dv[1] * w[1] - dv[0] * w[0];
                            hh[3] = dv[0] * w[1] + dv[1] * w[0];
                        } else {
                            hh[0] = 2 * dv[0] * w[0] - dv[1] * w[1] - dv[2] * w[2];
                            hh[1] = 2 * dv[1] * w[1] - dv[0] * w[0] - dv[2] * w[2];
                            hh[2] = 2 * dv[2] * w[2] - dv[0] * w[0] - dv[1] * w[1];
                            hh[5] = dv[1] * w[2] + dv[2] * w[1];
                            hh[4] = dv[0] * w[2] + dv[2] * w[0];
                            hh[3] = dv[0] * w[1] + dv[1] * w[0];
                        }
                        hh[0] *= 2.0 / 3.0;
                        hh[1] *= 2.0 / 3.0;
                        hh[2] *= 2.0 / 3.0;
                        for (int a = 0; a < 6; ++a) t[a] += s.m[j] * hh[a] / s.rho[j];
                    }
                    if (P.heat_artificial) {
                        double vd = 0;
                        for (int d = 0; d < dim; ++d) vd += dv[d] * w[d];
                        dvs += s.m[j] * vd;
                    }
                });
                if (P.visc)
                    for (int a = 0; a < 6; ++a) T[i * 6 + a] = t[a];
                if (P.heat_artificial) divv[i] = dvs / s.rho[i];
            }
        });
    }
    // Forces, heat and rates (internal_force.f, art_visc.f, art_heat.f).
    std::vector<double> dv(n * dim, 0.0), du(n, 0.0);
    const bool heat_on = P.heat_external && (double(its) * dt <= P.heat_t_end);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        PairGeom<double, double> pg;
        static const int tidx[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
        for (int64_t i = b; i < e; ++i) {
            if (!s.fluid(i)) continue;
            double a[3] = {0, 0, 0}, he_sum = 0, av_du = 0, ah_du = 0;
            const double ri = s.rho[i], ri2 = ri * ri, Pi = s.p[i] / ri2;
            double psi_i = 0;
            if (P.heat_artificial)
                psi_i = P.ah_g1 * s.h[i] * s.c[i] +
                        P.ah_g2 * s.h[i] * s.h[i] * (std::fabs(divv[i]) - divv[i]);
            for_neighbours(ci, dim, x, h, P.periodic, i, [&](int j) {
                geom(i, j, pg);
                const double* w = pg.dwdx;
                const double rj = s.rho[j], rj2 = rj * rj;
                double vji[3] = {0, 0, 0};
                for (int d = 0; d < dim; ++d) vji[d] = s.v[(int64_t)j * dim + d] - s.v[i * dim + d];
                double he = 0;
                for (int d = 0; d < dim; ++d) {
                    double hv;
                    if (P.pa_sph == 0) {
                        hv = -(s.p[i] + s.p[j]) * w[d];
                        he += vji[d] * hv;
                        if (P.visc)
                            for (int bb = 0; bb < dim; ++bb)
                                hv += (P.eta * T[i * 6 + tidx[d][bb]] +
                                       P.eta * T[(int64_t)j * 6 + tidx[d][bb]]) * w[bb];
                        hv /= ri * rj;
                    } else {
                        hv = -(Pi + s.p[j] / rj2) * w[d];
                        he += vji[d] * hv;
                        if (P.visc)
                            for (int bb = 0; bb < dim; ++bb)
                                hv += (P.eta * T[i * 6 + tidx[d][bb]] / ri2 +
                                       P.eta * T[(int64_t)j * 6 + tidx[d][bb]] / rj2) * w[bb];
                    }
                    a[d] += s.m[j] * hv;
                }
                if (P.pa_sph == 0) he /= ri * rj;
                he_sum += s.m[j] * he;
                if (P.visc_artificial) {
                    double vr = 0, vdw = 0;
                    for (int d = 0; d < dim; ++d) {
                        vr += -vji[d] * pg.dx[d];
                        vdw += -vji[d] * w[d];
                    }
                    if (vr < 0) {
                        double hh = pg.mh * P.av_eta;
                        double phi = pg.mh * vr / (pg.r2 + hh * hh);
                        double mc = 0.5 * (s.c[i] + s.c[j]);
                        double mrho = 0.5 * (ri + rj);
                        double piv = (P.av_beta * phi - P.av_alpha * mc) * phi / mrho;
                        for (int d = 0; d < dim; ++d) a[d] -= s.m[j] * piv * w[d];
                        av_du += 0.5 * s.m[j] * piv * vdw;
                    }
                }
                if (P.heat_artificial) {
                    double mrho = 0.5 * (ri + rj);
                    double rdw = 0;
                    for (int d = 0; d < dim; ++d) rdw += pg.dx[d] * w[d];
                    double psi_j = P.ah_g1 * s.h[j] * s.c[j] +
                                   P.ah_g2 * s.h[j] * s.h[j] * (std::fabs(divv[j]) - divv[j]);
                    double hh = pg.mh * P.ah_eta;
                    double psi = (2.0 * 0.5 * (psi_i + psi_j)) / (mrho * (pg.r2 + hh * hh)) * rdw;
                    ah_du += s.m[j] * psi * (s.u[i] - s.u[j]);
                }
            });
            double tds = 0;
            if (P.visc) {
                const double* t = &T[i * 6];
                double q = (dim == 2) ? t[0] * t[0] + t[1] * t[1] + 2 * t[3] * t[3]
                                      : t[0] * t[0] + t[1] * t[1] + t[2] * t[2] + 2 * t[5] * t[5] +
                                            2 * t[4] * t[4] + 2 * t[3] * t[3];
                tds = 0.5 * P.eta / ri * q;
            }
            double dui = tds + 0.5 * he_sum + av_du + ah_du;
            if (heat_on) {
                double d2 = 0;
                for (int d = 0; d < dim; ++d) {
                    double ee = s.x[i * dim + d] - P.heat_center[d];
                    d2 += ee * ee;
                }
                dui += P.heat_q0 * std::exp(-d2 / (2 * P.heat_sigma * P.heat_sigma)) / ri;
            }
            for (int d = 0; d < dim; ++d) dv[i * dim + d] = a[d] + P.gravity[d];
            du[i] = dui;
        }
    });
    // Corrector (time_integration.f:186-218).
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            if (!s.fluid(i)) continue;
            if (its != 1) {
                s.u[i] = u_min[i] + dt * du[i];
                if (s.u[i] < 0) s.u[i] = 0;
                for (int d = 0; d < dim; ++d) {
                    s.v[i * dim + d] = v_min[i * dim + d] + dt * dv[i * dim + d];
                    s.x[i * dim + d] += dt * s.v[i * dim + d];
                }
            } else {
                s.u[i] += hdt * du[i];
                if (s.u[i] < 0) s.u[i] = 0;
                for (int d = 0; d < dim; ++d) {
                    s.v[i * dim + d] += hdt * dv[i * dim + d];
                    s.x[i * dim + d] += dt * s.v[i * dim + d];
                }
            }
            wrap_periodic(s, P, i);
        }
    });
    s.dvdt.swap(dv);
    s.dudt.swap(du);
}

}  // namespace ao
