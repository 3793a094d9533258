// armando_oracle.hpp -- CPU restatement of Armando's weakly-compressible SPH
// step, used ONLY as the checker of the GPU library (tests, smoke check and the
// CPU baseline leg of the benchmark). Nothing in the product links or calls it.
//
// It restates, in the reference's pair-loop form (i < j pairs, contributions
// scattered to both partners):
//   time_integration  CERNsource/time_integration.f:131-218 (leapfrog)
//   single_step       CERNsource/single_step.f:92-234
//   link_list         CERNsource/link_list.f:1-224 (scale_k = 2)
//   direct_find       CERNsource/direct_find.f:1-61
//   sum_density       CERNsource/density.f:1-62
//   int_force         CERNsource/internal_force.f:57-435 (pa_sph 0 and 1, visc)
//   art_visc          CERNsource/art_visc.f:55-101 (alpha, beta, eta as parameters)
//   art_heat          CERNsource/art_heat.f:42-97 (g1, g2, eta as parameters)
//   Tait EOS          FORTRANsource/eos.f90:255-283 (c = c0, pmin clamp)
//   Wendland kernel   ArmandoThrust/armando.cu:137-191 with the 2D constant of
//                     ArmandoThrust/acpu.c:162 and the C2 3D constant noted at
//                     acpu.c:159 (15/16pi of armando.cu:150 behind a switch)
//   external heat     du += q(x)/rho as CERNsource/fluka_heat.f:337-338, with
//                     the analytic Gaussian of Code/armando.cu:1058-1071
//   gravity           FORTRANsource/time_integration.f90:148-152
//
// Deliberate, documented departures from the Fortran text (each one removes
// reference undefined behaviour, none changes a defined result):
//   * T_ab and div(v) are zeroed for every particle each step. The Fortran zeroes
//     them only for 1..np (internal_force.f:58-71, art_heat.f:42-44) and
//     accumulates wall entries into stale storage.
//   * eta (dynamic viscosity) and c (= c0) are set for wall particles too; the
//     Fortran leaves them unset for j > np (single_step.f:120-186).
//   * pi is M_PI (acpu.c); CERN options.inc declares pi with a single-precision
//     literal.
// Scalar type R: double (oracle), float (FP32 mirror), or a dual / counting
// type. Coordinates used for the neighbour grid and the pair test have their
// own type Rc so the FP32 cell ids / neighbour sets of the GPU can be mirrored
// bit for bit (compile with -ffp-contract=off).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <thread>
#include <vector>

namespace ao {

constexpr double kPi = 3.14159265358979323846;

template <class R>
struct Params {
    int dim = 2, pa_sph = 1, visc = 0, visc_artificial = 0, heat_artificial = 0,
        heat_external = 0, kernel_3d_legacy = 0;
    int periodic[3] = {0, 0, 0};
    R rho0 = R(1000), c0 = R(1), pmin = R(-INFINITY), eta = R(0);
    R av_alpha = R(1), av_beta = R(1), av_eta = R(0.1);
    R ah_g1 = R(0.1), ah_g2 = R(1), ah_eta = R(0.1);
    R gravity[3] = {R(0), R(0), R(0)};
    R heat_q0 = R(0), heat_sigma = R(1), heat_center[3] = {R(0), R(0), R(0)};
    double heat_t_end = INFINITY;
    double period_lo[3] = {0, 0, 0}, period_hi[3] = {0, 0, 0};
    // Wall treatment: 0 virtual particles (every pair alike), 1 and 2 the GPU-C
    // pushes between different itype (1 push only, 2 push and every sum),
    // 3 virtual particles plus mirror ghosts (ghost_particles).
    int wall_model = 0;
    // single_step options: density 0 summation, 1 continuity, 2 normalised
    // summation; XSPH (av_vel.f); smoothing-length evolution (hsml.f).
    int density_form = 0, average_velocity = 0, sle = 0;
};

// Whether pairs of different itype push (wall_model 1 and 2).
template <class R>
inline bool repulsive_walls(const Params<R>& P) {
    return P.wall_model == 1 || P.wall_model == 2;
}

// ---------------------------------------------------------------------------
// Wendland C2 kernel, support 2h (armando.cu:137-191).
//   W(r,h)   = alpha (1 - q/2)^4 (1 + 2q),      q = r/h < 2
//   dW/dr    = alpha/h * 5/8 * q (q - 2)^3
//   dW/dx_d  = dW/dr * dx_d / r = alpha * 5/(8 h^2) * (q - 2)^3 * dx_d
// alpha_2D = 7/(4 pi h^2) (acpu.c:162); alpha_3D = 21/(16 pi h^3) (acpu.c:159),
// or 15/(16 pi h^3) with kernel_3d_legacy (armando.cu:150).
// ---------------------------------------------------------------------------
// Periodic box length, fixed as the FP32 difference of the FP32 bounds (the
// library computes it the same way).
template <class P>
inline double period_length(const P& prm, int d) {
    return (double)((float)prm.period_hi[d] - (float)prm.period_lo[d]);
}

template <class R>
inline R kernel_alpha(const R& h, int dim, int legacy3d) {
    if (dim == 2) return R(7.0) / (R(4.0) * R(kPi) * h * h);
    return R(legacy3d ? 15.0 : 21.0) / (R(16.0) * R(kPi) * h * h * h);
}

template <class R>
inline R kernel_w(const R& r, const R& h, int dim, int legacy3d) {
    R q = r / h;
    if (!(q < R(2))) return R(0);
    R t = R(1) - R(0.5) * q;
    t = t * t;
    t = t * t;
    return kernel_alpha(h, dim, legacy3d) * t * (R(1) + R(2) * q);
}

// Gradient with respect to x_i of W(|x_i - x_j|, h); dx = x_i - x_j.
template <class R>
inline void kernel_dwdx(const R* dx, const R& r, const R& h, int dim, int legacy3d,
                        R* dwdx) {
    R q = r / h;
    if (!(q < R(2))) {
        for (int d = 0; d < dim; ++d) dwdx[d] = R(0);
        return;
    }
    R t = q - R(2);
    R f = kernel_alpha(h, dim, legacy3d) * R(5.0 / 8.0) / (h * h) * t * t * t;
    for (int d = 0; d < dim; ++d) dwdx[d] = f * dx[d];
}

// dW/dr exactly as the reference writes it (used by the acpu.c pin tests).
template <class R>
inline R kernel_dwdr(const R& r, const R& h, int dim, int legacy3d) {
    R q = r / h;
    if (!(q < R(2))) return R(0);
    R t = q - R(2);
    return R(5.0 / 8.0) * q * t * t * t * kernel_alpha(h, dim, legacy3d) / h;
}

// ---------------------------------------------------------------------------
// Neighbour grid of link_list.f:39-88, in coordinate precision Rc.
// ---------------------------------------------------------------------------
template <class Rc>
struct Grid {
    Rc o[3] = {0, 0, 0};
    Rc size[3] = {1, 1, 1};
    Rc period[3] = {0, 0, 0};
    Rc half_period[3] = {0, 0, 0};
    int n[3] = {1, 1, 1};
    int64_t ncells = 1;
};

// Minimum-image difference on a periodic axis (absent from the reference,
// which only has commented-out wrap code, ArmandoList/armando2Dlist.cu:856-870).
template <class Rc>
inline Rc min_image(Rc dx, const Grid<Rc>& g, int d, const int* periodic) {
    if (periodic[d]) {
        if (dx > g.half_period[d]) dx = dx - g.period[d];
        else if (dx < -g.half_period[d]) dx = dx + g.period[d];
    }
    return dx;
}

// Grid over all particles: bbox expanded by the largest h, cell edge
// scale_k * mh with scale_k = 2 (link_list.f:29-57). A periodic axis uses the
// box [lo, hi) split into n = floor(L / (2 mh)) >= 3 equal cells.
template <class Rc>
Grid<Rc> make_grid(int64_t nt, int dim, const Rc* x, const Rc* h, const int* periodic,
                   const double* lo, const double* hi) {
    Grid<Rc> g;
    Rc gmin[3], gmax[3];
    for (int d = 0; d < 3; ++d) {
        gmin[d] = Rc(1.0e30);
        gmax[d] = Rc(-1.0e30);
    }
    Rc mh = Rc(0);
    for (int64_t i = 0; i < nt; ++i) {
        for (int d = 0; d < dim; ++d) {
            Rc xv = x[i * dim + d];
            if (xv < gmin[d]) gmin[d] = xv;
            if (xv > gmax[d]) gmax[d] = xv;
        }
        if (h[i] > mh) mh = h[i];
    }
    Rc cell = Rc(2) * mh;
    g.ncells = 1;
    for (int d = 0; d < dim; ++d) {
        if (periodic[d]) {
            Rc L = Rc((float)hi[d] - (float)lo[d]);
            int n = (int)(L / cell);
            if (n < 3) throw std::runtime_error("periodic axis shorter than 3 cells");
            g.o[d] = Rc(lo[d]);
            g.n[d] = n;
            g.size[d] = L / Rc(n);
            g.period[d] = L;
            g.half_period[d] = Rc(0.5) * L;
        } else {
            Rc lo_d = gmin[d] - mh;
            Rc hi_d = gmax[d] + mh;
            g.o[d] = lo_d;
            g.size[d] = cell;
            g.n[d] = (int)((hi_d - lo_d) / cell) + 1;
        }
        g.ncells *= g.n[d];
    }
    return g;
}

// Cell coordinate of x along d: int((x - grid_min)/(scale_k mh)) (link_list.f:76-78).
template <class Rc>
inline int cell_coord(Rc xv, const Grid<Rc>& g, int d) {
    int c = (int)((xv - g.o[d]) / g.size[d]);
    if (c < 0) c = 0;
    if (c > g.n[d] - 1) c = g.n[d] - 1;
    return c;
}

// Linear cell id g = n1*n2*k + n1*j + i (link_list.f:80-85, 0-based).
template <class Rc>
inline int64_t cell_id(const Rc* xi, const Grid<Rc>& g, int dim) {
    int64_t c = 0;
    for (int d = dim - 1; d >= 0; --d) c = c * g.n[d] + cell_coord(xi[d], g, d);
    return c;
}

// Pair test of link_list.f:154-159: dr^2 < (scale_k * (h_i + h_j)/2)^2, with
// dr^2 summed over axes in order; (2 * ((h_i+h_j)/2)) is exactly h_i + h_j.
template <class Rc>
inline bool pair_test(const Rc* xi, const Rc* xj, Rc hi, Rc hj, int dim, const Grid<Rc>& g,
                      const int* periodic) {
    Rc dr2 = Rc(0);
    for (int d = 0; d < dim; ++d) {
        Rc dx = min_image(Rc(xi[d] - xj[d]), g, d, periodic);
        Rc sq = dx * dx;
        dr2 = (d == 0) ? sq : Rc(dr2 + sq);
    }
    Rc s = hi + hj;
    return dr2 < Rc(s * s);
}

struct PairList {
    std::vector<int> pi, pj;
};

// link_list.f:1-224: counting sort of particles into cells, then for every i
// the 3^dim stencil, pairs (i, j) with j > i that pass the test.
template <class Rc>
Grid<Rc> link_list(int64_t nt, int dim, const Rc* x, const Rc* h, const int* periodic,
                   const double* lo, const double* hi, PairList& out,
                   std::vector<int64_t>* cell_of = nullptr) {
    Grid<Rc> g = make_grid<Rc>(nt, dim, x, h, periodic, lo, hi);
    std::vector<int64_t> cid(nt);
    std::vector<int64_t> start(g.ncells + 1, 0);
    for (int64_t i = 0; i < nt; ++i) {
        cid[i] = cell_id(x + i * dim, g, dim);
        start[cid[i] + 1]++;
    }
    for (int64_t c = 0; c < g.ncells; ++c) start[c + 1] += start[c];
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    std::vector<int> part(nt);
    for (int64_t i = 0; i < nt; ++i) part[fill[cid[i]]++] = (int)i;
    out.pi.clear();
    out.pj.clear();
    for (int64_t i = 0; i < nt; ++i) {
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
                    for (int64_t k = start[c]; k < start[c + 1]; ++k) {
                        int j = part[k];
                        if (j <= i) continue;
                        if (pair_test(x + i * dim, x + (int64_t)j * dim, h[i], h[j], dim, g,
                                      periodic)) {
                            out.pi.push_back((int)i);
                            out.pj.push_back(j);
                        }
                    }
                }
    }
    if (cell_of) *cell_of = cid;
    return g;
}

// direct_find.f:1-61: all pairs i < j with sqrt(dr^2) < scale_k * mh.
template <class Rc>
void direct_find(int64_t nt, int dim, const Rc* x, const Rc* h, const int* periodic,
                 const Grid<Rc>& g, PairList& out) {
    out.pi.clear();
    out.pj.clear();
    for (int64_t i = 0; i + 1 < nt; ++i)
        for (int64_t j = i + 1; j < nt; ++j) {
            Rc dr2 = Rc(0);
            for (int d = 0; d < dim; ++d) {
                Rc dx = min_image(Rc(x[i * dim + d] - x[j * dim + d]), g, d, periodic);
                dr2 = (d == 0) ? Rc(dx * dx) : Rc(dr2 + dx * dx);
            }
            Rc mh = (h[i] + h[j]) / Rc(2);
            if (std::sqrt(dr2) < Rc(2) * mh) {
                out.pi.push_back((int)i);
                out.pj.push_back((int)j);
            }
        }
}

// ---------------------------------------------------------------------------
// Step state (particle-major like the Fortran x(dim, maxn)).
// ---------------------------------------------------------------------------
template <class R>
struct State {
    int64_t n = 0;
    int dim = 2;
    std::vector<R> x, v, m, rho, p, u, h, c;
    std::vector<int> itype;
    std::vector<R> dvdt, dudt;  // rates of the last single_step (carried)
    std::vector<R> drho;        // drho/dt of the last single_step (density_form 1; carried)
    bool fluid(int64_t i) const { return itype[i] > 0; }
};

template <class R>
struct Rates {
    std::vector<R> dv, du, tdsdt, divv, drho, av;
};

// Pair geometry shared by every pair loop: dx = x_i - x_j (minimum image),
// r, mh = (h_i + h_j)/2, W and dW/dx_i.
template <class R, class Rc>
struct PairGeom {
    R dx[3], r2, r, mh, w, dwdx[3];
};

template <class R, class Rc>
inline void pair_geom(const State<R>& s, const Grid<Rc>& g, const Params<R>& P, int i, int j,
                      PairGeom<R, Rc>& pg) {
    (void)g;  // the geometry needs no grid: the minimum image uses the period of P
    const int dim = s.dim;
    pg.r2 = R(0);
    for (int d = 0; d < dim; ++d) {
        R dx = s.x[(int64_t)i * dim + d] - s.x[(int64_t)j * dim + d];
        if (P.periodic[d]) {
            R L = R(period_length(P, d));
            if (dx > R(0.5) * L) dx = dx - L;
            else if (dx < -R(0.5) * L) dx = dx + L;
        }
        pg.dx[d] = dx;
        pg.r2 = pg.r2 + dx * dx;
    }
    using std::sqrt;
    pg.r = sqrt(pg.r2);
    pg.mh = R(0.5) * (s.h[i] + s.h[j]);
    pg.w = kernel_w(pg.r, pg.mh, dim, P.kernel_3d_legacy);
    kernel_dwdx(pg.dx, pg.r, pg.mh, dim, P.kernel_3d_legacy, pg.dwdx);
}

// density.f:1-62 (sum_density): rho_i = m_i W(0, h_i) + sum_j m_j W_ij, fluid only.
template <class R, class Rc>
void sum_density(State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl) {
    for (int64_t i = 0; i < s.n; ++i)
        if (s.fluid(i)) s.rho[i] = kernel_w(R(0), s.h[i], s.dim, P.kernel_3d_legacy) * s.m[i];
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        if (s.fluid(i)) s.rho[i] = s.rho[i] + s.m[j] * pg.w;
        if (s.fluid(j)) s.rho[j] = s.rho[j] + s.m[i] * pg.w;
    }
}

// density.f:161-218 (con_density): drho_i = sum_j m_j (v_i - v_j) . grad_i W_ij,
// fluid only.
template <class R, class Rc>
void con_density(const State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl,
                 std::vector<R>& drho) {
    const int dim = s.dim;
    drho.assign(s.n, R(0));
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        const int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        R vcc = R(0);
        for (int d = 0; d < dim; ++d)
            vcc = vcc + (s.v[(int64_t)i * dim + d] - s.v[(int64_t)j * dim + d]) * pg.dwdx[d];
        if (s.fluid(i)) drho[i] = drho[i] + s.m[j] * vcc;
        if (s.fluid(j)) drho[j] = drho[j] + s.m[i] * vcc;
    }
}

// density.f:65-158 (nor_density): rho_i = (m_i W(0) + sum_j m_j W_ij) /
// (m_i W(0)/rho_i + sum_j m_j/rho_j W_ij), the denominator on the densities
// the iteration starts with; fluid only.
template <class R, class Rc>
void nor_density(State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl) {
    std::vector<R> wi(s.n, R(0)), num(s.n, R(0));
    for (int64_t i = 0; i < s.n; ++i)
        if (s.fluid(i)) {
            const R w0 = kernel_w(R(0), s.h[i], s.dim, P.kernel_3d_legacy);
            wi[i] = w0 * s.m[i] / s.rho[i];
            num[i] = w0 * s.m[i];
        }
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        const int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        if (s.fluid(i)) {
            wi[i] = wi[i] + s.m[j] / s.rho[j] * pg.w;
            num[i] = num[i] + s.m[j] * pg.w;
        }
        if (s.fluid(j)) {
            wi[j] = wi[j] + s.m[i] / s.rho[i] * pg.w;
            num[j] = num[j] + s.m[i] * pg.w;
        }
    }
    for (int64_t i = 0; i < s.n; ++i)
        if (s.fluid(i)) s.rho[i] = num[i] / wi[i];
}

// av_vel.f:1-62: XSPH, av_i = -eps sum_j m_j / rho_ij (v_i - v_j) W_ij with
// rho_ij = (rho_i + rho_j)/2, eps = 0.3; fluid only.
template <class R, class Rc>
void av_vel(const State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl,
            std::vector<R>& av) {
    const int dim = s.dim;
    const R eps = R(0.3);
    av.assign(s.n * dim, R(0));
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        const int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        const R mrho = (s.rho[i] + s.rho[j]) / R(2);
        for (int d = 0; d < dim; ++d) {
            const R dv = s.v[(int64_t)i * dim + d] - s.v[(int64_t)j * dim + d];
            if (s.fluid(i)) av[(int64_t)i * dim + d] = av[(int64_t)i * dim + d] - eps * s.m[j] / mrho * dv * pg.w;
            if (s.fluid(j)) av[(int64_t)j * dim + d] = av[(int64_t)j * dim + d] + eps * s.m[i] / mrho * dv * pg.w;
        }
    }
}

// hsml.f (h_upgrade) on the fluid particles, after the rates: sle 1,
// h = 2 (m/rho)^(1/dim) (the exponent is the Fortran's single-precision 1./dim);
// sle 2, dh/dt = (h/dim) div v with div v_i = sum_j m_j/rho_j (v_j - v_i) . grad_i W,
// h += dt dh unless that leaves h <= 0.
template <class R, class Rc>
void h_upgrade(State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl, double dt) {
    using std::pow;
    const int dim = s.dim;
    if (P.sle == 1) {
        const double e = (double)(1.0f / (float)dim);
        for (int64_t i = 0; i < s.n; ++i)
            if (s.fluid(i)) s.h[i] = R(2) * pow(s.m[i] / s.rho[i], e);
        return;
    }
    if (P.sle != 2) return;
    std::vector<R> divv(s.n, R(0));
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        const int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        R vdw = R(0);
        for (int d = 0; d < dim; ++d)
            vdw = vdw + (s.v[(int64_t)j * dim + d] - s.v[(int64_t)i * dim + d]) * pg.dwdx[d];
        divv[i] = divv[i] + s.m[j] / s.rho[j] * vdw;
        divv[j] = divv[j] + s.m[i] / s.rho[i] * vdw;
    }
    for (int64_t i = 0; i < s.n; ++i) {
        if (!s.fluid(i)) continue;
        const R dh = (s.h[i] / R(dim)) * divv[i];
        const R hn = s.h[i] + R(dt) * dh;
        if (!(hn <= R(0))) s.h[i] = hn;
    }
}

// Tait EOS (eos.f90:255-283): p = rho0 c0^2/7 ((rho/rho0)^7 - 1), c = c0; if
// p < pmin then p = 0 and rho = rho0. Fluid particles only (single_step.f:120).
template <class R>
inline void eos_tait(R& rho, R& p, const Params<R>& P) {
    R ratio = rho / P.rho0;
    R r2 = ratio * ratio;
    R r7 = r2 * r2 * r2 * ratio;
    p = P.rho0 * P.c0 * P.c0 / R(7) * (r7 - R(1));
    if (p < P.pmin) {
        p = R(0);
        rho = P.rho0;
    }
}

// internal_force.f:1-437 (int_force).
template <class R, class Rc>
void int_force(const State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl,
               std::vector<R>& dvdt, std::vector<R>& dudt, std::vector<R>& tdsdt) {
    const int dim = s.dim;
    const int64_t n = s.n;
    std::vector<R> T(n * 6, R(0));  // txx tyy tzz txy txz tyz
    dvdt.assign(n * dim, R(0));
    dudt.assign(n, R(0));
    tdsdt.assign(n, R(0));
    PairGeom<R, Rc> pg;
    if (P.visc) {
        // Shear tensor T_ab = v_a,b + v_b,a - 2/3 delta_ab v_c,c (internal_force.f:75-152).
        for (size_t k = 0; k < pl.pi.size(); ++k) {
            int i = pl.pi[k], j = pl.pj[k];
            pair_geom(s, g, P, i, j, pg);
            R dv[3] = {R(0), R(0), R(0)};
            for (int d = 0; d < dim; ++d) dv[d] = s.v[(int64_t)j * dim + d] - s.v[(int64_t)i * dim + d];
            const R* w = pg.dwdx;
            R hxx, hyy, hzz = R(0), hxy, hxz = R(0), hyz = R(0);
            if (dim == 2) {
                hxx = R(2) * dv[0] * w[0] - dv[1] * w[1];
                hyy = R(2) * dv[1] * w[1] - dv[0] * w[0];
                hxy = dv[0] * w[1] + dv[1] * w[0];
            } else {
                hxx = R(2) * dv[0] * w[0] - dv[1] * w[1] - dv[2] * w[2];
                hyy = R(2) * dv[1] * w[1] - dv[0] * w[0] - dv[2] * w[2];
                hzz = R(2) * dv[2] * w[2] - dv[0] * w[0] - dv[1] * w[1];
                hyz = dv[1] * w[2] + dv[2] * w[1];
                hxz = dv[0] * w[2] + dv[2] * w[0];
                hxy = dv[0] * w[1] + dv[1] * w[0];
            }
            hxx = R(2.0 / 3.0) * hxx;
            hyy = R(2.0 / 3.0) * hyy;
            hzz = R(2.0 / 3.0) * hzz;
            R hh[6] = {hxx, hyy, hzz, hxy, hxz, hyz};
            for (int a = 0; a < 6; ++a) {
                T[(int64_t)i * 6 + a] = T[(int64_t)i * 6 + a] + s.m[j] * hh[a] / s.rho[j];
                T[(int64_t)j * 6 + a] = T[(int64_t)j * 6 + a] + s.m[i] * hh[a] / s.rho[i];
            }
        }
        // Viscous entropy T ds/dt = 1/2 eta/rho T_ab T_ab (internal_force.f:156-171).
        for (int64_t i = 0; i < n; ++i) {
            if (!s.fluid(i)) continue;
            const R* t = &T[i * 6];
            R q;
            if (dim == 2) q = t[0] * t[0] + t[1] * t[1] + R(2) * t[3] * t[3];
            else
                q = t[0] * t[0] + t[1] * t[1] + t[2] * t[2] + R(2) * t[5] * t[5] +
                    R(2) * t[4] * t[4] + R(2) * t[3] * t[3];
            tdsdt[i] = R(0.5) * P.eta / s.rho[i] * q;
        }
    }
    // Pressure force, viscous force and -p/rho div v (internal_force.f:178-429).
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        const R* w = pg.dwdx;
        R he = R(0);
        R hv[3];
        const R* ti = &T[(int64_t)i * 6];
        const R* tj = &T[(int64_t)j * 6];
        // Rows of the symmetric tensor as (row a, column b) -> index.
        static const int tidx[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
        if (P.pa_sph == 0) {
            R rr = s.rho[i] * s.rho[j];
            for (int d = 0; d < dim; ++d) {
                R h = -(s.p[i] + s.p[j]) * w[d];
                he = he + (s.v[(int64_t)j * dim + d] - s.v[(int64_t)i * dim + d]) * h;
                if (P.visc)
                    for (int b = 0; b < dim; ++b)
                        h = h + (P.eta * ti[tidx[d][b]] + P.eta * tj[tidx[d][b]]) * w[b];
                hv[d] = h / rr;
            }
            he = he / rr;
        } else {
            R pi2 = s.p[i] / (s.rho[i] * s.rho[i]);
            R pj2 = s.p[j] / (s.rho[j] * s.rho[j]);
            R ri2 = s.rho[i] * s.rho[i], rj2 = s.rho[j] * s.rho[j];
            for (int d = 0; d < dim; ++d) {
                R h = -(pi2 + pj2) * w[d];
                he = he + (s.v[(int64_t)j * dim + d] - s.v[(int64_t)i * dim + d]) * h;
                if (P.visc)
                    for (int b = 0; b < dim; ++b)
                        h = h + (P.eta * ti[tidx[d][b]] / ri2 + P.eta * tj[tidx[d][b]] / rj2) * w[b];
                hv[d] = h;
            }
        }
        for (int d = 0; d < dim; ++d) {
            dvdt[(int64_t)i * dim + d] = dvdt[(int64_t)i * dim + d] + s.m[j] * hv[d];
            dvdt[(int64_t)j * dim + d] = dvdt[(int64_t)j * dim + d] - s.m[i] * hv[d];
        }
        dudt[i] = dudt[i] + s.m[j] * he;
        dudt[j] = dudt[j] + s.m[i] * he;
    }
    // de/dt = T ds/dt + 1/2 (sum) (internal_force.f:433-435).
    for (int64_t i = 0; i < n; ++i) dudt[i] = tdsdt[i] + R(0.5) * dudt[i];
}

// art_visc.f:1-103.
template <class R, class Rc>
void art_visc(const State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl,
              std::vector<R>& dvdt, std::vector<R>& dudt) {
    const int dim = s.dim;
    dvdt.assign(s.n * dim, R(0));
    dudt.assign(s.n, R(0));
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        R vr = R(0), vdwdx = R(0);
        for (int d = 0; d < dim; ++d) {
            R dv = s.v[(int64_t)i * dim + d] - s.v[(int64_t)j * dim + d];
            vr = vr + dv * pg.dx[d];
            vdwdx = vdwdx + dv * pg.dwdx[d];
        }
        if (vr < R(0)) {
            R he = pg.mh * P.av_eta;
            R phi = (pg.mh * vr) / (pg.r2 + he * he);
            R mc = R(0.5) * (s.c[i] + s.c[j]);
            R mrho = R(0.5) * (s.rho[i] + s.rho[j]);
            R piv = (P.av_beta * phi - P.av_alpha * mc) * phi / mrho;
            for (int d = 0; d < dim; ++d) {
                dvdt[(int64_t)i * dim + d] = dvdt[(int64_t)i * dim + d] - s.m[j] * piv * pg.dwdx[d];
                dvdt[(int64_t)j * dim + d] = dvdt[(int64_t)j * dim + d] + s.m[i] * piv * pg.dwdx[d];
            }
            dudt[i] = dudt[i] + R(0.5) * s.m[j] * piv * vdwdx;
            dudt[j] = dudt[j] + R(0.5) * s.m[i] * piv * vdwdx;
        }
    }
}

// art_heat.f:1-99. divv is returned for diagnostics.
template <class R, class Rc>
void art_heat(const State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl,
              std::vector<R>& dudt, std::vector<R>& divv) {
    const int dim = s.dim;
    dudt.assign(s.n, R(0));
    divv.assign(s.n, R(0));
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        R vdwdx = R(0);
        for (int d = 0; d < dim; ++d)
            vdwdx = vdwdx + (s.v[(int64_t)j * dim + d] - s.v[(int64_t)i * dim + d]) * pg.dwdx[d];
        divv[i] = divv[i] + s.m[j] / s.rho[i] * vdwdx;
        divv[j] = divv[j] + s.m[i] / s.rho[j] * vdwdx;
    }
    using std::fabs;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        R mrho = R(0.5) * (s.rho[i] + s.rho[j]);
        R rdwdx = R(0);
        for (int d = 0; d < dim; ++d) rdwdx = rdwdx + pg.dx[d] * pg.dwdx[d];
        R psi_i = P.ah_g1 * s.h[i] * s.c[i] + P.ah_g2 * s.h[i] * s.h[i] * (fabs(divv[i]) - divv[i]);
        R psi_j = P.ah_g1 * s.h[j] * s.c[j] + P.ah_g2 * s.h[j] * s.h[j] * (fabs(divv[j]) - divv[j]);
        R psi_ij = R(0.5) * (psi_i + psi_j);
        R he = pg.mh * P.ah_eta;
        R psi = (R(2) * psi_ij) / (mrho * (pg.r2 + he * he)) * rdwdx;
        dudt[i] = dudt[i] + s.m[j] * psi * (s.u[i] - s.u[j]);
        dudt[j] = dudt[j] + s.m[i] * psi * (s.u[j] - s.u[i]);
    }
}

// Pairs of equal and of different itype. Returns the pairs the density, force
// and heat sums run over: all of them, except for wall_model 1, where pairs of
// different itype take part in none of those sums (ArmandoThrust/armando.cu:
// 472-506 acts on same-material pairs only) and only push (wall_repulsion).
template <class R>
const PairList& split_by_itype(const State<R>& s, const Params<R>& P, const PairList& pl,
                               PairList& same, PairList& other) {
    if (!repulsive_walls(P)) return pl;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        PairList& dst = (s.itype[pl.pi[k]] == s.itype[pl.pj[k]]) ? same : other;
        dst.pi.push_back(pl.pi[k]);
        dst.pj.push_back(pl.pj[k]);
    }
    return (P.wall_model == 1) ? same : pl;
}

// Push between particles of different itype (the GPU-C codes' boundary
// repulsion, momentum only, along (x_i - x_j)/r, c = c0, W at h = (h_i+h_j)/2):
//   wall_model 1, ArmandoThrust/armando.cu:507-513:  f = 0.5 W m_j / (rho_j h_j) c_j^2
//   wall_model 2, ArmandoThrust/acpu.c:424-429:      f = 0.02 (W / W(0)) c_i c_j / r
//                                                        * m_j / (m_i + m_j)
// (the reference evaluates W with h_i; identical for uniform h). A coincident
// pair has no direction and pushes nothing. Walls are not integrated, so only
// fluid particles keep their rate.
template <class R, class Rc>
void wall_repulsion(const State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl,
                    std::vector<R>& dvdt) {
    const int dim = s.dim;
    dvdt.assign(s.n * dim, R(0));
    PairGeom<R, Rc> pg;
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        int i = pl.pi[k], j = pl.pj[k];
        pair_geom(s, g, P, i, j, pg);
        if (!(pg.r > R(0))) continue;
        const R w_rel = pg.w / kernel_w(R(0), pg.mh, dim, P.kernel_3d_legacy);
        R fi, fj;  // push on i (from j) and on j (from i), per unit (x_i - x_j)/r
        if (P.wall_model == 1) {
            fi = R(0.5) * pg.w * s.m[j] / (s.rho[j] * s.h[j]) * s.c[j] * s.c[j];
            fj = R(0.5) * pg.w * s.m[i] / (s.rho[i] * s.h[i]) * s.c[i] * s.c[i];
        } else {
            const R base = R(0.02) * w_rel * s.c[i] * s.c[j] / pg.r;
            fi = base * s.m[j] / (s.m[i] + s.m[j]);
            fj = base * s.m[i] / (s.m[i] + s.m[j]);
        }
        for (int d = 0; d < dim; ++d) {
            const R e = pg.dx[d] / pg.r;
            if (s.fluid(i)) dvdt[(int64_t)i * dim + d] = dvdt[(int64_t)i * dim + d] + fi * e;
            if (s.fluid(j)) dvdt[(int64_t)j * dim + d] = dvdt[(int64_t)j * dim + d] - fj * e;
        }
    }
}

// External volumetric heat, du_i += q(x_i)/rho_i (fluka_heat.f:337-338), with
// q(x) = q0 exp(-|x - xc|^2 / (2 sigma^2)).
template <class R>
void ext_heat(const State<R>& s, const Params<R>& P, std::vector<R>& dudt) {
    dudt.assign(s.n, R(0));
    using std::exp;
    for (int64_t i = 0; i < s.n; ++i) {
        if (!s.fluid(i)) continue;
        R d2 = R(0);
        for (int d = 0; d < s.dim; ++d) {
            R e = s.x[i * s.dim + d] - P.heat_center[d];
            d2 = d2 + e * e;
        }
        R q = P.heat_q0 * exp(-d2 / (R(2) * P.heat_sigma * P.heat_sigma));
        dudt[i] = q / s.rho[i];
    }
}

// Mirror ghost particles (wall_model 3): CERNsource/ghost.f:1-86, rebuilt
// every iteration after the predictor (time_integration.f:156-161). A fluid
// particle i whose pairs include wall particles (itype <= 0) takes the
// nearest one, w, whose velocity entry holds its inward unit normal n (the
// Fortran's virtual-particle files carry normals there, input.f:256-314), and
// gains the ghost
//   x_g = x_i - 2 n ((x_i - x_w) . n),   v_g = v_i - 2 n (v_i . n)
// (ghost.f:67-75) with m and h of i; rho, p and u of i are copied to it after
// the density and EOS of the iteration (single_step.f:188-196). Ghosts follow
// the real particles, in the order of their owners (ghost.f:60-84).
// Departures, each without effect on a defined result:
//   * candidates are the pairs at the current positions; the Fortran reuses
//     the previous iteration's pair list. The two differ only where the
//     nearest wall particle sits at the edge of the support, and such a ghost
//     lies beyond the reach of every fluid particle.
//   * the nearest is chosen on the squared distance in coordinate precision
//     Rc (that of the pair test), ties to the lower index; the Fortran compares
//     in FP64 and keeps the first in pair order.
//   * ghosts have c = c0 and itype 0; the Fortran leaves both unset.
// The ghosts' neighbour-search coordinates are computed in Rc from the Rc
// coordinates, in the library's operation order (xc).
template <class R, class Rc>
struct Ghosts {
    int64_t n_real = 0;
    std::vector<int64_t> owner, wall;  // of ghost k = particle n_real + k
    std::vector<Rc> xc;                // [k * dim + d]
};

template <class R, class Rc>
void ghost_particles(State<R>& s, const Params<R>& P, Ghosts<R, Rc>& G) {
    const int dim = s.dim;
    const int64_t n = s.n;
    for (int d = 0; d < dim; ++d)
        if (P.periodic[d]) throw std::runtime_error("mirror ghosts need a system without periodic axes");
    G.n_real = n;
    G.owner.clear();
    G.wall.clear();
    G.xc.clear();
    std::vector<Rc> xc(n * dim), hc(n);
    for (int64_t i = 0; i < n * dim; ++i) xc[i] = Rc(s.x[i]);
    for (int64_t i = 0; i < n; ++i) hc[i] = Rc(s.h[i]);
    PairList pl;
    link_list<Rc>(n, dim, xc.data(), hc.data(), P.periodic, P.period_lo, P.period_hi, pl);
    std::vector<int64_t> best(n, -1);
    std::vector<Rc> bestd(n, Rc(0));
    auto offer = [&](int64_t a, int64_t w) {
        Rc dd = Rc(0);
        for (int d = 0; d < dim; ++d) {  // ghost.f:49-52, (x_w - x_i)^2 summed over axes
            Rc t = Rc(xc[w * dim + d] - xc[a * dim + d]);
            Rc sq = t * t;
            dd = (d == 0) ? sq : Rc(dd + sq);
        }
        if (best[a] < 0 || dd < bestd[a] || (dd == bestd[a] && w < best[a])) {
            best[a] = w;
            bestd[a] = dd;
        }
    };
    for (size_t k = 0; k < pl.pi.size(); ++k) {
        const int64_t a = pl.pi[k], b = pl.pj[k];
        if (s.fluid(a) && !s.fluid(b)) offer(a, b);
        else if (s.fluid(b) && !s.fluid(a)) offer(b, a);
    }
    for (int64_t a = 0; a < n; ++a)
        if (best[a] >= 0) {
            G.owner.push_back(a);
            G.wall.push_back(best[a]);
        }
    const int64_t ng = (int64_t)G.owner.size(), nt = n + ng;
    s.x.resize(nt * dim);
    s.v.resize(nt * dim);
    for (auto* a : {&s.m, &s.rho, &s.p, &s.u, &s.h, &s.c}) a->resize(nt);
    s.itype.resize(nt);
    s.dvdt.resize(nt * dim, R(0));
    s.dudt.resize(nt, R(0));
    G.xc.resize(ng * dim);
    for (int64_t k = 0; k < ng; ++k) {
        const int64_t a = G.owner[k], w = G.wall[k], g = n + k;
        R dd1 = R(0), dd2 = R(0);
        Rc e = Rc(0);
        for (int d = 0; d < dim; ++d) {  // ghost.f:66-70
            const R nd = s.v[w * dim + d];
            const R t1 = (s.x[a * dim + d] - s.x[w * dim + d]) * nd;
            const R t2 = s.v[a * dim + d] * nd;
            dd1 = (d == 0) ? t1 : R(dd1 + t1);
            dd2 = (d == 0) ? t2 : R(dd2 + t2);
            const Rc tc = Rc(Rc(xc[a * dim + d] - xc[w * dim + d]) * Rc(nd));
            e = (d == 0) ? tc : Rc(e + tc);
        }
        for (int d = 0; d < dim; ++d) {  // ghost.f:72-75
            const R nd = s.v[w * dim + d];
            s.x[g * dim + d] = s.x[a * dim + d] - R(2) * nd * dd1;
            s.v[g * dim + d] = s.v[a * dim + d] - R(2) * nd * dd2;
            G.xc[k * dim + d] = Rc(xc[a * dim + d] - Rc(Rc(Rc(2) * Rc(nd)) * e));
            s.dvdt[g * dim + d] = R(0);
        }
        s.m[g] = s.m[a];  // ghost.f:77-80
        s.h[g] = s.h[a];
        s.rho[g] = s.rho[a];
        s.p[g] = s.p[a];
        s.u[g] = s.u[a];
        s.c[g] = P.c0;
        s.itype[g] = 0;
        s.dudt[g] = R(0);
    }
    s.n = nt;
}

// Drops the ghosts again after the iteration (time_integration.f:190-205
// advances particles 1..np only).
template <class R, class Rc>
void drop_ghosts(State<R>& s, const Ghosts<R, Rc>& G) {
    const int64_t n = G.n_real;
    const int dim = s.dim;
    s.x.resize(n * dim);
    s.v.resize(n * dim);
    for (auto* a : {&s.m, &s.rho, &s.p, &s.u, &s.h, &s.c}) a->resize(n);
    s.itype.resize(n);
    s.n = n;
}

// single_step.f:92-234 for summation density and the Tait family:
// fills s.rho, s.p (fluid), s.c, and rates dv, du (zero for walls).
template <class R, class Rc>
void single_step(State<R>& s, const Grid<Rc>& g, const Params<R>& P, const PairList& pl, int its,
                 double dt, Rates<R>& out, const Ghosts<R, Rc>* ghosts = nullptr) {
    const int dim = s.dim;
    const int64_t n = s.n;
    PairList same, other;
    const PairList& body = split_by_itype(s, P, pl, same, other);
    if (P.density_form == 1) con_density(s, g, P, body, out.drho);  // single_step.f:106-108
    else if (P.density_form == 2) nor_density(s, g, P, body);
    else sum_density(s, g, P, body);
    for (int64_t i = 0; i < n; ++i) {
        s.c[i] = P.c0;
        if (s.fluid(i)) eos_tait(s.rho[i], s.p[i], P);
    }
    if (ghosts)  // single_step.f:188-196
        for (size_t k = 0; k < ghosts->owner.size(); ++k) {
            const int64_t gi = ghosts->n_real + (int64_t)k, o = ghosts->owner[k];
            s.rho[gi] = s.rho[o];
            s.p[gi] = s.p[o];
            s.u[gi] = s.u[o];
        }
    std::vector<R> indvdt, indudt, avdvdt, avdudt, ahdudt, exdudt, rpdvdt;
    int_force(s, g, P, body, indvdt, indudt, out.tdsdt);
    if (P.visc_artificial) art_visc(s, g, P, body, avdvdt, avdudt);
    if (P.heat_artificial) art_heat(s, g, P, body, ahdudt, out.divv);
    if (repulsive_walls(P)) wall_repulsion(s, g, P, other, rpdvdt);
    if (P.average_velocity) av_vel(s, g, P, body, out.av);  // single_step.f:214-216
    if (P.heat_external && (double(its) * dt <= P.heat_t_end)) ext_heat(s, P, exdudt);
    if (P.sle) h_upgrade(s, g, P, body, dt);  // single_step.f:224-226
    out.dv.assign(n * dim, R(0));
    out.du.assign(n, R(0));
    for (int64_t i = 0; i < n; ++i) {
        if (!s.fluid(i)) continue;
        for (int d = 0; d < dim; ++d) {
            R a = indvdt[i * dim + d] + P.gravity[d];
            if (P.visc_artificial) a = a + avdvdt[i * dim + d];
            if (repulsive_walls(P)) a = a + rpdvdt[i * dim + d];
            out.dv[i * dim + d] = a;
        }
        R du = indudt[i];
        if (P.visc_artificial) du = du + avdudt[i];
        if (P.heat_artificial) du = du + ahdudt[i];
        if (!exdudt.empty()) du = du + exdudt[i];
        out.du[i] = du;
    }
}

template <class R>
inline void wrap_periodic(State<R>& s, const Params<R>& P, int64_t i) {
    for (int d = 0; d < s.dim; ++d) {
        if (!P.periodic[d]) continue;
        R lo = R(P.period_lo[d]), hi = R(P.period_hi[d]), L = R(period_length(P, d));
        R& xv = s.x[i * s.dim + d];
        if (!(xv < hi)) xv = xv - L;
        else if (xv < lo) xv = xv + L;
    }
}

// Neighbour search for the physics: link_list in coordinate precision Rc on
// the current positions.
template <class R, class Rc>
Grid<Rc> neighbour_search(const State<R>& s, const Params<R>& P, PairList& pl,
                          const Ghosts<R, Rc>* ghosts = nullptr) {
    std::vector<Rc> xc(s.n * s.dim), hc(s.n);
    for (int64_t i = 0; i < s.n * s.dim; ++i) xc[i] = Rc(s.x[i]);
    for (int64_t i = 0; i < s.n; ++i) hc[i] = Rc(s.h[i]);
    if (ghosts)
        for (size_t k = 0; k < ghosts->xc.size(); ++k) xc[ghosts->n_real * s.dim + (int64_t)k] = ghosts->xc[k];
    return link_list<Rc>(s.n, s.dim, xc.data(), hc.data(), P.periodic, P.period_lo, P.period_hi,
                         pl);
}

// One iteration `its` of time_integration.f:131-218 (refresh_step = 1).
// s.dvdt / s.dudt carry the previous rates in and the new rates out.
template <class R, class Rc = R>
void leapfrog_step(State<R>& s, const Params<R>& P, int its, double dt, Rates<R>* rates_out = nullptr,
                   PairList* pairs_out = nullptr) {
    const int dim = s.dim;
    const int64_t n = s.n;
    const R hdt = R(dt / 2.0), fdt = R(dt);
    std::vector<R> u_min, v_min, rho_min;
    const bool cont = P.density_form == 1;
    if (cont && (int64_t)s.drho.size() != n) s.drho.assign(n, R(0));
    if (its != 1) {
        u_min = s.u;
        v_min = s.v;
        rho_min = s.rho;
        for (int64_t i = 0; i < n; ++i) {
            if (!s.fluid(i)) continue;
            s.u[i] = s.u[i] + hdt * s.dudt[i];
            if (s.u[i] < R(0)) s.u[i] = R(0);
            if (cont) s.rho[i] = s.rho[i] + hdt * s.drho[i];  // time_integration.f:144-147
            for (int d = 0; d < dim; ++d) s.v[i * dim + d] = s.v[i * dim + d] + hdt * s.dvdt[i * dim + d];
        }
    }
    Ghosts<R, Rc> G;
    const bool ghosts = P.wall_model == 3;
    if (ghosts) ghost_particles(s, P, G);
    PairList pl;
    Grid<Rc> g = neighbour_search<R, Rc>(s, P, pl, ghosts ? &G : nullptr);
    Rates<R> r;
    single_step(s, g, P, pl, its, dt, r, ghosts ? &G : nullptr);
    if (ghosts) {
        drop_ghosts(s, G);
        r.dv.resize(n * dim);
        r.du.resize(n);
        if (!r.drho.empty()) r.drho.resize(n);
        if (!r.av.empty()) r.av.resize(n * dim);
    }
    for (int64_t i = 0; i < n; ++i) {
        if (!s.fluid(i)) continue;
        if (its != 1) {
            s.u[i] = u_min[i] + fdt * r.du[i];
            if (s.u[i] < R(0)) s.u[i] = R(0);
            if (cont) s.rho[i] = rho_min[i] + fdt * r.drho[i];  // time_integration.f:191-193
            for (int d = 0; d < dim; ++d) {
                s.v[i * dim + d] = v_min[i * dim + d] + fdt * r.dv[i * dim + d];
                if (P.average_velocity) s.v[i * dim + d] = s.v[i * dim + d] + r.av[i * dim + d];
                s.x[i * dim + d] = s.x[i * dim + d] + fdt * s.v[i * dim + d];
            }
        } else {
            s.u[i] = s.u[i] + hdt * r.du[i];
            if (s.u[i] < R(0)) s.u[i] = R(0);
            if (cont) s.rho[i] = s.rho[i] + hdt * r.drho[i];  // time_integration.f:207-209
            for (int d = 0; d < dim; ++d) {
                s.v[i * dim + d] = s.v[i * dim + d] + hdt * r.dv[i * dim + d];
                s.x[i * dim + d] = s.x[i * dim + d] + fdt * s.v[i * dim + d];
            }
        }
        wrap_periodic(s, P, i);
    }
    s.dvdt = r.dv;
    s.dudt = r.du;
    if (cont) s.drho = r.drho;
    if (rates_out) *rates_out = r;
    if (pairs_out) *pairs_out = std::move(pl);
}

}  // namespace ao
