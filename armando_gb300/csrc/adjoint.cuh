// adjoint.cuh -- reverse mode of one leapfrog step (hand-written adjoint).
//
// The step is the forward of kernels.cuh: predictor, summation density, Tait
// EOS, pressure force + Monaghan artificial viscosity + pressure work, external
// heat, gravity, corrector (CERNsource time_integration.f:131-218 with
// single_step.f, density.f, eos.f90:255-283, internal_force.f pa_sph = 1,
// art_visc.f). Its reverse runs as three gathers over the step's neighbour
// sets (the topology of the step is frozen), with no atomics:
//   k_adj_out      cotangents of the corrector: a_bar, du_bar of every particle
//   k_adj_force    pair adjoints of every (i, j) and (j, i) a particle takes
//                  part in, then the EOS and external-heat adjoints of the
//                  particle: x_bar, vh_bar (predicted velocity), rho_bar
//   k_adj_density  adjoint of the summation density, assembly of the input
//                  cotangents, scatter to the slot order of the step's input
// Non-smooth points follow the value: art_visc acts while v_ij . r_ij < 0,
// u = max(0, .) and the Tait clamp pass no gradient where they bind.
// Artificial heat (art_heat.f:42-97), when on: du_i += sum_j m_j (psi_i + psi_j)
// A_ij (u_i - u_j), A = G r^2 / (rho_bar (r^2 + (eta h_bar)^2)), psi_i =
// g1 h_i c0 + g2 h_i^2 (|divv_i| - divv_i), divv_i = sum_j m_j G_ij (vh_j - vh_i)
// . (x_i - x_j) / rho_i. k_adj_force takes the psi, u_half, rho, x cotangents of
// those pair terms (walls included: their psi enters their neighbours' rates)
// and turns psi_bar into the cotangent of each particle's divergence sum;
// k_adj_density gathers that sum's reverse onto velocities and positions. |divv|
// follows its sign (no gradient at divv = 0 from one side).
// Physical viscosity (internal_force.f:75-171), when on: tau_i = eta/rho_i^2 T_i,
// T_i = sum_j m_j/rho_j H(vh_j - vh_i, G_ij d_ij) (the shear tensor of every
// particle, walls included), a_i += sum_j m_j (tau_i + tau_j) G_ij d_ij, du_i +=
// eta/(2 rho_i) T_i:T_i. k_adj_force takes the tau cotangents of the pair
// forces and turns them, with the heating term's, into cotangents of each
// particle's shear tensor; k_adj_shear gathers the shear sums' reverse onto
// velocities, positions and densities before the density reverse.
// Supported: pa_sph = 1.
#pragma once
#include "kernels.cuh"

namespace ag {

// Cotangents of the carried state (x, v, u, previous a, previous du), in one
// slot order: xb {x_bar, -}, vb {v_bar, u_bar}, ab {a_bar, du_bar}.
struct AdjState {
    float4* xb;
    float4* vb;
    float4* ab;
};

enum AdjParam { ADJ_ALPHA = 0, ADJ_BETA = 1, ADJ_C0 = 2, ADJ_Q0 = 3, ADJ_NPARAM = 4 };

// What the reverse of one iteration reads, saved when the iteration runs
// forward: the cell-order working set, the neighbour structure (sorted keys,
// cell table, grid, the cell slot -> input slot permutation) and the energy
// rate the iteration output. About 116 B per particle in 2D.
struct TapeSlot {
    float4* xh;
    float4* vm;
    float4* vmin;
    float4* rp;
    float* p;
    int* itype;
    unsigned* nmask;  // mask_words<DIM>() words per slot, word-major
    unsigned* keys;
    int* perm;
    float* du;
    int* start;
    DevGrid* grid;
    float* ulo;  // rounding residual of the predicted energy (artificial heat only)
    float4* tau;   // physical viscosity: eta/rho^2 T {xx, yy, xy, zz}
    float4* tau2;  // 3D: {xz, yz, -, -}
};

template <int DIM>
__global__ void k_tape_save(StateB B, const unsigned* __restrict__ keys,
                            const int* __restrict__ perm, const float4* __restrict__ ap,
                            TapeSlot T, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    T.xh[s] = B.xh[s];
    T.vm[s] = B.vm[s];
    T.vmin[s] = B.vmin[s];
    T.rp[s] = B.rp[s];
    T.p[s] = B.p[s];
    T.itype[s] = B.itype[s];
    if (B.mtpp == 1) {  // chunks of 4 words, chunk-major (the lane is the slot)
#pragma unroll
        for (int c = 0; c < mask_words<DIM>() / 4; ++c)
            reinterpret_cast<uint4*>(T.nmask)[(size_t)c * n + s] =
                reinterpret_cast<const uint4*>(B.nmask)[(size_t)c * B.mstride + s];
    }
    T.keys[s] = keys[s];
    T.perm[s] = perm[s];
    T.du[s] = ap[s].w;
    if (T.ulo) T.ulo[s] = B.ulo ? B.ulo[s] : 0.f;
    if (T.tau) T.tau[s] = B.tau[s];
    if (T.tau2) T.tau2[s] = B.tau2[s];
}

// The working set of a taped iteration as the pass kernels see it.
inline StateB tape_view(StateB B, const TapeSlot& T, int n) {
    B.xh = T.xh;
    B.vm = T.vm;
    B.vmin = T.vmin;
    B.rp = T.rp;
    B.p = T.p;
    B.itype = T.itype;
    B.nmask = T.nmask;
    B.mstride = n;
    B.ulo = T.ulo;
    if (T.tau) {
        B.tau = T.tau;
        B.tau2 = T.tau2;
    }
    return B;
}

// Caller-order cotangents -> slot order of the final state (A.id).
template <int DIM>
__global__ void k_adj_load(const int* __restrict__ id, const float* __restrict__ xbar,
                           const float* __restrict__ vbar, const float* __restrict__ ubar,
                           const float* __restrict__ abar, const float* __restrict__ dubar,
                           const float* __restrict__ pbar, AdjState G, float* __restrict__ pbar_s,
                           int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = id[s];
    auto v3 = [&](const float* a) {
        if (!a) return make_float4(0.f, 0.f, 0.f, 0.f);
        return make_float4(a[DIM * i], a[DIM * i + 1], DIM == 3 ? a[DIM * i + 2] : 0.f, 0.f);
    };
    float4 xb = v3(xbar), vb = v3(vbar), ab = v3(abar);
    vb.w = ubar ? ubar[i] : 0.f;
    ab.w = dubar ? dubar[i] : 0.f;
    G.xb[s] = xb;
    G.vb[s] = vb;
    G.ab[s] = ab;
    pbar_s[s] = pbar ? pbar[i] : 0.f;
}

// Slot order (= caller order after the gather of the inputs) -> caller arrays.
template <int DIM>
__global__ void k_adj_store(AdjState G, int n, float* __restrict__ xbar, float* __restrict__ vbar,
                            float* __restrict__ ubar, float* __restrict__ abar,
                            float* __restrict__ dubar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xb = G.xb[i], vb = G.vb[i], ab = G.ab[i];
    const float xs[3] = {xb.x, xb.y, xb.z}, vs[3] = {vb.x, vb.y, vb.z}, as[3] = {ab.x, ab.y, ab.z};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        if (xbar) xbar[DIM * i + d] = xs[d];
        if (vbar) vbar[DIM * i + d] = vs[d];
        if (abar) abar[DIM * i + d] = as[d];
    }
    if (ubar) ubar[i] = vb.w;
    if (dubar) dubar[i] = ab.w;
}

// Corrector reverse: x' = x + dt v', v' = v + kdt a, u' = max(0, u + kdt du),
// outputs also carry a and du to the next predictor.
__global__ void k_adj_out(StateB B, const float* __restrict__ du_out, AdjState G, StepArgs S,
                          float4* __restrict__ abar, float4* __restrict__ xpart,
                          float4* __restrict__ vpart, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    if (B.itype[s] <= 0) {
        abar[s] = z;
        xpart[s] = z;
        vpart[s] = z;
        return;
    }
    const float4 xb = G.xb[s], vb = G.vb[s], ab = G.ab[s];
    const float4 vt = make_float4(fmaf(S.dt, xb.x, vb.x), fmaf(S.dt, xb.y, vb.y),
                                  fmaf(S.dt, xb.z, vb.z), 0.f);
    const float du = du_out[s];
    const bool clamped = fmaf(S.kdt, du, B.vmin[s].w) < 0.f;
    const float ub = clamped ? 0.f : vb.w;
    abar[s] = make_float4(fmaf(S.kdt, vt.x, ab.x), fmaf(S.kdt, vt.y, ab.y), fmaf(S.kdt, vt.z, ab.z),
                          fmaf(S.kdt, ub, ab.w));
    xpart[s] = make_float4(xb.x, xb.y, xb.z, 0.f);
    vpart[s] = make_float4(vt.x, vt.y, vt.z, ub);
}

// Adjoint of the force and energy-rate terms of pair (i, j), i fluid:
//   a_i  += -S d,   du_i += -S (w.d)/2,   S = m_j (P_i + P_j + Pi_ij) G(r),
// d = x_i - x_j, w = vh_j - vh_i, Pi_ij the art_visc term (0 unless w.d > 0).
// ab = {a_bar_i, du_bar_i}. Outputs cotangents on d and w, on P_i and P_j
// (equal), on rho_i and rho_j (equal halves of rho_bar), and on alpha, beta, c0.
struct PairAdj {
    float db[3], wb[3];
    float Pb, rb, al, be, c0;
};

template <int DIM>
__device__ __forceinline__ void pair_adjoint(const float* d, const float* w, float dr2, float G,
                                             float dGdr_r, float mh, float rho_bar, float Pi,
                                             float Pj, float mj, const float4& ab,
                                             const DevParams& P, PairAdj& o) {
    float wd = w[0] * d[0] + w[1] * d[1];
    float ad = ab.x * d[0] + ab.y * d[1];
    if (DIM == 3) {
        wd += w[2] * d[2];
        ad += ab.z * d[2];
    }
    const float vr = -wd;  // (vh_i - vh_j) . (x_i - x_j)
    float pv = 0.f, phi = 0.f, den = 1.f;
    const bool av = P.visc_art && vr < 0.f;
    if (av) {
        den = dr2 + mh * mh * P.av_eta2;
        phi = mh * vr / den;
        pv = (P.av_beta * phi - P.av_alpha * P.c0) * phi / rho_bar;
    }
    const float T = Pi + Pj + pv;
    const float Sv = mj * T * G;
    const float Sb = -(ad + 0.5f * ab.w * wd);
    const float abv[3] = {ab.x, ab.y, ab.z};
    const float Gb = mj * T * Sb;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        o.db[k] = -Sv * (abv[k] + 0.5f * ab.w * w[k]) + Gb * dGdr_r * d[k];
        o.wb[k] = -0.5f * Sv * ab.w * d[k];
    }
    const float Tb = mj * G * Sb;
    o.Pb = Tb;
    o.rb = o.al = o.be = o.c0 = 0.f;
    if (av) {
        const float pb = Tb;
        const float phib = pb * (2.f * P.av_beta * phi - P.av_alpha * P.c0) / rho_bar;
        o.rb = -0.5f * pb * pv / rho_bar;
        o.al = -pb * P.c0 * phi / rho_bar;
        o.be = pb * phi * phi / rho_bar;
        o.c0 = -pb * P.av_alpha * phi / rho_bar;
        const float vrb = phib * mh / den;
        const float r2b = -phib * phi / den;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            o.wb[k] -= vrb * d[k];
            o.db[k] += -vrb * w[k] + 2.f * r2b * d[k];
        }
    }
}

// Neighbours of a fluid particle in warp-converged rounds (same candidates and
// pair test as the forward passes; 2D reuses the density pass's bit mask).
template <int DIM>
struct NbrStream {
    Cursor cu;
    bool done, from_mask;
    int wi, rbase;
    unsigned wbits;
    uint4 ch;
};

// use_mask: the density pass left this slot's bits (fluid particles); walls
// test their candidates.
template <int DIM>
__device__ __forceinline__ void nbr_init(NbrStream<DIM>& ns, const StateB& B, const DevGrid& g,
                                         int s, bool work, bool use_mask = true) {
    ns.cu = cursor_begin<DIM>(g);
    ns.done = !work;
    ns.from_mask = false;
    ns.wbits = 0u;
    ns.ch = make_uint4(0u, 0u, 0u, 0u);
    // masks of several lanes per particle are not in this layout: test instead
    if (work && use_mask && B.mtpp == 1) {
        ns.ch = mask_load_chunk<mask_words<DIM>()>(B.nmask, B.mstride, s, 0);
        ns.wbits = ns.ch.x;
        ns.from_mask = !(ns.ch.x == ~0u && ns.ch.y == ~0u);
    }
    ns.wi = 0;
    ns.rbase = 0;
}

template <int DIM>
__device__ __forceinline__ int nbr_fill(NbrStream<DIM>& ns, const StateB& B, const DevGrid& g,
                                        const int* __restrict__ start, const CellCoord& cc,
                                        const float4& xi, int s, int (*s_list)[kPassThreads]) {
    const int tid = threadIdx.x;
    int nl = 0;
    while (!ns.done && ns.from_mask) {
        if (nl == kListCap) break;
        while (ns.wbits == 0u && ns.wi < mask_words<DIM>() - 1) {
            ++ns.wi;
            if (ns.wi % 4 == 0)
                ns.ch = mask_load_chunk<mask_words<DIM>()>(B.nmask, B.mstride, s, ns.wi / 4);
            ns.wbits = chunk_word(ns.ch, ns.wi % 4);
        }
        if (ns.wbits == 0u) {
            ns.done = true;
            break;
        }
        const int o = 32 * ns.wi + __ffs(ns.wbits) - 1;
        ns.wbits &= ns.wbits - 1u;
        bool in_rows = true;
        while (o >= ns.rbase + (ns.cu.ke - ns.cu.k)) {
            ns.rbase += ns.cu.ke - ns.cu.k;
            if (!cursor_next<DIM>(g, start, cc, ns.cu)) {
                in_rows = false;
                break;
            }
        }
        if (!in_rows) {
            ns.done = true;
            break;
        }
        s_list[nl++][tid] = ns.cu.k + (o - ns.rbase);
    }
    while (!ns.done && !ns.from_mask) {
        if (ns.cu.k >= ns.cu.ke) {
            if (!cursor_next<DIM>(g, start, cc, ns.cu)) {
                ns.done = true;
                break;
            }
        }
        if (nl == kListCap) break;
        const int k = ns.cu.k++;
        if (k == s) continue;
        float d[3], dr2;
        if (pair_delta<DIM>(xi, __ldg(B.xh + k), g, d, dr2)) s_list[nl++][tid] = k;
    }
    return nl;
}

// Symmetric tensors as stored by the shear pass: a {xx, yy, xy, zz}, b {xz, yz}.
// H(dv, w) is the shear pass's pair term: diagonal (2/3)(2 dv_a w_a - sum of
// the others), off-diagonal dv_a w_b + dv_b w_a. A . H(dv, w) = dv^T M(A) w,
// M(A) symmetric with M_aa = (2/3)(2 A_aa - the other diagonal entries) and
// M_ab = A_ab.
template <int DIM>
__device__ __forceinline__ void sym_apply(const float4& a, const float4& b, const float* x,
                                          float* y) {  // y = S x, S = {a, b}
    y[0] = a.x * x[0] + a.z * x[1];
    y[1] = a.z * x[0] + a.y * x[1];
    y[2] = 0.f;
    if (DIM == 3) {
        y[0] += b.x * x[2];
        y[1] += b.y * x[2];
        y[2] = b.x * x[0] + b.y * x[1] + a.w * x[2];
    }
}

template <int DIM>
__device__ __forceinline__ void shear_m(const float4& a, const float4& b, float4& ma, float4& mb) {
    const float tr = (DIM == 3) ? a.x + a.y + a.w : a.x + a.y;
    // (2/3)(2 A_aa - (tr - A_aa)) = (2/3)(3 A_aa - tr)
    ma = make_float4((2.f / 3.f) * (3.f * a.x - tr), (2.f / 3.f) * (3.f * a.y - tr), a.z,
                     DIM == 3 ? (2.f / 3.f) * (3.f * a.w - tr) : 0.f);
    mb = b;
}

// Forward pair geometry shared by the adjoint gathers.
template <int DIM>
struct PairGeo {
    float d[3], dr2, G, dGdr_r, mh;
};

template <int DIM>
__device__ __forceinline__ void pair_geo(const float4& xi, const float4& xj, const DevGrid& g,
                                         const DevParams& P, PairGeo<DIM>& pg) {
    pair_delta<DIM>(xi, xj, g, pg.d, pg.dr2);
    refine_periodic<DIM>(xi, xj, g, pg.d, pg.dr2);
    const float ih = (xj.w == xi.w) ? __fdividef(1.0f, xi.w) : __fdividef(2.0f, xi.w + xj.w);
    const float kgih = P.kg * pow_grad<DIM>(ih);
    const float r = fast_sqrt_pos(pg.dr2);
    const float t = r * ih - 2.0f;
    pg.G = kgih * t * t * t;
    pg.dGdr_r = r > 0.f ? 3.0f * kgih * ih * t * t / r : 0.f;
    pg.mh = 0.5f * (xi.w + xj.w);
}

template <int DIM>
__global__ void __launch_bounds__(kPassThreads)
    k_adj_force(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
                const DevGrid* __restrict__ gp, DevParams P, StepArgs S,
                const float4* __restrict__ abar, const float* __restrict__ pbar_loss,
                float* __restrict__ rhobar, float4* __restrict__ xF, float4* __restrict__ vhb,
                float* __restrict__ divsb, float4* __restrict__ tbar, float4* __restrict__ tbar2,
                double* __restrict__ block_part, int n) {
    __shared__ int s_list[kListCap][kPassThreads];
    __shared__ double s_red[ADJ_NPARAM][kPassThreads / 32];
    const int tid = threadIdx.x;
    const int s = blockIdx.x * blockDim.x + tid;
    const bool valid = s < n;
    const DevGrid g = *gp;
    const bool ah = P.heat_art != 0;
    const bool vs = P.visc != 0;
    const int it = valid ? B.itype[s] : 0;
    const bool work = valid && g.ok && it > 0;
    // walls take part for artificial heat (their psi enters their neighbours'
    // energy rates) and physical viscosity (their tau, their neighbours' forces)
    const bool act = valid && g.ok && (it > 0 || ah || vs);
    float4 xi = make_float4(0.f, 0.f, 0.f, 1.f), vi = xi, rpi = xi, abi = make_float4(0.f, 0.f, 0.f, 0.f);
    float pi = 0.f, uloi = 0.f;
    if (act) {
        xi = B.xh[s];
        vi = B.vm[s];
        rpi = B.rp[s];
        pi = B.p[s];
        if (work) abi = abar[s];
        if (ah && B.ulo) uloi = B.ulo[s];
    }
    const float mi = mass_of<DIM>(xi, vi);
    CellCoord cc = {{0, 0, 0}};
    if (act) cc = decode_key<DIM>(keys[s], g);
    float4 tai = make_float4(0.f, 0.f, 0.f, 0.f), tbi = tai;  // tau_i
    float4 tba = tai, tbb = tai;                              // tau_bar_i
    if (act && vs) {
        tai = B.tau[s];
        if (DIM == 3) tbi = B.tau2[s];
    }
    float xb[3] = {0.f, 0.f, 0.f}, vb[3] = {0.f, 0.f, 0.f}, Pb = 0.f, rb = 0.f;
    float psib = 0.f, uhb = 0.f;  // artificial heat: psi_bar, u_half_bar of this particle
    // parameter cotangents, float-float (hi in pa, rounding residuals in palo):
    // pair terms of both signs cancel in these sums
    float pa[ADJ_NPARAM] = {0.f, 0.f, 0.f, 0.f}, palo[ADJ_NPARAM] = {0.f, 0.f, 0.f, 0.f};
    auto pacc = [&](int q, float v) {
        const sph::ff t = sph::two_sum(pa[q], v);
        pa[q] = t.hi;
        palo[q] += t.lo;
    };
    NbrStream<DIM> ns;
    nbr_init<DIM>(ns, B, g, s, act, work);
    while (__any_sync(0xffffffffu, !ns.done)) {
        const int nl = nbr_fill<DIM>(ns, B, g, start, cc, xi, s, s_list);
        const int ml = __reduce_max_sync(0xffffffffu, nl);
        for (int t = 0; t < ml; ++t) {
            if (t >= nl) continue;
            const int j = s_list[t][tid];
            const float4 xj = __ldg(B.xh + j);
            const float4 vj = __ldg(B.vm + j);
            const float4 rpj = __ldg(B.rp + j);
            const float4 abj = __ldg(abar + j);
            const float mj = mass_of<DIM>(xj, vj);
            PairGeo<DIM> pg;
            pair_geo<DIM>(xi, xj, g, P, pg);
            const float rho_bar = 0.5f * (rpi.x + rpj.x);
            float w[3] = {vj.x - vi.x, vj.y - vi.y, DIM == 3 ? vj.z - vi.z : 0.f};
            PairAdj o;
            if (work) {
                // Pair (s, j): the rates of s.
                pair_adjoint<DIM>(pg.d, w, pg.dr2, pg.G, pg.dGdr_r, pg.mh, rho_bar, rpi.y, rpj.y,
                                  mj, abi, P, o);
#pragma unroll
                for (int k = 0; k < DIM; ++k) {
                    xb[k] += o.db[k];
                    vb[k] -= o.wb[k];
                }
                Pb += o.Pb;
                rb += o.rb;
                pacc(ADJ_ALPHA, o.al);
                pacc(ADJ_BETA, o.be);
                pacc(ADJ_C0, o.c0);
                // Pair (j, s): the rates of j (zero cotangents for walls).
                if (abj.x != 0.f || abj.y != 0.f || abj.z != 0.f || abj.w != 0.f) {
                    float dn[3] = {-pg.d[0], -pg.d[1], -pg.d[2]};
                    float wn[3] = {-w[0], -w[1], -w[2]};
                    pair_adjoint<DIM>(dn, wn, pg.dr2, pg.G, pg.dGdr_r, pg.mh, rho_bar, rpj.y,
                                      rpi.y, mi, abj, P, o);
#pragma unroll
                    for (int k = 0; k < DIM; ++k) {
                        xb[k] -= o.db[k];
                        vb[k] += o.wb[k];
                    }
                    Pb += o.Pb;
                    rb += o.rb;
                }
            }
            if (ah) {
                // du_s and du_j terms m (psi_s + psi_j) A (u_s - u_j), A(r^2):
                // weights du_bar_s m_j - du_bar_j m_s on the pair (s, j).
                const float e = pg.mh * pg.mh * P.ah_eta2;
                const float den = rho_bar * (e + pg.dr2);
                const float A = pg.G * pg.dr2 / den;
                const float dAds = (0.5f * pg.dGdr_r * pg.dr2 + pg.G) / den - A / (e + pg.dr2);
                const float ps = rpi.w + rpj.w;
                const float ulj = B.ulo ? __ldg(B.ulo + j) : 0.f;
                const float du = (rpi.z - rpj.z) + (uloi - ulj);
                const float cdu = abi.w * mj - abj.w * mi;
                psib = fmaf(A * du, cdu, psib);
                uhb = fmaf(ps * A, cdu, uhb);
                rb -= 0.5f * ps * A * du * cdu / rho_bar;
                const float cx = 2.f * dAds * ps * du * cdu;
#pragma unroll
                for (int k = 0; k < DIM; ++k) xb[k] = fmaf(cx, pg.d[k], xb[k]);
            }
            if (vs) {
                // a_s += m_j (tau_s + tau_j) w, a_j += m_s (tau_j + tau_s) (-w), w = G d:
                // cotangent b = m_j a_bar_s - m_s a_bar_j on (tau_s + tau_j) w.
                const float4 taj = __ldg(B.tau + j);
                float4 tbj = make_float4(0.f, 0.f, 0.f, 0.f);
                if (DIM == 3) tbj = __ldg(B.tau2 + j);
                const float bv[3] = {mj * abi.x - mi * abj.x, mj * abi.y - mi * abj.y,
                                     DIM == 3 ? mj * abi.z - mi * abj.z : 0.f};
                const float w0 = pg.G * pg.d[0], w1 = pg.G * pg.d[1];
                const float w2 = (DIM == 3) ? pg.G * pg.d[2] : 0.f;
                tba.x = fmaf(bv[0], w0, tba.x);
                tba.y = fmaf(bv[1], w1, tba.y);
                tba.z += bv[0] * w1 + bv[1] * w0;
                if (DIM == 3) {
                    tba.w = fmaf(bv[2], w2, tba.w);
                    tbb.x += bv[0] * w2 + bv[2] * w0;
                    tbb.y += bv[1] * w2 + bv[2] * w1;
                }
                if (work) {  // d_bar = J u, u = (tau_s + tau_j) b, J = G I + (G'/r) d d^T
                    const float4 sa = make_float4(tai.x + taj.x, tai.y + taj.y, tai.z + taj.z,
                                                  tai.w + taj.w);
                    const float4 sb = make_float4(tbi.x + tbj.x, tbi.y + tbj.y, 0.f, 0.f);
                    float u[3];
                    sym_apply<DIM>(sa, sb, bv, u);
                    float du_ = u[0] * pg.d[0] + u[1] * pg.d[1];
                    if (DIM == 3) du_ += u[2] * pg.d[2];
#pragma unroll
                    for (int k = 0; k < DIM; ++k)
                        xb[k] += pg.G * u[k] + pg.dGdr_r * du_ * pg.d[k];
                }
            }
        }
    }
    if (act && vs) {
        // tau = sc T, sc = eta / rho^2; du += tds = eta/(2 rho) T:T (fluid only).
        const float rho = rpi.x;
        const float sc = P.eta / (rho * rho);
        const float isc = P.eta != 0.f ? 1.f / sc : 0.f;
        const float4 Ta = make_float4(tai.x * isc, tai.y * isc, tai.z * isc, tai.w * isc);
        const float4 Tb = make_float4(tbi.x * isc, tbi.y * isc, 0.f, 0.f);
        const float tdsb = work ? abi.w : 0.f;
        const float k = tdsb * P.eta / rho;  // d tds / d T_aa = eta/rho T_aa, off-diagonal 2x
        float4 Ga = make_float4(fmaf(sc, tba.x, k * Ta.x), fmaf(sc, tba.y, k * Ta.y),
                                fmaf(sc, tba.z, 2.f * k * Ta.z), 0.f);
        float4 Gb = make_float4(0.f, 0.f, 0.f, 0.f);
        float q = Ta.x * Ta.x + Ta.y * Ta.y + 2.f * Ta.z * Ta.z;
        float tt = tba.x * tai.x + tba.y * tai.y + tba.z * tai.z;
        if (DIM == 3) {
            Ga.w = fmaf(sc, tba.w, k * Ta.w);
            Gb = make_float4(fmaf(sc, tbb.x, 2.f * k * Tb.x), fmaf(sc, tbb.y, 2.f * k * Tb.y), 0.f,
                             0.f);
            q += Ta.w * Ta.w + 2.f * (Tb.x * Tb.x + Tb.y * Tb.y);
            tt += tba.w * tai.w + tbb.x * tbi.x + tbb.y * tbi.y;
        }
        if (work) rb += -2.f * tt / rho - tdsb * 0.5f * P.eta * q / (rho * rho);
        tbar[s] = Ga;
        if (DIM == 3) tbar2[s] = Gb;
    } else if (valid && vs) {
        tbar[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (DIM == 3) tbar2[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float dsb = 0.f;  // cotangent of the divergence sum (artificial heat)
    if (act && ah) {
        // psi = g1 h c0 + g2 h^2 (|divv| - divv), divv = divs / rho: divv from psi
        const float h = xi.w, base = P.ah_g1 * h * P.c0;
        pacc(ADJ_C0, psib * P.ah_g1 * h);
        if (P.ah_g2 != 0.f && rpi.w > base) {  // divv < 0
            const float k2 = 2.f * P.ah_g2 * h * h;
            const float divv = -(rpi.w - base) / k2;
            const float divvb = -k2 * psib;
            dsb = divvb / rpi.x;
            if (work) rb -= divvb * divv / rpi.x;
        }
    }
    if (work) {
        const float rho = rpi.x;
        if (S.heat_on) {  // du += q0 exp(-|x - xc|^2 k) / rho
            const float e0 = xi.x - P.heat_center[0], e1 = xi.y - P.heat_center[1];
            const float e2 = (DIM == 3) ? xi.z - P.heat_center[2] : 0.f;
            const float ex = expf(-(e0 * e0 + e1 * e1 + e2 * e2) * P.heat_k);
            const float dub = abi.w;
            pacc(ADJ_Q0, dub * ex / rho);
            rb -= dub * P.heat_q0 * ex / (rho * rho);
            const float gx = -2.f * P.heat_k * dub * P.heat_q0 * ex / rho;
            xb[0] += gx * e0;
            xb[1] += gx * e1;
            if (DIM == 3) xb[2] += gx * e2;
        }
        // Tait EOS and P = p/rho^2 (the clamp p < pmin sets constants: no gradient).
        const bool clamped = (P.pmin > -FLT_MAX) && pi == 0.f && rho == P.rho0;
        float rtot = 0.f;
        if (!clamped) {
            const float pb = Pb / (rho * rho) + pbar_loss[s];
            const float ratio = rho * P.inv_rho0;
            const float r3 = ratio * ratio * ratio;
            rtot = rb - 2.f * Pb * pi / (rho * rho * rho) + pb * P.c0 * P.c0 * r3 * r3;
            if (P.c0 > 0.f) pacc(ADJ_C0, pb * 2.f * pi / P.c0);
        }
        rhobar[s] = rtot;
        xF[s] = make_float4(xb[0], xb[1], xb[2], 0.f);
        // .w: u_half_bar (the predicted energy of artificial heat)
        vhb[s] = make_float4(vb[0], vb[1], vb[2], ah ? uhb : 0.f);
    } else if (valid) {
        rhobar[s] = 0.f;
        xF[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        vhb[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (valid && divsb) divsb[s] = dsb;
    // Deterministic per-block partial sums of the parameter cotangents, in
    // double (a fixed shuffle order, then the warps in order).
#pragma unroll
    for (int q = 0; q < ADJ_NPARAM; ++q) {
        double v = (double)pa[q] + (double)palo[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) s_red[q][tid >> 5] = v;
    }
    __syncthreads();
    if (tid < ADJ_NPARAM) {
        double v = 0.0;
        for (int w2 = 0; w2 < kPassThreads / 32; ++w2) v += s_red[tid][w2];
        block_part[blockIdx.x * ADJ_NPARAM + tid] = v;
    }
}

// Shear-tensor reverse (physical viscosity): T_j = sum_k m_k/rho_k H(vh_k - vh_j,
// G_jk d_jk) for every particle j, cotangents tbar. For a fluid particle i the
// pair (i, j) enters T_i (weight m_j/rho_j) and T_j (weight m_i/rho_i, with
// dv and w both reversed: the same H): with Ab = m_j/rho_j tbar_i + m_i/rho_i
// tbar_j, vh_bar_i -= M(Ab) w, x_bar_i += J M(Ab) dv, and rho_i's weight in T_j
// gives rho_bar_i -= m_i/rho_i^2 dv^T M(tbar_j) w. Added to the force reverse's
// cotangents of i (the density's where the Tait clamp did not bind).
template <int DIM>
__global__ void __launch_bounds__(kPassThreads)
    k_adj_shear(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
                const DevGrid* __restrict__ gp, DevParams P, const float4* __restrict__ tbar,
                const float4* __restrict__ tbar2, float* __restrict__ rhobar,
                float4* __restrict__ xF, float4* __restrict__ vhb, int n) {
    __shared__ int s_list[kListCap][kPassThreads];
    const int tid = threadIdx.x;
    const int s = blockIdx.x * blockDim.x + tid;
    const bool valid = s < n;
    const DevGrid g = *gp;
    const bool work = valid && g.ok && B.itype[s] > 0;
    float4 xi = make_float4(0.f, 0.f, 0.f, 1.f), vi = xi;
    float4 tai = make_float4(0.f, 0.f, 0.f, 0.f), tbi = tai;
    float rhoi = 1.f;
    if (work) {
        xi = B.xh[s];
        vi = B.vm[s];
        rhoi = B.rp[s].x;
        tai = tbar[s];
        if (DIM == 3) tbi = tbar2[s];
    }
    const float mi = mass_of<DIM>(xi, vi);
    const float ci = mi / rhoi;
    CellCoord cc = {{0, 0, 0}};
    if (work) cc = decode_key<DIM>(keys[s], g);
    float xb[3] = {0.f, 0.f, 0.f}, vb[3] = {0.f, 0.f, 0.f}, rb = 0.f;
    NbrStream<DIM> ns;
    nbr_init<DIM>(ns, B, g, s, work);
    while (__any_sync(0xffffffffu, !ns.done)) {
        const int nl = nbr_fill<DIM>(ns, B, g, start, cc, xi, s, s_list);
        const int ml = __reduce_max_sync(0xffffffffu, nl);
        for (int t = 0; t < ml; ++t) {
            if (t >= nl) continue;
            const int j = s_list[t][tid];
            const float4 xj = __ldg(B.xh + j);
            const float4 vj = __ldg(B.vm + j);
            const float rhoj = __ldg(&B.rp[j].x);
            const float4 taj = __ldg(tbar + j);
            float4 tbj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (DIM == 3) tbj = __ldg(tbar2 + j);
            const float cj = mass_of<DIM>(xj, vj) / rhoj;
            PairGeo<DIM> pg;
            pair_geo<DIM>(xi, xj, g, P, pg);
            const float w[3] = {pg.G * pg.d[0], pg.G * pg.d[1], DIM == 3 ? pg.G * pg.d[2] : 0.f};
            const float dv[3] = {vj.x - vi.x, vj.y - vi.y, DIM == 3 ? vj.z - vi.z : 0.f};
            const float4 Aa = make_float4(cj * tai.x + ci * taj.x, cj * tai.y + ci * taj.y,
                                          cj * tai.z + ci * taj.z, cj * tai.w + ci * taj.w);
            const float4 Ab = make_float4(cj * tbi.x + ci * tbj.x, cj * tbi.y + ci * tbj.y, 0.f, 0.f);
            float4 ma, mb;
            shear_m<DIM>(Aa, Ab, ma, mb);
            float mw[3], mdv[3];
            sym_apply<DIM>(ma, mb, w, mw);
            sym_apply<DIM>(ma, mb, dv, mdv);
            float dmd = mdv[0] * pg.d[0] + mdv[1] * pg.d[1];
            if (DIM == 3) dmd += mdv[2] * pg.d[2];
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
                vb[k] -= mw[k];
                xb[k] += pg.G * mdv[k] + pg.dGdr_r * dmd * pg.d[k];
            }
            float4 mja, mjb;
            shear_m<DIM>(taj, tbj, mja, mjb);
            float mjw[3];
            sym_apply<DIM>(mja, mjb, w, mjw);
            float h = dv[0] * mjw[0] + dv[1] * mjw[1];
            if (DIM == 3) h += dv[2] * mjw[2];
            rb -= mi / (rhoi * rhoi) * h;
        }
    }
    if (!work) return;
    // the Tait clamp (p < pmin) set rho_i = rho0: no gradient reaches the sum
    const bool clamped = (P.pmin > -FLT_MAX) && B.p[s] == 0.f && rhoi == P.rho0;
    if (!clamped) rhobar[s] += rb;
    float4 f = xF[s];
    f.x += xb[0];
    f.y += xb[1];
    f.z += xb[2];
    xF[s] = f;
    float4 v = vhb[s];
    v.x += vb[0];
    v.y += vb[1];
    v.z += vb[2];
    vhb[s] = v;
}

// Density reverse (rho_i = m_i W(0) + sum m_j W_ij), the reverse of the
// divergence sums of artificial heat (divs_i = sum_j m_j G_ij (vh_j - vh_i) .
// d_ij, cotangents divsb), assembly, scatter to the slot order of the step's
// input (perm: cell slot -> input slot).
template <int DIM>
__global__ void __launch_bounds__(kPassThreads)
    k_adj_density(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
                  const DevGrid* __restrict__ gp, DevParams P, StepArgs S,
                  const float* __restrict__ rhobar, const float4* __restrict__ xF,
                  const float4* __restrict__ vhb, const float4* __restrict__ xpart,
                  const float4* __restrict__ vpart, const float* __restrict__ divsb,
                  const int* __restrict__ perm, AdjState Gp, int n) {
    __shared__ int s_list[kListCap][kPassThreads];
    const int tid = threadIdx.x;
    const int s = blockIdx.x * blockDim.x + tid;
    const bool valid = s < n;
    const DevGrid g = *gp;
    const bool work = valid && g.ok && B.itype[s] > 0;
    float4 xi = make_float4(0.f, 0.f, 0.f, 1.f), vi = xi;
    float rbi = 0.f;
    if (work) {
        xi = B.xh[s];
        vi = B.vm[s];
        rbi = rhobar[s];
    }
    const float mi = mass_of<DIM>(xi, vi);
    CellCoord cc = {{0, 0, 0}};
    if (work) cc = decode_key<DIM>(keys[s], g);
    const bool ah = P.heat_art != 0 && divsb != nullptr;
    const float dsi = (work && ah) ? divsb[s] : 0.f;
    float xb[3] = {0.f, 0.f, 0.f}, vdb[3] = {0.f, 0.f, 0.f};
    NbrStream<DIM> ns;
    nbr_init<DIM>(ns, B, g, s, work);
    while (__any_sync(0xffffffffu, !ns.done)) {
        const int nl = nbr_fill<DIM>(ns, B, g, start, cc, xi, s, s_list);
        const int ml = __reduce_max_sync(0xffffffffu, nl);
        for (int t = 0; t < ml; ++t) {
            if (t >= nl) continue;
            const int j = s_list[t][tid];
            const float4 xj = __ldg(B.xh + j);
            float4 vj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (DIM == 3 || ah) vj = __ldg(B.vm + j);
            const float mj = mass_of<DIM>(xj, vj);
            const float rbj = __ldg(rhobar + j);
            PairGeo<DIM> pg;
            pair_geo<DIM>(xi, xj, g, P, pg);
            const float c = (rbi * mj + rbj * mi) * pg.G;
#pragma unroll
            for (int k = 0; k < DIM; ++k) xb[k] = fmaf(c, pg.d[k], xb[k]);
            if (ah) {
                // d/d(vh_s), d/d(x_s) of divs_s (weight dsb_s m_j) and of divs_j
                // (weight dsb_j m_s, d_js = -d, w_js = -w): the same forms.
                const float cd = dsi * mj + __ldg(divsb + j) * mi;
                const float w[3] = {vj.x - vi.x, vj.y - vi.y, DIM == 3 ? vj.z - vi.z : 0.f};
                float wd = w[0] * pg.d[0] + w[1] * pg.d[1];
                if (DIM == 3) wd += w[2] * pg.d[2];
#pragma unroll
                for (int k = 0; k < DIM; ++k) {
                    vdb[k] = fmaf(-cd * pg.G, pg.d[k], vdb[k]);
                    xb[k] = fmaf(cd, pg.G * w[k] + pg.dGdr_r * pg.d[k] * wd, xb[k]);
                }
            }
        }
    }
    if (!valid) return;
    float4 gx = make_float4(0.f, 0.f, 0.f, 0.f), gv = gx, ga = gx;
    if (work) {
        const float4 xp = xpart[s], f = xF[s], vp = vpart[s];
        float4 vh = vhb[s];
        vh.x += vdb[0];
        vh.y += vdb[1];
        vh.z += vdb[2];
        // u_half = max(0, u + hdt du_prev): no gradient where it clamped to 0
        const float uh = (ah && B.rp[s].z != 0.f) ? vh.w : 0.f;
        gx = make_float4(xp.x + f.x + xb[0], xp.y + f.y + xb[1], xp.z + f.z + xb[2], 0.f);
        // predictor: vh = v + hdt a_prev (v_bar gets vh_bar; a_prev_bar = hdt vh_bar)
        gv = make_float4(vp.x + vh.x, vp.y + vh.y, vp.z + vh.z, vp.w + uh);
        ga = make_float4(S.hdt * vh.x, S.hdt * vh.y, S.hdt * vh.z, S.hdt * uh);
    }
    const int j = perm[s];
    Gp.xb[j] = gx;
    Gp.vb[j] = gv;
    Gp.ab[j] = ga;
}

// Adds the step's parameter cotangents (block partials, fixed order) to acc.
__global__ void __launch_bounds__(256)
    k_adj_params(const double* __restrict__ block_part, int nblocks, double* __restrict__ acc) {
    __shared__ double s[ADJ_NPARAM][256];
    for (int q = 0; q < ADJ_NPARAM; ++q) {
        double v = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v += block_part[b * ADJ_NPARAM + q];
        s[q][threadIdx.x] = v;
    }
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int q = 0; q < ADJ_NPARAM; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < ADJ_NPARAM) acc[threadIdx.x] += s[threadIdx.x][0];
}

}  // namespace ag
