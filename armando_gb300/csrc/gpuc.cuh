// gpuc.cuh -- the GPU-C step variant (armando_params.scheme 1 and 2).
//
// Third-order TVD Runge-Kutta with continuity density and one neighbour list
// per step, as the GPU-C codes run it (ArmandoThrust/acpu.c:2338-2379):
// X = X0 + alpha (X + dt dX/dt - X0) for alpha = 1, 1/4, 2/3. Pair rates:
//   scheme 1, the host path (acpu.c:346-437): every listed pair contributes
//     continuity m_j (x_ij . v_ij) W'/r, pressure -(p_i + p_j)/(rho_i rho_j),
//     the shock corrections of mass and momentum, and between different
//     itype a push 0.02 (W/W0) c_i c_j / r scaled by m_j/(m_i + m_j);
//   scheme 2, the device kernels (armando.cu:429-513): the same terms, with
//     pressure -(p_i/rho_i^2 + p_j/rho_j^2), for pairs of equal itype only;
//     pairs of different itype push 0.5 W m_j/(rho_j h_j) c_j^2.
// Energy: de/dt = p drho/dt / rho^2 (acpu.c:510-534); gravity and the load
// zones on itype > 0 (acpu.c:1047-1076); fix zones after the update.
// Update and EOS per material |itype| (acpu.c:873-966, armando.cu:987-1074).
// Kernels with h_i. The list of a step holds the j != i with
// sqrtf(|x0_i - x0_j|^2) < 2 h_i at the step's start (updateListHost,
// acpu.c:2201-2240), without the reference's 21-entry cap; each stage tests
// the candidates of the step's cell grid against the start positions (kept
// for the step anyway) and evaluates the physics at the stage's positions.
//
// State in cell order: the step's start (x0, v0, rho0/u0) and two working
// copies {x, v, (rho, u, p, c)} that the stages ping-pong between; the last
// stage's rates go out as dv/dt, de/dt.
#pragma once
#include "kernels.cuh"

namespace ag {

struct DevMaterial {
    int type;  // 0 boundary, 1 ideal gas, 2 polynomial, 3 shock, 4 Tait, 5 ESS
    float prop[10];
};

// Load and fix zones (acpu.c:33-48; armando.cu:43-58): open boxes lo < x < hi,
// x and y only in 2D (armando2D.cu:756-762).
struct DevLoadZone {
    float lo[3], hi[3], g[3], w;
};
struct DevFixZone {
    float lo[3], hi[3], v[3];
    float tau;  // 0: fix zone (velocity set after the update); > 0: pump zone (a rate)
};
struct DevZones {
    int n_load, n_fix;
    DevLoadZone load[10];
    DevFixZone fix[10];
};

template <int DIM>
__device__ __forceinline__ bool in_zone(const float* lo, const float* hi, const float4& x) {
    bool in = x.x > __ldg(lo) && x.x < __ldg(hi) && x.y > __ldg(lo + 1) && x.y < __ldg(hi + 1);
    if (DIM == 3) in = in && x.z > __ldg(lo + 2) && x.z < __ldg(hi + 2);
    return in;
}

struct GpucState {
    float4* x0;    // {x, y, m, h} (2D) / {x, y, z, h} (3D) at the step's start
    float4* v0;    // {v, -} (2D) / {v, m} (3D)
    float2* q0;    // {rho, u} at the step's start
    float4* xw[2];
    float4* vw[2];
    float4* sw[2];  // {rho, u, p, c}
    float4* rates;  // {dv/dt, de/dt} of the last stage
    int* itype;
    int* id;
    float4* xsort;  // lazy sorting: positions at the last sort (nullptr: every step sorts)
};

// The EOS of one particle after its update (acpu.c:932-962 with the property
// functions of acpu.c:560-870; ESS of Code/armando.cu:572-598 on absolute
// density). rho is clamped where the type clamps.
__device__ __forceinline__ void gpuc_eos(const DevMaterial& M, float& rho, float u, float& p, float& c) {
    const float* q = M.prop;
    switch (M.type) {
    case 0:  // boundary
        if (rho < 0.9f * q[0]) rho = 0.9f * q[0];
        p = 0.f;
        c = q[1];
        break;
    case 1:  // ideal gas
        p = __fadd_rn(__fmul_rn(__fmul_rn(q[1] - 1.0f, rho), u), q[2]);
        c = sqrtf(__fmul_rn(__fmul_rn(q[1], q[1] - 1.0f), u));
        break;
    case 2: {  // Mie-Gruneisen polynomial
        if (rho < 0.9f * q[0]) rho = 0.9f * q[0];
        const float mu = __fdiv_rn(rho - q[0], q[0]);
        const float mu2 = __fmul_rn(mu, mu);
        if (mu < 0.f)
            p = __fadd_rn(__fadd_rn(__fmul_rn(q[6], mu), __fmul_rn(q[7], mu2)),
                          __fmul_rn(__fmul_rn(q[4], q[0]), u));
        else
            p = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(q[1], mu), __fmul_rn(q[2], mu2)),
                                    __fmul_rn(q[3], __fmul_rn(mu2, mu))),
                          __fmul_rn(__fmul_rn(__fadd_rn(q[4], __fmul_rn(q[5], mu)), q[0]), u));
        c = sqrtf(__fdiv_rn(q[1], rho));
        break;
    }
    case 3: {  // Mie-Gruneisen shock
        if (rho < 0.9f * q[0]) rho = 0.9f * q[0];
        const float mu = __fdiv_rn(rho - q[0], q[0]);
        const float den = __fsub_rn(1.0f, __fmul_rn(q[3] - 1.0f, mu));
        const float ph = __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(q[0], __fmul_rn(q[1], q[1])), mu),
                                             1.0f + mu),
                                   __fmul_rn(den, den));
        const float corr = __fmul_rn(__fdiv_rn(__fmul_rn(0.5f, ph), q[0]), __fdiv_rn(mu, 1.0f + mu));
        p = __fadd_rn(ph, __fmul_rn(__fmul_rn(q[2], q[0]), __fsub_rn(u, corr)));
        c = q[1];
        break;
    }
    case 4: {  // Tait
        if (rho < 0.9f * q[0]) rho = 0.9f * q[0];
        const float r = __fdiv_rn(rho, q[0]);
        const float r2 = __fmul_rn(r, r), r4 = __fmul_rn(r2, r2);
        const float r7 = __fmul_rn(__fmul_rn(r4, r2), r);
        p = __fmul_rn(__fdiv_rn(__fmul_rn(q[0], __fmul_rn(q[1], q[1])), 7.0f), r7 - 1.0f);
        c = q[1];
        break;
    }
    case 5: {  // ESS
        const float mu = __fdiv_rn(rho, q[0]) - 1.0f;
        p = __fadd_rn(__fmul_rn(__fmul_rn(mu, q[0]), __fmul_rn(q[1], q[1])),
                      __fmul_rn(__fmul_rn(u, q[0]), q[2]));
        if (p < q[3]) p = q[3];
        c = q[1];
        break;
    }
    default:
        p = 0.f;
        break;
    }
}

__device__ __forceinline__ int gpuc_material(int itype, int n_mat, unsigned* flags) {
    const int k = itype < 0 ? -itype : itype;
    if (k >= n_mat) {
        atomicOr(flags, (unsigned)FLAG_BAD_MATERIAL);
        return 0;
    }
    return k;
}

// Cell order of the step: start state, first working copy, sound speeds.
// A is in the cell order of the last sort, so a step that does not sort
// (lazy sorting) takes it slot for slot.
template <int DIM>
__global__ void k_gpuc_gather(StateA A, const int* __restrict__ perm, GpucState S,
                              const DevMaterial* __restrict__ mat, int n_mat,
                              unsigned* __restrict__ flags, int n,
                              const int* __restrict__ resort = nullptr) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const bool sorted = !sort_skipped(resort);
    const int j = sorted ? perm[s] : s;
    const float4 xh = A.xh[j], vm = A.vm[j];
    if (sorted && S.xsort) S.xsort[s] = xh;
    const int it = A.itype[j];
    float rho = A.rho[j];
    const float u = A.u[j], p = A.p[j];
    float pp = 0.f, c = 0.f, r = rho;
    gpuc_eos(mat[gpuc_material(it, n_mat, flags)], r, u, pp, c);  // Sound of the last update
    S.x0[s] = xh;
    S.v0[s] = vm;
    S.q0[s] = make_float2(rho, u);
    S.xw[0][s] = xh;
    S.vw[0][s] = vm;
    S.sw[0][s] = make_float4(rho, u, p, c);
    S.itype[s] = it;
    S.id[s] = A.id[j];
}

// Wendland C2 with h_i as the GPU-C codes evaluate it (acpu.c:146-201):
// W = K/h^dim (1 - q/2)^4 (1 + 2q), dW/dr = K/h^(dim+1) 5/8 q (q - 2)^3.
// The particle's factors: ih = 1/h, alpha = K/h^dim (as K ih^dim).
template <int DIM>
__device__ __forceinline__ void gpuc_kernel_norm(float h, float K, float& ih, float& alpha) {
    ih = __frcp_rn(h);
    alpha = DIM == 2 ? __fmul_rn(K, __fmul_rn(ih, ih)) : __fmul_rn(K, __fmul_rn(__fmul_rn(ih, ih), ih));
}

template <int DIM>
__device__ __forceinline__ void gpuc_kernel(float r, float h, float ih, float alpha, float& w,
                                            float& dwdr) {
    const float q = __fdiv_rn(r, h);
    w = 0.f;
    dwdr = 0.f;
    if (!(q < 2.f)) return;
    float t = fmaf(-0.5f, q, 1.0f);
    t = __fmul_rn(t, t);
    t = __fmul_rn(t, t);
    w = __fmul_rn(__fmul_rn(t, fmaf(2.0f, q, 1.0f)), alpha);
    const float qm2 = q - 2.0f;
    dwdr = __fmul_rn(__fmul_rn(__fmul_rn(0.625f, q), __fmul_rn(__fmul_rn(qm2, qm2), qm2)),
                     __fmul_rn(alpha, ih));
}

// The smallest t with sqrt_rn(t) >= lim, so that sqrt_rn(r2) < lim exactly when
// r2 < t (sqrt_rn is monotone): updateListHost's test without a square root
// per candidate. lim^2 rounded lies within one step of t (checked on random
// FP32 lims over [1e-30, 1e19] against IEEE square roots, in the CPU tests);
// the loops allow four. lim <= 0 or NaN: no r2 passes.
__device__ __forceinline__ float sqrt_less_bound(float lim) {
    if (!(lim > 0.f)) return -INFINITY;
    float t = __fmul_rn(lim, lim);
    if (isinf(t)) return t;  // every finite r2 has sqrt_rn(r2) < lim
#pragma unroll 1
    for (int q = 0; q < 4 && __fsqrt_rn(t) < lim; ++q) t = nextafterf(t, INFINITY);
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const float d = nextafterf(t, 0.f);
        if (!(__fsqrt_rn(d) >= lim)) break;
        t = d;
    }
    return t;
}

// Neighbours a lane collects before it evaluates them (a longer list is
// evaluated in pieces of this length): about the lane's share of the 2D / 3D
// neighbours, at least 8, within 48 KB of static shared memory per CTA.
template <int DIM, int TPP, int BS>
__host__ __device__ constexpr int gpuc_list_len() {
    constexpr int want = (DIM == 2 ? 32 : 64) / TPP < 8 ? 8 : (DIM == 2 ? 32 : 64) / TPP;
    return want * BS * 4 > 48 * 1024 ? 48 * 1024 / (4 * BS) : want;
}

// One RK3 stage: rates of every particle from working copy `cur`, update into
// `nxt` (X0 + alpha (X + dt dX/dt - X0)), EOS. VAR 1: host path, 2: device.
// TPP lanes per particle split its candidates (lane `sub` takes slots
// k0 + sub, k0 + sub + TPP, ... of every cell range) and sum their rates with
// an xor butterfly; lane 0 updates. TPP = 1 sums in candidate order. Each lane
// first lists the candidates that pass the start-position test (in shared
// memory, candidate order kept) and then evaluates the list, so the lanes of a
// warp run the pair physics together instead of idling through candidates.
template <int DIM, int VAR, int TPP = 1, int BS = kPassThreads>
__global__ void __launch_bounds__(BS)
    k_gpuc_stage(GpucState S, int cur, const unsigned* __restrict__ keys,
                 const int* __restrict__ start, const DevGrid* __restrict__ gp, DevParams P,
                 const DevMaterial* __restrict__ mat, int n_mat, const DevZones* __restrict__ zones,
                 unsigned* __restrict__ flags, float alpha, float dt, int n) {
    const int i = blockIdx.x * (BS / TPP) + (int)threadIdx.x / TPP;
    const int sub = (TPP == 1) ? 0 : (int)(threadIdx.x & (TPP - 1));
    if (i >= n) return;  // whole groups: the lanes of a particle share i
    const DevGrid g = *gp;
    // working copies picked without indexing the parameter arrays (no stack)
    const float4* __restrict__ xc = cur ? S.xw[1] : S.xw[0];
    const float4* __restrict__ vc = cur ? S.vw[1] : S.vw[0];
    const float4* __restrict__ sc = cur ? S.sw[1] : S.sw[0];
    float4* __restrict__ xo = cur ? S.xw[0] : S.xw[1];
    float4* __restrict__ vo = cur ? S.vw[0] : S.vw[1];
    float4* __restrict__ so = cur ? S.sw[0] : S.sw[1];
    const float4 x0i = S.x0[i];
    const float4 xi = xc[i], vi = vc[i], si = sc[i];
    const int it = S.itype[i];
    const float hi = x0i.w;
    const float mi = (DIM == 2) ? x0i.z : S.v0[i].w;
    const float r2_bound = sqrt_less_bound(__fmul_rn(2.0f, hi));
    float ih, kal;
    gpuc_kernel_norm<DIM>(hi, P.kw_hi, ih, kal);
    float w0, d0;
    gpuc_kernel<DIM>(0.f, hi, ih, kal, w0, d0);
    // the device variant's own pressure term (armando.cu:483-485)
    const float p_i = (VAR == 2) ? __fdiv_rn(si.z, __fmul_rn(si.x, si.x)) : 0.f;
    float rd = 0.f, a0 = 0.f, a1 = 0.f, a2 = 0.f;
    auto pair = [&](int k) {
        const float4 xk = __ldg(xc + k), vk = __ldg(vc + k);
        const float4 sk = __ldg(sc + k);
        const int itk = __ldg(S.itype + k);
        const float dx = xi.x - xk.x, dy = xi.y - xk.y, dz = (DIM == 3) ? xi.z - xk.z : 0.f;
        const float dr = __fsqrt_rn(fmaf(dz, dz, fmaf(dy, dy, __fmul_rn(dx, dx))));
        if (dr < __fmul_rn(0.01f, hi)) return;  // dr := 100 h: W = dW/dr = 0 (acpu.c:379)
        float w, dwdr;
        gpuc_kernel<DIM>(dr, hi, ih, kal, w, dwdr);
        const float mk = mass_of<DIM>(xk, vk);  // the working copies carry m and h
        const float dvr = fmaf(dz, vi.z - vk.z, fmaf(dy, vi.y - vk.y, __fmul_rn(dx, vi.x - vk.x)));
        const float rhoi = si.x, rhok = sk.x;
        const float ir = __fdiv_rn(1.0f, dr);
        float f = 0.f;  // times dW/dr along (x_i - x_k)/dr
        const bool same = it == itk;
        if (VAR == 1 || same) {
            rd = fmaf(__fmul_rn(mk, dvr), __fmul_rn(dwdr, ir), rd);
            if (VAR == 1)
                f = __fmul_rn(mk, __fdiv_rn(-(si.z + sk.z), __fmul_rn(rhoi, rhok)));
            else
                f = __fmul_rn(mk, -(p_i + __fdiv_rn(sk.z, __fmul_rn(rhok, rhok))));
            const float cs = __fdiv_rn(__fmul_rn(2.0f, si.w), rhoi + rhok);
            rd = fmaf(__fmul_rn(mk, __fmul_rn(rhoi - rhok, cs)), dwdr, rd);
            if (dvr < 0.f) {
                const float sh = __fdiv_rn(__fmul_rn(dvr, hi), fmaf(0.01f * hi, hi, __fmul_rn(dr, dr)));
                f = fmaf(mk, __fmul_rn(__fmul_rn(sh, cs), 0.03f), f);
            }
        }
        float push = 0.f;
        if (!same) {
            if (VAR == 1)
                push = __fmul_rn(__fdiv_rn(mk, mi + mk),
                                 __fdiv_rn(__fmul_rn(__fmul_rn(0.02f, __fdiv_rn(w, w0)), __fmul_rn(si.w, sk.w)), dr));
            else
                push = __fmul_rn(__fdiv_rn(__fdiv_rn(__fmul_rn(__fmul_rn(0.5f, w), mk), rhok), xk.w),
                                 __fmul_rn(sk.w, sk.w));
        }
        const float tot = __fmul_rn(fmaf(f, dwdr, push), ir);
        a0 = fmaf(tot, dx, a0);
        a1 = fmaf(tot, dy, a1);
        if (DIM == 3) a2 = fmaf(tot, dz, a2);
    };
    if (g.ok) {
        constexpr int ML = gpuc_list_len<DIM, TPP, BS>();
        __shared__ int s_list[ML][BS];
        const int tid = threadIdx.x;
        int nl = 0;
        const CellCoord cc = decode_key<DIM>(keys[i], g);
        Cursor cu = cursor_begin<DIM>(g);
        while (cursor_next<DIM>(g, start, cc, cu))
            for (int k = cu.k + sub; k < cu.ke; k += TPP) {
                if (k == i) continue;
                // updateListHost's test on the step's start positions
                const float4 x0k = __ldg(S.x0 + k);
                const float e0 = __fsub_rn(x0i.x, x0k.x), e1 = __fsub_rn(x0i.y, x0k.y);
                float r2 = __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1));
                if (DIM == 3) {
                    const float e2 = __fsub_rn(x0i.z, x0k.z);
                    r2 = __fadd_rn(r2, __fmul_rn(e2, e2));
                }
                if (!(r2 < r2_bound)) continue;
                s_list[nl++][tid] = k;
                if (nl == ML) {  // a full list: evaluate it and go on collecting
                    for (int q = 0; q < ML; ++q) pair(s_list[q][tid]);
                    nl = 0;
                }
            }
        for (int q = 0; q < nl; ++q) pair(s_list[q][tid]);
    }
    if (TPP > 1) {  // the particle's lanes reach this point together
        rd = group_sum<TPP>(rd);
        a0 = group_sum<TPP>(a0);
        a1 = group_sum<TPP>(a1);
        if (DIM == 3) a2 = group_sum<TPP>(a2);
        if (sub != 0) return;
    }
    // the start state, read after the pair loop (not held in registers across it)
    const float4 v0i = S.v0[i];
    const float2 q0 = S.q0[i];
    float wz = 0.f;
    if (it > 0) {  // updateLoadsHost: gravity over every fluid particle, then the zones
        float g0 = P.gravity[0], g1 = P.gravity[1], g2 = P.gravity[2];
        const int nl = __ldg(&zones->n_load);
#pragma unroll 1
        for (int q = 0; q < nl; ++q) {
            const DevLoadZone* Z = zones->load + q;
            if (!in_zone<DIM>(Z->lo, Z->hi, xi)) continue;
            g0 = __fadd_rn(g0, __ldg(&Z->g[0]));
            g1 = __fadd_rn(g1, __ldg(&Z->g[1]));
            g2 = __fadd_rn(g2, __ldg(&Z->g[2]));
            wz = __fadd_rn(wz, __ldg(&Z->w));
        }
        const int np = __ldg(&zones->n_fix);
#pragma unroll 1
        for (int q = 0; q < np; ++q) {  // pump zones: (vel - v) / tau (Code/armando.cu:1046-1055)
            const DevFixZone* Z = zones->fix + q;
            const float tau = __ldg(&Z->tau);
            if (!(tau > 0.f) || !in_zone<DIM>(Z->lo, Z->hi, xi)) continue;
            g0 = __fadd_rn(g0, __fdiv_rn(__fsub_rn(__ldg(&Z->v[0]), vi.x), tau));
            g1 = __fadd_rn(g1, __fdiv_rn(__fsub_rn(__ldg(&Z->v[1]), vi.y), tau));
            if (DIM == 3) g2 = __fadd_rn(g2, __fdiv_rn(__fsub_rn(__ldg(&Z->v[2]), vi.z), tau));
        }
        a0 += g0;
        a1 += g1;
        if (DIM == 3) a2 += g2;
    }
    // balanceEnergyHost on top of the loads' w
    const float du = __fadd_rn(wz, __fdiv_rn(__fmul_rn(si.z, rd), __fmul_rn(si.x, si.x)));
    S.rates[i] = make_float4(a0, a1, a2, du);
    float4 xn = xi, vn = vi, sn = si;
    if (VAR == 2 || it != 0) {  // acpu.c:894 leaves itype 0 alone
        xn.x = fmaf(alpha, fmaf(dt, vi.x, xi.x) - x0i.x, x0i.x);
        xn.y = fmaf(alpha, fmaf(dt, vi.y, xi.y) - x0i.y, x0i.y);
        if (DIM == 3) xn.z = fmaf(alpha, fmaf(dt, vi.z, xi.z) - x0i.z, x0i.z);
        vn.x = fmaf(alpha, fmaf(dt, a0, vi.x) - v0i.x, v0i.x);
        vn.y = fmaf(alpha, fmaf(dt, a1, vi.y) - v0i.y, v0i.y);
        if (DIM == 3) vn.z = fmaf(alpha, fmaf(dt, a2, vi.z) - v0i.z, v0i.z);
        float rho = fmaf(alpha, fmaf(dt, rd, si.x) - q0.x, q0.x);
        const float u = fmaf(alpha, fmaf(dt, du, si.y) - q0.y, q0.y);
        const DevMaterial& M = mat[gpuc_material(it, n_mat, flags)];
        if (VAR == 1 && it <= 0) {  // acpu.c:910-914
            vn.x = v0i.x;
            vn.y = v0i.y;
            if (DIM == 3) vn.z = v0i.z;
        }
        const int nf = __ldg(&zones->n_fix);
#pragma unroll 1
        for (int q = 0; q < nf; ++q) {  // fix zones at the new position
            const DevFixZone* Z = zones->fix + q;
            if (__ldg(&Z->tau) > 0.f || !in_zone<DIM>(Z->lo, Z->hi, xn)) continue;  // pumps: above
            vn.x = __ldg(&Z->v[0]);
            vn.y = __ldg(&Z->v[1]);
            if (DIM == 3) vn.z = __ldg(&Z->v[2]);
        }
        if (M.type == 0) {  // boundary materials keep their velocity
            vn.x = v0i.x;
            vn.y = v0i.y;
            if (DIM == 3) vn.z = v0i.z;
        }
        float p = 0.f, c = si.w;
        gpuc_eos(M, rho, u, p, c);
        sn = make_float4(rho, u, p, c);
        const float chk = xn.x + xn.y + xn.z + vn.x + vn.y + vn.z + rho + u + p;
        if (!isfinite(chk)) atomicOr(flags, (unsigned)FLAG_NONFINITE);
    }
    xo[i] = xn;
    vo[i] = vn;
    so[i] = sn;
}

// The step's result back to A (cell order of this step, like the force pass).
// Lazy sorting: a particle farther than half the skin from where it was binned
// makes the next step sort (the cells of the last sort hold every pair within
// 2 max(h) of the step's start positions only while none is).
template <int DIM>
__global__ void k_gpuc_scatter(GpucState S, int cur, StateA A, int n,
                               const DevGrid* __restrict__ gp = nullptr,
                               unsigned* __restrict__ flags = nullptr) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float4 sv = (cur ? S.sw[1] : S.sw[0])[s];
    const float4 xn = (cur ? S.xw[1] : S.xw[0])[s];
    if (S.xsort && gp && flags) {
        const float h2 = gp->half_skin2;
        const float4 xb = S.xsort[s];
        const float e0 = xn.x - xb.x, e1 = xn.y - xb.y, e2 = (DIM == 3) ? xn.z - xb.z : 0.f;
        if (h2 > 0.f && e0 * e0 + e1 * e1 + e2 * e2 > h2 && *(volatile unsigned*)(flags + 2) == 0u)
            atomicExch(flags + 2, 1u);
    }
    A.xh[s] = xn;
    A.vm[s] = (cur ? S.vw[1] : S.vw[0])[s];
    A.rho[s] = sv.x;
    A.u[s] = sv.y;
    A.p[s] = sv.z;
    A.ap[s] = S.rates[s];
    A.itype[s] = S.itype[s];
    A.id[s] = S.id[s];
}

}  // namespace ag

namespace ag {

// ---------------------------------------------------------------------------
// Open boundaries (armando.cu:2640-2856): outlets and the box remove particles,
// keeping the order of the rest (a block scan over tiles of kGhostTile).
// ---------------------------------------------------------------------------
struct DevOutlet {
    float o[3], n[3], R;
};

struct OpenSpec {
    DevOutlet out[10];
    int n_out;
    float lo[3], hi[3];
};

// checkOutDevice (armando.cu:2682-2722) in FP32, operations in order, unfused.
template <int DIM>
__device__ __forceinline__ bool open_leaves(const float4& xh, const OpenSpec& O) {
    const float x[3] = {xh.x, xh.y, DIM == 3 ? xh.z : 0.f};
    for (int q = 0; q < O.n_out; ++q) {
        const DevOutlet& Q = O.out[q];
        float dn = 0.f;
        for (int d = 0; d < DIM; ++d) dn = __fadd_rn(dn, __fmul_rn(__fsub_rn(x[d], Q.o[d]), Q.n[d]));
        float dr = 0.f;
        for (int d = 0; d < DIM; ++d) {
            const float e = __fsub_rn(__fsub_rn(x[d], Q.o[d]), __fmul_rn(dn, Q.n[d]));
            dr = __fadd_rn(dr, __fmul_rn(e, e));
        }
        if (dn < 0.f && __fsqrt_rn(dr) < Q.R) return true;
    }
    for (int d = 0; d < DIM; ++d)
        if (x[d] > O.hi[d] || x[d] < O.lo[d]) return true;
    return false;
}

template <int DIM>
__global__ void __launch_bounds__(kGhostThreads)
    k_open_flags(StateA A, int n, OpenSpec O, int* __restrict__ keep,
                 unsigned* __restrict__ tile_count) {
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_total;
    unsigned mine = 0;
    for (int it = 0; it < kGhostItems; ++it) {
        const int i = blockIdx.x * kGhostTile + it * kGhostThreads + (int)threadIdx.x;
        if (i >= n) break;
        const int k = open_leaves<DIM>(A.xh[i], O) ? 0 : 1;
        keep[i] = k;
        mine += k;
    }
    block_excl_scan<kGhostThreads>(mine, s_warp, &s_total);
    if (threadIdx.x == 0) tile_count[blockIdx.x] = s_total;
}

// The kept particles of A, in order, into D.
__global__ void __launch_bounds__(kGhostThreads)
    k_open_compact(StateA A, StateA D, int n, const int* __restrict__ keep,
                   const unsigned* __restrict__ tile_off) {
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_total;
    unsigned base = tile_off[blockIdx.x];
    for (int it = 0; it < kGhostItems; ++it) {
        const int i = blockIdx.x * kGhostTile + it * kGhostThreads + (int)threadIdx.x;
        const int k = (i < n) ? keep[i] : 0;
        const unsigned rank = block_excl_scan<kGhostThreads>((unsigned)k, s_warp, &s_total);
        if (k) {
            const int o = (int)(base + rank);
            D.xh[o] = A.xh[i];
            D.vm[o] = A.vm[i];
            D.u[o] = A.u[i];
            D.ap[o] = A.ap[i];
            D.rho[o] = A.rho[i];
            D.p[o] = A.p[i];
            D.itype[o] = A.itype[i];
            D.id[o] = A.id[i];
        }
        base += s_total;
    }
}

// Keys of the output order: the particles' serial numbers.
__global__ void k_open_id_keys(StateA A, int n, unsigned* __restrict__ keys) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) keys[s] = (unsigned)A.id[s];
}

// Output r = the particle of rank r in serial order: every field, staged.
template <int DIM>
__global__ void k_open_out(StateA A, const int* __restrict__ order, int n, float* __restrict__ x,
                           float* __restrict__ v, float* __restrict__ m, float* __restrict__ rho,
                           float* __restrict__ p, float* __restrict__ u, float* __restrict__ h,
                           int* __restrict__ itype, float* __restrict__ dvdt,
                           float* __restrict__ dudt) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int s = order[r];
    const float4 a = A.xh[s], b = A.vm[s], q = A.ap[s];
    x[DIM * r] = a.x;
    x[DIM * r + 1] = a.y;
    v[DIM * r] = b.x;
    v[DIM * r + 1] = b.y;
    dvdt[DIM * r] = q.x;
    dvdt[DIM * r + 1] = q.y;
    if (DIM == 3) {
        x[3 * r + 2] = a.z;
        v[3 * r + 2] = b.z;
        dvdt[3 * r + 2] = q.z;
    }
    m[r] = (DIM == 2) ? a.z : b.w;
    h[r] = a.w;
    dudt[r] = q.w;
    u[r] = A.u[s];
    rho[r] = A.rho[s];
    p[r] = A.p[s];
    itype[r] = A.itype[s];
}

}  // namespace ag
