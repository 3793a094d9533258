// ghosts.cuh -- mirror ghost particles (wall_model 3).
//
// CERNsource/ghost.f:1-86 with virtual_part (time_integration.f:156-161,
// single_step.f:188-196): every iteration, after the predictor, each fluid
// particle i with a wall particle (itype <= 0) in reach takes the nearest one,
// w, whose velocity entry is its inward unit normal n, and gains the ghost
//   x_g = x_i - 2 n ((x_i - x_w) . n),   v_g = v_i - 2 n (v_i . n)
// with the mass and h of i. The ghosts join the step as wall-like particles
// (itype 0, ids n_real + k in the order of their owners); after the density
// pass each takes its owner's density, pressure and energy. Their rates are
// dropped and the next state goes back in caller order.
//
// Wall particles do not move, so one wall grid per call serves every
// iteration's nearest-wall search: cells of 2 max(h) over the walls' box, the
// walls sorted by cell with the step's radix sort (fluid keys past the last
// cell) and their positions and normals copied in cell order.
//
// The nearest wall is the smallest FP32 squared distance of link_list's pair
// test (ties to the lower index); the mirror is computed in FP32 without
// contraction, in the order of ghost.f's sums.
#pragma once
#include "kernels.cuh"

namespace ag {

struct WallGrid {
    float o[3];
    float size;  // cell edge: 2 max(h) over every particle, a little widened
    int n[3];
    int ncells;  // 0: no wall particle; -1: more cells than the call allows
};

constexpr int kWallGridThreads = 1024;
constexpr int kGhostThreads = 256;
constexpr int kGhostItems = 4;
constexpr int kGhostTile = kGhostThreads * kGhostItems;

// Box of the wall particles, their count and max h of all particles: partial
// results per CTA (8 floats each: min[3], max[3], max h, the count's bits).
template <int DIM>
__global__ void __launch_bounds__(256)
    k_wall_grid_partial(StateA A, int n, float* __restrict__ part) {
    __shared__ float s_red[7][8];
    __shared__ int s_cnt[8];
    float v[7] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f};
    int cnt = 0;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) {
        const float4 xh = A.xh[i];
        v[6] = fmaxf(v[6], xh.w);
        if (A.itype[i] <= 0) {
            const float c[3] = {xh.x, xh.y, DIM == 3 ? xh.z : 0.f};
            for (int d = 0; d < 3; ++d) {
                v[d] = fminf(v[d], c[d]);
                v[3 + d] = fmaxf(v[3 + d], c[d]);
            }
            ++cnt;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        for (int d = 0; d < 3; ++d) v[d] = fminf(v[d], __shfl_xor_sync(0xffffffffu, v[d], off));
        for (int d = 3; d < 7; ++d) v[d] = fmaxf(v[d], __shfl_xor_sync(0xffffffffu, v[d], off));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    }
    if (lane == 0) {
        for (int d = 0; d < 7; ++d) s_red[d][warp] = v[d];
        s_cnt[warp] = cnt;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < 8; ++w) {
        for (int d = 0; d < 3; ++d) v[d] = fminf(v[d], s_red[d][w]);
        for (int d = 3; d < 7; ++d) v[d] = fmaxf(v[d], s_red[d][w]);
        cnt += s_cnt[w];
    }
    float* o = part + 8 * blockIdx.x;
    for (int d = 0; d < 7; ++d) o[d] = v[d];
    o[7] = __int_as_float(cnt);
}

// The wall grid from the partials (one block): min / max / count are exact in
// any order, so the grid does not depend on how the particles were split.
template <int DIM>
__global__ void __launch_bounds__(kWallGridThreads)
    k_wall_grid(const float* __restrict__ part, int nparts, long long max_cells,
                WallGrid* __restrict__ wg) {
    __shared__ float s_red[7][32];
    __shared__ int s_cnt[32];
    float v[7] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f};
    int cnt = 0;
    for (int b = threadIdx.x; b < nparts; b += kWallGridThreads) {
        const float* q = part + 8 * b;
        for (int d = 0; d < 3; ++d) v[d] = fminf(v[d], q[d]);
        for (int d = 3; d < 7; ++d) v[d] = fmaxf(v[d], q[d]);
        cnt += __float_as_int(q[7]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        for (int d = 0; d < 3; ++d) v[d] = fminf(v[d], __shfl_xor_sync(0xffffffffu, v[d], off));
        for (int d = 3; d < 7; ++d) v[d] = fmaxf(v[d], __shfl_xor_sync(0xffffffffu, v[d], off));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    }
    if (lane == 0) {
        for (int d = 0; d < 7; ++d) s_red[d][warp] = v[d];
        s_cnt[warp] = cnt;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < kWallGridThreads / 32; ++w) {
        for (int d = 0; d < 3; ++d) v[d] = fminf(v[d], s_red[d][w]);
        for (int d = 3; d < 7; ++d) v[d] = fmaxf(v[d], s_red[d][w]);
        cnt += s_cnt[w];
    }
    WallGrid g;
    // 2 max(h) bounds every pair reach h_i + h_j; the widening keeps a pair in
    // reach within one cell of each other in spite of the division's rounding.
    g.size = 2.0f * v[6] * 1.00001f;
    long long cells = 1;
    for (int d = 0; d < 3; ++d) {
        g.o[d] = (d < DIM) ? v[d] - g.size : 0.f;
        g.n[d] = 1;
        if (d < DIM && cnt > 0 && g.size > 0.f) {
            const float span = (v[3 + d] - v[d] + 2.0f * g.size) / g.size;
            g.n[d] = (span < 1.0e9f) ? (int)span + 1 : 1000000000;
        }
        if (cells <= max_cells) cells *= g.n[d];  // saturates (no overflow)
    }
    if (cnt == 0 || !(g.size > 0.f)) g.ncells = 0;
    else g.ncells = (cells > max_cells) ? -1 : (int)cells;
    *wg = g;
}

template <int DIM>
__device__ __forceinline__ int wall_cell_axis(float x, const WallGrid& g, int d, int lo, int hi) {
    float c = floorf((x - g.o[d]) / g.size);
    c = fminf(fmaxf(c, (float)lo), (float)hi);
    return (int)c;
}

// Sort keys of the wall sort: the cell of each wall particle; fluid particles
// get ncells, past every cell.
template <int DIM>
__global__ void k_wall_keys(StateA A, int n, const WallGrid* __restrict__ wgp,
                            unsigned* __restrict__ keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const WallGrid g = *wgp;
    if (A.itype[i] > 0) {
        keys[i] = (unsigned)g.ncells;
        return;
    }
    const float4 xh = A.xh[i];
    const int cx = wall_cell_axis<DIM>(xh.x, g, 0, 0, g.n[0] - 1);
    const int cy = wall_cell_axis<DIM>(xh.y, g, 1, 0, g.n[1] - 1);
    const int cz = (DIM == 3) ? wall_cell_axis<DIM>(xh.z, g, 2, 0, g.n[2] - 1) : 0;
    keys[i] = (unsigned)(cx + g.n[0] * (cy + g.n[1] * cz));
}

// The walls in cell order: position {x, h} and normal of each, and its index.
__global__ void k_wall_gather(const int* __restrict__ order, const int* __restrict__ wstart,
                              const WallGrid* __restrict__ wgp, StateA A, int n,
                              float4* __restrict__ wall_xh, float4* __restrict__ wall_n,
                              int* __restrict__ wall_id) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int nc = wgp->ncells;
    if (nc <= 0 || k >= wstart[nc]) return;
    const int j = order[k];
    wall_xh[k] = A.xh[j];
    wall_n[k] = A.vm[j];
    wall_id[k] = j;
}

// Nearest wall particle in reach of every fluid particle (-1: none) and the
// number of ghosts of each tile of kGhostTile particles.
template <int DIM>
__global__ void __launch_bounds__(kGhostThreads)
    k_ghost_select(StateA A, int n, const WallGrid* __restrict__ wgp, const int* __restrict__ wstart,
                   const float4* __restrict__ wall_xh, const int* __restrict__ wall_id,
                   int* __restrict__ best, unsigned* __restrict__ tile_count) {
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_total;
    const WallGrid g = *wgp;
    unsigned mine = 0;
    for (int it = 0; it < kGhostItems; ++it) {
        const int i = blockIdx.x * kGhostTile + it * kGhostThreads + (int)threadIdx.x;
        if (i >= n) break;
        int pick = -1;
        if (A.itype[i] > 0 && g.ncells > 0) {
            const float4 xi = A.xh[i];
            const int cx = wall_cell_axis<DIM>(xi.x, g, 0, -1, g.n[0]);
            const int cy = wall_cell_axis<DIM>(xi.y, g, 1, -1, g.n[1]);
            const int cz = (DIM == 3) ? wall_cell_axis<DIM>(xi.z, g, 2, -1, g.n[2]) : 0;
            float bd = 0.f;
            int bid = 0;
            for (int dz = (DIM == 3 ? -1 : 0); dz <= (DIM == 3 ? 1 : 0); ++dz) {
                const int z = cz + dz;
                if (z < 0 || z >= g.n[2]) continue;
                for (int dy = -1; dy <= 1; ++dy) {
                    const int y = cy + dy;
                    if (y < 0 || y >= g.n[1]) continue;
                    for (int dx = -1; dx <= 1; ++dx) {
                        const int x = cx + dx;
                        if (x < 0 || x >= g.n[0]) continue;
                        const int c = x + g.n[0] * (y + g.n[1] * z);
                        const int k1 = wstart[c + 1];
                        for (int k = wstart[c]; k < k1; ++k) {
                            const float4 xw = wall_xh[k];
                            // link_list.f:154-159 in FP32, unfused, axes in order
                            const float e0 = __fsub_rn(xi.x, xw.x), e1 = __fsub_rn(xi.y, xw.y);
                            float dr2 = __fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1));
                            if (DIM == 3) {
                                const float e2 = __fsub_rn(xi.z, xw.z);
                                dr2 = __fadd_rn(dr2, __fmul_rn(e2, e2));
                            }
                            const float sh = __fadd_rn(xi.w, xw.w);
                            if (!(dr2 < __fmul_rn(sh, sh))) continue;
                            const int id = wall_id[k];
                            if (pick < 0 || dr2 < bd || (dr2 == bd && id < bid)) {
                                pick = k;
                                bd = dr2;
                                bid = id;
                            }
                        }
                    }
                }
            }
        }
        best[i] = pick;
        mine += (pick >= 0);
    }
    block_excl_scan<kGhostThreads>(mine, s_warp, &s_total);
    if (threadIdx.x == 0) tile_count[blockIdx.x] = s_total;
}

// Exclusive scan of the tile counts (one block); total = ghosts this iteration.
__global__ void __launch_bounds__(1024)
    k_ghost_scan(const unsigned* __restrict__ tile_count, int tiles, unsigned* __restrict__ tile_off,
                 int* __restrict__ total) {
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_total;
    const int per = (tiles + 1023) / 1024;
    const int b = (int)threadIdx.x * per, e = min(b + per, tiles);
    unsigned sum = 0;
    for (int t = b; t < e; ++t) sum += tile_count[t];
    unsigned off = block_excl_scan<1024>(sum, s_warp, &s_total);
    for (int t = b; t < e; ++t) {
        const unsigned c = tile_count[t];
        tile_off[t] = off;
        off += c;
    }
    if (threadIdx.x == 0) *total = (int)s_total;
}

// Writes the ghosts of one tile after the real particles, in owner order:
// slot n + k, id n + k, owner[k] = the fluid particle's index.
template <int DIM>
__global__ void __launch_bounds__(kGhostThreads)
    k_ghost_write(StateA A, int n, const int* __restrict__ best, const float4* __restrict__ wall_xh,
                  const float4* __restrict__ wall_n, const unsigned* __restrict__ tile_off,
                  int* __restrict__ owner, StepArgs S) {
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_total;
    unsigned base = tile_off[blockIdx.x];
    for (int it = 0; it < kGhostItems; ++it) {
        const int i = blockIdx.x * kGhostTile + it * kGhostThreads + (int)threadIdx.x;
        const int w = (i < n) ? best[i] : -1;
        const unsigned rank = block_excl_scan<kGhostThreads>(w >= 0 ? 1u : 0u, s_warp, &s_total);
        if (w >= 0) {
            const int k = (int)(base + rank);
            const int gslot = n + k;
            const float4 xi = A.xh[i];
            float4 vi = A.vm[i];
            if (S.hdt != 0.f) {  // the predictor of k_reorder_dim (fluid particles)
                const float4 ap = A.ap[i];
                vi.x = fmaf(S.hdt, ap.x, vi.x);
                vi.y = fmaf(S.hdt, ap.y, vi.y);
                if (DIM == 3) vi.z = fmaf(S.hdt, ap.z, vi.z);
            }
            const float4 xw = wall_xh[w], nw = wall_n[w];
            // ghost.f:66-70: dd1 = (x_i - x_w) . n, dd2 = v_i . n
            float dd1 = __fmul_rn(__fsub_rn(xi.x, xw.x), nw.x);
            dd1 = __fadd_rn(dd1, __fmul_rn(__fsub_rn(xi.y, xw.y), nw.y));
            float dd2 = __fmul_rn(vi.x, nw.x);
            dd2 = __fadd_rn(dd2, __fmul_rn(vi.y, nw.y));
            if (DIM == 3) {
                dd1 = __fadd_rn(dd1, __fmul_rn(__fsub_rn(xi.z, xw.z), nw.z));
                dd2 = __fadd_rn(dd2, __fmul_rn(vi.z, nw.z));
            }
            // ghost.f:72-75
            float4 xg = xi, vg = vi;
            xg.x = __fsub_rn(xi.x, __fmul_rn(__fmul_rn(2.f, nw.x), dd1));
            xg.y = __fsub_rn(xi.y, __fmul_rn(__fmul_rn(2.f, nw.y), dd1));
            vg.x = __fsub_rn(vi.x, __fmul_rn(__fmul_rn(2.f, nw.x), dd2));
            vg.y = __fsub_rn(vi.y, __fmul_rn(__fmul_rn(2.f, nw.y), dd2));
            if (DIM == 3) {
                xg.z = __fsub_rn(xi.z, __fmul_rn(__fmul_rn(2.f, nw.z), dd1));
                vg.z = __fsub_rn(vi.z, __fmul_rn(__fmul_rn(2.f, nw.z), dd2));
            }
            A.xh[gslot] = xg;  // 2D: .z keeps the mass; .w keeps h
            A.vm[gslot] = vg;  // 3D: .w keeps the mass
            A.u[gslot] = A.u[i];
            A.ap[gslot] = make_float4(0.f, 0.f, 0.f, 0.f);
            A.rho[gslot] = A.rho[i];
            A.p[gslot] = A.p[i];
            A.itype[gslot] = 0;
            A.id[gslot] = gslot;
            owner[k] = i;
        }
        base += s_total;
    }
}

// After the density pass: every ghost takes its owner's density, pressure and
// (predicted) energy of this iteration (single_step.f:188-196); with
// artificial heat its psi follows from its own div v sum, which the density
// pass left in tds, over that density.
template <int DIM>
__global__ void k_ghost_sync(StateB B, const int* __restrict__ slot_of, const int* __restrict__ owner,
                             DevParams P, int n_tot) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_tot) return;
    const int id = B.id[s];
    if (id < P.n_real) return;
    const int o = slot_of[owner[id - P.n_real]];
    float4 rp = B.rp[o];
    if (P.heat_art) {
        const float h = B.xh[s].w;
        const float divv = __fdiv_rn(B.tds[s], rp.x);
        rp.w = fmaf(P.ah_g2 * h * h, fabsf(divv) - divv, __fmul_rn(P.ah_g1 * h, P.c0));
    }
    B.rp[s] = rp;
    B.p[s] = B.p[o];
    if (B.ulo) B.ulo[s] = B.ulo[o];
    if (DIM == 2) {
        const float4 vi = B.vm[s];
        B.vr[s] = make_float4(vi.x, vi.y, rp.x, rp.y);
    }
}

}  // namespace ag
