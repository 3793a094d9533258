// kernels.cuh -- sm_103a kernels of one leapfrog step of Armando's SPH.
//
// Step pipeline (one CUDA graph per step):
//   bbox_partial -> bbox_final        grid of CERNsource/link_list.f:39-67
//   hash (+ digit-0 histogram)        cell id, link_list.f:75-88 / acpu.c:2085-2105
//   [hist] scan scatter  x passes     LSD radix sort of (cell, slot), 8-bit digits
//   cell_start                        first slot of every cell (empty cells included)
//   reorder                           gather state into cell order + leapfrog predictor
//                                     (time_integration.f:136-154)
//   density                           summation density + Tait EOS + div v
//                                     (density.f:1-62, eos.f90:255-283, art_heat.f:46-67)
//   shear (physical viscosity only)   shear tensor T_ab (internal_force.f:75-171)
//   force                             pressure + viscous force, art_visc, art_heat,
//                                     external heat, gravity, leapfrog corrector
//                                     (internal_force.f:178-435, art_visc.f:55-101,
//                                     art_heat.f:69-97, time_integration.f:186-218)
// Every pass is a gather over the 3^dim neighbour cells of a particle: no
// atomics on particle data, so a step is deterministic. Layout (float4, sorted
// by cell):
//   xh  2D {x, y, m, h}        3D {x, y, z, h}
//   vm  2D {vx, vy, 0, 0}      3D {vx, vy, vz, m}
//   rp  {rho, pf, u, psi}      pf = p/rho^2 (pa_sph 1) or p (pa_sph 0),
//                              psi = art_heat coefficient of the particle
#pragma once
#include <cfloat>
#include <cstdint>

#include "sph_math.cuh"

namespace ag {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;
constexpr int kPassThreads = 128;
constexpr int kBBoxBlocks = 608;  // 4 x 152 SMs

enum DevFlag : unsigned {
    FLAG_GRID_OVERFLOW = 1u,
    FLAG_NONFINITE = 2u,
    FLAG_OUT_OF_GRID = 4u,
    FLAG_PERIODIC_SMALL = 8u,
    FLAG_BAD_MATERIAL = 16u,  // an itype outside the material table (GPU-C schemes)
    FLAG_TIMEOUT = 32u,       // a bounded wait on a bulk copy gave up
};

struct DevGrid {
    float o[3], size[3], L[3], half[3];
    int n[3];
    int ncells;    // cells of this grid
    int ok;        // 0 when the grid did not fit; passes then do nothing
    int periodic[3];
    int cell_off;  // first cell of this grid in the shared cell table (batches)
    int reach;       // stencil half-width in cells: cell size (2 max(h) + skin) / reach
    float half_skin2;  // (skin / 2)^2: a particle this far from its binned position forces a sort
    float skin;        // sort skin (length): neighbour lists hold pairs within h_i + h_j + skin
};

// A unit of work of the persistent passes: slots [s0, s1) of one instance.
struct WorkItem {
    int s0, s1, inst, pad;
};

struct DevParams {
    int dim, pa_sph, visc, visc_art, heat_art, heat_ext;
    int periodic[3];
    float rho0, inv_rho0, B, c0, pmin, eta;
    float av_alpha, av_beta, av_eta2;
    float ah_g1, ah_g2, ah_eta2;
    float gravity[3];
    float heat_q0, heat_k, heat_center[3];
    float period_lo[3], period_hi[3], period_L[3], period_half[3];
    float kw_hi, kw_lo;  // K_dim as float-float
    float kg;            // K_dim * 5/8
    float dt;            // time step of this instance (batches)
    float heat_t_end;    // external heat gate its*dt <= heat_t_end
    int reach;           // neighbour-grid cells per support radius (tuning; 1 = link_list)
    float skin;          // sort skin as a fraction of max h (tuning; 0 = sort every step)
    // Wall treatment: 0 like any pair, 1 push only, 2 push and every sum between
    // different itype; 3 like 0 plus mirror ghosts (particles with id >= n_real).
    int wall_model;
    int n_real;          // real particles; ids from n_real on are mirror ghosts
    // single_step options: density 0 summation, 1 continuity, 2 normalised
    // summation; XSPH; smoothing-length evolution 0, 1, 2.
    int density_form, xsph, sle, pad2_;
};

__host__ __device__ inline bool repulsive_walls(const DevParams& P) {
    return P.wall_model == 1 || P.wall_model == 2;
}

struct StepArgs {
    float kdt;    // corrector step: dt (its > 1) or dt/2 (its == 1)
    float hdt;    // predictor half step: dt/2 (its > 1) or 0 (its == 1)
    float dt;     // drift
    int heat_on;  // external heat gate its*dt <= t_end
    int dform;    // density form (1: the predictor advances rho with the carried drho/dt)
};

struct StateA {  // integrated state (slot order of the last sort)
    float4* xh;
    float4* vm;
    float* u;
    float4* ap;  // previous rates {a, du}
    float* rho;
    float* p;
    int* itype;
    int* id;
    int* inst;  // instance of each slot (batches; nullptr for one system)
    float* drho;  // drho/dt of the last iteration (continuity density; else nullptr)
};

struct StateB {  // working set of one step (cell order)
    float4* xh;
    float4* vm;    // predicted velocity (+ mass in 3D)
    float4* vmin;  // velocity and energy at the start of the step
    float4* rp;
    float* p;
    int* itype;
    int* id;
    float4* tau;   // eta T_ab / rho^2 (or eta T_ab): {xx, yy, xy, zz}
    float4* tau2;  // {xz, yz, -, -}
    float* tds;    // T ds/dt
    float* ulo;    // rounding residual of the predicted energy u (rp.z + ulo exact)
    float* q;      // density at the iteration's start (continuity and normalised density)
    float* rlo;    // rounding residual of the predicted density (continuity)
    float4* vr;    // 2D: {vx, vy, rho, P} after the density pass (one neighbour load in the force pass)
    float4* xsort; // position of each slot when the particles were last sorted
    // Neighbour lists of a lazily sorting context (built on the iterations that
    // sort): row t of slot s at nlist[t * lstride + s], the candidates within
    // h_i + h_j + skin, first the near ones (q < list_near_q2() when sorted; in 3D
    // all) in cursor order, then the far ones in reverse cursor order;
    // ncount[s] = near | far << 16, -1 when more than lcap (that slot walks
    // its cells instead).
    int* nlist;
    int* ncount;
    int lcap;      // list entries per slot
    int lstride;   // slots per list row (the context's capacity)
    // Neighbour bits of each fluid slot over its first 32 * mask_words<DIM>()
    // candidates (cursor order); words 0 and 1 all ones: more candidates than
    // bits. With TPP lanes per particle, lane L = s * TPP + sub keeps
    // mask_words / TPP words of its own candidates, in chunks of up to 4 words
    // stored chunk-major (mask_word_index), so one vector load per warp reads
    // a chunk of every lane.
    unsigned* nmask;
    int* inst;     // instance of each slot (batches; nullptr for one system)
    int mstride;   // lanes: n * TPP
    int mtpp;      // the TPP the masks were written with
};

template <int DIM>
__host__ __device__ constexpr int mask_words() {
    return DIM == 2 ? 4 : 16;
}

// Words per chunk of a lane holding W mask words.
template <int W>
__host__ __device__ constexpr int mask_chunk() {
    return W < 4 ? W : 4;
}

// Word w of lane L (nl lanes).
template <int W>
__device__ __forceinline__ size_t mask_word_index(int w, size_t nl, size_t L) {
    constexpr int CW = mask_chunk<W>();
    return ((size_t)(w / CW) * nl + L) * CW + (size_t)(w % CW);
}

// Chunk c of lane L as up to four words.
template <int W>
__device__ __forceinline__ uint4 mask_load_chunk(const unsigned* __restrict__ m, size_t nl,
                                                 size_t L, int c) {
    constexpr int CW = mask_chunk<W>();
    const size_t at = (size_t)c * nl + L;
    if (CW == 4) return __ldg(reinterpret_cast<const uint4*>(m) + at);
    if (CW == 2) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(m) + at);
        return make_uint4(v.x, v.y, 0u, 0u);
    }
    return make_uint4(__ldg(m + at), 0u, 0u, 0u);
}

__device__ __forceinline__ unsigned chunk_word(const uint4& ch, int j) {
    return j == 0 ? ch.x : j == 1 ? ch.y : j == 2 ? ch.z : ch.w;
}

template <int DIM>
__device__ __forceinline__ float mass_of(const float4& xh, const float4& vm) {
    return DIM == 2 ? xh.z : vm.w;
}

// Lazy sorting (sort skin). resort[1] != 0 asks for a sort: the force pass
// sets it when a particle has moved more than half the skin from where it was
// binned, the host after loading a state. The first kernel of an iteration
// (resort_begin) turns it into resort[0] (this iteration sorts) and clears it.
// The grid, hash, sort and cell-table kernels return at once on an iteration
// that does not sort (their outputs from the last sort stay valid: cells of
// 2 max(h) + skin hold every pair within 2 max(h) while no particle is farther
// than skin / 2 from its binned position). resort == nullptr: always sort.
__device__ __forceinline__ bool sort_skipped(const int* resort) {
    return resort != nullptr && *(volatile const int*)resort == 0;
}

// Start of a lazily sorting iteration (one thread); counts the sorts.
__device__ __forceinline__ unsigned resort_begin(int* resort, int* sorts) {
    const unsigned sort = resort[1] != 0 ? 1u : 0u;
    resort[0] = (int)sort;
    resort[1] = 0;
    if (sort) ++sorts[0];
    return sort;
}

__global__ void k_resort_begin(int* __restrict__ resort, int* __restrict__ sorts) {
    if (threadIdx.x == 0 && blockIdx.x == 0) resort_begin(resort, sorts);
}

// Head of a lazily sorting step graph: starts the iteration; the IF node
// after it runs the grid, hash, sort and cell-table kernels only when this
// iteration sorts.
__global__ void k_resort_cond(cudaGraphConditionalHandle handle, int* __restrict__ resort,
                              int* __restrict__ sorts) {
    if (threadIdx.x == 0 && blockIdx.x == 0)
        cudaGraphSetConditional(handle, resort_begin(resort, sorts));
}

// ---------------------------------------------------------------------------
// Small block-level helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned warp_incl_scan(unsigned v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan of one value per thread over a block of NT threads.
template <int NT>
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned* s_warp,
                                                    unsigned* total = nullptr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned inc = warp_incl_scan(v);
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned w = (lane < NT / 32) ? s_warp[lane] : 0u;
        unsigned wi = warp_incl_scan(w);
        if (lane < NT / 32) s_warp[lane] = wi - w;
        if (lane == NT / 32 - 1 && total) *total = wi;
    }
    __syncthreads();
    unsigned r = s_warp[warp] + inc - v;
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------
// Grid: bbox of all particles and the link_list grid in FP32.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bbox_partial(const float4* __restrict__ xh, int n, int dim,
                                                      float* __restrict__ part,
    const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, mh = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = xh[i];
        mn[0] = fminf(mn[0], a.x);
        mx[0] = fmaxf(mx[0], a.x);
        mn[1] = fminf(mn[1], a.y);
        mx[1] = fmaxf(mx[1], a.y);
        if (dim == 3) {
            mn[2] = fminf(mn[2], a.z);
            mx[2] = fmaxf(mx[2], a.z);
        }
        mh = fmaxf(mh, a.w);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
        mh = fmaxf(mh, __shfl_xor_sync(0xffffffffu, mh, o));
    }
    __shared__ float s[8][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        for (int d = 0; d < 3; ++d) {
            s[warp][d] = mn[d];
            s[warp][3 + d] = mx[d];
        }
        s[warp][6] = mh;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        int k = threadIdx.x;
        float v = s[0][k];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            v = (k < 3) ? fminf(v, s[w][k]) : fmaxf(v, s[w][k]);
        part[blockIdx.x * 8 + k] = v;
    }
}

__device__ __forceinline__ DevGrid grid_from_bbox(const float* mm, const DevParams& P,
                                                  long long capacity, unsigned& fl);

__global__ void __launch_bounds__(256) k_bbox_final(const float* __restrict__ part, int nparts,
                                                    DevParams P, long long capacity,
                                                    DevGrid* __restrict__ grid,
                                                    unsigned* __restrict__ flags,
    const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    __shared__ float s[7][256];
    float v[7] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
        for (int k = 0; k < 7; ++k)
            v[k] = (k < 3) ? fminf(v[k], part[b * 8 + k]) : fmaxf(v[k], part[b * 8 + k]);
    for (int k = 0; k < 7; ++k) s[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int k = 0; k < 7; ++k)
                s[k][threadIdx.x] = (k < 3) ? fminf(s[k][threadIdx.x], s[k][threadIdx.x + st])
                                            : fmaxf(s[k][threadIdx.x], s[k][threadIdx.x + st]);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const float mm[7] = {s[0][0], s[1][0], s[2][0], s[3][0], s[4][0], s[5][0], s[6][0]};
    unsigned fl = 0;
    DevGrid g = grid_from_bbox(mm, P, capacity, fl);
    *grid = g;
    if (fl) atomicOr(flags, fl);
}

// The link_list grid (CERNsource/link_list.f:39-67) of a bbox mm = {min[3],
// max[3], max h}, in FP32; periodic axes split their box into >= 3 cells.
// With P.reach = f the cells are (2 mh + skin) / f wide, skin = P.skin * mh,
// and the passes search (2f + 1)^dim cells. Unless f = 1 and skin = 0 (which
// keep link_list's cell exactly) the cells are widened by a margin larger
// than the rounding of a cell index ((x - o) / size: a few ulp of the index,
// i.e. n * 2^-23 cells), so no pair the exact test accepts is outside the
// stencil.
__device__ __forceinline__ DevGrid grid_from_bbox(const float* mm, const DevParams& P,
                                                  long long capacity, unsigned& fl) {
    DevGrid g;
    const float mh = mm[6];
    const int f = P.reach > 1 ? P.reach : 1;
    const float skin = P.skin > 0.f ? P.skin * mh : 0.f;
    float cell = __fmul_rn(2.0f, mh);  // scale_k * mh, scale_k = 2
    if (f > 1 || skin > 0.f) {
        float span = 0.f;
        for (int d = 0; d < P.dim; ++d)
            span = fmaxf(span, P.periodic[d] ? P.period_L[d] : mm[3 + d] - mm[d] + 2.f * mh);
        const float cf = (cell + skin) / (float)f;
        const float nmax = span / fmaxf(cf, FLT_MIN);
        cell = cf * (1.0f + 0x1p-12f + fminf(nmax, 1.0e7f) * 0x1p-20f);
    }
    long long ncells = 1;
    for (int d = 0; d < 3; ++d) {
        g.periodic[d] = P.periodic[d];
        g.o[d] = 0.f;
        g.size[d] = 1.f;
        g.L[d] = 0.f;
        g.half[d] = 0.f;
        g.n[d] = 1;
        if (d >= P.dim) continue;
        if (P.periodic[d]) {
            const float L = P.period_L[d];
            float nf = __fdiv_rn(L, cell);
            const float nmin = (float)(2 * f + 1);
            int nn = (nf >= nmin && nf < 1.0e9f) ? (int)nf : 2 * f + 1;
            if (!(nf >= nmin)) fl |= FLAG_PERIODIC_SMALL;
            g.o[d] = P.period_lo[d];
            g.size[d] = __fdiv_rn(L, (float)nn);
            g.L[d] = L;
            g.half[d] = P.period_half[d];
            g.n[d] = nn;
        } else {
            const float lo = __fsub_rn(mm[d], mh);
            const float hi = __fadd_rn(mm[3 + d], mh);
            float nf = __fdiv_rn(__fsub_rn(hi, lo), cell);
            g.o[d] = lo;
            g.size[d] = cell;
            if (nf < 1.0e9f) {
                g.n[d] = (int)nf + 1;
            } else {
                g.n[d] = 1;
                fl |= FLAG_GRID_OVERFLOW;
            }
        }
        // Saturates once above the capacity: three axes of up to 1e9 cells
        // each would overflow the product (a far outlier in 3D).
        if (ncells <= capacity) ncells *= g.n[d];
    }
    g.ok = 1;
    g.cell_off = 0;
    g.reach = f;
    g.half_skin2 = 0.25f * skin * skin;
    g.skin = skin;
    if (ncells > capacity || (fl & FLAG_GRID_OVERFLOW) || (fl & FLAG_PERIODIC_SMALL)) {
        fl |= (ncells > capacity) ? FLAG_GRID_OVERFLOW : 0u;
        g.ok = 0;
        ncells = capacity;
    }
    g.ncells = (int)ncells;
    return g;
}

template <int DIM>
__device__ __forceinline__ unsigned cell_key(const float4& a, const DevGrid& g) {
    const float xv[3] = {a.x, a.y, a.z};
    unsigned key = 0;
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
        int c = (int)__fdiv_rn(__fsub_rn(xv[d], g.o[d]), g.size[d]);
        c = c < 0 ? 0 : (c > g.n[d] - 1 ? g.n[d] - 1 : c);
        key = key * (unsigned)g.n[d] + (unsigned)c;
    }
    if (!g.ok) key = 0;
    return key + (unsigned)g.cell_off;
}

// Cell key of every slot + per-tile histogram of its low digit.
template <int DIM>
__global__ void __launch_bounds__(kSortThreads)
    k_hash(const float4* __restrict__ xh, int n, const DevGrid* __restrict__ gp,
           unsigned* __restrict__ keys, unsigned* __restrict__ hist, int num_tiles,
    const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    __shared__ unsigned sh[kRadix];
    __shared__ DevGrid g;
    if (threadIdx.x == 0) g = *gp;
    sh[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        int i = base + k * kSortThreads + threadIdx.x;
        if (i < n) {
            unsigned key = cell_key<DIM>(xh[i], g);
            keys[i] = key;
            atomicAdd(&sh[key & 255u], 1u);
        }
    }
    __syncthreads();
    hist[threadIdx.x * num_tiles + blockIdx.x] = sh[threadIdx.x];
}

// Bbox partials straight from caller-layout arrays x[n*DIM], h[n].
template <int DIM>
__global__ void __launch_bounds__(256) k_bbox_partial_raw(const float* __restrict__ x,
                                                          const float* __restrict__ h, int n,
                                                          float* __restrict__ part) {
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, mh = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const float v = x[(size_t)DIM * i + d];
            mn[d] = fminf(mn[d], v);
            mx[d] = fmaxf(mx[d], v);
        }
        mh = fmaxf(mh, h[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
        mh = fmaxf(mh, __shfl_xor_sync(0xffffffffu, mh, o));
    }
    __shared__ float s[8][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        for (int d = 0; d < 3; ++d) {
            s[warp][d] = mn[d];
            s[warp][3 + d] = mx[d];
        }
        s[warp][6] = mh;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        int k = threadIdx.x;
        float v = s[0][k];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            v = (k < 3) ? fminf(v, s[w][k]) : fmaxf(v, s[w][k]);
        part[blockIdx.x * 8 + k] = v;
    }
}

// Cell keys straight from caller-layout positions x[n*DIM].
template <int DIM>
__global__ void k_keys_raw(const float* __restrict__ x, int n, const DevGrid* __restrict__ gp,
                           int* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    DevGrid g = *gp;
    const float4 a = make_float4(x[(size_t)DIM * i], x[(size_t)DIM * i + 1],
                                 DIM == 3 ? x[(size_t)DIM * i + 2] : 0.f, 0.f);
    out[i] = (int)cell_key<DIM>(a, g);
}

// Cell keys only (caller order), for the cell-id entry point.
template <int DIM>
__global__ void k_keys_only(const float4* __restrict__ xh, int n, const DevGrid* __restrict__ gp,
                            int* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    DevGrid g = *gp;
    out[i] = (int)cell_key<DIM>(xh[i], g);
}

// ---------------------------------------------------------------------------
// LSD radix sort, reduce-then-scan (no inter-block waiting).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSortThreads)
    k_radix_hist(const unsigned* __restrict__ keys, int n, int shift, unsigned* __restrict__ hist,
                 int num_tiles,
    const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    __shared__ unsigned sh[kRadix];
    sh[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        int i = base + k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&sh[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * num_tiles + blockIdx.x] = sh[threadIdx.x];
}

// Block d: exclusive scan of the tile counts of digit d; total per digit.
__global__ void __launch_bounds__(256)
    k_radix_scan(unsigned* __restrict__ hist, int num_tiles, unsigned* __restrict__ dtotal,
    const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_total;
    unsigned* row = hist + (size_t)blockIdx.x * num_tiles;
    const int per = (num_tiles + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per;
    const int e = min(b + per, num_tiles);
    unsigned sum = 0;
    for (int i = b; i < e; ++i) sum += row[i];
    unsigned off = block_excl_scan<256>(sum, s_warp, &s_total);
    for (int i = b; i < e; ++i) {
        unsigned c = row[i];
        row[i] = off;
        off += c;
    }
    if (threadIdx.x == 0) dtotal[blockIdx.x] = s_total;
}

// Stable scatter of one tile by one 8-bit digit. vals_in == nullptr means
// the values are the slot indices themselves.
__global__ void __launch_bounds__(kSortThreads)
    k_radix_scatter(const unsigned* __restrict__ keys_in, const int* __restrict__ vals_in,
                    unsigned* __restrict__ keys_out, int* __restrict__ vals_out, int n, int shift,
                    const unsigned* __restrict__ hist, const unsigned* __restrict__ dtotal,
                    int num_tiles,
    const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_base[kRadix];
    __shared__ unsigned s_tstart[kRadix];
    __shared__ unsigned s_wcnt[kSortThreads / 32][kRadix];
    __shared__ unsigned s_keys[kSortTile];
    __shared__ int s_vals[kSortTile];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x;
    const int tile_base = tile * kSortTile;
    const int tile_n = min(kSortTile, n - tile_base);

    unsigned excl = block_excl_scan<kSortThreads>(dtotal[tid], s_warp);
    s_base[tid] = excl + hist[(size_t)tid * num_tiles + tile];
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) s_wcnt[w][tid] = 0;
    __syncthreads();

    unsigned mykey[kSortItems];
    int myval[kSortItems];
    unsigned myrank[kSortItems];
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        const int idx = warp * (32 * kSortItems) + it * 32 + lane;
        const bool valid = idx < tile_n;
        unsigned key = valid ? keys_in[tile_base + idx] : 0u;
        int val = valid ? (vals_in ? vals_in[tile_base + idx] : tile_base + idx) : 0;
        unsigned d = (key >> shift) & 255u;
        unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 0x100u);
        unsigned lt = peers & ((1u << lane) - 1u);
        unsigned base = valid ? s_wcnt[warp][d] : 0u;
        __syncwarp();
        if (valid && lt == 0u) s_wcnt[warp][d] = base + __popc(peers);
        __syncwarp();
        mykey[it] = key;
        myval[it] = val;
        myrank[it] = base + __popc(lt);
    }
    __syncthreads();
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) {
        unsigned c = s_wcnt[w][tid];
        s_wcnt[w][tid] = run;
        run += c;
    }
    unsigned ts = block_excl_scan<kSortThreads>(run, s_warp);
    s_tstart[tid] = ts;
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        const int idx = warp * (32 * kSortItems) + it * 32 + lane;
        if (idx < tile_n) {
            unsigned d = (mykey[it] >> shift) & 255u;
            unsigned pos = s_tstart[d] + s_wcnt[warp][d] + myrank[it];
            s_keys[pos] = mykey[it];
            s_vals[pos] = myval[it];
        }
    }
    __syncthreads();
    for (int i = tid; i < tile_n; i += kSortThreads) {
        unsigned key = s_keys[i];
        unsigned d = (key >> shift) & 255u;
        unsigned dst = s_base[d] + (unsigned)i - s_tstart[d];
        keys_out[dst] = key;
        vals_out[dst] = s_vals[i];
    }
}

// start[c] = first sorted slot of cell c (the number of keys below c), for c in
// [0, ncells]; empty cells get start[c] == start[c+1]. One thread per slot
// s in [0, n]: slot s is the first slot of every cell in (key[s-1], key[s]]
// (slot n: of every cell after the last key, up to ncells), so each entry is
// written exactly once. Runs longer than a warp (empty regions of the grid;
// neighbouring slots often own one each, e.g. the empty rows between two walls)
// are queued in shared memory and written by the whole block, 256 entries at a
// time. Entries past `cap` (the table's last index) are never written.
constexpr int kCellStartThreads = 256;

__global__ void __launch_bounds__(kCellStartThreads)
    k_cell_start(const unsigned* __restrict__ keys, int n, const int* __restrict__ ncells_total,
                 int cap, int* __restrict__ start,
    const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    __shared__ int q_lo[kCellStartThreads], q_hi[kCellStartThreads], q_s[kCellStartThreads];
    __shared__ int q_n;
    if (threadIdx.x == 0) q_n = 0;
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = s <= n;
    int lo = 0, hi = -1;  // cells [lo, hi] start at slot s
    if (valid) {
        const int nc = min(*ncells_total, cap);
        lo = (s == 0) ? 0 : (int)__ldg(keys + s - 1) + 1;
        hi = (s == n) ? nc : (int)__ldg(keys + s);
        hi = min(hi, cap);
    }
    if (hi - lo + 1 <= 32) {
        for (int c = lo; c <= hi; ++c) start[c] = s;
    } else {
        const int k = atomicAdd(&q_n, 1);  // at most one entry per thread
        q_lo[k] = lo;
        q_hi[k] = hi;
        q_s[k] = s;
    }
    __syncthreads();
    const int nq = q_n;
    for (int q = 0; q < nq; ++q) {
        const int bs = q_s[q], bhi = q_hi[q];
        for (int c = q_lo[q] + (int)threadIdx.x; c <= bhi; c += kCellStartThreads) start[c] = bs;
    }
}

// ---------------------------------------------------------------------------
// State movement
// ---------------------------------------------------------------------------
// Caller arrays -> A, in two parts: what the grid and sort read (positions,
// h; the 2D mass rides in xh.z) and the rest. The input density and pressure
// of a fluid particle are read only where the step uses them (rho_fl, p_fl):
// summation density and the equation of state replace them otherwise.
template <int DIM>
__device__ __forceinline__ void gather_pos_one(int i, const float* __restrict__ x,
                                               const float* __restrict__ m,
                                               const float* __restrict__ h, StateA& A) {
    if (DIM == 2) A.xh[i] = make_float4(x[2 * i], x[2 * i + 1], m[i], h[i]);
    else A.xh[i] = make_float4(x[3 * i], x[3 * i + 1], x[3 * i + 2], h[i]);
    A.id[i] = i;
}
template <int DIM>
__device__ __forceinline__ void gather_rest_one(int i, const float* __restrict__ v,
                                                const float* __restrict__ m,
                                                const float* __restrict__ rho,
                                                const float* __restrict__ p,
                                                const float* __restrict__ u,
                                                const int* __restrict__ itype,
                                                const float* __restrict__ dvdt,
                                                const float* __restrict__ dudt, StateA& A,
                                                bool rho_fl, bool p_fl) {
    const int it = itype[i];
    if (DIM == 2) {
        A.vm[i] = make_float4(v[2 * i], v[2 * i + 1], 0.f, 0.f);
        A.ap[i] = dvdt ? make_float4(dvdt[2 * i], dvdt[2 * i + 1], 0.f, dudt[i])
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        A.vm[i] = make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], m[i]);
        A.ap[i] = dvdt ? make_float4(dvdt[3 * i], dvdt[3 * i + 1], dvdt[3 * i + 2], dudt[i])
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    A.u[i] = u[i];
    A.rho[i] = (rho_fl || it <= 0) ? rho[i] : 0.f;
    A.p[i] = (p_fl || it <= 0) ? p[i] : 0.f;
    A.itype[i] = it;
}

template <int DIM>
__global__ void k_gather_in(const float* __restrict__ x, const float* __restrict__ v,
                            const float* __restrict__ m, const float* __restrict__ rho,
                            const float* __restrict__ p, const float* __restrict__ u,
                            const float* __restrict__ h, const int* __restrict__ itype,
                            const float* __restrict__ dvdt, const float* __restrict__ dudt,
                            StateA A, int n, const int* __restrict__ inst0, int rho_fl,
                            int p_fl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (inst0) A.inst[i] = inst0[i];
    gather_pos_one<DIM>(i, x, m, h, A);
    gather_rest_one<DIM>(i, v, m, rho, p, u, itype, dvdt, dudt, A, rho_fl, p_fl);
}

// The two parts apart: a host-memory call loads the positions first and the
// rest from a few CTAs on a second stream while the sort runs.
template <int DIM>
__global__ void k_gather_pos(const float* __restrict__ x, const float* __restrict__ m,
                             const float* __restrict__ h, StateA A, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) gather_pos_one<DIM>(i, x, m, h, A);
}
template <int DIM>
__global__ void k_gather_rest(const float* __restrict__ v, const float* __restrict__ m,
                              const float* __restrict__ rho, const float* __restrict__ p,
                              const float* __restrict__ u, const int* __restrict__ itype,
                              const float* __restrict__ dvdt, const float* __restrict__ dudt,
                              StateA A, int n, int rho_fl, int p_fl) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        gather_rest_one<DIM>(i, v, m, rho, p, u, itype, dvdt, dudt, A, rho_fl, p_fl);
}

// Positions and h only (neighbour / cell-id entry points).
template <int DIM>
__global__ void k_load_xh(const float* __restrict__ x, const float* __restrict__ h, StateA A,
                          int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (DIM == 2) A.xh[i] = make_float4(x[2 * i], x[2 * i + 1], 0.f, h[i]);
    else A.xh[i] = make_float4(x[3 * i], x[3 * i + 1], x[3 * i + 2], h[i]);
    A.id[i] = i;
}

// inv[id[s]] = s: the cell-order slot of each caller index.
// dst[id[s]] = src[s]: a slot-order array back to caller order.
__global__ void k_scatter_by_id(const float* __restrict__ src, const int* __restrict__ id,
                                float* __restrict__ dst, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) dst[id[s]] = src[s];
}

// Smoothing lengths of A in caller order.
__global__ void k_hsml_out(StateA A, float* __restrict__ h, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) h[A.id[s]] = A.xh[s].w;
}

__global__ void k_invert_ids(const int* __restrict__ id, int* __restrict__ inv, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) inv[id[s]] = s;
}

// A -> caller arrays walking the caller order: the form for caller arrays in
// host memory that the device maps, where every write crosses the host link.
// The interleaved x, v, dv/dt of a block's kScatterSeq particles are staged in
// shared memory and written as one contiguous run each (consecutive threads,
// consecutive addresses: whole lines, no alignment needed); the reads of A are
// the scattered side.
constexpr int kScatterSeq = 256;

// The output density and pressure of a summation-density iteration, final
// after the density pass (the force pass copies them): written to the caller's
// arrays from a few CTAs on a second stream while the force pass runs. inv is
// the inverse of B.id.
__global__ void k_scatter_rp(StateB B, const int* __restrict__ inv, int n, float* __restrict__ rho,
                             float* __restrict__ p) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = inv[i];
        rho[i] = B.rp[s].x;
        p[i] = B.p[s];
    }
}

template <int DIM>
__global__ void __launch_bounds__(kScatterSeq)
    k_scatter_out_seq(StateA A, const int* __restrict__ inv, int n, float* __restrict__ x,
                      float* __restrict__ v, float* __restrict__ rho, float* __restrict__ p,
                      float* __restrict__ u, float* __restrict__ dvdt,
                      float* __restrict__ dudt) {
    __shared__ float sx[DIM * kScatterSeq], sv[DIM * kScatterSeq], sa[DIM * kScatterSeq];
    const int t = threadIdx.x;
    const int i0 = blockIdx.x * kScatterSeq;
    const int i = i0 + t;
    if (i < n) {
        const int s = inv[i];
        const float4 a = A.xh[s], b = A.vm[s], r = A.ap[s];
        sx[DIM * t] = a.x;
        sx[DIM * t + 1] = a.y;
        sv[DIM * t] = b.x;
        sv[DIM * t + 1] = b.y;
        sa[DIM * t] = r.x;
        sa[DIM * t + 1] = r.y;
        if (DIM == 3) {
            sx[3 * t + 2] = a.z;
            sv[3 * t + 2] = b.z;
            sa[3 * t + 2] = r.z;
        }
        dudt[i] = r.w;
        u[i] = A.u[s];
        if (rho) rho[i] = A.rho[s];  // (null: written earlier, k_scatter_rp)
        if (p) p[i] = A.p[s];
    }
    __syncthreads();
    const int cnt = DIM * min(kScatterSeq, n - i0);
    const size_t o = (size_t)DIM * i0;
    for (int k = t; k < cnt; k += kScatterSeq) {
        x[o + k] = sx[k];
        v[o + k] = sv[k];
        dvdt[o + k] = sa[k];
    }
}

template <int DIM>
__global__ void k_scatter_out(StateA A, int n, float* __restrict__ x, float* __restrict__ v,
                              float* __restrict__ rho, float* __restrict__ p,
                              float* __restrict__ u, float* __restrict__ dvdt,
                              float* __restrict__ dudt) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = A.id[s];
    const float4 a = A.xh[s], b = A.vm[s], r = A.ap[s];
    x[DIM * i] = a.x;
    x[DIM * i + 1] = a.y;
    v[DIM * i] = b.x;
    v[DIM * i + 1] = b.y;
    dvdt[DIM * i] = r.x;
    dvdt[DIM * i + 1] = r.y;
    if (DIM == 3) {
        x[3 * i + 2] = a.z;
        v[3 * i + 2] = b.z;
        dvdt[3 * i + 2] = r.z;
    }
    dudt[i] = r.w;
    u[i] = A.u[s];
    rho[i] = A.rho[s];
    p[i] = A.p[s];
}

// Cell-ordered working set + leapfrog predictor (time_integration.f:136-154).
template <int DIM>
// An iteration that does not sort keeps the slot order (perm = identity).
// only_sorted: an iteration that does not sort skips the copy (the passes of
// such an iteration read A themselves, FusedSrc).
__global__ void k_reorder_dim(StateA A, const int* __restrict__ perm, StateB B, StepArgs S,
                              int n, const int* __restrict__ resort = nullptr,
                              bool only_sorted = false) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const bool sorted = !sort_skipped(resort);
    if (only_sorted && !sorted) return;
    const int j = sorted ? perm[s] : s;
    const float4 xh = A.xh[j];
    if (sorted && B.xsort) B.xsort[s] = xh;
    float4 vm = A.vm[j];
    float u = A.u[j];
    const int it = A.itype[j];
    B.vmin[s] = make_float4(vm.x, vm.y, vm.z, u);
    float ulo = 0.f;
    if (it > 0 && S.hdt != 0.f) {
        const float4 ap = A.ap[j];
        vm.x = fmaf(S.hdt, ap.x, vm.x);
        vm.y = fmaf(S.hdt, ap.y, vm.y);
        if (DIM == 3) vm.z = fmaf(S.hdt, ap.z, vm.z);
        // u + dt/2 du kept as hi + lo: art_heat differences u_i - u_j of nearly
        // equal energies would otherwise carry the rounding of u_half.
        const sph::ff uh = sph::two_sum(u, __fmul_rn(S.hdt, ap.w));
        u = uh.hi;
        ulo = uh.lo;
        if (u < 0.f) {
            u = 0.f;
            ulo = 0.f;
        }
    }
    if (B.ulo) B.ulo[s] = ulo;
    // Continuity density: rho + dt/2 drho/dt as hi + lo (time_integration.f:
    // 144-147), the start density kept for the corrector.
    float rho = A.rho[j], rlo = 0.f;
    if (B.q) B.q[s] = rho;
    if (S.dform == 1 && it > 0 && S.hdt != 0.f) {
        const sph::ff rh = sph::two_sum(rho, __fmul_rn(S.hdt, A.drho[j]));
        rho = rh.hi;
        rlo = rh.lo;
    }
    if (B.rlo) B.rlo[s] = rlo;
    B.xh[s] = xh;
    B.vm[s] = vm;
    B.rp[s] = make_float4(rho, 0.f, u, 0.f);
    B.p[s] = A.p[j];
    B.itype[s] = it;
    B.id[s] = A.id[j];
}

// Positions in cell order on an iteration that sorts (B.xsort), read by the
// list build as contiguous candidate ranges.
__global__ void k_sorted_positions(StateA A, const int* __restrict__ perm, StateB B, int n,
                                   const int* __restrict__ resort) {
    if (sort_skipped(resort)) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    B.xsort[s] = A.xh[perm[s]];
}

// Positions only (neighbour entry point).
__global__ void k_reorder_xh(StateA A, const int* __restrict__ perm, StateB B, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int j = perm[s];
    B.xh[s] = A.xh[j];
    B.id[s] = A.id[j];
}

// ---------------------------------------------------------------------------
// Batched grid, hash and reorder (one cell grid per instance).
// ---------------------------------------------------------------------------
// Bbox partial {min[3], max[3], max h} of every work item.
__global__ void __launch_bounds__(kPassThreads)
    k_bbox_items(const float4* __restrict__ xh, const WorkItem* __restrict__ items, int dim,
                 float* __restrict__ part) {
    const WorkItem w = items[blockIdx.x];
    const int s = w.s0 + threadIdx.x;
    float v[7] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f};
    if (s < w.s1) {
        const float4 a = xh[s];
        v[0] = v[3] = a.x;
        v[1] = v[4] = a.y;
        if (dim == 3) v[2] = v[5] = a.z;
        v[6] = a.w;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const float t = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = (k < 3) ? fminf(v[k], t) : fmaxf(v[k], t);
        }
    __shared__ float sw[kPassThreads / 32][7];
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 7; ++k) sw[threadIdx.x >> 5][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 7) {
        const int k = threadIdx.x;
        float r = sw[0][k];
        for (int w2 = 1; w2 < kPassThreads / 32; ++w2) r = (k < 3) ? fminf(r, sw[w2][k]) : fmaxf(r, sw[w2][k]);
        part[blockIdx.x * 8 + k] = r;
    }
}

// Grid of instance blockIdx.x from the partials of its items.
__global__ void __launch_bounds__(256)
    k_bbox_final_batch(const float* __restrict__ part, const int* __restrict__ inst_items,
                       const DevParams* __restrict__ params, DevGrid* __restrict__ grids,
                       int* __restrict__ ncells_inst, unsigned* __restrict__ flags) {
    __shared__ float sv[7][256];
    const int k = blockIdx.x;
    float v[7] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f};
    for (int b = inst_items[k] + threadIdx.x; b < inst_items[k + 1]; b += blockDim.x)
        for (int q = 0; q < 7; ++q)
            v[q] = (q < 3) ? fminf(v[q], part[b * 8 + q]) : fmaxf(v[q], part[b * 8 + q]);
    for (int q = 0; q < 7; ++q) sv[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int q = 0; q < 7; ++q)
                sv[q][threadIdx.x] = (q < 3) ? fminf(sv[q][threadIdx.x], sv[q][threadIdx.x + st])
                                             : fmaxf(sv[q][threadIdx.x], sv[q][threadIdx.x + st]);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const float mm[7] = {sv[0][0], sv[1][0], sv[2][0], sv[3][0], sv[4][0], sv[5][0], sv[6][0]};
    unsigned fl = 0;
    DevGrid g = grid_from_bbox(mm, params[k], (long long)1 << 30, fl);
    grids[k] = g;
    ncells_inst[k] = g.ok ? g.ncells : 0;
    if (fl) atomicOr(flags, fl);
}

// Cell offsets of the instances in the shared table (exclusive scan of their
// cell counts); a total above the table's capacity disables every grid.
__global__ void __launch_bounds__(1024)
    k_cell_offsets(const int* __restrict__ ncells_inst, int n_inst, long long capacity,
                   DevGrid* __restrict__ grids, int* __restrict__ total_cells,
                   unsigned* __restrict__ flags) {
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_total;
    const int per = (n_inst + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(b + per, n_inst);
    unsigned sum = 0;
    for (int k = b; k < e; ++k) sum += (unsigned)ncells_inst[k];
    unsigned off = block_excl_scan<1024>(sum, s_warp, &s_total);
    const bool over = (long long)s_total > capacity;
    for (int k = b; k < e; ++k) {
        grids[k].cell_off = over ? 0 : (int)off;
        if (over) grids[k].ok = 0;
        off += (unsigned)ncells_inst[k];
    }
    if (threadIdx.x == 0) {
        *total_cells = over ? (int)capacity : (int)s_total;
        if (over) atomicOr(flags, (unsigned)FLAG_GRID_OVERFLOW);
    }
}

// Cell key of every slot under its instance's grid + digit-0 tile histogram.
template <int DIM>
__global__ void __launch_bounds__(kSortThreads)
    k_hash_batch(const float4* __restrict__ xh, const int* __restrict__ inst, int n,
                 const DevGrid* __restrict__ grids, unsigned* __restrict__ keys,
                 unsigned* __restrict__ hist, int num_tiles) {
    __shared__ unsigned sh[kRadix];
    sh[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        int i = base + k * kSortThreads + threadIdx.x;
        if (i < n) {
            const DevGrid g = grids[inst[i]];
            unsigned key = cell_key<DIM>(xh[i], g);
            keys[i] = key;
            atomicAdd(&sh[key & 255u], 1u);
        }
    }
    __syncthreads();
    hist[threadIdx.x * num_tiles + blockIdx.x] = sh[threadIdx.x];
}

// Cell-ordered working set + leapfrog predictor, per-instance time step.
template <int DIM>
__global__ void k_reorder_batch(StateA A, const int* __restrict__ perm, StateB B,
                                const DevParams* __restrict__ params, const int* __restrict__ its,
                                int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int j = perm[s];
    const int k = A.inst[j];
    const float hdt = (*its == 1) ? 0.f : 0.5f * __ldg(&params[k].dt);
    const float4 xh = A.xh[j];
    float4 vm = A.vm[j];
    float u = A.u[j];
    const int it = A.itype[j];
    B.vmin[s] = make_float4(vm.x, vm.y, vm.z, u);
    float ulo = 0.f;
    if (it > 0 && hdt != 0.f) {
        const float4 ap = A.ap[j];
        vm.x = fmaf(hdt, ap.x, vm.x);
        vm.y = fmaf(hdt, ap.y, vm.y);
        if (DIM == 3) vm.z = fmaf(hdt, ap.z, vm.z);
        const sph::ff uh = sph::two_sum(u, __fmul_rn(hdt, ap.w));
        u = uh.hi;
        ulo = uh.lo;
        if (u < 0.f) {
            u = 0.f;
            ulo = 0.f;
        }
    }
    B.ulo[s] = ulo;
    B.xh[s] = xh;
    B.vm[s] = vm;
    B.rp[s] = make_float4(A.rho[j], 0.f, u, 0.f);
    B.p[s] = A.p[j];
    B.itype[s] = it;
    B.id[s] = A.id[j];
    B.inst[s] = k;
}

__global__ void k_advance_its(int* its) { *its += 1; }

// ---------------------------------------------------------------------------
// Neighbour-cell iteration
// ---------------------------------------------------------------------------
struct CellCoord {
    int c[3];
};

template <int DIM>
__device__ __forceinline__ CellCoord decode_key(unsigned key, const DevGrid& g) {
    CellCoord cc;
    key -= (unsigned)g.cell_off;
    cc.c[0] = (int)(key % (unsigned)g.n[0]);
    unsigned t = key / (unsigned)g.n[0];
    if (DIM == 2) {
        cc.c[1] = (int)t;
        cc.c[2] = 0;
    } else {
        cc.c[1] = (int)(t % (unsigned)g.n[1]);
        cc.c[2] = (int)(t / (unsigned)g.n[1]);
    }
    return cc;
}

// Difference x_i - x_j (minimum image) and the exact pair test.
template <int DIM>
__device__ __forceinline__ bool pair_delta(const float4& xi, const float4& xj, const DevGrid& g,
                                           float* d, float& dr2) {
    d[0] = __fsub_rn(xi.x, xj.x);
    d[1] = __fsub_rn(xi.y, xj.y);
    d[2] = (DIM == 3) ? __fsub_rn(xi.z, xj.z) : 0.f;
#pragma unroll
    for (int a = 0; a < DIM; ++a)
        if (g.periodic[a]) d[a] = sph::min_image(d[a], g.L[a], g.half[a]);
    dr2 = sph::dist2_exact<DIM>(d);
    return sph::within_support(dr2, xi.w, xj.w);
}

// Exact pair difference x_i - x_j = dh + dl per axis, minimum image applied
// exactly on periodic axes (the wrap decision is the pair test's).
template <int DIM>
__device__ __forceinline__ void exact_delta(const float4& xi, const float4& xj, const DevGrid& g,
                                            float* dh, float* dl) {
    const float a[3] = {xi.x, xi.y, xi.z}, b[3] = {xj.x, xj.y, xj.z};
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        sph::ff s = sph::two_diff(a[k], b[k]);
        if (g.periodic[k]) {
            if (s.hi > g.half[k]) {
                sph::ff u = sph::two_sum(s.hi, -g.L[k]);
                s.hi = u.hi;
                s.lo = __fadd_rn(s.lo, u.lo);
            } else if (s.hi < -g.half[k]) {
                sph::ff u = sph::two_sum(s.hi, g.L[k]);
                s.hi = u.hi;
                s.lo = __fadd_rn(s.lo, u.lo);
            }
        }
        dh[k] = s.hi;
        dl[k] = s.lo;
    }
}

// On periodic axes the pair test's difference is rounded twice ((x_i - x_j)
// then +- L); the force passes use the correctly rounded one instead.
template <int DIM>
__device__ __forceinline__ void refine_periodic(const float4& xi, const float4& xj,
                                                const DevGrid& g, float* d, float& dr2) {
    if (!(g.periodic[0] | g.periodic[1] | g.periodic[2])) return;
    float dh[3], dl[3];
    exact_delta<DIM>(xi, xj, g, dh, dl);
#pragma unroll
    for (int k = 0; k < DIM; ++k)
        if (g.periodic[k]) d[k] = __fadd_rn(dh[k], dl[k]);
    dr2 = sph::dist2_exact<DIM>(d);
}

template <int DIM>
__device__ __forceinline__ sph::ff ff_pow_dim(sph::ff ih) {
    sph::ff a = sph::ff_sqr(ih);
    if (DIM == 3) a = sph::ff_mul(a, ih);
    return a;
}

template <int DIM>
__device__ __forceinline__ float pow_grad(float ih) {
    float ih2 = __fmul_rn(ih, ih);
    float ih4 = __fmul_rn(ih2, ih2);
    return DIM == 2 ? ih4 : __fmul_rn(ih4, ih);
}

// ---------------------------------------------------------------------------
// Candidate cursor and per-thread neighbour lists.
//
// A pass walks the candidate slots of its particle row by row (a "row" is the
// contiguous slot range of the 3 x-adjacent cells at one (y, z), or a single
// cell on a periodic x axis), tests them, and appends the neighbours to a list
// in shared memory (slot-major [t][thread], conflict-free). The physics then
// runs over the lists in a warp-converged loop, so lanes do not idle on
// candidates that failed the pair test. Lists hold kListCap entries; a
// particle with more neighbours takes several rounds.
// ---------------------------------------------------------------------------
constexpr int kListCap = 32;      // force pass list
// Neighbour-list entries per particle of a lazily sorting context (pairs
// within h_i + h_j + skin; the lattice counts are ~20 / ~85 at a 10% skin,
// ~28 / ~125 at 40%); a particle with more walks its cells. Each must fit the
// neighbour bits of one lane (mask_words * 32).
constexpr int kListCap2 = 64;
constexpr int kListCap3 = 256;
static_assert(kListCap2 <= 32 * mask_words<2>() && kListCap3 <= 32 * mask_words<3>(),
              "a list's neighbour bits fit one lane's mask");
constexpr int kListCapD = 24;     // density pass: near and far lists each
// With neighbour lists only the particles whose list overflowed fill these
// candidate lists: smaller ones leave the SM's shared storage to L1.
constexpr int kListCapLst = 4;
template <bool LST>
__host__ __device__ constexpr int cap_density() {
    return LST ? kListCapLst : kListCapD;
}
template <bool LST>
__host__ __device__ constexpr int cap_force() {
    return LST ? kListCapLst : kListCap;
}
constexpr int kTestBatch = 4;     // candidate loads issued together

// List entries whose loads a listed particle issues together, measured best:
// the force pass 4 in 2D, 2 in 3D (its registers); the density pass, which
// also loads the next batch's entries before evaluating this one, 2.
template <int DIM>
__host__ __device__ constexpr int list_batch() {
    return DIM == 2 ? 4 : 2;
}
template <int DIM>
__host__ __device__ constexpr int density_list_batch() {
    return 2;
}
// The 2D density pass's far entries (FP32 weights).
__host__ __device__ constexpr int density_far_batch() {
    return 2;
}

// A warp's neighbour-list rows (entry r of its 32 slots is one 128-byte run
// at nlist + r * lstride + s0) requested into L2 at once, one row per lane, so
// the walk's coalesced entry loads hit L2 instead of waiting on DRAM.

__device__ __forceinline__ void prefetch_list_rows(const int* nlist, int lstride, int s, int lc) {
    const int lane = (int)(threadIdx.x & 31u);
    const int rows = __reduce_max_sync(0xffffffffu, lc > 0 ? lc : 0);
    const int s0 = __shfl_sync(0xffffffffu, s, 0);
    for (int r = lane; r < rows; r += 32)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(nlist + (size_t)r * lstride + s0));
}

// A slot's list counts from ncount: near entries (-1: no list, walk the
// cells) and far entries.
__device__ __forceinline__ int list_near(int packed) { return packed >= 0 ? (packed & 0xffff) : -1; }
__device__ __forceinline__ int list_far(int packed) { return packed >= 0 ? (packed >> 16) : 0; }
// 2D density pairs with q = r/h < near_q() are evaluated in float-float, the
// others (W below ~1% of W(0) each, ~8 of ~20 pairs) in FP32. In 3D every pair
// is float-float: ~50 of ~80 pairs lie beyond q = 1.6, and the FP32 rounding of
// their sum (a few 1e-7 of ~1% of rho each) would exceed 1e-5 of the pressure
// of a quiescent flow, whose p is ~1e-5 of rho0 c0^2.
template <int DIM>
__host__ __device__ constexpr float near_q() {
    return DIM == 2 ? 1.6f : 2.0f;
}
// The 2D neighbour lists' split (at the sort): float-float below q = 1.5, under
// a lattice's second neighbours (r = 2 dx, q = 1.54 at h = 1.3 dx), which take
// the FP32 path with the farther ones: 2% of the step for a one-step pressure
// error of 1.5e-6 instead of 5.7e-7 at the cell walk's 1.6 (gate 1e-5).
__host__ __device__ constexpr float list_near_q2() { return 1.5f; }

// Candidate rows: for each (dy, dz) in [-f, f]^(DIM-1) the cells cx-f..cx+f of
// that row are consecutive keys, so one contiguous slot range. On a periodic x
// axis the part past either end (at most one side, as n[0] >= 2f + 1) is a
// second piece. Rows come in (dz, dy, piece) order, the same for every pass.
struct Cursor {
    int k, ke;  // current slot range [k, ke)
    int st;     // row state: dy + 8 (bits 0-3), dz + 8 (bits 4-7), piece (bit 8),
                // piece 0 the in-range cells, 1 the wrapped ones
};

template <int DIM>
__device__ __forceinline__ Cursor cursor_begin(const DevGrid& g) {
    Cursor c;
    c.k = c.ke = 0;
    const int dy = -g.reach - 1, dz = (DIM == 3) ? -g.reach : 0;
    c.st = (dy + 8) | ((dz + 8) << 4) | (1 << 8);
    return c;
}

// Advances to the next non-empty range; false when the candidates are
// exhausted (and stays false).
template <int DIM>
__device__ __forceinline__ bool cursor_next(const DevGrid& g, const int* __restrict__ start,
                                            const CellCoord& cc, Cursor& cu) {
    const int f = g.reach;
    const bool px = g.periodic[0] != 0;
    int dy = (cu.st & 15) - 8, dz = ((cu.st >> 4) & 15) - 8, pc = cu.st >> 8;
    bool found = false;
    for (;;) {
        if (px && pc == 0) {
            pc = 1;
        } else {
            pc = 0;
            if (++dy > f) {
                if (DIM == 2 || dz >= f) {
                    dy = f + 1;
                    cu.k = cu.ke = 0;
                    break;
                }
                dy = -f;
                ++dz;
            }
        }
        int cy = cc.c[1] + dy;
        if (cy < 0 || cy >= g.n[1]) {
            if (!g.periodic[1]) continue;
            cy += (cy < 0) ? g.n[1] : -g.n[1];
        }
        int cz = 0;
        if (DIM == 3) {
            cz = cc.c[2] + dz;
            if (cz < 0 || cz >= g.n[2]) {
                if (!g.periodic[2]) continue;
                cz += (cz < 0) ? g.n[2] : -g.n[2];
            }
        }
        const int row = g.cell_off + (cz * g.n[1] + cy) * g.n[0];
        const int cx = cc.c[0];
        int c0, c1;
        if (pc == 0) {
            c0 = max(cx - f, 0);
            c1 = min(cx + f, g.n[0] - 1);
        } else if (cx - f < 0) {
            c0 = cx - f + g.n[0];
            c1 = g.n[0] - 1;
        } else if (cx + f >= g.n[0]) {
            c0 = 0;
            c1 = cx + f - g.n[0];
        } else {
            continue;
        }
        const int kb = __ldg(start + row + c0), ke = __ldg(start + row + c1 + 1);
        if (kb < ke) {
            cu.k = kb;
            cu.ke = ke;
            found = true;
            break;
        }
    }
    cu.st = (dy + 8) | ((dz + 8) << 4) | (pc << 8);
    return found;
}

// Calls fn(k) for every candidate slot k of the particle in cell cc (its own
// slot included; callers skip it).
template <int DIM, class F>
__device__ __forceinline__ void for_candidates(const DevGrid& g, const int* __restrict__ start,
                                               const CellCoord& cc, F&& fn) {
    Cursor cu = cursor_begin<DIM>(g);
    while (cursor_next<DIM>(g, start, cc, cu))
        for (int k = cu.k; k < cu.ke; ++k) fn(k);
}

// Periodic wrap of a drifted coordinate (same branch order as the oracle).
__device__ __forceinline__ float wrap_axis(float c, const DevParams& P, int d, bool& outside) {
    if (!(c < P.period_hi[d])) c = __fsub_rn(c, P.period_L[d]);
    else if (c < P.period_lo[d]) c = __fadd_rn(c, P.period_L[d]);
    if (!(c >= P.period_lo[d] && c < P.period_hi[d])) outside = true;
    return c;
}

__device__ __forceinline__ float fast_sqrt_pos(float x) {
    return x > 0.f ? x * rsqrtf(x) : 0.f;
}

// Lanes of one particle: TPP consecutive threads split its candidates, lane
// `sub` taking slots kb + sub, kb + sub + TPP, ... of every candidate range.
template <int TPP>
__device__ __forceinline__ unsigned group_mask() {
    const unsigned lane = threadIdx.x & 31u;
    return (TPP == 1) ? (1u << lane) : (((1u << TPP) - 1u) << (lane & ~(unsigned)(TPP - 1)));
}

// Sum over the lanes of one particle (xor butterfly; every lane gets the same
// value, a + b being commutative).
template <int TPP>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = 1; o < TPP; o <<= 1) v += __shfl_xor_sync(group_mask<TPP>(), v, o);
    return v;
}

// The lane's candidates left in the cursor's current range.
template <int TPP>
__device__ __forceinline__ int lane_len(const Cursor& cu) {
    return cu.k < cu.ke ? (cu.ke - cu.k + TPP - 1) / TPP : 0;
}

// Candidates of a CTA staged in shared memory (staged passes, one thread per
// particle, no periodic axis): slot k of stencil row r sits at k + shift[r].
struct StageView {
    const float4* x;    // xh of the staged slots
    const float4* v;    // density 3D: vm (mass); force 2D: vr; force 3D: vm
    const float4* r;    // force 3D: rp
    const int* shift;   // per stencil row, cursor order
};

// The integrated state A of a lazily sorting context with lean physics, read
// by the passes on the iterations that do not sort: they skip the reorder
// copy into B, apply the leapfrog predictor (time_integration.f:136-154) on
// load, and the force pass writes the next state into the other A buffer.
// rs: the context's lazy-sort flags (which iterations sort).
struct FusedSrc {
    StateA A;
    const int* rs;
    float hdt;  // predictor half step of this iteration
};

// Stencil row of the cursor's current range (non-periodic grids: one piece
// per row), r = (dz + f) (2f + 1) + (dy + f).
template <int DIM>
__device__ __forceinline__ int cursor_row(const Cursor& cu, int f) {
    const int dy = (cu.st & 15) - 8, dz = ((cu.st >> 4) & 15) - 8;
    return DIM == 2 ? dy + f : (dz + f) * (2 * f + 1) + (dy + f);
}

// ---------------------------------------------------------------------------
// Pass 1: summation density (float-float near pairs), Tait EOS, div v.
// ---------------------------------------------------------------------------
// LEAN: the parameters have no physical viscosity and no artificial heat, so
// their operands and branches are compiled out.
// STG: the candidates come from the CTA's staged copy SV (LT: the list entry
// type, staged indices), else from global memory through L1.
// LST: a lazily sorting context's neighbour lists (B.nlist) replace the cell
// walk for slots whose list fits; those slots leave no neighbour bits (the
// force pass re-tests their lists).
// FUS: on iterations that do not sort, read the state from F.A (FusedSrc).
template <int DIM, int TPP = 1, int BS = kPassThreads, bool LEAN = false, bool OPT = false,
          bool STG = false, class LT = int, bool LST = false, bool FUS = false>
__device__ __forceinline__ void density_body(const StateB& B, const unsigned* __restrict__ keys,
                                             const int* __restrict__ start, const DevGrid& g,
                                             const DevParams& P, const int s, const bool valid,
                                             LT (*s_near)[BS], LT (*s_far)[BS],
                                             const StageView& SV = StageView{},
                                             const FusedSrc& F = FusedSrc{}) {
    static_assert(!STG || (TPP == 1 && LEAN && !OPT), "staged: one lane per particle, lean physics");
    static_assert(!LST || (TPP == 1 && !STG), "lists: one lane per particle, unstaged");
    static_assert(!FUS || (LST && LEAN && !OPT), "fused predictor: lists, lean physics");
    const int tid = threadIdx.x;
    const int sub = (TPP == 1) ? 0 : (tid & (TPP - 1));
    const bool need_div = !LEAN && P.heat_art != 0;
    const bool from_a = FUS && sort_skipped(F.rs);
    const float4* __restrict__ xsrc = from_a ? F.A.xh : B.xh;
    const float4* __restrict__ vsrc = from_a ? F.A.vm : B.vm;  // 3D masses (.w)
    float4 xi = make_float4(0.f, 0.f, 0.f, 1.f), vi = xi, rp = xi;
    float p = 0.f;
    int it_i = 0;
    bool fluid = false;
    if (valid && from_a) {
        xi = F.A.xh[s];
        it_i = F.A.itype[s];
        fluid = it_i > 0;
        vi = F.A.vm[s];
        p = F.A.p[s];
        rp = make_float4(F.A.rho[s], 0.f, 0.f, 0.f);
        if (fluid && F.hdt != 0.f) {  // predictor (k_reorder_dim's, same operations)
            const float4 ap = F.A.ap[s];
            vi.x = fmaf(F.hdt, ap.x, vi.x);
            vi.y = fmaf(F.hdt, ap.y, vi.y);
            if (DIM == 3) vi.z = fmaf(F.hdt, ap.z, vi.z);
        }
        if (DIM == 3) B.vm[s] = vi;  // the force pass reads neighbours' predicted v here
    } else if (valid) {
        xi = B.xh[s];
        rp = B.rp[s];
        p = B.p[s];
        it_i = B.itype[s];
        fluid = it_i > 0;
        vi = B.vm[s];
    }
    const bool work = valid && g.ok && (fluid || need_div);
    CellCoord cc = {{0, 0, 0}};
    if (work) cc = decode_key<DIM>(keys[s], g);
    const sph::ff kw = {P.kw_hi, P.kw_lo};
    const sph::ff ih_i = sph::ff_recip(xi.w);
    const sph::ff al_i = sph::ff_mul(kw, ff_pow_dim<DIM>(ih_i));
    const float mi = mass_of<DIM>(xi, vi);
    // Self density m_i W(0, h_i) (density.f:39-42), on the particle's first lane.
    sph::ff S = sph::ff_mul_f(al_i, mi);
    // Normalised summation (nor_density, density.f:65-158): the denominator
    // m_i W(0)/rho_i + sum_j m_j/rho_j W_ij on the start densities, float-float.
    const bool nor = OPT && P.density_form == 2 && fluid;
    sph::ff Wn = sph::ff{0.f, 0.f};
    if (nor) Wn = sph::ff_mul(S, sph::ff_recip(B.q[s]));
    if (sub != 0) S = Wn = sph::ff{0.f, 0.f};
    const float ihf = ih_i.hi;
    const float kgih_i = __fmul_rn(P.kg, pow_grad<DIM>(ihf));
    float divs = 0.f;
    constexpr int W = mask_words<DIM>() / TPP;  // mask words of this lane
    const size_t mlane = (size_t)s * TPP + sub;
    Cursor cu = cursor_begin<DIM>(g);
    bool done = !work;
    // (listed particles, LST, need no bits: the force pass re-tests their list)
    bool mask_on = work && fluid;
    int ord = 0;  // candidate ordinal (cursor order, self included)
    int wb = 0;   // the accumulator holds the bits of ordinals 32 wb .. 32 wb + 63
    unsigned long long cur = 0ull;
    int shift = 0;  // staged index - slot in the cursor's row
    const int lpk = (LST && work) ? __ldg(B.ncount + s) : -1;
    const int lc = list_near(lpk);  // near list entries (-1: walk the cells)
    const int lf = list_far(lpk);   // far list entries (2D)
    if (LST && lc >= 0) mask_on = false;
    if (LST) prefetch_list_rows(B.nlist, B.lstride, s, lc + lf);
    // A listed particle evaluates each list entry as it is read, the near
    // ones in float-float, the far ones (2D) like the cell walk's far pairs;
    // the kernel is zero beyond its support, so the entries need no pair
    // test: no candidate lists in shared memory, no second load. The cell
    // walk below serves the others.
    if (LST) {
        constexpr int NB = density_list_batch<DIM>();
        const int lcm = __reduce_max_sync(0xffffffffu, lc > 0 ? lc : 0);
        // (a lane past the last slot reads slot 0: its loads stay in bounds)
        auto entry = [&](int t) {
            return lc > 0 ? __ldg(B.nlist + (size_t)min(t, lc - 1) * B.lstride + s) : (valid ? s : 0);
        };
        int kn[NB];  // the next batch's entries, loaded one batch ahead
#pragma unroll
        for (int u = 0; u < NB; ++u) kn[u] = entry(u);
        for (int t0 = 0; t0 < lcm; t0 += NB) {
            int kb[NB];
            float4 xb[NB], vb[NB];
#pragma unroll
            for (int u = 0; u < NB; ++u) kb[u] = kn[u];
            if (t0 + NB < lcm) {
#pragma unroll
                for (int u = 0; u < NB; ++u) kn[u] = entry(t0 + NB + u);
            }
#pragma unroll
            for (int u = 0; u < NB; ++u) {
                xb[u] = __ldg(xsrc + kb[u]);
                vb[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (DIM == 3 || need_div) vb[u] = __ldg(vsrc + kb[u]);
            }
#pragma unroll
            for (int u = 0; u < NB; ++u) {
                const int k = kb[u];
                const float4 xj = xb[u];
                // no pair test: the kernel's support (W = 0 for q >= 2) drops the
                // entries beyond it
                bool in = t0 + u < lc;
                if (!LEAN && P.wall_model == 1 && __ldg(B.itype + k) != it_i) in = false;  // push only
                const float mj = mass_of<DIM>(xj, vb[u]);
                float dh[3], dl[3];
                exact_delta<DIM>(xi, xj, g, dh, dl);
                sph::ff ih = ih_i, al = al_i;
                if (xj.w != xi.w) {
                    ih = sph::ff_recip(__fmul_rn(0.5f, __fadd_rn(xi.w, xj.w)));
                    al = sph::ff_mul(kw, ff_pow_dim<DIM>(ih));
                }
                if (fluid) {
                    const sph::ff wm = sph::wendland_mw_ff<DIM, true>(dh, dl, ih, al, mj);
                    if (in) {
                        sph::ff_acc(S, wm);
                        if (nor) sph::ff_acc(Wn, sph::ff_mul(wm, sph::ff_recip(__ldg(B.q + k))));
                    }
                }
                if (need_div && in) {
                    const float4 vj = vb[u];
                    const float r2 = sph::dist2_exact<DIM>(dh);
                    float gw = sph::wendland_grad_factor<DIM>(
                        fast_sqrt_pos(r2), ih.hi, __fmul_rn(P.kg, pow_grad<DIM>(ih.hi)));
                    if (!(fast_sqrt_pos(r2) * ih.hi < 2.0f)) gw = 0.f;  // beyond the support
                    float vd = fmaf(vj.y - vi.y, dh[1], __fmul_rn(vj.x - vi.x, dh[0]));
                    if (DIM == 3) vd = fmaf(vj.z - vi.z, dh[2], vd);
                    divs = fmaf(mj * gw, vd, divs);
                }
            }
        }
        // 2D far entries (the rows after the near ones): FP32 weights with
        // the float-float prefactor, zero beyond the support.
        if constexpr (DIM == 2) {
            constexpr int NF = density_far_batch();
            const int lfm = __reduce_max_sync(0xffffffffu, lf);
            auto fentry = [&](int t) {
                return lf > 0 ? __ldg(B.nlist + (size_t)(lc + min(t, lf - 1)) * B.lstride + s)
                              : (valid ? s : 0);
            };
            int kf[NF];
#pragma unroll
            for (int u = 0; u < NF; ++u) kf[u] = fentry(u);
            for (int t0 = 0; t0 < lfm; t0 += NF) {
                int kb[NF];
                float4 xb[NF], vb[NF];
#pragma unroll
                for (int u = 0; u < NF; ++u) kb[u] = kf[u];
                if (t0 + NF < lfm) {
#pragma unroll
                    for (int u = 0; u < NF; ++u) kf[u] = fentry(t0 + NF + u);
                }
#pragma unroll
                for (int u = 0; u < NF; ++u) {
                    xb[u] = __ldg(xsrc + kb[u]);
                    vb[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (need_div) vb[u] = __ldg(vsrc + kb[u]);
                }
#pragma unroll
                for (int u = 0; u < NF; ++u) {
                    const int k = kb[u];
                    const float4 xj = xb[u];
                    bool in = t0 + u < lf;
                    if (!LEAN && P.wall_model == 1 && __ldg(B.itype + k) != it_i) in = false;  // push only
                    const float mj = mass_of<DIM>(xj, vb[u]);
                    float d[3], dr2;
                    pair_delta<DIM>(xi, xj, g, d, dr2);
                    refine_periodic<DIM>(xi, xj, g, d, dr2);
                    sph::ff ih = ih_i, al = al_i;
                    float kgih = kgih_i;
                    if (xj.w != xi.w) {
                        ih = sph::ff_recip(__fmul_rn(0.5f, __fadd_rn(xi.w, xj.w)));
                        al = sph::ff_mul(kw, ff_pow_dim<DIM>(ih));
                        kgih = P.kg * pow_grad<DIM>(ih.hi);
                    }
                    float r = 0.f;
                    if (dr2 > 0.f) {
                        const float rs = rsqrtf(dr2);
                        r = __fmul_rn(dr2, rs);
                        r = fmaf(fmaf(-r, r, dr2), 0.5f * rs, r);
                    }
                    const float q = fmaf(r, ih.hi, __fmul_rn(r, ih.lo));
                    if (fluid && in) {
                        float tt = fmaxf(fmaf(-0.5f, q, 1.0f), 0.0f);  // 0 beyond the support
                        tt = tt * tt;
                        tt = tt * tt;
                        const float f = tt * fmaf(2.0f, q, 1.0f);
                        const sph::ff c = sph::ff_mul_f(al, mj);
                        const float wm = fmaf(c.hi, f, __fmul_rn(c.lo, f));
                        sph::ff_acc(S, sph::ff{wm, 0.f});
                        if (nor) sph::ff_acc(Wn, sph::ff{__fdiv_rn(wm, __ldg(B.q + k)), 0.f});
                    }
                    if (need_div && in && q < 2.0f) {
                        const float4 vj = vb[u];
                        const float t3 = q - 2.0f;
                        const float gw = kgih * t3 * t3 * t3;
                        float vd = fmaf(vj.y - vi.y, d[1], __fmul_rn(vj.x - vi.x, d[0]));
                        divs = fmaf(mj * gw, vd, divs);
                    }
                }
            }
        }
        if (lc >= 0) done = true;
    }
    while (__any_sync(0xffffffffu, !done)) {
        int nn = 0, nf = 0;
        // Test phase: fill the near / far lists, kTestBatch candidate loads in flight.
        while (!done) {
            int kb[kTestBatch];
            int cnt;
            float4 xb[kTestBatch];
            if (cu.k >= cu.ke) {
                if (!cursor_next<DIM>(g, start, cc, cu)) {
                    done = true;
                    break;
                }
                if (STG) shift = SV.shift[cursor_row<DIM>(cu, g.reach)];
                if (TPP > 1) {
                    cu.k += sub;
                    continue;
                }
            }
            if (nn > cap_density<LST>() - kTestBatch || nf > cap_density<LST>() - kTestBatch) break;
            const int k0 = cu.k;
            cnt = min(kTestBatch, lane_len<TPP>(cu));
#pragma unroll
            for (int u = 0; u < kTestBatch; ++u) {
                const int ku = min(k0 + u * TPP, cu.ke - 1);
                kb[u] = k0 + u * TPP;
                xb[u] = STG ? SV.x[ku + shift] : __ldg(xsrc + ku);
            }
            cu.k += cnt * TPP;
            unsigned pb = 0u;  // pass bits of this batch
#pragma unroll
            for (int u = 0; u < kTestBatch; ++u) {
                float d[3], dr2;
                const int k = kb[u];
                if (u >= cnt || k == s || !pair_delta<DIM>(xi, xb[u], g, d, dr2)) continue;
                pb |= 1u << u;
                const float hs = xi.w + xb[u].w;  // near: q < near_q() with h = hs/2
                const LT e = (LT)(STG ? k + shift : k);
                if (DIM == 3 || dr2 < (0.25f * near_q<DIM>() * near_q<DIM>()) * hs * hs)
                    s_near[nn++][tid] = e;
                else
                    s_far[nf++][tid] = e;
            }
            if (ord - 32 * wb >= 32) {  // word wb is complete
                if (mask_on && wb < W) B.nmask[mask_word_index<W>(wb, B.mstride, mlane)] = (unsigned)cur;
                cur >>= 32;
                ++wb;
            }
            cur |= (unsigned long long)pb << (ord - 32 * wb);
            ord += cnt;
        }
        const int mn = __reduce_max_sync(0xffffffffu, nn);
        const int mf = __reduce_max_sync(0xffffffffu, nf);
        // Near pairs: float-float weights on the exact pair difference.
        for (int t = 0; t < mn; ++t) {
            if (t >= nn) continue;
            const int k = (int)s_near[t][tid];
            if (!LEAN && P.wall_model == 1 && __ldg(B.itype + k) != it_i) continue;  // push only
            const float4 xj = STG ? SV.x[k] : __ldg(xsrc + k);
            float4 vj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (DIM == 3 || need_div) vj = STG ? SV.v[k] : __ldg(vsrc + k);
            const float mj = mass_of<DIM>(xj, vj);
            float dh[3], dl[3];
            exact_delta<DIM>(xi, xj, g, dh, dl);
            sph::ff ih = ih_i, al = al_i;
            if (xj.w != xi.w) {
                ih = sph::ff_recip(__fmul_rn(0.5f, __fadd_rn(xi.w, xj.w)));
                al = sph::ff_mul(kw, ff_pow_dim<DIM>(ih));
            }
            if (fluid) {
                const sph::ff wm = sph::wendland_mw_ff<DIM>(dh, dl, ih, al, mj);
                sph::ff_acc(S, wm);
                if (nor) sph::ff_acc(Wn, sph::ff_mul(wm, sph::ff_recip(__ldg(B.q + k))));
            }
            if (need_div) {
                const float dr2 = sph::dist2_exact<DIM>(dh);
                const float gw = sph::wendland_grad_factor<DIM>(
                    fast_sqrt_pos(dr2), ih.hi, __fmul_rn(P.kg, pow_grad<DIM>(ih.hi)));
                float vd = fmaf(vj.y - vi.y, dh[1], __fmul_rn(vj.x - vi.x, dh[0]));
                if (DIM == 3) vd = fmaf(vj.z - vi.z, dh[2], vd);
                divs = fmaf(mj * gw, vd, divs);
            }
        }
        // Far pairs: FP32 weights (each below ~1% of the self term).
        for (int t = 0; t < mf; ++t) {
            if (t >= nf) continue;
            const int k = (int)s_far[t][tid];
            if (!LEAN && P.wall_model == 1 && __ldg(B.itype + k) != it_i) continue;
            const float4 xj = STG ? SV.x[k] : __ldg(xsrc + k);
            float4 vj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (DIM == 3 || need_div) vj = STG ? SV.v[k] : __ldg(vsrc + k);
            const float mj = mass_of<DIM>(xj, vj);
            float d[3], dr2;
            pair_delta<DIM>(xi, xj, g, d, dr2);
            refine_periodic<DIM>(xi, xj, g, d, dr2);
            // With uniform h and m every pair would share the rounding of
            // K m / h^dim and of 1/h: a bias that adds up over the far pairs.
            // So the prefactor and 1/h stay float-float, r is the
            // Newton-corrected square root, and q is rounded once.
            sph::ff ih = ih_i, al = al_i;
            float kgih = kgih_i;
            if (xj.w != xi.w) {
                ih = sph::ff_recip(__fmul_rn(0.5f, __fadd_rn(xi.w, xj.w)));
                al = sph::ff_mul(kw, ff_pow_dim<DIM>(ih));
                kgih = P.kg * pow_grad<DIM>(ih.hi);
            }
            float r = 0.f;
            if (dr2 > 0.f) {
                const float rs = rsqrtf(dr2);
                r = __fmul_rn(dr2, rs);
                r = fmaf(fmaf(-r, r, dr2), 0.5f * rs, r);
            }
            // one rounding of r (ih.hi + ih.lo): rounding r ih.hi first and then
            // adding r ih.lo would lose the correction, the same way for all pairs
            const float q = fmaf(r, ih.hi, __fmul_rn(r, ih.lo));
            if (fluid) {
                float tt = fmaf(-0.5f, q, 1.0f);
                tt = tt * tt;
                tt = tt * tt;
                const float f = tt * fmaf(2.0f, q, 1.0f);
                const sph::ff c = sph::ff_mul_f(al, mj);
                const float wm = fmaf(c.hi, f, __fmul_rn(c.lo, f));
                sph::ff_acc(S, sph::ff{wm, 0.f});
                if (nor) sph::ff_acc(Wn, sph::ff{__fdiv_rn(wm, __ldg(B.q + k)), 0.f});
            }
            if (need_div) {
                const float t3 = q - 2.0f;
                const float gw = kgih * t3 * t3 * t3;
                float vd = fmaf(vj.y - vi.y, d[1], __fmul_rn(vj.x - vi.x, d[0]));
                if (DIM == 3) vd = fmaf(vj.z - vi.z, d[2], vd);
                divs = fmaf(mj * gw, vd, divs);
            }
        }
    }
    if (TPP > 1) {  // the particle's lanes reach this point together
        const unsigned gm = group_mask<TPP>();
#pragma unroll
        for (int o = 1; o < TPP; o <<= 1) {
            const sph::ff t = {__shfl_xor_sync(gm, S.hi, o), __shfl_xor_sync(gm, S.lo, o)};
            sph::ff_acc(S, t);
            if (OPT) {
                const sph::ff tw = {__shfl_xor_sync(gm, Wn.hi, o), __shfl_xor_sync(gm, Wn.lo, o)};
                sph::ff_acc(Wn, tw);
            }
        }
        divs = group_sum<TPP>(divs);
    }
    if (!valid) return;
    if (mask_on) {
        if (ord > 32 * W) {
            B.nmask[mask_word_index<W>(0, B.mstride, mlane)] = ~0u;
            if (W > 1) B.nmask[mask_word_index<W>(1, B.mstride, mlane)] = ~0u;
        } else {
            for (; wb < W; ++wb) {
                B.nmask[mask_word_index<W>(wb, B.mstride, mlane)] = (unsigned)cur;
                cur >>= 32;
            }
        }
    }
    if (sub != 0) return;
    if (!work) {  // wall without div v (or no grid): fixed rho and p
        rp.y = (P.pa_sph == 1) ? __fdiv_rn(p, __fmul_rn(rp.x, rp.x)) : p;
        B.rp[s] = rp;
        if (DIM == 2) B.vr[s] = make_float4(vi.x, vi.y, rp.x, rp.y);
        return;
    }
    float rho = rp.x;
    if (fluid) {
        float drho;
        if (OPT && P.density_form == 1) {  // continuity: the predicted density
            drho = __fadd_rn(__fsub_rn(rp.x, P.rho0), B.rlo[s]);
        } else if (nor) {  // S / Wn to float-float accuracy
            const float qh = __fdiv_rn(S.hi, Wn.hi);
            const float res = fmaf(-qh, Wn.hi, S.hi) + S.lo - qh * Wn.lo;
            drho = __fadd_rn(__fsub_rn(qh, P.rho0), __fdiv_rn(res, Wn.hi));
        } else {
            drho = __fadd_rn(__fsub_rn(S.hi, P.rho0), S.lo);
        }
        p = sph::tait_poly(__fmul_rn(drho, P.inv_rho0), P.B);
        if (p < P.pmin) {  // eos.f90:277-280
            p = 0.f;
            drho = 0.f;
        }
        rho = __fadd_rn(P.rho0, drho);
        B.p[s] = p;
    }
    rp.x = rho;
    rp.y = (P.pa_sph == 1) ? __fdiv_rn(p, __fmul_rn(rho, rho)) : p;
    if (need_div) {
        // a mirror ghost's psi waits for its owner's density (k_ghost_sync)
        if (P.wall_model == 3 && !fluid) B.tds[s] = divs;
        const float divv = __fdiv_rn(divs, rho);
        rp.w = fmaf(P.ah_g2 * xi.w * xi.w, fabsf(divv) - divv, __fmul_rn(P.ah_g1 * xi.w, P.c0));
    }
    B.rp[s] = rp;
    if (DIM == 2) B.vr[s] = make_float4(vi.x, vi.y, rp.x, rp.y);
}

// ---------------------------------------------------------------------------
// Pass 1b: shear tensor (physical viscosity), every particle.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void shear_body(const StateB& B, const unsigned* __restrict__ keys,
                                           const int* __restrict__ start, const DevGrid& g,
                                           const DevParams& P, const int s, const bool valid) {
    if (!valid || !g.ok) return;
    const float4 xi = B.xh[s];
    const float4 vi = B.vm[s];
    const float rhoi = B.rp[s].x;
    const CellCoord cc = decode_key<DIM>(keys[s], g);
    const float ihf = __frcp_rn(xi.w);
    const float kgih_i = __fmul_rn(P.kg, pow_grad<DIM>(ihf));
    float t[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // xx yy zz xy xz yz
    const int it_i = B.itype[s];
    for_candidates<DIM>(g, start, cc, [&](int k) {
        if (k == s) return;
        if (P.wall_model == 1 && __ldg(B.itype + k) != it_i) return;  // push only
        const float4 xj = __ldg(B.xh + k);
        float d[3], dr2;
        if (!pair_delta<DIM>(xi, xj, g, d, dr2)) return;
        refine_periodic<DIM>(xi, xj, g, d, dr2);
        const float4 vj = __ldg(B.vm + k);
        const float mj = mass_of<DIM>(xj, vj);
        const float rhoj = __ldg(&B.rp[k].x);
        float ih = ihf, kgih = kgih_i;
        if (xj.w != xi.w) {
            ih = __frcp_rn(__fmul_rn(0.5f, __fadd_rn(xi.w, xj.w)));
            kgih = __fmul_rn(P.kg, pow_grad<DIM>(ih));
        }
        const float gw = sph::wendland_grad_factor<DIM>(__fsqrt_rn(dr2), ih, kgih);
        const float w0 = gw * d[0], w1 = gw * d[1], w2 = gw * d[2];
        const float dv0 = vj.x - vi.x, dv1 = vj.y - vi.y, dv2 = (DIM == 3) ? vj.z - vi.z : 0.f;
        float hxx, hyy, hzz = 0.f, hxy, hxz = 0.f, hyz = 0.f;
        // explicit fused / unfused products: every instantiation rounds alike
        const float e00 = __fmul_rn(dv0, w0), e11 = __fmul_rn(dv1, w1);
        if (DIM == 2) {
            hxx = fmaf(2.f, e00, -e11);
            hyy = fmaf(2.f, e11, -e00);
            hxy = fmaf(dv1, w0, __fmul_rn(dv0, w1));
        } else {
            const float e22 = __fmul_rn(dv2, w2);
            hxx = fmaf(2.f, e00, -e11) - e22;
            hyy = fmaf(2.f, e11, -e00) - e22;
            hzz = fmaf(2.f, e22, -e00) - e11;
            hyz = fmaf(dv2, w1, __fmul_rn(dv1, w2));
            hxz = fmaf(dv2, w0, __fmul_rn(dv0, w2));
            hxy = fmaf(dv1, w0, __fmul_rn(dv0, w1));
        }
        const float c = mj / rhoj;
        const float c23 = c * (2.f / 3.f);
        t[0] = fmaf(c23, hxx, t[0]);
        t[1] = fmaf(c23, hyy, t[1]);
        t[2] = fmaf(c23, hzz, t[2]);
        t[3] = fmaf(c, hxy, t[3]);
        t[4] = fmaf(c, hxz, t[4]);
        t[5] = fmaf(c, hyz, t[5]);
    });
    float q = fmaf(2.f * t[3], t[3], fmaf(t[1], t[1], __fmul_rn(t[0], t[0])));
    if (DIM == 3) q = fmaf(2.f * t[4], t[4], fmaf(2.f * t[5], t[5], fmaf(t[2], t[2], q)));
    B.tds[s] = 0.5f * P.eta / rhoi * q;
    const float sc = (P.pa_sph == 1) ? P.eta / (rhoi * rhoi) : P.eta;
    B.tau[s] = make_float4(sc * t[0], sc * t[1], sc * t[3], sc * t[2]);
    if (DIM == 3) B.tau2[s] = make_float4(sc * t[4], sc * t[5], 0.f, 0.f);
}

// ---------------------------------------------------------------------------
// Pass 2: forces, heat, leapfrog corrector. Reads B, writes the next state A.
// ---------------------------------------------------------------------------
// STG: neighbours from the CTA's staged copy SV (see density_body).
// FUS: on iterations that do not sort, the state comes from F.A (FusedSrc);
// A is then the other buffer, which receives the next state.
template <int DIM, int TPP = 1, int BS = kPassThreads, bool LEAN = false, bool OPT = false,
          bool STG = false, class LT = int, bool LST = false, bool FUS = false>
__device__ __forceinline__ void force_body(const StateB& B, const StateA& A,
                                           const unsigned* __restrict__ keys,
                                           const int* __restrict__ start, const DevGrid& g,
                                           const DevParams& P, const StepArgs& S,
                                           unsigned* __restrict__ flags, const int s,
                                           const bool valid, LT (*s_list)[BS],
                                           const StageView& SV = StageView{},
                                           const FusedSrc& F = FusedSrc{}) {
    static_assert(!STG || (TPP == 1 && LEAN && !OPT), "staged: one lane per particle, lean physics");
    static_assert(!LST || (TPP == 1 && !STG), "lists: one lane per particle, unstaged");
    static_assert(!FUS || (LST && LEAN && !OPT), "fused predictor: lists, lean physics");
    const int tid = threadIdx.x;
    const int sub = (TPP == 1) ? 0 : (tid & (TPP - 1));
    const bool from_a = FUS && sort_skipped(F.rs);
    const float4* __restrict__ xsrc = from_a ? F.A.xh : B.xh;
    float4 xi = make_float4(0.f, 0.f, 0.f, 1.f), vi = xi, rpi = xi;
    int it = 0;
    if (valid && from_a) {
        xi = F.A.xh[s];
        it = F.A.itype[s];
        vi = F.A.vm[s];
        rpi = B.rp[s];
        if (it > 0 && F.hdt != 0.f) {  // predictor, as the density pass applied it
            const float4 ap = F.A.ap[s];
            vi.x = fmaf(F.hdt, ap.x, vi.x);
            vi.y = fmaf(F.hdt, ap.y, vi.y);
            if (DIM == 3) vi.z = fmaf(F.hdt, ap.z, vi.z);
        }
    } else if (valid) {
        xi = B.xh[s];
        it = B.itype[s];
        vi = B.vm[s];
        rpi = B.rp[s];
    }
    // The next state goes to the slot of this sort, or with mirror ghosts
    // (wall_model 3) to the particle's own index, the ghosts being dropped.
    const bool ghosts = !LEAN && P.wall_model == 3;
    if (valid && (it <= 0 || !g.ok) && sub == 0) {  // wall: fixed state, zero rates
        const int id = from_a ? F.A.id[s] : B.id[s];
        if (!ghosts || id < P.n_real) {
            const int o = ghosts ? id : s;
            A.xh[o] = xi;
            A.vm[o] = vi;
            A.u[o] = from_a ? F.A.u[s] : B.vmin[s].w;
            A.ap[o] = make_float4(0.f, 0.f, 0.f, 0.f);
            A.rho[o] = rpi.x;
            A.p[o] = from_a ? F.A.p[s] : B.p[s];
            A.itype[o] = it;
            A.id[o] = id;
            if (A.inst) A.inst[o] = B.inst[s];
        }
    }
    const bool work = valid && it > 0 && g.ok;
    CellCoord cc = {{0, 0, 0}};
    if (work) cc = decode_key<DIM>(keys[s], g);
    const float ihf = __fdividef(1.0f, xi.w);
    const float kgih_i = P.kg * pow_grad<DIM>(ihf);
    float4 ti = make_float4(0.f, 0.f, 0.f, 0.f), ti2 = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool visc = !LEAN && P.visc, heat_art = !LEAN && P.heat_art;
    if (work && visc) {
        ti = B.tau[s];
        if (DIM == 3) ti2 = B.tau2[s];
    }
    const float ulo_i = (work && heat_art) ? B.ulo[s] : 0.f;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, he_sum = 0.f, av_du = 0.f, ah_du = 0.f;
    // single_step options: continuity drho/dt, XSPH velocity, div v for h
    const bool cont = OPT && P.density_form == 1, xsph = OPT && P.xsph, sle2 = OPT && P.sle == 2;
    float drho_s = 0.f, divh = 0.f, x0s = 0.f, x1s = 0.f, x2s = 0.f;
    constexpr int W = mask_words<DIM>() / TPP;  // mask words of this lane
    const size_t mlane = (size_t)s * TPP + sub;
    Cursor cu = cursor_begin<DIM>(g);
    bool done = !work;
    // The density pass left the neighbour bits of the candidates (word-major).
    constexpr int CW = mask_chunk<W>();
    bool from_mask = false;
    uint4 ch = make_uint4(0u, 0u, 0u, 0u);  // mask chunk being decoded
    unsigned wbits = 0u;                    // bits left of word wi
    // A listed particle walks its neighbour list (coalesced rows of entries)
    // and re-tests each entry; the others decode the density pass's bits.
    const int lpk = (LST && work) ? __ldg(B.ncount + s) : -1;
    const int lc = lpk >= 0 ? list_near(lpk) + list_far(lpk) : -1;  // entries (-1: no list)
    if (LST) prefetch_list_rows(B.nlist, B.lstride, s, lc);
    if (work && !(LST && lc >= 0)) {
        ch = mask_load_chunk<W>(B.nmask, B.mstride, mlane, 0);
        wbits = ch.x;
        from_mask = !(ch.x == ~0u && (W == 1 || ch.y == ~0u));
    }
    int wi = 0, rbase = 0;  // index of wbits; ordinal of the cursor row's first slot
    int shift = 0;          // staged index - slot in the cursor's row
    // One pair's terms (pressure, viscosity, art_visc, art_heat, options).
    // va, vb: the neighbour's 2D {vx, vy, rho, P} (vb unused) or 3D v and
    // {rho, P, u, psi}; d, dr2 from the pair test.
    auto pair_terms = [&](const int k, const float4& xj, const float4& va, const float4& vb,
                          float* d, float dr2) {
            float4 vj, rpj;
            if (DIM == 2) {  // u and psi only for art_heat
                vj = make_float4(va.x, va.y, 0.f, 0.f);
                rpj = make_float4(va.z, va.w, 0.f, 0.f);
                if (heat_art) {
                    const float4 r = __ldg(B.rp + k);
                    rpj.z = r.z;
                    rpj.w = r.w;
                }
            } else {
                vj = va;
                rpj = vb;
            }
            refine_periodic<DIM>(xi, xj, g, d, dr2);
            const float mj = mass_of<DIM>(xj, vj);
            float ih = ihf, kgih = kgih_i;
            if (xj.w != xi.w) {
                ih = __fdividef(2.0f, xi.w + xj.w);
                kgih = P.kg * pow_grad<DIM>(ih);
            }
            const float q = __fmul_rn(fast_sqrt_pos(dr2), ih);
            if (!LEAN && repulsive_walls(P) && __ldg(B.itype + k) != it) {
                // Push between particles of different type (ArmandoThrust/armando.cu:507-513
                // for wall_model 1, acpu.c:424-429 for 2) along (x_i - x_j)/r, c = c0.
                const float r = fast_sqrt_pos(dr2);
                if (r > 0.f) {
                    float tt = fmaf(-0.5f, q, 1.0f);
                    tt = tt * tt;
                    tt = tt * tt;
                    tt *= fmaf(2.0f, q, 1.0f);  // W / W(0)
                    const float c2 = P.c0 * P.c0;
                    float f;
                    if (P.wall_model == 1) {
                        const float alpha = P.kw_hi * (DIM == 2 ? ih * ih : ih * ih * ih);
                        f = 0.5f * alpha * tt * mj / (rpj.x * xj.w) * c2;
                    } else {
                        f = 0.02f * tt * c2 / r * mj / (mass_of<DIM>(xi, vi) + mj);
                    }
                    f /= r;
                    a0 = fmaf(f, d[0], a0);
                    a1 = fmaf(f, d[1], a1);
                    if (DIM == 3) a2 = fmaf(f, d[2], a2);
                }
                if (P.wall_model == 1) return;  // no other interaction
            }
            const float t3 = q - 2.0f;
            const float gw = kgih * t3 * t3 * t3;
            const float w0 = gw * d[0], w1 = gw * d[1], w2 = (DIM == 3) ? gw * d[2] : 0.f;
            const float vx = vj.x - vi.x, vy = vj.y - vi.y, vz = (DIM == 3) ? vj.z - vi.z : 0.f;
            if (cont || sle2) {  // (v_j - v_i) . grad_i W
                float vdw = fmaf(vy, w1, __fmul_rn(vx, w0));
                if (DIM == 3) vdw = fmaf(vz, w2, vdw);
                if (cont) drho_s = fmaf(-mj, vdw, drho_s);  // con_density, density.f:203-216
                if (sle2) divh = fmaf(__fdiv_rn(mj, rpj.x), vdw, divh);  // hsml.f:75-90
            }
            if (xsph) {  // av_vel.f:47-58: -eps m_j / rho_ij (v_i - v_j) W_ij, eps = 0.3
                float tt = fmaf(-0.5f, q, 1.0f);
                tt = tt * tt;
                tt = tt * tt;
                const float wv = P.kw_hi * (DIM == 2 ? ih * ih : ih * ih * ih) * tt * fmaf(2.0f, q, 1.0f);
                const float c = __fdiv_rn(0.3f * mj * wv, 0.5f * (rpi.x + rpj.x));
                x0s = fmaf(c, vx, x0s);
                x1s = fmaf(c, vy, x1s);
                if (DIM == 3) x2s = fmaf(c, vz, x2s);
            }
            // Pressure (internal_force.f:309-428 for pa_sph 1, 179-306 for pa_sph 0).
            const float fs = -(rpi.y + rpj.y);
            // Products that feed a sum are written out (fmaf / __fmul_rn) so that
            // every instantiation of this body rounds alike (no free contraction).
            float h0 = fs * w0, h1 = fs * w1, h2 = fs * w2;
            float he = fmaf(vy, h1, __fmul_rn(vx, h0));
            if (DIM == 3) he = fmaf(vz, h2, he);
            if (visc) {
                const float4 tj = __ldg(B.tau + k);
                float4 tj2 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (DIM == 3) tj2 = __ldg(B.tau2 + k);
                const float sxx = ti.x + tj.x, syy = ti.y + tj.y, sxy = ti.z + tj.z;
                if (DIM == 2) {
                    h0 = fmaf(sxy, w1, fmaf(sxx, w0, h0));
                    h1 = fmaf(syy, w1, fmaf(sxy, w0, h1));
                } else {
                    const float szz = ti.w + tj.w, sxz = ti2.x + tj2.x, syz = ti2.y + tj2.y;
                    h0 = fmaf(sxz, w2, fmaf(sxy, w1, fmaf(sxx, w0, h0)));
                    h1 = fmaf(syz, w2, fmaf(syy, w1, fmaf(sxy, w0, h1)));
                    h2 = fmaf(szz, w2, fmaf(syz, w1, fmaf(sxz, w0, h2)));
                }
            }
            if (P.pa_sph != 1) {
                const float inv_rr = __fdividef(1.0f, rpi.x * rpj.x);
                h0 *= inv_rr;
                h1 *= inv_rr;
                h2 *= inv_rr;
                he *= inv_rr;
            }
            a0 = fmaf(mj, h0, a0);
            a1 = fmaf(mj, h1, a1);
            if (DIM == 3) a2 = fmaf(mj, h2, a2);
            he_sum = fmaf(mj, he, he_sum);
            const float mh = 0.5f * (xi.w + xj.w);
            const float rho_bar = 0.5f * (rpi.x + rpj.x);
            // art_visc.f:71-100.
            if (P.visc_art) {
                float vr = fmaf(vy, d[1], __fmul_rn(vx, d[0]));
                if (DIM == 3) vr = fmaf(vz, d[2], vr);
                if (vr > 0.f) {  // (v_i - v_j) . (x_i - x_j) = -vr < 0
                    const float phi = __fdividef(-mh * vr, fmaf(__fmul_rn(mh, mh), P.av_eta2, dr2));
                    const float piv = __fdividef(
                        fmaf(P.av_beta, phi, -__fmul_rn(P.av_alpha, P.c0)) * phi, rho_bar);
                    const float mp = mj * piv;
                    a0 = fmaf(-mp, w0, a0);
                    a1 = fmaf(-mp, w1, a1);
                    if (DIM == 3) a2 = fmaf(-mp, w2, a2);
                    float vdw = fmaf(vy, w1, __fmul_rn(vx, w0));
                    if (DIM == 3) vdw = fmaf(vz, w2, vdw);
                    av_du = fmaf(-0.5f * mp, vdw, av_du);
                }
            }
            // art_heat.f:69-97.
            if (heat_art) {
                float rdw = fmaf(d[1], w1, __fmul_rn(d[0], w0));
                if (DIM == 3) rdw = fmaf(d[2], w2, rdw);
                const float psi = __fdividef(
                    rpi.w + rpj.w, rho_bar * fmaf(__fmul_rn(mh, mh), P.ah_eta2, dr2)) * rdw;
                const float du_ij = (rpi.z - rpj.z) + (ulo_i - __ldg(B.ulo + k));
                ah_du = fmaf(mj * psi, du_ij, ah_du);
            }
    };
    // A listed particle takes each entry's terms as the entry is read and
    // passes the pair test, without a candidate list; the mask decoding and
    // cell walk below serve the others.
    if (LST) {
        constexpr int NB = list_batch<DIM>();
        const int lcm = __reduce_max_sync(0xffffffffu, lc > 0 ? lc : 0);
        // (a lane past the last slot reads slot 0: its loads stay in bounds)
        auto entry = [&](int t) {
            return lc > 0 ? __ldg(B.nlist + (size_t)min(t, lc - 1) * B.lstride + s) : (valid ? s : 0);
        };
        for (int t0 = 0; t0 < lcm; t0 += NB) {
            int kb[NB];
            float4 xb[NB];
#pragma unroll
            for (int u = 0; u < NB; ++u) kb[u] = entry(t0 + u);
            // 2D: the neighbours' {vx, vy, rho, P} load with their positions; 3D
            // loads v and {rho, P} once the pair test passed (registers).
            float4 vr[NB];
#pragma unroll
            for (int u = 0; u < NB; ++u) {
                xb[u] = __ldg(xsrc + kb[u]);
                if (DIM == 2) vr[u] = __ldg(B.vr + kb[u]);
            }
#pragma unroll
            for (int u = 0; u < NB; ++u) {
                float d[3], dr2;
                if (t0 + u < lc && kb[u] != s && pair_delta<DIM>(xi, xb[u], g, d, dr2)) {
                    if (DIM == 2)
                        pair_terms(kb[u], xb[u], vr[u], vr[u], d, dr2);
                    else
                        pair_terms(kb[u], xb[u], __ldg(B.vm + kb[u]), __ldg(B.rp + kb[u]), d, dr2);
                }
            }
        }
        if (lc >= 0) done = true;
    }
    while (__any_sync(0xffffffffu, !done)) {
        int nl = 0;
        while (!done && from_mask) {
            if (nl == cap_force<LST>()) break;
            while (wbits == 0u && wi < W - 1) {
                ++wi;
                if (W > CW && wi % CW == 0) ch = mask_load_chunk<W>(B.nmask, B.mstride, mlane, wi / CW);
                wbits = chunk_word(ch, wi % CW);
            }
            if (wbits == 0u) {
                done = true;
                break;
            }
            const int o = 32 * wi + __ffs(wbits) - 1;
            wbits &= wbits - 1u;
            bool in_rows = true;
            while (o >= rbase + lane_len<TPP>(cu)) {  // move to the range holding ordinal o
                rbase += lane_len<TPP>(cu);
                if (!cursor_next<DIM>(g, start, cc, cu)) {
                    in_rows = false;
                    break;
                }
                cu.k += sub;
                if (STG) shift = SV.shift[cursor_row<DIM>(cu, g.reach)];
            }
            if (!in_rows) {  // cannot happen for a mask of this step's candidates
                done = true;
                break;
            }
            s_list[nl++][tid] = (LT)(cu.k + TPP * (o - rbase) + (STG ? shift : 0));
        }
        while (!done && !from_mask) {
            int kb[kTestBatch];
            int cnt;
            float4 xb[kTestBatch];
            if (cu.k >= cu.ke) {
                if (!cursor_next<DIM>(g, start, cc, cu)) {
                    done = true;
                    break;
                }
                if (STG) shift = SV.shift[cursor_row<DIM>(cu, g.reach)];
                if (TPP > 1) {
                    cu.k += sub;
                    continue;
                }
            }
            if (nl > cap_force<LST>() - kTestBatch) break;
            const int k0 = cu.k;
            cnt = min(kTestBatch, lane_len<TPP>(cu));
#pragma unroll
            for (int u = 0; u < kTestBatch; ++u) {
                const int ku = min(k0 + u * TPP, cu.ke - 1);
                kb[u] = k0 + u * TPP;
                xb[u] = STG ? SV.x[ku + shift] : __ldg(xsrc + ku);
            }
            cu.k += cnt * TPP;
#pragma unroll
            for (int u = 0; u < kTestBatch; ++u) {
                float d[3], dr2;
                const int k = kb[u];
                if (u < cnt && k != s && pair_delta<DIM>(xi, xb[u], g, d, dr2))
                    s_list[nl++][tid] = (LT)(STG ? k + shift : k);
            }
        }
        const int ml = __reduce_max_sync(0xffffffffu, nl);
        for (int t = 0; t < ml; ++t) {
            if (t >= nl) continue;
            const int k = (int)s_list[t][tid];
            const float4 xj = STG ? SV.x[k] : __ldg(xsrc + k);
            float4 va, vb = make_float4(0.f, 0.f, 0.f, 0.f);
            if (DIM == 2) {
                va = STG ? SV.v[k] : __ldg(B.vr + k);
            } else {
                va = STG ? SV.v[k] : __ldg(B.vm + k);
                vb = STG ? SV.r[k] : __ldg(B.rp + k);
            }
            float d[3], dr2;
            pair_delta<DIM>(xi, xj, g, d, dr2);
            pair_terms(k, xj, va, vb, d, dr2);
        }
    }
    if (TPP > 1) {  // the particle's lanes reach this point together
        a0 = group_sum<TPP>(a0);
        a1 = group_sum<TPP>(a1);
        if (DIM == 3) a2 = group_sum<TPP>(a2);
        he_sum = group_sum<TPP>(he_sum);
        av_du = group_sum<TPP>(av_du);
        ah_du = group_sum<TPP>(ah_du);
        if (cont) drho_s = group_sum<TPP>(drho_s);
        if (sle2) divh = group_sum<TPP>(divh);
        if (xsph) {
            x0s = group_sum<TPP>(x0s);
            x1s = group_sum<TPP>(x1s);
            if (DIM == 3) x2s = group_sum<TPP>(x2s);
        }
    }
    if (!work || sub != 0) return;
    float du = __fadd_rn(fmaf(0.5f, he_sum, av_du), ah_du);  // internal_force.f:433-435
    if (visc) du += B.tds[s];
    if (S.heat_on) {
        float e0 = xi.x - P.heat_center[0], e1 = xi.y - P.heat_center[1];
        float dd = fmaf(e1, e1, __fmul_rn(e0, e0));
        if (DIM == 3) {
            float e2 = xi.z - P.heat_center[2];
            dd = fmaf(e2, e2, dd);
        }
        du += P.heat_q0 * expf(-dd * P.heat_k) / rpi.x;
    }
    a0 += P.gravity[0];
    a1 += P.gravity[1];
    if (DIM == 3) a2 += P.gravity[2];
    // Corrector (time_integration.f:186-218).
    float4 vmin;
    if (from_a) {
        const float4 v0 = F.A.vm[s];
        vmin = make_float4(v0.x, v0.y, v0.z, F.A.u[s]);
    } else {
        vmin = B.vmin[s];
    }
    float4 vn = vi;
    vn.x = fmaf(S.kdt, a0, vmin.x);
    vn.y = fmaf(S.kdt, a1, vmin.y);
    if (DIM == 3) vn.z = fmaf(S.kdt, a2, vmin.z);
    if (xsph && S.hdt != 0.f) {  // time_integration.f:195: v = v_min + dt dv + av
        vn.x += x0s;
        vn.y += x1s;
        if (DIM == 3) vn.z += x2s;
    }
    float un = fmaf(S.kdt, du, vmin.w);
    if (un < 0.f) un = 0.f;
    float4 xn = xi;
    float rho_out = rpi.x;
    if (cont) rho_out = fmaf(S.kdt, drho_s, B.q[s]);  // time_integration.f:191-193, 207-209
    if (OPT && P.sle == 1) {  // hsml.f:45-48, exponent the single-precision 1./dim
        const float mr = __fdiv_rn(mass_of<DIM>(xi, vi), rpi.x);
        xn.w = 2.0f * (DIM == 2 ? sqrtf(mr) : powf(mr, 1.0f / 3.0f));
    } else if (sle2) {  // hsml.f:92-96
        const float hn = fmaf(S.dt, __fmul_rn(xi.w * (1.0f / DIM), divh), xi.w);
        if (!(hn <= 0.f)) xn.w = hn;
    }
    xn.x = fmaf(S.dt, vn.x, xi.x);
    xn.y = fmaf(S.dt, vn.y, xi.y);
    if (DIM == 3) xn.z = fmaf(S.dt, vn.z, xi.z);
    bool outside = false;
    if (P.periodic[0]) xn.x = wrap_axis(xn.x, P, 0, outside);
    if (P.periodic[1]) xn.y = wrap_axis(xn.y, P, 1, outside);
    if (DIM == 3 && P.periodic[2]) xn.z = wrap_axis(xn.z, P, 2, outside);
    if (outside) atomicOr(flags, (unsigned)FLAG_OUT_OF_GRID);
    if (g.half_skin2 > 0.f && B.xsort) {  // moved more than half the skin since the sort: sort next
        const float4 x0 = B.xsort[s];
        const float e0 = xn.x - x0.x, e1 = xn.y - x0.y, e2 = (DIM == 3) ? xn.z - x0.z : 0.f;
        if (e0 * e0 + e1 * e1 + e2 * e2 > g.half_skin2 && *(volatile unsigned*)(flags + 2) == 0u)
            atomicExch(flags + 2, 1u);
    }
    const float chk = xn.x + xn.y + xn.z + vn.x + vn.y + vn.z + un + a0 + a1 + a2 + du;
    if (!isfinite(chk)) atomicOr(flags, (unsigned)FLAG_NONFINITE);
    const int id = from_a ? F.A.id[s] : B.id[s];
    const int o = ghosts ? id : s;
    A.xh[o] = xn;
    A.vm[o] = vn;
    A.u[o] = un;
    A.ap[o] = make_float4(a0, a1, a2, du);
    A.rho[o] = rho_out;
    if (A.drho) A.drho[o] = drho_s;
    A.p[o] = B.p[s];
    A.itype[o] = it;
    A.id[o] = id;
    if (A.inst) A.inst[o] = B.inst[s];
}

// ---------------------------------------------------------------------------
// Pass kernels of one particle system: one CTA per 128 consecutive slots.
// ---------------------------------------------------------------------------
// The grid of a pass; PER = false (no periodic axis) makes the periodic flags
// compile-time zeros, so the minimum-image code and its registers drop out.
template <bool PER>
__device__ __forceinline__ DevGrid load_grid(const DevGrid* __restrict__ gp) {
    DevGrid g = *gp;
    if (!PER) g.periodic[0] = g.periodic[1] = g.periodic[2] = 0;
    return g;
}

// One CTA per BS / TPP consecutive slots.
template <int DIM, int TPP, int BS, bool PER, bool LEAN, bool OPT = false, bool LST = false,
          bool FUS = false>
__global__ void __launch_bounds__(BS, 1024 / BS)
    k_density(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
              const DevGrid* __restrict__ gp, DevParams P, int n, FusedSrc F) {
    __shared__ int s_near[cap_density<LST>()][BS];
    __shared__ int s_far[cap_density<LST>()][BS];
    const int s = blockIdx.x * (BS / TPP) + (int)threadIdx.x / TPP;
    const DevGrid g = load_grid<PER>(gp);
    density_body<DIM, TPP, BS, LEAN, OPT, false, int, LST, FUS>(B, keys, start, g, P, s, s < n,
                                                                s_near, s_far, StageView{}, F);
}

// Neighbour lists of an iteration that sorts (lazy sorting), built in the
// sort's conditional body after the cell table: for each slot s of the new
// order, the candidates k != s (cursor order) within h_s + h_k + skin, the
// bound widened by 2^-14 over the rounding of the FP32 distances; in 2D the
// pairs the density pass evaluates in FP32 (q >= list_near_q2() at the sort) go
// after the others (filled from the last row down, then moved up). Positions
// are read through the sort's permutation (the reorder into cell order comes
// later in the iteration). Until the next sort every particle stays within
// half the skin of where it was binned, so every pair the exact test accepts
// (r < h_i + h_j) on those iterations is in the list.
template <int DIM, bool PER>
__global__ void __launch_bounds__(kPassThreads)
    k_build_list(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
                 const DevGrid* __restrict__ gp, int n, const int* __restrict__ resort = nullptr) {
    if (sort_skipped(resort)) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevGrid g = load_grid<PER>(gp);
    if (!g.ok) {
        B.ncount[s] = 0;
        return;
    }
    const float4 xi = B.xsort[s];
    const CellCoord cc = decode_key<DIM>(keys[s], g);
    const float pad = (1.0f + 0x1p-14f);
    int cn = 0, cf = 0;  // near and far entries
    Cursor cu = cursor_begin<DIM>(g);
    while (cursor_next<DIM>(g, start, cc, cu)) {
        for (int k0 = cu.k; k0 < cu.ke; k0 += kTestBatch) {
            float4 xb[kTestBatch];
#pragma unroll
            for (int u = 0; u < kTestBatch; ++u) xb[u] = __ldg(B.xsort + min(k0 + u, cu.ke - 1));
#pragma unroll
            for (int u = 0; u < kTestBatch; ++u) {
                const int k = k0 + u;
                if (k >= cu.ke || k == s) continue;
                float d[3], dr2;
                pair_delta<DIM>(xi, xb[u], g, d, dr2);
                const float lim = __fmul_rn(__fadd_rn(__fadd_rn(xi.w, xb[u].w), g.skin), pad);
                if (!(dr2 < __fmul_rn(lim, lim))) continue;
                const float hs = xi.w + xb[u].w;  // the density pass's near test
                const bool near =
                    DIM == 3 || dr2 < (0.25f * list_near_q2() * list_near_q2()) * hs * hs;
                if (cn + cf < B.lcap) B.nlist[(size_t)(near ? cn : B.lcap - 1 - cf) * B.lstride + s] = k;
                if (near) ++cn;
                else ++cf;
            }
        }
    }
    if (cn + cf <= B.lcap) {
        // the far entries, written from the last row down, moved up behind the
        // near ones (rows in increasing order: each source row is read before
        // a later copy could overwrite it)
        for (int i = 0; i < cf; ++i)
            B.nlist[(size_t)(cn + i) * B.lstride + s] =
                B.nlist[(size_t)(B.lcap - cf + i) * B.lstride + s];
        B.ncount[s] = cn | (cf << 16);
    } else {
        B.ncount[s] = -1;
    }
}

template <int DIM>
__global__ void __launch_bounds__(kPassThreads)
    k_shear(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
            const DevGrid* __restrict__ gp, DevParams P, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const DevGrid g = *gp;
    shear_body<DIM>(B, keys, start, g, P, s, s < n);
}

template <int DIM, int TPP, int BS, bool PER, bool LEAN, bool OPT = false, bool LST = false,
          bool FUS = false>
__global__ void __launch_bounds__(BS, 1024 / BS)
    k_force(StateB B, StateA A, const unsigned* __restrict__ keys, const int* __restrict__ start,
            const DevGrid* __restrict__ gp, DevParams P, StepArgs S, unsigned* __restrict__ flags,
            int n, FusedSrc F) {
    __shared__ int s_list[cap_force<LST>()][BS];
    const int s = blockIdx.x * (BS / TPP) + (int)threadIdx.x / TPP;
    const DevGrid g = load_grid<PER>(gp);
    force_body<DIM, TPP, BS, LEAN, OPT, false, int, LST, FUS>(B, A, keys, start, g, P, S, flags, s,
                                                              s < n, s_list, StageView{}, F);
}

// ---------------------------------------------------------------------------
// Batched (multi-instance) pass kernels: persistent CTAs pull work items
// (one instance's slots [s0, s1), at most kPassThreads) from an atomic queue;
// the item's instance parameters, grid and step arguments are staged in shared
// memory for the CTA. Items are independent, so the order in which CTAs take
// them does not change any result.
// ---------------------------------------------------------------------------
struct ItemCtx {
    DevParams P;
    DevGrid g;
    StepArgs S;
    WorkItem w;
};

template <class T>
__device__ __forceinline__ void copy_to_shared(T* dst, const T* __restrict__ src) {
    static_assert(sizeof(T) % 4 == 0, "word copy");
    const int* a = reinterpret_cast<const int*>(src);
    int* b = reinterpret_cast<int*>(dst);
    for (int k = threadIdx.x; k < (int)(sizeof(T) / 4); k += blockDim.x) b[k] = __ldg(a + k);
}

// Takes the next item; false when the queue is empty. Ends with a barrier.
// Step arguments of iteration `its` of an instance (time_integration.f:131-218).
__device__ __forceinline__ StepArgs step_args_dev(const DevParams& P, int its) {
    StepArgs S;
    S.dt = P.dt;
    S.kdt = (its == 1) ? 0.5f * P.dt : P.dt;
    S.hdt = (its == 1) ? 0.f : 0.5f * P.dt;
    S.heat_on = P.heat_ext && ((double)its * (double)P.dt <= (double)P.heat_t_end);
    return S;
}

__device__ __forceinline__ bool next_item(ItemCtx& c, const WorkItem* __restrict__ items,
                                          int n_items, int* __restrict__ queue,
                                          const DevParams* __restrict__ params,
                                          const DevGrid* __restrict__ grids,
                                          const int* __restrict__ its) {
    __shared__ int s_it;
    __syncthreads();  // every thread is done with the previous item
    if (threadIdx.x == 0) s_it = atomicAdd(queue, 1);
    __syncthreads();
    const int it = s_it;
    if (it >= n_items) return false;
    if (threadIdx.x == 0) {
        c.w = items[it];
        if (its) c.S = step_args_dev(params[c.w.inst], *its);
    }
    __syncthreads();
    const int inst = c.w.inst;
    copy_to_shared(&c.P, params + inst);
    copy_to_shared(&c.g, grids + inst);
    __syncthreads();
    return true;
}

// LEAN: no instance uses physical viscosity, artificial heat, a wall model
// or a single_step option (the passes' lean variant).
template <int DIM, bool LEAN = false>
__global__ void __launch_bounds__(kPassThreads, 8)
    k_density_batch(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
                    const DevGrid* __restrict__ grids, const DevParams* __restrict__ params,
                    const WorkItem* __restrict__ items, int n_items, int* __restrict__ queue) {
    __shared__ int s_near[kListCapD][kPassThreads];
    __shared__ int s_far[kListCapD][kPassThreads];
    __shared__ ItemCtx c;
    while (next_item(c, items, n_items, queue, params, grids, nullptr)) {
        const int s = c.w.s0 + threadIdx.x;
        density_body<DIM, 1, kPassThreads, LEAN>(B, keys, start, c.g, c.P, s, s < c.w.s1, s_near,
                                                 s_far);
    }
}

template <int DIM>
__global__ void __launch_bounds__(kPassThreads)
    k_shear_batch(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
                  const DevGrid* __restrict__ grids, const DevParams* __restrict__ params,
                  const WorkItem* __restrict__ items, int n_items, int* __restrict__ queue) {
    __shared__ ItemCtx c;
    while (next_item(c, items, n_items, queue, params, grids, nullptr)) {
        const int s = c.w.s0 + threadIdx.x;
        if (c.P.visc) shear_body<DIM>(B, keys, start, c.g, c.P, s, s < c.w.s1);
    }
}

template <int DIM, bool LEAN = false>
__global__ void __launch_bounds__(kPassThreads, 8)
    k_force_batch(StateB B, StateA A, const unsigned* __restrict__ keys,
                  const int* __restrict__ start, const DevGrid* __restrict__ grids,
                  const DevParams* __restrict__ params, const int* __restrict__ its,
                  unsigned* __restrict__ flags, const WorkItem* __restrict__ items, int n_items,
                  int* __restrict__ queue) {
    __shared__ int s_list[kListCap][kPassThreads];
    __shared__ ItemCtx c;
    while (next_item(c, items, n_items, queue, params, grids, its)) {
        const int s = c.w.s0 + threadIdx.x;
        force_body<DIM, 1, kPassThreads, LEAN>(B, A, keys, start, c.g, c.P, c.S, flags, s,
                                               s < c.w.s1, s_list);
    }
}

// ---------------------------------------------------------------------------
// Neighbour lists (diagnostic entry point)
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void k_count_nbrs(StateB B, const unsigned* __restrict__ keys,
                             const int* __restrict__ start, const DevGrid* __restrict__ gp,
                             int* __restrict__ cnt_by_id, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevGrid g = *gp;
    const float4 xi = B.xh[s];
    const CellCoord cc = decode_key<DIM>(keys[s], g);
    int c = 0;
    for_candidates<DIM>(g, start, cc, [&](int k) {
        if (k == s) return;
        float d[3], dr2;
        if (pair_delta<DIM>(xi, B.xh[k], g, d, dr2)) ++c;
    });
    cnt_by_id[B.id[s]] = c;
}

template <int DIM>
__global__ void k_fill_nbrs(StateB B, const unsigned* __restrict__ keys,
                            const int* __restrict__ start, const DevGrid* __restrict__ gp,
                            const long long* __restrict__ offs_by_id, int* __restrict__ nbr,
                            int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevGrid g = *gp;
    const float4 xi = B.xh[s];
    const CellCoord cc = decode_key<DIM>(keys[s], g);
    long long o = offs_by_id[B.id[s]];
    for_candidates<DIM>(g, start, cc, [&](int k) {
        if (k == s) return;
        float d[3], dr2;
        if (pair_delta<DIM>(xi, B.xh[k], g, d, dr2)) nbr[o++] = B.id[k];
    });
}

}  // namespace ag
