// armando.cu -- C-ABI of the GB300 SPH step (declared in include/armando.h).
//
// A context owns the device working set of one particle system. Caller arrays
// are gathered into cell order at the start of a call, the leapfrog loop runs
// as replayed CUDA graphs on the context's stream, and the results are scattered
// back to the caller's order at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../../include/armando.h"
#include "kernels.cuh"
#include "staged.cuh"
#include "adjoint.cuh"
#include "ghosts.cuh"
#include "gpuc.cuh"
#include "deck_io.h"

using namespace ag;

namespace {

// Last error of context-less calls; a fixed buffer so that setting it never
// allocates.
thread_local char g_last_error[256] = "no error";

void set_last_error(const char* msg) {
    std::strncpy(g_last_error, msg, sizeof(g_last_error) - 1);
    g_last_error[sizeof(g_last_error) - 1] = '\0';
}

struct GraphKey {
    float kdt, hdt, dt;
    int heat_on;
    int par;  // 0: one state buffer; 1, 2: which of the two is current (fused predictor)
    int lst;  // neighbour lists in use
    bool operator<(const GraphKey& o) const {
        return std::tie(kdt, hdt, dt, heat_on, par, lst) <
               std::tie(o.kdt, o.hdt, o.dt, o.heat_on, o.par, o.lst);
    }
};

template <class T>
T* dalloc(size_t count, cudaError_t& err) {
    void* p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) err = e;
    return static_cast<T*>(p);
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

constexpr int kFlagWords = 4;

}  // namespace

struct armando_ctx {
    int device = 0;
    // The stream the context launches on: its own stream (created blocking, so
    // it is ordered with the legacy default stream both ways), or the caller's
    // (armando_set_stream). Graphs are captured on cap_stream and launched here.
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t cap_stream = nullptr;
    // A device-memory call returned before its work completed: its device
    // status words are being copied to h_flags; armando_sync reports them.
    bool pending = false;
    // Stage the neighbour passes' candidates in shared memory where the
    // variant allows it (ARMANDO_STAGING=1 at creation; otherwise global
    // memory through L1; both give the same bits).
    bool staging = false;
    // Neighbour lists between sorts (ARMANDO_NEIGHBOUR_LISTS=0 at creation:
    // walk the cells every iteration; 2D results are the same bits).
    bool lists = true;
    // Fused predictor on the iterations between sorts (ARMANDO_FUSED_PREDICTOR=0
    // at creation: a reorder copy every iteration; the same bits).
    bool fuse_ok = true;
    // Inside armando_forward_checkpointed or a replay of armando_backward.
    bool reverse_run = false;
    armando_params prm{};
    DevParams dp{};
    int dim = 2;
    int64_t n = 0, nf = 0, nw = 0;
    // Particle slots of the step arrays: n, plus one mirror ghost per fluid
    // particle for contexts created with wall_model 3. n_work: particles of
    // the iteration being launched (n + its ghosts).
    int64_t cap = 0, n_work = 0;
    int mem_kind = ARMANDO_MEM_HOST;
    StateA A{};
    StateB B{};
    unsigned* keys[2] = {nullptr, nullptr};
    int* vals[2] = {nullptr, nullptr};
    unsigned* hist = nullptr;
    unsigned* dtotal = nullptr;
    int num_tiles = 0;
    int* start = nullptr;
    long long cell_cap = 0;
    int passes = 0;
    float* bbox_part = nullptr;
    DevGrid* grid = nullptr;
    unsigned* flags = nullptr;
    unsigned* h_flags = nullptr;  // pinned
    DevGrid* h_grid = nullptr;    // pinned
    // Device copies of caller arrays (host memory kind).
    float *s_x = nullptr, *s_v = nullptr, *s_m = nullptr, *s_rho = nullptr, *s_p = nullptr,
          *s_u = nullptr, *s_h = nullptr, *s_dvdt = nullptr, *s_dudt = nullptr;
    int* s_itype = nullptr;
    std::vector<void*> owned;
    int* inv = nullptr;  // caller index -> cell-order slot (outputs to mapped host memory)
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::string err = "no error";
    int64_t steps_done = 0, launches = 0;
    int launches_per_step = 0;
    int lazy_body = 0;  // kernels in the conditional body of the lazy step graph (run on sorting steps)
    DevGrid last_grid{};
    bool have_grid = false;
    float last_dt = 0.f;  // dt and next its of the state left on the device
    int next_its = 0;
    // Batches of independent instances (n_inst > 1): packed state, one cell
    // grid per instance, persistent passes over work items.
    int n_inst = 1;
    std::vector<int64_t> inst_n;            // particles per instance
    std::vector<armando_params> prm_inst;   // parameters per instance
    std::vector<float> inst_dt;             // time step per instance
    int* d_inst0 = nullptr;                 // instance of each caller index
    DevParams* d_params = nullptr;          // [n_inst]
    DevGrid* d_grids = nullptr;             // [n_inst]
    int* d_ncells_inst = nullptr;           // [n_inst]
    int* d_inst_items = nullptr;            // [n_inst + 1] first work item per instance
    WorkItem* d_items = nullptr;
    int n_items = 0;
    float* d_part_items = nullptr;          // [n_items * 8] bbox partials
    int* d_total_cells = nullptr;
    int* d_queue = nullptr;                 // [4] work-queue heads, reset every step
    int* d_its = nullptr;
    int any_visc = 0;
    bool batch_lean = false;  // every instance has lean physics: the lean passes
    int grid_density = 0, grid_shear = 0, grid_force = 0;  // persistent CTAs
    cudaGraphExec_t batch_graph = nullptr;
    // Reverse mode (armando_forward_checkpointed / armando_backward).
    std::vector<StateA> ckpts;           // state before iterations its0 + k*K
    armando_tuning tune{1, 1, 128, 0};   // neighbour-pass tuning (armando_set_tuning)
    int64_t sorts_done = 0;              // lazily sorting iterations that sorted (device count)
    int64_t sorts_host = 0;              // iterations that always sort
    cudaStream_t stream2 = nullptr;      // captures the conditional sort body; copies beside the step
    // A host-memory call's copies beside the step (overlapped_call): events
    // {inputs start, rest of the inputs loaded, density done, rho and p written}.
    cudaEvent_t ev_ovl[4] = {nullptr, nullptr, nullptr, nullptr};
    int ovl_ctas = 0;                    // CTAs of the copy kernels beside the step
    bool split_in = false;               // load_inputs left the rest of the inputs on stream2
    bool no_conditional = false;         // conditional graphs failed to build here
    float4* xsort_buf = nullptr;
    std::vector<TapeSlot> tape;          // intermediates of each iteration of one segment
    int tape_seg = -1;                   // the segment the tape holds (-1: none)
    AdjState adjG{}, adjGp{};            // cotangents (output / input slot order)
    float4 *adj_abar = nullptr, *adj_xpart = nullptr, *adj_vpart = nullptr, *adj_xF = nullptr,
           *adj_vhb = nullptr;
    float *adj_rhobar = nullptr, *adj_pbar = nullptr;
    double* adj_blk = nullptr;   // per-block parameter cotangents
    float* adj_divsb = nullptr;  // cotangents of the divergence sums (artificial heat)
    float4 *adj_tbar = nullptr, *adj_tbar2 = nullptr;  // shear-tensor cotangents (viscosity)
    double* adj_pacc = nullptr;
    int adj_its0 = 0, adj_steps = 0, adj_K = 0;
    float adj_dt = 0.f;
    bool adj_ready = false;
    // Mirror ghosts (wall_model 3): the wall grid of the call, the walls in
    // cell order, and per iteration the nearest wall of each particle and the
    // ghosts' owners.
    WallGrid* wgrid = nullptr;
    WallGrid* h_wgrid = nullptr;  // pinned
    int* wstart = nullptr;
    long long wstart_cap = 0;
    int wall_cells = 0;
    float4 *wall_xh = nullptr, *wall_n = nullptr;
    int *wall_id = nullptr, *g_best = nullptr, *g_owner = nullptr, *g_slot = nullptr,
        *d_ng = nullptr, *h_ng = nullptr;
    unsigned *g_tile_count = nullptr, *g_tile_off = nullptr;
    int64_t ghosts_last = 0;
    // Open boundaries of the GPU-C schemes: inlets (with their distances since
    // the last emission), outlets and box, the compaction buffers.
    bool open_set = false;
    std::vector<armando_inlet> inlets;
    std::vector<float> inlet_dist;
    OpenSpec open{};
    StateA A2{};
    // Fused predictor (lazily sorting, lean physics, lists): the force pass
    // writes the next state into A_alt, then the two swap; acur counts swaps.
    StateA A_alt{};
    int acur = 0;
    bool open_ready = false;
    int *open_keep = nullptr, *d_open_n = nullptr, *h_open_n = nullptr;
    unsigned *open_tc = nullptr, *open_to = nullptr;
    // single_step options: drho/dt carried between calls in caller order
    // (continuity density) and the buffers of the options, allocated on first use.
    float* drho_caller = nullptr;
    bool options_ready = false;
    // GPU-C schemes (scheme 1, 2): the RK3 working state in cell order and the
    // material table (default: Tait with rho0, c0 for every |itype|).
    GpucState gs{};
    bool gs_ready = false;
    DevMaterial* d_mat = nullptr;
    std::vector<armando_material> materials;  // set by armando_set_materials
    DevZones* d_zones = nullptr;               // load and fix zones (armando_set_zones)
    std::vector<armando_load_zone> loads;
    std::vector<armando_fix_zone> fixes;
};

namespace {

armando_status fail(armando_ctx* c, armando_status st, const std::string& msg) {
    if (c) c->err = msg;
    set_last_error(msg.c_str());
    return st;
}

armando_status cuda_fail(armando_ctx* c, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return fail(c, e == cudaErrorMemoryAllocation ? ARMANDO_ERR_OOM : ARMANDO_ERR_CUDA, m);
}

#define CK(call)                                                          \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);          \
    } while (0)

armando_status validate_params(const armando_params* p, int dim, std::string& why) {
    if (!p) {
        why = "params is NULL";
        return ARMANDO_ERR_INVALID_ARG;
    }
    if (p->dim != dim || (dim != 2 && dim != 3)) {
        why = "dim must be 2 or 3 and match params->dim";
        return ARMANDO_ERR_INVALID_ARG;
    }
    if (p->pa_sph != 0 && p->pa_sph != 1) {
        why = "pa_sph must be 0 or 1";
        return ARMANDO_ERR_INVALID_ARG;
    }
    if (!(p->rho0 > 0.f) || !(p->c0 >= 0.f) || !std::isfinite(p->c0)) {
        why = "rho0 must be > 0 and c0 finite and >= 0";
        return ARMANDO_ERR_INVALID_ARG;
    }
    if (p->heat_external && !(p->heat_sigma > 0.f)) {
        why = "heat_sigma must be > 0 with heat_external";
        return ARMANDO_ERR_INVALID_ARG;
    }
    for (int d = 0; d < dim; ++d)
        if (p->periodic[d] && !(p->period_hi[d] > p->period_lo[d])) {
            why = "periodic axis needs period_hi > period_lo";
            return ARMANDO_ERR_INVALID_ARG;
        }
    if (p->wall_model < 0 || p->wall_model > 3) {
        why = "wall_model must be 0, 1, 2 or 3";
        return ARMANDO_ERR_INVALID_ARG;
    }
    if (p->wall_model == 3)
        for (int d = 0; d < dim; ++d)
            if (p->periodic[d]) {
                why = "mirror ghosts (wall_model 3) need a system without periodic axes";
                return ARMANDO_ERR_INVALID_ARG;
            }
    if (p->density_form < 0 || p->density_form > 2 || (p->average_velocity != 0 && p->average_velocity != 1) ||
        p->sle < 0 || p->sle > 2) {
        why = "density_form must be 0-2, average_velocity 0 or 1, sle 0-2";
        return ARMANDO_ERR_INVALID_ARG;
    }
    if (p->scheme < 0 || p->scheme > 2) {
        why = "scheme must be 0, 1 or 2";
        return ARMANDO_ERR_INVALID_ARG;
    }
    if (p->scheme != 0) {
        if (p->wall_model != 0) {
            why = "the GPU-C schemes carry their own wall treatment: wall_model must be 0";
            return ARMANDO_ERR_INVALID_ARG;
        }
        for (int d = 0; d < dim; ++d)
            if (p->periodic[d]) {
                why = "the GPU-C schemes have no periodic axes";
                return ARMANDO_ERR_INVALID_ARG;
            }
    }
    return ARMANDO_OK;
}

DevParams make_dev_params(const armando_params& p, int reach = 1) {
    DevParams d{};
    d.reach = reach;
    d.wall_model = p.wall_model;
    d.density_form = p.density_form;
    d.xsph = p.average_velocity;
    d.sle = p.sle;
    d.dim = p.dim;
    d.pa_sph = p.pa_sph;
    d.visc = p.visc;
    d.visc_art = p.visc_artificial;
    d.heat_art = p.heat_artificial;
    d.heat_ext = p.heat_external;
    d.rho0 = p.rho0;
    d.inv_rho0 = (float)(1.0 / (double)p.rho0);
    d.B = (float)((double)p.rho0 * (double)p.c0 * (double)p.c0 / 7.0);
    d.c0 = p.c0;
    d.pmin = p.pmin;
    d.eta = p.eta;
    d.av_alpha = p.av_alpha;
    d.av_beta = p.av_beta;
    d.av_eta2 = p.av_eta * p.av_eta;
    d.ah_g1 = p.ah_g1;
    d.ah_g2 = p.ah_g2;
    d.ah_eta2 = p.ah_eta * p.ah_eta;
    d.heat_q0 = p.heat_q0;
    d.heat_k = p.heat_sigma > 0.f ? (float)(1.0 / (2.0 * (double)p.heat_sigma * p.heat_sigma)) : 0.f;
    for (int k = 0; k < 3; ++k) {
        d.periodic[k] = (k < p.dim) ? p.periodic[k] : 0;
        d.gravity[k] = p.gravity[k];
        d.heat_center[k] = p.heat_center[k];
        d.period_lo[k] = p.period_lo[k];
        d.period_hi[k] = p.period_hi[k];
        const float L = p.period_hi[k] - p.period_lo[k];  // FP32, as the oracle
        d.period_L[k] = L;
        d.period_half[k] = 0.5f * L;
    }
    const double pi = 3.14159265358979323846;
    double K = (p.dim == 2) ? 7.0 / (4.0 * pi) : (p.kernel_3d_legacy ? 15.0 : 21.0) / (16.0 * pi);
    d.kw_hi = (float)K;
    d.kw_lo = (float)(K - (double)d.kw_hi);
    d.kg = (float)(K * 5.0 / 8.0);
    return d;
}

StepArgs make_args(const armando_ctx* c, float dt, int its) {
    StepArgs s;
    s.dt = dt;
    s.kdt = (its == 1) ? 0.5f * dt : dt;
    s.hdt = (its == 1) ? 0.f : 0.5f * dt;
    s.heat_on = c->prm.heat_external && ((double)its * (double)dt <= (double)c->prm.heat_t_end);
    s.dform = c->prm.density_form;
    return s;
}

void free_graphs(armando_ctx* c) {
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
    c->batch_graph = nullptr;
}

// Captures on the context's private capture stream for the scope's life; the
// launch stream (the context's own or the caller's) is never put in capture
// mode, so a caller's stream that synchronises with the legacy default stream
// needs no care, and the instantiated graph is launched on it afterwards.
struct CaptureScope {
    armando_ctx* c;
    cudaStream_t run;
    explicit CaptureScope(armando_ctx* ctx) : c(ctx), run(ctx->stream) { c->stream = c->cap_stream; }
    ~CaptureScope() { c->stream = run; }
};

// ---- launch sequences -------------------------------------------------------

// The context's lazy-sort flags (see sort_skipped); nullptr: always sort.
const int* resort_flags(armando_ctx* ctx) { return reinterpret_cast<const int*>(ctx->flags + 1); }

// The next iteration rebuilds the grid and sorts (the state in A was loaded
// or replaced since the last sort).
armando_status force_sort(armando_ctx* ctx) {
    CK(cudaMemsetAsync(ctx->flags + 2, 0x01, sizeof(unsigned), ctx->stream));
    return ARMANDO_OK;
}

bool use_lists(const armando_ctx* ctx);
template <int DIM>
int launch_build_list(armando_ctx* ctx, const int* rs, cudaStream_t st);

// lists: also rebuild the neighbour lists (a lazily sorting step).
template <int DIM>
int launch_grid_and_sort(armando_ctx* ctx, const int* rs, cudaStream_t st, bool lists = false) {
    const int n = (int)ctx->n_work;
    int L = 0;
    k_bbox_partial<<<kBBoxBlocks, 256, 0, st>>>(ctx->A.xh, n, DIM, ctx->bbox_part, rs);
    k_bbox_final<<<1, 256, 0, st>>>(ctx->bbox_part, kBBoxBlocks, ctx->dp, ctx->cell_cap, ctx->grid,
                                    ctx->flags, rs);
    k_hash<DIM><<<ctx->num_tiles, kSortThreads, 0, st>>>(ctx->A.xh, n, ctx->grid, ctx->keys[0],
                                                          ctx->hist, ctx->num_tiles, rs);
    L += 3;
    for (int p = 0; p < ctx->passes; ++p) {
        const int shift = 8 * p;
        const int a = p & 1, b = (p + 1) & 1;
        if (p > 0) {
            k_radix_hist<<<ctx->num_tiles, kSortThreads, 0, st>>>(ctx->keys[a], n, shift,
                                                                   ctx->hist, ctx->num_tiles, rs);
            ++L;
        }
        k_radix_scan<<<kRadix, 256, 0, st>>>(ctx->hist, ctx->num_tiles, ctx->dtotal, rs);
        k_radix_scatter<<<ctx->num_tiles, kSortThreads, 0, st>>>(
            ctx->keys[a], p == 0 ? nullptr : ctx->vals[a], ctx->keys[b], ctx->vals[b], n, shift,
            ctx->hist, ctx->dtotal, ctx->num_tiles, rs);
        L += 2;
    }
    k_cell_start<<<blocks_for((int64_t)n + 1, kCellStartThreads), kCellStartThreads, 0, st>>>(ctx->keys[ctx->passes & 1], n,
                                                                   &ctx->grid->ncells, (int)ctx->cell_cap,
                                                                   ctx->start, rs);
    if (lists) L += launch_build_list<DIM>(ctx, rs, st);
    return L + 1;
}

// Whether the context sorts lazily (a sort skin; one particle system).
bool lazy(const armando_ctx* ctx) { return ctx->tune.skin > 0 && ctx->n_inst == 1; }

// Neighbour lists: a lazily sorting CERN step with one lane per particle and
// the lists allocated (ensure_lists); the iterations between sorts then read
// the lists instead of walking the cells.
// Not in reverse mode: its iterations sort every time, and the adjoint passes
// decode the neighbour bits that the density pass leaves only for particles
// walking their cells.
bool use_lists(const armando_ctx* ctx) {
    return lazy(ctx) && ctx->tune.threads_per_particle == 1 && ctx->prm.scheme == 0 &&
           ctx->B.nlist != nullptr && !ctx->reverse_run;
}

template <int DIM>
int launch_build_list(armando_ctx* ctx, const int* rs, cudaStream_t st) {
    const int n = (int)ctx->n_work;
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    k_sorted_positions<<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, perm, ctx->B, n, rs);
    if (ctx->dp.periodic[0] || ctx->dp.periodic[1] || ctx->dp.periodic[2])
        k_build_list<DIM, true><<<blocks_for(n, kPassThreads), kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->grid, n, rs);
    else
        k_build_list<DIM, false><<<blocks_for(n, kPassThreads), kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->grid, n, rs);
    return 2;
}

// Start of a lazily sorting iteration launched without the step graph's
// head: it sorts if the last one (or the host) asked for it.
int launch_resort_begin(armando_ctx* ctx) {
    k_resort_begin<<<1, 32, 0, ctx->stream>>>(reinterpret_cast<int*>(ctx->flags + 1),
                                              reinterpret_cast<int*>(ctx->flags + 3));
    return 1;
}

// Calls f(tpp, block, periodic, lean, opt) with the context's tuning, whether
// any axis is periodic, whether the physics is lean (no physical viscosity, no
// artificial heat, no wall push, no step option) and whether a single_step
// option (continuity or normalised density, XSPH, h evolution) is on, as
// compile-time constants. Lean variants exist for one thread per particle.
template <class F>
void with_tuning(const armando_tuning& t, bool per, bool lean, bool opt, bool lst, F&& f) {
    using std::integral_constant;
    // lists (one lane per particle only) as a compile-time flag, last argument
    auto pick_lst = [&](auto tpp, auto bs, auto pr, auto ln, auto op) {
        if constexpr (decltype(tpp)::value == 1) {
            if (lst) f(tpp, bs, pr, ln, op, std::true_type{});
            else f(tpp, bs, pr, ln, op, std::false_type{});
        } else {
            f(tpp, bs, pr, ln, op, std::false_type{});
        }
    };
    auto pick_lean = [&](auto tpp, auto bs, auto pr) {
        if (opt) pick_lst(tpp, bs, pr, std::false_type{}, std::true_type{});
        else if (decltype(tpp)::value == 1 && lean) pick_lst(tpp, bs, pr, std::true_type{}, std::false_type{});
        else pick_lst(tpp, bs, pr, std::false_type{}, std::false_type{});
    };
    auto pick_per = [&](auto tpp, auto bs) {
        if (per) pick_lean(tpp, bs, std::true_type{});
        else pick_lean(tpp, bs, std::false_type{});
    };
    auto pick_tpp = [&](auto bs) {
        if (t.threads_per_particle == 4) pick_per(integral_constant<int, 4>{}, bs);
        else if (t.threads_per_particle == 2) pick_per(integral_constant<int, 2>{}, bs);
        else pick_per(integral_constant<int, 1>{}, bs);
    };
    if (t.block == 256) pick_tpp(integral_constant<int, 256>{});
    else pick_tpp(integral_constant<int, 128>{});
}

bool any_periodic(const DevParams& p) { return p.periodic[0] || p.periodic[1] || p.periodic[2]; }
bool lean_physics(const DevParams& p) {
    return !p.visc && !p.heat_art && p.wall_model == 0 && p.density_form == 0 && !p.xsph && !p.sle;
}

// Whether the parameters use a single_step option beyond summation density.
bool step_options(const armando_params& p) {
    return p.density_form != 0 || p.average_velocity != 0 || p.sle != 0;
}

// Whether every iteration must sort (no sort skin): mirror ghosts change every
// iteration and an evolving h outgrows cells sized for the h of the last sort.
// (The GPU-C schemes sort lazily like the CERN step: their stage test against
// the step's start positions needs the same cells; open runs sort every step.)
bool sorts_every_step(const armando_params& p) {
    return p.wall_model == 3 || p.sle != 0;
}

// The passes read the state themselves on iterations that do not sort (no
// reorder copy) and write the next state into the other buffer: lists, lean
// physics, no step option.
bool fused_wanted(const armando_ctx* ctx) {
    return ctx->fuse_ok && use_lists(ctx) && lean_physics(ctx->dp) && !step_options(ctx->prm);
}
bool fused(const armando_ctx* ctx) { return fused_wanted(ctx) && ctx->A_alt.xh != nullptr; }

// After a fused iteration the next state is in A_alt: make it current.
void swap_state(armando_ctx* ctx) {
    StateA& a = ctx->A;
    StateA& b = ctx->A_alt;
    std::swap(a.xh, b.xh);
    std::swap(a.vm, b.vm);
    std::swap(a.u, b.u);
    std::swap(a.ap, b.ap);
    std::swap(a.rho, b.rho);
    std::swap(a.p, b.p);
    std::swap(a.itype, b.itype);
    std::swap(a.id, b.id);
    ctx->acur ^= 1;
}

// The staged passes serve one thread per particle, lean physics, no periodic
// axis, no single_step option and no mirror ghosts (the other variants read
// their candidates from global memory).
bool staged_passes(const armando_ctx* ctx) {
    return ctx->staging && !use_lists(ctx) && ctx->tune.threads_per_particle == 1 && lean_physics(ctx->dp) && !any_periodic(ctx->dp) &&
           !step_options(ctx->prm) && ctx->n_inst == 1 && ctx->prm.wall_model != 3;
}

template <int DIM, int BS>
void launch_density_staged(armando_ctx* ctx, const unsigned* skeys) {
    const int n = (int)ctx->n_work;
    const int reach = ctx->tune.reach;
    const int cap = stage_cap(DIM, reach, BS, false);
    const int bytes = stage_smem_bytes(DIM, reach, BS, false);
    cudaFuncSetAttribute(k_density_st<DIM, BS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    k_density_st<DIM, BS><<<blocks_for(n, BS), BS, bytes, ctx->stream>>>(
        ctx->B, skeys, ctx->start, ctx->grid, ctx->dp, n, cap, ctx->flags);
}

template <int DIM, int BS>
void launch_force_staged(armando_ctx* ctx, const unsigned* skeys, const StepArgs& S) {
    const int n = (int)ctx->n_work;
    const int reach = ctx->tune.reach;
    const int cap = stage_cap(DIM, reach, BS, true);
    const int bytes = stage_smem_bytes(DIM, reach, BS, true);
    cudaFuncSetAttribute(k_force_st<DIM, BS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    k_force_st<DIM, BS><<<blocks_for(n, BS), BS, bytes, ctx->stream>>>(
        ctx->B, ctx->A, skeys, ctx->start, ctx->grid, ctx->dp, S, ctx->flags, n, cap);
}

template <int DIM>
void launch_density(armando_ctx* ctx, const unsigned* skeys, const StepArgs& S) {
    const int n = (int)ctx->n_work;
    const bool fuse = fused(ctx);
    const FusedSrc F{ctx->A, fuse ? resort_flags(ctx) : nullptr, S.hdt};
    if (staged_passes(ctx)) {
        if (ctx->tune.block == 256) launch_density_staged<DIM, 256>(ctx, skeys);
        else launch_density_staged<DIM, 128>(ctx, skeys);
        return;
    }
    with_tuning(ctx->tune, any_periodic(ctx->dp), lean_physics(ctx->dp), step_options(ctx->prm),
                use_lists(ctx), [&](auto tpp, auto bs, auto per, auto lean, auto opt, auto lst) {
        constexpr int T = decltype(tpp)::value, BSZ = decltype(bs)::value;
        constexpr bool PER = decltype(per)::value, LEAN = decltype(lean)::value && T == 1;
        constexpr bool OPT = decltype(opt)::value, LST = decltype(lst)::value;
        constexpr bool FUS_OK = LST && LEAN && !OPT;
        const int grid = blocks_for((int64_t)n * T, BSZ);
        if constexpr (FUS_OK) {
            if (fuse) {
                k_density<DIM, T, BSZ, PER, LEAN, OPT, LST, true><<<grid, BSZ, 0, ctx->stream>>>(
                    ctx->B, skeys, ctx->start, ctx->grid, ctx->dp, n, F);
                return;
            }
        }
        k_density<DIM, T, BSZ, PER, LEAN, OPT, LST><<<grid, BSZ, 0, ctx->stream>>>(
            ctx->B, skeys, ctx->start, ctx->grid, ctx->dp, n, F);
    });
}

template <int DIM>
void launch_force(armando_ctx* ctx, const unsigned* skeys, const StepArgs& S) {
    const int n = (int)ctx->n_work;
    const bool fuse = fused(ctx);
    const FusedSrc F{ctx->A, fuse ? resort_flags(ctx) : nullptr, S.hdt};
    if (staged_passes(ctx)) {
        if (ctx->tune.block == 256) launch_force_staged<DIM, 256>(ctx, skeys, S);
        else launch_force_staged<DIM, 128>(ctx, skeys, S);
        return;
    }
    with_tuning(ctx->tune, any_periodic(ctx->dp), lean_physics(ctx->dp), step_options(ctx->prm),
                use_lists(ctx), [&](auto tpp, auto bs, auto per, auto lean, auto opt, auto lst) {
        constexpr int T = decltype(tpp)::value, BSZ = decltype(bs)::value;
        constexpr bool PER = decltype(per)::value, LEAN = decltype(lean)::value && T == 1;
        constexpr bool OPT = decltype(opt)::value, LST = decltype(lst)::value;
        constexpr bool FUS_OK = LST && LEAN && !OPT;
        const int grid = blocks_for((int64_t)n * T, BSZ);
        if constexpr (FUS_OK) {
            if (fuse) {  // the next state into the other buffer
                k_force<DIM, T, BSZ, PER, LEAN, OPT, LST, true><<<grid, BSZ, 0, ctx->stream>>>(
                    ctx->B, ctx->A_alt, skeys, ctx->start, ctx->grid, ctx->dp, S, ctx->flags, n, F);
                return;
            }
        }
        k_force<DIM, T, BSZ, PER, LEAN, OPT, LST><<<grid, BSZ, 0, ctx->stream>>>(
            ctx->B, ctx->A, skeys, ctx->start, ctx->grid, ctx->dp, S, ctx->flags, n, F);
    });
}

// Reorder/predictor and the pair passes.
// reorder = false: the caller launched the reorder copy itself (the fused
// predictor's step graph, where only iterations that sort need it).
template <int DIM>
int launch_passes(armando_ctx* ctx, const StepArgs& S, const int* rs, bool reorder = true) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n_work;
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    int L = 1;
    if (reorder) {
        k_reorder_dim<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, perm, ctx->B, S, n, rs,
                                                               fused(ctx));
        ++L;
    }
    launch_density<DIM>(ctx, skeys, S);
    if (n > ctx->n) {  // mirror ghosts take their owners' density, pressure, energy
        k_invert_ids<<<blocks_for(n, 256), 256, 0, st>>>(ctx->B.id, ctx->g_slot, n);
        k_ghost_sync<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->B, ctx->g_slot, ctx->g_owner,
                                                               ctx->dp, n);
        L += 2;
    }
    if (ctx->dp.visc) {
        k_shear<DIM><<<blocks_for(n, kPassThreads), kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->grid, ctx->dp, n);
        ++L;
    }
    launch_force<DIM>(ctx, skeys, S);
    ++L;
    return L;
}

// One iteration as a plain launch sequence (lazy sorting: the grid and sort
// kernels test the flag and return at once when the iteration does not sort).
template <int DIM>
int launch_step(armando_ctx* ctx, const StepArgs& S) {
    const int* rs = lazy(ctx) ? resort_flags(ctx) : nullptr;
    const int L0 = rs ? launch_resort_begin(ctx) : 0;
    const int L = launch_grid_and_sort<DIM>(ctx, rs, ctx->stream, use_lists(ctx));
    return L0 + L + launch_passes<DIM>(ctx, S, rs);
}

// One lazily sorting iteration as a graph whose grid and sort kernels sit in
// the body of a conditional (IF) node: a one-thread kernel sets the condition
// from the flag, so iterations that do not sort launch none of them. The body
// is captured from a second stream into the node's child graph.
template <int DIM>
int launch_gpuc_passes(armando_ctx* ctx, const StepArgs& S, const int* rs);

template <int DIM>
armando_status build_lazy_graph(armando_ctx* ctx, const StepArgs& S, cudaGraphExec_t* out,
                                int* launches) {
    cudaError_t e = cudaSuccess;
    if (!ctx->stream2 && (e = cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(ctx, e, "cudaStreamCreate");
    cudaGraph_t graph = nullptr;
    if ((e = cudaGraphCreate(&graph, 0)) != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphCreate");
    bool main_cap = false, body_cap = false;
    auto fail_graph = [&](cudaError_t err, const char* where) {
        cudaGraph_t g = nullptr;
        if (body_cap) cudaStreamEndCapture(ctx->stream2, &g);
        if (main_cap && cudaStreamEndCapture(ctx->stream, &g) == cudaSuccess && g && g != graph)
            cudaGraphDestroy(g);
        cudaGraphDestroy(graph);
        cudaGetLastError();
        return cuda_fail(ctx, err, where);
    };
    cudaGraphConditionalHandle h;
    if ((e = cudaGraphConditionalHandleCreate(&h, graph, 0, 0)) != cudaSuccess)
        return fail_graph(e, "cudaGraphConditionalHandleCreate");
    if ((e = cudaStreamBeginCaptureToGraph(ctx->stream, graph, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return fail_graph(e, "cudaStreamBeginCaptureToGraph");
    main_cap = true;
    k_resort_cond<<<1, 32, 0, ctx->stream>>>(h, reinterpret_cast<int*>(ctx->flags + 1),
                                              reinterpret_cast<int*>(ctx->flags + 3));
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if ((e = cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, nullptr, &deps, nullptr, &nd)) != cudaSuccess)
        return fail_graph(e, "cudaStreamGetCaptureInfo");
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t cnode;
    if ((e = cudaGraphAddNode(&cnode, graph, deps, nullptr, nd, &p)) != cudaSuccess)
        return fail_graph(e, "cudaGraphAddNode(conditional)");
    if ((e = cudaStreamUpdateCaptureDependencies(ctx->stream, &cnode, nullptr, 1,
                                                 cudaStreamSetCaptureDependencies)) != cudaSuccess)
        return fail_graph(e, "cudaStreamUpdateCaptureDependencies");
    if ((e = cudaStreamBeginCaptureToGraph(ctx->stream2, p.conditional.phGraph_out[0], nullptr,
                                           nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return fail_graph(e, "cudaStreamBeginCaptureToGraph(body)");
    body_cap = true;
    int body = launch_grid_and_sort<DIM>(ctx, nullptr, ctx->stream2,
                                         ctx->prm.scheme == 0 && use_lists(ctx));
    // With the fused predictor only the iterations that sort copy the state
    // into cell order: the copy joins the body.
    const bool body_reorder = ctx->prm.scheme == 0 && fused(ctx);
    if (body_reorder) {
        const int n = (int)ctx->n_work;
        k_reorder_dim<DIM><<<blocks_for(n, 256), 256, 0, ctx->stream2>>>(
            ctx->A, ctx->vals[ctx->passes & 1], ctx->B, S, n);
        ++body;
    }
    int L = 1 + body;
    cudaGraph_t body_out = nullptr;
    e = cudaStreamEndCapture(ctx->stream2, &body_out);
    body_cap = false;
    if (e != cudaSuccess) return fail_graph(e, "cudaStreamEndCapture(body)");
    L += ctx->prm.scheme != 0 ? launch_gpuc_passes<DIM>(ctx, S, resort_flags(ctx))
                              : launch_passes<DIM>(ctx, S, resort_flags(ctx), !body_reorder);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_graph(e, "kernel launch during capture");
    cudaGraph_t g_out = nullptr;
    e = cudaStreamEndCapture(ctx->stream, &g_out);
    main_cap = false;
    if (e != cudaSuccess) return fail_graph(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(ctx, e, "cudaGraphInstantiate(conditional)");
    }
    *launches = L;
    ctx->lazy_body = body;
    return ARMANDO_OK;
}

// One GPU-C RK3 step: grid and sort on the step's start positions, the cell
// order state, three stages ping-ponging between the working copies, the
// result back to A.
template <int DIM>
int launch_gpuc_passes(armando_ctx* ctx, const StepArgs& S, const int* rs) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n_work;
    const int nm = ctx->materials.empty() ? ARMANDO_MAX_MATERIALS : (int)ctx->materials.size();
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    ctx->gs.xsort = rs ? ctx->xsort_buf : nullptr;
    k_gpuc_gather<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, perm, ctx->gs, ctx->d_mat, nm,
                                                           ctx->flags, n, rs);
    static const float alphas[3] = {1.0f, 0.25f, 2.0f / 3.0f};
    for (int q = 0; q < 3; ++q) {
        const int cur = q & 1;
        with_tuning(ctx->tune, false, false, false, false, [&](auto tpp, auto bs, auto, auto, auto, auto) {
            constexpr int T = decltype(tpp)::value, BSZ = decltype(bs)::value;
            const int blocks = blocks_for((int64_t)n * T, BSZ);
            if (ctx->prm.scheme == 1)
                k_gpuc_stage<DIM, 1, T, BSZ><<<blocks, BSZ, 0, st>>>(
                    ctx->gs, cur, skeys, ctx->start, ctx->grid, ctx->dp, ctx->d_mat, nm, ctx->d_zones,
                    ctx->flags, alphas[q], S.dt, n);
            else
                k_gpuc_stage<DIM, 2, T, BSZ><<<blocks, BSZ, 0, st>>>(
                    ctx->gs, cur, skeys, ctx->start, ctx->grid, ctx->dp, ctx->d_mat, nm, ctx->d_zones,
                    ctx->flags, alphas[q], S.dt, n);
        });
    }
    k_gpuc_scatter<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->gs, 1, ctx->A, n, ctx->grid,
                                                            ctx->flags);
    return 5;
}

// rs: the lazy-sorting flags (nullptr: the step sorts).
template <int DIM>
int launch_gpuc_step(armando_ctx* ctx, const StepArgs& S, const int* rs) {
    const int L0 = rs ? launch_resort_begin(ctx) : 0;
    const int L = launch_grid_and_sort<DIM>(ctx, rs, ctx->stream);
    return L0 + L + launch_gpuc_passes<DIM>(ctx, S, rs);
}

int launch_step_any(armando_ctx* ctx, const StepArgs& S) {
    const int* rs = lazy(ctx) ? resort_flags(ctx) : nullptr;
    if (ctx->prm.scheme != 0)
        return ctx->dim == 2 ? launch_gpuc_step<2>(ctx, S, rs) : launch_gpuc_step<3>(ctx, S, rs);
    return ctx->dim == 2 ? launch_step<2>(ctx, S) : launch_step<3>(ctx, S);
}

// Grid, hash and sort of a batch (one grid per instance, one shared table).
template <int DIM>
int launch_batch_grid_and_sort(armando_ctx* ctx, long long capacity) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n;
    int L = 0;
    k_bbox_items<<<ctx->n_items, kPassThreads, 0, st>>>(ctx->A.xh, ctx->d_items, DIM,
                                                        ctx->d_part_items);
    k_bbox_final_batch<<<ctx->n_inst, 256, 0, st>>>(ctx->d_part_items, ctx->d_inst_items,
                                                    ctx->d_params, ctx->d_grids,
                                                    ctx->d_ncells_inst, ctx->flags);
    k_cell_offsets<<<1, 1024, 0, st>>>(ctx->d_ncells_inst, ctx->n_inst, capacity, ctx->d_grids,
                                       ctx->d_total_cells, ctx->flags);
    L += 3;
    if (!ctx->start) return L;  // planning: grids only
    k_hash_batch<DIM><<<ctx->num_tiles, kSortThreads, 0, st>>>(
        ctx->A.xh, ctx->A.inst, n, ctx->d_grids, ctx->keys[0], ctx->hist, ctx->num_tiles);
    ++L;
    for (int p = 0; p < ctx->passes; ++p) {
        const int shift = 8 * p;
        const int a = p & 1, b = (p + 1) & 1;
        if (p > 0) {
            k_radix_hist<<<ctx->num_tiles, kSortThreads, 0, st>>>(ctx->keys[a], n, shift,
                                                                   ctx->hist, ctx->num_tiles);
            ++L;
        }
        k_radix_scan<<<kRadix, 256, 0, st>>>(ctx->hist, ctx->num_tiles, ctx->dtotal);
        k_radix_scatter<<<ctx->num_tiles, kSortThreads, 0, st>>>(
            ctx->keys[a], p == 0 ? nullptr : ctx->vals[a], ctx->keys[b], ctx->vals[b], n, shift,
            ctx->hist, ctx->dtotal, ctx->num_tiles);
        L += 2;
    }
    return L;
}

// One leapfrog step of every instance; ev (optional, ARMANDO_N_PHASES + 1
// events) brackets the phases as in launch_step_phased.
template <int DIM>
int launch_batch_step(armando_ctx* ctx, cudaEvent_t* ev) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n;
    if (ev) cudaEventRecord(ev[0], st);
    cudaMemsetAsync(ctx->d_queue, 0, 4 * sizeof(int), st);
    int L = launch_batch_grid_and_sort<DIM>(ctx, ctx->cell_cap);
    if (ev) {  // grid + hash | sort are not split for batches
        cudaEventRecord(ev[1], st);
        cudaEventRecord(ev[2], st);
    }
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    k_cell_start<<<blocks_for((int64_t)n + 1, kCellStartThreads), kCellStartThreads, 0, st>>>(skeys, n, ctx->d_total_cells,
                                                                   (int)ctx->cell_cap, ctx->start);
    k_reorder_batch<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, perm, ctx->B, ctx->d_params,
                                                             ctx->d_its, n);
    if (ev) cudaEventRecord(ev[3], st);
    if (ctx->batch_lean)
        k_density_batch<DIM, true><<<ctx->grid_density, kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->d_grids, ctx->d_params, ctx->d_items, ctx->n_items,
            ctx->d_queue + 0);
    else
        k_density_batch<DIM><<<ctx->grid_density, kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->d_grids, ctx->d_params, ctx->d_items, ctx->n_items,
            ctx->d_queue + 0);
    if (ev) cudaEventRecord(ev[4], st);
    L += 3;
    if (ctx->any_visc) {
        k_shear_batch<DIM><<<ctx->grid_shear, kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->d_grids, ctx->d_params, ctx->d_items, ctx->n_items,
            ctx->d_queue + 1);
        ++L;
    }
    if (ev) cudaEventRecord(ev[5], st);
    if (ctx->batch_lean)
        k_force_batch<DIM, true><<<ctx->grid_force, kPassThreads, 0, st>>>(
            ctx->B, ctx->A, skeys, ctx->start, ctx->d_grids, ctx->d_params, ctx->d_its, ctx->flags,
            ctx->d_items, ctx->n_items, ctx->d_queue + 2);
    else
        k_force_batch<DIM><<<ctx->grid_force, kPassThreads, 0, st>>>(
            ctx->B, ctx->A, skeys, ctx->start, ctx->d_grids, ctx->d_params, ctx->d_its, ctx->flags,
            ctx->d_items, ctx->n_items, ctx->d_queue + 2);
    k_advance_its<<<1, 1, 0, st>>>(ctx->d_its);
    if (ev) cudaEventRecord(ev[6], st);
    return L + 2;
}

int launch_batch_step_any(armando_ctx* ctx, cudaEvent_t* ev) {
    return ctx->dim == 2 ? launch_batch_step<2>(ctx, ev) : launch_batch_step<3>(ctx, ev);
}

// The kernels of launch_step with an event recorded after each phase
// (ev[0] before the step, ev[k+1] after phase k).
template <int DIM>
int launch_step_phased(armando_ctx* ctx, const StepArgs& S, cudaEvent_t* ev) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n;
    int L = 0;
    cudaEventRecord(ev[0], st);
    const int* rs = lazy(ctx) ? resort_flags(ctx) : nullptr;
    if (rs) L += launch_resort_begin(ctx);
    k_bbox_partial<<<kBBoxBlocks, 256, 0, st>>>(ctx->A.xh, n, DIM, ctx->bbox_part, rs);
    k_bbox_final<<<1, 256, 0, st>>>(ctx->bbox_part, kBBoxBlocks, ctx->dp, ctx->cell_cap, ctx->grid,
                                    ctx->flags, rs);
    k_hash<DIM><<<ctx->num_tiles, kSortThreads, 0, st>>>(ctx->A.xh, n, ctx->grid, ctx->keys[0],
                                                          ctx->hist, ctx->num_tiles, rs);
    L += 3;
    cudaEventRecord(ev[1], st);
    for (int p = 0; p < ctx->passes; ++p) {
        const int shift = 8 * p;
        const int a = p & 1, b = (p + 1) & 1;
        if (p > 0) {
            k_radix_hist<<<ctx->num_tiles, kSortThreads, 0, st>>>(ctx->keys[a], n, shift,
                                                                   ctx->hist, ctx->num_tiles, rs);
            ++L;
        }
        k_radix_scan<<<kRadix, 256, 0, st>>>(ctx->hist, ctx->num_tiles, ctx->dtotal, rs);
        k_radix_scatter<<<ctx->num_tiles, kSortThreads, 0, st>>>(
            ctx->keys[a], p == 0 ? nullptr : ctx->vals[a], ctx->keys[b], ctx->vals[b], n, shift,
            ctx->hist, ctx->dtotal, ctx->num_tiles, rs);
        L += 2;
    }
    cudaEventRecord(ev[2], st);
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    k_cell_start<<<blocks_for((int64_t)n + 1, kCellStartThreads), kCellStartThreads, 0, st>>>(skeys, n, &ctx->grid->ncells,
                                                                   (int)ctx->cell_cap, ctx->start, rs);
    if (use_lists(ctx)) L += launch_build_list<DIM>(ctx, rs, st);
    k_reorder_dim<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, perm, ctx->B, S, n, rs,
                                                           fused(ctx));
    cudaEventRecord(ev[3], st);
    launch_density<DIM>(ctx, skeys, S);
    cudaEventRecord(ev[4], st);
    L += 3;
    if (ctx->dp.visc) {
        k_shear<DIM><<<blocks_for(n, kPassThreads), kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->grid, ctx->dp, n);
        ++L;
    }
    cudaEventRecord(ev[5], st);
    launch_force<DIM>(ctx, skeys, S);
    cudaEventRecord(ev[6], st);
    return L + 1;
}

armando_status run_batch_step(armando_ctx* ctx) {
    if (!ctx->batch_graph) {
        cudaGraph_t graph = nullptr;
        CaptureScope cap(ctx);
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int L = launch_batch_step_any(ctx, nullptr);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        if (le != cudaSuccess) return cuda_fail(ctx, le, "kernel launch during capture");
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        cudaError_t ie = cudaGraphInstantiate(&ctx->batch_graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_fail(ctx, ie, "cudaGraphInstantiate");
        ctx->launches_per_step = L;
    }
    CK(cudaGraphLaunch(ctx->batch_graph, ctx->stream));
    ctx->launches += ctx->launches_per_step;
    ctx->steps_done += 1;
    return ARMANDO_OK;
}

// One iteration with mirror ghosts (wall_model 3), as direct launches: the
// nearest-wall search and the ghost write, one read-back of the ghost count,
// then the step over the real particles and their ghosts.
template <int DIM>
armando_status run_ghost_step(armando_ctx* ctx, const StepArgs& S) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n;
    int ng = 0, L = 0;
    if (ctx->wall_cells > 0 && n > 0) {
        const int tiles = blocks_for(n, kGhostTile);
        k_ghost_select<DIM><<<tiles, kGhostThreads, 0, st>>>(ctx->A, n, ctx->wgrid, ctx->wstart,
                                                             ctx->wall_xh, ctx->wall_id,
                                                             ctx->g_best, ctx->g_tile_count);
        k_ghost_scan<<<1, 1024, 0, st>>>(ctx->g_tile_count, tiles, ctx->g_tile_off, ctx->d_ng);
        k_ghost_write<DIM><<<tiles, kGhostThreads, 0, st>>>(ctx->A, n, ctx->g_best, ctx->wall_xh,
                                                            ctx->wall_n, ctx->g_tile_off,
                                                            ctx->g_owner, S);
        L += 3;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(ctx->h_ng, ctx->d_ng, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        ng = *ctx->h_ng;
        if (ng < 0 || (int64_t)ng > ctx->nf)
            return fail(ctx, ARMANDO_ERR_CUDA, "mirror ghost count out of range");
    }
    ctx->n_work = (int64_t)n + ng;
    ctx->num_tiles = blocks_for(ctx->n_work, kSortTile);
    L += launch_grid_and_sort<DIM>(ctx, nullptr, st);
    L += launch_passes<DIM>(ctx, S, nullptr);
    ctx->n_work = n;
    ctx->num_tiles = blocks_for(n, kSortTile);
    CK(cudaGetLastError());
    ctx->ghosts_last = ng;
    ctx->launches += L;
    ctx->launches_per_step = L;
    ctx->steps_done += 1;
    ctx->sorts_host += 1;
    return ARMANDO_OK;
}

armando_status alloc_stateA(armando_ctx* ctx, StateA& a);

template <class T>
T* mapped_host(T* p);

// One iteration of a host-memory call beside its copies (load_inputs left the
// rest of the inputs loading on the second stream): the grid and sort run on
// the positions meanwhile, the reorder waits for the rest; after the density
// pass the second stream writes the output density and pressure (final then)
// back while the force pass runs. Direct launches: the events belong to this
// call. Same kernels, same order of operations as the step graph: the same
// results.
template <int DIM>
int launch_overlapped_step(armando_ctx* ctx, const StepArgs& S, float* rho_out, float* p_out) {
    cudaStream_t st = ctx->stream, s2 = ctx->stream2;
    const int n = (int)ctx->n_work;
    int L = launch_grid_and_sort<DIM>(ctx, nullptr, st);
    cudaStreamWaitEvent(st, ctx->ev_ovl[1], 0);  // the rest of the inputs
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    k_reorder_dim<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, perm, ctx->B, S, n);
    launch_density<DIM>(ctx, skeys, S);
    cudaEventRecord(ctx->ev_ovl[2], st);
    cudaStreamWaitEvent(s2, ctx->ev_ovl[2], 0);
    k_invert_ids<<<blocks_for(n, 256), 256, 0, s2>>>(ctx->B.id, ctx->inv, n);
    k_scatter_rp<<<ctx->ovl_ctas, 256, 0, s2>>>(ctx->B, ctx->inv, n, rho_out, p_out);
    cudaEventRecord(ctx->ev_ovl[3], s2);
    L += 4;
    if (ctx->dp.visc) {
        k_shear<DIM><<<blocks_for(n, kPassThreads), kPassThreads, 0, st>>>(
            ctx->B, skeys, ctx->start, ctx->grid, ctx->dp, n);
        ++L;
    }
    launch_force<DIM>(ctx, skeys, S);
    cudaStreamWaitEvent(st, ctx->ev_ovl[3], 0);  // the inverse ids serve the other outputs
    return L + 1;
}

armando_status run_overlapped_step(armando_ctx* ctx, const StepArgs& S, float* rho_out,
                                   float* p_out) {
    float* mr = mapped_host(rho_out);
    float* mp = mapped_host(p_out);
    if (!mr || !mp) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "output arrays are not mapped");
    const int L = ctx->dim == 2 ? launch_overlapped_step<2>(ctx, S, mr, mp)
                                : launch_overlapped_step<3>(ctx, S, mr, mp);
    CK(cudaGetLastError());
    ctx->launches += L;
    ctx->steps_done += 1;
    ctx->sorts_host += 1;
    return ARMANDO_OK;
}

armando_status run_step(armando_ctx* ctx, const StepArgs& S) {
    if (ctx->n_inst > 1) return run_batch_step(ctx);
    if (ctx->prm.wall_model == 3)
        return ctx->dim == 2 ? run_ghost_step<2>(ctx, S) : run_ghost_step<3>(ctx, S);
    if (fused_wanted(ctx) && !ctx->A_alt.xh) {  // the second state buffer, on first use
        armando_status as = alloc_stateA(ctx, ctx->A_alt);
        if (as != ARMANDO_OK) return as;
        free_graphs(ctx);
    }
    const bool fuse = fused(ctx);
    GraphKey key{S.kdt, S.hdt, S.dt, S.heat_on, fuse ? 1 + ctx->acur : 0, use_lists(ctx) ? 1 : 0};
    auto itg = ctx->graphs.find(key);
    cudaGraphExec_t exec = nullptr;
    if (itg == ctx->graphs.end() && lazy(ctx) && !ctx->no_conditional) {
        int L = 0;
        armando_status gs;
        {
            CaptureScope cap(ctx);
            gs = ctx->dim == 2 ? build_lazy_graph<2>(ctx, S, &exec, &L)
                               : build_lazy_graph<3>(ctx, S, &exec, &L);
        }
        if (gs == ARMANDO_OK) {
            ctx->graphs[key] = exec;
            ctx->launches_per_step = L;
            itg = ctx->graphs.find(key);
        } else {
            ctx->no_conditional = true;  // the plain sequence below instead
            exec = nullptr;
        }
    }
    if (itg == ctx->graphs.end()) {
        cudaGraph_t graph = nullptr;
        int L = 0;
        cudaError_t le = cudaSuccess, ce = cudaSuccess;
        {
            CaptureScope cap(ctx);
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            L = launch_step_any(ctx, S);
            le = cudaGetLastError();
            ce = cudaStreamEndCapture(ctx->stream, &graph);
        }
        if (le != cudaSuccess) return cuda_fail(ctx, le, "kernel launch during capture");
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_fail(ctx, ie, "cudaGraphInstantiate");
        ctx->graphs[key] = exec;
        ctx->launches_per_step = L;
        ctx->lazy_body = 0;
    } else {
        exec = itg->second;
    }
    CK(cudaGraphLaunch(exec, ctx->stream));
    // the conditional body's kernels are counted when the device reports its sorts
    ctx->launches += ctx->launches_per_step - ctx->lazy_body;
    ctx->steps_done += 1;
    if (!lazy(ctx)) ctx->sorts_host += 1;
    if (fuse) swap_state(ctx);
    return ARMANDO_OK;
}

armando_status alloc_state(armando_ctx* ctx) {
    cudaError_t e = cudaSuccess;
    const size_t n = (size_t)std::max<int64_t>(ctx->cap, 1);  // step slots (ghosts included)
    auto F4 = [&](float4*& p) { p = dalloc<float4>(n, e); ctx->owned.push_back(p); };
    auto F1 = [&](float*& p, size_t k) { p = dalloc<float>(k, e); ctx->owned.push_back(p); };
    auto I1 = [&](int*& p) { p = dalloc<int>(n, e); ctx->owned.push_back(p); };
    F4(ctx->A.xh);
    F4(ctx->A.vm);
    F1(ctx->A.u, n);
    F4(ctx->A.ap);
    F1(ctx->A.rho, n);
    F1(ctx->A.p, n);
    I1(ctx->A.itype);
    I1(ctx->A.id);
    F4(ctx->B.xh);
    F4(ctx->B.vm);
    F4(ctx->B.vmin);
    F4(ctx->B.rp);
    F1(ctx->B.p, n);
    I1(ctx->B.itype);
    I1(ctx->B.id);
    F4(ctx->B.tau);
    F4(ctx->B.tau2);
    F1(ctx->B.tds, n);
    F1(ctx->B.ulo, n);
    ctx->B.vr = dalloc<float4>(ctx->dim == 2 ? n : 1, e);
    ctx->owned.push_back(ctx->B.vr);
    ctx->xsort_buf = dalloc<float4>(n, e);  // B.xsort points here while sorting lazily
    ctx->owned.push_back(ctx->xsort_buf);
    ctx->B.nmask = dalloc<unsigned>(n * (ctx->dim == 2 ? mask_words<2>() : mask_words<3>()), e);
    ctx->B.mstride = (int)n;
    ctx->B.mtpp = 1;
    ctx->owned.push_back(ctx->B.nmask);
    ctx->num_tiles = blocks_for(ctx->cap, kSortTile);  // sizes the histogram; set per sort below
    for (int k = 0; k < 2; ++k) {
        ctx->keys[k] = dalloc<unsigned>(n, e);
        ctx->vals[k] = dalloc<int>(n, e);
        ctx->owned.push_back(ctx->keys[k]);
        ctx->owned.push_back(ctx->vals[k]);
    }
    ctx->hist = dalloc<unsigned>((size_t)kRadix * std::max(ctx->num_tiles, 1), e);
    ctx->num_tiles = blocks_for(ctx->n, kSortTile);
    ctx->dtotal = dalloc<unsigned>(kRadix, e);
    ctx->bbox_part = dalloc<float>(kBBoxBlocks * 8, e);
    ctx->grid = dalloc<DevGrid>(1, e);
    // [0] status bits, [1] this iteration sorts, [2] the next one must, [3] sorts done
    ctx->flags = dalloc<unsigned>(kFlagWords, e);
    for (void* p : {(void*)ctx->hist, (void*)ctx->dtotal, (void*)ctx->bbox_part, (void*)ctx->grid,
                    (void*)ctx->flags})
        ctx->owned.push_back(p);
    if (ctx->mem_kind == ARMANDO_MEM_HOST) {
        const size_t nc = (size_t)std::max<int64_t>(ctx->n, 1), nd = nc * ctx->dim;
        F1(ctx->s_x, nd);
        F1(ctx->s_v, nd);
        F1(ctx->s_dvdt, nd);
        F1(ctx->s_m, nc);
        F1(ctx->s_rho, nc);
        F1(ctx->s_p, nc);
        F1(ctx->s_u, nc);
        F1(ctx->s_h, nc);
        F1(ctx->s_dudt, nc);
        ctx->s_itype = dalloc<int>(nc, e);
        ctx->owned.push_back(ctx->s_itype);
    }
    if (ctx->prm.wall_model == 3) {  // mirror ghosts
        const size_t nr = (size_t)std::max<int64_t>(ctx->n, 1);
        const size_t tiles = (size_t)std::max(blocks_for(ctx->n, kGhostTile), 1);
        ctx->wgrid = dalloc<WallGrid>(1, e);
        ctx->wall_xh = dalloc<float4>(nr, e);
        ctx->wall_n = dalloc<float4>(nr, e);
        ctx->wall_id = dalloc<int>(nr, e);
        ctx->g_best = dalloc<int>(nr, e);
        ctx->g_owner = dalloc<int>((size_t)std::max<int64_t>(ctx->nf, 1), e);
        ctx->g_slot = dalloc<int>(n, e);
        ctx->d_ng = dalloc<int>(1, e);
        ctx->g_tile_count = dalloc<unsigned>(tiles, e);
        ctx->g_tile_off = dalloc<unsigned>(tiles, e);
        for (void* q : {(void*)ctx->wgrid, (void*)ctx->wall_xh, (void*)ctx->wall_n,
                        (void*)ctx->wall_id, (void*)ctx->g_best, (void*)ctx->g_owner,
                        (void*)ctx->g_slot, (void*)ctx->d_ng, (void*)ctx->g_tile_count,
                        (void*)ctx->g_tile_off})
            ctx->owned.push_back(q);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc");
    CK(cudaMemset(ctx->flags, 0, kFlagWords * sizeof(unsigned)));
    cudaError_t he = cudaMallocHost((void**)&ctx->h_flags, kFlagWords * sizeof(unsigned));
    if (he != cudaSuccess) return cuda_fail(ctx, he, "cudaMallocHost");
    he = cudaMallocHost((void**)&ctx->h_grid, sizeof(DevGrid));
    if (he != cudaSuccess) return cuda_fail(ctx, he, "cudaMallocHost");
    if (ctx->prm.wall_model == 3) {
        he = cudaMallocHost((void**)&ctx->h_wgrid, sizeof(WallGrid));
        if (he == cudaSuccess) he = cudaMallocHost((void**)&ctx->h_ng, sizeof(int));
        if (he != cudaSuccess) return cuda_fail(ctx, he, "cudaMallocHost");
    }
    return ARMANDO_OK;
}

// Sizes the cell table from the grid of the current positions (A.xh): twice
// the cells of that grid. A later grid larger than that ends a call with
// ARMANDO_ERR_GRID_OVERFLOW (link_list.f:61-66 `stop`s in the same case).
armando_status plan_grid_batch(armando_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    const int L = ctx->dim == 2 ? launch_batch_grid_and_sort<2>(ctx, (long long)INT32_MAX)
                                : launch_batch_grid_and_sort<3>(ctx, (long long)INT32_MAX);
    ctx->launches += L;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    int total = 0;
    unsigned fl = 0;
    CK(cudaMemcpy(&total, ctx->d_total_cells, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&fl, ctx->flags, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (fl & (FLAG_GRID_OVERFLOW | FLAG_PERIODIC_SMALL))
        return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "an instance's neighbour grid is too large or its periodic box shorter than 3 cells");
    long long cap = std::max<long long>(2LL * total, 4096);
    if (cap > (1LL << 30)) return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "the batch's neighbour grids need more than 2^30 cells");
    int bits = 1;
    while ((1LL << bits) < cap) ++bits;
    ctx->passes = (bits + 7) / 8;
    ctx->cell_cap = cap;
    cudaError_t e = cudaSuccess;
    ctx->start = dalloc<int>((size_t)cap + 1, e);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(cell table)");
    ctx->owned.push_back(ctx->start);
    CK(cudaMemsetAsync(ctx->flags, 0, sizeof(unsigned), st));
    free_graphs(ctx);
    return ARMANDO_OK;
}

armando_status plan_grid(armando_ctx* ctx) {
    if (ctx->start) return ARMANDO_OK;
    if (ctx->n_inst > 1) return plan_grid_batch(ctx);
    cudaStream_t st = ctx->stream;
    k_bbox_partial<<<kBBoxBlocks, 256, 0, st>>>(ctx->A.xh, (int)ctx->n_work, ctx->dim, ctx->bbox_part);
    k_bbox_final<<<1, 256, 0, st>>>(ctx->bbox_part, kBBoxBlocks, ctx->dp, (long long)INT32_MAX,
                                    ctx->grid, ctx->flags);
    ctx->launches += 2;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_grid, ctx->grid, sizeof(DevGrid), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const DevGrid g = *ctx->h_grid;
    if (!g.ok) return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "neighbour grid too large or periodic box shorter than 3 cells");
    long long cap = std::max<long long>(2LL * g.ncells, 4096);
    if (cap > (1LL << 30)) return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "neighbour grid needs more than 2^30 cells");
    int bits = 1;
    while ((1LL << bits) < cap) ++bits;
    ctx->passes = (bits + 7) / 8;
    ctx->cell_cap = cap;
    cudaError_t e = cudaSuccess;
    ctx->start = dalloc<int>((size_t)cap + 1, e);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(cell table)");
    ctx->owned.push_back(ctx->start);
    CK(cudaMemsetAsync(ctx->flags, 0, sizeof(unsigned), st));
    free_graphs(ctx);
    return ARMANDO_OK;
}

// The wall grid of a call with mirror ghosts: the walls do not move within
// the call, so their grid, cell order and copies serve every iteration.
template <int DIM>
armando_status build_wall_grid_dim(armando_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n;
    k_wall_grid_partial<DIM><<<kBBoxBlocks, 256, 0, st>>>(ctx->A, n, ctx->bbox_part);
    k_wall_grid<DIM><<<1, kWallGridThreads, 0, st>>>(ctx->bbox_part, kBBoxBlocks, 1LL << 28, ctx->wgrid);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_wgrid, ctx->wgrid, sizeof(WallGrid), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const WallGrid g = *ctx->h_wgrid;
    ctx->launches += 2;
    if (g.ncells < 0) return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "wall grid of the mirror ghosts needs more than 2^28 cells");
    ctx->wall_cells = g.ncells;
    if (g.ncells == 0) return ARMANDO_OK;
    if ((long long)g.ncells + 1 > ctx->wstart_cap) {
        cudaError_t e = cudaSuccess;
        if (ctx->wstart) {
            auto it = std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->wstart);
            if (it != ctx->owned.end()) ctx->owned.erase(it);
            cudaFree(ctx->wstart);
        }
        ctx->wstart_cap = 2LL * g.ncells + 1;
        ctx->wstart = dalloc<int>((size_t)ctx->wstart_cap, e);
        if (e != cudaSuccess) {
            ctx->wstart = nullptr;
            ctx->wstart_cap = 0;
            return cuda_fail(ctx, e, "cudaMalloc(wall cell table)");
        }
        ctx->owned.push_back(ctx->wstart);
    }
    // Sort the walls by cell (fluid keys = ncells sort after them).
    int bits = 1;
    while ((1LL << bits) <= (long long)g.ncells) ++bits;
    const int passes = (bits + 7) / 8;
    const int tiles = blocks_for(n, kSortTile);
    k_wall_keys<DIM><<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, n, ctx->wgrid, ctx->keys[0]);
    int L = 1;
    for (int p = 0; p < passes; ++p) {
        const int a = p & 1, b = (p + 1) & 1;
        k_radix_hist<<<tiles, kSortThreads, 0, st>>>(ctx->keys[a], n, 8 * p, ctx->hist, tiles);
        k_radix_scan<<<kRadix, 256, 0, st>>>(ctx->hist, tiles, ctx->dtotal);
        k_radix_scatter<<<tiles, kSortThreads, 0, st>>>(ctx->keys[a], p == 0 ? nullptr : ctx->vals[a],
                                                        ctx->keys[b], ctx->vals[b], n, 8 * p,
                                                        ctx->hist, ctx->dtotal, tiles);
        L += 3;
    }
    k_cell_start<<<blocks_for((int64_t)n + 1, kCellStartThreads), kCellStartThreads, 0, st>>>(
        ctx->keys[passes & 1], n, &ctx->wgrid->ncells, g.ncells, ctx->wstart);
    k_wall_gather<<<blocks_for(n, 256), 256, 0, st>>>(ctx->vals[passes & 1], ctx->wstart, ctx->wgrid,
                                                      ctx->A, n, ctx->wall_xh, ctx->wall_n,
                                                      ctx->wall_id);
    ctx->launches += L + 2;
    CK(cudaGetLastError());
    return ARMANDO_OK;
}

armando_status build_wall_grid(armando_ctx* ctx) {
    if (ctx->prm.wall_model != 3) return ARMANDO_OK;
    return ctx->dim == 2 ? build_wall_grid_dim<2>(ctx) : build_wall_grid_dim<3>(ctx);
}

// single_step options: the buffers on first use (graphs that captured the old
// pointers are dropped) and the carried drho/dt into A (caller order after
// load_inputs).
armando_status prepare_options(armando_ctx* ctx) {
    if (!step_options(ctx->prm)) return ARMANDO_OK;
    cudaError_t e = cudaSuccess;
    if (!ctx->options_ready) {
        const size_t n = (size_t)std::max<int64_t>(ctx->cap, 1);
        ctx->A.drho = dalloc<float>(n, e);
        ctx->B.q = dalloc<float>(n, e);
        ctx->B.rlo = dalloc<float>(n, e);
        ctx->drho_caller = dalloc<float>(n, e);
        for (void* q : {(void*)ctx->A.drho, (void*)ctx->B.q, (void*)ctx->B.rlo, (void*)ctx->drho_caller})
            ctx->owned.push_back(q);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(step options)");
        CK(cudaMemsetAsync(ctx->drho_caller, 0, n * sizeof(float), ctx->stream));
        ctx->options_ready = true;
        free_graphs(ctx);
    }
    CK(cudaMemcpyAsync(ctx->A.drho, ctx->drho_caller, (size_t)ctx->n * sizeof(float),
                       cudaMemcpyDeviceToDevice, ctx->stream));
    return ARMANDO_OK;
}

// After a call: drho/dt back to caller order for the next call.
armando_status keep_options(armando_ctx* ctx) {
    if (!ctx->options_ready || ctx->n == 0) return ARMANDO_OK;
    const int n = (int)ctx->n;
    k_scatter_by_id<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(ctx->A.drho, ctx->A.id,
                                                                 ctx->drho_caller, n);
    ctx->launches += 1;
    CK(cudaGetLastError());
    return ARMANDO_OK;
}

armando_status alloc_stateA(armando_ctx* ctx, StateA& a);

// Open boundaries: the compaction buffers (first use).
armando_status prepare_open(armando_ctx* ctx) {
    if (ctx->open_ready) return ARMANDO_OK;
    armando_status st = alloc_stateA(ctx, ctx->A2);
    if (st != ARMANDO_OK) return st;
    cudaError_t e = cudaSuccess;
    const size_t n = (size_t)std::max<int64_t>(ctx->n, 1);
    const size_t tiles = (size_t)std::max(blocks_for(ctx->n, kGhostTile), 1);
    ctx->open_keep = dalloc<int>(n, e);
    ctx->open_tc = dalloc<unsigned>(tiles, e);
    ctx->open_to = dalloc<unsigned>(tiles, e);
    ctx->d_open_n = dalloc<int>(1, e);
    for (void* q : {(void*)ctx->open_keep, (void*)ctx->open_tc, (void*)ctx->open_to, (void*)ctx->d_open_n})
        ctx->owned.push_back(q);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(open boundaries)");
    CK(cudaMallocHost((void**)&ctx->h_open_n, sizeof(int)));
    ctx->open_ready = true;
    return ARMANDO_OK;
}

// inletDevice (ArmandoThrust/armando.cu:2792-2845), on the host: each live
// inlet advances its distance by speed dt; past hsml/1.2 it emits a lattice of
// particles (3D: a disk across the normal w, rows along the axis u of w's
// smallest |component| and v = w x u; 2D: a segment along (-w_y, w_x)), FP32 in
// the reference's operation order. The new particles go to A at [n, n + p)
// with serial numbers from *next_id on. Returns ARMANDO_ERR_INVALID_ARG when
// they outgrow the context's capacity.
armando_status emit_inlets(armando_ctx* ctx, float dt, int64_t& n, int64_t& next_id) {
    const int dim = ctx->dim;
    std::vector<float4> xh, vm;
    std::vector<float> uu, rho;
    std::vector<int> it, id;
    for (size_t k = 0; k < ctx->inlets.size(); ++k) {
        const armando_inlet& I = ctx->inlets[k];
        if (I.itype == 0) continue;
        float& dist = ctx->inlet_dist[k];
        dist = dist + I.speed * dt;
        if (!(dist > I.hsml / 1.2f)) continue;
        dist = dist - I.hsml / 1.2f;
        const float len = std::sqrt(I.normal[0] * I.normal[0] + I.normal[1] * I.normal[1] +
                                    I.normal[2] * I.normal[2]);
        const float w[3] = {I.normal[0] / len, I.normal[1] / len, I.normal[2] / len};
        const float sp = I.hsml / 1.2f;
        const int nn = (int)std::lround(1.2f * I.radius / I.hsml);
        auto add = [&](const float r[3]) {
            const float px = I.origin[0] + r[0], py = I.origin[1] + r[1], pz = I.origin[2] + r[2];
            if (dim == 2) {
                xh.push_back(make_float4(px, py, I.mass, I.hsml));
                vm.push_back(make_float4(I.speed * w[0], I.speed * w[1], 0.f, 0.f));
            } else {
                xh.push_back(make_float4(px, py, pz, I.hsml));
                vm.push_back(make_float4(I.speed * w[0], I.speed * w[1], I.speed * w[2], I.mass));
            }
            uu.push_back(I.u);
            rho.push_back(I.rho);
            it.push_back(I.itype);
            id.push_back((int)next_id++);
        };
        if (dim == 2) {
            const float u[2] = {-w[1], w[0]};
            for (int iu = -nn; iu <= nn; ++iu) {
                const float r[3] = {((float)iu * u[0]) * sp, ((float)iu * u[1]) * sp, 0.f};
                if (std::sqrt(r[0] * r[0] + r[1] * r[1]) < I.radius) add(r);
            }
        } else {
            float u[3] = {0.f, 0.f, 0.f};
            const float a[3] = {std::fabs(w[0]), std::fabs(w[1]), std::fabs(w[2])};
            if (a[0] <= a[1] && a[0] <= a[2]) u[0] = 1.f, u[1] = 0.f, u[2] = 0.f;
            if (a[1] <= a[0] && a[1] <= a[2]) u[0] = 0.f, u[1] = 1.f, u[2] = 0.f;
            if (a[2] <= a[0] && a[2] <= a[1]) u[0] = 0.f, u[1] = 0.f, u[2] = 1.f;
            const float v[3] = {w[1] * u[2] - w[2] * u[1], w[2] * u[0] - w[0] * u[2],
                                w[0] * u[1] - w[1] * u[0]};
            for (int iv = -nn; iv <= nn; ++iv)
                for (int iu = -nn; iu <= nn; ++iu) {
                    float r[3];
                    for (int d = 0; d < 3; ++d) r[d] = ((float)iu * u[d] + (float)iv * v[d]) * sp;
                    if (std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) < I.radius) add(r);
                }
        }
    }
    const size_t p = xh.size();
    if (p == 0) return ARMANDO_OK;
    if (n + (int64_t)p > ctx->n)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "inflow exceeds the context's particle capacity");
    cudaStream_t st = ctx->stream;
    std::vector<float4> zero(p, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float> pz(p, 0.f);
    auto H2D = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    CK(H2D(ctx->A.xh + n, xh.data(), p * sizeof(float4)));
    CK(H2D(ctx->A.vm + n, vm.data(), p * sizeof(float4)));
    CK(H2D(ctx->A.ap + n, zero.data(), p * sizeof(float4)));
    CK(H2D(ctx->A.u + n, uu.data(), p * sizeof(float)));
    CK(H2D(ctx->A.rho + n, rho.data(), p * sizeof(float)));
    CK(H2D(ctx->A.p + n, pz.data(), p * sizeof(float)));
    CK(H2D(ctx->A.itype + n, it.data(), p * sizeof(int)));
    CK(H2D(ctx->A.id + n, id.data(), p * sizeof(int)));
    n += (int64_t)p;
    return ARMANDO_OK;
}

// checkOutDevice (armando.cu:2682-2722) and the removal of neighbourListDevice
// (armando.cu:3137-3138): the particles that left are dropped, the others keep
// their order (compacted into A2, which then becomes A).
template <int DIM>
armando_status remove_outflow(armando_ctx* ctx, int64_t& n) {
    if (n == 0) return ARMANDO_OK;
    cudaStream_t st = ctx->stream;
    const int nn = (int)n;
    const int tiles = blocks_for(nn, kGhostTile);
    k_open_flags<DIM><<<tiles, kGhostThreads, 0, st>>>(ctx->A, nn, ctx->open, ctx->open_keep, ctx->open_tc);
    k_ghost_scan<<<1, 1024, 0, st>>>(ctx->open_tc, tiles, ctx->open_to, ctx->d_open_n);
    k_open_compact<<<tiles, kGhostThreads, 0, st>>>(ctx->A, ctx->A2, nn, ctx->open_keep, ctx->open_to);
    ctx->launches += 3;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_open_n, ctx->d_open_n, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const int kept = *ctx->h_open_n;
    if (kept < 0 || kept > nn) return fail(ctx, ARMANDO_ERR_CUDA, "open-boundary count out of range");
    std::swap(ctx->A, ctx->A2);
    n = kept;
    return ARMANDO_OK;
}

// Enough cells for the open run's box at the grid's cell size.
armando_status fit_cells_to_box(armando_ctx* ctx) {
    const DevGrid g = *ctx->h_grid;
    long long cells = 1;
    for (int d = 0; d < ctx->dim; ++d) {
        const double span = (double)ctx->open.hi[d] - (double)ctx->open.lo[d];
        const double c = span / (double)g.size[d] + 3.0;
        if (!(c < 1e9)) return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "open-boundary box needs too many cells");
        cells *= (long long)c;
    }
    if (cells <= ctx->cell_cap) return ARMANDO_OK;
    if (cells > (1LL << 30)) return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "open-boundary box needs more than 2^30 cells");
    auto it = std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->start);
    if (it != ctx->owned.end()) ctx->owned.erase(it);
    cudaFree(ctx->start);
    cudaError_t e = cudaSuccess;
    ctx->start = dalloc<int>((size_t)cells + 1, e);
    if (e != cudaSuccess) {
        ctx->start = nullptr;
        return cuda_fail(ctx, e, "cudaMalloc(cell table)");
    }
    ctx->owned.push_back(ctx->start);
    ctx->cell_cap = cells;
    int bits = 1;
    while ((1LL << bits) < cells) ++bits;
    ctx->passes = (bits + 7) / 8;
    free_graphs(ctx);
    return ARMANDO_OK;
}

// The output order of an open run: ascending serial number (survivors of the
// input in input order, then the new particles in emission order).
template <int DIM>
armando_status store_open(armando_ctx* ctx, int64_t n, float* x, float* vx, float* mass,
                          float* rho, float* p, float* u, float* hsml, int32_t* itype,
                          float* dvdt, float* dudt) {
    if (n == 0) return ARMANDO_OK;
    cudaStream_t st = ctx->stream;
    const int nn = (int)n;
    const int tiles = blocks_for(nn, kSortTile);
    k_open_id_keys<<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A, nn, ctx->keys[0]);
    int L = 1;
    for (int q = 0; q < 4; ++q) {
        const int a = q & 1, b = (q + 1) & 1;
        k_radix_hist<<<tiles, kSortThreads, 0, st>>>(ctx->keys[a], nn, 8 * q, ctx->hist, tiles);
        k_radix_scan<<<kRadix, 256, 0, st>>>(ctx->hist, tiles, ctx->dtotal);
        k_radix_scatter<<<tiles, kSortThreads, 0, st>>>(ctx->keys[a], q == 0 ? nullptr : ctx->vals[a],
                                                        ctx->keys[b], ctx->vals[b], nn, 8 * q,
                                                        ctx->hist, ctx->dtotal, tiles);
        L += 3;
    }
    const bool host = ctx->mem_kind == ARMANDO_MEM_HOST;
    float* dx = host ? ctx->s_x : x;
    float* dv = host ? ctx->s_v : vx;
    float* dm = host ? ctx->s_m : mass;
    float* drho = host ? ctx->s_rho : rho;
    float* dp = host ? ctx->s_p : p;
    float* du = host ? ctx->s_u : u;
    float* dh = host ? ctx->s_h : hsml;
    int* dit = host ? ctx->s_itype : itype;
    float* ddv = host ? ctx->s_dvdt : dvdt;
    float* ddu = host ? ctx->s_dudt : dudt;
    k_open_out<DIM><<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A, ctx->vals[0], nn, dx, dv, dm, drho,
                                                         dp, du, dh, dit, ddv, ddu);
    ctx->launches += L + 1;
    CK(cudaGetLastError());
    if (host) {
        const size_t nd = (size_t)nn * DIM;
        auto D2H = [&](void* dst, const void* src, size_t bytes) {
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
        };
        CK(D2H(x, ctx->s_x, nd * 4));
        CK(D2H(vx, ctx->s_v, nd * 4));
        CK(D2H(dvdt, ctx->s_dvdt, nd * 4));
        CK(D2H(mass, ctx->s_m, (size_t)nn * 4));
        CK(D2H(rho, ctx->s_rho, (size_t)nn * 4));
        CK(D2H(p, ctx->s_p, (size_t)nn * 4));
        CK(D2H(u, ctx->s_u, (size_t)nn * 4));
        CK(D2H(hsml, ctx->s_h, (size_t)nn * 4));
        CK(D2H(itype, ctx->s_itype, (size_t)nn * 4));
        CK(D2H(dudt, ctx->s_dudt, (size_t)nn * 4));
    }
    return ARMANDO_OK;
}

// GPU-C schemes: the working state (first use) and the material table of
// this call.
armando_status prepare_gpuc(armando_ctx* ctx) {
    if (ctx->prm.scheme == 0) return ARMANDO_OK;
    cudaError_t e = cudaSuccess;
    if (!ctx->gs_ready) {
        const size_t n = (size_t)std::max<int64_t>(ctx->n, 1);
        GpucState& g = ctx->gs;
        g.x0 = dalloc<float4>(n, e);
        g.v0 = dalloc<float4>(n, e);
        g.q0 = dalloc<float2>(n, e);
        for (int k = 0; k < 2; ++k) {
            g.xw[k] = dalloc<float4>(n, e);
            g.vw[k] = dalloc<float4>(n, e);
            g.sw[k] = dalloc<float4>(n, e);
        }
        g.rates = dalloc<float4>(n, e);
        g.itype = dalloc<int>(n, e);
        g.id = dalloc<int>(n, e);
        ctx->d_mat = dalloc<DevMaterial>(ARMANDO_MAX_MATERIALS, e);
        ctx->d_zones = dalloc<DevZones>(1, e);
        for (void* q : {(void*)g.x0, (void*)g.v0, (void*)g.q0, (void*)g.xw[0], (void*)g.xw[1],
                        (void*)g.vw[0], (void*)g.vw[1], (void*)g.sw[0], (void*)g.sw[1],
                        (void*)g.rates, (void*)g.itype, (void*)g.id, (void*)ctx->d_mat,
                        (void*)ctx->d_zones})
            ctx->owned.push_back(q);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(GPU-C state)");
        ctx->gs_ready = true;
    }
    std::vector<DevMaterial> tab(ARMANDO_MAX_MATERIALS);
    for (int k = 0; k < ARMANDO_MAX_MATERIALS; ++k) {
        DevMaterial& M = tab[k];
        std::memset(&M, 0, sizeof M);
        if (ctx->materials.empty()) {
            M.type = 4;
            M.prop[0] = ctx->prm.rho0;
            M.prop[1] = ctx->prm.c0;
        } else if (k < (int)ctx->materials.size()) {
            M.type = ctx->materials[k].eos;
            std::memcpy(M.prop, ctx->materials[k].prop, sizeof M.prop);
        }
    }
    CK(cudaMemcpy(ctx->d_mat, tab.data(), sizeof(DevMaterial) * tab.size(), cudaMemcpyHostToDevice));
    DevZones z;
    std::memset(&z, 0, sizeof z);
    z.n_load = (int)ctx->loads.size();
    z.n_fix = (int)ctx->fixes.size();
    for (int k = 0; k < z.n_load; ++k) {
        const armando_load_zone& L = ctx->loads[k];
        for (int d = 0; d < 3; ++d) {
            z.load[k].lo[d] = L.lo[d];
            z.load[k].hi[d] = L.hi[d];
            z.load[k].g[d] = L.accel[d];
        }
        z.load[k].w = L.w;
    }
    for (int k = 0; k < z.n_fix; ++k) {
        const armando_fix_zone& F = ctx->fixes[k];
        for (int d = 0; d < 3; ++d) {
            z.fix[k].lo[d] = F.lo[d];
            z.fix[k].hi[d] = F.hi[d];
            z.fix[k].v[d] = F.vel[d];
        }
        z.fix[k].tau = F.tau;
    }
    CK(cudaMemcpy(ctx->d_zones, &z, sizeof z, cudaMemcpyHostToDevice));
    return ARMANDO_OK;
}

// Enqueues the copy of the device status words and the last grid to the
// pinned host mirrors (complete once the stream passes this point).
armando_status copy_flags(armando_ctx* ctx) {
    CK(cudaMemcpyAsync(ctx->h_flags, ctx->flags, kFlagWords * sizeof(unsigned),
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ctx->h_grid, ctx->n_inst > 1 ? ctx->d_grids : ctx->grid, sizeof(DevGrid),
                       cudaMemcpyDeviceToHost, ctx->stream));
    return ARMANDO_OK;
}

armando_status eval_flags(armando_ctx* ctx);

// Synchronous status of a call: waits for the stream, then reads the flags.
armando_status check_flags(armando_ctx* ctx) {
    armando_status st = copy_flags(ctx);
    if (st != ARMANDO_OK) return st;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->pending = false;
    return eval_flags(ctx);
}

// End of a call. Device memory: stream-ordered and asynchronous, the status
// words follow the work and armando_sync reports them. Host memory: the
// outputs are in the caller's arrays on return, so the call waits.
armando_status finish_call(armando_ctx* ctx) {
    if (ctx->mem_kind != ARMANDO_MEM_DEVICE) return check_flags(ctx);
    armando_status st = copy_flags(ctx);
    if (st != ARMANDO_OK) return st;
    ctx->pending = true;
    return ARMANDO_OK;
}

// Clears the error word at a call's start, unless an asynchronous call's
// status has not been reported yet (device errors stay until armando_sync).
armando_status clear_flags(armando_ctx* ctx) {
    if (!ctx->pending) CK(cudaMemsetAsync(ctx->flags, 0, sizeof(unsigned), ctx->stream));
    return ARMANDO_OK;
}

// Host side of the status words copied by copy_flags (the copy has landed).
armando_status eval_flags(armando_ctx* ctx) {
    ctx->last_grid = *ctx->h_grid;
    ctx->have_grid = true;
    if ((int64_t)ctx->h_flags[3] >= ctx->sorts_done)
        ctx->launches += ((int64_t)ctx->h_flags[3] - ctx->sorts_done) * ctx->lazy_body;
    ctx->sorts_done = ctx->h_flags[3];
    const unsigned f = *ctx->h_flags;
    if (f & FLAG_PERIODIC_SMALL) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "periodic box shorter than 3 cells of 2*max(h)");
    if (f & FLAG_GRID_OVERFLOW) return fail(ctx, ARMANDO_ERR_GRID_OVERFLOW, "neighbour grid exceeded the context's cell capacity");
    if (f & FLAG_NONFINITE) return fail(ctx, ARMANDO_ERR_NONFINITE, "non-finite value in a fluid particle's state");
    if (f & FLAG_OUT_OF_GRID) return fail(ctx, ARMANDO_ERR_OUT_OF_GRID, "a particle left the periodic box by more than one period");
    if (f & FLAG_BAD_MATERIAL) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "an |itype| outside the material table");
    if (f & FLAG_TIMEOUT) return fail(ctx, ARMANDO_ERR_TIMEOUT, "a bounded wait on a shared-memory staging copy gave up");
    return ARMANDO_OK;
}

// Caller arrays -> A (caller order, id = index).
// Device address of a page-locked host array the device maps, or nullptr: for
// those, the copy kernels read and write the caller's memory across the host
// link directly instead of staging through copies. Pageable memory (and any
// pointer the runtime does not know) takes the staged copies.
template <class T>
T* mapped_host(T* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return static_cast<T*>(a.devicePointer);
}

// Whether the step reads the input density / pressure of fluid particles: the
// GPU-C schemes integrate both and the single_step options start from the
// input density; summation density and the equation of state replace them
// otherwise. Batches read all.
bool fluid_rho_read(const armando_ctx* ctx) {
    return ctx->n_inst > 1 || ctx->prm.scheme != 0 || step_options(ctx->prm) ||
           ctx->prm.wall_model == 3;
}
bool fluid_p_read(const armando_ctx* ctx) { return ctx->n_inst > 1 || ctx->prm.scheme != 0; }

// A one-iteration call on host memory that the device maps whose step can run
// beside its copies (launch_overlapped_step): one CERN-scheme particle system
// without mirror ghosts, single_step options or lazy sorting, outside reverse
// mode.
bool overlap_eligible(const armando_ctx* ctx, int steps) {
    return steps == 1 && ctx->mem_kind == ARMANDO_MEM_HOST && ctx->n_inst == 1 &&
           ctx->prm.scheme == 0 && ctx->prm.wall_model != 3 && !step_options(ctx->prm) &&
           !lazy(ctx) && !ctx->reverse_run && ctx->n_work == ctx->n;
}

// The second stream, its events and the inverse ids, on first use.
armando_status ensure_overlap(armando_ctx* ctx) {
    cudaError_t e = cudaSuccess;
    if (!ctx->stream2 && (e = cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(ctx, e, "cudaStreamCreate");
    for (cudaEvent_t& ev : ctx->ev_ovl)
        if (!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_fail(ctx, e, "cudaEventCreate");
    if (!ctx->ovl_ctas) {
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
        ctx->ovl_ctas = 2 * std::max(sms, 1);
    }
    if (!ctx->inv) {
        ctx->inv = dalloc<int>((size_t)std::max<int64_t>(ctx->n, 1), e);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(inverse ids)");
        ctx->owned.push_back(ctx->inv);
    }
    return ARMANDO_OK;
}

// split: the call may load the inputs in two parts (overlap_eligible); with
// the arrays mapped it does, and sets ctx->split_in.
armando_status load_inputs(armando_ctx* ctx, const float* x, const float* vx, const float* mass,
                           const float* rho, const float* p, const float* u, const float* hsml,
                           const int32_t* itype, const float* dvdt, const float* dudt,
                           bool split = false) {
    ctx->split_in = false;
    const size_t n = (size_t)ctx->n, nd = n * ctx->dim;
    cudaStream_t st = ctx->stream;
    const float *mx = nullptr, *mv = nullptr, *mm = nullptr, *mrho = nullptr, *mp = nullptr,
                *mu = nullptr, *mh = nullptr, *mdv = nullptr, *mdu = nullptr;
    const int32_t* mit = nullptr;
    bool zero_copy = false;
    if (ctx->mem_kind == ARMANDO_MEM_HOST) {
        mx = mapped_host(x), mv = mapped_host(vx), mm = mapped_host(mass);
        mrho = mapped_host(rho), mp = mapped_host(p), mu = mapped_host(u), mh = mapped_host(hsml);
        mit = mapped_host(itype), mdv = mapped_host(dvdt), mdu = mapped_host(dudt);
        zero_copy = mx && mv && mm && mrho && mp && mu && mh && mit && (!dvdt || mdv) &&
                    (!dudt || mdu);
    }
    if (zero_copy) {
        x = mx, vx = mv, mass = mm, rho = mrho, p = mp, u = mu, hsml = mh, itype = mit;
        dvdt = mdv, dudt = mdu;
    } else if (ctx->mem_kind == ARMANDO_MEM_HOST) {
        auto H2D = [&](void* dst, const void* src, size_t bytes) {
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
        };
        CK(H2D(ctx->s_x, x, nd * 4));
        CK(H2D(ctx->s_v, vx, nd * 4));
        CK(H2D(ctx->s_m, mass, n * 4));
        CK(H2D(ctx->s_rho, rho, n * 4));
        CK(H2D(ctx->s_p, p, n * 4));
        CK(H2D(ctx->s_u, u, n * 4));
        CK(H2D(ctx->s_h, hsml, n * 4));
        CK(H2D(ctx->s_itype, itype, n * 4));
        if (dvdt) CK(H2D(ctx->s_dvdt, dvdt, nd * 4));
        if (dudt) CK(H2D(ctx->s_dudt, dudt, n * 4));
        x = ctx->s_x;
        vx = ctx->s_v;
        mass = ctx->s_m;
        rho = ctx->s_rho;
        p = ctx->s_p;
        u = ctx->s_u;
        hsml = ctx->s_h;
        itype = ctx->s_itype;
        dvdt = dvdt ? ctx->s_dvdt : nullptr;
        dudt = dudt ? ctx->s_dudt : nullptr;
    }
    // Device memory: stream order only. The context's own stream is ordered
    // after earlier work on the legacy default stream; a caller producing the
    // arrays on another stream passes it with armando_set_stream.
    if (dvdt && !dudt) dvdt = nullptr;
    const int nn = (int)ctx->n;
    const int rfl = fluid_rho_read(ctx) ? 1 : 0, pfl = fluid_p_read(ctx) ? 1 : 0;
    if (split && zero_copy) {
        // positions and h now; the rest from a few CTAs on the second stream,
        // which the step waits for before its reorder
        armando_status os = ensure_overlap(ctx);
        if (os != ARMANDO_OK) return os;
        cudaStream_t s2 = ctx->stream2;
        CK(cudaEventRecord(ctx->ev_ovl[0], st));
        CK(cudaStreamWaitEvent(s2, ctx->ev_ovl[0], 0));
        if (ctx->dim == 2) {
            k_gather_pos<2><<<blocks_for(nn, 256), 256, 0, st>>>(x, mass, hsml, ctx->A, nn);
            k_gather_rest<2><<<ctx->ovl_ctas, 256, 0, s2>>>(vx, mass, rho, p, u, itype, dvdt, dudt,
                                                            ctx->A, nn, rfl, pfl);
        } else {
            k_gather_pos<3><<<blocks_for(nn, 256), 256, 0, st>>>(x, mass, hsml, ctx->A, nn);
            k_gather_rest<3><<<ctx->ovl_ctas, 256, 0, s2>>>(vx, mass, rho, p, u, itype, dvdt, dudt,
                                                            ctx->A, nn, rfl, pfl);
        }
        CK(cudaEventRecord(ctx->ev_ovl[1], s2));
        ctx->launches += 2;
        ctx->split_in = true;
        CK(cudaGetLastError());
        return force_sort(ctx);
    }
    if (ctx->dim == 2)
        k_gather_in<2><<<blocks_for(nn, 256), 256, 0, st>>>(x, vx, mass, rho, p, u, hsml, itype,
                                                            dvdt, dudt, ctx->A, nn, ctx->d_inst0,
                                                            rfl, pfl);
    else
        k_gather_in<3><<<blocks_for(nn, 256), 256, 0, st>>>(x, vx, mass, rho, p, u, hsml, itype,
                                                            dvdt, dudt, ctx->A, nn, ctx->d_inst0,
                                                            rfl, pfl);
    ctx->launches += 1;
    CK(cudaGetLastError());
    return force_sort(ctx);  // A is in caller order now
}

// A -> caller arrays.
// rp_done: an overlapped step wrote rho and p already (k_scatter_rp) and left
// the inverse ids in ctx->inv.
armando_status store_outputs(armando_ctx* ctx, float* x, float* vx, float* rho, float* p, float* u,
                             float* dvdt, float* dudt, bool rp_done = false) {
    const size_t n = (size_t)ctx->n, nd = n * ctx->dim;
    cudaStream_t st = ctx->stream;
    const bool host = ctx->mem_kind == ARMANDO_MEM_HOST;
    const int nn = (int)ctx->n;
    if (host) {
        float *mx = mapped_host(x), *mv = mapped_host(vx), *mrho = mapped_host(rho);
        float *mp = mapped_host(p), *mu = mapped_host(u), *mdv = mapped_host(dvdt);
        float* mdu = mapped_host(dudt);
        if (mx && mv && mrho && mp && mu && mdv && mdu) {
            if (!ctx->inv) {
                cudaError_t e = cudaSuccess;
                ctx->inv = dalloc<int>(n, e);
                if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(inverse ids)");
                ctx->owned.push_back(ctx->inv);
            }
            if (rp_done) {
                mrho = mp = nullptr;
            } else {
                k_invert_ids<<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A.id, ctx->inv, nn);
                ctx->launches += 1;
            }
            if (ctx->dim == 2)
                k_scatter_out_seq<2><<<blocks_for(nn, kScatterSeq), kScatterSeq, 0, st>>>(
                    ctx->A, ctx->inv, nn, mx, mv, mrho, mp, mu, mdv, mdu);
            else
                k_scatter_out_seq<3><<<blocks_for(nn, kScatterSeq), kScatterSeq, 0, st>>>(
                    ctx->A, ctx->inv, nn, mx, mv, mrho, mp, mu, mdv, mdu);
            ctx->launches += 1;
            CK(cudaGetLastError());
            return ARMANDO_OK;
        }
    }
    float* dx = host ? ctx->s_x : x;
    float* dv = host ? ctx->s_v : vx;
    float* drho = host ? ctx->s_rho : rho;
    float* dp = host ? ctx->s_p : p;
    float* du = host ? ctx->s_u : u;
    float* ddvdt = host ? ctx->s_dvdt : dvdt;
    float* ddudt = host ? ctx->s_dudt : dudt;
    if (ctx->dim == 2)
        k_scatter_out<2><<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A, nn, dx, dv, drho, dp, du,
                                                              ddvdt, ddudt);
    else
        k_scatter_out<3><<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A, nn, dx, dv, drho, dp, du,
                                                              ddvdt, ddudt);
    ctx->launches += 1;
    CK(cudaGetLastError());
    if (host) {
        auto D2H = [&](void* dst, const void* src, size_t bytes) {
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
        };
        CK(D2H(x, ctx->s_x, nd * 4));
        CK(D2H(vx, ctx->s_v, nd * 4));
        CK(D2H(rho, ctx->s_rho, n * 4));
        CK(D2H(p, ctx->s_p, n * 4));
        CK(D2H(u, ctx->s_u, n * 4));
        CK(D2H(dvdt, ctx->s_dvdt, nd * 4));
        CK(D2H(dudt, ctx->s_dudt, n * 4));
    }
    return ARMANDO_OK;
}

// ---- reverse mode ------------------------------------------------------------
armando_status alloc_stateA(armando_ctx* ctx, StateA& a) {
    cudaError_t e = cudaSuccess;
    const size_t n = (size_t)std::max<int64_t>(ctx->n, 1);
    a.xh = dalloc<float4>(n, e);
    a.vm = dalloc<float4>(n, e);
    a.u = dalloc<float>(n, e);
    a.ap = dalloc<float4>(n, e);
    a.rho = dalloc<float>(n, e);
    a.p = dalloc<float>(n, e);
    a.itype = dalloc<int>(n, e);
    a.id = dalloc<int>(n, e);
    a.inst = nullptr;
    for (void* p : {(void*)a.xh, (void*)a.vm, (void*)a.u, (void*)a.ap, (void*)a.rho, (void*)a.p,
                    (void*)a.itype, (void*)a.id})
        ctx->owned.push_back(p);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(checkpoint)");
    return ARMANDO_OK;
}

armando_status copy_stateA(armando_ctx* ctx, const StateA& dst, const StateA& src) {
    const size_t n = (size_t)ctx->n;
    cudaStream_t st = ctx->stream;
    CK(cudaMemcpyAsync(dst.xh, src.xh, n * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dst.vm, src.vm, n * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dst.u, src.u, n * 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dst.ap, src.ap, n * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dst.rho, src.rho, n * 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dst.p, src.p, n * 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dst.itype, src.itype, n * 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dst.id, src.id, n * 4, cudaMemcpyDeviceToDevice, st));
    return ARMANDO_OK;
}

armando_status alloc_adjoint(armando_ctx* ctx) {
    if (ctx->adj_abar) return ARMANDO_OK;
    cudaError_t e = cudaSuccess;
    const size_t n = (size_t)std::max<int64_t>(ctx->n, 1);
    for (AdjState* g : {&ctx->adjG, &ctx->adjGp}) {
        g->xb = dalloc<float4>(n, e);
        g->vb = dalloc<float4>(n, e);
        g->ab = dalloc<float4>(n, e);
        for (void* p : {(void*)g->xb, (void*)g->vb, (void*)g->ab}) ctx->owned.push_back(p);
    }
    ctx->adj_abar = dalloc<float4>(n, e);
    ctx->adj_xpart = dalloc<float4>(n, e);
    ctx->adj_vpart = dalloc<float4>(n, e);
    ctx->adj_xF = dalloc<float4>(n, e);
    ctx->adj_vhb = dalloc<float4>(n, e);
    ctx->adj_rhobar = dalloc<float>(n, e);
    ctx->adj_pbar = dalloc<float>(n, e);
    ctx->adj_blk = dalloc<double>((size_t)blocks_for(ctx->n, kPassThreads) * ADJ_NPARAM + 4, e);
    ctx->adj_pacc = dalloc<double>(ADJ_NPARAM, e);
    if (ctx->prm.heat_artificial) ctx->adj_divsb = dalloc<float>(n, e);
    if (ctx->prm.visc) {
        ctx->adj_tbar = dalloc<float4>(n, e);
        if (ctx->dim == 3) ctx->adj_tbar2 = dalloc<float4>(n, e);
    }
    for (void* p : {(void*)ctx->adj_abar, (void*)ctx->adj_xpart, (void*)ctx->adj_vpart,
                    (void*)ctx->adj_xF, (void*)ctx->adj_vhb, (void*)ctx->adj_rhobar,
                    (void*)ctx->adj_pbar, (void*)ctx->adj_blk, (void*)ctx->adj_pacc,
                    (void*)ctx->adj_divsb, (void*)ctx->adj_tbar, (void*)ctx->adj_tbar2})
        ctx->owned.push_back(p);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(adjoint)");
    return ARMANDO_OK;
}

armando_status alloc_tape(armando_ctx* ctx, int count) {
    cudaError_t e = cudaSuccess;
    const size_t n = (size_t)std::max<int64_t>(ctx->n, 1);
    while ((int)ctx->tape.size() < count) {
        TapeSlot T{};
        T.xh = dalloc<float4>(n, e);
        T.vm = dalloc<float4>(n, e);
        T.vmin = dalloc<float4>(n, e);
        T.rp = dalloc<float4>(n, e);
        T.p = dalloc<float>(n, e);
        T.itype = dalloc<int>(n, e);
        T.nmask = dalloc<unsigned>(n * (ctx->dim == 2 ? mask_words<2>() : mask_words<3>()), e);
        T.keys = dalloc<unsigned>(n, e);
        T.perm = dalloc<int>(n, e);
        T.du = dalloc<float>(n, e);
        T.start = dalloc<int>((size_t)ctx->cell_cap + 1, e);
        T.grid = dalloc<DevGrid>(1, e);
        if (ctx->prm.heat_artificial) T.ulo = dalloc<float>(n, e);
        if (ctx->prm.visc) {
            T.tau = dalloc<float4>(n, e);
            if (ctx->dim == 3) T.tau2 = dalloc<float4>(n, e);
        }
        for (void* p : {(void*)T.xh, (void*)T.vm, (void*)T.vmin, (void*)T.rp, (void*)T.p,
                        (void*)T.itype, (void*)T.nmask, (void*)T.keys, (void*)T.perm, (void*)T.du,
                        (void*)T.start, (void*)T.grid, (void*)T.ulo, (void*)T.tau, (void*)T.tau2})
            ctx->owned.push_back(p);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "cudaMalloc(adjoint tape; a smaller checkpoint_every needs less)");
        ctx->tape.push_back(T);
    }
    return ARMANDO_OK;
}

// Saves the intermediates of the iteration that just ran into tape slot t.
armando_status save_tape(armando_ctx* ctx, int t) {
    const TapeSlot& T = ctx->tape[t];
    const int n = (int)ctx->n;
    cudaStream_t st = ctx->stream;
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    if (ctx->dim == 2)
        k_tape_save<2><<<blocks_for(n, 256), 256, 0, st>>>(ctx->B, skeys, perm, ctx->A.ap, T, n);
    else
        k_tape_save<3><<<blocks_for(n, 256), 256, 0, st>>>(ctx->B, skeys, perm, ctx->A.ap, T, n);
    ctx->launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(T.start, ctx->start, ((size_t)ctx->cell_cap + 1) * sizeof(int),
                       cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(T.grid, ctx->grid, sizeof(DevGrid), cudaMemcpyDeviceToDevice, st));
    return ARMANDO_OK;
}

// Reverse of the iteration held in tape slot t: cotangents adjG (its output
// slot order) -> adjGp (its input slot order); then the two swap roles.
template <int DIM>
int launch_adjoint(armando_ctx* ctx, const StepArgs& S, const TapeSlot& T) {
    cudaStream_t st = ctx->stream;
    const int n = (int)ctx->n;
    const int nb = blocks_for(n, kPassThreads);
    const StateB Bv = tape_view(ctx->B, T, n);
    k_adj_out<<<blocks_for(n, 256), 256, 0, st>>>(Bv, T.du, ctx->adjG, S, ctx->adj_abar,
                                                  ctx->adj_xpart, ctx->adj_vpart, n);
    k_adj_force<DIM><<<nb, kPassThreads, 0, st>>>(Bv, T.keys, T.start, T.grid, ctx->dp, S,
                                                 ctx->adj_abar, ctx->adj_pbar, ctx->adj_rhobar,
                                                 ctx->adj_xF, ctx->adj_vhb, ctx->adj_divsb,
                                                 ctx->adj_tbar, ctx->adj_tbar2, ctx->adj_blk, n);
    int L = 4;
    if (ctx->dp.visc) {
        k_adj_shear<DIM><<<nb, kPassThreads, 0, st>>>(Bv, T.keys, T.start, T.grid, ctx->dp,
                                                     ctx->adj_tbar, ctx->adj_tbar2,
                                                     ctx->adj_rhobar, ctx->adj_xF, ctx->adj_vhb, n);
        ++L;
    }
    k_adj_density<DIM><<<nb, kPassThreads, 0, st>>>(Bv, T.keys, T.start, T.grid, ctx->dp, S,
                                                   ctx->adj_rhobar, ctx->adj_xF, ctx->adj_vhb,
                                                   ctx->adj_xpart, ctx->adj_vpart, ctx->adj_divsb,
                                                   T.perm, ctx->adjGp, n);
    k_adj_params<<<1, 256, 0, st>>>(ctx->adj_blk, nb, ctx->adj_pacc);
    return L;
}

armando_status run_adjoint(armando_ctx* ctx, const StepArgs& S, int t) {
    const TapeSlot& T = ctx->tape[t];
    ctx->launches += ctx->dim == 2 ? launch_adjoint<2>(ctx, S, T) : launch_adjoint<3>(ctx, S, T);
    CK(cudaGetLastError());
    std::swap(ctx->adjG, ctx->adjGp);
    return ARMANDO_OK;
}

armando_status check_adjoint_support(armando_ctx* ctx) {
    if (ctx->n_inst > 1) return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "reverse mode of one particle system only");
    const armando_params& p = ctx->prm;
    if (p.pa_sph != 1 || p.wall_model != 0 || p.scheme != 0 || step_options(p))
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED,
                    "reverse mode supports pa_sph = 1, wall_model 0, summation density, without "
                    "XSPH or h evolution");
    return ARMANDO_OK;
}

// Per-instance device parameters (the time step of each instance included).
armando_status upload_batch_params(armando_ctx* ctx) {
    std::vector<DevParams> hp(ctx->n_inst);
    for (int k = 0; k < ctx->n_inst; ++k) {
        hp[k] = make_dev_params(ctx->prm_inst[k], ctx->tune.reach);
        hp[k].dt = ctx->inst_dt[k];
        hp[k].heat_t_end = ctx->prm_inst[k].heat_t_end;
    }
    CK(cudaMemcpy(ctx->d_params, hp.data(), sizeof(DevParams) * ctx->n_inst, cudaMemcpyHostToDevice));
    return ARMANDO_OK;
}

// Instance bookkeeping of a batch: instance ids, work items (<= kPassThreads
// slots of one instance each), persistent grid sizes.
armando_status alloc_batch(armando_ctx* ctx) {
    cudaError_t e = cudaSuccess;
    const size_t n = (size_t)std::max<int64_t>(ctx->n, 1);
    const int ni = ctx->n_inst;
    ctx->A.inst = dalloc<int>(n, e);
    ctx->B.inst = dalloc<int>(n, e);
    ctx->d_inst0 = dalloc<int>(n, e);
    ctx->d_params = dalloc<DevParams>(ni, e);
    ctx->d_grids = dalloc<DevGrid>(ni, e);
    ctx->d_ncells_inst = dalloc<int>(ni, e);
    ctx->d_inst_items = dalloc<int>(ni + 1, e);
    ctx->d_total_cells = dalloc<int>(1, e);
    ctx->d_queue = dalloc<int>(4, e);
    ctx->d_its = dalloc<int>(1, e);
    std::vector<int> inst0(n, 0), inst_items(ni + 1, 0);
    std::vector<WorkItem> items;
    int64_t s0 = 0;
    for (int k = 0; k < ni; ++k) {
        inst_items[k] = (int)items.size();
        for (int64_t b = 0; b < ctx->inst_n[k]; b += kPassThreads) {
            WorkItem w;
            w.s0 = (int)(s0 + b);
            w.s1 = (int)std::min<int64_t>(s0 + b + kPassThreads, s0 + ctx->inst_n[k]);
            w.inst = k;
            w.pad = 0;
            items.push_back(w);
        }
        for (int64_t i = 0; i < ctx->inst_n[k]; ++i) inst0[s0 + i] = k;
        s0 += ctx->inst_n[k];
    }
    inst_items[ni] = (int)items.size();
    ctx->n_items = (int)items.size();
    ctx->d_items = dalloc<WorkItem>(std::max(ctx->n_items, 1), e);
    ctx->d_part_items = dalloc<float>((size_t)std::max(ctx->n_items, 1) * 8, e);
    for (void* p : {(void*)ctx->A.inst, (void*)ctx->B.inst, (void*)ctx->d_inst0, (void*)ctx->d_params,
                    (void*)ctx->d_grids, (void*)ctx->d_ncells_inst, (void*)ctx->d_inst_items,
                    (void*)ctx->d_total_cells, (void*)ctx->d_queue, (void*)ctx->d_its,
                    (void*)ctx->d_items, (void*)ctx->d_part_items})
        ctx->owned.push_back(p);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(batch)");
    CK(cudaMemcpy(ctx->d_inst0, inst0.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_inst_items, inst_items.data(), sizeof(int) * (ni + 1), cudaMemcpyHostToDevice));
    if (ctx->n_items)
        CK(cudaMemcpy(ctx->d_items, items.data(), sizeof(WorkItem) * ctx->n_items, cudaMemcpyHostToDevice));
    ctx->any_visc = 0;
    ctx->batch_lean = true;
    for (const auto& q : ctx->prm_inst) {
        ctx->any_visc |= q.visc ? 1 : 0;
        ctx->batch_lean = ctx->batch_lean && lean_physics(make_dev_params(q)) && !step_options(q);
    }
    int sms = 0, bd = 0, bs = 0, bf = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    auto occ = [&](auto kd, auto ks, auto kf) -> cudaError_t {
        cudaError_t e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bd, kd, kPassThreads, 0);
        if (e2 == cudaSuccess) e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, ks, kPassThreads, 0);
        if (e2 == cudaSuccess) e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bf, kf, kPassThreads, 0);
        return e2;
    };
    if (ctx->dim == 2) {
        CK(ctx->batch_lean ? occ(k_density_batch<2, true>, k_shear_batch<2>, k_force_batch<2, true>)
                           : occ(k_density_batch<2>, k_shear_batch<2>, k_force_batch<2>));
    } else {
        CK(ctx->batch_lean ? occ(k_density_batch<3, true>, k_shear_batch<3>, k_force_batch<3, true>)
                           : occ(k_density_batch<3>, k_shear_batch<3>, k_force_batch<3>));
    }
    ctx->grid_density = std::max(1, std::min(sms * bd, ctx->n_items));
    ctx->grid_shear = std::max(1, std::min(sms * bs, ctx->n_items));
    ctx->grid_force = std::max(1, std::min(sms * bf, ctx->n_items));
    return upload_batch_params(ctx);
}

armando_status check_step_args(armando_ctx* ctx, const void* x, const void* vx, const void* mass,
                               const void* rho, const void* p, const void* u, const void* hsml,
                               const void* itype, const void* dvdt, const void* dudt, float dt,
                               int its) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    if (!x || !vx || !mass || !rho || !p || !u || !hsml || !itype || !dvdt || !dudt)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL particle array");
    if (!(dt > 0.f) || !std::isfinite(dt)) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "dt must be finite and > 0");
    if (its < 1) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "its must be >= 1");
    return ARMANDO_OK;
}


// ---- Allocation-free cell ids (armando_cell_ids_noalloc) -------------------
// Scratch of the grid reduction in a file-scope device array instead of
// cudaMalloc'd memory. It is held by every device that loads the library until
// the process exits, and shared by every call (which is why overlapping calls
// race on it).
constexpr size_t kNoAllocScratchBytes = 32768;
constexpr size_t kNoAllocPartOff = 0;  // kBBoxBlocks x 8 floats of bbox partials
constexpr size_t kNoAllocGridOff = (size_t)kBBoxBlocks * 8 * sizeof(float);
constexpr size_t kNoAllocFlagsOff = (kNoAllocGridOff + sizeof(DevGrid) + 255) & ~(size_t)255;
constexpr int64_t kNoAllocMaxParticles = (int64_t)1 << 30;
constexpr long long kNoAllocMaxCells = (long long)1 << 30;
static_assert(kNoAllocFlagsOff + sizeof(unsigned) <= kNoAllocScratchBytes, "scratch too small");
static_assert(kNoAllocGridOff % 16 == 0, "grid record alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (the host-side symbol is not a device address).
armando_status noalloc_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error("armando_cell_ids_noalloc: cudaGetDevice failed");
        return ARMANDO_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_last_error("armando_cell_ids_noalloc: device ordinal out of range");
        return ARMANDO_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            set_last_error("armando_cell_ids_noalloc: cudaGetSymbolAddress of the scratch failed");
            return ARMANDO_ERR_CUDA;
        }
        g_noalloc_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_addr[dev];
    return ARMANDO_OK;
}

armando_status noalloc_fail(armando_status st, const char* msg) {
    set_last_error(msg);
    return st;
}

}  // namespace

extern "C" {

armando_status armando_cell_ids_noalloc(const armando_params* params, const float* x,
                                        const float* hsml, int64_t n, int32_t* cell,
                                        void* stream) {
    if (!params) return noalloc_fail(ARMANDO_ERR_INVALID_ARG, "armando_cell_ids_noalloc: params is NULL");
    const int dim = params->dim;
    if (dim != 2 && dim != 3) return noalloc_fail(ARMANDO_ERR_INVALID_ARG, "armando_cell_ids_noalloc: dim must be 2 or 3");
    for (int d = 0; d < dim; ++d)
        if (params->periodic[d] && !(params->period_hi[d] > params->period_lo[d]))
            return noalloc_fail(ARMANDO_ERR_INVALID_ARG, "armando_cell_ids_noalloc: periodic axis needs period_hi > period_lo");
    if (n < 0 || n > kNoAllocMaxParticles)
        return noalloc_fail(ARMANDO_ERR_INVALID_ARG,
                            "armando_cell_ids_noalloc: n must be in [0, 2^30] (limit of the static scratch's grid reduction)");
    if (n == 0) return ARMANDO_OK;
    if (!x || !hsml || !cell) return noalloc_fail(ARMANDO_ERR_INVALID_ARG, "armando_cell_ids_noalloc: NULL array");
    unsigned char* base = nullptr;
    armando_status st = noalloc_scratch(&base);
    if (st != ARMANDO_OK) return st;
    float* part = reinterpret_cast<float*>(base + kNoAllocPartOff);
    DevGrid* grid = reinterpret_cast<DevGrid*>(base + kNoAllocGridOff);
    unsigned* flags = reinterpret_cast<unsigned*>(base + kNoAllocFlagsOff);
    const DevParams dp = make_dev_params(*params);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nn = (int)n;
    // The status word keeps the previous call's value: clear it first.
    if (cudaMemsetAsync(flags, 0, sizeof(unsigned), s) != cudaSuccess) {
        cudaGetLastError();
        return noalloc_fail(ARMANDO_ERR_CUDA, "armando_cell_ids_noalloc: cudaMemsetAsync failed");
    }
    if (dim == 2) k_bbox_partial_raw<2><<<kBBoxBlocks, 256, 0, s>>>(x, hsml, nn, part);
    else k_bbox_partial_raw<3><<<kBBoxBlocks, 256, 0, s>>>(x, hsml, nn, part);
    k_bbox_final<<<1, 256, 0, s>>>(part, kBBoxBlocks, dp, kNoAllocMaxCells, grid, flags);
    if (dim == 2) k_keys_raw<2><<<blocks_for(nn, 256), 256, 0, s>>>(x, nn, grid, reinterpret_cast<int*>(cell));
    else k_keys_raw<3><<<blocks_for(nn, 256), 256, 0, s>>>(x, nn, grid, reinterpret_cast<int*>(cell));
    if (cudaGetLastError() != cudaSuccess) return noalloc_fail(ARMANDO_ERR_CUDA, "armando_cell_ids_noalloc: kernel launch failed");
    unsigned hflags = 0;
    if (cudaMemcpyAsync(&hflags, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return noalloc_fail(ARMANDO_ERR_CUDA, "armando_cell_ids_noalloc: stream synchronisation failed");
    }
    if (hflags & FLAG_PERIODIC_SMALL)
        return noalloc_fail(ARMANDO_ERR_INVALID_ARG, "armando_cell_ids_noalloc: periodic box shorter than 3 cells of 2*max(h)");
    if (hflags & FLAG_GRID_OVERFLOW)
        return noalloc_fail(ARMANDO_ERR_GRID_OVERFLOW, "armando_cell_ids_noalloc: grid has more than 2^30 cells");
    return ARMANDO_OK;
}

void armando_params_default(armando_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->dim = 2;
    p->pa_sph = 1;
    p->rho0 = 1000.f;
    p->c0 = 1.f;
    p->pmin = -INFINITY;
    p->av_alpha = 1.f;
    p->av_beta = 1.f;
    p->av_eta = 0.1f;
    p->ah_g1 = 0.1f;
    p->ah_g2 = 1.f;
    p->ah_eta = 0.1f;
    p->heat_sigma = 1.f;
    p->heat_t_end = INFINITY;
}

int32_t armando_abi_version(void) { return ARMANDO_ABI_VERSION; }

armando_status armando_binary_version(int32_t* version) {
    if (!version) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "version is NULL");
    cudaFuncAttributes a{};
    const cudaError_t e = cudaFuncGetAttributes(&a, k_advance_its);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(nullptr, e == cudaErrorNoDevice ? ARMANDO_ERR_NO_DEVICE : ARMANDO_ERR_CUDA,
                    cudaGetErrorString(e));
    }
    *version = a.binaryVersion;
    return ARMANDO_OK;
}

static armando_status create_impl(armando_ctx** out, int32_t n_inst, const armando_params* params,
                                  int32_t dim, const int64_t* n_fluid, const int64_t* n_wall,
                                  int32_t mem_kind) {
    armando_ctx* ctx = nullptr;
    if (!out) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (n_inst < 1 || !params || !n_fluid || !n_wall)
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "need at least one instance with params and counts");
    int64_t total = 0;
    for (int k = 0; k < n_inst; ++k) {
        std::string why;
        armando_status vs = validate_params(params + k, dim, why);
        if (vs != ARMANDO_OK) return fail(nullptr, vs, why);
        if (n_fluid[k] < 0 || n_wall[k] < 0)
            return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "particle counts out of range");
        total += n_fluid[k] + n_wall[k];
        if (total > (int64_t)INT32_MAX / 2)
            return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "particle counts out of range");
    }
    if (mem_kind != ARMANDO_MEM_HOST && mem_kind != ARMANDO_MEM_DEVICE)
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "mem_kind must be ARMANDO_MEM_HOST or ARMANDO_MEM_DEVICE");
    int dev = 0, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(nullptr, ARMANDO_ERR_NO_DEVICE, "no CUDA device visible");
    }
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return fail(nullptr, ARMANDO_ERR_NO_DEVICE, "cudaGetDeviceProperties failed");
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(nullptr, ARMANDO_ERR_NO_DEVICE,
                    std::string("library is built for sm_103a; device is ") + prop.name);
    ctx = new armando_ctx();
    ctx->device = dev;
    ctx->prm = params[0];
    ctx->dp = make_dev_params(params[0], ctx->tune.reach);
    ctx->dim = dim;
    ctx->n_inst = n_inst;
    for (int k = 0; k < n_inst; ++k) {
        ctx->nf += n_fluid[k];
        ctx->nw += n_wall[k];
        ctx->inst_n.push_back(n_fluid[k] + n_wall[k]);
        ctx->prm_inst.push_back(params[k]);
        ctx->inst_dt.push_back(0.f);
    }
    ctx->n = total;
    ctx->n_work = total;
    ctx->cap = total + (params[0].wall_model == 3 ? ctx->nf : 0);
    ctx->dp.n_real = (int)total;
    ctx->mem_kind = mem_kind;
    if (n_inst > 1)
        for (int k = 0; k < n_inst; ++k)
            if (params[k].wall_model == 3 || params[k].scheme != 0 || step_options(params[k])) {
                delete ctx;
                return fail(nullptr, ARMANDO_ERR_UNSUPPORTED, "batches run the CERN summation-density step without mirror ghosts");
            }
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamDefault);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        armando_status st = cuda_fail(ctx, e, "cudaStreamCreate");
        if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
        delete ctx;
        return st;
    }
    ctx->stream = ctx->own_stream;
    if (const char* sv = std::getenv("ARMANDO_STAGING")) ctx->staging = std::strcmp(sv, "1") == 0;
    if (const char* lv = std::getenv("ARMANDO_NEIGHBOUR_LISTS")) ctx->lists = std::strcmp(lv, "0") != 0;
    if (const char* fv = std::getenv("ARMANDO_FUSED_PREDICTOR")) ctx->fuse_ok = std::strcmp(fv, "0") != 0;
    armando_status st = alloc_state(ctx);
    if (st == ARMANDO_OK && n_inst > 1) st = alloc_batch(ctx);
    if (st != ARMANDO_OK) {
        std::string m = ctx->err;
        armando_destroy(ctx);
        return fail(nullptr, st, m);
    }
    if (cudaMemsetAsync(ctx->flags, 0, sizeof(unsigned), ctx->stream) != cudaSuccess) {
        armando_destroy(ctx);
        return fail(nullptr, ARMANDO_ERR_CUDA, "cudaMemsetAsync");
    }
    *out = ctx;
    return ARMANDO_OK;
}

armando_status armando_create(armando_ctx** out, const armando_params* params, int32_t dim,
                              int64_t n_fluid, int64_t n_wall, int32_t mem_kind) {
    return create_impl(out, 1, params, dim, &n_fluid, &n_wall, mem_kind);
}

armando_status armando_batch_create(armando_ctx** out, int32_t n_instances,
                                    const armando_params* params, int32_t dim,
                                    const int64_t* n_fluid, const int64_t* n_wall,
                                    int32_t mem_kind) {
    return create_impl(out, n_instances, params, dim, n_fluid, n_wall, mem_kind);
}

armando_status armando_set_params(armando_ctx* ctx, const armando_params* params) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    if (ctx->n_inst > 1) return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "batch contexts take their parameters at creation");
    std::string why;
    armando_status vs = validate_params(params, ctx->dim, why);
    if (vs != ARMANDO_OK) return fail(ctx, vs, why);
    if (params->wall_model == 3 && ctx->cap < ctx->n + ctx->nf)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "mirror ghosts (wall_model 3) need a context created with wall_model 3");
    if (sorts_every_step(*params) && ctx->tune.skin != 0)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "mirror ghosts and h evolution sort every iteration: set a tuning with skin 0 first");
    ctx->prm = *params;
    ctx->dp = make_dev_params(*params, ctx->tune.reach);
    ctx->dp.n_real = (int)ctx->n;
    ctx->dp.skin = 0.01f * (float)ctx->tune.skin;
    free_graphs(ctx);
    return ARMANDO_OK;
}

// ---- tuning and autotuner -------------------------------------------------------

namespace {

void release(armando_ctx* c, void* p) {
    if (!p) return;
    auto it = std::find(c->owned.begin(), c->owned.end(), p);
    if (it != c->owned.end()) c->owned.erase(it);
    cudaFree(p);
}

armando_status check_tuning(armando_ctx* ctx, const armando_tuning& t) {
    if (t.reach < 1 || t.reach > 3) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "reach must be 1, 2 or 3");
    if (t.threads_per_particle != 1 && t.threads_per_particle != 2 && t.threads_per_particle != 4)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "threads_per_particle must be 1, 2 or 4");
    if (t.block != 128 && t.block != 256) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "block must be 128 or 256");
    if (t.skin < 0 || t.skin > 100) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "skin must be 0-100 (percent of max h)");
    if (ctx->n_inst > 1 && t.threads_per_particle != 1)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "batches run one thread per particle");
    if (ctx->n_inst > 1 && t.skin != 0)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "batches sort every iteration (skin 0)");
    if (sorts_every_step(ctx->prm) && t.skin != 0)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "mirror ghosts and h evolution sort every iteration (skin 0)");
    return ARMANDO_OK;
}

// Applies a checked tuning. A new reach changes the cell count, so the cell
// table (and the reverse-mode tape, which keeps copies of it) is re-planned on
// the next iteration; any change ends a pending backward sweep.
armando_status apply_tuning(armando_ctx* ctx, const armando_tuning& t) {
    const bool regrid = t.reach != ctx->tune.reach || t.skin != ctx->tune.skin;
    ctx->tune = t;
    ctx->B.mstride = (int)(ctx->cap * t.threads_per_particle);
    ctx->B.mtpp = t.threads_per_particle;
    ctx->dp.reach = t.reach;
    ctx->dp.skin = 0.01f * (float)t.skin;
    ctx->B.xsort = lazy(ctx) ? ctx->xsort_buf : nullptr;
    if (regrid) {
        if (ctx->n_inst > 1) {
            armando_status st = upload_batch_params(ctx);
            if (st != ARMANDO_OK) return st;
        }
        CK(cudaStreamSynchronize(ctx->stream));
        release(ctx, ctx->start);
        ctx->start = nullptr;
        for (const TapeSlot& T : ctx->tape)
            for (void* q : {(void*)T.xh, (void*)T.vm, (void*)T.vmin, (void*)T.rp, (void*)T.p,
                            (void*)T.itype, (void*)T.nmask, (void*)T.keys, (void*)T.perm,
                            (void*)T.du, (void*)T.start, (void*)T.grid, (void*)T.ulo,
                            (void*)T.tau, (void*)T.tau2})
                release(ctx, q);
        ctx->tape.clear();
    }
    ctx->tape_seg = -1;
    ctx->adj_ready = false;
    ctx->next_its = 0;  // the device state no longer belongs to the last call
    free_graphs(ctx);
    // Neighbour lists for a lazily sorting CERN step with one lane per
    // particle, allocated on first use and kept.
    if (ctx->lists && lazy(ctx) && t.threads_per_particle == 1 && ctx->prm.scheme == 0 &&
        !ctx->B.nlist && ctx->prm.wall_model != 3) {
        const int lcap = ctx->dim == 2 ? kListCap2 : kListCap3;
        cudaError_t e = cudaSuccess;
        int* nl = dalloc<int>((size_t)lcap * (size_t)std::max<int64_t>(ctx->cap, 1), e);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(neighbour lists)");
        ctx->owned.push_back(nl);
        int* nc = dalloc<int>((size_t)std::max<int64_t>(ctx->cap, 1), e);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(neighbour counts)");
        ctx->owned.push_back(nc);
        ctx->B.nlist = nl;
        ctx->B.ncount = nc;
        ctx->B.lcap = lcap;
        ctx->B.lstride = (int)ctx->cap;
    }
    return ARMANDO_OK;
}

}  // namespace

armando_status armando_get_tuning(armando_ctx* ctx, armando_tuning* out) {
    if (!ctx || !out) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    *out = ctx->tune;
    return ARMANDO_OK;
}

armando_status armando_set_tuning(armando_ctx* ctx, const armando_tuning* t) {
    if (!ctx || !t) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    armando_status st = check_tuning(ctx, *t);
    if (st != ARMANDO_OK) return st;
    CK(cudaSetDevice(ctx->device));
    if (t->reach == ctx->tune.reach && t->threads_per_particle == ctx->tune.threads_per_particle &&
        t->block == ctx->tune.block && t->skin == ctx->tune.skin)
        return ARMANDO_OK;
    return apply_tuning(ctx, *t);
}

armando_status armando_tuning_candidate(int32_t k, armando_tuning* out) {
    if (!out || k < 0 || k >= ARMANDO_N_TUNINGS)
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "candidate index out of range");
    static const int tpp[3] = {1, 2, 4};
    static const int skin[3] = {10, 20, 40};
    if (k >= 18) {  // a skin for the fastest of the first 18 with this reach
        *out = armando_tuning{1 + (k - 18) / 3, 0, 0, skin[(k - 18) % 3]};
        return ARMANDO_OK;
    }
    out->reach = 1 + k / 6;
    out->threads_per_particle = tpp[(k / 2) % 3];
    out->block = (k % 2) ? 256 : 128;
    out->skin = 0;
    return ARMANDO_OK;
}

armando_status armando_autotune(armando_ctx* ctx, const float* x, const float* vx,
                                const float* mass, const float* rho, const float* p,
                                const float* u, const float* hsml, const int32_t* itype,
                                const float* dvdt, const float* dudt, float dt, int32_t its0,
                                int32_t steps_per_trial, armando_tuning* best,
                                float* ms_per_step) {
    armando_status st = check_step_args(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt, its0);
    if (st != ARMANDO_OK) return st;
    if (ctx->n_inst > 1) return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "autotune one particle system at a time");
    if (steps_per_trial < 1) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "steps_per_trial must be >= 1");
    CK(cudaSetDevice(ctx->device));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    armando_tuning win = ctx->tune;
    float win_ms = -1.f;
    armando_tuning reach_win[4] = {};  // fastest of the first 18 per reach
    float reach_ms[4] = {-1.f, -1.f, -1.f, -1.f};
    for (int k = 0; k < ARMANDO_N_TUNINGS; ++k) {
        armando_tuning t;
        armando_tuning_candidate(k, &t);
        if (k >= 18) {  // second stage: a sort skin on that reach's fastest tuning
            if (reach_ms[t.reach] < 0.f) {
                if (ms_per_step) ms_per_step[k] = -1.f;
                continue;
            }
            const int skin = t.skin;
            t = reach_win[t.reach];
            t.skin = skin;
        }
        float ms = -1.f;
        if (t.skin != 0 && sorts_every_step(ctx->prm)) {  // sort every iteration
            if (ms_per_step) ms_per_step[k] = -1.f;
            continue;
        }
        if ((st = apply_tuning(ctx, t)) != ARMANDO_OK) break;
        if (armando_status cs = clear_flags(ctx); cs != ARMANDO_OK) return cs;
        st = load_inputs(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt);
        if (st == ARMANDO_OK) st = plan_grid(ctx);
        if (st == ARMANDO_OK) st = build_wall_grid(ctx);
        if (st == ARMANDO_OK) st = prepare_gpuc(ctx);
        if (st == ARMANDO_OK) st = prepare_options(ctx);
        // Two untimed iterations capture the graphs of the first and of the
        // following iterations; then the timed ones.
        for (int w = 0; w < 2 && st == ARMANDO_OK; ++w) st = run_step(ctx, make_args(ctx, dt, its0 + w));
        if (st == ARMANDO_OK) {
            CK(cudaEventRecord(e0, ctx->stream));
            for (int q = 0; q < steps_per_trial && st == ARMANDO_OK; ++q)
                st = run_step(ctx, make_args(ctx, dt, its0 + 2 + q));
            CK(cudaEventRecord(e1, ctx->stream));
        }
        if (st == ARMANDO_OK) st = check_flags(ctx);
        if (st == ARMANDO_OK) {
            float el = 0.f;
            CK(cudaEventElapsedTime(&el, e0, e1));
            ms = el / (float)steps_per_trial;
            if (win_ms < 0.f || ms < win_ms) {
                win_ms = ms;
                win = t;
            }
            if (k < 18 && (reach_ms[t.reach] < 0.f || ms < reach_ms[t.reach])) {
                reach_ms[t.reach] = ms;
                reach_win[t.reach] = t;
            }
        } else if (st == ARMANDO_ERR_CUDA) {
            break;  // a device error ends the search
        }
        st = ARMANDO_OK;  // a candidate that does not apply is skipped
        if (ms_per_step) ms_per_step[k] = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != ARMANDO_OK) return st;
    if (win_ms < 0.f) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "no candidate tuning runs on this state");
    if ((st = apply_tuning(ctx, win)) != ARMANDO_OK) return st;
    if (best) *best = win;
    return ARMANDO_OK;
}

armando_status armando_batch_integrate(armando_ctx* ctx, float* x, float* vx, const float* mass,
                                       float* rho, float* p, float* u, const float* hsml,
                                       const int32_t* itype, float* dvdt, float* dudt,
                                       const float* dt, int32_t its0, int32_t steps) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    if (!dt) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "dt is NULL");
    armando_status st = check_step_args(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt[0], its0);
    if (st != ARMANDO_OK) return st;
    if (ctx->n_inst == 1) return armando_integrate(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt[0], its0, steps);
    if (steps < 0) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "steps must be >= 0");
    bool changed = false;
    for (int k = 0; k < ctx->n_inst; ++k) {
        if (!(dt[k] > 0.f) || !std::isfinite(dt[k]))
            return fail(ctx, ARMANDO_ERR_INVALID_ARG, "every dt must be finite and > 0");
        changed |= dt[k] != ctx->inst_dt[k];
    }
    CK(cudaSetDevice(ctx->device));
    if (ctx->n == 0 || steps == 0) return ARMANDO_OK;
    if (changed) {
        for (int k = 0; k < ctx->n_inst; ++k) ctx->inst_dt[k] = dt[k];
        st = upload_batch_params(ctx);
        if (st != ARMANDO_OK) return st;
    }
    if (armando_status cs = clear_flags(ctx); cs != ARMANDO_OK) return cs;
    st = load_inputs(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt);
    if (st != ARMANDO_OK) return st;
    st = plan_grid(ctx);
    if (st != ARMANDO_OK) return st;
    const int its = its0;
    CK(cudaMemcpyAsync(ctx->d_its, &its, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    for (int k = 0; k < steps; ++k) {
        st = run_batch_step(ctx);
        if (st != ARMANDO_OK) return st;
    }
    ctx->last_dt = dt[0];
    ctx->next_its = its0 + steps;
    st = store_outputs(ctx, x, vx, rho, p, u, dvdt, dudt);
    if (st != ARMANDO_OK) return st;
    return finish_call(ctx);
}

static_assert(kPassThreads == ARMANDO_BATCH_BLOCK, "the batched passes' CTA size");

armando_status armando_batch_autotune(armando_ctx* ctx, const float* x, const float* vx,
                                      const float* mass, const float* rho, const float* p,
                                      const float* u, const float* hsml, const int32_t* itype,
                                      const float* dvdt, const float* dudt, const float* dt,
                                      int32_t its0, int32_t steps_per_trial, armando_tuning* best,
                                      float* ms_per_step) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    if (!dt) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "dt is NULL");
    if (ctx->n_inst == 1)
        return armando_autotune(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt[0], its0,
                                steps_per_trial, best, ms_per_step);
    armando_status st = check_step_args(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt[0], its0);
    if (st != ARMANDO_OK) return st;
    if (steps_per_trial < 1) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "steps_per_trial must be >= 1");
    bool changed = false;
    for (int k = 0; k < ctx->n_inst; ++k) {
        if (!(dt[k] > 0.f) || !std::isfinite(dt[k]))
            return fail(ctx, ARMANDO_ERR_INVALID_ARG, "every dt must be finite and > 0");
        changed |= dt[k] != ctx->inst_dt[k];
    }
    CK(cudaSetDevice(ctx->device));
    if (changed) {
        for (int k = 0; k < ctx->n_inst; ++k) ctx->inst_dt[k] = dt[k];
        if ((st = upload_batch_params(ctx)) != ARMANDO_OK) return st;
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    armando_tuning win = ctx->tune;
    float win_ms = -1.f;
    for (int k = 0; k < ARMANDO_N_TUNINGS; ++k) {
        armando_tuning t;
        armando_tuning_candidate(k, &t);
        float ms = -1.f;
        // The batched passes run one thread per particle in CTAs of one work
        // item and sort every iteration: the candidates differ in reach.
        if (k >= 18 || t.threads_per_particle != 1 || t.block != kPassThreads) {
            if (ms_per_step) ms_per_step[k] = ms;
            continue;
        }
        if ((st = apply_tuning(ctx, t)) != ARMANDO_OK) break;
        if ((st = clear_flags(ctx)) != ARMANDO_OK) break;
        st = load_inputs(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt);
        if (st == ARMANDO_OK) st = plan_grid(ctx);
        if (st == ARMANDO_OK) {
            const int its = its0;
            CK(cudaMemcpyAsync(ctx->d_its, &its, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
            st = run_batch_step(ctx);  // untimed: captures the step graph
        }
        if (st == ARMANDO_OK) {
            CK(cudaEventRecord(e0, ctx->stream));
            for (int q = 0; q < steps_per_trial && st == ARMANDO_OK; ++q) st = run_batch_step(ctx);
            CK(cudaEventRecord(e1, ctx->stream));
        }
        if (st == ARMANDO_OK) st = check_flags(ctx);
        if (st == ARMANDO_OK) {
            float el = 0.f;
            CK(cudaEventElapsedTime(&el, e0, e1));
            ms = el / (float)steps_per_trial;
            if (win_ms < 0.f || ms < win_ms) {
                win_ms = ms;
                win = t;
            }
        } else if (st == ARMANDO_ERR_CUDA) {
            break;
        }
        st = ARMANDO_OK;
        if (ms_per_step) ms_per_step[k] = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != ARMANDO_OK) return st;
    if (win_ms < 0.f) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "no candidate tuning runs on this batch");
    if ((st = apply_tuning(ctx, win)) != ARMANDO_OK) return st;
    if (best) *best = win;
    ctx->next_its = 0;  // the trials left the device state behind
    return ARMANDO_OK;
}

armando_status armando_integrate(armando_ctx* ctx, float* x, float* vx, const float* mass,
                                 float* rho, float* p, float* u, const float* hsml,
                                 const int32_t* itype, float* dvdt, float* dudt, float dt,
                                 int32_t its0, int32_t steps) {
    armando_status st = check_step_args(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt, its0);
    if (st != ARMANDO_OK) return st;
    ctx->adj_ready = false;
    if (ctx->n_inst > 1) {
        std::vector<float> dts(ctx->n_inst, dt);
        return armando_batch_integrate(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt,
                                       dts.data(), its0, steps);
    }
    if (steps < 0) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "steps must be >= 0");
    CK(cudaSetDevice(ctx->device));
    if (ctx->n == 0 || steps == 0) return ARMANDO_OK;
    if (armando_status cs = clear_flags(ctx); cs != ARMANDO_OK) return cs;
    st = load_inputs(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt,
                     overlap_eligible(ctx, steps));
    if (st != ARMANDO_OK) return st;
    const bool split = ctx->split_in;
    st = plan_grid(ctx);
    if (st != ARMANDO_OK) return st;
    st = build_wall_grid(ctx);
    if (st != ARMANDO_OK) return st;
    st = prepare_gpuc(ctx);
    if (st != ARMANDO_OK) return st;
    st = prepare_options(ctx);
    if (st != ARMANDO_OK) return st;
    for (int k = 0; k < steps; ++k) {
        st = split ? run_overlapped_step(ctx, make_args(ctx, dt, its0 + k), rho, p)
                   : run_step(ctx, make_args(ctx, dt, its0 + k));
        if (st != ARMANDO_OK) return st;
    }
    st = keep_options(ctx);
    if (st != ARMANDO_OK) return st;
    ctx->last_dt = dt;
    ctx->next_its = its0 + steps;
    st = store_outputs(ctx, x, vx, rho, p, u, dvdt, dudt, split);
    if (st != ARMANDO_OK) return st;
    return finish_call(ctx);
}

armando_status armando_step(armando_ctx* ctx, float* x, float* vx, const float* mass, float* rho,
                            float* p, float* u, const float* hsml, const int32_t* itype,
                            float* dvdt, float* dudt, float dt, int32_t its) {
    return armando_integrate(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt, its, 1);
}

armando_status armando_integrate_open(armando_ctx* ctx, float* x, float* vx, float* mass,
                                      float* rho, float* p, float* u, float* hsml,
                                      int32_t* itype, float* dvdt, float* dudt, float dt,
                                      int32_t its0, int32_t steps, int64_t* n_particles) {
    if (!ctx || !n_particles) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    armando_status st = check_step_args(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt, its0);
    if (st != ARMANDO_OK) return st;
    if (ctx->n_inst > 1 || ctx->prm.scheme == 0)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "open boundaries belong to the GPU-C schemes (scheme 1, 2) of one system");
    if (!ctx->open_set) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "call armando_set_open_boundaries first");
    if (steps < 0 || *n_particles < 0 || *n_particles > ctx->n)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "steps >= 0 and 0 <= *n_particles <= capacity");
    CK(cudaSetDevice(ctx->device));
    ctx->adj_ready = false;
    if (armando_status cs = clear_flags(ctx); cs != ARMANDO_OK) return cs;
    if ((st = load_inputs(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt)) != ARMANDO_OK) return st;
    int64_t n = *n_particles, next_id = n;
    if ((st = prepare_open(ctx)) != ARMANDO_OK) return st;
    if ((st = prepare_gpuc(ctx)) != ARMANDO_OK) return st;
    ctx->n_work = std::max<int64_t>(n, 1);
    st = plan_grid(ctx);
    ctx->n_work = ctx->n;
    if (st != ARMANDO_OK) return st;
    if ((st = fit_cells_to_box(ctx)) != ARMANDO_OK) return st;
    for (int k = 0; k < steps && st == ARMANDO_OK; ++k) {
        if ((st = emit_inlets(ctx, dt, n, next_id)) != ARMANDO_OK) break;
        st = ctx->dim == 2 ? remove_outflow<2>(ctx, n) : remove_outflow<3>(ctx, n);
        if (st != ARMANDO_OK || n == 0) continue;
        ctx->n_work = n;
        ctx->num_tiles = blocks_for(n, kSortTile);
        const StepArgs S = make_args(ctx, dt, its0 + k);
        const int L = ctx->dim == 2 ? launch_gpuc_step<2>(ctx, S, nullptr)
                                    : launch_gpuc_step<3>(ctx, S, nullptr);  // the count changes: sort
        ctx->launches += L;
        ctx->steps_done += 1;
        ctx->sorts_host += 1;
        ctx->n_work = ctx->n;
        ctx->num_tiles = blocks_for(ctx->n, kSortTile);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "kernel launch");
    }
    ctx->n_work = ctx->n;
    ctx->num_tiles = blocks_for(ctx->n, kSortTile);
    if (st != ARMANDO_OK) return st;
    st = ctx->dim == 2 ? store_open<2>(ctx, n, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt)
                       : store_open<3>(ctx, n, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt);
    if (st != ARMANDO_OK) return st;
    *n_particles = n;
    ctx->next_its = 0;  // the device state is the open run's, in its own order
    return check_flags(ctx);
}

armando_status armando_cell_ids(armando_ctx* ctx, const float* x, const float* hsml, int32_t* cell) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    if (ctx->n_inst > 1) return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "cell ids of one particle system only");
    if (!x || !hsml || !cell) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL array");
    CK(cudaSetDevice(ctx->device));
    if (ctx->n == 0) return ARMANDO_OK;
    const int nn = (int)ctx->n;
    const size_t n = (size_t)ctx->n, nd = n * ctx->dim;
    cudaStream_t st = ctx->stream;
    if (armando_status cs = clear_flags(ctx); cs != ARMANDO_OK) return cs;
    const float* dx = x;
    const float* dh = hsml;
    int* dcell = reinterpret_cast<int*>(cell);
    if (ctx->mem_kind == ARMANDO_MEM_HOST) {
        CK(cudaMemcpyAsync(ctx->s_x, x, nd * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->s_h, hsml, n * 4, cudaMemcpyHostToDevice, st));
        dx = ctx->s_x;
        dh = ctx->s_h;
        dcell = ctx->s_itype;  // scratch int[n]
    }
    if (ctx->dim == 2) k_load_xh<2><<<blocks_for(nn, 256), 256, 0, st>>>(dx, dh, ctx->A, nn);
    else k_load_xh<3><<<blocks_for(nn, 256), 256, 0, st>>>(dx, dh, ctx->A, nn);
    ctx->launches += 1;
    CK(cudaGetLastError());
    armando_status s = plan_grid(ctx);
    if (s != ARMANDO_OK) return s;
    DevParams dp1 = ctx->dp;  // link_list's own grid, whatever the tuning
    dp1.reach = 1;
    dp1.skin = 0.f;
    k_bbox_partial<<<kBBoxBlocks, 256, 0, st>>>(ctx->A.xh, nn, ctx->dim, ctx->bbox_part);
    k_bbox_final<<<1, 256, 0, st>>>(ctx->bbox_part, kBBoxBlocks, dp1, ctx->cell_cap, ctx->grid,
                                    ctx->flags);
    if (ctx->dim == 2) k_keys_only<2><<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A.xh, nn, ctx->grid, dcell);
    else k_keys_only<3><<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A.xh, nn, ctx->grid, dcell);
    ctx->launches += 3;
    CK(cudaGetLastError());
    if (ctx->mem_kind == ARMANDO_MEM_HOST)
        CK(cudaMemcpyAsync(cell, dcell, n * 4, cudaMemcpyDeviceToHost, st));
    return check_flags(ctx);
}

armando_status armando_neighbours(armando_ctx* ctx, const float* x, const float* hsml,
                                  int64_t* offs, int32_t* nbr, int64_t cap, int64_t* total) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    if (ctx->n_inst > 1) return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "neighbour lists of one particle system only");
    if (!x || !hsml || !offs || !total) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL array");
    CK(cudaSetDevice(ctx->device));
    const int nn = (int)ctx->n;
    const size_t n = (size_t)ctx->n, nd = n * ctx->dim;
    *total = 0;
    offs[0] = 0;
    if (nn == 0) return ARMANDO_OK;
    cudaStream_t st = ctx->stream;
    if (armando_status cs = clear_flags(ctx); cs != ARMANDO_OK) return cs;
    float* dx = nullptr;
    float* dh = nullptr;
    cudaError_t e = cudaSuccess;
    dx = dalloc<float>(nd, e);
    dh = dalloc<float>(n, e);
    int* cnt = dalloc<int>(n, e);
    long long* doffs = dalloc<long long>(n + 1, e);
    std::vector<void*> tmp = {dx, dh, cnt, doffs};
    auto cleanup = [&]() {
        for (void* q : tmp) cudaFree(q);
    };
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(ctx, e, "cudaMalloc");
    }
#define CKT(call)                                                    \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) {                                     \
            cleanup();                                               \
            return cuda_fail(ctx, e_, #call);                        \
        }                                                            \
    } while (0)
    CKT(cudaMemcpyAsync(dx, x, nd * 4, cudaMemcpyHostToDevice, st));
    CKT(cudaMemcpyAsync(dh, hsml, n * 4, cudaMemcpyHostToDevice, st));
    if (ctx->dim == 2) k_load_xh<2><<<blocks_for(nn, 256), 256, 0, st>>>(dx, dh, ctx->A, nn);
    else k_load_xh<3><<<blocks_for(nn, 256), 256, 0, st>>>(dx, dh, ctx->A, nn);
    CKT(cudaGetLastError());
    armando_status s = plan_grid(ctx);
    if (s != ARMANDO_OK) {
        cleanup();
        return s;
    }
    int L = ctx->dim == 2 ? launch_grid_and_sort<2>(ctx, nullptr, st)
                          : launch_grid_and_sort<3>(ctx, nullptr, st);
    ctx->next_its = 0;  // A now holds these positions, not a step's state
    const unsigned* skeys = ctx->keys[ctx->passes & 1];
    const int* perm = ctx->vals[ctx->passes & 1];
    k_reorder_xh<<<blocks_for(nn, 256), 256, 0, st>>>(ctx->A, perm, ctx->B, nn);
    if (ctx->dim == 2)
        k_count_nbrs<2><<<blocks_for(nn, 128), 128, 0, st>>>(ctx->B, skeys, ctx->start, ctx->grid, cnt, nn);
    else
        k_count_nbrs<3><<<blocks_for(nn, 128), 128, 0, st>>>(ctx->B, skeys, ctx->start, ctx->grid, cnt, nn);
    ctx->launches += L + 3;
    CKT(cudaGetLastError());
    std::vector<int> hc(n);
    CKT(cudaMemcpyAsync(hc.data(), cnt, n * 4, cudaMemcpyDeviceToHost, st));
    CKT(cudaStreamSynchronize(st));
    std::vector<long long> ho(n + 1, 0);
    for (size_t i = 0; i < n; ++i) ho[i + 1] = ho[i] + hc[i];
    *total = ho[n];
    for (size_t i = 0; i <= n; ++i) offs[i] = ho[i];
    if (ho[n] > cap || !nbr) {
        cleanup();
        armando_status fs = check_flags(ctx);
        if (fs != ARMANDO_OK) return fs;
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "neighbour capacity too small (see *total)");
    }
    int* dnbr = dalloc<int>((size_t)std::max<long long>(ho[n], 1), e);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(ctx, e, "cudaMalloc");
    }
    tmp.push_back(dnbr);
    CKT(cudaMemcpyAsync(doffs, ho.data(), (n + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
    if (ctx->dim == 2)
        k_fill_nbrs<2><<<blocks_for(nn, 128), 128, 0, st>>>(ctx->B, skeys, ctx->start, ctx->grid, doffs, dnbr, nn);
    else
        k_fill_nbrs<3><<<blocks_for(nn, 128), 128, 0, st>>>(ctx->B, skeys, ctx->start, ctx->grid, doffs, dnbr, nn);
    ctx->launches += 1;
    CKT(cudaGetLastError());
    CKT(cudaMemcpyAsync(nbr, dnbr, (size_t)ho[n] * 4, cudaMemcpyDeviceToHost, st));
    CKT(cudaStreamSynchronize(st));
    for (size_t i = 0; i < n; ++i) std::sort(nbr + ho[i], nbr + ho[i + 1]);
#undef CKT
    cleanup();
    return check_flags(ctx);
}

// Marks a reverse-mode forward run or replay for its duration.
struct ReverseScope {
    armando_ctx* c;
    explicit ReverseScope(armando_ctx* ctx) : c(ctx) { c->reverse_run = true; }
    ~ReverseScope() { c->reverse_run = false; }
};

armando_status armando_forward_checkpointed(armando_ctx* ctx, float* x, float* vx,
                                           const float* mass, float* rho, float* p, float* u,
                                           const float* hsml, const int32_t* itype, float* dvdt,
                                           float* dudt, float dt, int32_t its0, int32_t steps,
                                           int32_t checkpoint_every) {
    armando_status st = check_step_args(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt, dt, its0);
    if (st != ARMANDO_OK) return st;
    if ((st = check_adjoint_support(ctx)) != ARMANDO_OK) return st;
    if (steps < 1 || checkpoint_every < 1)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "steps and checkpoint_every must be >= 1");
    CK(cudaSetDevice(ctx->device));
    ctx->adj_ready = false;
    ReverseScope rv(ctx);
    if (armando_status cs = clear_flags(ctx); cs != ARMANDO_OK) return cs;
    if ((st = load_inputs(ctx, x, vx, mass, rho, p, u, hsml, itype, dvdt, dudt)) != ARMANDO_OK) return st;
    if ((st = plan_grid(ctx)) != ARMANDO_OK) return st;
    if ((st = alloc_adjoint(ctx)) != ARMANDO_OK) return st;
    const int K = checkpoint_every;
    const int nck = (steps + K - 1) / K;
    while ((int)ctx->ckpts.size() < nck) {
        StateA a{};
        if ((st = alloc_stateA(ctx, a)) != ARMANDO_OK) return st;
        ctx->ckpts.push_back(a);
    }
    if ((st = alloc_tape(ctx, std::min(K, steps))) != ARMANDO_OK) return st;
    // The last segment is taped as it runs: the backward sweep starts there
    // without a replay.
    const int last = (nck - 1) * K;
    ctx->tape_seg = -1;
    for (int k = 0; k < steps; ++k) {
        if (k % K == 0 && (st = copy_stateA(ctx, ctx->ckpts[k / K], ctx->A)) != ARMANDO_OK) return st;
        // Reverse mode sorts every iteration, so a replay from a checkpoint
        // repeats the forward bit for bit.
        if ((st = force_sort(ctx)) != ARMANDO_OK) return st;
        if ((st = run_step(ctx, make_args(ctx, dt, its0 + k))) != ARMANDO_OK) return st;
        if (k >= last && (st = save_tape(ctx, k - last)) != ARMANDO_OK) return st;
    }
    ctx->tape_seg = nck - 1;
    ctx->last_dt = dt;
    ctx->next_its = its0 + steps;
    ctx->adj_its0 = its0;
    ctx->adj_steps = steps;
    ctx->adj_K = K;
    ctx->adj_dt = dt;
    if ((st = store_outputs(ctx, x, vx, rho, p, u, dvdt, dudt)) != ARMANDO_OK) return st;
    if ((st = check_flags(ctx)) != ARMANDO_OK) return st;
    ctx->adj_ready = true;
    return ARMANDO_OK;
}

armando_status armando_backward(armando_ctx* ctx, const float* x_bar, const float* v_bar,
                                const float* u_bar, const float* p_bar, const float* dvdt_bar,
                                const float* dudt_bar, float* x0_bar, float* v0_bar,
                                float* u0_bar, float* dvdt0_bar, float* dudt0_bar,
                                armando_param_grads* grads) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    if (!ctx->adj_ready)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "call armando_forward_checkpointed first");
    CK(cudaSetDevice(ctx->device));
    armando_status st = ARMANDO_OK;
    const int nn = (int)ctx->n;
    const size_t n = (size_t)ctx->n, nd = n * ctx->dim;
    cudaStream_t sm = ctx->stream;
    const bool host = ctx->mem_kind == ARMANDO_MEM_HOST;
    // Output cotangents into the slot order of the final state (A after the forward).
    const float* in[6] = {x_bar, v_bar, u_bar, p_bar, dvdt_bar, dudt_bar};
    const size_t len[6] = {nd, nd, n, n, nd, n};
    float* stage[6] = {ctx->s_x, ctx->s_v, ctx->s_u, ctx->s_p, ctx->s_dvdt, ctx->s_dudt};
    const float* dev_in[6];
    for (int k = 0; k < 6; ++k) {
        dev_in[k] = in[k];
        if (host && in[k]) {
            CK(cudaMemcpyAsync(stage[k], in[k], len[k] * 4, cudaMemcpyHostToDevice, sm));
            dev_in[k] = stage[k];
        }
    }
    // Device memory: ordered by the context's stream (see load_inputs).
    if (ctx->dim == 2)
        k_adj_load<2><<<blocks_for(nn, 256), 256, 0, sm>>>(ctx->A.id, dev_in[0], dev_in[1], dev_in[2],
                                                         dev_in[4], dev_in[5], dev_in[3], ctx->adjG,
                                                         ctx->adj_pbar, nn);
    else
        k_adj_load<3><<<blocks_for(nn, 256), 256, 0, sm>>>(ctx->A.id, dev_in[0], dev_in[1], dev_in[2],
                                                         dev_in[4], dev_in[5], dev_in[3], ctx->adjG,
                                                         ctx->adj_pbar, nn);
    ctx->launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(ctx->adj_pacc, 0, sizeof(double) * ADJ_NPARAM, sm));
    const int K = ctx->adj_K, its0 = ctx->adj_its0, steps = ctx->adj_steps;
    const float dt = ctx->adj_dt;
    const int nck = (steps + K - 1) / K;
    bool first = true;
    for (int c = nck - 1; c >= 0; --c) {
        const int a0 = c * K, len = std::min(K, steps - a0);
        if (ctx->tape_seg != c) {  // replay the segment from its checkpoint, taping it
            ReverseScope rv(ctx);
            ctx->tape_seg = -1;
            if ((st = copy_stateA(ctx, ctx->A, ctx->ckpts[c])) != ARMANDO_OK) return st;
            for (int t = 0; t < len; ++t) {
                if ((st = force_sort(ctx)) != ARMANDO_OK) return st;
                if ((st = run_step(ctx, make_args(ctx, dt, its0 + a0 + t))) != ARMANDO_OK) return st;
                if ((st = save_tape(ctx, t)) != ARMANDO_OK) return st;
            }
            ctx->tape_seg = c;
        }
        for (int t = len - 1; t >= 0; --t) {
            const StepArgs S = make_args(ctx, dt, its0 + a0 + t);
            if ((st = run_adjoint(ctx, S, t)) != ARMANDO_OK) return st;
            if (first) {  // the pressure cotangent belongs to the last iteration only
                CK(cudaMemsetAsync(ctx->adj_pbar, 0, n * 4, sm));
                first = false;
            }
        }
    }
    // adjG is now in the slot order of the first input state = caller order.
    const bool want[5] = {x0_bar != nullptr, v0_bar != nullptr, u0_bar != nullptr,
                          dvdt0_bar != nullptr, dudt0_bar != nullptr};
    float* dst[5] = {x0_bar, v0_bar, u0_bar, dvdt0_bar, dudt0_bar};
    float* dstage[5] = {ctx->s_x, ctx->s_v, ctx->s_u, ctx->s_dvdt, ctx->s_dudt};
    float* kout[5];
    for (int k = 0; k < 5; ++k) kout[k] = want[k] ? (host ? dstage[k] : dst[k]) : nullptr;
    if (ctx->dim == 2)
        k_adj_store<2><<<blocks_for(nn, 256), 256, 0, sm>>>(ctx->adjG, nn, kout[0], kout[1], kout[2],
                                                          kout[3], kout[4]);
    else
        k_adj_store<3><<<blocks_for(nn, 256), 256, 0, sm>>>(ctx->adjG, nn, kout[0], kout[1], kout[2],
                                                          kout[3], kout[4]);
    ctx->launches += 1;
    CK(cudaGetLastError());
    const size_t olen[5] = {nd, nd, n, nd, n};
    if (host)
        for (int k = 0; k < 5; ++k)
            if (want[k]) CK(cudaMemcpyAsync(dst[k], dstage[k], olen[k] * 4, cudaMemcpyDeviceToHost, sm));
    double acc[ADJ_NPARAM];
    CK(cudaMemcpyAsync(acc, ctx->adj_pacc, sizeof(acc), cudaMemcpyDeviceToHost, sm));
    if ((st = check_flags(ctx)) != ARMANDO_OK) return st;
    if (grads) {
        grads->av_alpha = acc[ADJ_ALPHA];
        grads->av_beta = acc[ADJ_BETA];
        grads->c0 = acc[ADJ_C0];
        grads->heat_q0 = acc[ADJ_Q0];
    }
    // The forward's final state is gone from A; a further backward needs a new forward.
    ctx->adj_ready = false;
    ctx->tape_seg = -1;
    return ARMANDO_OK;
}

armando_status armando_get_stream(armando_ctx* ctx, void** stream) {
    if (!ctx || !stream) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    *stream = (void*)ctx->stream;
    return ARMANDO_OK;
}

armando_status armando_profile_phases(armando_ctx* ctx, int32_t steps, float* ms_per_phase) {
    if (!ctx || !ms_per_phase || steps < 1) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "bad argument");
    if (!ctx->start || ctx->next_its < 2 || !(ctx->last_dt > 0.f))
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "no device state: call armando_integrate first");
    if (ctx->prm.wall_model == 3 || ctx->prm.scheme != 0)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "phase timing covers the CERN scheme without mirror ghosts");
    CK(cudaSetDevice(ctx->device));
    cudaEvent_t ev[ARMANDO_N_PHASES + 1];
    for (auto& e : ev) CK(cudaEventCreate(&e));
    double acc[ARMANDO_N_PHASES] = {0, 0, 0, 0, 0, 0};
    armando_status st = ARMANDO_OK;
    for (int k = 0; k < steps && st == ARMANDO_OK; ++k) {
        const StepArgs S = make_args(ctx, ctx->last_dt, ctx->next_its);
        int L = ctx->n_inst > 1 ? launch_batch_step_any(ctx, ev)
                : ctx->dim == 2 ? launch_step_phased<2>(ctx, S, ev)
                                : launch_step_phased<3>(ctx, S, ev);
        ctx->launches += L;
        ctx->steps_done += 1;
        ctx->next_its += 1;
        if (ctx->n_inst == 1 && fused(ctx)) swap_state(ctx);
        cudaError_t e = cudaEventSynchronize(ev[ARMANDO_N_PHASES]);
        if (e != cudaSuccess) {
            st = cuda_fail(ctx, e, "profile step");
            break;
        }
        for (int ph = 0; ph < ARMANDO_N_PHASES; ++ph) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[ph], ev[ph + 1]);
            acc[ph] += ms;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (st != ARMANDO_OK) return st;
    for (int ph = 0; ph < ARMANDO_N_PHASES; ++ph) ms_per_phase[ph] = (float)(acc[ph] / steps);
    return check_flags(ctx);
}

armando_status armando_sync(armando_ctx* ctx) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!ctx->pending) return ARMANDO_OK;
    // The status of the asynchronous calls since the last report (the error
    // word is sticky until then): report it once, then start clean.
    ctx->pending = false;
    armando_status st = eval_flags(ctx);
    if (st != ARMANDO_OK) CK(cudaMemsetAsync(ctx->flags, 0, sizeof(unsigned), ctx->stream));
    return st;
}

armando_status armando_set_stream(armando_ctx* ctx, void* stream) {
    if (!ctx) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "ctx is NULL");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    if (next == ctx->stream) return ARMANDO_OK;
    // Work already enqueued on the previous stream comes first.
    cudaEvent_t ev = nullptr;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(next, ev, 0);
    cudaEventDestroy(ev);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "armando_set_stream");
    ctx->stream = next;
    return ARMANDO_OK;
}

armando_status armando_get_stats(const armando_ctx* cctx, armando_stats* out) {
    if (!cctx || !out) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    out->steps_done = cctx->steps_done;
    out->n_particles = cctx->n;
    out->cell_capacity = cctx->cell_cap;
    out->gpu_launches = cctx->launches;
    if (cctx->have_grid) {
        const DevGrid& g = cctx->last_grid;
        out->n_cells = g.ncells;
        for (int d = 0; d < 3; ++d) {
            out->grid_dims[d] = g.n[d];
            out->grid_origin[d] = g.o[d];
            out->grid_cell_size[d] = g.size[d];
        }
    }
    out->device_flags = cctx->h_flags ? *cctx->h_flags : 0u;
    out->sorts_done = cctx->sorts_done + cctx->sorts_host;
    out->ghosts = cctx->ghosts_last;
    return ARMANDO_OK;
}

const char* armando_last_error(const armando_ctx* ctx) {
    return ctx ? ctx->err.c_str() : g_last_error;
}

armando_status armando_set_open_boundaries(armando_ctx* ctx, int32_t n_inlets,
                                           const armando_inlet* inlets, int32_t n_outlets,
                                           const armando_outlet* outlets, const float box_lo[3],
                                           const float box_hi[3]) {
    if (!ctx || !box_lo || !box_hi || (n_inlets && !inlets) || (n_outlets && !outlets))
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    if (n_inlets < 0 || n_inlets > ARMANDO_MAX_OPEN || n_outlets < 0 || n_outlets > ARMANDO_MAX_OPEN)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "at most ARMANDO_MAX_OPEN inlets and outlets");
    for (int k = 0; k < n_inlets; ++k) {
        const armando_inlet& I = inlets[k];
        const float nn = I.normal[0] * I.normal[0] + I.normal[1] * I.normal[1] + I.normal[2] * I.normal[2];
        if (I.itype != 0 && (!(nn > 0.f) || !(I.hsml > 0.f) || !(I.radius >= 0.f) || !(I.speed >= 0.f) ||
                             !(I.mass > 0.f) || !(I.rho > 0.f)))
            return fail(ctx, ARMANDO_ERR_INVALID_ARG, "inlet needs a normal, hsml, mass, rho > 0 and radius, speed >= 0");
    }
    ctx->inlets.assign(inlets, inlets + n_inlets);
    ctx->inlet_dist.assign(n_inlets, 0.f);
    std::memset(&ctx->open, 0, sizeof ctx->open);
    ctx->open.n_out = n_outlets;
    for (int k = 0; k < n_outlets; ++k) {
        for (int d = 0; d < 3; ++d) {
            ctx->open.out[k].o[d] = outlets[k].origin[d];
            ctx->open.out[k].n[d] = outlets[k].normal[d];
        }
        ctx->open.out[k].R = outlets[k].radius;
    }
    for (int d = 0; d < 3; ++d) {
        if (!(box_hi[d] >= box_lo[d])) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "box_hi must be >= box_lo");
        ctx->open.lo[d] = box_lo[d];
        ctx->open.hi[d] = box_hi[d];
    }
    ctx->open_set = true;
    return ARMANDO_OK;
}

armando_status armando_get_hsml(armando_ctx* ctx, float* hsml) {
    if (!ctx || !hsml) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    if (ctx->n == 0) return ARMANDO_OK;
    CK(cudaSetDevice(ctx->device));
    const int n = (int)ctx->n;
    cudaStream_t st = ctx->stream;
    float* dst = hsml;
    if (ctx->mem_kind == ARMANDO_MEM_HOST) dst = ctx->s_h;
    k_hsml_out<<<blocks_for(n, 256), 256, 0, st>>>(ctx->A, dst, n);
    ctx->launches += 1;
    CK(cudaGetLastError());
    if (ctx->mem_kind == ARMANDO_MEM_HOST)
        CK(cudaMemcpyAsync(hsml, ctx->s_h, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return ARMANDO_OK;
}

armando_status armando_set_materials(armando_ctx* ctx, int32_t count, const armando_material* table) {
    if (!ctx || !table) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    if (count < 1 || count > ARMANDO_MAX_MATERIALS)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "material count must be 1..ARMANDO_MAX_MATERIALS");
    for (int k = 0; k < count; ++k) {
        if (table[k].eos < 0 || table[k].eos > 5)
            return fail(ctx, ARMANDO_ERR_INVALID_ARG, "material eos must be 0-5");
        for (float q : table[k].prop)
            if (!std::isfinite(q) && !(table[k].eos == 5 && std::isinf(q)))
                return fail(ctx, ARMANDO_ERR_INVALID_ARG, "material properties must be finite");
    }
    ctx->materials.assign(table, table + count);
    free_graphs(ctx);
    return ARMANDO_OK;
}

armando_status armando_set_zones(armando_ctx* ctx, int32_t n_loads, const armando_load_zone* loads,
                                 int32_t n_fixes, const armando_fix_zone* fixes) {
    if (!ctx) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL context");
    if (ctx->prm.scheme == 0)
        return fail(ctx, ARMANDO_ERR_UNSUPPORTED, "load and fix zones belong to the GPU-C schemes (scheme 1, 2)");
    if (n_loads < 0 || n_loads > ARMANDO_MAX_ZONES || n_fixes < 0 || n_fixes > ARMANDO_MAX_ZONES)
        return fail(ctx, ARMANDO_ERR_INVALID_ARG, "zone counts must be 0..ARMANDO_MAX_ZONES");
    if ((n_loads && !loads) || (n_fixes && !fixes)) return fail(ctx, ARMANDO_ERR_INVALID_ARG, "NULL zone table");
    auto box_ok = [](const float* lo, const float* hi) {
        for (int d = 0; d < 3; ++d)
            if (std::isnan(lo[d]) || std::isnan(hi[d])) return false;
        return true;
    };
    for (int k = 0; k < n_loads; ++k) {
        const armando_load_zone& L = loads[k];
        if (!box_ok(L.lo, L.hi) || !std::isfinite(L.accel[0]) || !std::isfinite(L.accel[1]) ||
            !std::isfinite(L.accel[2]) || !std::isfinite(L.w))
            return fail(ctx, ARMANDO_ERR_INVALID_ARG, "load zone: NaN bound or non-finite accel / w");
    }
    for (int k = 0; k < n_fixes; ++k) {
        const armando_fix_zone& F = fixes[k];
        if (!box_ok(F.lo, F.hi) || !std::isfinite(F.vel[0]) || !std::isfinite(F.vel[1]) ||
            !std::isfinite(F.vel[2]) || !std::isfinite(F.tau) || F.tau < 0.f)
            return fail(ctx, ARMANDO_ERR_INVALID_ARG, "fix zone: NaN bound, non-finite velocity or tau < 0");
    }
    ctx->loads.assign(loads, loads + n_loads);
    ctx->fixes.assign(fixes, fixes + n_fixes);
    return ARMANDO_OK;
}

armando_status armando_deck_count(const char* dir, int64_t* n_real, int64_t* n_virtual) {
    if (!dir || !n_real || !n_virtual) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    std::string err;
    const long long nr = deck::count(dir, "f", err);
    if (nr < 0)
        return fail(nullptr, ARMANDO_ERR_IO, err.empty() ? std::string("cannot open ") + dir + "/f_xv.dat" : err);
    const long long nv = deck::count(dir, "v", err);
    if (nv == -2) return fail(nullptr, ARMANDO_ERR_IO, err);
    *n_real = nr;
    *n_virtual = nv < 0 ? 0 : nv;
    return ARMANDO_OK;
}

armando_status armando_deck_read(const char* dir, int32_t dim, int64_t n_real, int64_t n_virtual,
                                 float* x, float* vx, float* mass, float* rho, float* p,
                                 float* u, float* hsml, int32_t* itype) {
    if (!dir || !x || !vx || !mass || !rho || !p || !u || !hsml || !itype)
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    if ((dim != 2 && dim != 3) || n_real < 0 || n_virtual < 0)
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "dim must be 2 or 3, counts >= 0");
    const deck::Arrays a{x, vx, mass, rho, p, u, hsml, itype};
    std::string err;
    if (!deck::read_set(dir, "f", dim, 0, n_real, a, err)) return fail(nullptr, ARMANDO_ERR_IO, err);
    if (n_virtual > 0 && !deck::read_set(dir, "v", dim, n_real, n_virtual, a, err))
        return fail(nullptr, ARMANDO_ERR_IO, err);
    return ARMANDO_OK;
}

armando_status armando_deck_write(const char* dir, int32_t dim, int64_t n_real,
                                  int64_t n_virtual, const float* x, const float* vx,
                                  const float* mass, const float* rho, const float* p,
                                  const float* u, const float* hsml, const int32_t* itype) {
    if (!dir || !x || !vx || !mass || !rho || !p || !u || !hsml || !itype)
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    if ((dim != 2 && dim != 3) || n_real < 0 || n_virtual < 0)
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "dim must be 2 or 3, counts >= 0");
    const deck::Arrays a{const_cast<float*>(x), const_cast<float*>(vx), const_cast<float*>(mass),
                         const_cast<float*>(rho), const_cast<float*>(p), const_cast<float*>(u),
                         const_cast<float*>(hsml), const_cast<int32_t*>(itype)};
    std::string err;
    if (!deck::write_set(dir, "f", dim, 0, n_real, a, err)) return fail(nullptr, ARMANDO_ERR_IO, err);
    if (!deck::write_set(dir, "v", dim, n_real, n_virtual, a, err)) return fail(nullptr, ARMANDO_ERR_IO, err);
    return ARMANDO_OK;
}

armando_status armando_write_vtk(const char* path, int32_t dim, int64_t n, const float* x,
                                 const float* vx, const float* rho, const float* p,
                                 const float* u, const int32_t* itype) {
    if (!path || (n > 0 && (!x || !vx || !rho || !p || !u || !itype)))
        return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "NULL argument");
    if ((dim != 2 && dim != 3) || n < 0) return fail(nullptr, ARMANDO_ERR_INVALID_ARG, "dim must be 2 or 3, n >= 0");
    std::string err;
    if (!deck::write_vtk(path, dim, n, x, vx, rho, p, u, itype, err)) return fail(nullptr, ARMANDO_ERR_IO, err);
    return ARMANDO_OK;
}

armando_status armando_destroy(armando_ctx* ctx) {
    if (!ctx) return ARMANDO_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_graphs(ctx);
    for (void* p : ctx->owned) cudaFree(p);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->h_grid) cudaFreeHost(ctx->h_grid);
    if (ctx->h_wgrid) cudaFreeHost(ctx->h_wgrid);
    if (ctx->h_ng) cudaFreeHost(ctx->h_ng);
    if (ctx->h_open_n) cudaFreeHost(ctx->h_open_n);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    for (cudaEvent_t ev : ctx->ev_ovl)
        if (ev) cudaEventDestroy(ev);
    delete ctx;
    return ARMANDO_OK;
}

}  // extern "C"
