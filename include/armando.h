/*
 * armando.h -- C ABI of the GB300 (sm_103a) weakly-compressible SPH step.
 *
 * This is the drop-in boundary for Armando's leapfrog step. One call of
 * armando_step() performs one iteration of the `do its = 1, steps` loop of
 * CERNsource/time_integration.f:131-235 (predictor, neighbour search,
 * single_step, corrector); armando_integrate() performs `steps` of them, which
 * is time_integration.f:1-247 without its file output.
 *
 * Particle arrays follow the reference's Fortran layout `x(dim, maxn)`:
 * particle-major, x[i*dim + d], 0-based here. Particles with itype > 0 are
 * fluid (the reference's 1..np); particles with itype <= 0 are fixed wall
 * ("virtual") particles (np+1..np+nv): they are neighbours of fluid particles
 * but are never integrated and keep their rho, p, u and prescribed velocity
 * (CERNsource/density.f:58-59, time_integration.f:137,188).
 *
 * All arithmetic is FP32. Every entry point returns an armando_status; no
 * entry point exits the process (the reference prints and `stop`s,
 * CERNsource/link_list.f:160-173).
 */
#ifndef ARMANDO_H
#define ARMANDO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ARMANDO_ABI_VERSION 2

typedef enum armando_status {
    ARMANDO_OK = 0,
    ARMANDO_ERR_INVALID_ARG = 1,   /* bad pointer, size, dim or parameter          */
    ARMANDO_ERR_OOM = 2,           /* device or pinned-host allocation failed       */
    ARMANDO_ERR_GRID_OVERFLOW = 3, /* cell grid larger than the context's capacity  */
    ARMANDO_ERR_NONFINITE = 4,     /* NaN/Inf produced in a fluid particle's state  */
    ARMANDO_ERR_OUT_OF_GRID = 5,   /* a particle left the periodic / bounded grid   */
    ARMANDO_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up            */
    ARMANDO_ERR_CUDA = 7,          /* a CUDA runtime call failed                    */
    ARMANDO_ERR_NO_DEVICE = 8,     /* no sm_103 device visible                      */
    ARMANDO_ERR_UNSUPPORTED = 9,   /* option the GPU step does not implement        */
    ARMANDO_ERR_IO = 10            /* a deck or output file failed to open, parse or
                                      write (armando_deck_*, armando_write_vtk)      */
} armando_status;

typedef enum armando_mem_kind {
    ARMANDO_MEM_HOST = 0,   /* caller arrays are host memory; the library stages them */
    ARMANDO_MEM_DEVICE = 1  /* caller arrays are device memory on the context's GPU   */
} armando_mem_kind;

/*
 * Physics parameters. They replace the reference's compile-time and hard-coded
 * constants (art_visc.f:38-44, art_heat.f:38-40, the `prop` material table of
 * single_step.f:120-186 for the Tait family of FORTRANsource/eos.f90:255-283).
 * The struct is plain data; armando_params_default() fills the reference
 * defaults.
 */
typedef struct armando_params {
    int32_t dim;              /* 2 or 3                                                     */
    int32_t pa_sph;           /* int_force form: 0 = -(p_i+p_j)/(rho_i rho_j),
                                 1 = -(p_i/rho_i^2 + p_j/rho_j^2)  (internal_force.f:178-429) */
    int32_t visc;             /* physical viscosity via the shear tensor T_ab (int_force)   */
    int32_t visc_artificial;  /* Monaghan artificial viscosity (art_visc.f)                 */
    int32_t heat_artificial;  /* Noh artificial heat conduction (art_heat.f)                */
    int32_t heat_external;    /* analytic Gaussian volumetric heat source, du += q(x)/rho  */
    int32_t kernel_3d_legacy; /* 1: 3D Wendland normalised 15/(16 pi h^3) as in
                                 ArmandoThrust/armando.cu:150; 0: 21/(16 pi h^3)            */
    int32_t periodic[3];      /* per-axis periodic wrap (minimum image), 0/1                */
    float rho0;               /* reference density                                          */
    float c0;                 /* Tait sound speed; c = c0 for every particle                */
    float pmin;               /* p < pmin -> p = 0 and rho = rho0 (eos.f90:277-280);
                                 -INFINITY disables the clamp                               */
    float eta;                /* dynamic viscosity of the shear-tensor term                 */
    float av_alpha, av_beta, av_eta;  /* art_visc alpha, beta, eta (ref: 1, 1, 0.1)         */
    float ah_g1, ah_g2, ah_eta;       /* art_heat g1, g2, eta (ref: 0.1, 1, 0.1)            */
    float gravity[3];         /* body acceleration of fluid particles                       */
    float heat_q0;            /* peak volumetric source, W/m^3                              */
    float heat_sigma;         /* Gaussian width, m                                          */
    float heat_center[3];     /* Gaussian centre, m                                         */
    float heat_t_end;         /* source active while its*dt <= heat_t_end (fluka_heat gate) */
    float period_lo[3];       /* periodic box lower bound per axis                          */
    float period_hi[3];       /* periodic box upper bound per axis                          */
    int32_t wall_model;       /* how particles of different itype interact:
                                 0 = CERN virtual particles: like any pair (density.f,
                                     internal_force.f);
                                 1 = GPU-C device kernel (ArmandoThrust/armando.cu:472-513):
                                     no density, pressure or viscosity between them; i is
                                     pushed from j by 0.5 W m_j/(rho_j h_j) c_j^2;
                                 2 = GPU-C host path (ArmandoThrust/acpu.c:390-429): like
                                     any pair, plus a push 0.02 (W/W(0)) c_i c_j
                                     m_j/((m_i + m_j) r). Pushes act along (x_i - x_j)/r on
                                     momentum only; c = c0; W at h = (h_i + h_j)/2;
                                 3 = CERN virtual particles plus mirror ghosts
                                     (CERNsource/ghost.f, single_step.f:188-196): every
                                     iteration, each fluid particle with a wall particle
                                     in reach is mirrored across the nearest one's plane;
                                     a wall particle's vx holds its inward unit normal
                                     (and, as in the Fortran, enters the pair sums as its
                                     velocity). Needs a context created with wall_model 3,
                                     no periodic axis, no sort skin; not in batches or
                                     the reverse mode.                                    */
    int32_t scheme;           /* the step's scheme:
                                 0 = CERN-F77 leapfrog with summation density (the
                                     default; CERNsource/time_integration.f:131-218);
                                 1 = GPU-C third-order TVD Runge-Kutta with continuity
                                     density and the host path's pair physics
                                     (ArmandoThrust/acpu.c:346-437, 873-966, 2293-2379);
                                 2 = the same with the device kernels' pair physics
                                     (ArmandoThrust/armando.cu:429-513, 987-1074).
                                 Schemes 1 and 2: one armando_step is one RK3 step (3
                                 rate evaluations, the neighbour list of its start);
                                 density evolves, EOS per material (|itype| indexes
                                 the table of armando_set_materials), shock
                                 corrections instead of art_visc/art_heat, h_i
                                 kernels, gravity on itype > 0; pa_sph, visc,
                                 visc_artificial, heat_*, pmin and wall_model do not
                                 apply (wall_model must be 0). No periodic axis,
                                 batch or reverse mode. A sort skin keeps the cells
                                 of the last sort as for scheme 0 (the candidate
                                 test against the step's start positions is exact
                                 in them); armando_integrate_open sorts every step. */
    /* Options of the CERN scheme's single_step (zero: the summation-density step
       above; CERNsource/single_step.f:106-116, 214-228):                         */
    int32_t density_form;     /* 0 summation (sum_density, density.f:1-62; the
                                 Fortran's density_method 1), 1 continuity
                                 (con_density, density.f:161-218, integrated with
                                 the leapfrog, time_integration.f:144-147, 191-197;
                                 density_method 0), 2 normalised summation
                                 (nor_density, density.f:65-158; density_method 2) */
    int32_t average_velocity; /* 1: XSPH velocity correction of av_vel.f (eps 0.3),
                                 added in the corrector from the second step on     */
    int32_t sle;              /* smoothing-length evolution (h_upgrade, hsml.f):
                                 0 fixed, 1 h = 2 (m/rho)^(1/dim), 2 dh/dt =
                                 (h/dim) div v; fluid particles, after the rates;
                                 armando_get_hsml reads the evolved h back        */
} armando_params;

/* EOS of one material of the GPU-C schemes (hMatType / hMatProp of
 * ArmandoThrust/acpu.c; ESS of Code/armando.cu:572-598 on absolute density):
 *   0 boundary  prop {rho0, c0}: rho >= 0.9 rho0, p = 0, c = c0, velocity kept
 *   1 ideal gas {-, gamma, pshift}: p = (gamma - 1) rho u + pshift,
 *               c = sqrt(gamma (gamma - 1) u)
 *   2 Mie-Gruneisen polynomial {rho0, a1, a2, a3, b0, b1, t1, t2}
 *   3 Mie-Gruneisen shock {rho0, c0, g0, s0}
 *   4 Tait {rho0, c0}: p = rho0 c0^2/7 ((rho/rho0)^7 - 1), c = c0
 *   5 ESS {rho0, c0, g0, pmin}: p = max(pmin, (rho/rho0 - 1) rho0 c0^2 + g0 rho0 u)
 * (2 and 3 clamp rho >= 0.9 rho0 as 0 and 4 do.) */
typedef struct armando_material {
    int32_t eos;
    float prop[10];
} armando_material;

#define ARMANDO_MAX_MATERIALS 64

/* Per-step statistics of the last completed call. */
typedef struct armando_stats {
    int64_t steps_done;       /* leapfrog steps executed by the context so far   */
    int64_t n_particles;      /* fluid + wall particles                          */
    int64_t n_cells;          /* cells of the last neighbour grid                */
    int64_t cell_capacity;    /* cells the context can hold                      */
    int64_t gpu_launches;     /* kernels launched by the context so far          */
    int32_t grid_dims[3];     /* cells per axis of the last grid                 */
    float grid_origin[3];     /* grid origin (link_list.f:53-57: bbox min - max h) */
    float grid_cell_size[3];  /* cell edge per axis (2 * max h when not periodic) */
    uint32_t device_flags;    /* raw device status word of the last check        */
    int64_t sorts_done;       /* iterations that rebuilt the grid and sorted (all
                                 of them unless the tuning has a sort skin)       */
    int64_t ghosts;           /* mirror ghosts of the last iteration (wall_model 3) */
} armando_stats;

typedef struct armando_ctx armando_ctx;

/* Fills *p with the reference defaults: dim 2, pa_sph 1, art_visc constants
 * 1/1/0.1, art_heat 0.1/1/0.1, rho0 1000, no clamp, no gravity. */
void armando_params_default(armando_params* p);

/*
 * Creates a context for n_fluid + n_wall particles on the current CUDA device.
 * Replaces the allocations of time_integration.f:89-95 (pair lists, rate
 * arrays); the caller keeps owning the particle arrays.
 * mem_kind selects how later calls interpret the caller's pointers.
 */
armando_status armando_create(armando_ctx** ctx, const armando_params* params,
                              int32_t dim, int64_t n_fluid, int64_t n_wall,
                              int32_t mem_kind);

/*
 * Batched form: n_instances independent particle systems (a parameter sweep)
 * in one context. The reference runs one domain per process (globals hRun,
 * dMatProp in ArmandoThrust/armando.cu:117-134); here instance k has its own
 * params[k], cell grid and time step, and all instances advance together in
 * the same kernels (persistent passes over per-instance work items). Particle
 * arrays are packed: instance k occupies particles [o_k, o_k + n_fluid[k] +
 * n_wall[k]), o_k the sum of the earlier instances' counts. All instances share
 * dim.
 */
armando_status armando_batch_create(armando_ctx** ctx, int32_t n_instances,
                                    const armando_params* params, int32_t dim,
                                    const int64_t* n_fluid, const int64_t* n_wall,
                                    int32_t mem_kind);

/* Replaces the context's parameters (same dim). Takes effect at the next call.
 * Batch contexts: ARMANDO_ERR_UNSUPPORTED. */
armando_status armando_set_params(armando_ctx* ctx, const armando_params* params);

/*
 * One leapfrog iteration `its` of CERNsource/time_integration.f:131-218.
 *   its == 1 : rates at (x, v, u); v += dt/2 dvdt; u += dt/2 dudt; x += dt v
 *   its  > 1 : predictor v_h = v + dt/2 dvdt_prev, u_h = max(0, u + dt/2 dudt_prev);
 *              rates at (x, v_h, u_h); v = v + dt dvdt; u = max(0, u + dt dudt);
 *              x += dt v
 * In: x[n*dim], vx[n*dim], mass[n], rho[n], p[n], u[n], hsml[n], itype[n], and
 * for its > 1 the previous rates dvdt[n*dim], dudt[n]. Out: x, vx, u (fluid),
 * rho, p (fluid; from summation density and the Tait EOS of this step), and the
 * new rates dvdt, dudt (zero for walls). Walls keep every input value.
 * Under summation density (density_form 0, scheme 0, no mirror ghosts) the
 * fluid particles' input rho and p are not read: the step replaces them.
 * The call is stream-ordered; with ARMANDO_MEM_HOST it returns after the
 * results are back in the caller's arrays. With page-locked (mapped) host
 * arrays and no sort skin, the copies run beside the step: the inputs other
 * than x, mass and hsml load while the sort runs, and rho and p are written
 * back while the force pass runs (a second stream of the context's).
 */
armando_status armando_step(armando_ctx* ctx, float* x, float* vx,
                            const float* mass, float* rho, float* p, float* u,
                            const float* hsml, const int32_t* itype,
                            float* dvdt, float* dudt, float dt, int32_t its);

/*
 * `steps` leapfrog iterations its0 .. its0+steps-1 (time_integration.f:131-235
 * with refresh_step = 1, i.e. a neighbour search every step). The state stays
 * on the device in cell-sorted order between iterations; the loop is replayed
 * as CUDA graphs. Same arrays and meaning as armando_step.
 */
armando_status armando_integrate(armando_ctx* ctx, float* x, float* vx,
                                 const float* mass, float* rho, float* p,
                                 float* u, const float* hsml,
                                 const int32_t* itype, float* dvdt,
                                 float* dudt, float dt, int32_t its0,
                                 int32_t steps);

/* armando_integrate on a batch context with a time step per instance, dt[k].
 * armando_integrate / armando_step on a batch use the one dt for every instance. */
armando_status armando_batch_integrate(armando_ctx* ctx, float* x, float* vx,
                                       const float* mass, float* rho, float* p,
                                       float* u, const float* hsml,
                                       const int32_t* itype, float* dvdt,
                                       float* dudt, const float* dt, int32_t its0,
                                       int32_t steps);

/* Cell id of every particle under the link_list.f grid of positions x (FP32
 * form of ArmandoThrust/acpu.c:2085-2105 / link_list.f:75-88), caller order.
 * Out: cell[n]; grid (origin, size, dims) through armando_get_stats. */
armando_status armando_cell_ids(armando_ctx* ctx, const float* x,
                                const float* hsml, int32_t* cell);

/*
 * Neighbour sets under the link_list.f pair test r^2 < (h_i + h_j)^2 (scale_k
 * = 2), as a CSR over caller particle ids: for particle i, its neighbours j != i
 * are nbr[offs[i] .. offs[i+1]), ascending. offs has n+1 entries; nbr has
 * capacity `cap`; *total receives the number of (ordered) neighbour entries.
 * Returns ARMANDO_ERR_INVALID_ARG with *total set when cap is too small.
 * Host memory only (test/diagnostic entry, the step itself never builds lists).
 */
armando_status armando_neighbours(armando_ctx* ctx, const float* x,
                                  const float* hsml, int64_t* offs,
                                  int32_t* nbr, int64_t cap, int64_t* total);

/* Gradients of a loss with respect to the parameters of the step. */
typedef struct armando_param_grads {
    double av_alpha;  /* art_visc alpha */
    double av_beta;   /* art_visc beta  */
    double c0;        /* Tait / art_visc sound speed */
    double heat_q0;   /* external heat source amplitude */
} armando_param_grads;

/*
 * Reverse mode, step 1: armando_integrate over `steps` iterations its0.., also
 * keeping the state before every checkpoint_every-th iteration on the device
 * for armando_backward. Outputs the final state like armando_integrate.
 * Supports pa_sph = 1 with artificial viscosity, artificial heat, physical
 * viscosity and the external heat source, wall_model 0, summation density
 * (ARMANDO_ERR_UNSUPPORTED otherwise: XSPH, h evolution, continuity or
 * normalised density, the wall models, the GPU-C schemes); one particle
 * system (no batch).
 */
armando_status armando_forward_checkpointed(armando_ctx* ctx, float* x, float* vx,
                                           const float* mass, float* rho, float* p, float* u,
                                           const float* hsml, const int32_t* itype,
                                           float* dvdt, float* dudt, float dt, int32_t its0,
                                           int32_t steps, int32_t checkpoint_every);

/*
 * Reverse mode, step 2: the hand-written adjoint of the leapfrog steps of the
 * last armando_forward_checkpointed, by recomputation from the checkpoints in
 * reverse. In (caller order, NULL = zero): cotangents of the final x, vx, u, of
 * the pressure p returned by the last iteration, and of the final dvdt, dudt.
 * Out (caller order, NULL = not wanted): cotangents of the initial x, vx, u,
 * dvdt, dudt, and in *grads those of alpha, beta, c0, q0. The neighbour
 * topology of each iteration is that iteration's (frozen within it).
 */
armando_status armando_backward(armando_ctx* ctx, const float* x_bar, const float* v_bar,
                                const float* u_bar, const float* p_bar,
                                const float* dvdt_bar, const float* dudt_bar,
                                float* x0_bar, float* v0_bar, float* u0_bar,
                                float* dvdt0_bar, float* dudt0_bar,
                                armando_param_grads* grads);

/* The CUDA stream (cudaStream_t) every call of the context is ordered on, so
 * a caller can bracket calls with its own CUDA events. */
armando_status armando_get_stream(armando_ctx* ctx, void** stream);

/* Phases of one step, in launch order, for armando_profile_phases. */
#define ARMANDO_N_PHASES 6
/* 0 grid (bbox + cell hash), 1 radix sort, 2 cell table + reorder/predictor,
 * 3 density + EOS, 4 shear tensor (physical viscosity only), 5 forces +
 * corrector. */

/*
 * Runs `steps` further leapfrog iterations on the state the last
 * armando_integrate / armando_step left on the device (same dt, its
 * continuing), launching the kernels directly with CUDA events between the
 * phases, and returns the mean device time per step of each phase in
 * ms_per_phase[ARMANDO_N_PHASES]. The per-kernel split of the step that the
 * reference reports for its GPU code (ArmandoOnGPU.pdf p.6 Tab.2), measured.
 */
armando_status armando_profile_phases(armando_ctx* ctx, int32_t steps, float* ms_per_phase);

/*
 * Tuning of the neighbour passes. No reference counterpart: the reference
 * fixes its cell at scale_k * max(h) = 2 max(h) (CERNsource/link_list.f:29-35)
 * and gives each particle one thread (ArmandoThrust/armando.cu:2886-2926).
 *   reach                the cells of the neighbour grid are 2 max(h) / reach
 *                        wide and a particle's candidates are the
 *                        (2 reach + 1)^dim cells around its own; 1 is
 *                        link_list's grid. 1, 2 or 3.
 *   threads_per_particle lanes that share one particle's candidates and
 *                        reduce its sums: 1, 2 or 4 (batches: 1).
 *   block                threads per CTA of the pair passes, i.e. the tile of
 *                        consecutive cell-ordered particles whose candidate
 *                        lists one CTA stages in shared memory: 128 or 256.
 *   skin                 sort skin in percent of max(h), 0-100: the cells grow
 *                        by skin and armando_integrate rebuilds the grid and
 *                        sorts only on iterations where some particle has
 *                        moved more than half the skin since the last sort
 *                        (0: every iteration; one-particle-system contexts
 *                        only; armando_step, which takes fresh arrays, and
 *                        the reverse mode always sort).
 * The neighbour sets do not depend on the tuning; the sums differ only by
 * their rounding (summation order). armando_cell_ids always uses reach 1.
 */
typedef struct armando_tuning {
    int32_t reach;
    int32_t threads_per_particle;
    int32_t block;
    int32_t skin;
} armando_tuning;

armando_status armando_get_tuning(armando_ctx* ctx, armando_tuning* out);
/* INVALID_ARG for a value outside the lists above; UNSUPPORTED for
 * threads_per_particle > 1 or skin > 0 on a batch context. */
armando_status armando_set_tuning(armando_ctx* ctx, const armando_tuning* t);

/* The autotuner's candidate tunings, k = 0 .. ARMANDO_N_TUNINGS - 1: k < 18
 * every (reach, threads_per_particle, block) with skin 0; k >= 18 a skin
 * (10, 20, 40 percent) applied to the fastest of the first 18 with the same
 * reach, returned here with threads_per_particle = block = 0. */
#define ARMANDO_N_TUNINGS 27
armando_status armando_tuning_candidate(int32_t k, armando_tuning* out);

/*
 * Autotuner: for every candidate tuning, loads the given state (caller
 * arrays in the context's memory kind, as for armando_step; none is
 * modified), runs one untimed iteration its0 and then times steps_per_trial
 * iterations its0 + 1 .. with CUDA events. Sets the fastest tuning on the
 * context and writes it to *best (may be NULL); ms_per_step (may be NULL,
 * else ARMANDO_N_TUNINGS floats) receives each candidate's mean time per
 * iteration, or a negative value for a candidate that does not apply (e.g.
 * a periodic box too short for its reach). One particle system only.
 */
armando_status armando_autotune(armando_ctx* ctx, const float* x, const float* vx,
                                const float* mass, const float* rho, const float* p,
                                const float* u, const float* hsml, const int32_t* itype,
                                const float* dvdt, const float* dudt, float dt, int32_t its0,
                                int32_t steps_per_trial, armando_tuning* best,
                                float* ms_per_step);

/*
 * Autotuner of a batch (armando_batch_create): as armando_autotune, on the
 * packed state of every instance with one time step per instance (dt[k], as
 * for armando_batch_integrate). The batched passes run one thread per
 * particle in CTAs of ARMANDO_BATCH_BLOCK threads and sort every iteration,
 * so the candidates with threads_per_particle 1, that block and skin 0 are
 * timed (they differ in reach, the cell size 2 max h / reach of every
 * instance's grid); the others receive -1 in ms_per_step. On a single-system
 * context this is armando_autotune with dt[0]. The fastest tuning is set.
 */
#define ARMANDO_BATCH_BLOCK 128
armando_status armando_batch_autotune(armando_ctx* ctx, const float* x, const float* vx,
                                      const float* mass, const float* rho, const float* p,
                                      const float* u, const float* hsml, const int32_t* itype,
                                      const float* dvdt, const float* dudt, const float* dt,
                                      int32_t its0, int32_t steps_per_trial, armando_tuning* best,
                                      float* ms_per_step);

/*
 * Allocation-free form of armando_cell_ids. It has no counterpart in the
 * reference.
 * For callers that must not allocate device memory: a host code that hands
 * the GPU's memory to its own pool at start-up and treats any later cudaMalloc
 * as an error, or a time loop that cannot afford the device-wide
 * synchronisation a cudaMalloc/cudaFree implies. It needs no context. x[n*dim]
 * and hsml[n] are device arrays (read), cell[n] a device array (written), all
 * on the current device; stream is a cudaStream_t (NULL: legacy default stream).
 * Its scratch (grid reduction partials, grid record, status word) is a fixed
 * 32 KiB static device array, which every GPU that loads the library holds
 * until the process exits. n is limited to 2^30 and the grid to 2^30 cells;
 * larger sizes return ARMANDO_ERR_INVALID_ARG / ARMANDO_ERR_GRID_OVERFLOW. The
 * first call on a device looks up the array's device address once
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. All calls share the one array: calls that overlap
 * on the GPU (other streams, other host threads) race on it. The call returns
 * after the stream has finished the work; the last error is readable with
 * armando_last_error(NULL).
 */
armando_status armando_cell_ids_noalloc(const armando_params* params, const float* x,
                                        const float* hsml, int64_t n, int32_t* cell,
                                        void* stream);

/* Material table of the GPU-C schemes (armando_params.scheme 1, 2), entry k for
 * the particles with |itype| = k; count <= ARMANDO_MAX_MATERIALS. Until it is set,
 * every entry is Tait with the context's rho0 and c0. */
armando_status armando_set_materials(armando_ctx* ctx, int32_t count, const armando_material* table);

/* ---- open boundaries of the GPU-C schemes (scheme 1, 2) ---------------------------
 * Inlets and outlets of ArmandoThrust/armando.cu:2640-2856. Every step, before its
 * neighbour list:
 *   inlets: distance += speed dt; past hsml/1.2 (the lattice spacing) it drops by
 *     that much and the inlet emits a lattice of new particles in its plane (a
 *     disk of radius `radius` in 3D, a segment across the normal in 2D), spacing
 *     hsml/1.2, velocity speed along the normal, with the inlet's itype, mass,
 *     hsml, rho and u;
 *   outlets: a particle behind an outlet's plane ((x - origin) . normal < 0) within
 *     `radius` of its axis leaves, and so does any particle outside [box_lo, box_hi].
 * The particle count then varies up to the context's capacity (n_fluid + n_wall at
 * creation); armando_integrate_open takes and returns it. Particles keep their
 * order: the survivors of the input come first, in input order, then the new ones
 * in emission order (inlets in table order, lattice rows in order). */
typedef struct armando_inlet {
    float origin[3], normal[3], radius;
    int32_t itype;       /* 0: inlet off                                   */
    float mass, hsml, speed, rho, u;
} armando_inlet;

typedef struct armando_outlet {
    float origin[3], normal[3], radius;
} armando_outlet;

#define ARMANDO_MAX_OPEN 10

/* Sets the open boundaries (at most ARMANDO_MAX_OPEN of each; resets the
 * inlets' distances) and the box outside which particles leave. */
armando_status armando_set_open_boundaries(armando_ctx* ctx, int32_t n_inlets,
                                           const armando_inlet* inlets, int32_t n_outlets,
                                           const armando_outlet* outlets, const float box_lo[3],
                                           const float box_hi[3]);
/* `steps` GPU-C steps with the open boundaries on *n_particles particles (in/out);
 * every array holds room for the context's capacity. */
armando_status armando_integrate_open(armando_ctx* ctx, float* x, float* vx, float* mass,
                                      float* rho, float* p, float* u, float* hsml,
                                      int32_t* itype, float* dvdt, float* dudt, float dt,
                                      int32_t its0, int32_t steps, int64_t* n_particles);

/* ---- load and fix zones of the GPU-C schemes (scheme 1, 2) ------------------------
 * The GPU-C codes' `struct load` and `struct fix` tables (ArmandoThrust/acpu.c:33-48,
 * hLoad / hFix; armando.cu:43-58). A zone is the open box lo < x < hi (every bound
 * strict; in 2D x and y only, as armando2D.cu:756-762 tests them):
 *   load: every rate evaluation, a particle with itype > 0 inside the box gains
 *     accel on dv/dt and w on de/dt (updateLoadsHost, acpu.c:1047-1076), zones in
 *     table order after params.gravity (the reference's load 0 over the whole box);
 *   fix: after every stage's update, a particle inside the box at its new position
 *     takes the velocity vel (acpu.c:916-926, armando.cu:1026-1036; the last
 *     matching zone wins); scheme 1 applies it to itype != 0 after resetting the
 *     velocity of itype <= 0, scheme 2 to every particle; boundary-type materials
 *     then keep their start velocity in both;
 *   pump (a fix zone with tau > 0, the pump / relaxation zones of
 *     Code/armando.cu:1046-1055): every rate evaluation, a particle with
 *     itype > 0 inside the box at the stage's position gains (vel - v) / tau on
 *     dv/dt, v its stage velocity; pump zones in table order after the loads.
 * Bounds may be infinite; the other fields must be finite, tau >= 0. */
typedef struct armando_load_zone {
    float lo[3], hi[3];
    float accel[3];
    float w;
} armando_load_zone;

typedef struct armando_fix_zone {
    float lo[3], hi[3];
    float vel[3];
    float tau;  /* 0: fix zone; > 0: pump zone relaxing to vel over time tau */
} armando_fix_zone;

#define ARMANDO_MAX_ZONES 10

/* Sets the zones (at most ARMANDO_MAX_ZONES of each; zero counts clear them).
 * ARMANDO_ERR_UNSUPPORTED for the CERN scheme (params.scheme 0). */
armando_status armando_set_zones(armando_ctx* ctx, int32_t n_loads, const armando_load_zone* loads,
                                 int32_t n_fixes, const armando_fix_zone* fixes);

/* Smoothing lengths of the context's particles after its last step or
 * integrate call, in caller order (evolved when params.sle != 0; otherwise the
 * ones passed in). With density_form 1 the context also keeps drho/dt between
 * calls, as time_integration.f keeps it between its iterations. */
armando_status armando_get_hsml(armando_ctx* ctx, float* hsml);

/* Calls are stream-ordered on the context's stream. With ARMANDO_MEM_DEVICE,
 * armando_step / armando_integrate / armando_batch_integrate return as soon as
 * their work is enqueued (the first call on a context, and calls with mirror
 * ghosts or open boundaries, read device counts back and block); the device
 * status of those calls (non-finite state, grid overflow, a particle out of
 * the periodic box) is sticky until armando_sync reports it, and
 * armando_get_stats is current after armando_sync. With ARMANDO_MEM_HOST a
 * call returns once its outputs are in the caller's arrays. The context's own
 * stream is created blocking, so it is ordered both ways with work on the
 * legacy default stream (where PyTorch's default stream puts its kernels).
 * Replaces the Fortran's synchronous calls (CERNsource/time_integration.f:1-8),
 * which have no notion of a stream. */

/* Blocks until the context's stream is idle and returns the status of the
 * asynchronous calls since the last report. */
armando_status armando_sync(armando_ctx* ctx);
/* Launch the context's work on the caller's stream (a cudaStream_t of the
 * context's device; NULL: the context's own stream). Work already enqueued on
 * the previous stream is ordered before later calls. Graphs are captured on a
 * private stream, so any stream may be passed. No counterpart in the
 * reference (its GPU code uses the default stream, ArmandoThrust/armando.cu). */
armando_status armando_set_stream(armando_ctx* ctx, void* stream);
armando_status armando_get_stats(const armando_ctx* ctx, armando_stats* out);
/* Last error message of the context (static string when ctx is NULL). */
const char* armando_last_error(const armando_ctx* ctx);
armando_status armando_destroy(armando_ctx* ctx);
int32_t armando_abi_version(void);
/* cudaFuncAttributes::binaryVersion of the library's device code on the
 * current device (103: built for sm_103a). No counterpart in the reference. */
armando_status armando_binary_version(int32_t* version);

/* ---- particle decks and snapshots (host only; no context, no GPU) --------------
 * Decks of the CERN-F77 code, in directory dir: real particles in f_xv.dat,
 * f_state.dat, f_other.dat (read by CERNsource/input.f:197-255, written by
 * output.f:31-54), virtual (wall) particles in v_xv.dat, v_state.dat,
 * v_other.dat (input.f:256-314, output.f:56-73). Arrays hold the n_real real
 * particles first, then the n_virtual virtual ones, in the step's layout
 * (x[i*dim + d]); itype is the deck's material number (<= 0: wall). Reading
 * is list-directed like the Fortran's; writing reproduces its formats
 * (1x,I6,6(2x,e14.8)), (1x,I6,7(2x,e14.8)), (1x,I6,2x,I4,2x,e14.8). A deck
 * without v_ files has n_virtual = 0. Errors: ARMANDO_ERR_IO (message in
 * armando_last_error(NULL)). */
armando_status armando_deck_count(const char* dir, int64_t* n_real, int64_t* n_virtual);
armando_status armando_deck_read(const char* dir, int32_t dim, int64_t n_real, int64_t n_virtual,
                                 float* x, float* vx, float* mass, float* rho, float* p,
                                 float* u, float* hsml, int32_t* itype);
armando_status armando_deck_write(const char* dir, int32_t dim, int64_t n_real,
                                  int64_t n_virtual, const float* x, const float* vx,
                                  const float* mass, const float* rho, const float* p,
                                  const float* u, const float* hsml, const int32_t* itype);
/* Legacy ASCII VTK snapshot of n particles in the format of the GPU-C code's
 * outputVTK (ArmandoThrust/armando.cu:1596-1670): points (z = 0 in 2D), one
 * vertex cell each, material, density, pressure, energy, velocity. */
armando_status armando_write_vtk(const char* path, int32_t dim, int64_t n, const float* x,
                                 const float* vx, const float* rho, const float* p,
                                 const float* u, const int32_t* itype);

#ifdef __cplusplus
}
#endif

#endif /* ARMANDO_H */
