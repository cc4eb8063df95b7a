/*
 * ppf.h -- C ABI of the GB300 explicit phase-field step.
 *
 * The reference program (jijn/phasefield_coarsening, one C file) has no
 * library interface: its hot path is the pair of functions
 *
 *   sweep_fields   phasefield.c:301-403   full step of etaS, etaL and c
 *   sweep_fields_c phasefield.c:406-476   c-only step (eta frozen)
 *
 * called from the time loop in main (phasefield.c:178-258) after the ghost
 * layers have been filled by apply_periodic_boundary_condition
 * (:1112-1148), apply_nonflux_boundary_condition (:1151-1189) or the MPI
 * halo exchange (:683-708, :762-826).  The state lives in ten global
 * arrays double[NI+2][NJ+2][NK+2] (:67-70) indexed [z][y][x].
 *
 * This header is the drop-in boundary for that path: an opaque context owns
 * the device copy of the state (3 fields, two ping-pong buffers, one ghost
 * layer per face); the caller owns host arrays that hold only the interior,
 * nz*ny*nx values in C order [z][y][x] -- the same order as the /etaS,
 * /etaL and /c HDF5 datasets the reference reads (:996-1049).
 *
 * Conventions:
 *   - every function returns 0 on success or a negative PPF_E* code;
 *     ppf_last_error() returns a message for the calling thread's last
 *     failure;
 *   - ppf_step / ppf_step_c_only queue work on the context's stream and
 *     return; ppf_upload*, ppf_download*, ppf_reduce and ppf_sync wait for
 *     it (errors of queued work surface there); one context must not be
 *     used from two threads at once; contexts are independent;
 *   - nothing here falls back to the CPU: without a usable CUDA device
 *     ppf_create fails with PPF_ECUDA.
 */
#ifndef PPF_H
#define PPF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes */
#define PPF_OK        0
#define PPF_EINVAL   (-1)   /* bad argument */
#define PPF_ECUDA    (-2)   /* CUDA runtime/driver error, or no device */
#define PPF_ENOMEM   (-3)   /* device or host allocation failed */
#define PPF_ESTATE   (-4)   /* call not valid in the context's state */
#define PPF_EIO      (-5)   /* file I/O (HDF5 subset) failed */
#define PPF_ETIMEOUT (-6)   /* a bounded device wait ran out */

/* boundary conditions: the values of USE_BC_TYPE, phasefield.c:15-16 */
#define PPF_BC_PERIODIC 0   /* ghost = opposite face, :1112-1148 */
#define PPF_BC_NOFLUX   1   /* ghost = adjacent interior cell, :1151-1189 */

/* storage + arithmetic precision of the step */
#define PPF_F64 0           /* the reference's double, phasefield.c:67-70 */
#define PPF_F32 1           /* float storage and arithmetic */

/* Material and numerical constants, phasefield.c:76-97.  Derived values
 * (ML, MS, h2, m, kappa, L) are computed from these exactly as the
 * reference does; see ppf_params_derive. */
typedef struct ppf_params {
    double AS, AL;      /* parabola curvatures, :76-77 */
    double CS, CL;      /* parabola offsets, :78-79 */
    double cS0, cL0;    /* parabola minima, :80-81 */
    double cSeq, cLeq;  /* compositions used by the mobility L, :82-83 */
    double DL, DS;      /* diffusivities, :84 */
    double sigma;       /* interface energy, :87 */
    double gamma;       /* Moelans gamma, :88 */
    double dx;          /* grid spacing, :90 */
    double dt;          /* time step, :92; <= 0 selects 0.125*dx*dx/DL */
    double l;           /* interface width, :94; <= 0 selects 7*dx */
} ppf_params;

typedef struct ppf_derived {
    double ML, MS;      /* DL/AL, DS/AS, :85 */
    double h2;          /* 1/dx^2, :91 */
    double dt;          /* effective time step */
    double l;           /* effective interface width */
    double m;           /* 6 sigma / l, :95 */
    double kappa;       /* 3/4 sigma l, :96 */
    double L;           /* 4/3 m/kappa (MS+ML)/2 / (cSeq-cLeq)^2, :97 */
    double dt_limit;    /* explicit limit of the solute equation, dx^2/(6 max(DL,DS)) */
} ppf_derived;

/* Reductions.  The first three are the reference's convergence sums over
 * the interior (phasefield.c:228-238), taken over the increments of the
 * most recent step; the rest are observables of the current state, all
 * accumulated in double on the device. */
typedef struct ppf_stats {
    double sum_dc2;       /* sum dc^2 of the last step ("c=" in :240) */
    double sum_detaS2;    /* sum detaS^2 ("S=") */
    double sum_detaL2;    /* sum detaL^2 ("L=") */
    double mass;          /* sum c (total solute, cell volume dx^3 not applied) */
    double solid;         /* sum hS, the solid phase fraction times cells */
    double solid_cells;   /* number of cells with etaS > 0.5 */
    double free_energy;   /* sum of the free-energy density times dx^3 */
    int64_t cells;        /* nz*ny*nx */
    int64_t nonfinite;    /* cells holding a NaN/Inf in any field */
    int64_t steps;        /* steps taken by this context since ppf_upload */
} ppf_stats;

typedef struct ppf_ctx ppf_ctx;

/* The reference's constants (phasefield.c:76-97). */
void ppf_params_default(ppf_params *p);

/* Derived constants exactly as phasefield.c:85-97 computes them. */
int ppf_params_derive(const ppf_params *p, ppf_derived *d);

/* Create a context for an nz x ny x nx interior grid on the current CUDA
 * device.  Replaces the global arrays of phasefield.c:67-70 and the
 * compile-time grid/BC macros of :13-56.  `bc` is PPF_BC_*; `precision`
 * is PPF_F64 or PPF_F32. */
int ppf_create(int nz, int ny, int nx, const ppf_params *p, int bc, int precision,
               ppf_ctx **out);
int ppf_destroy(ppf_ctx *ctx);

/* Grid and layout of a context. */
int ppf_get_dims(const ppf_ctx *ctx, int *nz, int *ny, int *nx);

/* Use the caller's CUDA stream (a cudaStream_t) for all later work;
 * NULL returns to the context's own stream. */
int ppf_set_stream(ppf_ctx *ctx, void *stream);

/* Host <-> device copies of the interior, replacing read_hdf5's fill of
 * the ghosted arrays (phasefield.c:996-1049) and the write-out of
 * write_hdf5 (:1052-1109).  Host arrays may be pageable or pinned.  The
 * ghost layers are filled on upload (the BC fill of :207-211). */
int ppf_upload(ppf_ctx *ctx, const double *etaS, const double *etaL, const double *c);
int ppf_download(ppf_ctx *ctx, double *etaS, double *etaL, double *c);

/* Same, from/to device memory (nz*ny*nx doubles each, C order). */
int ppf_upload_device(ppf_ctx *ctx, const double *etaS, const double *etaL, const double *c);
int ppf_download_device(ppf_ctx *ctx, double *etaS, double *etaL, double *c);

/* Advance `nsteps` full steps: for each, the BC fill (:207-211) followed by
 * sweep_fields (:301-403), fused into one kernel per step.  The increments
 * of the last step are reduced for ppf_reduce's sum_* fields. */
int ppf_step(ppf_ctx *ctx, int64_t nsteps);

/* Advance `nsteps` c-only steps: BC fill + sweep_fields_c (:406-476). */
int ppf_step_c_only(ppf_ctx *ctx, int64_t nsteps);

/* Reductions of the current state plus the last step's increments. */
int ppf_reduce(ppf_ctx *ctx, ppf_stats *out);

/* Wait for all work queued on the context's stream.  Returns
 * PPF_ETIMEOUT when a step's bounded device wait ran out since the last
 * check (the state of that step is then invalid: upload a new one). */
int ppf_sync(ppf_ctx *ctx);

/* Upper bound, in seconds, of every device-side wait of the step kernel
 * (default 1 s).  No counterpart in the reference. */
int ppf_set_wait_limit(ppf_ctx *ctx, double seconds);

/* Test hook, no counterpart in the reference: make the next step's kernel
 * wait on a copy that never completes, so that the wait limit runs out and
 * the failure path (error word, PPF_ETIMEOUT, usable context) can be
 * exercised without faulting the GPU. */
#define PPF_INJECT_NONE       0
#define PPF_INJECT_STALL_WAIT 1
int ppf_debug_inject(ppf_ctx *ctx, int fault);

/* Particle analysis of the current state (no counterpart in the
 * reference, which leaves it to MATLAB post-processing, README.md:26).
 * Particles are the 6-connected components of etaS > threshold, wrapping
 * across periodic faces. */
typedef struct ppf_particle_stats {
    int64_t count;           /* number of particles */
    double mean_radius;      /* R-bar: mean of (3V/4pi)^(1/3) over particles, in units of dx */
    double solid_volume;     /* solid cells x dx^3 */
    double largest_volume;   /* largest particle, cells x dx^3 */
    double interface_area;   /* solid/liquid cell faces x dx^2 */
} ppf_particle_stats;

/* `volumes` (may be NULL) receives up to `capacity` particle volumes in
 * cells, in no particular order; *nvolumes (may be NULL) the particle count.
 * Device scratch of 8 bytes per cell is allocated on the first call. */
int ppf_particles(ppf_ctx *ctx, double threshold, ppf_particle_stats *out, int64_t *volumes, int64_t capacity,
                  int64_t *nvolumes);

/* Launch choices of the fused step kernel.  No counterpart in the
 * reference (whose only tuning is the no-op cache blocking of
 * phasefield.c:58-62, :340-350). */
typedef struct ppf_tune {
    int zc;              /* z planes per work item of the persistent grid */
    int roll;            /* 1: one plane body (the default), 3: unrolled three times */
    int grid;            /* CTAs (derived from zc; ignored by ppf_set_tune) */
    int pdl;             /* 1 (the default): consecutive steps overlap by programmatic dependent
                            launch (the next step's CTAs are placed while this one's last CTAs
                            finish; every memory access still waits for the previous step);
                            0: plain launches.  With it, a step whose domain does not fill whole
                            tiles runs its edge tiles in the tail of its whole-tile launch. */
    int sched;           /* 1 (the default): CTAs take work items from a global counter, so that
                            faster CTAs take more; 0: items dealt round-robin.  Both give the
                            same bits. */
    int zc2;             /* > 0 and < zc: the top `tail` planes are cut into work items of zc2
                            planes instead of zc (short items end the step, so that its CTAs end
                            closer together); 0: every item zc planes */
    int tail;
    int split;           /* 1 (the default): a domain whose x or y edge is not a multiple of the
                            tile runs its whole tiles and its edge tiles as two launches, the
                            second in the first one's tail (with pdl); 0: one launch over every
                            tile.  Both give the same bits. */
    int tile;            /* tile shape of a work item's brick: 0 (the default) 64 x 16 cells in x, y;
                            1 (FP32 only) 32 x 32.  All give the same bits. */
    double us_per_step;  /* measured time of the winner (ppf_autotune only) */
} ppf_tune;

int ppf_get_tune(const ppf_ctx *ctx, ppf_tune *out);
int ppf_set_tune(ppf_ctx *ctx, const ppf_tune *t);

/* Time the candidate launch choices on the context's uploaded state for
 * `trial_steps` steps each, keep the fastest, and restore the state as it
 * was (the step count is unchanged).  `best` (may be NULL) receives the
 * choice and its time per step. */
int ppf_autotune(ppf_ctx *ctx, int trial_steps, ppf_tune *best);

/* Allocation-free observables.  No counterpart in the reference.
 *
 * For callers that may not allocate device memory: typically a hook that a
 * host application calls between its own steps, whose device memory belongs
 * to the application's pool or arena (a caching allocator, preallocated
 * communication buffers), where an unplanned cudaMalloc can fail on a full
 * device, fragment its memory pool, or hold up the application's streams.  The
 * caller passes its own device arrays -- etaS, etaL, c, each nz*ny*nx
 * doubles in C order [z][y][x] -- and a device array `out` of 5 doubles; the
 * call queues the reduction on `stream` (NULL: the default stream) and
 * returns.  out = {mass, solid, solid_cells, free_energy, nonfinite}, the
 * same quantities as the matching fields of ppf_reduce.  Nothing is
 * allocated: the partial sums go to a fixed device array of the library,
 * which limits a call to PPF_NOALLOC_MAX_CELLS cells (larger grids get
 * PPF_EINVAL with a message).  The first call on a device looks up that
 * array's device address (do it before any stream capture), as does the
 * first call after the device was reset.  Every call
 * shares the array: calls that overlap on the GPU race, so issue them on
 * one stream. */
#define PPF_NOALLOC_MAX_CELLS 134217728   /* 512^3 */
int ppf_observe_noalloc(int nz, int ny, int nx, const ppf_params *p, int bc, const double *etaS,
                        const double *etaL, const double *c, double *out, void *stream);

/* Ensembles: many independent domains of different sizes (same parameters,
 * BC and precision) advanced together -- one persistent launch of the
 * fused step per time step covers every domain's work items, and runs of
 * steps replay a captured CUDA graph.  No counterpart in the reference,
 * which runs one domain per program.  Each domain is an ordinary context
 * (ppf_ensemble_domain) for uploads, downloads and reductions; stepping
 * goes through the ensemble only. */
typedef struct ppf_ensemble ppf_ensemble;

/* dims: n triples (nz, ny, nx). */
int ppf_ensemble_create(int n, const int *dims, const ppf_params *p, int bc, int precision,
                        ppf_ensemble **out);
int ppf_ensemble_destroy(ppf_ensemble *ens);
int ppf_ensemble_domain(ppf_ensemble *ens, int d, ppf_ctx **ctx);
int ppf_ensemble_upload(ppf_ensemble *ens, int d, const double *etaS, const double *etaL, const double *c);
int ppf_ensemble_download(ppf_ensemble *ens, int d, double *etaS, double *etaL, double *c);
/* Every domain in one call: arrays of n host pointers per field (domain d's
 * compact [z][y][x] float64 arrays).  The copies of all domains are issued
 * first and one conversion launch covers them all, so that a caller that
 * streams ensembles through host memory while other ensembles step on the
 * same device waits for a free SM slot once per call, not once per domain.
 * Same results as n calls of ppf_ensemble_upload / ppf_ensemble_download. */
int ppf_ensemble_upload_all(ppf_ensemble *ens, const double *const *etaS, const double *const *etaL,
                            const double *const *c);
int ppf_ensemble_download_all(ppf_ensemble *ens, double *const *etaS, double *const *etaL, double *const *c);
/* nsteps full steps of every domain (all domains need an uploaded state);
 * the last step's increment sums go to each domain's ppf_reduce. */
int ppf_ensemble_step(ppf_ensemble *ens, int64_t nsteps);
int ppf_ensemble_reduce(ppf_ensemble *ens, int d, ppf_stats *out);
int ppf_ensemble_sync(ppf_ensemble *ens);
int ppf_ensemble_get_tune(const ppf_ensemble *ens, ppf_tune *out);
int ppf_ensemble_set_tune(ppf_ensemble *ens, const ppf_tune *t);
/* Like ppf_autotune, over the whole ensemble (states kept). */
int ppf_ensemble_autotune(ppf_ensemble *ens, int trial_steps, ppf_tune *best);

/* Slabs: one domain split into z slabs, one context each, with one
 * ghost-plane exchange per step -- the domain decomposition of the
 * reference's MPI build (init_mpi, phasefield.c:627-679; the halo exchange
 * exchange_ghost_layer, :683-708) along z.  After each step every slab's two
 * z ghost planes are overwritten with its neighbours' boundary planes (the
 * first and last slabs' outer planes wrap for PPF_BC_PERIODIC and keep
 * their own mirror for PPF_BC_NOFLUX), so the result equals stepping the
 * undivided domain bit for bit.  All slabs live on the current device. */
typedef struct ppf_slabs ppf_slabs;

/* The partition (no device needed): slab s holds planes [z0[s], z0[s] +
 * nzs[s]); lower[s] / upper[s] is the slab whose boundary plane fills its
 * lower / upper ghost plane, or -1 where the BC fills it.  Arrays hold
 * nslabs entries; 1 <= nslabs <= nz. */
int ppf_slabs_plan(int nz, int nslabs, int bc, int *z0, int *nzs, int *lower, int *upper);
int ppf_slabs_create(int nz, int ny, int nx, int nslabs, const ppf_params *p, int bc, int precision,
                     ppf_slabs **out);
int ppf_slabs_destroy(ppf_slabs *s);
/* Whole-domain host arrays, nz*ny*nx doubles in C order [z][y][x]. */
int ppf_slabs_upload(ppf_slabs *s, const double *etaS, const double *etaL, const double *c);
int ppf_slabs_download(ppf_slabs *s, double *etaS, double *etaL, double *c);
int ppf_slabs_step(ppf_slabs *s, int64_t nsteps);
/* Sums over the slabs of ppf_reduce's fields (steps: the slabs' count). */
int ppf_slabs_reduce(ppf_slabs *s, ppf_stats *out);
int ppf_slabs_sync(ppf_slabs *s);

/* Solute-mass projection of an FP32 state: sum(c) over the interior is set
 * to target_mass (FP64 arithmetic; the deficit is spread over the cells in
 * whole FP32 ulps, so the FP32 sum lands within about one ulp of it).  The
 * reference conserves mass in FP64 arithmetic alone (phasefield.c:374-384,
 * summed at :228-238); FP32 storage needs the projection for drift below
 * 1e-9 relative over long runs. */
int ppf_mass_project(ppf_ctx *ctx, double target_mass);

/* dst's state := src's current state (same shape, precision and BC). */
int ppf_copy_state(ppf_ctx *dst, ppf_ctx *src);

/* Learned time-stepping surrogate (no counterpart in the reference): a
 * six-layer 3x3x3 convolutional network, BF16 tensor-core implicit GEMMs
 * with FP32 accumulation, that advances an FP32 state by k_steps explicit
 * steps of sweep_fields (phasefield.c:301-403) per call:
 *   state += out_scale * net(etaS, etaL, (c - c_eq(h)) * in_scale_c)
 * followed by the FP64 mass projection back to the pre-call sum(c).
 * Trained on the device on (state, state after k_steps stencil steps)
 * pairs.  Domains: FP32 contexts whose x edge is a multiple of 128 and
 * whose y and z edges are at least 2; training on periodic domains.  A
 * surrogate keeps one workspace (for the last domain shape it ran on) and
 * is used by one host thread at a time. */
typedef struct ppf_surrogate ppf_surrogate;

typedef struct {
    int width;              /* hidden channels: 16 or 32 */
    int k_steps;            /* explicit steps one call stands for */
    double c_solid;         /* c_eq(h) = h c_solid + (1 - h) c_liquid */
    double c_liquid;
    double in_scale_c;      /* scale of the composition feature */
    double out_scale[3];    /* field change per unit of network output: etaS, etaL, c */
    double loss_weight[3];  /* per-field weights of the squared-error loss */
} ppf_surrogate_config;

void ppf_surrogate_config_default(ppf_surrogate_config *cfg);
int ppf_surrogate_create(const ppf_surrogate_config *cfg, ppf_surrogate **out);
int ppf_surrogate_destroy(ppf_surrogate *s);
int ppf_surrogate_get_config(const ppf_surrogate *s, ppf_surrogate_config *cfg);
/* Parameters: per layer W[27][c_out][c_in] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1),
 * out[v] = sum W_tap in[v + (dx,dy,dz)]) then b[c_out]; channels 16, width x5, 16. */
int64_t ppf_surrogate_num_params(const ppf_surrogate *s);
int ppf_surrogate_set_params(ppf_surrogate *s, const float *params, int64_t n);
int ppf_surrogate_get_params(ppf_surrogate *s, float *params, int64_t n);
/* Loss = sum over cells and fields of loss_weight (pred - (target - input) / out_scale)^2 / (3 cells),
 * and its gradient (grad may be NULL); no update. */
int ppf_surrogate_loss_grad(ppf_surrogate *s, ppf_ctx *input, ppf_ctx *target, double *loss, float *grad,
                            int64_t n);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on one (input, target) pair; loss may be NULL. */
int ppf_surrogate_train_step(ppf_surrogate *s, ppf_ctx *input, ppf_ctx *target, double lr, double *loss);
/* Predicted change out_scale * net(.) of etaS, etaL, c: 3 x cells doubles, [field][z][y][x]. */
int ppf_surrogate_predict(ppf_surrogate *s, ppf_ctx *ctx, double *out3);
/* ncalls surrogate calls on ctx's state (k_steps each, mass projected after each). */
int ppf_surrogate_advance(ppf_surrogate *s, ppf_ctx *ctx, int ncalls);
/* Test hook (as ppf_debug_inject): with PPF_INJECT_STALL_WAIT the next
 * convolution launch waits for an input row that never completes, its
 * bounded wait runs out (ppf_set_wait_limit of the context it runs on) and
 * the context's next synchronising call returns PPF_ETIMEOUT. */
int ppf_surrogate_debug_inject(ppf_surrogate *s, int fault);

/* Measured FP64 FMA rate of the current device in TFLOP/s (2 FLOPs per
 * FMA): the denominator of the FP64 step's roofline, which the FP64 pipe
 * bounds on this GPU.  No counterpart in the reference.  Takes ~0.1 s. */
int ppf_measure_fp64_peak(double *tflops);

/* Message for the calling thread's last failure ("" if none). */
const char *ppf_last_error(void);

/* Library version string. */
const char *ppf_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PPF_H */
