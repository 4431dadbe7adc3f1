/*
 * sphadjoint_gb300 — C ABI of the GB300 (sm_103a) forward + adjoint WCSPH step.
 *
 * A drop-in for the device path of the Julia package SPHAdjoint
 * (hanafsky/SPHAdjoint): each entry point below replaces one public function
 * or constructor of that package, cited as file:line in its source tree. The
 * Julia side binds them with `ccall` (a thin wrapper keeps the names
 * SPHParams / State / Tape / AdjointWorkspace / simulate! / backward!).
 *
 * Conventions (the reference's own):
 *   - T is Float64 (SPH_F64) or Float32 (SPH_F32), fixed per object.
 *   - Host arrays X, V, seeds, gradients: (2, N) column-major T, i.e.
 *     interleaved (x1, y1, x2, y2, ...). theta and dJ/dtheta: (ngy, ngx)
 *     column-major T.
 *   - Cell lists use 1-based particle ids in `order` and 0-based exclusive
 *     offsets in `starts`, exactly as CellList holds them.
 *   - Every call returns a status (SPH_OK = 0); on failure sph_last_error()
 *     gives the message. No exception crosses the ABI. There is no CPU
 *     fallback: without a CUDA device every device call fails loudly.
 *   - One library stream; a handle is used by one host thread at a time.
 */
#ifndef SPHADJOINT_GB300_H
#define SPHADJOINT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_API __attribute__((visibility("default")))

/* SPHParams{T} (src/params.jl:14-28). gx/gy default to 0 / -9.81 there.
   The trailing fields select model variants that have no counterpart in the
   reference (which has the linear EOS and Morris viscosity, README.md:505-519);
   all zero = the reference's model:
     eos   0 linear p = c^2 (rho - rho0); 1 Tait p = B ((rho/rho0)^gamma - 1),
           B = c^2 rho0 / gamma, integer gamma in [1, 15] (the bracket evaluated
           as s_{k+1} = s_k (1 + d) + d, s_1 = d = (rho - rho0)/rho0)
     visc  0 Morris (mu); 1 Monaghan artificial viscosity, a_i += K d with
           K = m alpha c h s F / ((r^2 + 0.01 h^2) (rho_i + rho_j) / 2) on
           approaching pairs (s = (v_i - v_j).d < 0), alpha >= 0 */
typedef struct sph_params {
    double h, m, rho0, c, mu, gx, gy, dt, Lx, Ly, kw;
    int32_t ngx, ngy;
    int32_t eos, gamma, visc, pad;
    double alpha;
} sph_params;

typedef struct sph_state_s *sph_state;         /* State          (src/driver.jl:5-36)   */
typedef struct sph_tape_s *sph_tape;           /* Tape           (src/driver.jl:45-65)  */
typedef struct sph_workspace_s *sph_workspace; /* AdjointWorkspace (src/driver.jl:117-133) */
typedef struct sph_field_s *sph_field;         /* device theta   (the `theta` argument)  */

enum { SPH_F64 = 0, SPH_F32 = 1 };

enum {
    SPH_OK = 0,
    SPH_ERR_ARG = 1,      /* ArgumentError in the reference */
    SPH_ERR_CAPACITY = 2, /* tape capacity exceeded (simulate!, src/driver.jl:94-99) */
    SPH_ERR_CUDA = 3,
    SPH_ERR_DTYPE = 4,
    SPH_ERR_NOMEM = 5,
    SPH_ERR_STATE = 6
};

/* neighbour-list flags read (and cleared) at the API boundary
   (check_neighbor_flags, src/neighbors.jl:282-290) */
enum {
    SPH_FLAG_NL_OVERFLOW = 1,  /* flags[1]: a row exceeded maxnb */
    SPH_FLAG_DISPLACEMENT = 2, /* flags[2]: displacement > skin*h before a rebuild */
    SPH_FLAG_NONFINITE = 4     /* non-finite position/velocity produced (no reference flag) */
};

SPH_API const char *sph_last_error(void);
SPH_API int32_t sph_version(void);
/* Use an external CUDA stream (cudaStream_t) instead of the library's own. */
SPH_API int32_t sph_set_stream(void *cuda_stream);
SPH_API int32_t sph_synchronize(void);

/* ---- design field theta: KernelAbstractions.allocate + copyto!(th, theta) ---- */
SPH_API int32_t sph_field_create(int32_t ngx, int32_t ngy, int32_t dtype, const void *theta,
                                 sph_field *out);
SPH_API int32_t sph_field_upload(sph_field th, const void *theta);
/* theta already on the device (e.g. a CuArray): device-to-device copy */
SPH_API int32_t sph_field_upload_device(sph_field th, const void *theta_dev);
SPH_API int32_t sph_field_destroy(sph_field th);

/* ---- State(backend, X0, V0, p; skin, interval, maxnb) (src/driver.jl:24-36) ---- */
SPH_API int32_t sph_state_create(const sph_params *p, int64_t N, const void *X0, const void *V0,
                                 int32_t dtype, double skin, int32_t interval, int32_t maxnb,
                                 sph_state *out);
SPH_API int32_t sph_state_destroy(sph_state st);
/* copyto!(st.X, X) / copyto!(st.V, V); either may be NULL */
SPH_API int32_t sph_state_set(sph_state st, const void *X, const void *V);
/* Array(st.X), Array(st.V) */
SPH_API int32_t sph_state_get(sph_state st, void *X, void *V);
/* Array(st.rho), st.pterm, st.invrho, st.a, st.alpha (a/alpha need keep_accel) */
SPH_API int32_t sph_state_fields(sph_state st, void *rho, void *pterm, void *invrho, void *a,
                                 void *alpha);
/* keep st.a and st.alpha up to date on every step (off by default: the fused
   accel+integrate kernel does not need them) */
SPH_API int32_t sph_state_keep_accel(sph_state st, int32_t on);
/* check_neighbor_flags (src/neighbors.jl:282-290): read and clear */
SPH_API int32_t sph_state_take_flags(sph_state st, uint32_t *flags);
SPH_API int32_t sph_state_grid(sph_state st, int32_t *nx, int32_t *ny, double *cs, int64_t *age);

/* build!(cl, X, p, backend) (src/neighbors.jl:97-114) */
SPH_API int32_t sph_build_cells(sph_state st);
/* build_neighbors!(nl, cl, X, p, backend) (src/neighbors.jl:252-263) */
SPH_API int32_t sph_build_neighbors(sph_state st);
/* CellList counts (ncell), starts (ncell, 0-based), order (N, 1-based ids) */
SPH_API int32_t sph_get_celllist(sph_state st, int32_t *counts, int32_t *starts, int32_t *order);
/* NeighborList rows, particle-major: indices[(i-1)*maxnb + m] (1-based ids) */
SPH_API int32_t sph_get_neighbors(sph_state st, int32_t *indices, int32_t *nbcount);

/* step!(st, theta, p, backend) (src/forward.jl:161-173); p may be NULL (use the
   state's parameters). Does not synchronise. */
SPH_API int32_t sph_step(sph_state st, sph_field theta, const sph_params *p);
/* simulate!(st, theta, p, backend, nsteps; tape) (src/driver.jl:92-115); tape
   may be NULL; *flags (may be NULL) receives the neighbour-list flags. */
SPH_API int32_t sph_simulate(sph_state st, sph_field theta, const sph_params *p, int64_t nsteps,
                             sph_tape tape, uint32_t *flags);

/* ---- Tape(backend, N, nsteps, p) (src/driver.jl:62-65): full (X, V) history ---- */
SPH_API int32_t sph_tape_create(int64_t N, int64_t nsteps, int32_t dtype, sph_tape *out);
/* Binomial checkpoint tape: keeps `nsnapshots` device snapshots (each holding the
   full state and its neighbour structure) and recomputes the forward during
   backward (no counterpart in the reference, which stores every step;
   src/driver.jl:56-60 names it as the next step). */
SPH_API int32_t sph_tape_create_checkpointed(int64_t N, int64_t nsteps, int32_t nsnapshots,
                                             int32_t dtype, sph_tape *out);
/* Tape mode chosen from a device-memory budget (no counterpart in the
   reference, whose Tape stores every step; src/driver.jl:56-60 names
   checkpointing as the way beyond that size). The full tape when its
   2 * 2 * sizeof(T) * N * nsteps bytes fit in budget_bytes; otherwise binomial
   checkpointing with as many snapshots as fit beside the recompute state (at
   most nsteps - 1: more would not save a recomputed step). A snapshot holds
   the state's core arrays and cell table, whose size follows from p (Lx, Ly,
   h) and skin. budget_bytes < 0: 90% of the device's free memory at the call.
   *nsnapshots: 0 = full tape; *bytes: the tape's device bytes (either may be
   NULL). SPH_ERR_NOMEM when not even one snapshot fits. sph_tape_plan only
   plans (host only when budget_bytes >= 0); sph_tape_create_auto creates the
   tape it plans, and sph_tape_snapshots reads a tape's mode back. */
SPH_API int32_t sph_tape_plan(const sph_params *p, int64_t N, int64_t nsteps, int32_t dtype,
                              double skin, int64_t budget_bytes, int32_t *nsnapshots,
                              int64_t *bytes);
SPH_API int32_t sph_tape_create_auto(const sph_params *p, int64_t N, int64_t nsteps,
                                     int32_t dtype, double skin, int64_t budget_bytes,
                                     sph_tape *out);
SPH_API int32_t sph_tape_snapshots(sph_tape tp, int32_t *nsnapshots);
SPH_API int32_t sph_tape_destroy(sph_tape tp);
/* reset!(tape) (src/driver.jl:71) */
SPH_API int32_t sph_tape_reset(sph_tape tp);
/* length(tape) (src/driver.jl:67) */
SPH_API int32_t sph_tape_length(sph_tape tp, int64_t *n);
/* tape.X[:, :, n], tape.V[:, :, n] (1-based n; full tapes only) */
SPH_API int32_t sph_tape_get(sph_tape tp, int64_t n, void *X, void *V);
/* forward steps recomputed by the last backward over this tape */
SPH_API int32_t sph_tape_recomputed_steps(sph_tape tp, int64_t *n);

/* ---- AdjointWorkspace(backend, N, p) (src/driver.jl:128-133) ---- */
SPH_API int32_t sph_workspace_create(int64_t N, const sph_params *p, int32_t dtype,
                                     sph_workspace *out);
SPH_API int32_t sph_workspace_destroy(sph_workspace ws);
/* backward!(ws, tape, theta, p, backend; seedX, seedV, scratch, skin, interval,
   maxnb) (src/driver.jl:141-207). seeds are host arrays (NULL = zero); scratch
   may be NULL (a fresh one, as in the reference). */
SPH_API int32_t sph_backward(sph_workspace ws, sph_tape tp, sph_field theta,
                             const sph_params *p, const void *seedX, const void *seedV,
                             sph_state scratch, double skin, int32_t interval, int32_t maxnb,
                             uint32_t *flags);
/* Array(ws.gX), Array(ws.gV), Array(ws.gtheta); any may be NULL */
SPH_API int32_t sph_workspace_get(sph_workspace ws, void *gX, void *gV, void *gtheta);

/* copyto!(dst, src) for whole States of the same configuration: positions,
   velocities, permutation and neighbour structure (device to device) */
SPH_API int32_t sph_state_assign(sph_state dst, sph_state src);

/* On-device objectives (the reference evaluates them on the host after
   Array(st.X)): J of the state's current (X, V), with the terminal seeds
   dJ/dX_T, dJ/dV_T left in the workspace for sph_backward_seeded.
   SPH_OBJ_TARGET is target_objective(X, xc, yc, sigma) (src/driver.jl:219-234),
   args = {xc, yc, sigma}; SPH_OBJ_KE_RIGHT is the kinetic energy of the
   particles with x > Lx/2 (args unused). J is summed in double in a fixed
   order (deterministic). p may be NULL (the state's parameters). */
enum { SPH_OBJ_KE_RIGHT = 0, SPH_OBJ_TARGET = 1 };
SPH_API int32_t sph_objective(sph_workspace ws, sph_state st, int32_t kind, const double *args,
                              const sph_params *p, double *J);
/* backward! with the seeds of the last sph_objective on this workspace (p may be
   NULL for a batch) */
SPH_API int32_t sph_backward_seeded(sph_workspace ws, sph_tape tp, sph_field theta,
                                    const sph_params *p, sph_state scratch, double skin,
                                    int32_t interval, int32_t maxnb, uint32_t *flags);

/* ---- batches ----
   No counterpart in the reference (one State per call there). B independent
   instances (their own SPHParams, particle counts, cell grids and design
   fields; shared neighbour-list knobs) packed into one State, design field and
   workspace, so every kernel of step!/simulate!/backward! runs once for all of
   them. Host arrays are packed: instance b's particles occupy ids
   [off_b, off_b + N[b]) with off_b = N[0] + ... + N[b-1]; its theta block
   ((ngy_b, ngx_b) column-major) follows instance b-1's. Each instance's
   results equal those of the same instance run alone (bit for bit in FP64).
   Use the State/Tape/workspace calls above on the packed handles (p = NULL:
   each instance keeps its own parameters; a tape is created for the total
   particle count). */
SPH_API int32_t sph_batch_create(int32_t B, const sph_params *params, const int64_t *N,
                                 const void *X0, const void *V0, int32_t dtype, double skin,
                                 int32_t interval, int32_t maxnb, sph_state *out);
SPH_API int32_t sph_batch_field_create(int32_t B, const int32_t *ngx, const int32_t *ngy,
                                       int32_t dtype, const void *theta, sph_field *out);
SPH_API int32_t sph_batch_workspace_create(int32_t B, const sph_params *params, const int64_t *N,
                                           int32_t dtype, sph_workspace *out);
SPH_API int32_t sph_batch_size(sph_state st, int32_t *B);
/* per-instance neighbour-list flags, flags[B] (read and cleared) */
SPH_API int32_t sph_batch_take_flags(sph_state st, uint32_t *flags);
/* per-instance objective J[B]; args: 3 values (xc, yc, sigma) per instance for
   SPH_OBJ_TARGET, NULL for SPH_OBJ_KE_RIGHT. Seeds stay in the workspace. */
SPH_API int32_t sph_batch_objective(sph_workspace ws, sph_state st, int32_t kind,
                                    const double *args, double *J);

/* ---- request server (continuous batching) ----
   No counterpart in the reference, whose optimisation driver calls
   simulate!/backward! one solve at a time (scripts/03_optimize.jl:228-254).
   `workers` host threads, each with its own CUDA stream, take forward+adjoint
   requests FIFO as soon as a worker is free and the request's device memory
   (states, tape or checkpoints, workspace; sph_request_bytes) fits within
   hbm_budget_bytes next to the requests already running: requests join while
   others run and their kernels overlap on the device. Each result equals the
   same request solved alone. Host inputs of a request (X0, V0, theta) must
   stay valid, and its outputs (gX, gV, gtheta; any may be NULL) are written,
   before sph_server_wait returns. A request whose gX, gV and gtheta are all
   NULL is forward only (objective_only in scripts/03_optimize.jl:248-254):
   no tape and no reverse sweep, J alone. Wait for every ticket before
   destroying. */
typedef struct sph_server_s *sph_server;
/* snapshots: 0 full tape; c > 0 binomial checkpoints with c snapshots; -1 the
   server chooses: the full tape when it takes at most an eighth of the HBM
   budget, else the checkpoint snapshots that fit in that eighth
   (sph_tape_plan). */
typedef struct sph_request {
    sph_params p;
    int64_t N;
    const void *X0, *V0;   /* (2, N) T, host */
    const void *theta;     /* (ngy, ngx) column-major T, host */
    int64_t nsteps;
    int32_t snapshots;     /* 0: full tape; c > 0: binomial checkpoints; -1: chosen */
    int32_t objective;     /* SPH_OBJ_KE_RIGHT or SPH_OBJ_TARGET */
    double obj_args[3];    /* (xc, yc, sigma) for SPH_OBJ_TARGET */
    double skin;
    int32_t interval, maxnb;
    void *gX, *gV, *gtheta; /* host outputs */
} sph_request;
SPH_API int32_t sph_server_create(int32_t workers, int64_t hbm_budget_bytes, int32_t dtype,
                                  sph_server *out);
/* The packed server: continuous batching at kernel granularity. One scheduler
   thread admits requests FIFO while their device bytes fit in
   hbm_budget_bytes and fewer than max_inflight are in flight; every request
   in flight advances one time step per tick (a forward step, or a reverse
   step with its recomputation), and each pass of a tick -- the gathers, every
   cell-list stage, density, forces, pass 1, pass 2, the design-node flush --
   is one launch over the particles of all of them. A request joins at the
   next tick after admission and leaves when its solve ends. Results equal the
   same request solved alone with one thread per particle (bit for bit in
   FP64). Same submit / wait / poll / stats calls as sph_server_create. */
SPH_API int32_t sph_server_create_packed(int32_t max_inflight, int64_t hbm_budget_bytes,
                                         int32_t dtype, sph_server *out);
SPH_API int32_t sph_server_destroy(sph_server s);
SPH_API int32_t sph_server_submit(sph_server s, const sph_request *req, int64_t *ticket);
/* blocks until the request is done; J, latency (submit to done) and flags */
SPH_API int32_t sph_server_wait(sph_server s, int64_t ticket, double *J, double *latency_ms,
                                uint32_t *flags);
SPH_API int32_t sph_server_poll(sph_server s, int64_t ticket, int32_t *done);
/* latency percentiles of completed requests, particle-steps/s over the span
   from the first submit to the last completion, completed count, peak
   admitted bytes and peak number of requests in flight */
SPH_API int32_t sph_server_stats(sph_server s, double *p50_ms, double *p99_ms,
                                 double *particle_steps_per_s, int64_t *completed,
                                 int64_t *peak_bytes, int32_t *peak_inflight);
SPH_API int32_t sph_server_reset_stats(sph_server s);
/* admission estimate of one request's device bytes */
SPH_API int64_t sph_request_bytes(const sph_request *req, int32_t dtype);

/* ---- design side of the topology-optimisation caller, on the device ----
   The design maths of scripts/03_optimize.jl around simulate!/backward!:
   alpha(rho) = alpha_max qp (1 - rho) / (qp + rho) and its derivative
   (:142-143), the linear-weight density filter of radius `radius` grid points
   (weights (r + 1) - dist, normalised; neighbours in the script's order) with
   its clamp to [0, 1] (:150-185) and its transposed adjoint (:187-195), the
   lower-bound volume projection by 60 bisections (:206-219) and the
   projected-gradient candidate rd - step g / max|g| of the line search
   (:314-341). Design variables are double whatever the particle precision;
   arrays are (ngy, ngx) column-major like theta. The handle keeps the design
   rd, its gradient and the last candidate on the device:
     sph_design_set / get       rd (host <-> device); get also returns the
                                filtered design and the gradient (any NULL)
     sph_design_to_theta        theta = alpha(filter(rd)) into a device field
     sph_design_gradient        grad = filter_adjoint(dJ/dtheta * dalpha(filter(rd)))
                                from the workspace's last backward (device to
                                device); *gmax (may be NULL) = max |grad|
     sph_design_candidate       cand = project(rd - step grad / max|grad|) and,
                                when theta is not NULL, theta of it
     sph_design_accept          rd = cand
     sph_design_apply           one operation on a host array (op below) */
typedef struct sph_design_s *sph_design;
enum {
    SPH_DESIGN_FILTER = 0,
    SPH_DESIGN_FILTER_ADJOINT = 1,
    SPH_DESIGN_PROJECT = 2,
    SPH_DESIGN_ALPHA = 3,
    SPH_DESIGN_DALPHA = 4
};
SPH_API int32_t sph_design_create(int32_t ngx, int32_t ngy, int32_t radius, double alpha_max,
                                  double qp, double volfrac, sph_design *out);
SPH_API int32_t sph_design_destroy(sph_design d);
SPH_API int32_t sph_design_set(sph_design d, const double *rd);
SPH_API int32_t sph_design_get(sph_design d, double *rd, double *rdf, double *grad);
SPH_API int32_t sph_design_to_theta(sph_design d, sph_field theta);
SPH_API int32_t sph_design_gradient(sph_design d, sph_workspace ws, double *gmax);
SPH_API int32_t sph_design_candidate(sph_design d, double step, sph_field theta);
SPH_API int32_t sph_design_accept(sph_design d);
SPH_API int32_t sph_design_apply(sph_design d, int32_t op, const double *in, double *out);

/* ---- cell list without allocation ----
   No counterpart in the reference. build!(cl, X, p, backend)
   (src/neighbors.jl:97-114) for callers that cannot let a library allocate
   device memory (their arrays come from their own pool or budgeted
   allocator). X_dev: N positions, interleaved T on the device; outputs are
   caller-owned device arrays: counts[nx*ny], starts[nx*ny] (0-based),
   order[N] (1-based ids, ascending within each cell), exactly as sph_build_cells
   + sph_get_celllist give them. cs is CellList.cs, nx/ny its grid. Work
   arrays live in a fixed device array (about 16 MiB per GPU, held until
   exit), so N <= SPH_NOALLOC_MAX_PARTICLES and nx*ny <= SPH_NOALLOC_MAX_CELLS;
   larger sizes return SPH_ERR_ARG. Calls no cudaMalloc/cudaFree. Enqueued on
   `stream` (a cudaStream_t, NULL = legacy default) and not synchronised.
   All calls share the work array: calls that overlap on the GPU race, so
   serialise them. Each call outside a stream capture resolves the array's
   device address (cudaGetSymbolAddress on the current device); a call while
   `stream` is captured reuses the last one, so make one uncaptured call on
   each device before capturing. A CUDA error already pending when the call
   starts is reported (SPH_ERR_CUDA) and nothing is launched. */
#define SPH_NOALLOC_MAX_PARTICLES (1 << 20)
#define SPH_NOALLOC_MAX_CELLS (1 << 20)
SPH_API int32_t sph_build_cells_noalloc(const void *X_dev, int64_t N, int32_t dtype, double cs,
                                        int32_t nx, int32_t ny, int32_t *counts_dev,
                                        int32_t *starts_dev, int32_t *order_dev, void *stream);

/* Block-size autotuner (no counterpart in the reference, which leaves the
   workgroup size to KernelAbstractions): times the neighbour-list build,
   density, accel+integrate and the three adjoint passes at 64/128/256 threads
   per block on this state's current positions (reps launches each) and uses
   the fastest from then on for every object of the same precision and kind
   (single or batched). blocks[6] (may be NULL) receives the choices in that
   order. Runs on the state's own arrays and a temporary workspace; the state's
   positions and velocities are not changed. */
SPH_API int32_t sph_autotune(sph_state st, sph_field theta, int32_t reps, int32_t *blocks);
/* Set or read the six block sizes directly (same order; each 64, 128 or 256,
   else SPH_ERR_ARG), for this state's precision and kind. A caller can time
   the kernels inside its own solves with sph_profile_* and keep the fastest
   per kernel (the Python mirror's autotune_in_solve does this): repeated
   launches of one kernel, as sph_autotune times them, can favour a size that
   is slower inside the solve's kernel sequence. */
SPH_API int32_t sph_set_block_sizes(sph_state st, const int32_t *blocks);
SPH_API int32_t sph_get_block_sizes(sph_state st, int32_t *blocks);

/* Lanes per particle of the neighbour-list and pair-sum kernels (no
   counterpart in the reference), process-wide. 0 (default): by state size --
   single states of up to 16384 particles give each particle a group of 32
   lanes (up to 512 particles in FP64, 2048 in FP32) or 16 lanes, larger
   states one thread. 1: always one thread. 16 or 32: groups for every
   single-instance state. Every setting adds each particle's pair terms in the
   same order, so FP64 results are bit-identical across settings; FP32 results
   may differ in the last bits (multiply-add contraction differs between the
   forms). Batches always use one thread per particle, so an FP32 batch member
   equals a solo run made with lanes = 1. Other values: SPH_ERR_ARG. */
SPH_API int32_t sph_set_group_lanes(int32_t lanes);
/* Density kernel form of FP32 states that run one thread per particle (no
   counterpart in the reference), process-wide: 0 walks each particle's
   neighbour row masks one candidate at a time; 1 (single states) uses the
   cell-tile form, where a warp stages the neighbouring cell rows of its 32
   consecutive particles in shared memory once and every lane scans all staged
   candidates; 2 (default) walks the masks taking two candidates per
   iteration, their kernel arithmetic in packed f32x2 instructions (7% faster
   than 0 on 1M particles; 1 is 3.4x slower). Every form adds the same
   terms in the same order; they may differ in the last bits of FP32 through
   multiply-add contraction. Other values: SPH_ERR_ARG. */
SPH_API int32_t sph_set_density_form(int32_t form);
/* Programmatic dependent launch (no counterpart in the reference),
   process-wide: 1 (default) launches the engine's kernels so that each may be
   scheduled while its predecessor on the stream still runs, waiting on the
   device for the predecessor's results, so the next kernel's blocks fill the
   SMs that the running kernel's last blocks leave free (1M FP32 particles:
   1558 vs 1483 M particle-steps/s). 0 launches them one after the other.
   Results do not depend on it; recorded groups of steps and captured
   sequences use plain launches. */
SPH_API int32_t sph_set_launch_overlap(int32_t on);
/* Steps per recorded group (no counterpart in the reference), process-wide:
   simulate and backward record the launches of `steps` consecutive steps
   (forward, recomputed and reverse steps alike, with the snapshot copies
   between them) and replay each group as one CUDA graph, which shortens the
   gaps between the short kernels of small states. It applies to FP64 states
   and to FP32 states of up to 2^18 particles (larger FP32 states run faster
   with programmatic dependent launch). A group is recorded again
   for every replay, so pointers and rebuild steps may differ between groups;
   graphs of the same shape are reused through an update. Default 32; 0
   launches every kernel on its own. Grouping is skipped inside a caller's
   capture and while a kernel timer is on. Results do not depend on it.
   Negative values: SPH_ERR_ARG. */
SPH_API int32_t sph_set_step_graphs(int32_t steps);
SPH_API int32_t sph_get_step_graphs(int32_t *steps);
/* Groups of steps replayed as graphs, and graphs instantiated for them, since
   the library was loaded (process-wide; either pointer may be NULL). */
SPH_API int32_t sph_step_graph_counts(int64_t *replays, int64_t *instantiations);
SPH_API int32_t sph_get_density_form(int32_t *form);
SPH_API int32_t sph_get_group_lanes(int32_t *lanes);

/* ---- captured sequences (no counterpart in the reference) ----
   sph_capture_begin records every call the calling thread makes on its library
   stream into a CUDA graph instead of running it; sph_capture_end instantiates
   the graph and sph_graph_launch replays it (enqueued, not waited for). While
   capturing, calls return no host results (J, flags: 0) and never wait; read
   them after a replay with sph_workspace_objective_value,
   sph_state_take_flags and sph_workspace_take_flags, and the state and
   gradients with the usual getters. Calls that would allocate device memory
   (the first use of a state, tape, snapshot or workspace) or copy host arrays
   (host seeds) fail while capturing: run the sequence once, then capture it.
   A graph replays only the device work; the handles' host bookkeeping
   (neighbour-list age, tape length, snapshot slots) stays as the capture left
   it, so capture a sequence that starts from a reset -- for instance one whole
   solve: sph_state_assign from a pristine state, sph_tape_reset, sph_simulate,
   sph_objective, sph_backward_seeded -- and replay it as a unit. */
typedef struct sph_graph_s *sph_graph;
SPH_API int32_t sph_capture_begin(void);
SPH_API int32_t sph_capture_end(sph_graph *out);
SPH_API int32_t sph_graph_launch(sph_graph g);
/* kernel launches one replay performs */
SPH_API int32_t sph_graph_nodes(sph_graph g, int64_t *nodes);
SPH_API int32_t sph_graph_destroy(sph_graph g);
/* J of the last sph_objective / sph_batch_objective (one per instance), read
   from the device; neighbour-list flags of the last backward's reverse sweep */
SPH_API int32_t sph_workspace_objective_value(sph_workspace ws, double *J);
SPH_API int32_t sph_workspace_take_flags(sph_workspace ws, uint32_t *flags);

/* ---- instrumentation ---- */
/* kernels launched by this library since load */
SPH_API int64_t sph_launch_count(void);
/* time every launch of one kernel id with CUDA events on the library stream */
SPH_API int32_t sph_profile_enable(int32_t kernel_id, int32_t on);
SPH_API int32_t sph_profile_read(int32_t kernel_id, double *total_ms, int64_t *launches);
SPH_API int32_t sph_profile_reset(void);
/* kernel ids for sph_profile_* */
enum {
    SPH_K_ASSIGN = 0, SPH_K_SCAN, SPH_K_BUCKET, SPH_K_RANK, SPH_K_NLBUILD, SPH_K_DENSITY,
    SPH_K_ACCEL_INTEGRATE, SPH_K_TAPE, SPH_K_GATHER, SPH_K_ACCEL_DRAG, SPH_K_PASS1,
    SPH_K_PASS2, SPH_K_THETA_NODE, SPH_K_MISC
};

/* binomial checkpoint schedule (host only): forward steps to reverse l steps
   with c snapshot slots, and the optimal first split */
SPH_API int64_t sph_plan_cost(int64_t l, int64_t c);
SPH_API int64_t sph_plan_split(int64_t l, int64_t c);

#ifdef __cplusplus
}
#endif

#endif
