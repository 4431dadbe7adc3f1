// Precision-independent interfaces between the C ABI (sph_capi.cu) and the
// two precision instantiations of the engine (sph_f32.cu, sph_f64.cu), plus the
// small runtime shared by both (stream, launch counter, kernel timers).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace sphgb {

// SPHParams (src/params.jl:14-28); fields are converted to T by the engine.
// eos / gamma / visc / alpha select the model variants (no counterpart in the
// reference): eos 0 linear, 1 Tait with integer exponent gamma; visc 0 Morris,
// 1 Monaghan artificial viscosity with coefficient alpha.
struct Params {
    double h, m, rho0, c, mu, gx, gy, dt, Lx, Ly, kw;
    int32_t ngx, ngy;
    int32_t eos = 0, gamma = 7, visc = 0, pad = 0;
    double alpha = 0.0;
};

// NeighborList knobs (src/neighbors.jl:174-175).
struct NLOpts {
    double skin;
    int32_t interval;
    int32_t maxnb;
};

enum Dtype : int32_t { F64 = 0, F32 = 1 };

// Error with a status code that the C ABI returns.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

enum Status : int32_t {
    OK = 0,
    ERR_ARG = 1,      // ArgumentError in the reference
    ERR_CAPACITY = 2, // tape capacity exceeded (ArgumentError in simulate!)
    ERR_CUDA = 3,
    ERR_DTYPE = 4,
    ERR_NOMEM = 5,
    ERR_STATE = 6,
};

void cuda_check(cudaError_t e, const char *what);
void set_last_error(const std::string &msg);
#define SPH_CK(call) ::sphgb::cuda_check((call), #call)

// ---- runtime ---------------------------------------------------------------
enum KernelId : int32_t {
    K_ASSIGN = 0,
    K_SCAN,
    K_BUCKET,
    K_RANK,
    K_NLBUILD,
    K_DENSITY,
    K_ACCEL_INTEGRATE,
    K_TAPE,
    K_GATHER,
    K_ACCEL_DRAG,
    K_PASS1,
    K_PASS2,
    K_THETA_NODE,
    K_MISC,
    K_COUNT
};

// The library stream of the calling host thread (created on first use unless
// the thread set its own with rt_set_stream).
cudaStream_t rt_stream();
void rt_set_stream(cudaStream_t s);
// Stream-ordered device allocation (the device's default memory pool, kept
// cached between requests).
cudaError_t rt_malloc(void **p, size_t bytes, cudaStream_t s);
void rt_free(void *p, cudaStream_t s);
void rt_before_launch(int kid);
void rt_after_launch(int kid);
void rt_check_launch(const char *name);
// Lanes per particle of the pair-sum kernels: 0 = by state size (groups of 16
// or 32 lanes for single states of up to 16384 particles, one thread otherwise), 1 = one thread,
// 16 or 32 = groups for every single-instance state.
int rt_group_lanes();
void rt_set_group_lanes(int lanes);
// Density kernel form of FP32 states with one thread per particle: 0 = the
// per-particle mask walk, 1 = the cell-tile form (single states), 2 (default)
// = the mask walk taking two candidates per iteration in packed f32x2
// arithmetic.
int rt_density_form();
void rt_set_density_form(int form);
// Programmatic dependent launch of the engine's kernels (default on).
bool rt_launch_overlap();
void rt_set_launch_overlap(bool on);
// Steps that simulate and backward record into one CUDA graph and replay
// (0: every kernel is launched on its own; default 32).
int rt_step_graph();
void rt_set_step_graph(int steps);
// True while the calling thread records its library stream into a CUDA graph
// (a caller's capture or a group of steps): host reads and synchronisations
// are skipped (results stay on the device) and device allocations are
// refused.
bool rt_capturing();
// True when any kernel timer is on (launches are then not grouped, so that
// each one is timed on its own).
bool rt_timers_on();

// The launches of a sequence of steps (a solve's forward or reverse sweep),
// recorded from the library stream in groups of rt_step_graph() steps; each
// group is replayed as one CUDA graph as soon as it is complete, so the
// device runs the same work in the same order as with direct launches, with
// graph launch costs between the kernels. A group is recorded again on the
// host every time (its pointers change) and replayed through an instantiated
// graph of the same shape when one is cached (cudaGraphExecUpdate), else
// through a new one.
class StepGraphs {
  public:
    StepGraphs() = default;
    StepGraphs(const StepGraphs &) = delete;
    StepGraphs &operator=(const StepGraphs &) = delete;
    ~StepGraphs();
    // start of a sequence: grouping applies when `eligible`, the switch is
    // on, the thread is not already capturing and no kernel timer is on
    void start(bool eligible = true);
    // around each step
    void before_step();
    void after_step();
    // end of the sequence: replays the open group
    void finish();
    // error path: ends an open recording and drops it
    void abandon() noexcept;

  private:
    void replay();
    struct Entry {
        uint64_t key;
        cudaGraphExec_t exec;
        uint64_t used;
    };
    std::vector<Entry> cache_;
    int per_ = 0, count_ = 0;
    bool on_ = false, open_ = false;
    uint64_t clock_ = 0;
};

// Ends an open group of a StepGraphs when the scope is left by an exception.
struct StepGraphsGuard {
    StepGraphs &g;
    ~StepGraphsGuard() { g.abandon(); }
};
// Wait for the library stream unless it is being captured.
void rt_sync();

class FieldI {
  public:
    virtual ~FieldI() {}
    virtual int dtype() const = 0;
    virtual int ngx() const = 0;
    virtual int ngy() const = 0;
    virtual void upload(const void *host_colmajor) = 0;
    virtual void upload_device(const void *dev_colmajor) = 0;
};

class TapeI {
  public:
    virtual ~TapeI() {}
    virtual int dtype() const = 0;
    virtual int64_t N() const = 0;
    virtual int64_t capacity() const = 0;
    virtual int64_t length() const = 0;
    virtual int32_t snapshots() const = 0; // 0: full history
    virtual void reset() = 0;
    virtual void get(int64_t n, void *X, void *V) = 0;
    virtual int64_t forward_steps() const = 0; // steps recomputed by the last backward
};

class StateI {
  public:
    virtual ~StateI() {}
    virtual int dtype() const = 0;
    virtual int64_t N() const = 0;
    virtual void set(const void *X, const void *V) = 0;
    virtual void get(void *X, void *V) = 0;
    virtual void fields(void *rho, void *pterm, void *invrho, void *a, void *alpha) = 0;
    virtual void keep_accel(bool on) = 0;
    virtual void step(FieldI *theta, const Params *p) = 0;
    virtual void simulate(FieldI *theta, const Params *p, int64_t nsteps, TapeI *tape) = 0;
    virtual void build_cells() = 0;
    virtual void build_neighbors() = 0;
    virtual void celllist(int32_t *counts, int32_t *starts, int32_t *order) = 0;
    virtual void neighbors(int32_t *indices, int32_t *nbcount) = 0;
    virtual uint32_t take_flags() = 0;
    virtual void grid(int32_t *nx, int32_t *ny, double *cs, int64_t *age) const = 0;
    virtual void sync() = 0;
    virtual void assign(StateI *src) = 0;
    virtual int batch() const = 0;
    virtual void take_flags_batch(uint32_t *per_instance) = 0;
    virtual void autotune(FieldI *theta, int reps, int *chosen) = 0;
    // threads per block of the six tuned kernels (build, density, accel,
    // drag, pass 1, pass 2) for this state's precision and kind
    virtual void set_blocks(const int *blocks) = 0;
    virtual void get_blocks(int *blocks) const = 0;
};

enum ObjectiveKind : int32_t {
    OBJ_KE_RIGHT = 0, // J = sum 1/2 m |v|^2 over x > Lx/2
    OBJ_TARGET = 1,   // target_objective(X, xc, yc, sigma) (src/driver.jl:219-234)
};

class WorkI {
  public:
    virtual ~WorkI() {}
    virtual int dtype() const = 0;
    virtual int64_t N() const = 0;
    virtual void backward(TapeI *tape, FieldI *theta, const Params *p, const void *seedX,
                          const void *seedV, StateI *scratch, NLOpts opts,
                          uint32_t *flags) = 0;
    virtual void get(void *gX, void *gV, void *gtheta) = 0;
    virtual int batch() const = 0;
    // J of each instance's current positions/velocities (J[b]); the terminal
    // seeds stay on the device for backward_seeded
    virtual void objective(StateI *st, int kind, const double *args, const Params *p,
                           double *J) = 0;
    virtual void backward_seeded(TapeI *tape, FieldI *theta, const Params *p, StateI *scratch,
                                 NLOpts opts, uint32_t *flags) = 0;
    // J of the last objective() as the device holds it (one per instance)
    virtual void objective_value(double *J) = 0;
    // neighbour-list flags of the last backward's reverse sweep (read and cleared)
    virtual uint32_t take_flags() = 0;
    // dJ/dtheta of the last backward on the device (double, n nodes; single
    // instance), for consumers that stay on the device
    virtual const double *gtheta_device(int64_t n) const = 0;
};

// One request of the packed engine (sph_pack.cuh): its model, initial state,
// design field, horizon, tape mode (0 full tape, c > 0 checkpoint snapshots),
// objective and neighbour-list knobs; adjoint = false runs the forward sweep
// and the objective only. Host pointers must stay valid until add() returns.
struct PackReq {
    Params p;
    int64_t N = 0;
    const void *X0 = nullptr, *V0 = nullptr, *theta = nullptr;
    int64_t nsteps = 0;
    int32_t snapshots = 0;
    int32_t objective = 0;
    double obj_args[3] = {0.0, 0.0, 1.0};
    NLOpts opts{0.2, 4, 64};
    bool adjoint = true;
};

// The packed engine: all requests it holds advance one step per tick, each
// pass of a tick one grouped launch over all of them (see sph_pack.cuh).
// Used by one host thread, on that thread's library stream.
class PackI {
  public:
    virtual ~PackI() {}
    // create the request's device objects (allocates; synchronises the stream)
    virtual int add(const PackReq &r) = 0;
    // enqueue one tick; returns the number of requests that took a step
    virtual int tick() = 0;
    // requests whose programs have completed on the device (block: wait for
    // the first unfinished one)
    virtual void reap(std::vector<int> &done, bool block) = 0;
    virtual int finishing() const = 0;
    // J, flags and (adjoint requests) gradients of a completed request,
    // copied on stream cs into host buffers (any may be NULL)
    virtual void result(int id, cudaStream_t cs, double *J, uint32_t *flags, void *gX, void *gV,
                        void *gtheta) = 0;
    virtual void release(int id) = 0;
    virtual int active() const = 0;
    virtual int64_t ticks() const = 0;
};

#define SPH_DECLARE_FACTORIES(SFX)                                                           \
    FieldI *make_field##SFX(const std::vector<int> &ngx, const std::vector<int> &ngy,        \
                            const void *host);                                               \
    TapeI *make_tape##SFX(int64_t N, int64_t cap, int32_t nsnap);                            \
    StateI *make_state##SFX(const std::vector<Params> &p, const std::vector<int64_t> &N,     \
                            const void *X0, const void *V0, NLOpts o);                       \
    WorkI *make_work##SFX(const std::vector<Params> &p, const std::vector<int64_t> &N);       \
    PackI *make_pack##SFX();

SPH_DECLARE_FACTORIES(_f32)
SPH_DECLARE_FACTORIES(_f64)

// ---- binomial checkpoint schedule (checkpoint_plan.cpp) ---------------------
// Minimal number of forward steps needed to reverse l steps when the state at
// the start of the range is held in one of c snapshot slots.
int64_t plan_cost(int64_t l, int64_t c);
// The split m in [1, l-1] that attains plan_cost (smallest such m).
int64_t plan_split(int64_t l, int64_t c);
// Snapshot positions taken while sweeping forward over l steps with c slots.
std::vector<int64_t> plan_descent(int64_t l, int64_t c);
// Tape mode of one state under a device-memory budget: *nsnap = 0 for the full
// tape, else the most checkpoint snapshots that fit (ERR_NOMEM when none does).
void tape_plan(const Params &p, int64_t N, int64_t nsteps, int dtype, double skin,
               int64_t budget, int32_t *nsnap, int64_t *bytes);

} // namespace sphgb
