// C ABI of the library, the shared runtime (stream, launch counter, kernel
// timers) and the binomial checkpoint schedule. Precision-specific work is
// done by the engines in sph_f32.cu / sph_f64.cu behind sph_iface.hpp.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sphadjoint_gb300.h"
#include "sph_iface.hpp"

namespace sphgb {

// ---------------------------------------------------------------------------
// runtime
// ---------------------------------------------------------------------------
namespace {
thread_local std::string g_err;
thread_local cudaStream_t g_stream = nullptr;
thread_local bool g_stream_external = false;
std::atomic<long long> g_launches{0};
std::atomic<int> g_group_lanes{0};
std::atomic<int> g_density_form{2};
std::atomic<bool> g_launch_overlap{true};
std::atomic<int> g_step_graph{32};
std::atomic<long long> g_sg_replays{0}, g_sg_inst{0};
thread_local bool g_capturing = false;
thread_local bool g_recording = false;
std::mutex g_pool_mu;
bool g_pool_ready[64] = {};

struct KTimer {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    int64_t launches = 0;
};
KTimer g_timer[K_COUNT];
} // namespace

void set_last_error(const std::string &msg) { g_err = msg; }

void cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw Error(ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

cudaStream_t rt_stream()
{
    if (!g_stream && !g_stream_external)
        cuda_check(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    return g_stream;
}

void rt_set_stream(cudaStream_t s)
{
    g_stream = s;
    g_stream_external = s != nullptr;
}

// Keep freed blocks in the device's default pool instead of returning them to
// the driver, so per-request allocations are served from the cache.
static void pool_init()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    std::lock_guard<std::mutex> g(g_pool_mu);
    if (g_pool_ready[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        (void)cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    (void)cudaGetLastError();
    g_pool_ready[dev] = true;
}

cudaError_t rt_malloc(void **p, size_t bytes, cudaStream_t s)
{
    pool_init();
    return cudaMallocAsync(p, bytes, s);
}

void rt_free(void *p, cudaStream_t s)
{
    if (cudaFreeAsync(p, s) != cudaSuccess) (void)cudaGetLastError();
}

static cudaEvent_t timer_event(KTimer &t)
{
    if (t.used == t.pool.size()) {
        cudaEvent_t e;
        cuda_check(cudaEventCreate(&e), "cudaEventCreate");
        t.pool.push_back(e);
    }
    return t.pool[t.used++];
}

void rt_before_launch(int kid)
{
    KTimer &t = g_timer[kid];
    if (t.on && !g_capturing) cuda_check(cudaEventRecord(timer_event(t), rt_stream()), "cudaEventRecord");
}

void rt_after_launch(int kid)
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    KTimer &t = g_timer[kid];
    if (t.on && !g_capturing) {
        cuda_check(cudaEventRecord(timer_event(t), rt_stream()), "cudaEventRecord");
        t.launches += 1;
    }
}

void rt_check_launch(const char *name) { cuda_check(cudaGetLastError(), name); }

bool rt_capturing() { return g_capturing || g_recording; }

bool rt_timers_on()
{
    for (const KTimer &t : g_timer)
        if (t.on) return true;
    return false;
}

void rt_sync()
{
    if (!rt_capturing()) cuda_check(cudaStreamSynchronize(rt_stream()), "cudaStreamSynchronize");
}

int rt_step_graph() { return g_step_graph.load(std::memory_order_relaxed); }
void rt_set_step_graph(int steps) { g_step_graph.store(steps, std::memory_order_relaxed); }

// ---- groups of steps replayed as graphs ---------------------------------------
StepGraphs::~StepGraphs()
{
    abandon();
    for (Entry &e : cache_) (void)cudaGraphExecDestroy(e.exec);
    (void)cudaGetLastError();
}

void StepGraphs::start(bool eligible)
{
    per_ = rt_step_graph();
    on_ = eligible && per_ > 0 && !rt_capturing() && !rt_timers_on();
    if (on_) {
        // a stream the caller records with the CUDA API itself: its launches
        // go into the caller's graph as they are
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(rt_stream(), &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
            (void)cudaGetLastError();
            on_ = false;
        }
    }
    count_ = 0;
}

void StepGraphs::before_step()
{
    if (!on_ || open_) return;
    // a stream that cannot be recorded (the legacy default stream) runs the
    // sequence launch by launch
    if (cudaStreamBeginCapture(rt_stream(), cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        (void)cudaGetLastError();
        on_ = false;
        return;
    }
    open_ = true;
    g_recording = true;
    count_ = 0;
}

void StepGraphs::after_step()
{
    if (!open_) return;
    if (++count_ >= per_) replay();
}

void StepGraphs::finish()
{
    if (open_) replay();
    on_ = false;
}

void StepGraphs::abandon() noexcept
{
    if (!open_) return;
    open_ = false;
    g_recording = false;
    cudaGraph_t g = nullptr;
    (void)cudaStreamEndCapture(rt_stream(), &g);
    if (g) (void)cudaGraphDestroy(g);
    (void)cudaGetLastError();
}

void StepGraphs::replay()
{
    open_ = false;
    g_recording = false;
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(rt_stream(), &g);
    if (ec != cudaSuccess || !g) {
        if (g) (void)cudaGraphDestroy(g);
        cuda_check(ec != cudaSuccess ? ec : cudaErrorStreamCaptureInvalidated,
                   "cudaStreamEndCapture (group of steps)");
    }
    struct Drop {
        cudaGraph_t g;
        ~Drop() { (void)cudaGraphDestroy(g); }
    } drop{g};
    // shape key: node count, node types and kernel functions in recording order
    size_t n = 0;
    cuda_check(cudaGraphGetNodes(g, nullptr, &n), "cudaGraphGetNodes");
    if (n == 0) return;
    std::vector<cudaGraphNode_t> nodes(n);
    cuda_check(cudaGraphGetNodes(g, nodes.data(), &n), "cudaGraphGetNodes");
    uint64_t key = 1469598103934665603ull ^ (uint64_t)n;
    auto mix = [&](uint64_t v) { key = (key ^ v) * 1099511628211ull; };
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        cuda_check(cudaGraphNodeGetType(nd, &t), "cudaGraphNodeGetType");
        mix((uint64_t)t);
        if (t == cudaGraphNodeTypeKernel) {
            cudaKernelNodeParams kp{};
            cuda_check(cudaGraphKernelNodeGetParams(nd, &kp), "cudaGraphKernelNodeGetParams");
            mix((uint64_t)(uintptr_t)kp.func);
        }
    }
    Entry *hit = nullptr;
    for (Entry &e : cache_)
        if (e.key == key) hit = &e;
    if (hit) {
        cudaGraphExecUpdateResultInfo info{};
        if (cudaGraphExecUpdate(hit->exec, g, &info) != cudaSuccess) {
            (void)cudaGetLastError();
            (void)cudaGraphExecDestroy(hit->exec);
            hit->exec = nullptr;
            cuda_check(cudaGraphInstantiate(&hit->exec, g, 0), "cudaGraphInstantiate");
            g_sg_inst.fetch_add(1, std::memory_order_relaxed);
        }
    } else {
        constexpr size_t kMaxCached = 16;
        if (cache_.size() >= kMaxCached) {
            auto lru = std::min_element(cache_.begin(), cache_.end(),
                                        [](const Entry &a, const Entry &b) { return a.used < b.used; });
            (void)cudaGraphExecDestroy(lru->exec);
            cache_.erase(lru);
        }
        cudaGraphExec_t x = nullptr;
        cuda_check(cudaGraphInstantiate(&x, g, 0), "cudaGraphInstantiate");
        g_sg_inst.fetch_add(1, std::memory_order_relaxed);
        cache_.push_back({key, x, 0});
        hit = &cache_.back();
    }
    hit->used = ++clock_;
    cuda_check(cudaGraphLaunch(hit->exec, rt_stream()), "cudaGraphLaunch");
    g_sg_replays.fetch_add(1, std::memory_order_relaxed);
}

int rt_group_lanes() { return g_group_lanes.load(std::memory_order_relaxed); }
void rt_set_group_lanes(int lanes) { g_group_lanes.store(lanes, std::memory_order_relaxed); }
int rt_density_form() { return g_density_form.load(std::memory_order_relaxed); }
bool rt_launch_overlap() { return g_launch_overlap.load(std::memory_order_relaxed); }
void rt_set_launch_overlap(bool on) { g_launch_overlap.store(on, std::memory_order_relaxed); }
void rt_set_density_form(int form) { g_density_form.store(form, std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// Binomial checkpointing (Griewank's revolve bound). With c snapshot slots and
// t the smallest integer with binom(c + t, t) >= l, reversing l steps needs
// t*l - binom(c + t, t - 1) forward steps, and no schedule needs fewer.
// ---------------------------------------------------------------------------
static int64_t binom_sat(int64_t n, int64_t k)
{
    // binom(n, k) saturating at 2^62
    if (k < 0 || k > n) return 0;
    k = std::min(k, n - k);
    const long double cap = 4.611686018427387904e18L;
    long double r = 1;
    for (int64_t i = 1; i <= k; ++i) {
        r = r * (long double)(n - k + i) / (long double)i;
        if (r >= cap) return (int64_t)4611686018427387904LL;
    }
    return (int64_t)std::llround((double)r);
}

int64_t plan_cost(int64_t l, int64_t c)
{
    if (l <= 1) return 0;
    if (c <= 1) return l * (l - 1) / 2;
    int64_t t = 0;
    while (binom_sat(c + t, t) < l) ++t;
    return t * l - binom_sat(c + t, t - 1);
}

int64_t plan_split(int64_t l, int64_t c)
{
    static std::mutex mu;
    static std::map<std::pair<int64_t, int64_t>, int64_t> memo;
    if (l <= 1) return 0;
    if (c <= 1) return 1;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = memo.find({l, c});
        if (it != memo.end()) return it->second;
    }
    int64_t best = 1, bestCost = INT64_MAX;
    for (int64_t m = 1; m < l; ++m) {
        const int64_t v = m + plan_cost(l - m, c - 1) + plan_cost(m, c);
        if (v < bestCost) {
            bestCost = v;
            best = m;
        }
    }
    std::lock_guard<std::mutex> g(mu);
    memo[{l, c}] = best;
    return best;
}

std::vector<int64_t> plan_descent(int64_t l, int64_t c)
{
    std::vector<int64_t> pos{0};
    int64_t p = 0, len = l;
    while (len > 1 && c >= 2) {
        const int64_t m = plan_split(len, c);
        p += m;
        len -= m;
        c -= 1;
        pos.push_back(p);
    }
    return pos;
}

} // namespace sphgb

using namespace sphgb;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
template <typename F> static int32_t guarded(F &&f)
{
    try {
        f();
        return SPH_OK;
    } catch (const Error &e) {
        g_err = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_err = "host allocation failed";
        return SPH_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_err = e.what();
        return SPH_ERR_STATE;
    }
}

static Params to_params(const sph_params *p)
{
    if (!p) throw Error(ERR_ARG, "params is NULL");
    Params q;
    q.h = p->h; q.m = p->m; q.rho0 = p->rho0; q.c = p->c; q.mu = p->mu; q.gx = p->gx;
    q.gy = p->gy; q.dt = p->dt; q.Lx = p->Lx; q.Ly = p->Ly; q.kw = p->kw;
    q.ngx = p->ngx; q.ngy = p->ngy;
    q.eos = p->eos; q.gamma = p->gamma; q.visc = p->visc; q.alpha = p->alpha;
    return q;
}

static void need(const void *h, const char *what)
{
    if (!h) throw Error(ERR_ARG, std::string(what) + " is NULL");
}

static void check_dtype(int32_t d)
{
    if (d != SPH_F64 && d != SPH_F32) throw Error(ERR_DTYPE, "dtype must be SPH_F64 or SPH_F32");
}

#define ST(x) reinterpret_cast<StateI *>(x)
#define TP(x) reinterpret_cast<TapeI *>(x)
#define WS(x) reinterpret_cast<WorkI *>(x)
#define FD(x) reinterpret_cast<FieldI *>(x)

extern "C" {

SPH_API const char *sph_last_error(void) { return g_err.c_str(); }
SPH_API int32_t sph_version(void) { return 100; }

SPH_API int32_t sph_set_stream(void *s)
{
    return guarded([&] { rt_set_stream((cudaStream_t)s); });
}

SPH_API int32_t sph_synchronize(void)
{
    return guarded([&] { cuda_check(cudaStreamSynchronize(rt_stream()), "synchronize"); });
}

SPH_API int32_t sph_field_create(int32_t ngx, int32_t ngy, int32_t dtype, const void *theta,
                                 sph_field *out)
{
    return guarded([&] {
        need(out, "out");
        check_dtype(dtype);
        const std::vector<int> gx{ngx}, gy{ngy};
        FieldI *f = dtype == SPH_F64 ? make_field_f64(gx, gy, theta) : make_field_f32(gx, gy, theta);
        *out = reinterpret_cast<sph_field>(f);
    });
}

SPH_API int32_t sph_field_upload(sph_field th, const void *theta)
{
    return guarded([&] {
        need(th, "theta");
        need(theta, "host theta");
        FD(th)->upload(theta);
    });
}

SPH_API int32_t sph_field_upload_device(sph_field th, const void *theta)
{
    return guarded([&] {
        need(th, "theta");
        need(theta, "device theta");
        FD(th)->upload_device(theta);
    });
}

SPH_API int32_t sph_field_destroy(sph_field th)
{
    return guarded([&] { delete FD(th); });
}

SPH_API int32_t sph_state_create(const sph_params *p, int64_t N, const void *X0, const void *V0,
                                 int32_t dtype, double skin, int32_t interval, int32_t maxnb,
                                 sph_state *out)
{
    return guarded([&] {
        need(out, "out");
        check_dtype(dtype);
        const Params q = to_params(p);
        NLOpts o{skin, interval, maxnb};
        const std::vector<Params> ps{q};
        const std::vector<int64_t> ns{N};
        StateI *s = dtype == SPH_F64 ? make_state_f64(ps, ns, X0, V0, o)
                                     : make_state_f32(ps, ns, X0, V0, o);
        *out = reinterpret_cast<sph_state>(s);
    });
}

SPH_API int32_t sph_state_destroy(sph_state st)
{
    return guarded([&] { delete ST(st); });
}

SPH_API int32_t sph_state_set(sph_state st, const void *X, const void *V)
{
    return guarded([&] { need(st, "state"); ST(st)->set(X, V); });
}

SPH_API int32_t sph_state_get(sph_state st, void *X, void *V)
{
    return guarded([&] { need(st, "state"); ST(st)->get(X, V); });
}

SPH_API int32_t sph_state_fields(sph_state st, void *rho, void *pterm, void *invrho, void *a,
                                 void *alpha)
{
    return guarded([&] { need(st, "state"); ST(st)->fields(rho, pterm, invrho, a, alpha); });
}

SPH_API int32_t sph_state_keep_accel(sph_state st, int32_t on)
{
    return guarded([&] { need(st, "state"); ST(st)->keep_accel(on != 0); });
}

SPH_API int32_t sph_state_take_flags(sph_state st, uint32_t *flags)
{
    return guarded([&] {
        need(st, "state");
        const uint32_t f = ST(st)->take_flags();
        if (flags) *flags = f;
    });
}

SPH_API int32_t sph_state_grid(sph_state st, int32_t *nx, int32_t *ny, double *cs, int64_t *age)
{
    return guarded([&] { need(st, "state"); ST(st)->grid(nx, ny, cs, age); });
}

SPH_API int32_t sph_build_cells(sph_state st)
{
    return guarded([&] { need(st, "state"); ST(st)->build_cells(); });
}

SPH_API int32_t sph_build_neighbors(sph_state st)
{
    return guarded([&] { need(st, "state"); ST(st)->build_neighbors(); });
}

SPH_API int32_t sph_get_celllist(sph_state st, int32_t *counts, int32_t *starts, int32_t *order)
{
    return guarded([&] { need(st, "state"); ST(st)->celllist(counts, starts, order); });
}

SPH_API int32_t sph_get_neighbors(sph_state st, int32_t *indices, int32_t *nbcount)
{
    return guarded([&] { need(st, "state"); ST(st)->neighbors(indices, nbcount); });
}

SPH_API int32_t sph_step(sph_state st, sph_field theta, const sph_params *p)
{
    return guarded([&] {
        need(st, "state");
        need(theta, "theta");
        Params q;
        if (p) q = to_params(p);
        ST(st)->step(FD(theta), p ? &q : nullptr);
    });
}

SPH_API int32_t sph_simulate(sph_state st, sph_field theta, const sph_params *p, int64_t nsteps,
                             sph_tape tape, uint32_t *flags)
{
    return guarded([&] {
        need(st, "state");
        need(theta, "theta");
        if (nsteps < 0) throw Error(ERR_ARG, "nsteps must be >= 0");
        Params q;
        if (p) q = to_params(p);
        ST(st)->simulate(FD(theta), p ? &q : nullptr, nsteps, tape ? TP(tape) : nullptr);
        const uint32_t f = rt_capturing() ? 0u : ST(st)->take_flags();
        if (flags) *flags = f;
    });
}

SPH_API int32_t sph_tape_create(int64_t N, int64_t nsteps, int32_t dtype, sph_tape *out)
{
    return guarded([&] {
        need(out, "out");
        check_dtype(dtype);
        TapeI *t = dtype == SPH_F64 ? make_tape_f64(N, nsteps, 0) : make_tape_f32(N, nsteps, 0);
        *out = reinterpret_cast<sph_tape>(t);
    });
}

SPH_API int32_t sph_tape_create_checkpointed(int64_t N, int64_t nsteps, int32_t nsnapshots,
                                             int32_t dtype, sph_tape *out)
{
    return guarded([&] {
        need(out, "out");
        check_dtype(dtype);
        if (nsnapshots < 1) throw Error(ERR_ARG, "need at least one snapshot slot");
        TapeI *t = dtype == SPH_F64 ? make_tape_f64(N, nsteps, nsnapshots)
                                    : make_tape_f32(N, nsteps, nsnapshots);
        *out = reinterpret_cast<sph_tape>(t);
    });
}

// Device bytes of the two tape modes of one state (the layouts of Sys and
// Tape in sph_engine.cuh): a snapshot is the state's contiguous core block
// (positions and velocities in both buffers, rebuild positions, permutation,
// inverse, cell centres, six mask words, cell starts), and a checkpoint tape
// also holds a recompute state (the core plus the neighbour-list work arrays,
// in-support masks, densities and staging).
static int64_t align256(int64_t b) { return (b + 255) & ~(int64_t)255; }

static void tape_sizes(const Params *p, int64_t N, int32_t dtype, double skin, int64_t *snap,
                       int64_t *recomp)
{
    const int64_t s = dtype == SPH_F64 ? 8 : 4;
    const int64_t n1 = std::max<int64_t>(N, 1);
    // cell grid as State builds it: rc = Float64(T(2) T(h)) (1 + skin),
    // nx = ceil(Lx / rc) + 2 (src/neighbors.jl:28-36)
    const double hT = dtype == SPH_F64 ? p->h : (double)(float)p->h;
    const double rc = (dtype == SPH_F64 ? 2.0 * hT : (double)(2.0f * (float)hT)) * (1.0 + skin);
    const double LxT = dtype == SPH_F64 ? p->Lx : (double)(float)p->Lx;
    const double LyT = dtype == SPH_F64 ? p->Ly : (double)(float)p->Ly;
    const int64_t nx = (int64_t)std::max(1.0, std::ceil(LxT / rc) + 2);
    const int64_t ny = (int64_t)std::max(1.0, std::ceil(LyT / rc) + 2);
    const int64_t ncell = nx * ny;
    *snap = 5 * align256(2 * s * n1) + 3 * align256(4 * n1) + align256(24 * n1) +
            align256(4 * (ncell + 1));
    *recomp = *snap + (16 + 24 + 6 * s) * n1 + 8 * ncell + 4 * (ncell / 2048 + 2) + 4;
}

static int64_t device_budget()
{
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    return (int64_t)(0.9 * (double)fr);
}

} // extern "C"

namespace sphgb {
void tape_plan(const Params &pr, int64_t N, int64_t nsteps, int dtype, double skin,
               int64_t budget, int32_t *nsnap, int64_t *bytes)
{
    const Params *p = &pr;
    if (N < 0 || nsteps < 0) throw Error(ERR_ARG, "negative tape size");
    const int64_t s = dtype == SPH_F64 ? 8 : 4;
    const int64_t L = std::max<int64_t>(nsteps, 1);
    const int64_t full = 4 * s * std::max<int64_t>(N, 1) * L;
    if (full <= budget || L <= 1) {
        *nsnap = 0;
        *bytes = full;
        return;
    }
    int64_t snap = 0, recomp = 0;
    tape_sizes(p, N, dtype, skin, &snap, &recomp);
    const int64_t c = budget > recomp ? std::min<int64_t>((budget - recomp) / snap, L - 1) : 0;
    if (c < 1)
        throw Error(ERR_NOMEM, "tape of " + std::to_string(N) + " particles x " +
                                   std::to_string(nsteps) + " steps: not even one snapshot (" +
                                   std::to_string((snap + recomp) >> 20) + " MiB with the "
                                   "recompute state) fits in " + std::to_string(budget >> 20) +
                                   " MiB");
    *nsnap = (int32_t)std::min<int64_t>(c, INT32_MAX);
    *bytes = *nsnap * snap + recomp;
}
} // namespace sphgb

extern "C" {

SPH_API int32_t sph_tape_plan(const sph_params *p, int64_t N, int64_t nsteps, int32_t dtype,
                              double skin, int64_t budget_bytes, int32_t *nsnapshots,
                              int64_t *bytes)
{
    return guarded([&] {
        need(p, "params");
        check_dtype(dtype);
        int32_t c = 0;
        int64_t b = 0;
        tape_plan(to_params(p), N, nsteps, dtype, skin,
                  budget_bytes < 0 ? device_budget() : budget_bytes, &c, &b);
        if (nsnapshots) *nsnapshots = c;
        if (bytes) *bytes = b;
    });
}

SPH_API int32_t sph_tape_create_auto(const sph_params *p, int64_t N, int64_t nsteps,
                                     int32_t dtype, double skin, int64_t budget_bytes,
                                     sph_tape *out)
{
    return guarded([&] {
        need(out, "out");
        need(p, "params");
        check_dtype(dtype);
        int32_t c = 0;
        int64_t b = 0;
        tape_plan(to_params(p), N, nsteps, dtype, skin,
                  budget_bytes < 0 ? device_budget() : budget_bytes, &c, &b);
        TapeI *t = dtype == SPH_F64 ? make_tape_f64(N, nsteps, c) : make_tape_f32(N, nsteps, c);
        *out = reinterpret_cast<sph_tape>(t);
    });
}

SPH_API int32_t sph_tape_snapshots(sph_tape tp, int32_t *nsnapshots)
{
    return guarded([&] {
        need(tp, "tape");
        need(nsnapshots, "nsnapshots");
        *nsnapshots = TP(tp)->snapshots();
    });
}

SPH_API int32_t sph_tape_destroy(sph_tape tp)
{
    return guarded([&] { delete TP(tp); });
}

SPH_API int32_t sph_tape_reset(sph_tape tp)
{
    return guarded([&] { need(tp, "tape"); TP(tp)->reset(); });
}

SPH_API int32_t sph_tape_length(sph_tape tp, int64_t *n)
{
    return guarded([&] { need(tp, "tape"); need(n, "n"); *n = TP(tp)->length(); });
}

SPH_API int32_t sph_tape_get(sph_tape tp, int64_t n, void *X, void *V)
{
    return guarded([&] { need(tp, "tape"); TP(tp)->get(n, X, V); });
}

SPH_API int32_t sph_tape_recomputed_steps(sph_tape tp, int64_t *n)
{
    return guarded([&] { need(tp, "tape"); need(n, "n"); *n = TP(tp)->forward_steps(); });
}

SPH_API int32_t sph_workspace_create(int64_t N, const sph_params *p, int32_t dtype,
                                     sph_workspace *out)
{
    return guarded([&] {
        need(out, "out");
        check_dtype(dtype);
        const Params q = to_params(p);
        const std::vector<Params> ps{q};
        const std::vector<int64_t> ns{N};
        WorkI *w = dtype == SPH_F64 ? make_work_f64(ps, ns) : make_work_f32(ps, ns);
        *out = reinterpret_cast<sph_workspace>(w);
    });
}

SPH_API int32_t sph_workspace_destroy(sph_workspace ws)
{
    return guarded([&] { delete WS(ws); });
}

SPH_API int32_t sph_backward(sph_workspace ws, sph_tape tp, sph_field theta, const sph_params *p,
                             const void *seedX, const void *seedV, sph_state scratch, double skin,
                             int32_t interval, int32_t maxnb, uint32_t *flags)
{
    return guarded([&] {
        need(ws, "workspace");
        need(tp, "tape");
        need(theta, "theta");
        Params q;
        if (p) q = to_params(p);
        NLOpts o{skin, interval, maxnb};
        if (o.interval < 1 || o.maxnb < 1) throw Error(ERR_ARG, "interval and maxnb must be positive");
        uint32_t f = 0;
        WS(ws)->backward(TP(tp), FD(theta), p ? &q : nullptr, seedX, seedV,
                         scratch ? ST(scratch) : nullptr, o, &f);
        if (flags) *flags = f;
    });
}

SPH_API int32_t sph_autotune(sph_state st, sph_field theta, int32_t reps, int32_t *blocks)
{
    return guarded([&] {
        need(st, "state");
        need(theta, "theta");
        int b[6] = {0, 0, 0, 0, 0, 0};
        ST(st)->autotune(FD(theta), reps, b);
        if (blocks)
            for (int k = 0; k < 6; ++k) blocks[k] = b[k];
    });
}

SPH_API int32_t sph_set_block_sizes(sph_state st, const int32_t *blocks)
{
    return guarded([&] {
        need(st, "state");
        need(blocks, "blocks");
        int b[6];
        for (int k = 0; k < 6; ++k) b[k] = blocks[k];
        ST(st)->set_blocks(b);
    });
}

SPH_API int32_t sph_get_block_sizes(sph_state st, int32_t *blocks)
{
    return guarded([&] {
        need(st, "state");
        need(blocks, "blocks");
        int b[6];
        ST(st)->get_blocks(b);
        for (int k = 0; k < 6; ++k) blocks[k] = b[k];
    });
}

SPH_API int32_t sph_set_density_form(int32_t form)
{
    return guarded([&] {
        if (form < 0 || form > 2) throw Error(ERR_ARG, "density form: 0, 1 or 2");
        rt_set_density_form(form);
    });
}

SPH_API int32_t sph_set_launch_overlap(int32_t on)
{
    return guarded([&] {
        if (on != 0 && on != 1) throw Error(ERR_ARG, "launch overlap: 0 or 1");
        rt_set_launch_overlap(on == 1);
    });
}

SPH_API int32_t sph_set_step_graphs(int32_t steps)
{
    return guarded([&] {
        if (steps < 0) throw Error(ERR_ARG, "steps per recorded group must be >= 0");
        rt_set_step_graph(steps);
    });
}

SPH_API int32_t sph_get_step_graphs(int32_t *steps)
{
    return guarded([&] {
        need(steps, "steps");
        *steps = rt_step_graph();
    });
}

SPH_API int32_t sph_step_graph_counts(int64_t *replays, int64_t *instantiations)
{
    return guarded([&] {
        if (replays) *replays = (int64_t)g_sg_replays.load();
        if (instantiations) *instantiations = (int64_t)g_sg_inst.load();
    });
}

SPH_API int32_t sph_get_density_form(int32_t *form)
{
    return guarded([&] {
        need(form, "form");
        *form = rt_density_form();
    });
}

SPH_API int32_t sph_set_group_lanes(int32_t lanes)
{
    return guarded([&] {
        if (lanes != 0 && lanes != 1 && lanes != 16 && lanes != 32)
            throw Error(ERR_ARG, "lanes per particle must be 0, 1, 16 or 32");
        rt_set_group_lanes(lanes);
    });
}

SPH_API int32_t sph_get_group_lanes(int32_t *lanes)
{
    return guarded([&] {
        need(lanes, "lanes");
        *lanes = rt_group_lanes();
    });
}

SPH_API int32_t sph_state_assign(sph_state dst, sph_state src)
{
    return guarded([&] {
        need(dst, "dst");
        need(src, "src");
        ST(dst)->assign(ST(src));
    });
}

SPH_API int32_t sph_objective(sph_workspace ws, sph_state st, int32_t kind, const double *args,
                              const sph_params *p, double *J)
{
    return guarded([&] {
        need(ws, "workspace");
        need(st, "state");
        Params q;
        if (p) q = to_params(p);
        if (WS(ws)->batch() != 1) throw Error(ERR_ARG, "use sph_batch_objective for a batch");
        double j = 0.0;
        WS(ws)->objective(ST(st), kind, args, p ? &q : nullptr, &j);
        if (J) *J = j;
    });
}

SPH_API int32_t sph_backward_seeded(sph_workspace ws, sph_tape tp, sph_field theta,
                                    const sph_params *p, sph_state scratch, double skin,
                                    int32_t interval, int32_t maxnb, uint32_t *flags)
{
    return guarded([&] {
        need(ws, "workspace");
        need(tp, "tape");
        need(theta, "theta");
        Params q;
        if (p) q = to_params(p);
        NLOpts o{skin, interval, maxnb};
        if (o.interval < 1 || o.maxnb < 1) throw Error(ERR_ARG, "interval and maxnb must be positive");
        uint32_t f = 0;
        WS(ws)->backward_seeded(TP(tp), FD(theta), p ? &q : nullptr,
                                scratch ? ST(scratch) : nullptr, o, &f);
        if (flags) *flags = f;
    });
}

// ---- batches: B independent instances packed into one State/field/workspace ----
static void batch_specs(int32_t B, const sph_params *params, const int64_t *N,
                        std::vector<Params> &ps, std::vector<int64_t> &ns)
{
    if (B < 1) throw Error(ERR_ARG, "batch size must be >= 1");
    need(params, "params");
    need(N, "N");
    for (int32_t b = 0; b < B; ++b) {
        ps.push_back(to_params(params + b));
        ns.push_back(N[b]);
    }
}

SPH_API int32_t sph_batch_create(int32_t B, const sph_params *params, const int64_t *N,
                                 const void *X0, const void *V0, int32_t dtype, double skin,
                                 int32_t interval, int32_t maxnb, sph_state *out)
{
    return guarded([&] {
        need(out, "out");
        check_dtype(dtype);
        std::vector<Params> ps;
        std::vector<int64_t> ns;
        batch_specs(B, params, N, ps, ns);
        NLOpts o{skin, interval, maxnb};
        StateI *s = dtype == SPH_F64 ? make_state_f64(ps, ns, X0, V0, o)
                                     : make_state_f32(ps, ns, X0, V0, o);
        *out = reinterpret_cast<sph_state>(s);
    });
}

SPH_API int32_t sph_batch_field_create(int32_t B, const int32_t *ngx, const int32_t *ngy,
                                       int32_t dtype, const void *theta, sph_field *out)
{
    return guarded([&] {
        need(out, "out");
        need(ngx, "ngx");
        need(ngy, "ngy");
        check_dtype(dtype);
        if (B < 1) throw Error(ERR_ARG, "batch size must be >= 1");
        const std::vector<int> gx(ngx, ngx + B), gy(ngy, ngy + B);
        FieldI *f = dtype == SPH_F64 ? make_field_f64(gx, gy, theta) : make_field_f32(gx, gy, theta);
        *out = reinterpret_cast<sph_field>(f);
    });
}

SPH_API int32_t sph_batch_workspace_create(int32_t B, const sph_params *params, const int64_t *N,
                                           int32_t dtype, sph_workspace *out)
{
    return guarded([&] {
        need(out, "out");
        check_dtype(dtype);
        std::vector<Params> ps;
        std::vector<int64_t> ns;
        batch_specs(B, params, N, ps, ns);
        WorkI *w = dtype == SPH_F64 ? make_work_f64(ps, ns) : make_work_f32(ps, ns);
        *out = reinterpret_cast<sph_workspace>(w);
    });
}

SPH_API int32_t sph_batch_size(sph_state st, int32_t *B)
{
    return guarded([&] {
        need(st, "state");
        need(B, "B");
        *B = ST(st)->batch();
    });
}

SPH_API int32_t sph_batch_take_flags(sph_state st, uint32_t *flags)
{
    return guarded([&] {
        need(st, "state");
        need(flags, "flags");
        ST(st)->take_flags_batch(flags);
    });
}

SPH_API int32_t sph_batch_objective(sph_workspace ws, sph_state st, int32_t kind,
                                    const double *args, double *J)
{
    return guarded([&] {
        need(ws, "workspace");
        need(st, "state");
        WS(ws)->objective(ST(st), kind, args, nullptr, J);
    });
}

SPH_API int32_t sph_workspace_get(sph_workspace ws, void *gX, void *gV, void *gtheta)
{
    return guarded([&] { need(ws, "workspace"); WS(ws)->get(gX, gV, gtheta); });
}

SPH_API int32_t sph_workspace_objective_value(sph_workspace ws, double *J)
{
    return guarded([&] {
        need(ws, "workspace");
        need(J, "J");
        WS(ws)->objective_value(J);
    });
}

SPH_API int32_t sph_workspace_take_flags(sph_workspace ws, uint32_t *flags)
{
    return guarded([&] {
        need(ws, "workspace");
        const uint32_t f = WS(ws)->take_flags();
        if (flags) *flags = f;
    });
}

// ---- captured sequences (CUDA graphs) ----------------------------------------
struct GraphH {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    int64_t nodes = 0;
};

SPH_API int32_t sph_capture_begin(void)
{
    return guarded([&] {
        if (g_capturing) throw Error(ERR_STATE, "this thread is already capturing");
        cuda_check(cudaStreamBeginCapture(rt_stream(), cudaStreamCaptureModeThreadLocal),
                   "cudaStreamBeginCapture");
        g_capturing = true;
    });
}

SPH_API int32_t sph_capture_end(sph_graph *out)
{
    return guarded([&] {
        if (!g_capturing) throw Error(ERR_STATE, "this thread is not capturing");
        g_capturing = false;
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(rt_stream(), &g);
        if (e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            throw Error(ERR_STATE, std::string("the captured sequence is invalid: ") +
                                       cudaGetErrorString(e));
        }
        need(out, "out");
        auto *h = new GraphH();
        h->g = g;
        // count the kernel nodes (the launch counter adds them per replay)
        size_t n = 0;
        (void)cudaGraphGetNodes(g, nullptr, &n);
        std::vector<cudaGraphNode_t> nodes(n);
        if (n) (void)cudaGraphGetNodes(g, nodes.data(), &n);
        for (size_t k = 0; k < n; ++k) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
                h->nodes += 1;
        }
        (void)cudaGetLastError();
        const cudaError_t ei = cudaGraphInstantiate(&h->x, g, 0);
        if (ei != cudaSuccess) {
            cudaGraphDestroy(g);
            delete h;
            cuda_check(ei, "cudaGraphInstantiate");
        }
        *out = reinterpret_cast<sph_graph>(h);
    });
}

SPH_API int32_t sph_graph_launch(sph_graph g)
{
    return guarded([&] {
        need(g, "graph");
        auto *h = reinterpret_cast<GraphH *>(g);
        cuda_check(cudaGraphLaunch(h->x, rt_stream()), "cudaGraphLaunch");
        g_launches.fetch_add(h->nodes, std::memory_order_relaxed);
    });
}

SPH_API int32_t sph_graph_nodes(sph_graph g, int64_t *nodes)
{
    return guarded([&] {
        need(g, "graph");
        need(nodes, "nodes");
        *nodes = reinterpret_cast<GraphH *>(g)->nodes;
    });
}

SPH_API int32_t sph_graph_destroy(sph_graph g)
{
    return guarded([&] {
        if (!g) return;
        auto *h = reinterpret_cast<GraphH *>(g);
        if (h->x) cudaGraphExecDestroy(h->x);
        if (h->g) cudaGraphDestroy(h->g);
        delete h;
    });
}

SPH_API int64_t sph_launch_count(void) { return (int64_t)g_launches.load(); }

SPH_API int32_t sph_profile_enable(int32_t kid, int32_t on)
{
    return guarded([&] {
        if (kid < 0 || kid >= K_COUNT) throw Error(ERR_ARG, "kernel id out of range");
        g_timer[kid].on = on != 0;
    });
}

SPH_API int32_t sph_profile_read(int32_t kid, double *total_ms, int64_t *launches)
{
    return guarded([&] {
        if (kid < 0 || kid >= K_COUNT) throw Error(ERR_ARG, "kernel id out of range");
        KTimer &t = g_timer[kid];
        cuda_check(cudaStreamSynchronize(rt_stream()), "synchronize");
        double ms = 0;
        for (size_t k = 0; k + 1 < t.used; k += 2) {
            float e = 0;
            cuda_check(cudaEventElapsedTime(&e, t.pool[k], t.pool[k + 1]), "cudaEventElapsedTime");
            ms += e;
        }
        if (total_ms) *total_ms = ms;
        if (launches) *launches = t.launches;
    });
}

SPH_API int32_t sph_profile_reset(void)
{
    return guarded([&] {
        for (auto &t : g_timer) {
            t.used = 0;
            t.launches = 0;
        }
    });
}

SPH_API int64_t sph_plan_cost(int64_t l, int64_t c) { return plan_cost(l, c); }
SPH_API int64_t sph_plan_split(int64_t l, int64_t c) { return plan_split(l, c); }

} // extern "C"
