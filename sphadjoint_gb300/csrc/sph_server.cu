// Request servers for forward + adjoint solves (no counterpart in the
// reference: its topology-optimisation driver, scripts/03_optimize.jl:228-254,
// calls simulate!/backward! one solve at a time).
//
// Two ways to run the requests a FIFO queue admits, both admitting the head
// of the queue as soon as its device memory (states, tape or checkpoints,
// workspace) fits in the HBM budget next to the requests already in flight:
//
//   packed (sph_server_create_packed): one scheduler thread and one stream.
//     Every admitted request joins the packed engine (sph_pack.cuh), which
//     advances all requests in flight one step per tick and runs each pass of
//     the tick as one grouped launch over all of them: continuous batching at
//     kernel granularity. A request joins at the next tick after admission and
//     leaves when its program ends.
//   streams (sph_server_create): W worker threads, each running whole solves
//     on its own CUDA stream; requests overlap on the device only through
//     concurrent streams.
//
// Each request runs the same deterministic per-particle arithmetic whatever
// else is in flight, so its result does not depend on the mix.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sphadjoint_gb300.h"
#include "sph_iface.hpp"

namespace sphgb {
namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    int64_t ticket = 0;
    sph_request spec{};
    int64_t bytes = 0;
    Clock::time_point submitted, started, finished;
    int status = 0; // 0 queued, 1 running, 2 done, 3 failed
    double J = 0.0;
    uint32_t flags = 0;
    int32_t err = SPH_OK;
    std::string msg;
};

// Device bytes a request holds while it runs (the admission estimate): two
// States (the solve and the reverse scratch) and a recompute State for
// checkpoint tapes, the adjoint workspace, and the tape itself.
int64_t request_bytes(const sph_request &r, int dtype)
{
    const int64_t s = dtype == SPH_F64 ? 8 : 4;
    const int64_t N = std::max<int64_t>(r.N, 1);
    const int64_t state = N * (12 * s + 64);   // positions, velocities, neighbour masks, ...
    const int64_t work = N * (22 * s + 8);     // gX, gV, abar, gXs, seeds, outputs, ...
    const double rc = 2.0 * r.p.h * (1.0 + r.skin);
    const int64_t cells = (int64_t)((r.p.Lx / rc + 3) * (r.p.Ly / rc + 3));
    const int64_t nodes = (int64_t)r.p.ngx * r.p.ngy;
    int64_t tape;
    if (!r.gX && !r.gV && !r.gtheta)
        return state + work + 8 * cells + 40 * nodes + (16 << 20);   // forward only
    if (r.snapshots > 0)
        tape = (int64_t)r.snapshots * (N * (6 * s + 40) + 4 * cells) + state;
    else
        tape = std::max<int64_t>(r.nsteps, 1) * N * 4 * s;
    return 3 * state + work + tape + 8 * cells + 40 * nodes + (16 << 20);
}

static Params params_of(const sph_params &s)
{
    Params p;
    p.h = s.h; p.m = s.m; p.rho0 = s.rho0; p.c = s.c; p.mu = s.mu;
    p.gx = s.gx; p.gy = s.gy; p.dt = s.dt; p.Lx = s.Lx; p.Ly = s.Ly;
    p.kw = s.kw; p.ngx = s.ngx; p.ngy = s.ngy;
    p.eos = s.eos; p.gamma = s.gamma; p.visc = s.visc; p.alpha = s.alpha;
    return p;
}

// A request's snapshot count when it asks the server to choose (snapshots <
// 0): the full tape when it takes at most an eighth of the budget, else the
// checkpoint snapshots that fit in that eighth.
static int32_t choose_snapshots(const sph_request &r, int dtype, int64_t budget)
{
    if (r.snapshots >= 0) return r.snapshots;
    int32_t c = 0;
    int64_t b = 0;
    tape_plan(params_of(r.p), r.N, r.nsteps, dtype, r.skin, budget / 8, &c, &b);
    return c;
}

class Server {
  public:
    Server(int64_t budget, int dtype) : budget_(budget), dtype_(dtype)
    {
        if (budget <= 0) throw Error(ERR_ARG, "HBM budget must be positive");
        if (dtype != SPH_F64 && dtype != SPH_F32) throw Error(ERR_DTYPE, "bad dtype");
        cuda_check(cudaGetDevice(&device_), "cudaGetDevice");
    }
    virtual ~Server() {}

    // stop and join the threads (every derived destructor calls it first)
    void stop()
    {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_work_.notify_all();
        for (auto &t : threads_) t.join();
        threads_.clear();
    }

    // device bytes a request holds while it runs
    virtual int64_t bytes_of(const sph_request &r) const { return request_bytes(r, dtype_); }

    int64_t submit(const sph_request &r0)
    {
        sph_request r = r0;
        if (r.N < 1 || r.nsteps < 1) throw Error(ERR_ARG, "request needs N >= 1 and nsteps >= 1");
        if (!r.X0 || !r.V0 || !r.theta) throw Error(ERR_ARG, "request inputs are NULL");
        if (r.objective != SPH_OBJ_KE_RIGHT && r.objective != SPH_OBJ_TARGET)
            throw Error(ERR_ARG, "unknown objective");
        if (r.gX || r.gV || r.gtheta) r.snapshots = choose_snapshots(r, dtype_, budget_);
        else r.snapshots = 0;
        auto q = std::make_shared<Req>();
        q->spec = r;
        q->bytes = bytes_of(r);
        if (q->bytes > budget_)
            throw Error(ERR_NOMEM, "request needs ~" + std::to_string(q->bytes >> 20) +
                                       " MiB, more than the whole HBM budget");
        std::lock_guard<std::mutex> g(mu_);
        q->ticket = ++next_;
        q->submitted = Clock::now();
        if (!anySubmitted_) {
            first_ = q->submitted;
            anySubmitted_ = true;
        }
        queue_.push_back(q);
        reqs_[q->ticket] = q;
        cv_work_.notify_all();
        return q->ticket;
    }

    std::shared_ptr<Req> find(int64_t t)
    {
        auto it = reqs_.find(t);
        if (it == reqs_.end()) throw Error(ERR_ARG, "unknown ticket");
        return it->second;
    }

    void wait(int64_t t, double *J, double *lat, uint32_t *flags)
    {
        std::unique_lock<std::mutex> g(mu_);
        auto q = find(t);
        cv_done_.wait(g, [&] { return q->status >= 2; });
        if (q->status == 3) throw Error(q->err, q->msg);
        if (J) *J = q->J;
        if (lat) *lat = std::chrono::duration<double, std::milli>(q->finished - q->submitted).count();
        if (flags) *flags = q->flags;
    }

    int poll(int64_t t)
    {
        std::lock_guard<std::mutex> g(mu_);
        return find(t)->status >= 2 ? 1 : 0;
    }

    void stats(double *p50, double *p99, double *pss, int64_t *done, int64_t *peakBytes,
               int32_t *peakInflight)
    {
        std::lock_guard<std::mutex> g(mu_);
        std::vector<double> lat = lat_;
        std::sort(lat.begin(), lat.end());
        auto pct = [&](double f) {
            if (lat.empty()) return 0.0;
            const double k = f * (lat.size() - 1);
            const size_t a = (size_t)k;
            const size_t b = std::min(a + 1, lat.size() - 1);
            return lat[a] + (lat[b] - lat[a]) * (k - a);
        };
        if (p50) *p50 = pct(0.50);
        if (p99) *p99 = pct(0.99);
        const double span = anyDone_ ? std::chrono::duration<double>(last_ - first_).count() : 0.0;
        if (pss) *pss = span > 0 ? psteps_ / span : 0.0;
        if (done) *done = (int64_t)lat.size();
        if (peakBytes) *peakBytes = peakBytes_;
        if (peakInflight) *peakInflight = peakInflight_;
    }

    void reset_stats()
    {
        std::lock_guard<std::mutex> g(mu_);
        lat_.clear();
        psteps_ = 0;
        anySubmitted_ = anyDone_ = false;
        peakBytes_ = 0;
        peakInflight_ = 0;
        for (auto it = reqs_.begin(); it != reqs_.end();)
            it = it->second->status >= 2 ? reqs_.erase(it) : std::next(it);
    }

  protected:
    void run_streams()
    {
        cudaSetDevice(device_);
        cudaStream_t s = nullptr;
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        rt_set_stream(s);
        for (;;) {
            std::shared_ptr<Req> q;
            {
                std::unique_lock<std::mutex> g(mu_);
                // FIFO admission: the head of the queue starts when its memory
                // fits next to the requests already running
                cv_work_.wait(g, [&] { return stop_ || admissible(); });
                if (stop_) break;
                q = queue_.front();
                queue_.pop_front();
                inflight_ += q->bytes;
                ++running_;
                peakBytes_ = std::max(peakBytes_, inflight_);
                peakInflight_ = std::max(peakInflight_, running_);
                q->status = 1;
                q->started = Clock::now();
            }
            const bool ok = solve(*q);
            {
                std::lock_guard<std::mutex> g(mu_);
                inflight_ -= q->bytes;
                --running_;
                q->finished = Clock::now();
                q->status = ok ? 2 : 3;
                if (ok) {
                    lat_.push_back(
                        std::chrono::duration<double, std::milli>(q->finished - q->submitted).count());
                    psteps_ += (double)q->spec.N * (double)q->spec.nsteps;
                    last_ = q->finished;
                    anyDone_ = true;
                }
            }
            cv_work_.notify_all();
            cv_done_.notify_all();
        }
        rt_set_stream(nullptr);
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }

    // FIFO admission: the head of the queue, when its memory fits next to the
    // requests in flight (and a slot is free)
    bool admissible() const
    {
        return !queue_.empty() && running_ < maxInflight_ &&
               inflight_ + queue_.front()->bytes <= budget_;
    }

    // Runs one request on this worker's stream; results go to the caller's
    // host buffers. Returns false (with q.err / q.msg set) on failure.
    bool solve(Req &q)
    {
        const sph_request &r = q.spec;
        try {
            Params p;
            p.h = r.p.h; p.m = r.p.m; p.rho0 = r.p.rho0; p.c = r.p.c; p.mu = r.p.mu;
            p.gx = r.p.gx; p.gy = r.p.gy; p.dt = r.p.dt; p.Lx = r.p.Lx; p.Ly = r.p.Ly;
            p.kw = r.p.kw; p.ngx = r.p.ngx; p.ngy = r.p.ngy;
            p.eos = r.p.eos; p.gamma = r.p.gamma; p.visc = r.p.visc; p.alpha = r.p.alpha;
            const NLOpts o{r.skin, r.interval, r.maxnb};
            const std::vector<Params> ps{p};
            const std::vector<int64_t> ns{r.N};
            const std::vector<int> gx{p.ngx}, gy{p.ngy};
            const bool f64 = dtype_ == SPH_F64;
            std::unique_ptr<StateI> st(f64 ? make_state_f64(ps, ns, r.X0, r.V0, o)
                                           : make_state_f32(ps, ns, r.X0, r.V0, o));
            std::unique_ptr<FieldI> th(f64 ? make_field_f64(gx, gy, r.theta)
                                           : make_field_f32(gx, gy, r.theta));
            // no output buffers: a forward-only request (no tape, no reverse sweep)
            const bool adjoint = r.gX || r.gV || r.gtheta;
            std::unique_ptr<TapeI> tp;
            if (adjoint)
                tp.reset(f64 ? make_tape_f64(r.N, r.nsteps, r.snapshots)
                             : make_tape_f32(r.N, r.nsteps, r.snapshots));
            std::unique_ptr<WorkI> ws(f64 ? make_work_f64(ps, ns) : make_work_f32(ps, ns));
            st->simulate(th.get(), nullptr, r.nsteps, tp.get());
            uint32_t f = st->take_flags();
            double J = 0.0;
            ws->objective(st.get(), r.objective, r.objective == SPH_OBJ_TARGET ? r.obj_args : nullptr,
                          nullptr, &J);
            uint32_t fb = 0;
            if (adjoint) {
                ws->backward_seeded(tp.get(), th.get(), &p, nullptr, o, &fb);
                ws->get(r.gX, r.gV, r.gtheta);
            }
            q.J = J;
            q.flags = f | fb;
            return true;
        } catch (const Error &e) {
            q.err = e.code;
            q.msg = e.what();
        } catch (const std::exception &e) {
            q.err = ERR_STATE;
            q.msg = e.what();
        }
        (void)cudaStreamSynchronize(rt_stream());
        return false;
    }

    const int64_t budget_;
    const int dtype_;
    int device_ = 0;
    int32_t maxInflight_ = INT32_MAX;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<std::shared_ptr<Req>> queue_;
    std::map<int64_t, std::shared_ptr<Req>> reqs_;
    std::vector<std::thread> threads_;
    bool stop_ = false;
    int64_t next_ = 0;
    int64_t inflight_ = 0, peakBytes_ = 0;
    int32_t running_ = 0, peakInflight_ = 0;
    std::vector<double> lat_;
    double psteps_ = 0;
    bool anySubmitted_ = false, anyDone_ = false;
    Clock::time_point first_, last_;
};

class StreamServer final : public Server {
  public:
    StreamServer(int workers, int64_t budget, int dtype) : Server(budget, dtype)
    {
        if (workers < 1) throw Error(ERR_ARG, "need at least one worker");
        for (int w = 0; w < workers; ++w) threads_.emplace_back([this] { run_streams(); });
    }
    ~StreamServer() override { stop(); }
};

// Device bytes of a request in the packed engine: the solve state (also the
// recompute state), the reverse scratch state, the workspace, the full tape
// or the snapshots, the design field and its accumulators.
int64_t packed_request_bytes(const sph_request &r, int dtype)
{
    const int64_t s = dtype == SPH_F64 ? 8 : 4;
    const int64_t N = std::max<int64_t>(r.N, 1);
    const double rc = 2.0 * r.p.h * (1.0 + r.skin);
    const int64_t cells = (int64_t)((r.p.Lx / rc + 3) * (r.p.Ly / rc + 3));
    const int64_t state = N * (12 * s + 64) + 12 * cells;
    const int64_t work = N * (22 * s + 8);
    const int64_t nodes = (int64_t)r.p.ngx * r.p.ngy;
    const int64_t fixed = 40 * nodes + (4 << 20);
    if (!r.gX && !r.gV && !r.gtheta) return state + work + fixed;
    const int64_t tape = r.snapshots > 0
                             ? (int64_t)r.snapshots * (N * (10 * s + 36) + 4 * cells + 2048)
                             : std::max<int64_t>(r.nsteps, 1) * N * 4 * s;
    return 2 * state + work + tape + fixed;
}

class PackedServer final : public Server {
  public:
    PackedServer(int maxInflight, int64_t budget, int dtype) : Server(budget, dtype)
    {
        if (maxInflight < 1) throw Error(ERR_ARG, "need at least one request in flight");
        // the packed engine's per-tick table holds 64 requests
        maxInflight_ = std::min(maxInflight, 64);
        threads_.emplace_back([this] { run_packed(); });
    }
    ~PackedServer() override { stop(); }
    int64_t bytes_of(const sph_request &r) const override { return packed_request_bytes(r, dtype_); }

  private:
    void fail(Req &q, int code, const std::string &msg)
    {
        std::lock_guard<std::mutex> g(mu_);
        q.err = code;
        q.msg = msg;
        q.status = 3;
        q.finished = Clock::now();
        inflight_ -= q.bytes;
        --running_;
    }

    void run_packed()
    {
        cudaSetDevice(device_);
        cudaStream_t s = nullptr, cs = nullptr;
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        rt_set_stream(s);
        std::unique_ptr<PackI> pack;
        std::map<int, std::shared_ptr<Req>> byId;
        try {
            pack.reset(dtype_ == SPH_F64 ? make_pack_f64() : make_pack_f32());
        } catch (const std::exception &) {
        }
        for (;;) {
            // admission (FIFO, by bytes and slots)
            std::vector<std::shared_ptr<Req>> admit;
            {
                std::unique_lock<std::mutex> g(mu_);
                if (byId.empty())
                    cv_work_.wait(g, [&] { return stop_ || admissible(); });
                if (stop_ && byId.empty()) break;
                while (admissible()) {
                    auto q = queue_.front();
                    queue_.pop_front();
                    inflight_ += q->bytes;
                    ++running_;
                    peakBytes_ = std::max(peakBytes_, inflight_);
                    peakInflight_ = std::max(peakInflight_, running_);
                    q->status = 1;
                    q->started = Clock::now();
                    admit.push_back(q);
                }
            }
            for (auto &q : admit) {
                const sph_request &r = q->spec;
                try {
                    if (!pack) throw Error(ERR_CUDA, "packed engine unavailable");
                    PackReq pr;
                    pr.p = params_of(r.p);
                    pr.N = r.N;
                    pr.X0 = r.X0;
                    pr.V0 = r.V0;
                    pr.theta = r.theta;
                    pr.nsteps = r.nsteps;
                    pr.snapshots = r.snapshots;
                    pr.objective = r.objective;
                    for (int k = 0; k < 3; ++k) pr.obj_args[k] = r.obj_args[k];
                    pr.opts = NLOpts{r.skin, r.interval, r.maxnb};
                    pr.adjoint = r.gX || r.gV || r.gtheta;
                    byId[pack->add(pr)] = q;
                } catch (const Error &e) {
                    fail(*q, e.code, e.what());
                    cv_done_.notify_all();
                } catch (const std::exception &e) {
                    fail(*q, ERR_STATE, e.what());
                    cv_done_.notify_all();
                }
            }
            if (byId.empty()) continue;
            std::vector<int> done;
            try {
                const int stepped = pack->tick();
                pack->reap(done, stepped == 0 && pack->finishing() > 0);
            } catch (const std::exception &e) {
                // a device error ends every request in flight
                (void)cudaStreamSynchronize(s);
                for (auto &kv : byId) {
                    fail(*kv.second, ERR_CUDA, std::string("packed engine: ") + e.what());
                    pack->release(kv.first);
                }
                byId.clear();
                cv_done_.notify_all();
                continue;
            }
            for (int id : done) {
                auto q = byId.at(id);
                double J = 0.0;
                uint32_t f = 0;
                bool ok = true;
                try {
                    pack->result(id, cs, &J, &f, q->spec.gX, q->spec.gV, q->spec.gtheta);
                } catch (const std::exception &e) {
                    fail(*q, ERR_CUDA, e.what());
                    ok = false;
                }
                pack->release(id);
                byId.erase(id);
                if (ok) {
                    std::lock_guard<std::mutex> g(mu_);
                    q->J = J;
                    q->flags = f;
                    q->finished = Clock::now();
                    q->status = 2;
                    inflight_ -= q->bytes;
                    --running_;
                    lat_.push_back(std::chrono::duration<double, std::milli>(q->finished -
                                                                             q->submitted)
                                       .count());
                    psteps_ += (double)q->spec.N * (double)q->spec.nsteps;
                    last_ = q->finished;
                    anyDone_ = true;
                }
            }
            if (!done.empty()) {
                cv_work_.notify_all();
                cv_done_.notify_all();
            }
        }
        pack.reset();
        rt_set_stream(nullptr);
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
        cudaStreamDestroy(cs);
    }
};

template <typename F> int32_t guard(F &&f)
{
    try {
        f();
        return SPH_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return SPH_ERR_STATE;
    }
}

} // namespace
} // namespace sphgb

using namespace sphgb;
#define SV(x) reinterpret_cast<Server *>(x)

extern "C" {

SPH_API int32_t sph_server_create(int32_t workers, int64_t hbm_budget_bytes, int32_t dtype,
                                  sph_server *out)
{
    return guard([&] {
        if (!out) throw Error(ERR_ARG, "out is NULL");
        *out = reinterpret_cast<sph_server>(
            static_cast<Server *>(new StreamServer(workers, hbm_budget_bytes, dtype)));
    });
}

SPH_API int32_t sph_server_create_packed(int32_t max_inflight, int64_t hbm_budget_bytes,
                                         int32_t dtype, sph_server *out)
{
    return guard([&] {
        if (!out) throw Error(ERR_ARG, "out is NULL");
        *out = reinterpret_cast<sph_server>(
            static_cast<Server *>(new PackedServer(max_inflight, hbm_budget_bytes, dtype)));
    });
}

SPH_API int32_t sph_server_destroy(sph_server s)
{
    return guard([&] { delete SV(s); });
}

SPH_API int32_t sph_server_submit(sph_server s, const sph_request *req, int64_t *ticket)
{
    return guard([&] {
        if (!s || !req) throw Error(ERR_ARG, "NULL server or request");
        const int64_t t = SV(s)->submit(*req);
        if (ticket) *ticket = t;
    });
}

SPH_API int32_t sph_server_wait(sph_server s, int64_t ticket, double *J, double *latency_ms,
                                uint32_t *flags)
{
    return guard([&] {
        if (!s) throw Error(ERR_ARG, "NULL server");
        SV(s)->wait(ticket, J, latency_ms, flags);
    });
}

SPH_API int32_t sph_server_poll(sph_server s, int64_t ticket, int32_t *done)
{
    return guard([&] {
        if (!s) throw Error(ERR_ARG, "NULL server");
        const int d = SV(s)->poll(ticket);
        if (done) *done = d;
    });
}

SPH_API int32_t sph_server_stats(sph_server s, double *p50_ms, double *p99_ms,
                                 double *particle_steps_per_s, int64_t *completed,
                                 int64_t *peak_bytes, int32_t *peak_inflight)
{
    return guard([&] {
        if (!s) throw Error(ERR_ARG, "NULL server");
        SV(s)->stats(p50_ms, p99_ms, particle_steps_per_s, completed, peak_bytes, peak_inflight);
    });
}

SPH_API int32_t sph_server_reset_stats(sph_server s)
{
    return guard([&] {
        if (!s) throw Error(ERR_ARG, "NULL server");
        SV(s)->reset_stats();
    });
}

SPH_API int64_t sph_request_bytes(const sph_request *req, int32_t dtype)
{
    return req ? request_bytes(*req, dtype) : 0;
}

} // extern "C"
