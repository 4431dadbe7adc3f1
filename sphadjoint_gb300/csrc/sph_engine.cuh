// Host side of the engine, one instantiation per precision.
//
//   Sys<T>    State: particles in cell order + cell list + neighbour masks
//             (src/driver.jl:5-36, src/neighbors.jl:9-36,150-190)
//   Tape<T>   Tape: full (X, V) history (src/driver.jl:45-83), or a binomial
//             checkpoint tape that keeps a fixed number of snapshots and
//             recomputes the rest during the reverse sweep
//   Work<T>   AdjointWorkspace + backward! (src/driver.jl:117-207)
//   Field<T>  the design field theta on the device
//
// Every public call is enqueued on the library stream; calls that return data
// to the host synchronise, like the reference's synchronize at its API exits.
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <utility>
#include <vector>

#include "sph_coop.cuh"
#include "sph_iface.hpp"
#include "sph_kernels.cuh"

namespace sphgb {

// Device array from the stream-ordered allocator: allocated and freed on the
// stream of the thread that created it, so freeing one request's buffers
// does not synchronise the device under other requests' work.
template <typename T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    bool own = true; // false: a view into a block owned elsewhere
    DevBuf() {}
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n), s(o.s), own(o.own) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            s = o.s;
            own = o.own;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void view(T *ptr, size_t count)
    {
        release();
        p = ptr;
        n = count;
        own = false;
    }
    void alloc(size_t count)
    {
        if (count && rt_capturing())
            throw Error(ERR_STATE, "device allocation while capturing a graph: run the sequence "
                                   "once before capturing it");
        release();
        own = true;
        n = count;
        if (count) {
            s = rt_stream();
            cudaError_t e = rt_malloc((void **)&p, sizeof(T) * count, s);
            if (e != cudaSuccess) {
                p = nullptr;
                n = 0;
                (void)cudaGetLastError();
                throw Error(e == cudaErrorMemoryAllocation ? ERR_NOMEM : ERR_CUDA,
                            std::string("device allocation failed: ") + cudaGetErrorString(e));
            }
        }
    }
    void release()
    {
        if (p && own) rt_free(p, s);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return sizeof(T) * n; }
    void zero() { if (n) SPH_CK(cudaMemsetAsync(p, 0, bytes(), rt_stream())); }
    void copy_from(const DevBuf &o) { if (n) SPH_CK(cudaMemcpyAsync(p, o.p, bytes(), cudaMemcpyDeviceToDevice, rt_stream())); }
};

inline unsigned grid_for(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

// States whose simulate/backward steps go out as recorded groups (graphs):
// every FP64 state and FP32 states of up to 2^18 particles. Measured per
// fwd+adjoint solve, FP32: graphs 58.4 M particle-steps/s against 53.7 with
// programmatic dependent launch at 2k particles, 1360 vs 1061 at 131k, 1771
// vs 1735 at 262k, but 1478 vs 1558 at 1M; FP64: 18.8 vs 13.5 at 2k, 67.9 vs
// 48.5 at 65k.
constexpr int64_t kStepGraphMaxN32 = int64_t(1) << 18;
template <typename T> inline bool step_graph_eligible(int64_t n)
{
    return sizeof(T) == 8 || n <= kStepGraphMaxN32;
}

// Launch on the library stream. Outside graph capture, and unless switched off
// (sph_set_launch_overlap), kernels go out with programmatic dependent launch:
// each may be scheduled while its predecessor still runs and waits on the
// device (pdl_enter) for the predecessor's results, which removes the launch
// gap between the many short kernels of a step.
template <typename... KArgs, typename... Args>
inline void launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, Args &&...args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = rt_stream();
    cudaLaunchAttribute at[1];
    if (rt_launch_overlap() && !rt_capturing()) {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
    }
    cuda_check(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...), "kernel launch");
}

// Threads per block of each tuned kernel, per precision and per single/batched
// variant; 256 until autotune() has measured the candidates on a real state.
template <typename T> int &tuned_block(int kid, bool multi)
{
    static int tab[K_COUNT][2] = {};
    int &b = tab[kid][multi ? 1 : 0];
    if (b == 0) b = kBlock;
    return b;
}

#define SPH_LAUNCH_TUNED(kid, multi, kern, n, ...)                                            \
    do {                                                                                      \
        if ((n) > 0) {                                                                        \
            const int bs_ = ::sphgb::tuned_block<T>(kid, multi);                              \
            ::sphgb::rt_before_launch(kid);                                                   \
            ::sphgb::launch_k(kern, dim3((unsigned)(((n) + bs_ - 1) / bs_)), dim3(bs_), 0, __VA_ARGS__); \
            ::sphgb::rt_after_launch(kid);                                                    \
        }                                                                                     \
    } while (0)

#define SPH_LAUNCH(kid, kern, n, ...)                                                         \
    do {                                                                                      \
        if ((n) > 0) {                                                                        \
            ::sphgb::rt_before_launch(kid);                                                   \
            ::sphgb::launch_k(kern, dim3(::sphgb::grid_for(n)), dim3(::sphgb::kBlock), 0, __VA_ARGS__); \
            ::sphgb::rt_after_launch(kid);                                                    \
        }                                                                                     \
    } while (0)

// Group-per-particle launch: kCoopBlock threads, kCoopBlock / G particles per
// block.
#define SPH_LAUNCH_COOP(kid, G, kern, n, ...)                                                \
    do {                                                                                      \
        if ((n) > 0) {                                                                        \
            const int per_ = ::sphgb::kCoopBlock / (G);                                       \
            ::sphgb::rt_before_launch(kid);                                                   \
            ::sphgb::launch_k(kern, dim3((unsigned)(((n) + per_ - 1) / per_)),                 \
                              dim3(::sphgb::kCoopBlock), 0, __VA_ARGS__);                       \
            ::sphgb::rt_after_launch(kid);                                                    \
        }                                                                                     \
    } while (0)

// Single states up to this many particles use lane groups by default: one
// thread per particle leaves most SMs idle (and, in FP64, bound by the slow
// FP64 pipe on the few SMs it uses). Kernel time per fwd+adjoint step,
// one thread / 16 / 32 lanes:
//   FP64: 240 particles 538 / 112 / 100 us, 1024: 560 / 112 / 123 us,
//         8288: 555 / 346 / 501 us;
//   FP32: 240 particles 99 / 78 / 73 us, 1024: 110 / 81 / 74 us,
//         2072: 115 / 82 / 79 us, 8288: 125 / 107 / 137 us.
// 32 lanes win only for small states, where the critical path of one group
// matters more than the total work.
constexpr int64_t kCoopMaxN = 16384;
template <typename T> constexpr int64_t coop32_max_n() { return sizeof(T) == 8 ? 512 : 2048; }

// Constants formed in T exactly as the reference kernels form them.
template <typename T> Phys<T> make_phys(const Params &q)
{
    Phys<T> p;
    p.h = (T)q.h; p.m = (T)q.m; p.rho0 = (T)q.rho0; p.c = (T)q.c; p.mu = (T)q.mu;
    p.gx = (T)q.gx; p.gy = (T)q.gy; p.dt = (T)q.dt; p.Lx = (T)q.Lx; p.Ly = (T)q.Ly;
    p.kw = (T)q.kw; p.ngx = q.ngx; p.ngy = q.ngy;
    const T pi = (T)3.14159265358979323846;
    p.A = (T)7 / ((T)4 * pi * (p.h * p.h));
    p.invh = (T)1 / p.h;
    p.r2max = (T)4 * p.h * p.h;
    p.Fc = (T)(-5) * p.A * p.invh * p.invh;
    p.Gc = (T)7.5 * p.A * p.invh * p.invh;
    p.twomumass = (T)2 * p.m * p.mu;
    p.c2 = p.c * p.c;
    p.ngx1 = (T)(q.ngx - 1);
    p.ngy1 = (T)(q.ngy - 1);
    p.hxg = p.Lx / p.ngx1;
    p.hyg = p.Ly / p.ngy1;
    p.gxmax = p.ngx1 - (T)1e-6;
    p.gymax = p.ngy1 - (T)1e-6;
    // model variants: Tait B = c^2 rho0 / gamma, dB = B gamma / rho0;
    // artificial viscosity avc = m alpha c h, eh2 = 0.01 h^2
    p.eos = q.eos;
    p.gam = q.gamma;
    p.visc = q.visc;
    const T gam = (T)(q.eos == 1 ? q.gamma : 1);
    p.B = p.c2 * p.rho0 / gam;
    p.dB = p.B * gam / p.rho0;
    p.avc = p.m * (T)q.alpha * p.c * p.h;
    p.eh2 = (T)0.01 * p.h * p.h;
    return p;
}

inline void check_params(const Params &p)
{
    if (!(p.h > 0)) throw Error(ERR_ARG, "h must be positive");
    if (p.ngx < 2 || p.ngy < 2) throw Error(ERR_ARG, "ngx and ngy must be at least 2");
    if (p.eos != 0 && p.eos != 1) throw Error(ERR_ARG, "eos must be 0 (linear) or 1 (Tait)");
    if (p.eos == 1 && (p.gamma < 1 || p.gamma > 15))
        throw Error(ERR_ARG, "Tait exponent gamma must be an integer in [1, 15]");
    if (p.visc != 0 && p.visc != 1)
        throw Error(ERR_ARG, "visc must be 0 (Morris) or 1 (artificial viscosity)");
    if (p.visc == 1 && !(p.alpha >= 0)) throw Error(ERR_ARG, "alpha must be >= 0");
}

// the model reads per-particle densities (Tait derivative, viscosity average)
inline bool needs_rho(const Params &p) { return p.eos == 1 || p.visc == 1; }

// exclusive scan of n int32 -> out[0..n] (+ optional copy); tmp >= blocks
inline void scan_excl(const int32_t *in, int64_t n, int32_t *out, int32_t *out2, int32_t *tmp)
{
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb <= 1) {
        rt_before_launch(K_SCAN);
        launch_k(k_scan_down, dim3(1), dim3(kBlock), 0, in, n, (const int32_t *)nullptr, out, out2);
        rt_after_launch(K_SCAN);
        return;
    }
    rt_before_launch(K_SCAN);
    launch_k(k_scan_reduce, dim3((unsigned)nb), dim3(kBlock), 0, in, n, tmp);
    launch_k(k_scan_top, dim3(1), dim3(1024), 0, tmp, nb);
    launch_k(k_scan_down, dim3((unsigned)nb), dim3(kBlock), 0, in, n, (const int32_t *)tmp, out, out2);
    rt_after_launch(K_SCAN);
}

// The design field theta of one instance, or the packed fields of a batch
// (instance b's (ngy, ngx) column-major block at node offset off[b]).
template <typename T> class Field final : public FieldI {
  public:
    std::vector<int> gx, gy;
    std::vector<int64_t> off;
    int nx_, ny_; // shape of instance 0
    DevBuf<T> th;
    Field(const std::vector<int> &ngx, const std::vector<int> &ngy, const void *host)
        : gx(ngx), gy(ngy)
    {
        if (gx.empty() || gx.size() != gy.size()) throw Error(ERR_ARG, "empty theta batch");
        int64_t tot = 0;
        for (size_t b = 0; b < gx.size(); ++b) {
            if (gx[b] < 2 || gy[b] < 2) throw Error(ERR_ARG, "theta must be at least 2 x 2");
            off.push_back(tot);
            tot += (int64_t)gx[b] * gy[b];
        }
        nx_ = gx[0];
        ny_ = gy[0];
        th.alloc((size_t)tot);
        if (host) upload(host); else th.zero();
    }
    int batch() const { return (int)gx.size(); }
    int dtype() const override { return sizeof(T) == 8 ? F64 : F32; }
    int ngx() const override { return nx_; }
    int ngy() const override { return ny_; }
    void upload(const void *host) override
    {
        SPH_CK(cudaMemcpyAsync(th.p, host, th.bytes(), cudaMemcpyHostToDevice, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
    }
    void upload_device(const void *dev) override
    {
        SPH_CK(cudaMemcpyAsync(th.p, dev, th.bytes(), cudaMemcpyDeviceToDevice, rt_stream()));
    }
};

// A copy of everything that determines the future of a Sys: the state in
// cell order, its permutation, and the neighbour structure of the last
// rebuild (so recomputation from a snapshot repeats the forward bit for bit).
// The arrays are one contiguous block (Sys::core), so a snapshot is a single
// device-to-device copy.
template <typename T> struct Snap {
    DevBuf<uint8_t> blob;
    int64_t age = INT64_MAX;
    int cur = 0;
    bool valid = false;
};

template <typename T> class Sys final : public StateI {
  public:
    Params prm;                 // parameters of instance 0 (the State's p)
    std::vector<Params> prms;   // per instance
    std::vector<Inst<T>> hinst; // instance table (host copy)
    DevBuf<Inst<T>> dinst;      // instance table (device)
    DevBuf<uint16_t> pinst;     // instance of each slot (batches only)
    int B = 1;
    int64_t N_;
    int nx, ny;                 // grid of instance 0
    int64_t ncell;              // cells of all instances
    int64_t nnode = 0;          // design nodes of all instances
    double cs_d, rc_d, dmax_d;  // instance 0
    NLOpts opts;
    int64_t age = INT64_MAX;
    DevBuf<uint8_t> core; // one block holding every array a snapshot must keep
    DevBuf<T2<T>> pos[2], vel[2];
    int cur = 0;
    DevBuf<T2<T>> xref;
    DevBuf<int32_t> perm, invperm, cellStart, nbcount, cellTmp, counts, cursor, bucketSrc,
        bucketId, scanTmp;
    DevBuf<uint32_t> center, flags;
    DevBuf<uint32_t> masks;  // 6 words per particle, word-major
    DevBuf<uint32_t> tmask;  // this step's in-support words (written by the density pass)
    DevBuf<T> rho;
    DevBuf<T2<T>> prho;
    DevBuf<T2<T>> accOut;
    DevBuf<T> alphaOut;
    DevBuf<T2<T>> stage2;
    DevBuf<T> stage1;
    DevBuf<int32_t> clStart, clOrder; // build! without a neighbour rebuild
    bool cellsOnlyLatest = false;
    bool keepAccel = false;
    StepGraphs graphs;   // simulate's steps, replayed in groups
    bool anyRho = false; // some instance's model reads densities in the adjoint
    bool anyAV = false;  // some instance uses the artificial viscosity

    Sys(const Params &p, int64_t N, const void *X0, const void *V0, NLOpts o)
        : Sys(std::vector<Params>{p}, std::vector<int64_t>{N}, X0, V0, o)
    {
    }

    // NeighborList / CellList constants of one instance (src/neighbors.jl:28-36,
    // 174-190): rc = Float64(support(p)) * (1 + skin), cs = rc, nx =
    // ceil(Lx / cs) + 2, dmax = Float64(h) * skin, r2min = eps(T) h h.
    static Inst<T> make_inst(const Params &p, const NLOpts &o, int64_t off, int64_t n,
                             int64_t coff, int64_t toff)
    {
        check_params(p);
        Inst<T> I;
        std::memset(&I, 0, sizeof(I));
        I.p = make_phys<T>(p);
        const T hT = (T)p.h;
        const T support = (T)2 * hT;
        const double rc = (double)support * (1.0 + o.skin);
        const double dmax = (double)hT * o.skin;
        const double LxT = (double)(T)p.Lx, LyT = (double)(T)p.Ly;
        const double nxd = std::max(1.0, std::ceil(LxT / rc) + 2);
        const double nyd = std::max(1.0, std::ceil(LyT / rc) + 2);
        if (!(rc > 0) || !(nxd <= 65535) || !(nyd <= 32767))
            throw Error(ERR_ARG, "cell grid too large (nx <= 65535, ny <= 32767)");
        I.off = (int)off;
        I.n = (int)n;
        I.nx = (int)nxd;
        I.ny = (int)nyd;
        I.coff = (int)coff;
        I.toff = (int)toff;
        I.maxnb = o.maxnb;
        int lg = 0;
        while (((int64_t)1 << lg) < n + 1 && lg < 62) ++lg;
        I.lgN = lg;
        I.cs = (T)rc;
        I.invcs = (T)1 / I.cs;
        I.rc2 = (T)(rc * rc);
        I.r2min = std::numeric_limits<T>::epsilon() * hT * hT;
        I.dmax2 = (T)(dmax * dmax);
        return I;
    }

    Sys(const std::vector<Params> &ps, const std::vector<int64_t> &ns, const void *X0,
        const void *V0, NLOpts o)
        : prm(ps.at(0)), prms(ps), N_(0), opts(o)
    {
        if (ps.empty() || ps.size() != ns.size()) throw Error(ERR_ARG, "empty instance list");
        if (ps.size() > 65535) throw Error(ERR_ARG, "at most 65535 instances per batch");
        if (o.maxnb < 1) throw Error(ERR_ARG, "maxnb must be positive");
        if (o.interval < 1) throw Error(ERR_ARG, "interval must be positive");
        B = (int)ps.size();
        int64_t off = 0, coff = 0, toff = 0;
        for (int b = 0; b < B; ++b) {
            if (ns[b] < 0) throw Error(ERR_ARG, "particle count out of range");
            Inst<T> I = make_inst(ps[b], o, off, ns[b], coff, toff);
            hinst.push_back(I);
            off += ns[b];
            coff += (int64_t)I.nx * I.ny;
            toff += (int64_t)ps[b].ngx * ps[b].ngy;
            if (off > (int64_t)INT32_MAX - 1 || coff > (int64_t)INT32_MAX - 1 ||
                toff > (int64_t)INT32_MAX - 1)
                throw Error(ERR_ARG, "batch too large for 32-bit slot, cell or node indices");
        }
        N_ = off;
        ncell = coff;
        nnode = toff;
        for (const Params &q : ps) {
            anyRho = anyRho || needs_rho(q);
            anyAV = anyAV || q.visc == 1;
        }
        nx = hinst[0].nx;
        ny = hinst[0].ny;
        {
            const T hT = (T)prm.h;
            rc_d = (double)((T)2 * hT) * (1.0 + o.skin);
            cs_d = rc_d;
            dmax_d = (double)hT * o.skin;
        }
        dinst.alloc((size_t)B);
        upload_inst();
        const int64_t N = N_;
        const size_t n1 = (size_t)std::max<int64_t>(N, 1);
        if (B > 1) {
            std::vector<uint16_t> pi(n1, 0);
            for (int b = 0; b < B; ++b)
                for (int64_t k = 0; k < ns[b]; ++k) pi[hinst[b].off + k] = (uint16_t)b;
            pinst.alloc(n1);
            SPH_CK(cudaMemcpyAsync(pinst.p, pi.data(), sizeof(uint16_t) * n1, cudaMemcpyHostToDevice, rt_stream()));
            SPH_CK(cudaStreamSynchronize(rt_stream()));
        }
        {
            // the state that determines the future, in one block: positions and
            // velocities (both buffers), rebuild positions, permutation, cell
            // table, cell centres and neighbour masks
            size_t off = 0;
            auto carve = [&](size_t bytes) {
                const size_t o = off;
                off += (bytes + 255) & ~(size_t)255;
                return o;
            };
            const size_t oPos0 = carve(sizeof(T2<T>) * n1), oPos1 = carve(sizeof(T2<T>) * n1);
            const size_t oVel0 = carve(sizeof(T2<T>) * n1), oVel1 = carve(sizeof(T2<T>) * n1);
            const size_t oXref = carve(sizeof(T2<T>) * n1);
            const size_t oPerm = carve(4 * n1), oInv = carve(4 * n1), oCtr = carve(4 * n1);
            const size_t oMask = carve(4 * 6 * n1);
            const size_t oCell = carve(4 * ((size_t)ncell + 1));
            core.alloc(off);
            uint8_t *c = core.p;
            pos[0].view((T2<T> *)(c + oPos0), n1);
            pos[1].view((T2<T> *)(c + oPos1), n1);
            vel[0].view((T2<T> *)(c + oVel0), n1);
            vel[1].view((T2<T> *)(c + oVel1), n1);
            xref.view((T2<T> *)(c + oXref), n1);
            perm.view((int32_t *)(c + oPerm), n1);
            invperm.view((int32_t *)(c + oInv), n1);
            center.view((uint32_t *)(c + oCtr), n1);
            masks.view((uint32_t *)(c + oMask), 6 * n1);
            cellStart.view((int32_t *)(c + oCell), (size_t)ncell + 1);
        }
        nbcount.alloc(n1);
        cellTmp.alloc(n1);
        counts.alloc((size_t)ncell);
        cursor.alloc((size_t)ncell);
        bucketSrc.alloc(n1);
        bucketId.alloc(n1);
        scanTmp.alloc((size_t)((ncell + kScanTile - 1) / kScanTile + 1));
        flags.alloc((size_t)B);
        tmask.alloc(6 * n1);
        rho.alloc(n1);
        prho.alloc(n1);
        stage2.alloc(n1);
        stage1.alloc(n1);
        flags.zero();
        xref.zero();
        masks.zero();
        center.zero();
        cellStart.zero();
        if (sizeof(T) == 4) {
            // the one-launch cell list of small FP32 states (set here, outside
            // any graph recording)
            static bool attr = false;
            if (!attr) {
                SPH_CK(cudaFuncSetAttribute(k_rebuild_small<T>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)(sizeof(int32_t) * (2 * kRebuildSmallMaxCells + 1 +
                                                                     3 * kRebuildSmallMaxN))));
                attr = true;
            }
        }
        init_identity();
        if (X0 || V0) set(X0, V0);
        else {
            pos[0].zero();
            vel[0].zero();
        }
    }

    int dtype() const override { return sizeof(T) == 8 ? F64 : F32; }
    int64_t N() const override { return N_; }
    int batch() const override { return B; }

    // lanes per particle of this state's pair-sum kernels (0: one thread)
    int group_lanes() const
    {
        if (B != 1) return 0;
        const int f = rt_group_lanes();
        if (f == 16 || f == 32) return f;
        if (f == 1 || N_ > kCoopMaxN) return 0;
        return N_ <= coop32_max_n<T>() ? 32 : 16;
    }

    void upload_inst()
    {
        SPH_CK(cudaMemcpyAsync(dinst.p, hinst.data(), sizeof(Inst<T>) * B, cudaMemcpyHostToDevice, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
    }

    // A call may pass its own SPHParams (the reference's kernels take p per
    // call): the physics constants follow it, the grid and neighbour-list
    // constants stay those of construction, as in the reference.
    void use_params(const Params *p)
    {
        if (!p) return;
        if (B != 1) throw Error(ERR_ARG, "a batch uses its per-instance parameters (pass NULL)");
        check_params(*p);
        if (std::memcmp(p, &prm, sizeof(Params)) == 0) return;
        if (p->ngx != prm.ngx || p->ngy != prm.ngy)
            throw Error(ERR_ARG, "params (ngx, ngy) differ from the state's");
        prm = *p;
        prms[0] = *p;
        hinst[0].p = make_phys<T>(*p);
        anyRho = needs_rho(*p);
        anyAV = p->visc == 1;
        upload_inst();
    }

    void init_identity()
    {
        std::vector<int32_t> id((size_t)std::max<int64_t>(N_, 1));
        for (int64_t i = 0; i < N_; ++i) id[i] = (int32_t)i;
        if (N_) {
            SPH_CK(cudaMemcpyAsync(perm.p, id.data(), sizeof(int32_t) * N_, cudaMemcpyHostToDevice, rt_stream()));
            SPH_CK(cudaMemcpyAsync(invperm.p, id.data(), sizeof(int32_t) * N_, cudaMemcpyHostToDevice, rt_stream()));
            SPH_CK(cudaStreamSynchronize(rt_stream()));
        }
    }

    NLView<T> view() const
    {
        NLView<T> v;
        v.N = N_;
        v.pos = pos[cur].p;
        v.xref = xref.p;
        v.center = center.p;
        v.masks = masks.p;
        v.tmask = nullptr;
        v.cellStart = cellStart.p;
        v.inst = dinst.p;
        v.pinst = pinst.p;
        v.one = hinst[0];
        return v;
    }

    // host (id order, interleaved T) -> cell order
    void set(const void *X, const void *V) override
    {
        if (!N_) return;
        if (X) {
            SPH_CK(cudaMemcpyAsync(stage2.p, X, stage2.bytes(), cudaMemcpyHostToDevice, rt_stream()));
            SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N_, N_, perm.p, stage2.p, pos[cur].p);
        }
        if (V) {
            SPH_CK(cudaMemcpyAsync(stage2.p, V, stage2.bytes(), cudaMemcpyHostToDevice, rt_stream()));
            SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N_, N_, perm.p, stage2.p, vel[cur].p);
        }
        SPH_CK(cudaStreamSynchronize(rt_stream()));
    }

    void get(void *X, void *V) override
    {
        if (!N_) return;
        if (X) {
            SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N_, N_, perm.p, pos[cur].p, stage2.p);
            SPH_CK(cudaMemcpyAsync(X, stage2.p, stage2.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
            SPH_CK(cudaStreamSynchronize(rt_stream()));
        }
        if (V) {
            SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N_, N_, perm.p, vel[cur].p, stage2.p);
            SPH_CK(cudaMemcpyAsync(V, stage2.p, stage2.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
            SPH_CK(cudaStreamSynchronize(rt_stream()));
        }
    }

    void get1(const T *src, void *out)
    {
        SPH_LAUNCH(K_MISC, k_scatter_to_ids1<T>, N_, N_, perm.p, src, stage1.p);
        SPH_CK(cudaMemcpyAsync(out, stage1.p, stage1.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
    }

    void fields(void *rhoOut, void *ptermOut, void *invrhoOut, void *aOut, void *alOut) override
    {
        if (!N_) return;
        if (rhoOut) get1(rho.p, rhoOut);
        if (ptermOut || invrhoOut) {
            std::vector<T> tmp(2 * (size_t)N_);
            SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N_, N_, perm.p, prho.p, stage2.p);
            SPH_CK(cudaMemcpyAsync(tmp.data(), stage2.p, stage2.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
            SPH_CK(cudaStreamSynchronize(rt_stream()));
            for (int64_t i = 0; i < N_; ++i) {
                if (ptermOut) ((T *)ptermOut)[i] = tmp[2 * i];
                if (invrhoOut) ((T *)invrhoOut)[i] = tmp[2 * i + 1];
            }
        }
        if (aOut) {
            if (!accOut.p) throw Error(ERR_STATE, "accelerations are kept only after keep_accel(1)");
            SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N_, N_, perm.p, accOut.p, stage2.p);
            SPH_CK(cudaMemcpyAsync(aOut, stage2.p, stage2.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
            SPH_CK(cudaStreamSynchronize(rt_stream()));
        }
        if (alOut) {
            if (!alphaOut.p) throw Error(ERR_STATE, "alpha is kept only after keep_accel(1)");
            get1(alphaOut.p, alOut);
        }
    }

    void keep_accel(bool on) override
    {
        keepAccel = on;
        if (on && !accOut.p) {
            accOut.alloc((size_t)std::max<int64_t>(N_, 1));
            alphaOut.alloc((size_t)std::max<int64_t>(N_, 1));
            accOut.zero();
            alphaOut.zero();
        }
    }

    // build_neighbors! (src/neighbors.jl:252-263): cell list, permutation of
    // the particle data (and of up to two extra per-particle arrays) into the
    // new cell order, neighbour masks. ex*N receive the permuted extras.
    void rebuild(const T2<T> *ex0 = nullptr, T2<T> *ex0N = nullptr, const T2<T> *ex1 = nullptr,
                 T2<T> *ex1N = nullptr)
    {
        const int check = age != INT64_MAX ? 1 : 0;
        if (sizeof(T) == 4 && N_ > 0 && B == 1 && N_ <= kRebuildSmallMaxN &&
            ncell <= kRebuildSmallMaxCells) {
            // small single FP32 state: the cell list in one launch (the
            // reference's GPU optimisation set-up, 1500 particles, runs 12%
            // faster; in FP64 the one block's double-precision cell
            // coordinates cost more than the launches saved)
            const int nxt = 1 - cur;
            const size_t smem = sizeof(int32_t) * (size_t)(2 * ncell + 1 + 3 * N_);
            rt_before_launch(K_RANK);
            launch_k(k_rebuild_small<T>, dim3(1), dim3(kRebuildSmallThreads), smem, (int)N_,
                     (int)ncell, hinst[0], check, (const T2<T> *)pos[cur].p,
                     (const T2<T> *)vel[cur].p, pos[nxt].p, vel[nxt].p, xref.p, perm.p,
                     invperm.p, cellStart.p, ex0, ex0N, ex1, ex1N, flags.p);
            rt_after_launch(K_RANK);
            cur = nxt;
            build_masks();
        } else if (N_ > 0) {
            counts.zero();
            auto ka = B > 1 ? &k_assign<T, true> : &k_assign<T, false>;
            SPH_LAUNCH(K_ASSIGN, ka, N_, N_, pos[cur].p, xref.p, check, hinst[0], dinst.p, pinst.p,
                       cellTmp.p, counts.p, flags.p);
            scan_excl(counts.p, ncell, cellStart.p, cursor.p, scanTmp.p);
            SPH_LAUNCH(K_BUCKET, k_bucket, N_, N_, cellTmp.p, perm.p, cursor.p, bucketSrc.p, bucketId.p);
            const int nxt = 1 - cur;
            SPH_LAUNCH(K_RANK, k_rank_permute<T>, N_, N_, cellTmp.p, cellStart.p, bucketSrc.p,
                       bucketId.p, pos[cur].p, vel[cur].p, pos[nxt].p, vel[nxt].p, xref.p, perm.p,
                       invperm.p, ex0, ex0N, ex1, ex1N);
            cur = nxt;
            build_masks();
        }
        age = 0;
        cellsOnlyLatest = false;
    }

    // _nl_build! on the freshly sorted particles
    void build_masks()
    {
        if (const int G = group_lanes()) {
            auto kn = G == 32 ? &k_nl_build_coop<T, 32> : &k_nl_build_coop<T, 16>;
            SPH_LAUNCH_COOP(K_NLBUILD, G, kn, N_, N_, hinst[0], pos[cur].p, cellStart.p,
                            center.p, masks.p, nbcount.p, flags.p);
        } else {
            auto kn = B > 1 ? &k_nl_build<T, true> : &k_nl_build<T, false>;
            SPH_LAUNCH_TUNED(K_NLBUILD, B > 1, kn, N_, N_, hinst[0], dinst.p, pinst.p,
                             pos[cur].p, cellStart.p, center.p, masks.p, nbcount.p, flags.p);
        }
    }

    void build_neighbors() override
    {
        rebuild();
        rt_check_launch("build_neighbors");
    }

    // build! alone (src/neighbors.jl:97-114): the cell list of the current
    // positions, without touching the particle order or the neighbour list.
    void build_cells() override
    {
        if (!clStart.p) {
            clStart.alloc((size_t)ncell + 1);
            clOrder.alloc((size_t)std::max<int64_t>(N_, 1));
        }
        if (N_ > 0) {
            counts.zero();
            auto ka = B > 1 ? &k_assign<T, true> : &k_assign<T, false>;
            SPH_LAUNCH(K_ASSIGN, ka, N_, N_, pos[cur].p, xref.p, 0, hinst[0], dinst.p, pinst.p,
                       cellTmp.p, counts.p, flags.p);
            scan_excl(counts.p, ncell, clStart.p, cursor.p, scanTmp.p);
            SPH_LAUNCH(K_BUCKET, k_bucket, N_, N_, cellTmp.p, perm.p, cursor.p, bucketSrc.p, bucketId.p);
            SPH_LAUNCH(K_RANK, k_rank_permute<T>, N_, N_, cellTmp.p, clStart.p, bucketSrc.p,
                       bucketId.p, pos[cur].p, vel[cur].p, (T2<T> *)nullptr, (T2<T> *)nullptr,
                       (T2<T> *)nullptr, clOrder.p, (int32_t *)nullptr, (const T2<T> *)nullptr,
                       (T2<T> *)nullptr, (const T2<T> *)nullptr, (T2<T> *)nullptr);
        } else {
            clStart.zero();
        }
        cellsOnlyLatest = true;
        rt_check_launch("build_cells");
    }

    void maybe_rebuild(const T2<T> *ex0 = nullptr, T2<T> *ex0N = nullptr,
                       const T2<T> *ex1 = nullptr, T2<T> *ex1N = nullptr, bool *did = nullptr)
    {
        // maybe_rebuild! (src/neighbors.jl:273-279): test, then count
        bool r = false;
        if (age >= opts.interval) {
            rebuild(ex0, ex0N, ex1, ex1N);
            r = true;
        }
        age += 1;
        if (did) *did = r;
    }

    // step! (src/forward.jl:161-173); tx/tv: optional tape slot (id order)
    void step_impl(const T *theta, T2<T> *tx, T2<T> *tv)
    {
        maybe_rebuild();
        if (N_ == 0) return;
        // the tape slot (tx, tv) is written by the accel pass from the same
        // pre-step state it reads
        NLView<T> v = view();
        const int nxt = 1 - cur;
        T2<T> *aO = keepAccel ? accOut.p : (T2<T> *)nullptr;
        T *alO = keepAccel ? alphaOut.p : (T *)nullptr;
        if (const int G = group_lanes()) {
            auto kd = G == 32 ? &k_density_eos_coop<T, 32> : &k_density_eos_coop<T, 16>;
            SPH_LAUNCH_COOP(K_DENSITY, G, kd, N_, v, rho.p, prho.p, tmask.p);
            v.tmask = tmask.p;
            auto ki = G == 32 ? &k_accel_integrate_coop<T, 32> : &k_accel_integrate_coop<T, 16>;
            SPH_LAUNCH_COOP(K_ACCEL_INTEGRATE, G, ki, N_, v, vel[cur].p, prho.p, rho.p, theta,
                            pos[nxt].p, vel[nxt].p, aO, alO, flags.p, perm.p, tx, tv);
        } else {
            launch_density(v, rho.p, prho.p);
            v.tmask = tmask.p;
            auto ki = B > 1 ? (anyAV ? &k_accel_integrate<T, true, true> : &k_accel_integrate<T, true>)
                            : (anyAV ? &k_accel_integrate<T, false, true> : &k_accel_integrate<T, false>);
            SPH_LAUNCH_TUNED(K_ACCEL_INTEGRATE, B > 1, ki, N_, v, vel[cur].p, prho.p, rho.p,
                             theta, pos[nxt].p, vel[nxt].p, aO, alO, flags.p, perm.p, tx, tv);
        }
        cur = nxt;
    }

    // density_kernel! + eos_kernel! with one thread per particle: the mask
    // walk, or for FP32 states the forms sph_set_density_form selects
    void launch_density(const NLView<T> &v, T *rhoOut, T2<T> *prhoOut)
    {
        const int form = sizeof(T) == 4 ? rt_density_form() : 0;
        if (form == 2) {
            auto kd = B > 1 ? &k_density_eos<T, true, true> : &k_density_eos<T, false, true>;
            SPH_LAUNCH_TUNED(K_DENSITY, B > 1, kd, N_, v, rhoOut, prhoOut, tmask.p);
            return;
        }
        if (form == 1 && B == 1) {
            const int bs = 32 * kTileWarps;
            rt_before_launch(K_DENSITY);
            launch_k(k_density_tile<T>, dim3((unsigned)((N_ + bs - 1) / bs)), dim3(bs), 0, v,
                     rhoOut, prhoOut, tmask.p);
            rt_after_launch(K_DENSITY);
            return;
        }
        auto kd = B > 1 ? &k_density_eos<T, true> : &k_density_eos<T, false>;
        SPH_LAUNCH_TUNED(K_DENSITY, B > 1, kd, N_, v, rhoOut, prhoOut, tmask.p);
    }

    // theta must hold one (ngy, ngx) block per instance, in instance order
    Field<T> *field_of(FieldI *f)
    {
        auto *t = dynamic_cast<Field<T> *>(f);
        if (!t) throw Error(ERR_DTYPE, "theta has a different precision than the state");
        if (t->batch() != B) throw Error(ERR_ARG, "theta has a different number of instances");
        for (int b = 0; b < B; ++b)
            if (t->gx[b] != prms[b].ngx || t->gy[b] != prms[b].ngy ||
                t->off[b] != hinst[b].toff)
                throw Error(ERR_ARG, "params (ngx, ngy) do not match the theta field");
        return t;
    }

    void step(FieldI *theta, const Params *p) override
    {
        use_params(p);
        Field<T> *th = field_of(theta);
        step_impl(th->th.p, nullptr, nullptr);
        rt_check_launch("step");
    }

    void simulate(FieldI *theta, const Params *p, int64_t nsteps, TapeI *tape) override;
    void autotune(FieldI *theta, int reps, int *chosen) override;
    static constexpr int kTunedIds[6] = {K_NLBUILD, K_DENSITY, K_ACCEL_INTEGRATE,
                                         K_ACCEL_DRAG, K_PASS1, K_PASS2};
    void set_blocks(const int *blocks) override
    {
        for (int k = 0; k < 6; ++k)
            if (blocks[k] != 64 && blocks[k] != 128 && blocks[k] != 256)
                throw Error(ERR_ARG, "block sizes must be 64, 128 or 256");
        for (int k = 0; k < 6; ++k) tuned_block<T>(kTunedIds[k], B > 1) = blocks[k];
    }
    void get_blocks(int *blocks) const override
    {
        for (int k = 0; k < 6; ++k) blocks[k] = tuned_block<T>(kTunedIds[k], B > 1);
    }

    void celllist(int32_t *countsOut, int32_t *startsOut, int32_t *orderOut) override
    {
        if (B != 1) throw Error(ERR_ARG, "cell lists are read per State (batch of one)");
        const int32_t *cst = cellsOnlyLatest ? clStart.p : cellStart.p;
        const int32_t *ord = cellsOnlyLatest ? clOrder.p : perm.p;
        std::vector<int32_t> s((size_t)ncell + 1);
        SPH_CK(cudaMemcpyAsync(s.data(), cst, sizeof(int32_t) * (ncell + 1), cudaMemcpyDeviceToHost, rt_stream()));
        std::vector<int32_t> o((size_t)std::max<int64_t>(N_, 1));
        if (N_) SPH_CK(cudaMemcpyAsync(o.data(), ord, sizeof(int32_t) * N_, cudaMemcpyDeviceToHost, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
        if (N_ == 0) std::fill(s.begin(), s.end(), 0);
        for (int64_t c = 0; c < ncell; ++c) {
            if (countsOut) countsOut[c] = s[c + 1] - s[c];
            if (startsOut) startsOut[c] = s[c];
        }
        if (orderOut)
            for (int64_t i = 0; i < N_; ++i) orderOut[i] = o[i] + 1; // 1-based ids
    }

    void neighbors(int32_t *indices, int32_t *nbc) override;

    // per-instance flags (read and cleared); returns their union
    uint32_t take_flags_all(uint32_t *per)
    {
        std::vector<uint32_t> f((size_t)B);
        SPH_CK(cudaMemcpyAsync(f.data(), flags.p, sizeof(uint32_t) * B, cudaMemcpyDeviceToHost, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
        flags.zero();
        uint32_t u = 0;
        for (int b = 0; b < B; ++b) {
            u |= f[b];
            if (per) per[b] = f[b];
        }
        return u;
    }
    uint32_t take_flags() override { return take_flags_all(nullptr); }
    void take_flags_batch(uint32_t *per) override { take_flags_all(per); }

    void grid(int32_t *nxo, int32_t *nyo, double *cso, int64_t *ageo) const override
    {
        if (nxo) *nxo = nx;
        if (nyo) *nyo = ny;
        if (cso) *cso = cs_d;
        if (ageo) *ageo = age;
    }

    void sync() override { SPH_CK(cudaStreamSynchronize(rt_stream())); }

    // ---- snapshots ----
    void reserve(Snap<T> &s)
    {
        if (!s.blob.p) s.blob.alloc(core.n);
    }
    void save(Snap<T> &s)
    {
        reserve(s);
        s.blob.copy_from(core);
        s.age = age;
        s.cur = cur;
        s.valid = true;
    }
    void restore(const Snap<T> &s)
    {
        if (!s.valid) throw Error(ERR_STATE, "restoring an empty snapshot");
        if (s.blob.n != core.n) throw Error(ERR_STATE, "snapshot of another configuration");
        core.copy_from(s.blob);
        age = s.age;
        cur = s.cur;
        cellsOnlyLatest = false;
    }
    void assign(StateI *src) override
    {
        auto *o = dynamic_cast<Sys<T> *>(src);
        if (!o) throw Error(ERR_DTYPE, "source state has a different precision");
        if (!same_config(*o)) throw Error(ERR_ARG, "source state has another configuration");
        if (o == this) return;
        core.copy_from(o->core);
        nbcount.copy_from(o->nbcount);
        flags.copy_from(o->flags);
        rho.copy_from(o->rho);
        prho.copy_from(o->prho);
        age = o->age;
        cur = o->cur;
        if (std::memcmp(hinst.data(), o->hinst.data(), sizeof(Inst<T>) * B) != 0) {
            prm = o->prm;
            prms = o->prms;
            hinst = o->hinst;
            anyRho = o->anyRho;
            anyAV = o->anyAV;
            upload_inst();
        }
        rho.copy_from(o->rho);
        cellsOnlyLatest = false;
    }

    void assign_params(const Sys &o)
    {
        if (std::memcmp(hinst.data(), o.hinst.data(), sizeof(Inst<T>) * B) != 0) {
            prm = o.prm;
            prms = o.prms;
            hinst = o.hinst;
            anyRho = o.anyRho;
            anyAV = o.anyAV;
            upload_inst();
        }
    }

    bool same_config(const Sys &o) const
    {
        if (N_ != o.N_ || B != o.B || opts.maxnb != o.opts.maxnb ||
            opts.interval != o.opts.interval || opts.skin != o.opts.skin)
            return false;
        for (int b = 0; b < B; ++b) {
            const Inst<T> &a = hinst[b], &c = o.hinst[b];
            if (a.off != c.off || a.n != c.n || a.nx != c.nx || a.ny != c.ny || a.coff != c.coff ||
                a.toff != c.toff || a.cs != c.cs)
                return false;
        }
        return true;
    }
};

// List the neighbour rows in the reference's particle-major layout
// (indices[(i-1)*maxnb + m], 1-based ids), same order as _nl_build!.
template <typename T>
__global__ void k_list_neighbors(NLView<T> v, const int32_t *__restrict__ perm,
                                 int32_t *__restrict__ out, int32_t *__restrict__ nbc)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    const int32_t id = perm[i];
    const Inst<T> &I = v.inst[inst_of(v, i)];
    int m = 0;
    for_each_neighbor<T>(v, I, i, [&](int j) {
        out[(int64_t)id * I.maxnb + m] = perm[j] + 1;
        ++m;
    });
    nbc[id] = m;
}

template <typename T> void Sys<T>::neighbors(int32_t *indices, int32_t *nbc)
{
    if (!N_) return;
    DevBuf<int32_t> out((size_t)N_ * opts.maxnb), cnt((size_t)N_);
    out.zero();
    SPH_LAUNCH(K_MISC, k_list_neighbors<T>, N_, view(), perm.p, out.p, cnt.p);
    if (indices) SPH_CK(cudaMemcpyAsync(indices, out.p, out.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
    if (nbc) SPH_CK(cudaMemcpyAsync(nbc, cnt.p, cnt.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
    SPH_CK(cudaStreamSynchronize(rt_stream()));
}

// ---------------------------------------------------------------------------
// On-device objectives: J (deterministic block-ordered reduction in double)
// and the terminal seeds dJ/dX_T, dJ/dV_T in particle-id order.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_objective(int64_t n, int64_t off, int kind, const int32_t *__restrict__ perm,
                            const T2<T> *__restrict__ pos, const T2<T> *__restrict__ vel, T m,
                            T Lx, T a0, T a1, T a2, T2<T> *__restrict__ seedX,
                            T2<T> *__restrict__ seedV, double *__restrict__ partial)
{
    pdl_enter();
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t t = off + k;
    double j = 0.0;
    if (k < n) {
        const int32_t id = perm[t];
        const T2<T> x = pos[t], v = vel[t];
        if (kind == OBJ_KE_RIGHT) {
            const bool right = x.x > Lx / (T)2;
            const T ke = (T)0.5 * m * (v.x * v.x + v.y * v.y);
            j = right ? (double)ke : 0.0;
            seedX[id] = mk2<T>((T)0, (T)0);
            seedV[id] = right ? mk2<T>(m * v.x, m * v.y) : mk2<T>((T)0, (T)0);
        } else {
            // target_objective: e = exp(-|x - c|^2 / (2 sigma^2)), J -= e,
            // seed = e * d / sigma^2
            const T s2 = a2 * a2;
            const T dx = x.x - a0, dy = x.y - a1;
            const T e = exp(-(dx * dx + dy * dy) / ((T)2 * s2));
            j = -(double)e;
            seedX[id] = mk2<T>(e * dx / s2, e * dy / s2);
            seedV[id] = mk2<T>((T)0, (T)0);
        }
    }
    __shared__ double sm[kBlock];
    sm[threadIdx.x] = j;
    __syncthreads();
    for (int o = kBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

// single block: fixed-order sum of the block partials
static __global__ void k_sum_partials(int64_t nb, const double *__restrict__ partial,
                                      double *__restrict__ out)
{
    pdl_enter();
    __shared__ double sm[kBlock];
    double a = 0.0;
    for (int64_t i = threadIdx.x; i < nb; i += blockDim.x) a += partial[i];
    sm[threadIdx.x] = a;
    __syncthreads();
    for (int o = kBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

// ---------------------------------------------------------------------------
// Tape
// ---------------------------------------------------------------------------
template <typename T> class Tape final : public TapeI {
  public:
    int64_t N_, cap_, n_ = 0;
    int32_t nsnap_;
    // full history: (X, V) before every step, id order
    DevBuf<T2<T>> hx, hv;
    // checkpoints
    std::vector<int64_t> descent;        // planned snapshot positions (0-based step index)
    std::vector<std::unique_ptr<Snap<T>>> slots;
    std::vector<int64_t> slotPos;        // position held by each slot (-1 = free)
    std::unique_ptr<Sys<T>> recomp;      // state used to recompute during backward
    int64_t fwdSteps = 0;

    Tape(int64_t N, int64_t cap, int32_t nsnap) : N_(N), cap_(cap), nsnap_(nsnap)
    {
        if (N < 0 || cap < 0) throw Error(ERR_ARG, "negative tape size");
        if (nsnap < 0) throw Error(ERR_ARG, "negative snapshot count");
        if (nsnap == 0) {
            const size_t n = (size_t)std::max<int64_t>(N, 1) * (size_t)std::max<int64_t>(cap, 1);
            hx.alloc(n);
            hv.alloc(n);
        } else {
            descent = plan_descent(std::max<int64_t>(cap, 1), nsnap);
            slots.resize((size_t)nsnap);
            slotPos.assign((size_t)nsnap, -1);
        }
    }
    int dtype() const override { return sizeof(T) == 8 ? F64 : F32; }
    int64_t N() const override { return N_; }
    int64_t capacity() const override { return cap_; }
    int64_t length() const override { return n_; }
    int32_t snapshots() const override { return nsnap_; }
    int64_t forward_steps() const override { return fwdSteps; }
    void reset() override
    {
        n_ = 0;
        std::fill(slotPos.begin(), slotPos.end(), -1);
    }
    void get(int64_t n, void *X, void *V) override
    {
        if (nsnap_) throw Error(ERR_STATE, "a checkpoint tape keeps no per-step history");
        if (n < 1 || n > n_) throw Error(ERR_ARG, "tape index out of range");
        const size_t off = (size_t)(n - 1) * N_;
        if (X) SPH_CK(cudaMemcpyAsync(X, hx.p + off, sizeof(T2<T>) * N_, cudaMemcpyDeviceToHost, rt_stream()));
        if (V) SPH_CK(cudaMemcpyAsync(V, hv.p + off, sizeof(T2<T>) * N_, cudaMemcpyDeviceToHost, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
    }
    Snap<T> &slot(int k)
    {
        if (!slots[k]) slots[k].reset(new Snap<T>());
        return *slots[k];
    }
    void bind(const Sys<T> &s)
    {
        if (s.N_ != N_) throw Error(ERR_ARG, "tape and state particle counts differ");
        if (nsnap_ && recomp && !recomp->same_config(s))
            throw Error(ERR_ARG, "checkpoint tape was bound to a state with another configuration");
        if (nsnap_ && !recomp) {
            std::vector<int64_t> ns;
            for (const auto &I : s.hinst) ns.push_back(I.n);
            recomp.reset(new Sys<T>(s.prms, ns, nullptr, nullptr, s.opts));
        }
        if (nsnap_) recomp->assign_params(s);
    }
};

// simulate! (src/driver.jl:92-115)
template <typename T>
void Sys<T>::simulate(FieldI *theta, const Params *p, int64_t nsteps, TapeI *tape)
{
    use_params(p);
    Field<T> *th = field_of(theta);
    Tape<T> *tp = nullptr;
    if (tape) {
        tp = dynamic_cast<Tape<T> *>(tape);
        if (!tp) throw Error(ERR_DTYPE, "tape has a different precision than the state");
        if (tp->n_ + nsteps > tp->cap_)
            throw Error(ERR_CAPACITY, "tape capacity " + std::to_string(tp->cap_) + " < " +
                                          std::to_string(tp->n_ + nsteps) + " steps needed");
        tp->bind(*this);
    }
    // the snapshot slots this call fills, allocated before any recording
    if (tp && tp->nsnap_)
        for (size_t k = 0; k < tp->descent.size(); ++k)
            if (tp->descent[k] >= tp->n_ && tp->descent[k] < tp->n_ + nsteps)
                reserve(tp->slot((int)k));
    graphs.start(step_graph_eligible<T>(N_));
    StepGraphsGuard guard{graphs};
    for (int64_t s = 0; s < nsteps; ++s) {
        graphs.before_step();
        T2<T> *tx = nullptr, *tv = nullptr;
        if (tp) {
            const int64_t n = tp->n_;
            if (tp->nsnap_ == 0) {
                tx = tp->hx.p + (size_t)n * N_;
                tv = tp->hv.p + (size_t)n * N_;
            } else {
                for (size_t k = 0; k < tp->descent.size(); ++k)
                    if (tp->descent[k] == n) {
                        save(tp->slot((int)k));
                        tp->slotPos[k] = n;
                    }
            }
            tp->n_ += 1;
        }
        step_impl(th->th.p, tx, tv);
        graphs.after_step();
    }
    graphs.finish();
    rt_sync();
    rt_check_launch("simulate");
}

// ---------------------------------------------------------------------------
// Adjoint workspace + backward!
// ---------------------------------------------------------------------------
template <typename T> class Work final : public WorkI {
  public:
    int64_t N_;
    int ngx, ngy;                // design grid of instance 0
    std::vector<Params> prms;    // per instance
    std::vector<int64_t> ns;     // particles per instance
    std::vector<int64_t> toffs;  // design-node offset per instance
    int B = 1;
    int64_t nnode = 0;
    DevBuf<T2<T>> gX[2], gV[2];
    int gcur = 0;
    DevBuf<T2<T>> abar, gXs, stage2;
    DevBuf<T> galpha, grho;
    DevBuf<unsigned long long> thetaAcc;
    DevBuf<int> emax;
    DevBuf<double> gtheta;
    DevBuf<T> gthetaT;
    DevBuf<T2<T>> outX, outV; // results in particle-id order
    DevBuf<T2<T>> devSeedX, devSeedV; // seeds written by objective()
    DevBuf<double> partial;
    std::unique_ptr<Sys<T>> own;
    Sys<T> *lastS = nullptr; // scratch state of the last backward (its flags)
    int64_t jOff = -1;       // J slots of the last objective in `partial`
    bool haveResult = false;
    bool haveDevSeeds = false;
    StepGraphs graphs; // backward's steps, replayed in groups

    Work(int64_t N, const Params &p) : Work(std::vector<Params>{p}, std::vector<int64_t>{N}) {}

    Work(const std::vector<Params> &ps, const std::vector<int64_t> &nsv)
        : N_(0), ngx(ps.at(0).ngx), ngy(ps.at(0).ngy), prms(ps), ns(nsv)
    {
        if (ps.empty() || ps.size() != nsv.size()) throw Error(ERR_ARG, "empty instance list");
        B = (int)ps.size();
        for (int b = 0; b < B; ++b) {
            check_params(ps[b]);
            if (nsv[b] < 0) throw Error(ERR_ARG, "particle count out of range");
            toffs.push_back(nnode);
            nnode += (int64_t)ps[b].ngx * ps[b].ngy;
            N_ += nsv[b];
        }
        const int64_t N = N_;
        const size_t n1 = (size_t)std::max<int64_t>(N, 1);
        for (int k = 0; k < 2; ++k) {
            gX[k].alloc(n1);
            gV[k].alloc(n1);
            gX[k].zero();
            gV[k].zero();
        }
        abar.alloc(n1); gXs.alloc(n1); stage2.alloc(n1); outX.alloc(n1); outV.alloc(n1);
        galpha.alloc(n1); grho.alloc(n1);
        thetaAcc.alloc(2 * (size_t)nnode);
        emax.alloc(2 * (size_t)B);
        gtheta.alloc((size_t)nnode);
        gthetaT.alloc((size_t)nnode);
        gtheta.zero();
    }
    int dtype() const override { return sizeof(T) == 8 ? F64 : F32; }
    int64_t N() const override { return N_; }
    int batch() const override { return B; }

    // One reverse step at the pre-state held in (sx, sv); srcInv maps particle
    // ids into the source's slots when the source is a recomputed state.
    // The design-node write-back of a reverse step is deferred into the next
    // step's gather launch (pendingTheta holds its parity) or flush_theta().
    int pendingTheta = -1;

    void flush_theta(Sys<T> &S)
    {
        if (pendingTheta < 0) return;
        SPH_LAUNCH(K_THETA_NODE, k_theta_node<T>, nnode, nnode, S.B, S.dinst.p, thetaAcc.p, emax.p,
                   pendingTheta, gtheta.p);
        pendingTheta = -1;
    }

    void reverse_step(Sys<T> &S, const T *theta, const T2<T> *sx, const T2<T> *sv,
                      const int32_t *srcInv, int parity)
    {
        if (pendingTheta >= 0 && N_ > 0) {
            const unsigned gN = grid_for(N_);
            const unsigned gT = grid_for(nnode);
            rt_before_launch(K_GATHER);
            launch_k(k_gather_theta<T>, dim3(gN + gT), dim3(kBlock), 0, N_, gN,
                     (const int32_t *)S.perm.p, srcInv, sx, sv, S.pos[S.cur].p, S.vel[S.cur].p,
                     nnode, S.B, (const Inst<T> *)S.dinst.p, thetaAcc.p, emax.p, pendingTheta,
                     gtheta.p);
            rt_after_launch(K_GATHER);
            pendingTheta = -1;
        } else {
            flush_theta(S);
            SPH_LAUNCH(K_GATHER, k_gather_state<T>, N_, N_, S.perm.p, srcInv, sx, sv,
                       S.pos[S.cur].p, S.vel[S.cur].p);
        }
        bool did = false;
        const int g2 = 1 - gcur;
        S.maybe_rebuild(gX[gcur].p, gX[g2].p, gV[gcur].p, gV[g2].p, &did);
        if (did) gcur = g2;
        NLView<T> v = S.view();
        const T2<T> *vel = S.vel[S.cur].p;
        T *rhoOut = S.anyRho ? S.rho.p : (T *)nullptr; // densities only where the model reads them
        if (const int G = S.group_lanes()) {
            const bool g32 = G == 32;
            auto kd = g32 ? &k_density_eos_coop<T, 32> : &k_density_eos_coop<T, 16>;
            auto ka = g32 ? &k_accel_drag_adj_coop<T, 32> : &k_accel_drag_adj_coop<T, 16>;
            auto k1 = g32 ? &k_pass1_design_coop<T, 32> : &k_pass1_design_coop<T, 16>;
            auto k2 = g32 ? &k_pass2_axpy_coop<T, 32> : &k_pass2_axpy_coop<T, 16>;
            SPH_LAUNCH_COOP(K_DENSITY, G, kd, N_, v, rhoOut, S.prho.p, S.tmask.p);
            v.tmask = S.tmask.p;
            SPH_LAUNCH_COOP(K_ACCEL_DRAG, G, ka, N_, v, vel, S.prho.p, S.rho.p, theta, gX[gcur].p,
                            gV[gcur].p, abar.p, galpha.p, emax.p, parity);
            SPH_LAUNCH_COOP(K_PASS1, G, k1, N_, v, vel, S.prho.p, S.rho.p, theta, abar.p,
                            galpha.p, gXs.p, grho.p, gV[gcur].p);
            SPH_LAUNCH_COOP(K_PASS2, G, k2, N_, v, grho.p, gXs.p, gX[gcur].p, galpha.p, emax.p,
                            parity, thetaAcc.p);
            pendingTheta = parity;
            return;
        }
        const bool multi = S.B > 1;
        const bool av = S.anyAV;
        auto ka = multi ? (av ? &k_accel_drag_adj<T, true, true> : &k_accel_drag_adj<T, true>)
                        : (av ? &k_accel_drag_adj<T, false, true> : &k_accel_drag_adj<T, false>);
        auto k1 = multi ? (av ? &k_pass1_design<T, true, true> : &k_pass1_design<T, true>)
                        : (av ? &k_pass1_design<T, false, true> : &k_pass1_design<T, false>);
        auto k2 = multi ? &k_pass2_axpy<T, true> : &k_pass2_axpy<T, false>;
        S.launch_density(v, rhoOut, S.prho.p);
        v.tmask = S.tmask.p;
        SPH_LAUNCH_TUNED(K_ACCEL_DRAG, multi, ka, N_, v, vel, S.prho.p, S.rho.p, theta, gX[gcur].p,
                         gV[gcur].p, abar.p, galpha.p, emax.p, parity);
        SPH_LAUNCH_TUNED(K_PASS1, multi, k1, N_, v, vel, S.prho.p, S.rho.p, theta, abar.p,
                         galpha.p, gXs.p, grho.p, gV[gcur].p);
        SPH_LAUNCH_TUNED(K_PASS2, multi, k2, N_, v, grho.p, gXs.p, gX[gcur].p, galpha.p, emax.p,
                         parity, thetaAcc.p);
        pendingTheta = parity;
    }

    void backward(TapeI *tape, FieldI *theta, const Params *p, const void *seedX,
                  const void *seedV, StateI *scratch, NLOpts opts, uint32_t *flags) override
    {
        run_backward(tape, theta, p, seedX, seedV, false, scratch, opts, flags);
    }
    void backward_seeded(TapeI *tape, FieldI *theta, const Params *p, StateI *scratch,
                         NLOpts opts, uint32_t *flags) override
    {
        if (!haveDevSeeds) throw Error(ERR_STATE, "no objective has written seeds to this workspace");
        run_backward(tape, theta, p, nullptr, nullptr, true, scratch, opts, flags);
    }
    void run_backward(TapeI *tape, FieldI *theta, const Params *p, const void *seedX,
                      const void *seedV, bool devSeeds, StateI *scratch, NLOpts opts,
                      uint32_t *flags);

    // J of every instance (J[b]); args: 3 values per instance for the target
    // objective (xc, yc, sigma), or NULL for the kinetic energy
    void objective(StateI *sti, int kind, const double *args, const Params *pp,
                   double *J) override
    {
        auto *st = dynamic_cast<Sys<T> *>(sti);
        if (!st) throw Error(ERR_DTYPE, "state has a different precision than the workspace");
        if (st->N_ != N_ || st->B != B) throw Error(ERR_ARG, "state and workspace shapes differ");
        if (kind != OBJ_KE_RIGHT && kind != OBJ_TARGET) throw Error(ERR_ARG, "unknown objective");
        if (kind == OBJ_TARGET && !args) throw Error(ERR_ARG, "target objective needs (xc, yc, sigma)");
        st->use_params(pp);
        const size_t n1 = (size_t)std::max<int64_t>(N_, 1);
        // block partials of every instance, then one J slot per instance
        int64_t nbTot = 0;
        for (int b = 0; b < B; ++b) nbTot += grid_for(st->hinst[b].n);
        if (!devSeedX.p) {
            devSeedX.alloc(n1);
            devSeedV.alloc(n1);
            partial.alloc((size_t)nbTot + (size_t)B + 1);
        }
        std::vector<double> Jb((size_t)B, 0.0);
        int64_t pofs = 0;
        for (int b = 0; b < B; ++b) {
            const Inst<T> &I = st->hinst[b];
            if (!I.n) continue;
            const Params &q = st->prms[b];
            const T a0 = args ? (T)args[3 * b] : (T)0, a1 = args ? (T)args[3 * b + 1] : (T)0,
                    a2 = args ? (T)args[3 * b + 2] : (T)1;
            SPH_LAUNCH(K_MISC, k_objective<T>, (int64_t)I.n, (int64_t)I.n, (int64_t)I.off, kind,
                       st->perm.p, st->pos[st->cur].p, st->vel[st->cur].p, (T)q.m, (T)q.Lx, a0, a1,
                       a2, devSeedX.p, devSeedV.p, partial.p + pofs);
            const int64_t nb = grid_for(I.n);
            rt_before_launch(K_MISC);
            launch_k(k_sum_partials, dim3(1), dim3(kBlock), 0, nb, (const double *)(partial.p + pofs),
                     partial.p + nbTot + b);
            rt_after_launch(K_MISC);
            pofs += nb;
        }
        jOff = nbTot;
        haveDevSeeds = true;
        // while capturing, or when the caller takes no J, J stays on the
        // device (objective_value) and nothing waits
        if (rt_capturing() || !J) return;
        SPH_CK(cudaMemcpyAsync(Jb.data(), partial.p + nbTot, sizeof(double) * B, cudaMemcpyDeviceToHost, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
        for (int b = 0; b < B; ++b)
            if (J) J[b] = st->hinst[b].n ? Jb[b] : 0.0;
    }

    void objective_value(double *J) override
    {
        if (jOff < 0) throw Error(ERR_STATE, "no objective has run on this workspace");
        std::vector<double> Jb((size_t)B, 0.0);
        SPH_CK(cudaMemcpyAsync(Jb.data(), partial.p + jOff, sizeof(double) * B, cudaMemcpyDeviceToHost, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
        for (int b = 0; b < B; ++b) J[b] = ns[b] ? Jb[b] : 0.0;
    }

    uint32_t take_flags() override { return lastS ? lastS->take_flags() : 0u; }

    const double *gtheta_device(int64_t n) const override
    {
        if (!haveResult) throw Error(ERR_STATE, "no backward pass has run on this workspace");
        if (n != nnode) throw Error(ERR_ARG, "design size differs from the workspace's theta");
        return gtheta.p;
    }

    void get(void *gXo, void *gVo, void *gth) override
    {
        if (!haveResult) throw Error(ERR_STATE, "no backward pass has run on this workspace");
        if (N_ && gXo) SPH_CK(cudaMemcpyAsync(gXo, outX.p, outX.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
        if (N_ && gVo) SPH_CK(cudaMemcpyAsync(gVo, outV.p, outV.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
        SPH_CK(cudaStreamSynchronize(rt_stream()));
        if (gth) {
            const int64_t nn = nnode;
            SPH_LAUNCH(K_MISC, k_to_T<T>, nn, nn, gtheta.p, gthetaT.p);
            SPH_CK(cudaMemcpyAsync(gth, gthetaT.p, gthetaT.bytes(), cudaMemcpyDeviceToHost, rt_stream()));
            SPH_CK(cudaStreamSynchronize(rt_stream()));
        }
    }
};

// Block-size autotuner: times each hot kernel of this state's kind (single or
// batched) at 64, 128 and 256 threads per block on the state's current
// positions and keeps the fastest. Forward kernels run on the state itself
// (they only write derived arrays); the adjoint kernels run on a temporary
// workspace with placeholder gradients, whose values do not change the work.
template <typename T> class Tuner {
  public:
    static void run(Sys<T> &S, Field<T> &th, int reps, int *chosen)
    {
        if (S.N_ == 0) return;
        if (S.age == INT64_MAX) S.rebuild();
        const bool multi = S.B > 1;
        const int cand[3] = {64, 128, 256};
        cudaEvent_t e0, e1;
        SPH_CK(cudaEventCreate(&e0));
        SPH_CK(cudaEventCreate(&e1));
        // three interleaved rounds over the candidates, each candidate's best
        // round kept: a single round let clock or cache noise pick a block
        // size up to 8% slower
        auto timeit = [&](const std::function<void(int)> &launch) {
            float tbest[3] = {1e30f, 1e30f, 1e30f};
            for (int c : cand) launch(c); // warm
            for (int round = 0; round < 3; ++round)
                for (int k = 0; k < 3; ++k) {
                    SPH_CK(cudaEventRecord(e0, rt_stream()));
                    for (int r = 0; r < reps; ++r) launch(cand[k]);
                    SPH_CK(cudaEventRecord(e1, rt_stream()));
                    SPH_CK(cudaEventSynchronize(e1));
                    float ms = 0;
                    SPH_CK(cudaEventElapsedTime(&ms, e0, e1));
                    tbest[k] = std::min(tbest[k], ms);
                }
            int k = 0;
            for (int q = 1; q < 3; ++q)
                if (tbest[q] < tbest[k]) k = q;
            return cand[k];
        };
        const int64_t N = S.N_;
        auto grid = [N](int b) { return (unsigned)((N + b - 1) / b); };
        cudaStream_t st = rt_stream();
        NLView<T> v = S.view();
        const int nxt = 1 - S.cur;
        auto kn = multi ? &k_nl_build<T, true> : &k_nl_build<T, false>;
        auto kd = multi ? &k_density_eos<T, true> : &k_density_eos<T, false>;
        auto ki = multi ? &k_accel_integrate<T, true> : &k_accel_integrate<T, false>;
        auto ka = multi ? &k_accel_drag_adj<T, true> : &k_accel_drag_adj<T, false>;
        auto k1 = multi ? &k_pass1_design<T, true> : &k_pass1_design<T, false>;
        auto k2 = multi ? &k_pass2_axpy<T, true> : &k_pass2_axpy<T, false>;
        int b;
        b = timeit([&](int c) {
            kn<<<grid(c), c, 0, st>>>(N, S.hinst[0], S.dinst.p, S.pinst.p, S.pos[S.cur].p,
                                      S.cellStart.p, S.center.p, S.masks.p, S.nbcount.p,
                                      S.flags.p);
        });
        tuned_block<T>(K_NLBUILD, multi) = b;
        b = timeit([&](int c) {
            kd<<<grid(c), c, 0, st>>>(v, S.rho.p, S.prho.p, S.tmask.p);
        });
        tuned_block<T>(K_DENSITY, multi) = b;
        v.tmask = S.tmask.p;
        b = timeit([&](int c) {
            ki<<<grid(c), c, 0, st>>>(v, S.vel[S.cur].p, S.prho.p, S.rho.p, th.th.p, S.pos[nxt].p,
                                      S.vel[nxt].p, nullptr, nullptr, S.flags.p, nullptr, nullptr,
                                      nullptr);
        });
        tuned_block<T>(K_ACCEL_INTEGRATE, multi) = b;
        // adjoint passes on placeholder gradients
        std::vector<int64_t> ns;
        for (const auto &I : S.hinst) ns.push_back(I.n);
        Work<T> w(S.prms, ns);
        for (int k = 0; k < 2; ++k) {
            SPH_CK(cudaMemsetAsync(w.gX[k].p, 0x3c, w.gX[k].bytes(), st));
            SPH_CK(cudaMemsetAsync(w.gV[k].p, 0x3c, w.gV[k].bytes(), st));
        }
        const std::vector<int> init(2 * (size_t)S.B, INT_MIN);
        SPH_CK(cudaMemcpyAsync(w.emax.p, init.data(), sizeof(int) * init.size(), cudaMemcpyHostToDevice, st));
        const T2<T> *vel = S.vel[S.cur].p;
        ka<<<grid(kBlock), kBlock, 0, st>>>(v, vel, S.prho.p, S.rho.p, th.th.p, w.gX[0].p,
                                            w.gV[0].p, w.abar.p, w.galpha.p, w.emax.p, 0);
        b = timeit([&](int c) {
            ka<<<grid(c), c, 0, st>>>(v, vel, S.prho.p, S.rho.p, th.th.p, w.gX[0].p, w.gV[1].p,
                                      w.abar.p, w.galpha.p, w.emax.p, 1);
        });
        tuned_block<T>(K_ACCEL_DRAG, multi) = b;
        b = timeit([&](int c) {
            k1<<<grid(c), c, 0, st>>>(v, vel, S.prho.p, S.rho.p, th.th.p, w.abar.p, w.galpha.p,
                                      w.gXs.p, w.grho.p, w.gV[1].p);
        });
        tuned_block<T>(K_PASS1, multi) = b;
        w.thetaAcc.zero(); // the placeholder sums only accumulate while timing
        b = timeit([&](int c) {
            k2<<<grid(c), c, 0, st>>>(v, w.grho.p, w.gXs.p, w.gX[1].p, w.galpha.p, w.emax.p, 0,
                                      w.thetaAcc.p);
        });
        tuned_block<T>(K_PASS2, multi) = b;
        SPH_CK(cudaStreamSynchronize(st));
        SPH_CK(cudaEventDestroy(e0));
        SPH_CK(cudaEventDestroy(e1));
        rt_check_launch("autotune");
        const int ids[6] = {K_NLBUILD, K_DENSITY, K_ACCEL_INTEGRATE, K_ACCEL_DRAG, K_PASS1, K_PASS2};
        if (chosen)
            for (int k = 0; k < 6; ++k) chosen[k] = tuned_block<T>(ids[k], multi);
    }
};

template <typename T> void Sys<T>::autotune(FieldI *theta, int reps, int *chosen)
{
    Field<T> *th = field_of(theta);
    Tuner<T>::run(*this, *th, std::max(1, reps), chosen);
}

template <typename T>
void Work<T>::run_backward(TapeI *tape, FieldI *theta, const Params *pp, const void *seedX,
                           const void *seedV, bool devSeeds, StateI *scratch, NLOpts opts,
                           uint32_t *flagsOut)
{
    auto *tp = dynamic_cast<Tape<T> *>(tape);
    if (!tp) throw Error(ERR_DTYPE, "tape has a different precision than the workspace");
    if (tp->N_ != N_) throw Error(ERR_ARG, "tape and workspace particle counts differ");
    auto *th = dynamic_cast<Field<T> *>(theta);
    if (!th) throw Error(ERR_DTYPE, "theta has a different precision than the workspace");
    if (th->batch() != B) throw Error(ERR_ARG, "theta has a different number of instances");
    for (int b = 0; b < B; ++b)
        if (th->gx[b] != prms[b].ngx || th->gy[b] != prms[b].ngy)
            throw Error(ERR_ARG, "theta shape does not match the workspace");
    std::vector<Params> ps = prms;
    if (pp) {
        if (B != 1) throw Error(ERR_ARG, "a batch uses its per-instance parameters (pass NULL)");
        check_params(*pp);
        if (pp->ngx != ngx || pp->ngy != ngy)
            throw Error(ERR_ARG, "params (ngx, ngy) do not match the workspace");
        ps[0] = *pp;
    } else if (B == 1) {
        throw Error(ERR_ARG, "backward needs the parameters");
    }

    // scratch State (src/driver.jl:153-156): fresh unless the caller passes one
    Sys<T> *S = nullptr;
    if (scratch) {
        S = dynamic_cast<Sys<T> *>(scratch);
        if (!S) throw Error(ERR_DTYPE, "scratch state has a different precision");
        if (S->N_ != N_ || S->B != B) throw Error(ERR_ARG, "scratch state shape differs");
        if (B == 1) S->use_params(&ps[0]);
    } else {
        bool same = own && own->opts.skin == opts.skin && own->opts.interval == opts.interval &&
                    own->opts.maxnb == opts.maxnb;
        if (same)
            for (int b = 0; b < B; ++b)
                same = same && own->prms[b].h == ps[b].h && own->prms[b].Lx == ps[b].Lx &&
                       own->prms[b].Ly == ps[b].Ly;
        if (!same) own.reset(new Sys<T>(ps, ns, nullptr, nullptr, opts));
        S = own.get();
        if (B == 1) S->use_params(&ps[0]);
        // a fresh State: neighbour list never built, no flags
        S->age = INT64_MAX;
        S->flags.zero();
    }

    // seeds: copyto!(gX, seedX), copyto!(gV, seedV), id order -> S's cell order
    if (rt_capturing() && !devSeeds && (seedX || seedV))
        throw Error(ERR_STATE, "host seeds cannot be captured: use the on-device objective and "
                               "backward_seeded inside a captured sequence");
    lastS = S;
    gcur = 0;
    if (N_ && devSeeds) {
        SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N_, N_, S->perm.p, devSeedX.p, gX[0].p);
        SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N_, N_, S->perm.p, devSeedV.p, gV[0].p);
    } else if (N_) {
        if (seedX) {
            SPH_CK(cudaMemcpyAsync(stage2.p, seedX, stage2.bytes(), cudaMemcpyHostToDevice, rt_stream()));
            SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N_, N_, S->perm.p, stage2.p, gX[0].p);
        } else {
            gX[0].zero();
        }
        if (seedV) {
            SPH_CK(cudaMemcpyAsync(stage2.p, seedV, stage2.bytes(), cudaMemcpyHostToDevice, rt_stream()));
            SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N_, N_, S->perm.p, stage2.p, gV[0].p);
        } else {
            gV[0].zero();
        }
    }
    gtheta.zero();
    thetaAcc.zero();
    SPH_LAUNCH(K_MISC, k_fill_int, 2 * (int64_t)B, 2 * (int64_t)B, emax.p, INT_MIN);

    const int64_t L = tp->n_;
    pendingTheta = -1;
    int64_t rstep = 0; // reverse steps done (parity of the exponent slot)
    tp->fwdSteps = 0;
    // reverse steps and recomputed forward steps go out in recorded groups
    if (tp->nsnap_ && L > 0)
        for (int k = 0; k < tp->nsnap_; ++k) tp->recomp->reserve(tp->slot(k));
    graphs.start(step_graph_eligible<T>(N_));
    StepGraphsGuard guard{graphs};
    if (tp->nsnap_ == 0) {
        for (int64_t n = L - 1; n >= 0; --n) {
            graphs.before_step();
            reverse_step(*S, th->th.p, tp->hx.p + (size_t)n * N_, tp->hv.p + (size_t)n * N_,
                         nullptr, (int)(rstep & 1));
            ++rstep;
            graphs.after_step();
        }
    } else if (L > 0) {
        Sys<T> &R = *tp->recomp;
        if (B == 1) R.use_params(&ps[0]);
        // snapshots taken by simulate!, in position order
        std::vector<std::pair<int64_t, int>> taken;
        for (size_t k = 0; k < tp->slotPos.size(); ++k)
            if (tp->slotPos[k] >= 0 && tp->slotPos[k] < L) taken.push_back({tp->slotPos[k], (int)k});
        std::sort(taken.begin(), taken.end());
        if (taken.empty() || taken[0].first != 0)
            throw Error(ERR_STATE, "checkpoint tape holds no snapshot of its first step");
        const int C = tp->nsnap_;
        // free slots: those not holding a descent snapshot (as a stack)
        std::vector<int> freeSlots;
        for (int k = C - 1; k >= 0; --k)
            if (tp->slotPos[k] < 0 || tp->slotPos[k] >= L) freeSlots.push_back(k);
        int64_t rpos = -1; // step the recompute state holds (-1: unknown)
        auto advance = [&](int64_t m) {
            for (int64_t s = 0; s < m; ++s) {
                graphs.before_step();
                R.step_impl(th->th.p, nullptr, nullptr);
                graphs.after_step();
            }
            tp->fwdSteps += m;
            rpos += m;
        };
        // the recompute state repeats the forward bit for bit, so it already
        // equals a snapshot of the step it holds
        auto restore_at = [&](int slot, int64_t a) {
            if (rpos != a) {
                R.restore(tp->slot(slot));
                rpos = a;
            }
        };
        auto rev_at_R = [&](int64_t n) {
            (void)n;
            graphs.before_step();
            reverse_step(*S, th->th.p, R.pos[R.cur].p, R.vel[R.cur].p, R.invperm.p,
                         (int)(rstep & 1));
            ++rstep;
            graphs.after_step();
        };
        // reverse steps [a, b) with the state at a in `slot`, c slots available
        // (including `slot`); recursion splits at plan_split.
        std::function<void(int64_t, int64_t, int, int64_t)> seg =
            [&](int64_t a, int64_t b, int slot, int64_t c) {
                if (b - a == 1) {
                    restore_at(slot, a);
                    rev_at_R(a);
                    return;
                }
                if (c <= 1 || freeSlots.empty()) {
                    for (int64_t i = b - 1; i >= a; --i) {
                        restore_at(slot, a);
                        advance(i - a);
                        rev_at_R(i);
                    }
                    return;
                }
                const int64_t m = plan_split(b - a, c);
                restore_at(slot, a);
                advance(m);
                const int ns = freeSlots.back();
                freeSlots.pop_back();
                R.save(tp->slot(ns));
                seg(a + m, b, ns, c - 1);
                freeSlots.push_back(ns);
                seg(a, a + m, slot, c);
            };
        const int K = (int)taken.size();
        for (int k = K - 1; k >= 0; --k) {
            const int64_t a = taken[k].first;
            const int64_t b = (k == K - 1) ? L : taken[k + 1].first;
            seg(a, b, taken[k].second, (int64_t)freeSlots.size() + 1);
            freeSlots.push_back(taken[k].second);
        }
    }
    graphs.finish();
    flush_theta(*S);
    SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N_, N_, S->perm.p, gX[gcur].p, outX.p);
    SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N_, N_, S->perm.p, gV[gcur].p, outV.p);
    haveResult = true;
    rt_sync();
    rt_check_launch("backward");
    // while capturing, the flags stay on the device (take_flags after a replay)
    const uint32_t f = rt_capturing() ? 0u : S->take_flags();
    if (flagsOut) *flagsOut = f;
}

} // namespace sphgb
