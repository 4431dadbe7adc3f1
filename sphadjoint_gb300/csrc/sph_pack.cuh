// Packed multi-request engine of the request server (no counterpart in the
// reference, whose optimisation driver runs one simulate!/backward! pair at a
// time, scripts/03_optimize.jl:228-254).
//
// Every request in flight is a small program of steps: forward steps (with a
// full tape, or snapshots of a binomial checkpoint schedule), its objective,
// and reverse steps (replayed from the full tape, or from forward steps
// recomputed between restored snapshots). The engine advances all of them in
// lock step, one step of each per tick, and runs each pass of the tick as ONE
// grouped launch over the particles of every request that takes part: one
// launch for all the gathers, one for each cell-list stage of the requests
// whose neighbour list is due, one density pass, the force passes (one for the
// forward accel + integrate of requests in their forward phase, one for the
// accel + drag VJP of requests in their reverse phase), one pass 1, one pass 2
// and one design-node flush. Requests join at the next tick after
// admission and leave when their program ends, so the set sharing a launch
// changes continuously.
//
// A block of a grouped launch finds its request by a binary search of the
// launch's block offsets; the request's arrays and constants come from a
// per-tick descriptor table uploaded once per tick. Each request runs the
// same per-particle arithmetic as the one-thread-per-particle kernels of a
// solo state, with its own cell list, neighbour masks, rebuild schedule and
// fixed-point dJ/dtheta accumulator, so its result does not depend on which
// other requests share its launches.
#pragma once

#include <deque>
#include <map>
#include <string>
#include <type_traits>
#include <memory>
#include <vector>

#include "sph_engine.cuh"

namespace sphgb {

constexpr int kPackBlock = 128; // threads per block of the per-particle grouped kernels
constexpr bool kAlignRebuilds = true; // start sweeps on ticks aligned to the rebuild interval

// One request's arrays and constants for one tick.
template <typename T> struct GSys {
    NLView<T> v;  // pair-kernel view: v.pos = positions after this tick's rebuild,
                  // v.tmask = this step's in-support masks
    int64_t n, ncell, nnode;
    int mode;     // 0 forward step, 1 reverse step
    int parity;   // exponent slot of the reverse step
    int check;    // displacement check of the rebuild
    T2<T> *posPre, *velPre; // current buffers before this tick's rebuild
    const T2<T> *vel;       // velocities the pair kernels read
    T2<T> *posN, *velN;     // rebuild outputs (the buffers v.pos / vel)
    T2<T> *posOut, *velOut; // forward step outputs
    T2<T> *xref;
    int32_t *perm, *invperm, *cellStart, *cellTmp, *counts, *cursor, *bucketSrc, *bucketId,
        *scanTmp, *nbcount;
    uint32_t *center, *masks, *tmask, *flags;
    T *rho;     // densities (NULL where the model does not read them in the reverse step)
    T *rhoAll;  // the density array the force passes read
    T2<T> *prho;
    const T *theta;
    T2<T> *tx, *tv; // full-tape slot written by a forward step (NULL otherwise)
    const int32_t *srcInv;
    const T2<T> *sx, *sv; // reverse step: source of the gathered pre-state
    const T2<T> *ex0;
    T2<T> *ex0N;
    const T2<T> *ex1;
    T2<T> *ex1N;
    T2<T> *gX, *gV, *abar, *gXs;
    T *galpha, *grho;
    int *emax;
    unsigned long long *thetaAcc;
    double *gtheta;
};

// The per-tick table in constant memory: the descriptors of the requests that
// take a step, and the block lists of the tick's grouped launches (list l:
// request sys[l][k] owns blocks [start[l][k], start[l][k+1])). A block reads
// its request's arrays and constants at a block-uniform index, through the
// constant cache, so they need not be held in registers. One table per
// translation unit: the includer defines SPH_PACK_T, its precision.
#ifndef SPH_PACK_T
#error "define SPH_PACK_T (this translation unit's precision) before including sph_pack.cuh"
#endif
constexpr int kMaxPackSys = 64; // requests one tick can hold
constexpr int kPackLists = 9;
enum PackList : int {
    PL_GATHER = 0, PL_CELLS, PL_SCANTOP, PL_SCANTILE, PL_PART, PL_ALL, PL_REV, PL_THETA, PL_FWD
};
struct PackLists {
    int32_t cnt[kPackLists];
    int32_t sys[kPackLists][kMaxPackSys];
    int32_t start[kPackLists][kMaxPackSys + 1];
};
template <typename T> struct PackTable {
    PackLists L;
    GSys<T> sys[kMaxPackSys];
};
__constant__ PackTable<SPH_PACK_T> c_pack;

template <typename T> __device__ __forceinline__ const GSys<T> &pack_sys(int k)
{
    static_assert(std::is_same<T, SPH_PACK_T>::value, "one packed precision per unit");
    return c_pack.sys[k];
}

// (request, block within the request) of this block in launch list l
__device__ __forceinline__ int2 glist_find(int l)
{
    const int b = (int)blockIdx.x;
    int lo = 0, hi = c_pack.L.cnt[l] - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (c_pack.L.start[l][mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return make_int2(c_pack.L.sys[l][lo], b - c_pack.L.start[l][lo]);
}

// _tape_load! of the reverse step's pre-state into cell order
template <typename T>
__global__ void __launch_bounds__(kPackBlock) g_gather(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t t = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (t >= d.n) return;
    int32_t s = d.perm[t];
    if (d.srcInv) s = d.srcInv[s];
    d.posPre[t] = d.sx[s];
    d.velPre[t] = d.sv[s];
}

template <typename T> __global__ void __launch_bounds__(kBlock) g_zero_counts(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t c = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (c < d.ncell) d.counts[c] = 0;
}

// k_assign of one request (single instance, cells from 0)
template <typename T>
__global__ void __launch_bounds__(kPackBlock) g_assign(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    const bool live = i < d.n;
    int32_t c = -1;
    if (live) {
        const Inst<T> &I = d.v.one;
        const T2<T> x = d.posPre[i];
        if (d.check) {
            const T2<T> xr = d.xref[i];
            const T d2 = r2_exact<T>(sub_rn(x.x, xr.x), sub_rn(x.y, xr.y));
            if (d2 > I.dmax2) atomicOr(d.flags, FLAG_DISPLACEMENT);
        }
        const T cs = I.cs;
        const int cx = cell_coord<T>(x.x / cs, I.nx);
        const int cy = cell_coord<T>(x.y / cs, I.ny);
        c = (cx - 1) + (cy - 1) * I.nx;
        d.cellTmp[i] = c;
    }
    const unsigned act = __ballot_sync(0xffffffffu, live);
    if (live) {
        const unsigned peers = __match_any_sync(act, c);
        if ((int)lane_id() == __ffs(peers) - 1) atomicAdd(d.counts + c, __popc(peers));
    }
}

// exclusive scan of each request's counts: tile sums, per-request scan of the
// tile sums (one block each), then the tiles with their offsets
template <typename T> __global__ void __launch_bounds__(kBlock) g_scan_reduce(int l)
{
    pdl_enter();
    __shared__ int32_t sw[33];
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t base = (int64_t)f.y * kScanTile;
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanTile / kBlock; ++k) {
        const int64_t i = base + (int64_t)k * kBlock + threadIdx.x;
        if (i < d.ncell) s += d.counts[i];
    }
    int32_t tot;
    block_excl_scan(s, sw, tot);
    if (threadIdx.x == 0) d.scanTmp[f.y] = tot;
}

template <typename T> __global__ void __launch_bounds__(kBlock) g_scan_top(int l)
{
    pdl_enter();
    __shared__ int32_t sw[33];
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t nb = (d.ncell + kScanTile - 1) / kScanTile;
    int32_t carry = 0;
    for (int64_t base = 0; base < nb; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const int32_t x = i < nb ? d.scanTmp[i] : 0;
        int32_t tot;
        const int32_t e = block_excl_scan(x, sw, tot);
        if (i < nb) d.scanTmp[i] = e + carry;
        carry += tot;
    }
}

template <typename T> __global__ void __launch_bounds__(kBlock) g_scan_down(int l)
{
    pdl_enter();
    __shared__ int32_t sw[33];
    constexpr int IPT = kScanTile / kBlock;
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t n = d.ncell;
    const int64_t base = (int64_t)f.y * kScanTile + (int64_t)threadIdx.x * IPT;
    int32_t v[IPT];
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int64_t i = base + k;
        v[k] = i < n ? d.counts[i] : 0;
        s += v[k];
    }
    int32_t tot;
    int32_t run = block_excl_scan(s, sw, tot) + d.scanTmp[f.y];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int64_t i = base + k;
        if (i < n) {
            d.cellStart[i] = run;
            d.cursor[i] = run;
        }
        run += v[k];
        if (i == n - 1) d.cellStart[n] = run;
    }
}

template <typename T>
__global__ void __launch_bounds__(kPackBlock) g_bucket(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    const bool live = i < d.n;
    const int32_t c = live ? d.cellTmp[i] : -1;
    const unsigned act = __ballot_sync(0xffffffffu, live);
    if (!live) return;
    const unsigned peers = __match_any_sync(act, c);
    const int leader = __ffs(peers) - 1;
    int32_t base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(d.cursor + c, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    const int32_t p = base + __popc(peers & ((1u << lane_id()) - 1u));
    d.bucketSrc[p] = (int32_t)i;
    d.bucketId[p] = d.perm[i];
}

template <typename T>
__global__ void __launch_bounds__(kPackBlock) g_rank(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t s = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (s >= d.n) return;
    const int32_t src = d.bucketSrc[s];
    const int32_t id = d.bucketId[s];
    const int32_t c = d.cellTmp[src];
    const int32_t b = d.cellStart[c], e = d.cellStart[c + 1];
    int32_t rank = 0;
    for (int32_t k = b; k < e; ++k) rank += (d.bucketId[k] < id) ? 1 : 0;
    const int32_t dst = b + rank;
    d.perm[dst] = id;
    const T2<T> x = d.posPre[src];
    d.posN[dst] = x;
    d.xref[dst] = x;
    d.velN[dst] = d.velPre[src];
    d.invperm[id] = dst;
    if (d.ex0) d.ex0N[dst] = d.ex0[src];
    if (d.ex1) d.ex1N[dst] = d.ex1[src];
}

template <typename T>
__global__ void __launch_bounds__(kPackBlock) g_nl_build(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    nl_build_one<T>(d.n, d.v.one, 0, i, d.v.pos, d.cellStart, d.center, d.masks, d.nbcount,
                    d.flags);
}

// The pair kernels cap their registers as the tuned single-state kernels do:
// the request's arrays and constants come from the descriptor table, and
// holding them all in registers would halve the resident warps.
template <typename T>
__global__ void __launch_bounds__(kPackBlock, sizeof(T) == 4 ? 10 : 1)
    g_density(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    NLView<T> v = d.v;
    v.tmask = nullptr;
    density_walk<T, false, true>(v, i, d.rho, d.prho, d.tmask);
}

// accel_kernel! + integrate_kernel! of the requests taking a forward step.
// The forward and reverse force passes are separate kernels so that each gets
// the registers of its own body (one kernel holding both spilled).
template <typename T, bool AV>
__global__ void __launch_bounds__(kPackBlock, (sizeof(T) == 4 && !AV) ? 10 : 1)
    g_accel_fwd(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const NLView<T> &v = d.v;
    const Inst<T> &I = v.one;
    const T2<T> xi = v.pos[i];
    const T2<T> vi = d.vel[i];
    T ax, ay;
    accel_sum<T, AV>(v, I, d.vel, d.prho, d.rhoAll, i, xi, vi, ax, ay);
    accel_integrate_finish<T>(I, 0, i, xi, vi, ax, ay, d.theta, d.posOut, d.velOut,
                              (T2<T> *)nullptr, (T *)nullptr, d.flags, d.perm, d.tx, d.tv);
}

// accel recompute + _adj_integrate! + _adj_drag! of the requests taking a
// reverse step, with the largest exponent of |galpha| (one atomic per warp)
template <typename T, bool AV>
__global__ void __launch_bounds__(kPackBlock, (sizeof(T) == 4 && !AV) ? 12 : 1)
    g_accel_rev(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    const bool live = i < d.n;
    int e = INT_MIN;
    if (live) {
        const NLView<T> &v = d.v;
        const Inst<T> &I = v.one;
        const T2<T> xi = v.pos[i];
        const T2<T> vi = d.vel[i];
        T ax, ay;
        accel_sum<T, AV>(v, I, d.vel, d.prho, d.rhoAll, i, xi, vi, ax, ay);
        e = drag_adj_finish<T>(I, i, xi, vi, ax, ay, d.theta, d.gX, d.gV, d.abar, d.galpha);
    }
    const unsigned act = __ballot_sync(0xffffffffu, live);
    if (!live) return;
    int mx = e;
    for (unsigned rest = act; rest; rest &= rest - 1) {
        const int y = __shfl_sync(act, e, __ffs(rest) - 1);
        mx = y > mx ? y : mx;
    }
    if ((int)lane_id() == __ffs(act) - 1 && mx != INT_MIN) atomicMax(d.emax + d.parity, mx);
}

// 8 blocks of 128 (55 registers, no spills): 3.5% faster than 9 blocks (56
// registers with spills); the reverse force pass keeps its 12 (relaxing it to
// 10 made it 10% slower)
template <typename T, bool AV>
__global__ void __launch_bounds__(kPackBlock, (sizeof(T) == 4 && !AV) ? 8 : 1)
    g_pass1(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const NLView<T> &v = d.v;
    const Inst<T> &I = v.one;
    const T2<T> xi = v.pos[i];
    const T2<T> vi = d.vel[i];
    const T2<T> ab = d.abar[i];
    const T2<T> pi = d.prho[i];
    T gx, gy, gvx, gvy, grh, sumS;
    pass1_sum<T, AV>(v, I, i, d.vel, d.prho, d.rhoAll, d.abar, xi, vi, ab, pi, gx, gy, gvx, gvy,
                     grh, sumS);
    const T rhoi = I.p.eos == 1 || (AV && I.p.visc == 1) ? d.rhoAll[i] : (T)0;
    pass1_finish<T>(I, i, xi, ab, pi, rhoi, gx, gy, gvx, gvy, grh, sumS, d.theta, d.galpha, d.gXs,
                    d.grho, d.gV);
}

template <typename T>
__global__ void __launch_bounds__(kPackBlock, sizeof(T) == 4 ? 12 : 1)
    g_pass2(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    const int64_t i = (int64_t)f.y * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const NLView<T> &v = d.v;
    const Inst<T> &I = v.one;
    const T2<T> xi = v.pos[i];
    T gx, gy;
    pass2_sum<T>(v, I, i, xi, d.grho, gx, gy);
    pass2_finish<T>(I, 0, i, xi, gx, gy, d.gXs, d.gX, d.galpha, d.emax, d.parity, d.thetaAcc);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) g_theta(int l)
{
    pdl_enter();
    const int2 f = glist_find(l);
    const GSys<T> &d = pack_sys<T>(f.x);
    theta_node<T>((int64_t)f.y * blockDim.x + threadIdx.x, d.nnode, 1, &d.v.one, d.thetaAcc,
                  d.emax, d.parity, d.gtheta);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
enum PackOpKind : uint8_t { OP_SAVE, OP_RESTORE, OP_FWD, OP_OBJ, OP_SEEDS, OP_REV, OP_FINISH };
struct PackOp {
    uint8_t kind;
    int32_t slot; // snapshot slot (SAVE / RESTORE)
    int64_t n;    // full-tape step (FWD: written, REV: read); -1 = none / from the solve state
};

// The program of one request: the forward sweep (snapshots at the positions
// of the checkpoint schedule's first descent, or a full tape), its objective,
// and the reverse sweep in the order of Work::run_backward (full tape from
// the last step down, or the binomial schedule's restores, recomputed steps,
// re-saves and reverse steps). The solve state doubles as the recompute state:
// after the objective it is only restored from snapshots.
inline std::vector<PackOp> pack_program(int64_t L, int32_t snaps, bool adjoint)
{
    std::vector<PackOp> prog;
    auto push = [&](uint8_t k, int32_t slot = -1, int64_t n = -1) { prog.push_back({k, slot, n}); };
    if (!adjoint) {
        for (int64_t s = 0; s < L; ++s) push(OP_FWD);
        push(OP_OBJ);
        push(OP_FINISH);
        return prog;
    }
    if (snaps == 0) {
        for (int64_t s = 0; s < L; ++s) push(OP_FWD, -1, s);
        push(OP_OBJ);
        push(OP_SEEDS);
        for (int64_t s = L - 1; s >= 0; --s) push(OP_REV, -1, s);
        push(OP_FINISH);
        return prog;
    }
    const std::vector<int64_t> descent = plan_descent(std::max<int64_t>(L, 1), snaps);
    std::vector<int64_t> slotPos((size_t)snaps, -1);
    for (int64_t s = 0; s < L; ++s) {
        for (size_t k = 0; k < descent.size(); ++k)
            if (descent[k] == s) {
                push(OP_SAVE, (int32_t)k);
                slotPos[k] = s;
            }
        push(OP_FWD);
    }
    push(OP_OBJ);
    push(OP_SEEDS);
    if (L > 0) {
        std::vector<std::pair<int64_t, int>> taken;
        for (size_t k = 0; k < slotPos.size(); ++k)
            if (slotPos[k] >= 0 && slotPos[k] < L) taken.push_back({slotPos[k], (int)k});
        std::sort(taken.begin(), taken.end());
        std::vector<int> freeSlots;
        for (int k = snaps - 1; k >= 0; --k)
            if (slotPos[k] < 0 || slotPos[k] >= L) freeSlots.push_back(k);
        int64_t rpos = -1;
        auto advance = [&](int64_t m) {
            for (int64_t s = 0; s < m; ++s) push(OP_FWD);
            rpos += m;
        };
        auto restore_at = [&](int slot, int64_t a) {
            if (rpos != a) {
                push(OP_RESTORE, slot);
                rpos = a;
            }
        };
        std::function<void(int64_t, int64_t, int, int64_t)> seg = [&](int64_t a, int64_t b,
                                                                       int slot, int64_t c) {
            if (b - a == 1) {
                restore_at(slot, a);
                push(OP_REV);
                return;
            }
            if (c <= 1 || freeSlots.empty()) {
                for (int64_t i = b - 1; i >= a; --i) {
                    restore_at(slot, a);
                    advance(i - a);
                    push(OP_REV);
                }
                return;
            }
            const int64_t m = plan_split(b - a, c);
            restore_at(slot, a);
            advance(m);
            const int ns = freeSlots.back();
            freeSlots.pop_back();
            push(OP_SAVE, ns);
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
    push(OP_FINISH);
    return prog;
}

template <typename T> class Packer final : public PackI {
    struct Req {
        PackReq spec;
        std::unique_ptr<Sys<T>> F, S;
        std::unique_ptr<Work<T>> W;
        std::unique_ptr<Field<T>> th;
        std::unique_ptr<Tape<T>> tape;
        std::vector<PackOp> prog;
        size_t pc = 0;
        bool fwdStarted = false, revStarted = false;
        int gcur = 0;
        int64_t rstep = 0;
        bool finishing = false;
        cudaEvent_t done = nullptr;
        ~Req()
        {
            if (done) cudaEventDestroy(done);
        }
    };

    // one tick's table, staged in pinned host memory for the asynchronous
    // copy into the constant table; the event marks when the copy is done
    struct Ring {
        uint8_t *host = nullptr;
        cudaEvent_t ev = nullptr;
        bool used = false;
    };
    static constexpr int kRing = 4;

    std::map<int, std::unique_ptr<Req>> reqs_;
    int next_ = 0;
    Ring ring_[kRing];
    int ringPos_ = 0;
    int64_t ticks_ = 0, launches_ = 0;

  public:
    Packer() {}
    ~Packer() override
    {
        (void)cudaStreamSynchronize(rt_stream());
        reqs_.clear();
        for (Ring &r : ring_) {
            if (r.host) cudaFreeHost(r.host);
            if (r.ev) cudaEventDestroy(r.ev);
        }
    }

    int add(const PackReq &r) override
    {
        auto q = std::make_unique<Req>();
        q->spec = r;
        const std::vector<Params> ps{r.p};
        const std::vector<int64_t> ns{r.N};
        q->F.reset(new Sys<T>(ps, ns, r.X0, r.V0, r.opts));
        q->th.reset(new Field<T>(std::vector<int>{r.p.ngx}, std::vector<int>{r.p.ngy}, r.theta));
        q->W.reset(new Work<T>(ps, ns));
        if (r.adjoint) {
            q->S.reset(new Sys<T>(ps, ns, nullptr, nullptr, r.opts));
            q->tape.reset(new Tape<T>(r.N, r.nsteps, r.snapshots));
        }
        q->prog = pack_program(r.nsteps, r.snapshots, r.adjoint);
        SPH_CK(cudaEventCreateWithFlags(&q->done, cudaEventDisableTiming));
        const int id = next_++;
        reqs_[id] = std::move(q);
        return id;
    }

    int active() const override { return (int)reqs_.size(); }

    int64_t ticks() const override { return ticks_; }

    // Run the request's immediate operations up to its next step. Returns
    // the step (FWD / REV) or OP_FINISH when the program has ended.
    PackOp advance(Req &q)
    {
        while (q.pc < q.prog.size()) {
            const PackOp op = q.prog[q.pc++];
            switch (op.kind) {
            case OP_SAVE: q.F->save(q.tape->slot(op.slot)); break;
            case OP_RESTORE: q.F->restore(q.tape->slot(op.slot)); break;
            case OP_OBJ:
                q.W->objective(q.F.get(), q.spec.objective,
                               q.spec.objective == OBJ_TARGET ? q.spec.obj_args : nullptr, nullptr,
                               nullptr);
                break;
            case OP_SEEDS: seeds(q); break;
            default: return op;
            }
        }
        return PackOp{OP_FINISH, -1, -1};
    }

    // backward!'s set-up (src/driver.jl:141-160): a fresh scratch state, the
    // objective's terminal seeds in its order, zeroed dJ/dtheta
    void seeds(Req &q)
    {
        Sys<T> &S = *q.S;
        Work<T> &W = *q.W;
        S.age = INT64_MAX;
        S.flags.zero();
        q.gcur = 0;
        q.rstep = 0;
        const int64_t N = S.N_;
        SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N, N, S.perm.p, W.devSeedX.p, W.gX[0].p);
        SPH_LAUNCH(K_MISC, k_gather_from_ids<T>, N, N, S.perm.p, W.devSeedV.p, W.gV[0].p);
        W.gtheta.zero();
        W.thetaAcc.zero();
        SPH_LAUNCH(K_MISC, k_fill_int, 2, 2, W.emax.p, INT_MIN);
    }

    void finish(Req &q)
    {
        if (q.spec.adjoint) {
            Sys<T> &S = *q.S;
            Work<T> &W = *q.W;
            const int64_t N = S.N_;
            SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N, N, S.perm.p, W.gX[q.gcur].p, W.outX.p);
            SPH_LAUNCH(K_MISC, k_scatter_to_ids<T>, N, N, S.perm.p, W.gV[q.gcur].p, W.outV.p);
            SPH_LAUNCH(K_MISC, k_to_T<T>, W.nnode, W.nnode, W.gtheta.p, W.gthetaT.p);
        }
        SPH_CK(cudaEventRecord(q.done, rt_stream()));
        q.finishing = true;
    }

    int tick() override
    {
        struct Part {
            Req *q;
            PackOp op;
        };
        std::vector<Part> parts;
        for (auto &kv : reqs_) {
            Req &q = *kv.second;
            if (q.finishing) continue;
            const PackOp op = advance(q);
            if (op.kind == OP_FINISH) {
                finish(q);
                continue;
            }
            // Start each sweep on a tick that is a multiple of the request's
            // rebuild interval: its state is rebuilt on its first step and
            // every interval steps after, so requests started this way
            // rebuild on the same ticks and share one set of cell-list
            // launches (otherwise every phase of the interval pays its own
            // small launches). Waiting moves only when the step runs.
            bool &started = op.kind == OP_FWD ? q.fwdStarted : q.revStarted;
            if (kAlignRebuilds && !started && ticks_ % q.spec.opts.interval != 0) {
                --q.pc;
                continue;
            }
            started = true;
            parts.push_back({&q, op});
        }
        ++ticks_;
        if (parts.empty()) return 0;
        const int P = (int)parts.size();
        if (P > kMaxPackSys)
            throw Error(ERR_STATE, "more requests in flight than one tick holds (" +
                                       std::to_string(kMaxPackSys) + ")");

        // descriptors, and the block lists of each grouped launch
        std::vector<GSys<T>> sys((size_t)P);
        struct List {
            std::vector<int32_t> sys, start{0};
            void add(int k, int64_t blocks)
            {
                if (blocks <= 0) return;
                sys.push_back(k);
                start.push_back(start.back() + (int32_t)blocks);
            }
            int32_t blocks() const { return start.back(); }
        };
        List lGather, lCells, lScanTop, lScanTile, lPart, lAll, lRev, lTheta, lFwd;
        bool anyAV = false;
        auto nb = [](int64_t n, int b) { return (n + b - 1) / b; };
        for (int k = 0; k < P; ++k) {
            Req &q = *parts[k].q;
            const bool rev = parts[k].op.kind == OP_REV;
            Sys<T> &Y = rev ? *q.S : *q.F;
            GSys<T> &d = sys[(size_t)k];
            std::memset(&d, 0, sizeof(d));
            const int64_t N = Y.N_;
            const bool rebuild = Y.age >= Y.opts.interval;
            const int pre = Y.cur, post = rebuild ? 1 - pre : pre;
            d.n = N;
            d.ncell = Y.ncell;
            d.mode = rev ? 1 : 0;
            d.check = Y.age != INT64_MAX ? 1 : 0;
            d.posPre = Y.pos[pre].p;
            d.velPre = Y.vel[pre].p;
            d.posN = Y.pos[post].p;
            d.velN = Y.vel[post].p;
            d.vel = Y.vel[post].p;
            d.xref = Y.xref.p;
            d.perm = Y.perm.p;
            d.invperm = Y.invperm.p;
            d.cellStart = Y.cellStart.p;
            d.cellTmp = Y.cellTmp.p;
            d.counts = Y.counts.p;
            d.cursor = Y.cursor.p;
            d.bucketSrc = Y.bucketSrc.p;
            d.bucketId = Y.bucketId.p;
            d.scanTmp = Y.scanTmp.p;
            d.nbcount = Y.nbcount.p;
            d.center = Y.center.p;
            d.masks = Y.masks.p;
            d.tmask = Y.tmask.p;
            d.flags = Y.flags.p;
            d.prho = Y.prho.p;
            d.rhoAll = Y.rho.p;
            d.theta = q.th->th.p;
            NLView<T> v = Y.view();
            v.pos = Y.pos[post].p;
            v.tmask = Y.tmask.p;
            v.inst = nullptr;
            v.pinst = nullptr;
            d.v = v;
            anyAV = anyAV || Y.anyAV;
            if (!rev) {
                d.rho = Y.rho.p;
                d.posOut = Y.pos[1 - post].p;
                d.velOut = Y.vel[1 - post].p;
                if (parts[k].op.n >= 0) {
                    d.tx = q.tape->hx.p + (size_t)parts[k].op.n * N;
                    d.tv = q.tape->hv.p + (size_t)parts[k].op.n * N;
                }
            } else {
                Work<T> &W = *q.W;
                d.rho = Y.anyRho ? Y.rho.p : nullptr;
                if (parts[k].op.n >= 0) {
                    d.sx = q.tape->hx.p + (size_t)parts[k].op.n * N;
                    d.sv = q.tape->hv.p + (size_t)parts[k].op.n * N;
                    d.srcInv = nullptr;
                } else {
                    Sys<T> &F = *q.F;
                    d.sx = F.pos[F.cur].p;
                    d.sv = F.vel[F.cur].p;
                    d.srcInv = F.invperm.p;
                }
                const int g2 = 1 - q.gcur;
                if (rebuild) {
                    d.ex0 = W.gX[q.gcur].p;
                    d.ex0N = W.gX[g2].p;
                    d.ex1 = W.gV[q.gcur].p;
                    d.ex1N = W.gV[g2].p;
                    q.gcur = g2;
                }
                d.gX = W.gX[q.gcur].p;
                d.gV = W.gV[q.gcur].p;
                d.abar = W.abar.p;
                d.gXs = W.gXs.p;
                d.galpha = W.galpha.p;
                d.grho = W.grho.p;
                d.emax = W.emax.p;
                d.parity = (int)(q.rstep & 1);
                d.thetaAcc = W.thetaAcc.p;
                d.gtheta = W.gtheta.p;
                d.nnode = W.nnode;
                lGather.add(k, nb(N, kPackBlock));
                lRev.add(k, nb(N, kPackBlock));
                lTheta.add(k, nb(W.nnode, kBlock));
                q.rstep += 1;
            }
            if (rebuild && N > 0) {
                lCells.add(k, nb(d.ncell, kBlock));
                lScanTop.add(k, 1);
                lScanTile.add(k, nb(d.ncell, kScanTile));
                lPart.add(k, nb(N, kPackBlock));
            }
            lAll.add(k, nb(N, kPackBlock));
            if (!rev) lFwd.add(k, nb(N, kPackBlock));
            // host bookkeeping of maybe_rebuild! and the step
            if (rebuild) Y.age = 0;
            Y.age += 1;
            Y.cellsOnlyLatest = false;
            Y.cur = rev ? post : 1 - post;
        }

        // upload: the block lists, then the descriptors, into the constant table
        Ring &R = ring_[ringPos_];
        ringPos_ = (ringPos_ + 1) % kRing;
        if (R.used) SPH_CK(cudaEventSynchronize(R.ev));
        const List *lists[kPackLists] = {&lGather, &lCells, &lScanTop, &lScanTile, &lPart,
                                         &lAll, &lRev, &lTheta, &lFwd};
        const size_t bytes = sizeof(PackLists) + sizeof(GSys<T>) * (size_t)P;
        if (!R.host) {
            SPH_CK(cudaHostAlloc((void **)&R.host, sizeof(PackTable<T>), cudaHostAllocDefault));
            SPH_CK(cudaEventCreateWithFlags(&R.ev, cudaEventDisableTiming));
        }
        PackTable<T> *tab = reinterpret_cast<PackTable<T> *>(R.host);
        for (int li = 0; li < kPackLists; ++li) {
            const List &l = *lists[li];
            tab->L.cnt[li] = (int32_t)l.sys.size();
            std::copy(l.sys.begin(), l.sys.end(), tab->L.sys[li]);
            std::copy(l.start.begin(), l.start.end(), tab->L.start[li]);
        }
        std::memcpy(tab->sys, sys.data(), sizeof(GSys<T>) * (size_t)P);
        cudaStream_t st = rt_stream();
        SPH_CK(cudaMemcpyToSymbolAsync(c_pack, R.host, bytes, 0, cudaMemcpyHostToDevice, st));
        auto launch = [&](int kid, int li, int bs, auto kern) {
            const List &l = *lists[li];
            if (l.blocks() <= 0) return;
            rt_before_launch(kid);
            launch_k(kern, dim3((unsigned)l.blocks()), dim3(bs), 0, li);
            rt_after_launch(kid);
            ++launches_;
        };
        launch(K_GATHER, PL_GATHER, kPackBlock, g_gather<T>);
        launch(K_ASSIGN, PL_CELLS, kBlock, g_zero_counts<T>);
        launch(K_ASSIGN, PL_PART, kPackBlock, g_assign<T>);
        launch(K_SCAN, PL_SCANTILE, kBlock, g_scan_reduce<T>);
        launch(K_SCAN, PL_SCANTOP, kBlock, g_scan_top<T>);
        launch(K_SCAN, PL_SCANTILE, kBlock, g_scan_down<T>);
        launch(K_BUCKET, PL_PART, kPackBlock, g_bucket<T>);
        launch(K_RANK, PL_PART, kPackBlock, g_rank<T>);
        launch(K_NLBUILD, PL_PART, kPackBlock, g_nl_build<T>);
        launch(K_DENSITY, PL_ALL, kPackBlock, g_density<T>);
        if (anyAV) launch(K_ACCEL_INTEGRATE, PL_FWD, kPackBlock, g_accel_fwd<T, true>);
        else launch(K_ACCEL_INTEGRATE, PL_FWD, kPackBlock, g_accel_fwd<T, false>);
        if (anyAV) launch(K_ACCEL_DRAG, PL_REV, kPackBlock, g_accel_rev<T, true>);
        else launch(K_ACCEL_DRAG, PL_REV, kPackBlock, g_accel_rev<T, false>);
        if (anyAV) launch(K_PASS1, PL_REV, kPackBlock, g_pass1<T, true>);
        else launch(K_PASS1, PL_REV, kPackBlock, g_pass1<T, false>);
        launch(K_PASS2, PL_REV, kPackBlock, g_pass2<T>);
        launch(K_THETA_NODE, PL_THETA, kBlock, g_theta<T>);
        SPH_CK(cudaEventRecord(R.ev, st));
        R.used = true;
        rt_check_launch("packed tick");
        return P;
    }

    // Requests whose programs have ended on the device.
    void reap(std::vector<int> &done, bool block) override
    {
        for (auto &kv : reqs_) {
            Req &q = *kv.second;
            if (!q.finishing) continue;
            cudaError_t e = block ? cudaEventSynchronize(q.done) : cudaEventQuery(q.done);
            if (e == cudaSuccess) {
                done.push_back(kv.first);
                block = false;
            } else if (e != cudaErrorNotReady) {
                cuda_check(e, "request completion");
            }
        }
    }

    int finishing() const override
    {
        int n = 0;
        for (auto &kv : reqs_) n += kv.second->finishing ? 1 : 0;
        return n;
    }

    // results of a finished request, copied on the calling thread's own copy
    // stream (they are complete: its completion event has fired)
    void result(int id, cudaStream_t cs, double *J, uint32_t *flags, void *gX, void *gV,
                void *gth) override
    {
        Req &q = *reqs_.at(id);
        Work<T> &W = *q.W;
        double j = 0.0;
        uint32_t f[2] = {0u, 0u};
        SPH_CK(cudaMemcpyAsync(&j, W.partial.p + W.jOff, sizeof(double), cudaMemcpyDeviceToHost, cs));
        SPH_CK(cudaMemcpyAsync(&f[0], q.F->flags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, cs));
        if (q.S) SPH_CK(cudaMemcpyAsync(&f[1], q.S->flags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, cs));
        const int64_t N = q.spec.N;
        if (q.spec.adjoint) {
            if (gX) SPH_CK(cudaMemcpyAsync(gX, W.outX.p, sizeof(T2<T>) * N, cudaMemcpyDeviceToHost, cs));
            if (gV) SPH_CK(cudaMemcpyAsync(gV, W.outV.p, sizeof(T2<T>) * N, cudaMemcpyDeviceToHost, cs));
            if (gth) SPH_CK(cudaMemcpyAsync(gth, W.gthetaT.p, W.gthetaT.bytes(), cudaMemcpyDeviceToHost, cs));
        }
        SPH_CK(cudaStreamSynchronize(cs));
        if (J) *J = N ? j : 0.0;
        if (flags) *flags = f[0] | f[1];
    }

    void release(int id) override { reqs_.erase(id); }
};

} // namespace sphgb
