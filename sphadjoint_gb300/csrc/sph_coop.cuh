// Group-per-particle variants of the neighbour-list and pair-sum kernels, for
// single states too small to fill the GPU one thread per particle (a 2072-
// particle dam break runs 17 blocks; in FP64 those 17 SMs are bound by the
// double-precision pipe while 135 SMs idle). With 16-lane groups the same
// state runs 259 blocks of 128 threads on every SM and its pass-1 kernel
// keeps the FP64 pipe ~70% busy.
//
// A group of G lanes (16 or 32) owns one particle. The particle's candidate
// neighbours (the set bits of its six mask words, in slot order = the
// reference's scan order) are dealt out G at a time: lane g of round r takes
// candidate r*G + g and computes that pair's terms with the same per-pair
// functions as the thread-per-particle kernels. The terms go to shared
// memory, and one lane per running sum adds them in candidate order, so
// every sum sees exactly the operations and the order of the serial loop:
// results are bit-identical to the thread-per-particle kernels (and, in the
// FP64 build, to the reference's). A particle whose rows spill past 64 slots
// (a compressed region: the small dam break has up to ~130 of them while its
// front runs along the floor) has masks for the first 64 slots only; its group scans the rows, keeps
// the reference's row in slot order in shared memory and deals that list out
// the same way (the serial path on one lane, used before, made those steps
// 6-10x slower). Only a row limit maxnb above kSpillList falls back to the
// serial walk on the group's first lane.
#pragma once

#include "sph_kernels.cuh"

namespace sphgb {

constexpr int kCoopBlock = 128;
constexpr int kSpillList = 64; // neighbour list of a spilled particle, in shared memory

// Lanes of one group inside its warp.
template <int G> struct Group {
    int gl;         // lane within the group
    int gi;         // group within the block
    int shift;      // first warp lane of the group
    unsigned mask;  // warp lanes of the group
    __device__ __forceinline__ Group()
    {
        const int lane = (int)(threadIdx.x & 31u);
        gl = lane & (G - 1);
        gi = (int)threadIdx.x / G;
        shift = lane & ~(G - 1);
        mask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << shift);
    }
    __device__ __forceinline__ unsigned ballot(bool p) const
    {
        return __ballot_sync(mask, p) >> shift;
    }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    template <typename V> __device__ __forceinline__ V from(V x, int src) const
    {
        return __shfl_sync(mask, x, src, G);
    }
};

// The candidates of a particle, numbered 0..total-1 in slot order: the set
// bits of its six words (row r = words 2r, 2r+1), or for a spilled particle
// the list spill_list built.
template <typename T> struct Cands {
    uint32_t wd[6];
    int bs[6];  // slot of bit 0 of each word
    int pre[7]; // candidates before each word
    const int32_t *lst; // spilled particle: its neighbour slots (shared memory)
    int nl;
    __device__ __forceinline__ void init_list(const int32_t *l, int n)
    {
        lst = l;
        nl = n;
    }
    __device__ __forceinline__ void init(const NLView<T> &v, const Inst<T> &I, int64_t i,
                                         uint32_t cc, const uint32_t *__restrict__ mk)
    {
        lst = nullptr;
        const int cx = (int)(cc & 0xffffu);
        const int cy = (int)((cc >> 16) & 0x7fffu);
        const int jx0 = cx - 1 > 1 ? cx - 1 : 1;
        const int row0 = I.coff + (jx0 - 1) + (cy - 2) * I.nx; // cell (jx0, cy - 1)
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            wd[2 * r] = mk[(int64_t)(2 * r) * v.N + i];
            wd[2 * r + 1] = mk[(int64_t)(2 * r + 1) * v.N + i];
            const int b = (wd[2 * r] | wd[2 * r + 1]) ? v.cellStart[row0 + r * I.nx] : 0;
            bs[2 * r] = b;
            bs[2 * r + 1] = b + 32;
        }
        pre[0] = 0;
#pragma unroll
        for (int w = 0; w < 6; ++w) pre[w + 1] = pre[w] + __popc(wd[w]);
    }
    __device__ __forceinline__ int total() const { return lst ? nl : pre[6]; }
    // slot of candidate k < total(); w, bit: its word and bit (w = -1 for a
    // listed candidate: a spilled particle has no in-support words)
    __device__ __forceinline__ int slot(int k, int &w, int &bit) const
    {
        if (lst) {
            w = -1;
            bit = 0;
            return lst[k];
        }
        uint32_t word = wd[0];
        int base = bs[0], rem = k;
        w = 0;
#pragma unroll
        for (int q = 1; q < 6; ++q)
            if (k >= pre[q]) {
                word = wd[q];
                base = bs[q];
                rem = k - pre[q];
                w = q;
            }
        bit = select_bit(word, rem);
        return base + bit;
    }
};

// The neighbour row of a spilled particle as the generic walk of
// for_each_neighbor visits it: r2min < r^2 < rc^2 on the rebuild positions,
// rows ddy = -1..1, slot order, at most maxnb (<= kSpillList) entries. Each
// round tests G consecutive slots; a ballot gives the kept ones, which are
// written to lst at their rank. Returns the count (the same on every lane).
template <typename T, int G>
__device__ __forceinline__ int spill_list(const Group<G> &g, const NLView<T> &v,
                                          const Inst<T> &I, int64_t i, uint32_t cc,
                                          int32_t *__restrict__ lst)
{
    const int cx = (int)(cc & 0xffffu);
    const int cy = (int)((cc >> 16) & 0x7fffu);
    const int jx0 = cx - 1 > 1 ? cx - 1 : 1;
    const int jx1 = cx + 1 < I.nx ? cx + 1 : I.nx;
    const T2<T> xr = v.xref[i];
    const int maxnb = I.maxnb;
    int cnt = 0;
#pragma unroll 1
    for (int r = 0; r < 3; ++r) {
        const int jy = cy + r - 1;
        if (jy < 1 || jy > I.ny) continue;
        const int row = I.coff + (jy - 1) * I.nx;
        const int b = v.cellStart[row + jx0 - 1];
        const int e = v.cellStart[row + jx1];
        for (int base = b; base < e && cnt < maxnb; base += G) {
            const int j = base + g.gl;
            bool pass = false;
            if (j < e) {
                const T2<T> xj = v.xref[j];
                const T r2 = r2_exact<T>(sub_rn(xr.x, xj.x), sub_rn(xr.y, xj.y));
                pass = lt_nonneg(I.r2min, r2) && lt_nonneg(r2, I.rc2);
            }
            uint32_t kept = g.ballot(pass);
            const int room = maxnb - cnt;
            if (__popc(kept) > room) kept &= (1u << select_bit(kept, room)) - 1u;
            if ((kept >> g.gl) & 1u) lst[cnt + __popc(kept & ((1u << g.gl) - 1u))] = j;
            cnt += __popc(kept);
        }
    }
    g.sync();
    return cnt;
}

// _nl_build! (src/neighbors.jl:192-245) with the row scan spread over the
// group: each round tests G consecutive slots, a ballot gives the passing
// ones, and the first (maxnb - kept) of them are kept, in slot order.
template <typename T, int G>
__global__ void __launch_bounds__(kCoopBlock)
    k_nl_build_coop(int64_t N, const Inst<T> I, const T2<T> *__restrict__ pos,
                    const int32_t *__restrict__ cellStart, uint32_t *__restrict__ center,
                    uint32_t *__restrict__ masks, int32_t *__restrict__ nbcount,
                    uint32_t *__restrict__ flags)
{
    pdl_enter();
    const Group<G> g;
    const int64_t i = (int64_t)blockIdx.x * (kCoopBlock / G) + g.gi;
    if (i >= N) return; // the whole group
    const int nx = I.nx, ny = I.ny, maxnb = I.maxnb;
    const T rc2 = I.rc2, r2min = I.r2min;
    const T2<T> xi = pos[i];
    const int cx = cell_coord<T>(xi.x * I.invcs, nx);
    const int cy = cell_coord<T>(xi.y * I.invcs, ny);
    const int jx0 = cx - 1 > 1 ? cx - 1 : 1;
    const int jx1 = cx + 1 < nx ? cx + 1 : nx;
    uint32_t spill = 0;
    int m = 0;
    bool over = false;
#pragma unroll 1
    for (int r = 0; r < 3; ++r) {
        uint32_t lo = 0, hi = 0;
        const int jy = cy + r - 1;
        if (jy >= 1 && jy <= ny) {
            const int row = I.coff + (jy - 1) * nx;
            const int b = cellStart[row + jx0 - 1];
            const int e = cellStart[row + jx1];
            if (e - b > 64) spill = 1;
            for (int base = b; base < e; base += G) {
                const int j = base + g.gl;
                bool pass = false;
                if (j < e) {
                    const T2<T> xj = pos[j];
                    const T r2 = r2_exact<T>(sub_rn(xi.x, xj.x), sub_rn(xi.y, xj.y));
                    pass = lt_nonneg(r2min, r2) && lt_nonneg(r2, rc2);
                }
                uint32_t kept = g.ballot(pass);
                const int np = __popc(kept), room = maxnb - m;
                if (np > room) {
                    over = true;
                    kept = room > 0 ? kept & ((1u << select_bit(kept, room)) - 1u) : 0u;
                }
                m += __popc(kept);
                const int off = base - b;
                if (off < 64) {
                    const uint64_t w64 = (uint64_t)kept << off;
                    lo |= (uint32_t)w64;
                    hi |= (uint32_t)(w64 >> 32);
                }
            }
        }
        if (g.gl == 0) {
            masks[(int64_t)(2 * r) * N + i] = lo;
            masks[(int64_t)(2 * r + 1) * N + i] = hi;
        }
    }
    if (g.gl == 0) {
        center[i] = (uint32_t)cx | ((uint32_t)cy << 16) | (spill << 31);
        nbcount[i] = m;
        if (over) atomicOr(flags, FLAG_NL_OVERFLOW);
    }
}

// density_kernel! + eos_kernel!, and this step's in-support words.
template <typename T, int G>
__global__ void __launch_bounds__(kCoopBlock)
    k_density_eos_coop(const __grid_constant__ NLView<T> v, T *__restrict__ rho,
                       T2<T> *__restrict__ prho, uint32_t *__restrict__ tmaskOut)
{
    pdl_enter();
    constexpr int NG = kCoopBlock / G;
    __shared__ T buf[NG][G];
    __shared__ uint32_t tws[NG][6];
    __shared__ int32_t lst[NG][kSpillList];
    const Group<G> g;
    const int64_t i = (int64_t)blockIdx.x * NG + g.gi;
    if (i >= v.N) return;
    const Inst<T> &I = v.one;
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, A = I.p.A;
    const T2<T> xi = v.pos[i];
    const uint32_t cc = v.center[i];
    if ((cc >> 31) && I.maxnb > kSpillList) {
        if (g.gl == 0) density_finish<T>(I, i, density_spill_sum<T>(v, I, i, xi, tmaskOut), rho, prho);
        return;
    }
    Cands<T> cd;
    if (cc >> 31) cd.init_list(lst[g.gi], spill_list<T, G>(g, v, I, i, cc, lst[g.gi]));
    else cd.init(v, I, i, cc, v.masks);
    const int K = cd.total();
    if (g.gl < 6) tws[g.gi][g.gl] = 0u;
    g.sync();
    T acc = (T)0;
    for (int base = 0; base < K; base += G) {
        const int k = base + g.gl;
        T c = (T)0;
        bool in = false;
        if (k < K) {
            int w, bit;
            const T2<T> xj = v.pos[cd.slot(k, w, bit)];
            const T dx = xi.x - xj.x;
            const T dy = xi.y - xj.y;
            const T r2 = dx * dx + dy * dy;
            if (lt_nonneg(r2, r2max)) {
                in = true;
                c = density_pair<T>(r2, invh, m, A);
                if (w >= 0) atomicOr(&tws[g.gi][w], 1u << bit);
            }
        }
        buf[g.gi][g.gl] = c;
        const unsigned inm = g.ballot(in);
        g.sync();
        if (g.gl == 0) {
            const int n = K - base < G ? K - base : G;
            for (int t = 0; t < n; ++t)
                if ((inm >> t) & 1u) acc += buf[g.gi][t];
        }
        g.sync();
    }
    if (tmaskOut && g.gl < 6) tmaskOut[(int64_t)g.gl * v.N + i] = tws[g.gi][g.gl];
    if (g.gl == 0) density_finish<T>(I, i, acc, rho, prho);
}

// Pressure + viscosity pair sum of one particle by its group; lane 0 returns
// (ax, ay).
// The candidates of particle i for a pass after the density pass: this step's
// in-support words, or for a spilled particle its listed row.
template <typename T, int G>
__device__ __forceinline__ Cands<T> pass_cands(const Group<G> &g, const NLView<T> &v,
                                               const Inst<T> &I, int64_t i, uint32_t cc,
                                               int32_t *__restrict__ lst)
{
    Cands<T> cd;
    if (cc >> 31) cd.init_list(lst, spill_list<T, G>(g, v, I, i, cc, lst));
    else cd.init(v, I, i, cc, v.tmask ? v.tmask : v.masks);
    return cd;
}

template <typename T, int G, int NG>
__device__ __forceinline__ void accel_sum_coop(const Group<G> &g, T (*buf)[4][G],
                                               const NLView<T> &v, const Inst<T> &I, int64_t i,
                                               const Cands<T> &cd, const T2<T> *__restrict__ vel,
                                               const T2<T> *__restrict__ prho,
                                               const T *__restrict__ rho, const T2<T> &xi,
                                               const T2<T> &vi, T &ax, T &ay)
{
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, Fc = I.p.Fc;
    const Visc<T> vc = visc_of<T>(I);
    const T2<T> pi = prho[i];
    const T pti = pi.x, iri = pi.y;
    const T rhoi = vc.kind == 1 ? rho[i] : (T)0;
    const int K = cd.total();
    T acc = (T)0; // lane 0: ax, lane 1: ay
    for (int base = 0; base < K; base += G) {
        const int k = base + g.gl;
        AccelPair<T> t = {(T)0, (T)0, (T)0, (T)0};
        bool in = false;
        if (k < K) {
            int w, bit;
            const int j = cd.slot(k, w, bit);
            const T2<T> xj = v.pos[j];
            const T dx = xi.x - xj.x;
            const T dy = xi.y - xj.y;
            const T r2 = dx * dx + dy * dy;
            if (lt_nonneg(r2, r2max)) {
                in = true;
                const T rhoj = vc.kind == 1 ? rho[j] : (T)0;
                t = accel_pair<T>(r2, dx, dy, invh, m, Fc, vc, pti, iri, rhoi, rhoj, vi, prho[j],
                                  vel[j]);
            }
        }
        buf[g.gi][0][g.gl] = t.px;
        buf[g.gi][1][g.gl] = t.py;
        buf[g.gi][2][g.gl] = t.cx;
        buf[g.gi][3][g.gl] = t.cy;
        const unsigned inm = g.ballot(in);
        g.sync();
        if (g.gl < 2) {
            const int n = K - base < G ? K - base : G;
            const T *ps = buf[g.gi][g.gl];
            const T *cs = buf[g.gi][2 + g.gl];
            for (int t2 = 0; t2 < n; ++t2)
                if ((inm >> t2) & 1u) {
                    acc -= ps[t2];
                    acc += cs[t2];
                }
        }
        g.sync();
    }
    ax = acc;
    ay = g.from(acc, 1);
}

// accel_kernel! + integrate_kernel!
template <typename T, int G>
__global__ void __launch_bounds__(kCoopBlock)
    k_accel_integrate_coop(const __grid_constant__ NLView<T> v, const T2<T> *__restrict__ vel,
                           const T2<T> *__restrict__ prho, const T *__restrict__ rho,
                           const T *__restrict__ theta,
                           T2<T> *__restrict__ posOut, T2<T> *__restrict__ velOut,
                           T2<T> *__restrict__ aOut, T *__restrict__ alphaOut,
                           uint32_t *__restrict__ flags, const int32_t *__restrict__ perm,
                           T2<T> *__restrict__ tx, T2<T> *__restrict__ tv)
{
    pdl_enter();
    constexpr int NG = kCoopBlock / G;
    __shared__ T buf[NG][4][G];
    __shared__ int32_t lst[NG][kSpillList];
    const Group<G> g;
    const int64_t i = (int64_t)blockIdx.x * NG + g.gi;
    if (i >= v.N) return;
    const Inst<T> &I = v.one;
    const T2<T> xi = v.pos[i];
    const T2<T> vi = vel[i];
    const uint32_t cc = v.center[i];
    T ax, ay;
    if ((cc >> 31) && I.maxnb > kSpillList) {
        if (g.gl != 0) return;
        accel_sum<T, true>(v, I, vel, prho, rho, i, xi, vi, ax, ay);
    } else {
        const Cands<T> cd = pass_cands<T, G>(g, v, I, i, cc, lst[g.gi]);
        accel_sum_coop<T, G, NG>(g, buf, v, I, i, cd, vel, prho, rho, xi, vi, ax, ay);
        if (g.gl != 0) return;
    }
    accel_integrate_finish<T>(I, 0, i, xi, vi, ax, ay, theta, posOut, velOut, aOut, alphaOut, flags,
                              perm, tx, tv);
}

// Accel recompute + _adj_integrate! + _adj_drag!; one exponent update per
// particle (these launches cover few particles).
template <typename T, int G>
__global__ void __launch_bounds__(kCoopBlock)
    k_accel_drag_adj_coop(const __grid_constant__ NLView<T> v, const T2<T> *__restrict__ vel,
                          const T2<T> *__restrict__ prho, const T *__restrict__ rho,
                          const T *__restrict__ theta,
                          const T2<T> *__restrict__ gX, T2<T> *__restrict__ gV,
                          T2<T> *__restrict__ abar, T *__restrict__ galpha,
                          int *__restrict__ emax, int parity)
{
    pdl_enter();
    constexpr int NG = kCoopBlock / G;
    __shared__ T buf[NG][4][G];
    __shared__ int32_t lst[NG][kSpillList];
    const Group<G> g;
    const int64_t i = (int64_t)blockIdx.x * NG + g.gi;
    if (i >= v.N) return;
    const Inst<T> &I = v.one;
    const T2<T> xi = v.pos[i];
    const T2<T> vi = vel[i];
    const uint32_t cc = v.center[i];
    T ax, ay;
    if ((cc >> 31) && I.maxnb > kSpillList) {
        if (g.gl != 0) return;
        accel_sum<T, true>(v, I, vel, prho, rho, i, xi, vi, ax, ay);
    } else {
        const Cands<T> cd = pass_cands<T, G>(g, v, I, i, cc, lst[g.gi]);
        accel_sum_coop<T, G, NG>(g, buf, v, I, i, cd, vel, prho, rho, xi, vi, ax, ay);
        if (g.gl != 0) return;
    }
    const int e = drag_adj_finish<T>(I, i, xi, vi, ax, ay, theta, gX, gV, abar, galpha);
    if (e != INT_MIN) atomicMax(emax + parity, e);
}

// adj_pass1_kernel! + the gXs half of adj_design_kernel! + _axpy2!(gV, gVs).
// Lanes 0..5 keep gx, gy, gvx, gvy, grho, S.
template <typename T, int G>
__global__ void __launch_bounds__(kCoopBlock)
    k_pass1_design_coop(const __grid_constant__ NLView<T> v, const T2<T> *__restrict__ vel,
                        const T2<T> *__restrict__ prho, const T *__restrict__ rho,
                        const T *__restrict__ theta,
                        const T2<T> *__restrict__ abar, const T *__restrict__ galpha,
                        T2<T> *__restrict__ gXs, T *__restrict__ grho, T2<T> *__restrict__ gV)
{
    pdl_enter();
    constexpr int NG = kCoopBlock / G;
    __shared__ T buf[NG][9][G]; // eight term slots and a row of zeros
    __shared__ int32_t lst[NG][kSpillList];
    const Group<G> g;
    const int64_t i = (int64_t)blockIdx.x * NG + g.gi;
    if (i >= v.N) return;
    const Inst<T> &I = v.one;
    const T2<T> xi = v.pos[i];
    const T2<T> vi = vel[i];
    const T2<T> ab = abar[i];
    const T2<T> pi = prho[i];
    const uint32_t cc = v.center[i];
    T gx, gy, gvx, gvy, grh, sumS;
    if ((cc >> 31) && I.maxnb > kSpillList) {
        if (g.gl != 0) return;
        pass1_sum<T, true>(v, I, i, vel, prho, rho, abar, xi, vi, ab, pi, gx, gy, gvx, gvy, grh,
                           sumS);
    } else {
        const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, Fc = I.p.Fc, Gc = I.p.Gc;
        const Visc<T> vc = visc_of<T>(I);
        const T pti = pi.x, iri = pi.y;
        const T rhoi = vc.kind == 1 ? rho[i] : (T)0;
        const Cands<T> cd = pass_cands<T, G>(g, v, I, i, cc, lst[g.gi]);
        const int K = cd.total();
        // term slots: 0 gx-, 1 gx+, 2 gy-, 3 gy+, 4 gvx+, 5 gvy+, 6 grho-, 7 S+,
        // 8 zeros. Every running sum takes "minus one slot, plus one slot" per
        // pair, a zero where it has no such term: a sum that starts at +0 never
        // becomes -0, so x - 0 and x + 0 leave it unchanged and each sum sees
        // exactly the serial loop's operations, while all six fold lanes run
        // the same instructions.
        T(*b)[G] = buf[g.gi];
        b[8][g.gl] = (T)0;
        const int fold = g.gl < 6 ? g.gl : 0;
        const T *fsub = b[fold == 0 ? 0 : fold == 1 ? 2 : fold == 4 ? 6 : 8];
        const T *fadd = b[fold == 0 ? 1 : fold == 1 ? 3 : fold == 2 ? 4 : fold == 3 ? 5 : fold == 5 ? 7 : 8];
        T acc = (T)0;
        for (int base = 0; base < K; base += G) {
            const int k = base + g.gl;
            Pass1Pair<T> t = {(T)0, (T)0, (T)0, (T)0, (T)0, (T)0, (T)0, (T)0};
            bool in = false;
            if (k < K) {
                int w, bit;
                const int j = cd.slot(k, w, bit);
                const T2<T> xj = v.pos[j];
                const T dx = xi.x - xj.x;
                const T dy = xi.y - xj.y;
                const T r2 = dx * dx + dy * dy;
                if (lt_nonneg(r2, r2max)) {
                    in = true;
                    const T rhoj = vc.kind == 1 ? rho[j] : (T)0;
                    t = pass1_pair<T>(r2, dx, dy, invh, m, Fc, Gc, vc, pti, iri, rhoi, rhoj, vi,
                                      ab, prho[j], abar[j], vel[j]);
                }
            }
            b[0][g.gl] = t.gxs;
            b[1][g.gl] = t.gxa;
            b[2][g.gl] = t.gys;
            b[3][g.gl] = t.gya;
            b[4][g.gl] = t.gvx;
            b[5][g.gl] = t.gvy;
            b[6][g.gl] = t.grs;
            b[7][g.gl] = t.sS;
            const unsigned inm = g.ballot(in);
            g.sync();
            if (g.gl < 6) {
                const int n = K - base < G ? K - base : G;
                for (int t2 = 0; t2 < n; ++t2)
                    if ((inm >> t2) & 1u) {
                        acc -= fsub[t2];
                        acc += fadd[t2];
                    }
            }
            g.sync();
        }
        gx = acc;
        gy = g.from(acc, 1);
        gvx = g.from(acc, 2);
        gvy = g.from(acc, 3);
        grh = g.from(acc, 4);
        sumS = g.from(acc, 5);
        if (g.gl != 0) return;
    }
    const T rhoi = needs_rho_dev(I) ? rho[i] : (T)0;
    pass1_finish<T>(I, i, xi, ab, pi, rhoi, gx, gy, gvx, gvy, grh, sumS, theta, galpha, gXs, grho,
                    gV);
}

// adj_pass2_kernel! + _axpy2!(gX, gXs) + the exact theta write-back.
template <typename T, int G>
__global__ void __launch_bounds__(kCoopBlock)
    k_pass2_axpy_coop(const __grid_constant__ NLView<T> v, const T *__restrict__ grho,
                      const T2<T> *__restrict__ gXs, T2<T> *__restrict__ gX,
                      const T *__restrict__ galpha, const int *__restrict__ emax, int parity,
                      unsigned long long *__restrict__ thetaAcc)
{
    pdl_enter();
    constexpr int NG = kCoopBlock / G;
    __shared__ T buf[NG][2][G];
    __shared__ int32_t lst[NG][kSpillList];
    const Group<G> g;
    const int64_t i = (int64_t)blockIdx.x * NG + g.gi;
    if (i >= v.N) return;
    const Inst<T> &I = v.one;
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, Fc = I.p.Fc;
    const T2<T> xi = v.pos[i];
    const T gri = grho[i];
    const uint32_t cc = v.center[i];
    T gx = (T)0, gy = (T)0;
    if ((cc >> 31) && I.maxnb > kSpillList) {
        if (g.gl != 0) return;
        for_each_neighbor<T>(v, I, i, [&](int j) {
            const T2<T> xj = v.pos[j];
            const T dx = xi.x - xj.x;
            const T dy = xi.y - xj.y;
            const T r2 = dx * dx + dy * dy;
            if (lt_nonneg(r2, r2max)) {
                const T w = pass2_weight<T>(r2, invh, m, Fc, gri, grho[j]);
                gx += w * dx;
                gy += w * dy;
            }
        });
    } else {
        const Cands<T> cd = pass_cands<T, G>(g, v, I, i, cc, lst[g.gi]);
        const int K = cd.total();
        T acc = (T)0;
        for (int base = 0; base < K; base += G) {
            const int k = base + g.gl;
            T tx = (T)0, ty = (T)0;
            bool in = false;
            if (k < K) {
                int w, bit;
                const int j = cd.slot(k, w, bit);
                const T2<T> xj = v.pos[j];
                const T dx = xi.x - xj.x;
                const T dy = xi.y - xj.y;
                const T r2 = dx * dx + dy * dy;
                if (lt_nonneg(r2, r2max)) {
                    in = true;
                    const T wt = pass2_weight<T>(r2, invh, m, Fc, gri, grho[j]);
                    tx = wt * dx;
                    ty = wt * dy;
                }
            }
            buf[g.gi][0][g.gl] = tx;
            buf[g.gi][1][g.gl] = ty;
            const unsigned inm = g.ballot(in);
            g.sync();
            if (g.gl < 2) {
                const int n = K - base < G ? K - base : G;
                const T *src = buf[g.gi][g.gl];
                for (int t2 = 0; t2 < n; ++t2)
                    if ((inm >> t2) & 1u) acc += src[t2];
            }
            g.sync();
        }
        gx = acc;
        gy = g.from(acc, 1);
        if (g.gl != 0) return;
    }
    pass2_finish<T>(I, 0, i, xi, gx, gy, gXs, gX, galpha, emax, parity, thetaAcc);
}

} // namespace sphgb
