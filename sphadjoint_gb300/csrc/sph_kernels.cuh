// sm_103a kernels of the forward + adjoint WCSPH step (one template, two
// instantiations: double with --fmad=false for reference-exact parity, float
// with contraction for throughput).
//
// Data layout in HBM (all arrays in *cell order* = the sorted order of the last
// rebuild, so every neighbour row is a contiguous slot range):
//   pos, vel, xref, abar, gX, gV, gXs : T2 per particle (8 B FP32 / 16 B FP64)
//   rho, galpha, grho                 : T per particle
//   prho                              : T2 {p/rho^2, 1/rho} per particle
//   perm / invperm                    : int32 slot -> particle id / id -> slot
//   center                            : uint32 per particle (cx | cy<<16 | spill<<31)
//   masks, tmask                      : 6 x uint32 per particle, word-major
//                                       (masks[w * N + i]; row r = words 2r, 2r+1);
//                                       tmask: this step's in-support subset
//   cellStart                         : int32 x (ncell + 1)
// Reference kernels restated: src/neighbors.jl:44-80,192-245 (cell list and
// neighbour list), src/forward.jl:25-147, src/adjoint.jl:30-228.
#pragma once

#include "sph_common.cuh"
#include "sph_fixed.cuh"

namespace sphgb {

constexpr int kBlock = 256;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Two FP32 lanes in one 64-bit register: Blackwell issues mul.rn.f32x2 and
// fma.rn.f32x2 as one instruction for both halves, each rounded as the scalar
// operation would be.
__device__ __forceinline__ float2 fmul2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

__device__ __forceinline__ float2 fsub2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

// FP32 pair sums of the reference model (Morris viscosity) in packed form:
// the x and y components of a pair's differences, force terms and running
// sums ride in one f32x2 register, so the pair loop issues one instruction
// where the scalar form issues two; each half rounds as the scalar
// operation with multiply-add contraction does.
constexpr bool kPackedPairs = true;

__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

// ---------------------------------------------------------------------------
// Exclusive scan (reduce-then-scan, three launches, no inter-block waits)
// ---------------------------------------------------------------------------
constexpr int kScanTile = 2048; // 256 threads x 8 items

__device__ __forceinline__ int32_t block_excl_scan(int32_t v, int32_t *smem_warp, int32_t &total)
{
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int32_t w = lane < (unsigned)nw ? smem_warp[lane] : 0;
        int32_t s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= (unsigned)o) s += y;
        }
        if (lane < (unsigned)nw) smem_warp[lane] = s - w;
        if (lane == (unsigned)nw - 1) smem_warp[32] = s;
    }
    __syncthreads();
    total = smem_warp[32];
    const int32_t r = x - v + smem_warp[warp];
    __syncthreads();
    return r;
}

static __global__ void k_scan_reduce(const int32_t *__restrict__ in, int64_t n, int32_t *__restrict__ bsum)
{
    pdl_enter();
    __shared__ int32_t sw[33];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanTile / kBlock; ++k) {
        const int64_t i = base + (int64_t)k * kBlock + threadIdx.x;
        if (i < n) s += in[i];
    }
    int32_t tot;
    block_excl_scan(s, sw, tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// single block: exclusive scan of nb block sums in place
static __global__ void k_scan_top(int32_t *__restrict__ bsum, int64_t nb)
{
    pdl_enter();
    __shared__ int32_t sw[33];
    int32_t carry = 0;
    for (int64_t base = 0; base < nb; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const int32_t v = i < nb ? bsum[i] : 0;
        int32_t tot;
        const int32_t e = block_excl_scan(v, sw, tot);
        if (i < nb) bsum[i] = e + carry;
        carry += tot;
    }
}

// out[i] = exclusive prefix; out[n] = total; out2 (optional) = copy of out[0..n)
static __global__ void k_scan_down(const int32_t *__restrict__ in, int64_t n,
                            const int32_t *__restrict__ bsum, int32_t *__restrict__ out,
                            int32_t *__restrict__ out2)
{
    pdl_enter();
    __shared__ int32_t sw[33];
    constexpr int IPT = kScanTile / kBlock;
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * IPT;
    int32_t v[IPT];
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int32_t tot;
    int32_t run = block_excl_scan(s, sw, tot) + (bsum ? bsum[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int64_t i = base + k;
        if (i < n) {
            out[i] = run;
            if (out2) out2[i] = run;
        }
        run += v[k];
        if (i == n - 1) out[n] = run;
    }
}

// ---------------------------------------------------------------------------
// Cell list: _cl_assign! / cumsum! / _cl_fill! / _cl_sort_cells!
// (src/neighbors.jl:44-114), fused with the permutation of particle data into
// the new cell order.
// ---------------------------------------------------------------------------

// Cell of every particle (division form x / cs as in cell_index), warp-
// aggregated histogram, and the displacement check of _nl_build!
// (src/neighbors.jl:207-213) against the previous rebuild positions. Cells are
// numbered in the packed table (instance offset + local cell).
template <typename T, bool MULTI>
__global__ void k_assign(int64_t N, const T2<T> *__restrict__ pos, const T2<T> *__restrict__ xref,
                         int check, const Inst<T> one, const Inst<T> *__restrict__ inst,
                         const uint16_t *__restrict__ pinst, int32_t *__restrict__ cellTmp,
                         int32_t *__restrict__ counts, uint32_t *__restrict__ flags)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < N;
    int32_t c = -1;
    if (live) {
        const int b = MULTI ? (int)pinst[i] : 0;
        decltype(auto) I = pick_inst<MULTI>(one, inst, b);
        const T2<T> x = pos[i];
        if (check) {
            const T2<T> xr = xref[i];
            const T d2 = r2_exact<T>(sub_rn(x.x, xr.x), sub_rn(x.y, xr.y));
            if (d2 > I.dmax2) atomicOr(flags + b, FLAG_DISPLACEMENT);
        }
        const T cs = I.cs;
        const int cx = cell_coord<T>(x.x / cs, I.nx);
        const int cy = cell_coord<T>(x.y / cs, I.ny);
        c = I.coff + (cx - 1) + (cy - 1) * I.nx;
        cellTmp[i] = c;
    }
    const unsigned act = __ballot_sync(0xffffffffu, live);
    if (live) {
        const unsigned peers = __match_any_sync(act, c);
        if ((int)lane_id() == __ffs(peers) - 1) atomicAdd(counts + c, __popc(peers));
    }
}

// Scatter every particle into its cell's bucket (arbitrary order inside the
// bucket; the rank step below makes it deterministic).
static __global__ void k_bucket(int64_t N, const int32_t *__restrict__ cellTmp,
                                const int32_t *__restrict__ perm, int32_t *__restrict__ cursor,
                                int32_t *__restrict__ bucketSrc, int32_t *__restrict__ bucketId)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < N;
    const int32_t c = live ? cellTmp[i] : -1;
    const unsigned act = __ballot_sync(0xffffffffu, live);
    if (!live) return;
    const unsigned peers = __match_any_sync(act, c);
    const int leader = __ffs(peers) - 1;
    int32_t base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(cursor + c, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    const int32_t pos = base + __popc(peers & ((1u << lane_id()) - 1u));
    bucketSrc[pos] = (int32_t)i;
    bucketId[pos] = perm[i];
}

// _cl_sort_cells! as a rank: each particle counts the smaller ids in its cell
// and moves its data straight to (cell start + rank) of the new order.
template <typename T>
__global__ void k_rank_permute(int64_t N, const int32_t *__restrict__ cellTmp,
                               const int32_t *__restrict__ cellStart,
                               const int32_t *__restrict__ bucketSrc,
                               const int32_t *__restrict__ bucketId,
                               const T2<T> *__restrict__ pos, const T2<T> *__restrict__ vel,
                               T2<T> *__restrict__ posN, T2<T> *__restrict__ velN,
                               T2<T> *__restrict__ xrefN, int32_t *__restrict__ permN,
                               int32_t *__restrict__ invperm, const T2<T> *__restrict__ ex0,
                               T2<T> *__restrict__ ex0N, const T2<T> *__restrict__ ex1,
                               T2<T> *__restrict__ ex1N)
{
    pdl_enter();
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const int32_t src = bucketSrc[s];
    const int32_t id = bucketId[s];
    const int32_t c = cellTmp[src];
    const int32_t b = cellStart[c], e = cellStart[c + 1];
    int32_t rank = 0;
    for (int32_t k = b; k < e; ++k) rank += (bucketId[k] < id) ? 1 : 0;
    const int32_t dst = b + rank;
    permN[dst] = id;
    if (!posN) return; // cell list only (build! without a neighbour rebuild)
    const T2<T> x = pos[src];
    posN[dst] = x;
    xrefN[dst] = x;
    velN[dst] = vel[src];
    invperm[id] = dst;
    if (ex0) ex0N[dst] = ex0[src];
    if (ex1) ex1N[dst] = ex1[src];
}

// The whole cell-list rebuild of a small single FP32 state in one block: cells
// and the displacement check (k_assign), the exclusive scan (k_scan_*), the
// bucket and the in-cell rank by particle id (k_bucket, k_rank_permute), with
// the histogram, scan and buckets in shared memory. Same arithmetic and the
// same deterministic order as the multi-launch path; it saves four launches
// per rebuild when the state is too small to keep the GPU busy anyway.
// Dynamic shared memory: 4 * (ncell + (ncell + 1) + 3 N) bytes.
constexpr int kRebuildSmallThreads = 1024;
constexpr int64_t kRebuildSmallMaxN = 4096;
constexpr int64_t kRebuildSmallMaxCells = 8192;

template <typename T>
__global__ void __launch_bounds__(kRebuildSmallThreads)
    k_rebuild_small(int N, int ncell, const Inst<T> I, int check, const T2<T> *__restrict__ pos,
                    const T2<T> *__restrict__ vel, T2<T> *__restrict__ posN,
                    T2<T> *__restrict__ velN, T2<T> *__restrict__ xref, int32_t *__restrict__ perm,
                    int32_t *__restrict__ invperm, int32_t *__restrict__ cellStart,
                    const T2<T> *__restrict__ ex0, T2<T> *__restrict__ ex0N,
                    const T2<T> *__restrict__ ex1, T2<T> *__restrict__ ex1N,
                    uint32_t *__restrict__ flags)
{
    pdl_enter();
    extern __shared__ int32_t sm[];
    int32_t *cursor = sm;                  // ncell: counts, then running cursors
    int32_t *starts = cursor + ncell;      // ncell + 1
    int32_t *cellOf = starts + ncell + 1;  // N
    int32_t *bucketSrc = cellOf + N;       // N
    int32_t *bucketId = bucketSrc + N;     // N
    __shared__ int32_t part[kRebuildSmallThreads / 32 + 1];
    const int t = (int)threadIdx.x, nt = (int)blockDim.x;
    for (int c = t; c < ncell; c += nt) cursor[c] = 0;
    __syncthreads();
    // cells (x / cs as in cell_index) and the displacement check
    bool moved = false;
    for (int i = t; i < N; i += nt) {
        const T2<T> x = pos[i];
        if (check) {
            const T2<T> xr = xref[i];
            const T d2 = r2_exact<T>(sub_rn(x.x, xr.x), sub_rn(x.y, xr.y));
            moved = moved || d2 > I.dmax2;
        }
        const int cx = cell_coord<T>(x.x / I.cs, I.nx);
        const int cy = cell_coord<T>(x.y / I.cs, I.ny);
        const int c = I.coff + (cx - 1) + (cy - 1) * I.nx;
        cellOf[i] = c;
        atomicAdd(&cursor[c], 1);
    }
    if (__syncthreads_or(moved) && t == 0) atomicOr(flags, FLAG_DISPLACEMENT);
    // exclusive scan of the counts: each thread sums a contiguous chunk
    const int chunk = (ncell + nt - 1) / nt;
    const int c0 = t * chunk, c1 = c0 + chunk < ncell ? c0 + chunk : ncell;
    int32_t sum = 0;
    for (int c = c0; c < c1; ++c) sum += cursor[c];
    int32_t x = sum;
    const int lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) part[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = nt >> 5;
        int32_t w = lane < nw ? part[lane] : 0, v = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane < nw) part[lane] = v - w;
    }
    __syncthreads();
    int32_t run = x - sum + part[warp];
    for (int c = c0; c < c1; ++c) {
        const int32_t n = cursor[c];
        starts[c] = run;
        cellStart[c] = run;
        cursor[c] = run;
        run += n;
    }
    if (t == 0) {
        starts[ncell] = N;
        cellStart[ncell] = N;
    }
    __syncthreads();
    // buckets: every particle into its cell's range (arbitrary order inside)
    for (int i = t; i < N; i += nt) {
        const int p = atomicAdd(&cursor[cellOf[i]], 1);
        bucketSrc[p] = i;
        bucketId[p] = perm[i];
    }
    __syncthreads();
    // in-cell rank by particle id, and the data into the new order
    for (int s = t; s < N; s += nt) {
        const int src = bucketSrc[s], id = bucketId[s], c = cellOf[src];
        const int b = starts[c], e = starts[c + 1];
        int rank = 0;
        for (int k = b; k < e; ++k) rank += bucketId[k] < id ? 1 : 0;
        const int dst = b + rank;
        perm[dst] = id;
        const T2<T> xs = pos[src];
        posN[dst] = xs;
        xref[dst] = xs;
        velN[dst] = vel[src];
        invperm[id] = dst;
        if (ex0) ex0N[dst] = ex0[src];
        if (ex1) ex1N[dst] = ex1[src];
    }
}

// _nl_build! (src/neighbors.jl:192-245): the scan centre uses x * invcs as
// the reference does; a neighbour is kept if r2min < r^2 < rc^2, in scan order,
// at most maxnb of them (overflow sets the flag, like flags[1]). Each row is
// scanned without branches on the predicate (slots 0-31 and 32-63 of the row
// into its two mask words, slots beyond 64 only counted); the maxnb limit is
// applied afterwards by keeping the first maxnb passing slots in scan order,
// which is the set the sequential loop keeps. On 1M particles this form runs
// 1.8x fewer warp instructions with 29 of 32 lanes active (22 when the limit
// was tested per slot): 56 instead of 93 us per launch.
template <typename T, typename IT>
__device__ __forceinline__ void nl_build_one(int64_t N, const IT &I, int bi, int64_t i,
                                             const T2<T> *__restrict__ pos,
                                             const int32_t *__restrict__ cellStart,
                                             uint32_t *__restrict__ center,
                                             uint32_t *__restrict__ masks,
                                             int32_t *__restrict__ nbcount,
                                             uint32_t *__restrict__ flags);

template <typename T, bool MULTI>
__global__ void k_nl_build(int64_t N, const Inst<T> one, const Inst<T> *__restrict__ inst,
                           const uint16_t *__restrict__ pinst, const T2<T> *__restrict__ pos,
                           const int32_t *__restrict__ cellStart, uint32_t *__restrict__ center,
                           uint32_t *__restrict__ masks, int32_t *__restrict__ nbcount,
                           uint32_t *__restrict__ flags)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int bi = MULTI ? (int)pinst[i] : 0;
    decltype(auto) I = pick_inst<MULTI>(one, inst, bi);
    nl_build_one<T>(N, I, bi, i, pos, cellStart, center, masks, nbcount, flags);
}

// One particle's neighbour rows (the body of k_nl_build); bi selects its
// instance's flag word.
template <typename T, typename IT>
__device__ __forceinline__ void nl_build_one(int64_t N, const IT &I, int bi, int64_t i,
                                             const T2<T> *__restrict__ pos,
                                             const int32_t *__restrict__ cellStart,
                                             uint32_t *__restrict__ center,
                                             uint32_t *__restrict__ masks,
                                             int32_t *__restrict__ nbcount,
                                             uint32_t *__restrict__ flags)
{
    const int nx = I.nx, ny = I.ny, maxnb = I.maxnb;
    const T rc2 = I.rc2, r2min = I.r2min;
    const T2<T> xi = pos[i];
    const int cx = cell_coord<T>(xi.x * I.invcs, nx);
    const int cy = cell_coord<T>(xi.y * I.invcs, ny);
    const int jx0 = cx - 1 > 1 ? cx - 1 : 1;
    const int jx1 = cx + 1 < nx ? cx + 1 : nx;
    uint32_t spill = 0;
    auto pass = [&](int j) -> uint32_t {
        const T2<T> xj = pos[j];
        T r2;
        if constexpr (sizeof(T) == 4 && kPackedPairs) {
            // the same separately rounded difference, squares and sum, with
            // the x and y halves in one f32x2 instruction each
            const float2 d = fsub2(xi, xj);
            const float2 q = fmul2(d, d);
            r2 = add_rn(q.x, q.y);
        } else {
            r2 = r2_exact<T>(sub_rn(xi.x, xj.x), sub_rn(xi.y, xj.y));
        }
        return (lt_nonneg(r2min, r2) && lt_nonneg(r2, rc2)) ? 1u : 0u;
    };
    uint32_t lo[3], hi[3];
    int cnt[3]; // passing slots of each row, beyond 64 included
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        lo[r] = hi[r] = 0u;
        cnt[r] = 0;
        const int jy = cy + r - 1;
        if (jy >= 1 && jy <= ny) {
            const int row = I.coff + (jy - 1) * nx;
            const int b = cellStart[row + jx0 - 1];
            const int e = cellStart[row + jx1];
            if (e - b > 64) spill = 1;
            const int e0 = e - b < 32 ? e : b + 32;
            const int e1 = e - b < 64 ? e : b + 64;
            uint32_t w = 0u;
            for (int j = b; j < e0; ++j) w |= pass(j) << (j - b);
            lo[r] = w;
            w = 0u;
            for (int j = b + 32; j < e1; ++j) w |= pass(j) << (j - b - 32);
            hi[r] = w;
            int extra = 0;
            for (int j = b + 64; j < e; ++j) extra += (int)pass(j);
            cnt[r] = __popc(lo[r]) + __popc(hi[r]) + extra;
        }
    }
    // keep the first maxnb passing slots in scan order
    const int total = cnt[0] + cnt[1] + cnt[2];
    if (total > maxnb) {
        int room = maxnb;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const int nlo = __popc(lo[r]), nhi = __popc(hi[r]);
            if (room <= 0) {
                lo[r] = hi[r] = 0u;
            } else if (room < nlo) {
                lo[r] &= (1u << select_bit(lo[r], room)) - 1u;
                hi[r] = 0u;
            } else if (room < nlo + nhi) {
                hi[r] &= (1u << select_bit(hi[r], room - nlo)) - 1u;
            }
            room -= cnt[r];
        }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        masks[(int64_t)(2 * r) * N + i] = lo[r];
        masks[(int64_t)(2 * r + 1) * N + i] = hi[r];
    }
    const int m = total < maxnb ? total : maxnb;
    const bool over = total > maxnb;
    center[i] = (uint32_t)cx | ((uint32_t)cy << 16) | (spill << 31);
    nbcount[i] = m;
    if (over) atomicOr(flags + bi, FLAG_NL_OVERFLOW);
}

// ---------------------------------------------------------------------------
// Forward: density_kernel! + eos_kernel! (fused), accel_kernel! +
// integrate_kernel! (fused; positions and velocities double-buffered because
// neighbours read the pre-step state).
// ---------------------------------------------------------------------------
// The model reads per-particle densities (Tait derivative, viscosity average).
template <typename IT> __device__ __forceinline__ bool needs_rho_dev(const IT &I)
{
    return I.p.eos == 1 || I.p.visc == 1;
}

// Per-pair terms, shared by the thread-per-particle kernels and the
// group-per-particle kernels (sph_coop.cuh): each kernel adds them into its
// running sums in slot order, so both forms round identically.

// density_kernel!: m W(r) = m (A u^4 (2q + 1)).
template <typename T>
__device__ __forceinline__ T density_pair(T r2, T invh, T m, T A)
{
    const T q = pair_sqrt(r2) * invh;
    const T u = (T)1 - half_of(q);
    const T u2 = u * u;
    return m * (A * u2 * u2 * (twice_of(q) + (T)1));
}

// Viscosity constants of one instance, hoisted out of the pair loops: kind 0
// Morris (2 m mu), kind 1 Monaghan artificial viscosity (m alpha c h, 0.01 h^2).
template <typename T> struct Visc {
    int kind;
    T twomumass, avc, eh2;
};
template <typename T, typename IT> __device__ __forceinline__ Visc<T> visc_of(const IT &I)
{
    Visc<T> c;
    c.kind = I.p.visc;
    c.twomumass = I.p.twomumass;
    c.avc = I.p.avc;
    c.eh2 = I.p.eh2;
    return c;
}

// accel_kernel!: a_i -= P F d, then a_i += C (v_i - v_j) (Morris), per
// component. Artificial viscosity instead adds K d on approaching pairs,
// K = avc s F / ((r^2 + eh2) (rho_i + rho_j) / 2), s = (v_i - v_j).d.
template <typename T> struct AccelPair {
    T px, py, cx, cy;
};
template <typename T, bool AV = true>
__device__ __forceinline__ AccelPair<T> accel_pair(T r2, T dx, T dy, T invh, T m, T Fc,
                                                   const Visc<T> &vc, T pti, T iri, T rhoi,
                                                   T rhoj, const T2<T> &vi, const T2<T> &pj,
                                                   const T2<T> &vj)
{
    const T q = pair_sqrt(r2) * invh;
    const T u = (T)1 - half_of(q);
    const T F = Fc * u * u * u;
    const T Pij = m * (pti + pj.x);
    AccelPair<T> o;
    o.px = Pij * F * dx;
    o.py = Pij * F * dy;
    if (AV && vc.kind == 1) {
        const T wx = vi.x - vj.x;
        const T wy = vi.y - vj.y;
        const T s = wx * dx + wy * dy;
        T K = (T)0;
        if (s < (T)0) {
            const T D = r2 + vc.eh2;
            const T rb = half_of(rhoi + rhoj);
            K = vc.avc * s * F / (D * rb);
        }
        o.cx = K * dx;
        o.cy = K * dy;
    } else {
        const T C = vc.twomumass * iri * pj.y * F;
        o.cx = C * (vi.x - vj.x);
        o.cy = C * (vi.y - vj.y);
    }
    return o;
}

// adj_pass1_kernel!: gx -= P F da_x, gx += w d_x (same for y), gv += C da,
// grho -= C ad_v ir_i, S += F ad_d.
template <typename T> struct Pass1Pair {
    T gxs, gxa, gys, gya, gvx, gvy, grs, sS;
};
// With artificial viscosity the Morris terms vanish and the pair adds the
// derivatives of (abar_i - abar_j).(K d): with A = (abar_i - abar_j).d,
//   d/dd   = K da + A (K/s) w + A ((K/F) G/(h r) - 2K/D) d   (into gx, gy)
//   d/dv_i = A (K/s) d                                        (into gvx, gvy)
//   d/drho_i = -A K / (2 rb)                                  (into grho)
template <typename T, bool AV = true>
__device__ __forceinline__ Pass1Pair<T> pass1_pair(T r2, T dx, T dy, T invh, T m, T Fc, T Gc,
                                                   const Visc<T> &vc, T pti, T iri, T rhoi,
                                                   T rhoj, const T2<T> &vi, const T2<T> &ab,
                                                   const T2<T> &pj, const T2<T> &abj,
                                                   const T2<T> &vj)
{
    const T twomumass = vc.twomumass;
    T r, rinv;
    if constexpr (sizeof(T) == 4) {
        rinv = r2 > (T)0 ? rsqrtf(r2) : (T)0;
        r = r2 * rinv;
    } else {
        r = sqrt(r2);
    }
    const T q = r * invh;
    const T u = (T)1 - half_of(q);
    const T F = Fc * u * u * u;
    const T G = Gc * u * u;
    const T Pij = m * (pti + pj.x);
    const T Cbase = twomumass * iri * pj.y;
    const T C = Cbase * F;
    const T dax = ab.x - abj.x;
    const T day = ab.y - abj.y;
    const T dvx = vi.x - vj.x;
    const T dvy = vi.y - vj.y;
    const T ad_d = -(dax * dx + day * dy);
    const T ad_v = dax * dvx + day * dvy;
    Pass1Pair<T> o;
    o.gxs = Pij * F * dax;
    o.gys = Pij * F * day;
    if (AV && vc.kind == 1) {
        const T s = dvx * dx + dvy * dy;
        const T Fbar = Pij * ad_d;
        T w;
        if constexpr (sizeof(T) == 4) w = Fbar * G * invh * rinv;
        else w = Fbar * G * invh / r;
        const T Ad = dax * dx + day * dy;
        T avx = (T)0, avy = (T)0, vx = (T)0, vy = (T)0, rs = (T)0;
        if (s < (T)0) {
            const T D = r2 + vc.eh2;
            const T rb = half_of(rhoi + rhoj);
            const T Drb = D * rb;
            const T K = vc.avc * s * F / Drb;
            const T Ks = vc.avc * F / Drb;
            const T KF = vc.avc * s / Drb;
            T cd;
            if constexpr (sizeof(T) == 4) cd = Ad * (KF * G * invh * rinv - twice_of(K) / D);
            else cd = Ad * (KF * G * invh / r - twice_of(K) / D);
            avx = K * dax + Ad * Ks * dvx + cd * dx;
            avy = K * day + Ad * Ks * dvy + cd * dy;
            vx = Ad * Ks * dx;
            vy = Ad * Ks * dy;
            rs = Ad * K / twice_of(rb);
        }
        o.gxa = w * dx + avx;
        o.gya = w * dy + avy;
        o.gvx = vx;
        o.gvy = vy;
        o.grs = rs;
        o.sS = F * ad_d;
        return o;
    }
    const T Fbar = Pij * ad_d + Cbase * ad_v;
    T w;
    if constexpr (sizeof(T) == 4) w = Fbar * G * invh * rinv;
    else w = Fbar * G * invh / r;
    o.gxa = w * dx;
    o.gya = w * dy;
    o.gvx = C * dax;
    o.gvy = C * day;
    o.grs = C * ad_v * iri;
    o.sS = F * ad_d;
    return o;
}

// adj_pass2_kernel!: gx += w d, w = m F (grho_i + grho_j).
template <typename T>
__device__ __forceinline__ T pass2_weight(T r2, T invh, T m, T Fc, T gri, T grj)
{
    const T q = pair_sqrt(r2) * invh;
    const T u = (T)1 - half_of(q);
    return m * (Fc * u * u * u) * (gri + grj);
}

// Density sum of a spilled particle (rows longer than 64 slots): the generic
// neighbour walk; its in-support words are all zero (later passes walk it the
// same way).
template <typename T, typename IT>
__device__ __forceinline__ T density_spill_sum(const NLView<T> &v, const IT &I, int64_t i,
                                               const T2<T> &xi, uint32_t *__restrict__ tmaskOut)
{
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, A = I.p.A;
    T acc = (T)0;
    for_each_neighbor<T>(v, I, i, [&](int j) {
        const T2<T> xj = v.pos[j];
        const T dx = xi.x - xj.x;
        const T dy = xi.y - xj.y;
        const T r2 = dx * dx + dy * dy;
        if (lt_nonneg(r2, r2max)) acc += density_pair<T>(r2, invh, m, A);
    });
    if (tmaskOut)
        for (int w = 0; w < 6; ++w) tmaskOut[(int64_t)w * v.N + i] = 0u;
    return acc;
}

// Self term and eos_kernel!: rho = sum + m A, pterm = c^2 (rho - rho0) / rho^2
// (Tait: B ((rho/rho0)^gamma - 1) / rho^2).
template <typename T, typename IT>
__device__ __forceinline__ void density_finish(const IT &I, int64_t i, T acc, T *__restrict__ rho,
                                               T2<T> *__restrict__ prho)
{
    const T m = I.p.m, A = I.p.A;
    // explicit roundings: the same result whichever kernel form inlines this
    // (a multiply-add contraction here would depend on the surrounding code)
    const T ri = add_rn(acc, mul_rn(m, A));
    if (rho) rho[i] = ri;
    const T inv = (T)1 / ri;
    T pt;
    if (I.p.eos == 1) pt = I.p.B * pow1m<T>((ri - I.p.rho0) / I.p.rho0, I.p.gam) * inv * inv;
    else pt = I.p.c2 * (ri - I.p.rho0) * inv * inv;
    prho[i] = mk2<T>(pt, inv);
}

// density_kernel! + eos_kernel!. It also records, for the rest of this step,
// which neighbour-list entries are inside the support (r^2 < 4h^2): the later
// passes of the step walk only those (same set, same order), skipping the
// candidates that the reference's own r^2 test would reject.
template <typename T, bool MULTI, bool PAIRS = false>
__device__ __forceinline__ void density_walk(const NLView<T> &v, int64_t i, T *__restrict__ rho,
                                             T2<T> *__restrict__ prho,
                                             uint32_t *__restrict__ tmaskOut);

template <typename T, bool MULTI, bool PAIRS = false>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? 6 : 4)
    k_density_eos(const __grid_constant__ NLView<T> v, T *__restrict__ rho,
                  T2<T> *__restrict__ prho, uint32_t *__restrict__ tmaskOut)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    density_walk<T, MULTI, PAIRS>(v, i, rho, prho, tmaskOut);
}

// FP32 density sum over the mask words, two candidates per iteration: both
// candidates' kernel arithmetic runs in packed f32x2 instructions (each half
// rounded as the scalar form rounds it) and their terms are added to the one
// running sum in slot order, so the sum equals the one-candidate loop's. A
// lone last candidate of a word is paired with itself and adds +0.
__device__ __forceinline__ float density_pairs_f32(const NLView<float> &v, int64_t i,
                                                   const float2 &xi, float r2max, float invh,
                                                   uint64_t m0, uint64_t m1, uint64_t m2, int b0,
                                                   int b1, int b2,
                                                   uint32_t *__restrict__ tmaskOut)
{
    const float2 ih2 = make_float2(invh, invh), mh = make_float2(-0.5f, -0.5f);
    const float2 one2 = make_float2(1.0f, 1.0f), two2 = make_float2(2.0f, 2.0f);
    float acc = 0.0f;
    uint32_t mw = (uint32_t)m0, tw = 0u;
    int base = b0;
    int w = 0;
    for (;;) {
        if (mw == 0u) {
            if (tmaskOut) tmaskOut[(int64_t)w * v.N + i] = tw; // word w is finished
            tw = 0u;
            if (++w == 6) break;
            const uint64_t mr = w < 2 ? m0 : (w < 4 ? m1 : m2);
            const int br = w < 2 ? b0 : (w < 4 ? b1 : b2);
            mw = (w & 1) ? (uint32_t)(mr >> 32) : (uint32_t)mr;
            base = br + ((w & 1) << 5);
            continue;
        }
        const int ka = __ffs((int)mw) - 1;
        mw &= mw - 1u;
        const bool two = mw != 0u;
        const int kb = two ? __ffs((int)mw) - 1 : ka;
        mw &= two ? mw - 1u : mw;
        const float2 da = fsub2(xi, v.pos[base + ka]);
        const float2 db = fsub2(xi, v.pos[base + kb]);
        const float r2a = da.x * da.x + da.y * da.y;
        const float r2b = db.x * db.x + db.y * db.y;
        const bool ina = r2a < r2max;
        const bool inb = two && r2b < r2max;
        tw |= ((uint32_t)ina << ka) | ((uint32_t)inb << kb);
        const float2 q = fmul2(make_float2(pair_sqrt(r2a), pair_sqrt(r2b)), ih2);
        float2 u = ffma2(q, mh, one2); // 1 - q/2
        u.x = ina ? u.x : 0.0f;
        u.y = inb ? u.y : 0.0f;
        const float2 u2 = fmul2(u, u);
        const float2 u4 = fmul2(u2, u2);
        const float2 t = ffma2(q, two2, one2); // 2q + 1
        acc = fmaf(u4.x, t.x, acc);
        acc = fmaf(u4.y, t.y, acc);
    }
    return acc;
}

// The per-particle mask walk of k_density_eos (one thread per particle).
template <typename T, bool MULTI, bool PAIRS>
__device__ __forceinline__ void density_walk(const NLView<T> &v, int64_t i, T *__restrict__ rho,
                                             T2<T> *__restrict__ prho,
                                             uint32_t *__restrict__ tmaskOut)
{
    decltype(auto) I = load_inst<MULTI>(v, i);
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, A = I.p.A;
    const T2<T> xi = v.pos[i];
    T acc = (T)0;
    const uint32_t cc = v.center[i];
    if (!(cc >> 31)) {
        // the walk of for_each_neighbor, keeping the passing bits
        const int cx = (int)(cc & 0xffffu);
        const int cy = (int)((cc >> 16) & 0x7fffu);
        const int jx0 = cx - 1 > 1 ? cx - 1 : 1;
        const int row0 = I.coff + (jx0 - 1) + (cy - 2) * I.nx;
        const uint64_t m0 = ((uint64_t)v.masks[v.N + i] << 32) | v.masks[i];
        const uint64_t m1 = ((uint64_t)v.masks[3 * v.N + i] << 32) | v.masks[2 * v.N + i];
        const uint64_t m2 = ((uint64_t)v.masks[5 * v.N + i] << 32) | v.masks[4 * v.N + i];
        const int b0 = m0 ? v.cellStart[row0] : 0;
        const int b1 = m1 ? v.cellStart[row0 + I.nx] : 0;
        const int b2 = m2 ? v.cellStart[row0 + 2 * I.nx] : 0;
        if constexpr (PAIRS && sizeof(T) == 4) {
            acc = density_pairs_f32(v, i, xi, r2max, invh, m0, m1, m2, b0, b1, b2, tmaskOut);
            acc = mul_rn(mul_rn(m, A), acc);
            density_finish<T>(I, i, acc, rho, prho);
            return;
        }
        uint32_t mw = (uint32_t)m0, tw = 0u;
        int base = b0;
        int w = 0;
        for (;;) {
            if (mw == 0u) {
                if (tmaskOut) tmaskOut[(int64_t)w * v.N + i] = tw; // word w is finished
                tw = 0u;
                if (++w == 6) break;
                const uint64_t mr = w < 2 ? m0 : (w < 4 ? m1 : m2);
                const int br = w < 2 ? b0 : (w < 4 ? b1 : b2);
                mw = (w & 1) ? (uint32_t)(mr >> 32) : (uint32_t)mr;
                base = br + ((w & 1) << 5);
                continue;
            }
            const int k = __ffs((int)mw) - 1;
            mw &= mw - 1u;
            const T2<T> xj = v.pos[base + k];
            const T dx = xi.x - xj.x;
            const T dy = xi.y - xj.y;
            const T r2 = dx * dx + dy * dy;
            if constexpr (sizeof(T) == 4) {
                // FP32: evaluate every candidate and select, instead of a
                // branch that diverges on the support test (13% faster on
                // 1M particles); an outside candidate has u = 0 and adds 0.
                // The common factor m A is applied once after the loop (8%).
                const bool in = lt_nonneg(r2, r2max);
                tw |= (uint32_t)in << k;
                const T q = pair_sqrt(r2) * invh;
                const T u = in ? (T)1 - half_of(q) : (T)0;
                const T u2 = u * u;
                acc += u2 * u2 * (twice_of(q) + (T)1);
            } else if (lt_nonneg(r2, r2max)) {
                // FP64: the pipe is the bottleneck, so skip outside candidates
                tw |= 1u << k;
                acc += density_pair<T>(r2, invh, m, A);
            }
        }
        if constexpr (sizeof(T) == 4) acc = mul_rn(mul_rn(m, A), acc);
    } else {
        acc = density_spill_sum<T>(v, I, i, xi, tmaskOut);
    }
    density_finish<T>(I, i, acc, rho, prho);
}

// Density in the cell-tile form: an alternative to the per-particle mask
// walk for FP32 single states, measured against it and kept off by default
// (sph_set_density_form 1). A warp takes 32 consecutive slots (its tile). When
// the tile lies in one cell row and no particle in it is spilled, the warp
// copies once into shared memory the slot ranges of the three neighbouring
// cell rows that cover all of its lanes' 3 x 3 cells (particles are stored in
// cell order, so each row's range is contiguous and the copy is coalesced);
// every lane then visits every staged candidate, broadcast from shared memory
// to the warp, and keeps those that are set in its own neighbour row masks
// and inside the support. Staged rows come in ddy order and slot order within
// a row, so each lane adds its terms in the reference's scan order
// (src/forward.jl:25-65). Other warps walk their masks as k_density_eos does.
constexpr int kTileWarps = 4;
constexpr int kTileStage = 512; // staged candidates per warp (three rows)

template <typename T>
__global__ void __launch_bounds__(32 * kTileWarps)
    k_density_tile(const __grid_constant__ NLView<T> v, T *__restrict__ rho,
                   T2<T> *__restrict__ prho, uint32_t *__restrict__ tmaskOut)
{
    pdl_enter();
    __shared__ T2<T> stage[kTileWarps][kTileStage];
    const int w = (int)(threadIdx.x >> 5);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < v.N;
    if (!__any_sync(0xffffffffu, live)) return;
    const Inst<T> &I = v.one;
    const uint32_t cc = live ? v.center[i] : 0u;
    const int cx = (int)(cc & 0xffffu);
    const int cy = (int)((cc >> 16) & 0x7fffu);
    const int cymin = __reduce_min_sync(0xffffffffu, live ? cy : INT_MAX);
    const int cymax = __reduce_max_sync(0xffffffffu, live ? cy : INT_MIN);
    const int cxmin = __reduce_min_sync(0xffffffffu, live ? cx : INT_MAX);
    const int cxmax = __reduce_max_sync(0xffffffffu, live ? cx : INT_MIN);
    const bool spilled = __any_sync(0xffffffffu, live && (cc >> 31));
    // the staged window: rows cy-1..cy+1, cells max(cxmin-1,1)..min(cxmax+1,nx)
    int sb[3], sn[3];
    int total = 0;
    if (cymin == cymax && !spilled) {
        const int xa = cxmin - 1 > 1 ? cxmin - 1 : 1;
        const int xb = cxmax + 1 < I.nx ? cxmax + 1 : I.nx;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const int jy = cymin + r - 1;
            sb[r] = 0;
            sn[r] = 0;
            if (jy >= 1 && jy <= I.ny) {
                const int row = I.coff + (jy - 1) * I.nx;
                sb[r] = v.cellStart[row + xa - 1];
                sn[r] = v.cellStart[row + xb] - sb[r];
            }
            total += sn[r];
        }
    }
    if (cymin != cymax || spilled || total > kTileStage) {
        if (live) density_walk<T, false>(v, i, rho, prho, tmaskOut);
        return;
    }
    for (int k = (int)(threadIdx.x & 31u); k < total; k += 32) {
        const int j = k < sn[0] ? sb[0] + k
                                : (k < sn[0] + sn[1] ? sb[1] + (k - sn[0]) : sb[2] + (k - sn[0] - sn[1]));
        stage[w][k] = v.pos[j];
    }
    __syncwarp();
    if (!live) return;
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, A = I.p.A;
    const T2<T> xi = v.pos[i];
    const int jx0 = cx - 1 > 1 ? cx - 1 : 1;
    const int row0 = I.coff + (jx0 - 1) + (cy - 2) * I.nx;
    T acc = (T)0;
    int k0 = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const uint64_t mr = ((uint64_t)v.masks[(2 * r + 1) * v.N + i] << 32) | v.masks[2 * r * v.N + i];
        // slot of the lane's first candidate in row r (its mask's bit 0)
        const int br = mr ? v.cellStart[row0 + r * I.nx] : 0;
        uint64_t tw = 0ull;
        for (int k = 0; k < sn[r]; ++k) {
            const T2<T> xj = stage[w][k0 + k];
            const int off = sb[r] + k - br;
            const bool listed = (unsigned)off < 64u && ((mr >> (off & 63)) & 1ull);
            const T dx = xi.x - xj.x;
            const T dy = xi.y - xj.y;
            const T r2 = dx * dx + dy * dy;
            const bool in = listed && lt_nonneg(r2, r2max);
            tw |= (uint64_t)in << (off & 63);
            const T q = pair_sqrt(r2) * invh;
            const T u = in ? (T)1 - half_of(q) : (T)0;
            const T u2 = u * u;
            acc += u2 * u2 * (twice_of(q) + (T)1);
        }
        k0 += sn[r];
        if (tmaskOut) {
            tmaskOut[(int64_t)(2 * r) * v.N + i] = (uint32_t)tw;
            tmaskOut[(int64_t)(2 * r + 1) * v.N + i] = (uint32_t)(tw >> 32);
        }
    }
    acc = mul_rn(mul_rn(m, A), acc);
    density_finish<T>(I, i, acc, rho, prho);
}

// Pressure + Morris viscosity (accel_kernel! pair loop).
template <typename T, bool AV = true>
__device__ __forceinline__ void accel_sum(const NLView<T> &v, const Inst<T> &I,
                                          const T2<T> *__restrict__ vel,
                                          const T2<T> *__restrict__ prho,
                                          const T *__restrict__ rho, int64_t i,
                                          const T2<T> &xi, const T2<T> &vi, T &ax, T &ay)
{
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, Fc = I.p.Fc;
    const Visc<T> vc = visc_of<T>(I);
    const T2<T> pi = prho[i];
    const T pti = pi.x, iri = pi.y;
    if constexpr (sizeof(T) == 4 && !AV && kPackedPairs) {
        // a_i -= (P_ij F) d, a_i += C (v_i - v_j), both components at once
        const float tmm = vc.twomumass;
        float2 acc = make_float2(0.0f, 0.0f);
        for_each_neighbor<T>(v, I, i, [&](int j) {
            // all of the neighbour's loads before the support test: the
            // in-support walk visits only pairs that pass it, and the later
            // loads then do not wait for the position's latency
            const float2 xj = v.pos[j];
            const float2 pj = prho[j];
            const float2 vj = vel[j];
            const float2 d = fsub2(xi, xj);
            const float r2 = d.x * d.x + d.y * d.y;
            if (lt_nonneg(r2, r2max)) {
                const float q = pair_sqrt(r2) * invh;
                const float u = 1.0f - 0.5f * q;
                const float F = Fc * u * u * u;
                const float PF = m * (pti + pj.x) * F;
                const float C = tmm * iri * pj.y * F;
                acc = ffma2(make_float2(-PF, -PF), d, acc);
                acc = ffma2(make_float2(C, C), fsub2(vi, vj), acc);
            }
        });
        ax = acc.x;
        ay = acc.y;
        return;
    }
    const T rhoi = (AV && vc.kind == 1) ? rho[i] : (T)0;
    ax = (T)0;
    ay = (T)0;
    for_each_neighbor<T>(v, I, i, [&](int j) {
        const T2<T> xj = v.pos[j];
        const T dx = xi.x - xj.x;
        const T dy = xi.y - xj.y;
        const T r2 = dx * dx + dy * dy;
        if (lt_nonneg(r2, r2max)) {
            const T rhoj = (AV && vc.kind == 1) ? rho[j] : (T)0;
            const AccelPair<T> t = accel_pair<T, AV>(r2, dx, dy, invh, m, Fc, vc, pti, iri, rhoi,
                                                     rhoj, vi, prho[j], vel[j]);
            ax -= t.px;
            ay -= t.py;
            ax += t.cx;
            ay += t.cy;
        }
    });
}

template <typename T, typename IT>
__device__ __forceinline__ void accel_integrate_finish(
    const IT &I, int b, int64_t i, const T2<T> &xi, const T2<T> &vi, T ax, T ay,
    const T *__restrict__ theta, T2<T> *__restrict__ posOut, T2<T> *__restrict__ velOut,
    T2<T> *__restrict__ aOut, T *__restrict__ alphaOut, uint32_t *__restrict__ flags,
    const int32_t *__restrict__ perm, T2<T> *__restrict__ tx, T2<T> *__restrict__ tv);

// accel_kernel! (pressure + viscosity + gravity + wall, and alpha) fused with
// integrate_kernel! (semi-implicit Euler, implicit Brinkman drag).
template <typename T, bool MULTI, bool AV = false>
__global__ void __launch_bounds__(kBlock)
    k_accel_integrate(const __grid_constant__ NLView<T> v, const T2<T> *__restrict__ vel,
                      const T2<T> *__restrict__ prho, const T *__restrict__ rho,
                      const T *__restrict__ theta, T2<T> *__restrict__ posOut,
                      T2<T> *__restrict__ velOut, T2<T> *__restrict__ aOut,
                      T *__restrict__ alphaOut, uint32_t *__restrict__ flags,
                      const int32_t *__restrict__ perm, T2<T> *__restrict__ tx,
                      T2<T> *__restrict__ tv)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    const int b = MULTI ? inst_of(v, i) : 0;
    decltype(auto) I = load_inst<MULTI>(v, i);
    const T2<T> xi = v.pos[i];
    const T2<T> vi = vel[i];
    T ax, ay;
    accel_sum<T, AV>(v, I, vel, prho, rho, i, xi, vi, ax, ay);
    accel_integrate_finish<T>(I, b, i, xi, vi, ax, ay, theta, posOut, velOut, aOut, alphaOut, flags,
                              perm, tx, tv);
}

// Gravity, wall, alpha and the integrator of one particle, after its pair sum.
template <typename T, typename IT>
__device__ __forceinline__ void accel_integrate_finish(
    const IT &I, int b, int64_t i, const T2<T> &xi, const T2<T> &vi, T ax, T ay,
    const T *__restrict__ theta, T2<T> *__restrict__ posOut, T2<T> *__restrict__ velOut,
    T2<T> *__restrict__ aOut, T *__restrict__ alphaOut, uint32_t *__restrict__ flags,
    const int32_t *__restrict__ perm, T2<T> *__restrict__ tx, T2<T> *__restrict__ tv)
{
    const Phys<T> &p = I.p;
    if (tx) {
        // _tape_store! (src/driver.jl:73-77) of the pre-step state, in
        // particle-id order
        const int32_t id = perm[i];
        tx[id] = xi;
        tv[id] = vi;
    }
    const T al = interp_alpha_value<T>(theta + I.toff, xi.x, xi.y, p);
    ax += p.gx + wall_accel<T>(xi.x, p.Lx, p.kw);
    ay += p.gy + wall_accel<T>(xi.y, p.Ly, p.kw);
    if (aOut) aOut[i] = mk2<T>(ax, ay);
    if (alphaOut) alphaOut[i] = al;
    const T dt = p.dt;
    const T D = (T)1 / ((T)1 + dt * al);
    const T v1 = (vi.x + dt * ax) * D;
    const T v2 = (vi.y + dt * ay) * D;
    const T x1 = xi.x + dt * v1;
    const T x2 = xi.y + dt * v2;
    velOut[i] = mk2<T>(v1, v2);
    posOut[i] = mk2<T>(x1, x2);
    if (!(isfinite(x1) && isfinite(x2) && isfinite(v1) && isfinite(v2)))
        atomicOr(flags + b, FLAG_NONFINITE);
}

// _tape_load! into cell order: slot t takes particle perm[t]; when srcInv is
// given the source is itself in cell order (a recomputed state) and the id is
// mapped through its inverse permutation.
template <typename T>
__global__ void k_gather_state(int64_t N, const int32_t *__restrict__ perm,
                               const int32_t *__restrict__ srcInv,
                               const T2<T> *__restrict__ sx, const T2<T> *__restrict__ sv,
                               T2<T> *__restrict__ pos, T2<T> *__restrict__ vel)
{
    pdl_enter();
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int32_t s = perm[t];
    if (srcInv) s = srcInv[s];
    pos[t] = sx[s];
    vel[t] = sv[s];
}

// id-ordered (interleaved) host layout <-> cell order
template <typename T>
__global__ void k_scatter_to_ids(int64_t N, const int32_t *__restrict__ perm,
                                 const T2<T> *__restrict__ a, T2<T> *__restrict__ out)
{
    pdl_enter();
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    out[perm[t]] = a[t];
}

template <typename T>
__global__ void k_scatter_to_ids1(int64_t N, const int32_t *__restrict__ perm,
                                  const T *__restrict__ a, T *__restrict__ out)
{
    pdl_enter();
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    out[perm[t]] = a[t];
}

template <typename T>
__global__ void k_gather_from_ids(int64_t N, const int32_t *__restrict__ perm,
                                  const T2<T> *__restrict__ a, T2<T> *__restrict__ out)
{
    pdl_enter();
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    out[t] = a[perm[t]];
}

// ---------------------------------------------------------------------------
// Adjoint (gather form, src/adjoint.jl)
// ---------------------------------------------------------------------------

// _adj_integrate! + _adj_drag! of one particle after its recomputed pair sum;
// returns the exponent bound of |galpha| (INT_MIN when it is zero).
template <typename T, typename IT>
__device__ __forceinline__ int drag_adj_finish(const IT &I, int64_t i, const T2<T> &xi,
                                               const T2<T> &vi, T ax, T ay,
                                               const T *__restrict__ theta,
                                               const T2<T> *__restrict__ gX,
                                               T2<T> *__restrict__ gV, T2<T> *__restrict__ abar,
                                               T *__restrict__ galpha)
{
    const Phys<T> &p = I.p;
    const T al = interp_alpha_value<T>(theta + I.toff, xi.x, xi.y, p);
    ax += p.gx + wall_accel<T>(xi.x, p.Lx, p.kw);
    ay += p.gy + wall_accel<T>(xi.y, p.Ly, p.kw);
    const T dt = p.dt;
    const T2<T> gx = gX[i];
    T2<T> gv = gV[i];
    gv.x += dt * gx.x;
    gv.y += dt * gx.y;
    const T D = (T)1 / ((T)1 + dt * al);
    const T vx = (vi.x + dt * ax) * D;
    const T vy = (vi.y + dt * ay) * D;
    abar[i] = mk2<T>(dt * D * gv.x, dt * D * gv.y);
    const T ga = -dt * D * (vx * gv.x + vy * gv.y);
    galpha[i] = ga;
    gV[i] = mk2<T>(D * gv.x, D * gv.y);
    return (ga != (T)0 && isfinite(ga)) ? ilogb((double)ga) + 1 : INT_MIN; // |ga| < 2^e
}

// Accel recompute (accel_kernel!, for a_rest and alpha) + _adj_integrate!
// (gV += dt gX) + _adj_drag! (implicit Brinkman VJP). Also records, per
// instance, the largest binary exponent of |galpha| for the exact theta
// reduction (emax holds two slots per instance, selected by step parity).
template <typename T, bool MULTI, bool AV = false>
__global__ void __launch_bounds__(kBlock)
    k_accel_drag_adj(const __grid_constant__ NLView<T> v, const T2<T> *__restrict__ vel,
                     const T2<T> *__restrict__ prho, const T *__restrict__ rho,
                     const T *__restrict__ theta, const T2<T> *__restrict__ gX,
                     T2<T> *__restrict__ gV, T2<T> *__restrict__ abar, T *__restrict__ galpha,
                     int *__restrict__ emax, int parity)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < v.N;
    int e = INT_MIN;
    int b = 0;
    if (live) {
        b = MULTI ? inst_of(v, i) : 0;
        decltype(auto) I = load_inst<MULTI>(v, i);
        const T2<T> xi = v.pos[i];
        const T2<T> vi = vel[i];
        T ax, ay;
        accel_sum<T, AV>(v, I, vel, prho, rho, i, xi, vi, ax, ay);
        e = drag_adj_finish<T>(I, i, xi, vi, ax, ay, theta, gX, gV, abar, galpha);
    }
    // max over the lanes of each instance present in the warp, one atomic each
    const unsigned act = __ballot_sync(0xffffffffu, live);
    if (!live) return;
    const unsigned peers = __match_any_sync(act, b);
    int mx = e;
    for (unsigned rest = peers; rest; rest &= rest - 1) {
        const int src = __ffs(rest) - 1;
        const int y = __shfl_sync(peers, e, src);
        mx = y > mx ? y : mx;
    }
    if ((int)lane_id() == __ffs(peers) - 1 && mx != INT_MIN) atomicMax(emax + 2 * b + parity, mx);
}

template <typename T, bool AV, typename IT>
__device__ __forceinline__ void pass1_sum(const NLView<T> &v, const IT &I, int64_t i,
                                          const T2<T> *__restrict__ vel,
                                          const T2<T> *__restrict__ prho,
                                          const T *__restrict__ rho,
                                          const T2<T> *__restrict__ abar, const T2<T> &xi,
                                          const T2<T> &vi, const T2<T> &ab, const T2<T> &pi,
                                          T &gx, T &gy, T &gvx, T &gvy, T &grh, T &sumS);
template <typename T, typename IT>
__device__ __forceinline__ void pass1_finish(const IT &I, int64_t i, const T2<T> &xi,
                                             const T2<T> &ab, const T2<T> &pi, T rhoi, T gx,
                                             T gy, T gvx, T gvy, T grh, T sumS,
                                             const T *__restrict__ theta,
                                             const T *__restrict__ galpha, T2<T> *__restrict__ gXs,
                                             T *__restrict__ grho, T2<T> *__restrict__ gV);

// adj_pass1_kernel! (src/adjoint.jl:30-122) + the per-particle half of
// adj_design_kernel! (gXs += galpha * grad alpha, src/adjoint.jl:173-175)
// + _axpy2!(gV, gVs).
template <typename T, bool MULTI, bool AV = false>
__global__ void __launch_bounds__(kBlock, (sizeof(T) == 4 && !MULTI && !AV) ? 6 : 1) // single FP32: <= 42 registers
    k_pass1_design(const __grid_constant__ NLView<T> v, const T2<T> *__restrict__ vel,
                   const T2<T> *__restrict__ prho, const T *__restrict__ rho,
                   const T *__restrict__ theta, const T2<T> *__restrict__ abar,
                   const T *__restrict__ galpha, T2<T> *__restrict__ gXs, T *__restrict__ grho,
                   T2<T> *__restrict__ gV)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    decltype(auto) I = load_inst<MULTI>(v, i);
    const T2<T> xi = v.pos[i];
    const T2<T> vi = vel[i];
    const T2<T> ab = abar[i];
    const T2<T> pi = prho[i];
    T gx, gy, gvx, gvy, grh, sumS;
    pass1_sum<T, AV>(v, I, i, vel, prho, rho, abar, xi, vi, ab, pi, gx, gy, gvx, gvy, grh, sumS);
    const T rhoi = I.p.eos == 1 || (AV && I.p.visc == 1) ? rho[i] : (T)0;
    pass1_finish<T>(I, i, xi, ab, pi, rhoi, gx, gy, gvx, gvy, grh, sumS, theta, galpha, gXs, grho,
                    gV);
}

// The pair loop of adj_pass1_kernel! (src/adjoint.jl:41-110).
template <typename T, bool AV, typename IT>
__device__ __forceinline__ void pass1_sum(const NLView<T> &v, const IT &I, int64_t i,
                                          const T2<T> *__restrict__ vel,
                                          const T2<T> *__restrict__ prho,
                                          const T *__restrict__ rho,
                                          const T2<T> *__restrict__ abar, const T2<T> &xi,
                                          const T2<T> &vi, const T2<T> &ab, const T2<T> &pi,
                                          T &gx, T &gy, T &gvx, T &gvy, T &grh, T &sumS)
{
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, Fc = I.p.Fc, Gc = I.p.Gc;
    const Visc<T> vc = visc_of<T>(I);
    const T pti = pi.x, iri = pi.y;
    if constexpr (sizeof(T) == 4 && !AV && kPackedPairs) {
        // the Morris-model pair of adj_pass1_kernel! with (x, y) packed:
        // g -= (P F) da, g += w d, gv += C da
        const float tmm = vc.twomumass;
        float2 g = make_float2(0.0f, 0.0f), gv = make_float2(0.0f, 0.0f);
        float gr = 0.0f, sS = 0.0f;
        for_each_neighbor<T>(v, I, i, [&](int j) {
            const float2 xj = v.pos[j];
            const float2 pj = prho[j];
            const float2 abj = abar[j];
            const float2 vj = vel[j];
            const float2 d = fsub2(xi, xj);
            const float r2 = d.x * d.x + d.y * d.y;
            if (lt_nonneg(r2, r2max)) {
                const float rinv = r2 > 0.0f ? rsqrtf(r2) : 0.0f;
                const float r = r2 * rinv;
                const float q = r * invh;
                const float u = 1.0f - 0.5f * q;
                const float F = Fc * u * u * u;
                const float G = Gc * u * u;
                const float PF = m * (pti + pj.x) * F;
                const float Cbase = tmm * iri * pj.y;
                const float C = Cbase * F;
                const float2 da = fsub2(ab, abj);
                const float2 dv = fsub2(vi, vj);
                const float ad_d = -(da.x * d.x + da.y * d.y);
                const float ad_v = da.x * dv.x + da.y * dv.y;
                const float Fbar = m * (pti + pj.x) * ad_d + Cbase * ad_v;
                const float w = Fbar * G * invh * rinv;
                g = ffma2(make_float2(-PF, -PF), da, g);
                g = ffma2(make_float2(w, w), d, g);
                gv = ffma2(make_float2(C, C), da, gv);
                gr -= C * ad_v * iri;
                sS += F * ad_d;
            }
        });
        gx = g.x;
        gy = g.y;
        gvx = gv.x;
        gvy = gv.y;
        grh = gr;
        sumS = sS;
        return;
    }
    const T rhoi = (AV && vc.kind == 1) ? rho[i] : (T)0;
    gx = 0, gy = 0, gvx = 0, gvy = 0, grh = 0, sumS = 0;
    for_each_neighbor<T>(v, I, i, [&](int j) {
        const T2<T> xj = v.pos[j];
        const T dx = xi.x - xj.x;
        const T dy = xi.y - xj.y;
        const T r2 = dx * dx + dy * dy;
        if (lt_nonneg(r2, r2max)) {
            const T rhoj = (AV && vc.kind == 1) ? rho[j] : (T)0;
            const Pass1Pair<T> t = pass1_pair<T, AV>(r2, dx, dy, invh, m, Fc, Gc, vc, pti, iri,
                                                     rhoi, rhoj, vi, ab, prho[j], abar[j], vel[j]);
            gx -= t.gxs;
            gy -= t.gys;
            gx += t.gxa;
            gy += t.gya;
            gvx += t.gvx;
            gvy += t.gvy;
            grh -= t.grs;
            sumS += t.sS;
        }
    });
}

// Per-particle tail of adj_pass1_kernel! (src/adjoint.jl:112-121), the gXs
// half of adj_design_kernel! and _axpy2!(gV, gVs).
template <typename T, typename IT>
__device__ __forceinline__ void pass1_finish(const IT &I, int64_t i, const T2<T> &xi,
                                             const T2<T> &ab, const T2<T> &pi, T rhoi, T gx,
                                             T gy, T gvx, T gvy, T grh, T sumS,
                                             const T *__restrict__ theta,
                                             const T *__restrict__ galpha, T2<T> *__restrict__ gXs,
                                             T *__restrict__ grho, T2<T> *__restrict__ gV)
{
    const T pti = pi.x, iri = pi.y;
    const Phys<T> &p = I.p;
    grh += ((T)(-2) * p.m * pti * iri) * sumS;
    if (p.eos == 1) grh += p.dB * pow_fold<T>(rhoi / p.rho0, p.gam - 1) * p.m * iri * iri * sumS;
    else grh += p.c2 * p.m * iri * iri * sumS;
    gx += ab.x * wall_daccel<T>(xi.x, p.Lx, p.kw);
    gy += ab.y * wall_daccel<T>(xi.y, p.Ly, p.kw);
    T al, dadx, dady;
    interp_alpha<T>(theta + I.toff, xi.x, xi.y, p, al, dadx, dady);
    const T ga = galpha[i];
    gXs[i] = mk2<T>(gx + ga * dadx, gy + ga * dady);
    grho[i] = grh;
    T2<T> g = gV[i];
    g.x += gvx;
    g.y += gvy;
    gV[i] = g;
}

// 128-bit two's-complement fixed-point accumulation: integer addition is
// associative, so the dJ/dtheta sums are exact and independent of the order in
// which particles arrive. acc[0] = low word, acc[1] = high word. Adds the grid
// value of one contribution (sph_fixed.cuh) with 64-bit integer atomics and
// an explicit carry.
template <typename C>
__device__ __forceinline__ void fixed_add(unsigned long long *acc, C c, int S)
{
    Fixed128 v;
    if (!fixed_of(c, S, v)) return;
    const unsigned long long old = atomicAdd(acc, v.lo);
    const unsigned long long h = v.hi + ((old + v.lo < old) ? 1ull : 0ull);
    if (h) atomicAdd(acc + 1, h);
}

// Scale 2^S of the fixed-point grid: every contribution of the step is below
// 2^emax and at most n of them reach one node, so sums stay below 2^124.
__host__ __device__ __forceinline__ int theta_scale(int emax, int lgN) { return 124 - emax - lgN; }

template <typename T, typename IT>
__device__ __forceinline__ void pass2_finish(const IT &I, int b, int64_t i, const T2<T> &xi,
                                             T gx, T gy, const T2<T> *__restrict__ gXs,
                                             T2<T> *__restrict__ gX,
                                             const T *__restrict__ galpha,
                                             const int *__restrict__ emax, int parity,
                                             unsigned long long *__restrict__ thetaAcc);

template <typename T, typename IT>
__device__ __forceinline__ void pass2_sum(const NLView<T> &v, const IT &I, int64_t i,
                                          const T2<T> &xi, const T *__restrict__ grho, T &gx,
                                          T &gy);

// adj_pass2_kernel! (src/adjoint.jl:126-156) + _axpy2!(gX, gXs) + the theta
// write-back of adj_design_kernel! (src/adjoint.jl:177-184), done as an exact
// deterministic reduction keyed by design node instead of float atomics.
template <typename T, bool MULTI>
__global__ void __launch_bounds__(kBlock)
    k_pass2_axpy(const __grid_constant__ NLView<T> v, const T *__restrict__ grho,
                 const T2<T> *__restrict__ gXs,
                 T2<T> *__restrict__ gX, const T *__restrict__ galpha,
                 const int *__restrict__ emax, int parity,
                 unsigned long long *__restrict__ thetaAcc)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    const int b = MULTI ? inst_of(v, i) : 0;
    decltype(auto) I = load_inst<MULTI>(v, i);
    const T2<T> xi = v.pos[i];
    T gx, gy;
    pass2_sum<T>(v, I, i, xi, grho, gx, gy);
    pass2_finish<T>(I, b, i, xi, gx, gy, gXs, gX, galpha, emax, parity, thetaAcc);
}

// The pair loop of adj_pass2_kernel! (src/adjoint.jl:126-156).
template <typename T, typename IT>
__device__ __forceinline__ void pass2_sum(const NLView<T> &v, const IT &I, int64_t i,
                                          const T2<T> &xi, const T *__restrict__ grho, T &gx,
                                          T &gy)
{
    const T r2max = I.p.r2max, invh = I.p.invh, m = I.p.m, Fc = I.p.Fc;
    const T gri = grho[i];
    if constexpr (sizeof(T) == 4 && kPackedPairs) {
        float2 acc = make_float2(0.0f, 0.0f);
        for_each_neighbor<T>(v, I, i, [&](int j) {
            const float2 xj = v.pos[j];
            const float grj = grho[j];
            const float2 d = fsub2(xi, xj);
            const float r2 = d.x * d.x + d.y * d.y;
            if (lt_nonneg(r2, r2max)) {
                const float w = pass2_weight<float>(r2, invh, m, Fc, gri, grj);
                acc = ffma2(make_float2(w, w), d, acc);
            }
        });
        gx = acc.x;
        gy = acc.y;
        return;
    }
    gx = 0;
    gy = 0;
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
}

// _axpy2!(gX, gXs) and the exact theta write-back of one particle after its
// pass-2 pair sum (gx, gy).
template <typename T, typename IT>
__device__ __forceinline__ void pass2_finish(const IT &I, int b, int64_t i, const T2<T> &xi,
                                             T gx, T gy, const T2<T> *__restrict__ gXs,
                                             T2<T> *__restrict__ gX,
                                             const T *__restrict__ galpha,
                                             const int *__restrict__ emax, int parity,
                                             unsigned long long *__restrict__ thetaAcc)
{
    T2<T> gs = gXs[i];
    gs.x += gx;
    gs.y += gy;
    T2<T> g = gX[i];
    g.x += gs.x;
    g.y += gs.y;
    gX[i] = g;

    const T ga = galpha[i];
    const int em = emax[2 * b + parity];
    if (ga != (T)0 && em != INT_MIN) {
        const Phys<T> &p = I.p;
        int i0, j0;
        T fx, fy, ax, ay;
        interp_cell<T>(xi.x, xi.y, p, i0, j0, fx, fy, ax, ay);
        const int S = theta_scale(em, I.lgN);
        unsigned long long *acc = thetaAcc + 2 * (int64_t)I.toff;
        const int64_t l00 = (int64_t)j0 + (int64_t)i0 * p.ngy;
        // T-typed contributions: FP32 ones take the integer conversion
        fixed_add(acc + 2 * l00, ga * ((T)1 - fx) * ((T)1 - fy), S);
        fixed_add(acc + 2 * (l00 + p.ngy), ga * fx * ((T)1 - fy), S);
        fixed_add(acc + 2 * (l00 + 1), ga * ((T)1 - fx) * fy, S);
        fixed_add(acc + 2 * (l00 + p.ngy + 1), ga * fx * fy, S);
    }
}

// Per design node: gtheta += one step's exact sum; clear the accumulator.
// Threads n < B also reset the exponent slot the following step will use.
template <typename T>
__device__ __forceinline__ void theta_node(int64_t n, int64_t nnode, int B,
                                           const Inst<T> *__restrict__ inst,
                                           unsigned long long *__restrict__ acc,
                                           int *__restrict__ emax, int parity,
                                           double *__restrict__ gtheta)
{
    if (n >= nnode) return;
    unsigned long long lo = acc[2 * n], hi = acc[2 * n + 1];
    if ((lo | hi) != 0ull) {
        // instance owning node n (design-node offsets are increasing)
        int lo_b = 0, hi_b = B - 1;
        while (lo_b < hi_b) {
            const int mid = (lo_b + hi_b + 1) >> 1;
            if (inst[mid].toff <= n) lo_b = mid; else hi_b = mid - 1;
        }
        const int b = lo_b;
        const int em = emax[2 * b + parity];
        acc[2 * n] = 0ull;
        acc[2 * n + 1] = 0ull;
        const bool neg = (long long)hi < 0;
        if (neg) {
            lo = ~lo + 1ull;
            hi = ~hi + (lo == 0ull ? 1ull : 0ull);
        }
        double vv = ldexp((double)hi, 64) + (double)lo;
        if (neg) vv = -vv;
        gtheta[n] += ldexp(vv, -theta_scale(em, inst[b].lgN));
    }
    if (n < B) emax[2 * n + (1 - parity)] = INT_MIN;
}

template <typename T>
__global__ void k_theta_node(int64_t nnode, int B, const Inst<T> *__restrict__ inst,
                             unsigned long long *__restrict__ acc, int *__restrict__ emax,
                             int parity, double *__restrict__ gtheta)
{
    pdl_enter();
    theta_node<T>((int64_t)blockIdx.x * blockDim.x + threadIdx.x, nnode, B, inst, acc, emax,
                  parity, gtheta);
}

// _tape_load! of the next reverse step fused with the design-node write-back
// of the previous one: the first gridN blocks gather, the rest flush nodes.
template <typename T>
__global__ void k_gather_theta(int64_t N, unsigned gridN, const int32_t *__restrict__ perm,
                               const int32_t *__restrict__ srcInv, const T2<T> *__restrict__ sx,
                               const T2<T> *__restrict__ sv, T2<T> *__restrict__ pos,
                               T2<T> *__restrict__ vel, int64_t nnode, int B,
                               const Inst<T> *__restrict__ inst,
                               unsigned long long *__restrict__ acc, int *__restrict__ emax,
                               int parity, double *__restrict__ gtheta)
{
    pdl_enter();
    if (blockIdx.x < gridN) {
        const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= N) return;
        int32_t s = perm[t];
        if (srcInv) s = srcInv[s];
        pos[t] = sx[s];
        vel[t] = sv[s];
    } else {
        theta_node<T>((int64_t)(blockIdx.x - gridN) * blockDim.x + threadIdx.x, nnode, B, inst,
                      acc, emax, parity, gtheta);
    }
}

static __global__ void k_fill_int(int64_t n, int *__restrict__ a, int v)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

template <typename T>
__global__ void k_to_T(int64_t n, const double *__restrict__ a, T *__restrict__ out)
{
    pdl_enter();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (T)a[i];
}

} // namespace sphgb
