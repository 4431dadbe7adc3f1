// Shared device types and the per-pair / per-particle math of the WCSPH step.
//
// Every formula keeps the reference's association and constants so that the
// FP64 build (compiled with --fmad=false, IEEE division and sqrt) reproduces
// the reference's rounding bit for bit:
//   Wendland C2 kernel ............ src/kernels.jl:15-44
//   relu^2 wall and its derivative  src/params.jl:36-46
//   bilinear design field alpha(x)  src/params.jl:54-82
// The FP32 build uses the same source with multiply-add contraction enabled.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sphgb {

template <typename T> struct vec2;
template <> struct vec2<float> { using type = float2; };
template <> struct vec2<double> { using type = double2; };
template <typename T> using T2 = typename vec2<T>::type;

template <typename T> __host__ __device__ __forceinline__ T2<T> mk2(T x, T y)
{
    T2<T> r;
    r.x = x;
    r.y = y;
    return r;
}

// Programmatic dependent launch. A kernel the engine launches with the
// programmatic-stream-serialisation attribute may be scheduled while its
// predecessor on the stream still runs: it first waits until the predecessor
// grid has completed and its writes are visible, before touching memory, and
// only then lets its own successor be scheduled (once all of its blocks have
// passed that point). So at most one kernel waits ahead of the running one;
// successive short kernels start without the launch gap. Triggering the
// successor before the wait instead lets every queued kernel's blocks become
// resident and wait at once, which halved the rate of small states. Without
// the attribute both instructions return at once.
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory");
}

// Products and sums that are never contracted into FMA, whatever the build
// flags: the neighbour-list predicates must see the same r^2 in every kernel.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

template <typename T> __device__ __forceinline__ T r2_exact(T dx, T dy)
{
    return add_rn(mul_rn(dx, dx), mul_rn(dy, dy));
}

// Exact FP64 operations done on the bits with integer instructions: GB300
// runs double-precision arithmetic at a small fraction of its integer rate,
// and small FP64 states are bound by that pipe. Each gives the bits of the
// FP64 instruction it replaces; the FP32 forms are the FP32 instructions.
//
// q / 2 (round to nearest even): the exponent minus one for a normal
// result; a right shift of the significand, ties to even, for a subnormal or
// zero one; inf and NaN unchanged.
template <typename T> __device__ __forceinline__ T half_of(T q) { return (T)0.5 * q; }
template <> __device__ __forceinline__ double half_of<double>(double q)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(q);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    unsigned long long r;
    if (e >= 2u && e != 0x7ffu) {
        r = b - (1ull << 52);
    } else if (e == 0x7ffu) {
        r = b;
    } else {
        const unsigned long long sign = b & (1ull << 63), m = b & ~(1ull << 63);
        r = sign | ((m >> 1) + (m & (m >> 1) & 1ull));
    }
    return __longlong_as_double((long long)r);
}

// 2 q: the exponent plus one for a normal result; a left shift for a
// subnormal or zero q (exact); infinity on overflow; inf and NaN unchanged.
template <typename T> __device__ __forceinline__ T twice_of(T q) { return (T)2 * q; }
template <> __device__ __forceinline__ double twice_of<double>(double q)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(q);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    const unsigned long long sign = b & (1ull << 63);
    unsigned long long r;
    if (e != 0u && e < 0x7feu) r = b + (1ull << 52);
    else if (e == 0u) r = sign | ((b & ~(1ull << 63)) << 1);
    else if (e == 0x7feu) r = sign | 0x7ff0000000000000ull;
    else r = b;
    return __longlong_as_double((long long)r);
}

// a < b for a, b >= 0 and neither -0 (squared distances and their bounds):
// non-negative doubles order like their bits as unsigned integers, and a NaN
// compares false either way.
template <typename T> __device__ __forceinline__ bool lt_nonneg(T a, T b) { return a < b; }
template <> __device__ __forceinline__ bool lt_nonneg<double>(double a, double b)
{
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    // a NaN has the largest exponent, so it is above every finite bound; a
    // negative NaN's sign bit puts it above every non-negative bit pattern
    return ua < ub && ub < 0x7ff0000000000001ull;
}

// Position of the r-th (0-based) set bit of m; requires r < popc(m).
__device__ __forceinline__ int select_bit(uint32_t m, int r)
{
    int pos = 0;
    int c = __popc(m & 0xffffu);
    if (r >= c) { r -= c; m >>= 16; pos += 16; }
    c = __popc(m & 0xffu);
    if (r >= c) { r -= c; m >>= 8; pos += 8; }
    c = __popc(m & 0xfu);
    if (r >= c) { r -= c; m >>= 4; pos += 4; }
    c = __popc(m & 0x3u);
    if (r >= c) { r -= c; m >>= 2; pos += 2; }
    if (r >= (int)(m & 1u)) pos += 1;
    return pos;
}

// SPHParams{T} (src/params.jl:14-28) plus the constants each reference kernel
// forms from it, formed on the host in T with the same association:
//   A = T(7)/(T(4)*T(pi)*h^2), invh = 1/h, r2max = T(4)*h*h,
//   Fc = -5*A*invh*invh, Gc = T(7.5)*A*invh*invh, twomumass = 2*m*mu,
//   c2 = c^2, hxg = Lx/(ngx-1), gxmax = T(ngx-1) - T(1e-6).
template <typename T> struct Phys {
    T h, m, rho0, c, mu, gx, gy, dt, Lx, Ly, kw;
    int ngx, ngy;
    T A, invh, r2max, Fc, Gc, twomumass, c2;
    T hxg, hyg, ngx1, ngy1, gxmax, gymax;
    // model variants (no counterpart in the reference): eos 1 = Tait with
    // exponent gam, visc 1 = Monaghan artificial viscosity; B = c^2 rho0 /
    // gam, dB = B gam / rho0, avc = m alpha c h, eh2 = 0.01 h^2
    int eos, gam, visc;
    T B, dB, avc, eh2;
};

// x^k as a left fold of products (the Tait derivative; same order in the oracle)
template <typename T> __device__ __forceinline__ T pow_fold(T x, int k)
{
    T y = (T)1;
    for (int t = 0; t < k; ++t) y = y * x;
    return y;
}

// (1 + delta)^k - 1 as s_1 = delta, s_{j+1} = s_j (1 + delta) + delta: the Tait
// bracket without the cancellation of x^k - 1 near rho0
template <typename T> __device__ __forceinline__ T pow1m(T delta, int k)
{
    T s = delta;
    const T x = (T)1 + delta;
    for (int t = 1; t < k; ++t) s = s * x + delta;
    return s;
}

// Per-instance constants. A State is one instance; a batch packs B instances
// (uneven particle counts, their own parameters, cell grids and design
// fields) into the same arrays: instance b owns particle slots/ids
// [off, off + n), cells [coff, coff + nx*ny) of the packed cell table and
// design nodes [toff, toff + ngx*ngy). Sorting by packed cell index keeps
// every instance in its own slot range, so one cell-list build serves all.
template <typename T> struct Inst {
    Phys<T> p;
    int off, n;       // particle range
    int nx, ny, coff; // cell grid and its offset in the packed cell table
    int toff;         // design-node offset
    int maxnb;
    int lgN;          // ceil(log2(n + 1)), for the exact dJ/dtheta scale
    T cs, invcs, rc2, r2min, dmax2;
};

// Arrays shared by all instances (cell order), plus the instance table.
template <typename T> struct NLView {
    int64_t N; // total particles
    const T2<T> *pos;
    const T2<T> *xref;
    const uint32_t *center;   // cx | cy << 16 | spill << 31 (1-based, instance grid)
    const uint32_t *masks;    // 6 words (row r: words 2r low, 2r+1 high), masks[w * N + i]
    const uint32_t *tmask;    // this step's words with r^2 < 4h^2 (nullptr: use masks)
    const int32_t *cellStart; // packed table, total cells + 1 exclusive offsets
    const Inst<T> *inst;      // instance table
    const uint16_t *pinst;    // instance of each slot (nullptr: one instance)
    Inst<T> one;              // the instance itself when there is only one
};

template <typename T> __device__ __forceinline__ int inst_of(const NLView<T> &v, int64_t i)
{
    return v.pinst ? (int)v.pinst[i] : 0;
}

// Instance constants of slot i: from the kernel parameters when the system
// holds one instance (constant bank, no memory traffic), from the table
// otherwise. Copied by value so only the fields a kernel uses are loaded.
template <bool MULTI, typename T>
__device__ __forceinline__ decltype(auto) load_inst(const NLView<T> &v, int64_t i)
{
    if constexpr (MULTI) return (v.inst[v.pinst[i]]); // const Inst<T>& into the table
    else return Inst<T>(v.one);                       // value from the parameters
}

template <bool MULTI, typename T>
__device__ __forceinline__ decltype(auto) pick_inst(const Inst<T> &one, const Inst<T> *inst, int b)
{
    if constexpr (MULTI) return (inst[b]);
    else return Inst<T>(one);
}

// Visit the neighbours of particle i in the reference's scan order
// (src/neighbors.jl:217-244): cell rows ddy = -1..1, within a row cells
// ddx = -1..1, within a cell ascending particle id. Because particles are
// stored sorted by (cell, id), each row is one contiguous slot range and the
// order is simply ascending slot. The fast path walks the bits of one 64-bit
// mask per row. A particle whose row range exceeds 64 slots is "spilled": it
// re-evaluates the rebuild-time predicate r2min < r^2 < rc^2 on the stored
// rebuild positions and truncates at maxnb, which is exactly what the
// reference's fixed-length neighbour rows hold.
template <typename T, typename F>
__device__ __forceinline__ void for_each_neighbor(const NLView<T> &v, const Inst<T> &I, int64_t i,
                                                  F &&f)
{
    const uint32_t cc = v.center[i];
    const int cx = (int)(cc & 0xffffu);
    const int cy = (int)((cc >> 16) & 0x7fffu);
    const int jx0 = cx - 1 > 1 ? cx - 1 : 1;
    if (!(cc >> 31)) {
        // Slot indices fit in 32 bits (N < 2^31). The three row masks are
        // walked as one sequence of six 32-bit words (row 0 low, row 0 high,
        // row 1 low, ...), bit order = slot order, in a single loop: a lane
        // that runs out of bits in one word moves to its next non-empty word
        // while the others keep visiting neighbours, so a warp pays for its
        // largest total neighbour count rather than the sum of its per-row
        // maxima (a row-by-row loop measured 17% slower), and empty words
        // cost no iteration (7% faster than visiting all six).
        const int row0 = I.coff + (jx0 - 1) + (cy - 2) * I.nx; // cell (jx0, cy - 1)
        const uint32_t *mk = v.tmask ? v.tmask : v.masks;
        const uint64_t m0 = ((uint64_t)mk[v.N + i] << 32) | mk[i];
        const uint64_t m1 = ((uint64_t)mk[3 * v.N + i] << 32) | mk[2 * v.N + i];
        const uint64_t m2 = ((uint64_t)mk[5 * v.N + i] << 32) | mk[4 * v.N + i];
        const int b0 = m0 ? v.cellStart[row0] : 0;
        const int b1 = m1 ? v.cellStart[row0 + I.nx] : 0;
        const int b2 = m2 ? v.cellStart[row0 + 2 * I.nx] : 0;
        // words that hold candidates; transitions jump straight to the next one
        const uint32_t ne = (uint32_t)((uint32_t)m0 != 0u) | ((uint32_t)((m0 >> 32) != 0u) << 1) |
                            ((uint32_t)((uint32_t)m1 != 0u) << 2) | ((uint32_t)((m1 >> 32) != 0u) << 3) |
                            ((uint32_t)((uint32_t)m2 != 0u) << 4) | ((uint32_t)((m2 >> 32) != 0u) << 5);
        uint32_t m = (uint32_t)m0;
        int base = b0;
        int w = 0;
        for (;;) {
            if (m == 0u) {
                const uint32_t rest = ne >> (w + 1);
                if (rest == 0u) break;
                w += __ffs((int)rest);
                const uint64_t mr = w < 2 ? m0 : (w < 4 ? m1 : m2);
                const int br = w < 2 ? b0 : (w < 4 ? b1 : b2);
                m = (w & 1) ? (uint32_t)(mr >> 32) : (uint32_t)mr;
                base = br + ((w & 1) << 5);
                continue;
            }
            const int k = __ffs((int)m) - 1;
            m &= m - 1u;
            f(base + k);
        }
    } else {
        const int jx1 = cx + 1 < I.nx ? cx + 1 : I.nx;
        const T2<T> xr = v.xref[i];
        int cnt = 0;
        for (int r = 0; r < 3; ++r) {
            const int jy = cy + r - 1;
            if (jy < 1 || jy > I.ny) continue;
            const int row = I.coff + (jy - 1) * I.nx;
            const int b = v.cellStart[row + jx0 - 1];
            const int e = v.cellStart[row + jx1];
            for (int j = b; j < e; ++j) {
                const T2<T> xj = v.xref[j];
                const T r2 = r2_exact<T>(sub_rn(xr.x, xj.x), sub_rn(xr.y, xj.y));
                if (lt_nonneg(I.r2min, r2) && lt_nonneg(r2, I.rc2)) {
                    if (cnt < I.maxnb) {
                        ++cnt;
                        f(j);
                    }
                }
            }
        }
    }
}

// Per-pair square root and reciprocal. FP64 keeps IEEE sqrt and division
// (reference-exact); FP32 uses the PTX approximate square root (one
// instruction, sqrt(+0) = +0, within a few ulp; the FP32 path is checked
// against FP64 by tolerance).
__device__ __forceinline__ double pair_sqrt(double r2) { return sqrt(r2); }
__device__ __forceinline__ float pair_sqrt(float r2)
{
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(r2));
    return r;
}

// clamp(unsafe_trunc(Int, floor(v)) + 2, 1, n) (src/neighbors.jl:38-42,217-218).
// The float clamp keeps the conversion defined; no finite result changes.
template <typename T> __host__ __device__ __forceinline__ int cell_coord(T v, int n)
{
    T f = floor(v);
    if (!(f > (T)(-4))) f = (T)(-4);
    if (f > (T)(n + 4)) f = (T)(n + 4);
    int c = (int)f + 2;
    c = c < 1 ? 1 : c;
    return c > n ? n : c;
}

// wall_accel / wall_daccel (src/params.jl:36-46); max(zero(T), -x) keeps +0.
template <typename T> __device__ __forceinline__ T wall_accel(T x, T L, T kw)
{
    const T lo = (-x > (T)0) ? -x : (T)0;
    const T hi = (x - L > (T)0) ? x - L : (T)0;
    return kw * (lo * lo - hi * hi);
}

template <typename T> __device__ __forceinline__ T wall_daccel(T x, T L, T kw)
{
    const T lo = (-x > (T)0) ? -x : (T)0;
    const T hi = (x - L > (T)0) ? x - L : (T)0;
    return kw * ((T)(-2) * lo - (T)2 * hi);
}

// interp_cell (src/params.jl:54-68), 0-based i0, j0.
template <typename T>
__device__ __forceinline__ void interp_cell(T x, T y, const Phys<T> &p, int &i0, int &j0, T &fx,
                                            T &fy, T &ax, T &ay)
{
    const T gx = x / p.hxg;
    const T gy = y / p.hyg;
    ax = ((gx > (T)0) & (gx < p.ngx1)) ? (T)1 : (T)0;
    ay = ((gy > (T)0) & (gy < p.ngy1)) ? (T)1 : (T)0;
    const T gxc = gx > p.gxmax ? p.gxmax : (gx < (T)0 ? (T)0 : gx);
    const T gyc = gy > p.gymax ? p.gymax : (gy < (T)0 ? (T)0 : gy);
    const T fgx = floor(gxc), fgy = floor(gyc);
    int a = (fgx == fgx) ? (int)fgx : 0;
    int b = (fgy == fgy) ? (int)fgy : 0;
    a = a < 0 ? 0 : (a > p.ngx - 2 ? p.ngx - 2 : a);
    b = b < 0 ? 0 : (b > p.ngy - 2 ? p.ngy - 2 : b);
    i0 = a;
    j0 = b;
    fx = gxc - (T)a;
    fy = gyc - (T)b;
}

// interp_alpha (src/params.jl:71-82); theta is (ngy, ngx) column-major.
template <typename T>
__device__ __forceinline__ void interp_alpha(const T *theta, T x, T y, const Phys<T> &p, T &a,
                                             T &dadx, T &dady)
{
    int i0, j0;
    T fx, fy, ax, ay;
    interp_cell(x, y, p, i0, j0, fx, fy, ax, ay);
    const int64_t l00 = (int64_t)j0 + (int64_t)i0 * p.ngy;
    const T t00 = __ldg(theta + l00);
    const T t01 = __ldg(theta + l00 + p.ngy);
    const T t10 = __ldg(theta + l00 + 1);
    const T t11 = __ldg(theta + l00 + p.ngy + 1);
    a = ((T)1 - fx) * ((T)1 - fy) * t00 + fx * ((T)1 - fy) * t01 + ((T)1 - fx) * fy * t10 +
        fx * fy * t11;
    dadx = (((T)1 - fy) * (t01 - t00) + fy * (t11 - t10)) / p.hxg * ax;
    dady = (((T)1 - fx) * (t10 - t00) + fx * (t11 - t01)) / p.hyg * ay;
}

template <typename T> __device__ __forceinline__ T interp_alpha_value(const T *theta, T x, T y,
                                                                      const Phys<T> &p)
{
    int i0, j0;
    T fx, fy, ax, ay;
    interp_cell(x, y, p, i0, j0, fx, fy, ax, ay);
    const int64_t l00 = (int64_t)j0 + (int64_t)i0 * p.ngy;
    const T t00 = __ldg(theta + l00);
    const T t01 = __ldg(theta + l00 + p.ngy);
    const T t10 = __ldg(theta + l00 + 1);
    const T t11 = __ldg(theta + l00 + p.ngy + 1);
    return ((T)1 - fx) * ((T)1 - fy) * t00 + fx * ((T)1 - fy) * t01 + ((T)1 - fx) * fy * t10 +
           fx * fy * t11;
}

// Status bits kept in a device word and returned at the API boundary.
enum : uint32_t {
    FLAG_NL_OVERFLOW = 1u,     // a neighbour row exceeded maxnb (reference flags[1])
    FLAG_DISPLACEMENT = 2u,    // displacement since rebuild > skin*h (reference flags[2])
    FLAG_NONFINITE = 4u,       // a non-finite position or velocity was produced
};

} // namespace sphgb
