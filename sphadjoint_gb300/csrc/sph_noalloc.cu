// Cell-list build (build!, src/neighbors.jl:97-114) that allocates nothing.
//
// Who needs this: callers that own all device memory themselves and cannot let
// a library call cudaMalloc — a Julia caller whose arrays come from CUDA.jl's
// pooled allocator (a raw cudaMalloc inside a ccall bypasses the pool and can
// fail or stall when the pool holds most of the device), code running under a
// memory budget enforced by its own allocator, or a host that must not create
// device allocations after start-up. They pass device pointers for the
// positions and for the three outputs; the working arrays the build needs (cell
// of each particle, bucket cursors, scan partials) live in one file-scope
// __device__ array of fixed size instead of per-call allocations.
//
// Limits and sharing:
//   * N <= SPH_NOALLOC_MAX_PARTICLES (2^20) and nx*ny <= SPH_NOALLOC_MAX_CELLS
//     (2^20); larger requests fail with SPH_ERR_ARG. The array takes
//     4 * (2 * 2^20 + 2 * (2^20 + 1) + 576) bytes (about 16 MiB) on every GPU
//     that loads this library, for the life of the process.
//   * All calls share that array and it keeps the previous call's contents;
//     this entry point writes every word it reads before reading it, and zeroes
//     the caller's `counts` itself. Calls that overlap on the GPU (two streams,
//     or two host threads) race on the array: serialise them.
//   * Each call resolves the array's device address with cudaGetSymbolAddress
//     on the current device, so the address stays right after a
//     cudaDeviceReset. While `stream` is being captured into a CUDA graph the
//     call uses the address from its last uncaptured call on that device
//     instead: make one uncaptured call on each device before capturing.
//   * A CUDA error already pending when the call starts (left by other code)
//     is reported as such, and nothing is launched.
#include <mutex>
#include <string>

#include "../../include/sphadjoint_gb300.h"
#include "sph_iface.hpp"
#include "sph_kernels.cuh"

namespace sphgb {
namespace {

constexpr int64_t kMaxParticles = SPH_NOALLOC_MAX_PARTICLES;
constexpr int64_t kMaxCells = SPH_NOALLOC_MAX_CELLS;
constexpr int64_t kScanSlots = (kMaxCells + kScanTile - 1) / kScanTile + 1;
// layout (int32 words): cell of each particle | bucket (particle ids)
// | cell starts (ncell + 1) | cursors (ncell + 1) | scan block sums
constexpr int64_t kOffCell = 0;
constexpr int64_t kOffSrc = kOffCell + kMaxParticles;
constexpr int64_t kOffStart = kOffSrc + kMaxParticles;
constexpr int64_t kOffCursor = kOffStart + kMaxCells + 1;
constexpr int64_t kOffScan = kOffCursor + kMaxCells + 1;
constexpr int64_t kWords = kOffScan + ((kScanSlots + 63) / 64) * 64;

static __device__ __align__(256) int32_t g_scratch[kWords];

inline unsigned grid_blocks(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

constexpr int kMaxDevices = 64;
std::mutex g_mu;
int32_t *g_ptr[kMaxDevices] = {};

// Device address of g_scratch on the current device: resolved on every call
// outside a stream capture (cheap, and right after a context reset), taken
// from the last such call while `s` is being captured.
int32_t *scratch_ptr(int dev, cudaStream_t s)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cuda_check(cudaStreamIsCapturing(s, &cap), "cudaStreamIsCapturing");
    std::lock_guard<std::mutex> g(g_mu);
    if (cap != cudaStreamCaptureStatusNone) {
        if (!g_ptr[dev])
            throw Error(ERR_STATE, "sph_build_cells_noalloc: make one call on this device "
                                   "outside stream capture first (it resolves the work "
                                   "array's device address)");
        return g_ptr[dev];
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
        (void)cudaGetLastError();
        throw Error(ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                  cudaGetErrorString(e));
    }
    g_ptr[dev] = static_cast<int32_t *>(p);
    return g_ptr[dev];
}

// _cl_assign! for one grid passed by value: cell of every particle (x / cs,
// as cell_index does) and a warp-aggregated histogram into `counts`.
template <typename T>
__global__ void k_na_assign(int64_t N, const T2<T> *__restrict__ pos, T cs, int nx, int ny,
                            int32_t *__restrict__ cellTmp, int32_t *__restrict__ counts)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < N;
    int32_t c = -1;
    if (live) {
        const T2<T> x = pos[i];
        const int cx = cell_coord<T>(x.x / cs, nx);
        const int cy = cell_coord<T>(x.y / cs, ny);
        c = (cx - 1) + (cy - 1) * nx;
        cellTmp[i] = c;
    }
    const unsigned act = __ballot_sync(0xffffffffu, live);
    if (live) {
        const unsigned peers = __match_any_sync(act, c);
        if ((int)lane_id() == __ffs(peers) - 1) atomicAdd(counts + c, __popc(peers));
    }
}

// k_bucket without a permutation: particle i is its own id.
__global__ void k_na_bucket(int64_t N, const int32_t *__restrict__ cellTmp,
                            int32_t *__restrict__ cursor, int32_t *__restrict__ bucketSrc)
{
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
    bucketSrc[base + __popc(peers & ((1u << lane_id()) - 1u))] = (int32_t)i;
}

// _cl_sort_cells! as a rank within the cell; writes 1-based ids to `order`.
__global__ void k_na_rank(int64_t N, const int32_t *__restrict__ cellTmp,
                          const int32_t *__restrict__ cellStart,
                          const int32_t *__restrict__ bucketSrc, int32_t *__restrict__ order)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const int32_t id = bucketSrc[s];
    const int32_t c = cellTmp[id];
    const int32_t b = cellStart[c], e = cellStart[c + 1];
    int32_t rank = 0;
    for (int32_t k = b; k < e; ++k) rank += (bucketSrc[k] < id) ? 1 : 0;
    order[b + rank] = id + 1;
}

template <typename T>
void build_cells_noalloc(const void *X, int64_t N, double cs, int nx, int ny, int32_t *counts,
                         int32_t *starts, int32_t *order, cudaStream_t s)
{
    // an error left pending by other code is not this call's failure: report
    // it as pending and launch nothing
    const cudaError_t pend = cudaPeekAtLastError();
    if (pend != cudaSuccess)
        throw Error(ERR_CUDA, std::string("sph_build_cells_noalloc: a CUDA error was already "
                                          "pending before the call: ") +
                                  cudaGetErrorString(pend));
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) throw Error(ERR_ARG, "device ordinal out of range");
    int32_t *w = scratch_ptr(dev, s);
    const int64_t ncell = (int64_t)nx * ny;
    int32_t *cellTmp = w + kOffCell, *src = w + kOffSrc, *start = w + kOffStart;
    int32_t *cursor = w + kOffCursor, *scan = w + kOffScan;
    const T csT = (T)cs;

    cuda_check(cudaMemsetAsync(counts, 0, sizeof(int32_t) * ncell, s), "cudaMemsetAsync(counts)");
    if (N > 0) {
        k_na_assign<T><<<grid_blocks(N), kBlock, 0, s>>>(N, (const T2<T> *)X, csT, nx, ny, cellTmp,
                                                         counts);
    }
    const int64_t nb = (ncell + kScanTile - 1) / kScanTile;
    if (nb <= 1) {
        k_scan_down<<<1, kBlock, 0, s>>>(counts, ncell, nullptr, start, cursor);
    } else {
        k_scan_reduce<<<(unsigned)nb, kBlock, 0, s>>>(counts, ncell, scan);
        k_scan_top<<<1, 1024, 0, s>>>(scan, nb);
        k_scan_down<<<(unsigned)nb, kBlock, 0, s>>>(counts, ncell, scan, start, cursor);
    }
    cuda_check(cudaMemcpyAsync(starts, start, sizeof(int32_t) * ncell, cudaMemcpyDeviceToDevice, s),
               "cudaMemcpyAsync(starts)");
    if (N > 0) {
        k_na_bucket<<<grid_blocks(N), kBlock, 0, s>>>(N, cellTmp, cursor, src);
        k_na_rank<<<grid_blocks(N), kBlock, 0, s>>>(N, cellTmp, start, src, order);
    }
    cuda_check(cudaGetLastError(), "build_cells_noalloc launch");
}

} // namespace
} // namespace sphgb

using namespace sphgb;

extern "C" SPH_API int32_t sph_build_cells_noalloc(const void *X, int64_t N, int32_t dtype,
                                                   double cs, int32_t nx, int32_t ny,
                                                   int32_t *counts, int32_t *starts,
                                                   int32_t *order, void *stream)
{
    try {
        if (dtype != SPH_F64 && dtype != SPH_F32) throw Error(ERR_DTYPE, "dtype must be SPH_F64 or SPH_F32");
        if (N < 0 || N > kMaxParticles)
            throw Error(ERR_ARG, "sph_build_cells_noalloc: N = " + std::to_string(N) +
                                     " exceeds the fixed scratch limit of " +
                                     std::to_string(kMaxParticles) + " particles");
        if (nx < 1 || ny < 1 || (int64_t)nx * ny > kMaxCells)
            throw Error(ERR_ARG, "sph_build_cells_noalloc: nx*ny = " +
                                     std::to_string((int64_t)nx * ny) +
                                     " cells is outside 1.." + std::to_string(kMaxCells));
        if (!(cs > 0)) throw Error(ERR_ARG, "sph_build_cells_noalloc: cell size must be positive");
        if ((N > 0 && (!X || !order)) || !counts || !starts)
            throw Error(ERR_ARG, "sph_build_cells_noalloc: NULL device pointer");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (dtype == SPH_F64)
            build_cells_noalloc<double>(X, N, cs, nx, ny, counts, starts, order, s);
        else
            build_cells_noalloc<float>(X, N, cs, nx, ny, counts, starts, order, s);
        return SPH_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return SPH_ERR_STATE;
    }
}
