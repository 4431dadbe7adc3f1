// The design side of the topology-optimisation caller on the device: the
// Borrvall-Petersson interpolation alpha(rho) and its derivative, the
// linear-weight density filter with its clamp and its transposed adjoint, the
// lower-bound volume projection by bisection, and the projected-gradient
// candidate of the line search (scripts/03_optimize.jl:142-219,314-341).
// Design variables are double whatever the particle precision, as the
// reference keeps them (TW = Float64). Compiled with --fmad=false: every
// product and sum is rounded separately, in the reference's order, so the
// filter, its adjoint and alpha(rho) equal the host restatement bit for bit.
//
// Layout: a design of ngy x ngx nodes is stored (ngy, ngx) column-major, node
// (j, i) at j + i * ngy (0-based), like theta. The filter is a CSR table: node
// k's neighbours in the reference's order (jj outer, ii inner) with their
// normalised weights. Its adjoint scatters out[jj, ii] += w g[j, i] over the
// nodes (j, i) in the reference's loop order (j outer, i inner); on the device
// that is a gather over a second CSR table holding, for every node, the nodes
// that list it, in that same order, so each sum is added in the reference's
// order.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/sphadjoint_gb300.h"
#include "sph_iface.hpp"

namespace sphgb {
namespace {

constexpr int kDB = 256;
constexpr int kProjThreads = 1024;

__device__ __forceinline__ double alpha_rho(double rd, double amax, double qp)
{
    return amax * qp * (1.0 - rd) / (qp + rd);
}

__device__ __forceinline__ double dalpha_rho(double rd, double amax, double qp)
{
    const double d = qp + rd;
    return -amax * qp * (qp + 1.0) / (d * d);
}

__device__ __forceinline__ double clamp01(double v) { return fmin(fmax(v, 0.0), 1.0); }

// apply_filter: y_k = clamp(sum_(m, w) w x_m, 0, 1)
__global__ void k_filter(int n, const int *__restrict__ start, const int *__restrict__ idx,
                         const double *__restrict__ w, const double *__restrict__ x,
                         double *__restrict__ y)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double acc = 0.0;
    for (int e = start[k]; e < start[k + 1]; ++e) acc += w[e] * x[idx[e]];
    y[k] = clamp01(acc);
}

// filter_adjoint as a gather: out_m = sum over the nodes k that list m, in the
// reference's scatter order, of w g_k
__global__ void k_filter_adj(int n, const int *__restrict__ start, const int *__restrict__ idx,
                             const double *__restrict__ w, const double *__restrict__ g,
                             double *__restrict__ out)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    double acc = 0.0;
    for (int e = start[m]; e < start[m + 1]; ++e) acc += w[e] * g[idx[e]];
    out[m] = acc;
}

// theta = alpha(rdf) in the field's precision
template <typename T>
__global__ void k_alpha(int n, const double *__restrict__ rdf, double amax, double qp,
                        T *__restrict__ theta, double *__restrict__ a64)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double a = alpha_rho(rdf[k], amax, qp);
    if (theta) theta[k] = (T)a;
    if (a64) a64[k] = a;
}

__global__ void k_dalpha(int n, const double *__restrict__ rdf, double amax, double qp,
                         double *__restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = dalpha_rho(rdf[k], amax, qp);
}

// grdf = gtheta * dalpha(rdf)
__global__ void k_chain(int n, const double *__restrict__ gtheta, const double *__restrict__ rdf,
                        double amax, double qp, double *__restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = gtheta[k] * dalpha_rho(rdf[k], amax, qp);
}

// Fixed-order block sum of v(k) over k < n (all threads get the result).
template <typename F> __device__ double block_sum(int n, F &&v)
{
    __shared__ double sm[kProjThreads];
    double a = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) a += v(k);
    sm[threadIdx.x] = a;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    const double s = sm[0];
    __syncthreads();
    return s;
}

// project_volume on one block: x = clamp(in); if mean(x) < volfrac, shift it
// up by the bisection of the reference (60 halvings of [0, 1]). With step !=
// 0 the input is the line-search candidate rd - step * g / gmax, gmax =
// max |g| computed here. Means are fixed-order sums / n.
__global__ void __launch_bounds__(kProjThreads)
    k_project(int n, const double *__restrict__ rd, const double *__restrict__ g, double step,
              double volfrac, double *__restrict__ out, double *__restrict__ gmaxOut)
{
    __shared__ double red[kProjThreads];
    double gmax = 1.0;
    if (g) {
        double mx = 0.0;
        for (int k = threadIdx.x; k < n; k += blockDim.x) mx = fmax(mx, fabs(g[k]));
        red[threadIdx.x] = mx;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
            __syncthreads();
        }
        gmax = red[0];
        __syncthreads();
        if (gmaxOut && threadIdx.x == 0) *gmaxOut = gmax;
    }
    auto xin = [&](int k) {
        const double v = g ? rd[k] - step * g[k] / gmax : rd[k];
        return clamp01(v);
    };
    for (int k = threadIdx.x; k < n; k += blockDim.x) out[k] = xin(k);
    __syncthreads();
    const double nd = (double)n;
    if (block_sum(n, [&](int k) { return out[k]; }) / nd >= volfrac) return;
    double lo = 0.0, hi = 1.0;
    for (int it = 0; it < 60; ++it) {
        const double mid = (lo + hi) / 2.0;
        const double m = block_sum(n, [&](int k) { return clamp01(out[k] + mid); }) / nd;
        if (m < volfrac) lo = mid;
        else hi = mid;
    }
    const double sh = (lo + hi) / 2.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) out[k] = clamp01(out[k] + sh);
}

__global__ void k_absmax(int n, const double *__restrict__ g, double *__restrict__ out)
{
    __shared__ double red[kDB];
    double mx = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) mx = fmax(mx, fabs(g[k]));
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

template <typename T> struct Dev {
    T *p = nullptr;
    size_t n = 0;
    void alloc(size_t c)
    {
        free();
        n = c;
        if (c) cuda_check(cudaMalloc((void **)&p, sizeof(T) * c), "cudaMalloc(design)");
    }
    void free()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~Dev() { free(); }
    void up(const T *h, cudaStream_t s)
    {
        cuda_check(cudaMemcpyAsync(p, h, sizeof(T) * n, cudaMemcpyHostToDevice, s), "design upload");
    }
    void down(T *h, cudaStream_t s) const
    {
        cuda_check(cudaMemcpyAsync(h, p, sizeof(T) * n, cudaMemcpyDeviceToHost, s), "design download");
    }
};

class Design {
  public:
    int ngx, ngy, n, r;
    double amax, qp, volfrac;
    Dev<int> fStart, fIdx, aStart, aIdx;
    Dev<double> fW, aW;
    Dev<double> rd, rdf, grad, cand, work, a64, scal;
    Dev<float> th32;
    Dev<double> th64;

    Design(int gx, int gy, int radius, double am, double q, double vf)
        : ngx(gx), ngy(gy), n(gx * gy), r(radius), amax(am), qp(q), volfrac(vf)
    {
        if (gx < 2 || gy < 2) throw Error(ERR_ARG, "design grid must be at least 2 x 2");
        if (radius < 0) throw Error(ERR_ARG, "filter radius must be >= 0");
        if ((int64_t)gx * gy > (1 << 28)) throw Error(ERR_ARG, "design grid too large");
        // build_filter (03_optimize.jl:150-165): weights (r + 1) - dist > 0,
        // normalised by their sum, neighbours jj outer, ii inner
        std::vector<int> fs{0}, fi;
        std::vector<double> fw;
        auto node = [&](int j, int i) { return j + i * ngy; };
        std::vector<std::vector<std::pair<int, double>>> rows((size_t)n);
        for (int j = 0; j < ngy; ++j)
            for (int i = 0; i < ngx; ++i) {
                std::vector<std::pair<int, double>> lst;
                double s = 0.0;
                for (int jj = std::max(0, j - r); jj <= std::min(ngy - 1, j + r); ++jj)
                    for (int ii = std::max(0, i - r); ii <= std::min(ngx - 1, i + r); ++ii) {
                        const double w = (double)(r + 1) -
                                         std::sqrt((double)((ii - i) * (ii - i) + (jj - j) * (jj - j)));
                        if (w > 0) {
                            lst.push_back({node(jj, ii), w});
                            s += w;
                        }
                    }
                for (auto &e : lst) e.second = e.second / s;
                rows[(size_t)node(j, i)] = lst;
            }
        for (int k = 0; k < n; ++k) {
            for (auto &e : rows[(size_t)k]) {
                fi.push_back(e.first);
                fw.push_back(e.second);
            }
            fs.push_back((int)fi.size());
        }
        // filter_adjoint (03_optimize.jl:187-195): for (j, i) in the loop order,
        // out[m] += w g[(j, i)] for every (m, w) of (j, i)'s list
        std::vector<std::vector<std::pair<int, double>>> into((size_t)n);
        for (int j = 0; j < ngy; ++j)
            for (int i = 0; i < ngx; ++i)
                for (auto &e : rows[(size_t)node(j, i)]) into[(size_t)e.first].push_back({node(j, i), e.second});
        std::vector<int> as{0}, ai;
        std::vector<double> aw;
        for (int m = 0; m < n; ++m) {
            for (auto &e : into[(size_t)m]) {
                ai.push_back(e.first);
                aw.push_back(e.second);
            }
            as.push_back((int)ai.size());
        }
        cudaStream_t s = rt_stream();
        fStart.alloc(fs.size()); fIdx.alloc(fi.size()); fW.alloc(fw.size());
        aStart.alloc(as.size()); aIdx.alloc(ai.size()); aW.alloc(aw.size());
        fStart.up(fs.data(), s); fIdx.up(fi.data(), s); fW.up(fw.data(), s);
        aStart.up(as.data(), s); aIdx.up(ai.data(), s); aW.up(aw.data(), s);
        rd.alloc(n); rdf.alloc(n); grad.alloc(n); cand.alloc(n); work.alloc(n); a64.alloc(n);
        scal.alloc(4);
        cuda_check(cudaMemsetAsync(grad.p, 0, sizeof(double) * n, s), "memset");
        cuda_check(cudaStreamSynchronize(s), "design set-up");
    }

    unsigned blocks() const { return (unsigned)((n + kDB - 1) / kDB); }

    void filter(const double *x, double *y)
    {
        k_filter<<<blocks(), kDB, 0, rt_stream()>>>(n, fStart.p, fIdx.p, fW.p, x, y);
    }
    void adjoint(const double *g, double *out)
    {
        k_filter_adj<<<blocks(), kDB, 0, rt_stream()>>>(n, aStart.p, aIdx.p, aW.p, g, out);
    }
    void project(const double *x, const double *g, double step, double *out)
    {
        k_project<<<1, kProjThreads, 0, rt_stream()>>>(n, x, g, step, volfrac, out,
                                                       g ? scal.p : nullptr);
    }
    // theta = alpha(filter(x)) written into the field (device to device)
    void to_theta(const double *x, FieldI *f)
    {
        if (f->ngx() != ngx || f->ngy() != ngy) throw Error(ERR_ARG, "field shape differs from the design");
        filter(x, rdf.p);
        if (f->dtype() == F64) {
            if (!th64.p) th64.alloc(n);
            k_alpha<double><<<blocks(), kDB, 0, rt_stream()>>>(n, rdf.p, amax, qp, th64.p, nullptr);
            f->upload_device(th64.p);
        } else {
            if (!th32.p) th32.alloc(n);
            k_alpha<float><<<blocks(), kDB, 0, rt_stream()>>>(n, rdf.p, amax, qp, th32.p, nullptr);
            f->upload_device(th32.p);
        }
    }
    // grad = filter_adjoint(gtheta * dalpha(filter(rd)))
    void gradient(const double *gtheta)
    {
        filter(rd.p, rdf.p);
        k_chain<<<blocks(), kDB, 0, rt_stream()>>>(n, gtheta, rdf.p, amax, qp, work.p);
        adjoint(work.p, grad.p);
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

Design *DS(sph_design d)
{
    if (!d) throw Error(ERR_ARG, "design is NULL");
    return reinterpret_cast<Design *>(d);
}

} // namespace
} // namespace sphgb

using namespace sphgb;

extern "C" {

SPH_API int32_t sph_design_create(int32_t ngx, int32_t ngy, int32_t radius, double alpha_max,
                                  double qp, double volfrac, sph_design *out)
{
    return guard([&] {
        if (!out) throw Error(ERR_ARG, "out is NULL");
        *out = reinterpret_cast<sph_design>(new Design(ngx, ngy, radius, alpha_max, qp, volfrac));
    });
}

SPH_API int32_t sph_design_destroy(sph_design d)
{
    return guard([&] {
        if (d) cuda_check(cudaStreamSynchronize(rt_stream()), "design destroy");
        delete reinterpret_cast<Design *>(d);
    });
}

SPH_API int32_t sph_design_set(sph_design d, const double *rd)
{
    return guard([&] {
        Design *D = DS(d);
        if (!rd) throw Error(ERR_ARG, "rd is NULL");
        D->rd.up(rd, rt_stream());
        cuda_check(cudaStreamSynchronize(rt_stream()), "design set");
    });
}

SPH_API int32_t sph_design_get(sph_design d, double *rd, double *rdf, double *grad)
{
    return guard([&] {
        Design *D = DS(d);
        cudaStream_t s = rt_stream();
        if (rd) D->rd.down(rd, s);
        if (rdf) {
            D->filter(D->rd.p, D->rdf.p);
            D->rdf.down(rdf, s);
        }
        if (grad) D->grad.down(grad, s);
        cuda_check(cudaStreamSynchronize(s), "design get");
    });
}

SPH_API int32_t sph_design_apply(sph_design d, int32_t op, const double *in, double *out)
{
    return guard([&] {
        Design *D = DS(d);
        if (!in || !out) throw Error(ERR_ARG, "NULL array");
        cudaStream_t s = rt_stream();
        D->work.up(in, s);
        switch (op) {
        case SPH_DESIGN_FILTER: D->filter(D->work.p, D->cand.p); break;
        case SPH_DESIGN_FILTER_ADJOINT: D->adjoint(D->work.p, D->cand.p); break;
        case SPH_DESIGN_PROJECT: D->project(D->work.p, nullptr, 0.0, D->cand.p); break;
        case SPH_DESIGN_ALPHA:
            k_alpha<double><<<D->blocks(), kDB, 0, s>>>(D->n, D->work.p, D->amax, D->qp, nullptr,
                                                        D->cand.p);
            break;
        case SPH_DESIGN_DALPHA:
            k_dalpha<<<D->blocks(), kDB, 0, s>>>(D->n, D->work.p, D->amax, D->qp, D->cand.p);
            break;
        default: throw Error(ERR_ARG, "unknown design operation");
        }
        cuda_check(cudaGetLastError(), "design apply");
        D->cand.down(out, s);
        cuda_check(cudaStreamSynchronize(s), "design apply");
    });
}

SPH_API int32_t sph_design_to_theta(sph_design d, sph_field theta)
{
    return guard([&] {
        Design *D = DS(d);
        if (!theta) throw Error(ERR_ARG, "theta is NULL");
        D->to_theta(D->rd.p, reinterpret_cast<FieldI *>(theta));
        cuda_check(cudaGetLastError(), "design to theta");
    });
}

SPH_API int32_t sph_design_gradient(sph_design d, sph_workspace ws, double *gmax)
{
    return guard([&] {
        Design *D = DS(d);
        if (!ws) throw Error(ERR_ARG, "workspace is NULL");
        WorkI *W = reinterpret_cast<WorkI *>(ws);
        if (W->batch() != 1) throw Error(ERR_ARG, "one instance per design");
        D->gradient(W->gtheta_device(D->n));
        if (gmax) {
            k_absmax<<<1, kDB, 0, rt_stream()>>>(D->n, D->grad.p, D->scal.p + 1);
            cuda_check(cudaMemcpyAsync(gmax, D->scal.p + 1, sizeof(double), cudaMemcpyDeviceToHost,
                                       rt_stream()),
                       "gmax");
            cuda_check(cudaStreamSynchronize(rt_stream()), "design gradient");
        }
        cuda_check(cudaGetLastError(), "design gradient");
    });
}

SPH_API int32_t sph_design_candidate(sph_design d, double step, sph_field theta)
{
    return guard([&] {
        Design *D = DS(d);
        D->project(D->rd.p, D->grad.p, step, D->cand.p);
        if (theta) D->to_theta(D->cand.p, reinterpret_cast<FieldI *>(theta));
        cuda_check(cudaGetLastError(), "design candidate");
    });
}

SPH_API int32_t sph_design_accept(sph_design d)
{
    return guard([&] {
        Design *D = DS(d);
        cuda_check(cudaMemcpyAsync(D->rd.p, D->cand.p, sizeof(double) * D->n,
                                   cudaMemcpyDeviceToDevice, rt_stream()),
                   "design accept");
    });
}

} // extern "C"
