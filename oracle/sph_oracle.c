/*
 * CPU parity oracle for the sphadjoint_gb300 CUDA library (test
 * infrastructure, never linked by the product).
 *
 * Restates the reference's Julia kernels (src/kernels.jl, src/params.jl,
 * src/neighbors.jl, src/forward.jl, src/adjoint.jl, src/driver.jl) in C,
 * instantiated for double (_f64) and float (_f32). Build with
 * -ffp-contract=off so no multiply-add is fused: Julia does not contract
 * without @fastmath / @muladd, and parity is checked bit for bit in FP64.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* SPHParams as the caller passes it (every field double; converted to T),
   plus the equation of state and viscosity model: eos 0 = linear
   (the reference), 1 = Tait with integer exponent gamma; visc 0 = Morris
   (the reference), 1 = Monaghan artificial viscosity with coefficient alpha.
   The two variants have no counterpart in the reference. */
typedef struct {
    double h, m, rho0, c, mu, gx, gy, dt, Lx, Ly, kw;
    int32_t ngx, ngy;
    int32_t eos, gamma, visc, pad;
    double alpha;
} orc_params;

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

#define R double
#define SFX _f64
#define FLOOR floor
#define SQRT sqrt
#define EPS_R DBL_EPSILON
#include "sph_oracle_body.h"
#undef R
#undef SFX
#undef FLOOR
#undef SQRT
#undef EPS_R
#undef TH

#define R float
#define SFX _f32
#define FLOOR floorf
#define SQRT sqrtf
#define EPS_R FLT_EPSILON
#include "sph_oracle_body.h"
