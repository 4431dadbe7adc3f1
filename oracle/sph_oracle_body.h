/*
 * CPU restatement of SPHAdjoint's forward + hand-written adjoint WCSPH step.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the parity oracle: the tests, the
 * smoke check and the bench's CPU-baseline leg call it to check (or time
 * beside) the CUDA library. The product never links or calls it.
 *
 * It is included twice by sph_oracle.c, once with R = double (suffix _f64)
 * and once with R = float (suffix _f32), exactly as the reference is generic
 * over T = Float64 / Float32.
 *
 * Arithmetic follows the reference kernels operation by operation (same
 * association, same constants, IEEE sqrt and division, no FMA: build with
 * -ffp-contract=off). Particle-parallel loops use OpenMP; each particle's
 * sums are sequential, so results do not depend on the thread count. The one
 * scatter (dJ/dtheta) runs serially in particle order.
 *
 * Array layouts are the reference's: X, V, a are (2, N) column-major, i.e.
 * interleaved (x0, y0, x1, y1, ...); theta is (ngy, ngx) column-major;
 * `order` holds 1-based particle ids, `starts` 0-based exclusive offsets.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

typedef struct {
    R h, m, rho0, c, mu, gx, gy, dt, Lx, Ly, kw;
    int ngx, ngy;
    int eos, gamma, visc;
    R alpha;
} FN(OP);

typedef struct {
    int64_t N;
    R *X, *V, *a, *rho, *pterm, *invrho, *alpha;
    /* cell list (src/neighbors.jl:9-19) */
    int32_t *cellof, *counts, *cum, *starts, *cursor, *order;
    int nx, ny;
    double cs;
    /* neighbour list, particle-major rows (src/neighbors.jl:150-162) */
    int32_t *indices, *nbcount;
    int32_t flags[2];
    R *Xref;
    int maxnb;
    double rc, dmax, skin;
    int interval;
    int64_t age;
} FN(OState);

typedef struct {
    int64_t N, cap, n;
    R *X, *V; /* (2, N, cap) */
} FN(OTape);

typedef struct {
    int64_t N;
    int ngx, ngy;
    R *gX, *gV, *gXs, *gVs, *abar, *grho, *galpha, *gtheta;
} FN(OWork);

/* ---- parameter conversion: SPHParams{T} holds every field as T ------------ */
static FN(OP) FN(to_params)(const orc_params *pp)
{
    FN(OP) p;
    p.h = (R)pp->h; p.m = (R)pp->m; p.rho0 = (R)pp->rho0; p.c = (R)pp->c;
    p.mu = (R)pp->mu; p.gx = (R)pp->gx; p.gy = (R)pp->gy; p.dt = (R)pp->dt;
    p.Lx = (R)pp->Lx; p.Ly = (R)pp->Ly; p.kw = (R)pp->kw;
    p.ngx = pp->ngx; p.ngy = pp->ngy;
    p.eos = pp->eos; p.gamma = pp->gamma; p.visc = pp->visc; p.alpha = (R)pp->alpha;
    return p;
}

/* ---- model variants (no counterpart in the reference) --------------------
   Tait: p = B ((rho/rho0)^gamma - 1), B = c^2 rho0 / gamma. With
   delta = (rho - rho0) / rho0 the bracket is s_gamma of s_1 = delta,
   s_{k+1} = s_k (1 + delta) + delta (no cancellation near rho0);
   dp/drho = (B gamma / rho0) (rho/rho0)^(gamma-1), the power a left fold.
   Monaghan viscosity on a pair with s = (v_i - v_j).d < 0:
   a_i += K d, K = m alpha c h s F / ((r^2 + 0.01 h^2) (rho_i + rho_j)/2). */
static inline R FN(pow_fold)(R x, int k)
{
    R y = (R)1;
    for (int t = 0; t < k; ++t) y = y * x;
    return y;
}

static inline R FN(pow1m)(R delta, int k)
{
    R s = delta;
    const R x = (R)1 + delta;
    for (int t = 1; t < k; ++t) s = s * x + delta;
    return s;
}

/* ---- src/kernels.jl:15-44 ------------------------------------------------- */
/* wnorm(h) = T(7) / (T(4) * T(pi) * h^2) */
static R FN(wnorm)(R h) { return (R)7 / ((R)4 * (R)M_PI * (h * h)); }

/* w_kern: A * u2 * u2 * (2q + 1), u = 1 - q/2 */
R FN(orc_w_kern)(R q, R A)
{
    if (q < (R)2) {
        R u = (R)1 - q / (R)2;
        R u2 = u * u;
        return A * u2 * u2 * ((R)2 * q + (R)1);
    }
    return (R)0;
}

/* f_kern: -5 * A * u^3 / h^2 */
R FN(orc_f_kern)(R q, R A, R h)
{
    if (q < (R)2) {
        R u = (R)1 - q / (R)2;
        return (R)(-5) * A * (u * u * u) / (h * h);
    }
    return (R)0;
}

/* g_kern: T(7.5) * A * u^2 / h^2 */
R FN(orc_g_kern)(R q, R A, R h)
{
    if (q < (R)2) {
        R u = (R)1 - q / (R)2;
        return (R)7.5 * A * (u * u) / (h * h);
    }
    return (R)0;
}

/* ---- src/params.jl:36-46 -------------------------------------------------- */
static inline R FN(wall_accel)(R x, R L, R kw)
{
    R lo = (-x > (R)0) ? -x : (R)0;        /* max(zero(T), -x) */
    R hi = (x - L > (R)0) ? x - L : (R)0;  /* max(zero(T), x - L) */
    return kw * (lo * lo - hi * hi);
}

static inline R FN(wall_daccel)(R x, R L, R kw)
{
    R lo = (-x > (R)0) ? -x : (R)0;
    R hi = (x - L > (R)0) ? x - L : (R)0;
    return kw * ((R)(-2) * lo - (R)2 * hi);
}

/* ---- src/params.jl:54-82 ------------------------------------------------- */
static inline R FN(clampR)(R x, R lo, R hi)
{
    /* Base.clamp: ifelse(x > hi, hi, ifelse(x < lo, lo, x)) */
    return x > hi ? hi : (x < lo ? lo : x);
}

static inline void FN(interp_cell)(R x, R y, const FN(OP) *p,
                                   int *i1, int *j1, R *fx, R *fy, R *ax, R *ay)
{
    R hx = p->Lx / (R)(p->ngx - 1);
    R hy = p->Ly / (R)(p->ngy - 1);
    R gx = x / hx;
    R gy = y / hy;
    *ax = ((gx > (R)0) & (gx < (R)(p->ngx - 1))) ? (R)1 : (R)0;
    *ay = ((gy > (R)0) & (gy < (R)(p->ngy - 1))) ? (R)1 : (R)0;
    R gxc = FN(clampR)(gx, (R)0, (R)(p->ngx - 1) - (R)1e-6);
    R gyc = FN(clampR)(gy, (R)0, (R)(p->ngy - 1) - (R)1e-6);
    /* gxc is finite and in [0, ngx-1) unless x is NaN; guard the conversion */
    R fgx = FLOOR(gxc), fgy = FLOOR(gyc);
    long i0 = (fgx == fgx) ? (long)fgx : 0;
    long j0 = (fgy == fgy) ? (long)fgy : 0;
    if (i0 < 0) i0 = 0;
    if (i0 > p->ngx - 2) i0 = p->ngx - 2;
    if (j0 < 0) j0 = 0;
    if (j0 > p->ngy - 2) j0 = p->ngy - 2;
    *fx = gxc - (R)i0;
    *fy = gyc - (R)j0;
    *i1 = (int)i0 + 1;
    *j1 = (int)j0 + 1;
}

/* theta is (ngy, ngx) column-major; theta[j, i] (1-based) */
#define TH(th, p, j, i) ((th)[((j) - 1) + (int64_t)((i) - 1) * (p)->ngy])

static inline void FN(interp_alpha)(const R *theta, R x, R y, const FN(OP) *p,
                                    R *a, R *dadx, R *dady)
{
    int i, j;
    R fx, fy, ax, ay;
    FN(interp_cell)(x, y, p, &i, &j, &fx, &fy, &ax, &ay);
    R t00 = TH(theta, p, j, i);
    R t01 = TH(theta, p, j, i + 1);
    R t10 = TH(theta, p, j + 1, i);
    R t11 = TH(theta, p, j + 1, i + 1);
    *a = ((R)1 - fx) * ((R)1 - fy) * t00 + fx * ((R)1 - fy) * t01 +
         ((R)1 - fx) * fy * t10 + fx * fy * t11;
    R hx = p->Lx / (R)(p->ngx - 1);
    R hy = p->Ly / (R)(p->ngy - 1);
    *dadx = (((R)1 - fy) * (t01 - t00) + fy * (t11 - t10)) / hx * ax;
    *dady = (((R)1 - fx) * (t10 - t00) + fx * (t11 - t01)) / hy * ay;
}

/* ---- cell list: src/neighbors.jl:28-114 ----------------------------------- */
static inline int32_t FN(cell_coord)(R v, int n)
{
    /* clamp(unsafe_trunc(Int, floor(v)) + 2, 1, n); the float clamp only keeps
       the conversion defined and does not change any finite result */
    R f = FLOOR(v);
    if (!(f > (R)(-4))) f = (R)(-4);
    if (f > (R)(n + 4)) f = (R)(n + 4);
    long c = (long)f + 2;
    if (c < 1) c = 1;
    if (c > n) c = n;
    return (int32_t)c;
}

static inline int32_t FN(cell_index)(R x, R y, R cs, int nx, int ny)
{
    int32_t cx = FN(cell_coord)(x / cs, nx);
    int32_t cy = FN(cell_coord)(y / cs, ny);
    return cx + (cy - 1) * nx;
}

void FN(orc_build_cells)(FN(OState) *st)
{
    const int64_t N = st->N;
    const int64_t ncell = (int64_t)st->nx * st->ny;
    const R cs = (R)st->cs;
    for (int64_t c = 0; c < ncell; ++c) st->counts[c] = 0;
    /* _cl_assign! */
    for (int64_t i = 0; i < N; ++i) {
        int32_t c = FN(cell_index)(st->X[2 * i], st->X[2 * i + 1], cs, st->nx, st->ny);
        st->cellof[i] = c;
        st->counts[c - 1] += 1;
    }
    /* cumsum!, starts = cum - counts, cursor = starts */
    int32_t acc = 0;
    for (int64_t c = 0; c < ncell; ++c) {
        acc += st->counts[c];
        st->cum[c] = acc;
        st->starts[c] = st->cum[c] - st->counts[c];
        st->cursor[c] = st->starts[c];
    }
    /* _cl_fill!: the atomic returns the new value = 1-based slot */
    for (int64_t i = 0; i < N; ++i) {
        int32_t c = st->cellof[i];
        int32_t pos = ++st->cursor[c - 1];
        st->order[pos - 1] = (int32_t)(i + 1);
    }
    /* _cl_sort_cells!: per-cell insertion sort by particle id */
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < ncell; ++c) {
        int32_t s = st->starts[c], n = st->counts[c];
        int32_t *o = st->order + s; /* o[k-1] == order[s+k] */
        for (int32_t k = 2; k <= n; ++k) {
            int32_t v = o[k - 1];
            int32_t j = k - 1;
            while (j >= 1 && o[j - 1] > v) {
                o[j] = o[j - 1];
                j -= 1;
            }
            o[j] = v;
        }
    }
}

/* ---- neighbour list: src/neighbors.jl:192-279 ----------------------------- */
void FN(orc_build_neighbors)(FN(OState) *st, R h)
{
    const int64_t N = st->N;
    FN(orc_build_cells)(st);
    int check = st->age != INT64_MAX;
    const R rc2 = (R)(st->rc * st->rc);
    const R r2min = EPS_R * h * h;
    const R cs = (R)st->cs;
    const R invcs = (R)1 / cs;
    const R dmax2 = (R)(st->dmax * st->dmax);
    const int nx = st->nx, ny = st->ny, mx = st->maxnb;
    int32_t f_over = 0, f_disp = 0;
#pragma omp parallel for schedule(static) reduction(| : f_over, f_disp)
    for (int64_t i = 0; i < N; ++i) {
        R xi = st->X[2 * i], yi = st->X[2 * i + 1];
        if (check) {
            R ddx = xi - st->Xref[2 * i];
            R ddy = yi - st->Xref[2 * i + 1];
            if (ddx * ddx + ddy * ddy > dmax2) f_disp = 1;
        }
        st->Xref[2 * i] = xi;
        st->Xref[2 * i + 1] = yi;
        int32_t cx = FN(cell_coord)(xi * invcs, nx);
        int32_t cy = FN(cell_coord)(yi * invcs, ny);
        int32_t m = 0;
        int32_t *row = st->indices + i * (int64_t)mx;
        for (int ddy = -1; ddy <= 1; ++ddy)
            for (int ddx = -1; ddx <= 1; ++ddx) {
                int32_t jx = cx + ddx, jy = cy + ddy;
                if (1 <= jx && jx <= nx && 1 <= jy && jy <= ny) {
                    int32_t c = jx + (jy - 1) * nx;
                    int32_t s = st->starts[c - 1], n = st->counts[c - 1];
                    for (int32_t k = 1; k <= n; ++k) {
                        int32_t j = st->order[s + k - 1];
                        R dx = xi - st->X[2 * (j - 1)];
                        R dy = yi - st->X[2 * (j - 1) + 1];
                        R r2 = dx * dx + dy * dy;
                        if (r2min < r2 && r2 < rc2) {
                            if (m < mx) {
                                row[m] = j;
                                m += 1;
                            } else {
                                f_over = 1;
                            }
                        }
                    }
                }
            }
        st->nbcount[i] = m;
    }
    if (f_over) st->flags[0] = 1;
    if (f_disp) st->flags[1] = 1;
    st->age = 0;
}

static void FN(maybe_rebuild)(FN(OState) *st, R h)
{
    if (st->age >= st->interval) FN(orc_build_neighbors)(st, h);
    st->age += 1;
}

/* ---- forward: src/forward.jl:25-147 --------------------------------------- */
void FN(orc_density)(FN(OState) *st, const FN(OP) *p)
{
    const int64_t N = st->N;
    const R h = p->h, mass = p->m;
    const R A = FN(wnorm)(h);
    const R invh = (R)1 / h;
    const R r2max = (R)4 * h * h;
    const int mx = st->maxnb;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        R xi = st->X[2 * i], yi = st->X[2 * i + 1];
        R acc = (R)0;
        const int32_t *row = st->indices + i * (int64_t)mx;
        for (int32_t m = 0; m < st->nbcount[i]; ++m) {
            int64_t j = row[m] - 1;
            R dx = xi - st->X[2 * j];
            R dy = yi - st->X[2 * j + 1];
            R r2 = dx * dx + dy * dy;
            if (r2 < r2max) {
                R q = SQRT(r2) * invh;
                R u = (R)1 - (R)0.5 * q;
                R u2 = u * u;
                acc += mass * (A * u2 * u2 * ((R)2 * q + (R)1));
            }
        }
        st->rho[i] = acc + mass * A;
    }
}

void FN(orc_eos)(FN(OState) *st, const FN(OP) *p)
{
    const R c2 = p->c * p->c;
    const R rho0 = p->rho0;
    const R B = c2 * rho0 / (R)p->gamma;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < st->N; ++i) {
        R ri = st->rho[i];
        R inv = (R)1 / ri;
        st->invrho[i] = inv;
        if (p->eos == 1)
            st->pterm[i] = B * FN(pow1m)((ri - rho0) / rho0, p->gamma) * inv * inv;
        else
            st->pterm[i] = c2 * (ri - rho0) * inv * inv;
    }
}

/* explicit != 0 restates the older explicit-drag integrator of
   tools/verify_adjoint.py:187-192,286-295 (a_i -= alpha_i v_i); the reference
   kernels use the implicit form. */
void FN(orc_accel)(FN(OState) *st, const R *theta, const FN(OP) *p, int explicit_drag)
{
    const int64_t N = st->N;
    const R h = p->h, mass = p->m;
    const R A = FN(wnorm)(h);
    const R invh = (R)1 / h;
    const R r2max = (R)4 * h * h;
    const R Fc = (R)(-5) * A * invh * invh;
    const R twomumass = (R)2 * mass * p->mu;
    const R avc = mass * p->alpha * p->c * h;
    const R eh2 = (R)0.01 * h * h;
    const int mx = st->maxnb;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        R xi = st->X[2 * i], yi = st->X[2 * i + 1];
        R vxi = st->V[2 * i], vyi = st->V[2 * i + 1];
        R pti = st->pterm[i];
        R iri = st->invrho[i];
        R rhoi = st->rho[i];
        R ax = (R)0, ay = (R)0;
        const int32_t *row = st->indices + i * (int64_t)mx;
        for (int32_t m = 0; m < st->nbcount[i]; ++m) {
            int64_t j = row[m] - 1;
            R dx = xi - st->X[2 * j];
            R dy = yi - st->X[2 * j + 1];
            R r2 = dx * dx + dy * dy;
            if (r2 < r2max) {
                R q = SQRT(r2) * invh;
                R u = (R)1 - (R)0.5 * q;
                R F = Fc * u * u * u;
                R Pij = mass * (pti + st->pterm[j]);
                ax -= Pij * F * dx;
                ay -= Pij * F * dy;
                if (p->visc == 1) {
                    R wx = vxi - st->V[2 * j];
                    R wy = vyi - st->V[2 * j + 1];
                    R s = wx * dx + wy * dy;
                    R K = (R)0;
                    if (s < (R)0) {
                        R D = r2 + eh2;
                        R rb = (rhoi + st->rho[j]) * (R)0.5;
                        K = avc * s * F / (D * rb);
                    }
                    ax += K * dx;
                    ay += K * dy;
                } else {
                    R C = twomumass * iri * st->invrho[j] * F;
                    ax += C * (vxi - st->V[2 * j]);
                    ay += C * (vyi - st->V[2 * j + 1]);
                }
            }
        }
        R al, d1, d2;
        FN(interp_alpha)(theta, xi, yi, p, &al, &d1, &d2);
        st->alpha[i] = al;
        ax += p->gx + FN(wall_accel)(xi, p->Lx, p->kw);
        ay += p->gy + FN(wall_accel)(yi, p->Ly, p->kw);
        if (explicit_drag) {
            ax -= al * vxi;
            ay -= al * vyi;
        }
        st->a[2 * i] = ax;
        st->a[2 * i + 1] = ay;
    }
}

void FN(orc_integrate)(FN(OState) *st, R dt, int explicit_drag)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < st->N; ++i) {
        R D = explicit_drag ? (R)1 : (R)1 / ((R)1 + dt * st->alpha[i]);
        R v1 = (st->V[2 * i] + dt * st->a[2 * i]) * D;
        R v2 = (st->V[2 * i + 1] + dt * st->a[2 * i + 1]) * D;
        st->V[2 * i] = v1;
        st->V[2 * i + 1] = v2;
        st->X[2 * i] += dt * v1;
        st->X[2 * i + 1] += dt * v2;
    }
}

/* step!: src/forward.jl:161-173 */
void FN(orc_step)(FN(OState) *st, const R *theta, const orc_params *pp, int explicit_drag)
{
    FN(OP) p = FN(to_params)(pp);
    FN(maybe_rebuild)(st, p.h);
    FN(orc_density)(st, &p);
    FN(orc_eos)(st, &p);
    FN(orc_accel)(st, theta, &p, explicit_drag);
    FN(orc_integrate)(st, p.dt, explicit_drag);
}

/* ---- state / tape / workspace objects (src/driver.jl:24-133) -------------- */
FN(OState) *FN(orc_state_new)(const orc_params *pp, int64_t N, const double *X0,
                             const double *V0, double skin, int interval, int maxnb)
{
    FN(OP) p = FN(to_params)(pp);
    FN(OState) *st = (FN(OState) *)calloc(1, sizeof(FN(OState)));
    st->N = N;
    st->X = (R *)malloc(sizeof(R) * 2 * (N ? N : 1));
    st->V = (R *)malloc(sizeof(R) * 2 * (N ? N : 1));
    st->a = (R *)calloc(2 * (N ? N : 1), sizeof(R));
    st->rho = (R *)calloc(N ? N : 1, sizeof(R));
    st->pterm = (R *)calloc(N ? N : 1, sizeof(R));
    st->invrho = (R *)calloc(N ? N : 1, sizeof(R));
    st->alpha = (R *)calloc(N ? N : 1, sizeof(R));
    for (int64_t k = 0; k < 2 * N; ++k) {
        st->X[k] = (R)X0[k];
        st->V[k] = (R)V0[k];
    }
    /* NeighborList: rc = Float64(support(p)) * (1 + skin), dmax = Float64(h)*skin */
    R support = (R)2 * p.h;
    st->skin = skin;
    st->rc = (double)support * (1.0 + skin);
    st->dmax = (double)p.h * skin;
    st->interval = interval;
    st->maxnb = maxnb;
    st->age = INT64_MAX;
    st->indices = (int32_t *)calloc((size_t)(N ? N : 1) * maxnb, sizeof(int32_t));
    st->nbcount = (int32_t *)calloc(N ? N : 1, sizeof(int32_t));
    st->Xref = (R *)calloc(2 * (N ? N : 1), sizeof(R));
    /* CellList(backend, N, p; cs = nl.rc) */
    st->cs = st->rc;
    st->nx = (int)ceil((double)p.Lx / st->cs) + 2;
    st->ny = (int)ceil((double)p.Ly / st->cs) + 2;
    if (st->nx < 1) st->nx = 1;
    if (st->ny < 1) st->ny = 1;
    int64_t ncell = (int64_t)st->nx * st->ny;
    st->cellof = (int32_t *)calloc(N ? N : 1, sizeof(int32_t));
    st->order = (int32_t *)calloc(N ? N : 1, sizeof(int32_t));
    st->counts = (int32_t *)calloc(ncell, sizeof(int32_t));
    st->cum = (int32_t *)calloc(ncell, sizeof(int32_t));
    st->starts = (int32_t *)calloc(ncell, sizeof(int32_t));
    st->cursor = (int32_t *)calloc(ncell, sizeof(int32_t));
    return st;
}

void FN(orc_state_free)(FN(OState) *st)
{
    if (!st) return;
    free(st->X); free(st->V); free(st->a); free(st->rho); free(st->pterm);
    free(st->invrho); free(st->alpha); free(st->indices); free(st->nbcount);
    free(st->Xref); free(st->cellof); free(st->order); free(st->counts);
    free(st->cum); free(st->starts); free(st->cursor);
    free(st);
}

FN(OTape) *FN(orc_tape_new)(int64_t N, int64_t cap)
{
    FN(OTape) *tp = (FN(OTape) *)calloc(1, sizeof(FN(OTape)));
    tp->N = N;
    tp->cap = cap;
    tp->n = 0;
    tp->X = (R *)malloc(sizeof(R) * 2 * (size_t)(N ? N : 1) * (cap ? cap : 1));
    tp->V = (R *)malloc(sizeof(R) * 2 * (size_t)(N ? N : 1) * (cap ? cap : 1));
    return tp;
}

void FN(orc_tape_free)(FN(OTape) *tp)
{
    if (!tp) return;
    free(tp->X); free(tp->V); free(tp);
}

FN(OWork) *FN(orc_work_new)(int64_t N, int ngx, int ngy)
{
    FN(OWork) *ws = (FN(OWork) *)calloc(1, sizeof(FN(OWork)));
    int64_t n2 = 2 * (N ? N : 1), n1 = N ? N : 1;
    ws->N = N; ws->ngx = ngx; ws->ngy = ngy;
    ws->gX = (R *)calloc(n2, sizeof(R)); ws->gV = (R *)calloc(n2, sizeof(R));
    ws->gXs = (R *)calloc(n2, sizeof(R)); ws->gVs = (R *)calloc(n2, sizeof(R));
    ws->abar = (R *)calloc(n2, sizeof(R));
    ws->grho = (R *)calloc(n1, sizeof(R)); ws->galpha = (R *)calloc(n1, sizeof(R));
    ws->gtheta = (R *)calloc((size_t)ngx * ngy, sizeof(R));
    return ws;
}

void FN(orc_work_free)(FN(OWork) *ws)
{
    if (!ws) return;
    free(ws->gX); free(ws->gV); free(ws->gXs); free(ws->gVs); free(ws->abar);
    free(ws->grho); free(ws->galpha); free(ws->gtheta); free(ws);
}

/* flags are read and cleared at the API boundary (check_neighbor_flags) */
int32_t FN(orc_take_flags)(FN(OState) *st)
{
    int32_t f = (st->flags[0] ? 1 : 0) | (st->flags[1] ? 2 : 0);
    st->flags[0] = st->flags[1] = 0;
    return f;
}

/* simulate!: src/driver.jl:92-115. Returns -1 on tape overflow (ArgumentError),
   else the neighbour-list flags (bit0 overflow, bit1 displacement). */
int32_t FN(orc_simulate)(FN(OState) *st, const R *theta, const orc_params *pp,
                         int64_t nsteps, FN(OTape) *tape, int explicit_drag)
{
    const int64_t N = st->N;
    if (tape && tape->n + nsteps > tape->cap) return -1;
    for (int64_t s = 0; s < nsteps; ++s) {
        if (tape) {
            tape->n += 1;
            R *tx = tape->X + 2 * N * (tape->n - 1);
            R *tv = tape->V + 2 * N * (tape->n - 1);
            memcpy(tx, st->X, sizeof(R) * 2 * N);
            memcpy(tv, st->V, sizeof(R) * 2 * N);
        }
        FN(orc_step)(st, theta, pp, explicit_drag);
    }
    return FN(orc_take_flags)(st);
}

/* ---- adjoint: src/adjoint.jl:30-228 ---------------------------------------- */
static void FN(adj_pass1)(FN(OWork) *ws, const FN(OState) *st, const R *theta,
                          const FN(OP) *p, int explicit_drag)
{
    const int64_t N = st->N;
    const R h = p->h, mass = p->m;
    const R A = FN(wnorm)(h);
    const R c2 = p->c * p->c;
    const R invh = (R)1 / h;
    const R r2max = (R)4 * h * h;
    const R Fc = (R)(-5) * A * invh * invh;
    const R Gc = (R)7.5 * A * invh * invh;
    const R twomumass = (R)2 * mass * p->mu;
    const R avc = mass * p->alpha * p->c * h;
    const R eh2 = (R)0.01 * h * h;
    const R dB = c2 * p->rho0 / (R)p->gamma * (R)p->gamma / p->rho0;
    const int mx = st->maxnb;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        R xi = st->X[2 * i], yi = st->X[2 * i + 1];
        R vxi = st->V[2 * i], vyi = st->V[2 * i + 1];
        R abx = ws->abar[2 * i], aby = ws->abar[2 * i + 1];
        R pti = st->pterm[i];
        R iri = st->invrho[i];
        R rhoi = st->rho[i];
        R gx = 0, gy = 0, gvx = 0, gvy = 0, grh = 0, sumS = 0;
        const int32_t *row = st->indices + i * (int64_t)mx;
        for (int32_t m = 0; m < st->nbcount[i]; ++m) {
            int64_t j = row[m] - 1;
            R dx = xi - st->X[2 * j];
            R dy = yi - st->X[2 * j + 1];
            R r2 = dx * dx + dy * dy;
            if (r2 < r2max) {
                R r = SQRT(r2);
                R q = r * invh;
                R u = (R)1 - (R)0.5 * q;
                R F = Fc * u * u * u;
                R G = Gc * u * u;
                R Pij = mass * (pti + st->pterm[j]);
                R Cbase = twomumass * iri * st->invrho[j];
                R C = Cbase * F;
                R dax = abx - ws->abar[2 * j];
                R day = aby - ws->abar[2 * j + 1];
                R dvx = vxi - st->V[2 * j];
                R dvy = vyi - st->V[2 * j + 1];
                R ad_d = -(dax * dx + day * dy);
                R ad_v = dax * dvx + day * dvy;
                gx -= Pij * F * dax;
                gy -= Pij * F * day;
                if (p->visc == 1) {
                    /* d/d(d, v, rho) of (abar_i - abar_j).(K d) */
                    R s = dvx * dx + dvy * dy;
                    R Fbar = Pij * ad_d;
                    R w = Fbar * G * invh / r;
                    R Ad = dax * dx + day * dy;
                    R avx = (R)0, avy = (R)0, vx = (R)0, vy = (R)0, rs = (R)0;
                    if (s < (R)0) {
                        R D = r2 + eh2;
                        R rb = (rhoi + st->rho[j]) * (R)0.5;
                        R Drb = D * rb;
                        R K = avc * s * F / Drb;
                        R Ks = avc * F / Drb;
                        R KF = avc * s / Drb;
                        R cd = Ad * (KF * G * invh / r - (R)2 * K / D);
                        avx = K * dax + Ad * Ks * dvx + cd * dx;
                        avy = K * day + Ad * Ks * dvy + cd * dy;
                        vx = Ad * Ks * dx;
                        vy = Ad * Ks * dy;
                        rs = Ad * K / ((R)2 * rb);
                    }
                    gx += w * dx + avx;
                    gy += w * dy + avy;
                    gvx += vx;
                    gvy += vy;
                    grh -= rs;
                    sumS += F * ad_d;
                } else {
                    R Fbar = Pij * ad_d + Cbase * ad_v;
                    R w = Fbar * G * invh / r;
                    gx += w * dx;
                    gy += w * dy;
                    gvx += C * dax;
                    gvy += C * day;
                    grh -= C * ad_v * iri;
                    sumS += F * ad_d;
                }
            }
        }
        grh += ((R)(-2) * mass * pti * iri) * sumS;
        if (p->eos == 1)
            grh += dB * FN(pow_fold)(rhoi / p->rho0, p->gamma - 1) * mass * iri * iri * sumS;
        else
            grh += c2 * mass * iri * iri * sumS;
        if (explicit_drag) {
            /* tools/verify_gather.py:87-90 */
            R al = st->alpha[i];
            gvx -= al * abx;
            gvy -= al * aby;
            ws->galpha[i] = -(abx * vxi + aby * vyi);
        }
        gx += abx * FN(wall_daccel)(xi, p->Lx, p->kw);
        gy += aby * FN(wall_daccel)(yi, p->Ly, p->kw);
        ws->gXs[2 * i] = gx;
        ws->gXs[2 * i + 1] = gy;
        ws->gVs[2 * i] = gvx;
        ws->gVs[2 * i + 1] = gvy;
        ws->grho[i] = grh;
    }
}

static void FN(adj_pass2)(FN(OWork) *ws, const FN(OState) *st, const FN(OP) *p)
{
    const int64_t N = st->N;
    const R h = p->h, mass = p->m;
    const R A = FN(wnorm)(h);
    const R invh = (R)1 / h;
    const R r2max = (R)4 * h * h;
    const R Fc = (R)(-5) * A * invh * invh;
    const int mx = st->maxnb;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        R xi = st->X[2 * i], yi = st->X[2 * i + 1];
        R gri = ws->grho[i];
        R gx = 0, gy = 0;
        const int32_t *row = st->indices + i * (int64_t)mx;
        for (int32_t m = 0; m < st->nbcount[i]; ++m) {
            int64_t j = row[m] - 1;
            R dx = xi - st->X[2 * j];
            R dy = yi - st->X[2 * j + 1];
            R r2 = dx * dx + dy * dy;
            if (r2 < r2max) {
                R q = SQRT(r2) * invh;
                R u = (R)1 - (R)0.5 * q;
                R w = mass * (Fc * u * u * u) * (gri + ws->grho[j]);
                gx += w * dx;
                gy += w * dy;
            }
        }
        ws->gXs[2 * i] += gx;
        ws->gXs[2 * i + 1] += gy;
    }
}

/* adj_design_kernel!: the theta scatter runs serially in particle order */
static void FN(adj_design)(FN(OWork) *ws, const FN(OState) *st, const R *theta,
                           const FN(OP) *p)
{
    const int64_t N = st->N;
    const int ny = p->ngy;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        R al, dadx, dady;
        FN(interp_alpha)(theta, st->X[2 * i], st->X[2 * i + 1], p, &al, &dadx, &dady);
        R ga = ws->galpha[i];
        ws->gXs[2 * i] += ga * dadx;
        ws->gXs[2 * i + 1] += ga * dady;
    }
    for (int64_t i = 0; i < N; ++i) {
        int ii, jj;
        R fx, fy, ax, ay;
        FN(interp_cell)(st->X[2 * i], st->X[2 * i + 1], p, &ii, &jj, &fx, &fy, &ax, &ay);
        R ga = ws->galpha[i];
        int64_t l00 = jj + (int64_t)(ii - 1) * ny; /* 1-based linear, column-major */
        ws->gtheta[l00 - 1] += ga * ((R)1 - fx) * ((R)1 - fy);
        ws->gtheta[l00 + ny - 1] += ga * fx * ((R)1 - fy);
        ws->gtheta[l00] += ga * ((R)1 - fx) * fy;
        ws->gtheta[l00 + ny] += ga * fx * fy;
    }
}

/* _adj_drag!: src/adjoint.jl:214-228 */
static void FN(adj_drag)(FN(OWork) *ws, const FN(OState) *st, R dt)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < st->N; ++i) {
        R D = (R)1 / ((R)1 + dt * st->alpha[i]);
        R vx = (st->V[2 * i] + dt * st->a[2 * i]) * D;
        R vy = (st->V[2 * i + 1] + dt * st->a[2 * i + 1]) * D;
        R gx = ws->gV[2 * i];
        R gy = ws->gV[2 * i + 1];
        ws->abar[2 * i] = dt * D * gx;
        ws->abar[2 * i + 1] = dt * D * gy;
        ws->galpha[i] = -dt * D * (vx * gx + vy * gy);
        ws->gV[2 * i] = D * gx;
        ws->gV[2 * i + 1] = D * gy;
    }
}

/* backward!: src/driver.jl:141-207. `scratch` may be NULL (a fresh one is made
   with the given neighbour-list knobs, like the reference). Returns the
   scratch state's neighbour-list flags. */
int32_t FN(orc_backward)(FN(OWork) *ws, const FN(OTape) *tape, const R *theta,
                         const orc_params *pp, const double *seedX, const double *seedV,
                         FN(OState) *scratch, double skin, int interval, int maxnb,
                         int explicit_drag)
{
    FN(OP) p = FN(to_params)(pp);
    const int64_t N = ws->N;
    for (int64_t k = 0; k < 2 * N; ++k) {
        ws->gX[k] = (R)seedX[k];
        ws->gV[k] = (R)seedV[k];
    }
    for (int64_t k = 0; k < (int64_t)p.ngx * p.ngy; ++k) ws->gtheta[k] = (R)0;
    int own = 0;
    if (!scratch) {
        double *z = (double *)calloc(2 * (N ? N : 1), sizeof(double));
        scratch = FN(orc_state_new)(pp, N, z, z, skin, interval, maxnb);
        free(z);
        own = 1;
    }
    for (int64_t n = tape->n; n >= 1; --n) {
        memcpy(scratch->X, tape->X + 2 * N * (n - 1), sizeof(R) * 2 * N);
        memcpy(scratch->V, tape->V + 2 * N * (n - 1), sizeof(R) * 2 * N);
        FN(maybe_rebuild)(scratch, p.h);
        FN(orc_density)(scratch, &p);
        FN(orc_eos)(scratch, &p);
        FN(orc_accel)(scratch, theta, &p, explicit_drag);
        /* _adj_integrate!: gV += dt * gX */
        for (int64_t k = 0; k < 2 * N; ++k) ws->gV[k] += p.dt * ws->gX[k];
        if (explicit_drag) {
            /* tools/verify_gather.py:145-146: abar = dt * gV' */
            for (int64_t k = 0; k < 2 * N; ++k) ws->abar[k] = p.dt * ws->gV[k];
        } else {
            FN(adj_drag)(ws, scratch, p.dt);
        }
        FN(adj_pass1)(ws, scratch, theta, &p, explicit_drag);
        FN(adj_design)(ws, scratch, theta, &p);
        FN(adj_pass2)(ws, scratch, &p);
        for (int64_t k = 0; k < 2 * N; ++k) {
            ws->gX[k] += ws->gXs[k];
            ws->gV[k] += ws->gVs[k];
        }
    }
    int32_t f = FN(orc_take_flags)(scratch);
    if (own) FN(orc_state_free)(scratch);
    return f;
}

/* ---- accessors for the ctypes wrapper ------------------------------------- */
void FN(orc_state_get)(const FN(OState) *st, double *X, double *V)
{
    for (int64_t k = 0; k < 2 * st->N; ++k) {
        if (X) X[k] = (double)st->X[k];
        if (V) V[k] = (double)st->V[k];
    }
}

void FN(orc_state_set)(FN(OState) *st, const double *X, const double *V)
{
    for (int64_t k = 0; k < 2 * st->N; ++k) {
        if (X) st->X[k] = (R)X[k];
        if (V) st->V[k] = (R)V[k];
    }
}

void FN(orc_state_fields)(const FN(OState) *st, double *rho, double *pterm, double *invrho,
                          double *a, double *alpha)
{
    for (int64_t i = 0; i < st->N; ++i) {
        if (rho) rho[i] = (double)st->rho[i];
        if (pterm) pterm[i] = (double)st->pterm[i];
        if (invrho) invrho[i] = (double)st->invrho[i];
        if (alpha) alpha[i] = (double)st->alpha[i];
        if (a) {
            a[2 * i] = (double)st->a[2 * i];
            a[2 * i + 1] = (double)st->a[2 * i + 1];
        }
    }
}

void FN(orc_state_grid)(const FN(OState) *st, int32_t *nx, int32_t *ny, double *cs,
                        int64_t *age)
{
    *nx = st->nx;
    *ny = st->ny;
    *cs = st->cs;
    *age = st->age;
}

void FN(orc_state_cells)(const FN(OState) *st, int32_t *counts, int32_t *starts,
                         int32_t *order, int32_t *cellof)
{
    int64_t ncell = (int64_t)st->nx * st->ny;
    if (counts) memcpy(counts, st->counts, sizeof(int32_t) * ncell);
    if (starts) memcpy(starts, st->starts, sizeof(int32_t) * ncell);
    if (order) memcpy(order, st->order, sizeof(int32_t) * st->N);
    if (cellof) memcpy(cellof, st->cellof, sizeof(int32_t) * st->N);
}

void FN(orc_state_neighbors)(const FN(OState) *st, int32_t *indices, int32_t *nbcount)
{
    if (indices) memcpy(indices, st->indices, sizeof(int32_t) * st->N * st->maxnb);
    if (nbcount) memcpy(nbcount, st->nbcount, sizeof(int32_t) * st->N);
}

void FN(orc_work_get)(const FN(OWork) *ws, double *gX, double *gV, double *gtheta)
{
    for (int64_t k = 0; k < 2 * ws->N; ++k) {
        if (gX) gX[k] = (double)ws->gX[k];
        if (gV) gV[k] = (double)ws->gV[k];
    }
    if (gtheta)
        for (int64_t k = 0; k < (int64_t)ws->ngx * ws->ngy; ++k) gtheta[k] = (double)ws->gtheta[k];
}

void FN(orc_tape_get)(const FN(OTape) *tp, int64_t n, double *X, double *V)
{
    /* n is 1-based like the reference's tape slices */
    const R *tx = tp->X + 2 * tp->N * (n - 1);
    const R *tv = tp->V + 2 * tp->N * (n - 1);
    for (int64_t k = 0; k < 2 * tp->N; ++k) {
        if (X) X[k] = (double)tx[k];
        if (V) V[k] = (double)tv[k];
    }
}

int64_t FN(orc_tape_length)(const FN(OTape) *tp) { return tp->n; }
void FN(orc_tape_reset)(FN(OTape) *tp) { tp->n = 0; }

/* The reference computes arrays of T internally; theta arrives from the
   caller as doubles and is converted once per call, like copyto!(th, theta). */
R *FN(orc_theta_new)(const double *theta, int ngx, int ngy)
{
    R *t = (R *)malloc(sizeof(R) * (size_t)ngx * ngy);
    for (int64_t k = 0; k < (int64_t)ngx * ngy; ++k) t[k] = (R)theta[k];
    return t;
}

void FN(orc_theta_free)(R *t) { free(t); }
