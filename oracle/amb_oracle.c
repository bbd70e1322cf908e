/*
 * ORACLE — test infrastructure, not the product.
 *
 * Plain-C CPU restatement of the reference's Active Model B+ explicit-Euler
 * step (tranqui/active-model-bplus, src/integrator.cu), used only by tests/,
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as the
 * checker. The CUDA library never links or calls it.
 *
 * Pinned against the reference itself: tests/test_oracle.py compares every
 * term and the one-step update with the reference's own CPU scheme
 * (test/tjhung_ambplus.h, compiled into oracle/_ref by oracle/build.py) at
 * 1e-12, and tests/golden/ holds fixtures made by that compiled reference.
 *
 * Layout: row-major (nrows = ny, ncols = nx), index = col + row * ncols
 * (src/integrator.cu:59); axis 0 = y (rows), axis 1 = x (cols); periodic wrap.
 *
 * Term by term (one site, field phi):
 *   lap   = dxInv^2 tj_xx(phi) + dyInv^2 tj_yy(phi)        src/finite_difference.cuh:179-183
 *   gy,gx = dyInv tj_y(phi), dxInv tj_x(phi)                src/finite_difference.cuh:166-176
 *   mu_p  = a phi + b phi^2 + c phi^3 - kappa lap           src/integrator.cu:34-37,99-100
 *   mu_a  = lambda (gy^2 + gx^2)                            src/integrator.cu:101
 *   J_c   = zeta lap (gy, gx)                               src/integrator.cu:103-104
 *   J_r   = sqrt(2T) sqrt(1/(dt dx dy)) (xi_y, xi_x)        src/integrator.cu:106-109, src/parameters.h:43-51,79-87
 *   J_p   = -(dyInv D8_y mu_p, dxInv D8_x mu_p)             src/integrator.cu:171-172
 *   J_l   = -(tj_y mu_a, tj_x mu_a) (scaled)                src/integrator.cu:174-175
 *   divJ  = tj_y(J_ly+J_cy) + tj_x(J_lx+J_cx)
 *         + D8_y(J_py+J_ry) + D8_x(J_px+J_rx)              src/integrator.cu:203-204,259-260
 *   phi  -= dt divJ                                         src/integrator.cu:261
 * with D8 the order-8 central first derivative (src/finite_difference.h:69-75)
 * and tj_* the Tjhung 3x3 stencils (src/finite_difference.h:379-453).
 * Stencil sums accumulate tap by tap in the reference's order
 * (src/finite_difference.h:218-236, 414-428).
 *
 * Noise (no counterpart in the reference, which seeds curand XORWOW
 * non-deterministically, src/integrator.cu:275-282,320-323): standard normals
 * xi keyed on (seed, step, site, component) by Philox4x32-10 (Salmon, Moraes,
 * Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11) and
 * Box-Muller. The definition is restated in orc_noise_normal() below (in
 * double precision); the CUDA kernels evaluate the same definition in single
 * precision, within 5e-5 of it.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_NTERMS 10
#define ORC_PI 3.14159265358979323846

/* Order-8 central first-derivative taps, offsets -4..4 (src/finite_difference.h:73). */
static const double D8[9] = {1. / 280, -4. / 105, 1. / 5, -4. / 5, 0, 4. / 5, -1. / 5, 4. / 105, -1. / 280};

/* Tjhung 3x3 taps indexed [row offset + 1][col offset + 1] (src/finite_difference.h:381-398). */
static const double TJ_FIRST_X[3][3] = {{-1. / 10, 0, 1. / 10}, {-3. / 10, 0, 3. / 10}, {-1. / 10, 0, 1. / 10}};
static const double TJ_SECOND_X[3][3] = {{-0.25, 0.5, -0.25}, {1.50, -3.0, 1.50}, {-0.25, 0.5, -0.25}};

static inline int wrap(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

/* Periodic index tables: rows[k] = wrap(k - PAD, ny) * nx, cols[k] = wrap(k - PAD, nx),
 * so tap offsets up to +-PAD need no modulo in the inner loops. */
#define ORC_PAD 9
typedef struct
{
    int ny, nx;
    size_t* rows;
    int* cols;
} orc_grid;

static int grid_init(orc_grid* g, int ny, int nx)
{
    g->ny = ny;
    g->nx = nx;
    g->rows = (size_t*)malloc(sizeof(size_t) * (ny + 2 * ORC_PAD));
    g->cols = (int*)malloc(sizeof(int) * (nx + 2 * ORC_PAD));
    if (!g->rows || !g->cols) return 1;
    for (int k = 0; k < ny + 2 * ORC_PAD; ++k) g->rows[k] = (size_t)wrap(k - ORC_PAD, ny) * nx;
    for (int k = 0; k < nx + 2 * ORC_PAD; ++k) g->cols[k] = wrap(k - ORC_PAD, nx);
    return 0;
}

static void grid_free(orc_grid* g)
{
    free(g->rows);
    free(g->cols);
}

#define ROW(g, r) ((g)->rows[(r) + ORC_PAD])
#define COL(g, c) ((g)->cols[(c) + ORC_PAD])

/* Apply a 3x3 Tjhung stencil; transpose=1 gives the y operator (src/finite_difference.h:404-412). */
static inline double tj_apply(const double* f, const orc_grid* g, int r, int c, const double w[3][3], int transpose)
{
    double acc = 0;
    for (int di = 0; di < 3; ++di)
        for (int dj = 0; dj < 3; ++dj)
        {
            double coef = transpose ? w[dj][di] : w[di][dj];
            acc += coef * f[COL(g, c + dj - 1) + ROW(g, r + di - 1)];
        }
    return acc;
}

static inline double d8_x(const double* f, const orc_grid* g, int r, int c)
{
    double acc = 0;
    for (int k = 0; k < 9; ++k) acc += D8[k] * f[COL(g, c + k - 4) + ROW(g, r)];
    return acc;
}

static inline double d8_y(const double* f, const orc_grid* g, int r, int c)
{
    double acc = 0;
    for (int k = 0; k < 9; ++k) acc += D8[k] * f[c + ROW(g, r + k - 4)];
    return acc;
}

/* ---------------------------------------------------------------- Philox */

/* Philox4x32-10 (Salmon et al. SC'11): 10 rounds of the 4x32 S-box with the
 * published multipliers and Weyl key increments. */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round)
    {
        uint64_t p0 = (uint64_t)M0 * c0;
        uint64_t p1 = (uint64_t)M1 * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += W0; k1 += W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* The noise definition shared with the CUDA kernels.
 *   counter = (col >> 2, row, step mod 2^32, (step >> 32) << 1 | comp), key = (seed lo, seed hi)
 *   x0..x3  = Philox4x32-10(counter, key)
 *   u_a = ((x_{2p} >> 8) + 1) 2^-24 in (0, 1],  u_b = (x_{2p+1} >> 8) 2^-24 in [0, 1)
 *   r = sqrt(-2 ln u_a), theta = 2 pi (u_b - 1/2)
 *   z_{2p} = r cos theta, z_{2p+1} = r sin theta   (p = 0, 1)
 *   xi(site, comp) = z[col & 3]
 * comp 0 = y component, 1 = x component. */
void orc_noise_bits(uint64_t seed, int64_t step, int row, int col, int comp, uint32_t out[4])
{
    uint32_t ctr[4] = {(uint32_t)col >> 2, (uint32_t)row, (uint32_t)(uint64_t)step,
                       (uint32_t)(((uint64_t)step >> 32) << 1) | (uint32_t)comp};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    orc_philox4x32_10(ctr, key, out);
}

double orc_noise_normal(uint64_t seed, int64_t step, int row, int col, int comp)
{
    uint32_t x[4];
    orc_noise_bits(seed, step, row, col, comp, x);
    int lane = col & 3, pair = lane >> 1;
    double ua = ((double)(x[2 * pair] >> 8) + 1.0) * (1.0 / 16777216.0);
    double ub = (double)(x[2 * pair + 1] >> 8) * (1.0 / 16777216.0);
    double r = sqrt(-2.0 * log(ua));
    double theta = 2.0 * ORC_PI * (ub - 0.5);
    return (lane & 1) ? r * sin(theta) : r * cos(theta);
}

void orc_normals(int ny, int nx, uint64_t seed, int64_t step, double* xi_y, double* xi_x)
{
#pragma omp parallel for schedule(static)
    for (int r = 0; r < ny; ++r)
        for (int c = 0; c < nx; ++c)
        {
            xi_y[c + (size_t)r * nx] = orc_noise_normal(seed, step, r, c, 0);
            xi_x[c + (size_t)r * nx] = orc_noise_normal(seed, step, r, c, 1);
        }
}

/* ---------------------------------------------------------------- terms */

/* params = {dt, dx, dy, a, b, c, kappa, lambda, zeta, temperature}
 * (src/parameters.h:23-25 HostStencilParams, :54-61 ActiveModelBPlusParams). */
typedef struct
{
    double dt, dx, dy, a, b, c, kappa, lambda, zeta, temperature;
} orc_params;

/* Every term of the reference's calculate_forces + calculate_local_currents
 * (src/integrator.cu:46-110, 112-176) at `phi`. out holds 10 planes of ny*nx:
 * mu_p, mu_a, J_p(y,x), J_l(y,x), J_c(y,x), J_r(y,x). xi_y/xi_x are standard
 * normals (or NULL for zero noise). Returns 0, or 1 on bad sizes. */
int orc_terms(int ny, int nx, const double* phi, const orc_params* p, const double* xi_y, const double* xi_x,
              double* out, int nthreads)
{
    if (ny < 1 || nx < 1) return 1;
    const size_t n = (size_t)ny * nx;
    const double dxInv = 1 / p->dx, dyInv = 1 / p->dy;
    const double mag = sqrt(2 * p->temperature) * sqrt(1. / (p->dt * p->dx * p->dy));
    double *mu_p = out, *mu_a = out + n, *jp_y = out + 2 * n, *jp_x = out + 3 * n;
    double *jl_y = out + 4 * n, *jl_x = out + 5 * n, *jc_y = out + 6 * n, *jc_x = out + 7 * n;
    double *jr_y = out + 8 * n, *jr_x = out + 9 * n;
    orc_grid g;
    if (grid_init(&g, ny, nx)) { grid_free(&g); return 2; }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif

#pragma omp parallel for schedule(static)
    for (int r = 0; r < ny; ++r)
        for (int c = 0; c < nx; ++c)
        {
            size_t i = c + (size_t)r * nx;
            double f = phi[i];
            double lap = dxInv * dxInv * tj_apply(phi, &g, r, c, TJ_SECOND_X, 0)
                       + dyInv * dyInv * tj_apply(phi, &g, r, c, TJ_SECOND_X, 1);
            double gy = dyInv * tj_apply(phi, &g, r, c, TJ_FIRST_X, 1);
            double gx = dxInv * tj_apply(phi, &g, r, c, TJ_FIRST_X, 0);
            mu_p[i] = (p->a * f + p->b * f * f + p->c * f * f * f) - p->kappa * lap;
            mu_a[i] = p->lambda * (gy * gy + gx * gx);
            jc_y[i] = p->zeta * lap * gy;
            jc_x[i] = p->zeta * lap * gx;
            jr_y[i] = xi_y ? mag * xi_y[i] : 0.0;
            jr_x[i] = xi_x ? mag * xi_x[i] : 0.0;
        }

#pragma omp parallel for schedule(static)
    for (int r = 0; r < ny; ++r)
        for (int c = 0; c < nx; ++c)
        {
            size_t i = c + (size_t)r * nx;
            jp_y[i] = -(dyInv * d8_y(mu_p, &g, r, c));
            jp_x[i] = -(dxInv * d8_x(mu_p, &g, r, c));
            jl_y[i] = -(dyInv * tj_apply(mu_a, &g, r, c, TJ_FIRST_X, 1));
            jl_x[i] = -(dxInv * tj_apply(mu_a, &g, r, c, TJ_FIRST_X, 0));
        }
    grid_free(&g);
    return 0;
}

/* divJ of the reference's step kernel (src/integrator.cu:199-260) from the
 * 10 planes of orc_terms; `work` holds 4 planes of scratch. */
int orc_divergence(int ny, int nx, const double* terms, const orc_params* p, double* divj, double* work, int nthreads)
{
    if (ny < 1 || nx < 1) return 1;
    const size_t n = (size_t)ny * nx;
    const double dxInv = 1 / p->dx, dyInv = 1 / p->dy;
    const double *jp_y = terms + 2 * n, *jp_x = terms + 3 * n, *jl_y = terms + 4 * n, *jl_x = terms + 5 * n;
    const double *jc_y = terms + 6 * n, *jc_x = terms + 7 * n, *jr_y = terms + 8 * n, *jr_x = terms + 9 * n;
    double *j1y = work, *j1x = work + n, *j2y = work + 2 * n, *j2x = work + 3 * n;
    orc_grid g;
    if (grid_init(&g, ny, nx)) { grid_free(&g); return 2; }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(static)
    for (int r = 0; r < ny; ++r)
        for (int c = 0; c < nx; ++c)
        {
            size_t i = c + (size_t)r * nx;
            j1y[i] = jp_y[i] + jr_y[i];
            j1x[i] = jp_x[i] + jr_x[i];
            j2y[i] = jl_y[i] + jc_y[i];
            j2x[i] = jl_x[i] + jc_x[i];
        }
#pragma omp parallel for schedule(static)
    for (int r = 0; r < ny; ++r)
        for (int c = 0; c < nx; ++c)
        {
            size_t i = c + (size_t)r * nx;
            divj[i] = dyInv * tj_apply(j2y, &g, r, c, TJ_FIRST_X, 1)
                    + dxInv * tj_apply(j2x, &g, r, c, TJ_FIRST_X, 0)
                    + dyInv * d8_y(j1y, &g, r, c)
                    + dxInv * d8_x(j1x, &g, r, c);
        }
    grid_free(&g);
    return 0;
}

/* Run `nsteps` explicit-Euler steps on phi in place, as the reference's
 * Integrator::run (src/integrator.cu:497-518): the currents used by the update
 * from step s to s+1 are evaluated at step s, with noise drawn for step s.
 * noise_mode: 0 = none (xi = 0), 1 = Philox (seed, step), 2 = injected
 * (`injected` holds nsteps x 2 planes: xi_y then xi_x per step).
 * Returns 0, 1 on bad arguments, 2 on allocation failure. */
int orc_run(int ny, int nx, double* phi, const orc_params* p, int64_t step0, int nsteps, int noise_mode,
            uint64_t seed, const double* injected, int nthreads)
{
    if (ny < 1 || nx < 1 || nsteps < 0 || noise_mode < 0 || noise_mode > 2) return 1;
    if (noise_mode == 2 && !injected) return 1;
    const size_t n = (size_t)ny * nx;
    double* terms = (double*)malloc(sizeof(double) * n * (ORC_NTERMS + 4 + 1 + 2));
    if (!terms) return 2;
    double* work = terms + ORC_NTERMS * n;
    double* divj = work + 4 * n;
    double* xi = divj + n;
    for (int s = 0; s < nsteps; ++s)
    {
        const double *xy = NULL, *xx = NULL;
        if (noise_mode == 1 && p->temperature != 0)
        {
            orc_normals(ny, nx, seed, step0 + s, xi, xi + n);
            xy = xi; xx = xi + n;
        }
        else if (noise_mode == 2)
        {
            xy = injected + (size_t)s * 2 * n;
            xx = xy + n;
        }
        orc_terms(ny, nx, phi, p, xy, xx, terms, nthreads);
        orc_divergence(ny, nx, terms, p, divj, work, nthreads);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; ++i) phi[i] -= p->dt * divj[i];
    }
    free(terms);
    return 0;
}

/* Float-storage counterpart used as the CPU reference for the FP32 kernels'
 * precision study: same update, field rounded to float after every step. */
int orc_run_f32(int ny, int nx, float* phi, const orc_params* p, int64_t step0, int nsteps, int noise_mode,
                uint64_t seed, int nthreads)
{
    const size_t n = (size_t)ny * nx;
    double* buf = (double*)malloc(sizeof(double) * n);
    if (!buf) return 2;
    int rc = 0;
    for (int s = 0; s < nsteps && rc == 0; ++s)
    {
        for (size_t i = 0; i < n; ++i) buf[i] = phi[i];
        rc = orc_run(ny, nx, buf, p, step0 + s, 1, noise_mode, seed, NULL, nthreads);
        for (size_t i = 0; i < n; ++i) phi[i] = (float)buf[i];
    }
    free(buf);
    return rc;
}

/* Sum of a float64 field with Kahan-Babuska (Neumaier) compensation: the
 * mass used for the conservation checks. */
double orc_sum(const double* f, long n)
{
    double s = 0, comp = 0;
    for (long i = 0; i < n; ++i)
    {
        double t = s + f[i];
        if (fabs(s) >= fabs(f[i])) comp += (s - t) + f[i];
        else comp += (f[i] - t) + s;
        s = t;
    }
    return s + comp;
}
