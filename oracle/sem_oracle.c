/*
 * sem_oracle.c -- CPU restatement of the reference SEM acoustic step (test infrastructure only;
 * see sem_oracle.h).  Compile with -ffp-contract=off: the float variant must round exactly where
 * the reference rounds.
 */
#include "sem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------------ */
/* mesh indexing                                                                                */
/* ------------------------------------------------------------------------------------------ */

void or_box_counts(int ex, int ey, int ez, int order,
                   int64_t *n_nodes, int64_t *n_elem, int64_t *n_interior)
{
    /* SEMmesh.cpp:28-54 (3-D branch) */
    int64_t nx = (int64_t)ex * order + 1, ny = (int64_t)ey * order + 1, nz = (int64_t)ez * order + 1;
    if (n_nodes) *n_nodes = nx * ny * nz;
    if (n_elem) *n_elem = (int64_t)ex * ey * ez;
    if (n_interior) *n_interior = (nx - 2) * (ny - 2) * (nz - 2);
}

void or_connectivity(int ex, int ey, int ez, int order, int32_t *conn)
{
    /* SEMmesh.cpp:205-231: element e = i + k*ex + j*ex*ez; local l + n(o+1) + m(o+1)^2;
     * global = offset + l + n*nx + m*nx*nz with offset = i*o + k*o*nx + j*o*nx*nz. */
    const int64_t nx = (int64_t)ex * order + 1, nz = (int64_t)ez * order + 1;
    const int o1 = order + 1, npe = o1 * o1 * o1;
    for (int j = 0; j < ey; j++)
        for (int k = 0; k < ez; k++)
            for (int i = 0; i < ex; i++) {
                int64_t e = i + (int64_t)k * ex + (int64_t)j * ex * ez;
                int64_t offset = (int64_t)i * order + (int64_t)k * order * nx + (int64_t)j * order * nx * nz;
                for (int m = 0; m < o1; m++)
                    for (int n = 0; n < o1; n++)
                        for (int l = 0; l < o1; l++)
                            conn[e * npe + l + n * o1 + m * o1 * o1] =
                                (int32_t)(offset + l + n * nx + m * nx * nz);
            }
}

void or_interior_nodes(int ex, int ey, int ez, int order, int32_t *list)
{
    /* SEMmesh.cpp:314-344 (3-D branch) */
    const int64_t nx = (int64_t)ex * order + 1, ny = (int64_t)ey * order + 1, nz = (int64_t)ez * order + 1;
    int64_t m = 0;
    for (int64_t k = 1; k < ny - 1; k++)
        for (int64_t j = 1; j < nz - 1; j++)
            for (int64_t i = 1; i < nx - 1; i++)
                list[m++] = (int32_t)(i + j * nx + k * nx * nz);
}

int64_t or_element_from_point(int ex, int ey, int ez, float lx, float ly, float lz,
                              float x, float y, float z)
{
    /* SEMmesh.cpp:266-285; hx = lx/(1.*ex) stored as float (SEMmesh.cpp:20-22). */
    float hx = (float)(lx / (1. * ex)), hy = (float)(ly / (1. * ey)), hz = (float)(lz / (1. * ez));
    int eX = 0, eY = 0, eZ = 0;
    for (int i = 0; i < ex; i++)
        if (x >= i * hx && x < (i + 1) * hx) eX = i;
    for (int i = 0; i < ey; i++)
        if (y >= i * hy && y < (i + 1) * hy) eY = i;
    for (int i = 0; i < ez; i++)
        if (z >= i * hz && z < (i + 1) * hz) eZ = i;
    return eX + (int64_t)eZ * ex + (int64_t)eY * ex * ez;
}

static int64_t nearest_axis(int ne, double len, int order, const double *xi, double c)
{
    const double h = len / ne;
    if (c <= 0.0) return 0;
    if (c >= len) return (int64_t)ne * order;
    int64_t e = (int64_t)floor(c / h);
    if (e >= ne) e = ne - 1;
    int64_t best = e * order;
    double bd = INFINITY;
    for (int l = 0; l <= order; l++) {
        double cl = e * h + (1.0 + xi[l]) * 0.5 * h;
        double d = fabs(cl - c);
        if (d < bd) { bd = d; best = e * order + l; }
    }
    return best;
}

int64_t or_nearest_node(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                        float x, float y, float z)
{
    double xi[8], w[8], dp[64];
    or_gll_tables(order, xi, w, dp);
    int64_t nx = (int64_t)ex * order + 1, nz = (int64_t)ez * order + 1;
    int64_t ix = nearest_axis(ex, lx, order, xi, x);
    int64_t iy = nearest_axis(ey, ly, order, xi, y);
    int64_t iz = nearest_axis(ez, lz, order, xi, z);
    return ix + iz * nx + iy * nx * nz;
}

/* float GLL points exactly as getCoordInOneDirection stores them (SEMmesh.cpp:85-126). */
static void ref_xi_float(int order, float *xi)
{
    switch (order) {
    case 1: xi[0] = -1.f; xi[1] = 1.f; break;
    case 2: xi[0] = -1.f; xi[1] = 0.f; xi[2] = 1.f; break;
    case 3: {
        const double s5 = sqrt(5.0);
        xi[0] = -1.f; xi[1] = (float)(-1. / s5); xi[2] = (float)(1. / s5); xi[3] = 1.f;
    } break;
    case 4: {
        const double s = sqrt(3.0 / 7.0);
        xi[0] = -1.f; xi[1] = (float)-s; xi[2] = 0.f; xi[3] = (float)s; xi[4] = 1.f;
    } break;
    case 5: {
        const double a = sqrt((7.0 + 2.0 * sqrt(7.0)) / 21.0), b = sqrt((7.0 - 2.0 * sqrt(7.0)) / 21.0);
        xi[0] = -1.f; xi[1] = (float)-a; xi[2] = (float)-b; xi[3] = (float)b; xi[4] = (float)a; xi[5] = 1.f;
    } break;
    default: break;
    }
}

/* getCoordInOneDirection (SEMmesh.cpp:81-139): h arrives as an int. */
static void coord_1d(int order, int h, int e, const float *xi, float *coord)
{
    float x0 = (float)(e * h);
    float x1 = (float)((e + 1) * h);
    float b = (float)((x1 + x0) / 2.);
    float a = b - x0;
    for (int j = 0; j < order + 1; j++) coord[j] = a * xi[j] + b;
}

void or_element_coords(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                       float *X, float *Z, float *Y)
{
    /* SEMmesh.cpp:168-202 */
    float hx = (float)(lx / (1. * ex)), hy = (float)(ly / (1. * ey)), hz = (float)(lz / (1. * ez));
    int ihx = (int)hx, ihy = (int)hy, ihz = (int)hz;
    const int o1 = order + 1, npe = o1 * o1 * o1;
    float xi[8], cx[8], cy[8], cz[8];
    ref_xi_float(order, xi);
    for (int n = 0; n < ey; n++) {
        coord_1d(order, ihy, n, xi, cy);
        for (int m = 0; m < ez; m++) {
            coord_1d(order, ihz, m, xi, cz);
            for (int l = 0; l < ex; l++) {
                coord_1d(order, ihx, l, xi, cx);
                int64_t e = l + (int64_t)m * ex + (int64_t)n * ex * ez;
                for (int k = 0; k < o1; k++)
                    for (int j = 0; j < o1; j++)
                        for (int i = 0; i < o1; i++) {
                            int64_t q = e * npe + i + o1 * j + k * o1 * o1;
                            X[q] = cx[i];
                            Z[q] = cz[j];
                            Y[q] = cy[k];
                        }
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* GLL tables: own derivation (Legendre recurrence + Newton), checked against the reference's  */
/* literals in tests.                                                                           */
/* ------------------------------------------------------------------------------------------ */

static void legendre(int n, double x, double *p, double *dp)
{
    double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
    if (n == 0) { *p = 1.0; *dp = 0.0; return; }
    for (int k = 2; k <= n; k++) {
        double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        double d2 = d0 + (2.0 * k - 1.0) * p1;
        p0 = p1; p1 = p2; d0 = d1; d1 = d2;
    }
    *p = p1; *dp = d1;
}

int or_gll_tables(int order, double *xi, double *w, double *dphi)
{
    if (order < 1 || order > 7) return -1;
    const int N = order, n1 = order + 1;
    /* interior points: roots of P_N', Newton from Chebyshev-Lobatto guesses */
    xi[0] = -1.0; xi[N] = 1.0;
    for (int i = 1; i < N; i++) {
        double x = -cos(M_PI * i / N);
        for (int it = 0; it < 100; it++) {
            /* f = P_N'(x); f' = P_N''(x) = (2x P_N' - N(N+1) P_N)/(1-x^2) */
            double p, dp;
            legendre(N, x, &p, &dp);
            double ddp = (2.0 * x * dp - N * (N + 1.0) * p) / (1.0 - x * x);
            double dx = dp / ddp;
            x -= dx;
            if (fabs(dx) < 1e-17) break;
        }
        xi[i] = x;
    }
    /* symmetrise (the reference's points are exactly antisymmetric) */
    for (int i = 0; i < n1 / 2; i++) {
        double a = 0.5 * (xi[N - i] - xi[i]);
        xi[i] = -a; xi[N - i] = a;
    }
    if (n1 % 2) xi[N / 2] = 0.0;
    double PN[8];
    for (int i = 0; i < n1; i++) {
        double p, dp;
        legendre(N, xi[i], &p, &dp);
        PN[i] = p;
        double wi = 2.0 / (N * (N + 1.0) * p * p);
        /* the reference tabulates weights to 8 decimals (SEMQkGLBasisFunctions.hpp:80-117) */
        w[i] = nearbyint(wi * 1e8) / 1e8;
    }
    for (int j = 0; j < n1; j++)
        for (int i = 0; i < n1; i++) {
            double d;
            if (i != j) d = PN[i] / (PN[j] * (xi[i] - xi[j]));
            else if (i == 0) d = -N * (N + 1.0) / 4.0;
            else if (i == N) d = N * (N + 1.0) / 4.0;
            else d = 0.0;
            dphi[j * n1 + i] = d;
        }
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Ricker wavelet (utils.hpp:11-57)                                                              */
/* ------------------------------------------------------------------------------------------ */

float or_ricker(float time_n, float f0, int order)
{
    float o_tpeak = (float)(1.0 / f0);
    float pulse = 0.0f;
    if ((time_n <= -0.9 * o_tpeak) || (time_n >= 2.9 * o_tpeak)) return pulse;
    const float pi = (float)M_PI;
    float lam = (f0 * pi) * (f0 * pi);
    float dtp = time_n - o_tpeak;
    switch (order) {
    case 2:
        pulse = (float)(2.0 * lam * (2.0 * lam * dtp * dtp - 1.0) * expf(-lam * dtp * dtp));
        break;
    case 1:
        pulse = (float)(-2.0 * lam * dtp * expf(-lam * dtp * dtp));
        break;
    case 0:
        pulse = (float)(-dtp * expf(-2 * lam * dtp * dtp));
        break;
    default:
        break;
    }
    return pulse;
}

void or_source_term(int n, float dt, float f0, int order, float *out)
{
    for (int i = 0; i < n; i++) {
        float t = i * dt;
        out[i] = or_ricker(t, f0, order);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* sponge profile (build definition, see header)                                                */
/* ------------------------------------------------------------------------------------------ */

static void sponge_axis(int ne, float len, int order, int thickness, double sigma,
                        const double *xi, float *s, double *sd)
{
    const double h = (double)len / ne;
    const int64_t n = (int64_t)ne * order + 1;
    for (int64_t i = 0; i < n; i++) {
        int64_t e = i / order;
        int l = (int)(i - e * order);
        if (e == ne) { e = ne - 1; l = order; }
        double c = e * h + (1.0 + xi[l]) * 0.5 * h;
        double d = fmin(c, len - c) / h;
        double v = 1.0;
        if (thickness > 0 && d < thickness) {
            double r = (thickness - d) / thickness;
            v = exp(-sigma * r * r);
        }
        if (s) s[i] = (float)v;
        if (sd) sd[i] = v;
    }
}

void or_sponge_profile(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                       int thickness, float sigma,
                       float *sx, float *sy, float *sz,
                       double *sxd, double *syd, double *szd)
{
    double xi[8], w[8], dphi[64];
    or_gll_tables(order, xi, w, dphi);
    sponge_axis(ex, lx, order, thickness, sigma, xi, sx, sxd);
    sponge_axis(ey, ly, order, thickness, sigma, xi, sy, syd);
    sponge_axis(ez, lz, order, thickness, sigma, xi, sz, szd);
}

/* ------------------------------------------------------------------------------------------ */
/* time stepping: instantiated for float and double                                             */
/* ------------------------------------------------------------------------------------------ */

#define REAL float
#define SFX(n) n##_f32
#include "sem_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX(n) n##_f64
#include "sem_oracle_impl.h"
#undef REAL
#undef SFX
