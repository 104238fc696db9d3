// host_util.cpp -- GLL tables, Ricker wavelet, box indexing and sponge profile (host side).
#include "host_util.h"

#include <cmath>

namespace semgb {

namespace {

// Legendre P_n and its derivative by the three-term recurrence.
void legendre(int n, double x, double &p, double &dp)
{
    double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
    if (n == 0) { p = 1.0; dp = 0.0; return; }
    for (int k = 2; k <= n; k++) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        const double d2 = d0 + (2.0 * k - 1.0) * p1;
        p0 = p1; p1 = p2; d0 = d1; d1 = d2;
    }
    p = p1; dp = d1;
}

}  // namespace

bool gll_tables(int order, Gll &g)
{
    if (order < kMinOrder || order > kMaxOrder) return false;
    const int N = order, n1 = order + 1;
    g.order = order;
    g.xi[0] = -1.0;
    g.xi[N] = 1.0;
    // interior points: Newton on P_N'(x), with P_N'' from the Legendre equation
    for (int i = 1; i < N; i++) {
        double x = -std::cos(M_PI * i / N);
        for (int it = 0; it < 100; it++) {
            double p, dp;
            legendre(N, x, p, dp);
            const double ddp = (2.0 * x * dp - N * (N + 1.0) * p) / (1.0 - x * x);
            const double dx = dp / ddp;
            x -= dx;
            if (std::fabs(dx) < 1e-17) break;
        }
        g.xi[i] = x;
    }
    for (int i = 0; i < n1 / 2; i++) {  // exact antisymmetry
        const double a = 0.5 * (g.xi[N - i] - g.xi[i]);
        g.xi[i] = -a;
        g.xi[N - i] = a;
    }
    if (n1 % 2) g.xi[N / 2] = 0.0;
    double PN[kMaxOrder + 1];
    for (int i = 0; i < n1; i++) {
        double p, dp;
        legendre(N, g.xi[i], p, dp);
        PN[i] = p;
        // the reference tabulates the weights to 8 decimals (SEMQkGLBasisFunctions.hpp:80-117)
        g.w[i] = std::nearbyint(2.0 / (N * (N + 1.0) * p * p) * 1e8) / 1e8;
    }
    for (int j = 0; j < n1; j++)
        for (int i = 0; i < n1; i++) {
            double d;
            if (i != j) d = PN[i] / (PN[j] * (g.xi[i] - g.xi[j]));
            else if (i == 0) d = -N * (N + 1.0) / 4.0;
            else if (i == N) d = N * (N + 1.0) / 4.0;
            else d = 0.0;
            g.dphi[j * n1 + i] = d;
        }
    return true;
}

void stencil_table(const Gll &g, float *T)
{
    const int o = g.order, o1 = o + 1, W = 2 * o + 1;
    double A[kMaxOrder + 1][kMaxOrder + 1];  // A(i, j) = sum_q w_q phi_i'(xi_q) phi_j'(xi_q)
    for (int i = 0; i < o1; i++)
        for (int j = 0; j < o1; j++) {
            double s = 0;
            for (int q = 0; q < o1; q++) s += g.w[q] * g.dphi[i * o1 + q] * g.dphi[j * o1 + q];
            A[i][j] = s;
        }
    for (int l = 0; l < o; l++)
        for (int d = -o; d <= o; d++) {
            double v = 0;
            if (l == 0) {
                if (d >= 0) v += A[0][d];       // element to the right (local 0)
                if (d <= 0) v += A[o][o + d];   // element to the left (local o)
            } else if (l + d >= 0 && l + d <= o) {
                v = A[l][l + d];
            }
            T[l * W + d + o] = (float)v;
        }
}

void element_stiffness_1d(const Gll &g, float (&S)[kMaxOrder + 1][kMaxOrder + 1])
{
    const int o1 = g.order + 1;
    for (int i = 0; i <= kMaxOrder; i++)
        for (int j = 0; j <= kMaxOrder; j++) {
            double s = 0;
            if (i < o1 && j < o1)
                for (int q = 0; q < o1; q++) s += g.w[q] * g.dphi[i * o1 + q] * g.dphi[j * o1 + q];
            S[i][j] = (float)s;
        }
}

void reference_element_rows(const Gll &g, double jx, double jz, double jy, std::vector<float> &rows)
{
    const int o = g.order, o1 = o + 1, op2 = o1 * o1, npe = op2 * o1;
    const double *w = g.w;
    auto D = [&](int a, int b) { return g.dphi[a * o1 + b]; };  // phi_a'(xi_b)
    // computeB (SEMQkGLIntegrals.hpp:316-349) with jac = diag(jx, jz, jy): the cofactors off the
    // diagonal vanish, detJ = |jx (jz jy)|, B_dd = adj_dd^2 / detJ; the same at every GLL point
    const double detJ = std::fabs(jx * (jz * jy));
    const double a00 = jz * jy, a11 = jx * jy, a22 = jx * jz;
    const double dm1 = 1. / detJ;
    const float B[3] = {(float)((a00 * a00) * dm1), (float)((a11 * a11) * dm1), (float)((a22 * a22) * dm1)};
    rows.assign((size_t)3 * npe * o1, 0.f);
    std::vector<float> R(npe);
    // gradPhiGradPhi (SEMQkGLIntegrals.hpp:427-513): the three line families in the reference's
    // order; the cross families add exact zeros here
    for (int i3 = 0; i3 < o1; i3++)
        for (int i2 = 0; i2 < o1; i2++)
            for (int i1 = 0; i1 < o1; i1++) {
                std::fill(R.begin(), R.end(), 0.f);
                for (int j1 = 0; j1 < o1; j1++) {
                    const int j = j1 + i2 * o1 + i3 * op2;
                    for (int l = 0; l < o1; l++)
                        R[j] = (float)((double)R[j] + w[l] * w[i2] * w[i3] * ((double)B[0] * D(i1, l) * D(j1, l)));
                }
                for (int j2 = 0; j2 < o1; j2++) {
                    const int j = i1 + j2 * o1 + i3 * op2;
                    for (int m = 0; m < o1; m++)
                        R[j] = (float)((double)R[j] + w[i1] * w[m] * w[i3] * ((double)B[1] * D(i2, m) * D(j2, m)));
                }
                for (int j3 = 0; j3 < o1; j3++) {
                    const int j = i1 + i2 * o1 + j3 * op2;
                    for (int n = 0; n < o1; n++)
                        R[j] = (float)((double)R[j] + w[i1] * w[i2] * w[n] * ((double)B[2] * D(i3, n) * D(j3, n)));
                }
                const int i = i1 + i2 * o1 + i3 * op2;
                for (int m = 0; m < o1; m++) {
                    rows[((size_t)0 * npe + i) * o1 + m] = R[m + i2 * o1 + i3 * op2];
                    if (m != i2) rows[((size_t)1 * npe + i) * o1 + m] = R[i1 + m * o1 + i3 * op2];
                    if (m != i3) rows[((size_t)2 * npe + i) * o1 + m] = R[i1 + i2 * o1 + m * op2];
                }
            }
}

void reference_class_table(const Gll &g, double jx, double jz, double jy, std::vector<float> &tab)
{
    const int o = g.order, o1 = o + 1, npe = o1 * o1 * o1, W = 2 * o + 1;
    std::vector<float> rows;
    reference_element_rows(g, jx, jz, jy, rows);
    tab.assign((size_t)reference_class_table_size(o), 0.f);
    // the elements holding a node of local index l along an axis: l itself, and for l = 0 also
    // the element before it, where the node has local index o
    auto members = [o](int l, int *loc) {
        loc[0] = l;
        if (l != 0) return 1;
        loc[1] = o;
        return 2;
    };
    for (int ly = 0; ly < o; ly++)
        for (int lz = 0; lz < o; lz++)
            for (int lx = 0; lx < o; lx++) {
                double acc[3][2 * kMaxOrder + 1] = {};
                int mx[2], mz[2], my[2];
                const int nx = members(lx, mx), nz = members(lz, mz), ny = members(ly, my);
                for (int a = 0; a < nx; a++)
                    for (int b = 0; b < nz; b++)
                        for (int c = 0; c < ny; c++) {
                            const int ix = mx[a], iz = mz[b], iy = my[c];
                            const int i = ix + iz * o1 + iy * o1 * o1;
                            const int own[3] = {ix, iz, iy};
                            for (int ax = 0; ax < 3; ax++)
                                for (int m = 0; m < o1; m++)
                                    acc[ax][m - own[ax] + o] += rows[((size_t)ax * npe + i) * o1 + m];
                        }
                for (int ax = 0; ax < 3; ax++)
                    for (int d = -o; d <= o; d++)
                        tab[((((size_t)ax * o + ly) * o + lz) * W + d + o) * o + lx] = (float)acc[ax][d + o];
            }
}

float ricker(float time_n, float f0, int order)
{
    // float/double mix of utils.hpp:11-46, kept so the samples match the reference bit for bit
    const float o_tpeak = (float)(1.0 / f0);
    float pulse = 0.0f;
    if ((time_n <= -0.9 * o_tpeak) || (time_n >= 2.9 * o_tpeak)) return pulse;
    const float pi = (float)M_PI;
    const float lam = (f0 * pi) * (f0 * pi);
    const float d = time_n - o_tpeak;
    switch (order) {
    case 2: pulse = (float)(2.0 * lam * (2.0 * lam * d * d - 1.0) * std::exp(-lam * d * d)); break;
    case 1: pulse = (float)(-2.0 * lam * d * std::exp(-lam * d * d)); break;
    case 0: pulse = -d * std::exp(-2 * lam * d * d); break;
    default: break;
    }
    return pulse;
}

bool make_box(int ex, int ey, int ez, float lx, float ly, float lz, int order, Box &b)
{
    if (ex < 1 || ey < 1 || ez < 1 || order < kMinOrder || order > kMaxOrder) return false;
    if (!(lx > 0) || !(ly > 0) || !(lz > 0)) return false;
    b.ex = ex; b.ey = ey; b.ez = ez; b.order = order;
    b.lx = lx; b.ly = ly; b.lz = lz;
    b.nx = (int64_t)ex * order + 1;
    b.ny = (int64_t)ey * order + 1;
    b.nz = (int64_t)ez * order + 1;
    b.n_nodes = b.nx * b.ny * b.nz;
    b.n_elem = (int64_t)ex * ey * ez;
    b.n_interior = (b.nx - 2) * (b.ny - 2) * (b.nz - 2);
    b.npe = (order + 1) * (order + 1) * (order + 1);
    b.nxp = (b.nx + kRowAlign - 1) / kRowAlign * kRowAlign;
    b.n_int = b.nxp * b.nz * b.ny;
    return true;
}

int64_t box_element_from_point(const Box &b, float x, float y, float z)
{
    // element sizes are floats there (SEMmesh.cpp:20-22) and the scan keeps the last match
    const float hx = (float)(b.lx / (1. * b.ex)), hy = (float)(b.ly / (1. * b.ey)),
                hz = (float)(b.lz / (1. * b.ez));
    int eX = 0, eY = 0, eZ = 0;
    for (int i = 0; i < b.ex; i++)
        if (x >= i * hx && x < (i + 1) * hx) eX = i;
    for (int i = 0; i < b.ey; i++)
        if (y >= i * hy && y < (i + 1) * hy) eY = i;
    for (int i = 0; i < b.ez; i++)
        if (z >= i * hz && z < (i + 1) * hz) eZ = i;
    return eX + (int64_t)eZ * b.ex + (int64_t)eY * b.ex * b.ez;
}

namespace {

int64_t nearest_on_axis(int ne, double len, int order, const double *xi, double c)
{
    const double h = len / ne;
    if (c <= 0.0) return 0;
    if (c >= len) return (int64_t)ne * order;
    int64_t e = (int64_t)std::floor(c / h);
    if (e >= ne) e = ne - 1;
    int64_t best = e * order;
    double bd = INFINITY;
    for (int l = 0; l <= order; l++) {
        const double d = std::fabs(e * h + (1.0 + xi[l]) * 0.5 * h - c);
        if (d < bd) { bd = d; best = e * order + l; }
    }
    return best;
}

void sponge_axis(int ne, double len, int order, const double *xi, int thickness, double sigma,
                 std::vector<float> &s)
{
    const double h = len / ne;
    const int64_t n = (int64_t)ne * order + 1;
    s.assign(n, 1.0f);
    for (int64_t i = 0; i < n; i++) {
        int64_t e = i / order;
        int l = (int)(i - e * order);
        if (e == ne) { e = ne - 1; l = order; }
        const double c = e * h + (1.0 + xi[l]) * 0.5 * h;
        const double d = std::fmin(c, len - c) / h;
        if (thickness > 0 && d < thickness) {
            const double r = (thickness - d) / thickness;
            s[i] = (float)std::exp(-sigma * r * r);
        }
    }
}

}  // namespace

int64_t box_nearest_node(const Box &b, const Gll &g, float x, float y, float z)
{
    const int64_t ix = nearest_on_axis(b.ex, b.lx, b.order, g.xi, x);
    const int64_t iy = nearest_on_axis(b.ey, b.ly, b.order, g.xi, y);
    const int64_t iz = nearest_on_axis(b.ez, b.lz, b.order, g.xi, z);
    return ix + iz * b.nx + iy * b.nx * b.nz;
}

void box_sponge_profile(const Box &b, const Gll &g, int thickness, double sigma,
                        std::vector<float> &sx, std::vector<float> &sy, std::vector<float> &sz)
{
    sponge_axis(b.ex, b.lx, b.order, g.xi, thickness, sigma, sx);
    sponge_axis(b.ey, b.ly, b.order, g.xi, thickness, sigma, sy);
    sponge_axis(b.ez, b.lz, b.order, g.xi, thickness, sigma, sz);
}

}  // namespace semgb
