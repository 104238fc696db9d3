// host_util.h -- host-side (CPU) pieces of the SEM solver: GLL tables, Ricker wavelet, box-mesh
// indexing, sponge profile.  Used by the C ABI (api.cu) and exported through it.
#pragma once
#include <cstdint>
#include <vector>

namespace semgb {

constexpr int kMinOrder = 1;
constexpr int kMaxOrder = 5;

struct Gll {
    int order = 0;
    double xi[kMaxOrder + 1];
    double w[kMaxOrder + 1];                       // 8-decimal values, as the reference tabulates
    double dphi[(kMaxOrder + 1) * (kMaxOrder + 1)];  // dphi[j*(o+1)+i] = phi_j'(xi_i)
};

// GLL points (roots of P_N' plus the end points), weights 2/(N(N+1)P_N(xi)^2) rounded to 8
// decimals, and the Lagrange derivative table at the points.  Returns false for a bad order.
bool gll_tables(int order, Gll &g);

// Assembled 1-D stiffness coupling of the uniform-box operator: T[l*(2o+1) + d + o] couples a node
// with local index l (0..o-1) to the node d places further along the same axis (|d| <= o); zero
// outside the node's element (l > 0) or element pair (l == 0).  From A = D^T diag(w) D of one
// element, in double, rounded once.
void stencil_table(const Gll &g, float *T);

// 1-D stiffness of one element, S[i][j] = sum_q w_q phi_i'(xi_q) phi_j'(xi_q) (symmetric), in
// double, rounded once; rows and columns past the order are zero.
void element_stiffness_1d(const Gll &g, float (&S)[kMaxOrder + 1][kMaxOrder + 1]);

// The reference's element stiffness rows (computeB and gradPhiGradPhi, SEMQkGLIntegrals.hpp:265-
// 513) on an axis-aligned element with Jacobian diag(jx, jz, jy) (reference directions xi1 -> x,
// xi2 -> z, xi3 -> y), rounded where the reference rounds: the metric B computed in double and
// stored as float, every row entry accumulated in float from double products in the reference's
// loop order.  The off-diagonal metric terms are exactly zero on such an element, so the non-zero
// entries of node i's row lie on the three coordinate lines through i.
// rows[(a*npe + i)*(o+1) + m], axis a (0: x, 1: z, 2: y), element node i (local numbering
// l + n(o+1) + m(o+1)^2): the entry toward the node of local index m along a.  The diagonal is
// held whole by the x entry (m = i's own x index); the z and y entries there are zero.
void reference_element_rows(const Gll &g, double jx, double jz, double jy, std::vector<float> &rows);

// Node-class coefficients of the operator the reference assembles from those rows on a uniform
// box: for an interior node with local indices (lx, lz, ly) in 0..o-1 (0: on element faces), the
// coefficient of the node d places along axis a, summed exactly over the elements that hold both
// nodes and rounded once to float; the diagonal sits in the x entry d = 0.
// tab[(((a*o + ly)*o + lz)*(2o+1) + d + o)*o + lx].
void reference_class_table(const Gll &g, double jx, double jz, double jy, std::vector<float> &tab);
constexpr int reference_class_table_size(int o) { return 3 * o * o * (2 * o + 1) * o; }

// Ricker wavelet in the reference's float arithmetic (utils.hpp:11-46).
float ricker(float t, float f0, int order);

// Device layout: rows along x are padded to nxp = nx rounded up to 32 floats (128 bytes), so
// every row starts on a 128-byte boundary (vector accesses and TMA tiles); internal node index
// = ix + iz*nxp + iy*nxp*nz.  Padding nodes hold zero.  The ABI speaks the reference numbering.
constexpr int kRowAlign = 32;

struct Box {
    int ex = 0, ey = 0, ez = 0, order = 0;
    float lx = 0, ly = 0, lz = 0;
    int64_t nx = 0, ny = 0, nz = 0;  // nodes per axis
    int64_t n_nodes = 0, n_elem = 0, n_interior = 0;
    int npe = 0;                    // nodes per element
    int64_t nxp = 0;                // padded row length of the device layout
    int64_t n_int = 0;              // nodes in the device layout, nxp*nz*ny
};

// Reference node index -> device-layout index.
inline int64_t to_internal(const Box &b, int64_t node)
{
    const int64_t iy = node / (b.nx * b.nz), r = node - iy * b.nx * b.nz, iz = r / b.nx, ix = r - iz * b.nx;
    return ix + iz * b.nxp + iy * b.nxp * b.nz;
}

// Device-layout index -> reference node index (the index must not be a padding node).
inline int64_t to_reference(const Box &b, int64_t q)
{
    const int64_t iy = q / (b.nxp * b.nz), r = q - iy * b.nxp * b.nz, iz = r / b.nxp, ix = r - iz * b.nxp;
    return ix + iz * b.nx + iy * b.nx * b.nz;
}

bool make_box(int ex, int ey, int ez, float lx, float ly, float lz, int order, Box &b);

// Reference connectivity of element e, local index l + n(o+1) + m(o+1)^2 (SEMmesh.cpp:205-231).
inline int64_t box_node(const Box &b, int64_t e, int local)
{
    const int o = b.order, o1 = o + 1;
    const int64_t ix = e % b.ex, iz = (e / b.ex) % b.ez, iy = e / ((int64_t)b.ex * b.ez);
    const int l = local % o1, n = (local / o1) % o1, m = local / (o1 * o1);
    return (ix * o + l) + (iz * o + n) * b.nx + (iy * o + m) * b.nx * b.nz;
}

// SEMmesh::getElementNumberFromPoints semantics (SEMmesh.cpp:266-285).
int64_t box_element_from_point(const Box &b, float x, float y, float z);

// Nearest GLL node per axis, ties to the lower index, clamped to the box.
int64_t box_nearest_node(const Box &b, const Gll &g, float x, float y, float z);

// Sponge factors along each axis (see semgb.h).
void box_sponge_profile(const Box &b, const Gll &g, int thickness, double sigma,
                        std::vector<float> &sx, std::vector<float> &sy, std::vector<float> &sz);

}  // namespace semgb
