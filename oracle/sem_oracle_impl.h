/*
 * sem_oracle_impl.h -- the step of sem_oracle.c, included once per REAL type (float, double).
 * Test infrastructure only (see sem_oracle.h).  Every expression keeps the reference's operand
 * types and evaluation order; comments name the reference lines.
 */

#define MAXO1 8
#define MAXNPE (MAXO1 * MAXO1 * MAXO1)

/* SEMQkGLIntegrals.hpp:206-359 (computeB V2, 3-D branch): per GLL point, the Jacobian from the
 * element's coordinate lines in double, detJ, B = adj(J) adj(J)^T / |detJ| stored as REAL, and
 * the local mass w_i w_j w_k |detJ| stored as REAL. */
static void SFX(compute_b)(int order, const double *w, const double *dphi,
                           const REAL *X, const REAL *Y, const REAL *Z,
                           REAL *massLocal, REAL (*B)[6])
{
    const int o1 = order + 1;
#define DPHI(a, b) dphi[(a) * o1 + (b)]
    for (int i3 = 0; i3 < o1; i3++)
        for (int i2 = 0; i2 < o1; i2++)
            for (int i1 = 0; i1 < o1; i1++) {
                int i = i1 + i2 * o1 + i3 * o1 * o1;
                double jac00 = 0, jac01 = 0, jac02 = 0, jac10 = 0, jac11 = 0, jac12 = 0,
                       jac20 = 0, jac21 = 0, jac22 = 0;
                for (int j1 = 0; j1 < o1; j1++) {
                    int j = j1 + i2 * o1 + i3 * o1 * o1;
                    double Xv = X[j], Yv = Y[j], Zv = Z[j];
                    jac00 += Xv * DPHI(j1, i1);
                    jac20 += Yv * DPHI(j1, i1);
                    jac10 += Zv * DPHI(j1, i1);
                }
                for (int j2 = 0; j2 < o1; j2++) {
                    int j = i1 + j2 * o1 + i3 * o1 * o1;
                    double Xv = X[j], Yv = Y[j], Zv = Z[j];
                    jac01 += Xv * DPHI(j2, i2);
                    jac21 += Yv * DPHI(j2, i2);
                    jac11 += Zv * DPHI(j2, i2);
                }
                for (int j3 = 0; j3 < o1; j3++) {
                    int j = i1 + i2 * o1 + j3 * o1 * o1;
                    double Xv = X[j], Yv = Y[j], Zv = Z[j];
                    jac02 += Xv * DPHI(j3, i3);
                    jac22 += Yv * DPHI(j3, i3);
                    jac12 += Zv * DPHI(j3, i3);
                }
                double detJ = fabs(jac00 * (jac11 * jac22 - jac21 * jac12)
                                   - jac01 * (jac10 * jac22 - jac20 * jac12)
                                   + jac02 * (jac10 * jac21 - jac20 * jac11));
                double a00 = jac11 * jac22 - jac12 * jac21;
                double a01 = jac02 * jac21 - jac01 * jac22;
                double a02 = jac01 * jac12 - jac02 * jac11;
                double a10 = jac12 * jac20 - jac10 * jac22;
                double a11 = jac00 * jac22 - jac02 * jac20;
                double a12 = jac02 * jac10 - jac00 * jac12;
                double a20 = jac10 * jac21 - jac11 * jac20;
                double a21 = jac01 * jac20 - jac00 * jac21;
                double a22 = jac00 * jac11 - jac01 * jac10;
                double d = 1. / detJ;
                B[i][0] = (REAL)((a00 * a00 + a01 * a01 + a02 * a02) * d);
                B[i][1] = (REAL)((a10 * a10 + a11 * a11 + a12 * a12) * d);
                B[i][2] = (REAL)((a20 * a20 + a21 * a21 + a22 * a22) * d);
                B[i][3] = (REAL)((a00 * a10 + a01 * a11 + a02 * a12) * d);
                B[i][4] = (REAL)((a00 * a20 + a01 * a21 + a02 * a22) * d);
                B[i][5] = (REAL)((a10 * a20 + a11 * a21 + a12 * a22) * d);
                massLocal[i] = (REAL)(w[i1] * w[i2] * w[i3] * detJ);
            }
#undef DPHI
}

/* SEMQkGLIntegrals.hpp:363-520 (gradPhiGradPhi, 3-D branch): for each node i the dense row
 * R[j] of the element stiffness, then Y[i] = sum_j R[j] p[j].  The reference's index forms of
 * the B13 and B23 families (:477-506) are kept as they are; they multiply off-diagonal metric
 * terms that vanish to roundoff on the axis-aligned boxes this mesh produces. */
static void SFX(grad_phi_grad_phi)(int order, const double *w, const double *dphi,
                                   REAL (*B)[6], const REAL *p, REAL *Y)
{
    const int o1 = order + 1, op2 = o1 * o1, npe = o1 * o1 * o1;
    REAL R[MAXNPE];
#define DPHI(a, b) dphi[(a) * o1 + (b)]
    for (int i3 = 0; i3 < o1; i3++)
        for (int i2 = 0; i2 < o1; i2++)
            for (int i1 = 0; i1 < o1; i1++) {
                for (int j = 0; j < npe; j++) R[j] = 0;
                /* B11 */
                for (int j1 = 0; j1 < o1; j1++) {
                    int j = j1 + i2 * o1 + i3 * op2;
                    for (int l = 0; l < o1; l++) {
                        int ll = l + i2 * o1 + i3 * op2;
                        R[j] += w[l] * w[i2] * w[i3] * (B[ll][0] * DPHI(i1, l) * DPHI(j1, l));
                    }
                }
                /* B22 */
                for (int j2 = 0; j2 < o1; j2++) {
                    int j = i1 + j2 * o1 + i3 * op2;
                    for (int m = 0; m < o1; m++) {
                        int mm = i1 + m * o1 + i3 * op2;
                        R[j] += w[i1] * w[m] * w[i3] * (B[mm][1] * DPHI(i2, m) * DPHI(j2, m));
                    }
                }
                /* B33 */
                for (int j3 = 0; j3 < o1; j3++) {
                    int j = i1 + i2 * o1 + j3 * op2;
                    for (int n = 0; n < o1; n++) {
                        int nn = i1 + i2 * o1 + n * op2;
                        R[j] += w[i1] * w[i2] * w[n] * (B[nn][2] * DPHI(i3, n) * DPHI(j3, n));
                    }
                }
                /* B12, B21 */
                for (int j2 = 0; j2 < o1; j2++)
                    for (int j1 = 0; j1 < o1; j1++) {
                        int j = j1 + j2 * o1 + i3 * op2;
                        int k = j1 + i2 * o1 + i3 * op2;
                        int l = i1 + j2 * o1 + i3 * op2;
                        R[j] += w[j1] * w[i2] * w[i3] * (B[k][3] * DPHI(i1, j1) * DPHI(j2, i2)) +
                                w[i1] * w[j2] * w[i3] * (B[l][3] * DPHI(j1, i1) * DPHI(i2, j2));
                    }
                /* B13, B31 */
                for (int j3 = 0; j3 < o1; j3++)
                    for (int j1 = 0; j1 < o1; j1++) {
                        int j = j1 + i2 * o1 + i3 * op2;
                        int k = j1 + i2 * o1 + i3 * op2;
                        int l = j1 + i2 * o1 + j3 * op2;
                        R[j] += w[j1] * w[i2] * w[i3] * (B[k][4] * DPHI(j1, i1) * DPHI(j3, i3)) +
                                w[j1] * w[i2] * w[j3] * (B[l][4] * DPHI(j1, i1) * DPHI(i3, j3));
                    }
                /* B23, B32 */
                for (int j3 = 0; j3 < o1; j3++)
                    for (int j2 = 0; j2 < o1; j2++) {
                        int j = i1 + j2 * o1 + j3 * op2;
                        int k = i1 + j2 * o1 + i3 * op2;
                        int l = i1 + i2 * o1 + j3 * op2;
                        R[j] += w[i1] * w[j2] * w[i3] * (B[k][5] * DPHI(i2, i2) * DPHI(j3, i3)) +
                                w[i1] * w[i2] * w[j3] * (B[l][5] * DPHI(j2, i2) * DPHI(i3, j3));
                    }
                int i = i1 + i2 * o1 + i3 * op2;
                Y[i] = 0;
                for (int j = 0; j < npe; j++) Y[i] += R[j] * p[j];
            }
#undef DPHI
}

/* Per-axis element-node coordinates of the REAL type, [n_elem_axis][order+1]: the float variant
 * restates the reference's float coordinates (getCoordInOneDirection, SEMmesh.cpp:81-139, with
 * the element size truncated to int); the double variant uses exact GLL points in double. */
static void SFX(axis_coords)(int order, int ne, float len, REAL *out)
{
    const int o1 = order + 1;
    if (sizeof(REAL) == sizeof(float)) {
        float xi[MAXO1], cc[MAXO1];
        float h = (float)(len / (1. * ne));
        ref_xi_float(order, xi);
        for (int e = 0; e < ne; e++) {
            coord_1d(order, (int)h, e, xi, cc);
            for (int i = 0; i < o1; i++) out[(int64_t)e * o1 + i] = (REAL)cc[i];
        }
    } else {
        double xi[MAXO1], w[MAXO1], dp[MAXO1 * MAXO1];
        or_gll_tables(order, xi, w, dp);
        double h = (double)len / ne;
        for (int e = 0; e < ne; e++)
            for (int i = 0; i < o1; i++) out[(int64_t)e * o1 + i] = (REAL)(e * h + (1.0 + xi[i]) * 0.5 * h);
    }
}

typedef struct {
    REAL *cx, *cy, *cz;   /* axis_coords for x, y, z */
} SFX(coords_t);

static int SFX(coords_init)(const or_config *c, SFX(coords_t) *k)
{
    const int o1 = c->order + 1;
    k->cx = (REAL *)malloc(sizeof(REAL) * c->ex * o1);
    k->cy = (REAL *)malloc(sizeof(REAL) * c->ey * o1);
    k->cz = (REAL *)malloc(sizeof(REAL) * c->ez * o1);
    if (!k->cx || !k->cy || !k->cz) return -1;
    SFX(axis_coords)(c->order, c->ex, c->lx, k->cx);
    SFX(axis_coords)(c->order, c->ey, c->ly, k->cy);
    SFX(axis_coords)(c->order, c->ez, c->lz, k->cz);
    return 0;
}

static void SFX(coords_free)(SFX(coords_t) *k) { free(k->cx); free(k->cy); free(k->cz); }

/* Element e's coordinate arrays X, Y, Z (SEMmesh.cpp:168-202 layout: x along local i, z along
 * local j, y along local k). */
static void SFX(element_coords)(const or_config *c, const SFX(coords_t) *k, int64_t e,
                                REAL *X, REAL *Y, REAL *Z)
{
    const int o1 = c->order + 1;
    const int64_t ex = c->ex, ez = c->ez;
    int64_t iy = e / (ex * ez), rem = e - iy * ex * ez, iz = rem / ex, ix = rem - iz * ex;
    const REAL *cx = k->cx + ix * o1, *cy = k->cy + iy * o1, *cz = k->cz + iz * o1;
    for (int kk = 0; kk < o1; kk++)
        for (int j = 0; j < o1; j++)
            for (int i = 0; i < o1; i++) {
                int q = i + o1 * j + kk * o1 * o1;
                X[q] = cx[i]; Z[q] = cz[j]; Y[q] = cy[kk];
            }
}

/* SEMQkGLIntegrals.hpp:547-565 (computeMassMatrixAndStiffnessVector V2) for element e. */
static void SFX(element_apply)(const or_config *c, const SFX(coords_t) *k, int64_t e,
                               const REAL *pl, REAL *Ml, REAL *Y)
{
    REAL X[MAXNPE], Yc[MAXNPE], Z[MAXNPE];
    REAL B[MAXNPE][6];
    SFX(element_coords)(c, k, e, X, Yc, Z);
    SFX(compute_b)(c->order, c->w, c->dphi, X, Yc, Z, Ml, B);
    SFX(grad_phi_grad_phi)(c->order, c->w, c->dphi, B, pl, Y);
}

/* One element of the loop SEMsolver.cpp:46-82: gather, local M and K.p, scatter. */
static void SFX(element_step)(const or_config *c, const SFX(coords_t) *k, int64_t e,
                              const int32_t *conn, const REAL *pn, REAL *M, REAL *y)
{
    const int o1 = c->order + 1, npe = o1 * o1 * o1;
    REAL pl[MAXNPE], Ml[MAXNPE], Y[MAXNPE];
    const int32_t *ce = conn + e * npe;
    for (int i = 0; i < npe; i++) pl[i] = pn[ce[i]];
    SFX(element_apply)(c, k, e, pl, Ml, Y);
    const REAL ve = (REAL)c->vel[e];
    for (int i = 0; i < npe; i++) {
        int g = ce[i];
        Ml[i] /= (ve * ve);
        M[g] += Ml[i];
        y[g] += Y[i];
    }
}

void SFX(or_element_apply)(const or_config *c, int64_t e, const float *p_local, float *M_local,
                           float *Y)
{
    const int o1 = c->order + 1, npe = o1 * o1 * o1;
    REAL pl[MAXNPE], Ml[MAXNPE], Yl[MAXNPE];
    SFX(coords_t) k;
    if (SFX(coords_init)(c, &k) != 0) { SFX(coords_free)(&k); return; }
    for (int i = 0; i < npe; i++) pl[i] = (REAL)p_local[i];
    SFX(element_apply)(c, &k, e, pl, Ml, Yl);
    SFX(coords_free)(&k);
    for (int i = 0; i < npe; i++) { M_local[i] = (float)Ml[i]; Y[i] = (float)Yl[i]; }
}

int SFX(or_run)(const or_config *c, REAL *p_cur, REAL *p_prev, REAL *traces)
{
    if (!c || c->order < 1 || c->order > 5 || c->ex < 1 || c->ey < 1 || c->ez < 1) return -1;
    if (!c->xi || !c->w || !c->dphi || !c->vel) return -2;
    if (c->nrec > 0 && (!c->rec_node || !traces)) return -3;
    const int o = c->order, o1 = o + 1, npe = o1 * o1 * o1;
    int64_t N, NE, NI;
    or_box_counts(c->ex, c->ey, c->ez, o, &N, &NE, &NI);
    const int64_t nx = (int64_t)c->ex * o + 1, nz = (int64_t)c->ez * o + 1;
    int32_t *conn = (int32_t *)malloc(sizeof(int32_t) * NE * npe);
    int32_t *inter = (int32_t *)malloc(sizeof(int32_t) * (NI > 0 ? NI : 1));
    REAL *M = (REAL *)malloc(sizeof(REAL) * N);
    REAL *y = (REAL *)malloc(sizeof(REAL) * N);
    SFX(coords_t) k;
    int kok = SFX(coords_init)(c, &k);
    if (!conn || !inter || !M || !y || kok != 0) {
        free(conn); free(inter); free(M); free(y); SFX(coords_free)(&k);
        return -4;
    }
    or_connectivity(c->ex, c->ey, c->ez, o, conn);
    if (NI > 0) or_interior_nodes(c->ex, c->ey, c->ez, o, inter);
    const REAL *sx = (const REAL *)c->sx, *sy = (const REAL *)c->sy, *sz = (const REAL *)c->sz;
    const int sponge = sx && sy && sz;
    const REAL dt = (REAL)c->dt;
    REAL *pc = p_cur, *pp = p_prev;   /* level i2 (current) and i1 (previous) */

    for (int s = 0; s < c->nsteps; s++) {
        const int n = c->step0 + s;
        /* SEMsolver.cpp:33-36 */
        for (int64_t i = 0; i < N; i++) { M[i] = 0; y[i] = 0; }
        /* SEMsolver.cpp:39-43: source on local node 0 of its element */
        for (int k = 0; k < c->nsrc; k++) {
            int64_t e = c->src_elem[k];
            int g = conn[e * npe];
            REAL ve = (REAL)c->vel[e];
            REAL r = (n < c->nsamples) ? (REAL)c->wavelet[(int64_t)k * c->nsamples + n] : (REAL)0;
            pc[g] += dt * dt * ve * ve * r;
        }
        /* SEMsolver.cpp:46-82 */
        if (c->nthreads <= 1) {
            for (int64_t e = 0; e < NE; e++) SFX(element_step)(c, &k, e, conn, pc, M, y);
        } else {
            /* 8-colour (parity) loop: elements of one colour share no node, so the scatter is
             * race-free; the reference's OpenMP build scatters with a plain += instead
             * (SEMmacros.hpp:50-56). */
            for (int col = 0; col < 8; col++) {
                const int cx = col & 1, cz = (col >> 1) & 1, cy = (col >> 2) & 1;
                const int64_t nxh = (c->ex - cx + 1) / 2, nzh = (c->ez - cz + 1) / 2,
                              nyh = (c->ey - cy + 1) / 2;
                const int64_t ncol = nxh * nzh * nyh;
#pragma omp parallel for schedule(static) num_threads(c->nthreads)
                for (int64_t q = 0; q < ncol; q++) {
                    int64_t a = q % nxh, b = (q / nxh) % nzh, d = q / (nxh * nzh);
                    int64_t e = (2 * a + cx) + (2 * b + cz) * c->ex + (2 * d + cy) * (int64_t)c->ex * c->ez;
                    SFX(element_step)(c, &k, e, conn, pc, M, y);
                }
            }
        }
        /* SEMsolver.cpp:85-89 */
#pragma omp parallel for schedule(static) num_threads(c->nthreads > 1 ? c->nthreads : 1)
        for (int64_t i = 0; i < NI; i++) {
            int I = inter[i];
            pp[I] = 2 * pc[I] - pp[I] - dt * dt * y[I] / M[I];
        }
        /* sponge on both levels (build definition) */
        if (sponge) {
#pragma omp parallel for schedule(static) num_threads(c->nthreads > 1 ? c->nthreads : 1)
            for (int64_t I = 0; I < N; I++) {
                int64_t iy = I / (nx * nz), r = I - iy * nx * nz, iz = r / nx, ix = r - iz * nx;
                REAL f = sx[ix] * sy[iy] * sz[iz];
                pp[I] = f * pp[I];
                pc[I] = f * pc[I];
            }
        }
        /* receivers sample the new level */
        for (int r = 0; r < c->nrec; r++) traces[(int64_t)s * c->nrec + r] = pp[c->rec_node[r]];
        /* swap (SEMproxy.cpp:53) */
        REAL *t = pc; pc = pp; pp = t;
    }
    /* leave the newest level in p_cur */
    if (pc != p_cur) {
        for (int64_t i = 0; i < N; i++) { REAL t = p_cur[i]; p_cur[i] = p_prev[i]; p_prev[i] = t; }
    }
    free(conn); free(inter); free(M); free(y); SFX(coords_free)(&k);
    return 0;
}
