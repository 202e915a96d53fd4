/*
 * anneal_oracle.c -- FP64 CPU restatement of the anneal 0.3.0 voxel SIMP hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU library and the timed
 * CPU baseline in bench.py. Nothing in the product links, calls or loads it.
 *
 * Every function restates the reference algorithm it cites (file:line within the
 * anneal project). The reference assembles a CSR matrix and solves with scipy CG and a
 * pyamg preconditioner; this restatement applies the same operator K = sum_e E_e Ke
 * element by element (no assembly), which is the same linear map.
 *
 * Grid conventions (fem.py:87-127): element e = i + nx*(j + ny*k); node
 * n = i + (nx+1)*(j + (ny+1)*k); DOF = 3*n + c; local node order LOCAL (fem.py:20-21).
 *
 * Build: oracle.build() in oracle/oracle.py (gcc -O3 -fopenmp -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* parallel regions only pay off on grids of a few thousand elements or more */
#define OMP_BIG(a, b, c) ((int64_t)(a) * (b) * (c) > 8192)

static const int LOCAL[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

/* ------------------------------------------------------------------ element matrix */

/* elasticity_D (fem.py:36-43): isotropic D for E = 1, Voigt xx yy zz xy yz zx. */
static void elasticity_D(double nu, double D[6][6]) {
    double c = 1.0 / ((1 + nu) * (1 - 2 * nu));
    memset(D, 0, sizeof(double) * 36);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) D[a][b] = nu * c;
    for (int a = 0; a < 3; ++a) D[a][a] = (1 - nu) * c;
    for (int a = 3; a < 6; ++a) D[a][a] = (1 - 2 * nu) / 2 * c;
}

/* _dN and _B (fem.py:46-68): shape-function derivatives and strain-displacement. */
static void strain_matrix(double xi, double eta, double zeta, double jac, double B[6][24]) {
    memset(B, 0, sizeof(double) * 6 * 24);
    for (int a = 0; a < 8; ++a) {
        double s0 = 2 * LOCAL[a][0] - 1, s1 = 2 * LOCAL[a][1] - 1, s2 = 2 * LOCAL[a][2] - 1;
        double dx = s0 * (1 + s1 * eta) * (1 + s2 * zeta) / 8 / jac;
        double dy = s1 * (1 + s0 * xi) * (1 + s2 * zeta) / 8 / jac;
        double dz = s2 * (1 + s0 * xi) * (1 + s1 * eta) / 8 / jac;
        B[0][3 * a] = dx;
        B[1][3 * a + 1] = dy;
        B[2][3 * a + 2] = dz;
        B[3][3 * a] = dy;
        B[3][3 * a + 1] = dx;
        B[4][3 * a + 1] = dz;
        B[4][3 * a + 2] = dy;
        B[5][3 * a] = dz;
        B[5][3 * a + 2] = dx;
    }
}

/* hex8_matrices (fem.py:71-84): 24x24 Ke for E = 1 on a cube of side h, 2x2x2 Gauss. */
void orc_hex8_ke(double nu, double h, double* ke /* 576 */) {
    double D[6][6], B[6][24], DB[6][24];
    elasticity_D(nu, D);
    memset(ke, 0, sizeof(double) * 576);
    double g = 1.0 / sqrt(3.0), jac = h / 2;
    for (int q = 0; q < 8; ++q) {
        double xi = (q & 1) ? g : -g, eta = (q & 2) ? g : -g, zeta = (q & 4) ? g : -g;
        /* the reference loops xi outermost; the sum over 8 points is order-independent
           up to rounding */
        strain_matrix(xi, eta, zeta, jac, B);
        for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 24; ++c) {
                double s = 0;
                for (int k = 0; k < 6; ++k) s += D[r][k] * B[k][c];
                DB[r][c] = s;
            }
        double w = jac * jac * jac;
        for (int r = 0; r < 24; ++r)
            for (int c = 0; c < 24; ++c) {
                double s = 0;
                for (int k = 0; k < 6; ++k) s += B[k][r] * DB[k][c];
                ke[r * 24 + c] += s * w;
            }
    }
}

/* ------------------------------------------------------------------ operator */

typedef struct {
    int nx, ny, nz;
} grid_t;

static inline int64_t node_id(const grid_t* g, int i, int j, int k) {
    return (int64_t)i + (int64_t)(g->nx + 1) * ((int64_t)j + (int64_t)(g->ny + 1) * k);
}

static inline void elem_dofs(const grid_t* g, int i, int j, int k, int64_t dof[24]) {
    for (int a = 0; a < 8; ++a) {
        int64_t n = node_id(g, i + LOCAL[a][0], j + LOCAL[a][1], k + LOCAL[a][2]);
        dof[3 * a] = 3 * n;
        dof[3 * a + 1] = 3 * n + 1;
        dof[3 * a + 2] = 3 * n + 2;
    }
}

/*
 * y = K u with K = sum_e E[e] * ke over elements with E[e] != 0, restricted to free DOFs
 * (dofmask[d] != 0): the reference's reduced matrix (fem.py:142-172, assemble :198-201)
 * acting on u_free, written back in full-grid layout with zeros on non-free DOFs.
 * Elements are visited in 8 parity colours so a colour's elements share no node.
 */
void orc_apply_K(int nx, int ny, int nz, const double* ke, const double* E, const uint8_t* dofmask,
                 const double* u, double* y) {
    grid_t g = {nx, ny, nz};
    int64_t ndof = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    memset(y, 0, sizeof(double) * ndof);
    for (int color = 0; color < 8; ++color) {
        int ci = color & 1, cj = (color >> 1) & 1, ck = (color >> 2) & 1;
#pragma omp parallel for collapse(2) schedule(static) if (OMP_BIG(nx, ny, nz))
        for (int k = ck; k < nz; k += 2)
            for (int j = cj; j < ny; j += 2)
                for (int i = ci; i < nx; i += 2) {
                    int64_t e = i + (int64_t)nx * (j + (int64_t)ny * k);
                    double Ee = E[e];
                    if (Ee == 0.0) continue;
                    int64_t dof[24];
                    double ue[24];
                    elem_dofs(&g, i, j, k, dof);
                    for (int a = 0; a < 24; ++a) ue[a] = dofmask[dof[a]] ? u[dof[a]] : 0.0;
                    for (int r = 0; r < 24; ++r) {
                        double s = 0;
                        const double* kr = ke + 24 * r;
                        for (int c = 0; c < 24; ++c) s += kr[c] * ue[c];
                        y[dof[r]] += Ee * s;
                    }
                }
    }
#pragma omp parallel for schedule(static) if (ndof > 65536)
    for (int64_t d = 0; d < ndof; ++d)
        if (!dofmask[d]) y[d] = 0.0;
}

/* Diagonal of K (free DOFs; 1 elsewhere so it can divide). */
void orc_diag(int nx, int ny, int nz, const double* ke, const double* E, const uint8_t* dofmask,
              double* dg) {
    grid_t g = {nx, ny, nz};
    int64_t ndof = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    memset(dg, 0, sizeof(double) * ndof);
    for (int color = 0; color < 8; ++color) {
        int ci = color & 1, cj = (color >> 1) & 1, ck = (color >> 2) & 1;
#pragma omp parallel for collapse(2) schedule(static) if (OMP_BIG(nx, ny, nz))
        for (int k = ck; k < nz; k += 2)
            for (int j = cj; j < ny; j += 2)
                for (int i = ci; i < nx; i += 2) {
                    int64_t e = i + (int64_t)nx * (j + (int64_t)ny * k);
                    if (E[e] == 0.0) continue;
                    int64_t dof[24];
                    elem_dofs(&g, i, j, k, dof);
                    for (int r = 0; r < 24; ++r) dg[dof[r]] += E[e] * ke[25 * r];
                }
    }
    for (int64_t d = 0; d < ndof; ++d)
        if (!dofmask[d] || dg[d] == 0.0) dg[d] = 1.0;
}

/* element_energy (fem.py:239-242): ce[e] = u_e^T ke u_e for every element with
   active[e] != 0 (the caller compacts to the active list). */
void orc_element_energy(int nx, int ny, int nz, const double* ke, const uint8_t* active,
                        const double* u, double* ce) {
    grid_t g = {nx, ny, nz};
#pragma omp parallel for collapse(2) schedule(static) if (OMP_BIG(nx, ny, nz))
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int64_t e = i + (int64_t)nx * (j + (int64_t)ny * k);
                if (!active[e]) {
                    ce[e] = 0.0;
                    continue;
                }
                int64_t dof[24];
                double ue[24];
                elem_dofs(&g, i, j, k, dof);
                for (int a = 0; a < 24; ++a) ue[a] = u[dof[a]];
                double s = 0;
                for (int r = 0; r < 24; ++r) {
                    double t = 0;
                    for (int c = 0; c < 24; ++c) t += ke[24 * r + c] * ue[c];
                    s += ue[r] * t;
                }
                ce[e] = s;
            }
}

/* ------------------------------------------------------------------ density filter */

/*
 * Filter (optimize.py:24-47): cone weights w = max(0, r - |d|) on a (2R+1)^3 box with
 * R = max(ceil(r) - 1, 1) (:28-31), zero padding (ndimage mode "constant").
 * mode 0: Hs = conv(active), zeros replaced by 1 (:32-33)
 * mode 1: forward  out = conv(in * active) / Hs          (:41-43)
 * mode 2: backward out = conv(in / Hs) * active          (:45-47)
 * Arrays are full-grid (nelem), x fastest; inactive entries of `in` must be 0.
 */
void orc_filter(int nx, int ny, int nz, double r, const uint8_t* active, const double* Hs,
                const double* in, double* out, int mode) {
    int R = (int)ceil(r) - 1;
    if (R < 1) R = 1;
    int W = 2 * R + 1;
    double* w = (double*)malloc(sizeof(double) * W * W * W);
    for (int dz = -R; dz <= R; ++dz)
        for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
                double v = r - sqrt((double)(dx * dx + dy * dy + dz * dz));
                w[(dx + R) + W * ((dy + R) + W * (dz + R))] = v > 0 ? v : 0.0;
            }
#pragma omp parallel for collapse(2) schedule(static) if (OMP_BIG(nx, ny, nz))
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int64_t e = i + (int64_t)nx * (j + (int64_t)ny * k);
                double s = 0;
                for (int dz = -R; dz <= R; ++dz) {
                    int kk = k + dz;
                    if (kk < 0 || kk >= nz) continue;
                    for (int dy = -R; dy <= R; ++dy) {
                        int jj = j + dy;
                        if (jj < 0 || jj >= ny) continue;
                        for (int dx = -R; dx <= R; ++dx) {
                            int ii = i + dx;
                            if (ii < 0 || ii >= nx) continue;
                            double wt = w[(dx + R) + W * ((dy + R) + W * (dz + R))];
                            if (wt == 0.0) continue;
                            int64_t f = ii + (int64_t)nx * (jj + (int64_t)ny * kk);
                            double v;
                            if (mode == 0) v = active[f] ? 1.0 : 0.0;
                            else if (mode == 1) v = active[f] ? in[f] : 0.0;
                            else v = active[f] ? in[f] / Hs[f] : 0.0;
                            s += wt * v;
                        }
                    }
                }
                if (mode == 0) out[e] = s == 0.0 ? 1.0 : s;
                else if (mode == 1) out[e] = s / Hs[e];
                else out[e] = active[e] ? s : 0.0;
            }
    free(w);
}

/* ------------------------------------------------------------------ vector helpers */

static double dot(int64_t n, const double* a, const double* b) {
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 65536)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* ------------------------------------------------------------------ geometric multigrid */
/*
 * The reference preconditions CG with pyamg smoothed aggregation (fem.py:212-215); pyamg
 * is not available, so the oracle offers Jacobi (tests) and a geometric V-cycle
 * (large grids). A preconditioner changes iteration counts, never the converged answer.
 * Coarse levels halve the element grid; coarse element scale = (sum of the 8 children)/4,
 * i.e. the children's mean at Ke(2h) = 2 Ke(h); transfer = trilinear interpolation and
 * its transpose; Chebyshev smoothing on D^-1 K; dense Cholesky on the coarsest level.
 * The smoother follows the GPU solver's, so that a CPU timing scaled by the GPU's CG
 * iteration count compares like with like: below the element bound lambda_max(Ke) / Ke_00
 * (an upper bound of the spectrum of D^-1 K for every design), `degree` steps over
 * [ORC_LO, 1] x bound on levels 0 and 1 and ORC_DEG_COARSE steps over [ORC_LO_COARSE, 1] x
 * bound below.
 */
#define ORC_LO 0.03
#define ORC_LO_COARSE 0.002
#define ORC_DEG_COARSE 8
typedef struct {
    int nx, ny, nz;
    int64_t nn, ndof;
    double* E;
    uint8_t* dofmask;
    uint8_t* used; /* per node */
    double* dg;
    double* x;
    double* b;
    double* r;
    double* d;
    double* chol; /* coarsest only, ndof x ndof */
} level_t;

typedef struct {
    int nlev;
    level_t lev[16];
    const double* ke;
    int degree;
    double bound; /* lambda_max(Ke) / Ke_00, slightly enlarged */
} mg_t;

static void level_alloc(level_t* L, int nx, int ny, int nz) {
    L->nx = nx;
    L->ny = ny;
    L->nz = nz;
    L->nn = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    L->ndof = 3 * L->nn;
    L->E = (double*)calloc((size_t)nx * ny * nz, sizeof(double));
    L->dofmask = (uint8_t*)calloc(L->ndof, 1);
    L->used = (uint8_t*)calloc(L->nn, 1);
    L->dg = (double*)calloc(L->ndof, sizeof(double));
    L->x = (double*)calloc(L->ndof, sizeof(double));
    L->b = (double*)calloc(L->ndof, sizeof(double));
    L->r = (double*)calloc(L->ndof, sizeof(double));
    L->d = (double*)calloc(L->ndof, sizeof(double));
    L->chol = NULL;
}

static void level_free(level_t* L) {
    free(L->E);
    free(L->dofmask);
    free(L->used);
    free(L->dg);
    free(L->x);
    free(L->b);
    free(L->r);
    free(L->d);
    free(L->chol);
}

static void mark_used(level_t* L) {
    memset(L->used, 0, L->nn);
    grid_t g = {L->nx, L->ny, L->nz};
    for (int k = 0; k < L->nz; ++k)
        for (int j = 0; j < L->ny; ++j)
            for (int i = 0; i < L->nx; ++i) {
                if (L->E[i + (int64_t)L->nx * (j + (int64_t)L->ny * k)] == 0.0) continue;
                for (int a = 0; a < 8; ++a)
                    L->used[node_id(&g, i + LOCAL[a][0], j + LOCAL[a][1], k + LOCAL[a][2])] = 1;
            }
}

/* 1D trilinear weights: fine index f maps to coarse coordinate f/2. */
static inline int coarse_span(int f, int* c0, double* w0, int* c1, double* w1) {
    if ((f & 1) == 0) {
        *c0 = f / 2;
        *w0 = 1.0;
        return 1;
    }
    *c0 = f / 2;
    *w0 = 0.5;
    *c1 = f / 2 + 1;
    *w1 = 0.5;
    return 2;
}

/* xf += P xc (prolongation), masked to free fine DOFs */
static void prolong_add(const level_t* F, const level_t* C, const double* xc, double* xf) {
    int fnx = F->nx + 1, fny = F->ny + 1, fnz = F->nz + 1;
    int cnx = C->nx + 1, cny = C->ny + 1;
#pragma omp parallel for collapse(2) schedule(static) if (OMP_BIG(fnx, fny, fnz))
    for (int k = 0; k < fnz; ++k)
        for (int j = 0; j < fny; ++j)
            for (int i = 0; i < fnx; ++i) {
                int ci[2], cj[2], ck[2];
                double wi[2], wj[2], wk[2];
                int ni = coarse_span(i, &ci[0], &wi[0], &ci[1], &wi[1]);
                int nj = coarse_span(j, &cj[0], &wj[0], &cj[1], &wj[1]);
                int nk = coarse_span(k, &ck[0], &wk[0], &ck[1], &wk[1]);
                double acc[3] = {0, 0, 0};
                for (int c = 0; c < nk; ++c)
                    for (int b = 0; b < nj; ++b)
                        for (int a = 0; a < ni; ++a) {
                            double w = wi[a] * wj[b] * wk[c];
                            int64_t cn = ci[a] + (int64_t)cnx * (cj[b] + (int64_t)cny * ck[c]);
                            acc[0] += w * xc[3 * cn];
                            acc[1] += w * xc[3 * cn + 1];
                            acc[2] += w * xc[3 * cn + 2];
                        }
                int64_t fn = i + (int64_t)fnx * (j + (int64_t)fny * k);
                for (int c = 0; c < 3; ++c)
                    if (F->dofmask[3 * fn + c]) xf[3 * fn + c] += acc[c];
            }
}

/* bc = P^T rf, masked to free coarse DOFs */
static void restrict_(const level_t* F, const level_t* C, const double* rf, double* bc) {
    int fnx = F->nx + 1, fny = F->ny + 1, fnz = F->nz + 1;
    int cnx = C->nx + 1, cny = C->ny + 1, cnz = C->nz + 1;
#pragma omp parallel for collapse(2) schedule(static) if (OMP_BIG(cnx, cny, cnz))
    for (int K = 0; K < cnz; ++K)
        for (int J = 0; J < cny; ++J)
            for (int I = 0; I < cnx; ++I) {
                double acc[3] = {0, 0, 0};
                for (int dk = -1; dk <= 1; ++dk) {
                    int k = 2 * K + dk;
                    if (k < 0 || k >= fnz) continue;
                    double wk = dk == 0 ? 1.0 : 0.5;
                    for (int dj = -1; dj <= 1; ++dj) {
                        int j = 2 * J + dj;
                        if (j < 0 || j >= fny) continue;
                        double wj = dj == 0 ? 1.0 : 0.5;
                        for (int di = -1; di <= 1; ++di) {
                            int i = 2 * I + di;
                            if (i < 0 || i >= fnx) continue;
                            double w = wk * wj * (di == 0 ? 1.0 : 0.5);
                            int64_t fn = i + (int64_t)fnx * (j + (int64_t)fny * k);
                            acc[0] += w * rf[3 * fn];
                            acc[1] += w * rf[3 * fn + 1];
                            acc[2] += w * rf[3 * fn + 2];
                        }
                    }
                }
                int64_t cn = I + (int64_t)cnx * (J + (int64_t)cny * K);
                for (int c = 0; c < 3; ++c) bc[3 * cn + c] = C->dofmask[3 * cn + c] ? acc[c] : 0.0;
            }
}

static void coarsen(const level_t* F, level_t* C) {
    level_alloc(C, (F->nx + 1) / 2, (F->ny + 1) / 2, (F->nz + 1) / 2);
    for (int K = 0; K < C->nz; ++K)
        for (int J = 0; J < C->ny; ++J)
            for (int I = 0; I < C->nx; ++I) {
                double s = 0;
                for (int c = 0; c < 8; ++c) {
                    int i = 2 * I + (c & 1), j = 2 * J + ((c >> 1) & 1), k = 2 * K + ((c >> 2) & 1);
                    if (i < F->nx && j < F->ny && k < F->nz) s += F->E[i + (int64_t)F->nx * (j + (int64_t)F->ny * k)];
                }
                C->E[I + (int64_t)C->nx * (J + (int64_t)C->ny * K)] = 0.25 * s;
            }
    mark_used(C);
    /* a coarse DOF is fixed if a used fine node within one fine spacing has it fixed */
    int fnx = F->nx + 1, fny = F->ny + 1, fnz = F->nz + 1;
    int cnx = C->nx + 1, cny = C->ny + 1, cnz = C->nz + 1;
    for (int K = 0; K < cnz; ++K)
        for (int J = 0; J < cny; ++J)
            for (int I = 0; I < cnx; ++I) {
                int64_t cn = I + (int64_t)cnx * (J + (int64_t)cny * K);
                int fixed[3] = {0, 0, 0};
                for (int dk = -1; dk <= 1; ++dk)
                    for (int dj = -1; dj <= 1; ++dj)
                        for (int di = -1; di <= 1; ++di) {
                            int i = 2 * I + di, j = 2 * J + dj, k = 2 * K + dk;
                            if (i < 0 || j < 0 || k < 0 || i >= fnx || j >= fny || k >= fnz) continue;
                            int64_t fn = i + (int64_t)fnx * (j + (int64_t)fny * k);
                            if (!F->used[fn]) continue;
                            for (int c = 0; c < 3; ++c)
                                if (!F->dofmask[3 * fn + c]) fixed[c] = 1;
                        }
                for (int c = 0; c < 3; ++c) C->dofmask[3 * cn + c] = C->used[cn] && !fixed[c];
            }
}

static void apply_level(const mg_t* mg, const level_t* L, const double* u, double* y) {
    orc_apply_K(L->nx, L->ny, L->nz, mg->ke, L->E, L->dofmask, u, y);
}

/* lambda_max(Ke) / Ke_00 by power iteration on the 24 x 24 element matrix */
static double element_bound(const double* ke) {
    double v[24], w[24], lam = 0.0;
    for (int i = 0; i < 24; ++i) v[i] = 1.0 + 0.01 * i * ((i % 3) + 1) * ((i & 1) ? -1.0 : 1.0);
    for (int it = 0; it < 500; ++it) {
        double nv = 0.0;
        for (int i = 0; i < 24; ++i) nv += v[i] * v[i];
        nv = sqrt(nv);
        for (int i = 0; i < 24; ++i) v[i] /= nv;
        for (int i = 0; i < 24; ++i) {
            double t = 0.0;
            for (int j = 0; j < 24; ++j) t += ke[24 * i + j] * v[j];
            w[i] = t;
        }
        lam = 0.0;
        for (int i = 0; i < 24; ++i) lam += v[i] * w[i];
        memcpy(v, w, sizeof(v));
    }
    return 1.001 * lam / ke[0];
}

static int chol_factor(double* A, int n) {
    for (int j = 0; j < n; ++j) {
        double s = A[(int64_t)j * n + j];
        for (int k = 0; k < j; ++k) s -= A[(int64_t)j * n + k] * A[(int64_t)j * n + k];
        if (s <= 0) return -1;
        s = sqrt(s);
        A[(int64_t)j * n + j] = s;
        for (int i = j + 1; i < n; ++i) {
            double t = A[(int64_t)i * n + j];
            for (int k = 0; k < j; ++k) t -= A[(int64_t)i * n + k] * A[(int64_t)j * n + k];
            A[(int64_t)i * n + j] = t / s;
        }
    }
    return 0;
}

static void chol_solve(const double* L, int n, double* x) {
    for (int i = 0; i < n; ++i) {
        double s = x[i];
        for (int k = 0; k < i; ++k) s -= L[(int64_t)i * n + k] * x[k];
        x[i] = s / L[(int64_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = x[i];
        for (int k = i + 1; k < n; ++k) s -= L[(int64_t)k * n + i] * x[k];
        x[i] = s / L[(int64_t)i * n + i];
    }
}

static int coarse_setup(const mg_t* mg, level_t* L) {
    int n = (int)L->ndof;
    L->chol = (double*)calloc((size_t)n * n, sizeof(double));
    grid_t g = {L->nx, L->ny, L->nz};
    for (int k = 0; k < L->nz; ++k)
        for (int j = 0; j < L->ny; ++j)
            for (int i = 0; i < L->nx; ++i) {
                double Ee = L->E[i + (int64_t)L->nx * (j + (int64_t)L->ny * k)];
                if (Ee == 0.0) continue;
                int64_t dof[24];
                elem_dofs(&g, i, j, k, dof);
                for (int a = 0; a < 24; ++a)
                    for (int b = 0; b < 24; ++b) L->chol[dof[a] * n + dof[b]] += Ee * mg->ke[24 * a + b];
            }
    for (int a = 0; a < n; ++a)
        if (!L->dofmask[a]) {
            for (int b = 0; b < n; ++b) L->chol[(int64_t)a * n + b] = L->chol[(int64_t)b * n + a] = 0.0;
            L->chol[(int64_t)a * n + a] = 1.0;
        }
    return chol_factor(L->chol, n);
}

/* Chebyshev smoothing of K x = b below the element bound, from the given x */
static void chebyshev(const mg_t* mg, level_t* L, int x_is_zero) {
    int64_t n = L->ndof;
    const int coarse = (L - mg->lev) >= 2;
    const int degree = coarse ? ORC_DEG_COARSE : mg->degree;
    double hi = mg->bound, lo = (coarse ? ORC_LO_COARSE : ORC_LO) * mg->bound;
    double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    double rho_old = 1.0 / sigma;
    if (x_is_zero) memcpy(L->r, L->b, sizeof(double) * n);
    else {
        apply_level(mg, L, L->x, L->r);
        for (int64_t i = 0; i < n; ++i) L->r[i] = L->b[i] - L->r[i];
    }
    for (int64_t i = 0; i < n; ++i) {
        L->d[i] = L->r[i] / L->dg[i] / theta;
        L->x[i] += L->d[i];
    }
    for (int s = 1; s < degree; ++s) {
        apply_level(mg, L, L->x, L->r);
        double rho = 1.0 / (2 * sigma - rho_old);
        for (int64_t i = 0; i < n; ++i) {
            double ri = L->b[i] - L->r[i];
            L->d[i] = rho * rho_old * L->d[i] + 2 * rho / delta * ri / L->dg[i];
            L->x[i] += L->d[i];
        }
        rho_old = rho;
    }
}

static void vcycle(const mg_t* mg, int l) {
    level_t* L = (level_t*)&mg->lev[l];
    int64_t n = L->ndof;
    if (l == mg->nlev - 1) {
        memcpy(L->x, L->b, sizeof(double) * n);
        chol_solve(L->chol, (int)n, L->x);
        for (int64_t i = 0; i < n; ++i)
            if (!L->dofmask[i]) L->x[i] = 0.0;
        return;
    }
    level_t* C = (level_t*)&mg->lev[l + 1];
    memset(L->x, 0, sizeof(double) * n);
    chebyshev(mg, L, 1);
    apply_level(mg, L, L->x, L->r);
    for (int64_t i = 0; i < n; ++i) L->r[i] = L->b[i] - L->r[i];
    restrict_(L, C, L->r, C->b);
    vcycle(mg, l + 1);
    prolong_add(L, C, C->x, L->x);
    chebyshev(mg, L, 0);
}

/* ------------------------------------------------------------------ PCG */

/*
 * Preconditioned CG on the free DOFs, FP64, one right-hand side (fem.py:206-232 with
 * scipy cg semantics: stop when ||b - K x|| <= rtol ||b|| on the recurrence residual,
 * x = 0 returned for b = 0). precond: 0 = Jacobi, 1 = geometric multigrid.
 * x holds the initial guess on entry (zeros on non-free DOFs).
 * Returns 0 on convergence, 1 if maxiter was reached, 2 on a non-finite value or a
 * singular coarse matrix. *iters gets the iteration count, *relres ||r||/||b||.
 */
int orc_pcg(int nx, int ny, int nz, const double* ke, const double* E, const uint8_t* dofmask,
            const double* b, double* x, double rtol, int maxiter, int precond, int mg_degree,
            int* iters_out, double* relres_out) {
    int64_t n = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    double* r = (double*)malloc(sizeof(double) * n);
    double* z = (double*)malloc(sizeof(double) * n);
    double* p = (double*)malloc(sizeof(double) * n);
    double* q = (double*)malloc(sizeof(double) * n);
    mg_t mg;
    memset(&mg, 0, sizeof(mg));
    mg.ke = ke;
    mg.degree = mg_degree > 0 ? mg_degree : 2;
    int status = 0;
    /* level 0 */
    level_alloc(&mg.lev[0], nx, ny, nz);
    memcpy(mg.lev[0].E, E, sizeof(double) * (size_t)nx * ny * nz);
    memcpy(mg.lev[0].dofmask, dofmask, n);
    mark_used(&mg.lev[0]);
    orc_diag(nx, ny, nz, ke, E, dofmask, mg.lev[0].dg);
    mg.nlev = 1;
    if (precond == 1) {
        while (mg.nlev < 16) {
            level_t* F = &mg.lev[mg.nlev - 1];
            if (F->ndof <= 400 || F->nx < 2 || F->ny < 2 || F->nz < 2) break;
            coarsen(F, &mg.lev[mg.nlev]);
            level_t* C = &mg.lev[mg.nlev];
            orc_diag(C->nx, C->ny, C->nz, ke, C->E, C->dofmask, C->dg);
            mg.nlev++;
        }
        mg.bound = element_bound(ke);
        if (mg.nlev == 1 || coarse_setup(&mg, &mg.lev[mg.nlev - 1]) != 0) {
            if (mg.nlev > 1) status = 2;
            precond = 0;
        }
    }
    for (int64_t i = 0; i < n; ++i)
        if (!dofmask[i]) x[i] = 0.0;
    double bnorm = sqrt(dot(n, b, b));
    int it = 0;
    double rnorm = 0;
    if (bnorm == 0.0) {
        memset(x, 0, sizeof(double) * n);
        *iters_out = 0;
        *relres_out = 0.0;
        goto done;
    }
    orc_apply_K(nx, ny, nz, ke, E, dofmask, x, q);
    for (int64_t i = 0; i < n; ++i) r[i] = dofmask[i] ? b[i] - q[i] : 0.0;
    rnorm = sqrt(dot(n, r, r));
    double rz = 0, rz_old = 0;
    while (rnorm > rtol * bnorm) {
        if (it >= maxiter) {
            status = status ? status : 1;
            break;
        }
        if (precond == 1) {
            memcpy(mg.lev[0].b, r, sizeof(double) * n);
            vcycle(&mg, 0);
            memcpy(z, mg.lev[0].x, sizeof(double) * n);
        } else {
            for (int64_t i = 0; i < n; ++i) z[i] = r[i] / mg.lev[0].dg[i];
        }
        rz = dot(n, r, z);
        if (it == 0) memcpy(p, z, sizeof(double) * n);
        else {
            double beta = rz / rz_old;
            for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        }
        orc_apply_K(nx, ny, nz, ke, E, dofmask, p, q);
        double pq = dot(n, p, q);
        double alpha = rz / pq;
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        rz_old = rz;
        rnorm = sqrt(dot(n, r, r));
        ++it;
        if (!isfinite(rnorm)) {
            status = 2;
            break;
        }
    }
    *iters_out = it;
    *relres_out = rnorm / bnorm;
done:
    for (int l = 0; l < mg.nlev; ++l) level_free(&mg.lev[l]);
    free(r);
    free(z);
    free(p);
    free(q);
    return status;
}

/* ------------------------------------------------------------------ OC update */

/*
 * OC bisection (optimize.py:144-161) over the active elements (compact arrays of length
 * nact, `act` = their full-grid indices). physical(xn) = filter forward, Heaviside
 * projection with beta (optimize.py:81-93; beta <= 0 means none), frozen set to 1.
 * Writes xd (the last evaluated xn, as the reference does) and returns the number of
 * bisection steps.
 */
int orc_oc(int nx, int ny, int nz, double r, const uint8_t* active, const double* Hs, int64_t nact,
           const int64_t* act, const double* x, const double* dcx, const double* dvx,
           const double* phi, const uint8_t* frozen, double move, double beta, double eta,
           double vtarget, double* xd) {
    int64_t ne = (int64_t)nx * ny * nz;
    double* full = (double*)calloc(ne, sizeof(double));
    double* filt = (double*)malloc(sizeof(double) * ne);
    double* xn = (double*)malloc(sizeof(double) * nact);
    /* scale = mean(-dcx[des]) / max(mean(dvx[des]), 1e-30) (optimize.py:145) */
    double sc = 0, sv = 0;
    int64_t nd = 0;
    for (int64_t a = 0; a < nact; ++a)
        if (!frozen[a]) {
            sc += -dcx[a];
            sv += dvx[a];
            ++nd;
        }
    double scale = 1.0;
    if (nd > 0) {
        double mv = sv / nd;
        scale = (sc / nd) / (mv > 1e-30 ? mv : 1e-30);
        if (!(scale > 1e-300)) scale = 1e-300;
    }
    double lo = scale * 1e-8, hi = scale * 1e8;
    double mvl = beta <= 1 ? move : move / 2;
    double t0 = 0, t1 = 0;
    if (beta > 0) {
        t0 = tanh(beta * eta);
        t1 = tanh(beta * (1 - eta));
    }
    int steps = 0;
    for (int s = 0; s < 100; ++s) {
        double lam = sqrt(lo * hi);
        for (int64_t a = 0; a < nact; ++a) {
            double num = -dcx[a] > 0 ? -dcx[a] : 0.0;
            double den = dvx[a] * lam > 1e-300 ? dvx[a] * lam : 1e-300;
            double ratio = sqrt(num / den);
            double v = x[a] * ratio;
            double lo_b = x[a] - mvl > 0.0 ? x[a] - mvl : 0.0;
            double hi_b = x[a] + mvl < 1.0 ? x[a] + mvl : 1.0;
            /* np.clip(v, lo_b, hi_b) = min(max(v, lo_b), hi_b) */
            v = v < lo_b ? lo_b : v;
            v = v > hi_b ? hi_b : v;
            xn[a] = frozen[a] ? 1.0 : v;
            full[act[a]] = xn[a];
        }
        orc_filter(nx, ny, nz, r, active, Hs, full, filt, 1);
        double vol = 0;
        for (int64_t a = 0; a < nact; ++a) {
            double xt = filt[act[a]];
            double xp = xt;
            if (beta > 0) xp = (t0 + tanh(beta * (xt - eta))) / (t0 + t1);
            if (frozen[a]) xp = 1.0;
            vol += phi[a] * xp;
        }
        if (vol > vtarget) lo = lam;
        else hi = lam;
        ++steps;
        if (hi / lo < 1 + 1e-9) break;
    }
    memcpy(xd, xn, sizeof(double) * nact);
    free(full);
    free(filt);
    free(xn);
    return steps;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
