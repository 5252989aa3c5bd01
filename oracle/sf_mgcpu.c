/* CPU geometric-multigrid PCG in FP64: the algorithm of the CUDA library's plain FP64 method run on the host's
 * cores with OpenMP, for the "CPU MGPCG FP64" baseline of the benchmark.
 *
 * BENCHMARK / TEST INFRASTRUCTURE ONLY.  It is timed beside the GPU arms; the library never links it.
 *
 * Method (the library's own design, restated for the host): cell-centred 2x2x2 aggregation down to dimensions
 * <= 8; the coarse operator A_c = 1/2 P^T A P kept in face-coefficient form (a coarse face is half the sum of its
 * four fine faces, a coarse diagonal excess half the sum of its eight children's); red-black Gauss-Seidel V(2,2)
 * (pre red->black, post black->red, so the cycle is symmetric); on the coarsest level, from x = 0, the
 * palindromic sequence red, (black, red) x pairs, with the mean of the right-hand side removed first when the level has no diagonal
 * excess (a pure-Neumann system); PCG stopping at ||b - A x|| <= tol ||b||.
 *
 * Operator in face-coefficient form on the dense cell grid (index (i*ny + j)*nz + k): ax, ay, az couple each cell
 * to its lower x / y / z neighbour (0 on the grid boundary and at inactive cells), dex is the diagonal excess,
 * D the diagonal (0 marks an inactive cell, whose unknown stays 0).  The converters read the assemblies of
 * sf_oracle.c, which reproduce the reference's:
 *   or_pressure_face_form  Pressure::BuildProjectionMatrix's CSR (core/Pressure.cpp:38-78), D from its diagonal;
 *   or_magnetic_face_form  MagneticField::BuildMatrix's face coefficients mu (core/MagneticField.cpp:62-90) as the
 *                          Neumann system: row 0 is not pinned; its natural right-hand side keeps the system
 *                          consistent, and the caller shifts the solution so that psi_0 = 0
 *                          (core/MagneticField.cpp:67-70).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int nx, ny, nz;
    int64_t n;
    double *ax, *ay, *az, *dex, *D, *invD;
    double *x, *b;
} mg_level;

static inline int64_t cix(const mg_level *l, int i, int j, int k) {
    return ((int64_t)i * l->ny + j) * l->nz + k;
}

/* ---------------------------------------------------------------------------------------------- converters */
void or_pressure_face_form(int nx, int ny, int nz, const int64_t *mat2grid, int64_t n, const int64_t *rowptr,
                           const int32_t *col, const double *val, double *ax, double *ay, double *az,
                           double *dex, double *D) {
    const int64_t N = (int64_t)nx * ny * nz, sx = (int64_t)ny * nz, sy = nz;
    memset(ax, 0, 8 * N);
    memset(ay, 0, 8 * N);
    memset(az, 0, 8 * N);
    memset(dex, 0, 8 * N);
    memset(D, 0, 8 * N);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; r++) {
        const int64_t c = mat2grid[r];
        double diag = 0, off = 0;
        for (int64_t e = rowptr[r]; e < rowptr[r + 1]; e++) {
            if (col[e] == r) {
                diag = val[e];
                continue;
            }
            const int64_t nb = mat2grid[col[e]];
            const double a = -val[e];
            off += a;
            if (nb == c - sx)
                ax[c] = a;
            else if (nb == c - sy)
                ay[c] = a;
            else if (nb == c - 1)
                az[c] = a;
        }
        D[c] = diag;
        dex[c] = diag - off;
    }
}

void or_magnetic_face_form(int nx, int ny, int nz, const double *mux, const double *muy, const double *muz,
                           double *ax, double *ay, double *az, double *dex, double *D) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t c = ((int64_t)i * ny + j) * nz + k;
                /* faces of cell (i, j, k): x (nx+1, ny, nz), y (nx, ny+1, nz), z (nx, ny, nz+1) */
                const double xl = mux[((int64_t)i * ny + j) * nz + k], xu = mux[((int64_t)(i + 1) * ny + j) * nz + k];
                const double yl = muy[((int64_t)i * (ny + 1) + j) * nz + k];
                const double yu = muy[((int64_t)i * (ny + 1) + j + 1) * nz + k];
                const double zl = muz[((int64_t)i * ny + j) * (nz + 1) + k];
                const double zu = muz[((int64_t)i * ny + j) * (nz + 1) + k + 1];
                /* in-grid faces only, in the order x-, x+, y-, y+, z-, z+ */
                double d = 0;
                if (i > 0) d += xl;
                if (i < nx - 1) d += xu;
                if (j > 0) d += yl;
                if (j < ny - 1) d += yu;
                if (k > 0) d += zl;
                if (k < nz - 1) d += zu;
                ax[c] = i > 0 ? xl : 0;
                ay[c] = j > 0 ? yl : 0;
                az[c] = k > 0 ? zl : 0;
                dex[c] = 0;
                D[c] = d;
            }
}

/* ---------------------------------------------------------------------------------------------- hierarchy */
static double *zalloc(int64_t n) { return (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

static void level_alloc(mg_level *l, int nx, int ny, int nz, int with_coef) {
    l->nx = nx;
    l->ny = ny;
    l->nz = nz;
    l->n = (int64_t)nx * ny * nz;
    if (with_coef) {
        l->ax = zalloc(l->n);
        l->ay = zalloc(l->n);
        l->az = zalloc(l->n);
        l->dex = zalloc(l->n);
        l->D = zalloc(l->n);
    }
    l->invD = zalloc(l->n);
    l->x = zalloc(l->n);
    l->b = zalloc(l->n);
}

static void level_free(mg_level *l, int with_coef) {
    if (with_coef) {
        free(l->ax);
        free(l->ay);
        free(l->az);
        free(l->dex);
        free(l->D);
    }
    free(l->invD);
    free(l->x);
    free(l->b);
}

/* coarse operator of level f: coarse faces and excesses, then D = in-grid couplings + excess */
static void coarsen(const mg_level *f, mg_level *c) {
#pragma omp parallel for schedule(static)
    for (int I = 0; I < c->nx; I++)
        for (int J = 0; J < c->ny; J++)
            for (int K = 0; K < c->nz; K++) {
                double fx = 0, fy = 0, fz = 0, ex = 0;
                for (int u = 0; u < 2; u++)
                    for (int v = 0; v < 2; v++) {
                        if (I > 0 && 2 * J + u < f->ny && 2 * K + v < f->nz) fx += f->ax[cix(f, 2 * I, 2 * J + u, 2 * K + v)];
                        if (J > 0 && 2 * I + u < f->nx && 2 * K + v < f->nz) fy += f->ay[cix(f, 2 * I + u, 2 * J, 2 * K + v)];
                        if (K > 0 && 2 * I + u < f->nx && 2 * J + v < f->ny) fz += f->az[cix(f, 2 * I + u, 2 * J + v, 2 * K)];
                        for (int w = 0; w < 2; w++)
                            if (2 * I + u < f->nx && 2 * J + v < f->ny && 2 * K + w < f->nz)
                                ex += f->dex[cix(f, 2 * I + u, 2 * J + v, 2 * K + w)];
                    }
                const int64_t q = cix(c, I, J, K);
                c->ax[q] = 0.5 * fx;
                c->ay[q] = 0.5 * fy;
                c->az[q] = 0.5 * fz;
                c->dex[q] = 0.5 * ex;
            }
#pragma omp parallel for schedule(static)
    for (int I = 0; I < c->nx; I++)
        for (int J = 0; J < c->ny; J++)
            for (int K = 0; K < c->nz; K++) {
                const int64_t q = cix(c, I, J, K);
                double d = c->ax[q] + c->ay[q] + c->az[q] + c->dex[q];
                if (I < c->nx - 1) d += c->ax[cix(c, I + 1, J, K)];
                if (J < c->ny - 1) d += c->ay[cix(c, I, J + 1, K)];
                if (K < c->nz - 1) d += c->az[cix(c, I, J, K + 1)];
                c->D[q] = d;
            }
}

static void set_inv(mg_level *l) {
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < l->n; q++) l->invD[q] = l->D[q] > 0 ? 1.0 / l->D[q] : 0.0;
}

/* sum over the in-grid neighbours of a * x_nb */
static inline double nbsum(const mg_level *l, const double *x, int i, int j, int k, int64_t c) {
    const int64_t sx = (int64_t)l->ny * l->nz, sy = l->nz;
    double s = 0;
    if (i > 0) s += l->ax[c] * x[c - sx];
    if (i < l->nx - 1) s += l->ax[c + sx] * x[c + sx];
    if (j > 0) s += l->ay[c] * x[c - sy];
    if (j < l->ny - 1) s += l->ay[c + sy] * x[c + sy];
    if (k > 0) s += l->az[c] * x[c - 1];
    if (k < l->nz - 1) s += l->az[c + 1] * x[c + 1];
    return s;
}

/* one colour of a red-black Gauss-Seidel sweep: x_c = (b_c + sum a x_nb) / D_c on active cells */
static void half_sweep(mg_level *l, const double *b, int colour) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < l->nx; i++)
        for (int j = 0; j < l->ny; j++) {
            const int k0 = (i + j + colour) & 1;
            for (int k = k0; k < l->nz; k += 2) {
                const int64_t c = cix(l, i, j, k);
                if (l->D[c] > 0) l->x[c] = (b[c] + nbsum(l, l->x, i, j, k, c)) * l->invD[c];
            }
        }
}

/* coarse right-hand side = sum of the children's residuals b - A x */
static void restrict_residual(const mg_level *f, mg_level *c) {
#pragma omp parallel for schedule(static)
    for (int I = 0; I < c->nx; I++)
        for (int J = 0; J < c->ny; J++)
            for (int K = 0; K < c->nz; K++) {
                double s = 0;
                for (int u = 0; u < 2; u++)
                    for (int v = 0; v < 2; v++)
                        for (int w = 0; w < 2; w++) {
                            const int i = 2 * I + u, j = 2 * J + v, k = 2 * K + w;
                            if (i >= f->nx || j >= f->ny || k >= f->nz) continue;
                            const int64_t q = cix(f, i, j, k);
                            if (f->D[q] > 0) s += f->b[q] - (f->D[q] * f->x[q] - nbsum(f, f->x, i, j, k, q));
                        }
                c->b[cix(c, I, J, K)] = s;
            }
}

static void prolong(mg_level *f, const mg_level *c) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < f->nx; i++)
        for (int j = 0; j < f->ny; j++)
            for (int k = 0; k < f->nz; k++) {
                const int64_t q = cix(f, i, j, k);
                if (f->D[q] > 0) f->x[q] += c->x[cix(c, i >> 1, j >> 1, k >> 1)];
            }
}

static void coarsest(mg_level *l, int pairs) {
    /* pure-Neumann level: remove the mean of b over the active cells (the restricted rhs misses a zero sum by
     * rounding, and Gauss-Seidel would drift along the constant) */
    double ex = 0, sb = 0;
    int64_t na = 0;
    for (int64_t q = 0; q < l->n; q++) {
        ex += fabs(l->dex[q]);
        if (l->D[q] > 0) {
            sb += l->b[q];
            na++;
        }
    }
    if (ex == 0 && na > 0) {
        const double m = sb / (double)na;
        for (int64_t q = 0; q < l->n; q++)
            if (l->D[q] > 0) l->b[q] -= m;
    }
    /* x = 0, then the palindromic sequence red, (black, red) x pairs */
    memset(l->x, 0, 8 * l->n);
    half_sweep(l, l->b, 0);
    for (int p = 0; p < pairs; p++) {
        half_sweep(l, l->b, 1);
        half_sweep(l, l->b, 0);
    }
}

/* z = M r: V(2,2) from level 0 (lv[0].b = r on entry, lv[0].x = z on exit) */
static void vcycle(mg_level *lv, int L, int l, int pairs) {
    mg_level *f = &lv[l];
    if (l == L - 1) {
        coarsest(f, pairs);
        return;
    }
    memset(f->x, 0, 8 * f->n);
    for (int s = 0; s < 2; s++) {
        half_sweep(f, f->b, 0);
        half_sweep(f, f->b, 1);
    }
    restrict_residual(f, &lv[l + 1]);
    vcycle(lv, L, l + 1, pairs);
    prolong(f, &lv[l + 1]);
    for (int s = 0; s < 2; s++) {
        half_sweep(f, f->b, 1);
        half_sweep(f, f->b, 0);
    }
}

static double dotv(int64_t n, const double *a, const double *b) {
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t q = 0; q < n; q++) s += a[q] * b[q];
    return s;
}

/* q = A p on level 0 */
static void apply(const mg_level *l, const double *p, double *q) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < l->nx; i++)
        for (int j = 0; j < l->ny; j++)
            for (int k = 0; k < l->nz; k++) {
                const int64_t c = cix(l, i, j, k);
                q[c] = l->D[c] > 0 ? l->D[c] * p[c] - nbsum(l, p, i, j, k, c) : 0.0;
            }
}

/* Solves A x = b (face form of level 0) from x = 0 to ||b - A x|| <= tol ||b||; coarse_dim 8, `pairs` coarsest
 * sweep pairs.  Returns the iterations (-1 on allocation failure); *relres = the recursive residual's ratio. */
int or_mgpcg_solve(int nx, int ny, int nz, const double *ax, const double *ay, const double *az, const double *dex,
                   const double *D, const double *b, double *x, double tol, int maxit, int pairs, double *relres) {
    mg_level lv[32];
    int L = 1;
    memset(lv, 0, sizeof(lv));
    level_alloc(&lv[0], nx, ny, nz, 0);
    lv[0].ax = (double *)ax;
    lv[0].ay = (double *)ay;
    lv[0].az = (double *)az;
    lv[0].dex = (double *)dex;
    lv[0].D = (double *)D;
    set_inv(&lv[0]);
    while (L < 32 && (lv[L - 1].nx > 8 || lv[L - 1].ny > 8 || lv[L - 1].nz > 8)) {
        const mg_level *f = &lv[L - 1];
        level_alloc(&lv[L], (f->nx + 1) / 2, (f->ny + 1) / 2, (f->nz + 1) / 2, 1);
        coarsen(f, &lv[L]);
        set_inv(&lv[L]);
        L++;
    }
    const int64_t n = lv[0].n;
    double *r = zalloc(n), *p = zalloc(n), *q = zalloc(n);
    int it = 0;
    if (!r || !p || !q) {
        it = -1;
        goto done;
    }
    memset(x, 0, 8 * n);
    memcpy(r, b, 8 * n);
    const double bb = dotv(n, b, b);
    double rr = bb;
    if (bb == 0) {
        *relres = 0;
        goto done;
    }
    memcpy(lv[0].b, r, 8 * n);
    vcycle(lv, L, 0, pairs);
    memcpy(p, lv[0].x, 8 * n);
    double rho = dotv(n, r, lv[0].x);
    while (it < maxit) {
        apply(&lv[0], p, q);
        const double pq = dotv(n, p, q);
        if (!(pq > 0)) break;
        const double alpha = rho / pq;
        double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (int64_t c = 0; c < n; c++) {
            x[c] += alpha * p[c];
            r[c] -= alpha * q[c];
            s += r[c] * r[c];
        }
        rr = s;
        it++;
        if (rr <= tol * tol * bb) break;
        memcpy(lv[0].b, r, 8 * n);
        vcycle(lv, L, 0, pairs);
        const double rho1 = dotv(n, r, lv[0].x);
        const double beta = rho1 / rho;
        rho = rho1;
        const double *z = lv[0].x;
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < n; c++) p[c] = z[c] + beta * p[c];
    }
    *relres = sqrt(rr / bb);
done:
    free(r);
    free(p);
    free(q);
    for (int l = 1; l < L; l++) level_free(&lv[l], 1);
    level_free(&lv[0], 0);
    return it;
}
