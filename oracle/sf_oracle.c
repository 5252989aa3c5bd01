/*
 * sf_oracle.c -- CPU restatement of the SimFerrofluid ghost-fluid pressure projection and the FDM
 * magnetostatic potential solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests, the smoke check and the CPU-baseline leg of the
 * benchmark call it to check (or time beside) the CUDA library.  Nothing in the product links it.
 *
 * Parity status: pinned to the reference's own code.  The reference ships no tests or golden vectors, so its
 * hot-path sources (core/Pressure.cpp, MagneticField.cpp, Collider.cpp, FastMarching.cpp, Extrapolation.cpp,
 * Reinitialization.cpp, CSG.cpp, Advection.h, TriLerp.h, TriCuInterp.h) are compiled unmodified into
 * oracle/_ref (oracle/ref.mk, with stand-in headers for Eigen, TBB, fmt/spdlog, yaml-cpp and the amgcl solver
 * call), and tests/test_ref_pin.py requires every function here to reproduce their outputs bit for bit: on the
 * committed fixtures tests/golden/ref_*.npz (written from oracle/_ref by tests/golden/make_ref_golden.py) and,
 * where the sources are present, on further seeded inputs against the live reference code.  Not compiled:
 * amgcl's solver (absent; the oracle solves the same systems tightly instead) and the jump producer of
 * core/Simulation.cpp:216-235 (or_pressure_jump; it needs the whole Simulation/Contour).
 *
 * Floating point: compiled with -ffp-contract=off so that every a*b+c rounds twice, as in the reference's
 * x86 build; the assembly loops evaluate each expression in the reference's order so that the CSR matrix
 * and right-hand side are bit-identical to what the reference assembles from the same inputs.
 *
 * Layout (core/Grid.h:28): cell (i,j,k) -> k + nz*(j + ny*i), z fastest.  Face grid of axis a has size
 * res + e_a (core/StaggeredGrid.h:16-20) with the same z-fastest indexing.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int nx, ny, nz;
    double h;
    double ox, oy, oz; /* staggered-grid corner (StaggeredGrid::GetOrigin) */
} or_grid;

static inline int64_t cidx(const or_grid *g, int i, int j, int k) {
    return (int64_t)k + (int64_t)g->nz * ((int64_t)j + (int64_t)g->ny * i);
}
static inline void fdims(const or_grid *g, int a, int *fx, int *fy, int *fz) {
    *fx = g->nx + (a == 0);
    *fy = g->ny + (a == 1);
    *fz = g->nz + (a == 2);
}
static inline int64_t fidx(const or_grid *g, int a, int i, int j, int k) {
    int fx, fy, fz;
    fdims(g, a, &fx, &fy, &fz);
    (void)fx;
    return (int64_t)k + (int64_t)fz * ((int64_t)j + (int64_t)fy * i);
}
static inline int cell_valid(const or_grid *g, int i, int j, int k) {
    return i >= 0 && j >= 0 && k >= 0 && i < g->nx && j < g->ny && k < g->nz;
}
/* Grid::NeighborOf / StaggeredGrid::FaceOfCell, FaceSideOfCell (core/Grid.h:37-40, core/StaggeredGrid.h:55-57):
 * ord 0..5 = (-x,+x,-y,+y,-z,+z); face of cell = cell + e_axis*(ord&1); side = ord&1 ? +1 : -1. */
static const int NB[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};

int or_version(void) { return 3; }

/* ------------------------------------------------------------------------------------------------------------
 * Pressure::SetUnKnowns (core/Pressure.cpp:104-123): liquid = phi <= 0, numbered in (x,y,z) lexicographic
 * order.  Returns n; fills grid2mat (N, -1 = air) and mat2grid (n).
 * ---------------------------------------------------------------------------------------------------------- */
int64_t or_pressure_unknowns(const or_grid *g, const double *phi, int32_t *grid2mat, int64_t *mat2grid) {
    int64_t n = 0, N = (int64_t)g->nx * g->ny * g->nz;
    for (int64_t c = 0; c < N; c++) {
        if (phi[c] <= 0) {
            grid2mat[c] = (int32_t)n;
            mat2grid[n++] = c;
        } else {
            grid2mat[c] = -1;
        }
    }
    return n;
}

/* Faces on the outer boundary of the grid have no cell on their far side.  The reference reads outside its
 * arrays when such a face is open (weight > 0); this restatement, like the CUDA library, treats them as
 * closed walls (weight 0).  The shipped scenes and every test scene have fraction 1 there. */
static inline double face_weight(const or_grid *g, const double *const frac[3], int a, int i, int j, int k,
                                 int ord) {
    int ni = i + NB[ord][0], nj = j + NB[ord][1], nk = k + NB[ord][2];
    if (!cell_valid(g, ni, nj, nk)) return 0.0;
    int fi = i + (a == 0) * (ord & 1), fj = j + (a == 1) * (ord & 1), fk = k + (a == 2) * (ord & 1);
    return 1.0 - frac[a][fidx(g, a, fi, fj, fk)];
}

/* ------------------------------------------------------------------------------------------------------------
 * Pressure::BuildProjectionMatrix (core/Pressure.cpp:38-78).  CSR with ascending columns per row (Eigen's
 * setFromTriplets order).  jump[a] is the per-face value J(axis, face, theta) of the reference's pressure-jump
 * callback (core/Pressure.h:20-22); the shipped callback ignores theta (core/Simulation.cpp:216-235).
 * us (solid velocity) and jump may be NULL (zero / no callback).  rowptr has n+1 entries; col/val up to 7n.
 * ---------------------------------------------------------------------------------------------------------- */
int64_t or_pressure_assemble(const or_grid *g, const double *phi, const double *const frac[3],
                             const double *const u[3], const double *const us[3], const double *const jump[3],
                             double volError, const int32_t *grid2mat, const int64_t *mat2grid, int64_t n,
                             int64_t *rowptr, int32_t *col, double *val, double *rhs) {
    int64_t nnz = 0;
    rowptr[0] = 0;
    for (int64_t r = 0; r < n; r++) {
        int64_t c = mat2grid[r];
        int i = (int)(c / g->nz / g->ny), j = (int)(c / g->nz % g->ny), k = (int)(c % g->nz);
        double diag = 0, div = 0;
        int32_t cc[7];
        double cv[7];
        int m = 0;
        for (int ord = 0; ord < 6; ord++) {
            int a = ord >> 1, side = (ord & 1) ? 1 : -1;
            int fi = i + (a == 0) * (ord & 1), fj = j + (a == 1) * (ord & 1), fk = k + (a == 2) * (ord & 1);
            int ni = i + NB[ord][0], nj = j + NB[ord][1], nk = k + NB[ord][2];
            double w = face_weight(g, frac, a, i, j, k, ord);
            int64_t f = fidx(g, a, fi, fj, fk);
            if (w > 0) {
                int64_t nb = cidx(g, ni, nj, nk);
                int32_t cn = grid2mat[nb];
                if (cn >= 0) {
                    diag += w;
                    cc[m] = cn;
                    cv[m] = -w;
                    m++;
                } else {
                    double theta = phi[c] / (phi[c] - phi[nb]);
                    double ic = 1. / (theta < .001 ? .001 : theta); /* std::max(theta, .001) */
                    diag += w * ic;
                    if (jump) div += jump[a][f] * w * ic;
                }
                div -= (double)side * w * u[a][f];
            }
            if (w < 1) {
                double usv = us ? us[a][f] : 0.0;
                div -= (double)side * (1 - w) * usv;
            }
        }
        div += volError;
        rhs[r] = div;
        cc[m] = (int32_t)r;
        cv[m] = diag != 0 ? diag : 1.;
        m++;
        /* insertion sort by column */
        for (int x = 1; x < m; x++) {
            int32_t kc = cc[x];
            double kv = cv[x];
            int y = x - 1;
            while (y >= 0 && cc[y] > kc) {
                cc[y + 1] = cc[y];
                cv[y + 1] = cv[y];
                y--;
            }
            cc[y + 1] = kc;
            cv[y + 1] = kv;
        }
        for (int x = 0; x < m; x++) {
            col[nnz] = cc[x];
            val[nnz] = cv[x];
            nnz++;
        }
        rowptr[r + 1] = nnz;
    }
    return nnz;
}

/* Pressure::SetRightHandSide (core/Pressure.cpp:80-102): divergence + solid + volError, no jump terms. */
void or_pressure_rhs(const or_grid *g, const double *const frac[3], const double *const u[3],
                     const double *const us[3], double volError, const int64_t *mat2grid, int64_t n, double *rhs) {
    for (int64_t r = 0; r < n; r++) {
        int64_t c = mat2grid[r];
        int i = (int)(c / g->nz / g->ny), j = (int)(c / g->nz % g->ny), k = (int)(c % g->nz);
        double div = 0;
        for (int ord = 0; ord < 6; ord++) {
            int a = ord >> 1, side = (ord & 1) ? 1 : -1;
            int fi = i + (a == 0) * (ord & 1), fj = j + (a == 1) * (ord & 1), fk = k + (a == 2) * (ord & 1);
            double w = face_weight(g, frac, a, i, j, k, ord);
            int64_t f = fidx(g, a, fi, fj, fk);
            if (w > 0) div -= (double)side * w * u[a][f];
            if (w < 1) {
                double usv = us ? us[a][f] : 0.0;
                div -= (double)side * (1 - w) * usv;
            }
        }
        div += volError;
        rhs[r] = div;
    }
}

/* ------------------------------------------------------------------------------------------------------------
 * Pressure::ApplyProjection (core/Pressure.cpp:137-166).  p is the reduced (liquid-only) solution.
 * ---------------------------------------------------------------------------------------------------------- */
void or_pressure_apply(const or_grid *g, const double *phi, const double *const frac[3], const double *const jump[3],
                       const int32_t *grid2mat, const double *p, double *const u[3]) {
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
#pragma omp parallel for collapse(2) schedule(static)
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    int64_t f = fidx(g, a, i, j, k);
                    /* AdjCellOfFace(axis, face, 0) = face - e_axis, (.., 1) = face */
                    int i0 = i - (a == 0), j0 = j - (a == 1), k0 = k - (a == 2);
                    if (!cell_valid(g, i0, j0, k0) || !cell_valid(g, i, j, k)) continue; /* closed wall */
                    double w = 1. - frac[a][f];
                    if (w == 0.) continue;
                    int64_t c0 = cidx(g, i0, j0, k0), c1 = cidx(g, i, j, k);
                    int32_t id0 = grid2mat[c0], id1 = grid2mat[c1];
                    if (id0 < 0 && id1 < 0) continue;
                    if (id0 >= 0 && id1 >= 0) {
                        u[a][f] -= (p[id1] - p[id0]) * w;
                    } else {
                        double phi0 = phi[c0], phi1 = phi[c1];
                        double theta = phi0 / (phi0 - phi1);
                        double pin = id0 >= 0 ? p[id0] : p[id1];
                        double pj = jump ? jump[a][f] : 0.;
                        double t = id0 >= 0 ? theta : 1 - theta;
                        double ic = 1. / (t < .001 ? .001 : t);
                        u[a][f] -= (id0 >= 0 ? +1 : -1) * (pj - pin) * ic * w;
                    }
                }
    }
}

/* ------------------------------------------------------------------------------------------------------------
 * Magnetic field (core/MagneticField.cpp, core/MagneticField.h:44-54, core/TriLerp.h:22-67).
 * The solve grid is a boundary-width-0 staggered grid whose center is origin + res*h/2 of the simulation
 * grid (core/MagneticField.cpp:13-16); its corner is recomputed from that center exactly as the reference
 * does, so it can differ from the simulation corner in the last bit.
 * ---------------------------------------------------------------------------------------------------------- */
static double heaviside(double phi, double bw) {
    const double pi = 3.141592653589793238462643383279502884;
    if (phi < -bw) return 0.;
    if (phi > bw) return 1.;
    return .5 * (1. + phi / bw + sin(pi * phi / bw) / pi);
}

/* TriLerp::Interpolate(levelSet, pos) with Grid::CalcLower<1>, CalcLowerFrac and clamped At(). */
static double trilerp_cell(const or_grid *g, const double *phi, double px, double py, double pz) {
    double co[3] = {g->ox + g->h / 2, g->oy + g->h / 2, g->oz + g->h / 2}; /* cell grid origin */
    double invh = 1 / g->h;
    double p[3] = {px, py, pz};
    int lo[3];
    double fr[3];
    int sz[3] = {g->nx, g->ny, g->nz};
    for (int a = 0; a < 3; a++) {
        lo[a] = (int)floor((p[a] - co[a]) * invh - 0.0);
        fr[a] = (p[a] - co[a] - (double)lo[a] * g->h) * invh;
    }
    double w[2][3];
    for (int a = 0; a < 3; a++) {
        w[0][a] = 1. - fr[a];
        w[1][a] = fr[a];
    }
    double val = 0;
    for (int q = 0; q < 8; q++) {
        int dx = q & 1, dy = (q >> 1) & 1, dz = (q >> 2) & 1;
        int ci[3] = {lo[0] + dx, lo[1] + dy, lo[2] + dz};
        for (int a = 0; a < 3; a++) ci[a] = ci[a] < 0 ? 0 : (ci[a] > sz[a] - 1 ? sz[a] - 1 : ci[a]);
        double wt = w[dx][0] * w[dy][1] * w[dz][2];
        val += phi[cidx(g, ci[0], ci[1], ci[2])] * wt;
    }
    return val;
}

void or_magnetic_grid_origin(const or_grid *g, double out[3]) {
    int res[3] = {g->nx, g->ny, g->nz};
    double o[3] = {g->ox, g->oy, g->oz};
    for (int a = 0; a < 3; a++) {
        double half = (double)res[a] * g->h / 2.;
        double center = o[a] + half;
        out[a] = center - (double)res[a] * g->h / 2;
    }
}

/* BuildMatrix coefficient pass (core/MagneticField.cpp:51-60): mu on every face; 1 on boundary faces. */
void or_magnetic_coeff(const or_grid *g, const double *phi, double chi, double bw, double *const mu[3]) {
    double eo[3];
    or_magnetic_grid_origin(g, eo);
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
        int res_a = a == 0 ? g->nx : (a == 1 ? g->ny : g->nz);
        double fo[3] = {eo[0] + (a == 0 ? 0 : 1) * g->h / 2, eo[1] + (a == 1 ? 0 : 1) * g->h / 2,
                        eo[2] + (a == 2 ? 0 : 1) * g->h / 2};
#pragma omp parallel for collapse(2) schedule(static)
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    int fa = a == 0 ? i : (a == 1 ? j : k);
                    int64_t f = fidx(g, a, i, j, k);
                    if (fa <= 0 || fa >= res_a) {
                        mu[a][f] = 1.;
                    } else {
                        double px = fo[0] + (double)i * g->h, py = fo[1] + (double)j * g->h,
                               pz = fo[2] + (double)k * g->h;
                        mu[a][f] = 1. + (1. - heaviside(trilerp_cell(g, phi, px, py, pz), bw)) * chi;
                    }
                }
    }
}

/* BuildMatrix matrix pass (core/MagneticField.cpp:62-90): row 0 pinned, column 0 dropped, Neumann walls. */
int64_t or_magnetic_assemble(const or_grid *g, const double *const mu[3], int64_t *rowptr, int32_t *col,
                             double *val) {
    int64_t N = (int64_t)g->nx * g->ny * g->nz, nnz = 0;
    rowptr[0] = 0;
    for (int64_t r = 0; r < N; r++) {
        if (r == 0) {
            col[nnz] = 0;
            val[nnz] = 1.;
            nnz++;
            rowptr[1] = nnz;
            continue;
        }
        int i = (int)(r / g->nz / g->ny), j = (int)(r / g->nz % g->ny), k = (int)(r % g->nz);
        double diag = 0.;
        int32_t cc[7];
        double cv[7];
        int m = 0;
        for (int ord = 0; ord < 6; ord++) {
            int ni = i + NB[ord][0], nj = j + NB[ord][1], nk = k + NB[ord][2];
            if (!cell_valid(g, ni, nj, nk)) continue;
            int a = ord >> 1;
            int fi = i + (a == 0) * (ord & 1), fj = j + (a == 1) * (ord & 1), fk = k + (a == 2) * (ord & 1);
            double w = mu[a][fidx(g, a, fi, fj, fk)];
            int64_t cn = cidx(g, ni, nj, nk);
            if (cn != 0) {
                cc[m] = (int32_t)cn;
                cv[m] = -w;
                m++;
            }
            diag += w;
        }
        cc[m] = (int32_t)r;
        cv[m] = diag;
        m++;
        for (int x = 1; x < m; x++) {
            int32_t kc = cc[x];
            double kv = cv[x];
            int y = x - 1;
            while (y >= 0 && cc[y] > kc) {
                cc[y + 1] = cc[y];
                cv[y + 1] = cv[y];
                y--;
            }
            cc[y + 1] = kc;
            cv[y + 1] = kv;
        }
        for (int x = 0; x < m; x++) {
            col[nnz] = cc[x];
            val[nnz] = cv[x];
            nnz++;
        }
        rowptr[r + 1] = nnz;
    }
    return nnz;
}

/* AssembleRHS (core/MagneticField.cpp:97-118).  rhs[0] = 0 as in the reference.  If rhs0_neumann is not NULL
 * it receives the value row 0 would have had without the pin (used to check the compatibility identity). */
void or_magnetic_rhs(const or_grid *g, const double *const mu[3], const double *const hext[3], double *rhs,
                     double *rhs0_neumann) {
    int64_t N = (int64_t)g->nx * g->ny * g->nz;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < N; r++) {
        int i = (int)(r / g->nz / g->ny), j = (int)(r / g->nz % g->ny), k = (int)(r % g->nz);
        double b = 0;
        for (int ord = 0; ord < 6; ord++) {
            int ni = i + NB[ord][0], nj = j + NB[ord][1], nk = k + NB[ord][2];
            if (!cell_valid(g, ni, nj, nk)) continue;
            int a = ord >> 1, side = (ord & 1) ? 1 : -1;
            int fi = i + (a == 0) * (ord & 1), fj = j + (a == 1) * (ord & 1), fk = k + (a == 2) * (ord & 1);
            int64_t f = fidx(g, a, fi, fj, fk);
            double w = mu[a][f];
            b += (w - 1.) * hext[a][f] * (double)(-side) * g->h;
        }
        if (r == 0) {
            if (rhs0_neumann) *rhs0_neumann = b;
            rhs[r] = 0;
        } else {
            rhs[r] = b;
        }
    }
}

/* AssignTotalField (core/MagneticField.cpp:125-143): H = (psi_c0 - psi_c1)/h + Hext, Hext on boundary faces. */
void or_magnetic_total_field(const or_grid *g, const double *psi, const double *const hext[3], double *const H[3]) {
    double invh = 1 / g->h;
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
#pragma omp parallel for collapse(2) schedule(static)
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    int64_t f = fidx(g, a, i, j, k);
                    int i0 = i - (a == 0), j0 = j - (a == 1), k0 = k - (a == 2);
                    double v = 0.;
                    if (cell_valid(g, i0, j0, k0) && cell_valid(g, i, j, k))
                        v = (psi[cidx(g, i0, j0, k0)] - psi[cidx(g, i, j, k)]) * invh;
                    v += hext[a][f];
                    H[a][f] = v;
                }
    }
}

/* ------------------------------------------------------------------------------------------------------------
 * CSR helpers and an FP64 Jacobi-preconditioned CG used to produce the reference solution of a restated
 * system to a tight tolerance.
 * ---------------------------------------------------------------------------------------------------------- */
void or_csr_spmv(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val, const double *x,
                 double *y) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; r++) {
        double s = 0;
        for (int64_t e = rowptr[r]; e < rowptr[r + 1]; e++) s += val[e] * x[col[e]];
        y[r] = s;
    }
}

static double dotp(int64_t n, const double *a, const double *b) {
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* Returns iterations (negative if not converged).  x is the initial guess on entry.  Stops on
 * ||b - A x|| <= tol * ||b||. */
int or_csr_pcg(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val, const double *b,
               double *x, double tol, int maxit, double *relres_out) {
    double *r = malloc(sizeof(double) * n), *z = malloc(sizeof(double) * n), *p = malloc(sizeof(double) * n),
           *q = malloc(sizeof(double) * n), *dinv = malloc(sizeof(double) * n);
    for (int64_t i = 0; i < n; i++) {
        double d = 0;
        for (int64_t e = rowptr[i]; e < rowptr[i + 1]; e++)
            if (col[e] == i) d = val[e];
        dinv[i] = d != 0 ? 1.0 / d : 1.0;
    }
    or_csr_spmv(n, rowptr, col, val, x, q);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) r[i] = b[i] - q[i];
    double nb = sqrt(dotp(n, b, b));
    if (nb == 0) nb = 1;
    double rr = sqrt(dotp(n, r, r));
    int it = 0;
    if (rr / nb <= tol) goto done;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        z[i] = dinv[i] * r[i];
        p[i] = z[i];
    }
    double rz = dotp(n, r, z);
    for (it = 1; it <= maxit; it++) {
        or_csr_spmv(n, rowptr, col, val, p, q);
        double alpha = rz / dotp(n, p, q);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        rr = sqrt(dotp(n, r, r));
        if (rr / nb <= tol) break;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) z[i] = dinv[i] * r[i];
        double rz2 = dotp(n, r, z);
        double beta = rz2 / rz;
        rz = rz2;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    }
done:
    /* true residual */
    or_csr_spmv(n, rowptr, col, val, x, q);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) r[i] = b[i] - q[i];
    if (relres_out) *relres_out = sqrt(dotp(n, r, r)) / nb;
    free(r);
    free(z);
    free(p);
    free(q);
    free(dinv);
    return it > maxit ? -maxit : it;
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------------------------------------------
 * Collider inputs of the pressure solve (core/Collider.cpp:8-19,21-45,47-73): the node level set of the domain
 * box walls, FastMarching::Solve(LevelSet, -1) (core/FastMarching.cpp:25-62) and the per-face solid fraction.
 * bw is the staggered grid's boundary width; the domain box is [origin + bw*h, origin + (res - bw)*h].
 * ---------------------------------------------------------------------------------------------------------- */
typedef struct {
    double v;
    int64_t i;
} heap_el;
typedef struct {
    heap_el *a;
    int64_t n, cap;
} heap_t;
static int hless(heap_el x, heap_el y) { return x.v < y.v || (x.v == y.v && x.i < y.i); }
static void hpush(heap_t *h, double v, int64_t i) {
    if (h->n == h->cap) {
        h->cap = h->cap ? h->cap * 2 : 1024;
        h->a = realloc(h->a, sizeof(heap_el) * h->cap);
    }
    int64_t c = h->n++;
    heap_el e = {v, i};
    while (c > 0) {
        int64_t p = (c - 1) / 2;
        if (!hless(e, h->a[p])) break;
        h->a[c] = h->a[p];
        c = p;
    }
    h->a[c] = e;
}
static heap_el hpop(heap_t *h) {
    heap_el top = h->a[0], last = h->a[--h->n];
    int64_t c = 0;
    for (;;) {
        int64_t l = 2 * c + 1, r = l + 1, m = c;
        heap_el best = last;
        if (l < h->n && hless(h->a[l], best)) {
            m = l;
            best = h->a[l];
        }
        if (r < h->n && hless(h->a[r], best)) m = r;
        if (m == c) break;
        h->a[c] = h->a[m];
        c = m;
    }
    if (h->n > 0) h->a[c] = last;
    return top;
}
static inline double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min(a, b) */

static double sq2(double p0, double p1, double dx) { /* SolveQuadratic(p0, p1, dx) */
    if (p0 > p1) {
        double t = p0;
        p0 = p1;
        p1 = t;
    }
    if (isinf(p1) || p1 - p0 > dx) return p0 + dx;
    return ((p0 + p1) + sqrt(2 * dx * dx - (p0 - p1) * (p0 - p1))) * .5;
}
static double sq3(double p0, double p1, double p2, double dx) { /* SolveQuadratic(p0, p1, p2, dx) */
    double t;
    if (p0 > p1) { t = p0; p0 = p1; p1 = t; }
    if (p1 > p2) { t = p1; p1 = p2; p2 = t; }
    if (isinf(p2) || (p2 - p0) * (p2 - p0) + (p2 - p1) * (p2 - p1) > dx * dx) return sq2(p0, p1, dx);
    return (p0 + p1 + p2 + sqrt((p0 + p1 + p2) * (p0 + p1 + p2) - 3 * (p0 * p0 + p1 * p1 + p2 * p2 - dx * dx))) / 3;
}

typedef struct {
    int sx, sy, sz;
    double h;
} ngrid;
static inline int nvalid(const ngrid *g, int i, int j, int k) {
    return i >= 0 && j >= 0 && k >= 0 && i < g->sx && j < g->sy && k < g->sz;
}
static inline int64_t nidx(const ngrid *g, int i, int j, int k) {
    return (int64_t)k + (int64_t)g->sz * ((int64_t)j + (int64_t)g->sy * i);
}
static double eikonal(const ngrid *g, int i, int j, int k, const int8_t *vis, const double *tent) {
    double tp[3] = {INFINITY, INFINITY, INFINITY};
    for (int ord = 0; ord < 6; ord++) {
        int ni = i + NB[ord][0], nj = j + NB[ord][1], nk = k + NB[ord][2];
        if (nvalid(g, ni, nj, nk) && vis[nidx(g, ni, nj, nk)]) tp[ord >> 1] = dmin(tp[ord >> 1], tent[nidx(g, ni, nj, nk)]);
    }
    return sq3(tp[0], tp[1], tp[2], g->h);
}
static void update_nbs(const ngrid *g, int i, int j, int k, const int8_t *vis, double *tent, heap_t *hp) {
    for (int ord = 0; ord < 6; ord++) {
        int ni = i + NB[ord][0], nj = j + NB[ord][1], nk = k + NB[ord][2];
        if (!nvalid(g, ni, nj, nk)) continue;
        int64_t nb = nidx(g, ni, nj, nk);
        if (vis[nb]) continue;
        double t = eikonal(g, ni, nj, nk, vis, tent);
        if (t < tent[nb]) {
            tent[nb] = t;
            hpush(hp, t, nb);
        }
    }
}

/* FastMarching::Solve(phi, maxSteps <= 0): full-grid redistancing of a node level set. */
void or_fast_marching(int sx, int sy, int sz, double h, double *phi) {
    ngrid g = {sx, sy, sz, h};
    int64_t M = (int64_t)sx * sy * sz;
    int8_t *vis = calloc(M, 1);
    double *tent = malloc(sizeof(double) * M);
    int64_t *intf = malloc(sizeof(int64_t) * M), nintf = 0;
    heap_t hp = {0, 0, 0};
    for (int64_t c = 0; c < M; c++) tent[c] = INFINITY;
    for (int i = 0; i < sx; i++)
        for (int j = 0; j < sy; j++)
            for (int k = 0; k < sz; k++) {
                int64_t c = nidx(&g, i, j, k);
                double tp[3] = {INFINITY, INFINITY, INFINITY};
                for (int ord = 0; ord < 6; ord++) {
                    int ni = i + NB[ord][0], nj = j + NB[ord][1], nk = k + NB[ord][2];
                    if (!nvalid(&g, ni, nj, nk)) continue;
                    int64_t nb = nidx(&g, ni, nj, nk);
                    if (phi[c] * phi[nb] <= 0) tp[ord >> 1] = dmin(tp[ord >> 1], phi[c] / (phi[c] - phi[nb]) * h);
                }
                if (isfinite(tp[0]) || isfinite(tp[1]) || isfinite(tp[2])) {
                    double a = 1. / tp[0], b = 1. / tp[1], d = 1. / tp[2];
                    tent[c] = 1. / sqrt((a * a + b * b) + d * d);
                    vis[c] = 1;
                    intf[nintf++] = c;
                }
            }
    for (int64_t q = 0; q < nintf; q++) {
        int64_t c = intf[q];
        update_nbs(&g, (int)(c / sz / sy), (int)(c / sz % sy), (int)(c % sz), vis, tent, &hp);
    }
    while (hp.n > 0) {
        heap_el e = hpop(&hp);
        if (tent[e.i] != e.v) continue;
        vis[e.i] = 1;
        update_nbs(&g, (int)(e.i / sz / sy), (int)(e.i / sz % sy), (int)(e.i % sz), vis, tent, &hp);
    }
    for (int64_t c = 0; c < M; c++) phi[c] = (phi[c] <= 0 ? -1 : 1) * tent[c];
    free(vis);
    free(tent);
    free(intf);
    free(hp.a);
}

/* ImplicitBox::SignedDistanceTo (core/ImplicitSurface.h:82-111). */
static double box_sdf(const double c[3], const double hl[3], const double p[3]) {
    double q[3];
    int inside = 1;
    for (int a = 0; a < 3; a++) {
        q[a] = fabs(p[a] - c[a]) - hl[a];
        if (!(q[a] <= 0)) inside = 0;
    }
    if (inside) {
        double m = q[0];
        if (q[1] > m) m = q[1];
        if (q[2] > m) m = q[2];
        return m;
    }
    double s = 0;
    double t[3];
    for (int a = 0; a < 3; a++) t[a] = q[a] > 0 ? q[a] : 0;
    s = (t[0] * t[0] + t[1] * t[1]) + t[2] * t[2];
    return sqrt(s);
}

/* Collider ctor node level set (core/Collider.cpp:14-18): LS = -0.01 h - sdf_box(node). */
void or_collider_box_levelset(const or_grid *g, int bw, double *ls) {
    int sx = g->nx + 1, sy = g->ny + 1, sz = g->nz + 1;
    int res[3] = {g->nx, g->ny, g->nz};
    double o[3] = {g->ox, g->oy, g->oz};
    double c[3], hl[3];
    for (int a = 0; a < 3; a++) {
        double mn = o[a] + (double)bw * g->h;
        double len = (double)(res[a] - bw * 2) * g->h;
        c[a] = mn + len / 2;
        hl[a] = len / 2;
    }
    for (int i = 0; i < sx; i++)
        for (int j = 0; j < sy; j++)
            for (int k = 0; k < sz; k++) {
                double p[3] = {o[0] + (double)i * g->h, o[1] + (double)j * g->h, o[2] + (double)k * g->h};
                ls[(int64_t)k + (int64_t)sz * ((int64_t)j + (int64_t)sy * i)] = -.01 * g->h - box_sdf(c, hl, p);
            }
}

static double tri_fraction(double p0, double p1, double p2) {
    double t;
    if (p0 > p1) { t = p0; p0 = p1; p1 = t; }
    if (p1 > p2) { t = p1; p1 = p2; p2 = t; }
    if (p0 > p1) { t = p0; p0 = p1; p1 = t; }
    if (p2 <= 0) return 1.;
    if (p1 <= 0) return 1. - (p2 / (p2 - p0)) * (p2 / (p2 - p1));
    if (p0 <= 0) return (p0 / (p0 - p1)) * (p0 / (p0 - p2));
    return 0.;
}

/* Collider::CalcFaceFraction (core/Collider.cpp:47-73) over all faces of the three face grids. */
void or_collider_face_fractions(const or_grid *g, const double *ls, double *const frac[3]) {
    int sy = g->ny + 1, sz = g->nz + 1;
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
        int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
#pragma omp parallel for collapse(2) schedule(static)
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    double p[4];
                    for (int q = 0; q < 4; q++) {
                        int n[3] = {i, j, k};
                        n[b1] += q & 1;
                        n[b2] += (q >> 1) & 1;
                        p[q] = ls[(int64_t)n[2] + (int64_t)sz * ((int64_t)n[1] + (int64_t)sy * n[0])];
                    }
                    double cp = (p[0] + p[1] + p[2] + p[3]) * .25;
                    double ff = (tri_fraction(cp, p[0], p[1]) + tri_fraction(cp, p[1], p[3]) +
                                 tri_fraction(cp, p[3], p[2]) + tri_fraction(cp, p[2], p[0])) * .25;
                    frac[a][fidx(g, a, i, j, k)] = ff > .9 ? 1. : ff;
                }
    }
}

/* ------------------------------------------------------------------------------------------------------------
 * Post-projection velocity pipeline (core/Simulation.cpp:237-241).
 * ---------------------------------------------------------------------------------------------------------- */

/* Validity of a face for the extrapolation (core/Simulation.cpp:237-240): fraction < 1 and one of the two
 * adjacent cells (AdjCellOfFace, core/StaggeredGrid.h:58: face - e_a and face) is liquid.  A cell outside the
 * grid counts as not liquid (the reference reads outside its array there; shipped scenes never reach it
 * because their boundary faces have fraction 1). */
static int face_valid_init(const or_grid *g, const double *phi, const double *const frac[3], int a, int i, int j,
                           int k) {
    if (!(frac[a][fidx(g, a, i, j, k)] < 1)) return 0;
    int c0[3] = {i, j, k};
    c0[a] -= 1;
    int l0 = cell_valid(g, c0[0], c0[1], c0[2]) && phi[cidx(g, c0[0], c0[1], c0[2])] <= 0;
    int l1 = cell_valid(g, i, j, k) && phi[cidx(g, i, j, k)] <= 0;
    return l0 || l1;
}

/* Extrapolation::Solve (core/Extrapolation.cpp:4-30) on each face grid: max_steps sweeps; an invalid face with
 * valid neighbours (6-neighbourhood on its own face grid, order -x,+x,-y,+y,-z,+z) takes their mean and becomes
 * valid for the next sweep, one without takes clear_val.  Valid faces are never written within a sweep, so the
 * in-place update reads only values of the previous sweep. */
void or_extrapolate_velocity(const or_grid *g, double *const u[3], const double *phi, const double *const frac[3],
                             double clear_val, int max_steps) {
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
        int64_t nf = (int64_t)fx * fy * fz;
        uint8_t *valid = (uint8_t *)malloc(nf), *valid1 = (uint8_t *)malloc(nf);
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) valid[fidx(g, a, i, j, k)] = (uint8_t)face_valid_init(g, phi, frac, a, i, j, k);
        memcpy(valid1, valid, nf);
        for (int it = 0; it < max_steps; it++) {
            for (int i = 0; i < fx; i++)
                for (int j = 0; j < fy; j++)
                    for (int k = 0; k < fz; k++) {
                        int64_t f = fidx(g, a, i, j, k);
                        if (!valid[f]) {
                            int cnt = 0;
                            double sum = 0;
                            for (int o = 0; o < 6; o++) {
                                int ni = i + NB[o][0], nj = j + NB[o][1], nk = k + NB[o][2];
                                if (ni < 0 || nj < 0 || nk < 0 || ni >= fx || nj >= fy || nk >= fz) continue;
                                int64_t nb = fidx(g, a, ni, nj, nk);
                                if (valid[nb]) {
                                    sum += u[a][nb];
                                    cnt++;
                                }
                            }
                            if (cnt > 0) {
                                u[a][f] = sum / cnt;
                                valid1[f] = 1;
                            } else {
                                u[a][f] = clear_val;
                            }
                        } else {
                            valid1[f] = 1;
                        }
                    }
            uint8_t *t = valid;
            valid = valid1;
            valid1 = t;
        }
        free(valid);
        free(valid1);
    }
}

/* FiniteDiff::CalcFirstDrv on the node grid (core/FiniteDiff.h:9-19, 50-52). */
static double node_drv(const double *ls, int sx, int sy, int sz, int i, int j, int k, int a, double invh) {
    int s3[3] = {sx, sy, sz};
    int c[3] = {i, j, k};
    double f[5];
    for (int o = -2; o <= 2; o++) {
        int q[3] = {i, j, k};
        q[a] += o;
        f[o + 2] = (q[a] >= 0 && q[a] < s3[a]) ? ls[(int64_t)q[2] + (int64_t)sz * ((int64_t)q[1] + (int64_t)sy * q[0])]
                                               : 0.0;
    }
    if (c[a] == 0) return (4 * f[3] - 3 * f[2] - f[4]) * invh * .5;
    if (c[a] + 1 == s3[a]) return (3 * f[2] - 4 * f[1] + f[0]) * invh * .5;
    return (f[3] - f[1]) * invh * .5;
}

/* Collider::Finish normals (core/Collider.cpp:30-44): normal[a] on each face of axis a = mean over the face's 4
 * nodes (NodeOfFace order, core/StaggeredGrid.h:64) of the a-derivative of the node level set. */
void or_collider_face_normals(const or_grid *g, const double *ls, double *const normal[3]) {
    int sx = g->nx + 1, sy = g->ny + 1, sz = g->nz + 1;
    double invh = 1 / g->h;
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
        int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    double sum = 0;
                    for (int q = 0; q < 4; q++) {
                        int n[3] = {i, j, k};
                        n[b1] += q & 1;
                        n[b2] += (q >> 1) & 1;
                        sum += node_drv(ls, sx, sy, sz, n[0], n[1], n[2], a, invh);
                    }
                    normal[a][fidx(g, a, i, j, k)] = sum / 4;
                }
    }
}

/* TriLerp::Interpolate of face grid b (size res + e_b, origin = grid corner + h/2 on the other axes) at p. */
static double trilerp_face(const or_grid *g, const double *v, int b, const double p[3]) {
    double o[3] = {g->ox, g->oy, g->oz};
    int sz3[3] = {g->nx, g->ny, g->nz};
    double co[3];
    int s[3];
    for (int a = 0; a < 3; a++) {
        co[a] = a == b ? o[a] : o[a] + g->h / 2; /* face grid origin (core/StaggeredGrid.h:16-20) */
        s[a] = sz3[a] + (a == b);
    }
    double invh = 1 / g->h;
    int lo[3];
    double fr[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = (int)floor((p[a] - co[a]) * invh - 0.0);
        fr[a] = (p[a] - co[a] - (double)lo[a] * g->h) * invh;
    }
    double w[2][3];
    for (int a = 0; a < 3; a++) {
        w[0][a] = 1. - fr[a];
        w[1][a] = fr[a];
    }
    double val = 0;
    for (int q = 0; q < 8; q++) {
        int dx = q & 1, dy = (q >> 1) & 1, dz = (q >> 2) & 1;
        int ci[3] = {lo[0] + dx, lo[1] + dy, lo[2] + dz};
        for (int a = 0; a < 3; a++) ci[a] = ci[a] < 0 ? 0 : (ci[a] > s[a] - 1 ? s[a] - 1 : ci[a]);
        double wt = w[dx][0] * w[dy][1] * w[dz][2];
        val += v[(int64_t)ci[2] + (int64_t)s[2] * ((int64_t)ci[1] + (int64_t)s[1] * ci[0])] * wt;
    }
    return val;
}

/* Collider::Enforce (core/Collider.cpp:75-86): on faces with fraction == 1 the fluid velocity becomes the
 * interpolated old velocity minus its normal component relative to the solid velocity (us == NULL: zero). */
void or_collider_enforce(const or_grid *g, double *const u[3], const double *const frac[3],
                         const double *const normal[3], const double *const us[3]) {
    double *old[3];
    for (int b = 0; b < 3; b++) {
        int fx, fy, fz;
        fdims(g, b, &fx, &fy, &fz);
        int64_t nf = (int64_t)fx * fy * fz;
        old[b] = (double *)malloc(8 * nf);
        memcpy(old[b], u[b], 8 * nf);
    }
    double o[3] = {g->ox, g->oy, g->oz};
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    int64_t f = fidx(g, a, i, j, k);
                    if (frac[a][f] != 1.) continue;
                    int c3[3] = {i, j, k};
                    double p[3];
                    for (int b = 0; b < 3; b++)
                        p[b] = (b == a ? o[b] : o[b] + g->h / 2) + (double)c3[b] * g->h; /* Grid::PositionOf */
                    double vel[3], vel0[3], n[3];
                    for (int b = 0; b < 3; b++) {
                        vel[b] = trilerp_face(g, old[b], b, p);
                        vel0[b] = us ? trilerp_face(g, us[b], b, p) : 0.0;
                        n[b] = trilerp_face(g, normal[b], b, p);
                    }
                    double nn = sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
                    if (nn > 0)
                        for (int b = 0; b < 3; b++) n[b] = n[b] / nn;
                    double dv[3] = {vel[0] - vel0[0], vel[1] - vel0[1], vel[2] - vel0[2]};
                    double dn = (dv[0] * n[0] + dv[1] * n[1]) + dv[2] * n[2];
                    u[a][f] = vel[a] - dn * n[a];
                }
    }
    for (int b = 0; b < 3; b++) free(old[b]);
}

/* ------------------------------------------------------------------------------------------------------------
 * Interface coupling: vertex magnetic pressures and the pressure jump (core/Simulation.cpp:204-235).
 * ---------------------------------------------------------------------------------------------------------- */

/* MagneticField::CalculateVertexPressures (core/MagneticField.cpp:37-48): H trilinear at each vertex position
 * (TriLerp of the three face grids of the total field), p = mu0/2 chi (|H|^2 + chi^2/(4chi+4) (H.n)^2) with
 * mu0 = 4e-7 pi (core/MagneticField.cpp:7-8).  positions / normals: nverts x 3, row-major. */
void or_vertex_pressures(const or_grid *g, double chi, const double *const H[3], const double *pos,
                         const double *nrm, int64_t nverts, double *out) {
    const double pi = 3.141592653589793238462643383279502884;
    const double mu0 = 4e-7 * pi;
    for (int64_t v = 0; v < nverts; v++) {
        const double *p = pos + 3 * v, *n = nrm + 3 * v;
        double h[3];
        for (int b = 0; b < 3; b++) h[b] = trilerp_face(g, H[b], b, p);
        double coeff = (h[0] * h[0] + h[1] * h[1]) + h[2] * h[2];
        double hn = (h[0] * n[0] + h[1] * n[1]) + h[2] * n[2];
        coeff += chi * chi / (4 * chi + 4) * hn * hn;
        out[v] = mu0 * 0.5 * chi * coeff;
    }
}

/* The pressure-jump callback of core/Simulation.cpp:216-235 evaluated on every face (theta is unused): with the
 * vertex of edge (axis, face - e_axis) (Contour::VertexIndexOf, core/Contour.h:19-21; edge grid of axis a has the
 * cell-grid size minus e_a, entries -1 where no vertex), J = kappa[v] sigma / rho / h dt (when curvature is
 * given) - p_m[v] / rho / h dt (when magnetic pressures are given); 0 without a vertex. */
void or_pressure_jump(const or_grid *g, const int32_t *const edge_mark[3], const double *kappa, const double *pm,
                      double sigma, double rho, double dt, double *const jump[3]) {
    double invh = 1 / g->h;
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
        int ex = g->nx - (a == 0), ey = g->ny - (a == 1), ez = g->nz - (a == 2);
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    int e[3] = {i, j, k};
                    e[a] -= 1;
                    int idx = -1;
                    if (e[0] >= 0 && e[1] >= 0 && e[2] >= 0 && e[0] < ex && e[1] < ey && e[2] < ez)
                        idx = edge_mark[a][(int64_t)e[2] + (int64_t)ez * ((int64_t)e[1] + (int64_t)ey * e[0])];
                    double pressure = 0;
                    if (kappa && idx >= 0) pressure += kappa[idx] * sigma / rho * invh * dt;
                    if (pm && idx >= 0) pressure -= pm[idx] / rho * invh * dt;
                    jump[a][fidx(g, a, i, j, k)] = pressure;
                }
    }
}

/* ------------------------------------------------------------------------------------------------------------
 * Level-set neighbours of the path (core/Simulation.cpp:164-165, 265): semi-Lagrangian advection and
 * WENO5/TVD-RK3 reinitialisation.
 * ---------------------------------------------------------------------------------------------------------- */

static inline double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max(a, b) */

/* TriLerp of the three face grids at p (TriLerp::Interpolate(SGridData), core/TriLerp.h:62-66). */
static void trilerp_flow(const or_grid *g, const double *const u[3], const double p[3], double out[3]) {
    for (int b = 0; b < 3; b++) out[b] = trilerp_face(g, u[b], b, p);
}

/* Advection::Trace<2> (core/Advection.h:15-18): the TVD Runge-Kutta trace of second order from p over dt. */
static void trace_rk2(const or_grid *g, const double *const u[3], const double p[3], double dt, double out[3]) {
    double v0[3], v1[3], q[3];
    trilerp_flow(g, u, p, v0);
    for (int a = 0; a < 3; a++) q[a] = p[a] + v0[a] * dt;
    trilerp_flow(g, u, q, v1);
    for (int a = 0; a < 3; a++) out[a] = p[a] + (v0[a] + v1[a]) * dt / 2;
}

/* TriCuInterp::Interpolate of the cell grid at p (core/TriCuInterp.h:12-37): CalcLower<3> = floor((p - o)/h - 1),
 * cubic Lagrange weights per axis, 64 points in (k, j, i) order, clamped At(). */
static double tricubic_cell(const or_grid *g, const double *f, const double p[3]) {
    double co[3] = {g->ox + g->h / 2, g->oy + g->h / 2, g->oz + g->h / 2};
    int sz[3] = {g->nx, g->ny, g->nz};
    double invh = 1 / g->h;
    int lo[3];
    double w[4][3];
    for (int a = 0; a < 3; a++) {
        lo[a] = (int)floor((p[a] - co[a]) * invh - 1.0);
        double fr = (p[a] - co[a] - (double)lo[a] * g->h) * invh;
        w[0][a] = (fr - 1) * (fr - 2) * (fr - 3) / -6;
        w[1][a] = fr * (fr - 2) * (fr - 3) / 2;
        w[2][a] = fr * (fr - 1) * (fr - 3) / -2;
        w[3][a] = fr * (fr - 1) * (fr - 2) / 6;
    }
    double val = 0;
    for (int k = 0; k < 4; k++)
        for (int j = 0; j < 4; j++)
            for (int i = 0; i < 4; i++) {
                int ci[3] = {lo[0] + i, lo[1] + j, lo[2] + k};
                for (int a = 0; a < 3; a++) ci[a] = ci[a] < 0 ? 0 : (ci[a] > sz[a] - 1 ? sz[a] - 1 : ci[a]);
                val += f[cidx(g, ci[0], ci[1], ci[2])] * (w[i][0] * w[j][1] * w[k][2]);
            }
    return val;
}

/* Advection::Solve<2>(levelSet, velocity, dt) (core/Advection.h:40-49): phi at the RK2 departure point of each
 * cell centre, by tricubic interpolation of the old phi.  phi_out must not alias phi. */
void or_advect_levelset(const or_grid *g, const double *phi, const double *const u[3], double dt, double *phi_out) {
    double co[3] = {g->ox + g->h / 2, g->oy + g->h / 2, g->oz + g->h / 2};
    for (int i = 0; i < g->nx; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                double p[3] = {co[0] + (double)i * g->h, co[1] + (double)j * g->h, co[2] + (double)k * g->h};
                double q[3];
                trace_rk2(g, u, p, -dt, q);
                phi_out[cidx(g, i, j, k)] = tricubic_cell(g, phi, q);
            }
}

/* Advection::Solve<2>(velocity, velocity, dt) (core/Advection.h:51-59): each face value at the RK2 departure
 * point of its face, by trilinear interpolation of its own old face grid.  u_out must not alias u. */
void or_advect_velocity(const or_grid *g, const double *const u[3], double dt, double *const u_out[3]) {
    double o[3] = {g->ox, g->oy, g->oz};
    for (int a = 0; a < 3; a++) {
        int fx, fy, fz;
        fdims(g, a, &fx, &fy, &fz);
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    int c3[3] = {i, j, k};
                    double p[3], q[3];
                    for (int b = 0; b < 3; b++) p[b] = (b == a ? o[b] : o[b] + g->h / 2) + (double)c3[b] * g->h;
                    trace_rk2(g, u, p, -dt, q);
                    u_out[a][fidx(g, a, i, j, k)] = trilerp_face(g, u[a], a, q);
                }
    }
}

/* GetDrv (core/Reinitialization.cpp:4-27): WENO5 one-sided derivatives (minus, plus) from 7 values. */
static void weno_drv(const double v[7], double invdx, double *dm, double *dp) {
    for (int s = 0; s < 2; s++) {
        double dev[5];
        if (s) {
            dev[0] = v[6] - v[5]; dev[1] = v[5] - v[4]; dev[2] = v[4] - v[3]; dev[3] = v[3] - v[2]; dev[4] = v[2] - v[1];
        } else {
            dev[0] = v[1] - v[0]; dev[1] = v[2] - v[1]; dev[2] = v[3] - v[2]; dev[3] = v[4] - v[3]; dev[4] = v[5] - v[4];
        }
        double eps = 0;
        for (int j = 0; j < 5; j++) eps = dmax(eps, dev[j] * dev[j]);
        eps = eps * 1e-6 + 1e-99;
        double phix1 = dev[0] / 3 - dev[1] * 7 / 6 + dev[2] * 11 / 6;
        double phix2 = -dev[1] / 6 + dev[2] * 5 / 6 + dev[3] / 3;
        double phix3 = dev[2] / 3 + dev[3] * 5 / 6 - dev[4] / 6;
        double t;
        t = dev[0] - 2 * dev[1] + dev[2];
        double s1 = t * t * 13 / 12;
        t = dev[0] - 4 * dev[1] + 3 * dev[2];
        s1 = s1 + t * t / 4;
        t = dev[1] - 2 * dev[2] + dev[3];
        double s2 = t * t * 13 / 12;
        t = dev[1] - dev[3];
        s2 = s2 + t * t / 4;
        t = dev[2] - 2 * dev[3] + dev[4];
        double s3 = t * t * 13 / 12;
        t = 3 * dev[2] - 4 * dev[3] + dev[4];
        s3 = s3 + t * t / 4;
        t = s1 + eps;
        double alpha1 = .1 / (t * t);
        t = s2 + eps;
        double alpha2 = .6 / (t * t);
        t = s3 + eps;
        double alpha3 = .3 / (t * t);
        double sum = alpha1 + alpha2 + alpha3;
        double d = (alpha1 * phix1 + alpha2 * phix2 + alpha3 * phix3) / sum * invdx;
        if (s) *dp = d; else *dm = d;
    }
}

/* Reinitialization::Advance (core/Reinitialization.cpp:48-74) into out (must not alias f). */
static void reinit_advance(const or_grid *g, const double *f, double *out, double dt) {
    int sz[3] = {g->nx, g->ny, g->nz};
    double invdx = 1 / g->h;
    for (int i = 0; i < g->nx; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                double dm[3], dp[3];
                for (int a = 0; a < 3; a++) {
                    double v[7];
                    for (int q = 0; q < 7; q++) {
                        int c[3] = {i, j, k};
                        c[a] += q - 3;
                        c[a] = c[a] < 0 ? 0 : (c[a] > sz[a] - 1 ? sz[a] - 1 : c[a]); /* At(): clamped */
                        v[q] = f[cidx(g, c[0], c[1], c[2])];
                    }
                    weno_drv(v, invdx, &dm[a], &dp[a]);
                }
                double fc = f[cidx(g, i, j, k)];
                double sum = 0, t;
                if (fc < 0) {
                    for (int a = 0; a < 3; a++) {
                        t = dm[a] < 0. ? dm[a] : 0.; /* std::min(x, 0.) */
                        sum += t * t;
                        t = dmax(dp[a], 0.);
                        sum += t * t;
                    }
                } else {
                    for (int a = 0; a < 3; a++) {
                        t = dmax(dm[a], 0.);
                        sum += t * t;
                        t = dp[a] < 0. ? dp[a] : 0.;
                        sum += t * t;
                    }
                }
                sum = sqrt(sum);
                double sp = g->h * sum;
                double sgn = fc / sqrt(fc * fc + sp * sp);
                out[cidx(g, i, j, k)] = fc + dt * sgn * (1. - sum);
            }
}

/* Reinitialization::Solve (core/Reinitialization.cpp:36-46): max_steps TVD-RK3 steps with dt = h / 2. */
void or_reinitialize(const or_grid *g, double *phi, int max_steps) {
    int64_t n = (int64_t)g->nx * g->ny * g->nz;
    double *p1 = (double *)malloc(8 * n), *p2 = (double *)malloc(8 * n);
    double dt = g->h * .5;
    for (int it = 0; it < max_steps; it++) {
        reinit_advance(g, phi, p1, dt);
        reinit_advance(g, p1, p2, dt);
        for (int64_t c = 0; c < n; c++) p1[c] = (phi[c] * 3 + p2[c]) / 4;
        reinit_advance(g, p1, p2, dt);
        for (int64_t c = 0; c < n; c++) phi[c] = (phi[c] + p2[c] * 2) / 3;
    }
    free(p1);
    free(p2);
}
