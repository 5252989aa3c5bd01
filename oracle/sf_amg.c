/*
 * sf_amg.c -- CPU restatement of the reference's linear solvers: amgcl's smoothed-aggregation AMG with SPAI-0
 * relaxation, preconditioning BiCGStab (pressure, core/Pressure.cpp:125-135, default parameters) or CG
 * (magnetic potential, core/MagneticField.h:17-21, core/MagneticField.cpp:92-94, tol 1e-6).
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): used as the timed CPU baseline and the reference arm of the
 * benchmark.  amgcl is an unpinned third-party dependency of the reference (xmake.lua:8, no version) and is
 * absent here; this file restates its published algorithm and documented defaults, not its code:
 *   - strength of connection a_ij^2 > eps^2 |a_ii a_jj|, eps_strong = 0.08 halved on every coarser level;
 *   - plain aggregation: a node whose strong neighbours are all free seeds an aggregate with them; remaining
 *     nodes join a neighbouring aggregate; nodes without strong connections stay unaggregated;
 *   - tentative prolongator = aggregate indicator (constant null space), smoothed once with damped Jacobi on
 *     the filtered matrix (weak connections lumped into the diagonal), omega = (4/3) / rho(D^-1 A_f) with rho
 *     bounded by the Gershgorin estimate;
 *   - Galerkin coarse operator R A P with R = P^T;
 *   - SPAI-0 smoother M = diag(a_ii / sum_j a_ij^2), one pre- and one post-sweep, V-cycle;
 *   - coarsest level (<= 3000 unknowns) solved directly (envelope Cholesky after reverse Cuthill-McKee);
 *   - the AMG hierarchy is rebuilt on every solve, as the reference does.
 * Stopping rule of both Krylov solvers: ||r|| <= tol ||b||; a zero right-hand side returns x = 0.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t n;
    int64_t *ptr;
    int32_t *col;
    double *val;
} csr_t;

static void csr_free(csr_t *a) {
    free(a->ptr);
    free(a->col);
    free(a->val);
    memset(a, 0, sizeof(*a));
}

static void spmv(const csr_t *A, const double *x, double *y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A->n; i++) {
        double s = 0;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) s += A->val[e] * x[A->col[e]];
        y[i] = s;
    }
}

static double dot(int64_t n, const double *a, const double *b) {
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* C = A * B (Gustavson, two passes, row-parallel). A: n x k, B: k x m. */
static csr_t spgemm(const csr_t *A, const csr_t *B, int64_t m) {
    csr_t C;
    C.n = A->n;
    C.ptr = calloc(A->n + 1, sizeof(int64_t));
#pragma omp parallel
    {
        int64_t *mark = malloc(sizeof(int64_t) * (m > 0 ? m : 1));
        for (int64_t q = 0; q < m; q++) mark[q] = -1;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < A->n; i++) {
            int64_t cnt = 0;
            for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
                int32_t k = A->col[e];
                for (int64_t f = B->ptr[k]; f < B->ptr[k + 1]; f++) {
                    int32_t j = B->col[f];
                    if (mark[j] != i) {
                        mark[j] = i;
                        cnt++;
                    }
                }
            }
            C.ptr[i + 1] = cnt;
        }
        free(mark);
    }
    for (int64_t i = 0; i < A->n; i++) C.ptr[i + 1] += C.ptr[i];
    C.col = malloc(sizeof(int32_t) * (C.ptr[A->n] > 0 ? C.ptr[A->n] : 1));
    C.val = malloc(sizeof(double) * (C.ptr[A->n] > 0 ? C.ptr[A->n] : 1));
#pragma omp parallel
    {
        int64_t *mark = malloc(sizeof(int64_t) * (m > 0 ? m : 1));
        for (int64_t q = 0; q < m; q++) mark[q] = -1;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < A->n; i++) {
            int64_t beg = C.ptr[i], end = beg;
            for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
                int32_t k = A->col[e];
                double av = A->val[e];
                for (int64_t f = B->ptr[k]; f < B->ptr[k + 1]; f++) {
                    int32_t j = B->col[f];
                    if (mark[j] < beg) {
                        mark[j] = end;
                        C.col[end] = j;
                        C.val[end] = av * B->val[f];
                        end++;
                    } else {
                        C.val[mark[j]] += av * B->val[f];
                    }
                }
            }
        }
        free(mark);
    }
    return C;
}

static csr_t transpose(const csr_t *A, int64_t m) {
    csr_t T;
    T.n = m;
    T.ptr = calloc(m + 1, sizeof(int64_t));
    int64_t nnz = A->ptr[A->n];
    for (int64_t e = 0; e < nnz; e++) T.ptr[A->col[e] + 1]++;
    for (int64_t i = 0; i < m; i++) T.ptr[i + 1] += T.ptr[i];
    T.col = malloc(sizeof(int32_t) * (nnz > 0 ? nnz : 1));
    T.val = malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    int64_t *pos = malloc(sizeof(int64_t) * (m + 1));
    memcpy(pos, T.ptr, sizeof(int64_t) * (m + 1));
    for (int64_t i = 0; i < A->n; i++)
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
            int64_t p = pos[A->col[e]]++;
            T.col[p] = (int32_t)i;
            T.val[p] = A->val[e];
        }
    free(pos);
    return T;
}

static double *diagonal(const csr_t *A) {
    double *d = malloc(sizeof(double) * (A->n > 0 ? A->n : 1));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A->n; i++) {
        d[i] = 0;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++)
            if (A->col[e] == i) d[i] = A->val[e];
    }
    return d;
}

/* ---------------------------------------------------------------------------------------- coarse direct solve */
typedef struct {
    int64_t n;
    int64_t *perm;  /* new -> old */
    int64_t *first; /* first column of row i in the envelope */
    int64_t *off;   /* offset of row i's envelope in L */
    double *L;      /* envelope of the Cholesky factor, row-wise, diagonal last */
} skyline_t;

static void skyline_free(skyline_t *s) {
    free(s->perm);
    free(s->first);
    free(s->off);
    free(s->L);
    memset(s, 0, sizeof(*s));
}

/* reverse Cuthill-McKee from a minimum-degree start, component by component */
static void rcm(const csr_t *A, int64_t *perm) {
    int64_t n = A->n;
    char *seen = calloc(n > 0 ? n : 1, 1);
    int64_t *q = perm, head = 0, tail = 0;
    while (tail < n) {
        int64_t start = -1, best = INT64_MAX;
        for (int64_t i = 0; i < n; i++)
            if (!seen[i] && A->ptr[i + 1] - A->ptr[i] < best) {
                best = A->ptr[i + 1] - A->ptr[i];
                start = i;
            }
        seen[start] = 1;
        q[tail++] = start;
        while (head < tail) {
            int64_t v = q[head++];
            int64_t b = tail;
            for (int64_t e = A->ptr[v]; e < A->ptr[v + 1]; e++) {
                int32_t w = A->col[e];
                if (!seen[w]) {
                    seen[w] = 1;
                    q[tail++] = w;
                }
            }
            /* order the new ones by degree */
            for (int64_t x = b + 1; x < tail; x++) {
                int64_t key = q[x], kd = A->ptr[key + 1] - A->ptr[key], y = x - 1;
                while (y >= b && A->ptr[q[y] + 1] - A->ptr[q[y]] > kd) {
                    q[y + 1] = q[y];
                    y--;
                }
                q[y + 1] = key;
            }
        }
    }
    for (int64_t i = 0; i < n / 2; i++) {
        int64_t t = perm[i];
        perm[i] = perm[n - 1 - i];
        perm[n - 1 - i] = t;
    }
    free(seen);
}

static int skyline_factor(const csr_t *A, skyline_t *s) {
    int64_t n = A->n;
    s->n = n;
    s->perm = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    rcm(A, s->perm);
    int64_t *inv = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) inv[s->perm[i]] = i;
    s->first = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    s->off = malloc(sizeof(int64_t) * (n + 1));
    for (int64_t i = 0; i < n; i++) {
        int64_t old = s->perm[i], f = i;
        for (int64_t e = A->ptr[old]; e < A->ptr[old + 1]; e++) {
            int64_t j = inv[A->col[e]];
            if (j < f) f = j;
        }
        s->first[i] = f;
    }
    s->off[0] = 0;
    for (int64_t i = 0; i < n; i++) s->off[i + 1] = s->off[i] + (i - s->first[i] + 1);
    s->L = calloc(s->off[n] > 0 ? s->off[n] : 1, sizeof(double));
    for (int64_t i = 0; i < n; i++) {
        int64_t old = s->perm[i];
        for (int64_t e = A->ptr[old]; e < A->ptr[old + 1]; e++) {
            int64_t j = inv[A->col[e]];
            if (j <= i) s->L[s->off[i] + (j - s->first[i])] += A->val[e];
        }
    }
    free(inv);
    /* envelope Cholesky: L[i][j] = (a_ij - sum_k L[i][k] L[j][k]) / L[j][j] */
    for (int64_t i = 0; i < n; i++) {
        double *Li = s->L + s->off[i];
        int64_t fi = s->first[i];
        for (int64_t j = fi; j < i; j++) {
            double *Lj = s->L + s->off[j];
            int64_t fj = s->first[j], k0 = fi > fj ? fi : fj;
            double acc = Li[j - fi];
            for (int64_t k = k0; k < j; k++) acc -= Li[k - fi] * Lj[k - fj];
            Li[j - fi] = acc / Lj[j - fj];
        }
        double d = Li[i - fi];
        for (int64_t k = fi; k < i; k++) d -= Li[k - fi] * Li[k - fi];
        if (!(d > 0)) d = d == 0 ? 1e-300 : fabs(d); /* singular (Neumann) coarse block: regularise */
        Li[i - fi] = sqrt(d);
    }
    return 0;
}

static void skyline_solve(const skyline_t *s, const double *b, double *x, double *w) {
    int64_t n = s->n;
    for (int64_t i = 0; i < n; i++) w[i] = b[s->perm[i]];
    for (int64_t i = 0; i < n; i++) {
        const double *Li = s->L + s->off[i];
        int64_t fi = s->first[i];
        double acc = w[i];
        for (int64_t k = fi; k < i; k++) acc -= Li[k - fi] * w[k];
        w[i] = acc / Li[i - fi];
    }
    for (int64_t i = n - 1; i >= 0; i--) {
        const double *Li = s->L + s->off[i];
        int64_t fi = s->first[i];
        w[i] /= Li[i - fi];
        double wi = w[i];
        for (int64_t k = fi; k < i; k++) w[k] -= Li[k - fi] * wi;
    }
    for (int64_t i = 0; i < n; i++) x[s->perm[i]] = w[i];
}

/* ---------------------------------------------------------------------------------------------- hierarchy */
#define AMG_MAX_LEVELS 32
typedef struct {
    int nlev;
    csr_t A[AMG_MAX_LEVELS], P[AMG_MAX_LEVELS], R[AMG_MAX_LEVELS];
    double *M[AMG_MAX_LEVELS]; /* SPAI-0 diagonal */
    double *x[AMG_MAX_LEVELS], *b[AMG_MAX_LEVELS], *t[AMG_MAX_LEVELS];
    skyline_t coarse;
    double *cw;
    int own_A0;
} amg_t;

static int64_t aggregate(const csr_t *A, const double *d, double eps, int32_t *agg, char *strong) {
    int64_t n = A->n;
    const double eps2 = eps * eps;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++)
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
            int32_t j = A->col[e];
            strong[e] = (j != i) && (A->val[e] * A->val[e] > eps2 * fabs(d[i] * d[j]));
        }
    /* nodes without strong connections are left out (-2); free nodes are -1 */
    for (int64_t i = 0; i < n; i++) {
        int has = 0;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) has |= strong[e];
        agg[i] = has ? -1 : -2;
    }
    int64_t na = 0;
    /* pass 1: root points whose strong neighbourhood is entirely free */
    for (int64_t i = 0; i < n; i++) {
        if (agg[i] != -1) continue;
        int ok = 1;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1] && ok; e++)
            if (strong[e] && agg[A->col[e]] != -1) ok = 0;
        if (!ok) continue;
        agg[i] = (int32_t)na;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++)
            if (strong[e]) agg[A->col[e]] = (int32_t)na;
        na++;
    }
    /* pass 2: join a strongly connected neighbour's aggregate; else start a new one */
    for (int64_t i = 0; i < n; i++) {
        if (agg[i] != -1) continue;
        int32_t a = -1;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++)
            if (strong[e] && agg[A->col[e]] >= 0) {
                a = agg[A->col[e]];
                break;
            }
        if (a < 0) {
            a = (int32_t)na++;
            for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++)
                if (strong[e] && agg[A->col[e]] == -1) agg[A->col[e]] = a;
        }
        agg[i] = a;
    }
    return na;
}

static void spai0(const csr_t *A, double *M) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A->n; i++) {
        double s = 0, d = 0;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
            s += A->val[e] * A->val[e];
            if (A->col[e] == i) d = A->val[e];
        }
        M[i] = s > 0 ? d / s : 0;
    }
}

/* smoothed prolongator P = (I - omega D_f^-1 A_f) P_tent */
static csr_t smoothed_prolongator(const csr_t *A, const char *strong, const int32_t *agg, int64_t na) {
    int64_t n = A->n;
    double *df = malloc(sizeof(double) * (n > 0 ? n : 1));
    double rho = 0;
#pragma omp parallel for schedule(static) reduction(max : rho)
    for (int64_t i = 0; i < n; i++) {
        double dd = 0, rs = 0;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
            int32_t j = A->col[e];
            if (j == i)
                dd += A->val[e];
            else if (!strong[e])
                dd += A->val[e]; /* lumped weak connection */
        }
        df[i] = dd;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
            int32_t j = A->col[e];
            if (j == i)
                rs += fabs(dd);
            else if (strong[e])
                rs += fabs(A->val[e]);
        }
        double r = dd != 0 ? rs / fabs(dd) : 0;
        if (r > rho) rho = r;
    }
    const double omega = (4.0 / 3.0) / (rho > 0 ? rho : 1.0);
    csr_t P;
    P.n = n;
    P.ptr = calloc(n + 1, sizeof(int64_t));
#pragma omp parallel
    {
        int64_t *mark = malloc(sizeof(int64_t) * (na > 0 ? na : 1));
        for (int64_t q = 0; q < na; q++) mark[q] = -1;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            int64_t cnt = 0;
            for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
                int32_t j = A->col[e];
                if ((j == i || strong[e]) && agg[j] >= 0 && mark[agg[j]] != i) {
                    mark[agg[j]] = i;
                    cnt++;
                }
            }
            P.ptr[i + 1] = cnt;
        }
        free(mark);
    }
    for (int64_t i = 0; i < n; i++) P.ptr[i + 1] += P.ptr[i];
    P.col = malloc(sizeof(int32_t) * (P.ptr[n] > 0 ? P.ptr[n] : 1));
    P.val = malloc(sizeof(double) * (P.ptr[n] > 0 ? P.ptr[n] : 1));
#pragma omp parallel
    {
        int64_t *mark = malloc(sizeof(int64_t) * (na > 0 ? na : 1));
        for (int64_t q = 0; q < na; q++) mark[q] = -1;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            int64_t beg = P.ptr[i], end = beg;
            const double s = df[i] != 0 ? omega / df[i] : 0;
            for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
                int32_t j = A->col[e];
                if (!(j == i || strong[e]) || agg[j] < 0) continue;
                double v = (j == i) ? 1.0 - s * df[i] : -s * A->val[e];
                int32_t a = agg[j];
                if (mark[a] < beg) {
                    mark[a] = end;
                    P.col[end] = a;
                    P.val[end] = v;
                    end++;
                } else {
                    P.val[mark[a]] += v;
                }
            }
        }
        free(mark);
    }
    free(df);
    return P;
}

static void amg_free(amg_t *h) {
    for (int l = 0; l < h->nlev; l++) {
        if (l > 0 || h->own_A0) csr_free(&h->A[l]);
        csr_free(&h->P[l]);
        csr_free(&h->R[l]);
        free(h->M[l]);
        free(h->x[l]);
        free(h->b[l]);
        free(h->t[l]);
    }
    skyline_free(&h->coarse);
    free(h->cw);
    memset(h, 0, sizeof(*h));
}

static void amg_setup(amg_t *h, const csr_t *A0) {
    memset(h, 0, sizeof(*h));
    const int64_t coarse_enough = 3000;
    double eps = 0.08;
    h->A[0] = *A0;
    int l = 0;
    for (;;) {
        csr_t *A = &h->A[l];
        h->x[l] = malloc(sizeof(double) * (A->n > 0 ? A->n : 1));
        h->b[l] = malloc(sizeof(double) * (A->n > 0 ? A->n : 1));
        h->t[l] = malloc(sizeof(double) * (A->n > 0 ? A->n : 1));
        if (A->n <= coarse_enough || l == AMG_MAX_LEVELS - 1) break;
        double *d = diagonal(A);
        int32_t *agg = malloc(sizeof(int32_t) * A->n);
        char *strong = malloc(A->ptr[A->n] > 0 ? A->ptr[A->n] : 1);
        int64_t na = aggregate(A, d, eps, agg, strong);
        if (na == 0 || na >= A->n) {
            free(d);
            free(agg);
            free(strong);
            break;
        }
        h->M[l] = malloc(sizeof(double) * A->n);
        spai0(A, h->M[l]);
        h->P[l] = smoothed_prolongator(A, strong, agg, na);
        h->R[l] = transpose(&h->P[l], na);
        csr_t AP = spgemm(A, &h->P[l], na);
        h->A[l + 1] = spgemm(&h->R[l], &AP, na);
        csr_free(&AP);
        free(d);
        free(agg);
        free(strong);
        eps *= 0.5;
        l++;
    }
    h->nlev = l + 1;
    skyline_factor(&h->A[l], &h->coarse);
    h->cw = malloc(sizeof(double) * (h->A[l].n > 0 ? h->A[l].n : 1));
}

static void cycle(amg_t *h, int l, const double *b, double *x) {
    csr_t *A = &h->A[l];
    int64_t n = A->n;
    if (l == h->nlev - 1) {
        skyline_solve(&h->coarse, b, x, h->cw);
        return;
    }
    double *t = h->t[l], *M = h->M[l];
    /* pre-relax from zero: x = M b */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) x[i] = M[i] * b[i];
    spmv(A, x, t);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) t[i] = b[i] - t[i];
    /* restrict */
    csr_t *R = &h->R[l];
    double *bc = h->b[l + 1], *xc = h->x[l + 1];
    spmv(R, t, bc);
    cycle(h, l + 1, bc, xc);
    /* prolongate */
    csr_t *P = &h->P[l];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double s = 0;
        for (int64_t e = P->ptr[i]; e < P->ptr[i + 1]; e++) s += P->val[e] * xc[P->col[e]];
        x[i] += s;
    }
    /* post-relax */
    spmv(A, x, t);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) x[i] += M[i] * (b[i] - t[i]);
}

/* ------------------------------------------------------------------------------------------------ Krylov */
typedef struct {
    int iters;
    double resid;
    int levels;
    double setup_s;
} amg_info_t;

static double now_s(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0;
#endif
}

/* kind 0: BiCGStab (pressure), kind 1: CG (potential).  x is the initial guess. Returns 0 on convergence. */
int or_amg_solve(int kind, int64_t n, int64_t *rowptr, int32_t *col, double *val, const double *b, double *x,
                 double tol, int maxiter, amg_info_t *info) {
    csr_t A = {n, rowptr, col, val};
    amg_t h;
    double t0 = now_s();
    amg_setup(&h, &A);
    if (info) {
        info->levels = h.nlev;
        info->setup_s = now_s() - t0;
    }
    double *r = malloc(sizeof(double) * n), *p = malloc(sizeof(double) * n), *q = malloc(sizeof(double) * n),
           *z = malloc(sizeof(double) * n), *s = malloc(sizeof(double) * n), *t = malloc(sizeof(double) * n),
           *rh = malloc(sizeof(double) * n), *sh = malloc(sizeof(double) * n);
    const double nb = sqrt(dot(n, b, b));
    int it = 0, conv = 0;
    double res = 0;
    if (nb == 0) {
        memset(x, 0, sizeof(double) * n);
        conv = 1;
        goto out;
    }
    spmv(&A, x, q);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) r[i] = b[i] - q[i];
    res = sqrt(dot(n, r, r)) / nb;
    if (res <= tol) {
        conv = 1;
        goto out;
    }
    if (kind == 1) {
        double rho = 0, rho_old = 1;
        for (it = 1; it <= maxiter; it++) {
            cycle(&h, 0, r, z);
            rho = dot(n, r, z);
            double beta = it == 1 ? 0 : rho / rho_old;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) p[i] = z[i] + (it == 1 ? 0 : beta * p[i]);
            spmv(&A, p, q);
            double alpha = rho / dot(n, p, q);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) {
                x[i] += alpha * p[i];
                r[i] -= alpha * q[i];
            }
            rho_old = rho;
            res = sqrt(dot(n, r, r)) / nb;
            if (res <= tol) {
                conv = 1;
                break;
            }
        }
    } else {
        double rho1 = 1, rho2 = 1, alpha = 1, omega = 1;
        memcpy(rh, r, sizeof(double) * n);
        memset(p, 0, sizeof(double) * n);
        memset(q, 0, sizeof(double) * n); /* v */
        for (it = 1; it <= maxiter; it++) {
            rho1 = dot(n, rh, r);
            if (rho1 == 0) break;
            if (it == 1) {
                memcpy(p, r, sizeof(double) * n);
            } else {
                double beta = (rho1 / rho2) * (alpha / omega);
#pragma omp parallel for schedule(static)
                for (int64_t i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - omega * q[i]);
            }
            cycle(&h, 0, p, z); /* z = M p */
            spmv(&A, z, q);     /* v = A z */
            alpha = rho1 / dot(n, rh, q);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) s[i] = r[i] - alpha * q[i];
            double sn = sqrt(dot(n, s, s)) / nb;
            if (sn <= tol) {
#pragma omp parallel for schedule(static)
                for (int64_t i = 0; i < n; i++) x[i] += alpha * z[i];
                res = sn;
                conv = 1;
                break;
            }
            cycle(&h, 0, s, sh);
            spmv(&A, sh, t);
            double tt = dot(n, t, t);
            omega = tt > 0 ? dot(n, t, s) / tt : 0;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) {
                x[i] += alpha * z[i] + omega * sh[i];
                r[i] = s[i] - omega * t[i];
            }
            rho2 = rho1;
            res = sqrt(dot(n, r, r)) / nb;
            if (res <= tol) {
                conv = 1;
                break;
            }
            if (omega == 0) break;
        }
    }
out:
    if (info) {
        info->iters = it;
        info->resid = res;
    }
    free(r);
    free(p);
    free(q);
    free(z);
    free(s);
    free(t);
    free(rh);
    free(sh);
    h.own_A0 = 0;
    amg_free(&h);
    return conv ? 0 : 1;
}
