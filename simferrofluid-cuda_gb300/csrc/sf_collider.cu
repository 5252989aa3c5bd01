// sf_collider.cu -- host-side Collider set-up: the solid-fraction inputs of the pressure solve.
//
// Collider(sgrid) builds a node level set of the domain-box walls (core/Collider.cpp:8-19), Finish()
// redistances it with FastMarching::Solve(LevelSet, -1) (core/FastMarching.cpp:25-62) and computes the
// per-face solid fraction (CalcFaceFraction, core/Collider.cpp:47-73).  It runs once per scene, so it stays
// on the host (a serial heap-ordered march); this file is compiled with -ffp-contract=off so the arithmetic
// rounds as the reference's does.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <queue>
#include <utility>
#include <vector>

#include "sfgpu.h"

namespace {

struct NodeGrid {
    int sx, sy, sz;
    double h;
    int64_t idx(int i, int j, int k) const { return (int64_t)k + (int64_t)sz * ((int64_t)j + (int64_t)sy * i); }
    bool valid(int i, int j, int k) const { return i >= 0 && j >= 0 && k >= 0 && i < sx && j < sy && k < sz; }
};

const int kNb[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};

inline double stdmin(double a, double b) { return (b < a) ? b : a; }

double solve_quadratic2(double p0, double p1, double dx) {
    if (p0 > p1) std::swap(p0, p1);
    if (std::isinf(p1) || p1 - p0 > dx) return p0 + dx;
    return ((p0 + p1) + std::sqrt(2 * dx * dx - (p0 - p1) * (p0 - p1))) * .5;
}

double solve_quadratic3(double p0, double p1, double p2, double dx) {
    if (p0 > p1) std::swap(p0, p1);
    if (p1 > p2) std::swap(p1, p2);
    if (std::isinf(p2) || (p2 - p0) * (p2 - p0) + (p2 - p1) * (p2 - p1) > dx * dx) return solve_quadratic2(p0, p1, dx);
    return (p0 + p1 + p2 + std::sqrt((p0 + p1 + p2) * (p0 + p1 + p2) - 3 * (p0 * p0 + p1 * p1 + p2 * p2 - dx * dx))) / 3;
}

using HeapEl = std::pair<double, int64_t>;
using Heap = std::priority_queue<HeapEl, std::vector<HeapEl>, std::greater<HeapEl>>;

double eikonal(const NodeGrid &g, int i, int j, int k, const std::vector<int8_t> &vis, const std::vector<double> &tent) {
    double t[3] = {INFINITY, INFINITY, INFINITY};
    for (int o = 0; o < 6; o++) {
        int ni = i + kNb[o][0], nj = j + kNb[o][1], nk = k + kNb[o][2];
        if (g.valid(ni, nj, nk) && vis[g.idx(ni, nj, nk)]) t[o >> 1] = stdmin(t[o >> 1], tent[g.idx(ni, nj, nk)]);
    }
    return solve_quadratic3(t[0], t[1], t[2], g.h);
}

void update_neighbours(const NodeGrid &g, int64_t c, const std::vector<int8_t> &vis, std::vector<double> &tent,
                       Heap &heap) {
    const int i = (int)(c / g.sz / g.sy), j = (int)(c / g.sz % g.sy), k = (int)(c % g.sz);
    for (int o = 0; o < 6; o++) {
        int ni = i + kNb[o][0], nj = j + kNb[o][1], nk = k + kNb[o][2];
        if (!g.valid(ni, nj, nk)) continue;
        const int64_t nb = g.idx(ni, nj, nk);
        if (vis[nb]) continue;
        const double t = eikonal(g, ni, nj, nk, vis, tent);
        if (t < tent[nb]) {
            tent[nb] = t;
            heap.push(HeapEl(t, nb));
        }
    }
}

// FastMarching::Solve(phi, maxSteps <= 0) on a node grid.
void fast_marching(const NodeGrid &g, double *phi) {
    const int64_t M = (int64_t)g.sx * g.sy * g.sz;
    std::vector<int8_t> vis(M, 0);
    std::vector<double> tent(M, std::numeric_limits<double>::infinity());
    std::vector<int64_t> intf;
    Heap heap;
    for (int i = 0; i < g.sx; i++)
        for (int j = 0; j < g.sy; j++)
            for (int k = 0; k < g.sz; k++) {
                const int64_t c = g.idx(i, j, k);
                double t[3] = {INFINITY, INFINITY, INFINITY};
                for (int o = 0; o < 6; o++) {
                    int ni = i + kNb[o][0], nj = j + kNb[o][1], nk = k + kNb[o][2];
                    if (!g.valid(ni, nj, nk)) continue;
                    const int64_t nb = g.idx(ni, nj, nk);
                    if (phi[c] * phi[nb] <= 0) t[o >> 1] = stdmin(t[o >> 1], phi[c] / (phi[c] - phi[nb]) * g.h);
                }
                if (std::isfinite(t[0]) || std::isfinite(t[1]) || std::isfinite(t[2])) {
                    const double a = 1. / t[0], b = 1. / t[1], d = 1. / t[2];
                    tent[c] = 1. / std::sqrt((a * a + b * b) + d * d);
                    vis[c] = 1;
                    intf.push_back(c);
                }
            }
    for (int64_t c : intf) update_neighbours(g, c, vis, tent, heap);
    while (!heap.empty()) {
        const HeapEl e = heap.top();
        heap.pop();
        if (tent[e.second] != e.first) continue;
        vis[e.second] = 1;
        update_neighbours(g, e.second, vis, tent, heap);
    }
    for (int64_t c = 0; c < M; c++) phi[c] = (phi[c] <= 0 ? -1 : 1) * tent[c];
}

// ImplicitBox::SignedDistanceTo (core/ImplicitSurface.h:82-111)
double box_sdf(const double c[3], const double hl[3], const double p[3]) {
    double q[3];
    bool inside = true;
    for (int a = 0; a < 3; a++) {
        q[a] = std::fabs(p[a] - c[a]) - hl[a];
        if (!(q[a] <= 0)) inside = false;
    }
    if (inside) {
        double m = q[0];
        if (q[1] > m) m = q[1];
        if (q[2] > m) m = q[2];
        return m;
    }
    double t[3];
    for (int a = 0; a < 3; a++) t[a] = q[a] > 0 ? q[a] : 0;
    return std::sqrt((t[0] * t[0] + t[1] * t[1]) + t[2] * t[2]);
}

// fraction of a triangle below zero (the `fraction` lambda of CalcFaceFraction)
double tri_fraction(double p0, double p1, double p2) {
    if (p0 > p1) std::swap(p0, p1);
    if (p1 > p2) std::swap(p1, p2);
    if (p0 > p1) std::swap(p0, p1);
    if (p2 <= 0) return 1.;
    if (p1 <= 0) return 1. - (p2 / (p2 - p0)) * (p2 / (p2 - p1));
    if (p0 <= 0) return (p0 / (p0 - p1)) * (p0 / (p0 - p2));
    return 0.;
}

}  // namespace

extern "C" {

SF_EXPORT sf_status sf_collider_face_fractions(const sf_grid *g, const double *node_ls, double *const frac[3]) {
    if (!g || g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || !node_ls || !frac || !frac[0] || !frac[1] || !frac[2])
        return SF_BAD_ARG;
    const int sy = g->ny + 1, sz = g->nz + 1;
    for (int a = 0; a < 3; a++) {
        const int fx = g->nx + (a == 0), fy = g->ny + (a == 1), fz = g->nz + (a == 2);
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    double p[4];
                    for (int q = 0; q < 4; q++) {  // StaggeredGrid::NodeOfFace
                        int n[3] = {i, j, k};
                        n[b1] += q & 1;
                        n[b2] += (q >> 1) & 1;
                        p[q] = node_ls[(int64_t)n[2] + (int64_t)sz * ((int64_t)n[1] + (int64_t)sy * n[0])];
                    }
                    const double cp = (p[0] + p[1] + p[2] + p[3]) * .25;
                    const double ff = (tri_fraction(cp, p[0], p[1]) + tri_fraction(cp, p[1], p[3]) +
                                       tri_fraction(cp, p[3], p[2]) + tri_fraction(cp, p[2], p[0])) * .25;
                    frac[a][(int64_t)k + (int64_t)fz * ((int64_t)j + (int64_t)fy * i)] = ff > .9 ? 1. : ff;
                }
    }
    return SF_OK;
}

// Collider::Finish normals (core/Collider.cpp:30-44): on each face of axis a, the mean over its four nodes
// (NodeOfFace order) of FiniteDiff::CalcFirstDrv of the node level set along a (core/FiniteDiff.h:9-19,50-52:
// one-sided second-order stencils at the node-grid ends).
SF_EXPORT sf_status sf_collider_face_normals(const sf_grid *g, const double *node_ls, double *const normal[3]) {
    if (!g || g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || !(g->h > 0) || !node_ls || !normal || !normal[0] ||
        !normal[1] || !normal[2])
        return SF_BAD_ARG;
    const int s3[3] = {g->nx + 1, g->ny + 1, g->nz + 1};
    const double invh = 1 / g->h;
    auto at = [&](int i, int j, int k) {
        return node_ls[(int64_t)k + (int64_t)s3[2] * ((int64_t)j + (int64_t)s3[1] * i)];
    };
    auto drv = [&](const int n[3], int a) {
        auto f = [&](int o) {
            int q[3] = {n[0], n[1], n[2]};
            q[a] += o;
            return at(q[0], q[1], q[2]);
        };
        if (n[a] == 0) return (4 * f(1) - 3 * f(0) - f(2)) * invh * .5;
        if (n[a] + 1 == s3[a]) return (3 * f(0) - 4 * f(-1) + f(-2)) * invh * .5;
        return (f(1) - f(-1)) * invh * .5;
    };
    for (int a = 0; a < 3; a++) {
        const int fx = g->nx + (a == 0), fy = g->ny + (a == 1), fz = g->nz + (a == 2);
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        for (int i = 0; i < fx; i++)
            for (int j = 0; j < fy; j++)
                for (int k = 0; k < fz; k++) {
                    double sum = 0;
                    for (int q = 0; q < 4; q++) {
                        int n[3] = {i, j, k};
                        n[b1] += q & 1;
                        n[b2] += (q >> 1) & 1;
                        sum += drv(n, a);
                    }
                    normal[a][(int64_t)k + (int64_t)fz * ((int64_t)j + (int64_t)fy * i)] = sum / 4;
                }
    }
    return SF_OK;
}

SF_EXPORT sf_status sf_collider_box_fractions(const sf_grid *g, int boundary_width, double *const frac[3],
                                              double *node_ls_out) {
    if (!g || g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || !(g->h > 0) || boundary_width < 0 || !frac)
        return SF_BAD_ARG;
    NodeGrid ng{g->nx + 1, g->ny + 1, g->nz + 1, g->h};
    const int64_t M = (int64_t)ng.sx * ng.sy * ng.sz;
    std::vector<double> own;
    double *ls = node_ls_out;
    if (!ls) {
        own.resize(M);
        ls = own.data();
    }
    const int res[3] = {g->nx, g->ny, g->nz};
    double c[3], hl[3];
    for (int a = 0; a < 3; a++) {  // ImplicitBox(GetDomainOrigin(), GetDomainLengths())
        const double mn = g->origin[a] + (double)boundary_width * g->h;
        const double len = (double)(res[a] - boundary_width * 2) * g->h;
        c[a] = mn + len / 2;
        hl[a] = len / 2;
    }
    for (int i = 0; i < ng.sx; i++)
        for (int j = 0; j < ng.sy; j++)
            for (int k = 0; k < ng.sz; k++) {
                const double p[3] = {g->origin[0] + (double)i * g->h, g->origin[1] + (double)j * g->h,
                                     g->origin[2] + (double)k * g->h};
                ls[ng.idx(i, j, k)] = -.01 * g->h - box_sdf(c, hl, p);
            }
    fast_marching(ng, ls);
    return sf_collider_face_fractions(g, ls, frac);
}

}  // extern "C"
