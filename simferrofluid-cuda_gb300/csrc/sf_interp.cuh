// sf_interp.cuh -- the reference's grid interpolations on the device (core/TriLerp.h, core/TriCuInterp.h,
// core/Grid.h:33-35, core/GridData.h:31), for translation units compiled with -fmad=false: each expression is
// evaluated in the reference's order, so the results are bit-identical to its C++ on the same inputs.
#pragma once
#include <cmath>

#include "sf_internal.cuh"

namespace sf {

struct Origin {
    double o[3];  // staggered-grid corner (StaggeredGrid::GetOrigin)
};

// TriLerp::Interpolate of face grid b (size res + e_b, origin = corner + h/2 on the other axes) at p:
// Grid::CalcLower<1> / CalcLowerFrac and clamped At().
__device__ __forceinline__ double trilerp_face(const Dims &d, const double *__restrict__ v, int b, const double o[3],
                                               double h, double invh, const double p[3]) {
    const int s[3] = {d.nx + (b == 0), d.ny + (b == 1), d.nz + (b == 2)};
    int lo[3];
    double w[2][3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double co = a == b ? o[a] : o[a] + h / 2;  // face grid origin (core/StaggeredGrid.h:16-20)
        lo[a] = (int)floor((p[a] - co) * invh - 0.0);
        const double fr = (p[a] - co - (double)lo[a] * h) * invh;
        w[0][a] = 1. - fr;
        w[1][a] = fr;
    }
    double val = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int dx = q & 1, dy = (q >> 1) & 1, dz = (q >> 2) & 1;
        int ci[3] = {lo[0] + dx, lo[1] + dy, lo[2] + dz};
#pragma unroll
        for (int a = 0; a < 3; a++) ci[a] = ci[a] < 0 ? 0 : (ci[a] > s[a] - 1 ? s[a] - 1 : ci[a]);
        const double wt = w[dx][0] * w[dy][1] * w[dz][2];
        val += v[(long long)ci[2] + (long long)s[2] * ((long long)ci[1] + (long long)s[1] * ci[0])] * wt;
    }
    return val;
}

// TriCuInterp::Interpolate of the cell grid at p (core/TriCuInterp.h:12-37): CalcLower<3> = floor((p - o)/h - 1),
// cubic Lagrange weights per axis, 64 points in (k, j, i) order, clamped At().
__device__ __forceinline__ double tricubic_cell(const Dims &d, const double *__restrict__ f, const double o[3],
                                                double h, double invh, const double p[3]) {
    const int sz[3] = {d.nx, d.ny, d.nz};
    int lo[3];
    double w[4][3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double co = o[a] + h / 2;  // cell grid origin
        lo[a] = (int)floor((p[a] - co) * invh - 1.0);
        const double fr = (p[a] - co - (double)lo[a] * h) * invh;
        w[0][a] = (fr - 1) * (fr - 2) * (fr - 3) / -6;
        w[1][a] = fr * (fr - 2) * (fr - 3) / 2;
        w[2][a] = fr * (fr - 1) * (fr - 3) / -2;
        w[3][a] = fr * (fr - 1) * (fr - 2) / 6;
    }
    double val = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                int ci[3] = {lo[0] + i, lo[1] + j, lo[2] + k};
#pragma unroll
                for (int a = 0; a < 3; a++) ci[a] = ci[a] < 0 ? 0 : (ci[a] > sz[a] - 1 ? sz[a] - 1 : ci[a]);
                val += f[cid(d, ci[0], ci[1], ci[2])] * (w[i][0] * w[j][1] * w[k][2]);
            }
    return val;
}

}  // namespace sf
