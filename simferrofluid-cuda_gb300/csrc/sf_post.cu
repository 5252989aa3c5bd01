// sf_post.cu -- the velocity pipeline after the pressure projection (core/Simulation.cpp:236-241): extrapolation
// of the projected velocity into the air (Extrapolation::Solve) and the collider's boundary condition
// (Collider::Enforce), on device-resident face arrays.
//
// Compiled with -fmad=false: each expression rounds as the reference's C++ does, so the results are bit-identical
// to the CPU restatement on the same inputs.
#include <cmath>

#include "sf_ops.h"

namespace sf {

namespace {

inline dim3 blk2() { return dim3(32, 8, 1); }
inline dim3 face_grid(const Dims &d, int a) {
    return dim3((d.nz + (a == 2) + 31) / 32, (d.ny + (a == 1) + 7) / 8, d.nx + (a == 0));
}

struct FDims {
    int fx, fy, fz;
};
__device__ __forceinline__ FDims fdims(const Dims &d, int a) { return FDims{d.nx + (a == 0), d.ny + (a == 1), d.nz + (a == 2)}; }
__device__ __forceinline__ long long fidx(const FDims &f, int i, int j, int k) {
    return (long long)k + (long long)f.fz * ((long long)j + (long long)f.fy * i);
}

// Extrapolation validity (core/Simulation.cpp:237-240): fraction < 1 and an adjacent cell (face - e_a, face)
// is liquid; a cell outside the grid is not liquid.
__global__ void __launch_bounds__(256) k_extrap_init(Dims d, int a, const double *__restrict__ phi,
                                                     const double *__restrict__ frac, uint8_t *__restrict__ valid) {
    const FDims f = fdims(d, a);
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= f.fz || j >= f.fy) return;
    const long long fi = fidx(f, i, j, k);
    uint8_t v = 0;
    if (frac[fi] < 1) {
        int c0[3] = {i, j, k};
        c0[a] -= 1;
        const bool in0 = c0[0] >= 0 && c0[1] >= 0 && c0[2] >= 0;
        const bool in1 = i < d.nx && j < d.ny && k < d.nz;
        const bool l0 = in0 && phi[cid(d, c0[0], c0[1], c0[2])] <= 0;
        const bool l1 = in1 && phi[cid(d, i, j, k)] <= 0;
        v = (l0 || l1) ? 1 : 0;
    }
    valid[fi] = v;
}

// One sweep of Extrapolation::Solve (core/Extrapolation.cpp:7-28) on face grid a: invalid faces take the mean of
// their valid 6-neighbours (order -x,+x,-y,+y,-z,+z) and become valid, or clear_val without any.  Valid faces are
// never written in a sweep, so the in-place update reads only values of the previous sweep.
__global__ void __launch_bounds__(256) k_extrap_step(Dims d, int a, double *__restrict__ u,
                                                     const uint8_t *__restrict__ valid, uint8_t *__restrict__ valid1,
                                                     double clear_val) {
    const FDims f = fdims(d, a);
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= f.fz || j >= f.fy) return;
    const long long fi = fidx(f, i, j, k);
    if (valid[fi]) {
        valid1[fi] = 1;
        return;
    }
    int cnt = 0;
    double sum = 0;
    const int n3[3] = {f.fx, f.fy, f.fz};
#pragma unroll
    for (int o = 0; o < 6; o++) {
        const int ax = o >> 1, s = (o & 1) ? 1 : -1;
        int q[3] = {i, j, k};
        q[ax] += s;
        if (q[ax] < 0 || q[ax] >= n3[ax]) continue;
        const long long nb = fidx(f, q[0], q[1], q[2]);
        if (valid[nb]) {
            sum += u[nb];
            cnt++;
        }
    }
    if (cnt > 0) {
        u[fi] = sum / cnt;
        valid1[fi] = 1;
    } else {
        u[fi] = clear_val;
        valid1[fi] = 0;
    }
}

// TriLerp::Interpolate (core/TriLerp.h:28-36, 54-58) of face grid b at p: Grid::CalcLower<1> / CalcLowerFrac
// (core/Grid.h:33-35) and clamped At() (core/GridData.h:31).
__device__ double trilerp_face(const Dims &d, const double *__restrict__ v, int b, const double o[3], double h,
                               double invh, const double p[3]) {
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

struct Origin {
    double o[3];
};

// Collider::Enforce (core/Collider.cpp:75-86) on the faces of axis a with fraction == 1: the interpolated old
// velocity minus its normal component relative to the solid velocity (us.p[0] == nullptr: zero).
__global__ void __launch_bounds__(256) k_enforce(Dims d, int a, Origin og, double h, double invh, Faces old,
                                                 Faces us, Faces normal, const double *__restrict__ frac,
                                                 double *__restrict__ u) {
    const FDims f = fdims(d, a);
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= f.fz || j >= f.fy) return;
    const long long fi = fidx(f, i, j, k);
    if (frac[fi] != 1.) return;
    const int c3[3] = {i, j, k};
    double p[3];
#pragma unroll
    for (int b = 0; b < 3; b++) p[b] = (b == a ? og.o[b] : og.o[b] + h / 2) + (double)c3[b] * h;  // PositionOf
    double vel[3], vel0[3], n[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        vel[b] = trilerp_face(d, old.p[b], b, og.o, h, invh, p);
        vel0[b] = us.p[0] ? trilerp_face(d, us.p[b], b, og.o, h, invh, p) : 0.0;
        n[b] = trilerp_face(d, normal.p[b], b, og.o, h, invh, p);
    }
    const double nn = sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);  // Vector3d::normalized
    if (nn > 0)
#pragma unroll
        for (int b = 0; b < 3; b++) n[b] = n[b] / nn;
    const double dv0 = vel[0] - vel0[0], dv1 = vel[1] - vel0[1], dv2 = vel[2] - vel0[2];
    const double dn = (dv0 * n[0] + dv1 * n[1]) + dv2 * n[2];
    u[fi] = vel[a] - dn * n[a];
}

// MagneticField::CalculateVertexPressures (core/MagneticField.cpp:37-48) for vertex v: H trilinear at its position,
// p = mu0/2 chi (|H|^2 + chi^2/(4chi+4) (H.n)^2), mu0 = 4e-7 pi (core/MagneticField.cpp:7-8).
__global__ void k_vertex_pressures(Dims d, Origin og, double h, double invh, Faces H, double chi,
                                   const double *__restrict__ pos, const double *__restrict__ nrm, long long nv,
                                   double *__restrict__ out) {
    const double pi = 3.141592653589793238462643383279502884;
    const double mu0 = 4e-7 * pi;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x) {
        const double p[3] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
        const double n[3] = {nrm[3 * v], nrm[3 * v + 1], nrm[3 * v + 2]};
        double hv[3];
#pragma unroll
        for (int b = 0; b < 3; b++) hv[b] = trilerp_face(d, H.p[b], b, og.o, h, invh, p);
        double coeff = (hv[0] * hv[0] + hv[1] * hv[1]) + hv[2] * hv[2];
        const double hn = (hv[0] * n[0] + hv[1] * n[1]) + hv[2] * n[2];
        coeff += chi * chi / (4 * chi + 4) * hn * hn;
        out[v] = mu0 * 0.5 * chi * coeff;
    }
}

struct EdgeMarks {
    const int32_t *p[3];
};

// The pressure-jump callback of core/Simulation.cpp:216-235 on the faces of axis a: the vertex of edge
// (a, face - e_a) (Contour::VertexIndexOf; edge grid of axis a = cell grid minus e_a, -1 = no vertex) gives
// J = kappa sigma / rho / h dt - p_m / rho / h dt (terms present when their arrays are), 0 without a vertex.
__global__ void __launch_bounds__(256) k_pressure_jump(Dims d, int a, EdgeMarks em, const double *__restrict__ kappa,
                                                       const double *__restrict__ pm, double sigma, double rho,
                                                       double invh, double dt, double *__restrict__ jump) {
    const FDims f = fdims(d, a);
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= f.fz || j >= f.fy) return;
    const int ex = d.nx - (a == 0), ey = d.ny - (a == 1), ez = d.nz - (a == 2);
    int e[3] = {i, j, k};
    e[a] -= 1;
    int idx = -1;
    if (e[0] >= 0 && e[1] >= 0 && e[2] >= 0 && e[0] < ex && e[1] < ey && e[2] < ez)
        idx = em.p[a][(long long)e[2] + (long long)ez * ((long long)e[1] + (long long)ey * e[0])];
    double pressure = 0;
    if (kappa && idx >= 0) pressure += kappa[idx] * sigma / rho * invh * dt;
    if (pm && idx >= 0) pressure -= pm[idx] / rho * invh * dt;
    jump[fidx(f, i, j, k)] = pressure;
}

}  // namespace

void launch_vertex_pressures(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &H,
                             double chi, const double *pos, const double *nrm, long long nv, double *out) {
    if (nv <= 0) return;
    Origin og{{origin[0], origin[1], origin[2]}};
    long long blocks = (nv + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_vertex_pressures<<<(unsigned)blocks, 256, 0, st>>>(d, og, h, 1 / h, H, chi, pos, nrm, nv, out);
}

void launch_pressure_jump(cudaStream_t st, const Dims &d, const int32_t *const edge_mark[3], const double *kappa,
                          const double *pm, double sigma, double rho, double h, double dt, double *const jump[3]) {
    EdgeMarks em{{edge_mark[0], edge_mark[1], edge_mark[2]}};
    for (int a = 0; a < 3; a++)
        k_pressure_jump<<<face_grid(d, a), blk2(), 0, st>>>(d, a, em, kappa, pm, sigma, rho, 1 / h, dt, jump[a]);
}

void launch_extrapolate(cudaStream_t st, const Dims &d, const double *phi, const Faces &frac, double *const u[3],
                        uint8_t *const valid[3], uint8_t *const valid1[3], double clear_val, int max_steps) {
    for (int a = 0; a < 3; a++) {
        k_extrap_init<<<face_grid(d, a), blk2(), 0, st>>>(d, a, phi, frac.p[a], valid[a]);
        uint8_t *v0 = valid[a], *v1 = valid1[a];
        for (int it = 0; it < max_steps; it++) {
            k_extrap_step<<<face_grid(d, a), blk2(), 0, st>>>(d, a, u[a], v0, v1, clear_val);
            uint8_t *t = v0;
            v0 = v1;
            v1 = t;
        }
    }
}

void launch_enforce(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &old,
                    const Faces &us, const Faces &normal, const Faces &frac, double *const u[3]) {
    Origin og{{origin[0], origin[1], origin[2]}};
    const double invh = 1 / h;  // Grid::m_InvSpacing
    for (int a = 0; a < 3; a++)
        k_enforce<<<face_grid(d, a), blk2(), 0, st>>>(d, a, og, h, invh, old, us, normal, frac.p[a], u[a]);
}

}  // namespace sf
