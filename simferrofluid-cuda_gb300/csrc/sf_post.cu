// sf_post.cu -- the velocity pipeline after the pressure projection (core/Simulation.cpp:236-241): extrapolation
// of the projected velocity into the air (Extrapolation::Solve) and the collider's boundary condition
// (Collider::Enforce), on device-resident face arrays.
//
// Compiled with -fmad=false: each expression rounds as the reference's C++ does, so the results are bit-identical
// to the CPU restatement on the same inputs.
#include <cmath>

#include "sf_interp.cuh"
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

// ------------------------------------------------------------------------------------------------ level set
// Advection::Trace<2> (core/Advection.h:15-18): TVD Runge-Kutta trace of second order from p over dt.
__device__ __forceinline__ void trace_rk2(const Dims &d, const Faces &u, const double o[3], double h, double invh,
                                          const double p[3], double dt, double out[3]) {
    double v0[3], v1[3], q[3];
#pragma unroll
    for (int b = 0; b < 3; b++) v0[b] = trilerp_face(d, u.p[b], b, o, h, invh, p);
#pragma unroll
    for (int b = 0; b < 3; b++) q[b] = p[b] + v0[b] * dt;
#pragma unroll
    for (int b = 0; b < 3; b++) v1[b] = trilerp_face(d, u.p[b], b, o, h, invh, q);
#pragma unroll
    for (int b = 0; b < 3; b++) out[b] = p[b] + (v0[b] + v1[b]) * dt / 2;
}

// Advection::Solve<2>(levelSet, velocity, dt) (core/Advection.h:40-49): phi at each cell centre's RK2 departure
// point (trace over -dt), by tricubic interpolation of the old phi.
__global__ void __launch_bounds__(256) k_advect_levelset(Dims d, Origin og, double h, double invh, Faces u,
                                                         double dt, const double *__restrict__ phi,
                                                         double *__restrict__ out) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= d.nz || j >= d.ny) return;
    const double p[3] = {og.o[0] + h / 2 + (double)i * h, og.o[1] + h / 2 + (double)j * h,
                         og.o[2] + h / 2 + (double)k * h};
    double q[3];
    trace_rk2(d, u, og.o, h, invh, p, -dt, q);
    out[cid(d, i, j, k)] = tricubic_cell(d, phi, og.o, h, invh, q);
}

// Advection::Solve<2>(velocity, velocity, dt) (core/Advection.h:51-59) for the faces of axis a: trilinear
// interpolation of the old face grid a at each face's RK2 departure point.
__global__ void __launch_bounds__(256) k_advect_velocity(Dims d, int a, Origin og, double h, double invh, Faces u,
                                                         const double *__restrict__ ua, double dt,
                                                         double *__restrict__ out) {
    const FDims f = fdims(d, a);
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= f.fz || j >= f.fy) return;
    const int c3[3] = {i, j, k};
    double p[3], q[3];
#pragma unroll
    for (int b = 0; b < 3; b++) p[b] = (b == a ? og.o[b] : og.o[b] + h / 2) + (double)c3[b] * h;
    trace_rk2(d, u, og.o, h, invh, p, -dt, q);
    out[fidx(f, i, j, k)] = trilerp_face(d, ua, a, og.o, h, invh, q);
}

__device__ __forceinline__ double dmax0(double a, double b) { return (a < b) ? b : a; }  // std::max(a, b)

// GetDrv (core/Reinitialization.cpp:4-27): WENO5 one-sided derivatives from 7 values (s = 0 minus, 1 plus).
__device__ __forceinline__ double weno_side(const double v[7], int s, double invdx) {
    double dev[5];
    if (s) {
        dev[0] = v[6] - v[5];
        dev[1] = v[5] - v[4];
        dev[2] = v[4] - v[3];
        dev[3] = v[3] - v[2];
        dev[4] = v[2] - v[1];
    } else {
        dev[0] = v[1] - v[0];
        dev[1] = v[2] - v[1];
        dev[2] = v[3] - v[2];
        dev[3] = v[4] - v[3];
        dev[4] = v[5] - v[4];
    }
    double eps = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) eps = dmax0(eps, dev[j] * dev[j]);
    eps = eps * 1e-6 + 1e-99;
    const double phix1 = dev[0] / 3 - dev[1] * 7 / 6 + dev[2] * 11 / 6;
    const double phix2 = -dev[1] / 6 + dev[2] * 5 / 6 + dev[3] / 3;
    const double phix3 = dev[2] / 3 + dev[3] * 5 / 6 - dev[4] / 6;
    double t = dev[0] - 2 * dev[1] + dev[2];
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
    const double alpha1 = .1 / (t * t);
    t = s2 + eps;
    const double alpha2 = .6 / (t * t);
    t = s3 + eps;
    const double alpha3 = .3 / (t * t);
    const double sum = alpha1 + alpha2 + alpha3;
    return (alpha1 * phix1 + alpha2 * phix2 + alpha3 * phix3) / sum * invdx;
}

// Reinitialization::Advance (core/Reinitialization.cpp:48-74): one explicit step of the reinitialisation
// equation with Godunov upwinding of the WENO5 derivatives (clamped stencils at the grid ends).
__global__ void __launch_bounds__(256) k_reinit_advance(Dims d, double h, double invdx, double dt,
                                                        const double *__restrict__ f, double *__restrict__ out) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= d.nz || j >= d.ny) return;
    const int c3[3] = {i, j, k};
    const int sz[3] = {d.nx, d.ny, d.nz};
    const double fc = f[cid(d, i, j, k)];
    double sum = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double v[7];
#pragma unroll
        for (int q = 0; q < 7; q++) {
            int c[3] = {c3[0], c3[1], c3[2]};
            c[a] += q - 3;
            c[a] = c[a] < 0 ? 0 : (c[a] > sz[a] - 1 ? sz[a] - 1 : c[a]);
            v[q] = f[cid(d, c[0], c[1], c[2])];
        }
        const double dm = weno_side(v, 0, invdx), dp = weno_side(v, 1, invdx);
        double t;
        if (fc < 0) {
            t = dm < 0. ? dm : 0.;
            sum += t * t;
            t = dmax0(dp, 0.);
            sum += t * t;
        } else {
            t = dmax0(dm, 0.);
            sum += t * t;
            t = dp < 0. ? dp : 0.;
            sum += t * t;
        }
    }
    sum = sqrt(sum);
    const double sp = h * sum;
    const double sgn = fc / sqrt(fc * fc + sp * sp);
    out[cid(d, i, j, k)] = fc + dt * sgn * (1. - sum);
}

// TVD-RK3 combinations of Reinitialization::Solve (core/Reinitialization.cpp:41-44).
__global__ void k_rk3_stage(long long n, const double *__restrict__ phi, const double *__restrict__ p2,
                            double *__restrict__ p1) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        p1[c] = (phi[c] * 3 + p2[c]) / 4;
}
__global__ void k_rk3_final(long long n, double *__restrict__ phi, const double *__restrict__ p2) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        phi[c] = (phi[c] + p2[c] * 2) / 3;
}

inline dim3 cell_grid(const Dims &d) { return dim3((d.nz + 31) / 32, (d.ny + 7) / 8, d.nx); }
inline unsigned flat_blocks(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

}  // namespace

void launch_advect_levelset(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &u,
                            double dt, const double *phi, double *out) {
    Origin og{{origin[0], origin[1], origin[2]}};
    k_advect_levelset<<<cell_grid(d), blk2(), 0, st>>>(d, og, h, 1 / h, u, dt, phi, out);
}

void launch_advect_velocity(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &u,
                            double dt, double *const out[3]) {
    Origin og{{origin[0], origin[1], origin[2]}};
    for (int a = 0; a < 3; a++)
        k_advect_velocity<<<face_grid(d, a), blk2(), 0, st>>>(d, a, og, h, 1 / h, u, u.p[a], dt, out[a]);
}

void launch_reinitialize(cudaStream_t st, const Dims &d, double h, double *phi, double *p1, double *p2,
                         int max_steps) {
    const double dt = h * .5, invdx = 1 / h;
    for (int it = 0; it < max_steps; it++) {
        k_reinit_advance<<<cell_grid(d), blk2(), 0, st>>>(d, h, invdx, dt, phi, p1);
        k_reinit_advance<<<cell_grid(d), blk2(), 0, st>>>(d, h, invdx, dt, p1, p2);
        k_rk3_stage<<<flat_blocks(d.n), 256, 0, st>>>(d.n, phi, p2, p1);
        k_reinit_advance<<<cell_grid(d), blk2(), 0, st>>>(d, h, invdx, dt, p1, p2);
        k_rk3_final<<<flat_blocks(d.n), 256, 0, st>>>(d.n, phi, p2);
    }
}

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
