// sf_ops.cu -- assembly and post-solve kernels of the pressure projection and the magnetic potential.
//
// Compiled with -fmad=false: every expression below rounds exactly as the reference's C++ does (no fused
// multiply-add), so the fine-level operator and right-hand side are bit-identical to the reference's CSR
// assembly on the same inputs, and the velocity / field updates are too.
#include <cmath>
#include <cstring>

#include "sf_ops.h"

namespace sf {

static inline dim3 blk2() { return dim3(32, 8, 1); }
static inline dim3 grid3(int nx, int ny, int nz) { return dim3((nz + 31) / 32, (ny + 7) / 8, nx); }

__device__ __forceinline__ long long fid(const Dims &d, int a, int i, int j, int k) {
    const int fy = d.ny + (a == 1), fz = d.nz + (a == 2);
    return (long long)k + (long long)fz * ((long long)j + (long long)fy * i);
}

// Comparisons as integer tests on the bits, so they do not occupy the FP64 pipe (the assembly kernels are
// bound by it).  le0(v) == (v <= 0) for every double, NaN included; is_zero(v) == (v == 0).
constexpr long long kOneBits = 0x3FF0000000000000LL;  // 1.0
__device__ __forceinline__ bool le0(double v) {
    const long long b = __double_as_longlong(v);
    return b == 0 || (b < 0 && (b & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL);
}
__device__ __forceinline__ bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }

// The split level-0 copies of a cell's stored coefficients (same roundings as the solver's own conversion) and
// its row's flag when the cell is active.
__device__ __forceinline__ void split_store(const SplitOut &so, const Dims &d, int i, int j, int k, double ax,
                                            double ay, double az, double dex, bool active) {
    const long long q = split_index(d, i, j, k);
    // converted on the integer pipe: this kernel is FP64-bound (same bits as the hardware conversion)
    const float fx = f64_to_f32(ax), fy = f64_to_f32(ay), fz = f64_to_f32(az), fd = f64_to_f32(dex);
    so.c32.ax[q] = fx;
    so.c32.ay[q] = fy;
    so.c32.az[q] = fz;
    so.c32.dex[q] = fd;
    so.c16.ax[q] = __float2half_rn(fx);
    so.c16.ay[q] = __float2half_rn(fy);
    so.c16.az[q] = __float2half_rn(fz);
    so.c16.dex[q] = __float2half_rn(fd);
    if (active) so.rows[(long long)i * d.ny + j] = 1;  // every writer stores 1
}

// ------------------------------------------------------------------------------------------------ pressure
// Pressure::SetUnKnowns + BuildProjectionMatrix (core/Pressure.cpp:104-123, 38-78) for one cell.
// Liquid cells are phi <= 0.  The face weight is w = 1 - fraction; faces on the outer grid boundary are
// closed (w = 0).  D is the reference's diagonal bit for bit (same summation order, 1 for an isolated cell).
//
// Fast path with the same bits: an interior cell whose six fractions are zero (w = 1 exactly) and, when the
// operator is built, whose six neighbours are liquid.  The general loop then sums six ones (D = 6), stores
// unit couplings, adds no ghost or solid-velocity term, and each face's -side * w * u is exactly -side * u,
// so the divergence is six additions / subtractions in the same order.
__global__ void __launch_bounds__(256) k_build_pressure(Dims d, const double *__restrict__ phi, Faces frac,
                                                        Faces u, Faces us, Faces jump, double vol_error,
                                                        Coef<double> cf, double *__restrict__ b, int rhs_only,
                                                        int want_invd, SplitOut so) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= d.nz || j >= d.ny) return;
    const long long c = cid(d, i, j, k);
    if (rhs_only) {
        // Pressure::SetRightHandSide (:80-102) on the unknowns of the last build (D > 0)
        if (!(cf.D[c] > 0)) {
            b[c] = 0;
            return;
        }
    }
    const double pc = phi[c];
    const bool liquid = rhs_only ? true : le0(pc);
    if (liquid && i > 0 && i < d.nx - 1 && j > 0 && j < d.ny - 1 && k > 0 && k < d.nz - 1) {
        const long long sx = (long long)d.ny * d.nz, sy = d.nz;
        const long long fx0 = fid(d, 0, i, j, k), fx1 = fid(d, 0, i + 1, j, k);
        const long long fy0 = fid(d, 1, i, j, k), fy1 = fid(d, 1, i, j + 1, k);
        const long long fz0 = fid(d, 2, i, j, k), fz1 = fid(d, 2, i, j, k + 1);
        bool open = is_zero(frac.p[0][fx0]) & is_zero(frac.p[0][fx1]) & is_zero(frac.p[1][fy0]) &
                    is_zero(frac.p[1][fy1]) & is_zero(frac.p[2][fz0]) & is_zero(frac.p[2][fz1]);
        if (open && !rhs_only)
            open = le0(phi[c - sx]) & le0(phi[c + sx]) & le0(phi[c - sy]) & le0(phi[c + sy]) & le0(phi[c - 1]) &
                   le0(phi[c + 1]);
        if (open) {
            double div = 0;
            div += u.p[0][fx0];  // ord -x: div -= (-1 * 1) * u
            div -= u.p[0][fx1];  // ord +x: div -= (+1 * 1) * u
            div += u.p[1][fy0];
            div -= u.p[1][fy1];
            div += u.p[2][fz0];
            div -= u.p[2][fz1];
            div += vol_error;
            b[c] = div;
            if (rhs_only) return;
            cf.ax[c] = 1.;
            cf.ay[c] = 1.;
            cf.az[c] = 1.;
            cf.dex[c] = 0.;
            cf.D[c] = 6.;
            if (want_invd) cf.invd[c] = 1. / 6.;
            if (so.rows) split_store(so, d, i, j, k, 1., 1., 1., 0., true);
            return;
        }
    }
    double lower[3] = {0, 0, 0};
    double diag = 0, dexv = 0, div = 0;
    if (liquid) {
        const int dn[3] = {d.nx, d.ny, d.nz};
#pragma unroll
        for (int ord = 0; ord < 6; ord++) {
            const int a = ord >> 1;
            const int up = ord & 1;
            const double side = up ? 1.0 : -1.0;
            int f3[3] = {i, j, k};
            f3[a] += up;
            int n3[3] = {i, j, k};
            n3[a] += up ? 1 : -1;
            const bool valid = n3[a] >= 0 && n3[a] < dn[a];
            const long long f = fid(d, a, f3[0], f3[1], f3[2]);
            const double w = valid ? 1. - frac.p[a][f] : 0.0;
            if (w > 0) {
                if (!rhs_only) {
                    const long long nb = cid(d, n3[0], n3[1], n3[2]);
                    const double pn = phi[nb];
                    if (le0(pn)) {
                        diag += w;
                        if (!up) lower[a] = w;
                    } else {
                        const double theta = pc / (pc - pn);
                        const double ic = 1. / (theta < .001 ? .001 : theta);
                        diag += w * ic;
                        dexv += w * ic;
                        if (jump.p[0]) div += jump.p[a][f] * w * ic;
                    }
                }
                div -= side * w * u.p[a][f];
            }
            if (w < 1) {
                const double usv = us.p[0] ? us.p[a][f] : 0.0;
                div -= side * (1 - w) * usv;
            }
        }
        div += vol_error;
    }
    b[c] = liquid ? div : 0.0;
    if (rhs_only) return;
    const double D = liquid ? (diag != 0 ? diag : 1.) : 0.0;
    if (liquid && diag == 0) dexv = 1.;
    cf.ax[c] = lower[0];
    cf.ay[c] = lower[1];
    cf.az[c] = lower[2];
    cf.dex[c] = dexv;
    cf.D[c] = D;
    if (want_invd) cf.invd[c] = liquid ? (D > 0 ? 1. / D : 0.0) : 0.0;
    if (so.rows) split_store(so, d, i, j, k, lower[0], lower[1], lower[2], dexv, D > 0);
}

// Pressure::ApplyProjection (core/Pressure.cpp:137-166).  One thread per node (i, j, k) of the cell grid updates
// the lower x, y and z faces of cell (i, j, k), in one launch over (nx + 1) x (ny + 1) x (nz + 1) points, so phi and
// p of the cell are loaded once for its three faces.  p is the solution on cells; liquid = phi <= 0.
// w = 1 - fraction is 0 exactly when the fraction is 1, and 1 exactly when it is zero, where (p1 - p0) * w is
// p1 - p0: both are tested on the bits, so air faces and open liquid faces take no FP64 operation beyond the
// update itself.
__device__ __forceinline__ void project_face(const Dims &d, int a, long long f, long long c0, long long c1, int fa,
                                             int na, const double *__restrict__ phi, const Faces &frac,
                                             const Faces &jump, const double *__restrict__ p, double *__restrict__ u,
                                             double phi1, bool l1) {
    if (fa <= 0 || fa >= na) return;  // closed boundary face
    const double fr = frac.p[a][f];
    if (__double_as_longlong(fr) == kOneBits) return;  // w == 0
    const double phi0 = phi[c0];
    const bool l0 = le0(phi0);
    if (!l0 && !l1) return;
    double v = u[f];
    if (l0 && l1 && is_zero(fr)) {
        v -= p[c1] - p[c0];  // w == 1
    } else if (l0 && l1) {
        v -= (p[c1] - p[c0]) * (1. - fr);
    } else {
        const double w = 1. - fr;
        const double theta = phi0 / (phi0 - phi1);
        const double pin = l0 ? p[c0] : p[c1];
        const double pj = jump.p[0] ? jump.p[a][f] : 0.;
        const double t = l0 ? theta : 1 - theta;
        const double ic = 1. / (t < .001 ? .001 : t);
        v -= (l0 ? 1.0 : -1.0) * (pj - pin) * ic * w;
    }
    u[f] = v;
}

__global__ void __launch_bounds__(256) k_apply_projection3(Dims d, const double *__restrict__ phi, Faces frac,
                                                           Faces jump, const double *__restrict__ p, Faces u) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k > d.nz || j > d.ny || i > d.nx) return;
    const bool cell = i < d.nx && j < d.ny && k < d.nz;
    const long long c1 = cell ? cid(d, i, j, k) : 0;
    const double phi1 = cell ? phi[c1] : 1.0;  // a face whose upper cell is outside the grid is a boundary face
    const bool l1 = cell && le0(phi1);
    const long long sx = (long long)d.ny * d.nz, sy = d.nz;
    if (j < d.ny && k < d.nz)
        project_face(d, 0, fid(d, 0, i, j, k), c1 - sx, c1, i, d.nx, phi, frac, jump, p, const_cast<double *>(u.p[0]),
                     phi1, l1);
    if (i < d.nx && k < d.nz)
        project_face(d, 1, fid(d, 1, i, j, k), c1 - sy, c1, j, d.ny, phi, frac, jump, p, const_cast<double *>(u.p[1]),
                     phi1, l1);
    if (i < d.nx && j < d.ny)
        project_face(d, 2, fid(d, 2, i, j, k), c1 - 1, c1, k, d.nz, phi, frac, jump, p, const_cast<double *>(u.p[2]),
                     phi1, l1);
}

// p_out on cells: solution in liquid cells (D > 0 in the stored operator), 0 elsewhere.
__global__ void k_gather_cells(long long n, const double *__restrict__ D, const double *__restrict__ x,
                               double *__restrict__ out) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        out[c] = D[c] > 0 ? x[c] : 0.0;
}

// ------------------------------------------------------------------------------------------------ magnetic
// MagneticField::Heaviside (core/MagneticField.h:44-54): 0 below -bw, 1 above bw (exactly, as the reference),
// and in the band .5 (1 + t + sin(pi t) / pi) with t = phi / bw.  In the band it is evaluated with 1 / bw formed
// on the host, sin(pi t) as sinpi(t) and a multiplication by 1 / pi: the reference's three FP64 divisions and
// sin(pi * phi / bw) bound this kernel by the FP64 rate, and these forms agree with them to a few ulp (band faces
// already differ from the reference's by the device's and the host's sin in the last bits).
__device__ __forceinline__ double heaviside(double phi, double bw, double inv_bw) {
    const double inv_pi = 0.318309886183790671537767526745028724;
    if (phi < -bw) return 0.;
    if (phi > bw) return 1.;
    const double t = phi * inv_bw;
    return .5 * (1. + t + sinpi(t) * inv_pi);
}

// mu on an interior face between cells lo and hi (core/MagneticField.cpp:57-58).  The reference samples phi
// trilinearly at the face centre; at a face centre the trilinear weights are exactly (1/2, 1/2, 0, ...) when
// the grid coordinates are exact binary fractions, which this expression reproduces bit for bit; otherwise
// it differs from the reference's weights (1/2 +- 1 ulp) by a few ulp of phi.
__device__ __forceinline__ double mu_face(double philo, double phihi, double chi, double bw, double inv_bw) {
    const double pf = 0.5 * philo + 0.5 * phihi;
    return 1. + (1. - heaviside(pf, bw, inv_bw)) * chi;
}

// Order-preserving integer key of a double (IEEE total order on finite values): comparisons of keys are
// integer instructions, so faces far from the interface are classified without FP64 arithmetic.
__device__ __forceinline__ long long okey(double v) {
    const long long b = __double_as_longlong(v);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// mu_face with a fast path: when both cell values lie beyond +-bw (1 + 2^-40) the face value is beyond +-bw
// too, so H is exactly 0 or 1 and mu is exactly 1 + chi (precomputed, same rounding) or 1.
__device__ __forceinline__ double mu_face_fast(double philo, double phihi, double chi, double bw, double inv_bw,
                                               long long khi, long long klo, double one_plus_chi) {
    const long long a = okey(philo), b = okey(phihi);
    if (a > khi && b > khi) return 1.;
    if (a < klo && b < klo) return one_plus_chi;
    return mu_face(philo, phihi, chi, bw, inv_bw);
}

// BuildMatrix, coefficient pass (core/MagneticField.cpp:51-60): mu on the lower x/y/z face of every cell,
// stored directly as the lower-face couplings ax/ay/az (0 on the grid boundary, where the reference's mu = 1
// is never used).  Each face is evaluated once.
__global__ void __launch_bounds__(256) k_magnetic_mu(Dims d, const double *__restrict__ phi, double chi, double bw,
                                                     double inv_bw, long long khi, long long klo,
                                                     double one_plus_chi, Coef<double> cf, SplitOut so) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= d.nz || j >= d.ny) return;
    const long long c = cid(d, i, j, k);
    const double pc = phi[c];
    const long long sx = (long long)d.ny * d.nz;
    const double mx = i > 0 ? mu_face_fast(phi[c - sx], pc, chi, bw, inv_bw, khi, klo, one_plus_chi) : 0.0;
    const double my = j > 0 ? mu_face_fast(phi[c - d.nz], pc, chi, bw, inv_bw, khi, klo, one_plus_chi) : 0.0;
    const double mz = k > 0 ? mu_face_fast(phi[c - 1], pc, chi, bw, inv_bw, khi, klo, one_plus_chi) : 0.0;
    cf.ax[c] = mx;
    cf.ay[c] = my;
    cf.az[c] = mz;
    // the excess is 0 on every potential row; the row flag is set by k_magnetic_rows (D > 0)
    if (so.rows) split_store(so, d, i, j, k, mx, my, mz, 0., false);
}

// BuildMatrix, row pass + AssembleRHS (core/MagneticField.cpp:62-118) in Neumann form: D = sum of mu over the
// in-grid faces in the reference's face order, rhs = sum (mu - 1) Hext (-side) h in the same order (faces with
// mu == 1 add a signed zero, which leaves the sum unchanged, and are skipped).  Row 0 keeps its unpinned value:
// the reference's pinned row 0 is recovered by the psi[0] = 0 gauge after the solve.
//
// Fast paths with the same bits, for interior cells whose six face values are one bit pattern: all 1 (air
// away from the interface) gives D = 6 (six ones summed exactly) and rhs = 0; all 1 + chi (liquid away from
// it) gives D = sv6, the six-term sum of 1 + chi formed on the host in the same order, and per face
// (mu - 1) = m1, also formed on the host; the sign -side is an exact negation.  Bit patterns are compared as
// integers, so air cells take no FP64 operation.
__global__ void __launch_bounds__(256) k_magnetic_rows(Dims d, Faces hext, double h, Coef<double> cf,
                                                       double *__restrict__ b, int want_invd,
                                                       long long liq_bits, double m1, double sv6,
                                                       double inv_sv6, uint8_t *__restrict__ rows) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= d.nz || j >= d.ny) return;
    const long long c = cid(d, i, j, k);
    const long long sx = (long long)d.ny * d.nz, sy = d.nz;
    if (rows) rows[(long long)i * d.ny + j] = 1;  // D > 0: every in-grid mu is at least 1
    if (i > 0 && i < d.nx - 1 && j > 0 && j < d.ny - 1 && k > 0 && k < d.nz - 1) {
        const long long m[6] = {__double_as_longlong(cf.ax[c]), __double_as_longlong(cf.ax[c + sx]),
                                __double_as_longlong(cf.ay[c]), __double_as_longlong(cf.ay[c + sy]),
                                __double_as_longlong(cf.az[c]), __double_as_longlong(cf.az[c + 1])};
        const bool air = (m[0] == kOneBits) & (m[1] == kOneBits) & (m[2] == kOneBits) & (m[3] == kOneBits) &
                         (m[4] == kOneBits) & (m[5] == kOneBits);
        const bool liq = (m[0] == liq_bits) & (m[1] == liq_bits) & (m[2] == liq_bits) & (m[3] == liq_bits) &
                         (m[4] == liq_bits) & (m[5] == liq_bits);
        if (air) {
            cf.dex[c] = 0.;
            cf.D[c] = 6.;
            if (want_invd) cf.invd[c] = 1. / 6.;
            b[c] = 0.;
            return;
        }
        if (liq) {
            double rhs = 0.;
            rhs += (m1 * hext.p[0][fid(d, 0, i, j, k)]) * h;       // ord -x: -side = +1
            rhs += -(m1 * hext.p[0][fid(d, 0, i + 1, j, k)]) * h;  // ord +x: -side = -1
            rhs += (m1 * hext.p[1][fid(d, 1, i, j, k)]) * h;
            rhs += -(m1 * hext.p[1][fid(d, 1, i, j + 1, k)]) * h;
            rhs += (m1 * hext.p[2][fid(d, 2, i, j, k)]) * h;
            rhs += -(m1 * hext.p[2][fid(d, 2, i, j, k + 1)]) * h;
            cf.dex[c] = 0.;
            cf.D[c] = sv6;
            if (want_invd) cf.invd[c] = inv_sv6;
            b[c] = rhs;
            return;
        }
    }
    double diag = 0., rhs = 0.;
    // (mu, valid, face index) in ord order -x, +x, -y, +y, -z, +z
#pragma unroll
    for (int ord = 0; ord < 6; ord++) {
        const int a = ord >> 1, up = ord & 1;
        const int ia = a == 0 ? i : (a == 1 ? j : k);
        const int na = a == 0 ? d.nx : (a == 1 ? d.ny : d.nz);
        if (up ? (ia >= na - 1) : (ia <= 0)) continue;
        const long long st = a == 0 ? sx : (a == 1 ? sy : 1);
        const double *arr = a == 0 ? cf.ax : (a == 1 ? cf.ay : cf.az);
        const double mu = up ? arr[c + st] : arr[c];
        diag += mu;
        if (__double_as_longlong(mu) != kOneBits) {
            const int fi = i + (a == 0) * up, fj = j + (a == 1) * up, fk = k + (a == 2) * up;
            const double side = up ? 1.0 : -1.0;
            rhs += (mu - 1.) * hext.p[a][fid(d, a, fi, fj, fk)] * (-side) * h;
        }
    }
    cf.dex[c] = 0.;
    cf.D[c] = diag;
    if (want_invd) cf.invd[c] = diag > 0 ? 1. / diag : 0.;
    b[c] = rhs;
}

// AssignTotalField (core/MagneticField.cpp:125-143): H = (psi_c0 - psi_c1) / h + Hext on faces with both cells in
// the grid, H = Hext on the grid's boundary faces.  One thread per node (i, j, k) of the cell grid writes the lower
// x, y and z faces of cell (i, j, k), in one launch over (nx + 1) x (ny + 1) x (nz + 1) points, so psi of the cell
// is loaded once for its three faces.
__global__ void __launch_bounds__(256) k_total_field3(Dims d, const double *__restrict__ psi, Faces hext, double invh,
                                                      Faces H) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k > d.nz || j > d.ny || i > d.nx) return;
    const bool cell = i < d.nx && j < d.ny && k < d.nz;
    const long long c1 = cell ? cid(d, i, j, k) : 0;
    const double p1 = cell ? psi[c1] : 0.0;
    const long long sx = (long long)d.ny * d.nz, sy = d.nz;
    if (j < d.ny && k < d.nz) {
        const long long f = fid(d, 0, i, j, k);
        double v = 0.;
        if (i > 0 && i < d.nx) v = (psi[c1 - sx] - p1) * invh;
        v += hext.p[0][f];
        const_cast<double *>(H.p[0])[f] = v;
    }
    if (i < d.nx && k < d.nz) {
        const long long f = fid(d, 1, i, j, k);
        double v = 0.;
        if (j > 0 && j < d.ny) v = (psi[c1 - sy] - p1) * invh;
        v += hext.p[1][f];
        const_cast<double *>(H.p[1])[f] = v;
    }
    if (i < d.nx && j < d.ny) {
        const long long f = fid(d, 2, i, j, k);
        double v = 0.;
        if (k > 0 && k < d.nz) v = (psi[c1 - 1] - p1) * invh;
        v += hext.p[2][f];
        const_cast<double *>(H.p[2])[f] = v;
    }
}

// ---------------------------------------------------------------------------------- allocation-free residual
// Scratch of the allocation-free residual: the deterministic reduction's block partials (2 sums per block and
// per group of kRedGroup blocks) and its tickets.  File-scope device memory (about 130 KB), so a call
// allocates nothing.  One copy per device; calls that overlap on the GPU share it and race.
constexpr int kNoAllocBlocks = 8192;  // = SF_NOALLOC_MAX_BLOCKS of the C ABI
constexpr int kNoAllocGroups = (kNoAllocBlocks + kRedGroup - 1) / kRedGroup;
static __device__ __align__(256) double g_noalloc_part[2 * (kNoAllocBlocks + kNoAllocGroups)];
static __device__ __align__(256) unsigned g_noalloc_ticket[1 + kNoAllocGroups];

// ||b - A psi|| / ||b|| on the reference's pinned system (core/MagneticField.cpp:62-118): row 0 is psi_0 = 0
// with b_0 = 0, the other rows drop column 0.  mu, D and b are formed per cell exactly as k_magnetic_mu and
// k_magnetic_rows form them (each face value is evaluated by both of its cells), so nothing is stored.
// Tiles of 32 (z) x 8 (y) cells, `xpb` x-planes per block; result[0] = relative residual, result[1] = ||b||.
__global__ void __launch_bounds__(256) k_magnetic_residual(Dims d, int xpb, const double *__restrict__ phi,
                                                           double chi, double bw, double inv_bw, long long khi,
                                                           long long klo,
                                                           double one_plus_chi, Faces hext, double h,
                                                           const double *__restrict__ psi, double *part,
                                                           unsigned *ticket, double *result) {
    double v[2] = {0., 0.};  // (r, r), (b, b)
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    if (k < d.nz && j < d.ny) {
        const long long sx = (long long)d.ny * d.nz, sy = d.nz;
        const int i_end = min(d.nx, (int)(blockIdx.z + 1) * xpb);
        for (int i = blockIdx.z * xpb; i < i_end; i++) {
            const long long c = cid(d, i, j, k);
            if (c == 0) {  // pinned row: 1 * psi_0 = 0
                const double r0 = -psi[0];
                v[0] += r0 * r0;
                continue;
            }
            const double pc = phi[c];
            double diag = 0., rhs = 0., s = 0.;
#pragma unroll
            for (int ord = 0; ord < 6; ord++) {  // -x, +x, -y, +y, -z, +z
                const int a = ord >> 1, up = ord & 1;
                const int ia = a == 0 ? i : (a == 1 ? j : k);
                const int na = a == 0 ? d.nx : (a == 1 ? d.ny : d.nz);
                if (up ? (ia >= na - 1) : (ia <= 0)) continue;
                const long long st = a == 0 ? sx : (a == 1 ? sy : 1);
                const long long nb = up ? c + st : c - st;
                const double pn = phi[nb];
                const double mu = up ? mu_face_fast(pc, pn, chi, bw, inv_bw, khi, klo, one_plus_chi)
                                     : mu_face_fast(pn, pc, chi, bw, inv_bw, khi, klo, one_plus_chi);
                diag += mu;
                if (mu != 1.) {
                    const int fi = i + (a == 0) * up, fj = j + (a == 1) * up, fk = k + (a == 2) * up;
                    const double side = up ? 1.0 : -1.0;
                    rhs += (mu - 1.) * hext.p[a][fid(d, a, fi, fj, fk)] * (-side) * h;
                }
                if (nb != 0) s += mu * psi[nb];
            }
            const double rc = (rhs - diag * psi[c]) + s;
            v[0] += rc * rc;
            v[1] += rhs * rhs;
        }
    }
    double tot[2];
    if (grid_reduce<2>(v, part, ticket, tot)) {
        result[0] = tot[1] > 0. ? sqrt(tot[0] / tot[1]) : sqrt(tot[0]);
        result[1] = sqrt(tot[1]);
    }
}

__global__ void k_copy(long long n, const double *__restrict__ a, double *__restrict__ o) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        o[c] = a[c];
}

static inline int flat_grid(long long n) {
    long long g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    if (g < 1) g = 1;
    return (int)g;
}

// ------------------------------------------------------------------------------------------------ launchers
void launch_build_pressure(cudaStream_t st, const Dims &d, const double *phi, const Faces &frac, const Faces &u,
                           const Faces &us, const Faces &jump, double vol_error, Coef<double> &cf, double *b,
                           bool rhs_only, bool want_invd, const SplitOut *so) {
    SplitOut o{};
    if (so && !rhs_only) {
        o = *so;
        cudaMemsetAsync(o.rows, 0, (size_t)d.nx * d.ny, st);
    }
    k_build_pressure<<<grid3(d.nx, d.ny, d.nz), blk2(), 0, st>>>(d, phi, frac, u, us, jump, vol_error, cf, b,
                                                                  rhs_only ? 1 : 0, want_invd ? 1 : 0, o);
}

void launch_apply_projection(cudaStream_t st, const Dims &d, const double *phi, const Faces &frac, const Faces &jump,
                             const double *p, const Faces &u) {
    k_apply_projection3<<<grid3(d.nx + 1, d.ny + 1, d.nz + 1), blk2(), 0, st>>>(d, phi, frac, jump, p, u);
}

void launch_gather_cells(cudaStream_t st, long long n, const double *D, const double *x, double *out) {
    k_gather_cells<<<flat_grid(n), 256, 0, st>>>(n, D, x, out);
}

int launch_build_magnetic(cudaStream_t st, const Dims &d, const double *phi, double chi, double bw,
                          const Faces &hext, double h, Coef<double> &cf, double *b, bool want_invd,
                          const SplitOut *so) {
    // band thresholds as integer keys: |phi| > bw (1 + 2^-40) on both cells implies |phi_face| > bw exactly
    const double t = bw * (1.0 + std::ldexp(1.0, -40));
    auto key = [](double v) {
        long long b;
        std::memcpy(&b, &v, 8);
        return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
    };
    const double one_plus_chi = 1. + (1. - 0.) * chi;  // the reference's expression with H = 0
    // the rows kernel's constants for cells whose six faces are 1 + chi: the diagonal summed in face order
    // from 0, its reciprocal, and mu - 1
    double sv6 = 0.;
    for (int q = 0; q < 6; q++) sv6 += one_plus_chi;
    const double m1 = one_plus_chi - 1.;
    long long liq_bits;
    std::memcpy(&liq_bits, &one_plus_chi, 8);
    SplitOut o{};
    if (so) o = *so;
    // two passes: mu of each face is formed once (band faces take FP64 sinpi, which a fused pass forming the
    // upper faces again would evaluate twice) and the row pass reads it back
    k_magnetic_mu<<<grid3(d.nx, d.ny, d.nz), blk2(), 0, st>>>(d, phi, chi, bw, 1.0 / bw, key(t), key(-t),
                                                              one_plus_chi, cf, o);
    k_magnetic_rows<<<grid3(d.nx, d.ny, d.nz), blk2(), 0, st>>>(d, hext, h, cf, b, want_invd ? 1 : 0, liq_bits, m1,
                                                                 sv6, sv6 > 0 ? 1. / sv6 : 0., o.rows);
    return 2;
}

bool noalloc_fits(const Dims &d) {
    return (long long)((d.nz + 31) / 32) * ((d.ny + 7) / 8) <= kNoAllocBlocks;
}

// Device addresses of the scratch in the calling thread's current context, looked up on every call (a host-side
// query, no allocation once the module is loaded), so that no address outlives its context (cudaDeviceReset, a
// caller that switches driver contexts on the same device).
namespace {
cudaError_t noalloc_scratch(double **part, unsigned **ticket) {
    void *p = nullptr, *t = nullptr;
    cudaError_t e;
    if ((e = cudaGetSymbolAddress(&p, g_noalloc_part)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress(&t, g_noalloc_ticket)) != cudaSuccess) return e;
    *part = static_cast<double *>(p);
    *ticket = static_cast<unsigned *>(t);
    return cudaSuccess;
}
}  // namespace

cudaError_t launch_magnetic_residual_noalloc(cudaStream_t st, const Dims &d, const double *phi, double chi,
                                             double bw, const Faces &hext, double h, const double *psi,
                                             double *result) {
    double *part = nullptr;
    unsigned *ticket = nullptr;
    cudaError_t e = noalloc_scratch(&part, &ticket);
    if (e != cudaSuccess) return e;
    // at most kNoAllocBlocks / tiles blocks along x: the grid never exceeds the scratch (tiles <= kNoAllocBlocks)
    const long long tiles = (long long)((d.nz + 31) / 32) * ((d.ny + 7) / 8);
    if (tiles > kNoAllocBlocks) return cudaErrorInvalidValue;
    const long long zmax = kNoAllocBlocks / tiles;
    const int xpb = (int)((d.nx + zmax - 1) / zmax);
    const dim3 grid((d.nz + 31) / 32, (d.ny + 7) / 8, (d.nx + xpb - 1) / xpb);
    // the tickets must start at zero (the reduction re-arms them, but a call cut short would not)
    if ((e = cudaMemsetAsync(ticket, 0, sizeof(g_noalloc_ticket), st)) != cudaSuccess) return e;
    const double t = bw * (1.0 + std::ldexp(1.0, -40));  // same band keys as launch_build_magnetic
    auto key = [](double v) {
        long long b;
        std::memcpy(&b, &v, 8);
        return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
    };
    const double one_plus_chi = 1. + (1. - 0.) * chi;
    k_magnetic_residual<<<grid, blk2(), 0, st>>>(d, xpb, phi, chi, bw, 1.0 / bw, key(t), key(-t), one_plus_chi, hext,
                                                 h, psi, part, ticket, result);
    return cudaGetLastError();
}

void launch_total_field(cudaStream_t st, const Dims &d, const double *psi, const Faces &hext, double invh,
                        const Faces &H) {
    k_total_field3<<<grid3(d.nx + 1, d.ny + 1, d.nz + 1), blk2(), 0, st>>>(d, psi, hext, invh, H);
}

__global__ void k_to_f32(long long n, const double *__restrict__ a, float *__restrict__ o) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        o[c] = f64_to_f32(a[c]);
}

void launch_to_f32(cudaStream_t st, long long n, const double *a, float *o) {
    k_to_f32<<<flat_grid(n), 256, 0, st>>>(n, a, o);
}

void launch_copy(cudaStream_t st, long long n, const double *a, double *o) {
    k_copy<<<flat_grid(n), 256, 0, st>>>(n, a, o);
}

}  // namespace sf
