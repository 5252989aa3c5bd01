// sf_ops.h -- launchers of the assembly and post-solve kernels (sf_ops.cu).
#pragma once
#include <cuda_runtime.h>

#include "sf_internal.cuh"

namespace sf {

// Three face arrays (x, y, z face grids) in the reference's layout; p[0] == nullptr means "absent".
struct Faces {
    const double *p[3];
};

void launch_build_pressure(cudaStream_t st, const Dims &d, const double *phi, const Faces &frac, const Faces &u,
                           const Faces &us, const Faces &jump, double vol_error, Coef<double> &cf, double *b,
                           bool rhs_only, bool want_invd, const SplitOut *so = nullptr);
void launch_apply_projection(cudaStream_t st, const Dims &d, const double *phi, const Faces &frac, const Faces &jump,
                             const double *p, const Faces &u);
void launch_gather_cells(cudaStream_t st, long long n, const double *D, const double *x, double *out);
int launch_build_magnetic(cudaStream_t st, const Dims &d, const double *phi, double chi, double bw,
                          const Faces &hext, double h, Coef<double> &cf, double *b, bool want_invd,
                          const SplitOut *so = nullptr);
void launch_total_field(cudaStream_t st, const Dims &d, const double *psi, const Faces &hext, double invh,
                        const Faces &H);
// Allocation-free residual of a potential on the pinned magnetostatic system (static scratch, see sf_ops.cu).
bool noalloc_fits(const Dims &d);
cudaError_t launch_magnetic_residual_noalloc(cudaStream_t st, const Dims &d, const double *phi, double chi,
                                             double bw, const Faces &hext, double h, const double *psi,
                                             double *result);
// Velocity pipeline after the projection (sf_post.cu).
void launch_extrapolate(cudaStream_t st, const Dims &d, const double *phi, const Faces &frac, double *const u[3],
                        uint8_t *const valid[3], uint8_t *const valid1[3], double clear_val, int max_steps);
void launch_enforce(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &old,
                    const Faces &us, const Faces &normal, const Faces &frac, double *const u[3]);
void launch_vertex_pressures(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &H,
                             double chi, const double *pos, const double *nrm, long long nv, double *out);
void launch_pressure_jump(cudaStream_t st, const Dims &d, const int32_t *const edge_mark[3], const double *kappa,
                          const double *pm, double sigma, double rho, double h, double dt, double *const jump[3]);
void launch_advect_levelset(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &u,
                            double dt, const double *phi, double *out);
void launch_advect_velocity(cudaStream_t st, const Dims &d, const double origin[3], double h, const Faces &u,
                            double dt, double *const out[3]);
void launch_reinitialize(cudaStream_t st, const Dims &d, double h, double *phi, double *p1, double *p2,
                         int max_steps);
void launch_copy(cudaStream_t st, long long n, const double *a, double *o);
void launch_to_f32(cudaStream_t st, long long n, const double *a, float *o);

}  // namespace sf
