// sf_api.cu -- the C ABI (include/sfgpu.h): context, host<->device staging and the two solve entry points.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "sf_ops.h"
#include "sf_solver.h"
#include "sf_unet.h"
#include "sfgpu.h"

using namespace sf;

namespace {

struct Ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::string err;
    std::unique_ptr<MGSolver> pres, mag;
    bool pres_ready = false;
    int pres_prec = -1;
    Dims pres_dims{0, 0, 0, 0};
    bool mag_has_x = false;
    Dims mag_dims{0, 0, 0, 0};
    // staging buffers for the host-pointer entry points
    DevBuf phi, frac[3], vel[3], us[3], jump[3], hext[3], H[3], cells;
    // velocity pipeline after the projection: extrapolation masks, enforce's copy of the old velocity, normals
    DevBuf mask[6], old[3], normal[3];
    // interface coupling: mesh vertices, vertex values and edge marks
    DevBuf vpos, vnrm, vval, kappa, edge[3];
    // level-set operations: two scratch cell fields
    DevBuf ls1, ls2;
    // learned form: attached network (not owned) and its buffers; every network created on this context is
    // registered so that destroying the context first leaves the network handles safe to destroy later
    UNet *net = nullptr;
    std::vector<void *> nets;
    DevBuf feat, guess;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // resident inputs: the collider (fractions, optional velocity) and a level set, read by calls that pass NULL
    DevBuf rfrac[3], rus[3], rphi;
    bool rcol = false, rcol_us = false, rls = false;
    Dims rcol_dims{0, 0, 0, 0}, rls_dims{0, 0, 0, 0};
    // applied field of a later magnetic call (sf_applied_field_prefetch), copied into its own buffers on a side
    // stream once the next pressure call's inputs are on the device, or by the magnetic call that reads it
    DevBuf pfield[3];
    cudaStream_t cst = nullptr;
    cudaEvent_t ev_in = nullptr, ev_field = nullptr;
    const double *field_src[3] = {nullptr, nullptr, nullptr};
    bool field_pending = false, field_ready = false, field_fresh = false;
    Dims field_dims{0, 0, 0, 0};
    long long field_n[3] = {0, 0, 0}, field_bytes = 0;
};

Ctx *C(void *p) { return reinterpret_cast<Ctx *>(p); }

sf_status fail(Ctx *c, sf_status s, const std::string &msg) {
    if (c) c->err = msg;
    return s;
}

sf_status cuda_fail(Ctx *c, cudaError_t e, const char *where) {
    return fail(c, e == cudaErrorMemoryAllocation ? SF_OUT_OF_MEMORY : SF_CUDA_ERROR,
                std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call);          \
    } while (0)

bool grid_ok(const sf_grid *g) {
    return g && g->nx > 0 && g->ny > 0 && g->nz > 0 && g->h > 0 && std::isfinite(g->h) &&
           (long long)g->nx * g->ny * g->nz < (1LL << 31) && (long long)(g->nx + 1) * (g->ny + 1) * (g->nz + 1) < (1LL << 31);
}

long long face_count(const sf_grid *g, int a) {
    return (long long)(g->nx + (a == 0)) * (g->ny + (a == 1)) * (g->nz + (a == 2));
}

SolverParams params_from(const sf_solve_opts *o, int which) {
    sf_solve_opts def;
    sf_default_opts(&def, which);
    if (!o) o = &def;
    SolverParams p;
    p.precision = o->precision == SF_PREC_FP64 ? 0 : 1;  // the learned form runs the mixed solver
    p.tol = o->tol > 0 ? o->tol : def.tol;
    p.max_iters = o->max_iters > 0 ? o->max_iters : def.max_iters;
    p.pre = o->pre_smooth > 0 ? o->pre_smooth : def.pre_smooth;
    p.post = o->post_smooth > 0 ? o->post_smooth : def.post_smooth;
    p.coarse_sweeps = o->coarse_sweeps > 0 ? o->coarse_sweeps : def.coarse_sweeps;
    p.coarse_pre = o->coarse_pre > 0 ? o->coarse_pre : p.pre;
    p.coarse_post = o->coarse_post > 0 ? o->coarse_post : p.post;
    p.max_levels = o->max_levels;
    p.coarse_dim = o->coarse_dim > 0 ? o->coarse_dim : def.coarse_dim;
    p.use_graph = o->use_graph != 0;
    p.check_every = o->check_every > 0 ? o->check_every : 1;
    p.inner_tol = o->inner_tol > 0 ? o->inner_tol : def.inner_tol;
    p.flexible = false;
    p.profile = o->profile != 0;
    p.smoother = o->smoother;
    p.tail = o->coarse_tail;
    p.full_sweeps = o->full_sweeps != 0;
    return p;
}

bool opts_ok(const sf_solve_opts *o) {
    if (!o) return true;
    if (o->precision != SF_PREC_FP64 && o->precision != SF_PREC_MIXED && o->precision != SF_PREC_LEARNED) return false;
    if (o->max_levels < 0 || o->coarse_dim < 0) return false;
    if (o->smoother < 0 || o->smoother > 3) return false;
    if (o->coarse_tail != 0 && o->coarse_tail != 1 && o->coarse_tail != 8 && o->coarse_tail != 16) return false;
    return true;
}

// Stage a host array into a device buffer (or pass a device pointer through).
sf_status stage_in(Ctx *c, DevBuf &buf, const double *src, long long n, bool dev, const double **out, long long &h2d) {
    if (!src) {
        *out = nullptr;
        return SF_OK;
    }
    if (dev) {
        *out = src;
        return SF_OK;
    }
    CK(buf.ensure(8 * (size_t)n));
    CK(cudaMemcpyAsync(buf.get(), src, 8 * (size_t)n, cudaMemcpyHostToDevice, c->st));
    h2d += 8 * n;
    *out = (const double *)buf.get();
    return SF_OK;
}

void fill_stats(sf_solve_stats *s, const SolveResult &r, long long unknowns) {
    if (!s) return;
    s->iters = r.iters;
    s->outer_iters = r.outer;
    s->levels = r.levels;
    s->converged = r.converged ? 1 : 0;
    s->unknowns = unknowns;
    s->smooth_launches = r.smooth_launches;
    s->smooth_ms = r.smooth_ms;
    s->smooth_bytes = r.smooth_bytes;
    s->guess_rel_residual = r.guess_relres;
    s->guess_energy_ratio = r.guess_energy;
    s->learned_steps = r.learned_steps;
}

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// The learned form's network as the solver's correction step: features of the assembled system are formed once
// per solve; each step rewrites their right-hand-side channel with the current residual and runs the U-Net.
struct NetStep final : LearnedStep {
    Ctx *c = nullptr;
    Dims d{0, 0, 0, 0};
    __nv_bfloat16 *feat = nullptr;
    cudaError_t predict(const float *r, double rr, float *y) override {
        const double cnt = c->net->active_cells() > 0 ? c->net->active_cells() : 1.0;
        const double rms = std::sqrt(rr / cnt);
        cudaError_t e = c->net->set_rhs_channel(d, r, rms > 0 ? 1.0 / rms : 0.0, feat);
        if (e != cudaSuccess) return e;
        if ((e = c->net->forward(d, feat, y, false)) != cudaSuccess) return e;
        if (c->net->mode() >= 1 && (e = c->net->check_device_errors()) != cudaSuccess) return e;
        return cudaSuccess;
    }
};

// Detaches the step from the solver when the solve returns, on every path.
struct LearnedScope {
    MGSolver *S = nullptr;
    ~LearnedScope() {
        if (S) S->set_learned(nullptr);
    }
};

sf_status learned_prepare(Ctx *c, MGSolver &S, const Dims &d, NetStep &step, LearnedScope &scope) {
    if (!c->net) return fail(c, SF_NOT_READY, "learned precision needs a network (sf_set_network)");
    CK(c->feat.ensure(2 * 16 * (size_t)d.n));
    step.c = c;
    step.d = d;
    step.feat = (__nv_bfloat16 *)c->feat.get();
    CK(c->net->features(d, S.fine(), S.b(), step.feat));
    S.set_learned(&step);
    scope.S = &S;
    return SF_OK;
}

bool same_dims(const Dims &a, const Dims &b) { return a.nx == b.nx && a.ny == b.ny && a.nz == b.nz; }

// Starts a pending applied-field prefetch on the side stream, after everything enqueued on the context's stream so
// far (a pressure call's input copies): the copy then runs under the pressure solve and its output copies.
sf_status start_field_copy(Ctx *c) {
    if (!c->field_pending) return SF_OK;
    c->field_pending = false;
    CK(cudaEventRecord(c->ev_in, c->st));
    CK(cudaStreamWaitEvent(c->cst, c->ev_in, 0));
    for (int a = 0; a < 3; a++)
        CK(cudaMemcpyAsync(c->pfield[a].get(), c->field_src[a], 8 * (size_t)c->field_n[a], cudaMemcpyDefault, c->cst));
    CK(cudaEventRecord(c->ev_field, c->cst));
    c->field_ready = true;
    c->field_fresh = true;
    return SF_OK;
}

// The resident level set (phi == NULL) or the staged / passed-through one.
sf_status level_set_in(Ctx *c, const double *phi, const Dims &d, bool dev, const double **out, long long &h2d) {
    if (phi) return stage_in(c, c->phi, phi, d.n, dev, out, h2d);
    if (!c->rls || !same_dims(c->rls_dims, d))
        return fail(c, SF_NOT_READY, "phi is NULL and no level set of this grid was uploaded (sf_levelset_upload)");
    *out = (const double *)c->rphi.get();
    return SF_OK;
}

// ------------------------------------------------------------------------------------------------ pressure
sf_status pressure_impl(Ctx *c, const sf_grid *g, double *const vel[3], const double *phi, const double *const frac[3],
                        const double *const us[3], const double *const jump[3], double vol_error, double *p_out,
                        const sf_solve_opts *opts, sf_solve_stats *stats, bool dev, bool reproject) {
    auto t0 = std::chrono::steady_clock::now();
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !vel || !opts_ok(opts)) return fail(c, SF_BAD_ARG, "bad grid, pointer or option");
    for (int a = 0; a < 3; a++)
        if (!vel[a] || (frac && !frac[a])) return fail(c, SF_BAD_ARG, "null velocity or fraction array");
    if (us)
        for (int a = 0; a < 3; a++)
            if (!us[a]) return fail(c, SF_BAD_ARG, "solid_vel must hold three arrays or be NULL");
    if (jump)
        for (int a = 0; a < 3; a++)
            if (!jump[a]) return fail(c, SF_BAD_ARG, "jump must hold three arrays or be NULL");
    if (!std::isfinite(vol_error)) return fail(c, SF_BAD_ARG, "vol_error is not finite");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    if (reproject && !(c->pres_ready && c->pres_dims.nx == d.nx && c->pres_dims.ny == d.ny && c->pres_dims.nz == d.nz &&
                       c->pres_prec == (opts ? opts->precision : SF_PREC_FP64)))
        return fail(c, SF_NOT_READY, "Reproject needs a previous Project on the same grid and precision");
    if (stats) memset(stats, 0, sizeof(*stats));
    long long h2d = 0, d2h = 0;
    const double *dphi;
    Faces ffrac{}, fvel{}, fus{}, fjump{};
    sf_status s;
    if (!frac && !(c->rcol && same_dims(c->rcol_dims, d)))
        return fail(c, SF_NOT_READY, "frac is NULL and no collider of this grid was uploaded (sf_collider_upload)");
    if ((s = level_set_in(c, phi, d, dev, &dphi, h2d)) != SF_OK) return s;
    for (int a = 0; a < 3; a++) {
        const long long nf = face_count(g, a);
        if (frac) {
            if ((s = stage_in(c, c->frac[a], frac[a], nf, dev, &ffrac.p[a], h2d)) != SF_OK) return s;
        } else {
            ffrac.p[a] = (const double *)c->rfrac[a].get();  // the resident collider
        }
        if ((s = stage_in(c, c->vel[a], vel[a], nf, dev, &fvel.p[a], h2d)) != SF_OK) return s;
        if (!frac && !us && c->rcol_us) {
            fus.p[a] = (const double *)c->rus[a].get();
        } else if ((s = stage_in(c, c->us[a], us ? us[a] : nullptr, nf, dev, &fus.p[a], h2d)) != SF_OK) {
            return s;
        }
        if ((s = stage_in(c, c->jump[a], jump ? jump[a] : nullptr, nf, dev, &fjump.p[a], h2d)) != SF_OK) return s;
    }
    if ((s = start_field_copy(c)) != SF_OK) return s;  // a prefetched applied field, under this solve
    if (!c->pres) c->pres = std::make_unique<MGSolver>(c->st);
    MGSolver &S = *c->pres;
    SolverParams prm = params_from(opts, 0);
    CK(S.configure(d, prm));
    CK(cudaEventRecord(c->ev[0], c->st));
    // 1/D is read only by FP64 smoothers
    launch_build_pressure(c->st, d, dphi, ffrac, fvel, fus, fjump, vol_error, S.fine(), S.b(), reproject,
                          prm.precision == 0, reproject ? nullptr : S.split_targets());
    if (!reproject) CK(S.build_hierarchy());
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->ev[1], c->st));
    SolveResult res;
    const bool zero = !reproject;  // Project starts from zero (core/Pressure.cpp:122); Reproject from the last p
    NetStep step;
    LearnedScope scope;
    if (opts && opts->precision == SF_PREC_LEARNED && !reproject) {
        sf_status ls = learned_prepare(c, S, d, step, scope);
        if (ls != SF_OK) return ls;
    }
    CK(S.solve(zero, res));
    double relres = res.relres, bn = res.bnorm;
    const bool report = !opts || opts->report_ref_residual;
    // the mixed form's refinement ends on an FP64 residual of the returned x: res.relres is already the true
    // relative residual; the FP64 form's PCG reports its recurrence, so it is recomputed
    if (report && prm.precision == 0) CK(S.true_relres(false, relres, bn));
    CK(cudaEventRecord(c->ev[2], c->st));
    launch_apply_projection(c->st, d, dphi, ffrac, fjump, S.x(), fvel);
    double *pdst = nullptr;
    if (p_out) {
        if (dev) {
            pdst = p_out;
        } else {
            CK(c->cells.ensure(8 * (size_t)d.n));
            pdst = (double *)c->cells.get();
        }
        launch_gather_cells(c->st, d.n, S.fine().D, S.x(), pdst);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->ev[3], c->st));
    if (!dev) {
        for (int a = 0; a < 3; a++) {
            const long long nf = face_count(g, a);
            CK(cudaMemcpyAsync(vel[a], fvel.p[a], 8 * (size_t)nf, cudaMemcpyDeviceToHost, c->st));
            d2h += 8 * nf;
        }
        if (p_out) {
            CK(cudaMemcpyAsync(p_out, pdst, 8 * (size_t)d.n, cudaMemcpyDeviceToHost, c->st));
            d2h += 8 * d.n;
        }
    }
    CK(cudaStreamSynchronize(c->st));
    c->pres_ready = true;
    c->pres_prec = prm.precision;
    c->pres_dims = d;
    fill_stats(stats, res, -1);
    if (stats) stats->kernel_launches = S.take_launches() + 1 + 1 + (p_out ? 1 : 0);
    if (stats) {
        stats->rel_residual = relres;
        stats->rel_residual_ref = relres;
        stats->ms_build = ev_ms(c->ev[0], c->ev[1]);
        stats->ms_solve = ev_ms(c->ev[1], c->ev[2]);
        stats->ms_post = ev_ms(c->ev[2], c->ev[3]);
        stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h;
        stats->status_detail = res.breakdown ? 1 : 0;
    }
    if (!res.converged) return fail(c, SF_NOT_CONVERGED, "pressure solve did not reach the tolerance");
    return res.fallback ? SF_STALLED_FALLBACK : SF_OK;
}

// ------------------------------------------------------------------------------------------------ magnetic
sf_status magnetic_impl(Ctx *c, const sf_grid *g, const double *phi, double chi, double bw, const double *const hext[3],
                        double *psi_out, double *const H_out[3], const sf_solve_opts *opts, sf_solve_stats *stats,
                        bool dev) {
    auto t0 = std::chrono::steady_clock::now();
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !opts_ok(opts) || !std::isfinite(chi) || !(bw > 0) || !std::isfinite(bw))
        return fail(c, SF_BAD_ARG, "bad grid, chi, band width or option");
    if (hext)
        for (int a = 0; a < 3; a++)
            if (!hext[a]) return fail(c, SF_BAD_ARG, "null applied-field array");
    if (H_out)
        for (int a = 0; a < 3; a++)
            if (!H_out[a]) return fail(c, SF_BAD_ARG, "H_out must hold three arrays or be NULL");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    if (stats) memset(stats, 0, sizeof(*stats));
    long long h2d = 0, d2h = 0;
    const double *dphi;
    Faces fh{};
    sf_status s;
    if ((s = level_set_in(c, phi, d, dev, &dphi, h2d)) != SF_OK) return s;
    if (hext) {
        for (int a = 0; a < 3; a++)
            if ((s = stage_in(c, c->hext[a], hext[a], face_count(g, a), dev, &fh.p[a], h2d)) != SF_OK) return s;
    } else {  // the prefetched applied field
        if ((s = start_field_copy(c)) != SF_OK) return s;
        if (!c->field_ready || !same_dims(c->field_dims, d))
            return fail(c, SF_NOT_READY,
                        "hext is NULL and no applied field of this grid was prefetched (sf_applied_field_prefetch)");
        CK(cudaStreamWaitEvent(c->st, c->ev_field, 0));
        for (int a = 0; a < 3; a++) fh.p[a] = (const double *)c->pfield[a].get();
        if (c->field_fresh) h2d += c->field_bytes;
        c->field_fresh = false;
    }
    if (!c->mag) c->mag = std::make_unique<MGSolver>(c->st);
    MGSolver &S = *c->mag;
    SolverParams prm = params_from(opts, 1);
    const bool same_grid = c->mag_has_x && c->mag_dims.nx == d.nx && c->mag_dims.ny == d.ny && c->mag_dims.nz == d.nz;
    CK(S.configure(d, prm));
    const bool warm = (!opts || opts->warm_start) && same_grid;
    CK(cudaEventRecord(c->ev[0], c->st));
    const int build_launches =
        launch_build_magnetic(c->st, d, dphi, chi, bw, fh, g->h, S.fine(), S.b(), prm.precision == 0, S.split_targets());
    CK(S.build_hierarchy());
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->ev[1], c->st));
    SolveResult res;
    const bool zero = !warm;
    NetStep step;
    LearnedScope scope;
    if (opts && opts->precision == SF_PREC_LEARNED) {
        sf_status ls = learned_prepare(c, S, d, step, scope);
        if (ls != SF_OK) return ls;
    }
    CK(S.solve(zero, res));
    CK(S.shift_to_zero_at_origin());
    double relres = res.relres, relref = res.relres, bn = res.bnorm;
    const bool report = !opts || opts->report_ref_residual;
    if (report) {
        // mixed form: res.relres is the FP64 residual of x before the shift, which changes it only by rounding
        // (the Neumann operator annihilates constants); the pinned system's residual is evaluated after it
        if (prm.precision == 0) CK(S.true_relres(false, relres, bn));
        CK(S.true_relres(true, relref, bn));
    }
    CK(cudaEventRecord(c->ev[2], c->st));
    const double invh = 1 / g->h;  // Grid::m_InvSpacing
    Faces fH{};
    if (H_out) {
        for (int a = 0; a < 3; a++) {
            if (dev) {
                fH.p[a] = H_out[a];
            } else {
                CK(c->H[a].ensure(8 * (size_t)face_count(g, a)));
                fH.p[a] = (const double *)c->H[a].get();
            }
        }
        launch_total_field(c->st, d, S.x(), fh, invh, fH);
    }
    if (psi_out && dev) launch_copy(c->st, d.n, S.x(), psi_out);
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->ev[3], c->st));
    if (!dev) {
        if (H_out)
            for (int a = 0; a < 3; a++) {
                const long long nf = face_count(g, a);
                CK(cudaMemcpyAsync(H_out[a], fH.p[a], 8 * (size_t)nf, cudaMemcpyDeviceToHost, c->st));
                d2h += 8 * nf;
            }
        if (psi_out) {
            CK(cudaMemcpyAsync(psi_out, S.x(), 8 * (size_t)d.n, cudaMemcpyDeviceToHost, c->st));
            d2h += 8 * d.n;
        }
    }
    CK(cudaStreamSynchronize(c->st));
    c->mag_has_x = true;
    c->mag_dims = d;
    fill_stats(stats, res, d.n);
    if (stats) stats->kernel_launches = S.take_launches() + build_launches + (H_out ? 1 : 0) + ((psi_out && dev) ? 1 : 0);
    if (stats) {
        stats->rel_residual = relres;
        stats->rel_residual_ref = relref;
        stats->ms_build = ev_ms(c->ev[0], c->ev[1]);
        stats->ms_solve = ev_ms(c->ev[1], c->ev[2]);
        stats->ms_post = ev_ms(c->ev[2], c->ev[3]);
        stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h;
        stats->status_detail = res.breakdown ? 1 : 0;
    }
    if (!res.converged) return fail(c, SF_NOT_CONVERGED, "magnetic solve did not reach the tolerance");
    return res.fallback ? SF_STALLED_FALLBACK : SF_OK;
}

// ----- velocity pipeline after the projection ------------------------------------------------------------
sf_status post_common(Ctx *c, const sf_grid *g, double *const vel[3]) {
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !vel) return fail(c, SF_BAD_ARG, "bad grid or velocity pointer");
    for (int a = 0; a < 3; a++)
        if (!vel[a]) return fail(c, SF_BAD_ARG, "null velocity array");
    return SF_OK;
}

sf_status stage_vel(Ctx *c, const sf_grid *g, double *const vel[3], bool dev, double *dvel[3], long long &h2d) {
    for (int a = 0; a < 3; a++) {
        const double *p;
        sf_status s = stage_in(c, c->vel[a], vel[a], face_count(g, a), dev, &p, h2d);
        if (s != SF_OK) return s;
        dvel[a] = const_cast<double *>(p);
    }
    return SF_OK;
}

sf_status unstage_vel(Ctx *c, const sf_grid *g, double *const vel[3], bool dev, double *const dvel[3]) {
    if (!dev)
        for (int a = 0; a < 3; a++)
            CK(cudaMemcpyAsync(vel[a], dvel[a], 8 * (size_t)face_count(g, a), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    CK(cudaGetLastError());
    return SF_OK;
}

sf_status extrapolate_impl(Ctx *c, const sf_grid *g, double *const vel[3], const double *phi,
                           const double *const frac[3], double clear_val, int max_steps, bool dev) {
    sf_status s = post_common(c, g, vel);
    if (s != SF_OK) return s;
    if (!phi || !frac || !frac[0] || !frac[1] || !frac[2] || max_steps < 0 || !std::isfinite(clear_val))
        return fail(c, SF_BAD_ARG, "bad level set, fraction pointer, step count or clear value");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    long long h2d = 0;
    double *dvel[3];
    const double *dphi;
    Faces ff{};
    if ((s = stage_vel(c, g, vel, dev, dvel, h2d)) != SF_OK) return s;
    if ((s = stage_in(c, c->phi, phi, d.n, dev, &dphi, h2d)) != SF_OK) return s;
    uint8_t *m0[3], *m1[3];
    for (int a = 0; a < 3; a++) {
        if ((s = stage_in(c, c->frac[a], frac[a], face_count(g, a), dev, &ff.p[a], h2d)) != SF_OK) return s;
        CK(c->mask[a].ensure((size_t)face_count(g, a)));
        CK(c->mask[3 + a].ensure((size_t)face_count(g, a)));
        m0[a] = (uint8_t *)c->mask[a].get();
        m1[a] = (uint8_t *)c->mask[3 + a].get();
    }
    launch_extrapolate(c->st, d, dphi, ff, dvel, m0, m1, clear_val, max_steps);
    CK(cudaGetLastError());
    return unstage_vel(c, g, vel, dev, dvel);
}

// Stage n elements of `bytes_per` bytes (host) into buf, or pass a device pointer through.
template <class T>
sf_status stage_raw(Ctx *c, DevBuf &buf, const T *src, long long n, bool dev, const T **out, long long &h2d) {
    if (!src || dev) {
        *out = src;
        return SF_OK;
    }
    CK(buf.ensure(sizeof(T) * (size_t)n));
    CK(cudaMemcpyAsync(buf.get(), src, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, c->st));
    h2d += (long long)sizeof(T) * n;
    *out = (const T *)buf.get();
    return SF_OK;
}

sf_status vertex_pressures_impl(Ctx *c, const sf_grid *g, double chi, const double *const H[3], const double *pos,
                                const double *nrm, long long nv, double *out, bool dev) {
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !H || !H[0] || !H[1] || !H[2] || nv < 0 || (nv > 0 && (!pos || !nrm || !out)) ||
        !std::isfinite(chi))
        return fail(c, SF_BAD_ARG, "bad grid, field, vertex arrays, count or susceptibility");
    if (nv == 0) return SF_OK;
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    long long h2d = 0;
    Faces fh{};
    sf_status s;
    for (int a = 0; a < 3; a++)
        if ((s = stage_in(c, c->H[a], H[a], face_count(g, a), dev, &fh.p[a], h2d)) != SF_OK) return s;
    const double *dpos, *dnrm;
    if ((s = stage_raw(c, c->vpos, pos, 3 * nv, dev, &dpos, h2d)) != SF_OK) return s;
    if ((s = stage_raw(c, c->vnrm, nrm, 3 * nv, dev, &dnrm, h2d)) != SF_OK) return s;
    double *dout = out;
    if (!dev) {
        CK(c->vval.ensure(8 * (size_t)nv));
        dout = (double *)c->vval.get();
    }
    launch_vertex_pressures(c->st, d, g->origin, g->h, fh, chi, dpos, dnrm, nv, dout);
    CK(cudaGetLastError());
    if (!dev) CK(cudaMemcpyAsync(out, dout, 8 * (size_t)nv, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return SF_OK;
}

sf_status pressure_jump_impl(Ctx *c, const sf_grid *g, const int32_t *const edge_mark[3], const double *kappa,
                             const double *pm, long long nv, double sigma, double rho, double dt,
                             double *const jump[3], bool dev) {
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !edge_mark || !jump || nv < 0 || !(rho != 0) || !std::isfinite(rho) || !std::isfinite(dt) ||
        !std::isfinite(sigma) || ((kappa || pm) && nv == 0))
        return fail(c, SF_BAD_ARG, "bad grid, edge marks, jump arrays, vertex count or constants");
    for (int a = 0; a < 3; a++)
        if (!edge_mark[a] || !jump[a]) return fail(c, SF_BAD_ARG, "edge marks and jump arrays come in threes");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    long long h2d = 0;
    sf_status s;
    const int32_t *dem[3];
    for (int a = 0; a < 3; a++) {
        const long long ne = (long long)(g->nx - (a == 0)) * (g->ny - (a == 1)) * (g->nz - (a == 2));
        if ((s = stage_raw(c, c->edge[a], edge_mark[a], ne > 0 ? ne : 0, dev, &dem[a], h2d)) != SF_OK) return s;
    }
    const double *dk, *dpm;
    if ((s = stage_raw(c, c->kappa, kappa, nv, dev, &dk, h2d)) != SF_OK) return s;
    if ((s = stage_raw(c, c->vval, pm, nv, dev, &dpm, h2d)) != SF_OK) return s;
    double *dj[3];
    for (int a = 0; a < 3; a++) {
        if (dev) {
            dj[a] = jump[a];
        } else {
            CK(c->jump[a].ensure(8 * (size_t)face_count(g, a)));
            dj[a] = (double *)c->jump[a].get();
        }
    }
    launch_pressure_jump(c->st, d, dem, dk, dpm, sigma, rho, g->h, dt, dj);
    CK(cudaGetLastError());
    if (!dev)
        for (int a = 0; a < 3; a++)
            CK(cudaMemcpyAsync(jump[a], dj[a], 8 * (size_t)face_count(g, a), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return SF_OK;
}

sf_status stage_cells_inout(Ctx *c, const sf_grid *g, double *phi, bool dev, double **dphi, long long &h2d) {
    const double *p;
    sf_status s = stage_in(c, c->phi, phi, (long long)g->nx * g->ny * g->nz, dev, &p, h2d);
    *dphi = const_cast<double *>(p);
    return s;
}

sf_status advect_levelset_impl(Ctx *c, const sf_grid *g, double *phi, const double *const vel[3], double dt,
                               bool dev) {
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !phi || !vel || !vel[0] || !vel[1] || !vel[2] || !std::isfinite(dt))
        return fail(c, SF_BAD_ARG, "bad grid, level set, velocity or time step");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    long long h2d = 0;
    sf_status s;
    double *dphi;
    if ((s = stage_cells_inout(c, g, phi, dev, &dphi, h2d)) != SF_OK) return s;
    Faces fu{};
    for (int a = 0; a < 3; a++)
        if ((s = stage_in(c, c->vel[a], vel[a], face_count(g, a), dev, &fu.p[a], h2d)) != SF_OK) return s;
    CK(c->ls1.ensure(8 * (size_t)d.n));
    double *out = (double *)c->ls1.get();
    launch_advect_levelset(c->st, d, g->origin, g->h, fu, dt, dphi, out);
    launch_copy(c->st, d.n, out, dphi);  // Advection::Solve replaces the field with the advected one
    CK(cudaGetLastError());
    if (!dev) CK(cudaMemcpyAsync(phi, dphi, 8 * (size_t)d.n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return SF_OK;
}

sf_status advect_velocity_impl(Ctx *c, const sf_grid *g, double *const vel[3], double dt, bool dev) {
    sf_status s = post_common(c, g, vel);
    if (s != SF_OK) return s;
    if (!std::isfinite(dt)) return fail(c, SF_BAD_ARG, "bad time step");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    long long h2d = 0;
    double *dvel[3];
    if ((s = stage_vel(c, g, vel, dev, dvel, h2d)) != SF_OK) return s;
    // the flow is the old velocity: trace and interpolate from copies, write the new values in place
    Faces fold{};
    for (int a = 0; a < 3; a++) {
        const long long nf = face_count(g, a);
        CK(c->old[a].ensure(8 * (size_t)nf));
        launch_copy(c->st, nf, dvel[a], (double *)c->old[a].get());
        fold.p[a] = (const double *)c->old[a].get();
    }
    launch_advect_velocity(c->st, d, g->origin, g->h, fold, dt, dvel);
    CK(cudaGetLastError());
    return unstage_vel(c, g, vel, dev, dvel);
}

sf_status reinitialize_impl(Ctx *c, const sf_grid *g, double *phi, int max_steps, bool dev) {
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !phi || max_steps < 0) return fail(c, SF_BAD_ARG, "bad grid, level set or step count");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    long long h2d = 0;
    sf_status s;
    double *dphi;
    if ((s = stage_cells_inout(c, g, phi, dev, &dphi, h2d)) != SF_OK) return s;
    CK(c->ls1.ensure(8 * (size_t)d.n));
    CK(c->ls2.ensure(8 * (size_t)d.n));
    launch_reinitialize(c->st, d, g->h, dphi, (double *)c->ls1.get(), (double *)c->ls2.get(), max_steps);
    CK(cudaGetLastError());
    if (!dev) CK(cudaMemcpyAsync(phi, dphi, 8 * (size_t)d.n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return SF_OK;
}

sf_status enforce_impl(Ctx *c, const sf_grid *g, double *const vel[3], const double *const frac[3],
                       const double *const normal[3], const double *const us[3], bool dev) {
    sf_status s = post_common(c, g, vel);
    if (s != SF_OK) return s;
    if (!frac || !normal) return fail(c, SF_BAD_ARG, "null fraction or normal arrays");
    for (int a = 0; a < 3; a++)
        if (!frac[a] || !normal[a] || (us && !us[a]))
            return fail(c, SF_BAD_ARG, "fraction, normal and solid-velocity arrays come in threes");
    CK(cudaSetDevice(c->device));
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    long long h2d = 0;
    double *dvel[3];
    Faces ff{}, fn{}, fus{}, fold{};
    if ((s = stage_vel(c, g, vel, dev, dvel, h2d)) != SF_OK) return s;
    for (int a = 0; a < 3; a++) {
        const long long nf = face_count(g, a);
        if ((s = stage_in(c, c->frac[a], frac[a], nf, dev, &ff.p[a], h2d)) != SF_OK) return s;
        if ((s = stage_in(c, c->normal[a], normal[a], nf, dev, &fn.p[a], h2d)) != SF_OK) return s;
        if ((s = stage_in(c, c->us[a], us ? us[a] : nullptr, nf, dev, &fus.p[a], h2d)) != SF_OK) return s;
        // Collider::Enforce interpolates the velocity as it was before the call
        CK(c->old[a].ensure(8 * (size_t)nf));
        launch_copy(c->st, nf, dvel[a], (double *)c->old[a].get());
        fold.p[a] = (const double *)c->old[a].get();
    }
    launch_enforce(c->st, d, g->origin, g->h, fold, fus, fn, ff, dvel);
    CK(cudaGetLastError());
    return unstage_vel(c, g, vel, dev, dvel);
}

}  // namespace

struct NetHandle {
    Ctx *ctx;  // nullptr once the context is destroyed
    std::unique_ptr<UNet> net;
};

// ------------------------------------------------------------------------------------------------ C ABI
extern "C" {

int sf_abi_version(void) { return SFGPU_ABI_VERSION; }

const char *sf_status_string(int s) {
    switch (s) {
        case SF_OK: return "ok";
        case SF_NOT_CONVERGED: return "not converged";
        case SF_BAD_ARG: return "bad argument";
        case SF_CUDA_ERROR: return "CUDA error";
        case SF_NO_DEVICE: return "no sm_103 CUDA device";
        case SF_OUT_OF_MEMORY: return "out of device memory";
        case SF_STALLED_FALLBACK: return "learned solve stalled; plain MGPCG finished it";
        case SF_NOT_READY: return "no previous projection on this context";
        case SF_TOO_LARGE: return "grid exceeds the allocation-free scratch (ceil(ny/8)*ceil(nz/32) > 8192)";
        default: return "unknown status";
    }
}

void sf_default_opts(sf_solve_opts *o, int which) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->precision = SF_PREC_FP64;
    o->tol = which == 1 ? 1e-6 : 1e-8;
    o->max_iters = 200;
    o->pre_smooth = 2;
    o->post_smooth = 2;
    // the potential's pure-Neumann coarsest level needs many sweeps; the pressure's, with ghost-fluid (Dirichlet)
    // terms, is well conditioned: 8 pairs take the same iterations at 256^3 and save 0.1 ms per mixed solve
    o->coarse_sweeps = which == 1 ? 48 : 8;
    o->max_levels = 0;
    o->coarse_dim = 8;
    o->warm_start = 1;
    o->use_graph = 1;
    o->check_every = 1;
    o->report_ref_residual = 1;
    o->inner_tol = 1e-3;
    o->smoother = 3;  // mixed form: FP16 smoothing copy, colour-split finest level; FP64: two colour passes
}

sf_status sf_create(int device, void *stream, void **out) {
    if (!out) return SF_BAD_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0 || device < 0 || device >= n) return SF_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return SF_NO_DEVICE;
    if (prop.major != 10 || prop.minor != 3) return SF_NO_DEVICE;  // built for sm_103a only
    auto *c = new Ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete c;
        return SF_NO_DEVICE;
    }
    if (stream) {
        c->st = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            return SF_CUDA_ERROR;
        }
        c->own_stream = true;
    }
    for (auto &e : c->ev) cudaEventCreate(&e);
    if (cudaStreamCreateWithFlags(&c->cst, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_field, cudaEventDisableTiming) != cudaSuccess) {
        sf_destroy(c);
        return SF_CUDA_ERROR;
    }
    *out = c;
    return SF_OK;
}

void sf_destroy(void *p) {
    Ctx *c = C(p);
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->cst) cudaStreamSynchronize(c->cst);
    // networks created on this context lose their device state; their handles stay valid for sf_unet_destroy
    for (void *p : c->nets) {
        auto *h = reinterpret_cast<NetHandle *>(p);
        h->net.reset();
        h->ctx = nullptr;
    }
    c->nets.clear();
    c->net = nullptr;
    c->pres.reset();
    c->mag.reset();
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->ev_in) cudaEventDestroy(c->ev_in);
    if (c->ev_field) cudaEventDestroy(c->ev_field);
    if (c->cst) cudaStreamDestroy(c->cst);
    if (c->own_stream) cudaStreamDestroy(c->st);
    delete c;
}

const char *sf_last_error(void *p) { return p ? C(p)->err.c_str() : "null context"; }

long long sf_device_bytes(void *p) {
    Ctx *c = C(p);
    if (!c) return 0;
    long long b = 0;
    if (c->pres) b += (long long)c->pres->device_bytes();
    if (c->mag) b += (long long)c->mag->device_bytes();
    DevBuf *bs[] = {&c->phi, &c->frac[0], &c->frac[1], &c->frac[2], &c->vel[0], &c->vel[1], &c->vel[2],
                    &c->us[0], &c->us[1], &c->us[2], &c->jump[0], &c->jump[1], &c->jump[2], &c->hext[0],
                    &c->hext[1], &c->hext[2], &c->H[0], &c->H[1], &c->H[2], &c->cells};
    for (DevBuf *x : bs) b += (long long)x->bytes();
    return b;
}

sf_status sf_pressure_project(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                              const double *const frac[3], const double *const solid_vel[3],
                              const double *const jump[3], double vol_error, double *p_out, const sf_solve_opts *opts,
                              sf_solve_stats *stats) {
    return pressure_impl(C(ctx), g, vel, phi, frac, solid_vel, jump, vol_error, p_out, opts, stats, false, false);
}
sf_status sf_pressure_project_dev(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                  const double *const frac[3], const double *const solid_vel[3],
                                  const double *const jump[3], double vol_error, double *p_out,
                                  const sf_solve_opts *opts, sf_solve_stats *stats) {
    return pressure_impl(C(ctx), g, vel, phi, frac, solid_vel, jump, vol_error, p_out, opts, stats, true, false);
}
sf_status sf_pressure_reproject(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                const double *const frac[3], const double *const solid_vel[3],
                                const double *const jump[3], double vol_error, double *p_out,
                                const sf_solve_opts *opts, sf_solve_stats *stats) {
    return pressure_impl(C(ctx), g, vel, phi, frac, solid_vel, jump, vol_error, p_out, opts, stats, false, true);
}
sf_status sf_pressure_reproject_dev(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                    const double *const frac[3], const double *const solid_vel[3],
                                    const double *const jump[3], double vol_error, double *p_out,
                                    const sf_solve_opts *opts, sf_solve_stats *stats) {
    return pressure_impl(C(ctx), g, vel, phi, frac, solid_vel, jump, vol_error, p_out, opts, stats, true, true);
}
sf_status sf_magnetic_solve(void *ctx, const sf_grid *g, const double *phi, double chi, double band_width,
                            const double *const hext[3], double *psi_out, double *const H_out[3],
                            const sf_solve_opts *opts, sf_solve_stats *stats) {
    return magnetic_impl(C(ctx), g, phi, chi, band_width, hext, psi_out, H_out, opts, stats, false);
}
sf_status sf_magnetic_solve_dev(void *ctx, const sf_grid *g, const double *phi, double chi, double band_width,
                                const double *const hext[3], double *psi_out, double *const H_out[3],
                                const sf_solve_opts *opts, sf_solve_stats *stats) {
    return magnetic_impl(C(ctx), g, phi, chi, band_width, hext, psi_out, H_out, opts, stats, true);
}
sf_status sf_extrapolate_velocity(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                  const double *const frac[3], double clear_val, int max_steps) {
    return extrapolate_impl(C(ctx), g, vel, phi, frac, clear_val, max_steps, false);
}
sf_status sf_extrapolate_velocity_dev(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                      const double *const frac[3], double clear_val, int max_steps) {
    return extrapolate_impl(C(ctx), g, vel, phi, frac, clear_val, max_steps, true);
}
sf_status sf_collider_enforce(void *ctx, const sf_grid *g, double *const vel[3], const double *const frac[3],
                              const double *const normal[3], const double *const solid_vel[3]) {
    return enforce_impl(C(ctx), g, vel, frac, normal, solid_vel, false);
}
sf_status sf_collider_enforce_dev(void *ctx, const sf_grid *g, double *const vel[3], const double *const frac[3],
                                  const double *const normal[3], const double *const solid_vel[3]) {
    return enforce_impl(C(ctx), g, vel, frac, normal, solid_vel, true);
}

sf_status sf_magnetic_vertex_pressures(void *ctx, const sf_grid *g, double chi, const double *const H[3],
                                      const double *positions, const double *normals, long long nverts,
                                      double *pressures) {
    return vertex_pressures_impl(C(ctx), g, chi, H, positions, normals, nverts, pressures, false);
}
sf_status sf_magnetic_vertex_pressures_dev(void *ctx, const sf_grid *g, double chi, const double *const H[3],
                                          const double *positions, const double *normals, long long nverts,
                                          double *pressures) {
    return vertex_pressures_impl(C(ctx), g, chi, H, positions, normals, nverts, pressures, true);
}
sf_status sf_pressure_jump(void *ctx, const sf_grid *g, const int32_t *const edge_mark[3], const double *curvature,
                           const double *mag_pressure, long long nverts, double st_coeff, double density, double dt,
                           double *const jump[3]) {
    return pressure_jump_impl(C(ctx), g, edge_mark, curvature, mag_pressure, nverts, st_coeff, density, dt, jump,
                              false);
}
sf_status sf_pressure_jump_dev(void *ctx, const sf_grid *g, const int32_t *const edge_mark[3],
                               const double *curvature, const double *mag_pressure, long long nverts,
                               double st_coeff, double density, double dt, double *const jump[3]) {
    return pressure_jump_impl(C(ctx), g, edge_mark, curvature, mag_pressure, nverts, st_coeff, density, dt, jump,
                              true);
}

sf_status sf_advect_levelset(void *ctx, const sf_grid *g, double *phi, const double *const vel[3], double dt) {
    return advect_levelset_impl(C(ctx), g, phi, vel, dt, false);
}
sf_status sf_advect_levelset_dev(void *ctx, const sf_grid *g, double *phi, const double *const vel[3], double dt) {
    return advect_levelset_impl(C(ctx), g, phi, vel, dt, true);
}
sf_status sf_advect_velocity(void *ctx, const sf_grid *g, double *const vel[3], double dt) {
    return advect_velocity_impl(C(ctx), g, vel, dt, false);
}
sf_status sf_advect_velocity_dev(void *ctx, const sf_grid *g, double *const vel[3], double dt) {
    return advect_velocity_impl(C(ctx), g, vel, dt, true);
}
sf_status sf_reinitialize(void *ctx, const sf_grid *g, double *phi, int max_steps) {
    return reinitialize_impl(C(ctx), g, phi, max_steps, false);
}
sf_status sf_reinitialize_dev(void *ctx, const sf_grid *g, double *phi, int max_steps) {
    return reinitialize_impl(C(ctx), g, phi, max_steps, true);
}

sf_status sf_magnetic_residual_noalloc(void *stream, const sf_grid *g, const double *phi, double chi,
                                       double band_width, const double *const hext[3], const double *psi,
                                       double *result) {
    static_assert(SF_NOALLOC_MAX_BLOCKS == 8192, "scratch size of sf_ops.cu");
    if (!grid_ok(g) || !phi || !hext || !psi || !result || !std::isfinite(chi) || !(band_width > 0) ||
        !std::isfinite(band_width))
        return SF_BAD_ARG;
    for (int a = 0; a < 3; a++)
        if (!hext[a]) return SF_BAD_ARG;
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    if (!noalloc_fits(d)) return SF_TOO_LARGE;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return SF_NO_DEVICE;
    const void *ptrs[6] = {phi, psi, result, hext[0], hext[1], hext[2]};
    for (const void *p : ptrs) {  // device (or managed) memory of the current device only
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
            cudaGetLastError();
            return SF_BAD_ARG;
        }
        if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) ||
            (at.type == cudaMemoryTypeDevice && at.device != dev))
            return SF_BAD_ARG;
    }
    Faces fh{{hext[0], hext[1], hext[2]}};
    const cudaError_t e = launch_magnetic_residual_noalloc((cudaStream_t)stream, d, phi, chi, band_width, fh, g->h,
                                                           psi, result);
    return e == cudaSuccess ? SF_OK : SF_CUDA_ERROR;
}

sf_status sf_magnetic_reset(void *ctx) {
    Ctx *c = C(ctx);
    if (!c) return SF_BAD_ARG;
    c->mag_has_x = false;
    return SF_OK;
}

sf_status sf_selftest_bounded_wait(void *ctx, double limit_ms, int *timed_out, double *waited_ms) {
    Ctx *c = C(ctx);
    if (!c) return SF_BAD_ARG;
    if (!(limit_ms > 0) || limit_ms > 10000 || !timed_out) return fail(c, SF_BAD_ARG, "limit_ms in (0, 10000]");
    CK(cudaSetDevice(c->device));
    CK(c->cells.ensure(16));
    auto *d = (unsigned long long *)c->cells.get();
    CK(selftest_bounded_wait(c->st, (unsigned long long)(limit_ms * 1e6), d));
    unsigned long long h[2] = {0, 0};
    CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    *timed_out = (int)h[0];
    if (waited_ms) *waited_ms = (double)h[1] * 1e-6;
    return SF_OK;
}

// ----- resident inputs ---------------------------------------------------------------------------------------
sf_status sf_collider_upload(void *ctx, const sf_grid *g, const double *const frac[3], const double *const solid_vel[3]) {
    Ctx *c = C(ctx);
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !frac) return fail(c, SF_BAD_ARG, "bad grid or fraction pointer");
    for (int a = 0; a < 3; a++)
        if (!frac[a] || (solid_vel && !solid_vel[a])) return fail(c, SF_BAD_ARG, "null fraction or velocity array");
    CK(cudaSetDevice(c->device));
    c->rcol = false;
    for (int a = 0; a < 3; a++) {
        const size_t bytes = 8 * (size_t)face_count(g, a);
        CK(c->rfrac[a].ensure(bytes));
        CK(cudaMemcpyAsync(c->rfrac[a].get(), frac[a], bytes, cudaMemcpyDefault, c->st));
        if (solid_vel) {
            CK(c->rus[a].ensure(bytes));
            CK(cudaMemcpyAsync(c->rus[a].get(), solid_vel[a], bytes, cudaMemcpyDefault, c->st));
        }
    }
    CK(cudaStreamSynchronize(c->st));
    c->rcol = true;
    c->rcol_us = solid_vel != nullptr;
    c->rcol_dims = make_dims(g->nx, g->ny, g->nz);
    return SF_OK;
}

sf_status sf_levelset_upload(void *ctx, const sf_grid *g, const double *phi) {
    Ctx *c = C(ctx);
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !phi) return fail(c, SF_BAD_ARG, "bad grid or level-set pointer");
    CK(cudaSetDevice(c->device));
    c->rls = false;
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    CK(c->rphi.ensure(8 * (size_t)d.n));
    CK(cudaMemcpyAsync(c->rphi.get(), phi, 8 * (size_t)d.n, cudaMemcpyDefault, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->rls = true;
    c->rls_dims = d;
    return SF_OK;
}

sf_status sf_applied_field_prefetch(void *ctx, const sf_grid *g, const double *const hext[3]) {
    Ctx *c = C(ctx);
    if (!c) return SF_BAD_ARG;
    if (!grid_ok(g) || !hext) return fail(c, SF_BAD_ARG, "bad grid or applied-field pointer");
    for (int a = 0; a < 3; a++)
        if (!hext[a]) return fail(c, SF_BAD_ARG, "null applied-field array");
    CK(cudaSetDevice(c->device));
    // a copy started earlier may still be running into the buffers
    CK(cudaStreamSynchronize(c->cst));
    c->field_pending = c->field_ready = c->field_fresh = false;
    c->field_bytes = 0;
    for (int a = 0; a < 3; a++) {
        const size_t bytes = 8 * (size_t)face_count(g, a);
        CK(c->pfield[a].ensure(bytes));
        c->field_src[a] = hext[a];
        c->field_n[a] = face_count(g, a);
        c->field_bytes += (long long)bytes;
    }
    c->field_dims = make_dims(g->nx, g->ny, g->nz);
    c->field_pending = true;
    return SF_OK;
}

// ----- learned form ------------------------------------------------------------------------------------------
sf_status sf_unet_create(void *ctx, void **out) {
    Ctx *c = C(ctx);
    if (!c || !out) return SF_BAD_ARG;
    CK(cudaSetDevice(c->device));
    auto *h = new NetHandle{c, std::make_unique<UNet>(c->st)};
    if (!h->net->last_error.empty()) {
        std::string m = h->net->last_error;
        delete h;
        return fail(c, SF_OUT_OF_MEMORY, m);
    }
    c->nets.push_back(h);
    *out = h;
    return SF_OK;
}
void sf_unet_destroy(void *net) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (!h) return;
    if (Ctx *c = h->ctx) {
        if (c->net == h->net.get()) c->net = nullptr;
        c->nets.erase(std::remove(c->nets.begin(), c->nets.end(), net), c->nets.end());
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->st);
    }
    delete h;
}
long long sf_unet_num_params(void *net) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    return (h && h->ctx) ? h->net->num_params() : 0;
}
sf_status sf_unet_set_params(void *net, const float *host, long long n) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (!h || !h->ctx || !host || n != h->net->num_params()) return SF_BAD_ARG;
    Ctx *c = h->ctx;
    CK(h->net->set_params(host));
    return SF_OK;
}
sf_status sf_unet_get_params(void *net, float *host, long long n) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (!h || !h->ctx || !host || n != h->net->num_params()) return SF_BAD_ARG;
    Ctx *c = h->ctx;
    CK(h->net->get_params(host));
    return SF_OK;
}
sf_status sf_unet_forward_dev(void *net, const sf_grid *g, const void *features, float *out) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (!h || !h->ctx || !grid_ok(g) || !features || !out) return SF_BAD_ARG;
    Ctx *c = h->ctx;
    CK(h->net->forward(make_dims(g->nx, g->ny, g->nz), (const __nv_bfloat16 *)features, out, false));
    if (h->net->check_device_errors() != cudaSuccess) return fail(c, SF_CUDA_ERROR, h->net->last_error);
    return SF_OK;
}
sf_status sf_unet_set_mode(void *net, int mode) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (!h || !h->ctx || mode < 0 || mode > 2) return SF_BAD_ARG;
    h->net->set_mode(mode);
    return SF_OK;
}
long long sf_unet_tc_launches(void *net) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    return (h && h->ctx) ? h->net->tc_launches() : 0;
}
sf_status sf_unet_backward_dev(void *net, const sf_grid *g, const void *features, const float *dout, float *grads) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (!h || !h->ctx || !grid_ok(g) || !features || !dout) return SF_BAD_ARG;
    Ctx *c = h->ctx;
    const Dims d = make_dims(g->nx, g->ny, g->nz);
    CK(h->net->forward(d, (const __nv_bfloat16 *)features, nullptr));
    CK(h->net->backward(d, dout));
    if (h->net->check_device_errors() != cudaSuccess) return fail(c, SF_CUDA_ERROR, h->net->last_error);
    if (grads) CK(h->net->get_grads(grads));
    CK(cudaStreamSynchronize(c->st));
    return SF_OK;
}
sf_status sf_unet_train_step_dev(void *net, const sf_grid *g, const void *features, const float *target, float lr,
                                 double *loss) {
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (!h || !h->ctx || !grid_ok(g) || !features || !target || !(lr > 0)) return SF_BAD_ARG;
    Ctx *c = h->ctx;
    double l = 0;
    CK(h->net->train_step(make_dims(g->nx, g->ny, g->nz), (const __nv_bfloat16 *)features, target, lr, l));
    if (loss) *loss = l;
    return SF_OK;
}
sf_status sf_set_network(void *ctx, void *net) {
    Ctx *c = C(ctx);
    if (!c) return SF_BAD_ARG;
    auto *h = reinterpret_cast<NetHandle *>(net);
    if (h && h->ctx != c) return fail(c, SF_BAD_ARG, "network belongs to another (or a destroyed) context");
    c->net = h ? h->net.get() : nullptr;
    return SF_OK;
}
sf_status sf_system_operator(void *ctx, int which, double *diag, double *const lower[3], double *rhs) {
    Ctx *c = C(ctx);
    if (!c || (which != 0 && which != 1)) return SF_BAD_ARG;
    MGSolver *S = which == 0 ? c->pres.get() : c->mag.get();
    if (!S || (which == 0 && !c->pres_ready) || (which == 1 && !c->mag_has_x))
        return fail(c, SF_NOT_READY, "no assembled system of that kind on this context");
    CK(cudaSetDevice(c->device));
    const Dims d = S->dims();
    const size_t bytes = 8 * (size_t)d.n;
    Coef<double> &cf = S->fine();
    if (diag) CK(cudaMemcpyAsync(diag, cf.D, bytes, cudaMemcpyDeviceToHost, c->st));
    if (lower) {
        double *src[3] = {cf.ax, cf.ay, cf.az};
        for (int a = 0; a < 3; a++)
            if (lower[a]) CK(cudaMemcpyAsync(lower[a], src[a], bytes, cudaMemcpyDeviceToHost, c->st));
    }
    if (rhs) CK(cudaMemcpyAsync(rhs, S->b(), bytes, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return SF_OK;
}

sf_status sf_system_features_dev(void *ctx, int which, void *features, float *solution) {
    Ctx *c = C(ctx);
    if (!c || (which != 0 && which != 1)) return SF_BAD_ARG;
    MGSolver *S = which == 0 ? c->pres.get() : c->mag.get();
    if (!S || (which == 0 && !c->pres_ready) || (which == 1 && !c->mag_has_x))
        return fail(c, SF_NOT_READY, "no assembled system of that kind on this context");
    if (!c->net) return fail(c, SF_NOT_READY, "features need a network (sf_set_network)");
    const Dims d = S->dims();
    if (features) CK(c->net->features(d, S->fine(), S->b(), (__nv_bfloat16 *)features));
    if (solution) launch_to_f32(c->st, d.n, S->x(), solution);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    return SF_OK;
}

}  // extern "C"
