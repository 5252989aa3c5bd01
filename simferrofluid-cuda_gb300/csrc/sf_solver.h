// sf_solver.h -- host interface of the matrix-free geometric-multigrid PCG solver (sm_103a).
//
// The solver owns every device buffer of one grid size: the FP64 fine-level operator (filled by the
// assembly kernels in sf_ops.cu), the right-hand side b, the solution x, the coarse hierarchy, the Krylov
// vectors and the CUDA graphs of one iteration.  Buffers are reused across solves on the same grid, which
// keeps graph node pointers stable.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "sf_internal.cuh"

namespace sf {

struct SolverParams {
    int precision = 0;  // 0 FP64 MGPCG, 1 mixed (FP32/FP16 V-cycle + FP32 FCG inside FP64 refinement)
    double tol = 1e-8;
    int max_iters = 200;
    int pre = 2, post = 2, coarse_sweeps = 48;
    int coarse_pre = 2, coarse_post = 2;  // levels 2 and coarser
    int max_levels = 0, coarse_dim = 8;
    bool use_graph = true;
    int check_every = 1;
    double inner_tol = 1e-3;
    bool flexible = false;  // Polak-Ribiere beta (needed when the preconditioner is not a fixed SPD operator)
    bool profile = false;   // time finest-level smoother launches with events (no graphs)
    int smoother = 0;       // 0: two in-place colour kernels, 1: fused one-pass red-black sweep
    int tail = 0;  // mixed form, levels of at most 65,536 cells: 0 one cluster launch (16 CTAs, else 8), 8 / 16 that
                   // cluster size, 1 separate kernels
    bool full_sweeps = false;  // FP64 form: every row, also rows without an active cell (else they are skipped)
};

// Counts kernel launches and, when profiling, brackets finest-level smoother launches with events.
struct Tracker {
    long long launches = 0;
    bool prof = false;
    double *sc = nullptr;  // the solver's scalar slots (S_ERR receives bounded-wait timeouts)
    std::vector<cudaEvent_t> ev;
    size_t used = 0;
    double bytes = 0;
    // profile: algorithmic bytes of one split level-0 half sweep, counted over the rows it processes and by row
    // kind (-1: not set, every cell at the general rate)
    double bytes0 = -1;
    bool tail_failed = false;
    // profile, FP64 form with row skipping: cells in active rows of level 0 (-1: every cell counts)
    double active0 = -1;  // a fused-tail cluster launch was rejected (the separate kernels ran instead)
    void before(cudaStream_t st, bool fine);
    void after(cudaStream_t st, bool fine, double algo_bytes);
    // after a stream sync: summed milliseconds, launch count and algorithmic bytes of the bracketed
    // launches; resets
    void collect(double &ms, int &n, double &b);
    ~Tracker();
};

struct SolveResult {
    long long launches = 0;
    double smooth_ms = 0, smooth_bytes = 0;
    int smooth_launches = 0;
    int iters = 0, outer = 0, levels = 0;
    bool converged = false;
    bool breakdown = false;
    bool fallback = false;      // learned form: the network stalled and the plain iteration finished the solve
    double guess_relres = -1;   // learned form: relative residual after the first learned step (x0 = gamma y)
    double guess_energy = -1;   // its squared A-norm error relative to that of zero
    int learned_steps = 0;      // learned correction steps applied
    double relres = 0, bnorm = 0;
};

// Launches the bounded-wait self-test (one CTA waits on an mbarrier that nothing completes, for limit_ns; device
// out[0] = 1 when it gave up, out[1] = nanoseconds waited).
cudaError_t selftest_bounded_wait(cudaStream_t st, unsigned long long limit_ns, unsigned long long *out);

// The learned form's correction of an inner solve: y = the network's prediction of A^-1 r for an FP32 residual r
// on the fine level's cells (natural layout), rr = (r, r).
struct LearnedStep {
    virtual ~LearnedStep() = default;
    virtual cudaError_t predict(const float *r, double rr, float *y) = 0;
};

class DevBuf {
   public:
    DevBuf() = default;
    ~DevBuf();
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    void *get() const { return p_; }
    size_t bytes() const { return n_; }
    cudaError_t ensure(size_t bytes);
    void release();

   private:
    void *p_ = nullptr;
    size_t n_ = 0;
};

class MGSolver {
   public:
    explicit MGSolver(cudaStream_t s);
    ~MGSolver();

    // (Re)allocate for grid d and the solver configuration; cheap when nothing changed.
    cudaError_t configure(const Dims &d, const SolverParams &p);
    const Dims &dims() const { return lev_dims_[0]; }
    int levels() const { return (int)lev_dims_.size(); }

    // Fine-level FP64 operator and vectors (device).  The assembly kernels write ax/ay/az/dex/D/invd and b.
    Coef<double> &fine() { return c64_[0]; }
    double *b() { return b_; }
    double *x() { return x_; }

    // Build coarse levels (and the FP32/FP16 copies for the mixed form) from the fine operator.
    cudaError_t build_hierarchy();

    // Where the assembly kernels may write the split level-0 copies and row flags directly (smoother 3 in the
    // mixed form), or nullptr; the next build_hierarchy then takes them as written.
    const SplitOut *split_targets();

    // Solve A x = b.  x holds the initial guess unless x_is_zero.  exclude_cell0_norm: report the residual
    // without row 0 (the potential's pinned row).
    cudaError_t solve(bool x_is_zero, SolveResult &res);

    // ||b - A x|| / ||b|| on the fine FP64 operator; with skip0 row 0 is left out of both norms.
    cudaError_t true_relres(bool skip0, double &relres, double &bnorm);

    // Learned correction steps for the next mixed-form solves (nullptr: none).  At the start of every inner solve
    // of the iterative refinement -- the first one from r = b -- the network's prediction y of A^-1 r is taken as
    // the inner solve's first step d = gamma y, gamma = (y, r) / (y, A y) (the multiple that minimises the A-norm
    // error along y), r -= gamma A y, and the flexible CG continues from there.  A step that reduces ||r|| by less
    // than 10 % (or is not finite) marks the network as stalled: the rest of the solve runs the plain MGPCG
    // iteration and SolveResult::fallback is set.
    void set_learned(LearnedStep *ls) { learned_ = ls; }

    // Shift x so that x[0] == 0 (potential gauge).
    cudaError_t shift_to_zero_at_origin();

    size_t device_bytes() const;
    long long take_launches() {
        long long n = tk_.launches;
        tk_.launches = 0;
        return n;
    }
    std::string last_error;

   private:
    template <class T, class C0, class Cc>
    friend struct HierOps;

    cudaStream_t st_;
    SolverParams prm_;
    std::vector<Dims> lev_dims_;
    std::vector<std::unique_ptr<DevBuf>> bufs_;
    size_t bytes_ = 0;
    bool configured_ = false;
    LearnedStep *learned_ = nullptr;
    DevBuf lrn_r_, lrn_y_;                      // natural-layout residual and prediction of a learned step
    double guess_yb_ = 0, guess_yay_ = 0;       // (y, b) and (y, A y) of the first learned step
    cudaError_t learned_step(double rr, bool first, bool &stalled, SolveResult &res);
    Dims cfg_dims_{0, 0, 0, 0};
    int cfg_prec_ = -1, cfg_levels_ = -1, cfg_cdim_ = -1, cfg_smoother_ = -1;
    bool rows64_ = false;  // FP64 form with row flags on every level (rows_): inactive rows are skipped

    // FP64 hierarchy (precision 0) or fine FP64 operator only (precision 1)
    std::vector<Coef<double>> c64_;
    std::vector<double *> x64_, b64_;  // coarse-level vectors (index 0 unused)
    std::vector<double *> t64_;        // smoother scratch per level
    // mixed: level 0 FP32, levels >= 1 FP16
    Coef<float> c32_{};
    std::vector<Coef<__half>> c16_;  // index l for level l >= 1
    Coef<__half> c16s0_{};           // level 0 in FP16, read only by the level-0 smoother (smoothers 2 and 3)
    // smoother 3 in effect: level 0's FP32 vectors and both of its operator copies are stored colour by colour
    // (sf_split.cuh); the FP64 operator and vectors keep the natural layout
    bool split0_ = false, cfg_split_ = false;
    // with split0_: per level, one byte per row (i, j), 0 when every cell of the row is inactive (D = 0)
    std::vector<uint8_t *> rows_;
    int *list_[3] = {nullptr, nullptr, nullptr};  // active rows of levels 0, 1 (and 2 when level 1 is split)
    int *count_ = nullptr;               // their counts (device)
    float *crow_ = nullptr;              // level 0: the coupling of each uniform row
    float *crow1_ = nullptr;             // level 1 (split): the same
    float4 *rc_[2] = {nullptr, nullptr}; // levels 0, 1: the half sweep's row constants (k_smooth_consts_s)
    float *dinv_[2] = {nullptr, nullptr}; // levels 0, 1: the half sweep's 1 / D on general rows
    bool split1_ = false;                // level 1 stored colour by colour too
    SplitOut so_{};                      // split_targets()
    bool copies_written_ = false;        // the assembly wrote the split copies and flags
    int tail_lt_ = -1, tail_smem_ = 0;   // first level of the fused tail (-1: none), its shared memory
    int tail_nc_ = 0;                    // its cluster size
    std::vector<float *> tail_op_;       // per level of at most 65,536 cells: the tail's FP32 operator (k_tail_op)
    void plan_tail();
    Coef<__half> c16s1_{};               // its split FP16 operator copy (the natural copy feeds level 2)
    int *list_cnt_ = nullptr;            // per block of rows: general and uniform counts (list building)
    std::vector<float *> x32_, b32_, t32_;

    double *x_ = nullptr, *b_ = nullptr;
    // Krylov vectors
    double *r_ = nullptr, *z_ = nullptr, *p_ = nullptr, *q_ = nullptr;
    float *r32_ = nullptr, *d32_ = nullptr, *ri32_ = nullptr, *z32_ = nullptr, *p32_ = nullptr, *q32_ = nullptr;
    double *sc_ = nullptr;       // scalar slots
    double *sc_host_ = nullptr;  // pinned mirror
    double *part_ = nullptr;     // reduction partials
    unsigned *ticket_ = nullptr;

    cudaGraphExec_t g_iter64_ = nullptr, g_iter32_ = nullptr;
    // the inner (flexible) CG loop of each form as one graph: a conditional WHILE node whose body is one iteration
    // and k_inner_ctl (loop_ok_ false: the loop is driven from the host, one graph launch per iteration)
    cudaGraphExec_t g_loop32_ = nullptr, g_loop64_ = nullptr;
    bool loop_ok_ = true;
    cudaError_t inner_loop(bool mixed, int budget, double tol2, double rr, int &iters);
    cudaError_t build_loop(bool mixed);
    cudaError_t run_iter_prepare();
    long long graph_key_ = -1;
    long long iter_launches64_ = 0, iter_launches32_ = 0;
    Tracker tk_;

    void *alloc(size_t bytes);
    void free_all();
    void destroy_graphs();
    bool drop_tail();  // after a rejected fused-tail launch: separate kernels from now on (true if it was on)
    cudaError_t solve64(bool x_is_zero, SolveResult &res);
    cudaError_t solve_mixed(bool x_is_zero, SolveResult &res);
    void enqueue_iter64(bool copy_slots = true);
    void enqueue_iter32(bool copy_slots = true);
    cudaError_t run_iter(bool mixed);
    cudaError_t read_slots();
};

// Launch helpers
constexpr int kMaxRedBlocks = 152 * 8;
constexpr int kStencilBlocks = 152 * 8;  // persistent grid of the FP64 residual
constexpr int kApplyBlocks = 16384;      // one work item per block for the memory-bound stencil reductions
constexpr int kStencilPlanes = 4;        // x planes per work item
constexpr int kMaxRedGrid = kApplyBlocks;
dim3 tile_grid(const Dims &d, int &xpb, int max_blocks);
dim3 tile_grid3(const Dims &d, int &xpb);

}  // namespace sf
