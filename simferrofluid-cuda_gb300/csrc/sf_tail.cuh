// sf_tail.cuh -- the coarse end of the mixed form's V-cycle as one thread-block cluster.  Included by sf_mg.cu.
//
// From the first level of at most kTailMaxCells cells down to the coarsest, every step of the V-cycle -- the
// pre-smoothing half sweeps and residual restrictions, the coarsest solve, the prolongations and post-smoothing
// half sweeps -- runs in one launch of NC CTAs (8, or 16 where the device runs clusters of 16) forming a cluster.
// Each CTA holds a contiguous range of x-planes of every level but the coarsest in its shared memory: the
// vectors x and b, and the operator per cell in FP32 (the three lower-face couplings, D and 1 / D, formed once
// per solve by k_tail_op).  Next to its planes it keeps halo copies of the x-planes on either side (and the
// x-couplings of the plane above); a CTA that updates a cell of its first or last plane also stores the value
// into the neighbouring CTA's halo (distributed shared memory).  The sweeps then read only the CTA's own shared
// memory; a restriction or prolongation reads a plane held by another CTA where the two levels' plane ranges do
// not line up, and the coarsest level (at most kCoarseMax cells) is held by CTA 0 and solved there.  Every step
// ends with a cluster barrier (the hardware barrier.cluster: no spin loop), whose release / acquire order makes
// the stores into other CTAs visible.  As separate kernels the same steps are about twenty latency-bound launches
// per V-cycle.
//
// Each cell's arithmetic is that of k_rbgs / k_rbgs4, k_resid_restrict, k_prolong and k_coarse_smem, in the same
// order, so the fused tail returns the same values.  Rows marked inactive there are skipped; here they are
// computed, which gives the value those kernels leave (0: D = 0 makes the update (b + s) * 0, with b and s zero or
// of either sign).

namespace cg = cooperative_groups;

constexpr int kTailThreads = 1024, kTailMaxLevels = 6;
constexpr long long kTailMaxCells = 65536;
constexpr int kTailMaxNz = 1024;       // a row's cells fit one pass of the block
constexpr int kTailOps = 5;            // operator floats per cell: ax, ay, az, D, 1 / D
constexpr int kTailSmem = 220 * 1024;  // dynamic shared memory per CTA at most

// The operator of a tail level per cell, from its FP16 copy with the arithmetic of the separate kernels:
// op[0..n) ax, [n..2n) ay, [2n..3n) az (exact conversions), [3n..4n) D = unscaled couplings summed -x, +x, -y, +y,
// -z, +z plus the unscaled excess, [4n..5n) 1 / D (0 where D = 0).
__global__ void __launch_bounds__(256) k_tail_op(Dims d, Coef<__half> cf, float *__restrict__ op) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= d.nz || j >= d.ny) return;
    const long long c = cid(d, i, j, k), n = d.n, plane = (long long)d.ny * d.nz;
    const float axl = __half2float(cf.ax[c]), ayl = __half2float(cf.ay[c]), azl = __half2float(cf.az[c]);
    float sa = 0.f;
    if (i > 0) sa += axl;
    if (i < d.nx - 1) sa += __half2float(cf.ax[c + plane]);
    if (j > 0) sa += ayl;
    if (j < d.ny - 1) sa += __half2float(cf.ay[c + d.nz]);
    if (k > 0) sa += azl;
    if (k < d.nz - 1) sa += __half2float(cf.az[c + 1]);
    sa *= cf.unscale;
    float e = __half2float(cf.dex[c]);
    e *= cf.unscale;
    const float D = sa + e;
    op[c] = axl;
    op[n + c] = ayl;
    op[2 * n + c] = azl;
    op[3 * n + c] = D;
    op[4 * n + c] = D > 0.f ? 1.f / D : 0.f;
}

struct TailLevel {
    Dims d;
    const float *op;  // k_tail_op's operator (every level but the coarsest)
    Coef<__half> cf;  // the FP16 operator (the coarsest level's solve)
    float unscale;
    int pmax;  // x-planes of the largest share (the coarsest: nx, all in CTA 0)
    int off;   // byte offset of the level's slot in shared memory
    int pre, post;
};
struct TailParams {
    int nlev;  // tail levels; the last is the coarsest (at most kCoarseMax cells)
    TailLevel lv[kTailMaxLevels];
    const float *b0;  // right-hand side of the first tail level (global)
    float *x0;        // its correction (global, written)
    int pairs;        // coarsest level: symmetric sweep pairs
};

// x-planes of CTA r: [tail_p0(r), tail_p0(r + 1)); the CTA holding plane i.  The coarsest level: all in CTA 0.
template <int NC>
__host__ __device__ __forceinline__ int tail_p0(int nx, int r) {
    return (r * nx) / NC;
}
template <int NC>
__host__ __device__ __forceinline__ int tail_owner(int nx, int i) {
    return (NC * (i + 1) - 1) / nx;
}

// a level's slot in one CTA's shared memory: S = pmax planes of cells, P = one plane
struct TailArr {
    float *x, *b, *ax, *ay, *az, *D, *inv;  // S each
    float *xlo, *xhi, *axhi;                // P each: halo planes p0 - 1 (x) and p1 (x, ax)
};
__device__ __forceinline__ TailArr tail_arr(unsigned char *s, int off, int S, int P) {
    float *f = (float *)(s + off);
    return TailArr{f,         f + S,     f + 2 * S,         f + 3 * S, f + 4 * S,
                   f + 5 * S, f + 6 * S, f + 7 * S, f + 7 * S + P, f + 7 * S + 2 * P};
}
__host__ __device__ __forceinline__ long long tail_slot_bytes(long long S, long long P) {
    return ((7 * S + 3 * P) * 4 + 15) / 16 * 16;
}

// one tail level as seen from one CTA
struct TailLv {
    const TailLevel *L;
    Dims d;
    bool coarsest;
    int p0, p1;  // this CTA's planes
    int plane;   // ny * nz
    int slot;
    TailArr a;         // own slot
    float *plo, *phi;  // the xhi halo of the CTA holding plane p0 - 1, the xlo halo of the one holding plane p1
};

template <int NC>
__device__ __forceinline__ TailLv tail_lv(cg::cluster_group &cl, const TailParams &P, int l, int rank,
                                          unsigned char *smem) {
    const TailLevel &L = P.lv[l];
    TailLv v;
    v.L = &L;
    v.d = L.d;
    v.coarsest = l == P.nlev - 1;
    v.p0 = v.coarsest ? (rank == 0 ? 0 : L.d.nx) : tail_p0<NC>(L.d.nx, rank);
    v.p1 = v.coarsest ? L.d.nx : tail_p0<NC>(L.d.nx, rank + 1);
    v.plane = L.d.ny * L.d.nz;
    v.slot = L.pmax * v.plane;
    v.a = tail_arr(smem, L.off, v.slot, v.plane);
    v.plo = v.phi = nullptr;
    if (!v.coarsest && v.p1 > v.p0) {
        if (v.p0 > 0) {
            unsigned char *s = (unsigned char *)cl.map_shared_rank((void *)smem, tail_owner<NC>(L.d.nx, v.p0 - 1));
            v.plo = tail_arr(s, L.off, v.slot, v.plane).xhi;
        }
        if (v.p1 < L.d.nx) {
            unsigned char *s = (unsigned char *)cl.map_shared_rank((void *)smem, tail_owner<NC>(L.d.nx, v.p1));
            v.phi = tail_arr(s, L.off, v.slot, v.plane).xlo;
        }
    }
    return v;
}

// the slot arrays of plane i (x, b, operator) in the CTA holding it, offset to the plane
template <int NC>
__device__ __forceinline__ TailArr tail_pl(cg::cluster_group &cl, const TailLv &v, unsigned char *smem, int i) {
    TailArr t = v.a;
    int lp = i - v.p0;
    if (i < v.p0 || i >= v.p1) {
        const int r = v.coarsest ? 0 : tail_owner<NC>(v.d.nx, i);
        lp = v.coarsest ? i : i - tail_p0<NC>(v.d.nx, r);
        t = tail_arr((unsigned char *)cl.map_shared_rank((void *)smem, r), v.L->off, v.slot, v.plane);
    }
    const int o = lp * v.plane;
    return TailArr{t.x + o, t.b + o, t.ax + o, t.ay + o, t.az + o, t.D + o, t.inv + o, nullptr, nullptr, nullptr};
}

// x (and ax) of neighbour plane i: this CTA's own planes, its halos, or the CTA holding it
template <int NC>
__device__ __forceinline__ void tail_nb(cg::cluster_group &cl, const TailLv &v, unsigned char *smem, int i,
                                        const float *&x, const float *&ax) {
    if (i >= v.p0 && i < v.p1) {
        x = v.a.x + (i - v.p0) * v.plane;
        ax = v.a.ax + (i - v.p0) * v.plane;
    } else if (i == v.p0 - 1) {
        x = v.a.xlo;
        ax = nullptr;  // not read: the -x term takes the cell's own coupling
    } else if (i == v.p1) {
        x = v.a.xhi;
        ax = v.a.axhi;
    } else {
        const TailArr t = tail_pl<NC>(cl, v, smem, i);
        x = t.x;
        ax = t.ax;
    }
}

// Row walk over npl planes of ny rows, S slots per row (S <= blockDim): thread t takes slot t % S of rows t / S,
// t / S + per, ... (per = blockDim / S).  f(local plane, j, slot).
template <class F>
__device__ __forceinline__ void tail_rows(int npl, int ny, int S, F &&f) {
    const int per = blockDim.x / S;
    const int t = threadIdx.x, r0 = t / S;
    if (r0 >= per) return;
    const int m = t - r0 * S;
    const int dpl = per / ny, dj = per - dpl * ny;
    int pl = r0 / ny, j = r0 - pl * ny;
    while (pl < npl) {
        f(pl, j, m);
        pl += dpl;
        j += dj;
        if (j >= ny) {
            j -= ny;
            pl++;
        }
    }
}

// this CTA's planes of a level (and its halos): operator copied from k_tail_op's arrays, x = 0, b = b0 (the first
// level) or 0.  One pass: a thread issues the loads of all fields of its cells before storing any (16-byte vectors
// where the plane and the level are multiples of 4 cells).  The coarsest level: x and b only (its solve reads the
// FP16 operator).
__device__ void tail_load(const TailLv &v, const float *b0) {
    const int cnt = (v.p1 - v.p0) * v.plane;
    if (cnt == 0) return;
    const long long n = v.d.n, c0 = (long long)v.p0 * v.plane;
    const TailArr &a = v.a;
    if (v.coarsest) {
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            a.x[q] = 0.f;
            a.b[q] = b0 ? b0[c0 + q] : 0.f;
        }
        return;
    }
    const float *op = v.L->op + c0;
    if (v.plane % 4 == 0 && n % 4 == 0) {
        const int n4 = cnt >> 2;
        const long long s4 = n >> 2;  // one field, in float4
        const float4 *o4 = reinterpret_cast<const float4 *>(op), *b4 = reinterpret_cast<const float4 *>(b0 + c0);
        for (int q = threadIdx.x; q < n4; q += blockDim.x) {
            const float4 vb = b0 ? __ldg(b4 + q) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 v0 = __ldg(o4 + q), v1 = __ldg(o4 + s4 + q), v2 = __ldg(o4 + 2 * s4 + q),
                         v3 = __ldg(o4 + 3 * s4 + q), v4 = __ldg(o4 + 4 * s4 + q);
            reinterpret_cast<float4 *>(a.x)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
            reinterpret_cast<float4 *>(a.b)[q] = vb;
            reinterpret_cast<float4 *>(a.ax)[q] = v0;
            reinterpret_cast<float4 *>(a.ay)[q] = v1;
            reinterpret_cast<float4 *>(a.az)[q] = v2;
            reinterpret_cast<float4 *>(a.D)[q] = v3;
            reinterpret_cast<float4 *>(a.inv)[q] = v4;
        }
    } else {
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const float vb = b0 ? __ldg(b0 + c0 + q) : 0.f;
            const float v0 = __ldg(op + q), v1 = __ldg(op + n + q), v2 = __ldg(op + 2 * n + q),
                        v3 = __ldg(op + 3 * n + q), v4 = __ldg(op + 4 * n + q);
            a.x[q] = 0.f;
            a.b[q] = vb;
            a.ax[q] = v0;
            a.ay[q] = v1;
            a.az[q] = v2;
            a.D[q] = v3;
            a.inv[q] = v4;
        }
    }
    const float *axh = v.p1 < v.d.nx ? v.L->op + (long long)v.p1 * v.plane : nullptr;
    for (int q = threadIdx.x; q < v.plane; q += blockDim.x) {
        a.xlo[q] = 0.f;
        a.xhi[q] = 0.f;
        a.axhi[q] = axh ? __ldg(axh + q) : 0.f;
    }
}

// x of cell q of local plane pl (index jk in the plane) = xn, and into the neighbouring CTA's halo when the plane
// is this CTA's first or last
__device__ __forceinline__ void tail_put(const TailLv &v, int pl, int npl, int q, int jk, float xn) {
    v.a.x[q] = xn;
    if (pl == 0 && v.plo) v.plo[jk] = xn;
    if (pl == npl - 1 && v.phi) v.phi[jk] = xn;
}

// one half sweep of colour col (k_rbgs4 / k_rbgs arithmetic); ZERO: the sweep starts from x = 0 (x not read)
template <bool ZERO>
__device__ void tail_half_sweep(cg::cluster_group &cl, const TailLv &v, int col) {
    const TailArr &a = v.a;
    const int nz = v.d.nz, ny = v.d.ny, plane = v.plane, npl = v.p1 - v.p0;
    const float u = v.L->unscale;
    tail_rows(npl, ny, (nz + 1) >> 1, [&](int pl, int j, int m) {
        const int i = v.p0 + pl;
        const int k = 2 * m + ((i + j + col) & 1);
        if (k >= nz) return;
        const int jk = j * nz + k, q = pl * plane + jk;
        float s = 0.f;
        if (!ZERO) {
            if (i > 0) {
                if (pl > 0)
                    s += a.ax[q] * a.x[q - plane];
                else
                    s += a.ax[q] * a.xlo[jk];
            }
            if (i < v.d.nx - 1) {
                if (pl < npl - 1)
                    s += a.ax[q + plane] * a.x[q + plane];
                else
                    s += a.axhi[jk] * a.xhi[jk];
            }
            if (j > 0) s += a.ay[q] * a.x[q - nz];
            if (j < ny - 1) s += a.ay[q + nz] * a.x[q + nz];
            if (k > 0) s += a.az[q] * a.x[q - 1];
            if (k < nz - 1) s += a.az[q + 1] * a.x[q + 1];
            s *= u;
        }
        tail_put(v, pl, npl, q, jk, (a.b[q] + s) * a.inv[q]);
    });
    cl.sync();
}

// nu sweeps: pre red-black (the first from x = 0), post black-red
__device__ void tail_smooth(cg::cluster_group &cl, const TailLv &v, int nu, bool pre) {
    for (int s = 0; s < nu; s++) {
        if (pre) {
            if (s == 0)
                tail_half_sweep<true>(cl, v, 0);
            else
                tail_half_sweep<false>(cl, v, 0);
            tail_half_sweep<false>(cl, v, 1);
        } else {
            tail_half_sweep<false>(cl, v, 1);
            tail_half_sweep<false>(cl, v, 0);
        }
    }
}

// b of the coarse level = the fine level's residual summed over each coarse cell's (up to) 8 children in the
// order of k_resid_restrict.  Coarse plane I is formed by the CTA holding fine plane 2 I and stored in the CTA
// holding plane I.
template <int NC>
__device__ void tail_restrict(cg::cluster_group &cl, const TailLv &f, const TailLv &c, unsigned char *smem) {
    const int nz = f.d.nz, ny = f.d.ny, nx = f.d.nx;
    const float u = f.L->unscale;
    const int I0 = (f.p0 + 1) >> 1, I1 = (f.p1 + 1) >> 1;  // 2 I in [p0, p1)
    tail_rows(I1 - I0, c.d.ny, c.d.nz, [&](int pl, int J, int K) {
        const int I = I0 + pl;
        float acc = 0.f;
#pragma unroll
        for (int di = 0; di < 2; di++) {
            const int i = 2 * I + di;
            if (i < nx) {
                const TailArr pc = tail_pl<NC>(cl, f, smem, i);
                const float *xm = nullptr, *xp = nullptr, *axm, *axp = nullptr;
                if (i > 0) tail_nb<NC>(cl, f, smem, i - 1, xm, axm);
                if (i < nx - 1) tail_nb<NC>(cl, f, smem, i + 1, xp, axp);
#pragma unroll
                for (int dj = 0; dj < 2; dj++) {
                    const int j = 2 * J + dj;
#pragma unroll
                    for (int dk = 0; dk < 2; dk++) {
                        const int k = 2 * K + dk;
                        if (j < ny && k < nz) {
                            const int jk = j * nz + k;
                            float s = 0.f;
                            if (i > 0) s += pc.ax[jk] * xm[jk];
                            if (i < nx - 1) s += axp[jk] * xp[jk];
                            if (j > 0) s += pc.ay[jk] * pc.x[jk - nz];
                            if (j < ny - 1) s += pc.ay[jk + nz] * pc.x[jk + nz];
                            if (k > 0) s += pc.az[jk] * pc.x[jk - 1];
                            if (k < nz - 1) s += pc.az[jk + 1] * pc.x[jk + 1];
                            s *= u;
                            acc += (pc.b[jk] - pc.D[jk] * pc.x[jk]) + s;
                        }
                    }
                }
            }
        }
        tail_pl<NC>(cl, c, smem, I).b[J * c.d.nz + K] = acc;
    });
    cl.sync();
}

// x of the fine level += x of the coarse level at the parent cell (k_prolong)
template <int NC>
__device__ void tail_prolong(cg::cluster_group &cl, const TailLv &f, const TailLv &c, unsigned char *smem) {
    const int npl = f.p1 - f.p0;
    tail_rows(npl, f.d.ny, f.d.nz, [&](int pl, int j, int k) {
        const TailArr pc = tail_pl<NC>(cl, c, smem, (f.p0 + pl) >> 1);
        const int jk = j * f.d.nz + k, q = pl * f.plane + jk;
        tail_put(f, pl, npl, q, jk, f.a.x[q] + pc.x[(j >> 1) * c.d.nz + (k >> 1)]);
    });
    cl.sync();
}

// The coarsest level solved on CTA 0 as k_coarse_smem does: b made consistent on a pure-Neumann level
// (coarse_consistent), x = 0, then the palindromic sequence red, (black, red) x pairs, each cell's couplings (FP16,
// global memory) pre-multiplied by the level's unscale.  x and b are the
// level's arrays in CTA 0, in natural order.
__device__ void tail_coarse(cg::cluster_group &cl, const TailLv &v, int rank, int pairs) {
    const Dims &d = v.d;
    const Coef<__half> &cf = v.L->cf;
    if (rank == 0) {
        float *xs = v.a.x;
        const int sx = d.ny * d.nz, sy = d.nz;
        const int c = threadIdx.x;
        float a[6], inv = 0.f, bc = 0.f;
        int has = 0, col = -1;
        if (c < d.n) {
            const int k = c % d.nz, j = (c / d.nz) % d.ny, i = c / (d.nz * d.ny);
            col = (i + j + k) & 1;
            has = (i > 0) | ((i < d.nx - 1) << 1) | ((j > 0) << 2) | ((j < d.ny - 1) << 3) | ((k > 0) << 4) |
                  ((k < d.nz - 1) << 5);
            float sum = 0.f;
#pragma unroll
            for (int f = 0; f < 6; f++) {
                const __half *arr = f < 2 ? cf.ax : (f < 4 ? cf.ay : cf.az);
                const int st = f < 2 ? sx : (f < 4 ? sy : 1);
                float av = 0.f;
                if (has & (1 << f)) {
                    av = __half2float(arr[(f & 1) ? c + st : c]);
                    av *= cf.unscale;
                    sum += av;
                }
                a[f] = av;
            }
            float e = __half2float(cf.dex[c]);
            e *= cf.unscale;
            const float D = sum + e;
            inv = D > 0.f ? 1.f / D : 0.f;
            bc = v.a.b[c];
            xs[c] = 0.f;
        }
        bc = coarse_consistent<float>(bc, c < d.n && inv > 0.f, c < d.n && __half2float(cf.dex[c]) != 0.f);
        __syncthreads();
        const int nh = 1 + 2 * pairs;
        for (int h = 0; h < nh; h++) {
            if (col == (h & 1)) {
                float s = 0.f;
#pragma unroll
                for (int f = 0; f < 6; f++) {
                    const int st = f < 2 ? sx : (f < 4 ? sy : 1);
                    if (has & (1 << f)) s += a[f] * xs[(f & 1) ? c + st : c - st];
                }
                xs[c] = (bc + s) * inv;
            }
            __syncthreads();
        }
    }
    cl.sync();
}

template <int NC>
__global__ void __launch_bounds__(kTailThreads, 1) k_tail(TailParams P) {
    extern __shared__ __align__(16) unsigned char tail_smem[];
    pdl_entry();
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int nl = P.nlev;
    for (int l = 0; l < nl; l++) tail_load(tail_lv<NC>(cl, P, l, rank, tail_smem), l == 0 ? P.b0 : nullptr);
    cl.sync();
    for (int l = 0; l + 1 < nl; l++) {
        const TailLv v = tail_lv<NC>(cl, P, l, rank, tail_smem);
        tail_smooth(cl, v, P.lv[l].pre, true);
        tail_restrict<NC>(cl, v, tail_lv<NC>(cl, P, l + 1, rank, tail_smem), tail_smem);
    }
    tail_coarse(cl, tail_lv<NC>(cl, P, nl - 1, rank, tail_smem), rank, P.pairs);
    for (int l = nl - 2; l >= 0; l--) {
        const TailLv v = tail_lv<NC>(cl, P, l, rank, tail_smem);
        tail_prolong<NC>(cl, v, tail_lv<NC>(cl, P, l + 1, rank, tail_smem), tail_smem);
        tail_smooth(cl, v, P.lv[l].post, false);
    }
    // the first level's correction back to global memory (own planes only: no peer is read after the last
    // cluster barrier)
    const TailLv v0 = tail_lv<NC>(cl, P, 0, rank, tail_smem);
    const long long c0 = (long long)v0.p0 * v0.plane;
    const int n0 = (v0.p1 - v0.p0) * v0.plane;
    for (int q = threadIdx.x; q < n0; q += blockDim.x) P.x0[c0 + q] = v0.a.x[q];
}

// Host side.  The tail of hierarchy dims from level lt on a cluster of nc CTAs (every level from lt: at most
// kTailMaxCells cells and nz at most kTailMaxNz; the coarsest at most kCoarseMax cells) and its shared-memory
// layout; false if it does not fit.
static bool tail_plan(const std::vector<Dims> &dims, int lt, int nc, TailParams &P, int &smem_bytes) {
    const int L = (int)dims.size();
    const int nlev = L - lt;
    if (lt < 1 || nlev < 2 || nlev > kTailMaxLevels || dims[L - 1].n > kCoarseMax) return false;
    long long off = 0;
    for (int l = 0; l < nlev; l++) {
        const Dims &d = dims[lt + l];
        if (d.n > kTailMaxCells || d.nz > kTailMaxNz) return false;
        int pmax = d.nx;
        if (l < nlev - 1) {
            pmax = 0;
            for (int r = 0; r < nc; r++) pmax = std::max(pmax, ((r + 1) * d.nx) / nc - (r * d.nx) / nc);
        }
        P.lv[l].d = d;
        P.lv[l].pmax = pmax;
        P.lv[l].off = (int)off;
        off += tail_slot_bytes((long long)pmax * d.ny * d.nz, (long long)d.ny * d.nz);
    }
    P.nlev = nlev;
    if (off > kTailSmem) return false;
    smem_bytes = (int)off;
    return true;
}

template <int NC>
static void tail_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *at, cudaStream_t st, int smem) {
    cfg = {};
    cfg.gridDim = dim3(NC);
    cfg.blockDim = dim3(kTailThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = NC;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
}

// whether one cluster of NC CTAs with smem bytes of dynamic shared memory each runs on this device.  The kernel's
// shared-memory ceiling is a property of the function, shared by every solver in the process: it is set to the
// largest layout any tail plans (kTailSmem), never to one solver's need.
template <int NC>
static bool tail_launchable(int smem) {
    if (cudaFuncSetAttribute(k_tail<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmem) != cudaSuccess ||
        (NC > 8 && cudaFuncSetAttribute(k_tail<NC>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at[1];
    tail_config<NC>(cfg, at, nullptr, smem);
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, k_tail<NC>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return nc >= 1;
}

// The launch's own status: a cluster launch the device rejects leaves the tail's levels untouched, and the caller
// runs the separate kernels instead.
static cudaError_t launch_tail(cudaStream_t st, int nc, const TailParams &P, int smem) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at[1];
    if (nc == 16) {
        tail_config<16>(cfg, at, st, smem);
        return cudaLaunchKernelEx(&cfg, k_tail<16>, P);
    }
    tail_config<8>(cfg, at, st, smem);
    return cudaLaunchKernelEx(&cfg, k_tail<8>, P);
}
