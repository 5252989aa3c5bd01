// sf_split.cuh -- finest level of the mixed form stored colour by colour (smoother 3).  Included by sf_mg.cu.
//
// Layout.  Cell (i, j, k) has colour col = (i + j + k) & 1.  Every FP32 vector of level 0 and both level-0
// operator copies (FP32 for the Krylov operator, FP16 for the smoother) hold colour 0 in their first half and
// colour 1 in their second half; inside a half, row (i, j) holds its nz / 2 cells of that colour in k order:
//     s(col, i, j, m) = col * n/2 + (i * ny + j) * nz/2 + m,      k = 2 m + ((i + j + col) & 1).
// (nz a multiple of 8, so every row of a colour is a whole number of 16-byte vectors.)  The same-k neighbours
// in x and y of a cell sit at the same m in the other colour's half; its z neighbours sit at m - 1 and m
// (k - 1, k + 1) when k is even, at m and m + 1 when k is odd.  A coarse cell's eight children are the
// entries m = K of both colours in four rows.
//
// Why: a red-black half sweep updates one colour from the other.  In the natural layout every launch streams
// both colours of x, b and the operator (about 20 bytes per cell); here it reads the updated colour's b,
// diagonal excess and lower couplings, the other colour's x and lower couplings above, and writes the updated
// colour (about 13 bytes per cell).  The arithmetic of every cell -- which couplings, in which order -- is the
// natural kernels' own; the restriction after the pre-smoothing sums only the colour that was not updated last
// (the other colour's residual is zero up to rounding), so a V-cycle agrees with the natural one to rounding.

// Grid-stride loop over the rows (i, j) of the split layout, blockDim.y rows per block and blockDim.x threads
// along a row, without a per-element division: for each m, cell k = 2m + p is colour 0 and k = 2m + 1 - p is
// colour 1 (p the row's parity), both stored at m of their colour's half.  `nat` is the row's first natural
// index and `sp` its first index inside a colour's half.
#define SPLIT_ROWS(d)                                                                                        \
    const int nh_ = (d).nz >> 1;                                                                              \
    const long long hn_ = (d).n >> 1, nrows_ = (long long)(d).nx * (d).ny;                                     \
    for (long long row = blockIdx.x * (long long)blockDim.y + threadIdx.y; row < nrows_;                     \
         row += (long long)gridDim.x * blockDim.y) {                                                          \
        const int i_ = (int)(row / (d).ny), j_ = (int)(row - (long long)i_ * (d).ny);                        \
        const int p = (i_ + j_) & 1;                                                                          \
        const long long nat = row * (d).nz, sp = row * nh_;                                                   \
        for (int m = threadIdx.x; m < nh_; m += blockDim.x) {                                                 \
            const long long n0 = nat + 2 * m + p, n1 = nat + 2 * m + 1 - p, s0 = sp + m, s1 = hn_ + sp + m;

#define SPLIT_ROWS_END \
    }                  \
    }

static inline int split_rows_grid(const Dims &d) {
    long long g = ((long long)d.nx * d.ny + 7) / 8;
    if (g > 152 * 16) g = 152 * 16;
    return (int)(g < 1 ? 1 : g);
}

// List of a level's active rows, in two segments: the general rows (flag 1) in ascending order, then the uniform
// rows (flag 2) in ascending order; an entry is (i << 16) | j, with bit 31 set on uniform rows (nx < 2^15,
// ny < 2^16); *count = their number.  Rows of one segment cost the same,
// so the persistent kernels' round-robin split of the list gives every warp an equal share of each kind.
// Two kernels over blocks of 1024 rows: per-block counts of each kind, then each block's entries at the offsets
// the counts give (deterministic).
constexpr int kListRows = 1024;
__global__ void __launch_bounds__(kListRows) k_rows_count(long long nrows, const uint8_t *__restrict__ rows,
                                                          int *__restrict__ cnt) {
    const long long r = blockIdx.x * (long long)kListRows + threadIdx.x;
    const uint8_t f = r < nrows ? rows[r] : 0;
    const int g = __syncthreads_count(f == 1), u = __syncthreads_count(f == 2);
    if (threadIdx.x == 0) {
        cnt[2 * blockIdx.x] = g;
        cnt[2 * blockIdx.x + 1] = u;
    }
}
__global__ void __launch_bounds__(kListRows) k_rows_scatter(long long nrows, int ny, const uint8_t *__restrict__ rows,
                                                            const int *__restrict__ cnt, int *__restrict__ list,
                                                            int *__restrict__ count) {
    __shared__ int wg[32], wu[32], off[2];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (w == 0) {  // offsets of this block's general and uniform entries, and the total
        int g_before = 0, u_before = 0, g_all = 0, u_all = 0;
        for (int b = lane; b < (int)gridDim.x; b += 32) {
            const int g = cnt[2 * b], u = cnt[2 * b + 1];
            g_all += g;
            u_all += u;
            if (b < (int)blockIdx.x) {
                g_before += g;
                u_before += u;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            g_before += __shfl_xor_sync(0xffffffffu, g_before, o);
            u_before += __shfl_xor_sync(0xffffffffu, u_before, o);
            g_all += __shfl_xor_sync(0xffffffffu, g_all, o);
            u_all += __shfl_xor_sync(0xffffffffu, u_all, o);
        }
        if (lane == 0) {
            off[0] = g_before;
            off[1] = g_all + u_before;
            if (blockIdx.x == 0) *count = g_all + u_all;
        }
    }
    const long long r = blockIdx.x * (long long)kListRows + t;
    const uint8_t f = r < nrows ? rows[r] : 0;
    const unsigned bg = __ballot_sync(0xffffffffu, f == 1), bu = __ballot_sync(0xffffffffu, f == 2);
    if (lane == 0) {
        wg[w] = __popc(bg);
        wu[w] = __popc(bu);
    }
    __syncthreads();
    int pg = off[0], pu = off[1];
    for (int q = 0; q < w; q++) {
        pg += wg[q];
        pu += wu[q];
    }
    const unsigned below = (1u << lane) - 1u;
    const unsigned e = ((unsigned)(r / ny) << 16) | (unsigned)(r % ny);
    if (f == 1) list[pg + __popc(bg & below)] = (int)e;
    if (f == 2) list[pu + __popc(bu & below)] = (int)(e | 0x80000000u);
}

// Persistent loop of a grid's warps (blockDim = (32, 8)) over the items (rep, list entry, chunk): `reps` passes
// (colours) over the *count listed rows, `nch` chunks of 32 lanes per row; warp w takes items w, w + W, ...
// Every warp gets an equal share of the active rows, and the assignment depends only on the grid and the list,
// so reductions stay deterministic.  f(rep, i, j, chunk, uniform).
// 32-bit item arithmetic (a level has fewer than 2^31 rows); reps is 1 or 2.
template <class F>
__device__ __forceinline__ void for_list_items(const int *__restrict__ list, const int *__restrict__ count, int reps,
                                               int nch, F &&f) {
    const unsigned n = (unsigned)*count;
    const unsigned nit = reps * n * (unsigned)nch, stride = gridDim.x * blockDim.y;
    auto split = [&](unsigned it, unsigned &rr, unsigned &ch) {
        if (nch == 1) {
            rr = it;
            ch = 0;
        } else {
            rr = it / (unsigned)nch;
            ch = it - rr * (unsigned)nch;
        }
    };
    auto entry = [&](unsigned it) {
        if (it >= nit) return 0;
        unsigned rr, ch;
        split(it, rr, ch);
        return list[rr >= n ? rr - n : rr];
    };
    unsigned it = blockIdx.x * blockDim.y + threadIdx.y;
    int e = entry(it);
    for (; it < nit; it += stride) {
        const int e_next = entry(it + stride);  // issued before this item's loads
        unsigned rr, ch;
        split(it, rr, ch);
        f(rr >= n ? 1 : 0, (e >> 16) & 0x7fff, e & 0xffff, (int)ch, e < 0);
        e = e_next;
    }
}

// The same loop seen per lane: f(rep, i, j, q4, uniform) for the lane's vector q4 of its row.  Rows of 32 or more
// vectors are split into chunks of 32 lanes (for_list_items); rows of fewer, nq a power of two, share a warp --
// 32 / nq rows per warp, nq lanes each -- so that no lane idles on the short rows of the coarser split level.
// The assignment depends only on the grid and the list (deterministic).  reps is 1 or 2.
template <class F>
__device__ __forceinline__ void for_list_lanes(const int *__restrict__ list, const int *__restrict__ count, int reps,
                                               int nq, F &&f) {
    if (nq >= 32 || (32 % nq) != 0) {
        for_list_items(list, count, reps, (nq + 31) / 32, [&](int rep, int i, int j, int ch, bool uni) {
            const int q4 = ch * 32 + threadIdx.x;
            if (q4 < nq) f(rep, i, j, q4, uni);
        });
        return;
    }
    const unsigned n = (unsigned)*count, per = 32u / (unsigned)nq;
    const unsigned groups = (n + per - 1) / per, nit = (unsigned)reps * groups, stride = gridDim.x * blockDim.y;
    const unsigned sub = threadIdx.x / (unsigned)nq, q4 = threadIdx.x - sub * (unsigned)nq;
    for (unsigned it = blockIdx.x * blockDim.y + threadIdx.y; it < nit; it += stride) {
        const unsigned rep = it >= groups ? 1u : 0u;
        const unsigned r = (it - rep * groups) * per + sub;
        if (r >= n) continue;
        const int e = list[r];
        f((int)rep, (e >> 16) & 0x7fff, e & 0xffff, (int)q4, e < 0);
    }
}

// Grid of a persistent row kernel: the blocks that fit on the device at once (its occupancy), at most one warp
// per item.  Occupancies are looked up once per device and kernel.
static int resident_grid(const void *kernel) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_pair(dev, kernel);
    const auto f = cache.find(key);
    if (f != cache.end()) return f->second;
    int nb = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, 256, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int g = (nb > 0 ? nb : 1) * (sms > 0 ? sms : 1);
    cache[key] = g;
    return g;
}
static int row_grid(const void *kernel, long long items) {
    const long long need = (items + 7) / 8;
    const long long g = resident_grid(kernel);
    return (int)(need < 1 ? 1 : (need < g ? need : g));
}

// FP64 level 0 -> split FP32 copy (Krylov operator) and FP16 copy (smoother) in one pass, with the roundings
// of k_to32 / k_to16, and the level's row flags (a row is active when one of its cells has D > 0).  One warp
// per row: blockDim = (32, 8).
__global__ void __launch_bounds__(256) k_to_split(Dims d, Coef<double> f, Coef<float> o32, Coef<__half> o16,
                                                  uint8_t *__restrict__ rows) {
    const int nh = d.nz >> 1;
    const long long hn = d.n >> 1, nrows = (long long)d.nx * d.ny;
    for (long long row = blockIdx.x * (long long)blockDim.y + threadIdx.y; row < nrows;
         row += (long long)gridDim.x * blockDim.y) {
        const int i = (int)row / d.ny, j = (int)row - i * d.ny;
        const int p = (i + j) & 1;
        const long long nat = row * d.nz, sp = row * nh;
        bool act = false;
        for (int m = threadIdx.x; m < nh; m += blockDim.x) {
            const long long n0 = nat + 2 * m + p, n1 = nat + 2 * m + 1 - p, s0 = sp + m, s1 = hn + sp + m;
            const double *src[4] = {f.ax, f.ay, f.az, f.dex};
            float *d32[4] = {o32.ax, o32.ay, o32.az, o32.dex};
            __half *d16[4] = {o16.ax, o16.ay, o16.az, o16.dex};
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const float v0 = f64_to_f32(src[a][n0]), v1 = f64_to_f32(src[a][n1]);
                d32[a][s0] = v0;
                d32[a][s1] = v1;
                d16[a][s0] = __float2half_rn(v0);
                d16[a][s1] = __float2half_rn(v1);
            }
            act |= (f.D[n0] > 0.0) | (f.D[n1] > 0.0);
        }
        act = __any_sync(0xffffffffu, act);
        if (threadIdx.x == 0) rows[row] = act ? 1 : 0;
    }
}

// Row flags of a coarse level from the next finer one: coarse row (I, J) is active when one of the fine rows
// (2I + di, 2J + dj) is (a coarse cell whose children are all inactive has an all-zero operator row).
__global__ void k_rows_coarsen(Dims df, const uint8_t *__restrict__ rf, Dims dc, uint8_t *__restrict__ rc) {
    const long long nrows = (long long)dc.nx * dc.ny;
    for (long long row = blockIdx.x * (long long)blockDim.x + threadIdx.x; row < nrows;
         row += (long long)gridDim.x * blockDim.x) {
        const int I = (int)row / dc.ny, J = (int)row - I * dc.ny;
        uint8_t a = 0;
        for (int di = 0; di < 2; di++)
            for (int dj = 0; dj < 2; dj++) {
                const int i = 2 * I + di, j = 2 * J + dj;
                if (i < df.nx && j < df.ny) a |= rf[(long long)i * df.ny + j];
            }
        rc[row] = a ? 1 : 0;
    }
}

// Uniform rows of the split level 0.  An active row (flag 1) becomes uniform (flag 2) when every cell of it has a
// zero diagonal excess and every in-grid coupling of its cells equals one FP32 value c > 0: the lower x, y, z
// faces of its cells, their upper z faces (the next cell's lower face, in the row) and their upper x and y
// faces (the lower faces of rows (i + 1, j) and (i, j + 1)).  Equal FP32 values have equal FP16 roundings, so
// both copies of the operator are c on the row.  crow[row] = c (as stored, FP16 values converted exactly).  One
// warp per row.  C is the type of the copy classified (FP32 on level 0, FP16 on a split level 1).
template <class C>
__global__ void __launch_bounds__(256) k_rows_uniform(Dims d, Coef<C> o, uint8_t *__restrict__ rows,
                                                      float *__restrict__ crow) {
    const int nh = d.nz >> 1;
    const long long hn = d.n >> 1, nrows = (long long)d.nx * d.ny;
    for (long long row = blockIdx.x * (long long)blockDim.y + threadIdx.y; row < nrows;
         row += (long long)gridDim.x * blockDim.y) {
        if (!rows[row]) continue;
        const int i = (int)row / d.ny, j = (int)row - i * d.ny;
        const int p = (i + j) & 1;
        const float c = nh > 0 ? ldv(o.az, (long long)(p ^ 1) * hn + row * nh) : 0.f;  // lower z face, k = 1
        bool ok = c > 0.f;
        for (int m = threadIdx.x; m < nh; m += blockDim.x)
#pragma unroll
            for (int col = 0; col < 2; col++) {
                const long long sidx = (long long)col * hn + row * nh + m, oth = (long long)(col ^ 1) * hn;
                const int k = 2 * m + ((p + col) & 1);
                ok &= ldv(o.dex, sidx) == 0.f;
                if (k > 0) ok &= ldv(o.az, sidx) == c;
                if (i > 0) ok &= ldv(o.ax, sidx) == c;
                if (j > 0) ok &= ldv(o.ay, sidx) == c;
                if (i < d.nx - 1) ok &= ldv(o.ax, oth + (row + d.ny) * nh + m) == c;
                if (j < d.ny - 1) ok &= ldv(o.ay, oth + (row + 1) * nh + m) == c;
            }
        ok = __all_sync(0xffffffffu, ok);
        if (threadIdx.x == 0) {
            crow[row] = c;
            if (ok) rows[row] = 2;
        }
    }
}

// Natural FP32 vector -> split copy.
__global__ void __launch_bounds__(256) k_vec_to_split(Dims d, const float *__restrict__ y, float *__restrict__ o) {
    SPLIT_ROWS(d)
    o[s0] = y[n0];
    o[s1] = y[n1];
    SPLIT_ROWS_END
}

// Split copy -> natural FP32 vector.
__global__ void __launch_bounds__(256) k_split_to_vec(Dims d, const float *__restrict__ s, float *__restrict__ y) {
    SPLIT_ROWS(d)
    y[n0] = s[s0];
    y[n1] = s[s1];
    SPLIT_ROWS_END
}

// First refinement step from x = 0 on the split level: r = (float) b in the split layout; slots rr = bb = (b, b).
__global__ void __launch_bounds__(256) k_cast_rhs_s(Dims d, const double *__restrict__ b, float *__restrict__ r,
                                                    int rr_slot, int bb_slot, double *sc, double *part,
                                                    unsigned *ticket) {
    double v[1] = {0};
    SPLIT_ROWS(d)
    const double b0 = b[n0], b1 = b[n1];
    r[s0] = f64_to_f32(b0);
    r[s1] = f64_to_f32(b1);
    v[0] += b0 * b0;
    v[0] += b1 * b1;
    SPLIT_ROWS_END
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) {
        sc[rr_slot] = tot[0];
        sc[bb_slot] = tot[0];
    }
}

// x64 += d32 with d32 in the split layout (zero in inactive rows, which are skipped).
__global__ void __launch_bounds__(256) k_ir_update_s(Dims d, double *__restrict__ x, const float *__restrict__ dlt,
                                                     const int *__restrict__ list, const int *__restrict__ count) {
    const int nh = d.nz >> 1;
    const long long hn = d.n >> 1;
    for_list_items(list, count, 1, (nh + 31) / 32, [&](int, int i, int j, int ch, bool) {
        const int m = ch * 32 + threadIdx.x;
        if (m >= nh) return;
        const long long row = (long long)i * d.ny + j;
        const int p = (i + j) & 1;
        const long long nat = row * d.nz + 2 * m, sp = row * nh + m;
        x[nat + p] += (double)dlt[sp];
        x[nat + 1 - p] += (double)dlt[hn + sp];
    });
}

// Krylov vector kernels of the split level: items are the rows of one colour (2 n_rows of them, float4 along a
// row), inactive rows skipped: (r, z) and (z, q) with the beta of k_dot_rz; p = z + beta p; x += alpha p,
// r -= alpha q, (r, r).
template <class F>
__device__ __forceinline__ void for_vec_rows(const Dims &d, const int *list, const int *count, F &&f) {
    const int nq = d.nz >> 3;  // float4 per row of a colour
    const long long nrows = (long long)d.nx * d.ny;
    for_list_items(list, count, 2, (nq + 31) / 32, [&](int col, int i, int j, int ch, bool) {
        const int t = ch * 32 + threadIdx.x;
        if (t < nq) f((col * nrows + (long long)i * d.ny + j) * nq + t);
    });
}

__global__ void __launch_bounds__(256) k_dot_rz_s(Dims d, const float *__restrict__ r, const float *__restrict__ z,
                                                  const float *__restrict__ q, const int *__restrict__ list,
                                                  const int *__restrict__ count, int flexible, double *sc,
                                                  double *part, unsigned *ticket) {
    pdl_entry();
    float a0 = 0.f, a1 = 0.f;
    for_vec_rows(d, list, count, [&](long long v4) {
        const float4 rv = reinterpret_cast<const float4 *>(r)[v4], zv = reinterpret_cast<const float4 *>(z)[v4],
                     qv = reinterpret_cast<const float4 *>(q)[v4];
        a0 += rv.x * zv.x;
        a0 += rv.y * zv.y;
        a0 += rv.z * zv.z;
        a0 += rv.w * zv.w;
        a1 += zv.x * qv.x;
        a1 += zv.y * qv.y;
        a1 += zv.z * qv.z;
        a1 += zv.w * qv.w;
    });
    float v[2] = {a0, a1};
    double tot[2];
    if (grid_reduce<2>(v, part, ticket, tot)) {
        const double rho = sc[S_RHO];
        double beta = flexible ? (-sc[S_ALPHA] * tot[1] / rho) : (tot[0] / rho);
        if (!isfinite(beta)) beta = 0;
        sc[S_RHONEW] = tot[0];
        sc[S_ZQ] = tot[1];
        sc[S_BETA] = beta;
        sc[S_RHO] = tot[0];
    }
}

__global__ void __launch_bounds__(256) k_xpby_s(Dims d, const float *__restrict__ z, float *__restrict__ p,
                                                const int *__restrict__ list, const int *__restrict__ count,
                                                const double *sc) {
    pdl_entry();
    const float beta = (float)sc[S_BETA];
    for_vec_rows(d, list, count, [&](long long v4) {
        const float4 zv = reinterpret_cast<const float4 *>(z)[v4];
        float4 pv = reinterpret_cast<float4 *>(p)[v4];
        pv.x = zv.x + beta * pv.x;
        pv.y = zv.y + beta * pv.y;
        pv.z = zv.z + beta * pv.z;
        pv.w = zv.w + beta * pv.w;
        reinterpret_cast<float4 *>(p)[v4] = pv;
    });
}

__global__ void __launch_bounds__(256) k_update_s(Dims d, float *__restrict__ x, float *__restrict__ r,
                                                  const float *__restrict__ p, const float *__restrict__ q,
                                                  const int *__restrict__ list, const int *__restrict__ count,
                                                  double *sc, double *part, unsigned *ticket) {
    pdl_entry();
    const float alpha = (float)sc[S_ALPHA];
    float acc = 0.f;
    for_vec_rows(d, list, count, [&](long long v4) {
        float4 xv = reinterpret_cast<float4 *>(x)[v4], rv = reinterpret_cast<float4 *>(r)[v4];
        const float4 pv = reinterpret_cast<const float4 *>(p)[v4], qv = reinterpret_cast<const float4 *>(q)[v4];
        xv.x += alpha * pv.x;
        xv.y += alpha * pv.y;
        xv.z += alpha * pv.z;
        xv.w += alpha * pv.w;
        rv.x = rv.x - alpha * qv.x;
        rv.y = rv.y - alpha * qv.y;
        rv.z = rv.z - alpha * qv.z;
        rv.w = rv.w - alpha * qv.w;
        reinterpret_cast<float4 *>(x)[v4] = xv;
        reinterpret_cast<float4 *>(r)[v4] = rv;
        acc += rv.x * rv.x;
        acc += rv.y * rv.y;
        acc += rv.z * rv.z;
        acc += rv.w * rv.w;
    });
    float v[1] = {acc};
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) sc[S_RR] = tot[0];
}

// Four consecutive operator entries held as loaded: FP32 as four floats, FP16 packed two to a register and
// converted where used (same values as ld4), which keeps the split kernels' register count at four blocks of
// 256 threads per SM.  Index with compile-time t.
template <class C>
struct Cv4;
template <>
struct Cv4<float> {
    float v[4];
    __device__ __forceinline__ void load(const float *p) { ld4(p, v); }
    __device__ __forceinline__ void zero() { v[0] = v[1] = v[2] = v[3] = 0.f; }
    __device__ __forceinline__ float operator[](int t) const { return v[t]; }
};
template <>
struct Cv4<__half> {
    uint2 r;
    __device__ __forceinline__ void load(const __half *p) { r = *reinterpret_cast<const uint2 *>(p); }
    __device__ __forceinline__ void zero() { r = make_uint2(0u, 0u); }
    __device__ __forceinline__ float operator[](int t) const {
        const unsigned w = t < 2 ? r.x : r.y;
        const __half2 h = *reinterpret_cast<const __half2 *>(&w);
        return (t & 1) ? __high2float(h) : __low2float(h);
    }
};


// Uniform rows (every in-grid coupling c, no excess; k_rows_uniform): the operator is c times the graph
// Laplacian of the in-grid faces, so no coefficient is loaded.  A cell with n in-grid faces has D = c n (exact:
// the general path's sum of n copies of c is exact too), neighbour sum s = sum x_nb in the general path's face
// order, and c s in place of sum c x_nb.  c_of returns the value the given copy holds (FP16 rounding, unscaled).
template <class C>
__device__ __forceinline__ float c_of(const Coef<C> &cf, float c32) {
    if (sizeof(C) == 2) return __half2float(__float2half_rn(c32)) * cf.unscale;
    return c32;
}

// Loads of a uniform-row update: the other colour's x around the colour-`col` cells m0 .. m0 + 3 of row (i, j).
struct Nb4 {
    float xm[4] = {0, 0, 0, 0}, xp[4] = {0, 0, 0, 0}, ym[4] = {0, 0, 0, 0}, yp[4] = {0, 0, 0, 0}, zo[4] = {0, 0, 0, 0};
    float zx = 0.f;  // the other colour's entry just outside the vector (m0 - 1 for even k, m0 + 4 for odd)
};
__device__ __forceinline__ void load_nb4(const Dims &d, const float *__restrict__ x, long long oth, int i, int j,
                                         int m0, int qz, Nb4 &v) {
    const int nh = d.nz >> 1;
    const long long sx = (long long)d.ny * nh, sy = nh;
    if (i > 0) ld4(x + oth - sx, v.xm);
    if (i < d.nx - 1) ld4(x + oth + sx, v.xp);
    if (j > 0) ld4(x + oth - sy, v.ym);
    if (j < d.ny - 1) ld4(x + oth + sy, v.yp);
    ld4(x + oth, v.zo);
    if (qz == 0) {
        if (m0 > 0) v.zx = x[oth - 1];
    } else if (m0 + 4 < nh) {
        v.zx = x[oth + 4];
    }
}
// sum of the in-grid neighbours of cell t (face order of the general path) and their count
template <int QZ, int t>
__device__ __forceinline__ void nb_sum(const Dims &d, const Nb4 &v, int i, int j, int m0, bool use_x, float &s,
                                       float &n) {
    const int k = 2 * (m0 + t) + QZ;
    s = 0.f;
    n = 0.f;
    if (i > 0) {
        if (use_x) s += v.xm[t];
        n += 1.f;
    }
    if (i < d.nx - 1) {
        if (use_x) s += v.xp[t];
        n += 1.f;
    }
    if (j > 0) {
        if (use_x) s += v.ym[t];
        n += 1.f;
    }
    if (j < d.ny - 1) {
        if (use_x) s += v.yp[t];
        n += 1.f;
    }
    if (k > 0) {
        if (use_x) s += QZ == 0 ? (t == 0 ? v.zx : v.zo[t == 0 ? 0 : t - 1]) : v.zo[t];
        n += 1.f;
    }
    if (k < d.nz - 1) {
        if (use_x) s += QZ == 0 ? v.zo[t] : (t == 3 ? v.zx : v.zo[t == 3 ? 3 : t + 1]);
        n += 1.f;
    }
}
template <class Fn>
__device__ __forceinline__ void for_cells4(int qz, Fn &&fn) {
    auto body = [&](auto qc) {
        constexpr int QZ = decltype(qc)::value;
        fn(qc, std::integral_constant<int, 0>{});
        fn(qc, std::integral_constant<int, 1>{});
        fn(qc, std::integral_constant<int, 2>{});
        fn(qc, std::integral_constant<int, 3>{});
        (void)QZ;
    };
    if (qz == 0)
        body(std::integral_constant<int, 0>{});
    else
        body(std::integral_constant<int, 1>{});
}

// 1 / (c n) for the row's interior cells (n = the in-grid x and y faces + 2) and for its two end cells (k = 0,
// k = nz - 1: one z face fewer); c n is exact, as in the general path.
__device__ __forceinline__ void row_inv(const Dims &d, float c, int i, int j, float &inv_in, float &inv_end) {
    const float nxy = (float)((i > 0) + (i < d.nx - 1) + (j > 0) + (j < d.ny - 1));
    const float di = c * (nxy + 2.f), de = c * (nxy + 1.f);
    inv_in = di > 0.f ? __frcp_rn(di) : 0.f;  // IEEE round-to-nearest reciprocal: the value of 1.f / di
    inv_end = de > 0.f ? __frcp_rn(de) : 0.f;
}

// Constants of the smoother's copy of a split level, formed once per build so that a half sweep loads them instead
// of forming them per cell on every sweep:
//   rc[row] = {c, 1 / (c n) of interior cells, 1 / (c n) of the row's two end cells, 0} on a uniform row, c being
//             the value the copy holds (c_of);
//   dinv[cell] = 1 / D on every cell of a general row (split layout), D the in-grid couplings of the copy summed in
//             the face order -x, +x, -y, +y, -z, +z, times the copy's unscale, plus the excess times the unscale;
//             0 where D = 0.
// Every FP32 operation is rounded explicitly (no contraction), and the reciprocals are IEEE round-to-nearest.
template <class C>
__device__ __forceinline__ float unscaled(const Coef<C> &cf, float v) {
    return sizeof(C) == 2 ? __fmul_rn(v, cf.unscale) : v;
}

template <class C>
__global__ void __launch_bounds__(256) k_smooth_consts_s(Dims d, Coef<C> cf, const uint8_t *__restrict__ rows,
                                                         const float *__restrict__ crow, float4 *__restrict__ rc,
                                                         float *__restrict__ dinv) {
    const int nh = d.nz >> 1;
    const long long hn = d.n >> 1, nrows = (long long)d.nx * d.ny;
    const long long sx = (long long)d.ny * nh, sy = nh;
    for (long long row = blockIdx.x * (long long)blockDim.y + threadIdx.y; row < nrows;
         row += (long long)gridDim.x * blockDim.y) {
        const uint8_t kind = rows[row];
        if (!kind) continue;
        const int i = (int)row / d.ny, j = (int)row - i * d.ny;
        if (kind == 2) {
            if (threadIdx.x == 0) {
                const float c = c_of(cf, crow[row]);
                float inv_in, inv_end;
                row_inv(d, c, i, j, inv_in, inv_end);
                rc[row] = make_float4(c, inv_in, inv_end, 0.f);
            }
            continue;
        }
        const bool xl = i > 0, xu = i < d.nx - 1, yl = j > 0, yu = j < d.ny - 1;
        for (int m = threadIdx.x; m < nh; m += blockDim.x)
#pragma unroll
            for (int col = 0; col < 2; col++) {
                const long long own = (long long)col * hn + row * nh + m, oth = (long long)(col ^ 1) * hn + row * nh + m;
                const int k = 2 * m + ((i + j + col) & 1);
                float sa = 0.f;
                if (xl) sa = __fadd_rn(sa, ldv(cf.ax, own));
                if (xu) sa = __fadd_rn(sa, ldv(cf.ax, oth + sx));
                if (yl) sa = __fadd_rn(sa, ldv(cf.ay, own));
                if (yu) sa = __fadd_rn(sa, ldv(cf.ay, oth + sy));
                // below: k even -> the other colour's m - 1 is the lower neighbour, whose coupling is this cell's az
                if (k > 0) sa = __fadd_rn(sa, ldv(cf.az, own));
                // above: the upper neighbour's lower z coupling (m of the other colour for k even, m + 1 for k odd)
                if (k < d.nz - 1) sa = __fadd_rn(sa, ldv(cf.az, (k & 1) ? oth + 1 : oth));
                const float D = __fadd_rn(unscaled(cf, sa), unscaled(cf, ldv(cf.dex, own)));
                dinv[own] = D > 0.f ? __frcp_rn(D) : 0.f;
            }
    }
}

template <bool ZERO>
__device__ __forceinline__ void rbgs4s_uniform(const Dims &d, float4 rcv, float *__restrict__ x,
                                               const float *__restrict__ b, int col, int i, int j, int m0) {
    const int nh = d.nz >> 1;
    const unsigned row = ((unsigned)i * (unsigned)d.ny + (unsigned)j) * (unsigned)nh + (unsigned)m0;
    const unsigned hn = (unsigned)(d.n >> 1);
    const unsigned own = (col ? hn : 0u) + row, oth = (col ? 0u : hn) + row;
    const int qz = (i + j + col) & 1;
    const float c = rcv.x, inv_in = rcv.y, inv_end = rcv.z;
    float bv[4], out[4];
    ld4(b + own, bv);
    Nb4 v;
    if (!ZERO) load_nb4(d, x, oth, i, j, m0, qz, v);
    for_cells4(qz, [&](auto qc, auto tc) {
        constexpr int QZ = decltype(qc)::value, t = decltype(tc)::value;
        float s, n;
        nb_sum<QZ, t>(d, v, i, j, m0, !ZERO, s, n);
        const int k = 2 * (m0 + t) + QZ;
        const float inv = (k == 0 || k == d.nz - 1) ? inv_end : inv_in;
        out[t] = (bv[t] + c * s) * inv;
    });
    *reinterpret_cast<float4 *>(x + own) = make_float4(out[0], out[1], out[2], out[3]);
}

__device__ __forceinline__ void resid4_uniform(const Dims &d, float c, const float *__restrict__ x,
                                               const float *__restrict__ b, int col, int i, int j, int m0,
                                               float (&r)[4]) {
    const int nh = d.nz >> 1;
    const long long row = ((long long)i * d.ny + j) * nh + m0;
    const long long own = (long long)col * (d.n >> 1) + row, oth = (long long)(col ^ 1) * (d.n >> 1) + row;
    const int qz = (i + j + col) & 1;
    float xc[4], bv[4];
    ld4(x + own, xc);
    ld4(b + own, bv);
    Nb4 v;
    load_nb4(d, x, oth, i, j, m0, qz, v);
    for_cells4(qz, [&](auto qc, auto tc) {
        constexpr int QZ = decltype(qc)::value, t = decltype(tc)::value;
        float s, n;
        nb_sum<QZ, t>(d, v, i, j, m0, true, s, n);
        r[t] = (bv[t] - (c * n) * xc[t]) + c * s;
    });
}

__device__ __forceinline__ void apply4s_uniform(const Dims &d, float c, const float *__restrict__ p,
                                                float *__restrict__ q, int col, int i, int j, int m0, float &acc) {
    const int nh = d.nz >> 1;
    const long long row = ((long long)i * d.ny + j) * nh + m0;
    const long long own = (long long)col * (d.n >> 1) + row, oth = (long long)(col ^ 1) * (d.n >> 1) + row;
    const int qz = (i + j + col) & 1;
    float pc[4], out[4];
    ld4(p + own, pc);
    Nb4 v;
    load_nb4(d, p, oth, i, j, m0, qz, v);
    for_cells4(qz, [&](auto qc, auto tc) {
        constexpr int QZ = decltype(qc)::value, t = decltype(tc)::value;
        float s, n;
        nb_sum<QZ, t>(d, v, i, j, m0, true, s, n);
        out[t] = (c * n) * pc[t] - c * s;
        acc += pc[t] * out[t];
    });
    *reinterpret_cast<float4 *>(q + own) = make_float4(out[0], out[1], out[2], out[3]);
}

// Both colours of a uniform row at once: cells m0 .. m0 + 3 of colour 0 and of colour 1 of row (i, j).  The
// neighbour rows of one colour are the other colour's, so the two colours' loads serve each other (the own
// values are the other colour's z row) and p is read from DRAM once per launch instead of once per colour.  Each
// cell's q is apply4s_uniform's.
__device__ __forceinline__ void apply4s_uniform2(const Dims &d, float c, const float *__restrict__ p,
                                                 float *__restrict__ q, int i, int j, int m0, float &acc) {
    const int nh = d.nz >> 1;
    const long long row = ((long long)i * d.ny + j) * nh + m0, hn = d.n >> 1;
    const int qz0 = (i + j) & 1;
    Nb4 v0, v1;  // v0: the colour-1 rows around colour 0 (v0.zo = colour 1's own row); v1 the converse
    load_nb4(d, p, hn + row, i, j, m0, qz0, v0);
    load_nb4(d, p, row, i, j, m0, qz0 ^ 1, v1);
    float out0[4], out1[4];
    for_cells4(qz0, [&](auto qc, auto tc) {
        constexpr int QZ = decltype(qc)::value, t = decltype(tc)::value;
        float s, n;
        nb_sum<QZ, t>(d, v0, i, j, m0, true, s, n);
        out0[t] = (c * n) * v1.zo[t] - c * s;
        acc += v1.zo[t] * out0[t];
    });
    for_cells4(qz0 ^ 1, [&](auto qc, auto tc) {
        constexpr int QZ = decltype(qc)::value, t = decltype(tc)::value;
        float s, n;
        nb_sum<QZ, t>(d, v1, i, j, m0, true, s, n);
        out1[t] = (c * n) * v0.zo[t] - c * s;
        acc += v0.zo[t] * out1[t];
    });
    *reinterpret_cast<float4 *>(q + row) = make_float4(out0[0], out0[1], out0[2], out0[3]);
    *reinterpret_cast<float4 *>(q + hn + row) = make_float4(out1[0], out1[1], out1[2], out1[3]);
}

// Red-black half sweep of colour `col` in the split layout (the counterpart of k_rbgs4), on the four
// colour-`col` cells m0 .. m0 + 3 of row (i, j); QZ = (i + j + col) & 1 is uniform over a warp (one row) and
// selects where the z neighbours sit.
template <class C, bool ZERO>
__device__ __forceinline__ void rbgs4s_cells(const Dims &d, const Coef<C> &cf, float *__restrict__ x,
                                             const float *__restrict__ b, const float *__restrict__ dinv, int col,
                                             int i, int j, int m0) {
    const int nh = d.nz >> 1;
    const unsigned row = ((unsigned)i * (unsigned)d.ny + (unsigned)j) * (unsigned)nh + (unsigned)m0;
    const unsigned hn = (unsigned)(d.n >> 1);
    const unsigned own = (col ? hn : 0u) + row, oth = (col ? 0u : hn) + row;
    const unsigned sx = (unsigned)d.ny * (unsigned)nh, sy = (unsigned)nh;
    const bool xl = i > 0, xu = i < d.nx - 1, yl = j > 0, yu = j < d.ny - 1;
    float xm[4] = {0, 0, 0, 0}, xp[4] = {0, 0, 0, 0}, ym[4] = {0, 0, 0, 0}, yp[4] = {0, 0, 0, 0}, zo[4] = {0, 0, 0, 0};
    float bv[4], iv[4];
    Cv4<C> axl, axu, ayl, ayu, azl, azo;
    axu.zero();
    ayu.zero();
    axl.load(cf.ax + own);
    if (xu) axu.load(cf.ax + oth + sx);
    ayl.load(cf.ay + own);
    if (yu) ayu.load(cf.ay + oth + sy);
    azl.load(cf.az + own);
    azo.load(cf.az + oth);
    ld4(dinv + own, iv);
    ld4(b + own, bv);
    if (!ZERO) {
        if (xl) ld4(x + oth - sx, xm);
        if (xu) ld4(x + oth + sx, xp);
        if (yl) ld4(x + oth - sy, ym);
        if (yu) ld4(x + oth + sy, yp);
        ld4(x + oth, zo);
    }
    float out[4];
    auto sweep = [&](auto qc) {
        constexpr int QZ = decltype(qc)::value;
        // the other colour's entry just outside the vector: m0 - 1 (below, k even) or m0 + 4 (above, k odd)
        float zx = 0.f, azx = 0.f;
        if (QZ == 0) {
            if (!ZERO && m0 > 0) zx = x[oth - 1];
        } else if (m0 + 4 < nh) {
            if (!ZERO) zx = x[oth + 4];
            azx = ldv(cf.az, oth + 4);
        }
        auto upd = [&](auto tc) {
            constexpr int t = decltype(tc)::value;
            const int k = 2 * (m0 + t) + QZ;
            float s = 0.f;
            if (!ZERO) {
                if (xl) s += axl[t] * xm[t];
                if (xu) s += axu[t] * xp[t];
                if (yl) s += ayl[t] * ym[t];
                if (yu) s += ayu[t] * yp[t];
                // below: m - 1 (k even) or m (k odd) of the other colour
                if (k > 0) s += azl[t] * (QZ == 0 ? (t == 0 ? zx : zo[t == 0 ? 0 : t - 1]) : zo[t]);
                // above: m (k even) or m + 1 (k odd), whose lower z coupling is this face's
                if (k < d.nz - 1)
                    s += (QZ == 0 ? azo[t] : (t == 3 ? azx : azo[t == 3 ? 3 : t + 1])) *
                         (QZ == 0 ? zo[t] : (t == 3 ? zx : zo[t == 3 ? 3 : t + 1]));
                if (sizeof(C) == 2) s *= cf.unscale;
            }
            out[t] = (bv[t] + s) * iv[t];  // iv: 1 / D of the copy (k_smooth_consts_s)
        };
        upd(std::integral_constant<int, 0>{});
        upd(std::integral_constant<int, 1>{});
        upd(std::integral_constant<int, 2>{});
        upd(std::integral_constant<int, 3>{});
    };
    if (((i + j + col) & 1) == 0)
        sweep(std::integral_constant<int, 0>{});
    else
        sweep(std::integral_constant<int, 1>{});
    *reinterpret_cast<float4 *>(x + own) = make_float4(out[0], out[1], out[2], out[3]);
}

// Persistent half sweep: warps over the active rows' chunks of 32 vectors.  rc, dinv: k_smooth_consts_s.
template <class C, bool ZERO>
__global__ void __launch_bounds__(256, 4) k_rbgs4s(Dims d, Coef<C> cf, float *__restrict__ x,
                                                  const float *__restrict__ b, int col, const int *__restrict__ list,
                                                  const int *__restrict__ count, const float4 *__restrict__ rc,
                                                  const float *__restrict__ dinv) {
    pdl_entry();
    const int nq = d.nz >> 3;
    for_list_lanes(list, count, 1, nq, [&](int, int i, int j, int q4, bool uni) {
        if (uni)
            rbgs4s_uniform<ZERO>(d, rc[(unsigned)i * (unsigned)d.ny + (unsigned)j], x, b, col, i, j, 4 * q4);
        else
            rbgs4s_cells<C, ZERO>(d, cf, x, b, dinv, col, i, j, 4 * q4);
    });
}

// Residuals b - A x of the four colour-`col` cells m0 .. m0 + 3 of row (i, j), each evaluated as nbsum +
// diag_of do for the natural layout, with vector loads.
template <class C>
__device__ __forceinline__ void resid4_split(const Dims &d, const Coef<C> &cf, const float *__restrict__ x,
                                             const float *__restrict__ b, int col, int i, int j, int m0,
                                             float (&r)[4]) {
    const int nh = d.nz >> 1;
    const long long row = ((long long)i * d.ny + j) * nh + m0;
    const long long own = (long long)col * (d.n >> 1) + row, oth = (long long)(col ^ 1) * (d.n >> 1) + row;
    const long long sx = (long long)d.ny * nh, sy = nh;
    const bool xl = i > 0, xu = i < d.nx - 1, yl = j > 0, yu = j < d.ny - 1;
    float xc[4], xm[4] = {0, 0, 0, 0}, xp[4] = {0, 0, 0, 0}, ym[4] = {0, 0, 0, 0}, yp[4] = {0, 0, 0, 0}, zo[4];
    float bv[4];
    Cv4<C> axl, axu, ayl, ayu, azl, azo, dx;
    axu.zero();
    ayu.zero();
    ld4(x + own, xc);
    ld4(x + oth, zo);
    if (xl) ld4(x + oth - sx, xm);
    if (xu) ld4(x + oth + sx, xp);
    if (yl) ld4(x + oth - sy, ym);
    if (yu) ld4(x + oth + sy, yp);
    axl.load(cf.ax + own);
    if (xu) axu.load(cf.ax + oth + sx);
    ayl.load(cf.ay + own);
    if (yu) ayu.load(cf.ay + oth + sy);
    azl.load(cf.az + own);
    azo.load(cf.az + oth);
    dx.load(cf.dex + own);
    ld4(b + own, bv);
    auto body = [&](auto qc) {
        constexpr int QZ = decltype(qc)::value;
        float zx = 0.f, azx = 0.f;
        if (QZ == 0) {
            if (m0 > 0) zx = x[oth - 1];
        } else if (m0 + 4 < nh) {
            zx = x[oth + 4];
            azx = ldv(cf.az, oth + 4);
        }
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int k = 2 * (m0 + t) + QZ;
            float s = 0.f, sa = 0.f;
            if (xl) {
                const float a = axl[t];
                s += a * xm[t];
                sa += a;
            }
            if (xu) {
                const float a = axu[t];
                s += a * xp[t];
                sa += a;
            }
            if (yl) {
                const float a = ayl[t];
                s += a * ym[t];
                sa += a;
            }
            if (yu) {
                const float a = ayu[t];
                s += a * yp[t];
                sa += a;
            }
            if (k > 0) {
                const float a = azl[t];
                s += a * (QZ == 0 ? (t == 0 ? zx : zo[t == 0 ? 0 : t - 1]) : zo[t]);
                sa += a;
            }
            if (k < d.nz - 1) {
                const float a = QZ == 0 ? azo[t] : (t == 3 ? azx : azo[t == 3 ? 3 : t + 1]);
                s += a * (QZ == 0 ? zo[t] : (t == 3 ? zx : zo[t == 3 ? 3 : t + 1]));
                sa += a;
            }
            if (sizeof(C) == 2) {
                s *= cf.unscale;
                sa *= cf.unscale;
            }
            float e = dx[t];
            if (sizeof(C) == 2) e *= cf.unscale;
            const float D = sa + e;
            r[t] = (bv[t] - D * xc[t]) + s;
        }
    };
    if (((i + j + col) & 1) == 0)
        body(std::integral_constant<int, 0>{});
    else
        body(std::integral_constant<int, 1>{});
}

// Restriction of the split level-0 residual to the (natural) level 1, right after the pre-smoothing, whose
// last half sweep updates colour 1: a colour-1 cell's new value is (b + sum a x) / D of colour-0 values that
// did not change afterwards, so its residual is zero up to the rounding of that update, and only colour-0
// residuals are summed.  (The natural kernel evaluates all eight children; the difference is at rounding
// level.)  Thread (q4, J, I) sums coarse cells K0 = 4 q4 .. K0 + 3 over their x and y children, in the order
// of k_resid_restrict; in each fine row the colour-0 child of coarse cell K is the entry m = K.
// SOUT: the coarse level is split too: coarse cells K0, K0 + 2 (colour (I + J) & 1) and K0 + 1, K0 + 3 (the other)
// go to entries K0 / 2, K0 / 2 + 1 of their colour's half, as two float2.
template <class C, bool SOUT>
__device__ __forceinline__ void resid_restrict_s_cells(const Dims &d, const Coef<C> &cf, const float *__restrict__ x,
                                                       const float *__restrict__ b, const Dims &dc,
                                                       float *__restrict__ bc, const uint8_t *__restrict__ rows,
                                                       const float *__restrict__ crow, int I, int J, int K0) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int di = 0; di < 2; di++) {
        const int i = 2 * I + di;
        if (i >= d.nx) break;
        for (int dj = 0; dj < 2; dj++) {
            const int j = 2 * J + dj;
            if (j >= d.ny) break;
            if (!row_on(rows, d, i, j)) continue;  // residual zero
            float r[4];
            const long long fr = (long long)i * d.ny + j;
            if (rows && rows[fr] == 2)
                resid4_uniform(d, c_of(cf, crow[fr]), x, b, 0, i, j, K0, r);
            else
                resid4_split<C>(d, cf, x, b, 0, i, j, K0, r);
#pragma unroll
            for (int t = 0; t < 4; t++) acc[t] += r[t];
        }
    }
    if (SOUT) {
        const int pc = (I + J) & 1;
        const long long hc = dc.n >> 1, base = ((long long)I * dc.ny + J) * (dc.nz >> 1) + (K0 >> 1);
        *reinterpret_cast<float2 *>(bc + (long long)pc * hc + base) = make_float2(acc[0], acc[2]);
        *reinterpret_cast<float2 *>(bc + (long long)(pc ^ 1) * hc + base) = make_float2(acc[1], acc[3]);
    } else {
        *reinterpret_cast<float4 *>(bc + cid(dc, I, J, K0)) = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
}

template <class C, bool SOUT>
__global__ void __launch_bounds__(256) k_resid_restrict_s(Dims d, Coef<C> cf, const float *__restrict__ x,
                                                             const float *__restrict__ b, Dims dc,
                                                             float *__restrict__ bc, const uint8_t *__restrict__ rows,
                                                             const float *__restrict__ crow,
                                                             const int *__restrict__ list_c,
                                                             const int *__restrict__ count_c) {
    pdl_entry();
    const int nq = dc.nz >> 2;  // coarse float4 per row (dc.nz = nz / 2, a multiple of 4)
    for_list_items(list_c, count_c, 1, (nq + 31) / 32, [&](int, int I, int J, int ch, bool) {
        const int q4 = ch * 32 + threadIdx.x;
        if (q4 >= nq) return;
        resid_restrict_s_cells<C, SOUT>(d, cf, x, b, dc, bc, rows, crow, I, J, 4 * q4);
    });
}

// x += P xc on the split level 0 (piecewise constant): both colours' entries m of row (i, j) take coarse cell
// (i/2, j/2, m).
__global__ void __launch_bounds__(256) k_prolong_s(Dims d, float *__restrict__ x, Dims dc, const float *__restrict__ xc,
                                                   const int *__restrict__ list, const int *__restrict__ count) {
    pdl_entry();
    const int nh = d.nz >> 1, nq = nh >> 2;
    for_list_items(list, count, 1, (nq + 31) / 32, [&](int, int i, int j, int ch, bool) {
        const int q4 = ch * 32 + threadIdx.x;
        if (q4 >= nq) return;
        const long long r = (long long)i * d.ny + j;
        const int m0 = 4 * q4;
        float v[4];
        ld4(xc + cid(dc, i >> 1, j >> 1, m0), v);
        const long long row = r * nh + m0;
#pragma unroll
        for (int col = 0; col < 2; col++) {
            float *p = x + (long long)col * (d.n >> 1) + row;
            float4 t = *reinterpret_cast<float4 *>(p);
            t.x += v[0];
            t.y += v[1];
            t.z += v[2];
            t.w += v[3];
            *reinterpret_cast<float4 *>(p) = t;
        }
    });
}

// x += P xc with both levels split: fine entries m0 .. m0 + 3 of row (i, j) (either colour, k = 2m or 2m + 1) take
// coarse cells K = m0 .. m0 + 3 of coarse row (i/2, j/2): even K of colour (i/2 + j/2) & 1, odd K of the other,
// at entries K / 2 (two float2 loads).
__global__ void __launch_bounds__(256) k_prolong_ss(Dims d, float *__restrict__ x, Dims dc,
                                                    const float *__restrict__ xc, const int *__restrict__ list,
                                                    const int *__restrict__ count) {
    pdl_entry();
    const int nh = d.nz >> 1, nq = nh >> 2;
    const long long hc = dc.n >> 1;
    for_list_items(list, count, 1, (nq + 31) / 32, [&](int, int i, int j, int ch, bool) {
        const int q4 = ch * 32 + threadIdx.x;
        if (q4 >= nq) return;
        const long long r = (long long)i * d.ny + j;
        const int m0 = 4 * q4;
        const int I = i >> 1, J = j >> 1, pc = (I + J) & 1;
        const long long base = ((long long)I * dc.ny + J) * (dc.nz >> 1) + (m0 >> 1);
        const float2 ev = *reinterpret_cast<const float2 *>(xc + (long long)pc * hc + base);
        const float2 od = *reinterpret_cast<const float2 *>(xc + (long long)(pc ^ 1) * hc + base);
        const float v[4] = {ev.x, od.x, ev.y, od.y};
        const long long row = r * nh + m0;
#pragma unroll
        for (int col = 0; col < 2; col++) {
            float *p = x + (long long)col * (d.n >> 1) + row;
            float4 t = *reinterpret_cast<float4 *>(p);
            t.x += v[0];
            t.y += v[1];
            t.z += v[2];
            t.w += v[3];
            *reinterpret_cast<float4 *>(p) = t;
        }
    });
}

// q = A p and (p, q) on the split FP32 level-0 operator (the counterpart of k_apply_dot4; each cell's q as in
// k_apply_dot).  Persistent: warps over (colour row, chunk of 32 vectors), rows without an active cell skipped
// (q stays zero there).  Uniform rows are done for both colours in the colour-0 pass (apply4s_uniform2), so the
// colour-1 pass reads only the general rows again.
__global__ void __launch_bounds__(256, 3) k_apply_dot4s(Dims d, Coef<float> cf, const float *__restrict__ p,
                                                     float *__restrict__ q, const int *__restrict__ list,
                                                     const int *__restrict__ count, const float *__restrict__ crow,
                                                     double *sc, double *part, unsigned *ticket) {
    pdl_entry();
    float acc = 0.f;
    const int nh = d.nz >> 1, nq = nh >> 2;
    for_list_items(list, count, 2, (nq + 31) / 32, [&](int col, int i, int j, int ch, bool uni) {
        const int q4 = ch * 32 + threadIdx.x;
        if (q4 >= nq) return;
        const long long rw = (long long)i * d.ny + j;
        const int m0 = 4 * q4;
        if (uni) {  // both colours in the colour-0 pass
            if (col == 0) apply4s_uniform2(d, crow[rw], p, q, i, j, m0, acc);
            return;
        }
        const long long sx = (long long)d.ny * nh, sy = nh;
        const bool yl = j > 0, yu = j < d.ny - 1;
        {
            const long long row = rw * nh + m0;
            const long long own = (long long)col * (d.n >> 1) + row, oth = (long long)(col ^ 1) * (d.n >> 1) + row;
            const bool xl = i > 0, xu = i < d.nx - 1;
            const int qz = (i + j + col) & 1;
            float pc[4], po[4];
            float pxm[4] = {0, 0, 0, 0}, pxp[4] = {0, 0, 0, 0}, pym[4] = {0, 0, 0, 0}, pyp[4] = {0, 0, 0, 0};
            float axl[4], axu[4] = {0, 0, 0, 0}, ayl[4], ayu[4] = {0, 0, 0, 0}, azl[4], azo[4], dx[4];
            ld4(p + own, pc);
            ld4(p + oth, po);
            if (xl) ld4(p + oth - sx, pxm);
            if (xu) ld4(p + oth + sx, pxp);
            if (yl) ld4(p + oth - sy, pym);
            if (yu) ld4(p + oth + sy, pyp);
            ld4(cf.ax + own, axl);
            if (xu) ld4(cf.ax + oth + sx, axu);
            ld4(cf.ay + own, ayl);
            if (yu) ld4(cf.ay + oth + sy, ayu);
            ld4(cf.az + own, azl);
            ld4(cf.az + oth, azo);
            ld4(cf.dex + own, dx);
            float out[4];
            auto body = [&](auto qc) {
                constexpr int QZ = decltype(qc)::value;
                float zx = 0.f, azx = 0.f;
                if (QZ == 0) {
                    if (m0 > 0) zx = p[oth - 1];
                } else if (m0 + 4 < nh) {
                    zx = p[oth + 4];
                    azx = cf.az[oth + 4];
                }
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int k = 2 * (m0 + t) + QZ;
                    float s = 0.f, sa = 0.f;
                    if (xl) {
                        s += axl[t] * pxm[t];
                        sa += axl[t];
                    }
                    if (xu) {
                        s += axu[t] * pxp[t];
                        sa += axu[t];
                    }
                    if (yl) {
                        s += ayl[t] * pym[t];
                        sa += ayl[t];
                    }
                    if (yu) {
                        s += ayu[t] * pyp[t];
                        sa += ayu[t];
                    }
                    if (k > 0) {
                        const float a = azl[t];
                        s += a * (QZ == 0 ? (t == 0 ? zx : po[t == 0 ? 0 : t - 1]) : po[t]);
                        sa += a;
                    }
                    if (k < d.nz - 1) {
                        const float a = QZ == 0 ? azo[t] : (t == 3 ? azx : azo[t == 3 ? 3 : t + 1]);
                        s += a * (QZ == 0 ? po[t] : (t == 3 ? zx : po[t == 3 ? 3 : t + 1]));
                        sa += a;
                    }
                    const float D = sa + dx[t];
                    out[t] = D * pc[t] - s;
                    acc += pc[t] * out[t];
                }
            };
            if (qz == 0)
                body(std::integral_constant<int, 0>{});
            else
                body(std::integral_constant<int, 1>{});
            *reinterpret_cast<float4 *>(q + own) = make_float4(out[0], out[1], out[2], out[3]);
        }
    });
    float v[1] = {acc};
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) {
        sc[S_PQ] = tot[0];
        if (tot[0] > 0 && isfinite(tot[0])) {
            sc[S_ALPHA] = sc[S_RHO] / tot[0];
        } else {
            sc[S_ALPHA] = 0;
            sc[S_AUX0] = 1;  // breakdown
        }
    }
}

// Level 1 of the mixed form (FP16, scaled) from the split FP32 level 0: A_c = 1/2 P^T A P as k_coarsen forms
// it (a coarse face is half the sum of its four fine faces, a coarse excess half the sum of its eight children's),
// summed in FP32 from the FP32 copy instead of FP64 from the FP64 operator (the result is stored in FP16).  Fine
// row (i, j) holds both children k = 2K, 2K + 1 of coarse cell K at m = K: colour (i + j) & 1 for k = 2K.
// cs: when its arrays are set, the same values also go to a split copy of the coarse level (nz / 2 % 8 == 0).
__global__ void __launch_bounds__(256) k_coarsen_s(Dims d, Coef<float> f, Dims dc, Coef<__half> cc, Coef<__half> cs) {
    const int K = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int I = blockIdx.z;
    if (K >= dc.nz || J >= dc.ny) return;
    const int nh = d.nz >> 1;
    const long long hn = d.n >> 1;
    // entry m = K of colour col in fine row (i, j)
    auto at = [&](const float *a, int col, int i, int j) {
        return a[(long long)col * hn + ((long long)i * d.ny + j) * nh + K];
    };
    float fx = 0.f, fy = 0.f, fz = 0.f, dex = 0.f;
    for (int u = 0; u < 2; u++)
        for (int v = 0; v < 2; v++) {
            // lower x faces of fine cells (2I, 2J + u, 2K + v); lower y faces of (2I + u, 2J, 2K + v)
            if (I > 0 && 2 * J + u < d.ny) fx += at(f.ax, (u + v) & 1, 2 * I, 2 * J + u);
            if (J > 0 && 2 * I + u < d.nx) fy += at(f.ay, (u + v) & 1, 2 * I + u, 2 * J);
            // lower z faces of fine cells (2I + u, 2J + v, 2K): colour (u + v) & 1
            if (K > 0 && 2 * I + u < d.nx && 2 * J + v < d.ny) fz += at(f.az, (u + v) & 1, 2 * I + u, 2 * J + v);
            if (2 * I + u < d.nx && 2 * J + v < d.ny) {
                dex += at(f.dex, 0, 2 * I + u, 2 * J + v);
                dex += at(f.dex, 1, 2 * I + u, 2 * J + v);
            }
        }
    const float sc = 0.5f * cc.scale;
    const long long c = cid(dc, I, J, K);
    const __half hx = __float2half_rn(fx * sc), hy = __float2half_rn(fy * sc), hz = __float2half_rn(fz * sc),
                 hd = __float2half_rn(dex * sc);
    cc.ax[c] = hx;
    cc.ay[c] = hy;
    cc.az[c] = hz;
    cc.dex[c] = hd;
    if (cs.ax) {
        const long long q = split_index(dc, I, J, K);
        cs.ax[q] = hx;
        cs.ay[q] = hy;
        cs.az[q] = hz;
        cs.dex[q] = hd;
    }
}

// Items of the persistent split kernels: rows x chunks of 32 float4.
static inline long long split_items(long long nrows, int nq) { return nrows * ((nq + 31) / 32); }

static void apply_dot32s(cudaStream_t st, const Dims &d, const Coef<float> &cf, const float *p, float *q,
                         const int *list, const int *count, const float *crow, double *sc, double *part,
                         unsigned *ticket) {
    const int g = row_grid((const void *)k_apply_dot4s, split_items(2LL * d.nx * d.ny, d.nz >> 3));
    launch_pdl(k_apply_dot4s, g, dim3(32, 8), st, d, cf, p, q, list, count, crow, sc, part, ticket);
}
