// Warp-cooperative spreading / interpolation kernels (included by nufft_spread.cu and
// nufft_interp.cu).
//
// One CTA per subproblem (a bin of the fine grid, or a <= maxsub slice of a dense bin).
// Points are sorted by bin, then by the origin of their kernel window (see point_key in
// nufft.cu), so consecutive points of a subproblem mostly share the whole w^3 window.  Each
// warp walks a contiguous run of the subproblem's points, 32 at a time: the lanes load 32
// points' coordinates (and strengths) with coalesced loads, then the warp treats the points
// one after another, broadcasting each with a shuffle.  The window is split over the lanes:
// lane = (bl, e), e = lane % EW the z offset, bl = lane / EW the first y offset, the lane
// covering y offsets b = bl + r * (32 / EW) for r < ROUNDS and every x offset a < w.  Shared
// subgrid rows have a pitch P with P mod 32 in {8, 24} (EW = 8) or 16 (EW = 16), so the 32
// addresses of a shared-memory instruction fall in 32 distinct banks.  Complex grids are
// planar (re | im).  The 3w kernel values of a point are evaluated once, one per lane, and
// gathered with shuffles.
//
// W > 0 fixes the kernel width at compile time; the lane's ROUNDS x W window cells then
// live in registers across a run of points with the same window origin: spreading
// accumulates into them and touches shared memory (shared atomics) only when the origin
// changes; interpolation loads them once per run.  W = 0 reads the width at run time
// (w <= 16) and works on shared memory point by point.  The flush adds a subproblem's
// subgrid to the fine grid once (global atomics only there, where neighbouring bins'
// halos overlap).

template <int W>
struct WarpLayout {
    static constexpr int EW = (W > 0 && W <= 8) ? 8 : 16;  // z lanes
    static constexpr int BR = 32 / EW;                      // y offsets per round
    static constexpr int KMAX = W > 0 ? W : MAXW;           // unroll bound of the x loop
    static constexpr int RMAX = W > 0 ? (W + BR - 1) / BR : 8;
};

// value q (< 3w) of the point's kernel values, held in lane q % 32 of v0 (q < 32) or v1
template <typename T>
__device__ __forceinline__ T getk(T v0, T v1, int q, bool two)
{
    T a = __shfl_sync(0xffffffffu, v0, q & 31);
    if (!two) return a;
    T b = __shfl_sync(0xffffffffu, v1, q & 31);
    return q < 32 ? a : b;
}

// Window origin (relative to the bin origin) of a point, and this lane's share of its 3w
// kernel values.
template <typename T>
__device__ __forceinline__ void point_origin(T px, T py, T pz, int w, int &lx, int &ly, int &lz)
{
    const T hw = T(0.5) * T(w);
    lx = (int)ceil(px - hw);
    ly = (int)ceil(py - hw);
    lz = (int)ceil(pz - hw);
}

template <typename T>
__device__ __forceinline__ void point_values(T px, T py, T pz, int lx, int ly, int lz, int w, T beta, int lane,
                                             T &v0, T &v1)
{
    const T inv = T(2) / T(w);
    auto val = [&](int q) -> T {
        if (q >= 3 * w) return T(0);
        int d = q / w, k = q - d * w;
        T u = d == 0 ? px : (d == 1 ? py : pz);
        int l0 = d == 0 ? lx : (d == 1 ? ly : lz);
        T t = (T(l0 + k) - u) * inv;
        return es_eval(t * t, beta);
    };
    v0 = val(lane);
    v1 = 3 * w > 32 ? val(lane + 32) : T(0);
}

__device__ __forceinline__ int wrapi(int g, int n) { return g + (g < 0 ? n : (g >= n ? -n : 0)); }

// the contiguous run [t0, t1) of a subproblem's cnt points handled by warp `warp`
__device__ __forceinline__ void warp_run(int cnt, int warp, int nwarps, int &t0, int &t1)
{
    int chunk = (cnt + nwarps - 1) / nwarps;
    t0 = min(cnt, warp * chunk);
    t1 = min(cnt, t0 + chunk);
}

// origins are bin-relative, in [-w/2, bs] with bs <= 32: pack them into one int
__device__ __forceinline__ int origin_key(int lx, int ly, int lz) { return ((lx + 16) * 64 + (ly + 16)) * 64 + lz + 16; }

// ------------------------------------------------------------------ spread (type 1)

// CPLX: complex strengths (interleaved in c), else real (c == nullptr: all ones).
// PRIV: per-warp private subgrid copies (plain adds), else one copy with shared atomics.
// Fine grid: complex n^3 interleaved (CPLX) or real with row stride rs (in-place R2C layout).
template <typename T, bool CPLX, int W, bool PRIV>
__global__ void __launch_bounds__(256) k_spread(const int *sub_bin, const int *sub_off, const int *bin_count,
                                                const int *bin_start, const int *perm, const T *ux, const T *uy,
                                                const T *uz, const T *c, SubgridGeom gm, T beta, T *fine)
{
    using L = WarpLayout<W>;
    extern __shared__ unsigned char smem_raw[];
    T *sg = reinterpret_cast<T *>(smem_raw);
    const int S = gm.S, P = gm.P, w = W > 0 ? W : gm.w, h = w / 2;
    const int rounds = (w + L::BR - 1) / L::BR;
    const bool two = 3 * w > 32;
    const int plane = S * P, copy = S * plane;
    const int nch = CPLX ? 2 : 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int ncopy = PRIV ? nwarps : 1;
    for (int i = threadIdx.x; i < ncopy * nch * copy; i += blockDim.x) sg[i] = T(0);
    __syncthreads();

    const int b = sub_bin[blockIdx.x];
    const int off = sub_off[blockIdx.x];
    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % L::EW, bl = lane / L::EW;
    const bool ez = e < w;
    T *mine = sg + (PRIV ? warp * nch * copy : 0);
    auto add = [&](int idx, T v) {
        if (PRIV) mine[idx] += v;
        else atomicAdd(&mine[idx], v);
    };

    // register window of the current run (W > 0)
    T acc[L::RMAX][L::KMAX], aci[L::RMAX][L::KMAX];
    int cur_key = -1, cur_base = 0;
    auto flush = [&]() {
        if constexpr (W > 0) {
            if (cur_key < 0) return;
#pragma unroll
            for (int r = 0; r < L::RMAX; ++r) {
                const int bb = bl + r * L::BR;
                const bool ok = ez && bb < w;
#pragma unroll
                for (int a = 0; a < L::KMAX; ++a) {
                    if (ok) {
                        const int idx = cur_base + bb * P + a * plane;
                        add(idx, acc[r][a]);
                        if (CPLX) add(copy + idx, aci[r][a]);
                    }
                    acc[r][a] = T(0);
                    aci[r][a] = T(0);
                }
            }
        }
    };
#pragma unroll
    for (int r = 0; r < L::RMAX; ++r)
#pragma unroll
        for (int a = 0; a < L::KMAX; ++a) {
            acc[r][a] = T(0);
            aci[r][a] = T(0);
        }

    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    const T cs = (T)gm.cscale;
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const bool valid = tl < t1;
        const int pos = p0 + (valid ? tl : t0);
        const T mx = ux[pos] * cs, my = uy[pos] * cs, mz = uz[pos] * cs;
        T mr = T(1), mi = T(0);
        if (c && valid) {
            const int64_t j = perm[pos];
            if (CPLX) {
                mr = c[2 * j];
                mi = c[2 * j + 1];
            } else {
                mr = c[j];
            }
        }
        const int nq = min(32, t1 - base);
        for (int q = 0; q < nq; ++q) {
            const T px = __shfl_sync(0xffffffffu, mx, q);
            const T py = __shfl_sync(0xffffffffu, my, q);
            const T pz = __shfl_sync(0xffffffffu, mz, q);
            const T vr = __shfl_sync(0xffffffffu, mr, q);
            const T vi = CPLX ? __shfl_sync(0xffffffffu, mi, q) : T(0);
            int lx, ly, lz;
            point_origin(px, py, pz, w, lx, ly, lz);
            T v0, v1;
            point_values(px, py, pz, lx, ly, lz, w, beta, lane, v0, v1);
            T kx[L::KMAX];
#pragma unroll
            for (int a = 0; a < L::KMAX; ++a) kx[a] = (W > 0 || a < w) ? getk(v0, v1, a, two) : T(0);
            const T kz = getk(v0, v1, 2 * w + (ez ? e : 0), two);
            const int base_idx = ((lx + h) * S + (ly + h)) * P + lz + h + e;
            if (W > 0) {
                const int key = origin_key(lx, ly, lz);  // warp-uniform
                if (key != cur_key) {
                    flush();
                    cur_key = key;
                    cur_base = base_idx;
                }
            }
#pragma unroll
            for (int r = 0; r < L::RMAX; ++r) {
                if (W == 0 && r >= rounds) break;
                const int bb = bl + r * L::BR;
                const T ky = getk(v0, v1, w + (bb < w ? bb : 0), two);
                const T kyz = ky * kz;
                const T wr = kyz * vr, wi = kyz * vi;
                if (W > 0) {
#pragma unroll
                    for (int a = 0; a < L::KMAX; ++a) {
                        acc[r][a] += kx[a] * wr;
                        if (CPLX) aci[r][a] += kx[a] * wi;
                    }
                } else {
                    if (!ez || bb >= w) continue;
                    int idx = base_idx + bb * P;
#pragma unroll
                    for (int a = 0; a < L::KMAX; ++a) {
                        if (a < w) {
                            add(idx, kx[a] * wr);
                            if (CPLX) add(copy + idx, kx[a] * wi);
                        }
                        idx += plane;
                    }
                }
            }
        }
    }
    flush();
    __syncthreads();
    const int bx = b / (gm.nb * gm.nb), by = (b / gm.nb) % gm.nb, bz = b % gm.nb;
    const int ox = bx * gm.bs - h, oy = by * gm.bs - h, oz = bz * gm.bs - h;
    const int n = gm.n;
    for (int i = threadIdx.x; i < S * S * S; i += blockDim.x) {
        const int a = i / (S * S), rem = i - a * S * S, bb = rem / S, ee = rem - bb * S;
        const int li = (a * S + bb) * P + ee;
        T sr = T(0), si = T(0);
        for (int k = 0; k < ncopy; ++k) {
            sr += sg[k * nch * copy + li];
            if (CPLX) si += sg[k * nch * copy + copy + li];
        }
        if (sr == T(0) && si == T(0)) continue;
        const int gx = wrapi(ox + a, n), gy = wrapi(oy + bb, n), gz = wrapi(oz + ee, n);
        if (CPLX) {
            const int64_t g = ((int64_t)gx * n + gy) * n + gz;
            atomicAdd(&fine[2 * g], sr);
            atomicAdd(&fine[2 * g + 1], si);
        } else {
            atomicAdd(&fine[((int64_t)gx * n + gy) * gm.rs + gz], sr);
        }
    }
}

// ------------------------------------------------------------------ table-driven spread

// 8 consecutive values to / from shared memory with 16-byte accesses (p 16-byte aligned).
template <typename T>
__device__ __forceinline__ void load8(const T *p, T (&v)[8])
{
    if constexpr (sizeof(T) == 4) {
        const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const double2 d = reinterpret_cast<const double2 *>(p)[i];
            v[2 * i] = d.x, v[2 * i + 1] = d.y;
        }
    }
}
template <typename T>
__device__ __forceinline__ void store8(T *p, const T (&v)[8])
{
    if constexpr (sizeof(T) == 4) {
        reinterpret_cast<float4 *>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
        reinterpret_cast<float4 *>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) reinterpret_cast<double2 *>(p)[i] = make_double2(v[2 * i], v[2 * i + 1]);
    }
}

// Owner-lane set-up of one point for the table-driven kernels: the window origin (with EXT
// the origin of the point's sort group on a derived plan's twice finer grid: point_key's
// coarse origin and refinement, the fine origin then being the group origin + d, d in
// {0,1} per dimension), the 3W kernel values, and the table record rec (16-byte aligned):
//   [0, 8)   x values by window column a (shifted by d with EXT; zero outside the window)
//   [8, 16)  y values in pairs (row b, row b + 4), b < 4
//   [16, ..) z values (ZMODE 0), z values times vr (1), or (z vr, z vi) pairs (2)
// Returns the origin key (origin_key) of the window.
template <typename T, int W, bool EXT, int ZMODE>
__device__ __forceinline__ int tab_prepare(T px, T py, T pz, T beta, T vr, T vi, T *rec)
{
    const T hw = T(0.5) * T(W), inv = T(2) / T(W);
    const int lx = (int)ceil(px - hw), ly = (int)ceil(py - hw), lz = (int)ceil(pz - hw);
    int gx = lx, gy = ly, gz = lz;
    if (EXT) {
        const int base_off = (W - 2 - (W & 1)) / 2;  // fine origin = 2 coarse origin + base_off + {0,1,2}
        const int cx = (int)ceil(px * T(0.5) - hw), cy = (int)ceil(py * T(0.5) - hw),
                  cz = (int)ceil(pz * T(0.5) - hw);
        gx = 2 * cx + base_off + 2 * ((lx - 2 * cx - base_off) >> 1);
        gy = 2 * cy + base_off + 2 * ((ly - 2 * cy - base_off) >> 1);
        gz = 2 * cz + base_off + 2 * ((lz - 2 * cz - base_off) >> 1);
    }
    const int dx = lx - gx, dy = ly - gy, dz = lz - gz;  // 0 or 1 (EXT), else 0
    T kx[W], ky[W], kz[W];
    if constexpr (sizeof(T) == 4) {
        // t_k = t_0 + k (2 / W): one FMA per kernel argument, branch-free evaluation
        const T ax = (T(lx) - px) * inv, ay = (T(ly) - py) * inv, az = (T(lz) - pz) * inv;
        const T bl2e = beta * T(1.4426950408889634);
#pragma unroll
        for (int k = 0; k < W; ++k) {
            kx[k] = es_eval_tab(fmaf(T(k), inv, ax), bl2e);
            ky[k] = es_eval_tab(fmaf(T(k), inv, ay), bl2e);
            kz[k] = es_eval_tab(fmaf(T(k), inv, az), bl2e);
        }
    } else {
#pragma unroll
        for (int k = 0; k < W; ++k) {
            const T tx = (T(lx + k) - px) * inv, ty = (T(ly + k) - py) * inv, tz = (T(lz + k) - pz) * inv;
            kx[k] = es_eval(tx * tx, beta);
            ky[k] = es_eval(ty * ty, beta);
            kz[k] = es_eval(tz * tz, beta);
        }
    }
    // the values by window column / row / z offset (shifted by d when EXT)
    auto col = [&](const T(&v)[W], int d, int a) -> T {
        const T v0 = a < W ? v[a < W ? a : 0] : T(0);
        if (!EXT) return v0;
        const T v1 = (a >= 1 && a - 1 < W) ? v[(a >= 1 && a - 1 < W) ? a - 1 : 0] : T(0);
        return d ? v1 : v0;
    };
    T o[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) o[a] = col(kx, dx, a);
    store8(rec, o);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        o[2 * q] = col(ky, dy, q);
        o[2 * q + 1] = col(ky, dy, q + 4);
    }
    store8(rec + 8, o);
    if (ZMODE == 2) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const T z = col(kz, dz, q);
            o[2 * q] = z * vr;
            o[2 * q + 1] = z * vi;
        }
        store8(rec + 16, o);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const T z = col(kz, dz, q + 4);
            o[2 * q] = z * vr;
            o[2 * q + 1] = z * vi;
        }
        store8(rec + 24, o);
    } else {
#pragma unroll
        for (int a = 0; a < 8; ++a) o[a] = ZMODE == 1 ? col(kz, dz, a) * vr : col(kz, dz, a);
        store8(rec + 16, o);
    }
    return origin_key(gx, gy, gz);
}

// Per-warp point table of k_spread_tab: 32 records (tab_prepare) of REC values, one per
// point of the current batch; the z part holds 8 reals or 8 (re, im) pairs.
template <typename T, bool CPLX>
struct SpreadTable {
    static constexpr int REC = CPLX ? 32 : 24;
    static constexpr size_t bytes_per_warp = 32 * REC * sizeof(T);
};

// Shared-memory bytes of k_spread_tab: the subgrid(s), 16-byte aligned, then one table per warp.
template <typename T, bool CPLX>
__host__ __device__ inline size_t spread_tab_smem(size_t subgrid_bytes, int warps)
{
    return ((subgrid_bytes * (CPLX ? 2 : 1) + 15) & ~(size_t)15) + warps * SpreadTable<T, CPLX>::bytes_per_warp;
}

// Table-driven spreading (kernel width W fixed at compile time).  Each warp walks its run
// of the subproblem's points in batches of 32.  Per batch, lane t prepares point t alone:
// coordinates, window origin, its 3W kernel values and strength, written as one record of
// the warp's table.  The warp then treats the 32 points in order; per point a lane reads the
// record's x values (two 16-byte broadcasts), its (y, y + 4) pair and its z value times the
// strength, and adds 2 x NX products into its register window: the lane (bl, e) owns
// window rows bl and bl + 4 at z offset e, all NX columns.  Shared memory is written only
// when the window origin changes (the register window is added with shared atomics).
//
// EXT (a derived plan's twice finer grid, cscale = 2): the register window is the
// (W+1)^3 extended window of the point's sort group (point_key's coarse origin and
// refinement); within a group the fine window origin is the group origin G plus d in {0,1}
// per dimension, and the owner lane writes its values already shifted by d, so runs span
// whole groups.  NX = W + 1 (EXT) or W columns, NX <= 8.
template <typename T, bool CPLX, int W, bool EXT>
__device__ __forceinline__ void spread_tab_sub(int b, int off, const int *bin_count, const int *bin_start,
                                               const int *perm, const T *ux, const T *uy, const T *uz, const T *c,
                                               const SubgridGeom &gm, T beta, T *fine)
{
    constexpr int NX = EXT ? W + 1 : W;
    static_assert(W >= 2 && NX <= 8, "table spreading needs a window of at most 8 columns");
    constexpr int EW = 8, BR = 4, RX = (NX + BR - 1) / BR;
    constexpr int REC = SpreadTable<T, CPLX>::REC;
    constexpr int nch = CPLX ? 2 : 1;
    using T2 = typename cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sg = reinterpret_cast<T *>(smem_raw);
    const int S = gm.S, P = gm.P, h = W / 2;
    const int plane = S * P, copy = S * plane;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const size_t sgb = ((size_t)nch * copy * sizeof(T) + 15) & ~(size_t)15;
    T *tab = reinterpret_cast<T *>(smem_raw + sgb) + warp * 32 * REC;
    for (int i = threadIdx.x; i < nch * copy; i += blockDim.x) sg[i] = T(0);
    __syncthreads();

    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % EW, bl = lane / EW;

    // FP32 real strengths: the window's columns in pairs, updated with the packed FP32 FMA
    // (fma.rn.f32x2: two independent round-to-nearest FMAs per instruction, fewer
    // instructions issued; the sums are held to the same tolerance as scalar ones, with no
    // claim of equal bits: a compensated sequence written with these builtins differed from
    // its scalar form on sm_103a); an odd width's last column keeps scalar FMAs
    // (acc[r][NX - 1]).
    constexpr bool PK = sizeof(T) == 4 && !CPLX;
    constexpr int NP = NX / 2;
    T acc[RX][NX], aci[RX][NX];
    float2 ap[RX][NP];
#pragma unroll
    for (int r = 0; r < RX; ++r) {
#pragma unroll
        for (int a = 0; a < NX; ++a) acc[r][a] = aci[r][a] = T(0);
#pragma unroll
        for (int k = 0; k < NP; ++k) ap[r][k] = make_float2(0.f, 0.f);
    }
    int cur_key = -1, X0 = 0, Y0 = 0, Z0 = 0;  // subgrid cell of the register window's corner
    auto flush = [&]() {
        if (cur_key < 0) return;
        const int zz = Z0 + e;
#pragma unroll
        for (int r = 0; r < RX; ++r) {
            const int yy = Y0 + bl + r * BR;
            const bool row_ok = e < NX && bl + r * BR < NX && (!EXT || (zz >= 0 && zz < S && yy >= 0 && yy < S));
#pragma unroll
            for (int a = 0; a < NX; ++a) {
                const int xx = X0 + a;
                const T v = PK && a < 2 * NP ? T((a & 1) ? ap[r][a >> 1].y : ap[r][a >> 1].x) : acc[r][a];
                // extended cells outside the subgrid never receive a contribution
                if (row_ok && (!EXT || (xx >= 0 && xx < S))) {
                    const int idx = (xx * S + yy) * P + zz;
                    if (v != T(0)) atomicAdd(&sg[idx], v);
                    if (CPLX && aci[r][a] != T(0)) atomicAdd(&sg[copy + idx], aci[r][a]);
                }
                acc[r][a] = aci[r][a] = T(0);
            }
#pragma unroll
            for (int k = 0; k < NP; ++k) ap[r][k] = make_float2(0.f, 0.f);
        }
    };

    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    const T cs = (T)gm.cscale;
    // point base + lane's coordinates and strength; FP32 real strengths on the plan's own grid
    // load the next batch's while the current one is walked (the strength is a gather through
    // the permutation; the extended-window form has no spare registers for it)
    auto fetch = [&](int base, T &fx, T &fy, T &fz, T &fr, T &fi) {
        const int tl = base + lane;
        const bool valid = tl < t1;
        const int pos = p0 + (valid ? tl : t0);
        fx = ux[pos];
        fy = uy[pos];
        fz = uz[pos];
        fr = T(1);
        fi = T(0);
        if (!valid) {
            fr = T(0);
        } else if (c) {
            const int64_t j = perm[pos];
            if (CPLX) {
                const T2 cv = reinterpret_cast<const T2 *>(c)[j];
                fr = cv.x;
                fi = cv.y;
            } else {
                fr = c[j];
            }
        }
    };
    constexpr bool PREF = sizeof(T) == 4 && !CPLX && !EXT;
    T nx = T(0), ny = T(0), nz = T(0), nr = T(0), ni = T(0);
    if (PREF && t0 < t1) fetch(t0, nx, ny, nz, nr, ni);
    for (int base = t0; base < t1; base += 32) {
        // ---- lane `lane` prepares point base + lane
        T px, py, pz, vr, vi;
        if constexpr (PREF) {
            px = nx, py = ny, pz = nz, vr = nr, vi = ni;
            if (base + 32 < t1) fetch(base + 32, nx, ny, nz, nr, ni);
        } else {
            fetch(base, px, py, pz, vr, vi);
        }
        px *= cs;
        py *= cs;
        pz *= cs;
        __syncwarp();  // the previous batch's records have been read
        const int my_key = tab_prepare<T, W, EXT, CPLX ? 2 : 1>(px, py, pz, beta, vr, vi, tab + lane * REC);
        __syncwarp();
        // ---- the warp adds the batch's points in order, run by run: bit q of `starts` marks
        // a point whose window origin differs from its predecessor's, so each run of equal
        // origins is one branch-free loop (the flush test happens once per run)
        const int nq = min(32, t1 - base);
        const int prev_key = __shfl_up_sync(0xffffffffu, my_key, 1);
        unsigned starts = __ballot_sync(0xffffffffu, lane == 0 || my_key != prev_key);
        starts &= nq >= 32 ? 0xffffffffu : ((1u << nq) - 1u);
        int q = 0;
        while (q < nq) {
            const unsigned later = starts & ~((2u << q) - 1u);  // starts after q (2u << 31 wraps to 0)
            const int qe = later ? __ffs(later) - 1 : nq;
            const int key = __shfl_sync(0xffffffffu, my_key, q);  // warp-uniform
            if (key != cur_key) {
                flush();
                cur_key = key;
                X0 = (key >> 12) - 16 + h;
                Y0 = ((key >> 6) & 63) - 16 + h;
                Z0 = (key & 63) - 16 + h;
            }
            const T *rq = tab + q * REC;
            const T *const rend = tab + qe * REC;
#pragma unroll 4
            for (; rq < rend; rq += REC) {
                T xv[8];
                load8(rq, xv);
                const T2 yv = reinterpret_cast<const T2 *>(rq + 8)[bl];
                if (CPLX) {
                    const T2 zv = reinterpret_cast<const T2 *>(rq + 16)[e];
                    const T wr0 = yv.x * zv.x, wi0 = yv.x * zv.y, wr1 = yv.y * zv.x, wi1 = yv.y * zv.y;
#pragma unroll
                    for (int a = 0; a < NX; ++a) {
                        acc[0][a] += xv[a] * wr0;
                        aci[0][a] += xv[a] * wi0;
                        if (RX > 1) {
                            acc[RX - 1][a] += xv[a] * wr1;
                            aci[RX - 1][a] += xv[a] * wi1;
                        }
                    }
                } else if constexpr (PK) {
                    const T zv = rq[16 + e];
                    const float w0 = yv.x * zv, w1 = yv.y * zv;
                    const float2 w0p = make_float2(w0, w0), w1p = make_float2(w1, w1);
#pragma unroll
                    for (int k = 0; k < NP; ++k) {
                        const float2 xk = make_float2(xv[2 * k], xv[2 * k + 1]);
                        ap[0][k] = __ffma2_rn(xk, w0p, ap[0][k]);
                        if (RX > 1) ap[RX - 1][k] = __ffma2_rn(xk, w1p, ap[RX - 1][k]);
                    }
                    if (NX % 2) {
                        acc[0][NX - 1] += xv[NX - 1] * w0;
                        if (RX > 1) acc[RX - 1][NX - 1] += xv[NX - 1] * w1;
                    }
                } else {
                    const T zv = rq[16 + e];
                    const T w0 = yv.x * zv, w1 = yv.y * zv;
#pragma unroll
                    for (int a = 0; a < NX; ++a) {
                        acc[0][a] += xv[a] * w0;
                        if (RX > 1) acc[RX - 1][a] += xv[a] * w1;
                    }
                }
            }
            q = qe;
        }
    }
    flush();
    __syncthreads();
    const int bx = b / (gm.nb * gm.nb), by = (b / gm.nb) % gm.nb, bz = b % gm.nb;
    const int ox = bx * gm.bs - h, oy = by * gm.bs - h, oz = bz * gm.bs - h;
    const int n = gm.n;
    for (int i = threadIdx.x; i < S * S * S; i += blockDim.x) {
        const int a = i / (S * S), rem = i - a * S * S, bb = rem / S, ee = rem - bb * S;
        const int li = (a * S + bb) * P + ee;
        const T sr = sg[li], si = CPLX ? sg[copy + li] : T(0);
        if (sr == T(0) && si == T(0)) continue;
        const int gxx = wrapi(ox + a, n), gyy = wrapi(oy + bb, n), gzz = wrapi(oz + ee, n);
        if (CPLX) {
            const int64_t g = ((int64_t)gxx * n + gyy) * n + gzz;
            atomicAdd(&fine[2 * g], sr);
            atomicAdd(&fine[2 * g + 1], si);
        } else {
            atomicAdd(&fine[((int64_t)gxx * n + gyy) * gm.rs + gzz], sr);
        }
    }
}

// One subproblem per CTA (sub_bin / sub_off list of one plan).
template <typename T, bool CPLX, int W, bool EXT>
__global__ void __launch_bounds__(256) k_spread_tab(const int *sub_bin, const int *sub_off, const int *bin_count,
                                                    const int *bin_start, const int *perm, const T *ux,
                                                    const T *uy, const T *uz, const T *c, SubgridGeom gm, T beta,
                                                    T *fine)
{
    spread_tab_sub<T, CPLX, W, EXT>(sub_bin[blockIdx.x], sub_off[blockIdx.x], bin_count, bin_start, perm, ux, uy, uz,
                                    c, gm, beta, fine);
}

// ------------------------------------------------------------------ batches of plans

// Persistent CTAs take the next work item from a device counter until the list is done.
// Returns the item index (all threads of the CTA see the same value).
__device__ __forceinline__ int next_item(int *next)
{
    __shared__ int item;
    __syncthreads();  // every thread is done with the previous item
    if (threadIdx.x == 0) item = atomicAdd(next, 1);
    __syncthreads();
    return item;
}

// Spreading over the subproblems of all plans of a batch (same precision, strength type and
// kernel width; bin size, grid size and points per plan), one persistent launch.  EXT: every
// plan is derived (a twice finer grid) and spreads through the extended register window.
template <typename T, bool CPLX, int W, bool EXT>
__global__ void __launch_bounds__(256) k_spread_tab_batch(const WorkItem *work, int nwork, const InstDesc<T> *inst,
                                                          T beta, int *next)
{
    for (;;) {
        const int it = next_item(next);
        if (it >= nwork) return;
        const WorkItem wk = work[it];
        const InstDesc<T> d = inst[wk.inst];
        spread_tab_sub<T, CPLX, W, EXT>(wk.bin, wk.off, d.bin_count, d.bin_start, d.perm, (const T *)d.ux,
                                          (const T *)d.uy, (const T *)d.uz, (const T *)d.in, d.gm, beta,
                                          (T *)d.out);
    }
}

// ------------------------------------------------------------------ table-driven interp

// Loads the subproblem's subgrid (padded rows; planar complex) from the fine grid.
template <typename T, bool CPLX>
__device__ __forceinline__ void load_subgrid(const T *fine, const SubgridGeom &gm, int b, T *sg)
{
    const int S = gm.S, P = gm.P, h = gm.w / 2, n = gm.n;
    const int copy = S * S * P;
    const int bx = b / (gm.nb * gm.nb), by = (b / gm.nb) % gm.nb, bz = b % gm.nb;
    const int ox = bx * gm.bs - h, oy = by * gm.bs - h, oz = bz * gm.bs - h;
    for (int i = threadIdx.x; i < S * S * S; i += blockDim.x) {
        const int a = i / (S * S), rem = i - a * S * S, bb = rem / S, ee = rem - bb * S;
        const int li = (a * S + bb) * P + ee;
        const int gx = wrapi(ox + a, n), gy = wrapi(oy + bb, n), gz = wrapi(oz + ee, n);
        if (CPLX) {
            const int64_t g = ((int64_t)gx * n + gy) * n + gz;
            sg[li] = fine[2 * g];
            sg[copy + li] = fine[2 * g + 1];
        } else {
            sg[li] = fine[((int64_t)gx * n + gy) * gm.rs + gz];
        }
    }
}

// Shared-memory bytes of k_interp_tab: the staged subgrid(s), then per warp a table of 32
// records (24 values) and 32 x 8 partial sums (values, or (re, im) pairs).
template <typename T, bool CPLX>
__host__ __device__ inline size_t interp_tab_smem(size_t subgrid_bytes, int warps)
{
    return ((subgrid_bytes * (CPLX ? 2 : 1) + 15) & ~(size_t)15) +
           warps * 32 * (24 + 8 * (CPLX ? 2 : 1)) * sizeof(T);
}

// Table-driven interpolation (kernel width W <= 8 fixed at compile time).  The subproblem's
// subgrid is staged in shared memory.  Per 32-point batch, lane t prepares point t's record
// (tab_prepare, no strength); the warp then walks the points in order: a lane keeps in
// registers the grid values of its cells of the current window (rows bl and bl + 4 at z
// offset e, all W columns), reloaded from the subgrid when the origin changes, and forms
// its partial sum kz * sum_b ky sum_a kx G from the record.  Two shuffles add the four row
// groups; the eight z lanes' sums go to the warp's partial buffer, and after the batch lane
// t adds point t's eight partials and writes the value in caller order.
// OUT: 0 complex values from the complex grid, 2 real values from the real grid.
template <typename T, int OUT, int W>
__device__ __forceinline__ void interp_tab_sub(int b, int off, const int *bin_count, const int *bin_start,
                                               const int *perm, const T *ux, const T *uy, const T *uz, const T *fine,
                                               const SubgridGeom &gm, T beta, T *out)
{
    static_assert(W >= 2 && W <= 8, "table interpolation needs 2 <= W <= 8");
    constexpr bool CPLX = OUT == 0;
    constexpr int EW = 8, BR = 4, RX = (W + BR - 1) / BR, REC = 24, NC = CPLX ? 2 : 1;
    using T2 = typename cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sg = reinterpret_cast<T *>(smem_raw);
    const int S = gm.S, P = gm.P, h = W / 2;
    const int plane = S * P, copy = S * plane;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const size_t sgb = ((size_t)NC * copy * sizeof(T) + 15) & ~(size_t)15;
    T *tab = reinterpret_cast<T *>(smem_raw + sgb) + warp * 32 * (REC + 8 * NC);
    T *part = tab + 32 * REC;  // [32 points][8 z lanes] (x NC)
    load_subgrid<T, CPLX>(fine, gm, b, sg);
    __syncthreads();

    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % EW, bl = lane / EW;
    T gr[RX][W], gi[RX][W];
    // real output in FP32: the window's column pairs as float2 and each row's dot product as
    // two partial sums (even / odd columns) updated with the packed FP32 FMA (fma.rn.f32x2);
    // an odd width's last column is added with a scalar FMA
    constexpr bool PK = sizeof(T) == 4 && !CPLX;
    constexpr int NP = W / 2;
    float2 gp[RX][NP > 0 ? NP : 1];
    int cur_key = -1;
    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    const T cs = (T)gm.cscale;
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const bool valid = tl < t1;
        const int pos = p0 + (valid ? tl : t0);
        const T px = ux[pos] * cs, py = uy[pos] * cs, pz = uz[pos] * cs;
        __syncwarp();  // the previous batch's records and partials have been read
        const int my_key = tab_prepare<T, W, false, 0>(px, py, pz, beta, T(1), T(0), tab + lane * REC);
        __syncwarp();
        const int nq = min(32, t1 - base);
        // runs of equal window origins (as in spread_tab_sub): one reload test per run
        const int prev_key = __shfl_up_sync(0xffffffffu, my_key, 1);
        unsigned starts = __ballot_sync(0xffffffffu, lane == 0 || my_key != prev_key);
        starts &= nq >= 32 ? 0xffffffffu : ((1u << nq) - 1u);
        int q = 0;
        while (q < nq) {
            const unsigned later = starts & ~((2u << q) - 1u);
            const int qe = later ? __ffs(later) - 1 : nq;
            const int key = __shfl_sync(0xffffffffu, my_key, q);  // warp-uniform
            if (key != cur_key) {
                cur_key = key;
                const int X0 = (key >> 12) - 16 + h, Y0 = ((key >> 6) & 63) - 16 + h, Z0 = (key & 63) - 16 + h;
                const int idx0 = (X0 * S + Y0 + bl) * P + Z0 + e;
#pragma unroll
                for (int r = 0; r < RX; ++r) {
                    const bool ok = e < W && bl + r * BR < W;
#pragma unroll
                    for (int a = 0; a < W; ++a) {
                        const int idx = idx0 + a * plane + r * BR * P;
                        gr[r][a] = ok ? sg[idx] : T(0);
                        if (CPLX) gi[r][a] = ok ? sg[copy + idx] : T(0);
                    }
                    if constexpr (PK) {
#pragma unroll
                        for (int k = 0; k < NP; ++k) gp[r][k] = make_float2(gr[r][2 * k], gr[r][2 * k + 1]);
                    }
                }
            }
#pragma unroll 2
            for (; q < qe; ++q) {
                const T *rq = tab + q * REC;
                T xv[8];
                load8(rq, xv);
                const T2 yv = reinterpret_cast<const T2 *>(rq + 8)[bl];
                const T zv = rq[16 + e];
                T ar0 = T(0), ai0 = T(0), ar1 = T(0), ai1 = T(0);
                if constexpr (PK) {
                    float2 s0 = make_float2(0.f, 0.f), s1 = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < NP; ++k) {
                        const float2 xk = make_float2(xv[2 * k], xv[2 * k + 1]);
                        s0 = __ffma2_rn(xk, gp[0][k], s0);
                        if (RX > 1) s1 = __ffma2_rn(xk, gp[RX - 1][k], s1);
                    }
                    if (W % 2) {
                        s0.x = fmaf(xv[W - 1], gr[0][W - 1], s0.x);
                        if (RX > 1) s1.x = fmaf(xv[W - 1], gr[RX - 1][W - 1], s1.x);
                    }
                    ar0 = s0.x + s0.y;
                    ar1 = s1.x + s1.y;
                } else {
#pragma unroll
                    for (int a = 0; a < W; ++a) {
                        ar0 += xv[a] * gr[0][a];
                        if (CPLX) ai0 += xv[a] * gi[0][a];
                        if (RX > 1) {
                            ar1 += xv[a] * gr[RX - 1][a];
                            if (CPLX) ai1 += xv[a] * gi[RX - 1][a];
                        }
                    }
                }
                T sr = (yv.x * ar0 + yv.y * ar1) * zv;
                T si = CPLX ? (yv.x * ai0 + yv.y * ai1) * zv : T(0);
                sr += __shfl_xor_sync(0xffffffffu, sr, 8);
                sr += __shfl_xor_sync(0xffffffffu, sr, 16);
                if (CPLX) {
                    si += __shfl_xor_sync(0xffffffffu, si, 8);
                    si += __shfl_xor_sync(0xffffffffu, si, 16);
                }
                if (bl == 0) {
                    if (CPLX) reinterpret_cast<T2 *>(part)[q * 8 + e] = T2{sr, si};
                    else part[q * 8 + e] = sr;
                }
            }
        }
        __syncwarp();
        if (valid) {
            const int64_t j = perm[pos];
            T v[8];
            if (CPLX) {
                T w2[8];
                load8(part + lane * 16, v);
                load8(part + lane * 16 + 8, w2);
                out[2 * j] = ((v[0] + v[2]) + (v[4] + v[6])) + ((w2[0] + w2[2]) + (w2[4] + w2[6]));
                out[2 * j + 1] = ((v[1] + v[3]) + (v[5] + v[7])) + ((w2[1] + w2[3]) + (w2[5] + w2[7]));
            } else {
                load8(part + lane * 8, v);
                out[j] = ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
            }
        }
    }
}

// One subproblem per CTA (sub_bin / sub_off list of one plan).
template <typename T, int OUT, int W>
__global__ void __launch_bounds__(256, 4) k_interp_tab(const int *sub_bin, const int *sub_off, const int *bin_count,
                                                    const int *bin_start, const int *perm, const T *ux,
                                                    const T *uy, const T *uz, const T *fine, SubgridGeom gm, T beta,
                                                    T *out)
{
    interp_tab_sub<T, OUT, W>(sub_bin[blockIdx.x], sub_off[blockIdx.x], bin_count, bin_start, perm, ux, uy, uz, fine,
                              gm, beta, out);
}

// Interpolation over the subproblems of all plans of a batch, one persistent launch.
template <typename T, int OUT, int W>
__global__ void __launch_bounds__(256, 4) k_interp_tab_batch(const WorkItem *work, int nwork, const InstDesc<T> *inst,
                                                          T beta, int *next)
{
    for (;;) {
        const int it = next_item(next);
        if (it >= nwork) return;
        const WorkItem wk = work[it];
        const InstDesc<T> d = inst[wk.inst];
        interp_tab_sub<T, OUT, W>(wk.bin, wk.off, d.bin_count, d.bin_start, d.perm, (const T *)d.ux,
                                  (const T *)d.uy, (const T *)d.uz, (const T *)d.in, d.gm, beta, (T *)d.out);
    }
}

// ------------------------------------------------------------------ interp (type 2)

// Register window of the lane (W > 0): grid values of its cells for the current origin.
template <typename T, bool CPLX, int W>
struct Window {
    using L = WarpLayout<W>;
    T re[L::RMAX][L::KMAX], im[L::RMAX][L::KMAX];

    __device__ __forceinline__ void load(const T *sg, int copy, int plane, int P, int base_idx, int bl, bool ez,
                                         int w)
    {
#pragma unroll
        for (int r = 0; r < L::RMAX; ++r) {
            const int bb = bl + r * L::BR;
            const bool ok = ez && bb < w;
#pragma unroll
            for (int a = 0; a < L::KMAX; ++a) {
                const int idx = base_idx + bb * P + a * plane;
                re[r][a] = ok ? sg[idx] : T(0);
                if (CPLX) im[r][a] = ok ? sg[copy + idx] : T(0);
            }
        }
    }
};

// this lane's partial of the interpolated value at a point (shared-memory path, W = 0 or
// any W): sum over its cells of kx ky kz G
template <typename T, bool CPLX, int W>
__device__ __forceinline__ void interp_partial_smem(const T *sg, int copy, int P, int plane, int w, int rounds,
                                                    bool two, int base_idx, T v0, T v1, int e, int bl,
                                                    const T (&kx)[WarpLayout<W>::KMAX], T kz, T &sr, T &si)
{
    using L = WarpLayout<W>;
    sr = T(0);
    si = T(0);
#pragma unroll
    for (int r = 0; r < L::RMAX; ++r) {
        if (W == 0 && r >= rounds) break;
        const int bb = bl + r * L::BR;
        const T ky = getk(v0, v1, w + (bb < w ? bb : 0), two);
        if (e >= w || bb >= w) continue;
        int idx = base_idx + bb * P;
        T ar = T(0), ai = T(0);
#pragma unroll
        for (int a = 0; a < L::KMAX; ++a) {
            if (W > 0 || a < w) {
                ar += kx[a] * sg[idx];
                if (CPLX) ai += kx[a] * sg[copy + idx];
            }
            idx += plane;
        }
        sr += ky * ar;
        si += ky * ai;
    }
    sr *= kz;
    si *= kz;
}

// the same from the register window
template <typename T, bool CPLX, int W>
__device__ __forceinline__ void interp_partial_regs(const Window<T, CPLX, W> &win, int w, bool two, T v0, T v1,
                                                    int bl, const T (&kx)[WarpLayout<W>::KMAX], T kz, T &sr, T &si)
{
    using L = WarpLayout<W>;
    sr = T(0);
    si = T(0);
#pragma unroll
    for (int r = 0; r < L::RMAX; ++r) {
        const int bb = bl + r * L::BR;
        const T ky = getk(v0, v1, w + (bb < w ? bb : 0), two);
        T ar = T(0), ai = T(0);
#pragma unroll
        for (int a = 0; a < L::KMAX; ++a) {
            ar += kx[a] * win.re[r][a];
            if (CPLX) ai += kx[a] * win.im[r][a];
        }
        sr += ky * ar;
        si += ky * ai;
    }
    sr *= kz;
    si *= kz;
}

// OUT: 0 complex values from the complex grid, 2 real values from the real grid.
template <typename T, int OUT, int W>
__global__ void __launch_bounds__(256) k_interp(const int *sub_bin, const int *sub_off, const int *bin_count,
                                                const int *bin_start, const int *perm, const T *ux, const T *uy,
                                                const T *uz, const T *fine, SubgridGeom gm, T beta, T *out)
{
    using L = WarpLayout<W>;
    constexpr bool CPLX = OUT == 0;
    extern __shared__ unsigned char smem_raw[];
    T *sg = reinterpret_cast<T *>(smem_raw);
    const int S = gm.S, P = gm.P, w = W > 0 ? W : gm.w, h = w / 2;
    const int rounds = (w + L::BR - 1) / L::BR;
    const bool two = 3 * w > 32;
    const int plane = S * P, copy = S * plane;
    const int b = sub_bin[blockIdx.x];
    load_subgrid<T, CPLX>(fine, gm, b, sg);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int off = sub_off[blockIdx.x];
    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % L::EW, bl = lane / L::EW;
    const bool ez = e < w;
    Window<T, CPLX, W> win;
    int cur_key = -1;
    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    const T cs = (T)gm.cscale;
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const bool valid = tl < t1;
        const int pos = p0 + (valid ? tl : t0);
        const T mx = ux[pos] * cs, my = uy[pos] * cs, mz = uz[pos] * cs;
        T rr = T(0), ri = T(0);  // lane q keeps point q's result
        const int nq = min(32, t1 - base);
        for (int q = 0; q < nq; ++q) {
            const T px = __shfl_sync(0xffffffffu, mx, q);
            const T py = __shfl_sync(0xffffffffu, my, q);
            const T pz = __shfl_sync(0xffffffffu, mz, q);
            int lx, ly, lz;
            point_origin(px, py, pz, w, lx, ly, lz);
            T v0, v1;
            point_values(px, py, pz, lx, ly, lz, w, beta, lane, v0, v1);
            T kx[L::KMAX];
#pragma unroll
            for (int a = 0; a < L::KMAX; ++a) kx[a] = (W > 0 || a < w) ? getk(v0, v1, a, two) : T(0);
            const T kz = getk(v0, v1, 2 * w + (ez ? e : 0), two);
            const int base_idx = ((lx + h) * S + (ly + h)) * P + lz + h + e;
            T sr, si;
            if (W > 0) {
                const int key = origin_key(lx, ly, lz);
                if (key != cur_key) {
                    win.load(sg, copy, plane, P, base_idx, bl, ez, w);
                    cur_key = key;
                }
                interp_partial_regs<T, CPLX, W>(win, w, two, v0, v1, bl, kx, kz, sr, si);
            } else {
                interp_partial_smem<T, CPLX, W>(sg, copy, P, plane, w, rounds, two, base_idx, v0, v1, e, bl, kx, kz,
                                                sr, si);
            }
            for (int o = 16; o > 0; o >>= 1) {
                sr += __shfl_xor_sync(0xffffffffu, sr, o);
                if (CPLX) si += __shfl_xor_sync(0xffffffffu, si, o);
            }
            if (lane == q) {
                rr = sr;
                ri = si;
            }
        }
        if (valid) {
            const int64_t j = perm[pos];
            if (CPLX) {
                out[2 * j] = rr;
                out[2 * j + 1] = ri;
            } else {
                out[j] = rr;
            }
        }
    }
}

// ------------------------------------------------------------------ fused pair

// Interpolate from G1 (complex, shared by the CTA) and spread the value straight back into
// G2 (complex, one copy, shared atomics) with the same kernel values; flush G2.
template <typename T, int W>
__global__ void __launch_bounds__(256) k_pair(const int *sub_bin, const int *sub_off, const int *bin_count,
                                              const int *bin_start, const T *ux, const T *uy, const T *uz,
                                              const T *g1, SubgridGeom gm, T beta, T *g2)
{
    using L = WarpLayout<W>;
    extern __shared__ unsigned char smem_raw[];
    const int S = gm.S, P = gm.P, w = W > 0 ? W : gm.w, h = w / 2, n = gm.n;
    const int rounds = (w + L::BR - 1) / L::BR;
    const bool two = 3 * w > 32;
    const int plane = S * P, copy = S * plane;
    T *sa = reinterpret_cast<T *>(smem_raw);
    T *sb = sa + 2 * copy;
    const int b = sub_bin[blockIdx.x];
    for (int i = threadIdx.x; i < 2 * copy; i += blockDim.x) sb[i] = T(0);
    load_subgrid<T, true>(g1, gm, b, sa);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int off = sub_off[blockIdx.x];
    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % L::EW, bl = lane / L::EW;
    const bool ez = e < w;
    Window<T, true, W> win, acc;
    int cur_key = -1, cur_base = 0;
    auto flush = [&]() {
        if constexpr (W > 0) {
            if (cur_key < 0) return;
#pragma unroll
            for (int r = 0; r < L::RMAX; ++r) {
                const int bb = bl + r * L::BR;
                const bool ok = ez && bb < w;
#pragma unroll
                for (int a = 0; a < L::KMAX; ++a) {
                    if (ok) {
                        const int idx = cur_base + bb * P + a * plane;
                        atomicAdd(&sb[idx], acc.re[r][a]);
                        atomicAdd(&sb[copy + idx], acc.im[r][a]);
                    }
                    acc.re[r][a] = T(0);
                    acc.im[r][a] = T(0);
                }
            }
        }
    };
#pragma unroll
    for (int r = 0; r < L::RMAX; ++r)
#pragma unroll
        for (int a = 0; a < L::KMAX; ++a) {
            acc.re[r][a] = T(0);
            acc.im[r][a] = T(0);
        }
    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    const T cs = (T)gm.cscale;
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const int pos = p0 + (tl < t1 ? tl : t0);
        const T mx = ux[pos] * cs, my = uy[pos] * cs, mz = uz[pos] * cs;
        const int nq = min(32, t1 - base);
        for (int q = 0; q < nq; ++q) {
            const T px = __shfl_sync(0xffffffffu, mx, q);
            const T py = __shfl_sync(0xffffffffu, my, q);
            const T pz = __shfl_sync(0xffffffffu, mz, q);
            int lx, ly, lz;
            point_origin(px, py, pz, w, lx, ly, lz);
            T v0, v1;
            point_values(px, py, pz, lx, ly, lz, w, beta, lane, v0, v1);
            T kx[L::KMAX];
#pragma unroll
            for (int a = 0; a < L::KMAX; ++a) kx[a] = (W > 0 || a < w) ? getk(v0, v1, a, two) : T(0);
            const T kz = getk(v0, v1, 2 * w + (ez ? e : 0), two);
            const int base_idx = ((lx + h) * S + (ly + h)) * P + lz + h + e;
            T sr, si;
            if (W > 0) {
                const int key = origin_key(lx, ly, lz);
                if (key != cur_key) {
                    flush();
                    win.load(sa, copy, plane, P, base_idx, bl, ez, w);
                    cur_key = key;
                    cur_base = base_idx;
                }
                interp_partial_regs<T, true, W>(win, w, two, v0, v1, bl, kx, kz, sr, si);
            } else {
                interp_partial_smem<T, true, W>(sa, copy, P, plane, w, rounds, two, base_idx, v0, v1, e, bl, kx, kz,
                                                sr, si);
            }
            for (int o = 16; o > 0; o >>= 1) {
                sr += __shfl_xor_sync(0xffffffffu, sr, o);
                si += __shfl_xor_sync(0xffffffffu, si, o);
            }
            // every lane holds the interpolated value; spread it back with the same weights
#pragma unroll
            for (int r = 0; r < L::RMAX; ++r) {
                if (W == 0 && r >= rounds) break;
                const int bb = bl + r * L::BR;
                const T ky = getk(v0, v1, w + (bb < w ? bb : 0), two);
                const T kyz = ky * kz;
                const T wr = kyz * sr, wi = kyz * si;
                if (W > 0) {
#pragma unroll
                    for (int a = 0; a < L::KMAX; ++a) {
                        acc.re[r][a] += kx[a] * wr;
                        acc.im[r][a] += kx[a] * wi;
                    }
                } else {
                    if (!ez || bb >= w) continue;
                    int idx = base_idx + bb * P;
#pragma unroll
                    for (int a = 0; a < L::KMAX; ++a) {
                        if (a < w) {
                            atomicAdd(&sb[idx], kx[a] * wr);
                            atomicAdd(&sb[copy + idx], kx[a] * wi);
                        }
                        idx += plane;
                    }
                }
            }
        }
    }
    flush();
    __syncthreads();
    const int bx = b / (gm.nb * gm.nb), by = (b / gm.nb) % gm.nb, bz = b % gm.nb;
    const int ox = bx * gm.bs - h, oy = by * gm.bs - h, oz = bz * gm.bs - h;
    for (int i = threadIdx.x; i < S * S * S; i += blockDim.x) {
        const int a = i / (S * S), rem = i - a * S * S, bb = rem / S, ee = rem - bb * S;
        const int li = (a * S + bb) * P + ee;
        const T vr = sb[li], vi = sb[copy + li];
        if (vr == T(0) && vi == T(0)) continue;
        const int64_t g = ((int64_t)wrapi(ox + a, n) * n + wrapi(oy + bb, n)) * n + wrapi(oz + ee, n);
        atomicAdd(&g2[2 * g], vr);
        atomicAdd(&g2[2 * g + 1], vi);
    }
}

// ------------------------------------------------------------------ table-driven fused pair

// Per-warp table of k_pair_tab: 32 records of PAIR_REC values (x 8, y pairs 8, then z 8
// and later (z c) pairs 16; padded so that the owner lanes' 16-byte record accesses fall in
// distinct banks) and 32 rows of PAIR_PART values (8 complex partial sums, padded likewise).
constexpr int PAIR_REC = 36, PAIR_PART = 20;

// Shared-memory bytes of k_pair_tab: the two complex subgrids (G1 staged, G2 accumulated),
// 16-byte aligned, then the per-warp tables.
template <typename T>
__host__ __device__ inline size_t pair_tab_smem(size_t subgrid_bytes, int warps)
{
    return ((4 * subgrid_bytes + 15) & ~(size_t)15) + warps * 32 * (PAIR_REC + PAIR_PART) * sizeof(T);
}

// Table-driven fused type-2 then type-1 pair on one subproblem (kernel width W <= 8): the
// complex subgrid G1 is staged in shared memory and a second one, G2, accumulates.  Per batch
// of 32 points, lane t prepares point t's record once (window origin and its 3W kernel
// values, tab_prepare).  Pass A walks the batch run by run like k_interp_tab: a lane keeps
// its cells of G1's current window in registers and forms its partials of each point's
// value; lane t then adds point t's eight partials, c_t = sum_k G1_k phi_k(x_t), and rewrites
// its record's z part as (z c_t) pairs.  Pass B walks the batch again like k_spread_tab with
// complex strengths c_t, adding into a register window of G2 that goes to shared memory
// (atomics) when the window origin changes.  G2 is added to the fine grid once.  Kernel
// values are evaluated once per point for both directions, and no N-sized intermediate is
// written.
template <typename T, int W>
__device__ __forceinline__ void pair_tab_sub(int b, int off, const int *bin_count, const int *bin_start, const T *ux,
                                             const T *uy, const T *uz, const T *g1, const SubgridGeom &gm, T beta,
                                             T *g2)
{
    static_assert(W >= 2 && W <= 8, "table pair needs a window of at most 8 columns");
    constexpr int EW = 8, BR = 4, RX = (W + BR - 1) / BR, REC = PAIR_REC;
    using T2 = typename cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int S = gm.S, P = gm.P, h = W / 2, n = gm.n;
    const int plane = S * P, copy = S * plane;
    T *sa = reinterpret_cast<T *>(smem_raw);
    T *sb = sa + 2 * copy;
    const size_t sgb = ((size_t)4 * copy * sizeof(T) + 15) & ~(size_t)15;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    T *tab = reinterpret_cast<T *>(smem_raw + sgb) + warp * 32 * (REC + PAIR_PART);
    T *part = tab + 32 * REC;  // per point a row of PAIR_PART: 8 z lanes' (re, im) partials
    for (int i = threadIdx.x; i < 2 * copy; i += blockDim.x) sb[i] = T(0);
    load_subgrid<T, true>(g1, gm, b, sa);
    __syncthreads();

    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % EW, bl = lane / EW;

    // FP32: both walks pair the window's columns (2k, 2k + 1) and update them with the packed
    // FP32 FMA (fma.rn.f32x2), pass A as even / odd partial sums, pass B as the accumulators
    // themselves; an odd width's last column stays scalar
    constexpr bool PK = sizeof(T) == 4;
    constexpr int NP = W / 2;
    // pass A state: G1 window (rows bl, bl + 4 at z offset e, all W columns)
    T gr[RX][W], gi[RX][W];
    float2 grp[RX][NP > 0 ? NP : 1], gip[RX][NP > 0 ? NP : 1];
    int key_a = -1;
    // pass B state: G2 accumulation window
    T acc[RX][W], aci[RX][W];
    float2 acp[RX][NP > 0 ? NP : 1], aip[RX][NP > 0 ? NP : 1];
#pragma unroll
    for (int r = 0; r < RX; ++r) {
#pragma unroll
        for (int a = 0; a < W; ++a) acc[r][a] = aci[r][a] = T(0);
#pragma unroll
        for (int k = 0; k < NP; ++k) acp[r][k] = aip[r][k] = make_float2(0.f, 0.f);
    }
    int key_b = -1, X0 = 0, Y0 = 0, Z0 = 0;
    auto flush = [&]() {
        if (key_b < 0) return;
        const int zz = Z0 + e;
#pragma unroll
        for (int r = 0; r < RX; ++r) {
            const int yy = Y0 + bl + r * BR;
            const bool row_ok = e < W && bl + r * BR < W;
#pragma unroll
            for (int a = 0; a < W; ++a) {
                const bool pk = PK && a < 2 * NP;
                const T vr = pk ? T((a & 1) ? acp[r][a >> 1].y : acp[r][a >> 1].x) : acc[r][a];
                const T vi = pk ? T((a & 1) ? aip[r][a >> 1].y : aip[r][a >> 1].x) : aci[r][a];
                if (row_ok) {
                    const int idx = ((X0 + a) * S + yy) * P + zz;
                    if (vr != T(0)) atomicAdd(&sb[idx], vr);
                    if (vi != T(0)) atomicAdd(&sb[copy + idx], vi);
                }
                acc[r][a] = aci[r][a] = T(0);
            }
#pragma unroll
            for (int k = 0; k < NP; ++k) acp[r][k] = aip[r][k] = make_float2(0.f, 0.f);
        }
    };

    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    const T cs = (T)gm.cscale;
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const bool valid = tl < t1;
        const int pos = p0 + (valid ? tl : t0);
        const T px = ux[pos] * cs, py = uy[pos] * cs, pz = uz[pos] * cs;
        __syncwarp();  // the previous batch's records and partials have been read
        T *rec = tab + lane * REC;
        const int my_key = tab_prepare<T, W, false, 0>(px, py, pz, beta, T(1), T(0), rec);
        __syncwarp();
        const int nq = min(32, t1 - base);
        const int prev_key = __shfl_up_sync(0xffffffffu, my_key, 1);
        unsigned starts = __ballot_sync(0xffffffffu, lane == 0 || my_key != prev_key);
        starts &= nq >= 32 ? 0xffffffffu : ((1u << nq) - 1u);

        // ---- pass A: interpolate every point of the batch from G1
        for (int q = 0; q < nq;) {
            const unsigned later = starts & ~((2u << q) - 1u);
            const int qe = later ? __ffs(later) - 1 : nq;
            const int key = __shfl_sync(0xffffffffu, my_key, q);  // warp-uniform
            if (key != key_a) {
                key_a = key;
                const int XA = (key >> 12) - 16 + h, YA = ((key >> 6) & 63) - 16 + h, ZA = (key & 63) - 16 + h;
                const int idx0 = (XA * S + YA + bl) * P + ZA + e;
#pragma unroll
                for (int r = 0; r < RX; ++r) {
                    const bool ok = e < W && bl + r * BR < W;
#pragma unroll
                    for (int a = 0; a < W; ++a) {
                        const int idx = idx0 + a * plane + r * BR * P;
                        gr[r][a] = ok ? sa[idx] : T(0);
                        gi[r][a] = ok ? sa[copy + idx] : T(0);
                    }
                    if constexpr (PK) {
#pragma unroll
                        for (int k = 0; k < NP; ++k) {
                            grp[r][k] = make_float2(gr[r][2 * k], gr[r][2 * k + 1]);
                            gip[r][k] = make_float2(gi[r][2 * k], gi[r][2 * k + 1]);
                        }
                    }
                }
            }
            for (; q < qe; ++q) {
                const T *rq = tab + q * REC;
                T xv[8];
                load8(rq, xv);
                const T2 yv = reinterpret_cast<const T2 *>(rq + 8)[bl];
                const T zv = rq[16 + e];
                T ar0 = T(0), ai0 = T(0), ar1 = T(0), ai1 = T(0);
                if constexpr (PK) {
                    float2 r0 = make_float2(0.f, 0.f), i0 = r0, r1 = r0, i1 = r0;
#pragma unroll
                    for (int k = 0; k < NP; ++k) {
                        const float2 xk = make_float2(xv[2 * k], xv[2 * k + 1]);
                        r0 = __ffma2_rn(xk, grp[0][k], r0);
                        i0 = __ffma2_rn(xk, gip[0][k], i0);
                        if (RX > 1) {
                            r1 = __ffma2_rn(xk, grp[RX - 1][k], r1);
                            i1 = __ffma2_rn(xk, gip[RX - 1][k], i1);
                        }
                    }
                    if (W % 2) {
                        r0.x = fmaf(xv[W - 1], gr[0][W - 1], r0.x);
                        i0.x = fmaf(xv[W - 1], gi[0][W - 1], i0.x);
                        if (RX > 1) {
                            r1.x = fmaf(xv[W - 1], gr[RX - 1][W - 1], r1.x);
                            i1.x = fmaf(xv[W - 1], gi[RX - 1][W - 1], i1.x);
                        }
                    }
                    ar0 = r0.x + r0.y;
                    ai0 = i0.x + i0.y;
                    ar1 = r1.x + r1.y;
                    ai1 = i1.x + i1.y;
                } else {
#pragma unroll
                    for (int a = 0; a < W; ++a) {
                        ar0 += xv[a] * gr[0][a];
                        ai0 += xv[a] * gi[0][a];
                        if (RX > 1) {
                            ar1 += xv[a] * gr[RX - 1][a];
                            ai1 += xv[a] * gi[RX - 1][a];
                        }
                    }
                }
                T sr = (yv.x * ar0 + yv.y * ar1) * zv;
                T si = (yv.x * ai0 + yv.y * ai1) * zv;
                sr += __shfl_xor_sync(0xffffffffu, sr, 8);
                sr += __shfl_xor_sync(0xffffffffu, sr, 16);
                si += __shfl_xor_sync(0xffffffffu, si, 8);
                si += __shfl_xor_sync(0xffffffffu, si, 16);
                if (bl == 0) reinterpret_cast<T2 *>(part + q * PAIR_PART)[e] = T2{sr, si};
            }
        }
        __syncwarp();
        // ---- lane t: point t's value, folded into its record as (z c) pairs
        {
            T v[8], w2[8];
            load8(part + lane * PAIR_PART, v);
            load8(part + lane * PAIR_PART + 8, w2);
            T cr = ((v[0] + v[2]) + (v[4] + v[6])) + ((w2[0] + w2[2]) + (w2[4] + w2[6]));
            T ci = ((v[1] + v[3]) + (v[5] + v[7])) + ((w2[1] + w2[3]) + (w2[5] + w2[7]));
            if (!valid) cr = ci = T(0);
            T z[8], o[8];
            load8(rec + 16, z);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                o[2 * k] = z[k] * cr;
                o[2 * k + 1] = z[k] * ci;
            }
            T o2[8];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                o2[2 * k] = z[k + 4] * cr;
                o2[2 * k + 1] = z[k + 4] * ci;
            }
            store8(rec + 16, o);
            store8(rec + 24, o2);
        }
        __syncwarp();
        // ---- pass B: spread every point's value back into G2 with the same kernel values
        for (int q = 0; q < nq;) {
            const unsigned later = starts & ~((2u << q) - 1u);
            const int qe = later ? __ffs(later) - 1 : nq;
            const int key = __shfl_sync(0xffffffffu, my_key, q);  // warp-uniform
            if (key != key_b) {
                flush();
                key_b = key;
                X0 = (key >> 12) - 16 + h;
                Y0 = ((key >> 6) & 63) - 16 + h;
                Z0 = (key & 63) - 16 + h;
            }
            for (; q < qe; ++q) {
                const T *rq = tab + q * REC;
                T xv[8];
                load8(rq, xv);
                const T2 yv = reinterpret_cast<const T2 *>(rq + 8)[bl];
                const T2 zv = reinterpret_cast<const T2 *>(rq + 16)[e];
                const T wr0 = yv.x * zv.x, wi0 = yv.x * zv.y, wr1 = yv.y * zv.x, wi1 = yv.y * zv.y;
                if constexpr (PK) {
                    const float2 wr0p = make_float2(wr0, wr0), wi0p = make_float2(wi0, wi0),
                                 wr1p = make_float2(wr1, wr1), wi1p = make_float2(wi1, wi1);
#pragma unroll
                    for (int k = 0; k < NP; ++k) {
                        const float2 xk = make_float2(xv[2 * k], xv[2 * k + 1]);
                        acp[0][k] = __ffma2_rn(xk, wr0p, acp[0][k]);
                        aip[0][k] = __ffma2_rn(xk, wi0p, aip[0][k]);
                        if (RX > 1) {
                            acp[RX - 1][k] = __ffma2_rn(xk, wr1p, acp[RX - 1][k]);
                            aip[RX - 1][k] = __ffma2_rn(xk, wi1p, aip[RX - 1][k]);
                        }
                    }
                    if (W % 2) {
                        acc[0][W - 1] += xv[W - 1] * wr0;
                        aci[0][W - 1] += xv[W - 1] * wi0;
                        if (RX > 1) {
                            acc[RX - 1][W - 1] += xv[W - 1] * wr1;
                            aci[RX - 1][W - 1] += xv[W - 1] * wi1;
                        }
                    }
                } else {
#pragma unroll
                    for (int a = 0; a < W; ++a) {
                        acc[0][a] += xv[a] * wr0;
                        aci[0][a] += xv[a] * wi0;
                        if (RX > 1) {
                            acc[RX - 1][a] += xv[a] * wr1;
                            aci[RX - 1][a] += xv[a] * wi1;
                        }
                    }
                }
            }
        }
    }
    flush();
    __syncthreads();
    const int bx = b / (gm.nb * gm.nb), by = (b / gm.nb) % gm.nb, bz = b % gm.nb;
    const int ox = bx * gm.bs - h, oy = by * gm.bs - h, oz = bz * gm.bs - h;
    for (int i = threadIdx.x; i < S * S * S; i += blockDim.x) {
        const int a = i / (S * S), rem = i - a * S * S, bb = rem / S, ee = rem - bb * S;
        const int li = (a * S + bb) * P + ee;
        const T vr = sb[li], vi = sb[copy + li];
        if (vr == T(0) && vi == T(0)) continue;
        const int64_t g = ((int64_t)wrapi(ox + a, n) * n + wrapi(oy + bb, n)) * n + wrapi(oz + ee, n);
        atomicAdd(&g2[2 * g], vr);
        atomicAdd(&g2[2 * g + 1], vi);
    }
}

template <typename T, int W>
__global__ void __launch_bounds__(256) k_pair_tab(const int *sub_bin, const int *sub_off, const int *bin_count,
                                                  const int *bin_start, const T *ux, const T *uy, const T *uz,
                                                  const T *g1, SubgridGeom gm, T beta, T *g2)
{
    pair_tab_sub<T, W>(sub_bin[blockIdx.x], sub_off[blockIdx.x], bin_count, bin_start, ux, uy, uz, g1, gm, beta, g2);
}
