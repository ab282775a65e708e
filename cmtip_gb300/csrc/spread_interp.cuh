// Warp-cooperative spreading / interpolation kernels (included by nufft_spread.cu and
// nufft_interp.cu).
//
// One CTA per subproblem (a bin of the fine grid, or a <= maxsub slice of a dense bin).
// Each warp walks a contiguous run of the subproblem's points, 32 at a time: the lanes load
// 32 points' coordinates (and strengths) with coalesced loads, then the warp treats the
// points one after another, broadcasting each with a shuffle.  The w^3 window of a point is
// split over the lanes: lane = (bl, e), e = lane % EW the z offset, bl = lane / EW the first
// y offset, the lane visiting y offsets b = bl + r * (32 / EW) for r < ROUNDS and every x
// offset a < w.  Shared subgrid rows have a pitch P with P mod 32 in {8, 24} (EW = 8) or 16
// (EW = 16), so the 32 addresses of a shared-memory instruction sit in 32 distinct banks.
// Complex grids are planar (re | im).  The 3w kernel values of a point are evaluated once,
// one per lane, and gathered with shuffles.  W > 0 fixes the kernel width at compile time
// (all loops unrolled, constant divisions); W = 0 reads it at run time (w <= 16).
//
// Spreading accumulates into one shared copy with shared atomics, or (real strengths,
// SPREAD_PRIV) into per-warp private copies with plain read-modify-write; the flush adds
// the subgrid to the fine grid once per subproblem (global atomics only there, where
// neighbouring bins' halos overlap).

template <int W>
struct WarpLayout {
    static constexpr int EW = (W > 0 && W <= 8) ? 8 : 16;  // z lanes
    static constexpr int BR = 32 / EW;                      // y offsets per round
    static constexpr int KMAX = W > 0 ? W : MAXW;           // unroll bound of the x loop
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

// Window starts (relative to the bin origin) and this lane's share of the 3w kernel values.
template <typename T, int W>
__device__ __forceinline__ void point_window(T px, T py, T pz, int w, T beta, int lane, int &lx, int &ly, int &lz,
                                             T &v0, T &v1)
{
    const T hw = T(0.5) * T(w);
    lx = (int)ceil(px - hw);
    ly = (int)ceil(py - hw);
    lz = (int)ceil(pz - hw);
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

// ------------------------------------------------------------------ spread (type 1)

// CPLX: complex strengths (interleaved in c), else real (c == nullptr: all ones).
// PRIV: per-warp private subgrid copies (no atomics), else one copy with shared atomics.
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
    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const bool valid = tl < t1;
        const int pos = p0 + (valid ? tl : t0);
        const T cs = (T)gm.cscale;
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
            T v0, v1;
            point_window<T, W>(px, py, pz, w, beta, lane, lx, ly, lz, v0, v1);
            T kx[L::KMAX];
#pragma unroll
            for (int a = 0; a < L::KMAX; ++a) kx[a] = (W > 0 || a < w) ? getk(v0, v1, a, two) : T(0);
            const T kz = getk(v0, v1, 2 * w + (ez ? e : 0), two);
            const int base_idx = ((lx + h) * S + (ly + h)) * P + lz + h + e;
#pragma unroll
            for (int r = 0; r < (W > 0 ? (W + L::BR - 1) / L::BR : 8); ++r) {
                if (W == 0 && r >= rounds) break;
                const int bb = bl + r * L::BR;
                const T ky = getk(v0, v1, w + (bb < w ? bb : 0), two);
                if (!ez || bb >= w) continue;
                const T kyz = ky * kz;
                const T wr = kyz * vr, wi = kyz * vi;
                int idx = base_idx + bb * P;
#pragma unroll
                for (int a = 0; a < L::KMAX; ++a) {
                    if (W > 0 || a < w) {
                        if (PRIV) {
                            mine[idx] += kx[a] * wr;
                            if (CPLX) mine[copy + idx] += kx[a] * wi;
                        } else {
                            atomicAdd(&mine[idx], kx[a] * wr);
                            if (CPLX) atomicAdd(&mine[copy + idx], kx[a] * wi);
                        }
                    }
                    idx += plane;
                }
            }
        }
    }
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

// ------------------------------------------------------------------ interp (type 2)

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

// this lane's partial of the interpolated value at a point
template <typename T, bool CPLX, int W>
__device__ __forceinline__ void interp_partial(const T *sg, int copy, int S, int P, int plane, int w, int h, int rounds,
                                               bool two, int lx, int ly, int lz, T v0, T v1, int e, int bl, T &sr,
                                               T &si, T (&kx)[WarpLayout<W>::KMAX], T &kz)
{
    using L = WarpLayout<W>;
    const bool ez = e < w;
#pragma unroll
    for (int a = 0; a < L::KMAX; ++a) kx[a] = (W > 0 || a < w) ? getk(v0, v1, a, two) : T(0);
    kz = getk(v0, v1, 2 * w + (ez ? e : 0), two);
    const int base_idx = ((lx + h) * S + (ly + h)) * P + lz + h + e;
    sr = T(0);
    si = T(0);
#pragma unroll
    for (int r = 0; r < (W > 0 ? (W + L::BR - 1) / L::BR : 8); ++r) {
        if (W == 0 && r >= rounds) break;
        const int bb = bl + r * L::BR;
        const T ky = getk(v0, v1, w + (bb < w ? bb : 0), two);
        if (!ez || bb >= w) continue;
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
    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const bool valid = tl < t1;
        const int pos = p0 + (valid ? tl : t0);
        const T cs = (T)gm.cscale;
        const T mx = ux[pos] * cs, my = uy[pos] * cs, mz = uz[pos] * cs;
        T rr = T(0), ri = T(0);  // lane q keeps point q's result
        const int nq = min(32, t1 - base);
        for (int q = 0; q < nq; ++q) {
            const T px = __shfl_sync(0xffffffffu, mx, q);
            const T py = __shfl_sync(0xffffffffu, my, q);
            const T pz = __shfl_sync(0xffffffffu, mz, q);
            int lx, ly, lz;
            T v0, v1, kz, sr, si;
            T kx[L::KMAX];
            point_window<T, W>(px, py, pz, w, beta, lane, lx, ly, lz, v0, v1);
            interp_partial<T, CPLX, W>(sg, copy, S, P, plane, w, h, rounds, two, lx, ly, lz, v0, v1, e, bl, sr, si,
                                       kx, kz);
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
    int t0, t1;
    warp_run(cnt, warp, nwarps, t0, t1);
    for (int base = t0; base < t1; base += 32) {
        const int tl = base + lane;
        const int pos = p0 + (tl < t1 ? tl : t0);
        const T cs = (T)gm.cscale;
        const T mx = ux[pos] * cs, my = uy[pos] * cs, mz = uz[pos] * cs;
        const int nq = min(32, t1 - base);
        for (int q = 0; q < nq; ++q) {
            const T px = __shfl_sync(0xffffffffu, mx, q);
            const T py = __shfl_sync(0xffffffffu, my, q);
            const T pz = __shfl_sync(0xffffffffu, mz, q);
            int lx, ly, lz;
            T v0, v1, kz, sr, si;
            T kx[L::KMAX];
            point_window<T, W>(px, py, pz, w, beta, lane, lx, ly, lz, v0, v1);
            interp_partial<T, true, W>(sa, copy, S, P, plane, w, h, rounds, two, lx, ly, lz, v0, v1, e, bl, sr, si,
                                       kx, kz);
            for (int o = 16; o > 0; o >>= 1) {
                sr += __shfl_xor_sync(0xffffffffu, sr, o);
                si += __shfl_xor_sync(0xffffffffu, si, o);
            }
            // every lane holds the interpolated value; spread it back with the same weights
            const int base_idx = ((lx + h) * S + (ly + h)) * P + lz + h + e;
#pragma unroll
            for (int r = 0; r < (W > 0 ? (W + L::BR - 1) / L::BR : 8); ++r) {
                if (W == 0 && r >= rounds) break;
                const int bb = bl + r * L::BR;
                const T ky = getk(v0, v1, w + (bb < w ? bb : 0), two);
                if (!ez || bb >= w) continue;
                const T kyz = ky * kz;
                const T wr = kyz * sr, wi = kyz * si;
                int idx = base_idx + bb * P;
#pragma unroll
                for (int a = 0; a < L::KMAX; ++a) {
                    if (W > 0 || a < w) {
                        atomicAdd(&sb[idx], kx[a] * wr);
                        atomicAdd(&sb[copy + idx], kx[a] * wi);
                    }
                    idx += plane;
                }
            }
        }
    }
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
