// Warp-cooperative spreading / interpolation kernels (included by nufft.cu).
//
// One CTA per subproblem (a bin of the fine grid, or a <= maxsub slice of a dense bin),
// one POINT per warp at a time.  The w^3 window of the point is split over the lanes:
// lane = (bl, e) with e = lane % EW the z offset and bl = lane / EW the first y offset, the
// lane visiting y offsets b = bl + r * (32 / EW), r = 0, 1, ...  The shared subgrid keeps
// rows of pitch P with P mod 32 in {8, 24} (EW = 8) or 16 (EW = 16), so the 32 addresses of
// every shared-memory instruction fall in 32 distinct banks: no bank conflicts and no two
// lanes of an instruction on one address.  Complex grids are stored planar (re | im).
// The 3w kernel values of a point are evaluated once, one per lane, and gathered with
// warp shuffles.
//
// Spreading accumulates either into per-warp private copies of the subgrid (no atomics,
// summed at the flush; used when they fit) or into one copy with shared atomics; the
// flush adds the subgrid to the fine grid once per subproblem (global atomics only there,
// where neighbouring bins' halos overlap).

// gathers kernel value q (0 <= q < 3w) held as value q % 32 of register v0 (q < 32) or v1
template <typename T>
__device__ __forceinline__ T getk(T v0, T v1, int q)
{
    T a = __shfl_sync(0xffffffffu, v0, q & 31);
    T b = __shfl_sync(0xffffffffu, v1, q & 31);
    return q < 32 ? a : b;
}

// Window starts (relative to the bin origin) and this lane's share of the 3w kernel values.
template <typename T>
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

struct SubgridGeom {
    int n, rs, bs, nb, w, S, P, maxsub;
};

__device__ __forceinline__ int wrapi(int g, int n) { return g + (g < 0 ? n : (g >= n ? -n : 0)); }

// ------------------------------------------------------------------ spread (type 1)

// CPLX: complex strengths (interleaved in c), else real (c == nullptr: all ones).
// PRIV: per-warp private subgrid copies (no atomics), else one copy with shared atomics.
// Fine grid: complex n^3 interleaved (CPLX) or real with row stride rs (in-place R2C layout).
template <typename T, bool CPLX, int EW, bool PRIV>
__global__ void __launch_bounds__(256) k_spread(const int *sub_bin, const int *sub_off, const int *bin_count,
                                                const int *bin_start, const int *perm, const T *ux, const T *uy,
                                                const T *uz, const T *c, SubgridGeom gm, T beta, T *fine)
{
    constexpr int BR = 32 / EW;
    extern __shared__ unsigned char smem_raw[];
    T *sg = reinterpret_cast<T *>(smem_raw);
    const int S = gm.S, P = gm.P, w = gm.w, h = w / 2;
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
    const int e = lane % EW, bl = lane / EW;
    const int rounds = (w + BR - 1) / BR;
    T *mine = sg + (PRIV ? warp * nch * copy : 0);
    for (int t = warp; t < cnt; t += nwarps) {
        const int pos = p0 + t;
        const T px = ux[pos], py = uy[pos], pz = uz[pos];
        T vr = T(1), vi = T(0);
        if (c) {
            const int64_t j = perm[pos];
            if (CPLX) {
                vr = c[2 * j];
                vi = c[2 * j + 1];
            } else {
                vr = c[j];
            }
        }
        int lx, ly, lz;
        T v0, v1;
        point_window<T>(px, py, pz, w, beta, lane, lx, ly, lz, v0, v1);
        T kx[MAXW];
#pragma unroll
        for (int a = 0; a < MAXW; ++a) kx[a] = a < w ? getk(v0, v1, a) : T(0);
        const T kz = getk(v0, v1, 2 * w + (e < w ? e : 0));
        const bool ez = e < w;
        for (int r = 0; r < rounds; ++r) {
            const int bb = bl + r * BR;
            const T ky = getk(v0, v1, w + (bb < w ? bb : 0));
            if (!ez || bb >= w) continue;
            const T kyz = ky * kz;
            const T wr = kyz * vr, wi = kyz * vi;
            int idx = ((lx + h) * S + (ly + h + bb)) * P + lz + h + e;
#pragma unroll
            for (int a = 0; a < MAXW; ++a) {
                if (a < w) {
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

// OUT: 0 complex values, 2 real grid (real values).  Output in caller order via perm.
template <typename T, int OUT, int EW>
__global__ void __launch_bounds__(256) k_interp(const int *sub_bin, const int *sub_off, const int *bin_count,
                                                const int *bin_start, const int *perm, const T *ux, const T *uy,
                                                const T *uz, const T *fine, SubgridGeom gm, T beta, T *out)
{
    constexpr int BR = 32 / EW;
    constexpr bool CPLX = OUT == 0;
    extern __shared__ unsigned char smem_raw[];
    T *sg = reinterpret_cast<T *>(smem_raw);
    const int S = gm.S, P = gm.P, w = gm.w, h = w / 2, n = gm.n;
    const int plane = S * P, copy = S * plane;
    const int b = sub_bin[blockIdx.x];
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
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int off = sub_off[blockIdx.x];
    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % EW, bl = lane / EW;
    const int rounds = (w + BR - 1) / BR;
    for (int t = warp; t < cnt; t += nwarps) {
        const int pos = p0 + t;
        int lx, ly, lz;
        T v0, v1;
        point_window<T>(ux[pos], uy[pos], uz[pos], w, beta, lane, lx, ly, lz, v0, v1);
        T kx[MAXW];
#pragma unroll
        for (int a = 0; a < MAXW; ++a) kx[a] = a < w ? getk(v0, v1, a) : T(0);
        const T kz = getk(v0, v1, 2 * w + (e < w ? e : 0));
        T sr = T(0), si = T(0);
        for (int r = 0; r < rounds; ++r) {
            const int bb = bl + r * BR;
            const T ky = getk(v0, v1, w + (bb < w ? bb : 0));
            if (e >= w || bb >= w) continue;
            int idx = ((lx + h) * S + (ly + h + bb)) * P + lz + h + e;
            T ar = T(0), ai = T(0);
#pragma unroll
            for (int a = 0; a < MAXW; ++a) {
                if (a < w) {
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
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            if (CPLX) si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0) {
            const int64_t j = perm[pos];
            if (CPLX) {
                out[2 * j] = sr;
                out[2 * j + 1] = si;
            } else {
                out[j] = sr;
            }
        }
    }
}

// ------------------------------------------------------------------ fused pair

// Interpolate from G1 (complex, shared by the CTA) and spread the value straight back
// into G2 (complex, one copy, shared atomics) with the same kernel values; flush G2.
template <typename T, int EW>
__global__ void __launch_bounds__(256) k_pair(const int *sub_bin, const int *sub_off, const int *bin_count,
                                              const int *bin_start, const T *ux, const T *uy, const T *uz,
                                              const T *g1, SubgridGeom gm, T beta, T *g2)
{
    constexpr int BR = 32 / EW;
    extern __shared__ unsigned char smem_raw[];
    const int S = gm.S, P = gm.P, w = gm.w, h = w / 2, n = gm.n;
    const int plane = S * P, copy = S * plane;
    T *sa = reinterpret_cast<T *>(smem_raw);
    T *sb = sa + 2 * copy;
    const int b = sub_bin[blockIdx.x];
    const int bx = b / (gm.nb * gm.nb), by = (b / gm.nb) % gm.nb, bz = b % gm.nb;
    const int ox = bx * gm.bs - h, oy = by * gm.bs - h, oz = bz * gm.bs - h;
    for (int i = threadIdx.x; i < 2 * copy; i += blockDim.x) sb[i] = T(0);
    for (int i = threadIdx.x; i < S * S * S; i += blockDim.x) {
        const int a = i / (S * S), rem = i - a * S * S, bb = rem / S, ee = rem - bb * S;
        const int li = (a * S + bb) * P + ee;
        const int64_t g = ((int64_t)wrapi(ox + a, n) * n + wrapi(oy + bb, n)) * n + wrapi(oz + ee, n);
        sa[li] = g1[2 * g];
        sa[copy + li] = g1[2 * g + 1];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int off = sub_off[blockIdx.x];
    const int cnt = min(gm.maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int e = lane % EW, bl = lane / EW;
    const int rounds = (w + BR - 1) / BR;
    for (int t = warp; t < cnt; t += nwarps) {
        const int pos = p0 + t;
        int lx, ly, lz;
        T v0, v1;
        point_window<T>(ux[pos], uy[pos], uz[pos], w, beta, lane, lx, ly, lz, v0, v1);
        T kx[MAXW];
#pragma unroll
        for (int a = 0; a < MAXW; ++a) kx[a] = a < w ? getk(v0, v1, a) : T(0);
        const T kz = getk(v0, v1, 2 * w + (e < w ? e : 0));
        T sr = T(0), si = T(0);
        for (int r = 0; r < rounds; ++r) {
            const int bb = bl + r * BR;
            const T ky = getk(v0, v1, w + (bb < w ? bb : 0));
            if (e >= w || bb >= w) continue;
            int idx = ((lx + h) * S + (ly + h + bb)) * P + lz + h + e;
            T ar = T(0), ai = T(0);
#pragma unroll
            for (int a = 0; a < MAXW; ++a) {
                if (a < w) {
                    ar += kx[a] * sa[idx];
                    ai += kx[a] * sa[copy + idx];
                }
                idx += plane;
            }
            sr += ky * ar;
            si += ky * ai;
        }
        sr *= kz;
        si *= kz;
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        // every lane now holds the interpolated value c_j; spread it back
        for (int r = 0; r < rounds; ++r) {
            const int bb = bl + r * BR;
            const T ky = getk(v0, v1, w + (bb < w ? bb : 0));
            if (e >= w || bb >= w) continue;
            const T kyz = ky * kz;
            const T wr = kyz * sr, wi = kyz * si;
            int idx = ((lx + h) * S + (ly + h + bb)) * P + lz + h + e;
#pragma unroll
            for (int a = 0; a < MAXW; ++a) {
                if (a < w) {
                    atomicAdd(&sb[idx], kx[a] * wr);
                    atomicAdd(&sb[copy + idx], kx[a] * wi);
                }
                idx += plane;
            }
        }
    }
    __syncthreads();
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
