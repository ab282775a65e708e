// 3D type-1 / type-2 NUFFT for sm_103a with an exponential-of-semicircle kernel.
//
// Points are counting-sorted into cubic bins of the upsampled ("fine") grid once per
// set_pts; the plan keeps, in bin order, each point's coordinates relative to its
// bin origin (fine-grid units) and the permutation back to caller order.  Execution:
//   type 1: spread   -> one CTA per subproblem (a bin or a <= maxsub slice of it)
//                       accumulates into a shared-memory subgrid, then flushes it
//                       once to the fine grid; cuFFT; deconvolve + crop (fused).
//   type 2: deconvolve + zero-pad (fused, one pass over the fine grid); cuFFT;
//                       interpolate from a shared-memory copy of the bin's subgrid.
//   pair  : type 2 then type 1 on the same points with the interpolated value
//           spread straight back from registers (no N-sized intermediate).
// Real-valued strengths (type 1) and real-part outputs (type 2) use R2C / C2R
// transforms on a real fine grid, halving spreading/interpolation work.
//
// The reference calls cufinufft/finufft for these transforms
// (cmtip/nufft/forward.py:40,77-79; cmtip/nufft/adjoint.py:33,73-75).
#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "cmt_common.cuh"
#include "nufft_plan.cuh"
#include "df.cuh"

namespace cmt {

static constexpr double kPi = 3.14159265358979323846;

static thread_local char g_err[2048] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

// ------------------------------------------------------------------ host helpers

// Gauss-Legendre nodes/weights on [-1, 1] by Newton iteration on P_n.
static void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w)
{
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
        double z = cos(kPi * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// psi_hat(xi) = int_{-w/2}^{w/2} phi(t) cos(xi t) dt
static double kernel_ft(double xi, int w, double beta, const std::vector<double> &gx,
                        const std::vector<double> &gw)
{
    double s = 0.0, half = 0.5 * w;
    for (size_t i = 0; i < gx.size(); ++i) {
        double t = 0.5 * half * (gx[i] + 1.0);  // [0, w/2]
        double z = 2.0 * t / w;
        double a = 1.0 - z * z;
        double phi = a > 0 ? exp(beta * (sqrt(a) - 1.0)) : 0.0;
        s += 0.5 * half * gw[i] * phi * cos(xi * t);
    }
    return 2.0 * s;
}

static int next_nice(int n)
{
    int m = std::max(n, 2);
    for (;; ++m) {
        if (m & 1) continue;
        int r = m;
        for (int p : {2, 3, 5, 7})
            while (r % p == 0) r /= p;
        if (r == 1) return m;
    }
}

// ------------------------------------------------------------------ plan

}  // namespace cmt


namespace cmt {

// ------------------------------------------------------------------ device helpers

// Split u (fine-grid units, any real) into the integer cell and the fraction.
template <typename T>
__device__ __forceinline__ void cell_and_frac(T x, T s_hi, T s_lo, int n, unsigned n_magic, int &cell, T &frac)
{
    // u = x * (s_hi + s_lo) carried as p + lo with p = fl(x s_hi) and lo its exact error
    T p = x * s_hi;
    T lo = fma(x, s_hi, -p);
    lo = fma(x, s_lo, lo);
    T fp = floor(p);
    T f = (p - fp) + lo;
    // p - fp is in [0, 1] (1 where it rounds up, for p just below an integer) and |lo| is
    // about an ulp of p, so f lies in (-1, 2) and t = floor(f) is -1, 0 or 1: f - t is
    // f + 1 / f / f - 1, one fix-up either way (f is never -0: p - fp is +0 or positive)
    const T t = floor(f);
    f -= t;
    int c = (int)fp + (int)t;
    // c mod n: k_bin_count calls this only for |x| < 3 pi, where c lies in [-1.5 n - 2,
    // 1.5 n + 1], inside [-2n, 3n) (n >= 2w >= 4); u = c + 2n is in [0, 5n), below 2^32 / n
    // when n_magic is set, so u / n is the multiply-high quotient (div_magic)
    if (n_magic) {
        const unsigned u = (unsigned)(c + 2 * n);
        c = (int)(u - __umulhi(u, n_magic) * (unsigned)n);
    } else {
        c += n & -(int)(c < 0);
        c += n & -(int)(c < 0);
        c -= n & -(int)(c >= n);
        c -= n & -(int)(c >= n);
    }
    cell = c;
    frac = f;
}

// floor(x / d) for 0 <= x < 2^32 / d as the high word of x * m, m = ceil(2^32 / d)
// (Granlund & Montgomery 1994: with m d = 2^32 + e, 0 <= e < d, the error x e / (d 2^32) is
// below 1/d, less than the distance from x / d to the next integer).
__device__ __forceinline__ unsigned div_magic(unsigned x, unsigned m) { return __umulhi(x, m); }

inline unsigned magic32(unsigned d) { return (unsigned)((0x100000000ULL + d - 1) / d); }  // d >= 2
inline unsigned long long magic64(unsigned long long d)                                  // d >= 2
{
    return ~0ULL / d + 1ULL;  // ceil(2^64 / d)
}

// Coordinates of point j.  MODE 0: arrays of the plan's precision; MODE 1: rotation.
struct QuatSrc {
    const double *inv_rot;
    const double *ppr;
    int64_t n_pix;
    double rext;
    // FP32 plans: inv_rot and ppr split into double-float pairs and padded for 16-byte loads
    // (k_split_quat): 10 pairs per image (inv(R) row-major, one pad), 4 per pixel (x, y, z, pad)
    const float2 *rot_df;
    const float2 *ppr_df;
    float2 scale_df;       // pi / rext as a double-float pair
    unsigned long long npix_magic;  // ceil(2^64 / n_pix) (n_pix >= 2), else 0
};

// (image, pixel) of point j < 2^31: j / n_pix as the high word of j * ceil(2^64 / n_pix),
// exact for all j < 2^64 / n_pix
__device__ __forceinline__ void img_pix(int64_t j, const QuatSrc &q, unsigned &img, unsigned &pix)
{
    img = q.npix_magic ? (unsigned)__umul64hi((unsigned long long)j, q.npix_magic) : (unsigned)j;
    pix = (unsigned)j - img * (unsigned)q.n_pix;
}

__device__ __forceinline__ float2 split_df(double v)
{
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}

// The rotations (n_img x 9, row-major inv(R)) and q-vectors (3 x n_pix, component-major) as
// double-float pairs in QuatSrc's padded layout; one thread per output pair
__global__ void k_split_quat(const double *rot, int64_t n_img, const double *ppr, int64_t n_pix, float2 *rot_out,
                             float2 *ppr_out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 10 * n_img) {
        const int64_t img = i / 10;
        const int k = (int)(i - 10 * img);
        rot_out[i] = k < 9 ? split_df(rot[9 * img + k]) : make_float2(0.f, 0.f);
    } else if (i < 10 * n_img + 4 * n_pix) {
        const int64_t t = i - 10 * n_img, pix = t / 4;
        const int c = (int)(t - 4 * pix);
        ppr_out[t] = c < 3 ? split_df(ppr[c * n_pix + pix]) : make_float2(0.f, 0.f);
    }
}

template <typename T>
__device__ __forceinline__ void point_coords(int mode, int64_t j, const T *x, const T *y, const T *z,
                                             QuatSrc q, T &px, T &py, T &pz, bool &bad)
{
    if (mode == 0) {
        px = x[j];
        py = y[j];
        pz = z[j];
    } else if (sizeof(T) == 4) {
        // the chain below at FP32 throughput: float32(H) of H = inv(R) . p by a compensated
        // dot product, then float32(H) * (pi / extent), with the rotations, q-vectors and
        // pi / extent pre-split into (hi, lo) float pairs; both results are rounded once from
        // values within ~2^-46 of the exact ones, so they equal the float64 chain's roundings
        // except where that chain's value lies within ~2^-46 of a float32 rounding boundary
        // N < 2^31 (set_pts_impl), so 32-bit index arithmetic
        unsigned img, pix;
        img_pix(j, q, img, pix);
        const float4 *R4 = reinterpret_cast<const float4 *>(q.rot_df) + 5 * img;
        const float4 *P4 = reinterpret_cast<const float4 *>(q.ppr_df) + 2 * pix;
        const float4 r0 = R4[0], r1 = R4[1], r2 = R4[2], r3 = R4[3], r4 = R4[4], pa = P4[0], pb = P4[1];
        const float2 R[9] = {make_float2(r0.x, r0.y), make_float2(r0.z, r0.w), make_float2(r1.x, r1.y),
                             make_float2(r1.z, r1.w), make_float2(r2.x, r2.y), make_float2(r2.z, r2.w),
                             make_float2(r3.x, r3.y), make_float2(r3.z, r3.w), make_float2(r4.x, r4.y)};
        const float2 a0 = make_float2(pa.x, pa.y), a1 = make_float2(pa.z, pa.w), a2 = make_float2(pb.x, pb.y);
        float o[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            o[r] = df_scale_to_float(df_dot3_to_float(R[3 * r], a0, R[3 * r + 1], a1, R[3 * r + 2], a2), q.scale_df);
        px = (T)o[0];
        py = (T)o[1];
        pz = (T)o[2];
    } else {
        // float32(inv(R) . p) / reciprocal_extent * pi, as in align.py:52-57 and
        // autocorrelation.py:27,210 + setup_linops :133-135 (products not fused).
        // N < 2^31 (set_pts_impl), so 32-bit index arithmetic
        unsigned img, pix;
        img_pix(j, q, img, pix);
        const double *R = q.inv_rot + 9 * img;
        double p0 = q.ppr[pix], p1 = q.ppr[q.n_pix + pix], p2 = q.ppr[2 * q.n_pix + pix];
        double h = __dadd_rn(__dadd_rn(__dmul_rn(R[0], p0), __dmul_rn(R[1], p1)), __dmul_rn(R[2], p2));
        double k = __dadd_rn(__dadd_rn(__dmul_rn(R[3], p0), __dmul_rn(R[4], p1)), __dmul_rn(R[5], p2));
        double l = __dadd_rn(__dadd_rn(__dmul_rn(R[6], p0), __dmul_rn(R[7], p1)), __dmul_rn(R[8], p2));
        const double pi = 3.141592653589793;
        double xh = __dmul_rn(__ddiv_rn((double)__double2float_rn(h), q.rext), pi);
        double xk = __dmul_rn(__ddiv_rn((double)__double2float_rn(k), q.rext), pi);
        double xl = __dmul_rn(__ddiv_rn((double)__double2float_rn(l), q.rext), pi);
        px = (T)xh;
        py = (T)xk;
        pz = (T)xl;
    }
    const T lim = T(3.0 * 3.141592653589793);
    bad = !(fabs(px) < lim && fabs(py) < lim && fabs(pz) < lim);
}

template <typename T>
__device__ __forceinline__ int bin_of(T px, T py, T pz, T s_hi, T s_lo, int n, unsigned n_magic, int bs,
                                      unsigned bs_magic, int nb, T &rx, T &ry, T &rz)
{
    int cx, cy, cz;
    T fx, fy, fz;
    cell_and_frac(px, s_hi, s_lo, n, n_magic, cx, fx);
    cell_and_frac(py, s_hi, s_lo, n, n_magic, cy, fy);
    cell_and_frac(pz, s_hi, s_lo, n, n_magic, cz, fz);
    int bx, by, bz;
    if (bs_magic) {
        bx = (int)div_magic((unsigned)cx, bs_magic);
        by = (int)div_magic((unsigned)cy, bs_magic);
        bz = (int)div_magic((unsigned)cz, bs_magic);
    } else {
        bx = cx / bs, by = cy / bs, bz = cz / bs;
    }
    rx = T(cx - bx * bs) + fx;
    ry = T(cy - by * bs) + fy;
    rz = T(cz - bz * bs) + fz;
    return (bx * nb + by) * nb + bz;
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Sort key of a point: its bin, then (within the bin) the origin of its kernel window on
// this grid, then the origin's offset on a grid twice as fine (0/1 per dimension).  Points
// sharing a key share their whole w^3 window on this grid and on a derived plan's twice
// finer grid, so the kernels can keep a window in registers across runs of such points.
// Keys per bin: kb = 1 (fine_sort 0: bin only), (bs+1)^(fine_sort - 1) (2..4: x / x, y /
// x, y, z window origin) or (bs+1)^3 * 8 (1: origin and refinement).
template <typename T, typename K = int64_t>
__device__ __forceinline__ K point_key(int b, T rx, T ry, T rz, int w, int bs, int fine_sort)
{
    if (!fine_sort) return b;
    const T hw = T(0.5) * T(w);
    const int h = w / 2, O = bs + 1;
    int lx = (int)ceil(rx - hw), ly = (int)ceil(ry - hw), lz = (int)ceil(rz - hw);
    int ox = min(max(lx + h, 0), bs), oy = min(max(ly + h, 0), bs), oz = min(max(lz + h, 0), bs);
    if (fine_sort == 2) return ((K)b * O + ox);                     // origin x
    if (fine_sort == 3) return ((K)b * O + ox) * O + oy;            // origin x, y
    if (fine_sort == 4) return (((K)b * O + ox) * O + oy) * O + oz; // origin
    // On the twice finer grid the origin is 2l + base + d with d in {0, 1} (even w) or
    // {0, 1, 2} (odd w); the refinement splits d = 2 off, so within one refined group the fine
    // origins differ by at most one per dimension.
    const int base = (w - 2 - (w & 1)) / 2;
    int dx = (int)ceil(T(2) * rx - hw) - 2 * lx - base;
    int dy = (int)ceil(T(2) * ry - hw) - 2 * ly - base;
    int dz = (int)ceil(T(2) * rz - hw) - 2 * lz - base;
    dx = min(max(dx, 0), 2) >> 1;
    dy = min(max(dy, 0), 2) >> 1;
    dz = min(max(dz, 0), 2) >> 1;
    return ((((K)b * O + ox) * O + oy) * O + oz) * 8 + dx * 4 + dy * 2 + dz;
}

struct SortGeom {
    int n, bs, nb, w, fine_sort;
    unsigned bs_magic;  // ceil(2^32 / bs) for cells below 2^32 / bs, else 0 (plain division)
    unsigned n_magic;   // ceil(2^32 / n) when 5 n^2 < 2^32 (cell wrap by multiply-high), else 0
};

// A point between the two counting passes: its sort key (-1: out of range) and its
// bin-relative fine-grid coordinates, written by pass 1 in caller order so that pass 2
// does not evaluate the coordinate chain again.
template <typename T> struct PtRec;
template <> struct __align__(16) PtRec<float> {
    int key;
    float x, y, z;
};
template <> struct __align__(16) PtRec<double> {
    long long key;
    double x, y, z;
};

// A point in key order after pass 2: coordinates and caller index in one 16-byte (FP32) or
// 32-byte (FP64) record, so the scatter writes one stream per key instead of four.
template <typename T> struct SortedRec;
template <> struct __align__(16) SortedRec<float> {
    float x, y, z;
    int perm;
};
template <> struct __align__(16) SortedRec<double> {
    double x, y, z;
    int perm, pad;
};

// Pass 1: coordinates, bin and key of every point (range check), stored as records; per-key
// counts with warp-aggregated atomics.
template <typename T>
__global__ void k_bin_count(int mode, int64_t N, const T *x, const T *y, const T *z, QuatSrc q, T s_hi, T s_lo,
                            SortGeom sg, int *count, PtRec<T> *rec, int *flag)
{
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t base = (int64_t)blockIdx.x * blockDim.x;
    // FP32 plans keep 32-bit keys (their records hold an int key; set_pts_impl bounds the key
    // count below 2^27 when origins are keyed): 32-bit key arithmetic and warp match
    using K = typename std::conditional<sizeof(T) == 4, int, long long>::type;
    for (; base < N; base += stride) {
        int64_t j = base + threadIdx.x;
        K key = -1;
        if (j < N) {
            T px, py, pz, rx = 0, ry = 0, rz = 0;
            bool bad;
            point_coords<T>(mode, j, x, y, z, q, px, py, pz, bad);
            if (bad) {
                atomicOr(flag, 1);
            } else {
                int b = bin_of<T>(px, py, pz, s_hi, s_lo, sg.n, sg.n_magic, sg.bs, sg.bs_magic, sg.nb, rx, ry, rz);
                key = point_key<T, K>(b, rx, ry, rz, sg.w, sg.bs, sg.fine_sort);
            }
            PtRec<T> r;
            r.key = key;
            r.x = rx;
            r.y = ry;
            r.z = rz;
            rec[j] = r;
        }
        unsigned peers = __match_any_sync(0xffffffffu, key);
        int leader = __ffs(peers) - 1;
        if (key >= 0 && (int)(threadIdx.x & 31) == leader) atomicAdd(&count[key], __popc(peers));
    }
}

// Pass 2: scatter permutation and coordinates into key order.  next[key] starts at the
// key's first position; start[key + 1] bounds it.
template <typename T>
__global__ void k_bin_scatter(int64_t N, const PtRec<T> *rec, const int *start, int *next, SortedRec<T> *out,
                              int *flag)
{
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t base = (int64_t)blockIdx.x * blockDim.x;
    for (; base < N; base += stride) {
        int64_t j = base + threadIdx.x;
        long long key = -1;
        PtRec<T> r{};
        if (j < N) {
            r = rec[j];
            key = r.key;
        }
        unsigned peers = __match_any_sync(0xffffffffu, key);
        int lane = threadIdx.x & 31;
        int leader = __ffs(peers) - 1;
        int off = 0;
        if (key >= 0 && lane == leader) off = atomicAdd(&next[key], __popc(peers));
        off = __shfl_sync(peers, off, leader);
        if (key >= 0) {
            int pos = off + __popc(peers & lanemask_lt());
            if (pos >= start[key + 1]) {  // counts and keys disagree: never write out of the key's range
                atomicOr(flag, 2);
                continue;
            }
            SortedRec<T> o{};
            o.x = r.x;
            o.y = r.y;
            o.z = r.z;
            o.perm = (int)j;
            out[pos] = o;
        }
    }
}

// 16-byte asynchronous global -> shared copies (cp.async, completion by commit groups)
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Pass 2 for FP32 plans, tile by tile: a CTA groups a tile of SCAT_TILE records (caller
// order) by key in a shared-memory hash table, reserves each key's share of its sorted range
// with one atomic per key and tile, and writes the tile's records of a key to consecutive
// positions.  Caller order is image by image along detector rows, so a tile holds an
// image's points of a window origin (about a dozen) together: each key receives them as
// one contiguous run instead of one run per warp, which L2 merges into full sectors
// before they reach DRAM.  Same output as k_bin_scatter up to the order within a key.
constexpr int SCAT_THREADS = 256, SCAT_PER = 8, SCAT_TILE = SCAT_THREADS * SCAT_PER, SCAT_SLOTS = 2 * SCAT_TILE;
static_assert(SCAT_SLOTS <= 4096 && SCAT_TILE <= 4096, "slot and rank are packed in 12 bits each");

__global__ void __launch_bounds__(SCAT_THREADS, 4) k_bin_scatter_tiled(int64_t N, const PtRec<float> *rec,
                                                                   const int *start, int *next,
                                                                   SortedRec<float> *out, int *flag)
{
    __shared__ int hkey[SCAT_SLOTS];   // key of a slot, -1 empty
    __shared__ int hval[SCAT_SLOTS];   // the key's count in the tile, then its first position
    __shared__ short used[SCAT_TILE];  // slots taken in this tile
    __shared__ int n_used;
    const int lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < SCAT_SLOTS; i += blockDim.x) {
        hkey[i] = -1;
        hval[i] = 0;
    }
    if (threadIdx.x == 0) n_used = 0;
    __syncthreads();
    for (int64_t t0 = (int64_t)blockIdx.x * SCAT_TILE; t0 < N; t0 += (int64_t)gridDim.x * SCAT_TILE) {
        float4 r[SCAT_PER];
        int key[SCAT_PER], sr[SCAT_PER];  // sr: slot | rank << 12 (both < 4096), -1 without a key
#pragma unroll
        for (int k = 0; k < SCAT_PER; ++k) {
            const int64_t j = t0 + k * SCAT_THREADS + threadIdx.x;
            key[k] = -1;
            if (j < N) {
                r[k] = *reinterpret_cast<const float4 *>(rec + j);
                key[k] = __float_as_int(r[k].x);
            }
        }
        // group: the leader of each warp-level group of equal keys finds or takes the key's
        // slot (linear probing; a tile has at most SCAT_TILE keys in 2 x SCAT_TILE slots, so
        // a free slot is always found) and takes the group's ranks
#pragma unroll
        for (int k = 0; k < SCAT_PER; ++k) {
            const unsigned peers = __match_any_sync(0xffffffffu, key[k]);
            const int leader = __ffs(peers) - 1;
            int sl = 0, base = 0;
            if (key[k] >= 0 && lane == leader) {
                sl = (int)(((unsigned)key[k] * 2654435761u) >> 20) & (SCAT_SLOTS - 1);
                for (int probe = 0; probe < SCAT_SLOTS; ++probe) {
                    const int prev = atomicCAS(&hkey[sl], -1, key[k]);
                    if (prev == -1) {
                        used[atomicAdd(&n_used, 1)] = (short)sl;
                        break;
                    }
                    if (prev == key[k]) break;
                    sl = (sl + 1) & (SCAT_SLOTS - 1);
                }
                base = atomicAdd(&hval[sl], __popc(peers));
            }
            sl = __shfl_sync(0xffffffffu, sl, leader);
            base = __shfl_sync(0xffffffffu, base, leader) + __popc(peers & lanemask_lt());
            sr[k] = key[k] >= 0 ? sl | base << 12 : -1;
        }
        __syncthreads();
        // reserve each key's run: one global atomic per key of the tile
        const int nu = n_used;
        for (int u = threadIdx.x; u < nu; u += blockDim.x) {
            const int sl = used[u], k = hkey[sl], c = hval[sl];
            const int first = atomicAdd(&next[k], c);
            if (first + c > start[k + 1]) {  // counts and keys disagree: never write out of the key's range
                atomicOr(flag, 2);
                hval[sl] = -1;
            } else {
                hval[sl] = first;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SCAT_PER; ++k) {
            if (sr[k] < 0) continue;
            const int first = hval[sr[k] & (SCAT_SLOTS - 1)];
            if (first < 0) continue;
            SortedRec<float> o;
            o.x = r[k].y;
            o.y = r[k].z;
            o.z = r[k].w;
            o.perm = (int)(t0 + k * SCAT_THREADS + threadIdx.x);
            out[first + (sr[k] >> 12)] = o;
        }
        __syncthreads();
        for (int u = threadIdx.x; u < nu; u += blockDim.x) {
            const int sl = used[u];
            hkey[sl] = -1;
            hval[sl] = 0;
        }
        if (threadIdx.x == 0) n_used = 0;
        __syncthreads();
    }
}

// Records -> the plan's coordinate and permutation arrays without reordering (plans whose
// subproblem sort does not fit in shared memory).
template <typename T>
__global__ void k_rec_to_arrays(int64_t N, const SortedRec<T> *in, int *perm, T *ux, T *uy, T *uz)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const SortedRec<T> r = in[i];
        perm[i] = r.perm;
        ux[i] = r.x;
        uy[i] = r.y;
        uz[i] = r.z;
    }
}

// ---- exclusive scan of n ints (n < 2^31 total), three kernels: tile scan, scan of the
// tile sums (one CTA), tile offsets
constexpr int SCAN_THREADS = 256, SCAN_PER = 8, SCAN_TILE = SCAN_THREADS * SCAN_PER;

__device__ __forceinline__ int block_exclusive_scan(int v, int *sh, int &total)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    int prefix = (wid > 0 ? sh[wid - 1] : 0) + x - v;
    total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return prefix;
}

__global__ void k_scan_tiles(const int *in, int *out, int64_t n, int *tile_sums)
{
    __shared__ int sh[32];
    int64_t t0 = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER;
    int v[SCAN_PER];
    int s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_PER; ++i) {
        v[i] = t0 + i < n ? in[t0 + i] : 0;
        s += v[i];
    }
    int total;
    int run = block_exclusive_scan(s, sh, total);
#pragma unroll
    for (int i = 0; i < SCAN_PER; ++i) {
        if (t0 + i < n) out[t0 + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_single(int *a, int n)
{
    __shared__ int sh[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = i < n ? a[i] : 0;
        int total;
        int pre = block_exclusive_scan(v, sh, total);
        if (i < n) a[i] = carry + pre;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

__global__ void k_add_tile_offsets(int *out, int64_t n, const int *tile_off)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_off[i / SCAN_TILE];
}

// Within-subproblem sort by window origin (one CTA per subproblem), out of place: reads the
// subproblem's records as the global passes left them and writes them, counting-sorted by
// the window origin on this grid and its offset on a twice finer grid (point_key's
// refinement), to the same positions of the plan's coordinate and permutation arrays.  The global
// passes order by bin and by x, y origin; runs of points sharing a window on this grid or on
// a derived plan's grid become contiguous for the spreading / interpolation kernels.
// smem: nsk counters + maxsub 16-bit keys.  Keys repeat along the input, so the atomics are
// warp-aggregated (__match_any_sync).
template <typename T>
__global__ void k_subsort(const int *sub_bin, const int *sub_off, const int *bin_count, const int *bin_start, int w,
                          int bs, int maxsub, int nsk, const SortedRec<T> *in, int *perm_o, T *ux_o, T *uy_o,
                          T *uz_o)
{
    extern __shared__ unsigned char smem_raw[];
    int *cnt_s = reinterpret_cast<int *>(smem_raw);
    unsigned short *skey = reinterpret_cast<unsigned short *>(cnt_s + nsk);
    const int b = sub_bin[blockIdx.x];
    const int off = sub_off[blockIdx.x];
    const int cnt = min(maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    for (int i = threadIdx.x; i < nsk; i += blockDim.x) cnt_s[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int cnt_up = (cnt + 31) & ~31;
    for (int i = threadIdx.x; i < cnt_up; i += blockDim.x) {
        int key = -1;
        if (i < cnt) {
            const SortedRec<T> r = in[p0 + i];
            key = (int)point_key<T>(0, r.x, r.y, r.z, w, bs, 1);  // < nsk: bin 0, clamped origin
            skey[i] = (unsigned short)key;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&cnt_s[key], __popc(peers));
    }
    __syncthreads();
    // exclusive scan of the nsk counters: per-thread contiguous ranges + block scan
    __shared__ int sh[32];
    const int per = (nsk + blockDim.x - 1) / blockDim.x;
    const int lo = min((int)threadIdx.x * per, nsk), hi = min(lo + per, nsk);
    int s = 0;
    for (int i = lo; i < hi; ++i) s += cnt_s[i];
    int total;
    int run = block_exclusive_scan(s, sh, total);
    for (int i = lo; i < hi; ++i) {
        int c = cnt_s[i];
        cnt_s[i] = run;
        run += c;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < cnt_up; i += blockDim.x) {
        const int key = i < cnt ? (int)skey[i] : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        int base = 0;
        if (key >= 0 && lane == leader) base = atomicAdd(&cnt_s[key], __popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (key >= 0) {
            const SortedRec<T> r = in[p0 + i];
            const int dst = p0 + base + __popc(peers & lanemask_lt());
            perm_o[dst] = r.perm;
            ux_o[dst] = r.x;
            uy_o[dst] = r.y;
            uz_o[dst] = r.z;
        }
    }
}

// k_subsort for FP32 plans whose global passes ordered every bin by its window origin, whole
// (fine_sort 4) or its x, y part (fine_sort 3): the CTA walks its subproblem in chunks of
// SUBSORT_PER records per thread, held in registers, so each record is read from memory
// once (k_subsort reads it twice, once for the counts and once for the scatter), the next
// chunk arriving in shared memory while the current one is sorted.  The input
// is in origin order, so a chunk's keys span only the origins between its first and last
// record: that range of counters is cleared and scanned per chunk.  Sorting chunk by chunk
// keeps the global order; the origin classes of the key a chunk boundary cuts (its
// refinement classes, or with x, y keys its z origins) come out as two runs each (the
// earlier chunk's part first), which the kernels treat as two runs of one window.  The
// sorted chunk is assembled in shared memory and then written to
// the four output arrays in order, so every warp store is one contiguous 128-byte line
// (scattered 4-byte stores straight to the arrays are bound by L2 sector writes).
constexpr int SUBSORT_PER = 8, SUBSORT_THREADS = 256, SUBSORT_CHUNK = SUBSORT_PER * SUBSORT_THREADS;

__global__ void __launch_bounds__(SUBSORT_THREADS, 3)
    k_subsort_chunked(const int *sub_bin, const int *sub_off, const int *bin_count, const int *bin_start, int w,
                      int bs, int maxsub, int nsk, const SortedRec<float> *in, int *perm_o, float *ux_o,
                      float *uy_o, float *uz_o)
{
    // two chunk buffers: the next chunk's records arrive by cp.async while the current one is
    // sorted; a chunk's buffer then receives its sorted records for the copy-out
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *buf = reinterpret_cast<float4 *>(smem_raw);                       // 2 x SUBSORT_CHUNK records
    int *cnt_s = reinterpret_cast<int *>(smem_raw + 2 * SUBSORT_CHUNK * 16);  // nsk counters, indexed key - lo
    __shared__ int sh[32];
    __shared__ int range[2];
    const int b = sub_bin[blockIdx.x];
    const int off = sub_off[blockIdx.x];
    const int cnt = min(maxsub, bin_count[b] - off);
    const int p0 = bin_start[b] + off;
    const int lane = threadIdx.x & 31;
    const int chunk = SUBSORT_CHUNK;  // blockDim.x == SUBSORT_THREADS
    auto prefetch = [&](int c0, float4 *dst) {
        const int n = min(chunk, cnt - c0);
        const SortedRec<float> *src = in + p0 + c0;
#pragma unroll
        for (int k = 0; k < SUBSORT_PER; ++k) {
            const int i = k * SUBSORT_THREADS + threadIdx.x;
            if (i < n) cp_async16(dst + i, src + i);
        }
        cp_async_commit();
    };
    if (cnt > 0) prefetch(0, buf);
    int cur = 0;
    for (int c0 = 0; c0 < cnt; c0 += chunk, cur ^= 1) {
        const int n = min(chunk, cnt - c0);
        float4 *stage = buf + cur * SUBSORT_CHUNK;
        // the other buffer held the previous chunk, whose copy-out ended with a barrier
        if (c0 + chunk < cnt) {
            prefetch(c0 + chunk, buf + (cur ^ 1) * SUBSORT_CHUNK);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // every thread's copies of this chunk have landed
        float4 r[SUBSORT_PER];
        int key[SUBSORT_PER];
        int kmin = 0x7fffffff, kmax = -1;
#pragma unroll
        for (int k = 0; k < SUBSORT_PER; ++k) {
            const int i = k * SUBSORT_THREADS + threadIdx.x;
            key[k] = -1;
            if (i < n) {
                r[k] = stage[i];
                key[k] = (int)point_key<float>(0, r[k].x, r[k].y, r[k].z, w, bs, 1);  // in [0, nsk)
                kmin = min(kmin, key[k]);
                kmax = max(kmax, key[k]);
            }
        }
        if (threadIdx.x == 0) {
            range[0] = 0x7fffffff;
            range[1] = -1;
        }
        __syncthreads();
        kmin = __reduce_min_sync(0xffffffffu, kmin);
        kmax = __reduce_max_sync(0xffffffffu, kmax);
        if (lane == 0 && kmax >= 0) {
            atomicMin(&range[0], kmin);
            atomicMax(&range[1], kmax);
        }
        __syncthreads();
        const int lo = range[0], nr = range[1] - range[0] + 1;  // n >= 1: 1 <= nr <= nsk
        for (int i = threadIdx.x; i < nr; i += blockDim.x) cnt_s[i] = 0;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SUBSORT_PER; ++k) {
            const unsigned peers = __match_any_sync(0xffffffffu, key[k]);
            if (key[k] >= 0 && lane == __ffs(peers) - 1) atomicAdd(&cnt_s[key[k] - lo], __popc(peers));
        }
        __syncthreads();
        const int per = (nr + blockDim.x - 1) / blockDim.x;
        const int a0 = min((int)threadIdx.x * per, nr), a1 = min(a0 + per, nr);
        int s = 0;
        for (int i = a0; i < a1; ++i) s += cnt_s[i];
        int total;
        int run = block_exclusive_scan(s, sh, total);
        for (int i = a0; i < a1; ++i) {
            const int c = cnt_s[i];
            cnt_s[i] = run;
            run += c;
        }
        __syncthreads();  // also: every thread has its records in registers, the buffer is free
#pragma unroll
        for (int k = 0; k < SUBSORT_PER; ++k) {
            const unsigned peers = __match_any_sync(0xffffffffu, key[k]);
            const int leader = __ffs(peers) - 1;
            int base = 0;
            if (key[k] >= 0 && lane == leader) base = atomicAdd(&cnt_s[key[k] - lo], __popc(peers));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (key[k] >= 0) stage[base + __popc(peers & lanemask_lt())] = r[k];  // < n
        }
        __syncthreads();
        float *const ux_c = ux_o + p0 + c0, *const uy_c = uy_o + p0 + c0, *const uz_c = uz_o + p0 + c0;
        int *const perm_c = perm_o + p0 + c0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const float4 v = stage[i];
            ux_c[i] = v.x;
            uy_c[i] = v.y;
            uz_c[i] = v.z;
            perm_c[i] = __float_as_int(v.w);
        }
        __syncthreads();  // the copy-out has read this buffer before the next prefetch into it
    }
}

// bins from the key scan: bin b's points are [start[b*kb], start[(b+1)*kb])
__global__ void k_bins_from_keys(int nbins, int64_t kb, const int *key_start, int *bin_count, int *bin_start)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbins) return;
    int s = key_start[(int64_t)b * kb], e = key_start[(int64_t)(b + 1) * kb];
    bin_start[b] = s;
    bin_count[b] = e - s;
}

// Exclusive scan of bin counts and of per-bin subproblem counts (one CTA).
__global__ void k_scan_bins(int nbins, const int *count, int *start, int *sub_start, int maxsub, long long *tot)
{
    __shared__ long long s_pts[1024], s_sub[1024];
    int t = threadIdx.x, T = blockDim.x;
    int per = (nbins + T - 1) / T;
    int lo = min(t * per, nbins), hi = min(lo + per, nbins);
    long long a = 0, b = 0;
    for (int i = lo; i < hi; ++i) {
        a += count[i];
        b += (count[i] + maxsub - 1) / maxsub;
    }
    s_pts[t] = a;
    s_sub[t] = b;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        long long va = t >= off ? s_pts[t - off] : 0, vb = t >= off ? s_sub[t - off] : 0;
        __syncthreads();
        s_pts[t] += va;
        s_sub[t] += vb;
        __syncthreads();
    }
    long long ra = s_pts[t] - a, rb = s_sub[t] - b;
    for (int i = lo; i < hi; ++i) {
        start[i] = (int)ra;
        sub_start[i] = (int)rb;
        ra += count[i];
        rb += (count[i] + maxsub - 1) / maxsub;
    }
    if (t == T - 1) {
        tot[0] = s_sub[t];
        tot[1] = s_pts[t];
    }
}

__global__ void k_sub_list(int nbins, const int *count, const int *sub_start, int maxsub, int *sub_bin, int *sub_off)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbins) return;
    int c = count[b];
    int s0 = sub_start[b];
    for (int s = 0; s * maxsub < c; ++s) {
        sub_bin[s0 + s] = b;
        sub_off[s0 + s] = s * maxsub;
    }
}

// inv(R(q)) per quaternion: float32 element products (skopi, float32 quaternions),
// inverse by the adjugate in float64.
__global__ void k_inverse_rotations(const float *quat, int64_t n, double *out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float w = quat[4 * i], x = quat[4 * i + 1], y = quat[4 * i + 2], z = quat[4 * i + 3];
    float q01 = __fmul_rn(w, x), q02 = __fmul_rn(w, y), q03 = __fmul_rn(w, z);
    float q11 = __fmul_rn(x, x), q12 = __fmul_rn(x, y), q13 = __fmul_rn(x, z);
    float q22 = __fmul_rn(y, y), q23 = __fmul_rn(y, z), q33 = __fmul_rn(z, z);
    double r[9];
    r[0] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(q22, q33)));
    r[1] = __fmul_rn(2.f, __fsub_rn(q12, q03));
    r[2] = __fmul_rn(2.f, __fadd_rn(q13, q02));
    r[3] = __fmul_rn(2.f, __fadd_rn(q12, q03));
    r[4] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(q11, q33)));
    r[5] = __fmul_rn(2.f, __fsub_rn(q23, q01));
    r[6] = __fmul_rn(2.f, __fsub_rn(q13, q02));
    r[7] = __fmul_rn(2.f, __fadd_rn(q23, q01));
    r[8] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(q11, q22)));
    double c00 = r[4] * r[8] - r[5] * r[7], c01 = r[5] * r[6] - r[3] * r[8], c02 = r[3] * r[7] - r[4] * r[6];
    double det = r[0] * c00 + r[1] * c01 + r[2] * c02;
    double id = 1.0 / det;
    double *o = out + 9 * i;
    o[0] = c00 * id;
    o[1] = (r[2] * r[7] - r[1] * r[8]) * id;
    o[2] = (r[1] * r[5] - r[2] * r[4]) * id;
    o[3] = c01 * id;
    o[4] = (r[0] * r[8] - r[2] * r[6]) * id;
    o[5] = (r[2] * r[3] - r[0] * r[5]) * id;
    o[6] = c02 * id;
    o[7] = (r[1] * r[6] - r[0] * r[7]) * id;
    o[8] = (r[0] * r[4] - r[1] * r[3]) * id;
}

// Kernel values phi((l0 + a) - u) for the w grid points of one dimension; returns the
// window start relative to the bin origin (>= -floor(w/2)).
template <typename T>
__device__ __forceinline__ int kernel_vals(T u, int w, T beta, T *k)
{
    int l0 = (int)ceil(u - T(0.5) * T(w));
    T inv = T(2) / T(w);
#pragma unroll
    for (int a = 0; a < MAXW; ++a) {
        if (a < w) {
            T t = (T(l0 + a) - u) * inv;
            k[a] = es_eval(t * t, beta);
        }
    }
    return l0;
}

// ------------------------------------------------------------------ deconvolution stages

__device__ __forceinline__ int freq_of(int i, int n) { return i <= n / 2 ? i : i - n; }

// Type 2 (and the first half of the pair): fine-grid spectrum from the modes.
// HERM: write the half spectrum (n x n x (n/2+1)) of the Hermitian part of the modes for
// a C2R transform (real-part output); else the full n^3 spectrum for C2C.
// f: modes (complex or real), centred unless fftord.  support multiplies the modes.
template <typename T, bool REAL_IN, bool HERM>
__global__ void k_pad_deconv(const T *f, const float *support, const T *deconv, int M, int n, int fftord,
                             int conj_out, T *spec)
{
    const int nz = HERM ? n / 2 + 1 : n;
    int64_t total = (int64_t)n * n * nz;
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    int i3 = (int)(idx % nz);
    int64_t r = idx / nz;
    int i2 = (int)(r % n), i1 = (int)(r / n);
    int k1 = freq_of(i1, n), k2 = freq_of(i2, n), k3 = HERM ? i3 : freq_of(i3, n);
    const int kmin = -(M / 2), kmax = M - 1 - M / 2;
    T vr = T(0), vi = T(0);
    auto load = [&](int a, int b, int c, T &re, T &im) {
        re = T(0);
        im = T(0);
        if (a < kmin || a > kmax || b < kmin || b > kmax || c < kmin || c > kmax) return;
        int ia, ib, ic;
        if (fftord) {
            ia = a < 0 ? a + M : a;
            ib = b < 0 ? b + M : b;
            ic = c < 0 ? c + M : c;
        } else {
            ia = a - kmin;
            ib = b - kmin;
            ic = c - kmin;
        }
        int64_t m = ((int64_t)ia * M + ib) * M + ic;
        T s = support ? (T)support[m] : T(1);
        if (REAL_IN) {
            re = f[m] * s;
        } else {
            re = f[2 * m] * s;
            im = f[2 * m + 1] * s;
        }
    };
    int lim = M / 2;
    if (abs(k1) <= lim && abs(k2) <= lim && abs(k3) <= lim) {
        if (HERM) {
            T ar, ai, br, bi;
            load(k1, k2, k3, ar, ai);
            load(-k1, -k2, -k3, br, bi);
            vr = T(0.5) * (ar + br);
            vi = T(0.5) * (ai - bi);
        } else {
            load(k1, k2, k3, vr, vi);
        }
        T p = deconv[abs(k1)] * deconv[abs(k2)] * deconv[abs(k3)];
        vr *= p;
        vi *= p;
        if (conj_out) vi = -vi;
    }
    spec[2 * idx] = vr;
    spec[2 * idx + 1] = vi;
}

// Type 1: modes from the transformed fine grid.  HALF: the grid is an R2C half spectrum
// (n x n x (n/2+1)), else a full C2C spectrum.  The transform computed
// sum_l b_l e^{-i k l h} (HALF, or C2C forward) or e^{+i k l h} (C2C inverse); sgn_flip
// says the requested isign is the opposite one, which for a real grid is a conjugation.
template <typename T, bool HALF, bool REAL_OUT>
__global__ void k_crop_deconv(const T *spec, const float *support, const T *deconv, int M, int n, int fftord,
                              int sgn_flip, T scale, T *f)
{
    int64_t total = (int64_t)M * M * M;
    int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= total) return;
    int ic = (int)(m % M);
    int64_t r = m / M;
    int ib = (int)(r % M), ia = (int)(r / M);
    int k1, k2, k3;
    if (fftord) {
        k1 = ia <= (M - 1) / 2 ? ia : ia - M;
        k2 = ib <= (M - 1) / 2 ? ib : ib - M;
        k3 = ic <= (M - 1) / 2 ? ic : ic - M;
        // FFT ordering with even M: index M/2 holds mode -M/2
        if (!(M & 1)) {
            if (ia == M / 2) k1 = -M / 2;
            if (ib == M / 2) k2 = -M / 2;
            if (ic == M / 2) k3 = -M / 2;
        }
    } else {
        k1 = ia - M / 2;
        k2 = ib - M / 2;
        k3 = ic - M / 2;
    }
    T vr, vi;
    if (HALF) {
        bool neg = k3 < 0;
        int a = neg ? -k1 : k1, b = neg ? -k2 : k2, c = neg ? -k3 : k3;
        a = a < 0 ? a + n : a;
        b = b < 0 ? b + n : b;
        int64_t g = ((int64_t)a * n + b) * (n / 2 + 1) + c;
        vr = spec[2 * g];
        vi = spec[2 * g + 1];
        // B(k) stored for k3 >= 0; B(-k) = conj(B(k)) for a real grid
        bool conj = neg != (bool)sgn_flip;
        if (conj) vi = -vi;
    } else {
        int a = k1 < 0 ? k1 + n : k1, b = k2 < 0 ? k2 + n : k2, c = k3 < 0 ? k3 + n : k3;
        int64_t g = ((int64_t)a * n + b) * n + c;
        vr = spec[2 * g];
        vi = spec[2 * g + 1];
    }
    T p = deconv[abs(k1)] * deconv[abs(k2)] * deconv[abs(k3)] * scale;
    if (support) p *= (T)support[m];
    if (REAL_OUT) {
        f[m] = vr * p;
    } else {
        f[2 * m] = vr * p;
        f[2 * m + 1] = vi * p;
    }
}

// ------------------------------------------------------------------ host side


static void unborrow(Plan &p);
static void sync_borrowed(Plan &p);

// smallest pitch >= S whose residue mod 32 spreads the 32/EW row offsets over distinct banks
static int padded_pitch(int S, int ew)
{
    for (int P = S;; ++P) {
        int r = P % 32;
        if (ew == 8 && (r == 8 || r == 24)) return P;
        if (ew == 16 && r == 16) return P;
    }
}

static int choose_params(Plan &p)
{
    double eps = p.eps;
    double floor_eps = p.prec == 32 ? 1e-7 : 1e-14;
    if (!(eps > 0) || eps < floor_eps) eps = floor_eps;
    double sigma = p.sigma > 1.0 ? p.sigma : 2.0;
    int w;
    if (sigma == 2.0)
        w = (int)ceil(log10(1.0 / eps)) + 1;
    else
        w = (int)ceil(log(1.0 / eps) / (kPi * sqrt(1.0 - 1.0 / sigma)));
    w = std::max(2, std::min(w, MAXW));
    p.w = w;
    p.sigma = sigma;
    p.beta = 0.97 * kPi * w * (1.0 - 0.5 / sigma);
    p.n = next_nice(std::max((int)ceil(sigma * p.M), 2 * w));
    // Warp layout: z offsets over EW lanes (8 for w <= 8, else 16); subgrid rows padded to a
    // pitch P with P mod 32 = 8/24 (EW 8) or 16 (EW 16) for conflict-free shared access.
    // Bin size: the largest whose pair-kernel footprint (two complex subgrids) allows two
    // CTAs per SM; without room for the padding the rows stay unpadded.
    p.ew = w <= 8 ? 8 : 16;
    const size_t budget = 100 * 1024;
    p.bs = 0;
    for (int pad = 1; pad >= 0 && p.bs == 0; --pad) {
        for (int bs = 16; bs >= 2 && p.bs == 0; bs /= 2) {
            int bsc = std::min(bs, p.n);
            int S = bsc + w;
            int P = pad ? padded_pitch(S, p.ew) : S;
            if ((size_t)S * S * P * 4 * elem(p) <= budget) {
                p.bs = bsc;
                p.S = S;
                p.P = P;
            }
        }
    }
    if (p.bs == 0) {  // very wide kernels: smallest bins, unpadded rows
        p.bs = 2;
        p.S = 2 + w;
        p.P = p.S;
    }
    p.nb = (p.n + p.bs - 1) / p.bs;
    return CMT_OK;
}

template <typename T>
static int upload_deconv(Plan &p)
{
    std::vector<double> gx, gw;
    gauss_legendre(std::max(64, 4 * p.w), gx, gw);
    int K = p.M / 2 + 2;
    std::vector<T> h(K);
    for (int k = 0; k < K; ++k) h[k] = (T)(1.0 / kernel_ft(k * 2.0 * kPi / p.n, p.w, p.beta, gx, gw));
    CMT_TRY_CUDA(cudaMalloc(&p.deconv, K * sizeof(T)));
    CMT_TRY_CUDA(cudaMemcpy(p.deconv, h.data(), K * sizeof(T), cudaMemcpyHostToDevice));
    return CMT_OK;
}

static int ensure_fft(Plan &p, int kind)
{
    int n = p.n;
    bool dbl = p.prec == 64;
    if (kind == 0 && !p.has_c2c) {
        CMT_TRY_CUFFT(cufftPlan3d(&p.fft_c2c, n, n, n, dbl ? CUFFT_Z2Z : CUFFT_C2C));
        CMT_TRY_CUFFT(cufftSetStream(p.fft_c2c, p.stream));
        p.has_c2c = true;
    }
    if (kind == 1 && !p.has_r2c) {
        CMT_TRY_CUFFT(cufftPlan3d(&p.fft_r2c, n, n, n, dbl ? CUFFT_D2Z : CUFFT_R2C));
        CMT_TRY_CUFFT(cufftSetStream(p.fft_r2c, p.stream));
        p.has_r2c = true;
    }
    if (kind == 2 && !p.has_c2r) {
        CMT_TRY_CUFFT(cufftPlan3d(&p.fft_c2r, n, n, n, dbl ? CUFFT_Z2D : CUFFT_C2R));
        CMT_TRY_CUFFT(cufftSetStream(p.fft_c2r, p.stream));
        p.has_c2r = true;
    }
    return CMT_OK;
}

static int grid_for(int64_t N)
{
    int64_t blocks = (N + 255) / 256;
    return (int)std::min<int64_t>(std::max<int64_t>(blocks, 1), 152 * 16);
}

// The scratch block comes from the device's default stream-ordered memory pool.  By default
// the pool hands freed memory back to the system at every synchronisation, so each set_pts
// would map its scratch anew; this process keeps freed pool memory for reuse instead (a
// setting of this process's pool, not of the device).
static void keep_pool_memory()
{
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done[dev] = true;
}

// one block of sorted points for capacity C: coordinates x | y | z (C values each), then the
// permutation (C ints); the T arrays come first so every array stays aligned
template <typename T>
static size_t pts_block_bytes(int64_t C)
{
    // also holds C sorted records (16 / 32 bytes) while the points are being sorted
    return (size_t)C * std::max(3 * sizeof(T) + sizeof(int), sizeof(SortedRec<T>));
}

template <typename T>
static void set_pts_pointers(Plan &p, void *block, int64_t C)
{
    T *b = reinterpret_cast<T *>(block);
    p.ux = b;
    p.uy = b + C;
    p.uz = b + 2 * C;
    p.perm = reinterpret_cast<int *>(b + 3 * C);
}

template <typename T>
static int set_pts_impl(Plan &p, int mode, int64_t N, const T *x, const T *y, const T *z, QuatSrc q)
{
    unborrow(p);
    p.N = 0;
    // the sort's buffers come from the stream-ordered pool (cudaMallocAsync on the plan's
    // stream): a plan created and sorted afresh reuses pool memory instead of cudaMalloc,
    // which maps new memory and synchronises the device
    cudaStream_t st = p.stream;
    keep_pool_memory();
    CMT_CHECK_ARG(N > 0 && N <= 0x7fffffffLL, "number of points %lld outside [1, 2^31-1]", (long long)N);
    int nbins = p.nb * p.nb * p.nb;
    // Global passes sort by bin and by the window origin on this grid ((bs+1)^3 keys per bin,
    // a few million counters that stay in L2), so a dense bin's subproblems hold contiguous
    // ranges of origins and points that share a window land next to each other; k_subsort
    // then orders each subproblem by origin and refinement (point_key).  The scatter writes
    // one 16-byte record per point, one write stream per key, which L2 still merges at this
    // key count.  The plan's sort_keys sets the number of origin coordinates keyed
    // (CMT_SORT_KEYS = 1..3 overrides, for comparison).  Plans without sort_origin, and grids
    // with too many keys, sort by bin only.
    const int64_t O = p.bs + 1;
    int kd = std::min(3, std::max(1, p.sort_keys));
    if (const char *env = getenv("CMT_SORT_KEYS")) kd = std::min(3, std::max(1, atoi(env)));
    const int64_t kbo = kd == 1 ? O : (kd == 2 ? O * O : O * O * O);
    const int fine_sort = p.sort_origin && (int64_t)nbins * kbo < (1LL << 27) ? 1 + kd : 0;
    const int64_t kb = fine_sort ? kbo : 1;
    const int nsk = (int)(O * O * O * 8);
    const int sub_smem = (int)(nsk * sizeof(int) + (size_t)p.maxsub * sizeof(unsigned short));
    const bool do_subsort = nsk <= 65535 && sub_smem <= 200 * 1024;
    const int64_t nkeys = (int64_t)nbins * kb;
    const int64_t ntiles = (nkeys + 1 + SCAN_TILE - 1) / SCAN_TILE;
    if (!p.dflag) {
        CMT_TRY_CUDA(cudaMallocAsync(&p.dflag, sizeof(int) * 4, st));
        CMT_TRY_CUDA(cudaMallocAsync(&p.dtot, sizeof(long long) * 2, st));
    }
    if (nbins > p.cap_bins) {  // first points, or a retuned bin size
        if (p.bin_count) cudaFreeAsync(p.bin_count, st);
        if (p.bin_fill) cudaFreeAsync(p.bin_fill, st);
        if (p.bin_start) cudaFreeAsync(p.bin_start, st);
        p.bin_count = p.bin_fill = p.bin_start = nullptr;
        p.cap_bins = 0;
        CMT_TRY_CUDA(cudaMallocAsync(&p.bin_count, sizeof(int) * nbins, st));
        CMT_TRY_CUDA(cudaMallocAsync(&p.bin_fill, sizeof(int) * nbins, st));
        CMT_TRY_CUDA(cudaMallocAsync(&p.bin_start, sizeof(int) * nbins, st));
        p.cap_bins = nbins;
    }
    if (nkeys + 1 > p.cap_keys) {
        if (p.key_start) cudaFreeAsync(p.key_start, st);
        if (p.key_next) cudaFreeAsync(p.key_next, st);
        if (p.tile_sums) cudaFreeAsync(p.tile_sums, st);
        p.key_start = p.key_next = p.tile_sums = nullptr;
        p.cap_keys = 0;
        CMT_TRY_CUDA(cudaMallocAsync(&p.key_start, sizeof(int) * (nkeys + 1), st));
        CMT_TRY_CUDA(cudaMallocAsync(&p.key_next, sizeof(int) * (nkeys + 1), st));
        CMT_TRY_CUDA(cudaMallocAsync(&p.tile_sums, sizeof(int) * ntiles, st));
        p.cap_keys = nkeys + 1;
    }
    // Sorted points live in one block (x, y, z coordinates, then the permutation).  A scratch
    // block of the same capacity holds the pass-1 records, then receives the subproblem sort's
    // output, after which the two blocks swap and the old one is freed.
    const size_t blk = pts_block_bytes<T>(N);
    const size_t scratch_bytes = std::max(blk, sizeof(PtRec<T>) * (size_t)N);
    // pass 1 writes records (caller order) to the scratch block, pass 2 sorted records to the
    // plan block, the subproblem sort (or a plain copy) the final arrays to the scratch block,
    // and the blocks swap.  Both blocks come from the stream-ordered pool, which keeps freed
    // memory: the block the first call frees is the next call's scratch, so only the first
    // call maps new memory.
    if (N > p.cap_pts) {
        if (p.pts_block) cudaFreeAsync(p.pts_block, st);
        p.pts_block = nullptr;
        p.perm = nullptr;
        p.ux = p.uy = p.uz = nullptr;
        p.cap_pts = 0;
        CMT_TRY_CUDA(cudaMallocAsync(&p.pts_block, blk, st));
        p.cap_pts = N;
    }
    set_pts_pointers<T>(p, p.pts_block, p.cap_pts);
    void *scratch = nullptr;
    CMT_TRY_CUDA(cudaMallocAsync(&scratch, scratch_bytes, st));
    struct ScratchGuard {
        void *&ptr;
        cudaStream_t st;
        ~ScratchGuard() { if (ptr) cudaFreeAsync(ptr, st); }
    } guard{scratch, st};
    CMT_TRY_CUDA(cudaMemsetAsync(p.key_next, 0, sizeof(int) * (nkeys + 1), st));
    CMT_TRY_CUDA(cudaMemsetAsync(p.dflag, 0, sizeof(int) * 4, st));
    double s = p.n / (2.0 * kPi);
    T s_hi = (T)s, s_lo = (T)(s - (double)s_hi);
    // cells are below n <= 2^20, so the multiply-high division is exact for bs <= 4096
    SortGeom sgeo{p.n, p.bs, p.nb, p.w, fine_sort,
                  p.bs >= 2 && (uint64_t)p.n * p.bs < (1ULL << 32) ? magic32((unsigned)p.bs) : 0u,
                  p.n >= 2 && 5ULL * p.n * p.n < (1ULL << 32) ? magic32((unsigned)p.n) : 0u};
    int g = grid_for(N);
    // pass 1: counts per key (into key_next), then key_start = exclusive scan (with the total
    // at key_start[nkeys])
    k_bin_count<T><<<g, 256, 0, st>>>(mode, N, x, y, z, q, s_hi, s_lo, sgeo, p.key_next, (PtRec<T> *)scratch,
                                      p.dflag);
    CMT_LAUNCH_CHECK();
    k_scan_tiles<<<(unsigned)ntiles, SCAN_THREADS, 0, st>>>(p.key_next, p.key_start, nkeys + 1, p.tile_sums);
    k_scan_single<<<1, 1024, 0, st>>>(p.tile_sums, (int)ntiles);
    k_add_tile_offsets<<<(unsigned)ceil_div(nkeys + 1, 256), 256, 0, st>>>(p.key_start, nkeys + 1, p.tile_sums);
    k_bins_from_keys<<<ceil_div(nbins, 256), 256, 0, st>>>(nbins, kb, p.key_start, p.bin_count, p.bin_start);
    CMT_LAUNCH_CHECK();
    int *sub_start = p.bin_fill;  // scratch for the subproblem scan
    k_scan_bins<<<1, 1024, 0, st>>>(nbins, p.bin_count, p.bin_start, sub_start, p.maxsub, p.dtot);
    CMT_LAUNCH_CHECK();
    long long tot[2];
    int flag = 0;
    CMT_TRY_CUDA(cudaMemcpyAsync(tot, p.dtot, sizeof tot, cudaMemcpyDeviceToHost, st));
    CMT_TRY_CUDA(cudaMemcpyAsync(&flag, p.dflag, sizeof flag, cudaMemcpyDeviceToHost, st));
    CMT_TRY_CUDA(cudaStreamSynchronize(st));
    if (flag) {
        set_error("nonuniform point outside (-3 pi, 3 pi) (cmtip asserts |x| < 3 pi)");
        return CMT_ERR_RANGE;
    }
    p.nsub = tot[0];
    if (p.nsub > p.cap_sub) {
        if (p.sub_bin) cudaFreeAsync(p.sub_bin, st);
        if (p.sub_off) cudaFreeAsync(p.sub_off, st);
        p.sub_bin = p.sub_off = nullptr;
        p.cap_sub = 0;
        CMT_TRY_CUDA(cudaMallocAsync(&p.sub_bin, sizeof(int) * p.nsub, st));
        CMT_TRY_CUDA(cudaMallocAsync(&p.sub_off, sizeof(int) * p.nsub, st));
        p.cap_sub = p.nsub;
    }
    k_sub_list<<<ceil_div(nbins, 256), 256, 0, st>>>(nbins, p.bin_count, sub_start, p.maxsub, p.sub_bin, p.sub_off);
    CMT_LAUNCH_CHECK();
    // pass 2: scatter, key_next starting at each key's first position
    CMT_TRY_CUDA(cudaMemcpyAsync(p.key_next, p.key_start, sizeof(int) * (nkeys + 1), cudaMemcpyDeviceToDevice, st));
    SortedRec<T> *srec = reinterpret_cast<SortedRec<T> *>(p.pts_block);
    if (sizeof(T) == 4) {
        k_bin_scatter_tiled<<<(unsigned)std::min<int64_t>(ceil_div(N, (int64_t)SCAT_TILE), 152 * 8), SCAT_THREADS, 0,
                              st>>>(N, reinterpret_cast<const PtRec<float> *>(scratch), p.key_start, p.key_next,
                                    reinterpret_cast<SortedRec<float> *>(srec), p.dflag);
    } else {
        k_bin_scatter<T><<<g, 256, 0, st>>>(N, (const PtRec<T> *)scratch, p.key_start, p.key_next, srec, p.dflag);
    }
    CMT_LAUNCH_CHECK();
    {
        Plan o = p;
        set_pts_pointers<T>(o, scratch, N);
        const int csm = 2 * SUBSORT_CHUNK * 16 + nsk * (int)sizeof(int);
        if (do_subsort && p.nsub > 0 && sizeof(T) == 4 && fine_sort >= 3 && csm <= 200 * 1024) {
            CMT_TRY(prep_smem(k_subsort_chunked, csm));
            k_subsort_chunked<<<(unsigned)p.nsub, SUBSORT_THREADS, csm, st>>>(
                p.sub_bin, p.sub_off, p.bin_count, p.bin_start, p.w, p.bs, p.maxsub, nsk,
                reinterpret_cast<const SortedRec<float> *>(srec), o.perm, (float *)o.ux, (float *)o.uy,
                (float *)o.uz);
        } else if (do_subsort && p.nsub > 0) {
            CMT_TRY(prep_smem(k_subsort<T>, sub_smem));
            k_subsort<T><<<(unsigned)p.nsub, 512, sub_smem, st>>>(p.sub_bin, p.sub_off, p.bin_count, p.bin_start,
                                                                  p.w, p.bs, p.maxsub, nsk, srec, o.perm, (T *)o.ux,
                                                                  (T *)o.uy, (T *)o.uz);
        } else {
            k_rec_to_arrays<T><<<g, 256, 0, st>>>(N, srec, o.perm, (T *)o.ux, (T *)o.uy, (T *)o.uz);
        }
        CMT_LAUNCH_CHECK();
        std::swap(p.pts_block, scratch);  // the guard frees the old block after the kernels
        p.cap_pts = N;
        set_pts_pointers<T>(p, p.pts_block, N);
    }
    CMT_TRY_CUDA(cudaMemcpyAsync(&flag, p.dflag, sizeof flag, cudaMemcpyDeviceToHost, st));
    CMT_TRY_CUDA(cudaStreamSynchronize(st));
    if (flag) {
        set_error("internal error: bin assignment differs between counting passes");
        return CMT_ERR_STATE;
    }
    p.N = N;
    ++p.pts_version;
    return CMT_OK;
}

// Phases of an execute: grid preparation (zeroing; or deconvolution, padding and FFT), the
// spreading / interpolation kernel, and the FFT and deconvolution after spreading.  A batch
// of plans runs every plan's preparation, one kernel launch over all plans, then the rest.
enum { PH_PRE = 1, PH_KERNEL = 2, PH_POST = 4, PH_ALL = 7 };

template <typename T>
static int exec_type1(Plan &p, const T *c, T *f, const float *support, double scale, int flags, int phases = PH_ALL)
{
    bool real_in = flags & CMT_REAL_IN, real_out = flags & CMT_REAL_OUT, fftord = flags & CMT_MODEORD_FFT;
    cudaStream_t st = p.stream;
    int n = p.n;
    T beta = (T)p.beta;
    int M = p.M;
    int64_t mt = (int64_t)M * M * M;
    if (real_in) {
        int rs = n + 2;
        if (phases & PH_PRE) {
            CMT_TRY(ensure_fft(p, 1));
            CMT_TRY_CUDA(cudaMemsetAsync(p.fine, 0, sizeof(T) * (size_t)n * n * rs, st));
        }
        if (phases & PH_KERNEL) CMT_TRY(launch_spread(p, c, false, rs));
        if (!(phases & PH_POST)) return CMT_OK;
        if (p.prec == 64)
            CMT_TRY_CUFFT(cufftExecD2Z(p.fft_r2c, (double *)p.fine, (cufftDoubleComplex *)p.fine));
        else
            CMT_TRY_CUFFT(cufftExecR2C(p.fft_r2c, (float *)p.fine, (cufftComplex *)p.fine));
        int sgn_flip = p.isign > 0;  // R2C computed e^{-i}
        unsigned gb = (unsigned)ceil_div(mt, 256);
        if (real_out)
            k_crop_deconv<T, true, true><<<gb, 256, 0, st>>>((T *)p.fine, support, (T *)p.deconv, M, n, fftord,
                                                             sgn_flip, (T)scale, f);
        else
            k_crop_deconv<T, true, false><<<gb, 256, 0, st>>>((T *)p.fine, support, (T *)p.deconv, M, n, fftord,
                                                              sgn_flip, (T)scale, f);
        CMT_LAUNCH_CHECK();
    } else {
        if (phases & PH_PRE) {
            CMT_TRY(ensure_fft(p, 0));
            CMT_TRY_CUDA(cudaMemsetAsync(p.fine, 0, sizeof(T) * 2 * (size_t)n * n * n, st));
        }
        if (phases & PH_KERNEL) CMT_TRY(launch_spread(p, c, true, n));
        if (!(phases & PH_POST)) return CMT_OK;
        int dir = p.isign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE;
        if (p.prec == 64)
            CMT_TRY_CUFFT(cufftExecZ2Z(p.fft_c2c, (cufftDoubleComplex *)p.fine, (cufftDoubleComplex *)p.fine, dir));
        else
            CMT_TRY_CUFFT(cufftExecC2C(p.fft_c2c, (cufftComplex *)p.fine, (cufftComplex *)p.fine, dir));
        unsigned gb = (unsigned)ceil_div(mt, 256);
        if (real_out)
            k_crop_deconv<T, false, true><<<gb, 256, 0, st>>>((T *)p.fine, support, (T *)p.deconv, M, n, fftord, 0,
                                                              (T)scale, f);
        else
            k_crop_deconv<T, false, false><<<gb, 256, 0, st>>>((T *)p.fine, support, (T *)p.deconv, M, n, fftord, 0,
                                                               (T)scale, f);
        CMT_LAUNCH_CHECK();
    }
    return CMT_OK;
}

template <typename T>
static int exec_type2(Plan &p, T *c, const T *f, const float *support, double scale, int flags, int phases = PH_ALL)
{
    bool real_in = flags & CMT_REAL_IN, real_out = flags & CMT_REAL_OUT, fftord = flags & CMT_MODEORD_FFT;
    CMT_CHECK_ARG(scale == 1.0, "type-2 execute takes scale = 1");
    cudaStream_t st = p.stream;
    int n = p.n;
    T beta = (T)p.beta;
    int M = p.M;
    if (real_out) {
        // Re(c) = sum_k g_k e^{isign i k.x} with g the Hermitian part of f: real fine grid
        if (!(phases & PH_PRE)) {
            if (phases & PH_KERNEL) CMT_TRY(launch_interp(p, 2, n + 2, c));
            return CMT_OK;
        }
        CMT_TRY(ensure_fft(p, 2));
        int64_t tot = (int64_t)n * n * (n / 2 + 1);
        unsigned gb = (unsigned)ceil_div(tot, 256);
        int conj_out = p.isign < 0;  // C2R computes e^{+i}
        if (real_in)
            k_pad_deconv<T, true, true><<<gb, 256, 0, st>>>(f, support, (T *)p.deconv, M, n, fftord, conj_out,
                                                            (T *)p.fine);
        else
            k_pad_deconv<T, false, true><<<gb, 256, 0, st>>>(f, support, (T *)p.deconv, M, n, fftord, conj_out,
                                                             (T *)p.fine);
        CMT_LAUNCH_CHECK();
        if (p.prec == 64)
            CMT_TRY_CUFFT(cufftExecZ2D(p.fft_c2r, (cufftDoubleComplex *)p.fine, (double *)p.fine));
        else
            CMT_TRY_CUFFT(cufftExecC2R(p.fft_c2r, (cufftComplex *)p.fine, (float *)p.fine));
        if (phases & PH_KERNEL) CMT_TRY(launch_interp(p, 2, n + 2, c));
    } else {
        if (!(phases & PH_PRE)) {
            if (phases & PH_KERNEL) CMT_TRY(launch_interp(p, 0, n, c));
            return CMT_OK;
        }
        CMT_TRY(ensure_fft(p, 0));
        int64_t tot = (int64_t)n * n * n;
        unsigned gb = (unsigned)ceil_div(tot, 256);
        if (real_in)
            k_pad_deconv<T, true, false><<<gb, 256, 0, st>>>(f, support, (T *)p.deconv, M, n, fftord, 0, (T *)p.fine);
        else
            k_pad_deconv<T, false, false><<<gb, 256, 0, st>>>(f, support, (T *)p.deconv, M, n, fftord, 0,
                                                              (T *)p.fine);
        CMT_LAUNCH_CHECK();
        int dir = p.isign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE;
        if (p.prec == 64)
            CMT_TRY_CUFFT(cufftExecZ2Z(p.fft_c2c, (cufftDoubleComplex *)p.fine, (cufftDoubleComplex *)p.fine, dir));
        else
            CMT_TRY_CUFFT(cufftExecC2C(p.fft_c2c, (cufftComplex *)p.fine, (cufftComplex *)p.fine, dir));
        if (phases & PH_KERNEL) CMT_TRY(launch_interp(p, 0, n, c));
    }
    return CMT_OK;
}

template <typename T>
static int exec_pair(Plan &p, const T *fin, T *fout, const float *support, double scale)
{
    cudaStream_t st = p.stream;
    int n = p.n;
    int M = p.M;
    CMT_TRY(ensure_fft(p, 0));
    if (!p.fine2) CMT_TRY_CUDA(cudaMalloc(&p.fine2, 2 * elem(p) * (size_t)n * n * n));
    int64_t tot = (int64_t)n * n * n;
    unsigned gb = (unsigned)ceil_div(tot, 256);
    // A: modes -> fine grid, isign -1 (cmtip's forward, forward.py:40)
    k_pad_deconv<T, true, false><<<gb, 256, 0, st>>>(fin, support, (T *)p.deconv, M, n, 0, 0, (T *)p.fine);
    CMT_LAUNCH_CHECK();
    if (p.prec == 64)
        CMT_TRY_CUFFT(cufftExecZ2Z(p.fft_c2c, (cufftDoubleComplex *)p.fine, (cufftDoubleComplex *)p.fine, CUFFT_FORWARD));
    else
        CMT_TRY_CUFFT(cufftExecC2C(p.fft_c2c, (cufftComplex *)p.fine, (cufftComplex *)p.fine, CUFFT_FORWARD));
    CMT_TRY_CUDA(cudaMemsetAsync(p.fine2, 0, 2 * elem(p) * (size_t)n * n * n, st));
    CMT_TRY(launch_pair(p, false));
    // A^H: isign +1 (cmtip's adjoint, adjoint.py:33)
    if (p.prec == 64)
        CMT_TRY_CUFFT(cufftExecZ2Z(p.fft_c2c, (cufftDoubleComplex *)p.fine2, (cufftDoubleComplex *)p.fine2, CUFFT_INVERSE));
    else
        CMT_TRY_CUFFT(cufftExecC2C(p.fft_c2c, (cufftComplex *)p.fine2, (cufftComplex *)p.fine2, CUFFT_INVERSE));
    unsigned gm = (unsigned)ceil_div((int64_t)M * M * M, 256);
    k_crop_deconv<T, false, true><<<gm, 256, 0, st>>>((T *)p.fine2, support, (T *)p.deconv, M, n, 0, 0, (T)scale, fout);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

// a derived plan follows its source's current points (the source may have been given new
// points since the derivation)
static void sync_borrowed(Plan &p)
{
    const Plan *s = p.points_of;
    if (!s) return;
    if (p.nb != s->nb || p.bs != 2 * s->bs || p.maxsub != s->maxsub) {  // the source was retuned
        p.bs = 2 * s->bs;
        p.nb = s->nb;
        p.S = p.bs + p.w;
        p.P = padded_pitch(p.S, p.ew);
        p.maxsub = s->maxsub;
    }
    p.N = s->N;
    p.nsub = s->nsub;
    p.bin_count = s->bin_count;
    p.bin_start = s->bin_start;
    p.sub_bin = s->sub_bin;
    p.sub_off = s->sub_off;
    p.perm = s->perm;
    p.ux = s->ux;
    p.uy = s->uy;
    p.uz = s->uz;
}

// a plan that borrowed another plan's points drops the borrowed pointers (not its own)
static void unborrow(Plan &p)
{
    if (!p.points_of) return;
    p.bin_count = p.bin_fill = p.bin_start = p.sub_bin = p.sub_off = p.perm = nullptr;
    p.ux = p.uy = p.uz = nullptr;
    p.dflag = nullptr;
    p.dtot = nullptr;
    p.cap_pts = p.cap_sub = p.cap_bins = 0;
    p.N = p.nsub = 0;
    p.points_of = nullptr;
    p.cscale = 1.0;
}

static void destroy(Plan *p)
{
    if (!p) return;
    // the sort's buffers are pool allocations, which cudaFree releases without waiting for
    // work still using them: let every launch finish first
    cudaDeviceSynchronize();
    unborrow(*p);
    cudaFree(p->bin_count);
    cudaFree(p->bin_fill);
    cudaFree(p->key_start);
    cudaFree(p->key_next);
    cudaFree(p->tile_sums);
    cudaFree(p->bin_start);
    cudaFree(p->sub_bin);
    cudaFree(p->sub_off);
    cudaFree(p->pts_block);
    cudaFree(p->dflag);
    cudaFree(p->dtot);
    cudaFree(p->fine);
    cudaFree(p->fine2);
    cudaFree(p->deconv);
    for (int i = 0; i < 2 * Plan::PROF_CAP; ++i)
        if (p->ev[i]) cudaEventDestroy(p->ev[i]);
    if (p->has_c2c) cufftDestroy(p->fft_c2c);
    if (p->has_r2c) cufftDestroy(p->fft_r2c);
    if (p->has_c2r) cufftDestroy(p->fft_c2r);
}

}  // namespace cmt

// ====================================================================== C ABI

using namespace cmt;

extern "C" const char *cmt_last_error(void) { return cmt::g_err; }

extern "C" const char *cmt_version(void) { return "cmtip_gb300 0.1 (sm_103a)"; }

extern "C" int cmt_plan_create(int type, int M, int prec, double eps, int isign, double upsampfac, void *stream,
                               cmt_plan **out)
{
    CMT_CHECK_ARG(out, "null plan pointer");
    *out = nullptr;
    CMT_CHECK_ARG(type == 1 || type == 2, "type must be 1 or 2 (got %d)", type);
    CMT_CHECK_ARG(prec == 32 || prec == 64, "prec must be 32 or 64 (got %d)", prec);
    CMT_CHECK_ARG(M >= 1 && M <= 1024, "M must be in [1, 1024] (got %d)", M);
    CMT_CHECK_ARG(isign == 1 || isign == -1, "isign must be +1 or -1");
    cmt_plan *p = new (std::nothrow) cmt_plan();
    if (!p) {
        set_error("host allocation failed");
        return CMT_ERR_OOM;
    }
    p->type = type;
    p->M = M;
    p->prec = prec;
    p->eps = eps;
    p->isign = isign;
    p->sigma = upsampfac > 1.0 ? upsampfac : 2.0;
    p->stream = (cudaStream_t)stream;
    choose_params(*p);
    // FP32 interpolation plans with table-driven widths: bins of 5 fine cells keep the staged
    // subgrid and the point tables small enough for more resident CTAs and make the sort's
    // subproblems finer; measured at 1.31e9 points, M = 81, w = 7: sort + interpolation
    // 148.5 ms against 194.5 ms (complex values) and 107.6 ms against 132 ms (real part)
    // with the default bins of 8 (type-1 plans gain nothing from it)
    if (type == 2 && prec == 32 && p->w >= 2 && p->w <= 8 && p->n >= 5) {
        p->bs = 5;
        p->S = p->bs + p->w;
        p->P = padded_pitch(p->S, p->ew);
        p->nb = (p->n + p->bs - 1) / p->bs;
    }
    // layout override for tuning: CMT_SPREAD_PRIV=1 spreads real strengths into per-warp
    // private subgrids instead of one subgrid with shared atomics
    if (const char *env = getenv("CMT_SPREAD_PRIV")) p->spread_priv = atoi(env) != 0;
    // CMT_SPREAD_TAB=0 / CMT_INTERP_TAB=0 select the per-point spreading / interpolation
    // kernels for every width, for comparison
    if (const char *env = getenv("CMT_SPREAD_TAB")) p->spread_tab = atoi(env) != 0;
    if (const char *env = getenv("CMT_INTERP_TAB")) p->interp_tab = atoi(env) != 0;
    // Spreading plans sort each bin by the whole window origin (long runs of shared windows
    // across the bin, for this plan and a derived one); FP32 interpolation plans by its x, y
    // part, which keeps the scatter's key streams few and lets the per-subproblem sort read
    // each record once (k_subsort_chunked); FP64 interpolation plans by bin only.
    // CMT_SORT_ORIGIN=0/1 overrides, for comparison.
    p->sort_origin = type == 1 || prec == 32;
    p->sort_keys = type == 1 ? 3 : 2;
    if (const char *env = getenv("CMT_SORT_ORIGIN")) p->sort_origin = atoi(env) != 0;
    int rc = CMT_OK;
    size_t bytes = 2 * elem(*p) * (size_t)p->n * p->n * p->n;
    cudaError_t e = cudaMalloc(&p->fine, bytes);
    if (e != cudaSuccess) {
        set_error("fine grid allocation (%zu bytes): %s", bytes, cudaGetErrorString(e));
        rc = CMT_ERR_OOM;
    }
    if (rc == CMT_OK) rc = prec == 64 ? upload_deconv<double>(*p) : upload_deconv<float>(*p);
    if (rc != CMT_OK) {
        destroy(p);
        delete p;
        return rc;
    }
    *out = p;
    return CMT_OK;
}

// A plan on the points of src with a fine grid exactly twice as fine: bins twice as large
// (in fine cells) cover the same regions, so src's bin order, permutation and subproblem
// list apply unchanged and the stored coordinates are scaled by 2 on the fly.  Used for
// the Toeplitz kernel of the autocorrelation solve (2M modes on the points that the M-mode
// plan already sorted).  src must keep its points and outlive this plan (or until this
// plan gets points of its own through set_pts).
extern "C" int cmt_plan_create_derived(const cmt_plan *src, int type, int M, int isign, cmt_plan **out)
{
    CMT_CHECK_ARG(src && out, "null argument");
    *out = nullptr;
    CMT_CHECK_ARG(type == 1 || type == 2, "type must be 1 or 2");
    CMT_CHECK_ARG(isign == 1 || isign == -1, "isign must be +1 or -1");
    CMT_CHECK_ARG(M >= 1 && 2 * src->n >= 2 * src->w && 2 * src->n > M, "M too large for a grid of %d", 2 * src->n);
    cmt_plan *p = new (std::nothrow) cmt_plan();
    if (!p) return CMT_ERR_OOM;
    p->type = type;
    p->M = M;
    p->prec = src->prec;
    p->eps = src->eps;
    p->isign = isign;
    p->stream = src->stream;
    p->n = 2 * src->n;
    p->sigma = (double)p->n / M;
    p->w = src->w;
    p->beta = src->beta;
    p->ew = src->ew;
    p->bs = 2 * src->bs;
    p->nb = src->nb;
    p->S = p->bs + p->w;
    p->P = padded_pitch(p->S, p->ew);
    p->maxsub = src->maxsub;
    p->spread_priv = 0;
    p->points_of = src;
    p->cscale = 2.0 * src->cscale;
    // real spreading through the extended register window (k_spread_tab); CMT_SPREAD_EXT=0
    // selects the plain per-origin kernel, for comparison
    p->spread_ext = p->cscale == 2.0 && p->w + 1 <= 8;
    if (const char *env = getenv("CMT_SPREAD_EXT")) p->spread_ext = p->spread_ext && atoi(env) != 0;
    p->spread_tab = src->spread_tab;
    p->interp_tab = src->interp_tab;
    if (const char *env = getenv("CMT_SPREAD_TAB")) p->spread_tab = atoi(env) != 0;
    if (const char *env = getenv("CMT_INTERP_TAB")) p->interp_tab = atoi(env) != 0;
    p->N = src->N;
    p->nsub = src->nsub;
    p->bin_count = src->bin_count;
    p->bin_start = src->bin_start;
    p->sub_bin = src->sub_bin;
    p->sub_off = src->sub_off;
    p->perm = src->perm;
    p->ux = src->ux;
    p->uy = src->uy;
    p->uz = src->uz;
    int rc = CMT_OK;
    size_t bytes = 2 * elem(*p) * (size_t)p->n * p->n * p->n;
    cudaError_t e = cudaMalloc(&p->fine, bytes);
    if (e != cudaSuccess) {
        set_error("fine grid allocation (%zu bytes): %s", bytes, cudaGetErrorString(e));
        rc = CMT_ERR_OOM;
    }
    if (rc == CMT_OK) rc = p->prec == 64 ? upload_deconv<double>(*p) : upload_deconv<float>(*p);
    if (rc != CMT_OK) {
        destroy(p);
        delete p;
        return rc;
    }
    *out = p;
    return CMT_OK;
}

extern "C" int cmt_plan_info(const cmt_plan *p, int *n_fine, int *width, double *beta, int *bin_size,
                             int64_t *n_sub)
{
    CMT_CHECK_ARG(p, "null plan");
    if (n_fine) *n_fine = p->n;
    if (width) *width = p->w;
    if (beta) *beta = p->beta;
    if (bin_size) *bin_size = p->bs;
    if (n_sub) *n_sub = p->nsub;
    return CMT_OK;
}

// Largest shared-memory need of this plan's kernels (spreading / interpolation of complex
// values through the point table, the fused pair) for bin size bs.
static size_t plan_smem_need(const Plan &p, int bs)
{
    Plan q = p;
    q.bs = bs;
    q.S = bs + p.w;
    q.P = padded_pitch(q.S, p.ew);
    size_t need = 4 * sub_bytes(q);  // pair kernel: two complex subgrids
    need = std::max(need, batch_smem(q, true, true));
    need = std::max(need, batch_smem(q, false, true));
    return need;
}

// Bin size (fine cells per bin edge) and points per subproblem, for the autotuner; the
// plan's points are dropped (set_pts again).  bin_size 0 / maxsub 0 keep the current value.
extern "C" int cmt_plan_set_tuning(cmt_plan *p, int bin_size, int maxsub)
{
    CMT_CHECK_ARG(p, "null plan");
    CMT_CHECK_ARG(!p->points_of, "a derived plan follows its source's tuning");
    if (bin_size == 0) bin_size = p->bs;
    if (maxsub == 0) maxsub = p->maxsub;
    CMT_CHECK_ARG(bin_size >= 2 && bin_size <= 32, "bin size %d outside [2, 32]", bin_size);
    CMT_CHECK_ARG(maxsub >= 256 && maxsub <= (1 << 20), "points per subproblem %d outside [256, 2^20]", maxsub);
    const size_t need = plan_smem_need(*p, bin_size);
    CMT_CHECK_ARG(need <= 227 * 1024, "bin size %d needs %zu bytes of shared memory per CTA", bin_size, need);
    if (bin_size != p->bs || maxsub != p->maxsub) {
        p->bs = std::min(bin_size, p->n);
        p->S = p->bs + p->w;
        p->P = padded_pitch(p->S, p->ew);
        p->nb = (p->n + p->bs - 1) / p->bs;
        p->maxsub = maxsub;
        p->N = 0;
        p->nsub = 0;
        ++p->pts_version;
    }
    return CMT_OK;
}

extern "C" int cmt_plan_get_tuning(const cmt_plan *p, int *bin_size, int *maxsub)
{
    CMT_CHECK_ARG(p, "null plan");
    if (bin_size) *bin_size = p->bs;
    if (maxsub) *maxsub = p->maxsub;
    return CMT_OK;
}

extern "C" int cmt_set_pts(cmt_plan *p, int64_t N, const void *x, const void *y, const void *z)
{
    CMT_CHECK_ARG(p && x && y && z, "null argument");
    QuatSrc q{nullptr, nullptr, 1, 1.0, nullptr, nullptr, make_float2(0.f, 0.f), 0ULL};
    if (p->prec == 64) return set_pts_impl<double>(*p, 0, N, (const double *)x, (const double *)y, (const double *)z, q);
    return set_pts_impl<float>(*p, 0, N, (const float *)x, (const float *)y, (const float *)z, q);
}

extern "C" int cmt_set_pts_quat(cmt_plan *p, int64_t n_img, const double *inv_rot, int64_t n_pix, const double *ppr,
                                double rext)
{
    CMT_CHECK_ARG(p && inv_rot && ppr, "null argument");
    CMT_CHECK_ARG(n_img > 0 && n_pix > 0, "empty image set");
    CMT_CHECK_ARG(rext > 0, "reciprocal_extent must be positive");
    QuatSrc q{inv_rot, ppr, n_pix, rext, nullptr, nullptr, make_float2(0.f, 0.f),
              n_pix >= 2 ? magic64((unsigned long long)n_pix) : 0ULL};
    int64_t N = n_img * n_pix;
    if (p->prec == 64) return set_pts_impl<double>(*p, 1, N, nullptr, nullptr, nullptr, q);
    // FP32 plans evaluate the float64 coordinate chain in double-float arithmetic
    float2 *split = nullptr;  // pool blocks start 256-byte aligned; 80 n_img bytes keep ppr_df 16-byte aligned
    int64_t ns = 10 * n_img + 4 * n_pix;
    CMT_TRY_CUDA(cudaMallocAsync(&split, sizeof(float2) * ns, p->stream));
    k_split_quat<<<(unsigned)ceil_div(ns, 256), 256, 0, p->stream>>>(inv_rot, n_img, ppr, n_pix, split,
                                                                     split + 10 * n_img);
    if (cudaError_t e = cudaGetLastError()) {
        cudaFreeAsync(split, p->stream);
        set_error("%s:%d k_split_quat launch: %s", __FILE__, __LINE__, cudaGetErrorString(e));
        return CMT_ERR_CUDA;
    }
    double s = kPi / rext;
    float sh = (float)s;
    q.rot_df = split;
    q.ppr_df = split + 10 * n_img;
    q.scale_df = make_float2(sh, (float)(s - (double)sh));
    int rc = set_pts_impl<float>(*p, 1, N, nullptr, nullptr, nullptr, q);
    cudaFreeAsync(split, p->stream);
    return rc;
}

extern "C" int cmt_execute(cmt_plan *p, void *c, void *f, const float *support, double scale, int flags)
{
    // type 1 with real strengths accepts c == NULL: every strength is 1 (the Toeplitz
    // kernel's adjoint of ones, autocorrelation.py:141-147)
    CMT_CHECK_ARG(p && f && (c || (p->type == 1 && (flags & CMT_REAL_IN))), "null argument");
    sync_borrowed(*p);
    if (p->N <= 0) {
        set_error("execute before set_pts");
        return CMT_ERR_STATE;
    }
    if (p->type == 1) {
        if (p->prec == 64) return exec_type1<double>(*p, (const double *)c, (double *)f, support, scale, flags);
        return exec_type1<float>(*p, (const float *)c, (float *)f, support, scale, flags);
    }
    if (p->prec == 64) return exec_type2<double>(*p, (double *)c, (const double *)f, support, scale, flags);
    return exec_type2<float>(*p, (float *)c, (const float *)f, support, scale, flags);
}

extern "C" int cmt_execute_pair(cmt_plan *p, const void *fin, void *fout, const float *support, double scale)
{
    CMT_CHECK_ARG(p && fin && fout, "null argument");
    sync_borrowed(*p);
    if (p->N <= 0) {
        set_error("execute before set_pts");
        return CMT_ERR_STATE;
    }
    if (p->prec == 64) return exec_pair<double>(*p, (const double *)fin, (double *)fout, support, scale);
    return exec_pair<float>(*p, (const float *)fin, (float *)fout, support, scale);
}

// Per-launch timing of the spread / interpolation kernels.  enable != 0 creates the events
// and starts recording (at most 256 launches until the next read); 0 stops.
extern "C" int cmt_plan_profile(cmt_plan *p, int enable)
{
    CMT_CHECK_ARG(p, "null plan");
    if (enable && !p->ev[0])
        for (int i = 0; i < 2 * Plan::PROF_CAP; ++i) CMT_TRY_CUDA(cudaEventCreate(&p->ev[i]));
    p->prof = enable != 0 && p->ev[0];
    p->nev = 0;
    return CMT_OK;
}

// Read (and clear) the recorded launches: ms[i] duration, kinds[i] 1 spread / 2 interp.
extern "C" int cmt_plan_profile_read(cmt_plan *p, float *ms, int *kinds, int max, int *count)
{
    CMT_CHECK_ARG(p && count, "null argument");
    int n = std::min(p->nev, max);
    for (int i = 0; i < n; ++i) {
        CMT_TRY_CUDA(cudaEventSynchronize(p->ev[2 * i + 1]));
        float t = 0.f;
        CMT_TRY_CUDA(cudaEventElapsedTime(&t, p->ev[2 * i], p->ev[2 * i + 1]));
        if (ms) ms[i] = t;
        if (kinds) kinds[i] = p->kind[i];
    }
    *count = n;
    p->nev = 0;
    return CMT_OK;
}

extern "C" int cmt_plan_set_stream(cmt_plan *p, void *stream)
{
    CMT_CHECK_ARG(p, "null plan");
    p->stream = (cudaStream_t)stream;
    if (p->has_c2c) CMT_TRY_CUFFT(cufftSetStream(p->fft_c2c, p->stream));
    if (p->has_r2c) CMT_TRY_CUFFT(cufftSetStream(p->fft_r2c, p->stream));
    if (p->has_c2r) CMT_TRY_CUFFT(cufftSetStream(p->fft_c2r, p->stream));
    return CMT_OK;
}

extern "C" int cmt_plan_prepare_pair(cmt_plan *p)
{
    CMT_CHECK_ARG(p, "null plan");
    CMT_TRY(ensure_fft(*p, 0));
    if (!p->fine2) CMT_TRY_CUDA(cudaMalloc(&p->fine2, 2 * elem(*p) * (size_t)p->n * p->n * p->n));
    CMT_TRY(launch_pair(*p, true));
    return CMT_OK;
}

extern "C" int cmt_plan_destroy(cmt_plan *p)
{
    if (!p) return CMT_OK;
    destroy(p);
    delete p;
    return CMT_OK;
}

// ====================================================================== batches of plans

namespace cmt {

// Several independent plans (one per reconstruction, each with its own modes M, points and
// fine grid; one precision, type and kernel width) executed together: every plan's grid
// preparation, then ONE persistent spreading / interpolation launch whose CTAs take work
// items (plan, bin, offset) from a device counter across all plans, then every plan's FFT
// and deconvolution.  The batch owns the concatenated work list (rebuilt when a plan gets
// new points or new tuning) and the per-plan descriptors.
struct Batch {
    std::vector<cmt_plan *> plans;
    std::vector<int64_t> versions;
    cudaStream_t stream = nullptr;
    WorkItem *work = nullptr;
    int64_t cap_work = 0;
    int nwork = 0;
    void *inst = nullptr;       // device InstDesc array
    void *inst_host = nullptr;  // pinned staging of the descriptors
    cudaEvent_t staged = nullptr;
    int *next = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
};

__global__ void k_fill_work(WorkItem *work, int inst, const int *sub_bin, const int *sub_off, int64_t nsub)
{
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsub) work[s] = WorkItem{inst, sub_bin[s], sub_off[s]};
}

static int batch_rebuild_work(Batch &b)
{
    int64_t total = 0;
    for (auto *p : b.plans) total += p->nsub;
    CMT_CHECK_ARG(total < (1LL << 31), "batch work list too long");
    if (total > b.cap_work) {
        cudaFree(b.work);
        b.work = nullptr;
        b.cap_work = 0;
        CMT_TRY_CUDA(cudaMalloc(&b.work, sizeof(WorkItem) * std::max<int64_t>(total, 1)));
        b.cap_work = total;
    }
    int64_t base = 0;
    for (size_t i = 0; i < b.plans.size(); ++i) {
        Plan &p = *b.plans[i];
        if (p.nsub > 0)
            k_fill_work<<<ceil_div(p.nsub, 256), 256, 0, b.stream>>>(b.work + base, (int)i, p.sub_bin, p.sub_off,
                                                                       p.nsub);
        CMT_LAUNCH_CHECK();
        base += p.nsub;
        b.versions[i] = p.points_of ? p.points_of->pts_version : p.pts_version;
    }
    b.nwork = (int)total;
    return CMT_OK;
}

template <typename T>
static int batch_execute(Batch &b, void *const *c, void *const *f, const float *const *support,
                         const double *scale, int flags)
{
    const Plan &p0 = *b.plans[0];
    const bool t1 = p0.type == 1;
    const bool real_in = flags & CMT_REAL_IN, real_out = flags & CMT_REAL_OUT;
    const bool cplx = t1 ? !real_in : !real_out;
    const int K = (int)b.plans.size();
    for (int i = 0; i < K; ++i) {
        Plan &p = *b.plans[i];
        sync_borrowed(p);
        CMT_CHECK_ARG(p.N > 0, "batch plan %d has no points", i);
        CMT_CHECK_ARG(c[i] || (t1 && real_in), "batch plan %d: null values", i);
        CMT_CHECK_ARG(f[i], "batch plan %d: null modes", i);
    }
    bool stale = false;
    for (int i = 0; i < K; ++i) {
        Plan &p = *b.plans[i];
        sync_borrowed(p);  // a derived plan follows its source's points and tuning
        const int64_t v = p.points_of ? p.points_of->pts_version : p.pts_version;
        stale |= b.versions[i] != v;
    }
    std::vector<cudaStream_t> own(K);
    for (int i = 0; i < K; ++i) {
        own[i] = b.plans[i]->stream;
        CMT_TRY(cmt_plan_set_stream(b.plans[i], b.stream));
    }
    int rc = CMT_OK;
    auto run = [&]() -> int {
        if (stale) CMT_TRY(batch_rebuild_work(b));
        // 1. every plan's grid preparation
        size_t smem = 0;
        for (int i = 0; i < K; ++i) {
            Plan &p = *b.plans[i];
            if (t1) CMT_TRY(exec_type1<T>(p, (const T *)c[i], (T *)f[i], support ? support[i] : nullptr,
                                          scale ? scale[i] : 1.0, flags, PH_PRE));
            else CMT_TRY(exec_type2<T>(p, (T *)c[i], (const T *)f[i], support ? support[i] : nullptr, 1.0, flags,
                                       PH_PRE));
            smem = std::max(smem, batch_smem(p, t1, cplx));
        }
        // 2. the descriptors and one persistent launch over all plans' subproblems
        CMT_TRY_CUDA(cudaEventSynchronize(b.staged));  // the previous call's copy has been read
        InstDesc<T> *h = (InstDesc<T> *)b.inst_host;
        for (int i = 0; i < K; ++i) {
            Plan &p = *b.plans[i];
            const int rs = cplx ? p.n : p.n + 2;
            h[i] = InstDesc<T>{p.bin_count, p.bin_start, p.perm, p.ux, p.uy, p.uz,
                               t1 ? (const void *)c[i] : (const void *)p.fine, t1 ? p.fine : c[i], geom(p, rs)};
        }
        CMT_TRY_CUDA(cudaMemcpyAsync(b.inst, h, sizeof(InstDesc<T>) * K, cudaMemcpyHostToDevice, b.stream));
        CMT_TRY_CUDA(cudaEventRecord(b.staged, b.stream));
        CMT_TRY_CUDA(cudaMemsetAsync(b.next, 0, sizeof(int), b.stream));
        if (b.timed) CMT_TRY_CUDA(cudaEventRecord(b.ev0, b.stream));
        if (b.nwork > 0) {
            // derived plans keep their extended register window when the whole batch is derived
            bool ext = t1 && !cplx && p0.w <= 7;
            for (int i = 0; i < K; ++i) ext = ext && b.plans[i]->spread_ext && b.plans[i]->spread_tab;
            if (t1)
                CMT_TRY(launch_spread_batch(p0.prec, cplx, ext, p0.w, b.work, b.nwork, b.inst, p0.beta, b.next, smem,
                                            b.stream));
            else
                CMT_TRY(launch_interp_batch(p0.prec, cplx ? 0 : 2, p0.w, b.work, b.nwork, b.inst, p0.beta, b.next,
                                            smem, b.stream));
        }
        if (b.timed) CMT_TRY_CUDA(cudaEventRecord(b.ev1, b.stream));
        // 3. every plan's FFT and deconvolution (type 1)
        if (t1)
            for (int i = 0; i < K; ++i)
                CMT_TRY(exec_type1<T>(*b.plans[i], (const T *)c[i], (T *)f[i], support ? support[i] : nullptr,
                                      scale ? scale[i] : 1.0, flags, PH_POST));
        return CMT_OK;
    };
    rc = run();
    for (int i = 0; i < K; ++i) cmt_plan_set_stream(b.plans[i], own[i]);
    return rc;
}

}  // namespace cmt

struct cmt_batch : cmt::Batch {};

extern "C" int cmt_batch_destroy(cmt_batch *b);

extern "C" int cmt_batch_create(int n_plans, cmt_plan *const *plans, void *stream, cmt_batch **out)
{
    CMT_CHECK_ARG(out && plans && n_plans >= 1, "bad argument");
    *out = nullptr;
    const Plan &a = *plans[0];
    for (int i = 0; i < n_plans; ++i) {
        CMT_CHECK_ARG(plans[i], "null plan %d", i);
        const Plan &p = *plans[i];
        CMT_CHECK_ARG(p.type == a.type && p.prec == a.prec && p.w == a.w && p.isign == a.isign && p.beta == a.beta,
                      "plan %d differs from plan 0 in type, precision, kernel width or sign", i);
    }
    CMT_CHECK_ARG(a.w >= 2 && a.w <= 8, "batches need a kernel width in 2..8 (eps >= 1e-7), got %d", a.w);
    cmt_batch *b = new (std::nothrow) cmt_batch();
    if (!b) return CMT_ERR_OOM;
    b->plans.assign(plans, plans + n_plans);
    b->versions.assign(n_plans, -1);
    b->stream = (cudaStream_t)stream;
    size_t desc = sizeof(InstDesc<double>) * n_plans;
    int rc = CMT_OK;
    if (cudaMalloc(&b->inst, desc) != cudaSuccess || cudaMallocHost(&b->inst_host, desc) != cudaSuccess ||
        cudaMalloc(&b->next, sizeof(int)) != cudaSuccess || cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
        set_error("batch allocation failed");
        rc = CMT_ERR_OOM;
    }
    if (rc == CMT_OK) rc = cudaEventRecord(b->staged, b->stream) == cudaSuccess ? CMT_OK : CMT_ERR_CUDA;
    if (rc != CMT_OK) {
        cmt_batch_destroy(b);
        return rc;
    }
    *out = b;
    return CMT_OK;
}

// c[i], f[i]: plan i's values and modes, as for cmt_execute (type 1: c in, f out; type 2:
// f in, c out); support / scale: per-plan arrays or NULL.  Stream-ordered on the batch's
// stream (each plan's own stream is restored afterwards).
extern "C" int cmt_batch_execute(cmt_batch *b, void *const *c, void *const *f, const float *const *support,
                                 const double *scale, int flags)
{
    CMT_CHECK_ARG(b && c && f, "null argument");
    return b->plans[0]->prec == 64 ? batch_execute<double>(*b, c, f, support, scale, flags)
                                   : batch_execute<float>(*b, c, f, support, scale, flags);
}

// Time (ms) of the last batched kernel launch when timing is on (CUDA events on the batch
// stream; synchronises with it).
extern "C" int cmt_batch_profile(cmt_batch *b, int enable)
{
    CMT_CHECK_ARG(b, "null batch");
    b->timed = enable != 0;
    return CMT_OK;
}

extern "C" int cmt_batch_last_ms(cmt_batch *b, float *ms, int64_t *n_work)
{
    CMT_CHECK_ARG(b && ms, "null argument");
    *ms = 0.f;
    if (n_work) *n_work = b->nwork;
    if (!b->timed) return CMT_OK;
    CMT_TRY_CUDA(cudaEventSynchronize(b->ev1));
    CMT_TRY_CUDA(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    return CMT_OK;
}

extern "C" int cmt_batch_destroy(cmt_batch *b)
{
    if (!b) return CMT_OK;
    if (b->staged) cudaEventSynchronize(b->staged);
    cudaFree(b->work);
    cudaFree(b->inst);
    cudaFreeHost(b->inst_host);
    cudaFree(b->next);
    if (b->staged) cudaEventDestroy(b->staged);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
    return CMT_OK;
}

extern "C" int cmt_inverse_rotations(const float *quat, int64_t n, double *out, void *stream)
{
    CMT_CHECK_ARG(quat && out && n >= 0, "bad argument");
    if (n == 0) return CMT_OK;
    k_inverse_rotations<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(quat, n, out);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}
