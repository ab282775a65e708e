// Orientation matching: weighted euclidean distances between data images and model slices
// with a running top-k / argmin epilogue (cmtip/alignment/align.py:68-132).
//
//   d(r, i)^2 = || w . (s_r m_r - x_i) ||^2 = s_r^2 |w m_r|^2 + |w x_i|^2 - 2 s_r (w m_r).(w x_i)
//
// (weights w multiply both operands as in align.py:127-128; s_r = std(data) / std(model batch)
// of the reference batch holding r, align.py:122-124).  For the argmin over r only
// g(r, i) = s_r^2 |w m_r|^2 - 2 s_r (w m_r).(w x_i) matters, so the kernels compute the
// cross term as a GEMM and keep, per image, the TOPK best g in registers; the distance
// matrix never reaches HBM.  A merge kernel then re-scores those candidates exactly
// (FP64 accumulation of the FP32 inputs) and picks the argmin (first index on ties, as
// numpy's argmin), counting near-ties whose best two distances differ by less than one
// FP32 rounding.
//
// Forms: BF16 operands on the 5th-generation tensor cores (tcgen05.mma, TMEM accumulators,
// TMA loads with 128B swizzle, warp-specialised pipeline); plain FP32 and plain FP64
// SIMT kernels (the comparison forms).
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "cmt_common.cuh"
#include "df.cuh"

namespace cmt {

constexpr int TOPK = 8;
constexpr float SCORE_INF = 3.0e38f;

__device__ __forceinline__ void topk_insert(float (&s)[TOPK], int (&id)[TOPK], float g, int r)
{
    if (!(g < s[TOPK - 1])) return;
    s[TOPK - 1] = g;
    id[TOPK - 1] = r;
#pragma unroll
    for (int k = TOPK - 1; k > 0; --k) {
        if (s[k] < s[k - 1]) {
            float ts = s[k];
            s[k] = s[k - 1];
            s[k - 1] = ts;
            int ti = id[k];
            id[k] = id[k - 1];
            id[k - 1] = ti;
        }
    }
}

// ------------------------------------------------------------------ operand preparation

__device__ __forceinline__ void block_sum3(double &a, double &b, double &c)
{
    __shared__ double sh[3][32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
        sh[2][wid] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0, tb = 0, tc = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            ta += sh[0][i];
            tb += sh[1][i];
            tc += sh[2][i];
        }
        a = ta;
        b = tb;
        c = tc;
    }
}

// One CTA per row: sum and sum of squares of the raw values (batch standard deviations).
template <typename TI>
__global__ void k_row_stats(const TI *v, int64_t n_pix, double *rsum, double *rsq)
{
    int64_t row = blockIdx.x;
    const TI *src = v + row * n_pix;
    double a = 0.0, b = 0.0, c = 0.0;
    if constexpr (sizeof(TI) == 4) {  // float rows: compensated float sums (Dot2), FP64 per thread
        Dot2 sa{0.f, 0.f}, sb{0.f, 0.f};
        for (int64_t p = threadIdx.x; p < n_pix; p += blockDim.x) {
            const float x = src[p];
            dot2_add1(sa, x);
            dot2_add(sb, x, x);
        }
        a = dot2_value(sa);
        b = dot2_value(sb);
    } else {
        for (int64_t p = threadIdx.x; p < n_pix; p += blockDim.x) {
            double x = (double)src[p];
            a += x;
            b += x * x;
        }
    }
    block_sum3(a, b, c);
    if (threadIdx.x == 0) {
        rsum[row] = a;
        rsq[row] = b;
    }
}

// Centre: c_p = mean_i w_p x_ip.  Distances are unchanged when both operands are shifted by
// the same vector; shifting by the mean weighted image removes the component all images
// share (the radial intensity fall-off), so the cross term no longer cancels against
// |x|^2 and reduced-precision operands keep their accuracy on the distance itself.
template <typename TI>
__global__ void k_col_mean(const TI *x, const double *w, int64_t n_img, int64_t n_pix, double *c, float *cf)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pix) return;
    double s = 0.0;
    if constexpr (sizeof(TI) == 4) {  // the column sum in float error-free arithmetic (FP64 is slow)
        Dot2 d{0.f, 0.f};
        for (int64_t i = 0; i < n_img; ++i) dot2_add1(d, x[i * n_pix + p]);
        s = dot2_value(d);
    } else {
        for (int64_t i = 0; i < n_img; ++i) s += (double)x[i * n_pix + p];
    }
    c[p] = w[p] * s / (double)n_img;
    cf[p] = (float)c[p];
}

template <typename TO> __device__ __forceinline__ TO to_op(double v) { return (TO)v; }
template <> __device__ __forceinline__ __nv_bfloat16 to_op<__nv_bfloat16>(double v) { return __double2bfloat16(v); }
template <typename TO> __device__ __forceinline__ double from_op(TO v) { return (double)v; }
template <> __device__ __forceinline__ double from_op<__nv_bfloat16>(__nv_bfloat16 v) { return (double)__bfloat162float(v); }

// One CTA per row: u = scale_row * w . v - c (FP64), written as the GEMM operand row.
// terms == 1: [u] (Kp wide).  terms == 3 (bf16 only): the split u = hi + lo in bf16 laid
// out along K so that one GEMM yields hi.hi' + hi.lo' + lo.hi':
//   side 0 (images):     [hi, hi, lo]      side 1 (references): [hi, lo, hi]
// Also |u|^2 (of the unrounded values) when norm2 is given.
template <typename TI, typename TO>
__global__ void k_build_op(const TI *v, const double *w, const double *c, const float2 *wdf, const float *cf,
                           const double *scale, int64_t n_pix, int Kp, int terms, int side, TO *op, double *norm2)
{
    int64_t row = blockIdx.x;
    const TI *src = v + row * n_pix;
    const int64_t ld = (int64_t)Kp * terms;
    TO *dst = op + row * ld;
    double sr = scale ? scale[row] : 1.0;
    double a = 0.0, b = 0.0, cc = 0.0;
    if constexpr (std::is_same<TO, __nv_bfloat16>::value && sizeof(TI) == 4) {
        // BF16 operands (8 significant bits) from float inputs: u in FP32 (the FP64 pipe is
        // slow), rounded once to BF16; |u|^2 by compensated float sums
        const float srf = (float)sr;
        Dot2 nn{0.f, 0.f};
        for (int64_t p = threadIdx.x; p < Kp; p += blockDim.x) {
            float u = 0.f;
            if (p < n_pix) u = fmaf(srf * wdf[p].x, src[p], -cf[p]);
            dot2_add(nn, u, u);
            const __nv_bfloat16 hi = __float2bfloat16(u);
            if (terms == 1) {
                dst[p] = hi;
            } else {
                const __nv_bfloat16 lo = __float2bfloat16(u - __bfloat162float(hi));
                dst[p] = hi;
                dst[Kp + p] = side == 0 ? hi : lo;
                dst[2 * (int64_t)Kp + p] = side == 0 ? lo : hi;
            }
        }
        a = dot2_value(nn);
    } else {
        for (int64_t p = threadIdx.x; p < Kp; p += blockDim.x) {
            double u = 0.0;
            if (p < n_pix) u = sr * w[p] * (double)src[p] - c[p];
            a += u * u;
            TO hi = to_op<TO>(u);
            if (terms == 1) {
                dst[p] = hi;
            } else {
                TO lo = to_op<TO>(u - from_op<TO>(hi));
                dst[p] = hi;
                dst[Kp + p] = side == 0 ? hi : lo;
                dst[2 * (int64_t)Kp + p] = side == 0 ? lo : hi;
            }
        }
    }
    block_sum3(a, b, cc);
    if (threadIdx.x == 0 && norm2) norm2[row] = a;
}

// score coefficients: g = ca_r - cb_r * (a_r . b_i) with ca_r = |a_r|^2, cb_r = 2; padding
// columns get +inf so they never enter a candidate list
__global__ void k_score_coeffs(const double *norm2, int64_t n_ref, int64_t n_ref_pad, float *ca, float *cb)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_ref_pad) return;
    ca[r] = r < n_ref ? (float)norm2[r] : SCORE_INF;
    cb[r] = r < n_ref ? 2.0f : 0.0f;
}

// Per-batch scale s_b = std(data) / std(model batch b) (numpy std, ddof 0), per reference.
// Single CTA, fixed summation order.
__global__ void k_batch_scales(const double *dsum, const double *dsq, int64_t n_img, const double *msum,
                               const double *msq, int64_t n_ref, int nbatches, int64_t n_pix, double *sref,
                               double *stats)
{
    __shared__ double sh[2][1024];
    int t = threadIdx.x;
    // data std over all images
    double a = 0, b = 0;
    for (int64_t i = t; i < n_img; i += blockDim.x) {
        a += dsum[i];
        b += dsq[i];
    }
    sh[0][t] = a;
    sh[1][t] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (t < o) {
            sh[0][t] += sh[0][t + o];
            sh[1][t] += sh[1][t + o];
        }
        __syncthreads();
    }
    double nd = (double)n_img * n_pix;
    double dmean = sh[0][0] / nd;
    double dstd = sqrt(fmax(sh[1][0] / nd - dmean * dmean, 0.0));
    __syncthreads();
    int64_t quot = n_ref / nbatches;
    for (int bt = 0; bt < nbatches; ++bt) {
        a = 0;
        b = 0;
        for (int64_t r = bt * quot + t; r < (bt + 1) * quot; r += blockDim.x) {
            a += msum[r];
            b += msq[r];
        }
        sh[0][t] = a;
        sh[1][t] = b;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (t < o) {
                sh[0][t] += sh[0][t + o];
                sh[1][t] += sh[1][t + o];
            }
            __syncthreads();
        }
        double nm = (double)quot * n_pix;
        double mmean = sh[0][0] / nm;
        double mstd = sqrt(fmax(sh[1][0] / nm - mmean * mmean, 0.0));
        double s = dstd / mstd;
        if (t == 0 && stats) stats[bt] = s;
        for (int64_t r = bt * quot + t; r < (bt + 1) * quot; r += blockDim.x) sref[r] = s;
        __syncthreads();
    }
    if (t == 0 && stats) stats[nbatches] = dstd;
}

// ------------------------------------------------------------------ plain SIMT forms

// 64 images x 64 references per CTA, 16x16 threads with 4x4 register tiles.
// Output: per (reference tile, image) the TOPK best scores.
template <typename T>
__global__ void __launch_bounds__(256) k_dist_simt(const T *X, const T *Y, int n_img, int n_ref, int Kp,
                                                   const float *ca, const float *cb, float *pscore, int *pidx,
                                                   int nimg_pad)
{
    constexpr int KC = 16;
    __shared__ T Xs[KC][64 + 1];
    __shared__ T Ys[KC][64 + 1];
    __shared__ float S[64][64 + 1];
    int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    int i0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
    for (int k0 = 0; k0 < Kp; k0 += KC) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int idx = tid + 256 * j;
            int row = idx / KC, k = idx % KC;
            int gi = i0 + row, gr = r0 + row;
            Xs[k][row] = gi < n_img ? X[(int64_t)gi * Kp + k0 + k] : T(0);
            Ys[k][row] = gr < n_ref ? Y[(int64_t)gr * Kp + k0 + k] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KC; ++kk) {
            T av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = Xs[kk][ty * 4 + a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Ys[kk][tx * 4 + b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            int r = r0 + tx * 4 + b;
            S[ty * 4 + a][tx * 4 + b] = r < n_ref ? (float)((double)ca[r] - (double)cb[r] * (double)acc[a][b]) : SCORE_INF;
        }
    __syncthreads();
    if (tid < 64) {
        float s[TOPK];
        int id[TOPK];
#pragma unroll
        for (int k = 0; k < TOPK; ++k) {
            s[k] = SCORE_INF;
            id[k] = -1;
        }
        for (int c = 0; c < 64; ++c) topk_insert(s, id, S[tid][c], r0 + c);
        int64_t o = ((int64_t)blockIdx.y * nimg_pad + i0 + tid) * TOPK;
#pragma unroll
        for (int k = 0; k < TOPK; ++k) {
            pscore[o + k] = s[k];
            pidx[o + k] = id[k];
        }
    }
}

// ------------------------------------------------------------------ tcgen05 BF16 form

constexpr int TC_BM = 128;   // images per tile (TMEM lanes)
constexpr int TC_BN = 256;   // default references per tile (TMEM columns per accumulator; 128 or 256)
constexpr int TC_BK = 64;    // K per stage: one 128-byte swizzle row of bf16
constexpr int TC_STAGES = 4;  // default TMA ring depth
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;
constexpr int TC_THREADS = 192;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2-5 epilogue
// shared memory of a (BN, STAGES) instantiation: the TMA ring, 1 KB alignment, barriers
constexpr int tc_smem(int bn, int stages) { return stages * (TC_A_BYTES + bn * TC_BK * 2) + 1024 + 256; }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Bounded wait on an mbarrier phase: gives up after limit_ns of %globaltimer (or, with an
// abort flag, as soon as another role has given up) and reports false; the caller records
// the timeout and unwinds.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                          uint64_t limit_ns)
{
    uint64_t t0 = 0;
    for (uint32_t it = 0;; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & 255) == 0) {
            if (abort_flag && *abort_flag) return false;
            uint64_t t = globaltimer();
            if (t0 == 0) t0 = t;
            else if (t - t0 > limit_ns) {
                if (abort_flag) *abort_flag = 1;
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c0, int c1)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            dst),
        "l"((uint64_t)map), "r"(bar), "r"(c0), "r"(c1)
        : "memory");
}

// K-major operand, 128-byte swizzle, 8-row core groups 1024 bytes apart (tcgen05 smem descriptor)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;             // SWIZZLE_128B
    return d;
}

// kind::f16 instruction descriptor: BF16 A/B, FP32 D, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accum)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// One distance problem of a launch: its image-major (image tile, reference tile) units are
// [ustart, ustart + n_itiles * n_rtiles) of the launch's unit list.
struct TcProblem {
    long long ustart;
    int n_rtiles;
    int KB;      // K blocks of TC_BK per unit (padded pixels x terms / TC_BK)
    int maxseg;  // most image tiles of this problem one CTA touches (output segments per CTA)
    const float *ca, *cb;
    float *pscore;  // [cta][segment][row][TOPK]
    int *pidx;
};

constexpr int TC_MAXP = 16;  // problems per launch

struct TcGroup {
    CUtensorMap tmA[TC_MAXP], tmB[TC_MAXP];
    TcProblem p[TC_MAXP];
    int np;
    const long long *cta_u;     // CTA c owns units [cta_u[c], cta_u[c + 1])
    unsigned long long wait_ns;  // limit of every pipeline wait
    int stall_loads;             // test of the timeout path: the producer issues no loads
};

// advance p to the problem holding unit u (units are visited in increasing order)
__device__ __forceinline__ int problem_of(const TcGroup &g, long long u, int p)
{
    while (p + 1 < g.np && u >= g.p[p + 1].ustart) ++p;
    return p;
}

// Persistent over the units of one or more problems (an instance each: its own images,
// references, pixel count, score coefficients and outputs): CTA c owns a contiguous range
// of the concatenated unit list, balanced by cost on the host, keeps each image's running
// top-k across the reference tiles in the epilogue threads' registers and writes it once
// per image tile it touched.
template <int BN, int STAGES>
__global__ void __launch_bounds__(TC_THREADS, 1) k_dist_tc(const __grid_constant__ TcGroup g, int *err)
{
    constexpr int B_BYTES = BN * TC_BK * 2, STAGE_BYTES = TC_A_BYTES + B_BYTES;
    constexpr uint32_t TMEM_COLS = 2 * BN;  // two accumulators of BN columns
    extern __shared__ unsigned char smem_raw[];
    uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    unsigned char *gbase = smem_raw + (base - smem_u32(smem_raw));
    uint32_t sA0 = base, sB0 = base + STAGES * TC_A_BYTES;
    uint64_t *bars = reinterpret_cast<uint64_t *>(gbase + STAGES * STAGE_BYTES);
    // bars: full[S], empty[S], accf[2], acce[2], drain
    uint32_t bar0 = smem_u32(bars);
    auto full_b = [&](int s) { return bar0 + 8u * s; };
    auto empty_b = [&](int s) { return bar0 + 8u * (STAGES + s); };
    auto accf_b = [&](int b) { return bar0 + 8u * (2 * STAGES + b); };
    auto acce_b = [&](int b) { return bar0 + 8u * (2 * STAGES + 2 + b); };
    const uint32_t drain_b = bar0 + 8u * (2 * STAGES + 4);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(gbase + STAGES * STAGE_BYTES + 8 * (2 * STAGES + 5));
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long u0 = g.cta_u[blockIdx.x], u1 = g.cta_u[blockIdx.x + 1];
    if (u0 >= u1) return;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full_b(s), 1);
            mbar_init(empty_b(s), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(accf_b(b), 1);
            mbar_init(acce_b(b), 4);
        }
        mbar_init(drain_b, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int s = 0;
            uint32_t ph = 0;
            bool ok = true;
            int p = 0;
            unsigned used = 0;           // stages with a load issued
            uint32_t used_ph[STAGES];  // the phase of each stage's last load
            for (long long u = u0; u < u1 && ok && !g.stall_loads; ++u) {
                p = problem_of(g, u, p);
                const long long lu = u - g.p[p].ustart;
                const int m = (int)(lu / g.p[p].n_rtiles), t = (int)(lu % g.p[p].n_rtiles);
                const int KB = g.p[p].KB;
                for (int kb = 0; kb < KB; ++kb) {
                    if (!mbar_wait(empty_b(s), ph ^ 1, abort_flag, g.wait_ns)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(full_b(s), STAGE_BYTES);
                    tma_load_2d(sA0 + s * TC_A_BYTES, &g.tmA[p], full_b(s), kb * TC_BK, m * TC_BM);
                    tma_load_2d(sB0 + s * B_BYTES, &g.tmB[p], full_b(s), kb * TC_BK, t * BN);
                    used |= 1u << s;
                    used_ph[s] = ph;
                    if (++s == STAGES) {
                        s = 0;
                        ph ^= 1;
                    }
                }
            }
            // before the CTA can exit, every load this thread issued has landed (on the normal
            // path the MMA warp has already consumed them; after a timeout they may still be
            // in flight): a bounded wait per stage that does not stop on the abort flag
            for (int st = 0; st < STAGES; ++st)
                if ((used >> st) & 1u)
                    if (!mbar_wait(full_b(st), used_ph[st], nullptr, g.wait_ns)) ok = false;
            if (!ok) atomicOr(err, 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(TC_BM, BN);
            int s = 0;
            uint32_t ph = 0;
            bool ok = true;
            int lt = 0, p = 0;
            for (long long u = u0; u < u1 && ok; ++u, ++lt) {
                p = problem_of(g, u, p);
                const int KB = g.p[p].KB;
                int b = lt & 1;
                if (!mbar_wait(acce_b(b), ((lt >> 1) & 1) ^ 1, abort_flag, g.wait_ns)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                uint32_t dt = tmem + (uint32_t)(b * BN);
                for (int kb = 0; kb < KB; ++kb) {
                    if (!mbar_wait(full_b(s), ph, abort_flag, g.wait_ns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    uint64_t ad = sw128_desc(sA0 + s * TC_A_BYTES), bd = sw128_desc(sB0 + s * B_BYTES);
#pragma unroll
                    for (int k = 0; k < TC_BK / 16; ++k)
                        umma_bf16(dt, ad + 2 * k, bd + 2 * k, idesc, (kb | k) != 0);
                    umma_commit(empty_b(s));
                    if (++s == STAGES) {
                        s = 0;
                        ph ^= 1;
                    }
                }
                if (ok) umma_commit(accf_b(b));
            }
            // every MMA this thread issued has completed before TMEM can be released (after a
            // timeout some may still run): one more commit, and a bounded wait on it
            umma_commit(drain_b);
            if (!mbar_wait(drain_b, 0, nullptr, g.wait_ns)) ok = false;
            if (!ok) atomicOr(err, 1);
        }
    } else {
        // epilogue: warps 2..5, TMEM lane quarter = warp % 4
        const int q = warp & 3;
        const int row = q * 32 + lane;
        float s[TOPK];
        int id[TOPK];
#pragma unroll
        for (int k = 0; k < TOPK; ++k) {
            s[k] = SCORE_INF;
            id[k] = -1;
        }
        int lt = 0;
        int cur_p = problem_of(g, u0, 0);
        // the first image tile of problem p this CTA touches
        auto first_tile = [&](int p) {
            const long long ub = u0 > g.p[p].ustart ? u0 : g.p[p].ustart;
            return (int)((ub - g.p[p].ustart) / g.p[p].n_rtiles);
        };
        int cur_m = first_tile(cur_p), m_first = cur_m;
        bool ok = true;
        auto flush = [&](int p, int m) {
            const TcProblem &pr = g.p[p];
            long long o = (((long long)blockIdx.x * pr.maxseg + (m - m_first)) * TC_BM + row) * TOPK;
#pragma unroll
            for (int k = 0; k < TOPK; ++k) {
                pr.pscore[o + k] = s[k];
                pr.pidx[o + k] = id[k];
                s[k] = SCORE_INF;
                id[k] = -1;
            }
        };
        for (long long u = u0; u < u1; ++u, ++lt) {
            const int p = problem_of(g, u, cur_p);
            const long long lu = u - g.p[p].ustart;
            const int m = (int)(lu / g.p[p].n_rtiles), t = (int)(lu % g.p[p].n_rtiles);
            if (p != cur_p || m != cur_m) {
                flush(cur_p, cur_m);
                if (p != cur_p) m_first = first_tile(p);
                cur_p = p;
                cur_m = m;
            }
            const float *ca = g.p[p].ca, *cb = g.p[p].cb;
            int b = lt & 1;
            if (!mbar_wait(accf_b(b), (lt >> 1) & 1, abort_flag, g.wait_ns)) {
                ok = false;
                break;
            }
            tc_fence_after();
            uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN);
            const int rbase = t * BN;
#pragma unroll 1
            for (int c = 0; c < BN / 32; ++c) {
                uint32_t v[32];
                tmem_ld32(tbase + c * 32, v);
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    int r = rbase + c * 32 + j;
                    float g = __ldg(ca + r) - __ldg(cb + r) * __uint_as_float(v[j]);
                    topk_insert(s, id, g, r);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce_b(b));
        }
        if (ok) flush(cur_p, cur_m);
        else if (lane == 0) atomicOr(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// ------------------------------------------------------------------ merge + exact re-scoring

__global__ void k_split_weights(const double *w, int64_t n, float2 *out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DF d = df_from(w[i]);
    out[i] = make_float2(d.hi, d.lo);
}

struct SegInfo {
    int mode;       // 0: SIMT layout [ref tile][image]; 1: tcgen05 layout [cta][seg][row]
    int nseg;       // mode 0: reference tiles
    int nimg_pad;   // mode 0
    int n_ref;                    // candidates outside [0, n_ref) are ignored
    long long ustart, G;          // mode 1: the problem's first unit, CTAs of the launch
    int n_rtiles, maxseg;
    const long long *cta_u;       // mode 1: CTA c owned units [cta_u[c], cta_u[c + 1])
};

// One warp per image.  T: type of the raw model / data values (float or double).
template <typename T>
__global__ void k_merge_rescore(SegInfo si, const float *pscore, const int *pidx, int n_img, const T *model,
                                const T *data, const double *w, const float2 *wdf, const double *sref,
                                int64_t n_pix, int *best_idx, double *best_d, double *second_d, int *near_tie)
{
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n_img) return;
    const int i = warp;
    float s[TOPK];
    int id[TOPK];
#pragma unroll
    for (int k = 0; k < TOPK; ++k) {
        s[k] = SCORE_INF;
        id[k] = -1;
    }
    // a list is read only as far as its valid entries go: after a timed-out distance
    // launch the lists hold whatever the buffers held, and no index outside [0, n_ref) may
    // reach the re-scoring's model reads
    auto take = [&](long long o) {
        for (int k = 0; k < TOPK; ++k) {
            int r = pidx[o + k];
            if (r < 0 || r >= si.n_ref) break;
            topk_insert(s, id, pscore[o + k], r);
        }
    };
    if (si.mode == 0) {
        for (int t = lane; t < si.nseg; t += 32) take(((long long)t * si.nimg_pad + i) * TOPK);
    } else {
        int m = i / TC_BM, row = i % TC_BM;
        long long ub = si.ustart + (long long)m * si.n_rtiles, ue = ub + si.n_rtiles;
        for (long long c = lane; c < si.G; c += 32) {
            long long c0 = si.cta_u[c], c1 = si.cta_u[c + 1];
            if (c0 >= c1 || c1 <= ub || c0 >= ue) continue;
            int seg = m - (int)(((c0 > si.ustart ? c0 : si.ustart) - si.ustart) / si.n_rtiles);
            take(((c * si.maxseg + seg) * TC_BM + row) * TOPK);
        }
    }
    // warp-wide merge of the 32 sorted lists: TOPK rounds of (score, index) minimum
    int cand[TOPK];
    int head = 0;
    for (int k = 0; k < TOPK; ++k) {
        float hs = SCORE_INF;
        int hi = 0x7fffffff;
#pragma unroll
        for (int j = 0; j < TOPK; ++j)
            if (j == head) {
                hs = s[j];
                hi = id[j] < 0 ? 0x7fffffff : id[j];
            }
        float bs = hs;
        int bi = hi;
        for (int o = 16; o > 0; o >>= 1) {
            float os = __shfl_xor_sync(0xffffffffu, bs, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (os < bs || (os == bs && oi < bi)) {
                bs = os;
                bi = oi;
            }
        }
        cand[k] = bi == 0x7fffffff ? -1 : bi;
        if (hi == bi && bi != 0x7fffffff && head < TOPK) ++head;
    }
    // exact distances of the candidates, d^2 = sum_p (w_p (s_r m_rp - x_ip))^2: FP64 for
    // double inputs; for float inputs double-float arithmetic (about 48 significant bits, at
    // FP32 rate), all eight candidates in one pass over the image
    const T *x = data + (int64_t)i * n_pix;
    double d2[TOPK];
    if constexpr (sizeof(T) == 4) {
        DF acc[TOPK], sr[TOPK];
        const float *mr[TOPK];
#pragma unroll
        for (int k = 0; k < TOPK; ++k) {
            const int r = cand[k] < 0 ? 0 : cand[k];
            acc[k] = DF{0.0f, 0.0f};
            sr[k] = df_from(sref[r]);
            mr[k] = reinterpret_cast<const float *>(model) + (int64_t)r * n_pix;
        }
        // two pixels per lane and step, all loads first (the loop is bound by load latency);
        // an empty candidate slot reads row 0 and is discarded below, so the loop has no
        // branch; a pixel past the end has weight 0
        for (int64_t p = lane; p < n_pix; p += 64) {
            const bool two = p + 32 < n_pix;
            const float xa = (float)x[p], xb = two ? (float)x[p + 32] : 0.0f;
            const float2 wa = wdf[p], wb = two ? wdf[p + 32] : make_float2(0.0f, 0.0f);
            float ma[TOPK], mb[TOPK];
#pragma unroll
            for (int k = 0; k < TOPK; ++k) {
                ma[k] = mr[k][p];
                mb[k] = two ? mr[k][p + 32] : 0.0f;
            }
            const DF wva{wa.x, wa.y}, wvb{wb.x, wb.y};
#pragma unroll
            for (int k = 0; k < TOPK; ++k) {
                const DF da = df_mul(df_add_f(df_mul_f(sr[k], ma[k]), -xa), wva);
                const DF db = df_mul(df_add_f(df_mul_f(sr[k], mb[k]), -xb), wvb);
                acc[k] = df_add(acc[k], df_add(df_mul(da, da), df_mul(db, db)));
            }
        }
#pragma unroll
        for (int k = 0; k < TOPK; ++k) {
            double a = df_to_double(acc[k]);
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            d2[k] = cand[k] < 0 ? INFINITY : a;
        }
    } else {
        for (int k = 0; k < TOPK; ++k) {
            d2[k] = INFINITY;
            int r = cand[k];
            if (r < 0) continue;
            const T *mr = model + (int64_t)r * n_pix;
            double sr = sref[r];
            double acc = 0.0;
            for (int64_t p = lane; p < n_pix; p += 32) {
                double dv = w[p] * (sr * (double)mr[p] - (double)x[p]);
                acc += dv * dv;
            }
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            d2[k] = acc;
        }
    }
    if (lane == 0) {
        int b1 = -1, b2 = -1;
        for (int k = 0; k < TOPK; ++k) {
            if (cand[k] < 0) continue;
            if (b1 < 0 || d2[k] < d2[b1] || (d2[k] == d2[b1] && cand[k] < cand[b1])) {
                b2 = b1;
                b1 = k;
            } else if (b2 < 0 || d2[k] < d2[b2] || (d2[k] == d2[b2] && cand[k] < cand[b2])) {
                b2 = k;
            }
        }
        double d1 = b1 >= 0 ? sqrt(d2[b1]) : INFINITY, dd2 = b2 >= 0 ? sqrt(d2[b2]) : INFINITY;
        best_idx[i] = b1 >= 0 ? cand[b1] : -1;
        best_d[i] = d1;
        second_d[i] = dd2;
        // near tie: the best two distances are within one FP32 rounding of each other
        near_tie[i] = (b2 >= 0 && dd2 - d1 <= ldexp(d1, -23)) ? 1 : 0;
    }
}

// ------------------------------------------------------------------ host object

struct Match {
    int mode = 0;  // 0 bf16 tcgen05, 1 fp32 SIMT, 2 fp64 SIMT, 3 bf16x3 tcgen05
    int terms = 1; // bf16 terms per product (3: hi.hi + hi.lo + lo.hi laid out along K)
    int64_t n_pix = 0;
    int Kp = 0;
    double *cen = nullptr;                         // mean weighted image (operand centre)
    float *cenf = nullptr;                         // the centre rounded to float (BF16 operands)
    cudaStream_t stream = nullptr;
    int num_sms = 152;
    int64_t n_img = 0, n_ref = 0, n_ref_pad = 0;
    const void *data = nullptr, *model = nullptr;  // caller-owned raw values
    double *w = nullptr;                           // owned copy of the weights
    float2 *wdf = nullptr;                         // the weights as double-float pairs
    void *opA = nullptr, *opB = nullptr;           // weighted operands (mode type)
    int64_t capA = 0, capB = 0;
    double *dsum = nullptr, *dsq = nullptr, *msum = nullptr, *msq = nullptr, *mnorm = nullptr, *sref = nullptr;
    float *ca = nullptr, *cb = nullptr;
    double *stats = nullptr;
    int nbatches = 1;
    float *pscore = nullptr;
    int *pidx = nullptr;
    int64_t cap_part = 0;
    int *err = nullptr;
    int *near = nullptr;
    double *scratch_d = nullptr;
    long long *cta_u = nullptr;  // CTA unit ranges of the last tensor-core launch (num_sms + 1)
    int64_t cap_img = 0;         // bytes of dsum / dsq
    int64_t cap_ref = 0;         // references of msum .. cb
    // optional CUDA-event timing of the stages (cmt_match_profile): set_data, set_refs,
    // the distance kernel and the re-scoring of the last calls
    bool timed = false;
    cudaEvent_t ev[7] = {};
    double wait_s = 2.0;  // limit of the tensor-core pipeline's waits
    int tile_bn = TC_BN, stages = TC_STAGES;  // reference tile and TMA ring depth (cmt_match_set_tile)
    int stall_loads = 0;  // test of the timeout path (cmt_match_stall_loads)
};

static void mark(const Match &m, int k)
{
    if (m.timed) cudaEventRecord(m.ev[k], m.stream);
}

}  // namespace cmt

struct cmt_match : cmt::Match {};

namespace cmt {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

static int make_map(CUtensorMap *map, const void *ptr, int64_t rows, int64_t Kld, int box_rows)
{
    EncodeTiledFn enc = get_encode();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled unavailable");
        return CMT_ERR_CUDA;
    }
    cuuint64_t dims[2] = {(cuuint64_t)Kld, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kld * 2};
    cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return CMT_ERR_CUDA;
    }
    return CMT_OK;
}

static size_t op_size(int mode) { return (mode == 0 || mode == 3) ? 2 : (mode == 1 ? 4 : 8); }

static int ensure(void **p, int64_t &cap, int64_t need)
{
    if (need <= cap) return CMT_OK;
    cudaFree(*p);
    *p = nullptr;
    cap = 0;
    CMT_TRY_CUDA(cudaMalloc(p, need));
    cap = need;
    return CMT_OK;
}

// operand rows u = scale . w . v - centre for the mode's operand type
static void build_op(const Match &m, const void *v, int64_t rows, const double *scale, int side, void *op,
                     double *norm2)
{
    unsigned g = (unsigned)rows;
    if (m.mode == 0 || m.mode == 3)
        k_build_op<float, __nv_bfloat16><<<g, 256, 0, m.stream>>>((const float *)v, m.w, m.cen, m.wdf, m.cenf, scale,
                                                                  m.n_pix, m.Kp, m.terms, side, (__nv_bfloat16 *)op,
                                                                  norm2);
    else if (m.mode == 1)
        k_build_op<float, float><<<g, 256, 0, m.stream>>>((const float *)v, m.w, m.cen, m.wdf, m.cenf, scale, m.n_pix,
                                                          m.Kp, 1, side, (float *)op, norm2);
    else
        k_build_op<double, double><<<g, 256, 0, m.stream>>>((const double *)v, m.w, m.cen, m.wdf, m.cenf, scale,
                                                            m.n_pix, m.Kp, 1, side, (double *)op, norm2);
}

static void row_stats(const Match &m, const void *v, int64_t rows, double *rsum, double *rsq)
{
    if (m.mode == 2)
        k_row_stats<double><<<(unsigned)rows, 256, 0, m.stream>>>((const double *)v, m.n_pix, rsum, rsq);
    else
        k_row_stats<float><<<(unsigned)rows, 256, 0, m.stream>>>((const float *)v, m.n_pix, rsum, rsq);
}

// One tensor-core launch over the matchers ms[0 .. n) (modes 0 / 3, n <= TC_MAXP), on the
// stream st: each matcher's (image tile, reference tile) units are concatenated and split
// over min(units, SMs) persistent CTAs in contiguous ranges of about equal cost (a unit
// costs its K blocks plus a constant for the epilogue), so instances of very different
// size share the GPU in one launch.  si[i] receives matcher i's segment layout for
// k_merge_rescore; the CTA ranges live in ms[0]->cta_u until its next launch.
typedef void (*TcKernel)(TcGroup, int *);

// the instantiations a matcher's tile may select: (references per tile, ring stages)
static TcKernel tc_kernel(int bn, int stages)
{
    if (bn == 256 && stages == 4) return k_dist_tc<256, 4>;
    if (bn == 256 && stages == 3) return k_dist_tc<256, 3>;
    if (bn == 128 && stages == 6) return k_dist_tc<128, 6>;
    if (bn == 128 && stages == 4) return k_dist_tc<128, 4>;
    return nullptr;
}

static int tc_launch(int n, cmt_match *const *ms, cudaStream_t st, SegInfo *si)
{
    const int bn = ms[0]->tile_bn, stages = ms[0]->stages;
    TcKernel kern = tc_kernel(bn, stages);
    CMT_CHECK_ARG(kern, "no tensor-core kernel for a %d-reference tile with %d stages", bn, stages);
    std::vector<long long> ustart(n + 1, 0), unit_cost(n);
    std::vector<int> n_rt(n), n_it(n), KB(n);
    long long cost_total = 0;
    for (int i = 0; i < n; ++i) {
        const Match &m = *ms[i];
        n_it[i] = (int)((m.n_img + TC_BM - 1) / TC_BM);
        n_rt[i] = (int)(m.n_ref_pad / bn);
        KB[i] = (int)((int64_t)m.Kp * m.terms / TC_BK);
        unit_cost[i] = KB[i] + 16;
        const long long U = (long long)n_it[i] * n_rt[i];
        ustart[i + 1] = ustart[i] + U;
        cost_total += U * unit_cost[i];
    }
    const long long U = ustart[n];
    const long long G = std::min<long long>(U, ms[0]->num_sms);
    // CTA c starts at the first unit whose preceding cost reaches c * cost_total / G
    std::vector<long long> cta(G + 1);
    {
        int i = 0;
        long long cum = 0;  // cost of the units of the problems before i
        for (long long c = 0; c < G; ++c) {
            const long long target = (long long)((__int128)c * cost_total / G);
            while (i < n - 1 && cum + (ustart[i + 1] - ustart[i]) * unit_cost[i] <= target) {
                cum += (ustart[i + 1] - ustart[i]) * unit_cost[i];
                ++i;
            }
            long long u = ustart[i] + (target - cum + unit_cost[i] - 1) / unit_cost[i];
            u = std::min(u, ustart[i + 1]);
            cta[c] = std::max(u, c ? cta[c - 1] : 0LL);
        }
        cta[G] = U;
    }
    int64_t cap = 0;
    if (!ms[0]->cta_u) {
        CMT_TRY_CUDA(cudaMalloc(&ms[0]->cta_u, sizeof(long long) * (ms[0]->num_sms + 1)));
    }
    CMT_TRY_CUDA(cudaMemcpyAsync(ms[0]->cta_u, cta.data(), sizeof(long long) * (G + 1), cudaMemcpyHostToDevice, st));
    TcGroup g;  // the parameter block (copied at launch)
    memset(&g, 0, sizeof g);
    g.np = n;
    g.cta_u = ms[0]->cta_u;
    g.wait_ns = (unsigned long long)(ms[0]->wait_s * 1e9);
    for (int i = 0; i < n; ++i) g.stall_loads |= ms[i]->stall_loads;
    for (int i = 0; i < n; ++i) {
        Match &m = *ms[i];
        int maxseg = 1;
        for (long long c = 0; c < G; ++c) {
            const long long a = std::max(cta[c], ustart[i]), b = std::min(cta[c + 1], ustart[i + 1]);
            if (a < b) maxseg = std::max<int>(maxseg, (int)((b - 1 - ustart[i]) / n_rt[i] - (a - ustart[i]) / n_rt[i] + 1));
        }
        const int64_t need = G * maxseg * TC_BM * TOPK;
        cap = m.cap_part;
        CMT_TRY(ensure((void **)&m.pscore, cap, need * 4));
        int64_t cap2 = m.cap_part;
        CMT_TRY(ensure((void **)&m.pidx, cap2, need * 4));
        m.cap_part = std::min(cap, cap2);
        const int64_t kld = (int64_t)m.Kp * m.terms;
        CMT_TRY(make_map(&g.tmA[i], m.opA, m.n_img, kld, TC_BM));
        CMT_TRY(make_map(&g.tmB[i], m.opB, m.n_ref, kld, bn));
        g.p[i] = TcProblem{ustart[i], n_rt[i], KB[i], maxseg, m.ca, m.cb, m.pscore, m.pidx};
        si[i] = SegInfo{};
        si[i].mode = 1;
        si[i].n_ref = (int)m.n_ref;
        si[i].ustart = ustart[i];
        si[i].G = G;
        si[i].n_rtiles = n_rt[i];
        si[i].maxseg = maxseg;
        si[i].cta_u = ms[0]->cta_u;
    }
    const int smem = tc_smem(bn, stages);
    CMT_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    CMT_TRY_CUDA(cudaMemsetAsync(ms[0]->err, 0, sizeof(int), st));
    kern<<<(unsigned)G, TC_THREADS, smem, st>>>(g, ms[0]->err);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

static void merge(const Match &m, const SegInfo &si, cudaStream_t st, int *best_idx, double *best_d, double *second_d,
                  int *near_tie)
{
    unsigned blocks = (unsigned)((m.n_img * 32 + 255) / 256);
    if (m.mode == 2)
        k_merge_rescore<double><<<blocks, 256, 0, st>>>(si, m.pscore, m.pidx, (int)m.n_img, (const double *)m.model,
                                                        (const double *)m.data, m.w, m.wdf, m.sref, m.n_pix, best_idx,
                                                        best_d, second_d, near_tie);
    else
        k_merge_rescore<float><<<blocks, 256, 0, st>>>(si, m.pscore, m.pidx, (int)m.n_img, (const float *)m.model,
                                                       (const float *)m.data, m.w, m.wdf, m.sref, m.n_pix, best_idx,
                                                       best_d, second_d, near_tie);
}

static int count_near(const Match &m, const int *near_tie, int *n_near)
{
    std::vector<int> h(m.n_img);
    CMT_TRY_CUDA(cudaMemcpy(h.data(), near_tie, sizeof(int) * m.n_img, cudaMemcpyDeviceToHost));
    int c = 0;
    for (int v : h) c += v;
    *n_near = c;
    return CMT_OK;
}

}  // namespace cmt

using namespace cmt;

extern "C" int cmt_match_create(int64_t n_pix, int mode, void *stream, cmt_match **out)
{
    CMT_CHECK_ARG(out, "null output");
    *out = nullptr;
    CMT_CHECK_ARG(n_pix > 0 && n_pix < (1LL << 30), "bad pixel count");
    CMT_CHECK_ARG(mode >= 0 && mode <= 3, "mode must be 0 (bf16 tensor cores), 1 (fp32), 2 (fp64) or 3 (bf16x3)");
    cmt_match *m = new (std::nothrow) cmt_match();
    if (!m) return CMT_ERR_OOM;
    m->mode = mode;
    m->terms = mode == 3 ? 3 : 1;
    m->n_pix = n_pix;
    m->Kp = (int)((n_pix + 63) / 64 * 64);
    m->stream = (cudaStream_t)stream;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaMalloc(&m->w, sizeof(double) * n_pix) != cudaSuccess || cudaMalloc(&m->cen, sizeof(double) * n_pix) != cudaSuccess ||
        cudaMalloc(&m->cenf, sizeof(float) * n_pix) != cudaSuccess ||
        cudaMalloc(&m->wdf, sizeof(float2) * n_pix) != cudaSuccess ||
        cudaMalloc(&m->err, sizeof(int) * 2) != cudaSuccess ||
        cudaMalloc(&m->stats, sizeof(double) * 1025) != cudaSuccess) {
        set_error("match allocation failed");
        return CMT_ERR_OOM;
    }
    *out = m;
    return CMT_OK;
}

// data: n_img x n_pix raw images (float for modes 0/1, double for mode 2); weights: n_pix
// float64 (generate_weights, align.py:11-24).  The data pointer is used again by run().
extern "C" int cmt_match_set_data(cmt_match *m, int64_t n_img, const void *data, const double *weights)
{
    CMT_CHECK_ARG(m && data && weights && n_img > 0, "bad argument");
    mark(*m, 0);
    m->n_img = n_img;
    m->data = data;
    CMT_TRY_CUDA(cudaMemcpyAsync(m->w, weights, sizeof(double) * m->n_pix, cudaMemcpyDeviceToDevice, m->stream));
    k_split_weights<<<(unsigned)ceil_div(m->n_pix, 256), 256, 0, m->stream>>>(m->w, m->n_pix, m->wdf);
    int64_t cap = m->capA;
    CMT_TRY(ensure(&m->opA, cap, (int64_t)op_size(m->mode) * n_img * m->Kp * m->terms));
    m->capA = cap;
    // per-image buffers are kept while large enough (a cudaFree would synchronise the device)
    int64_t capd = m->cap_img, capq = m->cap_img;
    CMT_TRY(ensure((void **)&m->dsum, capd, (int64_t)sizeof(double) * n_img));
    CMT_TRY(ensure((void **)&m->dsq, capq, (int64_t)sizeof(double) * n_img));
    m->cap_img = std::min(capd, capq);
    unsigned gp = (unsigned)ceil_div(m->n_pix, 256);
    if (m->mode == 2)
        k_col_mean<double><<<gp, 256, 0, m->stream>>>((const double *)data, m->w, n_img, m->n_pix, m->cen, m->cenf);
    else
        k_col_mean<float><<<gp, 256, 0, m->stream>>>((const float *)data, m->w, n_img, m->n_pix, m->cen, m->cenf);
    row_stats(*m, data, n_img, m->dsum, m->dsq);
    build_op(*m, data, n_img, nullptr, 0, m->opA, nullptr);
    CMT_LAUNCH_CHECK();
    mark(*m, 1);
    return CMT_OK;
}

// model: n_ref x n_pix raw model slices (unscaled); references split into nbatches equal
// batches for the std scaling (n_ref must be a multiple of nbatches, align.py:96-101).
extern "C" int cmt_match_set_refs(cmt_match *m, int64_t n_ref, const void *model, int nbatches)
{
    CMT_CHECK_ARG(m && model && n_ref > 0, "bad argument");
    CMT_CHECK_ARG(nbatches >= 1 && nbatches <= 1024 && n_ref % nbatches == 0,
                  "n_ref must be a positive multiple of nbatches (<= 1024)");
    CMT_CHECK_ARG(m->n_img > 0, "set_data before set_refs");
    mark(*m, 2);
    m->n_ref = n_ref;
    m->model = model;
    m->nbatches = nbatches;
    int64_t tile = (m->mode == 0 || m->mode == 3) ? TC_BN : 64;
    m->n_ref_pad = (n_ref + tile - 1) / tile * tile;
    int64_t cap = m->capB;
    CMT_TRY(ensure(&m->opB, cap, (int64_t)op_size(m->mode) * n_ref * m->Kp * m->terms));
    m->capB = cap;
    // per-reference buffers are kept while large enough (a cudaFree would synchronise the device)
    if (m->n_ref_pad > m->cap_ref) {
        void *bufs[] = {m->msum, m->msq, m->mnorm, m->sref, m->ca, m->cb};
        for (void *b : bufs) cudaFree(b);
        m->msum = m->msq = m->mnorm = m->sref = nullptr;
        m->ca = m->cb = nullptr;
        m->cap_ref = 0;
        CMT_TRY_CUDA(cudaMalloc(&m->msum, sizeof(double) * m->n_ref_pad));
        CMT_TRY_CUDA(cudaMalloc(&m->msq, sizeof(double) * m->n_ref_pad));
        CMT_TRY_CUDA(cudaMalloc(&m->mnorm, sizeof(double) * m->n_ref_pad));
        CMT_TRY_CUDA(cudaMalloc(&m->sref, sizeof(double) * m->n_ref_pad));
        CMT_TRY_CUDA(cudaMalloc(&m->ca, sizeof(float) * m->n_ref_pad));
        CMT_TRY_CUDA(cudaMalloc(&m->cb, sizeof(float) * m->n_ref_pad));
        m->cap_ref = m->n_ref_pad;
    }
    row_stats(*m, model, n_ref, m->msum, m->msq);
    k_batch_scales<<<1, 1024, 0, m->stream>>>(m->dsum, m->dsq, m->n_img, m->msum, m->msq, n_ref, nbatches, m->n_pix,
                                              m->sref, m->stats);
    build_op(*m, model, n_ref, m->sref, 1, m->opB, m->mnorm);
    k_score_coeffs<<<ceil_div(m->n_ref_pad, 256), 256, 0, m->stream>>>(m->mnorm, n_ref, m->n_ref_pad, m->ca, m->cb);
    CMT_LAUNCH_CHECK();
    mark(*m, 3);
    return CMT_OK;
}

// Per image: best reference index (int32), its distance and the second-best distance
// (float64, exact re-scoring), near-tie flags (int32).  n_near (host, optional): count.
extern "C" int cmt_match_run(cmt_match *m, int *best_idx, double *best_d, double *second_d, int *near_tie,
                             int *n_near_host)
{
    CMT_CHECK_ARG(m && best_idx && best_d && second_d && near_tie, "null argument");
    CMT_CHECK_ARG(m->n_img > 0 && m->n_ref > 0, "set_data and set_refs first");
    cudaStream_t st = m->stream;
    SegInfo si{};
    mark(*m, 4);
    if (m->mode == 0 || m->mode == 3) {
        cmt_match *one[1] = {m};
        CMT_TRY(tc_launch(1, one, st, &si));
    } else {
        int n_it = (int)((m->n_img + 63) / 64), n_rt = (int)(m->n_ref_pad / 64);
        int nimg_pad = n_it * 64;
        int64_t need = (int64_t)n_rt * nimg_pad * TOPK;
        si.mode = 0;
        si.n_ref = (int)m->n_ref;
        si.nseg = n_rt;
        si.nimg_pad = nimg_pad;
        int64_t cap = m->cap_part;
        CMT_TRY(ensure((void **)&m->pscore, cap, need * 4));
        int64_t cap2 = m->cap_part;
        CMT_TRY(ensure((void **)&m->pidx, cap2, need * 4));
        m->cap_part = std::min(cap, cap2);
        dim3 grid(n_it, n_rt);
        if (m->mode == 1)
            k_dist_simt<float><<<grid, 256, 0, st>>>((const float *)m->opA, (const float *)m->opB, (int)m->n_img,
                                                     (int)m->n_ref, m->Kp, m->ca, m->cb, m->pscore, m->pidx, nimg_pad);
        else
            k_dist_simt<double><<<grid, 256, 0, st>>>((const double *)m->opA, (const double *)m->opB, (int)m->n_img,
                                                      (int)m->n_ref, m->Kp, m->ca, m->cb, m->pscore, m->pidx,
                                                      nimg_pad);
        CMT_LAUNCH_CHECK();
    }
    mark(*m, 5);
    merge(*m, si, st, best_idx, best_d, second_d, near_tie);
    CMT_LAUNCH_CHECK();
    mark(*m, 6);
    if (m->mode == 0 || m->mode == 3 || n_near_host) {
        int herr = 0;
        if (m->mode == 0 || m->mode == 3) CMT_TRY_CUDA(cudaMemcpyAsync(&herr, m->err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CMT_TRY_CUDA(cudaStreamSynchronize(st));
        if (herr) {
            set_error("tensor-core distance kernel: a bounded pipeline wait timed out");
            return CMT_ERR_TIMEOUT;
        }
        if (n_near_host) CMT_TRY(count_near(*m, near_tie, n_near_host));
    }
    return CMT_OK;
}

// The tensor-core runs of n matchers (modes 0 / 3, any sizes) in one launch per TC_MAXP
// matchers, then each one's re-scoring, with one host synchronisation at the end; outputs
// as for cmt_match_run, per matcher.  Runs on the stream of ms[0].
extern "C" int cmt_match_run_many(int n, cmt_match *const *ms, int *const *best_idx, double *const *best_d,
                                  double *const *second_d, int *const *near_tie, int *n_near_host)
{
    CMT_CHECK_ARG(n >= 1 && ms && best_idx && best_d && second_d && near_tie, "bad argument");
    for (int i = 0; i < n; ++i) {
        CMT_CHECK_ARG(ms[i] && best_idx[i] && best_d[i] && second_d[i] && near_tie[i], "null argument at %d", i);
        CMT_CHECK_ARG(ms[i]->mode == 0 || ms[i]->mode == 3, "matcher %d is not a tensor-core form (mode 0 or 3)", i);
        CMT_CHECK_ARG(ms[i]->n_img > 0 && ms[i]->n_ref > 0, "matcher %d: set_data and set_refs first", i);
        for (int j = 0; j < i; ++j) CMT_CHECK_ARG(ms[j] != ms[i], "matcher %d given twice", i);
    }
    cudaStream_t st = ms[0]->stream;
    std::vector<SegInfo> si(n);
    std::vector<int> err_at;
    for (int b = 0; b < n; b += TC_MAXP) {
        const int k = std::min(TC_MAXP, n - b);
        CMT_TRY(tc_launch(k, ms + b, st, si.data() + b));
        // the CTA ranges in ms[b]->cta_u are read by these merges before the next launch
        for (int i = b; i < b + k; ++i) merge(*ms[i], si[i], st, best_idx[i], best_d[i], second_d[i], near_tie[i]);
        CMT_LAUNCH_CHECK();
        err_at.push_back(b);
    }
    std::vector<int> herr(err_at.size(), 0);
    for (size_t j = 0; j < err_at.size(); ++j)
        CMT_TRY_CUDA(cudaMemcpyAsync(&herr[j], ms[err_at[j]]->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CMT_TRY_CUDA(cudaStreamSynchronize(st));
    for (int e : herr)
        if (e) {
            set_error("tensor-core distance kernel: a bounded pipeline wait timed out");
            return CMT_ERR_TIMEOUT;
        }
    if (n_near_host)
        for (int i = 0; i < n; ++i) CMT_TRY(count_near(*ms[i], near_tie[i], n_near_host + i));
    return CMT_OK;
}

// batch scale factors s_b (nbatches values) followed by std(data), as float64 on the host
extern "C" int cmt_match_stats(cmt_match *m, double *host_out)
{
    CMT_CHECK_ARG(m && host_out, "null argument");
    CMT_TRY_CUDA(cudaMemcpyAsync(host_out, m->stats, sizeof(double) * (m->nbatches + 1), cudaMemcpyDeviceToHost,
                                 m->stream));
    CMT_TRY_CUDA(cudaStreamSynchronize(m->stream));
    return CMT_OK;
}

// Limit (seconds, 1e-3 .. 60) of every wait of the tensor-core pipeline; a wait that runs
// out makes cmt_match_run return CMT_ERR_TIMEOUT with the context still usable.
// Tile of the tensor-core kernel: references per tile (bn: 128 or 256) and TMA ring stages
// (256: 3 or 4; 128: 4 or 6).  Picked by the autotuner; the default is 256 x 4.  A grouped
// run (cmt_match_run_many) uses the first matcher's tile.
extern "C" int cmt_match_set_tile(cmt_match *m, int bn, int stages)
{
    CMT_CHECK_ARG(m, "null matcher");
    CMT_CHECK_ARG(tc_kernel(bn, stages), "tile %d x %d stages is not one of 256 x 4, 256 x 3, 128 x 6, 128 x 4", bn,
                  stages);
    m->tile_bn = bn;
    m->stages = stages;
    return CMT_OK;
}

extern "C" int cmt_match_set_wait_limit(cmt_match *m, double seconds)
{
    CMT_CHECK_ARG(m, "null matcher");
    CMT_CHECK_ARG(seconds >= 1e-3 && seconds <= 60.0, "wait limit must be in [1e-3, 60] seconds");
    m->wait_s = seconds;
    return CMT_OK;
}

// Test of the timeout path: while enabled, the tensor-core kernel's producer issues no loads,
// so the MMA and epilogue waits run out after the wait limit; every role then unwinds (the
// TMEM allocation is released) and the run returns CMT_ERR_TIMEOUT.
extern "C" int cmt_match_stall_loads(cmt_match *m, int enable)
{
    CMT_CHECK_ARG(m, "null matcher");
    m->stall_loads = enable != 0;
    return CMT_OK;
}

// CUDA-event timing of the matcher's stages (enable 0/1); cmt_match_last_ms then gives, in
// ms, the last set_data (image operands), set_refs (reference statistics and operands),
// distance kernel and re-scoring.  Used by benchmarks.
extern "C" int cmt_match_profile(cmt_match *m, int enable)
{
    CMT_CHECK_ARG(m, "null matcher");
    if (enable && !m->ev[0])
        for (auto &e : m->ev) CMT_TRY_CUDA(cudaEventCreate(&e));
    m->timed = enable != 0;
    return CMT_OK;
}

extern "C" int cmt_match_last_ms(cmt_match *m, float *ms)
{
    CMT_CHECK_ARG(m && ms, "null argument");
    CMT_CHECK_ARG(m->timed, "profiling is off (cmt_match_profile)");
    CMT_TRY_CUDA(cudaEventSynchronize(m->ev[6]));
    const int pairs[4][2] = {{0, 1}, {2, 3}, {4, 5}, {5, 6}};
    for (int k = 0; k < 4; ++k) CMT_TRY_CUDA(cudaEventElapsedTime(&ms[k], m->ev[pairs[k][0]], m->ev[pairs[k][1]]));
    return CMT_OK;
}

extern "C" int cmt_match_destroy(cmt_match *m)
{
    if (!m) return CMT_OK;
    for (auto e : m->ev)
        if (e) cudaEventDestroy(e);
    void *bufs[] = {m->w, m->wdf, m->cen, m->cenf, m->opA, m->opB, m->dsum, m->dsq, m->msum, m->msq, m->mnorm, m->sref,
                    m->ca, m->cb, m->stats, m->pscore, m->pidx, m->err, m->near, m->scratch_d, m->cta_u};
    for (void *b : bufs) cudaFree(b);
    delete m;
    return CMT_OK;
}
