// Conjugate-gradient autocorrelation solve on the device.
//
// Normal equations of cmtip/autocorrelation/autocorrelation.py:113-173 (setup_linops):
//   W x = a * S . conv_{2M}(T, S x)        (Toeplitz data term, core_problem_convolution :32-63)
//       + r * x                            (Tikhonov)
//       + f * S . Re(IFFT(FFT(S x) . A))   (Fourier antisupport, fourier_reg :88-110)
// with T = Re(type-1 of ones onto 2M modes) / (2M)^3 (:141-148).  The data term can instead
// be applied as the explicit fused type-2 then type-1 pair on the points (cmt_execute_pair).
// Both FFT convolutions use real-to-complex transforms: the operands are real and the
// multipliers Hermitian, which is what the reference's .real projections compute.
//
// The iteration is scipy's cg (scipy/sparse/linalg/_isolve/iterative.py, called at
// autocorrelation.py:239): no preconditioner, convergence test ||r|| < max(atol, rtol ||b||)
// at the top of each iteration, r0 = b - W x0 only if x0 has a nonzero entry.  Vectors
// live in the solver precision (float for the mixed form, double for the FP64 form);
// every inner product and residual norm is accumulated to FP64 accuracy and the alpha/beta
// scalars are FP64.  With float vectors the per-element work stays in FP32 error-free
// arithmetic (compensated dot products, Dot2, per thread, then FP64 across threads; vector
// updates x + alpha p rounded once from their exact value), since GB300 runs FP64 at a small
// fraction of its FP32 rate.  One iteration
// is a fixed launch sequence with no host synchronisation, so it is captured once into a
// CUDA graph and replayed; a device-side flag turns the updates into no-ops after
// convergence.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "cmt_common.cuh"
#include "df.cuh"

namespace cmt {

struct CgScalars {
    double rho, rho_prev, pq, alpha, atol, bnorm, beta;
    float alpha_hi, alpha_lo, beta_hi, beta_lo;  // alpha, beta as float pairs (float vectors' updates)
    int it, done;
    unsigned ticket[4];
};

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 1216;  // 8 x 152 SMs (a few elements per thread; no per-thread FP64 work)

struct Cg {
    int M = 0, prec = 32, op = 0;  // op 0 Toeplitz, 1 explicit pair
    cudaStream_t stream = nullptr;
    double alambda = 1, rlambda = 0, flambda = 0;
    int64_t m3 = 0, m2 = 0;  // M^3, (2M)^3
    // device buffers
    void *x = nullptr, *r = nullptr, *p = nullptr, *q = nullptr, *b = nullptr;
    void *sx = nullptr, *pad = nullptr, *conv = nullptr, *spec = nullptr, *spec2 = nullptr, *reg = nullptr;
    void *spec_in = nullptr;  // (2M)x(2M)x(M+1) complex: 2D transforms of the M data slices, zero beyond
    void *kern_hat = nullptr;  // (2M)x(2M)x(M+1) complex: FFT of T / (2M)^3
    void *mask_hat = nullptr;  // M x M x (M/2+1) real: Hermitian part of ifftshift(antisupport) / M^3
    float *support = nullptr;  // M^3
    double *partial = nullptr;
    CgScalars *sc = nullptr;
    CgScalars *host_sc = nullptr;  // pinned host copy of sc, read after a solve
    // (2M)^3 convolution of a vector padded into the [0, M)^3 corner, pruned to the slices
    // that hold data: 2D R2C of the first M slices (r2c_2d), the 1D transform along the
    // slice axis of all (2M)x(M+1) columns (c2c_x, both directions), 2D C2R back to the
    // first M slices (c2r_2d).  r2c_big (the full 3D R2C) transforms the Toeplitz kernel.
    cufftHandle r2c_big = 0, r2c_2d = 0, c2c_x = 0, c2r_2d = 0, r2c_small = 0, c2r_small = 0;
    bool have_big = false, have_small = false;
    cmt_plan *pair_plan = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t cap_stream = nullptr;  // private stream the iteration is captured on
    // the Fourier-regulariser branch of the Toeplitz matvec runs on a side stream, beside
    // the (2M)^3 convolution (fork / join events; inside a capture they become graph edges)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool ready = false;
};

}  // namespace cmt

struct cmt_cg : cmt::Cg {};

namespace cmt {

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum of the block's compensated float pairs: the warps combine their (s, c) pairs in FP32
// (TwoSum of the leading parts, the errors added to c), thread 0 adds the warps' pairs in
// FP64.  Keeps the FP64 work to one thread per block.
__device__ __forceinline__ double block_sum_dot2(Dot2 d)
{
    __shared__ float ss[RED_THREADS / 32], cs[RED_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, d.s, o), c2 = __shfl_down_sync(0xffffffffu, d.c, o);
        const float s = __fadd_rn(d.s, s2), bs = __fsub_rn(s, d.s);
        const float e = __fadd_rn(__fsub_rn(d.s, __fsub_rn(s, bs)), __fsub_rn(s2, bs));
        d.s = s;
        d.c = __fadd_rn(__fadd_rn(d.c, c2), e);
    }
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = d.s;
        cs[threadIdx.x >> 5] = d.c;
    }
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < RED_THREADS / 32; ++i) t += (double)ss[i] + (double)cs[i];
    return t;  // in thread 0
}

// Block partial of a sum; the last block to finish reduces all partials in a fixed
// order (deterministic) and returns true in thread 0 with the total in *out.
// With block_total, v in thread 0 already holds the block's sum (block_sum_dot2).
__device__ bool block_reduce_last(double v, double *partial, unsigned *ticket, double *out, bool block_total = false)
{
    __shared__ double s[RED_THREADS / 32];
    __shared__ bool last;
    if (!block_total) {
        v = warp_sum(v);
        if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
        __syncthreads();
    }
    if (threadIdx.x < 32) {
        double t = v;
        if (!block_total) {
            t = threadIdx.x < RED_THREADS / 32 ? s[threadIdx.x] : 0.0;
            t = warp_sum(t);
        }
        if (threadIdx.x == 0) {
            partial[blockIdx.x] = t;
            __threadfence();
            unsigned k = atomicAdd(ticket, 1u);
            last = (k == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += ((volatile double *)partial)[i];
    // fixed-order tree over the block
    t = warp_sum(t);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int i = 0; i < RED_THREADS / 32; ++i) tot += s[i];
        *out = tot;
        *ticket = 0u;
    }
    return threadIdx.x == 0;
}

// dot(a, b) (or |a|^2) -> sc->field, plus optional companion sum of b^2 (for ||b||)
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_dot(const T *a, const T *b, int64_t n, double *partial,
                                                     unsigned *ticket, double *out)
{
    double v = 0.0;
    Dot2 v2{0.f, 0.f};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if constexpr (sizeof(T) == 4)
            dot2_add(v2, a[i], b[i]);
        else
            v += (double)a[i] * (double)b[i];
    }
    if constexpr (sizeof(T) == 4)
        block_reduce_last(block_sum_dot2(v2), partial, ticket, out, true);
    else
        block_reduce_last(v, partial, ticket, out);
}

// scipy's convergence test before the next iteration and that iteration's beta, once rho
// has changed (the start of a solve, the end of an iteration); one thread, FP64.
__device__ void next_step_scalars(CgScalars *sc)
{
    if (sc->done) return;
    if (sqrt(sc->rho) < sc->atol) {
        sc->done = 1;
        return;
    }
    const double beta = sc->it > 0 ? sc->rho / sc->rho_prev : 0.0;
    sc->beta = beta;
    sc->beta_hi = (float)beta;
    sc->beta_lo = (float)(beta - (double)(float)beta);
}

__global__ void k_next_step(CgScalars *sc) { next_step_scalars(sc); }

// Start of an iteration: p = r (+ beta p), S p into the padded corner (Toeplitz) and into the
// M^3 buffer for the Fourier regulariser; the convergence test and beta were evaluated when
// rho last changed (next_step_scalars).  With float vectors, p = r + beta p is the FP64 value
// rounded to float, computed in float error-free arithmetic (axpy_rn): GB300's FP64 pipe runs
// at a small fraction of its FP32 rate.  Indices fit 32 bits ((2M)^3 <= 2^30).
template <typename T>
__global__ void k_iter_begin(CgScalars *sc, const T *__restrict__ r, T *__restrict__ p,
                             const float *__restrict__ support, int M, int use_pad, T *__restrict__ pad,
                             T *__restrict__ sx)
{
    if (sc->done) return;
    const bool first = sc->it == 0;
    const float bh = sc->beta_hi, bl = sc->beta_lo;
    const int m3 = M * M * M, mm = M * M, M2 = 2 * M;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m3; i += gridDim.x * blockDim.x) {
        T pv;
        if (first) {
            pv = r[i];
        } else if constexpr (sizeof(T) == 4) {
            pv = axpy_rn(r[i], bh, bl, p[i]);
        } else {
            pv = (T)((double)r[i] + sc->beta * (double)p[i]);
        }
        p[i] = pv;
        const T v = pv * (T)support[i];
        sx[i] = v;
        if (use_pad) {
            const int a = i / mm, rem = i - a * mm, bb = rem / M, c = rem - bb * M;
            pad[(a * M2 + bb) * M2 + c] = v;
        }
    }
}

// S x for a given vector (matvec outside the iteration)
template <typename T>
__global__ void k_apply_support(const T *v, const float *support, int M, int use_pad, T *pad, T *sx)
{
    const int m3 = M * M * M, mm = M * M, M2 = 2 * M;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m3; i += gridDim.x * blockDim.x) {
        T s = v[i] * (T)support[i];
        sx[i] = s;
        if (use_pad) {
            const int a = i / mm, rem = i - a * mm, bb = rem / M, c = rem - bb * M;
            pad[(a * M2 + bb) * M2 + c] = s;
        }
    }
}

template <typename T>
__global__ void k_mul_complex(cplx_t<T> *a, const cplx_t<T> *b, int64_t n, const CgScalars *sc)
{
    if (sc && sc->done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        cplx_t<T> u = a[i], v = b[i];
        a[i] = {u.x * v.x - u.y * v.y, u.x * v.y + u.y * v.x};
    }
}

template <typename T>
__global__ void k_mul_real(cplx_t<T> *a, const T *m, int64_t n, const CgScalars *sc)
{
    if (sc && sc->done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        cplx_t<T> u = a[i];
        T s = m[i];
        a[i] = {u.x * s, u.y * s};
    }
}

// q = a S conv + r v + f S reg; conv read from the (2M)^3 corner (stride 2M) or an M^3 grid.
// With dot: pq = v . q -> alpha = rho / pq (float vectors: per-thread compensated sums, Dot2,
// then FP64 across threads).
template <typename T>
__global__ void __launch_bounds__(RED_THREADS)
    k_combine(CgScalars *sc, const T *__restrict__ v, const T *__restrict__ conv, int conv_pad,
              const T *__restrict__ reg, const float *__restrict__ support, int M, T al, T rl, T fl,
              T *__restrict__ q, int with_dot, double *partial)
{
    if (with_dot && sc->done) return;
    const int m3 = M * M * M, mm = M * M, M2 = 2 * M;
    double acc = 0.0;
    Dot2 acc2{0.f, 0.f};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m3; i += gridDim.x * blockDim.x) {
        T cv;
        if (conv_pad) {
            const int a = i / mm, rem = i - a * mm, bb = rem / M, c = rem - bb * M;
            cv = conv[(a * M2 + bb) * M2 + c];
        } else {
            cv = conv[i];
        }
        const T s = (T)support[i], vi = v[i];
        const T out = al * s * cv + rl * vi + fl * s * reg[i];
        q[i] = out;
        if constexpr (sizeof(T) == 4)
            dot2_add(acc2, vi, out);
        else
            acc += (double)vi * (double)out;
    }
    if (!with_dot) return;
    if constexpr (sizeof(T) == 4) acc = block_sum_dot2(acc2);
    double tot;
    if (block_reduce_last(acc, partial, &sc->ticket[0], &tot, sizeof(T) == 4)) {
        const double alpha = sc->rho / tot;
        sc->pq = tot;
        sc->alpha = alpha;
        sc->alpha_hi = (float)alpha;
        sc->alpha_lo = (float)(alpha - (double)(float)alpha);
    }
}

// x += alpha p ; r -= alpha q ; rho_new = r . r.  Float vectors: the FP64 updates rounded to
// float (axpy_rn) and a per-thread compensated r . r (Dot2), FP64 across threads.
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_update(CgScalars *sc, T *__restrict__ x, T *__restrict__ r,
                                                        const T *__restrict__ p, const T *__restrict__ q, int M,
                                                        double *partial)
{
    if (sc->done) return;
    const int m3 = M * M * M;
    const double alpha = sc->alpha;
    const float ah = sc->alpha_hi, al = sc->alpha_lo;
    double acc = 0.0;
    Dot2 acc2{0.f, 0.f};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m3; i += gridDim.x * blockDim.x) {
        if constexpr (sizeof(T) == 4) {
            x[i] = axpy_rn(x[i], ah, al, p[i]);
            const float rn = axpy_rn(r[i], -ah, -al, q[i]);
            r[i] = rn;
            dot2_add(acc2, rn, rn);
        } else {
            x[i] = (T)((double)x[i] + alpha * (double)p[i]);
            T rn = (T)((double)r[i] - alpha * (double)q[i]);
            r[i] = rn;
            acc += (double)rn * (double)rn;
        }
    }
    if constexpr (sizeof(T) == 4) acc = block_sum_dot2(acc2);
    double tot;
    if (block_reduce_last(acc, partial, &sc->ticket[1], &tot, sizeof(T) == 4)) {
        sc->rho_prev = sc->rho;
        sc->rho = tot;
        sc->it += 1;
        next_step_scalars(sc);
    }
}

// Scalars at the start of a solve, on the device (no host round trip): ||b|| from the
// b.b that k_dot left in sc->bnorm, the stopping threshold max(atol, rtol ||b||), and
// done = 1 when ||b|| = 0 (scipy then returns b itself).
__global__ void k_begin_scalars(CgScalars *sc, double rtol, double atol)
{
    const double bnorm = sqrt(sc->bnorm);
    sc->bnorm = bnorm;
    sc->atol = fmax(atol, rtol * bnorm);
    sc->it = 0;
    sc->done = bnorm == 0.0 ? 1 : 0;
    sc->pq = 0.0;
}

// x = b where the solve is trivial (||b|| = 0)
template <typename T>
__global__ void k_copy_if_done(const CgScalars *sc, const T *b, T *x, int64_t n)
{
    if (!sc->done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = b[i];
}

// r = b - q  (q = W x0)
template <typename T>
__global__ void k_residual(const T *b, const T *q, T *r, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = (T)((double)b[i] - (double)q[i]);
}

template <typename T>
__global__ void k_scale(T *a, int64_t n, double s)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (T)((double)a[i] * s);
}

// Hermitian part of a real M^3 multiplier in FFT order, stored as the R2C half (M x M x (M/2+1)),
// times s.  For a real-even multiplier (odd M, symmetric antisupport) this is just the half.
template <typename T>
__global__ void k_mask_half(const float *m_fft, int M, double s, T *half)
{
    int hz = M / 2 + 1;
    int64_t n = (int64_t)M * M * hz;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = (int)(i % hz);
    int64_t r = i / hz;
    int b = (int)(r % M), a = (int)(r / M);
    int na = (M - a) % M, nb = (M - b) % M, nc = (M - c) % M;
    double v = 0.5 * ((double)m_fft[((int64_t)a * M + b) * M + c] + (double)m_fft[((int64_t)na * M + nb) * M + nc]);
    half[i] = (T)(v * s);
}

// scipy.ndimage.gaussian_filter(est, sigma=0.5) > 1e-12 (truncate 4 -> radius 2, mode
// 'reflect'), one axis per pass with the float32 rounding of each pass, taps combined
// symmetrically in float64 as ndimage's correlate1d does.
__global__ void k_gauss_axis(const float *in, float *out, int M, int axis, double w0, double w1, double w2)
{
    int64_t m3 = (int64_t)M * M * M;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m3) return;
    int64_t c[3] = {i / ((int64_t)M * M), (i / M) % M, i % M};
    int64_t stride = axis == 0 ? (int64_t)M * M : (axis == 1 ? M : 1);
    int64_t pos = c[axis];
    auto refl = [&](int64_t k) -> int64_t {
        // half-sample symmetric reflection: d c b a | a b c d | d c b a
        int64_t period = 2 * M;
        k %= period;
        if (k < 0) k += period;
        return k < M ? k : period - 1 - k;
    };
    const float *base = in + (i - pos * stride);
    double v0 = base[pos * stride];
    double a1 = (double)base[refl(pos - 1) * stride] + (double)base[refl(pos + 1) * stride];
    double a2 = (double)base[refl(pos - 2) * stride] + (double)base[refl(pos + 2) * stride];
    double t = v0 * w0;
    t += a1 * w1;
    t += a2 * w2;
    out[i] = (float)t;
}

__global__ void k_threshold(const float *sm, float *support, float *est, int64_t n, double thr)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = sm[i] > thr ? 1.0f : 0.0f;
    support[i] = s;
    if (est) est[i] *= s;
}

// ---------------------------------------------------------------- host

static size_t esz(const Cg &c) { return c.prec == 64 ? 8 : 4; }

static int grid_elems(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 152 * 8); }

template <typename T>
static int matvec_impl(Cg &c, const T *v, T *out, bool in_iteration)
{
    cudaStream_t st = c.stream;
    int M = c.M;
    bool toe = c.op == 0;
    int g = grid_elems(c.m3);
    if (!in_iteration) {
        k_apply_support<T><<<g, 256, 0, st>>>(v, c.support, M, toe, (T *)c.pad, (T *)c.sx);
        CMT_LAUNCH_CHECK();
    }
    CgScalars *sc = in_iteration ? c.sc : nullptr;
    int64_t hbig = (int64_t)(2 * M) * (2 * M) * (M + 1);
    int64_t hsmall = (int64_t)M * M * (M / 2 + 1);
    // the regulariser's M^3 transforms are small, latency-bound launches: with the Toeplitz
    // operator they run on the side stream while the (2M)^3 convolution runs on st
    const bool fork = toe && c.flambda != 0.0 && c.side;
    if (fork) {
        CMT_TRY_CUDA(cudaEventRecord(c.ev_fork, st));
        CMT_TRY_CUDA(cudaStreamWaitEvent(c.side, c.ev_fork, 0));
        CMT_TRY_CUFFT(cufftSetStream(c.r2c_small, c.side));
        CMT_TRY_CUFFT(cufftSetStream(c.c2r_small, c.side));
    }
    cudaStream_t st_reg = fork ? c.side : st;
    if (c.flambda != 0.0) {
        if (c.prec == 64) {
            CMT_TRY_CUFFT(cufftExecD2Z(c.r2c_small, (double *)c.sx, (cufftDoubleComplex *)c.spec2));
        } else {
            CMT_TRY_CUFFT(cufftExecR2C(c.r2c_small, (float *)c.sx, (cufftComplex *)c.spec2));
        }
        k_mul_real<T><<<grid_elems(hsmall), 256, 0, st_reg>>>((cplx_t<T> *)c.spec2, (const T *)c.mask_hat, hsmall,
                                                               sc);
        CMT_LAUNCH_CHECK();
        if (c.prec == 64) {
            CMT_TRY_CUFFT(cufftExecZ2D(c.c2r_small, (cufftDoubleComplex *)c.spec2, (double *)c.reg));
        } else {
            CMT_TRY_CUFFT(cufftExecC2R(c.c2r_small, (cufftComplex *)c.spec2, (float *)c.reg));
        }
    } else {
        CMT_TRY_CUDA(cudaMemsetAsync(c.reg, 0, esz(c) * c.m3, st));
    }
    if (fork) {
        CMT_TRY_CUDA(cudaEventRecord(c.ev_join, c.side));
        CMT_TRY_CUFFT(cufftSetStream(c.r2c_small, st));
        CMT_TRY_CUFFT(cufftSetStream(c.c2r_small, st));
    }
    if (toe) {
        // conv = IFFT(kern_hat . FFT(pad)) over (2M)^3, pruned: pad is zero outside slices
        // [0, M) (2D R2C of those slices into spec_in, whose other slices stay zero), and
        // only slices [0, M) of the result are read (2D C2R of those slices)
        if (c.prec == 64) {
            CMT_TRY_CUFFT(cufftExecD2Z(c.r2c_2d, (double *)c.pad, (cufftDoubleComplex *)c.spec_in));
            CMT_TRY_CUFFT(cufftExecZ2Z(c.c2c_x, (cufftDoubleComplex *)c.spec_in, (cufftDoubleComplex *)c.spec,
                                       CUFFT_FORWARD));
        } else {
            CMT_TRY_CUFFT(cufftExecR2C(c.r2c_2d, (float *)c.pad, (cufftComplex *)c.spec_in));
            CMT_TRY_CUFFT(cufftExecC2C(c.c2c_x, (cufftComplex *)c.spec_in, (cufftComplex *)c.spec, CUFFT_FORWARD));
        }
        k_mul_complex<T><<<grid_elems(hbig), 256, 0, st>>>((cplx_t<T> *)c.spec, (const cplx_t<T> *)c.kern_hat, hbig, sc);
        CMT_LAUNCH_CHECK();
        if (c.prec == 64) {
            CMT_TRY_CUFFT(cufftExecZ2Z(c.c2c_x, (cufftDoubleComplex *)c.spec, (cufftDoubleComplex *)c.spec,
                                       CUFFT_INVERSE));
            CMT_TRY_CUFFT(cufftExecZ2D(c.c2r_2d, (cufftDoubleComplex *)c.spec, (double *)c.conv));
        } else {
            CMT_TRY_CUFFT(cufftExecC2C(c.c2c_x, (cufftComplex *)c.spec, (cufftComplex *)c.spec, CUFFT_INVERSE));
            CMT_TRY_CUFFT(cufftExecC2R(c.c2r_2d, (cufftComplex *)c.spec, (float *)c.conv));
        }
    } else {
        // explicit pair: conv = Re(A^H A (S v)) S / (2M)^3 on the M^3 grid
        CMT_TRY(cmt_execute_pair(c.pair_plan, in_iteration ? c.p : v, c.conv, c.support,
                                 1.0 / ((double)(2 * M) * (2 * M) * (2 * M))));
    }
    if (fork) CMT_TRY_CUDA(cudaStreamWaitEvent(st, c.ev_join, 0));
    // the pair already applied S and the 1/(2M)^3; the Toeplitz conv is unscaled (kern_hat holds it)
    k_combine<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>(c.sc, in_iteration ? (const T *)c.p : v, (const T *)c.conv,
                                                     toe ? 1 : 0, (const T *)c.reg, c.support, M, (T)c.alambda,
                                                     (T)c.rlambda, (T)c.flambda, out, in_iteration ? 1 : 0,
                                                     c.partial);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

template <typename T>
static int iteration(Cg &c)
{
    cudaStream_t st = c.stream;
    int g = grid_elems(c.m3);
    k_iter_begin<T><<<g, 256, 0, st>>>(c.sc, (const T *)c.r, (T *)c.p, c.support, c.M, c.op == 0, (T *)c.pad,
                                       (T *)c.sx);
    CMT_LAUNCH_CHECK();
    CMT_TRY(matvec_impl<T>(c, (const T *)c.p, (T *)c.q, true));
    k_update<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>(c.sc, (T *)c.x, (T *)c.r, (const T *)c.p, (const T *)c.q, c.M,
                                                    c.partial);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

static void cg_destroy(Cg *c)
{
    if (!c) return;
    void *bufs[] = {c->x, c->r, c->p, c->q, c->b, c->sx, c->pad, c->conv, c->spec, c->spec_in, c->spec2, c->reg,
                    c->kern_hat, c->mask_hat, c->support, c->partial, c->sc};
    for (void *b : bufs) cudaFree(b);
    if (c->host_sc) cudaFreeHost(c->host_sc);
    if (c->have_big) {
        cufftDestroy(c->r2c_big);
        cufftDestroy(c->r2c_2d);
        cufftDestroy(c->c2c_x);
        cufftDestroy(c->c2r_2d);
    }
    if (c->have_small) {
        cufftDestroy(c->r2c_small);
        cufftDestroy(c->c2r_small);
    }
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
}

// Route every launch of the solver (its kernels, its cuFFT plans, the pair plan) to s.
static int route_to(Cg &c, cudaStream_t s)
{
    c.stream = s;
    if (c.have_big) {
        CMT_TRY_CUFFT(cufftSetStream(c.r2c_big, s));
        CMT_TRY_CUFFT(cufftSetStream(c.r2c_2d, s));
        CMT_TRY_CUFFT(cufftSetStream(c.c2c_x, s));
        CMT_TRY_CUFFT(cufftSetStream(c.c2r_2d, s));
    }
    if (c.have_small) {
        CMT_TRY_CUFFT(cufftSetStream(c.r2c_small, s));
        CMT_TRY_CUFFT(cufftSetStream(c.c2r_small, s));
    }
    if (c.pair_plan) CMT_TRY(cmt_plan_set_stream(c.pair_plan, s));
    return CMT_OK;
}

// Capture one iteration on the private stream (legacy-default-stream callers cannot be
// captured) and instantiate it; the graph is then launched on the caller's stream.
template <typename T> static int iteration(Cg &c);

// Capture one iteration on the private stream (legacy-default-stream callers cannot be
// captured) into *out (not instantiated); the solver's launches are routed back to its
// stream afterwards.
template <typename T>
static int capture_graph(Cg &c, cudaGraph_t *out)
{
    *out = nullptr;
    if (!c.cap_stream) CMT_TRY_CUDA(cudaStreamCreateWithFlags(&c.cap_stream, cudaStreamNonBlocking));
    cudaStream_t user = c.stream;
    CMT_TRY(route_to(c, c.cap_stream));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c.cap_stream, cudaStreamCaptureModeThreadLocal);
    int rc = e == cudaSuccess ? iteration<T>(c) : CMT_ERR_CUDA;
    cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(c.cap_stream, &graph) : e;
    int rc2 = route_to(c, user);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        set_error("CG graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
        if (graph) cudaGraphDestroy(graph);
        return CMT_ERR_CUDA;
    }
    if (rc != CMT_OK || rc2 != CMT_OK) {
        cudaGraphDestroy(graph);
        return rc != CMT_OK ? rc : rc2;
    }
    *out = graph;
    return CMT_OK;
}

// Capture one iteration and instantiate it; the graph is then launched on the caller's stream.
template <typename T>
static int capture_iteration(Cg &c)
{
    if (c.graph) {
        cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
    }
    cudaGraph_t graph = nullptr;
    CMT_TRY(capture_graph<T>(c, &graph));
    cudaError_t e = cudaGraphInstantiate(&c.graph, graph, 0);
    cudaGraphDestroy(graph);
    CMT_TRY_CUDA(e);
    c.ready = true;
    return CMT_OK;
}

// Start of a solve (scipy's cg before its loop), stream-ordered: b = d, x = x0, ||b||,
// threshold max(atol, rtol ||b||), r0 = b - W x0, rho = r0.r0.  scipy skips the matvec when
// x0 is all zeros; W 0 is exactly 0, so with the Toeplitz operator r0 = b - W x0 is computed
// either way and the start needs no host round trip (the explicit pair, whose matvec costs a
// NUFFT pair, checks x0 on the host).  When ||b|| = 0 the done flag is set and x = b (scipy
// returns b itself).
template <typename T>
static int solve_begin(Cg &c, const T *d, T *x, double rtol, double atol)
{
    cudaStream_t st = c.stream;
    size_t bytes = sizeof(T) * c.m3;
    int g = grid_elems(c.m3);
    CMT_TRY_CUDA(cudaMemsetAsync(c.sc, 0, sizeof(CgScalars), st));
    CMT_TRY_CUDA(cudaMemcpyAsync(c.b, d, bytes, cudaMemcpyDeviceToDevice, st));
    CMT_TRY_CUDA(cudaMemcpyAsync(c.x, x, bytes, cudaMemcpyDeviceToDevice, st));
    CgScalars *sc = c.sc;
    k_dot<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>((const T *)c.b, (const T *)c.b, c.m3, c.partial, &sc->ticket[2],
                                                 &sc->bnorm);
    CMT_LAUNCH_CHECK();
    k_begin_scalars<<<1, 1, 0, st>>>(sc, rtol, atol);
    CMT_LAUNCH_CHECK();
    bool x0_zero = false;
    if (c.op == 1) {
        // the explicit pair's matvec is a full NUFFT pair over the points: skip it for a zero
        // x0 as scipy does, at the price of one host round trip
        k_dot<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>((const T *)c.x, (const T *)c.x, c.m3, c.partial,
                                                     &sc->ticket[3], &sc->pq);
        CMT_LAUNCH_CHECK();
        CMT_TRY_CUDA(cudaMemcpyAsync(c.host_sc, sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, st));
        CMT_TRY_CUDA(cudaStreamSynchronize(st));
        x0_zero = c.host_sc->pq == 0.0;
    }
    if (x0_zero) {
        CMT_TRY_CUDA(cudaMemcpyAsync(c.r, c.b, bytes, cudaMemcpyDeviceToDevice, st));
    } else {
        CMT_TRY(matvec_impl<T>(c, (const T *)c.x, (T *)c.q, false));
        k_residual<T><<<g, 256, 0, st>>>((const T *)c.b, (const T *)c.q, (T *)c.r, c.m3);
        CMT_LAUNCH_CHECK();
    }
    k_dot<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>((const T *)c.r, (const T *)c.r, c.m3, c.partial, &sc->ticket[2],
                                                 &sc->rho);
    CMT_LAUNCH_CHECK();
    k_next_step<<<1, 1, 0, st>>>(sc);
    CMT_LAUNCH_CHECK();
    k_copy_if_done<T><<<g, 256, 0, st>>>(sc, (const T *)c.b, (T *)c.x, c.m3);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

// End of a solve, stream-ordered: x out, and the scalars into the solver's pinned host copy
// (read by solve_result once the stream has passed this point).
template <typename T>
static int solve_end(Cg &c, T *x)
{
    CMT_TRY_CUDA(cudaMemcpyAsync(x, c.x, sizeof(T) * c.m3, cudaMemcpyDeviceToDevice, c.stream));
    CMT_TRY_CUDA(cudaMemcpyAsync(c.host_sc, c.sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, c.stream));
    return CMT_OK;
}

static void solve_result(const Cg &c, int *iters, double *final_rho)
{
    if (iters) *iters = c.host_sc->it;
    if (final_rho) *final_rho = c.host_sc->rho;
}

}  // namespace cmt

using namespace cmt;

extern "C" int cmt_cg_create(int M, int prec, int op, void *stream, cmt_cg **out)
{
    CMT_CHECK_ARG(out, "null output pointer");
    *out = nullptr;
    CMT_CHECK_ARG(M >= 2 && M <= 512, "M must be in [2, 512]");
    CMT_CHECK_ARG(prec == 32 || prec == 64, "prec must be 32 or 64");
    CMT_CHECK_ARG(op == 0 || op == 1, "op must be 0 (Toeplitz) or 1 (explicit pair)");
    cmt_cg *c = new (std::nothrow) cmt_cg();
    if (!c) return CMT_ERR_OOM;
    c->M = M;
    c->prec = prec;
    c->op = op;
    c->stream = (cudaStream_t)stream;
    c->m3 = (int64_t)M * M * M;
    c->m2 = (int64_t)(2 * M) * (2 * M) * (2 * M);
    size_t e = esz(*c);
    int64_t hbig = (int64_t)(2 * M) * (2 * M) * (M + 1), hsmall = (int64_t)M * M * (M / 2 + 1);
    auto fail = [&](int code) {
        cg_destroy(c);
        delete c;
        return code;
    };
    struct A {
        void **p;
        size_t n;
    } allocs[] = {{&c->x, e * c->m3},       {&c->r, e * c->m3},         {&c->p, e * c->m3},
                  {&c->q, e * c->m3},       {&c->b, e * c->m3},         {&c->sx, e * c->m3},
                  {&c->reg, e * c->m3},     {&c->spec2, 2 * e * hsmall}, {&c->mask_hat, e * hsmall},
                  {(void **)&c->support, (size_t)(4 * c->m3)}, {(void **)&c->partial, (size_t)8 * RED_BLOCKS},
                  {(void **)&c->sc, sizeof(CgScalars)}};
    for (auto &a : allocs) {
        cudaError_t err = cudaMalloc(a.p, a.n);
        if (err != cudaSuccess) {
            set_error("cg allocation of %zu bytes: %s", a.n, cudaGetErrorString(err));
            return fail(CMT_ERR_OOM);
        }
    }
    if (op == 0) {  // the regulariser branch's side stream and its fork / join events
        cudaError_t err = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
        if (err != cudaSuccess) {
            set_error("cg side stream: %s", cudaGetErrorString(err));
            return fail(CMT_ERR_CUDA);
        }
    }
    {
        cudaError_t err = cudaMallocHost((void **)&c->host_sc, sizeof(CgScalars));
        if (err != cudaSuccess) {
            set_error("cg pinned scalars: %s", cudaGetErrorString(err));
            return fail(CMT_ERR_OOM);
        }
        memset(c->host_sc, 0, sizeof(CgScalars));
    }
    if (op == 0) {
        struct A big[] = {{&c->pad, e * c->m2},          {&c->conv, e * c->m2},
                          {&c->spec, 2 * e * hbig},      {&c->spec_in, 2 * e * hbig},
                          {&c->kern_hat, 2 * e * hbig}};
        for (auto &a : big) {
            cudaError_t err = cudaMalloc(a.p, a.n);
            if (err != cudaSuccess) {
                set_error("cg allocation of %zu bytes: %s", a.n, cudaGetErrorString(err));
                return fail(CMT_ERR_OOM);
            }
        }
        // the padding (outside the [0, M)^3 corner) and spec_in's slices from M on stay zero
        cudaMemset(c->pad, 0, e * c->m2);
        cudaMemset(c->spec_in, 0, 2 * e * hbig);
        int n2 = 2 * M, h = M + 1;
        int n2d[2] = {n2, n2}, real2d[2] = {n2, n2}, half2d[2] = {n2, h}, n1d[1] = {n2};
        const int col = n2 * h;  // complex elements per slice of the half spectrum
        const bool dp = prec == 64;
        if (cufftPlan3d(&c->r2c_big, n2, n2, n2, dp ? CUFFT_D2Z : CUFFT_R2C) != CUFFT_SUCCESS ||
            cufftPlanMany(&c->r2c_2d, 2, n2d, real2d, 1, n2 * n2, half2d, 1, col, dp ? CUFFT_D2Z : CUFFT_R2C, M) !=
                CUFFT_SUCCESS ||
            cufftPlanMany(&c->c2c_x, 1, n1d, n1d, col, 1, n1d, col, 1, dp ? CUFFT_Z2Z : CUFFT_C2C, col) !=
                CUFFT_SUCCESS ||
            cufftPlanMany(&c->c2r_2d, 2, n2d, half2d, 1, col, real2d, 1, n2 * n2, dp ? CUFFT_Z2D : CUFFT_C2R, M) !=
                CUFFT_SUCCESS) {
            set_error("cuFFT plans for the (2M)^3 convolution failed");
            return fail(CMT_ERR_CUFFT);
        }
        c->have_big = true;
        cufftSetStream(c->r2c_big, c->stream);
        cufftSetStream(c->r2c_2d, c->stream);
        cufftSetStream(c->c2c_x, c->stream);
        cufftSetStream(c->c2r_2d, c->stream);
    } else {
        cudaError_t err = cudaMalloc(&c->conv, e * c->m3);
        if (err != cudaSuccess) return fail(CMT_ERR_OOM);
    }
    if (cufftPlan3d(&c->r2c_small, M, M, M, prec == 64 ? CUFFT_D2Z : CUFFT_R2C) != CUFFT_SUCCESS ||
        cufftPlan3d(&c->c2r_small, M, M, M, prec == 64 ? CUFFT_Z2D : CUFFT_C2R) != CUFFT_SUCCESS) {
        set_error("cuFFT plan M^3 failed");
        return fail(CMT_ERR_CUFFT);
    }
    c->have_small = true;
    cufftSetStream(c->r2c_small, c->stream);
    cufftSetStream(c->c2r_small, c->stream);
    cudaMemsetAsync(c->sc, 0, sizeof(CgScalars), c->stream);
    *out = c;
    return CMT_OK;
}

// Toeplitz kernel from its real circular (FFT-ordered) values T_circ on the (2M)^3 grid
// (already divided by (2M)^3, the adjoint's scale, autocorrelation.py:141-147); stores
// FFT(T_circ) / (2M)^3, the second factor being numpy's ifftn normalisation (:54).
extern "C" int cmt_cg_set_kernel(cmt_cg *c, const void *t_circ)
{
    CMT_CHECK_ARG(c && t_circ, "null argument");
    CMT_CHECK_ARG(c->op == 0, "the kernel belongs to the Toeplitz operator");
    int64_t hbig = (int64_t)(2 * c->M) * (2 * c->M) * (c->M + 1);
    if (c->prec == 64) {
        CMT_TRY_CUFFT(cufftExecD2Z(c->r2c_big, (double *)t_circ, (cufftDoubleComplex *)c->kern_hat));
        k_scale<double><<<grid_elems(2 * hbig), 256, 0, c->stream>>>((double *)c->kern_hat, 2 * hbig, 1.0 / c->m2);
    } else {
        CMT_TRY_CUFFT(cufftExecR2C(c->r2c_big, (float *)t_circ, (cufftComplex *)c->kern_hat));
        k_scale<float><<<grid_elems(2 * hbig), 256, 0, c->stream>>>((float *)c->kern_hat, 2 * hbig, 1.0 / c->m2);
    }
    CMT_LAUNCH_CHECK();
    c->ready = false;
    return CMT_OK;
}

// Fourier-space multiplier of the regulariser: ifftshift(F_antisupport) as float M^3
// (FFT order, autocorrelation.py:105), support S (M^3 float) and the three lambdas
// (alambda, rlambda, flambda of autocorrelation.py:223-225).
extern "C" int cmt_cg_set_operator(cmt_cg *c, const float *mask_fft, const float *support, double alambda,
                                   double rlambda, double flambda)
{
    CMT_CHECK_ARG(c && support, "null argument");
    CMT_CHECK_ARG(mask_fft || flambda == 0.0, "mask required when flambda != 0");
    int M = c->M;
    int64_t hsmall = (int64_t)M * M * (M / 2 + 1);
    if (mask_fft) {
        double s = 1.0 / (double)c->m3;  // numpy ifftn normalisation of fourier_reg (:106)
        if (c->prec == 64)
            k_mask_half<double><<<ceil_div(hsmall, 256), 256, 0, c->stream>>>(mask_fft, M, s, (double *)c->mask_hat);
        else
            k_mask_half<float><<<ceil_div(hsmall, 256), 256, 0, c->stream>>>(mask_fft, M, s, (float *)c->mask_hat);
        CMT_LAUNCH_CHECK();
    }
    CMT_TRY_CUDA(cudaMemcpyAsync(c->support, support, 4 * c->m3, cudaMemcpyDeviceToDevice, c->stream));
    c->alambda = alambda;
    c->rlambda = rlambda;
    c->flambda = flambda;
    c->ready = false;
    return CMT_OK;
}

// Explicit-pair data term: the plan (type 1, M modes, same precision) holds the points.
extern "C" int cmt_cg_set_pair_plan(cmt_cg *c, cmt_plan *plan)
{
    CMT_CHECK_ARG(c && plan, "null argument");
    CMT_CHECK_ARG(c->op == 1, "pair plan applies to the explicit-pair operator");
    CMT_TRY(cmt_plan_prepare_pair(plan));
    c->pair_plan = plan;
    c->ready = false;
    return CMT_OK;
}

// y = W x (solver precision vectors of M^3 elements)
extern "C" int cmt_cg_matvec(cmt_cg *c, const void *x, void *y)
{
    CMT_CHECK_ARG(c && x && y, "null argument");
    CMT_CHECK_ARG(c->op == 0 || c->pair_plan, "pair operator without a plan");
    if (c->prec == 64) return matvec_impl<double>(*c, (const double *)x, (double *)y, false);
    return matvec_impl<float>(*c, (const float *)x, (float *)y, false);
}

template <typename T>
static int solve_impl(Cg &c, const T *d, T *x, int maxiter, double rtol, double atol, int use_graph, int *iters,
                      double *final_rho)
{
    CMT_TRY(solve_begin<T>(c, d, x, rtol, atol));
    if (use_graph) {
        if (!c.ready) CMT_TRY(capture_iteration<T>(c));
        for (int it = 0; it < maxiter; ++it) CMT_TRY_CUDA(cudaGraphLaunch(c.graph, c.stream));
    } else {
        for (int it = 0; it < maxiter; ++it) CMT_TRY(iteration<T>(c));
    }
    CMT_TRY(solve_end<T>(c, x));
    if (iters || final_rho) {
        CMT_TRY_CUDA(cudaStreamSynchronize(c.stream));
        solve_result(c, iters, final_rho);
    }
    return CMT_OK;
}

// Several solvers at once: each one's iteration is captured as a child graph of one parent
// graph with no edges between the children, so one launch of the parent runs one iteration
// of every solve and the independent branches overlap on the GPU.  Every solver keeps its own
// operator, scalars and stopping test; all run on the stream of the first.
template <typename T>
static int solve_many_impl(int n, cmt_cg *const *cgs, const void *const *d, void *const *x, int maxiter, double rtol,
                           double atol, int *iters, double *final_rho)
{
    cudaStream_t st = cgs[0]->stream;
    std::vector<cudaStream_t> own(n);
    for (int i = 0; i < n; ++i) {
        own[i] = cgs[i]->stream;
        CMT_TRY(route_to(*cgs[i], st));
    }
    auto restore = [&]() {
        for (int i = 0; i < n; ++i) route_to(*cgs[i], own[i]);
    };
    int rc = CMT_OK;
    for (int i = 0; i < n && rc == CMT_OK; ++i) rc = solve_begin<T>(*cgs[i], (const T *)d[i], (T *)x[i], rtol, atol);
    cudaGraph_t parent = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (rc == CMT_OK) {
        cudaError_t e = cudaGraphCreate(&parent, 0);
        if (e != cudaSuccess) {
            set_error("cudaGraphCreate: %s", cudaGetErrorString(e));
            rc = CMT_ERR_CUDA;
        }
    }
    for (int i = 0; i < n && rc == CMT_OK; ++i) {
        cudaGraph_t child = nullptr;
        rc = capture_graph<T>(*cgs[i], &child);
        if (rc != CMT_OK) break;
        cudaGraphNode_t node;
        cudaError_t e = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, child);
        cudaGraphDestroy(child);  // the parent holds a copy
        if (e != cudaSuccess) {
            set_error("cudaGraphAddChildGraphNode: %s", cudaGetErrorString(e));
            rc = CMT_ERR_CUDA;
        }
    }
    if (rc == CMT_OK) {
        cudaError_t e = cudaGraphInstantiate(&exec, parent, 0);
        if (e != cudaSuccess) {
            set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
            rc = CMT_ERR_CUDA;
        }
    }
    for (int it = 0; it < maxiter && rc == CMT_OK; ++it) {
        cudaError_t e = cudaGraphLaunch(exec, st);
        if (e != cudaSuccess) {
            set_error("cudaGraphLaunch: %s", cudaGetErrorString(e));
            rc = CMT_ERR_CUDA;
        }
    }
    for (int i = 0; i < n && rc == CMT_OK; ++i) rc = solve_end<T>(*cgs[i], (T *)x[i]);
    if (rc == CMT_OK && (iters || final_rho)) {
        cudaError_t e = cudaStreamSynchronize(st);  // one host synchronisation for all solves
        if (e != cudaSuccess) {
            set_error("cudaStreamSynchronize: %s", cudaGetErrorString(e));
            rc = CMT_ERR_CUDA;
        }
        for (int i = 0; i < n && rc == CMT_OK; ++i)
            solve_result(*cgs[i], iters ? iters + i : nullptr, final_rho ? final_rho + i : nullptr);
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (parent) cudaGraphDestroy(parent);
    restore();
    return rc;
}

// Solve W x = d from x (in: x0, out: solution) with at most maxiter iterations,
// scipy's stopping rule ||r|| < max(atol, rtol ||d||).  use_graph replays one captured
// iteration (the first call captures; capture happens outside any user capture).
extern "C" int cmt_cg_solve(cmt_cg *c, const void *d, void *x, int maxiter, double rtol, double atol, int use_graph,
                            int *iters, double *final_rho)
{
    CMT_CHECK_ARG(c && d && x, "null argument");
    CMT_CHECK_ARG(maxiter >= 0, "maxiter must be >= 0");
    CMT_CHECK_ARG(c->op == 0 || c->pair_plan, "pair operator without a plan");
    if (c->prec == 64)
        return solve_impl<double>(*c, (const double *)d, (double *)x, maxiter, rtol, atol, use_graph, iters, final_rho);
    return solve_impl<float>(*c, (const float *)d, (float *)x, maxiter, rtol, atol, use_graph, iters, final_rho);
}

// Run the solves of n solvers (same precision and device) together: d[i], x[i] as for
// cmt_cg_solve on cgs[i]; iters[i] / final_rho[i] optional (host arrays of n).  Used for the
// lambda sweep of cmtip/autocorrelation/autocorrelation_mpi.py:139-186, whose ranks solve
// the same data with different lambdas.
extern "C" int cmt_cg_solve_many(int n, cmt_cg *const *cgs, const void *const *d, void *const *x, int maxiter,
                                 double rtol, double atol, int *iters, double *final_rho)
{
    CMT_CHECK_ARG(n >= 1 && n <= 64 && cgs && d && x, "need 1..64 solvers and their d / x arrays");
    CMT_CHECK_ARG(maxiter >= 0, "maxiter must be >= 0");
    for (int i = 0; i < n; ++i) {
        CMT_CHECK_ARG(cgs[i] && d[i] && x[i], "null solver, d or x at %d", i);
        CMT_CHECK_ARG(cgs[i]->prec == cgs[0]->prec, "solvers of one call share a precision");
        CMT_CHECK_ARG(cgs[i]->op == 0 || cgs[i]->pair_plan, "pair operator without a plan at %d", i);
        for (int j = 0; j < i; ++j) {
            CMT_CHECK_ARG(cgs[j] != cgs[i], "solver %d given twice", i);
            CMT_CHECK_ARG(!cgs[i]->pair_plan || cgs[j]->pair_plan != cgs[i]->pair_plan,
                          "solvers %d and %d share a pair plan (its grids would race)", j, i);
        }
    }
    if (cgs[0]->prec == 64)
        return solve_many_impl<double>(n, cgs, d, x, maxiter, rtol, atol, iters, final_rho);
    return solve_many_impl<float>(n, cgs, d, x, maxiter, rtol, atol, iters, final_rho);
}

extern "C" int cmt_cg_destroy(cmt_cg *c)
{
    if (!c) return CMT_OK;
    cg_destroy(c);
    delete c;
    return CMT_OK;
}

// support = gaussian_filter(est, 0.5) > 1e-12 (float 0/1), est *= support in place when
// est_inplace is non-zero (autocorrelation.py:217-220).  scratch: 2 M^3 floats.
extern "C" int cmt_support_from_estimate(float *est, int M, float *support, float *scratch, int est_inplace,
                                         void *stream)
{
    CMT_CHECK_ARG(est && support && scratch && M > 0, "bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    int64_t m3 = (int64_t)M * M * M;
    // ndimage _gaussian_kernel1d(sigma=0.5, radius=2): normalised taps exp(-k^2 / (2 sigma^2))
    double phi[5], w[3];
    for (int k = -2; k <= 2; ++k) phi[k + 2] = exp(-0.5 / (0.5 * 0.5) * k * k);
    double tot = 0.0;
    for (double v : phi) tot += v;
    for (int k = 0; k <= 2; ++k) w[k] = phi[k + 2] / tot;
    float *a = scratch, *b = scratch + m3;
    unsigned gb = (unsigned)ceil_div(m3, 256);
    k_gauss_axis<<<gb, 256, 0, st>>>(est, a, M, 0, w[0], w[1], w[2]);
    k_gauss_axis<<<gb, 256, 0, st>>>(a, b, M, 1, w[0], w[1], w[2]);
    k_gauss_axis<<<gb, 256, 0, st>>>(b, a, M, 2, w[0], w[1], w[2]);
    k_threshold<<<gb, 256, 0, st>>>(a, support, est_inplace ? est : nullptr, m3, 1e-12);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

// ---------------------------------------------------------------- allocation-free variant
//
// Same computation as cmt_support_from_estimate, for callers that cannot allocate device
// memory: a host whose own pool has reserved the GPU's memory and forbids any other
// allocator from taking or returning blocks, or a latency-bound caller that cannot take
// the device-wide synchronisation a cudaMalloc / cudaFree may cause.  The two M^3 float
// grids of scratch live in a file-scope device array, so every GPU that loads the library
// holds CMT_NOALLOC_MAX_M^3 * 2 floats (16 MiB) until the process exits.
static __device__ __align__(256) float g_support_scratch[2 * CMT_NOALLOC_MAX_M * CMT_NOALLOC_MAX_M *
                                                         CMT_NOALLOC_MAX_M];

namespace {
std::mutex g_scratch_mu;
constexpr int kMaxDevices = 128;
float *g_scratch_ptr[kMaxDevices] = {};
}  // namespace

// Device address of the scratch array on the current device.  Host code only sees a
// host-side stand-in under the array's name, so the address is looked up once per
// device (with that device current) and cached by device ordinal; a cudaDeviceReset
// invalidates the cached address, and callers must not use this entry point after one.
static int scratch_address(float **out)
{
    int dev = 0;
    CMT_TRY_CUDA(cudaGetDevice(&dev));
    CMT_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        float *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_support_scratch);
        if (e != cudaSuccess) {
            set_error("cudaGetSymbolAddress of the support scratch: %s", cudaGetErrorString(e));
            return CMT_ERR_CUDA;
        }
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return CMT_OK;
}

extern "C" int cmt_support_from_estimate_noalloc(float *est, int M, float *support, int est_inplace, void *stream)
{
    CMT_CHECK_ARG(est && support, "null argument");
    CMT_CHECK_ARG(M > 0 && M <= CMT_NOALLOC_MAX_M,
                  "M = %d outside [1, %d]: the allocation-free support filter has a fixed scratch for grids of at "
                  "most %d^3 voxels (use cmt_support_from_estimate with caller scratch)",
                  M, CMT_NOALLOC_MAX_M, CMT_NOALLOC_MAX_M);
    float *scratch = nullptr;
    CMT_TRY(scratch_address(&scratch));
    cudaStream_t st = (cudaStream_t)stream;
    int64_t m3 = (int64_t)M * M * M;
    double phi[5], tot = 0.0;
    for (int k = -2; k <= 2; ++k) {
        phi[k + 2] = exp(-0.5 / (0.5 * 0.5) * k * k);
        tot += phi[k + 2];
    }
    // every pass writes all M^3 entries of its scratch grid before the next one reads it,
    // so nothing left from an earlier call is read and no clearing is needed
    float *a = scratch, *b = scratch + m3;
    unsigned gb = (unsigned)ceil_div(m3, 256);
    k_gauss_axis<<<gb, 256, 0, st>>>(est, a, M, 0, phi[2] / tot, phi[3] / tot, phi[4] / tot);
    k_gauss_axis<<<gb, 256, 0, st>>>(a, b, M, 1, phi[2] / tot, phi[3] / tot, phi[4] / tot);
    k_gauss_axis<<<gb, 256, 0, st>>>(b, a, M, 2, phi[2] / tot, phi[3] / tot, phi[4] / tot);
    k_threshold<<<gb, 256, 0, st>>>(a, support, est_inplace ? est : nullptr, m3, 1e-12);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}
