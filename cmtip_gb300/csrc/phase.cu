// Phase retrieval of an oversampled autocorrelation on the device
// (cmtip/phasing/phase.py:11-219): amplitudes from the filtered autocorrelation
// (phase.py:186-192), the initial support (create_support_, :47-64), Error Reduction and
// Hybrid Input-Output iterations (ER :83-99, HIO :102-119, step_phase :122-144), shrink-wrap
// (:147-162), recentring (center_of_mass / recenter, :11-44) and the phased autocorrelation
// (:214-217).
//
// The reference works on full complex M^3 spectra of real densities and keeps
// Re(ifftn(...)).  Here every transform is real-to-complex / complex-to-real on the
// Hermitian half (M x M x (M/2+1)): the projection kernel forms the Hermitian part of the
// reference's modified spectrum from the element and its mirror, which is exactly what
// taking the real part of the inverse transform does, for any amplitude array and mask.
// One iteration (R2C, projection, C2R, density update) has no host synchronisation and is
// captured once into a CUDA graph and replayed.  The Gaussian filters follow
// scipy.ndimage.gaussian_filter: one axis per pass in order 0, 1, 2, double line arithmetic
// with the taps of a symmetric kernel added outermost first, each pass rounded to the
// array's type, 'constant' (zero) or 'wrap' boundaries.
#include <algorithm>
#include <cmath>
#include <new>

#include "cmt_common.cuh"

namespace cmt {

constexpr int PH_THREADS = 256;
constexpr int PH_RED_BLOCKS = 304;  // 2 x 152 SMs
constexpr int PH_MAX_RADIUS = 8;

struct PhFilter {
    double w[PH_MAX_RADIUS + 1];  // w[d]: weight at distance d
    int radius;
};

struct PhGraph {
    cudaGraphExec_t exec = nullptr;
    const void *key[6] = {};
    double beta = 0, rho_max = 0;
    int kind = -1;
};

struct Phaser {
    int M = 0, prec = 64;
    int64_t m3 = 0, hn = 0;  // M^3, M * M * (M/2 + 1)
    cudaStream_t stream = nullptr, cap = nullptr;
    void *spec = nullptr;     // hn complex double (also used as complex float)
    void *rmod = nullptr;     // m3 of the precision: modulus-projected density / roll scratch
    double *fa = nullptr, *fb = nullptr;  // m3 double: filter passes, final transform
    uint8_t *tmp8 = nullptr;  // m3 bytes: support roll scratch
    double *partial = nullptr;  // 4 * PH_RED_BLOCKS
    double *scal = nullptr;     // 4 device scalars
    cufftHandle d2z = 0, z2d = 0, r2c = 0, c2r = 0;
    bool have64 = false, have32 = false;
    PhGraph graphs[2];
};

}  // namespace cmt

struct cmt_phaser : cmt::Phaser {};

namespace cmt {

__device__ __forceinline__ double ph_sqrt(double x) { return __dsqrt_rn(x); }
__device__ __forceinline__ float ph_sqrt(float x) { return __fsqrt_rn(x); }
__device__ __forceinline__ double ph_hypot(double a, double b) { return hypot(a, b); }
__device__ __forceinline__ float ph_hypot(float a, float b) { return hypotf(a, b); }
__device__ __forceinline__ double ph_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float ph_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double ph_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float ph_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double ph_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float ph_sub(float a, float b) { return __fsub_rn(a, b); }

// Modulus projection of step_phase (phase.py:136-142) on the half spectrum, with the
// inverse transform's 1/M^3.  The reference's modified spectrum X(k) is amp(k) e^{i phi(k)}
// where the mask is set and the density's spectrum z(k) elsewhere; Re(ifftn(X)) equals the
// inverse of its Hermitian part (X(k) + conj(X(-k))) / 2.  With z(-k) = conj(z(k)) that is
// e^{i phi(k)} (a(k) + a(-k)) / 2, a = amp where masked and |z| where not; phi(0 + 0i) = 0
// as numpy's angle.
template <typename T>
__global__ void k_project(cplx_t<T> *spec, const T *amp, const uint8_t *mask, int M, T scale)
{
    int hz = M / 2 + 1;
    int64_t hn = (int64_t)M * M * hz;
    int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= hn) return;
    int k = (int)(h % hz);
    int64_t r = h / hz;
    int j = (int)(r % M), i = (int)(r / M);
    int64_t f = ((int64_t)i * M + j) * M + k;
    int64_t g = ((int64_t)((M - i) % M) * M + (M - j) % M) * M + (M - k) % M;
    cplx_t<T> z = spec[h];
    bool mf = mask[f] != 0, mg = mask[g] != 0;
    cplx_t<T> out;
    if (!mf && !mg) {
        out.x = ph_mul(z.x, scale);
        out.y = ph_mul(z.y, scale);
    } else {
        T mag = ph_hypot(z.x, z.y);
        T ux = mag > (T)0 ? z.x / mag : (T)1, uy = mag > (T)0 ? z.y / mag : (T)0;
        T a = (mf && mg) ? (amp[f] == amp[g] ? amp[f] : ph_mul(ph_add(amp[f], amp[g]), (T)0.5))
                         : ph_mul(ph_add(mf ? amp[f] : mag, mg ? amp[g] : mag), (T)0.5);
        T s = ph_mul(a, scale);
        out.x = ph_mul(ux, s);
        out.y = ph_mul(uy, s);
    }
    spec[h] = out;
}

// ER density update (phase.py:97-99): support* = support & rho_mod > 0.
template <typename T>
__global__ void k_update_er(T *rho, const T *rmod, const uint8_t *support, int64_t n, T rho_max)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T m = rmod[i];
    T r = (support[i] != 0 && m > (T)0) ? m : (T)0;
    if (m > rho_max) r = rho_max;
    rho[i] = r;
}

// HIO density update (phase.py:117-119).
template <typename T>
__global__ void k_update_hio(T *rho, const T *rmod, const uint8_t *support, int64_t n, T beta, T rho_max)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T m = rmod[i];
    T r = (support[i] != 0 && m > (T)0) ? m : ph_sub(rho[i], ph_mul(beta, m));
    if (m > rho_max) r = ph_add(r, ph_sub(ph_mul(ph_mul((T)2, beta), m), rho_max));
    rho[i] = r;
}

// step_phase's support* output (phase.py:143).
template <typename T>
__global__ void k_support_star(const T *rmod, const uint8_t *support, uint8_t *star, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    star[i] = (support[i] != 0 && rmod[i] > (T)0) ? 1 : 0;
}

// One pass of scipy.ndimage.gaussian_filter along `axis`.  pre: 0 none, 1 |x|, 2 max(x, 0)
// on the loaded samples (first pass only).  wrap: periodic boundary, else zeros.
// shift_out: write element c at (c + M - M/2) mod M on every axis (ifftshift).
template <typename TI, typename TO>
__global__ void k_filter_axis(const TI *in, TO *out, int M, int axis, int wrap, int pre, PhFilter fw, int shift_out)
{
    int64_t m3 = (int64_t)M * M * M;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m3) return;
    int c0 = (int)(i / ((int64_t)M * M)), c1 = (int)((i / M) % M), c2 = (int)(i % M);
    int pos = axis == 0 ? c0 : (axis == 1 ? c1 : c2);
    int64_t stride = axis == 0 ? (int64_t)M * M : (axis == 1 ? M : 1);
    const TI *base = in + (i - (int64_t)pos * stride);
    auto load = [&](int p) -> double {
        if (wrap) {
            p %= M;
            if (p < 0) p += M;
        } else if (p < 0 || p >= M) {
            return 0.0;
        }
        double v = (double)base[(int64_t)p * stride];
        if (pre == 1) v = fabs(v);
        else if (pre == 2) v = v < 0.0 ? 0.0 : v;
        return v;
    };
    double t = __dmul_rn(load(pos), fw.w[0]);
    for (int d = fw.radius; d >= 1; --d) t = __dadd_rn(t, __dmul_rn(__dadd_rn(load(pos - d), load(pos + d)), fw.w[d]));
    int64_t o = i;
    if (shift_out) {
        int s = M - M / 2;
        o = ((int64_t)((c0 + s) % M) * M + (c1 + s) % M) * M + (c2 + s) % M;
    }
    out[o] = (TO)t;
}

// amplitudes_ = sqrt(|fftn(ac_filt_)|) on the full M^3 grid from the D2Z half spectrum
// (phase.py:190-192); elements past the half are the mirrored ones' magnitudes.
template <typename TO>
__global__ void k_amplitudes(const double2 *spec, TO *amp, int M)
{
    int64_t m3 = (int64_t)M * M * M;
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m3) return;
    int hz = M / 2 + 1;
    int k = (int)(f % M);
    int64_t r = f / M;
    int j = (int)(r % M), i = (int)(r / M);
    int64_t h = k < hz ? ((int64_t)i * M + j) * hz + k : ((int64_t)((M - i) % M) * M + (M - j) % M) * hz + (M - k);
    double2 z = spec[h];
    amp[f] = (TO)__dsqrt_rn(hypot(z.x, z.y));
}

// create_support_ (phase.py:57-64): centred cube [Mquat, M - Mquat)^3 (empty for Mquat = 0,
// as slice(0, -0)), ifftshifted, and ac_filt_ > 1e-2 * max(ac_filt_).
__global__ void k_create_support(const double *acf, int M, int mquat, const double *maxv, uint8_t *sup)
{
    int64_t m3 = (int64_t)M * M * M;
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m3) return;
    int c[3] = {(int)(f / ((int64_t)M * M)), (int)((f / M) % M), (int)(f % M)};
    bool in = mquat > 0;
    for (int a = 0; a < 3; ++a) {
        int cc = (c[a] + M / 2) % M;  // ifftshift: element f holds centred index (f + M/2) mod M
        in = in && cc >= mquat && cc < M - mquat;
    }
    sup[f] = (in && acf[f] > __dmul_rn(1e-2, *maxv)) ? 1 : 0;
}

// shrink_wrap threshold (phase.py:162): filtered |rho| > max|rho| * cutoff, in the array type.
template <typename T>
__global__ void k_wrap_threshold(const T *filt, const double *maxabs, double cutoff, uint8_t *sup, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T thr = ph_mul((T)*maxabs, (T)cutoff);
    sup[i] = filt[i] > thr ? 1 : 0;
}

__device__ __forceinline__ double nanmax(double a, double b) { return (b > a || b != b) ? b : a; }

// Block partial of max(x) (absval: max|x|), NaN-propagating as numpy's max.
template <typename T>
__global__ void __launch_bounds__(PH_THREADS) k_max_partial(const T *a, int64_t n, int absval, double *partial)
{
    __shared__ double s[PH_THREADS / 32];
    double m = -INFINITY;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = (double)a[i];
        m = nanmax(m, absval ? fabs(v) : v);
    }
    for (int o = 16; o > 0; o >>= 1) m = nanmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = s[0];
        for (int w = 1; w < PH_THREADS / 32; ++w) t = nanmax(t, s[w]);
        partial[blockIdx.x] = t;
    }
}

__global__ void k_max_final(const double *partial, int nb, double *out)
{
    if (threadIdx.x != 0) return;
    double t = -INFINITY;
    for (int b = 0; b < nb; ++b) t = nanmax(t, partial[b]);
    *out = t;
}

// numpy.linspace(-1, 1, M + 1) edge k: k * (2 / M) + (-1), the last edge exactly 1.
__device__ __forceinline__ double lin_edge(int k, int M)
{
    return k == M ? 1.0 : __dadd_rn(__dmul_rn((double)k, 2.0 / (double)M), -1.0);
}

// center_of_mass sums (phase.py:20-22): sum |rho| * hkl_a (a = 0, 1, 2) and sum |rho|, with
// hkl_ either given (3 x M^3, FFT order) or recenter's grid (phase.py:34-38): ifftshifted
// midpoints of linspace(-1, 1, M + 1).  Block partials, reduced in a fixed order.
template <typename T>
__global__ void __launch_bounds__(PH_THREADS) k_com_partial(const T *rho, const double *hkl, int M, double *partial)
{
    __shared__ double s[4][PH_THREADS / 32];
    int64_t m3 = (int64_t)M * M * M;
    double acc[4] = {0, 0, 0, 0};
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < m3; f += (int64_t)gridDim.x * blockDim.x) {
        double v = fabs((double)rho[f]);
        double h[3];
        if (hkl) {
            h[0] = hkl[f];
            h[1] = hkl[m3 + f];
            h[2] = hkl[2 * m3 + f];
        } else {
            int c[3] = {(int)(f / ((int64_t)M * M)), (int)((f / M) % M), (int)(f % M)};
            for (int a = 0; a < 3; ++a) {
                int k = (c[a] + M / 2) % M;
                h[a] = __dmul_rn(__dadd_rn(lin_edge(k, M), lin_edge(k + 1, M)), 0.5);
            }
        }
        for (int a = 0; a < 3; ++a) acc[a] += __dmul_rn(v, h[a]);
        acc[3] += v;
    }
    for (int q = 0; q < 4; ++q) {
        double t = acc[q];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if ((threadIdx.x & 31) == 0) s[q][threadIdx.x >> 5] = t;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < PH_THREADS / 32; ++w) t += s[threadIdx.x][w];
        partial[4 * blockIdx.x + threadIdx.x] = t;
    }
}

__global__ void k_com_final(const double *partial, int nb, double *out)
{
    if (threadIdx.x >= 4) return;
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += partial[4 * b + threadIdx.x];
    out[threadIdx.x] = t;
}

// np.roll(a, -s_a, a) on all three axes: dst[j] = src[(j + s) mod M].
template <typename T>
__global__ void k_roll(const T *src, T *dst, int M, int s0, int s1, int s2)
{
    int64_t m3 = (int64_t)M * M * M;
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m3) return;
    int c0 = (int)(f / ((int64_t)M * M)), c1 = (int)((f / M) % M), c2 = (int)(f % M);
    int64_t g = ((int64_t)((c0 + s0) % M) * M + (c1 + s1) % M) * M + (c2 + s2) % M;
    dst[f] = src[g];
}

template <typename T>
__global__ void k_to_double(const T *a, double *b, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (double)a[i];
}

// |z|^2 / M^3 as a real spectrum (phase.py:214 and the 1/M^3 of :216's ifftn).
__global__ void k_abs2_half(double2 *spec, int64_t hn, double scale)
{
    int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= hn) return;
    double2 z = spec[h];
    double a = hypot(z.x, z.y);
    spec[h] = make_double2(__dmul_rn(__dmul_rn(a, a), scale), 0.0);
}

// ac_phased = fftshift(|ac_phased_|) (phase.py:216-217): element c reads (c + M - M/2) mod M.
__global__ void k_abs_fftshift(const double *in, double *out, int M)
{
    int64_t m3 = (int64_t)M * M * M;
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m3) return;
    int s = M - M / 2;
    int c0 = (int)(c / ((int64_t)M * M)), c1 = (int)((c / M) % M), c2 = (int)(c % M);
    int64_t g = ((int64_t)((c0 + s) % M) * M + (c1 + s) % M) * M + (c2 + s) % M;
    out[c] = fabs(in[g]);
}

// ---------------------------------------------------------------- host

static int blocks_for(int64_t n) { return (int)std::max<int64_t>((n + PH_THREADS - 1) / PH_THREADS, 1); }

static void phaser_free(Phaser *p)
{
    void *bufs[] = {p->spec, p->rmod, p->fa, p->fb, p->tmp8, p->partial, p->scal};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (p->have64) {
        cufftDestroy(p->d2z);
        cufftDestroy(p->z2d);
    }
    if (p->have32) {
        cufftDestroy(p->r2c);
        cufftDestroy(p->c2r);
    }
    for (auto &g : p->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (p->cap) cudaStreamDestroy(p->cap);
}

static int route_fft(Phaser &p, cudaStream_t s)
{
    CMT_TRY_CUFFT(cufftSetStream(p.d2z, s));
    CMT_TRY_CUFFT(cufftSetStream(p.z2d, s));
    if (p.have32) {
        CMT_TRY_CUFFT(cufftSetStream(p.r2c, s));
        CMT_TRY_CUFFT(cufftSetStream(p.c2r, s));
    }
    return CMT_OK;
}

static int fft_forward(Phaser &p, const void *rho)
{
    if (p.prec == 64) CMT_TRY_CUFFT(cufftExecD2Z(p.d2z, (double *)rho, (cufftDoubleComplex *)p.spec));
    else CMT_TRY_CUFFT(cufftExecR2C(p.r2c, (float *)rho, (cufftComplex *)p.spec));
    return CMT_OK;
}

static int fft_inverse(Phaser &p, void *out)
{
    if (p.prec == 64) CMT_TRY_CUFFT(cufftExecZ2D(p.z2d, (cufftDoubleComplex *)p.spec, (double *)out));
    else CMT_TRY_CUFFT(cufftExecC2R(p.c2r, (cufftComplex *)p.spec, (float *)out));
    return CMT_OK;
}

enum { PH_ER = 0, PH_HIO = 1, PH_STEP = 2 };

// One step_phase followed by the ER / HIO update, on stream st.  For PH_STEP the modulus
// projection lands in rmod_out and support* in star.
template <typename T>
static int iteration(Phaser &p, cudaStream_t st, int kind, T *rho, const T *amp, const uint8_t *mask,
                     const uint8_t *support, double beta, double rho_max, T *rmod_out, uint8_t *star)
{
    int M = p.M;
    CMT_TRY(fft_forward(p, rho));
    k_project<T><<<blocks_for(p.hn), PH_THREADS, 0, st>>>((cplx_t<T> *)p.spec, amp, mask, M,
                                                         (T)(1.0 / ((double)M * M * M)));
    CMT_LAUNCH_CHECK();
    T *rm = kind == PH_STEP ? rmod_out : (T *)p.rmod;
    CMT_TRY(fft_inverse(p, rm));
    int g = blocks_for(p.m3);
    if (kind == PH_ER) k_update_er<T><<<g, PH_THREADS, 0, st>>>(rho, rm, support, p.m3, (T)rho_max);
    else if (kind == PH_HIO) k_update_hio<T><<<g, PH_THREADS, 0, st>>>(rho, rm, support, p.m3, (T)beta, (T)rho_max);
    else k_support_star<T><<<g, PH_THREADS, 0, st>>>(rm, support, star, p.m3);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

template <typename T>
static int run_loops(Phaser &p, int kind, T *rho, const T *amp, const uint8_t *mask, const uint8_t *support,
                     double beta, double rho_max, int n_loops)
{
    if (n_loops <= 0) return CMT_OK;
    PhGraph &g = p.graphs[kind];
    const void *key[6] = {rho, amp, mask, support, nullptr, nullptr};
    bool same = g.exec && g.kind == kind && g.beta == beta && g.rho_max == rho_max;
    for (int i = 0; same && i < 6; ++i) same = g.key[i] == key[i];
    if (!same) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        if (!p.cap) CMT_TRY_CUDA(cudaStreamCreateWithFlags(&p.cap, cudaStreamNonBlocking));
        CMT_TRY(route_fft(p, p.cap));
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(p.cap, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? iteration<T>(p, p.cap, kind, rho, amp, mask, support, beta, rho_max, nullptr, nullptr)
                                  : CMT_ERR_CUDA;
        cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(p.cap, &graph) : e;
        int rc2 = route_fft(p, p.stream);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            set_error("phasing graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
            if (graph) cudaGraphDestroy(graph);
            return CMT_ERR_CUDA;
        }
        if (rc != CMT_OK || rc2 != CMT_OK) {
            cudaGraphDestroy(graph);
            return rc != CMT_OK ? rc : rc2;
        }
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        CMT_TRY_CUDA(e);
        g.kind = kind;
        g.beta = beta;
        g.rho_max = rho_max;
        for (int i = 0; i < 6; ++i) g.key[i] = key[i];
    }
    for (int it = 0; it < n_loops; ++it) CMT_TRY_CUDA(cudaGraphLaunch(g.exec, p.stream));
    return CMT_OK;
}

static int make_filter(const double *weights, int radius, PhFilter *fw)
{
    CMT_CHECK_ARG(weights && radius >= 0 && radius <= PH_MAX_RADIUS,
                  "filter radius %d outside [0, %d] (truncate * sigma too large)", radius, PH_MAX_RADIUS);
    for (int d = 0; d <= radius; ++d) fw->w[d] = weights[radius + d];
    fw->radius = radius;
    return CMT_OK;
}

static int max_into(Phaser &p, const void *a, bool dbl, int absval, double *out)
{
    cudaStream_t st = p.stream;
    if (dbl) k_max_partial<double><<<PH_RED_BLOCKS, PH_THREADS, 0, st>>>((const double *)a, p.m3, absval, p.partial);
    else k_max_partial<float><<<PH_RED_BLOCKS, PH_THREADS, 0, st>>>((const float *)a, p.m3, absval, p.partial);
    k_max_final<<<1, 32, 0, st>>>(p.partial, PH_RED_BLOCKS, out);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

}  // namespace cmt

using namespace cmt;

extern "C" int cmt_phase_create(int M, int prec, void *stream, cmt_phaser **out)
{
    CMT_CHECK_ARG(out, "null output pointer");
    *out = nullptr;
    CMT_CHECK_ARG(M >= 1 && M <= 1024, "M must be in [1, 1024]");
    CMT_CHECK_ARG(prec == 32 || prec == 64, "prec must be 32 or 64");
    cmt_phaser *p = new (std::nothrow) cmt_phaser();
    if (!p) return CMT_ERR_OOM;
    p->M = M;
    p->prec = prec;
    p->stream = (cudaStream_t)stream;
    p->m3 = (int64_t)M * M * M;
    p->hn = (int64_t)M * M * (M / 2 + 1);
    size_t e = prec == 64 ? 8 : 4;
    auto fail = [&](int code) {
        phaser_free(p);
        delete p;
        return code;
    };
    struct A {
        void **ptr;
        size_t n;
    } allocs[] = {{&p->spec, 16 * (size_t)p->hn},       {&p->rmod, e * (size_t)p->m3},
                  {(void **)&p->fa, 8 * (size_t)p->m3}, {(void **)&p->fb, 8 * (size_t)p->m3},
                  {(void **)&p->tmp8, (size_t)p->m3},   {(void **)&p->partial, 8 * 4 * (size_t)PH_RED_BLOCKS},
                  {(void **)&p->scal, 8 * 4}};
    for (auto &a : allocs) {
        cudaError_t err = cudaMalloc(a.ptr, a.n);
        if (err != cudaSuccess) {
            set_error("phasing allocation of %zu bytes: %s", a.n, cudaGetErrorString(err));
            return fail(CMT_ERR_OOM);
        }
    }
    if (cufftPlan3d(&p->d2z, M, M, M, CUFFT_D2Z) != CUFFT_SUCCESS) {
        set_error("cuFFT D2Z plan M^3 failed");
        return fail(CMT_ERR_CUFFT);
    }
    if (cufftPlan3d(&p->z2d, M, M, M, CUFFT_Z2D) != CUFFT_SUCCESS) {
        cufftDestroy(p->d2z);
        set_error("cuFFT Z2D plan M^3 failed");
        return fail(CMT_ERR_CUFFT);
    }
    p->have64 = true;
    if (prec == 32) {
        if (cufftPlan3d(&p->r2c, M, M, M, CUFFT_R2C) != CUFFT_SUCCESS) {
            set_error("cuFFT R2C plan M^3 failed");
            return fail(CMT_ERR_CUFFT);
        }
        if (cufftPlan3d(&p->c2r, M, M, M, CUFFT_C2R) != CUFFT_SUCCESS) {
            cufftDestroy(p->r2c);
            set_error("cuFFT C2R plan M^3 failed");
            return fail(CMT_ERR_CUFFT);
        }
        p->have32 = true;
    }
    int rc = route_fft(*p, p->stream);
    if (rc != CMT_OK) return fail(rc);
    *out = p;
    return CMT_OK;
}

extern "C" int cmt_phase_set_stream(cmt_phaser *p, void *stream)
{
    CMT_CHECK_ARG(p, "null phaser");
    p->stream = (cudaStream_t)stream;
    return route_fft(*p, p->stream);
}

extern "C" int cmt_phase_amplitudes(cmt_phaser *p, const double *ac, const double *weights, int radius,
                                    double *ac_filt_, void *amplitudes_)
{
    CMT_CHECK_ARG(p && ac && ac_filt_ && amplitudes_, "null argument");
    PhFilter fw;
    CMT_TRY(make_filter(weights, radius, &fw));
    cudaStream_t st = p->stream;
    int M = p->M, g = blocks_for(p->m3);
    k_filter_axis<double, double><<<g, PH_THREADS, 0, st>>>(ac, p->fa, M, 0, 0, 2, fw, 0);
    k_filter_axis<double, double><<<g, PH_THREADS, 0, st>>>(p->fa, p->fb, M, 1, 0, 0, fw, 0);
    k_filter_axis<double, double><<<g, PH_THREADS, 0, st>>>(p->fb, ac_filt_, M, 2, 0, 0, fw, 1);
    CMT_LAUNCH_CHECK();
    CMT_TRY_CUFFT(cufftExecD2Z(p->d2z, (double *)ac_filt_, (cufftDoubleComplex *)p->spec));
    if (p->prec == 64) k_amplitudes<double><<<g, PH_THREADS, 0, st>>>((const double2 *)p->spec, (double *)amplitudes_, M);
    else k_amplitudes<float><<<g, PH_THREADS, 0, st>>>((const double2 *)p->spec, (float *)amplitudes_, M);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

extern "C" int cmt_phase_create_support(cmt_phaser *p, const double *ac_filt_, int mquat, uint8_t *support_)
{
    CMT_CHECK_ARG(p && ac_filt_ && support_, "null argument");
    CMT_CHECK_ARG(mquat >= 0, "Mquat must be non-negative");
    CMT_TRY(max_into(*p, ac_filt_, true, 0, p->scal));
    k_create_support<<<blocks_for(p->m3), PH_THREADS, 0, p->stream>>>(ac_filt_, p->M, mquat, p->scal, support_);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

extern "C" int cmt_phase_step(cmt_phaser *p, const void *rho_, const void *amplitudes_, const uint8_t *amp_mask_,
                              const uint8_t *support_, void *rho_mod_, uint8_t *support_star_)
{
    CMT_CHECK_ARG(p && rho_ && amplitudes_ && amp_mask_ && support_ && rho_mod_ && support_star_, "null argument");
    if (p->prec == 64)
        return iteration<double>(*p, p->stream, PH_STEP, (double *)rho_, (const double *)amplitudes_, amp_mask_,
                                 support_, 0.0, 0.0, (double *)rho_mod_, support_star_);
    return iteration<float>(*p, p->stream, PH_STEP, (float *)rho_, (const float *)amplitudes_, amp_mask_, support_,
                            0.0, 0.0, (float *)rho_mod_, support_star_);
}

extern "C" int cmt_phase_er(cmt_phaser *p, void *rho_, const void *amplitudes_, const uint8_t *amp_mask_,
                            const uint8_t *support_, double rho_max, int n_loops)
{
    CMT_CHECK_ARG(p && rho_ && amplitudes_ && amp_mask_ && support_, "null argument");
    CMT_CHECK_ARG(n_loops >= 0, "n_loops must be non-negative");
    if (p->prec == 64)
        return run_loops<double>(*p, PH_ER, (double *)rho_, (const double *)amplitudes_, amp_mask_, support_, 0.0,
                                 rho_max, n_loops);
    return run_loops<float>(*p, PH_ER, (float *)rho_, (const float *)amplitudes_, amp_mask_, support_, 0.0, rho_max,
                            n_loops);
}

extern "C" int cmt_phase_hio(cmt_phaser *p, double beta, void *rho_, const void *amplitudes_,
                             const uint8_t *amp_mask_, const uint8_t *support_, double rho_max, int n_loops)
{
    CMT_CHECK_ARG(p && rho_ && amplitudes_ && amp_mask_ && support_, "null argument");
    CMT_CHECK_ARG(n_loops >= 0, "n_loops must be non-negative");
    if (p->prec == 64)
        return run_loops<double>(*p, PH_HIO, (double *)rho_, (const double *)amplitudes_, amp_mask_, support_, beta,
                                 rho_max, n_loops);
    return run_loops<float>(*p, PH_HIO, (float *)rho_, (const float *)amplitudes_, amp_mask_, support_, beta, rho_max,
                            n_loops);
}

extern "C" int cmt_phase_shrink_wrap(cmt_phaser *p, double cutoff, const double *weights, int radius,
                                     const void *rho_, uint8_t *support_)
{
    CMT_CHECK_ARG(p && rho_ && support_, "null argument");
    PhFilter fw;
    CMT_TRY(make_filter(weights, radius, &fw));
    cudaStream_t st = p->stream;
    int M = p->M, g = blocks_for(p->m3);
    if (p->prec == 64) {
        double *a = p->fa, *b = p->fb;
        k_filter_axis<double, double><<<g, PH_THREADS, 0, st>>>((const double *)rho_, a, M, 0, 1, 1, fw, 0);
        k_filter_axis<double, double><<<g, PH_THREADS, 0, st>>>(a, b, M, 1, 1, 0, fw, 0);
        k_filter_axis<double, double><<<g, PH_THREADS, 0, st>>>(b, a, M, 2, 1, 0, fw, 0);
        CMT_LAUNCH_CHECK();
        CMT_TRY(max_into(*p, rho_, true, 1, p->scal));
        k_wrap_threshold<double><<<g, PH_THREADS, 0, st>>>(a, p->scal, cutoff, support_, p->m3);
    } else {
        float *a = (float *)p->fa, *b = (float *)p->fb;
        k_filter_axis<float, float><<<g, PH_THREADS, 0, st>>>((const float *)rho_, a, M, 0, 1, 1, fw, 0);
        k_filter_axis<float, float><<<g, PH_THREADS, 0, st>>>(a, b, M, 1, 1, 0, fw, 0);
        k_filter_axis<float, float><<<g, PH_THREADS, 0, st>>>(b, a, M, 2, 1, 0, fw, 0);
        CMT_LAUNCH_CHECK();
        CMT_TRY(max_into(*p, rho_, false, 1, p->scal));
        k_wrap_threshold<float><<<g, PH_THREADS, 0, st>>>(a, p->scal, cutoff, support_, p->m3);
    }
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

extern "C" int cmt_phase_center_of_mass(cmt_phaser *p, const void *rho_, const double *hkl_, double *sums)
{
    CMT_CHECK_ARG(p && rho_ && sums, "null argument");
    cudaStream_t st = p->stream;
    if (p->prec == 64)
        k_com_partial<double><<<PH_RED_BLOCKS, PH_THREADS, 0, st>>>((const double *)rho_, hkl_, p->M, p->partial);
    else
        k_com_partial<float><<<PH_RED_BLOCKS, PH_THREADS, 0, st>>>((const float *)rho_, hkl_, p->M, p->partial);
    k_com_final<<<1, 32, 0, st>>>(p->partial, PH_RED_BLOCKS, sums);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

extern "C" int cmt_phase_roll(cmt_phaser *p, void *rho_, uint8_t *support_, int s0, int s1, int s2)
{
    CMT_CHECK_ARG(p, "null phaser");
    cudaStream_t st = p->stream;
    int M = p->M, g = blocks_for(p->m3);
    auto norm = [M](int s) { return ((s % M) + M) % M; };
    s0 = norm(s0);
    s1 = norm(s1);
    s2 = norm(s2);
    if (rho_) {
        size_t bytes = (p->prec == 64 ? 8 : 4) * (size_t)p->m3;
        CMT_TRY_CUDA(cudaMemcpyAsync(p->rmod, rho_, bytes, cudaMemcpyDeviceToDevice, st));
        if (p->prec == 64) k_roll<double><<<g, PH_THREADS, 0, st>>>((const double *)p->rmod, (double *)rho_, M, s0, s1, s2);
        else k_roll<float><<<g, PH_THREADS, 0, st>>>((const float *)p->rmod, (float *)rho_, M, s0, s1, s2);
        CMT_LAUNCH_CHECK();
    }
    if (support_) {
        CMT_TRY_CUDA(cudaMemcpyAsync(p->tmp8, support_, (size_t)p->m3, cudaMemcpyDeviceToDevice, st));
        k_roll<uint8_t><<<g, PH_THREADS, 0, st>>>(p->tmp8, support_, M, s0, s1, s2);
        CMT_LAUNCH_CHECK();
    }
    return CMT_OK;
}

extern "C" int cmt_phase_autocorrelation(cmt_phaser *p, const void *rho_, double *ac_phased)
{
    CMT_CHECK_ARG(p && rho_ && ac_phased, "null argument");
    cudaStream_t st = p->stream;
    int M = p->M, g = blocks_for(p->m3);
    const double *r = (const double *)rho_;
    if (p->prec == 32) {
        k_to_double<float><<<g, PH_THREADS, 0, st>>>((const float *)rho_, p->fa, p->m3);
        CMT_LAUNCH_CHECK();
        r = p->fa;
    }
    CMT_TRY_CUFFT(cufftExecD2Z(p->d2z, (double *)r, (cufftDoubleComplex *)p->spec));
    k_abs2_half<<<blocks_for(p->hn), PH_THREADS, 0, st>>>((double2 *)p->spec, p->hn, 1.0 / ((double)M * M * M));
    CMT_LAUNCH_CHECK();
    CMT_TRY_CUFFT(cufftExecZ2D(p->z2d, (cufftDoubleComplex *)p->spec, p->fb));
    k_abs_fftshift<<<g, PH_THREADS, 0, st>>>(p->fb, ac_phased, M);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

extern "C" int cmt_phase_destroy(cmt_phaser *p)
{
    if (!p) return CMT_OK;
    phaser_free(p);
    delete p;
    return CMT_OK;
}
