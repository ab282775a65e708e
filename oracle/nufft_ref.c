/*
 * ORACLE (test infrastructure only) -- FP64 CPU restatement of the spreading and
 * interpolation loops of a 3D exponential-of-semicircle (ES) kernel NUFFT.
 *
 * The reference (cmtip) delegates its NUFFTs to the third-party finufft library
 * (call sites: cmtip/nufft/forward.py:40 `nufft3d2`, cmtip/nufft/adjoint.py:33
 * `nufft3d1`; versions unpinned in setup.py:11).  finufft is not vendored in the
 * reference, so this file restates its published algorithm (Barnett, Magland and
 * af Klinteberg, "A parallel non-uniform fast Fourier transform library based on an
 * exponential of semicircle kernel", SIAM J. Sci. Comput. 41(5), 2019):
 *
 *   type 1:  b_l = sum_j c_j phi(u_j - l)      (spread, periodic fine grid of size n)
 *   type 2:  c_j = sum_l b_l phi(u_j - l)      (interpolate)
 *
 * with u_j = x_j * n / (2 pi) folded into [0, n) and
 * phi(t) = exp(beta * (sqrt(1 - (2t/w)^2) - 1)) for |t| <= w/2, else 0.
 * The FFT and deconvolution stages live in oracle/nufft.py (numpy).
 *
 * Only tests/, the smoke check and bench.py's CPU-baseline leg use this code.
 * Grids are C-ordered (axis 0 <-> x, axis 2 <-> z, fastest), complex values are
 * interleaved (re, im) doubles, matching numpy complex128.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXW 32
#define CMTO_PI 3.14159265358979323846

static inline double fold(double u, int n)
{
    /* map grid coordinate u to [0, n) */
    double r = u - (double)n * floor(u / (double)n);
    if (r >= (double)n) r -= (double)n;
    if (r < 0.0) r = 0.0;
    return r;
}

static inline void kernel_1d(double u, int w, double beta, int *l0, double *k)
{
    /* window starts at ceil(u - w/2); k[i] = phi(u - (l0 + i)) */
    int start = (int)ceil(u - 0.5 * (double)w);
    *l0 = start;
    double inv = 2.0 / (double)w;
    for (int i = 0; i < w; ++i) {
        double t = (u - (double)(start + i)) * inv;
        double s = 1.0 - t * t;
        k[i] = (s > 0.0) ? exp(beta * (sqrt(s) - 1.0)) : 0.0;
    }
}

static inline int wrap(int l, int n)
{
    l %= n;
    return l < 0 ? l + n : l;
}

/* type 1 spreading.  Thread t owns x-planes [t*n/T, (t+1)*n/T), so every grid cell
 * has one writer and no atomics are needed; each thread scans all points. */
void cmto_spread(int64_t N, const double *x, const double *y, const double *z,
                 const double *c, int n, int w, double beta, double *grid, int nthreads)
{
    const double scale = (double)n / (2.0 * CMTO_PI);
    memset(grid, 0, sizeof(double) * 2 * (size_t)n * n * n);
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        int T = 1, t = 0;
#ifdef _OPENMP
        T = omp_get_num_threads();
        t = omp_get_thread_num();
#endif
        int p0 = (int)((int64_t)t * n / T), p1 = (int)((int64_t)(t + 1) * n / T);
        double kx[MAXW], ky[MAXW], kz[MAXW];
        for (int64_t j = 0; j < N; ++j) {
            double ux = fold(x[j] * scale, n);
            int lx;
            int start = (int)ceil(ux - 0.5 * (double)w);
            /* quick rejection: does the x-window touch [p0, p1)? */
            int hit = 0;
            for (int i = 0; i < w; ++i) {
                int q = wrap(start + i, n);
                if (q >= p0 && q < p1) { hit = 1; break; }
            }
            if (!hit) continue;
            kernel_1d(ux, w, beta, &lx, kx);
            double uy = fold(y[j] * scale, n), uz = fold(z[j] * scale, n);
            int ly, lz;
            kernel_1d(uy, w, beta, &ly, ky);
            kernel_1d(uz, w, beta, &lz, kz);
            double cr = c[2 * j], ci = c[2 * j + 1];
            for (int a = 0; a < w; ++a) {
                int ia = wrap(lx + a, n);
                if (ia < p0 || ia >= p1) continue;
                double va = kx[a];
                for (int b = 0; b < w; ++b) {
                    int ib = wrap(ly + b, n);
                    double vab = va * ky[b];
                    double *row = grid + 2 * ((size_t)ia * n + ib) * n;
                    for (int e = 0; e < w; ++e) {
                        int ie = wrap(lz + e, n);
                        double v = vab * kz[e];
                        row[2 * ie] += v * cr;
                        row[2 * ie + 1] += v * ci;
                    }
                }
            }
        }
    }
}

/* type 2 interpolation, parallel over points. */
void cmto_interp(int64_t N, const double *x, const double *y, const double *z,
                 int n, int w, double beta, const double *grid, double *c, int nthreads)
{
    const double scale = (double)n / (2.0 * CMTO_PI);
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t j = 0; j < N; ++j) {
        double kx[MAXW], ky[MAXW], kz[MAXW];
        int lx, ly, lz;
        kernel_1d(fold(x[j] * scale, n), w, beta, &lx, kx);
        kernel_1d(fold(y[j] * scale, n), w, beta, &ly, ky);
        kernel_1d(fold(z[j] * scale, n), w, beta, &lz, kz);
        int iz[MAXW];
        for (int e = 0; e < w; ++e) iz[e] = wrap(lz + e, n);
        double sr = 0.0, si = 0.0;
        for (int a = 0; a < w; ++a) {
            int ia = wrap(lx + a, n);
            for (int b = 0; b < w; ++b) {
                int ib = wrap(ly + b, n);
                const double *row = grid + 2 * ((size_t)ia * n + ib) * n;
                double rr = 0.0, ri = 0.0;
                for (int e = 0; e < w; ++e) {
                    rr += kz[e] * row[2 * iz[e]];
                    ri += kz[e] * row[2 * iz[e] + 1];
                }
                double v = kx[a] * ky[b];
                sr += v * rr;
                si += v * ri;
            }
        }
        c[2 * j] = sr;
        c[2 * j + 1] = si;
    }
}

int cmto_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
