// Data preparation on the device (cmtip/prep_data.py): detector binning by block means and
// resolution clipping, fused into one pass over the image stack.
//
// bin_data (prep_data.py:181-212) averages bin x bin blocks of each panel as
// arr.reshape(..., nx/b, b, ny/b, b).mean(-1).mean(3): for each block row i the mean of its b
// values (numpy's order for a contiguous axis, row_sum, then divided by b), then the mean of
// those b row means (summed in order, divided by b), in the array's precision.  The kernel
// evaluates exactly that order, so its results equal numpy's bit for bit.  clip_data (prep_data.py:149-163) keeps the
// pixels whose resolution exceeds the limit: the host computes the kept indices from the
// (binned) q-vectors and the kernel gathers them, so each output is written once and each
// input read once.
#include "cmt_common.cuh"

#include <algorithm>

namespace cmt {

// Sum of n contiguous values in numpy's order for a contiguous axis (pairwise summation):
// sequential below 8 values; from 8 to 128, eight interleaved partial sums combined as
// ((r0 + r1) + (r2 + r3)) + ((r4 + r5) + (r6 + r7)), then the remainder in order.
template <typename T>
__device__ __forceinline__ T row_sum(const T *a, int n)
{
    if (n < 8) {
        T s = T(0);
        for (int j = 0; j < n; ++j) s += a[j];
        return s;
    }
    T r[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = a[k];
    int i = 8;
    for (; i + 8 <= n; i += 8)
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] += a[i + k];
    T s = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; ++i) s += a[i];
    return s;
}

// kept indices outside the binned pixel range seen by the last call (the host reads it back)
static __device__ int g_bad_index;

// Grid: x over the kept pixels, y over image slabs.  A thread decomposes its pixel's index
// once and then walks the images, so the index arithmetic is amortised and every image's
// reads and writes are contiguous across the warp.
template <typename T>
__global__ void k_bin_clip(const T *in, int64_t n_img, int n_panels, int px, int py, int b, const int64_t *keep,
                           int64_t n_keep, T *out)
{
    const int bx_n = px / b, by_n = py / b;
    const int64_t n_binned = (int64_t)n_panels * bx_n * by_n;
    const int64_t per_img_in = (int64_t)n_panels * px * py;
    const T inv = T(b);
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n_keep; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = keep ? keep[q] : q;  // index into the binned (panel, bx, by) pixels
        if (k < 0 || k >= n_binned) {          // never read outside the stack
            g_bad_index = 1;
            for (int64_t img = blockIdx.y; img < n_img; img += gridDim.y) out[img * n_keep + q] = T(0);
            continue;
        }
        const int panel = (int)(k / ((int64_t)bx_n * by_n));
        const int rem = (int)(k - (int64_t)panel * bx_n * by_n);
        const int bx = rem / by_n, by = rem - bx * by_n;
        const int64_t off = ((int64_t)panel * px + (int64_t)bx * b) * py + (int64_t)by * b;
        for (int64_t img = blockIdx.y; img < n_img; img += gridDim.y) {
            const T *src = in + img * per_img_in + off;
            T acc = T(0);
            for (int i = 0; i < b; ++i) acc += row_sum(src + (int64_t)i * py, b) / inv;
            out[img * n_keep + q] = acc / inv;
        }
    }
}

}  // namespace cmt

using namespace cmt;

extern "C" int cmt_bin_clip(int prec, const void *in, int64_t n_img, int n_panels, int px, int py, int bin,
                            const int64_t *keep, int64_t n_keep, void *out, void *stream)
{
    CMT_CHECK_ARG(in && out, "null argument");
    CMT_CHECK_ARG(prec == 32 || prec == 64, "prec must be 32 or 64");
    CMT_CHECK_ARG(n_img > 0 && n_panels > 0 && px > 0 && py > 0, "empty image stack");
    CMT_CHECK_ARG(bin >= 1 && bin <= 128 && px % bin == 0 && py % bin == 0,
                  "panel shape %d x %d not divisible by bin %d (1..128)", px, py, bin);
    const int64_t n_binned = (int64_t)n_panels * (px / bin) * (py / bin);
    if (!keep) n_keep = n_binned;
    CMT_CHECK_ARG(n_keep >= 0 && n_keep <= n_binned, "n_keep %lld outside [0, %lld]", (long long)n_keep,
                  (long long)n_binned);
    if (n_keep == 0) return CMT_OK;
    int dev = 0, sms = 0;
    CMT_TRY_CUDA(cudaGetDevice(&dev));
    CMT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int gx = (int)std::min<int64_t>((n_keep + 255) / 256, (int64_t)sms * 8);
    const int gy = (int)std::max<int64_t>(1, std::min<int64_t>(n_img, ((int64_t)sms * 8 + gx - 1) / gx));
    const dim3 grid(gx, gy);
    cudaStream_t st = (cudaStream_t)stream;
    int *bad = nullptr;
    CMT_TRY_CUDA(cudaGetSymbolAddress((void **)&bad, g_bad_index));
    CMT_TRY_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
    if (prec == 64)
        k_bin_clip<double><<<grid, 256, 0, st>>>((const double *)in, n_img, n_panels, px, py, bin, keep, n_keep,
                                                 (double *)out);
    else
        k_bin_clip<float><<<grid, 256, 0, st>>>((const float *)in, n_img, n_panels, px, py, bin, keep, n_keep,
                                                (float *)out);
    CMT_LAUNCH_CHECK();
    if (keep) {
        int hbad = 0;
        CMT_TRY_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        CMT_TRY_CUDA(cudaStreamSynchronize(st));
        CMT_CHECK_ARG(!hbad, "kept pixel index outside [0, %lld)", (long long)n_binned);
    }
    return CMT_OK;
}
