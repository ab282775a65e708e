// Launchers of the interpolation (type 2) and fused pair kernels.
#include "cmt_common.cuh"
#include "nufft_plan.cuh"

#include <algorithm>

namespace cmt {

#include "spread_interp.cuh"

namespace {

template <typename T>
using InterpFn = void (*)(const int *, const int *, const int *, const int *, const int *, const T *, const T *,
                          const T *, const T *, SubgridGeom, T, T *);
template <typename T>
using PairFn = void (*)(const int *, const int *, const int *, const int *, const T *, const T *, const T *,
                        const T *, SubgridGeom, T, T *);

template <typename T, int OUT>
InterpFn<T> pick_interp(int w)
{
    switch (w) {
    case 2: return k_interp<T, OUT, 2>;
    case 3: return k_interp<T, OUT, 3>;
    case 4: return k_interp<T, OUT, 4>;
    case 5: return k_interp<T, OUT, 5>;
    case 6: return k_interp<T, OUT, 6>;
    case 7: return k_interp<T, OUT, 7>;
    case 8: return k_interp<T, OUT, 8>;
    default: return k_interp<T, OUT, 0>;
    }
}

template <typename T>
PairFn<T> pick_pair(int w)
{
    switch (w) {
    case 2: return k_pair<T, 2>;
    case 3: return k_pair<T, 3>;
    case 4: return k_pair<T, 4>;
    case 5: return k_pair<T, 5>;
    case 6: return k_pair<T, 6>;
    case 7: return k_pair<T, 7>;
    case 8: return k_pair<T, 8>;
    default: return k_pair<T, 0>;
    }
}

template <typename T, int OUT>
InterpFn<T> pick_interp_tab(int w)
{
    switch (w) {
    case 2: return k_interp_tab<T, OUT, 2>;
    case 3: return k_interp_tab<T, OUT, 3>;
    case 4: return k_interp_tab<T, OUT, 4>;
    case 5: return k_interp_tab<T, OUT, 5>;
    case 6: return k_interp_tab<T, OUT, 6>;
    case 7: return k_interp_tab<T, OUT, 7>;
    case 8: return k_interp_tab<T, OUT, 8>;
    default: return nullptr;
    }
}

// Widths 2..8 interpolate through the per-warp point table (k_interp_tab); wider kernels
// use the per-point kernel (k_interp).
template <typename T, int OUT>
int run_interp(Plan &p, int rs, void *out)
{
    const bool tab = p.interp_tab && p.w >= 2 && p.w <= 8;
    InterpFn<T> k = tab ? pick_interp_tab<T, OUT>(p.w) : pick_interp<T, OUT>(p.w);
    int sm = (int)(tab ? interp_tab_smem<T, OUT == 0>(sub_bytes(p), 8) : sub_bytes(p) * (OUT == 0 ? 2 : 1));
    CMT_TRY(prep_smem(k, sm));
    prof_begin(p);
    k<<<(unsigned)p.nsub, 256, sm, p.stream>>>(p.sub_bin, p.sub_off, p.bin_count, p.bin_start, p.perm,
                                                (const T *)p.ux, (const T *)p.uy, (const T *)p.uz, (const T *)p.fine,
                                                geom(p, rs), (T)p.beta, (T *)out);
    CMT_LAUNCH_CHECK();
    prof_end(p, PROF_INTERP);
    return CMT_OK;
}

template <typename T>
PairFn<T> pick_pair_tab(int w)
{
    switch (w) {
    case 2: return k_pair_tab<T, 2>;
    case 3: return k_pair_tab<T, 3>;
    case 4: return k_pair_tab<T, 4>;
    case 5: return k_pair_tab<T, 5>;
    case 6: return k_pair_tab<T, 6>;
    case 7: return k_pair_tab<T, 7>;
    case 8: return k_pair_tab<T, 8>;
    default: return nullptr;
    }
}

// Widths 2..8 run the table-driven pair (k_pair_tab) when its two subgrids and tables fit
// in shared memory; wider kernels (or larger subgrids) the per-point pair (k_pair).
template <typename T>
int run_pair(Plan &p, bool prepare_only)
{
    int dev = 0, max_sm = 0;
    CMT_TRY_CUDA(cudaGetDevice(&dev));
    CMT_TRY_CUDA(cudaDeviceGetAttribute(&max_sm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t tab_sm = pair_tab_smem<T>(sub_bytes(p), 8);
    const bool tab = p.spread_tab && p.interp_tab && p.w >= 2 && p.w <= 8 && tab_sm <= (size_t)max_sm;
    PairFn<T> k = tab ? pick_pair_tab<T>(p.w) : pick_pair<T>(p.w);
    int sm = (int)(tab ? tab_sm : 4 * sub_bytes(p));
    CMT_TRY(prep_smem(k, sm));
    if (prepare_only) return CMT_OK;
    prof_begin(p);
    k<<<(unsigned)p.nsub, 256, sm, p.stream>>>(p.sub_bin, p.sub_off, p.bin_count, p.bin_start, (const T *)p.ux,
                                                (const T *)p.uy, (const T *)p.uz, (const T *)p.fine, geom(p, p.n),
                                                (T)p.beta, (T *)p.fine2);
    CMT_LAUNCH_CHECK();
    prof_end(p, PROF_PAIR);
    return CMT_OK;
}

template <typename T, int OUT>
using BatchFn = void (*)(const WorkItem *, int, const InstDesc<T> *, T, int *);

template <typename T, int OUT>
BatchFn<T, OUT> pick_batch(int w)
{
    switch (w) {
    case 2: return k_interp_tab_batch<T, OUT, 2>;
    case 3: return k_interp_tab_batch<T, OUT, 3>;
    case 4: return k_interp_tab_batch<T, OUT, 4>;
    case 5: return k_interp_tab_batch<T, OUT, 5>;
    case 6: return k_interp_tab_batch<T, OUT, 6>;
    case 7: return k_interp_tab_batch<T, OUT, 7>;
    case 8: return k_interp_tab_batch<T, OUT, 8>;
    default: return nullptr;
    }
}

template <typename T, int OUT>
int run_batch(int w, const WorkItem *work, int nwork, const void *inst, double beta, int *next, size_t smem,
              cudaStream_t st)
{
    BatchFn<T, OUT> k = pick_batch<T, OUT>(w);
    CMT_CHECK_ARG(k, "batched interpolation needs a kernel width in 2..8 (got %d)", w);
    CMT_TRY(prep_smem(k, (int)smem));
    int per_sm = 0, dev = 0, sms = 0;
    CMT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem));
    CMT_TRY_CUDA(cudaGetDevice(&dev));
    CMT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CMT_CHECK_ARG(per_sm > 0, "batched interpolation: %zu bytes of shared memory per CTA do not fit", smem);
    const int grid = std::max(1, std::min(nwork, per_sm * sms));
    k<<<grid, 256, smem, st>>>(work, nwork, (const InstDesc<T> *)inst, (T)beta, next);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

}  // namespace

int launch_interp_batch(int prec, int out_mode, int w, const WorkItem *work, int nwork, const void *inst,
                        double beta, int *next, size_t smem, cudaStream_t st)
{
    if (prec == 64)
        return out_mode == 0 ? run_batch<double, 0>(w, work, nwork, inst, beta, next, smem, st)
                             : run_batch<double, 2>(w, work, nwork, inst, beta, next, smem, st);
    return out_mode == 0 ? run_batch<float, 0>(w, work, nwork, inst, beta, next, smem, st)
                         : run_batch<float, 2>(w, work, nwork, inst, beta, next, smem, st);
}

int launch_interp(Plan &p, int out_mode, int rs, void *out)
{
    if (p.prec == 64) return out_mode == 0 ? run_interp<double, 0>(p, rs, out) : run_interp<double, 2>(p, rs, out);
    return out_mode == 0 ? run_interp<float, 0>(p, rs, out) : run_interp<float, 2>(p, rs, out);
}

int launch_pair(Plan &p, bool prepare_only)
{
    return p.prec == 64 ? run_pair<double>(p, prepare_only) : run_pair<float>(p, prepare_only);
}

}  // namespace cmt
