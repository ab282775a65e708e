// Launchers of the spreading kernels (type 1): precision x strengths x layout x kernel width.
#include "cmt_common.cuh"
#include "nufft_plan.cuh"

#include <algorithm>

namespace cmt {

#include "spread_interp.cuh"

namespace {

template <typename T>
using SpreadFn = void (*)(const int *, const int *, const int *, const int *, const int *, const T *, const T *,
                          const T *, const T *, SubgridGeom, T, T *);

// per-point kernel: any width (W = 0 reads it at run time), optional private subgrids
template <typename T, bool CPLX, bool PRIV>
SpreadFn<T> pick(int w)
{
    switch (w) {
    case 2: return k_spread<T, CPLX, 2, PRIV>;
    case 3: return k_spread<T, CPLX, 3, PRIV>;
    case 4: return k_spread<T, CPLX, 4, PRIV>;
    case 5: return k_spread<T, CPLX, 5, PRIV>;
    case 6: return k_spread<T, CPLX, 6, PRIV>;
    case 7: return k_spread<T, CPLX, 7, PRIV>;
    case 8: return k_spread<T, CPLX, 8, PRIV>;
    default: return k_spread<T, CPLX, 0, PRIV>;
    }
}

// table-driven kernel: widths 2..8 (2..7 with the extended window)
template <typename T, bool CPLX, bool EXT>
SpreadFn<T> pick_tab(int w)
{
    switch (w) {
    case 2: return k_spread_tab<T, CPLX, 2, EXT>;
    case 3: return k_spread_tab<T, CPLX, 3, EXT>;
    case 4: return k_spread_tab<T, CPLX, 4, EXT>;
    case 5: return k_spread_tab<T, CPLX, 5, EXT>;
    case 6: return k_spread_tab<T, CPLX, 6, EXT>;
    case 7: return k_spread_tab<T, CPLX, 7, EXT>;
    case 8: if constexpr (!EXT) return k_spread_tab<T, CPLX, 8, false>;
    [[fallthrough]];
    default: return nullptr;
    }
}

template <typename T>
int run(Plan &p, SpreadFn<T> k, const void *c, int rs, int threads, size_t sm)
{
    CMT_CHECK_ARG(k, "no spreading kernel for width %d", p.w);
    CMT_TRY(prep_smem(k, (int)sm));
    prof_begin(p);
    k<<<(unsigned)p.nsub, threads, sm, p.stream>>>(p.sub_bin, p.sub_off, p.bin_count, p.bin_start, p.perm,
                                                    (const T *)p.ux, (const T *)p.uy, (const T *)p.uz,
                                                    (const T *)c, geom(p, rs), (T)p.beta, (T *)p.fine);
    CMT_LAUNCH_CHECK();
    prof_end(p, PROF_SPREAD);
    return CMT_OK;
}

template <typename T>
int dispatch(Plan &p, const void *c, bool cplx, int rs)
{
    const size_t one = sub_bytes(p);
    const bool priv = !cplx && p.spread_priv && one * 4 <= SMEM_BUDGET;
    if (p.spread_tab && !priv && p.w >= 2 && p.w <= 8) {
        if (cplx) return run<T>(p, pick_tab<T, true, false>(p.w), c, rs, 256, spread_tab_smem<T, true>(one, 8));
        const size_t sm = spread_tab_smem<T, false>(one, 8);
        if (p.spread_ext && p.w <= 7) return run<T>(p, pick_tab<T, false, true>(p.w), c, rs, 256, sm);
        return run<T>(p, pick_tab<T, false, false>(p.w), c, rs, 256, sm);
    }
    if (cplx) return run<T>(p, pick<T, true, false>(p.w), c, rs, 256, 2 * one);
    if (priv) return run<T>(p, pick<T, false, true>(p.w), c, rs, 128, 4 * one);
    return run<T>(p, pick<T, false, false>(p.w), c, rs, 256, one);
}

template <typename T, bool CPLX>
using BatchFn = void (*)(const WorkItem *, int, const InstDesc<T> *, T, int *);

template <typename T, bool CPLX, bool EXT>
BatchFn<T, CPLX> pick_batch(int w)
{
    switch (w) {
    case 2: return k_spread_tab_batch<T, CPLX, 2, EXT>;
    case 3: return k_spread_tab_batch<T, CPLX, 3, EXT>;
    case 4: return k_spread_tab_batch<T, CPLX, 4, EXT>;
    case 5: return k_spread_tab_batch<T, CPLX, 5, EXT>;
    case 6: return k_spread_tab_batch<T, CPLX, 6, EXT>;
    case 7: return k_spread_tab_batch<T, CPLX, 7, EXT>;
    case 8: if constexpr (!EXT) return k_spread_tab_batch<T, CPLX, 8, false>;
    [[fallthrough]];
    default: return nullptr;
    }
}

template <typename T, bool CPLX, bool EXT>
int run_batch(int w, const WorkItem *work, int nwork, const void *inst, double beta, int *next, size_t smem,
              cudaStream_t st)
{
    BatchFn<T, CPLX> k = pick_batch<T, CPLX, EXT>(w);
    CMT_CHECK_ARG(k, "batched spreading needs a kernel width in 2..8 (2..7 on derived plans; got %d)", w);
    CMT_TRY(prep_smem(k, (int)smem));
    int per_sm = 0, dev = 0, sms = 0;
    CMT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem));
    CMT_TRY_CUDA(cudaGetDevice(&dev));
    CMT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CMT_CHECK_ARG(per_sm > 0, "batched spreading: %zu bytes of shared memory per CTA do not fit", smem);
    const int grid = std::max(1, std::min(nwork, per_sm * sms));
    k<<<grid, 256, smem, st>>>(work, nwork, (const InstDesc<T> *)inst, (T)beta, next);
    CMT_LAUNCH_CHECK();
    return CMT_OK;
}

}  // namespace

int launch_spread_batch(int prec, bool cplx, bool ext, int w, const WorkItem *work, int nwork, const void *inst,
                        double beta, int *next, size_t smem, cudaStream_t st)
{
    if (prec == 64) {
        if (cplx) return run_batch<double, true, false>(w, work, nwork, inst, beta, next, smem, st);
        return ext ? run_batch<double, false, true>(w, work, nwork, inst, beta, next, smem, st)
                   : run_batch<double, false, false>(w, work, nwork, inst, beta, next, smem, st);
    }
    if (cplx) return run_batch<float, true, false>(w, work, nwork, inst, beta, next, smem, st);
    return ext ? run_batch<float, false, true>(w, work, nwork, inst, beta, next, smem, st)
               : run_batch<float, false, false>(w, work, nwork, inst, beta, next, smem, st);
}

// Shared memory of the batched kernels for plan p (the batch takes the largest).
size_t batch_smem(const Plan &p, bool spread, bool cplx)
{
    const size_t one = sub_bytes(p);
    if (spread)
        return p.prec == 64 ? (cplx ? spread_tab_smem<double, true>(one, 8) : spread_tab_smem<double, false>(one, 8))
                            : (cplx ? spread_tab_smem<float, true>(one, 8) : spread_tab_smem<float, false>(one, 8));
    return p.prec == 64 ? (cplx ? interp_tab_smem<double, true>(one, 8) : interp_tab_smem<double, false>(one, 8))
                        : (cplx ? interp_tab_smem<float, true>(one, 8) : interp_tab_smem<float, false>(one, 8));
}

// Widths 2..8 spread through the per-warp point table (k_spread_tab; on a derived plan's
// doubled grid with the extended register window); wider kernels, or a plan that asks for
// per-warp private subgrids, use the per-point kernel (k_spread).
int launch_spread(Plan &p, const void *c, bool cplx, int rs)
{
    return p.prec == 64 ? dispatch<double>(p, c, cplx, rs) : dispatch<float>(p, c, cplx, rs);
}

}  // namespace cmt
