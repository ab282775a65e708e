// Launchers of the spreading kernel (type 1): precision x strengths x layout x kernel width.
#include "cmt_common.cuh"
#include "nufft_plan.cuh"

namespace cmt {

#include "spread_interp.cuh"

namespace {

template <typename T, bool CPLX, bool PRIV>
using SpreadFn = void (*)(const int *, const int *, const int *, const int *, const int *, const T *, const T *,
                          const T *, const T *, SubgridGeom, T, T *);

template <typename T, bool CPLX, bool PRIV>
SpreadFn<T, CPLX, PRIV> pick(int w)
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

template <typename T, bool CPLX, bool PRIV>
int run(Plan &p, const void *c, int rs, int threads, int sm)
{
    SpreadFn<T, CPLX, PRIV> k = pick<T, CPLX, PRIV>(p.w);
    CMT_TRY(prep_smem(k, sm));
    prof_begin(p);
    k<<<(unsigned)p.nsub, threads, sm, p.stream>>>(p.sub_bin, p.sub_off, p.bin_count, p.bin_start, p.perm,
                                                    (const T *)p.ux, (const T *)p.uy, (const T *)p.uz,
                                                    (const T *)c, geom(p, rs), (T)p.beta, (T *)p.fine);
    CMT_LAUNCH_CHECK();
    prof_end(p, PROF_SPREAD);
    return CMT_OK;
}

}  // namespace

// Real strengths accumulate into per-warp private subgrids (4 warps) when the plan asks for
// it and they fit; otherwise one subgrid with shared atomics (8 warps).
int launch_spread(Plan &p, const void *c, bool cplx, int rs)
{
    size_t one = sub_bytes(p) * (cplx ? 2 : 1);
    bool priv = !cplx && p.spread_priv && one * 4 <= SMEM_BUDGET;
    int threads = priv ? 128 : 256;
    int sm = (int)(priv ? 4 * one : one);
    if (p.prec == 64) {
        if (cplx) return run<double, true, false>(p, c, rs, threads, sm);
        return priv ? run<double, false, true>(p, c, rs, threads, sm) : run<double, false, false>(p, c, rs, threads, sm);
    }
    if (cplx) return run<float, true, false>(p, c, rs, threads, sm);
    return priv ? run<float, false, true>(p, c, rs, threads, sm) : run<float, false, false>(p, c, rs, threads, sm);
}

}  // namespace cmt
