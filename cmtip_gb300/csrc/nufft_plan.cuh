// Plan object of the NUFFT and the interface between its host code (nufft.cu) and the
// spreading / interpolation kernels (nufft_spread.cu, nufft_interp.cu).
#pragma once

#include "cmt_common.cuh"

namespace cmt {

struct Plan {
    int type = 1, prec = 32, M = 0, isign = 1;
    double eps = 1e-6, sigma = 2.0;
    int n = 0, w = 0, bs = 8, nb = 0, S = 0;  // fine size, width, bin size, bins/dim, subgrid size
    int P = 0, ew = 8;                         // subgrid row pitch, z lanes of the warp layout
    int spread_priv = 0;                       // real spreading into per-warp private subgrids
    int spread_ext = 0;                        // derived plan: (w+1)^3 register window per group
    int spread_tab = 1;                        // widths <= 8: table-driven spreading kernel
    int interp_tab = 1;                        // widths <= 8: table-driven interpolation kernel
    int sort_origin = 1;                       // global sort by bin and window origin (else bin)
    int sort_keys = 3;                         // origin coordinates in the global key (1: x, 2: x y, 3: x y z)
    double cscale = 1.0;                       // coordinate scale of borrowed points
    const Plan *points_of = nullptr;           // set: the point arrays belong to this plan
    double beta = 0.0;
    int maxsub = 8192;                         // points per subproblem (CTA)
    int64_t pts_version = 0;                   // incremented by every set_pts
    int64_t cap_bins = 0;                      // bins the bin arrays were allocated for
    cudaStream_t stream = nullptr;

    int64_t N = 0;
    int64_t nsub = 0;
    int *bin_count = nullptr, *bin_start = nullptr, *bin_fill = nullptr;
    int *sub_bin = nullptr, *sub_off = nullptr;
    int *key_start = nullptr, *key_next = nullptr, *tile_sums = nullptr;  // point-sort keys
    int64_t cap_keys = 0;
    int *perm = nullptr;
    void *ux = nullptr, *uy = nullptr, *uz = nullptr;  // bin-relative sorted coordinates
    void *pts_block = nullptr;                          // owns ux | uy | uz | perm (not when borrowed)
    int64_t cap_pts = 0, cap_sub = 0;
    int *dflag = nullptr;      // device: range error flag, totals
    long long *dtot = nullptr; // device: [total subproblems]

    void *fine = nullptr;   // 2 n^3 elements of prec (complex n^3 or padded real)
    void *fine2 = nullptr;  // second grid for the pair operator
    void *deconv = nullptr; // |k| -> 1/psi_hat(k h), k = 0 .. M/2 + 1
    cufftHandle fft_c2c = 0, fft_r2c = 0, fft_c2r = 0;
    bool has_c2c = false, has_r2c = false, has_c2r = false;

    // optional per-launch timing of the spread / interp / pair kernels (CUDA events on the
    // plan's stream, read back after the timed region)
    static constexpr int PROF_CAP = 256;
    bool prof = false;
    cudaEvent_t ev[2 * PROF_CAP] = {};
    int kind[PROF_CAP] = {};
    int nev = 0;
};

enum { PROF_SPREAD = 1, PROF_INTERP = 2, PROF_PAIR = 3 };

// A launch is timed only outside stream capture (inside, an event record would become a
// node of the captured graph instead of a timestamp of this launch).
static inline bool prof_on(const Plan &p)
{
    if (!p.prof || p.nev >= Plan::PROF_CAP) return false;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(p.stream, &st) == cudaSuccess && st == cudaStreamCaptureStatusNone;
}

static inline void prof_begin(Plan &p)
{
    if (prof_on(p)) cudaEventRecord(p.ev[2 * p.nev], p.stream);
}

static inline void prof_end(Plan &p, int kind)
{
    if (prof_on(p)) {
        cudaEventRecord(p.ev[2 * p.nev + 1], p.stream);
        p.kind[p.nev++] = kind;
    }
}


// Geometry handed to the spreading / interpolation kernels.
struct SubgridGeom {
    int n, rs, bs, nb, w, S, P, maxsub;
    float cscale;  // bin-relative coordinates are stored / cscale (derived plans share points)
};

inline size_t elem(const Plan &p) { return p.prec == 64 ? sizeof(double) : sizeof(float); }

inline SubgridGeom geom(const Plan &p, int rs)
{
    return SubgridGeom{p.n, rs, p.bs, p.nb, p.w, p.S, p.P, p.maxsub, (float)p.cscale};
}

// bytes of one channel of one padded subgrid copy
inline size_t sub_bytes(const Plan &p) { return (size_t)p.S * p.S * p.P * elem(p); }

constexpr size_t SMEM_BUDGET = 100 * 1024;  // two CTAs per SM

template <typename K>
int prep_smem(K kernel, int bytes)
{
    if (bytes > 48 * 1024) CMT_TRY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return CMT_OK;
}

// Kernel launchers (dispatch on precision, kernel width and layout).
//   launch_spread: c = strengths (nullptr: all ones), cplx = complex strengths, rs = row
//                  stride of a real fine grid; accumulates into p.fine (zeroed by the caller).
//   launch_interp: out_mode 0 complex values from the complex grid, 2 real values from the
//                  real grid (row stride rs); writes out in caller order.
//   launch_pair:   interpolate from p.fine, spread into p.fine2; prepare_only sets the
//                  kernel attributes and launches nothing.
int launch_spread(Plan &p, const void *c, bool cplx, int rs);
int launch_interp(Plan &p, int out_mode, int rs, void *out);
int launch_pair(Plan &p, bool prepare_only);

// Batches of plans: one subproblem of one plan, and the plan's arrays and geometry.
// Spreading: in = strengths (nullptr: ones), out = fine grid; interpolation: in = fine
// grid, out = values in caller order.
struct WorkItem {
    int inst, bin, off;
};
template <typename T>
struct InstDesc {
    const int *bin_count, *bin_start, *perm;
    const void *ux, *uy, *uz;  // T
    const void *in;            // T
    void *out;                 // T
    SubgridGeom gm;
};

// One persistent launch over the work list of a batch (all plans of one precision and
// kernel width 2..8); smem = the largest plan's shared-memory need (batch_smem).
// ext: every plan of the batch is derived and spreads through the extended register window.
int launch_spread_batch(int prec, bool cplx, bool ext, int w, const WorkItem *work, int nwork, const void *inst,
                        double beta, int *next, size_t smem, cudaStream_t st);
int launch_interp_batch(int prec, int out_mode, int w, const WorkItem *work, int nwork, const void *inst,
                        double beta, int *next, size_t smem, cudaStream_t st);
size_t batch_smem(const Plan &p, bool spread, bool cplx);

}  // namespace cmt

struct cmt_plan : cmt::Plan {};
