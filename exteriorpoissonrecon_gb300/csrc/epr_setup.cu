// Build phase on the device: ordered sampling, the density estimator, the frame splat, S(E), and
// the screening (R), constraint (B) and Dirichlet (K) stencils with their Galerkin hierarchy.
//
// Reference correspondence (paths relative to the reference checkout):
//   sort by cell             OrderedSampler                      Include/OrderedSamples.inl:32-85
//   density splat            TreeEstimator ctor / addSamples     Include/GridSamples.inl:361-391,436-491,740-771
//   estimator queries        TreeEstimator::operator()/depth     Include/GridSamples.inl:774-896
//   frame splat              Reconstructor ctor                  ExteriorPoissonRecon/ExteriorPoisson.h:181-264
//   S(E)                     TreeSplatter::operator()(p)         Include/GridSamples.inl:600-651
//   R                        ScalarFunctions::deltaMass          Include/Hat.scalars.inl:977-1063
//   B, c                     ScalarFunctions::stiffness, ctor    Include/Hat.scalars.inl:1585-1690, SystemEnergy.h:447-462
//   K                        StiffnessStencil / FullIntegrationStencil  Include/Hat.scalars.inl:261-293,528-545
//   Galerkin                 SingleCycleCascadicSystemEnergy::restrict  Include/SystemEnergy.h:464-477
//
// The reference's trees (RegularTreeNode) are stored here as dense per-depth vertex grids: a node
// that the reference never creates never receives data, so its dense value is zero.  The only
// structural information the reference uses is which cells have children (the depth of the leaf
// containing a point); it is kept as one byte per cell and depth.
//
// Splats are deterministic gathers: samples are sorted by the Morton key of their cell, so the
// samples of any coarser cell are one contiguous range; every output vertex is reduced by one
// warp in a fixed order.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include <cub/cub.cuh>

#include "epr_common.cuh"
#include "epr_context.h"

namespace epr {

namespace {

constexpr int kMaxDeg = 9;  // 2 * 4 + 1

// ---------------------------------------------------------------------------------------------
// small device helpers
// ---------------------------------------------------------------------------------------------
__device__ inline void bspline_eval(int deg, double x, double *v)
{
    // iterative form of the recursive evaluation of GridSamples.inl:50-65
    v[deg] = 1.;
    for (int k = 1; k <= deg; k++)
    {
        const double scale = 1. / k;
        int b = deg - k;
        v[b] = v[b + 1] * (1. - x) * scale;
        for (int i = 1; i < k; i++)
        {
            double x1 = (x - i + k), x2 = (-x + i + 1);
            v[b + i] = (v[b + i] * x1 + v[b + i + 1] * x2) * scale;
        }
        v[b + k] *= x * scale;
    }
}

template <int D>
__host__ __device__ inline int64_t morton(const int *E, int bits)
{
    int64_t k = 0;
    for (int b = bits - 1; b >= 0; b--)
        for (int d = 0; d < D; d++) k = (k << 1) | ((E[d] >> b) & 1);
    return k;
}

template <int D>
__host__ __device__ inline void demorton(int64_t k, int bits, int *E)
{
    for (int d = 0; d < D; d++) E[d] = 0;
    for (int b = 0; b < bits; b++)
        for (int d = D - 1; d >= 0; d--) { E[d] |= (int)(k & 1) << b; k >>= 1; }
}

// first index in sorted keys[0..n) with key >= v
__device__ inline int64_t lower_bound(const int64_t *keys, int64_t n, int64_t v)
{
    int64_t lo = 0, hi = n;
    while (lo < hi)
    {
        int64_t mid = (lo + hi) >> 1;
        if (keys[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// cell of p at resolution res as the reference's tree descent finds it (strict ">" at splits,
// Misha/RegularTree.inl:538-543): points on a face belong to the lower cell
__device__ inline int tree_cell(double p, int res)
{
    double s = p * res;
    int o = (int)floor(s);
    if ((double)o == s && o > 0) o--;
    return o;
}

__device__ inline double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

inline unsigned int nblocks(int64_t n, int t) { return (unsigned int)((n + t - 1) / t); }

// ---------------------------------------------------------------------------------------------
// ordered sampling
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void cell_keys_kernel(const double *pos, int64_t n, int depth, int64_t *keys, int *vals)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int r = 1 << depth;
    int E[D];
    for (int d = 0; d < D; d++)
    {
        int e = (int)floor(pos[i * D + d] * r);
        E[d] = e < 0 ? 0 : (e > r - 1 ? r - 1 : e);
    }
    keys[i] = morton<D>(E, depth);
    vals[i] = (int)i;
}

__global__ void cell_flags_kernel(const int64_t *keys, int64_t n, int *flags)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void cell_start_kernel(const int64_t *keys, const int *flags, const int *ids, int64_t n, int *cellStart,
                                  int64_t *cellKey)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flags[i]) { cellStart[ids[i]] = (int)i; cellKey[ids[i]] = keys[i]; }
    // ids is the exclusive scan of the flags: the last sample's cell is ids + flags - 1
    if (i == n - 1) cellStart[ids[i] + flags[i]] = (int)n;
}

template <int D>
__global__ void finest_map_kernel(const int64_t *cellKey, int64_t ncells, int depth, int *map)
{
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ncells) return;
    int E[D];
    demorton<D>(cellKey[k], depth, E);
    int r = 1 << depth;
    int64_t e = 0;
    for (int d = 0; d < D; d++) e = e * r + E[d];
    map[e] = (int)k;
}

// merged sample of each occupied cell: mean position and (count, sum p, sum p p^T)
// (GridSamples.inl:381-388 with DensityAndNoiseInfo(p, 1), :74)
template <int D>
__global__ void merge_cells_kernel(const double *pos, const int *order, const int *cellStart, int64_t ncells,
                                   double *mean, double *datum)
{
    constexpr int W = 1 + D + D * D;
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ncells) return;
    double p[D], dat[W];
    for (int d = 0; d < D; d++) p[d] = 0;
    for (int w = 0; w < W; w++) dat[w] = 0;
    for (int j = cellStart[k]; j < cellStart[k + 1]; j++)
    {
        const double *q = pos + (int64_t)order[j] * D;
        for (int d = 0; d < D; d++) p[d] += q[d];
        dat[0] += 1.;
        for (int d = 0; d < D; d++) dat[1 + d] += q[d];
        for (int a = 0; a < D; a++)
            for (int b = 0; b < D; b++) dat[1 + D + a * D + b] += q[a] * q[b];
    }
    double cnt = (double)(cellStart[k + 1] - cellStart[k]);
    for (int d = 0; d < D; d++) mean[k * D + d] = p[d] / cnt;
    for (int w = 0; w < W; w++) datum[k * W + w] = dat[w];
}

// ---------------------------------------------------------------------------------------------
// tree structure: refined[t][cell] = 1 when the depth-t cell has children (RegularTree.inl:728-845)
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void refine_kernel(const int64_t *cellKey, int64_t ncells, int depth, int t, int KR, const uint8_t *prevRefined,
                              uint8_t *refined)
{
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ncells) return;
    int E[D];
    demorton<D>(cellKey[k], depth, E);
    int lo[D], hi[D], I[D];
    int side = 1 << t, pside = 1 << (t - 1);
    for (int d = 0; d < D; d++)
    {
        int ct = E[d] >> (depth - t);  // ancestor at tree depth t+1
        lo[d] = (ct - KR) >> 1;
        hi[d] = (ct + KR + 1) >> 1;
        I[d] = lo[d];
    }
    while (true)
    {
        bool ok = true;
        int64_t li = 0, pi = 0;
        for (int d = 0; d < D; d++)
        {
            if (I[d] < 0 || I[d] >= side) ok = false;
            li = li * side + I[d];
            pi = pi * pside + (I[d] >> 1);
        }
        if (ok && (t == 1 || prevRefined[pi])) refined[li] = 1;
        int d = D - 1;
        for (; d >= 0; d--) { if (++I[d] <= hi[d]) break; I[d] = lo[d]; }
        if (d < 0) break;
    }
}

// ---------------------------------------------------------------------------------------------
// splat gathers: one warp per vertex of tree depth t (resolution 2^(t-1))
// ---------------------------------------------------------------------------------------------
struct SplatArgs
{
    const int64_t *cellKey;
    const int *cellStart;
    int64_t ncells;
    int depth;  // finest depth
    int t;      // tree depth of the grid
    int KR;     // kernel radius (B-spline degree 2 KR + 1)
    const int *rlo = nullptr, *rhi = nullptr;  // occupied-cell range of every depth-t cell, by Morton code
};

// range of occupied cells inside the depth-t cell C
template <int D>
__device__ inline void cell_range(const SplatArgs &a, const int *C, int64_t &lo, int64_t &hi)
{
    if (a.rlo)
    {
        const int res = 1 << (a.t - 1);
        int64_t li = 0;
        for (int d = 0; d < D; d++) li = li * res + C[d];
        lo = a.rlo[li];
        hi = a.rhi[li];
        return;
    }
    int64_t m = morton<D>(C, a.t - 1);
    int s = a.depth + 1 - a.t;  // levels between depth-t cells and finest cells
    lo = lower_bound(a.cellKey, a.ncells, m << (D * s));
    hi = lower_bound(a.cellKey, a.ncells, (m + 1) << (D * s));
}

// Occupied-cell range of every depth-t cell: the occupied finest cells are sorted by Morton key, so
// the ones below a depth-t cell are contiguous; mark where each ancestor's run starts and ends.
// (stored by the row-major index of the depth-t cell)
template <int D>
__global__ void level_ranges_kernel(const int64_t *cellKey, int64_t ncells, int t, int shift, int *rlo, int *rhi)
{
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ncells) return;
    int64_t anc = cellKey[k] >> shift;
    int C[D];
    demorton<D>(anc, t - 1, C);
    const int res = 1 << (t - 1);
    int64_t li = 0;
    for (int d = 0; d < D; d++) li = li * res + C[d];
    if (k == 0 || (cellKey[k - 1] >> shift) != anc) rlo[li] = (int)k;
    if (k == ncells - 1 || (cellKey[k + 1] >> shift) != anc) rhi[li] = (int)(k + 1);
}

// ---------------------------------------------------------------------------------------------
// Chunked gathers for the coarse tree levels.  There a vertex's window covers a large part of the
// domain, so one warp per vertex would walk hundreds of thousands of items.  Instead each vertex's
// item list (the concatenation, in window order, of the items of its window cells) is cut into
// chunks of kChunk items, one warp reduces each chunk into a partial sum, and a final pass adds a
// vertex's partials in chunk order: the result is still deterministic.
// ---------------------------------------------------------------------------------------------
constexpr int kChunk = 2048;

// Item range of one window cell: occupied-cell indices (merged density data) or sample positions
// in the sorted order (frame samples).
template <int D, bool Samples>
__device__ inline void item_range(const SplatArgs &a, const int *C, int &lo, int &hi)
{
    int64_t l, h;
    cell_range<D>(a, C, l, h);
    if (Samples) { lo = a.cellStart[l]; hi = a.cellStart[h]; }
    else { lo = (int)l; hi = (int)h; }
}

template <int D>
__device__ inline void vertex_of(int64_t vi, int nv, int *v)
{
    for (int d = D - 1; d >= 0; d--) { v[d] = (int)(vi % nv); vi /= nv; }
}

template <int D>
__device__ inline bool window_next(int *C, const int *clo, const int *chi)
{
    int d = D - 1;
    for (; d >= 0; d--) { if (++C[d] <= chi[d]) return true; C[d] = clo[d]; }
    return false;
}

template <int D, bool Samples>
__global__ void vertex_chunks_kernel(SplatArgs a, int *nchunks)
{
    int res = 1 << (a.t - 1), nv = res + 1;
    int64_t NV = 1;
    for (int d = 0; d < D; d++) NV *= nv;
    int64_t vi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (vi >= NV) return;
    int v[D], clo[D], chi[D], C[D];
    vertex_of<D>(vi, nv, v);
    for (int d = 0; d < D; d++) { clo[d] = max(0, v[d] - a.KR - 1); chi[d] = min(res - 1, v[d] + a.KR); C[d] = clo[d]; }
    int64_t count = 0;
    do
    {
        int lo, hi;
        item_range<D, Samples>(a, C, lo, hi);
        count += hi - lo;
    } while (window_next<D>(C, clo, chi));
    nchunks[vi] = (int)((count + kChunk - 1) / kChunk);
}

// Contribution of item `it` to vertex v through window cell C, added to acc.
// Density: a merged cell (mean position, summed (1, p, p p^T)) splatted with the degree 2 KR + 1
// B-spline weights of its mean and the estimator's depth weight (TreeSplatter::_addSample,
// GridSamples.inl:458-491; TreeEstimator ctor :749-760).  The window is centred on the depth-t
// ancestor of the item's cell while the weights come from floor(p res), as in the reference.
// The per-axis B-spline values of every item at the level are tabulated once (item_bspline_kernel)
// instead of once per (vertex, item) pair; the products keep the reference's order.
template <int D>
struct DensityItem
{
    static constexpr int W = 1 + D + D * D;
    const double *bs;  // per item: D x (deg + 1) B-spline values at this level
    const double *datum;
    double depthWeight;
    __device__ void operator()(const SplatArgs &a, int it, const int *v, const int *C, double *acc) const
    {
        const int nb = 2 * a.KR + 2;
        double wt = depthWeight;
        const double *b = bs + (int64_t)it * D * nb;
        for (int d = 0; d < D; d++) wt *= b[d * nb + v[d] - (C[d] - a.KR)];
        for (int w = 0; w < W; w++) acc[w] += wt * datum[(int64_t)it * W + w];
    }
};

// Frame sample: normalised frame times the sample's measure and 2^(2 depth), split between the two
// tree depths bracketing its estimated depth with weights 2^((d-1) D) (ExteriorPoisson.h:181-228,
// GridSamples.inl:436-456), B-spline weights of the sample position.  Per sorted sample: the
// level weight and B-spline values (skew_level_kernel) and the scaled frame (skew_frame_kernel).
template <int D>
struct SkewItem
{
    static constexpr int W = D * (D - 1) / 2;
    const double *bs;     // per sorted sample: D x (deg + 1) B-spline values at this level
    const double *lw;     // per sorted sample: level weight at this level
    const double *frame;  // per sorted sample: W scaled frame values
    __device__ void operator()(const SplatArgs &a, int j, const int *v, const int *C, double *acc) const
    {
        const double l = lw[j];
        if (l == 0) return;
        const int nb = 2 * a.KR + 2;
        double wt = l;
        const double *b = bs + (int64_t)j * D * nb;
        for (int d = 0; d < D; d++) wt *= b[d * nb + v[d] - (C[d] - a.KR)];
        for (int k = 0; k < W; k++) acc[k] += wt * frame[(int64_t)j * W + k];
    }
};

// per-axis B-spline values of n points (pts[idx[j]] or pts[j]) at the resolution of tree depth t
template <int D>
__global__ void item_bspline_kernel(const double *pts, const int *idx, int64_t n, int t, int deg, const double *lw, double *bs)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    if (lw && lw[j] == 0) return;
    const int64_t s = idx ? idx[j] : j;
    const int res = 1 << (t - 1);
    for (int d = 0; d < D; d++)
    {
        double pr = pts[s * D + d] * res;
        int e = (int)floor(pr);
        bspline_eval(deg, pr - e, bs + (j * D + d) * (deg + 1));
    }
}

// level weight of every sorted frame sample at tree depth t
__global__ void skew_level_kernel(const double *sdepth, const int *order, int64_t n, int t, int depth, int D, double *lw)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int maxT = depth + 1;
    double dd = sdepth[order[j]] + 1.;
    double w = 0;
    if (dd >= maxT) w = (t == maxT) ? (double)(1ull << (depth * D)) : 0.;
    else if (dd <= 1) w = (t == 1) ? 1. : 0.;
    else
    {
        int d1 = (int)floor(dd), d2 = d1 + 1;
        double f = dd - d1;
        if (t == d1) w = (1. - f) * (double)(1ull << ((d1 - 1) * D));
        else if (t == d2) w = f * (double)(1ull << ((d2 - 1) * D));
    }
    lw[j] = w;
}

// normalised frame times measure and 2^(2 depth), per sorted sample
template <int D>
__global__ void skew_frame_kernel(const double *skew, const double *measure, const int *order, int64_t n, int depth, double *frame)
{
    constexpr int W = D * (D - 1) / 2;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int s = order[j];
    const double *sk = skew + (int64_t)s * W;
    double nrm = 0;
    for (int k = 0; k < W; k++) nrm += 2 * sk[k] * sk[k];
    nrm = sqrt(nrm);
    double m = measure[s], sc = (double)(1ull << (depth * 2));
    for (int k = 0; k < W; k++) frame[j * W + k] = sk[k] / nrm * m * sc;
}

// One warp per chunk.  The vertex's window cells are taken 32 at a time: each lane looks up one
// cell's item range, a warp scan places the cells' items end to end, and the warp then walks the
// part of those items that falls into the chunk 32 items at a time, every lane finding the cell of
// its item by a binary search over the scanned offsets (shuffles).  Lanes stay busy however the
// items spread over the cells, and every lane's order of accumulation is fixed by the item index.
template <int D, bool Samples, class Item>
__global__ void chunk_gather_kernel(SplatArgs a, Item item, const int *chunkStart, int64_t NV, int64_t nchunks, double *partial)
{
    constexpr int W = Item::W;
    const unsigned full = 0xffffffffu;
    int64_t chunk = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (chunk >= nchunks) return;  // whole warps
    // vertex owning the chunk: last vi with chunkStart[vi] <= chunk
    int64_t lo = 0, hi = NV;
    while (hi - lo > 1)
    {
        int64_t mid = (lo + hi) >> 1;
        if (chunkStart[mid] <= chunk) lo = mid; else hi = mid;
    }
    const int64_t vi = lo;
    const int64_t first = (chunk - chunkStart[vi]) * kChunk, last = first + kChunk;
    int res = 1 << (a.t - 1), nv = res + 1;
    int v[D], clo[D], wd[D];
    vertex_of<D>(vi, nv, v);
    int ncell = 1;
    for (int d = 0; d < D; d++)
    {
        clo[d] = max(0, v[d] - a.KR - 1);
        wd[d] = min(res - 1, v[d] + a.KR) - clo[d] + 1;
        ncell *= wd[d];
    }
    double acc[W];
    for (int w = 0; w < W; w++) acc[w] = 0;
    int64_t base = 0;  // items of the window cells before the current batch
    for (int kb = 0; kb < ncell && base < last; kb += 32)
    {
        // this lane's cell (window order: last axis fastest) and its items
        const int k = kb + lane;
        int C[D], ilo = 0, cnt = 0;
        {
            int t = k < ncell ? k : 0;
            for (int d = D - 1; d >= 0; d--) { C[d] = clo[d] + t % wd[d]; t /= wd[d]; }
        }
        if (k < ncell)
        {
            int ihi;
            item_range<D, Samples>(a, C, ilo, ihi);
            cnt = ihi - ilo;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            int n = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += n;
        }
        const int excl = incl - cnt;
        const int total = __shfl_sync(full, incl, 31);
        const int64_t b0 = max(base, first), b1 = min(base + (int64_t)total, last);
        for (int64_t t0 = b0; t0 < b1; t0 += 32)
        {
            const int64_t t = t0 + lane;
            const int r = (int)(t - base);  // position among this batch's items
            int own = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
            {
                const int cand = own + step;
                const int e = __shfl_sync(full, excl, cand & 31);
                if (cand < 32 && e <= r) own = cand;
            }
            const int olo = __shfl_sync(full, ilo, own), oex = __shfl_sync(full, excl, own);
            int Co[D];
#pragma unroll
            for (int d = 0; d < D; d++) Co[d] = __shfl_sync(full, C[d], own);
            if (t < b1) item(a, olo + (r - oex), v, Co, acc);
        }
        base += total;
    }
    for (int w = 0; w < W; w++)
    {
        double sum = warp_sum(acc[w]);
        if (lane == 0) partial[chunk * W + w] = sum;
    }
}

template <int W>
__global__ void chunk_finish_kernel(const int *chunkStart, int64_t NV, const double *partial, double scale, double *grid)
{
    int64_t vi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (vi >= NV) return;
    double acc[W];
    for (int w = 0; w < W; w++) acc[w] = 0;
    for (int c = chunkStart[vi]; c < chunkStart[vi + 1]; c++)
        for (int w = 0; w < W; w++) acc[w] += partial[(int64_t)c * W + w];
    for (int w = 0; w < W; w++) grid[vi * W + w] = acc[w] * scale;
}

// ---------------------------------------------------------------------------------------------
// estimator queries (GridSamples.inl:774-896)
// ---------------------------------------------------------------------------------------------
template <int D>
struct DensityGrids
{
    const double *g[12];
    int depth;
};

// Interpolated splat data at p from tree depth t; only the first NW of the W components (the
// sample count alone for the depth search), each summed exactly as in the full interpolation.
template <int D, int NW = 1 + D + D * D>
__device__ void density_interp(const DensityGrids<D> &G, int t, const double *p, double *out)
{
    constexpr int W = 1 + D + D * D;
    for (int w = 0; w < NW; w++) out[w] = 0;
    if (t < 1) return;  // the root carries no data
    int res = 1 << (t - 1), nv = res + 1;
    int e[D];
    double lv[D][2];
    for (int d = 0; d < D; d++)
    {
        double s = p[d] * res;
        int f = (int)floor(s);
        double x = s - f;
        lv[d][0] = 1. - x;
        lv[d][1] = x;
        e[d] = tree_cell(p[d], res);
    }
    const double *g = G.g[t - 1];
    for (int c = 0; c < (1 << D); c++)
    {
        double s = 1.;
        int64_t vi = 0;
        bool in = true;
        for (int d = 0; d < D; d++)
        {
            int b = (c >> (D - 1 - d)) & 1;
            int o = e[d] + b;
            if (o < 0 || o > res) in = false;
            s *= lv[d][b];
            vi = vi * nv + o;
        }
        if (!in) continue;
        for (int w = 0; w < NW; w++) out[w] += g[vi * W + w] * s;
    }
}

template <int D>
__device__ double samples_per_cell(const DensityGrids<D> &G, int t, const double *p)
{
    double count;
    density_interp<D, 1>(G, t, p, &count);
    return count / (double)(1u << ((t - 1) * (D - 2)));
}

template <int D>
__device__ double est_depth_raw(const DensityGrids<D> &G, int maxT, const double *p)
{
    const double tg = (double)(1 << (D - 2));
    int d1 = maxT, d2 = maxT + 1;
    // s1: samples per cell at depth d1 (computed by the search), s2 at d2 = d1 + 1 (the previous s1)
    double s1 = samples_per_cell<D>(G, d1, p), s2 = 0;
    bool have2 = false;
    while (d2 > 1 && s1 < tg)
    {
        d1--, d2--;
        s2 = s1;
        have2 = true;
        s1 = d1 >= 1 ? samples_per_cell<D>(G, d1, p) : 0;
    }
    if (d2 == 1 || d2 == maxT + 1)
    {
        int d = (d2 == 1) ? 1 : maxT;
        double spc = (d2 == 1) ? s2 : s1;
        return d + log(spc / tg) / log(2.);
    }
    if (!have2) s2 = samples_per_cell<D>(G, d2, p);
    if (!s2) return d1;
    return d1 + log(tg / s1) / log(s2 / s1);
}

// ascending eigenvalues of a symmetric D x D matrix (cyclic Jacobi)
template <int D>
__device__ void sym_eigenvalues(double a[D][D], double *ev)
{
    for (int sweep = 0; sweep < 64; sweep++)
    {
        double off = 0;
        for (int i = 0; i < D; i++)
            for (int j = i + 1; j < D; j++) off += a[i][j] * a[i][j];
        if (off == 0) break;
        for (int p = 0; p < D; p++)
            for (int q = p + 1; q < D; q++)
            {
                if (a[p][q] == 0) continue;
                double theta = (a[q][q] - a[p][p]) / (2 * a[p][q]);
                double t = (theta >= 0 ? 1. : -1.) / (fabs(theta) + sqrt(theta * theta + 1));
                double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < D; k++)
                {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < D; k++)
                {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
            }
    }
    for (int i = 0; i < D; i++) ev[i] = a[i][i];
    for (int i = 1; i < D; i++)
        for (int j = i; j > 0 && ev[j - 1] > ev[j]; j--) { double t = ev[j]; ev[j] = ev[j - 1]; ev[j - 1] = t; }
}

template <int D>
__global__ void estimator_kernel(DensityGrids<D> G, const double *pos, int64_t n, double *measure, double *noise, double *sdepth)
{
    constexpr int W = 1 + D + D * D;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double p[D];
    for (int d = 0; d < D; d++) p[d] = pos[i * D + d];
    int maxT = G.depth + 1;
    double dd = est_depth_raw<D>(G, maxT, p);
    double info[W];
    if (dd >= maxT) density_interp<D>(G, maxT, p, info);
    else if (dd < 0) density_interp<D>(G, 1, p, info);
    else
    {
        int d1 = (int)floor(dd), d2 = d1 + 1;
        double f = dd - d1, b[W];
        density_interp<D>(G, d1, p, info);
        density_interp<D>(G, d2, p, b);
        for (int w = 0; w < W; w++) info[w] = info[w] * (1. - f) + b[w] * f;
    }
    double wsum = info[0];
    measure[i] = 1. / wsum;
    double C[D][D];
    for (int a = 0; a < D; a++)
        for (int b = 0; b < D; b++) C[a][b] = info[1 + D + a * D + b] / wsum - info[1 + a] / wsum * info[1 + b] / wsum;
    double ev[D];
    sym_eigenvalues<D>(C, ev);
    double sum = 0, low = 0;
    for (int d = 0; d < D; d++) { sum += ev[d]; if (d < 2) low += ev[d]; }
    noise[i] = (low * D) / (sum * 2);
    sdepth[i] = dd - 1.;  // depth(p) of the estimator: leaf of a sample is at the finest depth
}

// S(E) at element centres, summed over tree depths down to the leaf containing the centre
template <int D>
struct SkewGrids
{
    const double *g[12];
    const uint8_t *refined[12];
    int depth;
};

// FitBlade (ExteriorPoisson.h:411-438) of a packed skew matrix (entry (i, j), j < i, in (i, j)
// order; the matrix m(i, j) = p, m(j, i) = -p in the reference's (column, row) indexing,
// Hat.inl:45-52): the power iteration v2 = Next(v1), v1 <- -Next(v2) with
// Next(v) = normalised (m v - (v . m v) v), stopped when |v1 - v1'|^2 < 1e-10 or after 1000 steps
// (the command line's ProjectionIterations / ProjectionEpslion, ExteriorPoissonRecon.cpp:48-49);
// then a, b = v1, v2 scaled by |m|^(1/2) (Frobenius) and p(i, j) = (a_j b_i - a_i b_j) / 2.  The
// iteration starts from m's largest column (in m's image, never in its kernel; the reference starts
// from a random unit vector, which converges to the same blade).
template <int D>
__device__ void project_blade(double *p)
{
    double m[D][D];
    double sq = 0;
    for (int i = 0; i < D; i++) m[i][i] = 0;
    for (int i = 0, idx = 0; i < D; i++)
        for (int j = 0; j < i; j++, idx++)
        {
            // the reference's SquareMatrix is indexed (column, row) and S() * v sums over columns:
            // as a row-major matrix, row j column i holds p and row i column j holds -p
            m[j][i] = p[idx];
            m[i][j] = -p[idx];
            sq += 2 * p[idx] * p[idx];
        }
    if (sq == 0) return;
    auto next = [&](const double *v, double *out) {
        double w[D], dot = 0, n2 = 0;
        for (int i = 0; i < D; i++)
        {
            w[i] = 0;
            for (int j = 0; j < D; j++) w[i] += m[i][j] * v[j];
        }
        for (int i = 0; i < D; i++) dot += v[i] * w[i];
        for (int i = 0; i < D; i++) { w[i] -= dot * v[i]; n2 += w[i] * w[i]; }
        const double n = sqrt(n2);
        for (int i = 0; i < D; i++) out[i] = w[i] / n;
    };
    double v1[D], v2[D];
    int best = 0;
    double bn = -1;
    for (int k = 0; k < D; k++)
    {
        double n2 = 0;
        for (int i = 0; i < D; i++) n2 += m[i][k] * m[i][k];
        if (n2 > bn) { bn = n2; best = k; }
    }
    for (int i = 0; i < D; i++) { v1[i] = m[i][best] / sqrt(bn); v2[i] = 0; }
    for (int s = 0; s < 1000; s++)
    {
        double nv1[D];
        next(v1, v2);
        next(v2, nv1);
        double d2 = 0;
        for (int i = 0; i < D; i++) { nv1[i] = -nv1[i]; d2 += (v1[i] - nv1[i]) * (v1[i] - nv1[i]); }
        if (d2 < 1e-10) break;
        for (int i = 0; i < D; i++) v1[i] = nv1[i];
    }
    const double scale = sqrt(sqrt(sq));
    for (int i = 0, idx = 0; i < D; i++)
        for (int j = 0; j < i; j++, idx++) p[idx] = ((v1[j] * scale) * (v2[i] * scale) - (v1[i] * scale) * (v2[j] * scale)) / 2.;
}

template <int D>
__global__ void element_frame_kernel(SkewGrids<D> G, double *S, int *leaf, int project)
{
    constexpr int K = D * (D - 1) / 2;
    int r = 1 << G.depth;
    int64_t NE = 1;
    for (int d = 0; d < D; d++) NE *= r;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= NE) return;
    int E[D];
    Grid<D>(G.depth).elem(e, E);
    double p[D];
    for (int d = 0; d < D; d++) p[d] = (E[d] + 0.5) / r;
    int L = 1;
    while (L <= G.depth)
    {
        int side = 1 << L, res = 1 << (L - 1);
        int64_t li = 0;
        for (int d = 0; d < D; d++) li = li * side + tree_cell(p[d], res);
        if (!G.refined[L][li]) break;
        L++;
    }
    double acc[K];
    for (int k = 0; k < K; k++) acc[k] = 0;
    for (int t = 1; t <= L; t++)
    {
        int res = 1 << (t - 1), nv = res + 1;
        int c[D];
        double lv[D][2];
        for (int d = 0; d < D; d++)
        {
            double s = p[d] * res;
            int f = (int)floor(s);
            double x = s - f;
            lv[d][0] = 1. - x;
            lv[d][1] = x;
            c[d] = tree_cell(p[d], res);
        }
        const double *g = G.g[t - 1];
        for (int cc = 0; cc < (1 << D); cc++)
        {
            double w = 1.;
            int64_t vi = 0;
            for (int d = 0; d < D; d++)
            {
                int b = (cc >> (D - 1 - d)) & 1;
                w *= lv[d][b];
                vi = vi * nv + (c[d] + b);
            }
            for (int k = 0; k < K; k++) acc[k] += g[vi * K + k] * w;
        }
    }
    if (project) project_blade<D>(acc);
    for (int k = 0; k < K; k++) S[e * K + k] = acc[k];
    leaf[e] = L;
}

// ---------------------------------------------------------------------------------------------
// deterministic sums
// ---------------------------------------------------------------------------------------------
__global__ void sum_kernel(const double *v, int64_t n, int stride, int comps, double *partial)
{
    __shared__ double sh[32];
    double acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int k = 0; k < comps; k++) { double x = v[i * stride + k]; acc += (comps == 1) ? x : 2 * x * x; }
    acc = warp_sum(acc);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = acc;
    __syncthreads();
    if (w == 0)
    {
        double t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.;
        t = warp_sum(t);
        if (lane == 0) partial[blockIdx.x] = t;
    }
}
__global__ void sum_finish_kernel(const double *partial, int nb, double *out)
{
    double s = 0;
    for (int b = threadIdx.x; b < nb; b += 32) s += partial[b];
    s = warp_sum(s);
    if (threadIdx.x == 0) out[0] = s;
}

// ---------------------------------------------------------------------------------------------
// stencils
// ---------------------------------------------------------------------------------------------
__host__ __device__ inline double mass1(int a, int b) { return a == b ? 1. / 3. : 1. / 6.; }
__host__ __device__ inline double stiff1(int a, int b) { return a == b ? 1. : -1.; }
__host__ __device__ inline double mixed1(int a) { return (a ? 1. : -1.) * 0.5; }

// R = sWeight * mean(measure) * sum_samples w phi_a phi_b, gathered per column node a
template <int D>
__global__ void screening_kernel(const double *pos, const double *noise, const int *order, const int *cellStart,
                                 const int *cellOfFinest, int depth, double nSigma, const double *scaleDev, double *A)
{
    constexpr int S = Dims<D>::S;
    Grid<D> g(depth);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    int I[D];
    g.node(i, I);
    double acc[S];
    for (int o = 0; o < S; o++) acc[o] = 0;
    bool any = false;
    for (int a = 0; a < (1 << D); a++)
    {
        int E[D];
        bool ok = true;
        for (int d = 0; d < D; d++) { E[d] = I[d] - ((a >> (D - 1 - d)) & 1); if (E[d] < 0 || E[d] >= g.r) ok = false; }
        if (!ok) continue;
        int k = cellOfFinest[g.elem(E)];
        if (k < 0) continue;
        any = true;
        for (int j = cellStart[k]; j < cellStart[k + 1]; j++)
        {
            int s = order[j];
            double nz = noise[s];
            double w = exp(-nz * nz / (2. * nSigma * nSigma));
            double lv[D][2];
            for (int d = 0; d < D; d++) { double x = pos[(int64_t)s * D + d] * g.r - E[d]; lv[d][0] = 1. - x; lv[d][1] = x; }
            double pa = 1.;
            for (int d = 0; d < D; d++) pa *= lv[d][(a >> (D - 1 - d)) & 1];
            for (int b = 0; b < (1 << D); b++)
            {
                double pb = 1.;
                int o = 0;
                for (int d = 0; d < D; d++)
                {
                    int cb = (b >> (D - 1 - d)) & 1, ca = (a >> (D - 1 - d)) & 1;
                    pb *= lv[d][cb];
                    o = o * 3 + (cb - ca + 1);
                }
                acc[o] += pa * pb * w;
            }
        }
    }
    if (!any) return;
    double sc = *scaleDev;
    for (int o = 0; o < S; o++) A[(int64_t)o * g.N + i] = acc[o] * sc;
}

// B(f2, f1) = sum_E sum_{a != b} S_E(b, a) int_E d_a phi_f1 d_b phi_f2 (column f1)
// (elements whose frame is zero contribute nothing and are skipped; the element and corner loops
// are unrolled so that the 3^D accumulators stay in registers)
template <int D>
__global__ void __launch_bounds__(128) constraint_kernel(const double *Sel, int depth, double *B)
{
    constexpr int S = Dims<D>::S;
    Grid<D> g(depth);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    int I[D];
    g.node(i, I);
    double acc[S];
#pragma unroll
    for (int o = 0; o < S; o++) acc[o] = 0;
    const double invr = 1. / g.r;
#pragma unroll
    for (int a = 0; a < (1 << D); a++)
    {
        int E[D];
        bool ok = true;
        for (int d = 0; d < D; d++) { E[d] = I[d] - ((a >> (D - 1 - d)) & 1); if (E[d] < 0 || E[d] >= g.r) ok = false; }
        if (!ok) continue;
        const double *s = Sel + g.elem(E) * Dims<D>::K;
        bool zero = true;
        for (int k = 0; k < Dims<D>::K; k++) zero = zero && s[k] == 0;
        if (zero) continue;
#pragma unroll
        for (int b = 0; b < (1 << D); b++)
        {
            int o = 0;
            for (int d = 0; d < D; d++) o = o * 3 + (((b >> (D - 1 - d)) & 1) - ((a >> (D - 1 - d)) & 1) + 1);
            double sum = 0;
            for (int x = 0; x < D; x++)
                for (int y = 0; y < D; y++)
                {
                    if (x == y) continue;
                    // S_E(y, x): full matrix entry (column y, row x) from the packed lower triangle
                    double syx = y > x ? s[y * (y - 1) / 2 + x] : -s[x * (x - 1) / 2 + y];
                    if (syx == 0) continue;
                    double v = 1.;
                    for (int d = 0; d < D; d++)
                    {
                        int ca = (a >> (D - 1 - d)) & 1, cb = (b >> (D - 1 - d)) & 1;
                        if (d == x) v *= mixed1(ca);
                        else if (d == y) v *= mixed1(cb);
                        else v *= mass1(ca, cb) * invr;
                    }
                    sum += syx * v;
                }
            acc[o] += sum;
        }
    }
    for (int o = 0; o < S; o++) B[(int64_t)o * g.N + i] = acc[o];
}

// dst += w K with K the Dirichlet stiffness of the level.  At resolution 1 the reference's
// full-integration stencil table holds only node 0's row (Hat.scalars.inl:261-293: the interior
// case maps to index res/2 = 0 and the upper boundary case is never filled).
template <int D>
__global__ void dirichlet_kernel(int level, double w, double *dst)
{
    constexpr int S = Dims<D>::S;
    Grid<D> g(level);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    if (g.r == 1 && i != 0) return;
    int I[D];
    g.node(i, I);
    const double h = 1. / g.r;
    // The elements shared by nodes I and J form a tensor product of per-axis sets, so
    // int grad phi_I . grad phi_J = sum_k prod_d (k == d ? s_d : m_d) with the per-axis sums of the
    // 1-D stiffness (s_d) and mass (m_d) entries over the shared 1-D elements.
    double sd[D][3], md[D][3];
    for (int d = 0; d < D; d++)
        for (int o = -1; o <= 1; o++)
        {
            int J = I[d] + o;
            double sv = 0, mv = 0;
            if (J >= 0 && J <= g.r)
            {
                int lo = max(max(I[d], J) - 1, 0), hi = min(min(I[d], J), g.r - 1);
                for (int e = lo; e <= hi; e++)
                {
                    int a = I[d] - e, b = J - e;
                    sv += stiff1(a, b) / h;
                    mv += mass1(a, b) * h;
                }
            }
            sd[d][o + 1] = sv;
            md[d][o + 1] = mv;
        }
    for (int o = 0; o < S; o++)
    {
        int off[D];
        stencil_offset<D>(o, off);
        bool ok = true;
        for (int d = 0; d < D; d++)
        {
            int J = I[d] + off[d];
            if (J < 0 || J > g.r) ok = false;
        }
        if (!ok) continue;
        double sum = 0;
        for (int k = 0; k < D; k++)
        {
            double v = 1.;
            for (int d = 0; d < D; d++) v *= (d == k) ? sd[d][off[d] + 1] : md[d][off[d] + 1];
            sum += v;
        }
        dst[(int64_t)o * g.N + i] += w * sum;
    }
}

// 3D Galerkin with every index compile-time: for a coarse node J and fine offsets (go, fo) the
// parity of F = 2 J + go + fo, hence the coarse parents of F relative to J, depend on go and fo
// only, so the 27 accumulators stay in registers.  Same sums, same order as the generic kernel.
__global__ void __launch_bounds__(64) galerkin3_kernel(int fineLevel, const double *Mf, double *Mc)
{
    constexpr int D = 3, S = 27;
    Grid<D> gf(fineLevel), gc(fineLevel - 1);
    int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (J >= gc.N) return;
    int Jc[D];
    gc.node(J, Jc);
    double acc[S];
#pragma unroll
    for (int o = 0; o < S; o++) acc[o] = 0;
#pragma unroll
    for (int go = 0; go < S; go++)
    {
        const int g0 = go / 9 - 1, g1 = (go / 3) % 3 - 1, g2 = go % 3 - 1;
        const int G0 = 2 * Jc[0] + g0, G1 = 2 * Jc[1] + g1, G2 = 2 * Jc[2] + g2;
        if (G0 < 0 || G0 > gf.r || G1 < 0 || G1 > gf.r || G2 < 0 || G2 > gf.r) continue;
        const double wg = (g0 ? 0.5 : 1.) * (g1 ? 0.5 : 1.) * (g2 ? 0.5 : 1.);
        const int64_t gi = ((int64_t)G0 * (gf.r + 1) + G1) * (gf.r + 1) + G2;
#pragma unroll
        for (int fo = 0; fo < S; fo++)
        {
            const double v = Mf[(int64_t)fo * gf.N + gi];
            if (v == 0) continue;
            const int f[3] = {g0 + fo / 9 - 1, g1 + (fo / 3) % 3 - 1, g2 + fo % 3 - 1};  // F - 2 J
            const int n1 = (f[0] & 1) + (f[1] & 1) + (f[2] & 1);
#pragma unroll
            for (int c = 0; c < (1 << n1); c++)
            {
                double w = wg * v;
                int o = 0, bit = 0;
#pragma unroll
                for (int d = 0; d < D; d++)
                {
                    int rel;  // coarse parent of F minus J, + 1
                    if (f[d] & 1) { rel = ((f[d] - 1) >> 1) + ((c >> bit) & 1) + 1; bit++; w *= 0.5; }
                    else rel = (f[d] >> 1) + 1;
                    o = o * 3 + rel;
                }
                acc[o] += w;
            }
        }
    }
#pragma unroll
    for (int o = 0; o < S; o++) Mc[(int64_t)o * gc.N + J] = acc[o];
}

// Galerkin P^T M P of a column stencil, one coarse column per thread
template <int D>
__global__ void galerkin_kernel(int fineLevel, const double *Mf, double *Mc)
{
    constexpr int S = Dims<D>::S;
    Grid<D> gf(fineLevel), gc(fineLevel - 1);
    int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (J >= gc.N) return;
    int Jc[D];
    gc.node(J, Jc);
    double acc[S];
    for (int o = 0; o < S; o++) acc[o] = 0;
    for (int go = 0; go < S; go++)
    {
        int goff[D], G[D];
        stencil_offset<D>(go, goff);
        bool ok = true;
        double wg = 1.;
        for (int d = 0; d < D; d++) { G[d] = 2 * Jc[d] + goff[d]; if (G[d] < 0 || G[d] > gf.r) ok = false; if (goff[d]) wg *= 0.5; }
        if (!ok) continue;
        int64_t gi = gf.node(G);
        for (int fo = 0; fo < S; fo++)
        {
            double v = Mf[(int64_t)fo * gf.N + gi];
            if (v == 0) continue;
            int foff[D], F[D];
            stencil_offset<D>(fo, foff);
            for (int d = 0; d < D; d++) F[d] = G[d] + foff[d];
            int n1 = 0;
            for (int d = 0; d < D; d++) n1 += F[d] & 1;
            for (int c = 0; c < (1 << n1); c++)
            {
                double w = wg * v;
                int o = 0, bit = 0;
                for (int d = 0; d < D; d++)
                {
                    int Ic;
                    if (F[d] & 1) { Ic = ((F[d] - 1) >> 1) + ((c >> bit) & 1); bit++; w *= 0.5; }
                    else Ic = F[d] >> 1;
                    o = o * 3 + (Ic - Jc[d] + 1);
                }
                acc[o] += w;
            }
        }
    }
    for (int o = 0; o < S; o++) Mc[(int64_t)o * gc.N + J] = acc[o];
}

__global__ void scale_by_kernel(double *v, const double *num, double mult, int64_t den)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) v[0] = num[0] * mult / (double)den;
}

template <typename T>
bool dalloc(Context &c, T **p, size_t count, const char *what)
{
    return c.alloc((void **)p, sizeof(T) * count, what);
}

// deterministic device sum of n values (comps==1) or of the Frobenius norms 2 sum v^2 of
// n packed K-vectors (comps==K); result left in *out (device)
bool device_sum(Context &c, const double *v, int64_t n, int comps, double *out)
{
    const int nb = 1024;
    double *partial = nullptr;
    if (!dalloc(c, &partial, nb, "alloc partial")) return false;
    sum_kernel<<<nb, 256, 0, c.stream>>>(v, n, comps, comps, partial);
    sum_finish_kernel<<<1, 32, 0, c.stream>>>(partial, nb, out);
    c.release(partial);
    return c.launch_ok("sum");
}

// Chunked gather of one tree level into grid (NV x W); returns false on a CUDA error.
template <int D, bool Samples, class Item>
bool chunked_level(Context &c, const SplatArgs &a, const Item &item, double scale, double *grid)
{
    constexpr int W = Item::W;
    cudaStream_t s = c.stream;
    int nv = (1 << (a.t - 1)) + 1;
    int64_t NV = 1;
    for (int d = 0; d < D; d++) NV *= nv;
    int *nch = nullptr, *start = nullptr;
    if (!dalloc(c, &nch, NV + 1, "chunks") || !dalloc(c, &start, NV + 1, "chunks")) return false;
    cudaMemsetAsync(nch + NV, 0, sizeof(int), s);
    vertex_chunks_kernel<D, Samples><<<nblocks(NV, 128), 128, 0, s>>>(a, nch);
    {
        size_t tmpBytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tmpBytes, nch, start, (int)(NV + 1), s);
        void *tmp = nullptr;
        if (!c.alloc(&tmp, tmpBytes, "scan tmp")) return false;
        cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, nch, start, (int)(NV + 1), s);
        c.release(tmp);
    }
    int total = 0;
    if (!c.cuda_ok(cudaMemcpyAsync(&total, start + NV, sizeof(int), cudaMemcpyDeviceToHost, s), "copy") ||
        !c.cuda_ok(cudaStreamSynchronize(s), "sync"))
        return false;
    double *partial = nullptr;
    if (total > 0)
    {
        if (!dalloc(c, &partial, (size_t)total * W, "partials")) return false;
        chunk_gather_kernel<D, Samples, Item><<<nblocks((int64_t)total * 32, 256), 256, 0, s>>>(a, item, start, NV, total, partial);
    }
    chunk_finish_kernel<W><<<nblocks(NV, 128), 128, 0, s>>>(start, NV, partial, scale, grid);
    c.release(partial);
    c.release(nch);
    c.release(start);
    return c.launch_ok("chunked gather");
}

template <int D>
bool build_impl(Context &c, Setup &st)
{
    constexpr int K = Dims<D>::K;
    constexpr int W = 1 + D + D * D;
    const int depth = c.depth;
    const int64_t n = (int64_t)st.n;
    cudaStream_t s = c.stream;
    st.release_built(c);
    cudaEventRecord(c.ev0, s);

    // ---- ordered sampling: Morton keys of the finest cells, stable radix sort ----
    int64_t *keys = nullptr, *keysSorted = nullptr;
    int *vals = nullptr, *flags = nullptr, *ids = nullptr;
    if (!dalloc(c, &keys, n, "keys") || !dalloc(c, &keysSorted, n, "keys") || !dalloc(c, &vals, n, "vals") ||
        !dalloc(c, &st.order, n, "order") || !dalloc(c, &flags, n, "flags") || !dalloc(c, &ids, n, "ids"))
        return false;
    cell_keys_kernel<D><<<nblocks(n, 256), 256, 0, s>>>(st.pos, n, depth, keys, vals);
    {
        size_t tmpBytes = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, keys, keysSorted, vals, st.order, (int)n, 0, D * depth, s);
        void *tmp = nullptr;
        if (!c.alloc(&tmp, tmpBytes, "sort tmp")) return false;
        cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, keys, keysSorted, vals, st.order, (int)n, 0, D * depth, s);
        c.release(tmp);
    }
    cell_flags_kernel<<<nblocks(n, 256), 256, 0, s>>>(keysSorted, n, flags);
    {
        size_t tmpBytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tmpBytes, flags, ids, (int)n, s);
        void *tmp = nullptr;
        if (!c.alloc(&tmp, tmpBytes, "scan tmp")) return false;
        cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, flags, ids, (int)n, s);
        c.release(tmp);
    }
    int lastId = 0, lastFlag = 0;
    if (!c.cuda_ok(cudaMemcpyAsync(&lastId, ids + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s), "copy") ||
        !c.cuda_ok(cudaMemcpyAsync(&lastFlag, flags + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s), "copy") ||
        !c.cuda_ok(cudaStreamSynchronize(s), "sync"))
        return false;
    st.ncells = lastId + lastFlag;
    const int64_t nc = st.ncells;
    if (!dalloc(c, &st.cellStart, nc + 1, "cellStart") || !dalloc(c, &st.cellKey, nc, "cellKey")) return false;
    cell_start_kernel<<<nblocks(n, 256), 256, 0, s>>>(keysSorted, flags, ids, n, st.cellStart, st.cellKey);
    c.release(keys); c.release(keysSorted); c.release(vals); c.release(flags); c.release(ids);
    {
        int first = -1, last = -1;
        if (!c.cuda_ok(cudaMemcpyAsync(&first, st.cellStart, sizeof(int), cudaMemcpyDeviceToHost, s), "copy") ||
            !c.cuda_ok(cudaMemcpyAsync(&last, st.cellStart + nc, sizeof(int), cudaMemcpyDeviceToHost, s), "copy") ||
            !c.cuda_ok(cudaStreamSynchronize(s), "sync"))
            return false;
        if (first != 0 || last != (int)n)
        {
            c.fail(EPR_ERR_STATE, "ordered sampling produced inconsistent cell ranges (%d, %d, %lld)", first, last, (long long)n);
            return false;
        }
    }
    Grid<D> gfine(depth);
    if (!dalloc(c, &st.cellOfFinest, gfine.NE, "cell map")) return false;
    cudaMemsetAsync(st.cellOfFinest, 0xff, sizeof(int) * gfine.NE, s);
    finest_map_kernel<D><<<nblocks(nc, 256), 256, 0, s>>>(st.cellKey, nc, depth, st.cellOfFinest);
    if (!c.launch_ok("ordered sampling")) return false;

    // ---- tree structure of both trees ----
    auto buildRefined = [&](std::vector<uint8_t *> &ref, int KR) -> bool {
        ref.assign(depth + 2, nullptr);
        for (int t = 1; t <= depth; t++)
        {
            int64_t cells = 1;
            for (int d = 0; d < D; d++) cells *= (int64_t)1 << t;
            if (!dalloc(c, &ref[t], cells, "refined")) return false;
            cudaMemsetAsync(ref[t], 0, cells, s);
            refine_kernel<D><<<nblocks(nc, 256), 256, 0, s>>>(st.cellKey, nc, depth, t, KR, t > 1 ? ref[t - 1] : nullptr, ref[t]);
        }
        return c.launch_ok("refine");
    };
    if (!buildRefined(st.refinedD, c.P.d_radius)) return false;
    if (!buildRefined(st.refinedS, c.P.t_radius)) return false;

    // ---- occupied-cell ranges of every depth-t cell (shared by both trees) ----
    std::vector<int *> rlo(depth + 2, nullptr), rhi(depth + 2, nullptr);
    for (int t = 1; t <= depth + 1; t++)
    {
        int64_t cells = (int64_t)1 << (D * (t - 1));
        if (!dalloc(c, &rlo[t], cells, "ranges") || !dalloc(c, &rhi[t], cells, "ranges")) return false;
        cudaMemsetAsync(rlo[t], 0, sizeof(int) * cells, s);
        cudaMemsetAsync(rhi[t], 0, sizeof(int) * cells, s);
        level_ranges_kernel<D><<<nblocks(nc, 256), 256, 0, s>>>(st.cellKey, nc, t, D * (depth + 1 - t), rlo[t], rhi[t]);
    }
    if (!c.launch_ok("level ranges")) return false;

    // ---- density splat of the merged cells ----
    double *mean = nullptr, *datum = nullptr;
    if (!dalloc(c, &mean, nc * D, "mean") || !dalloc(c, &datum, nc * W, "datum")) return false;
    merge_cells_kernel<D><<<nblocks(nc, 128), 128, 0, s>>>(st.pos, st.order, st.cellStart, nc, mean, datum);
    st.density.assign(depth + 1, nullptr);
    {
        int KR = c.P.d_radius;
        std::vector<double> bsv(2 * KR + 2);
        {
            // B-spline value at 1/2 of the centre piece (GridSamples.inl:753-756), on the host
            int deg = 2 * KR + 1;
            std::vector<double> v(deg + 1);
            v[deg] = 1.;
            for (int k = 1; k <= deg; k++)
            {
                const double scale = 1. / k;
                int b = deg - k;
                v[b] = v[b + 1] * (1. - 0.5) * scale;
                for (int i = 1; i < k; i++) v[b + i] = (v[b + i] * (0.5 - i + k) + v[b + i + 1] * (-0.5 + i + 1)) * scale;
                v[b + k] *= 0.5 * scale;
            }
            bsv = v;
        }
        double scale = std::pow(1. / bsv[KR + 1], 2);
        double *bs = nullptr;
        if (!dalloc(c, &bs, (size_t)nc * D * (2 * KR + 2), "bspline table")) return false;
        for (int t = 1; t <= depth + 1; t++)
        {
            Grid<D> gl(t - 1);
            if (!dalloc(c, &st.density[t - 1], gl.N * W, "density")) return false;
            SplatArgs a{st.cellKey, st.cellStart, nc, depth, t, KR, rlo[t], rhi[t]};
            double dw = scale / std::pow(std::pow(0.5, t - 1), D - 2);
            item_bspline_kernel<D><<<nblocks(nc, 256), 256, 0, s>>>(mean, nullptr, nc, t, 2 * KR + 1, nullptr, bs);
            DensityItem<D> item{bs, datum, dw};
            if (!chunked_level<D, false>(c, a, item, 1.0, st.density[t - 1])) return false;
        }
        c.release(bs);
    }
    c.release(mean); c.release(datum);
    if (!c.launch_ok("density splat")) return false;

    // ---- estimator queries per sample ----
    if (!dalloc(c, &st.measure, n, "measure") || !dalloc(c, &st.noise, n, "noise") || !dalloc(c, &st.sdepth, n, "depth")) return false;
    {
        DensityGrids<D> G;
        for (int l = 0; l <= depth; l++) G.g[l] = st.density[l];
        G.depth = depth;
        estimator_kernel<D><<<nblocks(n, 128), 128, 0, s>>>(G, st.pos, n, st.measure, st.noise, st.sdepth);
    }
    if (!c.launch_ok("estimator")) return false;

    // ---- frame splat ----
    st.skewGrid.assign(depth + 1, nullptr);
    {
        const int TR = c.P.t_radius;
        double *bs = nullptr, *lw = nullptr, *frame = nullptr;
        if (!dalloc(c, &bs, (size_t)n * D * (2 * TR + 2), "bspline table") || !dalloc(c, &lw, n, "level weights") ||
            !dalloc(c, &frame, (size_t)n * K, "frames"))
            return false;
        skew_frame_kernel<D><<<nblocks(n, 256), 256, 0, s>>>(st.skew, st.measure, st.order, n, depth, frame);
        for (int t = 1; t <= depth + 1; t++)
        {
            Grid<D> gl(t - 1);
            if (!dalloc(c, &st.skewGrid[t - 1], gl.N * K, "skew grid")) return false;
            SplatArgs a{st.cellKey, st.cellStart, nc, depth, t, TR, rlo[t], rhi[t]};
            skew_level_kernel<<<nblocks(n, 256), 256, 0, s>>>(st.sdepth, st.order, n, t, depth, D, lw);
            item_bspline_kernel<D><<<nblocks(n, 256), 256, 0, s>>>(st.pos, st.order, n, t, 2 * TR + 1, lw, bs);
            SkewItem<D> item{bs, lw, frame};
            if (!chunked_level<D, true>(c, a, item, std::pow(std::pow(0.5, depth), 1.5 * 2), st.skewGrid[t - 1])) return false;
        }
        c.release(bs); c.release(lw); c.release(frame);
    }
    if (!c.launch_ok("frame splat")) return false;

    for (int t = 1; t <= depth + 1; t++) { c.release(rlo[t]); c.release(rhi[t]); }

    // ---- S(E), leaf depths, c ----
    if (!dalloc(c, &st.S, gfine.NE * K, "S") || !dalloc(c, &st.leaf, gfine.NE, "leaf")) return false;
    {
        SkewGrids<D> G;
        for (int l = 0; l <= depth; l++) G.g[l] = st.skewGrid[l];
        for (int t = 0; t <= depth + 1 && t < 12; t++) G.refined[t] = st.refinedS[t];
        G.depth = depth;
        element_frame_kernel<D><<<nblocks(gfine.NE, 128), 128, 0, s>>>(G, st.S, st.leaf, c.P.project);
    }
    // the adaptive indexer: its tables, and the frame field restricted to its elements for c and B
    const double *Sfit = st.S;
    double *Smasked = nullptr;
    if (c.P.adaptive_radius >= 0)
    {
        if (!build_adaptive(c, st.cellOfFinest) || !masked_frames(c, st.S, gfine.NE, K, &Smasked)) return false;
        Sfit = Smasked;
    }
    else c.release_adaptive();
    double *dsum = nullptr;
    if (!dalloc(c, &dsum, 4, "sums")) return false;
    if (!device_sum(c, Sfit, gfine.NE, K, dsum)) return false;
    double csum = 0;
    if (!c.cuda_ok(cudaMemcpyAsync(&csum, dsum, sizeof(double), cudaMemcpyDeviceToHost, s), "copy") ||
        !c.cuda_ok(cudaStreamSynchronize(s), "sync"))
        return false;
    c.c = csum / (double)gfine.NE;

    // ---- finest stencils: R (into A64), B ----
    Level &Lf = c.levels[depth];
    const int S = Dims<D>::S;
    cudaMemsetAsync(Lf.A64, 0, sizeof(double) * S * Lf.N, s);
    if (c.P.s_weight > 0)
    {
        if (!device_sum(c, st.measure, n, 1, dsum + 1)) return false;
        scale_by_kernel<<<1, 32, 0, s>>>(dsum + 2, dsum + 1, c.P.s_weight, n);
        screening_kernel<D><<<nblocks(Lf.N, 128), 128, 0, s>>>(st.pos, st.noise, st.order, st.cellStart, st.cellOfFinest, depth,
                                                               c.P.n_sigma, dsum + 2, Lf.A64);
    }
    constraint_kernel<D><<<nblocks(Lf.N, 128), 128, 0, s>>>(Sfit, depth, Lf.B64);
    c.release(Smasked);
    if (!c.launch_ok("finest stencils")) return false;

    // ---- Galerkin hierarchy of R and B, then A = R + dWeight K on every level ----
    for (int l = depth; l > 0; l--)
    {
        Grid<D> gc(l - 1);
        launch_galerkin<D>(l, c.levels[l].A64, c.levels[l - 1].A64, s);
        launch_galerkin<D>(l, c.levels[l].B64, c.levels[l - 1].B64, s);
    }
    if (!c.launch_ok("galerkin")) return false;
    for (int l = 0; l <= depth; l++)
    {
        if (!add_dirichlet(c, l)) return false;
        if (!c.sync_system32(l)) return false;
    }
    c.release(dsum);
    cudaEventRecord(c.ev1, s);
    if (!c.cuda_ok(cudaStreamSynchronize(s), "build sync")) return false;
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    c.stats.build_ms = ms;
    c.have_system = true;
    return true;
}

}  // namespace

bool add_dirichlet_to(Context &c, int level, double *dst, double w)
{
    int64_t N = c.levels[level].N;
    if (c.dim == 3) dirichlet_kernel<3><<<nblocks(N, 128), 128, 0, c.stream>>>(level, w, dst);
    else dirichlet_kernel<4><<<nblocks(N, 128), 128, 0, c.stream>>>(level, w, dst);
    return c.launch_ok("dirichlet");
}

bool add_dirichlet(Context &c, int level) { return add_dirichlet_to(c, level, c.levels[level].A64, c.P.d_weight); }

bool Setup::set_samples(Context &c, size_t n_, const double *pos_, const double *skew_)
{
    release(c);
    n = n_;
    size_t K = (size_t)(c.dim * (c.dim - 1) / 2);
    if (!dalloc(c, &pos, n * c.dim, "pos") || !dalloc(c, &skew, n * K, "skew")) return false;
    return c.cuda_ok(cudaMemcpyAsync(pos, pos_, sizeof(double) * n * c.dim, cudaMemcpyHostToDevice, c.stream), "upload pos") &&
           c.cuda_ok(cudaMemcpyAsync(skew, skew_, sizeof(double) * n * K, cudaMemcpyHostToDevice, c.stream), "upload skew") &&
           c.cuda_ok(cudaStreamSynchronize(c.stream), "sync");
}

bool Setup::build(Context &c)
{
    if (c.dim == 3) return build_impl<3>(c, *this);
    return build_impl<4>(c, *this);
}

bool Setup::get(Context &c, const std::string &name, double *out, size_t cap, size_t *count)
{
    auto copy_d = [&](const double *src, size_t num) -> bool {
        if (count) *count = num;
        if (!out) return true;
        if (!src) { c.fail(EPR_ERR_STATE, "'%s' is not available before epr_build", name.c_str()); return false; }
        if (cap < num) { c.fail(EPR_ERR_ARG, "output too small (%zu < %zu)", cap, num); return false; }
        return c.cuda_ok(cudaMemcpyAsync(out, src, sizeof(double) * num, cudaMemcpyDeviceToHost, c.stream), "copy") &&
               c.cuda_ok(cudaStreamSynchronize(c.stream), "sync");
    };
    size_t K = (size_t)(c.dim * (c.dim - 1) / 2);
    int64_t NE = 1;
    for (int d = 0; d < c.dim; d++) NE *= (int64_t)1 << c.depth;
    if (name == "measure") return copy_d(measure, n);
    if (name == "noise") return copy_d(noise, n);
    if (name == "depth") return copy_d(sdepth, n);
    if (name == "S") return copy_d(S, (size_t)NE * K);
    if (name == "leaf_depth")
    {
        if (count) *count = (size_t)NE;
        if (!out) return true;
        if (!leaf) { c.fail(EPR_ERR_STATE, "not built"); return false; }
        if (cap < (size_t)NE) { c.fail(EPR_ERR_ARG, "output too small"); return false; }
        std::vector<int> h(NE);
        if (!c.cuda_ok(cudaMemcpyAsync(h.data(), leaf, sizeof(int) * NE, cudaMemcpyDeviceToHost, c.stream), "copy") ||
            !c.cuda_ok(cudaStreamSynchronize(c.stream), "sync"))
            return false;
        for (int64_t e = 0; e < NE; e++) out[e] = h[e];
        return true;
    }
    if (name == "ncells")
    {
        if (count) *count = 1;
        if (out && cap >= 1) out[0] = (double)ncells;
        return true;
    }
    c.fail(EPR_ERR_ARG, "unknown array '%s'", name.c_str());
    return false;
}

// Galerkin coarsening of any column stencil (used by the linear multigrid of epr_mg.cu)
template <int D>
void launch_galerkin(int fineLevel, const double *Mf, double *Mc, cudaStream_t s)
{
    Grid<D> gc(fineLevel - 1);
    if constexpr (D == 3) galerkin3_kernel<<<nblocks(gc.N, 64), 64, 0, s>>>(fineLevel, Mf, Mc);
    else galerkin_kernel<D><<<nblocks(gc.N, 64), 64, 0, s>>>(fineLevel, Mf, Mc);
}
template void launch_galerkin<3>(int, const double *, double *, cudaStream_t);
template void launch_galerkin<4>(int, const double *, double *, cudaStream_t);

// the products of a build (everything but the samples), so that a context can be built again
void Setup::release_built(Context &c)
{
    c.release(order); c.release(cellKey); c.release(cellStart); c.release(cellOfFinest);
    c.release(measure); c.release(noise); c.release(sdepth); c.release(S); c.release(leaf);
    for (double *p : density) c.release(p);
    for (double *p : skewGrid) c.release(p);
    for (uint8_t *p : refinedD) c.release(p);
    for (uint8_t *p : refinedS) c.release(p);
    density.clear(); skewGrid.clear(); refinedD.clear(); refinedS.clear();
    measure = noise = sdepth = S = nullptr;
    order = cellStart = cellOfFinest = leaf = nullptr;
    cellKey = nullptr;
    ncells = 0;
}

void Setup::release(Context &c)
{
    release_built(c);
    c.release(pos); c.release(skew);
    pos = skew = nullptr;
    n = 0;
}

}  // namespace epr
