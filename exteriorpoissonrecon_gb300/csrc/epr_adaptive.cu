// The adaptive indexer (Hat::HierarchicalAdaptedIndexer, Include/Hat.adaptive.inl:342-732) on the
// dense level grids, built on the device.
//
// What the indexer holds, level by level (d = 0 .. depth, resolution r = 2^d):
//   * active functions: every node I with 0 <= I <= r inside the window A - K .. A + K + 1 of the
//     level-d ancestor A of an occupied finest cell (K = aRadius; _addSamples, :565-643).  They are
//     the only ones the Gauss-Seidel sweeps relax;
//   * indexed functions: the active ones and every node within one step (3^Dim window) of one
//     (_finalize, :646-728); the others do not exist (their coefficients are zero);
//   * elements: every element with an active corner (the lower-side elements of the active
//     functions' windows).
// Index order (the order of the .tree file and of the random start's draws): active functions in
// the tree's depth-first order, which is Morton order with axis 0 in the lowest bit of every level;
// then the inactive indexed functions, and separately the elements, in the order the finalisation
// discovers them: active functions in index order, each one's 3^Dim neighbours in window order
// (axis 0 slowest).
//
// GPU formulation: the window conditions are box dilations of occupancy grids, computed as one
// pass per axis; the Morton order is a radix sort of interleaved keys; the discovery order is the
// smallest (function index, window slot) key that reaches a node (integer atomicMin over the
// active functions) followed by a radix sort.  Everything is integer work, so the tables are exact
// and independent of scheduling.
#include <cstdio>
#include <cstring>
#include <vector>

#include <cub/cub.cuh>

#include "epr_common.cuh"
#include "epr_context.h"

namespace epr {
namespace {

constexpr unsigned long long kNoKey = ~0ull;

inline unsigned int nblk(int64_t n, int t) { return (unsigned int)((n + t - 1) / t); }

template <int D>
struct Box
{
    int n[D];
    __host__ __device__ int64_t count() const
    {
        int64_t c = 1;
        for (int d = 0; d < D; d++) c *= n[d];
        return c;
    }
};

// One axis of a box dilation: `out` has the shape of `in` with axis `ax` of length outLen, and
// out[.., i, ..] = OR of in[.., a, ..] over a in [i + lo, i + hi] clipped to the input's extent.
template <int D>
__global__ void dilate_axis_kernel(const uint8_t *in, Box<D> inShape, int ax, int outLen, int lo, int hi, uint8_t *out, int64_t nOut)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= nOut) return;
    int c[D];
    int64_t u = o;
    for (int d = D - 1; d >= 0; d--)
    {
        const int len = d == ax ? outLen : inShape.n[d];
        c[d] = (int)(u % len);
        u /= len;
    }
    int64_t stride = 1;
    for (int d = D - 1; d > ax; d--) stride *= inShape.n[d];
    int64_t base = 0;
    for (int d = 0; d < D; d++) base = base * inShape.n[d] + (d == ax ? 0 : c[d]);
    const int a0 = max(c[ax] + lo, 0), a1 = min(c[ax] + hi, inShape.n[ax] - 1);
    uint8_t v = 0;
    for (int a = a0; a <= a1 && !v; a++) v = in[base + (int64_t)a * stride];
    out[o] = v;
}

// occupancy of the finest cells (cell map >= 0)
__global__ void finest_occupancy_kernel(const int *cellOfFinest, int64_t n, uint8_t *occ)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < n) occ[e] = cellOfFinest[e] >= 0 ? 1 : 0;
}

// occupancy of level d from level d + 1: a cell is occupied when one of its children is
template <int D>
__global__ void coarsen_occupancy_kernel(const uint8_t *fine, int rc, uint8_t *coarse)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t n = 1;
    for (int d = 0; d < D; d++) n *= rc;
    if (e >= n) return;
    int E[D];
    int64_t u = e;
    for (int d = D - 1; d >= 0; d--) { E[d] = (int)(u % rc); u /= rc; }
    uint8_t v = 0;
    for (int c = 0; c < (1 << D) && !v; c++)
    {
        int64_t f = 0;
        for (int d = 0; d < D; d++) f = f * (2 * rc) + 2 * E[d] + ((c >> d) & 1);
        v = fine[f];
    }
    coarse[e] = v;
}

// status = 2 (active) / 1 (within one step of an active node) / 0
__global__ void status_kernel(const uint8_t *active, const uint8_t *padded, int64_t n, uint8_t *status)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) status[i] = active[i] ? 2 : (padded[i] ? 1 : 0);
}

// Morton key of every active node (axis 0 in the lowest bit of each level, `bits` levels); the
// others get a key above every Morton key
template <int D>
__global__ void active_keys_kernel(const uint8_t *status, Grid<D> g, int bits, unsigned long long *keys, int64_t *vals)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    vals[i] = i;
    if (status[i] != 2) { keys[i] = 1ull << (D * bits); return; }
    int I[D];
    g.node(i, I);
    unsigned long long k = 0;
    for (int b = bits - 1; b >= 0; b--)
    {
        unsigned long long c = 0;
        for (int d = 0; d < D; d++) c |= (unsigned long long)((I[d] >> b) & 1) << d;
        k = (k << D) | c;
    }
    keys[i] = k;
}

// first discovery of every inactive indexed node and every element by the finalisation's loop:
// key = (active function index) * 3^Dim + (window slot)
template <int D>
__global__ void discover_kernel(const int64_t *fnodes, int64_t nA, const uint8_t *status, Grid<D> g, unsigned long long *keyF,
                                unsigned long long *keyE)
{
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= nA) return;
    constexpr int S = Dims<D>::S;
    int I[D];
    g.node(fnodes[a], I);
    for (int w = 0; w < S; w++)
    {
        int n[D];
        bool fn = true, el = true;
        int rem = w;
        for (int d = D - 1; d >= 0; d--)
        {
            const int off = rem % 3 - 1;
            rem /= 3;
            n[d] = I[d] + off;
            if (n[d] < 0 || n[d] > g.r) fn = false;
            if (n[d] < 0 || n[d] >= g.r || off > 0) el = false;
        }
        const unsigned long long key = (unsigned long long)a * S + w;
        if (fn)
        {
            const int64_t j = g.node(n);
            if (status[j] == 1) atomicMin(&keyF[j], key);
        }
        if (el) atomicMin(&keyE[g.elem(n)], key);
    }
}

// 1 for the colour's nodes that are active (colour-local index jc, Colour::node order)
template <int D>
__global__ void colour_active_flags_kernel(const uint8_t *status, Grid<D> g, Colour<D> col, uint8_t *flags)
{
    const int64_t jc = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (jc >= col.n) return;
    int I[D];
    col.node(jc, I);
    flags[jc] = status[g.node(I)] == 2 ? 1 : 0;
}

__global__ void iota32_kernel(int *v, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = (int)i;
}

__global__ void iota_kernel(int64_t *v, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

__global__ void fill_key_kernel(unsigned long long *v, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = kNoKey;
}

// counts[0] += #(status == 2), counts[1] += #(status == 1)
__global__ void count_status_kernel(const uint8_t *status, int64_t n, unsigned long long *counts)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const uint8_t s = i < n ? status[i] : 0;
    const unsigned a = __ballot_sync(0xffffffffu, s == 2), p = __ballot_sync(0xffffffffu, s == 1);
    if ((threadIdx.x & 31) == 0)
    {
        if (a) atomicAdd(&counts[0], (unsigned long long)__popc(a));
        if (p) atomicAdd(&counts[1], (unsigned long long)__popc(p));
    }
}

__global__ void count_keys_kernel(const unsigned long long *keys, int64_t n, unsigned long long *count)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const unsigned m = __ballot_sync(0xffffffffu, i < n && keys[i] != kNoKey);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

__global__ void indexed_elements_kernel(const unsigned long long *keyE, int64_t n, uint8_t *out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = keyE[i] != kNoKey ? 1 : 0;
}

// rows of a packed frame field (n x K) zeroed where the element is not held by the indexer
__global__ void mask_rows_kernel(const double *S, const uint8_t *keep, int64_t n, int K, double *out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n * K) out[i] = keep[i / K] ? S[i] : 0.0;
}

template <typename T>
bool dalloc(Context &c, T **p, size_t count, const char *what)
{
    return c.alloc((void **)p, sizeof(T) * count, what);
}

// D passes of dilate_axis_kernel: in (shape inShape) -> out (every axis of length outLen), window
// [i + lo, i + hi] on every axis
template <int D>
bool box_dilate(Context &c, const uint8_t *in, Box<D> inShape, int lo, int hi, int outLen, uint8_t *out)
{
    Box<D> shape = inShape;
    const uint8_t *src = in;
    uint8_t *tmp[2] = {nullptr, nullptr};
    for (int ax = 0; ax < D; ax++)
    {
        Box<D> next = shape;
        next.n[ax] = outLen;
        const int64_t n = next.count();
        uint8_t *dst = out;
        if (ax < D - 1)
        {
            uint8_t *&t = tmp[ax & 1];
            c.release(t);
            t = nullptr;
            if (!dalloc(c, &t, (size_t)n, "dilation")) { c.release(tmp[0]); c.release(tmp[1]); return false; }
            dst = t;
        }
        dilate_axis_kernel<D><<<nblk(n, 256), 256, 0, c.stream>>>(src, shape, ax, outLen, lo, hi, dst, n);
        src = dst;
        shape = next;
    }
    const bool ok = c.launch_ok("dilation") && c.cuda_ok(cudaStreamSynchronize(c.stream), "dilation sync");
    c.release(tmp[0]);
    c.release(tmp[1]);
    return ok;
}

template <typename K, typename V>
bool sort_pairs(Context &c, const K *kin, K *kout, const V *vin, V *vout, int64_t n, int bits)
{
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout, (int)n, 0, bits, c.stream);
    void *tmp = nullptr;
    if (!c.alloc(&tmp, bytes, "adaptive sort")) return false;
    cub::DeviceRadixSort::SortPairs(tmp, bytes, kin, kout, vin, vout, (int)n, 0, bits, c.stream);
    const bool ok = c.launch_ok("adaptive sort");
    c.release(tmp);
    return ok;
}

int bits_for(unsigned long long v)
{
    int b = 1;
    while (b < 64 && (v >> b)) b++;
    return b;
}

template <int D>
bool build_impl(Context &c, const int *cellOfFinest)
{
    const int depth = c.depth, K = c.P.adaptive_radius;
    cudaStream_t s = c.stream;
    c.release_adaptive();
    c.adapt.assign(depth + 1, AdaptiveLevel{});
    constexpr int S = Dims<D>::S;

    // occupancy of every level's cells, finest first
    std::vector<uint8_t *> occ(depth + 1, nullptr);
    auto freeOcc = [&]() { for (uint8_t *p : occ) c.release(p); };
    {
        Grid<D> gf(depth);
        if (!dalloc(c, &occ[depth], (size_t)gf.NE, "occupancy")) return false;
        finest_occupancy_kernel<<<nblk(gf.NE, 256), 256, 0, s>>>(cellOfFinest, gf.NE, occ[depth]);
        for (int d = depth - 1; d >= 0; d--)
        {
            Grid<D> g(d);
            if (!dalloc(c, &occ[d], (size_t)g.NE, "occupancy")) { freeOcc(); return false; }
            coarsen_occupancy_kernel<D><<<nblk(g.NE, 256), 256, 0, s>>>(occ[d + 1], g.r, occ[d]);
        }
        if (!c.launch_ok("occupancy")) { freeOcc(); return false; }
    }

    unsigned long long *counts = nullptr;
    if (!dalloc(c, &counts, 4, "counts")) { freeOcc(); return false; }
    bool ok = true;
    for (int d = 0; ok && d <= depth; d++)
    {
        Grid<D> g(d);
        AdaptiveLevel &A = c.adapt[d];
        uint8_t *active = nullptr, *padded = nullptr;
        unsigned long long *keys = nullptr, *keysOut = nullptr, *keyE = nullptr;
        int64_t *vals = nullptr, *valsOut = nullptr;
        Box<D> cells, nodes;
        for (int k = 0; k < D; k++) { cells.n[k] = g.r; nodes.n[k] = g.r + 1; }
        ok = dalloc(c, &active, (size_t)g.N, "active") && dalloc(c, &padded, (size_t)g.N, "padded") &&
             dalloc(c, &A.status, (size_t)g.N, "status") &&
             // active: a node in the (K, K+1) window of an occupied cell, i.e. an occupied cell in
             // the node's window [I - K - 1, I + K]
             box_dilate<D>(c, occ[d], cells, -K - 1, K, g.r + 1, active) &&
             // indexed: within one step of an active node
             box_dilate<D>(c, active, nodes, -1, 1, g.r + 1, padded);
        if (ok)
        {
            status_kernel<<<nblk(g.N, 256), 256, 0, s>>>(active, padded, g.N, A.status);
            cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * 4, s);
            count_status_kernel<<<nblk(g.N, 256), 256, 0, s>>>(A.status, g.N, counts);
            ok = c.launch_ok("status");
        }
        c.release(active);
        c.release(padded);
        unsigned long long hc[2] = {0, 0};
        ok = ok && c.cuda_ok(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, s), "copy") &&
             c.cuda_ok(cudaStreamSynchronize(s), "sync");
        A.nA = (int64_t)hc[0];
        A.nF = (int64_t)(hc[0] + hc[1]);
        // active functions in Morton order
        ok = ok && dalloc(c, &keys, (size_t)g.N, "keys") && dalloc(c, &keysOut, (size_t)g.N, "keys") &&
             dalloc(c, &vals, (size_t)g.N, "vals") && dalloc(c, &valsOut, (size_t)g.N, "vals") &&
             dalloc(c, &A.fnodes, (size_t)std::max<int64_t>(A.nF, 1), "function nodes") &&
             dalloc(c, &keyE, (size_t)g.NE, "element keys");
        if (ok)
        {
            active_keys_kernel<D><<<nblk(g.N, 256), 256, 0, s>>>(A.status, g, d + 1, keys, vals);
            ok = c.launch_ok("morton keys") && sort_pairs(c, keys, keysOut, vals, valsOut, g.N, D * (d + 1) + 1) &&
                 c.cuda_ok(cudaMemcpyAsync(A.fnodes, valsOut, sizeof(int64_t) * A.nA, cudaMemcpyDeviceToDevice, s), "copy");
        }
        // first discoveries of the inactive indexed functions and of the elements
        if (ok)
        {
            fill_key_kernel<<<nblk(g.N, 256), 256, 0, s>>>(keys, g.N);
            fill_key_kernel<<<nblk(g.NE, 256), 256, 0, s>>>(keyE, g.NE);
            if (A.nA) discover_kernel<D><<<nblk(A.nA, 128), 128, 0, s>>>(A.fnodes, A.nA, A.status, g, keys, keyE);
            iota_kernel<<<nblk(g.N, 256), 256, 0, s>>>(vals, g.N);
            const int kb = bits_for((unsigned long long)A.nA * S) + 1;
            ok = c.launch_ok("discovery") && sort_pairs(c, keys, keysOut, vals, valsOut, g.N, kb);
            if (ok && A.nF > A.nA)
                ok = c.cuda_ok(cudaMemcpyAsync(A.fnodes + A.nA, valsOut, sizeof(int64_t) * (A.nF - A.nA), cudaMemcpyDeviceToDevice, s), "copy");
            if (ok)
            {
                cudaMemsetAsync(counts, 0, sizeof(unsigned long long), s);
                count_keys_kernel<<<nblk(g.NE, 256), 256, 0, s>>>(keyE, g.NE, counts);
                iota_kernel<<<nblk(g.NE, 256), 256, 0, s>>>(vals, g.NE);
                unsigned long long ne = 0;
                ok = c.launch_ok("element count") && c.cuda_ok(cudaMemcpyAsync(&ne, counts, sizeof(ne), cudaMemcpyDeviceToHost, s), "copy") &&
                     c.cuda_ok(cudaStreamSynchronize(s), "sync");
                A.nE = (int64_t)ne;
                if (ok && d == depth)
                {
                    ok = dalloc(c, &c.elem_indexed, (size_t)g.NE, "indexed elements");
                    if (ok) indexed_elements_kernel<<<nblk(g.NE, 256), 256, 0, s>>>(keyE, g.NE, c.elem_indexed);
                }
                ok = ok && dalloc(c, &A.enodes, (size_t)std::max<int64_t>(A.nE, 1), "element nodes") &&
                     sort_pairs(c, keyE, keys, vals, valsOut, g.NE, kb) &&
                     c.cuda_ok(cudaMemcpyAsync(A.enodes, valsOut, sizeof(int64_t) * A.nE, cudaMemcpyDeviceToDevice, s), "copy") &&
                     c.cuda_ok(cudaStreamSynchronize(s), "sync");
            }
        }
        c.release(keys); c.release(keysOut); c.release(vals); c.release(valsOut); c.release(keyE);
        // every colour's active nodes as colour-local indices, in colour order (the relaxation's
        // work lists)
        uint8_t *flags = nullptr;
        int *num = nullptr, *seq = nullptr;
        ok = ok && dalloc(c, &A.clist, (size_t)std::max<int64_t>(A.nA, 1), "colour lists") && dalloc(c, &flags, (size_t)g.N, "flags") &&
             dalloc(c, &num, 1, "count") && dalloc(c, &seq, (size_t)g.N, "sequence");
        if (ok) iota32_kernel<<<nblk(g.N, 256), 256, 0, s>>>(seq, g.N);
        A.coff[0] = 0;
        for (int col = 0; ok && col < (1 << D); col++)
        {
            Colour<D> cl(g, col);
            colour_active_flags_kernel<D><<<nblk(cl.n, 256), 256, 0, s>>>(A.status, g, cl, flags);
            size_t bytes = 0;
            cub::DeviceSelect::Flagged(nullptr, bytes, seq, flags, A.clist + A.coff[col], num, (int)cl.n, s);
            void *tmp = nullptr;
            ok = c.alloc(&tmp, bytes, "colour lists");
            if (ok) cub::DeviceSelect::Flagged(tmp, bytes, seq, flags, A.clist + A.coff[col], num, (int)cl.n, s);
            int h = 0;
            ok = ok && c.launch_ok("colour lists") && c.cuda_ok(cudaMemcpyAsync(&h, num, sizeof(int), cudaMemcpyDeviceToHost, s), "copy") &&
                 c.cuda_ok(cudaStreamSynchronize(s), "sync");
            c.release(tmp);
            A.coff[col + 1] = A.coff[col] + h;
        }
        if (ok && A.coff[1 << D] != A.nA)
        {
            c.fail(EPR_ERR_STATE, "adaptive level %d: colour lists hold %d of %lld active nodes", d, A.coff[1 << D], (long long)A.nA);
            ok = false;
        }
        c.release(flags);
        c.release(num);
        c.release(seq);
    }
    c.release(counts);
    freeOcc();
    return ok;
}

// nodes of a level's grid that are active, written as 1 into the (side)^Dim grid of tree depth
// level + 1 (a level's functions are the tree nodes of that depth with offsets 0 .. 2^level)
template <int D>
__global__ void embed_active_kernel(const uint8_t *status, Grid<D> g, int side, uint8_t *out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= g.N || status[i] != 2) return;
    int I[D];
    g.node(i, I);
    int64_t o = 0;
    for (int d = 0; d < D; d++) o = o * side + I[d];
    out[o] = 1;
}

__global__ void or_kernel(uint8_t *a, const uint8_t *b, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) a[i] |= b[i];
}

// Which nodes of the adaptive indexer's tree have children, per tree depth t = 0 .. depth + 1
// ((2^t)^Dim flags each).  The indexer creates (RegularTree.inl:728-845, getNeighbors with node
// creation) the children of every parent of a node in (a) the (K, K+1) window of a sample cell's
// ancestor at every depth (Hat.adaptive.inl:583-604) and (b) the one-ring window of every ancestor
// of an active function (Hat.adaptive.inl:676-701).  M_t marks those nodes at tree depth t:
// (a) is the occupancy of level t-1 dilated by [o - K - 1, o + K] onto the (2^t)^Dim grid, (b) the
// one-ring dilation of Q_t = the active functions of level t-1 plus the parents of Q_{t+1}; a node
// of depth t-1 has children when one of its children is marked.
template <int D>
bool refinement_impl(Context &c, const int *cellOfFinest, std::vector<std::vector<uint8_t>> &refined)
{
    const int depth = c.depth, K = c.P.adaptive_radius;
    cudaStream_t s = c.stream;
    refined.assign(depth + 2, {});
    refined[0].assign(1, 1);
    refined[depth + 1].assign((size_t)1 << (D * (depth + 1)), 0);
    std::vector<uint8_t *> occ(depth + 1, nullptr);
    uint8_t *Q = nullptr, *Qnext = nullptr, *Ma = nullptr, *Mb = nullptr, *flags = nullptr;
    auto cleanup = [&]() {
        for (uint8_t *p : occ) c.release(p);
        c.release(Q); c.release(Qnext); c.release(Ma); c.release(Mb); c.release(flags);
    };
    {
        Grid<D> gf(depth);
        if (!dalloc(c, &occ[depth], (size_t)gf.NE, "occupancy")) { cleanup(); return false; }
        finest_occupancy_kernel<<<nblk(gf.NE, 256), 256, 0, s>>>(cellOfFinest, gf.NE, occ[depth]);
        for (int d = depth - 1; d >= 0; d--)
        {
            Grid<D> g(d);
            if (!dalloc(c, &occ[d], (size_t)g.NE, "occupancy")) { cleanup(); return false; }
            coarsen_occupancy_kernel<D><<<nblk(g.NE, 256), 256, 0, s>>>(occ[d + 1], g.r, occ[d]);
        }
    }
    for (int t = depth + 1; t >= 1; t--)
    {
        const int side = 1 << t;
        Box<D> cellsBelow, grid;
        for (int k = 0; k < D; k++) { cellsBelow.n[k] = side / 2; grid.n[k] = side; }
        const int64_t n = grid.count();
        c.release(Q);
        Q = nullptr;
        if (!dalloc(c, &Q, (size_t)n, "tree marks") || !dalloc(c, &Ma, (size_t)n, "tree marks") || !dalloc(c, &Mb, (size_t)n, "tree marks"))
        {
            cleanup();
            return false;
        }
        // Q_t: the active functions of level t-1 and the parents of Q_{t+1}
        if (Qnext) coarsen_occupancy_kernel<D><<<nblk(n, 256), 256, 0, s>>>(Qnext, side, Q);
        else cudaMemsetAsync(Q, 0, (size_t)n, s);
        {
            Grid<D> g(t - 1);
            embed_active_kernel<D><<<nblk(g.N, 256), 256, 0, s>>>(c.adapt[t - 1].status, g, side, Q);
        }
        if (!c.launch_ok("tree marks") || !box_dilate<D>(c, occ[t - 1], cellsBelow, -K - 1, K, side, Ma) ||
            !box_dilate<D>(c, Q, grid, -1, 1, side, Mb))
        {
            cleanup();
            return false;
        }
        or_kernel<<<nblk(n, 256), 256, 0, s>>>(Ma, Mb, n);
        // depth t-1: children where a child is marked
        const int64_t np = n >> D;
        if (!dalloc(c, &flags, (size_t)np, "tree flags")) { cleanup(); return false; }
        coarsen_occupancy_kernel<D><<<nblk(np, 256), 256, 0, s>>>(Ma, side / 2, flags);
        if (t - 1 >= 1)
        {
            refined[t - 1].resize((size_t)np);
            if (!c.cuda_ok(cudaMemcpyAsync(refined[t - 1].data(), flags, (size_t)np, cudaMemcpyDeviceToHost, s), "copy"))
            {
                cleanup();
                return false;
            }
        }
        if (!c.cuda_ok(cudaStreamSynchronize(s), "sync")) { cleanup(); return false; }
        c.release(flags); c.release(Ma); c.release(Mb); c.release(Qnext);
        flags = Ma = Mb = nullptr;
        Qnext = Q;
        Q = nullptr;
    }
    cleanup();
    return true;
}

}  // namespace

bool adaptive_tree_refinement(Context &c, std::vector<std::vector<uint8_t>> &refined)
{
    if (c.adapt.empty() || !c.setup.cellOfFinest)
    {
        c.fail(EPR_ERR_STATE, "the adaptive indexer's tree is not available before epr_build");
        return false;
    }
    if (c.dim == 3) return refinement_impl<3>(c, c.setup.cellOfFinest, refined);
    return refinement_impl<4>(c, c.setup.cellOfFinest, refined);
}

bool build_adaptive(Context &c, const int *cellOfFinest)
{
    if (c.dim == 3) return build_impl<3>(c, cellOfFinest);
    return build_impl<4>(c, cellOfFinest);
}

// S with the rows of elements outside the indexer zeroed (the constraint and c integrate the
// indexer's elements only, Hat.scalars.inl:1585-1690, SystemEnergy.h:452-461)
bool masked_frames(Context &c, const double *S, int64_t nElements, int K, double **out)
{
    *out = nullptr;
    if (!c.alloc((void **)out, sizeof(double) * nElements * K, "masked frames")) return false;
    mask_rows_kernel<<<nblk(nElements * K, 256), 256, 0, c.stream>>>(S, c.elem_indexed, nElements, K, *out);
    return c.launch_ok("mask frames");
}

void Context::release_adaptive()
{
    for (AdaptiveLevel &A : adapt)
    {
        release(A.status);
        release(A.fnodes);
        release(A.enodes);
        release(A.clist);
    }
    adapt.clear();
    release(elem_indexed);
    elem_indexed = nullptr;
}

}  // namespace epr
