// Solve-path kernels: energy, quadratic fit, paired Gauss-Seidel colour sweep, Gauss-Newton
// matvec, prolongation / restriction.  Templated on the dimension (3, 4) and the arithmetic type
// (double for the parity path, float for the fast path).
//
// Reference correspondence:
//   energy        SingleCycleCascadicSystemEnergy::energies          SystemEnergy.h:486-497
//   node fit      SingleCycleCascadicSystemEnergy::quadraticFit      SystemEnergy.h:542-643
//   GS colour     PairedGaussSeidelSolve (one parity colour)         ExteriorPoissonSolvers.h:156-196
//   prolongation  ScalarFunctions::prolongation                      Hat.scalars.inl:1747-1779
//   restriction   its transpose (the Galerkin restriction of MG.h:120-127)
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include <cooperative_groups.h>

#include "epr_common.cuh"
#include "epr_element.cuh"
#include "epr_kernels.h"

namespace epr {

namespace {

constexpr int kThreads = 128;

template <typename Real>
__device__ __forceinline__ Real2<Real> ld2(const Real *xy, int64_t i)
{
    return reinterpret_cast<const Real2<Real> *>(xy)[i];
}

// r^(4-D)/2: scale from reference-element sums to physical integrals
template <int D>
__device__ __forceinline__ double wedge_scale(int r)
{
    return (D == 3 ? (double)r : 1.0) * 0.5;
}

template <int D>
struct NodeCtx
{
    int I[D];
    int64_t stride[D];
};

// Gather the corners of the element whose local corner A is the node I.
template <int D, typename Real>
__device__ __forceinline__ bool gather_element(const Grid<D> &g, const NodeCtx<D> &nc, int64_t i, int A, const Real *xy,
                                               Real *x, Real *y)
{
#pragma unroll
    for (int d = 0; d < D; d++)
    {
        int e = nc.I[d] - cbit<D>(A, d);
        if (e < 0 || e >= g.r) return false;
    }
#pragma unroll
    for (int c = 0; c < (1 << D); c++)
    {
        int64_t j = i;
#pragma unroll
        for (int d = 0; d < D; d++) j += (int64_t)(cbit<D>(c, d) - cbit<D>(A, d)) * nc.stride[d];
        Real2<Real> v = ld2(xy, j);
        x[c] = v.x;
        y[c] = v.y;
    }
    return true;
}

// stencil index of the neighbour at offset (o_0, ..., o_{D-1}), o_d in {-1, 0, 1}
template <int D>
__host__ __device__ constexpr int nb_index(const int *off)
{
    int o = 0;
    for (int d = 0; d < D; d++) o = o * 3 + (off[d] + 1);
    return o;
}

// Wedge part of the quadratic model of node i, elements in canonical orientation.
template <int D, typename Real>
__device__ __forceinline__ void node_wedge_fit(const Grid<D> &g, const NodeCtx<D> &nc, int64_t i, const Real *xy, Real *h)
{
    if constexpr (D == 3)
    {
        // the 27-node neighbourhood in registers; out-of-domain neighbours are never used
        Real2<Real> nb[27];
#pragma unroll
        for (int o = 0; o < 27; o++)
        {
            const int o0 = o / 9 - 1, o1 = (o / 3) % 3 - 1, o2 = o % 3 - 1;
            bool ok = (nc.I[0] + o0 >= 0) && (nc.I[0] + o0 <= g.r) && (nc.I[1] + o1 >= 0) && (nc.I[1] + o1 <= g.r) &&
                      (nc.I[2] + o2 >= 0) && (nc.I[2] + o2 <= g.r);
            int64_t j = i + o0 * nc.stride[0] + o1 * nc.stride[1] + o2 * nc.stride[2];
            nb[o] = ok ? ld2(xy, j) : Real2<Real>{0, 0};
        }
#pragma unroll
        for (int A = 0; A < 8; A++)
        {
            const int a0 = (A >> 2) & 1, a1 = (A >> 1) & 1, a2 = A & 1;
            bool ok = (nc.I[0] - a0 >= 0) && (nc.I[0] - a0 < g.r) && (nc.I[1] - a1 >= 0) && (nc.I[1] - a1 < g.r) &&
                      (nc.I[2] - a2 >= 0) && (nc.I[2] - a2 < g.r);
            if (!ok) continue;
            Corners<3, Real> c;
#pragma unroll
            for (int cc = 0; cc < 8; cc++)
            {
                int off[3] = {(a0 ? -1 : 1) * ((cc >> 2) & 1), (a1 ? -1 : 1) * ((cc >> 1) & 1), (a2 ? -1 : 1) * (cc & 1)};
                Real2<Real> v = nb[nb_index<3>(off)];
                c.x[cc] = v.x;
                c.y[cc] = v.y;
            }
            Fit5<Real> f = element_fit_canonical<3, Real>(c);
#pragma unroll
            for (int k = 0; k < 5; k++) h[k] += f.h[k];
        }
    }
    else
    {
#pragma unroll 1
        for (int A = 0; A < (1 << D); A++)
        {
            bool ok = true;
#pragma unroll
            for (int d = 0; d < D; d++)
            {
                int e = nc.I[d] - cbit<D>(A, d);
                ok = ok && e >= 0 && e < g.r;
            }
            if (!ok) continue;
            Corners<D, Real> c;
#pragma unroll
            for (int cc = 0; cc < (1 << D); cc++)
            {
                int64_t j = i;
#pragma unroll
                for (int d = 0; d < D; d++) j += (int64_t)(cbit<D>(A, d) ? -cbit<D>(cc, d) : cbit<D>(cc, d)) * nc.stride[d];
                Real2<Real> v = ld2(xy, j);
                c.x[cc] = v.x;
                c.y[cc] = v.y;
            }
            Fit5<Real> f = element_fit_canonical<D, Real>(c);
#pragma unroll
            for (int k = 0; k < 5; k++) h[k] += f.h[k];
        }
    }
}

// Quadratic model of E(x + s e_i, y + t e_i): q = (Q20, Q02, Q11, Q10, Q01)
template <int D, typename Real>
__device__ __forceinline__ void node_fit(const LevelPtrs<Real> &L, const Grid<D> &g, const NodeCtx<D> &nc, int64_t i,
                                         const Real *xy, Real *q)
{
    Real h[5] = {0, 0, 0, 0, 0};
    node_wedge_fit<D, Real>(g, nc, i, xy, h);
    const Real sc = (Real)wedge_scale<D>(g.r);
    q[0] = h[0] * sc;
    q[1] = h[1] * sc;
    q[2] = (Real)2 * h[2] * sc;
    q[3] = (Real)2 * h[3] * sc;
    q[4] = (Real)2 * h[4] * sc;
    // screening + Dirichlet (A column) and frame constraint (B column, without its diagonal)
    constexpr int S = Dims<D>::S;
    Real ax = 0, ay = 0, bx = 0, by = 0, acen = 0;
#pragma unroll 3
    for (int o = 0; o < S; o++)
    {
        int off[D];
        stencil_offset<D>(o, off);
        bool ok = true;
        int64_t j = i;
#pragma unroll
        for (int d = 0; d < D; d++)
        {
            int t = nc.I[d] + off[d];
            ok = ok && (t >= 0) && (t <= g.r);
            j += (int64_t)off[d] * nc.stride[d];
        }
        if (!ok) continue;
        Real a = L.A[(int64_t)o * L.N + i];
        Real b = L.B[(int64_t)o * L.N + i];
        Real2<Real> v = ld2(xy, j);
        ax += a * v.x;
        ay += a * v.y;
        if (o == Dims<D>::CENTER) acen = a;
        else { bx += b * v.x; by += b * v.y; }
    }
    q[0] += acen;
    q[1] += acen;
    q[3] += (Real)2 * ax - (Real)2 * by;
    q[4] += (Real)2 * ay + (Real)2 * bx;
}

template <int D>
__device__ __forceinline__ void make_ctx(const Grid<D> &g, int64_t i, NodeCtx<D> &nc)
{
    g.node(i, nc.I);
#pragma unroll
    for (int d = 0; d < D; d++) nc.stride[d] = g.stride(d);
}

// ---------------------------------------------------------------------------------------------
// deterministic block reduction of up to 3 doubles
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ void block_sum_store(double *v, double *dst)
{
    __shared__ double sh[NV][32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
    {
        double t = warp_sum(v[k]);
        if (lane == 0) sh[k][w] = t;
    }
    __syncthreads();
    if (w == 0)
    {
        int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int k = 0; k < NV; k++)
        {
            double t = lane < nw ? sh[k][lane] : 0.0;
            t = warp_sum(t);
            if (lane == 0) dst[k] = t;
        }
    }
}

template <int D, typename Real>
__global__ void __launch_bounds__(kThreads) energy_kernel(LevelPtrs<Real> L, const Real *xy, double *partial)
{
    Grid<D> g(L.level);
    double acc[3] = {0, 0, 0};
    const int64_t total = g.N > g.NE ? g.N : g.NE;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    {
        if (t < g.NE)
        {
            int E[D];
            g.elem(t, E);
            Real x[1 << D], y[1 << D];
            int64_t base = 0;
#pragma unroll
            for (int d = 0; d < D; d++) base = base * (g.r + 1) + E[d];
#pragma unroll
            for (int c = 0; c < (1 << D); c++)
            {
                int64_t j = base;
#pragma unroll
                for (int d = 0; d < D; d++) j += cbit<D>(c, d) * g.stride(d);
                Real2<Real> v = ld2(xy, j);
                x[c] = v.x;
                y[c] = v.y;
            }
            acc[0] += (double)element_wedge<D, Real>(x, y);
        }
        if (t < g.N)
        {
            NodeCtx<D> nc;
            make_ctx<D>(g, t, nc);
            Real2<Real> me = ld2(xy, t);
            double xb = 0, xa = 0;
            constexpr int S = Dims<D>::S;
            for (int o = 0; o < S; o++)
            {
                int off[D];
                stencil_offset<D>(o, off);
                bool ok = true;
                int64_t j = t;
#pragma unroll
                for (int d = 0; d < D; d++)
                {
                    int q = nc.I[d] + off[d];
                    ok = ok && (q >= 0) && (q <= g.r);
                    j += (int64_t)off[d] * nc.stride[d];
                }
                if (!ok) continue;
                Real2<Real> v = ld2(xy, j);
                double a = (double)L.A[(int64_t)o * L.N + t], b = (double)L.B[(int64_t)o * L.N + t];
                xb += b * (double)v.y;
                xa += a * ((double)me.x * (double)v.x + (double)me.y * (double)v.y);
            }
            acc[1] += (double)me.x * xb;
            acc[2] += xa;
        }
    }
    block_sum_store<3>(acc, partial + 4 * blockIdx.x);
}

__global__ void finish_kernel(const double *partial, int nblocks, int nv, double *out, double scale0)
{
    // one warp per value, fixed order
    int v = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (v >= nv) return;
    double s = 0;
    for (int b = lane; b < nblocks; b += 32) s += partial[4 * b + v];
    s = warp_sum(s);
    if (lane == 0) out[v] = (v == 0) ? s * scale0 : s;
}

template <int D, typename Real>
__global__ void __launch_bounds__(kThreads) quadfit_kernel(LevelPtrs<Real> L, const Real *xy, double *out)
{
    Grid<D> g(L.level);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    NodeCtx<D> nc;
    make_ctx<D>(g, i, nc);
    Real q[5];
    node_fit<D, Real>(L, g, nc, i, xy, q);
#pragma unroll
    for (int k = 0; k < 5; k++) out[i * 5 + k] = (double)q[k];
}

// sum over the nodes of |dE/dx_i|^2 + |dE/dy_i|^2 (the linear coefficients of the node fits)
template <int D, typename Real>
__global__ void __launch_bounds__(kThreads) grad_norm_kernel(LevelPtrs<Real> L, const Real *xy, double *partial)
{
    Grid<D> g(L.level);
    double acc[1] = {0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < g.N; i += (int64_t)gridDim.x * blockDim.x)
    {
        NodeCtx<D> nc;
        make_ctx<D>(g, i, nc);
        Real q[5];
        node_fit<D, Real>(L, g, nc, i, xy, q);
        acc[0] += (double)q[3] * (double)q[3] + (double)q[4] * (double)q[4];
    }
    block_sum_store<1>(acc, partial + 4 * blockIdx.x);
}

// Node step from the quadratic model q = (Q20, Q02, Q11, Q10, Q01) with H = [[2 Q20, Q11], [Q11, 2 Q02]]
// and grad = (Q10, Q01).  Paired (ExteriorPoissonSolvers.h:173-181): -H^{-1} grad / 2 when
// |det H| > 1e-20.  Separate (ExteriorPoissonSolvers.h:216-235): p0 = -grad0 / (2 H00) when
// H00 > 1e-20, then p1 = -((H10 + H01) p0 + grad1) / (2 H11) when H11 > 1e-20.
template <typename Real>
__device__ __forceinline__ bool node_step(const Real *q, int separate, Real &p0, Real &p1)
{
    Real h00 = (Real)2 * q[0], h11 = (Real)2 * q[1], h01 = q[2];
    if (separate)
    {
        p0 = 0;
        p1 = 0;
        if ((double)h00 > 1e-20) p0 = -((h01 + h01) * p1 + q[3]) / ((Real)2 * h00);
        if ((double)h11 > 1e-20) p1 = -((h01 + h01) * p0 + q[4]) / ((Real)2 * h11);
        return true;
    }
    Real det = h00 * h11 - h01 * h01;
    if (!(fabs((double)det) > 1e-20)) return false;
    p0 = -(h11 * q[3] - h01 * q[4]) / det / (Real)2;
    p1 = -(-h01 * q[3] + h00 * q[4]) / det / (Real)2;
    return true;
}

// Whether the Gauss-Seidel step of node i is applied: every node of the regular grid, the active
// functions of the adaptive indexer (its colour lists hold those only, ExteriorPoisson.h:161-169)
template <typename Real>
__device__ __forceinline__ bool relaxed(const LevelPtrs<Real> &L, int64_t i)
{
    return L.status == nullptr || L.status[i] == 2;
}

// Comparisons and finiteness tests in a level's own arithmetic: a double-float tests its pair
// without converting to FP64 where the leading float decides.
template <typename Real>
__device__ __forceinline__ bool exceeds(Real v, double t)
{
    return (double)v > t;
}
// a double-float compares by its leading float unless that is within a factor of two of t
template <>
__device__ __forceinline__ bool exceeds<df>(df v, double t)
{
    const float tf = (float)t;
    if (v.hi > 2.f * tf) return true;
    if (v.hi < 0.5f * tf) return false;
    return (double)v.hi + (double)v.lo > t;
}
template <typename Real>
__device__ __forceinline__ Real abs_value(Real v)
{
    return v < (Real)0 ? -v : v;
}
template <>
__device__ __forceinline__ df abs_value<df>(df v)
{
    return v.hi < 0.f ? -v : v;
}
template <typename Real>
__device__ __forceinline__ bool finite_value(Real v)
{
    return isfinite((double)v);
}
template <>
__device__ __forceinline__ bool finite_value<df>(df v)
{
    return isfinite(v.hi) && isfinite(v.lo);
}

// node_step with the singularity tests in the level's own arithmetic
template <typename Real>
__device__ __forceinline__ bool node_step_tiny(const Real *q, int separate, Real &p0, Real &p1)
{
    Real h00 = (Real)2 * q[0], h11 = (Real)2 * q[1], h01 = q[2];
    if (separate)
    {
        p0 = 0;
        p1 = 0;
        if (exceeds<Real>(h00, 1e-20)) p0 = -((h01 + h01) * p1 + q[3]) / ((Real)2 * h00);
        if (exceeds<Real>(h11, 1e-20)) p1 = -((h01 + h01) * p0 + q[4]) / ((Real)2 * h11);
        return true;
    }
    Real det = h00 * h11 - h01 * h01;
    if (!exceeds<Real>(abs_value<Real>(det), 1e-20)) return false;
    // -H^{-1} grad / 2 with one division
    const Real m = (Real)-0.5 / det;
    p0 = (h11 * q[3] - h01 * q[4]) * m;
    p1 = (-h01 * q[3] + h00 * q[4]) * m;
    return true;
}

// Paired Gauss-Seidel update of node j of a parity colour.
template <int D, typename Real>
__device__ __forceinline__ void gs_update(const LevelPtrs<Real> &L, const Grid<D> &g, const Colour<D> &col, int64_t j, unsigned int *err,
                                          int separate)
{
    NodeCtx<D> nc;
    col.node(j, nc.I);
#pragma unroll
    for (int d = 0; d < D; d++) nc.stride[d] = g.stride(d);
    int64_t i = g.node(nc.I);
    Real q[5];
    node_fit<D, Real>(L, g, nc, i, L.xy, q);
    Real p0, p1;
    if (relaxed(L, i) && node_step<Real>(q, separate, p0, p1))
    {
        Real2<Real> v = ld2(L.xy, i);
        v.x += p0;
        v.y += p1;
        if (!isfinite((double)v.x) || !isfinite((double)v.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
        reinterpret_cast<Real2<Real> *>(L.xy)[i] = v;
    }
}

// One parity colour: same-colour nodes share no element, so all of them are updated in parallel
// exactly as the reference's per-colour ParallelFor does.
template <int D, typename Real>
__global__ void __launch_bounds__(kThreads) gs_colour_kernel(LevelPtrs<Real> L, Colour<D> col, unsigned int *err, int separate)
{
    Grid<D> g(L.level);
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= col.n) return;
    gs_update<D, Real>(L, g, col, j, err, separate);
}

// Lane-parallel variant: a group of 2^D consecutive lanes updates one node, lane A integrating the
// node's element A (canonical orientation) and a share of its stencil column; the group reduces
// with shuffles in a fixed order and its first lane writes the update.
template <int D>
__device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = (1 << D) / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, 1 << D);
    return v;
}
template <int D>
__device__ __forceinline__ double group_sum(double v)
{
#pragma unroll
    for (int o = (1 << D) / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, 1 << D);
    return v;
}
template <int D>
__device__ __forceinline__ df group_sum(df v)
{
#pragma unroll
    for (int o = (1 << D) / 2; o > 0; o >>= 1) v += shfl_xor_any(v, o, 1 << D);
    return v;
}

// Power-of-two shift that brings the largest stored magnitude |hi| of a double-float level into
// [1, 2), or 0 while it stays within [2^-8, 2^9) (or the level is zero).  The whole block calls it;
// it ends with a barrier.
__device__ __forceinline__ int df_rescale_shift(const df *v, int64_t n)
{
    __shared__ float wmax[32];
    __shared__ int shift;
    float m = 0.f;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) m = fmaxf(m, fabsf(v[k].hi));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        float mm = 0.f;
        for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) mm = fmaxf(mm, wmax[w]);
        const int e = mm > 0.f ? ilogbf(mm) : 0;
        shift = (mm > 0.f && (e < -8 || e > 8)) ? -e : 0;
    }
    __syncthreads();
    return shift;
}

// Factor of the wedge integrals of a level kept in double-float at the exponent k of its level
// (coefficients stored as x 2^-k): the fit's wedge terms carry two more powers of the coefficients
// than its stencil terms, so they are multiplied by 2^(2k) (exactly 1 for float and double levels).
template <typename Real>
__device__ __forceinline__ Real wedge_mult(const int *kexp, int level)
{
    if constexpr (std::is_same<Real, df>::value) return kexp ? ldexp_df(df(1), 2 * kexp[level]) : df(1);
    else return (Real)1;
}

// A block's row of nodes staged in shared memory (3D lane kernel): the (x, y) pairs of the 3 x 3 x W
// grid points around the row (W = 2 nodes-per-block + 1 along the last axis) and the rows' stencil
// columns, loaded once per block with coalesced loads, so that a node's 8 lanes read their corners
// and neighbours from shared memory instead of re-fetching them through L1 / L2.
template <typename Real>
struct LaneStage
{
    const Real2<Real> *tile = nullptr;
    int tcentre = 0;  // tile index of the node (the tile's row length is a template parameter)
    const Real *As = nullptr, *Bs = nullptr;  // column o of the block's t-th node at o npb + t
    int npb = 0, t = 0;
};

// Ac, Bc (optional): the colour's block of the colour-blocked stencils, the node being the colour's
// jc-th of nc; otherwise the natural stencils L.A, L.B are read.  Staged (3D): corners, neighbours
// and stencil columns come from stg (the same values, so the same arithmetic).
template <int D, typename Real, bool Packed = false, bool Staged = false, int SW = 1>
__device__ __forceinline__ void gs_update_lanes_at(const LevelPtrs<Real> &L, Real *xy, const Grid<D> &g, const int *I, bool active,
                                                   int A, unsigned int *err, int separate = 0, const Real *Ac = nullptr,
                                                   const Real *Bc = nullptr, int64_t jc = 0, int64_t nc = 0,
                                                   Real wmul = (Real)1, const LaneStage<Real> &stg = LaneStage<Real>())
{
    constexpr int C = 1 << D, S = Dims<D>::S;
    int64_t i = 0;
    Real h[5] = {0, 0, 0, 0, 0};
    Real ax = 0, ay = 0, bx = 0, by = 0, acen = 0;
    if (active)
    {
        // node indices in 32 bits (every supported grid has < 2^32 nodes); signed strides of the
        // element mirrored so that the node is its corner 0
        int st[D], sd[D];
        st[D - 1] = 1;
#pragma unroll
        for (int d = D - 2; d >= 0; d--) st[d] = st[d + 1] * (g.r + 1);
        // strides of the staged tile (3 x 3 x SW), compile-time constants
        constexpr int tst[3] = {3 * SW, SW, 1};
        uint32_t iu = 0;
        bool ok = true;
#pragma unroll
        for (int d = 0; d < D; d++)
        {
            iu += (uint32_t)I[d] * (uint32_t)st[d];
            sd[d] = cbit<D>(A, d) ? -st[d] : st[d];
            int e = I[d] - cbit<D>(A, d);
            ok = ok && e >= 0 && e < g.r;
        }
        i = iu;
        if (ok)
        {
            if constexpr (std::is_same<Real, float>::value && Packed)
            {
                // the (x, y) corner pairs as loaded, on the two-wide FP32 instructions
                float2 c2[C];
#pragma unroll
                for (int cc = 0; cc < C; cc++)
                {
                    if constexpr (Staged)
                    {
                        int tj = stg.tcentre;
#pragma unroll
                        for (int d = 0; d < 3; d++)
                            if (cbit<3>(cc, d)) tj += cbit<3>(A, d) ? -tst[d] : tst[d];
                        c2[cc] = stg.tile[tj];
                    }
                    else
                    {
                        int jj = (int)iu;
#pragma unroll
                        for (int d = 0; d < D; d++)
                            if (cbit<D>(cc, d)) jj += sd[d];
                        c2[cc] = ld2(xy, (int64_t)(uint32_t)jj);
                    }
                }
                element_fit_packed<D>(c2, h);
            }
            else
            {
                Real x[C], y[C];
#pragma unroll
                for (int cc = 0; cc < C; cc++)
                {
                    Real2<Real> v;
                    if constexpr (Staged)
                    {
                        int tj = stg.tcentre;
#pragma unroll
                        for (int d = 0; d < 3; d++)
                            if (cbit<3>(cc, d)) tj += cbit<3>(A, d) ? -tst[d] : tst[d];
                        v = stg.tile[tj];
                    }
                    else
                    {
                        int jj = (int)iu;
#pragma unroll
                        for (int d = 0; d < D; d++)
                            if (cbit<D>(cc, d)) jj += sd[d];
                        v = ld2(xy, (int64_t)(uint32_t)jj);
                    }
                    x[cc] = v.x;
                    y[cc] = v.y;
                }
                element_fit<D, Real>(x, y, 0, h);
            }
        }
        for (int o = A; o < S; o += C)
        {
            int off[D];
            stencil_offset<D>(o, off);
            bool in = true;
            int jj = (int)iu;
#pragma unroll
            for (int d = 0; d < D; d++)
            {
                int t = I[d] + off[d];
                in = in && (t >= 0) && (t <= g.r);
                jj += off[d] * st[d];
            }
            if (!in) continue;
            Real a, b;
            if constexpr (Staged)
            {
                a = stg.As[o * stg.npb + stg.t];
                b = stg.Bs[o * stg.npb + stg.t];
            }
            else if (Ac)
            {
                a = Ac[(int64_t)o * nc + jc];
                b = Bc[(int64_t)o * nc + jc];
            }
            else
            {
                a = L.A[(int64_t)o * L.N + i];
                b = L.B[(int64_t)o * L.N + i];
            }
            Real2<Real> v;
            if constexpr (Staged) v = stg.tile[stg.tcentre + off[0] * tst[0] + off[1] * tst[1] + off[2] * tst[2]];
            else v = ld2(xy, (int64_t)(uint32_t)jj);
            ax += a * v.x;
            ay += a * v.y;
            if (o == Dims<D>::CENTER) acen = a;
            else { bx += b * v.x; by += b * v.y; }
        }
    }
#pragma unroll
    for (int k = 0; k < 5; k++) h[k] = group_sum<D>(h[k]);
    ax = group_sum<D>(ax); ay = group_sum<D>(ay); bx = group_sum<D>(bx); by = group_sum<D>(by); acen = group_sum<D>(acen);
    if (!active || A != 0) return;
    const Real sc = (Real)wedge_scale<D>(g.r) * wmul;
    Real q[5];
    q[0] = h[0] * sc + acen;
    q[1] = h[1] * sc + acen;
    q[2] = (Real)2 * h[2] * sc;
    q[3] = (Real)2 * h[3] * sc + (Real)2 * ax - (Real)2 * by;
    q[4] = (Real)2 * h[4] * sc + (Real)2 * ay + (Real)2 * bx;
    Real p0, p1;
    if (relaxed(L, i) && node_step<Real>(q, separate, p0, p1))
    {
        Real2<Real> v = ld2(xy, i);
        v.x += p0;
        v.y += p1;
        if (!isfinite((double)v.x) || !isfinite((double)v.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
        reinterpret_cast<Real2<Real> *>(xy)[i] = v;
    }
}

// Warp-per-node variant for the coarsest 3D levels, where a colour has at most a few dozen nodes
// and the update latency (not throughput) sets the pace: lane 3 A + K (A < 8, K < 3) integrates
// component K of element A alone, lanes 24-31 take the stencil column.  Every (A, K) pair runs the
// same code: the element is mirrored so that the node is its corner 0 and its axes are permuted so
// that component K's axes (P, Q) and the remaining axis become component 0's (1, 0) and 2; the
// integrals are invariant under both maps (each term carries one P- and one Q-derivative).

template <typename Real>
__device__ __forceinline__ void gs_update_warp3(const LevelPtrs<Real> &L, Real *xy, const Grid<3> &g, const int *I, bool active,
                                                unsigned int *err, int separate, Real wmul = (Real)1)
{
    constexpr int S = 27;
    const int lane = threadIdx.x & 31;
    // v[0..4]: wedge integrals h0..h4 on lanes 0-23; stencil sums ax, ay, bx, by, acen on lanes 24-31
    Real v[5] = {0, 0, 0, 0, 0};
    const int s1 = g.r + 1, s0 = s1 * s1;
    const int i = I[0] * s0 + I[1] * s1 + I[2];
    if (active)
    {
        const int st[3] = {s0, s1, 1};
        if (lane < 24)
        {
            const int A = lane / 3, K = lane - 3 * (lane / 3);
            // physical axis of canonical axes 0, 1, 2 (= Q, P, R of component K)
            const int pax[3] = {(K == 2) ? 1 : 0, (K == 0) ? 1 : 2, (K == 0) ? 2 : (K == 1 ? 1 : 0)};
            bool ok = true;
#pragma unroll
            for (int d = 0; d < 3; d++)
            {
                int e = I[d] - cbit<3>(A, d);
                ok = ok && e >= 0 && e < g.r;
            }
            if (ok)
            {
                int sd[3];
#pragma unroll
                for (int a = 0; a < 3; a++) sd[a] = cbit<3>(A, pax[a]) ? -st[pax[a]] : st[pax[a]];
                Real x[8], y[8];
#pragma unroll
                for (int cc = 0; cc < 8; cc++)
                {
                    int jj = i;
#pragma unroll
                    for (int a = 0; a < 3; a++)
                        if (cbit<3>(cc, a)) jj += sd[a];
                    Real2<Real> p = ld2(xy, jj);
                    x[cc] = p.x;
                    y[cc] = p.y;
                }
                component_fit<3, 0, Real>(x, y, 0, v);
            }
        }
        else
        {
            for (int o = lane - 24; o < S; o += 8)
            {
                const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
                bool in = true;
#pragma unroll
                for (int d = 0; d < 3; d++) { int t = I[d] + off[d]; in = in && t >= 0 && t <= g.r; }
                if (!in) continue;
                const int jj = i + off[0] * s0 + off[1] * s1 + off[2];
                Real a = L.A[(int64_t)o * L.N + i];
                Real b = L.B[(int64_t)o * L.N + i];
                Real2<Real> p = ld2(xy, jj);
                v[0] += a * p.x;
                v[1] += a * p.y;
                if (o == 13) v[4] = a;
                else { v[2] += b * p.x; v[3] += b * p.y; }
            }
        }
    }
    // sums within the four 8-lane groups (the wedge groups 0-2 and the stencil group 3), then lane 0
    // adds the three wedge groups in order and takes the stencil group's sums
#pragma unroll
    for (int k = 0; k < 5; k++)
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) v[k] += shfl_xor_any(v[k], o);
    Real h[5], st5[5];
#pragma unroll
    for (int k = 0; k < 5; k++)
    {
        const Real g1 = shfl_any(v[k], 8), g2 = shfl_any(v[k], 16);
        st5[k] = shfl_any(v[k], 24);
        h[k] = (v[k] + g1) + g2;
    }
    if (!active || lane != 0) return;
    const Real ax = st5[0], ay = st5[1], bx = st5[2], by = st5[3], acen = st5[4];
    const Real sc = (Real)wedge_scale<3>(g.r) * wmul;
    Real q[5];
    q[0] = h[0] * sc + acen;
    q[1] = h[1] * sc + acen;
    q[2] = (Real)2 * h[2] * sc;
    q[3] = (Real)2 * h[3] * sc + (Real)2 * ax - (Real)2 * by;
    q[4] = (Real)2 * h[4] * sc + (Real)2 * ay + (Real)2 * bx;
    Real p0, p1;
    if (relaxed(L, i) && node_step<Real>(q, separate, p0, p1))
    {
        Real2<Real> cur = ld2(xy, i);
        cur.x += p0;
        cur.y += p1;
        if (!isfinite((double)cur.x) || !isfinite((double)cur.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
        reinterpret_cast<Real2<Real> *>(xy)[i] = cur;
    }
}

// Point-split variant for the latency-bound small 3D levels: 128 threads per node.  Thread
// u < 96 takes the Gauss points with (gp, gq) = (u & 3) >> 1, u & 1 of component K of element A,
// 3 A + K = u >> 2 (canonical orientation and axis permutation as above), so that the work of the
// existing elements is packed into as few warps as possible (the FP64 pipe is charged per warp
// instruction, whatever the number of active lanes); threads 96-122 take one stencil offset each.
// Each warp sums its lanes, the node's four warps meet in shared memory (part: 4 x 5 values per
// node: warps 0-2 the wedge integrals, warp 3 the stencil sums) and the node's first thread adds
// them in a fixed order and applies the step.  Every thread of the block must call this (block
// barriers).
template <typename Real>
__device__ __forceinline__ void gs_update_split3(const LevelPtrs<Real> &L, Real *xy, const Grid<3> &g, const int *I, bool active,
                                                 unsigned int *err, int separate, const Real *Ac, const Real *Bc, int64_t jc,
                                                 int64_t nc, Real (*part)[5], Real wmul = (Real)1)
{
    const int t = threadIdx.x & 127, wp = t >> 5, lane = t & 31;
    Real v[5] = {0, 0, 0, 0, 0};
    const int s1 = g.r + 1, s0 = s1 * s1;
    const int i = I[0] * s0 + I[1] * s1 + I[2];
    if (active)
    {
        const int st[3] = {s0, s1, 1};
        if (t < 96)
        {
            const int ak = t >> 2, pq = t & 3;
            const int A = ak / 3, K = ak - 3 * (ak / 3);
            const int pax[3] = {(K == 2) ? 1 : 0, (K == 0) ? 1 : 2, (K == 0) ? 2 : (K == 1 ? 1 : 0)};
            bool ok = true;
#pragma unroll
            for (int d = 0; d < 3; d++)
            {
                int e = I[d] - cbit<3>(A, d);
                ok = ok && e >= 0 && e < g.r;
            }
            if (ok)
            {
                int sd[3];
#pragma unroll
                for (int a = 0; a < 3; a++) sd[a] = cbit<3>(A, pax[a]) ? -st[pax[a]] : st[pax[a]];
                Real x[8], y[8];
#pragma unroll
                for (int cc = 0; cc < 8; cc++)
                {
                    int jj = i;
#pragma unroll
                    for (int a = 0; a < 3; a++)
                        if (cbit<3>(cc, a)) jj += sd[a];
                    Real2<Real> q = ld2(xy, jj);
                    x[cc] = q.x;
                    y[cc] = q.y;
                }
                component_fit_pq3<Real>(x, y, pq >> 1, pq & 1, v);
            }
        }
        else if (t < 96 + 27)
        {
            const int o = t - 96;
            const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
            bool in = true;
#pragma unroll
            for (int d = 0; d < 3; d++) { int q = I[d] + off[d]; in = in && q >= 0 && q <= g.r; }
            if (in)
            {
                const int jj = i + off[0] * s0 + off[1] * s1 + off[2];
                const Real a = Ac ? Ac[(int64_t)o * nc + jc] : L.A[(int64_t)o * L.N + i];
                const Real b = Bc ? Bc[(int64_t)o * nc + jc] : L.B[(int64_t)o * L.N + i];
                const Real2<Real> q = ld2(xy, jj);
                v[0] = a * q.x;
                v[1] = a * q.y;
                if (o == 13) v[4] = a;
                else { v[2] = b * q.x; v[3] = b * q.y; }
            }
        }
    }
    // warp sums, the rounds rolled (small code for the instruction cache; the same additions)
#pragma unroll 1
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 5; k++) v[k] += shfl_xor_any(v[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 5; k++) part[wp][k] = v[k];
    __syncthreads();
    if (active && t == 0)
    {
        Real h[5];
#pragma unroll
        for (int k = 0; k < 5; k++) h[k] = (part[0][k] + part[1][k]) + part[2][k];
        const Real ax = part[3][0], ay = part[3][1], bx = part[3][2], by = part[3][3], acen = part[3][4];
        const Real sc = (Real)wedge_scale<3>(g.r) * wmul;
        Real q[5];
        q[0] = h[0] * sc + acen;
        q[1] = h[1] * sc + acen;
        q[2] = (Real)2 * h[2] * sc;
        q[3] = (Real)2 * h[3] * sc + (Real)2 * ax - (Real)2 * by;
        q[4] = (Real)2 * h[4] * sc + (Real)2 * ay + (Real)2 * bx;
        Real p0, p1;
        // double-float levels test and divide in pair arithmetic (no FP64 conversions, one
        // division); float and FP64 levels keep the two-division form of the other kernels
        constexpr bool pair = std::is_same<Real, df>::value;
        if (relaxed(L, i) && (pair ? node_step_tiny<Real>(q, separate, p0, p1) : node_step<Real>(q, separate, p0, p1)))
        {
            Real2<Real> cur = ld2(xy, i);
            cur.x += p0;
            cur.y += p1;
            if (!finite_value<Real>(cur.x) || !finite_value<Real>(cur.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
            reinterpret_cast<Real2<Real> *>(xy)[i] = cur;
        }
    }
    __syncthreads();
}

// one colour of a small 3D level, point-split: 128 threads per node, kSplitNodes nodes per block;
// used for colours of at most kSplitMaxColourNodes nodes (3D levels up to 3), whose launches are
// latency-bound
constexpr int kSplitNodes = 2;
constexpr int64_t kSplitMaxColourNodes = 125;
// NPB nodes per block (block = 128 NPB threads); the block shape does not change any node's arithmetic
template <typename Real, int NPB>
__device__ __forceinline__ void gs_split3_body(const LevelPtrs<Real> &L, const Colour<3> &col, int64_t cbBase, unsigned int *err,
                                               int separate, const int *kexp, int block)
{
    __shared__ Real part[NPB][4][5];
    const Real wmul = wedge_mult<Real>(kexp, L.level);
    Grid<3> g(L.level);
    const int64_t j = (int64_t)block * NPB + (threadIdx.x >> 7);
    const bool active = j < col.n;
    int I[3] = {0, 0, 0};
    if (active) col.node(j, I);
    const Real *Ac = L.Acb ? L.Acb + cbBase : nullptr, *Bc = L.Bcb ? L.Bcb + cbBase : nullptr;
    gs_update_split3<Real>(L, L.xy, g, I, active, err, separate, Ac, Bc, j, col.n, part[threadIdx.x >> 7], wmul);
}
template <typename Real>
__global__ void __launch_bounds__(128 * kSplitNodes) gs_colour_split3_kernel(LevelPtrs<Real> L, Colour<3> col, int64_t cbBase,
                                                                              unsigned int *err, int separate,
                                                                              const int *kexp = nullptr)
{
    gs_split3_body<Real, kSplitNodes>(L, col, cbBase, err, separate, kexp, blockIdx.x);
}
// the same colour of every reconstruction of a lockstep batch: grid.y = reconstruction
template <typename Real, int NPB>
__global__ void __launch_bounds__(128 * NPB) gs_colour_split3_batch_kernel(const BatchJob<Real> *jobs, Colour<3> col, int64_t cbBase)
{
    const BatchJob<Real> &b = jobs[blockIdx.y];
    gs_split3_body<Real, NPB>(b.L, col, cbBase, b.err, b.separate, b.kexp, blockIdx.x);
}

template <int D, typename Real>
__device__ __forceinline__ void gs_update_lanes(const LevelPtrs<Real> &L, const Grid<D> &g, const Colour<D> &col, int64_t j,
                                                bool active, int A, unsigned int *err)
{
    int I[D];
    if (active) col.node(j, I);
    else
        for (int d = 0; d < D; d++) I[d] = 0;
    gs_update_lanes_at<D, Real>(L, L.xy, g, I, active, A, err);
}

// Launch geometry without 64-bit index division: block = (128 >> D) nodes along the last axis
// times 2^D lanes; grid.y = the colour's count on axis D-2; grid.z = the counts on the remaining
// leading axes.
// 3D float: cap registers at 48 (10 resident blocks, 40 warps per SM instead of 32 at 64 registers)
template <int D, typename Real>
constexpr int lanes_min_blocks() { return (D == 3 && sizeof(Real) == 4) ? 10 : 1; }

template <int D, typename Real, bool Packed, int TPB, bool Stage = false>
__device__ __forceinline__ void gs_lanes_body(const LevelPtrs<Real> &L, const Colour<D> &col, int64_t cbBase, unsigned int *err,
                                              int separate, int bx, int by, int bz)
{
    Grid<D> g(L.level);
    constexpr int NPB = TPB >> D;
    const int A = threadIdx.x & ((1 << D) - 1);
    const int tl = bx * NPB + (threadIdx.x >> D);
    int I[D];
    I[D - 1] = 2 * tl + col.par[D - 1];
    I[D - 2] = 2 * by + col.par[D - 2];
    if constexpr (D == 3) I[0] = 2 * bz + col.par[0];
    else
    {
        I[1] = 2 * (bz % col.cnt[1]) + col.par[1];
        I[0] = 2 * (bz / col.cnt[1]) + col.par[0];
    }
    // index of the node in the colour (axis 0 slowest)
    const int64_t jc = ((int64_t)bz * col.cnt[D - 2] + by) * col.cnt[D - 1] + tl;
    const Real *Ac = L.Acb ? L.Acb + cbBase : nullptr, *Bc = L.Bcb ? L.Bcb + cbBase : nullptr;
    if constexpr (D == 3 && Stage)
        if (Ac)
        {
            // stage the row's 3 x 3 x W neighbourhood and its nodes' stencil columns (every thread of
            // the block takes part; Ac is the same for the whole block)
            constexpr int W = 2 * NPB + 1, S = Dims<3>::S;
            __shared__ Real2<Real> tile[9 * W];
            __shared__ Real As[S * NPB], Bs[S * NPB];
            const int x0 = 2 * bx * NPB + col.par[2] - 1, y0 = I[1] - 1, z0 = I[0] - 1;
            for (int k = threadIdx.x; k < 9 * W; k += TPB)
            {
                const int lz = k / (3 * W), ly = (k / W) % 3, lx = k % W;
                const int gz = z0 + lz, gy = y0 + ly, gx = x0 + lx;
                if (gz >= 0 && gz <= g.r && gy >= 0 && gy <= g.r && gx >= 0 && gx <= g.r)
                    tile[k] = ld2(L.xy, ((int64_t)gz * (g.r + 1) + gy) * (g.r + 1) + gx);
            }
            const int nrow = min(NPB, col.cnt[2] - bx * NPB);  // the block's nodes in the colour
            const int64_t jc0 = ((int64_t)bz * col.cnt[1] + by) * col.cnt[2] + (int64_t)bx * NPB;
            for (int k = threadIdx.x; k < S * NPB; k += TPB)
            {
                const int o = k / NPB, t = k - o * NPB;
                if (t < nrow)
                {
                    As[k] = Ac[(int64_t)o * col.n + jc0 + t];
                    Bs[k] = Bc[(int64_t)o * col.n + jc0 + t];
                }
            }
            __syncthreads();
            LaneStage<Real> stg;
            stg.tile = tile;
            stg.t = tl - bx * NPB;
            stg.tcentre = 4 * W + 2 * stg.t + 1;
            stg.As = As;
            stg.Bs = Bs;
            stg.npb = NPB;
            gs_update_lanes_at<D, Real, Packed, true, W>(L, L.xy, g, I, tl < col.cnt[D - 1], A, err, separate, Ac, Bc, jc,
                                                        col.n, (Real)1, stg);
            return;
        }
    gs_update_lanes_at<D, Real, Packed>(L, L.xy, g, I, tl < col.cnt[D - 1], A, err, separate, Ac, Bc, jc, col.n);
}

template <int D, typename Real, int MinBlocks = lanes_min_blocks<D, Real>(), bool Packed = false, bool Stage = false>
__global__ void __launch_bounds__(kThreads, MinBlocks) gs_colour_lanes_kernel(LevelPtrs<Real> L, Colour<D> col,
                                                                              int64_t cbBase, unsigned int *err,
                                                                              int separate)
{
    gs_lanes_body<D, Real, Packed, kThreads, Stage>(L, col, cbBase, err, separate, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One colour of an adaptive level: the colour's active nodes from its list (colour-local indices),
// 2^Dim lanes per node as gs_colour_lanes_kernel, each node's update computed the same way
template <int D, typename Real, int MinBlocks = lanes_min_blocks<D, Real>(), bool Packed = false>
__global__ void __launch_bounds__(kThreads, MinBlocks) gs_colour_lanes_list_kernel(LevelPtrs<Real> L, Colour<D> col,
                                                                                   int64_t cbBase, const int *list, int count,
                                                                                   unsigned int *err, int separate)
{
    constexpr int NPB = kThreads >> D;
    Grid<D> g(L.level);
    const int A = threadIdx.x & ((1 << D) - 1);
    const int k = blockIdx.x * NPB + (threadIdx.x >> D);
    const bool active = k < count;
    const int64_t jc = active ? list[k] : 0;
    int I[D];
    col.node(jc, I);
    const Real *Ac = L.Acb ? L.Acb + cbBase : nullptr, *Bc = L.Bcb ? L.Bcb + cbBase : nullptr;
    gs_update_lanes_at<D, Real, Packed>(L, L.xy, g, I, active, A, err, separate, Ac, Bc, jc, col.n);
}

// the same colour of every reconstruction of a lockstep batch (3D): block = TPB threads (TPB / 8
// nodes along the last axis), grid.z = reconstruction x the colour's count on axis 0
template <typename Real, int TPB, int MinBlocks, bool Packed>
__global__ void __launch_bounds__(TPB, MinBlocks) gs_colour_lanes_batch_kernel(const BatchJob<Real> *jobs, Colour<3> col,
                                                                               int64_t cbBase)
{
    const int m = blockIdx.z / col.cnt[0], bz = blockIdx.z - m * col.cnt[0];
    const BatchJob<Real> &b = jobs[m];
    gs_lanes_body<3, Real, Packed, TPB>(b.L, col, cbBase, b.err, b.separate, blockIdx.x, blockIdx.y, bz);
}

// Flat variant: consecutive groups of 2^D threads take consecutive nodes of the colour (32-bit
// decomposition), so no block row is left partly empty.
template <int D, typename Real>
__global__ void __launch_bounds__(kThreads) gs_colour_flat_kernel(LevelPtrs<Real> L, Colour<D> col, unsigned int *err, int separate)
{
    Grid<D> g(L.level);
    const int A = threadIdx.x & ((1 << D) - 1);
    const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> D;
    const bool active = j < col.n;
    int I[D];
    if (active) col.node(j, I);
    else
        for (int d = 0; d < D; d++) I[d] = 0;
    gs_update_lanes_at<D, Real>(L, L.xy, g, I, active, A, err, separate);
}

// All sweeps of a small level in one thread block: the colours follow each other behind a block
// barrier, which also makes each colour's writes visible to the next.  Used for the coarse levels
// of the cascadic schedule, whose thousands of tiny sweeps would otherwise be bound by launch
// latency.  The level's coefficients, and its stencils when they fit, live in shared memory for the
// whole schedule.  The block holds up to MaxThreads threads (1024 where the lane update fits in 64
// registers: 3D float) so that a colour takes as few passes as possible.
template <int D, typename Real>
constexpr int persistent_threads() { return (D == 3 && sizeof(Real) == 4) ? 1024 : 256; }
template <int D, typename Real, bool SmemStencil, int MaxThreads, int Mode>
__global__ void __launch_bounds__(MaxThreads) gs_level_kernel(LevelPtrs<Real> L, int iters, unsigned int *err, int separate,
                                                              int *kexp = nullptr)
{
    Grid<D> g(L.level);
    constexpr int S = Dims<D>::S;
    constexpr bool kDF = std::is_same<Real, df>::value;
    Real wmul = wedge_mult<Real>(kexp, L.level);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *xy = reinterpret_cast<Real *>(smem_raw);
    for (int64_t k = threadIdx.x; k < 2 * g.N; k += blockDim.x) xy[k] = L.xy[k];
    LevelPtrs<Real> Ls = L;
    if constexpr (SmemStencil)
    {
        Real *A = xy + 2 * g.N, *B = A + S * g.N;
        for (int64_t k = threadIdx.x; k < S * g.N; k += blockDim.x) { A[k] = L.A[k]; B[k] = L.B[k]; }
        Ls.A = A;
        Ls.B = B;
    }
    __syncthreads();
    for (int it = 0; it < iters; it++)
    {
        for (int c = 0; c < (1 << D); c++)
        {
            Colour<D> col(g, c);
            if constexpr (Mode == 2 && D == 3)
            {
                // 128 threads per node, the block holds every node of the largest colour
                __shared__ Real part[8][4][5];
                const int64_t j = threadIdx.x >> 7;
                const bool active = j < col.n;
                int I[3] = {0, 0, 0};
                if (active) col.node(j, I);
                gs_update_split3<Real>(Ls, xy, g, I, active, err, separate, nullptr, nullptr, 0, 0, part[threadIdx.x >> 7], wmul);
            }
            else if constexpr (Mode == 1 && D == 3)
            {
                // one warp per node; the block holds a warp for every node of the largest colour
                const int64_t j = threadIdx.x >> 5;
                const bool active = j < col.n;
                int I[3] = {0, 0, 0};
                if (active) col.node(j, I);
                gs_update_warp3<Real>(Ls, xy, g, I, active, err, separate, wmul);
            }
            else
            {
                const int per = blockDim.x >> D;  // nodes per pass of the block
                const int A = threadIdx.x & ((1 << D) - 1);
                for (int64_t j0 = 0; j0 < col.n; j0 += per)
                {
                    int64_t j = j0 + (threadIdx.x >> D);
                    bool active = j < col.n;
                    int I[D];
                    if (active) col.node(j, I);
                    else
                        for (int d = 0; d < D; d++) I[d] = 0;
                    gs_update_lanes_at<D, Real>(Ls, xy, g, I, active, A, err, separate, nullptr, nullptr, 0, 0, wmul);
                }
            }
            __syncthreads();
        }
        if constexpr (kDF)
            if (kexp)
            {
                // keep the stored coefficients near 1: a new power-of-two exponent after every sweep
                const int shift = df_rescale_shift(xy, 2 * g.N);
                if (shift)
                {
                    for (int64_t k = threadIdx.x; k < 2 * g.N; k += blockDim.x) xy[k] = ldexp_df(xy[k], shift);
                    if (threadIdx.x == 0) kexp[L.level] -= shift;
                    __syncthreads();
                    wmul = wedge_mult<Real>(kexp, L.level);
                }
            }
    }
    for (int64_t k = threadIdx.x; k < 2 * g.N; k += blockDim.x) L.xy[k] = xy[k];
}


// ---------------------------------------------------------------------------------------------
// The two coarsest 3D levels (resolution 1 and 2: 8 and 27 nodes), all sweeps in one block with
// one warp per (node, element) incidence of a colour.  Every colour of these levels has the same
// number of incidences (resolution 1: one node with its one element; resolution 2: eight, e.g. the
// eight corner nodes with one element each, or the centre node with all eight), so warp w owns the
// w-th incidence of every colour (nodes in colour order, elements in corner order).  Lanes 0-11
// integrate the element's wedge component K = lane / 4 at the Gauss-point pair lane % 4 in the
// canonical orientation (as gs_update_split3); lanes 16-31 take the node's stencil column (offsets
// lane - 16 and lane) in the node's first incidence; each half-warp sums with shuffles.  At
// resolution 1 the single warp applies the step itself (no block barrier at all); at resolution 2
// the warps of a node meet in shared memory, two barriers per colour.  The coefficients and both
// stencils live in shared memory for the whole schedule.  Double-float levels rescale their stored
// coefficients after every sweep as the other kernels do.
// ---------------------------------------------------------------------------------------------
template <typename Real, int LEVEL>
__device__ __forceinline__ void gs_tiny_body(const LevelPtrs<Real> &L, int iters, unsigned int *err, int separate, int *kexp)
{
    static_assert(LEVEL == 0 || LEVEL == 1, "resolution 1 or 2");
    constexpr int NW = LEVEL == 0 ? 1 : 8;  // incidences per colour
    constexpr int R = 1 << LEVEL, N1 = R + 1, NN = N1 * N1 * N1, S = 27;
    constexpr int s0 = N1 * N1, s1 = N1;
    constexpr bool kDF = std::is_same<Real, df>::value;
    __shared__ Real2<Real> xy[NN];
    __shared__ Real As[S * NN], Bs[S * NN];
    __shared__ Real part[NW][10];
    // each warp's incidence of each colour: node index, node coordinates, element corner A, whether
    // it is the node's first incidence and how many the node has (shared memory, so that the
    // colour loop indexes it without a local-memory stack)
    __shared__ int incNode[8][NW], incA[8][NW], incCnt[8][NW], incI[8][NW][3], incFirst[8][NW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < NN; k += blockDim.x) xy[k] = ld2(L.xy, k);
    for (int k = threadIdx.x; k < S * NN; k += blockDim.x)
    {
        As[k] = L.A[k];
        Bs[k] = L.B[k];
    }
    if (threadIdx.x < 8)
    {
        const int c = threadIdx.x;
        const Grid<3> g(LEVEL);
        const Colour<3> col(g, c);
        int w = 0;
        for (int j = 0; j < (int)col.n; j++)
        {
            int I[3];
            col.node(j, I);
            int cnt = 0;
            for (int A = 0; A < 8; A++)
            {
                bool ok = true;
                for (int d = 0; d < 3; d++) { const int e = I[d] - cbit<3>(A, d); ok = ok && e >= 0 && e < R; }
                if (ok) cnt++;
            }
            int k = 0;
            for (int A = 0; A < 8; A++)
            {
                bool ok = true;
                for (int d = 0; d < 3; d++) { const int e = I[d] - cbit<3>(A, d); ok = ok && e >= 0 && e < R; }
                if (!ok || w >= NW) continue;
                incNode[c][w] = (I[0] * N1 + I[1]) * N1 + I[2];
                incA[c][w] = A;
                incFirst[c][w] = k == 0;
                incCnt[c][w] = cnt;
                for (int d = 0; d < 3; d++) incI[c][w][d] = I[d];
                w++;
                k++;
            }
        }
    }
    __syncthreads();
    Real wmul = wedge_mult<Real>(kexp, LEVEL);
    for (int it = 0; it < iters; it++)
    {
#pragma unroll 1
        for (int c = 0; c < 8; c++)
        {
            const int i = incNode[c][warp], A = incA[c][warp];
            const bool first = incFirst[c][warp] != 0;
            Real r[5] = {0, 0, 0, 0, 0};
            if (lane < 12)
            {
                const int K = lane >> 2, pq = lane & 3;
                const int pax[3] = {(K == 2) ? 1 : 0, (K == 0) ? 1 : 2, (K == 0) ? 2 : (K == 1 ? 1 : 0)};
                int sd[3];
#pragma unroll
                for (int a = 0; a < 3; a++)
                {
                    const int stride = pax[a] == 0 ? s0 : (pax[a] == 1 ? s1 : 1);
                    sd[a] = ((A >> (2 - pax[a])) & 1) ? -stride : stride;
                }
                Real x[8], y[8];
#pragma unroll
                for (int cc = 0; cc < 8; cc++)
                {
                    int jj = i;
#pragma unroll
                    for (int a = 0; a < 3; a++)
                        if (cbit<3>(cc, a)) jj += sd[a];
                    const Real2<Real> v = xy[jj];
                    x[cc] = v.x;
                    y[cc] = v.y;
                }
                component_fit_pq3<Real>(x, y, pq >> 1, pq & 1, r);
            }
            else if (lane >= 16 && first)
            {
#pragma unroll
                for (int half = 0; half < 2; half++)
                {
                    const int o = lane - 16 + 16 * half;
                    if (o >= S) continue;
                    const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
                    bool in = true;
#pragma unroll
                    for (int d = 0; d < 3; d++) { const int q = incI[c][warp][d] + off[d]; in = in && q >= 0 && q <= R; }
                    if (!in) continue;
                    const int jj = i + off[0] * s0 + off[1] * s1 + off[2];
                    const Real a = As[o * NN + i], b = Bs[o * NN + i];
                    const Real2<Real> q = xy[jj];
                    r[0] += a * q.x;
                    r[1] += a * q.y;
                    if (o == 13) r[4] = a;
                    else { r[2] += b * q.x; r[3] += b * q.y; }
                }
            }
            // sums within each half-warp: lane 0 the wedge integrals, lane 16 the stencil sums (in
            // double-float at resolution 1 the rounds stay rolled: with one warp, instruction fetch
            // is the bound, and the pair additions' code then fits the instruction cache)
            if constexpr (kDF && LEVEL == 0)
            {
#pragma unroll 1
                for (int o = 8; o > 0; o >>= 1)
#pragma unroll
                    for (int k = 0; k < 5; k++) r[k] += shfl_xor_any(r[k], o);
            }
            else
            {
#pragma unroll
                for (int o = 8; o > 0; o >>= 1)
#pragma unroll
                    for (int k = 0; k < 5; k++) r[k] += shfl_xor_any(r[k], o);
            }
            Real stc[5];
#pragma unroll
            for (int k = 0; k < 5; k++) stc[k] = shfl_any(r[k], 16);
            bool apply = false;
            Real h[5], sv[5];
            if (NW == 1)
            {
                apply = lane == 0;
#pragma unroll
                for (int k = 0; k < 5; k++) { h[k] = r[k]; sv[k] = stc[k]; }
            }
            else
            {
                if (lane == 0)
#pragma unroll
                    for (int k = 0; k < 5; k++) { part[warp][k] = r[k]; part[warp][5 + k] = stc[k]; }
                __syncthreads();
                apply = lane == 0 && first;
                if (apply)
                {
#pragma unroll
                    for (int k = 0; k < 5; k++)
                    {
                        h[k] = part[warp][k];
                        sv[k] = part[warp][5 + k];
                    }
                    for (int w2 = 1; w2 < incCnt[c][warp]; w2++)
#pragma unroll
                        for (int k = 0; k < 5; k++) h[k] += part[warp + w2][k];
                }
            }
            if (apply)
            {
                const Real sc = (Real)wedge_scale<3>(R) * wmul;
                Real q[5];
                q[0] = h[0] * sc + sv[4];
                q[1] = h[1] * sc + sv[4];
                q[2] = (Real)2 * h[2] * sc;
                q[3] = (Real)2 * h[3] * sc + (Real)2 * sv[0] - (Real)2 * sv[3];
                q[4] = (Real)2 * h[4] * sc + (Real)2 * sv[1] + (Real)2 * sv[2];
                Real p0, p1;
                if (relaxed(L, i) && node_step_tiny<Real>(q, separate, p0, p1))
                {
                    Real2<Real> cur = xy[i];
                    cur.x += p0;
                    cur.y += p1;
                    if (!finite_value<Real>(cur.x) || !finite_value<Real>(cur.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
                    xy[i] = cur;
                }
            }
            if (NW == 1) __syncwarp();
            else __syncthreads();
        }
        if constexpr (kDF)
            if (kexp)
            {
                // keep the stored coefficients near 1: a new power-of-two exponent after every sweep
                const int shift = df_rescale_shift(reinterpret_cast<const df *>(xy), 2 * NN);
                if (shift)
                {
                    df *v = reinterpret_cast<df *>(xy);
                    for (int k = threadIdx.x; k < 2 * NN; k += blockDim.x) v[k] = ldexp_df(v[k], shift);
                    if (threadIdx.x == 0) kexp[LEVEL] -= shift;
                    __syncthreads();
                    wmul = wedge_mult<Real>(kexp, LEVEL);
                }
            }
    }
    for (int k = threadIdx.x; k < NN; k += blockDim.x) reinterpret_cast<Real2<Real> *>(L.xy)[k] = xy[k];
}

// Level 0 (resolution 1: 8 nodes, one element, one node per colour) with four warps instead of
// one: warp K < 3 integrates wedge component K of the node's element, lane = (Gauss-point pair,
// other-axis point) (12 lanes, one point each), warp 3 the node's stencil column (lane = offset);
// warp sums, one block barrier, thread 0 the node step.  A colour phase's dependent path is then one
// point's setup and terms instead of three, spread over the SM's four sub-partitions.
template <typename Real>
__device__ __forceinline__ void gs_tiny0_body(const LevelPtrs<Real> &L, int iters, unsigned int *err, int separate, int *kexp)
{
    constexpr int NN = 8, S = 27, s0 = 4, s1 = 2;
    constexpr bool kDF = std::is_same<Real, df>::value;
    __shared__ Real2<Real> xy[NN];
    __shared__ Real As[S * NN], Bs[S * NN];
    __shared__ Real part[4][5];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < NN; k += blockDim.x) xy[k] = ld2(L.xy, k);
    for (int k = threadIdx.x; k < S * NN; k += blockDim.x)
    {
        As[k] = L.A[k];
        Bs[k] = L.B[k];
    }
    __syncthreads();
    Real wmul = wedge_mult<Real>(kexp, 0);
    for (int it = 0; it < iters; it++)
    {
#pragma unroll 1
        for (int c = 0; c < 8; c++)
        {
            // the colour's node: coordinate d = parity bit d of the colour; the element's corner of
            // the node has the node's coordinates as its bits
            const int I0 = c & 1, I1 = (c >> 1) & 1, I2 = (c >> 2) & 1;
            const int i = (I0 * 2 + I1) * 2 + I2;
            const int A = (I0 << 2) | (I1 << 1) | I2;
            Real r[5] = {0, 0, 0, 0, 0};
            if (warp < 3 && lane < 12)
            {
                const int K = warp, pq = lane / 3, go = lane - 3 * (lane / 3);
                const int pax[3] = {(K == 2) ? 1 : 0, (K == 0) ? 1 : 2, (K == 0) ? 2 : (K == 1 ? 1 : 0)};
                int sd[3];
#pragma unroll
                for (int a = 0; a < 3; a++)
                {
                    const int stride = pax[a] == 0 ? s0 : (pax[a] == 1 ? s1 : 1);
                    sd[a] = ((A >> (2 - pax[a])) & 1) ? -stride : stride;
                }
                Real x[8], y[8];
#pragma unroll
                for (int cc = 0; cc < 8; cc++)
                {
                    int jj = i;
#pragma unroll
                    for (int a = 0; a < 3; a++)
                        if (cbit<3>(cc, a)) jj += sd[a];
                    const Real2<Real> v = xy[jj];
                    x[cc] = v.x;
                    y[cc] = v.y;
                }
                PairTables<Real> t;
                component_setup_pq3<Real>(x, y, pq >> 1, pq & 1, t);
                component_point_pq3<Real>(t, go, r);
            }
            else if (warp == 3 && lane < S)
            {
                const int o = lane;
                const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
                const int q0 = I0 + off[0], q1 = I1 + off[1], q2 = I2 + off[2];
                if (q0 >= 0 && q0 <= 1 && q1 >= 0 && q1 <= 1 && q2 >= 0 && q2 <= 1)
                {
                    const Real a = As[o * NN + i], b = Bs[o * NN + i];
                    const Real2<Real> q = xy[i + off[0] * s0 + off[1] * s1 + off[2]];
                    r[0] = a * q.x;
                    r[1] = a * q.y;
                    if (o == 13) r[4] = a;
                    else { r[2] = b * q.x; r[3] = b * q.y; }
                }
            }
            // warp sums (in double-float the rounds stay rolled: small code for the instruction cache)
            if constexpr (kDF)
            {
#pragma unroll 1
                for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                    for (int k = 0; k < 5; k++) r[k] += shfl_xor_any(r[k], o);
            }
            else
            {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                    for (int k = 0; k < 5; k++) r[k] += shfl_xor_any(r[k], o);
            }
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < 5; k++) part[warp][k] = r[k];
            __syncthreads();
            if (threadIdx.x == 0)
            {
                Real h[5], sv[5];
#pragma unroll
                for (int k = 0; k < 5; k++)
                {
                    h[k] = (part[0][k] + part[1][k]) + part[2][k];
                    sv[k] = part[3][k];
                }
                const Real sc = (Real)wedge_scale<3>(1) * wmul;
                Real q[5];
                q[0] = h[0] * sc + sv[4];
                q[1] = h[1] * sc + sv[4];
                q[2] = (Real)2 * h[2] * sc;
                q[3] = (Real)2 * h[3] * sc + (Real)2 * sv[0] - (Real)2 * sv[3];
                q[4] = (Real)2 * h[4] * sc + (Real)2 * sv[1] + (Real)2 * sv[2];
                Real p0, p1;
                if (relaxed(L, i) && node_step_tiny<Real>(q, separate, p0, p1))
                {
                    Real2<Real> cur = xy[i];
                    cur.x += p0;
                    cur.y += p1;
                    if (!finite_value<Real>(cur.x) || !finite_value<Real>(cur.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
                    xy[i] = cur;
                }
            }
            __syncthreads();
        }
        if constexpr (kDF)
            if (kexp)
            {
                // keep the stored coefficients near 1: a new power-of-two exponent after every sweep
                const int shift = df_rescale_shift(reinterpret_cast<const df *>(xy), 2 * NN);
                if (shift)
                {
                    df *v = reinterpret_cast<df *>(xy);
                    for (int k = threadIdx.x; k < 2 * NN; k += blockDim.x) v[k] = ldexp_df(v[k], shift);
                    if (threadIdx.x == 0) kexp[0] -= shift;
                    __syncthreads();
                    wmul = wedge_mult<Real>(kexp, 0);
                }
            }
    }
    for (int k = threadIdx.x; k < NN; k += blockDim.x) reinterpret_cast<Real2<Real> *>(L.xy)[k] = xy[k];
}

// Level 1 (resolution 2: 27 nodes, 8 node-element incidences per colour) on a cluster of two
// blocks of four warps, one warp per incidence, so that each SM sub-partition issues for one warp
// (in one block of eight warps two share each sub-partition and a colour phase takes both warps'
// instructions).  Each block keeps a replica of the level's coefficients in its shared memory; a
// warp writes its incidence's sums into both blocks, the node's owner (the warp of its first
// incidence) applies the step to both replicas, and two cluster barriers order each colour.  The
// arithmetic and its order are gs_tiny_body<Real, 1>'s, so the results are its bits.
template <typename Real>
__device__ __forceinline__ void gs_tiny1_cluster_body(const LevelPtrs<Real> &L, int iters, unsigned int *err, int separate, int *kexp)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    constexpr int NW = 8, R = 2, N1 = 3, NN = 27, S = 27, s0 = 9, s1 = 3;
    constexpr bool kDF = std::is_same<Real, df>::value;
    __shared__ Real2<Real> xy[NN];
    __shared__ Real As[S * NN], Bs[S * NN];
    __shared__ Real part[NW][10];
    __shared__ int incNode[8][NW], incA[8][NW], incCnt[8][NW], incI[8][NW][3], incFirst[8][NW];
    const unsigned rank = cluster.block_rank();
    const int warp = (int)rank * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;  // the incidence
    Real2<Real> *peerXY = cluster.map_shared_rank(xy, rank ^ 1u);
    Real *peerPart = cluster.map_shared_rank(&part[0][0], rank ^ 1u);
    for (int k = threadIdx.x; k < NN; k += blockDim.x) xy[k] = ld2(L.xy, k);
    for (int k = threadIdx.x; k < S * NN; k += blockDim.x)
    {
        As[k] = L.A[k];
        Bs[k] = L.B[k];
    }
    if (threadIdx.x < 8)
    {
        const int c = threadIdx.x;
        const Grid<3> g(1);
        const Colour<3> col(g, c);
        int w = 0;
        for (int j = 0; j < (int)col.n; j++)
        {
            int I[3];
            col.node(j, I);
            int cnt = 0;
            for (int A = 0; A < 8; A++)
            {
                bool ok = true;
                for (int d = 0; d < 3; d++) { const int e = I[d] - cbit<3>(A, d); ok = ok && e >= 0 && e < R; }
                if (ok) cnt++;
            }
            int k = 0;
            for (int A = 0; A < 8; A++)
            {
                bool ok = true;
                for (int d = 0; d < 3; d++) { const int e = I[d] - cbit<3>(A, d); ok = ok && e >= 0 && e < R; }
                if (!ok || w >= NW) continue;
                incNode[c][w] = (I[0] * N1 + I[1]) * N1 + I[2];
                incA[c][w] = A;
                incFirst[c][w] = k == 0;
                incCnt[c][w] = cnt;
                for (int d = 0; d < 3; d++) incI[c][w][d] = I[d];
                w++;
                k++;
            }
        }
    }
    cluster.sync();  // both replicas and tables ready before any remote write
    Real wmul = wedge_mult<Real>(kexp, 1);
    for (int it = 0; it < iters; it++)
    {
#pragma unroll 1
        for (int c = 0; c < 8; c++)
        {
            const int i = incNode[c][warp], A = incA[c][warp];
            const bool first = incFirst[c][warp] != 0;
            Real r[5] = {0, 0, 0, 0, 0};
            if (lane < 12)
            {
                const int K = lane >> 2, pq = lane & 3;
                const int pax[3] = {(K == 2) ? 1 : 0, (K == 0) ? 1 : 2, (K == 0) ? 2 : (K == 1 ? 1 : 0)};
                int sd[3];
#pragma unroll
                for (int a = 0; a < 3; a++)
                {
                    const int stride = pax[a] == 0 ? s0 : (pax[a] == 1 ? s1 : 1);
                    sd[a] = ((A >> (2 - pax[a])) & 1) ? -stride : stride;
                }
                Real x[8], y[8];
#pragma unroll
                for (int cc = 0; cc < 8; cc++)
                {
                    int jj = i;
#pragma unroll
                    for (int a = 0; a < 3; a++)
                        if (cbit<3>(cc, a)) jj += sd[a];
                    const Real2<Real> v = xy[jj];
                    x[cc] = v.x;
                    y[cc] = v.y;
                }
                component_fit_pq3<Real>(x, y, pq >> 1, pq & 1, r);
            }
            else if (lane >= 16 && first)
            {
#pragma unroll
                for (int half = 0; half < 2; half++)
                {
                    const int o = lane - 16 + 16 * half;
                    if (o >= S) continue;
                    const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
                    bool in = true;
#pragma unroll
                    for (int d = 0; d < 3; d++) { const int q = incI[c][warp][d] + off[d]; in = in && q >= 0 && q <= R; }
                    if (!in) continue;
                    const int jj = i + off[0] * s0 + off[1] * s1 + off[2];
                    const Real a = As[o * NN + i], b = Bs[o * NN + i];
                    const Real2<Real> q = xy[jj];
                    r[0] += a * q.x;
                    r[1] += a * q.y;
                    if (o == 13) r[4] = a;
                    else { r[2] += b * q.x; r[3] += b * q.y; }
                }
            }
#pragma unroll
            for (int o = 8; o > 0; o >>= 1)
#pragma unroll
                for (int k = 0; k < 5; k++) r[k] += shfl_xor_any(r[k], o);
            Real stc[5];
#pragma unroll
            for (int k = 0; k < 5; k++) stc[k] = shfl_any(r[k], 16);
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < 5; k++)
                {
                    part[warp][k] = r[k];
                    part[warp][5 + k] = stc[k];
                    peerPart[warp * 10 + k] = r[k];
                    peerPart[warp * 10 + 5 + k] = stc[k];
                }
            cluster.sync();  // every incidence's sums in both blocks
            if (lane == 0 && first)
            {
                Real h[5], sv[5];
#pragma unroll
                for (int k = 0; k < 5; k++)
                {
                    h[k] = part[warp][k];
                    sv[k] = part[warp][5 + k];
                }
                for (int w2 = 1; w2 < incCnt[c][warp]; w2++)
#pragma unroll
                    for (int k = 0; k < 5; k++) h[k] += part[warp + w2][k];
                const Real sc = (Real)wedge_scale<3>(R) * wmul;
                Real q[5];
                q[0] = h[0] * sc + sv[4];
                q[1] = h[1] * sc + sv[4];
                q[2] = (Real)2 * h[2] * sc;
                q[3] = (Real)2 * h[3] * sc + (Real)2 * sv[0] - (Real)2 * sv[3];
                q[4] = (Real)2 * h[4] * sc + (Real)2 * sv[1] + (Real)2 * sv[2];
                Real p0, p1;
                if (relaxed(L, i) && node_step_tiny<Real>(q, separate, p0, p1))
                {
                    Real2<Real> cur = xy[i];
                    cur.x += p0;
                    cur.y += p1;
                    if (!finite_value<Real>(cur.x) || !finite_value<Real>(cur.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
                    xy[i] = cur;
                    peerXY[i] = cur;
                }
            }
            cluster.sync();  // both replicas updated before the next colour reads them
        }
        if constexpr (kDF)
            if (kexp)
            {
                // both replicas hold the same values, so both blocks pick the same new exponent
                const int shift = df_rescale_shift(reinterpret_cast<const df *>(xy), 2 * NN);
                if (shift)
                {
                    df *v = reinterpret_cast<df *>(xy);
                    for (int k = threadIdx.x; k < 2 * NN; k += blockDim.x) v[k] = ldexp_df(v[k], shift);
                    if (rank == 0 && threadIdx.x == 0) kexp[1] -= shift;
                }
                // no remote write of the next sweep before the peer's rescale; the new exponent
                // (written by the first block) visible to both
                cluster.sync();
                if (shift) wmul = wedge_mult<Real>(kexp, 1);
            }
    }
    if (rank == 0)
        for (int k = threadIdx.x; k < NN; k += blockDim.x) reinterpret_cast<Real2<Real> *>(L.xy)[k] = xy[k];
    cluster.sync();  // no block leaves while its peer may still address its shared memory
}

template <typename Real>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(128) gs_tiny1_kernel(LevelPtrs<Real> L, int iters, unsigned int *err,
                                                                                int separate, int *kexp)
{
    gs_tiny1_cluster_body<Real>(L, iters, err, separate, kexp);
}

template <typename Real>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(128) gs_tiny1_batch_kernel(const BatchJob<Real> *jobs)
{
    const BatchJob<Real> &b = jobs[blockIdx.x >> 1];
    gs_tiny1_cluster_body<Real>(b.L, b.iters, b.err, b.separate, b.kexp);
}

// ---------------------------------------------------------------------------------------------
// 3D level 2 (resolution R = 4: 125 nodes) in double-float, all sweeps in one launch on a cluster
// of kClusterBlocks blocks of NWB warps.  Every block keeps a replica of the level's coefficients
// and stencils in shared memory.  Every element has exactly one corner in each parity colour, so a
// colour's (node, element) incidences are the level's R^3 = 64 elements, one per warp.  A colour
// phase: (1) lanes 0-11 of a warp integrate its element's wedge component x Gauss-point pair in the
// canonical orientation of the element's colour node (as gs_tiny1_kernel), lanes 16-31 the node's
// stencil column when the element is the node's designated one (the element on the lower side of
// the node on every axis where there is one), and lane 0 writes the element's ten sums into the
// block that owns the node (colour index mod the cluster size) through distributed shared memory;
// cluster barrier; (2) one thread of the owner block per node adds its elements' sums in a fixed
// order, takes the node step and writes the new pair into every replica; cluster barrier.  The
// replicas are rescaled after every sweep as the other double-float kernels do.  One launch
// replaces the level's 8 x 640 colour launches and their rescales at depth 8: 28.6 ms on 16 blocks
// (30.4 on 8) against 33.5 ms.  It is opt-in (EPR_CLUSTER_LEVELS=1): reconstructions solved
// concurrently (threaded batches: 149 against 141 solves/s, their end-to-end runs 36 against 25)
// lose more than the single solve gains, since a cluster holds its SMs for the whole level.
// The same design measured slower elsewhere, so it is not used there: level 2 in double 65.2
// against 58.1 ms (the FP64 fits of 64 warps on 8 SMs), and level 3 (512 elements, 8 blocks of
// 32 warps, two elements per warp, 64 registers) 81.8 against 17.7 ms in double-float.
// ---------------------------------------------------------------------------------------------
template <int LEVEL, int NC>
struct ClusterLevel
{
    static constexpr int R = 1 << LEVEL, N1 = R + 1, NN = N1 * N1 * N1, NE = R * R * R, S = 27;
    static constexpr int NWB = NE / NC;  // one warp per element
    static constexpr bool kSmemStencil = true;
    template <typename Real>
    static constexpr size_t xy_bytes() { return (sizeof(Real2<Real>) * NN + 15) / 16 * 16; }
    template <typename Real>
    static constexpr size_t part_bytes() { return sizeof(Real) * 10 * NE; }
    // a 16-block cluster asks for more shared memory than it uses, so that no two of its blocks
    // share an SM (each SM sub-partition then issues for one warp)
    template <typename Real>
    static constexpr size_t smem_bytes()
    {
        const size_t used = xy_bytes<Real>() + part_bytes<Real>() + (kSmemStencil ? 2 * sizeof(Real) * S * NN : 0);
        return NC == 16 && used < 116 * 1024 ? 116 * 1024 : used;
    }
};

template <typename Real, int LEVEL, int NC>
__device__ __forceinline__ void gs_cluster_body(const LevelPtrs<Real> &L, int iters, unsigned int *err, int separate, int *kexp)
{
    namespace cg = cooperative_groups;
    using CL = ClusterLevel<LEVEL, NC>;
    constexpr int R = CL::R, N1 = CL::N1, NN = CL::NN, NE = CL::NE, S = CL::S, s0 = N1 * N1, s1 = N1;
    constexpr int W = NC * CL::NWB;
    constexpr bool kDF = std::is_same<Real, df>::value;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char cl_smem[];
    Real2<Real> *xy = reinterpret_cast<Real2<Real> *>(cl_smem);
    Real *part = reinterpret_cast<Real *>(cl_smem + CL::template xy_bytes<Real>());
    Real *As = part + 10 * NE, *Bs = As + S * NN;
    const Real *Ag = CL::kSmemStencil ? As : L.A, *Bg = CL::kSmemStencil ? Bs : L.B;
    const unsigned rank = cluster.block_rank();
    const int lane = threadIdx.x & 31, gw = (int)rank * CL::NWB + (threadIdx.x >> 5);
    for (int k = threadIdx.x; k < NN; k += blockDim.x) xy[k] = ld2(L.xy, k);
    if constexpr (CL::kSmemStencil)
        for (int k = threadIdx.x; k < S * NN; k += blockDim.x)
        {
            As[k] = L.A[k];
            Bs[k] = L.B[k];
        }
    cluster.sync();  // every replica ready before any remote write
    Real wmul = wedge_mult<Real>(kexp, LEVEL);
    const Grid<3> g(LEVEL);
    for (int it = 0; it < iters; it++)
    {
#pragma unroll 1
        for (int c = 0; c < 8; c++)
        {
            const int par[3] = {c & 1, (c >> 1) & 1, (c >> 2) & 1};
            const int cnt1 = par[1] ? R / 2 : R / 2 + 1, cnt2 = par[2] ? R / 2 : R / 2 + 1;
            // (1) element incidences
#pragma unroll 1
            for (int e = gw; e < NE; e += W)
            {
                const int E[3] = {e / (R * R), (e / R) % R, e % R};
                int I[3], b[3];
                bool designated = true;
#pragma unroll
                for (int d = 0; d < 3; d++)
                {
                    b[d] = par[d] ^ (E[d] & 1);
                    I[d] = E[d] + b[d];
                    designated = designated && E[d] == (I[d] > 0 ? I[d] - 1 : 0);
                }
                const int i = (I[0] * N1 + I[1]) * N1 + I[2];
                const int A = (b[0] << 2) | (b[1] << 1) | b[2];
                Real r[5] = {0, 0, 0, 0, 0};
                if (lane < 12)
                {
                    const int K = lane >> 2, pq = lane & 3;
                    const int pax[3] = {(K == 2) ? 1 : 0, (K == 0) ? 1 : 2, (K == 0) ? 2 : (K == 1 ? 1 : 0)};
                    int sd[3];
#pragma unroll
                    for (int a = 0; a < 3; a++)
                    {
                        const int stride = pax[a] == 0 ? s0 : (pax[a] == 1 ? s1 : 1);
                        sd[a] = ((A >> (2 - pax[a])) & 1) ? -stride : stride;
                    }
                    Real x[8], y[8];
#pragma unroll
                    for (int cc = 0; cc < 8; cc++)
                    {
                        int jj = i;
#pragma unroll
                        for (int a = 0; a < 3; a++)
                            if (cbit<3>(cc, a)) jj += sd[a];
                        const Real2<Real> v = xy[jj];
                        x[cc] = v.x;
                        y[cc] = v.y;
                    }
                    component_fit_pq3<Real>(x, y, pq >> 1, pq & 1, r);
                }
                else if (lane >= 16 && designated)
                {
#pragma unroll
                    for (int half = 0; half < 2; half++)
                    {
                        const int o = lane - 16 + 16 * half;
                        if (o >= S) continue;
                        const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
                        bool in = true;
#pragma unroll
                        for (int d = 0; d < 3; d++) { const int q = I[d] + off[d]; in = in && q >= 0 && q <= R; }
                        if (!in) continue;
                        const int jj = i + off[0] * s0 + off[1] * s1 + off[2];
                        const Real a = Ag[o * NN + i], bb = Bg[o * NN + i];
                        const Real2<Real> q = xy[jj];
                        r[0] += a * q.x;
                        r[1] += a * q.y;
                        if (o == 13) r[4] = a;
                        else { r[2] += bb * q.x; r[3] += bb * q.y; }
                    }
                }
#pragma unroll
                for (int o = 8; o > 0; o >>= 1)
#pragma unroll
                    for (int k = 0; k < 5; k++) r[k] += shfl_xor_any(r[k], o);
                Real stc[5];
#pragma unroll
                for (int k = 0; k < 5; k++) stc[k] = shfl_any(r[k], 16);
                if (lane == 0)
                {
                    const int jc = ((I[0] >> 1) * cnt1 + (I[1] >> 1)) * cnt2 + (I[2] >> 1);
                    Real *dst = cluster.map_shared_rank(part, (unsigned)(jc % NC)) + 10 * e;
#pragma unroll
                    for (int k = 0; k < 5; k++)
                    {
                        dst[k] = r[k];
                        dst[5 + k] = designated ? stc[k] : (Real)0;
                    }
                }
            }
            cluster.sync();  // every element's sums in its node's owner block
            // (2) the owner block's nodes
            {
                const Colour<3> col(g, c);
                for (int jc = (int)rank + NC * (int)threadIdx.x; jc < (int)col.n; jc += NC * (int)blockDim.x)
                {
                    int I[3];
                    col.node(jc, I);
                    const int i = (I[0] * N1 + I[1]) * N1 + I[2];
                    Real h[5] = {0, 0, 0, 0, 0};
#pragma unroll 1
                    for (int bb = 0; bb < 8; bb++)
                    {
                        int E[3];
                        bool ok = true;
#pragma unroll
                        for (int d = 0; d < 3; d++) { E[d] = I[d] - ((bb >> (2 - d)) & 1); ok = ok && E[d] >= 0 && E[d] < R; }
                        if (!ok) continue;
                        const Real *pe = part + 10 * ((E[0] * R + E[1]) * R + E[2]);
#pragma unroll
                        for (int k = 0; k < 5; k++) h[k] += pe[k];
                    }
                    const int ed = ((I[0] > 0 ? I[0] - 1 : 0) * R + (I[1] > 0 ? I[1] - 1 : 0)) * R + (I[2] > 0 ? I[2] - 1 : 0);
                    const Real *sv = part + 10 * ed + 5;
                    const Real sc = (Real)wedge_scale<3>(R) * wmul;
                    Real q[5];
                    q[0] = h[0] * sc + sv[4];
                    q[1] = h[1] * sc + sv[4];
                    q[2] = (Real)2 * h[2] * sc;
                    q[3] = (Real)2 * h[3] * sc + (Real)2 * sv[0] - (Real)2 * sv[3];
                    q[4] = (Real)2 * h[4] * sc + (Real)2 * sv[1] + (Real)2 * sv[2];
                    Real p0, p1;
                    if (relaxed(L, i) && node_step_tiny<Real>(q, separate, p0, p1))
                    {
                        Real2<Real> cur = xy[i];
                        cur.x += p0;
                        cur.y += p1;
                        if (!finite_value<Real>(cur.x) || !finite_value<Real>(cur.y)) atomicOr(err, (unsigned int)ERR_NONFINITE);
#pragma unroll 1
                        for (int k = 0; k < NC; k++) cluster.map_shared_rank(xy, (unsigned)k)[i] = cur;
                    }
                }
            }
            cluster.sync();  // every replica updated before the next colour reads it
        }
        if constexpr (kDF)
            if (kexp)
            {
                // the replicas hold the same values, so every block picks the same exponent
                const int shift = df_rescale_shift(reinterpret_cast<const df *>(xy), 2 * NN);
                if (shift)
                {
                    df *v = reinterpret_cast<df *>(xy);
                    for (int k = threadIdx.x; k < 2 * NN; k += blockDim.x) v[k] = ldexp_df(v[k], shift);
                    if (rank == 0 && threadIdx.x == 0) kexp[LEVEL] -= shift;
                }
                cluster.sync();  // the new exponent visible, no remote write before every rescale
                if (shift) wmul = wedge_mult<Real>(kexp, LEVEL);
            }
    }
    if (rank == 0)
        for (int k = threadIdx.x; k < NN; k += blockDim.x) reinterpret_cast<Real2<Real> *>(L.xy)[k] = xy[k];
    cluster.sync();  // no block leaves while another may still address its shared memory
}

// launched with a cluster of NC blocks (cudaLaunchKernelEx, launch_cluster_level)
template <typename Real, int LEVEL, int NC>
__global__ void __launch_bounds__(ClusterLevel<LEVEL, NC>::NWB * 32)
    gs_cluster_kernel(LevelPtrs<Real> L, int iters, unsigned int *err, int separate, int *kexp)
{
    gs_cluster_body<Real, LEVEL, NC>(L, iters, err, separate, kexp);
}

// one cluster per reconstruction of a lockstep batch
template <typename Real, int LEVEL, int NC>
__global__ void __launch_bounds__(ClusterLevel<LEVEL, NC>::NWB * 32) gs_cluster_batch_kernel(const BatchJob<Real> *jobs)
{
    const BatchJob<Real> &b = jobs[blockIdx.x / NC];
    gs_cluster_body<Real, LEVEL, NC>(b.L, b.iters, b.err, b.separate, b.kexp);
}

// a launch of `count` clusters of NC blocks
template <typename Kernel, typename... Args>
cudaError_t launch_clusters(Kernel kernel, int nc, int count, int threads, size_t smem, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nc * count), 1, 1);
    cfg.blockDim = dim3((unsigned)threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)nc;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <typename Real>
__global__ void __launch_bounds__(128) gs_tiny0_kernel(LevelPtrs<Real> L, int iters, unsigned int *err, int separate, int *kexp)
{
    gs_tiny0_body<Real>(L, iters, err, separate, kexp);
}

template <typename Real>
__global__ void __launch_bounds__(128) gs_tiny0_batch_kernel(const BatchJob<Real> *jobs)
{
    const BatchJob<Real> &b = jobs[blockIdx.x];
    gs_tiny0_body<Real>(b.L, b.iters, b.err, b.separate, b.kexp);
}

template <typename Real, int LEVEL>
__global__ void __launch_bounds__(LEVEL == 0 ? 32 : 256) gs_tiny_kernel(LevelPtrs<Real> L, int iters, unsigned int *err,
                                                                          int separate, int *kexp)
{
    gs_tiny_body<Real, LEVEL>(L, iters, err, separate, kexp);
}

// every reconstruction of a lockstep batch at once: one block per reconstruction, each with its
// own sweep count
template <typename Real, int LEVEL>
__global__ void __launch_bounds__(LEVEL == 0 ? 32 : 256) gs_tiny_batch_kernel(const BatchJob<Real> *jobs)
{
    const BatchJob<Real> &b = jobs[blockIdx.x];
    gs_tiny_body<Real, LEVEL>(b.L, b.iters, b.err, b.separate, b.kexp);
}

template <int D, typename Real>
__global__ void __launch_bounds__(kThreads) gn_matvec_kernel(LevelPtrs<Real> L, const Real *xy, const Real *dxy, Real *out)
{
    Grid<D> g(L.level);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    NodeCtx<D> nc;
    make_ctx<D>(g, i, nc);
    Real s[2] = {0, 0};
#pragma unroll 1
    for (int A = 0; A < (1 << D); A++)
    {
        Real x[1 << D], y[1 << D], dx[1 << D], dy[1 << D];
        if (!gather_element<D, Real>(g, nc, i, A, xy, x, y)) continue;
        gather_element<D, Real>(g, nc, i, A, dxy, dx, dy);
        element_gn<D, Real>(x, y, dx, dy, A, s);
    }
    const Real sc = (Real)wedge_scale<D>(g.r);
    Real ox = s[0] * sc, oy = s[1] * sc;
    constexpr int S = Dims<D>::S;
    for (int o = 0; o < S; o++)
    {
        int off[D];
        stencil_offset<D>(o, off);
        bool ok = true;
        int64_t j = i;
#pragma unroll
        for (int d = 0; d < D; d++)
        {
            int t = nc.I[d] + off[d];
            ok = ok && (t >= 0) && (t <= g.r);
            j += (int64_t)off[d] * nc.stride[d];
        }
        if (!ok) continue;
        Real a = L.A[(int64_t)o * L.N + i];
        Real2<Real> v = ld2(dxy, j);
        ox += a * v.x;
        oy += a * v.y;
    }
    reinterpret_cast<Real2<Real> *>(out)[i] = Real2<Real>{ox, oy};
}

template <int D, typename Real>
__device__ __forceinline__ void prolong_at(int coarseLevel, const Real *coarse, Real *fine, int add, int64_t i,
                                           const uint8_t *fineStatus = nullptr)
{
    Grid<D> gc(coarseLevel), gf(coarseLevel + 1);
    if (i >= gf.N) return;
    // the adaptive prolongation reaches indexed fine functions only (ffChildNeighbors,
    // Hat.scalars.inl:1747-1779); the others stay zero
    if (fineStatus && fineStatus[i] == 0)
    {
        if (!add) reinterpret_cast<Real2<Real> *>(fine)[i] = Real2<Real>{(Real)0, (Real)0};
        return;
    }
    int F[D];
    gf.node(i, F);
    Real sx = 0, sy = 0;
#pragma unroll
    for (int c = 0; c < (1 << D); c++)
    {
        bool use = true;
        Real w = 1;
        int I[D];
#pragma unroll
        for (int d = 0; d < D; d++)
        {
            int b = (c >> d) & 1;
            if (F[d] & 1) { I[d] = (F[d] >> 1) + b; w *= (Real)0.5; }
            else { I[d] = F[d] >> 1; if (b) use = false; }
        }
        if (!use) continue;
        Real2<Real> v = ld2(coarse, gc.node(I));
        sx += w * v.x;
        sy += w * v.y;
    }
    Real2<Real> *o = reinterpret_cast<Real2<Real> *>(fine);
    if (add) { Real2<Real> cur = o[i]; o[i] = Real2<Real>{cur.x + sx, cur.y + sy}; }
    else o[i] = Real2<Real>{sx, sy};
}
template <int D, typename Real>
__global__ void prolong_kernel(int coarseLevel, const Real *coarse, Real *fine, int add, const uint8_t *fineStatus)
{
    prolong_at<D, Real>(coarseLevel, coarse, fine, add, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, fineStatus);
}
// grid.y = reconstruction of a lockstep batch
template <typename Real>
__global__ void prolong_add_batch_kernel(const XferJob *jobs, int coarseLevel)
{
    const XferJob &j = jobs[blockIdx.y];
    prolong_at<3, Real>(coarseLevel, (const Real *)j.src, (Real *)j.dst, 1, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}
__global__ void f2d_batch_kernel(const XferJob *jobs, int64_t n)
{
    const XferJob &j = jobs[blockIdx.y];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) ((double *)j.dst)[i] = (double)((const float *)j.src)[i];
}
__global__ void d2f_batch_kernel(const XferJob *jobs, int64_t n)
{
    const XferJob &j = jobs[blockIdx.y];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) ((float *)j.dst)[i] = (float)((const double *)j.src)[i];
}

template <int D, typename Real>
__global__ void restrict_kernel(int coarseLevel, const Real *fine, Real *coarse)
{
    Grid<D> gc(coarseLevel), gf(coarseLevel + 1);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= gc.N) return;
    int I[D];
    gc.node(i, I);
    Real sx = 0, sy = 0;
    constexpr int S = Dims<D>::S;
#pragma unroll 3
    for (int o = 0; o < S; o++)
    {
        int off[D], F[D];
        stencil_offset<D>(o, off);
        bool ok = true;
        Real w = 1;
#pragma unroll
        for (int d = 0; d < D; d++)
        {
            F[d] = 2 * I[d] + off[d];
            ok = ok && F[d] >= 0 && F[d] <= gf.r;
            if (off[d]) w *= (Real)0.5;
        }
        if (!ok) continue;
        Real2<Real> v = ld2(fine, gf.node(F));
        sx += w * v.x;
        sy += w * v.y;
    }
    reinterpret_cast<Real2<Real> *>(coarse)[i] = Real2<Real>{sx, sy};
}

template <typename Real>
__global__ void scale_kernel(Real *v, int64_t n, double s)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = (Real)((double)v[i] * s);
}
template <typename Real>
__global__ void axpy_kernel(Real *y, const Real *x, int64_t n, double a)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = (Real)((double)y[i] + a * (double)x[i]);
}
__global__ void d2f_kernel(const double *in, float *out, int64_t n)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}
__global__ void f2d_kernel(const float *in, double *out, int64_t n)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

inline unsigned int blocks_for(int64_t n, int t = kThreads) { return (unsigned int)((n + t - 1) / t); }

int g_lanes_variant = 1;  // 0: scalar float element fit in the lane kernel, 1: packed
int g_cluster_levels = 0;  // 1: 3D level 2 in double-float by gs_cluster_kernel (8 / 16: that cluster size)
int g_cluster_blocks = 8;  // the cluster size chosen by prepare_cluster_kernels
int g_tiny_levels = 1;    // 1: 3D levels 0-1 by gs_tiny0_kernel / gs_tiny1_kernel, 2: level 0 by the one-warp
                          // gs_tiny_kernel, 3: level 1 by the one-block gs_tiny_kernel, 0: by the block
                          // kernels of gs_level_kernel
int g_gs_variant = 1;  // 0: one thread per node, 1: 2^D lanes per node (row grid), 2: 2^D lanes per node (flat grid),
                       // 4: as 1 without the point-split update of the small 3D levels

}  // namespace

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
template <int D, typename Real>
void launch_energy(const LevelPtrs<Real> &L, const Real *xy, const Reduce &red, cudaStream_t s)
{
    Grid<D> g(L.level);
    int64_t total = g.N > g.NE ? g.N : g.NE;
    int nb = (int)blocks_for(total);
    if (nb > Reduce::kMaxBlocks) nb = Reduce::kMaxBlocks;
    if (nb < 1) nb = 1;
    energy_kernel<D, Real><<<nb, kThreads, 0, s>>>(L, xy, red.partial);
    double scale0 = (D == 3 ? (double)g.r : 1.0) * 0.5;
    finish_kernel<<<1, 96, 0, s>>>(red.partial, nb, 3, red.out, scale0);
}

template <int D, typename Real>
void launch_grad_norm(const LevelPtrs<Real> &L, const Real *xy, const Reduce &red, cudaStream_t s)
{
    Grid<D> g(L.level);
    int nb = (int)blocks_for(g.N);
    if (nb > Reduce::kMaxBlocks) nb = Reduce::kMaxBlocks;
    if (nb < 1) nb = 1;
    grad_norm_kernel<D, Real><<<nb, kThreads, 0, s>>>(L, xy, red.partial);
    finish_kernel<<<1, 32, 0, s>>>(red.partial, nb, 1, red.out, 1.0);
}

template <int D, typename Real>
void launch_quadfit(const LevelPtrs<Real> &L, const Real *xy, double *out, cudaStream_t s)
{
    Grid<D> g(L.level);
    quadfit_kernel<D, Real><<<blocks_for(g.N), kThreads, 0, s>>>(L, xy, out);
}

template <int D, typename Real>
void launch_gs_colour(const LevelPtrs<Real> &L, int colour, unsigned int *err, cudaStream_t s, int separate)
{
    Grid<D> g(L.level);
    Colour<D> col(g, colour);
    if (col.n == 0) return;
    if constexpr (D == 3)
        if (g_gs_variant != 0 && g_gs_variant != 4 && col.n <= kSplitMaxColourNodes)
        {
            // small levels: point-split update, 128 threads per node
            gs_colour_split3_kernel<Real><<<(unsigned)((col.n + kSplitNodes - 1) / kSplitNodes), 128 * kSplitNodes, 0, s>>>(
                L, col, colour_block_base<D>(g, colour), err, separate);
            return;
        }
    if (L.alist)
    {
        // adaptive level: only the colour's active nodes
        const int count = L.aoff[colour + 1] - L.aoff[colour];
        if (count == 0) return;
        constexpr int NPB = kThreads >> D;
        const unsigned nb = (unsigned)((count + NPB - 1) / NPB);
        const int64_t cb = colour_block_base<D>(g, colour);
        const int *list = L.alist + L.aoff[colour];
        if constexpr (std::is_same<Real, float>::value)
            if (g_lanes_variant != 0)
            {
                gs_colour_lanes_list_kernel<D, Real, D == 3 ? 9 : 1, true><<<nb, kThreads, 0, s>>>(L, col, cb, list, count, err, separate);
                return;
            }
        gs_colour_lanes_list_kernel<D, Real><<<nb, kThreads, 0, s>>>(L, col, cb, list, count, err, separate);
        return;
    }
    if (g_gs_variant == 0) gs_colour_kernel<D, Real><<<blocks_for(col.n), kThreads, 0, s>>>(L, col, err, separate);
    else if (g_gs_variant == 2)
        gs_colour_flat_kernel<D, Real><<<blocks_for(col.n << D), kThreads, 0, s>>>(L, col, err, separate);
    else
    {
        constexpr int NPB = kThreads >> D;
        dim3 grid((unsigned)((col.cnt[D - 1] + NPB - 1) / NPB), (unsigned)col.cnt[D - 2],
                  (unsigned)(D == 3 ? col.cnt[0] : col.cnt[0] * col.cnt[1]));
        const int64_t cb = colour_block_base<D>(g, colour);
        // float: the element integrals on the packed two-wide FP32 instructions (3D: 0.614 against
        // 0.680 ms per depth-8 colour; registers capped at 56, 9 resident blocks, where the
        // scalar fit ran best at 48); EPR_LANES_VARIANT=0 selects the scalar fit
        // (EPR_LANES_VARIANT 2 and 3: the block's row of nodes staged in shared memory, 9 or 8
        // resident blocks: 0.741 and 0.785 against 0.601 ms per depth-8 colour -- the kernel is
        // bound by instruction issue, and the staging adds instructions and a block barrier)
        if constexpr (std::is_same<Real, float>::value)
            if (g_lanes_variant != 0)
            {
                if (g_lanes_variant == 2)
                    gs_colour_lanes_kernel<D, Real, D == 3 ? 9 : 1, true, true><<<grid, kThreads, 0, s>>>(L, col, cb, err, separate);
                else if (g_lanes_variant == 3)
                    gs_colour_lanes_kernel<D, Real, D == 3 ? 8 : 1, true, true><<<grid, kThreads, 0, s>>>(L, col, cb, err, separate);
                else
                    gs_colour_lanes_kernel<D, Real, D == 3 ? 9 : 1, true><<<grid, kThreads, 0, s>>>(L, col, cb, err, separate);
                return;
            }
        gs_colour_lanes_kernel<D, Real><<<grid, kThreads, 0, s>>>(L, col, cb, err, separate);
    }
}

void set_gs_variant(int v) { g_gs_variant = v; }
void set_lanes_variant(int v) { g_lanes_variant = v; }
void set_tiny_levels(int v) { g_tiny_levels = v; }
void set_cluster_levels(int v) { g_cluster_levels = v; }
bool cluster_level(int level, bool isDF) { return g_cluster_levels && isDF && level == 2; }

// all sweeps of a 3D level 0 or 1 in gs_tiny_kernel (one warp per incidence of a colour)
template <typename Real>
bool launch_tiny_level(const LevelPtrs<Real> &L, int iters, unsigned int *err, cudaStream_t s, int separate, int *kexp)
{
    // level 2 in double-float: one launch on a cluster (EPR_CLUSTER_LEVELS=1; by default a launch
    // per colour)
    if constexpr (std::is_same<Real, df>::value)
        if (cluster_level(L.level, true))
        {
            if (g_cluster_blocks == 16)
                launch_clusters(gs_cluster_kernel<Real, 2, 16>, 16, 1, ClusterLevel<2, 16>::NWB * 32, ClusterLevel<2, 16>::smem_bytes<Real>(), s,
                                L, iters, err, separate, kexp);
            else
                launch_clusters(gs_cluster_kernel<Real, 2, 8>, 8, 1, ClusterLevel<2, 8>::NWB * 32, ClusterLevel<2, 8>::smem_bytes<Real>(), s, L,
                                iters, err, separate, kexp);
            return true;
        }
    if (!g_tiny_levels || L.level > 1) return false;
    if (L.level == 0)
    {
        if (g_tiny_levels == 2) gs_tiny_kernel<Real, 0><<<1, 32, 0, s>>>(L, iters, err, separate, kexp);
        else gs_tiny0_kernel<Real><<<1, 128, 0, s>>>(L, iters, err, separate, kexp);
    }
    // level 1: the two-block cluster in double-float and double (33.7 against 43.0 ms, 73 against 112
    // ms at depth 8); float keeps the one-block kernel (8.8 against 11.4 ms: its phases are short
    // enough for the cluster barriers to dominate)
    else if (g_tiny_levels == 3 || std::is_same<Real, float>::value) gs_tiny_kernel<Real, 1><<<1, 256, 0, s>>>(L, iters, err, separate, kexp);
    else gs_tiny1_kernel<Real><<<2, 128, 0, s>>>(L, iters, err, separate, kexp);
    return true;
}

// shared-memory carve-out of the single-block level kernels whose stencils live in shared memory
constexpr size_t kLevelSmemLimit = 200 * 1024;

// block size bound of the point-split level kernel (128 threads per node)
constexpr int kSplitThreads = 1024;

template <int D, typename Real>
static void prepare_level_kernels()
{
    constexpr int MT = persistent_threads<D, Real>();
    cudaFuncSetAttribute(gs_level_kernel<D, Real, true, MT, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLevelSmemLimit);
    if constexpr (D == 3)
    {
        cudaFuncSetAttribute(gs_level_kernel<D, Real, true, MT, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLevelSmemLimit);
        cudaFuncSetAttribute(gs_level_kernel<D, Real, true, kSplitThreads, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kLevelSmemLimit);
    }
}

// the level-2 cluster's size: 16 blocks (one warp per SM sub-partition) where the device can hold
// such a cluster with one block per SM, else 8 (EPR_CLUSTER_LEVELS=8 or 16 forces one)
static void prepare_cluster_kernels()
{
    cudaFuncSetAttribute(gs_cluster_kernel<df, 2, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ClusterLevel<2, 8>::smem_bytes<df>());
    cudaFuncSetAttribute(gs_cluster_batch_kernel<df, 2, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)ClusterLevel<2, 4>::smem_bytes<df>());
    const int smem16 = (int)ClusterLevel<2, 16>::smem_bytes<df>();
    bool ok16 = true;
    for (auto k : {(const void *)gs_cluster_kernel<df, 2, 16>})
    {
        ok16 = ok16 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
               cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem16) == cudaSuccess;
    }
    int clusters = 0;
    if (ok16)
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(16, 1, 1);
        cfg.blockDim = dim3(ClusterLevel<2, 16>::NWB * 32, 1, 1);
        cfg.dynamicSmemBytes = (size_t)smem16;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 16;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        if (cudaOccupancyMaxActiveClusters(&clusters, (const void *)gs_cluster_kernel<df, 2, 16>, &cfg) != cudaSuccess) clusters = 0;
    }
    cudaGetLastError();  // an unsupported query leaves no error behind
    if (g_cluster_levels == 8 || g_cluster_levels == 16) g_cluster_blocks = g_cluster_levels;
    else g_cluster_blocks = clusters >= 1 ? 16 : 8;
}

void prepare_gs_kernels()
{
    prepare_cluster_kernels();
    prepare_level_kernels<3, float>();
    prepare_level_kernels<3, double>();
    prepare_level_kernels<3, df>();
    prepare_level_kernels<4, float>();
    prepare_level_kernels<4, double>();
}

template <int D, typename Real>
int launch_gs_sweeps(const LevelPtrs<Real> &L, int iters, unsigned int *err, cudaStream_t s, int separate, int64_t persistentMaxNodes)
{
    Grid<D> g(L.level);
    if (iters <= 0) return 0;
    if constexpr (D == 3)
        if (g.N <= persistentMaxNodes && launch_tiny_level<Real>(L, iters, err, s, separate, nullptr)) return 1;
    if (g.N <= persistentMaxNodes)
    {
        constexpr int MT = persistent_threads<D, Real>();
        const int64_t colour0 = Colour<D>(g, 0).n;  // the colour of even nodes is the largest
        const size_t xyBytes = 2 * g.N * sizeof(Real), stBytes = 2 * (size_t)Dims<D>::S * g.N * sizeof(Real);
        const bool smemStencil = xyBytes + stBytes <= kLevelSmemLimit;
        const size_t smem = xyBytes + (smemStencil ? stBytes : 0);
        // the single node of a colour at resolution 1 is point-split (17 against 24 ms float, 146
        // against 234 ms double for the level's 2560 sweeps at depth 8); resolution 2 takes a warp
        // per node (13 against 16 ms float, 145 against 182 ms double)
        if constexpr (D == 3)
            if (g_gs_variant != 4 && colour0 == 1)
            {
                // 128 threads per node: the tiny levels, where the update latency sets the pace
                const int threads = (int)colour0 * 128;
                if (smemStencil) gs_level_kernel<D, Real, true, kSplitThreads, 2><<<1, threads, smem, s>>>(L, iters, err, separate);
                else gs_level_kernel<D, Real, false, kSplitThreads, 2><<<1, threads, smem, s>>>(L, iters, err, separate);
                return 1;
            }
        if constexpr (D == 3)
            if (colour0 <= 8 && colour0 * 32 <= MT)
            {
                const int threads = (int)colour0 * 32;
                if (smemStencil) gs_level_kernel<D, Real, true, MT, 1><<<1, threads, smem, s>>>(L, iters, err, separate);
                else gs_level_kernel<D, Real, false, MT, 1><<<1, threads, smem, s>>>(L, iters, err, separate);
                return 1;
            }
        // lanes per node: one pass per colour where the block allows it, whole warps
        const int threads = (int)std::min<int64_t>(MT, ((colour0 << D) + 31) / 32 * 32);
        if (smemStencil) gs_level_kernel<D, Real, true, MT, 0><<<1, threads, smem, s>>>(L, iters, err, separate);
        else gs_level_kernel<D, Real, false, MT, 0><<<1, threads, smem, s>>>(L, iters, err, separate);
        return 1;
    }
    int n = 0;
    for (int it = 0; it < iters; it++)
        for (int c = 0; c < (1 << D); c++) { launch_gs_colour<D, Real>(L, c, err, s, separate); n++; }
    return n;
}

// ---------------------------------------------------------------------------------------------
// double-float levels (3D levels 0-3 of the float solve's coarse band)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void df_rescale_body(df *xy, int64_t n, int *kexp, int level)
{
    const int shift = df_rescale_shift(xy, n);
    if (!shift) return;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) xy[k] = ldexp_df(xy[k], shift);
    if (threadIdx.x == 0) kexp[level] -= shift;
}
__global__ void df_rescale_kernel(df *xy, int64_t n, int *kexp, int level) { df_rescale_body(xy, n, kexp, level); }
// one block per reconstruction of a lockstep batch
__global__ void df_rescale_batch_kernel(const BatchJob<df> *jobs)
{
    const BatchJob<df> &b = jobs[blockIdx.x];
    df_rescale_body(b.L.xy, 2 * b.L.N, b.kexp, b.L.level);
}

// double coefficients -> pairs at the level's new exponent (the largest magnitude in [1, 2))
__device__ __forceinline__ void df_push_body(const double *in, df *out, int64_t n, int *kexp, int level)
{
    __shared__ double wmax[32];
    __shared__ int k;
    double m = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(in[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double mm = 0.0;
        for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) mm = fmax(mm, wmax[w]);
        k = mm > 0.0 ? ilogb(mm) : 0;
        kexp[level] = k;
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) out[i] = df(ldexp(in[i], -k));
}
__global__ void df_push_kernel(const double *in, df *out, int64_t n, int *kexp, int level) { df_push_body(in, out, n, kexp, level); }
__global__ void df_push_batch_kernel(const XferJob *jobs, int64_t n, int level)
{
    const XferJob &j = jobs[blockIdx.x];
    df_push_body((const double *)j.src, (df *)j.dst, n, j.kexp, level);
}
__global__ void df_pull_batch_kernel(const XferJob *jobs, int64_t n, int level)
{
    const XferJob &j = jobs[blockIdx.y];
    const int k = j.kexp[level];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) ((double *)j.dst)[i] = ldexp((double)((const df *)j.src)[i], k);
}

__global__ void df_pull_kernel(const df *in, double *out, int64_t n, const int *kexp, int level)
{
    const int k = kexp[level];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = ldexp((double)in[i], k);
}

__global__ void d2df_kernel(const double *in, df *out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) out[i] = df(in[i]);
}

void launch_df_push(const double *in, df *out, int64_t n, int *kexp, int level, cudaStream_t s)
{
    df_push_kernel<<<1, 256, 0, s>>>(in, out, n, kexp, level);
}
void launch_df_pull(const df *in, double *out, int64_t n, const int *kexp, int level, cudaStream_t s)
{
    df_pull_kernel<<<(unsigned)std::min<int64_t>(blocks_for(n, 256), 1024), 256, 0, s>>>(in, out, n, kexp, level);
}
void launch_d2df(const double *in, df *out, int64_t n, cudaStream_t s)
{
    if (n) d2df_kernel<<<(unsigned)std::min<int64_t>(blocks_for(n, 256), 1024), 256, 0, s>>>(in, out, n);
}

// one colour of a double-float level with the per-colour kernel of the sweeps below (profiling)
void launch_gs_colour_df(const LevelPtrs<df> &L, int colour, unsigned int *err, cudaStream_t s, int *kexp)
{
    Grid<3> g(L.level);
    Colour<3> col(g, colour);
    if (col.n == 0) return;
    gs_colour_split3_kernel<df><<<(unsigned)((col.n + kSplitNodes - 1) / kSplitNodes), 128 * kSplitNodes, 0, s>>>(L, col, 0, err, 0, kexp);
}

// Paired GS sweeps of a 3D double-float level (levels 0-3): the same kernels as a float or double
// level of that size, with the wedge factor of the level's exponent and a new exponent after every
// sweep.
int launch_gs_sweeps_df(const LevelPtrs<df> &L, int iters, unsigned int *err, cudaStream_t s, int separate,
                        int64_t persistentMaxNodes, int *kexp)
{
    Grid<3> g(L.level);
    if (iters <= 0) return 0;
    if ((g.N <= persistentMaxNodes || cluster_level(L.level, true)) && launch_tiny_level<df>(L, iters, err, s, separate, kexp)) return 1;
    if (g.N <= persistentMaxNodes)
    {
        constexpr int MT = persistent_threads<3, df>();
        const int64_t colour0 = Colour<3>(g, 0).n;
        const size_t xyBytes = 2 * g.N * sizeof(df), stBytes = 2 * (size_t)Dims<3>::S * g.N * sizeof(df);
        const bool smemStencil = xyBytes + stBytes <= kLevelSmemLimit;
        const size_t smem = xyBytes + (smemStencil ? stBytes : 0);
        if (colour0 == 1)
        {
            if (smemStencil) gs_level_kernel<3, df, true, kSplitThreads, 2><<<1, 128, smem, s>>>(L, iters, err, separate, kexp);
            else gs_level_kernel<3, df, false, kSplitThreads, 2><<<1, 128, smem, s>>>(L, iters, err, separate, kexp);
            return 1;
        }
        if (colour0 <= 8 && colour0 * 32 <= MT)
        {
            const int threads = (int)colour0 * 32;
            if (smemStencil) gs_level_kernel<3, df, true, MT, 1><<<1, threads, smem, s>>>(L, iters, err, separate, kexp);
            else gs_level_kernel<3, df, false, MT, 1><<<1, threads, smem, s>>>(L, iters, err, separate, kexp);
            return 1;
        }
        const int threads = (int)std::min<int64_t>(MT, ((colour0 << 3) + 31) / 32 * 32);
        if (smemStencil) gs_level_kernel<3, df, true, MT, 0><<<1, threads, smem, s>>>(L, iters, err, separate, kexp);
        else gs_level_kernel<3, df, false, MT, 0><<<1, threads, smem, s>>>(L, iters, err, separate, kexp);
        return 1;
    }
    int n = 0;
    for (int it = 0; it < iters; it++)
    {
        for (int c = 0; c < 8; c++)
        {
            Colour<3> col(g, c);
            if (col.n == 0) continue;
            // colours of levels up to 3 have at most 125 nodes: point-split, 128 threads per node
            gs_colour_split3_kernel<df><<<(unsigned)((col.n + kSplitNodes - 1) / kSplitNodes), 128 * kSplitNodes, 0, s>>>(
                L, col, 0, err, separate, kexp);
            n++;
        }
        df_rescale_kernel<<<1, 256, 0, s>>>(L.xy, 2 * g.N, kexp, L.level);
        n++;
    }
    return n;
}

template <int D, typename Real>
void launch_gn_matvec(const LevelPtrs<Real> &L, const Real *xy, const Real *dxy, Real *out, cudaStream_t s)
{
    Grid<D> g(L.level);
    gn_matvec_kernel<D, Real><<<blocks_for(g.N), kThreads, 0, s>>>(L, xy, dxy, out);
}

template <int D, typename Real>
void launch_prolong(int coarseLevel, const Real *coarse, Real *fine, int add, cudaStream_t s, const uint8_t *fineStatus)
{
    Grid<D> gf(coarseLevel + 1);
    prolong_kernel<D, Real><<<blocks_for(gf.N, 256), 256, 0, s>>>(coarseLevel, coarse, fine, add, fineStatus);
}

template <int D, typename Real>
void launch_restrict(int coarseLevel, const Real *fine, Real *coarse, cudaStream_t s)
{
    Grid<D> gc(coarseLevel);
    restrict_kernel<D, Real><<<blocks_for(gc.N, 256), 256, 0, s>>>(coarseLevel, fine, coarse);
}

template <typename Real>
void launch_scale(Real *v, int64_t n, double sc, cudaStream_t st)
{
    if (n) scale_kernel<Real><<<blocks_for(n, 256), 256, 0, st>>>(v, n, sc);
}
template <typename Real>
void launch_axpy(Real *y, const Real *x, int64_t n, double a, cudaStream_t st)
{
    if (n) axpy_kernel<Real><<<blocks_for(n, 256), 256, 0, st>>>(y, x, n, a);
}
__global__ void split_pairs_kernel(const double *xy, double *x, double *y, int64_t n)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) { double2 v = reinterpret_cast<const double2 *>(xy)[i]; x[i] = v.x; y[i] = v.y; }
}
__global__ void merge_pairs_kernel(const double *x, const double *y, double *xy, int64_t n)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) reinterpret_cast<double2 *>(xy)[i] = double2{x[i], y[i]};
}
void launch_split_pairs(const double *xy, double *x, double *y, int64_t n, cudaStream_t st)
{
    if (n) split_pairs_kernel<<<blocks_for(n, 256), 256, 0, st>>>(xy, x, y, n);
}
void launch_merge_pairs(const double *x, const double *y, double *xy, int64_t n, cudaStream_t st)
{
    if (n) merge_pairs_kernel<<<blocks_for(n, 256), 256, 0, st>>>(x, y, xy, n);
}
void launch_convert_d2f(const double *in, float *out, int64_t n, cudaStream_t st)
{
    if (n) d2f_kernel<<<blocks_for(n, 256), 256, 0, st>>>(in, out, n);
}
void launch_convert_f2d(const float *in, double *out, int64_t n, cudaStream_t st)
{
    if (n) f2d_kernel<<<blocks_for(n, 256), 256, 0, st>>>(in, out, n);
}

// ---------------------------------------------------------------------------------------------
// lockstep batches (3D)
// ---------------------------------------------------------------------------------------------
template <typename Real>
void launch_tiny_batch(const BatchJob<Real> *jobs, int level, int count, cudaStream_t s)
{
    if (count <= 0) return;
    if constexpr (std::is_same<Real, df>::value)
        if (cluster_level(level, true))
        {
            // clusters of 4 blocks of 16 warps: a member's phases take longer than on the solo
            // solve's 16 blocks, but four SMs a member let 38 members relax at once (the node sums
            // run in the same order whatever the cluster size, so the bits are the solo solve's)
            launch_clusters(gs_cluster_batch_kernel<Real, 2, 4>, 4, count, ClusterLevel<2, 4>::NWB * 32,
                            ClusterLevel<2, 4>::smem_bytes<Real>(), s, jobs);
            return;
        }
    if (level == 0)
    {
        if (g_tiny_levels == 2) gs_tiny_batch_kernel<Real, 0><<<count, 32, 0, s>>>(jobs);
        else gs_tiny0_batch_kernel<Real><<<count, 128, 0, s>>>(jobs);
    }
    else if (g_tiny_levels == 3 || std::is_same<Real, float>::value) gs_tiny_batch_kernel<Real, 1><<<count, 256, 0, s>>>(jobs);
    else gs_tiny1_batch_kernel<Real><<<2 * count, 128, 0, s>>>(jobs);
}

template <typename Real, int TPB>
static void launch_lanes_batch(const BatchJob<Real> *jobs, const Grid<3> &g, const Colour<3> &col, int64_t cb, int count,
                               cudaStream_t s)
{
    constexpr bool kFloat = std::is_same<Real, float>::value;
    // float: the packed fit with the solo kernel's register cap (9 blocks of 128 threads per SM)
    constexpr int MinBlocks = kFloat ? (TPB == 64 ? 18 : TPB == 128 ? 9 : 4) : 1;
    constexpr int NPB = TPB >> 3;
    // grid.z = reconstruction x axis-0 count, at most 65,535: chunks of reconstructions
    const int per = std::max(1, 65535 / col.cnt[0]);
    for (int m0 = 0; m0 < count; m0 += per)
    {
        const int cnt = std::min(per, count - m0);
        dim3 grid((unsigned)((col.cnt[2] + NPB - 1) / NPB), (unsigned)col.cnt[1], (unsigned)(cnt * col.cnt[0]));
        gs_colour_lanes_batch_kernel<Real, TPB, MinBlocks, kFloat><<<grid, TPB, 0, s>>>(jobs + m0, col, cb);
    }
}

template <typename Real, int NPB>
static void launch_split3_batch(const BatchJob<Real> *jobs, const Colour<3> &col, int64_t cb, int count, cudaStream_t s)
{
    for (int m0 = 0; m0 < count; m0 += 65535)
    {
        const int cnt = std::min(65535, count - m0);
        dim3 grid((unsigned)((col.n + NPB - 1) / NPB), (unsigned)cnt);
        gs_colour_split3_batch_kernel<Real, NPB><<<grid, 128 * NPB, 0, s>>>(jobs + m0, col, cb);
    }
}

template <typename Real>
void launch_colour_batch(const BatchJob<Real> *jobs, int level, int colour, int count, int tile, cudaStream_t s)
{
    if (count <= 0) return;
    Grid<3> g(level);
    Colour<3> col(g, colour);
    if (col.n == 0) return;
    const int64_t cb = colour_block_base<3>(g, colour);
    if (col.n <= kSplitMaxColourNodes)
    {
        // the solo solve's choice for these levels (the point-split kernel)
        if (tile == 0) launch_split3_batch<Real, 1>(jobs, col, cb, count, s);
        else if (tile == 2) launch_split3_batch<Real, 4>(jobs, col, cb, count, s);
        else launch_split3_batch<Real, 2>(jobs, col, cb, count, s);
        return;
    }
    if constexpr (std::is_same<Real, df>::value) return;  // double-float levels are 3D levels <= 3
    else
    {
        if (tile == 0) launch_lanes_batch<Real, 64>(jobs, g, col, cb, count, s);
        else if (tile == 2) launch_lanes_batch<Real, 256>(jobs, g, col, cb, count, s);
        else launch_lanes_batch<Real, 128>(jobs, g, col, cb, count, s);
    }
}

void launch_df_rescale_batch(const BatchJob<df> *jobs, int count, cudaStream_t s)
{
    if (count > 0) df_rescale_batch_kernel<<<count, 256, 0, s>>>(jobs);
}

template <typename Real>
void launch_prolong_add_batch(const XferJob *jobs, int coarseLevel, int count, cudaStream_t s)
{
    if (count <= 0) return;
    Grid<3> gf(coarseLevel + 1);
    prolong_add_batch_kernel<Real><<<dim3(blocks_for(gf.N, 256), (unsigned)count), 256, 0, s>>>(jobs, coarseLevel);
}
void launch_f2d_batch(const XferJob *jobs, int64_t n, int count, cudaStream_t s)
{
    if (count > 0 && n) f2d_batch_kernel<<<dim3(blocks_for(n, 256), (unsigned)count), 256, 0, s>>>(jobs, n);
}
void launch_d2f_batch(const XferJob *jobs, int64_t n, int count, cudaStream_t s)
{
    if (count > 0 && n) d2f_batch_kernel<<<dim3(blocks_for(n, 256), (unsigned)count), 256, 0, s>>>(jobs, n);
}
void launch_df_pull_batch(const XferJob *jobs, int64_t n, int level, int count, cudaStream_t s)
{
    if (count > 0 && n) df_pull_batch_kernel<<<dim3(blocks_for(n, 256), (unsigned)count), 256, 0, s>>>(jobs, n, level);
}
void launch_df_push_batch(const XferJob *jobs, int64_t n, int level, int count, cudaStream_t s)
{
    if (count > 0 && n) df_push_batch_kernel<<<count, 256, 0, s>>>(jobs, n, level);
}

template void launch_tiny_batch<float>(const BatchJob<float> *, int, int, cudaStream_t);
template void launch_tiny_batch<double>(const BatchJob<double> *, int, int, cudaStream_t);
template void launch_tiny_batch<df>(const BatchJob<df> *, int, int, cudaStream_t);
template void launch_colour_batch<float>(const BatchJob<float> *, int, int, int, int, cudaStream_t);
template void launch_colour_batch<double>(const BatchJob<double> *, int, int, int, int, cudaStream_t);
template void launch_colour_batch<df>(const BatchJob<df> *, int, int, int, int, cudaStream_t);
template void launch_prolong_add_batch<float>(const XferJob *, int, int, cudaStream_t);
template void launch_prolong_add_batch<double>(const XferJob *, int, int, cudaStream_t);

#define EPR_INSTANTIATE(D, R)                                                                          \
    template void launch_energy<D, R>(const LevelPtrs<R> &, const R *, const Reduce &, cudaStream_t);   \
    template void launch_quadfit<D, R>(const LevelPtrs<R> &, const R *, double *, cudaStream_t);        \
    template void launch_grad_norm<D, R>(const LevelPtrs<R> &, const R *, const Reduce &, cudaStream_t); \
    template void launch_gs_colour<D, R>(const LevelPtrs<R> &, int, unsigned int *, cudaStream_t, int); \
    template int launch_gs_sweeps<D, R>(const LevelPtrs<R> &, int, unsigned int *, cudaStream_t, int, int64_t); \
    template void launch_gn_matvec<D, R>(const LevelPtrs<R> &, const R *, const R *, R *, cudaStream_t); \
    template void launch_prolong<D, R>(int, const R *, R *, int, cudaStream_t, const uint8_t *);                         \
    template void launch_restrict<D, R>(int, const R *, R *, cudaStream_t);

EPR_INSTANTIATE(3, double)
EPR_INSTANTIATE(3, float)
EPR_INSTANTIATE(4, double)
EPR_INSTANTIATE(4, float)
template void launch_scale<double>(double *, int64_t, double, cudaStream_t);
template void launch_scale<float>(float *, int64_t, double, cudaStream_t);
template void launch_axpy<double>(double *, const double *, int64_t, double, cudaStream_t);
template void launch_axpy<float>(float *, const float *, int64_t, double, cudaStream_t);

}  // namespace epr
