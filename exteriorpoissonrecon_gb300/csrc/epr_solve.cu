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

// Quadratic model of E(x + s e_i, y + t e_i): q = (Q20, Q02, Q11, Q10, Q01)
template <int D, typename Real>
__device__ __forceinline__ void node_fit(const LevelPtrs<Real> &L, const Grid<D> &g, const NodeCtx<D> &nc, int64_t i,
                                         const Real *xy, Real *q)
{
    Real h[5] = {0, 0, 0, 0, 0};
#pragma unroll 1
    for (int A = 0; A < (1 << D); A++)
    {
        Real x[1 << D], y[1 << D];
        if (gather_element<D, Real>(g, nc, i, A, xy, x, y)) element_fit<D, Real>(x, y, A, h);
    }
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

// Paired Gauss-Seidel update of node j of a parity colour.
template <int D, typename Real>
__device__ __forceinline__ void gs_update(const LevelPtrs<Real> &L, const Grid<D> &g, const Colour<D> &col, int64_t j, unsigned int *err)
{
    NodeCtx<D> nc;
    col.node(j, nc.I);
#pragma unroll
    for (int d = 0; d < D; d++) nc.stride[d] = g.stride(d);
    int64_t i = g.node(nc.I);
    Real q[5];
    node_fit<D, Real>(L, g, nc, i, L.xy, q);
    // H = [[2 Q20, Q11], [Q11, 2 Q02]], grad = (Q10, Q01); step = -H^{-1} grad / 2
    Real h00 = (Real)2 * q[0], h11 = (Real)2 * q[1], h01 = q[2];
    Real det = h00 * h11 - h01 * h01;
    if (fabs((double)det) > 1e-20)
    {
        Real p0 = -(h11 * q[3] - h01 * q[4]) / det / (Real)2;
        Real p1 = -(-h01 * q[3] + h00 * q[4]) / det / (Real)2;
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
__global__ void __launch_bounds__(kThreads) gs_colour_kernel(LevelPtrs<Real> L, Colour<D> col, unsigned int *err)
{
    Grid<D> g(L.level);
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= col.n) return;
    gs_update<D, Real>(L, g, col, j, err);
}

// All sweeps of a small level in one thread block: the colours follow each other behind a block
// barrier, which also makes each colour's writes visible to the next.  Used for the coarse levels
// of the cascadic schedule, whose thousands of tiny sweeps would otherwise be bound by launch
// latency.
constexpr int kPersistentThreads = 256;
template <int D, typename Real>
__global__ void __launch_bounds__(kPersistentThreads) gs_level_kernel(LevelPtrs<Real> L, int iters, unsigned int *err)
{
    Grid<D> g(L.level);
    for (int it = 0; it < iters; it++)
        for (int c = 0; c < (1 << D); c++)
        {
            Colour<D> col(g, c);
            for (int64_t j = threadIdx.x; j < col.n; j += blockDim.x) gs_update<D, Real>(L, g, col, j, err);
            __syncthreads();
        }
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
__global__ void prolong_kernel(int coarseLevel, const Real *coarse, Real *fine, int add)
{
    Grid<D> gc(coarseLevel), gf(coarseLevel + 1);
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= gf.N) return;
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
void launch_quadfit(const LevelPtrs<Real> &L, const Real *xy, double *out, cudaStream_t s)
{
    Grid<D> g(L.level);
    quadfit_kernel<D, Real><<<blocks_for(g.N), kThreads, 0, s>>>(L, xy, out);
}

template <int D, typename Real>
void launch_gs_colour(const LevelPtrs<Real> &L, int colour, unsigned int *err, cudaStream_t s)
{
    Grid<D> g(L.level);
    Colour<D> col(g, colour);
    if (col.n == 0) return;
    gs_colour_kernel<D, Real><<<blocks_for(col.n), kThreads, 0, s>>>(L, col, err);
}

template <int D, typename Real>
int launch_gs_sweeps(const LevelPtrs<Real> &L, int iters, unsigned int *err, cudaStream_t s)
{
    Grid<D> g(L.level);
    if (iters <= 0) return 0;
    if (g.N <= kPersistentMaxNodes)
    {
        gs_level_kernel<D, Real><<<1, kPersistentThreads, 0, s>>>(L, iters, err);
        return 1;
    }
    int n = 0;
    for (int it = 0; it < iters; it++)
        for (int c = 0; c < (1 << D); c++) { launch_gs_colour<D, Real>(L, c, err, s); n++; }
    return n;
}

template <int D, typename Real>
void launch_gn_matvec(const LevelPtrs<Real> &L, const Real *xy, const Real *dxy, Real *out, cudaStream_t s)
{
    Grid<D> g(L.level);
    gn_matvec_kernel<D, Real><<<blocks_for(g.N), kThreads, 0, s>>>(L, xy, dxy, out);
}

template <int D, typename Real>
void launch_prolong(int coarseLevel, const Real *coarse, Real *fine, int add, cudaStream_t s)
{
    Grid<D> gf(coarseLevel + 1);
    prolong_kernel<D, Real><<<blocks_for(gf.N, 256), 256, 0, s>>>(coarseLevel, coarse, fine, add);
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
void launch_convert_d2f(const double *in, float *out, int64_t n, cudaStream_t st)
{
    if (n) d2f_kernel<<<blocks_for(n, 256), 256, 0, st>>>(in, out, n);
}
void launch_convert_f2d(const float *in, double *out, int64_t n, cudaStream_t st)
{
    if (n) f2d_kernel<<<blocks_for(n, 256), 256, 0, st>>>(in, out, n);
}

#define EPR_INSTANTIATE(D, R)                                                                          \
    template void launch_energy<D, R>(const LevelPtrs<R> &, const R *, const Reduce &, cudaStream_t);   \
    template void launch_quadfit<D, R>(const LevelPtrs<R> &, const R *, double *, cudaStream_t);        \
    template void launch_gs_colour<D, R>(const LevelPtrs<R> &, int, unsigned int *, cudaStream_t);      \
    template int launch_gs_sweeps<D, R>(const LevelPtrs<R> &, int, unsigned int *, cudaStream_t);       \
    template void launch_gn_matvec<D, R>(const LevelPtrs<R> &, const R *, const R *, R *, cudaStream_t); \
    template void launch_prolong<D, R>(int, const R *, R *, int, cudaStream_t);                         \
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
