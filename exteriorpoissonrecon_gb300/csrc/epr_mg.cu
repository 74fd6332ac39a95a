// Linear multigrid and the solvers built on it.
//
// Reference correspondence:
//   linear GS sweep     GSRelaxer::operator()(b, x, mcIndices)        MG.h:57-72
//   V-cycle             MGSolver ctor (Galerkin hierarchy) / vCycle   MG.h:81-187
//   half-step systems   quadraticApproximation1/2 as AlternatingSolve uses them
//                                                                     ExteriorPoissonSolvers.h:96-131
//   alternating solve   AlternatingSolve                              ExteriorPoissonSolvers.h:86-154
//   bi-quadratic fit    SingleCycleCascadicSystemEnergy::biQuadraticFit SystemEnergy.h:499-540
//   line searches       stepSize / newtonUpdate                       SystemEnergy.h:256-303
//
// Layout.  The Galerkin hierarchy is built in double from natural offset-major column stencils
// (coef[o * N + i]).  Each level is then re-laid out *colour-blocked* for relaxation: the nodes of
// parity colour c are numbered j = 0 .. n_c - 1 (axis 0 slowest) and coefficient o of node j sits
// at block_c + o * n_c + j, so one colour sweep streams its own coefficients contiguously (the
// natural layout would touch every other 32-byte sector).  Vectors stay in natural order.  In the
// float mode the colour-blocked copies are float, the coarsest level (resolution 1) is solved in
// double, and the finest-level residual and update are double (iterative refinement), so a V-cycle
// of M x = b computes x += V(b - M x) with V the float V-cycle of the residual equation from zero.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epr.h"
#include "epr_common.cuh"
#include "epr_context.h"
#include "epr_element.cuh"
#include "epr_kernels.h"
#include "epr_mg.h"

namespace epr {

namespace {

constexpr int kThreads = 256;
inline unsigned int blocks(int64_t n, int t = kThreads) { return (unsigned int)((n + t - 1) / t); }

template <int D>
struct ColourBlocks
{
    int64_t base[1 << D];   // first coefficient of colour c's block
    int64_t count[1 << D];  // nodes of colour c
};

template <int D>
ColourBlocks<D> colour_blocks(int level)
{
    Grid<D> g(level);
    ColourBlocks<D> cb;
    int64_t at = 0;
    for (int c = 0; c < (1 << D); c++)
    {
        Colour<D> col(g, c);
        cb.base[c] = at;
        cb.count[c] = col.n;
        at += col.n * Dims<D>::S;
    }
    return cb;
}

// The multigrid's colour-blocked stencils in 16-byte vectors: coefficient o of the j-th node of
// colour c sits at base[c] + ((o / W) n_c + j) W + o % W with W = 16 / sizeof(Real), a node's last
// vector padded with zeros, so that a thread loads its node's column with ceil(S / W) 128-bit
// loads (consecutive threads, consecutive vectors) instead of S scalar ones.
template <int D, typename Real>
struct VecLayout
{
    static constexpr int W = 16 / (int)sizeof(Real);
    static constexpr int G = (Dims<D>::S + W - 1) / W;
    using Vec = typename std::conditional<sizeof(Real) == 4, float4, double2>::type;
};

template <int D, typename Real>
ColourBlocks<D> colour_blocks_vec(int level)
{
    Grid<D> g(level);
    ColourBlocks<D> cb;
    int64_t at = 0;
    for (int c = 0; c < (1 << D); c++)
    {
        Colour<D> col(g, c);
        cb.base[c] = at;
        cb.count[c] = col.n;
        at += col.n * VecLayout<D, Real>::G * VecLayout<D, Real>::W;
    }
    return cb;
}

// neighbour of node i at stencil offset o, or -1 outside the grid
template <int D>
__device__ __forceinline__ int64_t neighbour(const Grid<D> &g, const int *I, int64_t i, int o)
{
    int64_t j = i, s = 1;
    int t = o;
#pragma unroll
    for (int d = D - 1; d >= 0; d--)
    {
        int off = t % 3 - 1;
        t /= 3;
        int q = I[d] + off;
        if (q < 0 || q > g.r) return -1;
        j += off * s;
        s *= g.r + 1;
    }
    return j;
}

// natural offset-major double stencil -> colour-blocked Real stencil; grid.y = colour
template <int D, typename Real>
__global__ void to_colour_blocks_kernel(int level, const double *M, ColourBlocks<D> cb, Real *out)
{
    const int c = blockIdx.y;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= cb.count[c]) return;
    Grid<D> g(level);
    Colour<D> col(g, c);
    int I[D];
    col.node(j, I);
    const int64_t i = g.node(I);
    Real *dst = out + cb.base[c] + j;
    const int64_t n = cb.count[c];
    for (int o = 0; o < Dims<D>::S; o++) dst[o * n] = (Real)M[(int64_t)o * g.N + i];
}

// natural offset-major double stencil -> the multigrid's vector colour blocks; grid.y = colour
template <int D, typename Real>
__global__ void to_colour_blocks_vec_kernel(int level, const double *M, ColourBlocks<D> cb, Real *out)
{
    using V = VecLayout<D, Real>;
    const int c = blockIdx.y;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= cb.count[c]) return;
    Grid<D> g(level);
    Colour<D> col(g, c);
    int I[D];
    col.node(j, I);
    const int64_t i = g.node(I);
    Real *dst = out + cb.base[c];
    const int64_t n = cb.count[c];
    for (int o = 0; o < V::G * V::W; o++)
        dst[((int64_t)(o / V::W) * n + j) * V::W + o % V::W] = o < Dims<D>::S ? (Real)M[(int64_t)o * g.N + i] : (Real)0;
}

// component d of stencil offset o (axis 0 slowest), in {-1, 0, 1}
template <int D>
__host__ __device__ constexpr int offset_of(int o, int d)
{
    for (int k = D - 1; k > d; k--) o /= 3;
    return o % 3 - 1;
}

// Node I (and its index) of the j-th node of a parity colour; 32-bit arithmetic (every supported
// grid has fewer than 2^32 nodes)
template <int D>
__device__ __forceinline__ uint32_t colour_node(const Colour<D> &col, const uint32_t *st, uint32_t j, int *I)
{
    uint32_t i = 0;
#pragma unroll
    for (int d = D - 1; d >= 0; d--)
    {
        const uint32_t c = (uint32_t)col.cnt[d];
        const uint32_t q = j / c;
        I[d] = 2 * (int)(j - q * c) + col.par[d];
        i += (uint32_t)I[d] * st[d];
        j = q;
    }
    return i;
}

// sum_o M[o] x[i + off(o)] over the stencil of node i: interior nodes take the unrolled path with
// compile-time offsets, boundary nodes check every neighbour.
// coefficient load: read-only path, or streaming (evict-first: the coefficients are read once per
// sweep, the x vector is what should stay cached)
template <bool Streaming, typename Real>
__device__ __forceinline__ Real coef_load(const Real *p)
{
    if constexpr (Streaming) return __ldcs(p);
    else return __ldg(p);
}
template <bool Streaming, typename Vec>
__device__ __forceinline__ Vec vec_load(const Vec *p)
{
    if constexpr (Streaming) return __ldcs(p);
    else return __ldg(p);
}
template <typename Vec, typename Real>
__device__ __forceinline__ Real vec_at(const Vec &v, int e)
{
    if constexpr (sizeof(Real) == 4) return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
    else return e == 0 ? v.x : v.y;
}

// sum_o M[o] x[i + off(o)] over the stencil of node i, the coefficients from the vector colour
// blocks (Mc = the colour's block); interior nodes take the unrolled path with compile-time
// offsets, boundary nodes check every neighbour.  centre receives M[centre].  The sum runs over o
// in increasing order, as with scalar loads.
template <int D, typename Real, bool Streaming = false>
__device__ __forceinline__ Real stencil_dot(const Real *__restrict__ Mc, int64_t n, int64_t j, const Real *x, uint32_t i,
                                            const int *I, const uint32_t *st, int r, Real &centre)
{
    using V = VecLayout<D, Real>;
    using Vec = typename V::Vec;
    constexpr int S = Dims<D>::S;
    const Vec *Mv = reinterpret_cast<const Vec *>(Mc) + j;
    bool interior = true;
#pragma unroll
    for (int d = 0; d < D; d++) interior = interior && I[d] > 0 && I[d] < r;
    Real s = 0;
    centre = 0;
#pragma unroll
    for (int gv = 0; gv < V::G; gv++)
    {
        const Vec v = vec_load<Streaming>(Mv + (int64_t)gv * n);
#pragma unroll
        for (int e = 0; e < V::W; e++)
        {
            const int o = gv * V::W + e;
            if (o >= S) break;
            const Real m = vec_at<Vec, Real>(v, e);
            if (o == Dims<D>::CENTER) centre = m;
            int64_t k = (int64_t)i;
            bool ok = true;
#pragma unroll
            for (int d = 0; d < D; d++)
            {
                const int off = offset_of<D>(o, d);
                if (!interior)
                {
                    const int q = I[d] + off;
                    ok = ok && q >= 0 && q <= r;
                }
                k += (int64_t)off * (int64_t)st[d];
            }
            if (interior || ok) s += m * x[k];
        }
    }
    return s;
}

template <int D>
__device__ __forceinline__ void node_strides(int r, uint32_t *st)
{
    st[D - 1] = 1;
#pragma unroll
    for (int d = D - 2; d >= 0; d--) st[d] = st[d + 1] * (uint32_t)(r + 1);
}

// x_i += (b_i - sum_j M(j, i) x_j) / M(i, i) for the nodes of one colour (the GSRelaxer update,
// which reads column i of M; M is symmetric)
template <int D, typename Real, int MinBlocks = 1, bool Streaming = false>
__global__ void __launch_bounds__(kThreads, MinBlocks) linear_gs_colour_kernel(int level, int colour, const Real *__restrict__ Mc,
                                                                                int64_t n, const Real *__restrict__ b, Real *x)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int r = 1 << level;
    Grid<D> g(level);
    Colour<D> col(g, colour);
    uint32_t st[D];
    node_strides<D>(r, st);
    int I[D];
    const uint32_t i = colour_node<D>(col, st, (uint32_t)j, I);
    Real centre;
    const Real s = stencil_dot<D, Real, Streaming>(Mc, n, j, x, i, I, st, r, centre);
    x[i] += (__ldg(b + i) - s) / centre;
}

// r = b - M x over every node, colour-blocked coefficients; grid.y = colour
template <int D, typename Real>
__global__ void __launch_bounds__(kThreads) residual_cb_kernel(int level, const Real *M, ColourBlocks<D> cb, const Real *b,
                                                                const Real *x, Real *r)
{
    const int c = blockIdx.y;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t n = cb.count[c];
    if (j >= n) return;
    const int res = 1 << level;
    Grid<D> g(level);
    Colour<D> col(g, c);
    uint32_t st[D];
    node_strides<D>(res, st);
    int I[D];
    const uint32_t i = colour_node<D>(col, st, (uint32_t)j, I);
    Real centre;
    r[i] = b[i] - stencil_dot<D, Real>(M + cb.base[c], n, j, x, i, I, st, res, centre);
}

// r = b - M x with the natural double stencil (the refinement residual of the float mode)
template <int D>
__global__ void __launch_bounds__(kThreads) residual_nat_kernel(int level, const double *M, const double *b, const double *x,
                                                                 float *r)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    Grid<D> g(level);
    if (i >= g.N) return;
    int I[D];
    g.node(i, I);
    double s = 0;
#pragma unroll 27
    for (int o = 0; o < Dims<D>::S; o++)
    {
        int64_t k = neighbour<D>(g, I, i, o);
        if (k >= 0) s += M[o * g.N + i] * x[k];
    }
    r[i] = (float)(b[i] - s);
}

// coarse = P^T fine (scalar; the sum runs in the wider of the two precisions)
template <int D, typename RF, typename RC>
__global__ void restrict1_kernel(int coarseLevel, const RF *fine, RC *coarse)
{
    using Real = decltype(RF() + RC());
    Grid<D> gc(coarseLevel), gf(coarseLevel + 1);
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= gc.N) return;
    int I[D];
    gc.node(i, I);
    Real s = 0;
    for (int o = 0; o < Dims<D>::S; o++)
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
        if (ok) s += w * (Real)fine[gf.node(F)];
    }
    coarse[i] = (RC)s;
}

// fine += P coarse (scalar)
template <int D, typename RC, typename RF>
__global__ void prolong_add1_kernel(int coarseLevel, const RC *coarse, RF *fine)
{
    using Real = decltype(RF() + RC());
    Grid<D> gc(coarseLevel), gf(coarseLevel + 1);
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= gf.N) return;
    int F[D];
    gf.node(i, F);
    Real s = 0;
#pragma unroll
    for (int c = 0; c < (1 << D); c++)
    {
        bool use = true;
        Real w = 1;
        int I[D];
#pragma unroll
        for (int d = 0; d < D; d++)
        {
            int bit = (c >> d) & 1;
            if (F[d] & 1) { I[d] = (F[d] >> 1) + bit; w *= (Real)0.5; }
            else { I[d] = F[d] >> 1; if (bit) use = false; }
        }
        if (use) s += w * (Real)coarse[gc.node(I)];
    }
    fine[i] = (RF)((Real)fine[i] + s);
}

// Exact solve at resolution 1 (2^D nodes) by a dense LDL^T factorisation in double, one thread;
// stands in for the SimplicialLDLT of the coarsest MGSolver level (MG.h:105, 131).
template <int D, typename Real>
__global__ void coarse_solve_kernel(const double *M, const Real *b, Real *x)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    constexpr int N = 1 << D;
    Grid<D> g(0);
    double A[N][N], L[N][N], Dg[N], z[N];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) { A[i][j] = 0; L[i][j] = 0; }
    for (int i = 0; i < N; i++)
    {
        int I[D];
        g.node(i, I);
        for (int o = 0; o < Dims<D>::S; o++)
        {
            int64_t k = neighbour<D>(g, I, i, o);
            if (k >= 0) A[k][i] = M[(int64_t)o * N + i];
        }
    }
    for (int j = 0; j < N; j++)
    {
        double d = A[j][j];
        for (int k = 0; k < j; k++) d -= L[j][k] * L[j][k] * Dg[k];
        Dg[j] = d;
        L[j][j] = 1.;
        for (int i = j + 1; i < N; i++)
        {
            double v = A[i][j];
            for (int k = 0; k < j; k++) v -= L[i][k] * L[j][k] * Dg[k];
            L[i][j] = v / d;
        }
    }
    for (int i = 0; i < N; i++)
    {
        double v = (double)b[i];
        for (int k = 0; k < i; k++) v -= L[i][k] * z[k];
        z[i] = v;
    }
    for (int i = 0; i < N; i++) z[i] /= Dg[i];
    double xs[N];
    for (int ii = N - 1; ii >= 0; ii--)
    {
        double v = z[ii];
        for (int k = ii + 1; k < N; k++) v -= L[k][ii] * xs[k];
        xs[ii] = v;
    }
    for (int i = 0; i < N; i++) x[i] = (Real)xs[i];
}

template <typename Real>
__global__ void component_get_kernel(const double *xy, int which, int64_t n, Real *v)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = (Real)xy[2 * i + which];
}
__global__ void component_set_kernel(double *xy, int which, int64_t n, const double *v)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) xy[2 * i + which] = v[i];
}
__global__ void add_f2d_kernel(double *y, const float *x, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] += (double)x[i];
}

// ---------------------------------------------------------------------------------------------
// Half-step systems of the alternating solve.  For a fixed field f the wedge is linear in the
// other one: |W(f, v)|^2 = v^T G_f v with G_f(j, i) = int <W(f, phi_j), W(f, phi_i)>.  The Gram
// column of node i is integrated per incident element in the canonical orientation (node i at
// corner 0; mirroring flips the sign of both W(f, phi_j) and W(f, phi_i), so each product keeps
// its sign) with the same exact Gauss rule as the energy.
// ---------------------------------------------------------------------------------------------
template <int D, int K, typename Real>
__device__ __forceinline__ void component_gram(const Real *f, Real *loc)
{
    using Cp = Component<D, K>;
    constexpr int M = Cp::M;
    constexpr int NG = ipow(3, M);
    constexpr int C = 1 << D;
    Real fP[2 * NG], fQ[2 * NG];
    derivative_table<D, K, true, Real>(f, fP);
    derivative_table<D, K, false, Real>(f, fQ);
#pragma unroll
    for (int go = 0; go < NG; go++)
    {
        const Real wo = (Real)other_weight<M>(go);
#pragma unroll
        for (int gp = 0; gp < 2; gp++)
#pragma unroll
            for (int gq = 0; gq < 2; gq++)
            {
                const Real w = (Real)(Gauss::W2(gp) * Gauss::W2(gq)) * wo;
                const Real xp = fP[gq * NG + go], xq = fQ[gp * NG + go];
                Real V[C];
#pragma unroll
                for (int B = 0; B < C; B++)
                {
                    const int bP = cbit<D>(B, Cp::P), bQ = cbit<D>(B, Cp::Q);
                    Real lo;
                    if constexpr (M == 1) lo = hat3<Real>(cbit<D>(B, Cp::other(0)), go);
                    else lo = hat3<Real>(cbit<D>(B, Cp::other(0)), go / 3) * hat3<Real>(cbit<D>(B, Cp::other(1)), go % 3);
                    const Real phP = (bP ? (Real)1 : (Real)-1) * hat2<Real>(bQ, gq) * lo;
                    const Real phQ = (bQ ? (Real)1 : (Real)-1) * hat2<Real>(bP, gp) * lo;
                    V[B] = phP * xq - xp * phQ;
                }
                const Real wV0 = w * V[0];
#pragma unroll
                for (int B = 0; B < C; B++) loc[B] += wV0 * V[B];
            }
    }
}

template <int D, typename Real>
__device__ __noinline__ void element_gram_canonical(const Real *f, Real *loc)
{
#pragma unroll
    for (int B = 0; B < (1 << D); B++) loc[B] = 0;
    component_gram<D, 0, Real>(f, loc);
    component_gram<D, 1, Real>(f, loc);
    component_gram<D, 2, Real>(f, loc);
    if constexpr (D == 4)
    {
        component_gram<D, 3, Real>(f, loc);
        component_gram<D, 4, Real>(f, loc);
        component_gram<D, 5, Real>(f, loc);
    }
}

// sum_j B(j, i) v_j over the off-diagonal neighbours (natural offset-major B)
template <int D>
__device__ __forceinline__ double b_column_dot(const Grid<D> &g, const int *I, int64_t i, const double *B, const double *xy,
                                               int comp)
{
    double s = 0;
    for (int o = 0; o < Dims<D>::S; o++)
    {
        if (o == Dims<D>::CENTER) continue;
        int64_t k = neighbour<D>(g, I, i, o);
        if (k >= 0) s += B[(int64_t)o * g.N + i] * xy[2 * k + comp];
    }
    return s;
}

// M = 2 (G_f + A) and b of one half-step: which 1 -> y free (f = x, b = 2 B x), which 0 -> x
// free (f = y, b = 2 B^T y); B x = -(column sums) since B is antisymmetric.
// The Gram integrals run in Real (float in the float mode: the half-step system only steers the
// outer iteration, whose gradient is evaluated in double); M and b are written in double.
template <int D, typename Real>
__global__ void __launch_bounds__(128) alternating_system_kernel(int level, const double *xy, int which, const double *A,
                                                                  const double *B, double *M, double *b)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    Grid<D> g(level);
    if (i >= g.N) return;
    constexpr int S = Dims<D>::S;
    int I[D];
    g.node(i, I);
    const int fc = which ? 0 : 1;  // component of the fixed field
    Real col[S];
#pragma unroll
    for (int o = 0; o < S; o++) col[o] = 0;
#pragma unroll 1
    for (int mirror = 0; mirror < (1 << D); mirror++)
    {
        // element whose corner `mirror` is node i (bit D-1-d of mirror: node is the upper corner on axis d)
        bool ok = true;
        for (int d = 0; d < D; d++)
        {
            int e = I[d] - cbit<D>(mirror, d);
            ok = ok && e >= 0 && e < g.r;
        }
        if (!ok) continue;
        Real f[1 << D], loc[1 << D];
#pragma unroll
        for (int cc = 0; cc < (1 << D); cc++)
        {
            int64_t j = i, s = 1;
            for (int d = D - 1; d >= 0; d--)
            {
                int step = cbit<D>(cc, d);
                j += (cbit<D>(mirror, d) ? -step : step) * s;
                s *= g.r + 1;
            }
            f[cc] = (Real)xy[2 * j + fc];
        }
        element_gram_canonical<D, Real>(f, loc);
#pragma unroll
        for (int B2 = 0; B2 < (1 << D); B2++)
        {
            int o = 0;
            for (int d = 0; d < D; d++) o = o * 3 + 1 + (cbit<D>(mirror, d) ? -cbit<D>(B2, d) : cbit<D>(B2, d));
            col[o] += loc[B2];
        }
    }
    const double sc = (D == 3 ? (double)g.r : 1.0) * 0.5;
    for (int o = 0; o < S; o++) M[(int64_t)o * g.N + i] = 2. * ((double)col[o] * sc + A[(int64_t)o * g.N + i]);
    const double bd = b_column_dot<D>(g, I, i, B, xy, which ? 0 : 1);
    b[i] = which ? -2. * bd : 2. * bd;
}

// ---------------------------------------------------------------------------------------------
// Bi-quadratic fit: 10 wedge products per element and 10 stencil forms per node, block sums
// ---------------------------------------------------------------------------------------------
constexpr int kBQ = 20;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int D, int K>
__device__ __forceinline__ void component_biquad(const double *x, const double *y, const double *dx, const double *dy,
                                                 double *acc)
{
    constexpr int NG = ipow(3, D - 2);
    double xP[2 * NG], xQ[2 * NG], yP[2 * NG], yQ[2 * NG], XP[2 * NG], XQ[2 * NG], YP[2 * NG], YQ[2 * NG];
    derivative_table<D, K, true, double>(x, xP);
    derivative_table<D, K, false, double>(x, xQ);
    derivative_table<D, K, true, double>(y, yP);
    derivative_table<D, K, false, double>(y, yQ);
    derivative_table<D, K, true, double>(dx, XP);
    derivative_table<D, K, false, double>(dx, XQ);
    derivative_table<D, K, true, double>(dy, YP);
    derivative_table<D, K, false, double>(dy, YQ);
#pragma unroll
    for (int gp = 0; gp < 2; gp++)
#pragma unroll
        for (int gq = 0; gq < 2; gq++)
#pragma unroll
            for (int go = 0; go < NG; go++)
            {
                const double w = Gauss::W2(gp) * Gauss::W2(gq) * other_weight<D - 2>(go);
                const int ip = gq * NG + go, iq = gp * NG + go;
                // W(u, v) = d_P v d_Q u - d_P u d_Q v (reference units, the 1/2 folded into the scale)
                const double Wxy = yP[ip] * xQ[iq] - xP[ip] * yQ[iq];
                const double WXy = yP[ip] * XQ[iq] - XP[ip] * yQ[iq];
                const double WxY = YP[ip] * xQ[iq] - xP[ip] * YQ[iq];
                const double WXY = YP[ip] * XQ[iq] - XP[ip] * YQ[iq];
                acc[0] += w * WXY * WXY;
                acc[1] += w * WXY * WXy;
                acc[2] += w * WXY * WxY;
                acc[3] += w * WXy * WXy;
                acc[4] += w * WxY * WxY;
                acc[5] += w * WXy * WxY;
                acc[6] += w * WXY * Wxy;
                acc[7] += w * WXy * Wxy;
                acc[8] += w * WxY * Wxy;
                acc[9] += w * Wxy * Wxy;
            }
}

// xy: current (x, y) pairs; dxy: direction pairs.  A = R + dWeight K; K2 (optional) adds kw K.
template <int D>
__global__ void __launch_bounds__(128) biquad_kernel(int level, const double *xy, const double *dxy, const double *A,
                                                      const double *K2, double kw, const double *B, double *partial)
{
    Grid<D> g(level);
    double acc[kBQ];
#pragma unroll
    for (int k = 0; k < kBQ; k++) acc[k] = 0;
    const int64_t total = g.N > g.NE ? g.N : g.NE;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    {
        if (t < g.NE)
        {
            int E[D];
            g.elem(t, E);
            double x[1 << D], y[1 << D], X[1 << D], Y[1 << D];
            int64_t base = 0;
            for (int d = 0; d < D; d++) base = base * (g.r + 1) + E[d];
#pragma unroll
            for (int c = 0; c < (1 << D); c++)
            {
                int64_t j = base;
                for (int d = 0; d < D; d++) j += cbit<D>(c, d) * g.stride(d);
                x[c] = xy[2 * j];
                y[c] = xy[2 * j + 1];
                X[c] = dxy[2 * j];
                Y[c] = dxy[2 * j + 1];
            }
            component_biquad<D, 0>(x, y, X, Y, acc);
            component_biquad<D, 1>(x, y, X, Y, acc);
            component_biquad<D, 2>(x, y, X, Y, acc);
            if constexpr (D == 4)
            {
                component_biquad<D, 3>(x, y, X, Y, acc);
                component_biquad<D, 4>(x, y, X, Y, acc);
                component_biquad<D, 5>(x, y, X, Y, acc);
            }
        }
        if (t < g.N)
        {
            int I[D];
            g.node(t, I);
            double Adx = 0, Ax = 0, Ady = 0, Ay = 0, Bdy = 0, By = 0;
            for (int o = 0; o < Dims<D>::S; o++)
            {
                int64_t k = neighbour<D>(g, I, t, o);
                if (k < 0) continue;
                double a = A[(int64_t)o * g.N + t];
                if (K2) a += kw * K2[(int64_t)o * g.N + t];
                const double b = B[(int64_t)o * g.N + t];
                Adx += a * dxy[2 * k];
                Ax += a * xy[2 * k];
                Ady += a * dxy[2 * k + 1];
                Ay += a * xy[2 * k + 1];
                Bdy += b * dxy[2 * k + 1];
                By += b * xy[2 * k + 1];
            }
            const double xi = xy[2 * t], yi = xy[2 * t + 1], Xi = dxy[2 * t], Yi = dxy[2 * t + 1];
            acc[10] += Xi * Adx;  // dx A dx
            acc[11] += xi * Adx;  // x A dx
            acc[12] += xi * Ax;   // x A x
            acc[13] += Yi * Ady;  // dy A dy
            acc[14] += yi * Ady;  // y A dy
            acc[15] += yi * Ay;   // y A y
            acc[16] += Xi * Bdy;  // dy^T B dx
            acc[17] += xi * Bdy;  // dy^T B x
            acc[18] += Xi * By;   // y^T B dx
            acc[19] += xi * By;   // y^T B x
        }
    }
    __shared__ double sh[kBQ][4];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kBQ; k++)
    {
        double v = warp_sum(acc[k]);
        if (lane == 0) sh[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < kBQ)
    {
        double s = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sh[threadIdx.x][q];
        partial[(int64_t)blockIdx.x * kBQ + threadIdx.x] = s;
    }
}

__global__ void biquad_finish_kernel(const double *partial, int nblocks, double *out)
{
    const int v = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (v >= kBQ) return;
    double s = 0;
    for (int b = lane; b < nblocks; b += 32) s += partial[(int64_t)b * kBQ + v];
    s = warp_sum(s);
    if (lane == 0) out[v] = s;
}

}  // namespace

template <int D, typename Real>
void launch_to_colour_blocks(int level, const double *M, Real *out, cudaStream_t s)
{
    ColourBlocks<D> cb = colour_blocks<D>(level);
    to_colour_blocks_kernel<D, Real><<<dim3(blocks(cb.count[0]), 1 << D), kThreads, 0, s>>>(level, M, cb, out);
}
template void launch_to_colour_blocks<3, float>(int, const double *, float *, cudaStream_t);
template void launch_to_colour_blocks<3, double>(int, const double *, double *, cudaStream_t);
template void launch_to_colour_blocks<4, float>(int, const double *, float *, cudaStream_t);
template void launch_to_colour_blocks<4, double>(int, const double *, double *, cudaStream_t);

// =============================================================================================
// Host side
// =============================================================================================

// Levels with fewer nodes than this relax in double even in the float mode: they cost nothing,
// and the coarse Galerkin systems are the ill-conditioned ones, where a float right-hand side
// would be amplified by the exact coarse solve.
constexpr int64_t kFloatMinNodes = 1 << 15;

// Per-level storage of the linear multigrid
struct MGLevel
{
    int64_t N = 0;
    bool f32 = false;       // the level relaxes in float
    double *M64 = nullptr;  // natural offset-major stencil (double)
    void *Mcb = nullptr;    // colour-blocked stencil (the level's precision)
    void *x = nullptr, *b = nullptr, *r = nullptr;  // the level's vectors
};

struct MGHierarchy
{
    int top = -1;
    int mode = -1;  // precision and double band the levels were allocated for
    std::vector<MGLevel> L;
    double *x64 = nullptr, *b64 = nullptr;  // finest-level double vectors (solution, right-hand side)
};

void release_mg(Context &c)
{
    if (!c.mg) return;
    for (MGLevel &l : c.mg->L)
    {
        c.release(l.M64); c.release(l.Mcb); c.release(l.x); c.release(l.b); c.release(l.r);
    }
    c.release(c.mg->x64);
    c.release(c.mg->b64);
    delete c.mg;
    c.mg = nullptr;
}

// values per node of the vector colour blocks
template <typename Real>
static size_t vec_stencil_values(int dim)
{
    return dim == 3 ? (size_t)VecLayout<3, Real>::G * VecLayout<3, Real>::W : (size_t)VecLayout<4, Real>::G * VecLayout<4, Real>::W;
}

// (re)allocates the hierarchy for levels 0..top
static bool mg_prepare(Context &c, int top)
{
    const int mode = (c.P.precision * 1024 + c.P.fp64_levels) * 1024 + c.P.fp64_from;
    if (c.mg && c.mg->top >= top && c.mg->mode == mode) return true;
    release_mg(c);
    c.mg = new MGHierarchy;
    MGHierarchy &h = *c.mg;
    h.top = top;
    h.mode = mode;
    h.L.resize(top + 1);
    const size_t S = (size_t)c.stencil();
    for (int l = 0; l <= top; l++)
    {
        MGLevel &m = h.L[l];
        m.N = c.nodes(l);
        m.f32 = c.lvl32(l) && m.N >= kFloatMinNodes;
        const size_t rs = m.f32 ? sizeof(float) : sizeof(double);
        if (!c.alloc((void **)&m.M64, sizeof(double) * S * m.N, "alloc mg stencil") ||
            !c.alloc(&m.Mcb, (m.f32 ? vec_stencil_values<float>(c.dim) : vec_stencil_values<double>(c.dim)) * rs * m.N,
                     "alloc mg stencil") ||
            !c.alloc(&m.x, rs * m.N, "alloc mg x") ||
            !c.alloc(&m.b, rs * m.N, "alloc mg b") || !c.alloc(&m.r, rs * m.N, "alloc mg r"))
            return false;
    }
    const int64_t N = h.L[top].N;
    return c.alloc((void **)&h.x64, sizeof(double) * N, "alloc mg x64") && c.alloc((void **)&h.b64, sizeof(double) * N, "alloc mg b64");
}

template <typename F>
static int mg_dim(Context &c, F &&f)
{
    if (c.dim == 3) return f(std::integral_constant<int, 3>{});
    return f(std::integral_constant<int, 4>{});
}

// calls f(float{}) or f(double{})
template <typename F>
static void with_real(bool f32, F &&f)
{
    if (f32) f(0.0f);
    else f(0.0);
}

// Galerkin hierarchy of L[top].M64 down to level 0 and the colour-blocked copies of levels
// lo..top (lo = top for relaxation only)
static bool mg_build(Context &c, int top, int lo)
{
    MGHierarchy &h = *c.mg;
    mg_dim(c, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        if (lo < top)
            for (int l = top; l > 0; l--) launch_galerkin<D>(l, h.L[l].M64, h.L[l - 1].M64, c.stream);
        for (int l = std::max(lo, 1); l <= top; l++)
        {
            with_real(h.L[l].f32, [&](auto rv) {
                using R = decltype(rv);
                ColourBlocks<D> cb = colour_blocks_vec<D, R>(l);
                dim3 grid(blocks(cb.count[0]), 1 << D);
                to_colour_blocks_vec_kernel<D, R><<<grid, kThreads, 0, c.stream>>>(l, h.L[l].M64, cb, (R *)h.L[l].Mcb);
            });
            c.launches++;
        }
        c.launches += (lo < top) ? top : 0;
        return 0;
    });
    return c.launch_ok("mg hierarchy");
}

// variant of the linear GS colour kernel (EPR_LGS_VARIANT): 0 default (32 registers, 8 blocks of 256
// threads per SM, streaming coefficient loads: the coefficients are read once per sweep, the x
// vector stays in L2; depth 8, one colour: 0.060 ms float = 0.78 of the measured copy bandwidth,
// 0.187 ms double), 1 the same, 2 no register cap (0.094 / 0.204 ms), 3 32 registers + read-only
// loads (0.063 / 0.187 ms)
static int lgs_variant()
{
    static const int v = [] {
        const char *e = getenv("EPR_LGS_VARIANT");
        return e ? atoi(e) : 0;
    }();
    return v;
}

template <int D, typename Real>
static void launch_lgs_colour(int l, int col, const Real *Mc, int64_t n, const Real *b, Real *x, cudaStream_t s)
{
    const int v = lgs_variant();
    if (v == 1)
        linear_gs_colour_kernel<D, Real, 8, true><<<blocks(n), kThreads, 0, s>>>(l, col, Mc, n, b, x);
    else if (v == 2)
        linear_gs_colour_kernel<D, Real, 1, false><<<blocks(n), kThreads, 0, s>>>(l, col, Mc, n, b, x);
    else if (v == 3)
        linear_gs_colour_kernel<D, Real, 8, false><<<blocks(n), kThreads, 0, s>>>(l, col, Mc, n, b, x);
    else
        linear_gs_colour_kernel<D, Real, 8, true><<<blocks(n), kThreads, 0, s>>>(l, col, Mc, n, b, x);
}

template <int D, typename Real>
static void mg_sweeps(Context &c, int l, const Real *b, Real *x, int iters)
{
    MGLevel &m = c.mg->L[l];
    ColourBlocks<D> cb = colour_blocks_vec<D, Real>(l);
    for (int it = 0; it < iters; it++)
        for (int col = 0; col < (1 << D); col++)
        {
            launch_lgs_colour<D, Real>(l, col, (const Real *)m.Mcb + cb.base[col], cb.count[col], b, x, c.stream);
            c.launches++;
        }
}

// One V-cycle (MGSolver::vCycle, MG.h:150-187) of M x = b on levels 0..top with the vectors of
// L[top] as b and x; every level computes in its own precision.
template <int D>
static void mg_vcycle(Context &c, int top, int iters)
{
    MGHierarchy &h = *c.mg;
    for (int l = top; l > 0; l--)
    {
        MGLevel &m = h.L[l], &mc = h.L[l - 1];
        with_real(m.f32, [&](auto rv) {
            using R = decltype(rv);
            mg_sweeps<D, R>(c, l, (const R *)m.b, (R *)m.x, iters);
            ColourBlocks<D> cb = colour_blocks_vec<D, R>(l);
            residual_cb_kernel<D, R><<<dim3(blocks(cb.count[0]), 1 << D), kThreads, 0, c.stream>>>(
                l, (const R *)m.Mcb, cb, (const R *)m.b, (const R *)m.x, (R *)m.r);
            with_real(mc.f32, [&](auto cv) {
                using RC = decltype(cv);
                restrict1_kernel<D, R, RC><<<blocks(mc.N), kThreads, 0, c.stream>>>(l - 1, (const R *)m.r, (RC *)mc.b);
                cudaMemsetAsync(mc.x, 0, sizeof(RC) * mc.N, c.stream);
            });
        });
        c.launches += 2;
    }
    with_real(h.L[0].f32, [&](auto rv) {
        using R = decltype(rv);
        coarse_solve_kernel<D, R><<<1, 32, 0, c.stream>>>(h.L[0].M64, (const R *)h.L[0].b, (R *)h.L[0].x);
    });
    c.launches++;
    for (int l = 1; l <= top; l++)
    {
        MGLevel &m = h.L[l], &mc = h.L[l - 1];
        with_real(m.f32, [&](auto rv) {
            using R = decltype(rv);
            with_real(mc.f32, [&](auto cv) {
                using RC = decltype(cv);
                prolong_add1_kernel<D, RC, R><<<blocks(m.N), kThreads, 0, c.stream>>>(l - 1, (const RC *)mc.x, (R *)m.x);
            });
            mg_sweeps<D, R>(c, l, (const R *)m.b, (R *)m.x, iters);
        });
        c.launches++;
    }
}

// cycles V-cycles of L[top].M64 x64 = b64 (x64 updated in place).  A float top level relaxes the
// residual equation (residual formed in double) and adds each correction in double.
static bool mg_cycles(Context &c, int top, int iters, int cycles)
{
    MGHierarchy &h = *c.mg;
    MGLevel &m = h.L[top];
    mg_dim(c, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        for (int k = 0; k < cycles; k++)
        {
            if (!m.f32)
            {
                cudaMemcpyAsync(m.x, h.x64, sizeof(double) * m.N, cudaMemcpyDeviceToDevice, c.stream);
                cudaMemcpyAsync(m.b, h.b64, sizeof(double) * m.N, cudaMemcpyDeviceToDevice, c.stream);
                if (top == 0)
                {
                    coarse_solve_kernel<D, double><<<1, 32, 0, c.stream>>>(h.L[0].M64, (const double *)m.b, (double *)m.x);
                    c.launches++;
                }
                else mg_vcycle<D>(c, top, iters);
                cudaMemcpyAsync(h.x64, m.x, sizeof(double) * m.N, cudaMemcpyDeviceToDevice, c.stream);
            }
            else
            {
                residual_nat_kernel<D><<<blocks(m.N), kThreads, 0, c.stream>>>(top, m.M64, h.b64, h.x64, (float *)m.b);
                cudaMemsetAsync(m.x, 0, sizeof(float) * m.N, c.stream);
                mg_vcycle<D>(c, top, iters);
                add_f2d_kernel<<<blocks(m.N), kThreads, 0, c.stream>>>(h.x64, (const float *)m.x, m.N);
                c.launches += 2;
            }
        }
        return 0;
    });
    return c.launch_ok("mg v-cycle");
}

// iters coloured GS sweeps of L[top].M64 x64 = b64 (colour-blocked copy of top must be current)
static bool mg_relax(Context &c, int top, int iters)
{
    MGHierarchy &h = *c.mg;
    MGLevel &m = h.L[top];
    mg_dim(c, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        if (!m.f32)
        {
            mg_sweeps<D, double>(c, top, h.b64, h.x64, iters);
        }
        else
        {
            launch_convert_d2f(h.x64, (float *)m.x, m.N, c.stream);
            launch_convert_d2f(h.b64, (float *)m.b, m.N, c.stream);
            mg_sweeps<D, float>(c, top, (const float *)m.b, (float *)m.x, iters);
            launch_convert_f2d((const float *)m.x, h.x64, m.N, c.stream);
            c.launches += 3;
        }
        return 0;
    });
    return c.launch_ok("mg relax");
}

// host node-major stencil -> L[top].M64, host vectors -> b64 / x64
static bool mg_upload(Context &c, int top, const double *M, const double *b, const double *x)
{
    MGHierarchy &h = *c.mg;
    const int64_t N = h.L[top].N;
    const size_t S = (size_t)c.stencil();
    std::vector<double> t(S * N);
    for (int64_t i = 0; i < N; i++)
        for (size_t o = 0; o < S; o++) t[o * N + i] = M[i * S + o];
    return c.cuda_ok(cudaMemcpyAsync(h.L[top].M64, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, c.stream), "upload M") &&
           c.cuda_ok(cudaMemcpyAsync(h.b64, b, sizeof(double) * N, cudaMemcpyHostToDevice, c.stream), "upload b") &&
           c.cuda_ok(cudaMemcpyAsync(h.x64, x, sizeof(double) * N, cudaMemcpyHostToDevice, c.stream), "upload x") &&
           c.cuda_ok(cudaStreamSynchronize(c.stream), "sync");
}

bool linear_gs(Context &c, int level, const double *M, const double *b, double *x, int iters)
{
    if (!mg_prepare(c, level) || !mg_upload(c, level, M, b, x) || !mg_build(c, level, level) || !mg_relax(c, level, iters)) return false;
    return c.cuda_ok(cudaMemcpyAsync(x, c.mg->x64, sizeof(double) * c.mg->L[level].N, cudaMemcpyDeviceToHost, c.stream), "download x") &&
           c.cuda_ok(cudaStreamSynchronize(c.stream), "sync");
}

bool mg_vcycles(Context &c, int level, const double *M, const double *b, double *x, int iters, int cycles)
{
    if (!mg_prepare(c, level) || !mg_upload(c, level, M, b, x) || !mg_build(c, level, 0) || !mg_cycles(c, level, iters, cycles)) return false;
    return c.cuda_ok(cudaMemcpyAsync(x, c.mg->x64, sizeof(double) * c.mg->L[level].N, cudaMemcpyDeviceToHost, c.stream), "download x") &&
           c.cuda_ok(cudaStreamSynchronize(c.stream), "sync");
}

// assembles the half-step system of `which` from the level's double coefficients into
// L[level].M64 and b64
static bool assemble_system(Context &c, int level, int which)
{
    MGHierarchy &h = *c.mg;
    Level &Lv = c.levels[level];
    mg_dim(c, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        with_real(h.L[level].f32, [&](auto rv) {
            using R = decltype(rv);
            alternating_system_kernel<D, R><<<blocks(Lv.N, 128), 128, 0, c.stream>>>(level, Lv.xy64, which, Lv.A64, Lv.B64,
                                                                                     h.L[level].M64, h.b64);
        });
        return 0;
    });
    c.launches++;
    return c.launch_ok("alternating system");
}

bool alternating_system(Context &c, int level, int which, double *M, double *b)
{
    if (!mg_prepare(c, level) || !c.pull_xy(level) || !assemble_system(c, level, which)) return false;
    const int64_t N = c.levels[level].N;
    const size_t S = (size_t)c.stencil();
    std::vector<double> t(S * N);
    if (!c.cuda_ok(cudaMemcpyAsync(t.data(), c.mg->L[level].M64, sizeof(double) * t.size(), cudaMemcpyDeviceToHost, c.stream), "download M") ||
        !c.cuda_ok(cudaMemcpyAsync(b, c.mg->b64, sizeof(double) * N, cudaMemcpyDeviceToHost, c.stream), "download b") ||
        !c.cuda_ok(cudaStreamSynchronize(c.stream), "sync"))
        return false;
    for (int64_t i = 0; i < N; i++)
        for (size_t o = 0; o < S; o++) M[i * S + o] = t[o * N + i];
    return true;
}

// AlternatingSolve (ExteriorPoissonSolvers.h:86-154) on the level's coefficients: iters rounds of
// (y with x fixed, then x with y fixed), each vCycles V-cycles of gsIters relaxations (MULTIGRID)
// or gsIters * vCycles sweeps (SINGLE_LEVEL).
bool alternating_solve(Context &c, int level, int iters, int vcycles, int gsIters, bool singleLevel)
{
    if (!mg_prepare(c, level) || !c.pull_xy(level)) return false;
    MGHierarchy &h = *c.mg;
    Level &Lv = c.levels[level];
    for (int it = 0; it < iters; it++)
        for (int which = 1; which >= 0; which--)
        {
            if (!assemble_system(c, level, which)) return false;
            component_get_kernel<double><<<blocks(Lv.N), kThreads, 0, c.stream>>>(Lv.xy64, which, Lv.N, h.x64);
            c.launches++;
            bool ok = singleLevel ? (mg_build(c, level, level) && mg_relax(c, level, gsIters * vcycles))
                                  : (mg_build(c, level, 0) && mg_cycles(c, level, gsIters, vcycles));
            if (!ok) return false;
            component_set_kernel<<<blocks(Lv.N), kThreads, 0, c.stream>>>(Lv.xy64, which, Lv.N, h.x64);
            c.launches++;
        }
    if (!c.push_xy(level)) return false;
    return c.launch_ok("alternating solve");
}

// q[i*3+j]: coefficient of s^i t^j of E(x + s dx, y + t dy) at the level's coefficients
bool biquadratic_fit(Context &c, int level, const double *ddxy, bool asReference, double *q)
{
    if (!c.pull_xy(level)) return false;
    Level &Lv = c.levels[level];
    const size_t S = (size_t)c.stencil();
    const int nb = 1024;
    double *partial = nullptr, *out = nullptr, *K = nullptr;
    bool ok = c.alloc((void **)&partial, sizeof(double) * kBQ * nb, "alloc partial") && c.alloc((void **)&out, sizeof(double) * kBQ, "alloc out");
    if (ok && asReference)
        ok = c.alloc((void **)&K, sizeof(double) * S * Lv.N, "alloc K") &&
             c.cuda_ok(cudaMemsetAsync(K, 0, sizeof(double) * S * Lv.N, c.stream), "memset K") && add_dirichlet_to(c, level, K, 1.0);
    double h[kBQ];
    if (ok)
    {
        mg_dim(c, [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            biquad_kernel<D><<<nb, 128, 0, c.stream>>>(level, Lv.xy64, ddxy, Lv.A64, K, 1.0 - c.P.d_weight, Lv.B64, partial);
            biquad_finish_kernel<<<1, 32 * kBQ, 0, c.stream>>>(partial, nb, out);
            return 0;
        });
        c.launches += 2;
        ok = c.launch_ok("biquadratic fit") && c.cuda_ok(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c.stream), "copy") &&
             c.cuda_ok(cudaStreamSynchronize(c.stream), "sync");
    }
    c.release(partial); c.release(out); c.release(K);
    if (!ok) return false;
    const double sc = (c.dim == 3 ? (double)(1 << level) : 1.0) * 0.5;
    double w[10];
    for (int k = 0; k < 10; k++) w[k] = h[k] * sc;
    for (int k = 0; k < 9; k++) q[k] = 0;
    auto Q = [&](int i, int j) -> double & { return q[i * 3 + j]; };
    Q(2, 2) += w[0];
    Q(2, 1) += 2 * w[1];
    Q(1, 2) += 2 * (asReference ? w[6] : w[2]);
    Q(2, 0) += w[3];
    Q(0, 2) += w[4];
    Q(1, 1) += 2 * w[5] + 2 * w[6];
    Q(1, 0) += 2 * w[7];
    Q(0, 1) += 2 * w[8];
    Q(0, 0) += w[9];
    Q(2, 0) += h[10]; Q(1, 0) += 2 * h[11]; Q(0, 0) += h[12];
    Q(0, 2) += h[13]; Q(0, 1) += 2 * h[14]; Q(0, 0) += h[15];
    Q(1, 1) += -2 * h[16]; Q(0, 1) += -2 * h[17]; Q(1, 0) += -2 * h[18]; Q(0, 0) += -2 * h[19];
    Q(0, 0) += c.c;
    return true;
}

// Times `reps` launches of one multigrid kernel at `level` on the context's stream (CUDA events):
//   "lgs"       one colour (0) of the linear Gauss-Seidel sweep on the y half-step system,
//   "residual"  the colour-blocked residual of that system,
//   "assemble"  the half-step system assembly,
//   "biquad"    the bi-quadratic fit reduction along (x, y).
bool time_mg_kernel(Context &c, const char *kernel, int level, int reps, double *ms)
{
    std::string k(kernel);
    if (k != "lgs" && k != "residual" && k != "assemble" && k != "biquad")
    {
        c.fail(EPR_ERR_ARG, "unknown kernel '%s'", kernel);
        return false;
    }
    if (!mg_prepare(c, level) || !c.pull_xy(level) || !assemble_system(c, level, 1) || !mg_build(c, level, level)) return false;
    MGHierarchy &h = *c.mg;
    Level &Lv = c.levels[level];
    MGLevel &m = h.L[level];
    if (m.f32) launch_convert_d2f(h.b64, (float *)m.b, m.N, c.stream);
    else cudaMemcpyAsync(m.b, h.b64, sizeof(double) * m.N, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemsetAsync(m.x, 0, (m.f32 ? sizeof(float) : sizeof(double)) * m.N, c.stream);
    double *partial = nullptr;
    if (k == "biquad" && !c.alloc((void **)&partial, sizeof(double) * kBQ * 1024, "alloc partial")) return false;
    auto run = [&]() {
        mg_dim(c, [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            ColourBlocks<D> cb = m.f32 ? colour_blocks_vec<D, float>(level) : colour_blocks_vec<D, double>(level);
            if (k == "lgs")
            {
                if (m.f32)
                    launch_lgs_colour<D, float>(level, 0, (const float *)m.Mcb, cb.count[0], (const float *)m.b, (float *)m.x, c.stream);
                else
                    launch_lgs_colour<D, double>(level, 0, (const double *)m.Mcb, cb.count[0], (const double *)m.b, (double *)m.x,
                                                 c.stream);
            }
            else if (k == "residual")
            {
                dim3 grid(blocks(cb.count[0]), 1 << D);
                if (m.f32)
                    residual_cb_kernel<D, float><<<grid, kThreads, 0, c.stream>>>(level, (const float *)m.Mcb, cb, (const float *)m.b,
                                                                                 (const float *)m.x, (float *)m.r);
                else
                    residual_cb_kernel<D, double><<<grid, kThreads, 0, c.stream>>>(level, (const double *)m.Mcb, cb, (const double *)m.b,
                                                                                  (const double *)m.x, (double *)m.r);
            }
            else if (k == "assemble")
            {
                if (m.f32)
                    alternating_system_kernel<D, float><<<blocks(Lv.N, 128), 128, 0, c.stream>>>(level, Lv.xy64, 1, Lv.A64, Lv.B64, m.M64, h.b64);
                else
                    alternating_system_kernel<D, double><<<blocks(Lv.N, 128), 128, 0, c.stream>>>(level, Lv.xy64, 1, Lv.A64, Lv.B64, m.M64, h.b64);
            }
            else
                biquad_kernel<D><<<1024, 128, 0, c.stream>>>(level, Lv.xy64, Lv.xy64, Lv.A64, nullptr, 0.0, Lv.B64, partial);
            return 0;
        });
    };
    run();
    cudaEventRecord(c.ev0, c.stream);
    for (int i = 0; i < reps; i++) run();
    cudaEventRecord(c.ev1, c.stream);
    bool ok = c.launch_ok("time mg kernel") && c.cuda_ok(cudaEventSynchronize(c.ev1), "sync");
    float t = 0;
    if (ok) cudaEventElapsedTime(&t, c.ev0, c.ev1);
    *ms = (double)t / reps;
    c.release(partial);
    return ok;
}

bool grad_norm(Context &c, int level, double *out)
{
    if (!c.pull_xy(level)) return false;
    Level &Lv = c.levels[level];
    LevelPtrs<double> P;
    P.level = level;
    P.N = Lv.N;
    P.xy = Lv.xy64;
    P.A = Lv.A64;
    P.B = Lv.B64;
    mg_dim(c, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        launch_grad_norm<D, double>(P, Lv.xy64, c.red, c.stream);
        return 0;
    });
    c.launches += 2;
    double h = 0;
    if (!c.launch_ok("gradient norm") || !c.cuda_ok(cudaMemcpyAsync(&h, c.red.out, sizeof(double), cudaMemcpyDeviceToHost, c.stream), "copy") ||
        !c.cuda_ok(cudaStreamSynchronize(c.stream), "sync"))
        return false;
    *out = std::sqrt(h);
    return true;
}

bool relax_alternating(Context &c, int level, bool finest)
{
    double g0 = 0, g = 0;
    if (!grad_norm(c, level, &g0)) return false;
    g = g0;
    int rounds = 0;
    while (rounds < c.P.max_cycles && g > c.P.tolerance * g0)
    {
        if (!alternating_solve(c, level, 1, 1, c.P.gs_iters, false) || !grad_norm(c, level, &g)) return false;
        rounds++;
        if (c.P.verbose) printf("\t\tGradient[%d][%d]: %g\n", 1 << level, rounds, g);
    }
    c.stats.cycles += rounds;
    if (finest)
    {
        c.stats.grad_norm0 = g0;
        c.stats.grad_norm = g;
    }
    return true;
}

}  // namespace epr
