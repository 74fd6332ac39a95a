// Shared device definitions of the regular-grid hat-basis system.
//
// Grid conventions (identical to the reference's regular indexer, Hat.scalars.inl:439-509, and to
// the CPU oracle):
//   * level l has resolution r = 2^l, (r+1)^Dim nodes and r^Dim elements;
//   * node index: axis 0 most significant;  element index: axis 0 most significant;
//   * corner c of an element: bit (Dim-1-d) of c is the element-local coordinate on axis d;
//   * column stencils: 3^Dim coefficients per node i, entry o = sum_d (off_d+1) 3^(Dim-1-d) holds
//     M(i + off, i); stored offset-major ("SoA": coef[o * N + i]) so that a warp reads coalesced.
//   * unknowns: interleaved (x, y) pairs per node.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "epr_df.cuh"

namespace epr {

constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

template <int D>
struct Dims
{
    static constexpr int K = D * (D - 1) / 2;  // packed skew coefficients
    static constexpr int S = ipow(3, D);       // stencil width (3^D)
    static constexpr int C = 1 << D;           // element corners
    static constexpr int CENTER = (S - 1) / 2; // stencil centre
};

template <typename Real> struct Pair;
template <> struct Pair<double> { using type = double2; };
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<df> { using type = df2; };
template <typename Real> using Real2 = typename Pair<Real>::type;

// 3- and 2-point Gauss-Legendre rules on [0,1]
struct Gauss
{
    __host__ __device__ static constexpr double X3(int g) { return g == 0 ? 0.11270166537925831148207346002176 : g == 1 ? 0.5 : 0.88729833462074168851792653997824; }
    __host__ __device__ static constexpr double W3(int g) { return g == 1 ? 8.0 / 18.0 : 5.0 / 18.0; }
    __host__ __device__ static constexpr double X2(int g) { return g == 0 ? 0.21132486540518711774542560974902 : 0.78867513459481288225457439025098; }
    __host__ __device__ static constexpr double W2(int) { return 0.5; }
};

template <int D>
struct Grid
{
    int r;        // elements per axis
    int64_t N;    // nodes
    int64_t NE;   // elements
    __host__ __device__ Grid() : r(0), N(0), NE(0) {}
    __host__ __device__ explicit Grid(int level)
    {
        r = 1 << level;
        N = 1;
        NE = 1;
        for (int d = 0; d < D; d++) { N *= (r + 1); NE *= r; }
    }
    __host__ __device__ int64_t node(const int *I) const
    {
        int64_t i = 0;
        for (int d = 0; d < D; d++) i = i * (r + 1) + I[d];
        return i;
    }
    // 32-bit arithmetic: every supported grid (3D depth <= 10, 4D depth <= 7) has < 2^32 nodes
    __host__ __device__ void node(int64_t i, int *I) const
    {
        uint32_t u = (uint32_t)i;
        const uint32_t n = (uint32_t)(r + 1);
        for (int d = D - 1; d >= 0; d--) { uint32_t q = u / n; I[d] = (int)(u - q * n); u = q; }
    }
    __host__ __device__ int64_t elem(const int *E) const
    {
        int64_t i = 0;
        for (int d = 0; d < D; d++) i = i * r + E[d];
        return i;
    }
    __host__ __device__ void elem(int64_t i, int *E) const
    {
        uint32_t u = (uint32_t)i;
        const uint32_t n = (uint32_t)r;
        for (int d = D - 1; d >= 0; d--) { uint32_t q = u / n; E[d] = (int)(u - q * n); u = q; }
    }
    // node stride along axis d
    __host__ __device__ int64_t stride(int d) const
    {
        int64_t s = 1;
        for (int k = D - 1; k > d; k--) s *= (r + 1);
        return s;
    }
};

template <int D>
__host__ __device__ inline void stencil_offset(int o, int *off)
{
    for (int d = D - 1; d >= 0; d--) { off[d] = o % 3 - 1; o /= 3; }
}

// Nodes of one parity colour: colour bit d set <=> node index on axis d is odd
// (ExteriorPoisson.h:161-169).  count_d = number of indices in [0, r] with that parity.
template <int D>
struct Colour
{
    int par[D];
    int cnt[D];
    int64_t n;
    __host__ __device__ Colour() : n(0) {}
    __host__ __device__ Colour(const Grid<D> &g, int colour)
    {
        n = 1;
        for (int d = 0; d < D; d++)
        {
            par[d] = (colour >> d) & 1;
            cnt[d] = par[d] ? (g.r + 1) / 2 : (g.r / 2 + 1);
            n *= cnt[d];
        }
    }
    // j-th node of the colour (axis 0 slowest)
    __host__ __device__ void node(int64_t j, int *I) const
    {
        uint32_t u = (uint32_t)j;
        for (int d = D - 1; d >= 0; d--)
        {
            const uint32_t c = (uint32_t)cnt[d], q = u / c;
            I[d] = 2 * (int)(u - q * c) + par[d];
            u = q;
        }
    }
};

// Colour-blocked stencil layout: the nodes of colour c (in Colour::node order) form one block; the
// block of colour c starts after the blocks of colours 0..c-1, and coefficient o of the colour's
// j-th node sits at block + o * n_c + j.  One colour sweep then streams its coefficients
// contiguously instead of every other element of each sector.
template <int D>
__host__ __device__ inline int64_t colour_block_base(const Grid<D> &g, int colour)
{
    int64_t at = 0;
    for (int c = 0; c < colour; c++) at += Colour<D>(g, c).n * ipow(3, D);
    return at;
}

// Error flags written by kernels and read by the host after a step
enum ErrorBits : unsigned int
{
    ERR_NONFINITE = 1u,
    ERR_INDEX = 2u,
};

}  // namespace epr
