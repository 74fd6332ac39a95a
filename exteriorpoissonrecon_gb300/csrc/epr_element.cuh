// Exact element integrals of the quartic "wedge" term of the energy.
//
// On one element the fields x, y are multilinear; the 2-form
//     W(x,y)_{PQ} = (d_P y d_Q x - d_P x d_Q y) / 2         (P > Q)
// is the reference's alternating product grad x ^ grad y (Include/Hat.inl:32-37, 243-248:
// packed entry (i,j), i > j, of (v1 v2^T - v2 v1^T)/2 with v1 = grad x, v2 = grad y), and the
// fitting energy integrates its Frobenius norm (Hat.inl:358-370: the packed inner product counts
// every off-diagonal entry twice).  The reference evaluates these integrals through precomputed
// per-node stencils of 1,358 (3D) / 22,952 (4D) coefficients (Hat.products.inl:32-107).  Here
// they are integrated per element and per component:
//   component (P,Q) of W is linear in xi_P and xi_Q and quadratic in the other coordinates, so the
//   product of two such components is integrated exactly by a 2 x 2 x 3^(D-2) Gauss rule
//   (12 points in 3D, 36 in 4D).  Gradients at the Gauss points come from sum factorisation:
//   corner differences along one axis, then 1-D interpolation axis by axis.
//
// All routines work in reference-element units; integrals over the physical element (side 1/r)
// are the returned sums times r^(4-D)/2, which the callers apply (a power of two: exact).
#pragma once
#include <type_traits>

#include "epr_common.cuh"
#include "epr_df.cuh"

namespace epr {

template <int D>
__host__ __device__ constexpr int cbit(int c, int d) { return (c >> (D - 1 - d)) & 1; }

// The two axes (P > Q) of packed component k, in the reference's packing order
// (k = P(P-1)/2 + Q, Hat.inl:32-37), and the remaining axes in increasing order.
template <int D, int K>
struct Component
{
    static constexpr int P = (K == 0) ? 1 : (K <= 2) ? 2 : (K <= 5) ? 3 : -1;
    static constexpr int Q = K - P * (P - 1) / 2;
    static constexpr int M = D - 2;
    // the m-th axis that is neither P nor Q (Q < P): branch-free, so that with m a constant after
    // unrolling every corner index below folds to a constant and the corner arrays the callers
    // index stay in registers
    static constexpr int other(int m)
    {
        const int a = m + (m >= Q ? 1 : 0);
        return a + (a >= P ? 1 : 0);
    }
    // corner index with the given bits on P, Q and the others (others: bit (M-1-m) of bo <-> axis other(m))
    static constexpr int corner(int bP, int bQ, int bo)
    {
        int c = bP << (D - 1 - P) | bQ << (D - 1 - Q);
        for (int m = 0; m < M; m++) c |= ((bo >> (M - 1 - m)) & 1) << (D - 1 - other(m));
        return c;
    }
};

// 1-D hat pieces at Gauss points
template <typename Real>
__device__ __forceinline__ Real hat2(int b, int g) { return b ? (Real)Gauss::X2(g) : (Real)(1.0 - Gauss::X2(g)); }
template <typename Real>
__device__ __forceinline__ Real hat3(int b, int g) { return b ? (Real)Gauss::X3(g) : (Real)(1.0 - Gauss::X3(g)); }
template <typename Real>
__host__ __device__ constexpr Real hat3c(int b, int g) { return b ? Real(Gauss::X3(g)) : Real(1.0 - Gauss::X3(g)); }

// Derivative of a multilinear corner field along axis A (the "derived" axis), tabulated at
// 2 Gauss points of axis B (the partner axis of the component) and 3 Gauss points of each other
// axis.  out[g * 3^M + go] with go enumerating the others (first other slowest).
template <int D, int K, bool AisP, typename Real>
__device__ __forceinline__ void derivative_table(const Real *f, Real *out)
{
    using Cp = Component<D, K>;
    constexpr int M = Cp::M;
    constexpr int NO = 1 << M;      // other-axis corners
    constexpr int NG = ipow(3, M);  // other-axis Gauss points
    // difference along A, indexed [bB][bo]
    Real dif[2][NO];
#pragma unroll
    for (int bB = 0; bB < 2; bB++)
#pragma unroll
        for (int bo = 0; bo < NO; bo++)
        {
            int c1 = AisP ? Cp::corner(1, bB, bo) : Cp::corner(bB, 1, bo);
            int c0 = AisP ? Cp::corner(0, bB, bo) : Cp::corner(bB, 0, bo);
            dif[bB][bo] = f[c1] - f[c0];
        }
    // interpolate along B at the 2-point rule
    Real t[2][NO];
#pragma unroll
    for (int g = 0; g < 2; g++)
#pragma unroll
        for (int bo = 0; bo < NO; bo++) t[g][bo] = hat2<Real>(0, g) * dif[0][bo] + hat2<Real>(1, g) * dif[1][bo];
    // interpolate along the others at the 3-point rule
    if constexpr (M == 1)
    {
#pragma unroll
        for (int g = 0; g < 2; g++)
#pragma unroll
            for (int go = 0; go < 3; go++) out[g * NG + go] = hat3<Real>(0, go) * t[g][0] + hat3<Real>(1, go) * t[g][1];
    }
    else
    {
#pragma unroll
        for (int g = 0; g < 2; g++)
#pragma unroll
            for (int g0 = 0; g0 < 3; g0++)
            {
                Real u0 = hat3<Real>(0, g0) * t[g][0] + hat3<Real>(1, g0) * t[g][2];  // bo = b0*2 + b1
                Real u1 = hat3<Real>(0, g0) * t[g][1] + hat3<Real>(1, g0) * t[g][3];
#pragma unroll
                for (int g1 = 0; g1 < 3; g1++) out[g * NG + g0 * 3 + g1] = hat3<Real>(0, g1) * u0 + hat3<Real>(1, g1) * u1;
            }
    }
}

// The two steps of derivative_table separately, for callers that evaluate the other-axis points
// one at a time (fewer live registers in 4D): the A-differences interpolated along B ...
template <int D, int K, bool AisP, typename Real>
__device__ __forceinline__ void derivative_partial(const Real *f, Real (&t)[2][1 << (D - 2)])
{
    using Cp = Component<D, K>;
    constexpr int NO = 1 << Cp::M;
    Real dif[2][NO];
#pragma unroll
    for (int bB = 0; bB < 2; bB++)
#pragma unroll
        for (int bo = 0; bo < NO; bo++)
        {
            int c1 = AisP ? Cp::corner(1, bB, bo) : Cp::corner(bB, 1, bo);
            int c0 = AisP ? Cp::corner(0, bB, bo) : Cp::corner(bB, 0, bo);
            dif[bB][bo] = f[c1] - f[c0];
        }
#pragma unroll
    for (int g = 0; g < 2; g++)
#pragma unroll
        for (int bo = 0; bo < NO; bo++) t[g][bo] = hat2<Real>(0, g) * dif[0][bo] + hat2<Real>(1, g) * dif[1][bo];
}

// ... and then at the other-axis Gauss point go (the same operations as derivative_table)
template <int M, typename Real>
__device__ __forceinline__ Real derivative_at(const Real *t, int go)
{
    if constexpr (M == 1) return hat3<Real>(0, go) * t[0] + hat3<Real>(1, go) * t[1];
    else
    {
        const int g0 = go / 3, g1 = go % 3;
        Real u0 = hat3<Real>(0, g0) * t[0] + hat3<Real>(1, g0) * t[2];
        Real u1 = hat3<Real>(0, g0) * t[1] + hat3<Real>(1, g0) * t[3];
        return hat3<Real>(0, g1) * u0 + hat3<Real>(1, g1) * u1;
    }
}

template <int M>
__device__ __forceinline__ double other_weight(int go)
{
    if constexpr (M == 1) return Gauss::W3(go);
    else return Gauss::W3(go / 3) * Gauss::W3(go % 3);
}

// ---------------------------------------------------------------------------------------------
// sum over the Gauss points of |W|^2 (reference units), one component
// ---------------------------------------------------------------------------------------------
template <int D, int K, typename Real>
__device__ __forceinline__ Real component_wedge(const Real *x, const Real *y)
{
    constexpr int NG = ipow(3, D - 2);
    Real xP[2 * NG], xQ[2 * NG], yP[2 * NG], yQ[2 * NG];
    derivative_table<D, K, true>(x, xP);
    derivative_table<D, K, false>(x, xQ);
    derivative_table<D, K, true>(y, yP);
    derivative_table<D, K, false>(y, yQ);
    Real s = 0;
#pragma unroll
    for (int gp = 0; gp < 2; gp++)
#pragma unroll
        for (int gq = 0; gq < 2; gq++)
#pragma unroll
            for (int go = 0; go < NG; go++)
            {
                Real w = (Real)(Gauss::W2(gp) * Gauss::W2(gq) * other_weight<D - 2>(go));
                Real W = yP[gq * NG + go] * xQ[gp * NG + go] - xP[gq * NG + go] * yQ[gp * NG + go];
                s += w * W * W;
            }
    return s;
}

template <int D, typename Real>
__device__ __forceinline__ Real element_wedge(const Real *x, const Real *y)
{
    Real s = component_wedge<D, 0>(x, y) + component_wedge<D, 1>(x, y) + component_wedge<D, 2>(x, y);
    if constexpr (D == 4) s += component_wedge<D, 3>(x, y) + component_wedge<D, 4>(x, y) + component_wedge<D, 5>(x, y);
    return s;
}

// ---------------------------------------------------------------------------------------------
// Quadratic-fit integrals of corner A of the element, one component (reference units):
//   h0 = sum |U|^2, h1 = sum |V|^2, h2 = sum <U,V>, h3 = sum <W,U>, h4 = sum <W,V>
// with U = W(phi_A, y), V = W(x, phi_A) (the derivatives of W along x_A and y_A).
// ---------------------------------------------------------------------------------------------
template <int D, int K, typename Real>
__device__ __forceinline__ void component_fit(const Real *x, const Real *y, int A, Real *h)
{
    using Cp = Component<D, K>;
    constexpr int M = Cp::M;
    constexpr int NG = ipow(3, M);
    if constexpr (M == 2)
    {
        // 4D: derivatives evaluated per other-axis point (same values, same summation order)
        Real txP[2][4], txQ[2][4], tyP[2][4], tyQ[2][4];
        derivative_partial<D, K, true>(x, txP);
        derivative_partial<D, K, false>(x, txQ);
        derivative_partial<D, K, true>(y, tyP);
        derivative_partial<D, K, false>(y, tyQ);
        const int aP = cbit<D>(A, Cp::P), aQ = cbit<D>(A, Cp::Q);
        const Real sP = aP ? (Real)1 : (Real)-1, sQ = aQ ? (Real)1 : (Real)-1;
        const int ao0 = cbit<D>(A, Cp::other(0)), ao1 = cbit<D>(A, Cp::other(1));
#pragma unroll
        for (int go = 0; go < NG; go++)
        {
            const Real lo = hat3<Real>(ao0, go / 3) * hat3<Real>(ao1, go % 3);
            const Real wo = (Real)other_weight<M>(go);
            Real xPg[2], xQg[2], yPg[2], yQg[2];
#pragma unroll
            for (int g = 0; g < 2; g++)
            {
                xPg[g] = derivative_at<M, Real>(txP[g], go);
                xQg[g] = derivative_at<M, Real>(txQ[g], go);
                yPg[g] = derivative_at<M, Real>(tyP[g], go);
                yQg[g] = derivative_at<M, Real>(tyQ[g], go);
            }
#pragma unroll
            for (int gp = 0; gp < 2; gp++)
#pragma unroll
                for (int gq = 0; gq < 2; gq++)
                {
                    Real w = (Real)(Gauss::W2(gp) * Gauss::W2(gq)) * wo;
                    Real phP = sP * hat2<Real>(aQ, gq) * lo;
                    Real phQ = sQ * hat2<Real>(aP, gp) * lo;
                    Real xp = xPg[gq], xq = xQg[gp];
                    Real yp = yPg[gq], yq = yQg[gp];
                    Real W = yp * xq - xp * yq;
                    Real U = yp * phQ - phP * yq;
                    Real V = phP * xq - xp * phQ;
                    Real wU = w * U, wV = w * V;
                    h[0] += wU * U;
                    h[1] += wV * V;
                    h[2] += wU * V;
                    h[3] += wU * W;
                    h[4] += wV * W;
                }
        }
        return;
    }
    Real xP[2 * NG], xQ[2 * NG], yP[2 * NG], yQ[2 * NG];
    derivative_table<D, K, true>(x, xP);
    derivative_table<D, K, false>(x, xQ);
    derivative_table<D, K, true>(y, yP);
    derivative_table<D, K, false>(y, yQ);
    const int aP = cbit<D>(A, Cp::P), aQ = cbit<D>(A, Cp::Q);
    const Real sP = aP ? (Real)1 : (Real)-1, sQ = aQ ? (Real)1 : (Real)-1;
    int ao[M > 0 ? M : 1];
#pragma unroll
    for (int m = 0; m < M; m++) ao[m] = cbit<D>(A, Cp::other(m));
#pragma unroll
    for (int go = 0; go < NG; go++)
    {
        Real lo;
        if constexpr (M == 1) lo = hat3<Real>(ao[0], go);
        else lo = hat3<Real>(ao[0], go / 3) * hat3<Real>(ao[1], go % 3);
        Real wo = (Real)other_weight<M>(go);
#pragma unroll
        for (int gp = 0; gp < 2; gp++)
#pragma unroll
            for (int gq = 0; gq < 2; gq++)
            {
                Real w = (Real)(Gauss::W2(gp) * Gauss::W2(gq)) * wo;
                Real phP = sP * hat2<Real>(aQ, gq) * lo;
                Real phQ = sQ * hat2<Real>(aP, gp) * lo;
                Real xp = xP[gq * NG + go], xq = xQ[gp * NG + go];
                Real yp = yP[gq * NG + go], yq = yQ[gp * NG + go];
                Real W = yp * xq - xp * yq;
                Real U = yp * phQ - phP * yq;
                Real V = phP * xq - xp * phQ;
                Real wU = w * U, wV = w * V;
                h[0] += wU * U;
                h[1] += wV * V;
                h[2] += wU * V;
                h[3] += wU * W;
                h[4] += wV * W;
            }
    }
}

// The two steps of component_fit_pq3 for callers that spread a pair's three other-axis points
// over threads: the pair's derivative tables (setup) and one point's terms (point).
template <typename Real>
struct PairTables
{
    Real xP[2], xQ[2], yP[2], yQ[2], w2, hq, hp;
};

template <typename Real>
__device__ __forceinline__ void component_setup_pq3(const Real *x, const Real *y, int gp, int gq, PairTables<Real> &t)
{
    using Cp = Component<3, 0>;
    const Real q0 = gq ? hat2<Real>(0, 1) : hat2<Real>(0, 0), q1 = gq ? hat2<Real>(1, 1) : hat2<Real>(1, 0);
    const Real p0 = gp ? hat2<Real>(0, 1) : hat2<Real>(0, 0), p1 = gp ? hat2<Real>(1, 1) : hat2<Real>(1, 0);
#pragma unroll
    for (int bo = 0; bo < 2; bo++)
    {
        // derivative along P interpolated at Q's point gq, and along Q at P's point gp
        t.xP[bo] = q0 * (x[Cp::corner(1, 0, bo)] - x[Cp::corner(0, 0, bo)]) + q1 * (x[Cp::corner(1, 1, bo)] - x[Cp::corner(0, 1, bo)]);
        t.yP[bo] = q0 * (y[Cp::corner(1, 0, bo)] - y[Cp::corner(0, 0, bo)]) + q1 * (y[Cp::corner(1, 1, bo)] - y[Cp::corner(0, 1, bo)]);
        t.xQ[bo] = p0 * (x[Cp::corner(0, 1, bo)] - x[Cp::corner(0, 0, bo)]) + p1 * (x[Cp::corner(1, 1, bo)] - x[Cp::corner(1, 0, bo)]);
        t.yQ[bo] = p0 * (y[Cp::corner(0, 1, bo)] - y[Cp::corner(0, 0, bo)]) + p1 * (y[Cp::corner(1, 1, bo)] - y[Cp::corner(1, 0, bo)]);
    }
    t.w2 = gp == gq ? (gp ? (Real)(Gauss::W2(1) * Gauss::W2(1)) : (Real)(Gauss::W2(0) * Gauss::W2(0)))
                    : (Real)(Gauss::W2(0) * Gauss::W2(1));
    t.hq = gq ? hat2<Real>(0, 1) : hat2<Real>(0, 0);
    t.hp = p0;
}

template <typename Real>
__device__ __forceinline__ void component_point_pq3(const PairTables<Real> &t, int go, Real *h)
{
    constexpr Real kLo[3] = {hat3c<Real>(0, 0), hat3c<Real>(0, 1), hat3c<Real>(0, 2)};
    constexpr Real kHi[3] = {hat3c<Real>(1, 0), hat3c<Real>(1, 1), hat3c<Real>(1, 2)};
    constexpr Real kW[3] = {(Real)Gauss::W3(0), (Real)Gauss::W3(1), (Real)Gauss::W3(2)};
    const Real lo = go == 0 ? kLo[0] : go == 1 ? kLo[1] : kLo[2];
    const Real hi = go == 0 ? kHi[0] : go == 1 ? kHi[1] : kHi[2];
    const Real w = t.w2 * (go == 0 ? kW[0] : go == 1 ? kW[1] : kW[2]);
    const Real phP = (Real)-1 * t.hq * lo;
    const Real phQ = (Real)-1 * t.hp * lo;
    const Real xp = lo * t.xP[0] + hi * t.xP[1], xq = lo * t.xQ[0] + hi * t.xQ[1];
    const Real yp = lo * t.yP[0] + hi * t.yP[1], yq = lo * t.yQ[0] + hi * t.yQ[1];
    const Real W = yp * xq - xp * yq;
    const Real U = yp * phQ - phP * yq;
    const Real V = phP * xq - xp * phQ;
    const Real wU = w * U, wV = w * V;
    h[0] += wU * U;
    h[1] += wV * V;
    h[2] += wU * V;
    h[3] += wU * W;
    h[4] += wV * W;
}

// Component 0 of a 3D element in the canonical orientation (corner 0), restricted to the Gauss
// points with the given (gp, gq): the share of one of four threads that split a component's
// integral (the values of the points are those of component_fit).  The pair is a run-time value:
// the A-differences are interpolated along B with the hat values of the pair's own Gauss point
// (scalars picked from two constants), so that threads with different pairs run one instruction
// stream and the corner arrays stay constant-indexed in registers.
template <typename Real>
__device__ __forceinline__ void component_fit_pq3(const Real *x, const Real *y, int gp, int gq, Real *h)
{
    using Cp = Component<3, 0>;
    const Real q0 = gq ? hat2<Real>(0, 1) : hat2<Real>(0, 0), q1 = gq ? hat2<Real>(1, 1) : hat2<Real>(1, 0);
    const Real p0 = gp ? hat2<Real>(0, 1) : hat2<Real>(0, 0), p1 = gp ? hat2<Real>(1, 1) : hat2<Real>(1, 0);
    Real xP[2], xQ[2], yP[2], yQ[2];
#pragma unroll
    for (int bo = 0; bo < 2; bo++)
    {
        // derivative along P interpolated at Q's point gq, and along Q at P's point gp
        xP[bo] = q0 * (x[Cp::corner(1, 0, bo)] - x[Cp::corner(0, 0, bo)]) + q1 * (x[Cp::corner(1, 1, bo)] - x[Cp::corner(0, 1, bo)]);
        yP[bo] = q0 * (y[Cp::corner(1, 0, bo)] - y[Cp::corner(0, 0, bo)]) + q1 * (y[Cp::corner(1, 1, bo)] - y[Cp::corner(0, 1, bo)]);
        xQ[bo] = p0 * (x[Cp::corner(0, 1, bo)] - x[Cp::corner(0, 0, bo)]) + p1 * (x[Cp::corner(1, 1, bo)] - x[Cp::corner(1, 0, bo)]);
        yQ[bo] = p0 * (y[Cp::corner(0, 1, bo)] - y[Cp::corner(0, 0, bo)]) + p1 * (y[Cp::corner(1, 1, bo)] - y[Cp::corner(1, 0, bo)]);
    }
    const Real w2 = gp == gq ? (gp ? (Real)(Gauss::W2(1) * Gauss::W2(1)) : (Real)(Gauss::W2(0) * Gauss::W2(0)))
                             : (Real)(Gauss::W2(0) * Gauss::W2(1));
    const Real hq = gq ? hat2<Real>(0, 1) : hat2<Real>(0, 0), hp = p0;
    constexpr Real kLo[3] = {hat3c<Real>(0, 0), hat3c<Real>(0, 1), hat3c<Real>(0, 2)};
    constexpr Real kHi[3] = {hat3c<Real>(1, 0), hat3c<Real>(1, 1), hat3c<Real>(1, 2)};
    constexpr Real kW[3] = {(Real)Gauss::W3(0), (Real)Gauss::W3(1), (Real)Gauss::W3(2)};
    auto point = [&](int go) {
        const Real lo = go == 0 ? kLo[0] : go == 1 ? kLo[1] : kLo[2];
        const Real hi = go == 0 ? kHi[0] : go == 1 ? kHi[1] : kHi[2];
        const Real w = w2 * (go == 0 ? kW[0] : go == 1 ? kW[1] : kW[2]);
        const Real phP = (Real)-1 * hq * lo;
        const Real phQ = (Real)-1 * hp * lo;
        const Real xp = lo * xP[0] + hi * xP[1], xq = lo * xQ[0] + hi * xQ[1];
        const Real yp = lo * yP[0] + hi * yP[1], yq = lo * yQ[0] + hi * yQ[1];
        const Real W = yp * xq - xp * yq;
        const Real U = yp * phQ - phP * yq;
        const Real V = phP * xq - xp * phQ;
        const Real wU = w * U, wV = w * V;
        h[0] += wU * U;
        h[1] += wV * V;
        h[2] += wU * V;
        h[3] += wU * W;
        h[4] += wV * W;
    };
    // the three other-axis points: in double-float a rolled loop (the hat values and weights
    // picked from constants), a third of the code of the unrolled one, for the kernels that run
    // this fit for thousands of dependent single-node updates and are bound by instruction fetch
    if constexpr (std::is_same<Real, df>::value)
    {
#pragma unroll 1
        for (int go = 0; go < 3; go++) point(go);
    }
    else
    {
#pragma unroll
        for (int go = 0; go < 3; go++) point(go);
    }
}

template <int D, typename Real>
__device__ __forceinline__ void element_fit(const Real *x, const Real *y, int A, Real *h)
{
    component_fit<D, 0>(x, y, A, h);
    component_fit<D, 1>(x, y, A, h);
    component_fit<D, 2>(x, y, A, h);
    if constexpr (D == 4)
    {
        component_fit<D, 3>(x, y, A, h);
        component_fit<D, 4>(x, y, A, h);
        component_fit<D, 5>(x, y, A, h);
    }
}

// ---------------------------------------------------------------------------------------------
// Packed float version of element_fit for corner 0 (canonical orientation), on Blackwell's
// two-wide FP32 instructions (FFMA2 / FMUL2: two lanes of arithmetic per issue slot).  The x and
// y fields travel together as (x, y) pairs, so every derivative table is one packed table; at a
// Gauss point, with p = (x_P, y_P), q = (x_Q, y_Q) the P- and Q-derivatives,
//   T = phP q - phQ p = (V, -U),   W = y_P x_Q - x_P y_Q,
// and the five integrals accumulate as (h1, h0) += (w T) * T, (h4, -h3) += (w T) * W and
// h2 += wU V.  The sums are those of element_fit in another association order (float rounding
// differs in the last bits); the fast float relaxation uses it, the double path keeps the scalar
// code.
// ---------------------------------------------------------------------------------------------
struct PackedFit
{
    float2 hv = {0.f, 0.f};  // (h1, h0)
    float2 hw = {0.f, 0.f};  // (h4, -h3)
    float h2 = 0.f;
    __device__ __forceinline__ void add_to(float *h) const
    {
        h[0] += hv.y;
        h[1] += hv.x;
        h[2] += h2;
        h[3] -= hw.y;
        h[4] += hw.x;
    }
};

__device__ __forceinline__ float2 splat2(float v) { return make_float2(v, v); }

// derivative_partial on (x, y) pairs (a - b formed as fma(b, -1, a), which rounds once like a - b)
template <int D, int K, bool AisP>
__device__ __forceinline__ void derivative_partial_packed(const float2 *f, float2 (&t)[2][1 << (D - 2)])
{
    using Cp = Component<D, K>;
    constexpr int NO = 1 << Cp::M;
    float2 dif[2][NO];
#pragma unroll
    for (int bB = 0; bB < 2; bB++)
#pragma unroll
        for (int bo = 0; bo < NO; bo++)
        {
            int c1 = AisP ? Cp::corner(1, bB, bo) : Cp::corner(bB, 1, bo);
            int c0 = AisP ? Cp::corner(0, bB, bo) : Cp::corner(bB, 0, bo);
            dif[bB][bo] = __ffma2_rn(f[c0], splat2(-1.f), f[c1]);
        }
#pragma unroll
    for (int g = 0; g < 2; g++)
#pragma unroll
        for (int bo = 0; bo < NO; bo++)
            t[g][bo] = __ffma2_rn(splat2(hat2<float>(1, g)), dif[1][bo], __fmul2_rn(splat2(hat2<float>(0, g)), dif[0][bo]));
}

// ... and its value at the other-axis Gauss point go (derivative_at on pairs)
template <int M>
__device__ __forceinline__ float2 derivative_at_packed(const float2 *t, int go)
{
    if constexpr (M == 1) return __ffma2_rn(splat2(hat3<float>(1, go)), t[1], __fmul2_rn(splat2(hat3<float>(0, go)), t[0]));
    else
    {
        const int g0 = go / 3, g1 = go % 3;
        const float2 a0 = splat2(hat3<float>(0, g0)), a1 = splat2(hat3<float>(1, g0));
        const float2 u0 = __ffma2_rn(a1, t[2], __fmul2_rn(a0, t[0]));
        const float2 u1 = __ffma2_rn(a1, t[3], __fmul2_rn(a0, t[1]));
        return __ffma2_rn(splat2(hat3<float>(1, g1)), u1, __fmul2_rn(splat2(hat3<float>(0, g1)), u0));
    }
}

template <int D, int K>
__device__ __forceinline__ void component_fit_packed(const float2 *c, PackedFit &acc)
{
    using Cp = Component<D, K>;
    constexpr int M = Cp::M;
    constexpr int NG = ipow(3, M);
    float2 tP[2][1 << M], tQ[2][1 << M];
    derivative_partial_packed<D, K, true>(c, tP);
    derivative_partial_packed<D, K, false>(c, tQ);
#pragma unroll
    for (int go = 0; go < NG; go++)
    {
        // corner 0: every hat factor is the one of bit 0, both signs are -1
        float lo;
        if constexpr (M == 1) lo = hat3<float>(0, go);
        else lo = hat3<float>(0, go / 3) * hat3<float>(0, go % 3);
        const float wo = (float)other_weight<M>(go);
        float2 Pg[2], Qg[2];
#pragma unroll
        for (int g = 0; g < 2; g++)
        {
            Pg[g] = derivative_at_packed<M>(tP[g], go);
            Qg[g] = derivative_at_packed<M>(tQ[g], go);
        }
#pragma unroll
        for (int gp = 0; gp < 2; gp++)
#pragma unroll
            for (int gq = 0; gq < 2; gq++)
            {
                const float w = (float)(Gauss::W2(gp) * Gauss::W2(gq)) * wo;
                const float phP = -hat2<float>(0, gq) * lo;
                const float phQ = -hat2<float>(0, gp) * lo;
                const float2 p = Pg[gq], q = Qg[gp];
                const float W = fmaf(p.y, q.x, -(p.x * q.y));
                const float2 T = __ffma2_rn(splat2(phP), q, __fmul2_rn(splat2(-phQ), p));
                const float2 wT = __fmul2_rn(splat2(w), T);
                acc.hv = __ffma2_rn(wT, T, acc.hv);
                acc.hw = __ffma2_rn(wT, splat2(W), acc.hw);
                acc.h2 = fmaf(-wT.y, T.x, acc.h2);
            }
    }
}

// element_fit<D, float>(x, y, 0, h) on interleaved (x, y) corners
template <int D>
__device__ __forceinline__ void element_fit_packed(const float2 *c, float *h)
{
    PackedFit acc;
    component_fit_packed<D, 0>(c, acc);
    component_fit_packed<D, 1>(c, acc);
    component_fit_packed<D, 2>(c, acc);
    if constexpr (D == 4)
    {
        component_fit_packed<D, 3>(c, acc);
        component_fit_packed<D, 4>(c, acc);
        component_fit_packed<D, 5>(c, acc);
    }
    acc.add_to(h);
}

// ---------------------------------------------------------------------------------------------
// Canonical orientation.  Mirroring an element along axis d (xi_d -> 1 - xi_d) flips the sign of
// every d-derivative; each component of W, U and V carries exactly one derivative along each of
// its two axes, so all the products in the fit integrals keep their sign.  Any corner A can
// therefore be evaluated as corner 0 of the element mirrored along the axes where A has a 1 bit,
// which makes every hat factor a compile-time constant.
// ---------------------------------------------------------------------------------------------
template <int D, typename Real>
struct Corners
{
    Real x[1 << D];
    Real y[1 << D];
};
template <typename Real>
struct Fit5
{
    Real h[5];
};

template <int D, typename Real>
__device__ __noinline__ Fit5<Real> element_fit_canonical(Corners<D, Real> c)
{
    Fit5<Real> f;
#pragma unroll
    for (int k = 0; k < 5; k++) f.h[k] = 0;
    component_fit<D, 0>(c.x, c.y, 0, f.h);
    component_fit<D, 1>(c.x, c.y, 0, f.h);
    component_fit<D, 2>(c.x, c.y, 0, f.h);
    if constexpr (D == 4)
    {
        component_fit<D, 3>(c.x, c.y, 0, f.h);
        component_fit<D, 4>(c.x, c.y, 0, f.h);
        component_fit<D, 5>(c.x, c.y, 0, f.h);
    }
    return f;
}

// ---------------------------------------------------------------------------------------------
// Gauss-Newton products for corner A: J(d) = W(dx, y) + W(x, dy);
//   s[0] = sum <J(d), U>,  s[1] = sum <J(d), V>   (reference units)
// ---------------------------------------------------------------------------------------------
template <int D, int K, typename Real>
__device__ __forceinline__ void component_gn(const Real *x, const Real *y, const Real *dx, const Real *dy, int A, Real *s)
{
    using Cp = Component<D, K>;
    constexpr int M = Cp::M;
    constexpr int NG = ipow(3, M);
    Real xP[2 * NG], xQ[2 * NG], yP[2 * NG], yQ[2 * NG];
    Real dxP[2 * NG], dxQ[2 * NG], dyP[2 * NG], dyQ[2 * NG];
    derivative_table<D, K, true>(x, xP);
    derivative_table<D, K, false>(x, xQ);
    derivative_table<D, K, true>(y, yP);
    derivative_table<D, K, false>(y, yQ);
    derivative_table<D, K, true>(dx, dxP);
    derivative_table<D, K, false>(dx, dxQ);
    derivative_table<D, K, true>(dy, dyP);
    derivative_table<D, K, false>(dy, dyQ);
    const int aP = cbit<D>(A, Cp::P), aQ = cbit<D>(A, Cp::Q);
    const Real sP = aP ? (Real)1 : (Real)-1, sQ = aQ ? (Real)1 : (Real)-1;
    int ao[M > 0 ? M : 1];
#pragma unroll
    for (int m = 0; m < M; m++) ao[m] = cbit<D>(A, Cp::other(m));
#pragma unroll
    for (int go = 0; go < NG; go++)
    {
        Real lo;
        if constexpr (M == 1) lo = hat3<Real>(ao[0], go);
        else lo = hat3<Real>(ao[0], go / 3) * hat3<Real>(ao[1], go % 3);
        Real wo = (Real)other_weight<M>(go);
#pragma unroll
        for (int gp = 0; gp < 2; gp++)
#pragma unroll
            for (int gq = 0; gq < 2; gq++)
            {
                Real w = (Real)(Gauss::W2(gp) * Gauss::W2(gq)) * wo;
                Real phP = sP * hat2<Real>(aQ, gq) * lo;
                Real phQ = sQ * hat2<Real>(aP, gp) * lo;
                int ip = gq * NG + go, iq = gp * NG + go;
                Real J = (yP[ip] * dxQ[iq] - dxP[ip] * yQ[iq]) + (dyP[ip] * xQ[iq] - xP[ip] * dyQ[iq]);
                Real U = yP[ip] * phQ - phP * yQ[iq];
                Real V = phP * xQ[iq] - xP[ip] * phQ;
                s[0] += w * J * U;
                s[1] += w * J * V;
            }
    }
}

template <int D, typename Real>
__device__ __forceinline__ void element_gn(const Real *x, const Real *y, const Real *dx, const Real *dy, int A, Real *s)
{
    component_gn<D, 0>(x, y, dx, dy, A, s);
    component_gn<D, 1>(x, y, dx, dy, A, s);
    component_gn<D, 2>(x, y, dx, dy, A, s);
    if constexpr (D == 4)
    {
        component_gn<D, 3>(x, y, dx, dy, A, s);
        component_gn<D, 4>(x, y, dx, dy, A, s);
        component_gn<D, 5>(x, y, dx, dy, A, s);
    }
}

}  // namespace epr
