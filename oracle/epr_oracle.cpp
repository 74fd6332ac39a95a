// CPU restatement of the reference's regular-grid reconstruction path.
//
// TEST INFRASTRUCTURE ONLY: this is the oracle that the CUDA path is compared against and the
// CPU baseline that bench.py times beside it.  The product library never links it.
//
// The reference computes the quartic "wedge" energy through per-node stencils of 1,358 (3D) /
// 22,952 (4D) coefficients (Hat.products.inl:32-107, 189-231).  This restatement integrates the
// same energy element by element with a tensor 3-point Gauss-Legendre rule, which is exact for
// the integrand (degree <= 4 per axis), so the two agree to rounding.  Every other step follows
// the reference's algorithm directly; each function cites the reference file:line it restates.
//
// Parity of this file against the reference itself is pinned by tests/test_oracle_golden.py on
// fixtures written by oracle/_ref/ref_harness (the reference headers compiled unmodified).

#include "epr_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// 3-point Gauss-Legendre on [0,1]
const double GQ_X[3] = {0.5 - 0.5 * 0.77459666924148337703585307995647992, 0.5, 0.5 + 0.5 * 0.77459666924148337703585307995647992};
const double GQ_W[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};

template <int D>
struct Traits
{
    static constexpr int K = D * (D - 1) / 2;  // packed skew coefficients
    static constexpr int S = ipow(3, D);       // stencil width
    static constexpr int C = 1 << D;           // element corners
    static constexpr int Q = ipow(3, D);       // quadrature points
};

inline size_t NumNodes(int D, int level)
{
    size_t n = 1;
    for (int d = 0; d < D; d++) n *= (size_t)((1 << level) + 1);
    return n;
}

template <int D>
struct GridIdx
{
    int r;  // resolution (elements per axis)
    explicit GridIdx(int r_) : r(r_) {}
    size_t nodes() const { size_t n = 1; for (int d = 0; d < D; d++) n *= (size_t)(r + 1); return n; }
    size_t elems() const { size_t n = 1; for (int d = 0; d < D; d++) n *= (size_t)r; return n; }
    size_t node(const int *I) const { size_t i = 0; for (int d = 0; d < D; d++) i = i * (r + 1) + I[d]; return i; }
    void node(size_t i, int *I) const { for (int d = D - 1; d >= 0; d--) { I[d] = (int)(i % (r + 1)); i /= (r + 1); } }
    size_t elem(const int *E) const { size_t i = 0; for (int d = 0; d < D; d++) i = i * r + E[d]; return i; }
    void elem(size_t i, int *E) const { for (int d = D - 1; d >= 0; d--) { E[d] = (int)(i % r); i /= r; } }
};

template <int D>
inline int StencilOffsetIndex(const int *off)
{
    int o = 0;
    for (int d = 0; d < D; d++) o = o * 3 + (off[d] + 1);
    return o;
}
template <int D>
inline void StencilOffset(int o, int *off)
{
    for (int d = D - 1; d >= 0; d--) { off[d] = o % 3 - 1; o /= 3; }
}

// ------------------------------------------------------------------------------------------------
// B-splines (GridSamples.inl:32-48): values of the degree-`deg` uniform B-spline pieces at x in [0,1]
// ------------------------------------------------------------------------------------------------
void BSplineEvaluate(int degree, double x, double *values)
{
    if (degree == 0) { values[0] = 1.; return; }
    const double scale = 1. / degree;
    BSplineEvaluate(degree - 1, x, values + 1);
    values[0] = values[1] * (1. - x) * scale;
    for (int i = 1; i < degree; i++)
    {
        double x1 = (x - i + degree), x2 = (-x + i + 1);
        values[i] = (values[i] * x1 + values[i + 1] * x2) * scale;
    }
    values[degree] *= x * scale;
}

// ------------------------------------------------------------------------------------------------
// Symmetric eigenvalues (ascending) by cyclic Jacobi rotations; stands in for Eigen's
// SelfAdjointEigenSolver used by DensityAndNoiseInfo::noise (GridSamples.inl:82-102).
// ------------------------------------------------------------------------------------------------
template <int D>
void SymEigenvalues(double A[D][D], double *ev)
{
    double a[D][D];
    for (int i = 0; i < D; i++) for (int j = 0; j < D; j++) a[i][j] = A[i][j];
    for (int sweep = 0; sweep < 64; sweep++)
    {
        double off = 0;
        for (int i = 0; i < D; i++) for (int j = i + 1; j < D; j++) off += a[i][j] * a[i][j];
        if (off == 0) break;
        for (int p = 0; p < D; p++) for (int q = p + 1; q < D; q++)
        {
            if (a[p][q] == 0) continue;
            double theta = (a[q][q] - a[p][p]) / (2 * a[p][q]);
            double t = (theta >= 0 ? 1. : -1.) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
            double c = 1 / std::sqrt(t * t + 1), s = t * c;
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
    std::sort(ev, ev + D);
}

// ------------------------------------------------------------------------------------------------
// The per-level system: A = R + dWeight K and B as column stencils, c shared by all levels.
// ------------------------------------------------------------------------------------------------
struct LevelSystem
{
    std::vector<double> A, B, R;
};

// Dense per-tree-level splat storage: tree depth t (1..D+1) has resolution 2^(t-1) and
// (2^(t-1)+1)^D vertices; level index l = t-1.
// FitBlade (ExteriorPoisson.h:411-438): the skew matrix p (packed as the reference's
// SkewSymmetricMatrix: entry (i, j), j < i, in (i, j) order; the matrix m(i, j) = p, m(j, i) = -p in
// the reference's (column, row) indexing, Hat.inl:45-52) replaced by
// the blade a ^ b of the power iteration v2 = Next(v1), v1 <- -Next(v2), Next(v) = normalised
// (m v - (v . m v) v), stopped when |v1 - v1'|^2 < 1e-10 or after 1000 steps
// (ExteriorPoissonRecon.cpp:48-49), then a, b = v1, v2 scaled by |m|^(1/2) (Frobenius norm) and
// p(i, j) = (a_j b_i - a_i b_j) / 2.  The start is the column of m with the largest norm (it lies in
// m's image, so the iteration never meets m's kernel); the reference starts from a random unit
// vector, which converges to the same blade.
template <int D>
static void ProjectBlade(double *p)
{
    double m[D][D] = {};
    double sq = 0;
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
        const double n = std::sqrt(n2);
        for (int i = 0; i < D; i++) out[i] = w[i] / n;
    };
    double v1[D], v2[D] = {};
    int best = 0;
    double bn = -1;
    for (int k = 0; k < D; k++)
    {
        double n2 = 0;
        for (int i = 0; i < D; i++) n2 += m[i][k] * m[i][k];
        if (n2 > bn) { bn = n2; best = k; }
    }
    for (int i = 0; i < D; i++) v1[i] = m[i][best] / std::sqrt(bn);
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
    const double scale = std::sqrt(std::sqrt(sq));
    for (int i = 0, idx = 0; i < D; i++)
        for (int j = 0; j < i; j++, idx++) p[idx] = ((v1[j] * scale) * (v2[i] * scale) - (v1[i] * scale) * (v2[j] * scale)) / 2.;
}

template <int D>
struct DenseTree
{
    int maxLevel = 0;
    int width = 0;                            // payload doubles per vertex
    std::vector<std::vector<double>> data;    // per level l: (2^l+1)^D * width
    std::vector<std::vector<uint8_t>> refined; // per tree depth t (0..D+1): cells (2^t)^D, 1 if children exist
};

// -------------------------------------------------------------------------------------------
// Line searches on the bi-quadratic fit (SystemEnergy.h:256-303).  q[i*3+j] = coefficient of
// s^i t^j.  Real roots of polynomials up to degree 3 follow Polynomial::Roots
// (Misha/Polynomial.inl:653-708: a constant term below 1e-14 in magnitude is taken as the root 0
// and the polynomial deflated; a vanishing leading coefficient lowers the degree) and, for the
// cubic, the trigonometric / Cardano method for x^3 + a x^2 + b x + c (three real roots when
// R^2 <= Q^3 + eps, Q = (a^2 - 3b)/9, R = (2a^3 - 9ab + 27c)/54; otherwise one real root, or a
// double root when the imaginary part falls below eps).
// -------------------------------------------------------------------------------------------
static int RealRoots(const double *p, int degree, double *r, double eps = 1e-14)
{
    if (degree == 0) return 0;
    if (std::fabs(p[0]) < eps)
    {
        r[0] = 0;
        return RealRoots(p + 1, degree - 1, r + 1, eps) + 1;
    }
    if (degree == 1) { if (p[1] == 0) return 0; r[0] = -p[0] / p[1]; return 1; }
    if (p[degree] == 0) return RealRoots(p, degree - 1, r, eps);
    if (degree == 2)
    {
        double disc = p[1] * p[1] - 4. * p[0] * p[2];
        if (disc < 0) return 0;
        if (disc == 0) { r[0] = -p[1] / (2 * p[2]); return 1; }
        disc = std::sqrt(disc);
        r[0] = (-p[1] - disc) / (2 * p[2]);
        r[1] = (-p[1] + disc) / (2 * p[2]);
        return 2;
    }
    double a = p[2] / p[3], b = p[1] / p[3], cc = p[0] / p[3];
    double Qv = (a * a - 3 * b) / 9, Rv = (a * (2 * a * a - 9 * b) + 27 * cc) / 54;
    double Q3 = Qv * Qv * Qv, R2 = Rv * Rv;
    if (R2 <= Q3 + eps)
    {
        double t = Rv / std::sqrt(Q3);
        t = std::max(-1., std::min(1., t));
        double th = std::acos(t), m = -2 * std::sqrt(Qv);
        const double twoPi = 6.283185307179586476925286766559;
        r[0] = m * std::cos(th / 3) - a / 3;
        r[1] = m * std::cos((th + twoPi) / 3) - a / 3;
        r[2] = m * std::cos((th - twoPi) / 3) - a / 3;
        return 3;
    }
    double Av = -std::cbrt(std::fabs(Rv) + std::sqrt(R2 - Q3));
    if (Rv < 0) Av = -Av;
    double Bv = Av == 0 ? 0 : Qv / Av;
    r[0] = (Av + Bv) - a / 3;
    double im = 0.5 * std::sqrt(3.) * (Av - Bv);
    if (std::fabs(im) < eps) { r[1] = -0.5 * (Av + Bv) - a / 3; return 2; }
    return 1;
}

// coefficients (degree 4) of s -> P(c0 + s d0, c1 + s d1)
static void PullBack(const double *q, double c0, double d0, double c1, double d1, double *out)
{
    for (int k = 0; k < 5; k++) out[k] = 0;
    double ps[3][3] = {{1, 0, 0}, {c0, d0, 0}, {c0 * c0, 2 * c0 * d0, d0 * d0}};  // (c0 + s d0)^i
    double pt[3][3] = {{1, 0, 0}, {c1, d1, 0}, {c1 * c1, 2 * c1 * d1, d1 * d1}};
    for (int i = 0; i <= 2; i++)
        for (int j = 0; j <= 2; j++)
            for (int a = 0; a <= 2; a++)
                for (int b = 0; b <= 2; b++) out[a + b] += q[i * 3 + j] * ps[i][a] * pt[j][b];
}

static double Poly1(const double *p, int deg, double s)
{
    double v = 0;
    for (int k = deg; k >= 0; k--) v = v * s + p[k];
    return v;
}

// the minimiser of the quartic p among the real roots of its derivative
static double QuarticArgMin(const double *p)
{
    double dp[4] = {p[1], 2 * p[2], 3 * p[3], 4 * p[4]}, roots[3];
    int n = RealRoots(dp, 3, roots);
    if (n <= 0) return 0;
    double s = roots[0];
    for (int i = 1; i < n; i++) if (Poly1(p, 4, roots[i]) < Poly1(p, 4, s)) s = roots[i];
    return s;
}

// stepSize (SystemEnergy.h:256-270): argmin over s of P(s, s)
static double StepSize(const double *q)
{
    double p[5];
    PullBack(q, 0, 1, 0, 1, p);
    return QuarticArgMin(p);
}

// newtonUpdate (SystemEnergy.h:272-303): Newton directions from (0,0), each followed by an exact
// line search along the direction
static void NewtonUpdate(const double *q, int steps, double *st)
{
    double c0 = 0, c1 = 0;
    for (int k = 0; k < steps; k++)
    {
        auto Q = [&](int i, int j) { return q[i * 3 + j]; };
        // gradient and Hessian of sum q_ij s^i t^j at (c0, c1)
        double g0 = 0, g1 = 0, h00 = 0, h01 = 0, h11 = 0;
        for (int i = 0; i <= 2; i++)
            for (int j = 0; j <= 2; j++)
            {
                double v = Q(i, j);
                double si = std::pow(c0, i), tj = std::pow(c1, j);
                if (i >= 1) g0 += v * i * std::pow(c0, i - 1) * tj;
                if (j >= 1) g1 += v * j * si * std::pow(c1, j - 1);
                if (i >= 2) h00 += v * i * (i - 1) * std::pow(c0, i - 2) * tj;
                if (j >= 2) h11 += v * j * (j - 1) * si * std::pow(c1, j - 2);
                if (i >= 1 && j >= 1) h01 += v * i * j * std::pow(c0, i - 1) * std::pow(c1, j - 1);
            }
        double det = h00 * h11 - h01 * h01;
        double d0 = -(h11 * g0 - h01 * g1) / det, d1 = -(-h01 * g0 + h00 * g1) / det;
        if (d0 * d0 + d1 * d1 < 1e-20) break;
        double p[5];
        PullBack(q, c0, d0, c1, d1, p);
        double s = QuarticArgMin(p);
        c0 += d0 * s;
        c1 += d1 * s;
    }
    st[0] = c0;
    st[1] = c1;
}

template <int D>
struct Oracle
{
    using T = Traits<D>;
    int depth;
    epr_oracle_params P;
    size_t n = 0;
    std::vector<double> pos, skew;  // unit cube positions, packed skew
    // ordered sampler
    std::vector<std::array<int, D>> cells;
    std::vector<size_t> cellStart;  // size cells+1
    std::vector<size_t> cellOrder;  // sample ids grouped by cell
    // estimator
    DenseTree<D> density, skewTree;
    std::vector<double> measure, noise, sdepth;
    // finest constraint
    std::vector<double> S;          // #E x K
    std::vector<int> leafDepth;
    double c = 0;
    std::vector<LevelSystem> levels;
    // adaptive indexer (empty for the regular grid): per level the node status (0 none, 1 indexed,
    // 2 active), the node of every function index, the element of every element index
    std::vector<std::vector<uint8_t>> status;
    std::vector<std::vector<int64_t>> fnodes, enodes;
    std::vector<int64_t> nActive;
    std::vector<uint8_t> elemIndexed;  // finest level
    bool adaptive() const { return !status.empty(); }

    Oracle(int depth_, const epr_oracle_params &p) : depth(depth_), P(p) { levels.resize(depth + 1); }

    // -------------------------------------------------------------------------------------------
    // OrderedSampler (OrderedSamples.inl:32-85): cell = clamp(floor(p r)), samples grouped by cell
    // in lexicographic cell order (Index operator<, axis 0 first), stable within a cell.
    // -------------------------------------------------------------------------------------------
    void orderSamples()
    {
        int r = 1 << depth;
        std::vector<std::array<int, D>> key(n);
        for (size_t i = 0; i < n; i++)
            for (int d = 0; d < D; d++) key[i][d] = std::max(0, std::min((int)std::floor(pos[i * D + d] * r), r - 1));
        std::vector<size_t> idx(n);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return key[a] < key[b]; });
        cells.clear(); cellStart.clear(); cellOrder = idx;
        for (size_t i = 0; i < n; i++)
        {
            if (i == 0 || key[idx[i]] != key[idx[i - 1]]) { cells.push_back(key[idx[i]]); cellStart.push_back(i); }
        }
        cellStart.push_back(n);
    }

    // -------------------------------------------------------------------------------------------
    // Tree structure of TreeSplatter (GridSamples.inl:361-391 insertion, RegularTree.inl:728-845
    // neighbour creation): every occupied finest cell creates, at every tree depth t, the children
    // of the parents of its window [c_t - KR, c_t + KR + 1]; depth-1 nodes are the root's children.
    // refined[t][cell] = 1 when that depth-t cell has children.
    // -------------------------------------------------------------------------------------------
    void buildRefinement(DenseTree<D> &tree, int KR)
    {
        tree.refined.assign(depth + 2, {});
        auto cellCount = [](int t) { size_t n = 1; for (int d = 0; d < D; d++) n *= (size_t)(1 << t); return n; };
        tree.refined[0].assign(1, 1);
        for (int t = 1; t <= depth + 1; t++) tree.refined[t].assign(cellCount(t), 0);
        // exists(t, o) <=> refined(t-1, o>>1), exists(1, o) for o in [0,2)^D
        for (int t = 1; t <= depth; t++)
        {
            int side = 1 << t;
            std::vector<uint8_t> &ref = tree.refined[t];
            const std::vector<uint8_t> &pref = tree.refined[t - 1];
            int pside = 1 << (t - 1);
            for (size_t ci = 0; ci < cells.size(); ci++)
            {
                // ancestor of the occupied cell at tree depth t+1
                int ct[D];
                for (int d = 0; d < D; d++) ct[d] = cells[ci][d] >> (depth - t);
                int lo[D], hi[D];
                for (int d = 0; d < D; d++) { lo[d] = (ct[d] - KR) >> 1; hi[d] = (ct[d] + KR + 1) >> 1; }
                int I[D];
                for (int d = 0; d < D; d++) I[d] = lo[d];
                while (true)
                {
                    bool ok = true;
                    size_t li = 0, pi = 0;
                    for (int d = 0; d < D; d++)
                    {
                        if (I[d] < 0 || I[d] >= side) { ok = false; break; }
                        li = li * side + I[d];
                        pi = pi * pside + (I[d] >> 1);
                    }
                    if (ok)
                    {
                        bool exists = (t == 1) ? true : (pref[pi] != 0);
                        if (exists) ref[li] = 1;
                    }
                    int d = D - 1;
                    for (; d >= 0; d--) { if (++I[d] <= hi[d]) break; I[d] = lo[d]; }
                    if (d < 0) break;
                }
            }
        }
    }

    // Cell of a point at resolution res as the tree descent finds it: a child is the upper one
    // only when p is strictly above the split (RegularTree.inl:538-543, 248-262), so points on a
    // face belong to the lower cell.
    static int TreeCell(double p, int res)
    {
        double s = p * res;
        int o = (int)std::floor(s);
        if ((double)o == s && o > 0) o--;
        return o;
    }

    // tree depth of the leaf containing p (RegularTreeNode::getLeafNode)
    int leafDepthAt(const DenseTree<D> &tree, const double *p) const
    {
        int t = 1;
        while (t <= depth)
        {
            int side = 1 << t, res = 1 << (t - 1);
            size_t li = 0;
            for (int d = 0; d < D; d++)
            {
                int o = TreeCell(p[d], res);
                if (o < 0 || o >= side) return t;
                li = li * side + o;
            }
            if (!tree.refined[t][li]) return t;
            t++;
        }
        return t;
    }

    // -------------------------------------------------------------------------------------------
    // Splat one datum at tree depth t with B-spline weights of degree 2 KR + 1
    // (TreeSplatter::_addSample, GridSamples.inl:458-491)
    // -------------------------------------------------------------------------------------------
    // The window is placed around the tree cell `center` (the depth-t ancestor of the inserted
    // cell) while the B-spline weights come from floor(p res); the two differ only for positions on
    // cell faces or clamped into the last cell, where the reference behaves the same way.
    void splat(DenseTree<D> &tree, int KR, int t, const double *p, const int *finestCell, const double *datum, double w)
    {
        int res = 1 << (t - 1), deg = 2 * KR + 1, nv = res + 1;
        double bs[D][10];
        int E[D];
        for (int d = 0; d < D; d++)
        {
            int e = (int)std::floor(p[d] * res);
            BSplineEvaluate(deg, p[d] * res - e, bs[d]);
            E[d] = finestCell[d] >> (depth + 1 - t);
        }
        std::vector<double> &g = tree.data[t - 1];
        int W = tree.width;
        int I[D];
        for (int d = 0; d < D; d++) I[d] = 0;
        while (true)
        {
            bool in = true;
            double s = 1.;
            size_t vi = 0;
            for (int d = 0; d < D; d++)
            {
                int o = E[d] - KR + I[d];
                s *= bs[d][I[d]];
                if (o < 0 || o > res) in = false;
                vi = vi * nv + (in ? o : 0);
            }
            if (in)
            {
                double sc = s * w;
                for (int k = 0; k < W; k++) g[vi * W + k] += sc * datum[k];
            }
            int d = D - 1;
            for (; d >= 0; d--) { if (++I[d] <= deg) break; I[d] = 0; }
            if (d < 0) break;
        }
    }

    void allocTree(DenseTree<D> &tree, int width)
    {
        tree.width = width;
        tree.maxLevel = depth;
        tree.data.assign(depth + 1, {});
        for (int l = 0; l <= depth; l++) tree.data[l].assign(NumNodes(D, l) * width, 0.);
    }

    // multilinear interpolation of tree level t at p (KernelRadius 0 queries, GridSamples.inl:552-598)
    void interp(const DenseTree<D> &tree, int t, const double *p, double *out) const
    {
        int W = tree.width;
        for (int k = 0; k < W; k++) out[k] = 0;
        if (t < 1) return;  // the root carries no data
        int res = 1 << (t - 1), nv = res + 1;
        int e[D];
        double v[D][2];
        for (int d = 0; d < D; d++)
        {
            int f = (int)std::floor(p[d] * res);
            double x = p[d] * res - f;
            v[d][0] = 1. - x;
            v[d][1] = x;
            e[d] = TreeCell(p[d], res);
        }
        const std::vector<double> &g = tree.data[t - 1];
        for (int c = 0; c < (1 << D); c++)
        {
            double s = 1.;
            size_t vi = 0;
            bool in = true;
            for (int d = 0; d < D; d++)
            {
                int b = (c >> (D - 1 - d)) & 1;
                int o = e[d] + b;
                if (o < 0 || o > res) in = false;
                s *= v[d][b];
                vi = vi * nv + (in ? o : 0);
            }
            if (!in) continue;
            for (int k = 0; k < W; k++) out[k] += g[vi * W + k] * s;
        }
    }

    // -------------------------------------------------------------------------------------------
    // TreeEstimator (GridSamples.inl:740-896)
    // -------------------------------------------------------------------------------------------
    static constexpr int DW = 1 + D + D * D;
    double target() const { return std::pow(2., D - 2); }

    double samplesPerCell(int t, const double *p) const
    {
        double info[DW];
        interp(density, t, p, info);
        return info[0] / (double)(1u << ((t - 1) * (D - 2)));
    }

    // _depth (GridSamples.inl:864-896)
    double estDepthRaw(int maxT, const double *p) const
    {
        const double tg = target();
        int d1 = maxT, d2 = maxT + 1;
        while (d2 > 1 && samplesPerCell(d1, p) < tg) d1--, d2--;
        if (d2 == 1 || d2 == maxT + 1)
        {
            int d = (d2 == 1) ? 1 : maxT;
            double spc = samplesPerCell(d, p);
            return d + std::log(spc / tg) / std::log(2.);
        }
        double s1 = samplesPerCell(d1, p), s2 = samplesPerCell(d2, p);
        if (!s2) return d1;
        return d1 + std::log(tg / s1) / std::log(s2 / s1);
    }

    void estInfo(const double *p, double *info) const
    {
        int maxT = depth + 1;
        double dd = estDepthRaw(maxT, p);
        if (dd >= maxT) interp(density, maxT, p, info);
        else if (dd < 0) interp(density, 1, p, info);
        else
        {
            int d1 = (int)std::floor(dd), d2 = d1 + 1;
            double f = dd - d1;
            double a[DW], b[DW];
            interp(density, d1, p, a);
            interp(density, d2, p, b);
            for (int k = 0; k < DW; k++) info[k] = a[k] * (1. - f) + b[k] * f;
        }
    }

    static double InfoNoise(const double *info)
    {
        double w = info[0];
        double C[D][D];
        for (int i = 0; i < D; i++)
            for (int j = 0; j < D; j++) C[i][j] = info[1 + D + i * D + j] / w - info[1 + i] / w * info[1 + j] / w;
        double ev[D];
        SymEigenvalues<D>(C, ev);
        double sum = 0, low = 0;
        for (int d = 0; d < D; d++) { sum += ev[d]; if (d < 2) low += ev[d]; }
        return (low * D) / (sum * 2);
    }

    void buildDensity()
    {
        int KR = P.d_radius;
        allocTree(density, DW);
        buildRefinement(density, KR);
        double bsv[10];
        BSplineEvaluate(2 * KR + 1, 0.5, bsv);
        double scale = std::pow(1. / bsv[KR + 1], 2);
        std::vector<double> scales(depth + 1);
        for (int d = 0; d <= depth; d++) scales[d] = scale / std::pow(std::pow(0.5, d), D - 2);
        int r = 1 << depth;
        (void)r;
        for (size_t ci = 0; ci < cells.size(); ci++)
        {
            // merged sample: mean position, summed (w=1, p, p p^T) (GridSamples.inl:381-388, 761)
            double p[D] = {0}, datum[DW] = {0};
            for (size_t j = cellStart[ci]; j < cellStart[ci + 1]; j++)
            {
                const double *q = &pos[cellOrder[j] * D];
                for (int d = 0; d < D; d++) p[d] += q[d];
                datum[0] += 1.;
                for (int d = 0; d < D; d++) datum[1 + d] += q[d];
                for (int a = 0; a < D; a++) for (int b = 0; b < D; b++) datum[1 + D + a * D + b] += q[a] * q[b];
            }
            double cnt = (double)(cellStart[ci + 1] - cellStart[ci]);
            for (int d = 0; d < D; d++) p[d] /= cnt;
            for (int t = 1; t <= depth + 1; t++) splat(density, KR, t, p, cells[ci].data(), datum, scales[t - 1]);
        }
        measure.resize(n); noise.resize(n); sdepth.resize(n);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; i++)
        {
            double info[DW];
            estInfo(&pos[i * D], info);
            measure[i] = 1. / info[0];
            noise[i] = InfoNoise(info);
            sdepth[i] = estDepthRaw(depth + 1, &pos[i * D]) - 1.;
        }
    }

    // -------------------------------------------------------------------------------------------
    // Skew splat (ExteriorPoisson.h:181-264, GridSamples.inl:393-456)
    // -------------------------------------------------------------------------------------------
    void buildSkew()
    {
        int KR = P.t_radius;
        allocTree(skewTree, T::K);
        buildRefinement(skewTree, KR);
        auto depthWeight = [](int d) { return (double)(1u << (d * D)); };
        for (size_t ci = 0; ci < cells.size(); ci++)
            for (size_t j = cellStart[ci]; j < cellStart[ci + 1]; j++)
            {
                size_t s = cellOrder[j];
                double v[T::K], nrm = 0;
                for (int k = 0; k < T::K; k++) { v[k] = skew[s * T::K + k]; nrm += 2 * v[k] * v[k]; }
                nrm = std::sqrt(nrm);
                for (int k = 0; k < T::K; k++) { v[k] /= nrm; v[k] *= measure[s]; v[k] *= (double)(1u << (depth * 2)); }
                double dd = sdepth[s] + 1.;
                const double *p = &pos[s * D];
                const int *E = cells[ci].data();
                if (dd >= depth + 1) splat(skewTree, KR, depth + 1, p, E, v, depthWeight(depth));
                else if (dd <= 1) splat(skewTree, KR, 1, p, E, v, depthWeight(0));
                else
                {
                    int d1 = (int)std::floor(dd), d2 = d1 + 1;
                    double f = dd - d1;
                    double a[T::K], b[T::K];
                    for (int k = 0; k < T::K; k++) { a[k] = v[k] * (1. - f); b[k] = v[k] * f; }
                    splat(skewTree, KR, d1, p, E, a, depthWeight(d1 - 1));
                    splat(skewTree, KR, d2, p, E, b, depthWeight(d2 - 1));
                }
            }
        double scale = std::pow(std::pow(0.5, depth), 1.5 * 2);
        for (auto &g : skewTree.data) for (double &x : g) x *= scale;
    }

    // S(E) at element centres, summed over the tree depths down to the leaf containing the centre
    // (GridSamples.inl:600-651; ExteriorPoisson.h:290-307)
    void buildS()
    {
        int r = 1 << depth;
        GridIdx<D> g(r);
        size_t NE = g.elems();
        S.assign(NE * T::K, 0.);
        leafDepth.assign(NE, 0);
#pragma omp parallel for schedule(static)
        for (long e = 0; e < (long)NE; e++)
        {
            int E[D];
            g.elem((size_t)e, E);
            double p[D];
            for (int d = 0; d < D; d++) p[d] = (E[d] + 0.5) / r;
            int L = leafDepthAt(skewTree, p);
            leafDepth[e] = L;
            double acc[T::K] = {0}, tmp[T::K];
            for (int t = 1; t <= L; t++)
            {
                interp(skewTree, t, p, tmp);
                for (int k = 0; k < T::K; k++) acc[k] += tmp[k];
            }
            if (P.project) ProjectBlade<D>(acc);
            for (int k = 0; k < T::K; k++) S[e * T::K + k] = acc[k];
        }
        // c: the elements of the indexer (SystemEnergy.h:452-461), divided by all r^Dim
        double cc = 0;
        for (size_t e = 0; e < NE; e++)
        {
            if (!elemIndexed.empty() && !elemIndexed[e]) continue;
            double s2 = 0;
            for (int k = 0; k < T::K; k++) s2 += 2 * S[e * T::K + k] * S[e * T::K + k];
            cc += s2;
        }
        c = cc / (double)NE;
    }

    // -------------------------------------------------------------------------------------------
    // 1D element integrals on [0,1] of the hat pieces l0 = 1-x, l1 = x and their derivatives.
    // -------------------------------------------------------------------------------------------
    static double MassLocal(int a, int b) { return a == b ? 1. / 3. : 1. / 6.; }
    static double StiffLocal(int a, int b) { return a == b ? 1. : -1.; }
    static double MixedLocal(int a /*derivative*/, int b) { (void)b; return (a ? 1. : -1.) * 0.5; }

    // Dirichlet stiffness K(i, i+off) = sum_E int grad phi_i . grad phi_j (Hat.scalars.inl:528-545)
    std::vector<double> stiffnessStencil(int level) const
    {
        int r = 1 << level;
        GridIdx<D> g(r);
        size_t N = g.nodes();
        std::vector<double> K(N * T::S, 0.);
        double h = 1. / r;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++)
        {
            int I[D];
            g.node((size_t)i, I);
            for (int o = 0; o < T::S; o++)
            {
                int off[D], J[D];
                StencilOffset<D>(o, off);
                bool ok = true;
                for (int d = 0; d < D; d++) { J[d] = I[d] + off[d]; if (J[d] < 0 || J[d] > r) ok = false; }
                if (!ok) continue;
                // elements containing both nodes
                int lo[D], hi[D];
                for (int d = 0; d < D; d++) { lo[d] = std::max(std::max(I[d], J[d]) - 1, 0); hi[d] = std::min(std::min(I[d], J[d]), r - 1); if (lo[d] > hi[d]) ok = false; }
                if (!ok) continue;
                double sum = 0;
                int E[D];
                for (int d = 0; d < D; d++) E[d] = lo[d];
                while (true)
                {
                    for (int k = 0; k < D; k++)
                    {
                        double v = 1.;
                        for (int d = 0; d < D; d++)
                        {
                            int a = I[d] - E[d], b = J[d] - E[d];
                            v *= (d == k) ? StiffLocal(a, b) / h : MassLocal(a, b) * h;
                        }
                        sum += v;
                    }
                    int d = D - 1;
                    for (; d >= 0; d--) { if (++E[d] <= hi[d]) break; E[d] = lo[d]; }
                    if (d < 0) break;
                }
                K[(size_t)i * T::S + o] = sum;
            }
        }
        // At resolution 1 the reference's full-integration stencil table only holds the row of
        // node 0: the interior case maps to index res/2 = 0 and the upper boundary case is never
        // filled (Hat.scalars.inl:261-293), so every other node has an empty Dirichlet row.
        if (r == 1)
            for (size_t i = 1; i < N; i++)
                for (int o = 0; o < T::S; o++) K[i * T::S + o] = 0.;
        return K;
    }

    // full skew matrix entry S(a,b) from packed storage
    static double SkewEntry(const double *s, int a, int b)
    {
        if (a == b) return 0;
        if (a > b) return s[a * (a - 1) / 2 + b];
        return -s[b * (b - 1) / 2 + a];
    }

    // B(f2, f1) = sum_E sum_{a,b} S_E(b, a) int_E d_a phi_f1 d_b phi_f2 (Hat.scalars.inl:1585-1690,
    // FullStiffnessStencil :550-565).  Column stencil: entry (f1, off) = B(f1 + off, f1).
    std::vector<double> constraintStencil() const
    {
        int r = 1 << depth;
        GridIdx<D> g(r);
        size_t N = g.nodes();
        std::vector<double> B(N * T::S, 0.);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++)
        {
            int I[D];
            g.node((size_t)i, I);
            for (int o = 0; o < T::S; o++)
            {
                int off[D], J[D];
                StencilOffset<D>(o, off);
                bool ok = true;
                for (int d = 0; d < D; d++) { J[d] = I[d] + off[d]; if (J[d] < 0 || J[d] > r) ok = false; }
                if (!ok) continue;
                int lo[D], hi[D];
                for (int d = 0; d < D; d++) { lo[d] = std::max(std::max(I[d], J[d]) - 1, 0); hi[d] = std::min(std::min(I[d], J[d]), r - 1); if (lo[d] > hi[d]) ok = false; }
                if (!ok) continue;
                double sum = 0;
                int E[D];
                for (int d = 0; d < D; d++) E[d] = lo[d];
                while (true)
                {
                    const double *s = &S[g.elem(E) * T::K];
                    // the adaptive indexer's stiffness integrates its own elements only
                    // (Hat.scalars.inl:1634-1643: elements without an index contribute nothing)
                    const bool counted = elemIndexed.empty() || elemIndexed[g.elem(E)];
                    for (int a = 0; counted && a < D; a++)
                        for (int b = 0; b < D; b++)
                        {
                            if (a == b) continue;
                            double sab = SkewEntry(s, b, a);
                            if (sab == 0) continue;
                            double v = 1.;
                            for (int d = 0; d < D; d++)
                            {
                                int ca = I[d] - E[d], cb = J[d] - E[d];
                                if (d == a) v *= MixedLocal(ca, cb);
                                else if (d == b) v *= MixedLocal(cb, ca);
                                else v *= MassLocal(ca, cb) / r;
                            }
                            sum += sab * v;
                        }
                    int d = D - 1;
                    for (; d >= 0; d--) { if (++E[d] <= hi[d]) break; E[d] = lo[d]; }
                    if (d < 0) break;
                }
                B[(size_t)i * T::S + o] = sum;
            }
        }
        return B;
    }

    // R = sWeight * mean(measure) * sum_samples w(noise) phi_a phi_b (Hat.scalars.inl:977-1063,
    // ExteriorPoisson.h:267-287)
    std::vector<double> screeningStencil() const
    {
        int r = 1 << depth;
        GridIdx<D> g(r);
        size_t N = g.nodes();
        std::vector<double> R(N * T::S, 0.);
        if (P.s_weight <= 0) return R;
        double m = 0;
        for (size_t i = 0; i < n; i++) m += measure[i];
        m /= (double)n;
        double scale = P.s_weight * m;
        for (size_t ci = 0; ci < cells.size(); ci++)
        {
            const std::array<int, D> &E = cells[ci];
            double M[1 << D][1 << D] = {{0}};
            for (size_t j = cellStart[ci]; j < cellStart[ci + 1]; j++)
            {
                size_t s = cellOrder[j];
                double w = std::exp(-noise[s] * noise[s] / (2. * P.n_sigma * P.n_sigma));
                double lv[D][2];
                for (int d = 0; d < D; d++) { double x = pos[s * D + d] * r - E[d]; lv[d][0] = 1. - x; lv[d][1] = x; }
                double phi[1 << D];
                for (int a = 0; a < (1 << D); a++)
                {
                    double v = 1.;
                    for (int d = 0; d < D; d++) v *= lv[d][(a >> (D - 1 - d)) & 1];
                    phi[a] = v;
                }
                for (int a = 0; a < (1 << D); a++) for (int b = 0; b < (1 << D); b++) M[a][b] += phi[a] * phi[b] * w;
            }
            for (int a = 0; a < (1 << D); a++)
                for (int b = 0; b < (1 << D); b++)
                {
                    int Ia[D], off[D];
                    for (int d = 0; d < D; d++) { int ca = (a >> (D - 1 - d)) & 1, cb = (b >> (D - 1 - d)) & 1; Ia[d] = E[d] + ca; off[d] = cb - ca; }
                    // column a holds R(b, a)
                    R[g.node(Ia) * T::S + StencilOffsetIndex<D>(off)] += M[a][b] * scale;
                }
        }
        return R;
    }

    // Galerkin coarsening P^T M P of a column stencil (SystemEnergy.h:464-477, prolongation
    // weights Hat.scalars.inl:373-386: 1/2 per off-parity axis).
    std::vector<double> galerkin(const std::vector<double> &Mf, int fineLevel) const
    {
        int rf = 1 << fineLevel, rc = rf >> 1;
        GridIdx<D> gf(rf), gc(rc);
        size_t Nc = gc.nodes();
        std::vector<double> Mc(Nc * T::S, 0.);
#pragma omp parallel for schedule(static)
        for (long J = 0; J < (long)Nc; J++)
        {
            int Jc[D];
            gc.node((size_t)J, Jc);
            for (int go = 0; go < T::S; go++)
            {
                int goff[D], G[D];
                StencilOffset<D>(go, goff);
                bool ok = true;
                double wg = 1.;
                for (int d = 0; d < D; d++) { G[d] = 2 * Jc[d] + goff[d]; if (G[d] < 0 || G[d] > rf) ok = false; if (goff[d]) wg *= 0.5; }
                if (!ok) continue;
                const double *col = &Mf[gf.node(G) * T::S];
                for (int fo = 0; fo < T::S; fo++)
                {
                    double v = col[fo];
                    if (v == 0) continue;
                    int foff[D], F[D];
                    StencilOffset<D>(fo, foff);
                    for (int d = 0; d < D; d++) F[d] = G[d] + foff[d];
                    // coarse nodes I with P(F, I) != 0
                    int nopt[D], opt[D][2];
                    double ow[D][2];
                    for (int d = 0; d < D; d++)
                    {
                        if (F[d] & 1) { nopt[d] = 2; opt[d][0] = (F[d] - 1) / 2; opt[d][1] = (F[d] + 1) / 2; ow[d][0] = ow[d][1] = 0.5; }
                        else { nopt[d] = 1; opt[d][0] = F[d] / 2; ow[d][0] = 1.; }
                    }
                    int sel[D];
                    for (int d = 0; d < D; d++) sel[d] = 0;
                    while (true)
                    {
                        double w = wg * v;
                        int off[D];
                        for (int d = 0; d < D; d++) { w *= ow[d][sel[d]]; off[d] = opt[d][sel[d]] - Jc[d]; }
                        Mc[(size_t)J * T::S + StencilOffsetIndex<D>(off)] += w;
                        int d = D - 1;
                        for (; d >= 0; d--) { if (++sel[d] < nopt[d]) break; sel[d] = 0; }
                        if (d < 0) break;
                    }
                }
            }
        }
        return Mc;
    }

    // -------------------------------------------------------------------------------------------
    // HierarchicalAdaptedIndexer (Hat.adaptive.inl:342-732) on the dense grids.
    // Active functions of level d (_addSamples, :565-643): every interior node I (0 <= I <= 2^d) in
    // the window A - K .. A + K + 1 of the level-d ancestor A = E >> (depth - d) of a sample cell E
    // (K = aRadius; the window is the (K, K+1) element-function neighbour key of the cell's tree node
    // at every depth).  Their indices follow the tree's depth-first order, i.e. Morton order with
    // axis 0 in the lowest bit of every level (child c of a tree node has offset 2 O + bit d of c).
    // _finalize (:646-728): for the active functions of each level in index order and their 3^Dim
    // neighbours in window order (axis 0 slowest), a neighbour that is an interior node without an
    // index gets the next function index (an indexed but inactive function), and a neighbour that
    // is an interior element (0 <= E < 2^d) on the lower side of the function (E <= I on every
    // axis) without an index gets the next element index.
    // -------------------------------------------------------------------------------------------
    void buildAdaptive()
    {
        const int K = P.adaptive_radius;
        status.assign(depth + 1, {});
        fnodes.assign(depth + 1, {});
        enodes.assign(depth + 1, {});
        nActive.assign(depth + 1, 0);
        for (int d = 0; d <= depth; d++)
        {
            const int r = 1 << d;
            GridIdx<D> g(r);
            std::vector<uint8_t> &st = status[d];
            st.assign(g.nodes(), 0);
            for (size_t ci = 0; ci < cells.size(); ci++)
            {
                int lo[D], hi[D];
                for (int k = 0; k < D; k++)
                {
                    const int A = cells[ci][k] >> (depth - d);
                    lo[k] = std::max(A - K, 0);
                    hi[k] = std::min(A + K + 1, r);
                }
                int I[D];
                for (int k = 0; k < D; k++) I[k] = lo[k];
                while (true)
                {
                    st[g.node(I)] = 2;
                    int k = D - 1;
                    for (; k >= 0; k--) { if (++I[k] <= hi[k]) break; I[k] = lo[k]; }
                    if (k < 0) break;
                }
            }
            // active functions in Morton order
            std::vector<std::pair<uint64_t, int64_t>> act;
            for (size_t i = 0; i < st.size(); i++)
                if (st[i] == 2)
                {
                    int I[D];
                    g.node(i, I);
                    uint64_t key = 0;
                    for (int b = d; b >= 0; b--)
                    {
                        uint64_t c = 0;
                        for (int k = 0; k < D; k++) c |= (uint64_t)((I[k] >> b) & 1) << k;
                        key = (key << D) | c;
                    }
                    act.push_back({key, (int64_t)i});
                }
            std::sort(act.begin(), act.end());
            nActive[d] = (int64_t)act.size();
            for (auto &a : act) fnodes[d].push_back(a.second);
            std::vector<uint8_t> elemSeen((size_t)std::pow(r, D), 0);
            for (size_t a = 0; a < act.size(); a++)
            {
                int I[D];
                g.node((size_t)act[a].second, I);
                for (int w = 0; w < T::S; w++)
                {
                    int off[D], Nn[D];
                    StencilOffset<D>(w, off);
                    bool fn = true, el = true;
                    for (int k = 0; k < D; k++)
                    {
                        Nn[k] = I[k] + off[k];
                        if (Nn[k] < 0 || Nn[k] > r) fn = false;
                        if (Nn[k] < 0 || Nn[k] >= r || off[k] > 0) el = false;
                    }
                    if (fn)
                    {
                        const size_t ni = g.node(Nn);
                        if (st[ni] == 0) { st[ni] = 1; fnodes[d].push_back((int64_t)ni); }
                    }
                    if (el)
                    {
                        const size_t ei = g.elem(Nn);
                        if (!elemSeen[ei]) { elemSeen[ei] = 1; enodes[d].push_back((int64_t)ei); }
                    }
                }
            }
            if (d == depth) elemIndexed = elemSeen;
        }
    }

    void build()
    {
        orderSamples();
        if (P.adaptive_radius >= 0) buildAdaptive();
        buildDensity();
        buildSkew();
        buildS();
        LevelSystem &L = levels[depth];
        L.R = screeningStencil();
        L.B = constraintStencil();
        std::vector<double> K = stiffnessStencil(depth);
        L.A.resize(L.R.size());
        for (size_t i = 0; i < L.A.size(); i++) L.A[i] = L.R[i] + P.d_weight * K[i];
        for (int l = depth - 1; l >= 0; l--)
        {
            levels[l].R = galerkin(levels[l + 1].R, l + 1);
            levels[l].B = galerkin(levels[l + 1].B, l + 1);
            std::vector<double> Kc = stiffnessStencil(l);
            levels[l].A.resize(levels[l].R.size());
            for (size_t i = 0; i < levels[l].A.size(); i++) levels[l].A[i] = levels[l].R[i] + P.d_weight * Kc[i];
        }
    }

    // -------------------------------------------------------------------------------------------
    // Element kernels: exact integrals of the wedge term over one element.
    // Gradients at Gauss point q of a multilinear function with corner values v[c] (corner bit
    // for axis d is (c >> (D-1-d)) & 1); grad scaled by r.
    // W(a,b) = (d_a y d_b x - d_a x d_b y)/2, <P,Q>_F = 2 sum_{a>b} P(a,b) Q(a,b).
    // -------------------------------------------------------------------------------------------
    static void CornerGrad(const double *v, const double *xi, double r, double *g)
    {
        for (int k = 0; k < D; k++)
        {
            double s = 0;
            for (int c = 0; c < (1 << D); c++)
            {
                double w = 1.;
                for (int d = 0; d < D; d++)
                {
                    int b = (c >> (D - 1 - d)) & 1;
                    w *= (d == k) ? (b ? 1. : -1.) : (b ? xi[d] : 1. - xi[d]);
                }
                s += w * v[c];
            }
            g[k] = s * r;
        }
    }
    static void HatGrad(int corner, const double *xi, double r, double *g)
    {
        for (int k = 0; k < D; k++)
        {
            double w = 1.;
            for (int d = 0; d < D; d++)
            {
                int b = (corner >> (D - 1 - d)) & 1;
                w *= (d == k) ? (b ? 1. : -1.) : (b ? xi[d] : 1. - xi[d]);
            }
            g[k] = w * r;
        }
    }

    // wedge energy of one element with corner values x[C], y[C]
    static double ElementWedge(const double *x, const double *y, int r)
    {
        double vol = std::pow(1. / r, D), sum = 0;
        for (int q = 0; q < T::Q; q++)
        {
            double xi[D], w = vol;
            int t = q;
            for (int d = D - 1; d >= 0; d--) { xi[d] = GQ_X[t % 3]; w *= GQ_W[t % 3]; t /= 3; }
            double gx[D], gy[D];
            CornerGrad(x, xi, r, gx);
            CornerGrad(y, xi, r, gy);
            double s = 0;
            for (int a = 0; a < D; a++) for (int b = 0; b < a; b++) { double W = 0.5 * (gy[a] * gx[b] - gx[a] * gy[b]); s += 2 * W * W; }
            sum += w * s;
        }
        return sum;
    }

    // contributions of one element to the quadratic fit of its corner `corner`:
    // h[0] = int |U|^2, h[1] = int |V|^2, h[2] = int <U,V>, h[3] = int <W,U>, h[4] = int <W,V>
    static void ElementFit(const double *x, const double *y, int corner, int r, double *h)
    {
        double vol = std::pow(1. / r, D);
        for (int k = 0; k < 5; k++) h[k] = 0;
        for (int q = 0; q < T::Q; q++)
        {
            double xi[D], w = vol;
            int t = q;
            for (int d = D - 1; d >= 0; d--) { xi[d] = GQ_X[t % 3]; w *= GQ_W[t % 3]; t /= 3; }
            double gx[D], gy[D], gp[D];
            CornerGrad(x, xi, r, gx);
            CornerGrad(y, xi, r, gy);
            HatGrad(corner, xi, r, gp);
            double uu = 0, vv = 0, uv = 0, wu = 0, wv = 0;
            for (int a = 0; a < D; a++)
                for (int b = 0; b < a; b++)
                {
                    double W = 0.5 * (gy[a] * gx[b] - gx[a] * gy[b]);
                    double U = 0.5 * (gy[a] * gp[b] - gp[a] * gy[b]);
                    double V = 0.5 * (gp[a] * gx[b] - gx[a] * gp[b]);
                    uu += 2 * U * U; vv += 2 * V * V; uv += 2 * U * V; wu += 2 * W * U; wv += 2 * W * V;
                }
            h[0] += w * uu; h[1] += w * vv; h[2] += w * uv; h[3] += w * wu; h[4] += w * wv;
        }
    }

    void gatherElement(const GridIdx<D> &g, const int *E, const double *x, const double *y, double *xc, double *yc) const
    {
        for (int c = 0; c < (1 << D); c++)
        {
            int I[D];
            for (int d = 0; d < D; d++) I[d] = E[d] + ((c >> (D - 1 - d)) & 1);
            size_t i = g.node(I);
            xc[c] = x[i];
            yc[c] = y[i];
        }
    }

    // stencil apply at node i: sum_o M(i+off, i) v[i+off]
    static double ColumnDot(const GridIdx<D> &g, const double *col, const int *I, const double *v)
    {
        double s = 0;
        for (int o = 0; o < T::S; o++)
        {
            if (col[o] == 0) continue;
            int off[D], J[D];
            StencilOffset<D>(o, off);
            bool ok = true;
            for (int d = 0; d < D; d++) { J[d] = I[d] + off[d]; if (J[d] < 0 || J[d] > g.r) ok = false; }
            if (ok) s += col[o] * v[g.node(J)];
        }
        return s;
    }

    // energies() (SystemEnergy.h:486-497)
    void energy(int level, const double *x, const double *y, double *out) const
    {
        const LevelSystem &L = levels[level];
        int r = 1 << level;
        GridIdx<D> g(r);
        size_t NE = g.elems(), N = g.nodes();
        double W = 0, xBy = 0, xAx = 0;
#pragma omp parallel for reduction(+ : W) schedule(static)
        for (long e = 0; e < (long)NE; e++)
        {
            int E[D];
            g.elem((size_t)e, E);
            double xc[1 << D], yc[1 << D];
            gatherElement(g, E, x, y, xc, yc);
            W += ElementWedge(xc, yc, r);
        }
#pragma omp parallel for reduction(+ : xBy, xAx) schedule(static)
        for (long i = 0; i < (long)N; i++)
        {
            int I[D];
            g.node((size_t)i, I);
            xBy += x[i] * ColumnDot(g, &L.B[(size_t)i * T::S], I, y);
            xAx += x[i] * ColumnDot(g, &L.A[(size_t)i * T::S], I, x) + y[i] * ColumnDot(g, &L.A[(size_t)i * T::S], I, y);
        }
        out[0] = W - 2. * xBy + c;
        out[1] = xAx;
        out[2] = W;
    }

    // quadraticFit (SystemEnergy.h:542-643): q = (Q20, Q02, Q11, Q10, Q01)
    void quadfitNode(int level, const GridIdx<D> &g, size_t i, const double *x, const double *y, double *q) const
    {
        const LevelSystem &L = levels[level];
        int r = g.r;
        int I[D];
        g.node(i, I);
        for (int k = 0; k < 5; k++) q[k] = 0;
        // wedge term over the elements around the node
        for (int c = 0; c < (1 << D); c++)
        {
            int E[D];
            bool ok = true;
            for (int d = 0; d < D; d++) { E[d] = I[d] - ((c >> (D - 1 - d)) & 1); if (E[d] < 0 || E[d] >= r) ok = false; }
            if (!ok) continue;
            double xc[1 << D], yc[1 << D], h[5];
            gatherElement(g, E, x, y, xc, yc);
            ElementFit(xc, yc, c, r, h);
            q[0] += h[0]; q[1] += h[1]; q[2] += 2 * h[2]; q[3] += 2 * h[3]; q[4] += 2 * h[4];
        }
        const double *a = &L.A[i * T::S];
        const double *b = &L.B[i * T::S];
        int oc = (T::S - 1) / 2;
        q[0] += a[oc];
        q[1] += a[oc];
        q[3] += 2. * ColumnDot(g, a, I, x);
        q[4] += 2. * ColumnDot(g, a, I, y);
        // B column without its diagonal
        double by = 0, bx = 0;
        for (int o = 0; o < T::S; o++)
        {
            if (o == oc || b[o] == 0) continue;
            int off[D], J[D];
            StencilOffset<D>(o, off);
            bool ok = true;
            for (int d = 0; d < D; d++) { J[d] = I[d] + off[d]; if (J[d] < 0 || J[d] > r) ok = false; }
            if (!ok) continue;
            size_t j = g.node(J);
            by += b[o] * y[j];
            bx += b[o] * x[j];
        }
        q[3] -= 2. * by;
        q[4] += 2. * bx;
    }

    void quadfit(int level, const double *x, const double *y, double *out) const
    {
        GridIdx<D> g(1 << level);
        size_t N = g.nodes();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++) quadfitNode(level, g, (size_t)i, x, y, &out[(size_t)i * 5]);
    }

    // paired Gauss-Seidel (ExteriorPoissonSolvers.h:156-196), colours by per-axis parity
    // (ExteriorPoisson.h:161-169): colour bit d set when node index on axis d is odd.
    void gs(int level, double *x, double *y, int iters, const double *tx = nullptr, const double *ty = nullptr) const
    {
        GridIdx<D> g(1 << level);
        size_t N = g.nodes();
        std::vector<std::vector<size_t>> colours(1 << D);
        for (size_t i = 0; i < N; i++)
        {
            int I[D];
            g.node(i, I);
            int m = 0;
            for (int d = 0; d < D; d++) if (I[d] & 1) m |= 1 << d;
            // the colour lists hold the active functions only (ExteriorPoisson.h:161-169)
            if (adaptive() && status[level][i] != 2) continue;
            colours[m].push_back(i);
        }
        for (int it = 0; it < iters; it++)
            for (int cidx = 0; cidx < (1 << D); cidx++)
            {
                const std::vector<size_t> &list = colours[cidx];
#pragma omp parallel for schedule(static)
                for (long j = 0; j < (long)list.size(); j++)
                {
                    size_t i = list[j];
                    double q[5];
                    quadfitNode(level, g, i, x, y, q);
                    if (tx) { q[3] -= tx[i]; q[4] -= ty[i]; }
                    double h00 = 2 * q[0], h11 = 2 * q[1], h01 = q[2];
                    if (P.separate)
                    {
                        // SeparateGaussSeidelSolve (ExteriorPoissonSolvers.h:216-235)
                        double p0 = 0, p1 = 0;
                        if (h00 > 1e-20) p0 = -((h01 + h01) * p1 + q[3]) / (2 * h00);
                        if (h11 > 1e-20) p1 = -((h01 + h01) * p0 + q[4]) / (2 * h11);
                        x[i] += p0;
                        y[i] += p1;
                        continue;
                    }
                    double det = h00 * h11 - h01 * h01;
                    if (std::fabs(det) > 1e-20)
                    {
                        double g0 = q[3], g1 = q[4];
                        double p0 = -(h11 * g0 - h01 * g1) / det / 2.;
                        double p1 = -(-h01 * g0 + h00 * g1) / det / 2.;
                        x[i] += p0;
                        y[i] += p1;
                    }
                }
            }
    }

    // prolongation x_f = P x_c (Hat.scalars.inl:1747-1779)
    void prolong(int level, const double *xc, double *xf) const
    {
        GridIdx<D> gc(1 << level), gf(1 << (level + 1));
        size_t Nf = gf.nodes();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)Nf; i++)
        {
            int F[D];
            gf.node((size_t)i, F);
            int nopt[D], opt[D][2];
            for (int d = 0; d < D; d++)
            {
                if (F[d] & 1) { nopt[d] = 2; opt[d][0] = (F[d] - 1) / 2; opt[d][1] = (F[d] + 1) / 2; }
                else { nopt[d] = 1; opt[d][0] = F[d] / 2; }
            }
            int sel[D];
            for (int d = 0; d < D; d++) sel[d] = 0;
            double s = 0;
            while (true)
            {
                double w = 1.;
                int I[D];
                for (int d = 0; d < D; d++) { I[d] = opt[d][sel[d]]; if (nopt[d] == 2) w *= 0.5; }
                s += w * xc[gc.node(I)];
                int d = D - 1;
                for (; d >= 0; d--) { if (++sel[d] < nopt[d]) break; sel[d] = 0; }
                if (d < 0) break;
            }
            // the adaptive prolongation reaches the indexed fine functions only (ffChildNeighbors,
            // Hat.scalars.inl:1747-1779)
            xf[i] = adaptive() && status[level + 1][i] == 0 ? 0. : s;
        }
    }

    // restriction v_c = P^T v_f (the transpose of prolong)
    void restrictT(int level, const double *vf, double *vc) const
    {
        GridIdx<D> gc(1 << level), gf(1 << (level + 1));
        size_t Nc = gc.nodes();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)Nc; i++)
        {
            int I[D];
            gc.node((size_t)i, I);
            double s = 0;
            for (int o = 0; o < T::S; o++)
            {
                int off[D], F[D];
                StencilOffset<D>(o, off);
                bool ok = true;
                double w = 1.;
                for (int d = 0; d < D; d++) { F[d] = 2 * I[d] + off[d]; if (F[d] < 0 || F[d] > gf.r) ok = false; if (off[d]) w *= 0.5; }
                if (ok) s += w * vf[gf.node(F)];
            }
            vc[i] = s;
        }
    }

    // gradient of E at (x,y): dE/dx_i = Q10(i), dE/dy_i = Q01(i)
    void gradient(int level, const double *x, const double *y, double *gx, double *gy) const
    {
        GridIdx<D> g(1 << level);
        size_t N = g.nodes();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++)
        {
            double q[5];
            quadfitNode(level, g, (size_t)i, x, y, q);
            gx[i] = q[3];
            gy[i] = q[4];
        }
    }

    // Gauss-Newton operator: (J^T J + A) applied to (dx, dy), with J(dx,dy) = W(dx,y) + W(x,dy)
    // the linearisation of the wedge residual; the result is half the Hessian of the GN model.
    void gnMatvec(int level, const double *x, const double *y, const double *dx, const double *dy, double *ox, double *oy) const
    {
        GridIdx<D> g(1 << level);
        size_t N = g.nodes();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++) gnNode(level, g, (size_t)i, x, y, dx, dy, &ox[i], &oy[i]);
    }

    // the Gauss-Newton product at the nodes idx[0..n) only (out[k] belongs to node idx[k]): the
    // same per-node arithmetic, for comparisons at sizes where the whole product is too slow here
    void gnMatvecAt(int level, const double *x, const double *y, const double *dx, const double *dy, const int64_t *idx,
                    size_t n, double *ox, double *oy) const
    {
        GridIdx<D> g(1 << level);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < (long)n; k++) gnNode(level, g, (size_t)idx[k], x, y, dx, dy, &ox[k], &oy[k]);
    }

    void quadfitAt(int level, const double *x, const double *y, const int64_t *idx, size_t n, double *out) const
    {
        GridIdx<D> g(1 << level);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < (long)n; k++) quadfitNode(level, g, (size_t)idx[k], x, y, &out[(size_t)k * 5]);
    }

    void gnNode(int level, const GridIdx<D> &g, size_t i, const double *x, const double *y, const double *dx,
                const double *dy, double *ox, double *oy) const
    {
        const LevelSystem &L = levels[level];
        int r = 1 << level;
        double vol = std::pow(1. / r, D);
        {
            int I[D];
            g.node(i, I);
            double sx = 0, sy = 0;
            for (int c = 0; c < (1 << D); c++)
            {
                int E[D];
                bool ok = true;
                for (int d = 0; d < D; d++) { E[d] = I[d] - ((c >> (D - 1 - d)) & 1); if (E[d] < 0 || E[d] >= r) ok = false; }
                if (!ok) continue;
                double xc[1 << D], yc[1 << D], dxc[1 << D], dyc[1 << D];
                gatherElement(g, E, x, y, xc, yc);
                gatherElement(g, E, dx, dy, dxc, dyc);
                for (int q = 0; q < T::Q; q++)
                {
                    double xi[D], w = vol;
                    int t = q;
                    for (int d = D - 1; d >= 0; d--) { xi[d] = GQ_X[t % 3]; w *= GQ_W[t % 3]; t /= 3; }
                    double gx[D], gy[D], gdx[D], gdy[D], gp[D];
                    CornerGrad(xc, xi, r, gx);
                    CornerGrad(yc, xi, r, gy);
                    CornerGrad(dxc, xi, r, gdx);
                    CornerGrad(dyc, xi, r, gdy);
                    HatGrad(c, xi, r, gp);
                    for (int a = 0; a < D; a++)
                        for (int b = 0; b < a; b++)
                        {
                            double Jd = 0.5 * (gy[a] * gdx[b] - gdx[a] * gy[b]) + 0.5 * (gdy[a] * gx[b] - gx[a] * gdy[b]);
                            double U = 0.5 * (gy[a] * gp[b] - gp[a] * gy[b]);
                            double V = 0.5 * (gp[a] * gx[b] - gx[a] * gp[b]);
                            sx += w * 2 * Jd * U;
                            sy += w * 2 * Jd * V;
                        }
                }
            }
            const double *a = &L.A[(size_t)i * T::S];
            *ox = sx + ColumnDot(g, a, I, dx);
            *oy = sy + ColumnDot(g, a, I, dy);
        }
    }

    // -------------------------------------------------------------------------------------------
    // Linear multigrid on column stencils (MG.h:37-195)
    // -------------------------------------------------------------------------------------------
    // one coloured Gauss-Seidel sweep of M x = b (GSRelaxer::operator() with colours, MG.h:57-72):
    // x_i += (b_i - sum_j M(j,i) x_j) / M(i,i), colours in order, nodes of a colour in parallel
    void linearGS(int level, const double *M, const double *b, double *x) const
    {
        GridIdx<D> g(1 << level);
        size_t N = g.nodes();
        const int oc = (T::S - 1) / 2;
        for (int col = 0; col < (1 << D); col++)
        {
#pragma omp parallel for schedule(static)
            for (long i = 0; i < (long)N; i++)
            {
                int I[D];
                g.node((size_t)i, I);
                int m = 0;
                for (int d = 0; d < D; d++) if (I[d] & 1) m |= 1 << d;
                if (m != col) continue;
                double v = ColumnDot(g, &M[(size_t)i * T::S], I, x);
                x[i] += (b[i] - v) / M[(size_t)i * T::S + oc];
            }
        }
    }

    // out = M x (matrix rows: M(i,j) is entry -off of node j's column, j = i + off)
    void applyRows(int level, const double *M, const double *x, double *out) const
    {
        GridIdx<D> g(1 << level);
        size_t N = g.nodes();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++)
        {
            int I[D];
            g.node((size_t)i, I);
            double s = 0;
            for (int o = 0; o < T::S; o++)
            {
                int off[D], J[D];
                StencilOffset<D>(o, off);
                bool ok = true;
                for (int d = 0; d < D; d++) { J[d] = I[d] + off[d]; if (J[d] < 0 || J[d] > g.r) ok = false; }
                if (!ok) continue;
                size_t j = g.node(J);
                s += M[j * T::S + (T::S - 1 - o)] * x[j];
            }
            out[i] = s;
        }
    }

    // dense LDL^T solve of the coarsest level (stands in for SimplicialLDLT, MG.h:105,131)
    static void DenseSolve(const GridIdx<D> &g, const double *M, const double *b, double *x)
    {
        size_t N = g.nodes();
        std::vector<double> A(N * N, 0.), L(N * N, 0.), Dg(N, 0.), z(N);
        for (size_t i = 0; i < N; i++)
        {
            int I[D];
            g.node(i, I);
            for (int o = 0; o < T::S; o++)
            {
                int off[D], J[D];
                StencilOffset<D>(o, off);
                bool ok = true;
                for (int d = 0; d < D; d++) { J[d] = I[d] + off[d]; if (J[d] < 0 || J[d] > g.r) ok = false; }
                if (ok) A[g.node(J) * N + i] = M[i * T::S + o];  // A(row j, col i)
            }
        }
        for (size_t j = 0; j < N; j++)
        {
            double d = A[j * N + j];
            for (size_t k = 0; k < j; k++) d -= L[j * N + k] * L[j * N + k] * Dg[k];
            Dg[j] = d;
            L[j * N + j] = 1.;
            for (size_t i = j + 1; i < N; i++)
            {
                double v = A[i * N + j];
                for (size_t k = 0; k < j; k++) v -= L[i * N + k] * L[j * N + k] * Dg[k];
                L[i * N + j] = v / d;
            }
        }
        for (size_t i = 0; i < N; i++)
        {
            double v = b[i];
            for (size_t k = 0; k < i; k++) v -= L[i * N + k] * z[k];
            z[i] = v;
        }
        for (size_t i = 0; i < N; i++) z[i] /= Dg[i];
        for (size_t ii = N; ii-- > 0;)
        {
            double v = z[ii];
            for (size_t k = ii + 1; k < N; k++) v -= L[k * N + ii] * x[k];
            x[ii] = v;
        }
    }

    void prolongScalar(int level, const double *c, double *f) const { prolong(level, c, f); }

    // V-cycle (MGSolver::vCycle with colours, MG.h:150-187) of M x = b on levels 0..top, with the
    // Galerkin hierarchy Ms (Ms[top] = M)
    void vcycle(const std::vector<std::vector<double>> &Ms, int top, const double *b, double *x, int iters) const
    {
        std::vector<std::vector<double>> Bs(top + 1), Xs(top + 1);
        for (int l = 0; l <= top; l++) { Bs[l].assign(NumNodes(D, l), 0.); Xs[l].assign(NumNodes(D, l), 0.); }
        std::copy(b, b + NumNodes(D, top), Bs[top].begin());
        std::copy(x, x + NumNodes(D, top), Xs[top].begin());
        for (int l = top; l > 0; l--)
        {
            for (int i = 0; i < iters; i++) linearGS(l, Ms[l].data(), Bs[l].data(), Xs[l].data());
            std::vector<double> r(NumNodes(D, l));
            applyRows(l, Ms[l].data(), Xs[l].data(), r.data());
            for (size_t i = 0; i < r.size(); i++) r[i] = Bs[l][i] - r[i];
            restrictT(l - 1, r.data(), Bs[l - 1].data());
            std::fill(Xs[l - 1].begin(), Xs[l - 1].end(), 0.);
        }
        DenseSolve(GridIdx<D>(1), Ms[0].data(), Bs[0].data(), Xs[0].data());
        for (int l = 1; l <= top; l++)
        {
            std::vector<double> p(NumNodes(D, l));
            prolong(l - 1, Xs[l - 1].data(), p.data());
            for (size_t i = 0; i < p.size(); i++) Xs[l][i] += p[i];
            for (int i = 0; i < iters; i++) linearGS(l, Ms[l].data(), Bs[l].data(), Xs[l].data());
        }
        std::copy(Xs[top].begin(), Xs[top].end(), x);
    }

    // Galerkin hierarchy of a finest-level operator (MGSolver ctor, MG.h:93-107)
    std::vector<std::vector<double>> hierarchy(const double *M, int top) const
    {
        std::vector<std::vector<double>> Ms(top + 1);
        Ms[top].assign(M, M + NumNodes(D, top) * T::S);
        for (int l = top; l > 0; l--) Ms[l - 1] = galerkin(Ms[l], l);
        return Ms;
    }

    // -------------------------------------------------------------------------------------------
    // Alternating solve (ExteriorPoissonSolvers.h:86-154)
    // -------------------------------------------------------------------------------------------
    // Gram matrix of the wedge with a fixed field f as a column stencil:
    //   G(j, i) = int <W(f, phi_j), W(f, phi_i)>_F,   so that  |W(f, v)|^2 = v^T G v
    // (and |W(v, f)|^2 too: W is antisymmetric in its arguments).
    void wedgeGram(int level, const double *f, double *G) const
    {
        int r = 1 << level;
        GridIdx<D> g(r);
        size_t N = g.nodes();
        double vol = std::pow(1. / r, D);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++)
        {
            int I[D];
            g.node((size_t)i, I);
            double *col = &G[(size_t)i * T::S];
            for (int o = 0; o < T::S; o++) col[o] = 0;
            for (int A = 0; A < (1 << D); A++)
            {
                int E[D];
                bool ok = true;
                for (int d = 0; d < D; d++) { E[d] = I[d] - ((A >> (D - 1 - d)) & 1); if (E[d] < 0 || E[d] >= r) ok = false; }
                if (!ok) continue;
                double fc[1 << D], dummy[1 << D];
                gatherElement(g, E, f, f, fc, dummy);
                for (int q = 0; q < T::Q; q++)
                {
                    double xi[D], w = vol;
                    int t = q;
                    for (int d = D - 1; d >= 0; d--) { xi[d] = GQ_X[t % 3]; w *= GQ_W[t % 3]; t /= 3; }
                    double gf[D], ga[D];
                    CornerGrad(fc, xi, r, gf);
                    HatGrad(A, xi, r, ga);
                    for (int Bc = 0; Bc < (1 << D); Bc++)
                    {
                        double gb[D];
                        HatGrad(Bc, xi, r, gb);
                        double s = 0;
                        for (int a = 0; a < D; a++)
                            for (int b = 0; b < a; b++)
                            {
                                double Va = 0.5 * (ga[a] * gf[b] - gf[a] * ga[b]);
                                double Vb = 0.5 * (gb[a] * gf[b] - gf[a] * gb[b]);
                                s += 2 * Va * Vb;
                            }
                        int off[D];
                        for (int d = 0; d < D; d++) off[d] = ((Bc >> (D - 1 - d)) & 1) - ((A >> (D - 1 - d)) & 1);
                        col[StencilOffsetIndex<D>(off)] += w * s;
                    }
                }
            }
        }
    }

    // sum_j B(j, i) v_j without the diagonal (B is antisymmetric, so this is also -(B v)_i)
    double BColumnDot(const GridIdx<D> &g, const double *col, const int *I, const double *v) const
    {
        double s = 0;
        for (int o = 0; o < T::S; o++)
        {
            if (o == (T::S - 1) / 2 || col[o] == 0) continue;
            int off[D], J[D];
            StencilOffset<D>(o, off);
            bool ok = true;
            for (int d = 0; d < D; d++) { J[d] = I[d] + off[d]; if (J[d] < 0 || J[d] > g.r) ok = false; }
            if (ok) s += col[o] * v[g.node(J)];
        }
        return s;
    }

    // The linear system of one alternating half-step, as AlternatingSolve forms it from a
    // quadratic approximation q (q.q *= 2, q.l = -q.l; ExteriorPoissonSolvers.h:101-104, 120-123):
    //   which == 1 (y free, x fixed):  2 (G_x + A) y = 2 B x
    //   which == 0 (x free, y fixed):  2 (G_y + A) x = 2 B^T y
    // from E = |W(x,y)|^2 - 2 y^T B x + c + x^T A x + y^T A y.
    void alternatingSystem(int level, const double *x, const double *y, int which, double *M, double *b) const
    {
        const LevelSystem &L = levels[level];
        GridIdx<D> g(1 << level);
        size_t N = g.nodes();
        wedgeGram(level, which ? x : y, M);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)N; i++)
        {
            int I[D];
            g.node((size_t)i, I);
            for (int o = 0; o < T::S; o++) M[(size_t)i * T::S + o] = 2. * (M[(size_t)i * T::S + o] + L.A[(size_t)i * T::S + o]);
            const double *bc = &L.B[(size_t)i * T::S];
            b[i] = which ? -2. * BColumnDot(g, bc, I, x) : 2. * BColumnDot(g, bc, I, y);
        }
    }

    // AlternatingSolve with sType MULTIGRID (V-cycles on the Galerkin hierarchy down to level 0)
    // or SINGLE_LEVEL (gsIters * vCycles coloured GS sweeps)
    void alternatingSolve(int level, double *x, double *y, int iters, int vCycles, int gsIters, bool singleLevel) const
    {
        size_t N = NumNodes(D, level);
        std::vector<double> M(N * T::S), b(N);
        for (int it = 0; it < iters; it++)
        {
            for (int which = 1; which >= 0; which--)
            {
                double *v = which ? y : x;
                alternatingSystem(level, x, y, which, M.data(), b.data());
                if (singleLevel)
                    for (int k = 0; k < gsIters * vCycles; k++) linearGS(level, M.data(), b.data(), v);
                else
                {
                    auto Ms = hierarchy(M.data(), level);
                    for (int k = 0; k < vCycles; k++) vcycle(Ms, level, b.data(), v, gsIters);
                }
            }
        }
    }

    // -------------------------------------------------------------------------------------------
    // Bi-quadratic fit P(s,t) = E(x + s dx, y + t dy); q[i*3 + j] is the coefficient of s^i t^j.
    // asReference reproduces SingleCycleCascadicSystemEnergy::biQuadraticFit (SystemEnergy.h:
    // 499-540) term by term, which differs from the exact expansion in two places:
    //   * the s t^2 coefficient is 2 <W(dx,dy), W(x,y)> (SystemEnergy.h:506) where the expansion
    //     has 2 <W(dx,dy), W(x,dy)>;
    //   * the stiffness term enters with weight 1 (SystemEnergy.h:522-530) where energies() weights
    //     it by sWeight (= dWeight, SystemEnergy.h:494).
    // -------------------------------------------------------------------------------------------
    void biQuadraticFit(int level, const double *x, const double *y, const double *dx, const double *dy, double *q,
                        bool asReference = false) const
    {
        const LevelSystem &L = levels[level];
        std::vector<double> Aref;
        const double *Abase = L.A.data();
        if (asReference)
        {
            std::vector<double> K = stiffnessStencil(level);
            Aref.resize(L.A.size());
            for (size_t i = 0; i < Aref.size(); i++) Aref[i] = L.A[i] + (1. - P.d_weight) * K[i];
            Abase = Aref.data();
        }
        int r = 1 << level;
        GridIdx<D> g(r);
        size_t NE = g.elems(), N = g.nodes();
        double vol = std::pow(1. / r, D);
        // <P,Q> of the four wedges W(x,y), W(dx,y), W(x,dy), W(dx,dy)
        double w00 = 0, w20 = 0, w02 = 0, w22 = 0, w21 = 0, w12 = 0, w11a = 0, w11b = 0, w10 = 0, w01 = 0;
#pragma omp parallel for schedule(static) reduction(+ : w00, w20, w02, w22, w21, w12, w11a, w11b, w10, w01)
        for (long e = 0; e < (long)NE; e++)
        {
            int E[D];
            g.elem((size_t)e, E);
            double xc[1 << D], yc[1 << D], dxc[1 << D], dyc[1 << D];
            gatherElement(g, E, x, y, xc, yc);
            gatherElement(g, E, dx, dy, dxc, dyc);
            for (int qp = 0; qp < T::Q; qp++)
            {
                double xi[D], w = vol;
                int t = qp;
                for (int d = D - 1; d >= 0; d--) { xi[d] = GQ_X[t % 3]; w *= GQ_W[t % 3]; t /= 3; }
                double gx[D], gy[D], gdx[D], gdy[D];
                CornerGrad(xc, xi, r, gx);
                CornerGrad(yc, xi, r, gy);
                CornerGrad(dxc, xi, r, gdx);
                CornerGrad(dyc, xi, r, gdy);
                for (int a = 0; a < D; a++)
                    for (int b = 0; b < a; b++)
                    {
                        auto W = [&](const double *u, const double *v) { return 0.5 * (v[a] * u[b] - u[a] * v[b]); };
                        double Wxy = W(gx, gy), WXy = W(gdx, gy), WxY = W(gx, gdy), WXY = W(gdx, gdy);
                        double s = 2 * w;
                        w22 += s * WXY * WXY;
                        w21 += s * WXY * WXy;
                        w12 += s * WXY * WxY;
                        w20 += s * WXy * WXy;
                        w02 += s * WxY * WxY;
                        w11a += s * WXy * WxY;
                        w11b += s * WXY * Wxy;
                        w10 += s * WXy * Wxy;
                        w01 += s * WxY * Wxy;
                        w00 += s * Wxy * Wxy;
                    }
            }
        }
        double aXX = 0, axX = 0, axx = 0, aYY = 0, ayY = 0, ayy = 0, bYX = 0, bYx = 0, byX = 0, byx = 0;
#pragma omp parallel for schedule(static) reduction(+ : aXX, axX, axx, aYY, ayY, ayy, bYX, bYx, byX, byx)
        for (long i = 0; i < (long)N; i++)
        {
            int I[D];
            g.node((size_t)i, I);
            const double *a = &Abase[(size_t)i * T::S], *b = &L.B[(size_t)i * T::S];
            double Adx = ColumnDot(g, a, I, dx), Ax = ColumnDot(g, a, I, x);
            double Ady = ColumnDot(g, a, I, dy), Ay = ColumnDot(g, a, I, y);
            double Bdy = ColumnDot(g, b, I, dy), By = ColumnDot(g, b, I, y);
            aXX += dx[i] * Adx; axX += x[i] * Adx; axx += x[i] * Ax;
            aYY += dy[i] * Ady; ayY += y[i] * Ady; ayy += y[i] * Ay;
            // y^T B x = sum_i x_i sum_j B(j,i) y_j, as in energy()
            bYX += dx[i] * Bdy; bYx += x[i] * Bdy; byX += dx[i] * By; byx += x[i] * By;
        }
        for (int k = 0; k < 9; k++) q[k] = 0;
        auto Q = [&](int i, int j) -> double & { return q[i * 3 + j]; };
        Q(2, 2) += w22;
        Q(2, 1) += 2 * w21;
        Q(1, 2) += 2 * (asReference ? w11b : w12);
        Q(2, 0) += w20;
        Q(0, 2) += w02;
        Q(1, 1) += 2 * w11a + 2 * w11b;
        Q(1, 0) += 2 * w10;
        Q(0, 1) += 2 * w01;
        Q(0, 0) += w00;
        Q(2, 0) += aXX; Q(1, 0) += 2 * axX; Q(0, 0) += axx;
        Q(0, 2) += aYY; Q(0, 1) += 2 * ayY; Q(0, 0) += ayy;
        Q(1, 1) += -2 * bYX; Q(0, 1) += -2 * bYx; Q(1, 0) += -2 * byX; Q(0, 0) += -2 * byx;
        Q(0, 0) += c;
    }

    // Random<double> (Misha/Geometry.inl:430-438) on the C library generator
    static double RandomDouble()
    {
        const unsigned long long ULL_RAND_MAX = (unsigned long long)(RAND_MAX) + 1;
        const double RAND_MAX_SQUARED = double(ULL_RAND_MAX * ULL_RAND_MAX - 1);
        unsigned long long r1 = rand();
        unsigned long long r2 = rand();
        long long v = (long long)(r1 * ULL_RAND_MAX + r2);
        return double(v) / RAND_MAX_SQUARED;
    }

    // the unscaled random start: two draws per function in function-index order
    // (ExteriorPoisson.h:333-334), the adaptive indexer's order when there is one
    void randomStart(int l, std::vector<double> &X, std::vector<double> &Y) const
    {
        if (!adaptive())
        {
            for (size_t i = 0; i < X.size(); i++) { X[i] = RandomDouble(); Y[i] = RandomDouble(); }
            return;
        }
        for (int64_t node : fnodes[l]) { X[(size_t)node] = RandomDouble(); Y[(size_t)node] = RandomDouble(); }
    }

    // cascadic solve (ExteriorPoisson.h:315-409)
    void solve(double *xout, double *yout, double *eout)
    {
        int minD = std::min(P.min_solve_depth, depth);
        int maxD = P.max_solve_depth < 0 ? depth : std::min(P.max_solve_depth, depth);
        std::vector<std::vector<double>> X(depth + 1), Y(depth + 1);
        for (int l = 0; l <= depth; l++) { X[l].assign(NumNodes(D, l), 0.); Y[l].assign(NumNodes(D, l), 0.); }
        srand(P.seed);
        randomStart(minD, X[minD], Y[minD]);
        {
            double e[3];
            energy(minD, X[minD].data(), Y[minD].data(), e);
            double s = std::sqrt(std::sqrt(c / e[2]));
            for (size_t i = 0; i < X[minD].size(); i++) { X[minD][i] *= s; Y[minD][i] *= s; }
        }
        if (P.single_level)
        {
            // ExteriorPoisson.h:342-360
            for (int l = minD; l < maxD; l++)
            {
                prolong(l, X[l].data(), X[l + 1].data());
                prolong(l, Y[l].data(), Y[l + 1].data());
            }
            for (int l = minD; l < maxD; l++)
            {
                std::fill(X[l].begin(), X[l].end(), 0.);
                std::fill(Y[l].begin(), Y[l].end(), 0.);
            }
            gs(maxD, X[maxD].data(), Y[maxD].data(), P.gs_iters);
        }
        for (int l = minD; !P.single_level && l <= maxD; l++)
        {
            int iters = (int)std::ceil(std::pow(P.i_mult, depth - l) * P.gs_iters);
            if (P.alt_rounds > 0) alternatingSolve(l, X[l].data(), Y[l].data(), P.alt_rounds, 1, P.gs_iters, false);
            else gs(l, X[l].data(), Y[l].data(), iters);
            if (l < maxD)
            {
                std::vector<double> px(X[l + 1].size()), py(Y[l + 1].size());
                prolong(l, X[l].data(), px.data());
                prolong(l, Y[l].data(), py.data());
                for (size_t i = 0; i < px.size(); i++) { X[l + 1][i] += px[i]; Y[l + 1][i] += py[i]; }
            }
        }
        double e[3];
        energy(maxD, X[maxD].data(), Y[maxD].data(), e);
        eout[0] = c; eout[1] = e[0]; eout[2] = e[1];
        for (int l = maxD; l < depth; l++)
        {
            prolong(l, X[l].data(), X[l + 1].data());
            prolong(l, Y[l].data(), Y[l + 1].data());
        }
        for (int l = depth; l > 0; l--)
        {
            std::vector<double> px(X[l].size()), py(Y[l].size());
            prolong(l - 1, X[l - 1].data(), px.data());
            prolong(l - 1, Y[l - 1].data(), py.data());
            for (size_t i = 0; i < px.size(); i++) { X[l][i] -= px[i]; Y[l][i] -= py[i]; }
        }
        size_t off = 0;
        for (int l = 0; l <= depth; l++)
        {
            std::copy(X[l].begin(), X[l].end(), xout + off);
            std::copy(Y[l].begin(), Y[l].end(), yout + off);
            off += X[l].size();
        }
    }

    // The cascadic schedule of solve() (ExteriorPoisson.h:315-409, paired GS only) run in pieces,
    // so that a caller can time one whole solve in several bounded parts: begin() sets the random
    // start, advance() relaxes whole sweeps in schedule order (prolonging at each level's end)
    // until `target` node updates have been done since begin(), finish() returns the energies.
    // The arithmetic is solve()'s, sweep for sweep.
    struct Stepper
    {
        std::vector<std::vector<double>> X, Y;
        int level = 0, sweep = 0, minD = 0, maxD = 0;
        int64_t done = 0, total = 0;
    } st;

    int64_t sweepsAt(int l) const { return (int64_t)std::ceil(std::pow(P.i_mult, depth - l) * P.gs_iters); }

    int64_t solveBegin()
    {
        st = Stepper();
        st.minD = std::min(P.min_solve_depth, depth);
        st.maxD = P.max_solve_depth < 0 ? depth : std::min(P.max_solve_depth, depth);
        st.X.resize(depth + 1);
        st.Y.resize(depth + 1);
        for (int l = 0; l <= depth; l++) { st.X[l].assign(NumNodes(D, l), 0.); st.Y[l].assign(NumNodes(D, l), 0.); }
        srand(P.seed);
        std::vector<double> &X0 = st.X[st.minD], &Y0 = st.Y[st.minD];
        randomStart(st.minD, X0, Y0);
        double e[3];
        energy(st.minD, X0.data(), Y0.data(), e);
        double s = std::sqrt(std::sqrt(c / e[2]));
        for (size_t i = 0; i < X0.size(); i++) { X0[i] *= s; Y0[i] *= s; }
        st.level = st.minD;
        for (int l = st.minD; l <= st.maxD; l++) st.total += sweepsAt(l) * (int64_t)NumNodes(D, l);
        return st.total;
    }

    // returns 1 when the schedule is complete
    int solveAdvance(int64_t target)
    {
        while (st.level <= st.maxD && st.done < target)
        {
            const int l = st.level;
            gs(l, st.X[l].data(), st.Y[l].data(), 1);
            st.done += (int64_t)NumNodes(D, l);
            if (++st.sweep == sweepsAt(l))
            {
                if (l < st.maxD)
                {
                    std::vector<double> px(st.X[l + 1].size()), py(st.Y[l + 1].size());
                    prolong(l, st.X[l].data(), px.data());
                    prolong(l, st.Y[l].data(), py.data());
                    for (size_t i = 0; i < px.size(); i++) { st.X[l + 1][i] += px[i]; st.Y[l + 1][i] += py[i]; }
                }
                st.level++;
                st.sweep = 0;
            }
        }
        return st.level > st.maxD ? 1 : 0;
    }

    void solveFinish(double *eout)
    {
        double e[3];
        energy(st.maxD, st.X[st.maxD].data(), st.Y[st.maxD].data(), e);
        eout[0] = c; eout[1] = e[0]; eout[2] = e[1];
    }

    long get(const std::string &name, int level, double *out) const
    {
        auto put = [&](const std::vector<double> &v) { if (out) std::copy(v.begin(), v.end(), out); return (long)v.size(); };
        if (name == "measure") return put(measure);
        if (name == "noise") return put(noise);
        if (name == "depth") return put(sdepth);
        if (name == "S") return put(S);
        if (name == "c") return put(std::vector<double>{c});
        if (name == "leaf_depth") { std::vector<double> v(leafDepth.begin(), leafDepth.end()); return put(v); }
        if (name == "cells")
        {
            std::vector<double> v;
            for (size_t i = 0; i < cells.size(); i++) for (int d = 0; d < D; d++) v.push_back(cells[i][d]);
            return put(v);
        }
        if (name == "cell_counts")
        {
            std::vector<double> v;
            for (size_t i = 0; i < cells.size(); i++) v.push_back((double)(cellStart[i + 1] - cellStart[i]));
            return put(v);
        }
        if (name == "density_refined")
        {
            // 1 where the density tree's depth-`level` cell has children (level 0..depth+1)
            if (level < 0 || level > depth + 1) return -1;
            std::vector<double> v(density.refined[level].begin(), density.refined[level].end());
            return put(v);
        }
        if (level < 0 || level > depth) return -1;
        if (name == "status" || name == "fnodes" || name == "enodes" || name == "nactive")
        {
            if (!adaptive()) return -1;
            if (name == "nactive") return put(std::vector<double>{(double)nActive[level]});
            const auto &src = name == "fnodes" ? fnodes[level] : enodes[level];
            std::vector<double> v;
            if (name == "status") v.assign(status[level].begin(), status[level].end());
            else v.assign(src.begin(), src.end());
            return put(v);
        }
        if (name == "R") return put(levels[level].R);
        if (name == "B") return put(levels[level].B);
        if (name == "A") return put(levels[level].A);
        if (name == "density") return put(density.data[level]);
        if (name == "skew") return put(skewTree.data[level]);
        return -1;
    }
};

}  // namespace

struct epr_oracle
{
    int dim;
    void *impl;
};

#define DISPATCH(o, ...)                                                         \
    do {                                                                         \
        if ((o)->dim == 3) { auto *self = (Oracle<3> *)(o)->impl; __VA_ARGS__; } \
        else { auto *self = (Oracle<4> *)(o)->impl; __VA_ARGS__; }               \
    } while (0)

extern "C" {

void epr_oracle_default_params(epr_oracle_params *p)
{
    p->s_weight = 100.;
    p->d_weight = 0.00625;
    p->n_sigma = 0.25;
    p->i_mult = 2.;
    p->project = 0;
    p->t_radius = 1;
    p->d_radius = 1;
    p->gs_iters = 10;
    p->min_solve_depth = 0;
    p->max_solve_depth = -1;
    p->seed = 0;
    p->threads = 0;
    p->single_level = 0;
    p->separate = 0;
    p->alt_rounds = 0;
    p->adaptive_radius = -1;
}

int epr_oracle_unit_cube(int dim, size_t n, double scale, double *pos, double *xform)
{
    if (dim != 3 && dim != 4) return -1;
    if (n == 0) return -2;
    int D = dim;
    std::vector<double> lo(pos, pos + D), hi(pos, pos + D);
    for (size_t i = 1; i < n; i++)
        for (int d = 0; d < D; d++) { lo[d] = std::min(lo[d], pos[i * D + d]); hi[d] = std::max(hi[d], pos[i * D + d]); }
    double ext = hi[0] - lo[0];
    for (int d = 1; d < D; d++) ext = std::max(ext, hi[d] - lo[d]);
    double k = 1. / (ext * scale);
    // xform = t1 * s * t2 in the reference's (column, row) layout
    int W = D + 1;
    for (int i = 0; i < W * W; i++) xform[i] = 0;
    std::vector<double> t(D);
    for (int d = 0; d < D; d++)
    {
        double c2 = -(lo[d] + hi[d]) / 2.;
        t[d] = c2 * k + 0.5;
        xform[d * W + d] = k;
        xform[D * W + d] = t[d];
    }
    xform[D * W + D] = 1.;
    for (size_t i = 0; i < n; i++)
        for (int d = 0; d < D; d++) pos[i * D + d] = pos[i * D + d] * k + t[d];
    return 0;
}

epr_oracle *epr_oracle_create(int dim, int depth, const epr_oracle_params *p)
{
    if ((dim != 3 && dim != 4) || depth < 1 || depth > 12) return nullptr;
    epr_oracle_params pp;
    if (p) pp = *p; else epr_oracle_default_params(&pp);
#ifdef _OPENMP
    if (pp.threads > 0) omp_set_num_threads(pp.threads);
#endif
    epr_oracle *o = new epr_oracle;
    o->dim = dim;
    if (dim == 3) o->impl = new Oracle<3>(depth, pp);
    else o->impl = new Oracle<4>(depth, pp);
    return o;
}

void epr_oracle_destroy(epr_oracle *o)
{
    if (!o) return;
    if (o->dim == 3) delete (Oracle<3> *)o->impl;
    else delete (Oracle<4> *)o->impl;
    delete o;
}

int epr_oracle_set_samples(epr_oracle *o, size_t n, const double *pos, const double *skew)
{
    if (!o || !n) return -1;
    DISPATCH(o, {
        self->n = n;
        self->pos.assign(pos, pos + n * o->dim);
        self->skew.assign(skew, skew + n * (o->dim * (o->dim - 1) / 2));
    });
    return 0;
}

int epr_oracle_build(epr_oracle *o)
{
    if (!o) return -1;
    DISPATCH(o, { if (!self->n) return -2; self->build(); });
    return 0;
}

int epr_oracle_set_level_system(epr_oracle *o, int level, const double *R, const double *B, double c)
{
    if (!o) return -1;
    DISPATCH(o, {
        if (level < 0 || level > self->depth) return -2;
        size_t N = NumNodes(o->dim, level), S = (size_t)std::pow(3, o->dim);
        LevelSystem &L = self->levels[level];
        L.R.assign(R, R + N * S);
        L.B.assign(B, B + N * S);
        std::vector<double> K = self->stiffnessStencil(level);
        L.A.resize(N * S);
        for (size_t i = 0; i < N * S; i++) L.A[i] = L.R[i] + self->P.d_weight * K[i];
        self->c = c;
    });
    return 0;
}

long epr_oracle_get(epr_oracle *o, const char *name, int level, double *out)
{
    if (!o) return -1;
    DISPATCH(o, { return self->get(name, level, out); });
    return -1;
}

size_t epr_oracle_num_nodes(int dim, int level) { return NumNodes(dim, level); }

int epr_oracle_energy(epr_oracle *o, int level, const double *x, const double *y, double *out)
{
    if (!o) return -1;
    DISPATCH(o, { self->energy(level, x, y, out); });
    return 0;
}

int epr_oracle_quadfit(epr_oracle *o, int level, const double *x, const double *y, double *out)
{
    if (!o) return -1;
    DISPATCH(o, { self->quadfit(level, x, y, out); });
    return 0;
}

int epr_oracle_quadfit_at(epr_oracle *o, int level, const double *x, const double *y, const int64_t *idx, size_t n,
                          double *out)
{
    if (!o) return -1;
    DISPATCH(o, { self->quadfitAt(level, x, y, idx, n, out); });
    return 0;
}

int epr_oracle_gn_matvec_at(epr_oracle *o, int level, const double *x, const double *y, const double *dx,
                            const double *dy, const int64_t *idx, size_t n, double *ox, double *oy)
{
    if (!o) return -1;
    DISPATCH(o, { self->gnMatvecAt(level, x, y, dx, dy, idx, n, ox, oy); });
    return 0;
}

int epr_oracle_gradient(epr_oracle *o, int level, const double *x, const double *y, double *gx, double *gy)
{
    if (!o) return -1;
    DISPATCH(o, { self->gradient(level, x, y, gx, gy); });
    return 0;
}

int epr_oracle_gs(epr_oracle *o, int level, double *x, double *y, int iters)
{
    if (!o) return -1;
    DISPATCH(o, { self->gs(level, x, y, iters); });
    return 0;
}

int epr_oracle_gs_shifted(epr_oracle *o, int level, double *x, double *y, int iters, const double *tx, const double *ty)
{
    if (!o) return -1;
    DISPATCH(o, { self->gs(level, x, y, iters, tx, ty); });
    return 0;
}

int epr_oracle_linear_gs(epr_oracle *o, int level, const double *M, const double *b, double *x)
{
    if (!o) return -1;
    DISPATCH(o, { self->linearGS(level, M, b, x); });
    return 0;
}

int epr_oracle_mg_vcycle(epr_oracle *o, int level, const double *M, const double *b, double *x, int iters, int cycles)
{
    if (!o) return -1;
    DISPATCH(o, {
        auto Ms = self->hierarchy(M, level);
        for (int c = 0; c < cycles; c++) self->vcycle(Ms, level, b, x, iters);
    });
    return 0;
}

int epr_oracle_wedge_gram(epr_oracle *o, int level, const double *f, double *G)
{
    if (!o) return -1;
    DISPATCH(o, { self->wedgeGram(level, f, G); });
    return 0;
}

int epr_oracle_alternating_system(epr_oracle *o, int level, const double *x, const double *y, int which, double *M, double *b)
{
    if (!o) return -1;
    DISPATCH(o, { self->alternatingSystem(level, x, y, which, M, b); });
    return 0;
}

int epr_oracle_alternating_solve(epr_oracle *o, int level, double *x, double *y, int iters, int vcycles, int gs_iters, int single_level)
{
    if (!o) return -1;
    DISPATCH(o, { self->alternatingSolve(level, x, y, iters, vcycles, gs_iters, single_level != 0); });
    return 0;
}

int epr_oracle_biquadratic_fit(epr_oracle *o, int level, const double *x, const double *y, const double *dx, const double *dy, double *q9,
                               int as_reference)
{
    if (!o) return -1;
    DISPATCH(o, { self->biQuadraticFit(level, x, y, dx, dy, q9, as_reference != 0); });
    return 0;
}

double epr_oracle_step_size(const double *q9) { return StepSize(q9); }

void epr_oracle_newton_update(const double *q9, int steps, double *st) { NewtonUpdate(q9, steps, st); }

int epr_oracle_restrict(epr_oracle *o, int level, const double *fine, double *coarse)
{
    if (!o) return -1;
    DISPATCH(o, { self->restrictT(level, fine, coarse); });
    return 0;
}

int epr_oracle_prolong(epr_oracle *o, int level, const double *coarse, double *fine)
{
    if (!o) return -1;
    DISPATCH(o, { self->prolong(level, coarse, fine); });
    return 0;
}

int epr_oracle_gn_matvec(epr_oracle *o, int level, const double *x, const double *y, const double *dx,
                         const double *dy, double *ox, double *oy)
{
    if (!o) return -1;
    DISPATCH(o, { self->gnMatvec(level, x, y, dx, dy, ox, oy); });
    return 0;
}

int64_t epr_oracle_solve_begin(epr_oracle *o)
{
    if (!o) return -1;
    DISPATCH(o, { return self->solveBegin(); });
    return -1;
}

int epr_oracle_solve_advance(epr_oracle *o, int64_t target_node_updates)
{
    if (!o) return -1;
    DISPATCH(o, { return self->solveAdvance(target_node_updates); });
    return -1;
}

int epr_oracle_solve_finish(epr_oracle *o, double *energies_out)
{
    if (!o) return -1;
    DISPATCH(o, { self->solveFinish(energies_out); });
    return 0;
}

int epr_oracle_solve(epr_oracle *o, double *x_out, double *y_out, double *energies_out)
{
    if (!o) return -1;
    DISPATCH(o, { self->solve(x_out, y_out, energies_out); });
    return 0;
}

}  // extern "C"
