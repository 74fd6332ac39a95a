// Test-infrastructure only: a dump tool that links the reference implementation's own headers
// (compiled from the reference checkout by oracle/Makefile into oracle/_ref/) and writes the
// intermediate quantities of the regular-grid reconstruction as .npy files, so that the CPU
// restatement in oracle/epr_oracle.cpp and the CUDA path can be pinned against the reference.
//
// It is never shipped and never timed.  It calls the reference API as a user would:
//   ToUnitCube / OrderedSampler / TreeEstimator / Reconstructor  (ExteriorPoisson.h:100-313,
//   ExteriorPoissonRecon.cpp:163-245), SingleCycleCascadicSystemEnergy::energies / quadraticFit
//   (SystemEnergy.h:486-643), PairedGaussSeidelSolve (ExteriorPoissonSolvers.h:156-196).
//
// usage: ref_harness <in.ply> <depth> <outdir> [--sWeight v] [--dWeight v] [--nSigma v]
//                    [--tRadius k] [--dRadius k] [--gsIters k] [--iMult v] [--seed k] [--scale v]
//                    [--minSolveDepth k] [--solve 0|1] [--aRadius k]

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <string>
#include <vector>
#include <random>
#include <fstream>
#include <sstream>
#include <iostream>
#include <iomanip>
#include <functional>
#include <map>
#include <unordered_map>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <typeinfo>
#include <sys/stat.h>

// The reference keeps the members this harness inspects (system matrices, solution levels,
// tree nodes) protected; expose them for reading.
#define protected public
#define private public
#include "Misha/Miscellany.h"
#include "Misha/Geometry.h"
#include "Misha/Ply.h"
#include "Misha/PlyVertexData.h"
#include "Misha/MultiThreading.h"
#include "ExteriorPoissonRecon/ExteriorPoisson.h"
#undef protected
#undef private

using namespace MishaK;

// ------------------------------------------------------------------------------------------
// .npy writer
// ------------------------------------------------------------------------------------------
static void WriteNpy(const std::string &path, const char *descr, size_t elemSize, const void *data,
                     const std::vector<size_t> &shape)
{
    std::string sh = "(";
    for (size_t i = 0; i < shape.size(); i++) sh += std::to_string(shape[i]) + (shape.size() == 1 ? "," : (i + 1 < shape.size() ? ", " : ""));
    sh += ")";
    std::string dict = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + sh + ", }";
    size_t headerLen = 10 + dict.size() + 1;
    size_t pad = (64 - headerLen % 64) % 64;
    dict += std::string(pad, ' ') + "\n";
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(1); }
    const unsigned char magic[] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    fwrite(magic, 1, 8, fp);
    uint16_t hl = (uint16_t)dict.size();
    fwrite(&hl, 2, 1, fp);
    fwrite(dict.data(), 1, dict.size(), fp);
    size_t n = 1;
    for (size_t s : shape) n *= s;
    fwrite(data, elemSize, n, fp);
    fclose(fp);
}
static void SaveF64(const std::string &p, const std::vector<double> &v, std::vector<size_t> shape) { WriteNpy(p, "<f8", 8, v.data(), shape); }
static void SaveI64(const std::string &p, const std::vector<int64_t> &v, std::vector<size_t> shape) { WriteNpy(p, "<i8", 8, v.data(), shape); }

// ------------------------------------------------------------------------------------------
// parameters
// ------------------------------------------------------------------------------------------
struct Params
{
    double sWeight = 100., dWeight = 0.00625, nSigma = 0.25, iMult = 2., scale = 1.1;
    unsigned int tRadius = 1, dRadius = 1, gsIters = 10, seed = 0, minSolveDepth = 0;
    int solve = 1;
    int separate = 0, singleLevel = 0;
    int project = 0;  // --project: the reference's blade projection of S(E) (ExteriorPoisson.h:300-305)
    int aRadius = -1;  // --aRadius >= 0: the adaptive indexer (ExteriorPoissonRecon.cpp:191-198)
};

template <unsigned int Dim>
static std::vector<std::pair<Point<double, Dim>, Hat::SkewSymmetricMatrix<double, Dim>>> ReadSamples(const std::string &fileName)
{
    std::vector<std::pair<Point<double, Dim>, Hat::SkewSymmetricMatrix<double, Dim>>> hermiteData;
    using Factory = VertexFactory::Factory<double, VertexFactory::PositionFactory<double, Dim>, VertexFactory::MatrixFactory<double, Dim, Dim>>;
    Factory factory = Factory(VertexFactory::PositionFactory<double, Dim>(), VertexFactory::MatrixFactory<double, Dim, Dim>("skew"));
    std::vector<typename Factory::VertexType> vertices;
    std::vector<SimplexIndex<Dim - 2, unsigned int>> simplexIndices;
    PLY::ReadSimplices(fileName, factory, vertices, simplexIndices, NULL);
    hermiteData.resize(vertices.size());
    for (size_t i = 0; i < vertices.size(); i++)
    {
        hermiteData[i].first = vertices[i].template get<0>();
        hermiteData[i].second = Hat::SkewSymmetricMatrix<double, Dim>(vertices[i].template get<1>());
    }
    return hermiteData;
}

// Stencil layout used by every dump: entry o of node i holds M(i + off(o), i), where the offset
// index o = sum_d (off[d] + 1) * 3^(Dim-1-d) enumerates {-1,0,1}^Dim with axis 0 slowest, and the
// node index is the reference function index (axis 0 most significant, Hat.scalars.inl:476-481).
// For the adaptive indexer the matrix rows and columns are the indexer's function indices; `offsets`
// maps each to its grid offset, and the stencil of the grid node of that offset is written.
template <unsigned int Dim>
static std::vector<double> ColumnStencil(const Eigen::SparseMatrix<double> &M, unsigned int res,
                                         const std::vector<Hat::Index<Dim>> *offsets = nullptr)
{
    const unsigned int S = (unsigned int)std::pow(3, Dim);
    size_t N = (size_t)std::pow(res + 1, Dim);
    std::vector<double> out(N * S, 0.);
    auto offsetOf = [&](size_t f) { return offsets ? (*offsets)[f] : Hat::ScalarFunctions<Dim>::FunctionIndex(f, res); };
    for (int col = 0; col < M.outerSize(); col++)
        for (Eigen::SparseMatrix<double>::InnerIterator it(M, col); it; ++it)
        {
            Hat::Index<Dim> I = offsetOf((size_t)col);
            Hat::Index<Dim> J = offsetOf((size_t)it.row());
            unsigned int o = 0;
            size_t node = 0;
            for (unsigned int d = 0; d < Dim; d++)
            {
                int off = J[d] - I[d];
                if (off < -1 || off > 1) { fprintf(stderr, "stencil entry out of window\n"); exit(1); }
                o = o * 3 + (unsigned int)(off + 1);
                node = node * (res + 1) + (size_t)I[d];
            }
            out[node * S + o] += it.value();
        }
    return out;
}

static std::vector<double> ToVec(const Eigen::VectorXd &v) { return std::vector<double>(v.data(), v.data() + v.size()); }

template <unsigned int Dim>
static void Run(const std::string &in, unsigned int depth, const std::string &outDir, const Params &P)
{
    using Indexer = Hat::HierarchicalRegularIndexer<Dim>;
    using Energy = SingleCycleCascadicSystemEnergy<Dim, typename Indexer::Indexer>;
    const unsigned int K = Dim * (Dim - 1) / 2;
    auto path = [&](const std::string &s) { return outDir + "/" + s + ".npy"; };

    auto hermite = ReadSamples<Dim>(in);
    size_t n = hermite.size();
    {
        std::vector<double> pos(n * Dim), skew(n * K);
        for (size_t i = 0; i < n; i++)
        {
            for (unsigned int d = 0; d < Dim; d++) pos[i * Dim + d] = hermite[i].first[d];
            for (unsigned int k = 0; k < K; k++) skew[i * K + k] = hermite[i].second[k];
        }
        SaveF64(path("world_pos"), pos, {n, Dim});
        SaveF64(path("skew"), skew, {n, K});
    }

    // Unit cube transform (ExteriorPoissonRecon.cpp:166-172)
    ::SquareMatrix<double, Dim + 1> w2u = ExteriorPoisson::ToUnitCube<Dim>([&](size_t i) { return hermite[i].first; }, n, P.scale);
    for (size_t i = 0; i < n; i++) hermite[i].first = w2u(hermite[i].first);
    {
        std::vector<double> m((Dim + 1) * (Dim + 1));
        for (unsigned int c = 0; c < Dim + 1; c++) for (unsigned int r = 0; r < Dim + 1; r++) m[c * (Dim + 1) + r] = w2u(c, r);
        SaveF64(path("world_to_unit"), m, {Dim + 1, Dim + 1});
        std::vector<double> pos(n * Dim);
        for (size_t i = 0; i < n; i++) for (unsigned int d = 0; d < Dim; d++) pos[i * Dim + d] = hermite[i].first[d];
        SaveF64(path("pos"), pos, {n, Dim});
    }

    Indexer hIndexer(depth);
    OrderedSampler<Dim> orderedSampler([&](size_t i) { return hermite[i].first; }, n, 1 << depth);
    {
        std::vector<int64_t> cells, counts, order;
        for (size_t i = 0; i < orderedSampler.size(); i++)
        {
            for (unsigned int d = 0; d < Dim; d++) cells.push_back(orderedSampler[i].first[d]);
            counts.push_back((int64_t)orderedSampler[i].second.size());
            for (size_t j : orderedSampler[i].second) order.push_back((int64_t)j);
        }
        SaveI64(path("cells"), cells, {orderedSampler.size(), Dim});
        SaveI64(path("cell_counts"), counts, {orderedSampler.size()});
        SaveI64(path("cell_order"), order, {n});
    }

    GridSamples::TreeEstimator<Dim, 2> estimator(P.dRadius, depth, [&](size_t i) { return hermite[i].first; }, orderedSampler, true);
    {
        std::vector<double> m(n), no(n), de(n);
        for (size_t i = 0; i < n; i++)
        {
            m[i] = estimator.measure(hermite[i].first, 0);
            no[i] = estimator.noise(hermite[i].first, 0);
            de[i] = estimator.depth(hermite[i].first, 0);
        }
        SaveF64(path("est_measure"), m, {n});
        SaveF64(path("est_noise"), no, {n});
        SaveF64(path("est_depth"), de, {n});
        // density tree node data per tree level, densely: level l (=tree depth-1) has (2^l+1)^Dim vertices
        const unsigned int W = 1 + Dim + Dim * Dim;
        for (unsigned int l = 0; l <= depth; l++)
        {
            size_t r1 = (1u << l) + 1, NV = (size_t)std::pow(r1, Dim);
            std::vector<double> g(NV * W, 0.);
            std::vector<int64_t> ex(NV, 0);
            auto F = [&](unsigned int dd, Hat::Index<Dim> I, const GridSamples::DensityAndNoiseInfo<Dim> &data) {
                if (dd != l) return;
                size_t idx = 0;
                for (unsigned int d = 0; d < Dim; d++) idx = idx * r1 + I[d];
                double *o = &g[idx * W];
                o[0] = data.weightSum;
                for (unsigned int d = 0; d < Dim; d++) o[1 + d] = data.positionSum[d];
                for (unsigned int a = 0; a < Dim; a++) for (unsigned int b = 0; b < Dim; b++) o[1 + Dim + a * Dim + b] = data.covarianceSum(a, b);
                ex[idx] = 1;
            };
            static_cast<const GridSamples::TreeSplatter<Dim, GridSamples::DensityAndNoiseInfo<Dim>> &>(estimator).process(F);
            SaveF64(path("density_l" + std::to_string(l)), g, {NV, W});
            SaveI64(path("density_exists_l" + std::to_string(l)), ex, {NV});
        }
    }

    // Skew splat replica through the public TreeSplatter API, to expose S(E) and the leaf depths
    // (the reconstructor builds the same tree internally, ExteriorPoisson.h:177-264, 290-307).
    {
        const unsigned int CoDim = 2;
        GridSamples::TreeSplatter<Dim, Hat::SkewSymmetricMatrix<double, Dim>> splatter(depth);
        std::vector<Point<double, Dim>> sp(n);
        std::vector<Hat::SkewSymmetricMatrix<double, Dim>> sv(n);
        std::vector<double> sd(n);
        for (size_t i = 0; i < n; i++)
        {
            Hat::SkewSymmetricMatrix<double, Dim> s = hermite[i].second;
            s /= sqrt(s.squareNorm());
            s *= estimator.measure(hermite[i].first, 0);
            s *= 1 << (depth * CoDim);
            sp[i] = hermite[i].first;
            sv[i] = s;
            sd[i] = estimator.depth(hermite[i].first, 0);
        }
        auto Fs = [&](size_t i) { return std::make_pair(sp[i], sv[i]); };
        auto Fd = [&](size_t i) { return sd[i]; };
        auto DW = [](unsigned int d) { return (double)(1 << (d * Dim)); };
        switch (P.tRadius)
        {
        case 0: splatter.template addSamples<0>(Fs, orderedSampler, Fd, DW, false); break;
        case 1: splatter.template addSamples<1>(Fs, orderedSampler, Fd, DW, false); break;
        case 2: splatter.template addSamples<2>(Fs, orderedSampler, Fd, DW, false); break;
        default: fprintf(stderr, "tRadius>2 not dumped\n"); exit(1);
        }
        double scale = pow(pow(0.5, depth), 1.5 * CoDim);
        splatter.process([&](unsigned int, Hat::Index<Dim>, Hat::SkewSymmetricMatrix<double, Dim> &s) { s *= scale; });
        for (unsigned int l = 0; l <= depth; l++)
        {
            size_t r1 = (1u << l) + 1, NV = (size_t)std::pow(r1, Dim);
            std::vector<double> g(NV * K, 0.);
            auto F = [&](unsigned int dd, Hat::Index<Dim> I, const Hat::SkewSymmetricMatrix<double, Dim> &data) {
                if (dd != l) return;
                size_t idx = 0;
                for (unsigned int d = 0; d < Dim; d++) idx = idx * r1 + I[d];
                for (unsigned int k = 0; k < K; k++) g[idx * K + k] = data[k];
            };
            static_cast<const GridSamples::TreeSplatter<Dim, Hat::SkewSymmetricMatrix<double, Dim>> &>(splatter).process(F);
            SaveF64(path("skew_l" + std::to_string(l)), g, {NV, K});
        }
        unsigned int res = 1u << depth;
        size_t NE = (size_t)std::pow(res, Dim);
        std::vector<double> S(NE * K);
        std::vector<int64_t> leaf(NE);
        Hat::ScalarFunctions<Dim> scalars(res);
        for (size_t e = 0; e < NE; e++)
        {
            // element index in "axis 0 most significant" order
            Hat::Index<Dim> E;
            size_t t = e;
            for (int d = Dim - 1; d >= 0; d--) { E[d] = (int)(t % res); t /= res; }
            Point<double, Dim> p;
            for (unsigned int d = 0; d < Dim; d++) p[d] = (E[d] + 0.5) / res;
            Hat::SkewSymmetricMatrix<double, Dim> s = splatter(p, 0);
            for (unsigned int k = 0; k < K; k++) S[e * K + k] = s[k];
            leaf[e] = splatter._spaceRoot->getLeafNode(p)->depth();
        }
        SaveF64(path("S"), S, {NE, K});
        SaveI64(path("leaf_depth"), leaf, {NE});
        if (P.project)
        {
            // the reference's FitBlade of every element's S, each with the full iteration budget of
            // the command line (ProjectionIterations, ProjectionEpslion: ExteriorPoissonRecon.cpp:48-49)
            std::vector<double> Sp(NE * K);
            srand(P.seed);
            for (size_t e = 0; e < NE; e++)
            {
                Hat::SkewSymmetricMatrix<double, Dim> s;
                for (unsigned int k = 0; k < K; k++) s[k] = S[e * K + k];
                unsigned int steps = 1000;
                std::pair<Point<double, Dim>, Point<double, Dim>> blade = ExteriorPoisson::FitBlade<Dim>(s, steps, 1e-10);
                Hat::SkewSymmetricMatrix<double, Dim> sp(blade.first, blade.second);
                for (unsigned int k = 0; k < K; k++) Sp[e * K + k] = sp[k];
            }
            SaveF64(path("S_project"), Sp, {NE, K});
        }
    }

    // Full reconstructor (ExteriorPoissonRecon.cpp:220-245)
    srand(P.seed);
    const double nSigma = P.nSigma;
    auto NoiseToWeight = [nSigma](double x) { return exp(-x * x / (2. * nSigma * nSigma)); };
    ExteriorPoisson::Reconstructor<Dim, Energy> recon(hIndexer, depth, P.minSolveDepth, depth,
        [&](size_t i) { return hermite[i]; }, orderedSampler, estimator, NoiseToWeight, P.dWeight, P.sWeight, P.tRadius,
        P.project ? 1000u : 0u, 1e-10, false);

    {
        std::vector<double> c = {recon._energies.back()._c};
        SaveF64(path("c"), c, {1});
    }
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(-1., 1.);
    for (unsigned int d = 0; d <= depth; d++)
    {
        const Energy &E = recon._energies[d];
        unsigned int res = 1u << d;
        size_t N = (size_t)std::pow(res + 1, Dim);
        const unsigned int S = (unsigned int)std::pow(3, Dim);
        std::string L = "_d" + std::to_string(d);
        SaveF64(path("R" + L), ColumnStencil<Dim>(E._R, res), {N, S});
        SaveF64(path("B" + L), ColumnStencil<Dim>(E._B, res), {N, S});
        Eigen::VectorXd x(N), y(N);
        for (size_t i = 0; i < N; i++) x[i] = U(rng), y[i] = U(rng);
        SaveF64(path("xr" + L), ToVec(x), {N});
        SaveF64(path("yr" + L), ToVec(y), {N});
        std::pair<double, double> e = E.energies(x, y);
        std::vector<double> ev = {e.first, e.second, E.wedgeSquareNorm(x, y)};
        SaveF64(path("energies" + L), ev, {3});
        std::vector<double> q(N * 5);
        for (size_t i = 0; i < N; i++)
        {
            Polynomial::Polynomial2D<2> Q = E.quadraticFit(x, y, (unsigned int)i, false, 0);
            q[i * 5 + 0] = Q.coefficient(2, 0);
            q[i * 5 + 1] = Q.coefficient(0, 2);
            q[i * 5 + 2] = Q.coefficient(1, 1);
            q[i * 5 + 3] = Q.coefficient(1, 0);
            q[i * 5 + 4] = Q.coefficient(0, 1);
        }
        SaveF64(path("quadfit" + L), q, {N, 5});
        // one paired Gauss-Seidel iteration (all 2^Dim colours)
        Eigen::VectorXd gx = x, gy = y;
        ExteriorPoissonSolvers::PairedGaussSeidelSolve<Dim>(d, recon._mcIndices[d], E, gx, gy, 1, false);
        SaveF64(path("gsx" + L), ToVec(gx), {N});
        SaveF64(path("gsy" + L), ToVec(gy), {N});
        if (d < depth)
        {
            Eigen::VectorXd px = E.prolongation(x);
            SaveF64(path("prolong" + L), ToVec(px), {(size_t)px.size()});
        }
    }

    // Linear multigrid of the reference (MG.h:37-195) on the finest level's screening+Dirichlet
    // operator M = R + dWeight K, with the reference's prolongations and parity colours:
    // one coloured GSRelaxer sweep and two V-cycles (2 relaxations per level) from x = 0.
    {
        const Energy &E = recon._energies[depth];
        Eigen::SparseMatrix<double> K = E.scalars.stiffness(E.indexer);
        Eigen::SparseMatrix<double> M = E._R + K * P.dWeight;
        size_t N = (size_t)M.rows();
        Eigen::VectorXd b(N);
        for (size_t i = 0; i < N; i++) b[i] = U(rng);
        auto MCI = [&](unsigned int d) -> const std::vector<std::vector<unsigned int>> & { return recon._mcIndices[d]; };
        Eigen::VectorXd g = Eigen::VectorXd::Zero(N);
        GSRelaxer relaxer(M);
        relaxer(b, g, recon._mcIndices[depth]);
        std::vector<Eigen::SparseMatrix<double>> Ps(depth);
        for (unsigned int d = 0; d < depth; d++) Ps[d] = recon._energies[d]._sP;  // level d -> d+1 lives on the coarser energy
        MGSolver mg(M, [&](unsigned int i) { return Ps[i]; }, depth);
        Eigen::VectorXd x1 = Eigen::VectorXd::Zero(N);
        mg.vCycle(b, x1, 2, MCI);
        Eigen::VectorXd x2 = x1;
        mg.vCycle(b, x2, 2, MCI);
        SaveF64(path("mg_M"), ColumnStencil<Dim>(M, 1u << depth), {N, (size_t)std::pow(3, Dim)});
        SaveF64(path("mg_b"), ToVec(b), {N});
        SaveF64(path("mg_gs1"), ToVec(g), {N});
        SaveF64(path("mg_v1"), ToVec(x1), {N});
        SaveF64(path("mg_v2"), ToVec(x2), {N});
    }

    // Quadratic models of the alternating solve (ExteriorPoissonSolvers.h:96-131) for the energy
    // the reconstructor uses.  SingleCycleCascadicSystemEnergy does not implement
    // quadraticApproximation1/2 (the SystemEnergy defaults abort, SystemEnergy.h:322-334), and the
    // product mass matrix (ProductFunctions::mass, Hat.products.h:136) does not compile, so the
    // wedge Gram matrices G_x (u^T G_x v = <x^u, x^v>) and G_y (<u^y, v^y>) are pinned through the
    // reference's own bilinear wedge integral wedges(indexer, _wMStencil, a, b, c, d) = <a^b, c^d>
    // (Hat.products.inl:189-231) on random probe pairs (u_k, v_k).  Then biQuadraticFit, stepSize
    // and newtonUpdate (SystemEnergy.h:256-303, 499-540) for random directions (dx, dy).
    {
        const unsigned int ql = depth, K = 6;
        const Energy &E = recon._energies[ql];
        unsigned int res = 1u << ql;
        size_t N = (size_t)std::pow(res + 1, Dim);
        Eigen::VectorXd x(N), y(N), dx(N), dy(N);
        for (size_t i = 0; i < N; i++) x[i] = U(rng), y[i] = U(rng), dx[i] = U(rng), dy[i] = U(rng);
        std::vector<double> us(K * N), vs(K * N), gx(K), gy(K);
        for (unsigned int k = 0; k < K; k++)
        {
            Eigen::VectorXd u(N), v(N);
            for (size_t i = 0; i < N; i++) u[i] = U(rng), v[i] = U(rng);
            for (size_t i = 0; i < N; i++) us[k * N + i] = u[i], vs[k * N + i] = v[i];
            gx[k] = E.wedges(E.indexer, E._wMStencil, x, u, x, v);
            gy[k] = E.wedges(E.indexer, E._wMStencil, u, y, v, y);
        }
        SaveF64(path("qa_x"), ToVec(x), {N});
        SaveF64(path("qa_y"), ToVec(y), {N});
        SaveF64(path("qa_dx"), ToVec(dx), {N});
        SaveF64(path("qa_dy"), ToVec(dy), {N});
        SaveF64(path("qa_u"), us, {K, N});
        SaveF64(path("qa_v"), vs, {K, N});
        SaveF64(path("qa_gx"), gx, {K});
        SaveF64(path("qa_gy"), gy, {K});
        Polynomial::Polynomial2D<4> Q = E.biQuadraticFit(x, y, dx, dy);
        std::vector<double> q(9);
        for (unsigned int i = 0; i <= 2; i++) for (unsigned int j = 0; j <= 2; j++) q[i * 3 + j] = Q.coefficient(i, j);
        SaveF64(path("qa_biquad"), q, {3, 3});
        std::vector<double> st = {E.stepSize(x, y, dx, dy)};
        SaveF64(path("qa_step"), st, {1});
        Point<double, 2> nu = E.newtonUpdate(x, y, dx, dy, 10);
        SaveF64(path("qa_newton"), std::vector<double>{nu[0], nu[1]}, {2});
    }

    if (P.solve)
    {
        // Cascadic solve with the reference schedule (ExteriorPoisson.h:315-409)
        std::streambuf *old = std::cout.rdbuf();
        std::stringstream sink;
        std::cout.rdbuf(sink.rdbuf());
        // Levels below minSolveDepth are never written by the reference's solve (Eigen resize leaves
        // them uninitialised, ExteriorPoisson.h:158-159, 349-351) yet enter its hierarchical output;
        // zero them so that the dump is well defined.
        for (unsigned int d = 0; d < P.minSolveDepth && d <= depth; d++) { recon._x[d].setZero(); recon._y[d].setZero(); }
        recon.solve(P.singleLevel != 0, P.iMult, P.gsIters, P.separate != 0, false);
        std::cout.rdbuf(old);
        for (unsigned int d = 0; d <= depth; d++)
        {
            std::string L = "_d" + std::to_string(d);
            SaveF64(path("solx" + L), ToVec(recon._x[d]), {(size_t)recon._x[d].size()});
            SaveF64(path("soly" + L), ToVec(recon._y[d]), {(size_t)recon._y[d].size()});
        }
        // regular (summed) finest coefficients and their energy
        Eigen::VectorXd X = recon._x[0], Y = recon._y[0];
        for (unsigned int d = 1; d <= depth; d++)
        {
            X = recon._energies[d - 1].prolongation(X) + recon._x[d];
            Y = recon._energies[d - 1].prolongation(Y) + recon._y[d];
        }
        std::pair<double, double> e = recon._energies[depth].energies(X, Y);
        std::vector<double> ev = {e.first, e.second};
        SaveF64(path("sol_energies"), ev, {2});
        SaveF64(path("solX"), ToVec(X), {(size_t)X.size()});
        SaveF64(path("solY"), ToVec(Y), {(size_t)Y.size()});
    }
    {
        std::vector<int64_t> h = {(int64_t)typeid(Hat::HierarchicalRegularIndexer<Dim>).hash_code()};
        SaveI64(path("indexer_hash"), h, {1});
    }
}

// The adaptive indexer (HierarchicalAdaptedIndexer, Hat.adaptive.inl:342-732) through the same
// reconstructor.  Every level's function and element tables are dumped as grid indices in the
// indexer's own order ("afn_d<l>": node of each function index, active ones first, "aact_d<l>" their
// number; "ael_d<l>": element of each element index), and every per-function quantity densely on the
// level's grid (zero where no function is indexed), so that the dense restatement compares directly.
template <unsigned int Dim>
static void RunAdapted(const std::string &in, unsigned int depth, const std::string &outDir, const Params &P)
{
    using HIndexer = Hat::HierarchicalAdaptedIndexer<Dim>;
    using Energy = SingleCycleCascadicSystemEnergy<Dim, typename HIndexer::Indexer>;
    auto path = [&](const std::string &s) { return outDir + "/" + s + ".npy"; };
    const unsigned int K = Dim * (Dim - 1) / 2;

    auto hermite = ReadSamples<Dim>(in);
    size_t n = hermite.size();
    {
        std::vector<double> pos(n * Dim), skew(n * K);
        for (size_t i = 0; i < n; i++)
        {
            for (unsigned int d = 0; d < Dim; d++) pos[i * Dim + d] = hermite[i].first[d];
            for (unsigned int k = 0; k < K; k++) skew[i * K + k] = hermite[i].second[k];
        }
        SaveF64(path("world_pos"), pos, {n, Dim});
        SaveF64(path("skew"), skew, {n, K});
    }
    ::SquareMatrix<double, Dim + 1> w2u = ExteriorPoisson::ToUnitCube<Dim>([&](size_t i) { return hermite[i].first; }, n, P.scale);
    for (size_t i = 0; i < n; i++) hermite[i].first = w2u(hermite[i].first);
    {
        std::vector<double> pos(n * Dim);
        for (size_t i = 0; i < n; i++) for (unsigned int d = 0; d < Dim; d++) pos[i * Dim + d] = hermite[i].first[d];
        SaveF64(path("pos"), pos, {n, Dim});
    }

    // ExteriorPoissonRecon.cpp:191-198, 205-245
    HIndexer hIndexer(n, [&](size_t i) { return hermite[i].first; }, (unsigned int)P.aRadius, depth);
    OrderedSampler<Dim> orderedSampler([&](size_t i) { return hermite[i].first; }, n, 1 << depth);
    GridSamples::TreeEstimator<Dim, 2> estimator(P.dRadius, depth, [&](size_t i) { return hermite[i].first; }, orderedSampler, true);
    srand(P.seed);
    const double nSigma = P.nSigma;
    auto NoiseToWeight = [nSigma](double x) { return exp(-x * x / (2. * nSigma * nSigma)); };
    ExteriorPoisson::Reconstructor<Dim, Energy> recon(hIndexer, depth, P.minSolveDepth, depth,
        [&](size_t i) { return hermite[i]; }, orderedSampler, estimator, NoiseToWeight, P.dWeight, P.sWeight, P.tRadius, 0u, 1e-10, false);
    SaveF64(path("c"), std::vector<double>{recon._energies.back()._c}, {1});

    std::vector<std::vector<Hat::Index<Dim>>> offsets(depth + 1);
    std::vector<std::vector<int64_t>> nodeOf(depth + 1);
    for (unsigned int d = 0; d <= depth; d++)
    {
        auto indexer = hIndexer[d];
        const size_t r1 = ((size_t)1 << d) + 1;
        const std::string L = "_d" + std::to_string(d);
        std::vector<int64_t> fn(indexer.numFunctions()), el(indexer.numElements());
        offsets[d].resize(indexer.numFunctions());
        for (size_t f = 0; f < indexer.numFunctions(); f++)
        {
            Hat::Index<Dim> I = indexer.functionIndex(f);
            offsets[d][f] = I;
            int64_t node = 0;
            for (unsigned int k = 0; k < Dim; k++) node = node * (int64_t)r1 + I[k];
            fn[f] = node;
        }
        for (size_t e = 0; e < indexer.numElements(); e++)
        {
            Hat::Index<Dim> E = indexer.elementIndex(e);
            int64_t node = 0;
            for (unsigned int k = 0; k < Dim; k++) node = node * (int64_t)(r1 - 1) + E[k];
            el[e] = node;
        }
        nodeOf[d] = fn;
        SaveI64(path("afn" + L), fn, {fn.size()});
        SaveI64(path("ael" + L), el, {el.size()});
        SaveI64(path("aact" + L), std::vector<int64_t>{(int64_t)indexer.numActiveFunctions()}, {1});
    }
    auto dense = [&](unsigned int d, const Eigen::VectorXd &v) {
        const size_t N = (size_t)std::pow(((size_t)1 << d) + 1, Dim);
        std::vector<double> out(N, 0.);
        for (size_t f = 0; f < (size_t)v.size(); f++) out[(size_t)nodeOf[d][f]] = v[f];
        return out;
    };

    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(-1., 1.);
    for (unsigned int d = 0; d <= depth; d++)
    {
        const Energy &E = recon._energies[d];
        const unsigned int res = 1u << d;
        const size_t N = (size_t)std::pow(res + 1, Dim), S = (size_t)std::pow(3, Dim), F = offsets[d].size();
        const std::string L = "_d" + std::to_string(d);
        SaveF64(path("R" + L), ColumnStencil<Dim>(E._R, res, &offsets[d]), {N, S});
        SaveF64(path("B" + L), ColumnStencil<Dim>(E._B, res, &offsets[d]), {N, S});
        Eigen::VectorXd x(F), y(F);
        for (size_t i = 0; i < F; i++) x[i] = U(rng), y[i] = U(rng);
        SaveF64(path("xr" + L), dense(d, x), {N});
        SaveF64(path("yr" + L), dense(d, y), {N});
        std::pair<double, double> e = E.energies(x, y);
        SaveF64(path("energies" + L), std::vector<double>{e.first, e.second, E.wedgeSquareNorm(x, y)}, {3});
        const size_t A = hIndexer[d].numActiveFunctions();
        std::vector<double> q(A * 5);
        for (size_t i = 0; i < A; i++)
        {
            Polynomial::Polynomial2D<2> Q = E.quadraticFit(x, y, (unsigned int)i, false, 0);
            q[i * 5 + 0] = Q.coefficient(2, 0);
            q[i * 5 + 1] = Q.coefficient(0, 2);
            q[i * 5 + 2] = Q.coefficient(1, 1);
            q[i * 5 + 3] = Q.coefficient(1, 0);
            q[i * 5 + 4] = Q.coefficient(0, 1);
        }
        SaveF64(path("quadfit" + L), q, {A, 5});
        Eigen::VectorXd gx = x, gy = y;
        ExteriorPoissonSolvers::PairedGaussSeidelSolve<Dim>(d, recon._mcIndices[d], E, gx, gy, 1, false);
        SaveF64(path("gsx" + L), dense(d, gx), {N});
        SaveF64(path("gsy" + L), dense(d, gy), {N});
        if (d < depth)
        {
            Eigen::VectorXd px = E.prolongation(x);
            std::vector<double> pd = dense(d + 1, px);
            SaveF64(path("prolong" + L), pd, {pd.size()});
        }
    }

    if (P.solve)
    {
        std::streambuf *old = std::cout.rdbuf();
        std::stringstream sink;
        std::cout.rdbuf(sink.rdbuf());
        for (unsigned int d = 0; d < P.minSolveDepth && d <= depth; d++) { recon._x[d].setZero(); recon._y[d].setZero(); }
        recon.solve(P.singleLevel != 0, P.iMult, P.gsIters, P.separate != 0, false);
        std::cout.rdbuf(old);
        for (unsigned int d = 0; d <= depth; d++)
        {
            const std::string L = "_d" + std::to_string(d);
            std::vector<double> sx = dense(d, recon._x[d]), sy = dense(d, recon._y[d]);
            SaveF64(path("solx" + L), sx, {sx.size()});
            SaveF64(path("soly" + L), sy, {sy.size()});
        }
        Eigen::VectorXd X = recon._x[0], Y = recon._y[0];
        for (unsigned int d = 1; d <= depth; d++)
        {
            X = recon._energies[d - 1].prolongation(X) + recon._x[d];
            Y = recon._energies[d - 1].prolongation(Y) + recon._y[d];
        }
        std::pair<double, double> e = recon._energies[depth].energies(X, Y);
        SaveF64(path("sol_energies"), std::vector<double>{e.first, e.second}, {2});
        std::vector<double> sX = dense(depth, X), sY = dense(depth, Y);
        SaveF64(path("solX"), sX, {sX.size()});
        SaveF64(path("solY"), sY, {sY.size()});
    }
    SaveI64(path("indexer_hash"), std::vector<int64_t>{(int64_t)typeid(HIndexer).hash_code()}, {1});
}

int main(int argc, char **argv)
{
    if (argc < 4)
    {
        fprintf(stderr, "usage: %s <in.ply> <depth> <outdir> [--param value]...\n", argv[0]);
        return 2;
    }
    std::string in = argv[1];
    unsigned int depth = (unsigned int)atoi(argv[2]);
    std::string out = argv[3];
    Params P;
    for (int i = 4; i + 1 < argc; i += 2)
    {
        std::string k = argv[i];
        double v = atof(argv[i + 1]);
        if (k == "--sWeight") P.sWeight = v;
        else if (k == "--dWeight") P.dWeight = v;
        else if (k == "--nSigma") P.nSigma = v;
        else if (k == "--iMult") P.iMult = v;
        else if (k == "--scale") P.scale = v;
        else if (k == "--tRadius") P.tRadius = (unsigned int)v;
        else if (k == "--dRadius") P.dRadius = (unsigned int)v;
        else if (k == "--gsIters") P.gsIters = (unsigned int)v;
        else if (k == "--seed") P.seed = (unsigned int)v;
        else if (k == "--minSolveDepth") P.minSolveDepth = (unsigned int)v;
        else if (k == "--solve") P.solve = (int)v;
        else if (k == "--separate") P.separate = (int)v;
        else if (k == "--singleLevel") P.singleLevel = (int)v;
        else if (k == "--project") P.project = (int)v;
        else if (k == "--aRadius") P.aRadius = (int)v;
        else { fprintf(stderr, "unknown flag %s\n", k.c_str()); return 2; }
    }
    mkdir(out.c_str(), 0755);
    VertexFactory::PositionFactory<double, 4> pf4;
    int ft;
    std::vector<GregTurk::PlyProperty> props = PLY::ReadVertexHeader(in, ft);
    const bool four = pf4.plyValidReadProperties(props);
    if (P.aRadius >= 0)
    {
        if (four) RunAdapted<4>(in, depth, out, P);
        else RunAdapted<3>(in, depth, out, P);
    }
    else if (four) Run<4>(in, depth, out, P);
    else Run<3>(in, depth, out, P);
    return 0;
}
