// epr_recon: drop-in replacement of the reference's ExteriorPoissonRecon command line
// (ExteriorPoissonRecon/ExteriorPoissonRecon.cpp:52-312), with both of its indexers: the adaptive
// one (--aRadius 0..5, default 3, as the reference) and the regular grid (--aRadius -1).  It reads the same PLY
// samples (x y z [w] + skew_c_r), maps them to the unit cube, runs the build and the solve on the
// GPU through the C ABI of include/epr.h, and writes the reference's <out>.tree (readable by the
// reference's Extract tool) and, with --grid, the regular coefficient grids <grid>.0.grid and
// <grid>.1.grid in the format of RegularGrid::Write (Misha/RegularGrid.inl:441-472).
//
// Differences from the reference (documented, deliberate):
//   * errors exit with a non-zero status (the reference prints and exits 0);
//   * --project fits every element's blade by the power iteration from a fixed start, each element
//     with the full iteration budget (1000 steps, 1e-10); the reference starts from random vectors
//     and passes one shared step budget by reference to all elements (FitBlade's `steps`,
//     ExteriorPoisson.h:303, 412), so in 4D its blades depend on thread timing.
// <out>.density.tree is written as the reference writes it (the estimator's tree, epr_write_density_tree),
// with zero words where the reference's file holds memory addresses.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/epr.h"

namespace {

struct Args
{
    std::string in, out, grid;
    double nSigma = 0.25, scale = 1.1, sWeight = 100., dWeight = 0.00625, iMult = 2., jitter = 0.;
    int depth = 5, seed = 0, tRadius = 1, dRadius = 1, aRadius = 3, minSolveDepth = 0, gsIters = 10, maxSolveDepth = -1;
    bool singleLevel = false, separate = false, verbose = false, project = false;
    std::string precision = "fp64", solver = "cascadic", bandPrecision = "fp64";
    int device = 0, fp64Levels = 0, fp64From = 0, maxCycles = 200;
    double tolerance = 1e-6;
};

[[noreturn]] void Fail(const std::string &msg, int code = 1)
{
    fprintf(stderr, "[ERROR] %s\n", msg.c_str());
    exit(code);
}

void Usage(const char *ex)
{
    printf("Usage %s:\n", ex);
    printf("\t --in <input points and frames>\n");
    printf("\t[--out <output tree header>]\n");
    printf("\t[--grid <output grid header>]\n");
    printf("\t[--depth <grid depth>=5]\n");
    printf("\t[--minSolveDepth <minimum hierarchy solver depth>=0]\n");
    printf("\t[--maxSolveDepth <maximum hierarchy solver depth>]\n");
    printf("\t[--nSigma <noise-to-weight sigma>=0.25]\n");
    printf("\t[--dRadius <density kernel radius>=1]\n");
    printf("\t[--tRadius <tensor kernel radius>=1]\n");
    printf("\t[--aRadius <adaptive radius>=3 (-1: the regular grid)]\n");
    printf("\t[--jitter <jitter magnitude>=0]\n");
    printf("\t[--gsIters <gs iterations>=10]\n");
    printf("\t[--seed <random seed>=0]\n");
    printf("\t[--sWeight <screening weight>=100]\n");
    printf("\t[--dWeight <dirichlet weight>=0.00625]\n");
    printf("\t[--scale <bounding box scale>=1.1]\n");
    printf("\t[--iMult <iteration multiplier>=2]\n");
    printf("\t[--precision fp64|fp32]\n");
    printf("\t[--fp64From <first level of the double band with --precision fp32>=0]\n");
    printf("\t[--fp64Levels <levels from --fp64From below this one relax in double with --precision fp32>=0]\n");
    printf("\t[--bandPrecision fp64|df <arithmetic of the band's 3D levels up to 3: double or double-float>]\n");
    printf("\t[--solver cascadic|multigrid]\n");
    printf("\t[--tolerance <multigrid: relative gradient per level>=1e-6]\n");
    printf("\t[--maxCycles <multigrid: alternating rounds per level>=200]\n");
    printf("\t[--device <CUDA device>=0]\n");
    printf("\t[--separate]\n\t[--singleLevel]\n\t[--verbose]\n");
}

Args Parse(int argc, char **argv)
{
    Args a;
    std::map<std::string, std::string *> strs = {{"in", &a.in}, {"out", &a.out}, {"grid", &a.grid}, {"precision", &a.precision},
                                                 {"solver", &a.solver}, {"bandPrecision", &a.bandPrecision}};
    std::map<std::string, double *> dbls = {{"nSigma", &a.nSigma}, {"scale", &a.scale}, {"sWeight", &a.sWeight},
                                            {"dWeight", &a.dWeight}, {"iMult", &a.iMult}, {"jitter", &a.jitter},
                                            {"tolerance", &a.tolerance}};
    std::map<std::string, int *> ints = {{"depth", &a.depth}, {"seed", &a.seed}, {"tRadius", &a.tRadius},
                                         {"dRadius", &a.dRadius}, {"aRadius", &a.aRadius}, {"minSolveDepth", &a.minSolveDepth},
                                         {"gsIters", &a.gsIters}, {"maxSolveDepth", &a.maxSolveDepth}, {"device", &a.device},
                                         {"fp64Levels", &a.fp64Levels}, {"fp64From", &a.fp64From}, {"maxCycles", &a.maxCycles}};
    std::map<std::string, bool *> flags = {{"singleLevel", &a.singleLevel}, {"separate", &a.separate},
                                           {"verbose", &a.verbose}, {"project", &a.project}};
    for (int i = 1; i < argc; i++)
    {
        std::string k = argv[i];
        if (k.rfind("--", 0) != 0) Fail("unexpected argument: " + k, 2);
        k = k.substr(2);
        if (flags.count(k)) { *flags[k] = true; continue; }
        if (i + 1 >= argc) Fail("missing value for --" + k, 2);
        std::string v = argv[++i];
        if (strs.count(k)) *strs[k] = v;
        else if (dbls.count(k)) *dbls[k] = atof(v.c_str());
        else if (ints.count(k)) *ints[k] = atoi(v.c_str());
        else Fail("unknown flag --" + k, 2);
    }
    return a;
}

// ------------------------------------------------------------------------------------------------
// PLY reader: vertex element with x y z [w] and skew_c_r (m(c, r)) properties, ascii or binary.
// ------------------------------------------------------------------------------------------------
struct Samples
{
    int dim = 0;
    std::vector<double> pos;     // n x dim
    std::vector<double> frames;  // n x dim x dim, frames[i*dim*dim + c*dim + r] = m(c, r)
    size_t n = 0;
};

int TypeSize(const std::string &t)
{
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
    if (t == "double" || t == "float64") return 8;
    return 0;
}

double ReadBinary(const unsigned char *p, const std::string &t, bool swap)
{
    unsigned char b[8];
    int sz = TypeSize(t);
    for (int i = 0; i < sz; i++) b[i] = swap ? p[sz - 1 - i] : p[i];
    if (t == "char" || t == "int8") { int8_t v; memcpy(&v, b, 1); return v; }
    if (t == "uchar" || t == "uint8") { uint8_t v; memcpy(&v, b, 1); return v; }
    if (t == "short" || t == "int16") { int16_t v; memcpy(&v, b, 2); return v; }
    if (t == "ushort" || t == "uint16") { uint16_t v; memcpy(&v, b, 2); return v; }
    if (t == "int" || t == "int32") { int32_t v; memcpy(&v, b, 4); return v; }
    if (t == "uint" || t == "uint32") { uint32_t v; memcpy(&v, b, 4); return v; }
    if (t == "float" || t == "float32") { float v; memcpy(&v, b, 4); return v; }
    double v;
    memcpy(&v, b, 8);
    return v;
}

Samples ReadPly(const std::string &file)
{
    std::ifstream f(file, std::ios::binary);
    if (!f) Fail("cannot open " + file);
    std::string line, format;
    size_t nvert = 0;
    std::vector<std::pair<std::string, std::string>> props;  // (name, type)
    bool inVertex = false, vertexFirst = true, sawElement = false;
    std::getline(f, line);
    if (line.rfind("ply", 0) != 0) Fail("not a PLY file: " + file);
    while (std::getline(f, line))
    {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ss(line);
        std::string tok;
        ss >> tok;
        if (tok == "format") ss >> format;
        else if (tok == "element")
        {
            std::string name;
            size_t cnt;
            ss >> name >> cnt;
            if (name == "vertex") { inVertex = true; nvert = cnt; if (sawElement) vertexFirst = false; }
            else inVertex = false;
            sawElement = true;
        }
        else if (tok == "property" && inVertex)
        {
            std::string type, name;
            ss >> type;
            if (type == "list") Fail("list properties on vertices are not supported");
            ss >> name;
            props.emplace_back(name, type);
        }
        else if (tok == "end_header") break;
    }
    if (!vertexFirst) Fail("the vertex element must be the first element of the PLY file");
    std::map<std::string, int> idx;
    for (size_t i = 0; i < props.size(); i++) idx[props[i].first] = (int)i;
    Samples s;
    s.dim = idx.count("w") ? 4 : 3;
    const char *axes[] = {"x", "y", "z", "w"};
    for (int d = 0; d < s.dim; d++)
        if (!idx.count(axes[d])) Fail(std::string("missing vertex property ") + axes[d]);
    for (int c = 0; c < s.dim; c++)
        for (int r = 0; r < s.dim; r++)
        {
            std::string nm = "skew_" + std::to_string(c) + "_" + std::to_string(r);
            if (!idx.count(nm)) Fail("missing vertex property " + nm + " (Invalid sample file)");
        }
    s.n = nvert;
    s.pos.resize(nvert * s.dim);
    s.frames.resize(nvert * s.dim * s.dim);
    std::vector<double> row(props.size());
    bool ascii = format == "ascii";
    bool swap = format == "binary_big_endian";
    size_t rowBytes = 0;
    std::vector<size_t> offs(props.size());
    for (size_t i = 0; i < props.size(); i++)
    {
        offs[i] = rowBytes;
        int sz = TypeSize(props[i].second);
        if (!sz) Fail("unsupported property type " + props[i].second);
        rowBytes += sz;
    }
    std::vector<unsigned char> buf(rowBytes);
    for (size_t v = 0; v < nvert; v++)
    {
        if (ascii)
        {
            for (size_t i = 0; i < props.size(); i++)
                if (!(f >> row[i])) Fail("truncated PLY vertex data");
        }
        else
        {
            if (!f.read((char *)buf.data(), rowBytes)) Fail("truncated PLY vertex data");
            for (size_t i = 0; i < props.size(); i++) row[i] = ReadBinary(buf.data() + offs[i], props[i].second, swap);
        }
        for (int d = 0; d < s.dim; d++) s.pos[v * s.dim + d] = row[idx[axes[d]]];
        for (int c = 0; c < s.dim; c++)
            for (int r = 0; r < s.dim; r++)
                s.frames[(v * s.dim + c) * s.dim + r] = row[idx["skew_" + std::to_string(c) + "_" + std::to_string(r)]];
    }
    return s;
}

// Random<double> (Misha/Geometry.inl:430-438) on the C library generator
double RandomDouble()
{
    const unsigned long long ULL_RAND_MAX = (unsigned long long)(RAND_MAX) + 1;
    const double RAND_MAX_SQUARED = double(ULL_RAND_MAX * ULL_RAND_MAX - 1);
    unsigned long long r1 = rand();
    unsigned long long r2 = rand();
    long long v = (long long)(r1 * ULL_RAND_MAX + r2);
    return double(v) / RAND_MAX_SQUARED;
}

// (Dim+1) x (Dim+1) matrices stored as m[c][r] (column, row) like the reference's SquareMatrix
struct Mat
{
    int n;
    std::vector<double> v;
    explicit Mat(int n_) : n(n_), v(n_ * n_, 0.) {}
    double &operator()(int c, int r) { return v[c * n + r]; }
    double operator()(int c, int r) const { return v[c * n + r]; }
    static Mat Identity(int n)
    {
        Mat m(n);
        for (int i = 0; i < n; i++) m(i, i) = 1;
        return m;
    }
    Mat operator*(const Mat &b) const
    {
        Mat o(n);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++) o(i, j) += b(i, k) * (*this)(k, j);
        return o;
    }
};

// inverse of an affine map [diag(k) | t]
Mat InverseAffine(const Mat &m)
{
    int D = m.n - 1;
    Mat o = Mat::Identity(m.n);
    for (int d = 0; d < D; d++)
    {
        o(d, d) = 1. / m(d, d);
        o(D, d) = -m(D, d) / m(d, d);
    }
    return o;
}

template <typename T>
void Put(FILE *fp, const T &v) { fwrite(&v, sizeof(T), 1, fp); }

void Check(epr_ctx *ctx, int rc, const char *what)
{
    if (rc != EPR_OK) Fail(std::string(what) + ": " + epr_last_error(ctx));
}

}  // namespace

int main(int argc, char **argv)
{
    Args a = Parse(argc, argv);
    if (a.in.empty()) { Usage(argv[0]); return EXIT_SUCCESS; }
    // the reference supports adaptive radii 0..5 (Hat.adaptive.inl:361-371) and -1 for the regular grid
    if (a.aRadius < -1 || a.aRadius > 5) Fail("Only kernel radius in the range [0,5] supported: " + std::to_string(a.aRadius), 2);
    if (a.precision != "fp32" && a.precision != "fp64") Fail("--precision must be fp64 or fp32", 2);
    if (a.solver != "cascadic" && a.solver != "multigrid") Fail("--solver must be cascadic or multigrid", 2);
    if (a.aRadius >= 0 && a.solver != "cascadic") Fail("the adaptive indexer is solved by the cascadic schedule only", 2);
    if (a.bandPrecision != "fp64" && a.bandPrecision != "df") Fail("--bandPrecision must be fp64 or df", 2);
    if (a.depth < 1) Fail("depth must be at least 1", 2);
    std::string ext = a.in.substr(a.in.find_last_of('.') + 1);
    if (ext != "ply") Fail("Only .ply files supported", 2);

    Samples s = ReadPly(a.in);
    const int D = s.dim, K = D * (D - 1) / 2;
    if (!s.n) Fail("Expected some samples: 0");

    // unit-cube map (ExteriorPoisson.h:100-123)
    std::vector<double> lo(s.pos.begin(), s.pos.begin() + D), hi = lo;
    for (size_t i = 1; i < s.n; i++)
        for (int d = 0; d < D; d++) { lo[d] = std::min(lo[d], s.pos[i * D + d]); hi[d] = std::max(hi[d], s.pos[i * D + d]); }
    double extn = hi[0] - lo[0];
    for (int d = 1; d < D; d++) extn = std::max(extn, hi[d] - lo[d]);
    Mat w2u = Mat::Identity(D + 1);
    {
        Mat t1 = Mat::Identity(D + 1), sc = Mat::Identity(D + 1), t2 = Mat::Identity(D + 1);
        for (int d = 0; d < D; d++) t2(D, d) = -(lo[d] + hi[d]) / 2.;
        for (int d = 0; d < D; d++) sc(d, d) = 1. / (extn * a.scale);
        for (int d = 0; d < D; d++) t1(D, d) = 0.5;
        w2u = t1 * sc * t2;
    }
    std::vector<double> pos(s.n * D);
    for (size_t i = 0; i < s.n; i++)
        for (int d = 0; d < D; d++)
        {
            double v = 0;
            for (int j = 0; j < D; j++) v += s.pos[i * D + j] * w2u(j, d);
            pos[i * D + d] = v + w2u(D, d);
        }
    Mat u2w = InverseAffine(w2u);
    if (a.jitter > 0)
    {
        // the translation is drawn before the seed is set (ExteriorPoissonRecon.cpp:174-180)
        Mat tr = Mat::Identity(D + 1);
        for (int d = 0; d < D; d++) tr(D, d) = (RandomDouble() * 2. - 1.) * a.jitter;
        for (size_t i = 0; i < s.n; i++)
            for (int d = 0; d < D; d++) pos[i * D + d] += tr(D, d);
        u2w = u2w * InverseAffine(tr);
    }
    std::vector<double> skew(s.n * K);
    for (size_t i = 0; i < s.n; i++)
        for (int r = 0, k = 0; r < D; r++)
            for (int c = 0; c < r; c++, k++)
            {
                const double *m = &s.frames[i * D * D];
                skew[i * K + k] = (m[r * D + c] - m[c * D + r]) / 2.;
            }

    epr_params p;
    epr_default_params(&p);
    p.s_weight = a.sWeight;
    p.d_weight = a.dWeight;
    p.n_sigma = a.nSigma;
    p.i_mult = a.iMult;
    p.t_radius = a.tRadius;
    p.d_radius = a.dRadius;
    p.gs_iters = a.gsIters;
    p.min_solve_depth = std::min(a.minSolveDepth, a.depth);
    p.max_solve_depth = a.maxSolveDepth < 0 ? -1 : std::min(a.maxSolveDepth, a.depth);
    p.seed = (unsigned)a.seed;
    p.precision = a.precision == "fp32" ? EPR_FP32 : EPR_FP64;
    p.fp64_levels = a.fp64Levels;
    p.fp64_from = a.fp64From;
    p.band_precision = a.bandPrecision == "df" ? EPR_BAND_DF : EPR_BAND_FP64;
    p.solver = a.solver == "multigrid" ? EPR_SOLVER_MULTIGRID : EPR_SOLVER_CASCADIC;
    p.tolerance = a.tolerance;
    p.max_cycles = a.maxCycles;
    p.verbose = a.verbose ? 1 : 0;
    p.device = a.device;
    p.single_level = a.singleLevel ? 1 : 0;
    p.separate = a.separate ? 1 : 0;
    p.project = a.project ? 1 : 0;
    p.adaptive_radius = a.aRadius;

    epr_ctx *ctx = epr_create(D, a.depth, &p);
    if (!ctx) Fail(std::string("epr_create: ") + epr_global_error());
    Check(ctx, epr_set_samples(ctx, s.n, pos.data(), skew.data()), "epr_set_samples");
    Check(ctx, epr_build(ctx), "epr_build");
    epr_stats st;
    Check(ctx, epr_solve(ctx, &st), "epr_solve");
    if (a.verbose)
        printf("Build: %.3f (s)\nSolve: %.3f (s)\n", st.build_ms / 1e3, st.solve_ms / 1e3);

    // voxel -> world (ExteriorPoissonRecon.cpp:252-257)
    Mat gridToCube = Mat::Identity(D + 1);
    for (int d = 0; d < D; d++) gridToCube(d, d) = 1. / (1 << a.depth);
    Mat v2w = u2w * gridToCube;

    if (!a.out.empty())
    {
        // <out>.tree: dim, indexer type hash, XForm, x levels, y levels, the indexer
        // (ExteriorPoissonRecon.cpp:259-270)
        std::vector<double> xf;
        for (int c = 0; c <= D; c++)
            for (int r = 0; r <= D; r++) xf.push_back(v2w(c, r));
        Check(ctx, epr_write_tree(ctx, xf.data(), (a.out + ".tree").c_str()), "epr_write_tree");
        // <out>.density.tree: the density estimator (ExteriorPoissonRecon.cpp:272-277)
        Check(ctx, epr_write_density_tree(ctx, xf.data(), (a.out + ".density.tree").c_str()), "epr_write_density_tree");
    }
    if (!a.grid.empty())
    {
        // regular coefficients of the finest level as <grid>.0.grid / <grid>.1.grid, as the
        // reference's Extract computes them from the .tree (regularCoefficients)
        size_t N = 1;
        int res = (1 << a.depth) + 1;
        for (int d = 0; d < D; d++) N *= (size_t)res;
        std::vector<double> x(N), y(N);
        Check(ctx, epr_get_regular_coefficients(ctx, x.data(), y.data()), "epr_get_regular_coefficients");
        for (int c = 0; c < 2; c++)
        {
            std::string fn = a.grid + "." + std::to_string(c) + ".grid";
            FILE *fp = fopen(fn.c_str(), "wb");
            if (!fp) Fail("cannot write " + fn);
            fprintf(fp, "G%d\n", D);
            fprintf(fp, "%d %s\n", 1, "DOUBLE");
            for (int d = 0; d < D; d++) fprintf(fp, d == D - 1 ? "%d\n" : "%d ", res);
            for (int j = 0; j <= D; j++)
                for (int i = 0; i <= D; i++) fprintf(fp, i == D ? "%f\n" : "%f ", (float)v2w(i, j));
            fwrite(c == 0 ? x.data() : y.data(), sizeof(double), N, fp);
            fclose(fp);
        }
    }
    epr_destroy(ctx);
    return EXIT_SUCCESS;
}
