// <out>.tree as the reference's ExteriorPoissonRecon writes it after the solve
// (ExteriorPoissonRecon/ExteriorPoissonRecon.cpp:259-270), for both of its indexers, and the
// adaptive indexer's tables.
//
//   u32 dim | u64 typeid(indexer).hash_code() (libstdc++; the reference's Extract picks the indexer
//   type by it, Extract/Extract.cpp:352-359) | XForm<double, dim+1> raw: one 8-byte word that is
//   not matrix data (written as 0), then (dim+1)^2 doubles in (column, row) order | x | y | indexer
//   x, y: u64 levels, then per level i64 n and n doubles: the hierarchical coefficients of each
//         level in the indexer's function order (Misha/Streams.h:91-130, Misha/EigenStreams.h:47-53)
//   regular indexer (HierarchicalRegularIndexer::write, Hat.adaptive.inl:198-203): u32 max depth
//   adaptive indexer (HierarchicalAdaptedIndexer::write, Hat.adaptive.inl:399-405): the node tree
//         (RegularTreeNode::write, Misha/RegularTree.inl:615-642; node = u16 depth, u16 offset[dim],
//         padding to 8 / 16 bytes, parent and children words, u64 functionIndex, u64 elementIndex,
//         -1 when none), then activeSizes (u64 count + u64 per level), then functionNodes and
//         elementNodes (u64 levels, per level u64 n and n node addresses, which the reader replaces:
//         written as zeros)
// The words that hold memory addresses in the reference's file are written as zeros and the
// children word of a node with children as 1 (its reader only tests it against null).
#include <cstdio>
#include <cstring>
#include <vector>

#include "epr_context.h"
#include "epr_kernels.h"
#include "epr_tree_walk.h"

namespace epr {
namespace {

constexpr int kMaxLevels = 16;
constexpr int64_t kChunkNodes = int64_t(1) << 20;

struct IndexMaps
{
    const int64_t *f[kMaxLevels];  // per level: function index of every grid node (-1 none)
    const int64_t *e[kMaxLevels];  // per level: element index of every grid element (-1 none)
};

__global__ void fill_kernel(int64_t *v, int64_t n, int64_t value)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = value;
}

// map[order[k]] = k
__global__ void scatter_index_kernel(const int64_t *order, int64_t n, int64_t *map)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) map[order[k]] = k;
}

// out[2k], out[2k+1] = function / element index of node k (lev < 0: the root, none)
__global__ void gather_node_index_kernel(IndexMaps M, const int8_t *lev, const int64_t *fnode, const int64_t *enode, int64_t n, int64_t *out)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int l = lev[k];
    out[2 * k] = l >= 0 && fnode[k] >= 0 ? M.f[l][fnode[k]] : -1;
    out[2 * k + 1] = l >= 0 && enode[k] >= 0 ? M.e[l][enode[k]] : -1;
}

// x[k], y[k] = the pair of node order[k] (order null: node k)
__global__ void gather_pairs_kernel(const double *xy, const int64_t *order, int64_t n, double *x, double *y)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t i = order ? order[k] : k;
    x[k] = xy[2 * i];
    y[k] = xy[2 * i + 1];
}

inline unsigned int nblk(int64_t n, int t) { return (unsigned int)((n + t - 1) / t); }

bool put(FILE *fp, const void *p, size_t bytes) { return std::fwrite(p, 1, bytes, fp) == bytes; }
template <typename T>
bool put(FILE *fp, const T &v) { return put(fp, &v, sizeof(T)); }

// bytes of zeros (the address words)
bool put_zeros(FILE *fp, size_t bytes)
{
    static const uint8_t z[4096] = {0};
    while (bytes)
    {
        const size_t n = bytes < sizeof(z) ? bytes : sizeof(z);
        if (!put(fp, z, n)) return false;
        bytes -= n;
    }
    return true;
}

}  // namespace
}  // namespace epr

extern "C" {

int epr_get_adaptive_index(epr_ctx *ctx, int level, int64_t *counts, int64_t *fnodes, size_t fcap, int64_t *enodes, size_t ecap)
{
    if (!ctx) return EPR_ERR_ARG;
    ctx->status = EPR_OK;
    cudaSetDevice(ctx->P.device);
    if (level < 0 || level > ctx->depth) { ctx->fail(EPR_ERR_ARG, "level %d out of range", level); return EPR_ERR_ARG; }
    if (ctx->adapt.empty())
    {
        ctx->fail(EPR_ERR_STATE, ctx->P.adaptive_radius < 0 ? "the context uses the regular grid (adaptive_radius -1)"
                                                             : "the adaptive indexer is not available before epr_build");
        return EPR_ERR_STATE;
    }
    const epr::AdaptiveLevel &A = ctx->adapt[level];
    if (counts) { counts[0] = A.nF; counts[1] = A.nA; counts[2] = A.nE; }
    if ((fnodes && fcap < (size_t)A.nF) || (enodes && ecap < (size_t)A.nE))
    {
        ctx->fail(EPR_ERR_ARG, "output too small");
        return EPR_ERR_ARG;
    }
    bool ok = true;
    if (fnodes && A.nF) ok = ctx->cuda_ok(cudaMemcpyAsync(fnodes, A.fnodes, sizeof(int64_t) * A.nF, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (ok && enodes && A.nE) ok = ctx->cuda_ok(cudaMemcpyAsync(enodes, A.enodes, sizeof(int64_t) * A.nE, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    ok = ok && ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync");
    return ok ? EPR_OK : (ctx->status ? ctx->status : EPR_ERR_CUDA);
}

int epr_get_regular_coefficients(epr_ctx *ctx, double *x, double *y)
{
    using namespace epr;
    if (!ctx) return EPR_ERR_ARG;
    ctx->status = EPR_OK;
    cudaSetDevice(ctx->P.device);
    if (!x || !y) { ctx->fail(EPR_ERR_ARG, "null output"); return EPR_ERR_ARG; }
    if (!ctx->solved) { ctx->fail(EPR_ERR_STATE, "epr_get_regular_coefficients needs a solved context"); return EPR_ERR_STATE; }
    cudaStream_t s = ctx->stream;
    // coef_0 = h_0; coef_d = h_d + P coef_{d-1} with the regular grid's prolongation
    double *a = nullptr, *b = nullptr, *planar = nullptr;
    const int64_t Nf = ctx->levels[ctx->depth].N;
    bool ok = ctx->alloc((void **)&a, sizeof(double) * 2 * Nf, "regular coefficients") &&
              ctx->alloc((void **)&b, sizeof(double) * 2 * Nf, "regular coefficients") &&
              ctx->alloc((void **)&planar, sizeof(double) * 2 * Nf, "regular coefficients") &&
              ctx->cuda_ok(cudaMemcpyAsync(a, ctx->levels[0].tmp64, sizeof(double) * 2 * ctx->levels[0].N, cudaMemcpyDeviceToDevice, s), "copy");
    for (int l = 1; ok && l <= ctx->depth; l++)
    {
        if (ctx->dim == 3) launch_prolong<3, double>(l - 1, a, b, 0, s);
        else launch_prolong<4, double>(l - 1, a, b, 0, s);
        launch_axpy<double>(b, ctx->levels[l].tmp64, 2 * ctx->levels[l].N, 1.0, s);
        std::swap(a, b);
        ok = ctx->launch_ok("regular coefficients");
    }
    if (ok)
    {
        gather_pairs_kernel<<<nblk(Nf, 256), 256, 0, s>>>(a, nullptr, Nf, planar, planar + Nf);
        ok = ctx->launch_ok("regular coefficients") &&
             ctx->cuda_ok(cudaMemcpyAsync(x, planar, sizeof(double) * Nf, cudaMemcpyDeviceToHost, s), "copy") &&
             ctx->cuda_ok(cudaMemcpyAsync(y, planar + Nf, sizeof(double) * Nf, cudaMemcpyDeviceToHost, s), "copy") &&
             ctx->cuda_ok(cudaStreamSynchronize(s), "sync");
    }
    ctx->release(a);
    ctx->release(b);
    ctx->release(planar);
    return ok ? EPR_OK : (ctx->status ? ctx->status : EPR_ERR_CUDA);
}

int epr_write_tree(epr_ctx *ctx, const double *voxel_to_world, const char *path)
{
    using namespace epr;
    if (!ctx) return EPR_ERR_ARG;
    ctx->status = EPR_OK;
    cudaSetDevice(ctx->P.device);
    if (!voxel_to_world || !path) { ctx->fail(EPR_ERR_ARG, "null transform or path"); return EPR_ERR_ARG; }
    if (!ctx->solved) { ctx->fail(EPR_ERR_STATE, "epr_write_tree needs a solved context"); return EPR_ERR_STATE; }
    const int D = ctx->dim, depth = ctx->depth;
    const bool adaptive = !ctx->adapt.empty();
    if (depth + 1 > kMaxLevels) { ctx->fail(EPR_ERR_ARG, "depth %d too large for the tree writer", depth); return EPR_ERR_ARG; }
    cudaStream_t s = ctx->stream;

    FILE *fp = std::fopen(path, "wb");
    if (!fp) { ctx->fail(EPR_ERR_ARG, "cannot write %s", path); return EPR_ERR_ARG; }
    std::vector<void *> owned;
    auto dev = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (!ctx->alloc(&p, bytes ? bytes : 8, "tree writer")) return nullptr;
        owned.push_back(p);
        return p;
    };
    auto finish = [&](bool ok) -> int {
        for (void *p : owned) ctx->release(p);
        if (std::fclose(fp) != 0) ok = false;
        if (!ok && ctx->status == EPR_OK) ctx->fail(EPR_ERR_ARG, "cannot write %s", path);
        return ok ? EPR_OK : ctx->status;
    };

    // header
    const uint64_t hash = adaptive ? (D == 3 ? 0xf40c6f40c49db503ull : 0xfb48bf69bf639a05ull)
                                   : (D == 3 ? 0x5aa89c06ecbfe5e7ull : 0xc7baa56b1ac9f6abull);
    bool ok = put(fp, (uint32_t)D) && put(fp, hash) && put(fp, (uint64_t)0) &&
              put(fp, voxel_to_world, sizeof(double) * (size_t)(D + 1) * (D + 1));

    // x, then y: every level's hierarchical coefficients in the indexer's order
    {
        std::vector<std::vector<double>> xs(depth + 1), ys(depth + 1);
        for (int l = 0; ok && l <= depth; l++)
        {
            const int64_t n = adaptive ? ctx->adapt[l].nF : ctx->levels[l].N;
            double *dx = (double *)dev(sizeof(double) * 2 * (size_t)n);
            if (!dx) return finish(false);
            if (n) gather_pairs_kernel<<<nblk(n, 256), 256, 0, s>>>(ctx->levels[l].tmp64, adaptive ? ctx->adapt[l].fnodes : nullptr, n, dx, dx + n);
            xs[l].resize((size_t)n);
            ys[l].resize((size_t)n);
            ok = ctx->launch_ok("tree writer") &&
                 ctx->cuda_ok(cudaMemcpyAsync(xs[l].data(), dx, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "copy") &&
                 ctx->cuda_ok(cudaMemcpyAsync(ys[l].data(), dx + n, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "copy") &&
                 ctx->cuda_ok(cudaStreamSynchronize(s), "sync");
        }
        for (auto *v : {&xs, &ys})
        {
            ok = ok && put(fp, (uint64_t)v->size());
            for (size_t l = 0; ok && l < v->size(); l++)
                ok = put(fp, (int64_t)(*v)[l].size()) && put(fp, (*v)[l].data(), sizeof(double) * (*v)[l].size());
        }
    }
    if (!ok) return finish(false);
    if (!adaptive) return finish(put(fp, (uint32_t)depth));

    // the adaptive indexer: its tree, node by node
    std::vector<std::vector<uint8_t>> refined;
    if (!adaptive_tree_refinement(*ctx, refined)) return finish(false);
    IndexMaps M{};
    for (int l = 0; l <= depth; l++)
    {
        const AdaptiveLevel &A = ctx->adapt[l];
        const int64_t N = ctx->levels[l].N, NE = (int64_t)1 << (D * l);
        int64_t *fm = (int64_t *)dev(sizeof(int64_t) * N), *em = (int64_t *)dev(sizeof(int64_t) * NE);
        if (!fm || !em) return finish(false);
        fill_kernel<<<nblk(N, 256), 256, 0, s>>>(fm, N, -1);
        fill_kernel<<<nblk(NE, 256), 256, 0, s>>>(em, NE, -1);
        if (A.nF) scatter_index_kernel<<<nblk(A.nF, 256), 256, 0, s>>>(A.fnodes, A.nF, fm);
        if (A.nE) scatter_index_kernel<<<nblk(A.nE, 256), 256, 0, s>>>(A.enodes, A.nE, em);
        M.f[l] = fm;
        M.e[l] = em;
    }
    if (!ctx->launch_ok("tree writer")) return finish(false);
    int8_t *dLev = (int8_t *)dev(kChunkNodes);
    int64_t *dF = (int64_t *)dev(sizeof(int64_t) * kChunkNodes), *dE = (int64_t *)dev(sizeof(int64_t) * kChunkNodes),
            *dOut = (int64_t *)dev(sizeof(int64_t) * 2 * kChunkNodes);
    if (!dLev || !dF || !dE || !dOut) return finish(false);

    const int ptrOff = D == 3 ? 8 : 16, dataOff = ptrOff + 16, nodeBytes = dataOff + 16;
    auto hasChildren = [&](const TreeNodeKey &k) -> bool {
        if (k.t == 0) return true;
        if (k.t > depth) return false;
        const int side = 1 << k.t;
        size_t li = 0;
        for (int d = 0; d < D; d++) li = li * side + k.O[d];
        return refined[k.t][li] != 0;
    };
    std::vector<TreeNodeKey> keys;
    std::vector<uint8_t> kids;
    std::vector<int8_t> lev;
    std::vector<int64_t> fnode, enode, idx;
    std::vector<uint8_t> bytes;
    auto flush = [&]() -> bool {
        const int64_t n = (int64_t)keys.size();
        if (!n) return true;
        idx.resize((size_t)n * 2);
        if (!ctx->cuda_ok(cudaMemcpyAsync(dLev, lev.data(), n, cudaMemcpyHostToDevice, s), "copy") ||
            !ctx->cuda_ok(cudaMemcpyAsync(dF, fnode.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s), "copy") ||
            !ctx->cuda_ok(cudaMemcpyAsync(dE, enode.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s), "copy"))
            return false;
        gather_node_index_kernel<<<nblk(n, 256), 256, 0, s>>>(M, dLev, dF, dE, n, dOut);
        if (!ctx->launch_ok("tree writer") ||
            !ctx->cuda_ok(cudaMemcpyAsync(idx.data(), dOut, sizeof(int64_t) * 2 * n, cudaMemcpyDeviceToHost, s), "copy") ||
            !ctx->cuda_ok(cudaStreamSynchronize(s), "sync"))
            return false;
        bytes.assign((size_t)n * nodeBytes, 0);
        for (int64_t k = 0; k < n; k++)
        {
            uint8_t *b = bytes.data() + (size_t)k * nodeBytes;
            const uint16_t dep = (uint16_t)keys[k].t;
            std::memcpy(b, &dep, 2);
            for (int d = 0; d < D; d++)
            {
                const uint16_t o = (uint16_t)keys[k].O[d];
                std::memcpy(b + 2 + 2 * d, &o, 2);
            }
            const uint64_t ch = kids[k] ? 1 : 0;
            std::memcpy(b + ptrOff + 8, &ch, 8);
            std::memcpy(b + dataOff, &idx[2 * k], 16);
        }
        if (!put(fp, bytes.data(), bytes.size())) return false;
        keys.clear(); kids.clear(); lev.clear(); fnode.clear(); enode.clear();
        return true;
    };
    ok = walk_tree(D, hasChildren, [&](const TreeNodeKey &k, bool has) -> bool {
        if ((int64_t)keys.size() >= kChunkNodes && !flush()) return false;
        // tree depth t >= 1 holds level t-1: its functions at offsets 0 .. 2^(t-1), its elements
        // at offsets below 2^(t-1)
        int l = k.t - 1;
        int64_t f = -1, e = -1;
        if (l >= 0)
        {
            const int r = 1 << l;
            bool inF = true, inE = true;
            int64_t fi = 0, ei = 0;
            for (int d = 0; d < D; d++)
            {
                if (k.O[d] > r) inF = false;
                if (k.O[d] >= r) inE = false;
                fi = fi * (r + 1) + k.O[d];
                ei = ei * r + k.O[d];
            }
            f = inF ? fi : -1;
            e = inE ? ei : -1;
        }
        keys.push_back(k);
        kids.push_back(has ? 1 : 0);
        lev.push_back((int8_t)l);
        fnode.push_back(f);
        enode.push_back(e);
        return true;
    });
    ok = ok && flush();
    // activeSizes, then the function and element node lists (counts; the addresses as zeros)
    ok = ok && put(fp, (uint64_t)(depth + 1));
    for (int l = 0; ok && l <= depth; l++) ok = put(fp, (uint64_t)ctx->adapt[l].nA);
    for (int which = 0; ok && which < 2; which++)
    {
        ok = put(fp, (uint64_t)(depth + 1));
        for (int l = 0; ok && l <= depth; l++)
        {
            const uint64_t n = (uint64_t)(which == 0 ? ctx->adapt[l].nF : ctx->adapt[l].nE);
            ok = put(fp, n) && put_zeros(fp, 8 * (size_t)n);
        }
    }
    return finish(ok);
}

}  // extern "C"
