// The density estimator's tree written as the reference's <out>.density.tree
// (ExteriorPoissonRecon/ExteriorPoissonRecon.cpp:272-277: the voxel-to-world XForm, then
// TreeEstimator::write, Include/GridSamples.inl:734-738, which is RegularTreeNode::write in its
// non-serialised form, Misha/RegularTree.inl:615-642, followed by targetSamplesPerCell).
//
// File layout (byte for byte the reference's, except the words that hold memory addresses or
// uninitialised padding there, which are written as zeros, and the children word of a node that
// has children, which is written as 1 -- the reference's reader only tests it against null,
// RegularTree.inl:649-660):
//   XForm<double, dim+1> as the reference writes it raw: one 8-byte word, then (dim+1)^2 doubles
//   nodes: the root, then, depth first, the 2^dim children of every node that has children as one
//          block before the subtrees of those children (child c: offset 2 O + bit d of c on axis d)
//   node (RegularTreeNode<dim, DensityAndNoiseInfo<dim>, unsigned short>, 136 bytes in 3D, 208 in
//          4D): u16 depth, u16 offset[dim], padding to 8 (3D) / 16 (4D) bytes, parent word,
//          children word, weightSum, positionSum[dim], an 8-byte padding word, covarianceSum[dim^2]
//   trailer: targetSamplesPerCell = 2^(dim-2) (GridSamples.h:241, codimension 2)
// A node of tree depth t >= 1 whose offset lies in [0, 2^(t-1)]^dim carries the splatted density of
// that vertex of the estimator's level t-1; the root and the nodes outside carry zeros.  Which nodes
// have children is the density tree's refinement (built with the density kernel radius).
//
// The node sequence is generated on the host in chunks; each chunk's data rows are gathered from
// the density levels in device memory by one kernel and copied back, so that host memory stays
// bounded by the chunk whatever the depth.
#include <cstdio>
#include <cstring>
#include <vector>

#include "epr_context.h"
#include "epr_tree_walk.h"

namespace epr {
namespace {

constexpr int kMaxTreeLevels = 16;
constexpr int64_t kChunkNodes = int64_t(1) << 20;

struct DensityLevels
{
    const double *g[kMaxTreeLevels];
};

// out[k * W + w] = density[lev[k]][idx[k] * W + w], or 0 for a node without a vertex (lev < 0)
__global__ void gather_node_data_kernel(DensityLevels L, const int8_t *lev, const int64_t *idx, int64_t n, int W, double *out)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n * W) return;
    const int64_t k = e / W;
    const int w = (int)(e - k * W);
    const int l = lev[k];
    out[e] = l < 0 ? 0.0 : L.g[l][idx[k] * W + w];
}

}  // namespace
}  // namespace epr

extern "C" {

int epr_get_density_refined(epr_ctx *ctx, int t, uint8_t *out, size_t cap, size_t *count)
{
    if (!ctx) return EPR_ERR_ARG;
    ctx->status = EPR_OK;
    cudaSetDevice(ctx->P.device);
    if (t < 0 || t > ctx->depth + 1) { ctx->fail(EPR_ERR_ARG, "tree depth %d out of range", t); return EPR_ERR_ARG; }
    const size_t num = (size_t)1 << (ctx->dim * t);
    if (count) *count = num;
    if (!out) return EPR_OK;
    if (cap < num) { ctx->fail(EPR_ERR_ARG, "output too small (%zu < %zu)", cap, num); return EPR_ERR_ARG; }
    if (ctx->setup.refinedD.empty())
    {
        ctx->fail(EPR_ERR_STATE, "the density tree is not available before epr_build");
        return EPR_ERR_STATE;
    }
    if (t == 0) { out[0] = 1; return EPR_OK; }  // the root always has children
    if (t == ctx->depth + 1) { std::memset(out, 0, num); return EPR_OK; }  // the finest cells are leaves
    if (!ctx->cuda_ok(cudaMemcpyAsync(out, ctx->setup.refinedD[t], num, cudaMemcpyDeviceToHost, ctx->stream), "copy") ||
        !ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync"))
        return ctx->status ? ctx->status : EPR_ERR_CUDA;
    return EPR_OK;
}

int epr_write_density_tree(epr_ctx *ctx, const double *voxel_to_world, const char *path)
{
    using namespace epr;
    if (!ctx) return EPR_ERR_ARG;
    ctx->status = EPR_OK;
    cudaSetDevice(ctx->P.device);
    if (!voxel_to_world || !path) { ctx->fail(EPR_ERR_ARG, "null transform or path"); return EPR_ERR_ARG; }
    const int D = ctx->dim, depth = ctx->depth;
    if (ctx->setup.refinedD.empty() || (int)ctx->setup.density.size() <= depth)
    {
        ctx->fail(EPR_ERR_STATE, "the density tree is not available before epr_build");
        return EPR_ERR_STATE;
    }
    if (depth + 1 > kMaxTreeLevels) { ctx->fail(EPR_ERR_ARG, "depth %d too large for the tree writer", depth); return EPR_ERR_ARG; }
    const int W = 1 + D + D * D;
    const int ptrOff = D == 3 ? 8 : 16, dataOff = ptrOff + 16;
    const int nodeBytes = dataOff + 8 * (W + 1);

    // refinement flags of tree depths 1..depth on the host
    std::vector<std::vector<uint8_t>> refined(depth + 1);
    for (int t = 1; t <= depth; t++)
    {
        refined[t].resize((size_t)1 << (D * t));
        if (!ctx->cuda_ok(cudaMemcpyAsync(refined[t].data(), ctx->setup.refinedD[t], refined[t].size(), cudaMemcpyDeviceToHost, ctx->stream), "copy"))
            return ctx->status;
    }
    if (!ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync")) return ctx->status;
    auto hasChildren = [&](const TreeNodeKey &k) -> bool {
        if (k.t == 0) return true;
        if (k.t > depth) return false;
        const int side = 1 << k.t;
        size_t li = 0;
        for (int d = 0; d < D; d++) li = li * side + k.O[d];
        return refined[k.t][li] != 0;
    };
    // the vertex of the estimator's level t-1 a node stands for, or -1
    auto vertex = [&](const TreeNodeKey &k, int &lev) -> int64_t {
        lev = -1;
        if (k.t == 0) return -1;
        const int r = 1 << (k.t - 1);
        int64_t idx = 0;
        for (int d = 0; d < D; d++)
        {
            if (k.O[d] > r) return -1;
            idx = idx * (r + 1) + k.O[d];
        }
        lev = k.t - 1;
        return idx;
    };

    FILE *fp = std::fopen(path, "wb");
    if (!fp) { ctx->fail(EPR_ERR_ARG, "cannot write %s", path); return EPR_ERR_ARG; }
    bool ok = true;
    {
        const uint64_t word = 0;
        ok = ok && std::fwrite(&word, 8, 1, fp) == 1;
        ok = ok && std::fwrite(voxel_to_world, sizeof(double), (size_t)(D + 1) * (D + 1), fp) == (size_t)(D + 1) * (D + 1);
    }

    DensityLevels G{};
    for (int l = 0; l <= depth; l++) G.g[l] = ctx->setup.density[l];
    int8_t *dLev = nullptr;
    int64_t *dIdx = nullptr;
    double *dOut = nullptr;
    if (!ctx->alloc((void **)&dLev, kChunkNodes, "tree writer") || !ctx->alloc((void **)&dIdx, sizeof(int64_t) * kChunkNodes, "tree writer") ||
        !ctx->alloc((void **)&dOut, sizeof(double) * W * kChunkNodes, "tree writer"))
    {
        std::fclose(fp);
        ctx->release(dLev); ctx->release(dIdx); ctx->release(dOut);
        return ctx->status ? ctx->status : EPR_ERR_NOMEM;
    }
    std::vector<TreeNodeKey> keys;
    std::vector<uint8_t> kids;
    std::vector<int8_t> lev;
    std::vector<int64_t> idx;
    std::vector<double> rows;
    std::vector<uint8_t> bytes;
    keys.reserve(kChunkNodes + 16); kids.reserve(kChunkNodes + 16); lev.reserve(kChunkNodes + 16); idx.reserve(kChunkNodes + 16);

    // writes the pending nodes: data gathered on the device, records assembled on the host
    auto flush = [&]() -> bool {
        const int64_t n = (int64_t)keys.size();
        if (!n) return true;
        rows.resize((size_t)n * W);
        if (!ctx->cuda_ok(cudaMemcpyAsync(dLev, lev.data(), n, cudaMemcpyHostToDevice, ctx->stream), "copy") ||
            !ctx->cuda_ok(cudaMemcpyAsync(dIdx, idx.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, ctx->stream), "copy"))
            return false;
        const int64_t total = n * W;
        gather_node_data_kernel<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(G, dLev, dIdx, n, W, dOut);
        if (!ctx->launch_ok("tree writer") ||
            !ctx->cuda_ok(cudaMemcpyAsync(rows.data(), dOut, sizeof(double) * total, cudaMemcpyDeviceToHost, ctx->stream), "copy") ||
            !ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync"))
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
            const double *r = rows.data() + (size_t)k * W;
            std::memcpy(b + dataOff, r, 8 * (1 + D));                               // weight, position sum
            std::memcpy(b + dataOff + 8 * (2 + D), r + 1 + D, 8 * (size_t)(D * D));  // covariance sum
        }
        if (std::fwrite(bytes.data(), 1, bytes.size(), fp) != bytes.size())
        {
            ctx->fail(EPR_ERR_ARG, "cannot write %s", path);
            return false;
        }
        keys.clear(); kids.clear(); lev.clear(); idx.clear();
        return true;
    };
    ok = ok && walk_tree(D, hasChildren, [&](const TreeNodeKey &k, bool has) -> bool {
        if ((int64_t)keys.size() >= kChunkNodes && !flush()) return false;
        int l;
        const int64_t v = vertex(k, l);
        keys.push_back(k);
        kids.push_back(has ? 1 : 0);
        lev.push_back((int8_t)l);
        idx.push_back(v);
        return true;
    });
    ok = ok && flush();
    if (ok)
    {
        const double target = (double)(1 << (D - 2));
        ok = std::fwrite(&target, sizeof(double), 1, fp) == 1;
        if (!ok) ctx->fail(EPR_ERR_ARG, "cannot write %s", path);
    }
    ctx->release(dLev);
    ctx->release(dIdx);
    ctx->release(dOut);
    if (std::fclose(fp) != 0 && ok)
    {
        ctx->fail(EPR_ERR_ARG, "cannot write %s", path);
        ok = false;
    }
    return ok ? EPR_OK : (ctx->status ? ctx->status : EPR_ERR_ARG);
}

}  // extern "C"
