// The learned warm start: a 3D convolutional U-Net that predicts the two-channel implicit function
// (x, y) of one coarse level of the cascadic solve from the splatted density and frame field of
// that level, trained on solves the method itself computes.  It has no counterpart in the
// reference, whose solve starts from random coefficients at its coarsest solve level
// (ExteriorPoisson.h:333-341); the prediction replaces that start and the levels below it.
//
// Network (node grids of resolution 2^L, 2^L + 1 nodes per axis; level L = 6: 65^3 nodes; the
// 15 input channels are listed at input_write_kernel):
//   enc0 conv(15 -> 16) @L, enc1 conv(16 -> 32) @L-1, enc2 conv(32 -> 64) @L-2, bott conv(64 -> 128)
//   @L-3, then dec2 conv(128 + 64 -> 64) @L-2, dec1 conv(64 + 32 -> 32) @L-1, dec0 conv(32 + 16 ->
//   16) @L, head conv(16 -> 2) @L; every conv 3x3x3 with zero padding, ReLU after all but the head.
//   Between levels: full-weighting restriction (the multilinear weights of the prolongation, 1/8
//   normalised) down, multilinear prolongation up (the solver's own grid transfer,
//   Hat.scalars.inl:370-386); skip connections by channel concatenation.
// Arithmetic: BF16 activations and weights, FP32 accumulation on the tensor cores (tcgen05), FP32
// master weights, Adam.  Loss: 1 - (a^2 + b^2) / (|p|^2 |t|^2) with a = <p, t>, b = <p x t> over
// the nodes' (x, y) pairs, which is invariant under scaling and rotating the prediction p, as the
// energy's minimisers are only defined up to a rotation of (x, y) (the wedge, screening, Dirichlet
// and frame terms are all invariant) and the scale is fitted at use.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/epr.h"
#include "epr_common.cuh"
#include "epr_context.h"
#include "epr_unet_kernels.cuh"

namespace epr {
namespace unet {

// ----------------------------------------------------------------------------------------------
// grid transfers between network levels (n_fine = 2 n_coarse - 1), 8 channels per thread
// ----------------------------------------------------------------------------------------------
struct Xfer
{
    const bf16 *src;
    int lds;
    bf16 *dst;
    int ldd;
    int C;  // channels (multiple of 8)
    int nsrc, ndst;
    float scale;
    const bf16 *add;  // optional: + add[v][c] (same grid as dst)
    int lda;
    const bf16 *mask;  // optional: x (mask[v][c] > 0)
    int ldm;
};

__device__ __forceinline__ void load8(const bf16 *p, float *f)
{
    const uint4 u = *reinterpret_cast<const uint4 *>(p);
    const bf16 *h = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
    for (int j = 0; j < 8; j++) f[j] = __bfloat162float(h[j]);
}

__device__ __forceinline__ void finish8(const Xfer &x, int v, float *acc)
{
    if (x.add)
    {
        float a[8];
        load8(x.add + (int64_t)v * x.lda, a);
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] += a[j];
    }
    if (x.mask)
    {
        float m[8];
        load8(x.mask + (int64_t)v * x.ldm, m);
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (!(m[j] > 0.f)) acc[j] = 0.f;
    }
    __align__(16) bf16 o[8];
#pragma unroll
    for (int j = 0; j < 8; j++) o[j] = __float2bfloat16(acc[j]);
    *reinterpret_cast<uint4 *>(x.dst + (int64_t)v * x.ldd) = *reinterpret_cast<const uint4 *>(o);
}

// dst (coarse) = scale * sum over the 3^3 fine neighbours of 2I of w(offset) src
__global__ void restrict_act_kernel(Xfer x)
{
    const int groups = x.C / 8;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nv = (int64_t)x.ndst * x.ndst * x.ndst;
    if (t >= nv * groups) return;
    const int v = (int)(t / groups), g = (int)(t - (int64_t)v * groups);
    int z, y, w;
    vox_coords(v, x.ndst, z, y, w);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int oz = -1; oz <= 1; oz++)
        for (int oy = -1; oy <= 1; oy++)
            for (int ox = -1; ox <= 1; ox++)
            {
                const int fz = 2 * z + oz, fy = 2 * y + oy, fx = 2 * w + ox;
                if ((unsigned)fz >= (unsigned)x.nsrc || (unsigned)fy >= (unsigned)x.nsrc || (unsigned)fx >= (unsigned)x.nsrc)
                    continue;
                const float wt = (oz ? 0.5f : 1.f) * (oy ? 0.5f : 1.f) * (ox ? 0.5f : 1.f) * x.scale;
                float f[8];
                load8(x.src + ((int64_t)(fz * x.nsrc + fy) * x.nsrc + fx) * x.lds + 8 * g, f);
#pragma unroll
                for (int j = 0; j < 8; j++) acc[j] += wt * f[j];
            }
    Xfer xo = x;
    xo.dst = x.dst + 8 * g;
    if (xo.add) xo.add += 8 * g;
    if (xo.mask) xo.mask += 8 * g;
    finish8(xo, v, acc);
}

// dst (fine) = scale * multilinear interpolation of src (coarse)
__global__ void prolong_act_kernel(Xfer x)
{
    const int groups = x.C / 8;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nv = (int64_t)x.ndst * x.ndst * x.ndst;
    if (t >= nv * groups) return;
    const int v = (int)(t / groups), g = (int)(t - (int64_t)v * groups);
    int c[3];
    vox_coords(v, x.ndst, c[0], c[1], c[2]);
    int lo[3], hi[3];
    float wlo[3], whi[3];
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
        lo[d] = c[d] >> 1;
        hi[d] = (c[d] + 1) >> 1;
        wlo[d] = (c[d] & 1) ? 0.5f : 1.f;
        whi[d] = (c[d] & 1) ? 0.5f : 0.f;
    }
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 8; k++)
    {
        const int iz = (k & 4) ? hi[0] : lo[0], iy = (k & 2) ? hi[1] : lo[1], ix = (k & 1) ? hi[2] : lo[2];
        const float wt = ((k & 4) ? whi[0] : wlo[0]) * ((k & 2) ? whi[1] : wlo[1]) * ((k & 1) ? whi[2] : wlo[2]) * x.scale;
        if (wt == 0.f) continue;
        float f[8];
        load8(x.src + ((int64_t)(iz * x.nsrc + iy) * x.nsrc + ix) * x.lds + 8 * g, f);
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] += wt * f[j];
    }
    Xfer xo = x;
    xo.dst = x.dst + 8 * g;
    if (xo.add) xo.add += 8 * g;
    if (xo.mask) xo.mask += 8 * g;
    finish8(xo, v, acc);
}

// ----------------------------------------------------------------------------------------------
// training pieces
// ----------------------------------------------------------------------------------------------
constexpr int kRedThreads = 256;

// per-block sums of (a, b, P, T) over nodes: a = sum p.t, b = sum p x t, P = |p|^2, T = |t|^2
__global__ void __launch_bounds__(kRedThreads) loss_partial_kernel(const float *pred, const float *tgt, int nvox, double *partial)
{
    double s[4] = {0, 0, 0, 0};
    for (int v = blockIdx.x * kRedThreads + threadIdx.x; v < nvox; v += gridDim.x * kRedThreads)
    {
        const double px = pred[2 * v], py = pred[2 * v + 1], tx = tgt[2 * v], ty = tgt[2 * v + 1];
        s[0] += px * tx + py * ty;
        s[1] += px * ty - py * tx;
        s[2] += px * px + py * py;
        s[3] += tx * tx + ty * ty;
    }
    __shared__ double sh[4][kRedThreads / 32];
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        double v = s[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4)
    {
        double v = 0;
        for (int w = 0; w < kRedThreads / 32; w++) v += sh[threadIdx.x][w];
        partial[4 * blockIdx.x + threadIdx.x] = v;
    }
}

// sums the block partials in a fixed order: out[0..3] = a, b, P, T; out[4] = the loss
__global__ void loss_finish_kernel(const double *partial, int nblocks, double *out)
{
    if (threadIdx.x < 4)
    {
        double v = 0;
        for (int b = 0; b < nblocks; b++) v += partial[4 * b + threadIdx.x];
        out[threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        const double P = out[2] > 0 ? out[2] : 1e-300, T = out[3] > 0 ? out[3] : 1e-300;
        out[4] = 1. - (out[0] * out[0] + out[1] * out[1]) / (P * T);
    }
}

// gradient of the loss with respect to the prediction, as the head's output gradient (16 BF16
// channels per voxel, channels 2-15 zero); `weight` scales it (1 / batch)
__global__ void loss_grad_kernel(const float *pred, const float *tgt, int nvox, const double *sums, float weight, bf16 *dz)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    const double a = sums[0], b = sums[1], P = sums[2] > 0 ? sums[2] : 1e-300, T = sums[3] > 0 ? sums[3] : 1e-300;
    const double nrm = a * a + b * b;
    const double px = pred[2 * v], py = pred[2 * v + 1], tx = tgt[2 * v], ty = tgt[2 * v + 1];
    const double gx = -((2 * a * tx + 2 * b * ty) * P - nrm * 2 * px) / (P * P * T);
    const double gy = -((2 * a * ty - 2 * b * tx) * P - nrm * 2 * py) / (P * P * T);
    __align__(16) bf16 o[16];
#pragma unroll
    for (int j = 0; j < 16; j++) o[j] = __float2bfloat16(0.f);
    o[0] = __float2bfloat16((float)(gx * weight));
    o[1] = __float2bfloat16((float)(gy * weight));
    uint4 *d = reinterpret_cast<uint4 *>(dz + (int64_t)v * 16);
    d[0] = reinterpret_cast<const uint4 *>(o)[0];
    d[1] = reinterpret_cast<const uint4 *>(o)[1];
}

// grad[m][c] (+)= sum over splits of partial[s][m][c]
__global__ void wgrad_reduce_kernel(const float *partial, int splits, int MN, float *grad, int accumulate)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MN) return;
    float s = 0.f;
    for (int k = 0; k < splits; k++) s += partial[(int64_t)k * MN + i];
    grad[i] = accumulate ? grad[i] + s : s;
}

// bias gradient: gb[c] (+)= sum_v dz[v][c], one block per channel, fixed-order block reduction
__global__ void __launch_bounds__(kRedThreads) bias_grad_kernel(const bf16 *dz, int ldz, int nvox, float *gb, int accumulate)
{
    const int c = blockIdx.x;
    float s = 0.f;
    for (int v = threadIdx.x; v < nvox; v += kRedThreads) s += __bfloat162float(dz[(int64_t)v * ldz + c]);
    __shared__ float sh[kRedThreads / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        float t = 0.f;
        for (int w = 0; w < kRedThreads / 32; w++) t += sh[w];
        gb[c] = accumulate ? gb[c] + t : t;
    }
}

// Adam (Kingma and Ba, 2015) on the FP32 master parameters
__global__ void adam_kernel(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2, float eps,
                            float c1, float c2)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// master weights [27 Cin][Cout] -> forward B operand [Npad][27 Cin] and data-gradient B operand
// [Cin][27 Cout] (BF16)
__global__ void relayout_kernel(const float *wm, int Cin, int Cout, int Npad, bf16 *wf, bf16 *wd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int K = 27 * Cin;
    if (i >= Npad * K) return;
    const int n = i / K, k = i - n * K;
    wf[i] = __float2bfloat16(n < Cout ? wm[(int64_t)k * Cout + n] : 0.f);
    if (wd && n < Cout)
    {
        const int t = k / Cin, ci = k - t * Cin;
        wd[(int64_t)ci * (27 * Cout) + t * Cout + n] = __float2bfloat16(wm[(int64_t)k * Cout + n]);
    }
}

// ----------------------------------------------------------------------------------------------
// the network's input and its use as a warm start
// ----------------------------------------------------------------------------------------------
// max over vertices of the density weight (channel 0 of 13) and of |frame| (3 channels), as the
// bit patterns of non-negative floats (order-independent, so deterministic)
__global__ void input_max_kernel(const double *density, const double *skew, int nvox, unsigned int *mx)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    float w = 0.f, s = 0.f;
    if (v < nvox)
    {
        w = fabsf((float)density[(int64_t)v * 13]);
        const double *k = skew + (int64_t)v * 3;
        s = (float)sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
        s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, o));
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicMax(mx, __float_as_uint(w));
        atomicMax(mx + 1, __float_as_uint(s));
    }
}

// channels (16, all scale-free): 0 density weight / max; 1-3 frame components / max |frame|;
// 4-6 the splatted samples' mean offset from the vertex, in cells (0 without weight); 7-9 the
// frame's direction (frame / |frame|, 0 where |frame| < 1e-3 max); 10 |frame| / max;
// 11-13 the vertex's coordinates in [-1, 1]; 14 log(1 + weight / max) / log 2; 15 zero
__global__ void input_write_kernel(const double *density, const double *skew, int nvox, const unsigned int *mx, bf16 *out)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    const float wm = __uint_as_float(mx[0]), sm = __uint_as_float(mx[1]);
    const float iw = wm > 0.f ? 1.f / wm : 0.f, is = sm > 0.f ? 1.f / sm : 0.f;
    int n = 1;
    while ((int64_t)n * n * n < nvox) n++;
    int z, y, x;
    vox_coords(v, n, z, y, x);
    const double *dv = density + (int64_t)v * 13;
    const double w = dv[0];
    float o32[16];
#pragma unroll
    for (int j = 0; j < 16; j++) o32[j] = 0.f;
    o32[0] = (float)w * iw;
    float sn = 0.f;
    for (int k = 0; k < 3; k++)
    {
        const float sk = (float)skew[(int64_t)v * 3 + k];
        o32[1 + k] = sk * is;
        sn += sk * sk;
    }
    sn = sqrtf(sn);
    if (w > 0)
    {
        const int c[3] = {z, y, x};
        for (int k = 0; k < 3; k++) o32[4 + k] = (float)(dv[1 + k] / w * (n - 1) - c[k]);
    }
    if (sn > 1e-3f * sm && sn > 0.f)
        for (int k = 0; k < 3; k++) o32[7 + k] = (float)skew[(int64_t)v * 3 + k] / sn;
    o32[10] = sn * is;
    o32[11] = 2.f * z / (n - 1) - 1.f;
    o32[12] = 2.f * y / (n - 1) - 1.f;
    o32[13] = 2.f * x / (n - 1) - 1.f;
    o32[14] = log1pf(o32[0]) / 0.69314718f;
    __align__(16) bf16 o[16];
#pragma unroll
    for (int j = 0; j < 16; j++) o[j] = __float2bfloat16(o32[j]);
    uint4 *d = reinterpret_cast<uint4 *>(out + (int64_t)v * 16);
    d[0] = reinterpret_cast<const uint4 *>(o)[0];
    d[1] = reinterpret_cast<const uint4 *>(o)[1];
}

// interleaved double coefficients (x, y) = scale * prediction
__global__ void pred_to_xy_kernel(const float *pred, int nvox, double sx, double sy, double *xy)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    xy[2 * v] = sx * (double)pred[2 * v];
    xy[2 * v + 1] = sy * (double)pred[2 * v + 1];
}

// target of a training pair: the level's regular double coefficients as FP32 pairs
__global__ void xy_to_target_kernel(const double *xy, int nvox, float *t)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    t[2 * v] = (float)xy[2 * v];
    t[2 * v + 1] = (float)xy[2 * v + 1];
}

inline int nblk(int64_t n, int t) { return (int)((n + t - 1) / t); }

template <int N>
void launch_conv_n(const ConvArgs &a, cudaStream_t s)
{
    const size_t smem = 2 * (size_t)kBM * kBK * 2 + 2 * (size_t)N * kBK * 2;
    static bool attr = false;  // set once per process (every device shares the value)
    if (!attr)
    {
        cudaFuncSetAttribute(conv3_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    conv3_kernel<N><<<nblk(a.nvox, kBM), kThreads, smem, s>>>(a);
}

template <int N>
void launch_wgrad_n(const WgradArgs &a, int splits, cudaStream_t s)
{
    const size_t smem = 2 * (size_t)kBM * kBK * 2 + 2 * (size_t)N * kBK * 2;
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(conv3_wgrad_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    dim3 grid(nblk(a.M, kBM), splits);
    conv3_wgrad_kernel<N><<<grid, kThreads, smem, s>>>(a);
}

bool conv_supported(int N) { return N == 16 || N == 32 || N == 48 || N == 64 || N == 96 || N == 128 || N == 192; }

void launch_conv(int N, const ConvArgs &a, cudaStream_t s)
{
    switch (N)
    {
    case 16: launch_conv_n<16>(a, s); break;
    case 32: launch_conv_n<32>(a, s); break;
    case 48: launch_conv_n<48>(a, s); break;
    case 64: launch_conv_n<64>(a, s); break;
    case 96: launch_conv_n<96>(a, s); break;
    case 128: launch_conv_n<128>(a, s); break;
    case 192: launch_conv_n<192>(a, s); break;
    default: break;
    }
}

void launch_wgrad(int N, const WgradArgs &a, int splits, cudaStream_t s)
{
    switch (N)
    {
    case 16: launch_wgrad_n<16>(a, splits, s); break;
    case 32: launch_wgrad_n<32>(a, splits, s); break;
    case 48: launch_wgrad_n<48>(a, splits, s); break;
    case 64: launch_wgrad_n<64>(a, splits, s); break;
    case 96: launch_wgrad_n<96>(a, splits, s); break;
    case 128: launch_wgrad_n<128>(a, splits, s); break;
    case 192: launch_wgrad_n<192>(a, splits, s); break;
    default: break;
    }
}

// voxels per split of the weight gradient: about two CTAs per SM over all M tiles, whole stages
int wgrad_split_voxels(int nvox, int mtiles)
{
    const int target = std::max(1, 2 * 148 / std::max(1, mtiles));
    int per = (nvox + target - 1) / target;
    per = (per + kBK - 1) / kBK * kBK;
    return std::max(per, kBK);
}

// ----------------------------------------------------------------------------------------------
// the network
// ----------------------------------------------------------------------------------------------
struct Layer
{
    int Cin, Cout, Npad, level;  // GEMM input channels (multiple of 16), output channels, padded N
    bool relu;
    size_t woff, boff;  // offsets of the master weights [27 Cin][Cout] and bias [Cout] in the flat array
    bf16 *wf = nullptr, *wd = nullptr;
    float *bias = nullptr;  // device view of the master bias (FP32)
};

// a channels-last activation buffer
struct Act
{
    bf16 *p = nullptr;
    int ld = 0, n = 0;
    int64_t vox() const { return (int64_t)n * n * n; }
};

enum LayerId { ENC0, ENC1, ENC2, BOTT, DEC2, DEC1, DEC0, HEAD, NLAYERS };

}  // namespace unet
}  // namespace epr

struct epr_unet
{
    int device = 0, level = 6;
    std::string err;
    cudaStream_t stream = nullptr;
    std::vector<epr::unet::Layer> L;
    size_t nparams = 0;
    float *params = nullptr, *grads = nullptr, *m1 = nullptr, *m2 = nullptr;
    int64_t adam_t = 0;
    int n[4] = {0, 0, 0, 0};  // nodes per axis at network levels 0..3
    // activations: input, concat buffers, encoder outputs below the top, decoder outputs
    epr::unet::Act in0, cat0, cat1, cat2, d0, d1, d2, b3, u2, u1, u0;
    float *pred = nullptr;
    // gradients
    epr::unet::Act dhead, du0, dcat0, dcat1, dcat2, db3, dd2, dd1, dd0, dz1, dz2, dzb, dze2, dze1, dze0;
    float *wpart = nullptr;
    size_t wpart_floats = 0;
    double *lred = nullptr;  // loss partials (4 x kLossBlocks) + sums (5)
    unsigned int *d_err = nullptr, *d_max = nullptr;
    std::vector<void *> allocs;

    bool fail(const char *fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return false;
    }
    bool cuda(cudaError_t e, const char *what)
    {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        return fail("%s: %s", what, cudaGetErrorString(e));
    }
    template <typename T>
    bool alloc(T **p, size_t count, const char *what)
    {
        void *q = nullptr;
        if (!cuda(cudaMalloc(&q, count * sizeof(T)), what)) return false;
        allocs.push_back(q);
        *p = (T *)q;
        return cuda(cudaMemsetAsync(q, 0, count * sizeof(T), stream), what);
    }
    bool act(epr::unet::Act &a, int nn, int ld, const char *what)
    {
        a.n = nn;
        a.ld = ld;
        return alloc(&a.p, (size_t)a.vox() * ld, what);
    }
    ~epr_unet()
    {
        if (stream) cudaStreamSynchronize(stream);
        for (void *p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace epr {
namespace unet {

constexpr int kLossBlocks = 256;

bool conv(epr_unet *net, const Layer &ly, const Act &in, int ldi_cin, const bf16 *w, int N, const float *bias, Act *out,
          int out_off, int nout, float *outf, int nf, const Act *mask, int relu, int flip, int Kcin)
{
    ConvArgs a{};
    a.in = in.p;
    a.ldi = in.ld;
    a.Cin = Kcin;
    a.W = w;
    a.K = 27 * Kcin;
    a.bias = bias;
    a.out = out ? out->p + out_off : nullptr;
    a.ldo = out ? out->ld : 0;
    a.nout = nout;
    a.outf = outf;
    a.ldf = 2;
    a.nf = nf;
    a.mask = mask ? mask->p : nullptr;
    a.ldm = mask ? mask->ld : 0;
    a.relu = relu;
    a.flip = flip;
    a.n = in.n;
    a.nvox = (int)in.vox();
    a.err = net->d_err;
    (void)ly;
    (void)ldi_cin;
    launch_conv(N, a, net->stream);
    return net->cuda(cudaGetLastError(), "conv");
}

bool xfer(epr_unet *net, bool restrict_, const bf16 *src, int lds, int nsrc, bf16 *dst, int ldd, int ndst, int C, float scale,
          const bf16 *add, int lda, const bf16 *mask, int ldm)
{
    Xfer x{src, lds, dst, ldd, C, nsrc, ndst, scale, add, lda, mask, ldm};
    const int64_t work = (int64_t)ndst * ndst * ndst * (C / 8);
    if (restrict_) restrict_act_kernel<<<nblk(work, 256), 256, 0, net->stream>>>(x);
    else prolong_act_kernel<<<nblk(work, 256), 256, 0, net->stream>>>(x);
    return net->cuda(cudaGetLastError(), "grid transfer");
}

bool relayout(epr_unet *net)
{
    for (Layer &ly : net->L)
    {
        const int total = ly.Npad * 27 * ly.Cin;
        relayout_kernel<<<nblk(total, 256), 256, 0, net->stream>>>(net->params + ly.woff, ly.Cin, ly.Cout, ly.Npad, ly.wf, ly.wd);
    }
    return net->cuda(cudaGetLastError(), "relayout");
}

bool forward(epr_unet *net, const Act &in)
{
    auto &L = net->L;
    const float s8 = 1.f / 8.f;
    // enc0 -> cat0[:, 32:48]
    if (!conv(net, L[ENC0], in, 0, L[ENC0].wf, 16, L[ENC0].bias, &net->cat0, 32, 16, nullptr, 0, nullptr, 1, 0, 16)) return false;
    if (!xfer(net, true, net->cat0.p + 32, net->cat0.ld, net->n[0], net->d0.p, net->d0.ld, net->n[1], 16, s8, nullptr, 0, nullptr, 0)) return false;
    if (!conv(net, L[ENC1], net->d0, 0, L[ENC1].wf, 32, L[ENC1].bias, &net->cat1, 64, 32, nullptr, 0, nullptr, 1, 0, 16)) return false;
    if (!xfer(net, true, net->cat1.p + 64, net->cat1.ld, net->n[1], net->d1.p, net->d1.ld, net->n[2], 32, s8, nullptr, 0, nullptr, 0)) return false;
    if (!conv(net, L[ENC2], net->d1, 0, L[ENC2].wf, 64, L[ENC2].bias, &net->cat2, 128, 64, nullptr, 0, nullptr, 1, 0, 32)) return false;
    if (!xfer(net, true, net->cat2.p + 128, net->cat2.ld, net->n[2], net->d2.p, net->d2.ld, net->n[3], 64, s8, nullptr, 0, nullptr, 0)) return false;
    if (!conv(net, L[BOTT], net->d2, 0, L[BOTT].wf, 128, L[BOTT].bias, &net->b3, 0, 128, nullptr, 0, nullptr, 1, 0, 64)) return false;
    // decoder
    if (!xfer(net, false, net->b3.p, net->b3.ld, net->n[3], net->cat2.p, net->cat2.ld, net->n[2], 128, 1.f, nullptr, 0, nullptr, 0)) return false;
    if (!conv(net, L[DEC2], net->cat2, 0, L[DEC2].wf, 64, L[DEC2].bias, &net->u2, 0, 64, nullptr, 0, nullptr, 1, 0, 192)) return false;
    if (!xfer(net, false, net->u2.p, net->u2.ld, net->n[2], net->cat1.p, net->cat1.ld, net->n[1], 64, 1.f, nullptr, 0, nullptr, 0)) return false;
    if (!conv(net, L[DEC1], net->cat1, 0, L[DEC1].wf, 32, L[DEC1].bias, &net->u1, 0, 32, nullptr, 0, nullptr, 1, 0, 96)) return false;
    if (!xfer(net, false, net->u1.p, net->u1.ld, net->n[1], net->cat0.p, net->cat0.ld, net->n[0], 32, 1.f, nullptr, 0, nullptr, 0)) return false;
    if (!conv(net, L[DEC0], net->cat0, 0, L[DEC0].wf, 16, L[DEC0].bias, &net->u0, 0, 16, nullptr, 0, nullptr, 1, 0, 48)) return false;
    return conv(net, L[HEAD], net->u0, 0, L[HEAD].wf, 16, L[HEAD].bias, nullptr, 0, 0, net->pred, 2, nullptr, 0, 0, 16);
}

bool wgrad(epr_unet *net, const Layer &ly, const Act &in, int in_off, const Act &dz, bool accumulate)
{
    WgradArgs a{};
    a.in = in.p + in_off;
    a.ldi = in.ld;
    a.Cin = ly.Cin;
    a.dz = dz.p;
    a.ldz = dz.ld;
    a.M = 27 * ly.Cin;
    a.n = in.n;
    a.nvox = (int)in.vox();
    a.err = net->d_err;
    const int mtiles = nblk(a.M, kBM);
    a.vox_per_split = wgrad_split_voxels(a.nvox, mtiles);
    const int splits = nblk(a.nvox, a.vox_per_split);
    const size_t need = (size_t)splits * a.M * ly.Npad;
    if (need > net->wpart_floats) return net->fail("weight-gradient scratch too small (%zu > %zu)", need, net->wpart_floats);
    a.partial = net->wpart;
    launch_wgrad(ly.Npad, a, splits, net->stream);
    // the master gradient is [27 Cin][Cout]: reduce the [27 Cin][Npad] partials (Npad == Cout for
    // every layer: the head's master weights are 16 wide with columns 2-15 kept at zero)
    const int MN = a.M * ly.Npad;
    wgrad_reduce_kernel<<<nblk(MN, 256), 256, 0, net->stream>>>(net->wpart, splits, MN, net->grads + ly.woff, accumulate);
    bias_grad_kernel<<<ly.Cout, kRedThreads, 0, net->stream>>>(dz.p, dz.ld, (int)dz.vox(), net->grads + ly.boff, accumulate);
    return net->cuda(cudaGetLastError(), "weight gradient");
}

// backward pass from the head's output gradient net->dhead; accumulate adds into the gradients
bool backward(epr_unet *net, const Act &in, bool acc)
{
    auto &L = net->L;
    const float s8 = 1.f / 8.f;
    // head: dz = dhead (no activation)
    if (!wgrad(net, L[HEAD], net->u0, 0, net->dhead, acc)) return false;
    if (!conv(net, L[HEAD], net->dhead, 0, L[HEAD].wd, 16, nullptr, &net->du0, 0, 16, nullptr, 0, &net->u0, 0, 1, 16)) return false;
    // dec0: dz = du0 (masked above); input cat0 (48)
    if (!wgrad(net, L[DEC0], net->cat0, 0, net->du0, acc)) return false;
    if (!conv(net, L[DEC0], net->du0, 0, L[DEC0].wd, 48, nullptr, &net->dcat0, 0, 48, nullptr, 0, nullptr, 0, 1, 16)) return false;
    // up0 backward: du1 = restrict(dcat0[:, 0:32]) masked by u1
    if (!xfer(net, true, net->dcat0.p, net->dcat0.ld, net->n[0], net->dz1.p, net->dz1.ld, net->n[1], 32, 1.f, nullptr, 0, net->u1.p, net->u1.ld)) return false;
    if (!wgrad(net, L[DEC1], net->cat1, 0, net->dz1, acc)) return false;
    if (!conv(net, L[DEC1], net->dz1, 0, L[DEC1].wd, 96, nullptr, &net->dcat1, 0, 96, nullptr, 0, nullptr, 0, 1, 32)) return false;
    if (!xfer(net, true, net->dcat1.p, net->dcat1.ld, net->n[1], net->dz2.p, net->dz2.ld, net->n[2], 64, 1.f, nullptr, 0, net->u2.p, net->u2.ld)) return false;
    if (!wgrad(net, L[DEC2], net->cat2, 0, net->dz2, acc)) return false;
    if (!conv(net, L[DEC2], net->dz2, 0, L[DEC2].wd, 192, nullptr, &net->dcat2, 0, 192, nullptr, 0, nullptr, 0, 1, 64)) return false;
    if (!xfer(net, true, net->dcat2.p, net->dcat2.ld, net->n[2], net->dzb.p, net->dzb.ld, net->n[3], 128, 1.f, nullptr, 0, net->b3.p, net->b3.ld)) return false;
    // bottleneck
    if (!wgrad(net, L[BOTT], net->d2, 0, net->dzb, acc)) return false;
    if (!conv(net, L[BOTT], net->dzb, 0, L[BOTT].wd, 64, nullptr, &net->dd2, 0, 64, nullptr, 0, nullptr, 0, 1, 128)) return false;
    // enc2 output gradient: skip part + prolong(dd2) / 8, masked by enc2's output
    if (!xfer(net, false, net->dd2.p, net->dd2.ld, net->n[3], net->dze2.p, net->dze2.ld, net->n[2], 64, s8,
              net->dcat2.p + 128, net->dcat2.ld, net->cat2.p + 128, net->cat2.ld)) return false;
    if (!wgrad(net, L[ENC2], net->d1, 0, net->dze2, acc)) return false;
    if (!conv(net, L[ENC2], net->dze2, 0, L[ENC2].wd, 32, nullptr, &net->dd1, 0, 32, nullptr, 0, nullptr, 0, 1, 64)) return false;
    if (!xfer(net, false, net->dd1.p, net->dd1.ld, net->n[2], net->dze1.p, net->dze1.ld, net->n[1], 32, s8,
              net->dcat1.p + 64, net->dcat1.ld, net->cat1.p + 64, net->cat1.ld)) return false;
    if (!wgrad(net, L[ENC1], net->d0, 0, net->dze1, acc)) return false;
    if (!conv(net, L[ENC1], net->dze1, 0, L[ENC1].wd, 16, nullptr, &net->dd0, 0, 16, nullptr, 0, nullptr, 0, 1, 32)) return false;
    if (!xfer(net, false, net->dd0.p, net->dd0.ld, net->n[1], net->dze0.p, net->dze0.ld, net->n[0], 16, s8,
              net->dcat0.p + 32, net->dcat0.ld, net->cat0.p + 32, net->cat0.ld)) return false;
    return wgrad(net, L[ENC0], in, 0, net->dze0, acc);
}

bool build_net(epr_unet *net, uint64_t seed)
{
    const int lv = net->level;
    for (int k = 0; k < 4; k++) net->n[k] = (1 << (lv - k)) + 1;
    struct Spec { int cin, cinReal, cout, level; bool relu; };
    const Spec spec[NLAYERS] = {{16, 15, 16, 0, true},   {16, 16, 32, 1, true},  {32, 32, 64, 2, true},  {64, 64, 128, 3, true},
                                {192, 192, 64, 2, true}, {96, 96, 32, 1, true}, {48, 48, 16, 0, true},  {16, 16, 16, 0, false}};
    size_t off = 0;
    net->L.resize(NLAYERS);
    for (int i = 0; i < NLAYERS; i++)
    {
        Layer &ly = net->L[i];
        ly.Cin = spec[i].cin;
        ly.Cout = spec[i].cout;
        ly.Npad = spec[i].cout;
        ly.level = spec[i].level;
        ly.relu = spec[i].relu;
        ly.woff = off;
        off += (size_t)27 * ly.Cin * ly.Cout;
        ly.boff = off;
        off += ly.Cout;
    }
    net->nparams = off;
    if (!net->alloc(&net->params, off, "params") || !net->alloc(&net->grads, off, "grads") || !net->alloc(&net->m1, off, "adam m") ||
        !net->alloc(&net->m2, off, "adam v"))
        return false;
    // He-normal initialisation on the host (fan-in of the real input channels), zero biases; the
    // padded input channels of enc0 and the padded output columns of the head start at zero
    std::vector<float> h(off, 0.f);
    std::mt19937_64 rng(seed);
    for (int i = 0; i < NLAYERS; i++)
    {
        const Layer &ly = net->L[i];
        const int coutReal = i == HEAD ? 2 : ly.Cout;
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (27.f * spec[i].cinReal)) * (i == HEAD ? 0.5f : 1.f));
        for (int k = 0; k < 27 * ly.Cin; k++)
            for (int c = 0; c < ly.Cout; c++)
            {
                const int ci = k % ly.Cin;
                const float val = nd(rng);
                if (ci < spec[i].cinReal && c < coutReal) h[ly.woff + (size_t)k * ly.Cout + c] = val;
            }
    }
    if (!net->cuda(cudaMemcpyAsync(net->params, h.data(), off * sizeof(float), cudaMemcpyHostToDevice, net->stream), "upload params"))
        return false;
    for (int i = 0; i < NLAYERS; i++)
    {
        Layer &ly = net->L[i];
        if (!net->alloc(&ly.wf, (size_t)ly.Npad * 27 * ly.Cin, "weights")) return false;
        if (i != ENC0 && !net->alloc(&ly.wd, (size_t)ly.Cin * 27 * ly.Cout, "weights")) return false;
        ly.bias = net->params + ly.boff;
    }
    const int *n = net->n;
    bool ok = net->act(net->in0, n[0], 16, "act") && net->act(net->cat0, n[0], 48, "act") && net->act(net->cat1, n[1], 96, "act") &&
              net->act(net->cat2, n[2], 192, "act") && net->act(net->d0, n[1], 16, "act") && net->act(net->d1, n[2], 32, "act") &&
              net->act(net->d2, n[3], 64, "act") && net->act(net->b3, n[3], 128, "act") && net->act(net->u2, n[2], 64, "act") &&
              net->act(net->u1, n[1], 32, "act") && net->act(net->u0, n[0], 16, "act") &&
              net->alloc(&net->pred, (size_t)2 * net->in0.vox(), "pred") && net->act(net->dhead, n[0], 16, "grad") &&
              net->act(net->du0, n[0], 16, "grad") && net->act(net->dcat0, n[0], 48, "grad") && net->act(net->dcat1, n[1], 96, "grad") &&
              net->act(net->dcat2, n[2], 192, "grad") && net->act(net->dd2, n[3], 64, "grad") && net->act(net->dd1, n[2], 32, "grad") &&
              net->act(net->dd0, n[1], 16, "grad") && net->act(net->dz1, n[1], 32, "grad") && net->act(net->dz2, n[2], 64, "grad") &&
              net->act(net->dzb, n[3], 128, "grad") && net->act(net->dze2, n[2], 64, "grad") && net->act(net->dze1, n[1], 32, "grad") &&
              net->act(net->dze0, n[0], 16, "grad") && net->alloc(&net->lred, 4 * kLossBlocks + 8, "loss") &&
              net->alloc(&net->d_err, 1, "flag") && net->alloc(&net->d_max, 2, "max");
    if (!ok) return false;
    // weight-gradient scratch: the largest splits x M x N over the layers
    size_t mx = 0;
    for (const Layer &ly : net->L)
    {
        const int nv = net->n[ly.level] * net->n[ly.level] * net->n[ly.level];
        const int M = 27 * ly.Cin, mt = nblk(M, kBM);
        const int per = wgrad_split_voxels(nv, mt);
        mx = std::max(mx, (size_t)nblk(nv, per) * M * ly.Npad);
    }
    net->wpart_floats = mx;
    if (!net->alloc(&net->wpart, mx, "weight-gradient scratch")) return false;
    return relayout(net) && net->cuda(cudaStreamSynchronize(net->stream), "sync");
}

bool check_flag(epr_unet *net)
{
    unsigned int h = 0;
    if (!net->cuda(cudaMemcpyAsync(&h, net->d_err, sizeof(h), cudaMemcpyDeviceToHost, net->stream), "flag") ||
        !net->cuda(cudaStreamSynchronize(net->stream), "sync"))
        return false;
    if (h & tc::kErrWaitTimeout) return net->fail("a tensor-core pipeline wait timed out");
    return true;
}

// loss of net->pred against target; writes the head's output gradient (x weight) when dz != null
bool loss(epr_unet *net, const float *target, float weight, bool grad, double *out)
{
    const int nv = (int)net->in0.vox();
    loss_partial_kernel<<<kLossBlocks, kRedThreads, 0, net->stream>>>(net->pred, target, nv, net->lred);
    loss_finish_kernel<<<1, 32, 0, net->stream>>>(net->lred, kLossBlocks, net->lred + 4 * kLossBlocks);
    if (grad) loss_grad_kernel<<<nblk(nv, 256), 256, 0, net->stream>>>(net->pred, target, nv, net->lred + 4 * kLossBlocks, weight, net->dhead.p);
    if (!net->cuda(cudaGetLastError(), "loss")) return false;
    if (out)
    {
        double h[5];
        if (!net->cuda(cudaMemcpyAsync(h, net->lred + 4 * kLossBlocks, sizeof(h), cudaMemcpyDeviceToHost, net->stream), "loss copy") ||
            !net->cuda(cudaStreamSynchronize(net->stream), "sync"))
            return false;
        *out = h[4];
    }
    return true;
}

}  // namespace unet
}  // namespace epr

// ==============================================================================================
// C ABI
// ==============================================================================================
using namespace epr::unet;

namespace {
thread_local std::string g_unet_error;
int prim_fail(const char *msg)
{
    g_unet_error = msg;
    return EPR_ERR_ARG;
}
}  // namespace

extern "C" {

const char *epr_conv_last_error(void) { return g_unet_error.c_str(); }

int epr_conv3(int device, int n, int cin, int cout, const void *in, int ldi, const void *w, const float *bias, void *out, int ldo,
              int relu, int flip, void *stream)
{
    if (n < 1 || n > 1025 || cin < 16 || cin % 16 || !conv_supported(cout)) return prim_fail("bad sizes (cin: multiple of 16; cout: 16, 32, 48, 64, 96, 128 or 192)");
    if (!in || !w || !out || ldi < cin || ldo < cout || ldi % 8 || ldo % 8) return prim_fail("bad pointers or row strides");
    if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(w) | reinterpret_cast<uintptr_t>(out)) & 15)
        return prim_fail("device buffers must be 16-byte aligned");
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != device && cudaSetDevice(device) != cudaSuccess) return prim_fail("cannot select the device");
    ConvArgs a{};
    a.in = (const bf16 *)in;
    a.ldi = ldi;
    a.Cin = cin;
    a.W = (const bf16 *)w;
    a.K = 27 * cin;
    a.bias = bias;
    a.out = (bf16 *)out;
    a.ldo = ldo;
    a.nout = cout;
    a.relu = relu;
    a.flip = flip;
    a.n = n;
    a.nvox = n * n * n;
    a.err = nullptr;
    launch_conv(cout, a, (cudaStream_t)stream);
    cudaError_t e = cudaGetLastError();
    if (cur != device) cudaSetDevice(cur);
    if (e != cudaSuccess) return prim_fail(cudaGetErrorString(e)), EPR_ERR_CUDA;
    return EPR_OK;
}

int epr_conv3_wgrad(int device, int n, int cin, int cout, const void *in, int ldi, const void *dz, int ldz, float *dw,
                    float *scratch, size_t scratch_floats, void *stream)
{
    if (n < 1 || n > 1025 || cin < 16 || cin % 16 || !conv_supported(cout)) return prim_fail("bad sizes");
    if (!in || !dz || !dw || !scratch || ldi < cin || ldz < cout || ldi % 8 || ldz % 8) return prim_fail("bad pointers or row strides");
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != device && cudaSetDevice(device) != cudaSuccess) return prim_fail("cannot select the device");
    WgradArgs a{};
    a.in = (const bf16 *)in;
    a.ldi = ldi;
    a.Cin = cin;
    a.dz = (const bf16 *)dz;
    a.ldz = ldz;
    a.M = 27 * cin;
    a.n = n;
    a.nvox = n * n * n;
    const int mtiles = nblk(a.M, kBM);
    a.vox_per_split = wgrad_split_voxels(a.nvox, mtiles);
    const int splits = nblk(a.nvox, a.vox_per_split);
    if ((size_t)splits * a.M * cout > scratch_floats)
    {
        if (cur != device) cudaSetDevice(cur);
        return prim_fail("scratch too small");
    }
    a.partial = scratch;
    cudaStream_t s = (cudaStream_t)stream;
    launch_wgrad(cout, a, splits, s);
    const int MN = a.M * cout;
    wgrad_reduce_kernel<<<nblk(MN, 256), 256, 0, s>>>(scratch, splits, MN, dw, 0);
    cudaError_t e = cudaGetLastError();
    if (cur != device) cudaSetDevice(cur);
    if (e != cudaSuccess) return prim_fail(cudaGetErrorString(e)), EPR_ERR_CUDA;
    return EPR_OK;
}

size_t epr_conv3_wgrad_scratch(int n, int cin, int cout)
{
    const int M = 27 * cin, nv = n * n * n;
    const int per = wgrad_split_voxels(nv, nblk(M, kBM));
    return (size_t)nblk(nv, per) * M * cout;
}

epr_unet *epr_unet_create(int device, int level, uint64_t seed)
{
    if (level < 3 || level > 8)
    {
        g_unet_error = "network level must be in 3..8";
        return nullptr;
    }
    if (cudaSetDevice(device) != cudaSuccess)
    {
        g_unet_error = "cannot select the device";
        return nullptr;
    }
    epr_unet *net = new epr_unet;
    net->device = device;
    net->level = level;
    if (cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) != cudaSuccess || !build_net(net, seed))
    {
        g_unet_error = net->err.empty() ? "CUDA initialisation failed" : net->err;
        delete net;
        return nullptr;
    }
    return net;
}

void epr_unet_destroy(epr_unet *net) { delete net; }

const char *epr_unet_last_error(const epr_unet *net) { return net ? net->err.c_str() : g_unet_error.c_str(); }

int epr_unet_params(epr_unet *net, float *host, size_t cap, size_t *count, int set)
{
    if (!net) return EPR_ERR_ARG;
    cudaSetDevice(net->device);
    if (count) *count = net->nparams;
    if (!host) return EPR_OK;
    if (cap < net->nparams) return net->fail("buffer too small"), EPR_ERR_ARG;
    bool ok;
    if (set)
        ok = net->cuda(cudaMemcpyAsync(net->params, host, net->nparams * sizeof(float), cudaMemcpyHostToDevice, net->stream), "upload") &&
             relayout(net);
    else
        ok = net->cuda(cudaMemcpyAsync(host, net->params, net->nparams * sizeof(float), cudaMemcpyDeviceToHost, net->stream), "download");
    ok = ok && net->cuda(cudaStreamSynchronize(net->stream), "sync");
    return ok ? EPR_OK : EPR_ERR_CUDA;
}

int epr_unet_grid(const epr_unet *net, int *nodes_per_axis, size_t *input_bytes, size_t *target_floats)
{
    if (!net) return EPR_ERR_ARG;
    const size_t nv = (size_t)net->in0.vox();
    if (nodes_per_axis) *nodes_per_axis = net->n[0];
    if (input_bytes) *input_bytes = nv * 16 * sizeof(bf16);
    if (target_floats) *target_floats = 2 * nv;
    return EPR_OK;
}

int epr_unet_forward(epr_unet *net, const void *dev_input, float *dev_pred, double *loss_out, const void *dev_target_v)
{
    if (!net) return EPR_ERR_ARG;
    cudaSetDevice(net->device);
    Act in = net->in0;
    if (dev_input) in.p = (bf16 *)dev_input;
    const float *dev_target = (const float *)dev_target_v;
    bool ok = forward(net, in);
    if (ok && dev_target && loss_out) ok = loss(net, dev_target, 1.f, false, loss_out);
    if (ok && dev_pred)
        ok = net->cuda(cudaMemcpyAsync(dev_pred, net->pred, sizeof(float) * 2 * net->in0.vox(), cudaMemcpyDeviceToDevice, net->stream), "copy");
    ok = ok && net->cuda(cudaStreamSynchronize(net->stream), "sync") && check_flag(net);
    return ok ? EPR_OK : EPR_ERR_CUDA;
}

int epr_unet_gradients(epr_unet *net, const void *dev_input, const void *dev_target_v, float *host_grads, double *loss_out)
{
    const float *dev_target = (const float *)dev_target_v;
    if (!net || !dev_input || !dev_target) return EPR_ERR_ARG;
    cudaSetDevice(net->device);
    Act in = net->in0;
    in.p = (bf16 *)dev_input;
    bool ok = forward(net, in) && loss(net, dev_target, 1.f, true, loss_out) && backward(net, in, false);
    if (ok && host_grads)
        ok = net->cuda(cudaMemcpyAsync(host_grads, net->grads, net->nparams * sizeof(float), cudaMemcpyDeviceToHost, net->stream), "copy");
    ok = ok && net->cuda(cudaStreamSynchronize(net->stream), "sync") && check_flag(net);
    return ok ? EPR_OK : EPR_ERR_CUDA;
}

int epr_unet_train_step(epr_unet *net, int batch, const void *const *inputs, const void *const *targets, float lr, double *loss_out)
{
    if (!net || batch < 1 || !inputs || !targets) return EPR_ERR_ARG;
    cudaSetDevice(net->device);
    double total = 0;
    bool ok = true;
    for (int b = 0; ok && b < batch; b++)
    {
        Act in = net->in0;
        in.p = (bf16 *)inputs[b];
        double l = 0;
        ok = forward(net, in) && loss(net, (const float *)targets[b], 1.f / batch, true, &l) && backward(net, in, b > 0);
        total += l;
    }
    if (ok)
    {
        net->adam_t++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)net->adam_t), c2 = 1.f - std::pow(b2, (float)net->adam_t);
        adam_kernel<<<nblk((int64_t)net->nparams, 256), 256, 0, net->stream>>>(net->params, net->grads, net->m1, net->m2,
                                                                               (int64_t)net->nparams, lr, b1, b2, 1e-8f, c1, c2);
        ok = net->cuda(cudaGetLastError(), "adam") && relayout(net) && net->cuda(cudaStreamSynchronize(net->stream), "sync") &&
             check_flag(net);
    }
    if (loss_out) *loss_out = total / batch;
    return ok ? EPR_OK : EPR_ERR_CUDA;
}

}  // extern "C"

// ----------------------------------------------------------------------------------------------
// warm start of a reconstruction context
// ----------------------------------------------------------------------------------------------
namespace epr {

// network input of a built 3D context at the network's level (density and frame splats)
bool unet_input(epr_unet *net, Context &c, bf16 *dst)
{
    const int L = net->level;
    if (c.dim != 3) return net->fail("the learned warm start is 3D");
    if (c.depth < L) return net->fail("the context's depth %d is below the network's level %d", c.depth, L);
    if ((int)c.setup.density.size() <= L || !c.setup.density[L] || !c.setup.skewGrid[L])
        return net->fail("the context has no splats (call epr_build first)");
    const int nv = (int)net->in0.vox();
    // the context's stream carries the build; the network's stream waits for it
    if (!net->cuda(cudaStreamSynchronize(c.stream), "sync")) return false;
    cudaMemsetAsync(net->d_max, 0, 2 * sizeof(unsigned int), net->stream);
    unet::input_max_kernel<<<unet::nblk(nv, 256), 256, 0, net->stream>>>(c.setup.density[L], c.setup.skewGrid[L], nv, net->d_max);
    unet::input_write_kernel<<<unet::nblk(nv, 256), 256, 0, net->stream>>>(c.setup.density[L], c.setup.skewGrid[L], nv, net->d_max, dst);
    return net->cuda(cudaGetLastError(), "network input");
}

}  // namespace epr

extern "C" {

int epr_unet_input(epr_unet *net, epr_ctx *ctx, void *dev_input)
{
    if (!net || !ctx) return EPR_ERR_ARG;
    cudaSetDevice(net->device);
    bool ok = epr::unet_input(net, *ctx, dev_input ? (bf16 *)dev_input : net->in0.p) &&
              net->cuda(cudaStreamSynchronize(net->stream), "sync");
    return ok ? EPR_OK : (net->err.empty() ? EPR_ERR_CUDA : EPR_ERR_ARG);
}

int epr_unet_target(epr_unet *net, epr_ctx *ctx, float *dev_target)
{
    if (!net || !ctx || !dev_target) return EPR_ERR_ARG;
    cudaSetDevice(net->device);
    const int L = net->level;
    if (ctx->depth < L || ctx->dim != 3) return net->fail("bad context"), EPR_ERR_ARG;
    // the level's regular double coefficients (a float or double-float level converted first)
    if (!ctx->pull_xy(L) || !net->cuda(cudaStreamSynchronize(ctx->stream), "sync")) return EPR_ERR_CUDA;
    const int nv = (int)net->in0.vox();
    epr::unet::xy_to_target_kernel<<<epr::unet::nblk(nv, 256), 256, 0, net->stream>>>(ctx->levels[L].xy64, nv, dev_target);
    bool ok = net->cuda(cudaGetLastError(), "target") && net->cuda(cudaStreamSynchronize(net->stream), "sync");
    return ok ? EPR_OK : EPR_ERR_CUDA;
}

int epr_unet_warm_start(epr_unet *net, epr_ctx *ctx, double *info)
{
    if (!net || !ctx) return EPR_ERR_ARG;
    cudaSetDevice(net->device);
    const int L = net->level;
    if (!epr::unet_input(net, *ctx, net->in0.p) || !forward(net, net->in0) || !check_flag(net))
        return net->err.empty() ? EPR_ERR_CUDA : EPR_ERR_ARG;
    // the prediction at unit scale as the level's coefficients, its energy terms, then the scale
    // that minimises E(s p) = s^4 W + s^2 (reg - 2 y^T B x) + c.  The reflection (x, -y) of the
    // prediction has the same W and reg and the opposite cross term (its wedge is the negated
    // one), so the same evaluation gives its quartic too: the orientation with the lower minimum
    // is taken.
    const int nv = (int)net->in0.vox();
    epr::unet::pred_to_xy_kernel<<<epr::unet::nblk(nv, 256), 256, 0, net->stream>>>(net->pred, nv, 1.0, 1.0, ctx->levels[L].xy64);
    if (!net->cuda(cudaGetLastError(), "prediction") || !net->cuda(cudaStreamSynchronize(net->stream), "sync")) return EPR_ERR_CUDA;
    double e[3];
    if (!ctx->push_xy(L) || !ctx->energy(L, e)) return ctx->status ? ctx->status : EPR_ERR_CUDA;
    const double cross = e[0] - e[2] - ctx->c;  // -2 y^T B x
    const bool reflect = cross > 0;
    const double W = e[2], a2 = e[1] + (reflect ? -cross : cross);
    double s = 0, epred = ctx->c;
    if (W > 0 && a2 < 0)
    {
        s = std::sqrt(-a2 / (2 * W));
        epred = ctx->c - a2 * a2 / (4 * W);
    }
    // the plain start the solve would otherwise use at this level (the reference's random start)
    double eplain = 0;
    if (!ctx->random_start(L, &eplain)) return ctx->status ? ctx->status : EPR_ERR_CUDA;
    const bool use = s > 0 && epred < eplain && epred < ctx->c;
    if (use)
    {
        epr::unet::pred_to_xy_kernel<<<epr::unet::nblk(nv, 256), 256, 0, net->stream>>>(net->pred, nv, s, reflect ? -s : s, ctx->levels[L].xy64);
        if (!net->cuda(cudaGetLastError(), "prediction") || !net->cuda(cudaStreamSynchronize(net->stream), "sync") || !ctx->push_xy(L))
            return EPR_ERR_CUDA;
    }
    if (info)
    {
        info[0] = use ? (reflect ? 2 : 1) : 0;
        info[1] = epred;
        info[2] = eplain;
        info[3] = s;
    }
    return cudaStreamSynchronize(ctx->stream) == cudaSuccess ? EPR_OK : EPR_ERR_CUDA;
}

}  // extern "C"
