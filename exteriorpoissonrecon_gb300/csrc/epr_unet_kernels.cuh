// Kernels of the learned warm start's network: 3x3x3 convolutions on node grids as implicit GEMMs
// on the fifth-generation tensor cores (BF16 operands staged in shared memory, FP32 accumulators
// in tensor memory), the grid transfers between network levels, and the elementwise pieces of
// training.  Activations are channels-last BF16: value (voxel v, channel c) at [v * ld + c], with
// ld and every channel offset a multiple of 8 (16-byte rows).  Voxels of an n^3 node grid are
// numbered with axis 0 slowest, as the solver's nodes.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

#include "epr_tc.cuh"

namespace epr {
namespace unet {

using bf16 = __nv_bfloat16;

constexpr int kBM = 128;  // voxels (output rows) per CTA = tensor-memory lanes
constexpr int kBK = 64;   // GEMM depth per pipeline stage (four MMAs of K = 16)
constexpr int kKC = kBK / 8;  // core matrices along K per stage
constexpr int kThreads = 128;

struct ConvArgs
{
    const bf16 *in;   // input activations (voxel rows of ldi, Cin channels from column 0)
    int ldi, Cin;     // Cin a multiple of 16
    const bf16 *W;    // GEMM B operand: [N][K] K-major, K = 27 Cin, k = tap * Cin + ci
    int K;
    const float *bias;  // N values or null
    bf16 *out;          // output rows of ldo (null: no BF16 output)
    int ldo, nout;      // the first nout (multiple of 8) of the N columns are stored
    float *outf;        // optional FP32 output rows of ldf, first nf columns
    int ldf, nf;
    const bf16 *mask;   // optional: the result is multiplied by (mask[v][c] > 0): ReLU backward
    int ldm;
    int relu;  // max(0, .) after the bias
    int flip;  // data gradient: neighbour v - off(tap) instead of v + off(tap)
    int n, nvox;
    unsigned int *err;
};

__device__ __forceinline__ void vox_coords(int v, int n, int &z, int &y, int &x)
{
    z = v / (n * n);
    const int r = v - z * n * n;
    y = r / n;
    x = r - y * n;
}

// neighbour of (z, y, x) through tap t (offsets (t / 9 - 1, t / 3 % 3 - 1, t % 3 - 1), negated when
// flip), or -1 outside the grid
__device__ __forceinline__ int tap_neighbour(int z, int y, int x, int t, int n, int flip)
{
    int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
    if (flip) { dz = -dz; dy = -dy; dx = -dx; }
    z += dz; y += dy; x += dx;
    if ((unsigned)z >= (unsigned)n || (unsigned)y >= (unsigned)n || (unsigned)x >= (unsigned)n) return -1;
    return (z * n + y) * n + x;
}

// out = act(in (*) W + bias): implicit GEMM with M = voxels (128 per CTA), N output channels,
// K = 27 Cin.  Each thread gathers one voxel row of the A tile (the 27-point neighbourhood, 16-byte
// asynchronous copies, zero where the neighbour is outside the grid) and a share of the B tile;
// thread 0 issues the MMAs of a stage and commits them to the stage's mbarrier, which the threads
// wait on before they overwrite the stage two steps later.  Epilogue: each warp reads its 32
// accumulator lanes from tensor memory.
template <int N>
__global__ void __launch_bounds__(kThreads) conv3_kernel(ConvArgs a)
{
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "MMA N");
    constexpr int kTmemCols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    constexpr uint32_t kABytes = kBM * kBK * 2, kBBytes = N * kBK * 2;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *As[2] = {smem, smem + kABytes};
    unsigned char *Bs[2] = {smem + 2 * kABytes, smem + 2 * kABytes + kBBytes};
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmem_base;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kBM;
    if (warp == 0) tc::tmem_alloc(&tmem_base, kTmemCols);
    if (tid == 0)
    {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;

    // this thread's A row
    const int v = m0 + tid;
    int z = 0, y = 0, x = 0;
    const bool rowOk = v < a.nvox;
    if (rowOk) vox_coords(v, a.n, z, y, x);
    const int nstages = (a.K + kBK - 1) / kBK;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, N);
    bool ok = true;
    for (int s = 0; s < nstages; s++)
    {
        const int buf = s & 1;
        if (s >= 2) ok = tc::mbar_wait(&bar[buf], ((s >> 1) - 1) & 1, a.err) && ok;
        const int k0 = s * kBK;
        // A: 8 core-matrix columns of this thread's row
#pragma unroll
        for (int kc = 0; kc < kKC; kc++)
        {
            const int k = k0 + 8 * kc;
            const bf16 *src = a.in;
            uint32_t bytes = 0;
            if (rowOk && k < a.K)
            {
                const int t = k / a.Cin, ci = k - t * a.Cin;
                const int nb = tap_neighbour(z, y, x, t, a.n, a.flip);
                if (nb >= 0)
                {
                    src = a.in + (int64_t)nb * a.ldi + ci;
                    bytes = 16;
                }
            }
            tc::cp_async16(As[buf] + tc::core_offset(tid, kc, kKC), src, bytes);
        }
        // B: N rows x 8 core-matrix columns
        for (int c = tid; c < N * kKC; c += kThreads)
        {
            const int row = c / kKC, kc = c - row * kKC;
            const int k = k0 + 8 * kc;
            const bf16 *src = a.W;
            uint32_t bytes = 0;
            if (k < a.K)
            {
                src = a.W + (int64_t)row * a.K + k;
                bytes = 16;
            }
            tc::cp_async16(Bs[buf] + tc::core_offset(row, kc, kKC), src, bytes);
        }
        tc::cp_async_commit();
        tc::cp_async_wait_all();
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0)
        {
            tc::tc_fence_after();
            const int kmmas = min(4, (a.K - k0) / 16);
            const uint32_t sa = tc::smem_addr(As[buf]), sb = tc::smem_addr(Bs[buf]);
            for (int g = 0; g < kmmas; g++)
            {
                const uint64_t ad = tc::smem_desc(sa + 256 * g, 128, 128 * kKC);
                const uint64_t bd = tc::smem_desc(sb + 256 * g, 128, 128 * kKC);
                tc::mma_bf16(tmem, ad, bd, idesc, (s > 0 || g > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bar[buf]);
        }
    }
    // the last commit covers every MMA issued before it
    {
        const int last = nstages - 1;
        ok = tc::mbar_wait(&bar[last & 1], (last >> 1) & 1, a.err) && ok;
    }
    tc::tc_fence_after();
    // epilogue: row = voxel m0 + 32 warp + lane
    const int vr = m0 + 32 * warp + lane;
    const bool vOk = vr < a.nvox && ok;
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16)
    {
        float acc[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, acc);
        if (!vOk) continue;
#pragma unroll
        for (int j = 0; j < 16; j++)
        {
            float val = acc[j] + (a.bias ? a.bias[c0 + j] : 0.f);
            if (a.relu) val = fmaxf(val, 0.f);
            acc[j] = val;
        }
        if (a.mask)
        {
            const bf16 *mrow = a.mask + (int64_t)vr * a.ldm + c0;
#pragma unroll
            for (int j = 0; j < 16; j++)
                if (c0 + j < a.nout && !(__bfloat162float(mrow[j]) > 0.f)) acc[j] = 0.f;
        }
        if (a.out && c0 < a.nout)
        {
            __align__(16) bf16 o[16];
#pragma unroll
            for (int j = 0; j < 16; j++) o[j] = __float2bfloat16(acc[j]);
            uint4 *dst = reinterpret_cast<uint4 *>(a.out + (int64_t)vr * a.ldo + c0);
            dst[0] = reinterpret_cast<const uint4 *>(o)[0];
            if (c0 + 8 < a.nout) dst[1] = reinterpret_cast<const uint4 *>(o)[1];
        }
        if (a.outf)
            for (int j = 0; j < 16; j++)
                if (c0 + j < a.nf) a.outf[(int64_t)vr * a.ldf + c0 + j] = acc[j];
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

struct WgradArgs
{
    const bf16 *in;  // forward input of the layer
    int ldi, Cin;
    const bf16 *dz;  // gradient of the layer's pre-activation output
    int ldz;
    float *partial;  // [gridDim.y][27 Cin][N] FP32 partial sums of this CTA's voxel range
    int M;           // 27 Cin
    int n, nvox, vox_per_split;
    unsigned int *err;
};

// dW[(tap, ci)][co] = sum_v in[v + off(tap)][ci] dz[v][co]: GEMM with M = 27 Cin rows (128 per
// CTA), N output channels and K = voxels, split over gridDim.y voxel ranges.  Both operands are
// gathered as 8 x 8 blocks (eight voxels x eight channels, 16-byte loads) and transposed in
// registers into K-major core matrices.
template <int N>
__global__ void __launch_bounds__(kThreads) conv3_wgrad_kernel(WgradArgs a)
{
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "MMA N");
    constexpr int kTmemCols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    constexpr uint32_t kABytes = kBM * kBK * 2, kBBytes = N * kBK * 2;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *As[2] = {smem, smem + kABytes};
    unsigned char *Bs[2] = {smem + 2 * kABytes, smem + 2 * kABytes + kBBytes};
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmem_base;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kBM;
    const int vbeg = blockIdx.y * a.vox_per_split;
    const int vend = min(a.nvox, vbeg + a.vox_per_split);
    if (warp == 0) tc::tmem_alloc(&tmem_base, kTmemCols);
    if (tid == 0)
    {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, N);

    // this thread's A core matrix: row group rg (8 rows = one tap, 8 channels), voxel group kc
    const int rg = tid >> 3, kcA = tid & 7;
    const int mA = m0 + 8 * rg;
    const int tapA = mA < a.M ? mA / a.Cin : 0, ciA = mA < a.M ? mA - tapA * a.Cin : 0;
    const int nstages = vend > vbeg ? (vend - vbeg + kBK - 1) / kBK : 0;
    bool ok = true;
    for (int s = 0; s < nstages; s++)
    {
        const int buf = s & 1;
        if (s >= 2) ok = tc::mbar_wait(&bar[buf], ((s >> 1) - 1) & 1, a.err) && ok;
        const int v0 = vbeg + s * kBK;
        {
            uint4 blk[8], tr[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
            {
                const int vv = v0 + 8 * kcA + j;
                blk[j] = make_uint4(0, 0, 0, 0);
                if (mA < a.M && vv < vend)
                {
                    int zz, yy, xx;
                    vox_coords(vv, a.n, zz, yy, xx);
                    const int nb = tap_neighbour(zz, yy, xx, tapA, a.n, 0);
                    if (nb >= 0) blk[j] = *reinterpret_cast<const uint4 *>(a.in + (int64_t)nb * a.ldi + ciA);
                }
            }
            tc::transpose8x8_b16(blk, tr);
#pragma unroll
            for (int r = 0; r < 8; r++)
                *reinterpret_cast<uint4 *>(As[buf] + tc::core_offset(8 * rg + r, kcA, kKC)) = tr[r];
        }
        for (int c = tid; c < (N / 8) * kKC; c += kThreads)
        {
            const int ng = c / kKC, kc = c - ng * kKC;
            uint4 blk[8], tr[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
            {
                const int vv = v0 + 8 * kc + j;
                blk[j] = vv < vend ? *reinterpret_cast<const uint4 *>(a.dz + (int64_t)vv * a.ldz + 8 * ng)
                                   : make_uint4(0, 0, 0, 0);
            }
            tc::transpose8x8_b16(blk, tr);
#pragma unroll
            for (int r = 0; r < 8; r++)
                *reinterpret_cast<uint4 *>(Bs[buf] + tc::core_offset(8 * ng + r, kc, kKC)) = tr[r];
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0)
        {
            tc::tc_fence_after();
            const uint32_t sa = tc::smem_addr(As[buf]), sb = tc::smem_addr(Bs[buf]);
#pragma unroll
            for (int g = 0; g < 4; g++)
            {
                const uint64_t ad = tc::smem_desc(sa + 256 * g, 128, 128 * kKC);
                const uint64_t bd = tc::smem_desc(sb + 256 * g, 128, 128 * kKC);
                tc::mma_bf16(tmem, ad, bd, idesc, (s > 0 || g > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bar[buf]);
        }
    }
    if (nstages > 0)
    {
        const int last = nstages - 1;
        ok = tc::mbar_wait(&bar[last & 1], (last >> 1) & 1, a.err) && ok;
    }
    tc::tc_fence_after();
    const int m = m0 + 32 * warp + lane;
    float *dst = a.partial + ((int64_t)blockIdx.y * a.M + m) * N;
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16)
    {
        float acc[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, acc);
        if (m < a.M)
#pragma unroll
            for (int j = 0; j < 16; j++) dst[c0 + j] = (nstages > 0 && ok) ? acc[j] : 0.f;
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

}  // namespace unet
}  // namespace epr
