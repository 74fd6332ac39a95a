// Synthetic point + frame samples generated on the device: the curves and surfaces of the
// reference's Sample tool (Include/Samples.h: torus knot, link of two circles, helix, Clifford torus)
// with its kinds of noise (Sample/Sample.cpp:137-199: Gaussian positional noise in unit-cube units,
// a random rotation of every frame, a fraction of uniform outliers with random frames), so that
// training or benchmark inputs at scale need no host round trip.  The shapes and the noise follow
// exteriorpoissonrecon_gb300/samples.py (the seeded host generator) formula for formula; the random
// numbers come from Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC 2011), a counter-based generator: sample i's numbers depend only on (seed, i), so
// the output does not depend on the launch shape.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epr.h"
#include "epr_context.h"

namespace epr {

namespace {

// Philox4x32 with 10 rounds: a counter of four 32-bit words and a key of two, multipliers and Weyl
// increments as published
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; r++)
    {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Two uniform doubles in (0, 1) (53 random bits each) from stream `s` of sample i
struct Rng
{
    uint2 key;
    uint64_t i;
    __device__ void uniforms(uint32_t s, double &u0, double &u1) const
    {
        const uint4 r = philox(make_uint4((uint32_t)i, (uint32_t)(i >> 32), s, 0x5eedu), key);
        const uint64_t a = ((uint64_t)r.x << 21) ^ (uint64_t)(r.y >> 11);
        const uint64_t b = ((uint64_t)r.z << 21) ^ (uint64_t)(r.w >> 11);
        u0 = ((double)(a & ((1ull << 53) - 1)) + 0.5) * 0x1p-53;
        u1 = ((double)(b & ((1ull << 53) - 1)) + 0.5) * 0x1p-53;
    }
    // two standard normals (Box-Muller)
    __device__ void normals(uint32_t s, double &z0, double &z1) const
    {
        double u0, u1;
        uniforms(s, u0, u1);
        const double rad = sqrt(-2.0 * log(u0)), th = 6.283185307179586476925286766559 * u1;
        z0 = rad * cos(th);
        z1 = rad * sin(th);
    }
};

// stream numbers
constexpr uint32_t kStreamShape = 0, kStreamPos = 1, kStreamRot = 3, kStreamSpot = 8;

template <int D>
__device__ __forceinline__ void pack(const double (&m)[D][D], double *out)
{
    int k = 0;
    for (int i = 1; i < D; i++)
        for (int j = 0; j < i; j++) out[k++] = 0.5 * (m[i][j] - m[j][i]);
}

// clean shape sample i (position and full frame matrix) followed by the frame rotation noise
template <int D>
__global__ void shape_kernel(epr_sampler sp, uint2 key, int64_t n, double *pos, double *skew)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rng rng{key, (uint64_t)i};
    double u0, u1;
    rng.uniforms(kStreamShape, u0, u1);
    double p[D] = {}, m[D][D] = {};
    const double tau = 6.283185307179586476925286766559;
    if constexpr (D == 3)
    {
        double T[3] = {0, 0, 0};
        if (sp.shape == EPR_SHAPE_TORUS_KNOT)
        {
            const double t = sp.regular ? (double)i * (tau / (double)n) : tau * u0;
            const double P = sp.a, Q = sp.b;
            const double r = 2.0 + cos(Q * t), dr = -Q * sin(Q * t);
            p[0] = r * cos(P * t); p[1] = r * sin(P * t); p[2] = sin(Q * t);
            T[0] = dr * cos(P * t) - r * P * sin(P * t);
            T[1] = dr * sin(P * t) + r * P * cos(P * t);
            T[2] = Q * cos(Q * t);
        }
        else if (sp.shape == EPR_SHAPE_LINK)
        {
            const double t = tau * u0, c = cos(t), s = sin(t);
            if (u1 < 0.5) { p[0] = c; p[1] = s; p[2] = 0; T[0] = -s; T[1] = c; T[2] = 0; }
            else { p[0] = 1.0 + c; p[1] = 0; p[2] = s; T[0] = -s; T[1] = 0; T[2] = c; }
        }
        else  // helix: a turns, radius b, height c along z
        {
            const double t = u0, ang = tau * sp.a * t;
            p[0] = sp.b * cos(ang); p[1] = sp.b * sin(ang); p[2] = sp.c * t;
            T[0] = -sp.b * tau * sp.a * sin(ang); T[1] = sp.b * tau * sp.a * cos(ang); T[2] = sp.c;
        }
        // Hodge dual of the unit tangent: m_ij = eps_ijk T_k
        const double nrm = sqrt(T[0] * T[0] + T[1] * T[1] + T[2] * T[2]);
        const double t0 = T[0] / nrm, t1 = T[1] / nrm, t2 = T[2] / nrm;
        m[0][1] = t2; m[1][0] = -t2; m[1][2] = t0; m[2][1] = -t0; m[2][0] = t1; m[0][2] = -t1;
    }
    else
    {
        // Clifford torus (cos u, sin u, cos v, sin v) / sqrt 2, frame d_u ^ d_v normalised
        const double u = tau * u0, v = tau * u1, k = 0.70710678118654752440084436210485;
        p[0] = k * cos(u); p[1] = k * sin(u); p[2] = k * cos(v); p[3] = k * sin(v);
        const double a[4] = {-k * sin(u), k * cos(u), 0, 0}, b[4] = {0, 0, -k * sin(v), k * cos(v)};
        double f = 0;
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) { m[r][c] = a[r] * b[c] - b[r] * a[c]; f += m[r][c] * m[r][c]; }
        f = sqrt(f);
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) m[r][c] /= f;
    }
    if (sp.angle_deg > 0)
    {
        // rotation by a normal angle in a uniformly random 2-plane (a, b): M -> R^T M R
        double z[2 * D + 2];
        for (int q = 0; q < D + 1; q++) rng.normals(kStreamRot + q, z[2 * q], z[2 * q + 1]);
        double a[D], b[D], na = 0, ab = 0, nb = 0;
        for (int d = 0; d < D; d++) { a[d] = z[d]; na += a[d] * a[d]; }
        na = sqrt(na);
        for (int d = 0; d < D; d++) { a[d] /= na; b[d] = z[D + d]; ab += b[d] * a[d]; }
        for (int d = 0; d < D; d++) { b[d] -= ab * a[d]; nb += b[d] * b[d]; }
        nb = sqrt(nb);
        for (int d = 0; d < D; d++) b[d] /= nb;
        const double th = z[2 * D] * sp.angle_deg * (3.14159265358979323846264338327950 / 180.0);
        const double c = cos(th) - 1.0, s = sin(th);
        double R[D][D], RM[D][D];
        for (int r = 0; r < D; r++)
            for (int q = 0; q < D; q++) R[r][q] = (r == q ? 1.0 : 0.0) + c * (a[r] * a[q] + b[r] * b[q]) + s * (b[r] * a[q] - a[r] * b[q]);
        for (int r = 0; r < D; r++)
            for (int q = 0; q < D; q++)
            {
                double acc = 0;
                for (int j = 0; j < D; j++) acc += R[j][r] * m[j][q];
                RM[r][q] = acc;
            }
        for (int r = 0; r < D; r++)
            for (int q = 0; q < D; q++)
            {
                double acc = 0;
                for (int j = 0; j < D; j++) acc += RM[r][j] * R[j][q];
                m[r][q] = acc;
            }
    }
    for (int d = 0; d < D; d++) pos[i * D + d] = p[d];
    pack<D>(m, skew + i * (D * (D - 1) / 2));
}

// positional noise N(0, sigma) on every coordinate of the first n samples
template <int D>
__global__ void jitter_kernel(uint2 key, int64_t n, double sigma, double *pos)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rng rng{key, (uint64_t)i};
    double z[4];
    rng.normals(kStreamPos, z[0], z[1]);
    rng.normals(kStreamPos + 1, z[2], z[3]);
    for (int d = 0; d < D; d++) pos[i * D + d] += sigma * z[d];
}

// outliers n .. n+m-1: uniform in the box [lo, hi], frame (S - S^T) of uniform S in [-1, 1]
template <int D>
__global__ void spot_kernel(uint2 key, int64_t n, int64_t m, const double *box, double *pos, double *skew)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int64_t i = n + j;
    Rng rng{key, (uint64_t)i};
    double u[2 + D * D + 2];
    for (int q = 0; q < (D + D * D + 1) / 2; q++) rng.uniforms(kStreamSpot + q, u[2 * q], u[2 * q + 1]);
    for (int d = 0; d < D; d++) pos[i * D + d] = fmin(box[D + d], box[d] + (box[D + d] - box[d]) * u[d]);  // inside the box
    double S[D][D];
    for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) S[r][c] = 2.0 * u[D + r * D + c] - 1.0;
    int k = 0;
    for (int r = 1; r < D; r++)
        for (int c = 0; c < r; c++) skew[i * (D * (D - 1) / 2) + k++] = S[r][c] - S[c][r];
}

// per-axis min and max: block partials, then one block
template <int D>
__global__ void box_partial_kernel(const double *pos, int64_t n, double *part)
{
    __shared__ double s[2 * D][256];
    double lo[D], hi[D];
    for (int d = 0; d < D; d++) { lo[d] = INFINITY; hi[d] = -INFINITY; }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < D; d++) { lo[d] = fmin(lo[d], pos[i * D + d]); hi[d] = fmax(hi[d], pos[i * D + d]); }
    for (int d = 0; d < D; d++) { s[d][threadIdx.x] = lo[d]; s[D + d][threadIdx.x] = hi[d]; }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1)
    {
        if ((int)threadIdx.x < w)
            for (int d = 0; d < D; d++)
            {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + w]);
                s[D + d][threadIdx.x] = fmax(s[D + d][threadIdx.x], s[D + d][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 2 * D) part[blockIdx.x * 2 * D + threadIdx.x] = s[threadIdx.x][0];
}

template <int D>
__global__ void box_final_kernel(const double *part, int nb, double *box)
{
    if (threadIdx.x >= 2 * D) return;
    const int d = threadIdx.x;
    double v = d < D ? INFINITY : -INFINITY;
    for (int b = 0; b < nb; b++) v = d < D ? fmin(v, part[b * 2 * D + d]) : fmax(v, part[b * 2 * D + d]);
    box[d] = v;
}

// the unit-cube map p -> p k + t with the two roundings of the host's p * k + t
__global__ void affine_kernel(double *pos, int64_t count, int D, const double *k, const double *t)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= count) return;
    const int d = (int)(q % D);
    pos[q] = __dadd_rn(__dmul_rn(pos[q], k[0]), t[d]);
}

unsigned int nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

struct Generated
{
    double *pos = nullptr, *skew = nullptr;
    int64_t total = 0;
    double box[8] = {};
};

bool check_sampler(const epr_sampler *sp, size_t n, std::string &err)
{
    if (!sp) { err = "null sampler"; return false; }
    if (n == 0) { err = "expected some samples: 0"; return false; }
    if (sp->shape < EPR_SHAPE_TORUS_KNOT || sp->shape > EPR_SHAPE_CLIFFORD) { err = "unknown shape"; return false; }
    if (!(sp->pos_sigma >= 0) || !(sp->angle_deg >= 0) || !(sp->spot_frac >= 0) || !(sp->spot_frac <= 1))
    {
        err = "noise parameters must be finite and non-negative (spot fraction at most 1)";
        return false;
    }
    if (sp->shape == EPR_SHAPE_TORUS_KNOT && !(sp->a > 0 && sp->b > 0)) { err = "torus knot needs p, q > 0"; return false; }
    if (sp->shape == EPR_SHAPE_HELIX && !(sp->a > 0 && sp->b > 0 && sp->c > 0)) { err = "helix needs turns, radius, height > 0"; return false; }
    return true;
}

int sampler_dim(const epr_sampler *sp) { return sp->shape == EPR_SHAPE_CLIFFORD ? 4 : 3; }

// generates into device memory allocated on the stream (freed by the caller); reads the box of the
// noisy samples back (it bounds the outliers and the unit-cube map)
template <int D>
cudaError_t generate(const epr_sampler &sp, int64_t n, cudaStream_t s, Generated &g)
{
    constexpr int K = D * (D - 1) / 2;
    const int64_t m = (int64_t)llround((double)n * sp.spot_frac);
    g.total = n + m;
    const uint2 key = make_uint2((uint32_t)sp.seed, (uint32_t)(sp.seed >> 32));
    cudaError_t e = cudaMallocAsync((void **)&g.pos, sizeof(double) * D * g.total, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&g.skew, sizeof(double) * K * g.total, s);
    const int nb = (int)std::min<int64_t>(nblk(n), 512);
    double *part = nullptr, *dbox = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&part, sizeof(double) * 2 * D * nb + sizeof(double) * 2 * D, s);
    if (e != cudaSuccess) return e;
    dbox = part + 2 * D * nb;
    shape_kernel<D><<<nblk(n), 256, 0, s>>>(sp, key, n, g.pos, g.skew);
    auto box = [&](double *h) {
        box_partial_kernel<D><<<nb, 256, 0, s>>>(g.pos, n, part);
        box_final_kernel<D><<<1, 32, 0, s>>>(part, nb, dbox);
        cudaError_t r = cudaMemcpyAsync(h, dbox, sizeof(double) * 2 * D, cudaMemcpyDeviceToHost, s);
        return r == cudaSuccess ? cudaStreamSynchronize(s) : r;
    };
    if (sp.pos_sigma > 0)
    {
        // sigma in unit-cube units: times the clean samples' largest extent x 1.1
        double b[2 * D];
        if ((e = box(b)) != cudaSuccess) { cudaFreeAsync(part, s); return e; }
        double ext = 0;
        for (int d = 0; d < D; d++) ext = std::max(ext, b[D + d] - b[d]);
        jitter_kernel<D><<<nblk(n), 256, 0, s>>>(key, n, sp.pos_sigma * ext * 1.1, g.pos);
    }
    if ((e = box(g.box)) != cudaSuccess) { cudaFreeAsync(part, s); return e; }
    if (m > 0) spot_kernel<D><<<nblk(m), 256, 0, s>>>(key, n, m, dbox, g.pos, g.skew);
    cudaFreeAsync(part, s);
    return cudaGetLastError();
}

}  // namespace

bool Setup::set_samples_device(Context &c, size_t n_, double *dpos, double *dskew)
{
    release(c);
    n = n_;
    pos = dpos;
    skew = dskew;
    return c.cuda_ok(cudaStreamSynchronize(c.stream), "sync");
}

}  // namespace epr

extern "C" {

int epr_generate_samples(int device, const epr_sampler *sp, size_t n, double *pos, double *skew, size_t *total)
{
    std::string err;
    if (!epr::check_sampler(sp, n, err)) { epr::set_global_error(err.c_str()); return EPR_ERR_ARG; }
    const int D = epr::sampler_dim(sp), K = D * (D - 1) / 2;
    const size_t m = (size_t)llround((double)n * sp->spot_frac);
    if (total) *total = n + m;
    if (!pos && !skew) return EPR_OK;
    if (!pos || !skew) { epr::set_global_error("null output"); return EPR_ERR_ARG; }
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); epr::set_global_error("cannot select CUDA device"); return EPR_ERR_CUDA; }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); epr::set_global_error("stream"); return EPR_ERR_CUDA; }
    epr::Generated g;
    cudaError_t e = D == 3 ? epr::generate<3>(*sp, (int64_t)n, s, g) : epr::generate<4>(*sp, (int64_t)n, s, g);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pos, g.pos, sizeof(double) * D * g.total, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(skew, g.skew, sizeof(double) * K * g.total, cudaMemcpyDeviceToHost, s);
    if (g.pos) cudaFreeAsync(g.pos, s);
    if (g.skew) cudaFreeAsync(g.skew, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess)
    {
        epr::set_global_error(cudaGetErrorString(e));
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? EPR_ERR_NOMEM : EPR_ERR_CUDA;
    }
    return EPR_OK;
}

int epr_set_generated_samples(epr_ctx *ctx_, const epr_sampler *sp, size_t n, double *xform)
{
    epr_ctx *ctx = ctx_;
    if (!ctx) { epr::set_global_error("null context"); return EPR_ERR_ARG; }
    ctx->status = EPR_OK;
    std::string err;
    if (!epr::check_sampler(sp, n, err)) { ctx->fail(EPR_ERR_ARG, "%s", err.c_str()); return EPR_ERR_ARG; }
    if (epr::sampler_dim(sp) != ctx->dim) { ctx->fail(EPR_ERR_ARG, "the shape is %dD, the context %dD", epr::sampler_dim(sp), ctx->dim); return EPR_ERR_ARG; }
    cudaSetDevice(ctx->P.device);
    const int D = ctx->dim;
    epr::Generated g;
    cudaError_t e = D == 3 ? epr::generate<3>(*sp, (int64_t)n, ctx->stream, g) : epr::generate<4>(*sp, (int64_t)n, ctx->stream, g);
    if (e != cudaSuccess)
    {
        if (g.pos) cudaFreeAsync(g.pos, ctx->stream);
        if (g.skew) cudaFreeAsync(g.skew, ctx->stream);
        ctx->cuda_ok(e, "generate samples");
        return ctx->status;
    }
    // ExteriorPoisson::ToUnitCube (ExteriorPoisson.h:100-123) on the device: centre the box, scale
    // by 1 / (largest extent x 1.1), shift by 1/2 (k and t computed as the host path computes them)
    double ext = 0;
    for (int d = 0; d < D; d++) ext = std::max(ext, g.box[D + d] - g.box[d]);
    const double k = 1.0 / (ext * 1.1);
    double kt[1 + 4];
    kt[0] = k;
    for (int d = 0; d < D; d++)
    {
        volatile double u = (-(g.box[d] + g.box[D + d]) / 2.0) * k;  // rounded before the add, as on the host
        kt[1 + d] = u + 0.5;
    }
    double *dkt = nullptr;
    bool ok = ctx->alloc((void **)&dkt, sizeof(kt), "alloc map") &&
              ctx->cuda_ok(cudaMemcpyAsync(dkt, kt, sizeof(kt), cudaMemcpyHostToDevice, ctx->stream), "upload map");
    if (ok)
    {
        epr::affine_kernel<<<epr::nblk(g.total * D), 256, 0, ctx->stream>>>(g.pos, g.total * D, D, dkt, dkt + 1);
        ok = ctx->launch_ok("unit cube");
    }
    ctx->release(dkt);
    if (ok && xform)
    {
        // (Dim+1)^2 matrix in the layout of the host's unit_cube: diagonal k, last row t
        for (int q = 0; q < (D + 1) * (D + 1); q++) xform[q] = 0;
        for (int d = 0; d < D; d++) { xform[d * (D + 1) + d] = k; xform[D * (D + 1) + d] = kt[1 + d]; }
        xform[D * (D + 1) + D] = 1.0;
    }
    if (!ok)
    {
        cudaFreeAsync(g.pos, ctx->stream);
        cudaFreeAsync(g.skew, ctx->stream);
        return ctx->status ? ctx->status : EPR_ERR_CUDA;
    }
    return ctx->setup.set_samples_device(*ctx, (size_t)g.total, g.pos, g.skew) ? EPR_OK : (ctx->status ? ctx->status : EPR_ERR_CUDA);
}

}  // extern "C"
