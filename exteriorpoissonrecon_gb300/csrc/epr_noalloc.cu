// Energy evaluation that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need an energy value: code
// running inside a CUDA stream capture that must not add allocation nodes, hosts whose device
// memory is owned by a pool or arena that forbids cudaMalloc from third-party libraries, and
// real-time loops where an allocation (and the implicit synchronisation cudaMalloc/cudaFree may
// cause) is not allowed.  epr_energy_noalloc serves them: the caller passes the coefficients, the
// two stencils and a 3-double output in its own device memory, and the block partial sums of the
// deterministic two-pass reduction live in the fixed array below instead of a cudaMalloc'ed
// buffer.
//
// The array is a file-scope __device__ variable, so every GPU that loads this library holds its
// 128 KiB + 32 B until the process exits.  All calls share it: two calls whose kernels overlap on
// the GPU (different streams, or different host threads on the same device) race on it and give
// undefined results, so callers serialise them (one stream, or their own ordering).  Each call
// overwrites every slot it later reads, so nothing has to be cleared between calls.
#include <cstdio>
#include <mutex>

#include "../../include/epr.h"
#include "epr_common.cuh"
#include "epr_kernels.h"

namespace epr {
namespace {

// block partials (4 per block, kMaxBlocks blocks) followed by the 4 raw sums of the final pass;
// the energy reduction never uses more than kMaxBlocks blocks whatever the level's size, so this
// array serves every level the library accepts (0..10 in 3D, 0..7 in 4D)
constexpr int kScratchDoubles = 4 * Reduce::kMaxBlocks + 4;
static __device__ __align__(256) double g_energy_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double *g_scratch_ptr[kMaxDevices] = {};

// fit = W - 2 y^T B x + c, reg = x^T A x + y^T A y, wedge = W
__global__ void energy_combine_kernel(const double *raw, double c, double *out3)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
    {
        out3[0] = raw[0] - 2. * raw[1] + c;
        out3[1] = raw[2];
        out3[2] = raw[0];
    }
}

// Host address of this device's copy of g_energy_scratch, looked up once per device (with that
// device current) and cached.  Returns nullptr and fills err on failure.
double *scratch_for_device(int device, const char **err)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_scratch_ptr[device]) return g_scratch_ptr[device];
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_energy_scratch);
    if (e != cudaSuccess)
    {
        *err = cudaGetErrorString(e);
        cudaGetLastError();
        return nullptr;
    }
    g_scratch_ptr[device] = (double *)p;
    return (double *)p;
}

thread_local char g_noalloc_error[256];

// Makes `device` current for the lifetime of the guard and puts the caller's current device back
// afterwards, so that a host passing another device than its current one keeps its own setting.
class DeviceGuard
{
  public:
    DeviceGuard() = default;
    bool select(int device)
    {
        if (cudaGetDevice(&saved_) != cudaSuccess) { cudaGetLastError(); return false; }
        if (saved_ == device) return true;
        if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return false; }
        restore_ = true;
        return true;
    }
    ~DeviceGuard()
    {
        if (restore_) cudaSetDevice(saved_);
    }

  private:
    int saved_ = 0;
    bool restore_ = false;
};

}  // namespace
}  // namespace epr

extern "C" const char *epr_noalloc_last_error(void) { return epr::g_noalloc_error; }

extern "C" int epr_energy_noalloc(int device, int dim, int level, int precision, const void *xy, const void *A,
                                  const void *B, double c, double *out3, void *stream)
{
    using namespace epr;
    auto fail = [](int code, const char *msg) {
        snprintf(g_noalloc_error, sizeof(g_noalloc_error), "%s", msg);
        return code;
    };
    g_noalloc_error[0] = 0;
    if (dim != 3 && dim != 4) return fail(EPR_ERR_ARG, "dim must be 3 or 4");
    const int maxLevel = dim == 3 ? 10 : 7;
    if (level < 0 || level > maxLevel) return fail(EPR_ERR_ARG, "level out of range (0..10 in 3D, 0..7 in 4D)");
    if (precision != EPR_FP64 && precision != EPR_FP32) return fail(EPR_ERR_ARG, "unknown precision");
    if (!xy || !A || !B || !out3) return fail(EPR_ERR_ARG, "null device pointer");
    if (device < 0 || device >= kMaxDevices) return fail(EPR_ERR_ARG, "device ordinal out of range");
    static_assert(kScratchDoubles >= 4 * Reduce::kMaxBlocks + 4, "the reduction's block partials must fit");
    int64_t N = 1;
    for (int d = 0; d < dim; d++) N *= (int64_t)((1 << level) + 1);
    DeviceGuard guard;
    if (!guard.select(device)) return fail(EPR_ERR_CUDA, "cannot select the CUDA device");
    const char *err = nullptr;
    double *scratch = scratch_for_device(device, &err);
    if (!scratch) return fail(EPR_ERR_CUDA, err ? err : "cudaGetSymbolAddress failed");
    Reduce red;
    red.partial = scratch;
    red.out = scratch + 4 * Reduce::kMaxBlocks;
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == EPR_FP64)
    {
        LevelPtrs<double> L;
        L.level = level;
        L.N = N;
        L.A = (const double *)A;
        L.B = (const double *)B;
        if (dim == 3) launch_energy<3, double>(L, (const double *)xy, red, s);
        else launch_energy<4, double>(L, (const double *)xy, red, s);
    }
    else
    {
        LevelPtrs<float> L;
        L.level = level;
        L.N = N;
        L.A = (const float *)A;
        L.B = (const float *)B;
        if (dim == 3) launch_energy<3, float>(L, (const float *)xy, red, s);
        else launch_energy<4, float>(L, (const float *)xy, red, s);
    }
    energy_combine_kernel<<<1, 32, 0, s>>>(red.out, c, out3);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(EPR_ERR_CUDA, cudaGetErrorString(e));
    return EPR_OK;
}
