// energy_noalloc.cu -- CalcFastEnergy over caller-owned device fields with no device allocation.
//
// Who this is for: callers whose device memory is owned by someone else and who therefore must
// not call cudaMalloc themselves. Examples are a host framework that hands out all device
// memory from its own caching pool or arena (a raw cudaMalloc would bypass its accounting and
// can fail once the pool has reserved the card), and deployments that forbid runtime allocation
// after start-up.  The call reads the result back and synchronizes the caller's stream.
// Such a caller already holds the voltage and current fields in device memory; this entry point
// reduces them with scratch that is part of the library image instead of allocated memory.
//
// Scratch: one file-scope __device__ array (below), sized for OEMS_NOALLOC_MAX_PLANES x-planes.
// Every GPU that loads this library holds it (128 KB) until the process exits.  The host code
// never uses the array's name as a pointer: it resolves the device address with
// cudaGetSymbolAddress once per device (first call on that device, with that device current)
// and passes that address to the kernels.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/oems_cuda.h"

namespace {

constexpr unsigned kMaxPlanes = OEMS_NOALLOC_MAX_PLANES;
constexpr unsigned kSlots = 2 * kMaxPlanes + 2;   // per-plane (E, H) partials + the final pair

// The scratch shared by every call on a device (contents persist between calls).
static __device__ __align__(256) double g_energy_scratch[kSlots];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// One block per x-plane x < Nx-1: sum of V^2 and I^2 over y < Ny-1, z < Nz-1 (float squares
// accumulated in double, as Engine_Interface_FDTD::CalcFastEnergy does). Every slot that the
// final kernel reads is written here first, so nothing has to start at zero.
__global__ void __launch_bounds__(256) k_plane_energy(const float* __restrict__ V, const float* __restrict__ I,
                                                       unsigned Nx, unsigned Ny, unsigned Nz, unsigned Pz,
                                                       double* __restrict__ scratch)
{
    const unsigned x = blockIdx.x;
    const unsigned long long S = (unsigned long long)Nx * Ny * Pz;
    const unsigned long long base = (unsigned long long)x * Ny * Pz;
    const unsigned plane = (Ny - 1) * (Nz - 1);
    double e = 0.0, h = 0.0;
    for (unsigned t = threadIdx.x; t < plane; t += blockDim.x) {
        const unsigned y = t / (Nz - 1), z = t - y * (Nz - 1);
        const unsigned long long o = base + (unsigned long long)y * Pz + z;
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const float v = V[n * S + o], c = I[n * S + o];
            e += (double)__fmul_rn(v, v);
            h += (double)__fmul_rn(c, c);
        }
    }
    __shared__ double se[256], sh[256];
    se[threadIdx.x] = e;
    sh[threadIdx.x] = h;
    __syncthreads();
    for (unsigned w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            se[threadIdx.x] += se[threadIdx.x + w];
            sh[threadIdx.x] += sh[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scratch[2 * x] = se[0];
        scratch[2 * x + 1] = sh[0];
    }
}

// planes summed in x order by one thread: the result does not depend on block scheduling
__global__ void k_sum_planes(unsigned planes, double* __restrict__ scratch)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double e = 0.0, h = 0.0;
    for (unsigned x = 0; x < planes; ++x) {
        e += scratch[2 * x];
        h += scratch[2 * x + 1];
    }
    scratch[2 * kMaxPlanes] = e;
    scratch[2 * kMaxPlanes + 1] = h;
}

// Resolve (once per device) the device address of the scratch array.
int scratch_address(int device, double** out)
{
    if (device < 0 || device >= kMaxDevices) return OEMS_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t c = cudaGetSymbolAddress(&p, g_energy_scratch);
        if (c != cudaSuccess || !p) {
            cudaGetLastError();
            return OEMS_ERR_CUDA;
        }
        g_scratch_addr[device] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[device];
    return OEMS_OK;
}

}  // namespace

extern "C" int oems_cuda_energy_noalloc(const float* volt_dev, const float* curr_dev, const unsigned int num_lines[3],
                                        unsigned int z_stride, void* stream, double* energy)
{
    if (!volt_dev || !curr_dev || !num_lines || !energy) return OEMS_ERR_ARG;
    const unsigned Nx = num_lines[0], Ny = num_lines[1], Nz = num_lines[2];
    if (Nx < 2 || Ny < 2 || Nz < 2 || z_stride < Nz) return OEMS_ERR_ARG;
    if (Nx - 1 > kMaxPlanes) return OEMS_ERR_TOO_LARGE;   // more x-planes than the scratch holds
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) { cudaGetLastError(); return OEMS_ERR_CUDA; }
    double* scratch = nullptr;
    int rc = scratch_address(device, &scratch);
    if (rc != OEMS_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_plane_energy<<<Nx - 1, 256, 0, s>>>(volt_dev, curr_dev, Nx, Ny, Nz, z_stride, scratch);
    cudaError_t c = cudaGetLastError();
    if (c != cudaSuccess) return OEMS_ERR_CUDA;   // nothing launched: do not read stale scratch
    k_sum_planes<<<1, 32, 0, s>>>(Nx - 1, scratch);
    c = cudaGetLastError();
    if (c != cudaSuccess) return OEMS_ERR_CUDA;
    double eh[2] = {0.0, 0.0};
    c = cudaMemcpyAsync(eh, scratch + 2 * kMaxPlanes, sizeof(eh), cudaMemcpyDeviceToHost, s);
    if (c == cudaSuccess) c = cudaStreamSynchronize(s);
    if (c != cudaSuccess) { cudaGetLastError(); return OEMS_ERR_CUDA; }
    *energy = 8.85418781762e-12 * eh[0] + 1.256637062e-6 * eh[1];
    return OEMS_OK;
}
