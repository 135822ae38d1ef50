// esp_energy_noalloc: the direct energy of every replica computed from
// caller-owned device arrays, allocating nothing.
//
// Who needs it: hosts that own all device memory themselves and cannot let a
// library call cudaMalloc -- a Fortran program whose arrays live in its own
// device data regions, a framework that hands out memory from its own caching
// allocator, or code that must not change the device's memory footprint in the
// middle of a run.  Such a caller passes its device pointers (the reference's
// ELL tables and spin_matrix(3,N,R)) and receives the energies in a device
// buffer it also owns.
//
// The per-block partial sums that esp_energy keeps in a per-handle device
// allocation live here in a file-scope device array of fixed size instead.
// Limits that follow from it: num_replicas <= ESP_NOALLOC_MAX_REPLICAS (4096)
// and num_sites * num_replicas < 2^31; larger requests are rejected with
// ESP_EINVAL.  Every GPU that loads the library holds the 1 MiB array until
// the process exits.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/espins_gpu.h"
#include "esp_errors.h"

namespace {

constexpr int kScratchDoubles = 131072;  // 1 MiB of partial sums
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

// Shared by every call on a device; each call writes every slot it later
// reads (one partial per (replica, block)), so nothing has to be cleared
// between calls.  Two calls that overlap on the GPU race on it.
static __device__ __align__(256) double g_energy_scratch[kScratchDoubles];

struct DeviceSetup {
    bool ready = false;
    double *scratch = nullptr;  // device address of g_energy_scratch
    int num_sms = 0;
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

// Per-site energy e_i = 1/2 sum_k pair_ik + Delta (s.a)^2 + f.s (the terms of
// energy_get, get_quant.F90:186-261) in FP32 from FP64 inputs, summed in FP64
// over the sites of one replica; blockIdx.y is the replica.
template <bool HB, bool HD>
__global__ void __launch_bounds__(kThreads) k_energy_noalloc_part(esp_energy_args a, double *scratch)
{
    __shared__ double s_acc[kThreads];
    const int N = a.num_sites, r = blockIdx.y;
    const double *s = a.spins + (size_t)3 * N * r;
    double e = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const size_t si = (size_t)3 * i;
        const float ox = (float)s[si], oy = (float)s[si + 1], oz = (float)s[si + 2];
        float pair = 0.f;
        for (int k = 0; k < a.j_nn[i]; ++k) {
            const size_t el = (size_t)k * N + i;
            const size_t sj = (size_t)3 * (a.j_nbors[el] - 1);
            const float d = ox * (float)s[sj] + oy * (float)s[sj + 1] + oz * (float)s[sj + 2];
            pair -= (float)a.j_val[el] * d;
        }
        if (HB)
            for (int k = 0; k < a.b_nn[i]; ++k) {
                const size_t el = (size_t)k * N + i;
                const size_t sj = (size_t)3 * (a.b_nbors[el] - 1);
                const float d = ox * (float)s[sj] + oy * (float)s[sj + 1] + oz * (float)s[sj + 2];
                pair += (float)a.b_val[el] * d * d;
            }
        if (HD)
            for (int k = 0; k < a.d_nn[i]; ++k) {
                const size_t el = (size_t)k * N + i;
                const size_t sj = (size_t)3 * (a.d_nbors[el] - 1);
                const float tx = (float)s[sj], ty = (float)s[sj + 1], tz = (float)s[sj + 2];
                const float cx = oy * tz - oz * ty, cy = oz * tx - ox * tz, cz = ox * ty - oy * tx;
                pair += (float)a.d_val[3 * el] * cx + (float)a.d_val[3 * el + 1] * cy + (float)a.d_val[3 * el + 2] * cz;
            }
        float site = 0.5f * pair;
        const int at = i % a.num_atoms;
        if (a.si_axis) {
            const float sa = ox * (float)a.si_axis[3 * at] + oy * (float)a.si_axis[3 * at + 1] + oz * (float)a.si_axis[3 * at + 2];
            site += (float)a.si_delta[at] * sa * sa;
        }
        if (a.field_axis) {
            const float fa = ox * (float)a.field_axis[3 * at] + oy * (float)a.field_axis[3 * at + 1] + oz * (float)a.field_axis[3 * at + 2];
            site += (float)a.field_val[at] * fa;
        }
        e += (double)site;
    }
    s_acc[threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s_acc[threadIdx.x] += s_acc[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) scratch[(size_t)r * gridDim.x + blockIdx.x] = s_acc[0];
}

// out[r] = sum of the replica's block partials, in block order.
__global__ void k_energy_noalloc_reduce(const double *scratch, int nblocks, int R, double *out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double acc = 0.0;
    for (int b = 0; b < nblocks; ++b) acc += scratch[(size_t)r * nblocks + b];
    out[r] = acc;
}

int setup_device(int dev, DeviceSetup *&out)
{
    if (dev < 0 || dev >= kMaxDevices) return ESP_EINVAL;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup &d = g_setup[dev];
    if (!d.ready) {
        // host code cannot use g_energy_scratch's name as a device address:
        // ask the runtime for it, on this device, once
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_energy_scratch) != cudaSuccess) return ESP_ECUDA;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ESP_ECUDA;
        d.scratch = static_cast<double *>(p);
        d.num_sms = sms;
        d.ready = true;
    }
    out = &d;
    return ESP_OK;
}

}  // namespace

extern "C" int esp_energy_noalloc(const esp_energy_args *a, double *energy_out, void *stream)
{
    using esp::set_global_error;
    if (!a || !energy_out || !a->spins || !a->j_nn || !a->j_nbors || !a->j_val) {
        set_global_error("esp_energy_noalloc: null argument (args, energy_out, spins and jij tables are required)");
        return ESP_EINVAL;
    }
    const int N = a->num_sites, R = a->num_replicas;
    if (N <= 0 || R <= 0 || a->num_atoms <= 0 || N % a->num_atoms != 0) {
        set_global_error("esp_energy_noalloc: bad sizes (num_sites %d, num_atoms %d, num_replicas %d)", N,
                         a->num_atoms, R);
        return ESP_EINVAL;
    }
    if (R > ESP_NOALLOC_MAX_REPLICAS) {
        set_global_error("esp_energy_noalloc: num_replicas %d exceeds the maximum %d of its static scratch", R,
                         ESP_NOALLOC_MAX_REPLICAS);
        return ESP_EINVAL;
    }
    if ((long long)N * R >= (1LL << 31)) {
        set_global_error("esp_energy_noalloc: num_sites * num_replicas must be below 2^31");
        return ESP_EINVAL;
    }
    const bool hb = a->b_nn != nullptr, hd = a->d_nn != nullptr;
    if ((a->si_axis == nullptr) != (a->si_delta == nullptr) || (a->field_axis == nullptr) != (a->field_val == nullptr) ||
        (hb && (!a->b_nbors || !a->b_val)) || (hd && (!a->d_nbors || !a->d_val))) {
        set_global_error("esp_energy_noalloc: incomplete optional tables");
        return ESP_EINVAL;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        set_global_error("esp_energy_noalloc: no current CUDA device");
        return ESP_ECUDA;
    }
    DeviceSetup *d = nullptr;
    int rc = setup_device(dev, d);
    if (rc != ESP_OK) {
        set_global_error("esp_energy_noalloc: set-up on device %d failed", dev);
        return rc;
    }
    // blocks per replica: enough to fill the GPU, within the scratch
    int gx = (N + kThreads - 1) / kThreads;
    int want = (4 * d->num_sms + R - 1) / R;  // about four blocks per SM in all
    if (want < 1) want = 1;
    if (gx > want) gx = want;
    if (gx > kScratchDoubles / R) gx = kScratchDoubles / R;
    if (gx < 1) {
        set_global_error("esp_energy_noalloc: num_replicas too large for the static scratch");
        return ESP_EINVAL;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const dim3 grid(gx, R);
    if (hb && hd) k_energy_noalloc_part<true, true><<<grid, kThreads, 0, st>>>(*a, d->scratch);
    else if (hb) k_energy_noalloc_part<true, false><<<grid, kThreads, 0, st>>>(*a, d->scratch);
    else if (hd) k_energy_noalloc_part<false, true><<<grid, kThreads, 0, st>>>(*a, d->scratch);
    else k_energy_noalloc_part<false, false><<<grid, kThreads, 0, st>>>(*a, d->scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_global_error("esp_energy_noalloc: launch failed: %s", cudaGetErrorString(e));
        return ESP_ECUDA;
    }
    k_energy_noalloc_reduce<<<(R + 127) / 128, 128, 0, st>>>(d->scratch, gx, R, energy_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_global_error("esp_energy_noalloc: launch failed: %s", cudaGetErrorString(e));
        return ESP_ECUDA;
    }
    return ESP_OK;
}
