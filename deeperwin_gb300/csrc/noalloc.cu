// log psi^2 without any device allocation by the caller or the library.
//
// Some callers cannot allocate device memory at the point where they evaluate the
// wavefunction: a host framework that owns all device memory through its own pool and
// forbids cudaMalloc inside a plug-in call, or an embedding that runs with a fixed memory
// budget. For them dw_log_psi_sqr_noalloc takes its scratch from a file-scope static
// __device__ array instead of a caller-provided workspace. The array has a fixed size
// (kStaticScratchBytes); every GPU that loads the library reserves it until the process exits.
#include "net.cuh"

#include <mutex>

namespace {

constexpr size_t kStaticScratchBytes = (size_t)64 << 20;   // 64 MiB
constexpr size_t kChunkBudget = kStaticScratchBytes - 8192;  // walker chunks sized to fit the array
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch per device, resolved on the first call on that device and
// re-resolved when the cached address no longer belongs to a live allocation (the device was
// reset with cudaDeviceReset, which unloads the module). Guarded by a mutex: calls from several
// host threads may race to fill it.
void* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

int scratch_for_current_device(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DW_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (g_scratch_ptr[dev]) {
        cudaPointerAttributes attr;
        if (cudaPointerGetAttributes(&attr, g_scratch_ptr[dev]) != cudaSuccess || attr.type != cudaMemoryTypeDevice ||
            attr.device != dev) {
            (void)cudaGetLastError();          // clear the query's error; re-resolve below
            g_scratch_ptr[dev] = nullptr;
        }
    }
    if (!g_scratch_ptr[dev]) {
        // the host-side symbol is only a stand-in: the kernels need the device address
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) { dw::set_last_cuda_error(e); return DW_ERR_CUDA; }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return DW_OK;
}

}  // namespace

extern "C" {

size_t dw_noalloc_scratch_bytes(void) { return kStaticScratchBytes; }

int dw_log_psi_sqr_noalloc(const DwArch* arch, int precision, const float* params, const void* prepared,
                           const float* r, int n_walkers, const float* R, const int32_t* Z, float* log_psi_sqr,
                           float* phase, void* stream) {
    dw::reset_launch_count();
    int st = dw::check_arch(arch);
    if (st != DW_OK) return st;
    if (!params || !prepared || !r || !R || !Z || !log_psi_sqr || n_walkers <= 0) return DW_ERR_ARG;
    // walkers run in chunks sized against the array; only an architecture whose single-walker
    // scratch exceeds it is refused
    const size_t need = dw::value_forward_bytes(arch, precision, n_walkers, kChunkBudget);
    if (need == 0) return DW_ERR_ARG;
    if (need > kStaticScratchBytes) return DW_ERR_WORKSPACE;
    void* scratch = nullptr;
    st = scratch_for_current_device(&scratch);
    if (st != DW_OK) return st;
    return dw::value_forward(arch, precision, params, prepared, r, n_walkers, R, Z, log_psi_sqr, phase, scratch,
                             kStaticScratchBytes, kChunkBudget, (cudaStream_t)stream);
}

}  // extern "C"
