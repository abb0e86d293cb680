// log psi^2 without any device allocation by the caller or the library.
//
// Some callers cannot allocate device memory at the point where they evaluate the
// wavefunction: a host framework that owns all device memory through its own pool and
// forbids cudaMalloc inside a plug-in call, or an embedding that runs with a fixed memory
// budget. For them dw_log_psi_sqr_noalloc takes its scratch from a file-scope static
// __device__ array instead of a caller-provided workspace. The array has a fixed size
// (kStaticScratchBytes); every GPU that loads the library reserves it until the process exits.
#include "net.cuh"

namespace {

constexpr size_t kStaticScratchBytes = (size_t)64 << 20;   // 64 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch per device, resolved on the first call on that device.
void* g_scratch_ptr[kMaxDevices] = {nullptr};

int scratch_for_current_device(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DW_ERR_CUDA;
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
    const size_t need = dw::value_forward_bytes(arch, precision, n_walkers);
    if (need == 0) return DW_ERR_ARG;
    if (need > kStaticScratchBytes) return DW_ERR_WORKSPACE;   // too many walkers for the fixed scratch
    void* scratch = nullptr;
    st = scratch_for_current_device(&scratch);
    if (st != DW_OK) return st;
    return dw::value_forward(arch, precision, params, prepared, r, n_walkers, R, Z, log_psi_sqr, phase, scratch,
                             kStaticScratchBytes, (cudaStream_t)stream);
}

}  // extern "C"
