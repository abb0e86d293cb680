// Host-side model description: architecture checks, the packed parameter layout and
// launch dimensions. The layout mirrors deeperwin_gb300/params.py (param_shapes): same
// tensor order, each tensor row-major and starting at a multiple of 64 floats.
#include "common.cuh"
#include <string.h>
#include <map>
#include <string>
#include <vector>

namespace dw {

static thread_local cudaError_t g_last_cuda = cudaSuccess;
static thread_local int64_t g_launches = 0;
void set_last_cuda_error(cudaError_t e) { g_last_cuda = e; }
void count_launch(int n) { g_launches += n; }
int64_t launch_count() { return g_launches; }
void reset_launch_count() { g_launches = 0; }

struct TimerSlot {
    std::vector<cudaEvent_t> pending;   // start/end pairs not yet read
    cudaEvent_t open = nullptr;
    double ms = 0, flops = 0, bytes = 0;
    int64_t launches = 0;
};
static std::map<std::string, TimerSlot> g_timers;
static bool g_timer_on = false;
bool timer_on() { return g_timer_on; }
void timer_begin(const char* tag, cudaStream_t s) {
    if (!g_timer_on) return;
    TimerSlot& t = g_timers[tag];
    cudaEventCreate(&t.open);
    cudaEventRecord(t.open, s);
}
void timer_end(const char* tag, cudaStream_t s, double flops, double bytes) {
    if (!g_timer_on) return;
    TimerSlot& t = g_timers[tag];
    if (!t.open) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    t.pending.push_back(t.open);
    t.pending.push_back(e);
    t.open = nullptr;
    t.flops += flops; t.bytes += bytes; t.launches += 1;
}

int check_arch(const DwArch* a) {
    if (!a) return DW_ERR_ARG;
    if (a->n_el < 2 || a->n_el > kMaxEl) return DW_ERR_ARCH;
    if (a->n_up < 1 || a->n_up > a->n_el - 1) return DW_ERR_ARCH;
    if (a->n_ions < 1 || a->n_ions > kMaxIons) return DW_ERR_ARCH;
    if (a->n_dets < 1 || a->n_dets > 128) return DW_ERR_ARCH;
    if (a->z_min < 1 || a->z_max < a->z_min || a->z_max > 118) return DW_ERR_ARCH;
    if (a->width_one != 256 || a->width_two != 32 || a->width_ion != 32) return DW_ERR_ARCH;
    if (a->jastrow0 != 64 || a->jastrow1 != 64) return DW_ERR_ARCH;
    return DW_OK;
}

static int64_t push(ParamLayout* L, int64_t& off, int64_t size) {
    int64_t o = off;
    L->off[L->n_entries] = o;
    L->size[L->n_entries] = size;
    L->n_entries++;
    off += (size + kAlignFloats - 1) / kAlignFloats * kAlignFloats;
    return o;
}

void make_layout(const DwArch* a, ParamLayout* L) {
    memset(L, 0, sizeof(*L));
    int64_t off = 0;
    const int D = a->width_one, E = a->width_two, I = a->width_ion, N = a->n_ions;
    const int64_t KN = (int64_t)a->n_dets * a->n_el;
    L->ion_embed = push(L, off, (int64_t)(a->z_max - a->z_min + 1) * I);
    for (int it = 0; it < 4; ++it) {
        int ee = it == 0 ? 1 : E;
        int hw = it == 0 ? 4 * N : D;
        int ei = it == 0 ? 4 : E;
        int inw = 3 * hw + E + ei;
        L->w_same_w[it] = push(L, off, (int64_t)ee * E);
        L->w_same_b[it] = push(L, off, E);
        L->w_diff_w[it] = push(L, off, (int64_t)ee * E);
        L->w_diff_b[it] = push(L, off, E);
        L->h_map_w[it] = push(L, off, (int64_t)hw * E);
        L->h_map_b[it] = push(L, off, E);
        L->h_ion_map_w[it] = push(L, off, (int64_t)I * ei);
        L->h_ion_map_b[it] = push(L, off, ei);
        L->h_el_w[it] = push(L, off, (int64_t)inw * D);
        L->h_el_b[it] = push(L, off, D);
        if (it < 3) {
            L->h_same_w[it] = push(L, off, (int64_t)ee * E);
            L->h_same_b[it] = push(L, off, E);
            L->h_diff_w[it] = push(L, off, (int64_t)ee * E);
            L->h_diff_b[it] = push(L, off, E);
            L->h_ei_w[it] = push(L, off, (int64_t)ei * E);
            L->h_ei_b[it] = push(L, off, E);
        }
    }
    L->bf_up = push(L, off, (int64_t)D * KN);
    L->bf_dn = push(L, off, (int64_t)D * KN);
    L->alpha_up = push(L, off, (int64_t)N * KN);
    L->alpha_dn = push(L, off, (int64_t)N * KN);
    L->weights_up = push(L, off, (int64_t)N * KN);
    L->weights_dn = push(L, off, (int64_t)N * KN);
    L->jas_w[0] = push(L, off, (int64_t)D * a->jastrow0);
    L->jas_b[0] = push(L, off, a->jastrow0);
    L->jas_w[1] = push(L, off, (int64_t)a->jastrow0 * a->jastrow1);
    L->jas_b[1] = push(L, off, a->jastrow1);
    L->jas_w[2] = push(L, off, (int64_t)a->jastrow1);
    L->total = off;
}

Dims make_dims(const DwArch* a, bool tangents) {
    Dims d;
    d.n = a->n_el; d.nu = a->n_up; d.nd = a->n_el - a->n_up; d.N = a->n_ions; d.K = a->n_dets;
    d.zmin = a->z_min; d.zmax = a->z_max;
    d.D = a->width_one; d.E = a->width_two; d.EI = a->width_ion; d.J0 = a->jastrow0; d.J1 = a->jastrow1;
    for (int it = 0; it < 4; ++it) {
        d.hw[it] = it == 0 ? 4 * d.N : d.D;
        d.eiw[it] = it == 0 ? 4 : d.E;
        d.eew[it] = it == 0 ? 1 : d.E;
        d.inw[it] = 3 * d.hw[it] + d.E + d.eiw[it];
        d.kw[it] = round_up(d.hw[it] + d.E + d.eiw[it], 64);
    }
    d.KN = d.K * d.n;
    if (tangents) {
        d.T = 3 * d.n + 2;
        d.Tp = next_pow2(d.T);
        d.lap = d.T - 1;
    } else {
        d.T = 1; d.Tp = 1; d.lap = -1;
    }
    d.seg = nullptr;
    d.nseg = 1;
    return d;
}

}  // namespace dw

extern "C" {

const char* dw_status_string(int s) {
    switch (s) {
        case DW_OK: return "ok";
        case DW_ERR_ARCH: return "unsupported architecture or shape";
        case DW_ERR_ARG: return "invalid argument";
        case DW_ERR_WORKSPACE: return "workspace too small";
        case DW_ERR_CUDA: return cudaGetErrorString(dw::g_last_cuda);
        case DW_ERR_TIMEOUT: return "bounded device wait timed out";
        case DW_ERR_UNSUPPORTED: return "unsupported on this device";
        default: return "unknown status";
    }
}

const char* dw_version(void) { return "dwgb 0.1 (sm_103a)"; }

int64_t dw_param_count(const DwArch* a) {
    if (dw::check_arch(a) != DW_OK) return -1;
    dw::ParamLayout L;
    dw::make_layout(a, &L);
    return L.total;
}

int dw_param_layout(const DwArch* a, int64_t* offsets, int64_t* sizes, int max_entries) {
    int s = dw::check_arch(a);
    if (s != DW_OK) return -s;
    dw::ParamLayout L;
    dw::make_layout(a, &L);
    for (int i = 0; i < L.n_entries && i < max_entries; ++i) {
        if (offsets) offsets[i] = L.off[i];
        if (sizes) sizes[i] = L.size[i];
    }
    return L.n_entries;
}

int64_t dw_last_launch_count(void) { return dw::launch_count(); }

// Enables (1) or disables (0) per-tag kernel timing and clears accumulated timings.
int dw_timer_enable(int on) {
    for (auto& kv : dw::g_timers)
        for (cudaEvent_t e : kv.second.pending) cudaEventDestroy(e);
    dw::g_timers.clear();
    dw::g_timer_on = on != 0;
    return DW_OK;
}

// Synchronizes the recorded events of `tag` and returns total milliseconds, launch count and
// the algorithmic FLOPs / bytes of those launches.
int dw_timer_read(const char* tag, double* ms, int64_t* launches, double* flops, double* bytes) {
    auto it = dw::g_timers.find(tag);
    if (it == dw::g_timers.end()) { *ms = 0; *launches = 0; *flops = 0; *bytes = 0; return DW_OK; }
    dw::TimerSlot& t = it->second;
    for (size_t k = 0; k + 1 < t.pending.size(); k += 2) {
        float x = 0.f;
        if (cudaEventSynchronize(t.pending[k + 1]) != cudaSuccess) return DW_ERR_CUDA;
        cudaEventElapsedTime(&x, t.pending[k], t.pending[k + 1]);
        t.ms += x;
        cudaEventDestroy(t.pending[k]);
        cudaEventDestroy(t.pending[k + 1]);
    }
    t.pending.clear();
    *ms = t.ms; *launches = t.launches; *flops = t.flops; *bytes = t.bytes;
    return DW_OK;
}

}  // extern "C"
