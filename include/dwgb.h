/*
 * dwgb.h - C ABI of the GB300-native DeepErwin VMC inner loop.
 *
 * One shared library (libdwgb.so) with extern "C" entry points taking plain device
 * pointers, sizes and a cudaStream_t passed as void*. No torch types cross this
 * boundary. Every entry point returns an int status (DW_OK == 0); no C++ exception
 * crosses the ABI. All device buffers are owned by the caller; the library never
 * allocates device memory on the compute entry points: scratch comes from a
 * caller-provided workspace whose size is queried with dw_workspace_bytes().
 *
 * Array conventions (row-major, float32 unless stated):
 *   r        [n_walkers, n_el, 3]  electron coordinates (bohr)
 *   R        [n_ions, 3]           nuclear coordinates
 *   Z        [n_ions] int32        nuclear charges
 *   params   packed float32 weights, layout from dw_param_layout()
 *   log_psi_sqr / phase / E_loc [n_walkers]
 *
 * The reference functions each entry point replaces are cited on the declaration
 * (paths relative to the reference's src/deeperwin/).
 */
#ifndef DWGB_H
#define DWGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Model shape: dpe4 embedding + envelope orbitals (full_det) + Jastrow.
 * ModelConfigDeepErwin4 (configuration.py:875-890), EmbeddingConfigDeepErwin4
 * (configuration.py:422-440), JastrowConfig(n_hidden=[64,64]) (configuration.py:809-816). */
typedef struct DwArch {
    int32_t n_el;        /* electrons, 2..64 */
    int32_t n_up;        /* spin-up electrons, 1..n_el-1 */
    int32_t n_ions;      /* nuclei, 1..16 */
    int32_t n_dets;      /* determinants K */
    int32_t z_min;       /* ion embedding table covers Z in [z_min, z_max] */
    int32_t z_max;
    int32_t width_one;   /* 1-el stream width (256) */
    int32_t width_two;   /* 2-el / el-ion stream width (32) */
    int32_t width_ion;   /* ion embedding width (32) */
    int32_t jastrow0;    /* Jastrow hidden widths (64, 64) */
    int32_t jastrow1;
} DwArch;

enum DwStatus {
    DW_OK = 0,
    DW_ERR_ARCH = 1,        /* unsupported architecture / shape */
    DW_ERR_ARG = 2,         /* null pointer, bad size, bad precision */
    DW_ERR_WORKSPACE = 3,   /* workspace too small or misaligned */
    DW_ERR_CUDA = 4,        /* a CUDA runtime call failed */
    DW_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    DW_ERR_UNSUPPORTED = 6  /* feature not available on this device */
};

enum DwPrecision {
    DW_PRECISION_FP32 = 0,  /* plain form: FP32 end to end (CUDA-core GEMMs, FP32 LU) */
    DW_PRECISION_MIXED = 1, /* tensor-core GEMMs on split-BF16 operands (hi + lo, three BF16 MMAs per
                               K step, FP32 accumulate) + FP64 LU / trace / reductions */
    DW_PRECISION_BF16 = 2,  /* single-pass BF16 tensor-core GEMMs + FP64 LU (fastest, least accurate) */
    DW_PRECISION_FP64 = 3,  /* FP64 end to end: every GEMM, activation, envelope, LU, inverse, determinant
                               tangent, Coulomb sum and reduction in double (the reference's
                               float_precision: float64 mode, configuration.py:1893 and
                               process_molecule.py:20-29); outputs are rounded to float32. Forward,
                               local energy and MCMC only (no parameter gradient) */
    DW_PRECISION_FP32_DET64 = 4, /* plain FP32 network (CUDA-core GEMMs) with the determinant algebra in
                                    FP64: LU, Gauss-Jordan inverse and tangent traces of the FP32 Slater
                                    channels. Forward, local energy and MCMC (no parameter gradient) */
    DW_PRECISION_MIXED_DET64 = 5 /* the mixed form's split-BF16 tensor-core network with the determinant
                                    algebra of DW_PRECISION_FP32_DET64. Forward, local energy and MCMC
                                    (no parameter gradient); uses the mixed form's prepared weights */
};

/* Human-readable text for a status code (static storage). */
const char* dw_status_string(int status);

/* Version / build info string. */
const char* dw_version(void);

/* Number of float32 values in the packed parameter vector. */
int64_t dw_param_count(const DwArch* arch);

/* Packed layout: offsets[i], sizes[i] (in floats) of the i-th tensor in the canonical
 * order (ion_embed, per iteration the conv maps, h_el, 2-el and el-ion streams, backflow,
 * envelopes, Jastrow). Writes at most max_entries and returns the total entry count
 * (or a negative status). Mirrors the haiku parameter tree built by
 * build_log_psi_squared (model/wavefunction.py:281-287). */
int dw_param_layout(const DwArch* arch, int64_t* offsets, int64_t* sizes, int max_entries);

/* Bytes of derived ("prepared") weights for a precision: re-ordered FP32 / BF16 copies
 * that the GEMM kernels read. */
size_t dw_prepared_bytes(const DwArch* arch, int precision);

/* Builds the prepared weights from the packed params (device -> device, stream-ordered).
 * Must be re-run after every parameter update. */
int dw_prepare_params(const DwArch* arch, int precision, const float* params,
                      void* prepared, size_t prepared_bytes, void* stream);

/* Workspace bytes for n_walkers walkers. mode: 0 = log psi^2 only, 1 = local energy,
 * 2 = MCMC steps, 3 = parameter gradient. */
size_t dw_workspace_bytes(const DwArch* arch, int precision, int n_walkers, int mode);

/* log psi^2 and phase for all walkers.
 * Replaces log_psi_sqr(params, n_up, n_dn, r, R, Z, fixed_params) -> (phase, log_psi_sqr)
 * (model/wavefunction.py:293, Wavefunction.__call__ :118-134). */
int dw_log_psi_sqr(const DwArch* arch, int precision, const float* params, const void* prepared,
                   const float* r, int n_walkers, const float* R, const int32_t* Z,
                   float* log_psi_sqr, float* phase,
                   void* workspace, size_t workspace_bytes, void* stream);

/* Local energy E_L = -1/2 (Laplacian log|psi| + |grad log|psi||^2) + V_Coulomb, with a
 * forward-mode Laplacian through the whole network.
 * Replaces get_local_energy(params, spin_state, r, R, Z, fixed_params) -> E_L
 * (hamiltonian.py:272-291; kinetic term hamiltonian.py:198-216, Coulomb :17-39).
 * log_psi_sqr may be NULL. grad_log_psi_sqr ([n_walkers, 3 n_el]) may be NULL. */
int dw_local_energy(const DwArch* arch, int precision, const float* params, const void* prepared,
                    const float* r, int n_walkers, const float* R, const int32_t* Z,
                    float* E_loc, float* log_psi_sqr, float* grad_log_psi_sqr,
                    void* workspace, size_t workspace_bytes, void* stream);

/* Coulomb potential energy only. Replaces get_potential_energy (hamiltonian.py:34-39). */
int dw_potential_energy(const float* r, int n_walkers, int n_el, const float* R, const int32_t* Z,
                        int n_ions, float* E_pot, void* stream);

/* Device-resident MCMC chain scalars (MCMCState stepsize / step_nr / acc_rate, mcmc.py:21-34). */
typedef struct DwMcmcScalars {
    double acc_rate;      /* running acceptance rate (EMA 0.9/0.1) */
    double last_acc;      /* all-walker mean acceptance of the last step (FP64 reduction) */
    float stepsize;
    int32_t step_nr;
    uint32_t ticket;      /* internal: block-completion counter, keep 0 */
    int32_t error;        /* internal */
} DwMcmcScalars;

/* Proposal rules of MetropolisHastingsMonteCarlo._build_proposal_function (mcmc.py:328-342). */
enum DwProposal {
    DW_PROPOSAL_NORMAL = 0,        /* r + s N(0, 1) (mcmc.py:175-180) */
    DW_PROPOSAL_CAUCHY = 1,        /* r + s Cauchy (mcmc.py:196-201) */
    DW_PROPOSAL_LANGEVIN = 2,      /* local step size + nuclear-attraction drift, with the proposal ratio
                                      (mcmc.py:204-215, :260-288) */
    DW_PROPOSAL_LOCAL = 3,         /* step size s clip(d_closest_ion, r_min, r_max) per electron, with the
                                      proposal ratio (mcmc.py:218-234) */
    DW_PROPOSAL_NORMAL_ONE_EL = 4, /* one electron (step_nr mod n_el) per step (mcmc.py:183-193) */
    DW_PROPOSAL_LOCAL_ONE_EL = 5   /* local step size, one electron per step (mcmc.py:237-257) */
};

typedef struct DwMcmcConfig {
    int32_t n_steps;
    int32_t max_age;
    int32_t stepsize_update_interval;
    float target_acceptance_rate;
    float min_stepsize;
    float max_stepsize;
    uint64_t seed;
    int32_t reevaluate;   /* 1: recompute log psi^2 of the current walkers first (mcmc.py:396) */
    int32_t proposal;     /* DwProposal */
    float r_min;          /* local / Langevin proposals: clip range of the closest-nucleus distance */
    float r_max;
    float langevin_scale; /* Langevin proposal: scale of the nuclear-attraction drift */
    float p_spin_swap;    /* probability of exchanging an electron of the first n_el / 2 with one of the
                             others after the proposal (mcmc.py:291-302, 349-354) */
    float p_spin_flip;    /* probability of reversing the electron order (mcmc.py:305-310, 355-356) */
} DwMcmcConfig;

/* n_steps all-walker Metropolis-Hastings steps with the proposal rule cfg->proposal and the
 * optional spin swaps / flips; acceptance exp(log psi^2' - log psi^2 + log q-ratio) > U.
 * r, log_psi_sqr, age (int32) and the device scalars are updated in place.
 * Random numbers: Philox-4x32-10 keyed by (seed, walker), counter = step number.
 * Replaces MetropolisHastingsMonteCarlo.run_mcmc_steps (mcmc.py:325-327, :389-406) with its
 * proposal functions (mcmc.py:175-310) and make_mcmc_step (mcmc.py:345-387). */
int dw_mcmc_steps(const DwArch* arch, int precision, const float* params, const void* prepared,
                  float* r, int n_walkers, const float* R, const int32_t* Z,
                  float* log_psi_sqr, int32_t* age, DwMcmcScalars* scalars_dev,
                  const DwMcmcConfig* cfg, void* workspace, size_t workspace_bytes, void* stream);

/* ---- Packed launches (continuous-batching serving) -------------------------------------
 * One launch over the walkers of nseg geometries (requests) that share n_el and n_up and one
 * weight set. Geometry g occupies R[g * n_ions .. ][3] and Z[g * n_ions ..]; a geometry with
 * fewer nuclei than arch->n_ions is padded with Z = 0 ions, which contribute exactly nothing
 * (input features, ion maps, envelopes, Coulomb). seg[b] in [0, nseg) names walker b's
 * geometry (device int32 array). 1 <= nseg <= 256. Every walker's result equals the result of
 * the same walker evaluated in a launch of its geometry alone. No counterpart in the reference,
 * which evaluates one geometry per call (get_log_psi_squared / get_local_energy with a single
 * fixed R, Z: model/wavefunction.py:152-171, hamiltonian.py:272-291). */
int dw_log_psi_sqr_packed(const DwArch* arch, int precision, const float* params, const void* prepared,
                          const float* r, int n_walkers, const float* R, const int32_t* Z, int nseg,
                          const int32_t* seg, float* log_psi_sqr, float* phase,
                          void* workspace, size_t workspace_bytes, void* stream);

int dw_local_energy_packed(const DwArch* arch, int precision, const float* params, const void* prepared,
                           const float* r, int n_walkers, const float* R, const int32_t* Z, int nseg,
                           const int32_t* seg, float* E_loc, float* log_psi_sqr, float* grad_log_psi_sqr,
                           void* workspace, size_t workspace_bytes, void* stream);

/* Packed Metropolis-Hastings: walker b runs in chain seg[b], which has its own scalars
 * scalars_dev[seg[b]] (step size, acceptance, step counter) and Philox key seeds[seg[b]]
 * (device uint64 array; cfg->seed is ignored), and draws its random numbers as walker
 * walker_index[b] of that chain. A chain therefore follows the same trajectory whatever it
 * is packed with. The other cfg fields apply to all chains. */
int dw_mcmc_steps_packed(const DwArch* arch, int precision, const float* params, const void* prepared,
                         float* r, int n_walkers, const float* R, const int32_t* Z, int nseg,
                         const int32_t* seg, const int32_t* walker_index, const uint64_t* seeds,
                         float* log_psi_sqr, int32_t* age, DwMcmcScalars* scalars_dev,
                         const DwMcmcConfig* cfg, void* workspace, size_t workspace_bytes, void* stream);

/* Forces on the nuclei (hamiltonian.py:309-338 calculate_forces): forces[I][c] = mean over walkers of
 * sum_i Z_I (r_i - R_I)_c / d'^3, d' = d / tanh(d / R_cut), plus the nucleus-nucleus repulsion
 * (hamiltonian.py:298-306). antithetic = 1: each walker is averaged with its mirror image (electrons
 * within R_core of their closest nucleus reflected through it) weighted by psi^2(mirror) / psi^2,
 * which evaluates log psi^2 at the mirrored walkers in the given precision form. log_psi_sqr: the
 * walkers' current log psi^2. forces [n_ions * 3] FP64; per_walker ([n_walkers, n_ions, 3] FP64,
 * electrons summed) may be NULL. Workspace: dw_forces_workspace_bytes. */
size_t dw_forces_workspace_bytes(const DwArch* arch, int precision, int n_walkers);
int dw_forces(const DwArch* arch, int precision, const float* params, const void* prepared,
              const float* r, int n_walkers, const float* R, const int32_t* Z, const float* log_psi_sqr,
              float R_cut, float R_core, int antithetic, double* forces, double* per_walker,
              void* workspace, size_t workspace_bytes, void* stream);

/* FP64 cross-walker statistics of a float32 vector: out[0]=mean, out[1]=variance
 * (population), out[2]=count of entries that are not NaN. Only NaNs are skipped, as jnp.nanmean
 * does (loss_function.py:94-95): an infinite entry makes the mean that infinity and the variance
 * infinite (NaN if both signs occur or no finite entry is left). Deterministic (fixed reduction
 * order). */
int dw_energy_stats(const float* E, int n, double* out_dev, void* stream);

/* tanh clipping of local energies around (center, width) and the clipped statistics
 * (loss_function.py:44-72): E_clip = c + tanh((E - c)/w) w; out = [mean_clip, var_clip,
 * new_center, new_width(=clip_by * std)]. */
int dw_clip_energies(const float* E, int n, double center, double width, double clip_by,
                     float* E_clip, double* out_dev, void* stream);

/* Gradient of sum_b coeff[b] * log psi^2_b w.r.t. all packed parameters (accumulated into
 * grad_params, which the caller zeroes). With coeff = (E_clip - mean E_clip) / B this is the
 * VMC gradient of loss_function.py:141-153. Activations are recomputed, not stored. */
int dw_log_psi_sqr_backward(const DwArch* arch, int precision, const float* params, const void* prepared,
                            const float* r, int n_walkers, const float* R, const int32_t* Z,
                            const float* coeff, float* grad_params,
                            void* workspace, size_t workspace_bytes, void* stream);

/* log psi^2 and phase like dw_log_psi_sqr, but with no workspace argument and no device
 * allocation anywhere: scratch comes from a fixed static device array of
 * dw_noalloc_scratch_bytes() bytes (64 MiB) that every GPU loading the library reserves until
 * process exit. For callers that cannot allocate device memory at call time (a host framework
 * owning all device memory through its own pool, or a fixed-budget embedding). The walkers run
 * in chunks sized to fit the array, so any walker count is accepted; an architecture whose
 * single-walker scratch exceeded the array would return DW_ERR_WORKSPACE. FP32, mixed and BF16
 * forms only (DW_PRECISION_FP64: DW_ERR_ARG). The first call on a device resolves the array's
 * device address with cudaGetSymbolAddress (again after a cudaDeviceReset of that device); make
 * that first call before any stream capture. All calls share the array and its contents persist
 * between calls, so calls that overlap on the GPU (different streams, or concurrent host
 * threads) race; serialize them. No counterpart in the reference. */
int dw_log_psi_sqr_noalloc(const DwArch* arch, int precision, const float* params, const void* prepared,
                           const float* r, int n_walkers, const float* R, const int32_t* Z,
                           float* log_psi_sqr, float* phase, void* stream);
/* Size in bytes of the static scratch array used by dw_log_psi_sqr_noalloc. */
size_t dw_noalloc_scratch_bytes(void);

/* Instrumentation of the mixed form's local energy: walkers whose predicted E_L error (the
 * magnitude of the terms the forward Laplacian cancels, times the split-BF16 entry accuracy) is
 * above the tolerance are re-evaluated with FP64 determinant algebra inside dw_local_energy /
 * dw_local_energy_packed (tier 0), and those whose cancelled magnitude exceeds 1e5 Ha by the FP64
 * form (tier 1). Returns the cumulative counts of a tier since its last reset: walkers seen,
 * walkers flagged, flagged walkers beyond the per-call capacity (those keep the previous tier's
 * values). Synchronizes the device. dw_guard_stats reads tier 0 and its reset clears both tiers.
 * No reference counterpart. */
int dw_guard_tier_stats(int tier, int64_t* walkers, int64_t* flagged, int64_t* overflow, int reset);
int dw_guard_stats(int64_t* walkers, int64_t* flagged, int64_t* overflow, int reset);

/* Instrumentation: determinant-tangent kernels. 0 = the default choice; 1 = the single-buffer
 * tile kernel instead of the pipelined one for n_el in {4, 8, 16} and the general kernel instead
 * of the tile kernel for n_el in 33..40. Returns the previous choice, or -DW_ERR_ARG. No
 * reference counterpart. */
int dw_debug_set_det_tangents_kernel(int which);

/* Instrumentation: network of the tier-0 re-evaluation, DW_PRECISION_FP32_DET64 (default) or
 * DW_PRECISION_MIXED_DET64. Returns the previous form, or -DW_ERR_ARG. No reference counterpart. */
int dw_debug_set_guard_form(int precision);

/* Number of kernel launches issued by the last call on this host thread (instrumentation). */
int64_t dw_last_launch_count(void);

/* Instrumentation: per-tag CUDA-event timing of selected kernels on their launch stream
 * ("layer_gemm" = the widened forward-Laplacian layer GEMMs of the production form,
 * "guard_layer_gemm" = those of the tail re-evaluation, "guard" = the whole tail re-evaluation,
 * "backward" = dw_log_psi_sqr_backward, "mh" = the Metropolis-Hastings kernel; the other tags
 * name the stages of the forward). dw_timer_enable clears the
 * accumulators; dw_timer_read synchronizes the recorded events and returns the total time (ms),
 * launch count, and the algorithmic FLOPs and bytes of those launches. No reference counterpart. */
int dw_timer_enable(int on);
int dw_timer_read(const char* tag, double* ms, int64_t* launches, double* flops, double* bytes);

#ifdef __cplusplus
}
#endif
#endif /* DWGB_H */
