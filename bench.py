#!/usr/bin/env python
"""Benchmark of the VMC inner loop on one GB300 (replicas on N GPUs under torchrun).

One step = one VMC inner iteration for all walkers of the workload: re-evaluate log psi^2,
10 Metropolis-Hastings steps (each a full log psi^2 forward), then the local energy with the
forward-mode Laplacian (mcmc.py:389-406 + hamiltonian.py:272-291). Metric: local-energy
walker-evals/s = walkers / seconds per step.

Default workload: the C2H4-shaped molecule (16 electrons, 32 determinants, 4096 walkers), mixed
precision (split-BF16 tensor-core GEMMs, FP64 LU / trace / reductions), one VMC optimisation
iteration per step (MH steps, local energy, clipped VMC gradient by the hand-written backward,
Adam update), random-init weights (seed 0), Gaussian walkers around the nuclei (seed 0). The
plain FP32 form is timed in the same run, and after the timed steps both forms are compared with
the FP64 form on the whole batch at the updated weights.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "local-energy walker-evals/s"
MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2h4", choices=["lih", "h10", "c2h4", "scale40"])
    ap.add_argument("--fp64-walkers", type=int, default=0,
                    help="walkers of the FP64 accuracy rerun (default: the whole batch, 1024 for scale40)")
    ap.add_argument("--walkers", type=int, default=0, help="override walker count")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--breakdown", action="store_true",
                    help="after the measurements, time two more steps by phase and by library timer tag")
    return ap.parse_args()


def workload(args):
    from deeperwin_gb300 import arch as A
    w = A.WORKLOADS[args.workload]
    mol = w.mol_fn()
    B = args.walkers or w.n_walkers
    return w, mol, A.arch_for(mol, w.n_dets), B


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- our arm
def peaks():
    if MEASURED_PEAKS.exists():
        d = json.loads(MEASURED_PEAKS.read_text())
        return d, "measured"
    return FALLBACK_PEAKS, "fallback"


def profile_traffic(name: str):
    """(DRAM bytes, algorithmic bytes) of the launch captured in the committed ncu summary."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None, None
    vals = {}
    for line in f.read_text().splitlines():
        for key in ("traffic_bytes_per_launch_full_workload:", "algorithmic_bytes_captured_launch:"):
            if line.startswith(key):
                try:
                    vals[key] = float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    pass
    return vals.get("traffic_bytes_per_launch_full_workload:"), vals.get("algorithmic_bytes_captured_launch:")


def run_ours(args, rank, world, dev):
    import torch
    from deeperwin_gb300 import api, _lib
    from deeperwin_gb300 import params as P
    import ctypes

    w, mol, a, B = workload(args)
    n_mh = w.n_mh_steps
    p_dict = P.init_params(a, seed=0)
    params = api.Params.from_dict(a, p_dict, w.precision, device=dev)
    state = api.MCMCState.initialize_around_nuclei(B, mol, seed=rank, device=dev)
    state.scalars[:] = torch.frombuffer(bytearray(bytes(_lib.DwMcmcScalars(0.0, 0.0, w.step_size, 0, 0, 0))),
                                        dtype=torch.uint8).to(dev)
    mh = api.MetropolisHastingsMonteCarlo(api.MCMCConfig(stepsize_update_interval=100))
    spin = (a.n_up, a.n_dn)
    L = _lib.lib()
    launches = [0]

    from deeperwin_gb300 import vmc, optim
    clip_state = [vmc.init_clipping_state()]
    optimizers = {}

    def mark(marks):
        if marks is not None:
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            marks.append(ev)

    def step(prm, marks=None):
        mark(marks)
        mh.run_mcmc_steps(None, state, prm, a.n_up, a.n_dn, None, n_steps=n_mh, reevaluate=True)
        launches[0] += api.last_launch_count()
        mark(marks)
        E = api.local_energy(prm, spin, state.r, state.R, state.Z)
        launches[0] += api.last_launch_count()
        mark(marks)
        if w.backward:
            # clipped VMC gradient (loss_function.py:75-156): tanh clipping with the previous
            # step's (center, width), coefficients (E_clip - mean) / B, hand-written backward
            Ec, cs = vmc._clip(E, clip_state[0][0], clip_state[0][1], 5.0)
            launches[0] += 1
            coeff = ((Ec.double() - cs[0]) / B).float()
            g = vmc.log_psi_sqr_backward(prm, state.r, state.R, state.Z, coeff)
            launches[0] += api.last_launch_count()
            mark(marks)
            # Adam update of the packed weights (optax.adam on the inverse schedule,
            # optimization/opt_utils.py:73-76) and the rebuilt derived weight copies
            opt = optimizers.get(id(prm))
            if opt is None:
                opt = optimizers[id(prm)] = optim.Adam(prm.flat)
            opt.step(prm, g)
            launches[0] += api.last_launch_count()
            c = cs[2:4].cpu()
            clip_state[0] = (float(c[0]), max(float(c[1]), 1e-12))
            mark(marks)
        return E

    def breakdown(n=2):
        """Milliseconds per step by phase (CUDA events on the current stream) and by library
        timer tag, over n steps after the measured ones."""
        tags = ["mh", "features", "streams", "conv", "spin_means", "mean_gemm", "map_gemm", "layer_gemm_value",
                "layer_gemm", "backflow_gemm", "envelope", "slogdet", "det_tangents", "jastrow", "combine",
                "guard", "guard_layer_gemm", "guard_fp64", "fp64_gemm", "fp64_tanh", "fp64_streams", "fp64_conv", "fp64_envelope", "fp64_lu",
                "fp64_det_tangents", "backward"]
        names = ["mcmc (11 forwards)", "local_energy", "backward", "adam"]
        tot = [0.0] * len(names)
        torch.cuda.synchronize()
        L.dw_timer_enable(1)
        for _ in range(n):
            marks = []
            step(params, marks)
            torch.cuda.synchronize()
            for i in range(len(marks) - 1):
                tot[i] += marks[i].elapsed_time(marks[i + 1]) / n
        out = {"phases_ms": {k: round(v, 3) for k, v in zip(names, tot) if v}, "tags_ms": {}}
        for t in tags:
            vals = [ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()]
            L.dw_timer_read(t.encode(), *[ctypes.byref(x) for x in vals])
            if vals[1].value:
                out["tags_ms"][t] = {"ms_per_step": round(vals[0].value / n, 3), "launches": vals[1].value // n}
        L.dw_timer_enable(0)
        return out

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(prm, K, W, sample_clocks=False, instrument=False):
        for _ in range(W):
            step(prm)
        torch.cuda.synchronize()
        barrier()
        launches[0] = 0
        if instrument:
            L.dw_timer_enable(1)
        clk = ClockSampler(torch.cuda.current_device()) if sample_clocks else None
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        barrier()
        e0.record(s)
        for _ in range(K):
            E = step(prm)
        e1.record(s)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / K
        clocks = clk.stop() if clk else None
        kt = None
        if instrument:
            vals = [ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()]
            L.dw_timer_read(b"layer_gemm", ctypes.byref(vals[0]), ctypes.byref(vals[1]), ctypes.byref(vals[2]),
                            ctypes.byref(vals[3]))
            L.dw_timer_enable(0)
            kt = {"ms": vals[0].value, "launches": vals[1].value, "flops": vals[2].value, "bytes": vals[3].value}
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms, E, clocks, kt, launches[0]

    def guard_stats(reset):
        out = {}
        for tier, name in ((0, "fp64_determinants"), (1, "fp64_form")):
            v = [ctypes.c_int64() for _ in range(3)]
            _lib.check(L.dw_guard_tier_stats(tier, *[ctypes.byref(x) for x in v], int(reset)), "dw_guard_tier_stats")
            out[name] = {"walkers": v[0].value, "flagged": v[1].value, "over_capacity": v[2].value,
                         "fraction": round(v[1].value / max(v[0].value, 1), 6)}
        return out

    guard_stats(True)
    ms, E_mixed, clocks, kt, n_launch = timed(params, args.steps, args.warmup, sample_clocks=True, instrument=True)
    gs = guard_stats(True)
    value = world * B / (ms / 1e3)
    # the chain's own state at the end of the timed steps: its walkers and the weights they were
    # equilibrated for (the end-to-end leg below restarts every step from one host copy of them)
    r_chain = state.r.clone()
    params_chain = api.Params(a, params.flat.clone(), w.precision)

    # end to end through the public API with host buffers: H2D of the walkers, D2H of E_L
    r_host = state.r.detach().cpu().pin_memory()
    E_host = torch.empty((args.steps, B), dtype=torch.float32).pin_memory()
    step(params)
    torch.cuda.synchronize()
    barrier()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for k in range(args.steps):
        state.r.copy_(r_host, non_blocking=True)
        E = step(params)
        E_host[k].copy_(E, non_blocking=True)
    e1.record(s)
    torch.cuda.synchronize()
    barrier()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms_e2e], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_e2e = float(t.item())
    e2e = {"value": world * B / (ms_e2e / 1e3), "unit": "walker-evals/s",
           "h2d_bytes_per_step": int(r_host.numel() * 4), "d2h_bytes_per_step": int(B * 4)}

    # walkers of the end-to-end leg at the weights the run ends with (the plain leg below moves
    # the shared chain)
    r_mixed = state.r.clone()
    plain = None
    if not args.no_plain and w.precision != "fp32":
        # with parameter updates the plain form optimises its own copy of the weights
        pparams = (api.Params(a, params.flat.clone(), "fp32") if w.backward else params.with_precision("fp32"))
        kp = max(2, args.steps // 2)
        ms_p, E_plain, _, _, _ = timed(pparams, kp, 1)
        # same walkers and weights through both forms: accuracy of the mixed form against plain
        # FP32 on the full batch
        pcmp = params_chain.with_precision("fp32")
        E_m = api.local_energy(params_chain, spin, r_chain, state.R, state.Z).double()
        E_p = api.local_energy(pcmp, spin, r_chain, state.R, state.Z).double()
        d = (E_m - E_p)
        ad = d.abs().cpu().numpy() * 1e3
        plain = {"value": world * B / (ms_p / 1e3), "ms_per_step": ms_p,
                 "mixed_over_plain": ms_p / ms,
                 "mixed_minus_plain_mean_E_mHa": float(d.mean().item() * 1e3),
                 "mixed_minus_plain_max_abs_mHa": float(ad.max()),
                 "abs_mixed_minus_plain_quantiles_mHa": {q: float(np.quantile(ad, float(q) / 100))
                                                         for q in ("50", "99", "99.9")}}

    out = None
    if rank == 0:
        pk, pk_kind = peaks()
        roof = None
        if kt and kt["launches"]:
            t_launch = kt["ms"] / kt["launches"] / 1e3
            gbs = kt["bytes"] / kt["launches"] / t_launch / 1e9
            tfs = kt["flops"] / kt["launches"] / t_launch / 1e12
            intensity = kt["flops"] / kt["bytes"]
            ridge = pk["bf16_tflops"] * 1e12 / (pk["hbm_gbs"] * 1e9)
            # ncu traffic of one captured layer-1 launch, scaled to the average launch by the ratio of
            # algorithmic bytes (DRAM traffic grows in proportion to the rows and K of a launch)
            prof_file = {"h10": "layer_gemm_h10.txt", "c2h4": "layer_gemm_c2h4.txt"}.get(w.name.split("_")[0])
            cap_traffic, cap_alg = profile_traffic(prof_file) if prof_file else (None, None)
            traffic = (round(cap_traffic / cap_alg * kt["bytes"] / kt["launches"])
                       if cap_traffic and cap_alg else None)
            if intensity < ridge:
                kname = {"mixed": "layer_gemm (tcgen05 split-BF16, forward-Laplacian h_el layers)",
                         "bf16": "layer_gemm (tcgen05 BF16, forward-Laplacian h_el layers)",
                         "fp32": "layer_gemm (FP32 CUDA-core GEMM + forward-Laplacian tanh, h_el layers)"}[w.precision]
                roof = {"kernel": kname, "bound": "hbm",
                        "achieved": round(gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                        "frac": round(gbs / pk["hbm_gbs"], 4), "traffic": traffic,
                        "traffic_source": (f"ncu dram read+write of an h_el layer launch of this workload (profiles/{prof_file}), "
                                           "scaled to the average launch by algorithmic bytes") if traffic else None,
                        "algorithmic_bytes_per_launch": kt["bytes"] / kt["launches"],
                        "avg_launch_ms": t_launch * 1e3, "tflops": round(tfs, 2),
                        "peak_source": pk_kind}
            else:
                roof = {"kernel": "layer_gemm", "bound": "tensor", "achieved": round(tfs, 2),
                        "peak": pk["bf16_tflops"], "unit": "TFLOP/s", "frac": round(tfs / pk["bf16_tflops"], 4),
                        "traffic": traffic, "avg_launch_ms": t_launch * 1e3, "peak_source": pk_kind}
        out = {
            "metric": METRIC, "value": round(value, 1), "unit": "walker-evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"mixed": "bf16x3 (split hi+lo) GEMMs, fp32 accumulate, fp64 LU/trace/reductions",
                      "fp32": "fp32", "bf16": "bf16"}[w.precision],
            "data": "synthetic: random-init weights (seed 0), Gaussian walkers around nuclei",
            "config": ours_config(w, mol, a, B, world),
            "e2e": e2e, "gpu_launches": int(n_launch), "clocks": clocks, "roofline": roof,
        }
        if plain:
            out["plain_fp32"] = plain
        if w.precision == "mixed":
            # walkers of the local energies (warm-up and timed steps) whose predicted E_L error was
            # above the tolerance and which were re-evaluated inside the mixed form: with FP64
            # determinant algebra, and (cancelled magnitude above 1e5 Ha) by the FP64 form
            out["tail_reevaluation"] = gs
    return out, (state, params, a, mol, w, r_mixed, breakdown, r_chain, params_chain)


def ours_config(w, mol, a, B, world):
    """The workload a step runs (the same dictionary on both arms)."""
    return {"workload": w.name, "molecule": mol.name, "n_el": a.n_el, "n_up": a.n_up,
            "n_ions": a.n_ions, "n_dets": a.n_dets, "walkers_per_gpu": B, "mh_steps_per_iter": w.n_mh_steps,
            "step": "reevaluate + %d MH forwards + forward-Laplacian E_L" % w.n_mh_steps
                    + (" + clipped VMC gradient (hand-written backward) + Adam update" if w.backward else ""),
            "precision": w.precision, "parallelism": "replicas" if world > 1 else "single",
            "l2": "working set (activations, several GB per step) exceeds L2; no flush needed"}


# ----------------------------------------------------------------------------- CPU legs (oracle)
def cpu_iteration(a, mol, p_dict, r_sample, threads, backward, dtype="float32"):
    """One VMC iteration of the CPU restatement on a walker sample, batched over the sample:
    11 log psi^2 forwards (re-evaluation + 10 MH proposals), the local energy (gradient and exact
    Laplacian by torch.func, vmapped over the walkers) and, for the gradient workloads, the clipped
    VMC gradient by autograd and an Adam update. Returns (seconds, E_L)."""
    import torch
    from oracle import dpe4 as O
    torch.set_num_threads(threads)
    dt = getattr(torch, dtype)
    p = {k: torch.as_tensor(np.asarray(v), dtype=dt) for k, v in p_dict.items()}
    r = torch.as_tensor(np.asarray(r_sample), dtype=dt)
    R = torch.as_tensor(np.asarray(mol.R), dtype=dt)
    gen = torch.Generator().manual_seed(0)
    t0 = time.perf_counter()
    with torch.no_grad():
        for _ in range(11):
            O.log_psi_sqr_raw(p, a, r + 0.1 * torch.randn(r.shape, generator=gen, dtype=dt), R, mol.Z)
    E = O.local_energy_batched(p, a, r, R, mol.Z).detach()
    if backward:
        c = E.mean()
        w = 5.0 * E.std(unbiased=False)
        Ec = c + torch.tanh((E - c) / w) * w
        coeff = (Ec - Ec.mean()) / len(Ec)
        pt = {k: v.clone().requires_grad_(True) for k, v in p.items()}
        (O.log_psi_sqr_raw(pt, a, r, R, mol.Z)[1] * coeff).sum().backward()
        with torch.no_grad():
            for k, v in pt.items():                      # optax.adam, first step (opt_utils.py:73-76)
                g = v.grad if v.grad is not None else torch.zeros_like(v)
                m, s2 = 0.1 * g, 0.001 * g * g
                v -= 1e-3 * (m / 0.1) / (torch.sqrt(s2 / 0.001) + 1e-8)
    return time.perf_counter() - t0, E.double().numpy()


def cpu_baseline(args, a, mol, r_sample, backward, p_dict=None):
    from deeperwin_gb300 import params as P
    threads = os.cpu_count() or 1
    p_dict = p_dict if p_dict is not None else P.init_params(a, seed=0)
    cpu_iteration(a, mol, p_dict, r_sample[:2], threads, backward)          # warm-up (thread pool, dispatch)
    dt, _ = cpu_iteration(a, mol, p_dict, r_sample, threads, backward)
    return {"value": round(len(r_sample) / dt, 4), "unit": "walker-evals/s", "cores": threads, "kind": "port",
            "sample": f"{len(r_sample)} walkers of the same workload, one VMC iteration batched over them "
                      f"(11 log psi^2 forwards + E_L{' + clipped VMC gradient + Adam update' if backward else ''}) "
                      f"by the FP32 CPU restatement of the reference algorithm (torch, {threads} threads), "
                      f"{dt:.1f} s"}


def accuracy_vs_fp64(a, mol, r_all, state, params, n_fp64, p_dict):
    """Both production forms against the FP64 form on the GPU over the whole batch (or its first
    n_fp64 walkers) of the mixed chain, at the weights the run ends with; the FP64 form itself is
    checked against the CPU FP64 oracle on the walkers where the mixed form is furthest from it."""
    import torch
    from deeperwin_gb300 import api
    from oracle import dpe4 as O
    spin = (a.n_up, a.n_dn)
    r = r_all[:n_fp64].contiguous()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E64 = api.local_energy(params.with_precision("fp64"), spin, r, state.R, state.Z).double()
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    out = {"walkers": int(r.shape[0]), "fp64_form_seconds": round(t64, 2),
           "E_mean_fp64_Ha": float(E64.mean())}
    errs = {}
    for name, prm in (("mixed", params), ("fp32", params.with_precision("fp32"))):
        E = api.local_energy(prm, spin, r, state.R, state.Z).double()
        e = (E - E64).cpu().numpy()
        ae = np.abs(e) * 1e3
        rel = np.abs(e) / np.abs(E64.cpu().numpy())
        errs[name] = e
        out[name] = {"mean_E_err_mHa": round(float(e.mean() * 1e3), 4),
                     "abs_err_quantiles_mHa": {q: round(float(np.quantile(ae, float(q) / 100)), 4)
                                               for q in ("50", "99", "99.9")},
                     "max_abs_err_mHa": round(float(ae.max()), 3),
                     "rel_err_quantiles": {q: float(np.quantile(rel, float(q) / 100)) for q in ("50", "99", "99.9")},
                     "frac_walkers_rel_err_le_1e-5": round(float((rel <= 1e-5).mean()), 5)}
    idx = np.argsort(-np.abs(errs["mixed"]))[:3]
    R32 = np.asarray(mol.R, np.float32).astype(np.float64)          # the nuclei as the library holds them
    E_o = O.local_energy(O.tparams(p_dict), a, r[idx].double().cpu().numpy(), R32, mol.Z)[0].numpy()
    out["fp64_form_vs_cpu_oracle_max_abs_mHa"] = float(np.abs(E64.cpu().numpy()[idx] - E_o).max() * 1e3)
    out["fp64_form_vs_cpu_oracle_walkers"] = "the 3 walkers with the largest |E_mixed - E_fp64|"
    return out


def run_reference(args):
    """Reference arm: the reference's JAX stack is not installed on this machine or the GPU machine, so
    the CPU restatement of its algorithm (oracle port) is timed on the host cores in the
    reference's default precision (float32), batched over a bounded walker sample per step."""
    from deeperwin_gb300 import arch as A
    from deeperwin_gb300 import params as P
    w, mol, a, B = workload(args)
    per = min(B, 64)
    r_all = A.init_walkers(mol, per * 2, seed=0)
    p_dict = P.init_params(a, seed=0)
    threads = os.cpu_count() or 1
    for _ in range(max(1, min(args.warmup, 1))):
        cpu_iteration(a, mol, p_dict, r_all[:4], threads, w.backward)
    times = []
    for k in range(args.steps):
        sample = r_all[(k % 2) * per:(k % 2) * per + per]
        dt, _ = cpu_iteration(a, mol, p_dict, sample, threads, w.backward)
        times.append(dt)
    sec = statistics.mean(times)
    value = per / sec
    cfg = ours_config(w, mol, a, B, world=1)
    out = {"metric": METRIC, "value": round(value, 4), "unit": "walker-evals/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 1),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
           "data": "synthetic: random-init weights (seed 0), Gaussian walkers around nuclei",
           "config": cfg, "impl": "reference", "sample_walkers_per_step": per,
           "cpu_baseline": {"value": round(value, 4), "unit": "walker-evals/s", "cores": threads, "kind": "port",
                            "sample": f"{per} walkers of the workload per step, one VMC iteration batched over them "
                                      "(11 log psi^2 forwards + E_L" + (" + clipped VMC gradient + Adam update"
                                                                         if w.backward else "") +
                                      "), FP32 CPU restatement of the reference algorithm (reference JAX stack not "
                                      "installed); ms_per_step is the measured time of one such sample"},
           "e2e": {"value": round(value, 4), "unit": "walker-evals/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=dev)
    from deeperwin_gb300 import _lib
    _lib.lib()
    out, ctx = run_ours(args, rank, world, dev)
    if rank == 0:
        from deeperwin_gb300 import params as P
        from deeperwin_gb300 import api
        state, params, a, mol, w, r_mixed, breakdown, r_chain, params_chain = ctx
        # the checks evaluate the weights the GPU holds now (updated ones after optimisation steps)
        p_now = P.unpack(a, params.flat.detach().cpu().numpy())
        if w.precision != "fp32" and not args.no_plain:
            n64 = args.fp64_walkers or (1024 if a.n_el > 30 else state.r.shape[0])
            n64 = min(n64, state.r.shape[0])
            p_chain = P.unpack(a, params_chain.flat.detach().cpu().numpy())
            out["accuracy_vs_fp64"] = accuracy_vs_fp64(a, mol, r_chain, state, params_chain, n64, p_chain)
            out["accuracy_vs_fp64"]["state"] = ("the mixed chain's walkers and weights at the end of the timed "
                                                "optimisation steps")
            # stress case: the end-to-end leg restarts every step from one host copy of the walkers
            # while the weights keep changing, so its final walkers sit closer to the new nodes
            out["accuracy_vs_fp64_restarted_walkers"] = accuracy_vs_fp64(a, mol, r_mixed, state, params, n64, p_now)
            out["accuracy_vs_fp64_restarted_walkers"]["state"] = (
                "the end-to-end leg's walkers (restarted every step from the walkers of the timed chain, 10 "
                "Metropolis-Hastings steps under weights that moved by up to 6 more Adam steps) at the final weights")
            # the same comparison at the random-init weights, on a chain equilibrated by 30 steps
            p0 = P.init_params(a, seed=0)
            params0 = api.Params.from_dict(a, p0, w.precision)
            st0 = api.MCMCState.initialize_around_nuclei(state.r.shape[0], mol, seed=1)
            st0.scalars[:] = torch.frombuffer(bytearray(bytes(_lib.DwMcmcScalars(0.0, 0.0, w.step_size, 0, 0, 0))),
                                              dtype=torch.uint8).cuda()
            api.MetropolisHastingsMonteCarlo(api.MCMCConfig(stepsize_update_interval=100)).run_mcmc_steps(
                None, st0, params0, a.n_up, a.n_dn, None, n_steps=30)
            out["accuracy_vs_fp64_initial_weights"] = accuracy_vs_fp64(a, mol, st0.r, st0, params0,
                                                                       min(n64, st0.r.shape[0]), p0)
            out["accuracy_vs_fp64_initial_weights"]["state"] = ("random-init weights (seed 0), walkers after 30 "
                                                                "Metropolis-Hastings steps from the Gaussian start")
        if not args.no_cpu_baseline:
            r_sample = state.r[:32].double().cpu().numpy()
            out["cpu_baseline"] = cpu_baseline(args, a, mol, r_sample, w.backward, p_now)
        if args.breakdown:
            out["breakdown"] = breakdown()
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
