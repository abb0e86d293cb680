#!/usr/bin/env python
"""Benchmark of the VMC inner loop on one GB300 (replicas on N GPUs under torchrun).

One step = one VMC inner iteration for all walkers of the workload: re-evaluate log psi^2,
10 Metropolis-Hastings steps (each a full log psi^2 forward), then the local energy with the
forward-mode Laplacian (mcmc.py:389-406 + hamiltonian.py:272-291). Metric: local-energy
walker-evals/s = walkers / seconds per step.

Default workload: H10 chain (10 electrons, 16 determinants, 8192 walkers), mixed precision
(split-BF16 tensor-core GEMMs, FP64 LU / trace / reductions), random-init weights (seed 0),
Gaussian walkers around the nuclei (seed 0). The plain FP32 form is timed in the same run.
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
    ap.add_argument("--workload", default="h10", choices=["lih", "h10", "c2h4", "scale40"])
    ap.add_argument("--walkers", type=int, default=0, help="override walker count")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
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

    def step(prm):
        mh.run_mcmc_steps(None, state, prm, a.n_up, a.n_dn, None, n_steps=n_mh, reevaluate=True)
        launches[0] += api.last_launch_count()
        E = api.local_energy(prm, spin, state.r, state.R, state.Z)
        launches[0] += api.last_launch_count()
        if w.backward:
            # clipped VMC gradient (loss_function.py:75-156): tanh clipping with the previous
            # step's (center, width), coefficients (E_clip - mean) / B, hand-written backward
            Ec, cs = vmc._clip(E, clip_state[0][0], clip_state[0][1], 5.0)
            launches[0] += 1
            coeff = ((Ec.double() - cs[0]) / B).float()
            g = vmc.log_psi_sqr_backward(prm, state.r, state.R, state.Z, coeff)
            launches[0] += api.last_launch_count()
            # Adam update of the packed weights (optax.adam on the inverse schedule,
            # optimization/opt_utils.py:73-76) and the rebuilt derived weight copies
            opt = optimizers.get(id(prm))
            if opt is None:
                opt = optimizers[id(prm)] = optim.Adam(prm.flat)
            opt.step(prm, g)
            launches[0] += api.last_launch_count()
            c = cs[2:4].cpu()
            clip_state[0] = (float(c[0]), max(float(c[1]), 1e-12))
        return E

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

    ms, E_mixed, clocks, kt, n_launch = timed(params, args.steps, args.warmup, sample_clocks=True, instrument=True)
    value = world * B / (ms / 1e3)

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

    plain = None
    if not args.no_plain and w.precision != "fp32":
        # with parameter updates the plain form optimises its own copy of the weights
        pparams = (api.Params(a, params.flat.clone(), "fp32") if w.backward else params.with_precision("fp32"))
        kp = max(2, args.steps // 2)
        ms_p, E_plain, _, _, _ = timed(pparams, kp, 1)
        # same walkers and weights through both forms: accuracy of the mixed form against plain
        # FP32 on the full batch
        pcmp = params.with_precision("fp32") if w.backward else pparams
        E_m = api.local_energy(params, spin, state.r, state.R, state.Z).double()
        E_p = api.local_energy(pcmp, spin, state.r, state.R, state.Z).double()
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
            cap_traffic, cap_alg = profile_traffic("layer_gemm_h10.txt") if w.name.startswith("h10") else (None, None)
            traffic = (round(cap_traffic / cap_alg * kt["bytes"] / kt["launches"])
                       if cap_traffic and cap_alg else None)
            if intensity < ridge:
                kname = {"mixed": "layer_gemm (tcgen05 split-BF16, forward-Laplacian h_el layers)",
                         "bf16": "layer_gemm (tcgen05 BF16, forward-Laplacian h_el layers)",
                         "fp32": "layer_gemm (FP32 CUDA-core GEMM + forward-Laplacian tanh, h_el layers)"}[w.precision]
                roof = {"kernel": kname, "bound": "hbm",
                        "achieved": round(gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                        "frac": round(gbs / pk["hbm_gbs"], 4), "traffic": traffic,
                        "traffic_source": ("ncu dram read+write of the h_el layer-1 launch (profiles/layer_gemm_h10.txt), "
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
            "config": {"workload": w.name, "molecule": mol.name, "n_el": a.n_el, "n_up": a.n_up,
                       "n_ions": a.n_ions, "n_dets": a.n_dets, "walkers_per_gpu": B, "mh_steps_per_iter": n_mh,
                       "step": "reevaluate + %d MH forwards + forward-Laplacian E_L" % n_mh
                               + (" + clipped VMC gradient (hand-written backward) + Adam update"
                                  if w.backward else ""),
                       "precision": w.precision, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "working set (activations, several GB per step) exceeds L2; no flush needed"},
            "e2e": e2e, "gpu_launches": int(n_launch), "clocks": clocks, "roofline": roof,
        }
        if plain:
            out["plain_fp32"] = plain
    return out, (state, params, a, mol, w)


# ----------------------------------------------------------------------------- CPU legs (oracle)
def cpu_sample(a, mol, p_dict, r_sample, threads):
    """One inner iteration of the FP64 oracle on a walker sample: 11 log psi^2 forwards + E_L."""
    import torch
    from oracle import dpe4 as O
    torch.set_num_threads(threads)
    tp = O.tparams(p_dict)
    t0 = time.perf_counter()
    for _ in range(11):
        O.log_psi_sqr(tp, a, r_sample, mol.R, mol.Z)
    E = O.local_energy(tp, a, r_sample, mol.R, mol.Z)[0]
    return time.perf_counter() - t0, E.numpy()


def cpu_baseline(args, a, mol, r_sample, gpu_E=None, p_dict=None):
    from deeperwin_gb300 import params as P
    threads = os.cpu_count() or 1
    p_dict = p_dict if p_dict is not None else P.init_params(a, seed=0)
    dt, E = cpu_sample(a, mol, p_dict, r_sample, threads)
    out = {"value": round(len(r_sample) / dt, 4), "unit": "walker-evals/s", "cores": threads, "kind": "port",
           "sample": f"{len(r_sample)} walkers x (11 log psi^2 forwards + E_L) of the same workload, FP64 oracle, "
                     f"{dt:.1f} s"}
    acc = None
    if gpu_E is not None:
        acc = {name: {"max_abs_mHa": float(np.abs(e - E).max() * 1e3), "mean_mHa": float((e - E).mean() * 1e3)}
               for name, e in gpu_E.items()}
    return out, acc


def worst_walkers(a, mol, state, params, p_dict=None, k=4):
    """The k walkers of the full batch where the mixed and plain forms differ most, each checked
    against the FP64 oracle: the tail of the per-walker error (ill-conditioned Slater matrices)."""
    import torch
    from deeperwin_gb300 import api
    from oracle import dpe4 as O
    from deeperwin_gb300 import params as P
    spin = (a.n_up, a.n_dn)
    E_m = api.local_energy(params, spin, state.r, state.R, state.Z).double()
    E_p = api.local_energy(params.with_precision("fp32"), spin, state.r, state.R, state.Z).double()
    idx = torch.argsort((E_m - E_p).abs(), descending=True)[:k]
    r = state.r[idx].double().cpu().numpy()
    p_dict = p_dict if p_dict is not None else P.init_params(a, seed=0)
    E_o = O.local_energy(O.tparams(p_dict), a, r, mol.R, mol.Z)[0].numpy()
    return {"selection": f"the {k} walkers of the full batch with the largest |E_mixed - E_plain|",
            "E_oracle_Ha": [round(float(x), 6) for x in E_o],
            "mixed_abs_err_mHa": [round(float(x), 3) for x in np.abs(E_m[idx].cpu().numpy() - E_o) * 1e3],
            "fp32_abs_err_mHa": [round(float(x), 3) for x in np.abs(E_p[idx].cpu().numpy() - E_o) * 1e3]}


def run_reference(args):
    """Reference arm: the reference's JAX code cannot run on this machine (no jax/haiku/folx),
    so the CPU restatement of its algorithm (the oracle port) is timed on the host cores."""
    from deeperwin_gb300 import arch as A
    w, mol, a, B = workload(args)
    r_all = A.init_walkers(mol, 64, seed=0)
    from deeperwin_gb300 import params as P
    p_dict = P.init_params(a, seed=0)
    threads = os.cpu_count() or 1
    per = 4 if a.n_el <= 10 else 1
    for k in range(args.warmup if args.warmup < 1 else 1):
        cpu_sample(a, mol, p_dict, r_all[:1], threads)
    times = []
    for k in range(args.steps):
        sample = r_all[(k * per) % 60:(k * per) % 60 + per]
        dt, _ = cpu_sample(a, mol, p_dict, sample, threads)
        times.append(dt / per)
    sec_per_walker = statistics.mean(times)
    value = 1.0 / sec_per_walker
    out = {"metric": METRIC, "value": round(value, 4), "unit": "walker-evals/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec_per_walker * B * 1e3, 1),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
           "data": "synthetic: random-init weights (seed 0), Gaussian walkers around nuclei",
           "config": {"workload": w.name, "walkers_per_gpu": B, "sample_walkers_per_step": per},
           "impl": "reference",
           "cpu_baseline": {"value": round(value, 4), "unit": "walker-evals/s", "cores": threads, "kind": "port",
                            "sample": f"{per} walker(s) per step x (11 log psi^2 forwards + E_L), FP64 restatement "
                                      "of the reference algorithm (reference JAX stack not installed)"},
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
        if not args.no_cpu_baseline:
            from deeperwin_gb300 import api
            from deeperwin_gb300 import params as P
            state, params, a, mol, w = ctx
            r_sample = state.r[:8].double().cpu().numpy()
            gpu_E = {"mixed" if w.precision != "fp32" else "fp32":
                     api.local_energy(params, (a.n_up, a.n_dn), r_sample, mol.R, mol.Z).double().cpu().numpy()}
            if w.precision != "fp32":
                gpu_E["fp32"] = api.local_energy(params.with_precision("fp32"), (a.n_up, a.n_dn), r_sample, mol.R,
                                                 mol.Z).double().cpu().numpy()
            # the oracle evaluates the weights the GPU holds now (updated ones after optimisation steps)
            p_now = P.unpack(a, params.flat.detach().cpu().numpy()) if w.backward else None
            cb, acc = cpu_baseline(args, a, mol, r_sample, gpu_E, p_now)
            out["cpu_baseline"] = cb
            out["accuracy_vs_fp64_oracle"] = acc
            if w.precision != "fp32" and not args.no_plain:
                out["accuracy_worst_walkers_vs_fp64_oracle"] = worst_walkers(a, mol, state, params, p_now)
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
