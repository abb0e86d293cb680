"""Reference-shaped Python API over the C ABI.

Mirrors the hot-path call surface of DeepErwin (paths relative to src/deeperwin):

* ``build_log_psi_squared`` -> ``log_psi_sqr(params, n_up, n_dn, r, R, Z, fixed_params)``
  returning ``(phase, log_psi_sqr)`` (model/wavefunction.py:262-299).
* ``build_local_energy`` -> ``get_local_energy(params, spin_state, r, R, Z, fixed_params)``
  (hamiltonian.py:272-291).
* ``MCMCState`` / ``MetropolisHastingsMonteCarlo.run_mcmc_steps`` (mcmc.py:21-151, :314-412).
* ``build_value_and_grad_func`` (optimization/loss_function.py:75-156) in ``deeperwin_gb300.vmc``.

All arrays are torch CUDA tensors; every call runs hand-written sm_103a kernels through
libdwgb.so on the current torch stream. Nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Dict, Optional, Tuple

import numpy as np
import torch

from . import _lib
from .arch import Arch, Molecule, arch_for, init_walkers
from .params import init_params, layout, pack

_C = ctypes.c_void_p


def _ptr(t: Optional[torch.Tensor]):
    return _C(t.data_ptr()) if t is not None else _C(0)


def _stream():
    return _C(torch.cuda.current_stream().cuda_stream)


def _require_cuda(*ts):
    for t in ts:
        if t is not None and (not t.is_cuda or not t.is_contiguous()):
            raise ValueError("dwgb expects contiguous CUDA tensors")


class _Workspace:
    """Grow-only scratch buffers, allocated through torch's caching allocator."""

    def __init__(self):
        self.bufs: Dict[str, torch.Tensor] = {}

    def get(self, key: str, nbytes: int, device) -> torch.Tensor:
        b = self.bufs.get(key)
        if b is None or b.numel() < nbytes or b.device != device:
            b = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
            self.bufs[key] = b
        return b


_WS = _Workspace()


@dataclasses.dataclass
class Params:
    """Packed float32 weights on the GPU plus the derived (prepared) copies the kernels read."""

    arch: Arch
    flat: torch.Tensor
    precision: str = "mixed"
    prepared: Optional[torch.Tensor] = None

    def __post_init__(self):
        _require_cuda(self.flat)
        self.c_arch = _lib.make_arch(self.arch)
        self.prepare()

    @property
    def prec(self) -> int:
        return _lib.DW_PRECISION[self.precision]

    def prepare(self) -> None:
        L = _lib.lib()
        nbytes = L.dw_prepared_bytes(ctypes.byref(self.c_arch), self.prec)
        if self.prepared is None or self.prepared.numel() < nbytes:
            self.prepared = torch.empty(nbytes, dtype=torch.uint8, device=self.flat.device)
        _lib.check(L.dw_prepare_params(ctypes.byref(self.c_arch), self.prec, _ptr(self.flat), _ptr(self.prepared),
                                       nbytes, _stream()), "dw_prepare_params")

    def with_precision(self, precision: str) -> "Params":
        return Params(self.arch, self.flat, precision)

    @staticmethod
    def from_dict(arch: Arch, params: Dict[str, np.ndarray], precision: str = "mixed", device="cuda") -> "Params":
        flat = torch.as_tensor(pack(arch, params), device=device)
        return Params(arch, flat, precision)


def _geometry(R, Z, device):
    Rt = torch.as_tensor(np.asarray(R, np.float32), device=device).contiguous()
    Zt = torch.as_tensor(np.asarray(Z, np.int32), device=device).contiguous()
    return Rt, Zt


def _as_walkers(r, device) -> torch.Tensor:
    if not torch.is_tensor(r):
        r = torch.as_tensor(np.asarray(r, np.float32))
    return r.to(device=device, dtype=torch.float32).contiguous()


def log_psi_sqr(params: Params, n_up: int, n_dn: int, r, R, Z, fixed_params=None
                ) -> Tuple[torch.Tensor, torch.Tensor]:
    """(phase, log psi^2) of all walkers, model/wavefunction.py:293."""
    a = params.arch
    if n_up != a.n_up or n_dn != a.n_dn:
        raise ValueError(f"spin state ({n_up},{n_dn}) does not match the model ({a.n_up},{a.n_dn})")
    dev = params.flat.device
    r = _as_walkers(r, dev)
    B = r.shape[0]
    Rt, Zt = (R, Z) if torch.is_tensor(R) and R.is_cuda else _geometry(R, Z, dev)
    lp = torch.empty(B, dtype=torch.float32, device=dev)
    ph = torch.empty(B, dtype=torch.float32, device=dev)
    L = _lib.lib()
    nbytes = L.dw_workspace_bytes(ctypes.byref(params.c_arch), params.prec, B, 0)
    ws = _WS.get("fwd", nbytes, dev)
    _lib.check(L.dw_log_psi_sqr(ctypes.byref(params.c_arch), params.prec, _ptr(params.flat), _ptr(params.prepared),
                                _ptr(r), B, _ptr(Rt), _ptr(Zt), _ptr(lp), _ptr(ph), _ptr(ws), nbytes, _stream()),
               "dw_log_psi_sqr")
    return ph, lp


def local_energy(params: Params, spin_state, r, R, Z, fixed_params=None, return_grad: bool = False):
    """E_L per walker (hamiltonian.py:280-289); optionally also log psi^2 and grad log psi^2."""
    a = params.arch
    dev = params.flat.device
    r = _as_walkers(r, dev)
    B = r.shape[0]
    Rt, Zt = (R, Z) if torch.is_tensor(R) and R.is_cuda else _geometry(R, Z, dev)
    E = torch.empty(B, dtype=torch.float32, device=dev)
    lp = torch.empty(B, dtype=torch.float32, device=dev)
    g = torch.empty(B, 3 * a.n_el, dtype=torch.float32, device=dev) if return_grad else None
    L = _lib.lib()
    nbytes = L.dw_workspace_bytes(ctypes.byref(params.c_arch), params.prec, B, 1)
    ws = _WS.get("lap", nbytes, dev)
    _lib.check(L.dw_local_energy(ctypes.byref(params.c_arch), params.prec, _ptr(params.flat), _ptr(params.prepared),
                                 _ptr(r), B, _ptr(Rt), _ptr(Zt), _ptr(E), _ptr(lp), _ptr(g), _ptr(ws), nbytes,
                                 _stream()), "dw_local_energy")
    if return_grad:
        return E, lp, g
    return E


def potential_energy(r, R, Z) -> torch.Tensor:
    r = _as_walkers(r, "cuda")
    B, n, _ = r.shape
    Rt, Zt = _geometry(R, Z, r.device)
    E = torch.empty(B, dtype=torch.float32, device=r.device)
    _lib.check(_lib.lib().dw_potential_energy(_ptr(r), B, n, _ptr(Rt), _ptr(Zt), len(Zt), _ptr(E), _stream()),
               "dw_potential_energy")
    return E


def calculate_forces(params: Params, r, R, Z, log_psi_sqr: torch.Tensor, R_cut: float = 0.1, R_core: float = 0.5,
                     use_antithetic_sampling: bool = False, per_walker: bool = False):
    """Forces on the nuclei, [n_ions, 3] FP64 (hamiltonian.py:309-338; ForceEvaluationConfig defaults,
    configuration.py:1225-1229). With per_walker, also the per-walker forces [B, n_ions, 3]."""
    a = params.arch
    dev = params.flat.device
    r = _as_walkers(r, dev)
    B = r.shape[0]
    Rt, Zt = (R, Z) if torch.is_tensor(R) and R.is_cuda else _geometry(R, Z, dev)
    F = torch.empty(a.n_ions, 3, dtype=torch.float64, device=dev)
    pw = torch.empty(B, a.n_ions, 3, dtype=torch.float64, device=dev) if per_walker else None
    L = _lib.lib()
    nbytes = L.dw_forces_workspace_bytes(ctypes.byref(params.c_arch), params.prec, B)
    ws = _WS.get("forces", nbytes, dev)
    _lib.check(L.dw_forces(ctypes.byref(params.c_arch), params.prec, _ptr(params.flat), _ptr(params.prepared), _ptr(r),
                           B, _ptr(Rt), _ptr(Zt), _ptr(log_psi_sqr.contiguous()), float(R_cut), float(R_core),
                           1 if use_antithetic_sampling else 0, _ptr(F), _ptr(pw), _ptr(ws), nbytes, _stream()),
               "dw_forces")
    return (F, pw) if per_walker else F


def build_log_psi_squared(mol: Molecule, n_dets: int, seed: int = 0, precision: str = "mixed",
                          z_min: int = 1, z_max: Optional[int] = None, device="cuda", **init_kw):
    """Seeded model for a molecule; returns (log_psi_sqr, params) like the reference's builder."""
    arch = arch_for(mol, n_dets, z_min=z_min, z_max=z_max)
    params = Params.from_dict(arch, init_params(arch, seed, **init_kw), precision, device)
    return log_psi_sqr, params


def build_local_energy(log_psi_squared=None, is_complex=False, is_periodic=False, include_heg_background=False,
                       forward_lap=True, max_batch_size=None):
    """Returns get_local_energy(params, spin_state, r, R, Z, fixed_params) -> E_L (hamiltonian.py:272-291).
    The forward Laplacian is always used; walker chunking is chosen by the library from its workspace."""
    if is_complex or is_periodic or include_heg_background:
        raise NotImplementedError("only real-valued molecular wavefunctions are supported")

    def get_local_energy(params: Params, spin_state, r, R, Z, fixed_params=None):
        return local_energy(params, spin_state, r, R, Z, fixed_params)
    return get_local_energy


# ---------------------------------------------------------------------------- MCMC
@dataclasses.dataclass
class MCMCConfig:
    """Defaults of MCMCConfigOptimization (configuration.py:1030-1034). ``proposal`` names the
    proposal rule (configuration.py:952-975, mcmc.py:328-342): "normal", "cauchy",
    "normal_one_el", "local", "local_one_el" or "langevin"; r_min / r_max default to the rule's
    config (local: 0.1 / 1.0, Langevin: 0.2 / 2.0); spin swaps and flips as p_spin_swap /
    p_spin_flip (configuration.py:1024-1028)."""

    n_inter_steps: int = 20
    n_burn_in: int = 1000
    max_age: int = 20
    stepsize_update_interval: int = 100
    n_walkers: int = 2048
    target_acceptance_rate: float = 0.5
    min_stepsize_scale: float = 1e-2
    max_stepsize_scale: float = 1.0
    proposal: str = "normal"
    r_min: Optional[float] = None
    r_max: Optional[float] = None
    langevin_scale: float = 1.0
    p_spin_swap: float = 0.0
    p_spin_flip: float = 0.0

    def c_config(self, n_steps: int, seed: int, reevaluate: bool) -> "_lib.DwMcmcConfig":
        if self.proposal not in _lib.DW_PROPOSAL:
            raise ValueError(f"unknown MCMC proposal {self.proposal!r}")
        lo, hi = (0.2, 2.0) if self.proposal == "langevin" else (0.1, 1.0)
        return _lib.DwMcmcConfig(int(n_steps), int(self.max_age), int(self.stepsize_update_interval),
                                 float(self.target_acceptance_rate), float(self.min_stepsize_scale),
                                 float(self.max_stepsize_scale), ctypes.c_uint64(seed).value, 1 if reevaluate else 0,
                                 _lib.DW_PROPOSAL[self.proposal], float(lo if self.r_min is None else self.r_min),
                                 float(hi if self.r_max is None else self.r_max), float(self.langevin_scale),
                                 float(self.p_spin_swap), float(self.p_spin_flip))


class MCMCState:
    """Device-resident chain state (mcmc.py:21-34): walkers, log psi^2, ages, and the
    stepsize / step_nr / acc_rate scalars in one device struct (DwMcmcScalars)."""

    def __init__(self, r: torch.Tensor, R, Z, seed: int = 0, stepsize: float = 1e-2):
        self.r = r.contiguous()
        dev = r.device
        self.R, self.Z = _geometry(R, Z, dev)
        B = r.shape[0]
        self.log_psi_sqr = torch.full((B,), -1000.0, dtype=torch.float32, device=dev)   # mcmc.py:87-88
        self.walker_age = torch.zeros(B, dtype=torch.int32, device=dev)
        self.seed = int(seed)
        s = _lib.DwMcmcScalars(0.0, 0.0, float(stepsize), 0, 0, 0)
        raw = bytes(s)
        self.scalars = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)

    def _host_scalars(self) -> _lib.DwMcmcScalars:
        return _lib.DwMcmcScalars.from_buffer_copy(bytes(self.scalars.cpu().numpy()))

    @property
    def stepsize(self) -> float:
        return self._host_scalars().stepsize

    @property
    def acc_rate(self) -> float:
        return self._host_scalars().acc_rate

    @property
    def step_nr(self) -> int:
        return self._host_scalars().step_nr

    @property
    def last_acceptance(self) -> float:
        return self._host_scalars().last_acc

    @classmethod
    def initialize_around_nuclei(cls, n_walkers: int, mol: Molecule, seed: int = 0, device="cuda") -> "MCMCState":
        """``init_method="gaussian"``, ``spin_initialization="ordered"`` (mcmc.py:52-67)."""
        r = torch.as_tensor(init_walkers(mol, n_walkers, seed).astype(np.float32), device=device)
        return cls(r, mol.R, mol.Z, seed=seed)


class MetropolisHastingsMonteCarlo:
    def __init__(self, config: MCMCConfig):
        self.config = config
        self._calls = 0

    def run_mcmc_steps(self, func, state: MCMCState, params: Params, n_up: int, n_dn: int, fixed_params=None,
                       n_steps: int = 1, reevaluate: bool = True, group=None) -> MCMCState:
        """mcmc.py:389-406: re-evaluate log psi^2, then n_steps fused propose/accept steps.

        With several ranks (torch.distributed initialised; `group` or the default group) each
        rank holds its own walkers and a distinct seed, and the acceptance rate is combined over
        ranks after every step as the reference's pmean (mcmc.py:367): the steps then run one
        per call (the noise is keyed by walker and step number, so n one-step calls give the
        walkers of one n-step call) with the chain scalars averaged in between."""
        from . import dist
        if dist.world(group) > 1 and n_steps > 1:
            total = 0
            for k in range(n_steps):
                self.run_mcmc_steps(func, state, params, n_up, n_dn, fixed_params, 1, reevaluate and k == 0, group)
                total += last_launch_count()
            _lib.launch_override = total         # last_launch_count() reports all n calls
            return state
        a = params.arch
        if (n_up, n_dn) != (a.n_up, a.n_dn):
            raise ValueError("spin state does not match the model")
        cfg = self.config.c_config(n_steps, state.seed, reevaluate)
        B = state.r.shape[0]
        L = _lib.lib()
        nbytes = L.dw_workspace_bytes(ctypes.byref(params.c_arch), params.prec, B, 2)
        ws = _WS.get("mcmc", nbytes, state.r.device)
        _lib.check(L.dw_mcmc_steps(ctypes.byref(params.c_arch), params.prec, _ptr(params.flat), _ptr(params.prepared),
                                   _ptr(state.r), B, _ptr(state.R), _ptr(state.Z), _ptr(state.log_psi_sqr),
                                   _ptr(state.walker_age), _ptr(state.scalars), ctypes.byref(cfg), _ptr(ws), nbytes,
                                   _stream()), "dw_mcmc_steps")
        if n_steps > 0:
            dist.sync_chain_scalars_(state.scalars, group)
        return state

    def run_inter_steps(self, func, state, params, n_up, n_dn, fixed_params=None):
        return self.run_mcmc_steps(func, state, params, n_up, n_dn, fixed_params, self.config.n_inter_steps)

    def run_burn_in(self, func, state, params, n_up, n_dn, fixed_params=None):
        return self.run_mcmc_steps(func, state, params, n_up, n_dn, fixed_params, self.config.n_burn_in)


def energy_stats(E: torch.Tensor) -> torch.Tensor:
    """FP64 [mean, var, count] of finite entries (loss_function.py:94-95)."""
    out = torch.empty(3, dtype=torch.float64, device=E.device)
    _lib.check(_lib.lib().dw_energy_stats(_ptr(E.contiguous()), E.numel(), _ptr(out), _stream()), "dw_energy_stats")
    return out


def last_launch_count() -> int:
    """Kernel launches of the last library call on this thread (of all its one-step calls when
    run_mcmc_steps split the steps across ranks)."""
    if _lib.launch_override is not None:
        return int(_lib.launch_override)
    return int(_lib.lib().dw_last_launch_count())
