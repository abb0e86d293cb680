"""Device-resident continuous-batching loop for VMC requests on one GPU.

A request asks for an energy estimate (``kind="energy"``: ``n_steps`` Metropolis-Hastings steps of
``n_walkers`` walkers initialised around the nuclei, then E_L of every walker and its FP64 mean and
variance) or one optimisation step (``kind="opt_step"``: the same, then the clipped VMC gradient of
the request's own copy of the weights and the first Adam update of that copy, from a fresh optimiser
state, as the VMC optimisation step makes it). It is the per-geometry work
of the reference's optimisation / evaluation loops (optimization/variational_optimization.py:139-186,
optimization/evaluation.py:143-201: MCMC inter-steps, get_local_energy, value_and_grad), served for
many geometries at once, which the reference does not do.

Design:

* Weights are shared: one random-init parameter set for (n_el_max = 30, n_ions_max = 8); the model of
  a molecule is its slice (``params.slice_shared``). Inside the loop every molecule is padded to
  n_ions_max ions with Z = 0, which contribute exactly nothing, so all requests with equal n_el use
  one weight slice and are packed into one launch (``dw_*_packed``).
* Each request's walkers, log psi^2, ages, chain scalars (step size, acceptance, step counter) and
  Philox key stay in HBM from admission to completion. A chain draws its random numbers by
  (request seed, walker index in the request, step counter), so its trajectory does not depend on
  what it is packed with: a request gives the same result alone and in the mix.
* Admission is by an HBM budget: a request reserves its state plus the workspace of its walkers
  evaluated alone (an upper bound of its share of any packed launch) and is admitted when the sum
  of the active reservations stays within the budget (and a slot is free).
* Every (n_el, n_up) group has a fixed CUDA stream and its own workspace; groups run concurrently.
  Requests join their group's pack at the next scheduling quantum (``quantum`` MH steps), so
  arrivals are admitted while earlier requests are on the GPU. The host issues work
  asynchronously and learns about completions from CUDA events.

Nothing here computes on the CPU except the walker initialisation (numpy, like
``init_walkers``) and the bookkeeping.
"""
from __future__ import annotations

import collections
import ctypes
import dataclasses
import math
import time
from typing import Deque, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib, optim
from .api import MCMCConfig, Params, _ptr
from .arch import Arch, Molecule, init_walkers, random_molecule
from .params import init_params, pack, slice_shared

N_IONS_MAX = 8
N_EL_MAX = 30
MAX_SEG = 256            # geometries per packed launch (kMaxSeg in the library)


@dataclasses.dataclass
class Request:
    rid: int
    mol: Molecule
    n_walkers: int
    n_steps: int = 20
    kind: str = "energy"          # "energy" | "opt_step"
    arrival: float = 0.0          # seconds after the start of the stream
    seed: int = 0
    lr: float = 1e-3              # Adam learning rate of kind="opt_step" (a fresh optimiser state)
    keep_walkers: bool = False    # keep the final walkers and E_L on the device in the result


@dataclasses.dataclass
class Result:
    rid: int
    n_el: int
    n_walkers: int
    E_mean: float
    E_var: float
    acc_rate: float
    last_acceptance: float
    stepsize: float
    t_arrival: float
    t_admit: float
    t_done: float
    E_loc: Optional[torch.Tensor] = None
    r: Optional[torch.Tensor] = None
    grad: Optional[torch.Tensor] = None
    new_params: Optional[torch.Tensor] = None
    loss: Optional[float] = None

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival


def stream_requests(n: int = 2000, rate: float = 2.0, seed: int = 0, walkers: Tuple[int, int] = (1024, 4096),
                    n_steps: int = 20, opt_fraction: float = 0.0) -> List[Request]:
    """Seeded request stream: Poisson arrivals at ``rate`` per second, random molecules
    (2-8 nuclei, Z in {1, 6, 7, 8}, 6-bohr cube, pairs >= 1.5 bohr, neutral, n_up = ceil(n_el / 2)),
    uniform walker counts."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        mol = random_molecule(rng)
        nw = int(rng.integers(walkers[0], walkers[1] + 1))
        kind = "opt_step" if rng.uniform() < opt_fraction else "energy"
        out.append(Request(k, mol, nw, n_steps, kind, t, seed=int(rng.integers(0, 2 ** 62))))
    return out


class SharedWeights:
    """One random-init weight set for (n_el_max, n_ions_max) and its per-n_el slices on the GPU."""

    def __init__(self, n_dets: int = 8, n_el_max: int = N_EL_MAX, n_ions_max: int = N_IONS_MAX, seed: int = 0,
                 precision: str = "mixed", device="cuda"):
        self.n_dets, self.n_el_max, self.n_ions_max = n_dets, n_el_max, n_ions_max
        self.big = Arch(n_el_max, (n_el_max + 1) // 2, n_ions_max, n_dets)
        self.params_np = init_params(self.big, seed)
        self.precision = precision
        self.device = device
        self._packed: Dict[Tuple[int, int, str], Params] = {}

    def arch(self, n_el: int, n_up: int, n_ions: Optional[int] = None) -> Arch:
        return Arch(n_el, n_up, self.n_ions_max if n_ions is None else n_ions, self.n_dets)

    def slice(self, n_el: int, n_up: int, n_ions: Optional[int] = None) -> Dict[str, np.ndarray]:
        return slice_shared(self.big, self.params_np, self.arch(n_el, n_up, n_ions))

    def params(self, n_el: int, n_up: int, precision: Optional[str] = None) -> Params:
        """Prepared weights of the padded (n_ions_max) model for one electron count."""
        prec = precision or self.precision
        key = (n_el, n_up, prec)
        p = self._packed.get(key)
        if p is None:
            a = self.arch(n_el, n_up)
            p = Params(a, torch.as_tensor(pack(a, self.slice(n_el, n_up)), device=self.device), prec)
            self._packed[key] = p
        return p

    def molecule_params(self, mol: Molecule, precision: Optional[str] = None) -> Params:
        """Unpadded model of one molecule (its own n_ions): the one-at-a-time path and the gradient."""
        a = self.arch(mol.n_el, mol.n_up, mol.n_ions)
        flat = torch.as_tensor(pack(a, self.slice(mol.n_el, mol.n_up, mol.n_ions)), device=self.device)
        return Params(a, flat, precision or self.precision)


def padded_geometry(mol: Molecule, n_ions_max: int = N_IONS_MAX) -> Tuple[np.ndarray, np.ndarray]:
    if mol.n_ions > n_ions_max:
        raise ValueError(f"molecule has {mol.n_ions} nuclei; the loop serves at most {n_ions_max}")
    R = np.zeros((n_ions_max, 3), np.float32)
    Z = np.zeros(n_ions_max, np.int32)
    R[:mol.n_ions] = mol.R
    Z[:mol.n_ions] = mol.Z
    return R, Z


def _scalars_init(stepsize: float) -> bytes:
    return bytes(_lib.DwMcmcScalars(0.0, 0.0, float(stepsize), 0, 0, 0))


class _State:
    """Device-resident state of one admitted request."""

    def __init__(self, req: Request, eng: "ServingEngine", t_admit: float):
        self.req = req
        self.t_admit = t_admit
        dev = eng.device
        mol = req.mol
        self.n_el, self.n_up = mol.n_el, mol.n_up
        Rp, Zp = padded_geometry(mol, eng.weights.n_ions_max)
        r0 = init_walkers(mol, req.n_walkers, seed=req.seed % (2 ** 32)).astype(np.float32)
        nw = req.n_walkers
        # one pinned staging buffer, one H2D copy
        host = torch.empty(nw * mol.n_el * 3 + Rp.size, dtype=torch.float32).pin_memory()
        host[:nw * mol.n_el * 3] = torch.from_numpy(r0.reshape(-1))
        host[nw * mol.n_el * 3:] = torch.from_numpy(Rp.reshape(-1))
        dbuf = host.to(dev, non_blocking=True)
        self._host_keepalive = host
        self.r = dbuf[:nw * mol.n_el * 3].view(nw, mol.n_el, 3)
        self.R = dbuf[nw * mol.n_el * 3:].view(-1, 3)
        self.Z = torch.as_tensor(Zp, device=dev)
        self.lp = torch.full((nw,), -1000.0, dtype=torch.float32, device=dev)     # mcmc.py:87-88
        self.age = torch.zeros(nw, dtype=torch.int32, device=dev)
        self.scalars = torch.frombuffer(bytearray(_scalars_init(eng.stepsize)), dtype=torch.uint8).to(dev)
        self.widx = torch.arange(nw, dtype=torch.int32, device=dev)
        self.seed = req.seed & ((1 << 63) - 1)
        self.steps_done = 0
        self.evaluated = False        # log psi^2 of the initial walkers computed
        self.reserved = eng.reservation(req)
        self.E: Optional[torch.Tensor] = None
        self.cancelled = False


class _Group:
    """Requests with one electron count: shared weights, one stream, one workspace."""

    def __init__(self, n_el: int, n_up: int, stream: torch.cuda.Stream):
        self.n_el, self.n_up = n_el, n_up
        self.stream = stream
        self.members: List[_State] = []
        self.pack_key: Optional[Tuple[int, ...]] = None
        self.pack: Optional[Dict[str, torch.Tensor]] = None


class ServingEngine:
    """Continuous-batching server. ``run(requests)`` replays a timed stream in real time;
    ``submit`` / ``poll`` / ``drain`` drive it by hand."""

    def __init__(self, weights: SharedWeights, hbm_budget_bytes: float = 150e9, max_active: int = 512,
                 quantum: int = 5, n_streams: int = 4, max_pack_walkers: int = 1 << 18, max_inflight: int = 2,
                 mcmc: Optional[MCMCConfig] = None, stepsize: float = 0.1, clip_by: float = 5.0):
        self.weights = weights
        self.device = torch.device(weights.device)
        self.precision = weights.precision
        self.budget = float(hbm_budget_bytes)
        self.max_active = max_active
        self.quantum = max(1, int(quantum))
        self.max_pack_walkers = max_pack_walkers
        self.max_inflight = max_inflight
        self.mcmc = mcmc or MCMCConfig()
        self.stepsize = stepsize
        self.clip_by = clip_by
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max(1, n_streams))]
        self.ws: List[Optional[torch.Tensor]] = [None] * len(self.streams)
        self.inflight: List[Deque[torch.cuda.Event]] = [collections.deque() for _ in self.streams]
        self.groups: Dict[Tuple[int, int], _Group] = {}     # keyed by (n_el, n_up)
        self.pending: Deque[Tuple[Request, float]] = collections.deque()    # (request, host arrival time)
        self.finishing: List[Tuple[torch.cuda.Event, List[_State], torch.Tensor, torch.Tensor]] = []
        self.results: Dict[int, Result] = {}
        self.cancelled = set()
        self.reserved = 0.0
        self.peak_reserved = 0.0
        self.n_active = 0
        self.t0 = time.perf_counter()
        self.launches = 0
        self._ws_bytes_cache: Dict[Tuple[int, int, int, int], int] = {}

    # ------------------------------------------------------------------ bookkeeping
    def now(self) -> float:
        return time.perf_counter() - self.t0

    def _ws_bytes(self, n_el: int, n_up: int, B: int, mode: int) -> int:
        key = (n_el, n_up, B, mode)
        v = self._ws_bytes_cache.get(key)
        if v is None:
            a = _lib.make_arch(self.weights.arch(n_el, n_up))
            v = int(_lib.lib().dw_workspace_bytes(ctypes.byref(a), _lib.DW_PRECISION[self.precision], B, mode))
            if v == 0:
                raise ValueError(f"unsupported request shape n_el={n_el}")
            self._ws_bytes_cache[key] = v
        return v

    def reservation(self, req: Request) -> float:
        """HBM reserved while a request is active: its state and the workspace of its walkers."""
        n, nw = req.mol.n_el, req.n_walkers
        state = nw * (n * 3 * 4 * 3 + 4 * 4 + 4 * 2) + 4096
        ws = max(self._ws_bytes(n, req.mol.n_up, nw, 1), self._ws_bytes(n, req.mol.n_up, nw, 2))
        if req.kind == "opt_step":
            a = _lib.make_arch(self.weights.arch(n, req.mol.n_up, req.mol.n_ions))
            ws = max(ws, int(_lib.lib().dw_workspace_bytes(ctypes.byref(a), _lib.DW_PRECISION[self.precision], nw, 3)))
            ws += 8 * int(_lib.lib().dw_param_count(ctypes.byref(a))) * 4
        return float(state + ws)

    def _workspace(self, si: int, nbytes: int) -> torch.Tensor:
        w = self.ws[si]
        if w is None or w.numel() < nbytes:
            self.ws[si] = None
            w = torch.empty(int(nbytes * 1.25) + 4096, dtype=torch.uint8, device=self.device)
            self.ws[si] = w
        return w

    def submit(self, req: Request, t_arrival: Optional[float] = None) -> None:
        if not (2 <= req.mol.n_el <= self.weights.n_el_max) or req.mol.n_ions > self.weights.n_ions_max:
            raise ValueError(f"request {req.rid}: molecule outside the served range")
        if req.n_walkers < 1:
            raise ValueError(f"request {req.rid}: n_walkers must be positive")
        if self.reservation(req) > self.budget:
            raise ValueError(f"request {req.rid}: needs more HBM than the whole budget")
        self.pending.append((req, self.now() if t_arrival is None else t_arrival))

    def cancel(self, rid: int) -> bool:
        """Cancels a request that is queued or active; its work already on the GPU completes, its
        state is released at the next quantum of its group and it yields no result."""
        for k, (req, _) in enumerate(self.pending):
            if req.rid == rid:
                del self.pending[k]
                self.cancelled.add(rid)
                return True
        for g in self.groups.values():
            for m in g.members:
                if m.req.rid == rid:
                    m.cancelled = True
                    self.cancelled.add(rid)
                    return True
        return False

    def _admit(self) -> None:
        while self.pending and self.n_active < self.max_active:
            req, t_arr = self.pending[0]
            need = self.reservation(req)
            if self.reserved + need > self.budget:
                break
            self.pending.popleft()
            g = self._group(req.mol.n_el, req.mol.n_up)
            with torch.cuda.stream(g.stream):
                st = _State(req, self, self.now())
            st.t_arrival = t_arr
            g.members.append(st)
            self.reserved += need
            self.peak_reserved = max(self.peak_reserved, self.reserved)
            self.n_active += 1

    def _group(self, n_el: int, n_up: int) -> _Group:
        # packed launches share one architecture, so a group holds one (n_el, n_up) spin state
        g = self.groups.get((n_el, n_up))
        if g is None:
            si = len(self.groups) % len(self.streams)
            g = _Group(n_el, n_up, self.streams[si])
            g.si = si
            self.groups[(n_el, n_up)] = g
        return g

    # ------------------------------------------------------------------ packed launches
    def _pack(self, g: _Group, members: Sequence[_State]) -> Dict[str, torch.Tensor]:
        """Packed tensors of `members` (built on the group's stream). When the member list is the
        one of the last pack, that pack is reused: every member's state is a view into it."""
        key = tuple(id(m) for m in members)
        if g.pack_key == key and g.pack is not None:
            return g.pack
        dev = self.device
        counts = [m.req.n_walkers for m in members]
        B = sum(counts)
        seg_host = np.repeat(np.arange(len(members), dtype=np.int32), counts)
        seeds = np.array([m.seed for m in members], dtype=np.int64)
        p = {
            "r": torch.cat([m.r for m in members]),
            "lp": torch.cat([m.lp for m in members]),
            "age": torch.cat([m.age for m in members]),
            "widx": torch.cat([m.widx for m in members]),
            "scalars": torch.stack([m.scalars for m in members]).contiguous(),
            "R": torch.stack([m.R for m in members]).contiguous(),
            "Z": torch.stack([m.Z for m in members]).contiguous(),
            "seg": torch.from_numpy(seg_host).pin_memory().to(dev, non_blocking=True),
            "seeds": torch.from_numpy(seeds).pin_memory().to(dev, non_blocking=True),
        }
        p["B"] = B
        off = 0
        for i, m in enumerate(members):
            n = m.req.n_walkers
            m.r, m.lp, m.age, m.widx = p["r"][off:off + n], p["lp"][off:off + n], p["age"][off:off + n], \
                p["widx"][off:off + n]
            m.scalars = p["scalars"][i]
            m.R, m.Z = p["R"][i], p["Z"][i]
            m.off = off
            off += n
        g.pack_key, g.pack = key, p
        return p

    def _log_psi(self, g: _Group, p, prm: Params) -> None:
        B = p["B"]
        nbytes = self._ws_bytes(g.n_el, g.n_up, B, 0)
        ws = self._workspace(g.si, nbytes)
        _lib.check(_lib.lib().dw_log_psi_sqr_packed(
            ctypes.byref(prm.c_arch), prm.prec, _ptr(prm.flat), _ptr(prm.prepared), _ptr(p["r"]), B, _ptr(p["R"]),
            _ptr(p["Z"]), len(p["scalars"]), _ptr(p["seg"]), _ptr(p["lp"]), None, _ptr(ws), ws.numel(),
            ctypes.c_void_p(g.stream.cuda_stream)), "dw_log_psi_sqr_packed")
        self.launches += int(_lib.lib().dw_last_launch_count())

    def _mh(self, g: _Group, p, prm: Params, n_steps: int) -> None:
        B = p["B"]
        cfg = self.mcmc.c_config(n_steps, 0, False)
        nbytes = self._ws_bytes(g.n_el, g.n_up, B, 2)
        ws = self._workspace(g.si, nbytes)
        _lib.check(_lib.lib().dw_mcmc_steps_packed(
            ctypes.byref(prm.c_arch), prm.prec, _ptr(prm.flat), _ptr(prm.prepared), _ptr(p["r"]), B, _ptr(p["R"]),
            _ptr(p["Z"]), len(p["scalars"]), _ptr(p["seg"]), _ptr(p["widx"]), _ptr(p["seeds"]), _ptr(p["lp"]),
            _ptr(p["age"]), _ptr(p["scalars"]), ctypes.byref(cfg), _ptr(ws), ws.numel(),
            ctypes.c_void_p(g.stream.cuda_stream)), "dw_mcmc_steps_packed")
        self.launches += int(_lib.lib().dw_last_launch_count())

    def _local_energy(self, g: _Group, p, prm: Params, E: torch.Tensor) -> None:
        B = p["B"]
        nbytes = self._ws_bytes(g.n_el, g.n_up, B, 1)
        ws = self._workspace(g.si, nbytes)
        _lib.check(_lib.lib().dw_local_energy_packed(
            ctypes.byref(prm.c_arch), prm.prec, _ptr(prm.flat), _ptr(prm.prepared), _ptr(p["r"]), B, _ptr(p["R"]),
            _ptr(p["Z"]), len(p["scalars"]), _ptr(p["seg"]), _ptr(E), None, None, _ptr(ws), ws.numel(),
            ctypes.c_void_p(g.stream.cuda_stream)), "dw_local_energy_packed")
        self.launches += int(_lib.lib().dw_last_launch_count())

    def _opt_step(self, g: _Group, m: _State, E: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        """Clipped VMC gradient of the request's own (unpadded) weight copy and its Adam update
        (loss_function.py:75-156 with tanh clipping, center = mean, width = clip_by * std of this batch)."""
        L = _lib.lib()
        mol = m.req.mol
        prm = self.weights.molecule_params(mol)
        nw = m.req.n_walkers
        cs = torch.empty(4, dtype=torch.float64, device=self.device)
        st = torch.empty(3, dtype=torch.float64, device=self.device)
        Ec = torch.empty_like(E)
        _lib.check(L.dw_energy_stats(_ptr(E), nw, _ptr(st), ctypes.c_void_p(g.stream.cuda_stream)), "dw_energy_stats")
        # center / width from this batch: the clipping state of a one-step request starts empty
        center = st[0]
        width = torch.sqrt(st[1]) * self.clip_by
        # the clipping kernel takes host scalars; one small sync per optimisation request
        c_h, w_h = float(center), float(width)
        _lib.check(L.dw_clip_energies(_ptr(E), nw, c_h, max(w_h, 1e-12), self.clip_by, _ptr(Ec), _ptr(cs),
                                      ctypes.c_void_p(g.stream.cuda_stream)), "dw_clip_energies")
        coeff = ((Ec.double() - cs[0]) / nw).float().contiguous()
        Rt = torch.as_tensor(np.asarray(mol.R, np.float32), device=self.device)
        Zt = torch.as_tensor(np.asarray(mol.Z, np.int32), device=self.device)
        grad = torch.zeros_like(prm.flat)
        nbytes = int(L.dw_workspace_bytes(ctypes.byref(prm.c_arch), prm.prec, nw, 3))
        ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        r = m.r.contiguous()
        _lib.check(L.dw_log_psi_sqr_backward(ctypes.byref(prm.c_arch), prm.prec, _ptr(prm.flat), _ptr(prm.prepared),
                                             _ptr(r), nw, _ptr(Rt), _ptr(Zt), _ptr(coeff), _ptr(grad), _ptr(ws),
                                             nbytes, ctypes.c_void_p(g.stream.cuda_stream)),
                   "dw_log_psi_sqr_backward")
        # optax.adam of the VMC step (opt_utils.py:73-76), first update, on a copy of the weights
        new = prm.flat.clone()
        optim.Adam(new, learning_rate=m.req.lr).update_(new, grad)
        return grad, new, cs[0]

    def _issue(self, g: _Group) -> bool:
        """One scheduling quantum of a group on its stream. Returns True if work was issued."""
        if any(m.cancelled for m in g.members):
            for m in [m for m in g.members if m.cancelled]:
                self.reserved -= m.reserved
                self.n_active -= 1
            g.members = [m for m in g.members if not m.cancelled]
            g.pack_key, g.pack = None, None
        if not g.members or len(self.inflight[g.si]) >= self.max_inflight:
            return False
        members = []
        B = 0
        for m in g.members:
            if len(members) >= MAX_SEG or (members and B + m.req.n_walkers > self.max_pack_walkers):
                break
            members.append(m)
            B += m.req.n_walkers
        with torch.cuda.stream(g.stream):
            prm = self.weights.params(g.n_el, g.n_up)     # built on this stream the first time
            fresh = [m for m in members if not m.evaluated]
            if fresh:                               # log psi^2 of newly admitted walkers (mcmc.py:396)
                pf = self._pack(g, fresh)
                self._log_psi(g, pf, prm)
                for m in fresh:
                    m.evaluated = True
            stepping = [m for m in members if m.steps_done < m.req.n_steps]
            if stepping:
                q = min(self.quantum, min(m.req.n_steps - m.steps_done for m in stepping))
                p = self._pack(g, stepping)
                self._mh(g, p, prm, q)
                for m in stepping:
                    m.steps_done += q
            done = [m for m in members if m.steps_done >= m.req.n_steps]
            if done:
                p = self._pack(g, done)
                E = torch.empty(p["B"], dtype=torch.float32, device=self.device)
                self._local_energy(g, p, prm, E)
                stats = torch.empty(len(done), 4, dtype=torch.float64, device=self.device)
                L = _lib.lib()
                for i, m in enumerate(done):
                    m.E = E[m.off:m.off + m.req.n_walkers]
                    _lib.check(L.dw_energy_stats(_ptr(m.E), m.req.n_walkers, _ptr(stats[i]),
                                                 ctypes.c_void_p(g.stream.cuda_stream)), "dw_energy_stats")
                    self.launches += 1
                extra = []
                for i, m in enumerate(done):
                    if m.req.kind == "opt_step":
                        grad, new, loss = self._opt_step(g, m, m.E)
                        m.grad, m.new_params = grad, new
                        stats[i, 3] = loss
                sc = torch.stack([m.scalars for m in done])
                host = torch.empty(stats.numel() * 8 + sc.numel(), dtype=torch.uint8).pin_memory()
                host[:stats.numel() * 8].copy_(stats.view(torch.uint8).view(-1), non_blocking=True)
                host[stats.numel() * 8:].copy_(sc.view(-1), non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(g.stream)
                self.finishing.append((ev, done, host, stats))
                g.members = [m for m in g.members if m not in done]
                g.pack_key, g.pack = None, None
            ev = torch.cuda.Event()
            ev.record(g.stream)
        self.inflight[g.si].append(ev)
        return True

    def _retire(self) -> int:
        """Collects finished requests whose results have reached the host."""
        for q in self.inflight:
            while q and q[0].query():
                q.popleft()
        n = 0
        keep = []
        for ev, done, host, stats in self.finishing:
            if not ev.query():
                keep.append((ev, done, host, stats))
                continue
            t = self.now()
            nb = stats.numel() * 8
            st = host[:nb].view(torch.float64).view(-1, 4).numpy()
            sc_raw = host[nb:].numpy().reshape(len(done), -1)
            for i, m in enumerate(done):
                sc = _lib.DwMcmcScalars.from_buffer_copy(bytes(sc_raw[i]))
                res = Result(m.req.rid, m.n_el, m.req.n_walkers, float(st[i, 0]), float(st[i, 1]), sc.acc_rate,
                             sc.last_acc, sc.stepsize, m.t_arrival, m.t_admit, t)
                if m.req.keep_walkers:
                    res.E_loc, res.r = m.E.clone(), m.r.clone()
                if m.req.kind == "opt_step":
                    res.grad, res.new_params, res.loss = m.grad, m.new_params, float(st[i, 3])
                self.results[m.req.rid] = res
                self.reserved -= m.reserved
                self.n_active -= 1
                n += 1
        self.finishing = keep
        return n

    def poll(self) -> int:
        """Admit, issue one quantum per idle group, retire. Returns the number of requests retired."""
        self._admit()
        for g in list(self.groups.values()):
            self._issue(g)
        return self._retire()

    def busy(self) -> bool:
        return bool(self.pending or self.n_active)

    def drain(self) -> None:
        while self.busy():
            self.poll()
            if self.busy():
                time.sleep(0.0002)

    def run(self, requests: Sequence[Request], realtime: bool = True) -> Dict[int, Result]:
        """Replays the stream: request k is submitted at its arrival time (real time) and the
        loop keeps admitting, packing and retiring until every request is done."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        self.t0 = time.perf_counter()
        k = 0
        while k < len(reqs) or self.busy():
            t = self.now()
            while k < len(reqs) and (not realtime or reqs[k].arrival <= t):
                self.submit(reqs[k], reqs[k].arrival if realtime else t)
                k += 1
            self.poll()
            if realtime and k < len(reqs) and not self.n_active and not self.pending:
                time.sleep(max(0.0, min(0.005, reqs[k].arrival - self.now())))
            elif self.busy():
                time.sleep(0.0002)
        torch.cuda.synchronize(self.device)
        return self.results


def one_at_a_time(weights: SharedWeights, req: Request, precision: str = "plain", stepsize: float = 0.1,
                  mcmc: Optional[MCMCConfig] = None) -> Tuple[float, float, float]:
    """The same request alone through the plain single-geometry API (unpadded model):
    returns (E_mean, E_var, seconds)."""
    from .api import MCMCState, MetropolisHastingsMonteCarlo, energy_stats, local_energy
    torch.cuda.synchronize()
    t = time.perf_counter()
    prm = weights.molecule_params(req.mol, precision)
    st = MCMCState(torch.as_tensor(init_walkers(req.mol, req.n_walkers, seed=req.seed % (2 ** 32)).astype(np.float32),
                                   device=weights.device), req.mol.R, req.mol.Z, seed=req.seed & ((1 << 63) - 1),
                   stepsize=stepsize)
    mh = MetropolisHastingsMonteCarlo(mcmc or MCMCConfig())
    mh.run_mcmc_steps(None, st, prm, req.mol.n_up, req.mol.n_el - req.mol.n_up, n_steps=req.n_steps)
    E = local_energy(prm, None, st.r, req.mol.R, req.mol.Z)
    s = energy_stats(E).cpu().numpy()
    torch.cuda.synchronize()
    return float(s[0]), float(s[1]), time.perf_counter() - t


def summarize(results: Dict[int, Result], requests: Sequence[Request], wall: float) -> Dict[str, float]:
    lat = np.array([results[r.rid].latency for r in requests])
    walkers = sum(r.n_walkers for r in requests)
    return {
        "requests": len(requests),
        "wall_s": wall,
        "p50_latency_s": float(np.percentile(lat, 50)),
        "p99_latency_s": float(np.percentile(lat, 99)),
        "mean_latency_s": float(lat.mean()),
        "requests_per_s": len(requests) / wall,
        "walker_evals_per_s": walkers / wall,
    }


def main(argv=None) -> None:
    """Serving benchmark: replays a seeded request stream in real time and prints one JSON line
    (p50 / p99 latency, throughput, HBM occupancy) with, beside it, the same requests (a seeded
    sample of them) run one at a time through the plain FP32 single-geometry API."""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=8.0, help="Poisson arrival rate, requests per second")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--n-dets", type=int, default=8)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--quantum", type=int, default=5)
    ap.add_argument("--streams", type=int, default=4)
    ap.add_argument("--baseline-sample", type=int, default=40,
                    help="requests of the stream (seeded sample) timed one at a time in the plain form; 0 = skip")
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    torch.cuda.init()
    reqs = stream_requests(args.requests, args.rate, args.seed)
    w = SharedWeights(n_dets=args.n_dets, seed=args.seed, precision="mixed")
    # warm-up: build every electron count's weights and workspaces once, outside the timed stream
    warm = ServingEngine(w, hbm_budget_bytes=args.budget_gb * 1e9, quantum=args.quantum, n_streams=args.streams)
    seen = {}
    for q in reqs:
        seen.setdefault(q.mol.n_el, q)
    for q in seen.values():
        warm.submit(Request(-1 - q.rid, q.mol, 256, n_steps=args.quantum, seed=1))
    warm.drain()
    torch.cuda.synchronize()
    eng = ServingEngine(w, hbm_budget_bytes=args.budget_gb * 1e9, quantum=args.quantum, n_streams=args.streams)
    eng.streams, eng.ws = warm.streams, warm.ws     # same streams, so the workspaces stay stream-ordered
    torch.cuda.reset_peak_memory_stats()
    base_alloc = torch.cuda.memory_allocated()
    t = time.perf_counter()
    res = eng.run(reqs, realtime=True)
    wall = time.perf_counter() - t
    out = summarize(res, reqs, wall)
    out.update({
        "metric": "serving stream: p50/p99 latency, walker-evals/s (walker x (n_steps MH + E_L))",
        "arrival_rate_per_s": args.rate,
        "n_dets": args.n_dets,
        "precision": "mixed (split-BF16 tensor-core GEMMs, FP64 LU / trace / reductions)",
        "hbm_budget_gb": args.budget_gb,
        "hbm_peak_reserved_gb": eng.peak_reserved / 1e9,
        "hbm_peak_allocated_gb": torch.cuda.max_memory_allocated() / 1e9,
        "hbm_allocated_before_gb": base_alloc / 1e9,
        "kernel_launches": eng.launches,
        "mean_n_el": float(np.mean([q.mol.n_el for q in reqs])),
        "mean_walkers": float(np.mean([q.n_walkers for q in reqs])),
        "E_mean_finite": int(sum(np.isfinite(r.E_mean) for r in res.values())),
    })
    if args.baseline_sample > 0:
        rng = np.random.default_rng(args.seed + 1)
        idx = rng.choice(len(reqs), size=min(args.baseline_sample, len(reqs)), replace=False)
        secs, walkers = 0.0, 0
        one_at_a_time(w, reqs[int(idx[0])], "plain")           # warm-up
        for k in idx:
            _, _, s = one_at_a_time(w, reqs[int(k)], "plain")
            secs += s
            walkers += reqs[int(k)].n_walkers
        tot_walkers = sum(q.n_walkers for q in reqs)
        out["one_at_a_time_plain"] = {
            "sample_requests": int(len(idx)),
            "walker_evals_per_s": walkers / secs,
            "est_wall_s_full_stream": secs * tot_walkers / walkers,
        }
        out["speedup_vs_one_at_a_time_plain"] = out["walker_evals_per_s"] / (walkers / secs)
    line = json.dumps(out)
    print(line)
    if args.out:
        with open(args.out, "w") as f:
            f.write(line + "\n")


if __name__ == "__main__":
    main()
