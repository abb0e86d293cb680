"""Continuous-batching serving loop on the GPU.

* packed launches (walkers of several geometries with equal n_el, ions padded with Z = 0) match
  the FP64 oracle on each molecule's own unpadded model: E_L within 1e-4 S for both forms, S as
  in test_gpu_parity (the plain FP32 form reaches 5.4e-5 S on a BH walker 0.67 bohr from the
  boron nucleus, padded or not: FP32 cancellation in the Laplacian, not the padding); log psi^2
  within 1e-5 relative + 1e-4 (plain) and 5e-4 relative + 1e-3 (mixed: the split-BF16 operands
  carry about 2^-17 relative rounding, and a walker with log psi^2 = -47 comes out 2e-4
  relative off);
* a chain in a packed MCMC launch follows exactly the trajectory of the same chain run alone
  through dw_mcmc_steps (bitwise);
* every request gives bitwise the same walkers, E_L, mean and variance alone and in a mix whose
  packs change while it runs (arrivals between quanta, other electron counts on other streams);
* admission keeps the reserved HBM within the budget; malformed, over-budget and cancelled
  requests are handled on the host;
* an optimisation-step request returns the clipped VMC gradient of its weight copy.
"""
import ctypes

import numpy as np
import pytest
import torch

from deeperwin_gb300 import _lib, api, serve, vmc
from deeperwin_gb300.arch import Molecule, init_walkers
from oracle import dpe4 as O

pytestmark = pytest.mark.gpu


def _mols6():
    a = Molecule(R=np.array([[0.0, 0, 0], [1.6, 0, 0], [3.2, 0.4, 0], [4.8, 0, 0.3], [6.4, 0, 0], [8.0, 0.5, 0]]),
                 Z=np.ones(6, np.int64), n_el=6, n_up=3, name="H6")
    b = Molecule(R=np.array([[0.0, 0, 0], [2.5, 0.3, 0], [-1.2, 2.0, 0.2], [0.4, -2.2, 1.0]]),
                 Z=np.array([3, 1, 1, 1]), n_el=6, n_up=3, name="LiH3")
    c = Molecule(R=np.array([[0.0, 0, 0], [2.2, 0, 0.5]]), Z=np.array([5, 1]), n_el=6, n_up=3, name="BH")
    return [a, b, c]


def _others():
    lih = Molecule(R=np.array([[0.0, 0, 0], [3.0, 0, 0]]), Z=np.array([3, 1]), n_el=4, n_up=2, name="LiH")
    h2 = Molecule(R=np.array([[0.0, 0, 0], [1.4, 0, 0]]), Z=np.array([1, 1]), n_el=2, n_up=1, name="H2")
    return [lih, h2]


@pytest.fixture(scope="module")
def weights(cuda):
    return serve.SharedWeights(n_dets=4, seed=3, precision="mixed")


def _packed_local_energy(prm, rs, mols, n_ions_max):
    counts = [len(r) for r in rs]
    r = torch.as_tensor(np.concatenate(rs).astype(np.float32), device="cuda").contiguous()
    geo = [serve.padded_geometry(m, n_ions_max) for m in mols]
    R = torch.as_tensor(np.stack([g[0] for g in geo]), device="cuda").contiguous()
    Z = torch.as_tensor(np.stack([g[1] for g in geo]), device="cuda").contiguous()
    seg = torch.as_tensor(np.repeat(np.arange(len(mols), dtype=np.int32), counts), device="cuda")
    B = r.shape[0]
    E = torch.empty(B, device="cuda")
    lp = torch.empty(B, device="cuda")
    L = _lib.lib()
    nb = L.dw_workspace_bytes(ctypes.byref(prm.c_arch), prm.prec, B, 1)
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    _lib.check(L.dw_local_energy_packed(ctypes.byref(prm.c_arch), prm.prec, api._ptr(prm.flat), api._ptr(prm.prepared),
                                        api._ptr(r), B, api._ptr(R), api._ptr(Z), len(mols), api._ptr(seg),
                                        api._ptr(E), api._ptr(lp), None, api._ptr(ws), nb, api._stream()),
               "dw_local_energy_packed")
    return E.cpu().numpy().astype(np.float64), lp.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("prec,tol,lp_rtol,lp_atol", [("fp32", 1e-4, 1e-5, 1e-4), ("mixed", 1e-4, 5e-4, 1e-3)])
def test_packed_local_energy_matches_oracle(weights, prec, tol, lp_rtol, lp_atol):
    mols = _mols6()
    rs = [init_walkers(m, 3, seed=20 + k) for k, m in enumerate(mols)]
    prm = weights.params(6, 3, prec)
    E, lp = _packed_local_energy(prm, rs, mols, weights.n_ions_max)
    off = 0
    for m, r in zip(mols, rs):
        a = weights.arch(m.n_el, m.n_up, m.n_ions)
        p = O.tparams(weights.slice(m.n_el, m.n_up, m.n_ions))
        E_ref, lp_ref, g, lap = O.local_energy(p, a, r, m.R, m.Z)
        S = 0.25 * np.abs(lap.numpy()) + 0.125 * (g.numpy() ** 2).sum(-1) + \
            np.abs(O.potential_energy(r, m.R, m.Z).numpy())
        n = len(r)
        assert np.all(np.abs(E[off:off + n] - E_ref.numpy()) <= tol * S), (m.name, E[off:off + n], E_ref)
        np.testing.assert_allclose(lp[off:off + n], lp_ref.numpy(), rtol=lp_rtol, atol=lp_atol)
        off += n


def test_packed_log_psi_equals_single_geometry_launch(weights):
    """A walker's log psi^2 in a packed launch equals the single-geometry launch of its padded model."""
    mols = _mols6()
    prm = weights.params(6, 3, "mixed")
    rs = [init_walkers(m, 50 + 7 * k, seed=k) for k, m in enumerate(mols)]
    r = torch.as_tensor(np.concatenate(rs).astype(np.float32), device="cuda")
    geo = [serve.padded_geometry(m) for m in mols]
    R = torch.as_tensor(np.stack([g[0] for g in geo]), device="cuda").contiguous()
    Z = torch.as_tensor(np.stack([g[1] for g in geo]), device="cuda").contiguous()
    seg = torch.as_tensor(np.repeat(np.arange(3, dtype=np.int32), [len(x) for x in rs]), device="cuda")
    B = r.shape[0]
    lp = torch.empty(B, device="cuda")
    L = _lib.lib()
    nb = L.dw_workspace_bytes(ctypes.byref(prm.c_arch), prm.prec, B, 0)
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    _lib.check(L.dw_log_psi_sqr_packed(ctypes.byref(prm.c_arch), prm.prec, api._ptr(prm.flat), api._ptr(prm.prepared),
                                       api._ptr(r), B, api._ptr(R), api._ptr(Z), 3, api._ptr(seg), api._ptr(lp), None,
                                       api._ptr(ws), nb, api._stream()), "dw_log_psi_sqr_packed")
    off = 0
    for k, x in enumerate(rs):
        _, lp1 = api.log_psi_sqr(prm, 3, 3, x, geo[k][0], geo[k][1])
        assert torch.equal(lp[off:off + len(x)], lp1), k
        off += len(x)


def _requests(n_steps=4, keep=True):
    mols = _mols6() + _others()
    return [serve.Request(k, m, 40 + 13 * k, n_steps=n_steps, seed=1000 + 17 * k, keep_walkers=keep)
            for k, m in enumerate(mols)]


def test_packed_chain_equals_single_chain(weights):
    """Engine chain (log psi pack, then 2 + 2 packed MH steps in a mix) == dw_mcmc_steps alone."""
    reqs = _requests()
    eng = serve.ServingEngine(weights, quantum=2, n_streams=2)
    for q in reqs:
        eng.submit(q)
    eng.drain()
    torch.cuda.synchronize()
    for q in reqs[:3]:
        m = q.mol
        prm = weights.params(m.n_el, m.n_up)
        Rp, Zp = serve.padded_geometry(m)
        st = api.MCMCState(torch.as_tensor(init_walkers(m, q.n_walkers, seed=q.seed % 2 ** 32).astype(np.float32),
                                           device="cuda"), Rp, Zp, seed=q.seed, stepsize=eng.stepsize)
        api.MetropolisHastingsMonteCarlo(eng.mcmc).run_mcmc_steps(None, st, prm, m.n_up, m.n_el - m.n_up,
                                                                  n_steps=q.n_steps)
        res = eng.results[q.rid]
        assert torch.equal(st.r, res.r), q.rid
        assert st.step_nr == q.n_steps
        assert abs(st.acc_rate - res.acc_rate) == 0.0


def test_alone_equals_mix(weights):
    reqs = _requests()
    alone = {}
    for q in reqs:
        eng = serve.ServingEngine(weights, quantum=2, n_streams=1)
        eng.submit(q)
        eng.drain()
        alone[q.rid] = eng.results[q.rid]
    # the mix: three requests start, the others arrive after the first quantum has been issued,
    # so the packs change while the first ones run
    eng = serve.ServingEngine(weights, quantum=2, n_streams=3)
    for q in reqs[:3]:
        eng.submit(q)
    eng.poll()
    for q in reqs[3:]:
        eng.submit(q)
    eng.drain()
    torch.cuda.synchronize()
    assert eng.launches > 0
    for q in reqs:
        a, b = alone[q.rid], eng.results[q.rid]
        assert torch.equal(a.r, b.r), q.rid
        assert torch.equal(a.E_loc, b.E_loc), q.rid
        assert a.E_mean == b.E_mean and a.E_var == b.E_var and a.acc_rate == b.acc_rate
        assert np.isfinite(b.E_mean)


def test_admission_budget_and_host_faults(weights):
    reqs = _requests(n_steps=2, keep=False)
    probe = serve.ServingEngine(weights)
    need = max(probe.reservation(q) for q in reqs)
    eng = serve.ServingEngine(weights, hbm_budget_bytes=2.2 * need, quantum=1, n_streams=2)
    # malformed requests are rejected on the host
    big = Molecule(R=np.zeros((1, 3)), Z=np.array([8]), n_el=40, n_up=20)
    with pytest.raises(ValueError):
        eng.submit(serve.Request(99, big, 16))
    with pytest.raises(ValueError):
        eng.submit(serve.Request(98, reqs[0].mol, 0))
    tiny = serve.ServingEngine(weights, hbm_budget_bytes=1e3)
    with pytest.raises(ValueError):
        tiny.submit(reqs[0])
    for q in reqs:
        eng.submit(q)
    assert eng.cancel(reqs[-1].rid)
    eng.poll()
    assert eng.peak_reserved <= eng.budget
    assert len(eng.pending) > 0              # the budget holds requests back
    eng.drain()
    assert eng.peak_reserved <= eng.budget
    assert set(eng.results) == {q.rid for q in reqs[:-1]}
    assert eng.reserved == pytest.approx(0.0, abs=1.0) and eng.n_active == 0


def test_opt_step_request_gradient(weights):
    m = _mols6()[1]
    q = serve.Request(0, m, 64, n_steps=2, kind="opt_step", seed=5, keep_walkers=True, lr=1e-2)
    eng = serve.ServingEngine(weights, quantum=2)
    eng.submit(q)
    eng.drain()
    res = eng.results[0]
    prm = weights.molecule_params(m)
    E = res.E_loc.double()
    mean, std = E.mean(), E.var(unbiased=False).sqrt()
    w = 5.0 * std
    Ec = mean + torch.tanh((E - mean) / w) * w
    coeff = ((Ec - Ec.mean()) / len(E)).float()
    g = vmc.log_psi_sqr_backward(prm, res.r, m.R, m.Z, coeff)
    torch.testing.assert_close(res.grad, g, rtol=1e-3, atol=1e-4 * g.abs().max().item())
    # first Adam update from a fresh state: theta - lr g / (|g| + eps)
    gd = res.grad.double()
    torch.testing.assert_close(res.new_params.double(), prm.flat.double() - 1e-2 * gd / (gd.abs() + 1e-8),
                               rtol=0, atol=2e-6)
    assert res.loss == pytest.approx(float(Ec.mean()), rel=1e-6)


def test_equal_electron_count_different_spin_states(weights):
    """Requests with the same n_el but different n_up run in separate groups: each result equals
    the request alone, and equals one_at_a_time's evaluation of its own spin state."""
    h6 = _mols6()[0]
    h6_open = Molecule(R=h6.R, Z=h6.Z, n_el=6, n_up=4, name="H6_triplet")
    reqs = [serve.Request(0, h6, 48, n_steps=3, seed=7, keep_walkers=True),
            serve.Request(1, h6_open, 40, n_steps=3, seed=9, keep_walkers=True)]
    alone = {}
    for q in reqs:
        eng = serve.ServingEngine(weights, quantum=2, n_streams=1)
        eng.submit(q)
        eng.drain()
        alone[q.rid] = eng.results[q.rid]
    eng = serve.ServingEngine(weights, quantum=2, n_streams=1)
    for q in reqs:
        eng.submit(q)
    eng.drain()
    torch.cuda.synchronize()
    assert sorted(eng.groups) == [(6, 3), (6, 4)]
    for q in reqs:
        a, b = alone[q.rid], eng.results[q.rid]
        assert torch.equal(a.r, b.r) and torch.equal(a.E_loc, b.E_loc), q.rid
    # the open-shell result is that of its own (n_up = 4) model
    prm = weights.params(6, 4)
    Rp, Zp = serve.padded_geometry(h6_open)
    E = api.local_energy(prm, (4, 2), eng.results[1].r, Rp, Zp)
    torch.testing.assert_close(E, eng.results[1].E_loc, rtol=1e-5, atol=1e-5)
