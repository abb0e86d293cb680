"""Walker sharding over ranks (no GPU): world_size-2 gloo process groups on CPU run the
cross-rank reductions of deeperwin_gb300.dist, and each result is checked against a
single-process restatement of the reference's pmap semantics over all ranks' walkers:
pmean = plain mean of per-device values (utils/utils.py:28-30), energy statistics
(loss_function.py:94-99), clipping state (:19-30, :60-71), gradients (:141-153, optimizers.py:133),
acceptance-rate EMA (mcmc.py:367-371)."""
import os
import tempfile

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from deeperwin_gb300 import _lib
from deeperwin_gb300 import dist

WORLD = 2
CLIP_BY = 5.0


def _rank_data(rank: int, nan: bool = False):
    """Per-rank walkers: energies (rank 1 has more walkers, and with `nan` a NaN walker) and a
    per-walker gradient matrix J (d log psi^2 / d theta rows) standing in for the backward pass."""
    rng = np.random.default_rng(10 + rank)
    B = 6 if rank == 0 else 9
    E = rng.normal(-2.0 + rank, 0.7, B)
    E[2] += 9.0 * (rank + 1)                      # outliers that the clipping bends
    if nan and rank == 1:
        E[4] = np.nan
    J = rng.standard_normal((B, 5))
    return E, J


def _nanmean(x):
    return np.nanmean(x)


def _nanvar(x):
    return np.nanmean((x - np.nanmean(x)) ** 2)


def _reference_step(clipping_state, from_previous_step):
    """The reference's total_energy + custom JVP under pmap, restated over the two ranks."""
    data = [_rank_data(r) for r in range(WORLD)]
    pmean = lambda vals: float(np.mean(vals))
    E_mean = pmean([_nanmean(E) for E, _ in data])
    E_var = pmean([np.nanmean((E - E_mean) ** 2) for E, _ in data])
    center, width = clipping_state
    if not from_previous_step:
        center, width = E_mean, np.sqrt(E_var) * CLIP_BY
    clipped = [center + np.tanh((E - center) / width) * width for E, _ in data]
    Ec_mean = pmean([_nanmean(c) for c in clipped])
    Ec_var = pmean([np.nanmean((c - Ec_mean) ** 2) for c in clipped])
    # per device: dot(tangents, E_clip - E_mean_clipped) / batch_size, then pmean of the grads
    grads = np.mean([(c - Ec_mean) @ J / len(c) for c, (_, J) in zip(clipped, data)], axis=0)
    return Ec_mean, (Ec_mean, np.sqrt(Ec_var) * CLIP_BY), E_mean, E_var, grads


def _worker(rank, init_file, out_dir, case):
    torch.distributed.init_process_group("gloo", init_method=f"file://{init_file}", rank=rank, world_size=WORLD)
    try:
        res = {}
        if case == "moments":
            E, _ = _rank_data(rank, nan=True)
            m, v = dist.combine_moments(torch.tensor(_nanmean(E)), torch.tensor(_nanvar(E)))
            res = {"mean": float(m), "var": float(v), "world": dist.world()}
        elif case == "scalars":
            # two chains' EMA over steps: local update, then the cross-rank average
            rng = np.random.default_rng(rank)
            s = _lib.DwMcmcScalars(0.3, 0.0, 0.05, 7, 0, 0)
            buf = torch.frombuffer(bytearray(bytes(s)), dtype=torch.uint8).clone()
            accs = []
            for t in range(6):
                x = float(rng.uniform())                      # this rank's accepted fraction
                accs.append(x)
                cur = _lib.DwMcmcScalars.from_buffer_copy(bytes(buf.numpy()))
                cur.acc_rate = 0.9 * cur.acc_rate + 0.1 * x     # what the MH kernel does locally
                cur.last_acc = x
                cur.step_nr += 1
                buf = torch.frombuffer(bytearray(bytes(cur)), dtype=torch.uint8).clone()
                dist.sync_chain_scalars_(buf)
            fin = _lib.DwMcmcScalars.from_buffer_copy(bytes(buf.numpy()))
            res = {"acc_rate": fin.acc_rate, "last_acc": fin.last_acc, "stepsize": fin.stepsize,
                   "step_nr": fin.step_nr, "accs": accs}
        elif case == "mcmc_loop":
            res = _mcmc_loop(rank)
        else:
            from_prev = case == "grad_prev"
            state = (-1.5, 3.0) if from_prev else (0.0, 1e12)
            E, J = _rank_data(rank)
            Et = torch.from_numpy(E)

            def stats_fn(e):
                x = e.numpy()
                return torch.tensor(_nanmean(x)), torch.tensor(_nanvar(x))

            def clip_fn(e, c, w):
                ec = c + torch.tanh((e - c) / w) * w
                x = ec.numpy()
                return ec, torch.tensor(_nanmean(x)), torch.tensor(_nanvar(x))

            Jt = torch.from_numpy(J)
            loss, new_state, aux, grads = dist.sharded_clipped_gradient(
                Et, state, CLIP_BY, from_prev, stats_fn, clip_fn, lambda coeff: coeff @ Jt)
            res = {"loss": float(loss), "state": new_state, "E_mean": float(aux["E_mean"]),
                   "E_var": float(aux["E_var"]), "grads": grads.numpy().tolist()}
        np.save(os.path.join(out_dir, f"{case}_{rank}.npy"), np.array([res], dtype=object))
    finally:
        torch.distributed.destroy_process_group()


def _accept_fraction(rank: int, step: int) -> float:
    return 0.2 + 0.1 * rank + 0.05 * step


def _mcmc_loop(rank: int):
    """api.MetropolisHastingsMonteCarlo.run_mcmc_steps over a stand-in library whose
    dw_mcmc_steps applies the MH kernel's update of the chain scalars (acc_rate EMA with this
    rank's accepted fraction, step_nr + 1) through the scalars pointer it is given."""
    import ctypes
    import types
    from deeperwin_gb300 import api
    from deeperwin_gb300.arch import Arch
    calls = []

    class FakeLib:
        def dw_workspace_bytes(self, *a):
            return 0

        def dw_last_launch_count(self):
            return 2 + (calls[-1][1] if calls else 0)    # stand-in count: 2, plus 1 with re-evaluation

        def dw_mcmc_steps(self, arch, prec, flat, prepared, r, B, R, Z, lp, age, scalars, cfg, ws, nbytes, stream):
            c = cfg._obj
            calls.append((c.n_steps, c.reevaluate))
            S = ctypes.cast(scalars, ctypes.POINTER(_lib.DwMcmcScalars)).contents
            for _ in range(c.n_steps):
                x = _accept_fraction(rank, S.step_nr)
                S.acc_rate = 0.9 * S.acc_rate + 0.1 * x
                S.last_acc = x
                S.step_nr += 1
            return 0

    api._stream = lambda: ctypes.c_void_p(0)
    _lib.lib = lambda: FakeLib()
    a = Arch(n_el=4, n_up=2, n_ions=2, n_dets=2, z_min=1, z_max=3)
    params = types.SimpleNamespace(arch=a, c_arch=_lib.make_arch(a), prec=1, flat=torch.zeros(4),
                                   prepared=torch.zeros(4))
    state = types.SimpleNamespace(r=torch.zeros(8, 4, 3), R=torch.zeros(2, 3), Z=torch.zeros(2, dtype=torch.int32),
                                  log_psi_sqr=torch.zeros(8), walker_age=torch.zeros(8, dtype=torch.int32), seed=rank,
                                  scalars=torch.frombuffer(bytearray(bytes(_lib.DwMcmcScalars(0.5, 0.0, 0.02, 0, 0, 0))),
                                                           dtype=torch.uint8).clone())
    mh = api.MetropolisHastingsMonteCarlo(api.MCMCConfig())
    mh.run_mcmc_steps(None, state, params, 2, 2, None, n_steps=5, reevaluate=True)
    fin = _lib.DwMcmcScalars.from_buffer_copy(bytes(state.scalars.numpy()))
    launches = api.last_launch_count()
    _lib.check(0)                                  # a later library call clears the sum
    return {"calls": calls, "acc_rate": fin.acc_rate, "step_nr": fin.step_nr, "launches": launches,
            "launches_after": api.last_launch_count()}


def _run(case):
    with tempfile.TemporaryDirectory() as d:
        init_file = os.path.join(d, "pg_init")
        mp.spawn(_worker, args=(init_file, d, case), nprocs=WORLD, join=True)
        return [np.load(os.path.join(d, f"{case}_{r}.npy"), allow_pickle=True)[0] for r in range(WORLD)]


def test_single_rank_is_identity():
    assert dist.world() == 1
    t = torch.tensor([1.0, 2.0])
    assert torch.equal(dist.pmean_(t.clone()), t)
    m, v = dist.combine_moments(torch.tensor(2.0), torch.tensor(3.0))
    assert float(m) == 2.0 and float(v) == 3.0


def test_energy_moments_pmean_over_two_ranks():
    out = _run("moments")
    data = [_rank_data(r, nan=True)[0] for r in range(WORLD)]
    E_mean = np.mean([np.nanmean(E) for E in data])
    E_var = np.mean([np.nanmean((E - E_mean) ** 2) for E in data])
    for res in out:
        assert res["world"] == WORLD
        np.testing.assert_allclose(res["mean"], E_mean, rtol=1e-14)
        np.testing.assert_allclose(res["var"], E_var, rtol=1e-13)


def test_acceptance_rate_ema_of_pmean():
    out = _run("scalars")
    acc = 0.3
    for t in range(6):
        acc = 0.9 * acc + 0.1 * np.mean([out[r]["accs"][t] for r in range(WORLD)])
    for res in out:
        np.testing.assert_allclose(res["acc_rate"], acc, rtol=1e-14)
        np.testing.assert_allclose(res["last_acc"], np.mean([o["accs"][-1] for o in out]), rtol=1e-14)
        assert res["step_nr"] == 13 and abs(res["stepsize"] - 0.05) < 1e-9     # other fields untouched


@pytest.mark.parametrize("case", ["grad_prev", "grad_fresh"])
def test_clipped_gradient_over_two_ranks(case):
    from_prev = case == "grad_prev"
    out = _run(case)
    loss, state, E_mean, E_var, grads = _reference_step((-1.5, 3.0) if from_prev else (0.0, 1e12), from_prev)
    for res in out:
        np.testing.assert_allclose(res["loss"], loss, rtol=1e-13)
        np.testing.assert_allclose(res["state"], state, rtol=1e-13)
        np.testing.assert_allclose(res["E_mean"], E_mean, rtol=1e-13)
        np.testing.assert_allclose(res["E_var"], E_var, rtol=1e-13)
        np.testing.assert_allclose(res["grads"], grads, rtol=1e-12, atol=1e-14)
    # every rank ends the step with the same gradient and clipping state
    assert out[0]["grads"] == out[1]["grads"] and out[0]["state"] == out[1]["state"]


def test_mcmc_steps_sync_acceptance_every_step():
    """With two ranks, n MH steps run as n one-step calls (re-evaluation on the first only) and
    the running acceptance rate is the EMA of the per-step mean over ranks (mcmc.py:367-371)."""
    out = _run("mcmc_loop")
    acc = 0.5
    for t in range(5):
        acc = 0.9 * acc + 0.1 * np.mean([_accept_fraction(r, t) for r in range(WORLD)])
    for res in out:
        assert res["calls"] == [(1, 1), (1, 0), (1, 0), (1, 0), (1, 0)]
        assert res["launches"] == 3 + 4 * 2 and res["launches_after"] == 2   # summed over the calls
        assert res["step_nr"] == 5
        np.testing.assert_allclose(res["acc_rate"], acc, rtol=1e-14)


def _single_worker(rank, out_dir):
    res = _mcmc_loop(0)
    np.save(os.path.join(out_dir, "single.npy"), np.array([res], dtype=object))


def test_mcmc_steps_single_rank_one_call():
    """Without a process group the n steps stay one fused call and the scalars are the kernel's."""
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_single_worker, args=(d,), nprocs=1, join=True)
        res = np.load(os.path.join(d, "single.npy"), allow_pickle=True)[0]
    acc = 0.5
    for t in range(5):
        acc = 0.9 * acc + 0.1 * _accept_fraction(0, t)
    assert res["calls"] == [(5, 1)] and res["step_nr"] == 5 and res["launches"] == 3
    np.testing.assert_allclose(res["acc_rate"], acc, rtol=1e-14)
