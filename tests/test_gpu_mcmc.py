"""GPU tests of the fused Metropolis-Hastings step against the oracle (replaying the same
Philox draws) and of the chain bookkeeping (mcmc.py:345-387)."""
import numpy as np
import pytest
import torch

from deeperwin_gb300 import api, arch as A, params as P
from oracle import dpe4 as O
from tests import philox_ref

pytestmark = pytest.mark.gpu


def _setup(prec="fp32", B=64, seed=0):
    mol = A.lih()
    a = A.arch_for(mol, 8)
    p = P.init_params(a, 0, bias_std=0.1, envelope_jitter=0.1)
    params = api.Params.from_dict(a, p, prec)
    state = api.MCMCState.initialize_around_nuclei(B, mol, seed=seed)
    return mol, a, p, params, state


def test_single_step_matches_oracle(cuda):
    mol, a, p, params, state = _setup()
    r0 = state.r.cpu().numpy().astype(np.float64)
    state.seed = 1234
    state.scalars[:] = torch.frombuffer(bytearray(bytes(api._lib.DwMcmcScalars(0.0, 0.0, 0.1, 0, 0, 0))),
                                        dtype=torch.uint8).cuda()
    cfg = api.MCMCConfig(max_age=20, stepsize_update_interval=1000)
    api.MetropolisHastingsMonteCarlo(cfg).run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=1)
    torch.cuda.synchronize()
    B = r0.shape[0]
    noise = philox_ref.proposal_noise(1234, B, a.n_el, 0).astype(np.float64)
    U = philox_ref.accept_uniform(1234, B, 0).astype(np.float64)
    tp = O.tparams(p)
    lp0 = O.log_psi_sqr(tp, a, r0, mol.R, mol.Z)[1].numpy()
    r_prop = (r0.astype(np.float32) + np.float32(0.1) * noise.astype(np.float32)).astype(np.float64)
    lp1 = O.log_psi_sqr(tp, a, r_prop, mol.R, mol.Z)[1].numpy()
    log_ratio = lp1 - lp0
    acc_ref = np.exp(log_ratio) > U
    clear = np.abs(log_ratio - np.log(U)) > 1e-3
    acc = (state.walker_age.cpu().numpy() == 0)
    assert clear.sum() > B * 0.8
    np.testing.assert_array_equal(acc[clear], acc_ref[clear])
    r1 = state.r.cpu().numpy()
    np.testing.assert_allclose(r1[acc], r_prop[acc], rtol=0, atol=2e-5)
    np.testing.assert_array_equal(r1[~acc], r0[~acc].astype(np.float32))
    lp_gpu = state.log_psi_sqr.cpu().numpy()
    np.testing.assert_allclose(lp_gpu[acc], lp1[acc], rtol=1e-5, atol=1e-3)
    np.testing.assert_allclose(lp_gpu[~acc], lp0[~acc], rtol=1e-5, atol=1e-3)
    assert state.step_nr == 1
    assert state.last_acceptance == pytest.approx(acc.mean())
    assert state.acc_rate == pytest.approx(0.1 * acc.mean())


def test_chain_is_reproducible_and_adapts_stepsize(cuda):
    results = []
    for _ in range(2):
        mol, a, p, params, state = _setup("mixed", B=256, seed=3)
        cfg = api.MCMCConfig(max_age=20, stepsize_update_interval=5)
        mh = api.MetropolisHastingsMonteCarlo(cfg)
        mh.run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=60)
        torch.cuda.synchronize()
        results.append((state.r.cpu().clone(), state.log_psi_sqr.cpu().clone(), state.stepsize, state.acc_rate,
                        state.step_nr))
    (r1, l1, s1, a1, n1), (r2, l2, s2, a2, n2) = results
    assert torch.equal(r1, r2) and torch.equal(l1, l2) and s1 == s2 and n1 == n2 == 60
    k = round(np.log(s1 / 1e-2) / np.log(1.05))
    assert s1 == pytest.approx(1e-2 * 1.05 ** k, rel=1e-4)       # multiplicative 1.05 steps from 0.01
    assert 0.0 < a1 < 1.0
    assert torch.isfinite(l1).all()


def test_max_age_forces_acceptance(cuda):
    mol, a, p, params, state = _setup(B=32)
    state.walker_age.fill_(20)
    # tiny stepsize and a log psi^2 of +inf for the current state make every Metropolis test fail
    cfg = api.MCMCConfig(max_age=20, stepsize_update_interval=1000)
    mh = api.MetropolisHastingsMonteCarlo(cfg)
    state.log_psi_sqr.fill_(float("inf"))
    mh.run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=1, reevaluate=False)
    torch.cuda.synchronize()
    assert (state.walker_age == 0).all()
    assert torch.isfinite(state.log_psi_sqr).all()


def test_one_step_calls_reproduce_a_multi_step_call(cuda):
    """n one-step calls (re-evaluation on the first only) give the walkers, log psi^2, ages and
    chain scalars of one n-step call: the noise and the uniforms are keyed by (walker, step
    number), and the accept-only phase updates the step size by the same rule as the fused
    accept / propose phase. The multi-rank loop of run_mcmc_steps relies on this."""
    mol, a, p, params, s1 = _setup("mixed", B=96, seed=3)
    _, _, _, _, s2 = _setup("mixed", B=96, seed=3)
    for s in (s1, s2):
        s.seed = 77
        s.scalars[:] = torch.frombuffer(bytearray(bytes(api._lib.DwMcmcScalars(0.4, 0.0, 0.05, 95, 0, 0))),
                                        dtype=torch.uint8).cuda()
    mh = api.MetropolisHastingsMonteCarlo(api.MCMCConfig(max_age=3, stepsize_update_interval=4))
    mh.run_mcmc_steps(None, s1, params, a.n_up, a.n_dn, None, n_steps=9, reevaluate=True)
    for k in range(9):
        mh.run_mcmc_steps(None, s2, params, a.n_up, a.n_dn, None, n_steps=1, reevaluate=(k == 0))
    torch.cuda.synchronize()
    assert torch.equal(s1.r, s2.r)
    assert torch.equal(s1.log_psi_sqr, s2.log_psi_sqr) and torch.equal(s1.walker_age, s2.walker_age)
    h1, h2 = s1._host_scalars(), s2._host_scalars()
    assert (h1.acc_rate, h1.last_acc, h1.stepsize, h1.step_nr) == (h2.acc_rate, h2.last_acc, h2.stepsize, h2.step_nr)
    assert h1.step_nr == 104 and abs(h1.stepsize - 0.05) > 1e-3   # the step-size rule ran (steps 96, 100, 104)


def test_evaluation_loop(cuda):
    """evaluation.evaluate_wavefunction: burn-in, inter-steps and the FP64 energy mean per epoch
    (optimization/evaluation.py:117-201), summarised with the autocorrelation-corrected sigma."""
    from deeperwin_gb300 import evaluation
    mol, a, p, params, state = _setup("mixed", B=128, seed=5)
    mh = api.MetropolisHastingsMonteCarlo(api.MCMCConfig(n_burn_in=20, n_inter_steps=5))
    hist, summ, st = evaluation.evaluate_wavefunction(params, state, mh, n_epochs=6)
    assert len(hist["E_mean"]) == 6 and np.all(np.isfinite(hist["E_mean"])) and np.all(np.array(hist["E_var"]) >= 0)
    E = api.local_energy(params, (a.n_up, a.n_dn), st.r, st.R, st.Z).double()
    assert abs(hist["E_mean"][-1] - E.mean().item()) <= 1e-9 * max(1.0, abs(E.mean().item()))
    assert st.step_nr == 20 + 6 * 5
    assert summ["E_mean_sigma"] >= 0 and np.isfinite(summ["E_mean_sigma_corr"])
