"""GPU tests of the Metropolis-Hastings proposal rules (mcmc.py:175-310) against the oracle.

One step of each rule through dw_mcmc_steps on LiH walkers; the oracle replays the same Philox
draws (tests/philox_ref.py) through its restatement of the reference's proposal functions, spin
swap / flip and acceptance with the proposal ratio. The wavefunction is evaluated in the FP64 form
so that the acceptance decisions compare exactly wherever log U is not within 1e-5 of the
acceptance exponent.
"""
import numpy as np
import pytest
import torch

from deeperwin_gb300 import api, arch as A, params as P
from oracle import dpe4 as O
from tests import philox_ref

pytestmark = pytest.mark.gpu

SEED = 4321


@pytest.mark.parametrize("kind,swap,flip", [("normal", 0.0, 0.0), ("cauchy", 0.0, 0.0), ("normal_one_el", 0.0, 0.0),
                                            ("local", 0.0, 0.0), ("local_one_el", 0.0, 0.0),
                                            ("langevin", 0.0, 0.0), ("normal", 0.5, 0.0), ("normal", 0.0, 0.5),
                                            ("langevin", 0.5, 0.5)])
def test_proposal_step_matches_oracle(cuda, kind, swap, flip):
    mol = A.lih()
    a = A.arch_for(mol, 4)
    p = {k: v.astype(np.float32).astype(np.float64) for k, v in P.init_params(a, 0, bias_std=0.1,
                                                                             envelope_jitter=0.1).items()}
    params = api.Params.from_dict(a, p, "fp64")
    B, step0, stepsize = 128, 3, 0.15
    state = api.MCMCState.initialize_around_nuclei(B, mol, seed=5)
    state.seed = SEED
    state.scalars[:] = torch.frombuffer(bytearray(bytes(api._lib.DwMcmcScalars(0.0, 0.0, stepsize, step0, 0, 0))),
                                        dtype=torch.uint8).cuda()
    cfg = api.MCMCConfig(max_age=50, stepsize_update_interval=1000, proposal=kind, p_spin_swap=swap,
                         p_spin_flip=flip)
    r0 = state.r.cpu().numpy().astype(np.float64)
    api.MetropolisHastingsMonteCarlo(cfg).run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=1)
    torch.cuda.synchronize()
    # replay: the proposal of step counter step0 with the chain's step size
    noise = philox_ref.proposal_noise(SEED, B, a.n_el, step0).astype(np.float64)
    cu = philox_ref.cauchy_uniforms(SEED, B, a.n_el, step0).astype(np.float64)
    lo, hi = (0.2, 2.0) if kind == "langevin" else (0.1, 1.0)
    r_prop, lq = O.propose(kind, r0, mol.R, mol.Z, np.float32(stepsize), step0, noise, cauchy_u=cu, r_min=lo, r_max=hi)
    su = philox_ref.spin_uniforms(SEED, B, step0).astype(np.float64)
    nh = a.n_el // 2
    if swap:
        iu = np.minimum((su[:, 1] * nh).astype(int), nh - 1)
        idn = nh + np.minimum((su[:, 2] * (a.n_el - nh)).astype(int), a.n_el - nh - 1)
        r_prop = O.spin_swap(r_prop, nh, swap, su[:, 0], iu, idn)
    if flip:
        r_prop = O.spin_flip(r_prop, flip, su[:, 3])
    r_prop = r_prop.numpy()
    tp = O.tparams(p)
    lp0 = O.log_psi_sqr(tp, a, r0, mol.R, mol.Z)[1].numpy()
    lp1 = O.log_psi_sqr(tp, a, r_prop, mol.R, mol.Z)[1].numpy()
    U = philox_ref.accept_uniform(SEED, B, step0).astype(np.float64)
    expo = lp1 - lp0 + lq.numpy()
    acc_ref = np.exp(expo) > U
    clear = np.abs(expo - np.log(U)) > 1e-4
    acc = state.walker_age.cpu().numpy() == 0
    assert clear.sum() > 0.9 * B and 0 < acc.sum() < B
    np.testing.assert_array_equal(acc[clear], acc_ref[clear])
    r1 = state.r.cpu().numpy()
    tol = 1e-5 * np.maximum(1.0, np.abs(r_prop))
    sel = acc & clear
    assert np.all(np.abs(r1[sel] - r_prop[sel]) <= tol[sel]), np.abs(r1[sel] - r_prop[sel]).max()
    np.testing.assert_array_equal(r1[~acc], r0[~acc].astype(np.float32))
    if kind.endswith("one_el"):
        moved = np.abs(r1 - r0.astype(np.float32)).max(-1) > 0
        assert not moved[:, [i for i in range(a.n_el) if i != step0 % a.n_el]].any()


def test_local_proposal_chain_adapts_and_stays_finite(cuda):
    mol = A.c2h4_shaped()
    a = A.arch_for(mol, 4)
    params = api.Params.from_dict(a, P.init_params(a, 1), "mixed")
    state = api.MCMCState.initialize_around_nuclei(512, mol, seed=2)
    cfg = api.MCMCConfig(stepsize_update_interval=2, proposal="langevin", p_spin_swap=0.1)
    api.MetropolisHastingsMonteCarlo(cfg).run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=12)
    torch.cuda.synchronize()
    assert torch.isfinite(state.r).all() and torch.isfinite(state.log_psi_sqr).all()
    assert state.step_nr == 12 and 0.0 < state.acc_rate < 1.0
