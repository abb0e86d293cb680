"""GPU tests of the forces on the nuclei (dw_forces, hamiltonian.py:293-338) against the oracle's
restatement, with and without antithetic sampling; FP64 arithmetic on float32 walkers, so the
oracle runs at the float32-rounded positions and the bound is FP64 summation error (1e-9
relative to the largest per-walker force)."""
import numpy as np
import pytest
import torch

from deeperwin_gb300 import api, arch as A, params as P
from oracle import dpe4 as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("antithetic", [False, True])
@pytest.mark.parametrize("mol_fn,K", [(A.lih, 4), (A.c2h4_shaped, 2)])
def test_forces_match_oracle(cuda, mol_fn, K, antithetic):
    mol = mol_fn()
    a = A.arch_for(mol, K)
    p = {k: v.astype(np.float32).astype(np.float64) for k, v in P.init_params(a, 2, bias_std=0.1,
                                                                             envelope_jitter=0.1).items()}
    params = api.Params.from_dict(a, p, "fp64")
    r = A.init_walkers(mol, 64, seed=3).astype(np.float32)
    _, lp = api.log_psi_sqr(params, a.n_up, a.n_dn, r, mol.R, mol.Z)
    F, pw = api.calculate_forces(params, r, mol.R, mol.Z, lp, R_cut=0.1, R_core=0.5,
                                 use_antithetic_sampling=antithetic, per_walker=True)
    ref = O.forces(O.tparams(p), a, r.astype(np.float64), mol.R.astype(np.float32).astype(np.float64), mol.Z,
                   lp.double().cpu().numpy(), 0.1, 0.5, antithetic).numpy()
    scale = np.abs(pw.cpu().numpy()).max()
    # antithetic: the mirror images are formed in float32 and their weights exp(log psi^2(mirror) -
    # log psi^2) inherit the float32 rounding of both log psi^2 values (about 5e-6 at |log psi^2| ~ 80)
    rtol, atol = (1e-4, 1e-5 * scale) if antithetic else (1e-6, 1e-9 * scale + 1e-9)
    np.testing.assert_allclose(F.cpu().numpy(), ref, rtol=rtol, atol=atol)
    # F minus the batch mean of the per-walker forces is the nucleus-nucleus repulsion
    R64 = mol.R.astype(np.float32).astype(np.float64)
    Z = np.asarray(mol.Z, np.float64)
    d = R64[:, None] - R64[None]
    dist = np.linalg.norm(d, axis=-1, keepdims=True) + 1e-8
    Zm = Z[:, None] * Z[None] - np.diag(Z ** 2)
    ion = (d * Zm[..., None] / dist ** 3).sum(1)
    np.testing.assert_allclose(F.cpu().numpy() - pw.mean(0).cpu().numpy(), ion, rtol=1e-9, atol=1e-9 * scale + 1e-9)


def test_antithetic_mirror_weights_are_one_for_symmetric_walkers(cuda):
    """Walkers with no electron within R_core of a nucleus are their own mirror image: the
    antithetic estimate equals the direct one."""
    mol = A.h_chain(4, 3.0)
    a = A.arch_for(mol, 2)
    params = api.Params.from_dict(a, P.init_params(a, 0), "fp32")
    r = (A.init_walkers(mol, 32, seed=1) + np.array([0.0, 0.0, 1.2])).astype(np.float32)   # off the chain axis
    _, lp = api.log_psi_sqr(params, a.n_up, a.n_dn, r, mol.R, mol.Z)
    far = np.linalg.norm(r[:, :, None, :] - mol.R[None, None], axis=-1).min(-1).min(-1) > 0.5
    r = r[far]
    lp = lp[torch.as_tensor(far, device="cuda")]
    F0 = api.calculate_forces(params, r, mol.R, mol.Z, lp, use_antithetic_sampling=False)
    F1 = api.calculate_forces(params, r, mol.R, mol.Z, lp, use_antithetic_sampling=True)
    torch.testing.assert_close(F0, F1, rtol=1e-6, atol=1e-9)
