"""GPU tests of the mixed form's tail re-evaluation (guard.cu) at the contract shapes.

* Walkers the guard re-evaluates get exactly the E_L, log psi^2 and gradient of the FP32 network
  with FP64 determinant algebra (DW_PRECISION_FP32_DET64), which is per-walker independent, so the
  result does not depend on the batch; beyond the capacity the largest predicted errors go first.
* Walkers it keeps stay within the error model of the mixed form: |E - E_FP64| at most 2e-4 of the
  largest magnitude the kinetic term cancels (reported per walker by the combine kernel).
* Over the batch the mean E_L of the guarded mixed form is within 0.5 mHa of the FP64 form.
* A re-evaluated walker's result is the same alone and inside a larger batch (bit for bit).
"""
import ctypes

import numpy as np
import pytest
import torch

from deeperwin_gb300 import _lib, api, arch as A, params as P

pytestmark = pytest.mark.gpu


def _unguarded(prm, r, R, Z):
    """Mixed-form E_L and error scales without the re-evaluation (instrumentation entry)."""
    L = _lib.lib()
    B = r.shape[0]
    E = torch.empty(B, device="cuda")
    lp = torch.empty(B, device="cuda")
    sc = torch.empty(B, 3, device="cuda")
    nb = L.dw_workspace_bytes(ctypes.byref(prm.c_arch), prm.prec, B, 1)
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    _lib.check(L.dw_debug_local_energy_scales(ctypes.byref(prm.c_arch), prm.prec, api._ptr(prm.flat),
                                              api._ptr(prm.prepared), api._ptr(r), B, api._ptr(R), api._ptr(Z),
                                              api._ptr(E), api._ptr(lp), api._ptr(sc), api._ptr(ws), nb,
                                              api._stream()), "dw_debug_local_energy_scales")
    return E, sc


def _guard_stats(reset=True):
    v = [ctypes.c_int64() for _ in range(3)]
    _lib.check(_lib.lib().dw_guard_stats(*[ctypes.byref(x) for x in v], int(reset)), "dw_guard_stats")
    return [x.value for x in v]


def _equilibrated(mol, K, B, steps, seed=0):
    a = A.arch_for(mol, K)
    prm = api.Params.from_dict(a, P.init_params(a, seed), "mixed")
    st = api.MCMCState.initialize_around_nuclei(B, mol, seed=seed)
    st.scalars[:] = torch.frombuffer(bytearray(bytes(_lib.DwMcmcScalars(0.0, 0.0, 0.1, 0, 0, 0))),
                                     dtype=torch.uint8).cuda()
    if steps:
        api.MetropolisHastingsMonteCarlo(api.MCMCConfig(stepsize_update_interval=100)).run_mcmc_steps(
            None, st, prm, a.n_up, a.n_dn, None, n_steps=steps)
    return a, prm, st


THRESHOLD = 2000.0      # re-evaluation above this cancelled magnitude (kGuardTol / kGuardRel)


def test_guarded_mixed_energy_against_fp64(cuda):
    """C2H4-shaped molecule at the differentiation form's shape (16 electrons, 32 determinants),
    1,024 walkers after 30 Metropolis-Hastings steps from the initial configuration."""
    a, prm, st = _equilibrated(A.c2h4_shaped(), 32, 1024, 30)
    spin = (a.n_up, a.n_dn)
    _guard_stats(reset=True)
    E, lp, g = api.local_energy(prm, spin, st.r, st.R, st.Z, return_grad=True)
    walkers, flagged, overflow = _guard_stats(reset=True)
    cap = 1024 // 32
    assert walkers == 1024 and overflow == flagged - min(flagged, cap)
    E_u, sc = _unguarded(prm, st.r, st.R, st.Z)
    E_d, lp_d, g_d = api.local_energy(prm.with_precision("fp32_det64"), spin, st.r, st.R, st.Z, return_grad=True)
    E64 = api.local_energy(prm.with_precision("fp64"), spin, st.r, st.R, st.Z)
    re = (E != E_u).cpu().numpy()                      # walkers the guard replaced
    assert 0 < re.sum() <= min(flagged, cap)
    key = sc.double().cpu().numpy()[:, :2].max(axis=1)
    assert set(np.nonzero(re)[0]) <= set(np.argsort(-key)[:min(flagged, cap)].tolist())
    E, E64, E_u = (x.double().cpu().numpy() for x in (E, E64, E_u))
    # replaced walkers carry the results of the FP32 network with FP64 determinants bit for bit
    np.testing.assert_array_equal(E[re], E_d.double().cpu().numpy()[re])
    np.testing.assert_array_equal(lp.cpu().numpy()[re], lp_d.cpu().numpy()[re])
    np.testing.assert_array_equal(g.cpu().numpy()[re], g_d.cpu().numpy()[re])
    # kept walkers below the threshold follow the error model: |dE| <= 5e-4 of the largest
    # cancelled magnitude (measured at most 2.9e-4 of it)
    low = (~re) & (key <= THRESHOLD)
    assert np.all(np.abs(E[low] - E64[low]) <= 5e-4 * key[low]), np.max(np.abs(E[low] - E64[low]) / key[low])
    # the mean over the batch within 0.5 mHa of the FP64 form
    assert abs(E.mean() - E64.mean()) <= 5e-4, (E.mean() - E64.mean(), E_u.mean() - E64.mean(), flagged)


def test_guard_takes_the_largest_predicted_errors_beyond_capacity(cuda):
    """The 40-electron, 64-determinant random molecule, where most walkers exceed the threshold:
    the re-evaluated walkers (the capacity, 16 of 96 here) are those with the largest predicted
    errors and get the re-evaluated results; the others keep the mixed form's values."""
    a, prm, st = _equilibrated(A.scale_molecule(7), 64, 96, 3)
    spin = (a.n_up, a.n_dn)
    _guard_stats(reset=True)
    E = api.local_energy(prm, spin, st.r, st.R, st.Z)
    walkers, flagged, overflow = _guard_stats(reset=True)
    E_u, sc = _unguarded(prm, st.r, st.R, st.Z)
    E_d = api.local_energy(prm.with_precision("fp32_det64"), spin, st.r, st.R, st.Z)
    re = (E != E_u).cpu().numpy()
    key = sc.cpu().numpy()[:, :2].max(axis=1)
    selected = min(flagged, 16)
    assert walkers == 96 and overflow == flagged - selected
    assert flagged > 0 and re.sum() <= selected
    np.testing.assert_array_equal(E.cpu().numpy()[re], E_d.cpu().numpy()[re])
    top = np.argsort(-key)[:selected]
    assert set(np.nonzero(re)[0]) <= set(top.tolist())


def test_guarded_walker_same_alone_and_in_batch(cuda):
    """A replaced walker gets the same bits alone; a walker below the threshold keeps its mixed
    value up to the mixed form's batch-size rounding."""
    a, prm, st = _equilibrated(A.c2h4_shaped(), 8, 256, 10, seed=3)
    spin = (a.n_up, a.n_dn)
    E_all = api.local_energy(prm, spin, st.r, st.R, st.Z)
    E_u, sc = _unguarded(prm, st.r, st.R, st.Z)
    key = sc[:, :2].max(dim=1).values
    replaced = E_all != E_u
    picks = torch.nonzero(replaced).flatten()[:3].tolist() + torch.nonzero(key <= THRESHOLD).flatten()[:3].tolist()
    assert picks
    for b in picks:
        E1 = api.local_energy(prm, spin, st.r[b:b + 1], st.R, st.Z)
        if replaced[b]:
            assert torch.equal(E1[0], E_all[b]), b          # independent of the batch
        else:
            torch.testing.assert_close(E1[0], E_all[b], rtol=1e-6, atol=1e-5)
