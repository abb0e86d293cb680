"""GPU tests of the mixed form's tail re-evaluation (guard.cu) at the contract shapes.

* Walkers the guard re-evaluates get exactly the E_L, log psi^2 and gradient of the FP32 network
  with FP64 determinant algebra (DW_PRECISION_FP32_DET64), which is per-walker independent, so the
  result does not depend on the batch; beyond the capacity the largest predicted errors go first.
* Walkers whose cancelled magnitude exceeds 1e5 Ha (the largest first, up to the second tier's
  capacity) get exactly the FP64 form's results.
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


def _guard_stats(reset=True, tier=0):
    v = [ctypes.c_int64() for _ in range(3)]
    _lib.check(_lib.lib().dw_guard_tier_stats(tier, *[ctypes.byref(x) for x in v], int(reset)), "dw_guard_tier_stats")
    return [x.value for x in v]


def _tier1(key, cap1):
    """Walkers of the FP64-form tier: cancelled magnitude above FP64_KEY, the largest first."""
    order = np.argsort(-key, kind="stable")
    return np.array([i for i in order[:cap1] if key[i] > FP64_KEY], dtype=np.int64)


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


THRESHOLD = 1000.0      # re-evaluation above this cancelled magnitude (kGuardTol / kGuardRel)
FP64_KEY = 1.0e5        # FP64-form re-evaluation above this cancelled magnitude (kGuardFp64Key)


def test_guarded_mixed_energy_against_fp64(cuda):
    """C2H4-shaped molecule at the differentiation form's shape (16 electrons, 32 determinants),
    1,024 walkers after 30 Metropolis-Hastings steps from the initial configuration."""
    a, prm, st = _equilibrated(A.c2h4_shaped(), 32, 1024, 30)
    spin = (a.n_up, a.n_dn)
    _guard_stats(reset=True)
    _guard_stats(reset=True, tier=1)
    E, lp, g = api.local_energy(prm, spin, st.r, st.R, st.Z, return_grad=True)
    walkers1, flagged1, overflow1 = _guard_stats(reset=True, tier=1)
    walkers, flagged, overflow = _guard_stats(reset=True)
    cap, cap1 = 1024 // 32, 8
    assert walkers == 1024 and overflow == flagged - min(flagged, cap)
    E_u, sc = _unguarded(prm, st.r, st.R, st.Z)
    E_d, lp_d, g_d = api.local_energy(prm.with_precision("fp32_det64"), spin, st.r, st.R, st.Z, return_grad=True)
    E64, lp64, g64 = api.local_energy(prm.with_precision("fp64"), spin, st.r, st.R, st.Z, return_grad=True)
    re = (E != E_u).cpu().numpy()                      # walkers the guard replaced
    assert 0 < re.sum() <= min(flagged, cap)
    key = sc.double().cpu().numpy()[:, :2].max(axis=1)
    assert set(np.nonzero(re)[0]) <= set(np.argsort(-key)[:min(flagged, cap)].tolist())
    t1 = _tier1(key, cap1)
    assert walkers1 == 1024 and flagged1 == int((key > FP64_KEY).sum()) and overflow1 == flagged1 - len(t1)
    t0 = re.copy()
    t0[t1] = False
    # the FP64-form tier carries the FP64 form's results bit for bit
    np.testing.assert_array_equal(E.cpu().numpy()[t1], E64.cpu().numpy()[t1])
    np.testing.assert_array_equal(lp.cpu().numpy()[t1], lp64.cpu().numpy()[t1])
    np.testing.assert_array_equal(g.cpu().numpy()[t1], g64.cpu().numpy()[t1])
    E, E64, E_u = (x.double().cpu().numpy() for x in (E, E64, E_u))
    # the other replaced walkers carry the results of the FP32 network with FP64 determinants
    np.testing.assert_array_equal(E[t0], E_d.double().cpu().numpy()[t0])
    np.testing.assert_array_equal(lp.cpu().numpy()[t0], lp_d.cpu().numpy()[t0])
    np.testing.assert_array_equal(g.cpu().numpy()[t0], g_d.cpu().numpy()[t0])
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
    E64 = api.local_energy(prm.with_precision("fp64"), spin, st.r, st.R, st.Z)
    re = (E != E_u).cpu().numpy()
    key = sc.double().cpu().numpy()[:, :2].max(axis=1)
    selected = min(flagged, 16)
    assert walkers == 96 and overflow == flagged - selected
    assert flagged > 0 and re.sum() <= selected
    t1 = _tier1(key, 8)
    t0 = re.copy()
    t0[t1] = False
    np.testing.assert_array_equal(E.cpu().numpy()[t1], E64.cpu().numpy()[t1])
    np.testing.assert_array_equal(E.cpu().numpy()[t0], E_d.cpu().numpy()[t0])
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


def test_mixed_det64_form(cuda):
    """DW_PRECISION_MIXED_DET64 (the split-BF16 network with the FP64 determinant algebra, measured as
    a cheaper first-tier re-evaluation and not used: its flagged-walker errors are 5-20x those of
    the FP32 network's): log psi^2 agrees with the mixed form's value pass, E_L follows the mixed
    form's error model against the FP64 form below the threshold."""
    a, prm, st = _equilibrated(A.c2h4_shaped(), 8, 256, 10, seed=3)
    spin = (a.n_up, a.n_dn)
    E5, lp5 = api.local_energy(prm.with_precision("mixed_det64"), spin, st.r, st.R, st.Z, return_grad=True)[:2]
    _, lpm = api.log_psi_sqr(prm, a.n_up, a.n_dn, st.r, st.R, st.Z)
    E64 = api.local_energy(prm.with_precision("fp64"), spin, st.r, st.R, st.Z).double().cpu().numpy()
    _, sc = _unguarded(prm, st.r, st.R, st.Z)
    key = sc.double().cpu().numpy()[:, :2].max(axis=1)
    torch.testing.assert_close(lp5, lpm, rtol=1e-5, atol=1e-4)
    E5 = E5.double().cpu().numpy()
    low = key <= THRESHOLD
    assert low.sum() > 0 and np.all(np.abs(E5[low] - E64[low]) <= 5e-4 * key[low])
    old = _lib.lib().dw_debug_set_guard_form(5)
    assert old == 4 and _lib.lib().dw_debug_set_guard_form(old) == 5
    assert _lib.lib().dw_debug_set_guard_form(1) == -2
