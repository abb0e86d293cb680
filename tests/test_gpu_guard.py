"""GPU tests of the mixed form's FP64 tail re-evaluation (guard.cu) at the contract shapes.

* Walkers the guard flags get exactly the FP64 form's E_L, log psi^2 and gradient (the FP64 pass
  is per-walker independent, so a walker's FP64 result does not depend on its batch).
* Walkers it keeps stay within the error model of the mixed form: |E - E_FP64| at most 2e-4 of the
  largest magnitude the kinetic term cancels (reported per walker by the combine kernel).
* Over the batch the mean E_L of the guarded mixed form is within 0.5 mHa of the FP64 form.
* A flagged walker's result is the same alone and inside a larger batch (bit for bit).
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


def test_guarded_mixed_energy_against_fp64(cuda):
    """C2H4-shaped molecule at the differentiation form's shape (16 electrons, 32 determinants),
    1,024 equilibrated walkers."""
    a, prm, st = _equilibrated(A.c2h4_shaped(), 32, 1024, 30)
    spin = (a.n_up, a.n_dn)
    _guard_stats(reset=True)
    E, lp, g = api.local_energy(prm, spin, st.r, st.R, st.Z, return_grad=True)
    walkers, flagged, overflow = _guard_stats(reset=True)
    assert walkers == 1024 and overflow == 0 and flagged <= 1024 // 64
    E_u, sc = _unguarded(prm, st.r, st.R, st.Z)
    E64, lp64, g64 = api.local_energy(prm.with_precision("fp64"), spin, st.r, st.R, st.Z, return_grad=True)
    re = (E != E_u).cpu().numpy()                      # walkers the guard replaced
    assert re.sum() <= flagged
    E, E64, E_u = (x.double().cpu().numpy() for x in (E, E64, E_u))
    # flagged walkers carry the FP64 form's results bit for bit
    np.testing.assert_array_equal(E[re], E64[re])
    np.testing.assert_array_equal(lp.cpu().numpy()[re], lp64.cpu().numpy()[re])
    np.testing.assert_array_equal(g.cpu().numpy()[re], g64.cpu().numpy()[re])
    # the kept walkers within the error model: |dE| <= 2e-4 of the largest cancelled magnitude
    # (measured at most 7.9e-5 of it), and below the flag threshold that magnitude is <= 33,333 Ha
    m = sc.double().cpu().numpy()[:, :2].max(axis=1)
    keep = ~re
    assert np.all(m[keep] <= 0.5 / 1.5e-5 * (1 + 1e-6))
    assert np.all(np.abs(E[keep] - E64[keep]) <= 2e-4 * m[keep]), np.max(np.abs(E[keep] - E64[keep]) / m[keep])
    # the mean over the batch within 0.5 mHa of the FP64 form
    assert abs(E.mean() - E64.mean()) <= 5e-4, (E.mean() - E64.mean(), E_u.mean() - E64.mean(), flagged)


def test_guard_takes_the_largest_predicted_errors_beyond_capacity(cuda):
    """The 40-electron, 64-determinant random molecule: most walkers exceed the tolerance, so the
    capacity (16 of 96) is filled with the walkers of the largest predicted errors, each of which
    gets the FP64 result; the others keep the mixed form's values."""
    a, prm, st = _equilibrated(A.scale_molecule(7), 64, 96, 3)
    spin = (a.n_up, a.n_dn)
    _guard_stats(reset=True)
    E = api.local_energy(prm, spin, st.r, st.R, st.Z)
    walkers, flagged, overflow = _guard_stats(reset=True)
    E_u, sc = _unguarded(prm, st.r, st.R, st.Z)
    E64 = api.local_energy(prm.with_precision("fp64"), spin, st.r, st.R, st.Z)
    re = (E != E_u).cpu().numpy()
    key = sc.cpu().numpy()[:, :2].max(axis=1)
    assert flagged > 16 and overflow == flagged - 16
    np.testing.assert_array_equal(E.cpu().numpy()[re], E64.cpu().numpy()[re])
    top = np.argsort(-key)[:16]
    assert set(np.nonzero(re)[0]) <= set(top.tolist())


def test_guarded_walker_same_alone_and_in_batch(cuda):
    a, prm, st = _equilibrated(A.c2h4_shaped(), 8, 256, 10, seed=3)
    spin = (a.n_up, a.n_dn)
    _guard_stats(reset=True)
    E_all = api.local_energy(prm, spin, st.r, st.R, st.Z)
    assert _guard_stats(reset=True)[2] == 0          # every flagged walker fit the capacity
    E_u, sc = _unguarded(prm, st.r, st.R, st.Z)
    picks = torch.argsort(sc[:, 1], descending=True)[:3].tolist() + [0, 17]
    flagged = (E_all != E_u)
    for b in picks:
        E1 = api.local_energy(prm, spin, st.r[b:b + 1], st.R, st.Z)
        if flagged[b]:
            assert torch.equal(E1[0], E_all[b]), b          # the FP64 result, independent of the batch
        else:
            torch.testing.assert_close(E1[0], E_all[b], rtol=1e-6, atol=1e-5)
