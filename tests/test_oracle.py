"""CPU tests of the FP64 oracle: golden vectors generated from the reference's own source,
closed forms, finite differences and the reference's invariances."""
import glob

import numpy as np
import pytest
import torch

from deeperwin_gb300 import arch as A, params as P
from oracle import dpe4 as O

GOLDEN = sorted(glob.glob(str(__import__("pathlib").Path(__file__).parent / "golden" / "*.npz")))


def _load(f):
    d = np.load(f)
    a = A.Arch(n_el=int(d["n_el"]), n_up=int(d["n_up"]), n_ions=len(d["Z"]), n_dets=int(d["n_dets"]),
               z_min=int(d["z_min"]), z_max=int(d["z_max"]))
    p = P.init_params(a, int(d["seed"]), float(d["bias_std"]), float(d["envelope_jitter"]))
    return d, a, p


@pytest.mark.parametrize("f", GOLDEN, ids=lambda f: f.split("/")[-1])
def test_golden_forward(f):
    d, a, p = _load(f)
    packed = P.pack(a, p).astype(np.float64)
    assert packed.sum() == pytest.approx(float(d["packed_sum"]), rel=1e-12, abs=1e-9)
    assert np.abs(packed).sum() == pytest.approx(float(d["packed_abs_sum"]), rel=1e-12)
    tp = O.tparams(p)
    ph, lp = O.log_psi_sqr(tp, a, d["r"], d["R"], d["Z"])
    np.testing.assert_allclose(lp.numpy(), d["log_psi_sqr"], rtol=1e-11, atol=1e-10)
    np.testing.assert_array_equal(ph.numpy(), d["phase"])
    ns = d["slater"].shape[0]           # the fixtures of the larger shapes keep the first walkers' matrices
    if ns:
        mo = O.slater_matrices(tp, a, d["r"][:ns], d["R"], d["Z"])
        np.testing.assert_allclose(mo.numpy(), d["slater"], rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("f", GOLDEN, ids=lambda f: f.split("/")[-1])
def test_golden_potential_and_clipping(f):
    d, a, p = _load(f)
    np.testing.assert_allclose(O.potential_energy(d["r"], d["R"], d["Z"]).numpy(), d["e_pot"], rtol=1e-12)
    clipped, (c, w) = O.clip_energies(d["clip_E"], *d["clip_in"])
    np.testing.assert_allclose(clipped.numpy(), d["clip_out"], rtol=1e-13)
    np.testing.assert_allclose([float(c), float(w)], d["clip_state_out"], rtol=1e-12)


def _small():
    mol = A.lih()
    a = A.arch_for(mol, 4)
    p = O.tparams(P.init_params(a, 3, bias_std=0.1, envelope_jitter=0.1))
    r = A.init_walkers(mol, 3, seed=5)
    return mol, a, p, r


def test_laplacian_matches_finite_differences():
    mol, a, p, r = _small()
    _, _, g, lap = O.local_energy(p, a, r, mol.R, mol.Z)
    h = 1e-4
    x = torch.tensor(r)
    f = lambda y: O.log_psi_sqr(p, a, y, mol.R, mol.Z)[1]
    f0 = f(x)
    lap_fd = torch.zeros(len(r), dtype=torch.float64)
    g_fd = torch.zeros(len(r), 3 * a.n_el, dtype=torch.float64)
    for i in range(a.n_el):
        for c in range(3):
            e = torch.zeros_like(x)
            e[:, i, c] = h
            fp, fm = f(x + e), f(x - e)
            lap_fd += (fp - 2 * f0 + fm) / h ** 2
            g_fd[:, 3 * i + c] = (fp - fm) / (2 * h)
    np.testing.assert_allclose(g.numpy(), g_fd.numpy(), rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(lap.numpy(), lap_fd.numpy(), rtol=1e-5, atol=1e-4)


def test_antisymmetry_same_spin_swap():
    mol, a, p, r = _small()
    ph, lp = O.log_psi_sqr(p, a, r, mol.R, mol.Z)
    r2 = r.copy()
    r2[:, [0, 1]] = r2[:, [1, 0]]          # both spin-up
    ph2, lp2 = O.log_psi_sqr(p, a, r2, mol.R, mol.Z)
    np.testing.assert_allclose(lp2.numpy(), lp.numpy(), rtol=1e-12)
    assert np.all(np.abs(ph2.numpy() - ph.numpy()) == pytest.approx(np.pi))


def test_coulomb_closed_form_h2():
    R = np.array([[0.0, 0, 0], [1.4, 0, 0]])
    Z = np.array([1, 1])
    r = np.array([[[0.0, 1.0, 0], [1.4, -1.0, 0]]])
    d12 = np.sqrt(1.4 ** 2 + 4.0)
    e_ei = -(1 / 1.0 + 1 / np.sqrt(1.4 ** 2 + 1) + 1 / np.sqrt(1.4 ** 2 + 1) + 1 / 1.0)
    expected = 1 / 1.4 + 1 / d12 + e_ei
    assert float(O.potential_energy(r, R, Z)[0]) == pytest.approx(expected, rel=1e-14)


def test_translation_invariance_of_local_energy():
    mol, a, p, r = _small()
    E1 = O.local_energy(p, a, r, mol.R, mol.Z)[0]
    shift = np.array([0.3, -1.2, 0.7])
    E2 = O.local_energy(p, a, r + shift, mol.R + shift, mol.Z)[0]
    np.testing.assert_allclose(E1.numpy(), E2.numpy(), rtol=1e-9, atol=1e-9)


def test_mh_step_known_answer():
    mol, a, p, r = _small()
    lp = O.log_psi_sqr(p, a, r, mol.R, mol.Z)[1]
    noise = np.zeros_like(r)
    U = np.array([0.0, 1.0, 0.5])           # accept / reject (p == 1 < U) / accept (p == 1 > 0.5)
    age = torch.tensor([0, 0, 20])
    r_out, lp_out, age_out, acc = O.mh_step(p, a, mol.R, mol.Z, r, lp, age, 0.1, noise, U, max_age=20)
    assert acc.tolist() == [True, False, True]
    assert age_out.tolist() == [0, 1, 0]
    np.testing.assert_allclose(r_out.numpy(), r)


def test_stepsize_rule():
    assert O.adjust_stepsize(100, 0.1, 0.2, 100) == pytest.approx(0.1 / 1.05)
    assert O.adjust_stepsize(100, 0.1, 0.7, 100) == pytest.approx(0.1 * 1.05)
    assert O.adjust_stepsize(99, 0.1, 0.7, 100) == 0.1
    assert O.adjust_stepsize(100, 0.0099, 0.0, 100) == 1e-2


def test_vmc_gradient_matches_finite_differences():
    mol, a, p, r = _small()
    E = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64)
    grads, _, _ = O.vmc_gradient(p, a, r, mol.R, mol.Z, E)
    coeff = (E - E.mean()) / len(E)         # no clipping at the initial (0, 1e12) state
    rng = np.random.default_rng(0)
    for name in ["h_el1.w", "bf_up.w", "jas0.w", "alpha_dn", "symm2.w_same.w"]:
        v = p[name]
        idx = tuple(int(rng.integers(0, s)) for s in v.shape)
        h = 1e-5
        vals = []
        for sgn in (1, -1):
            q = dict(p)
            w = v.clone()
            w[idx] += sgn * h
            q[name] = w
            vals.append((O.log_psi_sqr(q, a, r, mol.R, mol.Z)[1] * coeff).sum())
        fd = (vals[0] - vals[1]) / (2 * h)
        assert float(grads[name][idx]) == pytest.approx(float(fd), rel=1e-5, abs=1e-8)
