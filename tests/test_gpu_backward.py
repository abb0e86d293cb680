"""GPU tests of the hand-written d log psi^2 / d theta backward (VMC gradient)."""
import numpy as np
import pytest
import torch

from deeperwin_gb300 import api, arch as A, params as P, vmc
from oracle import dpe4 as O

pytestmark = pytest.mark.gpu


def _oracle_grad(a, p, r, mol, coeff, dtype=torch.float64):
    """d/dtheta sum_b coeff_b log psi^2_b from the oracle by autograd (FP64, or the same
    mathematics in FP32 to measure what FP32 arithmetic alone costs)."""
    old = O.T
    O.T = dtype
    try:
        return _oracle_grad_t(a, p, r, mol, coeff, dtype)
    finally:
        O.T = old


def _oracle_grad_t(a, p, r, mol, coeff, dtype):
    pt = {k: torch.tensor(v, dtype=dtype, requires_grad=True) for k, v in p.items()}
    lp = O.log_psi_sqr(pt, a, r, mol.R, mol.Z)[1]
    (lp * torch.tensor(coeff, dtype=dtype)).sum().backward()
    g = {k: v.grad.numpy() for k, v in pt.items()}
    lay, total = P.layout(a)
    flat = np.zeros(total)
    for k, (o, s) in lay.items():
        flat[o:o + s] = g[k].reshape(-1).astype(np.float64)
    return flat


def _o4h2():
    """34 electrons (n > 32: the shared-memory LU / inverse of the larger molecules)."""
    R = np.array([[0.0, 0, 0], [2.6, 0, 0], [0, 2.6, 0], [2.6, 2.6, 0], [1.3, 1.3, 2.2], [1.3, 1.3, -2.2]])
    return A.Molecule(R=R, Z=np.array([8, 8, 8, 8, 1, 1]), n_el=34, n_up=17, name="O4H2")


@pytest.mark.parametrize("case", ["lih", "h6", "c2h4", "o4h2"])
def test_backward_matches_oracle_autograd(cuda, case):
    mol, K, B = {"lih": (A.lih(), 4, 5), "h6": (A.h_chain(6), 4, 3), "c2h4": (A.c2h4_shaped(), 2, 2),
                 "o4h2": (_o4h2(), 2, 2)}[case]
    a = A.arch_for(mol, K)
    p = P.init_params(a, 2, bias_std=0.1, envelope_jitter=0.2)
    r = A.init_walkers(mol, B, seed=3)
    coeff = np.random.default_rng(0).standard_normal(B)
    params = api.Params.from_dict(a, p, "mixed")
    g = vmc.log_psi_sqr_backward(params, torch.tensor(r, dtype=torch.float32), mol.R, mol.Z,
                                 torch.tensor(coeff, dtype=torch.float32)).cpu().numpy().astype(np.float64)
    ref = _oracle_grad(a, p, r, mol, coeff)
    scale = np.abs(ref).max()
    err = np.abs(g - ref)
    # The kernels recompute the forward in FP32, so the error floor is that of FP32 arithmetic
    # on these Slater matrices (condition numbers 1e3 at 16 electrons, 2-6e4 at 34, where it
    # reaches 1e-4 to 8e-4 of the gradient scale depending on the host's FP32 op order): the
    # same oracle run in FP32 measures it. The bound is 1e-4 of the gradient scale or 5x that
    # floor (the kernels measured 2.7x at 34 electrons).
    floor = np.abs(_oracle_grad(a, p, r, mol, coeff, torch.float32) - ref)
    tol = max(1e-4 * scale, 5.0 * floor.max())
    tol_norm = max(1e-4 * np.linalg.norm(ref), 5.0 * np.linalg.norm(floor))
    lay, _ = P.layout(a)
    worst = sorted(((float(err[o:o + s].max() / scale), k) for k, (o, s) in lay.items()), reverse=True)[:3]
    assert err.max() <= tol, (worst, tol / scale)
    assert np.linalg.norm(g - ref) <= tol_norm, (worst, tol_norm)
    if case != "o4h2":
        assert err.max() <= 1e-4 * scale, worst


@pytest.mark.parametrize("case", ["lih_k4", "c2h4_k32"])
def test_backward_matches_central_finite_differences(cuda, case):
    """64 random parameters, central differences with h = 1e-3 on the FP64 oracle forward; the
    C2H4-shaped case is the differentiation form's own shape (16 electrons, 32 determinants)."""
    mol, K = (A.lih(), 4) if case == "lih_k4" else (A.c2h4_shaped(), 32)
    a = A.arch_for(mol, K)
    p = P.init_params(a, 5, bias_std=0.1, envelope_jitter=0.2)
    r = A.init_walkers(mol, 4, seed=8).astype(np.float32).astype(np.float64)
    coeff = np.array([0.7, -1.1, 0.4, 0.25])
    params = api.Params.from_dict(a, p, "mixed")
    g = vmc.log_psi_sqr_backward(params, torch.tensor(r, dtype=torch.float32), mol.R, mol.Z,
                                 torch.tensor(coeff, dtype=torch.float32)).cpu().numpy().astype(np.float64)
    lay, total = P.layout(a)
    flat = P.pack(a, p).astype(np.float64)
    valid = np.concatenate([np.arange(o, o + s) for o, s in lay.values()])
    idx = np.random.default_rng(1).choice(valid, size=64, replace=False)
    h = 1e-3

    def f(x):
        q = P.unpack(a, x)
        return float((O.log_psi_sqr(O.tparams(q), a, r, mol.R, mol.Z)[1].numpy() * coeff).sum())
    fd = []
    for k in idx:
        xp, xm = flat.copy(), flat.copy()
        xp[k] += h
        xm[k] -= h
        fd.append((f(xp) - f(xm)) / (2 * h))
    fd = np.array(fd)
    scale = np.abs(fd).max()
    assert np.abs(g[idx] - fd).max() <= 1e-4 * scale + 1e-6, np.abs(g[idx] - fd).max() / scale


def test_autograd_function_and_value_and_grad(cuda):
    mol = A.h_chain(4)
    a = A.arch_for(mol, 4)
    params = api.Params.from_dict(a, P.init_params(a, 1), "mixed")
    r = torch.tensor(A.init_walkers(mol, 64, seed=2), dtype=torch.float32, device="cuda")
    flat = params.flat.detach().clone().requires_grad_(True)
    params.flat = flat.detach()
    c = torch.randn(64, device="cuda")
    lp = vmc.LogPsiSqr.apply(flat, params, r, mol.R, mol.Z)
    (g,) = torch.autograd.grad((lp * c).sum(), flat)
    g2 = vmc.log_psi_sqr_backward(params, r, mol.R, mol.Z, c)
    # float atomics in the weight-gradient reductions make repeated calls differ in the last bits
    torch.testing.assert_close(g, g2, rtol=1e-4, atol=1e-4 * float(g2.abs().max()))
    vg = vmc.build_value_and_grad_func()
    (loss, (state, aux)), grads = vg(params, vmc.init_clipping_state(), (a.n_up, a.n_dn), (r, mol.R, mol.Z))
    E = aux["E_loc"].double()
    assert float(loss) == pytest.approx(float(E.mean()), rel=1e-6)     # no clipping at width 1e12
    coeff = (E - E.mean()) / E.numel()
    g3 = vmc.log_psi_sqr_backward(params, r, mol.R, mol.Z, coeff.float())
    torch.testing.assert_close(grads, g3, rtol=1e-4, atol=1e-6)
    assert state[1] == pytest.approx(5.0 * float(E.std(unbiased=False)), rel=1e-5)


def test_vmc_optimisation_step_with_adam(cuda):
    """One VMC optimisation step (the OptaxWrapper step, optimizers.py:113-140, with optax.adam):
    clipped gradient from the hand-written backward, Adam update of the packed weights on the GPU,
    derived weight copies rebuilt so that the next forward sees the new weights."""
    from deeperwin_gb300 import optim
    mol = A.lih()
    a = A.arch_for(mol, 4)
    params = api.Params.from_dict(a, P.init_params(a, 2, bias_std=0.1, envelope_jitter=0.2), "mixed")
    r = torch.tensor(A.init_walkers(mol, 64, seed=1), dtype=torch.float32, device="cuda")
    vg = vmc.build_value_and_grad_func()
    (loss, (clip_state, aux)), g = vg(params, vmc.init_clipping_state(), (a.n_up, a.n_dn), (r, mol.R, mol.Z))
    assert torch.isfinite(g).all() and g.abs().max() > 0
    flat0 = params.flat.clone()
    _, lp0 = api.log_psi_sqr(params, a.n_up, a.n_dn, r, mol.R, mol.Z)
    opt = optim.Adam(params.flat)
    opt.step(params, g)
    # first Adam step: theta - lr(0) g / (|g| + eps), lr(0) = 1e-3
    gd = g.double()
    torch.testing.assert_close(params.flat.double(), flat0.double() - 1e-3 * gd / (gd.abs() + 1e-8), rtol=0, atol=2e-7)
    _, lp1 = api.log_psi_sqr(params, a.n_up, a.n_dn, r, mol.R, mol.Z)
    fresh = api.Params.from_dict(a, P.unpack(a, params.flat.cpu().numpy()), "mixed")
    _, lp2 = api.log_psi_sqr(fresh, a.n_up, a.n_dn, r, mol.R, mol.Z)
    torch.testing.assert_close(lp1, lp2, rtol=0, atol=0)
    assert (lp1 - lp0).abs().max() > 1e-4


def test_sharded_gradient_composition_on_one_rank(cuda):
    """deeperwin_gb300.dist.sharded_clipped_gradient over the GPU statistics, clipping and backward
    kernels equals value_and_grad's single-rank result (loss, next clipping state, gradient)."""
    from deeperwin_gb300 import dist
    mol = A.lih()
    a = A.arch_for(mol, 4)
    params = api.Params.from_dict(a, P.init_params(a, 2, bias_std=0.1, envelope_jitter=0.2), "mixed")
    r = torch.tensor(A.init_walkers(mol, 64, seed=1), dtype=torch.float32, device="cuda")
    vg = vmc.build_value_and_grad_func()
    for state in [(-7.5, 3.0), (0.0, 1e12)]:
        (loss, (new_state, aux)), g = vg(params, state, (a.n_up, a.n_dn), (r, mol.R, mol.Z))
        E = aux["E_loc"]

        def stats_fn(e):
            s = api.energy_stats(e)
            return s[0], s[1]

        def clip_fn(e, c, w):
            ec, o = vmc._clip(e, c, w, 5.0)
            return ec, o[0], o[1]

        loss2, state2, aux2, g2 = dist.sharded_clipped_gradient(
            E, state, 5.0, True, stats_fn, clip_fn,
            lambda coeff: vmc.log_psi_sqr_backward(params, r, mol.R, mol.Z, coeff.float()))
        assert float(loss2) == float(loss)
        np.testing.assert_allclose(state2, new_state, rtol=1e-12)
        # the weight-gradient reductions accumulate with atomics: equal up to summation order
        torch.testing.assert_close(g2, g, rtol=1e-5, atol=1e-6 * float(g.abs().max()))
