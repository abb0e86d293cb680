"""CPU float64 restatement of DeepErwin's VMC inner loop (dpe4 model + Jastrow).

TEST INFRASTRUCTURE ONLY. This module is the oracle that the CUDA path is checked
against. Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it; the product path never does.

Every function cites the reference lines it restates (paths relative to the
reference's ``src/deeperwin``). The reference itself (JAX 0.4.23 / haiku / folx) cannot
be imported in this build environment; the forward pass and the Coulomb energy are
pinned against the reference's own source executed through a numpy stand-in for
jax/haiku (``tests/golden/make_golden.py``), and the derivatives against finite
differences and closed forms.
"""
from __future__ import annotations

import math
from typing import Dict, Optional, Tuple

import numpy as np
import torch

T = torch.float64
LOG_EPSILON = 1e-8  # model/wavefunction.py:64


def _t(x) -> torch.Tensor:
    return torch.as_tensor(np.asarray(x), dtype=T) if not torch.is_tensor(x) else x.to(T)


def tparams(params: Dict[str, np.ndarray]) -> Dict[str, torch.Tensor]:
    return {k: _t(v) for k, v in params.items()}


# --------------------------------------------------------------------------- distances
def el_el_dist(r: torch.Tensor) -> torch.Tensor:
    """``get_distance_matrix(full=True)`` (utils/utils.py:287-305): diff[i,j] = r_j - r_i,
    the diagonal padded by +1 before the norm and then zeroed (gradient-safe)."""
    n = r.shape[-2]
    diff = r[..., None, :, :] - r[..., :, None, :]
    eye = torch.eye(n, dtype=r.dtype)
    dist = torch.linalg.norm(diff + eye[..., None], dim=-1) * (1 - eye)
    return dist


def el_ion(r: torch.Tensor, R: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
    """``get_el_ion_distance_matrix`` (utils/utils.py:262-273): diff = r_i - R_I."""
    diff = r[..., :, None, :] - R[..., None, :, :]
    return diff, torch.linalg.norm(diff, dim=-1)


# --------------------------------------------------------------------------- MLP helpers
def dense(x, p, name, act=True):
    """haiku Linear + tanh (model/mlp.py:57-66)."""
    y = x @ p[name + ".w"]
    if (name + ".b") in p:
        y = y + p[name + ".b"]
    return torch.tanh(y) if act else y


def residual(update, old):
    """``residual_update`` (model/mlp.py:13-17): (old+update)/sqrt(2) only on equal shapes."""
    if old is None or old.shape != update.shape:
        return update
    return (old + update) / np.sqrt(2.0)


# --------------------------------------------------------------------------- wavefunction
def embedding(p, arch, r, R, Z):
    """InputPreprocessor (input_features.py:112-245) + FermiNetEmbedding (ferminet_embedding.py:207-267)."""
    n_up, n = arch.n_up, arch.n_el
    n_dn = n - n_up
    bdims = r.shape[:-2]
    dist_ee = el_el_dist(r)                                      # [B,n,n]
    diff_ei, dist_ei = el_ion(r, R)                              # [B,n,N,3], [B,n,N]
    feat_ei = torch.cat([dist_ei[..., None], diff_ei], dim=-1)   # PairwiseFeatures: [dist, diff] (input_features.py:56-66)
    h_el = feat_ei.reshape(bdims + (n, -1))                      # concatenate_el_ion_features (:237-239)
    z_idx = torch.as_tensor(np.asarray(Z) - arch.z_min, dtype=torch.long)
    h_ion = p["ion_embed"][z_idx]                                # Embed lookup (:185-191)
    h_ion = h_ion.expand(bdims + h_ion.shape)
    # _split_into_same_diff (ferminet_embedding.py:197-205)
    f = dist_ee[..., None]
    h_uu = f[..., :n_up, :n_up, :].reshape(bdims + (n_up * n_up, -1))
    h_ud = f[..., :n_up, n_up:, :].reshape(bdims + (n_up * n_dn, -1))
    h_du = f[..., n_up:, :n_up, :].reshape(bdims + (n_up * n_dn, -1))
    h_dd = f[..., n_up:, n_up:, :].reshape(bdims + (n_dn * n_dn, -1))
    h_same = torch.cat([h_uu, h_dd], dim=-2)
    h_diff = torch.cat([h_ud, h_du], dim=-2)
    h_ei = feat_ei                                               # [B,n,N,4]
    for it in range(arch.n_iter):
        s = f"symm{it}"
        # SymmetricFeatures (ferminet_embedding.py:52-94)
        avg_up = h_el[..., :n_up, :].mean(dim=-2, keepdim=True).expand(h_el.shape)
        avg_dn = h_el[..., n_up:, :].mean(dim=-2, keepdim=True).expand(h_el.shape)
        # ConvolutionalFeatures, dpe4 branch (ferminet_embedding.py:118-175)
        w_same = dense(h_same, p, f"{s}.w_same")
        w_diff = dense(h_diff, p, f"{s}.w_diff")
        w_uu = w_same[..., :n_up * n_up, :].reshape(bdims + (n_up, n_up, -1))
        w_ud = w_diff[..., :n_up * n_dn, :].reshape(bdims + (n_up, n_dn, -1))
        w_du = w_diff[..., n_up * n_dn:, :].reshape(bdims + (n_dn, n_up, -1))
        w_dd = w_same[..., n_up * n_up:, :].reshape(bdims + (n_dn, n_dn, -1))
        hm = dense(h_el, p, f"{s}.h_map")
        h_u = hm[..., None, :n_up, :]
        h_d = hm[..., None, n_up:, :]
        emb_up = (w_uu * h_u).sum(-2) + (w_ud * h_d).sum(-2)
        emb_dn = (w_du * h_u).sum(-2) + (w_dd * h_d).sum(-2)
        conv_ee = torch.cat([emb_up, emb_dn], dim=-2)
        him = dense(h_ion, p, f"{s}.h_ion_map")
        conv_ei = (h_ei * him[..., None, :, :]).sum(-2)
        x = torch.cat([h_el, avg_up, avg_dn, conv_ee, conv_ei], dim=-1)
        h_el = residual(dense(x, p, f"h_el{it}"), x)            # MLP(residual=True) (:233-241)
        if it == arch.n_iter - 1:
            break
        h_same = residual(dense(h_same, p, f"h_same{it}"), h_same)
        h_diff = residual(dense(h_diff, p, f"h_diff{it}"), h_diff)
        h_ei = residual(dense(h_ei, p, f"h_ei{it}"), h_ei)
    return h_el, dist_ei


def orbitals(p, arch, h_el, dist_ei):
    """EnvelopeOrbitals, full_det, isotropic exp envelope (envelope_orbitals.py:39-127)."""
    n_up, n, K = arch.n_up, arch.n_el, arch.n_dets
    n_dn = n - n_up
    bdims = h_el.shape[:-2]
    bf_up = h_el[..., :n_up, :] @ p["bf_up.w"]
    bf_dn = h_el[..., n_up:, :] @ p["bf_dn.w"]
    bf_up = bf_up.reshape(bdims + (n_up, K, n)).transpose(-3, -2)   # [B,K,n_up,n]
    bf_dn = bf_dn.reshape(bdims + (n_dn, K, n)).transpose(-3, -2)

    def env(alpha, w, d):
        e = torch.nn.functional.softplus(alpha) * d[..., None]        # [B,ns,N,K*n]
        o = (w * torch.exp(-e)).sum(-2)                               # [B,ns,K*n]
        return o.reshape(o.shape[:-1] + (K, n)).movedim(-2, -3)      # [B,K,ns,n]

    mo_up = env(p["alpha_up"], p["weights_up"], dist_ei[..., :n_up, :]) * bf_up
    mo_dn = env(p["alpha_dn"], p["weights_dn"], dist_ei[..., n_up:, :]) * bf_dn
    return torch.cat([mo_up, mo_dn], dim=-2)                          # [B,K,n,n]


def sum_of_determinants(mo):
    """``evaluate_sum_of_determinants`` full_det branch (wavefunction.py:63-83)."""
    sign, logdet = torch.linalg.slogdet(mo)
    shift = logdet.max(dim=-1, keepdim=True).values
    psi = (torch.exp(logdet - shift) * sign).sum(-1)
    log_psi_sqr = 2 * (torch.log(psi.abs() + LOG_EPSILON) + shift.squeeze(-1))
    phase = torch.where(psi < 0, torch.full_like(psi, math.pi), torch.zeros_like(psi))
    return phase, log_psi_sqr


def jastrow(p, arch, h_el):
    """JastrowFactor, differentiate_spins=False (wavefunction.py:57-59)."""
    x = h_el
    L = len(arch.jastrow) + 1
    for l in range(L):
        x = dense(x, p, f"jas{l}", act=(l < L - 1))
    return x.sum(dim=(-2, -1))


def log_psi_sqr(p, arch, r, R, Z):
    """``Wavefunction.__call__`` (wavefunction.py:118-134) -> (phase, log psi^2)."""
    r = _t(r)
    R = _t(R)
    h_el, dist_ei = embedding(p, arch, r, R, Z)
    mo = orbitals(p, arch, h_el, dist_ei)
    phase, lp = sum_of_determinants(mo)
    return phase, lp + jastrow(p, arch, h_el)


def slater_matrices(p, arch, r, R, Z):
    r = _t(r)
    h_el, dist_ei = embedding(p, arch, r, _t(R), Z)
    return orbitals(p, arch, h_el, dist_ei)


# --------------------------------------------------------------------------- Hamiltonian
def potential_energy(r, R, Z):
    """``get_potential_energy`` (hamiltonian.py:17-39)."""
    r, R = _t(r), _t(R)
    Zt = _t(np.asarray(Z, np.float64))
    _, d_ei = el_ion(r, R)
    e_ei = -(Zt / d_ei).sum(dim=(-2, -1))
    n = r.shape[-2]
    eye = torch.eye(n, dtype=T)
    d_ee = torch.linalg.norm(r[..., :, None, :] - r[..., None, :, :], dim=-1)
    e_ee = torch.triu(1.0 / (d_ee + eye), diagonal=1).sum(dim=(-2, -1))
    N = R.shape[-2]
    eyeN = torch.eye(N, dtype=T)
    d_ii = torch.linalg.norm(R[:, None, :] - R[None, :, :], dim=-1)
    e_ii = torch.triu((Zt[:, None] * Zt[None, :]) / (d_ii + eyeN), diagonal=1).sum()
    return e_ee + e_ei + e_ii


def grad_and_laplacian(p, arch, r, R, Z):
    """Exact gradient and Laplacian of log psi^2 w.r.t. all 3n coordinates per walker
    (full Hessian diagonal via torch.func, independent of any forward-Laplacian scheme)."""
    r = _t(r)
    R = _t(R)
    B, n, _ = r.shape

    def f(x):
        return log_psi_sqr(p, arch, x.reshape(1, n, 3), R, Z)[1][0]

    grads, laps, vals = [], [], []
    for b in range(B):
        x = r[b].reshape(-1).clone()
        g = torch.func.grad(f)(x)
        H = torch.func.jacfwd(torch.func.grad(f))(x)
        grads.append(g)
        laps.append(torch.diagonal(H).sum())
        vals.append(f(x))
    return torch.stack(vals), torch.stack(grads), torch.stack(laps)


def local_energy(p, arch, r, R, Z):
    """``get_local_energy`` (hamiltonian.py:206-216, 272-291):
    E_kin = -1/2 (1/2 Laplacian(log psi^2) + 1/4 |grad log psi^2|^2), plus Coulomb."""
    lp, g, lap = grad_and_laplacian(p, arch, r, R, Z)
    e_kin = -0.5 * (0.5 * lap + 0.25 * (g ** 2).sum(-1))
    return e_kin + potential_energy(r, R, Z), lp, g, lap


# --------------------------------------------------------------------------- batched, any dtype
def log_psi_sqr_raw(p, arch, r, R, Z):
    """``Wavefunction.__call__`` on tensors used as given (no float64 cast): the restatement in the
    dtype of ``p`` and ``r`` (float32 for the reference's default precision, configuration.py:1893)."""
    h_el, dist_ei = embedding(p, arch, r, R, Z)
    mo = orbitals(p, arch, h_el, dist_ei)
    phase, lp = sum_of_determinants(mo)
    return phase, lp + jastrow(p, arch, h_el)


def local_energy_batched(p, arch, r, R, Z):
    """E_L of a batch of walkers in the dtype of ``p`` / ``r``: gradient and exact Laplacian of
    log psi^2 by torch.func (Hessian diagonal of each walker, vmapped over the batch, like the
    reference's batched_vmap over get_local_energy, hamiltonian.py:272-291), Coulomb energy in the
    same dtype (hamiltonian.py:17-39)."""
    B, n, _ = r.shape

    def f(x):
        return log_psi_sqr_raw(p, arch, x.reshape(1, n, 3), R, Z)[1][0]

    x = r.reshape(B, 3 * n)
    g = torch.func.vmap(torch.func.grad(f))(x)
    H = torch.func.vmap(torch.func.jacfwd(torch.func.grad(f)))(x)
    lap = torch.diagonal(H, dim1=-2, dim2=-1).sum(-1)
    e_kin = -0.5 * (0.5 * lap + 0.25 * (g ** 2).sum(-1))
    Zt = torch.as_tensor(np.asarray(Z), dtype=r.dtype)
    d_ei = torch.linalg.norm(r[:, :, None, :] - R[None, None, :, :], dim=-1)
    e_ei = -(Zt / d_ei).sum(dim=(-2, -1))
    eye = torch.eye(n, dtype=r.dtype)
    d_ee = torch.linalg.norm(r[:, :, None, :] - r[:, None, :, :], dim=-1)
    e_ee = torch.triu(1.0 / (d_ee + eye), diagonal=1).sum(dim=(-2, -1))
    N = R.shape[0]
    d_ii = torch.linalg.norm(R[:, None, :] - R[None, :, :], dim=-1)
    e_ii = torch.triu((Zt[:, None] * Zt[None, :]) / (d_ii + torch.eye(N, dtype=r.dtype)), diagonal=1).sum()
    return e_kin + e_ee + e_ei + e_ii


def forces(p, arch, r, R, Z, log_psi_sqr, R_cut=0.1, R_core=0.5, antithetic=False):
    """``calculate_forces`` (hamiltonian.py:293-338): [N, 3] batch mean of the per-walker
    electron-nucleus forces with the tanh cut-off, optionally antithetic, plus the ion-ion term."""
    r, R = _t(r), _t(R)
    Zt = _t(np.asarray(Z, np.float64))

    def direct(x):
        diff, d = el_ion(x, R)                                       # diff = r_i - R_I
        d = d / torch.tanh(d / R_cut)
        return Zt[:, None] * diff / d[..., None] ** 3                 # [B, n, N, 3]
    f = direct(r)
    if antithetic:
        diff, d = el_ion(r, R)
        idx = d.argmin(dim=-1)
        dmin = d.min(dim=-1, keepdim=True).values
        to_closest = torch.gather(diff, 2, idx[..., None, None].expand(-1, -1, 1, 3))[:, :, 0]
        rm = torch.where(dmin < R_core, r - 2 * to_closest, r)
        w = torch.exp(log_psi_sqr_raw(p, arch, rm, R, Z)[1] - _t(log_psi_sqr))
        f = (f + direct(rm) * w[:, None, None, None]) * 0.5
    force = f.sum(1).mean(0)
    diffR = R[:, None, :] - R[None, :, :]
    dist = torch.linalg.norm(diffR, dim=-1, keepdim=True)
    Zm = Zt[:, None] * Zt[None, :] - torch.diag(Zt ** 2)
    return force + (diffR * Zm[..., None] / (dist + 1e-8) ** 3).sum(1)


# --------------------------------------------------------------------------- MCMC
def mh_step(p, arch, R, Z, r, lp, age, stepsize, noise, uniform, max_age):
    """One Metropolis-Hastings step with injected randomness
    (``_propose_normal`` mcmc.py:175-180, ``make_mcmc_step`` mcmc.py:345-366)."""
    r, lp = _t(r), _t(lp)
    r_new = r + _t(noise) * stepsize
    lp_new = log_psi_sqr(p, arch, r_new, R, Z)[1]
    p_acc = torch.exp(lp_new - lp)
    acc = p_acc > _t(uniform)
    age = torch.as_tensor(age)
    acc = acc | (age >= max_age)
    age_new = torch.where(acc, torch.zeros_like(age), age + 1)
    lp_out = torch.where(acc, lp_new, lp)
    r_out = torch.where(acc[:, None, None], r_new, r)
    return r_out, lp_out, age_new, acc


def _closest_ion_dist(r, R):
    return torch.linalg.norm(r[..., :, None, :] - R[None, None, :, :], dim=-1).min(dim=-1).values   # [B, n]


def propose(kind, r, R, Z, stepsize, step_nr, noise, cauchy_u=None, r_min=None, r_max=None, langevin_scale=1.0):
    """Proposal functions of mcmc.py:175-288 with injected randomness; returns (r_new, log_q_ratio).
    noise: standard normals [B, n, 3]; cauchy_u: uniforms in (0, 1) [B, n, 3] for the Cauchy proposal."""
    r, R = _t(r), _t(R)
    z = _t(noise)
    B, n, _ = r.shape
    zero = torch.zeros(B, dtype=T)
    if kind == "normal":                                                 # mcmc.py:175-180
        return r + z * stepsize, zero
    if kind == "cauchy":                                                 # mcmc.py:196-201
        return r + torch.tan(math.pi * (_t(cauchy_u) - 0.5)) * stepsize, zero
    if kind in ("normal_one_el", "local_one_el"):
        idx = step_nr % n                                                # mcmc.py:185, :240
        r_new = r.clone()
        if kind == "normal_one_el":                                      # mcmc.py:183-193
            r_new[:, idx] += z[:, idx] * stepsize
            return r_new, zero
        s = stepsize * torch.clamp(_closest_ion_dist(r, R)[:, idx], r_min, r_max)      # mcmc.py:237-245
        r_new[:, idx] += z[:, idx] * s[:, None]
        s_new = stepsize * torch.clamp(_closest_ion_dist(r_new, R)[:, idx], r_min, r_max)
        d2 = ((r_new[:, idx] - r[:, idx]) ** 2).sum(-1)
        return r_new, 3 * (torch.log(s) - torch.log(s_new)) + 0.5 * d2 * (1 / s ** 2 - 1 / s_new ** 2)
    if kind == "local":                                                  # mcmc.py:218-234
        s = stepsize * torch.clamp(_closest_ion_dist(r, R), r_min, r_max)
        r_new = r + z * s[..., None]
        s_new = stepsize * torch.clamp(_closest_ion_dist(r_new, R), r_min, r_max)
        d2 = ((r_new - r) ** 2).sum(-1)
        lq = 3 * (torch.log(s) - torch.log(s_new)) + 0.5 * d2 * (1 / s ** 2 - 1 / s_new ** 2)
        return r_new, lq.sum(-1)
    if kind == "langevin":                                               # mcmc.py:204-215, :260-288
        Zt = _t(np.asarray(Z, np.float64))

        def bias(x):
            diff = x[..., :, None, :] - R[None, None, :, :]
            dist = torch.linalg.norm(diff, dim=-1)
            s_ = stepsize * torch.clamp(dist.min(dim=-1, keepdim=True).values, r_min, r_max)
            g_ = -langevin_scale * (diff * Zt[:, None] / dist[..., None]).sum(-2)
            return s_, g_
        s, g = bias(r)
        r_new = r + z * s + g * s ** 2
        s_new, g_new = bias(r_new)
        d_fwd = ((r_new - r - g * s ** 2) ** 2).sum(-1)
        d_rev = ((r - r_new - g_new * s_new ** 2) ** 2).sum(-1)
        s, s_new = s[..., 0], s_new[..., 0]
        lq = 3 * (torch.log(s) - torch.log(s_new)) + 0.5 * (d_fwd / s ** 2 - d_rev / s_new ** 2)
        return r_new, lq.sum(-1)
    raise ValueError(kind)


def spin_swap(r, n_up, p_swap, u_select, ind_up, ind_dn):
    """``spin_swap`` (mcmc.py:291-302) with injected draws: ind_up in [0, n_up), ind_dn in
    [n_up, n_el); with probability p_swap the two electrons exchange positions."""
    r = _t(r).clone()
    for b in range(r.shape[0]):
        if u_select[b] < p_swap:
            i, j = int(ind_up[b]), int(ind_dn[b])
            r[b, [i, j]] = r[b, [j, i]]
    return r


def spin_flip(r, p_flip, u):
    """``spin_flip`` (mcmc.py:305-310): with probability p_flip the electron order is reversed."""
    r = _t(r)
    return torch.where(_t(u)[:, None, None] < p_flip, r.flip(-2), r)


def mh_accept(lp, lp_new, log_q, age, uniform, max_age):
    """Acceptance of ``make_mcmc_step`` (mcmc.py:357-366) with the proposal ratio."""
    lp, lp_new = _t(lp), _t(lp_new)
    acc = torch.exp(lp_new - lp + _t(log_q)) > _t(uniform)
    age = torch.as_tensor(age)
    return acc | (age >= max_age)


def adjust_stepsize(step_nr, stepsize, acc_rate_prev, interval, target=0.5, lo=1e-2, hi=1.0):
    """Step-size rule (mcmc.py:370-387): on every ``interval``-th step, divide by 1.05 if the
    previous running acceptance rate is below target, else multiply; clip to [lo, hi]."""
    if step_nr % interval == 0:
        stepsize = stepsize / 1.05 if acc_rate_prev < target else stepsize * 1.05
        stepsize = min(max(stepsize, lo), hi)
    return stepsize


# --------------------------------------------------------------------------- VMC gradient
def clip_energies(E, center, width, clip_by=5.0):
    """tanh clipping from the previous step's state (loss_function.py:44-72)."""
    E = _t(E)
    clipped = center + torch.tanh((E - center) / width) * width
    c_new = clipped.mean()
    w_new = torch.sqrt(((clipped - c_new) ** 2).mean()) * clip_by
    return clipped, (c_new, w_new)


def vmc_gradient(p, arch, r, R, Z, E_loc, clip_state=(0.0, 1e12)):
    """Gradient of the VMC loss (loss_function.py:111-153):
    g = (1/B) sum_b d/dtheta log psi^2_b * (E_clip_b - mean(E_clip)).
    Returns (grads dict, E_mean_clipped, new clip state)."""
    E_clip, new_state = clip_energies(E_loc, *clip_state)
    coeff = (E_clip - E_clip.mean()) / len(E_clip)
    pt = {k: v.detach().clone().requires_grad_(True) for k, v in p.items()}
    lp = log_psi_sqr(pt, arch, r, R, Z)[1]
    (lp * coeff.detach()).sum().backward()
    grads = {k: (v.grad if v.grad is not None else torch.zeros_like(v)) for k, v in pt.items()}
    return grads, E_clip.mean(), new_state
