"""GPU tests of the FP64 form (DW_PRECISION_FP64) against the FP64 oracle and the golden vectors
generated from the reference's source.

The FP64 form computes in double end to end and rounds its outputs to float32, so its tolerance
is float32 rounding of the result (2^-24 relative, bound 1.2e-7) plus the FP64 error of the
computation, which grows with the condition number kappa of the Slater matrices:
* log psi^2: 1.2e-7 |ref| + 1e-6 absolute + 1e-14 kappa;
* E_L: 1.2e-7 |E_ref| + (1e-11 + 1e-14 kappa) S, with S = 1/4 |Lap log psi^2| +
  1/8 |grad log psi^2|^2 + |V| the magnitude of the terms summed into E_L.
"""
import glob
from pathlib import Path

import numpy as np
import pytest
import torch

from deeperwin_gb300 import api, arch as A, params as P
from oracle import dpe4 as O

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(str(Path(__file__).parent / "golden" / "*.npz")))


def _r32(x):
    """Values as the library holds them: weights, walkers and nuclei are float32."""
    if isinstance(x, dict):
        return {k: _r32(v) for k, v in x.items()}
    return np.asarray(x, np.float64).astype(np.float32).astype(np.float64)


def _fixture(f):
    d = np.load(f)
    a = A.Arch(n_el=int(d["n_el"]), n_up=int(d["n_up"]), n_ions=len(d["Z"]), n_dets=int(d["n_dets"]),
               z_min=int(d["z_min"]), z_max=int(d["z_max"]))
    p = P.init_params(a, int(d["seed"]), float(d["bias_std"]), float(d["envelope_jitter"]))
    return d, a, p


def _kappa(p, a, r, mol):
    tp = O.tparams(p)
    h, de = O.embedding(tp, a, O._t(r), O._t(mol.R), mol.Z)
    mo = O.orbitals(tp, a, h, de).numpy()
    return np.array([max(np.linalg.cond(mo[b, k]) for k in range(mo.shape[1])) for b in range(mo.shape[0])])


def _scale(r, mol, g, lap):
    return 0.25 * np.abs(lap) + 0.125 * (g ** 2).sum(-1) + np.abs(O.potential_energy(r, mol.R, mol.Z).numpy())


@pytest.mark.parametrize("f", GOLDEN, ids=lambda f: f.split("/")[-1])
def test_fp64_forward_matches_reference_golden(cuda, f):
    """The library holds weights, walkers and nuclei in float32: against the oracle (pinned to the
    golden vectors to 1e-11) on the float32-rounded inputs the FP64 form agrees to float32
    rounding of its output; against the golden values on the float64 inputs the input rounding
    adds about 1e-6 relative."""
    d, a, p = _fixture(f)
    params = api.Params.from_dict(a, p, "fp64")
    ph, lp = api.log_psi_sqr(params, a.n_up, a.n_dn, d["r"], d["R"], d["Z"])
    lp = lp.cpu().numpy().astype(np.float64)
    ref32 = O.log_psi_sqr(O.tparams(_r32(p)), a, _r32(d["r"]), _r32(d["R"]), d["Z"])[1].numpy()
    np.testing.assert_allclose(lp, ref32, rtol=1.2e-7, atol=1e-6)
    np.testing.assert_allclose(lp, d["log_psi_sqr"], rtol=1e-5, atol=1e-5)
    np.testing.assert_array_equal(ph.cpu().numpy(), d["phase"].astype(np.float32))


def _molecule(name):
    if name == "lih":
        return A.lih(), 8, 6
    if name == "h10":
        return A.h_chain(10), 16, 3
    if name == "c2h4_k32":
        return A.c2h4_shaped(), 32, 4
    if name == "o4h2":
        R = np.array([[0.0, 0, 0], [2.6, 0, 0], [0, 2.6, 0], [2.6, 2.6, 0], [1.3, 1.3, 2.2], [1.3, 1.3, -2.2]])
        return A.Molecule(R=R, Z=np.array([8, 8, 8, 8, 1, 1]), n_el=34, n_up=17, name="O4H2"), 2, 2
    if name == "scale40_k64":
        return A.scale_molecule(7), 64, 2
    n = int(name[1:])
    return A.h_chain(n, 1.6), 2, 3


@pytest.mark.parametrize("name", ["lih", "h10", "c2h4_k32", "h3", "h7", "h13", "o4h2", "scale40_k64"])
def test_fp64_local_energy_matches_oracle(cuda, name):
    mol, K, B = _molecule(name)
    a = A.arch_for(mol, K)
    p = _r32(P.init_params(a, 3, bias_std=0.1, envelope_jitter=0.2))     # the library's input precision
    r = _r32(A.init_walkers(mol, B, seed=21))
    mol = A.Molecule(R=_r32(mol.R), Z=mol.Z, n_el=mol.n_el, n_up=mol.n_up, name=mol.name)
    E_ref, lp_ref, g_ref, lap = [x.numpy() for x in O.local_energy(O.tparams(p), a, r, mol.R, mol.Z)]
    S = _scale(r, mol, g_ref, lap)
    kappa = _kappa(p, a, r, mol)
    params = api.Params.from_dict(a, p, "fp64")
    E, lp, g = api.local_energy(params, (a.n_up, a.n_dn), r, mol.R, mol.Z, return_grad=True)
    E, lp, g = (x.cpu().numpy().astype(np.float64) for x in (E, lp, g))
    bound = 1.2e-7 * np.abs(E_ref) + (1e-11 + 1e-14 * kappa) * S
    assert np.all(np.abs(E - E_ref) <= bound), (name, E, E_ref, np.abs(E - E_ref) / S, kappa)
    np.testing.assert_allclose(lp, lp_ref, rtol=1.2e-7, atol=1e-6)
    gs = np.abs(g_ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(g - g_ref) <= 1.2e-7 * np.abs(g_ref) + (1e-11 + 1e-14 * kappa[:, None]) * gs)


def test_fp64_value_and_tangent_passes_agree(cuda):
    """log psi^2 of the value pass equals the value channel of the forward-Laplacian pass."""
    mol = A.c2h4_shaped()
    a = A.arch_for(mol, 8)
    p = P.init_params(a, 5, bias_std=0.1, envelope_jitter=0.2)
    r = A.init_walkers(mol, 33, seed=2)
    params = api.Params.from_dict(a, p, "fp64")
    _, lp_v = api.log_psi_sqr(params, a.n_up, a.n_dn, r, mol.R, mol.Z)
    _, lp_t = api.local_energy(params, (a.n_up, a.n_dn), r, mol.R, mol.Z, return_grad=True)[:2]
    torch.testing.assert_close(lp_v, lp_t, rtol=2.4e-7, atol=1e-6)


def test_fp64_mcmc_step_matches_oracle(cuda):
    from tests import philox_ref
    mol = A.lih()
    a = A.arch_for(mol, 8)
    p = _r32(P.init_params(a, 0, bias_std=0.1, envelope_jitter=0.1))
    params = api.Params.from_dict(a, p, "fp64")
    state = api.MCMCState.initialize_around_nuclei(64, mol, seed=0)
    r0 = state.r.cpu().numpy().astype(np.float64)
    state.seed = 99
    state.scalars[:] = torch.frombuffer(bytearray(bytes(api._lib.DwMcmcScalars(0.0, 0.0, 0.1, 0, 0, 0))),
                                        dtype=torch.uint8).cuda()
    cfg = api.MCMCConfig(max_age=20, stepsize_update_interval=1000)
    api.MetropolisHastingsMonteCarlo(cfg).run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=1)
    torch.cuda.synchronize()
    B = r0.shape[0]
    noise = philox_ref.proposal_noise(99, B, a.n_el, 0).astype(np.float64)
    U = philox_ref.accept_uniform(99, B, 0).astype(np.float64)
    tp = O.tparams(p)
    lp0 = O.log_psi_sqr(tp, a, r0, mol.R, mol.Z)[1].numpy()
    r_prop = (r0.astype(np.float32) + np.float32(0.1) * noise.astype(np.float32)).astype(np.float64)
    lp1 = O.log_psi_sqr(tp, a, r_prop, mol.R, mol.Z)[1].numpy()
    log_ratio = lp1 - lp0
    clear = np.abs(log_ratio - np.log(U)) > 1e-5
    acc = state.walker_age.cpu().numpy() == 0
    assert clear.sum() > B * 0.95
    np.testing.assert_array_equal(acc[clear], (np.exp(log_ratio) > U)[clear])
    lp_gpu = state.log_psi_sqr.cpu().numpy()
    np.testing.assert_allclose(lp_gpu[acc], lp1[acc], rtol=1.2e-7, atol=1e-6)
    np.testing.assert_allclose(lp_gpu[~acc], lp0[~acc], rtol=1.2e-7, atol=1e-6)


def test_fp64_packed_equals_alone(cuda):
    """Two geometries of equal electron count in one packed FP64 launch give each walker the
    result of its geometry alone, bit for bit."""
    import ctypes
    from deeperwin_gb300 import _lib
    L = _lib.lib()
    m1 = A.h_chain(6, 1.6)
    m2 = A.Molecule(R=np.array([[0.0, 0, 0], [2.0, 0.5, 0], [4.2, 0, 0.3]]), Z=np.array([2, 2, 2]), n_el=6, n_up=3,
                    name="He3")
    a = A.Arch(n_el=6, n_up=3, n_ions=6, n_dets=4, z_min=1, z_max=2)
    p = P.init_params(a, 1, bias_std=0.1, envelope_jitter=0.1)
    params = api.Params.from_dict(a, p, "fp64")
    r1 = A.init_walkers(m1, 5, seed=1)
    r2 = A.init_walkers(m2, 4, seed=2)
    R = np.zeros((2, 6, 3), np.float32)
    Z = np.zeros((2, 6), np.int32)
    R[0], Z[0] = m1.R, m1.Z
    R[1, :3], Z[1, :3] = m2.R, m2.Z
    E_alone = [api.local_energy(params, (3, 3), r, Rg, Zg).cpu() for r, Rg, Zg in ((r1, R[0], Z[0]), (r2, R[1], Z[1]))]
    r = torch.as_tensor(np.concatenate([r1, r2]).astype(np.float32), device="cuda")
    seg = torch.as_tensor([0] * 5 + [1] * 4, dtype=torch.int32, device="cuda")
    Rt = torch.as_tensor(R, device="cuda")
    Zt = torch.as_tensor(Z, device="cuda")
    B = 9
    E = torch.empty(B, device="cuda")
    nbytes = L.dw_workspace_bytes(ctypes.byref(params.c_arch), params.prec, B, 1)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    P_ = lambda t: ctypes.c_void_p(t.data_ptr())
    st = L.dw_local_energy_packed(ctypes.byref(params.c_arch), params.prec, P_(params.flat), P_(params.prepared),
                                  P_(r), B, P_(Rt), P_(Zt), 2, P_(seg), P_(E), ctypes.c_void_p(0), ctypes.c_void_p(0),
                                  P_(ws), nbytes, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.testing.assert_close(E.cpu(), torch.cat(E_alone), rtol=0, atol=0)


def test_fp64_backward_is_unsupported(cuda):
    mol = A.lih()
    a = A.arch_for(mol, 2)
    params = api.Params.from_dict(a, P.init_params(a, 0), "fp64")
    from deeperwin_gb300 import vmc
    r = torch.as_tensor(A.init_walkers(mol, 4, seed=0).astype(np.float32), device="cuda")
    with pytest.raises(RuntimeError, match="status 6"):
        vmc.log_psi_sqr_backward(params, r, *api._geometry(mol.R, mol.Z, "cuda"), torch.zeros(4, device="cuda"))
