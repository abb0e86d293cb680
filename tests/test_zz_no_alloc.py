"""The workspace-free log psi^2 entry point (dw_log_psi_sqr_noalloc).

Callers that cannot allocate device memory at call time (a host framework that owns all device
memory through its own pool, a fixed-budget embedding) use this entry point; its scratch is a
fixed static device array instead of a caller workspace. This file is collected last so a run
that stops at the first failure has already run every other test, and it also passes when run
alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from deeperwin_gb300 import _lib, api, arch as A, params as P

pytestmark = pytest.mark.gpu


def _call_noalloc(params, r, R, Z):
    B = r.shape[0]
    lp = torch.full((B,), float("nan"), device="cuda")
    ph = torch.full((B,), float("nan"), device="cuda")
    st = _lib.lib().dw_log_psi_sqr_noalloc(ctypes.byref(params.c_arch), params.prec, api._ptr(params.flat),
                                          api._ptr(params.prepared), api._ptr(r), B, api._ptr(R), api._ptr(Z),
                                          api._ptr(lp), api._ptr(ph), api._stream())
    return st, lp, ph


@pytest.mark.parametrize("prec", ["fp32", "mixed"])
def test_noalloc_matches_workspace_entry_point_twice(cuda, prec):
    mol = A.h_chain(6)
    a = A.arch_for(mol, 4)
    params = api.Params.from_dict(a, P.init_params(a, 3, bias_std=0.1), prec)
    R, Z = api._geometry(mol.R, mol.Z, torch.device("cuda"))
    for seed in (1, 2):                       # two calls in a row share (and overwrite) the static scratch
        r = torch.tensor(A.init_walkers(mol, 96, seed=seed), dtype=torch.float32, device="cuda")
        ph_ref, lp_ref = api.log_psi_sqr(params, a.n_up, a.n_dn, r, R, Z)
        st, lp, ph = _call_noalloc(params, r, R, Z)
        torch.cuda.synchronize()
        assert st == 0, _lib.lib().dw_status_string(st).decode()
        torch.testing.assert_close(lp, lp_ref, rtol=1e-6, atol=1e-5)
        torch.testing.assert_close(ph, ph_ref, rtol=0, atol=0)


def test_noalloc_chunks_batches_larger_than_the_static_scratch(cuda):
    """A batch whose value-pass scratch is many times the 64 MiB array runs in walker chunks that
    fit it, and gives the workspace entry point's results on two calls in a row."""
    mol = A.h_chain(10)
    a = A.arch_for(mol, 16)
    params = api.Params.from_dict(a, P.init_params(a, 0), "mixed")
    R, Z = api._geometry(mol.R, mol.Z, torch.device("cuda"))
    cap = _lib.lib().dw_noalloc_scratch_bytes()
    assert cap == 64 << 20
    B = 20000
    arch = params.c_arch
    assert _lib.lib().dw_workspace_bytes(ctypes.byref(arch), params.prec, B, 0) > 4 * cap
    for seed in (5, 6):
        r = torch.tensor(A.init_walkers(mol, B, seed=seed), dtype=torch.float32, device="cuda")
        ph_ref, lp_ref = api.log_psi_sqr(params, a.n_up, a.n_dn, r, R, Z)
        st, lp, ph = _call_noalloc(params, r, R, Z)
        torch.cuda.synchronize()
        assert st == 0, _lib.lib().dw_status_string(st).decode()
        torch.testing.assert_close(lp, lp_ref, rtol=1e-6, atol=1e-5)
        torch.testing.assert_close(ph, ph_ref, rtol=0, atol=0)


def test_noalloc_rejects_the_fp64_form(cuda):
    mol = A.lih()
    a = A.arch_for(mol, 2)
    params = api.Params.from_dict(a, P.init_params(a, 0), "fp64")
    R, Z = api._geometry(mol.R, mol.Z, torch.device("cuda"))
    r = torch.zeros((4, a.n_el, 3), device="cuda")
    st, _, _ = _call_noalloc(params, r, R, Z)
    assert st == 2          # DW_ERR_ARG: the workspace-free entry point offers the FP32 and tensor-core forms
