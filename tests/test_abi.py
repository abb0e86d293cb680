"""CPU tests of the C ABI: the library loads, exports every declared symbol, and its packed
parameter layout agrees with the Python packing. No compute calls (no GPU here)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from deeperwin_gb300 import _lib, arch as A, params as P

HEADER = Path(__file__).resolve().parents[1] / "include" / "dwgb.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(dw_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    syms = declared_symbols()
    assert len(syms) >= 12
    missing = [s for s in syms if getattr(L, s, None) is None]
    assert not missing, missing


@pytest.mark.parametrize("mol_fn,K", [(A.lih, 8), (A.h_chain, 16), (A.c2h4_shaped, 32), (A.scale_molecule, 64)])
def test_param_layout_matches_python(mol_fn, K):
    mol = mol_fn()
    a = A.arch_for(mol, K)
    L = _lib.lib()
    ca = _lib.make_arch(a)
    lay, total = P.layout(a)
    assert L.dw_param_count(ctypes.byref(ca)) == total
    n = len(lay)
    offs = (ctypes.c_int64 * 128)()
    sizes = (ctypes.c_int64 * 128)()
    assert L.dw_param_layout(ctypes.byref(ca), offs, sizes, 128) == n
    assert [offs[i] for i in range(n)] == [o for o, _ in lay.values()]
    assert [sizes[i] for i in range(n)] == [s for _, s in lay.values()]


def test_arch_rejected():
    L = _lib.lib()
    bad = _lib.DwArch(1, 1, 1, 1, 1, 1, 256, 32, 32, 64, 64)
    assert L.dw_param_count(ctypes.byref(bad)) < 0
    assert L.dw_status_string(1).decode()


def test_shared_weight_slicing_is_consistent():
    big = A.Arch(n_el=30, n_up=15, n_ions=8, n_dets=8, z_min=1, z_max=8)
    small = A.Arch(n_el=10, n_up=5, n_ions=3, n_dets=8, z_min=1, z_max=8)
    pb = P.init_params(big, 0)
    ps = P.slice_shared(big, pb, small)
    for name, shape in P.param_shapes(small).items():
        assert ps[name].shape == shape, name
