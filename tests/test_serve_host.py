"""Host-side logic of the serving loop (no GPU): the request stream, ion padding and the
weight-sharing slices."""
import numpy as np
import pytest

from deeperwin_gb300 import params as P
from deeperwin_gb300 import serve
from deeperwin_gb300.arch import Arch


def test_request_stream_matches_spec():
    reqs = serve.stream_requests(300, rate=3.0, seed=1)
    t = np.array([q.arrival for q in reqs])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 3.0) < 0.1                          # Poisson rate
    for q in reqs:
        m = q.mol
        assert 2 <= m.n_ions <= 8 and set(m.Z.tolist()) <= {1, 6, 7, 8}
        assert m.n_el == int(m.Z.sum()) and 2 <= m.n_el <= 30 and m.n_up == (m.n_el + 1) // 2
        d = np.linalg.norm(m.R[:, None] - m.R[None], axis=-1) + np.eye(m.n_ions) * 1e9
        assert d.min() >= 1.5 - 1e-9
        assert np.ptp(m.R, axis=0).max() <= 6.0 + 1e-9
        assert 1024 <= q.n_walkers <= 4096 and q.n_steps == 20
    # seeded: the same stream twice
    again = serve.stream_requests(300, rate=3.0, seed=1)
    assert all(a.seed == b.seed and a.n_walkers == b.n_walkers and np.array_equal(a.mol.R, b.mol.R)
               for a, b in zip(reqs, again))


def test_padded_geometry():
    reqs = serve.stream_requests(20, seed=2)
    for q in reqs:
        R, Z = serve.padded_geometry(q.mol)
        n = q.mol.n_ions
        assert R.shape == (8, 3) and Z.shape == (8,) and Z.dtype == np.int32
        assert np.array_equal(Z[:n], q.mol.Z) and np.all(Z[n:] == 0) and np.all(R[n:] == 0)
    big = reqs[0].mol
    with pytest.raises(ValueError):
        serve.padded_geometry(big, n_ions_max=1)


def test_shared_slices_agree_between_padded_and_unpadded_models():
    """The padded (8-ion) slice and a molecule's own slice hold the same numbers for the real
    ions; the padded rows belong to ions whose features are zero."""
    w = serve.SharedWeights(n_dets=4, seed=0, device="cpu")
    n_el, n_up, N = 13, 7, 3
    pad = w.slice(n_el, n_up)
    own = w.slice(n_el, n_up, N)
    f8, f3 = 4 * 8, 4 * N
    for k in range(3):
        np.testing.assert_array_equal(pad["h_el0.w"][k * f8:k * f8 + f3], own["h_el0.w"][k * f3:(k + 1) * f3])
    np.testing.assert_array_equal(pad["h_el0.w"][3 * f8:], own["h_el0.w"][3 * f3:])
    np.testing.assert_array_equal(pad["symm0.h_map.w"][:f3], own["symm0.h_map.w"])
    for name in ("alpha_up", "weights_dn", "bf_up.w"):
        src = pad[name]
        if name.startswith(("alpha", "weights")):
            np.testing.assert_array_equal(src[:N], own[name])
        else:
            np.testing.assert_array_equal(src, own[name])
    # the shapes are those of the sliced architectures
    for arch, d in ((w.arch(n_el, n_up), pad), (w.arch(n_el, n_up, N), own)):
        for name, shape in P.param_shapes(arch).items():
            assert d[name].shape == shape, name
