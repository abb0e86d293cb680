"""Reference checkpoint interop (no GPU): the haiku name map of the dpe4 model, reading run files
in the reference's format (checkpoints.py:26-91) with jax arrays and the MCMCState dataclass
pickled as the reference pickles them, and writing run files the reference's load_run reads.
Neither jax nor the reference is imported: the pickles are produced by stand-in modules that
carry the reference's module and class names."""
import dataclasses
import io
import pickle
import sys
import types
import zipfile

import numpy as np
import pytest

from deeperwin_gb300 import checkpoint as C
from deeperwin_gb300 import params as P
from deeperwin_gb300.arch import Arch

ARCH = Arch(n_el=6, n_up=3, n_ions=3, n_dets=4, z_min=1, z_max=8)


def test_name_map_covers_every_tensor_once():
    names = C.haiku_names(ARCH)
    assert set(names) == set(P.param_shapes(ARCH))
    assert len(set(names.values())) == len(names)
    assert names["ion_embed"] == ("wf/~/input/h_ion", "embeddings")
    assert names["symm1.w_same.b"] == (
        "wf/~_calculate_embedding/fermi_net_embedding/symm_features_1/convolutional_features/w_same/linear_0", "b")
    assert names["h_ei2.w"] == ("wf/~_calculate_embedding/fermi_net_embedding/h_el_ion_2/linear_0", "w")
    assert names["h_el3.w"] == ("wf/~_calculate_embedding/fermi_net_embedding/h_el_3/linear_0", "w")
    assert names["bf_dn.w"] == ("wf/~/orbitals/envelope_orbitals/bf_dn/linear_0", "w")
    assert names["alpha_up"] == ("wf/~/orbitals/envelope_orbitals", "alpha_up")
    assert names["jas2.w"] == ("wf/~/jastrow_factor/mlp/linear_2", "w")
    assert "jas2.b" not in names                      # Jastrow output layer has no bias (wavefunction.py:58)


def test_paths_match_what_the_reference_modules_request():
    """tests/golden/haiku_paths_lih_k8.txt lists every parameter the reference's own module code
    requests for LiH with 8 determinants (tests/golden/make_golden.py runs that code with a haiku
    stand-in that names modules by nesting, without haiku's "~" markers), with its shape."""
    from pathlib import Path
    from deeperwin_gb300 import arch as A
    a = A.arch_for(A.lih(), 8)
    recorded = {}
    for line in (Path(__file__).parent / "golden" / "haiku_paths_lih_k8.txt").read_text().splitlines():
        path, shape = line.split("\t")
        recorded[path] = tuple(int(x) for x in shape.split(","))
    shapes = P.param_shapes(a)
    ours = {C._canonical(mod) + "/" + p: shapes[name] for name, (mod, p) in C.haiku_names(a).items()}
    assert ours == recorded


def test_round_trip_through_haiku_tree():
    p = P.init_params(ARCH, seed=3, bias_std=0.1, envelope_jitter=0.2)
    tree = C.params_to_haiku(p, ARCH)
    back = C.params_from_haiku(tree, ARCH)
    for k, v in p.items():
        np.testing.assert_array_equal(back[k], v.astype(np.float32).astype(np.float64))
    # the same tensors under paths without the "~" components are read too
    plain = {"/".join(c for c in k.split("/") if not c.startswith("~")): v for k, v in tree.items()}
    assert "wf/orbitals/envelope_orbitals" in plain
    back2 = C.params_from_haiku(plain, ARCH)
    assert all(np.array_equal(back2[k], back[k]) for k in back)


def test_shape_and_name_errors():
    tree = C.params_to_haiku(P.init_params(ARCH, seed=0), ARCH)
    other = Arch(n_el=6, n_up=3, n_ions=2, n_dets=4, z_min=1, z_max=8)
    with pytest.raises(ValueError):
        C.params_from_haiku(tree, other)                # alpha/weights carry one row per ion
    del tree["wf/~/jastrow_factor/mlp/linear_1"]
    with pytest.raises(KeyError):
        C.params_from_haiku(tree, ARCH)


def _reference_style_modules():
    """Stand-ins for jax._src.array (arrays pickle through _reconstruct_array around numpy's own
    reduction) and deeperwin.mcmc.MCMCState (a dataclass)."""
    mods = {n: types.ModuleType(n) for n in ("jax", "jax._src", "jax._src.array", "deeperwin", "deeperwin.mcmc")}

    def _reconstruct_array(fun, args, arr_state, aval_state):
        raise AssertionError("never called by the reader")

    _reconstruct_array.__module__ = "jax._src.array"
    _reconstruct_array.__qualname__ = "_reconstruct_array"
    mods["jax._src.array"]._reconstruct_array = _reconstruct_array

    class ArrayImpl:
        def __init__(self, a):
            self.a = np.asarray(a)

        def __reduce__(self):
            fun, args, arr_state = self.a.__reduce__()
            return _reconstruct_array, (fun, args, arr_state, {"weak_type": False})

    @dataclasses.dataclass
    class MCMCState:
        r: object
        R: object
        Z: object
        log_psi_sqr: object
        walker_age: object
        rng_state: object
        stepsize: object
        step_nr: object
        acc_rate: object

    MCMCState.__module__ = "deeperwin.mcmc"
    MCMCState.__qualname__ = "MCMCState"
    mods["deeperwin.mcmc"].MCMCState = MCMCState
    return mods, ArrayImpl, MCMCState


def _reference_run_file(tree, with_state=True):
    mods, ArrayImpl, MCMCState = _reference_style_modules()
    saved = {n: sys.modules.get(n) for n in mods}
    sys.modules.update(mods)
    try:
        jtree = {k: {p: ArrayImpl(v) for p, v in d.items()} for k, d in tree.items()}
        rng = np.random.default_rng(0)
        st = MCMCState(r=ArrayImpl(rng.standard_normal((5, 6, 3)).astype(np.float32)), R=ArrayImpl(np.zeros((3, 3))),
                       Z=ArrayImpl(np.array([1, 3, 8])), log_psi_sqr=ArrayImpl(rng.standard_normal(5)),
                       walker_age=ArrayImpl(np.arange(5, dtype=np.int32)),
                       rng_state=ArrayImpl(np.zeros((5, 2), np.uint32)), stepsize=ArrayImpl(np.float32(0.02)),
                       step_nr=ArrayImpl(np.int32(40)), acc_rate=ArrayImpl(np.float32(0.51)))
        buf = io.BytesIO()
        with zipfile.ZipFile(buf, "w", zipfile.ZIP_BZIP2) as zf:
            zf.writestr("config.yml", "model:\n  name: dpe4\n")
            zf.writestr("params.pkl", pickle.dumps(jtree))
            if with_state:
                zf.writestr("mcmc_state.pkl", pickle.dumps(st))
            zf.writestr("clipping_state.pkl", pickle.dumps((ArrayImpl(np.float32(-7.5)), ArrayImpl(np.float32(2.0)))))
        return buf.getvalue(), st
    finally:
        for n, m in saved.items():
            if m is None:
                sys.modules.pop(n, None)
            else:
                sys.modules[n] = m


def test_read_reference_run_file(tmp_path):
    p = P.init_params(ARCH, seed=5, bias_std=0.05, envelope_jitter=0.1)
    data, st = _reference_run_file(C.params_to_haiku(p, ARCH))
    assert "deeperwin.mcmc" not in sys.modules and "jax._src.array" not in sys.modules   # stand-ins gone
    f = tmp_path / "chkpt000100.zip"
    f.write_bytes(data)
    run = C.load_run(f)
    assert run.config_yaml.startswith("model:")
    got = C.params_from_haiku(run.params, ARCH)
    for k, v in p.items():
        np.testing.assert_array_equal(got[k], v.astype(np.float32).astype(np.float64))
    w = run.walkers()
    np.testing.assert_array_equal(w["r"], st.r.a)
    np.testing.assert_array_equal(w["walker_age"], np.arange(5))
    assert float(np.asarray(w["stepsize"])) == pytest.approx(0.02) and int(np.asarray(w["step_nr"])) == 40
    assert float(np.asarray(run.clipping_state[0])) == -7.5


def test_written_file_reads_back_with_plain_pickle(tmp_path):
    """save_params writes what the reference's load_run unpickles: a dict of dicts of arrays."""
    p = P.init_params(ARCH, seed=1)
    f = tmp_path / "out.zip"
    C.save_params(f, p, ARCH, metadata={"n_epochs": 0})
    with zipfile.ZipFile(f) as zf:
        tree = pickle.loads(zf.read("params.pkl"))
        meta = pickle.loads(zf.read("metadata.pkl"))
    assert meta == {"n_epochs": 0}
    assert all(isinstance(v, dict) for v in tree.values())
    assert all(isinstance(x, np.ndarray) and x.dtype == np.float32 for d in tree.values() for x in d.values())
    back = C.params_from_haiku(tree, ARCH)
    assert all(np.array_equal(back[k], p[k].astype(np.float32)) for k in p)


def test_unknown_classes_are_inert():
    """Objects of classes outside numpy / builtins come back as records; their code never runs."""
    class Evil:
        def __reduce__(self):
            return (print, ("this must not run",))

    blob = pickle.dumps({"x": Evil()})
    out = C.loads(blob)
    assert isinstance(out["x"], C.PickledObject) and out["x"].args == ("this must not run",)
