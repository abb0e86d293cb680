"""Reference checkpoints: read DeepErwin run files (``chkpt*.zip``) into the packed layout and
write the packed weights back as a haiku parameter tree, without jax or haiku installed.

Format (``checkpoints.py:26-91``): a zip (bzip2) holding ``config.yml``, ``history.csv``,
``summary.csv`` and one pickle per ``RunData`` field (``params.pkl``, ``mcmc_state.pkl``,
``clipping_state.pkl``, ``opt_state.pkl``, ``fixed_params.pkl``, ``metadata.pkl``, ...).
``params.pkl`` is the haiku tree ``{module_path: {param_name: array}}``; the arrays are either
numpy arrays (``run_tools/convert_checkpoint.py:58`` stores them so) or jax arrays, which pickle as
a call of ``jax._src.array._reconstruct_array(fun, args, arr_state, aval_state)`` around numpy's
own array reduction. The reader unpickles with a restricted unpickler: numpy arrays and plain
containers are rebuilt, the jax hook is answered with the numpy array itself, and every other
class (the MCMCState dataclass, optax states, ...) becomes an inert record of its pickled state;
no code from the file is run.

Haiku parameter paths of the dpe4 model (``model/wavefunction.py:86-134``; haiku names a module
``parent/~/name`` when it is built in the parent's ``__init__``, ``parent/~method/name`` in another
method, ``parent/name`` in ``__call__``):

==========================  =====================================================================
packed name                 haiku path / parameter
==========================  =====================================================================
ion_embed                   wf/~/input/h_ion : embeddings (``model/input_features.py:184-191``)
symm{i}.{w_same,w_diff,     wf/~_calculate_embedding/fermi_net_embedding/symm_features_{i}/
h_map,h_ion_map}.{w,b}      convolutional_features/{...}/linear_0 : w, b
                            (``model/embeddings/ferminet_embedding.py:97-175, 218``)
h_el{i}.{w,b}               wf/~_calculate_embedding/fermi_net_embedding/h_el_{i}/linear_0
h_same{i}, h_diff{i},       .../fermi_net_embedding/h_same_{i}, h_diff_{i}, h_el_ion_{i}/linear_0
h_ei{i}                     (``ferminet_embedding.py:233-262``)
bf_up.w, bf_dn.w            wf/~/orbitals/envelope_orbitals/bf_up|bf_dn/linear_0 : w
                            (``model/orbitals/envelope_orbitals.py:46-70``)
alpha_*, weights_*          wf/~/orbitals/envelope_orbitals : alpha_up, ... (``:99-104``)
jas{l}.{w,b}                wf/~/jastrow_factor/mlp/linear_{l} (``model/wavefunction.py:42-60``)
==========================  =====================================================================

A module without a name is named after its class in snake case (``FermiNetEmbedding`` ->
``fermi_net_embedding``). Paths are matched with their ``~`` components removed, so both the
spelling above and the one without them (as ``model/wavefunction.py:346-353`` indexes
``wf/orbitals/envelope_orbitals``) are read; the ``~``-free paths are pinned by the list of
parameters the reference's own module code requests (``tests/golden/haiku_paths_lih_k8.txt``). Dense layers are haiku ``Linear`` (``w[d_in, d_out]``) in both layouts, and the rows of
``h_el0.w`` follow the reference's feature concatenation, so every tensor copies unchanged.
"""
from __future__ import annotations

import io
import pickle
import zipfile
from dataclasses import dataclass, field
from typing import Any, Dict, Mapping, Optional, Tuple

import numpy as np

from .arch import Arch
from .params import param_shapes

_EMB = "wf/~_calculate_embedding/fermi_net_embedding"
_ENV = "wf/~/orbitals/envelope_orbitals"


def haiku_names(a: Arch) -> Dict[str, Tuple[str, str]]:
    """packed name -> (haiku module path, parameter name) for the dpe4 model of `a`."""
    out: Dict[str, Tuple[str, str]] = {"ion_embed": ("wf/~/input/h_ion", "embeddings")}
    for name in param_shapes(a):
        if name == "ion_embed":
            continue
        if name.startswith("symm"):
            it, mod, p = name[4:].split(".")
            out[name] = (f"{_EMB}/symm_features_{it}/convolutional_features/{mod}/linear_0", p)
        elif name.startswith(("h_el", "h_same", "h_diff", "h_ei")):
            mod, p = name.split(".")
            stem = mod.rstrip("0123456789")
            it = mod[len(stem):]
            hk_mod = {"h_el": "h_el", "h_same": "h_same", "h_diff": "h_diff", "h_ei": "h_el_ion"}[stem]
            out[name] = (f"{_EMB}/{hk_mod}_{it}/linear_0", p)
        elif name.startswith("bf_"):
            mod, p = name.split(".")
            out[name] = (f"{_ENV}/{mod}/linear_0", p)
        elif name.startswith(("alpha_", "weights_")):
            out[name] = (_ENV, name)
        elif name.startswith("jas"):
            mod, p = name.split(".")
            out[name] = (f"wf/~/jastrow_factor/mlp/linear_{mod[3:]}", p)
        else:
            raise KeyError(name)
    return out


def _canonical(path: str) -> str:
    """A haiku module path without its ``~`` / ``~method`` components."""
    return "/".join(p for p in path.split("/") if not p.startswith("~"))


def params_from_haiku(tree: Mapping[str, Mapping[str, Any]], a: Arch) -> Dict[str, np.ndarray]:
    """The packed parameter dict (float64 arrays, as ``params.init_params`` returns) from a
    reference haiku tree. Raises KeyError for a missing tensor and ValueError for a shape that
    does not fit `a` (another architecture or molecule)."""
    by_canon = {_canonical(k): v for k, v in tree.items()}
    shapes = param_shapes(a)
    out: Dict[str, np.ndarray] = {}
    for name, (mod, p) in haiku_names(a).items():
        c = _canonical(mod)
        if c not in by_canon or p not in by_canon[c]:
            raise KeyError(f"{name}: no parameter {p!r} of module {mod!r} in the checkpoint")
        v = np.asarray(by_canon[c][p], dtype=np.float64)
        if v.shape != shapes[name]:
            raise ValueError(f"{name}: checkpoint shape {v.shape}, model shape {shapes[name]}")
        out[name] = v
    return out


def params_to_haiku(params: Mapping[str, np.ndarray], a: Arch) -> Dict[str, Dict[str, np.ndarray]]:
    """The haiku tree (float32 numpy arrays) of a packed parameter dict."""
    tree: Dict[str, Dict[str, np.ndarray]] = {}
    for name, (mod, p) in haiku_names(a).items():
        tree.setdefault(mod, {})[p] = np.asarray(params[name], dtype=np.float32)
    return tree


# ----------------------------------------------------------------------------- unpickling
class PickledObject:
    """An object of a class that is not rebuilt: its module, class name, constructor arguments
    and pickled state (``state`` is usually the instance ``__dict__``)."""

    _module = ""
    _qualname = ""

    def __new__(cls, *args, **kwargs):
        obj = object.__new__(cls)
        obj.args = args
        obj.state = None
        return obj

    def __init__(self, *args, **kwargs):
        pass

    def __setstate__(self, state):
        self.state = state

    def __getitem__(self, key):
        return self.state[key] if isinstance(self.state, dict) else self.args[key]

    def get(self, key, default=None):
        return self.state.get(key, default) if isinstance(self.state, dict) else default

    def __repr__(self):
        return f"<pickled {self._module}.{self._qualname}>"


def _jax_array(fun, args, arr_state, aval_state=None):
    """Stands in for jax's array reconstruction hook: returns the numpy array it wraps."""
    arr = fun(*args)
    arr.__setstate__(arr_state)
    return arr


_NUMPY_OK = {"_reconstruct", "ndarray", "dtype", "scalar", "_frombuffer"}
_BUILTINS_OK = {"complex", "float", "int", "bool", "str", "bytes", "bytearray", "list", "tuple", "dict", "set",
                "frozenset", "slice", "range", "object"}


class _ReferenceUnpickler(pickle.Unpickler):
    def find_class(self, module: str, name: str):
        if module == "jax._src.array" and name == "_reconstruct_array":
            return _jax_array
        if module.split(".")[0] == "numpy" and name in _NUMPY_OK:
            return super().find_class(module, name)
        if module == "builtins" and name in _BUILTINS_OK:
            return super().find_class(module, name)
        if (module, name) in {("collections", "OrderedDict"), ("copyreg", "_reconstructor"),
                              ("_codecs", "encode")}:
            return super().find_class(module, name)
        return type(name, (PickledObject,), {"_module": module, "_qualname": name})


def loads(data: bytes) -> Any:
    """Unpickles one member of a reference run file (see the module docstring)."""
    return _ReferenceUnpickler(io.BytesIO(data)).load()


@dataclass
class ReferenceRun:
    """The members of a reference run file. ``params`` is the haiku tree with numpy arrays;
    ``mcmc_state`` the pickled MCMCState record (``mcmc.py:21-34``), or None."""

    params: Optional[Dict[str, Dict[str, np.ndarray]]] = None
    mcmc_state: Optional[PickledObject] = None
    clipping_state: Any = None
    metadata: Any = None
    config_yaml: Optional[str] = None
    other: Dict[str, Any] = field(default_factory=dict)

    def walkers(self) -> Optional[Dict[str, Any]]:
        """r, log psi^2, walker ages, step size, step number and running acceptance of the
        stored chain (the jax PRNG state has no Philox counterpart and is not returned)."""
        if self.mcmc_state is None:
            return None
        s = self.mcmc_state.state if isinstance(self.mcmc_state, PickledObject) else vars(self.mcmc_state)
        keys = ("r", "log_psi_sqr", "walker_age", "stepsize", "step_nr", "acc_rate")
        return {k: (np.asarray(s[k]) if k in ("r", "log_psi_sqr", "walker_age") else s[k]) for k in keys if k in s}


def load_run(path) -> ReferenceRun:
    """Reads a reference run file (``checkpoints.py:71-91``)."""
    run = ReferenceRun()
    with zipfile.ZipFile(path, "r") as zf:
        for member in zf.namelist():
            stem, _, ext = member.rpartition(".")
            if ext == "yml" and stem == "config":
                run.config_yaml = zf.read(member).decode("utf-8")
            elif ext == "pkl":
                obj = loads(zf.read(member))
                if stem in ("params", "mcmc_state", "clipping_state", "metadata"):
                    setattr(run, stem, obj)
                else:
                    run.other[stem] = obj
    if run.params is not None:
        run.params = {k: {p: np.asarray(v) for p, v in _as_mapping(d).items()}
                      for k, d in _as_mapping(run.params).items()}
    return run


def _as_mapping(obj) -> Mapping:
    """A dict from a pickled mapping: a plain dict, or a record of a mapping class (older
    haiku trees pickle as their own FlatMapping class) holding its items as state or argument."""
    if isinstance(obj, Mapping):
        return obj
    if isinstance(obj, PickledObject):
        if isinstance(obj.state, Mapping) and obj.state:
            return obj.state
        for a in obj.args:
            try:
                return dict(a)
            except (TypeError, ValueError):
                continue
    raise TypeError(f"not a mapping: {obj!r}")


def save_params(path, params: Mapping[str, np.ndarray], a: Arch, metadata: Optional[dict] = None) -> None:
    """Writes a run file holding ``params.pkl`` (the haiku tree, numpy float32 arrays, as
    ``run_tools/convert_checkpoint.py`` stores them) and optionally ``metadata.pkl``; the
    reference's ``load_run`` reads it (members it does not find stay None)."""
    with zipfile.ZipFile(path, "w", zipfile.ZIP_BZIP2) as zf:
        with zf.open("params.pkl", "w", force_zip64=True) as f:
            pickle.dump(params_to_haiku(params, a), f)
        if metadata is not None:
            with zf.open("metadata.pkl", "w", force_zip64=True) as f:
                pickle.dump(dict(metadata), f)
