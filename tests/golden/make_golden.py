"""Generate golden vectors by executing the reference's own source code.

The reference is JAX/haiku code; neither library is installed here. Its model files,
however, only use array operations, haiku's Module/Linear/Embed/get_parameter and
``jax.nn.softplus``. This script supplies a small numpy stand-in for those names, takes
the reference's function and class definitions verbatim from its source files (with
``ast``, so the unrelated heavy imports of those files - pyscf, folx, kfac - are never
executed), and runs them in float64 on seeded weights and walkers.

Run from the repository root with the reference checked out:

    python tests/golden/make_golden.py /path/to/deeperwin [case ...]

It writes ``tests/golden/*.npz``. The fixtures hold the walkers, nuclei, the seed and
init settings of the weights (weights are regenerated by
``deeperwin_gb300.params.init_params``; a checksum of the packed weights is stored to
catch drift) and the reference's outputs: log psi^2, phase, the Slater matrices, the
potential energy and the energy-clipping statistics. It also writes
``tests/golden/haiku_paths_lih_k8.txt``: every parameter path (module nesting as the stand-in
names it, without haiku's "~" markers) and shape that the reference's modules request for the
LiH case; ``--paths-only`` writes that list alone.
"""
from __future__ import annotations

import ast
import enum
import re
import sys
import types
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from deeperwin_gb300 import arch as A  # noqa: E402
from deeperwin_gb300 import params as P  # noqa: E402

# --------------------------------------------------------------------------- numpy stand-ins
_STACK: list = []
_COUNTS: dict = {}
_PROVIDER = {"fn": None}


def _fix_axis(kw):
    if isinstance(kw.get("axis"), list):
        kw["axis"] = tuple(kw["axis"])
    return kw


class _JNP(types.ModuleType):
    def __getattr__(self, item):
        return getattr(np, item)

    def sum(self, x, *a, **kw):
        return np.sum(x, *a, **_fix_axis(kw))

    def mean(self, x, *a, **kw):
        return np.mean(x, *a, **_fix_axis(kw))

    def max(self, x, *a, **kw):
        return np.max(x, *a, **_fix_axis(kw))

    def nanmean(self, x, *a, **kw):
        return np.nanmean(x, *a, **_fix_axis(kw))


jnp = _JNP("jax.numpy")
jax = types.ModuleType("jax")
jax.numpy = jnp
jax.Array = np.ndarray
jax.nn = types.SimpleNamespace(softplus=lambda x: np.logaddexp(0.0, x),
                               one_hot=lambda x, n: np.eye(n)[x], silu=None, elu=None, relu=None, gelu=None)


def _snake(name):
    return re.sub(r"(?<!^)(?=[A-Z])", "_", name).lower()


class Module:
    def __init__(self, name=None):
        parent = _STACK[-1] if _STACK else ""
        base = name or _snake(type(self).__name__)
        path = f"{parent}/{base}" if parent else base
        c = _COUNTS.get(path, 0)
        _COUNTS[path] = c + 1
        self.module_name = path if c == 0 else f"{path}_{c}"
        _STACK.append(self.module_name)

    def __init_subclass__(cls, **kw):
        super().__init_subclass__(**kw)
        for k, v in list(cls.__dict__.items()):
            if not callable(v) or isinstance(v, type):
                continue
            if k == "__init__":
                setattr(cls, k, _wrap_init(v))
            elif k == "__call__" or not k.startswith("__"):
                setattr(cls, k, _wrap_method(v))


def _wrap_init(f):
    def g(self, *a, **k):
        depth = len(_STACK)
        try:
            return f(self, *a, **k)
        finally:
            del _STACK[depth:]
    return g


def _wrap_method(f):
    def g(self, *a, **k):
        _STACK.append(self.module_name)
        try:
            return f(self, *a, **k)
        finally:
            _STACK.pop()
    g.__name__ = getattr(f, "__name__", "f")
    return g


def get_parameter(name, shape, dtype=None, init=None):
    path = f"{_STACK[-1]}/{name}"
    v = _PROVIDER["fn"](path, tuple(shape))
    assert v.shape == tuple(shape), (path, v.shape, shape)
    return v


class Linear(Module):
    def __init__(self, output_size, with_bias=True, w_init=None, b_init=None, name=None):
        super().__init__(name=name)
        self.output_size = output_size
        self.with_bias = with_bias

    def __call__(self, x):
        w = get_parameter("w", [x.shape[-1], self.output_size])
        y = x @ w
        if self.with_bias:
            y = y + get_parameter("b", [self.output_size])
        return y


class EmbedLookupStyle(enum.Enum):
    ARRAY_INDEX = 1
    ONE_HOT = 2


class Embed(Module):
    def __init__(self, vocab_size, embed_dim, lookup_style=None, name=None):
        super().__init__(name=name)
        self.shape = (vocab_size, embed_dim)

    def __call__(self, ids):
        return get_parameter("embeddings", list(self.shape))[np.asarray(ids)]


class _Init:
    def __init__(self, *a, **k):
        pass


hk = types.ModuleType("haiku")
hk.Module = Module
hk.Linear = Linear
hk.Embed = Embed
hk.EmbedLookupStyle = EmbedLookupStyle
hk.get_parameter = get_parameter
hk.initializers = types.SimpleNamespace(VarianceScaling=_Init, TruncatedNormal=_Init)
hk.experimental = types.SimpleNamespace(name_like=lambda _n: (lambda f: f))
hk.LayerNorm = None


def _install_fake_modules():
    ruamel = types.ModuleType("ruamel")
    yaml = types.ModuleType("ruamel.yaml")

    class _YAML:
        def load(self, *_a, **_k):
            return {}

        def dump(self, *_a, **_k):
            pass
    yaml.YAML = _YAML
    yaml.comments = types.ModuleType("ruamel.yaml.comments")
    ruamel.yaml = yaml
    sys.modules.update({"ruamel": ruamel, "ruamel.yaml": yaml, "ruamel.yaml.comments": yaml.comments})


def _extract(path: Path, names, g: dict):
    """Execute only the named top-level definitions of ``path`` in namespace ``g``."""
    tree = ast.parse(path.read_text())
    body = [n for n in tree.body
            if isinstance(n, (ast.FunctionDef, ast.ClassDef)) and n.name in names]
    missing = set(names) - {n.name for n in body}
    if missing:
        raise RuntimeError(f"{path}: definitions not found: {missing}")
    mod = ast.Module(body=body, type_ignores=[])
    exec(compile(mod, str(path), "exec"), g)
    return g


def load_reference(src: Path) -> dict:
    """Returns a namespace with the reference's model/Hamiltonian/clipping definitions."""
    _install_fake_modules()
    dw = src / "src" / "deeperwin" if (src / "src").exists() else src
    cfg_mod = types.ModuleType("deeperwin_reference_configuration")
    cfg_mod.__file__ = str(dw / "configuration.py")
    sys.modules[cfg_mod.__name__] = cfg_mod
    exec(compile((dw / "configuration.py").read_text(), str(dw / "configuration.py"), "exec"), cfg_mod.__dict__)
    cfg_ns = cfg_mod.__dict__
    cfg = cfg_mod

    from collections import namedtuple  # definitions.py is plain namedtuples
    g: dict = {"jax": jax, "jnp": jnp, "np": np, "hk": hk, "haiku": hk, "functools": __import__("functools"),
               "Optional": object, "Dict": dict, "Tuple": tuple, "List": list, "Literal": object,
               "Iterable": object, "Callable": __import__("collections.abc").abc.Callable, "namedtuple": namedtuple}
    g.update({k: v for k, v in cfg_ns.items() if not k.startswith("__")})
    exec(compile((dw / "model" / "definitions.py").read_text(), "definitions.py", "exec"), g)
    _extract(dw / "utils" / "utils.py",
             ["get_el_ion_distance_matrix", "get_full_distance_matrix", "get_distance_matrix"], g)
    g.update(get_periodic_distance_matrix=None, get_periodic_el_ion_distance_matrix=None,
             append_across_leading_dims=None, register_scale_and_shift=lambda x, *a, **k: x,
             TransferableAtomicOrbitals=None, PeriodicEnvelopeOrbitals=None, BlochWaveEnvelope=None,
             MoonEmbedding=None, GNNEmbedding=None, TransformerEmbedding=None, AxialTransformerEmbedding=None,
             pmean=lambda x: x)
    _extract(dw / "model" / "mlp.py", ["residual_update", "MLP", "get_activation", "get_rbf_features",
                                       "get_gauss_env_features"], g)
    _extract(dw / "model" / "input_features.py", ["PairwiseFeatures", "init_particle_features",
                                                  "InputPreprocessor"], g)
    _extract(dw / "model" / "embeddings" / "ferminet_embedding.py",
             ["ScalarSymmetricProduct", "SymmetricFeatures", "ConvolutionalFeatures", "FermiNetEmbedding"], g)
    _extract(dw / "model" / "orbitals" / "envelope_orbitals.py",
             ["EnvelopeOrbitals", "_determine_n_output_orbitals", "_determine_elec_idxs"], g)
    _extract(dw / "model" / "orbitals" / "orbital_net.py", ["OrbitalNet"], g)
    _extract(dw / "model" / "wavefunction.py",
             ["JastrowFactor", "evaluate_sum_of_determinants", "Wavefunction", "construct_wavefunction_definition"], g)
    _extract(dw / "hamiltonian.py", ["get_el_el_potential_energy", "get_ion_ion_potential_energy",
                                     "get_potential_energy"], g)
    _extract(dw / "optimization" / "loss_function.py",
             ["init_clipping_state", "_get_clipping_center_and_width", "_update_clipping_state",
              "_get_clip_func", "_clip_energies"], g)
    g["cfg"] = cfg
    return g


# --------------------------------------------------------------------------- name mapping
_MAP = [
    (r"/h_ion/embeddings$", lambda m: "ion_embed"),
    (r"symm_features_(\d)/convolutional_features/(w_same|w_diff|h_map|h_ion_map)/linear_0/(w|b)$",
     lambda m: f"symm{m[1]}.{m[2]}.{m[3]}"),
    (r"/h_el_(\d)/linear_0/(w|b)$", lambda m: f"h_el{m[1]}.{m[2]}"),
    (r"/h_same_(\d)/linear_0/(w|b)$", lambda m: f"h_same{m[1]}.{m[2]}"),
    (r"/h_diff_(\d)/linear_0/(w|b)$", lambda m: f"h_diff{m[1]}.{m[2]}"),
    (r"/h_el_ion_(\d)/linear_0/(w|b)$", lambda m: f"h_ei{m[1]}.{m[2]}"),
    (r"envelope_orbitals/(bf_up|bf_dn)/linear_0/w$", lambda m: f"{m[1]}.w"),
    (r"envelope_orbitals/(alpha_up|alpha_dn|weights_up|weights_dn)$", lambda m: m[1]),
    (r"jastrow_factor/mlp/linear_(\d)/(w|b)$", lambda m: f"jas{m[1]}.{m[2]}"),
]


def provider_for(params: dict, seen: set, requested: dict = None):
    def fn(path, shape):
        if requested is not None:
            requested[path] = tuple(shape)
        for pat, name_fn in _MAP:
            m = re.search(pat, path)
            if m:
                name = name_fn(m)
                seen.add(name)
                return np.asarray(params[name], np.float64)
        raise KeyError(f"unmapped reference parameter {path} {shape}")
    return fn


def reference_forward(g: dict, arch: A.Arch, params: dict, r, R, Z, requested: dict = None):
    cfg = g["cfg"]
    model_cfg = cfg.ModelConfigDeepErwin4(
        orbitals=cfg.OrbitalsConfigFermiNet(n_determinants=arch.n_dets),
        jastrow=cfg.JastrowConfig(n_hidden=list(arch.jastrow)),
        Z_min=arch.z_min, Z_max=arch.z_max)
    wdef = g["WavefunctionDefinition"](Z_max=arch.z_max, Z_min=arch.z_min)
    seen: set = set()
    _PROVIDER["fn"] = provider_for(params, seen, requested)
    _COUNTS.clear()
    _STACK.clear()
    wf = g["Wavefunction"](model_cfg, wdef)
    phase, lp = wf(arch.n_up, arch.n_dn, np.asarray(r), np.asarray(R), np.asarray(Z), {})
    _COUNTS.clear()
    _STACK.clear()
    wf2 = g["Wavefunction"](model_cfg, wdef)
    mo_up, mo_dn = wf2.get_slater_matrices(arch.n_up, arch.n_dn, np.asarray(r), np.asarray(R), np.asarray(Z), {})
    unused = set(params) - seen
    if unused:
        raise RuntimeError(f"parameters not consumed by the reference model: {sorted(unused)}")
    return phase, lp, np.concatenate([mo_up, mo_dn], axis=-2)


CASES = [
    # name, molecule, n_dets, n_walkers, bias_std, envelope_jitter, walkers whose Slater matrices are kept
    ("lih_k8", A.lih, 8, 8, 0.1, 0.2, None),
    ("h6_k4", lambda: A.h_chain(6), 4, 4, 0.1, 0.2, None),
    ("c2h4_k2", A.c2h4_shaped, 2, 3, 0.1, 0.2, None),
    ("h10_k16_plain_init", A.h_chain, 16, 3, 0.0, 0.0, None),
    # the contract shapes: C2H4-shaped with 32 determinants, the 40-electron molecule with 64
    ("c2h4_k32", A.c2h4_shaped, 32, 16, 0.1, 0.2, 2),
    ("scale40_k64", A.scale_molecule, 64, 4, 0.1, 0.2, 0),
]


def main(ref_root: str, paths_only: bool = False, only=None):
    g = load_reference(Path(ref_root))
    out_dir = Path(__file__).resolve().parent
    for name, mol_fn, K, B, bstd, jit, n_slater in CASES:
        if only and name not in only:
            continue
        mol = mol_fn()
        arch = A.arch_for(mol, K)
        params = P.init_params(arch, seed=0, bias_std=bstd, envelope_jitter=jit)
        r = A.init_walkers(mol, B, seed=1)
        requested: dict = {}
        phase, lp, mo = reference_forward(g, arch, params, r, mol.R, mol.Z, requested)
        if name == "lih_k8":
            # every parameter path the reference's modules request (the stand-in names modules by
            # nesting only, without haiku's "~" markers), with its shape
            with open(out_dir / "haiku_paths_lih_k8.txt", "w") as f:
                for path in sorted(requested):
                    f.write(f"{path}\t{','.join(map(str, requested[path]))}\n")
        if paths_only:
            continue
        e_pot = g["get_potential_energy"](r, np.asarray(mol.R, np.float64), np.asarray(mol.Z, np.float64))
        # clipping statistics on a fixed synthetic energy vector (loss_function.py:44-72)
        rng = np.random.default_rng(3)
        E = rng.standard_normal(64) * 2.0 - 8.0
        E[5] = 40.0
        clip_cfg = g["cfg"].ClippingConfig()
        clipped, (c_new, w_new) = g["_clip_energies"](E, (np.float64(-7.5), np.float64(3.0)), clip_cfg)
        packed = P.pack(arch, params)
        np.savez_compressed(
            out_dir / f"{name}.npz",
            n_el=arch.n_el, n_up=arch.n_up, n_dets=K, z_min=arch.z_min, z_max=arch.z_max,
            seed=0, bias_std=bstd, envelope_jitter=jit, packed_sum=np.float64(packed.astype(np.float64).sum()),
            packed_abs_sum=np.float64(np.abs(packed.astype(np.float64)).sum()),
            R=np.asarray(mol.R, np.float64), Z=np.asarray(mol.Z, np.int64), r=r,
            log_psi_sqr=np.asarray(lp, np.float64), phase=np.asarray(phase, np.float64),
            slater=np.asarray(mo, np.float64)[:n_slater], e_pot=np.asarray(e_pot, np.float64),
            clip_E=E, clip_in=np.array([-7.5, 3.0]), clip_out=np.asarray(clipped, np.float64),
            clip_state_out=np.array([c_new, w_new], np.float64))
        print(f"{name}: log_psi_sqr={np.asarray(lp)[:3]} e_pot={np.asarray(e_pot)[:3]}")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not args:
        sys.exit("usage: make_golden.py <path of the reference checkout> [case ...] [--paths-only]")
    main(args[0], paths_only="--paths-only" in sys.argv, only=set(args[1:]) or None)
