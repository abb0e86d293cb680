"""Parameter tree of the DPE4 model, its seeded initialisation and the packed layout.

The names follow the haiku module nesting of the reference (``wf/...`` paths in
``model/wavefunction.py:346-353``), shortened. Every dense layer is stored as
haiku's ``Linear``: ``w[d_in, d_out]`` with ``y = x @ w + b``
(``model/mlp.py:57-62``).

The packed layout is one flat float32 vector: the tensors below in list order,
each row-major, each starting at a multiple of 64 floats (256 bytes). The same
order is computed by the C library (``dw_param_layout``); a CPU test checks that
the two agree.
"""
from __future__ import annotations

from collections import OrderedDict
from typing import Dict, List, Tuple

import numpy as np

from .arch import Arch

ALIGN = 64  # floats


def param_shapes(a: Arch) -> "OrderedDict[str, Tuple[int, ...]]":
    """Ordered name -> shape for every trainable tensor of the model."""
    e = a.width_two
    s: "OrderedDict[str, Tuple[int, ...]]" = OrderedDict()
    s["ion_embed"] = (a.z_max - a.z_min + 1, a.width_ion)   # input_features.py:185-190
    for it in range(a.n_iter):
        p = f"symm{it}"
        # ConvolutionalFeatures (ferminet_embedding.py:137-158, 172-174)
        s[f"{p}.w_same.w"] = (a.ee_width(it), e)
        s[f"{p}.w_same.b"] = (e,)
        s[f"{p}.w_diff.w"] = (a.ee_width(it), e)
        s[f"{p}.w_diff.b"] = (e,)
        s[f"{p}.h_map.w"] = (a.h_width(it), e)
        s[f"{p}.h_map.b"] = (e,)
        s[f"{p}.h_ion_map.w"] = (a.width_ion, a.ei_width(it))
        s[f"{p}.h_ion_map.b"] = (a.ei_width(it),)
        # h_el MLP (ferminet_embedding.py:233-241)
        s[f"h_el{it}.w"] = (a.in_width(it), a.width_one)
        s[f"h_el{it}.b"] = (a.width_one,)
        if it < a.n_iter - 1:
            # 2-el and el-ion streams (ferminet_embedding.py:247-262)
            s[f"h_same{it}.w"] = (a.ee_width(it), e)
            s[f"h_same{it}.b"] = (e,)
            s[f"h_diff{it}.w"] = (a.ee_width(it), e)
            s[f"h_diff{it}.b"] = (e,)
            s[f"h_ei{it}.w"] = (a.ei_width(it), e)
            s[f"h_ei{it}.b"] = (e,)
    # EnvelopeOrbitals (envelope_orbitals.py:46-70, 99-104)
    s["bf_up.w"] = (a.width_one, a.n_orb_cols)
    s["bf_dn.w"] = (a.width_one, a.n_orb_cols)
    s["alpha_up"] = (a.n_ions, a.n_orb_cols)
    s["alpha_dn"] = (a.n_ions, a.n_orb_cols)
    s["weights_up"] = (a.n_ions, a.n_orb_cols)
    s["weights_dn"] = (a.n_ions, a.n_orb_cols)
    # JastrowFactor MLP([64, 64, 1], linear_out, no output bias) (wavefunction.py:58)
    dims = (a.width_one,) + tuple(a.jastrow) + (1,)
    for l in range(len(dims) - 1):
        s[f"jas{l}.w"] = (dims[l], dims[l + 1])
        if l < len(dims) - 2:
            s[f"jas{l}.b"] = (dims[l + 1],)
    return s


def layout(a: Arch) -> Tuple["OrderedDict[str, Tuple[int, int]]", int]:
    """name -> (offset, size) in floats, and the total packed length."""
    off = 0
    out: "OrderedDict[str, Tuple[int, int]]" = OrderedDict()
    for name, shape in param_shapes(a).items():
        size = int(np.prod(shape))
        out[name] = (off, size)
        off += (size + ALIGN - 1) // ALIGN * ALIGN
    return out, off


def init_params(a: Arch, seed: int = 0, bias_std: float = 0.0, envelope_jitter: float = 0.0
                ) -> Dict[str, np.ndarray]:
    """Seeded init: weights N(0, 1/fan_in), biases N(0, bias_std^2) (0 by default, as
    ``MLPConfig.init_bias_scale=0``), envelope alpha = weights = 1 (``envelope_orbitals.py:34-37``)
    optionally jittered, ion embedding N(0, 1). numpy PCG64, so x86 and Arm hosts agree.
    """
    rng = np.random.default_rng(seed)
    p: Dict[str, np.ndarray] = {}
    for name, shape in param_shapes(a).items():
        if name == "ion_embed":
            v = rng.standard_normal(shape)
        elif name.startswith(("alpha_", "weights_")):
            v = np.ones(shape)
            if envelope_jitter:
                v = v + envelope_jitter * rng.standard_normal(shape)
        elif name.endswith(".b"):
            v = bias_std * rng.standard_normal(shape) if bias_std else np.zeros(shape)
        else:
            v = rng.standard_normal(shape) / np.sqrt(shape[0])
        p[name] = v.astype(np.float64)
    return p


def pack(a: Arch, params: Dict[str, np.ndarray]) -> np.ndarray:
    lay, total = layout(a)
    flat = np.zeros(total, np.float32)
    for name, (off, size) in lay.items():
        v = np.asarray(params[name], np.float32).reshape(-1)
        if v.size != size:
            raise ValueError(f"{name}: expected {size} values, got {v.size}")
        flat[off:off + size] = v
    return flat


def unpack(a: Arch, flat: np.ndarray) -> Dict[str, np.ndarray]:
    lay, _ = layout(a)
    shapes = param_shapes(a)
    return {n: np.asarray(flat[o:o + s], np.float64).reshape(shapes[n]) for n, (o, s) in lay.items()}


def slice_shared(big: Arch, params: Dict[str, np.ndarray], small: Arch) -> Dict[str, np.ndarray]:
    """Per-molecule view of weights generated for (N_max, n_max): the first N ion blocks of
    the ion-dependent input rows and the first n orbital columns per determinant.

    This is the weight-sharing rule of the serving path (the reference has no envelope-orbital
    mechanism for it).
    """
    if small.n_dets != big.n_dets or small.n_ions > big.n_ions or small.n_el > big.n_el:
        raise ValueError("small arch must fit inside the shared one")
    out: Dict[str, np.ndarray] = {}
    Nb, N = big.n_ions, small.n_ions
    K, nb, n = big.n_dets, big.n_el, small.n_el
    for name, v in params.items():
        if name == "ion_embed":
            v = v[small.z_min - big.z_min: small.z_max - big.z_min + 1]
        elif name == "h_el0.w":
            f_b, f_s = 4 * Nb, 4 * N
            blocks = [v[k * f_b:k * f_b + f_s] for k in range(3)]
            v = np.concatenate(blocks + [v[3 * f_b:]], axis=0)
        elif name == "symm0.h_map.w":
            v = v[:4 * N]
        elif name in ("bf_up.w", "bf_dn.w"):
            v = v.reshape(v.shape[0], K, nb)[:, :, :n].reshape(v.shape[0], K * n)
        elif name.startswith(("alpha_", "weights_")):
            v = v.reshape(Nb, K, nb)[:N, :, :n].reshape(N, K * n)
        out[name] = v.copy()
    return out
