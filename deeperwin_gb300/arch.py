"""Architecture, molecules and walker initialisation for the DPE4 VMC inner loop.

The network is DeepErwin's "dpe4" model with a Jastrow factor enabled:

* features: ``model/input_features.py:112-303`` with ``InputFeatureConfigDPE4``
  (``configuration.py:652-660``): el-el feature = [dist], el-ion feature =
  [dist, dx, dy, dz], h_one = ion-major concat of el-ion features, ion lookup
  embedding of width 32.
* embedding: ``model/embeddings/ferminet_embedding.py:191-267`` with
  ``EmbeddingConfigDeepErwin4`` (``configuration.py:422-440``): 4 iterations,
  1-el width 256, 2-el / el-ion width 32, same/diff 2-el streams, w-mapping,
  SchNet convolution features, spin averages of h_one.
* orbitals: ``model/orbitals/envelope_orbitals.py:39-127``, full_det, no bias.
* Jastrow: ``model/wavefunction.py:42-60`` with ``n_hidden=[64, 64]``.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np


@dataclasses.dataclass(frozen=True)
class Arch:
    """Static shape of one wavefunction model (one molecule size)."""

    n_el: int
    n_up: int
    n_ions: int
    n_dets: int
    z_min: int = 1
    z_max: int = 8
    width_one: int = 256      # n_hidden_one_el (configuration.py:426)
    width_two: int = 32       # n_hidden_two_el == n_hidden_el_ions == emb_dim
    width_ion: int = 32       # n_ion_features (configuration.py:588)
    jastrow: Tuple[int, ...] = (64, 64)
    n_iter: int = 4

    @property
    def n_dn(self) -> int:
        return self.n_el - self.n_up

    @property
    def n_orb_cols(self) -> int:
        """Columns of one backflow / envelope block: n_dets * n_el (full_det)."""
        return self.n_dets * self.n_el

    def in_width(self, it: int) -> int:
        """Width of the concatenated symmetric features entering h_el_{it}."""
        if it == 0:
            f = 4 * self.n_ions
            return 3 * f + self.width_two + 4
        return 3 * self.width_one + self.width_two + self.width_two

    def h_width(self, it: int) -> int:
        """Width of h_one entering iteration ``it``."""
        return 4 * self.n_ions if it == 0 else self.width_one

    def ei_width(self, it: int) -> int:
        """Width of the el-ion stream entering iteration ``it``."""
        return 4 if it == 0 else self.width_two

    def ee_width(self, it: int) -> int:
        """Width of the same/diff 2-el streams entering iteration ``it``."""
        return 1 if it == 0 else self.width_two

    def validate(self) -> None:
        if not (1 <= self.n_up <= self.n_el - 1):
            raise ValueError("need at least one electron of each spin (n_up in [1, n_el-1])")
        if self.n_el > 64:
            raise ValueError("n_el > 64 is not supported")
        if self.n_ions < 1 or self.n_ions > 16:
            raise ValueError("n_ions must be in [1, 16]")
        if self.width_one % 64 or self.width_two != 32 or self.width_ion != 32:
            raise ValueError("width_one must be a multiple of 64, width_two and width_ion must be 32")
        if self.n_iter != 4:
            raise ValueError("only the 4-iteration dpe4 embedding is supported")


@dataclasses.dataclass
class Molecule:
    R: np.ndarray            # [N, 3] bohr
    Z: np.ndarray            # [N] int
    n_el: int
    n_up: int
    name: str = ""

    @property
    def n_ions(self) -> int:
        return len(self.Z)


def ordered_el_ion_mapping(Z: Sequence[int]) -> np.ndarray:
    """``spin_initialization="ordered"``: concat([i]*Z_i) (mcmc.py:52-53)."""
    return np.concatenate([[i] * int(z) for i, z in enumerate(Z)]).astype(np.int64)


def init_walkers(mol: Molecule, n_walkers: int, seed: int = 0) -> np.ndarray:
    """Gaussian walkers around nuclei, ``initialize_around_nuclei`` (mcmc.py:64-67).

    r0 = N(0, 1) + R[el_ion_mapping]. Uses numpy's PCG64 with the given seed (the
    reference draws from JAX threefry; the distribution is the same).
    """
    mapping = ordered_el_ion_mapping(mol.Z)
    if len(mapping) != mol.n_el:
        # charged systems: wrap the mapping around the ions
        mapping = np.resize(mapping, mol.n_el)
    rng = np.random.default_rng(seed)
    r0 = rng.standard_normal((n_walkers, mol.n_el, 3))
    return (r0 + np.asarray(mol.R, np.float64)[mapping][None]).astype(np.float64)


# ---------------------------------------------------------------------------
# The five workloads of the inner loop (LiH, H10, C2H4-shaped, serving, 40 e-)
# ---------------------------------------------------------------------------

def lih() -> Molecule:
    return Molecule(R=np.array([[0.0, 0, 0], [3.0, 0, 0]]), Z=np.array([3, 1]), n_el=4, n_up=2, name="LiH")


def h_chain(n: int = 10, spacing: float = 1.8) -> Molecule:
    R = np.zeros((n, 3))
    R[:, 0] = np.arange(n) * spacing
    return Molecule(R=R, Z=np.ones(n, np.int64), n_el=n, n_up=(n + 1) // 2, name=f"H{n}")


def c2h4_shaped() -> Molecule:
    R = np.array([[1.26, 0, 0], [-1.26, 0, 0],
                  [2.33, 1.76, 0], [2.33, -1.76, 0], [-2.33, 1.76, 0], [-2.33, -1.76, 0]])
    Z = np.array([6, 6, 1, 1, 1, 1])
    return Molecule(R=R, Z=Z, n_el=16, n_up=8, name="C2H4")


def _place_nuclei(rng: np.random.Generator, n: int, box: float = 6.0, min_dist: float = 1.5) -> np.ndarray:
    """Uniform positions in a ``box``-bohr cube, resampled until all pairs are >= min_dist."""
    while True:
        R = rng.uniform(0.0, box, size=(n, 3))
        d = np.linalg.norm(R[:, None] - R[None], axis=-1) + np.eye(n) * 1e9
        if d.min() >= min_dist:
            return R - R.mean(axis=0)


def random_molecule(rng: np.random.Generator, n_min: int = 2, n_max: int = 8,
                    z_choices: Sequence[int] = (1, 6, 7, 8)) -> Molecule:
    """Serving-stream molecule: 2-8 nuclei, Z from {1,6,7,8}, 6-bohr cube, pairs >= 1.5 bohr.

    Neutral; n_up = ceil(n_el / 2). The draw is repeated until 2 <= n_el <= 30.
    """
    while True:
        n = int(rng.integers(n_min, n_max + 1))
        Z = rng.choice(np.asarray(z_choices), size=n)
        n_el = int(Z.sum())
        if 2 <= n_el <= 30:
            break
    R = _place_nuclei(rng, n)
    return Molecule(R=R, Z=Z.astype(np.int64), n_el=n_el, n_up=(n_el + 1) // 2, name=f"rand{n}")


def scale_molecule(seed: int = 7) -> Molecule:
    """40-electron molecule: 6 heavy nuclei Z in {6,7,8} plus H atoms up to 40 electrons.

    The heavy charges are redrawn until their sum is <= 40 - 1 (at least one H) and the
    number of H atoms keeps the nucleus count <= 16. Positions as for the serving
    stream (6-bohr cube, pairs >= 1.5 bohr; the cube grows by 1 bohr per failed
    1000 draws so that many nuclei fit).
    """
    rng = np.random.default_rng(seed)
    while True:
        Zh = rng.choice(np.array([6, 7, 8]), size=6)
        n_h = 40 - int(Zh.sum())
        if 1 <= n_h <= 10:
            break
    Z = np.concatenate([Zh, np.ones(n_h, np.int64)])
    box = 6.0
    for attempt in range(100000):
        R = rng.uniform(0.0, box, size=(len(Z), 3))
        d = np.linalg.norm(R[:, None] - R[None], axis=-1) + np.eye(len(Z)) * 1e9
        if d.min() >= 1.5:
            break
        if attempt % 1000 == 999:
            box += 1.0
    R = R - R.mean(axis=0)
    return Molecule(R=R, Z=Z.astype(np.int64), n_el=40, n_up=20, name="scale40")


@dataclasses.dataclass(frozen=True)
class Workload:
    name: str
    mol_fn: object
    n_dets: int
    n_walkers: int
    n_mh_steps: int
    precision: str           # "fp32" (plain) or "mixed"
    step_size: float = 0.1
    backward: bool = False   # the step also forms the clipped VMC gradient (hand-written backward)


WORKLOADS = {
    "lih": Workload("lih_4e_k8_b2048_fp32", lih, 8, 2048, 10, "fp32"),
    "h10": Workload("h10_10e_k16_b8192_mixed", h_chain, 16, 8192, 10, "mixed"),
    "c2h4": Workload("c2h4_16e_k32_b4096_mixed_grad", c2h4_shaped, 32, 4096, 10, "mixed", backward=True),
    "scale40": Workload("scale_40e_k64_b16384_mixed_grad", scale_molecule, 64, 16384, 10, "mixed", backward=True),
}


def arch_for(mol: Molecule, n_dets: int, z_min: int = 1, z_max: Optional[int] = None) -> Arch:
    if z_max is None:
        z_max = int(max(mol.Z))
    a = Arch(n_el=mol.n_el, n_up=mol.n_up, n_ions=mol.n_ions, n_dets=n_dets, z_min=z_min, z_max=z_max)
    a.validate()
    return a
