"""numpy restatement of the library's Philox-4x32-10 / Box-Muller draws (test infrastructure):
lets the oracle replay exactly the proposals and uniforms that the MCMC kernel used."""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, seed):
    c = [np.asarray(x, np.uint64) & MASK for x in (c0, c1, c2, c3)]
    k0, k1 = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [(hi1 ^ c[1] ^ np.uint64(k0)) & MASK, lo1, (hi0 ^ c[3] ^ np.uint64(k1)) & MASK, lo0]
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c


def _unit(u):
    return ((u >> np.uint64(8)).astype(np.float32) + np.float32(0.5)) * np.float32(1.0 / 16777216.0)


def _box_muller(a, b):
    u1, u2 = _unit(a), _unit(b)
    rad = np.sqrt(np.float32(-2.0) * np.log(u1))
    ang = np.float64(2.0 * np.pi) * u2.astype(np.float64)
    return (rad * np.cos(ang)).astype(np.float32), (rad * np.sin(ang)).astype(np.float32)


def proposal_noise(seed, n_walkers, n_el, step):
    n3 = 3 * n_el
    groups = (n3 + 3) // 4
    w = np.repeat(np.arange(n_walkers, dtype=np.uint64), groups)
    g = np.tile(np.arange(groups, dtype=np.uint64), n_walkers)
    x = philox4x32_10(w, np.full_like(w, step), g, np.full_like(w, 0xA511E9B3), seed)
    n0, n1 = _box_muller(x[0], x[1])
    n2, n3_ = _box_muller(x[2], x[3])
    z = np.stack([n0, n1, n2, n3_], -1).reshape(n_walkers, groups * 4)[:, :n3]
    return z.reshape(n_walkers, n_el, 3)


def accept_uniform(seed, n_walkers, step):
    w = np.arange(n_walkers, dtype=np.uint64)
    x = philox4x32_10(w, np.full_like(w, step), np.zeros_like(w), np.full_like(w, 0x63D83595), seed)
    return _unit(x[0])


def uniforms4(seed, n_walkers, step, group, tag):
    """Four uniforms per walker for Philox counter {walker, step, group, tag}: [n_walkers, 4]."""
    w = np.arange(n_walkers, dtype=np.uint64)
    x = philox4x32_10(w, np.full_like(w, step), np.full_like(w, group), np.full_like(w, tag), seed)
    return np.stack([_unit(v) for v in x], -1)


def cauchy_uniforms(seed, n_walkers, n_el, step):
    """The uniforms behind the Cauchy proposal of each coordinate: [n_walkers, n_el, 3]."""
    n3 = 3 * n_el
    groups = (n3 + 3) // 4
    u = np.stack([uniforms4(seed, n_walkers, step, g, 0xC4A3B1E7) for g in range(groups)], 1)
    return u.reshape(n_walkers, groups * 4)[:, :n3].reshape(n_walkers, n_el, 3)


def spin_uniforms(seed, n_walkers, step):
    """(select, up index, down index, flip) uniforms of the spin swap / flip: [n_walkers, 4]."""
    return uniforms4(seed, n_walkers, step, 0, 0x5F1A9C3D)
