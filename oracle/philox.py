"""ORACLE -- test infrastructure only.

Philox4x32-10 counter-based generator (Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3", SC'11), restated from the
published algorithm in numpy uint32/uint64 arithmetic, and the Box-Muller
normals the GPU Langevin integrator draws from it.  Checked against the
paper's reference implementation's published known-answer vectors in
tests/test_oracle_md.py.
"""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)      # round multipliers
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)      # key schedule (Weyl) increments
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: uint32 array [..., 4]; key: uint32 array [..., 2] -> uint32 [..., 4]."""
    c = [np.asarray(ctr[..., i], dtype=np.uint32).copy() for i in range(4)]
    k0 = np.asarray(key[..., 0], dtype=np.uint32).copy()
    k1 = np.asarray(key[..., 1], dtype=np.uint32).copy()
    with np.errstate(over="ignore"):
        for r in range(10):
            p0 = M0 * c[0].astype(np.uint64)
            p1 = M1 * c[2].astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & MASK).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & MASK).astype(np.uint32)
            c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
            if r < 9:
                k0 = k0 + W0
                k1 = k1 + W1
    return np.stack(c, axis=-1)


def langevin_normals(seed: int, step: int, n_atoms: int) -> np.ndarray:
    """Standard normals [n_atoms, 3] of one Langevin step: counter
    (step low, step high, atom, 0), key (seed low, seed high); uniforms
    u = (x + 0.5) / 2^32; Box-Muller on (u0, u1) and (u2, u3), the first
    three normals used."""
    a = np.arange(n_atoms, dtype=np.uint64)
    ctr = np.zeros((n_atoms, 4), dtype=np.uint32)
    ctr[:, 0] = np.uint32(step & 0xFFFFFFFF)
    ctr[:, 1] = np.uint32((step >> 32) & 0xFFFFFFFF)
    ctr[:, 2] = a.astype(np.uint32)
    key = np.zeros((n_atoms, 2), dtype=np.uint32)
    key[:, 0] = np.uint32(seed & 0xFFFFFFFF)
    key[:, 1] = np.uint32((seed >> 32) & 0xFFFFFFFF)
    x = philox4x32_10(ctr, key).astype(np.float64)
    u = (x + 0.5) * 2.0 ** -32
    r0 = np.sqrt(-2.0 * np.log(u[:, 0]))
    r1 = np.sqrt(-2.0 * np.log(u[:, 2]))
    t0 = 2.0 * np.pi * u[:, 1]
    t1 = 2.0 * np.pi * u[:, 3]
    return np.stack([r0 * np.cos(t0), r0 * np.sin(t0), r1 * np.cos(t1)], axis=1)


def vec_normals(seed: int, step: int, n_atoms: int) -> np.ndarray:
    """The six standard normals [n_atoms, 6] per atom of one step of the
    Vanden-Eijnden-Ciccotti Langevin integrator (xi: columns 0-2, eta:
    3-5): two Philox blocks with counters (step low, step high, atom, 1) and
    (..., 2), key (seed low, seed high); Box-Muller on (u0, u1) and (u2, u3)
    of each block, cosine then sine."""
    a = np.arange(n_atoms, dtype=np.uint64)
    key = np.zeros((n_atoms, 2), dtype=np.uint32)
    key[:, 0] = np.uint32(seed & 0xFFFFFFFF)
    key[:, 1] = np.uint32((seed >> 32) & 0xFFFFFFFF)
    out = []
    for word in (1, 2):
        ctr = np.zeros((n_atoms, 4), dtype=np.uint32)
        ctr[:, 0] = np.uint32(step & 0xFFFFFFFF)
        ctr[:, 1] = np.uint32((step >> 32) & 0xFFFFFFFF)
        ctr[:, 2] = a.astype(np.uint32)
        ctr[:, 3] = np.uint32(word)
        u = (philox4x32_10(ctr, key).astype(np.float64) + 0.5) * 2.0 ** -32
        r0, r1 = np.sqrt(-2.0 * np.log(u[:, 0])), np.sqrt(-2.0 * np.log(u[:, 2]))
        t0, t1 = 2.0 * np.pi * u[:, 1], 2.0 * np.pi * u[:, 3]
        out += [r0 * np.cos(t0), r0 * np.sin(t0), r1 * np.cos(t1), r1 * np.sin(t1)]
    return np.stack(out[:6], axis=1)
