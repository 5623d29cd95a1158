"""Deterministic test states for the sampling boundary fixtures, built from
integer hashing (splitmix64) so that every platform makes the same bits
without storing the state: amplitude k = (u1 - 1/2) + i (u2 - 1/2) times a
power of two, with u1, u2 the top 53 bits of two hashes of k.  The state is
not normalised: its total probability is below 1, so uniforms above it
exercise the end of the reference's walk too."""
import numpy as np

_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M
    return z ^ (z >> np.uint64(31))


def _unit(h):
    return (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def hash_state(num_amps: int, seed: int) -> np.ndarray:
    """num_amps complex128 amplitudes; sum |a|^2 is about num_amps / 6 * scale^2
    with scale = 2^-ceil(log4(num_amps / 6)): a total between 1/4 and 1."""
    k = np.arange(num_amps, dtype=np.uint64)
    s = np.uint64(seed) * np.uint64(0x100000001B3)
    with np.errstate(over="ignore"):
        u1 = _unit(_splitmix(k * np.uint64(2) + s))
        u2 = _unit(_splitmix(k * np.uint64(2) + np.uint64(1) + s))
    scale = 2.0 ** -int(np.ceil(np.log2(num_amps / 6.0) / 2)) if num_amps >= 6 else 1.0
    return ((u1 - 0.5) + 1j * (u2 - 0.5)) * scale


def reference_walk(prob: np.ndarray, index_size: int):
    """The reference's sums in its own order (QubitVector::sample_measure,
    qubitvector.hpp:2148-2228): block totals, the running block prefix P and,
    per block, the walk from P[j]; numpy's accumulate is sequential and its
    elementwise products are rounded separately, as the reference's are."""
    n_amps = prob.size
    nb = 1 << index_size
    if n_amps < nb:
        return None, None, np.add.accumulate(prob)
    L = n_amps // nb
    idxs = np.array([np.add.accumulate(prob[j * L:(j + 1) * L])[-1] for j in range(nb)])
    P = np.concatenate([[0.0], np.add.accumulate(idxs)])
    walk = np.concatenate([np.add.accumulate(np.concatenate([[P[j]], prob[j * L:(j + 1) * L]]))[1:]
                           for j in range(nb)])
    return idxs, P, walk
