"""Test helpers: seeded random inputs and error measures."""
import numpy as np


def haar(rng, d):
    """Haar-random unitary: QR of a complex Ginibre matrix with the phases of
    R's diagonal moved into Q (Mezzadri 2007)."""
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def gaussian_matrix(rng, d):
    return rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))


def gaussian_state(rng, num_amps, normalise=False):
    a = rng.normal(size=num_amps) + 1j * rng.normal(size=num_amps)
    if normalise:
        a /= np.linalg.norm(a)
    return a


def rel_err(got, ref):
    """max |got - ref| / max |ref| (NaN counts as failure)."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    d = np.max(np.abs(got - ref))
    if not np.isfinite(d):
        return np.inf
    return float(d / max(np.max(np.abs(ref)), 1e-300))


# tolerances per precision, relative to the largest amplitude
TOL = {"c128": 1e-12, "c128_native": 1e-13, "c64": 2e-5}
