"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (blob phantoms, random B-spline deformations,
multiplicative bias fields).  Arrays are indexed [z, y, x] / [y, x].

No public dataset is involved: the phantoms stand in for the clinical
series the reference's registration programs are used on.
"""
import numpy as np


def blob_phantom(shape, nblobs, sigma=(4.0, 12.0), amp=(50.0, 200.0), noise=2.0, seed=0):
    """Sum of isotropic Gaussian blobs with uniform centres, sigma and
    amplitude, plus N(0, noise) noise; float32."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape)
    grids = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in shape], indexing="ij")
    img = np.zeros(shape)
    for _ in range(nblobs):
        c = [rng.uniform(0, n) for n in shape]
        s = rng.uniform(*sigma)
        a = rng.uniform(*amp)
        r2 = sum((g - ci) ** 2 for g, ci in zip(grids, c))
        img += a * np.exp(-r2 / (2 * s * s))
    img += rng.normal(0.0, noise, size=shape)
    return img.astype(np.float32)


def bias_field(shape, sigma=0.1, seed=0):
    """exp of a degree-2 polynomial in coordinates normalised to [-1, 1]
    with N(0, sigma) coefficients."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape)
    axes = [np.linspace(-1.0, 1.0, n) for n in shape]
    g = np.meshgrid(*axes, indexing="ij")
    terms = [np.ones(shape)] + list(g)
    for i in range(len(g)):
        for j in range(i, len(g)):
            terms.append(g[i] * g[j])
    coef = rng.normal(0.0, sigma, size=len(terms))
    return np.exp(sum(c * t for c, t in zip(coef, terms))).astype(np.float32)


def spline_params(ncoef_nodes, dim, sigma, clip, seed=0):
    """Interleaved spline coefficient vector, N(0, sigma) clipped to +-clip."""
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, sigma, size=ncoef_nodes * dim)
    return np.clip(p, -clip, clip)


def smooth_params(csize_xyz, amplitude, seed=0, interior=True):
    """Smooth random coefficients (low-frequency sines) of amplitude
    `amplitude`; zero on the border coefficients when `interior`."""
    rng = np.random.default_rng(seed)
    dim = len(csize_xyz)
    shape = tuple(csize_xyz[::-1])
    g = np.meshgrid(*[np.linspace(0, 1, n) for n in shape], indexing="ij")
    out = np.zeros(shape + (dim,))
    for c in range(dim):
        ph = rng.uniform(0, 2 * np.pi, size=dim)
        fr = rng.uniform(0.5, 1.5, size=dim)
        v = np.ones(shape)
        for k in range(dim):
            v = v * np.sin(2 * np.pi * fr[k] * g[k] + ph[k])
        out[..., c] = amplitude * v
    return out.reshape(-1)
