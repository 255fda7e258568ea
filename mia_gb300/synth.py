"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (blob phantoms, random B-spline deformations,
multiplicative bias fields).  Arrays are indexed [z, y, x] / [y, x].

No public dataset is involved: the phantoms stand in for the clinical
series the reference's registration programs are used on.
"""
import numpy as np


def blob_phantom(shape, nblobs, sigma=(4.0, 12.0), amp=(50.0, 200.0), noise=2.0, seed=0):
    """Sum of isotropic Gaussian blobs with uniform centres, sigma and
    amplitude, plus N(0, noise) noise; float32.  Each blob is evaluated as
    the outer product of its per-axis Gaussians."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape)
    img = np.zeros(shape)
    for _ in range(nblobs):
        c = [rng.uniform(0, n) for n in shape]
        s = rng.uniform(*sigma)
        a = rng.uniform(*amp)
        blob = np.array(a)
        for n, ci in zip(shape, c):
            e = np.exp(-(np.arange(n, dtype=np.float64) - ci) ** 2 / (2 * s * s))
            blob = np.multiply.outer(blob, e)
        img += blob
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


SERIES_SIZES = [(96, 96), (128, 112), (160, 144), (192, 160)]   # (x, y)


def gamma_variate(t, t0=10.0, alpha=3.0, beta=1.5):
    """bolus passage curve normalised to peak 1 (zero before t0)"""
    t = np.asarray(t, dtype=np.float64)
    u = np.maximum(t - t0, 0.0)
    peak = (alpha * beta) ** alpha * np.exp(-alpha)
    return u ** alpha * np.exp(-u / beta) / peak


def perfusion_series(nframes, warp, rate=16.0, seed=4000):
    """(moving, reference) pairs of a synthetic 2D perfusion series: frame
    sizes drawn from SERIES_SIZES, one 8-blob anatomy per size, intensity
    scaled by 1 + gain * gamma_variate(frame) with gain U(1.5, 3), each
    moving frame deformed by its own random spline field (rate 16, N(0,1.5)
    clipped to 3 px).  The reference of every frame is frame 0's intensity
    (the anatomy itself).  `warp(image, rate, seed)` applies the random
    deformation."""
    rng = np.random.default_rng(seed)
    anatomy = {}
    pairs = []
    for f in range(nframes):
        sx, sy = SERIES_SIZES[rng.integers(len(SERIES_SIZES))]
        if (sx, sy) not in anatomy:
            anatomy[(sx, sy)] = blob_phantom((sy, sx), 8, sigma=(4.0, 12.0), noise=0.0, seed=seed + 100 + sx + sy)
        base = anatomy[(sx, sy)]
        gain = rng.uniform(1.5, 3.0)
        frame = (base * (1.0 + gain * gamma_variate(f))).astype(np.float32)
        mov = warp(frame, rate, seed + 1000 + f)
        mov = (mov + rng.normal(0.0, 2.0, size=mov.shape)).astype(np.float32)
        ref = (base + rng.normal(0.0, 2.0, size=base.shape)).astype(np.float32)
        pairs.append((mov, ref))
    return pairs


def cohort_pairs(npairs, warp, rate=8.0, seed=5000):
    """(moving, reference) pairs of a synthetic 3D cohort: each dimension
    drawn from {96, 112, ..., 224} (z at most 160), 40-blob phantoms
    (sigma U(4,16)), the moving volume deformed by its own random spline
    field (knot spacing 8, N(0,2) clipped to 4 voxels) and multiplied by a
    bias field (degree-2 exp polynomial, N(0,0.1)).  `warp(image, rate,
    seed)` applies the random deformation."""
    rng = np.random.default_rng(seed)
    pairs = []
    for p in range(npairs):
        sx = int(rng.choice(np.arange(96, 225, 16)))
        sy = int(rng.choice(np.arange(96, 225, 16)))
        sz = int(rng.choice(np.arange(96, 161, 16)))
        ref = blob_phantom((sz, sy, sx), 40, sigma=(4.0, 16.0), seed=seed + 100 + p)
        mov = warp(ref, rate, seed + 1000 + p)
        mov = (mov * bias_field(mov.shape, 0.1, seed=seed + 2000 + p)).astype(np.float32)
        pairs.append((mov, ref))
    return pairs
