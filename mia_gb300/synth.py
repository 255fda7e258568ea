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
    import os
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(seed)
    sizes = []
    for p in range(npairs):
        sx = int(rng.choice(np.arange(96, 225, 16)))
        sy = int(rng.choice(np.arange(96, 225, 16)))
        sz = int(rng.choice(np.arange(96, 161, 16)))
        sizes.append((sz, sy, sx))

    def make(p):   # every pair from its own seeds: the threads' order does not matter
        ref = blob_phantom(sizes[p], 40, sigma=(4.0, 16.0), seed=seed + 100 + p)
        mov = warp(ref, rate, seed + 1000 + p)
        mov = (mov * bias_field(mov.shape, 0.1, seed=seed + 2000 + p)).astype(np.float32)
        return mov, ref
    with ThreadPoolExecutor(max(1, min(8, os.cpu_count() or 1))) as ex:
        return list(ex.map(make, range(npairs)))


def _csize(n, rate):
    """coefficient count per axis of a spline transformation of `n` voxels
    at `rate`: floor((n - 1 + rate) / rate) in float, plus the border"""
    return int(np.float32(np.float32(n - 1) + np.float32(rate)) / np.float32(rate)) + 2


def _axis_weights(n, nc):
    """dense (n x nc) matrix of the cubic B-spline weights of the
    coefficients at the voxel coordinates i (nc - 3) / (n - 1) + 1"""
    x = np.arange(n, dtype=np.float64) * ((nc - 3) / (n - 1.0)) + 1.0
    t = np.abs(x[:, None] - np.arange(nc, dtype=np.float64)[None, :])
    w = np.where(t < 1.0, (4.0 + t * t * (3.0 * t - 6.0)) / 6.0, np.where(t < 2.0, (2.0 - t) ** 3 / 6.0, 0.0))
    return w


def spline_field_params(shape, rate, sigma, clip, seed):
    """random coefficients (N(0, sigma) clipped to +-clip) of a spline
    transformation at `rate` for an image of `shape` ([z,] y, x); returns
    the coefficient grid [.., dim] (x component first)"""
    dim = len(shape)
    cs = [_csize(n, rate) for n in shape]
    return spline_params(int(np.prod(cs)), dim, sigma, clip, seed=seed).reshape(tuple(cs) + (dim,))


def spline_warp_host(img, coeffs):
    """img sampled at x - u(x), u the cubic B-spline field of `coeffs`
    ([.., dim] on the coefficient grid of img's shape), with cubic B-spline
    interpolation and mirror boundary (scipy), in float32.  Used to make the
    benchmarks' moving images on the host, identically for every arm."""
    from scipy import ndimage
    shape = img.shape
    dim = len(shape)
    W = [_axis_weights(n, c) for n, c in zip(shape, coeffs.shape[:dim])]
    coords = []
    for k in range(dim):
        u = coeffs[..., dim - 1 - k]          # component of array axis k (x is the last axis)
        for ax in range(dim):
            u = np.tensordot(W[ax], u, axes=([1], [ax]))
            u = np.moveaxis(u, 0, ax)
        grid = np.arange(shape[k], dtype=np.float64).reshape([-1 if a == k else 1 for a in range(dim)])
        coords.append((grid - u).astype(np.float32))
    out = ndimage.map_coordinates(img.astype(np.float64), np.array(coords), order=3, mode="mirror")
    return out.astype(np.float32)


def host_warp_factory(dim):
    """warp(image, rate, seed): the random deformation of the benchmark
    workloads (2D: N(0, 1.5) clipped to 3 px; 3D: N(0, 2) clipped to 4
    voxels), applied on the host"""
    sig, clip = (1.5, 3.0) if dim == 2 else (2.0, 4.0)

    def warp(img, rate, seed):
        return spline_warp_host(img, spline_field_params(img.shape, rate, sig, clip, seed))
    return warp
