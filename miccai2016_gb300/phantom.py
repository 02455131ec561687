"""
Synthetic workloads: an analytic helix phantom with additive Gaussian noise,
and the host-side helpers of the reference's experiment that turn an image into
max-flow inputs (capacities, nonterminal weights) and score a segmentation.

The phantom stands in for the reference's VTK-voxelised toric helix
(src/helpers/helix_phantom.py), which needs VTK.  Definition:
  * centreline c(t) = (zc + pitch * t / 2pi, yc + R sin t, xc + R cos t), the
    helix axis along array axis 0 and centred in (y, x); t runs over the range
    that keeps the centreline `tube_radius + 1` voxels inside the z extent;
  * ground truth = 1 where the voxel centre's distance to the (finite)
    centreline is <= tube_radius, else 0;
  * noisy = truth + RandomState(seed).normal(scale=sigma, size=shape), in
    float64, then cast to float32 (phantom_experiment.py:200, 221-222).
"""
from __future__ import annotations

import numpy as np


def _helix_geometry(shape, tube_radius, helix_radius, pitch):
    d0, d1, d2 = shape
    zc, yc, xc = (d0 - 1) / 2.0, (d1 - 1) / 2.0, (d2 - 1) / 2.0
    a = pitch / (2 * np.pi)
    zlo = tube_radius + 1.0
    zhi = (d0 - 1) - (tube_radius + 1.0)
    return zc, yc, xc, a, (zlo - zc) / a, (zhi - zc) / a


def helix_nearest(shape, tube_radius, helix_radius, pitch, chunk=1 << 22):
    """Distance of every voxel centre to the helix centreline and the
    centreline parameter t of the nearest point (float64 arrays)."""
    d0, d1, d2 = shape
    zc, yc, xc, a, tmin, tmax = _helix_geometry(shape, tube_radius, helix_radius, pitch)
    R = float(helix_radius)
    n = d0 * d1 * d2
    dist = np.empty(n, np.float64)
    tbest = np.empty(n, np.float64)
    for s in range(0, n, chunk):
        idx = np.arange(s, min(n, s + chunk))
        z = idx // (d1 * d2)
        y = (idx // d2) % d1
        x = idx % d2
        dz, dy, dx = z - zc, y - yc, x - xc
        phi = np.arctan2(dy, dx)
        # the two windings nearest in z; Newton on d/dt |p - c(t)|^2 from each
        w = (dz / a - phi) / (2 * np.pi)
        k0 = np.round(w)
        k1 = k0 + np.where(w >= k0, 1.0, -1.0)
        best = np.full(idx.shape, np.inf)
        bt = np.zeros(idx.shape)
        for k in (k0, k1):
            t = phi + 2 * np.pi * k
            for _ in range(4):
                c, s_ = np.cos(t), np.sin(t)
                g = -a * dz + a * a * t - R * dy * c + R * dx * s_
                gp = a * a + R * dy * s_ + R * dx * c
                gp = np.where(gp > 1e-6, gp, a * a + R * R)
                t = t - np.clip(g / gp, -0.5, 0.5)
            t = np.clip(t, tmin, tmax)
            d2_ = (dz - a * t) ** 2 + (dy - R * np.sin(t)) ** 2 + (dx - R * np.cos(t)) ** 2
            better = d2_ < best
            best = np.where(better, d2_, best)
            bt = np.where(better, t, bt)
        dist[idx] = np.sqrt(best)
        tbest[idx] = bt
    return dist.reshape(shape), tbest.reshape(shape)


def helix_phantom(shape, tube_radius, helix_radius, pitch, sigma, seed=0, nearest=None):
    """(noisy float32, truth float32 in {0, 1}) for the analytic helix."""
    dist, _ = nearest if nearest is not None else helix_nearest(shape, tube_radius, helix_radius, pitch)
    truth = (dist <= tube_radius).astype(np.float64)
    noise = np.random.RandomState(seed).normal(size=shape, scale=sigma)
    noisy = (truth + noise).astype(np.float32)
    return noisy, truth.astype(np.float32)


def helix_tangents(shape, tube_radius, helix_radius, pitch, nearest=None):
    """Unit tangent (axis order z, y, x) of the nearest centreline point for
    every voxel, float32 (z, y, x, 3): an analytic stand-in for the direction
    field the vesselness/GVF stages produce."""
    _, t = nearest if nearest is not None else helix_nearest(shape, tube_radius, helix_radius, pitch)
    zc, yc, xc, a, _, _ = _helix_geometry(shape, tube_radius, helix_radius, pitch)
    R = float(helix_radius)
    v = np.stack([np.full(t.shape, a), R * np.cos(t), -R * np.sin(t)], axis=-1)
    v /= np.linalg.norm(v, axis=-1, keepdims=True)
    return v.astype(np.float32)


def squeeze_frames(v):
    """Squeezed quaternions (z-x-z Euler angles, the convention of the
    reference's qsqueeze) of the frames completed from unit vectors v as
    completeTransformations does (src/clcode/adjust_directions.cl:68-100);
    float64 numpy, used to build synthetic max-flow inputs."""
    v = np.asarray(v, dtype=np.float64)
    e0 = v / np.maximum(np.linalg.norm(v, axis=-1, keepdims=True), 1e-300)
    use0 = np.abs(e0[..., 0]) > np.abs(e0[..., 1])
    z = np.zeros(e0.shape[:-1])
    e1 = np.where(use0[..., None], np.stack([-e0[..., 2], z, e0[..., 0]], -1),
                  np.stack([z, e0[..., 2], -e0[..., 1]], -1))
    e1 /= np.maximum(np.linalg.norm(e1, axis=-1, keepdims=True), 1e-300)
    e2 = np.cross(e0, e1)
    m = np.stack([e0, e1, e2], axis=-1)            # columns e0, e1, e2
    tr = m[..., 0, 0] + m[..., 1, 1] + m[..., 2, 2]
    w = np.sqrt(np.maximum(0.0, 1 + tr)) / 2
    x = np.sqrt(np.maximum(0.0, 1 + m[..., 0, 0] - m[..., 1, 1] - m[..., 2, 2])) / 2
    y = np.sqrt(np.maximum(0.0, 1 - m[..., 0, 0] + m[..., 1, 1] - m[..., 2, 2])) / 2
    zq = np.sqrt(np.maximum(0.0, 1 - m[..., 0, 0] - m[..., 1, 1] + m[..., 2, 2])) / 2
    x = np.copysign(x, m[..., 2, 1] - m[..., 1, 2])
    y = np.copysign(y, m[..., 0, 2] - m[..., 2, 0])
    zq = np.copysign(zq, m[..., 1, 0] - m[..., 0, 1])
    # z-x-z Euler angles of the quaternion (w, x, y, zq)
    phi = np.arctan2(x * zq + y * w, x * w - y * zq)
    theta = np.arccos(np.clip(1 - 2 * (x * x + y * y), -1, 1))
    psi = np.arctan2(x * zq - y * w, x * w + y * zq)
    return np.stack([phi, theta, psi], axis=-1).astype(np.float32)


# ---- the reference experiment's host helpers ---------------------------------

def normpdf(x, mean, var):
    """phantom_experiment.py:29-35"""
    return np.exp((x - mean) ** 2 * (1 / (-2 * var))) * (1 / np.sqrt(2 * np.pi * var))


def bgfg_weights(image, noise_level, eps=1e-9):
    """(background, foreground) capacities from the Gaussian log-likelihood
    ratio, phantom_experiment.py:280-301 (float64)."""
    var = noise_level ** 2
    image = np.asarray(image, dtype=np.float64)
    bgp = normpdf(image, 0, var)
    fgp = normpdf(image, 1, var)
    p_hat = np.maximum(normpdf(0, 0, var), normpdf(1, 1, var))
    r = np.log((fgp + eps) / (bgp + eps))
    rq = 1 / np.log((p_hat + eps) / eps)
    return rq * np.maximum(-r, 0), rq * np.maximum(r, 0)


def grad_mag_sq(image):
    """|grad I|^2 with np.gradient's central differences (phantom_experiment.py:345)."""
    return np.linalg.norm(np.gradient(np.asarray(image, dtype=np.float64)), axis=0) ** 2


def nonterminal_weights(grad2, weighting, decay):
    """C = w * exp(-|grad I|^2 / decay^2) (phantom_experiment.py:359)."""
    return weighting * np.exp(((-1.) / (decay ** 2)) * grad2)


def fast_dice(segmentation, ground_truth):
    """phantom_experiment.py:38-49"""
    seg = np.asarray(segmentation) >= 0.5
    inter = np.multiply(seg, ground_truth)
    return 2 * np.sum(inter) / (np.sum(seg) + np.sum(ground_truth))


def dice_largest(segmentation, ground_truth):
    """Dice of the largest connected component (phantom_experiment.py:52-103)."""
    import scipy.ndimage
    seg = np.asarray(segmentation) >= 0.5
    lab, nlab = scipy.ndimage.label(seg)
    if nlab == 0:
        return 0.0
    sizes = np.bincount(lab.ravel())[1:]
    best = int(np.argmax(sizes)) + 1
    comp = lab == best
    return 2 * np.sum(np.multiply(comp, ground_truth)) / (sizes[best - 1] + np.sum(ground_truth))


def maxflow_inputs(cfg, eigs=None):
    """Max-flow inputs of a helix configuration: (noisy image, truth,
    squeezed quaternions of the helix frames, nonterminal weights, foreground
    and background capacities), all float32 except truth."""
    nearest = helix_nearest(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"])
    noisy, truth = helix_phantom(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"],
                                 cfg["sigma"], cfg["seed"], nearest=nearest)
    quats = squeeze_frames(helix_tangents(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"],
                                          nearest=nearest))
    bgw, fgw = bgfg_weights(noisy, cfg["sigma"])
    ntw = nonterminal_weights(grad_mag_sq(noisy), cfg["weighting"], cfg["decay"])
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    return f(noisy), truth, f(quats), f(ntw), f(fgw), f(bgw)


# ---- the configurations of the benchmarks -----------------------------------

CONFIG_PLAIN_64 = dict(shape=(64, 64, 64), tube_radius=3.0, helix_radius=16.0, pitch=20.0, sigma=1.5, seed=0,
                       weighting=10 ** -1.25, decay=10 ** 1.5, num_iter=300, gvf_iter=100, gvf_mu=0.2)
CONFIG_PLAIN_256 = dict(shape=(256, 256, 256), tube_radius=12.0, helix_radius=64.0, pitch=80.0, sigma=1.0,
                        seed=0, weighting=10 ** -1.25, decay=10 ** 1.5, num_iter=1000, gvf_iter=100, gvf_mu=0.2)
CONFIG_PLAIN_128 = dict(shape=(128, 128, 128), tube_radius=6.0, helix_radius=32.0, pitch=40.0, sigma=1.0,
                        seed=0, weighting=10 ** -1.25, decay=10 ** 1.5, num_iter=300, gvf_iter=100, gvf_mu=0.2)
# the batched grid search: 25 weightings x 17 decays (phantom_experiment.py:167-168)
CONFIG_GRID_128 = dict(shape=(128, 128, 128), tube_radius=6.0, helix_radius=32.0, pitch=40.0, sigma=1.5, seed=0,
                       scales=(2, 6, 3), gvf_mu=0.2, gvf_iter=100, num_iter=3000, update=30, error_bound=1e-4,
                       weightings=tuple(float(w) for w in __import__("numpy").logspace(-2.5, 0.5, 25)),
                       decays=tuple(float(d) for d in __import__("numpy").logspace(-1, 3, 17)))
ATV_EIGS = (1.0, 10 ** -1.5, 10 ** -1.5)   # phantom_experiment.py:154, 362
TV_EIGS = (1.0, 1.0, 1.0)
