"""Seeded synthetic oriented point clouds.

These stand in for the reference's scanned inputs (its Bunny/Eagle/Torso files
are not distributed).  Each generator returns ``(xyz, nrm)`` as float32 arrays of
shape (n, 3); normals are unit length before any perturbation.
"""
from __future__ import annotations

import numpy as np


def _unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def sphere(n: int = 50_000, radius: float = 0.35, center=(0.5, 0.5, 0.5), seed: int = 0):
    """Uniform samples on a sphere (normalised Gaussian directions), exact normals."""
    rng = np.random.default_rng(seed)
    d = _unit(rng.standard_normal((n, 3)))
    xyz = np.asarray(center) + radius * d
    return xyz.astype(np.float32), d.astype(np.float32)


def _vmf_perturb(nrm, kappa, rng):
    """Draw unit vectors from a von Mises-Fisher distribution around each row of nrm (Wood 1994, S^2)."""
    n = len(nrm)
    xi = rng.random(n)
    w = 1.0 + np.log(xi + (1.0 - xi) * np.exp(-2.0 * kappa)) / kappa
    # random tangent direction
    t = rng.standard_normal((n, 3))
    t -= (t * nrm).sum(1, keepdims=True) * nrm
    t = _unit(t)
    return _unit(w[:, None] * nrm + np.sqrt(np.clip(1 - w * w, 0, None))[:, None] * t)


def torus(n: int = 1_000_000, R: float = 0.3, r: float = 0.1, center=(0.5, 0.5, 0.5),
          density_gradient: float = 7.0, sigma: float = 0.001, kappa: float = 500.0, seed: int = 0):
    """Torus around the z axis; sample density proportional to 1 + 7u (u = normalised x across the torus),
    Gaussian position noise sigma, von Mises-Fisher normal noise kappa."""
    rng = np.random.default_rng(seed)
    cx = np.asarray(center, dtype=np.float64)
    out_p, out_n = [], []
    have = 0
    wmax = (R + r) * (1.0 + density_gradient)
    while have < n:
        m = int((n - have) * 2.5) + 1024
        th = rng.random(m) * 2 * np.pi
        ph = rng.random(m) * 2 * np.pi
        ring = R + r * np.cos(ph)
        x = ring * np.cos(th)
        u = (x + R + r) / (2 * (R + r))
        wgt = ring * (1.0 + density_gradient * u)
        keep = rng.random(m) * wmax < wgt
        th, ph, ring = th[keep], ph[keep], ring[keep]
        p = np.stack([ring * np.cos(th), ring * np.sin(th), r * np.sin(ph)], 1)
        nv = np.stack([np.cos(ph) * np.cos(th), np.cos(ph) * np.sin(th), np.sin(ph)], 1)
        out_p.append(p)
        out_n.append(nv)
        have += len(p)
    p = np.concatenate(out_p)[:n]
    nv = np.concatenate(out_n)[:n]
    p = p + cx + sigma * rng.standard_normal(p.shape)
    nv = _vmf_perturb(nv, kappa, rng)
    return p.astype(np.float32), nv.astype(np.float32)


def _random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a*a+b*b-c*c-d*d, 2*(b*c-a*d), 2*(b*d+a*c)],
                     [2*(b*c+a*d), a*a-b*b+c*c-d*d, 2*(c*d-a*b)],
                     [2*(b*d-a*c), 2*(c*d+a*b), a*a-b*b-c*c+d*d]])


def ellipsoid_union(seed: int, n_min: int = 20_000, n_max: int = 200_000):
    """Union of 3-8 rotated ellipsoids (centres in [0.2,0.8]^3, semi-axes 0.05-0.25); points are
    area-uniform samples of the union's outer surface, with exact normals."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(3, 9))
    n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
    cs = rng.uniform(0.2, 0.8, (k, 3))
    ax = rng.uniform(0.05, 0.25, (k, 3))
    rots = [_random_rotation(rng) for _ in range(k)]

    def inside_any(p, skip):
        res = np.zeros(len(p), bool)
        for j in range(k):
            if j == skip:
                continue
            q = (p - cs[j]) @ rots[j]
            res |= ((q / ax[j]) ** 2).sum(1) < 1.0
        return res

    # approximate surface areas (Knud Thomsen) to split the sample budget
    pth = 1.6075
    areas = np.array([4 * np.pi * (((a[0]*a[1])**pth + (a[0]*a[2])**pth + (a[1]*a[2])**pth) / 3) ** (1 / pth)
                      for a in ax])
    ps, ns = [], []
    have = 0
    while have < n:
        j = int(rng.choice(k, p=areas / areas.sum()))
        m = 4096
        d = _unit(rng.standard_normal((m, 3)))
        q = d * ax[j]
        # area element of the map sphere -> ellipsoid, for rejection to area-uniform
        g = np.sqrt((d[:, 0] * ax[j, 1] * ax[j, 2]) ** 2 + (d[:, 1] * ax[j, 0] * ax[j, 2]) ** 2
                    + (d[:, 2] * ax[j, 0] * ax[j, 1]) ** 2)
        keep = rng.random(m) * g.max() < g
        q = q[keep]
        nrm = _unit(q / ax[j] ** 2)
        p = q @ rots[j].T + cs[j]
        nrm = nrm @ rots[j].T
        out = ~inside_any(p, j)
        ps.append(p[out])
        ns.append(nrm[out])
        have += int(out.sum())
    return (np.concatenate(ps)[:n].astype(np.float32), np.concatenate(ns)[:n].astype(np.float32))


def superquadric(seed: int, n_min: int = 5_000, n_max: int = 500_000, sigma: float = 5e-4):
    """Random superquadric (exponents e1,e2 in [0.3,3], scales 0.1-0.4, random rotation, centred)."""
    rng = np.random.default_rng(seed)
    n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
    e1, e2 = rng.uniform(0.3, 3.0, 2)
    s = rng.uniform(0.1, 0.4, 3)
    rot = _random_rotation(rng)

    def spow(v, e):
        return np.sign(v) * np.abs(v) ** e

    m = n * 3
    eta = np.arcsin(rng.uniform(-1, 1, m))
    om = rng.uniform(-np.pi, np.pi, m)
    ce, se, co, so = np.cos(eta), np.sin(eta), np.cos(om), np.sin(om)
    p = np.stack([s[0] * spow(ce, e1) * spow(co, e2), s[1] * spow(ce, e1) * spow(so, e2), s[2] * spow(se, e1)], 1)
    nv = np.stack([spow(ce, 2 - e1) * spow(co, 2 - e2) / s[0], spow(ce, 2 - e1) * spow(so, 2 - e2) / s[1],
                   spow(se, 2 - e1) / s[2]], 1)
    ok = np.isfinite(nv).all(1) & (np.linalg.norm(nv, axis=1) > 0)
    p, nv = p[ok][:n], _unit(nv[ok][:n])
    p = p @ rot.T + 0.5 + sigma * rng.standard_normal(p.shape)
    nv = nv @ rot.T
    return p.astype(np.float32), nv.astype(np.float32)


def _value_noise(p, seed, base_freq=4.0, octaves=4, persistence=0.5):
    """Seeded trilinear lattice value noise, summed over octaves, amplitude-normalised to [-1, 1]."""
    rng = np.random.default_rng(seed)
    table = rng.uniform(-1, 1, 4096)
    perm = rng.permutation(4096)
    total = np.zeros(len(p))
    grad = np.zeros((len(p), 3))
    amp, freq, norm = 1.0, base_freq, 0.0
    for _ in range(octaves):
        q = p * freq
        i0 = np.floor(q).astype(np.int64)
        f = q - i0
        s = f * f * (3 - 2 * f)
        ds = 6 * f * (1 - f)

        def lat(ix, iy, iz):
            h = perm[(ix * 73856093 ^ iy * 19349663 ^ iz * 83492791) & 4095]
            return table[h]
        v = np.zeros(len(p))
        g = np.zeros((len(p), 3))
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    c = lat(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
                    wx = s[:, 0] if dx else 1 - s[:, 0]
                    wy = s[:, 1] if dy else 1 - s[:, 1]
                    wz = s[:, 2] if dz else 1 - s[:, 2]
                    v += c * wx * wy * wz
                    g[:, 0] += c * (ds[:, 0] if dx else -ds[:, 0]) * wy * wz
                    g[:, 1] += c * wx * (ds[:, 1] if dy else -ds[:, 1]) * wz
                    g[:, 2] += c * wx * wy * (ds[:, 2] if dz else -ds[:, 2])
        total += amp * v
        grad += amp * freq * g
        norm += amp
        amp *= persistence
        freq *= 2
    return total / norm, grad / norm


def displaced_sphere(n: int = 30_000_000, radius: float = 0.35, amplitude: float = 0.05, seed: int = 0,
                     chunk: int = 2_000_000, device=None):
    """Sphere radially displaced by 4-octave value noise; normals from the analytic gradient.
    With a torch CUDA device the directions are drawn and displaced there (float64, the same
    noise tables and formulas; a different seeded sample of the same distribution), which takes
    well under a second for 30M points instead of about a minute on the host."""
    if device is not None:
        return _displaced_sphere_torch(n, radius, amplitude, seed, device)
    rng = np.random.default_rng(seed)
    ps, ns = [], []
    for start in range(0, n, chunk):
        m = min(chunk, n - start)
        d = _unit(rng.standard_normal((m, 3)))
        h, g = _value_noise(d, seed)
        rad = radius + amplitude * h
        p = 0.5 + rad[:, None] * d
        # surface F(x) = |x-c| - radius - A*h(dir) ; gradient ~ dir - A * (tangential part of grad h)/|x-c|
        gt = g - (g * d).sum(1, keepdims=True) * d
        nv = _unit(d - amplitude * gt / rad[:, None])
        ps.append(p.astype(np.float32))
        ns.append(nv.astype(np.float32))
    return np.concatenate(ps), np.concatenate(ns)


def _displaced_sphere_torch(n, radius, amplitude, seed, device, chunk=8_000_000):
    import torch
    rng = np.random.default_rng(seed)
    table = torch.tensor(rng.uniform(-1, 1, 4096), dtype=torch.float64, device=device)
    perm = torch.tensor(rng.permutation(4096), dtype=torch.int64, device=device)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    ps, ns = [], []
    for start in range(0, n, chunk):
        m = min(chunk, n - start)
        d = torch.randn((m, 3), generator=gen, dtype=torch.float64, device=device)
        d = d / torch.linalg.norm(d, dim=1, keepdim=True)
        total = torch.zeros(m, dtype=torch.float64, device=device)
        grad = torch.zeros((m, 3), dtype=torch.float64, device=device)
        amp, freq, norm = 1.0, 4.0, 0.0
        for _ in range(4):
            q = d * freq
            i0 = torch.floor(q).to(torch.int64)
            f = q - i0
            sm = f * f * (3 - 2 * f)
            ds = 6 * f * (1 - f)
            v = torch.zeros(m, dtype=torch.float64, device=device)
            g = torch.zeros((m, 3), dtype=torch.float64, device=device)
            for dx in (0, 1):
                for dy in (0, 1):
                    for dz in (0, 1):
                        h = perm[((i0[:, 0] + dx) * 73856093 ^ (i0[:, 1] + dy) * 19349663 ^
                                  (i0[:, 2] + dz) * 83492791) & 4095]
                        c = table[h]
                        wx = sm[:, 0] if dx else 1 - sm[:, 0]
                        wy = sm[:, 1] if dy else 1 - sm[:, 1]
                        wz = sm[:, 2] if dz else 1 - sm[:, 2]
                        v += c * wx * wy * wz
                        g[:, 0] += c * (ds[:, 0] if dx else -ds[:, 0]) * wy * wz
                        g[:, 1] += c * wx * (ds[:, 1] if dy else -ds[:, 1]) * wz
                        g[:, 2] += c * wx * wy * (ds[:, 2] if dz else -ds[:, 2])
            total += amp * v
            grad += amp * freq * g
            norm += amp
            amp *= 0.5
            freq *= 2
        h, g = total / norm, grad / norm
        rad = radius + amplitude * h
        p = 0.5 + rad[:, None] * d
        gt = g - (g * d).sum(1, keepdim=True) * d
        nv = d - amplitude * gt / rad[:, None]
        nv = nv / torch.linalg.norm(nv, dim=1, keepdim=True)
        ps.append(p.float().cpu().numpy())
        ns.append(nv.float().cpu().numpy())
    return np.concatenate(ps), np.concatenate(ns)
