"""Seeded synthetic particle microstructures (initial conditions).

The reference ships no input files; its README (README.md:26-34) only
shows how to write /etaS, /etaL and /c with MATLAB.  This generator builds
the synthetic states the benchmark and tests use:

  * non-overlapping spherical solid particles placed at random (periodic
    minimum-image distances, centre distance >= R1 + R2 + gap);
  * etaS = 0.5 * (1 - tanh(2 (r - R) / w)), i.e. a tanh profile of width w
    cells (etaS goes from 0.88 to 0.12 across r = R -/+ w/2), max over
    particles; etaL = 1 - etaS;
  * c = h cS_eq + (1 - h) cL_eq + U(-noise, noise), with
    h = etaS^2 / (etaS^2 + etaL^2) the interpolation of phasefield.c:328-330
    and cS_eq, cL_eq the common-tangent compositions of the reference's
    parabolas (phasefield.c:76-81, 354-355): 0.47603 / 0.99903.
"""
from __future__ import annotations

import argparse
import math

import numpy as np

DEFAULT = dict(AS=1e9, AL=1e9, CS=-1e6, CL=1e7, cS0=0.455, cL0=0.978)


def equilibrium_compositions(AS=1e9, AL=1e9, CS=-1e6, CL=1e7, cS0=0.455, cL0=0.978):
    """Common tangent of fS = AS/2 (c-cS0)^2 + CS and fL = AL/2 (c-cL0)^2 + CL.

    Equal slopes mu = AS (cs - cS0) = AL (cl - cL0) and equal intercepts
    f - mu c give  -mu^2/2 (1/AS - 1/AL) - mu (cS0 - cL0) + (CS - CL) = 0.
    """
    a = -0.5 * (1.0 / AS - 1.0 / AL)
    b = -(cS0 - cL0)
    c = CS - CL
    if abs(a) < 1e-300:
        mu = -c / b
    else:
        disc = math.sqrt(b * b - 4 * a * c)
        r1, r2 = (-b + disc) / (2 * a), (-b - disc) / (2 * a)
        mu = r1 if abs(r1) < abs(r2) else r2
    return cS0 + mu / AS, cL0 + mu / AL


def _wrap(d, n):
    return d - n * np.round(d / n)


def _draw_radius(rng, radius):
    if radius[0] == "uniform":
        return rng.uniform(radius[1], radius[2])
    return radius[1] * math.exp(radius[2] * rng.standard_normal())


def place_particles(shape, rng, radius, count=None, vf=None, gap=1.0, tries_per_particle=4096, batch=64):
    """Random placement of non-overlapping spheres in a periodic box.

    radius: ("uniform", lo, hi) or ("lognormal", median, sigma).
    The radii are drawn first (`count` of them, or until their volume
    reaches `vf` of the box), sorted largest first, and each sphere takes
    the first of a stream of uniformly random centres whose periodic
    (minimum-image) distance to every placed sphere is >= R1 + R2 + gap;
    a sphere that finds no place within `tries_per_particle` draws is
    dropped.  Neighbour tests use a periodic k-d tree of the placed
    centres (rebuilt every 256 placements) plus a direct test against the
    centres placed since.  Returns centres (k, 3) in (z, y, x), radii (k,)."""
    from scipy.spatial import cKDTree

    dims = np.array(shape, dtype=np.float64)
    cells = float(np.prod(shape))
    cap = 0.45 * float(min(shape))
    radii = []
    vol = 0.0
    while (count is not None and len(radii) < count) or (count is None and vf is not None and vol / cells < vf):
        R = min(_draw_radius(rng, radius), cap)
        radii.append(R)
        vol += 4.0 / 3.0 * math.pi * R ** 3
    radii = np.sort(np.array(radii))[::-1]
    n = len(radii)
    cen = np.empty((n, 3))
    rad = np.empty(n)
    k = 0
    tree, tree_n = None, 0
    rmax = radii[0] if n else 0.0
    for R in radii:
        if k - tree_n >= 256:
            tree, tree_n = cKDTree(np.mod(cen[:k], dims), boxsize=dims), k
        for _ in range(max(1, tries_per_particle // batch)):
            P = rng.random((batch, 3)) * dims
            ok = np.ones(batch, bool)
            if k > tree_n:                      # centres not yet in the tree
                d = _wrap(P[:, None, :] - cen[None, tree_n:k, :], dims)
                dist2 = (d * d).sum(-1)
                ok &= ~np.any(dist2 < (rad[None, tree_n:k] + R + gap) ** 2, axis=1)
            if tree is not None:
                for ci in np.flatnonzero(ok):
                    nb = tree.query_ball_point(P[ci], R + rmax + gap)
                    if nb:
                        nb = np.asarray(nb)
                        d = _wrap(cen[nb] - P[ci], dims)
                        if np.any((d * d).sum(-1) < (rad[nb] + R + gap) ** 2):
                            ok[ci] = False
                            continue
                    break
            hit = np.flatnonzero(ok)
            if len(hit):
                cen[k] = P[hit[0]]
                rad[k] = R
                k += 1
                break
    return cen[:k], rad[:k]


def render(shape, centres, radii, width=4.0, noise=1e-3, rng=None, params=None):
    """etaS, etaL, c (float64, [z][y][x]) for the given spheres.

    etaS = 0.5 (1 - tanh(2 D / w)) with D the smallest (r - R) over the
    spheres, evaluated within R + 3w of each centre (etaS < 1e-5 beyond)."""
    D = np.full(shape, np.inf)
    for p, R in zip(centres, radii):
        ext = int(math.ceil(R + 3.0 * width)) + 1
        idx, off = [], []
        for ax, n in enumerate(shape):
            lo = int(math.floor(p[ax])) - ext
            # the whole axis when the box would wrap onto itself
            ii = np.arange(n) if 2 * ext + 2 >= n else np.arange(lo, lo + 2 * ext + 2)
            idx.append(np.mod(ii, n))
            off.append(_wrap((ii + 0.5) - p[ax], n))
        r = np.sqrt(off[0][:, None, None] ** 2 + off[1][None, :, None] ** 2 + off[2][None, None, :] ** 2)
        box = np.ix_(*idx)    # wrapped indices are unique per axis
        D[box] = np.minimum(D[box], r - R)
    etaS = 0.5 * (1.0 - np.tanh((2.0 / width) * D))
    etaL = 1.0 - etaS
    cs, cl = equilibrium_compositions(**(params or DEFAULT))
    h = etaS * etaS / (etaS * etaS + etaL * etaL)
    c = h * cs + (1.0 - h) * cl
    if noise:
        rng = rng if rng is not None else np.random.default_rng(0)
        c = c + rng.uniform(-noise, noise, size=shape)
    return etaS, etaL, c


# Workloads named by what they are (grid, particles, radii).
WORKLOADS = {
    # 64^3, 20 spheres, R ~ U[4, 8]
    "spheres64_uniform4to8": dict(shape=(64, 64, 64), radius=("uniform", 4.0, 8.0), count=20, vf=None),
    # 256^3, lognormal R (median 5, sigma 0.3), solid fraction 0.3
    "spheres256_lognormal5_vf30": dict(shape=(256, 256, 256), radius=("lognormal", 5.0, 0.3), count=None, vf=0.3),
    # 512^3, lognormal R (median 4, sigma 0.3), solid fraction 0.2
    "spheres512_lognormal4_vf20": dict(shape=(512, 512, 512), radius=("lognormal", 4.0, 0.3), count=None, vf=0.2),
}


def generate(shape, radius=("uniform", 4.0, 8.0), count=None, vf=None, seed=0, width=4.0, noise=1e-3,
             gap=1.0):
    """Particle microstructure; returns (etaS, etaL, c, info)."""
    if vf is not None and vf > 0.34:
        raise ValueError("random placement does not reach solid fractions above ~0.34")
    rng = np.random.default_rng(seed)
    if count is not None:
        R_max = radius[2] if radius[0] == "uniform" else radius[1] * math.exp(3 * radius[2])
        if math.pi * 4 / 3 * R_max ** 3 * count > 0.5 * np.prod(shape):
            raise ValueError("too many particles for the box")
    cen, rad = place_particles(shape, rng, radius, count=count, vf=vf, gap=gap)
    etaS, etaL, c = render(shape, cen, rad, width=width, noise=noise, rng=rng)
    info = {"particles": int(len(rad)), "mean_radius": float(rad.mean()) if len(rad) else 0.0,
            "sphere_fraction": float((4 / 3 * math.pi * rad ** 3).sum() / np.prod(shape)), "seed": seed}
    return etaS, etaL, c, info


def workload(name: str, seed: int = 0, shape=None):
    w = dict(WORKLOADS[name])
    if shape is not None:
        w["shape"] = tuple(shape)
    return generate(w["shape"], radius=w["radius"], count=w["count"], vf=w["vf"], seed=seed)


def ensemble_workload(n=64, edges=(48, 64, 96, 128), vf=(0.1, 0.4), radius=("lognormal", 5.0, 0.3), seed=0):
    """Ensemble of `n` cubic periodic domains: edge drawn from `edges`,
    target solid fraction from U[vf], lognormal radii, each domain with its
    own seed.  Targets above what random non-overlapping placement reaches
    (about 0.34 with a one-cell gap) are placed with touching allowed
    (gap 0); spheres that find no place are dropped, so the achieved
    fraction ("sphere_fraction" in each info) can fall below the target.
    Returns a list of (etaS, etaL, c, info)."""
    rng = np.random.default_rng(seed)
    out = []
    for d in range(n):
        e = int(rng.choice(edges))
        f = float(rng.uniform(*vf))
        shape = (e, e, e)
        r = np.random.default_rng([seed, d])
        cen, rad = place_particles(shape, r, radius, vf=f, gap=1.0 if f <= 0.3 else 0.0)
        etaS, etaL, c = render(shape, cen, rad, rng=r)
        info = {"edge": e, "target_fraction": f, "particles": int(len(rad)),
                "sphere_fraction": float((4 / 3 * math.pi * rad ** 3).sum() / np.prod(shape)), "seed": [seed, d]}
        out.append((etaS, etaL, c, info))
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description="write a seeded particle microstructure as an HDF5 input for ppf")
    ap.add_argument("out")
    ap.add_argument("--workload", default="spheres64_uniform4to8", choices=sorted(WORKLOADS))
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    from . import write_fields
    eS, eL, c, info = workload(a.workload, a.seed)
    write_fields(a.out, eS, eL, c)
    print(info)
