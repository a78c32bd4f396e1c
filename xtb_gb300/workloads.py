"""Seeded synthetic geometries for the GFN2 single-point workloads.

There is no public benchmark suite for this path, so these generators are the
benchmark inputs.  Geometries are built in Angstrom and converted once to Bohr
with autoaa = 0.52917726 (the reference's constant, src/mctc/convert.f90:25).

* ``alkane(n, sigma, seed)``: all-trans C_nH_{2n+2}, C-C 1.53 A, C-H 1.09 A,
  tetrahedral angles, Gaussian jitter sigma per coordinate.
* ``water_cluster(m, seed)``: rigid waters (O-H 0.9572 A, HOH 104.52 deg) with O
  on a cubic grid of spacing 3.1 A (ceil(m^(1/3))^3 sites, first m used), O
  jitter sigma = 0.15 A, uniformly random orientations; a molecule whose O lands
  closer than 2.6 A to an earlier O is redrawn.
"""
import math

import numpy as np

AUTOAA = 0.52917726
TET = math.radians(109.4712206)


def _unit(v):
    return v / np.linalg.norm(v)


def alkane(n, sigma=0.02, seed=0):
    """Return (Z[int], xyz[N,3] Bohr) for all-trans C_nH_{2n+2}."""
    rng = np.random.default_rng(seed)
    cc, ch = 1.53, 1.09
    half = TET / 2
    dx = cc * math.sin(half)
    dz = cc * math.cos(half)
    C = np.array([[k * dx, 0.0, dz * (k % 2)] for k in range(n)])
    Z = [6] * n
    H = []
    ey = np.array([0.0, 1.0, 0.0])
    for k in range(n):
        nb = [C[j] - C[k] for j in (k - 1, k + 1) if 0 <= j < n]
        nb = [_unit(v) for v in nb]
        if len(nb) == 2:
            b = -_unit(nb[0] + nb[1])
            w = _unit(np.cross(nb[0], nb[1]))
            for s in (1, -1):
                H.append(C[k] + ch * (b * math.cos(TET / 2) + s * w * math.sin(TET / 2)))
        elif len(nb) == 1:
            u = nb[0]
            # staggered CH3: one H anti-periplanar in the backbone plane
            ref = np.array([0.0, 0.0, 1.0 if k % 2 == 0 else -1.0])
            e1 = _unit(ref - u * (ref @ u))
            e2 = np.cross(u, e1)
            for phi in (0.0, 2 * math.pi / 3, 4 * math.pi / 3):
                d = u * math.cos(TET) + math.sin(TET) * (math.cos(phi) * e1 + math.sin(phi) * e2)
                H.append(C[k] + ch * d)
        else:  # methane
            dirs = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]]) / math.sqrt(3.0)
            for d in dirs:
                H.append(C[k] + ch * d)
    xyz = np.vstack([C, np.array(H)])
    Z = np.array(Z + [1] * len(H), dtype=np.int32)
    xyz = xyz + rng.normal(0.0, sigma, size=xyz.shape)
    return Z, xyz / AUTOAA


def _rand_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def water_cluster(m, seed=0, spacing=3.1, jitter=0.15, dmin=2.6):
    """Return (Z[int], xyz[3m,3] Bohr) for a seeded (H2O)_m cluster."""
    rng = np.random.default_rng(seed)
    g = int(math.ceil(m ** (1.0 / 3.0) - 1e-9))
    sites = np.array([(i, j, k) for i in range(g) for j in range(g) for k in range(g)], dtype=float)[:m] * spacing
    roh, ang = 0.9572, math.radians(104.52)
    h1 = roh * np.array([math.sin(ang / 2), 0.0, math.cos(ang / 2)])
    h2 = roh * np.array([-math.sin(ang / 2), 0.0, math.cos(ang / 2)])
    O = []
    out = []
    for s in sites:
        for _ in range(1000):
            o = s + rng.normal(0.0, jitter, size=3)
            if not O or np.min(np.linalg.norm(np.array(O) - o, axis=1)) >= dmin:
                break
        O.append(o)
        R = _rand_rotation(rng)
        out.extend([o, o + R @ h1, o + R @ h2])
    Z = np.array([8, 1, 1] * m, dtype=np.int32)
    return Z, np.array(out) / AUTOAA


def mixed_batch(count=4096, seed=0):
    """Half alkanes C_nH_{2n+2} (n ~ U{1..20}), half water clusters (m ~ U{2..30})."""
    rng = np.random.default_rng(seed)
    mols = []
    for k in range(count):
        if k % 2 == 0:
            n = int(rng.integers(1, 21))
            mols.append(alkane(n, 0.02, seed=int(rng.integers(1 << 31))))
        else:
            m = int(rng.integers(2, 31))
            mols.append(water_cluster(m, seed=int(rng.integers(1 << 31))))
    return mols


def served_stream(count=128, seed=0, rate=None, nmin=3, nmax=1500):
    """Seeded request stream of the served benchmark.

    Atom counts log-uniform in [nmin, nmax], rounded to the nearest size the generators
    make (alkane C_nH_{2n+2}: 3n + 2 atoms; water cluster (H2O)_m: 3m atoms); alkane or
    water with probability 1/2, gradient requested with probability 1/2.  ``rate`` (requests/s)
    gives Poisson arrival times; None makes every request arrive at t = 0.
    Returns a list of dicts: numbers, positions (Bohr), gradient, arrival, kind, size.
    """
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for _ in range(count):
        natoms = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        alk = rng.random() < 0.5
        grad = bool(rng.random() < 0.5)
        sub = int(rng.integers(1 << 31))
        if alk:
            n = max(1, int(round((natoms - 2) / 3.0)))
            Z, xyz = alkane(n, 0.02, seed=sub)
        else:
            m = max(1, int(round(natoms / 3.0)))
            Z, xyz = water_cluster(m, seed=sub)
        if rate:
            t += rng.exponential(1.0 / rate)
        out.append({"numbers": Z, "positions": xyz, "gradient": grad, "arrival": t,
                    "kind": "alkane" if alk else "water", "size": len(Z)})
    return out
