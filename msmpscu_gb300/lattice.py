"""Seeded synthetic inputs of the benchmark configurations (no datasets are involved).

fcc / bcc lattices, Gaussian displacements, vacancies, a <111> self-interstitial dumbbell and
Maxwell-Boltzmann velocities with the centre-of-mass motion removed.
Units: Angstrom, eV, fs; masses in eV*fs^2/A^2.
"""
import numpy as np

AMU = 103.642697          # 1 amu in eV*fs^2/A^2
KB = 8.617333262e-5       # Boltzmann constant, eV/K

# Cleri-Rosato parameters for Cu (A, xi in eV; p, q; r0 in A) and the cutoffs of the
# benchmark: rc midway between the 3rd (4.427 A) and 4th (5.112 A) fcc shells at a=3.615 A,
# list cutoff rc + 0.3 A skin.
CU_CR = dict(A=0.0855, xi=1.224, p=10.960, q=2.278, r0=2.5563)
CU_A = 3.615
CU_RC = 4.77
CU_RC_NL = 5.07
CU_MASS = 63.546 * AMU
W_A = 3.1652
W_RC = 5.4604375
W_RC_NL = W_RC + 0.3
W_MASS = 183.84 * AMU


def fcc(nx, ny, nz, a):
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 1, 3)
    pos = ((g + base[None]) * a).reshape(-1, 3)
    return pos, np.array([nx * a, ny * a, nz * a])


def bcc(nx, ny, nz, a):
    base = np.array([[0, 0, 0], [0.5, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 1, 3)
    pos = ((g + base[None]) * a).reshape(-1, 3)
    return pos, np.array([nx * a, ny * a, nz * a])


def hcp(nx, ny, nz, a, c):
    """hcp in its orthorhombic cell (a, a sqrt(3), c) of four atoms."""
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 5.0 / 6.0, 0.5], [0, 1.0 / 3.0, 0.5]])
    cell = np.array([a, a * np.sqrt(3.0), c])
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 1, 3)
    pos = ((g + base[None]) * cell).reshape(-1, 3)
    return pos, cell * np.array([nx, ny, nz])


def wrap(pos, lo, length):
    return lo + np.mod(pos - lo, length)


def displace(pos, sigma, rng, lo, length):
    return wrap(pos + rng.normal(0.0, sigma, pos.shape), lo, length)


def velocities(n, mass, temp, rng):
    """Maxwell-Boltzmann at temp (K) with zero total momentum (equal masses)."""
    if temp <= 0:
        return np.zeros((n, 3))
    v = rng.normal(0.0, np.sqrt(KB * temp / mass), (n, 3))
    return v - v.mean(0, keepdims=True)


def dumbbell_111(pos, length, a):
    """Replaces the lattice atom nearest the box centre by a <111> dumbbell: two atoms at
    +-b/3 along [111] (b = sqrt(3)/2 a, the bcc nearest-neighbour distance), so the dumbbell
    bond and its distances to the next atoms of the [111] row are all 2b/3 (unrelaxed)."""
    c = length / 2.0
    d = np.linalg.norm(pos - c, axis=1)
    k = int(np.argmin(d))
    centre = pos[k].copy()
    u = np.array([1.0, 1.0, 1.0]) / np.sqrt(3.0)
    half = (0.5 * np.sqrt(3.0) * a) / 3.0
    pos = pos.copy()
    pos[k] = centre - half * u
    return np.vstack([pos, centre + half * u])


def cu_config(ncell, sigma, temp, seed, vacancies=0):
    """fcc Cu block of ncell^3 cells: positions (wrapped), velocities, box length."""
    rng = np.random.default_rng(seed)
    pos, length = fcc(ncell, ncell, ncell, CU_A)
    if vacancies:
        keep = np.ones(len(pos), bool)
        keep[rng.choice(len(pos), vacancies, replace=False)] = False
        pos = pos[keep]
    pos = displace(pos, sigma, rng, np.zeros(3), length)
    vel = velocities(len(pos), CU_MASS, temp, rng)
    return pos, vel, length


def w_sia_config(ncell, sigma, seed):
    rng = np.random.default_rng(seed)
    pos, length = bcc(ncell, ncell, ncell, W_A)
    pos = dumbbell_111(pos, length, W_A)
    pos = displace(pos, sigma, rng, np.zeros(3), length) if sigma > 0 else wrap(pos, 0.0, length)
    return pos, length


def uneven_batch(nbox, seed, cmin=4, cmax=12, vac_max=3, tmin=300.0, tmax=1200.0, sigma=0.05):
    """nbox periodic Cu boxes with edge uniform in [cmin, cmax] cells, 0..vac_max vacancies,
    temperature uniform in [tmin, tmax]; returns a list of (pos, vel, length)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nbox):
        nc = int(rng.integers(cmin, cmax + 1))
        nv = int(rng.integers(0, vac_max + 1))
        t = float(rng.uniform(tmin, tmax))
        pos, length = fcc(nc, nc, nc, CU_A)
        if nv:
            keep = np.ones(len(pos), bool)
            keep[rng.choice(len(pos), nv, replace=False)] = False
            pos = pos[keep]
        pos = displace(pos, sigma, rng, np.zeros(3), length)
        out.append((pos, velocities(len(pos), CU_MASS, t, rng), length))
    return out
