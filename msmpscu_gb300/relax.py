"""Minimisation and saddle search on top of the device force and HVP calls.

The reference's ART method (MD_Method_ART_GPU.F90:375-732) activates along a displacement,
tests curvature with finite-difference force pairs and relaxes with its minimisers on the
host.  Here:

* ``lbfgs_quench``: limited-memory BFGS relaxation (two-loop recursion, initial inverse
  Hessian 1/alpha, step capped at ``maxstep`` per atom, no line search) with one device force
  call per iteration;
* ``saddle_search``: min-mode following to a first-order saddle point: the lowest curvature
  mode of the Hessian comes from Lanczos iterations over ``Engine.hvp`` (exact derivative of
  the table-mode force, warm-started from the previous mode), the force component along the
  mode is inverted (or, while the curvature is positive, only the push along the mode is
  kept) and FIRE integrates the modified force.

Positions travel through ``Engine.update_positions`` (the neighbour list is kept while the
atoms stay inside the skin).
"""
import numpy as np

from .lanczos import lanczos_lowest


def _force(e, x):
    e.update_positions(x)
    e.calforce()
    return e.get_force()


def energy(e, x):
    """Total potential energy (FP64 passes) at x."""
    e.update_positions(x)
    e.calepot()
    return float(e.get_epot().sum())


def lbfgs_quench(e, x0, fmax=1e-4, maxiter=2000, memory=20, alpha=70.0, maxstep=0.1):
    """Relaxes x0 (N,3) until max |F| < fmax.  Returns (x, F, iterations)."""
    x = np.array(x0, np.float64)
    f = _force(e, x)
    S, Y, R = [], [], []
    it = 0
    while it < maxiter and np.abs(f).max() >= fmax:
        g = -f.reshape(-1)
        q = g.copy()
        a = []
        for s, y, r in reversed(list(zip(S, Y, R))):
            ai = r * float(s @ q)
            q -= ai * y
            a.append(ai)
        z = q / alpha
        for (s, y, r), ai in zip(zip(S, Y, R), reversed(a)):
            b = r * float(y @ z)
            z += s * (ai - b)
        d = -z.reshape(-1, 3)
        if float(d.reshape(-1) @ g) >= 0.0:        # not a descent direction: restart
            S, Y, R = [], [], []
            d = f / alpha
        dmax = np.sqrt((d * d).sum(axis=1)).max()
        if dmax > maxstep:
            d *= maxstep / dmax
        x_new = x + d
        f_new = _force(e, x_new)
        s_vec, y_vec = d.reshape(-1), (f - f_new).reshape(-1)
        sy = float(s_vec @ y_vec)
        if sy > 1e-12:
            S.append(s_vec)
            Y.append(y_vec)
            R.append(1.0 / sy)
            if len(S) > memory:
                S.pop(0), Y.pop(0), R.pop(0)
        x, f = x_new, f_new
        it += 1
    return x, f, it


def saddle_search(e, x0, fmax=1e-3, maxiter=3000, lanczos_iters=20, dt=0.05, dtmax=0.2, maxstep=0.05,
                  mode0=None, seed=0):
    """Min-mode following from x0 (N,3) to a first-order saddle point.  Returns
    (x, F, lowest curvature, its mode, iterations); converged when max |F| < fmax with a
    negative lowest curvature."""
    x = np.array(x0, np.float64)
    n = len(x)
    v = np.zeros_like(x)
    mode = None if mode0 is None else np.asarray(mode0, np.float64)
    a_fire, n_pos = 0.1, 0
    lam = np.inf
    f = None
    for it in range(maxiter):
        f = _force(e, x)
        lam, mode, _, _ = lanczos_lowest(e.hvp, n, iters=lanczos_iters, seed=seed, v0=mode)
        fpar = float((f * mode).sum()) * mode
        if lam < 0.0:
            if np.abs(f).max() < fmax:
                return x, f, lam, mode, it
            feff = f - 2.0 * fpar
        else:
            # convex region: climb along the softest mode only
            feff = -fpar if float((f * mode).sum()) != 0.0 else mode * 0.1
        # FIRE on the modified force (unit masses)
        p = float((feff * v).sum())
        fn = np.linalg.norm(feff)
        if p > 0.0:
            vn = np.linalg.norm(v)
            v = (1.0 - a_fire) * v + a_fire * feff * (vn / max(fn, 1e-300))
            n_pos += 1
            if n_pos > 5:
                dt = min(dt * 1.1, dtmax)
                a_fire *= 0.99
        else:
            v[:] = 0.0
            dt *= 0.5
            a_fire, n_pos = 0.1, 0
        v += dt * feff
        dx = dt * v
        dmax = np.sqrt((dx * dx).sum(axis=1)).max()
        if dmax > maxstep:
            dx *= maxstep / dmax
        x = x + dx
    return x, f, lam, mode, maxiter
