"""Minimisation and saddle search on top of the device force and HVP calls.

The reference's ART method (MD_Method_ART_GPU.F90:375-732) activates along a displacement,
tests curvature with finite-difference force pairs and relaxes with its minimisers on the
host.  Here:

* ``lbfgs_quench``: limited-memory BFGS relaxation (two-loop recursion, initial inverse
  Hessian 1/alpha, step capped at ``maxstep`` per atom, no line search) with one device force
  call per iteration;
* ``saddle_search``: min-mode following to a first-order saddle point: the lowest curvature
  mode of the Hessian comes from Lanczos iterations over the HVP (exact derivative of the
  table-mode force, warm-started from the previous mode), the force component along the mode
  is inverted (or, while the curvature is positive, only the push along the mode is kept) and
  FIRE integrates the modified force.

Both work on torch tensors of shape (3, N), the library's XP layout.  With ``device="cuda"``
(or CUDA tensor inputs) every vector, the L-BFGS history and the Krylov basis stay in device
memory: positions, forces and HVPs pass to and from the library by device pointer
(``Engine.update_positions``, ``force_into``, ``hvp_into``), and only scalars reach the host.
Numpy (N, 3) inputs give numpy (N, 3) results.  The neighbour list is kept while the atoms
stay inside the skin.
"""
import numpy as np
import torch

from .lanczos import lanczos_lowest_t


def _prep(x, device):
    """(3, N) float64 tensor on the device; numpy (N, 3) input is transposed."""
    if isinstance(x, torch.Tensor):
        t = x.detach().to(torch.float64)
        return (t.to(device) if device is not None else t).contiguous(), False
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.float64).T))
    return (t.to(device) if device is not None else t).contiguous(), True


def _back(t, numpy_out):
    return t.T.cpu().numpy().copy() if numpy_out else t


def _force(e, x):
    e.update_positions(x)
    e.calforce()
    return e.force_into(torch.empty_like(x))


def energy(e, x):
    """Total potential energy (FP64 passes) at x: numpy (N, 3) or a (3, N) tensor."""
    t, _ = _prep(x, None)
    e.update_positions(t)
    e.calepot()
    return float(e.get_epot().sum())


def _atom_norm_max(d):
    return float(torch.sqrt((d * d).sum(dim=0)).max())


def lbfgs_quench(e, x0, fmax=1e-4, maxiter=2000, memory=20, alpha=70.0, maxstep=0.1, device=None):
    """Relaxes x0 until max |F| < fmax.  Returns (x, F, iterations) in x0's form."""
    x, npy = _prep(x0, device)
    f = _force(e, x)
    S, Y, R = [], [], []
    it = 0
    while it < maxiter and float(f.abs().max()) >= fmax:
        g = -f
        q = g.clone()
        a = []
        for s, y, r in reversed(list(zip(S, Y, R))):
            ai = r * float(torch.sum(s * q))
            q = q - ai * y
            a.append(ai)
        z = q / alpha
        for (s, y, r), ai in zip(zip(S, Y, R), reversed(a)):
            b = r * float(torch.sum(y * z))
            z = z + s * (ai - b)
        d = -z
        if float(torch.sum(d * g)) >= 0.0:          # not a descent direction: restart
            S, Y, R = [], [], []
            d = f / alpha
        dmax = _atom_norm_max(d)
        if dmax > maxstep:
            d = d * (maxstep / dmax)
        x_new = (x + d).contiguous()
        f_new = _force(e, x_new)
        y_vec = f - f_new
        sy = float(torch.sum(d * y_vec))
        if sy > 1e-12:
            S.append(d)
            Y.append(y_vec)
            R.append(1.0 / sy)
            if len(S) > memory:
                S.pop(0), Y.pop(0), R.pop(0)
        x, f = x_new, f_new
        it += 1
    return _back(x, npy), _back(f, npy), it


def saddle_search(e, x0, fmax=1e-3, maxiter=3000, lanczos_iters=20, dt=0.05, dtmax=0.2, maxstep=0.05,
                  mode0=None, seed=0, device=None):
    """Min-mode following from x0 to a first-order saddle point.  Returns (x, F, lowest
    curvature, its unit mode, iterations) in x0's form; converged when max |F| < fmax with
    a negative lowest curvature."""
    x, npy = _prep(x0, device)
    v = torch.zeros_like(x)
    mode = None if mode0 is None else _prep(mode0, x.device)[0]

    def hvp(u):
        return e.hvp_into(u.contiguous(), torch.empty_like(u))

    a_fire, n_pos = 0.1, 0
    lam = float("inf")
    f = None
    for it in range(maxiter):
        f = _force(e, x)
        lam, mode, _ = lanczos_lowest_t(hvp, x, iters=lanczos_iters, seed=seed, v0=mode)
        fm = float(torch.sum(f * mode))
        fpar = fm * mode
        if lam < 0.0:
            if float(f.abs().max()) < fmax:
                return _back(x, npy), _back(f, npy), lam, _back(mode, npy), it
            feff = f - 2.0 * fpar
        else:
            # convex region: climb along the softest mode only
            feff = -fpar if fm != 0.0 else mode * 0.1
        # FIRE on the modified force (unit masses)
        p = float(torch.sum(feff * v))
        fn = float(torch.linalg.norm(feff))
        if p > 0.0:
            vn = float(torch.linalg.norm(v))
            v = (1.0 - a_fire) * v + a_fire * feff * (vn / max(fn, 1e-300))
            n_pos += 1
            if n_pos > 5:
                dt = min(dt * 1.1, dtmax)
                a_fire *= 0.99
        else:
            v = torch.zeros_like(v)
            dt *= 0.5
            a_fire, n_pos = 0.1, 0
        v = v + dt * feff
        dx = dt * v
        dmax = _atom_norm_max(dx)
        if dmax > maxstep:
            dx = dx * (maxstep / dmax)
        x = (x + dx).contiguous()
    return _back(x, npy), _back(f, npy), lam, _back(mode, npy), maxiter
