"""Lowest-curvature mode search with the Hessian-vector product kernel.

The reference's ART method (MD_Method_ART_GPU.F90:375-658) pushes along the displacement and
projects the force on the host; a curvature there would need finite-difference force pairs
around every probe.  Here the Hessian acts through ``Engine.hvp`` (one forward-over-reverse
pass pair on the GPU) inside a Lanczos iteration with full reorthogonalisation.  The three
rigid translations of a periodic box are exact zero modes; they are projected out of every
Krylov vector so the lowest Ritz value is the lowest physical curvature.
"""
import numpy as np


def _project_translations(x):
    x = x.reshape(-1, 3)
    return (x - x.mean(axis=0, keepdims=True)).reshape(-1)


def lanczos_lowest(matvec, n_atoms, iters=50, seed=0, project=True, v0=None):
    """matvec(v[N,3]) -> H v [N,3].  Returns (lowest Ritz value, its unit mode [N,3],
    all Ritz values, per-iteration list of Krylov vectors used).  v0 (N,3) starts the Krylov
    space (e.g. the previous mode of a saddle search), else a seeded random vector."""
    rng = np.random.default_rng(seed)
    q = rng.normal(size=3 * n_atoms) if v0 is None else np.asarray(v0, np.float64).reshape(-1).copy()
    if project:
        q = _project_translations(q)
    q /= np.linalg.norm(q)
    Q, alpha, beta = [], [], []
    q_prev = np.zeros_like(q)
    b_prev = 0.0
    for _ in range(iters):
        w = matvec(q.reshape(-1, 3)).reshape(-1)
        if project:
            w = _project_translations(w)
        a = float(q @ w)
        w = w - a * q - b_prev * q_prev
        for qi in Q:                       # full reorthogonalisation
            w -= (qi @ w) * qi
        w -= (q @ w) * q
        Q.append(q)
        alpha.append(a)
        b = float(np.linalg.norm(w))
        if b < 1e-12:
            break
        beta.append(b)
        q_prev, q, b_prev = q, w / b, b
    m = len(alpha)
    T = np.diag(alpha) + np.diag(beta[:m - 1], 1) + np.diag(beta[:m - 1], -1)
    ev, evec = np.linalg.eigh(T)
    mode = np.array(Q).T @ evec[:, 0]
    mode /= np.linalg.norm(mode)
    return float(ev[0]), mode.reshape(-1, 3), ev, Q


def lanczos_lowest_t(matvec, like, iters=50, seed=0, project=True, v0=None):
    """The same Lanczos iteration on torch tensors of shape (3, N) (the library's XP layout)
    on like's device, so that a GPU-resident caller keeps every Krylov vector in device
    memory; only the small tridiagonal problem goes to the host.  matvec(v) -> H v, same
    shape.  Returns (lowest Ritz value, unit mode (3, N), all Ritz values)."""
    import torch
    if v0 is None:
        g = torch.Generator().manual_seed(int(seed))
        q = torch.randn(like.shape, generator=g, dtype=torch.float64).to(like.device)
    else:
        q = v0.detach().clone().to(like.device, torch.float64)
    if project:
        q = q - q.mean(dim=1, keepdim=True)
    q = q / torch.linalg.norm(q)
    Q, alpha, beta = [], [], []
    q_prev = torch.zeros_like(q)
    b_prev = 0.0
    for _ in range(iters):
        w = matvec(q)
        if project:
            w = w - w.mean(dim=1, keepdim=True)
        a = float(torch.sum(q * w))
        w = w - a * q - b_prev * q_prev
        for qi in Q:                       # full reorthogonalisation
            w = w - torch.sum(qi * w) * qi
        w = w - torch.sum(q * w) * q
        Q.append(q)
        alpha.append(a)
        b = float(torch.linalg.norm(w))
        if b < 1e-12:
            break
        beta.append(b)
        q_prev, q, b_prev = q, w / b, b
    m = len(alpha)
    T = np.diag(alpha) + np.diag(beta[:m - 1], 1) + np.diag(beta[:m - 1], -1)
    ev, evec = np.linalg.eigh(T)
    mode = torch.zeros_like(Q[0])
    for k, qk in enumerate(Q):
        mode = mode + float(evec[k, 0]) * qk
    mode = mode / torch.linalg.norm(mode)
    return float(ev[0]), mode, ev


def fd_hvp(force, x, v, delta=1e-4):
    """Central finite difference of the force along the unit vector v (the reference-style
    curvature probe): H v ~ -(F(x + delta v) - F(x - delta v)) / (2 delta)."""
    return -(force(x + delta * v) - force(x - delta * v)) / (2.0 * delta)
