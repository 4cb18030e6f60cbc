"""Convergence acceleration of the solver's own fixed-point iterations, on
the host above the C ABI.

The bump channel's iterations (explicit pseudo-time for the flow, the
transposed pseudo-time for the adjoint) contract by only ~1 - 3e-5 per
iteration once the fast transients are gone: the channel's acoustic mode,
reflected almost fully by the total-pressure inlet and the pressure outlet,
decays over ~10^5 iterations per decade.  A few slow modes carry that
decay, and Krylov methods remove a few modes in a few dozen products:

* ``gmres``: restarted GMRES (Saad & Schultz, SIAM J. Sci. Stat. Comput. 7,
  1986) with modified Gram-Schmidt and Givens rotations, for the adjoint's
  linear fixed point.  With G the k-step iteration matrix and S_k the k
  steps from zero, the fixed point x* of x <- G^k x + S_k(g) solves
  (I - G^k) x = S_k(g), and (I - G^k) v = -S_k(A^T v): each product is one
  residual VJP plus k pseudo-time steps (the iteration as preconditioner).
* ``anderson``: Anderson acceleration (Anderson, J. ACM 12, 1965; the
  "type II" form of Walker & Ni, SIAM J. Numer. Anal. 49, 2011) of a
  nonlinear fixed point x <- phi(x), phi = k iterations of the flow solver:
  each step solves a small least-squares problem over the last m
  differences of iterates and of their residuals phi(x) - x.

Both work on flat float64 numpy vectors; the callers supply the products
and maps (``fest3d.adjoint``)."""
import numpy as np


def gmres(matvec, b, x0=None, tol=1e-10, restart=40, maxiter=2000, callback=None):
    """x with ||b - matvec(x)|| <= tol ||b|| (2-norm), restarted every
    `restart` products, at most `maxiter` products.  Returns (x, products,
    history of the relative residual estimates)."""
    b = np.asarray(b, dtype=np.float64)
    n = b.size
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    bn = np.linalg.norm(b)
    hist = []
    if bn == 0.0:
        return np.zeros(n), 0, [0.0]
    products = 0
    r = b - matvec(x) if x0 is not None else b.copy()
    if x0 is not None:
        products += 1
    while products < maxiter:
        beta = np.linalg.norm(r)
        hist.append(beta / bn)
        if beta <= tol * bn:
            break
        m = restart
        V = np.zeros((m + 1, n))
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        e = np.zeros(m + 1)
        e[0] = beta
        V[0] = r / beta
        j_done = 0
        for j in range(m):
            w = matvec(V[j])
            products += 1
            for i in range(j + 1):  # modified Gram-Schmidt
                H[i, j] = np.dot(w, V[i])
                w = w - H[i, j] * V[i]
            H[j + 1, j] = np.linalg.norm(w)
            if H[j + 1, j] > 0.0:
                V[j + 1] = w / H[j + 1, j]
            for i in range(j):  # earlier rotations on the new column
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            d = np.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = (1.0, 0.0) if d == 0.0 else (H[j, j] / d, H[j + 1, j] / d)
            H[j, j] = d
            H[j + 1, j] = 0.0
            e[j + 1] = -sn[j] * e[j]
            e[j] = cs[j] * e[j]
            j_done = j + 1
            est = abs(e[j + 1]) / bn
            hist.append(est)
            if callback:
                callback(products, est)
            if est <= tol or products >= maxiter or H[j, j] == 0.0:
                break
        y = np.linalg.solve(np.triu(H[:j_done, :j_done]), e[:j_done]) if j_done else np.zeros(0)
        x = x + V[:j_done].T @ y
        r = b - matvec(x)  # the true residual at each restart
        products += 1
        if np.linalg.norm(r) <= tol * bn:
            hist.append(np.linalg.norm(r) / bn)
            break
    return x, products, hist


def anderson(phi, x0, m=20, maxiter=500, done=None, scale=None, reg=1e-12):
    """Anderson acceleration of x <- phi(x).  phi(x) returns (phi(x), info);
    done(info, k) ends the iteration when true.  The residuals f = phi(x) - x
    are weighted by 1/scale (per entry) in the least-squares problem, whose
    normal equations carry a relative Tikhonov term reg.  Returns (x, the
    last info, maps evaluated)."""
    x = np.array(x0, dtype=np.float64)
    w = 1.0 / scale if scale is not None else None
    dG, dF = [], []       # differences of the maps and of the weighted residuals
    G = np.zeros((0, 0))  # Gram matrix of the dF columns
    g_prev = f_prev = None
    info = None
    for k in range(maxiter):
        g, info = phi(x)
        f = g - x
        fw = f * w if w is not None else f
        if done is not None and done(info, k):
            return g, info, k + 1
        if f_prev is not None:
            dG.append(g - g_prev)
            dF.append(fw - f_prev)
            if len(dF) > m:
                dG.pop(0), dF.pop(0)
                G = G[1:, 1:]
            col = np.array([np.dot(dF[i], dF[-1]) for i in range(len(dF))])
            Gn = np.zeros((len(dF), len(dF)))
            Gn[:-1, :-1] = G
            Gn[-1, :] = col
            Gn[:, -1] = col
            G = Gn
        g_prev, f_prev = g, fw
        if dF:
            rhs = np.array([np.dot(c, fw) for c in dF])
            lam = reg * max(np.trace(G), 1e-300)
            gam = np.linalg.solve(G + lam * np.eye(len(dF)), rhs)
            x = g - sum(gam[i] * dG[i] for i in range(len(dG)))
        else:
            x = g
    return x, info, maxiter
