"""Oracle restatement of the stochastic-Galerkin operator, preconditioner and solvers.

Test infrastructure only (see ``oracle/__init__.py``).

Follows src/modelproblems/solvers_poisson_primal.jl:
  mul!                       :86-124   (per-G-nonzero SpMV, Dirichlet rows zeroed)
  MyPreconditionerPrimal     :23-44    (K_0 with 1e60 on boundary diagonals, LU)
  ldiv!                      :47-78    (one LU solve per mode)
  solve_primal!              :130-169  (RHS = x0 + e_1 (x) b0, boundary rows zeroed,
                                        left-preconditioned GMRES, atol = rtol = 1e-14)
  solve_full_primal!         :172-230  (Kronecker matrix, direct solve)
and src/modelproblems/solvers_logpoisson_primal.jl:87-127 for the
non-symmetric (lognormal) operator, which has the same shape with N_m.

Vectors use the reference layout: ``entries`` is column-major n x P, i.e.
mode mu occupies entries[mu*n:(mu+1)*n].  The LU factorisation is SciPy's
SuperLU, used as a library (the reference uses UMFPACK through SparseArrays).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def mul_literal(x, K0, Ks, G, bdofs, P):
    """mul!(Ax, S::MySystemPrimal, x), solvers_poisson_primal.jl:86-124.

    G is the dense (M*P) x P coupling array; Ks = [K_1..K_M] (CSR or CSC).
    """
    n = K0.shape[0]
    M = len(Ks)
    Ax = np.zeros(n * P)
    for mu in range(P):
        a, b = mu * n, (mu + 1) * n
        Ax[a:b] += K0 @ x[a:b]
        for nu in range(P):
            for e in range(M):
                g = G[e * P + mu, nu]
                if g != 0:
                    Ax[a:b] += g * (Ks[e] @ x[nu * n:(nu + 1) * n])
        Ax[a + bdofs] = 0.0
    return Ax


def apply_fast(x, K0, Ks, G, bdofs, P):
    """Same operator as mul_literal, grouped per matrix (Y = sum_m K_m X G_m^T);
    used only to keep large oracle runs short.  Equal to mul_literal up to
    floating-point summation order."""
    n = K0.shape[0]
    M = len(Ks)
    X = x.reshape(P, n).T  # n x P
    Y = K0 @ X
    for e in range(M):
        Gm = G[e * P:(e + 1) * P, :]
        cols = np.nonzero(np.any(Gm != 0, axis=0))[0]
        if len(cols) == 0:
            continue
        KX = Ks[e] @ X[:, cols]
        Y += KX @ Gm[:, cols].T
    Y[bdofs, :] = 0.0
    return Y.T.ravel().copy()


class MeanPreconditioner:
    """MyPreconditionerPrimal + ldiv!, solvers_poisson_primal.jl:23-78."""

    def __init__(self, K0, bdofs, P):
        A = sp.lil_matrix(K0.copy())
        for d in bdofs:
            A[d, d] = 1.0e60
        self.lu = spla.splu(sp.csc_matrix(A))
        self.n = K0.shape[0]
        self.P = P

    def ldiv(self, b):
        y = np.empty_like(b)
        n = self.n
        for mu in range(self.P):
            y[mu * n:(mu + 1) * n] = self.lu.solve(b[mu * n:(mu + 1) * n])
        return y


def reference_rhs(x0, b0, bdofs, P):
    """solvers_poisson_primal.jl:149-155: b = x0 + e_1 (x) b0, boundary rows zeroed."""
    n = len(b0)
    b = x0.copy()
    b[:n] += b0
    for mu in range(P):
        b[mu * n + bdofs] = 0.0
    return b


def gmres_left(apply, prec, b, x0, atol=1e-14, rtol=1e-14, itmax=400):
    """Left-preconditioned full GMRES with modified Gram-Schmidt and Givens
    rotations (Krylov.jl gmres with M=P, ldiv=true, restart=false, as called at
    solvers_poisson_primal.jl:160).  Stops when ||M^-1 r_k|| <= atol + rtol ||M^-1 r_0||."""
    r0 = b - apply(x0)
    q = prec(r0)
    beta = np.linalg.norm(q)
    eps = atol + rtol * beta
    stats = dict(niter=0, residuals=[beta], solved=beta <= eps)
    if beta == 0.0 or beta <= eps:
        return x0.copy(), stats
    V = [q / beta]
    R = np.zeros((itmax + 1, itmax + 1))
    cs = np.zeros(itmax)
    sn = np.zeros(itmax)
    z = np.zeros(itmax + 1)
    z[0] = beta
    k = 0
    for k in range(itmax):
        w = prec(apply(V[k]))
        for i in range(k + 1):
            R[i, k] = V[i] @ w
            w = w - R[i, k] * V[i]
        hbis = np.linalg.norm(w)
        for i in range(k):
            t = cs[i] * R[i, k] + sn[i] * R[i + 1, k]
            R[i + 1, k] = -sn[i] * R[i, k] + cs[i] * R[i + 1, k]
            R[i, k] = t
        denom = np.hypot(R[k, k], hbis)
        cs[k] = R[k, k] / denom
        sn[k] = hbis / denom
        R[k, k] = denom
        z[k + 1] = -sn[k] * z[k]
        z[k] = cs[k] * z[k]
        rnorm = abs(z[k + 1])
        stats["residuals"].append(rnorm)
        stats["niter"] = k + 1
        if rnorm <= eps or hbis == 0.0:
            stats["solved"] = True
            break
        V.append(w / hbis)
    kk = stats["niter"]
    y = np.linalg.solve(np.triu(R[:kk, :kk]), z[:kk])
    x = x0.copy()
    for i in range(kk):
        x += y[i] * V[i]
    return x, stats


def pcg(apply, prec, b, x0, interior_mask, tol=1e-10, itmax=1000):
    """Preconditioned CG on the interior dofs (boundary entries of every
    iterate stay at their x0 values).  Stops on the true-residual recurrence
    ||r_k|| <= tol ||b||."""
    x = x0.copy()
    r = b - apply(x)
    r[~interior_mask] = 0.0
    z = prec(r)
    z[~interior_mask] = 0.0
    p = z.copy()
    rho = r @ z
    nb = np.linalg.norm(b)
    hist = [np.linalg.norm(r) / nb]
    it = 0
    while hist[-1] > tol and it < itmax:
        q = apply(p)
        alpha = rho / (p @ q)
        x += alpha * p
        r -= alpha * q
        it += 1
        hist.append(np.linalg.norm(r) / nb)
        if hist[-1] <= tol:
            break
        z = prec(r)
        z[~interior_mask] = 0.0
        rho_new = r @ z
        p = z + (rho_new / rho) * p
        rho = rho_new
    return x, dict(niter=it, residuals=hist)


def kron_direct(K0, Ks, G, b0, bdofs, P):
    """solve_full_primal!, solvers_poisson_primal.jl:172-230 (small cases)."""
    n = K0.shape[0]
    M = len(Ks)
    blocks = [[None] * P for _ in range(P)]
    for j in range(P):
        blocks[j][j] = K0.copy().tolil()
    for j in range(P):
        for k in range(P):
            for e in range(M):
                g = G[e * P + j, k]
                if abs(g) > 1e-14:
                    add = g * Ks[e]
                    blocks[j][k] = (add if blocks[j][k] is None else blocks[j][k] + add)
    for j in range(P):
        for k in range(P):
            if blocks[j][k] is not None:
                blocks[j][k] = sp.lil_matrix(blocks[j][k])
    for m in range(P):
        for d in bdofs:
            blocks[m][m][d, d] = 1.0e60
    S = sp.bmat(blocks, format="csc")
    rhs = np.zeros(n * P)
    rhs[:n] = b0
    for m in range(P):
        rhs[m * n + bdofs] = 0.0
    return spla.spsolve(S, rhs)


def interior_mask(n, P, bdofs):
    m = np.ones(n * P, dtype=bool)
    for mu in range(P):
        m[mu * n + bdofs] = False
    return m


def kron_direct_full(K0, Ks, G, b_full, bdofs, P, gtol=1e-12):
    """solve_logpoisson_primal_full!, solvers_logpoisson_primal.jl:175-233 (small
    cases): the assembled SG matrix with A + N_0 on the diagonal blocks, g N_e for
    |g| > 1e-12, 1e60 on boundary diagonals; right-hand side blocks b_mu with
    boundary entries zeroed."""
    n = K0.shape[0]
    M = len(Ks)
    blocks = [[None] * P for _ in range(P)]
    for j in range(P):
        blocks[j][j] = K0.copy().tolil()
    for j in range(P):
        for k in range(P):
            for e in range(M):
                g = G[e * P + j, k]
                if abs(g) > gtol:
                    add = g * Ks[e]
                    blocks[j][k] = (add if blocks[j][k] is None else blocks[j][k] + add)
    for j in range(P):
        for k in range(P):
            if blocks[j][k] is not None:
                blocks[j][k] = sp.lil_matrix(blocks[j][k])
    for m in range(P):
        for d in bdofs:
            blocks[m][m][d, d] = 1.0e60
    S = sp.bmat(blocks, format="csc")
    rhs = np.array(b_full, dtype=np.float64).copy()
    for m in range(P):
        rhs[m * n + bdofs] = 0.0
    return spla.spsolve(S, rhs)
