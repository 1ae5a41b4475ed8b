"""The mixed-precision algorithm of the device-wide solve, restated in numpy
on oracle matrices (no GPU): a complex64 matvec; the Lanczos basis and work
vector stored in complex64 (or FP64, for comparison) with accurately computed
dots and updates; selective reorthogonalisation at 1e-7 |w|; a thick restart
keeping nev + 2 Ritz vectors; the Rayleigh-Ritz check over the Gram-
orthonormalised Ritz block with FP64 matvecs, accepted under the quadratic
bound r^2 <= 1e-10 |E| gap.  Storing the basis in complex64 must reach the
same accuracy (|dE|/|E| <= 1e-9) in about the same number of matvecs as
FP64-class storage: the storage rounding is the size of the complex64
matvec's own rounding."""
import numpy as np
import pytest
import scipy.sparse as sp

from cases import Case, oracle_objects
from realspace_exactdiagonalization_gb300 import lattice as L


def _q32(x):
    return x.astype(np.complex64).astype(np.complex128)


def _mixed_solve(H, nev_out, basis_c64, m=30, seed=5, sel=1e-7):
    n = H.shape[0]
    H32 = H.astype(np.complex64)
    nev = min(nev_out + 2, n)
    q = _q32 if basis_c64 else (lambda x: x)
    rng = np.random.default_rng(seed)
    V = np.zeros((n, m + 1), complex)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    V[:, 0] = q(v / np.linalg.norm(v))
    T = np.zeros((m, m))
    k, nmv, beta, tau, restarts = 0, 0, 0.0, 1e-6, 0
    best = [1e300] * 3
    while True:
        jend = m
        for j in range(k, m):
            w = q((H32 @ V[:, j].astype(np.complex64)).astype(np.complex128))
            nmv += 1
            l0 = max(j - 1, 0)
            c = V[:, l0:j + 1].conj().T @ w
            w = q(w - V[:, l0:j + 1] @ c)
            n0 = np.vdot(w, w).real
            cf = V[:, :j + 1].conj().T @ w
            alpha = c[-1].real
            if np.abs(cf).max() > sel * np.sqrt(n0):
                w = q(w - V[:, :j + 1] @ cf)
                alpha += cf[j].real
                nrm2 = np.vdot(w, w).real
                if nrm2 < 0.5 * n0:
                    c2 = V[:, :j + 1].conj().T @ w
                    w = q(w - V[:, :j + 1] @ c2)
                    alpha += c2[j].real
                    nrm2 = np.vdot(w, w).real
            else:
                nrm2 = n0
            beta = np.sqrt(nrm2)
            T[j, j] = alpha
            if j + 1 < m:
                T[j, j + 1] = T[j + 1, j] = beta
            if not beta > 1e-13 * max(1.0, abs(alpha)):
                jend = j + 1
                break
            V[:, j + 1] = q(w / beta)
        msz = jend
        th, Z = np.linalg.eigh(T[:msz, :msz])
        invariant = msz < m or msz == n
        scale = max(1.0, np.abs(th[:nev]).max())
        res = np.zeros(nev_out) if invariant else np.abs(beta * Z[msz - 1, :nev_out])
        maxr = res.max()
        stagnated = restarts >= 6 and maxr < 5e-5 * scale and maxr > 0.7 * best[2]
        best = [min(best[0], maxr), best[0], best[1]]
        done = (res <= tau * scale).all() or invariant or stagnated or restarts >= 300
        keep = min(msz - 1, nev + 2)
        R = V[:, :msz] @ Z[:, :keep]
        if done:
            nw = min(nev, msz)
            B = R[:, :nw]
            HB = H @ B
            M, G = B.conj().T @ HB, B.conj().T @ B
            Li = np.linalg.inv(np.linalg.cholesky(G))
            lam, U = np.linalg.eigh(0.5 * ((Li @ M @ Li.conj().T) + (Li @ M @ Li.conj().T).conj().T))
            X = Li.conj().T @ U
            r = np.linalg.norm(HB @ X - (B @ X) * lam, axis=0)
            gap = (th[nw] if msz > nw else np.inf) - lam
            ok = all(r[i] <= 1e-10 or (gap[i] > 0 and r[i] ** 2 <= 1e-10 * max(abs(lam[i]), 1e-6 * scale) * gap[i])
                     for i in range(nev_out))
            if ok:
                return lam[:nev_out], nmv
            assert not (invariant or stagnated or tau <= 1e-9), "complex64 run stagnated"
            tau *= 0.1
        V[:, :keep] = q(R)
        V[:, keep] = V[:, m]
        T[:] = 0
        T[np.arange(keep), np.arange(keep)] = th[:keep]
        T[keep, :keep] = T[:keep, keep] = beta * Z[msz - 1, :keep]
        k = keep
        restarts += 1


@pytest.mark.parametrize("label,spec,theta,sector,nev", [
    ("ring16_7", L.ring_xxz(16, 1.0, 2.0, n_filled=7), (0.21, 0.0), 1, 3),
    ("heisenberg18", L.heisenberg_ring(18), (0.0, 0.0), 0, 1),
    ("haldane2x4", L.haldane_honeycomb(2, 4), (0.3, 0.6), 2, 2),
])
def test_complex64_basis_matches_fp64_storage(oracle, label, spec, theta, sector, nev):
    case = Case(label, spec, theta=theta)
    _, _, op = oracle_objects(oracle, case, sector)
    r, c, v = op.matrix_coo()
    H = sp.csr_matrix((v, (r, c)), shape=(op.dim, op.dim))
    exact = np.linalg.eigvalsh(H.toarray())[:nev]
    e64, n64 = _mixed_solve(H, nev, basis_c64=False)
    e32, n32 = _mixed_solve(H, nev, basis_c64=True)
    for e in (e64, e32):
        assert np.max(np.abs(e - exact) / np.abs(exact)) <= 1e-9, (label, e, exact)
    assert abs(n32 - n64) <= max(6, 0.1 * n64), (label, n32, n64)
