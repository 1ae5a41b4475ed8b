"""The mixed-precision algorithm of the device-wide solve, restated in numpy
on oracle matrices (no GPU): a complex64 matvec; the Lanczos basis and work
vector stored in complex64 (or FP64, for comparison) with accurately computed
dots and updates; selective reorthogonalisation at 1e-7 |w|; a thick restart
keeping nev + 2 Ritz vectors; the Rayleigh-Ritz check over the Gram-
orthonormalised Ritz block with FP64 matvecs, accepted under the quadratic
bound r^2 <= 1e-10 |E| gap for isolated pairs.  Storing the basis in complex64 must reach the
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


def pair_accepted(i, lam, r, thL, tol, scale):
    """The library's mixed_pair_accepted: r_i <= tol, or pair i isolated
    (gap > 2 r_i) with r_i^2 / gap <= 1e-10 |E|, the gap taken to
    thL = theta_L - r_L, the lower end of the first Lanczos Ritz interval
    above the block."""
    if r[i] <= tol:
        return True
    gap = thL - lam[i]
    return gap > 2 * r[i] and r[i] ** 2 <= 1e-10 * max(abs(lam[i]), 1e-6 * scale) * gap


def _mixed_solve(H, nev_out, basis_c64, m=30, seed=5, sel=1e-7):
    """Returns (eigenvalues, matvecs, fp64_fallback): a run that stagnates at
    the complex64 noise floor is answered by an FP64 solve, as in the library
    (here a dense eigensolve stands in for it)."""
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
            rL = 0.0 if (invariant or msz <= nw) else abs(beta * Z[msz - 1, nw])
            thL = (th[nw] - rL) if msz > nw else np.inf
            if all(pair_accepted(i, lam, r, thL, 1e-10, scale) for i in range(nev_out)):
                return lam[:nev_out], nmv, False
            if invariant or stagnated or tau <= 1e-9:
                return np.linalg.eigvalsh(H.toarray())[:nev_out], nmv, True
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
    e64, n64, f64 = _mixed_solve(H, nev, basis_c64=False)
    e32, n32, f32 = _mixed_solve(H, nev, basis_c64=True)
    assert not f64 and not f32
    for e in (e64, e32):
        assert np.max(np.abs(e - exact) / np.abs(exact)) <= 1e-9, (label, e, exact)
    assert abs(n32 - n64) <= max(6, 0.1 * n64), (label, n32, n64)


@pytest.mark.parametrize("h_z", [1e-5, 1e-4, 1e-3])
@pytest.mark.parametrize("sector", [0, 2])
@pytest.mark.parametrize("seed", [1, 2, 3, 5])
@pytest.mark.parametrize("m", [24, 30])
def test_near_degenerate_cluster_is_never_accepted_wrong(oracle, h_z, sector, seed, m):
    """Hubbard 2x4 (8 electrons over all S^z) with a Zeeman term h_z: the third
    level of sectors 0 and 2 opens a cluster of five levels 2 h_z apart that
    straddles the polish block.  The acceptance test must never accept a
    Rayleigh-Ritz value mixed across the cluster: every run returns the lowest
    levels within 1e-9 relative, from the complex64 run or from the FP64
    fallback.  (With the gap taken to theta_L itself rather than to
    theta_L - r_L, and no isolation condition, values off by up to 1e-6
    relative were accepted at the smallest splittings.)  Clusters narrower
    than the complex64 run's residuals (h_z of a few 1e-6 here), which it
    never splits into distinct Ritz values, are outside what any residual test
    can see and are not asserted."""
    spec = L.hubbard_square(2, 4, n_filled=8)
    spec.density_terms = (list(spec.density_terms) + [(i + 1, i + 1, complex(h_z)) for i in range(8)]
                          + [(i + 9, i + 9, complex(-h_z)) for i in range(8)])
    _, _, op = oracle_objects(oracle, Case("hubbard2x4_zeeman", spec), sector)
    r, c, v = op.matrix_coo()
    H = sp.csr_matrix((v, (r, c)), shape=(op.dim, op.dim))
    exact = np.linalg.eigvalsh(H.toarray())[:3]
    e, _, _ = _mixed_solve(H, 3, basis_c64=True, m=m, seed=seed)
    assert np.max(np.abs(e - exact) / np.abs(exact)) <= 1e-9, (e - exact)
