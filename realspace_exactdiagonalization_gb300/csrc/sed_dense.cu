// sed_dense.cu -- the small-sector branch of diagonalize_block_matrixfree.
//
// For n <= 500 the reference builds the dense sector block from n unit-vector
// matvecs and calls eigen(Hermitian(H)) (src/symmetry_resolved_ed.jl:1004-1017),
// so degenerate levels come back with their full multiplicity.  The columns
// are built here with the device matvec in FP64; the Hermitian eigenproblem is
// solved on the host:
//   1. complex Householder tridiagonalisation (the upper triangle is used, as
//      Julia's Hermitian wrapper does),
//   2. a diagonal unitary scaling that makes the tridiagonal matrix real,
//   3. Sturm-sequence bisection for the lowest k eigenvalues,
//   4. inverse iteration for their eigenvectors (clusters orthogonalised),
//   5. back-transformation through the scaling and the reflectors.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <random>

#include "sed_internal.cuh"

namespace sed {

void op_apply_orbit64(OpImpl& op, const void* xs64, double* ypad, cudaStream_t s);
void compress_vec(const SectorImpl& S, const double* ypad, double* ysec, cudaStream_t s);

using cplx = std::complex<double>;

// Lowest k eigenpairs of the Hermitian n x n matrix whose upper triangle is
// read from column-major Hc; vecs receives k vectors of length n (vector-major).
void dense_eigh_lowest(int n, const cplx* Hc, int k, double* w, cplx* vecs) {
  std::vector<cplx> A((size_t)n * n);  // row-major working copy
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      const cplx v = Hc[(size_t)j * n + i];
      A[(size_t)i * n + j] = (i == j) ? cplx(v.real(), 0.0) : v;
      A[(size_t)j * n + i] = (i == j) ? cplx(v.real(), 0.0) : std::conj(v);
    }
  // 1. Householder: P_c = I - beta v v^H acting on rows/cols c+1..n-1
  std::vector<std::vector<cplx>> refl(std::max(n - 2, 0));
  std::vector<double> betas(std::max(n - 2, 0), 0.0);
  for (int c = 0; c + 2 < n; ++c) {
    const int m = n - c - 1;
    std::vector<cplx> v(m);
    double sig2 = 0.0;
    for (int i = 0; i < m; ++i) {
      v[i] = A[(size_t)(c + 1 + i) * n + c];
      sig2 += std::norm(v[i]);
    }
    const double sig = std::sqrt(sig2);
    if (sig == 0.0) continue;
    const double a0 = std::abs(v[0]);
    const cplx ph = a0 > 0.0 ? v[0] / a0 : cplx(1.0, 0.0);
    v[0] += ph * sig;
    const double vn2 = 2.0 * sig * (sig + a0);
    const double beta = 2.0 / vn2;
    // trailing block B = A[c+1.., c+1..]: p = beta B v, K = beta/2 v^H p, w = p - K v
    std::vector<cplx> p(m, 0.0);
    for (int i = 0; i < m; ++i) {
      cplx s = 0.0;
      const cplx* row = &A[(size_t)(c + 1 + i) * n + c + 1];
      for (int j = 0; j < m; ++j) s += row[j] * v[j];
      p[i] = beta * s;
    }
    cplx vp = 0.0;
    for (int i = 0; i < m; ++i) vp += std::conj(v[i]) * p[i];
    const cplx K = 0.5 * beta * vp;
    for (int i = 0; i < m; ++i) p[i] -= K * v[i];
    for (int i = 0; i < m; ++i) {
      cplx* row = &A[(size_t)(c + 1 + i) * n + c + 1];
      for (int j = 0; j < m; ++j) row[j] -= v[i] * std::conj(p[j]) + p[i] * std::conj(v[j]);
    }
    const cplx e = -ph * sig;
    A[(size_t)(c + 1) * n + c] = e;
    A[(size_t)c * n + c + 1] = std::conj(e);
    for (int i = 1; i < m; ++i) A[(size_t)(c + 1 + i) * n + c] = A[(size_t)c * n + c + 1 + i] = 0.0;
    refl[c] = std::move(v);
    betas[c] = beta;
  }
  // 2. real tridiagonal T' = D^H T D
  std::vector<double> d(n), f(std::max(n - 1, 0));
  std::vector<cplx> D(n, cplx(1.0, 0.0));
  for (int i = 0; i < n; ++i) d[i] = A[(size_t)i * n + i].real();
  for (int i = 0; i + 1 < n; ++i) {
    const cplx e = A[(size_t)(i + 1) * n + i];
    const double ae = std::abs(e);
    f[i] = ae;
    D[i + 1] = ae > 0.0 ? D[i] * (e / ae) : D[i];
  }
  // 3. bisection (Sturm count = number of eigenvalues below x)
  double lo = 1e300, hi = -1e300, tnorm = 0.0;
  for (int i = 0; i < n; ++i) {
    const double r = (i > 0 ? f[i - 1] : 0.0) + (i + 1 < n ? f[i] : 0.0);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
    tnorm = std::max(tnorm, std::fabs(d[i]) + r);
  }
  const double pivmin = std::max(1e-300, 1e-290 * tnorm * tnorm);
  auto count_below = [&](double x) {
    int cnt = 0;
    double q = d[0] - x;
    if (std::fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
    for (int i = 1; i < n; ++i) {
      q = d[i] - x - f[i - 1] * f[i - 1] / q;
      if (std::fabs(q) < pivmin) q = -pivmin;
      if (q < 0) ++cnt;
    }
    return cnt;
  };
  const double span = std::max(hi - lo, 1e-300);
  lo -= 1e-10 * span + 1e-300;
  hi += 1e-10 * span + 1e-300;
  for (int t = 0; t < k; ++t) {
    double a = lo, b = hi;
    for (int it = 0; it < 200 && b - a > 2.2e-16 * std::max(std::fabs(a), std::fabs(b)) + 1e-300; ++it) {
      const double mid = 0.5 * (a + b);
      if (count_below(mid) > t) b = mid;
      else a = mid;
    }
    w[t] = 0.5 * (a + b);
  }
  // 4. inverse iteration on T' - lambda I (tridiagonal LU with partial pivoting)
  std::mt19937_64 rng(0x5EED5EEDull);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::vector<std::vector<double>> Z(k, std::vector<double>(n));
  const double eps = 2.2e-16;
  int cluster_start = 0;
  for (int t = 0; t < k; ++t) {
    if (t > 0 && std::fabs(w[t] - w[t - 1]) > 1e-9 * std::max(tnorm, 1e-300)) cluster_start = t;
    const double lam = w[t];
    // LU of M = T' - lam I with row interchanges: rows hold (u0, u1, u2) bands
    std::vector<double> u0(n), u1(n), u2(n), l(n);
    std::vector<char> sw(n, 0);
    for (int i = 0; i < n; ++i) {
      u0[i] = d[i] - lam;
      u1[i] = i + 1 < n ? f[i] : 0.0;
      u2[i] = 0.0;
    }
    std::vector<double> sub(f);  // sub-diagonal of the not-yet-eliminated rows
    for (int i = 0; i + 1 < n; ++i) {
      if (std::fabs(u0[i]) >= std::fabs(sub[i])) {
        if (u0[i] == 0.0) u0[i] = eps * std::max(tnorm, 1e-300);
        l[i] = sub[i] / u0[i];
        u0[i + 1] -= l[i] * u1[i];
        sw[i] = 0;
      } else {  // swap rows i and i+1
        const double r0 = sub[i], r1 = u0[i + 1], r2 = i + 2 < n ? u1[i + 1] : 0.0;
        l[i] = u0[i] / r0;
        const double o1 = u1[i];
        u0[i] = r0;
        u1[i] = r1;
        u2[i] = r2;
        u0[i + 1] = o1 - l[i] * r1;
        if (i + 2 < n) u1[i + 1] = -l[i] * r2;
        sw[i] = 1;
      }
    }
    if (u0[n - 1] == 0.0) u0[n - 1] = eps * std::max(tnorm, 1e-300);
    std::vector<double>& z = Z[t];
    for (int i = 0; i < n; ++i) z[i] = U(rng);
    for (int iter = 0; iter < 4; ++iter) {
      // forward: apply the row interchanges and multipliers
      for (int i = 0; i + 1 < n; ++i) {
        if (sw[i]) std::swap(z[i], z[i + 1]);
        z[i + 1] -= l[i] * z[i];
      }
      // back substitution with the upper bands
      for (int i = n - 1; i >= 0; --i) {
        double s = z[i];
        if (i + 1 < n) s -= u1[i] * z[i + 1];
        if (i + 2 < n) s -= u2[i] * z[i + 2];
        z[i] = s / u0[i];
      }
      // orthogonalise within the cluster of (nearly) equal eigenvalues
      for (int pass = 0; pass < 2; ++pass)
        for (int q = cluster_start; q < t; ++q) {
          double dot = 0.0;
          for (int i = 0; i < n; ++i) dot += Z[q][i] * z[i];
          for (int i = 0; i < n; ++i) z[i] -= dot * Z[q][i];
        }
      double nr = 0.0;
      for (int i = 0; i < n; ++i) nr += z[i] * z[i];
      nr = std::sqrt(nr);
      if (!(nr > 0.0)) {
        for (int i = 0; i < n; ++i) z[i] = U(rng);
        continue;
      }
      for (int i = 0; i < n; ++i) z[i] /= nr;
    }
  }
  // 5. x = P_0 P_1 ... P_{n-3} D z
  for (int t = 0; t < k; ++t) {
    cplx* x = vecs + (size_t)t * n;
    for (int i = 0; i < n; ++i) x[i] = D[i] * Z[t][i];
    for (int c = n - 3; c >= 0; --c) {
      if (betas[c] == 0.0) continue;
      const std::vector<cplx>& v = refl[c];
      const int m = n - c - 1;
      cplx s = 0.0;
      for (int i = 0; i < m; ++i) s += std::conj(v[i]) * x[c + 1 + i];
      s *= betas[c];
      for (int i = 0; i < m; ++i) x[c + 1 + i] -= s * v[i];
    }
  }
}

__global__ void k_unit_xs(int64_t n_orb, uint32_t orbit, double scale, double2* __restrict__ xs) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x)
    xs[o] = make_double2(o == orbit ? scale : 0.0, 0.0);
}

// The dense branch: columns H e_j from the FP64 device matvec, then the host
// eigensolver.  Returns the lowest nev eigenvalues (and vectors when asked).
SolveResult solve_dense(OpImpl& op, int nev, double* evals, double* evecs) {
  SolveResult res;
  const SectorImpl& S = *op.sec;
  const CatalogImpl& C = *S.cat;
  const int64_t D = S.dim, n = C.n_orbits;
  cudaStream_t s = op.stream;
  std::vector<uint32_t> row_orbit(D);
  SED_CUDA(cudaMemcpyAsync(row_orbit.data(), S.row_orbit.p, (size_t)D * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
  DevBuf xs((size_t)n * 16), ypad((size_t)n * 16), Hd((size_t)D * D * 16);
  for (int64_t j = 0; j < D; ++j) {
    const uint32_t o = row_orbit[j];
    const double sq = std::sqrt((double)C.stab_host[o]);
    k_unit_xs<<<grid1(n, 256), 256, 0, s>>>(n, o, sq, xs.as<double2>());
    op_apply_orbit64(op, xs.p, ypad.as<double>(), s);
    compress_vec(S, ypad.as<double>(), Hd.as<double>() + (size_t)j * D * 2, s);
    ++res.matvecs64;
  }
  SED_CUDA(cudaGetLastError());
  std::vector<cplx> H((size_t)D * D);
  SED_CUDA(cudaMemcpyAsync(H.data(), Hd.p, (size_t)D * D * 16, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
  const int k = (int)std::min<int64_t>(nev, D);
  std::vector<cplx> V((size_t)k * D);
  dense_eigh_lowest((int)D, H.data(), k, evals, V.data());
  if (evecs) std::memcpy(evecs, V.data(), (size_t)k * D * 16);
  // residual check of the returned pairs against the assembled matrix
  double maxr = 0.0;
  for (int t = 0; t < k; ++t) {
    double r2 = 0.0;
    for (int64_t i = 0; i < D; ++i) {
      cplx acc = 0.0;
      for (int64_t j = 0; j < D; ++j) {
        const cplx h = j >= i ? H[(size_t)j * D + i] : std::conj(H[(size_t)i * D + j]);
        acc += (i == j ? cplx(h.real(), 0.0) : h) * V[(size_t)t * D + j];
      }
      r2 += std::norm(acc - evals[t] * V[(size_t)t * D + i]);
    }
    maxr = std::max(maxr, std::sqrt(r2));
  }
  res.converged = k;
  res.max_residual = maxr;
  return res;
}

}  // namespace sed
