// sed_lanczos.cu -- device-wide thick-restart Lanczos around the sector matvec.
//
// Replaces diagonalize_block_matrixfree (SRE:998-1030 of
// src/symmetry_resolved_ed.jl), which calls KrylovKit.eigsolve(H, x0, nev,
// :SR; tol=1e-10, maxiter=300).  This is a textbook thick-restart Lanczos
// (Wu & Simon 2000) with full reorthogonalisation by classical Gram-Schmidt
// applied twice; every vector operation is a fused, deterministic reduction
// kernel (fixed grid, fixed summation order), so a solve gives the same bits
// whether it runs alone or beside other work.  Vectors are orbit-indexed
// complex128; the projected matrix and its eigen-decomposition stay on the host.
//
// Mixed precision (SED_PREC_MIXED): the matvec reads complex64 inputs and
// accumulates in FP32, everything else stays FP64; once the Ritz residuals
// reach the FP32 floor, one Rayleigh-Ritz step with FP64 matvecs over
// span{x_i, H x_i - theta_i x_i} polishes the eigenvalues.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "sed_internal.cuh"

namespace sed {

void op_apply_orbit64(OpImpl& op, const void* xs64, double* ypad, cudaStream_t s);
void op_scale_to_xs_prec(OpImpl& op, const double* v, void* xs, bool fp32, cudaStream_t s);
void compress_vec(const SectorImpl& S, const double* ypad, double* ysec, cudaStream_t s);

// ------------------------------------------------------------ dense eigen
void eigh_real_sym(int n, std::vector<double>& A, std::vector<double>& w, std::vector<double>& Z) {
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double v = A[(size_t)i * n + j] * A[(size_t)i * n + j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-32 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        const double th = (aqq - app) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - s * akq;
          A[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - s * aqk;
          A[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double zkp = Z[(size_t)k * n + p], zkq = Z[(size_t)k * n + q];
          Z[(size_t)k * n + p] = c * zkp - s * zkq;
          Z[(size_t)k * n + q] = s * zkp + c * zkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int a, int b) { return A[(size_t)a * n + a] < A[(size_t)b * n + b]; });
  std::vector<double> Zs((size_t)n * n);
  w.assign(n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = A[(size_t)ord[j] * n + ord[j]];
    for (int i = 0; i < n; ++i) Zs[(size_t)i * n + j] = Z[(size_t)i * n + ord[j]];
  }
  Z.swap(Zs);
}

// Complex Hermitian Jacobi: each rotation first makes A_pq real with a phase
// on column q, then applies the real 2x2 rotation that zeroes it.
void eigh_complex_herm(int n, const std::vector<double>& H, std::vector<double>& w, std::vector<double>& Z) {
  std::vector<double> A(H);
  auto re = [&](std::vector<double>& M, int i, int j) -> double& { return M[((size_t)i * n + j) * 2]; };
  auto im = [&](std::vector<double>& M, int i, int j) -> double& { return M[((size_t)i * n + j) * 2 + 1]; };
  Z.assign((size_t)n * n * 2, 0.0);
  for (int i = 0; i < n; ++i) re(Z, i, i) = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double v = re(A, i, j) * re(A, i, j) + im(A, i, j) * im(A, i, j);
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-32 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double ar = re(A, p, q), ai = im(A, p, q);
        const double r = std::hypot(ar, ai);
        if (r == 0.0) continue;
        const double er = ar / r, ei = ai / r;  // e^{i psi}
        const double app = re(A, p, p), aqq = re(A, q, q);
        const double th = (aqq - app) / (2.0 * r);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        // columns: x_q' = x_q e^{-i psi}; new_p = c x_p - s x_q'; new_q = s x_p + c x_q'
        auto colop = [&](std::vector<double>& M) {
          for (int k = 0; k < n; ++k) {
            const double pr = re(M, k, p), pi = im(M, k, p);
            const double qr0 = re(M, k, q), qi0 = im(M, k, q);
            const double qr = qr0 * er + qi0 * ei, qi = qi0 * er - qr0 * ei;
            re(M, k, p) = c * pr - s * qr;
            im(M, k, p) = c * pi - s * qi;
            re(M, k, q) = s * pr + c * qr;
            im(M, k, q) = s * pi + c * qi;
          }
        };
        colop(A);
        // rows: r_q' = e^{i psi} r_q; new_p = c r_p - s r_q'; new_q = s r_p + c r_q'
        for (int k = 0; k < n; ++k) {
          const double pr = re(A, p, k), pi = im(A, p, k);
          const double qr0 = re(A, q, k), qi0 = im(A, q, k);
          const double qr = qr0 * er - qi0 * ei, qi = qi0 * er + qr0 * ei;
          re(A, p, k) = c * pr - s * qr;
          im(A, p, k) = c * pi - s * qi;
          re(A, q, k) = s * pr + c * qr;
          im(A, q, k) = s * pi + c * qi;
        }
        colop(Z);
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return re(A, a, a) < re(A, b, b); });
  std::vector<double> Zs((size_t)n * n * 2);
  w.assign(n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = re(A, ord[j], ord[j]);
    for (int i = 0; i < n; ++i) {
      Zs[((size_t)i * n + j) * 2] = re(Z, i, ord[j]);
      Zs[((size_t)i * n + j) * 2 + 1] = im(Z, i, ord[j]);
    }
  }
  Z.swap(Zs);
}

// ----------------------------------------------------------- vector kernels
static constexpr int kBS = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  return v;
}
// Block sum of (a, b) in a fixed order; result valid in thread 0.
__device__ __forceinline__ double2 block_sum2(double a, double b) {
  __shared__ double sa[32], sb[32];
  a = warp_sum(a);
  b = warp_sum(b);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sa[wid] = a;
    sb[wid] = b;
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    a = lane < nw ? sa[lane] : 0.0;
    b = lane < nw ? sb[lane] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
  }
  __syncthreads();
  return make_double2(a, b);
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Complex Gaussian start vector on the sector's orbits, zero elsewhere.
__global__ void k_start(int64_t n, const uint8_t* __restrict__ rowflag, uint64_t seed, double2* __restrict__ v) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
    if (!rowflag[o]) {
      v[o] = make_double2(0.0, 0.0);
      continue;
    }
    const uint64_t a = splitmix64(seed ^ splitmix64((uint64_t)o));
    const uint64_t b = splitmix64(a);
    const double u1 = ((a >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = ((b >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double r = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    v[o] = make_double2(r * cs, r * sn);
  }
}

__global__ void __launch_bounds__(kBS) k_norm2_part(int64_t n, const double2* __restrict__ v, double* __restrict__ part) {
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = v[i];
    s += x.x * x.x + x.y * x.y;
  }
  const double2 r = block_sum2(s, 0.0);
  if (threadIdx.x == 0) part[blockIdx.x] = r.x;
}

// part[l*nblk + b] = sum over block b's rows of conj(V_l) w
__global__ void __launch_bounds__(kBS) k_multidot(int64_t n, const double2* __restrict__ V, int64_t ld,
                                                  const double2* __restrict__ w, double2* __restrict__ part) {
  const int l = blockIdx.y;
  const double2* __restrict__ v = V + (size_t)l * ld;
  double sr = 0.0, si = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = v[i], b = w[i];
    sr += a.x * b.x + a.y * b.y;
    si += a.x * b.y - a.y * b.x;
  }
  const double2 r = block_sum2(sr, si);
  if (threadIdx.x == 0) part[(size_t)l * gridDim.x + blockIdx.x] = r;
}

// out[l] (=|+=) sum_b part[l*nblk + b]; one block per l, fixed order.
__global__ void __launch_bounds__(kBS) k_reduce_part2(const double2* __restrict__ part, int nblk,
                                                      double2* __restrict__ out, int accumulate) {
  const int l = blockIdx.x;
  double sr = 0.0, si = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    const double2 p = part[(size_t)l * nblk + b];
    sr += p.x;
    si += p.y;
  }
  const double2 r = block_sum2(sr, si);
  if (threadIdx.x == 0) {
    if (accumulate) {
      out[l].x += r.x;
      out[l].y += r.y;
    } else {
      out[l] = r;
    }
  }
}
__global__ void __launch_bounds__(kBS) k_reduce_part1(const double* __restrict__ part, int nblk,
                                                      double* __restrict__ out) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[b];
  const double2 r = block_sum2(s, 0.0);
  if (threadIdx.x == 0) *out = r.x;
}

// w -= sum_l c_l V_l  (and optionally the block partial of |w|^2)
__global__ void __launch_bounds__(kBS) k_multiaxpy(int64_t n, const double2* __restrict__ V, int64_t ld, int nv,
                                                   const double2* __restrict__ c, double2* __restrict__ w,
                                                   double* __restrict__ norm_part) {
  __shared__ double2 sc[128];
  for (int l = threadIdx.x; l < nv; l += blockDim.x) sc[l] = c[l];
  __syncthreads();
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 x = w[i];
    for (int l = 0; l < nv; ++l) {
      const double2 v = V[(size_t)l * ld + i];
      const double2 cl = sc[l];
      x.x -= cl.x * v.x - cl.y * v.y;
      x.y -= cl.x * v.y + cl.y * v.x;
    }
    w[i] = x;
    s += x.x * x.x + x.y * x.y;
  }
  if (norm_part) {
    const double2 r = block_sum2(s, 0.0);
    if (threadIdx.x == 0) norm_part[blockIdx.x] = r.x;
  }
}

// v = w / sqrt(nrm2); xs = sqrt(stab) v in the matvec precision
template <class V>
__global__ void k_normalize(int64_t n, const double2* __restrict__ w, const double* __restrict__ nrm2,
                            double2* __restrict__ v, const uint8_t* __restrict__ stab, V* __restrict__ xs) {
  const double inv = 1.0 / sqrt(*nrm2);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = w[i];
    const double2 y = make_double2(x.x * inv, x.y * inv);
    v[i] = y;
    if (xs) {
      const double sq = sqrt((double)stab[i]);
      xs[i].x = y.x * sq;
      xs[i].y = y.y * sq;
    }
  }
}

// out_c = sum_l V_l S[l][c] for c in [c0, c0+8): complex coefficients
__global__ void __launch_bounds__(kBS) k_rotate(int64_t n, const double2* __restrict__ V, int64_t ld, int msz,
                                                const double2* __restrict__ S, int keep, double2* __restrict__ out) {
  const int c0 = blockIdx.y * 8;
  const int cn = min(8, keep - c0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double ar[8], ai[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) ar[c] = ai[c] = 0.0;
    for (int l = 0; l < msz; ++l) {
      const double2 v = V[(size_t)l * ld + i];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (c < cn) {
          const double2 s = S[(size_t)l * keep + c0 + c];
          ar[c] += v.x * s.x - v.y * s.y;
          ai[c] += v.x * s.y + v.y * s.x;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (c < cn) out[(size_t)(c0 + c) * ld + i] = make_double2(ar[c], ai[c]);
  }
}

// out = a - theta * b
__global__ void k_residual(int64_t n, const double2* __restrict__ a, const double2* __restrict__ b, double theta,
                           double2* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = a[i], y = b[i];
    out[i] = make_double2(x.x - theta * y.x, x.y - theta * y.y);
  }
}

// ------------------------------------------------------------- host driver
namespace {

struct VecOps {
  int64_t n;
  int nblk;
  cudaStream_t s;
  DevBuf part, part1, coef, scal;  // partial sums, coefficients, scalars
  double* host = nullptr;          // pinned scratch
  explicit VecOps(int64_t n_, cudaStream_t s_) : n(n_), s(s_) {
    const int64_t sms = device_sm_count();
    nblk = (int)std::max<int64_t>(1, std::min<int64_t>((n + kBS * 4 - 1) / (kBS * 4), sms * 4));
    part.alloc((size_t)nblk * 130 * 16);
    part1.alloc((size_t)nblk * 8);
    coef.alloc(256 * 16);
    scal.alloc(64);
    SED_CUDA(cudaMallocHost((void**)&host, 4096));
  }
  ~VecOps() {
    if (host) cudaFreeHost(host);
  }
  // scal[slot] = |v|^2
  void norm2(const double2* v, int slot) {
    k_norm2_part<<<nblk, kBS, 0, s>>>(n, v, part1.as<double>());
    k_reduce_part1<<<1, kBS, 0, s>>>(part1.as<double>(), nblk, scal.as<double>() + slot);
  }
  // coef[off .. off+nv) (=|+=) V[0..nv)^H w
  void multidot(const double2* V, int64_t ld, int nv, const double2* w, int off, bool acc) {
    dim3 g(nblk, nv);
    k_multidot<<<g, kBS, 0, s>>>(n, V, ld, w, part.as<double2>());
    k_reduce_part2<<<nv, kBS, 0, s>>>(part.as<double2>(), nblk, coef.as<double2>() + off, acc ? 1 : 0);
  }
  // w -= V[0..nv) coef[off..], optionally scal[slot] = |w|^2
  void multiaxpy(const double2* V, int64_t ld, int nv, double2* w, int off, int norm_slot) {
    k_multiaxpy<<<nblk, kBS, 0, s>>>(n, V, ld, nv, coef.as<double2>() + off, w,
                                     norm_slot >= 0 ? part1.as<double>() : nullptr);
    if (norm_slot >= 0) k_reduce_part1<<<1, kBS, 0, s>>>(part1.as<double>(), nblk, scal.as<double>() + norm_slot);
  }
  void check() { SED_CUDA(cudaGetLastError()); }
};

}  // namespace

SolveResult solve(OpImpl& op, int nev, double tol, int maxiter, int krylovdim, uint64_t seed, double* evals,
                  double* evecs) {
  auto t0 = std::chrono::steady_clock::now();
  SolveResult res;
  const SectorImpl& S = *op.sec;
  const CatalogImpl& C = *S.cat;
  const int64_t n = C.n_orbits;
  const int64_t D = S.dim;
  SED_REQUIRE(nev >= 1, 1, "nev must be positive");
  SED_REQUIRE(maxiter >= 1, 1, "maxiter must be positive");
  if (D == 0) return res;
  nev = (int)std::min<int64_t>(nev, D);
  SED_REQUIRE(nev <= 32, 5, "nev must be at most 32");
  if (krylovdim <= 0) krylovdim = 30;
  const int m = (int)std::min<int64_t>(std::max(krylovdim, 2 * nev + 1), std::min<int64_t>(D, 120));
  const bool mixed = op.precision == 1;
  cudaStream_t s = op.stream;
  const int nslots = std::max(m + 1, 2 * nev + 2);
  const int64_t ld = n;
  DevBuf Vb((size_t)nslots * ld * 16), Wb((size_t)ld * 16), Rb((size_t)std::max(m, 3 * nev) * ld * 16);
  DevBuf xs((size_t)ld * 16), xs64((size_t)ld * 16), Sd((size_t)130 * 130 * 16);
  double2* V = Vb.as<double2>();
  double2* W = Wb.as<double2>();
  double2* R = Rb.as<double2>();
  VecOps ops(n, s);
  auto vec = [&](int j) { return V + (size_t)j * ld; };
  const int gblk = ops.nblk;
  auto normalize = [&](const double2* w, int slot, double2* out, bool to_xs) {
    if (mixed)
      k_normalize<float2><<<gblk, kBS, 0, s>>>(n, w, ops.scal.as<double>() + slot, out, C.stab.as<uint8_t>(),
                                               to_xs ? xs.as<float2>() : nullptr);
    else
      k_normalize<double2><<<gblk, kBS, 0, s>>>(n, w, ops.scal.as<double>() + slot, out, C.stab.as<uint8_t>(),
                                                to_xs ? xs.as<double2>() : nullptr);
  };
  // start vector
  k_start<<<gblk, kBS, 0, s>>>(n, S.rowflag.as<uint8_t>(), seed, W);
  ops.norm2(W, 0);
  normalize(W, 0, vec(0), true);
  ops.check();

  std::vector<double> T((size_t)m * m, 0.0), theta, Z;
  int k = 0;
  double beta = 0.0, best_prev[3] = {1e300, 1e300, 1e300};
  double scale = 1.0;
  for (;;) {
    int jend = m;
    for (int j = k; j < m; ++j) {
      op_apply_orbit(op, xs.p, (double*)W, s);
      // CGS2: two passes of w -= V (V^H w)
      ops.multidot(V, ld, j + 1, W, 0, false);
      ops.multiaxpy(V, ld, j + 1, W, 0, -1);
      ops.multidot(V, ld, j + 1, W, 128, false);
      ops.multiaxpy(V, ld, j + 1, W, 128, 1);
      ops.check();
      SED_CUDA(cudaMemcpyAsync(ops.host, ops.coef.as<double2>() + j, 16, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaMemcpyAsync(ops.host + 2, ops.coef.as<double2>() + 128 + j, 16, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaMemcpyAsync(ops.host + 4, ops.scal.as<double>() + 1, 8, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
      ++res.matvecs;
      const double alpha = ops.host[0] + ops.host[2];
      beta = std::sqrt(ops.host[4]);
      T[(size_t)j * m + j] = alpha;
      if (j + 1 < m) T[(size_t)j * m + j + 1] = T[(size_t)(j + 1) * m + j] = beta;
      if (!(beta > 1e-13 * std::max(1.0, std::fabs(alpha)))) {
        jend = j + 1;
        break;
      }
      normalize(W, 1, vec(j + 1), true);
    }
    const int msz = jend;
    std::vector<double> A((size_t)msz * msz);
    for (int i = 0; i < msz; ++i)
      for (int j = 0; j < msz; ++j) A[(size_t)i * msz + j] = T[(size_t)i * m + j];
    eigh_real_sym(msz, A, theta, Z);
    const bool invariant = msz < m || msz == D;
    scale = 1.0;
    for (int i = 0; i < std::min(nev, msz); ++i) scale = std::max(scale, std::fabs(theta[i]));
    const double tol_w = mixed ? std::max(tol, 2e-6 * scale) : tol;
    int nconv = 0;
    double maxr = 0.0;
    for (int i = 0; i < std::min(nev, msz); ++i) {
      const double r = invariant ? 0.0 : std::fabs(beta * Z[(size_t)(msz - 1) * msz + i]);
      maxr = std::max(maxr, r);
      if (r <= tol_w) ++nconv;
    }
    // FP32 matvec noise floor: stop when the residual no longer improves
    bool stagnated = false;
    if (mixed && res.restarts >= 6 && maxr < 1e-3 * scale && maxr > 0.7 * best_prev[2]) stagnated = true;
    best_prev[2] = best_prev[1];
    best_prev[1] = best_prev[0];
    best_prev[0] = std::min(best_prev[0], maxr);
    const bool done = (nconv >= nev) || invariant || stagnated || res.restarts >= maxiter;
    const int keep = done ? std::min(nev, msz) : std::min(msz - 1, std::max(nev + (m - nev) / 2, nev + 1));
    std::vector<double> Sc((size_t)msz * keep * 2, 0.0);
    for (int l = 0; l < msz; ++l)
      for (int c = 0; c < keep; ++c) Sc[((size_t)l * keep + c) * 2] = Z[(size_t)l * msz + c];
    SED_CUDA(cudaMemcpyAsync(Sd.p, Sc.data(), Sc.size() * 8, cudaMemcpyHostToDevice, s));
    k_rotate<<<dim3(gblk, (keep + 7) / 8), kBS, 0, s>>>(n, V, ld, msz, Sd.as<double2>(), keep, R);
    SED_CUDA(cudaMemcpyAsync(V, R, (size_t)keep * ld * 16, cudaMemcpyDeviceToDevice, s));
    ops.check();
    if (done) {
      res.converged = nconv;
      res.max_residual = maxr;
      res.status = (nconv >= nev || invariant || stagnated) ? 0 : 4;
      for (int i = 0; i < keep; ++i) evals[i] = theta[i];
      break;
    }
    // the last normalised residual direction (slot m) continues the basis
    SED_CUDA(cudaMemcpyAsync(vec(keep), vec(m), (size_t)ld * 16, cudaMemcpyDeviceToDevice, s));
    std::fill(T.begin(), T.end(), 0.0);
    for (int c = 0; c < keep; ++c) {
      T[(size_t)c * m + c] = theta[c];
      const double b = beta * Z[(size_t)(msz - 1) * msz + c];
      T[(size_t)c * m + keep] = T[(size_t)keep * m + c] = b;
    }
    k = keep;
    ++res.restarts;
  }

  if (mixed && res.status == 0) {
    // FP64 Rayleigh-Ritz over B = [Y | Q], Y = Ritz vectors, Q = orthonormal
    // FP64 residual directions; HB = [H Y | H Q] (slots of R).
    std::vector<double> th0(evals, evals + nev);
    double2* Y = V;
    double2* Q = V + (size_t)nev * ld;
    double2* HB = R;
    for (int i = 0; i < nev; ++i) {
      op_scale_to_xs_prec(op, (const double*)(Y + (size_t)i * ld), xs64.p, false, s);
      op_apply_orbit64(op, xs64.p, (double*)(HB + (size_t)i * ld), s);
      ++res.matvecs64;
    }
    int q = 0;
    for (int i = 0; i < nev; ++i) {
      double2* qv = Q + (size_t)q * ld;
      k_residual<<<gblk, kBS, 0, s>>>(n, HB + (size_t)i * ld, Y + (size_t)i * ld, th0[i], W);
      ops.norm2(W, 3);
      ops.multidot(V, ld, nev + q, W, 0, false);
      ops.multiaxpy(V, ld, nev + q, W, 0, -1);
      ops.multidot(V, ld, nev + q, W, 128, false);
      ops.multiaxpy(V, ld, nev + q, W, 128, 2);
      ops.check();
      SED_CUDA(cudaMemcpyAsync(ops.host, ops.scal.as<double>(), 32, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
      const double r0 = std::sqrt(ops.host[3]), r1 = std::sqrt(ops.host[2]);
      if (!(r1 > 1e-14 * scale) || !(r1 > 1e-3 * r0)) continue;  // nothing left to add
      normalize(W, 2, qv, false);
      op_scale_to_xs_prec(op, (const double*)qv, xs64.p, false, s);
      op_apply_orbit64(op, xs64.p, (double*)(HB + (size_t)(nev + q) * ld), s);
      ++res.matvecs64;
      ++q;
    }
    const int nb = nev + q;
    std::vector<double> M((size_t)nb * nb * 2);
    for (int b = 0; b < nb; ++b) {
      ops.multidot(V, ld, nb, HB + (size_t)b * ld, 0, false);
      ops.check();
      SED_CUDA(cudaMemcpyAsync(ops.host, ops.coef.p, (size_t)nb * 16, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
      for (int a = 0; a < nb; ++a) {
        M[((size_t)a * nb + b) * 2] = ops.host[2 * a];
        M[((size_t)a * nb + b) * 2 + 1] = ops.host[2 * a + 1];
      }
    }
    for (int a = 0; a < nb; ++a)  // Hermitian part
      for (int b = a; b < nb; ++b) {
        const double r = 0.5 * (M[((size_t)a * nb + b) * 2] + M[((size_t)b * nb + a) * 2]);
        const double i = 0.5 * (M[((size_t)a * nb + b) * 2 + 1] - M[((size_t)b * nb + a) * 2 + 1]);
        M[((size_t)a * nb + b) * 2] = r;
        M[((size_t)a * nb + b) * 2 + 1] = i;
        M[((size_t)b * nb + a) * 2] = r;
        M[((size_t)b * nb + a) * 2 + 1] = -i;
      }
    std::vector<double> lam, U;
    eigh_complex_herm(nb, M, lam, U);
    std::vector<double> Sc((size_t)nb * nev * 2);
    for (int l = 0; l < nb; ++l)
      for (int c = 0; c < nev; ++c) {
        Sc[((size_t)l * nev + c) * 2] = U[((size_t)l * nb + c) * 2];
        Sc[((size_t)l * nev + c) * 2 + 1] = U[((size_t)l * nb + c) * 2 + 1];
      }
    SED_CUDA(cudaMemcpyAsync(Sd.p, Sc.data(), Sc.size() * 8, cudaMemcpyHostToDevice, s));
    // refined vectors into R[nb ..) then back into V[0..nev)
    double2* out = R + (size_t)nb * ld;
    k_rotate<<<dim3(gblk, (nev + 7) / 8), kBS, 0, s>>>(n, V, ld, nb, Sd.as<double2>(), nev, out);
    SED_CUDA(cudaMemcpyAsync(V, out, (size_t)nev * ld * 16, cudaMemcpyDeviceToDevice, s));
    double maxd = 0.0, maxr = 0.0;
    for (int i = 0; i < nev; ++i) {
      maxd = std::max(maxd, std::fabs(lam[i] - th0[i]));
      evals[i] = lam[i];
      // true FP64 residual of the refined pair
      op_scale_to_xs_prec(op, (const double*)(V + (size_t)i * ld), xs64.p, false, s);
      op_apply_orbit64(op, xs64.p, (double*)W, s);
      ++res.matvecs64;
      k_residual<<<gblk, kBS, 0, s>>>(n, W, V + (size_t)i * ld, lam[i], W);
      ops.norm2(W, 4);
      SED_CUDA(cudaMemcpyAsync(ops.host, ops.scal.as<double>() + 4, 8, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
      maxr = std::max(maxr, std::sqrt(ops.host[0]));
    }
    res.max_delta = maxd;
    res.max_residual = maxr;
  }
  if (evecs) {
    DevBuf ys((size_t)std::max<int64_t>(D, 1) * 16);
    for (int i = 0; i < nev; ++i) {
      compress_vec(S, (const double*)(V + (size_t)i * ld), ys.as<double>(), s);
      SED_CUDA(cudaMemcpyAsync(evecs + (size_t)i * D * 2, ys.p, (size_t)D * 16, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
    }
  }
  SED_CUDA(cudaStreamSynchronize(s));
  res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return res;
}

}  // namespace sed
