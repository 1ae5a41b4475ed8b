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
// accumulates in FP32; the Lanczos basis, restart buffer and work vector are
// complex64, each value rounded once from an accurately computed one (see the
// complex64 kernels below); the full reorthogonalisation is selective
// (kSelReorth).  Once the Ritz estimates of the requested pairs fall below
// 1e-6 |E|, one Rayleigh-Ritz step with FP64 matvecs over the nev + 2 Ritz
// vectors polishes the eigenvalues, and the result is accepted by the
// quadratic bound |dE| <= |r|^2 / gap (see solve).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>

#include "../../include/sed_capi.h"
#include "sed_dfloat.cuh"
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
    if (off <= 1e-29 * std::max(tot, 1e-300)) break;  // rounding level of the off-diagonal part
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        if (std::fabs(apq) <= 1e-18 * (std::fabs(app) + std::fabs(aqq)) + 1e-300) continue;
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
    if (off <= 1e-29 * std::max(tot, 1e-300)) break;  // rounding level of the off-diagonal part
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
  __shared__ double s_sq[65];
  for (int i = threadIdx.x; i < 65; i += blockDim.x) s_sq[i] = sqrt((double)i);
  __syncthreads();
  const double inv = 1.0 / sqrt(*nrm2);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = w[i];
    const double2 y = make_double2(x.x * inv, x.y * inv);
    v[i] = y;
    if (xs) {
      const double sq = s_sq[stab[i]];
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

// ------------------------------------------------ complex64 basis (mixed)
// The mixed-precision solve keeps its Lanczos basis, work vector and restart
// buffer in complex64: 8 bytes per element, half the traffic of an FP64-class
// basis.  Each stored value is rounded once to FP32 from an accurately
// computed one:
// * dot products accumulate FP32 products per thread over short chains (a
//   grid-stride sweep gives each thread a few tens of elements) and sum the
//   thread partials in FP64;
// * updates w -= sum_l c_l v_l apply each coefficient as hi + lo floats, so
//   the large local coefficients (alpha, beta) cancel without losing bits;
// * restart rotations accumulate in double-float (TwoProd, TwoSum);
// * the normalisation multiplies by 1/|w| as hi + lo floats.
// The storage rounding (2^-24) is the size of the complex64 matvec's own
// rounding, which already perturbs the recurrence at that level (Paige's
// local-error model); the FP64 Rayleigh-Ritz check then bounds the
// eigenvalues.  Vectors sit cf_ld(n) elements apart, so each starts on a
// 512-byte boundary, as the kernels' 16-byte loads of element pairs need.
static inline int64_t cf_ld(int64_t n) { return (n + 63) / 64 * 64; }

// FP64 complex -> complex64
__global__ void k_d_to_cf(int64_t n, const double2* __restrict__ in, float2* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = in[i];
    out[i] = make_float2((float)x.x, (float)x.y);
  }
}

// vector blockIdx.y: complex64 (stride ldc) -> FP64 (stride ld)
__global__ void k_cf_to_d(int64_t n, const float2* __restrict__ v, int64_t ldc, double2* __restrict__ out,
                          int64_t ld) {
  const float2* __restrict__ src = v + (size_t)blockIdx.y * ldc;
  double2* __restrict__ dst = out + (size_t)blockIdx.y * ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 x = src[i];
    dst[i] = make_double2(x.x, x.y);
  }
}

__global__ void __launch_bounds__(kBS) k_cf_norm2_part(int64_t n, const float2* __restrict__ v,
                                                       double* __restrict__ part) {
  float s = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 x = v[i];
    s = __fmaf_rn(x.x, x.x, __fmaf_rn(x.y, x.y, s));
  }
  const double2 r = block_sum2((double)s, 0.0);
  if (threadIdx.x == 0) part[blockIdx.x] = r.x;
}

// part[l*nblk + b] = block b's share of conj(V_l) w for the kDotCh vectors of
// chunk blockIdx.y: w is read once per kDotCh basis vectors.  Each thread
// takes two consecutive elements per step (16-byte loads; vectors start on
// 512-byte boundaries), the last one of an odd n by thread 0 of block 0.  A
// bulk L2 prefetch ahead of the threads' loads measured slower here (3.6
// against 5.9 TB/s for 24 vectors of 14.1M elements); vectors of 2^18
// elements and more are staged through shared memory instead
// (k_cf_multidot_tma below), and this kernel serves the shorter ones.
static constexpr int kDotCh = 16;
__device__ __forceinline__ void cf_dot_acc(float& re, float& im, float2 v, float2 x) {
  re = __fmaf_rn(v.x, x.x, __fmaf_rn(v.y, x.y, re));
  im = __fmaf_rn(v.x, x.y, __fmaf_rn(-v.y, x.x, im));
}
__global__ void __launch_bounds__(kBS) k_cf_multidot(int64_t n, const float2* __restrict__ V, int64_t ld, int nv,
                                                     const float2* __restrict__ w, double2* __restrict__ part) {
  const int l0 = blockIdx.y * kDotCh;
  const int cn = min(kDotCh, nv - l0);
  float re[kDotCh], im[kDotCh];
#pragma unroll
  for (int c = 0; c < kDotCh; ++c) re[c] = im[c] = 0.f;
  const int64_t n2 = n >> 1;
  const float4* __restrict__ w4 = reinterpret_cast<const float4*>(w);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 x = w4[i];
#pragma unroll
    for (int c = 0; c < kDotCh; ++c)
      if (c < cn) {
        const float4 v = reinterpret_cast<const float4*>(V + (size_t)(l0 + c) * ld)[i];
        cf_dot_acc(re[c], im[c], make_float2(v.x, v.y), make_float2(x.x, x.y));
        cf_dot_acc(re[c], im[c], make_float2(v.z, v.w), make_float2(x.z, x.w));
      }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < kDotCh; ++c)
      if (c < cn) cf_dot_acc(re[c], im[c], V[(size_t)(l0 + c) * ld + n - 1], w[n - 1]);
  }
#pragma unroll
  for (int c = 0; c < kDotCh; ++c)
    if (c < cn) {
      const double2 r = block_sum2((double)re[c], (double)im[c]);
      if (threadIdx.x == 0) part[(size_t)(l0 + c) * gridDim.x + blockIdx.x] = r;
    }
}


// The same dot products with the vectors staged through shared memory by the
// bulk-copy (TMA) engine.  Each block takes tiles of `tile` elements (a grid
// stride over the tiles); for every tile, lanes 0..cn of warp 0 copy w and the
// chunk's cn vectors into one of two shared-memory stages with
// cp.async.bulk, completing on the stage's mbarrier, while the block reads
// the other stage.  The copy engine keeps a whole stage in flight per SM, which
// the register-held loads of k_cf_multidot cannot: on 4.0M-element vectors a
// 14-vector pass took 111 against 138 us, the two-vector local pass 32 against
// 43 us.  Requirements (checked by the caller): ld a multiple of 64 elements
// and V, w 16-byte aligned, so every copy starts on a 512-byte boundary and
// moves a multiple of 512 bytes; the elements in [n, ld) are read but not used.
// Every wait is bounded: a stage that does not complete within kTmaSpin polls
// sets *err, the block waits (bounded) for its copies still in flight and
// leaves without writing its partials.
static constexpr int kTmaStages = 2;
static constexpr size_t kTmaSmemBudget = 208000;  // bytes of staging per block (one block per SM)
static constexpr int kTmaMinN = 1 << 18;           // below this, too few tiles per block to pipeline
static constexpr uint32_t kTmaSpin = 1u << 26;
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// true when the phase of the given parity completed within kTmaSpin polls
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  for (uint32_t it = 0; it < kTmaSpin; ++it)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(b))
               : "memory");
}
// tile (elements, a multiple of 256) for a chunk of cn vectors plus w
static inline int tma_tile(int cn) {
  const int t = (int)(kTmaSmemBudget / ((size_t)kTmaStages * (cn + 1) * 8)) / 256 * 256;
  return std::max(256, std::min(t, 8192));
}
static inline size_t tma_smem(int cn, int tile) { return 128 + (size_t)kTmaStages * (cn + 1) * tile * 8; }

__global__ void __launch_bounds__(kBS, 1) k_cf_multidot_tma(int64_t n, const float2* __restrict__ V, int64_t ld,
                                                            int nv, const float2* __restrict__ w,
                                                            double2* __restrict__ part, int tile,
                                                            const int* __restrict__ skip, int* __restrict__ err) {
  if (skip && *skip) return;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);    // kTmaStages barriers
  float2* stage = reinterpret_cast<float2*>(smem + 128);  // [kTmaStages][cn + 1][tile]
  __shared__ int s_fail;
  const int l0 = blockIdx.y * kDotCh;
  const int cn = min(kDotCh, nv - l0);
  const int64_t n_tiles = (ld + tile - 1) / tile;
  const int64_t my_tiles = blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const size_t stage_el = (size_t)(cn + 1) * tile;
  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < kTmaStages; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  // warp 0: lane 0 arms the stage's barrier with the tile's bytes, then lane
  // c copies slot c (0: w, c > 0: vector l0 + c - 1)
  auto issue = [&](int64_t i) {
    const int s = (int)(i % kTmaStages);
    const int64_t e0 = (blockIdx.x + i * gridDim.x) * (int64_t)tile;
    const uint32_t bytes = (uint32_t)(min((int64_t)tile, ld - e0) * 8);
    if (lane == 0) mbar_expect_tx(&bar[s], bytes * (uint32_t)(cn + 1));
    __syncwarp();
    if (lane <= cn)
      bulk_g2s(stage + (size_t)s * stage_el + (size_t)lane * tile,
               lane == 0 ? w + e0 : V + (size_t)(l0 + lane - 1) * ld + e0, bytes, &bar[s]);
  };
  if (threadIdx.x < 32)
    for (int64_t i = 0; i < kTmaStages && i < my_tiles; ++i) issue(i);
  float re[kDotCh], im[kDotCh];
#pragma unroll
  for (int c = 0; c < kDotCh; ++c) re[c] = im[c] = 0.f;
  int64_t i = 0;
  for (; i < my_tiles; ++i) {
    const int s = (int)(i % kTmaStages);
    if (!mbar_wait(&bar[s], (uint32_t)((i / kTmaStages) & 1))) atomicExch(&s_fail, 1);
    __syncthreads();
    if (s_fail) break;
    const int64_t e0 = (blockIdx.x + i * gridDim.x) * (int64_t)tile;
    const float2* st = stage + (size_t)s * stage_el;
    for (int q = threadIdx.x; q < tile / 2; q += kBS) {  // element pairs
      const int64_t e = e0 + 2 * q;
      const float4 x = reinterpret_cast<const float4*>(st)[q];
      const bool ok0 = e < n, ok1 = e + 1 < n;
#pragma unroll
      for (int c = 0; c < kDotCh; ++c)
        if (c < cn) {
          const float4 v = reinterpret_cast<const float4*>(st + (size_t)(c + 1) * tile)[q];
          if (ok0) cf_dot_acc(re[c], im[c], make_float2(v.x, v.y), make_float2(x.x, x.y));
          if (ok1) cf_dot_acc(re[c], im[c], make_float2(v.z, v.w), make_float2(x.z, x.w));
        }
    }
    __syncthreads();  // the block is done with stage s: refill it
    if (threadIdx.x < 32 && i + kTmaStages < my_tiles) issue(i + kTmaStages);
  }
  if (s_fail) {
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      for (int64_t j = i; j < my_tiles && j < i + kTmaStages; ++j)
        mbar_wait(&bar[j % kTmaStages], (uint32_t)((j / kTmaStages) & 1));
    }
    __syncthreads();
    return;
  }
#pragma unroll
  for (int c = 0; c < kDotCh; ++c)
    if (c < cn) {
      const double2 r = block_sum2((double)re[c], (double)im[c]);
      if (threadIdx.x == 0) part[(size_t)(l0 + c) * gridDim.x + blockIdx.x] = r;
    }
}

// w -= sum_l c_l V_l, each FP64 coefficient applied as hi + lo floats;
// optionally the block partial of |w|^2.  skip: the device flag of the
// selective reorthogonalisation (no update this step).
__global__ void __launch_bounds__(kBS) k_cf_multiaxpy(int64_t n, const float2* __restrict__ V, int64_t ld, int nv,
                                                      const double2* __restrict__ c, float2* __restrict__ w,
                                                      double* __restrict__ norm_part, const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ float4 sc[128];  // (re_hi, im_hi, re_lo, im_lo)
  for (int l = threadIdx.x; l < nv; l += blockDim.x) {
    float4 t;
    d_to_df(c[l].x, t.x, t.z);
    d_to_df(c[l].y, t.y, t.w);
    sc[l] = t;
  }
  __syncthreads();
  float s = 0.f;
  // two consecutive elements per thread (16-byte loads and stores), the last
  // one of an odd n by thread 0 of block 0
  const int64_t n2 = n >> 1;
  float4* __restrict__ w4 = reinterpret_cast<float4*>(w);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    float4 x = w4[i];
    for (int l = 0; l < nv; ++l) {
      const float4 v = reinterpret_cast<const float4*>(V + (size_t)l * ld)[i];
      const float4 cc = sc[l];
      cf_sub(x.x, x.y, cc, make_float2(v.x, v.y));
      cf_sub(x.z, x.w, cc, make_float2(v.z, v.w));
    }
    w4[i] = x;
    s = __fmaf_rn(x.x, x.x, __fmaf_rn(x.y, x.y, s));
    s = __fmaf_rn(x.z, x.z, __fmaf_rn(x.w, x.w, s));
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    float2 x = w[n - 1];
    for (int l = 0; l < nv; ++l) cf_sub(x.x, x.y, sc[l], V[(size_t)l * ld + n - 1]);
    w[n - 1] = x;
    s = __fmaf_rn(x.x, x.x, __fmaf_rn(x.y, x.y, s));
  }
  if (norm_part) {
    const double2 r = block_sum2((double)s, 0.0);
    if (threadIdx.x == 0) norm_part[blockIdx.x] = r.x;
  }
}

// selective reorthogonalisation: skip = (max_l |c_l| <= eta |w|), with |c| bounded
// by |re| + |im| and |w|^2 from the local step
__global__ void k_sel_flag(const double2* __restrict__ c, int nv, const double* __restrict__ w2, double eta,
                           int* __restrict__ skip) {
  double m = 0.0;
  for (int l = threadIdx.x; l < nv; l += 32) m = fmax(m, fabs(c[l].x) + fabs(c[l].y));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if (threadIdx.x == 0) *skip = m <= eta * sqrt(*w2) ? 1 : 0;
}

// v = w / sqrt(nrm2) in complex64 (1/|w| as hi + lo floats, one rounding of
// the product); xs = sqrt(stab) v, the matvec input
__global__ void k_cf_normalize(int64_t n, const float2* __restrict__ w, const double* __restrict__ nrm2,
                               float2* __restrict__ v, const uint8_t* __restrict__ stab, float2* __restrict__ xs) {
  __shared__ float s_sq[65];
  __shared__ float s_inv[2];
  for (int i = threadIdx.x; i < 65; i += blockDim.x) s_sq[i] = (float)sqrt((double)i);
  if (threadIdx.x == 0) d_to_df(1.0 / sqrt(*nrm2), s_inv[0], s_inv[1]);
  __syncthreads();
  const float ih = s_inv[0], il = s_inv[1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 y = w[i];
    const float rx = __fmaf_rn(y.x, ih, __fmul_rn(y.x, il));
    const float ry = __fmaf_rn(y.y, ih, __fmul_rn(y.y, il));
    if (v) v[i] = make_float2(rx, ry);
    if (xs) {
      const float sq = s_sq[stab[i]];
      xs[i] = make_float2(__fmul_rn(rx, sq), __fmul_rn(ry, sq));
    }
  }
}


// Restart rotation out[c] = sum_l V[l] Z[l][c], Z real (the Ritz vectors of
// the real projected matrix) as double-float pairs, row-major [l][keep],
// accumulated in double-float and rounded once to complex64.
// Block row blockIdx.y takes outputs [c0, c0 + CH): up to kRotCh outputs per
// pass, so the basis is read ceil(keep / kRotCh) times.
// The chunk width CH is a template parameter, chosen per launch as the exact
// chunk size: an unrolled loop guarded by a runtime count would issue its
// masked-off iterations too.
static constexpr int kRotCh = 16;
template <int CH>
__global__ void __launch_bounds__(kBS) k_cf_rotate_re(int64_t n, const float2* __restrict__ V, int64_t ld, int msz,
                                                      const float2* __restrict__ Z, int keep,
                                                      float2* __restrict__ out) {
  __shared__ float2 sZ[121 * CH];
  const int c0 = blockIdx.y * CH;
  const int cn = min(CH, keep - c0);
  for (int idx = threadIdx.x; idx < msz * CH; idx += blockDim.x) {
    const int l = idx / CH, c = idx % CH;
    sZ[idx] = c < cn ? Z[(size_t)l * keep + c0 + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float4 acc[CH];  // (re_hi, im_hi, re_lo, im_lo)
#pragma unroll
    for (int c = 0; c < CH; ++c) acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int l = 0; l < msz; ++l) {
      const float2 v = V[(size_t)l * ld + i];
#pragma unroll
      for (int c = 0; c < CH; ++c) {  // padding columns of the last chunk have z = 0
        const float2 z = sZ[l * CH + c];
        df_mac1(acc[c].x, acc[c].z, v.x, z.x, z.y);
        df_mac1(acc[c].y, acc[c].w, v.y, z.x, z.y);
      }
    }
#pragma unroll
    for (int c = 0; c < CH; ++c)
      if (c < cn) out[(size_t)(c0 + c) * ld + i] = make_float2(__fadd_rn(acc[c].x, acc[c].z),
                                                               __fadd_rn(acc[c].y, acc[c].w));
  }
}

// out[0..keep) = V[0..msz) Z in ceil(keep / kRotCh) chunks of equal width
static void cf_rotate_re(int64_t n, const float2* V, int64_t ld, int msz, const float2* Z, int keep, float2* out,
                         int gblk, cudaStream_t s) {
  const int nch = (keep + kRotCh - 1) / kRotCh, cs = (keep + nch - 1) / nch;
  const dim3 g(gblk, nch);
  switch (cs) {
#define SED_ROT(W) \
  case W:          \
    k_cf_rotate_re<W><<<g, kBS, 0, s>>>(n, V, ld, msz, Z, keep, out); \
    break;
    SED_ROT(1) SED_ROT(2) SED_ROT(3) SED_ROT(4) SED_ROT(5) SED_ROT(6) SED_ROT(7) SED_ROT(8)
    SED_ROT(9) SED_ROT(10) SED_ROT(11) SED_ROT(12) SED_ROT(13) SED_ROT(14) SED_ROT(15) SED_ROT(16)
#undef SED_ROT
    default:
      SED_REQUIRE(false, 5, "internal error: rotation chunk width");
  }
}

// ------------------------------------------------ semi-orthogonal Ritz block
// Rayleigh-Ritz on a block B with Gram matrix G = B^H B (complex, row-major
// re/im pairs): G = L L^H (Cholesky), X = L^-1, and M = B^H H B is replaced
// by X M X^H, the projection onto the orthonormal block B X^H.
void gram_orthonormalise(int n, const std::vector<double>& G, std::vector<double>& M, std::vector<double>& X) {
  using C = std::complex<double>;
  std::vector<C> L((size_t)n * n, C(0.0, 0.0)), Xc((size_t)n * n, C(0.0, 0.0)), Mc((size_t)n * n), T((size_t)n * n);
  for (int i = 0; i < n * n; ++i) Mc[i] = C(M[2 * i], M[2 * i + 1]);
  for (int k = 0; k < n; ++k) {
    double d = G[((size_t)k * n + k) * 2];
    for (int p = 0; p < k; ++p) d -= std::norm(L[(size_t)k * n + p]);
    SED_REQUIRE(d > 0.0, 4, "Ritz block is numerically dependent");
    const double lkk = std::sqrt(d);
    L[(size_t)k * n + k] = lkk;
    for (int i = k + 1; i < n; ++i) {
      C sm(G[((size_t)i * n + k) * 2], G[((size_t)i * n + k) * 2 + 1]);
      for (int p = 0; p < k; ++p) sm -= L[(size_t)i * n + p] * std::conj(L[(size_t)k * n + p]);
      L[(size_t)i * n + k] = sm / lkk;
    }
  }
  for (int i = 0; i < n; ++i) {
    Xc[(size_t)i * n + i] = 1.0 / L[(size_t)i * n + i];
    for (int j = 0; j < i; ++j) {
      C sm(0.0, 0.0);
      for (int k = j; k < i; ++k) sm += L[(size_t)i * n + k] * Xc[(size_t)k * n + j];
      Xc[(size_t)i * n + j] = -sm / L[(size_t)i * n + i];
    }
  }
  for (int p = 0; p < n; ++p)  // T = M X^H
    for (int j = 0; j < n; ++j) {
      C sm(0.0, 0.0);
      for (int q = 0; q < n; ++q) sm += Mc[(size_t)p * n + q] * std::conj(Xc[(size_t)j * n + q]);
      T[(size_t)p * n + j] = sm;
    }
  X.assign((size_t)n * n * 2, 0.0);
  for (int i = 0; i < n; ++i)  // M = X T
    for (int j = 0; j < n; ++j) {
      C sm(0.0, 0.0);
      for (int p = 0; p < n; ++p) sm += Xc[(size_t)i * n + p] * T[(size_t)p * n + j];
      M[((size_t)i * n + j) * 2] = sm.real();
      M[((size_t)i * n + j) * 2 + 1] = sm.imag();
      X[((size_t)i * n + j) * 2] = Xc[(size_t)i * n + j].real();
      X[((size_t)i * n + j) * 2 + 1] = Xc[(size_t)i * n + j].imag();
    }
}

// block coefficients X^H U of the Ritz vectors (U: eigenvectors of X M X^H)
std::vector<double> gram_back(int n, const std::vector<double>& X, const std::vector<double>& U) {
  std::vector<double> R((size_t)n * n * 2, 0.0);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < n; ++c) {
      std::complex<double> sm(0.0, 0.0);
      for (int k = 0; k < n; ++k)
        sm += std::conj(std::complex<double>(X[((size_t)k * n + i) * 2], X[((size_t)k * n + i) * 2 + 1])) *
              std::complex<double>(U[((size_t)k * n + c) * 2], U[((size_t)k * n + c) * 2 + 1]);
      R[((size_t)i * n + c) * 2] = sm.real();
      R[((size_t)i * n + c) * 2 + 1] = sm.imag();
    }
  return R;
}

// ------------------------------------------------------------- host driver
namespace {

struct VecOps {
  int64_t n;
  int nblk, nblk_dot, sms;
  cudaStream_t s;
  DevBuf part, part1, coef, scal, flag, err;  // partial sums, coefficients, scalars, skip flag, wait-timeout flag
  double* host = nullptr;          // pinned scratch
  VecOps(int64_t n_, cudaStream_t s_, int sms_) : n(n_), sms(sms_), s(s_) {
    const int64_t sms = sms_;
    nblk = (int)std::max<int64_t>(1, std::min<int64_t>((n + kBS * 4 - 1) / (kBS * 4), sms * 4));
    // the complex64 dot kernel's grid is one full wave of its resident blocks
    int per_sm = 1;
    SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cf_multidot, kBS, 0));
    nblk_dot = (int)std::max<int64_t>(1, std::min<int64_t>((n + kBS * 4 - 1) / (kBS * 4),
                                                            sms * std::max(per_sm, 1)));
    part.alloc((size_t)std::max(nblk, nblk_dot) * 130 * 16);
    part1.alloc((size_t)nblk * 8);
    coef.alloc(256 * 16);
    scal.alloc(64);
    flag.alloc(16);
    err.alloc(16);
    SED_CUDA(cudaMemsetAsync(err.p, 0, 16, s));
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
  void norm2(const float2* v, int slot) {
    k_cf_norm2_part<<<nblk, kBS, 0, s>>>(n, v, part1.as<double>());
    k_reduce_part1<<<1, kBS, 0, s>>>(part1.as<double>(), nblk, scal.as<double>() + slot);
  }
  // coef[off .. off+nv) (=|+=) V[0..nv)^H w
  void multidot(const double2* V, int64_t ld, int nv, const double2* w, int off, bool acc) {
    k_multidot<<<dim3(nblk, nv), kBS, 0, s>>>(n, V, ld, w, part.as<double2>());
    k_reduce_part2<<<nv, kBS, 0, s>>>(part.as<double2>(), nblk, coef.as<double2>() + off, acc ? 1 : 0);
  }
  void multidot(const float2* V, int64_t ld, int nv, const float2* w, int off, bool acc) {
    const dim3 grid_y(1, (nv + kDotCh - 1) / kDotCh);
    if (n >= kTmaMinN && ld % 64 == 0 && ((uintptr_t)V | (uintptr_t)w) % 16 == 0) {
      // vectors staged through shared memory by the bulk-copy engine
      const int tile = tma_tile(std::min(kDotCh, nv));
      // one block per SM, at most as many as the partial-sum buffer holds
      const int g = (int)std::min<int64_t>({(ld + tile - 1) / tile, (int64_t)sms, (int64_t)std::max(nblk, nblk_dot)});
      {
        // every chunk's footprint is within 128 + kTmaSmemBudget bytes
        static std::mutex mu;
        static SmemOptIn optin;
        std::lock_guard<std::mutex> lock(mu);
        optin.ensure(k_cf_multidot_tma, 128 + kTmaSmemBudget);
      }
      k_cf_multidot_tma<<<dim3(g, grid_y.y), kBS, tma_smem(std::min(kDotCh, nv), tile), s>>>(
          n, V, ld, nv, w, part.as<double2>(), tile, nullptr, err.as<int>());
      k_reduce_part2<<<nv, kBS, 0, s>>>(part.as<double2>(), g, coef.as<double2>() + off, acc ? 1 : 0);
      return;
    }
    k_cf_multidot<<<dim3(nblk_dot, grid_y.y), kBS, 0, s>>>(n, V, ld, nv, w, part.as<double2>());
    k_reduce_part2<<<nv, kBS, 0, s>>>(part.as<double2>(), nblk_dot, coef.as<double2>() + off, acc ? 1 : 0);
  }
  // a bounded wait of the staged dot kernel ran out (its partials are not valid)
  bool timed_out() {
    int e = 0;
    SED_CUDA(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, s));
    SED_CUDA(cudaStreamSynchronize(s));
    return e != 0;
  }
  // w -= V[0..nv) coef[off..], optionally scal[slot] = |w|^2
  // (skip: device flag of the selective reorthogonalisation, complex64 only)
  void multiaxpy(const double2* V, int64_t ld, int nv, double2* w, int off, int norm_slot) {
    k_multiaxpy<<<nblk, kBS, 0, s>>>(n, V, ld, nv, coef.as<double2>() + off, w,
                                     norm_slot >= 0 ? part1.as<double>() : nullptr);
    if (norm_slot >= 0) k_reduce_part1<<<1, kBS, 0, s>>>(part1.as<double>(), nblk, scal.as<double>() + norm_slot);
  }
  void multiaxpy(const float2* V, int64_t ld, int nv, float2* w, int off, int norm_slot, const int* skip = nullptr) {
    k_cf_multiaxpy<<<nblk, kBS, 0, s>>>(n, V, ld, nv, coef.as<double2>() + off, w,
                                        norm_slot >= 0 ? part1.as<double>() : nullptr, skip);
    if (norm_slot >= 0) k_reduce_part1<<<1, kBS, 0, s>>>(part1.as<double>(), nblk, scal.as<double>() + norm_slot);
  }
  void check() { SED_CUDA(cudaGetLastError()); }
};

}  // namespace

SolveResult solve(OpImpl& op, int nev_out, double tol, int maxiter, int krylovdim, uint64_t seed, double* evals_out,
                  double* evecs) {
  auto t0 = std::chrono::steady_clock::now();
  SolveResult res;
  const SectorImpl& S = *op.sec;
  const CatalogImpl& C = *S.cat;
  const int64_t n = C.n_orbits;
  const int64_t D = S.dim;
  SED_REQUIRE(nev_out >= 1, 1, "nev must be positive");
  SED_REQUIRE(maxiter >= 1, 1, "maxiter must be positive");
  if (D == 0) return res;
  nev_out = (int)std::min<int64_t>(nev_out, D);
  SED_REQUIRE(nev_out <= 32, 5, "nev must be at most 32");
  if (D <= kDenseMaxDim) {  // SRE:1004-1017: small sectors are solved densely
    res = solve_dense(op, nev_out, evals_out, evecs);
    res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return res;
  }
  // a solve applies the operator hundreds of times: stream it from the hop
  // table when that fits (sed_optable.cu)
  if (op.tab_mode == 1 && !op.tab_built && !op.tab_refused) op.tab_refused = !op_build_table(op);
  const bool mixed = op.precision == 1;
  // Mixed precision carries two spare Ritz pairs into the FP64 polish, so a
  // level nearly degenerate with the first one not requested is still
  // resolved; convergence is judged on the requested pairs only.
  int nev = mixed ? (int)std::min<int64_t>(nev_out + 2, D) : nev_out;
  std::vector<double> evals_v(nev, 0.0);
  double* evals = evals_v.data();
  if (krylovdim <= 0) krylovdim = 30;
  const int m = (int)std::min<int64_t>(std::max(krylovdim, 2 * nev + 1), std::min<int64_t>(D, 120));
  cudaStream_t s = op.stream;
  const int nslots = std::max(m + 1, 3 * nev + 1);
  const int64_t ld = n;          // FP64 vectors
  const int64_t ldc = cf_ld(n);  // complex64 vectors
  // FP64 precision: basis V, work vector W, restart buffer R.  Mixed: the
  // complex64 basis Vc and restart buffer Rc (they trade places at every
  // restart) and work vector Wc; R is then the FP64 scratch of the start
  // vector, the gather fallback and the Rayleigh-Ritz check.
  DevBuf Vb(mixed ? 0 : (size_t)nslots * ld * 16), Wb(mixed ? 0 : (size_t)ld * 16);
  DevBuf Rb((size_t)(mixed ? 5 * nev : std::max(m, 5 * nev)) * ld * 16);
  DevBuf Vcb(mixed ? (size_t)nslots * ldc * 8 : 0), Rcb(mixed ? (size_t)nslots * ldc * 8 : 0);
  DevBuf Wcb(mixed ? (size_t)ldc * 8 : 0);
  DevBuf xs((size_t)ldc * 16), xs64((size_t)ld * 16), Sd((size_t)130 * 130 * 16);
  double2* V = Vb.as<double2>();
  double2* W = Wb.as<double2>();
  double2* R = Rb.as<double2>();
  float2* Vc = Vcb.as<float2>();
  float2* Rc = Rcb.as<float2>();
  float2* Wc = Wcb.as<float2>();
  const double2* Vout = V;  // where the returned eigenvectors end up (FP64)
  VecOps ops(n, s, op_sm_count(op));
  auto vec = [&](int j) { return V + (size_t)j * ld; };
  auto vecc = [&](int j) { return Vc + (size_t)j * ldc; };
  const int gblk = ops.nblk;
  // v_{j+1} = w / sqrt(scal[slot]) and the next matvec input xs
  auto normalize = [&](int slot, int j1) {
    if (mixed)
      k_cf_normalize<<<gblk, kBS, 0, s>>>(n, Wc, ops.scal.as<double>() + slot, vecc(j1), C.stab.as<uint8_t>(),
                                          xs.as<float2>());
    else
      k_normalize<double2><<<gblk, kBS, 0, s>>>(n, W, ops.scal.as<double>() + slot, vec(j1), C.stab.as<uint8_t>(),
                                                xs.as<double2>());
  };
  // start vector
  if (mixed) {
    k_start<<<gblk, kBS, 0, s>>>(n, S.rowflag.as<uint8_t>(), seed, R);
    k_d_to_cf<<<gblk, kBS, 0, s>>>(n, R, Wc);
    ops.norm2(Wc, 0);
  } else {
    k_start<<<gblk, kBS, 0, s>>>(n, S.rowflag.as<uint8_t>(), seed, W);
    ops.norm2(W, 0);
  }
  normalize(0, 0);
  ops.check();

  std::vector<double> T((size_t)m * m, 0.0), theta, Z;
  int k = 0;
  double beta = 0.0, best_prev[3] = {1e300, 1e300, 1e300};
  double scale = 1.0;
  double tau = 1e-6;  // mixed: relative Ritz-estimate threshold of the complex64 run
  for (;;) {
    int jend = m;
    for (int j = k; j < m; ++j) {
      // local step: CGS against the two newest basis vectors (they carry the
      // large alpha_j and beta_{j-1} components), then one full CGS pass
      // against the whole basis; a second full pass only when the first one
      // removed more than half of the norm (Daniel-Gragg-Kaufman-Stewart).
      const int l0 = j > 0 ? j - 1 : 0;
      if (mixed) {
        if (!op_apply_orbit_cf(op, xs.p, Wc, s)) {  // no hop table: the FP64-output gather
          op_apply_orbit(op, xs.p, (double*)R, s);
          k_d_to_cf<<<gblk, kBS, 0, s>>>(n, R, Wc);
        }
        ops.multidot(vecc(l0), ldc, j + 1 - l0, Wc, 0, false);
        ops.multiaxpy(vecc(l0), ldc, j + 1 - l0, Wc, 0, 5);
        ops.multidot(Vc, ldc, j + 1, Wc, 128, false);
        // the update only when the measured loss of orthogonality exceeds
        // kSelReorth (decided on the device)
        k_sel_flag<<<1, 32, 0, s>>>(ops.coef.as<double2>() + 128, j + 1, ops.scal.as<double>() + 5, kSelReorth,
                                    ops.flag.as<int>());
        ops.multiaxpy(Vc, ldc, j + 1, Wc, 128, 1, ops.flag.as<int>());
      } else {
        op_apply_orbit(op, xs.p, (double*)W, s);
        ops.multidot(vec(l0), ld, j + 1 - l0, W, 0, false);
        ops.multiaxpy(vec(l0), ld, j + 1 - l0, W, 0, 5);
        ops.multidot(V, ld, j + 1, W, 128, false);
        ops.multiaxpy(V, ld, j + 1, W, 128, 1);
      }
      ops.check();
      SED_CUDA(cudaMemcpyAsync(ops.host, ops.coef.as<double2>() + (j - l0), 16, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaMemcpyAsync(ops.host + 2, ops.coef.as<double2>() + 128 + j, 16, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaMemcpyAsync(ops.host + 4, ops.scal.as<double>() + 1, 8, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaMemcpyAsync(ops.host + 5, ops.scal.as<double>() + 5, 8, cudaMemcpyDeviceToHost, s));
      if (mixed) SED_CUDA(cudaMemcpyAsync(ops.host + 6, ops.flag.p, 4, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
      ++res.matvecs;
      int skipped = 0;
      if (mixed) std::memcpy(&skipped, ops.host + 6, 4);
      double alpha = ops.host[0] + (skipped ? 0.0 : ops.host[2]);
      double nrm2 = skipped ? ops.host[5] : ops.host[4];
      if (!skipped && nrm2 < 0.5 * ops.host[5]) {
        if (mixed) {
          ops.multidot(Vc, ldc, j + 1, Wc, 128, false);
          ops.multiaxpy(Vc, ldc, j + 1, Wc, 128, 1);
        } else {
          ops.multidot(V, ld, j + 1, W, 128, false);
          ops.multiaxpy(V, ld, j + 1, W, 128, 1);
        }
        ops.check();
        SED_CUDA(cudaMemcpyAsync(ops.host + 2, ops.coef.as<double2>() + 128 + j, 16, cudaMemcpyDeviceToHost, s));
        SED_CUDA(cudaMemcpyAsync(ops.host + 4, ops.scal.as<double>() + 1, 8, cudaMemcpyDeviceToHost, s));
        SED_CUDA(cudaStreamSynchronize(s));
        alpha += ops.host[2];
        nrm2 = ops.host[4];
      }
      beta = std::sqrt(nrm2);
      T[(size_t)j * m + j] = alpha;
      if (j + 1 < m) T[(size_t)j * m + j + 1] = T[(size_t)(j + 1) * m + j] = beta;
      if (!(beta > 1e-13 * std::max(1.0, std::fabs(alpha)))) {
        jend = j + 1;
        break;
      }
      normalize(1, j + 1);
    }
    const int msz = jend;
    std::vector<double> A((size_t)msz * msz);
    for (int i = 0; i < msz; ++i)
      for (int j = 0; j < msz; ++j) A[(size_t)i * msz + j] = T[(size_t)i * m + j];
    eigh_real_sym(msz, A, theta, Z);
    const bool invariant = msz < m || msz == D;
    scale = 1.0;
    for (int i = 0; i < std::min(nev, msz); ++i) scale = std::max(scale, std::fabs(theta[i]));
    const double tol_w = mixed ? std::max(tol, tau * scale) : tol;
    int nconv = 0;
    double maxr = 0.0;
    for (int i = 0; i < std::min(nev_out, msz); ++i) {
      const double r = invariant ? 0.0 : std::fabs(beta * Z[(size_t)(msz - 1) * msz + i]);
      maxr = std::max(maxr, r);
      if (r <= tol_w) ++nconv;
    }
    // FP32 matvec noise floor: stop when the residual no longer improves
    // (only once the residual is near that floor: Lanczos also plateaus for a
    // few restarts on clustered levels long before it)
    bool stagnated = false;
    if (mixed && res.restarts >= 6 && maxr < 5e-5 * scale && maxr > 0.7 * best_prev[2]) stagnated = true;
    best_prev[2] = best_prev[1];
    best_prev[1] = best_prev[0];
    best_prev[0] = std::min(best_prev[0], maxr);
    const bool done = (nconv >= nev_out) || invariant || stagnated || res.restarts >= maxiter;
    // a mixed-precision candidate keeps the full restart basis, so the
    // iteration can resume if the FP64 check rejects it
    const bool final_rot = done && (!mixed || invariant);
    // thick restart: mixed precision keeps nev + 2 Ritz vectors (its nev
    // already carries two spare pairs), FP64 half of the rest as well.  Fewer
    // kept vectors shorten the rotation and every later dot sweep: the
    // checkerboard 4x6 solve took 398 matvecs instead of 394 and 1.62 s
    // instead of 1.90 s
    const int keep = final_rot ? std::min(nev, msz)
                               : std::min(msz - 1, mixed ? nev + 2 : std::max(nev + (m - nev) / 2, nev + 1));
    if (mixed) {
      std::vector<float> Zf((size_t)msz * keep * 2);  // real Ritz vectors as double-float pairs
      for (int l = 0; l < msz; ++l)
        for (int c = 0; c < keep; ++c) {
          const double z = Z[(size_t)l * msz + c];
          const float h = (float)z;
          Zf[((size_t)l * keep + c) * 2] = h;
          Zf[((size_t)l * keep + c) * 2 + 1] = (float)(z - (double)h);
        }
      SED_CUDA(cudaMemcpyAsync(Sd.p, Zf.data(), Zf.size() * 4, cudaMemcpyHostToDevice, s));
      cf_rotate_re(n, Vc, ldc, msz, Sd.as<float2>(), keep, Rc, gblk, s);
      if (!final_rot)  // the last normalised residual direction (slot m) continues the basis
        SED_CUDA(cudaMemcpyAsync(Rc + (size_t)keep * ldc, vecc(m), (size_t)ldc * 8, cudaMemcpyDeviceToDevice, s));
      std::swap(Vc, Rc);  // the rotated vectors become the basis; no copy back
    } else {
      std::vector<double> Sc((size_t)msz * keep * 2, 0.0);
      for (int l = 0; l < msz; ++l)
        for (int c = 0; c < keep; ++c) Sc[((size_t)l * keep + c) * 2] = Z[(size_t)l * msz + c];
      SED_CUDA(cudaMemcpyAsync(Sd.p, Sc.data(), Sc.size() * 8, cudaMemcpyHostToDevice, s));
      k_rotate<<<dim3(gblk, (keep + 7) / 8), kBS, 0, s>>>(n, V, ld, msz, Sd.as<double2>(), keep, R);
      SED_CUDA(cudaMemcpyAsync(V, R, (size_t)keep * ld * 16, cudaMemcpyDeviceToDevice, s));
      if (!final_rot)  // the last normalised residual direction (slot m) continues the basis
        SED_CUDA(cudaMemcpyAsync(vec(keep), vec(m), (size_t)ld * 16, cudaMemcpyDeviceToDevice, s));
    }
    ops.check();
    if (done && !mixed) {
      res.converged = nconv;
      res.max_residual = maxr;
      res.status = (nconv >= nev_out || invariant || stagnated) ? 0 : 4;
      for (int i = 0; i < keep; ++i) evals[i] = theta[i];
      break;
    }
    if (done) {
      // FP64 check of the complex64 candidate: one Rayleigh-Ritz step with
      // FP64 matvecs over its nev + 2 Ritz vectors B = V[0..nw).  Accepted
      // when every requested pair meets the residual tolerance or the
      // quadratic eigenvalue bound |dE| <= |r|^2 / gap is below
      // kMixedRelTarget |E|, the gap measured to the lower end of the first
      // Lanczos Ritz interval outside the block; otherwise the Lanczos
      // resumes with a tighter threshold, and only a stagnated complex64 run
      // falls back to FP64.
      const int nw = std::min(nev, msz);
      double2* HB = R;
      double2* Yr = R + (size_t)nw * ld;
      double2* HYr = R + (size_t)(2 * nw) * ld;
      double2* B64 = R + (size_t)(3 * nw) * ld;  // FP64 copies of the Ritz vectors
      double2* Wr = R + (size_t)(4 * nw) * ld;   // residual scratch
      k_cf_to_d<<<dim3(gblk, nw), kBS, 0, s>>>(n, Vc, ldc, B64, ld);
      for (int i = 0; i < nw; ++i) {
        op_scale_to_xs_prec(op, (const double*)(B64 + (size_t)i * ld), xs64.p, false, s);
        op_apply_orbit64(op, xs64.p, (double*)(HB + (size_t)i * ld), s);
        ++res.matvecs64;
      }
      std::vector<double> M((size_t)nw * nw * 2), lam, U;
      for (int bcol = 0; bcol < nw; ++bcol) {
        ops.multidot(B64, ld, nw, HB + (size_t)bcol * ld, 0, false);
        ops.check();
        SED_CUDA(cudaMemcpyAsync(ops.host, ops.coef.p, (size_t)nw * 16, cudaMemcpyDeviceToHost, s));
        SED_CUDA(cudaStreamSynchronize(s));
        for (int a2 = 0; a2 < nw; ++a2) {
          M[((size_t)a2 * nw + bcol) * 2] = ops.host[2 * a2];
          M[((size_t)a2 * nw + bcol) * 2 + 1] = ops.host[2 * a2 + 1];
        }
      }
      // the block is only semi-orthogonal (kSelReorth): with its Gram matrix
      // G = B^H B = L L^H, B L^-H is orthonormal and projects H to L^-1 M L^-H
      std::vector<double> Gm((size_t)nw * nw * 2);
      for (int bcol = 0; bcol < nw; ++bcol) {
        ops.multidot(B64, ld, nw, B64 + (size_t)bcol * ld, 0, false);
        ops.check();
        SED_CUDA(cudaMemcpyAsync(ops.host, ops.coef.p, (size_t)nw * 16, cudaMemcpyDeviceToHost, s));
        SED_CUDA(cudaStreamSynchronize(s));
        for (int a2 = 0; a2 < nw; ++a2) {
          Gm[((size_t)a2 * nw + bcol) * 2] = ops.host[2 * a2];
          Gm[((size_t)a2 * nw + bcol) * 2 + 1] = ops.host[2 * a2 + 1];
        }
      }
      std::vector<double> X;
      gram_orthonormalise(nw, Gm, M, X);
      for (int a2 = 0; a2 < nw; ++a2)  // Hermitian part
        for (int b2 = a2; b2 < nw; ++b2) {
          const double r = 0.5 * (M[((size_t)a2 * nw + b2) * 2] + M[((size_t)b2 * nw + a2) * 2]);
          const double im = 0.5 * (M[((size_t)a2 * nw + b2) * 2 + 1] - M[((size_t)b2 * nw + a2) * 2 + 1]);
          M[((size_t)a2 * nw + b2) * 2] = r;
          M[((size_t)a2 * nw + b2) * 2 + 1] = im;
          M[((size_t)b2 * nw + a2) * 2] = r;
          M[((size_t)b2 * nw + a2) * 2 + 1] = -im;
        }
      eigh_complex_herm(nw, M, lam, U);
      U = gram_back(nw, X, U);  // Ritz vectors B X^H U
      SED_CUDA(cudaMemcpyAsync(Sd.p, U.data(), U.size() * 8, cudaMemcpyHostToDevice, s));
      k_rotate<<<dim3(gblk, (nw + 7) / 8), kBS, 0, s>>>(n, B64, ld, nw, Sd.as<double2>(), nw, Yr);
      k_rotate<<<dim3(gblk, (nw + 7) / 8), kBS, 0, s>>>(n, HB, ld, nw, Sd.as<double2>(), nw, HYr);
      for (int i = 0; i < nev_out; ++i) {
        k_residual<<<gblk, kBS, 0, s>>>(n, HYr + (size_t)i * ld, Yr + (size_t)i * ld, lam[i], Wr);
        ops.norm2(Wr, 4);
        SED_CUDA(cudaMemcpyAsync(ops.host + i, ops.scal.as<double>() + 4, 8, cudaMemcpyDeviceToHost, s));
      }
      ops.check();
      SED_CUDA(cudaStreamSynchronize(s));
      // every requested pair must pass mixed_pair_accepted: isolated, and the
      // quadratic bound with the gap to the lower end theta_L - r_L of the
      // first Lanczos Ritz interval above the block (an eigenvalue lies within
      // its Lanczos residual r_L of theta_L).  The bound holds as long as the
      // Krylov space has not missed an eigenvalue between the block and
      // theta_L, which the two spare pairs guard.
      const double rL = (msz > nw && !invariant) ? std::fabs(beta * Z[(size_t)(msz - 1) * msz + nw]) : 0.0;
      const double thL = msz > nw ? theta[nw] - rL : HUGE_VAL;
      bool ok = true;
      double maxr64 = 0.0, maxd = 0.0;
      for (int i = 0; i < nev_out; ++i) {
        maxr64 = std::max(maxr64, std::sqrt(ops.host[i]));
        maxd = std::max(maxd, std::fabs(lam[i] - theta[i]));
        ok = ok && mixed_pair_accepted(lam[i], ops.host[i], thL, tol, scale);
      }
      if (ok) {
        res.converged = nev_out;
        res.max_residual = maxr64;
        res.max_delta = maxd;
        res.status = 0;
        for (int i = 0; i < nw; ++i) evals[i] = lam[i];
        Vout = Yr;
        break;
      }
      if (invariant || stagnated || res.restarts >= maxiter || tau <= 1e-9) {
        // the complex64 run cannot resolve these levels to the target (e.g.
        // a gap below its noise floor): answer with a full FP64 solve instead
        // of returning an unconverged pair
        SED_REQUIRE(!ops.timed_out(), SED_ERR_TIMEOUT, "a bounded wait of the staged dot kernel ran out");
        const int mv32 = res.matvecs, mv64 = res.matvecs64, rs = res.restarts;
        op.precision = 0;
        SolveResult r64;
        try {
          r64 = solve(op, nev_out, tol, maxiter, krylovdim, seed, evals_out, evecs);
        } catch (...) {
          op.precision = 1;
          throw;
        }
        op.precision = 1;
        r64.matvecs64 += r64.matvecs + mv64;
        r64.matvecs = mv32;
        r64.restarts += rs;
        r64.max_delta = maxd;
        r64.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return r64;
      }
      tau *= 0.1;
    }
    std::fill(T.begin(), T.end(), 0.0);
    for (int c = 0; c < keep; ++c) {
      T[(size_t)c * m + c] = theta[c];
      const double b = beta * Z[(size_t)(msz - 1) * msz + c];
      T[(size_t)c * m + keep] = T[(size_t)keep * m + c] = b;
    }
    k = keep;
    ++res.restarts;
  }
  // a staged dot pass whose bounded wait ran out left partial sums that are
  // not valid
  SED_REQUIRE(!ops.timed_out(), SED_ERR_TIMEOUT, "a bounded wait of the staged dot kernel ran out");

  for (int i = 0; i < nev_out; ++i) evals_out[i] = evals[i];
  if (evecs) {
    DevBuf ys((size_t)std::max<int64_t>(D, 1) * 16);
    for (int i = 0; i < nev_out; ++i) {
      compress_vec(S, (const double*)(Vout + (size_t)i * ld), ys.as<double>(), s);
      SED_CUDA(cudaMemcpyAsync(evecs + (size_t)i * D * 2, ys.p, (size_t)D * 16, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
    }
  }
  SED_CUDA(cudaStreamSynchronize(s));
  res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return res;
}

}  // namespace sed
