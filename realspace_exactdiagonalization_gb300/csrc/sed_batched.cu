// sed_batched.cu -- many small sector solves in one persistent launch.
//
// Replaces the reference's sequential loops over sectors and flux twists
// (_ed_scan_sectors! SRE:1199-1256, ed_scan! flux branch SRE:1320-1355 of
// src/symmetry_resolved_ed.jl; many_body_chern_number.jl:193-210), each of
// which ends in diagonalize_block_matrixfree (SRE:998-1030).
//
// One thread block owns one request at a time and runs its whole solve:
//   1. momentum/twist set-up: tchi[k][h] = conj(t_k) chi(h), twisted site
//      phases, and the sector membership of every orbit (the compatibility test
//      of SRE:534-542, evaluated with the same separately rounded products as
//      the single-sector path, so the sector is bit-identical);
//   2. thick-restart Lanczos: the scaled sector vector lives in shared memory
//      (complex64), the Krylov basis in global memory (FP64); every hop of the
//      matvec reads one state word (L2-resident for these sizes) and one
//      shared-memory entry;
//   3. FP64 Rayleigh-Ritz polish over span{Y, H Y - Y Theta} (mixed precision).
// Requests come from a device-side counter (dynamic load balance over uneven
// sector dimensions); a request's result depends only on its own inputs and
// seed, never on the other requests in the launch.  No block waits on another.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/sed_capi.h"
#include "sed_internal.cuh"
#include "sed_rowgather.cuh"

namespace sed {

static constexpr int kBT = 512;      // threads per block
static constexpr int kMaxM = 32;     // Krylov dimension cap
static constexpr int kMaxNev = 8;
static constexpr int kNW = kBT / 32;

struct BatchArgs {
  int64_t n_orb, ld;
  int N, G, n_bil, n_terms, n_den;
  int nev, m, maxiter, n_req;
  double tol, atol;
  const uint64_t* reps;
  const uint8_t* stab;
  const uint64_t* state;
  const uint32_t* rank_tab;
  RankParams rp;
  const uint16_t* site_off;
  const uint32_t* rec;
  const uint8_t* perm_g;
  const uint8_t* inv;
  const double2* diag;
  const double2* chi;    // [n_req][G]
  const double2* phase;  // [n_req][G][N]
  const double2* amp;    // [n_req][n_bil]
  const uint64_t* seeds;
  double2 *V, *R, *W, *X64, *tchi64;
  uint8_t* rowflag;
  double* evals;
  int32_t* status;
  int64_t* dims;
  double* delta;
  int32_t* nmv;
  int64_t* hops;
  int64_t* t_ns;  // [n_req][2]
  unsigned int* queue;
};

struct BatchSmem {
  size_t x, tchi, eta, chi64, T, Z, theta, coef, red, isr, rank, rec, off, inv, perm, misc, total;
};

template <class VT>
static BatchSmem batch_layout(const BatchArgs& a, bool x_in_smem) {
  BatchSmem L{};
  size_t o = 0;
  auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
  L.x = o;
  o = al(o + (x_in_smem ? (size_t)a.n_orb * sizeof(VT) : 0));
  L.tchi = o;
  o = al(o + (size_t)a.n_bil * a.G * sizeof(VT));
  L.eta = o;
  o = al(o + (size_t)a.G * a.N * sizeof(VT));
  L.chi64 = o;
  o = al(o + (size_t)a.G * 16);
  L.T = o;
  o = al(o + kMaxM * kMaxM * 8);
  L.Z = o;
  o = al(o + kMaxM * kMaxM * 8);
  L.theta = o;
  o = al(o + kMaxM * 8);
  L.coef = o;
  o = al(o + 2 * (kMaxM + 8) * 16);
  L.red = o;
  o = al(o + kNW * 16 * 8);
  L.isr = o;
  o = al(o + 65 * 8);
  L.misc = o;
  o = al(o + 64 * 8);
  L.rank = o;
  o = al(o + (size_t)a.rp.total * 4);
  L.rec = o;
  o = al(o + (size_t)a.n_terms * 4);
  L.off = o;
  o = al(o + (size_t)(a.N + 1) * 2);
  L.inv = o;
  o = al(o + 64);
  L.perm = o;
  o = al(o + (size_t)a.G * 64);
  L.total = o;
  return L;
}

// ------------------------------------------------------------ block helpers
__device__ __forceinline__ double warp_allsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// Sum NV per-thread values over the block (fixed order); result in out[0..NV).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* red, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = warp_allsum(v[i]);
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) red[wid * 16 + i] = v[i];
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
    for (int w = 0; w < kNW; ++w) s += red[w * 16 + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

__device__ __forceinline__ double block_sum1(double v, double* red, double* out) {
  double a[1] = {v};
  block_sum<1>(a, red, out);
  return out[0];
}

// Warp-parallel cyclic Jacobi for a real symmetric n x n matrix (row stride
// ld) in shared memory; eigenvalues ascending in w, eigenvectors in Z columns.
__device__ void warp_jacobi(int n, double* A, double* Z, double* w) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < n * kMaxM; i += 32) Z[i] = 0.0;
  __syncwarp();
  for (int i = lane; i < n; i += 32) Z[i * kMaxM + i] = 1.0;
  __syncwarp();
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int e = lane; e < n * n; e += 32) {
      const int i = e / n, j = e % n;
      const double v = A[i * kMaxM + j] * A[i * kMaxM + j];
      tot += v;
      if (i != j) off += v;
    }
    off = warp_allsum(off);
    tot = warp_allsum(tot);
    if (off <= 1e-32 * fmax(tot, 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * kMaxM + q];
        if (apq == 0.0) continue;
        const double app = A[p * kMaxM + p], aqq = A[q * kMaxM + q];
        const double th = (aqq - app) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        __syncwarp();
        if (lane < n) {
          const double akp = A[lane * kMaxM + p], akq = A[lane * kMaxM + q];
          A[lane * kMaxM + p] = c * akp - s * akq;
          A[lane * kMaxM + q] = s * akp + c * akq;
        }
        __syncwarp();
        if (lane < n) {
          const double apk = A[p * kMaxM + lane], aqk = A[q * kMaxM + lane];
          A[p * kMaxM + lane] = c * apk - s * aqk;
          A[q * kMaxM + lane] = s * apk + c * aqk;
          const double zkp = Z[lane * kMaxM + p], zkq = Z[lane * kMaxM + q];
          Z[lane * kMaxM + p] = c * zkp - s * zkq;
          Z[lane * kMaxM + q] = s * zkp + c * zkq;
        }
        __syncwarp();
      }
  }
  __syncwarp();
  if (lane == 0) {
    for (int i = 0; i < n; ++i) w[i] = A[i * kMaxM + i];
    for (int i = 0; i < n; ++i) {  // selection sort with column swaps
      int b = i;
      for (int j = i + 1; j < n; ++j)
        if (w[j] < w[b]) b = j;
      if (b != i) {
        const double t = w[i];
        w[i] = w[b];
        w[b] = t;
        for (int r = 0; r < n; ++r) {
          const double z = Z[r * kMaxM + i];
          Z[r * kMaxM + i] = Z[r * kMaxM + b];
          Z[r * kMaxM + b] = z;
        }
      }
    }
  }
  __syncwarp();
}

// Complex Hermitian Jacobi (single thread; n <= 2 * kMaxNev).
__device__ void thread_jacobi_herm(int n, double2* A, double* w) {
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double v = A[i * 16 + j].x * A[i * 16 + j].x + A[i * 16 + j].y * A[i * 16 + j].y;
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-32 * fmax(tot, 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double ar = A[p * 16 + q].x, ai = A[p * 16 + q].y;
        const double r = hypot(ar, ai);
        if (r == 0.0) continue;
        const double er = ar / r, ei = ai / r;
        const double app = A[p * 16 + p].x, aqq = A[q * 16 + q].x;
        const double th = (aqq - app) / (2.0 * r);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double2 xp = A[k * 16 + p], xq0 = A[k * 16 + q];
          const double2 xq = make_double2(xq0.x * er + xq0.y * ei, xq0.y * er - xq0.x * ei);
          A[k * 16 + p] = make_double2(c * xp.x - s * xq.x, c * xp.y - s * xq.y);
          A[k * 16 + q] = make_double2(s * xp.x + c * xq.x, s * xp.y + c * xq.y);
        }
        for (int k = 0; k < n; ++k) {
          const double2 xp = A[p * 16 + k], xq0 = A[q * 16 + k];
          const double2 xq = make_double2(xq0.x * er - xq0.y * ei, xq0.y * er + xq0.x * ei);
          A[p * 16 + k] = make_double2(c * xp.x - s * xq.x, c * xp.y - s * xq.y);
          A[q * 16 + k] = make_double2(s * xp.x + c * xq.x, s * xp.y + c * xq.y);
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = A[i * 16 + i].x;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j)
      if (w[j] < w[i]) {
        const double t = w[i];
        w[i] = w[j];
        w[j] = t;
      }
}

__device__ __forceinline__ int64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return (int64_t)t;
}

__device__ __forceinline__ uint64_t bsplitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// ----------------------------------------------------------- block matvec
// w = H x (orbit-indexed), returns this thread's partial |w|^2
__device__ __forceinline__ int64_t count_row_hops(uint64_t m, const uint16_t* s_off, const uint32_t* s_rec) {
  int64_t c = 0;
  uint64_t occ = m;
  while (occ) {
    const int i = __ffsll((long long)occ) - 1;
    occ &= occ - 1;
    for (int t = s_off[i]; t < s_off[i + 1]; ++t) c += !((m >> (s_rec[t] & 0xFF)) & 1ULL);
  }
  return c;
}

template <class P, bool FERMI, bool PHASES>
__device__ __forceinline__ double block_matvec(const BatchArgs& a, const typename P::V* x,
                                               const typename P::V* tchi, const typename P::V* eta,
                                               const double* s_isr, const uint32_t* s_rank, const uint32_t* s_rec,
                                               const uint16_t* s_off, const uint8_t* s_inv,
                                               const uint8_t* __restrict__ rowflag, double2* __restrict__ w) {
  using V = typename P::V;
  using S = typename P::S;
  double nrm = 0.0;
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    if (!rowflag[o]) {
      w[o] = make_double2(0.0, 0.0);
      continue;
    }
    const double2 dg = a.diag[o];
    const V xo = x[o];
    S ar = (S)dg.x * xo.x - (S)dg.y * xo.y;
    S ai = (S)dg.x * xo.y + (S)dg.y * xo.x;
    row_gather<P, FERMI, PHASES, true>(a.reps[o], x, tchi, nullptr, a.G, eta, a.N, s_rank, a.rp, s_rec, s_off, s_inv,
                                       a.state, ar, ai);
    const double is = s_isr[a.stab[o]];
    const double2 y = make_double2((double)ar * is, (double)ai * is);
    w[o] = y;
    nrm += y.x * y.x + y.y * y.y;
  }
  return nrm;
}

// coef[l0..l0+nv) = V[0..nv)^H w, in chunks of 8 vectors
__device__ void block_dots(const BatchArgs& a, const double2* V, int nv, const double2* w, double* red,
                           double2* coef) {
  for (int l0 = 0; l0 < nv; l0 += 8) {
    double acc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = 0.0;
    const int cn = min(8, nv - l0);
    for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
      const double2 x = w[o];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) {
          const double2 v = V[(size_t)(l0 + c) * a.ld + o];
          acc[2 * c] += v.x * x.x + v.y * x.y;
          acc[2 * c + 1] += v.x * x.y - v.y * x.x;
        }
    }
    block_sum<16>(acc, red, reinterpret_cast<double*>(coef + l0));
  }
}

// w -= V[0..nv) coef; returns this thread's partial |w|^2
__device__ __forceinline__ double block_axpy(const BatchArgs& a, const double2* V, int nv, const double2* coef,
                                             double2* w) {
  double nrm = 0.0;
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    double2 x = w[o];
    for (int l = 0; l < nv; ++l) {
      const double2 v = V[(size_t)l * a.ld + o];
      const double2 c = coef[l];
      x.x -= c.x * v.x - c.y * v.y;
      x.y -= c.x * v.y + c.y * v.x;
    }
    w[o] = x;
    nrm += x.x * x.x + x.y * x.y;
  }
  return nrm;
}

// out[c] = sum_l V[l] S[l][c] for c < keep (S real, row stride kMaxM)
__device__ void block_rotate(const BatchArgs& a, const double2* V, int msz, const double* S, int keep, double2* out) {
  for (int c0 = 0; c0 < keep; c0 += 8) {
    const int cn = min(8, keep - c0);
    for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
      double ar[8], ai[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) ar[c] = ai[c] = 0.0;
      for (int l = 0; l < msz; ++l) {
        const double2 v = V[(size_t)l * a.ld + o];
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (c < cn) {
            const double s = S[l * kMaxM + c0 + c];
            ar[c] += v.x * s;
            ai[c] += v.y * s;
          }
      }
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) out[(size_t)(c0 + c) * a.ld + o] = make_double2(ar[c], ai[c]);
    }
  }
}

// v = w * inv and the scaled matvec input x = sqrt(stab) v
template <class VT>
__device__ __forceinline__ void block_normalize(const BatchArgs& a, const double2* w, double inv, double2* v, VT* x) {
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    const double2 y = make_double2(w[o].x * inv, w[o].y * inv);
    v[o] = y;
    if (x) {
      const double sq = sqrt((double)a.stab[o]);
      x[o].x = y.x * sq;
      x[o].y = y.y * sq;
    }
  }
}

// ---------------------------------------------------------------- the kernel
template <class P, bool FERMI, bool PHASES, bool X_SMEM>
__global__ void __launch_bounds__(kBT, 1) k_batch(BatchArgs a, BatchSmem L) {
  using V = typename P::V;
  extern __shared__ __align__(16) unsigned char smem[];
  V* s_x = reinterpret_cast<V*>(smem + L.x);
  V* s_tchi = reinterpret_cast<V*>(smem + L.tchi);
  V* s_eta = reinterpret_cast<V*>(smem + L.eta);
  double2* s_chi = reinterpret_cast<double2*>(smem + L.chi64);
  double* s_T = reinterpret_cast<double*>(smem + L.T);
  double* s_Z = reinterpret_cast<double*>(smem + L.Z);
  double* s_theta = reinterpret_cast<double*>(smem + L.theta);
  double2* s_coef = reinterpret_cast<double2*>(smem + L.coef);
  double* s_red = reinterpret_cast<double*>(smem + L.red);
  double* s_isr = reinterpret_cast<double*>(smem + L.isr);
  double* s_misc = reinterpret_cast<double*>(smem + L.misc);
  uint32_t* s_rank = reinterpret_cast<uint32_t*>(smem + L.rank);
  uint32_t* s_rec = reinterpret_cast<uint32_t*>(smem + L.rec);
  uint16_t* s_off = reinterpret_cast<uint16_t*>(smem + L.off);
  uint8_t* s_inv = reinterpret_cast<uint8_t*>(smem + L.inv);
  uint8_t* s_perm = reinterpret_cast<uint8_t*>(smem + L.perm);
  int* s_int = reinterpret_cast<int*>(s_misc + 48);

  for (int i = threadIdx.x; i < a.rp.total; i += blockDim.x) s_rank[i] = a.rank_tab[i];
  for (int i = threadIdx.x; i < a.n_terms; i += blockDim.x) s_rec[i] = a.rec[i];
  for (int i = threadIdx.x; i <= a.N; i += blockDim.x) s_off[i] = a.site_off[i];
  for (int i = threadIdx.x; i < a.G; i += blockDim.x) s_inv[i] = a.inv[i];
  for (int i = threadIdx.x; i < a.G * 64; i += blockDim.x) s_perm[i] = a.perm_g[i];
  for (int i = threadIdx.x; i < 65; i += blockDim.x) s_isr[i] = i ? 1.0 / sqrt((double)i) : 0.0;

  const size_t slots = (size_t)a.m + 1;
  const size_t rslots = (size_t)max(a.m, 3 * a.nev);
  double2* Vb = a.V + (size_t)blockIdx.x * slots * a.ld;
  double2* Rb = a.R + (size_t)blockIdx.x * rslots * a.ld;
  double2* W = a.W + (size_t)blockIdx.x * a.ld;
  double2* X64 = a.X64 + (size_t)blockIdx.x * a.ld;
  double2* tchi64 = a.tchi64 + (size_t)blockIdx.x * a.n_bil * a.G;
  uint8_t* rowflag = a.rowflag + (size_t)blockIdx.x * a.ld;
  V* x = X_SMEM ? s_x : reinterpret_cast<V*>(X64);

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_int[0] = (int)atomicAdd(a.queue, 1u);
    __syncthreads();
    const int b = s_int[0];
    if (b >= a.n_req) break;
    if (threadIdx.x == 0) a.t_ns[2 * (size_t)b] = global_ns();
    const double2* chi = a.chi + (size_t)b * a.G;
    const double2* phase = a.phase + (size_t)b * a.G * a.N;
    const double2* amp = a.amp + (size_t)b * a.n_bil;
    // ---- set-up: tables for this momentum / twist
    for (int i = threadIdx.x; i < a.G; i += blockDim.x) s_chi[i] = chi[i];
    for (int i = threadIdx.x; i < a.n_bil * a.G; i += blockDim.x) {
      const int k = i / a.G, h = i % a.G;
      const double2 t = amp[k], c = chi[h];
      const double2 v = make_double2(t.x * c.x + t.y * c.y, t.x * c.y - t.y * c.x);  // conj(t) chi
      tchi64[i] = v;
      s_tchi[i].x = v.x;
      s_tchi[i].y = v.y;
    }
    for (int i = threadIdx.x; i < a.G * a.N; i += blockDim.x) {
      s_eta[i].x = phase[i].x;
      s_eta[i].y = phase[i].y;
    }
    __syncthreads();
    // ---- sector membership (SRE:534-542) and the hop count of one matvec
    double cnt = 0.0, hcnt = 0.0;
    for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
      const uint64_t m = a.reps[o];
      int ok = 1;
      for (int g = 0; g < a.G; ++g) {
        double2 al;
        if (dev::apply_full(m, s_perm + g * 64, phase + (size_t)g * a.N, FERMI ? 1 : 0, &al) == m) {
          const double2 xg = s_chi[g];
          if (!((xg.x == al.x && xg.y == al.y) || hypot(xg.x - al.x, xg.y - al.y) <= a.atol)) ok = 0;
        }
      }
      rowflag[o] = (uint8_t)ok;
      cnt += ok;
      if (ok) hcnt += (double)count_row_hops(m, s_off, s_rec);
    }
    double sums[2] = {cnt, hcnt};
    block_sum<2>(sums, s_red, s_misc);
    const int64_t dim = (int64_t)s_misc[0];
    if (threadIdx.x == 0) a.hops[b] = (int64_t)s_misc[1];
    const int nev = (int)min((int64_t)a.nev, dim);
    const int m = (int)min((int64_t)a.m, dim);
    if (threadIdx.x == 0) a.dims[b] = dim;
    if (dim == 0) {
      if (threadIdx.x == 0) {
        a.status[b] = 0;
        a.nmv[b] = 0;
        a.delta[b] = 0.0;
        for (int i = 0; i < a.nev; ++i) a.evals[(size_t)b * a.nev + i] = nan("");
        a.t_ns[2 * (size_t)b + 1] = global_ns();
      }
      continue;
    }
    // ---- start vector (same generator as the single-sector path)
    double nrm = 0.0;
    const uint64_t seed = a.seeds[b];
    for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
      double2 v = make_double2(0.0, 0.0);
      if (rowflag[o]) {
        const uint64_t r1 = bsplitmix(seed ^ bsplitmix((uint64_t)o));
        const uint64_t r2 = bsplitmix(r1);
        const double u1 = ((r1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        const double u2 = ((r2 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        const double rr = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        v = make_double2(rr * cs, rr * sn);
      }
      W[o] = v;
      nrm += v.x * v.x + v.y * v.y;
    }
    nrm = block_sum1(nrm, s_red, s_misc);
    block_normalize<V>(a, W, 1.0 / sqrt(nrm), Vb, x);
    for (int i = threadIdx.x; i < kMaxM * kMaxM; i += blockDim.x) s_T[i] = 0.0;
    __syncthreads();

    int k = 0, restarts = 0, nmv = 0, status = 0;
    double beta = 0.0, prev_res = 1e300, best_prev = 1e300;
    for (;;) {
      int jend = m;
      for (int j = k; j < m; ++j) {
        double2* vj = Vb + (size_t)j * a.ld;
        double n0 = block_matvec<P, FERMI, PHASES>(a, x, s_tchi, s_eta, s_isr, s_rank, s_rec, s_off, s_inv, rowflag, W);
        __syncthreads();
        ++nmv;
        n0 = block_sum1(n0, s_red, s_misc);
        // full reorthogonalisation: CGS, second pass only when the first
        // removed more than half of the norm (Daniel-Gragg-Kaufman-Stewart)
        block_dots(a, Vb, j + 1, W, s_red, s_coef);
        double n1 = block_axpy(a, Vb, j + 1, s_coef, W);
        __syncthreads();
        n1 = block_sum1(n1, s_red, s_misc + 1);
        double alpha = s_coef[j].x;
        double nf = n1;
        if (n1 < 0.5 * n0) {
          block_dots(a, Vb, j + 1, W, s_red, s_coef + kMaxM + 8);
          double n2 = block_axpy(a, Vb, j + 1, s_coef + kMaxM + 8, W);
          __syncthreads();
          nf = block_sum1(n2, s_red, s_misc + 2);
          alpha += s_coef[kMaxM + 8 + j].x;
        }
        beta = sqrt(nf);
        if (threadIdx.x == 0) {
          s_T[j * kMaxM + j] = alpha;
          if (j + 1 < m) s_T[j * kMaxM + j + 1] = s_T[(j + 1) * kMaxM + j] = beta;
        }
        if (!(beta > 1e-13 * fmax(1.0, fabs(alpha)))) {
          jend = j + 1;
          break;
        }
        block_normalize<V>(a, W, 1.0 / beta, vj + a.ld, x);
        __syncthreads();
        (void)vj;
      }
      __syncthreads();
      const int msz = jend;
      // ---- Ritz values of the projected matrix (warp 0)
      if (threadIdx.x < 32) {
        double* A = s_Z + 0;  // scratch copy: Jacobi destroys its input
        (void)A;
      }
      if (threadIdx.x < 32) {
        // copy T into coef area as scratch? use s_T directly on a copy in s_red is too small;
        // Jacobi works on a copy placed in the second half of s_Z's rows.
      }
      __syncthreads();
      // copy T -> Zin (s_Z reused as input then overwritten), eigenvectors go to s_T
      for (int i = threadIdx.x; i < kMaxM * kMaxM; i += blockDim.x) s_Z[i] = s_T[i];
      __syncthreads();
      if (threadIdx.x < 32) warp_jacobi(msz, s_Z, s_T, s_theta);
      __syncthreads();
      // now s_T holds eigenvectors (columns), s_Z the diagonalised matrix
      const bool invariant = msz < m || (int64_t)msz == dim;
      double scale = 1.0;
      for (int i = 0; i < min(nev, msz); ++i) scale = fmax(scale, fabs(s_theta[i]));
      const bool mixed = sizeof(typename P::S) == 4;
      const double tol_w = mixed ? fmax(a.tol, 2e-6 * scale) : a.tol;
      int nconv = 0;
      double maxr = 0.0;
      for (int i = 0; i < min(nev, msz); ++i) {
        const double r = invariant ? 0.0 : fabs(beta * s_T[(msz - 1) * kMaxM + i]);
        maxr = fmax(maxr, r);
        if (r <= tol_w) ++nconv;
      }
      bool stagnated = mixed && restarts >= 6 && maxr < 1e-3 * scale && maxr > 0.7 * best_prev;
      best_prev = prev_res;
      prev_res = fmin(prev_res, maxr);
      const bool done = nconv >= nev || invariant || stagnated || restarts >= a.maxiter;
      const int keep = done ? min(nev, msz) : min(msz - 1, max(nev + (m - nev) / 2, nev + 1));
      block_rotate(a, Vb, msz, s_T, keep, Rb);
      __syncthreads();
      for (int c = 0; c < keep; ++c)
        for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x)
          Vb[(size_t)c * a.ld + o] = Rb[(size_t)c * a.ld + o];
      if (done) {
        status = (nconv >= nev || invariant || stagnated) ? 0 : SED_ERR_NOT_CONVERGED;
        __syncthreads();
        break;
      }
      for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x)
        Vb[(size_t)keep * a.ld + o] = Vb[(size_t)m * a.ld + o];
      __syncthreads();
      // arrowhead restart matrix
      const double bet = beta;
      __syncthreads();
      if (threadIdx.x == 0) {
        double arrow[kMaxM];
        for (int c = 0; c < keep; ++c) arrow[c] = bet * s_T[(msz - 1) * kMaxM + c];
        for (int i = 0; i < kMaxM * kMaxM; ++i) s_T[i] = 0.0;
        for (int c = 0; c < keep; ++c) {
          s_T[c * kMaxM + c] = s_theta[c];
          s_T[c * kMaxM + keep] = s_T[keep * kMaxM + c] = arrow[c];
        }
      }
      __syncthreads();
      k = keep;
      ++restarts;
    }
    // ---- results (and the FP64 polish in mixed precision)
    double dmax = 0.0;
    if (sizeof(typename P::S) == 4 && status == 0) {
      // H Y in FP64 (x = X64, tables in global FP64)
      for (int i = 0; i < nev; ++i) {
        block_normalize<double2>(a, Vb + (size_t)i * a.ld, 1.0, Rb + (size_t)(2 * kMaxNev) * 0 + (size_t)i * a.ld,
                                 X64);
        __syncthreads();
        block_matvec<P64, FERMI, PHASES>(a, X64, tchi64, phase, s_isr, s_rank, s_rec, s_off, s_inv, rowflag,
                                         Rb + (size_t)i * a.ld);
        __syncthreads();
      }
      // Q = orthonormal residual directions into V[nev + q]
      int q = 0;
      for (int i = 0; i < nev; ++i) {
        double2* Wq = W;
        double r0 = 0.0;
        for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
          const double2 hy = Rb[(size_t)i * a.ld + o], y = Vb[(size_t)i * a.ld + o];
          const double2 r = make_double2(hy.x - s_theta[i] * y.x, hy.y - s_theta[i] * y.y);
          Wq[o] = r;
          r0 += r.x * r.x + r.y * r.y;
        }
        __syncthreads();
        r0 = block_sum1(r0, s_red, s_misc);
        block_dots(a, Vb, nev + q, Wq, s_red, s_coef);
        block_axpy(a, Vb, nev + q, s_coef, Wq);
        __syncthreads();
        block_dots(a, Vb, nev + q, Wq, s_red, s_coef);
        double r1 = block_axpy(a, Vb, nev + q, s_coef, Wq);
        __syncthreads();
        r1 = block_sum1(r1, s_red, s_misc);
        // nothing left to add when the residual is at rounding level or lies in span(Y, Q)
        if (!(r1 > 1e-28) || !(r1 > 1e-6 * r0)) continue;
        block_normalize<double2>(a, Wq, 1.0 / sqrt(r1), Vb + (size_t)(nev + q) * a.ld, X64);
        __syncthreads();
        block_matvec<P64, FERMI, PHASES>(a, X64, tchi64, phase, s_isr, s_rank, s_rec, s_off, s_inv, rowflag,
                                         Rb + (size_t)(nev + q) * a.ld);
        __syncthreads();
        ++q;
      }
      const int nb = nev + q;
      double2* M = reinterpret_cast<double2*>(s_Z);  // 16 x 16 complex fits in kMaxM^2 doubles
      for (int bcol = 0; bcol < nb; ++bcol) {
        block_dots(a, Vb, nb, Rb + (size_t)bcol * a.ld, s_red, s_coef);
        if (threadIdx.x < nb) M[threadIdx.x * 16 + bcol] = s_coef[threadIdx.x];
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        for (int i = 0; i < nb; ++i)
          for (int j = i; j < nb; ++j) {
            const double re = 0.5 * (M[i * 16 + j].x + M[j * 16 + i].x);
            const double im = 0.5 * (M[i * 16 + j].y - M[j * 16 + i].y);
            M[i * 16 + j] = make_double2(re, im);
            M[j * 16 + i] = make_double2(re, -im);
          }
        double lam[16];
        thread_jacobi_herm(nb, M, lam);
        for (int i = 0; i < nev; ++i) {
          dmax = fmax(dmax, fabs(lam[i] - s_theta[i]));
          s_theta[i] = lam[i];
        }
        s_misc[3] = dmax;
      }
      __syncthreads();
      dmax = s_misc[3];
    }
    if (threadIdx.x == 0) {
      for (int i = 0; i < a.nev; ++i) a.evals[(size_t)b * a.nev + i] = i < nev ? s_theta[i] : nan("");
      a.status[b] = status;
      a.nmv[b] = nmv;
      a.delta[b] = dmax;
      a.t_ns[2 * (size_t)b + 1] = global_ns();
    }
  }
}

// ------------------------------------------------------------------ host side
struct BatchImpl {
  std::shared_ptr<CatalogImpl> cat;
  int precision = 1, nev = 4, m = 30, max_req = 0, n_bil = 0, n_den = 0, n_cta = 1;
  std::vector<int32_t> bil_ij;
  TermTables tt;
  DevBuf site_off, rec, diag, V, R, W, X64, tchi64, rowflag;
  DevBuf in_chi, in_phase, in_amp, in_seed, o_evals, o_status, o_dims, o_delta, o_nmv, o_hops, o_tns, queue;
  int last_n = 0;
  size_t smem = 0;
  int64_t ld = 0;
  size_t footprint = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool fermi = false;
  ~BatchImpl() {
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
};

template <class P, bool F, bool PH, bool XS>
static void batch_prepare(BatchImpl& B, const BatchArgs& a, BatchSmem& L, int& ncta) {
  auto kern = k_batch<P, F, PH, XS>;
  L = batch_layout<typename P::V>(a, XS);
  SED_REQUIRE(L.total <= 220 * 1024, 5, "batched solve tables exceed the shared-memory budget (sector too large)");
  SED_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
  int per_sm = 0;
  SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBT, L.total));
  SED_REQUIRE(per_sm >= 1, 5, "batched kernel cannot be resident with this shared-memory footprint");
  ncta = per_sm * device_sm_count();
}

template <class P, bool F, bool PH, bool XS>
static void batch_launch(const BatchArgs& a, const BatchSmem& L, int ncta, cudaStream_t s) {
  k_batch<P, F, PH, XS><<<ncta, kBT, L.total, s>>>(a, L);
  SED_CUDA(cudaGetLastError());
}

static BatchArgs base_args(BatchImpl& B) {
  const CatalogImpl& C = *B.cat;
  const GroupImpl& G = *C.group;
  BatchArgs a{};
  a.n_orb = C.n_orbits;
  a.ld = B.ld;
  a.N = G.n_site;
  a.G = G.n_ops;
  a.n_bil = B.n_bil;
  a.n_terms = B.tt.n_terms;
  a.nev = B.nev;
  a.m = B.m;
  a.reps = C.reps.as<uint64_t>();
  a.stab = C.stab.as<uint8_t>();
  a.state = C.state.as<uint64_t>();
  a.rank_tab = C.rank.dev.as<uint32_t>();
  a.rp = C.rank.rp;
  a.site_off = B.site_off.as<uint16_t>();
  a.rec = B.rec.as<uint32_t>();
  a.perm_g = C.perm_u8.as<uint8_t>();
  a.inv = C.inv_u8.as<uint8_t>();
  a.diag = B.diag.as<double2>();
  a.atol = 1e-12;
  return a;
}

static void dispatch_prepare(BatchImpl& B, const BatchArgs& a, BatchSmem& L, int& ncta, bool phases) {
  const bool mixed = B.precision == 1;
  // Each (precision, statistics) pair is compiled with the twisted-phase
  // product; untwisted requests multiply by exactly 1.
  if (mixed) {
    if (B.fermi) batch_prepare<P32, true, true, true>(B, a, L, ncta);
    else batch_prepare<P32, false, true, true>(B, a, L, ncta);
  } else {
    if (B.fermi) batch_prepare<P64, true, true, false>(B, a, L, ncta);
    else batch_prepare<P64, false, true, false>(B, a, L, ncta);
  }
  (void)phases;
}

static void dispatch_launch(BatchImpl& B, const BatchArgs& a, const BatchSmem& L, int ncta, cudaStream_t s) {
  if (B.precision == 1) {
    if (B.fermi) batch_launch<P32, true, true, true>(a, L, ncta, s);
    else batch_launch<P32, false, true, true>(a, L, ncta, s);
  } else {
    if (B.fermi) batch_launch<P64, true, true, false>(a, L, ncta, s);
    else batch_launch<P64, false, true, false>(a, L, ncta, s);
  }
}

std::shared_ptr<BatchImpl> make_batch(std::shared_ptr<CatalogImpl> cp, int n_bil, const int32_t* bil_ij, int n_den,
                                      const int32_t* den_ij, const double* den_v, int precision, int nev,
                                      int krylovdim, int max_req) {
  const CatalogImpl& C = *cp;
  const GroupImpl& G = *C.group;
  SED_REQUIRE(precision == 0 || precision == 1, 1, "precision must be SED_PREC_FP64 or SED_PREC_MIXED");
  SED_REQUIRE(nev >= 1 && nev <= kMaxNev, 5, "batched solves support 1 <= nev <= 8");
  SED_REQUIRE(max_req >= 1, 1, "max_requests must be positive");
  SED_REQUIRE(n_bil >= 0 && n_bil < 65535, 5, "at most 65534 bilinear terms");
  SED_REQUIRE(n_bil == 0 || bil_ij, 1, "bilinear index array must not be NULL");
  SED_REQUIRE(n_den == 0 || (den_ij && den_v), 1, "density arrays must not be NULL");
  if (krylovdim <= 0) krylovdim = 24;
  auto B = std::make_shared<BatchImpl>();
  B->cat = cp;
  B->precision = precision;
  B->nev = nev;
  B->m = std::min(std::max(krylovdim, 2 * nev + 1), kMaxM);
  B->max_req = max_req;
  B->n_bil = n_bil;
  B->n_den = n_den;
  B->fermi = G.stats == 1;
  B->bil_ij.assign(bil_ij, bil_ij + 2 * n_bil);
  // hop records: to-site | term index << 8, grouped by from-site
  std::vector<std::vector<std::pair<int, int>>> by_site(G.n_site);
  for (int k = 0; k < n_bil; ++k) {
    const int i = bil_ij[2 * k], j = bil_ij[2 * k + 1];
    SED_REQUIRE(i >= 0 && i < G.n_site && j >= 0 && j < G.n_site, 1, "bilinear term site index out of range");
    SED_REQUIRE(i != j, 1, "a bilinear term (i, i, t) changes the particle number; write it as a density term");
    by_site[i].push_back({j, k});
  }
  B->tt.site_off.assign(G.n_site + 1, 0);
  for (int i = 0; i < G.n_site; ++i) {
    B->tt.site_off[i] = (uint16_t)B->tt.rec.size();
    for (auto& p : by_site[i]) B->tt.rec.push_back((uint32_t)p.first | ((uint32_t)p.second << 8));
  }
  B->tt.site_off[G.n_site] = (uint16_t)B->tt.rec.size();
  B->tt.n_terms = (int)B->tt.rec.size();
  B->tt.n_site = G.n_site;
  SED_CUDA(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
  B->own_stream = true;
  cudaStream_t s = B->stream;
  upload(B->site_off, B->tt.site_off, s);
  upload(B->rec, B->tt.rec, s);
  std::vector<int32_t> dij(den_ij, den_ij + 2 * n_den);
  std::vector<double> dv(den_v, den_v + 2 * n_den);
  for (int k = 0; k < n_den; ++k)
    SED_REQUIRE(dij[2 * k] >= 0 && dij[2 * k] < G.n_site && dij[2 * k + 1] >= 0 && dij[2 * k + 1] < G.n_site, 1,
                "density term site index out of range");
  DevBuf ddij, ddv;
  upload(ddij, dij, s);
  upload(ddv, dv, s);
  const int64_t n = C.n_orbits;
  B->ld = ((n + 31) / 32) * 32;
  B->diag.alloc((size_t)std::max<int64_t>(n, 1) * 16);
  compute_diag(n, C.reps.as<uint64_t>(), nullptr, n_den, ddij.as<int32_t>(), ddv.as<double2>(), B->diag.as<double2>(),
               s);
  BatchArgs a = base_args(*B);
  BatchSmem L;
  int ncta = 1;
  dispatch_prepare(*B, a, L, ncta, true);
  B->smem = L.total;
  // per-block workspace, bounded to 16 GB
  const size_t per_cta = ((size_t)(B->m + 1) + (size_t)std::max(B->m, 3 * nev) + 2) * B->ld * 16 +
                         (size_t)n_bil * G.n_ops * 16 + B->ld;
  ncta = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)ncta, (int64_t)max_req,
                                                      (int64_t)((16ull << 30) / std::max<size_t>(per_cta, 1))}));
  B->n_cta = ncta;
  B->V.alloc((size_t)ncta * (B->m + 1) * B->ld * 16);
  B->R.alloc((size_t)ncta * std::max(B->m, 3 * nev) * B->ld * 16);
  B->W.alloc((size_t)ncta * B->ld * 16);
  B->X64.alloc((size_t)ncta * B->ld * 16);
  B->tchi64.alloc((size_t)ncta * std::max(n_bil * G.n_ops, 1) * 16);
  B->rowflag.alloc((size_t)ncta * B->ld);
  B->in_chi.alloc((size_t)max_req * G.n_ops * 16);
  B->in_phase.alloc((size_t)max_req * G.n_ops * G.n_site * 16);
  B->in_amp.alloc((size_t)max_req * std::max(n_bil, 1) * 16);
  B->in_seed.alloc((size_t)max_req * 8);
  B->o_evals.alloc((size_t)max_req * nev * 8);
  B->o_status.alloc((size_t)max_req * 4);
  B->o_dims.alloc((size_t)max_req * 8);
  B->o_delta.alloc((size_t)max_req * 8);
  B->o_nmv.alloc((size_t)max_req * 4);
  B->o_hops.alloc((size_t)max_req * 8);
  B->o_tns.alloc((size_t)max_req * 16);
  B->queue.alloc(16);
  B->footprint = per_cta * ncta + (size_t)max_req * (G.n_ops * (G.n_site + 1) * 16 + n_bil * 16 + 8 + nev * 8 + 24);
  SED_CUDA(cudaStreamSynchronize(s));
  return B;
}

static void validate_requests(BatchImpl& B, int n_req, const double* phase, const double* amp) {
  const GroupImpl& G = *B.cat->group;
  GroupImpl Gr = G;
  for (int b = 0; b < n_req; ++b) {
    Gr.phase.assign(phase + (size_t)b * G.n_ops * G.n_site * 2, phase + (size_t)(b + 1) * G.n_ops * G.n_site * 2);
    check_hermitian_symmetric(Gr, B.n_bil, B.bil_ij.data(), amp + (size_t)b * B.n_bil * 2);
  }
}

// Launch on device-resident buffers (asynchronous on the batch stream).
void batch_launch_device(BatchImpl& B, int n_req, const double* chi, const double* phase, const double* amp,
                         const uint64_t* seeds, double tol, int maxiter, double* evals, int32_t* status,
                         int64_t* dims, double* delta, int32_t* nmv) {
  SED_REQUIRE(n_req >= 0 && n_req <= B.max_req, 1, "n_req exceeds max_requests");
  SED_REQUIRE(tol > 0.0 && maxiter >= 1, 1, "tol and maxiter must be positive");
  SED_REQUIRE(chi && phase && seeds && evals && status && dims && delta && nmv, 1, "NULL argument");
  SED_REQUIRE(B.n_bil == 0 || amp, 1, "NULL bilinear amplitudes");
  B.last_n = n_req;
  if (n_req == 0) return;
  cudaStream_t s = B.stream;
  SED_CUDA(cudaMemsetAsync(B.queue.p, 0, 16, s));
  BatchArgs a = base_args(B);
  a.n_req = n_req;
  a.tol = tol;
  a.maxiter = maxiter;
  a.chi = (const double2*)chi;
  a.phase = (const double2*)phase;
  a.amp = (const double2*)amp;
  a.seeds = seeds;
  a.V = B.V.as<double2>();
  a.R = B.R.as<double2>();
  a.W = B.W.as<double2>();
  a.X64 = B.X64.as<double2>();
  a.tchi64 = B.tchi64.as<double2>();
  a.rowflag = B.rowflag.as<uint8_t>();
  a.evals = evals;
  a.status = status;
  a.dims = dims;
  a.delta = delta;
  a.nmv = nmv;
  a.hops = B.o_hops.as<int64_t>();
  a.t_ns = B.o_tns.as<int64_t>();
  a.queue = B.queue.as<unsigned int>();
  BatchSmem L;
  int ncta = 1;
  dispatch_prepare(B, a, L, ncta, true);
  ncta = std::min(B.n_cta, n_req);
  dispatch_launch(B, a, L, ncta, s);
}

void batch_run(BatchImpl& B, int n_req, const double* chi, const double* phase, const double* amp,
               const uint64_t* seeds, double tol, int maxiter, double* evals, int32_t* status, int64_t* dims,
               double* delta, int32_t* nmv) {
  const GroupImpl& G = *B.cat->group;
  SED_REQUIRE(n_req >= 0 && n_req <= B.max_req, 1, "n_req exceeds max_requests");
  SED_REQUIRE(chi && phase && seeds && evals, 1, "NULL argument");
  SED_REQUIRE(B.n_bil == 0 || amp, 1, "NULL bilinear amplitudes");
  if (n_req == 0) return;
  // every request's term list must be Hermitian and invariant under its group
  validate_requests(B, n_req, phase, amp);
  cudaStream_t s = B.stream;
  SED_CUDA(cudaMemcpyAsync(B.in_chi.p, chi, (size_t)n_req * G.n_ops * 16, cudaMemcpyHostToDevice, s));
  SED_CUDA(cudaMemcpyAsync(B.in_phase.p, phase, (size_t)n_req * G.n_ops * G.n_site * 16, cudaMemcpyHostToDevice, s));
  if (B.n_bil)
    SED_CUDA(cudaMemcpyAsync(B.in_amp.p, amp, (size_t)n_req * B.n_bil * 16, cudaMemcpyHostToDevice, s));
  SED_CUDA(cudaMemcpyAsync(B.in_seed.p, seeds, (size_t)n_req * 8, cudaMemcpyHostToDevice, s));
  batch_launch_device(B, n_req, B.in_chi.as<double>(), B.in_phase.as<double>(), B.in_amp.as<double>(),
                      B.in_seed.as<uint64_t>(), tol, maxiter, B.o_evals.as<double>(), B.o_status.as<int32_t>(),
                      B.o_dims.as<int64_t>(), B.o_delta.as<double>(), B.o_nmv.as<int32_t>());
  SED_CUDA(cudaMemcpyAsync(evals, B.o_evals.p, (size_t)n_req * B.nev * 8, cudaMemcpyDeviceToHost, s));
  if (status) SED_CUDA(cudaMemcpyAsync(status, B.o_status.p, (size_t)n_req * 4, cudaMemcpyDeviceToHost, s));
  if (dims) SED_CUDA(cudaMemcpyAsync(dims, B.o_dims.p, (size_t)n_req * 8, cudaMemcpyDeviceToHost, s));
  if (delta) SED_CUDA(cudaMemcpyAsync(delta, B.o_delta.p, (size_t)n_req * 8, cudaMemcpyDeviceToHost, s));
  if (nmv) SED_CUDA(cudaMemcpyAsync(nmv, B.o_nmv.p, (size_t)n_req * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

void batch_last_stats(const BatchImpl& B, int64_t* hops, int64_t* t0, int64_t* t1) {
  const int n = B.last_n;
  if (n == 0) return;
  cudaStream_t s = B.stream;
  SED_CUDA(cudaStreamSynchronize(s));
  if (hops) SED_CUDA(cudaMemcpy(hops, B.o_hops.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
  if (t0 || t1) {
    std::vector<int64_t> t((size_t)n * 2);
    SED_CUDA(cudaMemcpy(t.data(), B.o_tns.p, (size_t)n * 16, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
      if (t0) t0[i] = t[2 * (size_t)i];
      if (t1) t1[i] = t[2 * (size_t)i + 1];
    }
  }
}

}  // namespace sed

// ------------------------------------------------------------------ C ABI
struct sed_batch {
  std::shared_ptr<sed::BatchImpl> p;
};
struct sed_catalog {
  std::shared_ptr<sed::CatalogImpl> p;
};

template <class F>
static int bguard(F&& f) {
  try {
    f();
    return SED_OK;
  } catch (const sed::Error& e) {
    sed::set_error(e.msg);
    return e.code;
  } catch (const std::exception& e) {
    sed::set_error(e.what());
    return SED_ERR_ARG;
  }
}

extern "C" {

int sed_batch_create(const sed_catalog* c, int n_bil, const int32_t* bil_ij, int n_den, const int32_t* den_ij,
                     const double* den_v_reim, int precision, int nev, int krylovdim, int max_requests,
                     sed_batch** out) {
  return bguard([&] {
    SED_REQUIRE(c && out, 1, "NULL argument");
    *out = nullptr;
    auto b = sed::make_batch(c->p, n_bil, bil_ij, n_den, den_ij, den_v_reim, precision, nev, krylovdim, max_requests);
    *out = new sed_batch{b};
  });
}

int sed_batch_run(sed_batch* b, int n_req, const double* chi_reim, const double* group_phase_reim,
                  const double* bil_t_reim, const uint64_t* seeds, double tol, int maxiter, double* evals,
                  int32_t* status, int64_t* dims, double* delta_polish, int32_t* n_matvec) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    sed::batch_run(*b->p, n_req, chi_reim, group_phase_reim, bil_t_reim, seeds, tol, maxiter, evals, status, dims,
                   delta_polish, n_matvec);
  });
}

int sed_batch_last_stats(const sed_batch* b, int64_t* hops, int64_t* t_start_ns, int64_t* t_end_ns) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    sed::batch_last_stats(*b->p, hops, t_start_ns, t_end_ns);
  });
}

int sed_batch_run_device(sed_batch* b, int n_req, const double* d_chi, const double* d_group_phase,
                         const double* d_bil_t, const uint64_t* d_seeds, double tol, int maxiter, double* d_evals,
                         int32_t* d_status, int64_t* d_dims, double* d_delta, int32_t* d_n_matvec) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    sed::batch_launch_device(*b->p, n_req, d_chi, d_group_phase, d_bil_t, d_seeds, tol, maxiter, d_evals, d_status,
                             d_dims, d_delta, d_n_matvec);
  });
}

int sed_batch_set_stream(sed_batch* b, void* stream) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    if (b->p->own_stream && b->p->stream) cudaStreamDestroy(b->p->stream);
    b->p->own_stream = false;
    b->p->stream = (cudaStream_t)stream;
  });
}

int sed_batch_info(const sed_batch* b, int64_t* smem_bytes, int64_t* n_blocks, int64_t* footprint_bytes) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    if (smem_bytes) *smem_bytes = (int64_t)b->p->smem;
    if (n_blocks) *n_blocks = b->p->n_cta;
    if (footprint_bytes) *footprint_bytes = (int64_t)b->p->footprint;
  });
}

void sed_batch_destroy(sed_batch* b) { delete b; }

}  // extern "C"
