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
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <thread>
#include <type_traits>
#include <unordered_map>

#include "../../include/sed_capi.h"
#include "sed_handles.cuh"
#include "sed_internal.cuh"

#include "sed_dfloat.cuh"
#include "sed_rowgather.cuh"

namespace sed {

static constexpr int kBT = 512;      // threads per block
static constexpr int kMaxM = 32;     // Krylov dimension cap
static constexpr int kMaxNev = 8;
static constexpr int kNW = kBT / 32;
static constexpr int kPolCap = 22;         // polish basis capacity (complex Rayleigh-Ritz matrix <= 22 x 22)
static constexpr int kPolishFailed = 100;  // internal status: the FP64 polish missed its target

struct BatchArgs {
  int64_t n_orb, ld;
  int N, G, n_bil, n_terms, n_den;
  int nev, m, maxiter, n_req, kp1;
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
  const int32_t* req_list;  // requests to solve (NULL: 0..n_req-1)
  // hop table (use_tab != 0): SELL-32 records, per-slice offsets / widths,
  // phase-id descriptors and each group element's class representative sites
  int use_tab, n_phi, phi_cap;
  // gauge mode (use_tab != 0): every request's group phases become exactly 1
  // under its site gauge gauge_w[b][site], so a hop's coefficient is one
  // table entry times the sign its record carries (phase id 0: +, 1: -)
  int gauge;
  int tpr;                 // threads per row of the hop-table matvec (1 or 2)
  // coefficient table: tchi_n entries (a prime >= n_bil * G + 1).  Hop-table
  // runs store entry i (term k = i / G, element i % G; i = n_bil * G is the
  // padding records' zero) at (i * tchi_mul) mod tchi_n, which spreads the
  // entries that one warp step gathers over the shared-memory bank groups;
  // on-the-fly runs store it at i.
  int tchi_n, tchi_mul;
  const double2* gauge_w;  // [n_req][N]
  const int32_t* bil_dev;  // [n_bil][2] (from, to) sites of the bilinear terms
  const uint64_t* hop;
  const uint32_t* sl_off;
  const int32_t* sl_w;
  const uint32_t* phi_desc;
  const int8_t* rep_site;  // [G][4]
  double2* pwc64;          // per-block phase-id coefficients (FP64)
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
  // eigenvector output (NULL: none): request b's vector i in sector-row order
  // at evecs[(b * nev + i) * ev_ld + row], complex128, rows < dims[b]
  double2* evecs;
  int64_t ev_ld;
  // ring mode (ring_tail != NULL): the blocks claim request q while q < the
  // host-published tail, by compare-and-swap on the queue head, from slot
  // q % ring_cap; each request's outputs (in mapped host memory) are followed
  // by ring_done[slot] = q + 1.  A block that finds nothing to claim for
  // ring_spin waits, or sees ring_stop, exits.
  const unsigned int* ring_tail;
  const int* ring_stop;
  unsigned int* ring_done;
  int ring_cap;
  int ring_spin;
};

struct BatchSmem {
  size_t x, tchi, eta, chi64, T, Z, theta, coef, red, isr, rank, rec, off, inv, perm, misc, pw32, pw64, mask, basek,
      pwc, zdf, cdf, dfc, zc, total;
};

template <class VT>
static BatchSmem batch_layout(const BatchArgs& a, bool x_in_smem) {
  BatchSmem L{};
  size_t o = 0;
  auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
  L.x = o;
  o = al(o + (x_in_smem ? (size_t)a.n_orb * sizeof(VT) : 0));
  L.tchi = o;  // n_bil * G coefficients and a zero entry for padding records, tchi_n slots
  o = al(o + (size_t)a.tchi_n * sizeof(VT));
  L.eta = o;
  o = al(o + (size_t)a.G * a.N * sizeof(VT));
  L.chi64 = o;
  o = al(o + (size_t)a.G * 16);
  L.T = o;
  o = al(o + kMaxM * kMaxM * 8);
  L.Z = o;
  o = al(o + kMaxM * kMaxM * 8);
  L.theta = o;
  o = al(o + 3 * kMaxM * 8);
  L.coef = o;
  o = al(o + 2 * (kMaxM + 8) * 16);
  L.red = o;
  o = al(o + kNW * 16 * 8);
  L.isr = o;
  o = al(o + 130 * 8 + 130 * 4);
  L.zdf = o;
  o = al(o + kMaxM * kMaxM * 8);
  L.cdf = o;
  o = al(o + (kMaxM + 8) * 16);
  L.dfc = o;  // sqrt(stab) and 1/sqrt(stab) as double-float pairs
  o = al(o + 2 * 65 * 8);
  L.zc = o;  // complex polish rotation, double-float
  o = al(o + kMaxNev * kMaxNev * 16);
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
  L.pw64 = o;
  o = al(o + (size_t)a.G * kMaxCls * a.kp1 * 16);
  L.pw32 = o;
  o = al(o + (size_t)a.G * kMaxCls * a.kp1 * 8);
  L.mask = o;
  o = al(o + (size_t)a.G * kMaxCls * 8);
  L.basek = o;
  o = al(o + (size_t)a.G * 16);
  L.pwc = o;
  o = al(o + (size_t)a.phi_cap * sizeof(VT));
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

// ------------------------------------------------------- double-float vectors
// The Lanczos vectors of the batched solver are double-float numbers; the
// primitives (TwoSum / TwoProd) live in sed_dfloat.cuh.

// Sum 16 double-float values per thread over the block; FP64 results in
// out[0..16).  Within a warp a reduce-scatter butterfly leaves lane pairs
// holding one total each (16 adds per lane instead of 80); the 16 warp totals
// are summed in FP64 in fixed order.
__device__ __forceinline__ void block_sum_df16(float (&h)[16], float (&l)[16], double* red, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int st = 16, half = 8; st >= 2; st >>= 1, half >>= 1) {
    const bool up = (lane & st) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float sh = up ? h[i] : h[i + half], sl = up ? l[i] : l[i + half];
      const float rh = __shfl_xor_sync(0xFFFFFFFFu, sh, st), rl = __shfl_xor_sync(0xFFFFFFFFu, sl, st);
      if (up) {
        h[i] = h[i + half];
        l[i] = l[i + half];
      }
      df_add(h[i], l[i], rh, rl);
    }
  }
  {
    const float rh = __shfl_xor_sync(0xFFFFFFFFu, h[0], 1), rl = __shfl_xor_sync(0xFFFFFFFFu, l[0], 1);
    df_add(h[0], l[0], rh, rl);
  }
  const int idx = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
  if (!(lane & 1)) red[wid * 16 + idx] = df_to_d(h[0], l[0]);
  __syncthreads();
  if (threadIdx.x < 16) {
    double sum = 0.0;
    for (int w = 0; w < kNW; ++w) sum += red[w * 16 + threadIdx.x];
    out[threadIdx.x] = sum;
  }
  __syncthreads();
}

// store one matvec output row: double-float from an FP32 or FP64 accumulator
// (the FP64 kernel's work vector), or FP64 (the FP64 polish)
__device__ __forceinline__ void store_row(float4* w, int64_t o, float yr, float yi) {
  w[o] = make_float4(yr, yi, 0.f, 0.f);
}
__device__ __forceinline__ void store_row(float4* w, int64_t o, double yr, double yi) {
  float4 r;
  d_to_df(yr, r.x, r.z);
  d_to_df(yi, r.y, r.w);
  w[o] = r;
}
__device__ __forceinline__ void store_row(double2* w, int64_t o, double yr, double yi) { w[o] = make_double2(yr, yi); }
__device__ __forceinline__ void store_row(double2* w, int64_t o, float yr, float yi) {
  w[o] = make_double2((double)yr, (double)yi);
}
__device__ __forceinline__ void zero_row(float4* w, int64_t o) { w[o] = make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ void zero_row(double2* w, int64_t o) { w[o] = make_double2(0.0, 0.0); }
// complex64 rows (the mixed kernel's work vector)
__device__ __forceinline__ void store_row(float2* w, int64_t o, float yr, float yi) { w[o] = make_float2(yr, yi); }
__device__ __forceinline__ void store_row(float2* w, int64_t o, double yr, double yi) {
  w[o] = make_float2((float)yr, (float)yi);
}
__device__ __forceinline__ void zero_row(float2* w, int64_t o) { w[o] = make_float2(0.f, 0.f); }

// Jacobi rotation (c, s) for the 2x2 block [[app, apq], [apq, aqq]].  The
// angle only has to shrink apq, not zero it exactly, so it is computed in
// FP32 (GB300's FP64 divide and square root are slow); c and s are then
// normalised to FP64 precision by two Newton steps on 1/sqrt(c^2 + s^2), so
// the rotation is orthogonal to FP64 rounding and the decomposition keeps
// FP64 accuracy (unzeroed remainders are removed by the next sweep).
__device__ __forceinline__ void jacobi_cs(double app, double aqq, double apq, double* c, double* s) {
  const float th = (float)(aqq - app) / (2.0f * (float)apq);
  const float t = (th >= 0.f ? 1.f : -1.f) / (fabsf(th) + sqrtf(fmaf(th, th, 1.f)));
  const float cf = rsqrtf(fmaf(t, t, 1.f));
  double cc = (double)cf, ss = (double)(t * cf);
  for (int it = 0; it < 2; ++it) {
    const double n2 = cc * cc + ss * ss;
    const double f = 1.5 - 0.5 * n2;  // 1/sqrt(n2) to first order around 1
    cc *= f;
    ss *= f;
  }
  *c = cc;
  *s = ss;
}

// unit phase e = a / |a| of a complex number, normalised the same way
__device__ __forceinline__ void unit_phase(double2 a, double* er, double* ei, double* r) {
  const double n2 = a.x * a.x + a.y * a.y;
  double inv = (double)rsqrtf((float)n2);
  for (int it = 0; it < 3; ++it) inv = inv * (1.5 - 0.5 * n2 * inv * inv);
  *er = a.x * inv;
  *ei = a.y * inv;
  *r = n2 * inv;
}


// Pair k of step t of the round-robin (circle-method) ordering of np players
// (np even): over np - 1 steps every pair meets exactly once, and the pairs
// of one step are disjoint.
__device__ __forceinline__ void rr_pair(int t, int k, int np, int& p, int& q) {
  const int m = np - 1;
  if (k == 0) {
    p = t;
    q = m;
  } else {
    p = (t + k) % m;
    q = (t - k + m) % m;
  }
  if (p > q) {
    const int x = p;
    p = q;
    q = x;
  }
}

// Parallel cyclic Jacobi for a real symmetric n x n matrix A (n <= 32, row
// stride kMaxM) in shared memory, by the whole block.  Each round-robin step
// rotates the n/2 disjoint pairs at once, one warp per pair: lane 0 computes
// the rotation and shuffles it to its warp, lane i updates column i (rows p,
// q), and after one barrier row i (columns p, q of A and of the eigenvector
// matrix).  Everything inside the sweeps runs on the FP32 pipe in
// double-float arithmetic, with A and Z held as (hi, lo) float pairs in their
// own double slots: GB300 issues FP64 at 1/64 of the FP32 rate, and each FP64
// warp instruction, however few of its lanes are active, holds that pipe for
// many cycles.  The sweeps stop when the off-diagonal norm is below 1e-13 of
// the total (the double-float rounding level).  Eigenvalues ascending in w,
// eigenvectors (FP64) in the columns of Z; A is destroyed.  cs holds kMaxM
// ints of scratch, red the block-sum scratch, out2 two doubles.
__device__ __forceinline__ float2 df_rot(float ah, float al, float bh, float bl, float2 x, float2 y) {
  // a x + b y
  float h = 0.f, l = 0.f;
  df_mac(h, l, ah, al, x.x, x.y);
  df_mac(h, l, bh, bl, y.x, y.y);
  df_renorm(h, l);
  return make_float2(h, l);
}

// Rotation (c, s) zeroing the off-diagonal of [[app, apq], [apq, aqq]]
// (double-float entries).  The angle comes from the FP32 formula
// t = sign(th) / (|th| + sqrt(th^2 + 1)), th = (aqq - app) / (2 apq); it only
// has to shrink apq, and the next sweep removes what is left.  c and s are
// then normalised to double-float precision: with n2 = c^2 + s^2 = 1 + d
// evaluated exactly (TwoProd, TwoSum), 1/sqrt(n2) = 1 - d/2 + 3 d^2/8 to
// O(d^3) ~ 1e-21, so c^2 + s^2 = 1 within double-float rounding.
__device__ __forceinline__ void jacobi_cs_df(float2 app, float2 aqq, float2 apq, float& ch, float& cl, float& sh,
                                             float& sl) {
  const float d = __fadd_rn(__fsub_rn(aqq.x, app.x), __fsub_rn(aqq.y, app.y));
  const float th = d / (2.0f * __fadd_rn(apq.x, apq.y));
  const float t = (th >= 0.f ? 1.f : -1.f) / (fabsf(th) + sqrtf(fmaf(th, th, 1.f)));
  const float c = rsqrtf(fmaf(t, t, 1.f)), sn = t * c;
  const float p1 = __fmul_rn(c, c), e1 = __fmaf_rn(c, c, -p1);
  const float p2 = __fmul_rn(sn, sn), e2 = __fmaf_rn(sn, sn, -p2);
  float nh, nl;
  df_two_sum(p1, p2, nh, nl);
  const float dd = __fadd_rn(__fsub_rn(nh, 1.0f), __fadd_rn(nl, __fadd_rn(e1, e2)));  // n2 - 1, nh - 1 exact
  const float fl = __fmaf_rn(0.375f * dd, dd, -0.5f * dd);                            // 1/sqrt(n2) - 1
  ch = c;
  cl = c * fl;
  sh = sn;
  sl = sn * fl;
  df_renorm(ch, cl);
  df_renorm(sh, sl);
}

// sum of two floats over the block (fixed order); result in out[0..2)
__device__ __forceinline__ void block_sum2f(float a0, float a1, double* red, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_xor_sync(0xFFFFFFFFu, a0, o);
    a1 += __shfl_xor_sync(0xFFFFFFFFu, a1, o);
  }
  float* r = reinterpret_cast<float*>(red);
  if (lane == 0) {
    r[wid * 2] = a0;
    r[wid * 2 + 1] = a1;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    float sum = 0.f;
    for (int w = 0; w < kNW; ++w) sum += r[w * 2 + threadIdx.x];
    out[threadIdx.x] = sum;
  }
  __syncthreads();
}

__device__ void block_jacobi(int n, double* A, double* Z, double* w, double* cs, double* red, double* out2) {
  const int t = threadIdx.x, bd = blockDim.x, lane = t & 31, wid = t >> 5;
  const int np = (n + 1) & ~1;  // an odd size gets a dummy player n
  const int half = np / 2;
  float2* Ad = reinterpret_cast<float2*>(A);  // a double slot holds one (hi, lo) pair
  float2* Zd = reinterpret_cast<float2*>(Z);
  for (int e = t; e < n * n; e += bd) {
    const int i = e / n, j = e % n;
    float2 d;
    d_to_df(A[i * kMaxM + j], d.x, d.y);
    Ad[i * kMaxM + j] = d;
    Zd[i * kMaxM + j] = make_float2(i == j ? 1.f : 0.f, 0.f);
  }
  __syncthreads();
  for (int sweep = 0; sweep < 40; ++sweep) {
    float off = 0.f, tot = 0.f;  // squared norms (hi parts; a stopping test only)
    for (int e = t; e < n * n; e += bd) {
      const int i = e / n, j = e % n;
      const float v = Ad[i * kMaxM + j].x;
      tot = fmaf(v, v, tot);
      if (i != j) off = fmaf(v, v, off);
    }
    block_sum2f(off, tot, red, out2);
    if (out2[0] <= 1e-26 * fmax(out2[1], 1e-300)) break;
    for (int step = 0; step < np - 1; ++step) {
      int p = 0, q = n;
      float ch = 1.f, cl = 0.f, sh = 0.f, sl = 0.f;
      if (wid < half) {
        rr_pair(step, wid, np, p, q);
        if (q < n) {
          if (lane == 0) {
            const float2 dpq = Ad[p * kMaxM + q], dpp = Ad[p * kMaxM + p], dqq = Ad[q * kMaxM + q];
            if (!(fabsf(dpq.x) <= 1e-16f * (fabsf(dpp.x) + fabsf(dqq.x)) + 1e-36f))
              jacobi_cs_df(dpp, dqq, dpq, ch, cl, sh, sl);
          }
          ch = __shfl_sync(0xFFFFFFFFu, ch, 0);
          cl = __shfl_sync(0xFFFFFFFFu, cl, 0);
          sh = __shfl_sync(0xFFFFFFFFu, sh, 0);
          sl = __shfl_sync(0xFFFFFFFFu, sl, 0);
        }
      }
      const bool rot = q < n && sh != 0.f;  // uniform over the warp
      if (rot && lane < n) {                // rows p, q
        const float2 x = Ad[p * kMaxM + lane], y = Ad[q * kMaxM + lane];
        Ad[p * kMaxM + lane] = df_rot(ch, cl, -sh, -sl, x, y);
        Ad[q * kMaxM + lane] = df_rot(sh, sl, ch, cl, x, y);
      }
      __syncthreads();
      if (rot && lane < n) {  // columns p, q of A and of Z
        float2 x = Ad[lane * kMaxM + p], y = Ad[lane * kMaxM + q];
        Ad[lane * kMaxM + p] = df_rot(ch, cl, -sh, -sl, x, y);
        Ad[lane * kMaxM + q] = df_rot(sh, sl, ch, cl, x, y);
        x = Zd[lane * kMaxM + p];
        y = Zd[lane * kMaxM + q];
        Zd[lane * kMaxM + p] = df_rot(ch, cl, -sh, -sl, x, y);
        Zd[lane * kMaxM + q] = df_rot(sh, sl, ch, cl, x, y);
      }
      __syncthreads();
    }
  }
  // ascending order: rank every eigenvalue (ties by index), then permute the
  // eigenvector columns through A
  int* rank = reinterpret_cast<int*>(cs);
  if (t < n) {
    const float2 di = Ad[t * kMaxM + t];
    const double wi = df_to_d(di.x, di.y);
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const float2 dj = Ad[j * kMaxM + j];
      const double wj = df_to_d(dj.x, dj.y);
      r += (wj < wi) || (wj == wi && j < t);
    }
    rank[t] = r;
    w[r] = wi;
  }
  __syncthreads();
  for (int e = t; e < n * n; e += bd) {
    const int i = e / n, j = e % n;
    const float2 z = Zd[i * kMaxM + j];
    A[i * kMaxM + rank[j]] = df_to_d(z.x, z.y);
  }
  __syncthreads();
  for (int e = t; e < n * n; e += bd) {
    const int i = e / n, j = e % n;
    Z[i * kMaxM + j] = A[i * kMaxM + j];
  }
  __syncthreads();
}

// request inputs are read through L2 (not L1): in ring mode a slot is reused
// by later requests, and an L1 line of its earlier contents would be stale
__device__ __forceinline__ double2 ld_in(const double2* p) { return __ldcg(p); }

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

// Warp-parallel complex Hermitian Jacobi with eigenvectors (row stride
// kPolCap): each rotation makes A_pq real with a phase on column q, then
// zeroes it with a real 2x2 rotation.  Eigenvalues ascending in w.
__device__ void warp_jacobi_herm(int n, double2* A, double2* Z, double* w) {
  const int lane = threadIdx.x & 31;
  const int S = kPolCap;
  for (int i = lane; i < n * S; i += 32) Z[i] = make_double2(0.0, 0.0);
  __syncwarp();
  for (int i = lane; i < n; i += 32) Z[i * S + i] = make_double2(1.0, 0.0);
  __syncwarp();
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int e = lane; e < n * n; e += 32) {
      const int i = e / n, j = e % n;
      const double v = A[i * S + j].x * A[i * S + j].x + A[i * S + j].y * A[i * S + j].y;
      tot += v;
      if (i != j) off += v;
    }
    off = warp_allsum(off);
    tot = warp_allsum(tot);
    if (off <= 1e-29 * fmax(tot, 1e-300)) break;  // rounding level of the off-diagonal part
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double2 apq = A[p * S + q];
        if (fabs(apq.x) + fabs(apq.y) <= 1e-18 * (fabs(A[p * S + p].x) + fabs(A[q * S + q].x)) + 1e-300) continue;
        double er, ei, r;
        unit_phase(apq, &er, &ei, &r);
        double c, sn;
        jacobi_cs(A[p * S + p].x, A[q * S + q].x, r, &c, &sn);
        __syncwarp();
        if (lane < n) {
          const double2 xp = A[lane * S + p], q0 = A[lane * S + q];
          const double2 xq = make_double2(q0.x * er + q0.y * ei, q0.y * er - q0.x * ei);
          A[lane * S + p] = make_double2(c * xp.x - sn * xq.x, c * xp.y - sn * xq.y);
          A[lane * S + q] = make_double2(sn * xp.x + c * xq.x, sn * xp.y + c * xq.y);
          const double2 zp = Z[lane * S + p], z0 = Z[lane * S + q];
          const double2 zq = make_double2(z0.x * er + z0.y * ei, z0.y * er - z0.x * ei);
          Z[lane * S + p] = make_double2(c * zp.x - sn * zq.x, c * zp.y - sn * zq.y);
          Z[lane * S + q] = make_double2(sn * zp.x + c * zq.x, sn * zp.y + c * zq.y);
        }
        __syncwarp();
        if (lane < n) {
          const double2 xp = A[p * S + lane], q0 = A[q * S + lane];
          const double2 xq = make_double2(q0.x * er - q0.y * ei, q0.y * er + q0.x * ei);
          A[p * S + lane] = make_double2(c * xp.x - sn * xq.x, c * xp.y - sn * xq.y);
          A[q * S + lane] = make_double2(sn * xp.x + c * xq.x, sn * xp.y + c * xq.y);
        }
        __syncwarp();
      }
  }
  __syncwarp();
  if (lane == 0) {
    for (int i = 0; i < n; ++i) w[i] = A[i * S + i].x;
    for (int i = 0; i < n; ++i) {
      int b = i;
      for (int j = i + 1; j < n; ++j)
        if (w[j] < w[b]) b = j;
      if (b != i) {
        const double t = w[i];
        w[i] = w[b];
        w[b] = t;
        for (int r = 0; r < n; ++r) {
          const double2 z = Z[r * S + i];
          Z[r * S + i] = Z[r * S + b];
          Z[r * S + b] = z;
        }
      }
    }
  }
  __syncwarp();
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

template <class P, bool FERMI, bool PHASES, class WT>
__device__ __forceinline__ void block_matvec(const BatchArgs& a, const typename P::V* x, const typename P::V* tchi,
                                             const typename P::V* eta, const double* s_isr, const float* s_isrf,
                                             const uint32_t* s_rank, const uint32_t* s_rec, const uint16_t* s_off,
                                             const uint8_t* s_inv, const uint8_t* __restrict__ rowflag,
                                             WT* __restrict__ w, const PhaseClasses<typename P::V>& pcl) {
  using V = typename P::V;
  using S = typename P::S;
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    if (!rowflag[o]) {
      zero_row(w, o);
      continue;
    }
    const double2 dg = a.diag[o];
    const V xo = x[o];
    S ar = (S)dg.x * xo.x - (S)dg.y * xo.y;
    S ai = (S)dg.x * xo.y + (S)dg.y * xo.x;
    row_gather<P, FERMI, PHASES, true>(a.reps[o], x, tchi, nullptr, a.G, eta, a.N, s_rank, a.rp, s_rec, s_off, s_inv,
                                       a.state, ar, ai, pcl);
    const S is = sizeof(S) == 4 ? (S)s_isrf[a.stab[o]] : (S)s_isr[a.stab[o]];
    store_row(w, o, ar * is, ai * is);
  }
}

// sign of v flipped when bit 31 of f is set
__device__ __forceinline__ float flip_sign(float v, uint32_t f) { return __uint_as_float(__float_as_uint(v) ^ f); }
__device__ __forceinline__ double flip_sign(double v, uint32_t f) {
  return __longlong_as_double(__double_as_longlong(v) ^ ((unsigned long long)f << 32));
}

// one hop of the table matvec: coefficient and column value from shared
// memory, accumulated into (ar, ai)
template <class P, bool GAUGE>
__device__ __forceinline__ void hop_acc(uint64_t r, const typename P::V* x, const typename P::V* tchi,
                                        const typename P::V* pwc, typename P::S& ar, typename P::S& ai) {
  using V = typename P::V;
  using S = typename P::S;
  const V t = tchi[(uint32_t)(r >> 24) & 0x3FFFFu];
  const V xc = x[(uint32_t)r & 0xFFFFFFu];
  S cr, ci;
  if (GAUGE) {
    const uint32_t f = ((uint32_t)(r >> 42) & 1u) << 31;
    cr = flip_sign(t.x, f);
    ci = flip_sign(t.y, f);
  } else {
    const V ph = pwc[(uint32_t)(r >> 42)];
    cr = P::mad(t.x, ph.x, -t.y * ph.y);
    ci = P::mad(t.x, ph.y, t.y * ph.x);
  }
  ar = P::mad(cr, xc.x, ar);
  ar = P::mad(-ci, xc.y, ar);
  ai = P::mad(cr, xc.y, ai);
  ai = P::mad(ci, xc.x, ai);
}

// The same matvec through the hop table: one coalesced 8-byte record per hop
// (row 32s + l of slice s at sl_off[s] + 32k + l), then the column value and
// the coefficient from shared memory; the records carry the signs and
// phase-class counts, so a hop costs no rank lookup, state word or popcount.
//   GAUGE = false: coefficient = tchi[term x element] * pwc[phase id] (the
//     phase-id coefficient of the run's twist-phase classes);
//   GAUGE = true (site-gauge runs): the phase id is only the hop's sign (0 +,
//     1 -; padding records point at the zero coefficient), so a hop costs one
//     shared-memory gather fewer -- the random gathers, with their bank
//     conflicts, bound this matvec on the L1 data pipe.
// TPR threads share a row (1, or 2: a lane pair splits the row's records by
// parity and combines by a shuffle; 16 rows per warp), the batched launch's
// threads-per-row shape, chosen by the autotuner.  Passes are uniform over the
// block, so the pair shuffle never meets an exited lane.  The next pass's
// slice offset and width are loaded a pass ahead, and a row's flag and
// stabilizer order before its records: the row then waits on one L2 round
// trip (its first records) instead of three.
template <class P, bool GAUGE, int TPR, class WT>
__device__ __forceinline__ void block_matvec_tab(const BatchArgs& a, const typename P::V* x,
                                                 const typename P::V* tchi, const typename P::V* pwc,
                                                 const double* s_isr, const float* s_isrf,
                                                 const uint8_t* __restrict__ rowflag, WT* __restrict__ w) {
  using V = typename P::V;
  using S = typename P::S;
  const int sub = TPR == 1 ? 0 : (threadIdx.x & (TPR - 1));
  const int64_t rows_per_pass = blockDim.x / TPR;
  int64_t o = threadIdx.x / TPR;
  uint32_t off = 0;
  int wdt = 0;
  if (o < a.n_orb) {
    off = a.sl_off[o >> 5];
    wdt = a.sl_w[o >> 5];
  }
  for (; o - threadIdx.x / TPR < a.n_orb; o += rows_per_pass) {
    const bool valid = o < a.n_orb;
    const int64_t o_next = o + rows_per_pass;
    uint32_t off_next = 0;
    int wdt_next = 0;
    if (o_next < a.n_orb) {
      off_next = a.sl_off[o_next >> 5];
      wdt_next = a.sl_w[o_next >> 5];
    }
    S ar = 0, ai = 0;
    uint8_t flag = 0, st = 0;
    if (valid) {
      flag = rowflag[o];
      st = a.stab[o];
      const uint64_t* rp = a.hop + off + (o & 31);
      if (sub == 0) {
        const double2 dg = a.diag[o];
        const V xo = x[o];
        ar = (S)dg.x * xo.x - (S)dg.y * xo.y;
        ai = (S)dg.x * xo.y + (S)dg.y * xo.x;
      }
#pragma unroll 8
      for (int k = sub; k < wdt; k += TPR) hop_acc<P, GAUGE>(__ldg(rp + 32 * k), x, tchi, pwc, ar, ai);
    }
    off = off_next;
    wdt = wdt_next;
    if (TPR == 2) {
      ar += __shfl_xor_sync(0xFFFFFFFFu, ar, 1);
      ai += __shfl_xor_sync(0xFFFFFFFFu, ai, 1);
    }
    if (!valid || sub != 0) continue;
    if (!flag) {
      zero_row(w, o);
      continue;
    }
    const S is = sizeof(S) == 4 ? (S)s_isrf[st] : (S)s_isr[st];
    store_row(w, o, ar * is, ai * is);
  }
}

template <class P, class WT>
__device__ __forceinline__ void block_matvec_tab_any(const BatchArgs& a, const typename P::V* x,
                                                     const typename P::V* tchi, const typename P::V* pwc,
                                                     const double* s_isr, const float* s_isrf,
                                                     const uint8_t* __restrict__ rowflag, WT* __restrict__ w) {
  if (a.gauge) {
    if (a.tpr == 2) block_matvec_tab<P, true, 2>(a, x, tchi, pwc, s_isr, s_isrf, rowflag, w);
    else block_matvec_tab<P, true, 1>(a, x, tchi, pwc, s_isr, s_isrf, rowflag, w);
  } else {
    if (a.tpr == 2) block_matvec_tab<P, false, 2>(a, x, tchi, pwc, s_isr, s_isrf, rowflag, w);
    else block_matvec_tab<P, false, 1>(a, x, tchi, pwc, s_isr, s_isrf, rowflag, w);
  }
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

// ------------------------------------------------- L2 prefetch of the basis
// The basis streams from HBM (152 blocks x up to 33 vectors of 16 B per
// element exceed the L2 many times over), and with one 512-thread block per SM
// the threads' own loads leave too few bytes in flight to cover HBM latency.
// So the vector sweeps run in chunks of one block-stride of elements and, a
// chunk or two ahead of the loads, one thread per vector asks the TMA unit to
// bring that vector's next chunk into L2 (cp.async.bulk.prefetch: no
// registers, no shared memory, no completion to wait for).
__device__ __forceinline__ void l2_prefetch_bulk(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// chunks that the prefetch runs ahead: about 128 KB per block in flight
// (none for the two-vector local step, whose loads are few enough already)
__device__ __forceinline__ int prefetch_dist(int nv) { return nv <= 2 ? 0 : (nv <= 8 ? 2 : 1); }

// thread t < nv * nch issues chunk c0 + t / nv of vector t % nv (elements
// [chunk * span, chunk * span + span) clipped to n_orb; 16-byte aligned, a
// multiple of 16 bytes)
__device__ __forceinline__ void prefetch_chunks(const BatchArgs& a, const float4* V, int nv, int64_t c0, int nch,
                                                int span, int t) {
  if (nch > 0 && t < nv * nch) {
    const int64_t p0 = (c0 + t / nv) * span;
    if (p0 < a.n_orb)
      l2_prefetch_bulk(V + (size_t)(t % nv) * a.ld + p0, (uint32_t)min((int64_t)span, a.n_orb - p0) * 16u);
  }
}

// coef[l0..l0+nv) = V[0..nv)^H w for double-float vectors, in chunks of 8
__device__ void df_dots(const BatchArgs& a, const float4* V, int nv, const float4* w, double* red, double2* coef) {
  for (int l0 = 0; l0 < nv; l0 += 8) {
    float h[16], l[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) h[c] = l[c] = 0.f;
    const int cn = min(8, nv - l0);
    const int span = blockDim.x, pd = prefetch_dist(cn);
    const float4* Vl = V + (size_t)l0 * a.ld;
    prefetch_chunks(a, Vl, cn, 0, pd, span, threadIdx.x);
    for (int64_t o0 = 0, ch = 0; o0 < a.n_orb; o0 += span, ++ch) {
      if (pd) prefetch_chunks(a, Vl, cn, ch + pd, 1, span, threadIdx.x);
      const int64_t o = o0 + threadIdx.x;
      if (o >= a.n_orb) continue;
      const float4 x = w[o];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) {
          const float4 v = Vl[(size_t)c * a.ld + o];
          // conj(v) x = (vr xr + vi xi) + i (vr xi - vi xr)
          df_mac(h[2 * c], l[2 * c], v.x, v.z, x.x, x.z);
          df_mac(h[2 * c], l[2 * c], v.y, v.w, x.y, x.w);
          df_mac(h[2 * c + 1], l[2 * c + 1], v.x, v.z, x.y, x.w);
          df_mac(h[2 * c + 1], l[2 * c + 1], -v.y, -v.w, x.x, x.z);
        }
    }
    block_sum_df16(h, l, red, reinterpret_cast<double*>(coef + l0));
  }
}

// The local step's update folded into the first chunk of the full pass:
// w -= Vl[0..nl) cl (cl double-float in shared memory), then coef[0..cn) =
// V[0..cn)^H w (cn <= 7) and |w|^2 in the same sweep and the same block
// reduction (slot 14).  Returns |w|^2.  Out of line for the same register
// reason as df_axpy.
__device__ __noinline__ double df_dots_local(const BatchArgs& a, const float4* V, int cn, const float4* Vl, int nl,
                                const float4* cl, float4* w, double* red, double2* coef) {
  float h[16], l[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) h[c] = l[c] = 0.f;
  const int span = blockDim.x, pd = prefetch_dist(cn);
  prefetch_chunks(a, V, cn, 0, pd, span, threadIdx.x);
  for (int64_t o0 = 0, ch = 0; o0 < a.n_orb; o0 += span, ++ch) {
    if (pd) prefetch_chunks(a, V, cn, ch + pd, 1, span, threadIdx.x);
    const int64_t o = o0 + threadIdx.x;
    if (o >= a.n_orb) continue;
    float4 x = w[o];
    for (int q = 0; q < nl; ++q) {
      const float4 v = Vl[(size_t)q * a.ld + o];
      const float4 cf = cl[q];
      df_mac(x.x, x.z, -cf.x, -cf.z, v.x, v.z);
      df_mac(x.x, x.z, cf.y, cf.w, v.y, v.w);
      df_mac(x.y, x.w, -cf.x, -cf.z, v.y, v.w);
      df_mac(x.y, x.w, -cf.y, -cf.w, v.x, v.z);
    }
    df_renorm(x.x, x.z);
    df_renorm(x.y, x.w);
    w[o] = x;
    df_mac(h[14], l[14], x.x, x.z, x.x, x.z);
    df_mac(h[14], l[14], x.y, x.w, x.y, x.w);
#pragma unroll
    for (int c = 0; c < 7; ++c)
      if (c < cn) {
        const float4 v = V[(size_t)c * a.ld + o];
        df_mac(h[2 * c], l[2 * c], v.x, v.z, x.x, x.z);
        df_mac(h[2 * c], l[2 * c], v.y, v.w, x.y, x.w);
        df_mac(h[2 * c + 1], l[2 * c + 1], v.x, v.z, x.y, x.w);
        df_mac(h[2 * c + 1], l[2 * c + 1], -v.y, -v.w, x.x, x.z);
      }
  }
  double* out = reinterpret_cast<double*>(coef);
  block_sum_df16(h, l, red, out);
  return out[14];
}

// split FP64 coefficients into double-float (one thread each)
__device__ __forceinline__ void df_coefs(const double2* coef, int nv, float4* cdf) {
  if (threadIdx.x < nv) {
    float4 c;
    d_to_df(coef[threadIdx.x].x, c.x, c.z);
    d_to_df(coef[threadIdx.x].y, c.y, c.w);
    cdf[threadIdx.x] = c;
  }
  __syncthreads();
}

// w -= V[0..nv) c (c double-float in shared memory); returns this thread's
// partial |w|^2 in FP64.  The basis is read in groups of eight vectors whose
// loads are issued before the arithmetic, so a thread keeps eight 16-byte HBM
// reads in flight.  The function stays out of line: inlined, those registers
// would add to the solver's peak and spill.
__device__ __noinline__ double df_axpy(const BatchArgs& a, const float4* V, int nv, const float4* cdf,
                                          float4* w) {
  float nh = 0.f, nl = 0.f;
  const int span = blockDim.x, pd = prefetch_dist(nv);
  prefetch_chunks(a, V, nv, 0, pd, span, threadIdx.x);
  for (int64_t o0 = 0, ch = 0; o0 < a.n_orb; o0 += span, ++ch) {
    if (pd) prefetch_chunks(a, V, nv, ch + pd, 1, span, threadIdx.x);
    const int64_t o = o0 + threadIdx.x;
    if (o >= a.n_orb) continue;
    float4 x = w[o];
    for (int q0 = 0; q0 < nv; q0 += 8) {
      const int cn = min(8, nv - q0);
      float4 v[8];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) v[c] = V[(size_t)(q0 + c) * a.ld + o];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) {
          const float4 cf = cdf[q0 + c];
          // x -= c v: re -= cr vr - ci vi, im -= cr vi + ci vr
          df_mac(x.x, x.z, -cf.x, -cf.z, v[c].x, v[c].z);
          df_mac(x.x, x.z, cf.y, cf.w, v[c].y, v[c].w);
          df_mac(x.y, x.w, -cf.x, -cf.z, v[c].y, v[c].w);
          df_mac(x.y, x.w, -cf.y, -cf.w, v[c].x, v[c].z);
        }
    }
    df_renorm(x.x, x.z);
    df_renorm(x.y, x.w);
    w[o] = x;
    df_mac(nh, nl, x.x, x.z, x.x, x.z);
    df_mac(nh, nl, x.y, x.w, x.y, x.w);
  }
  return df_to_d(nh, nl);
}

// v = w * inv (double-float), and the scaled matvec input x = sqrt(stab) v:
// complex64 from the high parts, or FP64 for the FP64 matvec
template <class VT>
__device__ __forceinline__ void df_normalize(const BatchArgs& a, const float4* w, double inv, float4* v, VT* x,
                                             const float* s_sqrtf, const double* s_sqrt) {
  float ih, il;
  d_to_df(inv, ih, il);
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    const float4 y = w[o];
    float4 r;
    r.x = __fmul_rn(y.x, ih);
    r.z = __fmaf_rn(y.x, il, __fmaf_rn(y.z, ih, __fmaf_rn(y.x, ih, -r.x)));
    r.y = __fmul_rn(y.y, ih);
    r.w = __fmaf_rn(y.y, il, __fmaf_rn(y.w, ih, __fmaf_rn(y.y, ih, -r.y)));
    df_renorm(r.x, r.z);
    df_renorm(r.y, r.w);
    if (v) v[o] = r;
    if (x) {
      if (sizeof(VT) == 8) {
        const float sq = s_sqrtf[a.stab[o]];
        reinterpret_cast<float2*>(x)[o] = make_float2(r.x * sq, r.y * sq);
      } else {
        const double sq = s_sqrt[a.stab[o]];
        reinterpret_cast<double2*>(x)[o] = make_double2(df_to_d(r.x, r.z) * sq, df_to_d(r.y, r.w) * sq);
      }
    }
  }
}

// out[c] = sum_l V[l] Z[l][c] for c < keep, Z real double-float (row stride
// kMaxM).  Outputs go in chunks of eight accumulators.  With more than one
// chunk the block splits into two halves that sweep the same elements at the
// same time, half h taking chunks h, h + 2, ..., so each basis vector streams
// from HBM once and the other half's read of it hits the caches.  Loads are
// issued four vectors ahead of the arithmetic.
__device__ void df_rotate(const BatchArgs& a, const float4* V, int msz, const float2* Z, int keep, float4* out) {
  const int nch = (keep + 7) / 8;
  const int ng = nch > 1 ? 2 : 1;
  const int gsz = blockDim.x / ng, grp = threadIdx.x / gsz, t = threadIdx.x - grp * gsz;
  for (int ch = grp; ch < nch; ch += ng) {
    const int c0 = ch * 8, cn = min(8, keep - c0);
    for (int64_t o = t; o < a.n_orb; o += gsz) {
      float4 acc[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int q0 = 0; q0 < msz; q0 += 4) {
        const int qn = min(4, msz - q0);
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (u < qn) v[u] = V[(size_t)(q0 + u) * a.ld + o];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (u < qn) {
#pragma unroll
            for (int c = 0; c < 8; ++c)
              if (c < cn) {
                const float2 z = Z[(q0 + u) * kMaxM + c0 + c];
                df_mac(acc[c].x, acc[c].z, v[u].x, v[u].z, z.x, z.y);
                df_mac(acc[c].y, acc[c].w, v[u].y, v[u].w, z.x, z.y);
              }
          }
      }
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) {
          df_renorm(acc[c].x, acc[c].z);
          df_renorm(acc[c].y, acc[c].w);
          out[(size_t)(c0 + c) * a.ld + o] = acc[c];
        }
    }
  }
}

// x = sqrt(stab) v in double-float (the polish's matvec input)
__device__ __forceinline__ void df_scale_xs(const BatchArgs& a, const float4* v, float4* x, const float2* s_sq) {
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    const float4 y = v[o];
    const float2 q = s_sq[a.stab[o]];
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    df_mac(r.x, r.z, y.x, y.z, q.x, q.y);
    df_mac(r.y, r.w, y.y, y.w, q.x, q.y);
    df_renorm(r.x, r.z);
    df_renorm(r.y, r.w);
    x[o] = r;
  }
}

// The hop-table matvec in double-float (the FP64-class polish): per hop the
// coefficient tchi[uh] * pwc[phi] and its product with x[c], each a complex
// double-float product (TwoProd/TwoSum on the FP32 pipe); rows scaled by
// 1/sqrt(stab) in double-float.
__device__ __forceinline__ void block_matvec_tab_df(const BatchArgs& a, const float4* __restrict__ x,
                                                    const float4* __restrict__ tchi, const float4* __restrict__ pwc,
                                                    const float2* s_isr_df, const uint8_t* __restrict__ rowflag,
                                                    float4* __restrict__ w) {
  const int lane = threadIdx.x & 31;
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    if (!rowflag[o]) {
      w[o] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    const int64_t sl = o >> 5;
    const uint64_t* rp = a.hop + a.sl_off[sl] + lane;
    const int wdt = a.sl_w[sl];
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    {
      const double2 dg = a.diag[o];
      float2 dr, di;
      d_to_df(dg.x, dr.x, dr.y);
      d_to_df(dg.y, di.x, di.y);
      const float4 xo = x[o];
      df_mac(acc.x, acc.z, dr.x, dr.y, xo.x, xo.z);
      df_mac(acc.x, acc.z, -di.x, -di.y, xo.y, xo.w);
      df_mac(acc.y, acc.w, dr.x, dr.y, xo.y, xo.w);
      df_mac(acc.y, acc.w, di.x, di.y, xo.x, xo.z);
    }
#pragma unroll 2
    for (int k = 0; k < wdt; ++k) {
      const uint64_t r = __ldg(rp + 32 * k);
      const float4 t = tchi[(uint32_t)(r >> 24) & 0x3FFFFu];
      const float4 ph = pwc[(uint32_t)(r >> 42)];
      const float4 xc = x[(uint32_t)r & 0xFFFFFFu];
      float4 cf = make_float4(0.f, 0.f, 0.f, 0.f);
      df_mac(cf.x, cf.z, t.x, t.z, ph.x, ph.z);
      df_mac(cf.x, cf.z, -t.y, -t.w, ph.y, ph.w);
      df_mac(cf.y, cf.w, t.x, t.z, ph.y, ph.w);
      df_mac(cf.y, cf.w, t.y, t.w, ph.x, ph.z);
      df_renorm(cf.x, cf.z);
      df_renorm(cf.y, cf.w);
      df_mac(acc.x, acc.z, cf.x, cf.z, xc.x, xc.z);
      df_mac(acc.x, acc.z, -cf.y, -cf.w, xc.y, xc.w);
      df_mac(acc.y, acc.w, cf.x, cf.z, xc.y, xc.w);
      df_mac(acc.y, acc.w, cf.y, cf.w, xc.x, xc.z);
    }
    df_renorm(acc.x, acc.z);
    df_renorm(acc.y, acc.w);
    const float2 is = s_isr_df[a.stab[o]];
    float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
    df_mac(y.x, y.z, acc.x, acc.z, is.x, is.y);
    df_mac(y.y, y.w, acc.y, acc.w, is.x, is.y);
    df_renorm(y.x, y.z);
    df_renorm(y.y, y.w);
    w[o] = y;
  }
}

// out_c = sum_l V[l] S[l][c] for c < nw, S complex double-float (row stride kMaxNev)
__device__ void df_rotate_c(const BatchArgs& a, const float4* V, int nb, const float4* S, int nw, float4* out) {
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    float4 acc[kMaxNev];
#pragma unroll
    for (int c = 0; c < kMaxNev; ++c) acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int l = 0; l < nb; ++l) {
      const float4 v = V[(size_t)l * a.ld + o];
#pragma unroll
      for (int c = 0; c < kMaxNev; ++c)
        if (c < nw) {
          const float4 t = S[l * kMaxNev + c];
          df_mac(acc[c].x, acc[c].z, v.x, v.z, t.x, t.z);
          df_mac(acc[c].x, acc[c].z, -v.y, -v.w, t.y, t.w);
          df_mac(acc[c].y, acc[c].w, v.x, v.z, t.y, t.w);
          df_mac(acc[c].y, acc[c].w, v.y, v.w, t.x, t.z);
        }
    }
#pragma unroll
    for (int c = 0; c < kMaxNev; ++c)
      if (c < nw) {
        df_renorm(acc[c].x, acc[c].z);
        df_renorm(acc[c].y, acc[c].w);
        out[(size_t)c * a.ld + o] = acc[c];
      }
  }
}

// out_c = sum_l V[l] S[l][c], complex coefficients (row stride kPolCap)
__device__ void block_rotate_c(const BatchArgs& a, const double2* V, int nb, const double2* S, int nw, double2* out) {
  for (int c0 = 0; c0 < nw; c0 += 8) {
    const int cn = min(8, nw - c0);
    for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
      double ar[8], ai[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) ar[c] = ai[c] = 0.0;
      for (int l = 0; l < nb; ++l) {
        const double2 v = V[(size_t)l * a.ld + o];
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (c < cn) {
            const double2 sc = S[l * kPolCap + c0 + c];
            ar[c] += v.x * sc.x - v.y * sc.y;
            ai[c] += v.x * sc.y + v.y * sc.x;
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
__device__ __forceinline__ void block_normalize(const BatchArgs& a, const double2* w, double inv, double2* v, VT* x,
                                                const double* s_sqrt) {
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    const double2 y = make_double2(w[o].x * inv, w[o].y * inv);
    if (v) v[o] = y;
    if (x) {
      const double sq = s_sqrt[a.stab[o]];
      x[o].x = y.x * sq;
      x[o].y = y.y * sq;
    }
  }
}

// ------------------------------------------- complex64 vectors (mixed)
// In mixed precision the Lanczos basis, restart buffer and work vector are
// complex64: 8 bytes per element, half the traffic of the double-float
// vectors the FP64 kernel keeps.  Each stored value is rounded once to FP32
// from an accurately computed one:
// * dot products accumulate FP32 products per thread (a thread sums
//   n_orb / 512 elements) and add the thread partials in double-float, then
//   FP64, over the block;
// * updates w -= sum_q c_q v_q apply each coefficient as hi + lo floats, so
//   the large local coefficients (alpha, beta) cancel without losing bits,
//   and |w|^2 is summed in double-float;
// * restart rotations accumulate in double-float (TwoProd, TwoSum);
// * the normalisation multiplies by 1/|w| as hi + lo floats.
// The storage rounding (2^-24) is the size of the complex64 matvec's own
// rounding, which already perturbs the recurrence at that level; the
// FP64-class Rayleigh-Ritz check bounds the eigenvalues.  The check itself
// runs on double-float copies of the Ritz block.

// The complex64 sweeps rely on the threads' own loads: with half the bytes
// per element, the bulk L2 prefetch of the double-float sweeps measured
// slower here (1929 against 1971 sector solves/s on the flux-scan batch).
// Their loops step over the block's rows in block-wide chunks, a trip count
// uniform over the block, with the threads past the end skipping their row:
// the per-thread strided form of the same loops measured 10 % slower (1790
// sector solves/s).  Each thread takes element pairs, so every load moves 16
// bytes: 2177 against 1981 sector solves/s with one element per thread.

// coef[0..nv) = V[0..nv)^H w for complex64 vectors, in chunks of 8.  Each
// thread takes element pairs (16-byte loads; ld is even and vectors start on
// 16-byte boundaries), the last element of an odd n_orb by thread 0.
__device__ __forceinline__ void cf_acc(float& re, float& im, float vx, float vy, float xx, float xy) {
  // conj(v) x = (vr xr + vi xi) + i (vr xi - vi xr)
  re = __fmaf_rn(vx, xx, __fmaf_rn(vy, xy, re));
  im = __fmaf_rn(vx, xy, __fmaf_rn(-vy, xx, im));
}
__device__ void cf_dots(const BatchArgs& a, const float2* V, int nv, const float2* w, double* red, double2* coef) {
  const int64_t np = a.n_orb >> 1;
  for (int l0 = 0; l0 < nv; l0 += 8) {
    float h[16], l[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) h[c] = l[c] = 0.f;
    const int cn = min(8, nv - l0);
    const float2* Vl = V + (size_t)l0 * a.ld;
    for (int64_t p0 = 0; p0 < np; p0 += blockDim.x) {
      const int64_t p = p0 + threadIdx.x;
      if (p >= np) continue;
      const float4 x = reinterpret_cast<const float4*>(w)[p];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) {
          const float4 v = reinterpret_cast<const float4*>(Vl + (size_t)c * a.ld)[p];
          cf_acc(h[2 * c], h[2 * c + 1], v.x, v.y, x.x, x.y);
          cf_acc(h[2 * c], h[2 * c + 1], v.z, v.w, x.z, x.w);
        }
    }
    if ((a.n_orb & 1) && threadIdx.x == 0) {
      const float2 x = w[a.n_orb - 1];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) {
          const float2 v = Vl[(size_t)c * a.ld + a.n_orb - 1];
          cf_acc(h[2 * c], h[2 * c + 1], v.x, v.y, x.x, x.y);
        }
    }
    block_sum_df16(h, l, red, reinterpret_cast<double*>(coef + l0));
  }
}


// The local step's update folded into the first chunk of the full pass
// (complex64 counterpart of df_dots_local): w -= Vl[0..nl) cl, then
// coef[0..cn) = V[0..cn)^H w (cn <= 7) and |w|^2 (slot 14, double-float) in
// the same sweep and block reduction, on element pairs.  Returns |w|^2.
__device__ __forceinline__ void cf_local_one(const BatchArgs& a, const float2* V, int cn, const float2* Vl, int nl,
                                             const float4* cl, float2& x, int64_t o, float (&h)[16],
                                             float (&l)[16]) {
  for (int q = 0; q < nl; ++q) cf_sub(x.x, x.y, cl[q], Vl[(size_t)q * a.ld + o]);
  df_mac(h[14], l[14], x.x, 0.f, x.x, 0.f);
  df_mac(h[14], l[14], x.y, 0.f, x.y, 0.f);
#pragma unroll
  for (int c = 0; c < 7; ++c)
    if (c < cn) {
      const float2 v = V[(size_t)c * a.ld + o];
      cf_acc(h[2 * c], h[2 * c + 1], v.x, v.y, x.x, x.y);
    }
}
__device__ __noinline__ double cf_dots_local(const BatchArgs& a, const float2* V, int cn, const float2* Vl, int nl,
                                             const float4* cl, float2* w, double* red, double2* coef) {
  float h[16], l[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) h[c] = l[c] = 0.f;
  const int64_t np = a.n_orb >> 1;
  for (int64_t p0 = 0; p0 < np; p0 += blockDim.x) {
    const int64_t p = p0 + threadIdx.x;
    if (p >= np) continue;
    float4 x = reinterpret_cast<const float4*>(w)[p];
    for (int q = 0; q < nl; ++q) {
      const float4 v = reinterpret_cast<const float4*>(Vl + (size_t)q * a.ld)[p];
      cf_sub(x.x, x.y, cl[q], make_float2(v.x, v.y));
      cf_sub(x.z, x.w, cl[q], make_float2(v.z, v.w));
    }
    reinterpret_cast<float4*>(w)[p] = x;
    df_mac(h[14], l[14], x.x, 0.f, x.x, 0.f);
    df_mac(h[14], l[14], x.y, 0.f, x.y, 0.f);
    df_mac(h[14], l[14], x.z, 0.f, x.z, 0.f);
    df_mac(h[14], l[14], x.w, 0.f, x.w, 0.f);
#pragma unroll
    for (int c = 0; c < 7; ++c)
      if (c < cn) {
        const float4 v = reinterpret_cast<const float4*>(V + (size_t)c * a.ld)[p];
        cf_acc(h[2 * c], h[2 * c + 1], v.x, v.y, x.x, x.y);
        cf_acc(h[2 * c], h[2 * c + 1], v.z, v.w, x.z, x.w);
      }
  }
  if ((a.n_orb & 1) && threadIdx.x == 0) {
    const int64_t o = a.n_orb - 1;
    float2 x = w[o];
    cf_local_one(a, V, cn, Vl, nl, cl, x, o, h, l);
    w[o] = x;
  }
  double* out = reinterpret_cast<double*>(coef);
  block_sum_df16(h, l, red, out);
  return out[14];
}

// w -= V[0..nv) c (c as hi + lo floats in shared memory); returns this
// thread's partial |w|^2 (double-float, then FP64).  Element pairs; loads are
// issued in groups of eight vectors before the arithmetic; out of line like
// df_axpy.
__device__ __noinline__ double cf_axpy(const BatchArgs& a, const float2* V, int nv, const float4* cdf, float2* w) {
  float nh = 0.f, nl = 0.f;
  const int64_t np = a.n_orb >> 1;
  for (int64_t p0 = 0; p0 < np; p0 += blockDim.x) {
    const int64_t p = p0 + threadIdx.x;
    if (p >= np) continue;
    float4 x = reinterpret_cast<const float4*>(w)[p];
    for (int q0 = 0; q0 < nv; q0 += 8) {
      const int cn = min(8, nv - q0);
      float4 v[8];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) v[c] = reinterpret_cast<const float4*>(V + (size_t)(q0 + c) * a.ld)[p];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn) {
          cf_sub(x.x, x.y, cdf[q0 + c], make_float2(v[c].x, v[c].y));
          cf_sub(x.z, x.w, cdf[q0 + c], make_float2(v[c].z, v[c].w));
        }
    }
    reinterpret_cast<float4*>(w)[p] = x;
    df_mac(nh, nl, x.x, 0.f, x.x, 0.f);
    df_mac(nh, nl, x.y, 0.f, x.y, 0.f);
    df_mac(nh, nl, x.z, 0.f, x.z, 0.f);
    df_mac(nh, nl, x.w, 0.f, x.w, 0.f);
  }
  if ((a.n_orb & 1) && threadIdx.x == 0) {
    const int64_t o = a.n_orb - 1;
    float2 x = w[o];
    for (int q = 0; q < nv; ++q) cf_sub(x.x, x.y, cdf[q], V[(size_t)q * a.ld + o]);
    w[o] = x;
    df_mac(nh, nl, x.x, 0.f, x.x, 0.f);
    df_mac(nh, nl, x.y, 0.f, x.y, 0.f);
  }
  return df_to_d(nh, nl);
}

// v = w * inv (inv as hi + lo floats, one rounding of the product) and the
// complex64 matvec input x = sqrt(stab) v
__device__ __forceinline__ void cf_normalize(const BatchArgs& a, const float2* w, double inv, float2* v, float2* x,
                                             const float* s_sqrtf) {
  float ih, il;
  d_to_df(inv, ih, il);
  for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
    const float2 y = w[o];
    const float rx = __fmaf_rn(y.x, ih, __fmul_rn(y.x, il));
    const float ry = __fmaf_rn(y.y, ih, __fmul_rn(y.y, il));
    if (v) v[o] = make_float2(rx, ry);
    if (x) {
      const float sq = s_sqrtf[a.stab[o]];
      x[o] = make_float2(__fmul_rn(rx, sq), __fmul_rn(ry, sq));
    }
  }
}


// out[c] = sum_l V[l] Z[l][c] for c < keep (complex64 counterpart of
// df_rotate: same chunking and half-block split), accumulated in
// double-float and rounded once to complex64
__device__ void cf_rotate(const BatchArgs& a, const float2* V, int msz, const float2* Z, int keep, float2* out) {
  const int nch = (keep + 7) / 8;
  const int ng = nch > 1 ? 2 : 1;
  const int gsz = blockDim.x / ng, grp = threadIdx.x / gsz, t = threadIdx.x - grp * gsz;
  for (int ch = grp; ch < nch; ch += ng) {
    const int c0 = ch * 8, cn = min(8, keep - c0);
    for (int64_t o = t; o < a.n_orb; o += gsz) {
      float4 acc[8];  // (re_hi, im_hi, re_lo, im_lo)
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int q0 = 0; q0 < msz; q0 += 4) {
        const int qn = min(4, msz - q0);
        float2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (u < qn) v[u] = V[(size_t)(q0 + u) * a.ld + o];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (u < qn) {
#pragma unroll
            for (int c = 0; c < 8; ++c)
              if (c < cn) {
                const float2 z = Z[(q0 + u) * kMaxM + c0 + c];
                df_mac1(acc[c].x, acc[c].z, v[u].x, z.x, z.y);
                df_mac1(acc[c].y, acc[c].w, v[u].y, z.x, z.y);
              }
          }
      }
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c < cn)
          out[(size_t)(c0 + c) * a.ld + o] = make_float2(__fadd_rn(acc[c].x, acc[c].z), __fadd_rn(acc[c].y, acc[c].w));
    }
  }
}

// The Lanczos vector operations of k_batch, by basis type: double-float
// (float4, FP64 kernel) or complex64 (float2, mixed kernel).
__device__ __forceinline__ void lz_dots(const BatchArgs& a, const float4* V, int nv, const float4* w, double* red,
                                        double2* coef) {
  df_dots(a, V, nv, w, red, coef);
}
__device__ __forceinline__ void lz_dots(const BatchArgs& a, const float2* V, int nv, const float2* w, double* red,
                                        double2* coef) {
  cf_dots(a, V, nv, w, red, coef);
}
__device__ __forceinline__ double lz_dots_local(const BatchArgs& a, const float4* V, int cn, const float4* Vl, int nl,
                                                const float4* cl, float4* w, double* red, double2* coef) {
  return df_dots_local(a, V, cn, Vl, nl, cl, w, red, coef);
}
__device__ __forceinline__ double lz_dots_local(const BatchArgs& a, const float2* V, int cn, const float2* Vl, int nl,
                                                const float4* cl, float2* w, double* red, double2* coef) {
  return cf_dots_local(a, V, cn, Vl, nl, cl, w, red, coef);
}
__device__ __forceinline__ double lz_axpy(const BatchArgs& a, const float4* V, int nv, const float4* cdf, float4* w) {
  return df_axpy(a, V, nv, cdf, w);
}
__device__ __forceinline__ double lz_axpy(const BatchArgs& a, const float2* V, int nv, const float4* cdf, float2* w) {
  return cf_axpy(a, V, nv, cdf, w);
}
template <class VT>
__device__ __forceinline__ void lz_normalize(const BatchArgs& a, const float4* w, double inv, float4* v, VT* x,
                                             const float* s_sqrtf, const double* s_sqrt) {
  df_normalize<VT>(a, w, inv, v, x, s_sqrtf, s_sqrt);
}
template <class VT>
__device__ __forceinline__ void lz_normalize(const BatchArgs& a, const float2* w, double inv, float2* v, VT* x,
                                             const float* s_sqrtf, const double*) {
  static_assert(sizeof(VT) == 8, "the complex64 basis feeds the complex64 matvec");
  cf_normalize(a, w, inv, v, reinterpret_cast<float2*>(x), s_sqrtf);
}
__device__ __forceinline__ void lz_rotate(const BatchArgs& a, const float4* V, int msz, const float2* Z, int keep,
                                          float4* out) {
  df_rotate(a, V, msz, Z, keep, out);
}
__device__ __forceinline__ void lz_rotate(const BatchArgs& a, const float2* V, int msz, const float2* Z, int keep,
                                          float2* out) {
  cf_rotate(a, V, msz, Z, keep, out);
}
// one basis element as double-float and as FP64
__device__ __forceinline__ float4 lz_to_df(float4 v) { return v; }
__device__ __forceinline__ float4 lz_to_df(float2 v) { return make_float4(v.x, v.y, 0.f, 0.f); }
__device__ __forceinline__ double2 lz_to_d(float4 v) { return make_double2(df_to_d(v.x, v.z), df_to_d(v.y, v.w)); }
__device__ __forceinline__ double2 lz_to_d(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 lz_to_d(double2 v) { return v; }

// Eigenvector output of one request: vector i (i < nvec) of src (stride ld,
// orbit-indexed, in the site gauge when gw is set) into sector-row order.  A
// row's index is the number of sector orbits before it, counted by a
// block-wide scan over rowflag one block-stride at a time; in gauge mode a
// row's coefficient is multiplied by conj(prod_{j in rep} w_j), which undoes
// the gauge (W |r> = prod_{j in rep} w_j |r'> for the sector basis states).
// s_cnt holds kNW + 1 ints of shared scratch.
template <class SRC>
__device__ void block_write_vectors(const BatchArgs& a, const SRC* src, int64_t ld, int nvec,
                                    const uint8_t* __restrict__ rowflag, const double2* gw, double2* out,
                                    int* s_cnt) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int carry = 0;
  for (int64_t base = 0; base < a.n_orb; base += blockDim.x) {
    const int64_t o = base + threadIdx.x;
    const bool f = o < a.n_orb && rowflag[o];
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, f);
    if (lane == 0) s_cnt[wid] = __popc(bal);
    __syncthreads();
    int wpre = 0;
    for (int w = 0; w < wid; ++w) wpre += s_cnt[w];
    if (f) {
      const int64_t row = carry + wpre + __popc(bal & ((1u << lane) - 1u));
      double2 gc = make_double2(1.0, 0.0);  // conj(prod_{j in rep} w_j)
      if (gw) {
        uint64_t m = a.reps[o];
        while (m) {
          const int j = __ffsll((long long)m) - 1;
          m &= m - 1;
          const double2 w = gw[j];
          gc = make_double2(gc.x * w.x + gc.y * w.y, gc.y * w.x - gc.x * w.y);
        }
      }
      for (int i = 0; i < nvec; ++i) {
        const double2 v = lz_to_d(src[(size_t)i * ld + o]);
        out[(size_t)i * a.ev_ld + row] = make_double2(v.x * gc.x - v.y * gc.y, v.x * gc.y + v.y * gc.x);
      }
    }
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < kNW; ++w) tot += s_cnt[w];
      s_cnt[kNW] = carry + tot;
    }
    __syncthreads();
    carry = s_cnt[kNW];
    __syncthreads();
  }
}

// ---------------------------------------------------------------- the kernel
// Rayleigh-Ritz on a block B that is only semi-orthogonal (kSelReorth): with
// G = B^H B = L L^H (Cholesky), B L^-H is orthonormal and its projected matrix
// is L^-1 M L^-H, M = B^H H B.  M (row stride kPolCap) is overwritten by the
// projected matrix and G (row stride kMaxNev) by X = L^-1 (lower triangular);
// T is kMaxNev^2 of scratch.  The factorisation runs on thread 0 (nw <= 8),
// the products on nw^2 threads.
__device__ void rr_orthonormalise(int nw, double2* M, double2* G, double2* T) {
  constexpr int SG = kMaxNev;
  if (threadIdx.x == 0) {
    for (int k = 0; k < nw; ++k) {  // Cholesky, lower
      double d = G[k * SG + k].x;
      for (int p = 0; p < k; ++p) d -= G[k * SG + p].x * G[k * SG + p].x + G[k * SG + p].y * G[k * SG + p].y;
      const double lkk = sqrt(d), inv = 1.0 / lkk;
      G[k * SG + k] = make_double2(lkk, 0.0);
      for (int i = k + 1; i < nw; ++i) {
        double2 sm = G[i * SG + k];
        for (int p = 0; p < k; ++p) {  // -= L_ip conj(L_kp)
          const double2 u = G[i * SG + p], v = G[k * SG + p];
          sm.x -= u.x * v.x + u.y * v.y;
          sm.y -= u.y * v.x - u.x * v.y;
        }
        G[i * SG + k] = make_double2(sm.x * inv, sm.y * inv);
      }
    }
    // X = L^-1 in place, row by row: X_ij = -(sum_{k=j}^{i-1} L_ik X_kj) / L_ii
    // reads L_ik only for k >= j, so entry j of row i can be overwritten
    for (int i = 0; i < nw; ++i) {
      const double inv = 1.0 / G[i * SG + i].x;
      for (int j = 0; j < i; ++j) {
        double2 sm = make_double2(0.0, 0.0);
        for (int k = j; k < i; ++k) {
          const double2 u = G[i * SG + k], v = G[k * SG + j];
          sm.x += u.x * v.x - u.y * v.y;
          sm.y += u.x * v.y + u.y * v.x;
        }
        G[i * SG + j] = make_double2(-sm.x * inv, -sm.y * inv);
      }
      G[i * SG + i] = make_double2(inv, 0.0);
    }
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < nw * nw) {  // T = M X^H
    const int p = t / nw, j = t % nw;
    double2 sm = make_double2(0.0, 0.0);
    for (int q = 0; q <= j; ++q) {
      const double2 u = M[p * kPolCap + q], v = G[j * SG + q];
      sm.x += u.x * v.x + u.y * v.y;
      sm.y += u.y * v.x - u.x * v.y;
    }
    T[p * SG + j] = sm;
  }
  __syncthreads();
  if (t < nw * nw) {  // M = X T
    const int i = t / nw, j = t % nw;
    double2 sm = make_double2(0.0, 0.0);
    for (int p = 0; p <= i; ++p) {
      const double2 u = G[i * SG + p], v = T[p * SG + j];
      sm.x += u.x * v.x - u.y * v.y;
      sm.y += u.x * v.y + u.y * v.x;
    }
    M[i * kPolCap + j] = sm;
  }
  __syncthreads();
}

// eigenvectors U of the projected matrix (Z, row stride kPolCap) -> block
// coefficients C = X^H U, so that the Ritz vectors are B C
__device__ void rr_back(int nw, const double2* G, double2* Z, double2* T) {
  constexpr int SG = kMaxNev;
  const int t = threadIdx.x;
  if (t < nw * nw) {
    const int i = t / nw, c = t % nw;
    double2 sm = make_double2(0.0, 0.0);
    for (int k = i; k < nw; ++k) {  // conj(X_ki) U_kc
      const double2 u = G[k * SG + i], v = Z[k * kPolCap + c];
      sm.x += u.x * v.x + u.y * v.y;
      sm.y += u.x * v.y - u.y * v.x;
    }
    T[i * SG + c] = sm;
  }
  __syncthreads();
  if (t < nw * nw) Z[(t / nw) * kPolCap + t % nw] = T[(t / nw) * SG + t % nw];
  __syncthreads();
}

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
  double* s_theta = reinterpret_cast<double*>(smem + L.theta);  // Lanczos Ritz values
  double* s_lam = s_theta + kMaxM;                                // FP64 Rayleigh-Ritz values
  double* s_arrow = s_theta + 2 * kMaxM;                          // restart arrow column
  double2* s_coef = reinterpret_cast<double2*>(smem + L.coef);
  double* s_red = reinterpret_cast<double*>(smem + L.red);
  double* s_isr = reinterpret_cast<double*>(smem + L.isr);
  double* s_sqrt = s_isr + 65;
  float* s_isrf = reinterpret_cast<float*>(s_isr + 130);
  float* s_sqrtf = s_isrf + 65;
  float2* s_zdf = reinterpret_cast<float2*>(smem + L.zdf);
  float4* s_cdf = reinterpret_cast<float4*>(smem + L.cdf);
  double* s_misc = reinterpret_cast<double*>(smem + L.misc);
  uint32_t* s_rank = reinterpret_cast<uint32_t*>(smem + L.rank);
  uint32_t* s_rec = reinterpret_cast<uint32_t*>(smem + L.rec);
  uint16_t* s_off = reinterpret_cast<uint16_t*>(smem + L.off);
  uint8_t* s_inv = reinterpret_cast<uint8_t*>(smem + L.inv);
  uint8_t* s_perm = reinterpret_cast<uint8_t*>(smem + L.perm);
  double2* s_pw64 = reinterpret_cast<double2*>(smem + L.pw64);
  float2* s_pw32 = reinterpret_cast<float2*>(smem + L.pw32);
  uint64_t* s_mask = reinterpret_cast<uint64_t*>(smem + L.mask);
  double2* s_basek = reinterpret_cast<double2*>(smem + L.basek);
  V* s_pwc = reinterpret_cast<V*>(smem + L.pwc);
  float2* s_sq_df = reinterpret_cast<float2*>(smem + L.dfc);
  float2* s_isr_df = s_sq_df + 65;
  float4* s_zc = reinterpret_cast<float4*>(smem + L.zc);
  int* s_int = reinterpret_cast<int*>(s_misc + 48);

  for (int i = threadIdx.x; i < a.rp.total; i += blockDim.x) s_rank[i] = a.rank_tab[i];
  for (int i = threadIdx.x; i < a.n_terms; i += blockDim.x) s_rec[i] = a.rec[i];
  for (int i = threadIdx.x; i <= a.N; i += blockDim.x) s_off[i] = a.site_off[i];
  for (int i = threadIdx.x; i < a.G; i += blockDim.x) s_inv[i] = a.inv[i];
  for (int i = threadIdx.x; i < a.G * 64; i += blockDim.x) s_perm[i] = a.perm_g[i];
  for (int i = threadIdx.x; i < 65; i += blockDim.x) {
    s_isr[i] = i ? 1.0 / sqrt((double)i) : 0.0;
    s_sqrt[i] = sqrt((double)i);
    s_isrf[i] = (float)s_isr[i];
    s_sqrtf[i] = (float)s_sqrt[i];
    d_to_df(s_sqrt[i], s_sq_df[i].x, s_sq_df[i].y);
    d_to_df(s_isr[i], s_isr_df[i].x, s_isr_df[i].y);
  }

  // Lanczos basis, restart buffer and work vector: complex64 in the mixed
  // kernel, double-float in the FP64 kernel (each buffer holds 16 bytes per
  // element either way).  The basis and restart buffers have the same
  // capacity and trade places at every restart, so the rotated vectors are
  // never copied back.
  using BV = typename std::conditional<sizeof(typename P::S) == 4, float2, float4>::type;
  const size_t slots = (size_t)max(a.m + 1, 5 * (a.nev + 2));
  BV* Vb = reinterpret_cast<BV*>(a.V + (size_t)blockIdx.x * slots * a.ld);
  BV* Rb = reinterpret_cast<BV*>(a.R + (size_t)blockIdx.x * slots * a.ld);
  BV* W = reinterpret_cast<BV*>(a.W + (size_t)blockIdx.x * a.ld);
  double2* X64 = a.X64 + (size_t)blockIdx.x * a.ld;
  double2* tchi64 = a.tchi64 + (size_t)blockIdx.x * a.tchi_n;
  uint8_t* rowflag = a.rowflag + (size_t)blockIdx.x * a.ld;
  double2* pwc64 = a.pwc64 ? a.pwc64 + (size_t)blockIdx.x * a.phi_cap : nullptr;
  V* x = X_SMEM ? s_x : reinterpret_cast<V*>(X64);

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      long long qv = -1;
      if (a.ring_tail) {
        for (int it = 0; it < a.ring_spin;) {
          const unsigned int head = *reinterpret_cast<volatile unsigned int*>(a.queue);
          const unsigned int tail = *reinterpret_cast<const volatile unsigned int*>(a.ring_tail);
          if (head < tail) {
            if (atomicCAS(a.queue, head, head + 1u) == head) {
              qv = head;
              break;
            }
            continue;  // another block took it: look again at once
          }
          if (*reinterpret_cast<const volatile int*>(a.ring_stop)) break;
          __nanosleep(20000);
          ++it;
        }
      } else {
        qv = atomicAdd(a.queue, 1u);
      }
      s_int[0] = (int)(qv < 0 ? -1 : (qv & 0x7FFFFFFF));
      s_int[24] = (int)(qv < 0 ? 0 : (unsigned int)qv);
    }
    __syncthreads();
    const int q = s_int[0];
    if (q < 0 || (!a.ring_tail && q >= a.n_req)) break;
    const unsigned int q_seq = (unsigned int)s_int[24];
    const int b = a.ring_tail ? (int)(q_seq % (unsigned int)a.ring_cap) : a.req_list ? a.req_list[q] : q;
    if (threadIdx.x == 0 && !a.req_list) a.t_ns[2 * (size_t)b] = global_ns();
    const double2* chi = a.chi + (size_t)b * a.G;
    const double2* phase = a.phase + (size_t)b * a.G * a.N;
    const double2* amp = a.amp + (size_t)b * a.n_bil;
    // ---- set-up: tables for this momentum / twist
    for (int i = threadIdx.x; i < a.G; i += blockDim.x) s_chi[i] = ld_in(chi + i);
    // phase classes of every twisted group element (see sed_rowgather.cuh)
    if (threadIdx.x == 0) s_int[1] = 1;
    __syncthreads();
    for (int h = threadIdx.x; h < a.G; h += blockDim.x) {
      const double2* ph = phase + (size_t)h * a.N;
      double2 val[kMaxCls + 1];
      uint64_t msk[kMaxCls + 1];
      int nv = 0;
      bool over = false;
      for (int j = 0; j < a.N; ++j) {
        const double2 e = ld_in(ph + j);
        int c = 0;
        while (c < nv && !(val[c].x == e.x && val[c].y == e.y)) ++c;
        if (c == nv) {
          if (nv == kMaxCls + 1) {
            over = true;
            break;
          }
          val[nv] = e;
          msk[nv] = 0;
          ++nv;
        }
        msk[c] |= 1ULL << j;
      }
      if (over) {
        s_int[1] = 2;  // per-site product for this request
        continue;
      }
      int bc = 0;
      for (int c = 1; c < nv; ++c)
        if (__popcll(msk[c]) > __popcll(msk[bc])) bc = c;
      const double2 base = val[bc];
      double2 bk = make_double2(1.0, 0.0);
      for (int e = 0; e + 1 < a.kp1; ++e) bk = make_double2(bk.x * base.x - bk.y * base.y, bk.x * base.y + bk.y * base.x);
      s_basek[h] = bk;
      const double bn = base.x * base.x + base.y * base.y;
      int slot = 0;
      for (int c = 0; c < nv; ++c) {
        if (c == bc) continue;
        // r = v / base
        const double2 r = make_double2((val[c].x * base.x + val[c].y * base.y) / bn,
                                       (val[c].y * base.x - val[c].x * base.y) / bn);
        s_mask[h * kMaxCls + slot] = msk[c];
        double2 pw = make_double2(1.0, 0.0);
        for (int e = 0; e < a.kp1; ++e) {
          s_pw64[(h * kMaxCls + slot) * a.kp1 + e] = pw;
          s_pw32[(h * kMaxCls + slot) * a.kp1 + e] = make_float2((float)pw.x, (float)pw.y);
          pw = make_double2(pw.x * r.x - pw.y * r.y, pw.x * r.y + pw.y * r.x);
        }
        ++slot;
      }
      for (; slot < kMaxCls; ++slot) {
        s_mask[h * kMaxCls + slot] = 0;
        for (int e = 0; e < a.kp1; ++e) {
          s_pw64[(h * kMaxCls + slot) * a.kp1 + e] = make_double2(e == 0 ? 1.0 : 0.0, 0.0);
          s_pw32[(h * kMaxCls + slot) * a.kp1 + e] = make_float2(e == 0 ? 1.f : 0.f, 0.f);
        }
      }
    }
    __syncthreads();
    if (a.use_tab && a.gauge) {
      // gauge mode: no per-site phase product (base 1); phase ids 0 and 1
      // are the signs +1 and -1, entry 2 the zero of the padding records
      for (int h = threadIdx.x; h < a.G; h += blockDim.x) s_basek[h] = make_double2(1.0, 0.0);
      for (int f = threadIdx.x; f <= 2; f += blockDim.x) {
        const double p = f == 0 ? 1.0 : (f == 1 ? -1.0 : 0.0);
        reinterpret_cast<float4*>(pwc64)[f] = make_float4((float)p, 0.f, 0.f, 0.f);
        s_pwc[f].x = p;
        s_pwc[f].y = 0.0;
      }
    } else if (a.use_tab) {
      // family phase classes of the hop table: this request's phase on each
      // class (read at the class's first site; constant on the class by
      // construction), P_h(new) = v0^k prod_c (v_c / v0)^(n_c)
      for (int h = threadIdx.x; h < a.G; h += blockDim.x) {
        const double2* ph = phase + (size_t)h * a.N;
        const int8_t* rs = a.rep_site + h * 4;
        const double2 v0 = ph[rs[0]];
        double2 bk = make_double2(1.0, 0.0);
        for (int e = 0; e + 1 < a.kp1; ++e) bk = make_double2(bk.x * v0.x - bk.y * v0.y, bk.x * v0.y + bk.y * v0.x);
        s_basek[h] = bk;
        const double bn = v0.x * v0.x + v0.y * v0.y;
        for (int c = 0; c < kMaxCls; ++c) {
          double2 r = make_double2(1.0, 0.0);
          if (rs[c + 1] >= 0) {
            const double2 v = ph[rs[c + 1]];
            r = make_double2((v.x * v0.x + v.y * v0.y) / bn, (v.y * v0.x - v.x * v0.y) / bn);
          }
          double2 pw = make_double2(1.0, 0.0);
          for (int e = 0; e < a.kp1; ++e) {
            s_pw64[(h * kMaxCls + c) * a.kp1 + e] = pw;
            pw = make_double2(pw.x * r.x - pw.y * r.y, pw.x * r.y + pw.y * r.x);
          }
        }
      }
      __syncthreads();
      // phase-id coefficients: +-conj(prod_c r_c^(n_c)); entry n_phi is the
      // zero coefficient of the padding records
      for (int f = threadIdx.x; f <= a.n_phi; f += blockDim.x) {
        double2 p = make_double2(0.0, 0.0);
        if (f < a.n_phi) {
          const uint32_t d = a.phi_desc[f];
          const int h = d & 0x3F, n1 = (d >> 6) & 0x3F, n2 = (d >> 12) & 0x3F, n3 = (d >> 18) & 0x3F;
          const double2* pw = s_pw64 + (size_t)h * kMaxCls * a.kp1;
          const double2 p1 = pw[n1], p2 = pw[a.kp1 + n2], p3 = pw[2 * a.kp1 + n3];
          const double2 q = make_double2(p1.x * p2.x - p1.y * p2.y, p1.x * p2.y + p1.y * p2.x);
          p = make_double2(q.x * p3.x - q.y * p3.y, -(q.x * p3.y + q.y * p3.x));
          if ((d >> 24) & 1) p = make_double2(-p.x, -p.y);
        }
        // the polish reads double-float pairs (re_hi, im_hi, re_lo, im_lo)
        float4 pd;
        d_to_df(p.x, pd.x, pd.z);
        d_to_df(p.y, pd.y, pd.w);
        reinterpret_cast<float4*>(pwc64)[f] = pd;
        s_pwc[f].x = p.x;
        s_pwc[f].y = p.y;
      }
    }
    __syncthreads();
    const int pmode = s_int[1];
    if (pmode == 2 && !a.use_tab)
      for (int h = threadIdx.x; h < a.G; h += blockDim.x) s_basek[h] = make_double2(1.0, 0.0);
    __syncthreads();
    const double2* gw = (a.use_tab && a.gauge) ? a.gauge_w + (size_t)b * a.N : nullptr;
    for (int i = threadIdx.x; i <= a.n_bil * a.G; i += blockDim.x) {
      const int k = i / a.G, h = i % a.G;
      double2 v = make_double2(0.0, 0.0);  // entry n_bil * G: the padding records' zero
      if (i < a.n_bil * a.G) {
        double2 t = ld_in(amp + k);
        if (gw) {  // the hop i -> j in the site gauge: t w_j conj(w_i)
          const double2 wi = ld_in(gw + a.bil_dev[2 * k]), wj = ld_in(gw + a.bil_dev[2 * k + 1]);
          const double2 q = make_double2(wj.x * wi.x + wj.y * wi.y, wj.y * wi.x - wj.x * wi.y);
          t = make_double2(t.x * q.x - t.y * q.y, t.x * q.y + t.y * q.x);
        }
        const double2 c0 = s_chi[h], bk = s_basek[h];
        const double2 c = make_double2(c0.x * bk.x + c0.y * bk.y, c0.y * bk.x - c0.x * bk.y);  // chi conj(base^k)
        v = make_double2(t.x * c.x + t.y * c.y, t.x * c.y - t.y * c.x);                       // conj(t) chi'
      }
      const int pos = a.use_tab ? (int)((uint64_t)i * (uint64_t)a.tchi_mul % (uint64_t)a.tchi_n) : i;
      if (a.use_tab) {  // double-float pairs for the table-path polish
        float4 vd;
        d_to_df(v.x, vd.x, vd.z);
        d_to_df(v.y, vd.y, vd.w);
        reinterpret_cast<float4*>(tchi64)[pos] = vd;
      } else {
        tchi64[pos] = v;
      }
      s_tchi[pos].x = v.x;
      s_tchi[pos].y = v.y;
    }
    const PhaseClasses<V> pcl{pmode, a.kp1, s_mask, reinterpret_cast<const V*>(sizeof(V) == 8 ? (void*)s_pw32 : (void*)s_pw64)};
    const PhaseClasses<double2> pcl64{pmode, a.kp1, s_mask, s_pw64};
    for (int i = threadIdx.x; i < a.G * a.N; i += blockDim.x) {
      const double2 e = ld_in(phase + i);
      s_eta[i].x = e.x;
      s_eta[i].y = e.y;
    }
    __syncthreads();
    // ---- sector membership (SRE:534-542) and the hop count of one matvec
    double cnt = 0.0, hcnt = 0.0;
    for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
      const uint64_t m = a.reps[o];
      int ok = 1;
      for (int g = 0; g < a.G; ++g) {
        // the phase product (FP64) only for stabilizer elements
        if (dev::apply_perm(m, s_perm + g * 64) != m) continue;
        double2 al;
        dev::apply_full(m, s_perm + g * 64, phase + (size_t)g * a.N, FERMI ? 1 : 0, &al);
        const double2 xg = s_chi[g];
        if (!((xg.x == al.x && xg.y == al.y) || hypot(xg.x - al.x, xg.y - al.y) <= a.atol)) ok = 0;
      }
      rowflag[o] = (uint8_t)ok;
      cnt += ok;
      if (ok) hcnt += (double)count_row_hops(m, s_off, s_rec);
    }
    double sums[2] = {cnt, hcnt};
    block_sum<2>(sums, s_red, s_misc);
    const int64_t dim = (int64_t)s_misc[0];
    if (threadIdx.x == 0) a.hops[b] = (int64_t)s_misc[1];
    // mixed precision carries two spare Ritz pairs into the FP64 polish;
    // convergence is judged on the requested pairs only
    const int nev_out = (int)min((int64_t)a.nev, dim);
    const int nev = (int)min((int64_t)(sizeof(typename P::S) == 4 ? a.nev + 2 : a.nev), dim);
    const int m = (int)min((int64_t)a.m, dim);
    if (threadIdx.x == 0) a.dims[b] = dim;
    if (dim == 0) {
      if (threadIdx.x == 0) {
        a.status[b] = 0;
        a.nmv[b] = 0;
        a.delta[b] = 0.0;
        for (int i = 0; i < a.nev; ++i) a.evals[(size_t)b * a.nev + i] = nan("");
        a.t_ns[2 * (size_t)b + 1] = global_ns();
        if (a.ring_done) {
          __threadfence_system();
          *reinterpret_cast<volatile unsigned int*>(a.ring_done + b) = q_seq + 1u;
        }
      }
      continue;
    }
    // ---- start vector (same generator as the single-sector path)
    double nrm = 0.0;
    const uint64_t seed = __ldcg(a.seeds + b);
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
      store_row(W, o, v.x, v.y);
      nrm += v.x * v.x + v.y * v.y;
    }
    nrm = block_sum1(nrm, s_red, s_misc);
    lz_normalize<V>(a, W, 1.0 / sqrt(nrm), Vb, x, s_sqrtf, s_sqrt);
    for (int i = threadIdx.x; i < kMaxM * kMaxM; i += blockDim.x) s_T[i] = 0.0;
    __syncthreads();

    int k = 0, restarts = 0, nmv = 0, n64 = 0, status = 0;
    // where the returned eigenvectors end up: 0 the Ritz vectors in Vb (FP64
    // kernel), 1 the polished double-float block in the restart buffer (hop
    // table), 2 the polished FP64 block there (on-the-fly gather)
    int vec_src = 0, vec_nw = 0;
    double beta = 0.0, prev_res = 1e300, best_prev = 1e300, dmax = 0.0;
    double tau = 1e-6;  // mixed: relative Ritz-estimate threshold of the complex64 run
    const bool mixed = sizeof(typename P::S) == 4;
    for (;;) {
      int jend = m;
      for (int j = k; j < m; ++j) {
        BV* vj = Vb + (size_t)j * a.ld;
        if (a.use_tab)
          block_matvec_tab_any<P>(a, x, s_tchi, s_pwc, s_isr, s_isrf, rowflag, W);
        else
          block_matvec<P, FERMI, PHASES>(a, x, s_tchi, s_eta, s_isr, s_isrf, s_rank, s_rec, s_off, s_inv, rowflag, W,
                                         pcl);
        __syncthreads();
        ++nmv;
        // local step: CGS against the two newest basis vectors (they carry
        // the large alpha_j, beta_{j-1} components), then one full CGS pass;
        // a second full pass only when the first removed more than half of
        // the norm (Daniel-Gragg-Kaufman-Stewart).
        const int l0 = j > 0 ? j - 1 : 0;
        lz_dots(a, Vb + (size_t)l0 * a.ld, j + 1 - l0, W, s_red, s_coef);
        df_coefs(s_coef, j + 1 - l0, s_cdf);
        double alpha = s_coef[j - l0].x;
        // the local update rides on the first chunk of the full pass's dots
        const int c0n = min(7, j + 1);
        const double n0 = lz_dots_local(a, Vb, c0n, Vb + (size_t)l0 * a.ld, j + 1 - l0, s_cdf, W, s_red,
                                        s_coef + kMaxM + 8);
        if (j + 1 > c0n) lz_dots(a, Vb + (size_t)c0n * a.ld, j + 1 - c0n, W, s_red, s_coef + kMaxM + 8 + c0n);
        // mixed precision: update only when the measured loss of orthogonality
        // exceeds kSelReorth (the test is uniform over the block)
        double cmax = 0.0;
        if (mixed)
          for (int i = 0; i <= j; ++i) {
            const double2 c = s_coef[kMaxM + 8 + i];
            cmax = fmax(cmax, fabs(c.x) + fabs(c.y));
          }
        double nf = n0;
        if (!mixed || cmax > kSelReorth * sqrt(n0)) {
          df_coefs(s_coef + kMaxM + 8, j + 1, s_cdf);
          double n1 = lz_axpy(a, Vb, j + 1, s_cdf, W);
          alpha += s_coef[kMaxM + 8 + j].x;
          __syncthreads();
          n1 = block_sum1(n1, s_red, s_misc + 1);
          nf = n1;
          if (n1 < 0.5 * n0) {
            lz_dots(a, Vb, j + 1, W, s_red, s_coef + kMaxM + 8);
            df_coefs(s_coef + kMaxM + 8, j + 1, s_cdf);
            double n2 = lz_axpy(a, Vb, j + 1, s_cdf, W);
            alpha += s_coef[kMaxM + 8 + j].x;
            __syncthreads();
            nf = block_sum1(n2, s_red, s_misc + 2);
          }
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
        lz_normalize<V>(a, W, 1.0 / beta, vj + a.ld, x, s_sqrtf, s_sqrt);
        __syncthreads();
        (void)vj;
      }
      __syncthreads();
      const int msz = jend;
      // ---- Ritz values of the projected matrix (warp 0): Jacobi works on a
      // copy of T in s_Z and leaves the eigenvectors in s_T
      for (int i = threadIdx.x; i < kMaxM * kMaxM; i += blockDim.x) s_Z[i] = s_T[i];
      __syncthreads();
      block_jacobi(msz, s_Z, s_T, s_theta, reinterpret_cast<double*>(s_coef), s_red, s_misc + 40);
      // now s_T holds eigenvectors (columns), s_Z the diagonalised matrix
      const bool invariant = msz < m || (int64_t)msz == dim;
      double scale = 1.0;
      for (int i = 0; i < min(nev, msz); ++i) scale = fmax(scale, fabs(s_theta[i]));
      const double tol_w = mixed ? fmax(a.tol, tau * scale) : a.tol;
      int nconv = 0;
      double maxr = 0.0;
      for (int i = 0; i < min(nev_out, msz); ++i) {
        const double r = invariant ? 0.0 : fabs(beta * s_T[(msz - 1) * kMaxM + i]);
        maxr = fmax(maxr, r);
        if (r <= tol_w) ++nconv;
      }
      // FP32 noise floor: stop once the residual sits near it and no longer improves
      bool stagnated = mixed && restarts >= 6 && maxr < 5e-5 * scale && maxr > 0.7 * best_prev;
      best_prev = prev_res;
      prev_res = fmin(prev_res, maxr);
      const bool done = nconv >= nev_out || invariant || stagnated || restarts >= a.maxiter;
      // a mixed-precision candidate keeps the full restart basis, so the
      // iteration can resume if the FP64 check rejects it
      const bool final_rot = done && (!mixed || invariant);
      // thick restart: the mixed kernel keeps nev + 2 Ritz vectors (its nev
      // already carries two spare pairs), the FP64 kernel half of the rest as
      // well.  Fewer kept vectors shorten the rotation and every later dot
      // sweep; on the flux-scan batch keeping 8 of 24 instead of 15 cost 2 %
      // more matvecs and gave 2580 against 2167 sector solves/s, with no
      // fallback (18 kept: one FP64 fallback)
      const int keep = final_rot ? min(nev, msz)
                                 : min(msz - 1, mixed ? nev + 2 : max(nev + (m - nev) / 2, nev + 1));
      if (threadIdx.x < keep) s_arrow[threadIdx.x] = beta * s_T[(msz - 1) * kMaxM + threadIdx.x];
      // Lanczos residual of the first Ritz value after the polish block (the
      // lower end of its inclusion interval bounds the gap in the check below)
      if (threadIdx.x == 0) {
        const int nwb = min(nev, msz);
        s_misc[20] = (msz > nwb && !invariant) ? fabs(beta * s_T[(msz - 1) * kMaxM + nwb]) : 0.0;
      }
      for (int i = threadIdx.x; i < msz * keep; i += blockDim.x) {
        const int q = i / keep, c = i % keep;
        float2 z;
        d_to_df(s_T[q * kMaxM + c], z.x, z.y);
        s_zdf[q * kMaxM + c] = z;
      }
      __syncthreads();
      lz_rotate(a, Vb, msz, s_zdf, keep, Rb);
      if (!final_rot)  // the last normalised residual direction continues the basis
        for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x)
          Rb[(size_t)keep * a.ld + o] = Vb[(size_t)m * a.ld + o];
      __syncthreads();
      {
        BV* t = Vb;
        Vb = Rb;
        Rb = t;
      }
      if (done && !mixed) {
        status = (nconv >= nev_out || invariant || stagnated) ? 0 : SED_ERR_NOT_CONVERGED;
        break;
      }
      if (done) {
        // FP64 check of the complex64 candidate: one Rayleigh-Ritz step with
        // FP64 matvecs over its nev + 2 Ritz vectors B = Vb[0..nw), the block
        // orthonormalised through its Gram matrix (rr_orthonormalise); accepted
        // when every requested pair meets the residual tolerance or the
        // quadratic bound |dE| <= |r|^2 / gap (gap to the lower end of the
        // first Lanczos Ritz interval outside the block) is below
        // kMixedRelTarget |E|.  Otherwise
        // the Lanczos resumes with a tighter threshold; a stagnated run is
        // re-solved by the FP64 kernel (status kPolishFailed).
        const int nw = min(nev, msz);
        double2* M = reinterpret_cast<double2*>(s_Z);  // kPolCap^2 complex fit in kMaxM^2 doubles
        double2* Gm = M + kPolCap * kMaxNev;           // Gram matrix, then L^-1 (stride kMaxNev)
        double2* Tm = Gm + kMaxNev * kMaxNev;          // scratch
        double2* Zc = reinterpret_cast<double2*>(s_T);
        double rr[kMaxNev];
#pragma unroll
        for (int i = 0; i < kMaxNev; ++i) rr[i] = 0.0;
        if (a.use_tab) {
          // double-float polish: B = the Ritz block Vb[0..nw) in
          // double-float (Bd), H B through the hop table with double-float
          // coefficients, Rayleigh-Ritz and the FP64-class residuals of the
          // rotated pairs.  The free restart buffer holds HB, Yr, HYr and Bd
          // (4 nw <= slots double-float vectors).
          float4* R4 = reinterpret_cast<float4*>(Rb);
          float4* HB = R4;
          float4* Yr = R4 + (size_t)nw * a.ld;
          float4* HYr = R4 + (size_t)(2 * nw) * a.ld;
          float4* Bd = R4 + (size_t)(3 * nw) * a.ld;
          float4* Xd = reinterpret_cast<float4*>(X64);
          for (int i = 0; i < nw; ++i)
            for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x)
              Bd[(size_t)i * a.ld + o] = lz_to_df(Vb[(size_t)i * a.ld + o]);
          __syncthreads();
          for (int i = 0; i < nw; ++i) {
            df_scale_xs(a, Bd + (size_t)i * a.ld, Xd, s_sq_df);
            __syncthreads();
            block_matvec_tab_df(a, Xd, reinterpret_cast<const float4*>(tchi64),
                                reinterpret_cast<const float4*>(pwc64), s_isr_df, rowflag, HB + (size_t)i * a.ld);
            __syncthreads();
          }
          n64 += nw;
          for (int bcol = 0; bcol < nw; ++bcol) {
            df_dots(a, Bd, nw, HB + (size_t)bcol * a.ld, s_red, s_coef);
            if (threadIdx.x < nw) M[threadIdx.x * kPolCap + bcol] = s_coef[threadIdx.x];
            __syncthreads();
            df_dots(a, Bd, nw, Bd + (size_t)bcol * a.ld, s_red, s_coef);
            if (threadIdx.x < nw) Gm[threadIdx.x * kMaxNev + bcol] = s_coef[threadIdx.x];
            __syncthreads();
          }
          rr_orthonormalise(nw, M, Gm, Tm);
          if (threadIdx.x == 0)
            for (int i = 0; i < nw; ++i)
              for (int j = i; j < nw; ++j) {
                const double re = 0.5 * (M[i * kPolCap + j].x + M[j * kPolCap + i].x);
                const double im = 0.5 * (M[i * kPolCap + j].y - M[j * kPolCap + i].y);
                M[i * kPolCap + j] = make_double2(re, im);
                M[j * kPolCap + i] = make_double2(re, -im);
              }
          __syncthreads();
          if (threadIdx.x < 32) warp_jacobi_herm(nw, M, Zc, s_lam);
          __syncthreads();
          rr_back(nw, Gm, Zc, Tm);
          if (threadIdx.x < nw * nw) {
            const int l = threadIdx.x / nw, c = threadIdx.x % nw;
            const double2 z = Zc[l * kPolCap + c];
            float4 t;
            d_to_df(z.x, t.x, t.z);
            d_to_df(z.y, t.y, t.w);
            s_zc[l * kMaxNev + c] = t;
          }
          __syncthreads();
          df_rotate_c(a, Bd, nw, s_zc, nw, Yr);
          df_rotate_c(a, HB, nw, s_zc, nw, HYr);
          __syncthreads();
          float2 lam[kMaxNev];
#pragma unroll
          for (int i = 0; i < kMaxNev; ++i) lam[i] = make_float2(0.f, 0.f);
          for (int i = 0; i < nev_out; ++i) d_to_df(s_lam[i], lam[i].x, lam[i].y);
          for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x)
            for (int i = 0; i < nev_out; ++i) {
              float4 hy = HYr[(size_t)i * a.ld + o];
              const float4 y = Yr[(size_t)i * a.ld + o];
              df_mac(hy.x, hy.z, -lam[i].x, -lam[i].y, y.x, y.z);
              df_mac(hy.y, hy.w, -lam[i].x, -lam[i].y, y.y, y.w);
              float nh = 0.f, nl = 0.f;
              df_mac(nh, nl, hy.x, hy.z, hy.x, hy.z);
              df_mac(nh, nl, hy.y, hy.w, hy.y, hy.w);
              rr[i] += df_to_d(nh, nl);
            }
        } else {
          double2* Rb64 = reinterpret_cast<double2*>(Rb);  // the FP64 polish reuses the restart buffer
          double2* HB = Rb64;
          double2* Yr = Rb64 + (size_t)nw * a.ld;
          double2* HYr = Rb64 + (size_t)(2 * nw) * a.ld;
          double2* B64 = Rb64 + (size_t)(3 * nw) * a.ld;  // the Ritz vectors in FP64
          for (int i = 0; i < nw; ++i)
            for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
              B64[(size_t)i * a.ld + o] = lz_to_d(Vb[(size_t)i * a.ld + o]);
            }
          __syncthreads();
          for (int i = 0; i < nw; ++i) {
            block_normalize<double2>(a, B64 + (size_t)i * a.ld, 1.0, nullptr, X64, s_sqrt);
            __syncthreads();
            block_matvec<P64, FERMI, PHASES>(a, X64, tchi64, phase, s_isr, s_isrf, s_rank, s_rec, s_off, s_inv,
                                             rowflag, HB + (size_t)i * a.ld, pcl64);
            __syncthreads();
          }
          n64 += nw;
          for (int bcol = 0; bcol < nw; ++bcol) {
            block_dots(a, B64, nw, HB + (size_t)bcol * a.ld, s_red, s_coef);
            if (threadIdx.x < nw) M[threadIdx.x * kPolCap + bcol] = s_coef[threadIdx.x];
            __syncthreads();
            block_dots(a, B64, nw, B64 + (size_t)bcol * a.ld, s_red, s_coef);
            if (threadIdx.x < nw) Gm[threadIdx.x * kMaxNev + bcol] = s_coef[threadIdx.x];
            __syncthreads();
          }
          rr_orthonormalise(nw, M, Gm, Tm);
          if (threadIdx.x == 0)
            for (int i = 0; i < nw; ++i)
              for (int j = i; j < nw; ++j) {
                const double re = 0.5 * (M[i * kPolCap + j].x + M[j * kPolCap + i].x);
                const double im = 0.5 * (M[i * kPolCap + j].y - M[j * kPolCap + i].y);
                M[i * kPolCap + j] = make_double2(re, im);
                M[j * kPolCap + i] = make_double2(re, -im);
              }
          __syncthreads();
          if (threadIdx.x < 32) warp_jacobi_herm(nw, M, Zc, s_lam);
          __syncthreads();
          rr_back(nw, Gm, Zc, Tm);
          block_rotate_c(a, B64, nw, Zc, nw, Yr);
          block_rotate_c(a, HB, nw, Zc, nw, HYr);
          for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x)
            for (int i = 0; i < nev_out; ++i) {
              const double2 hy = HYr[(size_t)i * a.ld + o], y = Yr[(size_t)i * a.ld + o];
              const double rx = hy.x - s_lam[i] * y.x, ry = hy.y - s_lam[i] * y.y;
              rr[i] += rx * rx + ry * ry;
            }
        }
        block_sum<kMaxNev>(rr, s_red, s_misc + 8);
        // every requested pair must pass mixed_pair_accepted: isolated, and
        // the quadratic bound with the gap to the lower end theta_L - r_L of
        // the first Lanczos Ritz interval above the block
        const double thL = msz > nw ? s_theta[nw] - s_misc[20] : HUGE_VAL;
        bool ok = true;
        dmax = 0.0;
        for (int i = 0; i < nev_out; ++i) {
          dmax = fmax(dmax, fabs(s_lam[i] - s_theta[i]));
          ok = ok && mixed_pair_accepted(s_lam[i], s_misc[8 + i], thL, a.tol, scale);
        }
        __syncthreads();
        if (ok) {
          if (threadIdx.x < nw) s_theta[threadIdx.x] = s_lam[threadIdx.x];
          vec_src = a.use_tab ? 1 : 2;
          vec_nw = nw;
          __syncthreads();
          break;
        }
        if (invariant || stagnated || restarts >= a.maxiter || tau <= 1e-9) {
          status = kPolishFailed;  // the host re-solves this request in FP64
          break;
        }
        tau *= 0.1;
        if (!X_SMEM) {
          // the check used x's global buffer for its FP64-class vectors: the
          // Lanczos resumes from the continuation vector (slot keep), so its
          // scaled copy, as df_normalize wrote it, goes back into x
          const BV* vk = Vb + (size_t)keep * a.ld;
          for (int64_t o = threadIdx.x; o < a.n_orb; o += blockDim.x) {
            const BV v = vk[o];
            if (sizeof(V) == 8) {
              const float sq = s_sqrtf[a.stab[o]];
              reinterpret_cast<float2*>(x)[o] = make_float2(__fmul_rn(v.x, sq), __fmul_rn(v.y, sq));
            } else {
              const double sq = s_sqrt[a.stab[o]];
              const double2 d = lz_to_d(v);
              reinterpret_cast<double2*>(x)[o] = make_double2(d.x * sq, d.y * sq);
            }
          }
          __syncthreads();
        }
      }
      // arrowhead restart matrix
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int i = 0; i < kMaxM * kMaxM; ++i) s_T[i] = 0.0;
        for (int c = 0; c < keep; ++c) {
          s_T[c * kMaxM + c] = s_theta[c];
          s_T[c * kMaxM + keep] = s_T[keep * kMaxM + c] = s_arrow[c];
        }
      }
      __syncthreads();
      k = keep;
      ++restarts;
    }
    if (a.evecs && status != kPolishFailed) {
      double2* out = a.evecs + (size_t)b * a.nev * a.ev_ld;
      const double2* gwv = (a.use_tab && a.gauge) ? a.gauge_w + (size_t)b * a.N : nullptr;
      int* s_cnt = s_int + 2;
      if (vec_src == 0)
        block_write_vectors(a, Vb, a.ld, nev_out, rowflag, gwv, out, s_cnt);
      else if (vec_src == 1)
        block_write_vectors(a, reinterpret_cast<const float4*>(Rb) + (size_t)vec_nw * a.ld, a.ld, nev_out, rowflag,
                            gwv, out, s_cnt);
      else
        block_write_vectors(a, reinterpret_cast<const double2*>(Rb) + (size_t)vec_nw * a.ld, a.ld, nev_out,
                            rowflag, gwv, out, s_cnt);
    }
    if (threadIdx.x == 0) {
      for (int i = 0; i < a.nev; ++i) a.evals[(size_t)b * a.nev + i] = i < nev_out ? s_theta[i] : nan("");
      a.status[b] = status;
      a.nmv[b] = nmv + n64;
      a.delta[b] = dmax;
      a.t_ns[2 * (size_t)b + 1] = global_ns();
      if (a.ring_done) {
        __threadfence_system();
        *reinterpret_cast<volatile unsigned int*>(a.ring_done + b) = q_seq + 1u;
      }
    }
  }
}

// ------------------------------------------------------------------ host side
struct BatchImpl {
  std::shared_ptr<CatalogImpl> cat;
  int precision = 1, nev = 4, m = 30, max_req = 0, n_bil = 0, n_den = 0, n_cta = 1;
  int tchi_n = 1, tchi_mul = 1;  // coefficient table slots (prime) and hashing multiplier
  std::vector<int32_t> bil_ij, den_ij;
  std::vector<double> den_v;
  TermTables tt;
  DevBuf site_off, rec, diag, V, R, W, X64, tchi64, rowflag;
  DevBuf in_chi, in_phase, in_amp, in_seed, o_evals, o_status, o_dims, o_delta, o_nmv, o_hops, o_tns, queue;
  DevBuf o_evecs;  // device staging of the host eigenvector output
  int last_n = 0, n_fallback = 0;
  DevBuf redo;
  // hop table (built at the first run, rebuilt when the phase classes change)
  int phi_cap = 0;       // phase-id capacity of the shared-memory layout (0: no table)
  bool tab_valid = false;
  int n_phi = 0;
  std::vector<uint64_t> tab_fmask;  // [G][3] family class masks of the table
  std::vector<int8_t> tab_rep;      // [G][4] class representative sites
  std::vector<int32_t> row_cnt;     // hops per orbit row
  std::vector<uint32_t> h_sl_off;   // host copies of the slice offsets and widths
  std::vector<int32_t> h_sl_w;
  DevBuf hop, sl_off, sl_w, phi_desc, rep_site, pwc64, fmask_dev;
  int64_t hop_records = 0;
  // the table's records carry signs only (gauge mode) rather than phase ids
  bool tab_gauge = false;
  bool gauge_enabled = true;  // use gauge mode whenever every request allows it
  // launch shape: Krylov dimension and threads per row of the table matvec;
  // pinned (pin_m / pin_tpr > 0) or chosen by the autotuner per catalog shape
  bool m_fixed = false;
  int m_cap = 24, pin_m = 0, pin_tpr = 0, last_m = 0, last_tpr = 0;
  int tune_runs = 0;  // autotuner sweeps this batch object ran
  int last_gauge = 0;
  DevBuf gauge_w, bil_dev;  // [max_req][n_site] site gauges; [n_bil][2] term sites
  int last_tab = 0;
  bool tab_enabled = true;
  // complex64 matvec input in shared memory (else in global memory, for
  // sectors whose x does not fit beside the tables)
  bool x_smem = true;
  size_t smem = 0;
  int64_t ld = 0;
  size_t footprint = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool fermi = false;
  // ring mode (sed_batch_ring_*): one persistent launch fed from a request
  // ring; mapped host memory carries the published tail, the stop flag, the
  // done flags and every request's outputs, device memory the slots' inputs
  struct Ring {
    bool on = false;
    int cap = 0, n_cta = 0, spin = 0, fp64 = 0;
    unsigned int next = 0;  // the next request's sequence number
    int64_t launches = 0;
    unsigned int* tail = nullptr;  // mapped host allocations (host pointers)
    int* stop = nullptr;
    unsigned int* done = nullptr;
    double* evals = nullptr;
    int32_t* status = nullptr;
    int64_t* dims = nullptr;
    double* delta = nullptr;
    int32_t* nmv = nullptr;
    int64_t* hops = nullptr;
    int64_t* tns = nullptr;
    DevBuf chi, phase, amp, seed, gw, head;
    std::vector<char> busy;  // slot holds a request not yet collected
    cudaStream_t stream = nullptr, copy = nullptr;
    BatchArgs args{};
    BatchSmem L{};
    std::shared_ptr<BatchImpl> redo;  // FP64 batch for requests whose polish missed its target
  } ring;
  // start, submit, wait, info and stop may be called from different host
  // threads (one submitting, one collecting, one stopping): the host-side ring
  // state is guarded by ring_mu, which outlives every ring, and ring_gen counts
  // the rings started, so a waiter notices a stop (and a restart) between two
  // of its polls
  std::mutex ring_mu;
  uint64_t ring_gen = 0;
  // the captured launch (queue reset + persistent kernel) and the launch
  // configuration it was captured for
  std::vector<unsigned char> graph_key;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_captures = 0, graph_replays = 0;
  // the graph is recorded on a private stream: the caller's stream may be the
  // legacy default stream, which cannot be captured (the replay goes onto the
  // caller's stream, where it is ordered like a plain launch)
  cudaStream_t capture_stream = nullptr;
  void drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    graph_exec = nullptr;
    graph = nullptr;
    graph_key.clear();
  }
  void ring_free();
  ~BatchImpl() {
    ring_free();
    drop_graph();
    if (capture_stream) cudaStreamDestroy(capture_stream);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
};

// The shared-memory opt-in is a property of each kernel instantiation on each
// device, shared by every batch object (and host thread) that launches it: it
// is only ever raised, and raised-and-launched under one lock, so a concurrent
// batch with a smaller footprint cannot undercut a launch in progress.
template <class P, bool F, bool PH, bool XS>
struct KernelSmem {
  static std::mutex& mu() {
    static std::mutex m;
    return m;
  }
  static void ensure(size_t bytes) {
    static SmemOptIn optin;
    optin.ensure(k_batch<P, F, PH, XS>, bytes);
  }
};

template <class P, bool F, bool PH, bool XS>
static void batch_prepare(BatchImpl& B, const BatchArgs& a, BatchSmem& L, int& ncta) {
  auto kern = k_batch<P, F, PH, XS>;
  L = batch_layout<typename P::V>(a, XS);
  SED_REQUIRE(L.total <= 220 * 1024, 5, "batched solve tables exceed the shared-memory budget (sector too large)");
  using KS = KernelSmem<P, F, PH, XS>;
  std::lock_guard<std::mutex> lock(KS::mu());
  KS::ensure(L.total);
  int per_sm = 0;
  SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBT, L.total));
  SED_REQUIRE(per_sm >= 1, 5, "batched kernel cannot be resident with this shared-memory footprint");
  ncta = per_sm * device_sm_count();
}

template <class P, bool F, bool PH, bool XS>
static void batch_launch(const BatchArgs& a, const BatchSmem& L, int ncta, cudaStream_t s) {
  using KS = KernelSmem<P, F, PH, XS>;
  std::lock_guard<std::mutex> lock(KS::mu());
  KS::ensure(L.total);
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
  a.kp1 = C.n_filled + 1;
  a.phi_cap = B.phi_cap;
  a.bil_dev = B.bil_dev.as<int32_t>();
  a.tchi_n = B.tchi_n;
  a.tchi_mul = B.tchi_mul;
  return a;
}

static void dispatch_prepare(BatchImpl& B, const BatchArgs& a, BatchSmem& L, int& ncta, bool fp64) {
  const bool mixed = !fp64;
  // Each (precision, statistics) pair is compiled with the twisted-phase
  // product; untwisted requests multiply by exactly 1.
  if (mixed && B.x_smem) {
    if (B.fermi) batch_prepare<P32, true, true, true>(B, a, L, ncta);
    else batch_prepare<P32, false, true, true>(B, a, L, ncta);
  } else if (mixed) {
    if (B.fermi) batch_prepare<P32, true, true, false>(B, a, L, ncta);
    else batch_prepare<P32, false, true, false>(B, a, L, ncta);
  } else {
    if (B.fermi) batch_prepare<P64, true, true, false>(B, a, L, ncta);
    else batch_prepare<P64, false, true, false>(B, a, L, ncta);
  }
}

static void dispatch_launch(BatchImpl& B, const BatchArgs& a, const BatchSmem& L, int ncta, cudaStream_t s,
                            bool fp64) {
  if (!fp64 && B.x_smem) {
    if (B.fermi) batch_launch<P32, true, true, true>(a, L, ncta, s);
    else batch_launch<P32, false, true, true>(a, L, ncta, s);
  } else if (!fp64) {
    if (B.fermi) batch_launch<P32, true, true, false>(a, L, ncta, s);
    else batch_launch<P32, false, true, false>(a, L, ncta, s);
  } else {
    if (B.fermi) batch_launch<P64, true, true, false>(a, L, ncta, s);
    else batch_launch<P64, false, true, false>(a, L, ncta, s);
  }
}

// One batch launch -- the request-queue reset and the persistent kernel -- as
// a CUDA graph: captured the first time a launch configuration is seen
// (kernel arguments, shared-memory layout, grid, precision), replayed with
// cudaGraphLaunch while it repeats, as it does for every step of a flux scan
// or a serving lane.  Capture is thread-local, so host threads that allocate
// or launch on other streams meanwhile are not affected.
static void graph_launch(BatchImpl& B, const BatchArgs& a, const BatchSmem& L, int ncta, cudaStream_t s, bool fp64) {
  std::vector<unsigned char> key(sizeof(BatchArgs) + sizeof(BatchSmem) + 2 * sizeof(int));
  std::memcpy(key.data(), &a, sizeof(BatchArgs));
  std::memcpy(key.data() + sizeof(BatchArgs), &L, sizeof(BatchSmem));
  const int tail[2] = {ncta, fp64 ? 1 : 0};
  std::memcpy(key.data() + sizeof(BatchArgs) + sizeof(BatchSmem), tail, sizeof(tail));
  if (!B.graph_exec || key != B.graph_key) {
    B.drop_graph();
    cudaGraph_t g = nullptr;
    if (!B.capture_stream) SED_CUDA(cudaStreamCreateWithFlags(&B.capture_stream, cudaStreamNonBlocking));
    const cudaStream_t cs = B.capture_stream;
    SED_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
      SED_CUDA(cudaMemsetAsync(B.queue.p, 0, 16, cs));
      dispatch_launch(B, a, L, ncta, cs, fp64);
    } catch (...) {
      cudaStreamEndCapture(cs, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    SED_CUDA(cudaStreamEndCapture(cs, &g));
    cudaGraphExec_t x = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&x, g, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      SED_CUDA(e);
    }
    B.graph = g;
    B.graph_exec = x;
    B.graph_key.swap(key);
    ++B.graph_captures;
  } else {
    ++B.graph_replays;
  }
  SED_CUDA(cudaGraphLaunch(B.graph_exec, s));
}

// ------------------------------------------------------------ hop table
// Every request of a batch shares the catalog and the (i, j) term list, so the
// sparsity pattern of its sector matrix -- for each orbit row, the column
// orbit, group element, sign and twist-phase class counts of every hop -- is
// the same for all of them.  It is enumerated once into 64-bit records
//   c (24 bits) | u*G + h (18 bits) << 24 | phi (22 bits) << 42,
// phi indexing the distinct (h, class counts n_1..n_3, sign) combinations, and
// stored SELL-32: slice s holds rows 32s..32s+31, record k of row 32s+l at
// sl_off[s] + 32k + l, padded to the slice's longest row with records whose
// phi is the zero coefficient.  A request then only builds its coefficient
// tables; this is the batched counterpart of the reference's projection table
// (build_projection_table / _apply_table!, SRE:680-765), kept per hop.
static constexpr int kPhiCap = 2048;  // phase-id entries, the zero entry included
static constexpr int kGaugePhi = 3;   // gauge mode's phase ids: +1, -1, the padding zero

__global__ void k_hop_count(int64_t n_orb, const uint64_t* __restrict__ reps, const uint16_t* off,
                            const uint32_t* rec, int32_t* __restrict__ cnt) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x)
    cnt[o] = (int32_t)count_row_hops(reps[o], off, rec);
}

// records in HopIter order; phase key = h | n1 << 6 | n2 << 12 | n3 << 18 |
// sign << 24 (the host compacts the keys into phase ids)
template <bool FERMI>
__global__ void k_hop_fill(int64_t n_orb, const uint64_t* __restrict__ reps, const uint64_t* __restrict__ state,
                           const uint32_t* __restrict__ rank_tab, RankParams rp, const uint16_t* off,
                           const uint32_t* rec, const uint8_t* __restrict__ inv, int G,
                           const uint64_t* __restrict__ fmask, const uint32_t* __restrict__ sl_off,
                           const int32_t* __restrict__ sl_w, uint64_t* __restrict__ out,
                           uint32_t* __restrict__ key) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t base = (int64_t)sl_off[o >> 5] + (o & 31);
    const int wdt = sl_w[o >> 5];
    const uint64_t m = reps[o];
    HopIter it;
    it.init(m, off);
    uint32_t r;
    int from, k = 0;
    while (it.next(off, rec, r, from)) {
      const int j = r & 0xFF;
      const uint64_t nw = m ^ ((1ULL << from) | (1ULL << j));
      const uint64_t wd = state[dev::rank_of(nw, rank_tab, rp)];
      int neg = (int)((wd >> 40) & 1);
      if (FERMI) neg ^= __popcll(m & dev::bits_between(from, j)) & 1;
      const int h = (int)((wd >> 48) & 0xFF);
      const uint64_t* fm = fmask + 3 * h;
      const uint32_t n1 = __popcll(nw & fm[0]), n2 = __popcll(nw & fm[1]), n3 = __popcll(nw & fm[2]);
      out[base + 32 * (int64_t)k] = (uint64_t)(uint32_t)wd | ((uint64_t)((r >> 8) * G + h) << 24);
      key[base + 32 * (int64_t)k] = (uint32_t)h | n1 << 6 | n2 << 12 | n3 << 18 | (uint32_t)neg << 24;
      ++k;
    }
    for (; k < wdt; ++k) {
      out[base + 32 * (int64_t)k] = 0;
      key[base + 32 * (int64_t)k] = 0xFFFFFFFFu;
    }
  }
}

// Phase classes shared by the requests of one run: for every group element h,
// the coarsest partition of the sites on which every request's phase eta_h is
// constant (the common refinement of the requests' own partitions).  The
// largest class is the base; up to three others get masks.  False when some h
// needs more than four classes (the run then uses the on-the-fly matvec).
static bool family_classes(const GroupImpl& G, int n_req, const double* phase, const std::vector<uint64_t>& init,
                           std::vector<uint64_t>& fmask, std::vector<int8_t>& rep) {
  const int N = G.n_site, nG = G.n_ops;
  fmask.assign((size_t)nG * 3, 0);
  rep.assign((size_t)nG * 4, -1);
  std::vector<int> cls(N), ncls(N);
  struct Key {
    int c;
    double re, im;
    int id;
  };
  std::vector<Key> keys;
  for (int h = 0; h < nG; ++h) {
    // start from the given partition (the current table's), so a compatible
    // run keeps it
    int nc = 1;
    for (int q = 0; q < N; ++q) {
      cls[q] = 0;
      for (int c = 0; c < 3 && !init.empty(); ++c)
        if ((init[(size_t)h * 3 + c] >> q) & 1ULL) {
          cls[q] = c + 1;
          nc = std::max(nc, c + 2);
        }
    }
    for (int b = 0; b < n_req; ++b) {
      const double* ph = phase + ((size_t)b * nG + h) * N * 2;
      keys.clear();
      for (int q = 0; q < N; ++q) {
        const double re = ph[2 * q], im = ph[2 * q + 1];
        int id = -1;
        for (const Key& k : keys)
          if (k.c == cls[q] && k.re == re && k.im == im) id = k.id;
        if (id < 0) {
          id = (int)keys.size();
          if (id >= 4) return false;
          keys.push_back({cls[q], re, im, id});
        }
        ncls[q] = id;
      }
      cls.swap(ncls);
      nc = (int)keys.size();
    }
    std::vector<int> size(nc, 0);
    for (int q = 0; q < N; ++q) ++size[cls[q]];
    int bc = 0;
    for (int c = 1; c < nc; ++c)
      if (size[c] > size[bc]) bc = c;
    int slot = 0;
    for (int c = 0; c < nc; ++c) {
      int first = -1;
      uint64_t msk = 0;
      for (int q = 0; q < N; ++q)
        if (cls[q] == c) {
          if (first < 0) first = q;
          msk |= 1ULL << q;
        }
      if (c == bc) {
        rep[(size_t)h * 4] = (int8_t)first;
      } else {
        fmask[(size_t)h * 3 + slot] = msk;
        rep[(size_t)h * 4 + 1 + slot] = (int8_t)first;
        ++slot;
      }
    }
  }
  return true;
}

// A site gauge w_j = e^{i phi_j} for each request, under which its group
// phases become exactly 1: eta_g(j) w_{perm_g(j)} conj(w_j) = 1 for every g and
// site j.  The flux-twisted translation groups of build_translation_group
// (SRE:1374-1405) have one, w_j = exp(2 pi i theta . r_j / L): the twist then
// spreads evenly over the bonds, and U_g' = W U_g W^-1 is the plain
// permutation.  A breadth-first walk from one site per site orbit fixes w;
// every (g, j) is then checked to 1e-10.  Under the gauge the sector matrix
// becomes D H D^-1, D diagonal and unitary on the same orbits (the membership
// test still uses the request's own phases), so eigenvalues are unchanged; a
// hop (i -> j, t) carries t w_j conj(w_i) and no per-site phase product.
// False (nothing usable) when some request has no such gauge.
static bool site_gauges(const GroupImpl& G, int n_req, const double* phase, std::vector<double>& w) {
  const int N = G.n_site, nG = G.n_ops;
  w.assign((size_t)n_req * N * 2, 0.0);
  std::vector<char> seen(N);
  std::vector<int> fifo(N);
  for (int b = 0; b < n_req; ++b) {
    const double* ph = phase + (size_t)b * nG * N * 2;
    double* wb = w.data() + (size_t)b * N * 2;
    std::fill(seen.begin(), seen.end(), 0);
    for (int root = 0; root < N; ++root) {
      if (seen[root]) continue;
      seen[root] = 1;
      wb[2 * root] = 1.0;
      wb[2 * root + 1] = 0.0;
      int head = 0, tail = 0;
      fifo[tail++] = root;
      while (head < tail) {
        const int j = fifo[head++];
        for (int g = 0; g < nG; ++g) {
          const int q = G.perm[(size_t)g * N + j];
          if (seen[q]) continue;
          // w_q = w_j / eta_g(j)
          const double er = ph[((size_t)g * N + j) * 2], ei = ph[((size_t)g * N + j) * 2 + 1];
          const double n2 = er * er + ei * ei;
          if (!(n2 > 0.0)) return false;
          const double wr = wb[2 * j], wi = wb[2 * j + 1];
          wb[2 * q] = (wr * er + wi * ei) / n2;
          wb[2 * q + 1] = (wi * er - wr * ei) / n2;
          seen[q] = 1;
          fifo[tail++] = q;
        }
      }
    }
    for (int g = 0; g < nG; ++g)
      for (int j = 0; j < N; ++j) {
        const int q = G.perm[(size_t)g * N + j];
        const double er = ph[((size_t)g * N + j) * 2], ei = ph[((size_t)g * N + j) * 2 + 1];
        // eta * w_q * conj(w_j)
        const double ar = wb[2 * q] * wb[2 * j] + wb[2 * q + 1] * wb[2 * j + 1];
        const double ai = wb[2 * q + 1] * wb[2 * j] - wb[2 * q] * wb[2 * j + 1];
        const double re = er * ar - ei * ai, im = er * ai + ei * ar;
        if (std::hypot(re - 1.0, im) > 1e-10) return false;
      }
  }
  return true;
}

// Make the hop table match this run: in gauge mode the records carry signs
// only and serve every run; otherwise they carry phase ids of this run's phase
// classes.  Returns whether the run can use the table.  phase is the host copy
// of the requests' group phases.
// Bank-aware order of each row's records.  Step k of a warp's pass over a
// slice gathers, for its 32 rows' k-th records, x[col] and the coefficient
// (and, with phase classes, the phase-id coefficient) from shared memory.
// An E-byte gather is served 128 / E lanes at a time, and each further
// distinct word that falls into an already used bank group (E consecutive
// bytes of the 32 banks) costs one more shared-memory wavefront; with random
// columns that is about 5 wavefronts per gather, where 2 would do, and these
// gathers bound the matvec on the L1 data pipe.  A row's records may be summed
// in any order and its padding slots may sit anywhere, so the host reorders
// every slice, step by step and lane group by lane group:
//   - greedily: each lane takes the remaining record that raises the worst
//     bank-group load of its group least (ties: the emptier bank groups),
//     padding only where that raises it less than any record and the row can
//     still place the rest;
//   - then kBankRounds rounds of coordinate descent: each lane in turn puts
//     its pick back and chooses again against the others' picks.
// A padding record's coefficient is zero, so it takes a column another lane
// of its group reads (no extra word).  Slices are independent and are spread
// over up to eight host threads.
//   elem: bytes per gathered element (8 complex64, 16 complex128);
//   use_x: x is in shared memory (else only the coefficient gathers count);
//   use_p: records carry phase ids whose coefficients are gathered too;
//   pad_hi: bits 24.. of a padding record (its coefficient and phase id).
static constexpr int kBankRounds = 4;

namespace {
constexpr int kMaxLaneGroup = 16;
// distinct words per bank group of one lane group's gather, with use counts
struct BankBins {
  uint32_t word[kMaxLaneGroup][kMaxLaneGroup];
  int uses[kMaxLaneGroup][kMaxLaneGroup];
  int cnt[kMaxLaneGroup];
  int g = 16;
  void clear(int groups) {
    g = groups;
    for (int b = 0; b < g; ++b) cnt[b] = 0;
  }
  int worst() const {
    int m = 0;
    for (int b = 0; b < g; ++b) m = std::max(m, cnt[b]);
    return m;
  }
  // raise of the worst load `mx` and the bank group's load after adding w
  void cost(uint32_t w, int mx, int& raise, int& load) const {
    const int b = (int)(w % (uint32_t)g);
    for (int i = 0; i < cnt[b]; ++i)
      if (word[b][i] == w) {
        raise = 0;
        load = cnt[b];
        return;
      }
    load = cnt[b] + 1;
    raise = load > mx ? load - mx : 0;
  }
  void add(uint32_t w) {
    const int b = (int)(w % (uint32_t)g);
    for (int i = 0; i < cnt[b]; ++i)
      if (word[b][i] == w) {
        ++uses[b][i];
        return;
      }
    word[b][cnt[b]] = w;
    uses[b][cnt[b]++] = 1;
  }
  void remove(uint32_t w) {
    const int b = (int)(w % (uint32_t)g);
    for (int i = 0; i < cnt[b]; ++i)
      if (word[b][i] == w) {
        if (--uses[b][i] == 0) {
          --cnt[b];
          word[b][i] = word[b][cnt[b]];
          uses[b][i] = uses[b][cnt[b]];
        }
        return;
      }
  }
};

struct BankSched {
  int G;
  bool use_x, use_p;
  uint64_t pad_hi;
  uint32_t pad_t, pad_p;
  static constexpr uint64_t kPad = ~0ull;  // a padding pick (never a record: bits 42.. of records are < 2^22)
  BankBins bx, bt, bp;
  void add(uint64_t r) {
    if (r == kPad) {
      bt.add(pad_t);
      if (use_p) bp.add(pad_p);
      return;
    }
    if (use_x) bx.add((uint32_t)(r & 0xFFFFFFu));
    bt.add((uint32_t)(r >> 24) & 0x3FFFFu);
    if (use_p) bp.add((uint32_t)(r >> 42));
  }
  void remove(uint64_t r) {
    if (r == kPad) {
      bt.remove(pad_t);
      if (use_p) bp.remove(pad_p);
      return;
    }
    if (use_x) bx.remove((uint32_t)(r & 0xFFFFFFu));
    bt.remove((uint32_t)(r >> 24) & 0x3FFFFu);
    if (use_p) bp.remove((uint32_t)(r >> 42));
  }
  // take the best of rl (or padding, when slots_left allows it) out of rl
  uint64_t choose(std::vector<uint64_t>& rl, int slots_left) {
    const int mx = bx.worst(), mt = bt.worst(), mp = bp.worst();
    int best = -1, best_raise = INT_MAX, best_load = INT_MAX;
    for (int i = 0; i < (int)rl.size(); ++i) {
      const uint64_t r = rl[i];
      int ra = 0, lo = 0, r1, l1;
      if (use_x) {
        bx.cost((uint32_t)(r & 0xFFFFFFu), mx, r1, l1);
        ra += r1;
        lo += l1;
      }
      bt.cost((uint32_t)(r >> 24) & 0x3FFFFu, mt, r1, l1);
      ra += r1;
      lo += l1;
      if (use_p) {
        bp.cost((uint32_t)(r >> 42), mp, r1, l1);
        ra += r1;
        lo += l1;
      }
      if (ra < best_raise || (ra == best_raise && lo < best_load)) {
        best = i;
        best_raise = ra;
        best_load = lo;
      }
    }
    if ((int)rl.size() < slots_left) {
      int r1, l1, r2 = 0, l2 = 0;
      bt.cost(pad_t, mt, r1, l1);
      if (use_p) bp.cost(pad_p, mp, r2, l2);
      if (best < 0 || r1 + r2 < best_raise) return kPad;
    }
    const uint64_t r = rl[best];
    rl[best] = rl.back();
    rl.pop_back();
    return r;
  }
  void slice(uint64_t* base, int W, int lanes, std::vector<std::vector<uint64_t>>& rem) {
    for (int l = 0; l < lanes; ++l) {
      rem[l].clear();
      for (int k = 0; k < W; ++k) {
        const uint64_t r = base[32 * (size_t)k + l];
        if ((r >> 24) != pad_hi) rem[l].push_back(r);
      }
    }
    uint64_t pick[32];
    for (int k = 0; k < W; ++k) {
      for (int g0 = 0; g0 < lanes; g0 += G) {
        const int ge = std::min(lanes, g0 + G);
        bx.clear(G);
        bt.clear(G);
        bp.clear(G);
        for (int l = g0; l < ge; ++l) add(pick[l] = choose(rem[l], W - k));
        for (int round = 0; round < kBankRounds; ++round)
          for (int l = g0; l < ge; ++l) {
            remove(pick[l]);
            if (pick[l] != kPad) rem[l].push_back(pick[l]);
            add(pick[l] = choose(rem[l], W - k));
          }
        uint32_t any_col = 0;
        for (int l = g0; l < ge; ++l)
          if (pick[l] != kPad) {
            any_col = (uint32_t)(pick[l] & 0xFFFFFFu);
            break;
          }
        for (int l = g0; l < ge; ++l)
          base[32 * (size_t)k + l] = pick[l] == kPad ? (pad_hi << 24) | any_col : pick[l];
      }
    }
  }
};
}  // namespace

static void bank_schedule(std::vector<uint64_t>& recs, const std::vector<uint32_t>& off,
                          const std::vector<int32_t>& width, int64_t n_orb, int elem, bool use_x, bool use_p,
                          uint64_t pad_hi) {
  const int64_t n_sl = (int64_t)off.size();
  const int nthr = n_sl >= 64 ? (int)std::min(8u, std::max(1u, std::thread::hardware_concurrency())) : 1;
  auto work = [&](int t) {
    BankSched bs;
    bs.G = 128 / elem;
    bs.use_x = use_x;
    bs.use_p = use_p;
    bs.pad_hi = pad_hi;
    bs.pad_t = (uint32_t)(pad_hi & 0x3FFFFu);
    bs.pad_p = (uint32_t)(pad_hi >> 18);
    std::vector<std::vector<uint64_t>> rem(32);
    for (int64_t sl = t; sl < n_sl; sl += nthr)
      bs.slice(recs.data() + off[sl], width[sl], (int)std::min<int64_t>(32, n_orb - sl * 32), rem);
  };
  if (nthr == 1) {
    work(0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nthr; ++t) th.emplace_back(work, t);
  for (auto& t : th) t.join();
}

static bool bank_order_enabled() {
  const char* e = std::getenv("SED_BATCH_BANK_ORDER");
  return !(e && e[0] == '0');
}

static bool prepare_table(BatchImpl& B, int n_req, const double* phase, cudaStream_t s, bool gauge) {
  if (B.phi_cap == 0 || !B.tab_enabled) return false;
  const CatalogImpl& C = *B.cat;
  const GroupImpl& G = *C.group;
  if (C.n_orbits >= (1 << 24) || B.tchi_n >= (1 << 18) || C.n_filled > 63) return false;
  std::vector<uint64_t> fmask;
  std::vector<int8_t> rep;
  if (gauge) {
    if (B.tab_valid && B.tab_gauge) return true;
    fmask.assign((size_t)G.n_ops * 3, 0);  // no class counts: the keys hold h and the sign
    rep.assign((size_t)G.n_ops * 4, -1);
  } else {
    // refine the current table's partition; if that needs too many classes,
    // partition this run alone
    const std::vector<uint64_t> none;
    if (!(B.tab_valid && !B.tab_gauge && family_classes(G, n_req, phase, B.tab_fmask, fmask, rep)) &&
        !family_classes(G, n_req, phase, none, fmask, rep))
      return false;
  }
  if (B.tab_valid && !B.tab_gauge && !gauge && fmask == B.tab_fmask) {
    if (rep != B.tab_rep) {
      B.tab_rep = rep;
      upload(B.rep_site, B.tab_rep, s);
    }
    return true;
  }
  B.tab_valid = false;
  const int64_t n = C.n_orbits;
  const int64_t n_sl = (n + 31) / 32;
  const int grid = grid1(n, 256);
  if (B.row_cnt.empty()) {
    DevBuf cnt((size_t)std::max<int64_t>(n, 1) * 4);
    k_hop_count<<<grid, 256, 0, s>>>(n, C.reps.as<uint64_t>(), B.site_off.as<uint16_t>(), B.rec.as<uint32_t>(),
                                     cnt.as<int32_t>());
    SED_CUDA(cudaGetLastError());
    std::vector<int32_t> row_cnt(n);
    SED_CUDA(cudaMemcpyAsync(row_cnt.data(), cnt.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    SED_CUDA(cudaStreamSynchronize(s));
    std::vector<uint32_t> off(n_sl);
    std::vector<int32_t> w(n_sl);
    int64_t tot = 0;
    for (int64_t sl = 0; sl < n_sl; ++sl) {
      int mx = 0;
      for (int64_t o = sl * 32; o < std::min(n, sl * 32 + 32); ++o) mx = std::max(mx, row_cnt[o]);
      SED_REQUIRE(tot < (int64_t)UINT32_MAX, 5, "hop table too large");
      off[sl] = (uint32_t)tot;
      w[sl] = mx;
      tot += 32 * (int64_t)mx;
    }
    B.hop.alloc((size_t)std::max<int64_t>(tot, 1) * 8);
    upload(B.sl_off, off, s);
    upload(B.sl_w, w, s);
    B.h_sl_off = off;
    B.h_sl_w = w;
    B.hop_records = tot;
    B.row_cnt.swap(row_cnt);  // the slices exist from here on
  }
  upload(B.fmask_dev, fmask, s);
  const int64_t tot = B.hop_records;
  DevBuf keyd((size_t)std::max<int64_t>(tot, 1) * 4);
  // k_hop_fill writes the rows of the catalog only: the lanes past the last
  // orbit in the last slice are set here to padding (zero record, no phase
  // key), so the compaction below never reads what an allocation happened to
  // hold
  SED_CUDA(cudaMemsetAsync(keyd.p, 0xFF, (size_t)std::max<int64_t>(tot, 1) * 4, s));
  SED_CUDA(cudaMemsetAsync(B.hop.p, 0, (size_t)std::max<int64_t>(tot, 1) * 8, s));
  if (G.stats == 1)
    k_hop_fill<true><<<grid, 256, 0, s>>>(n, C.reps.as<uint64_t>(), C.state.as<uint64_t>(), C.rank.dev.as<uint32_t>(),
                                          C.rank.rp, B.site_off.as<uint16_t>(), B.rec.as<uint32_t>(),
                                          C.inv_u8.as<uint8_t>(), G.n_ops, B.fmask_dev.as<uint64_t>(),
                                          B.sl_off.as<uint32_t>(), B.sl_w.as<int32_t>(), B.hop.as<uint64_t>(),
                                          keyd.as<uint32_t>());
  else
    k_hop_fill<false><<<grid, 256, 0, s>>>(n, C.reps.as<uint64_t>(), C.state.as<uint64_t>(), C.rank.dev.as<uint32_t>(),
                                           C.rank.rp, B.site_off.as<uint16_t>(), B.rec.as<uint32_t>(),
                                           C.inv_u8.as<uint8_t>(), G.n_ops, B.fmask_dev.as<uint64_t>(),
                                           B.sl_off.as<uint32_t>(), B.sl_w.as<int32_t>(), B.hop.as<uint64_t>(),
                                           keyd.as<uint32_t>());
  SED_CUDA(cudaGetLastError());
  std::vector<uint64_t> recs(tot);
  std::vector<uint32_t> keys(tot);
  SED_CUDA(cudaMemcpyAsync(recs.data(), B.hop.p, (size_t)tot * 8, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaMemcpyAsync(keys.data(), keyd.p, (size_t)tot * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
  // compact the phase keys (first-appearance order) into phase ids; every
  // descriptor is checked against the tables the kernel indexes with it
  // (group element < |G|, class counts <= N_filled), so no key can reach
  // outside them
  std::unordered_map<uint32_t, uint32_t> id;
  std::vector<uint32_t> desc;
  const uint64_t n_tchi = (uint64_t)B.n_bil * G.n_ops;
  // a coefficient's slot in the hashed table layout of hop-table runs
  auto tslot = [&](uint64_t i) { return i * (uint64_t)B.tchi_mul % (uint64_t)B.tchi_n; };
  if (gauge) {
    // phase id = the sign; padding: the zero coefficient (tchi entry n_tchi,
    // phase id 2)
    for (int64_t t = 0; t < tot; ++t) {
      const bool pad = keys[t] == 0xFFFFFFFFu;
      SED_REQUIRE(pad || ((recs[t] & 0xFFFFFFu) < (uint64_t)C.n_orbits && ((recs[t] >> 24) & 0x3FFFFu) < n_tchi &&
                          (int)(keys[t] & 0x3F) < G.n_ops && (keys[t] >> 25) == 0),
                  5, "internal error: hop-table record out of range");
      const uint64_t ti = pad ? n_tchi : (recs[t] >> 24) & 0x3FFFFu;
      recs[t] = (pad ? 0 : recs[t] & 0xFFFFFFu) | (tslot(ti) << 24) | ((pad ? 2ULL : (uint64_t)(keys[t] >> 24)) << 42);
    }
    if (bank_order_enabled())
      bank_schedule(recs, B.h_sl_off, B.h_sl_w, C.n_orbits, B.precision == 1 ? 8 : 16, B.x_smem && B.precision == 1,
                    false, tslot(n_tchi) | (2ULL << 18));
    SED_CUDA(cudaMemcpyAsync(B.hop.p, recs.data(), (size_t)tot * 8, cudaMemcpyHostToDevice, s));
    SED_CUDA(cudaStreamSynchronize(s));
    B.n_phi = 2;
    B.tab_gauge = true;
    B.tab_fmask.clear();
    B.tab_valid = true;
    return true;
  }
  for (int64_t t = 0; t < tot; ++t) {
    if (keys[t] == 0xFFFFFFFFu) continue;
    auto it = id.find(keys[t]);
    if (it == id.end()) {
      const uint32_t d = keys[t];
      const int kf = C.n_filled;
      SED_REQUIRE((int)(d & 0x3F) < G.n_ops && (int)((d >> 6) & 0x3F) <= kf && (int)((d >> 12) & 0x3F) <= kf &&
                      (int)((d >> 18) & 0x3F) <= kf && (d >> 25) == 0,
                  5, "internal error: hop-table phase key out of range");
      if ((int)desc.size() + 1 >= B.phi_cap) return false;
      it = id.emplace(keys[t], (uint32_t)desc.size()).first;
      desc.push_back(keys[t]);
    }
  }
  const uint64_t zero_id = desc.size();
  for (int64_t t = 0; t < tot; ++t) {
    const bool pad = keys[t] == 0xFFFFFFFFu;
    SED_REQUIRE(pad || ((recs[t] & 0xFFFFFFu) < (uint64_t)C.n_orbits && ((recs[t] >> 24) & 0x3FFFFu) < n_tchi), 5,
                "internal error: hop-table record out of range");
    const uint64_t phi = pad ? zero_id : id[keys[t]];
    const uint64_t ti = pad ? n_tchi : (recs[t] >> 24) & 0x3FFFFu;
    recs[t] = (pad ? 0 : recs[t] & 0xFFFFFFu) | (tslot(ti) << 24) | (phi << 42);
  }
  if (bank_order_enabled())
    bank_schedule(recs, B.h_sl_off, B.h_sl_w, C.n_orbits, B.precision == 1 ? 8 : 16, B.x_smem && B.precision == 1,
                  true, tslot(n_tchi) | (zero_id << 18));
  SED_CUDA(cudaMemcpyAsync(B.hop.p, recs.data(), (size_t)tot * 8, cudaMemcpyHostToDevice, s));
  upload(B.phi_desc, desc, s);
  B.n_phi = (int)desc.size();
  B.tab_gauge = false;
  B.tab_fmask = fmask;
  B.tab_rep = rep;
  upload(B.rep_site, B.tab_rep, s);
  SED_CUDA(cudaStreamSynchronize(s));
  B.tab_valid = true;
  return true;
}

std::shared_ptr<BatchImpl> make_batch(std::shared_ptr<CatalogImpl> cp, int n_bil, const int32_t* bil_ij, int n_den,
                                      const int32_t* den_ij, const double* den_v, int precision, int nev,
                                      int krylovdim, int max_req) {
  const CatalogImpl& C = *cp;
  const GroupImpl& G = *C.group;
  SED_REQUIRE(precision == 0 || precision == 1, 1, "precision must be SED_PREC_FP64 or SED_PREC_MIXED");
  SED_REQUIRE(nev >= 1 && nev <= kMaxNev - 2, 5, "batched solves support 1 <= nev <= 6");
  SED_REQUIRE(max_req >= 1, 1, "max_requests must be positive");
  SED_REQUIRE(n_bil >= 0 && n_bil < 65535, 5, "at most 65534 bilinear terms");
  SED_REQUIRE(n_bil == 0 || bil_ij, 1, "bilinear index array must not be NULL");
  SED_REQUIRE(n_den == 0 || (den_ij && den_v), 1, "density arrays must not be NULL");
  auto B = std::make_shared<BatchImpl>();
  B->m_fixed = krylovdim > 0;  // else the autotuner picks the Krylov dimension
  if (krylovdim <= 0) krylovdim = 24;
  B->cat = cp;
  B->precision = precision;
  B->nev = nev;
  B->m = std::min(std::max(krylovdim, 2 * (nev + 2) + 1), kMaxM);
  B->m_cap = B->m_fixed ? B->m : std::max(B->m, std::min(28, kMaxM));
  B->max_req = max_req;
  B->n_bil = n_bil;
  B->n_den = n_den;
  B->den_ij.assign(den_ij, den_ij + 2 * n_den);
  B->den_v.assign(den_v, den_v + 2 * n_den);
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
  check_species_terms(C, n_bil, bil_ij);
  {
    std::vector<int32_t> bij(bil_ij, bil_ij + 2 * n_bil);
    B->bil_dev.alloc((size_t)std::max(2 * n_bil, 1) * 4);
    if (n_bil) SED_CUDA(cudaMemcpy(B->bil_dev.p, bij.data(), bij.size() * 4, cudaMemcpyHostToDevice));
    B->gauge_w.alloc((size_t)max_req * G.n_site * 16);
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
  // coefficient table slots: the smallest prime >= n_bil * G + 1, and a
  // multiplier near 0.618 of it (golden-ratio hashing; coprime to the prime)
  {
    auto is_prime = [](int64_t v) {
      if (v < 2) return false;
      for (int64_t d = 2; d * d <= v; ++d)
        if (v % d == 0) return false;
      return true;
    };
    int64_t p = (int64_t)n_bil * G.n_ops + 1;
    while (!is_prime(p)) ++p;
    B->tchi_n = (int)p;
    B->tchi_mul = (int)std::max<int64_t>(1, (int64_t)(0.6180339887498949 * (double)p));
  }
  // the hop table's phase-id coefficients need shared memory; a sector too
  // large for both keeps the on-the-fly matvec
  B->phi_cap = kPhiCap;
  BatchArgs a = base_args(*B);
  // Shared memory: the complex64 matvec input x stays in shared memory when it
  // fits beside the tables, with the hop table's phase coefficients if they
  // fit too; a sector whose x cannot fit keeps x in global memory (L2) and
  // the hop table.
  constexpr size_t kSmemBudget = 220 * 1024;
  // phase-id capacity: the full table, else the three entries of gauge mode
  // (+1, -1 and the padding zero: runs whose requests have site gauges keep
  // the hop table), else none
  auto fit_phi = [&](bool xs, auto vt) {
    using VT = decltype(vt);
    for (int cap : {kPhiCap, kGaugePhi, 0}) {
      a.phi_cap = cap;
      if (batch_layout<VT>(a, xs).total <= kSmemBudget) return true;
    }
    return false;
  };
  if (precision == 1) {
    if (!fit_phi(true, float2{})) {  // x in global memory only when it fits beside no table at all
      B->x_smem = false;
      fit_phi(false, float2{});
    }
  } else {
    fit_phi(false, double2{});
  }
  B->phi_cap = a.phi_cap;
  BatchSmem L;
  int ncta = 1;
  dispatch_prepare(*B, a, L, ncta, precision == 0);
  B->smem = L.total;
  // per-block workspace, bounded to 16 GB
  // basis and restart buffers of equal capacity (they trade places), work vector, FP64 input
  const size_t slots = (size_t)std::max(B->m_cap + 1, 5 * (nev + 2));  // the largest Krylov dimension tried
  const size_t per_cta = (2 * slots + 2) * B->ld * 16 + (size_t)B->tchi_n * 16 + B->ld;
  ncta = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)ncta, (int64_t)max_req,
                                                      (int64_t)((16ull << 30) / std::max<size_t>(per_cta, 1))}));
  B->n_cta = ncta;
  B->V.alloc((size_t)ncta * slots * B->ld * 16);
  B->R.alloc((size_t)ncta * slots * B->ld * 16);
  B->W.alloc((size_t)ncta * B->ld * 16);
  B->X64.alloc((size_t)ncta * B->ld * 16);
  B->tchi64.alloc((size_t)ncta * B->tchi_n * 16);
  B->rowflag.alloc((size_t)ncta * B->ld);
  if (B->phi_cap) B->pwc64.alloc((size_t)ncta * B->phi_cap * 16);
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

// Every request's term list must be Hermitian and invariant under its own
// group.  Large batches are checked on up to eight host threads (requests
// interleaved); the error reported is the one of the lowest failing request,
// as a serial check would report it.
static void validate_requests(BatchImpl& B, int n_req, const double* phase, const double* amp) {
  const GroupImpl& G = *B.cat->group;
  const int nthr = n_req >= 64 ? (int)std::min(8u, std::max(1u, std::thread::hardware_concurrency())) : 1;
  std::vector<int> first_bad(nthr, INT_MAX);
  std::vector<Error> err(nthr);
  auto work = [&](int t) {
    GroupImpl Gr = G;
    for (int b = t; b < n_req; b += nthr) {
      Gr.phase.assign(phase + (size_t)b * G.n_ops * G.n_site * 2, phase + (size_t)(b + 1) * G.n_ops * G.n_site * 2);
      try {
        check_hermitian_symmetric(Gr, B.n_bil, B.bil_ij.data(), amp + (size_t)b * B.n_bil * 2);
      } catch (const Error& e) {
        first_bad[t] = b;
        err[t] = e;
        return;
      }
    }
  };
  if (nthr == 1) {
    work(0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nthr; ++t) pool.emplace_back(work, t);
    for (auto& th : pool) th.join();
  }
  int tb = 0;
  for (int t = 1; t < nthr; ++t)
    if (first_bad[t] < first_bad[tb]) tb = t;
  if (first_bad[tb] != INT_MAX) throw err[tb];
}

// ------------------------------------------------------------ autotuner
// The batched launch's shape -- threads per row of the hop-table matvec (1,
// or a lane pair splitting each row's records) and, unless the caller fixed
// it, the Krylov dimension m of the thick-restart Lanczos (20, 24 or 28) -- is
// picked by measurement: on the first run of a catalog shape every candidate
// solves one wave of the run's own requests (at most one request per resident
// block), twice, timed with CUDA events on the batch stream, and the fastest
// is kept for that shape for the whole process.  SED_BATCH_SHAPE="m,tpr" in
// the environment or sed_batch_set_shape pins a shape.  Results depend on the
// shape only within the solver's tolerance (the Krylov space and a row's
// summation order change); a given shape is reproducible bit for bit.
struct BatchShapeKey {
  int64_t n_orb;
  int n_terms, n_ops, n_site, fermi, precision, nev, use_tab, gauge, m_fixed_to;
  bool operator<(const BatchShapeKey& o) const {
    return std::tie(n_orb, n_terms, n_ops, n_site, fermi, precision, nev, use_tab, gauge, m_fixed_to) <
           std::tie(o.n_orb, o.n_terms, o.n_ops, o.n_site, o.fermi, o.precision, o.nev, o.use_tab, o.gauge,
                    o.m_fixed_to);
  }
};
static std::mutex g_bshape_mu;
static std::map<BatchShapeKey, std::pair<int, int>> g_bshapes;

static bool env_batch_shape(int* m, int* tpr) {
  const char* e = std::getenv("SED_BATCH_SHAPE");
  if (!e) return false;
  int a = 0, b = 0;
  if (std::sscanf(e, "%d,%d", &a, &b) != 2 || (b != 1 && b != 2) || a < 2 || a > kMaxM) return false;
  *m = a;
  *tpr = b;
  return true;
}

static void choose_shape(BatchImpl& B, BatchArgs& a, int n_req, cudaStream_t s) {
  const int m_lo = 2 * (B.nev + 2) + 1;
  auto clamp_m = [&](int m) { return std::min(std::max(m, m_lo), B.m_cap); };
  int m = B.m, tpr = 1;
  if (B.pin_m > 0) {
    m = clamp_m(B.pin_m);
    tpr = B.pin_tpr;
  } else if (env_batch_shape(&m, &tpr)) {
    m = B.m_fixed ? B.m : clamp_m(m);
  } else {
    const CatalogImpl& C = *B.cat;
    const GroupImpl& G = *C.group;
    const BatchShapeKey key{C.n_orbits, B.tt.n_terms, G.n_ops, G.n_site, B.fermi ? 1 : 0, B.precision, B.nev,
                            a.use_tab, a.gauge, B.m_fixed ? B.m : 0};
    bool found = false;
    {
      std::lock_guard<std::mutex> lock(g_bshape_mu);
      auto it = g_bshapes.find(key);
      if (it != g_bshapes.end()) {
        m = it->second.first;
        tpr = it->second.second;
        found = true;
      }
    }
    if (!found) {
      std::vector<int> ms = B.m_fixed ? std::vector<int>{B.m} : std::vector<int>{24, 20, 28};
      std::vector<int> tprs = a.use_tab ? std::vector<int>{1, 2} : std::vector<int>{1};
      const int sample = std::min(n_req, B.n_cta);
      std::vector<int64_t> tns((size_t)sample * 2);
      cudaEvent_t e0, e1;
      SED_CUDA(cudaEventCreate(&e0));
      SED_CUDA(cudaEventCreate(&e1));
      float best = 1e30f;
      for (int mc : ms) {
        mc = clamp_m(mc);
        for (int tc : tprs) {
          BatchArgs t = a;
          t.m = mc;
          t.tpr = tc;
          t.n_req = sample;
          t.evecs = nullptr;  // the trial runs write only the caller's scalar outputs, overwritten below
          BatchSmem L;
          int ncta = 1;
          dispatch_prepare(B, t, L, ncta, B.precision == 0);
          ncta = std::min(B.n_cta, sample);
          // score: the mean request duration from the kernel's own per-request
          // timestamps. A multi-wave launch's throughput follows the mean,
          // whereas one wave's wall time is set by its slowest request.
          float ms_best = 1e30f;
          for (int rep = 0; rep < 2; ++rep) {
            SED_CUDA(cudaMemsetAsync(B.queue.p, 0, 16, s));
            SED_CUDA(cudaEventRecord(e0, s));
            dispatch_launch(B, t, L, ncta, s, B.precision == 0);
            SED_CUDA(cudaEventRecord(e1, s));
            SED_CUDA(cudaMemcpyAsync(tns.data(), t.t_ns, (size_t)sample * 16, cudaMemcpyDeviceToHost, s));
            SED_CUDA(cudaStreamSynchronize(s));
            float el = 0.f;
            SED_CUDA(cudaEventElapsedTime(&el, e0, e1));
            double sum = 0.0;
            int cnt = 0;
            for (int i = 0; i < sample; ++i) {
              const int64_t d = tns[2 * (size_t)i + 1] - tns[2 * (size_t)i];
              if (d > 0) sum += (double)d, ++cnt;
            }
            // the event time stands in when no request was timed (all sectors empty)
            const float score = cnt ? (float)(sum / cnt * 1e-6) : el;
            ms_best = std::min(ms_best, score);
          }
          if (ms_best < best) {
            best = ms_best;
            m = mc;
            tpr = tc;
          }
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      ++B.tune_runs;
      std::lock_guard<std::mutex> lock(g_bshape_mu);
      g_bshapes[key] = {m, tpr};
    }
  }
  if (!a.use_tab) tpr = 1;
  a.m = m;
  a.tpr = tpr;
  B.last_m = m;
  B.last_tpr = tpr;
}

// Launch on device-resident buffers (asynchronous on the batch stream).
void batch_launch_device(BatchImpl& B, int n_req, const double* chi, const double* phase, const double* amp,
                         const uint64_t* seeds, double tol, int maxiter, double* evals, int32_t* status,
                         int64_t* dims, double* delta, int32_t* nmv, const double* phase_host = nullptr,
                         double* evecs = nullptr, int64_t ev_ld = 0) {
  SED_REQUIRE(!evecs || ev_ld >= B.cat->n_orbits, 1,
              "eigenvector leading dimension must be at least the catalog's orbit count");
  SED_REQUIRE(n_req >= 0 && n_req <= B.max_req, 1, "n_req exceeds max_requests");
  SED_REQUIRE(tol > 0.0 && maxiter >= 1, 1, "tol and maxiter must be positive");
  SED_REQUIRE(chi && phase && seeds && evals && status && dims && delta && nmv, 1, "NULL argument");
  SED_REQUIRE(B.n_bil == 0 || amp, 1, "NULL bilinear amplitudes");
  SED_REQUIRE(!B.ring.on, 1, "the batch's request ring is running: stop it before a batch run");
  B.last_n = n_req;
  B.n_fallback = 0;
  if (n_req == 0) return;
  cudaStream_t s = B.stream;
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
  a.evecs = reinterpret_cast<double2*>(evecs);
  a.ev_ld = evecs ? ev_ld : 0;
  // hop table for this run's phase classes (needs the phases on the host)
  std::vector<double> ph_h;
  if (B.phi_cap > 0 && B.tab_enabled && !phase_host) {
    const GroupImpl& G = *B.cat->group;
    ph_h.resize((size_t)n_req * G.n_ops * G.n_site * 2);
    SED_CUDA(cudaMemcpyAsync(ph_h.data(), phase, ph_h.size() * 8, cudaMemcpyDeviceToHost, s));
    SED_CUDA(cudaStreamSynchronize(s));
    phase_host = ph_h.data();
  }
  // gauge mode when every request has a site gauge (sign-only records)
  std::vector<double> gw;
  const bool gauge = phase_host && B.gauge_enabled && B.phi_cap > 0 && B.tab_enabled &&
                     site_gauges(*B.cat->group, n_req, phase_host, gw);
  a.use_tab = phase_host && prepare_table(B, n_req, phase_host, s, gauge) ? 1 : 0;
  a.gauge = a.use_tab && gauge ? 1 : 0;
  if (a.gauge) {
    SED_CUDA(cudaMemcpyAsync(B.gauge_w.p, gw.data(), gw.size() * 8, cudaMemcpyHostToDevice, s));
    a.gauge_w = B.gauge_w.as<double2>();
  }
  B.last_gauge = a.gauge;
  if (a.use_tab) {
    a.n_phi = B.n_phi;
    a.hop = B.hop.as<uint64_t>();
    a.sl_off = B.sl_off.as<uint32_t>();
    a.sl_w = B.sl_w.as<int32_t>();
    a.phi_desc = B.phi_desc.as<uint32_t>();
    a.rep_site = B.rep_site.as<int8_t>();
    a.pwc64 = B.pwc64.as<double2>();
  }
  B.last_tab = a.use_tab;
  a.tpr = 1;
  choose_shape(B, a, n_req, s);
  BatchSmem L;
  int ncta = 1;
  dispatch_prepare(B, a, L, ncta, B.precision == 0);
  ncta = std::min(B.n_cta, n_req);
  graph_launch(B, a, L, ncta, s, B.precision == 0);
  if (B.precision == 1) {
    // requests whose FP64 polish missed its residual target are answered by
    // the all-FP64 kernel (same inputs, same seed), so no unconverged pair is
    // ever returned
    std::vector<int32_t> st(n_req);
    SED_CUDA(cudaMemcpyAsync(st.data(), status, (size_t)n_req * 4, cudaMemcpyDeviceToHost, s));
    SED_CUDA(cudaStreamSynchronize(s));
    std::vector<int32_t> redo;
    for (int i = 0; i < n_req; ++i)
      if (st[i] == kPolishFailed) redo.push_back(i);
    B.n_fallback = (int)redo.size();
    if (!redo.empty()) {
      upload(B.redo, redo, s);
      SED_CUDA(cudaMemsetAsync(B.queue.p, 0, 16, s));
      BatchArgs a2 = a;
      a2.n_req = (int)redo.size();
      a2.req_list = B.redo.as<int32_t>();
      BatchSmem L2;
      int nc2 = 1;
      dispatch_prepare(B, a2, L2, nc2, true);
      nc2 = std::min(B.n_cta, a2.n_req);
      dispatch_launch(B, a2, L2, nc2, s, true);
    }
  }
}

void batch_run(BatchImpl& B, int n_req, const double* chi, const double* phase, const double* amp,
               const uint64_t* seeds, double tol, int maxiter, double* evals, int32_t* status, int64_t* dims,
               double* delta, int32_t* nmv, double* evecs = nullptr, int64_t ev_ld = 0) {
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
  double* d_evecs = nullptr;
  if (evecs) {
    SED_REQUIRE(ev_ld >= B.cat->n_orbits, 1, "eigenvector leading dimension must be at least the catalog's orbit count");
    const size_t bytes = (size_t)n_req * B.nev * ev_ld * 16;
    if (B.o_evecs.bytes < bytes) B.o_evecs.alloc(bytes);
    d_evecs = B.o_evecs.as<double>();
  }
  batch_launch_device(B, n_req, B.in_chi.as<double>(), B.in_phase.as<double>(), B.in_amp.as<double>(),
                      B.in_seed.as<uint64_t>(), tol, maxiter, B.o_evals.as<double>(), B.o_status.as<int32_t>(),
                      B.o_dims.as<int64_t>(), B.o_delta.as<double>(), B.o_nmv.as<int32_t>(), phase, d_evecs, ev_ld);
  if (evecs)
    SED_CUDA(cudaMemcpyAsync(evecs, d_evecs, (size_t)n_req * B.nev * ev_ld * 16, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaMemcpyAsync(evals, B.o_evals.p, (size_t)n_req * B.nev * 8, cudaMemcpyDeviceToHost, s));
  if (status) SED_CUDA(cudaMemcpyAsync(status, B.o_status.p, (size_t)n_req * 4, cudaMemcpyDeviceToHost, s));
  if (dims) SED_CUDA(cudaMemcpyAsync(dims, B.o_dims.p, (size_t)n_req * 8, cudaMemcpyDeviceToHost, s));
  if (delta) SED_CUDA(cudaMemcpyAsync(delta, B.o_delta.p, (size_t)n_req * 8, cudaMemcpyDeviceToHost, s));
  if (nmv) SED_CUDA(cudaMemcpyAsync(nmv, B.o_nmv.p, (size_t)n_req * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

// ------------------------------------------------------------ ring mode
// A device-resident request loop: one persistent launch of the batched kernel
// whose blocks claim requests from a ring as the host publishes them
// (k_batch's ring_* arguments).  A request starts as soon as a block is free,
// with no launch per batch; a block that stays idle for idle_ms leaves, and
// the host relaunches when work arrives while no block is left.  The ring
// uses the site-gauge hop table, which does not depend on the requests, so
// every request must have a site gauge.  A request whose mixed-precision
// polish missed its target is re-solved by an FP64 batch when collected.

template <class T>
static T* host_mapped(size_t n) {
  void* p = nullptr;
  SED_CUDA(cudaHostAlloc(&p, std::max<size_t>(n, 1) * sizeof(T), cudaHostAllocMapped));
  std::memset(p, 0, std::max<size_t>(n, 1) * sizeof(T));
  return static_cast<T*>(p);
}
template <class T>
static T* device_view(T* host) {
  void* d = nullptr;
  SED_CUDA(cudaHostGetDevicePointer(&d, host, 0));
  return static_cast<T*>(d);
}

void BatchImpl::ring_free() {
  Ring& r = ring;
  if (r.on && r.stop) {
    *reinterpret_cast<volatile int*>(r.stop) = 1;
    if (r.stream) cudaStreamSynchronize(r.stream);  // every block leaves within one idle wait
  }
  for (void* p : {(void*)r.tail, (void*)r.stop, (void*)r.done, (void*)r.evals, (void*)r.status, (void*)r.dims,
                  (void*)r.delta, (void*)r.nmv, (void*)r.hops, (void*)r.tns})
    if (p) cudaFreeHost(p);
  if (r.stream) cudaStreamDestroy(r.stream);
  if (r.copy) cudaStreamDestroy(r.copy);
  r = Ring{};
}

static void ring_launch(BatchImpl& B) {
  BatchImpl::Ring& r = B.ring;
  BatchSmem L = r.L;
  dispatch_launch(B, r.args, L, r.n_cta, r.stream, r.fp64 != 0);
  ++r.launches;
}

static bool ring_running(BatchImpl& B) {
  const cudaError_t e = cudaStreamQuery(B.ring.stream);
  if (e == cudaErrorNotReady) {
    cudaGetLastError();  // "not ready" is a state, not an error: leave no trace of it
    return true;
  }
  SED_CUDA(e);
  return false;
}

void batch_ring_start(BatchImpl& B, int cap, int n_blocks, int idle_ms) {
  std::lock_guard<std::mutex> lock(B.ring_mu);
  SED_REQUIRE(!B.ring.on, 1, "the ring is already running");
  SED_REQUIRE(cap >= 1 && cap <= (1 << 20), 1, "ring capacity must be between 1 and 2^20");
  SED_REQUIRE(n_blocks >= 1, 1, "n_blocks must be positive");
  SED_REQUIRE(idle_ms >= 1 && idle_ms <= 60000, 1, "idle_ms must be between 1 and 60000");
  SED_REQUIRE(B.phi_cap > 0 && B.tab_enabled, 5, "ring mode needs the shared-memory hop table of this catalog");
  const GroupImpl& G = *B.cat->group;
  cudaStream_t s = B.stream;
  SED_REQUIRE(prepare_table(B, 0, nullptr, s, true), 5, "ring mode needs the site-gauge hop table");
  SED_CUDA(cudaStreamSynchronize(s));
  BatchImpl::Ring& r = B.ring;
  r = BatchImpl::Ring{};
  // a failure below releases what was already allocated
  struct Undo {
    BatchImpl& B;
    bool armed = true;
    ~Undo() {
      if (armed) B.ring_free();
    }
  } undo{B};
  r.cap = cap;
  r.spin = (int)std::max<int64_t>(1, (int64_t)idle_ms * 1000 / 20);  // 20 us per idle wait
  r.fp64 = B.precision == 0 ? 1 : 0;
  r.tail = host_mapped<unsigned int>(1);
  r.stop = host_mapped<int>(1);
  r.done = host_mapped<unsigned int>(cap);
  r.evals = host_mapped<double>((size_t)cap * B.nev);
  r.status = host_mapped<int32_t>(cap);
  r.dims = host_mapped<int64_t>(cap);
  r.delta = host_mapped<double>(cap);
  r.nmv = host_mapped<int32_t>(cap);
  r.hops = host_mapped<int64_t>(cap);
  r.tns = host_mapped<int64_t>((size_t)cap * 2);
  r.chi.alloc((size_t)cap * G.n_ops * 16);
  r.phase.alloc((size_t)cap * G.n_ops * G.n_site * 16);
  r.amp.alloc((size_t)cap * std::max(B.n_bil, 1) * 16);
  r.seed.alloc((size_t)cap * 8);
  r.gw.alloc((size_t)cap * G.n_site * 16);
  r.head.alloc(16);
  SED_CUDA(cudaMemset(r.head.p, 0, 16));
  r.busy.assign(cap, 0);
  SED_CUDA(cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking));
  SED_CUDA(cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking));
  BatchArgs a = base_args(B);
  a.n_req = 0;
  a.tol = 1e-10;
  a.maxiter = 300;
  a.chi = r.chi.as<double2>();
  a.phase = r.phase.as<double2>();
  a.amp = r.amp.as<double2>();
  a.seeds = r.seed.as<uint64_t>();
  a.V = B.V.as<double2>();
  a.R = B.R.as<double2>();
  a.W = B.W.as<double2>();
  a.X64 = B.X64.as<double2>();
  a.tchi64 = B.tchi64.as<double2>();
  a.rowflag = B.rowflag.as<uint8_t>();
  a.evals = device_view(r.evals);
  a.status = device_view(r.status);
  a.dims = device_view(r.dims);
  a.delta = device_view(r.delta);
  a.nmv = device_view(r.nmv);
  a.hops = device_view(r.hops);
  a.t_ns = device_view(r.tns);
  a.queue = r.head.as<unsigned int>();
  a.use_tab = 1;
  a.gauge = 1;
  a.gauge_w = r.gw.as<double2>();
  a.n_phi = B.n_phi;
  a.hop = B.hop.as<uint64_t>();
  a.sl_off = B.sl_off.as<uint32_t>();
  a.sl_w = B.sl_w.as<int32_t>();
  a.phi_desc = B.phi_desc.as<uint32_t>();
  a.rep_site = B.rep_site.as<int8_t>();
  a.pwc64 = B.pwc64.as<double2>();
  // launch shape: pinned, from the environment, remembered for this catalog
  // shape, else the batch's default (no timing runs: there are no requests yet)
  int m = B.m, tpr = 1;
  if (B.pin_m > 0) {
    m = B.pin_m;
    tpr = B.pin_tpr;
  } else if (!env_batch_shape(&m, &tpr)) {
    const BatchShapeKey key{B.cat->n_orbits, B.tt.n_terms, G.n_ops, G.n_site, B.fermi ? 1 : 0, B.precision, B.nev,
                            1, 1, B.m_fixed ? B.m : 0};
    std::lock_guard<std::mutex> lock(g_bshape_mu);
    auto it = g_bshapes.find(key);
    if (it != g_bshapes.end()) {
      m = it->second.first;
      tpr = it->second.second;
    }
  }
  a.m = std::min(std::max(m, 2 * (B.nev + 2) + 1), B.m_cap);
  a.tpr = tpr == 2 ? 2 : 1;
  a.ring_tail = device_view(r.tail);
  a.ring_stop = device_view(r.stop);
  a.ring_done = device_view(r.done);
  a.ring_cap = cap;
  a.ring_spin = r.spin;
  BatchSmem L;
  int ncta = 1;
  dispatch_prepare(B, a, L, ncta, r.fp64 != 0);
  r.n_cta = std::min({ncta, n_blocks, B.n_cta});
  r.args = a;
  r.L = L;
  r.on = true;
  ++B.ring_gen;
  undo.armed = false;
}

int64_t batch_ring_submit(BatchImpl& B, const double* chi, const double* phase, const double* amp, uint64_t seed) {
  BatchImpl::Ring& r = B.ring;
  std::lock_guard<std::mutex> lock(B.ring_mu);
  SED_REQUIRE(r.on, 1, "the ring is not running");
  SED_REQUIRE(chi && phase && (B.n_bil == 0 || amp), 1, "NULL argument");
  const GroupImpl& G = *B.cat->group;
  validate_requests(B, 1, phase, amp);
  std::vector<double> w;
  SED_REQUIRE(site_gauges(G, 1, phase, w), 1,
              "ring mode needs a site gauge for every request (flux-twisted translation groups have one)");
  const unsigned int q = r.next;
  const int slot = (int)(q % (unsigned int)r.cap);
  SED_REQUIRE(!r.busy[slot], 5, "the request ring is full: collect finished requests first");
  const size_t nG = G.n_ops, N = G.n_site;
  SED_CUDA(cudaMemcpyAsync(r.chi.as<double>() + (size_t)slot * nG * 2, chi, nG * 16, cudaMemcpyHostToDevice, r.copy));
  SED_CUDA(cudaMemcpyAsync(r.phase.as<double>() + (size_t)slot * nG * N * 2, phase, nG * N * 16,
                           cudaMemcpyHostToDevice, r.copy));
  if (B.n_bil)
    SED_CUDA(cudaMemcpyAsync(r.amp.as<double>() + (size_t)slot * B.n_bil * 2, amp, (size_t)B.n_bil * 16,
                             cudaMemcpyHostToDevice, r.copy));
  SED_CUDA(cudaMemcpyAsync(r.seed.as<uint64_t>() + slot, &seed, 8, cudaMemcpyHostToDevice, r.copy));
  SED_CUDA(cudaMemcpyAsync(r.gw.as<double>() + (size_t)slot * N * 2, w.data(), N * 16, cudaMemcpyHostToDevice,
                           r.copy));
  SED_CUDA(cudaStreamSynchronize(r.copy));
  r.busy[slot] = 1;
  r.next = q + 1;
  __atomic_store_n(r.tail, q + 1, __ATOMIC_RELEASE);  // publish: the slot's inputs are in place
  if (!ring_running(B)) ring_launch(B);
  return (int64_t)q;
}

// true when the ticket has finished (outputs filled, ticket released)
bool batch_ring_wait(BatchImpl& B, int64_t ticket, int timeout_ms, double* evals, int32_t* status, int64_t* dim) {
  BatchImpl::Ring& r = B.ring;
  const unsigned int q = (unsigned int)ticket;
  int slot = 0;
  uint64_t gen = 0;
  // the ticket is still this caller's to collect: same ring, issued, its slot
  // not yet reused by a later ticket and not yet collected (mutex held)
  auto check_ticket = [&] {
    SED_REQUIRE(r.on && B.ring_gen == gen, 1, "the ring was stopped");
    SED_REQUIRE(ticket >= 0 && (uint64_t)ticket < (uint64_t)r.next &&
                    (uint64_t)r.next - (uint64_t)ticket <= (uint64_t)r.cap,
                1, "unknown ticket");
    slot = (int)(q % (unsigned int)r.cap);
    SED_REQUIRE(r.busy[slot], 1, "ticket already collected");
  };
  {
    std::lock_guard<std::mutex> lock(B.ring_mu);
    SED_REQUIRE(r.on, 1, "the ring is not running");
    gen = B.ring_gen;
    check_ticket();
  }
  const auto t0 = std::chrono::steady_clock::now();
  std::unique_lock<std::mutex> lock(B.ring_mu, std::defer_lock);
  for (;;) {
    lock.lock();
    check_ticket();
    if (__atomic_load_n(r.done + slot, __ATOMIC_ACQUIRE) == q + 1) break;  // collected below, lock held
    // the blocks leave when idle; relaunch if this request is still queued
    if (!ring_running(B)) ring_launch(B);
    lock.unlock();
    const double el = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (el >= timeout_ms) return false;
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  int32_t st = r.status[slot];
  for (int i = 0; i < B.nev; ++i) evals[i] = r.evals[(size_t)slot * B.nev + i];
  int64_t d = r.dims[slot];
  if (st == kPolishFailed) {
    // the FP64 batch answers this request (same inputs, same seed)
    if (!r.redo) {
      r.redo = make_batch(B.cat, B.n_bil, B.bil_ij.data(), B.n_den, B.den_ij.data(), B.den_v.data(), 0, B.nev, 0, 1);
    }
    const GroupImpl& G = *B.cat->group;
    std::vector<double> chi((size_t)G.n_ops * 2), ph((size_t)G.n_ops * G.n_site * 2), amp((size_t)std::max(B.n_bil, 1) * 2);
    uint64_t seed = 0;
    SED_CUDA(cudaMemcpy(chi.data(), r.chi.as<double>() + (size_t)slot * G.n_ops * 2, chi.size() * 8,
                        cudaMemcpyDeviceToHost));
    SED_CUDA(cudaMemcpy(ph.data(), r.phase.as<double>() + (size_t)slot * G.n_ops * G.n_site * 2, ph.size() * 8,
                        cudaMemcpyDeviceToHost));
    if (B.n_bil)
      SED_CUDA(cudaMemcpy(amp.data(), r.amp.as<double>() + (size_t)slot * B.n_bil * 2, (size_t)B.n_bil * 16,
                          cudaMemcpyDeviceToHost));
    SED_CUDA(cudaMemcpy(&seed, r.seed.as<uint64_t>() + slot, 8, cudaMemcpyDeviceToHost));
    double delta = 0;
    int32_t nmv = 0;
    batch_run(*r.redo, 1, chi.data(), ph.data(), amp.data(), &seed, 1e-10, 300, evals, &st, &d, &delta, &nmv);
  }
  if (status) *status = st;
  if (dim) *dim = d;
  r.busy[slot] = 0;
  return true;
}

void batch_ring_stop(BatchImpl& B) {
  std::lock_guard<std::mutex> lock(B.ring_mu);
  SED_REQUIRE(B.ring.on, 1, "the ring is not running");
  B.ring_free();
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

int sed_batch_last_info(const sed_batch* b, int32_t* n_fallback, int32_t* hop_table, int64_t* hop_records) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    if (n_fallback) *n_fallback = b->p->n_fallback;
    if (hop_table) *hop_table = b->p->last_tab;
    if (hop_records) *hop_records = b->p->last_tab ? b->p->hop_records : 0;
  });
}

int sed_batch_set_shape(sed_batch* b, int krylovdim, int threads_per_row) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    SED_REQUIRE((krylovdim == 0 && threads_per_row == 0) ||
                    (krylovdim >= 2 && krylovdim <= sed::kMaxM && (threads_per_row == 1 || threads_per_row == 2)),
                1, "batch shape must be (0, 0) or (krylovdim <= 32, 1 or 2 threads per row)");
    SED_REQUIRE(krylovdim <= b->p->m_cap, 1, "krylovdim above the batch's workspace (create it with that krylovdim)");
    b->p->pin_m = krylovdim;
    b->p->pin_tpr = threads_per_row;
  });
}
int sed_batch_shape(const sed_batch* b, int32_t* krylovdim, int32_t* threads_per_row, int32_t* tune_runs) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    if (krylovdim) *krylovdim = b->p->last_m;
    if (threads_per_row) *threads_per_row = b->p->last_tpr;
    if (tune_runs) *tune_runs = b->p->tune_runs;
  });
}
int sed_batch_set_site_gauge(sed_batch* b, int enable) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    b->p->gauge_enabled = enable != 0;
  });
}
int sed_batch_last_gauge(const sed_batch* b, int32_t* gauge) {
  return bguard([&] {
    SED_REQUIRE(b && gauge, 1, "NULL argument");
    *gauge = b->p->last_gauge;
  });
}
int sed_batch_set_hop_table(sed_batch* b, int enable) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    b->p->tab_enabled = enable != 0;
  });
}

int sed_batch_run_vectors(sed_batch* b, int n_req, const double* chi_reim, const double* group_phase_reim,
                          const double* bil_t_reim, const uint64_t* seeds, double tol, int maxiter, double* evals,
                          int32_t* status, int64_t* dims, double* delta_polish, int32_t* n_matvec,
                          double* evecs_reim, int64_t ld) {
  return bguard([&] {
    SED_REQUIRE(b && evecs_reim, 1, "NULL argument");
    sed::batch_run(*b->p, n_req, chi_reim, group_phase_reim, bil_t_reim, seeds, tol, maxiter, evals, status, dims,
                   delta_polish, n_matvec, evecs_reim, ld);
  });
}
int sed_batch_run_device_vectors(sed_batch* b, int n_req, const double* d_chi, const double* d_group_phase,
                                 const double* d_bil_t, const uint64_t* d_seeds, double tol, int maxiter,
                                 double* d_evals, int32_t* d_status, int64_t* d_dims, double* d_delta,
                                 int32_t* d_n_matvec, double* d_evecs, int64_t ld) {
  return bguard([&] {
    SED_REQUIRE(b && d_evecs, 1, "NULL argument");
    sed::batch_launch_device(*b->p, n_req, d_chi, d_group_phase, d_bil_t, d_seeds, tol, maxiter, d_evals, d_status,
                             d_dims, d_delta, d_n_matvec, nullptr, d_evecs, ld);
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

int sed_batch_ring_start(sed_batch* b, int capacity, int n_blocks, int idle_ms) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    sed::batch_ring_start(*b->p, capacity, n_blocks, idle_ms);
  });
}
int sed_batch_ring_submit(sed_batch* b, const double* chi_reim, const double* group_phase_reim,
                          const double* bil_t_reim, uint64_t seed, int64_t* ticket) {
  return bguard([&] {
    SED_REQUIRE(b && ticket, 1, "NULL argument");
    *ticket = sed::batch_ring_submit(*b->p, chi_reim, group_phase_reim, bil_t_reim, seed);
  });
}
int sed_batch_ring_wait(sed_batch* b, int64_t ticket, int timeout_ms, double* evals, int32_t* status,
                        int64_t* dim) {
  return bguard([&] {
    SED_REQUIRE(b && evals, 1, "NULL argument");
    SED_REQUIRE(sed::batch_ring_wait(*b->p, ticket, std::max(timeout_ms, 0), evals, status, dim), SED_ERR_TIMEOUT,
                "request not finished");
  });
}
int sed_batch_ring_info(const sed_batch* b, int64_t* launches, int32_t* n_blocks, int32_t* running) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    sed::BatchImpl& B = *b->p;
    std::lock_guard<std::mutex> lock(B.ring_mu);
    if (launches) *launches = B.ring.launches;
    if (n_blocks) *n_blocks = B.ring.n_cta;
    if (running) *running = B.ring.on && B.ring.stream && cudaStreamQuery(B.ring.stream) == cudaErrorNotReady;
    cudaGetLastError();  // the query's not-ready status is not an error
  });
}
int sed_batch_ring_stop(sed_batch* b) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    sed::batch_ring_stop(*b->p);
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

int sed_batch_set_x_in_shared_memory(sed_batch* b, int enable) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    sed::BatchImpl& B = *b->p;
    if (enable && !B.x_smem) {
      sed::BatchArgs a = sed::base_args(B);
      SED_REQUIRE(B.precision == 1 && sed::batch_layout<float2>(a, true).total <= 220 * 1024, 5,
                  "the matvec input does not fit in shared memory beside this batch's tables");
    }
    B.x_smem = B.precision == 1 && enable != 0;
  });
}
int sed_batch_graph_info(const sed_batch* b, int* captures, int* replays) {
  return bguard([&] {
    SED_REQUIRE(b, 1, "NULL batch");
    if (captures) *captures = b->p->graph_captures;
    if (replays) *replays = b->p->graph_replays;
  });
}
void sed_batch_destroy(sed_batch* b) { delete b; }

}  // extern "C"
