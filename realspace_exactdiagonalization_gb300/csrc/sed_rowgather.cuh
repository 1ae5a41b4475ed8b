// sed_rowgather.cuh -- one row of the sector Hamiltonian, gathered.
//
// Shared by the device-wide matvec (sed_hamiltonian.cu) and the batched
// per-CTA solver (sed_batched.cu).  For the representative m of row r it walks
// the hops out of m (occupied site i -> empty site j, hop records grouped by
// from-site), and accumulates conj(H_cr) xs_c:
//   coef = tchi[u][h] * sign * conj(P_h(new)),  tchi[u][h] = conj(t_u) chi(h)
// (reference: apply_hamiltonian!, src/symmetry_resolved_ed.jl:813-878, whose
// column element is t * s_JW * alpha * conj(chi) * sqrt(stab_row/stab_col)).
// The hop walk is software-pipelined: the state-table load of the next hop is
// issued before the current hop is consumed, so every thread keeps two
// independent random loads in flight.
#pragma once

#include "sed_internal.cuh"

namespace sed {

struct P64 {
  using V = double2;
  using S = double;
  __device__ static __forceinline__ V make(S a, S b) { return make_double2(a, b); }
  __device__ static __forceinline__ S mad(S a, S b, S c) { return fma(a, b, c); }
  // x or -x by the sign bit alone (integer XOR on the high words, no FP64 op)
  __device__ static __forceinline__ V flip(V x, int neg) {
    const long long m = (long long)((unsigned long long)neg << 63);
    return make_double2(__longlong_as_double(__double_as_longlong(x.x) ^ m),
                        __longlong_as_double(__double_as_longlong(x.y) ^ m));
  }
};
struct P32 {
  using V = float2;
  using S = float;
  __device__ static __forceinline__ V make(S a, S b) { return make_float2(a, b); }
  __device__ static __forceinline__ S mad(S a, S b, S c) { return fmaf(a, b, c); }
  __device__ static __forceinline__ V flip(V x, int neg) {
    const unsigned m = (unsigned)neg << 31;
    return make_float2(__uint_as_float(__float_as_uint(x.x) ^ m), __uint_as_float(__float_as_uint(x.y) ^ m));
  }
};

// Iterator over the valid hops of one representative.
struct HopIter {
  uint64_t m, occ;
  int i, t, t1;
  __device__ __forceinline__ void init(uint64_t m_, const uint16_t* s_off) {
    m = m_;
    occ = m_;
    i = -1;
    t = t1 = 0;
  }
  // advance to the next hop with an empty target; false when exhausted
  __device__ __forceinline__ bool next(const uint16_t* s_off, const uint32_t* s_rec, uint32_t& rec, int& from) {
    for (;;) {
      while (t < t1) {
        const uint32_t r = s_rec[t++];
        if (!((m >> (r & 0xFF)) & 1ULL)) {
          rec = r;
          from = i;
          return true;
        }
      }
      if (!occ) return false;
      i = __ffsll((long long)occ) - 1;
      occ &= occ - 1;
      t = s_off[i];
      t1 = s_off[i + 1];
    }
  }
};

// Phase classes of a twisted group element h: its per-site phases take at
// most kMaxCls + 1 distinct values.  With the most frequent one as base,
// P_h(new) = base^k * prod_c r_c^popcount(new & mask_c); base^k is folded
// into tchi, and r_c^n (n = 0..k) is tabulated, so a hop costs kMaxCls
// popcounts and table reads instead of k complex products.  Unused classes
// have an empty mask and r^0 = 1.
static constexpr int kMaxCls = 3;
template <class V>
struct PhaseClasses {
  int mode;             // 0: no phases, 1: class tables, 2: per-site product (eta)
  int kp1;              // k + 1
  const uint64_t* mask; // [G][kMaxCls]
  const V* pw;          // [G][kMaxCls][k+1]
};

template <class P, bool FERMI, bool PHASES, bool TABLE>
__device__ __forceinline__ void row_gather(uint64_t m, const typename P::V* __restrict__ xs,
                                           const typename P::V* tab,  // TABLE ? tchi[u][G] : conj(t_u)
                                           const typename P::V* chi, int G, const typename P::V* __restrict__ eta,
                                           int N, const uint32_t* s_rank, const RankParams& rp,
                                           const uint32_t* s_rec, const uint16_t* s_off, const uint8_t* s_inv,
                                           const uint64_t* __restrict__ state, typename P::S& ar,
                                           typename P::S& ai,
                                           const PhaseClasses<typename P::V>& pc = PhaseClasses<typename P::V>{}) {
  using V = typename P::V;
  using S = typename P::S;
  HopIter it;
  it.init(m, s_off);
  uint32_t rec_n;
  int from_n;
  bool have = it.next(s_off, s_rec, rec_n, from_n);
  uint64_t w_n = 0;
  uint64_t nw_n = 0;
  if (have) {
    nw_n = m ^ ((1ULL << from_n) | (1ULL << (rec_n & 0xFF)));
    w_n = __ldg(state + dev::rank_of(nw_n, s_rank, rp));
  }
  while (have) {
    const uint32_t rec = rec_n;
    const int i = from_n;
    const uint64_t nw = nw_n;
    const uint64_t w = w_n;
    // prefetch the next hop's state word
    have = it.next(s_off, s_rec, rec_n, from_n);
    if (have) {
      nw_n = m ^ ((1ULL << from_n) | (1ULL << (rec_n & 0xFF)));
      w_n = __ldg(state + dev::rank_of(nw_n, s_rank, rp));
    }
    const int j = rec & 0xFF;
    const uint32_t c = (uint32_t)w;
    int neg = (int)((w >> 40) & 1);
    const V xc = xs[c];
    const int h = (int)((w >> 48) & 0xFF);  // inverse of the state's group element
    const int u = (int)(rec >> 8);
    V cf;
    if (TABLE) {
      cf = tab[u * G + h];
    } else {
      const V tt = tab[u], ch = chi[h];  // tt holds conj(t_u)
      cf = P::make(tt.x * ch.x - tt.y * ch.y, tt.x * ch.y + tt.y * ch.x);
    }
    if (FERMI) neg ^= __popcll(m & dev::bits_between(i, j)) & 1;
    if (PHASES) {
      S pr = 1, pi = 0;
      if (pc.mode == 1) {
        const uint64_t* mk = pc.mask + h * kMaxCls;
        const V* pw = pc.pw + (size_t)h * kMaxCls * pc.kp1;
#pragma unroll
        for (int cl = 0; cl < kMaxCls; ++cl) {
          const V e = pw[cl * pc.kp1 + __popcll(nw & mk[cl])];
          const S nr = pr * e.x - pi * e.y;
          pi = pr * e.y + pi * e.x;
          pr = nr;
        }
      } else if (pc.mode == 2) {
        uint64_t b = nw;
        const V* eh = eta + (size_t)h * N;
        while (b) {
          const int q = __ffsll((long long)b) - 1;
          b &= b - 1;
          const V e = eh[q];
          const S nr = pr * e.x - pi * e.y;
          pi = pr * e.y + pi * e.x;
          pr = nr;
        }
      }
      cf = P::make(cf.x * pr + cf.y * pi, cf.y * pr - cf.x * pi);  // * conj(P)
    }
    // (ar, ai) += sign * cf * xc as four fused multiply-adds, the sign
    // applied to xc's bits
    const V xq = P::flip(xc, neg);
    ar = P::mad(cf.x, xq.x, ar);
    ar = P::mad(-cf.y, xq.y, ar);
    ai = P::mad(cf.x, xq.y, ai);
    ai = P::mad(cf.y, xq.x, ai);
  }
}

// The same row split over TPR lanes: lane q of the row's group takes the
// hops whose index in the row's hop order is q mod TPR (the enumeration itself
// is cheap; the rank lookup, state word, gather and multiply-adds are not).
// The lanes' partial sums are combined by the caller.
template <class P, bool FERMI, bool PHASES, bool TABLE>
__device__ __forceinline__ void row_gather_split(uint64_t m, int q, int tpr, const typename P::V* __restrict__ xs,
                                                 const typename P::V* tab, const typename P::V* chi, int G,
                                                 const typename P::V* __restrict__ eta, int N,
                                                 const uint32_t* s_rank, const RankParams& rp,
                                                 const uint32_t* s_rec, const uint16_t* s_off,
                                                 const uint64_t* __restrict__ state, typename P::S& ar,
                                                 typename P::S& ai, const PhaseClasses<typename P::V>& pc) {
  using V = typename P::V;
  using S = typename P::S;
  HopIter it;
  it.init(m, s_off);
  uint32_t rec;
  int i;
  int t = 0;
  while (it.next(s_off, s_rec, rec, i)) {
    if ((t++ % tpr) != q) continue;
    const int j = rec & 0xFF;
    const uint64_t nw = m ^ ((1ULL << i) | (1ULL << j));
    const uint64_t w = __ldg(state + dev::rank_of(nw, s_rank, rp));
    const uint32_t c = (uint32_t)w;
    int neg = (int)((w >> 40) & 1);
    const V xc = xs[c];
    const int h = (int)((w >> 48) & 0xFF);
    const int u = (int)(rec >> 8);
    V cf;
    if (TABLE) {
      cf = tab[u * G + h];
    } else {
      const V tt = tab[u], ch = chi[h];
      cf = P::make(tt.x * ch.x - tt.y * ch.y, tt.x * ch.y + tt.y * ch.x);
    }
    if (FERMI) neg ^= __popcll(m & dev::bits_between(i, j)) & 1;
    if (PHASES) {
      S pr = 1, pi = 0;
      if (pc.mode == 1) {
        const uint64_t* mk = pc.mask + h * kMaxCls;
        const V* pw = pc.pw + (size_t)h * kMaxCls * pc.kp1;
#pragma unroll
        for (int cl = 0; cl < kMaxCls; ++cl) {
          const V e = pw[cl * pc.kp1 + __popcll(nw & mk[cl])];
          const S nr = pr * e.x - pi * e.y;
          pi = pr * e.y + pi * e.x;
          pr = nr;
        }
      } else if (pc.mode == 2) {
        uint64_t b = nw;
        const V* eh = eta + (size_t)h * N;
        while (b) {
          const int qq = __ffsll((long long)b) - 1;
          b &= b - 1;
          const V e = eh[qq];
          const S nr = pr * e.x - pi * e.y;
          pi = pr * e.y + pi * e.x;
          pr = nr;
        }
      }
      cf = P::make(cf.x * pr + cf.y * pi, cf.y * pr - cf.x * pi);
    }
    const V xq = P::flip(xc, neg);
    ar = P::mad(cf.x, xq.x, ar);
    ar = P::mad(-cf.y, xq.y, ar);
    ai = P::mad(cf.x, xq.y, ai);
    ai = P::mad(cf.y, xq.x, ai);
  }
}

}  // namespace sed
