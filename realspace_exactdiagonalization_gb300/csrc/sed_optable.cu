// sed_optable.cu -- the operator's hop table: the stored form of the sector matvec.
//
// A Lanczos solve applies the same sector Hamiltonian hundreds of times.  The
// reference prepares for that by building a projection table once
// (build_matrixfree_projection_table, src/symmetry_resolved_ed.jl:680-728: one
// (row, col, H_elem) triple of 32 bytes per hop) and streaming it in
// _apply_table! (:731-765).  GB300's 288 GB of HBM hold the same information
// compressed to 8 bytes per hop:
//   c (28 bits) | cid (36 bits) << 28,   cid = u * n_phi + phi,
// the column orbit and the index of the hop's coefficient
//   conj(t_u) chi(h) conj(base_h^k) conj(prod_c r_{h,c}^{n_c}) (-1)^neg,
// which depends only on the amplitude class u, the group element h, the
// twist-phase class counts n_1..n_3 of the new mask and the sign.  phi =
// ((h * P + n_1 + kp1 (n_2 + kp1 n_3)) << 1) | neg with P = kp1^K for the K
// classes in use, so the coefficient table is dense and small (|G| x 2 x the
// amplitude classes without a twist).  Rows are stored SELL-32 (slice s holds
// orbit rows 32s..32s+31, record k of row 32s+l at sl_off[s] + 32k + l) and
// padded with records pointing at a zero coefficient.
//
// The matvec then streams 8 bytes per hop with evict-first loads (they are
// read once per matvec and should not displace x from L2), gathers x and does
// four fused multiply-adds: no rank lookups, no state-table reads, no
// popcounts.  The table is built on the first solve of an operator when it
// fits the memory budget; sed_op_set_hop_table switches it off or builds it
// at once.
#include <algorithm>
#include <cmath>
#include <complex>
#include <mutex>
#include <vector>

#include "sed_internal.cuh"
#include "sed_rowgather.cuh"

namespace sed {

namespace {

constexpr int kTabBS = 512;
constexpr int kCBits = 28;
constexpr uint64_t kCMask = (1ULL << kCBits) - 1ULL;

__global__ void k_optab_count(int64_t n_orb, const uint64_t* __restrict__ reps, const uint8_t* __restrict__ rowflag,
                              const uint16_t* __restrict__ off, const uint32_t* __restrict__ rec,
                              int32_t* __restrict__ width) {
  // one thread per slice: the slice width is the longest of its 32 rows
  const int64_t n_sl = (n_orb + 31) / 32;
  for (int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; sl < n_sl; sl += (int64_t)gridDim.x * blockDim.x) {
    int w = 0;
    for (int64_t o = sl * 32; o < min(n_orb, sl * 32 + 32); ++o) {
      if (!rowflag[o]) continue;
      const uint64_t m = reps[o];
      uint64_t occ = m;
      int c = 0;
      while (occ) {
        const int i = __ffsll((long long)occ) - 1;
        occ &= occ - 1;
        for (int t = off[i]; t < off[i + 1]; ++t) c += !((m >> (rec[t] & 0xFF)) & 1ULL);
      }
      w = max(w, c);
    }
    width[sl] = w;
  }
}

// The rank table, the term records, the site offsets and the class masks
// are staged in shared memory (dynamic: rank | rec | mask | off), like the
// gather matvec's: every hop looks up one rank-table entry per byte of the
// target state, at addresses that differ across the warp.
struct FillSmem {
  size_t rank, rec, mask, off, total;
};
static FillSmem fill_layout(int rank_total, int n_terms, int n_mask, int n_site) {
  FillSmem L{};
  auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
  L.rank = 0;
  L.rec = al((size_t)rank_total * 4);
  L.mask = al(L.rec + (size_t)n_terms * 4);
  L.off = al(L.mask + (size_t)n_mask * 8);
  L.total = al(L.off + (size_t)(n_site + 1) * 2);
  return L;
}

template <bool FERMI>
__global__ void k_optab_fill(int64_t n_orb, const uint64_t* __restrict__ reps, const uint8_t* __restrict__ rowflag,
                             const uint64_t* __restrict__ state, const uint32_t* __restrict__ rank_tab, RankParams rp,
                             const uint16_t* __restrict__ off_g, int n_site, const uint32_t* __restrict__ rec_g,
                             int n_terms, const uint64_t* __restrict__ mask_g, int n_mask, FillSmem L, int K, int kp1,
                             int P, int64_t n_phi, uint64_t zero_cid, const int64_t* __restrict__ sl_off,
                             const int32_t* __restrict__ sl_w, uint64_t* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* s_rank = reinterpret_cast<uint32_t*>(smem + L.rank);
  uint32_t* rec = reinterpret_cast<uint32_t*>(smem + L.rec);
  uint64_t* mask = reinterpret_cast<uint64_t*>(smem + L.mask);
  uint16_t* off = reinterpret_cast<uint16_t*>(smem + L.off);
  for (int i = threadIdx.x; i < rp.total; i += blockDim.x) s_rank[i] = rank_tab[i];
  for (int i = threadIdx.x; i < n_terms; i += blockDim.x) rec[i] = rec_g[i];
  for (int i = threadIdx.x; i < n_mask; i += blockDim.x) mask[i] = mask_g[i];
  for (int i = threadIdx.x; i <= n_site; i += blockDim.x) off[i] = off_g[i];
  __syncthreads();
  // one warp per slice, its 32 lanes the slice's rows, in lockstep over the
  // slice's record positions: each position is stored by the whole warp at
  // once (256 contiguous bytes), and the next hop's state word is loaded one
  // hop ahead.  Lanes past the last row write padding records.
  const int lane = threadIdx.x & 31;
  const int64_t n_sl = (n_orb + 31) / 32;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t sl = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); sl < n_sl; sl += warps) {
    const int64_t o = sl * 32 + lane;
    uint64_t* dst = out + sl_off[sl] + lane;
    const int wdt = sl_w[sl];
    const uint64_t m = o < n_orb ? reps[o] : 0;
    HopIter it;
    it.init(m, off);
    uint32_t r_n = 0;
    int from_n = 0;
    uint64_t nw_n = 0, wd_n = 0;
    bool have = o < n_orb && rowflag[o] && it.next(off, rec, r_n, from_n);
    if (have) {
      nw_n = m ^ ((1ULL << from_n) | (1ULL << (r_n & 0xFF)));
      wd_n = __ldg(state + dev::rank_of(nw_n, s_rank, rp));
    }
    for (int k = 0; k < wdt; ++k) {
      uint64_t word = zero_cid << kCBits;
      if (have) {
        const uint32_t r = r_n;
        const int from = from_n;
        const uint64_t nw = nw_n, wd = wd_n;
        have = it.next(off, rec, r_n, from_n);
        if (have) {
          nw_n = m ^ ((1ULL << from_n) | (1ULL << (r_n & 0xFF)));
          wd_n = __ldg(state + dev::rank_of(nw_n, s_rank, rp));
        }
        const int j = r & 0xFF;
        int neg = (int)((wd >> 40) & 1);
        if (FERMI) neg ^= __popcll(m & dev::bits_between(from, j)) & 1;
        const int h = (int)((wd >> 48) & 0xFF);
        int pidx = 0, scale = 1;
        for (int c = 0; c < K; ++c) {
          pidx += scale * __popcll(nw & mask[h * kMaxCls + c]);
          scale *= kp1;
        }
        const uint64_t phi = ((uint64_t)(h * P + pidx) << 1) | (uint64_t)neg;
        const uint64_t cid = (uint64_t)(r >> 8) * (uint64_t)n_phi + phi;
        word = ((uint64_t)(uint32_t)wd & kCMask) | (cid << kCBits);
      }
      __syncwarp();
      dst[32 * (int64_t)k] = word;
    }
  }
}

// CF: the row is stored as complex64, the form the mixed-precision Lanczos
// keeps its vectors in (y is then read as float2)
template <class P, bool CF = false>
__global__ void __launch_bounds__(kTabBS) k_apply_tab(int64_t n_orb, const uint64_t* __restrict__ hop,
                                                      const int64_t* __restrict__ sl_off,
                                                      const int32_t* __restrict__ sl_w,
                                                      const typename P::V* __restrict__ coef, int smem_coef,
                                                      const typename P::V* __restrict__ xs,
                                                      const double2* __restrict__ diag,
                                                      const uint8_t* __restrict__ rowflag,
                                                      const uint8_t* __restrict__ stab, double2* __restrict__ y) {
  using V = typename P::V;
  using S = typename P::S;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double s_isr[65];
  V* s_coef = reinterpret_cast<V*>(smem);
  for (int i = threadIdx.x; i < 65; i += blockDim.x) s_isr[i] = i ? 1.0 / sqrt((double)i) : 0.0;
  for (int i = threadIdx.x; i < smem_coef; i += blockDim.x) s_coef[i] = coef[i];
  __syncthreads();
  const V* cf_tab = smem_coef ? s_coef : coef;
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // a row's flag, slice offset and width are loaded one grid-stride step
  // ahead, so a row waits on one DRAM round trip (its first records) instead
  // of three dependent ones
  int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint8_t flag = 0;
  int64_t off = 0;
  int wdt = 0;
  if (o < n_orb) {
    flag = rowflag[o];
    off = sl_off[o >> 5];
    wdt = sl_w[o >> 5];
  }
  for (; o < n_orb; o += stride) {
    const int64_t on = o + stride;
    uint8_t flag_n = 0;
    int64_t off_n = 0;
    int wdt_n = 0;
    if (on < n_orb) {
      flag_n = rowflag[on];
      off_n = sl_off[on >> 5];
      wdt_n = sl_w[on >> 5];
    }
    if (!flag) {
      if (CF)
        reinterpret_cast<float2*>(y)[o] = make_float2(0.f, 0.f);
      else
        y[o] = make_double2(0.0, 0.0);
    } else {
      const uint64_t* rp = hop + off + lane;
      const uint8_t st = stab[o];
      const double2 dg = diag[o];
      const V xo = xs[o];
      S ar = (S)dg.x * xo.x - (S)dg.y * xo.y;
      S ai = (S)dg.x * xo.y + (S)dg.y * xo.x;
#pragma unroll 8
      for (int k = 0; k < wdt; ++k) {
        const uint64_t r = __ldcs(reinterpret_cast<const unsigned long long*>(rp + 32 * (int64_t)k));
        const V cf = cf_tab[r >> kCBits];
        const V xc = xs[r & kCMask];
        ar = P::mad(cf.x, xc.x, ar);
        ar = P::mad(-cf.y, xc.y, ar);
        ai = P::mad(cf.x, xc.y, ai);
        ai = P::mad(cf.y, xc.x, ai);
      }
      const double is = s_isr[st];
      const double yr = (double)ar * is, yi = (double)ai * is;
      if (CF) {
        reinterpret_cast<float2*>(y)[o] = make_float2((float)yr, (float)yi);
      } else {
        y[o] = make_double2(yr, yi);
      }
    }
    flag = flag_n;
    off = off_n;
    wdt = wdt_n;
  }
}

}  // namespace

// Build the table; false (and nothing allocated) when the operator's twist
// needs the per-site phase product, a field would overflow, or the table
// would exceed the memory budget.
bool op_build_table(OpImpl& op) {
  const SectorImpl& S = *op.sec;
  const CatalogImpl& C = *S.cat;
  const GroupImpl& G = *S.group;
  const TermTables& tt = op.terms;
  cudaStream_t s = op.stream;
  const int64_t n = C.n_orbits;
  if (n == 0 || op.pc.mode == 2 || n > (int64_t)kCMask) return false;
  const int nG = G.n_ops, kp1 = op.pc.kp1;
  int K = 0;  // classes in use
  for (int h = 0; h < nG; ++h)
    for (int c = 0; c < kMaxCls; ++c)
      if (op.pc.mask[(size_t)h * kMaxCls + c]) K = std::max(K, c + 1);
  int64_t P = 1;
  for (int c = 0; c < K; ++c) P *= kp1;
  const int64_t n_phi = (int64_t)nG * P * 2;
  const int64_t n_coef = (int64_t)tt.n_class * n_phi + 1;  // + the zero coefficient
  if (n_coef > (1LL << 22)) return false;                 // 64 MB of FP64 coefficients
  // slice widths and the record count
  const int64_t n_sl = (n + 31) / 32;
  DevBuf wd((size_t)n_sl * 4);
  k_optab_count<<<grid1(n_sl, 256), 256, 0, s>>>(n, C.reps.as<uint64_t>(), S.rowflag.as<uint8_t>(),
                                                 op.site_off.as<uint16_t>(), op.rec.as<uint32_t>(), wd.as<int32_t>());
  SED_CUDA(cudaGetLastError());
  std::vector<int32_t> w(n_sl);
  SED_CUDA(cudaMemcpyAsync(w.data(), wd.p, (size_t)n_sl * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
  std::vector<int64_t> off(n_sl);
  int64_t tot = 0;
  for (int64_t i = 0; i < n_sl; ++i) {
    off[i] = tot;
    tot += 32 * (int64_t)w[i];
  }
  size_t free_b = 0, total_b = 0;
  SED_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const double bytes = (double)tot * 8 + (double)n_sl * 12 + (double)n_coef * 24;
  if (bytes > 0.35 * (double)free_b || bytes > 64e9) return false;
  // coefficients in the order the on-the-fly gather rounds them: tchi[u][h]
  // (conj(t_u) chi(h) conj(base^k)), times conj(prod_c r_c^(n_c)), times the sign
  std::vector<double> c64((size_t)n_coef * 2, 0.0);
  for (int u = 0; u < tt.n_class; ++u) {
    const std::complex<double> t(tt.amp[2 * u], -tt.amp[2 * u + 1]);
    for (int h = 0; h < nG; ++h) {
      const std::complex<double> br(op.pc.base_k[2 * h], -op.pc.base_k[2 * h + 1]);
      const std::complex<double> ch(S.chi[2 * h], S.chi[2 * h + 1]);
      const std::complex<double> chib(ch.real() * br.real() - ch.imag() * br.imag(),
                                      ch.real() * br.imag() + ch.imag() * br.real());
      const std::complex<double> tchi(t.real() * chib.real() - t.imag() * chib.imag(),
                                      t.real() * chib.imag() + t.imag() * chib.real());
      for (int64_t pidx = 0; pidx < P; ++pidx) {
        double pr = 1.0, pi = 0.0;
        int64_t rem = pidx;
        for (int c = 0; c < K; ++c) {
          const int e = (int)(rem % kp1);
          rem /= kp1;
          const size_t idx = (((size_t)h * kMaxCls + c) * kp1 + e) * 2;
          const double er = op.pc.pw[idx], ei = op.pc.pw[idx + 1];
          const double nr = pr * er - pi * ei;
          pi = pr * ei + pi * er;
          pr = nr;
        }
        // tchi * conj(P')
        const double cr = tchi.real() * pr + tchi.imag() * pi, ci = tchi.imag() * pr - tchi.real() * pi;
        for (int neg = 0; neg < 2; ++neg) {
          const int64_t cid = (int64_t)u * n_phi + (((int64_t)h * P + pidx) << 1 | neg);
          c64[2 * cid] = neg ? -cr : cr;
          c64[2 * cid + 1] = neg ? -ci : ci;
        }
      }
    }
  }
  std::vector<float> c32(c64.size());
  for (size_t i = 0; i < c64.size(); ++i) c32[i] = (float)c64[i];
  upload(op.tab_coef64, c64, s);
  upload(op.tab_coef32, c32, s);
  upload(op.tab_off, off, s);
  upload(op.tab_w, w, s);
  op.tab_hop.alloc((size_t)std::max<int64_t>(tot, 1) * 8);
  const int n_terms = tt.n_terms, n_mask = nG * kMaxCls;
  const FillSmem L = fill_layout(C.rank.rp.total, n_terms, n_mask, G.n_site);
  auto fill = G.stats == 1 ? k_optab_fill<true> : k_optab_fill<false>;
  {
    // the shared-memory opt-in is a property of the kernel on each device,
    // shared by every operator and host thread: raise it (never lower it) and
    // launch under one lock, so a concurrent build with a smaller rank table
    // cannot undercut this launch
    static std::mutex mu;
    static SmemOptIn optin[2];
    std::lock_guard<std::mutex> lock(mu);
    optin[G.stats == 1 ? 1 : 0].ensure(fill, L.total);
    int per_sm = 1;
    SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill, 512, L.total));
    const int fgrid = (int)std::max<int64_t>(
        1, std::min<int64_t>((n_sl + 15) / 16, (int64_t)device_sm_count() * std::max(per_sm, 1)));
    fill<<<fgrid, 512, L.total, s>>>(n, C.reps.as<uint64_t>(), S.rowflag.as<uint8_t>(), C.state.as<uint64_t>(),
                                     C.rank.dev.as<uint32_t>(), C.rank.rp, op.site_off.as<uint16_t>(), G.n_site,
                                     op.rec.as<uint32_t>(), n_terms, op.cls_mask.as<uint64_t>(), n_mask, L, K, kp1,
                                     (int)P, n_phi, (uint64_t)(n_coef - 1), op.tab_off.as<int64_t>(),
                                     op.tab_w.as<int32_t>(), op.tab_hop.as<uint64_t>());
    SED_CUDA(cudaGetLastError());
  }
  SED_CUDA(cudaStreamSynchronize(s));
  op.tab_records = tot;
  op.tab_coefs = n_coef;
  op.tab_built = true;
  return true;
}

void op_drop_table(OpImpl& op) {
  op.tab_built = false;
  op.tab_hop = DevBuf();
  op.tab_off = DevBuf();
  op.tab_w = DevBuf();
  op.tab_coef64 = DevBuf();
  op.tab_coef32 = DevBuf();
  op.tab_records = op.tab_coefs = 0;
}

void apply_table(OpImpl& op, bool fp32, const void* xs, double* ypad, cudaStream_t s, bool cf_out) {
  const SectorImpl& S = *op.sec;
  const CatalogImpl& C = *S.cat;
  const int64_t n = C.n_orbits;
  const size_t el = fp32 ? 8 : 16;
  // coefficients staged in shared memory when they fit the default 48 KB
  // (with the kernel's 520 bytes of static shared memory)
  const int smem_coef = op.tab_coefs * el <= 44 * 1024 ? (int)op.tab_coefs : 0;
  const size_t smem = (size_t)smem_coef * el;
  // one full wave of resident blocks: the kernel is bound by the latency of
  // its record and gather loads, so every resident warp helps
  const int64_t want = (n + kTabBS - 1) / kTabBS;
  int per_sm = 1;
  if (fp32 && cf_out)
    SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_tab<P32, true>, kTabBS, smem));
  else if (fp32)
    SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_tab<P32>, kTabBS, smem));
  else
    SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_tab<P64>, kTabBS, smem));
  const int grid =
      (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)op_sm_count(op) * std::max(per_sm, 1)));
  if (fp32 && cf_out)
    k_apply_tab<P32, true><<<grid, kTabBS, smem, s>>>(n, op.tab_hop.as<uint64_t>(), op.tab_off.as<int64_t>(),
                                                      op.tab_w.as<int32_t>(), op.tab_coef32.as<float2>(), smem_coef,
                                                      (const float2*)xs, op.diag.as<double2>(),
                                                      S.rowflag.as<uint8_t>(), C.stab.as<uint8_t>(), (double2*)ypad);
  else if (fp32)
    k_apply_tab<P32><<<grid, kTabBS, smem, s>>>(n, op.tab_hop.as<uint64_t>(), op.tab_off.as<int64_t>(),
                                                op.tab_w.as<int32_t>(), op.tab_coef32.as<float2>(), smem_coef,
                                                (const float2*)xs, op.diag.as<double2>(), S.rowflag.as<uint8_t>(),
                                                C.stab.as<uint8_t>(), (double2*)ypad);
  else
    k_apply_tab<P64><<<grid, kTabBS, smem, s>>>(n, op.tab_hop.as<uint64_t>(), op.tab_off.as<int64_t>(),
                                                op.tab_w.as<int32_t>(), op.tab_coef64.as<double2>(), smem_coef,
                                                (const double2*)xs, op.diag.as<double2>(), S.rowflag.as<uint8_t>(),
                                                C.stab.as<uint8_t>(), (double2*)ypad);
  SED_CUDA(cudaGetLastError());
}

}  // namespace sed
