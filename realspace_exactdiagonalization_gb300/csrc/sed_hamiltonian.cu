// sed_hamiltonian.cu -- the matrix-free sector Hamiltonian H|psi> on the GPU.
//
// Replaces apply_hamiltonian! (SRE:804-878) and the MatrixFreeHamiltonian
// functor (SRE:680-765, 880-884) of src/symmetry_resolved_ed.jl.  The
// reference scatters column by column into per-thread buffers; this kernel
// gathers row by row through Hermiticity, y_r = sum_c conj(H_cr) x_c, where
// column r of H is enumerated on the fly from the representative of row r:
//   for every occupied site i and every hop record i -> j with j empty
//     new  = m_r ^ (bit i | bit j)                (SRE:709-710, XOR hop)
//     s_JW = (-1)^popcount(m_r & between(i, j))   (SRE:646-654, fermions)
//     w    = state[rank(new)]                     (SRE:584-594, one table read)
//     H_cr = t * s_JW * conj(alpha_g(rep_c)) * conj(chi(h)) * sqrt(stab_c / stab_r)
// with h = g^-1.  Inputs are pre-scaled, xs_c = sqrt(stab_c) x_c, so a hop costs
// one table read, one vector read and one complex multiply-add:
//   y_r = (1/sqrt(stab_r)) * ( diag_r xs_r + sum_hops tchi[u][h] * sign * conj(P_h(new)) * xs_c )
// where tchi[u][h] = conj(t_u) chi(h) is tabulated per distinct amplitude u and
// P_h(new) is the per-site phase product of a flux-twisted group (1 otherwise).
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <tuple>
#include <cmath>
#include <complex>
#include <map>

#include <mutex>

#include "sed_internal.cuh"
#include "sed_rowgather.cuh"

namespace sed {

// ---------------------------------------------------------------- host checks
void build_term_tables(const GroupImpl& G, int n_bil, const int32_t* bil_ij, const double* bil_t, TermTables& tt) {
  const int N = G.n_site;
  SED_REQUIRE(n_bil >= 0 && n_bil < 65535, 5, "at most 65534 bilinear terms");
  std::vector<std::vector<std::pair<int, int>>> by_site(N);  // (to, class)
  std::map<std::pair<double, double>, int> cls;
  tt.amp.clear();
  for (int k = 0; k < n_bil; ++k) {
    const int i = bil_ij[2 * k], j = bil_ij[2 * k + 1];
    SED_REQUIRE(i >= 0 && i < N && j >= 0 && j < N, 1, "bilinear term site index out of range");
    SED_REQUIRE(i != j, 1, "a bilinear term (i, i, t) changes the particle number; write it as a density term");
    const double re = bil_t[2 * k], im = bil_t[2 * k + 1];
    if (re == 0.0 && im == 0.0) continue;
    auto key = std::make_pair(re, im);
    auto it = cls.find(key);
    int u;
    if (it == cls.end()) {
      u = (int)tt.amp.size() / 2;
      cls[key] = u;
      tt.amp.push_back(re);
      tt.amp.push_back(im);
    } else {
      u = it->second;
    }
    by_site[i].push_back({j, u});
  }
  tt.n_site = N;
  tt.n_class = (int)tt.amp.size() / 2;
  SED_REQUIRE(tt.n_class < (1 << 23), 5, "too many distinct hopping amplitudes");
  tt.site_off.assign(N + 1, 0);
  tt.rec.clear();
  for (int i = 0; i < N; ++i) {
    tt.site_off[i] = (uint16_t)tt.rec.size();
    for (auto& p : by_site[i]) tt.rec.push_back((uint32_t)p.first | ((uint32_t)p.second << 8));
  }
  tt.site_off[N] = (uint16_t)tt.rec.size();
  tt.n_terms = (int)tt.rec.size();
}

// The gather needs H = H^dagger and [H, U_g] = 0 for every g: every hop
// (i -> j, t) needs its partner (j -> i, conj t), and the group must map it to
// (perm_g(i) -> perm_g(j), t * eta_g(j) * conj(eta_g(i))).
void check_hermitian_symmetric(const GroupImpl& G, int n_bil, const int32_t* bil_ij, const double* bil_t) {
  // summed amplitude of every (i, j) in a dense N x N table (N <= 64), kept
  // zero between calls: a batch validates hundreds of requests per launch
  const int N = G.n_site;
  thread_local std::vector<double> tab(64 * 64 * 2, 0.0);
  thread_local std::vector<uint8_t> used(64 * 64, 0);
  std::vector<int> keys;
  keys.reserve(n_bil);
  struct Reset {  // restores the all-zero state on every exit, a throw included
    std::vector<int>& k;
    ~Reset() {
      for (int e : k) {
        tab[2 * e] = tab[2 * e + 1] = 0.0;
        used[e] = 0;
      }
    }
  } reset{keys};
  double scale = 0.0;
  for (int k = 0; k < n_bil; ++k) {
    const int i = bil_ij[2 * k], j = bil_ij[2 * k + 1];
    SED_REQUIRE(i >= 0 && i < N && j >= 0 && j < N, 1, "bilinear term site index out of range");
    const int e = i * N + j;
    if (!used[e]) {
      used[e] = 1;
      keys.push_back(e);
    }
    tab[2 * e] += bil_t[2 * k];
    tab[2 * e + 1] += bil_t[2 * k + 1];
    scale = std::max(scale, std::hypot(bil_t[2 * k], bil_t[2 * k + 1]));
  }
  std::sort(keys.begin(), keys.end());  // (i, j) in lexicographic order
  const double tol = 1e-9 * std::max(scale, 1e-300), tol2 = tol * tol;
  for (int e : keys) {
    const int i = e / N, j = e % N;
    const double tr = tab[2 * e], ti = tab[2 * e + 1];
    const int er = j * N + i;
    const double hr = tr - tab[2 * er], hi = ti + tab[2 * er + 1];
    SED_REQUIRE(hr * hr + hi * hi <= tol2, 6,
                "bilinear terms are not Hermitian-closed: (i, j, t) needs (j, i, conj(t))");
    for (int g = 0; g < G.n_ops; ++g) {
      const int pi = G.perm[(size_t)g * N + i], pj = G.perm[(size_t)g * N + j];
      const double eir = G.phase[((size_t)g * N + i) * 2], eii = G.phase[((size_t)g * N + i) * 2 + 1];
      const double ejr = G.phase[((size_t)g * N + j) * 2], eji = G.phase[((size_t)g * N + j) * 2 + 1];
      // t * eta_j * conj(eta_i)
      const double ar = ejr * eir + eji * eii, ai = eji * eir - ejr * eii;
      const double xr = tr * ar - ti * ai, xi = tr * ai + ti * ar;
      const int es = pi * N + pj;
      const double dr = xr - tab[2 * es], di = xi - tab[2 * es + 1];
      SED_REQUIRE(dr * dr + di * di <= tol2, 6,
                  "bilinear terms are not invariant under the symmetry group");
    }
  }
}

void compute_phase_classes(const GroupImpl& G, int k, PhaseClassTables& pc) {
  const int nG = G.n_ops, N = G.n_site;
  pc.kp1 = k + 1;
  pc.mask.assign((size_t)nG * kMaxCls, 0);
  pc.pw.assign((size_t)nG * kMaxCls * pc.kp1 * 2, 0.0);
  pc.base_k.assign((size_t)nG * 2, 0.0);
  for (int h = 0; h < nG; ++h) pc.base_k[2 * h] = 1.0;
  for (size_t i = 0; i < pc.pw.size() / 2; i += pc.kp1) pc.pw[2 * i] = 1.0;  // r^0 = 1 for every class
  if (!G.has_phases) {
    pc.mode = 0;
    return;
  }
  pc.mode = 1;
  for (int h = 0; h < nG && pc.mode == 1; ++h) {
    std::vector<std::pair<double, double>> val;
    std::vector<uint64_t> msk;
    for (int j = 0; j < N; ++j) {
      const double re = G.phase[((size_t)h * N + j) * 2], im = G.phase[((size_t)h * N + j) * 2 + 1];
      size_t c = 0;
      while (c < val.size() && !(val[c].first == re && val[c].second == im)) ++c;
      if (c == val.size()) {
        val.push_back({re, im});
        msk.push_back(0);
      }
      msk[c] |= 1ULL << j;
    }
    if (val.size() > (size_t)kMaxCls + 1) {
      pc.mode = 2;
      break;
    }
    size_t b = 0;
    for (size_t c = 1; c < val.size(); ++c)
      if (__builtin_popcountll(msk[c]) > __builtin_popcountll(msk[b])) b = c;
    const std::complex<double> base(val[b].first, val[b].second);
    std::complex<double> bk(1.0, 0.0);
    for (int e = 0; e < k; ++e) bk *= base;
    pc.base_k[2 * h] = bk.real();
    pc.base_k[2 * h + 1] = bk.imag();
    int slot = 0;
    for (size_t c = 0; c < val.size(); ++c) {
      if (c == b) continue;
      const std::complex<double> r = std::complex<double>(val[c].first, val[c].second) / base;
      pc.mask[(size_t)h * kMaxCls + slot] = msk[c];
      std::complex<double> pw(1.0, 0.0);
      for (int e = 0; e <= k; ++e) {
        const size_t idx = (((size_t)h * kMaxCls + slot) * pc.kp1 + e) * 2;
        pc.pw[idx] = pw.real();
        pc.pw[idx + 1] = pw.imag();
        pw *= r;
      }
      ++slot;
    }
  }
  if (pc.mode == 2) {  // per-site product: no folding, tables unused
    for (int h = 0; h < nG; ++h) {
      pc.base_k[2 * h] = 1.0;
      pc.base_k[2 * h + 1] = 0.0;
    }
  }
}

struct ApplyArgs {
  int64_t n_orb;
  int N, G, n_class, n_terms;
  int sms;  // SMs the grid is sized for (op_sm_count)
  const uint64_t* reps;
  const uint8_t* stab;
  const uint8_t* rowflag;
  const double2* diag;
  const uint64_t* state;
  const uint32_t* rank_tab;
  RankParams rp;
  const uint16_t* site_off;
  const uint32_t* rec;
  const void* tchi;  // [n_class][G] V  (table mode)
  const void* amp;   // [n_class] V     (on-the-fly mode)
  const void* chi;   // [G] V
  const uint8_t* inv;
  const void* eta;   // [G][N] V        (twisted groups, per-site product)
  const uint64_t* cls_mask;  // [G][3]
  const void* cls_pw;        // [G][3][k+1] V
  int phase_mode, kp1;
};

// Shared-memory image of the tables, 16-byte aligned pieces first.
template <class V>
struct SmemLayout {
  size_t tchi, chi, isr, pw, mask, rank, rec, site_off, inv, total;
  static SmemLayout make(const ApplyArgs& a, bool table) {
    SmemLayout L;
    size_t o = 0;
    auto al = [&](size_t x) { return (x + 15) & ~(size_t)15; };
    L.tchi = o;
    o = al(o + (table ? (size_t)a.n_class * a.G : (size_t)a.n_class) * sizeof(V));
    L.chi = o;
    o = al(o + (size_t)a.G * sizeof(V));
    L.isr = o;
    o = al(o + 65 * sizeof(double));
    L.pw = o;
    o = al(o + (a.phase_mode == 1 ? (size_t)a.G * kMaxCls * a.kp1 * sizeof(V) : 0));
    L.mask = o;
    o = al(o + (a.phase_mode == 1 ? (size_t)a.G * kMaxCls * 8 : 0));
    L.rank = o;
    o = al(o + (size_t)a.rp.total * 4);
    L.rec = o;
    o = al(o + (size_t)a.n_terms * 4);
    L.site_off = o;
    o = al(o + (size_t)(a.N + 1) * 2);
    L.inv = o;
    o = al(o + 64);
    L.total = o;
    return L;
  }
};

// 512-thread blocks: the shared tables (~50 KB for 48 sites) allow three
// resident blocks per SM, i.e. 1536 threads keeping random loads in flight.
static constexpr int kApplyBS = 512;

// TPR threads per row (1, 2, 4 or 8 lanes of one warp); the block size, and
// so the rows per block, is the launch's.  Both are picked per operator by the
// autotuner in launch_apply.
template <class P, bool FERMI, bool PHASES, bool TABLE, int TPR>
__global__ void __launch_bounds__(kApplyBS) k_apply(ApplyArgs a, SmemLayout<typename P::V> L,
                                               const typename P::V* __restrict__ xs, double2* __restrict__ y) {
  using V = typename P::V;
  using S = typename P::S;
  extern __shared__ __align__(16) unsigned char smem[];
  V* s_tchi = reinterpret_cast<V*>(smem + L.tchi);
  V* s_chi = reinterpret_cast<V*>(smem + L.chi);
  double* s_isr = reinterpret_cast<double*>(smem + L.isr);
  uint32_t* s_rank = reinterpret_cast<uint32_t*>(smem + L.rank);
  uint32_t* s_rec = reinterpret_cast<uint32_t*>(smem + L.rec);
  uint16_t* s_off = reinterpret_cast<uint16_t*>(smem + L.site_off);
  uint8_t* s_inv = reinterpret_cast<uint8_t*>(smem + L.inv);
  V* s_pw = reinterpret_cast<V*>(smem + L.pw);
  uint64_t* s_mask = reinterpret_cast<uint64_t*>(smem + L.mask);
  {
    if (PHASES && a.phase_mode == 1) {
      const V* pw = reinterpret_cast<const V*>(a.cls_pw);
      for (int i = threadIdx.x; i < a.G * kMaxCls * a.kp1; i += blockDim.x) s_pw[i] = pw[i];
      for (int i = threadIdx.x; i < a.G * kMaxCls; i += blockDim.x) s_mask[i] = a.cls_mask[i];
    }
    const int nt = TABLE ? a.n_class * a.G : a.n_class;
    const V* src = reinterpret_cast<const V*>(TABLE ? a.tchi : a.amp);
    for (int i = threadIdx.x; i < nt; i += blockDim.x) s_tchi[i] = src[i];
    const V* chi = reinterpret_cast<const V*>(a.chi);
    for (int i = threadIdx.x; i < a.G; i += blockDim.x) s_chi[i] = chi[i];
    for (int i = threadIdx.x; i < 65; i += blockDim.x) s_isr[i] = i ? 1.0 / sqrt((double)i) : 0.0;
    for (int i = threadIdx.x; i < a.rp.total; i += blockDim.x) s_rank[i] = a.rank_tab[i];
    for (int i = threadIdx.x; i < a.n_terms; i += blockDim.x) s_rec[i] = a.rec[i];
    for (int i = threadIdx.x; i <= a.N; i += blockDim.x) s_off[i] = a.site_off[i];
    for (int i = threadIdx.x; i < a.G; i += blockDim.x) s_inv[i] = a.inv[i];
  }
  __syncthreads();
  const V* __restrict__ eta = reinterpret_cast<const V*>(a.eta);
  const PhaseClasses<V> pcl{a.phase_mode, a.kp1, s_mask, s_pw};
  if (TPR == 1) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < a.n_orb;
         o += (int64_t)gridDim.x * blockDim.x) {
      if (!a.rowflag[o]) {
        y[o] = make_double2(0.0, 0.0);
        continue;
      }
      const double2 dg = a.diag[o];
      const V xo = xs[o];
      S ar = (S)dg.x * xo.x - (S)dg.y * xo.y;
      S ai = (S)dg.x * xo.y + (S)dg.y * xo.x;
      row_gather<P, FERMI, PHASES, TABLE>(a.reps[o], xs, s_tchi, s_chi, a.G, eta, a.N, s_rank, a.rp, s_rec, s_off,
                                          s_inv, a.state, ar, ai, pcl);
      const double is = s_isr[a.stab[o]];
      y[o] = make_double2((double)ar * is, (double)ai * is);
    }
    return;
  }
  // TPR consecutive lanes share a row; their partial sums meet by shuffles
  // within the group, and lane 0 of the group adds the diagonal and stores
  const int q = threadIdx.x % TPR;
  const unsigned gmask = ((1u << TPR) - 1u) << ((threadIdx.x & 31) & ~(TPR - 1));
  const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / TPR;
  for (int64_t o = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TPR; o < a.n_orb; o += ngrp) {
    const bool on = a.rowflag[o] != 0;
    S ar = 0, ai = 0;
    if (on) {
      if (q == 0) {
        const double2 dg = a.diag[o];
        const V xo = xs[o];
        ar = (S)dg.x * xo.x - (S)dg.y * xo.y;
        ai = (S)dg.x * xo.y + (S)dg.y * xo.x;
      }
      row_gather_split<P, FERMI, PHASES, TABLE>(a.reps[o], q, TPR, xs, s_tchi, s_chi, a.G, eta, a.N, s_rank, a.rp,
                                                s_rec, s_off, a.state, ar, ai, pcl);
    }
    __syncwarp(gmask);
#pragma unroll
    for (int off = TPR / 2; off > 0; off >>= 1) {
      ar += __shfl_xor_sync(gmask, ar, off);
      ai += __shfl_xor_sync(gmask, ai, off);
    }
    if (q == 0) {
      if (on) {
        const double is = s_isr[a.stab[o]];
        y[o] = make_double2((double)ar * is, (double)ai * is);
      } else {
        y[o] = make_double2(0.0, 0.0);
      }
    }
  }
}

// ----------------------------------------------------------------- helpers
__global__ void k_diag(int64_t n_orb, const uint64_t* __restrict__ reps, const uint8_t* __restrict__ rowflag,
                       int n_den, const int32_t* __restrict__ den_ij, const double2* __restrict__ den_v,
                       double2* __restrict__ diag) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t m = reps[o];
    double re = 0.0, im = 0.0;  // SRE:697-703: summed in term order from zero
    for (int t = 0; t < n_den; ++t)
      if (((m >> den_ij[2 * t]) & 1ULL) && ((m >> den_ij[2 * t + 1]) & 1ULL)) {
        re = __dadd_rn(re, den_v[t].x);
        im = __dadd_rn(im, den_v[t].y);
      }
    diag[o] = (!rowflag || rowflag[o]) ? make_double2(re, im) : make_double2(0.0, 0.0);
  }
}

__global__ void k_count_hops(int64_t n_orb, const uint64_t* __restrict__ reps, const uint8_t* __restrict__ rowflag,
                             int N, const uint16_t* __restrict__ site_off, const uint32_t* __restrict__ rec,
                             unsigned long long* __restrict__ total) {
  unsigned long long cnt = 0;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x) {
    if (!rowflag[o]) continue;
    const uint64_t m = reps[o];
    uint64_t occ = m;
    while (occ) {
      const int i = __ffsll((long long)occ) - 1;
      occ &= occ - 1;
      for (int t = site_off[i]; t < site_off[i + 1]; ++t) cnt += !((m >> (rec[t] & 0xFF)) & 1ULL);
    }
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(total, cnt);
}

template <class V>
__global__ void k_scale_xs(int64_t n_orb, const double2* __restrict__ v, const uint8_t* __restrict__ stab,
                           V* __restrict__ xs) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x) {
    const double s = sqrt((double)stab[o]);
    const double2 x = v[o];
    xs[o].x = x.x * s;
    xs[o].y = x.y * s;
  }
}

__global__ void k_expand_vec(int64_t dim, const uint32_t* __restrict__ row_orbit, const double2* __restrict__ xsec,
                             double2* __restrict__ xpad) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
    xpad[row_orbit[r]] = xsec[r];
}

__global__ void k_compress_vec(int64_t dim, const uint32_t* __restrict__ row_orbit, const double2* __restrict__ ypad,
                               double2* __restrict__ ysec) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
    ysec[r] = ypad[row_orbit[r]];
}

int grid1(int64_t work, int block) {
  const int64_t sms = device_sm_count();
  const int64_t g = (work + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, sms * 32));
}

void compute_diag(int64_t n_orb, const uint64_t* reps, const uint8_t* rowflag, int n_den, const int32_t* den_ij,
                  const double2* den_v, double2* diag, cudaStream_t s) {
  if (!n_orb) return;
  k_diag<<<grid1(n_orb, 256), 256, 0, s>>>(n_orb, reps, rowflag, n_den, den_ij, den_v, diag);
  SED_CUDA(cudaGetLastError());
}

OpImpl::~OpImpl() {
  if (own_stream && stream) cudaStreamDestroy(stream);
}

// -------------------------------------------------------------- op creation
std::shared_ptr<OpImpl> make_op(std::shared_ptr<SectorImpl> sp, int n_bil, const int32_t* bil_ij, const double* bil_t,
                                int n_den, const int32_t* den_ij, const double* den_v, int precision) {
  SED_REQUIRE(precision == 0 || precision == 1, 1, "precision must be SED_PREC_FP64 or SED_PREC_MIXED");
  SED_REQUIRE(n_bil == 0 || (bil_ij && bil_t), 1, "bilinear arrays must not be NULL");
  SED_REQUIRE(n_den == 0 || (den_ij && den_v), 1, "density arrays must not be NULL");
  const SectorImpl& S = *sp;
  const CatalogImpl& C = *S.cat;
  const GroupImpl& G = *S.group;
  check_hermitian_symmetric(G, n_bil, bil_ij, bil_t);
  check_species_terms(C, n_bil, bil_ij);
  for (int k = 0; k < n_den; ++k)
    SED_REQUIRE(den_ij[2 * k] >= 0 && den_ij[2 * k] < G.n_site && den_ij[2 * k + 1] >= 0 &&
                    den_ij[2 * k + 1] < G.n_site,
                1, "density term site index out of range");
  auto op = std::make_shared<OpImpl>();
  op->sec = sp;
  op->precision = precision;
  SED_CUDA(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  op->own_stream = true;
  cudaStream_t s = op->stream;
  build_term_tables(G, n_bil, bil_ij, bil_t, op->terms);
  const TermTables& tt = op->terms;
  upload(op->site_off, tt.site_off, s);
  upload(op->rec, tt.rec, s);
  // phase classes of the (twisted) group; base^k folds into tchi
  compute_phase_classes(G, C.n_filled, op->pc);
  upload(op->cls_mask, op->pc.mask, s);
  // tchi[u][h] = conj(t_u) * chi(h) * conj(base_h^k), and the plain amplitude / chi tables
  const int nG = G.n_ops;
  std::vector<double> tchi((size_t)tt.n_class * nG * 2);
  for (int u = 0; u < tt.n_class; ++u)
    for (int h = 0; h < nG; ++h) {
      const double tr = tt.amp[2 * u], ti = -tt.amp[2 * u + 1];
      const double br = op->pc.base_k[2 * h], bi = -op->pc.base_k[2 * h + 1];
      const double cr0 = S.chi[2 * h], ci0 = S.chi[2 * h + 1];
      const double cr = cr0 * br - ci0 * bi, ci = cr0 * bi + ci0 * br;  // chi(h) * conj(base^k)
      tchi[((size_t)u * nG + h) * 2] = tr * cr - ti * ci;
      tchi[((size_t)u * nG + h) * 2 + 1] = tr * ci + ti * cr;
    }
  std::vector<double> ampc(tt.amp);
  for (size_t u = 1; u < ampc.size(); u += 2) ampc[u] = -ampc[u];  // conj(t)
  auto to32 = [](const std::vector<double>& v) {
    std::vector<float> f(v.size());
    for (size_t i = 0; i < v.size(); ++i) f[i] = (float)v[i];
    return f;
  };
  // one buffer per precision holding [tchi | conj(amp) | chi | eta]
  std::vector<double> eta(G.phase);
  std::vector<double> pack;
  pack.insert(pack.end(), tchi.begin(), tchi.end());
  pack.insert(pack.end(), ampc.begin(), ampc.end());
  std::vector<double> chib(S.chi);  // chi * conj(base^k) for the on-the-fly coefficient
  for (int h = 0; h < nG; ++h) {
    const double br = op->pc.base_k[2 * h], bi = -op->pc.base_k[2 * h + 1];
    const double cr0 = S.chi[2 * h], ci0 = S.chi[2 * h + 1];
    chib[2 * h] = cr0 * br - ci0 * bi;
    chib[2 * h + 1] = cr0 * bi + ci0 * br;
  }
  pack.insert(pack.end(), chib.begin(), chib.end());
  pack.insert(pack.end(), eta.begin(), eta.end());
  pack.insert(pack.end(), op->pc.pw.begin(), op->pc.pw.end());
  upload(op->tchi64, pack, s);
  upload(op->tchi32, to32(pack), s);
  // density-density diagonal (SRE:697-703)
  op->den_ij.assign(den_ij, den_ij + 2 * n_den);
  op->den_v.assign(den_v, den_v + 2 * n_den);
  DevBuf dij, dv;
  upload(dij, op->den_ij, s);
  upload(dv, op->den_v, s);
  op->diag.alloc((size_t)std::max<int64_t>(C.n_orbits, 1) * 16);
  if (C.n_orbits) {
    k_diag<<<grid1(C.n_orbits, 256), 256, 0, s>>>(C.n_orbits, C.reps.as<uint64_t>(), S.rowflag.as<uint8_t>(), n_den,
                                             dij.as<int32_t>(), dv.as<double2>(), op->diag.as<double2>());
    SED_CUDA(cudaGetLastError());
  }
  SED_CUDA(cudaStreamSynchronize(s));
  op->tchi_in_smem = (size_t)tt.n_class * nG * 16 <= 48 * 1024;
  return op;
}

static ApplyArgs make_args(const OpImpl& op, bool fp32) {
  const SectorImpl& S = *op.sec;
  const CatalogImpl& C = *S.cat;
  const GroupImpl& G = *S.group;
  const TermTables& tt = op.terms;
  ApplyArgs a{};
  a.n_orb = C.n_orbits;
  a.sms = op_sm_count(op);
  a.N = G.n_site;
  a.G = G.n_ops;
  a.n_class = tt.n_class;
  a.n_terms = tt.n_terms;
  a.reps = C.reps.as<uint64_t>();
  a.stab = C.stab.as<uint8_t>();
  a.rowflag = S.rowflag.as<uint8_t>();
  a.diag = op.diag.as<double2>();
  a.state = C.state.as<uint64_t>();
  a.rank_tab = C.rank.dev.as<uint32_t>();
  a.rp = C.rank.rp;
  a.site_off = op.site_off.as<uint16_t>();
  a.rec = op.rec.as<uint32_t>();
  const size_t el = fp32 ? 8 : 16;
  const unsigned char* base = (const unsigned char*)(fp32 ? op.tchi32.p : op.tchi64.p);
  a.tchi = base;
  a.amp = base + (size_t)tt.n_class * G.n_ops * el;
  a.chi = base + ((size_t)tt.n_class * G.n_ops + tt.n_class) * el;
  a.eta = base + ((size_t)tt.n_class * G.n_ops + tt.n_class + G.n_ops) * el;
  a.cls_pw = base + ((size_t)tt.n_class * G.n_ops + tt.n_class + G.n_ops + (size_t)G.n_ops * G.n_site) * el;
  a.cls_mask = op.cls_mask.as<uint64_t>();
  a.phase_mode = op.pc.mode;
  a.kp1 = op.pc.kp1;
  a.inv = C.inv_u8.as<uint8_t>();
  return a;
}

// ------------------------------------------------------------ launch shape
// The gather's launch shape -- threads per row and threads (so rows) per
// block -- is chosen per operator by measurement (apply_shape below).
struct ApplyShape {
  int tpr, block;
};
static constexpr ApplyShape kApplyShapes[] = {{1, 512}, {1, 256}, {2, 512}, {2, 256},
                                              {4, 512}, {4, 256}, {8, 512}, {8, 256}};

template <class P, bool F, bool PH, bool T, int TPR>
static void launch_apply_tpr(const ApplyArgs& a, const void* xs, double* y, cudaStream_t s, int block) {
  using V = typename P::V;
  const SmemLayout<V> L = SmemLayout<V>::make(a, T);
  auto kern = k_apply<P, F, PH, T, TPR>;
  SED_REQUIRE(L.total <= 200 * 1024, 5, "operator tables exceed the shared-memory budget");
  // the shared-memory opt-in is a property of the kernel on each device,
  // shared by every operator: raise it (never lower it) and launch under one
  // lock, so a concurrent caller with a smaller footprint cannot undercut this
  // launch
  static std::mutex mu;
  static SmemOptIn optin;
  std::lock_guard<std::mutex> lock(mu);
  optin.ensure(kern, L.total);
  int blocks_per_sm = 0;
  SED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, block, L.total));
  blocks_per_sm = std::max(blocks_per_sm, 1);
  const int64_t rows_per_block = block / TPR;
  const int64_t want = (a.n_orb + rows_per_block - 1) / rows_per_block;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)a.sms * blocks_per_sm));
  kern<<<grid, block, L.total, s>>>(a, L, reinterpret_cast<const V*>(xs), reinterpret_cast<double2*>(y));
  SED_CUDA(cudaGetLastError());
}

template <class P, bool F, bool PH, bool T>
static void launch_apply(const ApplyArgs& a, const void* xs, double* y, cudaStream_t s, ApplyShape sh) {
  switch (sh.tpr) {
    case 1: launch_apply_tpr<P, F, PH, T, 1>(a, xs, y, s, sh.block); break;
    case 2: launch_apply_tpr<P, F, PH, T, 2>(a, xs, y, s, sh.block); break;
    case 4: launch_apply_tpr<P, F, PH, T, 4>(a, xs, y, s, sh.block); break;
    case 8: launch_apply_tpr<P, F, PH, T, 8>(a, xs, y, s, sh.block); break;
    default: SED_REQUIRE(false, 1, "threads per row must be 1, 2, 4 or 8");
  }
}

template <class P>
static void dispatch_apply(const ApplyArgs& a, bool fermi, bool phases, bool table, const void* xs, double* y,
                           cudaStream_t s, ApplyShape sh) {
  if (fermi) {
    if (phases) {
      if (table) launch_apply<P, true, true, true>(a, xs, y, s, sh);
      else launch_apply<P, true, true, false>(a, xs, y, s, sh);
    } else {
      if (table) launch_apply<P, true, false, true>(a, xs, y, s, sh);
      else launch_apply<P, true, false, false>(a, xs, y, s, sh);
    }
  } else {
    if (phases) {
      if (table) launch_apply<P, false, true, true>(a, xs, y, s, sh);
      else launch_apply<P, false, true, false>(a, xs, y, s, sh);
    } else {
      if (table) launch_apply<P, false, false, true>(a, xs, y, s, sh);
      else launch_apply<P, false, false, false>(a, xs, y, s, sh);
    }
  }
}

// The autotuner: the first gather matvec of an operator (per precision)
// times every shape of kApplyShapes on the operator's own input, one warm-up
// and two timed launches each (CUDA events on the operator's stream; the trial
// launches write the caller's output, which the chosen launch then
// overwrites), and keeps the fastest.  The choice is remembered per catalog
// shape (orbits, sites, filling, group order, hop records, precision,
// statistics, twist phases, coefficient placement) for the whole process,
// so later operators of the same family do not retune.  SED_APPLY_SHAPE=
// "tpr,block" in the environment, or sed_op_set_apply_shape, pins a shape.
// Results depend on the shape only through the order in which a row's hops
// are summed (the row split over tpr lanes).
struct ShapeKey {
  int64_t n_orb;
  int n_site, n_filled, n_ops, n_terms, fp32, fermi, phases, table;
  bool operator<(const ShapeKey& o) const {
    return std::tie(n_orb, n_site, n_filled, n_ops, n_terms, fp32, fermi, phases, table) <
           std::tie(o.n_orb, o.n_site, o.n_filled, o.n_ops, o.n_terms, o.fp32, o.fermi, o.phases, o.table);
  }
};
static std::mutex g_shape_mu;
static std::map<ShapeKey, ApplyShape> g_shapes;

static bool env_shape(ApplyShape* out) {
  const char* e = std::getenv("SED_APPLY_SHAPE");
  if (!e) return false;
  int t = 0, b = 0;
  if (std::sscanf(e, "%d,%d", &t, &b) != 2) return false;
  for (const ApplyShape& sh : kApplyShapes)
    if (sh.tpr == t && sh.block == b) {
      *out = sh;
      return true;
    }
  return false;
}

// allow_tune = false (the allocation-free matvec): no timing runs and no host
// synchronisation; the shape is the operator's, the pinned one, the one
// remembered for this catalog shape, or the default (1, 512), and nothing is
// stored on the operator, so a later allocating matvec still tunes.
template <class P>
static ApplyShape apply_shape(OpImpl& op, const ApplyArgs& a, bool fp32, const void* xs, double* ypad,
                              cudaStream_t s, bool allow_tune) {
  const int k = fp32 ? 1 : 0;
  if (op.apply_tpr[k] > 0) return ApplyShape{op.apply_tpr[k], op.apply_block[k]};
  ApplyShape best{1, 512};
  const GroupImpl& G = *op.sec->group;
  const bool fermi = G.stats == 1, phases = G.has_phases, table = op.tchi_in_smem;
  const ShapeKey key{a.n_orb, a.N, op.sec->cat->n_filled, a.G, a.n_terms, k, fermi, phases, table};
  bool found = env_shape(&best);
  if (!found) {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    auto it = g_shapes.find(key);
    if (it != g_shapes.end()) {
      best = it->second;
      found = true;
    }
  }
  if (!found && !allow_tune) return best;
  if (!found) {
    cudaEvent_t e0, e1;
    SED_CUDA(cudaEventCreate(&e0));
    SED_CUDA(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    for (const ApplyShape& sh : kApplyShapes) {
      dispatch_apply<P>(a, fermi, phases, table, xs, ypad, s, sh);
      SED_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < 2; ++r) dispatch_apply<P>(a, fermi, phases, table, xs, ypad, s, sh);
      SED_CUDA(cudaEventRecord(e1, s));
      SED_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      SED_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best_ms) {
        best_ms = ms;
        best = sh;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(g_shape_mu);
    g_shapes[key] = best;
  }
  op.apply_tpr[k] = best.tpr;
  op.apply_block[k] = best.block;
  return best;
}

void op_set_apply_shape(OpImpl& op, int tpr, int block) {
  if (tpr == 0 && block == 0) {  // choose again
    op.apply_tpr[0] = op.apply_tpr[1] = 0;
    return;
  }
  bool ok = false;
  for (const ApplyShape& sh : kApplyShapes) ok = ok || (sh.tpr == tpr && sh.block == block);
  SED_REQUIRE(ok, 1, "apply shape must be (1|2|4|8 threads per row, 256|512 threads per block)");
  op.apply_tpr[0] = op.apply_tpr[1] = tpr;
  op.apply_block[0] = op.apply_block[1] = block;
}

static void apply_impl(OpImpl& op, bool fp32, const void* xs, double* ypad, cudaStream_t s,
                       bool allow_tune = true) {
  const GroupImpl& G = *op.sec->group;
  if (op.sec->cat->n_orbits == 0) return;
  if (op.tab_built) {  // the stored form of the same matvec (sed_optable.cu)
    apply_table(op, fp32, xs, ypad, s);
    return;
  }
  const ApplyArgs a = make_args(op, fp32);
  if (fp32)
    dispatch_apply<P32>(a, G.stats == 1, G.has_phases, op.tchi_in_smem, xs, ypad, s,
                        apply_shape<P32>(op, a, true, xs, ypad, s, allow_tune));
  else
    dispatch_apply<P64>(a, G.stats == 1, G.has_phases, op.tchi_in_smem, xs, ypad, s,
                        apply_shape<P64>(op, a, false, xs, ypad, s, allow_tune));
}

void op_apply_orbit(OpImpl& op, const void* xs, double* ypad, cudaStream_t s) {
  apply_impl(op, op.precision == 1, xs, ypad, s);
}

void op_apply_orbit_untuned(OpImpl& op, const void* xs, double* ypad, cudaStream_t s) {
  apply_impl(op, op.precision == 1, xs, ypad, s, false);
}

bool op_apply_orbit_cf(OpImpl& op, const void* xs, float2* y, cudaStream_t s) {
  if (!(op.tab_built && op.precision == 1 && op.sec->cat->n_orbits > 0)) return false;
  apply_table(op, true, xs, reinterpret_cast<double*>(y), s, true);
  return true;
}

// FP64 matvec regardless of the op precision (the polish step of mixed solves)
void op_apply_orbit64(OpImpl& op, const void* xs64, double* ypad, cudaStream_t s) {
  apply_impl(op, false, xs64, ypad, s);
}

void op_scale_to_xs_prec(OpImpl& op, const double* v, void* xs, bool fp32, cudaStream_t s) {
  const CatalogImpl& C = *op.sec->cat;
  if (!C.n_orbits) return;
  if (fp32)
    k_scale_xs<float2><<<grid1(C.n_orbits, 256), 256, 0, s>>>(C.n_orbits, (const double2*)v, C.stab.as<uint8_t>(),
                                                          (float2*)xs);
  else
    k_scale_xs<double2><<<grid1(C.n_orbits, 256), 256, 0, s>>>(C.n_orbits, (const double2*)v, C.stab.as<uint8_t>(),
                                                           (double2*)xs);
  SED_CUDA(cudaGetLastError());
}

void op_scale_to_xs(OpImpl& op, const double* v, void* xs, cudaStream_t s) {
  op_scale_to_xs_prec(op, v, xs, op.precision == 1, s);
}

void expand_vec(const SectorImpl& S, const double* xsec, double* xpad, cudaStream_t s) {
  const int64_t n = S.cat->n_orbits;
  SED_CUDA(cudaMemsetAsync(xpad, 0, (size_t)n * 16, s));
  if (S.dim) {
    k_expand_vec<<<grid1(S.dim, 256), 256, 0, s>>>(S.dim, S.row_orbit.as<uint32_t>(), (const double2*)xsec,
                                              (double2*)xpad);
    SED_CUDA(cudaGetLastError());
  }
}

void compress_vec(const SectorImpl& S, const double* ypad, double* ysec, cudaStream_t s) {
  if (S.dim) {
    k_compress_vec<<<grid1(S.dim, 256), 256, 0, s>>>(S.dim, S.row_orbit.as<uint32_t>(), (const double2*)ypad,
                                                (double2*)ysec);
    SED_CUDA(cudaGetLastError());
  }
}

void op_apply_host(OpImpl& op, const double* x, double* y, int64_t n, bool device_ptrs) {
  const SectorImpl& S = *op.sec;
  SED_REQUIRE(n == S.dim, 1, "vector length must equal the sector dimension");
  SED_REQUIRE(x != nullptr && y != nullptr, 1, "x and y must not be NULL");
  const int64_t n_orb = S.cat->n_orbits;
  cudaStream_t s = op.stream;
  if (!op.xs.p) {
    op.xs.alloc((size_t)std::max<int64_t>(n_orb, 1) * 16);
    op.ypad.alloc((size_t)std::max<int64_t>(n_orb, 1) * 16);
  }
  const double* xsec = x;
  double* ysec = y;
  if (!device_ptrs) {
    if (!op.xsec.p) {
      op.xsec.alloc((size_t)std::max<int64_t>(n, 1) * 16);
      op.ysec.alloc((size_t)std::max<int64_t>(n, 1) * 16);
    }
    if (n) SED_CUDA(cudaMemcpyAsync(op.xsec.p, x, (size_t)n * 16, cudaMemcpyHostToDevice, s));
    xsec = op.xsec.as<double>();
    ysec = op.ysec.as<double>();
  }
  // ypad doubles as the expanded (unscaled) input before the matvec overwrites it
  expand_vec(S, xsec, op.ypad.as<double>(), s);
  op_scale_to_xs(op, op.ypad.as<double>(), op.xs.p, s);
  op_apply_orbit(op, op.xs.p, op.ypad.as<double>(), s);
  compress_vec(S, op.ypad.as<double>(), ysec, s);
  if (!device_ptrs) {
    if (n) SED_CUDA(cudaMemcpyAsync(y, op.ysec.p, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
    SED_CUDA(cudaStreamSynchronize(s));
  }
}

int64_t op_count_hops(OpImpl& op) {
  if (op.hops >= 0) return op.hops;
  const SectorImpl& S = *op.sec;
  const CatalogImpl& C = *S.cat;
  DevBuf tot(8);
  SED_CUDA(cudaMemsetAsync(tot.p, 0, 8, op.stream));
  if (C.n_orbits)
    k_count_hops<<<grid1(C.n_orbits, 256), 256, 0, op.stream>>>(C.n_orbits, C.reps.as<uint64_t>(), S.rowflag.as<uint8_t>(),
                                                           C.group->n_site, op.site_off.as<uint16_t>(),
                                                           op.rec.as<uint32_t>(), tot.as<unsigned long long>());
  SED_CUDA(cudaGetLastError());
  unsigned long long h = 0;
  SED_CUDA(cudaMemcpyAsync(&h, tot.p, 8, cudaMemcpyDeviceToHost, op.stream));
  SED_CUDA(cudaStreamSynchronize(op.stream));
  op.hops = (int64_t)h;
  return op.hops;
}

}  // namespace sed
