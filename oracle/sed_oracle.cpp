// sed_oracle.cpp -- CPU restatement of the reference's symmetry-resolved ED hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker and the timed CPU
// baseline ("port" of the reference algorithm).  Only tests/, the smoke check
// and bench.py's CPU-baseline / reference arm may load it.  The product path
// (realspace_exactdiagonalization_gb300/) never links or calls it.
//
// Every function restates one reference function of the Julia package
// RealSpace_ExactDiagonalization v0.1.0; the citation is the reference file and
// line range (SRE = src/symmetry_resolved_ed.jl).  Arithmetic follows the
// reference's evaluation order with plain (non-fused) IEEE multiplies and adds,
// built with -ffp-contract=off, so that amplitude tables are reproducible bit for
// bit.  Indices are 0-based at this C boundary; readback fields that the
// reference stores 1-based (rep_rank, rep_sym, stabilizer g) are returned
// 1-based, exactly as the reference holds them.
//
// Parity pins (golden vectors this restatement is checked against, see
// tests/golden/): colex rank table N=4,k=2 (doc/design.ipynb cell 22), LinTable
// == rank over C(12,3) (cell 24), Haldane 2x3 orbit/sector/nnz counts (cells
// 26, 43), and the stored orbit counts, sector dimensions and ground energies of
// benchmark/benchmark_data/benchmark_raw.csv.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct cd {
  double re, im;
};
inline cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
inline cd csub(cd a, cd b) { return {a.re - b.re, a.im - b.im}; }
inline cd cconj(cd a) { return {a.re, -a.im}; }
inline cd cscale(cd a, double s) { return {a.re * s, a.im * s}; }
inline bool cis_zero(cd a) { return a.re == 0.0 && a.im == 0.0; }

// Julia isapprox(x, y; atol) for ComplexF64 with atol > 0 (rtol defaults to 0):
// x == y || abs(x - y) <= atol, abs being hypot.
inline bool capprox(cd x, cd y, double atol) {
  if (x.re == y.re && x.im == y.im) return true;
  return std::hypot(x.re - y.re, x.im - y.im) <= atol;
}

inline int ctz64(uint64_t x) { return __builtin_ctzll(x); }
inline int popc64(uint64_t x) { return __builtin_popcountll(x); }

// ---------------------------------------------------------------- binomials
// SRE:214-222 (_binom_cached over Julia's binomial): exact Pascal table.
int64_t g_binom[65][65];
bool g_binom_ready = false;
void init_binom() {
  if (g_binom_ready) return;
  for (int n = 0; n <= 64; ++n)
    for (int k = 0; k <= 64; ++k) g_binom[n][k] = 0;
  for (int n = 0; n <= 64; ++n) {
    g_binom[n][0] = 1;
    for (int k = 1; k <= n; ++k) g_binom[n][k] = g_binom[n - 1][k - 1] + (k <= n - 1 ? g_binom[n - 1][k] : 0);
  }
  g_binom_ready = true;
}
inline int64_t binom(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  return g_binom[n][k];
}

// SRE:231-243 rank_combination: colex rank sum_j binom(b_j, j+1).
inline int64_t rank_combination(uint64_t m) {
  int64_t idx = 0;
  int j = 1;
  uint64_t tmp = m;
  while (tmp) {
    uint64_t lsb = tmp & (~tmp + 1);
    idx += binom(ctz64(lsb), j);
    ++j;
    tmp ^= lsb;
  }
  return idx;
}

// SRE:193-197 Gosper's hack; SRE:199-202 first mask.
inline uint64_t gosper_next(uint64_t x) {
  uint64_t c = x & (~x + 1);
  uint64_t r = x + c;
  return (((r ^ x) >> 2) / c) | r;
}
inline uint64_t first_combination_mask(int k) { return k == 0 ? 0ULL : ((1ULL << k) - 1ULL); }

// ---------------------------------------------------------------- group
struct Group {
  int n_site = 0, n_ops = 0, identity = 0, stats = 0;  // stats: 0 bosonic, 1 fermionic
  std::vector<int32_t> perm;                            // n_ops * n_site, 0-based targets
  std::vector<cd> phase;                                // n_ops * n_site
  std::vector<int32_t> inv;                             // 0-based inverse op index
};

// Bits of m at positions strictly above q (the reference's count_ones(new >> p)
// with p = q + 1, which is 0 when p == 64).
inline uint64_t bits_above(uint64_t m, int q) { return m & ~((2ULL << q) - 1ULL); }

// SRE:132-144 (bosonic) and SRE:146-163 (fermionic) apply_operation_to_mask.
inline void apply_op(const Group& G, int g, uint64_t m, uint64_t* out, cd* amp) {
  const int32_t* perm = &G.perm[(size_t)g * G.n_site];
  const cd* ph = &G.phase[(size_t)g * G.n_site];
  uint64_t tmp = m, nm = 0;
  cd phase{1.0, 0.0};
  int parity = 1;
  while (tmp) {
    uint64_t lsb = tmp & (~tmp + 1);
    int idx = ctz64(lsb);
    int p = perm[idx];
    if (G.stats == 1 && (popc64(bits_above(nm, p)) & 1)) parity = -parity;
    nm |= 1ULL << p;
    phase = cmul(phase, ph[idx]);
    tmp ^= lsb;
  }
  *out = nm;
  if (G.stats == 1)
    *amp = cscale(phase, (double)parity);
  else
    *amp = phase;
}

// SRE:174-187 get_canonical_representative: first strict minimum over G.
inline void canonical_representative(const Group& G, uint64_t m, uint64_t* repr, int* best_g, cd* best_amp) {
  uint64_t r = m;
  int bg = G.identity;
  cd ba{1.0, 0.0};
  for (int g = 0; g < G.n_ops; ++g) {
    uint64_t s;
    cd a;
    apply_op(G, g, m, &s, &a);
    if (s < r) {
      r = s;
      bg = g;
      ba = a;
    }
  }
  *repr = r;
  *best_g = bg;
  *best_amp = ba;
}

// SRE:109-117 _inverse_operation_indices (first matching h).
bool inverse_ops(Group& G, std::string* err) {
  const int N = G.n_site;
  G.inv.assign(G.n_ops, -1);
  for (int g = 0; g < G.n_ops; ++g) {
    const int32_t* pg = &G.perm[(size_t)g * N];
    const cd* eg = &G.phase[(size_t)g * N];
    for (int h = 0; h < G.n_ops; ++h) {
      const int32_t* ph = &G.perm[(size_t)h * N];
      const cd* eh = &G.phase[(size_t)h * N];
      bool ok = true;
      for (int i = 0; i < N && ok; ++i) ok = (ph[pg[i]] == i);
      for (int i = 0; i < N && ok; ++i) ok = capprox(cmul(eg[i], eh[pg[i]]), cd{1.0, 0.0}, 1e-12);
      if (ok) {
        G.inv[g] = h;
        break;
      }
    }
    if (G.inv[g] < 0) {
      *err = "Symmetry operations are not closed under inversion.";
      return false;
    }
  }
  return true;
}

// ---------------------------------------------------------------- catalog
struct Catalog {
  Group G;
  int n_filled = 0;
  int64_t n_states = 0;
  std::vector<uint64_t> reps;
  std::vector<int32_t> stab_order;
  std::vector<int64_t> stab_ptr;  // CSR over orbits
  std::vector<int32_t> stab_g;    // 1-based, like the reference
  std::vector<cd> stab_phase;
  std::vector<int32_t> rep_rank;  // 1-based orbit index, 0 = unset
  std::vector<int32_t> rep_sym;   // 1-based group element
  std::vector<cd> rep_amp;
};

// SRE:371-487 build_symmetry_orbit_catalog (serial Gosper loop, early-exit
// isrepresentative, one orbit-expansion pass per representative with the
// last write winning, and the n_filled in {0, n_site} special case).
void build_catalog(Catalog& C) {
  const Group& G = C.G;
  const int N = G.n_site, k = C.n_filled, nG = G.n_ops;
  C.n_states = binom(N, k);
  C.rep_rank.assign(C.n_states, 0);
  C.rep_sym.assign(C.n_states, 0);
  C.rep_amp.assign(C.n_states, cd{0.0, 0.0});
  C.stab_ptr.assign(1, 0);
  auto expand = [&](uint64_t m) {
    const int32_t rep_idx = (int32_t)C.reps.size() + 1;
    int32_t order = 0;
    for (int g = 0; g < nG; ++g) {
      uint64_t s;
      cd a;
      apply_op(G, g, m, &s, &a);
      int64_t idx = rank_combination(s);
      C.rep_rank[idx] = rep_idx;
      C.rep_sym[idx] = G.inv[g] + 1;
      C.rep_amp[idx] = cconj(a);
      if (s == m) {
        C.stab_g.push_back(g + 1);
        C.stab_phase.push_back(a);
        ++order;
      }
    }
    C.reps.push_back(m);
    C.stab_order.push_back(order);
    C.stab_ptr.push_back((int64_t)C.stab_g.size());
  };
  if (k == 0 || k == N) {
    // SRE:410-431: the single orbit; its stabilizer is the whole group.
    expand(first_combination_mask(k));
    return;
  }
  uint64_t x = first_combination_mask(k);
  const uint64_t upper = 1ULL << N;
  while (x < upper) {
    const uint64_t m = x;
    bool is_rep = true;
    for (int g = 0; g < nG; ++g) {
      uint64_t s;
      cd a;
      apply_op(G, g, m, &s, &a);
      if (s < m) {
        is_rep = false;
        break;
      }
    }
    if (is_rep) expand(m);
    x = gosper_next(x);
  }
}

// SRE:338-369 update_orbit_stabilizer_phases! (same permutations, new phases).
void update_phases(Catalog& C, const Group& Gn) {
  C.G = Gn;
  const Group& G = C.G;
  for (size_t o = 0; o < C.reps.size(); ++o) {
    for (int64_t j = C.stab_ptr[o]; j < C.stab_ptr[o + 1]; ++j) {
      uint64_t s;
      cd a;
      apply_op(G, C.stab_g[j] - 1, C.reps[o], &s, &a);
      C.stab_phase[j] = a;
    }
  }
  for (size_t o = 0; o < C.reps.size(); ++o) {
    for (int g = 0; g < G.n_ops; ++g) {
      uint64_t s;
      cd a;
      apply_op(G, g, C.reps[o], &s, &a);
      int64_t idx = rank_combination(s);
      if (C.rep_rank[idx] == (int32_t)o + 1) {
        C.rep_sym[idx] = G.inv[g] + 1;
        C.rep_amp[idx] = cconj(a);
      }
    }
  }
}

// ---------------------------------------------------------------- sector
struct Sector {
  const Catalog* cat = nullptr;
  std::vector<cd> chi;  // chi(g), g 0-based
  std::vector<uint64_t> reps;
  std::vector<int32_t> stab;
  std::vector<int32_t> orbit;  // catalog orbit index (0-based) of each row
};

// SRE:534-556 _is_orbit_compatible + build_symmetry_sector_basis (catalog order).
void build_sector(Sector& S, double atol) {
  const Catalog& C = *S.cat;
  for (size_t o = 0; o < C.reps.size(); ++o) {
    bool ok = true;
    for (int64_t j = C.stab_ptr[o]; j < C.stab_ptr[o + 1] && ok; ++j)
      ok = capprox(S.chi[C.stab_g[j] - 1], C.stab_phase[j], atol);
    if (ok) {
      S.reps.push_back(C.reps[o]);
      S.stab.push_back(C.stab_order[o]);
      S.orbit.push_back((int32_t)o);
    }
  }
}

// SRE:530-532 _basis_index: the reference probes a Dict{Mask,Int}; the sector
// reps are sorted ascending, so a binary search gives the same row.
inline int64_t basis_index(const Sector& S, uint64_t repr) {
  auto it = std::lower_bound(S.reps.begin(), S.reps.end(), repr);
  if (it == S.reps.end() || *it != repr) return -1;
  return it - S.reps.begin();
}

// SRE:584-594 get_canonical (table path, O(|G|) fallback when unset).
inline void get_canonical(const Sector& S, uint64_t m, uint64_t* repr, int* g, cd* amp) {
  const Catalog& C = *S.cat;
  int64_t idx = rank_combination(m);
  int32_t rep_idx = (idx >= 0 && idx < C.n_states) ? C.rep_rank[idx] : 0;
  if (rep_idx == 0) {
    canonical_representative(C.G, m, repr, g, amp);
    return;
  }
  *repr = C.reps[rep_idx - 1];
  *g = C.rep_sym[idx] - 1;
  *amp = C.rep_amp[idx];
}

// SRE:627-632 project_to_sector -> (row, alpha * conj(chi(g))) or none.
inline bool project_to_sector(const Sector& S, uint64_t m, int64_t* row, cd* coeff) {
  uint64_t repr;
  int g;
  cd a;
  get_canonical(S, m, &repr, &g, &a);
  int64_t r = basis_index(S, repr);
  if (r < 0) return false;
  *row = r;
  *coeff = cmul(a, cconj(S.chi[g]));
  return true;
}

// SRE:635-640 project_to_unnormalized_sector (O(|G|) canonicalization).
inline bool project_to_unnormalized_sector(const Sector& S, uint64_t m, int64_t* row, cd* coeff) {
  uint64_t repr;
  int g;
  cd a;
  canonical_representative(S.cat->G, m, &repr, &g, &a);
  int64_t r = basis_index(S, repr);
  if (r < 0) return false;
  *row = r;
  *coeff = cmul(a, cconj(S.chi[g]));
  return true;
}

// SRE:646-654 hopping_phase_for_stats (pre-hop mask, bits strictly between).
inline cd hopping_phase(int stats, uint64_t m, int i_from, int i_to) {
  if (stats == 0 || i_from == i_to) return cd{1.0, 0.0};
  int lo = std::min(i_from, i_to), hi = std::max(i_from, i_to);
  uint64_t between = (hi - lo <= 1) ? 0ULL : (((1ULL << (hi - lo - 1)) - 1ULL) << (lo + 1));
  return (popc64(m & between) & 1) ? cd{-1.0, 0.0} : cd{1.0, 0.0};
}

// ---------------------------------------------------------------- operator
struct Op {
  const Sector* sec = nullptr;
  std::vector<int32_t> bi, bj;  // 0-based sites, hop moves a particle bi -> bj
  std::vector<cd> bt;
  std::vector<int32_t> di, dj;
  std::vector<cd> dv;
  // projection table (SRE:680-728)
  std::vector<int64_t> row, col;
  std::vector<cd> vals;
  std::vector<cd> h_diag;
  bool table_built = false;
};

inline cd diag_of(const Op& H, uint64_t m) {
  cd d{0.0, 0.0};
  for (size_t t = 0; t < H.di.size(); ++t)
    if (((m >> H.di[t]) & 1ULL) && ((m >> H.dj[t]) & 1ULL)) d = cadd(d, H.dv[t]);
  return d;
}

// SRE:680-728 build_matrixfree_projection_table (serial, one projection per hop).
void build_table(Op& H) {
  const Sector& S = *H.sec;
  const int stats = S.cat->G.stats;
  const size_t D = S.reps.size();
  H.row.clear();
  H.col.clear();
  H.vals.clear();
  H.h_diag.assign(D, cd{0.0, 0.0});
  for (size_t c = 0; c < D; ++c) {
    const uint64_t m = S.reps[c];
    const int32_t stab_col = S.stab[c];
    H.h_diag[c] = diag_of(H, m);
    for (size_t t = 0; t < H.bi.size(); ++t) {
      const uint64_t from = 1ULL << H.bi[t];
      const uint64_t hop = from | (1ULL << H.bj[t]);
      if ((m & hop) != from) continue;
      int64_t r;
      cd coeff;
      if (!project_to_sector(S, m ^ hop, &r, &coeff)) continue;
      const int32_t stab_row = S.stab[r];
      cd e = cmul(cmul(H.bt[t], hopping_phase(stats, m, H.bi[t], H.bj[t])), coeff);
      e = cscale(e, std::sqrt((double)stab_row / (double)stab_col));
      H.row.push_back(r);
      H.col.push_back((int64_t)c);
      H.vals.push_back(e);
    }
  }
  H.table_built = true;
}

inline int n_threads_used(int req) {
#ifdef _OPENMP
  return req > 0 ? req : omp_get_max_threads();
#else
  (void)req;
  return 1;
#endif
}

// SRE:731-765 _apply_table!: serial diagonal, statically scheduled edge scatter
// into per-thread buffers, serial reduction over the buffers.
void apply_table(const Op& H, const cd* x, cd* y, int nthreads) {
  const int64_t n = (int64_t)H.sec->reps.size();
  const int T = n_threads_used(nthreads);
  std::vector<std::vector<cd>> yt(T, std::vector<cd>(n, cd{0.0, 0.0}));
  for (int64_t c = 0; c < n; ++c) {
    if (cis_zero(x[c])) continue;
    yt[0][c] = cadd(yt[0][c], cmul(H.h_diag[c], x[c]));
  }
  const int64_t nnz = (int64_t)H.row.size();
#pragma omp parallel num_threads(T)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<cd>& b = yt[tid];
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nnz; ++e) {
      const cd xc = x[H.col[e]];
      if (cis_zero(xc)) continue;
      b[H.row[e]] = cadd(b[H.row[e]], cmul(H.vals[e], xc));
    }
  }
  for (int64_t i = 0; i < n; ++i) y[i] = cd{0.0, 0.0};
  for (int t = 0; t < T; ++t)
    for (int64_t i = 0; i < n; ++i) y[i] = cadd(y[i], yt[t][i]);
}

// SRE:804-878 apply_hamiltonian! (on the fly, column-parallel scatter).
void apply_onthefly(const Op& H, const cd* x, cd* y, int nthreads) {
  const Sector& S = *H.sec;
  const int stats = S.cat->G.stats;
  const int64_t n = (int64_t)S.reps.size();
  const int T = n_threads_used(nthreads);
  std::vector<std::vector<cd>> yt(T, std::vector<cd>(n, cd{0.0, 0.0}));
#pragma omp parallel num_threads(T)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<cd>& b = yt[tid];
#pragma omp for schedule(static)
    for (int64_t c = 0; c < n; ++c) {
      const cd xc = x[c];
      if (cis_zero(xc)) continue;
      const uint64_t m = S.reps[c];
      const double inv_sqrt_stab_col = 1.0 / std::sqrt((double)S.stab[c]);
      b[c] = cadd(b[c], cmul(diag_of(H, m), xc));
      for (size_t t = 0; t < H.bi.size(); ++t) {
        const uint64_t from = 1ULL << H.bi[t];
        const uint64_t hop = from | (1ULL << H.bj[t]);
        if ((m & hop) != from) continue;
        int64_t r;
        cd coeff;
        if (!project_to_sector(S, m ^ hop, &r, &coeff)) continue;
        cd e = cmul(cmul(H.bt[t], hopping_phase(stats, m, H.bi[t], H.bj[t])), coeff);
        e = cscale(cscale(e, std::sqrt((double)S.stab[r])), inv_sqrt_stab_col);
        b[r] = cadd(b[r], cmul(e, xc));
      }
    }
  }
  for (int64_t i = 0; i < n; ++i) y[i] = cd{0.0, 0.0};
  for (int t = 0; t < T; ++t)
    for (int64_t i = 0; i < n; ++i) y[i] = cadd(y[i], yt[t][i]);
}

// SRE:903-963 build_ed_Hamiltonian_symmetry_block: COO triplets including one
// diagonal entry per column (duplicates summed and zeros dropped by the caller,
// like sparse() + dropzeros!).
void matrix_coo(const Op& H, std::vector<int64_t>& I, std::vector<int64_t>& J, std::vector<cd>& V) {
  const Sector& S = *H.sec;
  const int stats = S.cat->G.stats;
  for (size_t c = 0; c < S.reps.size(); ++c) {
    const uint64_t m = S.reps[c];
    const int32_t stab_col = S.stab[c];
    I.push_back((int64_t)c);
    J.push_back((int64_t)c);
    V.push_back(diag_of(H, m));
    for (size_t t = 0; t < H.bi.size(); ++t) {
      const uint64_t from = 1ULL << H.bi[t];
      const uint64_t hop = from | (1ULL << H.bj[t]);
      if ((m & hop) != from) continue;
      int64_t r;
      cd coeff;
      if (!project_to_sector(S, m ^ hop, &r, &coeff)) continue;
      const int32_t stab_row = S.stab[r];
      cd e = cmul(cmul(H.bt[t], hopping_phase(stats, m, H.bi[t], H.bj[t])), coeff);
      e = cscale(e, std::sqrt((double)stab_row / (double)stab_col));
      I.push_back(r);
      J.push_back((int64_t)c);
      V.push_back(e);
    }
  }
}

// ---------------------------------------------------------------- eigensolver
// Cyclic Jacobi for a real symmetric n x n matrix (row-major A, destroyed);
// eigenvalues ascending in w, eigenvectors as columns of Z (row-major n x n).
void jacobi_eigh(int n, std::vector<double>& A, std::vector<double>& w, std::vector<double>& Z) {
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double v = A[(size_t)i * n + j] * A[(size_t)i * n + j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-30 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A[(size_t)p * n + q];
        if (apq == 0.0) continue;
        double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - s * akq;
          A[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - s * aqk;
          A[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double zkp = Z[(size_t)k * n + p], zkq = Z[(size_t)k * n + q];
          Z[(size_t)k * n + p] = c * zkp - s * zkq;
          Z[(size_t)k * n + q] = s * zkp + c * zkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int a, int b) { return A[(size_t)a * n + a] < A[(size_t)b * n + b]; });
  std::vector<double> Zs((size_t)n * n);
  w.assign(n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = A[(size_t)ord[j] * n + ord[j]];
    for (int i = 0; i < n; ++i) Zs[(size_t)i * n + j] = Z[(size_t)i * n + ord[j]];
  }
  Z.swap(Zs);
}

// Thick-restart Lanczos with full (classical Gram-Schmidt, twice)
// reorthogonalisation: the CPU stand-in for the reference's KrylovKit call
// (SRE:1018-1026: eigsolve(H, x0, nev, :SR; tol, maxiter)).  KrylovKit itself
// is not restated; this is a textbook thick-restart Lanczos with the same
// stopping rule (absolute Ritz residual <= tol) and restart budget.
template <class MV>
int lanczos_tr(int64_t n, MV matvec, int nev, double tol, int maxiter, int krylovdim, uint64_t seed, double* evals,
               cd* evecs, int* n_restarts, int* n_matvec, double* resid_out, int nthreads) {
  if (n <= 0 || nev <= 0) return 0;
  nev = (int)std::min<int64_t>(nev, n);
  int m = (int)std::min<int64_t>(std::max(krylovdim, 2 * nev + 1), n);
  const int T = n_threads_used(nthreads);
  std::vector<cd> V((size_t)(m + 1) * n);
  std::vector<cd> w(n);
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  auto vec = [&](int j) { return &V[(size_t)j * n]; };
  auto norm2 = [&](const cd* a) {
    double s = 0;
#pragma omp parallel for reduction(+ : s) num_threads(T) schedule(static)
    for (int64_t i = 0; i < n; ++i) s += a[i].re * a[i].re + a[i].im * a[i].im;
    return std::sqrt(s);
  };
  for (int64_t i = 0; i < n; ++i) V[i] = cd{nd(rng), nd(rng)};
  {
    double s = norm2(vec(0));
    for (int64_t i = 0; i < n; ++i) V[i] = cscale(V[i], 1.0 / s);
  }
  std::vector<double> Tm((size_t)m * m, 0.0);
  int k = 0, restarts = 0, nmv = 0;
  double beta = 0.0;
  std::vector<double> theta, S;
  std::vector<cd> h(m + 1);
  int status = 1;
  for (;;) {
    int jend = m;
    for (int j = k; j < m; ++j) {
      matvec(vec(j), w.data());
      ++nmv;
      for (int pass = 0; pass < 2; ++pass) {
        for (int l = 0; l <= j; ++l) {
          const cd* v = vec(l);
          double sr = 0, si = 0;
#pragma omp parallel for reduction(+ : sr, si) num_threads(T) schedule(static)
          for (int64_t i = 0; i < n; ++i) {
            sr += v[i].re * w[i].re + v[i].im * w[i].im;
            si += v[i].re * w[i].im - v[i].im * w[i].re;
          }
          h[l] = pass == 0 ? cd{sr, si} : cadd(h[l], cd{sr, si});
          // modified Gram-Schmidt, applied twice
#pragma omp parallel for num_threads(T) schedule(static)
          for (int64_t i = 0; i < n; ++i) w[i] = csub(w[i], cmul(cd{sr, si}, v[i]));
        }
      }
      Tm[(size_t)j * m + j] = h[j].re;
      beta = norm2(w.data());
      if (j + 1 < m) {
        Tm[(size_t)j * m + j + 1] = Tm[(size_t)(j + 1) * m + j] = beta;
      }
      if (beta <= 1e-13 * std::max(1.0, std::fabs(h[j].re))) {
        jend = j + 1;
        break;
      }
      cd* vn = vec(j + 1);
      for (int64_t i = 0; i < n; ++i) vn[i] = cscale(w[i], 1.0 / beta);
    }
    const int msz = jend;
    std::vector<double> A((size_t)msz * msz);
    for (int i = 0; i < msz; ++i)
      for (int j = 0; j < msz; ++j) A[(size_t)i * msz + j] = Tm[(size_t)i * m + j];
    jacobi_eigh(msz, A, theta, S);
    const bool invariant = msz < m || msz == n;
    int nconv = 0;
    for (int i = 0; i < nev && i < msz; ++i) {
      double r = invariant ? 0.0 : std::fabs(beta * S[(size_t)(msz - 1) * msz + i]);
      if (resid_out) resid_out[i] = r;
      if (r <= tol) ++nconv;
    }
    const bool done = (nconv >= nev && msz >= nev) || invariant || restarts >= maxiter;
    int keep = done ? std::min(nev, msz) : std::min(msz - 1, std::max(nev + (m - nev) / 2, nev + 1));
    // rotate: V[:, 0:keep] = V[:, 0:msz] S[:, 0:keep]
    std::vector<cd> Vn((size_t)keep * n);
#pragma omp parallel for num_threads(T) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      for (int c = 0; c < keep; ++c) {
        cd s{0.0, 0.0};
        for (int l = 0; l < msz; ++l) s = cadd(s, cscale(V[(size_t)l * n + i], S[(size_t)l * msz + c]));
        Vn[(size_t)c * n + i] = s;
      }
    }
    if (done) {
      for (int i = 0; i < nev && i < msz; ++i) evals[i] = theta[i];
      if (evecs)
        for (int c = 0; c < std::min(nev, msz); ++c)
          for (int64_t i = 0; i < n; ++i) evecs[(size_t)c * n + i] = Vn[(size_t)c * n + i];
      status = (nconv >= nev || invariant) ? 0 : 4;
      break;
    }
    // residual direction becomes the next basis vector
    cd* vres = vec(keep);
    std::vector<cd> wres(n);
    for (int64_t i = 0; i < n; ++i) wres[i] = cscale(w[i], 1.0 / beta);
    for (int c = 0; c < keep; ++c)
      for (int64_t i = 0; i < n; ++i) V[(size_t)c * n + i] = Vn[(size_t)c * n + i];
    for (int64_t i = 0; i < n; ++i) vres[i] = wres[i];
    std::fill(Tm.begin(), Tm.end(), 0.0);
    for (int c = 0; c < keep; ++c) {
      Tm[(size_t)c * m + c] = theta[c];
      double b = beta * S[(size_t)(msz - 1) * msz + c];
      Tm[(size_t)c * m + keep] = Tm[(size_t)keep * m + c] = b;
    }
    k = keep;
    ++restarts;
  }
  if (n_restarts) *n_restarts = restarts;
  if (n_matvec) *n_matvec = nmv;
  return status;
}

thread_local std::string g_err;

}  // namespace

// ======================================================================= C ABI
extern "C" {

const char* or_last_error(void) { return g_err.c_str(); }

int64_t or_binom(int n, int k) {
  init_binom();
  return binom(n, k);
}
int64_t or_rank(uint64_t m) {
  init_binom();
  return rank_combination(m);
}
uint64_t or_gosper_next(uint64_t x) { return gosper_next(x); }

// SRE:262-292 _lin_table and SRE:295-299 lin_index.
int or_lin_table(int n_site, int n_filled, int64_t* left, int64_t* right) {
  init_binom();
  const int n_right = n_site / 2, n_left = n_site - n_right;
  for (int64_t v = 0; v < (1LL << n_right); ++v) right[v] = rank_combination((uint64_t)v);
  int64_t acc = 0;
  for (int64_t u = 0; u < (1LL << n_left); ++u) {
    left[u] = acc;
    int rem = n_filled - popc64((uint64_t)u);
    if (rem >= 0 && rem <= n_right) acc += binom(n_right, rem);
  }
  return n_right;
}
int64_t or_lin_index(uint64_t m, const int64_t* left, const int64_t* right, int n_right) {
  return left[m >> n_right] + right[m & ((1ULL << n_right) - 1ULL)];
}

static bool make_group(Group& G, int n_site, int n_ops, const int32_t* perm, const double* phase, int identity,
                       int stats) {
  if (n_site < 1 || n_site > 63) {
    g_err = "n_site must be in [1, 63]";
    return false;
  }
  if (n_ops < 1 || identity < 0 || identity >= n_ops) {
    g_err = "bad group size or identity index";
    return false;
  }
  G.n_site = n_site;
  G.n_ops = n_ops;
  G.identity = identity;
  G.stats = stats;
  G.perm.assign(perm, perm + (size_t)n_ops * n_site);
  G.phase.resize((size_t)n_ops * n_site);
  for (size_t i = 0; i < G.phase.size(); ++i) G.phase[i] = cd{phase[2 * i], phase[2 * i + 1]};
  for (int i = 0; i < n_site; ++i)
    if (G.perm[(size_t)identity * n_site + i] != i) {
      g_err = "Identity must have trivial permutation";
      return false;
    }
  return inverse_ops(G, &g_err);
}

void or_apply_op(int n_site, const int32_t* perm_row, const double* phase_row, int stats, uint64_t m, uint64_t* out,
                 double* amp) {
  Group G;
  G.n_site = n_site;
  G.n_ops = 1;
  G.stats = stats;
  G.perm.assign(perm_row, perm_row + n_site);
  G.phase.resize(n_site);
  for (int i = 0; i < n_site; ++i) G.phase[i] = cd{phase_row[2 * i], phase_row[2 * i + 1]};
  cd a;
  apply_op(G, 0, m, out, &a);
  amp[0] = a.re;
  amp[1] = a.im;
}

int or_inverse_ops(int n_site, int n_ops, const int32_t* perm, const double* phase, int identity, int stats,
                   int32_t* inv_out) {
  Group G;
  if (!make_group(G, n_site, n_ops, perm, phase, identity, stats)) return 1;
  for (int g = 0; g < n_ops; ++g) inv_out[g] = G.inv[g];
  return 0;
}

void* or_catalog_build(int n_site, int n_ops, const int32_t* perm, const double* phase, int identity, int stats,
                       int n_filled) {
  init_binom();
  Catalog* C = new Catalog();
  if (!make_group(C->G, n_site, n_ops, perm, phase, identity, stats) || n_filled < 0 || n_filled > n_site) {
    if (n_filled < 0 || n_filled > n_site) g_err = "n_filled out of range";
    delete C;
    return nullptr;
  }
  C->n_filled = n_filled;
  build_catalog(*C);
  return C;
}
int or_catalog_update_phases(void* cat, const double* phase) {
  Catalog* C = (Catalog*)cat;
  Group Gn = C->G;
  for (size_t i = 0; i < Gn.phase.size(); ++i) Gn.phase[i] = cd{phase[2 * i], phase[2 * i + 1]};
  if (!inverse_ops(Gn, &g_err)) return 1;
  update_phases(*C, Gn);
  return 0;
}
void or_catalog_free(void* cat) { delete (Catalog*)cat; }
int64_t or_catalog_n_states(void* cat) { return ((Catalog*)cat)->n_states; }
int64_t or_catalog_n_orbits(void* cat) { return (int64_t)((Catalog*)cat)->reps.size(); }
int64_t or_catalog_n_stab(void* cat) { return (int64_t)((Catalog*)cat)->stab_g.size(); }
// field: 0 reps u64, 1 stab_order i32, 2 stab_ptr i64 (n_orbits+1), 3 stab_g i32
// (1-based), 4 stab_phase f64x2, 5 rep_rank i32, 6 rep_sym i32, 7 rep_amp f64x2
int or_catalog_get(void* cat, int field, void* out) {
  Catalog* C = (Catalog*)cat;
  switch (field) {
    case 0: std::memcpy(out, C->reps.data(), C->reps.size() * 8); return 0;
    case 1: std::memcpy(out, C->stab_order.data(), C->stab_order.size() * 4); return 0;
    case 2: std::memcpy(out, C->stab_ptr.data(), C->stab_ptr.size() * 8); return 0;
    case 3: std::memcpy(out, C->stab_g.data(), C->stab_g.size() * 4); return 0;
    case 4: std::memcpy(out, C->stab_phase.data(), C->stab_phase.size() * 16); return 0;
    case 5: std::memcpy(out, C->rep_rank.data(), C->rep_rank.size() * 4); return 0;
    case 6: std::memcpy(out, C->rep_sym.data(), C->rep_sym.size() * 4); return 0;
    case 7: std::memcpy(out, C->rep_amp.data(), C->rep_amp.size() * 16); return 0;
  }
  g_err = "unknown catalog field";
  return 1;
}

void* or_sector_build(void* cat, const double* chi, double atol) {
  Sector* S = new Sector();
  S->cat = (Catalog*)cat;
  const int nG = S->cat->G.n_ops;
  S->chi.resize(nG);
  for (int g = 0; g < nG; ++g) S->chi[g] = cd{chi[2 * g], chi[2 * g + 1]};
  build_sector(*S, atol);
  return S;
}
void or_sector_free(void* s) { delete (Sector*)s; }
int64_t or_sector_dim(void* s) { return (int64_t)((Sector*)s)->reps.size(); }
void or_sector_get(void* s, uint64_t* reps, int32_t* stab, int32_t* orbit) {
  Sector* S = (Sector*)s;
  if (reps) std::memcpy(reps, S->reps.data(), S->reps.size() * 8);
  if (stab) std::memcpy(stab, S->stab.data(), S->stab.size() * 4);
  if (orbit) std::memcpy(orbit, S->orbit.data(), S->orbit.size() * 4);
}
// observables/entanglement_spectrum.jl:46-79 _expand_sector_state_to_fock_
// amplitudes: every column's coefficient spread over the group images of its
// representative, amplitudes of one mask summed in (column, g) order, entries
// with |amp| <= atol dropped, the rest normalised.  Output: dense complex128
// over the fixed-filling states in colex-rank order (dropped entries are 0).
// Returns 1 with the reference's message when the expanded norm vanishes.
int or_sector_expand_fock(void* s, const double* c_reim, double atol, double* fock_reim, double* norm2_out) {
  init_binom();
  Sector* S = (Sector*)s;
  const Catalog& C = *S->cat;
  const Group& G = C.G;
  const int nG = G.n_ops;
  std::unordered_map<uint64_t, cd> amps;
  std::vector<uint64_t> order;  // first-insertion order of the masks
  for (size_t col = 0; col < S->reps.size(); ++col) {
    const cd coeff{c_reim[2 * col], c_reim[2 * col + 1]};
    if (std::hypot(coeff.re, coeff.im) <= atol) continue;
    const double d = std::sqrt((double)(nG * S->stab[col]));
    const cd pre{coeff.re / d, coeff.im / d};
    for (int g = 0; g < nG; ++g) {
      uint64_t shifted;
      cd phase;
      apply_op(G, g, S->reps[col], &shifted, &phase);
      const cd amp = cmul(cmul(pre, cconj(S->chi[g])), phase);
      auto it = amps.find(shifted);
      if (it == amps.end()) {
        amps.emplace(shifted, amp);
        order.push_back(shifted);
      } else {
        it->second = cadd(it->second, amp);
      }
    }
  }
  double norm2 = 0.0;
  for (uint64_t m : order) {
    const cd a = amps[m];
    if (std::hypot(a.re, a.im) <= atol) {
      amps.erase(m);
      continue;
    }
    norm2 += a.re * a.re + a.im * a.im;
  }
  if (norm2_out) *norm2_out = norm2;
  if (!(norm2 > atol)) {
    g_err = "Expanded state has near-zero norm.";
    return 1;
  }
  const double invnorm = 1.0 / std::sqrt(norm2);
  for (int64_t i = 0; i < C.n_states; ++i) fock_reim[2 * i] = fock_reim[2 * i + 1] = 0.0;
  for (const auto& kv : amps) {
    const int64_t r = rank_combination(kv.first);
    fock_reim[2 * r] = kv.second.re * invnorm;
    fock_reim[2 * r + 1] = kv.second.im * invnorm;
  }
  return 0;
}

// project a mask: returns 1 and (row, coeff) when in sector; mode 0 = table
// (project_to_sector), 1 = O(|G|) (project_to_unnormalized_sector).
int or_project(void* s, uint64_t m, int mode, int64_t* row, double* coeff) {
  init_binom();
  Sector* S = (Sector*)s;
  cd c;
  bool ok = mode == 0 ? project_to_sector(*S, m, row, &c) : project_to_unnormalized_sector(*S, m, row, &c);
  if (!ok) return 0;
  coeff[0] = c.re;
  coeff[1] = c.im;
  return 1;
}
void or_canonical(void* cat, uint64_t m, uint64_t* repr, int* g, double* amp) {
  cd a;
  canonical_representative(((Catalog*)cat)->G, m, repr, g, &a);
  amp[0] = a.re;
  amp[1] = a.im;
}

// ------------------------------------------------- catalog-free, one mask at a time
// For sectors too large for an in-memory catalog (sampled parity checks): the
// same table entries and matrix elements, evaluated for single masks straight
// from the group.  Only the group is held.
void* or_group_create(int n_site, int n_ops, const int32_t* perm, const double* phase, int identity, int stats) {
  init_binom();
  Group* G = new Group();
  if (!make_group(*G, n_site, n_ops, perm, phase, identity, stats)) {
    delete G;
    return nullptr;
  }
  return G;
}
void or_group_free(void* g) { delete (Group*)g; }

// The catalog entries of one basis state m (SRE:371-487): its orbit's
// representative (the orbit minimum, SRE:442-453), the representative's
// stabilizer order, and rep_sym / rep_amp as the reference's orbit expansion
// leaves them -- the last g in 1..|G| with g(rep) = m wins (SRE:458-477):
// sym = inverse(g) (1-based), amp = conj(alpha_g(rep)).
void or_group_state_entry(void* gp, uint64_t m, uint64_t* rep_out, int32_t* stab_out, int32_t* sym_out,
                          double* amp_out) {
  const Group& G = *(Group*)gp;
  uint64_t rep = m;
  for (int g = 0; g < G.n_ops; ++g) {
    uint64_t s;
    cd a;
    apply_op(G, g, m, &s, &a);
    if (s < rep) rep = s;
  }
  int32_t order = 0, sym = 0;
  cd amp{0.0, 0.0};
  for (int g = 0; g < G.n_ops; ++g) {
    uint64_t s;
    cd a;
    apply_op(G, g, rep, &s, &a);
    if (s == rep) ++order;
    if (s == m) {
      sym = G.inv[g] + 1;
      amp = cconj(a);
    }
  }
  *rep_out = rep;
  *stab_out = order;
  *sym_out = sym;
  amp_out[0] = amp.re;
  amp_out[1] = amp.im;
}

// SRE:534-542 _is_orbit_compatible for one representative.
static bool group_compatible(const Group& G, const cd* chi, uint64_t rep, double atol) {
  for (int g = 0; g < G.n_ops; ++g) {
    uint64_t s;
    cd a;
    apply_op(G, g, rep, &s, &a);
    if (s == rep && !capprox(chi[g], a, atol)) return false;
  }
  return true;
}
int or_group_compatible(void* gp, const double* chi_reim, uint64_t rep, double atol) {
  const Group& G = *(Group*)gp;
  return group_compatible(G, (const cd*)chi_reim, rep, atol) ? 1 : 0;
}

// Column rep_c of the sector matrix by apply_hamiltonian!'s element formula
// (SRE:843-866): the diagonal, then for every bilinear term valid on rep_c
// (gate (m & hop) == from, XOR hop) the projected target (SRE:627-632, with the
// table entries of or_group_state_entry) and, when its orbit belongs to the
// sector, H[target, c] = t * s_JW * coeff * sqrt(stab_target) * (1/sqrt(stab_c)).
// Writes at most max_out entries (target representative, element); returns
// their number, or -1 when max_out is too small.
int64_t or_group_column(void* gp, const double* chi_reim, int n_bil, const int32_t* bil_ij, const double* bil_t,
                        int n_den, const int32_t* den_ij, const double* den_v, uint64_t rep_c, double atol,
                        double* diag_out, uint64_t* target_rep, double* elem, int64_t max_out) {
  const Group& G = *(Group*)gp;
  const cd* chi = (const cd*)chi_reim;
  cd d{0.0, 0.0};
  for (int t = 0; t < n_den; ++t)
    if (((rep_c >> den_ij[2 * t]) & 1ULL) && ((rep_c >> den_ij[2 * t + 1]) & 1ULL))
      d = cadd(d, cd{den_v[2 * t], den_v[2 * t + 1]});
  diag_out[0] = d.re;
  diag_out[1] = d.im;
  uint64_t r0;
  int32_t stab_c, sym0;
  double amp0[2];
  or_group_state_entry(gp, rep_c, &r0, &stab_c, &sym0, amp0);
  const double inv_sqrt_stab_col = 1.0 / std::sqrt((double)stab_c);
  int64_t n = 0;
  for (int t = 0; t < n_bil; ++t) {
    const int i = bil_ij[2 * t], j = bil_ij[2 * t + 1];
    const uint64_t from = 1ULL << i;
    const uint64_t hop = from | (1ULL << j);
    if ((rep_c & hop) != from) continue;
    const uint64_t nm = rep_c ^ hop;
    uint64_t rep;
    int32_t stab_r, sym;
    double amp[2];
    or_group_state_entry(gp, nm, &rep, &stab_r, &sym, amp);
    if (!group_compatible(G, chi, rep, atol)) continue;
    const cd coeff = cmul(cd{amp[0], amp[1]}, cconj(chi[sym - 1]));
    cd e = cmul(cmul(cd{bil_t[2 * t], bil_t[2 * t + 1]}, hopping_phase(G.stats, rep_c, i, j)), coeff);
    e = cscale(cscale(e, std::sqrt((double)stab_r)), inv_sqrt_stab_col);
    if (n >= max_out) return -1;
    target_rep[n] = rep;
    elem[2 * n] = e.re;
    elem[2 * n + 1] = e.im;
    ++n;
  }
  return n;
}

// Bilinear terms (i, j, t): a particle hops from site i to site j (0-based).
void* or_op_create(void* s, int n_bil, const int32_t* bil_ij, const double* bil_t, int n_den, const int32_t* den_ij,
                   const double* den_v) {
  init_binom();
  Op* H = new Op();
  H->sec = (Sector*)s;
  for (int t = 0; t < n_bil; ++t) {
    H->bi.push_back(bil_ij[2 * t]);
    H->bj.push_back(bil_ij[2 * t + 1]);
    H->bt.push_back(cd{bil_t[2 * t], bil_t[2 * t + 1]});
  }
  for (int t = 0; t < n_den; ++t) {
    H->di.push_back(den_ij[2 * t]);
    H->dj.push_back(den_ij[2 * t + 1]);
    H->dv.push_back(cd{den_v[2 * t], den_v[2 * t + 1]});
  }
  return H;
}
void or_op_free(void* h) { delete (Op*)h; }
int64_t or_op_build_table(void* h) {
  Op* H = (Op*)h;
  build_table(*H);
  return (int64_t)H->row.size();
}
void or_op_get_table(void* h, int64_t* row, int64_t* col, double* vals, double* diag) {
  Op* H = (Op*)h;
  if (row) std::memcpy(row, H->row.data(), H->row.size() * 8);
  if (col) std::memcpy(col, H->col.data(), H->col.size() * 8);
  if (vals) std::memcpy(vals, H->vals.data(), H->vals.size() * 16);
  if (diag) std::memcpy(diag, H->h_diag.data(), H->h_diag.size() * 16);
}
// mode 0: _apply_table! (builds the table on first use); 1: apply_hamiltonian!
void or_op_apply(void* h, const double* x, double* y, int mode, int nthreads) {
  Op* H = (Op*)h;
  if (mode == 0) {
    if (!H->table_built) build_table(*H);
    apply_table(*H, (const cd*)x, (cd*)y, nthreads);
  } else {
    apply_onthefly(*H, (const cd*)x, (cd*)y, nthreads);
  }
}
int64_t or_op_matrix_coo_count(void* h) {
  std::vector<int64_t> I, J;
  std::vector<cd> V;
  matrix_coo(*(Op*)h, I, J, V);
  return (int64_t)I.size();
}
void or_op_matrix_coo(void* h, int64_t* I, int64_t* J, double* V) {
  std::vector<int64_t> Iv, Jv;
  std::vector<cd> Vv;
  matrix_coo(*(Op*)h, Iv, Jv, Vv);
  std::memcpy(I, Iv.data(), Iv.size() * 8);
  std::memcpy(J, Jv.data(), Jv.size() * 8);
  std::memcpy(V, Vv.data(), Vv.size() * 16);
}
// CPU solve: projection table + _apply_table! under a thick-restart Lanczos.
int or_op_solve(void* h, int nev, double tol, int maxiter, int krylovdim, uint64_t seed, int nthreads, double* evals,
                double* evecs, int* n_restarts, int* n_matvec, double* resid) {
  Op* H = (Op*)h;
  if (!H->table_built) build_table(*H);
  const int64_t n = (int64_t)H->sec->reps.size();
  auto mv = [&](const cd* x, cd* y) { apply_table(*H, x, y, nthreads); };
  return lanczos_tr(n, mv, nev, tol, maxiter, krylovdim, seed, evals, (cd*)evecs, n_restarts, n_matvec, resid,
                    nthreads);
}
int or_max_threads(void) { return n_threads_used(0); }

}  // extern "C"
