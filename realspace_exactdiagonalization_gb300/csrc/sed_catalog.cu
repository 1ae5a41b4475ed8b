// sed_catalog.cu -- symmetry group, orbit catalog and sector basis on the GPU.
//
// Replaces the reference's serial construction (SRE = src/symmetry_resolved_ed.jl):
//   build_symmetry_orbit_catalog  SRE:371-487  -> k_find_reps + scan + k_expand
//   build_symmetry_sector_basis   SRE:534-556  -> k_sector_compat + scan + k_sector_rows
//   update_orbit_stabilizer_phases! SRE:338-369 -> catalog_update_phases (phases only)
// Every thread owns a run of 32 consecutive colex ranks: it unranks the first
// one (combinadic unranking) and walks the rest with Gosper's step, so the
// serial enumeration becomes a flat data-parallel sweep; representatives are
// compacted in catalog (ascending-mask) order by a prefix sum over the flag words.
#include <algorithm>
#include <cmath>
#include <cstring>

#include <atomic>
#include <mutex>

#include "sed_internal.cuh"

namespace sed {

// ------------------------------------------------------------------ binomials
static int64_t g_binom[65][65];
static std::once_flag g_binom_once;
// filled exactly once, whichever thread gets here first (the library is
// called from several host threads at once)
static void init_binom() {
  std::call_once(g_binom_once, [] {
    for (int n = 0; n <= 64; ++n)
      for (int k = 0; k <= 64; ++k) g_binom[n][k] = 0;
    for (int n = 0; n <= 64; ++n) {
      g_binom[n][0] = 1;
      for (int k = 1; k <= n; ++k) g_binom[n][k] = g_binom[n - 1][k - 1] + (k <= n - 1 ? g_binom[n - 1][k] : 0);
    }
  });
}
int64_t binom64(int n, int k) {
  init_binom();
  if (n < 0 || k < 0 || k > n || n > 64) return 0;
  return g_binom[n][k];
}

// Two conserved species (split L > 0): modes [0, L) hold klo particles and
// modes [L, N) hold khi, and the rank of a state is
//   rank_hi(m >> L) * binom(L, klo) + rank_lo(m & (2^L - 1)),
// each part a colex rank of its own subset.  Rank order is then ascending-mask
// order, the reference's catalog order restricted to the (klo, khi) block.
// Every low particle lies below bit L, so p (the set bits below chunk c)
// still determines each bit's index within its own species -- p itself below
// L, p - klo above it -- and rank_of reads the split tables unchanged.
// split = 0: one species of k = klo particles on all N modes.
void build_rank_table(int N, int split, int klo, int khi, RankTable& rt, cudaStream_t s) {
  init_binom();
  const int L = split > 0 ? split : N;
  const int k = split > 0 ? klo + khi : klo;
  if (split <= 0) khi = 0;
  const uint64_t clo = (uint64_t)binom64(L, klo);
  RankParams rp{};
  rp.nchunk = (N + 7) / 8;
  int total = 0;
  std::vector<int> pmaxs(rp.nchunk);
  for (int c = 0; c < rp.nchunk; ++c) {
    const int s0 = 8 * c;
    int pmin, pmax;
    if (s0 <= L) {  // every bit below the chunk is a low-species mode
      pmin = std::max(0, klo - (L - s0));
      pmax = std::min(klo, s0);
    } else {        // all klo low particles lie below the chunk
      pmin = klo + std::max(0, khi - (N - s0));
      pmax = klo + std::min(khi, s0 - L);
    }
    if (split <= 0) {
      pmin = std::max(0, k - (N - s0));
      pmax = std::min(k, s0);
    }
    rp.pmin[c] = pmin;
    rp.off[c] = total;
    pmaxs[c] = pmax;
    total += (std::max(pmax - pmin + 1, 1)) * 256;
  }
  rp.total = total;
  rt.host.assign(total, 0u);
  for (int c = 0; c < rp.nchunk; ++c) {
    const int s0 = 8 * c, pmin = rp.pmin[c], pmax = pmaxs[c];
    for (int p = pmin; p <= pmax; ++p)
      for (int v = 0; v < 256; ++v) {
        uint64_t sum = 0;
        int jl = s0 <= L ? p : klo, jh = s0 <= L ? 0 : p - klo;
        bool ok = true;
        for (int b = 0; b < 8; ++b)
          if ((v >> b) & 1) {
            const int pos = s0 + b;
            if (pos >= N) {
              ok = false;
            } else if (pos < L) {
              sum += (uint64_t)binom64(pos, jl + 1);
              ++jl;
            } else {
              sum += clo * (uint64_t)binom64(pos - L, jh + 1);
              ++jh;
            }
          }
        if (!ok || jl > (split > 0 ? klo : k) || jh > khi || sum > 0xFFFFFFFFull) sum = 0;
        rt.host[rp.off[c] + ((p - pmin) << 8) + v] = (uint32_t)sum;
      }
  }
  rt.rp = rp;
  upload(rt.dev, rt.host, s);
}

int current_device() {
  int d = 0;
  SED_CUDA(cudaGetDevice(&d));
  SED_REQUIRE(d >= 0 && d < kMaxDevices, 5, "device ordinal above the library's limit of 64");
  return d;
}

int device_sm_count() {
  // one entry per device, filled by the first query on that device (a failed
  // query throws and leaves it for the next call; concurrent first queries
  // store the same value)
  static std::atomic<int> sms[kMaxDevices];
  const int d = current_device();
  int n = sms[d].load(std::memory_order_relaxed);
  if (n <= 0) {
    SED_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d));
    sms[d].store(n, std::memory_order_relaxed);
  }
  return n;
}

// ---------------------------------------------------------------------- group
std::shared_ptr<GroupImpl> make_group(int n_site, int n_ops, const int32_t* perm, const double* phase, int identity,
                                      int stats) {
  SED_REQUIRE(n_site >= 1 && n_site <= SED_MAX_SITES, 5, "n_site must be in [1, 63]");
  SED_REQUIRE(n_ops >= 1 && n_ops <= SED_MAX_OPS, 5, "the group may hold at most 64 operations");
  SED_REQUIRE(identity >= 0 && identity < n_ops, 1, "identity index out of range");
  SED_REQUIRE(stats == 0 || stats == 1, 1, "stats must be SED_BOSONIC or SED_FERMIONIC");
  SED_REQUIRE(perm != nullptr && phase != nullptr, 1, "perm and phase must not be NULL");
  auto G = std::make_shared<GroupImpl>();
  G->n_site = n_site;
  G->n_ops = n_ops;
  G->identity = identity;
  G->stats = stats;
  G->perm.assign(perm, perm + (size_t)n_ops * n_site);
  G->phase.assign(phase, phase + (size_t)n_ops * n_site * 2);
  for (int g = 0; g < n_ops; ++g) {
    std::vector<char> seen(n_site, 0);
    for (int i = 0; i < n_site; ++i) {
      const int p = G->perm[(size_t)g * n_site + i];
      SED_REQUIRE(p >= 0 && p < n_site && !seen[p], 1, "every operation must permute the sites");
      seen[p] = 1;
    }
  }
  for (int i = 0; i < n_site; ++i)
    SED_REQUIRE(G->perm[(size_t)identity * n_site + i] == i, 1, "Identity must have trivial permutation");
  for (size_t i = 0; i < G->phase.size(); i += 2)
    if (G->phase[i] != 1.0 || G->phase[i + 1] != 0.0) G->has_phases = true;
  // _inverse_operation_indices (SRE:109-117): first h with h.perm[g.perm] == id
  // and eta_g(i) * eta_h(perm_g(i)) ~ 1 (atol 1e-12).
  G->inv.assign(n_ops, -1);
  for (int g = 0; g < n_ops; ++g) {
    const int32_t* pg = &G->perm[(size_t)g * n_site];
    const double* eg = &G->phase[(size_t)g * n_site * 2];
    for (int h = 0; h < n_ops && G->inv[g] < 0; ++h) {
      const int32_t* ph = &G->perm[(size_t)h * n_site];
      const double* eh = &G->phase[(size_t)h * n_site * 2];
      bool ok = true;
      for (int i = 0; i < n_site && ok; ++i) ok = ph[pg[i]] == i;
      for (int i = 0; i < n_site && ok; ++i) {
        const double ar = eg[2 * i], ai = eg[2 * i + 1];
        const double br = eh[2 * pg[i]], bi = eh[2 * pg[i] + 1];
        const double re = ar * br - ai * bi, im = ar * bi + ai * br;
        ok = (re == 1.0 && im == 0.0) || std::hypot(re - 1.0, im) <= 1e-12;
      }
      if (ok) G->inv[g] = h;
    }
    SED_REQUIRE(G->inv[g] >= 0, 1, "Symmetry operations are not closed under inversion.");
  }
  return G;
}

// ------------------------------------------------------------ block scan (u32)
static constexpr int kScanBS = 512;
static constexpr int kScanIPT = 8;
static constexpr int kScanTile = kScanBS * kScanIPT;

__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t v, uint32_t* wsum) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) wsum[wid] = v;
  __syncthreads();
  if (wid == 0) {
    uint32_t s = lane < nw ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += t;
    }
    wsum[lane] = s;
  }
  __syncthreads();
  if (wid > 0) v += wsum[wid - 1];
  __syncthreads();
  return v;
}

__global__ void __launch_bounds__(kScanBS) k_scan_reduce(const uint32_t* __restrict__ words, int64_t n,
                                                         uint32_t* __restrict__ bsum) {
  __shared__ uint32_t wsum[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
  for (int i = 0; i < kScanIPT; ++i) {
    const int64_t w = base + (int64_t)threadIdx.x * kScanIPT + i;
    if (w < n) s += __popc(words[w]);
  }
  const uint32_t incl = block_inclusive_scan(s, wsum);
  if (threadIdx.x == blockDim.x - 1) bsum[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(uint32_t* __restrict__ bsum, int64_t nb,
                                                      uint32_t* __restrict__ total) {
  __shared__ uint32_t wsum[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const uint32_t v = i < nb ? bsum[i] : 0u;
    const uint32_t incl = block_inclusive_scan(v, wsum);
    const uint32_t c = carry;
    if (i < nb) bsum[i] = c + incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanBS) k_scan_final(const uint32_t* __restrict__ words, int64_t n,
                                                        const uint32_t* __restrict__ bsum,
                                                        uint32_t* __restrict__ offs) {
  __shared__ uint32_t wsum[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanIPT;
  uint32_t v[kScanIPT];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanIPT; ++i) {
    v[i] = (base + i < n) ? (uint32_t)__popc(words[base + i]) : 0u;
    s += v[i];
  }
  const uint32_t incl = block_inclusive_scan(s, wsum);
  uint32_t run = bsum[blockIdx.x] + incl - s;
#pragma unroll
  for (int i = 0; i < kScanIPT; ++i) {
    if (base + i < n) offs[base + i] = run;
    run += v[i];
  }
}

// Exclusive prefix sum of popcount(words[w]); returns the total (synchronises).
static uint64_t scan_popcount(const uint32_t* words, int64_t n, uint32_t* offs, cudaStream_t s) {
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  DevBuf bsum((size_t)std::max<int64_t>(nb, 1) * 4), tot(8);
  if (n > 0) {
    k_scan_reduce<<<(unsigned)nb, kScanBS, 0, s>>>(words, n, bsum.as<uint32_t>());
    k_scan_blocks<<<1, 1024, 0, s>>>(bsum.as<uint32_t>(), nb, tot.as<uint32_t>());
    k_scan_final<<<(unsigned)nb, kScanBS, 0, s>>>(words, n, bsum.as<uint32_t>(), offs);
  } else {
    SED_CUDA(cudaMemsetAsync(tot.p, 0, 4, s));
  }
  SED_CUDA(cudaGetLastError());
  uint32_t total = 0;
  SED_CUDA(cudaMemcpyAsync(&total, tot.p, 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
  return total;
}

// ------------------------------------------------------------ catalog kernels
// Combinadic unranking: the colex k-subset of rank r (inverse of SRE:231-243).
__device__ __forceinline__ uint64_t unrank_colex(uint64_t r, int N, int k, const uint64_t* __restrict__ binom) {
  uint64_t m = 0;
  int b = N - 1;
  for (int j = k; j >= 1; --j) {
    while (b >= j && binom[b * 65 + j] > r) --b;
    m |= 1ULL << b;
    r -= binom[b * 65 + j];
    --b;
  }
  return m;
}

// The enumeration of a catalog's basis states in rank order: colex k-subsets
// of N modes, or (split L > 0) the two-species product with the high species
// as the major index (see build_rank_table).
struct EnumParams {
  int N, k;        // one species: k particles on N modes
  int L, klo, khi; // two species (L > 0): klo on [0, L), khi on [L, N)
  uint64_t clo;    // binom(L, klo)
};

__device__ __forceinline__ uint64_t enum_unrank(uint64_t r, const EnumParams& e, const uint64_t* __restrict__ binom) {
  if (e.L == 0) return unrank_colex(r, e.N, e.k, binom);
  return unrank_colex(r % e.clo, e.L, e.klo, binom) | (unrank_colex(r / e.clo, e.N - e.L, e.khi, binom) << e.L);
}

// the state after m in rank order (called only when one exists)
__device__ __forceinline__ uint64_t enum_next(uint64_t m, const EnumParams& e) {
  if (e.L == 0) return dev::gosper_next(m);
  const uint64_t lomask = (1ULL << e.L) - 1ULL;
  if (e.klo > 0) {
    const uint64_t nl = dev::gosper_next(m & lomask);
    if (!(nl >> e.L)) return (m & ~lomask) | nl;
  }
  if (e.khi == 0) return m;  // unreachable: no state follows the last one
  return ((1ULL << e.klo) - 1ULL) | (dev::gosper_next(m >> e.L) << e.L);
}

// SRE:434-455: a mask is a representative iff no group image is smaller
// (early exit on the first smaller image).  One flag bit per colex rank.
__global__ void __launch_bounds__(256) k_find_reps(int64_t n_states, EnumParams e, int G,
                                                   const uint8_t* __restrict__ perm_g,
                                                   const uint64_t* __restrict__ binom, uint32_t* __restrict__ flags) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  __syncthreads();
  const int64_t nw = (n_states + 31) / 32;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
    uint64_t m = enum_unrank((uint64_t)w * 32, e, binom);
    const int cnt = (int)min((int64_t)32, n_states - w * 32);
    uint32_t f = 0;
    for (int b = 0; b < cnt; ++b) {
      bool rep = true;
      for (int g = 0; g < G; ++g)
        if (dev::apply_perm(m, sperm + g * 64) < m) {
          rep = false;
          break;
        }
      if (rep) f |= 1u << b;
      if (b + 1 < cnt) m = enum_next(m, e);
    }
    flags[w] = f;
  }
}

// SRE:456-477: for every representative, one pass over g in ascending order
// writes the state word of g(rep) (the last g wins where the stabilizer is
// non-trivial, exactly as the reference's loop overwrites), plus the
// representative list and stabilizer order in catalog order.
__global__ void __launch_bounds__(256) k_expand(int64_t n_states, EnumParams e, int G, int fermi,
                                                const uint8_t* __restrict__ perm_g,
                                                const uint64_t* __restrict__ binom,
                                                const uint32_t* __restrict__ flags,
                                                const uint32_t* __restrict__ offs,
                                                const uint32_t* __restrict__ rank_tab, RankParams rp,
                                                const uint8_t* __restrict__ inv, uint64_t* __restrict__ state,
                                                uint64_t* __restrict__ reps, uint8_t* __restrict__ stab) {
  extern __shared__ uint32_t srank[];
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  __shared__ uint8_t sinv[SED_MAX_OPS];
  for (int i = threadIdx.x; i < rp.total; i += blockDim.x) srank[i] = rank_tab[i];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  for (int i = threadIdx.x; i < G; i += blockDim.x) sinv[i] = inv[i];
  __syncthreads();
  const int64_t nw = (n_states + 31) / 32;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t f = flags[w];
    if (!f) continue;
    uint64_t m = enum_unrank((uint64_t)w * 32, e, binom);
    int pos = 0;
    uint32_t o = offs[w];
    while (f) {
      const int b = __ffs(f) - 1;
      f &= f - 1;
      while (pos < b) {
        m = enum_next(m, e);
        ++pos;
      }
      int so = 0;
      for (int g = 0; g < G; ++g) so += dev::apply_perm(m, sperm + g * 64) == m;
      for (int g = 0; g < G; ++g) {
        int par = 0;
        const uint64_t img = dev::apply_perm_parity(m, sperm + g * 64, &par);
        const uint32_t idx = dev::rank_of(img, srank, rp);
        state[idx] = (uint64_t)o | ((uint64_t)g << 32) | ((uint64_t)(fermi ? par : 0) << 40) | ((uint64_t)so << 41) |
                     ((uint64_t)sinv[g] << 48);
      }
      reps[o] = m;
      stab[o] = (uint8_t)so;
      ++o;
    }
  }
}

CatalogImpl::~CatalogImpl() {
  if (own_stream && stream) cudaStreamDestroy(stream);
}

void CatalogImpl::upload_group_phases() {
  const GroupImpl& G = *group;
  std::vector<double> ph(G.phase);
  upload(phase, ph, stream);
}

static int grid_for(int64_t work, int block) {
  const int64_t sms = device_sm_count();
  int64_t g = (work + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, sms * 16));
}

std::shared_ptr<CatalogImpl> build_catalog(std::shared_ptr<GroupImpl> gp, int n_filled, int split, int n_lo,
                                           int n_hi) {
  const GroupImpl& G = *gp;
  int64_t n_states = 0;
  if (split > 0) {
    SED_REQUIRE(split < G.n_site, 1, "the species split must lie inside the lattice: 0 < n_split < n_site");
    SED_REQUIRE(n_lo >= 0 && n_lo <= split && n_hi >= 0 && n_hi <= G.n_site - split, 1,
                "species particle numbers must be in [0, modes of the species]");
    for (int g = 0; g < G.n_ops; ++g)
      for (int i = 0; i < G.n_site; ++i)
        SED_REQUIRE((G.perm[(size_t)g * G.n_site + i] < split) == (i < split), 1,
                    "every symmetry operation must map each species onto itself");
    n_filled = n_lo + n_hi;
    n_states = binom64(split, n_lo) * binom64(G.n_site - split, n_hi);
    SED_REQUIRE(n_states < (int64_t)0xFFFFFFFFll, 5,
                "binomial(n_split, n_lo) * binomial(n_site - n_split, n_hi) must be below 2^32");
  } else {
    SED_REQUIRE(n_filled >= 0 && n_filled <= G.n_site, 1, "n_filled must be in [0, n_site]");
    n_states = binom64(G.n_site, n_filled);
    SED_REQUIRE(n_states < (int64_t)0xFFFFFFFFll, 5, "binomial(n_site, n_filled) must be below 2^32");
    split = n_lo = n_hi = 0;
  }
  auto c = std::make_shared<CatalogImpl>();
  c->group = gp;
  c->n_filled = n_filled;
  c->split = split;
  c->n_lo = n_lo;
  c->n_hi = n_hi;
  c->n_states = n_states;
  SED_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->own_stream = true;
  cudaStream_t s = c->stream;
  build_rank_table(G.n_site, split, split > 0 ? n_lo : n_filled, n_hi, c->rank, s);
  SED_REQUIRE((size_t)c->rank.rp.total * 4 <= 160 * 1024, 5, "rank table exceeds the shared-memory budget");
  std::vector<uint8_t> perm_u8((size_t)G.n_ops * 64, 0);
  for (int g = 0; g < G.n_ops; ++g)
    for (int i = 0; i < G.n_site; ++i) perm_u8[(size_t)g * 64 + i] = (uint8_t)G.perm[(size_t)g * G.n_site + i];
  upload(c->perm_u8, perm_u8, s);
  std::vector<uint8_t> inv_u8(G.n_ops);
  for (int g = 0; g < G.n_ops; ++g) inv_u8[g] = (uint8_t)G.inv[g];
  upload(c->inv_u8, inv_u8, s);
  c->upload_group_phases();
  init_binom();
  std::vector<uint64_t> bn(65 * 65);
  for (int n = 0; n <= 64; ++n)
    for (int k = 0; k <= 64; ++k) bn[n * 65 + k] = (uint64_t)g_binom[n][k];
  upload(c->binom, bn, s);

  c->state.alloc((size_t)n_states * 8);
  SED_CUDA(cudaMemsetAsync(c->state.p, 0xFF, (size_t)n_states * 8, s));
  const int64_t nw = (n_states + 31) / 32;
  DevBuf flags((size_t)nw * 4), offs((size_t)nw * 4);
  EnumParams e{G.n_site, n_filled, split, n_lo, n_hi, split > 0 ? (uint64_t)binom64(split, n_lo) : 1};
  k_find_reps<<<grid_for(nw, 256), 256, 0, s>>>(n_states, e, G.n_ops, c->perm_u8.as<uint8_t>(),
                                                c->binom.as<uint64_t>(), flags.as<uint32_t>());
  SED_CUDA(cudaGetLastError());
  c->n_orbits = (int64_t)scan_popcount(flags.as<uint32_t>(), nw, offs.as<uint32_t>(), s);
  c->reps.alloc((size_t)c->n_orbits * 8);
  c->stab.alloc((size_t)c->n_orbits);
  const size_t smem = (size_t)c->rank.rp.total * 4;
  {
    // the opt-in covers the dynamic part (the kernel also holds 4 KB of static
    // shared memory); it is a property of the kernel on each device, shared
    // by every catalog and host thread, so it is only raised, and
    // raised-and-launched under one lock: a concurrent build with a smaller
    // rank table cannot undercut this launch
    static std::mutex mu;
    static SmemOptIn optin;
    std::lock_guard<std::mutex> lock(mu);
    optin.ensure(k_expand, smem);
    k_expand<<<grid_for(nw, 256), 256, smem, s>>>(n_states, e, G.n_ops, G.stats,
                                                  c->perm_u8.as<uint8_t>(), c->binom.as<uint64_t>(),
                                                  flags.as<uint32_t>(), offs.as<uint32_t>(),
                                                  c->rank.dev.as<uint32_t>(), c->rank.rp, c->inv_u8.as<uint8_t>(),
                                                  c->state.as<uint64_t>(), c->reps.as<uint64_t>(),
                                                  c->stab.as<uint8_t>());
    SED_CUDA(cudaGetLastError());
  }
  c->stab_host.resize(c->n_orbits);
  if (c->n_orbits)
    SED_CUDA(cudaMemcpyAsync(c->stab_host.data(), c->stab.p, c->n_orbits, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
  int64_t tot = 0;
  for (uint8_t v : c->stab_host) tot += v;
  c->n_stab_total = tot;
  return c;
}

void check_species_terms(const CatalogImpl& c, int n_bil, const int32_t* bil_ij) {
  if (c.split <= 0) return;
  for (int k = 0; k < n_bil; ++k)
    SED_REQUIRE((bil_ij[2 * k] < c.split) == (bil_ij[2 * k + 1] < c.split), 1,
                "a bilinear term moves a particle between the two conserved species");
}

void catalog_update_phases(CatalogImpl& c, std::shared_ptr<GroupImpl> g) {
  const GroupImpl& A = *c.group;
  const GroupImpl& B = *g;
  SED_REQUIRE(A.n_site == B.n_site && A.n_ops == B.n_ops && A.perm == B.perm && A.stats == B.stats, 1,
              "the new group must have the same permutations and statistics");
  c.group = g;
  std::vector<uint8_t> inv_u8(B.n_ops);
  for (int i = 0; i < B.n_ops; ++i) inv_u8[i] = (uint8_t)B.inv[i];
  upload(c.inv_u8, inv_u8, c.stream);
  c.upload_group_phases();
  SED_CUDA(cudaStreamSynchronize(c.stream));
}

// ------------------------------------------------------------------ readback
__global__ void k_rb_state(int64_t n_states, const uint64_t* __restrict__ state, const uint64_t* __restrict__ reps,
                           int G, int N, int fermi, const uint8_t* __restrict__ perm_g,
                           const uint8_t* __restrict__ inv, const double2* __restrict__ phase, int32_t* rank_out,
                           int32_t* sym_out, double2* amp_out) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_states;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t w = state[i];
    const uint32_t o = (uint32_t)w;
    if (o == SED_UNSET_ORBIT) {
      if (rank_out) rank_out[i] = 0;
      if (sym_out) sym_out[i] = 0;
      if (amp_out) amp_out[i] = make_double2(0.0, 0.0);
      continue;
    }
    const int g = (int)((w >> 32) & 0xFF);
    if (rank_out) rank_out[i] = (int32_t)o + 1;
    if (sym_out) sym_out[i] = (int32_t)inv[g] + 1;
    if (amp_out) {
      double2 a;
      dev::apply_full(reps[o], sperm + g * 64, phase + (size_t)g * N, fermi, &a);
      amp_out[i] = make_double2(a.x, -a.y);  // rep_amp = conj(alpha_g(rep))
    }
  }
}

__global__ void k_rb_stab(int64_t n_orb, const uint64_t* __restrict__ reps, const int64_t* __restrict__ ptr, int G,
                          int N, int fermi, const uint8_t* __restrict__ perm_g, const double2* __restrict__ phase,
                          int32_t* g_out, double2* ph_out) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  __syncthreads();
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t m = reps[o];
    int64_t j = ptr[o];
    for (int g = 0; g < G; ++g) {
      // integer image first; the FP64 phase product only for stabilizer elements
      if (dev::apply_perm(m, sperm + g * 64) != m) continue;
      double2 a;
      dev::apply_full(m, sperm + g * 64, phase + (size_t)g * N, fermi, &a);
      if (g_out) g_out[j] = g + 1;
      if (ph_out) ph_out[j] = a;
      ++j;
    }
  }
}

void catalog_readback(const CatalogImpl& c, int field, void* out, int64_t out_bytes) {
  const GroupImpl& G = *c.group;
  cudaStream_t s = c.stream;
  auto need = [&](int64_t bytes) {
    SED_REQUIRE(out != nullptr && out_bytes >= bytes, 1, "output buffer too small for the requested field");
  };
  switch (field) {
    case 0:
      need(c.n_orbits * 8);
      if (c.n_orbits) SED_CUDA(cudaMemcpyAsync(out, c.reps.p, c.n_orbits * 8, cudaMemcpyDeviceToHost, s));
      break;
    case 1: {
      need(c.n_orbits * 4);
      int32_t* o = (int32_t*)out;
      for (int64_t i = 0; i < c.n_orbits; ++i) o[i] = c.stab_host[i];
      break;
    }
    case 2: {
      need((c.n_orbits + 1) * 8);
      int64_t* o = (int64_t*)out;
      o[0] = 0;
      for (int64_t i = 0; i < c.n_orbits; ++i) o[i + 1] = o[i] + c.stab_host[i];
      break;
    }
    case 3:
    case 4: {
      need(c.n_stab_total * (field == 3 ? 4 : 16));
      std::vector<int64_t> ptr(c.n_orbits + 1, 0);
      for (int64_t i = 0; i < c.n_orbits; ++i) ptr[i + 1] = ptr[i] + c.stab_host[i];
      DevBuf dptr, dout((size_t)c.n_stab_total * (field == 3 ? 4 : 16));
      upload(dptr, ptr, s);
      k_rb_stab<<<grid_for(c.n_orbits, 256), 256, 0, s>>>(
          c.n_orbits, c.reps.as<uint64_t>(), dptr.as<int64_t>(), G.n_ops, G.n_site, G.stats, c.perm_u8.as<uint8_t>(),
          c.phase.as<double2>(), field == 3 ? dout.as<int32_t>() : nullptr,
          field == 4 ? dout.as<double2>() : nullptr);
      SED_CUDA(cudaGetLastError());
      SED_CUDA(cudaMemcpyAsync(out, dout.p, (size_t)c.n_stab_total * (field == 3 ? 4 : 16), cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
      break;
    }
    case 5:
    case 6:
    case 7: {
      const size_t el = field == 7 ? 16 : 4;
      need(c.n_states * (int64_t)el);
      DevBuf dout((size_t)c.n_states * el);
      k_rb_state<<<grid_for(c.n_states, 256), 256, 0, s>>>(
          c.n_states, c.state.as<uint64_t>(), c.reps.as<uint64_t>(), G.n_ops, G.n_site, G.stats,
          c.perm_u8.as<uint8_t>(), c.inv_u8.as<uint8_t>(), c.phase.as<double2>(),
          field == 5 ? dout.as<int32_t>() : nullptr, field == 6 ? dout.as<int32_t>() : nullptr,
          field == 7 ? dout.as<double2>() : nullptr);
      SED_CUDA(cudaGetLastError());
      SED_CUDA(cudaMemcpyAsync(out, dout.p, (size_t)c.n_states * el, cudaMemcpyDeviceToHost, s));
      SED_CUDA(cudaStreamSynchronize(s));
      break;
    }
    default:
      throw Error{1, "unknown catalog field"};
  }
  SED_CUDA(cudaStreamSynchronize(s));
}

// --------------------------------------------------------------------- sector
// SRE:534-542: orbit compatible iff chi(h) ~ alpha_h(rep) (atol) for every
// stabilizer element h; isapprox(x, y; atol) is x == y || hypot(x - y) <= atol.
__global__ void __launch_bounds__(256) k_sector_compat(int64_t n_orb, int G, int N, int fermi,
                                                       const uint64_t* __restrict__ reps,
                                                       const uint8_t* __restrict__ perm_g,
                                                       const double2* __restrict__ phase,
                                                       const double2* __restrict__ chi, double atol,
                                                       uint8_t* __restrict__ rowflag, uint32_t* __restrict__ words) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  __shared__ double2 schi[SED_MAX_OPS];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  for (int i = threadIdx.x; i < G; i += blockDim.x) schi[i] = chi[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * 32; base < n_orb; base += nwarps * 32) {
    const int64_t o = base + lane;
    int ok = 0;
    if (o < n_orb) {
      ok = 1;
      const uint64_t m = reps[o];
      for (int g = 0; g < G; ++g) {
        // the amplitude matters only for stabilizer elements: the integer
        // image first, the FP64 phase product (GB300's scarce FP64 pipe) only
        // when the image is the representative itself
        if (dev::apply_perm(m, sperm + g * 64) != m) continue;
        double2 a;
        dev::apply_full(m, sperm + g * 64, phase + (size_t)g * N, fermi, &a);
        const double2 x = schi[g];
        if (!((x.x == a.x && x.y == a.y) || hypot(x.x - a.x, x.y - a.y) <= atol)) ok = 0;
      }
      rowflag[o] = (uint8_t)ok;
    }
    const uint32_t word = __ballot_sync(0xFFFFFFFFu, ok);
    if (lane == 0) words[base >> 5] = word;
  }
}

__global__ void k_sector_rows(int64_t nw, const uint32_t* __restrict__ words, const uint32_t* __restrict__ offs,
                              uint32_t* __restrict__ row_orbit) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t f = words[w];
    uint32_t r = offs[w];
    while (f) {
      const int b = __ffs(f) - 1;
      f &= f - 1;
      row_orbit[r++] = (uint32_t)(w * 32 + b);
    }
  }
}

std::shared_ptr<SectorImpl> build_sector(std::shared_ptr<CatalogImpl> cp, const double* chi, double atol,
                                         std::shared_ptr<GroupImpl> gp) {
  CatalogImpl& c = *cp;
  if (!gp) gp = c.group;
  const GroupImpl& G = *gp;
  const GroupImpl& CG = *c.group;
  SED_REQUIRE(G.n_site == CG.n_site && G.n_ops == CG.n_ops && G.perm == CG.perm && G.stats == CG.stats &&
                  G.inv == CG.inv,
              1, "the sector's group must have the catalog's permutations and statistics");
  SED_REQUIRE(chi != nullptr, 1, "chi must not be NULL");
  auto S = std::make_shared<SectorImpl>();
  S->cat = cp;
  S->group = gp;
  S->chi.assign(chi, chi + 2 * G.n_ops);
  S->atol = atol;
  cudaStream_t s = c.stream;
  upload(S->phase, G.phase, s);
  const int64_t n = c.n_orbits;
  const int64_t nw = (n + 31) / 32;
  S->rowflag.alloc((size_t)std::max<int64_t>(n, 1));
  DevBuf dchi, words((size_t)std::max<int64_t>(nw, 1) * 4), offs((size_t)std::max<int64_t>(nw, 1) * 4);
  upload(dchi, S->chi, s);
  if (n > 0) {
    const int blocks = (int)std::min<int64_t>((nw * 32 + 255) / 256, (int64_t)device_sm_count() * 16);
    k_sector_compat<<<blocks, 256, 0, s>>>(n, G.n_ops, G.n_site, G.stats, c.reps.as<uint64_t>(),
                                           c.perm_u8.as<uint8_t>(), S->phase.as<double2>(), dchi.as<double2>(), atol,
                                           S->rowflag.as<uint8_t>(), words.as<uint32_t>());
    SED_CUDA(cudaGetLastError());
  }
  S->dim = (int64_t)scan_popcount(words.as<uint32_t>(), nw, offs.as<uint32_t>(), s);
  S->row_orbit.alloc((size_t)std::max<int64_t>(S->dim, 1) * 4);
  if (nw > 0) {
    k_sector_rows<<<grid_for(nw, 256), 256, 0, s>>>(nw, words.as<uint32_t>(), offs.as<uint32_t>(),
                                                    S->row_orbit.as<uint32_t>());
    SED_CUDA(cudaGetLastError());
  }
  SED_CUDA(cudaStreamSynchronize(s));
  return S;
}

__global__ void k_sector_gather(int64_t dim, const uint32_t* __restrict__ row_orbit, const uint64_t* __restrict__ reps,
                                const uint8_t* __restrict__ stab, uint64_t* reps_out, int32_t* stab_out,
                                int32_t* orb_out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t o = row_orbit[r];
    if (reps_out) reps_out[r] = reps[o];
    if (stab_out) stab_out[r] = stab[o];
    if (orb_out) orb_out[r] = (int32_t)o;
  }
}

// project_to_sector (SRE:627-632): rank -> state word -> (orbit, g); the
// coefficient is rep_amp * conj(chi(rep_sym)) with rep_amp = conj(alpha_g(rep)).
__global__ void k_sector_project(int64_t n, const uint64_t* __restrict__ masks, const uint64_t* __restrict__ state,
                                 const uint64_t* __restrict__ reps, const int32_t* __restrict__ orbit_row, int G,
                                 int N, int fermi, const uint8_t* __restrict__ perm_g, const uint8_t* __restrict__ inv,
                                 const double2* __restrict__ phase, const double2* __restrict__ chi,
                                 const uint32_t* __restrict__ rank_tab, RankParams rp, int64_t* row_out,
                                 double2* coeff_out) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t w = state[dev::rank_of(masks[i], rank_tab, rp)];
    const uint32_t o = (uint32_t)w;
    const int32_t r = o == SED_UNSET_ORBIT ? -1 : orbit_row[o];
    row_out[i] = r;
    if (r < 0) {
      coeff_out[i] = make_double2(0.0, 0.0);
      continue;
    }
    const int g = (int)((w >> 32) & 0xFF);
    double2 a;
    dev::apply_full(reps[o], sperm + g * 64, phase + (size_t)g * N, fermi, &a);
    a.y = -a.y;  // rep_amp
    const double2 c = chi[inv[g]];
    coeff_out[i] = dev::cmul_rn(a, make_double2(c.x, -c.y));
  }
}

// The reference's three tables at single masks (rank -> state word), for
// sampled checks of catalogs too large to read back whole.
__global__ void k_lookup(int64_t n, const uint64_t* __restrict__ masks, const uint64_t* __restrict__ state,
                         const uint64_t* __restrict__ reps, int G, int N, int fermi, const uint8_t* __restrict__ perm_g,
                         const uint8_t* __restrict__ inv, const double2* __restrict__ phase,
                         const uint32_t* __restrict__ rank_tab, RankParams rp, int32_t* rank_out, int32_t* sym_out,
                         double2* amp_out) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t w = state[dev::rank_of(masks[i], rank_tab, rp)];
    const uint32_t o = (uint32_t)w;
    if (o == SED_UNSET_ORBIT) {
      rank_out[i] = 0;
      sym_out[i] = 0;
      amp_out[i] = make_double2(0.0, 0.0);
      continue;
    }
    const int g = (int)((w >> 32) & 0xFF);
    rank_out[i] = (int32_t)o + 1;
    sym_out[i] = (int32_t)inv[g] + 1;
    double2 a;
    dev::apply_full(reps[o], sperm + g * 64, phase + (size_t)g * N, fermi, &a);
    amp_out[i] = make_double2(a.x, -a.y);
  }
}

void catalog_lookup(const CatalogImpl& c, int64_t n, const uint64_t* masks, int32_t* rank, int32_t* sym,
                    double* amp) {
  const GroupImpl& G = *c.group;
  SED_REQUIRE(n >= 0 && (n == 0 || (masks && rank && sym && amp)), 1, "NULL argument");
  const uint64_t valid = (1ULL << G.n_site) - 1ULL;
  for (int64_t i = 0; i < n; ++i)
    SED_REQUIRE((masks[i] & ~valid) == 0 && catalog_holds(c, masks[i]), 1,
                c.split > 0 ? "every mask must hold n_lo particles below n_split and n_hi above it"
                            : "every mask must hold n_filled particles on the lattice sites");
  if (n == 0) return;
  cudaStream_t s = c.stream;
  DevBuf dm((size_t)n * 8), dr((size_t)n * 4), ds((size_t)n * 4), da((size_t)n * 16);
  SED_CUDA(cudaMemcpyAsync(dm.p, masks, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  k_lookup<<<grid_for(n, 256), 256, 0, s>>>(n, dm.as<uint64_t>(), c.state.as<uint64_t>(), c.reps.as<uint64_t>(),
                                            G.n_ops, G.n_site, G.stats, c.perm_u8.as<uint8_t>(),
                                            c.inv_u8.as<uint8_t>(), c.phase.as<double2>(), c.rank.dev.as<uint32_t>(),
                                            c.rank.rp, dr.as<int32_t>(), ds.as<int32_t>(), da.as<double2>());
  SED_CUDA(cudaGetLastError());
  SED_CUDA(cudaMemcpyAsync(rank, dr.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaMemcpyAsync(sym, ds.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaMemcpyAsync(amp, da.p, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

__global__ void k_orbit_row(int64_t dim, const uint32_t* __restrict__ row_orbit, int32_t* __restrict__ orbit_row) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
    orbit_row[row_orbit[r]] = (int32_t)r;
}

void sector_project(const SectorImpl& S, int64_t n, const uint64_t* masks, int64_t* rows, double* coeff) {
  const CatalogImpl& c = *S.cat;
  const GroupImpl& G = *S.group;
  SED_REQUIRE(n >= 0 && (n == 0 || (masks && rows && coeff)), 1, "NULL argument");
  const uint64_t valid = G.n_site == 64 ? ~0ULL : ((1ULL << G.n_site) - 1ULL);
  for (int64_t i = 0; i < n; ++i)
    SED_REQUIRE((masks[i] & ~valid) == 0 && catalog_holds(c, masks[i]), 1,
                c.split > 0 ? "every mask must hold n_lo particles below n_split and n_hi above it"
                            : "every mask must hold n_filled particles on the lattice sites");
  if (n == 0) return;
  cudaStream_t s = c.stream;
  DevBuf orow((size_t)std::max<int64_t>(c.n_orbits, 1) * 4), dm((size_t)n * 8), dr((size_t)n * 8),
      dc((size_t)n * 16), dchi;
  SED_CUDA(cudaMemsetAsync(orow.p, 0xFF, (size_t)std::max<int64_t>(c.n_orbits, 1) * 4, s));
  if (S.dim)
    k_orbit_row<<<grid_for(S.dim, 256), 256, 0, s>>>(S.dim, S.row_orbit.as<uint32_t>(), orow.as<int32_t>());
  upload(dchi, S.chi, s);
  SED_CUDA(cudaMemcpyAsync(dm.p, masks, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  k_sector_project<<<grid_for(n, 256), 256, 0, s>>>(n, dm.as<uint64_t>(), c.state.as<uint64_t>(), c.reps.as<uint64_t>(),
                                                    orow.as<int32_t>(), G.n_ops, G.n_site, G.stats,
                                                    c.perm_u8.as<uint8_t>(), c.inv_u8.as<uint8_t>(),
                                                    S.phase.as<double2>(), dchi.as<double2>(),
                                                    c.rank.dev.as<uint32_t>(), c.rank.rp, dr.as<int64_t>(),
                                                    dc.as<double2>());
  SED_CUDA(cudaGetLastError());
  SED_CUDA(cudaMemcpyAsync(rows, dr.p, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaMemcpyAsync(coeff, dc.p, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

void sector_readback(const SectorImpl& S, uint64_t* reps, int32_t* stab, int32_t* orbit) {
  const CatalogImpl& c = *S.cat;
  cudaStream_t s = c.stream;
  if (S.dim == 0) return;
  DevBuf dr((size_t)S.dim * 8), ds((size_t)S.dim * 4), dorb((size_t)S.dim * 4);
  k_sector_gather<<<grid_for(S.dim, 256), 256, 0, s>>>(S.dim, S.row_orbit.as<uint32_t>(), c.reps.as<uint64_t>(),
                                                       c.stab.as<uint8_t>(), dr.as<uint64_t>(), ds.as<int32_t>(),
                                                       dorb.as<int32_t>());
  SED_CUDA(cudaGetLastError());
  if (reps) SED_CUDA(cudaMemcpyAsync(reps, dr.p, S.dim * 8, cudaMemcpyDeviceToHost, s));
  if (stab) SED_CUDA(cudaMemcpyAsync(stab, ds.p, S.dim * 4, cudaMemcpyDeviceToHost, s));
  if (orbit) SED_CUDA(cudaMemcpyAsync(orbit, dorb.p, S.dim * 4, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

}  // namespace sed
