// sed_internal.cuh -- shared definitions of the GB300 sector library.
//
// Device data layout (one catalog serves every momentum and every flux twist
// that shares the same permutations):
//   state[rank]   uint64 per fixed-filling basis state, indexed by the colex
//                 rank of its mask:
//                   bits  0..31 orbit index (0xFFFFFFFF = unset)
//                   bits 32..39 g, the last (largest) group element with
//                               g(rep) = state (SRE:461-466, last write wins)
//                   bit  40     sign of the fermionic reordering of g on rep
//                   bits 41..47 stabilizer order of the orbit
//                   bits 48..55 g^-1 (the element the gather's coefficient
//                               tables are indexed by)
//   reps[orbit]   uint64 representative mask (ascending = catalog order)
//   stab[orbit]   uint8 stabilizer order
// Sector vectors on the device are indexed by catalog orbit (length n_orbits);
// entries of orbits outside the sector are exactly zero.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#define SED_MAX_SITES 63
#define SED_MAX_OPS 64
#define SED_UNSET_ORBIT 0xFFFFFFFFu

namespace sed {

// ------------------------------------------------------------------ errors
void set_error(const std::string& msg);
struct Error {
  int code;
  std::string msg;
};
#define SED_CUDA(call)                                                                              \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      throw ::sed::Error{2, std::string(#call " failed: ") + cudaGetErrorString(e_) + " at " __FILE__}; \
  } while (0)
#define SED_REQUIRE(cond, code, msg)      \
  do {                                    \
    if (!(cond)) throw ::sed::Error{code, msg}; \
  } while (0)

// ------------------------------------------------------------ device buffer
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  explicit DevBuf(size_t n) { alloc(n); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { reset(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
    return *this;
  }
  ~DevBuf() { reset(); }
  void alloc(size_t n) {
    reset();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      throw Error{3, std::string("cudaMalloc of ") + std::to_string(n) + " bytes failed: " + cudaGetErrorString(e)};
    }
    bytes = n;
  }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

template <class T>
inline void upload(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
  b.alloc(v.size() * sizeof(T));
  if (!v.empty()) SED_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

// ------------------------------------------------------------ rank tables
// Colex rank of a k-subset, sum_j binom(b_j, j+1) (SRE:231-243), evaluated
// one byte of the mask at a time: entry [c][p][v] is the contribution of byte
// value v in chunk c when p set bits lie below the chunk.  Tables hold
// uint32 (binomial(n, k) < 2^32 is a library limit) and live in shared memory.
struct RankParams {
  int nchunk;
  int total;  // entries
  int off[8];
  int pmin[8];
};

struct RankTable {
  RankParams rp{};
  std::vector<uint32_t> host;
  DevBuf dev;
};
void build_rank_table(int n_site, int split, int klo, int khi, RankTable& rt, cudaStream_t s);

// host binomial table (exact int64)
int64_t binom64(int n, int k);

// ------------------------------------------------------------------ objects
struct GroupImpl {
  int n_site = 0, n_ops = 0, identity = 0, stats = 0;
  std::vector<int32_t> perm;  // n_ops * n_site
  std::vector<double> phase;  // n_ops * n_site * 2
  std::vector<int32_t> inv;
  bool has_phases = false;    // some eta differs from exactly 1+0i
};

struct CatalogImpl {
  std::shared_ptr<GroupImpl> group;
  int n_filled = 0;
  // two conserved species (split > 0): n_lo particles on modes [0, split),
  // n_hi on [split, n_site), n_filled = n_lo + n_hi; states are ranked
  // rank_hi * binom(split, n_lo) + rank_lo (build_rank_table)
  int split = 0, n_lo = 0, n_hi = 0;
  int64_t n_states = 0, n_orbits = 0, n_stab_total = 0;
  RankTable rank;
  DevBuf state, reps, stab;            // see layout above
  DevBuf perm_u8, inv_u8, phase, binom;  // perm_u8: [n_ops][64]
  std::vector<uint8_t> stab_host;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  ~CatalogImpl();
  void upload_group_phases();
};

struct SectorImpl {
  std::shared_ptr<CatalogImpl> cat;
  // the group whose per-site phases define this sector (the catalog's group,
  // or a twisted copy with the same permutations) and its device phases
  std::shared_ptr<GroupImpl> group;
  DevBuf phase;
  std::vector<double> chi;  // n_ops * 2
  double atol = 1e-12;
  int64_t dim = 0;
  DevBuf rowflag;    // uint8[n_orbits], 1 if the orbit belongs to the sector
  DevBuf row_orbit;  // uint32[dim]
  cudaStream_t stream() const { return cat->stream; }
};

// Hop records in shared memory: for every from-site i, records
// [site_off[i], site_off[i+1]) hold (to-site | amplitude-class << 8).
struct TermTables {
  int n_site = 0, n_terms = 0, n_class = 0;
  std::vector<uint16_t> site_off;  // n_site + 1
  std::vector<uint32_t> rec;       // n_terms
  std::vector<double> amp;         // n_class * 2: distinct amplitudes t
};

// Phase classes of every group element (see sed_rowgather.cuh): mode 0 = no
// phases, 1 = class tables, 2 = per-site product.
struct PhaseClassTables {
  int mode = 0, kp1 = 1;
  std::vector<uint64_t> mask;  // [G][3]
  std::vector<double> pw;      // [G][3][k+1] complex
  std::vector<double> base_k;  // [G] complex: base^k, folded into tchi
};
void compute_phase_classes(const GroupImpl& G, int k, PhaseClassTables& pc);

struct OpImpl {
  std::shared_ptr<SectorImpl> sec;
  int precision = 0;
  TermTables terms;
  std::vector<double> diag_host;  // density terms stay on the host until upload
  std::vector<int32_t> den_ij;
  std::vector<double> den_v;
  DevBuf site_off, rec;           // term tables
  DevBuf tchi64, tchi32;          // [n_class][n_ops] conj(t_u) * chi(h)
  DevBuf cls_mask;                // [n_ops][3] phase-class masks
  PhaseClassTables pc;
  DevBuf diag;                    // double2[n_orbits] density-density diagonal
  DevBuf xs, ypad, xsec, ysec;    // work vectors for sed_op_apply
  int64_t hops = -1;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t smem_bytes = 0;
  bool tchi_in_smem = true;
  // hop table (sed_optable.cu): 0 off, 1 built at the first solve when it
  // fits the memory budget, 2 requested now
  int tab_mode = 1;
  bool tab_built = false, tab_refused = false;
  DevBuf tab_hop, tab_off, tab_w, tab_coef64, tab_coef32;
  int64_t tab_records = 0, tab_coefs = 0;
  // the gather matvec's launch shape per precision [FP64, complex64]: threads
  // per row and threads per block (0: not chosen yet; the autotuner decides)
  int apply_tpr[2] = {0, 0}, apply_block[2] = {0, 0};
  // SMs the operator's matvec and solve kernels size their grids for (0: all
  // of the device's); a server that keeps other work resident on some SMs
  // gives its device-wide solves the rest, so their one-wave grids still
  // run in one wave
  int sm_limit = 0;
  ~OpImpl();
};
int op_sm_count(const OpImpl& op);  // sm_limit, or the device's SM count
void op_set_apply_shape(OpImpl& op, int tpr, int block);
bool op_build_table(OpImpl& op);
void op_drop_table(OpImpl& op);
void apply_table(OpImpl& op, bool fp32, const void* xs, double* ypad, cudaStream_t s, bool cf_out = false);

// ----------------------------------------------------------- entry points
std::shared_ptr<GroupImpl> make_group(int n_site, int n_ops, const int32_t* perm, const double* phase, int identity,
                                      int stats);
std::shared_ptr<CatalogImpl> build_catalog(std::shared_ptr<GroupImpl> g, int n_filled, int split = 0, int n_lo = 0,
                                           int n_hi = 0);
// the mask carries the catalog's particle numbers (per species when split)
inline bool catalog_holds(const CatalogImpl& c, uint64_t m) {
  if (c.split <= 0) return __builtin_popcountll(m) == c.n_filled;
  const uint64_t lo = m & ((1ULL << c.split) - 1ULL);
  return __builtin_popcountll(lo) == c.n_lo && __builtin_popcountll(m ^ lo) == c.n_hi;
}
// bilinear terms must keep every particle in its species (SED_ERR_ARG)
void check_species_terms(const CatalogImpl& c, int n_bil, const int32_t* bil_ij);
void catalog_readback(const CatalogImpl& c, int field, void* out, int64_t out_bytes);
void catalog_lookup(const CatalogImpl& c, int64_t n, const uint64_t* masks, int32_t* rank, int32_t* sym, double* amp);
void catalog_update_phases(CatalogImpl& c, std::shared_ptr<GroupImpl> g);
std::shared_ptr<SectorImpl> build_sector(std::shared_ptr<CatalogImpl> c, const double* chi, double atol,
                                         std::shared_ptr<GroupImpl> g = nullptr);
void sector_readback(const SectorImpl& s, uint64_t* reps, int32_t* stab, int32_t* orbit);
// flux-torus observables (sed_observables.cu)
void position_operator(const SectorImpl& to, const SectorImpl& from, const double* site_phase, int64_t* row_out,
                       double* elem_out);
void fock_overlaps(const double* A, int na, const double* B, int nb, int64_t n, int is_device, double* M);
void sector_project(const SectorImpl& s, int64_t n, const uint64_t* masks, int64_t* rows, double* coeff);
void sector_expand_fock(const SectorImpl& S, const double* c, int64_t dim, double atol, double* out,
                        int64_t n_states, int is_device, double* norm2_out);
std::shared_ptr<OpImpl> make_op(std::shared_ptr<SectorImpl> s, int n_bil, const int32_t* bil_ij, const double* bil_t,
                                int n_den, const int32_t* den_ij, const double* den_v, int precision);
void build_term_tables(const GroupImpl& G, int n_bil, const int32_t* bil_ij, const double* bil_t, TermTables& tt);
void check_hermitian_symmetric(const GroupImpl& G, int n_bil, const int32_t* bil_ij, const double* bil_t);
void op_apply_host(OpImpl& op, const double* x, double* y, int64_t n, bool device_ptrs);
// y_pad (complex128, orbit-indexed) = H x given xs = sqrt(stab) * x in the op precision
void op_apply_orbit(OpImpl& op, const void* xs, double* ypad, cudaStream_t s);
// the same without the launch-shape autotuner's timing runs (no host
// synchronisation): the shape pinned or remembered for the operator's catalog
// shape, else the default
void op_apply_orbit_untuned(OpImpl& op, const void* xs, double* ypad, cudaStream_t s);
// the mixed-precision matvec streamed from the hop table with a complex64
// output; false (nothing launched) when the operator has no hop table
bool op_apply_orbit_cf(OpImpl& op, const void* xs, float2* y, cudaStream_t s);
// xs = sqrt(stab) * v (cast to the op precision); v orbit-indexed complex128
void op_scale_to_xs(OpImpl& op, const double* v, void* xs, cudaStream_t s);
int64_t op_count_hops(OpImpl& op);

struct SolveResult {
  int status = 0;
  int restarts = 0, matvecs = 0, matvecs64 = 0, converged = 0;
  double max_residual = 0, max_delta = 0, seconds = 0;
};
SolveResult solve(OpImpl& op, int nev, double tol, int maxiter, int krylovdim, uint64_t seed, double* evals,
                  double* evecs);

// diagonalize_block_matrixfree's n <= 500 branch: dense block + Hermitian eigen
SolveResult solve_dense(OpImpl& op, int nev, double* evals, double* evecs);
static constexpr int64_t kDenseMaxDim = 500;
// Mixed precision: a polished eigenvalue is accepted when its quadratic error
// bound |r|^2 / gap is below this fraction of |E| (one tenth of the 1e-9
// relative accuracy the mixed path promises).
static constexpr double kMixedRelTarget = 1e-10;

// The acceptance test of one pair (value lam, squared FP64 residual r2) of a
// mixed-precision Rayleigh-Ritz block.  The Rayleigh-Ritz step removes the
// coupling between the block's own vectors, so the quadratic bound
// |dE| <= r^2 / gap needs the distance from lam to the eigenvalues outside
// the block: gap = thL - lam, thL the lower end theta_L - r_L of the first
// Lanczos Ritz interval above the block (an eigenvalue lies within r_L of
// theta_L; theta_L alone would overestimate the gap, since Ritz values bound
// eigenvalues from above).  The pair must also be isolated, gap > 2 r, for the
// bound to apply.  A pair whose FP64 residual meets tol is accepted outright.
// Levels the complex64 run has not separated into distinct Ritz values -- a
// cluster narrower than its residuals, about 1e-6 |E| -- are invisible to any
// residual-based test; wider clusters fail the test until the Lanczos
// resolves them, or the run stagnates and the pair is solved in FP64.
__host__ __device__ inline bool mixed_pair_accepted(double lam, double r2, double thL, double tol, double scale) {
  const double r = sqrt(r2);
  if (r <= tol) return true;
  const double gap = thL - lam;
  const double e = lam < 0 ? -lam : lam;
  const double floor_e = 1e-6 * scale;
  return gap > 2.0 * r && r2 <= kMixedRelTarget * (e > floor_e ? e : floor_e) * gap;
}
// Mixed precision reorthogonalises selectively: the full pass's dot products
// are always taken (FP64-class), and the update is applied only when the
// largest of them exceeds this fraction of |w|.  Between updates the basis
// stays orthogonal to about this level, the unit roundoff of the complex64
// matvec, so the projected matrix keeps the accuracy that matvec allows
// (Simon's semi-orthogonality); the Rayleigh-Ritz check orthonormalises its
// Ritz block explicitly (Gram matrix, Cholesky).
static constexpr double kSelReorth = 1e-7;

// small dense eigen-solvers (host)
void eigh_real_sym(int n, std::vector<double>& A, std::vector<double>& w, std::vector<double>& Z);
void eigh_complex_herm(int n, const std::vector<double>& Hreim, std::vector<double>& w, std::vector<double>& Zreim);

// Per-device facts.  A process may drive several GPUs (one host thread each):
// the SM count and every kernel's shared-memory opt-in are properties of the
// current device, so both are kept per device ordinal.
static constexpr int kMaxDevices = 64;
int current_device();  // cudaGetDevice, checked against kMaxDevices
int device_sm_count(); // SM count of the current device
inline int op_sm_count(const OpImpl& op) {
  const int n = device_sm_count();
  return op.sm_limit > 0 && op.sm_limit < n ? op.sm_limit : n;
}
// One kernel's dynamic shared-memory opt-in on every device.  ensure() raises
// it to at least `bytes` on the current device and never lowers it; callers
// hold their own lock from ensure() through the launch, so a concurrent caller
// with a smaller footprint cannot undercut a launch in progress.
struct SmemOptIn {
  size_t bytes[kMaxDevices] = {};
  template <class K>
  void ensure(K* kern, size_t need) {
    size_t& cfg = bytes[current_device()];
    if (need > cfg) {
      SED_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
      cfg = need;
    }
  }
};
int grid1(int64_t work, int block);
void compute_diag(int64_t n_orb, const uint64_t* reps, const uint8_t* rowflag, int n_den, const int32_t* den_ij,
                  const double2* den_v, double2* diag, cudaStream_t s);

}  // namespace sed

// ============================================================ device helpers
namespace sed {
namespace dev {

__device__ __forceinline__ uint64_t gosper_next(uint64_t x) {
  uint64_t c = x & (0ULL - x);
  uint64_t r = x + c;
  return (((r ^ x) >> 2) >> (__ffsll((long long)x) - 1)) | r;
}

// bits of m strictly above position q (q in [0, 63])
__device__ __forceinline__ uint64_t bits_above(uint64_t m, int q) { return m & ~((2ULL << q) - 1ULL); }

// bits strictly between positions a and b
__device__ __forceinline__ uint64_t bits_between(int a, int b) {
  int lo = min(a, b), hi = max(a, b);
  return (hi - lo <= 1) ? 0ULL : (((1ULL << (hi - lo - 1)) - 1ULL) << (lo + 1));
}

__device__ __forceinline__ uint32_t rank_of(uint64_t m, const uint32_t* __restrict__ tab, const RankParams& rp) {
  uint32_t r = 0;
  int p = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    if (c < rp.nchunk) {
      const uint32_t v = (uint32_t)(m >> (8 * c)) & 0xFFu;
      r += tab[rp.off[c] + ((p - rp.pmin[c]) << 8) + v];
      p += __popc(v);
    }
  }
  return r;
}

// Permutation image of m (bit i -> bit perm[i]) and the parity of the
// fermionic reordering (SRE:146-163 counts set bits above each new position).
__device__ __forceinline__ uint64_t apply_perm(uint64_t m, const uint8_t* perm) {
  uint64_t r = 0;
  while (m) {
    const int i = __ffsll((long long)m) - 1;
    m &= m - 1;
    r |= 1ULL << perm[i];
  }
  return r;
}
__device__ __forceinline__ uint64_t apply_perm_parity(uint64_t m, const uint8_t* perm, int* parity) {
  uint64_t r = 0;
  int s = 0;
  while (m) {
    const int i = __ffsll((long long)m) - 1;
    m &= m - 1;
    const int q = perm[i];
    s ^= __popcll(bits_above(r, q));
    r |= 1ULL << q;
  }
  *parity = s & 1;
  return r;
}

// Non-fused complex product (each multiply and add separately rounded), the
// evaluation the reference's tables are reproduced with.
__device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
  return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                      __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

// Full group action with amplitude (SRE:132-163): phase product in lsb-first
// order, times the reordering sign for fermions.
__device__ __forceinline__ uint64_t apply_full(uint64_t m, const uint8_t* perm, const double2* __restrict__ phase,
                                               int fermi, double2* amp) {
  uint64_t r = 0;
  double2 ph = make_double2(1.0, 0.0);
  int s = 0;
  while (m) {
    const int i = __ffsll((long long)m) - 1;
    m &= m - 1;
    const int q = perm[i];
    if (fermi) s ^= __popcll(bits_above(r, q));
    r |= 1ULL << q;
    ph = cmul_rn(ph, phase[i]);
  }
  if (fermi) {
    const double sg = (s & 1) ? -1.0 : 1.0;
    ph = make_double2(__dmul_rn(ph.x, sg), __dmul_rn(ph.y, sg));
  }
  *amp = ph;
  return r;
}

}  // namespace dev
}  // namespace sed
