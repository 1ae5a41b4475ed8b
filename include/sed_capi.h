/*
 * sed_capi.h -- C ABI of the GB300 symmetry-sector exact-diagonalization
 * library (libsed_gb300.so).
 *
 * Drop-in for the matrix-free hot path of the Julia package
 * RealSpace_ExactDiagonalization v0.1.0 (SRE = src/symmetry_resolved_ed.jl).
 * Each entry point names the reference function it replaces.  Conventions:
 *   - plain C types only; caller-owned host buffers unless a flag says device;
 *   - sites, group elements and sector rows are 0-based here (the reference is
 *     1-based; readback fields it stores 1-based are returned 1-based);
 *   - complex numbers are interleaved (re, im) doubles;
 *   - every call returns an int status (0 = SED_OK); sed_last_error() returns
 *     the message of the last failing call on the calling thread;
 *   - one CUDA stream per object (sed_*_set_stream overrides it); calls on one
 *     object are not thread-safe, distinct objects may be used concurrently.
 * Objects hold shared references to what they were built from (an operator
 * keeps its sector, catalog and group alive), so destroy order is free.
 */
#ifndef SED_CAPI_H
#define SED_CAPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SED_API_VERSION 1

/* status codes */
#define SED_OK 0
#define SED_ERR_ARG 1           /* invalid argument (the reference asserts or errors) */
#define SED_ERR_CUDA 2          /* CUDA runtime failure */
#define SED_ERR_NOMEM 3         /* device allocation failed / over budget */
#define SED_ERR_NOT_CONVERGED 4 /* SRE:1023 "Lanczos did not converge" */
#define SED_ERR_LIMIT 5         /* size outside what the library supports */
#define SED_ERR_NOT_HERMITIAN 6 /* term list not Hermitian-closed or not group-symmetric */
#define SED_ERR_TIMEOUT 7       /* a bounded device wait gave up */

#define SED_BOSONIC 0
#define SED_FERMIONIC 1

/* operator precision */
#define SED_PREC_FP64 0  /* complex128 matvec: the plain drop-in */
#define SED_PREC_MIXED 1 /* complex64 matvec, FP64 Lanczos + FP64 Rayleigh-Ritz polish */

/* catalog readback fields (SRE:305-327 Symmetry_Orbit_Catalog) */
#define SED_FIELD_REPS 0       /* uint64[n_orbits]   representative_mask_list */
#define SED_FIELD_STAB_ORDER 1 /* int32[n_orbits]    stabilizer_order_list */
#define SED_FIELD_STAB_PTR 2   /* int64[n_orbits+1]  CSR offsets of the stabilizer lists */
#define SED_FIELD_STAB_G 3     /* int32[n_stab]      stabilizer_g_indices_list (1-based) */
#define SED_FIELD_STAB_PHASE 4 /* f64x2[n_stab]      stabilizer_phases_list */
#define SED_FIELD_REP_RANK 5   /* int32[n_states]    rep_rank_table (1-based, 0 unset) */
#define SED_FIELD_REP_SYM 6    /* int32[n_states]    rep_sym_table (1-based) */
#define SED_FIELD_REP_AMP 7    /* f64x2[n_states]    rep_amp_table */

typedef struct sed_group sed_group;
typedef struct sed_catalog sed_catalog;
typedef struct sed_sector sed_sector;
typedef struct sed_op sed_op;

typedef struct sed_solve_info {
  int32_t n_restarts;      /* outer (thick-restart) iterations */
  int32_t n_matvec;        /* sector matvecs in the working precision */
  int32_t n_matvec_fp64;   /* FP64 matvecs of the polish step (mixed precision) */
  int32_t converged;       /* number of converged eigenpairs */
  double max_residual;     /* largest Ritz residual of the returned pairs */
  double max_delta_polish; /* max |E_polished - E_working| (mixed precision), else 0 */
  double seconds;          /* wall time of the solve */
} sed_solve_info;

/* ---------------------------------------------------------------- library */
const char* sed_last_error(void);
int sed_api_version(void);
/* Current device, its SM count and free/total memory (bytes). */
int sed_device_info(int* device, int* sm_count, int64_t* free_bytes, int64_t* total_bytes);

/* ------------------------------------------------------------------ group */
/* Finite_Symmetry_Group (SRE:90-104) with _inverse_operation_indices
 * (SRE:109-117).  perm: n_ops x n_site 0-based targets (perm[g*n_site+i] is
 * the image of site i); phase_reim: n_ops x n_site complex eta_g(i);
 * stats: SED_BOSONIC / SED_FERMIONIC.  Limits: n_site <= 63, n_ops <= 64. */
int sed_group_create(int n_site, int n_ops, const int32_t* perm, const double* phase_reim, int identity_idx,
                     int stats, sed_group** out);
/* 0-based inverse element of every operation. */
int sed_group_inverse(const sed_group* g, int32_t* inv_out);
void sed_group_destroy(sed_group* g);

/* ---------------------------------------------------------------- catalog */
/* build_symmetry_orbit_catalog (SRE:371-487), built on the device:
 * combinadic unranking in place of the serial Gosper loop, canonical test
 * over |G| permutations held in shared memory, orbit expansion into the
 * representative tables.  Limit: binomial(n_site, n_filled) < 2^32. */
int sed_catalog_build(const sed_group* g, int n_filled, sed_catalog** out);
/* The same catalog restricted to two separately conserved species (no
 * counterpart in the reference, which fixes only the total particle number,
 * SRE:1460-1466): n_lo particles on modes [0, n_split) and n_hi on
 * [n_split, n_site), e.g. spin-up at bit i and spin-down at bit i + n_site/2 of
 * a Hubbard model (benchmark/benchmark.jl:155-219) in one S^z sector.  Every
 * group element must map each species onto itself, and operators built on it
 * may not move particles between species (SED_ERR_ARG).  The basis states are
 * ranked rank_hi(m >> n_split) * binomial(n_split, n_lo) + rank_lo(low bits),
 * which is ascending-mask order, so the representatives, stabilizers and
 * rep_sym/rep_amp tables equal the total-particle catalog's entries for the
 * masks of this block, in the same order; REP_RANK numbers the orbits of the
 * block.  Limit: binomial(n_split, n_lo) * binomial(n_site - n_split, n_hi)
 * < 2^32. */
int sed_catalog_build_species(const sed_group* g, int n_split, int n_lo, int n_hi, sed_catalog** out);
/* n_split (0 for a one-species catalog) and the particle numbers of each
 * species (n_lo = n_filled and n_hi = 0 for one species). */
int sed_catalog_species(const sed_catalog* c, int* n_split, int* n_lo, int* n_hi);
int sed_catalog_info(const sed_catalog* c, int64_t* n_states, int64_t* n_orbits, int64_t* n_stab_total);
/* Read one table back to the host in the reference's layout (bit-exact). */
int sed_catalog_get(const sed_catalog* c, int field, void* out, int64_t out_bytes);
/* The three per-state tables of SED_FIELD_REP_RANK / REP_SYM / REP_AMP
 * (SRE:305-327, in the same 1-based layout) at n given masks, each holding the
 * catalog's particle number(s): the readback for catalogs whose tables are too
 * large to copy whole (SRE:584-594 get_canonical reads the same entries). */
int sed_catalog_lookup(const sed_catalog* c, int64_t n, const uint64_t* masks, int32_t* rep_rank, int32_t* rep_sym,
                       double* rep_amp_reim);
/* update_orbit_stabilizer_phases! (SRE:338-369): same permutations, new
 * per-site phases (a flux-twisted group); no re-enumeration. */
int sed_catalog_update_phases(sed_catalog* c, const sed_group* new_group);
int sed_catalog_set_stream(sed_catalog* c, void* cuda_stream);
void sed_catalog_destroy(sed_catalog* c);

/* ----------------------------------------------------------------- sector */
/* build_symmetry_sector_basis (SRE:534-556): orbits whose stabilizer phases
 * match chi (|chi(h) - alpha_h(rep)| <= atol), in catalog order. */
int sed_sector_build(const sed_catalog* c, const double* chi_reim, double atol, sed_sector** out, int64_t* dim);
/* The same with an explicit group g (same permutations and statistics as the
 * catalog's, e.g. the flux-twisted group of build_translation_group): the
 * sector and every operator built on it use g's phases, and the catalog is
 * left unchanged.  Equivalent to update_orbit_stabilizer_phases! (SRE:338-369)
 * followed by build_symmetry_sector_basis, without mutating the catalog, so
 * sectors of different twists can be built and solved concurrently. */
int sed_sector_build_group(const sed_catalog* c, const sed_group* g, const double* chi_reim, double atol,
                           sed_sector** out, int64_t* dim);
/* representative_mask_list, stabilizer_order_list and the catalog orbit index
 * of every sector row (any pointer may be NULL). */
int sed_sector_get(const sed_sector* s, uint64_t* reps, int32_t* stab_order, int32_t* orbit_index);
/* project_to_sector (SRE:627-632) for n masks with the catalog's filling:
 * row_out[i] = 0-based sector row of the orbit of masks[i] (-1 when the
 * orbit is not in the sector), coeff_out[i] = rep_amp * conj(chi(rep_sym)),
 * bit-exact with the reference's evaluation order. */
int sed_sector_project(const sed_sector* s, int64_t n, const uint64_t* masks, int64_t* row_out, double* coeff_reim);
/* _expand_sector_state_to_fock_amplitudes (observables/entanglement_spectrum.jl:46-79):
 * the sector vector c (dim complex128 in sector row order) spread over the
 * fixed-filling Fock states, amplitudes of one mask summed over the group
 * elements that reach it, |amp| <= atol dropped and the rest normalised.
 * fock_reim receives n_states (= the catalog's state count) complex128 in
 * colex-rank order, i.e. the r-th k-subset in ascending mask order; dropped
 * states are 0.  is_device_ptr: c and fock are device pointers.  norm2
 * (nullable) receives the squared norm before normalisation.  Fails with the
 * reference's "Expanded state has near-zero norm." */
int sed_sector_expand_fock(const sed_sector* s, const double* c_reim, int64_t dim, double atol, double* fock_reim,
                           int64_t n_states, int is_device_ptr, double* norm2);
void sed_sector_destroy(sed_sector* s);

/* ------------------------------------------------- flux-torus observables */
/* _position_operator_matrix (observables/charge_pump.jl:47-91): Resta's
 * position operator U_d = exp(2 pi i X_d / L_d), given by its per-site phases
 * site_phase_reim[n_site] (many_body_position_phases, charge_pump.jl:17-33),
 * projected from sector `from` to sector `to` of the same catalog and group.
 * U_d maps every orbit to itself, so column c of the (dim_to x dim_from)
 * matrix has one entry: row_to[c] (0-based, -1 when the representative is
 * not in `to` or the entry is below the reference's 1e-13 cut) with value
 * elem_reim[c] = (1/|G|) sum_g chi_to(g) conj(chi_from(g)) prod_{j in g(rep)}
 * phase_j.  Host output buffers of length dim_from. */
int sed_position_operator(const sed_sector* to, const sed_sector* from, const double* site_phase_reim,
                          int64_t* row_to, double* elem_reim);
/* _subspace_overlap_matrix / _fock_amplitude_overlap
 * (observables/many_body_chern_number.jl:46-71): m_reim[i * nb + j] =
 * <a_i|b_j> = sum_s conj(a_i[s]) b_j[s] for na + nb dense Fock-amplitude
 * vectors of n_states complex entries each (the layout of
 * sed_sector_expand_fock, rows contiguous).  With is_device_ptr the inputs
 * are device memory; m_reim is always host memory. */
int sed_fock_overlaps(const double* a_reim, int na, const double* b_reim, int nb, int64_t n_states, int is_device_ptr,
                      double* m_reim);

/* --------------------------------------------------------------- operator */
/* MatrixFreeHamiltonian (SRE:767-791) / hamiltonian_linear_operator
 * (SRE:891-897).  Bilinear term t moves a particle from site bil_ij[2k] to
 * site bil_ij[2k+1] (the reference's gate (m & hop) == from, SRE:709-710);
 * density term v counts n_i n_j.  The term list must be Hermitian-closed and
 * invariant under the group (SED_ERR_NOT_HERMITIAN otherwise): the device
 * kernel gathers rows through H_rc = conj(H_cr).  precision: SED_PREC_*. */
int sed_op_create(const sed_sector* s, int n_bil, const int32_t* bil_ij, const double* bil_t_reim, int n_den,
                  const int32_t* den_ij, const double* den_v_reim, int precision, sed_op** out);
/* Host-only validation of a bilinear term list against a group (no device
 * work): the checks sed_op_create applies before building an operator. */
int sed_terms_validate(const sed_group* g, int n_bil, const int32_t* bil_ij, const double* bil_t_reim);
/* apply_hamiltonian! (SRE:804-878) / H(x) (SRE:880-884): y = H x for
 * sector-ordered complex128 vectors of length n == sector dim.  With
 * is_device_ptr the pointers are device memory on this op's stream; the call
 * is then asynchronous. */
int sed_op_apply(sed_op* op, const double* x_reim, double* y_reim, int64_t n, int is_device_ptr);
/* Launch shape of the matrix-free gather (no reference counterpart): threads
 * per row (1, 2, 4 or 8 lanes of a warp split a row's hops) and threads per
 * block (256 or 512).  By default an autotuner times all eight shapes on an
 * operator's first gather matvec, per precision, and keeps the fastest,
 * remembered per catalog shape for the process; the environment variable
 * SED_APPLY_SHAPE="tpr,block" pins one.  sed_op_set_apply_shape pins a shape
 * for this operator ((0, 0) lets the autotuner choose again);
 * sed_op_apply_shape reports the shape in use (0, 0 before the first gather).
 * The shape changes results only through the order of a row's sum. */
int sed_op_set_apply_shape(sed_op* op, int threads_per_row, int threads_per_block);
int sed_op_apply_shape(const sed_op* op, int complex64, int* threads_per_row, int* threads_per_block);
/* dim = sector dimension, n_orbits = length of the orbit-indexed device
 * vectors, hops = valid hops one matvec evaluates (counted on the device). */
int sed_op_info(const sed_op* op, int64_t* dim, int64_t* n_orbits, int64_t* hops);
/* The operator's hop table: the sector matvec stored as 8 bytes per hop
 * (column orbit + coefficient index, SELL-32 slices), the compressed form of
 * the reference's projection table (build_matrixfree_projection_table,
 * SRE:680-728, streamed by _apply_table!, SRE:731-765).  mode 1 (default)
 * builds it at the first sed_solve when it fits 35 % of the free device memory;
 * 2 builds it now (SED_ERR_ARG when it cannot: memory budget, field widths, or
 * a twist whose phases take more than four values per group element); 0 drops
 * it and keeps the on-the-fly gather.  Every later sed_op_apply / sed_solve
 * uses it; results agree with the on-the-fly gather to rounding. */
int sed_op_set_hop_table(sed_op* op, int mode);
int sed_op_hop_table_info(const sed_op* op, int32_t* built, int64_t* records, int64_t* bytes);
int sed_op_set_stream(sed_op* op, void* cuda_stream);
/* Scheduling priority of the operator's own stream (no counterpart in the
 * reference, which runs one sector at a time): 1 = the device's greatest
 * stream priority, 0 = its least (the default).  The operator gets a new
 * stream of that priority, ordered after its previous work; when several
 * solves share the GPU, the kernels of a high-priority solve are scheduled
 * before the queued kernels of low-priority ones.  Replaces a stream set by
 * sed_op_set_stream. */
int sed_op_set_priority(sed_op* op, int high);
/* SM budget of the operator's kernels (no counterpart in the reference):
 * the matvec, the Lanczos vector kernels and the solve size their grids for
 * n_sm SMs instead of the whole device (0: the whole device, the default).
 * A server that keeps other kernels resident on some SMs (the persistent
 * batch) gives its device-wide solves the rest, so their one-wave grids still
 * complete in one wave.  Results do not change. */
int sed_op_set_sm_limit(sed_op* op, int n_sm);
/* Orbit-indexed matvec for benchmarking the kernel alone: xs_dev holds
 * sqrt(stab)*x in the op's precision (complex64 or complex128, length
 * n_orbits), y_dev receives complex128 H x (length n_orbits).  Asynchronous. */
int sed_op_apply_orbit(sed_op* op, const void* xs_dev, double* y_dev);
/* y = H x for device vectors (sector order, complex128, length n == sector
 * dim), allocating nothing: no counterpart in the reference.  For callers that
 * may not call cudaMalloc while they work (a host whose memory pool owns the
 * device memory, a serving loop that cannot afford cudaMalloc's implicit
 * device-wide synchronisation, code with a fixed memory budget after set-up).
 * Its work vectors live in a fixed 32 MiB device array inside this library,
 * which every GPU that loads it keeps until exit; sectors whose catalog has
 * more than 1048576 orbits are rejected with SED_ERR_LIMIT.  The first call on
 * a device looks up that array's device address; make it before any stream
 * capture.  The call never runs the gather's launch-shape autotuner: it uses
 * the operator's chosen or pinned shape, else the one remembered for the same
 * catalog shape, else one thread per row and 512 threads per block.  All
 * calls share the array, so calls that overlap on the GPU race: serialise
 * them.  Asynchronous on the operator's stream. */
int sed_op_apply_noalloc(sed_op* op, const double* x_dev, double* y_dev, int64_t n);
void sed_op_destroy(sed_op* op);

/* -------------------------------------------------------------------- solve */
/* diagonalize_block_matrixfree (SRE:998-1030): lowest nev eigenpairs.
 * Sectors of dimension <= 500 take the reference's dense branch (every
 * column from a device FP64 matvec, then a Hermitian eigensolve on the host);
 * larger ones a thick-restart Lanczos with full reorthogonalisation on the
 * device.  tol is the absolute Ritz-residual bound (the reference passes
 * 1e-10), maxiter the restart budget (300), krylovdim the basis size (0 = 30).
 * seed selects the complex Gaussian start vector.  evecs_reim (nullable)
 * receives nev sector-ordered complex128 vectors, vector-major.
 * Mixed-precision operators (SED_PREC_MIXED) run the Lanczos with complex64
 * vectors and matvec until the Ritz estimates of the requested pairs fall
 * below 1e-6 |E|, carrying two spare Ritz pairs; then one Rayleigh-Ritz step
 * with FP64 matvecs over those nev + 2 Ritz vectors, orthonormalised through
 * their Gram matrix, gives the eigenvalues and their FP64 residuals r.  A pair
 * is accepted when r <= tol, or when it is isolated (gap > 2 r) and
 * r^2 / gap <= 1e-10 |E|, gap being its distance to the lower end (Ritz value
 * minus its residual) of the first Lanczos Ritz interval above the block;
 * otherwise the Lanczos resumes with a 10x tighter threshold.  A run that
 * stagnates at the complex64 noise floor is solved again entirely in FP64.
 * Levels closer together than the complex64 run's residuals (about 1e-6 |E|)
 * that it never separates into distinct Ritz values cannot be told apart by
 * any residual test: such a cluster comes back as one level inside it (error
 * at most its width); request SED_PREC_FP64 for spectra with such clusters.
 * The first gather matvec of an operator (when it has no hop table) times
 * eight launch shapes and waits on the host for them; later solves of the same
 * catalog shape reuse the choice (see sed_op_set_apply_shape).  Mixed solves of
 * sectors with 2^18 orbits or more stage their dot products through shared
 * memory with bulk copies, under bounded waits: a wait that runs out makes the
 * call return SED_ERR_TIMEOUT rather than a result. */
int sed_solve(sed_op* op, int nev, double tol, int maxiter, int krylovdim, uint64_t seed, double* evals,
              double* evecs_reim, sed_solve_info* info);

/* ---------------------------------------------------------- batched solves */
/* Many small sector solves sharing one catalog (one set of permutations and
 * one (i, j) term list), run by a persistent kernel: every thread block takes
 * the next request from a device-side queue and runs a whole thick-restart
 * Lanczos for it, with the sector vector in shared memory.  This replaces the
 * reference's sequential per-sector / per-twist loop (SRE:1227-1254,
 * SRE:1320-1355).  Request b brings its own momentum chi (n_ops complex), its
 * group phases (n_ops x n_site complex: the flux-twisted group of
 * build_translation_group, SRE:1374-1405), its bilinear amplitudes (n_bil
 * complex, same (i, j) list for every request) and its start-vector seed, so
 * its result does not depend on which other requests share the launch.
 * precision: SED_PREC_MIXED or SED_PREC_FP64.  The mixed kernel follows the
 * mixed sed_solve (complex64 Lanczos to 1e-6 |E|, then one FP64-class
 * Rayleigh-Ritz step over the nev + 2 Ritz vectors, orthonormalised through
 * their Gram matrix, with the same acceptance test, else continued); a
 * request that stagnates at the complex64 noise floor is re-solved by the
 * FP64 kernel in a second launch.  Outputs per request: nev
 * eigenvalues (ascending), status (0 ok, SED_ERR_NOT_CONVERGED), sector
 * dimension, |E_polished - E_c64| and the matvec count.  The batch runs
 * Lanczos at every sector size (no dense branch for dimensions <= 500, unlike
 * sed_solve), so like the reference's KrylovKit branch it may list an exactly
 * degenerate level fewer times than its multiplicity; solve a small sector
 * with sed_solve to get every copy. */
typedef struct sed_batch sed_batch;
/* krylovdim: the Lanczos basis size (0: chosen by the autotuner, see
 * sed_batch_set_shape). */
int sed_batch_create(const sed_catalog* c, int n_bil, const int32_t* bil_ij, int n_den, const int32_t* den_ij,
                     const double* den_v_reim, int precision, int nev, int krylovdim, int max_requests,
                     sed_batch** out);
int sed_batch_run(sed_batch* b, int n_req, const double* chi_reim, const double* group_phase_reim,
                  const double* bil_t_reim, const uint64_t* seeds, double tol, int maxiter, double* evals,
                  int32_t* status, int64_t* dims, double* delta_polish, int32_t* n_matvec);
/* The same run returning eigenvectors as well (the (vals, vecs) layout of
 * ed_scan_at_irrep_matrixfree!, SRE:1124, per request): evecs_reim receives
 * n_req x nev complex128 vectors, vector i of request b at
 * evecs_reim[2 * ((b * nev + i) * ld + row)], row < dims[b] in the sector's
 * row order (ascending representative, as sed_sector_build_group orders the
 * sector of that request's momentum and group).  ld >= the catalog's orbit
 * count; entries at rows >= dims[b] are not written.  Each vector is in the
 * gauge of the request's own group (the site gauge of sed_batch_set_site_gauge
 * is undone).  The device variant takes device buffers. */
int sed_batch_run_vectors(sed_batch* b, int n_req, const double* chi_reim, const double* group_phase_reim,
                          const double* bil_t_reim, const uint64_t* seeds, double tol, int maxiter, double* evals,
                          int32_t* status, int64_t* dims, double* delta_polish, int32_t* n_matvec,
                          double* evecs_reim, int64_t ld);
int sed_batch_run_device_vectors(sed_batch* b, int n_req, const double* d_chi, const double* d_group_phase,
                                 const double* d_bil_t, const uint64_t* d_seeds, double tol, int maxiter,
                                 double* d_evals, int32_t* d_status, int64_t* d_dims, double* d_delta,
                                 int32_t* d_n_matvec, double* d_evecs, int64_t ld);
/* Per-request diagnostics of the last run (host buffers of n_req entries, any
 * may be NULL): hops evaluated by one matvec of the request's sector, and the
 * device clock (ns) when its block picked it up and when it finished. */
int sed_batch_last_stats(const sed_batch* b, int64_t* hops, int64_t* t_start_ns, int64_t* t_end_ns);
/* About the last run (any pointer may be NULL): how many requests the FP64
 * kernel re-solved because the complex64 run could not meet the mixed
 * precision target (0 for SED_PREC_FP64), whether the matvecs streamed the hop
 * table, and its size in 8-byte records. */
int sed_batch_last_info(const sed_batch* b, int32_t* n_fallback, int32_t* hop_table, int64_t* hop_records);
/* The batch launch (request-queue reset + persistent kernel) is a CUDA graph,
 * captured once per launch configuration and replayed while it repeats:
 * how many captures and replays this batch object has made. */
int sed_batch_graph_info(const sed_batch* b, int32_t* captures, int32_t* replays);
/* Where the mixed kernel keeps its complex64 matvec input: shared memory (the
 * default whenever it fits beside the tables) or global memory (the choice
 * for sectors too large for it; 0 forces it, e.g. to compare the two). */
int sed_batch_set_x_in_shared_memory(sed_batch* b, int enable);
/* The hop table (on by default): the requests of a batch share the catalog and
 * the (i, j) term list, hence every sector matrix's sparsity pattern, which is
 * enumerated once into 8-byte records (column orbit, term x group element,
 * phase id) and streamed by every matvec of every request, in place of
 * re-deriving each hop from the representative (rank lookups, state words,
 * popcounts).  Costs 8 bytes per hop of device memory; rebuilt when a run's
 * twist-phase classes differ from the last run's.  Runs whose group phases take
 * more than four distinct values per group element, or whose sectors leave no
 * shared memory for its coefficient tables, use the on-the-fly matvec.  The
 * records of each row are reordered so that a warp's shared-memory gathers
 * fall into different bank groups; SED_BATCH_BANK_ORDER=0 in the environment
 * keeps them in enumeration order (only the rounding of each row's sum
 * differs). */
int sed_batch_set_hop_table(sed_batch* b, int enable);
/* Launch shape of the batched solve (no counterpart in the reference): the
 * threads per row of the hop-table matvec (1, or 2 lanes splitting a row's
 * records) and the Krylov dimension of the thick-restart Lanczos.  By default
 * an autotuner times the candidates -- threads per row 1 and 2, and Krylov
 * dimensions 24, 20 and 28 when sed_batch_create got krylovdim 0 (else that
 * one) -- on one wave of the first run's requests per catalog shape, scoring
 * each by its mean request time from the kernel's per-request device clocks
 * (best of two trials; that run waits on the host), and keeps the fastest for
 * the process.  SED_BATCH_SHAPE="krylovdim,threads_per_row"
 * in the environment or sed_batch_set_shape pins a shape ((0, 0) returns to
 * the autotuner; krylovdim at most 28 or the one given at creation).
 * sed_batch_shape reports the shape of the last run and how many autotuner
 * sweeps this batch object ran.  The shape changes results only within the
 * solver's tolerance. */
int sed_batch_set_shape(sed_batch* b, int krylovdim, int threads_per_row);
int sed_batch_shape(const sed_batch* b, int32_t* krylovdim, int32_t* threads_per_row, int32_t* tune_runs);
/* Site gauge (on by default; no counterpart in the reference).  When every
 * request of a run has a site gauge w -- per-site phases under which its
 * group's phases all become 1, as the flux-twisted translation groups of
 * build_translation_group (SRE:1374-1405) do with w_j = exp(2 pi i theta .
 * r_j / L) -- the run solves W H W^-1 (the twist spread evenly over the
 * bonds; same sector, same eigenvalues): the hop table then carries only the
 * sign of each hop and a matvec gathers one coefficient per hop instead of
 * two.  Otherwise the run uses phase-class records.  sed_batch_last_gauge
 * reports which the last run used. */
int sed_batch_set_site_gauge(sed_batch* b, int enable);
int sed_batch_last_gauge(const sed_batch* b, int32_t* gauge);
/* Same solve with every buffer in device memory (inputs resident in HBM),
 * queued on the batch stream.  Device arrays have the layouts of
 * sed_batch_run; outputs may not be NULL.  SED_PREC_FP64 returns without
 * waiting; SED_PREC_MIXED waits once for the statuses of the first launch to
 * queue the FP64 re-solves. */
int sed_batch_run_device(sed_batch* b, int n_req, const double* d_chi, const double* d_group_phase,
                         const double* d_bil_t, const uint64_t* d_seeds, double tol, int maxiter, double* d_evals,
                         int32_t* d_status, int64_t* d_dims, double* d_delta, int32_t* d_n_matvec);
int sed_batch_set_stream(sed_batch* b, void* cuda_stream);
/* Dynamic shared memory per block, resident blocks (= concurrent requests)
 * and device bytes held by the batch object. */
int sed_batch_info(const sed_batch* b, int64_t* smem_bytes, int64_t* n_blocks, int64_t* footprint_bytes);
void sed_batch_destroy(sed_batch* b);

/* Device-resident request loop (no counterpart in the reference): one
 * persistent launch of the batched kernel on n_blocks SMs whose blocks claim
 * requests from a ring of `capacity` slots as the host publishes them, so a
 * request starts as soon as a block is free, with no launch per batch.  The
 * host copies a request's inputs (the layouts of sed_batch_run, one request)
 * into a slot and then publishes it in mapped memory; a block claims it by
 * compare-and-swap on the ring's head and leaves its outputs and a done flag
 * in mapped memory.  Every wait is bounded: a block that finds nothing to do
 * for idle_ms leaves, and the next submit or wait relaunches.  The ring uses
 * the site-gauge hop table, so every request's group must have a site gauge
 * (flux-twisted translation groups do; SED_ERR_ARG otherwise); a request
 * whose mixed-precision check failed is re-solved in FP64 when collected.
 * While the ring runs, sed_batch_run on the same object is refused.  Unlike
 * the other calls on one object, the ring calls are thread-safe among
 * themselves: one thread may submit while others wait and another stops the
 * ring (a wait then fails with "the ring was stopped"); a ticket is collected
 * once, by whichever wait gets it first. */
int sed_batch_ring_start(sed_batch* b, int capacity, int n_blocks, int idle_ms);
/* SED_ERR_LIMIT when every slot holds a request not yet collected. */
int sed_batch_ring_submit(sed_batch* b, const double* chi_reim, const double* group_phase_reim,
                          const double* bil_t_reim, uint64_t seed, int64_t* ticket);
/* Wait up to timeout_ms (0: poll): nev eigenvalues, the request's status and
 * sector dimension, and the slot is released; SED_ERR_TIMEOUT when the
 * request has not finished yet. */
int sed_batch_ring_wait(sed_batch* b, int64_t ticket, int timeout_ms, double* evals, int32_t* status, int64_t* dim);
/* Launches so far, blocks per launch, and whether blocks are resident now. */
int sed_batch_ring_info(const sed_batch* b, int64_t* launches, int32_t* n_blocks, int32_t* running);
/* Stop the loop (blocks leave within one idle wait or at the end of their
 * current request) and release the ring. */
int sed_batch_ring_stop(sed_batch* b);

/* ---------------------------------------------------------------- serving */
/* Continuous-batching server on the current device (no counterpart in the
 * reference, whose per-sector loops -- _ed_scan_sectors!, SRE:1199-1256, and
 * ed_scan!, SRE:1320-1355 -- answer one sector solve at a time).  Host threads
 * drive the library's own objects: families whose catalog has at most
 * small_max_orbits orbits are answered by batch_lanes persistent batched
 * solves (sed_batch_run) taking turns, the others by up to large_workers
 * concurrent device-wide solves (sed_solve), each admitted while the device
 * memory reserved by the solves in flight plus its own footprint stays within
 * budget_bytes.  A request's result depends only on its own inputs and seed,
 * not on the mix it is served in.  precision: SED_PREC_*; tol as sed_solve. */
typedef struct sed_server sed_server;
int sed_server_create(double budget_bytes, int batch_lanes, int large_workers, int64_t small_max_orbits,
                      int precision, double tol, sed_server** out);
/* Register a model family before the first request: its catalog (the server
 * keeps a reference), its bilinear (i, j) pairs with their default (untwisted)
 * amplitudes, its density terms and the most eigenvalues a request may ask
 * for (1..6).  A batched family's lanes are warmed up here on its untwisted
 * zero-momentum sector (hop tables built, launch shape chosen), so no request
 * waits for that.  Returns the family id. */
int sed_server_add_family(sed_server* s, const sed_catalog* c, int n_bil, const int32_t* bil_ij,
                          const double* bil_t_reim, int n_den, const int32_t* den_ij, const double* den_v_reim,
                          int nev_max, int32_t* family);
/* Submit one sector solve: the momentum characters chi (n_ops complex), the
 * group phases (n_ops x n_site complex: the flux-twisted group of
 * build_translation_group, SRE:1374-1405), the bilinear amplitudes (n_bil
 * complex, in the family's pair order), the start-vector seed and nev.  The
 * inputs are copied; returns a ticket. */
int sed_server_submit(sed_server* s, int32_t family, const double* chi_reim, const double* group_phase_reim,
                      const double* bil_t_reim, uint64_t seed, int nev, int64_t* ticket);
/* Wait up to timeout_ms (0: poll) for a ticket.  When it has finished: its
 * nev eigenvalues (ascending; NaN beyond the sector dimension), the request's
 * own status (0, or the error code of its solve, whose message sed_last_error
 * then returns) and its sector dimension, and the ticket is released.
 * SED_ERR_TIMEOUT when it has not finished yet. */
int sed_server_wait(sed_server* s, int64_t ticket, int timeout_ms, double* evals, int32_t* status, int64_t* dim);
/* The next request to finish, in completion order (any ticket not yet
 * collected): its ticket and outputs as sed_server_wait, which releases it.
 * evals must hold the largest nev submitted.  SED_ERR_TIMEOUT when none
 * finishes within timeout_ms. */
int sed_server_next(sed_server* s, int timeout_ms, int64_t* ticket, double* evals, int32_t* status, int64_t* dim);
/* Requests finished and waiting, the peak device memory reserved by the
 * device-wide solves, and the resident catalogs and batch workspaces. */
int sed_server_stats(const sed_server* s, int64_t* n_done, int64_t* n_pending, double* peak_reserved_bytes,
                     double* resident_bytes);
/* Stop accepting requests, finish the ones queued, join the threads. */
void sed_server_destroy(sed_server* s);

#ifdef __cplusplus
}
#endif

#endif /* SED_CAPI_H */
