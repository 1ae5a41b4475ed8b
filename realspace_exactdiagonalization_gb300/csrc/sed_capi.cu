// sed_capi.cu -- extern "C" entry points of libsed_gb300.so (see include/sed_capi.h).
// Each entry point converts C++ exceptions into an int status plus a
// thread-local message, so no exception ever crosses the ABI.
#include <cstring>
#include <string>

#include "../../include/sed_capi.h"
#include "sed_handles.cuh"
#include "sed_internal.cuh"

namespace sed {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
}  // namespace sed

template <class F>
static int guarded(F&& f) {
  try {
    f();
    return SED_OK;
  } catch (const sed::Error& e) {
    sed::set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    sed::set_error("host allocation failed");
    return SED_ERR_NOMEM;
  } catch (const std::exception& e) {
    sed::set_error(e.what());
    return SED_ERR_ARG;
  }
}

#define REQ(cond, msg) SED_REQUIRE(cond, SED_ERR_ARG, msg)

extern "C" {

const char* sed_last_error(void) { return sed::g_last_error.c_str(); }
int sed_api_version(void) { return SED_API_VERSION; }

int sed_device_info(int* device, int* sm_count, int64_t* free_bytes, int64_t* total_bytes) {
  return guarded([&] {
    int d = 0;
    SED_CUDA(cudaGetDevice(&d));
    size_t fr = 0, tot = 0;
    SED_CUDA(cudaMemGetInfo(&fr, &tot));
    if (device) *device = d;
    if (sm_count) *sm_count = sed::device_sm_count();
    if (free_bytes) *free_bytes = (int64_t)fr;
    if (total_bytes) *total_bytes = (int64_t)tot;
  });
}

int sed_group_create(int n_site, int n_ops, const int32_t* perm, const double* phase_reim, int identity_idx,
                     int stats, sed_group** out) {
  return guarded([&] {
    REQ(out != nullptr, "out must not be NULL");
    *out = nullptr;
    auto g = sed::make_group(n_site, n_ops, perm, phase_reim, identity_idx, stats);
    *out = new sed_group{g};
  });
}
int sed_group_inverse(const sed_group* g, int32_t* inv_out) {
  return guarded([&] {
    REQ(g && inv_out, "NULL argument");
    std::memcpy(inv_out, g->p->inv.data(), g->p->inv.size() * 4);
  });
}
void sed_group_destroy(sed_group* g) { delete g; }

int sed_catalog_build(const sed_group* g, int n_filled, sed_catalog** out) {
  return guarded([&] {
    REQ(g && out, "NULL argument");
    *out = nullptr;
    auto c = sed::build_catalog(g->p, n_filled);
    *out = new sed_catalog{c};
  });
}
int sed_catalog_build_species(const sed_group* g, int n_split, int n_lo, int n_hi, sed_catalog** out) {
  return guarded([&] {
    REQ(g && out, "NULL argument");
    *out = nullptr;
    REQ(n_split > 0, "n_split must be positive (sed_catalog_build serves one species)");
    auto c = sed::build_catalog(g->p, n_lo + n_hi, n_split, n_lo, n_hi);
    *out = new sed_catalog{c};
  });
}
int sed_catalog_lookup(const sed_catalog* c, int64_t n, const uint64_t* masks, int32_t* rep_rank, int32_t* rep_sym,
                       double* rep_amp_reim) {
  return guarded([&] {
    REQ(c, "NULL argument");
    sed::catalog_lookup(*c->p, n, masks, rep_rank, rep_sym, rep_amp_reim);
  });
}
int sed_catalog_species(const sed_catalog* c, int* n_split, int* n_lo, int* n_hi) {
  return guarded([&] {
    REQ(c, "NULL argument");
    if (n_split) *n_split = c->p->split;
    if (n_lo) *n_lo = c->p->split > 0 ? c->p->n_lo : c->p->n_filled;
    if (n_hi) *n_hi = c->p->split > 0 ? c->p->n_hi : 0;
  });
}
int sed_catalog_info(const sed_catalog* c, int64_t* n_states, int64_t* n_orbits, int64_t* n_stab_total) {
  return guarded([&] {
    REQ(c, "NULL catalog");
    if (n_states) *n_states = c->p->n_states;
    if (n_orbits) *n_orbits = c->p->n_orbits;
    if (n_stab_total) *n_stab_total = c->p->n_stab_total;
  });
}
int sed_catalog_get(const sed_catalog* c, int field, void* out, int64_t out_bytes) {
  return guarded([&] {
    REQ(c, "NULL catalog");
    sed::catalog_readback(*c->p, field, out, out_bytes);
  });
}
int sed_catalog_update_phases(sed_catalog* c, const sed_group* g) {
  return guarded([&] {
    REQ(c && g, "NULL argument");
    sed::catalog_update_phases(*c->p, g->p);
  });
}
int sed_catalog_set_stream(sed_catalog* c, void* stream) {
  return guarded([&] {
    REQ(c, "NULL catalog");
    if (c->p->own_stream && c->p->stream) cudaStreamDestroy(c->p->stream);
    c->p->own_stream = false;
    c->p->stream = (cudaStream_t)stream;
  });
}
void sed_catalog_destroy(sed_catalog* c) { delete c; }

int sed_sector_build(const sed_catalog* c, const double* chi_reim, double atol, sed_sector** out, int64_t* dim) {
  return guarded([&] {
    REQ(c && out, "NULL argument");
    REQ(atol >= 0.0, "atol must be non-negative");
    *out = nullptr;
    auto s = sed::build_sector(c->p, chi_reim, atol);
    if (dim) *dim = s->dim;
    *out = new sed_sector{s};
  });
}
int sed_sector_build_group(const sed_catalog* c, const sed_group* g, const double* chi_reim, double atol,
                           sed_sector** out, int64_t* dim) {
  return guarded([&] {
    REQ(c && g && out, "NULL argument");
    REQ(atol >= 0.0, "atol must be non-negative");
    *out = nullptr;
    auto s = sed::build_sector(c->p, chi_reim, atol, g->p);
    if (dim) *dim = s->dim;
    *out = new sed_sector{s};
  });
}
int sed_sector_get(const sed_sector* s, uint64_t* reps, int32_t* stab_order, int32_t* orbit_index) {
  return guarded([&] {
    REQ(s, "NULL sector");
    sed::sector_readback(*s->p, reps, stab_order, orbit_index);
  });
}
int sed_sector_project(const sed_sector* s, int64_t n, const uint64_t* masks, int64_t* row_out, double* coeff_reim) {
  return guarded([&] {
    REQ(s, "NULL sector");
    sed::sector_project(*s->p, n, masks, row_out, coeff_reim);
  });
}
int sed_sector_expand_fock(const sed_sector* s, const double* c_reim, int64_t dim, double atol, double* fock_reim,
                           int64_t n_states, int is_device_ptr, double* norm2) {
  return guarded([&] {
    REQ(s, "NULL sector");
    sed::sector_expand_fock(*s->p, c_reim, dim, atol, fock_reim, n_states, is_device_ptr, norm2);
  });
}
void sed_sector_destroy(sed_sector* s) { delete s; }
int sed_position_operator(const sed_sector* to, const sed_sector* from, const double* site_phase_reim,
                          int64_t* row_to, double* elem_reim) {
  return guarded([&] {
    REQ(to && from, "NULL sector");
    sed::position_operator(*to->p, *from->p, site_phase_reim, row_to, elem_reim);
  });
}
int sed_fock_overlaps(const double* a_reim, int na, const double* b_reim, int nb, int64_t n_states, int is_device_ptr,
                      double* m_reim) {
  return guarded([&] { sed::fock_overlaps(a_reim, na, b_reim, nb, n_states, is_device_ptr, m_reim); });
}

int sed_op_create(const sed_sector* s, int n_bil, const int32_t* bil_ij, const double* bil_t_reim, int n_den,
                  const int32_t* den_ij, const double* den_v_reim, int precision, sed_op** out) {
  return guarded([&] {
    REQ(s && out, "NULL argument");
    *out = nullptr;
    auto op = sed::make_op(s->p, n_bil, bil_ij, bil_t_reim, n_den, den_ij, den_v_reim, precision);
    *out = new sed_op{op};
  });
}
int sed_terms_validate(const sed_group* g, int n_bil, const int32_t* bil_ij, const double* bil_t_reim) {
  return guarded([&] {
    REQ(g, "NULL group");
    REQ(n_bil == 0 || (bil_ij && bil_t_reim), "bilinear arrays must not be NULL");
    sed::TermTables tt;
    sed::build_term_tables(*g->p, n_bil, bil_ij, bil_t_reim, tt);
    sed::check_hermitian_symmetric(*g->p, n_bil, bil_ij, bil_t_reim);
  });
}
int sed_op_set_apply_shape(sed_op* op, int threads_per_row, int threads_per_block) {
  return guarded([&] {
    REQ(op, "NULL operator");
    sed::op_set_apply_shape(*op->p, threads_per_row, threads_per_block);
  });
}
int sed_op_apply_shape(const sed_op* op, int complex64, int* threads_per_row, int* threads_per_block) {
  return guarded([&] {
    REQ(op, "NULL operator");
    const int k = complex64 ? 1 : 0;
    if (threads_per_row) *threads_per_row = op->p->apply_tpr[k];
    if (threads_per_block) *threads_per_block = op->p->apply_block[k];
  });
}
int sed_op_apply(sed_op* op, const double* x_reim, double* y_reim, int64_t n, int is_device_ptr) {
  return guarded([&] {
    REQ(op, "NULL operator");
    sed::op_apply_host(*op->p, x_reim, y_reim, n, is_device_ptr != 0);
  });
}
int sed_op_info(const sed_op* op, int64_t* dim, int64_t* n_orbits, int64_t* hops) {
  return guarded([&] {
    REQ(op, "NULL operator");
    if (dim) *dim = op->p->sec->dim;
    if (n_orbits) *n_orbits = op->p->sec->cat->n_orbits;
    if (hops) *hops = sed::op_count_hops(*op->p);
  });
}
int sed_op_set_hop_table(sed_op* op, int mode) {
  return guarded([&] {
    REQ(op, "NULL operator");
    REQ(mode >= 0 && mode <= 2, "mode must be 0 (off), 1 (at the first solve) or 2 (now)");
    sed::OpImpl& o = *op->p;
    o.tab_mode = mode;
    o.tab_refused = false;
    if (mode == 0) sed::op_drop_table(o);
    if (mode == 2 && !o.tab_built) {
      REQ(sed::op_build_table(o), "the hop table does not fit (memory budget, field widths or twist classes)");
    }
  });
}
int sed_op_hop_table_info(const sed_op* op, int32_t* built, int64_t* records, int64_t* bytes) {
  return guarded([&] {
    REQ(op, "NULL operator");
    const sed::OpImpl& o = *op->p;
    if (built) *built = o.tab_built ? 1 : 0;
    if (records) *records = o.tab_records;
    if (bytes) *bytes = o.tab_built ? (int64_t)(o.tab_hop.bytes + o.tab_off.bytes + o.tab_w.bytes + o.tab_coef64.bytes +
                                                o.tab_coef32.bytes)
                                    : 0;
  });
}
int sed_op_set_stream(sed_op* op, void* stream) {
  return guarded([&] {
    REQ(op, "NULL operator");
    if (op->p->own_stream && op->p->stream) cudaStreamDestroy(op->p->stream);
    op->p->own_stream = false;
    op->p->stream = (cudaStream_t)stream;
  });
}
int sed_op_set_priority(sed_op* op, int high) {
  return guarded([&] {
    REQ(op, "NULL operator");
    REQ(high == 0 || high == 1, "priority must be 0 or 1");
    int least = 0, greatest = 0;
    SED_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    cudaStream_t s = nullptr;
    SED_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, high ? greatest : least));
    if (op->p->stream) {  // the new stream starts after the operator's earlier work
      const cudaError_t e = cudaStreamSynchronize(op->p->stream);
      if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        SED_CUDA(e);
      }
      if (op->p->own_stream) cudaStreamDestroy(op->p->stream);
    }
    op->p->stream = s;
    op->p->own_stream = true;
  });
}
int sed_op_set_sm_limit(sed_op* op, int n_sm) {
  return guarded([&] {
    REQ(op, "NULL operator");
    REQ(n_sm >= 0, "SM limit must be >= 0");
    op->p->sm_limit = n_sm;
  });
}
int sed_op_apply_orbit(sed_op* op, const void* xs_dev, double* y_dev) {
  return guarded([&] {
    REQ(op && xs_dev && y_dev, "NULL argument");
    sed::op_apply_orbit(*op->p, xs_dev, y_dev, op->p->stream);
  });
}
void sed_op_destroy(sed_op* op) { delete op; }

int sed_solve(sed_op* op, int nev, double tol, int maxiter, int krylovdim, uint64_t seed, double* evals,
              double* evecs_reim, sed_solve_info* info) {
  sed::SolveResult r;
  int st = guarded([&] {
    REQ(op && evals, "NULL argument");
    REQ(tol > 0.0, "tol must be positive");
    r = sed::solve(*op->p, nev, tol, maxiter, krylovdim, seed, evals, evecs_reim);
  });
  if (info) {
    info->n_restarts = r.restarts;
    info->n_matvec = r.matvecs;
    info->n_matvec_fp64 = r.matvecs64;
    info->converged = r.converged;
    info->max_residual = r.max_residual;
    info->max_delta_polish = r.max_delta;
    info->seconds = r.seconds;
  }
  if (st == SED_OK && r.status != 0) {
    sed::set_error("Lanczos did not converge the requested eigenpairs within maxiter restarts.");
    return SED_ERR_NOT_CONVERGED;
  }
  return st;
}

}  // extern "C"
