// sed_server.cu -- continuous-batching server behind the C ABI (sed_server_*
// in include/sed_capi.h).
//
// The reference answers a stream of sector solves one at a time: the loops of
// _ed_scan_sectors! (src/symmetry_resolved_ed.jl:1199-1256) and ed_scan!
// (:1320-1355) call ed_scan_at_irrep_matrixfree! (:1092-1128) per sector.  The
// server keeps the GPU busy with many requests at once, on host threads that
// drive the library's own objects:
//   - every model family has one resident catalog; a request brings only its
//     momentum characters, its (flux-twisted) group phases, its bilinear
//     amplitudes and its seed;
//   - families whose catalog has at most small_max_orbits orbits go to batch
//     lanes: persistent batched solves (sed_batch_run), several lanes taking
//     turns, so requests that arrive during a launch start in the next one;
//   - the other families go to device-wide solves (sed_solve), several at
//     once on their own streams, each admitted while the reserved device
//     memory of the solves in flight plus its own footprint stays within the
//     budget;
// A request's result depends only on its own inputs and seed.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sed_capi.h"
#include "sed_handles.cuh"
#include "sed_internal.cuh"

namespace {

struct Family {
  sed_catalog* cat = nullptr;  // the server's own reference
  int n_site = 0, n_ops = 0, identity = 0, stats = 0;
  std::vector<int32_t> perm;  // the catalog group's permutations
  std::vector<int32_t> bil_ij, den_ij;
  std::vector<double> den_v;
  int n_bil = 0, n_den = 0, nev_max = 1;
  int64_t n_orbits = 0;
  bool batched = false;
  std::vector<sed_batch*> lanes;  // batched families: one batch object per lane
};

struct Request {
  int64_t ticket = 0;
  int family = 0, nev = 1;
  uint64_t seed = 0;
  std::vector<double> chi, phase, amp;
  // result
  bool done = false;
  int status = 0;
  int64_t dim = -1;
  std::vector<double> evals;
  std::string error;
};

// device bytes one device-wide mixed solve holds: complex64 Lanczos basis,
// restart buffer and work vector (8 B per element, padded to 64 elements), the
// FP64 polish block and matvec inputs (16 B per element), the operator's
// per-orbit tables
int64_t solve_footprint(int64_t n_orbits, int nev) {
  const int64_t nw = nev + 2, m = std::max<int64_t>(30, 2 * nw + 1);
  const int64_t slots8 = 2 * std::max(m + 1, 3 * nw + 1) + 1, slots16 = 5 * nw + 2;
  const int64_t padded = (n_orbits + 63) / 64 * 64;
  return slots8 * padded * 8 + slots16 * padded * 16 + n_orbits * 17 + (64LL << 20);
}

}  // namespace

struct sed_server {
  int device = 0;
  double budget = 0, resident = 0, reserved = 0, peak_reserved = 0;
  int n_lanes = 2, n_workers = 3, precision = SED_PREC_MIXED, max_batch = 512;
  int64_t small_max_orbits = 16384, priority_max_orbits = 2000000;
  double tol = 1e-10;
  std::vector<Family> families;
  std::mutex mu;
  std::condition_variable cv;       // work arrived / closing / memory released
  std::condition_variable done_cv;  // a request finished
  std::deque<Request*> pending_batch, pending_large;
  std::deque<int64_t> finished;  // tickets in completion order, for sed_server_next
  std::map<int64_t, std::unique_ptr<Request>> requests;
  int64_t next_ticket = 1, n_done = 0;
  bool started = false, closed = false;
  std::vector<std::thread> threads;

  void start_locked();
  void batch_lane(int lane);
  void large_worker();
  void finish(Request* r) {
    std::lock_guard<std::mutex> lock(mu);
    r->done = true;
    ++n_done;
    finished.push_back(r->ticket);
    done_cv.notify_all();
  }
  // copy a finished request's outputs and release its ticket (mu held)
  void collect(std::map<int64_t, std::unique_ptr<Request>>::iterator it, double* evals, int32_t* status,
               int64_t* dim) {
    Request* r = it->second.get();
    for (int i = 0; i < r->nev; ++i) evals[i] = i < (int)r->evals.size() ? r->evals[i] : std::nan("");
    if (status) *status = r->status;
    if (dim) *dim = r->dim;
    if (r->status != SED_OK) sed::set_error(r->error);
    requests.erase(it);
  }
};

void sed_server::start_locked() {
  if (started) return;
  started = true;
  for (int i = 0; i < n_lanes; ++i) threads.emplace_back([this, i] { batch_lane(i); });
  for (int i = 0; i < n_workers; ++i) threads.emplace_back([this] { large_worker(); });
}

void sed_server::batch_lane(int lane) {
  cudaSetDevice(device);
  for (;;) {
    std::vector<Request*> take;
    int fam = 0;
    {
      std::unique_lock<std::mutex> lock(mu);
      cv.wait(lock, [&] { return closed || !pending_batch.empty(); });
      if (pending_batch.empty()) return;  // closed and drained
      fam = pending_batch.front()->family;  // the oldest request decides the family
      const size_t cap = (size_t)max_batch;
      for (auto it = pending_batch.begin(); it != pending_batch.end() && take.size() < cap;) {
        if ((*it)->family == fam) {
          take.push_back(*it);
          it = pending_batch.erase(it);
        } else {
          ++it;
        }
      }
    }
    const Family& f = families[fam];
    sed_batch* b = f.lanes[lane % f.lanes.size()];
    const int n = (int)take.size();
    std::vector<double> chi((size_t)n * f.n_ops * 2), phase((size_t)n * f.n_ops * f.n_site * 2),
        amp((size_t)n * std::max(f.n_bil, 1) * 2);
    std::vector<uint64_t> seeds(n);
    for (int i = 0; i < n; ++i) {
      std::copy(take[i]->chi.begin(), take[i]->chi.end(), chi.begin() + (size_t)i * f.n_ops * 2);
      std::copy(take[i]->phase.begin(), take[i]->phase.end(), phase.begin() + (size_t)i * f.n_ops * f.n_site * 2);
      std::copy(take[i]->amp.begin(), take[i]->amp.end(), amp.begin() + (size_t)i * f.n_bil * 2);
      seeds[i] = take[i]->seed;
    }
    std::vector<double> evals((size_t)n * f.nev_max), delta(n);
    std::vector<int32_t> status(n), nmv(n);
    std::vector<int64_t> dims(n);
    const int st = sed_batch_run(b, n, chi.data(), phase.data(), amp.data(), seeds.data(), tol, 300, evals.data(),
                                 status.data(), dims.data(), delta.data(), nmv.data());
    const std::string msg = st == SED_OK ? "" : sed_last_error();
    for (int i = 0; i < n; ++i) {
      Request* r = take[i];
      if (st != SED_OK) {
        r->status = st;
        r->error = msg;
      } else {
        r->status = status[i];
        r->dim = dims[i];
        r->evals.assign(evals.begin() + (size_t)i * f.nev_max, evals.begin() + (size_t)i * f.nev_max + r->nev);
      }
      finish(r);
    }
  }
}

void sed_server::large_worker() {
  cudaSetDevice(device);
  for (;;) {
    Request* r = nullptr;
    int64_t need = 0;
    {
      std::unique_lock<std::mutex> lock(mu);
      for (;;) {
        if (!pending_large.empty()) {
          Request* q = pending_large.front();
          need = solve_footprint(families[q->family].n_orbits, q->nev);
          if (reserved + need <= budget - resident || reserved == 0) {
            pending_large.pop_front();
            reserved += need;
            peak_reserved = std::max(peak_reserved, reserved);
            r = q;
            break;
          }
        } else if (closed) {
          return;
        }
        cv.wait(lock);
      }
    }
    const Family& f = families[r->family];
    sed_group* g = nullptr;
    sed_sector* sec = nullptr;
    sed_op* op = nullptr;
    int64_t dim = 0;
    int st = sed_group_create(f.n_site, f.n_ops, f.perm.data(), r->phase.data(), f.identity, f.stats, &g);
    if (st == SED_OK) st = sed_sector_build_group(f.cat, g, r->chi.data(), 1e-12, &sec, &dim);
    r->evals.assign(r->nev, std::nan(""));
    if (st == SED_OK && dim > 0) {
      st = sed_op_create(sec, f.n_bil, f.bil_ij.data(), r->amp.data(), f.n_den, f.den_ij.data(), f.den_v.data(),
                         precision, &op);
      if (st == SED_OK && f.n_orbits <= priority_max_orbits) st = sed_op_set_priority(op, 1);
      if (st == SED_OK) {
        sed_solve_info info{};
        std::vector<double> ev(r->nev);
        // Krylov dimension 24: on the served mix's one-eigenvalue requests it
        // took 3.5 % less device time than 30, and 40 took 10 % more
        st = sed_solve(op, r->nev, tol, 300, 24, r->seed, ev.data(), nullptr, &info);
        if (st == SED_OK) {
          const int k = (int)std::min<int64_t>(r->nev, dim);
          for (int i = 0; i < k; ++i) r->evals[i] = ev[i];
        }
      }
    }
    r->status = st;
    r->dim = st == SED_OK ? dim : -1;
    if (st != SED_OK) r->error = sed_last_error();
    if (op) sed_op_destroy(op);
    if (sec) sed_sector_destroy(sec);
    if (g) sed_group_destroy(g);
    {
      std::lock_guard<std::mutex> lock(mu);
      reserved -= need;
    }
    cv.notify_all();
    finish(r);
  }
}

namespace {
template <class F>
int sguard(F&& f) {
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
#define SREQ(cond, msg) SED_REQUIRE(cond, SED_ERR_ARG, msg)
}  // namespace

extern "C" {

int sed_server_create(double budget_bytes, int batch_lanes, int large_workers, int64_t small_max_orbits,
                      int precision, double tol, sed_server** out) {
  return sguard([&] {
    SREQ(out, "NULL output");
    SREQ(budget_bytes > 0, "budget must be positive");
    SREQ(batch_lanes >= 1 && batch_lanes <= 16, "1 <= batch_lanes <= 16");
    SREQ(large_workers >= 1 && large_workers <= 16, "1 <= large_workers <= 16");
    SREQ(small_max_orbits >= 0, "small_max_orbits must be >= 0");
    SREQ(precision == SED_PREC_FP64 || precision == SED_PREC_MIXED, "precision must be SED_PREC_FP64 or MIXED");
    SREQ(tol > 0, "tol must be positive");
    auto s = std::make_unique<sed_server>();
    SED_CUDA(cudaGetDevice(&s->device));
    s->budget = budget_bytes;
    s->n_lanes = batch_lanes;
    s->n_workers = large_workers;
    s->small_max_orbits = small_max_orbits;
    s->precision = precision;
    s->tol = tol;
    *out = s.release();
  });
}

int sed_server_add_family(sed_server* s, const sed_catalog* c, int n_bil, const int32_t* bil_ij,
                          const double* bil_t_reim, int n_den, const int32_t* den_ij, const double* den_v_reim,
                          int nev_max, int32_t* family) {
  return sguard([&] {
    SREQ(s && c && family, "NULL argument");
    SREQ(n_bil >= 0 && n_den >= 0, "negative term count");
    SREQ(n_bil == 0 || (bil_ij && bil_t_reim), "NULL bilinear arrays");
    SREQ(n_den == 0 || (den_ij && den_v_reim), "NULL density arrays");
    SREQ(nev_max >= 1 && nev_max <= 6, "1 <= nev_max <= 6");
    {
      std::lock_guard<std::mutex> lock(s->mu);
      SREQ(!s->started, "families must be added before the first request");
    }
    const sed::GroupImpl& G = *c->p->group;
    Family f;
    f.n_site = G.n_site;
    f.n_ops = G.n_ops;
    f.identity = G.identity;
    f.stats = G.stats;
    f.perm = G.perm;
    f.bil_ij.assign(bil_ij, bil_ij + 2 * n_bil);
    f.den_ij.assign(den_ij, den_ij + 2 * n_den);
    f.den_v.assign(den_v_reim, den_v_reim + 2 * n_den);
    f.n_bil = n_bil;
    f.n_den = n_den;
    f.nev_max = nev_max;
    f.n_orbits = c->p->n_orbits;
    f.batched = f.n_orbits <= s->small_max_orbits;
    // the family's default terms must be valid for its own group
    const sed_group g0{c->p->group};
    int st = sed_terms_validate(&g0, n_bil, bil_ij, bil_t_reim);
    SED_REQUIRE(st == SED_OK, st, sed_last_error());
    f.cat = new sed_catalog{c->p};
    double resident = (double)c->p->n_states * 8 + (double)f.n_orbits * 9;
    if (f.batched) {
      for (int l = 0; l < s->n_lanes; ++l) {
        sed_batch* b = nullptr;
        st = sed_batch_create(f.cat, n_bil, bil_ij, n_den, den_ij, den_v_reim, s->precision, nev_max, 0,
                              s->max_batch, &b);
        if (st != SED_OK) {
          const std::string msg = sed_last_error();
          for (sed_batch* x : f.lanes) sed_batch_destroy(x);
          delete f.cat;
          SED_REQUIRE(false, st, msg);
        }
        f.lanes.push_back(b);
        int64_t smem = 0, nb = 0, fp = 0;
        sed_batch_info(b, &smem, &nb, &fp);
        resident += (double)fp;
      }
      // warm-up: one wave of the family's untwisted zero-momentum sector
      // through every lane, so each lane builds its hop table and the launch
      // autotuner picks the batch's shape before any request arrives
      int64_t smem = 0, nb = 0, fp = 0;
      sed_batch_info(f.lanes[0], &smem, &nb, &fp);
      const int n = (int)std::max<int64_t>(1, std::min<int64_t>(nb, s->max_batch));
      std::vector<double> chi((size_t)n * f.n_ops * 2, 0.0), phase((size_t)n * f.n_ops * f.n_site * 2, 0.0),
          amp((size_t)n * std::max(n_bil, 1) * 2, 0.0);
      for (size_t i = 0; i < chi.size(); i += 2) chi[i] = 1.0;
      for (size_t i = 0; i < phase.size(); i += 2) phase[i] = 1.0;
      for (int i = 0; i < n; ++i) std::copy(bil_t_reim, bil_t_reim + 2 * n_bil, amp.begin() + (size_t)i * n_bil * 2);
      std::vector<uint64_t> seeds(n);
      for (int i = 0; i < n; ++i) seeds[i] = 0x5EED0000ULL + (uint64_t)i;
      std::vector<double> ev((size_t)n * nev_max), delta(n);
      std::vector<int32_t> status(n), nmv(n);
      std::vector<int64_t> dims(n);
      for (sed_batch* b : f.lanes) {
        st = sed_batch_run(b, n, chi.data(), phase.data(), amp.data(), seeds.data(), s->tol, 300, ev.data(),
                           status.data(), dims.data(), delta.data(), nmv.data());
        if (st != SED_OK) {
          const std::string msg = sed_last_error();
          for (sed_batch* x : f.lanes) sed_batch_destroy(x);
          delete f.cat;
          SED_REQUIRE(false, st, msg);
        }
      }
    }
    // the families vector may only change while no worker thread reads it:
    // check and append under the lock that starts the workers
    std::lock_guard<std::mutex> lock(s->mu);
    const char* refuse = s->started ? "families must be added before the first request"
                         : s->resident + resident > s->budget
                             ? "resident catalogs and batch workspaces exceed the server's budget"
                             : nullptr;
    if (refuse) {
      for (sed_batch* x : f.lanes) sed_batch_destroy(x);
      delete f.cat;
      SED_REQUIRE(false, s->started ? SED_ERR_ARG : SED_ERR_NOMEM, refuse);
    }
    s->resident += resident;
    *family = (int32_t)s->families.size();
    s->families.push_back(std::move(f));
  });
}

int sed_server_submit(sed_server* s, int32_t family, const double* chi_reim, const double* group_phase_reim,
                      const double* bil_t_reim, uint64_t seed, int nev, int64_t* ticket) {
  return sguard([&] {
    SREQ(s && chi_reim && group_phase_reim && ticket, "NULL argument");
    // the family table is read under the lock: sed_server_add_family may be
    // appending to it from another thread until the first request starts the
    // workers
    std::lock_guard<std::mutex> lock(s->mu);
    SREQ(!s->closed, "the server is closed");
    SREQ(family >= 0 && family < (int32_t)s->families.size(), "unknown family");
    const Family& f = s->families[family];
    SREQ(f.n_bil == 0 || bil_t_reim, "NULL bilinear amplitudes");
    SREQ(nev >= 1 && nev <= f.nev_max, "nev must be between 1 and the family's nev_max");
    auto r = std::make_unique<Request>();
    r->family = family;
    r->nev = nev;
    r->seed = seed;
    r->chi.assign(chi_reim, chi_reim + 2 * f.n_ops);
    r->phase.assign(group_phase_reim, group_phase_reim + 2 * (size_t)f.n_ops * f.n_site);
    if (f.n_bil) r->amp.assign(bil_t_reim, bil_t_reim + 2 * f.n_bil);
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    Request* p = r.get();
    s->requests.emplace(r->ticket, std::move(r));
    (f.batched ? s->pending_batch : s->pending_large).push_back(p);
    s->start_locked();
    s->cv.notify_all();
  });
}

int sed_server_wait(sed_server* s, int64_t ticket, int timeout_ms, double* evals, int32_t* status, int64_t* dim) {
  return sguard([&] {
    SREQ(s && evals, "NULL argument");
    std::unique_lock<std::mutex> lock(s->mu);
    SREQ(s->requests.count(ticket), "unknown ticket (or already collected)");
    // the ticket is looked up again after every wake-up: another thread's
    // sed_server_wait or sed_server_next may have collected it meanwhile
    auto it = s->requests.end();
    const bool ready = s->done_cv.wait_for(lock, std::chrono::milliseconds(std::max(timeout_ms, 0)), [&] {
      it = s->requests.find(ticket);
      return it == s->requests.end() || it->second->done;
    });
    SREQ(it != s->requests.end(), "ticket collected by another caller");
    SED_REQUIRE(ready, SED_ERR_TIMEOUT, "request not finished");
    s->collect(it, evals, status, dim);
  });
}

int sed_server_next(sed_server* s, int timeout_ms, int64_t* ticket, double* evals, int32_t* status, int64_t* dim) {
  return sguard([&] {
    SREQ(s && ticket && evals, "NULL argument");
    std::unique_lock<std::mutex> lock(s->mu);
    for (;;) {
      // skip tickets already collected by sed_server_wait
      while (!s->finished.empty() && !s->requests.count(s->finished.front())) s->finished.pop_front();
      if (!s->finished.empty()) break;
      const bool woke = s->done_cv.wait_for(lock, std::chrono::milliseconds(std::max(timeout_ms, 0)), [&] {
        while (!s->finished.empty() && !s->requests.count(s->finished.front())) s->finished.pop_front();
        return !s->finished.empty();
      });
      SED_REQUIRE(woke, SED_ERR_TIMEOUT, "no request finished");
    }
    const int64_t t = s->finished.front();
    s->finished.pop_front();
    *ticket = t;
    s->collect(s->requests.find(t), evals, status, dim);
  });
}

int sed_server_stats(const sed_server* s, int64_t* n_done, int64_t* n_pending, double* peak_reserved_bytes,
                     double* resident_bytes) {
  return sguard([&] {
    SREQ(s, "NULL server");
    sed_server* m = const_cast<sed_server*>(s);
    std::lock_guard<std::mutex> lock(m->mu);
    if (n_done) *n_done = m->n_done;
    if (n_pending) *n_pending = (int64_t)(m->pending_batch.size() + m->pending_large.size());
    if (peak_reserved_bytes) *peak_reserved_bytes = m->peak_reserved;
    if (resident_bytes) *resident_bytes = m->resident;
  });
}

void sed_server_destroy(sed_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->closed = true;
  }
  s->cv.notify_all();
  for (auto& t : s->threads) t.join();
  for (Family& f : s->families) {
    for (sed_batch* b : f.lanes) sed_batch_destroy(b);
    delete f.cat;
  }
  delete s;
}

}  // extern "C"
