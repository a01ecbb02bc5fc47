// hc3d_serve.cpp -- a model-run server on one GPU: requests (a .par model,
// its Lucy iterations and a peeled iteration) are queued, admitted while
// their device footprint fits an HBM budget, and run on a fixed set of slots.
// Each slot is a worker thread with its own context and stream, so the runs
// of different requests overlap on the device: one model's long-history tail
// leaves SMs free that the kernels of the others fill.  A slot keeps its
// stream, packet pool and peel-off queue from one request to the next
// (hc3d_reset); each request's grid and tallies stay resident while it runs.
//
// Results do not depend on the mix: packet streams are keyed by (seed,
// iteration, packet id) and the tallies are int64 sums, so a request gives
// the same arrays whether it runs alone or beside others.
//
// The reference runs one model per process (newtts.F90); the request run
// below is its driver loop (newtts.F90:294-368) without the output files.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hc3d.h"
#include "../../include/hc3d_host.h"
#include "hc3d_model.h"

namespace {

using clk = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  std::string par, par_dir;
  bool has_dir = false;
  int n_lucy = -1;
  int64_t np_lucy = 0, np = 0;
  std::vector<double> thete, phie;
  double t_submit = 0;
};

struct Result {
  int status = HC3D_OK;
  std::string err;
  double t_submit = 0, t_admit = 0, t_done = 0;
  int64_t footprint = 0, packets = 0;
  int iterations = 0;
  double max_rel_change = 0;
  int nfreq = 0, nmu = 0, nph = 0, nap = 0, npeel = 0;
  std::vector<int64_t> si, nums, ti, numt;
  double stokes_scale = 0;
};

}  // namespace

struct hc3d_server {
  hc3d_server_opts opts{};
  int64_t budget = 0, in_use = 0, peak_in_use = 0;
  int running = 0, peak_running = 0;
  int64_t completed = 0, next_ticket = 1;
  bool stop = false;
  clk::time_point t0;
  std::deque<Request> queue;
  std::map<int64_t, Result> done;
  std::set<int64_t> claimed;  // tickets whose result was handed out
  std::set<int64_t> cancelled;  // running requests asked to stop at their next iteration
  std::mutex mu;
  std::condition_variable cv_queue, cv_mem, cv_done;
  std::vector<std::thread> workers;
  std::vector<hc3d_ctx*> ctxs;
};

namespace {

double since(const hc3d_server* s) { return std::chrono::duration<double>(clk::now() - s->t0).count(); }

// Device bytes a model run holds besides the slot's fixed pool and queue:
// the grid and temperature arrays and the Lucy tallies the context loads
// (hc3d_load_grid), the dust tables (hc3d_load_tables) and the SED, peeled
// SED and image tallies of the peeled iteration; with small grains their
// tallies, spectrum rows and the spectra.
int64_t footprint_bytes(const hc3d::Model& m, int npeel) {
  const int64_t ncell = m.ncells(), n4 = m.n4();
  const int64_t sg = m.sg_slot >= 0 ? ncell * (4 /*dsg*/ + 8 /*jsg*/ + 4 /*imean*/ + 8 /*imfract*/ + 8 /*vcell*/) +
                                          (int64_t)2 * hc3d::kNemit * hc3d::kNdraine * 8
                                    : 0;
  const int64_t grid = ncell * (4 * 4 /*rho f32*/ + 4 * 8 /*rho f64*/ + 2 * 4 * 8 /*tdust, massarr*/ + 4 * 4 /*tdust f32*/ +
                                1 /*peel mask*/ + 2 * 4 * 8 /*nabs, dtauabs*/ + 8 /*jmean*/ + 2 * 4 /*killed, dbig*/) +
                       sg;
  const int64_t walls = (int64_t)(m.nrg + m.ntg + m.npg) * 64 + n4 * 8 /*vcell*/;
  const int64_t tables = (int64_t)m.nT * m.nnu * 4 * 12 + (int64_t)m.nlammax * 4 * 5 * 12 + (1 << 20);
  const int64_t sed = (int64_t)m.nfreq * m.nmu * m.nph * m.nap * 8 * 9 * 8;
  const int64_t psed = (int64_t)m.nfreq * npeel * m.nap * 8 * 9 * 8;
  const int64_t img = (int64_t)npeel * m.nxhst * m.nxhst * 4 * 8;
  return grid + walls + tables + sed + psed + img;
}

int ctx_error(hc3d_ctx* c, int code, Result* res) {
  char buf[512];
  hc3d_get_error(c, buf, sizeof buf);
  res->status = code;
  res->err = buf;
  return code;
}

// One request on slot context c: the Lucy iterations (newtts.F90:294-330),
// then the peeled iteration (newtts.F90:333-368); the SED and peeled SED of
// the peeled iteration are returned.
int run_request(hc3d_server* s, hc3d_ctx* c, const Request& q, Result* res) {
  hc3d_model* hm = nullptr;
  char err[512] = {0};
  int r = hc3d_model_create(&hm, q.par.c_str(), q.has_dir ? q.par_dir.c_str() : nullptr, err, sizeof err);
  if (r) {
    res->status = r;
    res->err = err;
    return r;
  }
  hc3d::Model& m = hm->m;
  if (!q.thete.empty()) {
    m.npeel = (int)q.thete.size();
    m.thete = q.thete;
    m.phie = q.phie;
  }
  if (q.np > 0) m.np = q.np;
  if (q.np_lucy > 0) m.np_lucy = q.np_lucy;
  const int64_t fp = footprint_bytes(m, m.ipeel ? m.npeel : 0);
  res->footprint = fp;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    if (fp > s->budget) {
      res->status = HC3D_ERR_NOMEM;
      res->err = "the model's device footprint exceeds the server's HBM budget";
      hc3d_model_destroy(hm);
      return res->status;
    }
    s->cv_mem.wait(lk, [&] { return s->in_use + fp <= s->budget; });
    s->in_use += fp;
    s->peak_in_use = std::max(s->peak_in_use, s->in_use);
    s->running++;
    s->peak_running = std::max(s->peak_running, s->running);
    res->t_admit = since(s);
  }
  auto release = [&] {
    std::lock_guard<std::mutex> lk(s->mu);
    s->in_use -= fp;
    s->running--;
    s->cv_mem.notify_all();
  };
  hc3d_run_params p = m.params_view();
  std::vector<double> td(m.tdust);
  int iter = 0;
  if ((r = hc3d_reset(c)) || (r = hc3d_model_load(hm, c))) {
    ctx_error(c, r, res);
    release();
    hc3d_model_destroy(hm);
    return r;
  }
  // a cancelled request stops between iterations, with no kernel in flight
  auto stop_asked = [&] {
    std::lock_guard<std::mutex> lk(s->mu);
    return s->cancelled.count(q.ticket) != 0;
  };
  bool converge = q.n_lucy == 0;
  while (!converge) {
    if (stop_asked()) {
      r = HC3D_ERR_CANCELLED;
      break;
    }
    ++iter;
    p.np = m.np_lucy;
    m.set_shares(&p, p.np);
    p.ipeel = 0;
    p.iter = iter;
    double rel = 0;
    int conv = 0;
    if ((r = hc3d_zero_tallies(c)) || (r = hc3d_run_iteration(c, &p)) ||
        (r = hc3d_lucy_update(c, m.ltot, p.np, td.data(), &rel, &conv)))
      break;
    res->packets += p.np;
    res->max_rel_change = rel;
    if (q.n_lucy >= 0) {
      converge = iter >= q.n_lucy;
    } else {
      converge = conv != 0;
      if (iter < m.nimin) converge = false;
      if (iter >= m.nimax) converge = true;
    }
  }
  if (!r && stop_asked()) r = HC3D_ERR_CANCELLED;
  if (!r) {
    ++iter;
    p.np = m.np;
    m.set_shares(&p, p.np);
    p.ipeel = m.ipeel;
    p.iter = iter;
    res->nfreq = p.nfreq; res->nmu = p.nmu; res->nph = p.nph; res->nap = p.nap;
    res->npeel = p.ipeel ? p.npeel : 0;
    const size_t nsed = (size_t)p.nfreq * p.nmu * p.nph * p.nap * 8;
    const size_t npsed = (size_t)p.nfreq * res->npeel * p.nap * 8;
    res->si.assign(nsed, 0); res->nums.assign(nsed, 0);
    res->ti.assign(std::max<size_t>(npsed, 1), 0); res->numt.assign(std::max<size_t>(npsed, 1), 0);
    hc3d_tallies T;
    std::memset(&T, 0, sizeof T);
    T.si = res->si.data(); T.nums = res->nums.data();
    if (res->npeel) { T.ti = res->ti.data(); T.numt = res->numt.data(); }
    if (!(r = hc3d_zero_tallies(c)) && !(r = hc3d_run_iteration(c, &p)) && !(r = hc3d_get_tallies(c, &p, &T))) {
      res->packets += p.np;
      res->stokes_scale = T.stokes_scale;
    }
  }
  res->iterations = iter;
  if (r == HC3D_ERR_CANCELLED) {
    res->status = r;
    res->err = "the request was cancelled";
  } else if (r) {
    ctx_error(c, r, res);
  }
  release();
  hc3d_model_destroy(hm);
  return r;
}

void worker(hc3d_server* s, int slot) {
  hc3d_ctx* c = s->ctxs[slot];
  for (;;) {
    Request q;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_queue.wait(lk, [&] { return s->stop || !s->queue.empty(); });
      if (s->queue.empty()) return;  // stopping and drained
      q = std::move(s->queue.front());
      s->queue.pop_front();
    }
    Result res;
    res.t_submit = q.t_submit;
    run_request(s, c, q, &res);
    res.t_done = since(s);
    std::lock_guard<std::mutex> lk(s->mu);
    s->cancelled.erase(q.ticket);
    s->completed++;
    s->done[q.ticket] = std::move(res);
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" int hc3d_server_create(hc3d_server** out, const hc3d_server_opts* o) {
  if (!out || !o || o->slots < 1 || o->slots > 64 || o->hbm_budget < 0) return HC3D_ERR_INVALID;
  hc3d_server* s = new hc3d_server();
  s->opts = *o;
  s->t0 = clk::now();
  if (cudaSetDevice(o->device) != cudaSuccess) {
    delete s;
    return HC3D_ERR_CUDA;
  }
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    delete s;
    return HC3D_ERR_CUDA;
  }
  for (int k = 0; k < o->slots; ++k) {
    hc3d_device_opts d;
    std::memset(&d, 0, sizeof d);
    d.device = o->device;
    d.precision = o->precision;
    hc3d_ctx* c = nullptr;
    const int r = hc3d_create(&c, &d);
    if (r) {
      for (hc3d_ctx* x : s->ctxs) hc3d_destroy(x);
      delete s;
      return r;
    }
    s->ctxs.push_back(c);
  }
  s->budget = o->hbm_budget > 0 ? o->hbm_budget : (int64_t)(0.8 * (double)fr);
  for (int k = 0; k < o->slots; ++k) s->workers.emplace_back(worker, s, k);
  *out = s;
  return HC3D_OK;
}

extern "C" int hc3d_server_submit(hc3d_server* s, const hc3d_request* r, int64_t* ticket) {
  if (!s || !r || !r->par_path || !ticket) return HC3D_ERR_INVALID;
  if (r->npeel < 0 || r->npeel > 256 || (r->npeel > 0 && (!r->thete || !r->phie))) return HC3D_ERR_INVALID;
  Request q;
  q.par = r->par_path;
  if (r->par_dir) {
    q.par_dir = r->par_dir;
    q.has_dir = true;
  }
  q.n_lucy = r->n_lucy;
  q.np_lucy = r->np_lucy;
  q.np = r->np;
  if (r->npeel > 0) {
    q.thete.assign(r->thete, r->thete + r->npeel);
    q.phie.assign(r->phie, r->phie + r->npeel);
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return HC3D_ERR_STATE;
  q.ticket = s->next_ticket++;
  q.t_submit = since(s);
  *ticket = q.ticket;
  s->queue.push_back(std::move(q));
  s->cv_queue.notify_one();
  return HC3D_OK;
}

extern "C" int hc3d_server_wait(hc3d_server* s, int64_t ticket, hc3d_result* out) {
  if (!s || !out || ticket < 1) return HC3D_ERR_INVALID;
  Result res;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    // an unknown ticket, or one whose result was already handed out, would wait forever
    if (ticket >= s->next_ticket || s->claimed.count(ticket)) return HC3D_ERR_INVALID;
    s->claimed.insert(ticket);
    s->cv_done.wait(lk, [&] { return s->done.count(ticket) != 0; });
    res = std::move(s->done[ticket]);
    s->done.erase(ticket);
  }
  std::memset(out, 0, sizeof *out);
  out->status = res.status;
  std::snprintf(out->err, sizeof out->err, "%s", res.err.c_str());
  out->t_submit = res.t_submit; out->t_admit = res.t_admit; out->t_done = res.t_done;
  out->footprint_bytes = res.footprint; out->packets = res.packets; out->iterations = res.iterations;
  out->max_rel_change = res.max_rel_change;
  out->nfreq = res.nfreq; out->nmu = res.nmu; out->nph = res.nph; out->nap = res.nap; out->npeel = res.npeel;
  out->stokes_scale = res.stokes_scale;
  auto dup = [](const std::vector<int64_t>& v) {
    int64_t* p = (int64_t*)std::malloc(sizeof(int64_t) * std::max<size_t>(v.size(), 1));
    if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(int64_t) * v.size());
    return p;
  };
  if (res.status == HC3D_OK) {
    out->si = dup(res.si); out->nums = dup(res.nums); out->ti = dup(res.ti); out->numt = dup(res.numt);
    if (!out->si || !out->nums || !out->ti || !out->numt) {
      hc3d_result_free(out);
      out->status = HC3D_ERR_NOMEM;
    }
  }
  return out->status;
}

extern "C" int hc3d_server_cancel(hc3d_server* s, int64_t ticket) {
  if (!s || ticket < 1) return HC3D_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (ticket >= s->next_ticket || s->claimed.count(ticket)) return HC3D_ERR_INVALID;
  if (s->done.count(ticket)) return HC3D_ERR_STATE;  // finished: its result stands
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
    if (it->ticket != ticket) continue;
    Result res;
    res.status = HC3D_ERR_CANCELLED;
    res.err = "the request was cancelled before it was admitted";
    res.t_submit = it->t_submit;
    res.t_done = since(s);
    s->queue.erase(it);
    s->completed++;
    s->done[ticket] = std::move(res);
    s->cv_done.notify_all();
    return HC3D_OK;
  }
  s->cancelled.insert(ticket);  // running: it stops before its next iteration
  return HC3D_OK;
}

extern "C" void hc3d_result_free(hc3d_result* r) {
  if (!r) return;
  std::free(r->si); std::free(r->nums); std::free(r->ti); std::free(r->numt);
  r->si = r->nums = r->ti = r->numt = nullptr;
}

extern "C" int hc3d_server_get_stats(hc3d_server* s, hc3d_server_stats* st) {
  if (!s || !st) return HC3D_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  st->budget_bytes = s->budget;
  st->in_use_bytes = s->in_use;
  st->peak_in_use_bytes = s->peak_in_use;
  st->running = s->running;
  st->peak_running = s->peak_running;
  st->queued = (int64_t)s->queue.size();
  st->completed = s->completed;
  return HC3D_OK;
}

extern "C" void hc3d_server_destroy(hc3d_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_queue.notify_all();
  }
  for (std::thread& t : s->workers) t.join();
  for (hc3d_ctx* c : s->ctxs) hc3d_destroy(c);
  delete s;
}

extern "C" int64_t hc3d_model_footprint(const hc3d_model* m) {
  if (!m) return -1;
  return footprint_bytes(m->m, m->m.ipeel ? m->m.npeel : 0);
}
