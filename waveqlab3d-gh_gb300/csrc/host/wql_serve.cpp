// Request server: scenarios submitted from any thread are admitted by device
// memory footprint, advanced together in a continuous batch (wql_batch_*),
// retired when they reach their step count, and their seismograms and
// timings kept until released.  One worker thread owns the GPU work; it is
// written against the public C ABI only.
//
// Two threads own the GPU work.  The worker admits queued requests in
// arrival order while the head's peak footprint (wql_estimate_device_bytes)
// fits next to the bytes held or reserved by the admitted ones (the head is
// always admitted when nothing is admitted), hands each to the preparer,
// moves prepared scenarios into the batch, steps the batch by the smallest
// remaining step count of its members (at most round_steps) and retires
// finished members.  The preparer creates the admitted scenarios (host grid
// generation, uploads, set-up kernels on the scenario's own stream) while the
// batch steps, so the device does not wait for a new request's set-up.
// Requests that arrive while others run join the batch at the next round
// after their set-up.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../../include/wql.h"
#include "wql_input.h"

namespace {

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

struct Request {
  long long id = 0;
  std::string text;
  int precision = WQL_FP32C;
  int nsteps = 0;
  // copies of the caller's media arrays (the pointers need not outlive submit)
  std::vector<double> fault, topo[2], lam[2], mu[2], rho[2];
  bool has_media = false;
  long long peak = 0, resident = 0;
  double t_arrive = 0, t_admit = -1, t_done = -1;
  int status = 0;  // 0 queued/running, 1 done, < 0 failed (-WQL_E_*)
  std::string err;
  wql_scn* scn = nullptr;
  int nst[2] = {0, 0}, nrec = 0;
  std::vector<double> seis[2];
  std::vector<int> ijk[2];
};

std::string last_error() {
  char buf[1024];
  wql_last_error(buf, sizeof(buf));
  return buf;
}

}  // namespace

struct wql_server {
  wql_ctx* ctx = nullptr;
  long long budget = 0;
  int round_steps = 1;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  std::mutex mu;
  std::condition_variable cv;       // work for the worker
  std::condition_variable done_cv;  // a request finished
  bool stop = false;
  long long next_id = 1;
  std::deque<Request*> queue;     // submitted, waiting for admission
  std::deque<Request*> prep;      // admitted, waiting for the preparer
  std::vector<Request*> ready;    // created, waiting to join the batch
  int preparing = 0;              // admitted requests not yet in the batch
  bool worker_done = false;       // the worker has returned (the preparer may too)
  std::vector<Request*> active;
  std::condition_variable prep_cv;  // work for the preparer
  std::map<long long, std::unique_ptr<Request>> all;
  long long in_use = 0;
  long long completed = 0, steps_done = 0;
  wql_batch* batch = nullptr;
  std::thread worker, preparer;

  void run();
  void prepare();
  void finish(Request* r, int status, const std::string& err);
};

void wql_server::finish(Request* r, int status, const std::string& err) {
  std::lock_guard<std::mutex> lock(mu);
  r->status = status;
  r->err = err;
  r->t_done = now_s(t0);
  if (status == 1) completed += 1;
  done_cv.notify_all();
}

// Creates the admitted scenarios, one at a time, in admission order.
void wql_server::prepare() {
  for (;;) {
    Request* r = nullptr;
    {
      std::unique_lock<std::mutex> lock(mu);
      prep_cv.wait(lock, [&] { return worker_done || !prep.empty(); });
      if (prep.empty()) return;
      r = prep.front();
      prep.pop_front();
    }
    wql_media m;
    std::memset(&m, 0, sizeof(m));
    if (r->has_media) {
      m.fault_offset = r->fault.empty() ? nullptr : r->fault.data();
      for (int b = 0; b < 2; ++b) {
        m.topo_offset[b] = r->topo[b].empty() ? nullptr : r->topo[b].data();
        m.lam[b] = r->lam[b].empty() ? nullptr : r->lam[b].data();
        m.mu[b] = r->mu[b].empty() ? nullptr : r->mu[b].data();
        m.rho[b] = r->rho[b].empty() ? nullptr : r->rho[b].data();
      }
    }
    wql_scn* scn = nullptr;
    const int rc = wql_scenario_create_ex(ctx, r->text.c_str(), nullptr, r->precision, r->has_media ? &m : nullptr, &scn);
    if (rc) {
      const std::string e = last_error();
      {
        std::lock_guard<std::mutex> lock(mu);
        preparing -= 1;
        in_use -= r->peak;
        cv.notify_all();
      }
      finish(r, -rc, e);
      continue;
    }
    wql_info info;
    wql_get_info(scn, &info);
    std::lock_guard<std::mutex> lock(mu);
    r->scn = scn;
    in_use += info.device_bytes - r->peak;  // the reservation becomes the bytes held
    r->resident = info.device_bytes;
    ready.push_back(r);
    cv.notify_all();
  }
}

void wql_server::run() {
  for (;;) {
    std::vector<Request*> joining, act;
    {
      std::unique_lock<std::mutex> lock(mu);
      for (;;) {
        // admit: reserve the head's peak bytes and hand it to the preparer
        while (!queue.empty()) {
          Request* head = queue.front();
          if ((!active.empty() || preparing > 0) && in_use + head->peak > budget) break;
          queue.pop_front();
          in_use += head->peak;
          preparing += 1;
          prep.push_back(head);
          prep_cv.notify_one();
        }
        joining.swap(ready);
        if (!joining.empty() || !active.empty()) break;
        if (stop && queue.empty() && preparing == 0) {
          worker_done = true;
          prep_cv.notify_all();
          return;
        }
        cv.wait(lock);
      }
      preparing -= (int)joining.size();
    }
    for (auto* r : joining) {
      wql_batch_add(batch, r->scn);
      std::lock_guard<std::mutex> lock(mu);
      r->t_admit = now_s(t0);
      active.push_back(r);
    }
    {
      std::lock_guard<std::mutex> lock(mu);
      act = active;
    }
    // step
    int k = round_steps;
    for (auto* r : act) {
      wql_info info;
      wql_get_info(r->scn, &info);
      k = std::min(k, r->nsteps - info.nstep);
    }
    if (k > 0) {
      const int rc = wql_batch_step(batch, k);
      if (rc) {
        const std::string e = last_error();
        for (auto* r : act) {
          wql_batch_remove(batch, r->scn);
          wql_scenario_destroy(r->scn);
          r->scn = nullptr;
          {
            std::lock_guard<std::mutex> lock(mu);
            in_use -= r->resident;
            active.erase(std::find(active.begin(), active.end(), r));
          }
          finish(r, -rc, e);
        }
        continue;
      }
      std::lock_guard<std::mutex> lock(mu);
      steps_done += k;
    }
    // retire
    for (auto* r : act) {
      wql_info info;
      wql_get_info(r->scn, &info);
      if (info.nstep < r->nsteps) continue;
      int rc = wql_sync(r->scn, 1);
      for (int b = 0; b < 2 && !rc; ++b) {
        rc = wql_station_count(r->scn, b, &r->nst[b], &r->nrec);
        if (rc) break;
        r->ijk[b].resize(3 * r->nst[b]);
        r->seis[b].resize((size_t)r->nrec * r->nst[b] * 4);
        if (r->nst[b]) rc = wql_station_index(r->scn, b, r->ijk[b].data());
        if (!rc && r->nst[b]) rc = wql_get_seismograms(r->scn, b, r->seis[b].data());
      }
      const std::string e = rc ? last_error() : std::string();
      wql_batch_remove(batch, r->scn);
      wql_scenario_destroy(r->scn);
      r->scn = nullptr;
      {
        std::lock_guard<std::mutex> lock(mu);
        in_use -= r->resident;
        active.erase(std::find(active.begin(), active.end(), r));
      }
      finish(r, rc ? -rc : 1, e);
    }
  }
}

extern "C" {

int wql_server_create(wql_ctx* ctx, long long hbm_budget_bytes, int round_steps, wql_server** out) {
  if (!ctx || !out || hbm_budget_bytes <= 0 || round_steps <= 0) return WQL_E_INPUT;
  std::unique_ptr<wql_server> s(new wql_server());
  s->ctx = ctx;
  s->budget = hbm_budget_bytes;
  s->round_steps = round_steps;
  int rc = wql_batch_create(ctx, &s->batch);
  if (rc) return rc;
  wql_server* p = s.release();
  p->worker = std::thread([p] { p->run(); });
  p->preparer = std::thread([p] { p->prepare(); });
  *out = p;
  return WQL_OK;
}

int wql_server_submit(wql_server* s, const char* in_text, int precision, const wql_media* media, int nsteps,
                      long long* id) {
  if (!s || !in_text || !id || nsteps <= 0) return WQL_E_INPUT;
  auto r = std::make_unique<Request>();
  r->text = in_text;
  r->precision = precision;
  r->nsteps = nsteps;
  int rc = wql_estimate_device_bytes(in_text, nullptr, precision, &r->resident, &r->peak);
  if (rc) return rc;
  // copy the media arrays now (sizes from the parsed block dimensions)
  if (media) {
    wql::Problem P;
    std::string perr;
    if (wql::parse_in_text(in_text, "", P, perr)) return WQL_E_INPUT;
    r->has_media = true;
    const long long nr0 = P.btp[0].nqrs[1], ns0 = P.btp[0].nqrs[2];
    if (media->fault_offset) r->fault.assign(media->fault_offset, media->fault_offset + nr0 * ns0);
    for (int b = 0; b < 2; ++b) {
      const long long nq = P.btp[b].nqrs[0], nr = P.btp[b].nqrs[1], ns = P.btp[b].nqrs[2];
      const long long np = nq * nr * ns;
      if (media->topo_offset[b]) r->topo[b].assign(media->topo_offset[b], media->topo_offset[b] + nq * ns);
      if (media->lam[b]) r->lam[b].assign(media->lam[b], media->lam[b] + np);
      if (media->mu[b]) r->mu[b].assign(media->mu[b], media->mu[b] + np);
      if (media->rho[b]) r->rho[b].assign(media->rho[b], media->rho[b] + np);
    }
  }
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->stop) return WQL_E_STATE;
  r->id = s->next_id++;
  r->t_arrive = now_s(s->t0);
  *id = r->id;
  s->queue.push_back(r.get());
  s->all[r->id] = std::move(r);
  s->cv.notify_all();
  return WQL_OK;
}

int wql_server_wait(wql_server* s, long long id, double timeout_s, int* status) {
  if (!s || !status) return WQL_E_INPUT;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return WQL_E_INPUT;
  Request* r = it->second.get();
  s->done_cv.wait_for(lock, std::chrono::duration<double>(timeout_s), [&] { return r->status != 0; });
  *status = r->status;
  return WQL_OK;
}

int wql_server_result(wql_server* s, long long id, int block, int* nstations, int* nrecords, double* seis,
                      double* times) {
  if (!s || block < 0 || block > 1) return WQL_E_INPUT;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return WQL_E_INPUT;
  Request* r = it->second.get();
  if (r->status == 0) return WQL_E_STATE;
  if (nstations) *nstations = r->nst[block];
  if (nrecords) *nrecords = r->nrec;
  if (seis && !r->seis[block].empty()) std::memcpy(seis, r->seis[block].data(), r->seis[block].size() * sizeof(double));
  if (times) {
    times[0] = r->t_arrive;
    times[1] = r->t_admit;
    times[2] = r->t_done;
  }
  return r->status == 1 ? WQL_OK : -r->status;
}

int wql_server_release(wql_server* s, long long id) {
  if (!s) return WQL_E_INPUT;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end() || it->second->status == 0) return WQL_E_STATE;
  s->all.erase(it);
  return WQL_OK;
}

int wql_server_stats(wql_server* s, long long* completed, long long* queued, long long* active, long long* bytes_in_use) {
  if (!s) return WQL_E_INPUT;
  std::lock_guard<std::mutex> lock(s->mu);
  if (completed) *completed = s->completed;
  if (queued) *queued = (long long)s->queue.size() + s->preparing;  // admitted ones in set-up too
  if (active) *active = (long long)s->active.size();
  if (bytes_in_use) *bytes_in_use = s->in_use;
  return WQL_OK;
}

int wql_server_destroy(wql_server* s) {
  if (!s) return WQL_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
    s->cv.notify_all();
    s->prep_cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  if (s->preparer.joinable()) s->preparer.join();
  wql_batch_destroy(s->batch);
  delete s;
  return WQL_OK;
}

}  // extern "C"
