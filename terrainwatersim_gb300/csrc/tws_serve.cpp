// tws_serve.cpp -- the serving loop: continuous batching of simulation
// requests over one GPU, written against the public C ABI (include/tws.h).
//
// Batched mode, per iteration:
//   1. enqueue one chain (up to chain_steps steps) for every resident grid;
//   2. while the GPU runs it, take the requests whose arrival time has passed
//      and, in arrival order, admit those whose state fits the memory budget:
//      create the grid and generate its scene on the grid's own stream;
//   3. wait for the chain; retire the grids that finished (FP64 volume, time
//      to completion, memory released);
//   4. the grids admitted in step 2 join the batch for the next chain.
// Serial mode (the baseline): one request at a time, in arrival order, each
// through the single-grid path with the plain kernel.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/tws.h"

namespace {

using Clock = std::chrono::steady_clock;

// Work per chain when chains are sized automatically: about 15 ms at
// 100 G cell-steps/s.
constexpr double kChainCellSteps = 1.5e9;

struct Admitted {
  tws_request req;
  tws_grid* grid = nullptr;
  int left = 0;
  double admit_s = 0.0;
  double bytes = 0.0;
};

}  // namespace

struct tws_server {
  tws_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv;
  std::deque<tws_request> submitted;  // not yet taken by the loop
  bool closed = false;
  std::vector<tws_result> results;
  double cell_steps = 0.0, seconds = 0.0, peak_bytes = 0.0;
  uint64_t chains = 0;
};

namespace {

double since(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

bool valid_request(const tws_request& r) {
  return r.width >= 1 && r.height >= 1 && r.steps >= 0 && r.nsources >= 0 &&
         r.nsources <= TWS_MAX_SOURCES && r.arrival_s >= 0.0;
}

// Create the grid of a request and queue its scene on the grid's stream.
int make_grid(const tws_server_config& cfg, const tws_request& r, tws_grid** out) {
  tws_grid* g = nullptr;
  int rc = tws_create(r.width, r.height, &r.params, cfg.flux_storage, nullptr, &g);
  if (rc != TWS_OK) return rc;
  rc = tws_generate_scene(g, r.seed, r.height_scale, r.fill);
  if (rc == TWS_OK) rc = tws_set_sources(g, r.sources, r.nsources);
  if (rc != TWS_OK) {
    tws_destroy(g);
    return rc;
  }
  *out = g;
  return TWS_OK;
}

tws_result result_of(const tws_request& r, int status) {
  tws_result res{};
  res.id = r.id;
  res.status = status;
  res.arrival_s = r.arrival_s;
  res.admit_s = res.done_s = -1.0;
  return res;
}

// Move every submitted request whose arrival time has passed into `ready`
// (kept in arrival order).  Returns the earliest arrival still in the future
// (or a negative number).
double take_arrivals(tws_server* s, double now, std::vector<tws_request>& ready, bool* closed) {
  std::lock_guard<std::mutex> lk(s->mu);
  double next = -1.0;
  for (auto it = s->submitted.begin(); it != s->submitted.end();) {
    if (it->arrival_s <= now) {
      ready.push_back(*it);
      it = s->submitted.erase(it);
    } else {
      next = next < 0 ? it->arrival_s : std::min(next, it->arrival_s);
      ++it;
    }
  }
  std::stable_sort(ready.begin(), ready.end(), [](const tws_request& a, const tws_request& b) {
    return a.arrival_s < b.arrival_s;
  });
  *closed = s->closed && s->submitted.empty();
  return next;
}

void wait_for_work(tws_server* s, Clock::time_point t0, double next_arrival) {
  std::unique_lock<std::mutex> lk(s->mu);
  if (next_arrival >= 0) {
    const auto until = t0 + std::chrono::duration_cast<Clock::duration>(
                                std::chrono::duration<double>(next_arrival));
    s->cv.wait_until(lk, until);
  } else if (!s->closed) {
    s->cv.wait_for(lk, std::chrono::milliseconds(50));
  }
}

int run_batched(tws_server* s) {
  const tws_server_config& cfg = s->cfg;
  const int chain = cfg.chain_steps > 0 ? cfg.chain_steps : 16;  // fixed chain length
  tws_batch* batch = nullptr;
  int rc = tws_batch_create(cfg.flux_storage, nullptr, &batch);
  if (rc != TWS_OK) return rc;
  if (cfg.batch_variant >= 0) tws_batch_set_variant(batch, cfg.batch_variant);
  bool tuned = cfg.batch_variant >= 0;

  const auto t0 = Clock::now();
  std::vector<tws_request> ready;
  std::vector<Admitted> active, joining;
  double resident = 0.0;
  bool closed = false;

  auto admit = [&](double now) {
    const double next = take_arrivals(s, now, ready, &closed);
    size_t taken = 0;
    for (; taken < ready.size(); ++taken) {
      const tws_request& r = ready[taken];
      const double bytes = tws_grid_bytes(r.width, r.height, cfg.flux_storage);
      if (bytes > cfg.memory_budget_bytes) {  // can never fit
        s->results.push_back(result_of(r, TWS_ERR_BUSY));
        continue;
      }
      if (resident + bytes > cfg.memory_budget_bytes) break;  // admit in arrival order
      Admitted a;
      a.req = r;
      a.left = r.steps;
      a.bytes = bytes;
      a.admit_s = since(t0);
      const int mrc = make_grid(cfg, r, &a.grid);
      if (mrc != TWS_OK) {
        tws_result res = result_of(r, mrc);
        res.admit_s = a.admit_s;
        s->results.push_back(res);
        continue;
      }
      resident += bytes;
      s->peak_bytes = std::max(s->peak_bytes, resident);
      joining.push_back(a);
    }
    ready.erase(ready.begin(), ready.begin() + (long)taken);
    return next;
  };

  auto retire = [&](Admitted& a, int status, double done) {
    tws_result res = result_of(a.req, status);
    res.steps = a.req.steps - a.left;
    res.admit_s = a.admit_s;
    res.done_s = done;
    if (a.grid) {
      tws_volume(a.grid, &res.volume);
      if (a.grid && tws_batch_size(batch) > 0) tws_batch_remove(batch, a.grid);
      if (cfg.keep_grids) {
        res.grid = a.grid;
      } else {
        tws_destroy(a.grid);
      }
    }
    resident -= a.bytes;
    s->results.push_back(res);
  };

  for (;;) {
    // grids admitted during the last chain join now
    for (Admitted& a : joining) {
      if (a.req.steps == 0) {
        retire(a, TWS_OK, since(t0));
        continue;
      }
      const int arc = tws_batch_add(batch, a.grid);
      if (arc != TWS_OK) {
        retire(a, arc, since(t0));
        continue;
      }
      active.push_back(a);
    }
    joining.clear();

    if (active.empty()) {
      const double next = admit(since(t0));
      if (!joining.empty()) continue;
      if (closed && ready.empty()) break;
      wait_for_work(s, t0, next);
      continue;
    }
    if (!tuned) {
      int v = 0;
      tws_batch_autotune(batch, 16, &v);
      tuned = true;
    }
    // Steps this chain: fixed, or (chain_steps <= 0) sized so a chain is about
    // kChainCellSteps cell-steps of work -- long enough that the host work
    // between chains is small, short enough that new arrivals join soon.
    int this_chain = chain;
    if (cfg.chain_steps <= 0) {
      double cells = 0.0;
      for (const Admitted& a : active) cells += (double)a.req.width * a.req.height;
      const double want = kChainCellSteps / std::max(1.0, cells);
      this_chain = std::max(16, std::min(512, (int)(want / 16.0) * 16));
    }
    std::vector<int> steps(active.size());
    for (size_t i = 0; i < active.size(); ++i) steps[i] = std::min(active[i].left, this_chain);
    rc = tws_batch_step_each(batch, steps.data(), (int)steps.size());
    if (rc != TWS_OK) break;
    ++s->chains;
    admit(since(t0));  // host work overlaps the chain on the GPU
    const int src = tws_batch_sync(batch);
    const double done = since(t0);
    std::vector<Admitted> still;
    for (size_t i = 0; i < active.size(); ++i) {
      Admitted& a = active[i];
      a.left -= steps[i];
      s->cell_steps += (double)a.req.width * a.req.height * steps[i];
      if (src != TWS_OK || a.left == 0) {
        retire(a, src, done);
      } else {
        still.push_back(a);
      }
    }
    active.swap(still);
    if (src != TWS_OK) {
      rc = src;
      break;
    }
  }
  for (Admitted& a : active) retire(a, rc == TWS_OK ? TWS_ERR_CUDA : rc, since(t0));
  for (Admitted& a : joining) retire(a, rc == TWS_OK ? TWS_ERR_CUDA : rc, since(t0));
  s->seconds = since(t0);
  tws_batch_destroy(batch);
  return rc;
}

int run_serial(tws_server* s) {
  const tws_server_config& cfg = s->cfg;
  const auto t0 = Clock::now();
  std::vector<tws_request> ready;
  bool closed = false;
  for (;;) {
    const double next = take_arrivals(s, since(t0), ready, &closed);
    if (ready.empty()) {
      if (closed) break;
      wait_for_work(s, t0, next);
      continue;
    }
    const tws_request r = ready.front();
    ready.erase(ready.begin());
    tws_result res = result_of(r, TWS_OK);
    res.admit_s = since(t0);
    tws_grid* g = nullptr;
    int rc = make_grid(cfg, r, &g);
    if (rc == TWS_OK) {
      s->peak_bytes = std::max(s->peak_bytes, tws_grid_bytes(r.width, r.height, cfg.flux_storage));
      rc = tws_set_variant(g, 0);  // the plain one-step kernel
      if (rc == TWS_OK) rc = tws_step(g, r.steps);
      if (rc == TWS_OK) rc = tws_sync(g);
      if (rc == TWS_OK) rc = tws_volume(g, &res.volume);
      if (rc == TWS_OK) {
        res.steps = r.steps;
        s->cell_steps += (double)r.width * r.height * r.steps;
      }
    }
    res.status = rc;
    res.done_s = since(t0);
    if (g) {
      if (cfg.keep_grids && rc == TWS_OK)
        res.grid = g;
      else
        tws_destroy(g);
    }
    s->results.push_back(res);
  }
  s->seconds = since(t0);
  return TWS_OK;
}

}  // namespace

extern "C" {

TWS_API int tws_server_create(const tws_server_config* cfg, tws_server** out) {
  if (!cfg || !out || !(cfg->memory_budget_bytes > 0) ||
      (cfg->flux_storage != TWS_FLUX_F32 && cfg->flux_storage != TWS_FLUX_F16))
    return TWS_ERR_INVALID;
  tws_server* s = new (std::nothrow) tws_server();
  if (!s) return TWS_ERR_OOM;
  s->cfg = *cfg;
  *out = s;
  return TWS_OK;
}

TWS_API int tws_server_destroy(tws_server* s) {
  if (!s) return TWS_ERR_INVALID;
  delete s;
  return TWS_OK;
}

TWS_API int tws_server_submit(tws_server* s, const tws_request* r) {
  if (!s || !r || !valid_request(*r)) return TWS_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->closed) return TWS_ERR_INVALID;
    s->submitted.push_back(*r);
  }
  s->cv.notify_all();
  return TWS_OK;
}

TWS_API int tws_server_close(tws_server* s) {
  if (!s) return TWS_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->closed = true;
  }
  s->cv.notify_all();
  return TWS_OK;
}

TWS_API int tws_server_run(tws_server* s, int serial) {
  if (!s) return TWS_ERR_INVALID;
  s->results.clear();
  s->cell_steps = s->seconds = s->peak_bytes = 0.0;
  s->chains = 0;
  return serial ? run_serial(s) : run_batched(s);
}

TWS_API int tws_server_result_count(tws_server* s) { return s ? (int)s->results.size() : 0; }

TWS_API int tws_server_result(tws_server* s, int i, tws_result* out) {
  if (!s || !out || i < 0 || i >= (int)s->results.size()) return TWS_ERR_INVALID;
  *out = s->results[i];
  return TWS_OK;
}

TWS_API int tws_server_stats(tws_server* s, double* cell_steps, double* seconds, double* peak_bytes,
                             uint64_t* chains) {
  if (!s) return TWS_ERR_INVALID;
  if (cell_steps) *cell_steps = s->cell_steps;
  if (seconds) *seconds = s->seconds;
  if (peak_bytes) *peak_bytes = s->peak_bytes;
  if (chains) *chains = s->chains;
  return TWS_OK;
}

}  // extern "C"
