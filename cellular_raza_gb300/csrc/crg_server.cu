// crg_server.cu -- serving many simulation requests with continuous batching.
//
// chili runs one simulation per run_simulation! call (cellular_raza-core-proc-macro/src/
// run_sim.rs:411-480).  The server keeps many simulations resident on the device at once:
//   * requests are queued on submit (inputs copied) and admitted first-come first-served
//     while their estimated HBM footprint fits the budget -- counting the copy of a class's
//     running simulations that exists while its pack is rebuilt (crg_repack copies them into
//     the new pack before the old one is freed);
//   * admitted simulations join the pack of their class (agent kind, dimension, vertex count,
//     precision, solver order) through crg_repack: the running simulations keep their
//     device-resident state, the new ones are uploaded, all advance in the same launches;
//   * each simulation gets a stop step, so it freezes exactly after its requested number of
//     steps even in the middle of a tick; finished simulations are downloaded, their waiters
//     woken, and they leave the pack at the next repack;
//   * a device error raised by one simulation fails that request only;
//   * every class's pack has its own stream, and the launches of all packs for a tick are
//     enqueued before the server waits for any of them, so the classes overlap on the device.
// One background thread drives the device; submit/wait may be called from any thread.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/crg.h"
#include "crg_host.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t ticket = 0;
  crg_domain dom;
  crg_model mod;
  int64_t n = 0, steps = 0;
  std::vector<double> pos, vel;  // inputs; outputs after completion
  std::vector<uint64_t> ids;
  double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
  int64_t footprint = 0;
  bool counted = false;   // footprint counted in the server's bytes in use
  int64_t remaining = 0;  // steps left at the last repack of its pack
  int32_t status = CRG_OK;
  bool done = false;
  bool failed_in_pack = false;
  // Lifetime: the request is freed by whichever comes last, its waiter collecting it or
  // the server thread dropping it from its pack (both under the server mutex).
  bool in_pack = false;
  bool collected = false;
};

struct Class {
  crg_ctx *pack = nullptr;
  std::vector<Request *> sims;  // index in the pack -> request
  int64_t steps_since_repack = 0;
};

uint64_t class_key(const crg_domain &d, const crg_model &m) {
  return ((uint64_t)m.kind << 32) | ((uint64_t)d.dim << 24) | ((uint64_t)m.n_vertices << 16) |
         ((uint64_t)m.precision << 8) | (uint64_t)m.solver_order;
}

// Device bytes a simulation occupies in a pack: per agent the state and its "next" twin
// (positions, velocities), ids and keys (x2), FP32 offsets, the sort slot and the upload
// staging row, plus solver history; per voxel the histogram, cell starts and owner index.
int64_t footprint_bytes(const crg_domain &d, const crg_model &m, int64_t n) {
  const int nv = m.kind == CRG_KIND_ROD ? m.n_vertices : 1;
  const int64_t nc = (int64_t)nv * d.dim;
  int64_t per_agent = 4 * nc * 8 + 2 * 8 + 2 * 4 + nc * 4 + 8 + nc * 8;
  if (m.solver_order > 1) per_agent += 4 * nc * 8 + 2;
  if (m.kind == CRG_KIND_ROD)  // force buffer, pass counts and a pass list of 12 per rod
    per_agent += nc * 8 + 2 * 4 + 12 * (2 * 4 + 1 + nc * 8);
  double nvox = 1.0;
  for (int i = 0; i < d.dim; ++i) {
    double k = d.voxel_mode == 0 ? std::floor((d.max[i] - d.min[i]) / d.interaction_range)
                                 : (double)d.n_voxels[i];
    nvox *= std::max(1.0, k);
  }
  return n * per_agent + (int64_t)nvox * 12 + 4096;
}

}  // namespace

struct crg_server {
  int64_t budget = 0;
  int32_t tick = 32;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  int64_t in_use = 0;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::map<uint64_t, Class> classes;
  std::thread thread;
  int64_t n_active = 0, n_completed = 0, agent_steps = 0;
  int32_t fatal = CRG_OK;
};

namespace {

// Returns r's footprint to the budget (under the server mutex): once its state has left the
// device, i.e. when its pack dropped it or it never got into one.
void release(crg_server *s, Request *r) {
  if (r->counted) {
    s->in_use -= r->footprint;
    r->counted = false;
  }
}

void finish(crg_server *s, Request *r, int32_t status) {
  std::lock_guard<std::mutex> lk(s->mu);
  r->status = status;
  r->done = true;
  r->t_done = now_s();
  if (!r->in_pack) release(s, r);  // else its state stays on the device until it leaves
  s->n_active -= 1;
  s->n_completed += 1;
  s->cv_done.notify_all();
  s->cv_work.notify_all();
}

// The server thread drops r (it left its pack): its device memory is gone; free it if its
// waiter already collected it.
void leave_pack(crg_server *s, Request *r) {
  std::lock_guard<std::mutex> lk(s->mu);
  r->in_pack = false;
  release(s, r);
  if (r->collected) s->reqs.erase(r->ticket);
}

void leave_all(crg_server *s, Class &c) {
  for (Request *r : c.sims) leave_pack(s, r);
  c.sims.clear();
}

// Rebuilds the pack of one class: keeps the unfinished simulations, adds `incoming`.
int32_t repack(crg_server *s, Class &c, std::vector<Request *> &incoming) {
  std::vector<int32_t> keep;
  std::vector<Request *> kept;
  for (size_t k = 0; k < c.sims.size(); ++k)
    if (!c.sims[k]->done) {
      keep.push_back((int32_t)k);
      kept.push_back(c.sims[k]);
    }
  if (keep.empty() && incoming.empty()) {
    if (c.pack) crg_destroy(c.pack);
    c.pack = nullptr;
    leave_all(s, c);
    c.steps_since_repack = 0;
    return CRG_OK;
  }
  std::vector<crg_domain> doms;
  std::vector<crg_model> mods;
  std::vector<int64_t> caps, counts;
  size_t n_new_agents = 0;
  for (Request *r : incoming) {
    doms.push_back(r->dom);
    mods.push_back(r->mod);
    caps.push_back(r->n);
    counts.push_back(r->n);
    n_new_agents += (size_t)r->n;
  }
  const int nc = incoming.empty() ? 0
                                  : (incoming[0]->mod.kind == CRG_KIND_ROD ? incoming[0]->mod.n_vertices : 1) *
                                        incoming[0]->dom.dim;
  std::vector<double> pos(n_new_agents * (size_t)nc), vel(n_new_agents * (size_t)nc);
  size_t o = 0;
  for (Request *r : incoming) {
    std::memcpy(pos.data() + o, r->pos.data(), sizeof(double) * r->pos.size());
    std::memcpy(vel.data() + o, r->vel.data(), sizeof(double) * r->vel.size());
    o += r->pos.size();
  }
  crg_ctx *np = nullptr;
  int32_t rc = crg_repack(c.pack, (int32_t)keep.size(), keep.data(), (int32_t)incoming.size(),
                          doms.data(), mods.data(), caps.data(), counts.data(), pos.data(),
                          vel.data(), &np);
  if (rc != CRG_OK) return rc;
  if (c.pack) crg_destroy(c.pack);
  c.pack = np;
  for (Request *r : c.sims)
    if (r->done) leave_pack(s, r);
  c.sims.clear();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (Request *r : incoming) r->in_pack = true;
  }
  for (Request *r : incoming) {
    r->remaining = r->steps;
    c.sims.push_back(r);
  }
  for (Request *r : kept) {
    r->remaining -= c.steps_since_repack;
    c.sims.push_back(r);
  }
  c.steps_since_repack = 0;
  for (size_t k = 0; k < c.sims.size(); ++k) {
    rc = crg_set_sim_stop(c.pack, (int32_t)k, c.sims[k]->remaining);
    if (rc != CRG_OK) return rc;
  }
  return CRG_OK;
}

// Device bytes of a class's unfinished simulations: what a rebuild of its pack holds twice.
int64_t active_bytes(const Class &c) {
  int64_t b = 0;
  for (const Request *r : c.sims)
    if (!r->done) b += r->footprint;
  return b;
}

// Advances every pack by one tick.  All packs' launches are enqueued first (each pack on its
// own stream), then each is waited for; a device error of one simulation fails that request,
// which is frozen (stop step 0) and leaves at the next repack.
void tick_all(crg_server *s) {
  struct Tick {
    Class *c;
    int64_t before, target;
    int32_t rc;
  };
  std::vector<Tick> ticks;
  for (auto &kv : s->classes) {
    Class &c = kv.second;
    if (!c.pack) continue;
    Tick t{&c, 0, 0, CRG_OK};
    for (Request *r : c.sims)
      if (!r->done)
        t.before += std::max<int64_t>(0, std::min<int64_t>(s->tick, r->remaining - c.steps_since_repack)) * r->n;
    int64_t t_now = 0;
    crg_step_count(c.pack, &t_now);
    t.target = t_now + s->tick;
    t.rc = s->tick <= 256 ? crg::step_launch(c.pack, s->tick) : CRG_EINVAL;
    ticks.push_back(t);
  }
  for (Tick &t : ticks) {
    Class &c = *t.c;
    int64_t t_now = 0;
    int32_t rc = t.rc == CRG_OK ? crg::step_wait(c.pack, s->tick) : CRG_OK;
    crg_step_count(c.pack, &t_now);
    if (t.rc != CRG_OK) {  // not launched (a tick above 256 steps): step synchronously
      rc = crg_step(c.pack, t.target - t_now);
      crg_step_count(c.pack, &t_now);
    }
    bool dead = false;
    while (rc != CRG_OK) {
      int32_t sim = -1;
      const int32_t code = crg_clear_error(c.pack, &sim);
      if (sim < 0 || sim >= (int32_t)c.sims.size() || code == CRG_ECUDA ||
          code == CRG_EINTERNAL) {
        s->fatal = code;  // not attributable to one simulation
        for (Request *r : c.sims)
          if (!r->done) finish(s, r, code);
        dead = true;
        break;
      }
      Request *bad = c.sims[sim];
      if (!bad->done) finish(s, bad, code);
      crg_set_sim_stop(c.pack, sim, 0);  // freeze it; it leaves at the next repack
      if (t_now >= t.target) break;
      rc = crg_step(c.pack, t.target - t_now);
      crg_step_count(c.pack, &t_now);
    }
    if (dead) {
      crg_destroy(c.pack);
      c.pack = nullptr;
      leave_all(s, c);
      c.steps_since_repack = 0;
      continue;
    }
    c.steps_since_repack += s->tick;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->agent_steps += t.before;
    }
    // completions
    for (size_t k = 0; k < c.sims.size(); ++k) {
      Request *r = c.sims[k];
      if (r->done || c.steps_since_repack < r->remaining) continue;
      int64_t n = 0;
      const size_t len = (size_t)r->n * (r->pos.size() / std::max<int64_t>(r->n, 1));
      r->pos.assign(len, 0.0);
      r->vel.assign(len, 0.0);
      r->ids.assign((size_t)r->n, 0);
      int32_t rc2 = crg_sim_download(c.pack, (int32_t)k, &n, r->pos.data(), r->vel.data(),
                                     r->ids.data());
      finish(s, r, rc2);
    }
  }
}

void serve_loop(crg_server *s) {
  cudaSetDevice(s->device);
  for (;;) {
    std::vector<Request *> admitted;
    bool any_active = false;
    // bytes each class holds that a rebuild of its pack would copy, before this tick's
    // admissions (read on the server thread, which alone changes the packs)
    std::map<uint64_t, int64_t> dup;
    for (auto &kv : s->classes) dup[kv.first] = active_bytes(kv.second);
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop) break;
      // Admit while the resident state plus the largest rebuild copy of any class fits:
      // a class's rebuild holds its unfinished simulations twice (this tick's admissions
      // become unfinished simulations of the next rebuild).
      while (!s->queue.empty()) {
        Request *r = s->queue.front();
        const uint64_t k = class_key(r->dom, r->mod);
        int64_t worst = dup[k] + r->footprint;
        for (auto &d : dup) worst = std::max(worst, d.second);
        if (r->footprint + worst > s->budget - s->in_use) break;
        s->queue.pop_front();
        s->in_use += r->footprint;
        r->counted = true;
        dup[k] += r->footprint;
        s->n_active += 1;
        r->t_admit = now_s();
        admitted.push_back(r);
      }
      for (auto &kv : s->classes)
        if (!kv.second.sims.empty()) any_active = true;
      if (admitted.empty() && !any_active) {
        s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
    }
    // fold new simulations and drop finished ones, class by class
    std::map<uint64_t, std::vector<Request *>> by_class;
    for (Request *r : admitted) by_class[class_key(r->dom, r->mod)].push_back(r);
    for (auto &kv : s->classes) by_class.emplace(kv.first, std::vector<Request *>());
    for (auto &kv : by_class) {
      Class &c = s->classes[kv.first];
      bool finished = false;
      for (Request *r : c.sims) finished |= r->done;
      if (kv.second.empty() && !finished) continue;
      int32_t rc = repack(s, c, kv.second);
      if (rc != CRG_OK) {
        // the new simulations could not be placed: fail them, keep the class as it was
        for (Request *r : kv.second) finish(s, r, rc);
      }
    }
    tick_all(s);
  }
  for (auto &kv : s->classes) {
    if (kv.second.pack) crg_destroy(kv.second.pack);
    leave_all(s, kv.second);
  }
  s->classes.clear();
}

}  // namespace

extern "C" {

int32_t crg_server_create(int64_t hbm_budget_bytes, int32_t steps_per_tick, crg_server **out) {
  if (!out || hbm_budget_bytes <= 0 || steps_per_tick <= 0) return CRG_EINVAL;
  crg_server *s = new (std::nothrow) crg_server();
  if (!s) return CRG_ENOMEM;
  s->budget = hbm_budget_bytes;
  s->tick = steps_per_tick;
  cudaGetDevice(&s->device);
  s->thread = std::thread(serve_loop, s);
  *out = s;
  return CRG_OK;
}

int32_t crg_server_submit(crg_server *s, const crg_domain *d, const crg_model *m, int64_t n,
                          const double *pos, const double *vel, int64_t n_steps,
                          uint64_t *ticket) {
  if (!s || !d || !m || n <= 0 || !pos || !vel || n_steps < 0 || !ticket) return CRG_EINVAL;
  auto r = std::make_unique<Request>();
  r->dom = *d;
  r->mod = *m;
  r->n = n;
  r->steps = n_steps;
  const int nv = m->kind == CRG_KIND_ROD ? m->n_vertices : 1;
  const size_t len = (size_t)n * nv * d->dim;
  r->pos.assign(pos, pos + len);
  r->vel.assign(vel, vel + len);
  r->footprint = footprint_bytes(*d, *m, n);
  if (2 * r->footprint > s->budget) return CRG_ENOMEM;  // could never be admitted
  r->t_submit = now_s();
  std::lock_guard<std::mutex> lk(s->mu);
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  s->queue.push_back(r.get());
  s->reqs.emplace(r->ticket, std::move(r));
  s->cv_work.notify_all();
  return CRG_OK;
}

int32_t crg_server_wait(crg_server *s, uint64_t ticket, double timeout_s, int64_t *n,
                        double *pos, double *vel, uint64_t *ids, double *latency_s) {
  if (!s) return CRG_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second->collected) return CRG_EINVAL;
  Request *r = it->second.get();
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                            std::chrono::duration<double>(timeout_s < 0 ? 1e9 : timeout_s));
  while (!r->done)
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !r->done)
      return CRG_ETIMEDOUT;
  const int32_t status = r->status;
  if (n) *n = r->n;
  if (status == CRG_OK) {
    if (pos) std::memcpy(pos, r->pos.data(), sizeof(double) * r->pos.size());
    if (vel) std::memcpy(vel, r->vel.data(), sizeof(double) * r->vel.size());
    if (ids) std::memcpy(ids, r->ids.data(), sizeof(uint64_t) * r->ids.size());
  }
  if (latency_s) *latency_s = r->t_done - r->t_submit;
  r->collected = true;
  if (!r->in_pack) s->reqs.erase(it);  // else the server thread frees it when it drops it
  return status;
}

int32_t crg_server_stats(crg_server *s, int64_t *queued, int64_t *active, int64_t *completed,
                         int64_t *bytes_in_use, int64_t *agent_steps) {
  if (!s) return CRG_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (queued) *queued = (int64_t)s->queue.size();
  if (active) *active = s->n_active;
  if (completed) *completed = s->n_completed;
  if (bytes_in_use) *bytes_in_use = s->in_use;
  if (agent_steps) *agent_steps = s->agent_steps;
  return s->fatal;
}

int32_t crg_server_destroy(crg_server *s) {
  if (!s) return CRG_EINVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->thread.joinable()) s->thread.join();
  delete s;
  return CRG_OK;
}

}  // extern "C"
