// Serving loop (vs_server_* in include/vs.h): frames from many sessions as
// they arrive, continuous batching, admission by HBM budget.
//
// Threads.  The caller's threads submit frames: a frame is copied into the
// session's pinned ring (queue_depth frames) and stamped with its arrival
// time.  A worker thread forms a step from the sessions that have a frame not
// yet launched (round robin, one frame per session, at most max_batch) and
// launches it through a batch runner.  There are `lanes` runners, each on its
// own stream with its own completion thread: steps of different lanes run on
// the GPU at the same time, so one step's latency-bound phases (ICP closes,
// kernel tails) overlap another step's work.  A lane keeps up to `pipeline`
// steps in flight, so the host prepares and enqueues step k+1 while step k
// runs.  A lane's completion thread waits for its steps in order, stamps each
// frame's result, releases its ring slot and retires closed sessions.
//
// Ring of a session: frames [head, sent) are on the GPU, [sent, tail) wait
// for a step, slots of frames before head are free.  A session's frames run
// in submission order: with one lane its frame k+1 can only join a step
// launched after the step holding frame k, on the same stream; with several
// lanes a session joins a step only when none of its frames is in flight.
//
// Admission.  A session is resident (volume, pose, pyramid and maps on the
// device) while it is open.  It is admitted when a resident slot is free and
// its vs_session_bytes fit the budget next to the resident ones; otherwise it
// waits in FIFO order (a later, smaller session may pass a waiting larger
// one), buffering frames, and is admitted when a closed session frees memory.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "vs.h"
#include "vs_host.h"
#include "vs_internal.cuh"

using namespace vs;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct SrvSession {
  int id = 0;
  vs_config cfg;
  size_t bytes = 0;
  int state = VS_SESSION_WAITING;
  bool admitting = false;
  bool closing = false;
  vs_session* sess = nullptr;
  size_t frame_px = 0;
  uint16_t* staging = nullptr;   // pinned, queue_depth frames
  std::vector<double> t_submit;  // per ring slot
  uint64_t head = 0, sent = 0, tail = 0;
};

constexpr int kMaxLanes = 4;

struct StepRec {
  int ring = 0;
  int n = 0;
  int ids[kMaxSlots];
  uint64_t frame[kMaxSlots];
  double t_sub[kMaxSlots];
};

}  // namespace

struct vs_server {
  vs_server_config cfg;
  int device = 0;
  vs_batch* batch[kMaxLanes] = {};
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_res;
  std::map<int, SrvSession*> sessions;
  std::deque<int> waiting;
  std::deque<StepRec> inflight[kMaxLanes];
  std::deque<vs_result> results;
  int next_id = 0;
  int rr = 0;
  size_t bytes_resident = 0;
  int resident = 0, closed = 0;
  uint64_t steps = 0, frames = 0, batch_sum = 0;
  int max_batch_seen = 0;
  uint64_t submitted_resident = 0, completed = 0;
  bool stop = false;
  int error = 0;
  std::string error_msg;
  std::thread worker, completer[kMaxLanes];
};

namespace {

int server_error(vs_server* s) {
  if (s->error) fail_code(s->error, s->error_msg);
  return s->error;
}

void set_server_error(vs_server* s, int code, const std::string& m) {
  if (!s->error) {
    s->error = code;
    s->error_msg = m;
  }
  s->cv_work.notify_all();
  s->cv_done.notify_all();
  s->cv_res.notify_all();
}

bool fits(const vs_server* s, const SrvSession* r) {
  return s->resident < s->cfg.max_resident && s->bytes_resident + r->bytes <= s->cfg.hbm_budget;
}

// Admits waiting sessions that fit; creation runs with the lock released.
// Returns with the lock held.
void admit(vs_server* s, std::unique_lock<std::mutex>& lk) {
  for (;;) {
    SrvSession* pick = nullptr;
    for (auto it = s->waiting.begin(); it != s->waiting.end(); ++it) {
      SrvSession* r = s->sessions[*it];
      if (fits(s, r)) {
        pick = r;
        s->waiting.erase(it);
        break;
      }
    }
    if (!pick) return;
    pick->admitting = true;
    s->resident += 1;
    s->bytes_resident += pick->bytes;
    lk.unlock();
    vs_session* sess = nullptr;
    int rc = vs_session_create(&pick->cfg, &sess);
    std::string msg = rc ? vs_last_error() : "";
    lk.lock();
    pick->admitting = false;
    if (rc) {
      s->resident -= 1;
      s->bytes_resident -= pick->bytes;
      set_server_error(s, rc, "admitting session " + std::to_string(pick->id) + ": " + msg);
      return;
    }
    pick->sess = sess;
    pick->state = VS_SESSION_RESIDENT;
    s->submitted_resident += pick->tail - pick->head;
    s->cv_work.notify_all();
  }
}

bool any_admissible(const vs_server* s) {
  for (int id : s->waiting) {
    auto it = s->sessions.find(id);
    if (it != s->sessions.end() && fits(s, it->second)) return true;
  }
  return false;
}

// a frame the worker may put into a step: waiting, and with several lanes
// none of the session's frames still in flight
bool ready(const vs_server* s, const SrvSession* r) {
  return r->state == VS_SESSION_RESIDENT && r->sent < r->tail && (s->cfg.lanes == 1 || r->sent == r->head);
}

bool any_ready(const vs_server* s) {
  for (const auto& kv : s->sessions)
    if (ready(s, kv.second)) return true;
  return false;
}

// the lane with the fewest steps in flight, or -1 when every lane is full
int free_lane(const vs_server* s) {
  int best = -1;
  for (int l = 0; l < s->cfg.lanes; l++)
    if ((int)s->inflight[l].size() < s->cfg.pipeline && (best < 0 || s->inflight[l].size() < s->inflight[best].size()))
      best = l;
  return best;
}

void worker_main(vs_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  std::vector<SrvSession*> order;
  for (;;) {
    admit(s, lk);
    s->cv_work.wait(lk, [&] {
      return s->stop || s->error || any_admissible(s) || (free_lane(s) >= 0 && any_ready(s));
    });
    if (s->stop || s->error) return;
    const int lane = free_lane(s);
    if (lane < 0 || !any_ready(s)) continue;
    // round robin over the resident sessions, one frame each
    order.clear();
    for (const auto& kv : s->sessions) order.push_back(kv.second);
    StepRec rec;
    vs_session* ss[kMaxSlots];
    const uint16_t* fp[kMaxSlots];
    const int m = (int)order.size();
    int last = s->rr;
    for (int j = 0; j < m && rec.n < s->cfg.max_batch; j++) {
      const int idx = (s->rr + j) % m;
      SrvSession* r = order[idx];
      if (!ready(s, r)) continue;
      const size_t slot = r->sent % (uint64_t)s->cfg.queue_depth;
      rec.ids[rec.n] = r->id;
      rec.frame[rec.n] = r->sent;
      rec.t_sub[rec.n] = r->t_submit[slot];
      ss[rec.n] = r->sess;
      fp[rec.n] = r->staging + slot * r->frame_px;
      r->sent += 1;
      rec.n += 1;
      last = idx + 1;
    }
    s->rr = m ? last % m : 0;
    lk.unlock();
    int ring = 0;
    const int rc = batch_launch_host(s->batch[lane], ss, rec.n, fp, &ring);
    const std::string msg = rc ? vs_last_error() : "";
    lk.lock();
    if (rc) {
      set_server_error(s, rc, "step launch: " + msg);
      return;
    }
    rec.ring = ring;
    s->inflight[lane].push_back(rec);
    s->steps += 1;
    s->batch_sum += rec.n;
    if (rec.n > s->max_batch_seen) s->max_batch_seen = rec.n;
    s->cv_done.notify_all();
  }
}

void retire(vs_server* s, SrvSession* r, std::unique_lock<std::mutex>& lk) {
  // called with the lock held for a closing session whose frames are done
  vs_session* sess = r->sess;
  r->sess = nullptr;
  r->state = VS_SESSION_CLOSED;
  lk.unlock();
  if (sess) vs_session_destroy(sess);
  lk.lock();
  s->resident -= 1;
  s->bytes_resident -= r->bytes;
  s->closed += 1;
  s->cv_work.notify_all();
}

void completer_main(vs_server* s, int lane) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  std::deque<StepRec>& q = s->inflight[lane];
  for (;;) {
    s->cv_done.wait(lk, [&] { return s->stop || s->error || !q.empty(); });
    if (q.empty() || s->error) {
      if (s->stop || s->error) return;
      continue;
    }
    const StepRec rec = q.front();
    lk.unlock();
    const cudaError_t e = cudaEventSynchronize(batch_done(s->batch[lane], rec.ring));
    const double t = now_s();
    std::vector<vs_result> out(rec.n);
    const unsigned char* heads = batch_heads(s->batch[lane], rec.ring);
    for (int i = 0; i < rec.n; i++) {
      const Pose* p = reinterpret_cast<const Pose*>(heads + (size_t)i * kPoseHeadBytes);
      vs_result& o = out[i];
      o.session = rec.ids[i];
      o.frame = (int)rec.frame[i];
      o.tracked = p->tracked;
      o.batch = rec.n;
      std::memcpy(o.T_gc, p->Tgc, sizeof(o.T_gc));
      o.t_submit = rec.t_sub[i];
      o.t_done = t;
      o.latency_ms = 1000.0 * (t - rec.t_sub[i]);
    }
    lk.lock();
    if (e != cudaSuccess) {
      set_server_error(s, VS_ERR_CUDA, std::string("step: ") + cudaGetErrorString(e));
      return;
    }
    q.pop_front();
    for (int i = 0; i < rec.n; i++) {
      SrvSession* r = s->sessions[rec.ids[i]];
      r->head += 1;
      s->results.push_back(out[i]);
    }
    s->completed += rec.n;
    s->frames += rec.n;
    for (int i = 0; i < rec.n; i++) {
      SrvSession* r = s->sessions[rec.ids[i]];
      if (r->closing && r->state == VS_SESSION_RESIDENT && r->head == r->tail) retire(s, r, lk);
    }
    s->cv_work.notify_all();
    s->cv_res.notify_all();
  }
}

void free_record(SrvSession* r) {
  if (r->sess) vs_session_destroy(r->sess);
  if (r->staging) cudaFreeHost(r->staging);
  delete r;
}

}  // namespace

extern "C" {

double vs_server_clock(void) { return now_s(); }

void vs_server_config_default(vs_server_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->hbm_budget = (size_t)150 << 30;
  c->max_resident = kMaxSlots;
  c->max_batch = kMaxSlots;
  c->queue_depth = 8;
  c->pipeline = 1;
  c->lanes = 3;
}

int vs_server_create(const vs_server_config* c, vs_server** out) {
  if (!out) return fail_code(VS_ERR_ARG, "null output");
  *out = nullptr;
  vs_server_config k;
  vs_server_config_default(&k);
  if (c) {
    if (c->hbm_budget) k.hbm_budget = c->hbm_budget;
    if (c->max_resident) k.max_resident = c->max_resident;
    if (c->max_batch) k.max_batch = c->max_batch;
    if (c->queue_depth) k.queue_depth = c->queue_depth;
    if (c->pipeline) k.pipeline = c->pipeline;
    if (c->lanes) k.lanes = c->lanes;
  }
  if (k.max_resident < 1 || k.max_resident > kMaxSlots || k.max_batch < 1 || k.max_batch > kMaxSlots ||
      k.queue_depth < 1 || k.queue_depth > 256 || k.pipeline < 1 || k.pipeline > 2 || k.lanes < 1 ||
      k.lanes > kMaxLanes)
    return fail_code(VS_ERR_ARG, "server config out of range");
  vs_server* s = new vs_server;
  s->cfg = k;
  cudaGetDevice(&s->device);
  for (int l = 0; l < k.lanes; l++) {
    const int rc = vs_batch_create(&s->batch[l]);
    if (rc) {
      for (int m = 0; m < l; m++) vs_batch_destroy(s->batch[m]);
      delete s;
      return rc;
    }
  }
  s->worker = std::thread(worker_main, s);
  for (int l = 0; l < k.lanes; l++) s->completer[l] = std::thread(completer_main, s, l);
  *out = s;
  return VS_OK;
}

int vs_server_open(vs_server* s, const vs_config* cfg, int* id) {
  if (!s || !cfg || !id) return fail_code(VS_ERR_ARG, "null argument");
  const size_t bytes = vs_session_bytes(cfg);
  if (!bytes) return fail_code(VS_ERR_ARG, std::string("bad session config: ") + vs_last_error());
  if (bytes > s->cfg.hbm_budget)
    return fail_code(VS_ERR_MEMORY, "session needs " + std::to_string(bytes) + " bytes, more than the budget");
  SrvSession* r = new SrvSession;
  r->cfg = *cfg;
  r->bytes = bytes;
  r->frame_px = (size_t)cfg->width * cfg->height;
  r->t_submit.assign(s->cfg.queue_depth, 0.0);
  cudaError_t e = cudaMallocHost(&r->staging, r->frame_px * 2 * s->cfg.queue_depth);
  if (e != cudaSuccess) {
    delete r;
    return cuda_fail_code(e, "frame staging");
  }
  {
    std::unique_lock<std::mutex> lk(s->mu);
    int err = server_error(s);
    if (err) {
      lk.unlock();
      free_record(r);
      return err;
    }
    r->id = s->next_id++;
    s->sessions[r->id] = r;
    s->waiting.push_back(r->id);
    *id = r->id;
    admit(s, lk);
    err = server_error(s);
    if (err) return err;
  }
  return VS_OK;
}

int vs_server_state(vs_server* s, int id, int* state) {
  if (!s || !state) return fail_code(VS_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->sessions.find(id);
  if (it == s->sessions.end()) return fail_code(VS_ERR_ARG, "unknown session id");
  *state = it->second->state;
  return VS_OK;
}

int vs_server_submit(vs_server* s, int id, const uint16_t* depth_mm_host) {
  if (!s || !depth_mm_host) return fail_code(VS_ERR_ARG, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  int err = server_error(s);
  if (err) return err;
  auto it = s->sessions.find(id);
  if (it == s->sessions.end()) return fail_code(VS_ERR_ARG, "unknown session id");
  SrvSession* r = it->second;
  if (r->closing || r->state == VS_SESSION_CLOSED) return fail_code(VS_ERR_STATE, "session is closed");
  if (r->tail - r->head >= (uint64_t)s->cfg.queue_depth) return fail_code(VS_ERR_BUSY, "session queue full");
  const size_t slot = r->tail % (uint64_t)s->cfg.queue_depth;
  // the slot's earlier frame has finished and nothing reads slots at or past
  // tail, so the copy runs without the lock (one submitting thread per session)
  const double t = now_s();
  lk.unlock();
  std::memcpy(r->staging + slot * r->frame_px, depth_mm_host, r->frame_px * 2);
  lk.lock();
  r->t_submit[slot] = t;
  r->tail += 1;
  if (r->state == VS_SESSION_RESIDENT) s->submitted_resident += 1;
  s->cv_work.notify_all();
  return VS_OK;
}

int vs_server_close(vs_server* s, int id) {
  if (!s) return fail_code(VS_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->sessions.find(id);
  if (it == s->sessions.end()) return fail_code(VS_ERR_ARG, "unknown session id");
  SrvSession* r = it->second;
  if (r->closing || r->state == VS_SESSION_CLOSED) return VS_OK;
  r->closing = true;
  if (r->state == VS_SESSION_WAITING && !r->admitting) {
    for (auto w = s->waiting.begin(); w != s->waiting.end(); ++w)
      if (*w == id) {
        s->waiting.erase(w);
        break;
      }
    r->state = VS_SESSION_CLOSED;
    s->closed += 1;
    return VS_OK;
  }
  if (r->state == VS_SESSION_RESIDENT && r->head == r->tail) retire(s, r, lk);
  return server_error(s);
}

int vs_server_poll(vs_server* s, vs_result* out, int max, int timeout_ms) {
  if (!s || (!out && max > 0)) return fail_code(VS_ERR_ARG, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->results.empty() && timeout_ms > 0)
    s->cv_res.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !s->results.empty() || s->error; });
  int n = 0;
  while (n < max && !s->results.empty()) {
    out[n++] = s->results.front();
    s->results.pop_front();
  }
  if (n == 0) {
    int err = server_error(s);
    if (err) return err;
  }
  return n;
}

int vs_server_drain(vs_server* s) {
  if (!s) return fail_code(VS_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_res.wait(lk, [&] { return s->error || s->completed >= s->submitted_resident; });
  return server_error(s);
}

int vs_server_get_session(vs_server* s, int id, vs_session** out) {
  if (!s || !out) return fail_code(VS_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->sessions.find(id);
  if (it == s->sessions.end() || it->second->state != VS_SESSION_RESIDENT)
    return fail_code(VS_ERR_STATE, "session is not resident");
  *out = it->second->sess;
  return VS_OK;
}

int vs_server_get_stats(vs_server* s, vs_server_stats* st) {
  if (!s || !st) return fail_code(VS_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(st, 0, sizeof(*st));
  st->steps = s->steps;
  st->frames = s->frames;
  st->mean_batch = s->steps ? (double)s->batch_sum / (double)s->steps : 0.0;
  st->max_batch_seen = s->max_batch_seen;
  st->resident = s->resident;
  st->waiting = (int)s->waiting.size();
  st->closed = s->closed;
  st->bytes_resident = s->bytes_resident;
  st->bytes_budget = s->cfg.hbm_budget;
  return VS_OK;
}

int vs_server_destroy(vs_server* s) {
  if (!s) return VS_OK;
  vs_server_drain(s);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_done.notify_all();
  s->cv_res.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (int l = 0; l < s->cfg.lanes; l++)
    if (s->completer[l].joinable()) s->completer[l].join();
  for (int l = 0; l < s->cfg.lanes; l++) vs_batch_sync(s->batch[l]);
  for (auto& kv : s->sessions) free_record(kv.second);
  s->sessions.clear();
  for (int l = 0; l < s->cfg.lanes; l++) vs_batch_destroy(s->batch[l]);
  delete s;
  return VS_OK;
}

}  // extern "C"
