// Serving: a request loop on one context (include/orion_gpu.h, orion_server_*).
//
// There is no serving layer in the reference; each request is one
// Integrator::render() (src/integrator/path.cpp:15-37) of a scene view.
// The worker thread repeats:
//   1. admit queued requests in arrival order while their film (and, for a
//      scene not yet resident, its BVH and shading data) fits the memory
//      budget; unreferenced resident scenes are evicted least recently used
//      first; scene uploads happen outside the server lock, so submitting
//      and polling never wait for them;
//   2. one batched launch over every running request, each advancing by
//      `spp_chunk` samples per pixel (its next sample passes), accumulating
//      into the request's own FP64 device film;
//   3. mark requests that reached their spp done.
// Requests that arrive during a launch join the next one (continuous
// batching). A request's film is the sum over its own sample passes, so it
// is the same whichever requests shared its launches.
#include <cuda_runtime.h>

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

#include "../../include/orion_gpu.h"
#include "internal.h"

using namespace orion_gb300;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  const orion_host_scene* host = nullptr;
  orion_render_params params{};
  bool has_camera = false;
  orion_camera camera{};
  orion_scene_id sid = 0;
  int width = 0, height = 0, spp = 0;
  int spp_done = 0;
  int state = ORION_REQ_QUEUED;
  void* film = nullptr;  // device: sum (W*H*3 f64) | sumsq (W*H*3 f64) | count (W*H u32)
  size_t film_bytes = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  std::string error;
};

struct Resident {
  orion_scene_id sid = 0;
  int64_t bytes = 0;
  int refs = 0;
  uint64_t last_use = 0;
};

size_t film_size(int w, int h) { return (size_t)w * h * (3 * 8 * 2 + 4); }

}  // namespace

struct orion_server {
  orion_gpu_ctx* ctx = nullptr;
  int64_t budget = 0;
  int spp_chunk = 4;
  int max_jobs = 512;
  std::mutex mu;
  std::condition_variable cv, done_cv;
  bool stop = false;
  std::thread worker;
  std::deque<Request*> queued;
  std::vector<Request*> running;
  std::map<int64_t, std::unique_ptr<Request>> reqs;
  std::map<const orion_host_scene*, Resident> resident;
  int64_t next_ticket = 1;
  uint64_t tick = 0;
  int64_t film_bytes = 0, scene_bytes = 0;
  orion_server_stats stats{};
  Clock::time_point t0 = Clock::now();

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  int64_t in_use() const { return film_bytes + scene_bytes + ctx_pool_bytes(ctx); }
};

namespace {

// Estimate of a scene's device bytes before it is uploaded (nodes, Woop
// records, primitive map, shading records).
int64_t scene_bytes_estimate(const orion_host_scene* host) {
  orion_scene_desc d;
  if (orion_scene_get_desc(host, &d) != ORION_OK) return 0;
  return d.num_prims * (64 + 48 + 4 + 96) + 4096;
}

// Frees unreferenced resident scenes, least recently used first, until
// `need` more bytes fit. Called with the server lock held; returns the scene
// ids to release (released by the caller outside the lock).
std::vector<orion_scene_id> evict_for(orion_server* s, int64_t need) {
  std::vector<orion_scene_id> out;
  while (s->in_use() + need > s->budget) {
    auto victim = s->resident.end();
    for (auto it = s->resident.begin(); it != s->resident.end(); ++it)
      if (it->second.refs == 0 && (victim == s->resident.end() || it->second.last_use < victim->second.last_use))
        victim = it;
    if (victim == s->resident.end()) break;
    s->scene_bytes -= victim->second.bytes;
    out.push_back(victim->second.sid);
    s->resident.erase(victim);
  }
  return out;
}

void fail_request(orion_server* s, Request* r, const std::string& msg) {
  r->state = ORION_REQ_FAILED;
  r->error = msg;
  r->t_done = s->now();
  s->done_cv.notify_all();
}

// Admission, in arrival order. Returns when the head request does not fit.
void admit(orion_server* s) {
  while (true) {
    Request* r;
    bool is_resident;
    int64_t need;
    std::vector<orion_scene_id> evicted;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      while (!s->queued.empty() && s->queued.front()->state != ORION_REQ_QUEUED) s->queued.pop_front();
      if (s->queued.empty() || (int)s->running.size() >= s->max_jobs) return;
      r = s->queued.front();
      auto it = s->resident.find(r->host);
      is_resident = it != s->resident.end();
      int w = r->width, h = r->height;
      if (!r->has_camera && is_resident) {
        int spp, depth;
        ctx_scene_info(s->ctx, it->second.sid, &w, &h, &spp, &depth);
      }
      need = (int64_t)film_size(std::max(w, 1), std::max(h, 1)) + (is_resident ? 0 : scene_bytes_estimate(r->host));
      if (s->in_use() + need > s->budget) evicted = evict_for(s, need);
      if (s->in_use() + need > s->budget) {
        if (s->running.empty() && s->resident.empty() && s->film_bytes == 0) {
          s->queued.pop_front();
          fail_request(s, r, "request does not fit the memory budget");
          continue;
        }
        for (orion_scene_id id : evicted) orion_gpu_scene_release(s->ctx, id);
        return;
      }
      r->state = ORION_REQ_RUNNING;  // reserved: not re-examined while its scene uploads
      s->queued.pop_front();
    }
    for (orion_scene_id id : evicted) orion_gpu_scene_release(s->ctx, id);
    orion_scene_id sid = 0;
    int64_t bytes = 0;
    int rc = ORION_OK;
    if (!is_resident) {
      rc = orion_gpu_scene_upload(s->ctx, r->host, &sid);
      if (rc == ORION_OK) orion_gpu_scene_bytes(s->ctx, sid, &bytes);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (rc != ORION_OK) {
      fail_request(s, r, std::string("scene upload failed: ") + orion_last_error());
      continue;
    }
    if (!is_resident) {
      auto it = s->resident.find(r->host);  // another admission may have uploaded it meanwhile
      if (it == s->resident.end()) {
        s->resident[r->host] = Resident{sid, bytes, 0, 0};
        s->scene_bytes += bytes;
      } else {
        orion_gpu_scene_release(s->ctx, sid);
      }
    }
    Resident& res = s->resident[r->host];
    res.refs += 1;
    res.last_use = ++s->tick;
    r->sid = res.sid;
    int w, h, spp, depth;
    ctx_scene_info(s->ctx, r->sid, &w, &h, &spp, &depth);
    if (!r->has_camera) {
      r->width = w;
      r->height = h;
    }
    r->spp = r->params.spp > 0 ? r->params.spp : spp;
    r->film_bytes = film_size(r->width, r->height);
    cudaSetDevice(ctx_device(s->ctx));
    if (cudaMalloc(&r->film, r->film_bytes) != cudaSuccess || cudaMemset(r->film, 0, r->film_bytes) != cudaSuccess) {
      if (r->film) cudaFree(r->film);
      r->film = nullptr;
      res.refs -= 1;
      fail_request(s, r, "film allocation failed");
      continue;
    }
    s->film_bytes += (int64_t)r->film_bytes;
    r->t_admit = s->now();
    if (r->state == ORION_REQ_RUNNING)
      s->running.push_back(r);
    else
      res.refs -= 1;  // cancelled while its scene was uploading
  }
}

void worker_main(orion_server* s) {
  cudaSetDevice(ctx_device(s->ctx));
  while (true) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return s->stop || !s->queued.empty() || !s->running.empty(); });
      if (s->stop) return;
    }
    admit(s);
    std::vector<Request*> batch;
    std::vector<DeviceFilmJob> jobs;
    std::vector<int> chunk;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (Request* r : s->running) {
        if (r->state != ORION_REQ_RUNNING) continue;
        DeviceFilmJob j;
        j.scene = r->sid;
        j.params = r->params;
        const int c = std::min(s->spp_chunk, r->spp - r->spp_done);
        j.params.spp = c;
        j.params.first_pass = r->params.first_pass + r->spp_done;
        j.camera = r->has_camera ? &r->camera : nullptr;
        const size_t wh = (size_t)r->width * r->height;
        j.sum = static_cast<double*>(r->film);
        j.sumsq = j.sum + 3 * wh;
        j.count = reinterpret_cast<unsigned int*>(j.sumsq + 3 * wh);
        jobs.push_back(j);
        chunk.push_back(c);
        batch.push_back(r);
      }
    }
    if (batch.empty()) {
      std::unique_lock<std::mutex> lk(s->mu);
      // Nothing admitted and nothing running: wait for a change (a release or a new request).
      s->running.erase(std::remove_if(s->running.begin(), s->running.end(),
                                      [](Request* r) { return r->state != ORION_REQ_RUNNING; }),
                       s->running.end());
      if (s->running.empty()) s->cv.wait_for(lk, std::chrono::milliseconds(20));
      continue;
    }
    double ms = 0;
    int64_t paths = 0;
    int rc = ctx_run_device_jobs(s->ctx, jobs.data(), (int)jobs.size(), &ms, &paths);
    std::string err = rc == ORION_OK ? std::string() : std::string(orion_last_error());
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.launches += 1;
    s->stats.paths += paths;
    s->stats.device_ms += ms;
    const double t = s->now();
    for (size_t i = 0; i < batch.size(); ++i) {
      Request* r = batch[i];
      if (rc != ORION_OK) {
        if (r->state == ORION_REQ_RUNNING) fail_request(s, r, "launch failed: " + err);
        continue;
      }
      r->spp_done += chunk[i];
      if (r->state == ORION_REQ_RUNNING && r->spp_done >= r->spp) {
        r->state = ORION_REQ_DONE;
        r->t_done = t;
        s->stats.completed += 1;
      }
    }
    std::vector<Request*> keep;
    for (Request* r : s->running) {
      if (r->state == ORION_REQ_RUNNING) {
        keep.push_back(r);
      } else {
        auto it = s->resident.find(r->host);
        if (it != s->resident.end()) it->second.refs -= 1;
      }
    }
    s->running.swap(keep);
    s->done_cv.notify_all();
  }
}

Request* find(orion_server* s, int64_t ticket) {
  auto it = s->reqs.find(ticket);
  return it == s->reqs.end() ? nullptr : it->second.get();
}

}  // namespace

extern "C" int orion_server_create(orion_gpu_ctx* ctx, const orion_server_opts* opts, orion_server** out) {
  if (!ctx || !out) return ctx_fail(ORION_ERR_INVALID, "null argument");
  std::unique_ptr<orion_server> s(new orion_server());
  s->ctx = ctx;
  size_t free_b = 0, total_b = 0;
  cudaSetDevice(ctx_device(ctx));
  cudaMemGetInfo(&free_b, &total_b);
  s->budget = (opts && opts->memory_budget > 0) ? opts->memory_budget : (int64_t)(free_b * 0.9);
  s->spp_chunk = (opts && opts->spp_chunk > 0) ? opts->spp_chunk : 4;
  s->max_jobs = (opts && opts->max_jobs > 0) ? opts->max_jobs : 512;
  orion_server* raw = s.get();
  s->worker = std::thread(worker_main, raw);
  *out = s.release();
  return ORION_OK;
}

extern "C" int orion_server_submit(orion_server* s, const orion_host_scene* scene, const orion_render_params* params,
                                   const orion_camera* camera, int64_t* ticket) {
  if (!s || !scene || !ticket) return ctx_fail(ORION_ERR_INVALID, "null argument");
  if (camera && (camera->width <= 0 || camera->height <= 0)) return ctx_fail(ORION_ERR_INVALID, "bad film size");
  std::unique_ptr<Request> r(new Request());
  r->host = scene;
  if (params) {
    r->params = *params;
  } else {
    r->params.max_depth = -1;
    r->params.rr_depth = 3;
  }
  if (camera) {
    r->has_camera = true;
    r->camera = *camera;
    r->width = camera->width;
    r->height = camera->height;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  r->ticket = s->next_ticket++;
  r->t_submit = s->now();
  *ticket = r->ticket;
  s->queued.push_back(r.get());
  s->reqs[r->ticket] = std::move(r);
  s->stats.submitted += 1;
  s->cv.notify_all();
  return ORION_OK;
}

extern "C" int orion_server_status(orion_server* s, int64_t ticket, orion_request_status* out) {
  if (!s || !out) return ctx_fail(ORION_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* r = find(s, ticket);
  if (!r) return ctx_fail(ORION_ERR_INVALID, "unknown ticket");
  std::memset(out, 0, sizeof(*out));
  out->state = r->state;
  out->spp_done = r->spp_done;
  out->spp_total = r->spp;
  out->width = r->width;
  out->height = r->height;
  out->t_submit = r->t_submit;
  out->t_admit = r->t_admit;
  out->t_done = r->t_done;
  return ORION_OK;
}

extern "C" int orion_server_wait(orion_server* s, int64_t ticket, double timeout_s) {
  if (!s) return ctx_fail(ORION_ERR_INVALID, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  Request* r = find(s, ticket);
  if (!r) return ctx_fail(ORION_ERR_INVALID, "unknown ticket");
  auto ready = [&] { return r->state == ORION_REQ_DONE || r->state == ORION_REQ_FAILED || r->state == ORION_REQ_CANCELLED; };
  if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
    return ctx_fail(ORION_ERR_NOT_READY, "request still running");
  if (r->state == ORION_REQ_FAILED) return ctx_fail(ORION_ERR_DEVICE, r->error.c_str());
  if (r->state == ORION_REQ_CANCELLED) return ctx_fail(ORION_ERR_CANCELLED, "request cancelled");
  return ORION_OK;
}

extern "C" int orion_server_result(orion_server* s, int64_t ticket, double* sum, double* sumsq, uint32_t* count) {
  if (!s) return ctx_fail(ORION_ERR_INVALID, "null argument");
  void* film;
  size_t wh;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    Request* r = find(s, ticket);
    if (!r) return ctx_fail(ORION_ERR_INVALID, "unknown ticket");
    if (!r->film) return ctx_fail(ORION_ERR_NOT_READY, "request not admitted yet");
    film = r->film;
    wh = (size_t)r->width * r->height;
  }
  const char* base = static_cast<const char*>(film);
  int rc = ORION_OK;
  if (sum && rc == ORION_OK) rc = ctx_copy_to_host(s->ctx, sum, base, wh * 24);
  if (sumsq && rc == ORION_OK) rc = ctx_copy_to_host(s->ctx, sumsq, base + wh * 24, wh * 24);
  if (count && rc == ORION_OK) rc = ctx_copy_to_host(s->ctx, count, base + wh * 48, wh * 4);
  return rc;
}

extern "C" int orion_server_preview(orion_server* s, int64_t ticket, uint8_t* bgra, int32_t flags) {
  if (!s || !bgra) return ctx_fail(ORION_ERR_INVALID, "null argument");
  void* film;
  int w, h;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    Request* r = find(s, ticket);
    if (!r) return ctx_fail(ORION_ERR_INVALID, "unknown ticket");
    if (!r->film) return ctx_fail(ORION_ERR_NOT_READY, "request not admitted yet");
    film = r->film;
    w = r->width;
    h = r->height;
  }
  return ctx_film_preview(s->ctx, film, w, h, (flags & ORION_PREVIEW_BOTTOM_UP) != 0, bgra);
}

extern "C" int orion_server_cancel(orion_server* s, int64_t ticket) {
  if (!s) return ctx_fail(ORION_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* r = find(s, ticket);
  if (!r) return ctx_fail(ORION_ERR_INVALID, "unknown ticket");
  if (r->state == ORION_REQ_QUEUED || r->state == ORION_REQ_RUNNING) {
    r->state = ORION_REQ_CANCELLED;
    r->t_done = s->now();
    s->done_cv.notify_all();
  }
  return ORION_OK;
}

extern "C" int orion_server_release(orion_server* s, int64_t ticket) {
  if (!s) return ctx_fail(ORION_ERR_INVALID, "null argument");
  void* film = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    Request* r = find(s, ticket);
    if (!r) return ctx_fail(ORION_ERR_INVALID, "unknown ticket");
    if (r->state == ORION_REQ_QUEUED || r->state == ORION_REQ_RUNNING)
      return ctx_fail(ORION_ERR_NOT_READY, "request still running; cancel it first");
    // A request cancelled mid-launch is still referenced by that launch.
    if (std::find(s->running.begin(), s->running.end(), r) != s->running.end())
      return ctx_fail(ORION_ERR_NOT_READY, "request is in the current launch");
    film = r->film;
    s->film_bytes -= (int64_t)r->film_bytes;
    s->reqs.erase(ticket);
  }
  if (film) {
    cudaSetDevice(ctx_device(s->ctx));
    cudaFree(film);
  }
  std::lock_guard<std::mutex> lk(s->mu);
  s->cv.notify_all();
  return ORION_OK;
}

extern "C" int orion_server_stats_get(orion_server* s, orion_server_stats* out) {
  if (!s || !out) return ctx_fail(ORION_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->resident_scenes = (int64_t)s->resident.size();
  out->bytes_in_use = s->in_use();
  return ORION_OK;
}

extern "C" int orion_server_destroy(orion_server* s) {
  if (!s) return ORION_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(ctx_device(s->ctx));
  for (auto& kv : s->reqs)
    if (kv.second->film) cudaFree(kv.second->film);
  for (auto& kv : s->resident) orion_gpu_scene_release(s->ctx, kv.second.sid);
  delete s;
  return ORION_OK;
}
