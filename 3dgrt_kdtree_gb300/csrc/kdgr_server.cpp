// kdgr_server.cpp -- the serving form: resident scenes under an HBM budget,
// continuous batching of render requests into persistent launches.
//
// No reference counterpart: the reference renders one camera per frame call
// (cudaRenderer.cu:3099-3484).  Design:
//   * scenes are created into slots of a device scene table and count
//     against the budget together with one output arena (allocated at
//     create); a scene that would exceed the budget is refused;
//   * a request (scene, 1..N views, host output buffer) is validated at
//     submit and queued; the scheduler thread admits requests in arrival
//     order while their output fits in the arena, and launches everything
//     admitted as ONE persistent multi-scene launch on a free lane (stream);
//     a request whose buffer is page-locked host memory takes no arena
//     space: the kernel writes its frames straight into the buffer (each
//     view of a launch carries its own output base);
//     with several lanes, requests that arrive while a launch runs are
//     admitted into the next lane's launch, so their work overlaps on the
//     device (continuous batching: no fixed tick, a lane launches as soon as
//     it is free and work is queued);
//   * the completion thread waits for launches in launch order, copies the
//     frames of each arena request to its host buffer, frees the arena range
//     and wakes waiters; latency = completion - submit;
//   * every ray depends only on its own view, so a request's frames are the
//     same alone and in any mix (tests/test_serving.py checks bit equality).
// Waits on the host are bounded (kdgr_server_wait takes a timeout); the
// kernels have no inter-block waits.
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
#include <unordered_map>
#include <vector>

#include "kdgr_internal.h"
#include "scene.h"

using namespace kdgr;
using Clock = std::chrono::steady_clock;

namespace {

constexpr int kMaxSlots = kSceneSlots;
// launch-table bytes per view: its ViewDesc and its output base
constexpr size_t kTableEntry = sizeof(ViewDesc) + sizeof(float*);
static_assert(sizeof(ViewDesc) % alignof(float*) == 0, "output bases follow the views");

// First-fit allocator over the output arena (units: RGB pixels).
struct Arena {
  std::map<size_t, size_t> free_;  // offset -> length
  size_t total = 0;
  void init(size_t n) {
    total = n;
    free_.clear();
    free_[0] = n;
  }
  bool alloc(size_t n, size_t* off) {
    n = (n + 63) & ~size_t(63);  // 64-pixel granularity
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= n) {
        *off = it->first;
        const size_t rest = it->second - n, start = it->first + n;
        free_.erase(it);
        if (rest) free_[start] = rest;
        return true;
      }
    return false;
  }
  void release(size_t off, size_t n) {
    n = (n + 63) & ~size_t(63);
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

enum ReqState { kQueued, kRunning, kDone };

struct Request {
  uint64_t id = 0;
  int slot = 0;
  std::vector<kdgr_view> views;  // out_offset relative to the request
  uint64_t pixels = 0, rays = 0;
  float* host_rgb = nullptr;
  bool direct = false;      // page-locked host_rgb: the kernel writes it, no arena range
  float* out_dev = nullptr; // host_rgb's device address when direct
  size_t dev_off = 0;       // first pixel of the request in the arena
  ReqState state = kQueued;
  int status = KDGR_OK;
  bool cancel = false;
  Clock::time_point t_submit, t_launch, t_done;
};

struct Lane {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  // launch table: k views, then k output bases (float*); h_views is pinned
  ViewDesc* d_views = nullptr;
  ViewDesc* h_views = nullptr;
  uint32_t* d_queue = nullptr;
  bool busy = false;
  std::vector<Request*> reqs;
};

struct Slot {
  kdgr_scene_t scene = nullptr;
  uint64_t bytes = 0;
  int inflight = 0;  // launches in flight that reference the slot
  bool removing = false;
};

}  // namespace

struct kdgr_server_s {
  kdgr_server_config cfg{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_sched, cv_compl, cv_done;
  bool stop = false;
  Slot slots[kMaxSlots];
  SceneTable table{};  // device views of the slots' scenes (launch parameters)
  uint64_t resident = 0;
  float* d_arena = nullptr;
  Arena arena;
  uint32_t* d_status = nullptr;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  uint64_t next_id = 1;
  std::vector<Lane> lanes;
  std::deque<int> inflight;
  std::thread sched, compl_;
  // statistics
  std::vector<float> lat_ms;
  uint64_t rays_done = 0, launches = 0, views_launched = 0, max_views = 0, cancelled = 0;
  bool have_first = false;
  Clock::time_point t_first, t_last;
  int fatal = KDGR_OK;
  std::string fatal_msg;

  void scheduler();
  void completer();
};

void kdgr_server_s::scheduler() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  while (true) {
    cv_sched.wait(lk, [&] {
      if (stop) return true;
      if (queue.empty()) return false;
      for (const Lane& l : lanes)
        if (!l.busy) return true;
      return false;
    });
    if (stop) break;
    int li = -1;
    for (size_t i = 0; i < lanes.size(); ++i)
      if (!lanes[i].busy) {
        li = (int)i;
        break;
      }
    Lane& L = lanes[li];
    std::vector<Request*> admitted;
    size_t nv = 0;
    while (!queue.empty()) {
      Request* r = queue.front();
      if (r->cancel || slots[r->slot].removing) {
        queue.pop_front();
        r->state = kDone;
        r->status = KDGR_ERR_CANCELLED;
        r->t_done = Clock::now();
        ++cancelled;
        cv_done.notify_all();
        continue;
      }
      if (!admitted.empty() && nv + r->views.size() > (size_t)cfg.max_views_per_launch) break;
      size_t off = 0;
      if (!r->direct && !arena.alloc(r->pixels, &off)) break;  // arrival order: wait for space
      queue.pop_front();
      r->dev_off = off;
      r->state = kRunning;
      admitted.push_back(r);
      nv += r->views.size();
    }
    if (admitted.empty()) {
      // queue head waits for arena space: sleep until a completion frees some
      cv_sched.wait_for(lk, std::chrono::milliseconds(50));
      continue;
    }
    // view table: every view of every admitted request, blocks numbered in
    // order; output bases follow the views
    size_t nt = 0;
    for (Request* r : admitted) nt += r->views.size();
    float** h_outs = reinterpret_cast<float**>(L.h_views + nt);
    uint64_t cbase = 0;
    size_t k = 0;
    for (Request* r : admitted) {
      for (const kdgr_view& v : r->views) {
        h_outs[k] = r->direct ? r->out_dev : d_arena;
        ViewDesc& d = L.h_views[k++];
        d.cam = make_caminfo(v.cam, v.width, v.height);
        d.W = v.width;
        d.H = v.height;
        d.wt_x = 0;
        d.wt_base = 0;
        d.cb_x = (uint32_t)((v.width + 15) / 16);
        d.cb_base = (uint32_t)cbase;
        d.out_off = (r->direct ? 0 : r->dev_off) + v.out_offset;
        d.scene = (uint32_t)r->slot;
        d.pad = 0;
        cbase += (uint64_t)d.cb_x * (uint64_t)((v.height + 7) / 8);
      }
      ++slots[r->slot].inflight;
    }
    const Clock::time_point now = Clock::now();
    for (Request* r : admitted) r->t_launch = now;
    L.busy = true;
    L.reqs = std::move(admitted);
    ++launches;
    views_launched += k;
    max_views = std::max<uint64_t>(max_views, k);
    const bool packed = cfg.precision != 0;
    const SceneTable tbl = table;  // add_scene may fill another slot meanwhile
    lk.unlock();
    cudaError_t e = cudaMemcpyAsync(L.d_views, L.h_views, k * kTableEntry, cudaMemcpyHostToDevice, L.st);
    if (e == cudaSuccess) e = cudaMemsetAsync(L.d_queue, 0, kQueueBytes, L.st);
    if (e == cudaSuccess)
      e = launch_multi(tbl, packed, L.d_views, (int)k, (uint32_t)cbase,
                       reinterpret_cast<float* const*>(L.d_views + k), L.d_queue, d_status, L.st);
    if (e == cudaSuccess) e = cudaEventRecord(L.ev, L.st);
    lk.lock();
    if (e != cudaSuccess) {
      fatal = KDGR_ERR_CUDA;
      fatal_msg = std::string("serving launch: ") + cudaGetErrorString(e);
    }
    inflight.push_back(li);
    cv_compl.notify_all();
  }
}

void kdgr_server_s::completer() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  while (true) {
    cv_compl.wait(lk, [&] { return stop || !inflight.empty(); });
    if (inflight.empty()) {
      if (stop) break;
      continue;
    }
    const int li = inflight.front();
    Lane& L = lanes[li];
    lk.unlock();
    cudaError_t e = cudaEventSynchronize(L.ev);
    for (Request* r : L.reqs)
      if (e == cudaSuccess && !r->direct)
        e = cudaMemcpy(r->host_rgb, d_arena + 3 * r->dev_off, 12ull * r->pixels, cudaMemcpyDeviceToHost);
    lk.lock();
    const Clock::time_point now = Clock::now();
    for (Request* r : L.reqs) {
      if (!r->direct) arena.release(r->dev_off, r->pixels);
      --slots[r->slot].inflight;
      r->state = kDone;
      r->t_done = now;
      if (e != cudaSuccess) {
        r->status = KDGR_ERR_CUDA;
        fatal = KDGR_ERR_CUDA;
        fatal_msg = std::string("serving completion: ") + cudaGetErrorString(e);
      } else {
        r->status = KDGR_OK;
        lat_ms.push_back(std::chrono::duration<float, std::milli>(now - r->t_submit).count());
        rays_done += r->rays;
        t_last = now;
      }
    }
    L.reqs.clear();
    L.busy = false;
    inflight.pop_front();
    cv_sched.notify_all();
    cv_done.notify_all();
  }
}

static uint64_t estimate_scene_bytes(uint32_t n_nodes, uint32_t n_offsets, uint32_t n, bool packed) {
  const uint64_t per = packed ? (96 + 4) : (4 + 192);  // SH, opacity
  // ID, padded-order ID and leaf-order record (packed: plus an allowance of
  // 8 B per entry for the FP32 pairs of flagged entries, which hold about
  // 1 entry in 10 in the cluster scenes); each leaf may add one padding
  // entry.  Nodes: exact and fast trees, plus the packed form's leaf and aux
  // words.  The exact bytes are checked after creation.
  const uint64_t per_entry = 8 + (packed ? 32 + 8 : 48);
  const uint64_t per_node = packed ? 32 : 16;
  return per_node * n_nodes + per_entry * (n_offsets + n_nodes / 2 + 1) + per * n;
}

extern "C" {

void kdgr_server_config_default(kdgr_server_config* c) {
  if (!c) return;
  c->hbm_budget_bytes = 60ull << 30;
  c->arena_bytes = 2ull << 30;
  c->max_views_per_launch = 256;
  c->lanes = 2;
  c->precision = 0;
}

int kdgr_server_create(const kdgr_server_config* cfg, kdgr_server_t* out) {
  if (!out) {
    set_error("kdgr_server_create: null output handle");
    return KDGR_ERR_INVALID_ARG;
  }
  *out = nullptr;
  std::unique_ptr<kdgr_server_s> s(new kdgr_server_s);
  if (cfg) s->cfg = *cfg;
  else kdgr_server_config_default(&s->cfg);
  kdgr_server_config& c = s->cfg;
  if (c.lanes < 1 || c.lanes > 8 || c.max_views_per_launch < 1 || c.max_views_per_launch > 65536 ||
      c.arena_bytes < 4096 || c.arena_bytes > c.hbm_budget_bytes) {
    set_error("kdgr_server_create: bad config (lanes 1..8, max_views_per_launch 1..65536, "
              "4 KiB <= arena_bytes <= hbm_budget_bytes)");
    return KDGR_ERR_INVALID_ARG;
  }
  cudaGetDevice(&s->device);
  cudaError_t e = cudaMalloc(&s->d_arena, c.arena_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_status, 4);
  if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, 4);
  s->lanes.resize(c.lanes);
  for (Lane& L : s->lanes) {
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&L.d_views, kTableEntry * c.max_views_per_launch);
    if (e == cudaSuccess) e = cudaMallocHost(&L.h_views, kTableEntry * c.max_views_per_launch);
    if (e == cudaSuccess) e = cudaMalloc(&L.d_queue, kQueueBytes);
  }
  if (e != cudaSuccess) {
    kdgr_server_destroy(s.release());
    return cuda_fail(e, "kdgr_server_create");
  }
  s->arena.init(c.arena_bytes / 12);
  s->resident = c.arena_bytes;
  kdgr_server_s* raw = s.get();
  s->sched = std::thread([raw] { raw->scheduler(); });
  s->compl_ = std::thread([raw] { raw->completer(); });
  *out = s.release();
  return KDGR_OK;
}

int kdgr_server_add_scene(kdgr_server_t s, const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets,
                          uint32_t n_offsets, const float aabb[6], const float* gaussians, uint32_t n_gaussians,
                          uint32_t flags, int* slot_out) {
  if (!s || !slot_out) {
    set_error("kdgr_server_add_scene: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  DeviceScope ds(s->device);  // the scene lives on the server's device
  const bool packed = s->cfg.precision != 0;
  int slot = -1;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    const uint64_t est = estimate_scene_bytes(n_nodes, n_offsets, n_gaussians, packed);
    if (s->resident + est > s->cfg.hbm_budget_bytes) {
      set_error("kdgr_server_add_scene: scene (~" + std::to_string(est >> 20) + " MiB) exceeds the HBM budget (" +
                std::to_string((s->cfg.hbm_budget_bytes - s->resident) >> 20) + " MiB left)");
      return KDGR_ERR_BUDGET;
    }
    for (int i = 0; i < kMaxSlots; ++i)
      if (!s->slots[i].scene && !s->slots[i].removing) {
        slot = i;
        break;
      }
    if (slot < 0) {
      set_error("kdgr_server_add_scene: all 64 scene slots in use");
      return KDGR_ERR_LIMIT;
    }
    s->slots[slot].removing = true;  // reserve while uploading
  }
  kdgr_scene_t sc = nullptr;
  const uint32_t form = packed ? KDGR_FORM_PACKED : KDGR_FORM_FAST;
  int rc = kdgr_scene_create(nodes, n_nodes, offsets, n_offsets, aabb, gaussians, n_gaussians,
                             (flags & KDGR_SCALES_INVERTED) | form, &sc);
  std::lock_guard<std::mutex> lk(s->mu);
  s->slots[slot].removing = false;
  if (rc != KDGR_OK) return rc;
  kdgr_scene_info info;
  kdgr_scene_info_get(sc, &info);
  if (s->resident + info.device_bytes > s->cfg.hbm_budget_bytes) {
    kdgr_scene_destroy(sc);
    set_error("kdgr_server_add_scene: scene exceeds the HBM budget");
    return KDGR_ERR_BUDGET;
  }
  s->table.s[slot] = sc->fast_view(s->cfg.precision != 0);
  s->slots[slot].scene = sc;
  s->slots[slot].bytes = info.device_bytes;
  s->resident += info.device_bytes;
  *slot_out = slot;
  return KDGR_OK;
}

int kdgr_server_remove_scene(kdgr_server_t s, int slot) {
  if (!s || slot < 0 || slot >= kMaxSlots) {
    set_error("kdgr_server_remove_scene: bad slot");
    return KDGR_ERR_INVALID_ARG;
  }
  std::unique_lock<std::mutex> lk(s->mu);
  if (!s->slots[slot].scene) {
    set_error("kdgr_server_remove_scene: empty slot");
    return KDGR_ERR_INVALID_ARG;
  }
  s->slots[slot].removing = true;  // queued requests of the slot are cancelled
  s->cv_sched.notify_all();
  // bounded wait for launches that reference the slot
  if (!s->cv_done.wait_for(lk, std::chrono::seconds(60), [&] { return s->slots[slot].inflight == 0; })) {
    set_error("kdgr_server_remove_scene: launches still in flight after 60 s");
    return KDGR_ERR_TIMEOUT;
  }
  for (Request* r : std::vector<Request*>(s->queue.begin(), s->queue.end()))
    if (r->slot == slot) r->cancel = true;
  kdgr_scene_destroy(s->slots[slot].scene);
  s->table.s[slot] = FastView{};
  s->resident -= s->slots[slot].bytes;
  s->slots[slot] = Slot();
  s->slots[slot].removing = false;
  s->cv_sched.notify_all();
  return KDGR_OK;
}

int kdgr_server_submit(kdgr_server_t s, int slot, const kdgr_view* views, int n_views, float* host_rgb,
                       uint64_t* ticket) {
  if (!s || !views || n_views <= 0 || !host_rgb || !ticket) {
    set_error("kdgr_server_submit: null argument or no views");
    return KDGR_ERR_INVALID_ARG;
  }
  if (n_views > s->cfg.max_views_per_launch) {
    set_error("kdgr_server_submit: more views than max_views_per_launch");
    return KDGR_ERR_LIMIT;
  }
  std::unique_ptr<Request> r(new Request);
  r->views.assign(views, views + n_views);
  for (const kdgr_view& v : r->views) {
    if (v.width <= 0 || v.height <= 0) {
      set_error("kdgr_server_submit: empty view");
      return KDGR_ERR_INVALID_ARG;
    }
    r->pixels = std::max<uint64_t>(r->pixels, v.out_offset + (uint64_t)v.width * v.height);
    r->rays += (uint64_t)v.width * v.height;
  }
  {
    // page-locked from the first float to the last: written by the kernel
    DeviceScope ds(s->device);
    const float* last = host_rgb + 3 * r->pixels - 1;
    cudaPointerAttributes a{}, b{};
    if (ds.err == cudaSuccess && cudaPointerGetAttributes(&a, host_rgb) == cudaSuccess &&
        cudaPointerGetAttributes(&b, last) == cudaSuccess && a.type == cudaMemoryTypeHost &&
        b.type == cudaMemoryTypeHost && a.devicePointer &&
        (const char*)b.devicePointer - (const char*)a.devicePointer == (const char*)last - (const char*)host_rgb) {
      r->direct = true;
      r->out_dev = static_cast<float*>(a.devicePointer);
    }
    cudaGetLastError();  // a pageable pointer is not an error of this call
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->fatal != KDGR_OK) {
    set_error(s->fatal_msg);
    return s->fatal;
  }
  if (slot < 0 || slot >= kMaxSlots || !s->slots[slot].scene || s->slots[slot].removing) {
    set_error("kdgr_server_submit: no scene in slot " + std::to_string(slot));
    return KDGR_ERR_INVALID_ARG;
  }
  if (!r->direct && ((r->pixels + 63) & ~uint64_t(63)) > s->arena.total) {
    set_error("kdgr_server_submit: request output exceeds the arena (HBM budget)");
    return KDGR_ERR_BUDGET;
  }
  r->id = s->next_id++;
  r->slot = slot;
  r->host_rgb = host_rgb;
  r->t_submit = Clock::now();
  if (!s->have_first) {
    s->have_first = true;
    s->t_first = r->t_submit;
  }
  *ticket = r->id;
  s->queue.push_back(r.get());
  s->reqs[r->id] = std::move(r);
  s->cv_sched.notify_all();
  return KDGR_OK;
}

int kdgr_server_wait(kdgr_server_t s, uint64_t ticket, int timeout_ms, kdgr_request_stats* st) {
  if (!s) return KDGR_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    set_error("kdgr_server_wait: unknown ticket");
    return KDGR_ERR_INVALID_ARG;
  }
  Request* r = it->second.get();
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                           [&] { return r->state == kDone; })) {
    set_error("kdgr_server_wait: request not finished within the timeout");
    return KDGR_ERR_TIMEOUT;
  }
  if (st) {
    st->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    st->queue_ms = r->status == KDGR_OK ? std::chrono::duration<double, std::milli>(r->t_launch - r->t_submit).count()
                                        : st->latency_ms;
    st->rays = r->rays;
  }
  const int status = r->status;
  s->reqs.erase(it);
  return status;
}

int kdgr_server_cancel(kdgr_server_t s, uint64_t ticket) {
  if (!s) return KDGR_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    set_error("kdgr_server_cancel: unknown ticket");
    return KDGR_ERR_INVALID_ARG;
  }
  Request* r = it->second.get();
  if (r->state != kQueued) {
    set_error("kdgr_server_cancel: request already launched");
    return KDGR_ERR_INVALID_ARG;
  }
  s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
  r->state = kDone;
  r->status = KDGR_ERR_CANCELLED;
  r->t_done = Clock::now();
  ++s->cancelled;
  s->cv_done.notify_all();
  return KDGR_OK;
}

int kdgr_server_stats_get(kdgr_server_t s, kdgr_server_stats* out) {
  if (!s || !out) return KDGR_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  memset(out, 0, sizeof(*out));
  std::vector<float> l = s->lat_ms;
  out->completed = l.size();
  out->cancelled = s->cancelled;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return (double)l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = l.back();
    double sum = 0;
    for (float x : l) sum += x;
    out->mean_ms = sum / l.size();
  }
  if (s->have_first && s->rays_done) {
    const double secs = std::chrono::duration<double>(s->t_last - s->t_first).count();
    out->mrays_per_s = secs > 0 ? s->rays_done / secs / 1e6 : 0;
  }
  out->rays = s->rays_done;
  out->launches = s->launches;
  out->views_launched = s->views_launched;
  out->max_views_per_launch = s->max_views;
  out->resident_bytes = s->resident;
  out->queued = s->queue.size();
  return KDGR_OK;
}

int kdgr_server_reset_stats(kdgr_server_t s) {
  if (!s) return KDGR_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->lat_ms.clear();
  s->rays_done = s->launches = s->views_launched = s->max_views = s->cancelled = 0;
  s->have_first = false;
  return KDGR_OK;
}

int kdgr_server_destroy(kdgr_server_t s) {
  if (!s) return KDGR_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (Request* r : s->queue) {
      r->state = kDone;
      r->status = KDGR_ERR_CANCELLED;
    }
    s->queue.clear();
    s->cv_sched.notify_all();
    s->cv_compl.notify_all();
    s->cv_done.notify_all();
  }
  if (s->sched.joinable()) s->sched.join();
  if (s->compl_.joinable()) s->compl_.join();
  DeviceScope ds(s->device);
  for (Lane& L : s->lanes) {
    if (L.st) cudaStreamSynchronize(L.st);
    if (L.st) cudaStreamDestroy(L.st);
    if (L.ev) cudaEventDestroy(L.ev);
    if (L.d_views) cudaFree(L.d_views);
    if (L.h_views) cudaFreeHost(L.h_views);
    if (L.d_queue) cudaFree(L.d_queue);
  }
  for (Slot& sl : s->slots)
    if (sl.scene) kdgr_scene_destroy(sl.scene);
  if (s->d_arena) cudaFree(s->d_arena);
  if (s->d_status) cudaFree(s->d_status);
  delete s;
  return KDGR_OK;
}

}  // extern "C"
