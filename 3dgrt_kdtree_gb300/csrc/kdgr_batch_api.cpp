// kdgr_batch_api.cpp -- C ABI of the batching form: one-shot batches,
// CUDA-graph-captured batches and the autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kdgr_internal.h"
#include "scene.h"

using namespace kdgr;

struct kdgr_batch_s {
  kdgr_scene_t scene = nullptr;
  kdgr_batch_config cfg{};
  ViewDesc* d_views = nullptr;
  uint32_t* d_queue = nullptr;
  int n_views = 0;
  uint32_t totals[3] = {0, 0, 0};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

int batch_args(kdgr_scene_t s, const kdgr_view* views, int n_views, float* rgb, const kdgr_batch_config* cfg,
               kdgr_batch_config& c, const char* who) {
  if (!s || !views || n_views <= 0 || !rgb) {
    set_error(std::string(who) + ": null scene/views/output or no views");
    return KDGR_ERR_INVALID_ARG;
  }
  if (cfg) c = *cfg;
  else kdgr_batch_config_default(&c);
  int rc = check_batch_config(s, c);
  if (rc != KDGR_OK) set_error(std::string(who) + ": " + kdgr_last_error());
  return rc;
}

// The library's stream-ordered memory pool on the current device, created
// on first use.  Its release threshold keeps freed scratch mapped between
// calls: the device's default pool (shared with the application, so its
// attributes stay untouched) hands memory back at every synchronisation by
// default, and mapping it again cost about 0.1 ms per call.
cudaError_t scratch_pool(cudaMemPool_t* out) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return e;
    }
    pools[dev] = pool;
  }
  *out = pools[dev];
  return cudaSuccess;
}

// Stream-ordered scratch for one launch: view table + queue counter, from
// the library's pool; the table travels in a staging kernel's parameters
// (up to 256 views) or by one copy.
int run_once(kdgr_scene_t s, const kdgr_batch_config& c, const std::vector<ViewDesc>& table,
             const uint32_t totals[3], float* rgb, float* alpha, float* depth, cudaStream_t st, const char* who) {
  const size_t vbytes = table.size() * sizeof(ViewDesc);
  cudaMemPool_t pool = nullptr;
  cudaError_t e = scratch_pool(&pool);
  if (e != cudaSuccess) return cuda_fail(e, who);
  void* scratch = nullptr;
  e = cudaMallocFromPoolAsync(&scratch, ((vbytes + 127) & ~size_t(127)) + kQueueBytes, pool, st);
  if (e != cudaSuccess) return cuda_fail(e, who);
  ViewDesc* d_views = static_cast<ViewDesc*>(scratch);
  uint32_t* d_queue = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + ((vbytes + 127) & ~size_t(127)));
  e = stage_views(table.data(), (int)table.size(), d_views, d_queue, st);
  if (e == cudaSuccess)
    e = launch_batch(s, c, d_views, (int)table.size(), totals, rgb, alpha, depth, d_queue, st);
  const cudaError_t ef = cudaFreeAsync(scratch, st);
  if (e == cudaSuccess) e = ef;
  if (e != cudaSuccess) return cuda_fail(e, who);
  return KDGR_OK;
}

}  // namespace

extern "C" {

void kdgr_batch_config_default(kdgr_batch_config* c) {
  if (!c) return;
  // SM strips, 64 registers (8 CTAs per SM), warp packets: the autotuner's
  // pick on GB300 for one 1080p view, 64 mixed views and the 3M scene
  c->schedule = KDGR_SCHED_SM_STRIPS;
  c->min_blocks = 8;
  c->blocks_per_sm = 0;
  c->chunk = 1;
  c->precision = 0;
  c->hit_buffer = 4;
  c->traversal = KDGR_TRAV_PACKET;
  c->tile_shape = KDGR_TILE_8X4;
  c->rays_per_warp = 32;
}

int kdgr_render_batch(kdgr_scene_t s, const kdgr_view* views, int n_views, float* rgb, float* alpha, float* depth,
                      const kdgr_batch_config* cfg, void* stream, float* ms_out) {
  kdgr_batch_config c;
  int rc = batch_args(s, views, n_views, rgb, cfg, c, "kdgr_render_batch");
  if (rc != KDGR_OK) return rc;
  std::vector<ViewDesc> table;
  uint32_t totals[3] = {0, 0, 0};
  rc = make_view_table(views, n_views, table, totals);
  if (rc != KDGR_OK) return rc;
  DeviceScope on(s->device);
  if (on.err != cudaSuccess) return cuda_fail(on.err, "kdgr_render_batch");
  const cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ms_out) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
  }
  rc = run_once(s, c, table, totals, rgb, alpha, depth, st, "kdgr_render_batch");
  if (ms_out) {
    cudaEventRecord(e1, st);
    const cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *ms_out = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == KDGR_OK && e != cudaSuccess) rc = cuda_fail(e, "kdgr_render_batch");
  }
  return rc;
}

int kdgr_render_fast(kdgr_scene_t s, const kdgr_camera* cam, int width, int height, float* rgb, float* alpha,
                     float* depth, int precision, void* stream, float* ms_out) {
  if (!cam) {
    set_error("kdgr_render_fast: null camera");
    return KDGR_ERR_INVALID_ARG;
  }
  kdgr_view v;
  v.cam = *cam;
  v.width = width;
  v.height = height;
  v.out_offset = 0;
  kdgr_batch_config c;
  kdgr_batch_config_default(&c);
  c.precision = precision ? 1 : 0;
  return kdgr_render_batch(s, &v, 1, rgb, alpha, depth, &c, stream, ms_out);
}

int kdgr_batch_create(kdgr_scene_t s, const kdgr_view* views, int n_views, float* rgb, float* alpha, float* depth,
                      const kdgr_batch_config* cfg, kdgr_batch_t* out) {
  if (!out) {
    set_error("kdgr_batch_create: null output handle");
    return KDGR_ERR_INVALID_ARG;
  }
  *out = nullptr;
  kdgr_batch_config c;
  int rc = batch_args(s, views, n_views, rgb, cfg, c, "kdgr_batch_create");
  if (rc != KDGR_OK) return rc;
  std::vector<ViewDesc> table;
  uint32_t totals[3] = {0, 0, 0};
  rc = make_view_table(views, n_views, table, totals);
  if (rc != KDGR_OK) return rc;
  DeviceScope on(s->device);
  if (on.err != cudaSuccess) return cuda_fail(on.err, "kdgr_batch_create");
  kdgr_batch_s* b = new kdgr_batch_s;
  b->scene = s;
  b->cfg = c;
  b->n_views = n_views;
  for (int i = 0; i < 3; ++i) b->totals[i] = totals[i];
  cudaStream_t cap = nullptr;
  cudaError_t e = cudaMalloc(&b->d_views, table.size() * sizeof(ViewDesc));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_queue, kQueueBytes);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_views, table.data(), table.size() * sizeof(ViewDesc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t le = cudaMemsetAsync(b->d_queue, 0, kQueueBytes, cap);
    if (le == cudaSuccess)
      le = launch_batch(s, c, b->d_views, n_views, totals, rgb, alpha, depth, b->d_queue, cap);
    e = cudaStreamEndCapture(cap, &b->graph);
    if (e == cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (cap) cudaStreamDestroy(cap);
  if (e != cudaSuccess) {
    kdgr_batch_destroy(b);
    return cuda_fail(e, "kdgr_batch_create");
  }
  *out = b;
  return KDGR_OK;
}

int kdgr_batch_run(kdgr_batch_t b, void* stream) {
  if (!b || !b->exec) {
    set_error("kdgr_batch_run: invalid batch");
    return KDGR_ERR_INVALID_ARG;
  }
  DeviceScope on(b->scene->device);
  cudaError_t e = on.err;
  if (e == cudaSuccess) e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_batch_run");
  return KDGR_OK;
}

int kdgr_batch_destroy(kdgr_batch_t b) {
  if (!b) return KDGR_ERR_INVALID_ARG;
  DeviceScope on(b->scene->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->d_views) cudaFree(b->d_views);
  if (b->d_queue) cudaFree(b->d_queue);
  delete b;
  return KDGR_OK;
}

int kdgr_autotune(kdgr_scene_t s, const kdgr_view* views, int n_views, int precision, float* rgb,
                  kdgr_batch_config* best, char* report, int report_len) {
  if (!best) {
    set_error("kdgr_autotune: null output config");
    return KDGR_ERR_INVALID_ARG;
  }
  kdgr_batch_config base;
  kdgr_batch_config_default(&base);
  base.precision = precision ? 1 : 0;
  int rc = batch_args(s, views, n_views, rgb, &base, base, "kdgr_autotune");
  if (rc != KDGR_OK) return rc;
  std::vector<ViewDesc> table;
  uint32_t totals[3] = {0, 0, 0};
  rc = make_view_table(views, n_views, table, totals);
  if (rc != KDGR_OK) return rc;
  DeviceScope on(s->device);
  if (on.err != cudaSuccess) return cuda_fail(on.err, "kdgr_autotune");
  std::vector<kdgr_batch_config> cands;
  for (int minb : {0, 6, 8})
    for (int sched : {KDGR_SCHED_WARP_TILES, KDGR_SCHED_CTA_BLOCKS, KDGR_SCHED_SM_STRIPS, KDGR_SCHED_WARP_STRIPS})
      for (int chunk : {1, 2}) {
        // strips take one item per claim
        if ((sched == KDGR_SCHED_SM_STRIPS || sched == KDGR_SCHED_WARP_STRIPS) && chunk != 1) continue;
        kdgr_batch_config c = base;
        c.min_blocks = minb;
        c.schedule = sched;
        c.chunk = chunk;
        c.blocks_per_sm = 0;
        cands.push_back(c);
      }
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_autotune");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::string rep;
  float best_ms = 1e30f;
  // stage 1: schedule x register cap x chunk with warp packets, 8x4 tiles
  // and the 4-entry hit buffer; stage 2: the winner with the 8-entry buffer
  // (dense leaves re-scan less), with per-ray traversal, with 4x8 and 16x2
  // warp tiles, and with 16 or 8 rays per warp (either traversal)
  bool stage2 = false;
  for (size_t ci = 0; ci < cands.size() || !stage2; ++ci) {
    if (ci == cands.size()) {  // reached once: appends the stage-2 candidates
      stage2 = true;
      if (rc != KDGR_OK || best_ms >= 1e30f) break;
      kdgr_batch_config c8 = *best, cr = *best;
      c8.hit_buffer = 8;
      cr.traversal = KDGR_TRAV_RAY;
      cands.push_back(c8);
      cands.push_back(cr);
      if (best->schedule != KDGR_SCHED_WARP_TILES)
        for (int tile : {KDGR_TILE_4X8, KDGR_TILE_16X2}) {
          kdgr_batch_config ct = *best;
          ct.tile_shape = tile;
          cands.push_back(ct);
        }
      // fewer rays per warp (2 or 4 lanes sharing each ray), on warp strips,
      // with either traversal
      for (int trav : {KDGR_TRAV_PACKET, KDGR_TRAV_RAY})
        for (int rpw : {16, 8}) {
          kdgr_batch_config cg = *best;
          cg.schedule = KDGR_SCHED_WARP_STRIPS;
          cg.chunk = 1;
          cg.traversal = trav;
          cg.tile_shape = KDGR_TILE_8X4;
          cg.rays_per_warp = rpw;
          cands.push_back(cg);
        }
    }
    const kdgr_batch_config c = cands[ci];
    rc = run_once(s, c, table, totals, rgb, nullptr, nullptr, st, "kdgr_autotune");  // warm-up
    if (rc != KDGR_OK) break;
    std::vector<float> ts;
    for (int r = 0; r < 3 && rc == KDGR_OK; ++r) {
      cudaEventRecord(e0, st);
      rc = run_once(s, c, table, totals, rgb, nullptr, nullptr, st, "kdgr_autotune");
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ts.push_back(ms);
    }
    if (rc != KDGR_OK) break;
    std::sort(ts.begin(), ts.end());
    const float med = ts[ts.size() / 2];
    char line[256];
    snprintf(line, sizeof(line),
             "{\"schedule\": %d, \"min_blocks\": %d, \"chunk\": %d, \"precision\": %d, \"hit_buffer\": %d, "
             "\"traversal\": %d, \"tile_shape\": %d, \"rays_per_warp\": %d, \"ms\": %.4f}\n",
             c.schedule, c.min_blocks, c.chunk, c.precision, c.hit_buffer, c.traversal, c.tile_shape,
             c.rays_per_warp, med);
    rep += line;
    if (med < best_ms) {
      best_ms = med;
      *best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  if (report && report_len > 0) {
    strncpy(report, rep.c_str(), (size_t)report_len - 1);
    report[report_len - 1] = '\0';
  }
  return rc;
}

}  // extern "C"
