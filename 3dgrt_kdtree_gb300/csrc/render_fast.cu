// render_fast.cu -- the batching and precision forms: a persistent kernel
// that draws pixel tiles of many views from an atomic work queue.
//
// Same algorithm as the plain kernel (render_exact.cu): short-stack kd-tree
// traversal front to back, per-leaf max-response test, hits composited in t
// order until the opacity threshold.  What changes, for throughput:
//   * arithmetic: FMA, rsqrt, __expf; the ray-Gaussian test reads the
//     precomputed rows of M = diag(1/s) R^T with b = M mu folded in
//     (gro = M o - b, grdu = M d), so t* = -(grd . gro) / |grdu| needs no
//     per-candidate quaternion expansion or reciprocal;
//   * hits are accepted with t* in the half-open interval [t_near, t_far),
//     so a Gaussian straddling a split plane is composited in one leaf only;
//   * the top levels of the tree (breadth-first, up to 2047 nodes) are
//     staged once per CTA in shared memory; the persistent CTAs amortise it;
//   * the short stack (ring semantics and root restart as the reference) is
//     in shared memory, [slot][thread];
//   * a leaf's candidates are fetched two at a time (both ID and record loads
//     in flight before either test), doubling the memory-level parallelism
//     of the latency-bound candidate loop;
//   * work items are either 8x4 tiles taken per warp or 16x8 blocks taken per
//     CTA (its four warps render neighbouring tiles and share L1); the
//     autotuner picks one.
//   * precision form: FP16 inverse scales / quaternion / opacity and BF16
//     SH (32 + 96 bytes per Gaussian instead of 64 + 192); Gaussians whose
//     scale ratio exceeds 1e3 read factors from the FP64 upload precompute.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "kdgr_internal.h"
#include "scene.h"

namespace kdgr {

static_assert(sizeof(ViewDesc) == 88, "ViewDesc layout (bench.py counts 88 B per view)");

namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kTileW = 8, kTileH = 4;     // pixels per warp tile
constexpr int kBlockW = 16, kBlockH = 8;  // pixels per CTA block (4 warps of 8x4)
constexpr int kHits = 8;                  // hit-buffer entries
constexpr uint32_t kMaxTop = 2047;

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 mk(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
  return mk(fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x));
}

__device__ __forceinline__ float bf16lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }
__device__ __forceinline__ float2 h2f(uint32_t w) {
  __half2 h;
  memcpy(&h, &w, 4);
  return __half22float2(h);
}

// ----------------------------------------------------------- candidate test
// Records of one candidate as loaded from memory.
struct Rec {
  float4 a, b, c;  // FP32: (M0,b0)(M1,b1)(M2,b2).  Packed: a = (mu, +-opacity), b = halves
};

template <bool PACKED>
__device__ __forceinline__ Rec load_rec(const FastView& S, uint32_t gid) {
  Rec r;
  if (!PACKED) {
    const float4* p = S.test + 3ull * gid;
    r.a = __ldg(p);
    r.b = __ldg(p + 1);
    r.c = __ldg(p + 2);
  } else {
    const uint4 u0 = __ldg(S.packed + 2ull * gid), u1 = __ldg(S.packed + 2ull * gid + 1);
    r.a = make_float4(__uint_as_float(u0.x), __uint_as_float(u0.y), __uint_as_float(u0.z), __uint_as_float(u0.w));
    r.b = make_float4(__uint_as_float(u1.x), __uint_as_float(u1.y), __uint_as_float(u1.z), __uint_as_float(u1.w));
    r.c = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  return r;
}

// t* and the squared Mahalanobis distance of the ray (cudaRenderer.cu:
// 1115-1127) from the rows of M = diag(1/s) R^T:
// grdu = M d, t* = -(grdu . gro) / |grdu|^2, gray = |grdu x gro|^2 / |grdu|^2.
__device__ __forceinline__ bool finish_test(F3 m0, F3 m1, F3 m2, F3 gro, F3 d, float t_near, float t_far,
                                            float* t_out, float* gray_out) {
  const F3 grdu = mk(dot3(m0, d), dot3(m1, d), dot3(m2, d));
  const float r2 = __fdividef(1.f, dot3(grdu, grdu));
  const float t = -dot3(grdu, gro) * r2;
  if (!(t >= t_near && t < t_far)) return false;
  const F3 c = cross3(grdu, gro);
  const float gray = dot3(c, c) * r2;
  *t_out = t;
  *gray_out = gray;
  return gray < 8.f;
}

template <bool PACKED>
__device__ __forceinline__ bool test_rec(const FastView& S, uint32_t gid, const Rec& r, F3 o, F3 d, float t_near,
                                         float t_far, float* t_out, float* gray_out) {
  if (!PACKED) {
    const F3 m0 = mk(r.a.x, r.a.y, r.a.z), m1 = mk(r.b.x, r.b.y, r.b.z), m2 = mk(r.c.x, r.c.y, r.c.z);
    const F3 gro = mk(dot3(m0, o) - r.a.w, dot3(m1, o) - r.b.w, dot3(m2, o) - r.c.w);
    return finish_test(m0, m1, m2, gro, d, t_near, t_far, t_out, gray_out);
  }
  if (__float_as_uint(r.a.w) >> 31) {  // anisotropic: factors from the FP64 upload precompute
    const float4* p = S.aniso + 3ull * __ldg(S.aniso_idx + gid);
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    const F3 m0 = mk(a.x, a.y, a.z), m1 = mk(b.x, b.y, b.z), m2 = mk(c.x, c.y, c.z);
    const F3 gro = mk(dot3(m0, o) - a.w, dot3(m1, o) - b.w, dot3(m2, o) - c.w);
    return finish_test(m0, m1, m2, gro, d, t_near, t_far, t_out, gray_out);
  }
  const float2 s01 = h2f(__float_as_uint(r.b.x)), s2 = h2f(__float_as_uint(r.b.y));
  const float2 qwx = h2f(__float_as_uint(r.b.z)), qyz = h2f(__float_as_uint(r.b.w));
  float qr = qwx.x, x = qwx.y, y = qyz.x, z = qyz.y;
  const float qn = rsqrtf(fmaf(qr, qr, fmaf(x, x, fmaf(y, y, z * z))));
  qr *= qn;
  x *= qn;
  y *= qn;
  z *= qn;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
  const float rx = qr * x, ry = qr * y, rz = qr * z;
  const F3 m0 = mk(s01.x * (1.f - 2.f * (yy + zz)), s01.x * 2.f * (xy + rz), s01.x * 2.f * (xz - ry));
  const F3 m1 = mk(s01.y * 2.f * (xy - rz), s01.y * (1.f - 2.f * (xx + zz)), s01.y * 2.f * (yz + rx));
  const F3 m2 = mk(s2.x * 2.f * (xz + ry), s2.x * 2.f * (yz - rx), s2.x * (1.f - 2.f * (xx + yy)));
  const F3 q = mk(o.x - r.a.x, o.y - r.a.y, o.z - r.a.z);
  const F3 gro = mk(dot3(m0, q), dot3(m1, q), dot3(m2, q));
  return finish_test(m0, m1, m2, gro, d, t_near, t_far, t_out, gray_out);
}

template <bool PACKED>
__device__ __forceinline__ float gauss_opacity(const FastView& S, uint32_t gid) {
  if (!PACKED) return __ldg(S.opacity + gid);
  return fabsf(__uint_as_float(__ldg(&S.packed[2ull * gid].w)));
}

// eval_sh_final(3, dir, g) (cudaRenderer.cu:487-558), FMA form.
template <bool PACKED>
__device__ __forceinline__ F3 eval_sh_fast(const FastView& S, uint32_t gid, F3 d) {
  float c[48];
  if (!PACKED) {
    const float4* p = S.sh + 12ull * gid;
#pragma unroll
    for (int i = 0; i < 12; ++i) {
      const float4 v = __ldg(p + i);
      c[4 * i] = v.x;
      c[4 * i + 1] = v.y;
      c[4 * i + 2] = v.z;
      c[4 * i + 3] = v.w;
    }
  } else {
    const uint4* p = S.sh_bf16 + 6ull * gid;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const uint4 v = __ldg(p + i);
      c[8 * i] = bf16lo(v.x);
      c[8 * i + 1] = bf16hi(v.x);
      c[8 * i + 2] = bf16lo(v.y);
      c[8 * i + 3] = bf16hi(v.y);
      c[8 * i + 4] = bf16lo(v.z);
      c[8 * i + 5] = bf16hi(v.z);
      c[8 * i + 6] = bf16lo(v.w);
      c[8 * i + 7] = bf16hi(v.w);
    }
  }
  const float x = d.x, y = d.y, z = d.z;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  float b[16];
  b[0] = 0.28209479177387814f;
  b[1] = -0.4886025119029199f * y;
  b[2] = 0.4886025119029199f * z;
  b[3] = -0.4886025119029199f * x;
  b[4] = 1.0925484305920792f * xy;
  b[5] = -1.0925484305920792f * yz;
  b[6] = 0.31539156525252005f * (2.f * zz - xx - yy);
  b[7] = -1.0925484305920792f * xz;
  b[8] = 0.5462742152960396f * (xx - yy);
  b[9] = -0.5900435899266435f * y * (3.f * xx - yy);
  b[10] = 2.890611442640554f * xy * z;
  b[11] = -0.4570457994644658f * y * (4.f * zz - xx - yy);
  b[12] = 0.3731763325901154f * z * (2.f * zz - 3.f * xx - 3.f * yy);
  b[13] = -0.4570457994644658f * x * (4.f * zz - xx - yy);
  b[14] = 1.445305721320277f * z * (xx - yy);
  b[15] = -0.5900435899266435f * x * (xx - 3.f * yy);
  float r = 0.5f, g = 0.5f, bl = 0.5f;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    r = fmaf(b[k], c[3 * k], r);
    g = fmaf(b[k], c[3 * k + 1], g);
    bl = fmaf(b[k], c[3 * k + 2], bl);
  }
  return mk(fmaxf(r, 0.f), fmaxf(g, 0.f), fmaxf(bl, 0.f));
}

// K smallest (t, leaf position) keys of a leaf pass, ascending; equal t keep
// leaf order (the stable sortHits, cudaRenderer.cu:415-426).
struct HitBuf {
  float t[kHits], g[kHits];
  uint32_t i[kHits];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int k = 0; k < kHits; ++k) {
      t[k] = __int_as_float(0x7f800000);
      g[k] = 0.f;
      i[k] = 0u;
    }
  }
  // returns true when an entry fell off the end (the leaf needs another pass)
  __device__ __forceinline__ bool insert(float ct, float cg, uint32_t ci) {
    bool placed = false;
#pragma unroll
    for (int k = 0; k < kHits; ++k) {
      const bool sw = placed || (ct < t[k]);
      const float t0 = t[k], g0 = g[k];
      const uint32_t i0 = i[k];
      t[k] = sw ? ct : t0;
      g[k] = sw ? cg : g0;
      i[k] = sw ? ci : i0;
      ct = sw ? t0 : ct;
      cg = sw ? g0 : cg;
      ci = sw ? i0 : ci;
      placed = sw;
    }
    return ct != __int_as_float(0x7f800000);
  }
};

// ------------------------------------------------------------------ one ray
template <int SD, bool PACKED, bool STAGE>
__device__ __forceinline__ void trace_ray(const FastView& S, const uint2* s_top, uint32_t n_top,
                                          uint32_t (*s_id)[kThreads], float (*s_t)[kThreads], int tid,
                                          const CamInfo& C, int x, int y, uint32_t* status, float* acc_out) {
  auto fetch = [&](uint32_t i) -> uint2 { return (STAGE && i < n_top) ? s_top[i] : __ldg(S.nodes + i); };
  const float sx = (float)x + 0.5f, sy = (float)y + 0.5f;
  const F3 o = mk(__ldg(&C.eye[0]), __ldg(&C.eye[1]), __ldg(&C.eye[2]));
  F3 d;
  {
    const float sxx = sx * __ldg(&C.step_x), syy = sy * __ldg(&C.step_y);
    d.x = __ldg(&C.start[0]) + __ldg(&C.u[0]) * sxx - __ldg(&C.v[0]) * syy - o.x;
    d.y = __ldg(&C.start[1]) + __ldg(&C.u[1]) * sxx - __ldg(&C.v[1]) * syy - o.y;
    d.z = __ldg(&C.start[2]) + __ldg(&C.u[2]) * sxx - __ldg(&C.v[2]) * syy - o.z;
    const float il = rsqrtf(dot3(d, d));
    d.x *= il;
    d.y *= il;
    d.z *= il;
  }
  const float inv[3] = {1.f / d.x, 1.f / d.y, 1.f / d.z};
  const float oo[3] = {o.x, o.y, o.z};
  float acc_r = 0.f, acc_g = 0.f, acc_b = 0.f, A = 0.f, D = 0.f;
  float tmin = 1e-2f, tmax = FLT_MAX;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float l1 = (S.bmin[a] - oo[a]) * inv[a];
    const float l2 = (S.bmax[a] - oo[a]) * inv[a];
    tmin = fmaxf(fminf(l1, l2), tmin);
    tmax = fminf(fmaxf(l1, l2), tmax);
  }
  if ((tmax >= tmin) & (tmax >= 0.f)) {
    const float t_scene_far = tmax;
    float t_near = tmin, t_far = tmax;
    uint32_t cur = 0, steps = 0;
    unsigned top = SD - 1, quant = 0;
    while (A < 0.99f) {
      uint2 nd = fetch(cur);
      if (++steps > kMaxRaySteps) {
        atomicOr(status, kStatusStepLimit);
        break;
      }
      bool bad = false;
      while ((nd.x & 7u) != 3u) {
        const uint32_t child = nd.x >> 3;
        const uint32_t axis = nd.x & 3u;
        const float o_a = axis == 0 ? oo[0] : axis == 1 ? oo[1] : oo[2];
        const float i_a = axis == 0 ? inv[0] : axis == 1 ? inv[1] : inv[2];
        const float t_split = (__uint_as_float(nd.y) - o_a) * i_a;
        const unsigned sign = __float_as_uint(i_a) >> 31;
        const uint32_t idx = child + (sign ^ (t_split <= t_near ? 1u : 0u));
        if (t_near < t_split && t_split < t_far) {
          if (++top == SD) top = 0;
          quant = min(quant + 1, (unsigned)SD);
          s_id[top][tid] = child + (sign ^ 1u);
          s_t[top][tid] = t_far;
          t_far = t_split;
        }
        if (child + 1 >= S.n_nodes || ++steps > kMaxRaySteps) {
          atomicOr(status, child + 1 >= S.n_nodes ? kStatusBadNode : kStatusStepLimit);
          bad = true;
          break;
        }
        cur = idx;
        nd = fetch(cur);
      }
      if (bad) break;
      const uint32_t cnt = nd.x >> 3, base = nd.y;
      if ((uint64_t)base + cnt > S.n_offsets) {
        atomicOr(status, kStatusBadLeaf);
        break;
      }
      bool have_last = false, saturated = false;
      float last_t = 0.f;
      uint32_t last_i = 0;
      while (true) {
        HitBuf hb;
        hb.clear();
        bool overflow = false;
        for (uint32_t i = 0; i < cnt; i += 2) {
          const bool two = i + 1 < cnt;
          const uint32_t g0 = __ldg(S.offsets + base + i);
          const uint32_t g1 = two ? __ldg(S.offsets + base + i + 1) : g0;
          if (g0 >= S.n_gauss || g1 >= S.n_gauss) {
            atomicOr(status, kStatusBadId);
            bad = true;
            break;
          }
          const Rec r0 = load_rec<PACKED>(S, g0);
          const Rec r1 = load_rec<PACKED>(S, g1);
          float t, g;
          if (test_rec<PACKED>(S, g0, r0, o, d, t_near, t_far, &t, &g) &&
              (!have_last || t > last_t || (t == last_t && i > last_i)))
            overflow |= hb.insert(t, g, i);
          if (two && test_rec<PACKED>(S, g1, r1, o, d, t_near, t_far, &t, &g) &&
              (!have_last || t > last_t || (t == last_t && i + 1 > last_i)))
            overflow |= hb.insert(t, g, i + 1);
        }
        if (bad) break;
#pragma unroll
        for (int k = 0; k < kHits; ++k) {
          if (hb.t[k] == __int_as_float(0x7f800000)) break;
          const uint32_t gid = __ldg(S.offsets + base + hb.i[k]);
          const float gres = __expf(-0.0555555555556f * hb.g[k] * hb.g[k]);
          const float alpha = fminf(0.99f, gauss_opacity<PACKED>(S, gid) * gres);
          if (gres < 0.0113f || alpha < 1.0f / 255.0f) continue;
          const F3 c = eval_sh_fast<PACKED>(S, gid, d);
          const float w = alpha * (1.f - A);
          acc_r = fmaf(c.x, w, acc_r);
          acc_g = fmaf(c.y, w, acc_g);
          acc_b = fmaf(c.z, w, acc_b);
          D = fmaf(hb.t[k], w, D);
          A += w;
          if (A > 0.99f) {
            saturated = true;
            break;
          }
        }
        if (saturated || !overflow) break;
        have_last = true;
        last_t = hb.t[kHits - 1];
        last_i = hb.i[kHits - 1];
      }
      if (bad) break;
      if ((A > 0.99f) | (t_far >= t_scene_far)) break;
      if (quant == 0) {
        cur = 0;
        t_near = t_far;
        t_far = t_scene_far;
      } else {
        const uint32_t id = s_id[top][tid];
        const float tm = s_t[top][tid];
        if (top == 0) top = SD;
        --top;
        --quant;
        cur = id;
        t_near = t_far;
        t_far = tm;
      }
    }
  }
  acc_out[0] = acc_r;
  acc_out[1] = acc_g;
  acc_out[2] = acc_b;
  acc_out[3] = A;
  acc_out[4] = D;
}

template <int SD, bool PACKED, bool STAGE, bool CTA>
__global__ void __launch_bounds__(kThreads) k_render_batch(FastView S, const ViewDesc* __restrict__ views, int n_views,
                                                           uint32_t total_items, float* __restrict__ rgb,
                                                           float* __restrict__ alpha_out,
                                                           float* __restrict__ depth_out, uint32_t* queue,
                                                           uint32_t* status, int chunk) {
  __shared__ uint2 s_top[STAGE ? kMaxTop : 1];
  __shared__ uint32_t s_id[SD][kThreads];
  __shared__ float s_t[SD][kThreads];
  __shared__ uint32_t s_work;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t n_top = STAGE ? min(S.top_nodes, kMaxTop) : 0u;
  if constexpr (STAGE) {
    for (uint32_t i = tid; i < n_top; i += kThreads) s_top[i] = __ldg(S.nodes + i);
    __syncthreads();
  }
  while (true) {
    uint32_t first;
    if constexpr (CTA) {
      // the CTA takes `chunk` 16x8 blocks; its warps render the four quarters
      __syncthreads();
      if (tid == 0) s_work = atomicAdd(queue, (uint32_t)chunk);
      __syncthreads();
      first = s_work;
    } else {
      // each warp takes `chunk` 8x4 tiles
      uint32_t f = 0;
      if (lane == 0) f = atomicAdd(queue, (uint32_t)chunk);
      first = __shfl_sync(0xFFFFFFFFu, f, 0);
    }
    if (first >= total_items) break;
    const uint32_t last = min(first + (uint32_t)chunk, total_items);
    for (uint32_t item = first; item < last; ++item) {
      int lo = 0, hi = n_views - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const uint32_t b = CTA ? __ldg(&views[mid].cb_base) : __ldg(&views[mid].wt_base);
        if (b <= item) lo = mid;
        else hi = mid - 1;
      }
      const ViewDesc& V = views[lo];
      int x, y;
      if (CTA) {
        const uint32_t lb = item - __ldg(&V.cb_base), nx = __ldg(&V.cb_x);
        x = (int)(lb % nx) * kBlockW + (warp & 1) * kTileW + (lane & 7);
        y = (int)(lb / nx) * kBlockH + (warp >> 1) * kTileH + (lane >> 3);
      } else {
        const uint32_t lt = item - __ldg(&V.wt_base), nx = __ldg(&V.wt_x);
        x = (int)(lt % nx) * kTileW + (lane & 7);
        y = (int)(lt / nx) * kTileH + (lane >> 3);
      }
      const int W = __ldg(&V.W), H = __ldg(&V.H);
      if (x >= W || y >= H) continue;
      float acc[5];
      trace_ray<SD, PACKED, STAGE>(S, s_top, n_top, s_id, s_t, tid, V.cam, x, y, status, acc);
      const size_t idx = (size_t)__ldg(&V.out_off) + (size_t)(H - 1 - y) * W + x;
      rgb[3 * idx] = acc[0];
      rgb[3 * idx + 1] = acc[1];
      rgb[3 * idx + 2] = acc[2];
      if (alpha_out) alpha_out[idx] = acc[3];
      if (depth_out) depth_out[idx] = acc[4];
    }
  }
}

// FP64 precompute of M = diag(1/s) R^T and b = M mu for anisotropic
// Gaussians (upload time only).  src: 10 floats per entry (inverse scale x3,
// quaternion w,x,y,z, mean x3).
__global__ void k_aniso_fp64(const float* __restrict__ src, uint32_t n, float4* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* p = src + 10ull * i;
  double r = p[3], x = p[4], y = p[5], z = p[6];
  const double qn = 1.0 / sqrt(r * r + x * x + y * y + z * z);
  r *= qn;
  x *= qn;
  y *= qn;
  z *= qn;
  const double xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
  const double rx = r * x, ry = r * y, rz = r * z;
  const double m[3][3] = {{1 - 2 * (yy + zz), 2 * (xy + rz), 2 * (xz - ry)},
                          {2 * (xy - rz), 1 - 2 * (xx + zz), 2 * (yz + rx)},
                          {2 * (xz + ry), 2 * (yz - rx), 1 - 2 * (xx + yy)}};
  for (int row = 0; row < 3; ++row) {
    const double s = p[row];
    const double a = s * m[row][0], b = s * m[row][1], c = s * m[row][2];
    const double bb = a * p[7] + b * p[8] + c * p[9];
    out[3ull * i + row] = make_float4((float)a, (float)b, (float)c, (float)bb);
  }
}

using KernelFn = void (*)(FastView, const ViewDesc*, int, uint32_t, float*, float*, float*, uint32_t*, uint32_t*,
                          int);

template <bool PACKED, bool STAGE, bool CTA>
KernelFn pick_sd(int stack) {
  return stack >= 24 ? k_render_batch<24, PACKED, STAGE, CTA> : k_render_batch<16, PACKED, STAGE, CTA>;
}

template <bool PACKED, bool STAGE>
KernelFn pick_cta(const kdgr_batch_config& c) {
  return c.cta_tiles ? pick_sd<PACKED, STAGE, true>(c.stack) : pick_sd<PACKED, STAGE, false>(c.stack);
}

KernelFn pick_kernel(const kdgr_batch_config& c) {
  if (c.precision) return c.stage_top ? pick_cta<true, true>(c) : pick_cta<true, false>(c);
  return c.stage_top ? pick_cta<false, true>(c) : pick_cta<false, false>(c);
}

int g_num_sms = 0;

int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

}  // namespace

// Host: view table and total tile count for a list of views.
int make_view_table(const kdgr_view* views, int n_views, std::vector<ViewDesc>& out, uint32_t* total_tiles,
                    uint32_t* total_blocks) {
  out.resize(n_views);
  uint64_t wbase = 0, cbase = 0;
  for (int v = 0; v < n_views; ++v) {
    const kdgr_view& kv = views[v];
    if (kv.width <= 0 || kv.height <= 0) {
      set_error("view " + std::to_string(v) + " has an empty image");
      return KDGR_ERR_INVALID_ARG;
    }
    ViewDesc& d = out[v];
    d.cam = make_caminfo(kv.cam, kv.width, kv.height);
    d.W = kv.width;
    d.H = kv.height;
    d.wt_x = (uint32_t)((kv.width + kTileW - 1) / kTileW);
    d.wt_base = (uint32_t)wbase;
    d.cb_x = (uint32_t)((kv.width + kBlockW - 1) / kBlockW);
    d.cb_base = (uint32_t)cbase;
    d.out_off = kv.out_offset;
    wbase += (uint64_t)d.wt_x * (uint64_t)((kv.height + kTileH - 1) / kTileH);
    cbase += (uint64_t)d.cb_x * (uint64_t)((kv.height + kBlockH - 1) / kBlockH);
    if (wbase > 0xF0000000ull) {
      set_error("batch too large: more than 2^32 tiles");
      return KDGR_ERR_LIMIT;
    }
  }
  *total_tiles = (uint32_t)wbase;
  *total_blocks = (uint32_t)cbase;
  return KDGR_OK;
}

int check_batch_config(kdgr_scene_t s, const kdgr_batch_config& c) {
  if (c.precision && !(s->forms & KDGR_FORM_PACKED)) {
    set_error("precision form requested but the scene was created without KDGR_FORM_PACKED");
    return KDGR_ERR_INVALID_ARG;
  }
  if (!c.precision && !(s->forms & KDGR_FORM_FAST)) {
    set_error("FP32 fast form requested but the scene was created without KDGR_FORM_FAST");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.chunk < 1 || c.chunk > 64) {
    set_error("batch config: chunk must be in 1..64");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.kbuf != kHits || (c.stack != 16 && c.stack != 24)) {
    set_error("batch config: kbuf must be 8 and stack 16 or 24");
    return KDGR_ERR_INVALID_ARG;
  }
  return KDGR_OK;
}

// Launch the persistent kernel.  `queue` must read 0 when the kernel starts.
cudaError_t launch_batch(kdgr_scene_t s, const kdgr_batch_config& c, const ViewDesc* d_views, int n_views,
                         uint32_t total_tiles, uint32_t total_blocks, float* rgb, float* alpha, float* depth,
                         uint32_t* queue, cudaStream_t st) {
  KernelFn fn = pick_kernel(c);
  int per_sm = c.blocks_per_sm;
  if (per_sm <= 0) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kThreads, 0);
    if (e != cudaSuccess) return e;
    per_sm = occ > 0 ? occ : 1;
  }
  const uint32_t total = c.cta_tiles ? total_blocks : total_tiles;
  uint64_t blocks = (uint64_t)num_sms() * per_sm;
  const uint64_t grabs = ((uint64_t)total + c.chunk - 1) / c.chunk;
  const uint64_t cap = c.cta_tiles ? grabs : (grabs + kWarps - 1) / kWarps;
  if (blocks > cap) blocks = cap > 0 ? cap : 1;
  fn<<<(unsigned)blocks, kThreads, 0, st>>>(s->fast_view(), d_views, n_views, total, rgb, alpha, depth, queue,
                                            s->d_status, c.chunk);
  return cudaGetLastError();
}

int pack_precision(kdgr_scene_s* s, const float* g, const float* giscl, const float* sh, DevAlloc& A) {
  const size_t n = s->n_gauss;
  std::vector<uint32_t> packed(8 * n);
  std::vector<uint16_t> shb(48 * n);
  std::vector<uint32_t> aidx(n, 0xFFFFFFFFu);
  std::vector<float> aniso_src;
  uint32_t n_aniso = 0;
  auto pk = [](float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    uint32_t w;
    memcpy(&w, &h, 4);
    return w;
  };
  for (size_t i = 0; i < n; ++i) {
    const float* r = g + 64 * i;
    const float* gs = giscl + 3 * i;
    uint32_t* p = packed.data() + 8 * i;
    const double smax = 1.0 / std::min(std::min((double)gs[0], (double)gs[1]), (double)gs[2]);
    const double smin = 1.0 / std::max(std::max((double)gs[0], (double)gs[1]), (double)gs[2]);
    const bool aniso = smax > kAnisoRatio * smin;
    uint32_t op_bits;
    memcpy(&op_bits, &r[3], 4);
    op_bits = (op_bits & 0x7FFFFFFFu) | (aniso ? 0x80000000u : 0u);  // sign bit flags the FP64 factor table
    memcpy(&p[0], &r[0], 4);
    memcpy(&p[1], &r[1], 4);
    memcpy(&p[2], &r[2], 4);
    p[3] = op_bits;
    p[4] = pk(gs[0], gs[1]);
    p[5] = pk(gs[2], 0.f);
    p[6] = pk(r[8], r[9]);
    p[7] = pk(r[10], r[11]);
    if (aniso) {
      aidx[i] = n_aniso++;
      const float src[10] = {gs[0], gs[1], gs[2], r[8], r[9], r[10], r[11], r[0], r[1], r[2]};
      aniso_src.insert(aniso_src.end(), src, src + 10);
    }
    for (int k = 0; k < 48; ++k) {
      __nv_bfloat16 b = __float2bfloat16_rn(sh[48 * i + k]);
      memcpy(&shb[48 * i + k], &b, 2);
    }
  }
  s->d_packed = A.alloc<uint4>(2 * n);
  s->d_sh_bf16 = A.alloc<uint4>(6 * n);
  s->d_aniso_idx = A.alloc<uint32_t>(n);
  s->d_aniso = A.alloc<float4>(3 * (size_t)(n_aniso ? n_aniso : 1));
  float* d_src = nullptr;
  if (A.err != cudaSuccess) return cuda_fail(A.err, "kdgr_scene_create: cudaMalloc (packed)");
  cudaError_t e = cudaMemcpy(s->d_packed, packed.data(), packed.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_sh_bf16, shb.data(), shb.size() * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_aniso_idx, aidx.data(), aidx.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n_aniso) {
    e = cudaMalloc(&d_src, aniso_src.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(d_src, aniso_src.data(), aniso_src.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      k_aniso_fp64<<<(n_aniso + 127) / 128, 128>>>(d_src, n_aniso, s->d_aniso);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (d_src) cudaFree(d_src);
  }
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_scene_create: packed upload");
  s->n_aniso = n_aniso;
  return KDGR_OK;
}

int batch_sms() { return num_sms(); }

}  // namespace kdgr
