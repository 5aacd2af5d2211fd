// render_fast.cu -- the batching and precision forms: a persistent kernel
// that draws pixel tiles of many views from an atomic work queue.
//
// Same algorithm as the plain kernel (render_exact.cu): short-stack kd-tree
// traversal front to back, per-leaf max-response test, hits composited in t
// order until the opacity threshold.  What changes, for throughput:
//   * arithmetic: FMA, fast reciprocal, __expf; the ray-Gaussian test reads
//     the precomputed rows of M = diag(1/s) R^T (with b = M mu folded in for
//     the FP32 form), forms ng = M (mu - o) and grdu = M d, accepts t* on
//     the leaf interval without a reciprocal (by the signs of two fused
//     multiply-adds) and only then evaluates the Mahalanobis distance;
//   * hits are accepted with t* in the half-open interval [t_near, t_far),
//     so a Gaussian straddling a split plane is composited in one leaf only;
//   * the tree is relaid out with its top levels breadth-first (they stay
//     hot in L1/L2) and the rest depth-first, and validated at upload, so
//     node steps carry no bounds checks;
//   * the short stack (ring semantics and root restart as the reference) is
//     in shared memory, [slot][thread];
//   * candidate records are stored a second time in leaf order, padded to
//     whole pairs per leaf, so a leaf's candidates are one contiguous run:
//     no ID-then-record dependent load per candidate; the ID is read only
//     for accepted hits;
//   * both forms store leaf entries in interleaved pairs and test them two
//     at a time with Blackwell's packed FP32x2 instructions
//     (fma/mul/add/sub.rn.f32x2), half the arithmetic instructions per test;
//   * warp packets (the default traversal): the 32 rays of a warp tile walk
//     the tree together, each with its own interval and decisions, so a
//     leaf's records are warp-uniform loads (pkt_trace below);
//   * lane groups (16 or 8 rays per warp): 2 or 4 lanes hold each ray and
//     split its leaves' candidate pairs, the group taking its hits in key
//     order from the lanes' buffers -- shorter rays and more warps in flight
//     for small batches, the same pixels bit for bit;
//   * pixels are handed out in spatially coherent units (8x4 warp tiles,
//     16x8 CTA blocks, or blocks / tiles from per-SM contiguous strips) so
//     the rays sharing an SM's L1 are neighbours; the autotuner picks the
//     schedule, the register cap (occupancy), the hit-buffer size, the
//     traversal, the warp tile shape and the rays per warp;
//   * precision form: FP16 rows of M with an FP32 mean and BF16 SH (32 + 96
//     bytes per Gaussian instead of 48 + 192); Gaussians whose scale ratio
//     exceeds 1e3 (or whose factors leave the FP16 range) read FP32 factors
//     from the FP64 upload precompute.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "kdgr_internal.h"
#include "scene.h"

namespace kdgr {

static_assert(sizeof(ViewDesc) == 96, "ViewDesc layout (bench.py counts 96 B per view)");

namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kTileW = 8, kTileH = 4;     // pixels per warp tile
constexpr int kBlockW = 16, kBlockH = 8;  // pixels per CTA block (4 warp tiles)
#ifndef KDGR_FAST_HITS
#define KDGR_FAST_HITS 4
#endif
#ifndef KDGR_FAST_STACK
#define KDGR_FAST_STACK 12
#endif
constexpr int kHits = KDGR_FAST_HITS;  // hit-buffer entries per leaf pass (a leaf averages <1 hit)

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 mk(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }

__device__ __forceinline__ float bf16lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }
__device__ __forceinline__ float2 h2f(uint32_t w) {
  __half2 h;
  memcpy(&h, &w, 4);
  return __half22float2(h);
}

// ----------------------------------------------------------- candidate test
// Candidate records.  FP32 form: rows of M = diag(1/s) R^T with b = M mu
// (FP64 upload precompute), read as interleaved pairs (load_pair below).
// Storing Sigma^-1 = M^T M instead would square the condition number (a
// scale ratio of 2500 gives ~6e6, beyond FP32), so the factor is kept.
// ------------------------------------------------- paired FP32x2 candidate test
// Both forms store leaf entries in pairs: pair p holds entries 2p and 2p+1
// interleaved, so every quantity of the test is one 64-bit register with
// entry 2p in the low and entry 2p+1 in the high half, and one packed FP32x2
// instruction (fma/mul/add/sub.rn.f32x2) does the work of two.
// FP32 pair, 6 x 16 bytes, for rows i = 0..2 of M and b = M mu:
//   q[2i]   = (M_i0 lo, M_i0 hi, M_i1 lo, M_i1 hi)
//   q[2i+1] = (M_i2 lo, M_i2 hi, b_i lo, b_i hi)
// Packed pair, 4 x 16 bytes (FP32 means, FP16 M as half2 (lo, hi)):
//   w[0] = (mu.x lo, mu.x hi, mu.y lo, mu.y hi)
//   w[1] = (mu.z lo, mu.z hi, M00, M01)
//   w[2] = (M02, M10, M11, M12)
//   w[3] = (M20, M21, M22, flags)   flags bit k: entry k reads the FP32 factors
//                                   of the FP64 upload precompute instead; its
//                                   mean.x slot then holds the table index
typedef unsigned long long f2;

__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 bcast2(float x) {
  f2 d;
  asm("mov.b64 %0, {%1, %1};" : "=l"(d) : "f"(x));
  return d;
}
__device__ __forceinline__ void split2(f2 v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 join2(float lo, float hi) {
  f2 d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ f2 h2f2(uint32_t w) {  // half2 -> (lo, hi) FP32 pair
  const float2 f = h2f(w);
  return join2(f.x, f.y);
}
__device__ __forceinline__ f2 u2f2(uint32_t lo, uint32_t hi) {
  return join2(__uint_as_float(lo), __uint_as_float(hi));
}

struct PairRec {
  ulonglong2 q[6];
};

__device__ __forceinline__ PairRec load_pair(const FastView& S, uint32_t p) {
  const ulonglong2* a = reinterpret_cast<const ulonglong2*>(S.leaf_pairs) + 6ull * p;
  PairRec r;
#pragma unroll
  for (int k = 0; k < 6; ++k) r.q[k] = __ldg(a + k);
  return r;
}

// Ray constants of the pair test, broadcast to both halves once per leaf.
struct Ray2 {
  f2 nox, noy, noz, dx, dy, dz;
};
__device__ __forceinline__ Ray2 ray2(F3 o, F3 d) {
  return Ray2{bcast2(-o.x), bcast2(-o.y), bcast2(-o.z), bcast2(d.x), bcast2(d.y), bcast2(d.z)};
}

// The M-form test (grdu = M d, ng = M (mu - o), t* = (grdu . ng) / |grdu|^2,
// gray = |grdu x ng|^2 / |grdu|^2) for both entries of a pair, in two steps:
// pair_t decides t* in [t_near, t_far), pair_g the response bound, so a warp
// packet can skip the second step together when no lane's t* is in range.
struct PairT {
  f2 ng[3], gd[3];
  float q0, q1, a0, a1;
};
__device__ __forceinline__ unsigned pair_t(PairT& p, float t_near, float t_far) {
  const f2 q = fma2(p.gd[0], p.gd[0], fma2(p.gd[1], p.gd[1], mul2(p.gd[2], p.gd[2])));
  const f2 a = fma2(p.gd[0], p.ng[0], fma2(p.gd[1], p.ng[1], mul2(p.gd[2], p.ng[2])));
  // t* = a / q in [t_near, t_far)  <=>  a - t_near q >= 0 and a - t_far q < 0  (q > 0),
  // each difference formed by one fused multiply-add and read by its sign.
  // A leaf's t_far is the next leaf's t_near, so one rounded difference
  // decides both sides of a split plane: a Gaussian straddling it is
  // accepted in exactly one of the two leaves.  Padding entries (q = a = 0)
  // give +0 on both sides and are refused.
  const f2 lo = fma2(q, bcast2(-t_near), a), hi = fma2(q, bcast2(-t_far), a);
  float q0, q1, a0, a1, l0, l1, h0, h1;
  split2(q, q0, q1);
  split2(a, a0, a1);
  split2(lo, l0, l1);
  split2(hi, h0, h1);
  p.q0 = q0;
  p.q1 = q1;
  p.a0 = a0;
  p.a1 = a1;
  const uint32_t m0 = __float_as_uint(h0) & ~__float_as_uint(l0), m1 = __float_as_uint(h1) & ~__float_as_uint(l1);
  return (m0 >> 31) | ((m1 >> 31) << 1);
}
// FP32 pair: ng = b - M o.
__device__ __forceinline__ void setup_pair(const PairRec& r, const Ray2& w, PairT& p) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const f2 m0 = r.q[2 * i].x, m1 = r.q[2 * i].y, m2 = r.q[2 * i + 1].x, b = r.q[2 * i + 1].y;
    p.ng[i] = fma2(m0, w.nox, fma2(m1, w.noy, fma2(m2, w.noz, b)));
    p.gd[i] = fma2(m0, w.dx, fma2(m1, w.dy, mul2(m2, w.dz)));
  }
}

struct PPairRec {
  uint4 w[4];
};

// Packed pair: FP16 rows of M, FP32 mean, ng = M (mu - o) (no M o - M mu
// cancellation, so the FP16 rounding stays a small consistent perturbation
// of the Gaussian).
__device__ __forceinline__ void setup_ppair(const PPairRec& r, const Ray2& w, PairT& p) {
  const f2 nqx = add2(u2f2(r.w[0].x, r.w[0].y), w.nox);
  const f2 nqy = add2(u2f2(r.w[0].z, r.w[0].w), w.noy);
  const f2 nqz = add2(u2f2(r.w[1].x, r.w[1].y), w.noz);
  const uint32_t mw[9] = {r.w[1].z, r.w[1].w, r.w[2].x, r.w[2].y, r.w[2].z, r.w[2].w, r.w[3].x, r.w[3].y, r.w[3].z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const f2 m0 = h2f2(mw[3 * i]), m1 = h2f2(mw[3 * i + 1]), m2 = h2f2(mw[3 * i + 2]);
    p.ng[i] = fma2(m0, nqx, fma2(m1, nqy, mul2(m2, nqz)));
    p.gd[i] = fma2(m0, w.dx, fma2(m1, w.dy, mul2(m2, w.dz)));
  }
}

__device__ __forceinline__ PPairRec load_ppair(const FastView& S, uint32_t p) {
  const uint4* a = S.leaf_packed + 4ull * p;
  PPairRec r;
#pragma unroll
  for (int k = 0; k < 4; ++k) r.w[k] = __ldg(a + k);
  return r;
}

// A leaf of either form: `np` pairs of the main stream from pair `pb`
// (FP32 pairs, or packed FP16 pairs), then in the packed form `nf` FP32
// pairs of its flagged entries from pair `fb` (leaf_pairs holds that stream).
struct LeafRef {
  uint32_t pb, np, fb, nf;
};

template <bool PACKED>
__device__ __forceinline__ LeafRef leaf_ref(const FastView& S, uint32_t node, uint2 nd) {
  LeafRef L{nd.y, ((nd.x >> 3) + 1) >> 1, 0u, 0u};
  if constexpr (PACKED) {
    const uint2 a = __ldg(S.leaf_aux + node);
    L.fb = a.x;
    L.nf = (a.y + 1) >> 1;
  }
  return L;
}

__device__ __forceinline__ bool leaf_in_bounds(const FastView& S, const LeafRef& L) {
  return 2ull * ((uint64_t)L.pb + L.np) <= S.n_offsets && 2ull * ((uint64_t)L.fb + L.nf) <= S.n_flag;
}

// The t* step for pair j of leaf L.
template <bool PACKED>
__device__ __forceinline__ unsigned leaf_pair_t(const FastView& S, const LeafRef& L, uint32_t j, const Ray2& w,
                                                float t_near, float t_far, PairT& p) {
  if (PACKED && j < L.np) {
    setup_ppair(load_ppair(S, L.pb + j), w, p);
  } else {
    setup_pair(load_pair(S, PACKED ? L.fb + (j - L.np) : L.pb + j), w, p);
  }
  return pair_t(p, t_near, t_far);
}

// Gaussian of leaf entry ik.
template <bool PACKED>
__device__ __forceinline__ uint32_t leaf_gid(const FastView& S, const LeafRef& L, uint32_t ik) {
  if (PACKED && ik >= 2 * L.np) return __ldg(S.flag_offsets + 2 * L.fb + (ik - 2 * L.np));
  return __ldg(S.offsets + 2 * L.pb + ik);
}

__device__ __forceinline__ unsigned test_pair_g(const PairT& p, unsigned m, float t[2], float g[2]) {
  const float r0 = __fdividef(1.f, p.q0), r1 = __fdividef(1.f, p.q1);
  t[0] = p.a0 * r0;
  t[1] = p.a1 * r1;
  const f2 c0 = sub2(mul2(p.gd[1], p.ng[2]), mul2(p.gd[2], p.ng[1]));
  const f2 c1 = sub2(mul2(p.gd[2], p.ng[0]), mul2(p.gd[0], p.ng[2]));
  const f2 c2 = sub2(mul2(p.gd[0], p.ng[1]), mul2(p.gd[1], p.ng[0]));
  const f2 cc = fma2(c0, c0, fma2(c1, c1, mul2(c2, c2)));
  float cc0, cc1;
  split2(cc, cc0, cc1);
  g[0] = cc0 * r0;
  g[1] = cc1 * r1;
  if (!(g[0] < 8.f)) m &= ~1u;
  if (!(g[1] < 8.f)) m &= ~2u;
  return m;
}

template <bool PACKED>
__device__ __forceinline__ float gauss_opacity(const FastView& S, uint32_t gid) {
  return __ldg(S.opacity + gid);
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
template <int K>
struct HitBuf {
  float t[K], g[K];
  uint32_t i[K];
  // only t: g and i are read where t is finite, and insert moves them with t
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int k = 0; k < K; ++k) t[k] = __int_as_float(0x7f800000);
  }
  // returns true when an entry fell off the end (the leaf needs another pass)
  __device__ __forceinline__ bool insert(float ct, float cg, uint32_t ci) {
    // t is ascending, so c[k] = ct < t[k] is false up to the insertion point
    // and true after it: every slot takes its old value, the new key or its
    // left neighbour's old value, decided without a chain between slots
    bool c[K];
#pragma unroll
    for (int k = 0; k < K; ++k) c[k] = ct < t[k];
    const float out = c[K - 1] ? t[K - 1] : ct;  // the key that falls off
#pragma unroll
    for (int k = K - 1; k > 0; --k) {
      t[k] = c[k] ? (c[k - 1] ? t[k - 1] : ct) : t[k];
      g[k] = c[k] ? (c[k - 1] ? g[k - 1] : cg) : g[k];
      i[k] = c[k] ? (c[k - 1] ? i[k - 1] : ci) : i[k];
    }
    t[0] = c[0] ? ct : t[0];
    g[0] = c[0] ? cg : g[0];
    i[0] = c[0] ? ci : i[0];
    return out != __int_as_float(0x7f800000);
  }
};

// ------------------------------------------------------------------ one ray
constexpr int kStack = KDGR_FAST_STACK;  // short-stack ring entries (ring + root restart as the reference)

// Per-lane ray state; one leaf is processed per call of leaf_step.
// The colour and depth accumulators of this thread's ray (r, g, b, depth),
// in shared memory: they change only when a hit is blended and are read
// once when the pixel is stored, so keeping them out of registers through
// the candidate loop and the descent leaves those loops fewer spills
// (64-register cap).
__device__ __forceinline__ float4* acc_slot() {
  __shared__ float4 s_acc[kThreads];
  return &s_acc[threadIdx.x];
}

struct Ray {
  F3 o, d, inv;
  float t_near, t_far, t_scene_far;
  float A;  // opacity; colour and depth accumulate in acc_slot()
  uint32_t cur, steps;
  unsigned top, quant;
};

__device__ __forceinline__ float sel3(const F3& v, uint32_t axis) { return axis == 0 ? v.x : axis == 1 ? v.y : v.z; }

// Ray generation (cudaRenderer.cu:2336-2339) and the scene-box slab test
// (:379-399).  Returns false when the ray misses the box.
__device__ __forceinline__ bool ray_init(const FastView& S, const CamInfo& C, int x, int y, Ray& R) {
  const float sx = (float)x + 0.5f, sy = (float)y + 0.5f;
  R.o = mk(__ldg(&C.eye[0]), __ldg(&C.eye[1]), __ldg(&C.eye[2]));
  const float sxx = sx * __ldg(&C.step_x), syy = sy * __ldg(&C.step_y);
  F3 d;
  d.x = __ldg(&C.start[0]) + __ldg(&C.u[0]) * sxx - __ldg(&C.v[0]) * syy - R.o.x;
  d.y = __ldg(&C.start[1]) + __ldg(&C.u[1]) * sxx - __ldg(&C.v[1]) * syy - R.o.y;
  d.z = __ldg(&C.start[2]) + __ldg(&C.u[2]) * sxx - __ldg(&C.v[2]) * syy - R.o.z;
  const float il = rsqrtf(dot3(d, d));
  R.d = mk(d.x * il, d.y * il, d.z * il);
  R.inv = mk(1.f / R.d.x, 1.f / R.d.y, 1.f / R.d.z);
  R.A = 0.f;
  *acc_slot() = make_float4(0.f, 0.f, 0.f, 0.f);
  float tmin = 1e-2f, tmax = FLT_MAX;
  const float oo[3] = {R.o.x, R.o.y, R.o.z}, iv[3] = {R.inv.x, R.inv.y, R.inv.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float l1 = (S.bmin[a] - oo[a]) * iv[a];
    const float l2 = (S.bmax[a] - oo[a]) * iv[a];
    tmin = fmaxf(fminf(l1, l2), tmin);
    tmax = fminf(fmaxf(l1, l2), tmax);
  }
  R.t_near = tmin;
  R.t_far = tmax;
  R.t_scene_far = tmax;
  R.cur = 0;
  R.steps = 0;
  R.top = kStack - 1;
  R.quant = 0;
  return (tmax >= tmin) & (tmax >= 0.f);
}

// ------------------------------------------------------------ lane groups
// With fewer than 32 rays per warp, each ray is held by a group of LPR
// consecutive lanes (LPR = 2 or 4).  The lanes of a group hold the same ray
// state and take the same decisions; lane `sub` of the group tests pairs
// sub, sub + LPR, ... of each leaf, and the group takes its hits in key
// order from the lanes' buffers.  `mask` names the lanes that make the
// collective calls together: the whole warp (packets) or the group
// (independent rays).

// Minimum over the group of the keys (t, i), carrying g.
template <int LPR>
__device__ __forceinline__ void group_min(float& t, uint32_t& i, float& g, unsigned mask) {
#pragma unroll
  for (int o = 1; o < LPR; o <<= 1) {
    const float ot = __shfl_xor_sync(mask, t, o);
    const uint32_t oi = __shfl_xor_sync(mask, i, o);
    const float og = __shfl_xor_sync(mask, g, o);
    if (ot < t || (ot == t && oi < i)) {
      t = ot;
      i = oi;
      g = og;
    }
  }
}

__device__ __forceinline__ unsigned group_mask(int LPR) {
  const unsigned lane = threadIdx.x & 31u;
  return ((1u << LPR) - 1u) << (lane & ~(unsigned)(LPR - 1));
}

// The candidate scan of one leaf pass for this lane's share of the pairs:
// the K smallest (t, leaf position) keys above the last key taken, on
// [tn, t_far).  Returns true when the share had more accepted hits than K.
template <int K, bool PACKED, int LPR>
__device__ __forceinline__ bool scan_share(const FastView& S, const LeafRef& L, const Ray& R, float tn,
                                           unsigned mask, bool have_last, float last_t, uint32_t last_i,
                                           HitBuf<K>& hb) {
  const unsigned sub = threadIdx.x & (LPR - 1u);
  bool overflow = false;
  hb.clear();
  const Ray2 w = ray2(R.o, R.d);
  const uint32_t np = L.np + L.nf;
  for (uint32_t pb = 0; pb < np; pb += LPR) {
    const uint32_t p = pb + sub;
    float t2[2], g2[2];
    PairT pt;
    // a lane past the end of the leaf tests its last pair again and drops it
    unsigned m = leaf_pair_t<PACKED>(S, L, LPR == 1 || p < np ? p : np - 1u, w, tn, R.t_far, pt);
    if (LPR > 1 && p >= np) m = 0u;
    // uniform branches: most pairs have no lane with t* in range
    if (__any_sync(mask, m != 0u)) {
      m = test_pair_g(pt, m, t2, g2);
      if (__any_sync(mask, m != 0u)) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const uint32_t ik = 2 * p + k;
          if (((m >> k) & 1u) && (!have_last || t2[k] > last_t || (t2[k] == last_t && ik > last_i)))
            overflow |= hb.insert(t2[k], g2[k], ik);
        }
      }
    }
  }
  return overflow;
}

// Composite one accepted hit (t, g) of Gaussian gid: response, alpha with
// the 0.99 cap, the 0.0113 / (1/255) skips, SH colour, front-to-back update.
template <bool PACKED>
__device__ __forceinline__ void blend_hit(const FastView& S, Ray& R, float t, float g, uint32_t gid) {
  const float gres = __expf(-0.0555555555556f * g * g);
  const float alpha = fminf(0.99f, gauss_opacity<PACKED>(S, gid) * gres);
  if (gres < 0.0113f || alpha < 1.0f / 255.0f) return;
  const F3 c = eval_sh_fast<PACKED>(S, gid, R.d);
  const float w = alpha * (1.f - R.A);
  float4* acc = acc_slot();
  float4 v = *acc;
  v.x = fmaf(c.x, w, v.x);
  v.y = fmaf(c.y, w, v.y);
  v.z = fmaf(c.z, w, v.z);
  v.w = fmaf(t, w, v.w);
  *acc = v;
  R.A += w;
}

// The group takes its hits of one leaf pass in key order: the smallest
// head key of the lanes' buffers, popped from the lane that holds it, as
// long as no lane whose share overflowed has run out of buffered keys (its
// next key is not known).  Every lane of the group blends the same hits.
// Stops once A > 0.99.  Returns whether the group must re-scan the leaf
// above (last_t, last_i).
template <int K, bool PACKED, int LPR>
__device__ __forceinline__ bool take_group_hits(const FastView& S, const LeafRef& L, Ray& R, const HitBuf<K>& hb,
                                                bool overflow, unsigned mask, bool active, bool& ok,
                                                float& last_t, uint32_t& last_i, uint32_t* status) {
  const float kInf = __int_as_float(0x7f800000);
  const unsigned gm = group_mask(LPR);
  uint32_t h = 0;  // next unconsumed entry of this lane's buffer
#pragma unroll 1
  for (int it = 0; it < K * LPR; ++it) {
    float kt = kInf, kg = 0.f;
    uint32_t ki = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (h == (uint32_t)k) {
        kt = hb.t[k];
        kg = hb.g[k];
        ki = hb.i[k];
      }
    const bool blocked = (__ballot_sync(mask, overflow && h == (uint32_t)K) & gm) != 0u;
    float mt = kt, mg = kg;
    uint32_t mi = ki;
    group_min<LPR>(mt, mi, mg, mask);
    const bool act = active && ok && !blocked && mt != kInf && !(R.A > 0.99f);
    if (!__any_sync(mask, act)) break;
    if (act) {
      if (kt == mt && ki == mi) ++h;
      last_t = mt;
      last_i = mi;
      const uint32_t gid = leaf_gid<PACKED>(S, L, mi);
      if (gid >= S.n_gauss) {
        atomicOr(status, kStatusBadId);
        ok = false;
      } else {
        blend_hit<PACKED>(S, R, mt, mg, gid);
      }
    }
  }
  return (__ballot_sync(mask, overflow) & gm) != 0u;
}

// Descend from R.cur to the next leaf, test and composite it, then pop or
// restart (singlePassIntersectGaussian_sortNode_onlyShortStack,
// cudaRenderer.cu:1552-1708).  Returns true when the ray is finished.  With
// LPR > 1 the lanes of a group walk the same ray together and split each
// leaf's candidates.
template <int K, bool PACKED, int LPR>
__device__ __forceinline__ bool leaf_step(const FastView& S, uint32_t (*s_id)[kThreads], float (*s_t)[kThreads],
                                          int tid, Ray& R, uint32_t* status) {
  uint2 nd = __ldg(S.nodes + R.cur);
  if (++R.steps > kMaxRaySteps) {
    atomicOr(status, kStatusStepLimit);
    return true;
  }
  while ((nd.x & 7u) != 3u) {
    const uint32_t child = nd.x >> 3;
    const uint32_t axis = nd.x & 3u;
    const float i_a = sel3(R.inv, axis);
    const float t_split = (__uint_as_float(nd.y) - sel3(R.o, axis)) * i_a;
    const unsigned sign = __float_as_uint(i_a) >> 31;
    const uint32_t idx = child + (sign ^ (t_split <= R.t_near ? 1u : 0u));
    if (R.t_near < t_split && t_split < R.t_far) {
      if (++R.top == kStack) R.top = 0;
      R.quant = min(R.quant + 1, (unsigned)kStack);
      s_id[R.top][tid] = child + (sign ^ 1u);
      s_t[R.top][tid] = R.t_far;
      R.t_far = t_split;
    }
    R.cur = idx;
    nd = __ldg(S.nodes + R.cur);
  }
  const LeafRef L = leaf_ref<PACKED>(S, R.cur, nd);
  if (!leaf_in_bounds(S, L)) {
    atomicOr(status, kStatusBadLeaf);
    return true;
  }
  bool have_last = false;
  float last_t = 0.f;
  uint32_t last_i = 0;
  if constexpr (LPR > 1) {
    const unsigned gm = group_mask(LPR);
    bool ok = true;
    while (true) {
      HitBuf<K> hb;
      const bool overflow = scan_share<K, PACKED, LPR>(S, L, R, R.t_near, gm, have_last, last_t, last_i, hb);
      const bool again = take_group_hits<K, PACKED, LPR>(S, L, R, hb, overflow, gm, true, ok, last_t, last_i, status);
      if (!ok || R.A > 0.99f) return true;
      if (!again) break;
      have_last = true;
    }
  } else {
    while (true) {
      HitBuf<K> hb;
      hb.clear();
      bool overflow = false;
      {
        const Ray2 w = ray2(R.o, R.d);
        for (uint32_t p = 0; p < L.np + L.nf; ++p) {
          float t2[2], g2[2];
          PairT pt;
          unsigned m = leaf_pair_t<PACKED>(S, L, p, w, R.t_near, R.t_far, pt);  // padding never passes
          if (m) {
            m = test_pair_g(pt, m, t2, g2);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              const uint32_t ik = 2 * p + k;
              if (((m >> k) & 1u) && (!have_last || t2[k] > last_t || (t2[k] == last_t && ik > last_i)))
                overflow |= hb.insert(t2[k], g2[k], ik);
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (hb.t[k] == __int_as_float(0x7f800000)) break;
        const uint32_t gid = leaf_gid<PACKED>(S, L, hb.i[k]);
        if (gid >= S.n_gauss) {
          atomicOr(status, kStatusBadId);
          return true;
        }
        blend_hit<PACKED>(S, R, hb.t[k], hb.g[k], gid);
        if (R.A > 0.99f) return true;
      }
      if (!overflow) break;
      have_last = true;
      last_t = hb.t[K - 1];
      last_i = hb.i[K - 1];
    }
  }
  if (R.t_far >= R.t_scene_far) return true;
  if (R.quant == 0) {
    R.cur = 0;
    R.t_near = R.t_far;
    R.t_far = R.t_scene_far;
  } else {
    const uint32_t id = s_id[R.top][tid];
    const float tm = s_t[R.top][tid];
    if (R.top == 0) R.top = kStack;
    --R.top;
    --R.quant;
    R.cur = id;
    R.t_near = R.t_far;
    R.t_far = tm;
  }
  return false;
}

// ------------------------------------------------------------ warp packets
// Packet traversal of one warp tile (32 rays): the warp walks the tree together.
// Primary rays of a tile share the eye point and, away from the image lines
// where a direction component changes sign, the sign of every direction
// component, so the front-to-back child order at a node is the same for all
// of them.  Each lane keeps its own interval and makes the per-ray decision
// of leaf_step (near child when t_split > t_near, far child when t_split <=
// t_near or t_split < t_far); the warp enters a child when any lane needs it
// and masks the others there.  A lane therefore meets exactly its own leaves,
// in its own order, with its own [t_near, t_far), and the leaf's records are
// warp-uniform loads.  Stack entries: (node, lane mask) per warp and
// (t_near, t_far) per lane, a ring of kStack entries; when the ring has lost
// entries the unfinished lanes restart at the root from the end of their
// last leaf, as the per-ray short stack does.
struct PktEnt {
  uint32_t node, mask;
};

// Leaf L for the lanes with part set; every lane runs the same candidate
// loop (lanes without part test against an empty interval).  With LPR > 1
// the lanes of each group split the leaf's candidates and take the group's
// hits in key order.  Inside the leaf a ray stops compositing once
// A > 0.99.  Returns false on a bad Gaussian ID (status set).
template <int K, bool PACKED, int LPR>
__device__ __forceinline__ bool pkt_leaf(const FastView& S, const LeafRef& L, Ray& R, bool part,
                                         uint32_t* status) {
  const unsigned full = 0xFFFFFFFFu;
  const float kInf = __int_as_float(0x7f800000);
  bool have_last = false, ok = true;
  float last_t = 0.f;
  uint32_t last_i = 0;
  bool more = part;
  while (__any_sync(full, more)) {
    HitBuf<K> hb;
    const bool overflow =
        scan_share<K, PACKED, LPR>(S, L, R, more ? R.t_near : kInf, full, have_last, last_t, last_i, hb);
    if constexpr (LPR > 1) {
      const bool again = take_group_hits<K, PACKED, LPR>(S, L, R, hb, overflow, full, more, ok, last_t, last_i,
                                                         status);
      more = more && ok && again && !(R.A > 0.99f);
    } else {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (hb.t[k] == kInf || R.A > 0.99f) break;
        const uint32_t gid = leaf_gid<PACKED>(S, L, hb.i[k]);
        if (gid >= S.n_gauss) {
          atomicOr(status, kStatusBadId);
          ok = false;
          break;
        }
        blend_hit<PACKED>(S, R, hb.t[k], hb.g[k], gid);
      }
      more = more && ok && overflow && !(R.A > 0.99f);
      last_t = hb.t[K - 1];
      last_i = hb.i[K - 1];
    }
    have_last = true;
  }
  return ok;
}

// Trace the warp's rays as one packet.  live: the lane's ray entered the
// scene box; sgn: bit a = sign of direction component a (warp-uniform).
template <int K, bool PACKED, int LPR>
__device__ __forceinline__ void pkt_trace(const FastView& S, Ray& R, bool live, unsigned sgn,
                                          uint32_t (*s_tn)[kThreads], float (*s_tf)[kThreads],
                                          PktEnt (*s_ent)[kWarps], int tid, int warp, uint32_t* status) {
  const unsigned full = 0xFFFFFFFFu;
  bool act = live, done = !live;
  float t_done = R.t_near;  // end of the part of the ray already composited
  uint32_t cur = 0, steps = 0;
  unsigned top = kStack - 1, quant = 0;
  while (true) {
    if (++steps > kMaxRaySteps) {
      if ((tid & 31) == 0) atomicOr(status, kStatusStepLimit);
      break;
    }
    uint2 nd = __ldg(S.nodes + cur);
    bool leaf = true;
    while ((nd.x & 7u) != 3u) {
      const uint32_t child = nd.x >> 3, axis = nd.x & 3u;
      const unsigned sign = (sgn >> axis) & 1u;
      const float t_split = (__uint_as_float(nd.y) - sel3(R.o, axis)) * sel3(R.inv, axis);
      const bool wn = act && !(t_split <= R.t_near);
      const bool wf = act && ((t_split <= R.t_near) || (t_split < R.t_far));
      const unsigned bn = __ballot_sync(full, wn), bf = __ballot_sync(full, wf);
      if (bn && bf) {
        if (++top == kStack) top = 0;
        quant = min(quant + 1, (unsigned)kStack);
        s_ent[top][warp] = PktEnt{child + (sign ^ 1u), bf};
        s_tn[top][tid] = __float_as_uint(wn ? t_split : R.t_near);
        s_tf[top][tid] = R.t_far;
        if (wn && wf) R.t_far = t_split;
        act = wn;
        cur = child + sign;
      } else if (bn) {
        cur = child + sign;
      } else if (bf) {
        cur = child + (sign ^ 1u);
      } else {
        leaf = false;
        break;
      }
      nd = __ldg(S.nodes + cur);
    }
    if (leaf) {
      const LeafRef L = leaf_ref<PACKED>(S, cur, nd);
      if (!leaf_in_bounds(S, L)) {
        if ((tid & 31) == 0) atomicOr(status, kStatusBadLeaf);
        break;
      }
      const bool part = act && !done;
      if (__any_sync(full, part)) {
        if (!pkt_leaf<K, PACKED, LPR>(S, L, R, part, status)) done = true;
        if (part) {
          t_done = R.t_far;
          // inside a leaf only A > 0.99 stops a ray; at a leaf boundary the
          // walk goes on only while A < 0.99 (A == 0.99 stops here)
          if (!(R.A < 0.99f) || R.t_far >= R.t_scene_far) done = true;
        }
      }
    }
    // next subtree: pop entries until one holds an unfinished lane
    bool found = false;
    while (quant > 0) {
      const PktEnt e = s_ent[top][warp];
      const float tn = __uint_as_float(s_tn[top][tid]), tf = s_tf[top][tid];
      if (top == 0) top = kStack;
      --top;
      --quant;
      act = ((e.mask >> (tid & 31)) & 1u) && !done;
      if (act) {
        R.t_near = tn;
        R.t_far = tf;
      }
      if (__any_sync(full, act)) {
        cur = e.node;
        found = true;
        break;
      }
    }
    if (!found) {
      // the ring lost entries: unfinished lanes restart at the root
      act = !done;
      if (!__any_sync(full, act)) break;
      cur = 0;
      if (act) {
        R.t_near = t_done;
        R.t_far = R.t_scene_far;
      }
    }
  }
}

__device__ __forceinline__ int find_view(const ViewDesc* views, int n_views, uint32_t item, int sched) {
  int lo = 0, hi = n_views - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const uint32_t b = sched == KDGR_SCHED_WARP_TILES ? __ldg(&views[mid].wt_base) : __ldg(&views[mid].cb_base);
    if (b <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Store the ray of pixel (x, y) of view V.
__device__ __forceinline__ void store_px(const ViewDesc& V, int x, int y, const Ray& R, float* rgb, float* alpha_out,
                                         float* depth_out) {
  const int W = __ldg(&V.W), H = __ldg(&V.H);
  const size_t idx = (size_t)__ldg(&V.out_off) + (size_t)(H - 1 - y) * W + x;  // rows flipped per view
  const float4 v = *acc_slot();
  rgb[3 * idx] = v.x;
  rgb[3 * idx + 1] = v.y;
  rgb[3 * idx + 2] = v.z;
  if (alpha_out) alpha_out[idx] = R.A;
  if (depth_out) depth_out[idx] = v.w;
}

// Render the ray of pixel (x, y) of view V to completion and store it.
// PKT: warp packets (every lane of the warp calls this together);
// otherwise one independent ray per lane.  With LPR > 1 each group of LPR
// consecutive lanes has the same pixel and its first lane stores it.
template <int K, bool PACKED, bool PKT, int LPR>
__device__ __forceinline__ void render_px(const FastView& S, const ViewDesc& V, int x, int y,
                                          uint32_t (*s_id)[kThreads], float (*s_t)[kThreads],
                                          PktEnt (*s_ent)[kWarps], int tid, float* rgb, float* alpha_out,
                                          float* depth_out, uint32_t* status) {
  const int W = __ldg(&V.W), H = __ldg(&V.H);
  if constexpr (PKT) {
    const bool inimg = x < W && y < H;
    Ray R;
    const bool live = ray_init(S, V.cam, inimg ? x : 0, inimg ? y : 0, R) && inimg;
    // one packet per direction-sign pattern among the warp's rays (almost
    // always one; two or more only for tiles on a sign-change line)
    const unsigned my_sgn = (__float_as_uint(R.inv.x) >> 31) | ((__float_as_uint(R.inv.y) >> 31) << 1) |
                            ((__float_as_uint(R.inv.z) >> 31) << 2);
    unsigned pending = __ballot_sync(0xFFFFFFFFu, live);
    while (pending) {
      const unsigned sgn = __shfl_sync(0xFFFFFFFFu, my_sgn, __ffs(pending) - 1);
      const bool in = live && my_sgn == sgn && ((pending >> (tid & 31)) & 1u);
      pending &= ~__ballot_sync(0xFFFFFFFFu, in);
      pkt_trace<K, PACKED, LPR>(S, R, in, sgn, s_id, s_t, s_ent, tid, tid >> 5, status);
    }
    if (!inimg || (tid & (LPR - 1)) != 0) return;
    store_px(V, x, y, R, rgb, alpha_out, depth_out);
  } else {
    if (x >= W || y >= H) return;
    Ray R;
    if (ray_init(S, V.cam, x, y, R)) {
      while (R.A < 0.99f && !leaf_step<K, PACKED, LPR>(S, s_id, s_t, tid, R, status)) {
      }
    }
    if ((tid & (LPR - 1)) != 0) return;
    store_px(V, x, y, R, rgb, alpha_out, depth_out);
  }
}

// Pixel of lane `lane` in quarter q (0..3) of the 16x8 block whose top-left
// pixel is (bx, by), for the warp tile shape (KDGR_TILE_*): 8x4 tiles in a
// 2x2 arrangement, 4x8 tiles side by side, or 16x2 tiles stacked.
__device__ __forceinline__ void block_pixel(int tile, int bx, int by, int q, int lane, int& x, int& y) {
  if (tile == KDGR_TILE_4X8) {
    x = bx + 4 * q + (lane & 3);
    y = by + (lane >> 2);
  } else if (tile == KDGR_TILE_16X2) {
    x = bx + (lane & 15);
    y = by + 2 * q + (lane >> 4);
  } else {
    x = bx + (q & 1) * kTileW + (lane & 7);
    y = by + (q >> 1) * kTileH + (lane >> 3);
  }
}

// Pixel of lane `lane` in item q (0 .. 4 LPR - 1) of the 16x8 block at
// (bx, by) when LPR lanes share a ray: the block is cut into 4 x (8 / LPR)
// tiles of 32 / LPR rays, 4 across and LPR down.
template <int LPR>
__device__ __forceinline__ void group_pixel(int bx, int by, int q, int lane, int& x, int& y) {
  const int gi = lane / LPR;
  x = bx + 4 * (q & 3) + (gi & 3);
  y = by + (8 / LPR) * (q >> 2) + (gi >> 2);
}

// Persistent kernel.  Schedules (include/kdgr.h):
//   WARP_TILES: each warp takes `chunk` 8x4 tiles from the global queue;
//   WARP_STRIPS: each warp takes the next quarter of a 16x8 block of
//               its SM's strip of the block list, then steals from the
//               following strips;
//   CTA_BLOCKS: each CTA takes `chunk` 16x8 blocks (barrier per block) and
//               its four warps render the four quarters, so the rays sharing
//               the SM's L1 are neighbours.
// MINB caps registers so that MINB CTAs fit per SM (0: compiler's choice).
// Strip k of n over total items: [total * k / n, total * (k + 1) / n).
__device__ __forceinline__ uint32_t strip_lo(uint32_t total, uint32_t n, uint32_t k) {
  return (uint32_t)((uint64_t)total * k / n);
}

// The first strip after k in visiting order (k + 1, k + 2, ... mod n) whose
// claim counter (queue word 1 + j) is still below its size, or n when every
// strip is exhausted; called by a whole warp.  The lanes read the counters
// together, from L2 (they move by atomics, so not through L1), one load
// each per 32 strips, all issued before the first vote.  Trying the strips
// one claim at a time instead cost a warp up to n sequential atomic round
// trips at the end of a launch, after its last item.  A strip read as open
// may be exhausted by the time the caller claims from it; the caller then
// asks again, and since a counter only grows, every failed claim closes a
// strip for good.
__device__ __forceinline__ uint32_t next_open_strip(const uint32_t* queue, uint32_t total, uint32_t n, uint32_t k,
                                                    unsigned lane) {
  constexpr int kRounds = (kMaxStrips + 31) / 32;
  bool open[kRounds];
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    const uint32_t off = 1u + 32u * r + lane;  // off == n is k itself
    open[r] = false;
    if (off <= n) {
      const uint32_t j = (k + off) % n;
      open[r] = __ldcg(queue + 1 + j) < strip_lo(total, n, j + 1) - strip_lo(total, n, j);
    }
  }
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, open[r]);
    if (m) return (k + 1u + 32u * r + (uint32_t)(__ffs(m) - 1)) % n;
  }
  return n;
}

template <bool PACKED, int SCHED, int MINB, int KB, bool PKT, int LPR>
__global__ void __launch_bounds__(kThreads, MINB) k_render_batch(FastView S, const ViewDesc* __restrict__ views,
                                                                 int n_views, uint32_t total_items,
                                                                 float* __restrict__ rgb,
                                                                 float* __restrict__ alpha_out,
                                                                 float* __restrict__ depth_out, uint32_t* queue,
                                                                 uint32_t* status, int chunk, int tile) {
  __shared__ uint32_t s_id[kStack][kThreads];
  __shared__ float s_t[kStack][kThreads];
  __shared__ PktEnt s_ent[kStack][kWarps];
  __shared__ uint32_t s_work;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if constexpr (SCHED == KDGR_SCHED_WARP_STRIPS) {
    // items are quarters of 16x8 blocks (warp tiles in block order), or with
    // LPR lanes per ray 4 LPR tiles of 32 / LPR rays; each warp claims the
    // next item of its SM's strip, no CTA barrier
    uint32_t smid;
    asm("mov.u32 %0, %%smid;" : "=r"(smid));
    const uint32_t n = (uint32_t)chunk;  // number of strips
    uint32_t k = smid % n, fails = 0;
    while (fails <= n) {  // a warp's claims fail at most once per strip
      const uint32_t b0 = strip_lo(total_items, n, k), b1 = strip_lo(total_items, n, k + 1);
      uint32_t it = 0;
      if (lane == 0) it = b0 + atomicAdd(queue + 1 + k, 1u);
      it = __shfl_sync(0xFFFFFFFFu, it, 0);
      if (it >= b1) {
        ++fails;
        k = next_open_strip(queue, total_items, n, k, (unsigned)lane);
        if (k >= n) break;
        continue;
      }
      const uint32_t blk = it / (4u * LPR), q = it % (4u * LPR);
      const ViewDesc& V = views[find_view(views, n_views, blk, KDGR_SCHED_CTA_BLOCKS)];
      const uint32_t lb = blk - __ldg(&V.cb_base), nx = __ldg(&V.cb_x);
      int x, y;
      if constexpr (LPR == 1) block_pixel(tile, (int)(lb % nx) * kBlockW, (int)(lb / nx) * kBlockH, (int)q, lane, x, y);
      else group_pixel<LPR>((int)(lb % nx) * kBlockW, (int)(lb / nx) * kBlockH, (int)q, lane, x, y);
      render_px<KB, PACKED, PKT, LPR>(S, V, x, y, s_id, s_t, s_ent, tid, rgb, alpha_out, depth_out,
                                      status);
    }
  } else if constexpr (SCHED == KDGR_SCHED_SM_STRIPS) {
    // strip of this SM: [total * k / n, total * (k + 1) / n), k = smid mod n
    __shared__ uint32_t s_strip;
    uint32_t smid;
    asm("mov.u32 %0, %%smid;" : "=r"(smid));
    const uint32_t n = (uint32_t)chunk;  // number of strips (the SM count; chunk is reused for it)
    if (tid == 0) s_strip = smid % n;
    while (true) {
      __syncthreads();
      if (warp == 0) {
        // claim the next item of this CTA's strip, or move on to the next
        // strip with items left (a failed claim closes its strip for good)
        uint32_t k = s_strip, item = 0xFFFFFFFFu;
        for (uint32_t fails = 0; fails <= n; ++fails) {
          const uint32_t b0 = strip_lo(total_items, n, k), b1 = strip_lo(total_items, n, k + 1);
          uint32_t it = 0;
          if (lane == 0) it = b0 + atomicAdd(queue + 1 + k, 1u);
          it = __shfl_sync(0xFFFFFFFFu, it, 0);
          if (it < b1) {
            item = it;
            break;
          }
          k = next_open_strip(queue, total_items, n, k, (unsigned)lane);
          if (k >= n) break;
        }
        if (lane == 0) {
          s_work = item;
          if (k < n) s_strip = k;
        }
      }
      __syncthreads();
      const uint32_t item = s_work;
      if (item == 0xFFFFFFFFu) break;
      const ViewDesc& V = views[find_view(views, n_views, item, KDGR_SCHED_CTA_BLOCKS)];
      const uint32_t lb = item - __ldg(&V.cb_base), nx = __ldg(&V.cb_x);
      int x, y;
      block_pixel(tile, (int)(lb % nx) * kBlockW, (int)(lb / nx) * kBlockH, warp, lane, x, y);
      render_px<KB, PACKED, PKT, 1>(S, V, x, y, s_id, s_t, s_ent, tid, rgb, alpha_out, depth_out, status);
    }
  } else {
    while (true) {
      uint32_t first;
      if constexpr (SCHED == KDGR_SCHED_CTA_BLOCKS) {
        __syncthreads();
        if (tid == 0) s_work = atomicAdd(queue, (uint32_t)chunk);
        __syncthreads();
        first = s_work;
      } else {
        uint32_t f = 0;
        if (lane == 0) f = atomicAdd(queue, (uint32_t)chunk);
        first = __shfl_sync(0xFFFFFFFFu, f, 0);
      }
      if (first >= total_items) break;
      const uint32_t last = min(first + (uint32_t)chunk, total_items);
      for (uint32_t item = first; item < last; ++item) {
        const ViewDesc& V = views[find_view(views, n_views, item, SCHED)];
        int x, y;
        if (SCHED == KDGR_SCHED_CTA_BLOCKS) {
          const uint32_t lb = item - __ldg(&V.cb_base), nx = __ldg(&V.cb_x);
          block_pixel(tile, (int)(lb % nx) * kBlockW, (int)(lb / nx) * kBlockH, warp, lane, x, y);
        } else {
          const uint32_t lt = item - __ldg(&V.wt_base), nx = __ldg(&V.wt_x);
          x = (int)(lt % nx) * kTileW + (lane & 7);
          y = (int)(lt / nx) * kTileH + (lane >> 3);
        }
        render_px<KB, PACKED, PKT, 1>(S, V, x, y, s_id, s_t, s_ent, tid, rgb, alpha_out, depth_out, status);
      }
    }
  }
}

// Multi-scene form of the warp-strip schedule for the serving loop: every
// view names a scene slot and each warp renders its quarter-block against
// that slot's arrays (the slot table travels in the launch parameters, so
// the warp-uniform field reads hit the constant cache).  One persistent launch
// serves the requests of all resident scenes queued in a tick.  Items are
// quarters of 16x8 blocks; queue word 1 + k counts the claims of strip k.
// outs[v] is view v's output base (the device arena, or a request's
// page-locked host buffer); the view's out_off counts pixels from it.
template <bool PACKED>
__global__ void __launch_bounds__(kThreads, 8) k_render_multi(const __grid_constant__ SceneTable scenes,
                                                              const ViewDesc* __restrict__ views, int n_views,
                                                              uint32_t total_items, float* const* __restrict__ outs,
                                                              uint32_t* queue, uint32_t* status, int n_strips) {
  __shared__ uint32_t s_id[kStack][kThreads];
  __shared__ float s_t[kStack][kThreads];
  __shared__ PktEnt s_ent[kStack][kWarps];
  const int tid = threadIdx.x, lane = tid & 31;
  uint32_t smid;
  asm("mov.u32 %0, %%smid;" : "=r"(smid));
  const uint32_t n = (uint32_t)n_strips;
  uint32_t k = smid % n, fails = 0;
  while (fails <= n) {  // a warp's claims fail at most once per strip
    const uint32_t b0 = strip_lo(total_items, n, k), b1 = strip_lo(total_items, n, k + 1);
    uint32_t it = 0;
    if (lane == 0) it = b0 + atomicAdd(queue + 1 + k, 1u);
    it = __shfl_sync(0xFFFFFFFFu, it, 0);
    if (it >= b1) {
      ++fails;
      k = next_open_strip(queue, total_items, n, k, (unsigned)lane);
      if (k >= n) break;
      continue;
    }
    const uint32_t blk = it >> 2;
    const int vi = find_view(views, n_views, blk, KDGR_SCHED_CTA_BLOCKS);
    const ViewDesc& V = views[vi];
    const FastView& S = scenes.s[__ldg(&V.scene) & (kSceneSlots - 1)];
    float* const rgb = outs[vi];
    const uint32_t lb = blk - __ldg(&V.cb_base), nx = __ldg(&V.cb_x);
    int x, y;
    block_pixel(KDGR_TILE_8X4, (int)(lb % nx) * kBlockW, (int)(lb / nx) * kBlockH, (int)(it & 3u), lane, x, y);
    render_px<kHits, PACKED, true, 1>(S, V, x, y, s_id, s_t, s_ent, tid, rgb, nullptr, nullptr, status);
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
                          int, int);

template <bool PACKED, int SCHED, int KB, bool PKT, int LPR>
KernelFn pick_minb(int minb) {
  if (minb >= 8) return k_render_batch<PACKED, SCHED, 8, KB, PKT, LPR>;
  if (minb >= 6) return k_render_batch<PACKED, SCHED, 6, KB, PKT, LPR>;
  return k_render_batch<PACKED, SCHED, 0, KB, PKT, LPR>;
}

// Lanes per ray: 32 / rays_per_warp (warp-strip schedule only).
int lanes_per_ray(const kdgr_batch_config& c) {
  return c.rays_per_warp == 8 ? 4 : c.rays_per_warp == 16 ? 2 : 1;
}

template <bool PACKED, int KB, bool PKT>
KernelFn pick_sched_k(const kdgr_batch_config& c) {
  if (c.schedule == KDGR_SCHED_CTA_BLOCKS) return pick_minb<PACKED, KDGR_SCHED_CTA_BLOCKS, KB, PKT, 1>(c.min_blocks);
  if (c.schedule == KDGR_SCHED_SM_STRIPS) return pick_minb<PACKED, KDGR_SCHED_SM_STRIPS, KB, PKT, 1>(c.min_blocks);
  if (c.schedule == KDGR_SCHED_WARP_STRIPS) {
    if (lanes_per_ray(c) == 4) return pick_minb<PACKED, KDGR_SCHED_WARP_STRIPS, KB, PKT, 4>(c.min_blocks);
    if (lanes_per_ray(c) == 2) return pick_minb<PACKED, KDGR_SCHED_WARP_STRIPS, KB, PKT, 2>(c.min_blocks);
    return pick_minb<PACKED, KDGR_SCHED_WARP_STRIPS, KB, PKT, 1>(c.min_blocks);
  }
  return pick_minb<PACKED, KDGR_SCHED_WARP_TILES, KB, PKT, 1>(c.min_blocks);
}

template <bool PACKED, bool PKT>
KernelFn pick_sched_t(const kdgr_batch_config& c) {
  return c.hit_buffer == 8 ? pick_sched_k<PACKED, 8, PKT>(c) : pick_sched_k<PACKED, kHits, PKT>(c);
}

template <bool PACKED>
KernelFn pick_sched(const kdgr_batch_config& c) {
  return c.traversal == KDGR_TRAV_RAY ? pick_sched_t<PACKED, false>(c) : pick_sched_t<PACKED, true>(c);
}

KernelFn pick_kernel(const kdgr_batch_config& c) {
  return c.precision ? pick_sched<true>(c) : pick_sched<false>(c);
}

// SM count of the current device, cached per device.  Threads may race on
// the first query of a device; they all store the same value.
constexpr int kMaxSmCacheDevices = 64;
std::atomic<int> g_num_sms[kMaxSmCacheDevices];

int num_sms() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  const bool cacheable = dev >= 0 && dev < kMaxSmCacheDevices;
  if (cacheable) n = g_num_sms[dev].load(std::memory_order_relaxed);
  if (n > 0) return n;
  if (dev < 0 || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
  if (cacheable) g_num_sms[dev].store(n, std::memory_order_relaxed);
  return n;
}

// Resident 128-thread CTAs per SM of a kernel on the current device (at
// least 1), cached per kernel and device: the query costs microseconds and
// every batched launch needs it.
cudaError_t resident_ctas(const void* fn, int* out) {
  static std::mutex mu;
  static std::vector<std::pair<std::pair<const void*, int>, int>> cache;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lk(mu);
    for (const auto& it : cache)
      if (it.first.first == fn && it.first.second == dev) {
        *out = it.second;
        return cudaSuccess;
      }
  }
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kThreads, 0);
  if (e != cudaSuccess) return e;
  occ = occ > 0 ? occ : 1;
  std::lock_guard<std::mutex> lk(mu);
  cache.push_back({{fn, dev}, occ});
  *out = occ;
  return cudaSuccess;
}
template <typename F>
cudaError_t resident_ctas(F* fn, int* out) {
  return resident_ctas(reinterpret_cast<const void*>(fn), out);
}

}  // namespace

// Host: view table and total tile count for a list of views.
int make_view_table(const kdgr_view* views, int n_views, std::vector<ViewDesc>& out, uint32_t totals[3]) {
  out.resize(n_views);
  return fill_view_table(views, n_views, out.data(), totals);
}

// The view table of n_views views into a caller-provided array (no
// allocation); make_view_table and the allocation-free entry point share it.
int fill_view_table(const kdgr_view* views, int n_views, ViewDesc* out, uint32_t totals[3]) {
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
    d.scene = 0;
    d.pad = 0;
    wbase += (uint64_t)d.wt_x * (uint64_t)((kv.height + kTileH - 1) / kTileH);
    cbase += (uint64_t)d.cb_x * (uint64_t)((kv.height + kBlockH - 1) / kBlockH);
    if (wbase > 0xF0000000ull) {
      set_error("batch too large: more than 2^32 tiles");
      return KDGR_ERR_LIMIT;
    }
  }
  totals[0] = (uint32_t)wbase;
  totals[1] = (uint32_t)cbase;
  totals[2] = 0;
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
  if (c.schedule != KDGR_SCHED_WARP_TILES && c.schedule != KDGR_SCHED_CTA_BLOCKS &&
      c.schedule != KDGR_SCHED_SM_STRIPS && c.schedule != KDGR_SCHED_WARP_STRIPS) {
    set_error("batch config: unknown schedule");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.hit_buffer != 0 && c.hit_buffer != 4 && c.hit_buffer != 8) {
    set_error("batch config: hit_buffer must be 0, 4 or 8");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.min_blocks != 0 && c.min_blocks != 6 && c.min_blocks != 8) {
    set_error("batch config: min_blocks must be 0, 6 or 8");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.tile_shape != KDGR_TILE_8X4 && c.tile_shape != KDGR_TILE_4X8 && c.tile_shape != KDGR_TILE_16X2) {
    set_error("batch config: tile_shape must be KDGR_TILE_8X4, KDGR_TILE_4X8 or KDGR_TILE_16X2");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.tile_shape != KDGR_TILE_8X4 && c.schedule == KDGR_SCHED_WARP_TILES) {
    set_error("batch config: the warp-tile schedule renders 8x4 tiles only");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.traversal != KDGR_TRAV_PACKET && c.traversal != KDGR_TRAV_RAY) {
    set_error("batch config: traversal must be KDGR_TRAV_PACKET or KDGR_TRAV_RAY");
    return KDGR_ERR_INVALID_ARG;
  }
  if (c.rays_per_warp != 0 && c.rays_per_warp != 32 && c.rays_per_warp != 16 && c.rays_per_warp != 8) {
    set_error("batch config: rays_per_warp must be 0, 32, 16 or 8");
    return KDGR_ERR_INVALID_ARG;
  }
  if (lanes_per_ray(c) > 1 && (c.schedule != KDGR_SCHED_WARP_STRIPS || c.tile_shape != KDGR_TILE_8X4)) {
    set_error("batch config: 16 or 8 rays per warp need the warp-strip schedule and the default tile shape");
    return KDGR_ERR_INVALID_ARG;
  }
  return KDGR_OK;
}

// Launch the persistent kernel.  `queue` must read 0 when the kernel starts.
cudaError_t launch_batch(kdgr_scene_t s, const kdgr_batch_config& c, const ViewDesc* d_views, int n_views,
                         const uint32_t totals[3], float* rgb, float* alpha, float* depth, uint32_t* queue,
                         cudaStream_t st) {
  const uint32_t total_tiles = totals[0], total_blocks = totals[1];
  KernelFn fn = pick_kernel(c);
  int per_sm = c.blocks_per_sm;
  if (per_sm <= 0) {
    cudaError_t e = resident_ctas(fn, &per_sm);
    if (e != cudaSuccess) return e;
  }
  const bool warp_strips = c.schedule == KDGR_SCHED_WARP_STRIPS;
  const bool per_warp = c.schedule == KDGR_SCHED_WARP_TILES || warp_strips;
  if (warp_strips && total_blocks > 0x3FFFFFFFu) return cudaErrorInvalidValue;
  const uint32_t lpr = (uint32_t)lanes_per_ray(c);
  if (warp_strips && total_blocks > 0x3FFFFFFFu / lpr) return cudaErrorInvalidValue;
  const uint32_t total = warp_strips ? 4u * lpr * total_blocks : per_warp ? total_tiles : total_blocks;
  // SM strips: the kernel's `chunk` argument carries the number of strips
  const bool strips = c.schedule == KDGR_SCHED_SM_STRIPS || warp_strips;
  const int chunk = strips ? std::min(num_sms(), kMaxStrips) : c.chunk;
  uint64_t blocks = (uint64_t)num_sms() * per_sm;
  const uint64_t grabs = strips ? total : ((uint64_t)total + chunk - 1) / chunk;
  const uint64_t cap = per_warp ? (grabs + kWarps - 1) / kWarps : grabs;
  if (blocks > cap) blocks = cap > 0 ? cap : 1;
  fn<<<(unsigned)blocks, kThreads, 0, st>>>(s->fast_view(c.precision != 0), d_views, n_views, total, rgb, alpha,
                                            depth, queue, s->d_status, chunk, c.tile_shape);
  return cudaGetLastError();
}

// The precision form from the device packing kernel's outputs (d_packed:
// FP32 mean + FP16 M per Gaussian; d_aniso: flagged Gaussians; BF16 SH and
// opacity already in the scene): the flagged Gaussians get FP64-precomputed
// factors (k_aniso_fp64) and each leaf is laid out as its plain entries in
// FP16 pairs followed by its flagged entries in FP32 pairs of a second stream.
int pack_precision(kdgr_scene_s* s, const float* d_rec, const float* d_giscl, const uint32_t* d_packed,
                   const uint8_t* d_aniso, const std::vector<uint32_t>& relaid,
                   const std::vector<uint32_t>& pair_gid, DevAlloc& A) {
  const size_t n = s->n_gauss;
  std::vector<uint8_t> flag(n);
  if (cudaMemcpy(flag.data(), d_aniso, n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return cuda_fail(cudaGetLastError(), "kdgr_scene_create: aniso flags");
  std::vector<uint32_t> aidx(n, 0xFFFFFFFFu);
  uint32_t n_aniso = 0;
  for (size_t i = 0; i < n; ++i)
    if (flag[i]) aidx[i] = n_aniso++;
  // The packed form's leaf layout: per leaf its plain entries in FP16 pairs,
  // then its flagged entries in FP32 pairs of a second stream, both padded
  // to whole pairs; the leaf words and per-node aux words say where.
  std::vector<uint32_t> nodes_p(relaid), gid_plain, gid_flag;
  std::vector<uint32_t> aux(relaid.size(), 0u);
  std::vector<uint32_t> plain, flagged;
  for (size_t nd = 0; 2 * nd < relaid.size(); ++nd) {
    const uint32_t x = relaid[2 * nd];
    if ((x & 7u) != 3u) continue;
    const uint32_t cnt = x >> 3, e0 = 2 * relaid[2 * nd + 1];
    plain.clear();
    flagged.clear();
    for (uint32_t k = 0; k < cnt; ++k) {
      const uint32_t gid = pair_gid[e0 + k];
      (aidx[gid] == 0xFFFFFFFFu ? plain : flagged).push_back(gid);
    }
    nodes_p[2 * nd] = ((uint32_t)plain.size() << 3) | 3u;
    nodes_p[2 * nd + 1] = (uint32_t)(gid_plain.size() / 2);
    aux[2 * nd] = (uint32_t)(gid_flag.size() / 2);
    aux[2 * nd + 1] = (uint32_t)flagged.size();
    gid_plain.insert(gid_plain.end(), plain.begin(), plain.end());
    if (plain.size() & 1u) gid_plain.push_back(kPadGid);
    gid_flag.insert(gid_flag.end(), flagged.begin(), flagged.end());
    if (flagged.size() & 1u) gid_flag.push_back(kPadGid);
  }
  if (gid_plain.size() > 0xFFFFFFF0ull || gid_flag.size() > 0xFFFFFFF0ull) {
    set_error("kdgr_scene_create: more than 2^32 leaf entries after pair padding");
    return KDGR_ERR_LIMIT;
  }
  s->n_plain_entries = (uint32_t)gid_plain.size();
  s->n_flag_entries = (uint32_t)gid_flag.size();
  s->n_aniso = n_aniso;
  s->d_nodes_packed = A.alloc<uint2>(relaid.size() / 2);
  s->d_leaf_aux = A.alloc<uint2>(relaid.size() / 2);
  s->d_gid_plain = A.alloc<uint32_t>(gid_plain.size() + 2);
  s->d_gid_flag = A.alloc<uint32_t>(gid_flag.size() + 2);
  s->d_leaf_packed = A.alloc<uint4>(2 * (gid_plain.size() + 2));
  s->d_flag_pairs = A.alloc<float4>(3 * (gid_flag.size() + 2));
  if (A.err != cudaSuccess) return cuda_fail(A.err, "kdgr_scene_create: cudaMalloc (packed)");
  uint32_t* d_aidx = nullptr;
  float* d_src = nullptr;
  float4* d_table = nullptr;
  auto up = [](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  cudaError_t e = up(s->d_nodes_packed, nodes_p.data(), nodes_p.size() * 4);
  if (e == cudaSuccess) e = up(s->d_leaf_aux, aux.data(), aux.size() * 4);
  if (e == cudaSuccess) e = up(s->d_gid_plain, gid_plain.data(), gid_plain.size() * 4);
  if (e == cudaSuccess) e = up(s->d_gid_flag, gid_flag.data(), gid_flag.size() * 4);
  if (e == cudaSuccess) e = build_packed_pairs(s->d_gid_plain, s->n_plain_entries, d_packed, s->d_leaf_packed);
  if (e == cudaSuccess && n_aniso) {
    e = cudaMalloc(&d_src, 40ull * n_aniso);
    if (e == cudaSuccess) e = cudaMalloc(&d_table, 3 * sizeof(float4) * n_aniso);
    if (e == cudaSuccess) e = cudaMalloc(&d_aidx, aidx.size() * 4);
    if (e == cudaSuccess) e = up(d_aidx, aidx.data(), aidx.size() * 4);
    if (e == cudaSuccess) e = launch_gather_aniso(d_rec, d_giscl, d_aidx, (uint32_t)n, d_src, nullptr);
    if (e == cudaSuccess) {
      k_aniso_fp64<<<(n_aniso + 127) / 128, 128>>>(d_src, n_aniso, d_table);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = build_flag_pairs(s->d_gid_flag, s->n_flag_entries, d_aidx, d_table, s->d_flag_pairs);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  for (void* q : {(void*)d_src, (void*)d_table, (void*)d_aidx})
    if (q) cudaFree(q);
  if (e != cudaSuccess) return cuda_fail(e, "kdgr_scene_create: packed upload");
  return KDGR_OK;
}

// Pair p of the packed plain records (layout at PPairRec) from the
// per-Gaussian staging words: mean x, y, z (FP32), half2 (M22, 0),
// half2 (M00, M01), (M02, M10), (M11, M12), (M20, M21).  Padding entries
// are zero.
__global__ void k_build_ppairs(const uint32_t* __restrict__ gid, uint32_t n, const uint32_t* __restrict__ src,
                               uint4* __restrict__ out) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n / 2) return;
  uint32_t a[8], b[8];
  const uint32_t g0 = __ldg(gid + 2 * p), g1 = __ldg(gid + 2 * p + 1);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    a[i] = g0 == kPadGid ? 0u : __ldg(src + 8ull * g0 + i);
    b[i] = g1 == kPadGid ? 0u : __ldg(src + 8ull * g1 + i);
  }
  auto lo = [](uint32_t x) { return x & 0xFFFFu; };
  auto hi = [](uint32_t x) { return x >> 16; };
  auto h2 = [](uint32_t l, uint32_t h) { return l | (h << 16); };
  out[4 * p] = make_uint4(a[0], b[0], a[1], b[1]);
  out[4 * p + 1] = make_uint4(a[2], b[2], h2(lo(a[4]), lo(b[4])), h2(hi(a[4]), hi(b[4])));
  out[4 * p + 2] = make_uint4(h2(lo(a[5]), lo(b[5])), h2(hi(a[5]), hi(b[5])), h2(lo(a[6]), lo(b[6])),
                              h2(hi(a[6]), hi(b[6])));
  out[4 * p + 3] = make_uint4(h2(lo(a[7]), lo(b[7])), h2(hi(a[7]), hi(b[7])), h2(lo(a[3]), lo(b[3])), 0u);
}

// Pair p of the packed form's flagged stream, in the FP32 pair layout, from
// the FP64-precomputed rows (M row i, b_i) of Gaussian-order table entry
// aidx[gid]; padding entries are zero.
__global__ void k_build_flag_pairs(const uint32_t* __restrict__ gid, uint32_t n, const uint32_t* __restrict__ aidx,
                                   const float4* __restrict__ table, float4* __restrict__ pairs) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n / 2) return;
  const uint32_t g0 = __ldg(gid + 2 * p), g1 = __ldg(gid + 2 * p + 1);
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 a = g0 == kPadGid ? z : __ldg(table + 3ull * __ldg(aidx + g0) + i);
    const float4 b = g1 == kPadGid ? z : __ldg(table + 3ull * __ldg(aidx + g1) + i);
    pairs[6 * p + 2 * i] = make_float4(a.x, b.x, a.y, b.y);
    pairs[6 * p + 2 * i + 1] = make_float4(a.z, b.z, a.w, b.w);
  }
}

// Pair p of the FP32 leaf records: entries 2p and 2p+1, rows of M and b
// interleaved lo/hi; a padding entry gets zeros.
__global__ void k_build_pairs(const uint32_t* __restrict__ gid, uint32_t n, const float4* __restrict__ test,
                              float4* __restrict__ pairs) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n / 2) return;
  const uint32_t g0 = __ldg(gid + 2 * p), g1 = __ldg(gid + 2 * p + 1);
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 a = g0 == kPadGid ? z : __ldg(test + 3ull * g0 + i);
    const float4 b = g1 == kPadGid ? z : __ldg(test + 3ull * g1 + i);
    pairs[6 * p + 2 * i] = make_float4(a.x, b.x, a.y, b.y);
    pairs[6 * p + 2 * i + 1] = make_float4(a.z, b.z, a.w, b.w);
  }
}

cudaError_t build_leaf_pairs(const uint32_t* d_gid, uint32_t n_entries, const float4* test, float4* pairs) {
  if (n_entries == 0) return cudaSuccess;
  const size_t np = (size_t)n_entries / 2;
  k_build_pairs<<<(unsigned)((np + 255) / 256), 256>>>(d_gid, n_entries, test, pairs);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e;
}

cudaError_t build_packed_pairs(const uint32_t* d_gid, uint32_t n_entries, const uint32_t* src, uint4* pairs) {
  if (n_entries == 0) return cudaSuccess;
  const size_t np = (size_t)n_entries / 2;
  k_build_ppairs<<<(unsigned)((np + 255) / 256), 256>>>(d_gid, n_entries, src, pairs);
  return cudaGetLastError();
}

cudaError_t build_flag_pairs(const uint32_t* d_gid, uint32_t n_entries, const uint32_t* aidx, const float4* table,
                             float4* pairs) {
  if (n_entries == 0) return cudaSuccess;
  const size_t np = (size_t)n_entries / 2;
  k_build_flag_pairs<<<(unsigned)((np + 255) / 256), 256>>>(d_gid, n_entries, aidx, table, pairs);
  return cudaGetLastError();
}

int batch_sms() { return num_sms(); }

namespace {
constexpr int kStageViews = 256;
struct ViewStage {
  ViewDesc views[kStageViews];
  int32_t n_views;
};
static_assert(sizeof(ViewStage) <= 32764, "kernel parameters are limited to 32,764 bytes");
static_assert(kQueueBytes / sizeof(uint32_t) <= 256, "queue words are zeroed by one 256-thread block");

__global__ void __launch_bounds__(256) k_stage_views(const __grid_constant__ ViewStage p, ViewDesc* table,
                                                     uint32_t* queue) {
  const int i = threadIdx.x;
  if (i < p.n_views) table[i] = p.views[i];
  if (i < (int)(kQueueBytes / sizeof(uint32_t))) queue[i] = 0u;
}
}  // namespace

cudaError_t stage_views(const ViewDesc* views, int n_views, ViewDesc* d_views, uint32_t* d_queue, cudaStream_t st) {
  if (n_views < 0) return cudaErrorInvalidValue;
  if (n_views > kStageViews) {
    cudaError_t e = cudaMemcpyAsync(d_views, views, (size_t)n_views * sizeof(ViewDesc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_queue, 0, kQueueBytes, st);
    return e;
  }
  ViewStage p;
  p.n_views = n_views;
  std::memcpy(p.views, views, (size_t)n_views * sizeof(ViewDesc));
  k_stage_views<<<1, 256, 0, st>>>(p, d_views, d_queue);
  return cudaGetLastError();
}

cudaError_t launch_multi(const SceneTable& scenes, bool packed, const ViewDesc* d_views, int n_views,
                         uint32_t total_blocks, float* const* d_outs, uint32_t* queue, uint32_t* status,
                         cudaStream_t st) {
  auto fn = packed ? k_render_multi<true> : k_render_multi<false>;
  int occ = 0;
  cudaError_t e = resident_ctas(reinterpret_cast<const void*>(fn), &occ);
  if (e != cudaSuccess) return e;
  if (total_blocks > 0x3FFFFFFFu) return cudaErrorInvalidValue;
  const uint32_t quarters = 4u * total_blocks;
  uint64_t blocks = (uint64_t)num_sms() * (occ > 0 ? occ : 1);
  const uint64_t cap = ((uint64_t)quarters + kWarps - 1) / kWarps;
  if (blocks > cap) blocks = cap > 0 ? cap : 1;
  fn<<<(unsigned)blocks, kThreads, 0, st>>>(scenes, d_views, n_views, quarters, d_outs, queue, status,
                                            std::min(num_sms(), kMaxStrips));
  return cudaGetLastError();
}

}  // namespace kdgr
