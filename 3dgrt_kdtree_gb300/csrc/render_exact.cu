// render_exact.cu -- the plain drop-in render kernel (oracle-matching form).
//
// Replaces renderKernelGaussian_sortNode -> singlePassIntersectGaussian_
// sortNode_onlyShortStack (cudaRenderer.cu:2313-2390, 1488-1709) for the
// hybrid tree (PRIMITIVE_TYPE 2).  Per ray it performs the reference's
// operations in the reference's order, in IEEE round-to-nearest FP32 with no
// fused multiply-add (every operation is an explicit __f*_rn intrinsic), so
// the visited-leaf sequence, the hit sequence and the composited colour match
// the CPU oracle (oracle/oracle.cpp) bit for bit.  The documented deviations
// from the reference binary -- IEEE division instead of __fdividef, 1/sqrt
// instead of rsqrtf, the project exponential instead of CUDA expf -- are the
// oracle's as well.
//
// GB300 layout choices, none of which change a result:
//   * one thread per ray; a warp covers an 8x4 pixel tile, a 128-thread
//     block a 16x8 tile, so the 32 rays of a warp start coherent;
//   * the 12-entry ring short stack (cudaRenderer.cu:184-210, restart from
//     the root when it runs dry, :1694-1708) lives in shared memory laid out
//     [slot][thread], bank-conflict free;
//   * Gaussians are split SoA: a 64-byte test record (the fields the test
//     reads, with the reciprocal of the inverted scale precomputed by the same
//     IEEE division) and a separate 192-byte SH record read only for
//     composited hits;
//   * the reference collects every hit of a leaf into a 256-entry local array
//     (no overflow check, :1126-1133) and insertion-sorts it.  Here a K-entry
//     register buffer keeps the K smallest (t, leaf position) keys; a leaf
//     with more than K accepted hits is re-scanned for the next K keys, so
//     any leaf size gives the same stable t order with no overflow.
#include <cfloat>
#include <cstdint>

#include "device_common.cuh"
#include "kdgr_math.h"

namespace kdgr {
namespace {

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fq(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ F3 mk(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return mk(fa(a.x, b.x), fa(a.y, b.y), fa(a.z, b.z)); }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return mk(fs(a.x, b.x), fs(a.y, b.y), fs(a.z, b.z)); }
__device__ __forceinline__ F3 mulv(F3 a, F3 b) { return mk(fm(a.x, b.x), fm(a.y, b.y), fm(a.z, b.z)); }
__device__ __forceinline__ F3 muls(F3 a, float s) { return mk(fm(a.x, s), fm(a.y, s), fm(a.z, s)); }
__device__ __forceinline__ float dot(F3 a, F3 b) { return fa(fa(fm(a.x, b.x), fm(a.y, b.y)), fm(a.z, b.z)); }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
  return mk(fs(fm(a.y, b.z), fm(a.z, b.y)), fs(fm(a.z, b.x), fm(a.x, b.z)), fs(fm(a.x, b.y), fm(a.y, b.x)));
}

// quaternionWXYZToMatrixTranspose (cudaRenderer.cu:808-828)
__device__ __forceinline__ void quat_rt(float r, float x, float y, float z, F3 m[3]) {
  const float xx = fm(x, x), yy = fm(y, y), zz = fm(z, z);
  const float xy = fm(x, y), xz = fm(x, z), yz = fm(y, z);
  const float rx = fm(r, x), ry = fm(r, y), rz = fm(r, z);
  m[0] = mk(fs(1.f, fm(2.f, fa(yy, zz))), fm(2.f, fa(xy, rz)), fm(2.f, fs(xz, ry)));
  m[1] = mk(fm(2.f, fs(xy, rz)), fs(1.f, fm(2.f, fa(xx, zz))), fm(2.f, fa(yz, rx)));
  m[2] = mk(fm(2.f, fa(xz, ry)), fm(2.f, fs(yz, rx)), fs(1.f, fm(2.f, fa(xx, yy))));
}
__device__ __forceinline__ F3 mat_mul(F3 p, const F3 m[3]) { return mk(dot(m[0], p), dot(m[1], p), dot(m[2], p)); }

// rayPrimIntersect with VOLUME_ISECT (cudaRenderer.cu:1070-1135).
__device__ __forceinline__ bool exact_test(F3 o, F3 d, const float4* __restrict__ rec, float t_near, float t_far,
                                           float* t_out, float* gray_out) {
  const float4 r0 = __ldg(rec), r1 = __ldg(rec + 1), r2 = __ldg(rec + 2), r3 = __ldg(rec + 3);
  const F3 pos = mk(r0.x, r0.y, r0.z);
  const F3 giscl = mk(r1.x, r1.y, r1.z);
  const F3 pscale = mk(r1.w, r2.x, r2.y);
  F3 rt[3];
  quat_rt(r2.z, r2.w, r3.x, r3.y, rt);
  const F3 gposc = sub(o, pos);
  const F3 gposcr = mat_mul(gposc, rt);
  const F3 gro = mulv(giscl, gposcr);
  const F3 ray_dir_r = mat_mul(d, rt);
  const F3 grdu = mulv(ray_dir_r, giscl);
  // safe_normalize with rsqrtf -> 1/sqrtf
  const float l = fa(fa(fm(grdu.x, grdu.x), fm(grdu.y, grdu.y)), fm(grdu.z, grdu.z));
  const F3 grd = l > 0.f ? muls(grdu, fd(1.f, fq(l))) : grdu;
  const float grp = -dot(grd, gro);
  const F3 grds = muls(mulv(pscale, grd), grp);
  const float t = fm(grp < 0.f ? -1.f : 1.f, fq(dot(grds, grds)));
  if (t < t_near || t > t_far) return false;
  const F3 gcrod = cross(grd, gro);
  const float gray = dot(gcrod, gcrod);
  *t_out = t;
  *gray_out = gray;
  return gray < 8.f;
}

// eval_sh_final(3, dir, g) (cudaRenderer.cu:487-558), constants
// cudaRenderer.h:33-48.
__device__ __forceinline__ F3 eval_sh(F3 d, const float4* __restrict__ shp) {
  float c[48];
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const float4 v = __ldg(shp + i);
    c[4 * i] = v.x;
    c[4 * i + 1] = v.y;
    c[4 * i + 2] = v.z;
    c[4 * i + 3] = v.w;
  }
#define SH(k) mk(c[3 * (k)], c[3 * (k) + 1], c[3 * (k) + 2])
  const float C0 = 0.28209479177387814f, C1 = 0.4886025119029199f;
  const float C20 = 1.0925484305920792f, C21 = -1.0925484305920792f, C22 = 0.31539156525252005f,
              C23 = -1.0925484305920792f, C24 = 0.5462742152960396f;
  const float C30 = -0.5900435899266435f, C31 = 2.890611442640554f, C32 = -0.4570457994644658f,
              C33 = 0.3731763325901154f, C34 = -0.4570457994644658f, C35 = 1.445305721320277f,
              C36 = -0.5900435899266435f;
  F3 rad = muls(SH(0), C0);
  const float x = d.x, y = d.y, z = d.z;
  rad = sub(add(sub(rad, muls(SH(1), fm(C1, y))), muls(SH(2), fm(C1, z))), muls(SH(3), fm(C1, x)));
  const float xx = fm(x, x), yy = fm(y, y), zz = fm(z, z);
  const float xy = fm(x, y), yz = fm(y, z), xz = fm(x, z);
  rad = add(rad, muls(SH(4), fm(C20, xy)));
  rad = add(rad, muls(SH(5), fm(C21, yz)));
  rad = add(rad, muls(SH(6), fm(C22, fs(fs(fm(2.f, zz), xx), yy))));
  rad = add(rad, muls(SH(7), fm(C23, xz)));
  rad = add(rad, muls(SH(8), fm(C24, fs(xx, yy))));
  rad = add(rad, muls(SH(9), fm(fm(C30, y), fs(fm(3.f, xx), yy))));
  rad = add(rad, muls(SH(10), fm(fm(C31, xy), z)));
  rad = add(rad, muls(SH(11), fm(fm(C32, y), fs(fs(fm(4.f, zz), xx), yy))));
  rad = add(rad, muls(SH(12), fm(fm(C33, z), fs(fs(fm(2.f, zz), fm(3.f, xx)), fm(3.f, yy)))));
  rad = add(rad, muls(SH(13), fm(fm(C34, x), fs(fs(fm(4.f, zz), xx), yy))));
  rad = add(rad, muls(SH(14), fm(fm(C35, z), fs(xx, yy))));
  rad = add(rad, muls(SH(15), fm(fm(C36, x), fs(xx, fm(3.f, yy)))));
#undef SH
  rad = add(rad, mk(0.5f, 0.5f, 0.5f));
  return mk(fmaxf(rad.x, 0.f), fmaxf(rad.y, 0.f), fmaxf(rad.z, 0.f));
}

constexpr int kStack = 12;       // SHORT_STACK_DEPTH, Kd-treeConverter.h:117
constexpr int kBlock = 128;

// Trace-mode counters and sequence hashes of one ray (kdgr_ray_trace).
struct RayStats {
  uint32_t n_inner = 0, n_leaf = 0, n_cand = 0, n_hit = 0, n_blend = 0, n_restart = 0, n_found = 0, max_sort = 0;
  uint64_t hl = kFnvInit, hh = kFnvInit, hb = kFnvInit;
};

// singlePassIntersectGaussian_sortNode_onlyShortStack (cudaRenderer.cu:
// 1488-1709): slab test, descent with the ring stack, per-leaf tests, stable
// hit order, compositing into acc/A/D.  The accumulators are the caller's and
// are not reset, as in the reference (the secondary-ray kernel keeps them
// across bounces).  max_t clips the scene interval (SECONDARY_RAY, :1537-1538;
// FLT_MAX leaves it as is).  Returns false after raising a status bit.
template <int K, bool TRACE>
__device__ __forceinline__ bool trace_exact(const ExactView& S, const F3 o, const F3 d, const float max_t, F3& acc,
                                            float& A, float& D, RayStats& rs, uint32_t (*s_id)[kBlock],
                                            float (*s_t)[kBlock], const int tid, uint32_t* status) {
  // BoundsRayIntersect (cudaRenderer.cu:379-399) with IEEE division
  float tmin = 1e-2f, tmax = FLT_MAX;
  {
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float l1 = fd(fs(S.bmin[a], oo[a]), dd[a]);
      const float l2 = fd(fs(S.bmax[a], oo[a]), dd[a]);
      tmin = fmaxf(fminf(l1, l2), tmin);
      tmax = fminf(fmaxf(l1, l2), tmax);
    }
  }
  if (!((tmax >= tmin) & (tmax >= 0.f))) return true;
  tmax = fminf(tmax, max_t);
  if (tmin > tmax) return true;
  const float t_scene_far = tmax;
  float t_near = tmin, t_far = tmax;
  uint32_t cur = 0, steps = 0;
  unsigned top = kStack - 1, quant = 0;
  while (A < 0.99f) {
    uint2 nd = __ldg(S.nodes + cur);
    if (++steps > kMaxRaySteps) {
      atomicOr(status, kStatusStepLimit);
      return false;
    }
    while ((nd.x & 7u) != 3u) {
      if (++steps > kMaxRaySteps) {
        atomicOr(status, kStatusStepLimit);
        return false;
      }
      const uint32_t child = nd.x >> 3;
      const uint32_t axis = nd.x & 3u;
      const float o_a = axis == 0 ? o.x : axis == 1 ? o.y : o.z;
      const float d_a = axis == 0 ? d.x : axis == 1 ? d.y : d.z;
      const float t_split = fd(fs(__uint_as_float(nd.y), o_a), d_a);
      const unsigned sign = __float_as_uint(d_a) >> 31;
      const uint32_t idx = child + (sign ^ (t_split <= t_near ? 1u : 0u));
      if (t_near < t_split && t_split < t_far) {
        if (++top == kStack) top = 0;
        quant = min(quant + 1, (unsigned)kStack);
        s_id[top][tid] = child + (sign ^ 1u);
        s_t[top][tid] = t_far;
        t_far = t_split;
      }
      if (child + 1 >= S.n_nodes) {
        atomicOr(status, kStatusBadNode);
        return false;
      }
      if (TRACE) ++rs.n_inner;
      cur = idx;
      nd = __ldg(S.nodes + cur);
    }
    if (TRACE) {
      ++rs.n_leaf;
      rs.hl = fnv_add(rs.hl, cur);
    }
    {
      const uint32_t cnt = nd.x >> 3, base = nd.y;
      if ((uint64_t)base + cnt > S.n_offsets) {
        atomicOr(status, kStatusBadLeaf);
        return false;
      }
      if (TRACE) rs.n_cand += cnt;
      bool have_last = false, saturated = false;
      uint32_t n_acc = 0;  // accepted in this leaf, counted on the first pass
      float last_t = 0.f;
      uint32_t last_i = 0;
      while (true) {
        float bt[K], bg[K];
        uint32_t bi[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
          bt[k] = __int_as_float(0x7f800000);
          bg[k] = 0.f;
          bi[k] = 0u;
        }
        bool overflow = false;
        for (uint32_t i = 0; i < cnt; ++i) {
          const uint32_t gid = __ldg(S.offsets + base + i);
          if (gid >= S.n_gauss) {
            atomicOr(status, kStatusBadId);
            return false;
          }
          float t, g;
          if (!exact_test(o, d, S.test + 4ull * gid, t_near, t_far, &t, &g)) continue;
          if (TRACE && !have_last) ++n_acc;
          if (have_last && !(t > last_t || (t == last_t && i > last_i))) continue;
          float ct = t, cg = g;
          uint32_t ci = i;
          bool placed = false;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const bool sw = placed || (ct < bt[k]);
            if (sw) {
              const float t0 = bt[k], g0 = bg[k];
              const uint32_t i0 = bi[k];
              bt[k] = ct;
              bg[k] = cg;
              bi[k] = ci;
              ct = t0;
              cg = g0;
              ci = i0;
              placed = true;
            }
          }
          if (ct != __int_as_float(0x7f800000)) overflow = true;
        }
        // composite the buffered hits in order (cudaRenderer.cu:1611-1687)
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (bt[k] == __int_as_float(0x7f800000)) break;
          const uint32_t gid = __ldg(S.offsets + base + bi[k]);
          if (TRACE) {
            ++rs.n_hit;
            rs.hh = fnv_add(rs.hh, gid);
          }
          const float opacity = __ldg(&S.test[4ull * gid].w);
          const float gres = kdgr_expf(fm(fm(-0.0555555555556f, bg[k]), bg[k]));
          const float alpha = fminf(0.99f, fm(opacity, gres));
          if (gres < 0.0113f || alpha < 1.0f / 255.0f) continue;
          const F3 c = eval_sh(d, S.sh + 12ull * gid);
          const float w = fm(alpha, fs(1.f, A));
          acc = add(acc, muls(muls(c, alpha), fs(1.f, A)));
          D = fa(D, fm(bt[k], w));
          A = fa(A, fm(alpha, fs(1.f, A)));
          if (TRACE) {
            ++rs.n_blend;
            rs.hb = fnv_add(rs.hb, gid);
          }
          if (A > 0.99f) {
            saturated = true;
            break;
          }
        }
        if (TRACE && !have_last) {
          rs.n_found += n_acc;
          rs.max_sort = max(rs.max_sort, n_acc);
        }
        if (saturated || !overflow) break;
        have_last = true;
        last_t = bt[K - 1];
        last_i = bi[K - 1];
      }
    }
    if ((A > 0.99f) | (t_far >= t_scene_far)) break;
    if (quant == 0) {
      cur = 0;
      if (TRACE) ++rs.n_restart;
      t_near = t_far;
      t_far = t_scene_far;
    } else {
      const uint32_t id = s_id[top][tid];
      const float tm = s_t[top][tid];
      if (top == 0) top = kStack;
      --top;
      --quant;
      cur = id;
      t_near = t_far;
      t_far = tm;
    }
  }
  return true;
}

// Pixel of thread `tid` in a 16x8 block: warps cover 8x4 tiles.
__device__ __forceinline__ void block_pixel(int tid, int* x, int* y) {
  const int lane = tid & 31, warp = tid >> 5;
  *x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  *y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
}

// Ray generation (cudaRenderer.cu:2336-2339): direction through the pixel
// centre, normalised as v * (1 / sqrt(v.v)).
__device__ __forceinline__ F3 primary_dir(const CamInfo& C, int x, int y) {
  const float sx = fa((float)x, 0.5f), sy = fa((float)y, 0.5f);
  const F3 start = mk(C.start[0], C.start[1], C.start[2]);
  const F3 cu = mk(C.u[0], C.u[1], C.u[2]), cv = mk(C.v[0], C.v[1], C.v[2]);
  const F3 o = mk(C.eye[0], C.eye[1], C.eye[2]);
  const F3 dir = sub(add(start, muls(muls(cu, sx), C.step_x)), muls(muls(cv, sy), C.step_y));
  const F3 dv = sub(dir, o);
  return muls(dv, fd(1.f, fq(dot(dv, dv))));
}

__device__ __forceinline__ F3 normalize3(F3 v) { return muls(v, fd(1.f, fq(dot(v, v)))); }

template <int K, bool TRACE>
__global__ void __launch_bounds__(kBlock) k_render_exact(ExactView S, CamInfo C, int W, int H, float* __restrict__ rgb,
                                                         float* __restrict__ alpha_out, float* __restrict__ depth_out,
                                                         kdgr_ray_trace* __restrict__ trace, uint32_t* status) {
  __shared__ uint32_t s_id[kStack][kBlock];
  __shared__ float s_t[kStack][kBlock];
  const int tid = threadIdx.x;
  int x, y;
  block_pixel(tid, &x, &y);
  if (x >= W || y >= H) return;
  const F3 o = mk(C.eye[0], C.eye[1], C.eye[2]);
  const F3 d = primary_dir(C, x, y);
  F3 acc = mk(0.f, 0.f, 0.f);
  float A = 0.f, D = 0.f;
  RayStats rs;
  trace_exact<K, TRACE>(S, o, d, FLT_MAX, acc, A, D, rs, s_id, s_t, tid, status);
  const size_t idx = (size_t)(H - 1 - y) * W + x;  // rows flipped (cudaRenderer.cu:2370)
  rgb[3 * idx] = acc.x;
  rgb[3 * idx + 1] = acc.y;
  rgb[3 * idx + 2] = acc.z;
  if (alpha_out) alpha_out[idx] = A;
  if (depth_out) depth_out[idx] = D;
  if (TRACE) {
    kdgr_ray_trace tr;
    tr.n_inner = rs.n_inner;
    tr.n_leaf = rs.n_leaf;
    tr.n_cand = rs.n_cand;
    tr.n_hit = rs.n_hit;
    tr.n_blend = rs.n_blend;
    tr.n_restart = rs.n_restart;
    tr.n_found = rs.n_found;
    tr.max_sort = rs.max_sort;
    tr.h_leaf = rs.hl;
    tr.h_hit = rs.hh;
    tr.h_blend = rs.hb;
    trace[(size_t)y * W + x] = tr;
  }
}

// ------------------------------------------------------------ secondary rays
// renderKernelGaussian_Mesh_Hybrid (cudaRenderer.cu:2217-2311): up to five
// bounces; per bounce the closest secondary primitive (spheres,
// intersectSphere :2149-2210, and triangles, intersectTriangleMesh :2114-2147
// with rayTriIntersect :2085-2112) clips the Gaussian pass, then the hit
// reflects, refracts or terminates the ray.  The Gaussian accumulators carry
// over between bounces, as in the reference.
struct SecHit {
  bool hit, front;
  float t;
  F3 n, p;
  int mat;
  float refl, ior;
  F3 color;
};

constexpr float kEps = 0.00001f;  // EPSILON, DefineConst.h:24

__device__ __forceinline__ void sec_material(SecHit& h, const float* m) {
  h.mat = __float_as_int(m[0]);
  h.refl = m[1];
  h.ior = m[2];
  h.color = mk(m[3], m[4], m[5]);
}

__device__ __forceinline__ void sec_set_normal(SecHit& h, const F3 d, F3 n) {
  if (dot(d, n) > 0.0f) {
    h.n = muls(n, -1.0f);
    h.front = false;
  } else {
    h.n = n;
    h.front = true;
  }
}

__device__ SecHit intersect_secondary(const HybridView& M, const F3 o, const F3 d) {
  SecHit h;
  h.hit = false;
  h.t = 1e8f;
  for (int i = 0; i < M.n_spheres; ++i) {
    const float* s = M.spheres + 10 * i;  // center xyz, radius, material words
    const F3 ctr = mk(s[0], s[1], s[2]);
    const F3 oc = sub(o, ctr);
    const float a = dot(d, d);
    const float b = fm(2.0f, dot(oc, d));
    const float c = fs(dot(oc, oc), fm(s[3], s[3]));
    const float disc = fs(fm(b, b), fm(fm(4.0f, a), c));
    if (disc >= 0.0f) {
      const float sq = fq(disc);
      float root = fd(fs(-b, sq), fm(2.0f, a));
      if (root < kEps) root = fd(fa(-b, sq), fm(2.0f, a));
      if (root > kEps && root < h.t) {
        h.hit = true;
        h.t = root;
        h.p = add(o, muls(d, root));
        sec_set_normal(h, d, normalize3(sub(h.p, ctr)));
        sec_material(h, s + 4);
      }
    }
  }
  for (uint32_t i = 0; i < M.n_tris; ++i) {
    const float* v = M.tris + 9ull * i;
    const F3 v0 = mk(v[0], v[1], v[2]), v1 = mk(v[3], v[4], v[5]), v2 = mk(v[6], v[7], v[8]);
    const F3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    const F3 hv = cross(d, e2);
    const float a = dot(e1, hv);
    if (a > -kEps && a < kEps) continue;
    const float f = fd(1.0f, a);
    const F3 sv = sub(o, v0);
    const float u = fm(f, dot(sv, hv));
    if (u < 0.0f || u > 1.0f) continue;
    const F3 q = cross(sv, e1);
    const float vv = fm(f, dot(d, q));
    if (vv < 0.0f || fa(u, vv) > 1.0f) continue;
    const float t = fm(f, dot(e2, q));
    if (!(t > kEps)) continue;
    if (t < h.t) {
      h.hit = true;
      h.t = t;
      h.p = add(o, muls(d, t));
      sec_set_normal(h, d, normalize3(cross(sub(v1, v0), sub(v2, v0))));
      sec_material(h, M.tri_material);
    }
  }
  return h;
}

template <int K>
__global__ void __launch_bounds__(kBlock) k_render_hybrid(ExactView S, CamInfo C, int W, int H, HybridView M,
                                                          float* __restrict__ rgb, uint32_t* status) {
  __shared__ uint32_t s_id[kStack][kBlock];
  __shared__ float s_t[kStack][kBlock];
  const int tid = threadIdx.x;
  int x, y;
  block_pixel(tid, &x, &y);
  if (x >= W || y >= H) return;
  F3 o = mk(C.eye[0], C.eye[1], C.eye[2]);
  F3 d = primary_dir(C, x, y);
  F3 fin = mk(0.f, 0.f, 0.f), thr = mk(1.f, 1.f, 1.f), acc = mk(0.f, 0.f, 0.f);
  float A = 0.f, D = 0.f;
  RayStats rs;
  for (int bounce = 0; bounce < 5; ++bounce) {
    const SecHit h = intersect_secondary(M, o, d);
    const float max_t = h.hit ? h.t : 1e8f;
    if (!trace_exact<K, false>(S, o, d, max_t, acc, A, D, rs, s_id, s_t, tid, status)) break;
    fin = add(fin, mulv(thr, acc));
    thr = muls(thr, fs(1.0f, A));
    if (thr.x < 0.01f && thr.y < 0.01f && thr.z < 0.01f) break;
    if (!h.hit) break;
    const F3 N = h.n, I = d;
    if (h.mat == 1) {  // mirror
      const F3 rdir = sub(I, muls(muls(N, 2.0f), dot(I, N)));
      o = add(h.p, muls(N, 1e-4f));
      d = normalize3(rdir);
      const F3 mc = bounce > 0 ? mk(0.f, 0.f, 0.f) : h.color;
      fin = add(fin, mulv(muls(thr, fs(1.0f, h.refl)), mc));
      thr = muls(thr, h.refl);
    } else if (h.mat == 2) {  // glass
      const float eta = h.front ? fd(1.0f, h.ior) : h.ior;
      const float cos_i = -dot(N, I);
      const float sin_t2 = fm(fm(eta, eta), fs(1.0f, fm(cos_i, cos_i)));
      if (sin_t2 > 1.0f) {  // total internal reflection
        const F3 rdir = sub(I, muls(muls(N, 2.0f), dot(I, N)));
        o = add(h.p, muls(N, 1e-4f));
        d = normalize3(rdir);
      } else {
        const float cos_t = fq(fs(1.0f, sin_t2));
        const F3 tdir = add(muls(I, eta), muls(N, fs(fm(eta, cos_i), cos_t)));
        o = sub(h.p, muls(N, 1e-4f));
        d = normalize3(tdir);
      }
      thr = mulv(thr, h.color);
    } else {  // opaque
      fin = add(fin, mulv(thr, h.color));
      break;
    }
  }
  const size_t idx = (size_t)(H - 1 - y) * W + x;
  rgb[3 * idx] = fminf(fin.x, 1.0f);
  rgb[3 * idx + 1] = fminf(fin.y, 1.0f);
  rgb[3 * idx + 2] = fminf(fin.z, 1.0f);
}

template <int K>
cudaError_t launch_k(const ExactView& s, const CamInfo& cam, int W, int H, float* rgb, float* alpha, float* depth,
                     kdgr_ray_trace* trace, uint32_t* status, cudaStream_t st) {
  dim3 grid((W + 15) / 16, (H + 7) / 8);
  if (trace)
    k_render_exact<K, true><<<grid, kBlock, 0, st>>>(s, cam, W, H, rgb, alpha, depth, trace, status);
  else
    k_render_exact<K, false><<<grid, kBlock, 0, st>>>(s, cam, W, H, rgb, alpha, depth, trace, status);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_exact(const ExactView& s, const CamInfo& cam, int W, int H, float* rgb, float* alpha, float* depth,
                         kdgr_ray_trace* trace, uint32_t* status, int kbuf, cudaStream_t st) {
  switch (kbuf) {
    case 4:
      return launch_k<4>(s, cam, W, H, rgb, alpha, depth, trace, status, st);
    case 16:
      return launch_k<16>(s, cam, W, H, rgb, alpha, depth, trace, status, st);
    default:
      return launch_k<8>(s, cam, W, H, rgb, alpha, depth, trace, status, st);
  }
}

cudaError_t launch_hybrid(const ExactView& s, const CamInfo& cam, int W, int H, const HybridView& m, float* rgb,
                          uint32_t* status, cudaStream_t st) {
  dim3 grid((W + 15) / 16, (H + 7) / 8);
  k_render_hybrid<8><<<grid, kBlock, 0, st>>>(s, cam, W, H, m, rgb, status);
  return cudaGetLastError();
}

}  // namespace kdgr
