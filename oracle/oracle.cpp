// oracle.cpp -- CPU restatement of the reference render kernel.
// TEST INFRASTRUCTURE ONLY: see oracle.h.  Compiled with -ffp-contract=off.
//
// Every function follows a reference function of
// Kd-treeConverter_v0.9/Kd-treeConverter/cudaRenderer.cu line by line, in
// the same types and operation order (operator semantics from
// SGRTx2Lib/cuda_math.h:260-420, e.g. dot = a.x*b.x + a.y*b.y + a.z*b.z).
// The template parameter R is float for the oracle-matching build and
// double for the FP64 twin.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename R>
struct V3 {
  R x, y, z;
};
template <typename R>
inline V3<R> mk(R x, R y, R z) {
  return V3<R>{x, y, z};
}
template <typename R>
inline V3<R> add(V3<R> a, V3<R> b) {
  return mk<R>(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename R>
inline V3<R> sub(V3<R> a, V3<R> b) {
  return mk<R>(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <typename R>
inline V3<R> mulv(V3<R> a, V3<R> b) {
  return mk<R>(a.x * b.x, a.y * b.y, a.z * b.z);
}
template <typename R>
inline V3<R> muls(V3<R> a, R s) {
  return mk<R>(a.x * s, a.y * s, a.z * s);
}
template <typename R>
inline R dot(V3<R> a, V3<R> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename R>
inline V3<R> cross(V3<R> a, V3<R> b) {
  return mk<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// normalize (cuda_math.h:403-407): v * (1/sqrt(dot(v,v)))
template <typename R>
inline V3<R> normalize(V3<R> v) {
  R inv = R(1) / std::sqrt(dot(v, v));
  return muls(v, inv);
}
// safe_normalize (cudaRenderer.cu:53-56) with rsqrtf -> 1/sqrt.
template <typename R>
inline V3<R> safe_normalize(V3<R> v) {
  const R l = v.x * v.x + v.y * v.y + v.z * v.z;
  return l > R(0) ? muls(v, R(1) / std::sqrt(l)) : v;
}

// The exponential of the oracle-matching arithmetic.  The reference calls
// CUDA's expf in particleResponse (cudaRenderer.cu:676-680); a CPU
// restatement cannot reproduce a vendor-library result, so the oracle and
// the plain kernel both use one published method instead, each in its own
// code: Cody-Waite reduction x = k ln2 + r with ln2 split into C1 = 355/512
// (9 significant bits, so k*C1 is exact) and C2 = ln2 - C1 (W. J. Cody and
// W. Waite, "Software Manual for the Elementary Functions", 1980), then
// e^r by its Taylor series to degree 7 in Horner form, scaled by 2^k.  In
// FP32 round-to-nearest without contraction, in this order, the two give
// the same bits; tests/test_oracle.py checks that on a dense sample of the
// response domain and bounds the error against double-precision exp.
inline float oracle_expf(float x) {
  if (!(x >= -87.3f)) return (x != x) ? x : 0.0f;
  if (x > 88.0f) return HUGE_VALF;
  const float k = std::floor(x * 1.44269504088896341f + 0.5f);  // round(x / ln2)
  float r = x - k * 0.693359375f;                               // C1 = 355/512
  r = r + k * 2.12194440e-4f;                                    // -C2
  static const float kTaylor[8] = {1.0f / 5040, 1.0f / 720, 1.0f / 120, 1.0f / 24,
                                   1.0f / 6,    0.5f,       1.0f,       1.0f};
  float p = kTaylor[0];
  for (int i = 1; i < 8; ++i) p = p * r + kTaylor[i];
  const uint32_t bits = (uint32_t)((int)k + 127) << 23;
  float scale;
  std::memcpy(&scale, &bits, 4);
  return p * scale;
}

inline float rexp(float x) { return oracle_expf(x); }
inline double rexp(double x) { return std::exp(x); }

// quaternionWXYZToMatrixTranspose (cudaRenderer.cu:808-828).
template <typename R>
inline void quat_rt(const float* q, V3<R> m[3]) {
  const R r = q[0], x = q[1], y = q[2], z = q[3];
  const R xx = x * x, yy = y * y, zz = z * z;
  const R xy = x * y, xz = x * z, yz = y * z;
  const R rx = r * x, ry = r * y, rz = r * z;
  m[0] = mk<R>((R(1) - R(2) * (yy + zz)), R(2) * (xy + rz), R(2) * (xz - ry));
  m[1] = mk<R>(R(2) * (xy - rz), (R(1) - R(2) * (xx + zz)), R(2) * (yz + rx));
  m[2] = mk<R>(R(2) * (xz + ry), R(2) * (yz - rx), (R(1) - R(2) * (xx + yy)));
}
// float3 * float33 (cudaRenderer.cu:48-50): (dot(m[0],p), dot(m[1],p), dot(m[2],p))
template <typename R>
inline V3<R> mat_mul(V3<R> p, const V3<R> m[3]) {
  return mk<R>(dot(m[0], p), dot(m[1], p), dot(m[2], p));
}

// eval_sh_final(3, dir, g) (cudaRenderer.cu:487-558); SH constants from
// cudaRenderer.h:33-48.  Coefficient k>=1 is (f_rest[k-1], f_rest[15+k-1],
// f_rest[30+k-1]) (:498).
template <typename R>
inline V3<R> eval_sh(V3<R> d, const float* g) {
  const float* dc = g + 12;
  const float* rest = g + 15;
  auto sh = [&](int k) -> V3<R> {
    if (k == 0) return mk<R>(dc[0], dc[1], dc[2]);
    return mk<R>(rest[k - 1], rest[15 + k - 1], rest[30 + k - 1]);
  };
  const R C0 = 0.28209479177387814f, C1 = 0.4886025119029199f;
  const R C20 = 1.0925484305920792f, C21 = -1.0925484305920792f, C22 = 0.31539156525252005f,
          C23 = -1.0925484305920792f, C24 = 0.5462742152960396f;
  const R C30 = -0.5900435899266435f, C31 = 2.890611442640554f, C32 = -0.4570457994644658f,
          C33 = 0.3731763325901154f, C34 = -0.4570457994644658f, C35 = 1.445305721320277f,
          C36 = -0.5900435899266435f;
  V3<R> rad = muls(sh(0), C0);
  const R x = d.x, y = d.y, z = d.z;
  rad = sub(add(sub(rad, muls(sh(1), C1 * y)), muls(sh(2), C1 * z)), muls(sh(3), C1 * x));
  const R xx = x * x, yy = y * y, zz = z * z;
  const R xy = x * y, yz = y * z, xz = x * z;
  rad = add(rad, muls(sh(4), C20 * xy));
  rad = add(rad, muls(sh(5), C21 * yz));
  rad = add(rad, muls(sh(6), C22 * (R(2) * zz - xx - yy)));
  rad = add(rad, muls(sh(7), C23 * xz));
  rad = add(rad, muls(sh(8), C24 * (xx - yy)));
  rad = add(rad, muls(sh(9), C30 * y * (R(3) * xx - yy)));
  rad = add(rad, muls(sh(10), C31 * xy * z));
  rad = add(rad, muls(sh(11), C32 * y * (R(4) * zz - xx - yy)));
  rad = add(rad, muls(sh(12), C33 * z * (R(2) * zz - R(3) * xx - R(3) * yy)));
  rad = add(rad, muls(sh(13), C34 * x * (R(4) * zz - xx - yy)));
  rad = add(rad, muls(sh(14), C35 * z * (xx - yy)));
  rad = add(rad, muls(sh(15), C36 * x * (xx - R(3) * yy)));
  rad = add(rad, mk<R>(R(0.5f), R(0.5f), R(0.5f)));
  return mk<R>(std::fmax(rad.x, R(0)), std::fmax(rad.y, R(0)), std::fmax(rad.z, R(0)));
}

struct Fnv {
  uint64_t h = 14695981039346656037ull;
  void add(uint32_t v) {
    for (int i = 0; i < 4; ++i) {
      h ^= (v >> (8 * i)) & 0xFFu;
      h *= 1099511628211ull;
    }
  }
};

template <typename R>
struct Hit {
  R t;
  uint32_t id;
};

template <typename R>
struct Ray {
  V3<R> o, d;
};

// The ray-Gaussian test of rayPrimIntersect with VOLUME_ISECT
// (cudaRenderer.cu:1070-1135).  Returns true and t on acceptance.
template <typename R>
inline bool intersect(const Ray<R>& ray, const float* g, R t_near, R t_far, R* t_out) {
  const V3<R> pos = mk<R>(g[0], g[1], g[2]);
  const V3<R> giscl = mk<R>(g[4], g[5], g[6]);
  const V3<R> pscale = mk<R>(R(1) / giscl.x, R(1) / giscl.y, R(1) / giscl.z);
  V3<R> rt[3];
  quat_rt<R>(g + 8, rt);
  const V3<R> gposc = sub(ray.o, pos);
  const V3<R> gposcr = mat_mul(gposc, rt);
  const V3<R> gro = mulv(giscl, gposcr);
  const V3<R> ray_dir_r = mat_mul(ray.d, rt);
  const V3<R> grdu = mulv(ray_dir_r, giscl);
  const V3<R> grd = safe_normalize(grdu);
  const R grp = -dot(grd, gro);
  const V3<R> grds = muls(mulv(pscale, grd), grp);
  const R t = (grp < R(0) ? R(-1) : R(1)) * std::sqrt(dot(grds, grds));
  if (t < t_near || t > t_far) return false;
  const V3<R> gcrod = cross(grd, gro);
  const R gray = dot(gcrod, gcrod);
  if (gray < R(8)) {
    *t_out = t;
    return true;
  }
  return false;
}

// The per-hit body of the compositing loop (cudaRenderer.cu:1611-1687).
// Returns true when the ray is saturated (A > OPACITY_THRESHOLD).
template <typename R>
inline bool composite(const Ray<R>& ray, const float* g, R t, V3<R>& C, R& A, R& D, bool* blended) {
  *blended = false;
  const V3<R> pos = mk<R>(g[0], g[1], g[2]);
  const V3<R> giscl = mk<R>(g[4], g[5], g[6]);
  V3<R> rt[3];
  quat_rt<R>(g + 8, rt);
  const V3<R> gposc = sub(ray.o, pos);
  const V3<R> gposcr = mat_mul(gposc, rt);
  const V3<R> gro = mulv(giscl, gposcr);
  const V3<R> ray_dir_r = mat_mul(ray.d, rt);
  const V3<R> grdu = mulv(giscl, ray_dir_r);
  const V3<R> grd = normalize(grdu);
  const V3<R> gcrod = cross(grd, gro);
  const R gray = dot(gcrod, gcrod);
  // particleResponse<4> (cudaRenderer.cu:676-680): exp(s * g * g)
  const R gres = rexp(R(-0.0555555555556f) * gray * gray);
  const R alpha = std::fmin(R(0.99f), R(g[3]) * gres);
  if (gres < R(0.0113f) || alpha < R(1.0f / 255.0f)) return false;
  const V3<R> c = eval_sh<R>(ray.d, g);
  const R w = alpha * (R(1) - A);
  C = add(C, muls(muls(c, alpha), (R(1) - A)));
  D = D + t * w;
  A = A + alpha * (R(1) - A);
  *blended = true;
  return A > R(0.99f);
}

// singlePassIntersectGaussian_sortNode_onlyShortStack, ELLIPSOID_BY_TRI
// branch (cudaRenderer.cu:1488-1709) with BoundsRayIntersect (:379-399),
// the 12-entry ring stack (:184-210) and the stable sortHits (:415-426).
// The accumulators C, A, D are the caller's and are not reset (the
// secondary-ray kernel keeps them across bounces, cudaRenderer.cu:2233-2255);
// max_t clips the scene interval (SECONDARY_RAY, :1537-1538).
template <typename R>
void trace_core(const orc_scene* S, const Ray<R>& ray, R max_t, V3<R>& C, R& A, R& D, kdgr_ray_trace* tr,
                std::vector<Hit<R>>& hits) {
  uint32_t n_inner = 0, n_leaf = 0, n_cand = 0, n_hit = 0, n_blend = 0, n_restart = 0, n_found = 0, max_sort = 0;
  Fnv hl, hh, hb;
  R tmin = R(1e-2f), tmax = R(FLT_MAX);
  const R bmin[3] = {S->aabb[0], S->aabb[1], S->aabb[2]};
  const R bmax[3] = {S->aabb[3], S->aabb[4], S->aabb[5]};
  const R o[3] = {ray.o.x, ray.o.y, ray.o.z};
  const R d[3] = {ray.d.x, ray.d.y, ray.d.z};
  for (int a = 0; a < 3; ++a) {
    const R l1 = (bmin[a] - o[a]) / d[a];
    const R l2 = (bmax[a] - o[a]) / d[a];
    tmin = std::fmax(std::fmin(l1, l2), tmin);
    tmax = std::fmin(std::fmax(l1, l2), tmax);
  }
  if ((tmax >= tmin) & (tmax >= R(0)) & !(tmin > std::fmin(tmax, max_t))) {
    tmax = std::fmin(tmax, max_t);
    const R t_scene_far = tmax;
    uint32_t cur = 0;
    R t_near = tmin, t_far = tmax;
    struct Entry {
      uint32_t id;
      R tmax;
    } ring[12];
    unsigned top = 11, quant = 0;
    while (A < R(0.99f)) {
      uint32_t x = S->nodes[2 * cur], y = S->nodes[2 * cur + 1];
      while ((x & 7u) != 3u) {
        const uint32_t child = x >> 3;
        const uint32_t axis = x & 3u;
        const R o_a = axis == 0 ? ray.o.x : axis == 1 ? ray.o.y : ray.o.z;
        const R d_a = axis == 0 ? ray.d.x : axis == 1 ? ray.d.y : ray.d.z;
        float split;
        memcpy(&split, &y, 4);
        const R t_split = (R(split) - o_a) / d_a;
        const unsigned sign = std::signbit(d_a) ? 1u : 0u;
        const uint32_t idx = child + (sign ^ (t_split <= t_near ? 1u : 0u));
        if (t_near < t_split && t_split < t_far) {
          if (++top == 12) top = 0;
          quant = quant + 1 < 12 ? quant + 1 : 12;
          ring[top].id = child + (sign ^ 1u);
          ring[top].tmax = t_far;
          t_far = t_split;
        }
        ++n_inner;
        cur = idx;
        x = S->nodes[2 * cur];
        y = S->nodes[2 * cur + 1];
      }
      ++n_leaf;
      hl.add(cur);
      const uint32_t cnt = x >> 3, base = y;
      hits.clear();
      for (uint32_t i = base; i < base + cnt; ++i) {
        const uint32_t gid = S->offsets[i];
        ++n_cand;
        R t;
        if (intersect<R>(ray, S->gauss + (size_t)gid * 64, t_near, t_far, &t)) hits.push_back({t, gid});
      }
      // HIT_AND_NODE_COUNT_DEBUG counters (cudaRenderer.cu:1602-1606)
      n_found += (uint32_t)hits.size();
      max_sort = std::max(max_sort, (uint32_t)hits.size());
      // stable insertion sort by t (sortHits)
      for (size_t i = 1; i < hits.size(); ++i) {
        Hit<R> key = hits[i];
        long j = (long)i - 1;
        while (j >= 0 && hits[j].t > key.t) {
          hits[j + 1] = hits[j];
          --j;
        }
        hits[j + 1] = key;
      }
      for (size_t i = 0; i < hits.size(); ++i) {
        ++n_hit;
        hh.add(hits[i].id);
        bool blended;
        const bool done = composite<R>(ray, S->gauss + (size_t)hits[i].id * 64, hits[i].t, C, A, D, &blended);
        if (blended) {
          ++n_blend;
          hb.add(hits[i].id);
        }
        if (done) break;
      }
      if ((A > R(0.99f)) | (t_far >= t_scene_far)) break;
      if (quant == 0) {
        cur = 0;
        ++n_restart;
        t_near = t_far;
        t_far = t_scene_far;
      } else {
        const Entry e = ring[top];
        if (top == 0) top = 12;
        --top;
        --quant;
        cur = e.id;
        t_near = t_far;
        t_far = e.tmax;
      }
    }
  }
  if (tr) {
    tr->n_inner = n_inner;
    tr->n_leaf = n_leaf;
    tr->n_cand = n_cand;
    tr->n_hit = n_hit;
    tr->n_blend = n_blend;
    tr->n_restart = n_restart;
    tr->n_found = n_found;
    tr->max_sort = max_sort;
    tr->h_leaf = hl.h;
    tr->h_hit = hh.h;
    tr->h_blend = hb.h;
  }
}

template <typename R>
void trace_ray(const orc_scene* S, const Ray<R>& ray, V3<R>& C, R& A, R& D, kdgr_ray_trace* tr,
               std::vector<Hit<R>>& hits) {
  C = mk<R>(0, 0, 0);
  A = 0;
  D = 0;
  trace_core<R>(S, ray, R(FLT_MAX), C, A, D, tr, hits);
}

// Ray generation of renderKernelGaussian_sortNode (cudaRenderer.cu:2336-2339).
template <typename R>
inline Ray<R> gen_ray(const orc_caminfo* c, int x, int y) {
  const R sx = R(float(x)) + R(0.5f), sy = R(float(y)) + R(0.5f);
  const V3<R> start = mk<R>(c->start[0], c->start[1], c->start[2]);
  const V3<R> u = mk<R>(c->u[0], c->u[1], c->u[2]);
  const V3<R> v = mk<R>(c->v[0], c->v[1], c->v[2]);
  const V3<R> eye = mk<R>(c->eye[0], c->eye[1], c->eye[2]);
  const V3<R> dir = sub(add(start, muls(muls(u, sx), R(c->step_x))), muls(muls(v, sy), R(c->step_y)));
  Ray<R> r;
  r.o = eye;
  r.d = normalize(sub(dir, eye));
  return r;
}

template <typename R>
int render(const orc_scene* s, const orc_caminfo* c, int width, int height, const uint32_t* pix, uint32_t n_pix,
           R* rgb, R* alpha, R* depth, kdgr_ray_trace* trace, int threads) {
  if (!s || !c || !pix || width <= 0 || height <= 0) return KDGR_ERR_INVALID_ARG;
  int nt = threads;
#ifdef _OPENMP
  if (nt <= 0) nt = omp_get_max_threads();
#else
  nt = 1;
#endif
  size_t max_leaf = 1;
  for (uint32_t i = 0; i < s->n_nodes; ++i)
    if ((s->nodes[2 * i] & 7u) == 3u && (s->nodes[2 * i] >> 3) > max_leaf) max_leaf = s->nodes[2 * i] >> 3;
#pragma omp parallel num_threads(nt)
  {
    std::vector<Hit<R>> hits;
    hits.reserve(max_leaf);
#pragma omp for schedule(dynamic, 64)
    for (long i = 0; i < (long)n_pix; ++i) {
      const int px = (int)(pix[i] % (uint32_t)width), py = (int)(pix[i] / (uint32_t)width);
      const Ray<R> ray = gen_ray<R>(c, px, py);
      V3<R> C;
      R A, D;
      trace_ray<R>(s, ray, C, A, D, trace ? trace + i : nullptr, hits);
      if (rgb) {
        rgb[3 * i] = C.x;
        rgb[3 * i + 1] = C.y;
        rgb[3 * i + 2] = C.z;
      }
      if (alpha) alpha[i] = A;
      if (depth) depth[i] = D;
    }
  }
  return KDGR_OK;
}

// ---------------------------------------------------------------- secondary
// renderKernelGaussian_Mesh_Hybrid (cudaRenderer.cu:2217-2311) with
// intersectSphere (:2170-2214), intersectTriangleMesh (:2111-2147) and
// rayTriIntersect (:2085-2109); EPSILON = 1e-5f (DefineConst.h:24).
struct SecHit {
  bool hit = false, front = false;
  float t = 1e8f;
  V3<float> n{0, 0, 0}, p{0, 0, 0};
  int mat = 0;
  float refl = 0, ior = 0;
  V3<float> color{0, 0, 0};
};

void sec_material(SecHit& h, const float* m) {
  memcpy(&h.mat, &m[0], 4);
  h.refl = m[1];
  h.ior = m[2];
  h.color = mk<float>(m[3], m[4], m[5]);
}

void sec_normal(SecHit& h, V3<float> d, V3<float> n) {
  if (dot(d, n) > 0.0f) {
    h.n = muls(n, -1.0f);
    h.front = false;
  } else {
    h.n = n;
    h.front = true;
  }
}

SecHit intersect_secondary(const float* sph, int n_sph, const float* tri, uint32_t n_tri, const float* tri_mat,
                           V3<float> o, V3<float> d) {
  const float eps = 0.00001f;
  SecHit h;
  for (int i = 0; i < n_sph; ++i) {
    const float* s = sph + 10 * i;
    const V3<float> ctr = mk<float>(s[0], s[1], s[2]);
    const V3<float> oc = sub(o, ctr);
    const float a = dot(d, d);
    const float b = 2.0f * dot(oc, d);
    const float c = dot(oc, oc) - s[3] * s[3];
    const float disc = b * b - 4.0f * a * c;
    if (disc >= 0.0f) {
      const float sq = std::sqrt(disc);
      float root = (-b - sq) / (2.0f * a);
      if (root < eps) root = (-b + sq) / (2.0f * a);
      if (root > eps && root < h.t) {
        h.hit = true;
        h.t = root;
        h.p = add(o, muls(d, root));
        sec_normal(h, d, normalize(sub(h.p, ctr)));
        sec_material(h, s + 4);
      }
    }
  }
  for (uint32_t i = 0; i < n_tri; ++i) {
    const float* v = tri + 9ull * i;
    const V3<float> v0 = mk<float>(v[0], v[1], v[2]), v1 = mk<float>(v[3], v[4], v[5]),
                    v2 = mk<float>(v[6], v[7], v[8]);
    const V3<float> e1 = sub(v1, v0), e2 = sub(v2, v0);
    const V3<float> hv = cross(d, e2);
    const float a = dot(e1, hv);
    if (a > -eps && a < eps) continue;
    const float f = 1.0f / a;
    const V3<float> sv = sub(o, v0);
    const float u = f * dot(sv, hv);
    if (u < 0.0f || u > 1.0f) continue;
    const V3<float> q = cross(sv, e1);
    const float vv = f * dot(d, q);
    if (vv < 0.0f || u + vv > 1.0f) continue;
    const float t = f * dot(e2, q);
    if (!(t > eps)) continue;
    if (t < h.t) {
      h.hit = true;
      h.t = t;
      h.p = add(o, muls(d, t));
      sec_normal(h, d, normalize(cross(sub(v1, v0), sub(v2, v0))));
      sec_material(h, tri_mat);
    }
  }
  return h;
}

V3<float> hybrid_pixel(const orc_scene* S, const orc_caminfo* c, int px, int py, const float* sph, int n_sph,
                       const float* tri, uint32_t n_tri, const float* tri_mat, std::vector<Hit<float>>& hits) {
  Ray<float> ray = gen_ray<float>(c, px, py);
  V3<float> fin = mk<float>(0, 0, 0), thr = mk<float>(1, 1, 1), acc = mk<float>(0, 0, 0);
  float A = 0, D = 0;
  for (int bounce = 0; bounce < 5; ++bounce) {
    const SecHit h = intersect_secondary(sph, n_sph, tri, n_tri, tri_mat, ray.o, ray.d);
    const float max_t = h.hit ? h.t : 1e8f;
    trace_core<float>(S, ray, max_t, acc, A, D, nullptr, hits);
    fin = add(fin, mulv(thr, acc));
    thr = muls(thr, 1.0f - A);
    if (thr.x < 0.01f && thr.y < 0.01f && thr.z < 0.01f) break;
    if (!h.hit) break;
    const V3<float> N = h.n, I = ray.d;
    if (h.mat == 1) {
      const V3<float> rdir = sub(I, muls(muls(N, 2.0f), dot(I, N)));
      ray.o = add(h.p, muls(N, 1e-4f));
      ray.d = normalize(rdir);
      const V3<float> mc = bounce > 0 ? mk<float>(0, 0, 0) : h.color;
      fin = add(fin, mulv(muls(thr, 1.0f - h.refl), mc));
      thr = muls(thr, h.refl);
    } else if (h.mat == 2) {
      const float eta = h.front ? 1.0f / h.ior : h.ior;
      const float cos_i = -dot(N, I);
      const float sin_t2 = eta * eta * (1.0f - cos_i * cos_i);
      if (sin_t2 > 1.0f) {
        const V3<float> rdir = sub(I, muls(muls(N, 2.0f), dot(I, N)));
        ray.o = add(h.p, muls(N, 1e-4f));
        ray.d = normalize(rdir);
      } else {
        const float cos_t = std::sqrt(1.0f - sin_t2);
        const V3<float> tdir = add(muls(I, eta), muls(N, eta * cos_i - cos_t));
        ray.o = sub(h.p, muls(N, 1e-4f));
        ray.d = normalize(tdir);
      }
      thr = mulv(thr, h.color);
    } else {
      fin = add(fin, mulv(thr, h.color));
      break;
    }
  }
  return mk<float>(std::fmin(fin.x, 1.0f), std::fmin(fin.y, 1.0f), std::fmin(fin.z, 1.0f));
}

}  // namespace

extern "C" {

int orc_render_hybrid_f32(const orc_scene* s, const orc_caminfo* c, int width, int height, const uint32_t* pix,
                          uint32_t n_pix, const float* spheres, int n_spheres, const float* tris, uint32_t n_tris,
                          const float* tri_material, float* rgb, int threads) {
  if (!s || !c || !pix || !rgb || width <= 0 || height <= 0) return KDGR_ERR_INVALID_ARG;
  int nt = threads;
#ifdef _OPENMP
  if (nt <= 0) nt = omp_get_max_threads();
#else
  nt = 1;
#endif
#pragma omp parallel num_threads(nt)
  {
    std::vector<Hit<float>> hits;
#pragma omp for schedule(dynamic, 64)
    for (long i = 0; i < (long)n_pix; ++i) {
      const int px = (int)(pix[i] % (uint32_t)width), py = (int)(pix[i] / (uint32_t)width);
      const V3<float> C = hybrid_pixel(s, c, px, py, spheres, n_spheres, tris, n_tris, tri_material, hits);
      rgb[3 * i] = C.x;
      rgb[3 * i + 1] = C.y;
      rgb[3 * i + 2] = C.z;
    }
  }
  return KDGR_OK;
}


void orc_caminfo_from_camera(const kdgr_camera* cam, int width, int height, orc_caminfo* out) {
  const float kPi = 3.14159265358979323846f;  // M_PI, cudaRenderer.h:31
  const float fov_rad = (float)(cam->fovy * (kPi / 180.0f));
  const float plane_height = (float)(2.0f * cam->near_c * tanf(fov_rad * 0.5f));
  const float plane_width = (float)(plane_height * cam->aspect);
  out->step_x = plane_width / width;
  out->step_y = plane_height / height;
  const float nc = (float)cam->near_c;
  for (int i = 0; i < 3; ++i) {
    out->eye[i] = cam->pos[i];
    out->u[i] = cam->uaxis[i];
    out->v[i] = cam->vaxis[i];
  }
  for (int i = 0; i < 3; ++i) {
    const float a = cam->pos[i] - cam->naxis[i] * nc;
    const float b = a - cam->uaxis[i] * (plane_width * 0.5f);
    out->start[i] = b + cam->vaxis[i] * (plane_height * 0.5f);
  }
}

int orc_render_f32(const orc_scene* s, const orc_caminfo* c, int width, int height, const uint32_t* pix,
                   uint32_t n_pix, float* rgb, float* alpha, float* depth, kdgr_ray_trace* trace, int threads) {
  return render<float>(s, c, width, height, pix, n_pix, rgb, alpha, depth, trace, threads);
}

int orc_render_f64(const orc_scene* s, const orc_caminfo* c, int width, int height, const uint32_t* pix,
                   uint32_t n_pix, double* rgb, double* alpha, double* depth, kdgr_ray_trace* trace,
                   int threads) {
  return render<double>(s, c, width, height, pix, n_pix, rgb, alpha, depth, trace, threads);
}

float orc_expf(float x) { return oracle_expf(x); }

void orc_expf_n(const float* x, float* y, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) y[i] = oracle_expf(x[i]);
}

}  // extern "C"
