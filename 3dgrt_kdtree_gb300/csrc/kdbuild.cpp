// kdbuild.cpp -- host kd-tree builder for the hybrid Gaussian kd-tree.
//
// Produces the same tree, bit for bit, as the reference builder
// (Kd-treeConstructor.cpp, PRIMITIVE_TYPE 2 / COUNT_BY_GID 1) run through the
// reference's headless build (Kd-treeConverterMain.cpp:3738-3762), but is
// organised for speed: per-node work is O(n log n) sorts of plain float arrays
// instead of per-edge hash-map updates, and subtrees build in parallel.
//
// Why a set-based sweep gives the reference's tree.  try_to_split
// (Kd-treeConstructor.cpp:579-868) sorts the 2*T triangle edges of a node on
// one axis and sweeps the distinct positions.  Under COUNT_BY_GID a Gaussian
// ID is counted as "started" at the first position where any of its
// triangles starts (seen_starts, :616-663) and as "ended" at the position
// where its last END edge is seen (seen_ends == total_ends, :656-661).  So
// each ID acts as one interval [gmin, gmax] = the union of its triangles'
// clipped extents, and at every candidate position p:
//   open  = #{gmin < p},  close = #{gmax < p},
//   local_open = #{gmin == p != gmax}, local_close = #{gmax == p != gmin},
//   planar = #{gmin == gmax == p}.
// The candidate positions are all distinct triangle-edge values, including
// ones where no ID changes state; every one is scored, as in the reference.
// Nothing in the score, the split choice (first minimum, axis 0 first), the
// partition (push_triangles_to_child_vector :545-577) or the clip
// (clip_triangle :364-486) depends on the order of triangles inside a node,
// and leaves list their unique IDs in ascending order (std::set, :1543-1549),
// so the tree is a function of the triangle set alone.  Node slots are then
// numbered exactly as the reference allocates them (pairs of children taken
// from a running counter in depth-first, left-first order, :1606-1622) and
// leaf ID lists are appended in the same order.
//
// Floating point: every expression keeps the reference's types and operation
// order (float extents and cell area, double probabilities and costs), and
// this file is compiled with -ffp-contract=off.  Known non-reproducible
// corner: a split candidate exactly at +0.0/-0.0, where the reference's
// qsort decides which zero's bits become the split plane.

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "kdgr_internal.h"

namespace kdgr {
namespace {

struct Tri {
  float v[3][3];       // original proxy triangle vertices (never clipped)
  float lo[3], hi[3];  // current (clipped) bounding box
  uint32_t gid;
  uint32_t pad;
};

struct Node {
  int axis = -1;  // -1: leaf
  float split = 0.f;
  std::unique_ptr<Node> kid[2];
  std::vector<uint32_t> ids;  // leaf: sorted unique Gaussian IDs
};

struct Params {
  int max_level;
  int force_split;
  float isect_cost;
  int sah_mode;
  float sort_cost;
};

constexpr float kTravCost = 1.0f;    // TRAVL_COST, Kd-treeConverter.h:44
constexpr float kEmptyBonus = 0.9f;  // EMTPY_BONUS, Kd-treeConverter.h:45
constexpr unsigned kMinPrim = 16;    // MIN_TRI, Kd-treeConverter.h:63
constexpr float kEps = 0.00001f;     // KD_TREE_EPSILON, Kd-treeConstructor.h:10

inline float ref_min(float a, float b) { return a < b ? a : b; }  // MyMIN
inline float ref_max(float a, float b) { return a > b ? a : b; }  // MyMAX

struct SplitChoice {
  double cost;
  float pos;
  int axis;
  int planar_side;  // 0: planar IDs go left (BoundEdge::START), 1: right
};

// Radix sort of float keys (ascending, -0 before +0 as distinct keys).
void sort_floats(std::vector<float>& a, std::vector<uint32_t>& tmp_keys) {
  const size_t n = a.size();
  if (n < 4096) {
    std::sort(a.begin(), a.end());
    return;
  }
  std::vector<uint32_t> k(n);
  for (size_t i = 0; i < n; ++i) {
    uint32_t u;
    memcpy(&u, &a[i], 4);
    k[i] = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  }
  tmp_keys.resize(n);
  uint32_t* src = k.data();
  uint32_t* dst = tmp_keys.data();
  for (int pass = 0; pass < 3; ++pass) {
    const int shift = pass * 11;
    const uint32_t mask = pass == 2 ? 0x3FFu : 0x7FFu;
    size_t cnt[2048] = {0};
    for (size_t i = 0; i < n; ++i) cnt[(src[i] >> shift) & mask]++;
    size_t s = 0;
    for (int b = 0; b < 2048; ++b) {
      size_t c = cnt[b];
      cnt[b] = s;
      s += c;
    }
    for (size_t i = 0; i < n; ++i) dst[cnt[(src[i] >> shift) & mask]++] = src[i];
    std::swap(src, dst);
  }
  for (size_t i = 0; i < n; ++i) {
    uint32_t u = src[i];
    u = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    memcpy(&a[i], &u, 4);
  }
}

// Score every candidate position on one axis; update `best` (strict <).
void try_axis(int axis, const float blo[3], const float bhi[3], const std::vector<Tri>& tris,
              const std::vector<uint32_t>& run_start, const Params& P, SplitChoice& best) {
  const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
  float ext[3];
  ext[0] = bhi[0] - blo[0];
  ext[1] = bhi[1] - blo[1];
  ext[2] = bhi[2] - blo[2];
  const float cell_area_f = (ext[0] * ext[1]) + (ext[1] * ext[2]) + (ext[0] * ext[2]);
  const double cell_area = cell_area_f;
  const double cell_area_rcp = 1 / cell_area;
  const double area_mul = double(ext[a1]) + double(ext[a2]);
  const double area_add = double(ext[a1]) * double(ext[a2]);
  const float cell_min = blo[axis];
  const float cell_max = bhi[axis];
  const float lim_lo = cell_min + kEps;
  const float lim_hi = cell_max - kEps;

  const size_t G = run_start.size() - 1;
  std::vector<float> gmin(G), gmax(G), planar;
  std::vector<float> cand;
  cand.reserve(tris.size() * 2);
  for (size_t g = 0; g < G; ++g) {
    float mn = FLT_MAX, mx = -FLT_MAX;
    bool first = true;
    for (uint32_t t = run_start[g]; t < run_start[g + 1]; ++t) {
      const float l = tris[t].lo[axis], h = tris[t].hi[axis];
      if (first) {
        mn = l;
        mx = h;
        first = false;
      } else {
        if (l < mn) mn = l;
        if (h > mx) mx = h;
      }
      cand.push_back(l);
      cand.push_back(h);
    }
    gmin[g] = mn;
    gmax[g] = mx;
    if (mn == mx) planar.push_back(mn);
  }
  std::vector<uint32_t> tmp;
  sort_floats(cand, tmp);
  sort_floats(gmin, tmp);
  sort_floats(gmax, tmp);
  std::sort(planar.begin(), planar.end());

  size_t imn = 0, imx = 0, ipl = 0;  // pointers into gmin/gmax/planar
  const size_t nc = cand.size();
  size_t c = 0;
  while (c < nc) {
    const float p = cand[c];
    // advance over equal candidates (-0 == +0 compare equal, as the
    // reference's group loop does)
    size_t c2 = c + 1;
    while (c2 < nc && cand[c2] == p) ++c2;
    c = c2;
    while (imn < G && gmin[imn] < p) ++imn;
    while (imx < G && gmax[imx] < p) ++imx;
    while (ipl < planar.size() && planar[ipl] < p) ++ipl;
    size_t emn = imn, emx = imx, epl = ipl;
    while (emn < G && gmin[emn] == p) ++emn;
    while (emx < G && gmax[emx] == p) ++emx;
    while (epl < planar.size() && planar[epl] == p) ++epl;
    const int num_planars = int(epl - ipl);
    const int local_close = int(emx - imx) - num_planars;
    const int open = int(imn);
    const int close = int(imx);

    if (p <= lim_lo) continue;
    if (p >= lim_hi) break;

    const double extent_l = double(p) - cell_min;
    const double extent_r = cell_max - double(p);
    const double prob_l = (extent_l * area_mul + area_add) * cell_area_rcp;
    const double prob_r = (extent_r * area_mul + area_add) * cell_area_rcp;
    const int n_left_only = close + local_close;
    const int n_cross = open - n_left_only;
    const int n_right_only = int(G) - (n_left_only + n_cross + num_planars);
    const int tl[2] = {n_left_only + n_cross + num_planars, n_left_only + n_cross};
    const int tr[2] = {n_right_only + n_cross, n_right_only + n_cross + num_planars};
    const float eb[2] = {(tl[0] == 0 || tr[0] == 0) ? kEmptyBonus : 1.0f,
                         (tl[1] == 0 || tr[1] == 0) ? kEmptyBonus : 1.0f};
    double sah[2];
    for (int s = 0; s < 2; ++s) {
      switch (P.sah_mode) {
        case 0:
          sah[s] = kTravCost + P.isect_cost * (double(tl[s]) * prob_l + double(tr[s]) * prob_r) * eb[s];
          break;
        case 4: {
          auto scp = [](int n) -> double {
            if (n == 0) return 0.0;
            const double x = double(n);
            return x * std::pow(x / 16.0, 0.5);
          };
          sah[s] = kTravCost + P.isect_cost * (scp(tl[s]) * prob_l + scp(tr[s]) * prob_r) * eb[s];
          break;
        }
        case 7:
          sah[s] = kTravCost + P.isect_cost * (double(tl[s]) * prob_l + double(tr[s]) * prob_r) * eb[s] +
                   P.sort_cost * (double(tl[s]) * double(tl[s]) * prob_l + double(tr[s]) * double(tr[s]) * prob_r);
          break;
        default: {  // 1: balance-penalised SAH (Kd-treeConstructor.cpp:800-812)
          const double n_total = double(tl[s] + tr[s]);
          const double diff = std::abs(double(tl[s]) - double(tr[s]));
          const double ratio = (n_total > 0.0) ? (diff / n_total) : 0.0;
          const double penalty = 1.0 + (ratio * 0.1);
          sah[s] = kTravCost + P.isect_cost * (double(tl[s]) * prob_l + double(tr[s]) * prob_r) * eb[s] * penalty;
          break;
        }
      }
    }
    double cost;
    int side;
    if (sah[0] <= sah[1]) {
      cost = sah[0];
      side = 0;
    } else {
      cost = sah[1];
      side = 1;
    }
    if (cost < best.cost) {
      best.cost = cost;
      best.pos = p;
      best.axis = axis;
      best.planar_side = side;
    }
  }
}

bool edge_plane(const float* p0, const float* p1, const float* pp, const float* pn, float* hit) {
  float u[3], w[3];
  u[0] = p1[0] - p0[0];
  u[1] = p1[1] - p0[1];
  u[2] = p1[2] - p0[2];
  w[0] = p0[0] - pp[0];
  w[1] = p0[1] - pp[1];
  w[2] = p0[2] - pp[2];
  const float D = pn[0] * u[0] + pn[1] * u[1] + pn[2] * u[2];
  const float N = -(pn[0] * w[0] + pn[1] * w[1] + pn[2] * w[2]);
  if (std::fabs(D) < kEps) return false;
  const float sI = N / D;
  if (sI < 0.f || sI > 1.f) return false;
  hit[0] = p0[0] + u[0] * sI;
  hit[1] = p0[1] + u[1] * sI;
  hit[2] = p0[2] + u[2] * sI;
  return true;
}

// clip_triangle (Kd-treeConstructor.cpp:364-486) for one straddling triangle.
void clip_tri(Tri& t, int axis, float split, int side) {
  float pn[3] = {0.f, 0.f, 0.f};
  pn[axis] = 1.f;
  const float pp[3] = {pn[0] * split, pn[1] * split, pn[2] * split};
  float L[9][3], R[9][3];
  int nl = 0, nr = 0;
  for (int k = 0; k < 3; ++k) {
    float* dst = (t.v[k][axis] < split) ? L[nl++] : R[nr++];
    dst[0] = t.v[k][0];
    dst[1] = t.v[k][1];
    dst[2] = t.v[k][2];
  }
  const int l0 = nl, r0 = nr;
  for (int j = 0; j < l0; ++j)
    for (int k = 0; k < r0; ++k) {
      float h[3];
      if (edge_plane(L[j], R[k], pp, pn, h)) {
        memcpy(L[nl++], h, 12);
        memcpy(R[nr++], h, 12);
      }
    }
  float (*V)[3] = side == 0 ? L : R;
  const int nv = side == 0 ? nl : nr;
  float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};
  if (nv > 0) {
    for (int d = 0; d < 3; ++d) lo[d] = hi[d] = V[0][d];
    for (int j = 1; j < nv; ++j)
      for (int d = 0; d < 3; ++d) {
        lo[d] = ref_min(lo[d], V[j][d]);
        hi[d] = ref_max(hi[d], V[j][d]);
      }
    for (int d = 0; d < 3; ++d) {
      lo[d] = ref_max(lo[d], t.lo[d]);
      hi[d] = ref_min(hi[d], t.hi[d]);
    }
  }
  for (int d = 0; d < 3; ++d) {
    t.lo[d] = lo[d];
    t.hi[d] = hi[d];
  }
}

struct Builder {
  Params P;
  std::atomic<int> spare_threads{0};
  std::atomic<uint32_t> max_depth{0};

  std::unique_ptr<Node> build(std::vector<Tri> tris, const float blo[3], const float bhi[3], unsigned level) {
    auto node = std::make_unique<Node>();
    uint32_t md = max_depth.load();
    while (level > md && !max_depth.compare_exchange_weak(md, level)) {
    }
    // runs of equal Gaussian ID (tris stay sorted by ID through partitions)
    std::vector<uint32_t> run_start;
    run_start.reserve(tris.size() / 8 + 2);
    for (uint32_t i = 0; i < tris.size(); ++i)
      if (i == 0 || tris[i].gid != tris[i - 1].gid) run_start.push_back(i);
    run_start.push_back((uint32_t)tris.size());
    const size_t G = run_start.size() - 1;

    SplitChoice best;
    best.cost = double(G) * P.isect_cost;
    if (P.sah_mode == 6) best.cost = best.cost + P.sort_cost * G * std::log2((double)G);
    else if (P.sah_mode == 7) best.cost = best.cost + P.sort_cost * G * G;
    if (P.force_split && tris.size() > (size_t)P.force_split) best.cost = DBL_MAX;
    best.axis = -1;
    best.pos = FLT_MAX;
    best.planar_side = -1;

    if (level < (unsigned)P.max_level && G > kMinPrim) {
      SplitChoice ax[3] = {best, best, best};
      if (tris.size() > 200000) {
        std::thread th1([&] { try_axis(1, blo, bhi, tris, run_start, P, ax[1]); });
        std::thread th2([&] { try_axis(2, blo, bhi, tris, run_start, P, ax[2]); });
        try_axis(0, blo, bhi, tris, run_start, P, ax[0]);
        th1.join();
        th2.join();
      } else {
        for (int a = 0; a < 3; ++a) try_axis(a, blo, bhi, tris, run_start, P, ax[a]);
      }
      for (int a = 0; a < 3; ++a)
        if (ax[a].cost < best.cost) best = ax[a];
    }

    if (best.axis < 0) {
      node->ids.reserve(G);
      for (size_t g = 0; g < G; ++g) node->ids.push_back(tris[run_start[g]].gid);
      return node;
    }

    const int axis = best.axis;
    const float split = best.pos;
    std::vector<Tri> left, right;
    left.reserve(tris.size() / 2 + 16);
    right.reserve(tris.size() / 2 + 16);
    for (const Tri& t : tris) {
      const float mn = t.lo[axis], mx = t.hi[axis];
      if (mn != mx) {
        if (mn < split) left.push_back(t);
        if (mx > split) right.push_back(t);
      } else {
        if (mn < split) left.push_back(t);
        else if (mn > split) right.push_back(t);
        else if (best.planar_side == 0) left.push_back(t);
        else right.push_back(t);
      }
    }
    std::vector<Tri>().swap(tris);
    for (Tri& t : left)
      if (t.lo[axis] < split && t.hi[axis] > split) clip_tri(t, axis, split, 0);
    for (Tri& t : right)
      if (t.lo[axis] < split && t.hi[axis] > split) clip_tri(t, axis, split, 1);

    float llo[3], lhi[3], rlo[3], rhi[3];
    memcpy(llo, blo, 12);
    memcpy(lhi, bhi, 12);
    memcpy(rlo, blo, 12);
    memcpy(rhi, bhi, 12);
    lhi[axis] = split;
    rlo[axis] = split;
    node->axis = axis;
    node->split = split;

    const bool fork = left.size() > 20000 && right.size() > 20000 && spare_threads.fetch_sub(1) > 0;
    if (fork) {
      std::unique_ptr<Node> lk;
      std::thread th([&, l = std::move(left)]() mutable { lk = build(std::move(l), llo, lhi, level + 1); });
      node->kid[1] = build(std::move(right), rlo, rhi, level + 1);
      th.join();
      spare_threads.fetch_add(1);
      node->kid[0] = std::move(lk);
    } else {
      if (!fork && left.size() > 20000 && right.size() > 20000) spare_threads.fetch_add(1);
      node->kid[0] = build(std::move(left), llo, lhi, level + 1);
      node->kid[1] = build(std::move(right), rlo, rhi, level + 1);
    }
    return node;
  }
};

// Number nodes as the reference allocates them and append leaf ID lists.
void serialize(const Node* root, std::vector<uint32_t>& nodes, std::vector<uint32_t>& offsets, uint32_t& n_leaves,
               uint32_t& max_leaf) {
  struct Item {
    const Node* n;
    uint32_t slot;
  };
  std::vector<Item> stack;
  nodes.assign(2, 0);
  stack.push_back({root, 0});
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    const Node* n = it.n;
    if (n->axis < 0) {
      const uint32_t cnt = (uint32_t)n->ids.size();
      nodes[2 * it.slot] = (cnt << 3) | 3u;
      nodes[2 * it.slot + 1] = (uint32_t)offsets.size();
      offsets.insert(offsets.end(), n->ids.begin(), n->ids.end());
      ++n_leaves;
      if (cnt > max_leaf) max_leaf = cnt;
    } else {
      const uint32_t c = (uint32_t)(nodes.size() / 2);
      nodes.resize(nodes.size() + 4, 0);
      uint32_t bits;
      memcpy(&bits, &n->split, 4);
      nodes[2 * it.slot] = (c << 3) | (uint32_t)n->axis;
      nodes[2 * it.slot + 1] = bits;
      // left subtree allocates before right: push right first
      stack.push_back({n->kid[1].get(), c + 1});
      stack.push_back({n->kid[0].get(), c});
    }
  }
}

}  // namespace

const float kIcosaVerts[12][3] = {{-1.f, 1.618033988749895f, 0.f}, {1.f, 1.618033988749895f, 0.f},
                                  {0.f, 1.f, -1.618033988749895f}, {-1.618033988749895f, 0.f, -1.f},
                                  {-1.618033988749895f, 0.f, 1.f}, {0.f, 1.f, 1.618033988749895f},
                                  {1.618033988749895f, 0.f, 1.f},  {0.f, -1.f, 1.618033988749895f},
                                  {-1.f, -1.618033988749895f, 0.f}, {0.f, -1.f, -1.618033988749895f},
                                  {1.618033988749895f, 0.f, -1.f}, {1.f, -1.618033988749895f, 0.f}};
const int kIcosaFaces[20][3] = {{0, 1, 2},  {0, 2, 3},  {0, 3, 4},   {0, 4, 5},   {0, 5, 1},
                                {6, 1, 5},  {6, 5, 7},  {6, 7, 11},  {6, 11, 10}, {6, 10, 1},
                                {8, 4, 3},  {8, 3, 9},  {8, 9, 11},  {8, 11, 7},  {8, 7, 4},
                                {9, 3, 2},  {9, 2, 10}, {9, 10, 11}, {5, 4, 7},   {1, 10, 2}};

namespace {

inline void cross3(const float* a, const float* b, float* o) {
  o[0] = ((a[1] * b[2]) - (a[2] * b[1]));
  o[1] = -((a[0] * b[2]) - (a[2] * b[0]));
  o[2] = ((a[0] * b[1]) - (a[1] * b[0]));
}

}  // namespace

// Proxy triangles for one Gaussian: the 20-face icosahedron scaled by
// k_iso * scale, rotated by the quaternion and moved to the mean
// (Kd-treeConverterMain.cpp:1860-1922, 1975-2095).  Returns false when the
// Gaussian is cut (sigma < 0.0113 or sigma < 1/255, :1990-1997).
bool proxy_kiso(const float* g, float* k_iso) {
  const float sigma = g[3];
  const float kmin = 0.0113f;
  if (sigma < kmin || sigma < 1 / 255.0f) return false;
  float k = 0.0f;
  if (sigma / kmin > 1.0f) k = sqrtf(2.0f * logf(sigma / kmin)) * 0.5257311121191335703f;
  *k_iso = k;
  return true;
}

bool proxy_icosahedron(const float* g, float out[20][3][3]) {
  float k_iso;
  if (!proxy_kiso(g, &k_iso)) return false;
  const float fs[3] = {g[4] * k_iso, g[5] * k_iso, g[6] * k_iso};
  const float* q = g + 8;
  const float qv[3] = {q[1], q[2], q[3]};
  for (int f = 0; f < 20; ++f)
    for (int l = 0; l < 3; ++l) {
      const float* vc = kIcosaVerts[kIcosaFaces[f][l]];
      const float vs[3] = {vc[0] * fs[0], vc[1] * fs[1], vc[2] * fs[2]};
      float t[3], tt[3];
      cross3(qv, vs, t);
      for (int i = 0; i < 3; ++i) t[i] *= 2.0f;
      cross3(qv, t, tt);
      for (int i = 0; i < 3; ++i) out[f][l][i] = (vs[i] + q[0] * t[i] + tt[i]) + g[i];
    }
  return true;
}

int build_tree(const float* gauss, uint32_t n, const BuildParams& bp, HostTree& out, BuildStats* stats) {
  auto t0 = std::chrono::steady_clock::now();
  std::vector<Tri> tris;
  tris.reserve((size_t)n * 20);
  float aabb[6] = {FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX};  // xmin,xmax,ymin,...
  out.valid.assign(n, 0);
  float tv[20][3][3];
  uint32_t n_valid = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const float* g = gauss + (size_t)i * 64;
    if (!proxy_icosahedron(g, tv)) continue;
    out.valid[i] = 1;
    ++n_valid;
    for (int f = 0; f < 20; ++f) {
      Tri t;
      memcpy(t.v, tv[f], sizeof(t.v));
      for (int d = 0; d < 3; ++d) {
        t.lo[d] = ref_min(ref_min(t.v[0][d], t.v[1][d]), t.v[2][d]);
        t.hi[d] = ref_max(ref_max(t.v[0][d], t.v[1][d]), t.v[2][d]);
      }
      for (int l = 0; l < 3; ++l) {
        // generate_gaussian_mesh's AABB update uses cudaRenderer.h's
        // fminf/fmaxf overloads: (b > a) ? a : b and (b < a) ? a : b.
        for (int d = 0; d < 3; ++d) {
          const float x = t.v[l][d];
          aabb[2 * d] = (x > aabb[2 * d]) ? aabb[2 * d] : x;
          aabb[2 * d + 1] = (x < aabb[2 * d + 1]) ? aabb[2 * d + 1] : x;
        }
      }
      t.gid = i;
      t.pad = 0;
      tris.push_back(t);
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  Builder B;
  B.P = {bp.max_level, bp.force_split, bp.isect_cost, bp.sah_mode, bp.sort_cost};
  int hw = (int)std::thread::hardware_concurrency();
  B.spare_threads = std::max(0, (bp.threads > 0 ? bp.threads : hw) - 1);
  const float blo[3] = {aabb[0], aabb[2], aabb[4]};
  const float bhi[3] = {aabb[1], aabb[3], aabb[5]};
  const size_t ntri = tris.size();
  std::unique_ptr<Node> root = B.build(std::move(tris), blo, bhi, 0);
  auto t2 = std::chrono::steady_clock::now();
  out.nodes.clear();
  out.offsets.clear();
  uint32_t n_leaves = 0, max_leaf = 0;
  serialize(root.get(), out.nodes, out.offsets, n_leaves, max_leaf);
  // .kdt header order: xmin, ymin, zmin, xmax, ymax, zmax
  out.aabb[0] = aabb[0];
  out.aabb[1] = aabb[2];
  out.aabb[2] = aabb[4];
  out.aabb[3] = aabb[1];
  out.aabb[4] = aabb[3];
  out.aabb[5] = aabb[5];
  out.depth = B.max_depth.load();
  out.n_leaves = n_leaves;
  out.max_leaf = max_leaf;
  // free the pointer tree iteratively (deep trees)
  {
    std::vector<std::unique_ptr<Node>> st;
    st.push_back(std::move(root));
    while (!st.empty()) {
      std::unique_ptr<Node> nd = std::move(st.back());
      st.pop_back();
      if (nd->kid[0]) st.push_back(std::move(nd->kid[0]));
      if (nd->kid[1]) st.push_back(std::move(nd->kid[1]));
    }
  }
  auto t3 = std::chrono::steady_clock::now();
  if (stats) {
    stats->proxy_s = std::chrono::duration<double>(t1 - t0).count();
    stats->build_s = std::chrono::duration<double>(t2 - t1).count();
    stats->serialize_s = std::chrono::duration<double>(t3 - t2).count();
    stats->n_triangles = ntri;
    stats->n_valid = n_valid;
  }
  return 0;
}

}  // namespace kdgr
