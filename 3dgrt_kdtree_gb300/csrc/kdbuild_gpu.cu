// kdbuild_gpu.cu -- the kd-tree builder on the GPU.
//
// Builds the same tree, bit for bit, as the host builder (kdbuild.cpp),
// which itself reproduces the reference builder (Kd-treeConstructor.cpp,
// PRIMITIVE_TYPE 2 / COUNT_BY_GID 1): proxy icosahedra per Gaussian
// (Kd-treeConverterMain.cpp:1860-2095), SAH split search over every distinct
// triangle-edge position with per-Gaussian-ID counting (try_to_split,
// Kd-treeConstructor.cpp:579-868), partition and clip (:364-486, :545-577),
// leaves holding their sorted unique Gaussian IDs (:1543-1549).
//
// The host builder recurses depth first; here the tree grows breadth first,
// one level per step, every node of the level at once:
//   1. runs of equal Gaussian ID inside each node (triangles stay sorted by
//      node, then ID, through every partition) give per-ID intervals
//      [gmin, gmax] on each axis;
//   2. the candidate positions (both edges of every triangle), the interval
//      starts, ends and planar positions of every splittable node are sorted
//      at once as 64-bit keys (axis, node, position) -- one device radix sort
//      per list per level;
//   3. one thread per distinct candidate counts by binary search in the
//      sorted start/end/planar segments of its node and scores the SAH cost
//      in the host builder's types and operation order (double costs, float
//      extents); a two-pass atomic reduction keeps the first minimum in
//      ascending position, axis 0 first on ties, as the sequential sweep does;
//   4. triangles are partitioned stably into the children (two exclusive
//      scans give every triangle its slot) and straddling ones are clipped
//      with the host's float arithmetic;
//   5. leaves write the IDs of their runs into one pool.
// The node records come back to the host, which numbers the nodes as the
// reference allocates them (child pairs in depth-first, left-first order) and
// appends the leaf ID lists in the same order.
//
// This unit is compiled with --fmad=false and IEEE division, so every float
// and double expression rounds as on the host (compiled -ffp-contract=off).
// The per-Gaussian proxy scale k_iso (a logf) is computed on the host by the
// host builder's own function, so no device math library result enters the
// tree.  Known difference: the scene box is a min/max reduction, so a box
// face exactly at -0 versus +0 may take the other zero's bits than the
// sequential host loop would.
#include <cub/cub.cuh>

#include <cfloat>
#include <cstdio>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "kdgr.h"
#include "kdgr_internal.h"

namespace kdgr {
namespace {

constexpr float kTravCost = 1.0f;    // TRAVL_COST
constexpr float kEmptyBonus = 0.9f;  // EMTPY_BONUS
constexpr unsigned kMinPrim = 16;    // MIN_TRI
constexpr float kEps = 0.00001f;     // KD_TREE_EPSILON
constexpr uint32_t kNone = 0xFFFFFFFFu;

struct Params {
  int max_level;
  int force_split;
  float isect_cost;
  int sah_mode;
  float sort_cost;
};

// ------------------------------------------------------------ device buffers
// The build's stream and its own memory pool: the pool keeps what it has
// mapped until the build ends (the device's default pool would hand it back
// at every stream synchronisation, and the level loop synchronises often).
struct Stream {
  cudaStream_t s = nullptr;
  cudaMemPool_t pool = nullptr;
  cudaError_t err = cudaSuccess;
  void check(cudaError_t e) {
    if (err == cudaSuccess && e != cudaSuccess) err = e;
  }
};

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  Stream* st = nullptr;
  DBuf() = default;
  DBuf(Stream& s, size_t count) { alloc(s, count); }
  void alloc(Stream& s, size_t count) {
    release();
    st = &s;
    n = count;
    if (count) st->check(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p), count * sizeof(T), st->pool, st->s));
  }
  void release() {
    if (p && st) cudaFreeAsync(p, st->s);
    p = nullptr;
    n = 0;
  }
  void zero() {
    if (p) st->check(cudaMemsetAsync(p, 0, n * sizeof(T), st->s));
  }
  void fill_ff() {
    if (p) st->check(cudaMemsetAsync(p, 0xFF, n * sizeof(T), st->s));
  }
  ~DBuf() { release(); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), st(o.st) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      st = o.st;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
};

// Triangles of one level, SoA: v[k*cap + t] for the 9 vertex floats,
// lo/hi[a*cap + t] for the clipped box, the Gaussian ID and the node index.
struct TriSet {
  DBuf<float> v, lo, hi;
  DBuf<uint32_t> gid, node;
  size_t cap = 0;
  void alloc(Stream& s, size_t c) {
    cap = c;
    v.alloc(s, 9 * c);
    lo.alloc(s, 3 * c);
    hi.alloc(s, 3 * c);
    gid.alloc(s, c);
    node.alloc(s, c);
  }
};

template <typename T>
void exclusive_sum(Stream& s, const T* in, T* out, size_t n) {
  if (n == 0) return;
  size_t bytes = 0;
  s.check(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int64_t)n, s.s));
  DBuf<uint8_t> tmp(s, bytes);
  s.check(cub::DeviceScan::ExclusiveSum(tmp.p, bytes, in, out, (int64_t)n, s.s));
}

void sort_keys(Stream& s, DBuf<uint64_t>& keys, DBuf<uint64_t>& alt, size_t n, int end_bit) {
  if (n == 0) return;
  cub::DoubleBuffer<uint64_t> db(keys.p, alt.p);
  size_t bytes = 0;
  s.check(cub::DeviceRadixSort::SortKeys(nullptr, bytes, db, (int64_t)n, 0, end_bit, s.s));
  DBuf<uint8_t> tmp(s, bytes);
  s.check(cub::DeviceRadixSort::SortKeys(tmp.p, bytes, db, (int64_t)n, 0, end_bit, s.s));
  if (db.Current() != keys.p) std::swap(keys.p, alt.p);
}

template <typename T>
T read_one(Stream& s, const T* dev) {
  T v{};
  s.check(cudaMemcpyAsync(&v, dev, sizeof(T), cudaMemcpyDeviceToHost, s.s));
  s.check(cudaStreamSynchronize(s.s));
  return v;
}

// at least one block: every kernel checks its own bounds
inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)std::max<size_t>(1, (n + block - 1) / block); }

// ------------------------------------------------------------ key encoding
// (axis, node, position) -> 64-bit key ordered by axis, then node, then
// position (the float's bits mapped to an order-preserving unsigned; -0
// sorts before +0 as a distinct key, like the host radix sort).
__device__ __forceinline__ uint32_t ordf(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unordf(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
__device__ __forceinline__ uint64_t make_key(int axis, uint32_t node, float p, int nb) {
  return ((uint64_t)axis << (32 + nb)) | ((uint64_t)node << 32) | ordf(p);
}
__device__ __forceinline__ float key_pos(uint64_t k) { return unordf((uint32_t)k); }

// Elements of the sorted segment [b, b + n) whose position compares < p,
// and those that compare == p (float comparison: -0 == +0).
__device__ __forceinline__ uint32_t count_less(const uint64_t* k, size_t b, uint32_t n, float p) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (key_pos(k[b + mid]) < p) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ uint32_t count_le(const uint64_t* k, size_t b, uint32_t n, float p) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (key_pos(k[b + mid]) <= p) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The same counts with the answer known to lie in [lo, hi].
__device__ __forceinline__ uint32_t count_less_in(const uint64_t* k, size_t b, uint32_t lo, uint32_t hi, float p) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (key_pos(k[b + mid]) < p) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ uint32_t count_le_in(const uint64_t* k, size_t b, uint32_t lo, uint32_t hi, float p) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (key_pos(k[b + mid]) <= p) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Bounds for the counts of a warp whose 32 lanes hold consecutive sorted
// candidates of one segment: every lane's count lies between lane 0's
// count_less and lane 31's count_le, found once by those two lanes.
struct Bracket {
  uint32_t lo, hi;
};
__device__ __forceinline__ Bracket warp_bracket(const uint64_t* k, size_t b, uint32_t n, float p, int lane) {
  uint32_t v = 0;
  if (lane == 0) v = count_less(k, b, n, p);
  if (lane == 31) v = count_le(k, b, n, p);
  return Bracket{__shfl_sync(0xFFFFFFFFu, v, 0), __shfl_sync(0xFFFFFFFFu, v, 31)};
}

__device__ __forceinline__ float ref_min(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float ref_max(float a, float b) { return a > b ? a : b; }

// ------------------------------------------------------------ proxy mesh
__constant__ float c_ico_v[12][3];
__constant__ int c_ico_f[20][3];

__device__ __forceinline__ void cross3(const float* a, const float* b, float* o) {
  o[0] = ((a[1] * b[2]) - (a[2] * b[1]));
  o[1] = -((a[0] * b[2]) - (a[2] * b[0]));
  o[2] = ((a[0] * b[1]) - (a[1] * b[0]));
}

// One thread per proxy triangle: the icosahedron face scaled by k_iso *
// scale, rotated by the quaternion, moved to the mean (the host builder's
// proxy_icosahedron, operation for operation).  g: 10 floats per valid
// Gaussian (pos, scale, quaternion w,x,y,z).
__global__ void k_proxy(const float* __restrict__ g, const float* __restrict__ kiso, const uint32_t* __restrict__ ids,
                        uint32_t n_valid, float* v, float* lo, float* hi, uint32_t* gid,
                        uint32_t* node, size_t cap) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n_valid * 20) return;
  const uint32_t j = (uint32_t)(t / 20), f = (uint32_t)(t % 20);
  const float* gj = g + 10ull * j;
  const float k = kiso[j];
  const float fs[3] = {gj[3] * k, gj[4] * k, gj[5] * k};
  const float q0 = gj[6];
  const float qv[3] = {gj[7], gj[8], gj[9]};
  float out[3][3];
  for (int l = 0; l < 3; ++l) {
    const float* vc = c_ico_v[c_ico_f[f][l]];
    const float vs[3] = {vc[0] * fs[0], vc[1] * fs[1], vc[2] * fs[2]};
    float tv[3], tt[3];
    cross3(qv, vs, tv);
    for (int i = 0; i < 3; ++i) tv[i] *= 2.0f;
    cross3(qv, tv, tt);
    for (int i = 0; i < 3; ++i) out[l][i] = (vs[i] + q0 * tv[i] + tt[i]) + gj[i];
  }
  for (int l = 0; l < 3; ++l)
    for (int i = 0; i < 3; ++i) v[(3 * l + i) * cap + t] = out[l][i];
  for (int d = 0; d < 3; ++d) {
    lo[d * cap + t] = ref_min(ref_min(out[0][d], out[1][d]), out[2][d]);
    hi[d * cap + t] = ref_max(ref_max(out[0][d], out[1][d]), out[2][d]);
  }
  gid[t] = ids[j];
  node[t] = 0;
}

// Scene box over every proxy vertex: per-block reduction of order-mapped
// keys, then one atomic per block and bound.
__global__ void k_scene_box(const float* __restrict__ v, size_t cap, size_t n, uint32_t* box) {
  uint32_t mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0, 0, 0};
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    for (int l = 0; l < 3; ++l)
      for (int d = 0; d < 3; ++d) {
        const uint32_t k = ordf(v[(3 * l + d) * cap + t]);
        mn[d] = min(mn[d], k);
        mx[d] = max(mx[d], k);
      }
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[d] = min(mn[d], __shfl_xor_sync(0xFFFFFFFFu, mn[d], o));
      mx[d] = max(mx[d], __shfl_xor_sync(0xFFFFFFFFu, mx[d], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&box[2 * d], mn[d]);
      atomicMax(&box[2 * d + 1], mx[d]);
    }
  }
}

__global__ void k_box_decode(const uint32_t* box, float* node_lo, float* node_hi) {
  if (threadIdx.x < 3) {
    node_lo[threadIdx.x] = unordf(box[2 * threadIdx.x]);
    node_hi[threadIdx.x] = unordf(box[2 * threadIdx.x + 1]);
  }
}

// ------------------------------------------------------------ level kernels
__global__ void k_run_heads(const uint32_t* __restrict__ gid, const uint32_t* __restrict__ node, size_t T,
                            uint32_t* flag) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t > T) return;
  flag[t] = (t < T && (t == 0 || gid[t] != gid[t - 1] || node[t] != node[t - 1])) ? 1u : 0u;
}

__global__ void k_run_scatter(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ ridx,
                              const uint32_t* __restrict__ node, size_t T, uint32_t* run_start, uint32_t* run_node) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T || !flag[t]) return;
  run_start[ridx[t]] = (uint32_t)t;
  run_node[ridx[t]] = node[t];
}

// First run of every node: runs are ordered by node, so node n's runs start
// at the run index of its first triangle (an empty node gets the next node's
// first run), and G[n] = rb[n+1] - rb[n].  rb[N] = R.
__global__ void k_node_runs(const uint32_t* __restrict__ tb, const uint32_t* __restrict__ ridx, uint32_t N,
                            uint32_t* rb, uint32_t* G) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n > N) return;
  rb[n] = ridx[tb[n]];
  if (n < N) G[n] = ridx[tb[n + 1]] - ridx[tb[n]];
}

struct NodeConst {
  double cell_area_rcp[3], area_mul[3], area_add[3];
  float cell_min[3], cell_max[3], lim_lo[3], lim_hi[3];
  double init_cost;
  uint32_t G, T;
  int elig;
};

// Per node: leaf cost, eligibility and the per-axis cell constants of
// try_to_split, in the host builder's types.
__global__ void k_node_setup(const uint32_t* __restrict__ tb, const uint32_t* __restrict__ G,
                             const float* __restrict__ nlo, const float* __restrict__ nhi, uint32_t N, int level,
                             Params P, NodeConst* nc, uint32_t* eT, uint32_t* eG) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  NodeConst c;
  c.T = tb[n + 1] - tb[n];
  c.G = G[n];
  const size_t Gs = c.G;
  double cost = double(Gs) * P.isect_cost;
  if (P.sah_mode == 7) cost = cost + P.sort_cost * Gs * Gs;
  if (P.force_split && (size_t)c.T > (size_t)P.force_split) cost = DBL_MAX;
  c.init_cost = cost;
  c.elig = (level < P.max_level && c.G > kMinPrim) ? 1 : 0;
  float blo[3], bhi[3], ext[3];
  for (int d = 0; d < 3; ++d) {
    blo[d] = nlo[3 * n + d];
    bhi[d] = nhi[3 * n + d];
    ext[d] = bhi[d] - blo[d];
  }
  const float cell_area_f = (ext[0] * ext[1]) + (ext[1] * ext[2]) + (ext[0] * ext[2]);
  const double cell_area = cell_area_f;
  for (int a = 0; a < 3; ++a) {
    const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
    c.cell_area_rcp[a] = 1 / cell_area;
    c.area_mul[a] = double(ext[a1]) + double(ext[a2]);
    c.area_add[a] = double(ext[a1]) * double(ext[a2]);
    c.cell_min[a] = blo[a];
    c.cell_max[a] = bhi[a];
    c.lim_lo[a] = blo[a] + kEps;
    c.lim_hi[a] = bhi[a] - kEps;
  }
  nc[n] = c;
  eT[n] = c.elig ? c.T : 0u;
  eG[n] = c.elig ? c.G : 0u;
}

// Per run: the ID's interval on each axis (first triangle's box, then
// strict comparisons, in triangle order, as the host sweep builds it) and
// the keys of the interval starts, ends and planar positions.
__global__ void k_run_bounds(const uint32_t* __restrict__ run_start, const uint32_t* __restrict__ run_node,
                             uint32_t R, size_t T, const float* __restrict__ lo, const float* __restrict__ hi,
                             size_t cap, const NodeConst* __restrict__ nc, const uint32_t* __restrict__ rb,
                             const uint32_t* __restrict__ grb, size_t eGT, int nb, uint64_t* kmin, uint64_t* kmax,
                             uint64_t* kpl, uint32_t* pl_cnt, unsigned long long* pl_fill, uint32_t N) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const uint32_t n = run_node[r];
  if (!nc[n].elig) return;
  const uint32_t t0 = run_start[r], t1 = r + 1 < R ? run_start[r + 1] : (uint32_t)T;
  const size_t slot = grb[n] + (r - rb[n]);
  for (int a = 0; a < 3; ++a) {
    float mn = lo[a * cap + t0], mx = hi[a * cap + t0];
    for (uint32_t t = t0 + 1; t < t1; ++t) {
      const float l = lo[a * cap + t], h = hi[a * cap + t];
      if (l < mn) mn = l;
      if (h > mx) mx = h;
    }
    kmin[a * eGT + slot] = make_key(a, n, mn, nb);
    kmax[a * eGT + slot] = make_key(a, n, mx, nb);
    if (mn == mx) {
      const unsigned long long at = atomicAdd(pl_fill, 1ull);
      kpl[at] = make_key(a, n, mn, nb);
      atomicAdd(&pl_cnt[(size_t)a * N + n], 1u);
    }
  }
}

// Candidate positions of a run (one Gaussian's triangles in one node): the
// lo and hi edges of its triangles on axis a, bitwise duplicates removed
// (-0 and +0 stay distinct, as in the full sorted list; the sweep groups
// equal positions anyway, so the scored candidates are the same).  A run
// holds at most 20 triangles; longer runs (not produced by the proxy mesh)
// keep every edge.
constexpr int kRunEdges = 64;

template <bool WRITE>
__device__ __forceinline__ uint32_t run_edges(const float* __restrict__ lo, const float* __restrict__ hi, size_t cap,
                                              uint32_t t0, uint32_t t1, int a, uint32_t n, int nb, uint64_t* out) {
  const uint32_t m = 2 * (t1 - t0);
  uint32_t count = 0;
  if (m > (uint32_t)kRunEdges) {
    for (uint32_t t = t0; t < t1; ++t) {
      if (WRITE) {
        out[count] = make_key(a, n, lo[a * cap + t], nb);
        out[count + 1] = make_key(a, n, hi[a * cap + t], nb);
      }
      count += 2;
    }
    return count;
  }
  uint32_t v[kRunEdges];
  for (uint32_t t = t0; t < t1; ++t) {
    v[2 * (t - t0)] = __float_as_uint(lo[a * cap + t]);
    v[2 * (t - t0) + 1] = __float_as_uint(hi[a * cap + t]);
  }
  for (uint32_t j = 0; j < m; ++j) {
    bool seen = false;
    for (uint32_t k = 0; k < j && !seen; ++k) seen = v[k] == v[j];
    if (seen) continue;
    if (WRITE) out[count] = make_key(a, n, __uint_as_float(v[j]), nb);
    ++count;
  }
  return count;
}

// Pass 1: distinct candidate count per (axis, run); 0 for runs of nodes that
// are not split candidates.
__global__ void k_run_cand_count(const uint32_t* __restrict__ run_start, const uint32_t* __restrict__ run_node,
                                 uint32_t R, size_t T, const float* __restrict__ lo, const float* __restrict__ hi,
                                 size_t cap, const NodeConst* __restrict__ nc, unsigned long long* cnt) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const uint32_t n = run_node[r];
  const uint32_t t0 = run_start[r], t1 = r + 1 < R ? run_start[r + 1] : (uint32_t)T;
  for (int a = 0; a < 3; ++a)
    cnt[(size_t)a * R + r] = nc[n].elig ? run_edges<false>(lo, hi, cap, t0, t1, a, n, 0, nullptr) : 0u;
}

// Pass 2: the keys, at the scanned offsets.
__global__ void k_run_cand_write(const uint32_t* __restrict__ run_start, const uint32_t* __restrict__ run_node,
                                 uint32_t R, size_t T, const float* __restrict__ lo, const float* __restrict__ hi,
                                 size_t cap, const NodeConst* __restrict__ nc, const unsigned long long* __restrict__ off,
                                 int nb, uint64_t* kc) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const uint32_t n = run_node[r];
  if (!nc[n].elig) return;
  const uint32_t t0 = run_start[r], t1 = r + 1 < R ? run_start[r + 1] : (uint32_t)T;
  for (int a = 0; a < 3; ++a) run_edges<true>(lo, hi, cap, t0, t1, a, n, nb, kc + off[(size_t)a * R + r]);
}

__device__ __forceinline__ void decode(uint64_t k, int nb, int* a, uint32_t* n) {
  *a = (int)(k >> (32 + nb));
  *n = (uint32_t)((k >> 32) & ((1ull << nb) - 1));
}

// One thread per sorted candidate: the SAH score of the first candidate of
// each group of equal positions inside (cell_min + eps, cell_max - eps).
__global__ void k_eval(const uint64_t* __restrict__ kc, size_t n_cand, const unsigned long long* __restrict__ coff,
                       const uint32_t* __restrict__ rb, uint32_t R, int nb,
                       const uint64_t* __restrict__ kmin, const uint64_t* __restrict__ kmax,
                       const uint64_t* __restrict__ kpl, size_t eGT, const uint32_t* __restrict__ grb,
                       const uint32_t* __restrict__ plb,
                       const uint32_t* __restrict__ pl_cnt, const NodeConst* __restrict__ nc, uint32_t N, Params P,
                       double* cost_out, uint8_t* side_out, unsigned long long* best_bits) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  double cost = __longlong_as_double(0x7FF0000000000000ll);  // +inf: not a candidate
  uint8_t side = 0;
  uint32_t seg = kNone;
  // warp-wide brackets when all 32 lanes sit in one (axis, node) segment
  uint32_t my_seg = kNone;
  float my_p = 0.f;
  if (i < n_cand) {
    int a0;
    uint32_t n0;
    decode(kc[i], nb, &a0, &n0);
    my_seg = (uint32_t)a0 * N + n0;
    my_p = key_pos(kc[i]);
  }
  const bool uniform = __all_sync(0xFFFFFFFFu, my_seg == __shfl_sync(0xFFFFFFFFu, my_seg, 0) && my_seg != kNone);
  Bracket bmin{0, 0}, bmax{0, 0}, bpl{0, 0};
  if (uniform) {
    const uint32_t a0 = my_seg / N, n0 = my_seg % N;
    const uint32_t G0 = nc[n0].G;
    const size_t gb0 = (size_t)a0 * eGT + grb[n0];
    bmin = warp_bracket(kmin, gb0, G0, my_p, lane);
    bmax = warp_bracket(kmax, gb0, G0, my_p, lane);
    bpl = warp_bracket(kpl, plb[my_seg], pl_cnt[my_seg], my_p, lane);
  }
  if (i < n_cand) {
    const uint64_t k = kc[i];
    int a;
    uint32_t n;
    decode(k, nb, &a, &n);
    const float p = key_pos(k);
    const size_t s0 = coff[(size_t)a * R + rb[n]];
    const NodeConst& c = nc[n];
    const bool head = (i == s0) || !(key_pos(kc[i - 1]) == p);
    if (head && p > c.lim_lo[a] && p < c.lim_hi[a]) {
      const uint32_t G = c.G;
      const size_t gb = (size_t)a * eGT + grb[n];
      const size_t pb = plb[(size_t)a * N + n];
      const uint32_t pn = pl_cnt[(size_t)a * N + n];
      uint32_t open, close, eq_max, pl_lt, pl_le;
      if (uniform) {
        open = count_less_in(kmin, gb, bmin.lo, bmin.hi, p);
        close = count_less_in(kmax, gb, bmax.lo, bmax.hi, p);
        eq_max = count_le_in(kmax, gb, close, bmax.hi, p) - close;
        pl_lt = count_less_in(kpl, pb, bpl.lo, bpl.hi, p);
        pl_le = count_le_in(kpl, pb, pl_lt, bpl.hi, p);
      } else {
        open = count_less(kmin, gb, G, p);
        close = count_less(kmax, gb, G, p);
        eq_max = count_le(kmax, gb, G, p) - close;
        pl_lt = count_less(kpl, pb, pn, p);
        pl_le = count_le(kpl, pb, pn, p);
      }
      const int num_planars = (int)(pl_le - pl_lt);
      const int local_close = (int)eq_max - num_planars;

      const double extent_l = double(p) - c.cell_min[a];
      const double extent_r = c.cell_max[a] - double(p);
      const double prob_l = (extent_l * c.area_mul[a] + c.area_add[a]) * c.cell_area_rcp[a];
      const double prob_r = (extent_r * c.area_mul[a] + c.area_add[a]) * c.cell_area_rcp[a];
      const int n_left_only = (int)close + local_close;
      const int n_cross = (int)open - n_left_only;
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
            // n * pow(n / 16, 0.5) with the square root, which is what a
            // correctly rounded pow returns for the exponent 0.5
            const double xl = double(tl[s]), xr = double(tr[s]);
            const double sl = tl[s] == 0 ? 0.0 : xl * sqrt(xl / 16.0);
            const double sr = tr[s] == 0 ? 0.0 : xr * sqrt(xr / 16.0);
            sah[s] = kTravCost + P.isect_cost * (sl * prob_l + sr * prob_r) * eb[s];
            break;
          }
          case 7:
            sah[s] = kTravCost + P.isect_cost * (double(tl[s]) * prob_l + double(tr[s]) * prob_r) * eb[s] +
                     P.sort_cost * (double(tl[s]) * double(tl[s]) * prob_l + double(tr[s]) * double(tr[s]) * prob_r);
            break;
          default: {
            const double n_total = double(tl[s] + tr[s]);
            const double diff = fabs(double(tl[s]) - double(tr[s]));
            const double ratio = (n_total > 0.0) ? (diff / n_total) : 0.0;
            const double penalty = 1.0 + (ratio * 0.1);
            sah[s] = kTravCost + P.isect_cost * (double(tl[s]) * prob_l + double(tr[s]) * prob_r) * eb[s] * penalty;
            break;
          }
        }
      }
      const double cst = sah[0] <= sah[1] ? sah[0] : sah[1];
      if (cst < c.init_cost) {
        cost = cst;
        side = sah[0] <= sah[1] ? 0 : 1;
        seg = (uint32_t)a * N + n;
      }
    }
    cost_out[i] = cost;
    side_out[i] = side;
  }
  // min over the segment: a warp whose valid lanes share one segment
  // reduces first; a block whose warps all share one segment reduces again
  // and issues one atomic (the top levels have three segments and tens of
  // millions of candidates)
  unsigned long long bits = (unsigned long long)__double_as_longlong(cost);
  uint32_t lead = seg;
  for (int o = 16; o > 0; o >>= 1) lead = min(lead, __shfl_xor_sync(0xFFFFFFFFu, lead, o));
  const bool warp_uniform = __all_sync(0xFFFFFFFFu, seg == lead || seg == kNone);
  if (warp_uniform) {
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_xor_sync(0xFFFFFFFFu, bits, o);
      bits = other < bits ? other : bits;
    }
  } else if (seg != kNone) {
    atomicMin(&best_bits[seg], bits);
  }
  __shared__ uint32_t s_seg[8];
  __shared__ unsigned long long s_bits[8];
  const int w = threadIdx.x >> 5;
  if (lane == 0) {
    s_seg[w] = warp_uniform ? lead : 0xFFFFFFFEu;  // 0xFFFFFFFE: this warp has already issued its atomics
    s_bits[w] = bits;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (int)(blockDim.x >> 5);
    uint32_t bs = kNone;
    bool same = true;
    for (int k = 0; k < nw; ++k) {
      if (s_seg[k] == kNone) continue;
      if (s_seg[k] == 0xFFFFFFFEu || (bs != kNone && s_seg[k] != bs)) same = false;
      if (bs == kNone && s_seg[k] != 0xFFFFFFFEu) bs = s_seg[k];
    }
    if (same && bs != kNone) {
      unsigned long long m = ~0ull;
      for (int k = 0; k < nw; ++k)
        if (s_seg[k] == bs && s_bits[k] < m) m = s_bits[k];
      atomicMin(&best_bits[bs], m);
    } else {
      for (int k = 0; k < nw; ++k)
        if (s_seg[k] != kNone && s_seg[k] != 0xFFFFFFFEu) atomicMin(&best_bits[s_seg[k]], s_bits[k]);
    }
  }
}

// Second pass: the first (lowest sorted index) candidate with the minimum.
__global__ void k_argmin(const uint64_t* __restrict__ kc, const double* __restrict__ cost, size_t n_cand, int nb,
                         uint32_t N, const unsigned long long* __restrict__ best_bits, unsigned long long* best_idx) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_cand) return;
  const double c = cost[i];
  if (isinf(c)) return;
  int a;
  uint32_t n;
  decode(kc[i], nb, &a, &n);
  const size_t seg = (size_t)a * N + n;
  if ((unsigned long long)__double_as_longlong(c) == best_bits[seg]) atomicMin(&best_idx[seg], (unsigned long long)i);
}

struct Decision {
  int axis;  // -1: leaf
  float split;
  int side;
};

__global__ void k_choose(const NodeConst* __restrict__ nc, uint32_t N, const unsigned long long* __restrict__ best_bits,
                         const unsigned long long* __restrict__ best_idx, const uint64_t* __restrict__ kc,
                         const uint8_t* __restrict__ side, Decision* dec, uint32_t* is_split) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double cur = nc[n].init_cost;
  Decision d{-1, 0.f, 0};
  if (nc[n].elig) {
    for (int a = 0; a < 3; ++a) {
      const size_t seg = (size_t)a * N + n;
      if (best_idx[seg] == ~0ull) continue;
      const double c = __longlong_as_double((long long)best_bits[seg]);
      if (c < cur) {
        cur = c;
        d.axis = a;
        d.split = key_pos(kc[best_idx[seg]]);
        d.side = side[best_idx[seg]];
      }
    }
  }
  dec[n] = d;
  is_split[n] = d.axis >= 0 ? 1u : 0u;
}

// Which children a triangle goes to (push_triangles_to_child_vector).
__device__ __forceinline__ void sides_of(float mn, float mx, const Decision& d, bool* l, bool* r) {
  if (mn != mx) {
    *l = mn < d.split;
    *r = mx > d.split;
  } else {
    *l = mn < d.split || (mn == d.split && d.side == 0);
    *r = mn > d.split || (mn == d.split && d.side != 0);
  }
}

__global__ void k_part_flags(const float* __restrict__ lo, const float* __restrict__ hi, size_t cap, size_t T,
                             const uint32_t* __restrict__ node, const Decision* __restrict__ dec, uint32_t* fl,
                             uint32_t* fr) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t > T) return;
  bool l = false, r = false;
  if (t < T) {
    const Decision d = dec[node[t]];
    if (d.axis >= 0) sides_of(lo[d.axis * cap + t], hi[d.axis * cap + t], d, &l, &r);
  }
  fl[t] = l;
  fr[t] = r;
}

__global__ void k_child_counts(const uint32_t* __restrict__ tb, const uint32_t* __restrict__ sl,
                               const uint32_t* __restrict__ sr, const uint32_t* __restrict__ is_split,
                               const uint32_t* __restrict__ ns, uint32_t N, uint32_t* cc) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N || !is_split[n]) return;
  cc[2 * ns[n]] = sl[tb[n + 1]] - sl[tb[n]];
  cc[2 * ns[n] + 1] = sr[tb[n + 1]] - sr[tb[n]];
}

// clip_triangle for one straddling triangle (host clip_tri, same arithmetic).
__device__ bool edge_plane(const float* p0, const float* p1, const float* pp, const float* pn, float* hit) {
  float u[3], w[3];
  u[0] = p1[0] - p0[0];
  u[1] = p1[1] - p0[1];
  u[2] = p1[2] - p0[2];
  w[0] = p0[0] - pp[0];
  w[1] = p0[1] - pp[1];
  w[2] = p0[2] - pp[2];
  const float D = pn[0] * u[0] + pn[1] * u[1] + pn[2] * u[2];
  const float Nn = -(pn[0] * w[0] + pn[1] * w[1] + pn[2] * w[2]);
  if (fabsf(D) < kEps) return false;
  const float sI = Nn / D;
  if (sI < 0.f || sI > 1.f) return false;
  hit[0] = p0[0] + u[0] * sI;
  hit[1] = p0[1] + u[1] * sI;
  hit[2] = p0[2] + u[2] * sI;
  return true;
}

__device__ void clip_box(const float v[3][3], float lo[3], float hi[3], int axis, float split, int side) {
  float pn[3] = {0.f, 0.f, 0.f};
  pn[axis] = 1.f;
  const float pp[3] = {pn[0] * split, pn[1] * split, pn[2] * split};
  float L[9][3], R[9][3];
  int nl = 0, nr = 0;
  for (int k = 0; k < 3; ++k) {
    float* dst = (v[k][axis] < split) ? L[nl++] : R[nr++];
    dst[0] = v[k][0];
    dst[1] = v[k][1];
    dst[2] = v[k][2];
  }
  const int l0 = nl, r0 = nr;
  for (int j = 0; j < l0; ++j)
    for (int k = 0; k < r0; ++k) {
      float h[3];
      if (edge_plane(L[j], R[k], pp, pn, h)) {
        for (int d = 0; d < 3; ++d) {
          L[nl][d] = h[d];
          R[nr][d] = h[d];
        }
        ++nl;
        ++nr;
      }
    }
  float(*V)[3] = side == 0 ? L : R;
  const int nv = side == 0 ? nl : nr;
  float nlo[3] = {0.f, 0.f, 0.f}, nhi[3] = {0.f, 0.f, 0.f};
  if (nv > 0) {
    for (int d = 0; d < 3; ++d) nlo[d] = nhi[d] = V[0][d];
    for (int j = 1; j < nv; ++j)
      for (int d = 0; d < 3; ++d) {
        nlo[d] = ref_min(nlo[d], V[j][d]);
        nhi[d] = ref_max(nhi[d], V[j][d]);
      }
    for (int d = 0; d < 3; ++d) {
      nlo[d] = ref_max(nlo[d], lo[d]);
      nhi[d] = ref_min(nhi[d], hi[d]);
    }
  }
  for (int d = 0; d < 3; ++d) {
    lo[d] = nlo[d];
    hi[d] = nhi[d];
  }
}

__global__ void k_part_scatter(const float* __restrict__ v, const float* __restrict__ lo, const float* __restrict__ hi,
                               const uint32_t* __restrict__ gid, const uint32_t* __restrict__ node, size_t cap,
                               size_t T, const uint32_t* __restrict__ tb, const Decision* __restrict__ dec,
                               const uint32_t* __restrict__ ns, const uint32_t* __restrict__ sl,
                               const uint32_t* __restrict__ sr, const uint32_t* __restrict__ ntb, float* v2,
                               float* lo2, float* hi2, uint32_t* gid2, uint32_t* node2, size_t cap2) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const uint32_t n = node[t];
  const Decision d = dec[n];
  if (d.axis < 0) return;
  bool gl, gr;
  sides_of(lo[d.axis * cap + t], hi[d.axis * cap + t], d, &gl, &gr);
  if (!gl && !gr) return;
  float vv[3][3], blo[3], bhi[3];
  for (int l = 0; l < 3; ++l)
    for (int i = 0; i < 3; ++i) vv[l][i] = v[(3 * l + i) * cap + t];
  for (int a = 0; a < 3; ++a) {
    blo[a] = lo[a * cap + t];
    bhi[a] = hi[a * cap + t];
  }
  const bool straddle = blo[d.axis] < d.split && bhi[d.axis] > d.split;
  for (int s = 0; s < 2; ++s) {
    if (s == 0 ? !gl : !gr) continue;
    const uint32_t child = 2 * ns[n] + s;
    const size_t pos = ntb[child] + (s == 0 ? (sl[t] - sl[tb[n]]) : (sr[t] - sr[tb[n]]));
    float clo[3] = {blo[0], blo[1], blo[2]}, chi[3] = {bhi[0], bhi[1], bhi[2]};
    if (straddle) clip_box(vv, clo, chi, d.axis, d.split, s);
    for (int k = 0; k < 9; ++k) v2[k * cap2 + pos] = v[k * cap + t];
    for (int a = 0; a < 3; ++a) {
      lo2[a * cap2 + pos] = clo[a];
      hi2[a * cap2 + pos] = chi[a];
    }
    gid2[pos] = gid[t];
    node2[pos] = child;
  }
}

__global__ void k_child_boxes(const float* __restrict__ nlo, const float* __restrict__ nhi,
                              const Decision* __restrict__ dec, const uint32_t* __restrict__ ns, uint32_t N,
                              float* clo, float* chi) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N || dec[n].axis < 0) return;
  for (int s = 0; s < 2; ++s) {
    const uint32_t c = 2 * ns[n] + s;
    for (int d = 0; d < 3; ++d) {
      clo[3 * c + d] = nlo[3 * n + d];
      chi[3 * c + d] = nhi[3 * n + d];
    }
    if (s == 0) chi[3 * c + dec[n].axis] = dec[n].split;
    else clo[3 * c + dec[n].axis] = dec[n].split;
  }
}

__global__ void k_leaf_sizes(const uint32_t* __restrict__ is_split, const uint32_t* __restrict__ G, uint32_t N,
                             uint32_t* lsz) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < N) lsz[n] = is_split[n] ? 0u : G[n];
}

__global__ void k_leaf_ids(const uint32_t* __restrict__ run_start, const uint32_t* __restrict__ run_node, uint32_t R,
                           const uint32_t* __restrict__ gid, const uint32_t* __restrict__ is_split,
                           const uint32_t* __restrict__ rb, const uint32_t* __restrict__ loff, uint32_t* pool) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const uint32_t n = run_node[r];
  if (is_split[n]) return;
  pool[loff[n] + (r - rb[n])] = gid[run_start[r]];
}

// Host record of one node, breadth-first numbering.
struct Rec {
  int axis;
  float split;
  uint32_t first_child;  // global BFS index of the left child
  uint32_t leaf_off, leaf_cnt;
};

}  // namespace

int build_tree_gpu(const float* gauss, uint32_t n, const BuildParams& bp, HostTree& out, BuildStats* stats,
                   std::string& err) {
  using clk = std::chrono::steady_clock;
  auto t0 = clk::now();
  // per-Gaussian proxy scale on the host (the host builder's function)
  std::vector<float> gv;
  std::vector<float> kiso;
  std::vector<uint32_t> ids;
  gv.reserve((size_t)n * 10);
  out.valid.assign(n, 0);
  for (uint32_t i = 0; i < n; ++i) {
    const float* g = gauss + (size_t)i * 64;
    float k;
    if (!proxy_kiso(g, &k)) continue;
    out.valid[i] = 1;
    gv.insert(gv.end(), {g[0], g[1], g[2], g[4], g[5], g[6], g[8], g[9], g[10], g[11]});
    kiso.push_back(k);
    ids.push_back(i);
  }
  const uint32_t n_valid = (uint32_t)ids.size();
  if (n_valid == 0) {
    err = "every Gaussian is below the opacity cut; nothing to build";
    return KDGR_ERR_INVALID_ARG;
  }
  bool limit_hit = false;
  Stream S;
  S.check(cudaStreamCreateWithFlags(&S.s, cudaStreamNonBlocking));
  {
    int dev = 0;
    S.check(cudaGetDevice(&dev));
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    S.check(cudaMemPoolCreate(&S.pool, &props));
    uint64_t keep = UINT64_MAX;
    if (S.pool) S.check(cudaMemPoolSetAttribute(S.pool, cudaMemPoolAttrReleaseThreshold, &keep));
  }
  S.check(cudaMemcpyToSymbolAsync(c_ico_v, kIcosaVerts, sizeof kIcosaVerts, 0, cudaMemcpyHostToDevice, S.s));
  S.check(cudaMemcpyToSymbolAsync(c_ico_f, kIcosaFaces, sizeof kIcosaFaces, 0, cudaMemcpyHostToDevice, S.s));
  const Params P{bp.max_level, bp.force_split, bp.isect_cost, bp.sah_mode, bp.sort_cost};
  std::vector<Rec> recs;  // all nodes, breadth first
  DBuf<uint32_t> pool;
  size_t pool_used = 0;
  uint32_t depth = 0;
  float box_lo[3] = {0, 0, 0}, box_hi[3] = {0, 0, 0};
  {
    DBuf<float> d_g(S, gv.size()), d_k(S, kiso.size());
    DBuf<uint32_t> d_ids(S, ids.size());
    S.check(cudaMemcpyAsync(d_g.p, gv.data(), gv.size() * 4, cudaMemcpyHostToDevice, S.s));
    S.check(cudaMemcpyAsync(d_k.p, kiso.data(), kiso.size() * 4, cudaMemcpyHostToDevice, S.s));
    S.check(cudaMemcpyAsync(d_ids.p, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice, S.s));
    size_t T = (size_t)n_valid * 20;
    TriSet cur;
    cur.alloc(S, T);
    k_proxy<<<grid_for(T, 256), 256, 0, S.s>>>(d_g.p, d_k.p, d_ids.p, n_valid, cur.v.p, cur.lo.p, cur.hi.p,
                                               cur.gid.p, cur.node.p, cur.cap);
    S.check(cudaGetLastError());
    DBuf<uint32_t> d_box(S, 6);
    const uint32_t box_init[6] = {0xFFFFFFFFu, 0, 0xFFFFFFFFu, 0, 0xFFFFFFFFu, 0};
    S.check(cudaMemcpyAsync(d_box.p, box_init, sizeof box_init, cudaMemcpyHostToDevice, S.s));
    k_scene_box<<<1024, 256, 0, S.s>>>(cur.v.p, cur.cap, T, d_box.p);
    DBuf<float> nlo(S, 3), nhi(S, 3);
    k_box_decode<<<1, 32, 0, S.s>>>(d_box.p, nlo.p, nhi.p);
    S.check(cudaMemcpyAsync(box_lo, nlo.p, 12, cudaMemcpyDeviceToHost, S.s));
    S.check(cudaMemcpyAsync(box_hi, nhi.p, 12, cudaMemcpyDeviceToHost, S.s));
    DBuf<uint32_t> tb(S, 2);
    const uint32_t tb0[2] = {0, (uint32_t)T};
    S.check(cudaMemcpyAsync(tb.p, tb0, 8, cudaMemcpyHostToDevice, S.s));
    S.check(cudaStreamSynchronize(S.s));
    uint32_t N = 1;
    if (T > 0xFFFFFFF0ull) {  // leave through the normal exit so every buffer is freed first
      err = "more than 2^32 proxy triangles";
      limit_hit = true;
      N = 0;
    }
    auto t1 = clk::now();
    if (stats) stats->proxy_s = std::chrono::duration<double>(t1 - t0).count();
    if (stats) stats->n_triangles = T;
    if (stats) stats->n_valid = n_valid;

    uint32_t base = 0;  // global BFS index of the level's first node
    for (int level = 0; N > 0 && S.err == cudaSuccess; ++level) {
#ifdef KDGR_BUILD_TRACE  // compile-time diagnostic: per-level wall time and sizes on stderr
      const auto lt0 = clk::now();
      struct LevelTrace {
        std::chrono::steady_clock::time_point t0;
        int level;
        const uint32_t* n;
        const size_t* t;
        ~LevelTrace() {
          fprintf(stderr, "[kdbuild_gpu] level %d: %u nodes, %zu triangles, %.2f ms\n", level, *n, *t,
                  std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
        }
      };
      const uint32_t n_in = N;
      const size_t t_in = T;
      LevelTrace trace_guard{lt0, level, &n_in, &t_in};
#endif
      depth = (uint32_t)level;
      int nb = 1;
      while ((1u << nb) < N) ++nb;
      // 1. runs of (node, ID)
      DBuf<uint32_t> flag(S, T + 1), ridx(S, T + 1);
      k_run_heads<<<grid_for(T + 1, 256), 256, 0, S.s>>>(cur.gid.p, cur.node.p, T, flag.p);
      exclusive_sum(S, flag.p, ridx.p, T + 1);
      const uint32_t R = read_one(S, ridx.p + T);
      DBuf<uint32_t> run_start(S, R + 1), run_node(S, R + 1), G(S, N + 1), rb(S, N + 1);
      k_run_scatter<<<grid_for(T, 256), 256, 0, S.s>>>(flag.p, ridx.p, cur.node.p, T, run_start.p, run_node.p);
      k_node_runs<<<grid_for((size_t)N + 1, 128), 128, 0, S.s>>>(tb.p, ridx.p, N, rb.p, G.p);
      flag.release();
      ridx.release();
      // 2. node constants, eligible-node compaction
      DBuf<NodeConst> nc(S, N);
      DBuf<uint32_t> eT(S, N + 1), eG(S, N + 1), ctb(S, N + 1), grb(S, N + 1);
      eT.zero();
      eG.zero();
      k_node_setup<<<grid_for(N, 128), 128, 0, S.s>>>(tb.p, G.p, nlo.p, nhi.p, N, level, P, nc.p, eT.p, eG.p);
      exclusive_sum(S, eT.p, ctb.p, N + 1);
      exclusive_sum(S, eG.p, grb.p, N + 1);
      const size_t eTT = read_one(S, ctb.p + N), eGT = read_one(S, grb.p + N);
      DBuf<Decision> dec(S, N);
      DBuf<uint32_t> is_split(S, N + 1);
      if (eTT > 0) {
        // 3. keys, sorts, scores
        DBuf<unsigned long long> ccnt(S, 3 * (size_t)R + 1), coff(S, 3 * (size_t)R + 1);
        ccnt.zero();
        k_run_cand_count<<<grid_for(R, 128), 128, 0, S.s>>>(run_start.p, run_node.p, R, T, cur.lo.p, cur.hi.p,
                                                            cur.cap, nc.p, ccnt.p);
        exclusive_sum(S, ccnt.p, coff.p, 3 * (size_t)R + 1);
        ccnt.release();
        const size_t nc_keys = read_one(S, coff.p + 3 * (size_t)R);
        DBuf<uint64_t> kc(S, nc_keys), kc_alt(S, nc_keys);
        k_run_cand_write<<<grid_for(R, 128), 128, 0, S.s>>>(run_start.p, run_node.p, R, T, cur.lo.p, cur.hi.p,
                                                            cur.cap, nc.p, coff.p, nb, kc.p);
        DBuf<uint64_t> kmin(S, 3 * eGT), kmax(S, 3 * eGT), kpl(S, 3 * eGT), alt(S, 3 * eGT);
        DBuf<uint32_t> pl_cnt(S, 3 * (size_t)N + 1), plb(S, 3 * (size_t)N + 1);
        DBuf<unsigned long long> pl_fill(S, 1);
        pl_cnt.zero();
        pl_fill.zero();
        k_run_bounds<<<grid_for(R, 128), 128, 0, S.s>>>(run_start.p, run_node.p, R, T, cur.lo.p, cur.hi.p, cur.cap,
                                                        nc.p, rb.p, grb.p, eGT, nb, kmin.p, kmax.p, kpl.p, pl_cnt.p,
                                                        pl_fill.p, N);
        exclusive_sum(S, pl_cnt.p, plb.p, 3 * (size_t)N + 1);
        const size_t n_pl = read_one(S, pl_fill.p);
        const int end_bit = 32 + nb + 2;
        sort_keys(S, kc, kc_alt, nc_keys, end_bit);
        kc_alt.release();
        sort_keys(S, kmin, alt, 3 * eGT, end_bit);
        sort_keys(S, kmax, alt, 3 * eGT, end_bit);
        sort_keys(S, kpl, alt, n_pl, end_bit);
        alt.release();
        DBuf<double> cost(S, nc_keys);
        DBuf<uint8_t> side(S, nc_keys);
        DBuf<unsigned long long> best_bits(S, 3 * (size_t)N), best_idx(S, 3 * (size_t)N);
        best_bits.fill_ff();
        best_idx.fill_ff();
        k_eval<<<grid_for(nc_keys, 256), 256, 0, S.s>>>(kc.p, nc_keys, coff.p, rb.p, R, nb, kmin.p, kmax.p, kpl.p,
                                                        eGT, grb.p, plb.p, pl_cnt.p, nc.p, N, P, cost.p, side.p,
                                                        best_bits.p);
        k_argmin<<<grid_for(nc_keys, 256), 256, 0, S.s>>>(kc.p, cost.p, nc_keys, nb, N, best_bits.p, best_idx.p);
        k_choose<<<grid_for(N, 128), 128, 0, S.s>>>(nc.p, N, best_bits.p, best_idx.p, kc.p, side.p, dec.p,
                                                    is_split.p);
      } else {
        std::vector<Decision> leafs(N, Decision{-1, 0.f, 0});
        S.check(cudaMemcpyAsync(dec.p, leafs.data(), N * sizeof(Decision), cudaMemcpyHostToDevice, S.s));
        is_split.zero();
      }
      S.check(cudaGetLastError());
      // 4. leaves: their run IDs into the pool
      DBuf<uint32_t> lsz(S, N + 1), loff(S, N + 1);
      lsz.zero();
      k_leaf_sizes<<<grid_for(N, 128), 128, 0, S.s>>>(is_split.p, G.p, N, lsz.p);
      exclusive_sum(S, lsz.p, loff.p, N + 1);
      const size_t leaf_total = read_one(S, loff.p + N);
      if (pool_used + leaf_total > pool.n) {
        DBuf<uint32_t> bigger(S, std::max(pool.n * 2, pool_used + leaf_total + 1024));
        if (pool_used)
          S.check(cudaMemcpyAsync(bigger.p, pool.p, pool_used * 4, cudaMemcpyDeviceToDevice, S.s));
        pool = std::move(bigger);
      }
      k_leaf_ids<<<grid_for(R, 256), 256, 0, S.s>>>(run_start.p, run_node.p, R, cur.gid.p, is_split.p, rb.p, loff.p,
                                                    pool.p + pool_used);
      // 5. partition into the next level
      DBuf<uint32_t> ns(S, N + 1);
      S.check(cudaMemsetAsync(is_split.p + N, 0, 4, S.s));
      exclusive_sum(S, is_split.p, ns.p, N + 1);
      const uint32_t n_split = read_one(S, ns.p + N);
      // host records of this level
      {
        std::vector<Decision> hd(N);
        std::vector<uint32_t> hns(N), hG(N), hloff(N);
        S.check(cudaMemcpyAsync(hd.data(), dec.p, N * sizeof(Decision), cudaMemcpyDeviceToHost, S.s));
        S.check(cudaMemcpyAsync(hns.data(), ns.p, N * 4, cudaMemcpyDeviceToHost, S.s));
        S.check(cudaMemcpyAsync(hG.data(), G.p, N * 4, cudaMemcpyDeviceToHost, S.s));
        S.check(cudaMemcpyAsync(hloff.data(), loff.p, N * 4, cudaMemcpyDeviceToHost, S.s));
        S.check(cudaStreamSynchronize(S.s));
        for (uint32_t i = 0; i < N; ++i) {
          Rec r;
          r.axis = hd[i].axis;
          r.split = hd[i].split;
          r.first_child = base + N + 2 * hns[i];
          r.leaf_off = (uint32_t)(pool_used + hloff[i]);
          r.leaf_cnt = hd[i].axis < 0 ? hG[i] : 0;
          recs.push_back(r);
        }
      }
      pool_used += leaf_total;
      if (n_split == 0) break;
      const uint32_t N2 = 2 * n_split;
      DBuf<uint32_t> fl(S, T + 1), fr(S, T + 1), sl(S, T + 1), sr(S, T + 1);
      k_part_flags<<<grid_for(T + 1, 256), 256, 0, S.s>>>(cur.lo.p, cur.hi.p, cur.cap, T, cur.node.p, dec.p, fl.p,
                                                          fr.p);
      exclusive_sum(S, fl.p, sl.p, T + 1);
      exclusive_sum(S, fr.p, sr.p, T + 1);
      fl.release();
      fr.release();
      DBuf<uint32_t> cc(S, N2 + 1), ntb(S, N2 + 1);
      cc.zero();
      k_child_counts<<<grid_for(N, 128), 128, 0, S.s>>>(tb.p, sl.p, sr.p, is_split.p, ns.p, N, cc.p);
      exclusive_sum(S, cc.p, ntb.p, N2 + 1);
      const size_t T2 = read_one(S, ntb.p + N2);
      if (T2 > 0xFFFFFFF0ull) {
        err = "more than 2^32 triangle references in one level";
        limit_hit = true;
        break;
      }
      TriSet nxt;
      nxt.alloc(S, std::max<size_t>(T2, 1));
      k_part_scatter<<<grid_for(T, 256), 256, 0, S.s>>>(cur.v.p, cur.lo.p, cur.hi.p, cur.gid.p, cur.node.p, cur.cap,
                                                        T, tb.p, dec.p, ns.p, sl.p, sr.p, ntb.p, nxt.v.p, nxt.lo.p,
                                                        nxt.hi.p, nxt.gid.p, nxt.node.p, nxt.cap);
      DBuf<float> clo(S, 3 * (size_t)N2), chi(S, 3 * (size_t)N2);
      k_child_boxes<<<grid_for(N, 128), 128, 0, S.s>>>(nlo.p, nhi.p, dec.p, ns.p, N, clo.p, chi.p);
      S.check(cudaGetLastError());
      S.check(cudaStreamSynchronize(S.s));
      cur = std::move(nxt);
      nlo = std::move(clo);
      nhi = std::move(chi);
      tb = std::move(ntb);
      base += N;
      N = N2;
      T = T2;
    }
  }
  std::vector<uint32_t> hpool(pool_used);
  if (pool_used)
    S.check(cudaMemcpyAsync(hpool.data(), pool.p, pool_used * 4, cudaMemcpyDeviceToHost, S.s));
  pool.release();
  S.check(cudaStreamSynchronize(S.s));
  const cudaError_t e = S.err;
  cudaStreamDestroy(S.s);
  if (S.pool) cudaMemPoolDestroy(S.pool);
  if (limit_hit && e == cudaSuccess) return KDGR_ERR_LIMIT;
  if (e != cudaSuccess) {
    if (err.empty()) err = std::string("CUDA error in the device build: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? KDGR_ERR_OUT_OF_MEMORY : KDGR_ERR_CUDA;
  }
  auto t2 = clk::now();
  // number as the reference allocates: child pairs in depth-first,
  // left-first order; leaf ID lists appended in the same order
  out.nodes.assign(2, 0);
  out.offsets.clear();
  out.offsets.reserve(pool_used);
  uint32_t n_leaves = 0, max_leaf = 0;
  struct Item {
    uint32_t rec, slot;
  };
  std::vector<Item> st{{0, 0}};
  while (!st.empty()) {
    const Item it = st.back();
    st.pop_back();
    const Rec& r = recs[it.rec];
    if (r.axis < 0) {
      out.nodes[2 * it.slot] = (r.leaf_cnt << 3) | 3u;
      out.nodes[2 * it.slot + 1] = (uint32_t)out.offsets.size();
      out.offsets.insert(out.offsets.end(), hpool.begin() + r.leaf_off, hpool.begin() + r.leaf_off + r.leaf_cnt);
      ++n_leaves;
      max_leaf = std::max(max_leaf, r.leaf_cnt);
    } else {
      const uint32_t c = (uint32_t)(out.nodes.size() / 2);
      out.nodes.resize(out.nodes.size() + 4, 0);
      uint32_t bits;
      memcpy(&bits, &r.split, 4);
      out.nodes[2 * it.slot] = (c << 3) | (uint32_t)r.axis;
      out.nodes[2 * it.slot + 1] = bits;
      st.push_back({r.first_child + 1, c + 1});
      st.push_back({r.first_child, c});
    }
  }
  out.aabb[0] = box_lo[0];
  out.aabb[1] = box_lo[1];
  out.aabb[2] = box_lo[2];
  out.aabb[3] = box_hi[0];
  out.aabb[4] = box_hi[1];
  out.aabb[5] = box_hi[2];
  out.depth = depth;
  out.n_leaves = n_leaves;
  out.max_leaf = max_leaf;
  auto t3 = clk::now();
  if (stats) {
    stats->build_s = std::chrono::duration<double>(t2 - t0).count() - stats->proxy_s;
    stats->serialize_s = std::chrono::duration<double>(t3 - t2).count();
  }
  return KDGR_OK;
}

}  // namespace kdgr
