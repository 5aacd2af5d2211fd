// kdgr_debug.cpp -- headless form of the reference's HIT_AND_NODE_COUNT_DEBUG
// report (cudaRenderer.cu:3173-3400): per-pixel traversal counters reduced to
// averages, maxima and totals, node/leaf visit histograms, heatmap images and
// CSV matrices, and the raw per-pixel count files.  Host code only: it reads
// kdgr_ray_trace records that kdgr_render_trace copied back (or the CPU
// oracle wrote), so it runs without a GPU.
//
// Output files, by the reference's names, all in pixel order y*W + x (the
// kernel's row order, not the flipped framebuffer order):
//   renderStats.txt                    averages, maxima, totals (:3312-3337)
//   render_stats.csv                   node and leaf visit histograms (:3046-3066)
//   heatmap_<counter>.png / .csv       six counters (:3271-3306)
//   isectCnt_kd.bin, blendCnt_kd.bin   u32 per pixel (:3285-3303)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "kdgr.h"
#include "kdgr_internal.h"

namespace kdgr {
namespace {

// ------------------------------------------------------------ PNG writer
// 8-bit RGB, zlib stream of stored (uncompressed) deflate blocks: enough for
// a debug image and needs no compression library.
struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[i] = c;
    }
  }
};

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
  static const CrcTable table;  // thread-safe one-time initialisation
  for (size_t i = 0; i < n; ++i) crc = table.t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
  return crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void put_chunk(std::vector<uint8_t>& out, const char type[4], const std::vector<uint8_t>& data) {
  put_be32(out, (uint32_t)data.size());
  const size_t at = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  const uint32_t crc = crc32_update(0xFFFFFFFFu, out.data() + at, 4 + data.size()) ^ 0xFFFFFFFFu;
  put_be32(out, crc);
}

bool write_png_rgb(const std::string& path, const uint8_t* rgb, int W, int H) {
  std::vector<uint8_t> raw;
  raw.reserve((size_t)H * (3 * (size_t)W + 1));
  for (int y = 0; y < H; ++y) {
    raw.push_back(0);  // filter: none
    raw.insert(raw.end(), rgb + (size_t)y * W * 3, rgb + (size_t)(y + 1) * W * 3);
  }
  std::vector<uint8_t> z = {0x78, 0x01};
  uint32_t a = 1, b = 0;  // Adler-32
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  size_t pos = 0;
  do {
    const size_t n = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + n == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)(n & 0xFF));
    z.push_back((uint8_t)(n >> 8));
    z.push_back((uint8_t)(~n & 0xFF));
    z.push_back((uint8_t)((~n >> 8) & 0xFF));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
    pos += n;
  } while (pos < raw.size());
  put_be32(z, (b << 16) | a);

  std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  std::vector<uint8_t> ihdr;
  put_be32(ihdr, (uint32_t)W);
  put_be32(ihdr, (uint32_t)H);
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit, truecolour, deflate, no filter set, no interlace
  put_chunk(png, "IHDR", ihdr);
  put_chunk(png, "IDAT", z);
  put_chunk(png, "IEND", {});
  FILE* fp = fopen(path.c_str(), "wb");
  if (!fp) return false;
  const bool ok = fwrite(png.data(), 1, png.size(), fp) == png.size();
  return (fclose(fp) == 0) && ok;
}

// ------------------------------------------------------------ heatmap colour
// The Turbo colormap's published polynomial approximation (A. Mikhailov,
// "Turbo, An Improved Rainbow Colormap for Visualization", Google AI blog,
// 2019; polynomial fit by R. Du), evaluated in FP32 in the order the
// reference's host helper uses (cudaRenderer.cu:2985-3007), so the bytes of
// the image match.  Values <= 0 are black; others are scaled by 1/max.
inline float clamp01(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }

inline uint8_t to_byte(float v) {
  float s = v * 255.0f + 0.5f;
  s = s < 0.f ? 0.f : (s > 255.f ? 255.f : s);
  return (uint8_t)s;
}

void turbo(float x, uint8_t out[3]) {
  static const float c4[3][4] = {{0.13572138f, 4.61539260f, -42.66032258f, 132.13108234f},
                                 {0.09140261f, 2.19418839f, 4.84296658f, -14.18503333f},
                                 {0.10667330f, 12.64194608f, -60.58204836f, 110.36276771f}};
  static const float c2[3][2] = {{-152.94239396f, 59.28637943f}, {4.27729857f, 2.82956604f},
                                 {-89.90310912f, 27.34824973f}};
  x = clamp01(x);
  const float p[4] = {1.0f, x, x * x, x * x * x};
  const float q[2] = {p[2] * p[2], p[3] * p[2]};
  for (int c = 0; c < 3; ++c) {
    const float s4 = c4[c][0] * p[0] + c4[c][1] * p[1] + c4[c][2] * p[2] + c4[c][3] * p[3];
    const float s2 = c2[c][0] * q[0] + c2[c][1] * q[1];
    out[c] = to_byte(s4 + s2);
  }
}

bool write_heatmap(const std::string& path, const std::vector<float>& v, int W, int H, float max_val) {
  std::vector<uint8_t> img((size_t)W * H * 3, 0);
  for (size_t i = 0; i < v.size(); ++i) {
    if (v[i] <= 0.0f) continue;
    turbo(clamp01((v[i] - 0.0f) / (max_val - 0.0f)), &img[3 * i]);
  }
  return write_png_rgb(path, img.data(), W, H);
}

bool write_matrix_csv(const std::string& path, const std::vector<float>& v, int W, int H) {
  FILE* fp = fopen(path.c_str(), "w");
  if (!fp) return false;
  std::string line;
  for (int y = 0; y < H; ++y) {
    line.clear();
    for (int x = 0; x < W; ++x) {
      line += std::to_string((int)v[(size_t)y * W + x]);
      line += x + 1 < W ? ',' : '\n';
    }
    fputs(line.c_str(), fp);
  }
  return fclose(fp) == 0;
}

bool write_u32(const std::string& path, const std::vector<uint32_t>& v) {
  FILE* fp = fopen(path.c_str(), "wb");
  if (!fp) return false;
  const bool ok = fwrite(v.data(), 4, v.size(), fp) == v.size();
  return (fclose(fp) == 0) && ok;
}

void print_stat(FILE* fp, const char* name, int tabs, float sum, uint32_t n, bool is_avg) {
  fputs(name, fp);
  for (int i = 0; i < tabs; ++i) fputc('\t', fp);
  if (is_avg && n == 0)
    fputs(": nan\n", fp);  // no pixel blended anything; printf's NaN spelling is platform specific
  else
    fprintf(fp, ": %f\n", (double)(is_avg ? sum / (float)n : sum));
}

}  // namespace
}  // namespace kdgr

using namespace kdgr;

extern "C" int kdgr_debug_report(const kdgr_ray_trace* trace, int width, int height, const char* out_dir,
                                 float heat_max, kdgr_debug_stats* out) {
  if (!trace || width <= 0 || height <= 0 || !(heat_max > 0.f)) {
    set_error("kdgr_debug_report: null trace, empty image or heat_max <= 0");
    return KDGR_ERR_INVALID_ARG;
  }
  const size_t n = (size_t)width * height;
  // counters in the reference's order: node visits, leaf visits,
  // intersection tests, hits found, blend ops, max sort size
  auto counter = [&](size_t i, int k) -> uint32_t {
    const kdgr_ray_trace& t = trace[i];
    switch (k) {
      case 0: return t.n_inner;
      case 1: return t.n_leaf;
      case 2: return t.n_cand;
      case 3: return t.n_found;
      case 4: return t.n_blend;
      default: return t.max_sort;
    }
  };
  kdgr_debug_stats st;
  memset(&st, 0, sizeof st);
  float sum[6] = {0, 0, 0, 0, 0, 0};
  std::vector<int> hist_node(1024, 0), hist_leaf(1024, 0);
  auto add_hist = [](std::vector<int>& h, uint32_t v) {
    if (v >= h.size()) h.resize((size_t)v + 1, 0);
    ++h[v];
  };
  for (size_t i = 0; i < n; ++i) {
    for (int k = 0; k < 6; ++k) {
      // the reference keeps the counters as floats (float3 buffers) and casts back to int
      const int v = (int)(float)counter(i, k);
      if (v > st.max[k]) st.max[k] = v;
    }
    if (trace[i].n_blend != 0) {  // averages over pixels that blended something (:3245)
      for (int k = 0; k < 6; ++k) sum[k] += (float)counter(i, k);
      ++st.n_pixels;
      add_hist(hist_node, trace[i].n_inner);
      add_hist(hist_leaf, trace[i].n_leaf);
    }
  }
  for (int k = 0; k < 6; ++k) {
    st.total[k] = sum[k];
    st.avg[k] = st.n_pixels ? sum[k] / (float)st.n_pixels : NAN;
  }
  if (out) *out = st;
  if (!out_dir) return KDGR_OK;

  const std::string dir = std::string(out_dir) + "/";
  static const char* kNames[6] = {"node_visits", "leaf_visits", "intersection", "hits_found", "blend_ops",
                                  "max_sort_size"};
  bool ok = true;
  std::vector<float> buf(n);
  for (int k = 0; k < 6; ++k) {
    for (size_t i = 0; i < n; ++i) buf[i] = (float)counter(i, k);
    ok = ok && write_heatmap(dir + "heatmap_" + kNames[k] + ".png", buf, width, height, heat_max);
    ok = ok && write_matrix_csv(dir + "heatmap_" + kNames[k] + ".csv", buf, width, height);
  }
  std::vector<uint32_t> cnt(n);
  for (size_t i = 0; i < n; ++i) cnt[i] = trace[i].n_found;
  ok = ok && write_u32(dir + "isectCnt_kd.bin", cnt);
  // the reference writes hits_found into this file as well (:3296); blend
  // operations are what its name and comment announce, and what is written here
  for (size_t i = 0; i < n; ++i) cnt[i] = trace[i].n_blend;
  ok = ok && write_u32(dir + "blendCnt_kd.bin", cnt);

  if (FILE* fp = fopen((dir + "render_stats.csv").c_str(), "w")) {
    fputs("Value,Node_Visits,Leaf_Visits\n", fp);
    const size_t range = std::max(hist_node.size(), hist_leaf.size());
    for (size_t i = 0; i < range; ++i) {
      const int v1 = i < hist_node.size() ? hist_node[i] : 0, v2 = i < hist_leaf.size() ? hist_leaf[i] : 0;
      if (v1 > 0 || v2 > 0) fprintf(fp, "%zu,%d,%d\n", i, v1, v2);
    }
    ok = (fclose(fp) == 0) && ok;
  } else {
    ok = false;
  }

  if (FILE* fp = fopen((dir + "renderStats.txt").c_str(), "w")) {
    static const char* kStat[6] = {"node_visits", "leaf_visits", "intersection_tests", "hits_found",
                                   "blend_ops", "max_sort_size"};
    static const int kTabs[6] = {2, 2, 1, 2, 2, 1};  // column alignment of the reference's file
    const char* rule = "===========================================\n";
    fprintf(fp, "\n%s", rule);
    for (int k = 0; k < 6; ++k)
      print_stat(fp, ("avg_" + std::string(kStat[k])).c_str(), kTabs[k], sum[k], st.n_pixels, true);
    fputs(rule, fp);
    for (int k = 0; k < 6; ++k) {
      fprintf(fp, "max_%s", kStat[k]);
      for (int t = 0; t < kTabs[k]; ++t) fputc('\t', fp);
      fprintf(fp, ": %d\n", st.max[k]);
    }
    fputs(rule, fp);
    for (int k = 0; k < 6; ++k)
      print_stat(fp, ("tot_" + std::string(kStat[k])).c_str(), kTabs[k], sum[k], st.n_pixels, false);
    fputs(rule, fp);
    ok = (fclose(fp) == 0) && ok;
  } else {
    ok = false;
  }
  if (!ok) {
    set_error("kdgr_debug_report: cannot write the report files under " + std::string(out_dir));
    return KDGR_ERR_IO;
  }
  return KDGR_OK;
}
