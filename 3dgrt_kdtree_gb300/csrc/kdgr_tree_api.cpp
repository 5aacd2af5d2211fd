// kdgr_tree_api.cpp -- C ABI for tree building, `.kdt` I/O and validation.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kdgr.h"
#include "kdgr_internal.h"

namespace kdgr {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

int write_kdt(const HostTree& t, const char* path, std::string& err) {
  FILE* fp = fopen(path, "wb");
  if (!fp) {
    err = std::string("cannot open ") + path + " for writing";
    return KDGR_ERR_IO;
  }
  // Kd-treeConverter.cpp:320-342: f32 version 0.1, f32 aabb[6], i32 n_nodes,
  // nodes (8 B each), i32 n_offsets, u32 offsets.
  const float version = 0.1f;
  const int32_t nn = (int32_t)(t.nodes.size() / 2);
  const int32_t no = (int32_t)t.offsets.size();
  bool ok = fwrite(&version, 4, 1, fp) == 1 && fwrite(t.aabb, 4, 6, fp) == 6 && fwrite(&nn, 4, 1, fp) == 1 &&
            fwrite(t.nodes.data(), 8, nn, fp) == (size_t)nn && fwrite(&no, 4, 1, fp) == 1 &&
            fwrite(t.offsets.data(), 4, no, fp) == (size_t)no;
  ok = (fclose(fp) == 0) && ok;
  if (!ok) {
    err = std::string("short write to ") + path;
    return KDGR_ERR_IO;
  }
  return KDGR_OK;
}

int read_kdt(const char* path, HostTree& t, std::string& err) {
  FILE* fp = fopen(path, "rb");
  if (!fp) {
    err = std::string("cannot open ") + path;
    return KDGR_ERR_IO;
  }
  float version = 0.f;
  int32_t nn = -1, no = -1;
  int rc = KDGR_OK;
  if (fread(&version, 4, 1, fp) != 1 || fread(t.aabb, 4, 6, fp) != 6 || fread(&nn, 4, 1, fp) != 1) {
    err = "truncated .kdt header";
    rc = KDGR_ERR_FORMAT;
  } else if (version != 0.1f) {
    err = "unsupported .kdt version (expected 0.1)";
    rc = KDGR_ERR_FORMAT;
  } else if (nn <= 0) {
    err = "bad .kdt node count";
    rc = KDGR_ERR_FORMAT;
  } else {
    t.nodes.resize((size_t)nn * 2);
    if (fread(t.nodes.data(), 8, nn, fp) != (size_t)nn || fread(&no, 4, 1, fp) != 1 || no < 0) {
      err = "truncated .kdt node array";
      rc = KDGR_ERR_FORMAT;
    } else {
      t.offsets.resize((size_t)no);
      if (no > 0 && fread(t.offsets.data(), 4, no, fp) != (size_t)no) {
        err = "truncated .kdt offset array";
        rc = KDGR_ERR_FORMAT;
      }
    }
  }
  fclose(fp);
  return rc;
}

// ASCII form of dump_kd_tree_for_composite_object / read_kd_tree_from_file
// (Kd-treeConverter.cpp:345-380, 496-541): "n<count>", one line per node
// ("<X|Y|Z>|<split %f> <child><><child+1>" or "L cnt:<n> off:<offset>"),
// "o<count>", one Gaussian ID per line.  No scene box; splits carry six
// decimals, so a round trip through this format moves split planes.
int write_kdt_ascii(const HostTree& t, const char* path, std::string& err) {
  FILE* fp = fopen(path, "w");
  if (!fp) {
    err = std::string("cannot open ") + path + " for writing";
    return KDGR_ERR_IO;
  }
  const size_t nn = t.nodes.size() / 2;
  bool ok = fprintf(fp, "n%d\n", (int)nn) > 0;
  static const char kAxis[3] = {'X', 'Y', 'Z'};
  for (size_t i = 0; i < nn && ok; ++i) {
    const uint32_t x = t.nodes[2 * i], y = t.nodes[2 * i + 1];
    if ((x & 7u) == 3u) {
      ok = fprintf(fp, "L cnt:%d off:%d\n", (int)(x >> 3), (int)y) > 0;
    } else {
      float split;
      memcpy(&split, &y, 4);
      const int child = (int)(x >> 3);
      ok = fprintf(fp, "%c|%f %d<>%d\n", kAxis[x & 3u], (double)split, child, child + 1) > 0;
    }
  }
  ok = ok && fprintf(fp, "o%d\n", (int)t.offsets.size()) > 0;
  for (size_t i = 0; i < t.offsets.size() && ok; ++i) ok = fprintf(fp, "%d\n", (int)t.offsets[i]) > 0;
  ok = (fclose(fp) == 0) && ok;
  if (!ok) {
    err = std::string("short write to ") + path;
    return KDGR_ERR_IO;
  }
  return KDGR_OK;
}

int read_kdt_ascii(const char* path, HostTree& t, std::string& err) {
  FILE* fp = fopen(path, "r");
  if (!fp) {
    err = std::string("cannot open ") + path;
    return KDGR_ERR_IO;
  }
  char line[1024];
  auto next = [&]() { return fgets(line, sizeof line, fp) != nullptr; };
  int rc = KDGR_OK;
  int nn = -1, no = -1;
  memset(t.aabb, 0, sizeof t.aabb);
  if (!next() || line[0] != 'n' || sscanf(line + 1, "%d", &nn) != 1 || nn <= 0) {
    err = "bad ASCII .kdt header (expected n<node count>)";
    rc = KDGR_ERR_FORMAT;
  }
  if (rc == KDGR_OK) t.nodes.resize(2 * (size_t)nn);
  for (int i = 0; rc == KDGR_OK && i < nn; ++i) {
    int a = 0, b = 0;
    float split = 0.f;
    if (!next()) {
      err = "truncated ASCII .kdt node list";
      rc = KDGR_ERR_FORMAT;
    } else if (line[0] == 'L') {
      if (sscanf(line + 2, "cnt:%d off:%d", &a, &b) != 2 || a < 0 || b < 0) {
        err = "bad leaf line " + std::to_string(i);
        rc = KDGR_ERR_FORMAT;
      } else {
        t.nodes[2 * i] = ((uint32_t)a << 3) | 3u;
        t.nodes[2 * i + 1] = (uint32_t)b;
      }
    } else if (line[0] >= 'X' && line[0] <= 'Z' && line[1] == '|' &&
               sscanf(line + 2, "%f %d", &split, &a) == 2 && a > 0) {
      uint32_t bits;
      memcpy(&bits, &split, 4);
      t.nodes[2 * i] = ((uint32_t)a << 3) | (uint32_t)(line[0] - 'X');
      t.nodes[2 * i + 1] = bits;
    } else {
      err = "bad node line " + std::to_string(i);
      rc = KDGR_ERR_FORMAT;
    }
  }
  if (rc == KDGR_OK && (!next() || line[0] != 'o' || sscanf(line + 1, "%d", &no) != 1 || no < 0)) {
    err = "bad ASCII .kdt offset header (expected o<count>)";
    rc = KDGR_ERR_FORMAT;
  }
  if (rc == KDGR_OK) t.offsets.resize((size_t)no);
  for (int i = 0; rc == KDGR_OK && i < no; ++i) {
    long long id = -1;
    if (!next() || sscanf(line, "%lld", &id) != 1 || id < 0 || id > 0xFFFFFFFFll) {
      err = "bad Gaussian ID line " + std::to_string(i);
      rc = KDGR_ERR_FORMAT;
    } else {
      t.offsets[i] = (uint32_t)id;
    }
  }
  fclose(fp);
  return rc;
}

int validate_tree(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                  uint32_t n_gaussians, std::string& err, uint32_t* depth_out) {
  if (n_nodes == 0) {
    err = "tree has no nodes";
    return KDGR_ERR_FORMAT;
  }
  std::vector<uint8_t> seen(n_nodes, 0);
  struct It {
    uint32_t id, depth;
  };
  std::vector<It> st{{0, 0}};
  uint32_t maxd = 0;
  while (!st.empty()) {
    It it = st.back();
    st.pop_back();
    if (seen[it.id]) {
      err = "node " + std::to_string(it.id) + " reachable twice";
      return KDGR_ERR_FORMAT;
    }
    seen[it.id] = 1;
    if (it.depth > maxd) maxd = it.depth;
    const uint32_t x = nodes[2 * it.id], y = nodes[2 * it.id + 1];
    if ((x & 7u) == 3u) {
      const uint64_t cnt = x >> 3, off = y;
      if (off + cnt > n_offsets) {
        err = "leaf " + std::to_string(it.id) + " ID range outside the offset array";
        return KDGR_ERR_FORMAT;
      }
      for (uint64_t i = off; i < off + cnt; ++i)
        if (offsets[i] >= n_gaussians) {
          err = "leaf " + std::to_string(it.id) + " references Gaussian " + std::to_string(offsets[i]) +
                " >= " + std::to_string(n_gaussians);
          return KDGR_ERR_FORMAT;
        }
    } else {
      if ((x & 4u) != 0u || (x & 3u) == 3u) {
        err = "inner node " + std::to_string(it.id) + " has a bad axis field";
        return KDGR_ERR_FORMAT;
      }
      const uint64_t c = x >> 3;
      if (c + 1 >= n_nodes || c == 0) {
        err = "inner node " + std::to_string(it.id) + " child index out of range";
        return KDGR_ERR_FORMAT;
      }
      st.push_back({(uint32_t)c + 1, it.depth + 1});
      st.push_back({(uint32_t)c, it.depth + 1});
    }
  }
  if (depth_out) *depth_out = maxd;
  return KDGR_OK;
}

static int fill_out(HostTree& t, uint32_t n_gauss, kdgr_tree* out) {
  memset(out, 0, sizeof(*out));
  out->n_nodes = (uint32_t)(t.nodes.size() / 2);
  out->n_offsets = (uint32_t)t.offsets.size();
  out->nodes = (uint32_t*)malloc(sizeof(uint32_t) * (t.nodes.size() + 1));
  out->offsets = (uint32_t*)malloc(sizeof(uint32_t) * (t.offsets.size() + 1));
  out->valid = (uint8_t*)malloc(t.valid.size() + 1);
  if (!out->nodes || !out->offsets || !out->valid) {
    free(out->nodes);
    free(out->offsets);
    free(out->valid);
    memset(out, 0, sizeof(*out));
    set_error("host allocation failed for tree arrays");
    return KDGR_ERR_OUT_OF_MEMORY;
  }
  memcpy(out->nodes, t.nodes.data(), sizeof(uint32_t) * t.nodes.size());
  memcpy(out->offsets, t.offsets.data(), sizeof(uint32_t) * t.offsets.size());
  if (!t.valid.empty()) memcpy(out->valid, t.valid.data(), t.valid.size());
  memcpy(out->aabb, t.aabb, sizeof(out->aabb));
  out->depth = t.depth;
  out->n_leaves = t.n_leaves;
  out->max_leaf = t.max_leaf;
  out->n_gaussians = n_gauss;
  return KDGR_OK;
}

}  // namespace kdgr

using namespace kdgr;

extern "C" {

const char* kdgr_last_error(void) { return kdgr::last_error(); }

void kdgr_build_params_default(kdgr_build_params* p) {
  if (!p) return;
  p->max_level = 24;
  p->force_split = 16;
  p->isect_cost = 5.0f;
  p->sah_mode = 1;
  p->sort_cost = 0.5f;
  p->threads = 0;
}

int kdgr_build_tree(const float* gaussians, uint32_t n_gaussians, const kdgr_build_params* params,
                    kdgr_tree* out, kdgr_build_stats* stats) {
  if (!gaussians || n_gaussians == 0 || !out) {
    set_error("kdgr_build_tree: null input or zero Gaussians");
    return KDGR_ERR_INVALID_ARG;
  }
  BuildParams bp;
  if (params) {
    bp.max_level = params->max_level;
    bp.force_split = params->force_split;
    bp.isect_cost = params->isect_cost;
    bp.sah_mode = params->sah_mode;
    bp.sort_cost = params->sort_cost;
    bp.threads = params->threads;
  }
  if (bp.sah_mode != 0 && bp.sah_mode != 1 && bp.sah_mode != 4 && bp.sah_mode != 7) {
    set_error("kdgr_build_tree: sah_mode must be 0, 1, 4 or 7");
    return KDGR_ERR_INVALID_ARG;
  }
  HostTree t;
  BuildStats bs;
  int rc;
  try {
    rc = build_tree(gaussians, n_gaussians, bp, t, &bs);
  } catch (const std::bad_alloc&) {
    set_error("kdgr_build_tree: host allocation failed");
    return KDGR_ERR_OUT_OF_MEMORY;
  }
  if (rc != KDGR_OK) return rc;
  if (bs.n_valid == 0) {
    set_error("kdgr_build_tree: every Gaussian is below the opacity cut; nothing to build");
    return KDGR_ERR_INVALID_ARG;
  }
  if (stats) {
    stats->proxy_s = bs.proxy_s;
    stats->build_s = bs.build_s + bs.serialize_s;
    stats->n_triangles = bs.n_triangles;
    stats->n_valid = bs.n_valid;
    stats->serialize_s = bs.serialize_s;
  }
  return fill_out(t, n_gaussians, out);
}

static int finish_read(HostTree& t, const char* who, kdgr_tree* out) {
  std::string err;
  uint32_t depth = 0;
  int rc = validate_tree(t.nodes.data(), (uint32_t)(t.nodes.size() / 2), t.offsets.data(),
                         (uint32_t)t.offsets.size(), 0xFFFFFFFFu, err, &depth);
  if (rc != KDGR_OK) {
    set_error(std::string(who) + ": " + err);
    return rc;
  }
  t.depth = depth;
  for (size_t i = 0; i < t.nodes.size(); i += 2)
    if ((t.nodes[i] & 7u) == 3u) {
      ++t.n_leaves;
      if ((t.nodes[i] >> 3) > t.max_leaf) t.max_leaf = t.nodes[i] >> 3;
    }
  return fill_out(t, 0, out);
}

int kdgr_build_tree_gpu(const float* gaussians, uint32_t n_gaussians, const kdgr_build_params* params,
                        kdgr_tree* out, kdgr_build_stats* stats) {
  if (!gaussians || n_gaussians == 0 || !out) {
    set_error("kdgr_build_tree_gpu: null input or zero Gaussians");
    return KDGR_ERR_INVALID_ARG;
  }
  BuildParams bp;
  if (params) {
    bp.max_level = params->max_level;
    bp.force_split = params->force_split;
    bp.isect_cost = params->isect_cost;
    bp.sah_mode = params->sah_mode;
    bp.sort_cost = params->sort_cost;
  }
  if (bp.sah_mode != 0 && bp.sah_mode != 1 && bp.sah_mode != 4 && bp.sah_mode != 7) {
    set_error("kdgr_build_tree_gpu: sah_mode must be 0, 1, 4 or 7");
    return KDGR_ERR_INVALID_ARG;
  }
  if (bp.max_level < 0 || bp.max_level > 60) {
    set_error("kdgr_build_tree_gpu: max_level must be in [0, 60]");
    return KDGR_ERR_INVALID_ARG;
  }
  HostTree t;
  BuildStats bs;
  std::string err;
  int rc;
  try {
    rc = build_tree_gpu(gaussians, n_gaussians, bp, t, &bs, err);
  } catch (const std::bad_alloc&) {
    set_error("kdgr_build_tree_gpu: host allocation failed");
    return KDGR_ERR_OUT_OF_MEMORY;
  }
  if (rc != KDGR_OK) {
    set_error("kdgr_build_tree_gpu: " + err);
    return rc;
  }
  if (stats) {
    stats->proxy_s = bs.proxy_s;
    stats->build_s = bs.build_s + bs.serialize_s;
    stats->n_triangles = bs.n_triangles;
    stats->n_valid = bs.n_valid;
    stats->serialize_s = bs.serialize_s;
  }
  return fill_out(t, n_gaussians, out);
}

int kdgr_read_kdt(const char* path, kdgr_tree* out) {
  if (!path || !out) {
    set_error("kdgr_read_kdt: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  HostTree t;
  std::string err;
  int rc = read_kdt(path, t, err);
  if (rc != KDGR_OK) {
    set_error("kdgr_read_kdt: " + err);
    return rc;
  }
  return finish_read(t, "kdgr_read_kdt", out);
}

int kdgr_read_kdt_ascii(const char* path, kdgr_tree* out) {
  if (!path || !out) {
    set_error("kdgr_read_kdt_ascii: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  HostTree t;
  std::string err;
  int rc = read_kdt_ascii(path, t, err);
  if (rc != KDGR_OK) {
    set_error("kdgr_read_kdt_ascii: " + err);
    return rc;
  }
  return finish_read(t, "kdgr_read_kdt_ascii", out);
}

int kdgr_write_kdt_ascii(const kdgr_tree* tree, const char* path) {
  if (!tree || !path || !tree->nodes) {
    set_error("kdgr_write_kdt_ascii: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  HostTree t;
  t.nodes.assign(tree->nodes, tree->nodes + 2 * (size_t)tree->n_nodes);
  t.offsets.assign(tree->offsets, tree->offsets + tree->n_offsets);
  std::string err;
  int rc = write_kdt_ascii(t, path, err);
  if (rc != KDGR_OK) set_error("kdgr_write_kdt_ascii: " + err);
  return rc;
}

int kdgr_write_kdt(const kdgr_tree* tree, const char* path) {
  if (!tree || !path || !tree->nodes) {
    set_error("kdgr_write_kdt: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  HostTree t;
  t.nodes.assign(tree->nodes, tree->nodes + 2 * (size_t)tree->n_nodes);
  t.offsets.assign(tree->offsets, tree->offsets + tree->n_offsets);
  memcpy(t.aabb, tree->aabb, sizeof(t.aabb));
  std::string err;
  int rc = write_kdt(t, path, err);
  if (rc != KDGR_OK) set_error("kdgr_write_kdt: " + err);
  return rc;
}

int kdgr_validate_tree(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                       uint32_t n_gaussians) {
  if (!nodes || (n_offsets && !offsets)) {
    set_error("kdgr_validate_tree: null argument");
    return KDGR_ERR_INVALID_ARG;
  }
  std::string err;
  int rc = validate_tree(nodes, n_nodes, offsets, n_offsets, n_gaussians, err, nullptr);
  if (rc != KDGR_OK) set_error("kdgr_validate_tree: " + err);
  return rc;
}

void kdgr_tree_free(kdgr_tree* tree) {
  if (!tree) return;
  free(tree->nodes);
  free(tree->offsets);
  free(tree->valid);
  memset(tree, 0, sizeof(*tree));
}

}  // extern "C"
