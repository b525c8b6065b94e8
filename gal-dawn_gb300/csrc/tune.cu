// Autotuner: per-graph choice of the traversal's speed settings.
//
// The reference fixes its launch shapes in the tools
// (algorithm/gpu/mssp_gpu/mssp_gpu.cu:16-17: block size 1024, 4 streams).
// Here the settings that change only speed are handle options (batch width,
// learned selector or heuristic, push ratio, heavy-row pull segment, CTAs
// per SM of the persistent grids), and dawn_autotune measures them on the
// caller's own graph: a coordinate search, one option at a time, each
// candidate timed with CUDA events on a sample of the caller's sources
// (best of two runs).  Batched candidates run in closeness mode, so no
// distance block is written and nothing is allocated per candidate beyond
// the handle's usual buffers.  A candidate replaces the current choice only
// when it is at least 2% faster, which keeps the defaults on ties.  Chosen
// settings go into a process-wide cache keyed by device and graph class.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "dawn_internal.cuh"

namespace dawn {
namespace {

struct Settings {
  int32_t width, ratio, seg, bps, learned;
};

std::mutex g_cache_mu;
std::map<std::string, dawn_tuning> g_cache;

std::string device_name(int device) {
  static std::mutex mu;
  static std::map<int, std::string> names;
  std::lock_guard<std::mutex> lock(mu);
  auto it = names.find(device);
  if (it != names.end()) return it->second;
  cudaDeviceProp prop;
  std::string dev = "unknown";
  if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) dev = prop.name;
  for (char& c : dev)
    if (c == ' ' || c == '\t' || c == '|') c = '_';
  names[device] = dev;
  return dev;
}

std::string class_key(const dawn_graph* g, int32_t nsrc) {
  const std::string dev = device_name(g->device);
  const int ln = (int)std::floor(std::log2((double)g->n + 1.0));
  const int ld = (int)std::floor(std::log2((double)g->m / (double)(g->n > 0 ? g->n : 1) + 1.0));
  const int sc = nsrc <= 1 ? 1 : nsrc <= 64 ? 2 : nsrc <= 128 ? 3 : 4;
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s|n%d|d%d|%s|s%d", dev.c_str(), ln, ld, g->symmetric ? "sym" : "dir", sc);
  return buf;
}

void apply(dawn_graph* g, const Settings& s) {
  g->bs_width = s.width;
  g->bs_push_ratio = s.ratio;
  g->pull_seg = s.seg;
  if (g->blocks_per_sm != s.bps) {
    g->blocks_per_sm = s.bps;
    drop_graphs(g);
  }
  g->auto_learned = s.learned != 0;
}

// Device time of one traversal of the sample under the handle's current
// settings; best of `reps` runs.
dawn_status time_sample(dawn_graph* g, const int32_t* src, int32_t k, bool batched, bool learned, int reps,
                        float* ms) {
  *ms = 0.0f;
  float best = -1.0f;
  for (int r = 0; r < reps; r++) {
    if (batched) {
      DAWN_CHECK(ensure(g->cc_out, 2 * sizeof(unsigned long long) * (size_t)k, g->stream));
      unsigned long long* sum = g->cc_out.as<unsigned long long>();
      DAWN_CUDA(cudaMemsetAsync(sum, 0, 2 * sizeof(unsigned long long) * (size_t)k, g->stream));
      DAWN_CHECK(call_selector(g, learned ? DAWN_VARIANT_LEARNED : DAWN_VARIANT_BITSET, &g->sel_call));
      DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
      DAWN_CHECK(bfs_bitset(g, src, k, nullptr, sum, sum + k));
    } else {
      DAWN_CHECK(ensure(g->dist_stage, sizeof(int32_t) * (size_t)k * (size_t)g->n, g->stream));
      DAWN_CHECK(call_selector(g, DAWN_VARIANT_DO, &g->sel_call));
      DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
      DAWN_CHECK(bfs_single(g, src, k, g->dist_stage.as<int32_t>(), DAWN_VARIANT_DO));
    }
    DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
    DAWN_CUDA(cudaEventSynchronize(g->ev1));
    float t = 0.0f;
    DAWN_CUDA(cudaEventElapsedTime(&t, g->ev0, g->ev1));
    if (best < 0.0f || t < best) best = t;
  }
  *ms = best;
  return DAWN_OK;
}

int32_t default_width(int32_t nsrc) { return nsrc > 128 ? 4 : nsrc > 64 ? 2 : 1; }

}  // namespace

dawn_status autotune(dawn_graph* g, const int32_t* sources, int32_t nsrc, uint32_t flags, dawn_tuning* out) {
  std::memset(out, 0, sizeof(*out));
  const std::string key = class_key(g, nsrc);
  if (flags & DAWN_TUNE_USE_CACHE) {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      *out = it->second;
      out->from_cache = 1;
      apply(g, Settings{out->bitset_width, out->push_ratio, out->pull_segment, out->blocks_per_sm, out->learned});
      return DAWN_OK;
    }
  }
  const bool batched = nsrc >= 2;
  const int32_t k = batched ? (nsrc < 256 ? nsrc : 256) : 1;
  const int32_t ks = batched ? k : (nsrc < 4 ? nsrc : 4);
  Settings cur{batched && nsrc > 64 ? default_width(nsrc) : 0, 4, 1024, 0, 0};
  apply(g, cur);
  float cur_ms = 0.0f;
  // one untimed run builds the pull lists and the captured graphs
  DAWN_CHECK(time_sample(g, sources, ks, batched, false, 1, &cur_ms));
  DAWN_CHECK(time_sample(g, sources, ks, batched, false, 2, &cur_ms));
  const float default_ms = cur_ms;

  auto try_values = [&](int32_t Settings::*field, const std::vector<int32_t>& values) -> dawn_status {
    for (int32_t v : values) {
      if (v == cur.*field) continue;
      Settings cand = cur;
      cand.*field = v;
      apply(g, cand);
      float ms = 0.0f;
      DAWN_CHECK(time_sample(g, sources, ks, batched, cand.learned != 0, 1, &ms));  // warm (lists, graphs)
      DAWN_CHECK(time_sample(g, sources, ks, batched, cand.learned != 0, 2, &ms));
      if (ms < 0.98f * cur_ms) {
        cur = cand;
        cur_ms = ms;
      }
    }
    apply(g, cur);
    return DAWN_OK;
  };
  if (batched) {
    if (nsrc > 64) DAWN_CHECK(try_values(&Settings::width, {1, 2, 4}));
    DAWN_CHECK(try_values(&Settings::learned, {0, 1}));
    DAWN_CHECK(try_values(&Settings::ratio, {2, 4, 8, 16}));
    DAWN_CHECK(try_values(&Settings::seg, {512, 1024, 2048, 4096}));
  }
  DAWN_CHECK(try_values(&Settings::bps, {0, 1, 2, 4}));

  out->bitset_width = cur.width;
  out->push_ratio = cur.ratio;
  out->pull_segment = cur.seg;
  out->blocks_per_sm = cur.bps;
  out->learned = cur.learned;
  out->from_cache = 0;
  out->ms = cur_ms;
  out->default_ms = default_ms;
  std::lock_guard<std::mutex> lock(g_cache_mu);
  g_cache[key] = *out;
  return DAWN_OK;
}

dawn_status tune_cache_save(const char* path) {
  std::lock_guard<std::mutex> lock(g_cache_mu);
  FILE* f = std::fopen(path, "w");
  if (!f) {
    set_error("cannot write %s", path);
    return DAWN_ERR_INVALID_ARG;
  }
  std::fprintf(f, "# dawn_gb300 tuning cache: class width ratio segment blocks_per_sm learned ms default_ms\n");
  for (const auto& kv : g_cache) {
    const dawn_tuning& t = kv.second;
    std::fprintf(f, "%s %d %d %d %d %d %.6g %.6g\n", kv.first.c_str(), t.bitset_width, t.push_ratio,
                 t.pull_segment, t.blocks_per_sm, t.learned, t.ms, t.default_ms);
  }
  std::fclose(f);
  return DAWN_OK;
}

dawn_status tune_cache_load(const char* path) {
  FILE* f = std::fopen(path, "r");
  if (!f) {
    set_error("cannot read %s", path);
    return DAWN_ERR_INVALID_ARG;
  }
  char line[512];
  std::map<std::string, dawn_tuning> loaded;
  int lineno = 0;
  while (std::fgets(line, sizeof(line), f)) {
    lineno++;
    if (line[0] == '#' || line[0] == '\n') continue;
    char key[256];
    dawn_tuning t = {};
    if (std::sscanf(line, "%255s %d %d %d %d %d %g %g", key, &t.bitset_width, &t.push_ratio, &t.pull_segment,
                    &t.blocks_per_sm, &t.learned, &t.ms, &t.default_ms) != 8 ||
        (t.bitset_width != 0 && t.bitset_width != 1 && t.bitset_width != 2 && t.bitset_width != 4) ||
        t.push_ratio < 1 || t.push_ratio > (1 << 20) || t.pull_segment < 128 || t.pull_segment > 65536 ||
        t.blocks_per_sm < 0 || t.blocks_per_sm > 32 || (t.learned != 0 && t.learned != 1)) {
      std::fclose(f);
      set_error("%s:%d: malformed tuning entry", path, lineno);
      return DAWN_ERR_INVALID_ARG;
    }
    loaded[key] = t;
  }
  std::fclose(f);
  std::lock_guard<std::mutex> lock(g_cache_mu);
  for (const auto& kv : loaded) g_cache[kv.first] = kv.second;
  return DAWN_OK;
}

}  // namespace dawn
