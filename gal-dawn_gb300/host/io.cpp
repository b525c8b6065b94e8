// MatrixMarket readers, source lists and text output (API and semantics of
// src/io.cpp:2-281 in the reference project).
//
// Reader semantics kept from the reference:
//   * every line whose first character is not '%' is an entry "row col
//     [val]" with 1-based indices (the size line, having row == col, is
//     dropped by the self-loop rule like any diagonal entry);
//   * self loops are dropped; duplicates are kept;
//   * symmetric files store each entry in both directions;
//   * entries are sorted by (row, col) or (row, col, val) before the CSR is
//     built.
// The file is read once, parsed in parallel chunks and sorted in parallel,
// instead of the reference's per-line stringstream and priority_queue; the
// sort fixes the order, so the CSR is identical.  Differences, all on input
// the reference handles with undefined behaviour: a blank or unparsable
// line is skipped (the reference re-reads the previous line's column), an
// index outside the matrix is an error, and a weighted read of a line
// without a value uses weight 1.
// Opt-in, not in the reference: DAWN_DEDUP=1 drops repeated (row, col)
// entries of an unweighted read (hop distances do not depend on them; the
// edge count and the TEPS numerator then count each edge once).  Weighted
// reads keep them, because the source-row rule (the last repeated entry's
// weight) makes distances depend on the repeats.
#include <dawn/io.hxx>

#include <sys/stat.h>

#include <algorithm>
#include <cstdlib>
#include <parallel/algorithm>
#include <tuple>

namespace DAWN {
namespace IO {

namespace {

bool read_all(const std::string& path, std::string* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out->resize(len > 0 ? (size_t)len : 0);
  const size_t got = len > 0 ? std::fread(&(*out)[0], 1, (size_t)len, f) : 0;
  std::fclose(f);
  out->resize(got);
  return true;
}

inline const char* skip_ws(const char* p, const char* e) {
  while (p < e && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
  return p;
}

// Parses an int like `stream >> int` does for well-formed input.
inline bool parse_int(const char*& p, const char* e, long long* v) {
  p = skip_ws(p, e);
  bool neg = false;
  if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
  if (p >= e || *p < '0' || *p > '9') return false;
  long long x = 0;
  while (p < e && *p >= '0' && *p <= '9') x = x * 10 + (*p++ - '0');
  *v = neg ? -x : x;
  return true;
}

inline bool parse_float(const char*& p, const char* e, float* v) {
  p = skip_ws(p, e);
  if (p >= e) return false;
  char buf[64];
  size_t k = 0;
  while (p + k < e && k < sizeof(buf) - 1 && p[k] != ' ' && p[k] != '\t' && p[k] != '\r' && p[k] != '\n') {
    buf[k] = p[k];
    k++;
  }
  buf[k] = 0;
  char* end = nullptr;
  const float x = std::strtof(buf, &end);
  if (end == buf) return false;
  p += end - buf;
  *v = x;
  return true;
}

struct Entry {
  int r, c;
  float v;
};

// Parses every entry line of a MatrixMarket body in parallel chunks.
std::vector<Entry> parse_entries(const std::string& text, bool weighted, int rows, const std::string& path) {
  const char* base = text.data();
  const size_t len = text.size();
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  if (len < ((size_t)1 << 20)) nt = 1;
  std::vector<size_t> cut(nt + 1, len);
  cut[0] = 0;
  for (int t = 1; t < nt; t++) {
    size_t p = len * t / nt;
    while (p < len && base[p - 1] != '\n') p++;
    cut[t] = p;
  }
  std::vector<std::vector<Entry>> part(nt);
  std::vector<int> bad(nt, 0);
#pragma omp parallel for num_threads(nt) schedule(static, 1)
  for (int t = 0; t < nt; t++) {
    const char* p = base + cut[t];
    const char* end = base + cut[t + 1];
    auto& out = part[t];
    while (p < end) {
      const char* eol = static_cast<const char*>(std::memchr(p, '\n', end - p));
      if (!eol) eol = end;
      if (*p != '%') {
        const char* q = p;
        long long r, c;
        if (parse_int(q, eol, &r) && parse_int(q, eol, &c)) {
          float v = 1.0f;
          if (weighted && !parse_float(q, eol, &v)) v = 1.0f;
          r -= 1;
          c -= 1;
          if (r != c) {
            if (r < 0 || c < 0 || r >= rows || c >= rows)
              bad[t] = 1;
            else
              out.push_back(Entry{(int)r, (int)c, v});
          }
        }
      }
      p = eol + 1;
    }
  }
  for (int t = 0; t < nt; t++)
    if (bad[t]) {
      std::cerr << "Error: an entry of " << path << " lies outside the " << rows << " x " << rows << " matrix"
                << std::endl;
      exit(EXIT_FAILURE);
    }
  size_t total = 0;
  for (auto& v : part) total += v.size();
  std::vector<Entry> all;
  all.reserve(total);
  for (auto& v : part) all.insert(all.end(), v.begin(), v.end());
  return all;
}

bool dedup_requested() {
  const char* env = std::getenv("DAWN_DEDUP");
  return env && *env && std::string(env) != "0";
}

void build(DAWN::Graph::Graph_t& graph, std::vector<Entry>& e, bool symmetric, bool weighted, bool dedup) {
  if (symmetric) {
    const size_t k = e.size();
    e.resize(2 * k);
    for (size_t i = 0; i < k; i++) e[k + i] = Entry{e[i].c, e[i].r, e[i].v};
  }
  if (weighted) {
    __gnu_parallel::sort(e.begin(), e.end(), [](const Entry& a, const Entry& b) {
      return std::tie(a.r, a.c, a.v) < std::tie(b.r, b.c, b.v);
    });
  } else {
    std::vector<uint64_t> key(e.size());
#pragma omp parallel for
    for (size_t i = 0; i < e.size(); i++) key[i] = ((uint64_t)(uint32_t)e[i].r << 32) | (uint32_t)e[i].c;
    __gnu_parallel::sort(key.begin(), key.end());
    if (dedup) {
      key.erase(std::unique(key.begin(), key.end()), key.end());
      e.resize(key.size());
    }
#pragma omp parallel for
    for (size_t i = 0; i < e.size(); i++) e[i] = Entry{(int)(key[i] >> 32), (int)(uint32_t)key[i], 0.0f};
  }
  const int nnz = (int)e.size();
  graph.nnz = (uint64_t)nnz;
  graph.coo.row = new int[nnz > 0 ? nnz : 1];
  graph.coo.col = new int[nnz > 0 ? nnz : 1];
  graph.coo.val = weighted ? new float[nnz > 0 ? nnz : 1] : nullptr;
#pragma omp parallel for
  for (int i = 0; i < nnz; i++) {
    graph.coo.row[i] = e[i].r;
    graph.coo.col[i] = e[i].c;
    if (weighted) graph.coo.val[i] = e[i].v;
  }
  if (weighted)
    DAWN::Matrix::coo2Csr_Weighted(graph.rows, nnz, graph.csr, graph.coo);
  else
    DAWN::Matrix::coo2Csr(graph.rows, nnz, graph.csr, graph.coo);
  delete[] graph.coo.row;
  delete[] graph.coo.col;
  delete[] graph.coo.val;
  graph.coo.row = graph.coo.col = nullptr;
  graph.coo.val = nullptr;
}

// --- binary CSR cache -----------------------------------------------------
//
// Parsing a large MatrixMarket file dominates a tool's run time; the CSR it
// yields depends only on the file and on the reader (symmetric or directed,
// weighted or not).  With DAWN_CSR_CACHE set, the CSR is stored after the
// first parse as <file name>.<s|d><w|u>[x].dawncsr (x: DAWN_DEDUP), beside the input file
// (DAWN_CSR_CACHE=1) or in the directory the variable names, together with
// the input's size and modification time; a later load of the same,
// unchanged file with the same reader reads the arrays back instead.  A
// cache that does not match (other file, changed file, other reader, short
// or damaged) is ignored and rewritten.

struct CacheHeader {
  char magic[8];
  uint32_t version, flags;  // flags: 1 symmetric, 2 weighted
  int64_t src_size, src_mtime_ns;
  int32_t rows, pad;
  int64_t nnz;
};
constexpr char kCacheMagic[8] = {'D', 'A', 'W', 'N', 'C', 'S', 'R', '1'};

std::string cache_path(const std::string& input, bool symmetric, bool weighted, bool dedup) {
  const char* env = std::getenv("DAWN_CSR_CACHE");
  if (!env || !*env || std::string(env) == "0") return "";
  std::string name = input;
  std::string dir;
  if (std::string(env) != "1") {
    const size_t slash = input.find_last_of('/');
    name = slash == std::string::npos ? input : input.substr(slash + 1);
    dir = std::string(env) + "/";
  }
  return dir + name + "." + (symmetric ? "s" : "d") + (weighted ? "w" : "u") + (dedup ? "x" : "") + ".dawncsr";
}

bool source_stat(const std::string& input, int64_t* size, int64_t* mtime_ns) {
  struct stat st;
  if (stat(input.c_str(), &st) != 0) return false;
  *size = (int64_t)st.st_size;
  *mtime_ns = (int64_t)st.st_mtim.tv_sec * 1000000000LL + (int64_t)st.st_mtim.tv_nsec;
  return true;
}

bool load_cache(const std::string& cpath, const std::string& input, DAWN::Graph::Graph_t& graph, bool symmetric,
                bool weighted, bool dedup) {
  int64_t size = 0, mtime = 0;
  if (!source_stat(input, &size, &mtime)) return false;
  FILE* f = std::fopen(cpath.c_str(), "rb");
  if (!f) return false;
  CacheHeader h;
  bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, kCacheMagic, 8) == 0 && h.version == 1 &&
            h.flags == (uint32_t)((symmetric ? 1 : 0) | (weighted ? 2 : 0) | (dedup ? 4 : 0)) && h.src_size == size &&
            h.src_mtime_ns == mtime && h.rows == graph.rows && h.nnz >= 0 && h.nnz <= INT32_MAX;
  if (ok) {
    const int nnz = (int)h.nnz;
    int* rp = new int[graph.rows + 1];
    int* col = new int[nnz > 0 ? nnz : 1];
    float* val = weighted ? new float[nnz > 0 ? nnz : 1] : nullptr;
    ok = std::fread(rp, sizeof(int), (size_t)graph.rows + 1, f) == (size_t)graph.rows + 1 &&
         std::fread(col, sizeof(int), (size_t)nnz, f) == (size_t)nnz &&
         (!weighted || std::fread(val, sizeof(float), (size_t)nnz, f) == (size_t)nnz) && rp[0] == 0 &&
         rp[graph.rows] == nnz;
    // A damaged cache must not reach the GPU unchecked (the device-side CSR
    // check can be switched off): rows never shrink, columns in [0, rows).
    for (int v = 0; ok && v < graph.rows; v++) ok = rp[v] <= rp[v + 1];
    for (int k = 0; ok && k < nnz; k++) ok = col[k] >= 0 && col[k] < graph.rows;
    if (ok) {
      graph.nnz = (uint64_t)nnz;
      graph.csr.row_ptr = rp;
      graph.csr.col = col;
      graph.csr.val = val;
    } else {
      delete[] rp;
      delete[] col;
      delete[] val;
    }
  }
  std::fclose(f);
  return ok;
}

void store_cache(const std::string& cpath, const std::string& input, const DAWN::Graph::Graph_t& graph,
                 bool symmetric, bool weighted, bool dedup) {
  CacheHeader h = {};
  std::memcpy(h.magic, kCacheMagic, 8);
  h.version = 1;
  h.flags = (symmetric ? 1 : 0) | (weighted ? 2 : 0) | (dedup ? 4 : 0);
  if (!source_stat(input, &h.src_size, &h.src_mtime_ns)) return;
  h.rows = graph.rows;
  h.nnz = (int64_t)graph.nnz;
  const std::string tmp = cpath + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return;  // no cache (read-only directory, say): the load itself succeeded
  const size_t nnz = (size_t)graph.nnz;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
            std::fwrite(graph.csr.row_ptr, sizeof(int), (size_t)graph.rows + 1, f) == (size_t)graph.rows + 1 &&
            std::fwrite(graph.csr.col, sizeof(int), nnz, f) == nnz &&
            (!weighted || std::fwrite(graph.csr.val, sizeof(float), nnz, f) == nnz);
  ok = std::fclose(f) == 0 && ok;
  if (ok)
    std::rename(tmp.c_str(), cpath.c_str());
  else
    std::remove(tmp.c_str());
}

void read_any(std::string& input_path, DAWN::Graph::Graph_t& graph, bool symmetric, bool weighted) {
  const bool dedup = !weighted && dedup_requested();
  const std::string cpath = cache_path(input_path, symmetric, weighted, dedup);
  if (!cpath.empty() && load_cache(cpath, input_path, graph, symmetric, weighted, dedup)) return;
  std::string text;
  if (!read_all(input_path, &text)) {
    std::cerr << "Error opening file " << input_path << std::endl;
    return;
  }
  std::vector<Entry> e = parse_entries(text, weighted, graph.rows, input_path);
  build(graph, e, symmetric, weighted, dedup);
  if (!cpath.empty()) store_cache(cpath, input_path, graph, symmetric, weighted, dedup);
}

}  // namespace

void readGraph(std::string& input_path, DAWN::Graph::Graph_t& graph) { read_any(input_path, graph, true, false); }

void readGraph_Weighted(std::string& input_path, DAWN::Graph::Graph_t& graph) {
  read_any(input_path, graph, true, true);
}

void readGraph_Directed(std::string& input_path, DAWN::Graph::Graph_t& graph) {
  read_any(input_path, graph, false, false);
}

void readGraph_Directed_Weighted(std::string& input_path, DAWN::Graph::Graph_t& graph) {
  read_any(input_path, graph, false, true);
}

void readList(std::string& input_path, DAWN::Graph::Graph_t& graph) {
  std::ifstream file(input_path);
  if (!file.is_open()) {
    std::cerr << "Error opening file " << input_path << std::endl;
    return;
  }
  std::string line;
  while (std::getline(file, line)) {
    if (!line.empty() && line[0] == '%') continue;
    std::stringstream ss(line);
    int source = 0;
    ss >> source;
    graph.msource.push_back(source);
  }
}

namespace {

// Text output: lines are formatted in parallel chunks (each thread fills its
// own buffer) and written in order, in rounds that bound the memory held.
// fmt(j, line) writes line j into `line` and returns its length (0: no line).
template <class Fmt>
void write_lines(FILE* f, int n, Fmt&& fmt) {
  constexpr int kChunk = 1 << 15;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  const int nchunks = (n + kChunk - 1) / kChunk;
  const int round = 4 * nt;
  std::vector<std::string> bufs((size_t)round);
  for (int c0 = 0; c0 < nchunks; c0 += round) {
    const int cn = std::min(round, nchunks - c0);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int b = 0; b < cn; b++) {
      std::string& s = bufs[(size_t)b];
      s.clear();
      char line[128];
      const int j0 = (c0 + b) * kChunk, j1 = std::min(n, j0 + kChunk);
      for (int j = j0; j < j1; j++) {
        const int k = fmt(j, line);
        if (k > 0) s.append(line, (size_t)k);
      }
    }
    for (int b = 0; b < cn; b++) std::fwrite(bufs[(size_t)b].data(), 1, bufs[(size_t)b].size(), f);
  }
}

// printf's %d, digit for digit.
inline char* put_int(char* p, int v) {
  uint32_t u = (uint32_t)v;
  if (v < 0) {
    *p++ = '-';
    u = 0u - u;
  }
  char tmp[10];
  int k = 0;
  do {
    tmp[k++] = (char)('0' + u % 10);
    u /= 10;
  } while (u);
  while (k) *p++ = tmp[--k];
  return p;
}

FILE* open_out(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) std::cerr << "Error opening file " << path << std::endl;
  return f;
}

}  // namespace

void outfile(int n, int* result, int source, std::string& output_path) {
  FILE* f = open_out(output_path);
  if (!f) return;
  std::cout << "Start outfile" << std::endl;
  write_lines(f, n, [&](int j, char* line) -> int {
    if (source == j || result[j] <= 0) return 0;
    char* p = put_int(line, source);
    *p++ = ' ';
    p = put_int(p, j);
    *p++ = ' ';
    p = put_int(p, result[j]);
    *p++ = '\n';
    return (int)(p - line);
  });
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

// Default ostream formatting of a float is printf's %g with precision 6.
void outfile(int n, float* result, int source, std::string& output_path) {
  FILE* f = open_out(output_path);
  if (!f) return;
  std::cout << "Start outfile" << std::endl;
  write_lines(f, n, [&](int j, char* line) -> int {
    if (source == j || result[j] == 0) return 0;
    return std::snprintf(line, 128, "%d %d %g\n", source, j, (double)result[j]);
  });
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

void outfile(int n, int* result, std::string& output_path) {
  FILE* f = open_out(output_path);
  if (!f) return;
  std::cout << "Start outfile" << std::endl;
  write_lines(f, n, [&](int j, char* line) -> int {
    if (result[j] <= 0) return 0;
    char* p = put_int(line, j);
    *p++ = ' ';
    p = put_int(p, result[j]);
    *p++ = '\n';
    return (int)(p - line);
  });
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

void outfile(int n, float* result, std::string& output_path) {
  FILE* f = open_out(output_path);
  if (!f) return;
  std::cout << "Start outfile" << std::endl;
  write_lines(f, n, [&](int j, char* line) -> int {
    if (result[j] == 0) return 0;
    return std::snprintf(line, 128, "%d %.6f\n", j, (double)result[j]);
  });
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

}  // namespace IO
}  // namespace DAWN
