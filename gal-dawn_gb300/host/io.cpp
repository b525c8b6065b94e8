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
#include <dawn/io.hxx>

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

void build(DAWN::Graph::Graph_t& graph, std::vector<Entry>& e, bool symmetric, bool weighted) {
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

void read_any(std::string& input_path, DAWN::Graph::Graph_t& graph, bool symmetric, bool weighted) {
  std::string text;
  if (!read_all(input_path, &text)) {
    std::cerr << "Error opening file " << input_path << std::endl;
    return;
  }
  std::vector<Entry> e = parse_entries(text, weighted, graph.rows, input_path);
  build(graph, e, symmetric, weighted);
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

// Buffered text writer: the bytes of `ofstream << ... << std::endl` lines,
// without a flush per line.
struct Writer {
  FILE* f;
  std::vector<char> buf;
  explicit Writer(FILE* file) : f(file) { buf.reserve(1 << 20); }
  void put(const char* s, int k) {
    buf.insert(buf.end(), s, s + k);
    if (buf.size() > (1u << 20)) flush();
  }
  void flush() {
    if (!buf.empty()) std::fwrite(buf.data(), 1, buf.size(), f);
    buf.clear();
  }
};

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
  Writer w(f);
  char line[64];
  for (int j = 0; j < n; j++)
    if (source != j && result[j] > 0) w.put(line, std::snprintf(line, sizeof(line), "%d %d %d\n", source, j, result[j]));
  w.flush();
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

// Default ostream formatting of a float is printf's %g with precision 6.
void outfile(int n, float* result, int source, std::string& output_path) {
  FILE* f = open_out(output_path);
  if (!f) return;
  std::cout << "Start outfile" << std::endl;
  Writer w(f);
  char line[96];
  for (int j = 0; j < n; j++)
    if (source != j && result[j] != 0)
      w.put(line, std::snprintf(line, sizeof(line), "%d %d %g\n", source, j, (double)result[j]));
  w.flush();
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

void outfile(int n, int* result, std::string& output_path) {
  FILE* f = open_out(output_path);
  if (!f) return;
  std::cout << "Start outfile" << std::endl;
  Writer w(f);
  char line[64];
  for (int j = 0; j < n; j++)
    if (result[j] > 0) w.put(line, std::snprintf(line, sizeof(line), "%d %d\n", j, result[j]));
  w.flush();
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

void outfile(int n, float* result, std::string& output_path) {
  FILE* f = open_out(output_path);
  if (!f) return;
  std::cout << "Start outfile" << std::endl;
  Writer w(f);
  char line[96];
  for (int j = 0; j < n; j++)
    if (result[j] != 0) w.put(line, std::snprintf(line, sizeof(line), "%d %.6f\n", j, (double)result[j]));
  w.flush();
  std::cout << "End outfile" << std::endl;
  std::fclose(f);
}

}  // namespace IO
}  // namespace DAWN
