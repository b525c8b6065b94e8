// dump_csr: loads a MatrixMarket file through DAWN::Graph::createGraph and
// writes the CSR as raw little-endian arrays (loader checks):
//   int32 rows, int32 cols, int64 nnz, int32 directed, int32 source,
//   int32 row_ptr[rows+1], int32 col[nnz], float val[nnz] (weighted only)
// usage: dump_csr <file.mtx> <weighted 0|1> <source> <out.bin>
#include <dawn/dawn.hxx>

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: dump_csr <file.mtx> <weighted 0|1> <source> <out.bin>\n");
    return 2;
  }
  std::string in = argv[1];
  DAWN::Graph::Graph_t g;
  g.weighted = std::atoi(argv[2]) != 0;
  g.source = std::atoi(argv[3]);
  DAWN::Graph::createGraph(in, g);
  FILE* f = std::fopen(argv[4], "wb");
  if (!f) return 1;
  const int32_t hdr[2] = {g.rows, g.cols};
  const int64_t nnz = (int64_t)g.nnz;
  const int32_t tail[2] = {g.directed ? 1 : 0, g.source};
  std::fwrite(hdr, sizeof(hdr), 1, f);
  std::fwrite(&nnz, sizeof(nnz), 1, f);
  std::fwrite(tail, sizeof(tail), 1, f);
  std::fwrite(g.csr.row_ptr, sizeof(int32_t), (size_t)g.rows + 1, f);
  std::fwrite(g.csr.col, sizeof(int32_t), (size_t)nnz, f);
  if (g.weighted) std::fwrite(g.csr.val, sizeof(float), (size_t)nnz, f);
  std::fclose(f);
  return 0;
}
