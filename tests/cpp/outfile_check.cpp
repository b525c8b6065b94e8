// Writes the four DAWN::IO::outfile forms for values read from a binary
// file (n, source, n int32, n float32), for the text-output tests.
#include <dawn/io.hxx>

#include <cstdio>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int n = 0, source = 0;
  if (std::fread(&n, 4, 1, f) != 1 || std::fread(&source, 4, 1, f) != 1) return 4;
  std::vector<int> iv(n);
  std::vector<float> fv(n);
  if (std::fread(iv.data(), 4, n, f) != (size_t)n || std::fread(fv.data(), 4, n, f) != (size_t)n) return 5;
  std::fclose(f);
  std::string base = argv[2];
  std::string p1 = base + ".is", p2 = base + ".fs", p3 = base + ".i", p4 = base + ".f";
  DAWN::IO::outfile(n, iv.data(), source, p1);
  DAWN::IO::outfile(n, fv.data(), source, p2);
  DAWN::IO::outfile(n, iv.data(), p3);
  DAWN::IO::outfile(n, fv.data(), p4);
  return 0;
}
