// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Progress and averaging helpers (API of src/tool.cpp in the reference).
#include <dawn/tool.hxx>

namespace DAWN {
namespace Tool {

float average(int* result, int n) {
  int64_t sum = 0;
  int cnt = 0;
  for (int j = 0; j < n; j++)
    if (result[j] > 0) {
      sum += result[j];
      ++cnt;
    }
  return 1.0f * sum / cnt;
}

float average(float* result, int n) {
  int cnt = 0;
  float sum = 0.0f;
  for (int j = 0; j < n; j++)
    if (result[j] > 0) {
      sum += result[j];
      ++cnt;
    }
  return sum / cnt;
}

// Prints progress every total/interval entries.  The reference divides by
// total/interval unguarded (src/tool.cpp:32), which traps when total <
// interval; here such a run prints at every entry instead.
void infoprint(int entry, int total, int interval, int thread, float elapsed_time) {
  int step = interval > 0 ? total / interval : 0;
  if (step <= 0) step = 1;
  if (entry % step == 0) {
    float completion = static_cast<float>(entry * 100.0f) / static_cast<float>(total);
    std::cout << "Progress: " << completion << "%" << std::endl;
    std::cout << "Elapsed Time :" << static_cast<double>(elapsed_time) / (thread * 1000) << " s" << std::endl;
  }
}

}  // namespace Tool
}  // namespace DAWN
