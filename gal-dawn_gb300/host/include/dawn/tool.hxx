// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Small helpers, API of include/dawn/tool.hxx in the reference project.
#pragma once
#include <dawn/include.hxx>

namespace DAWN {
namespace Tool {

float average(int* result, int n);
float average(float* result, int n);
void infoprint(int entry, int total, int interval, int thread, float elapsed_time);

}  // namespace Tool
}  // namespace DAWN
