// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Standard headers the DAWN API and its command-line tools rely on.
#pragma once
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <algorithm>
#include <chrono>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#else
inline int omp_get_num_threads() { return 1; }
#endif
