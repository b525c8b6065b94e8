// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// GPU-side umbrella header.  The algorithms behind it run on the GB300
// kernels of libdawn_gb300.so through the C ABI (dawn_gb300.h); no CUDA or
// Thrust type appears in this API, so callers build with a plain C++ compiler.
#pragma once
#include <dawn/dawn.hxx>
