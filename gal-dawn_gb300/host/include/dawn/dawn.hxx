// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
#pragma once
#include <dawn/graph.hxx>
#include <dawn/io.hxx>
#include <dawn/matrix.hxx>
#include <dawn/parameters.hxx>
#include <dawn/tool.hxx>
