#pragma once
#include <dawn/graph.hxx>
#include <dawn/io.hxx>
#include <dawn/matrix.hxx>
#include <dawn/parameters.hxx>
#include <dawn/tool.hxx>
