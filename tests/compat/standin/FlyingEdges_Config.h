// Stand-in for the reference's flyingEdges/util/FlyingEdges_Config.h in the
// shim test: only the names the shim uses.
#pragma once
#include <array>
#include <cstddef>
using std::size_t;
using scalar_t = float;
