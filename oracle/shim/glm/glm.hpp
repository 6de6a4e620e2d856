// Shim for the reference build only (oracle/_ref): glm vector subset, see vec3.hpp.  The reference's
// headers (e.g. include/simulation/data/Grid3D.h) use std::unordered_map / std::map without including them
// and rely on them arriving through this header, so it includes them.
#pragma once
#include <algorithm>
#include <map>
#include <unordered_map>
#include "vec3.hpp"
