// Shim for the reference build only (oracle/_ref).  The reference's glm submodule is empty; this header
// restates the part of glm's published vector semantics the reference's CPU step uses: packed float
// vec2/vec3 (8 / 12 bytes), component-wise +, -, *, / with vectors and scalars, compound assignment,
// operator[], and glm::length(v) = sqrt(dot(v, v)) with dot summed x, then y, then z.
#pragma once
#include "vec2.hpp"
