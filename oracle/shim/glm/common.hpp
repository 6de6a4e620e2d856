// Shim for the reference build only (oracle/_ref): glm vector subset, see vec3.hpp.
#pragma once
#include "vec3.hpp"
