// Declarations the reference's continuous-collision query needs when
// build_ref.sh compiles the lines holding it (stp, the root finders, the
// face / edge distances and ccdCollisionTest of intersections.cu, read from
// the reference's own file) as one C++ unit.  TEST INFRASTRUCTURE ONLY.
//
// On the GPU, sqrt and abs of a float are CUDA's float overloads; the global
// using-declarations give the host compile the same overloads (otherwise an
// unqualified abs(float) could bind to the C library's int abs).
#pragma once
#include <cfloat>
#include <cmath>

#define GLM_ENABLE_EXPERIMENTAL
#include <glm/glm.hpp>
#include <glm/gtx/norm.hpp>

#include <collision/aabb.h>

using std::abs;
using std::sqrt;
using glm::cross;
using glm::dot;
using glm::length;
using glm::length2;
using glm::normalize;
