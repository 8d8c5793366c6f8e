// Declarations the reference's fixed-body and drag-selection code needs when
// build_ref.sh compiles the lines holding it (read from the reference's own
// files) as one C++ unit.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <ostream>

#include <collision/rigid/cylinder.h>
#include <collision/rigid/plane.h>
#include <collision/rigid/sphere.h>
#include <glm/gtc/matrix_transform.hpp>

namespace utilityCore {
glm::mat4 modelMatrix(const glm::vec3& pos, const glm::vec3& rot, const glm::vec3& scale);
}
