// Interface between the two translation units of the reference harness:
// ref_harness.cpp (the PD step) and the scene unit that build_ref.sh
// compiles from the reference's fixed-body and drag-selection code.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <glm/glm.hpp>

struct RefFixedSpec {  // one fixed body as the scene file gives it (context.cpp:225-310)
    int type;          // 0 sphere, 1 plane, 2 cylinder
    float pos[3], rot[3], scale[3];  // sphere radius = scale[0]
};

// Builds the reference's Sphere / Plane / Cylinder objects.
void* ref_make_fixed(int n, const RefFixedSpec* specs);
void ref_free_fixed(void* fixed);
// FixedBodyData::HandleCollisions: spheres, then planes, then cylinders.
void ref_handle_collisions(void* fixed, glm::vec3* X, glm::vec3* V, int nv, float muT, float muN);
// SimulationCUDAContext::ResetMoreDBC while dragging (Control_Kernel, control_mag 10).
void ref_control(glm::vec3* X, float* DBC, float* moreDBC, glm::vec3* OffsetX, int nv, int select_v);
